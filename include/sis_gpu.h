/*
 * sis_gpu.h -- C ABI of libsisgpu.so, the GB300 (sm_103a) engine for the SIS
 * coarse-grained RNA model's force and integration hot path.
 *
 * The reference (Hori-Lab/SIS, Fortran) exposes this path as subroutines on
 * module-global state:
 *     subroutine force(irep, forces)                     src/force.F90:1,14-15
 *     subroutine energy_sumup(irep, tempK_in, energies)  src/energy_sumup.F90:1,11-13
 *     subroutine neighbor_list(irep)                     src/neighbor_list.F90:1
 *     the GJF-2GJ / Ermak-McCammon update                src/job_md.F90:360-460
 * Here the state lives on the device inside an opaque context; every entry
 * point takes the replica (instance) index explicitly, copies caller-owned
 * host buffers in or out, and returns an int status instead of aborting.
 *
 * Units and layouts follow the reference: Angstrom, kcal/mol, K, mol/L;
 * coordinates of one instance are xyz(3,nmp) column-major (bead-major xyz
 * triples); pair lists use 1-based bead indices local to the instance.
 *
 * Instances generalise the reference's replicas: the reference runs nrep
 * copies of one topology; a context holds n_inst instances which may each
 * have their own chains, temperature, salt and box.  One host thread per
 * context; calls are stream-ordered on the context's own CUDA stream.
 */
#ifndef SIS_GPU_H
#define SIS_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes (the reference has none: it calls sis_abort, src/sis_abort.F90) */
#define SIS_OK 0
#define SIS_ERR_ARG -1          /* invalid argument */
#define SIS_ERR_CUDA -2         /* CUDA runtime error; see sis_gpu_last_error */
#define SIS_ERR_LIST_OVERFLOW -3/* a neighbour list exceeded its capacity */
#define SIS_ERR_NONFINITE -4    /* NaN/Inf detected in coordinates or forces */
#define SIS_ERR_NOMEM -5        /* device allocation failed */
#define SIS_ERR_STATE -6        /* call out of order (e.g. force before set_state) */
#define SIS_ERR_TIMEOUT -7      /* a bounded device wait ran out (the grid barrier of the trigger/rebuild kernel) */

/* arithmetic of the force terms */
#define SIS_PREC_FP64 0  /* all terms and the integration in FP64 (plain path) */
#define SIS_PREC_MIXED 1 /* FP32 pair/bonded terms accumulated per bead into FP64, FP64 integration */

/* integrators, const_idx.F90 INTGRT */
#define SIS_INTGRT_GJF2GJ 1
#define SIS_INTGRT_BD_EM 2

/* energies(0:10) slots, const_idx.F90:7-21 ENE */
#define SIS_ENE_TOTAL 0
#define SIS_ENE_BOND 1
#define SIS_ENE_ANGL 2
#define SIS_ENE_DIHE 3
#define SIS_ENE_BP 4
#define SIS_ENE_EXV 5
#define SIS_ENE_ELE 6
#define SIS_ENE_MAX 10

/* list kinds for sis_gpu_get_list */
#define SIS_LIST_WCA 0 /* wca_mp(2,n)  src/var_potential.F90 */
#define SIS_LIST_ELE 1 /* ele_mp(2,n) */
#define SIS_LIST_BP 2  /* bp_mp(7,n)  */
/* the WCA / electrostatic pairs (2,n) of the per-block kernel's inner lists
 * (contexts of small instances, instances of 256 moving beads or more: the
 * list entries within their cutoff + 2.5 A, as last filtered by the kernel) */
#define SIS_LIST_WCA_INNER 3
#define SIS_LIST_ELE_INNER 4

/* Model parameters: the .ff file (src/read_force_field.F90) and the input
 * TOML sections [Basepair] [Electrostatic] [MD] (src/read_input.F90). */
typedef struct sis_params {
    double bond_k, bond_r0;          /* [potential.bond] k, r0 */
    int32_t angl_reb;                /* 1: [potential.angle_ReB] instead of [potential.angle] */
    double angl_k, angl_t0;          /* k, a0 */
    int32_t dih_type;                /* 0 none, 1 [potential.dihedral], 2 [potential.dihedral_exp] */
    double dih_k, dih_w, dih_p0;
    double wca_sigma, wca_eps;       /* [potential.wca] */
    int32_t bp_model;                /* [Basepair] model: 1, 3, 4 or 5 */
    int32_t bp_min_loop;             /* [Basepair] min_loop */
    int32_t bp_jnext_compat;         /* 1: reproduce src/neighbor_list.F90:212 (jmp+1 of the pair
                                        tested against the length of imp's chain) */
    double bp_cutoff_energy;         /* [potential.basepair] cutoff_energy */
    /* [potential.basepair.GC|AU|GU]: U0 bond_k bond_r angl_k1..4 angl_theta1..4
       dihd_k1 dihd_k2 dihd_phi1 dihd_phi2 */
    double bp_ff[3][15];
    double nn_dH[21], nn_dS[21];     /* [NN.dH] [NN.dS] in NNT order (src/const_idx.F90) */
    double dH0, dS0;
    int32_t nnend;
    double nnend_dH[6], nnend_dS[6], dHend0, dSend0;
    int32_t flg_ele;                 /* [Electrostatic] present */
    int32_t ele_cutoff_type;         /* 1: cutoff in Angstrom, 2: in units of the Debye length */
    double ele_cutoff_inp, length_per_charge;
    int32_t ele_excl_bond, ele_excl_angle;
    int32_t temp_independent;
    double tempK_ref;
    int32_t integrator;              /* SIS_INTGRT_* */
    double dt, viscosity_Pas, nl_margin;
    int32_t nstep_bp_mc;             /* [Basepair] nstep_MC: Monte Carlo removal every n steps (0: none) */
    int32_t max_bp_per_nt;           /* [Basepair] max_bp_per_nt */
    /* engine options (no counterpart in the reference) */
    int32_t precision;               /* SIS_PREC_* */
    uint64_t seed;                   /* Philox key for the Langevin noise */
    int32_t nbr_cap;                 /* per-bead pair-list capacity (0: automatic) */
    int32_t bp_cap;                  /* per-bead base-pair candidate capacity (0: automatic) */
} sis_params;

/* Topology and conditions of all instances. */
typedef struct sis_topology {
    int32_t n_inst;
    const int32_t *inst_chain_off;   /* [n_inst+1]: chains of instance k are [off[k], off[k+1]) */
    const int32_t *chain_len;        /* [n_chains] nmp_chain */
    const int32_t *chain_moltype;    /* [n_chains] 1 linearRNA, 2 circRNA (MOLT) */
    const int32_t *seq;              /* [n_beads] SEQT: A=0 U=1 G=2 C=3 D=4 */
    const uint8_t *has_charge;       /* [n_beads] */
    const double *tempK;             /* [n_inst] */
    const double *ionic_strength;    /* [n_inst] mol/L */
    const double *box;               /* [3*n_inst] PBC box, or NULL / zeros for no PBC */
    const uint32_t *stream;          /* [n_inst] Philox noise stream per instance, or NULL (= index) */
} sis_topology;

typedef struct sis_ctx sis_ctx;

typedef struct sis_stats {
    int64_t steps;          /* MD steps taken */
    int64_t rebuilds;       /* instance neighbour-list rebuilds (sum over instances) */
    int64_t pair_entries;   /* current full pair-list entries (both directions) */
    int64_t wca_pairs;      /* current half-list WCA pairs */
    int64_t ele_pairs;      /* current half-list ele pairs */
    int64_t bp_pairs;       /* current base-pair candidates */
    int32_t error_flags;    /* bit 0 pair overflow, bit 1 bp overflow, bit 2 nonfinite, bit 3 barrier timeout */
    int32_t n_beads;
    int32_t n_inst;
    int32_t lanes_per_bead; /* group width of the step kernel (sis_gpu_set_lanes) */
    int64_t capped;         /* bead-steps at which sis_gpu_set_force_cap's cap bound */
    int32_t bp_blocks;      /* block count of the base-pair evaluation */
    int32_t overlap;        /* 1: pair forces in their own kernel (sis_gpu_set_overlap) */
    int32_t small_blocks;   /* blocks of the per-block kernel of small instances (0: not used) */
    int32_t small_threads;  /* threads per block of that kernel */
    int64_t cluster_pairs;  /* mixed path: current cluster-pair list entries (i-cluster x j-cluster) */
    int32_t i_clusters;     /* mixed path: i-clusters of 8 beads (those whose j-clusters fit) */
    int32_t reserved;
} sis_stats;

/* Creates a context and uploads topology and parameters.  Replaces the
 * set-up the reference does in init_bp, init_ele/set_ele, list_local and
 * set_md_coef (src/init_bp.F90, src/set_ele.F90, src/list_local.F90,
 * src/job_md.F90:94-133,700-767).  Before any device work it refuses with
 * SIS_ERR_ARG: a sequence code outside A U G C D (0-4), a molecule type
 * other than 1 or 2, an empty chain, a non-positive or non-finite
 * temperature, salt (with electrostatics) or time step, a negative or
 * non-finite box component, viscosity <= 0, a negative list margin or
 * capacity, an unknown precision, integrator, base-pair model (0-5) or
 * cutoff type, and base-pair Monte Carlo with max_bp_per_nt < 1. */
int sis_gpu_create(const sis_topology *top, const sis_params *par, sis_ctx **out);
void sis_gpu_destroy(sis_ctx *ctx);
/* number of beads of instance inst (nmp), or of all instances for inst = -1 */
int sis_gpu_nmp(const sis_ctx *ctx, int32_t inst);

/* State of instance inst: xyz/velos/accels (3,nmp); NULL leaves a field
 * unchanged.  inst = -1 addresses all beads of all instances at once.
 * (src/var_state.F90 xyz, velos, accels) */
int sis_gpu_set_state(sis_ctx *ctx, int32_t inst, const double *xyz, const double *velos, const double *accels);
int sis_gpu_get_state(sis_ctx *ctx, int32_t inst, double *xyz, double *velos, double *accels);
/* Maxwell-Boltzmann velocities and initial GJF-2GJ accels from the Philox
 * stream (src/job_md.F90:214-238). */
int sis_gpu_init_velocities(sis_ctx *ctx);

/* neighbor_list(irep): pbc_wrap + list rebuild of instance inst (-1: all);
 * replaces src/neighbor_list.F90:1 and src/pbc.F90:196-226. */
int sis_gpu_neighbor_list(sis_ctx *ctx, int32_t inst);
/* Copies a list of instance inst (kind SIS_LIST_*, 1-based local indices,
 * records (2,n) or (7,n) in unspecified order).  *n_out = number of records.
 * The inner kinds need a context of small instances (SIS_ERR_ARG otherwise). */
int sis_gpu_get_list(sis_ctx *ctx, int32_t inst, int32_t kind, int32_t *out, int32_t cap, int32_t *n_out);
/* bp_coef(2,n) (dH, dS) aligned with the SIS_LIST_BP records of the last get_list call order */
int sis_gpu_get_bp_coef(sis_ctx *ctx, int32_t inst, double *out, int32_t cap, int32_t *n_out);

/* force(irep, forces): forces(3,nmp) of instance inst at the current
 * coordinates (src/force.F90:1).  Also caches the base-pair energies as the
 * reference's flg_bp_energy does. */
int sis_gpu_force(sis_ctx *ctx, int32_t inst, double *forces);
/* forces of one term: 1 bond, 2 angle, 3 dihedral, 4 base pair, 5 WCA, 6 DH */
int sis_gpu_force_term(sis_ctx *ctx, int32_t inst, int32_t term, double *forces);
/* energy_sumup(irep, tempK_in, energies(0:10)) (src/energy_sumup.F90:1).
 * The base-pair slot uses the energies cached by the last force evaluation
 * while that cache is valid, as src/energy_bp.F90 does. */
int sis_gpu_energy_sumup(sis_ctx *ctx, int32_t inst, double tempK, double *energies11);
/* energy_rg (src/energy_rg.F90:17-26): unweighted radius of gyration of the
 * current coordinates, for one instance or (inst = -1) every instance. */
int sis_gpu_rg(sis_ctx *ctx, int32_t inst, double *rg);
/* energy_kinetic (src/energy_kinetic.F90) */
int sis_gpu_energy_kinetic(sis_ctx *ctx, int32_t inst, double *ekin);
/* invalidates the base-pair energy cache (flg_bp_energy = .False.) */
int sis_gpu_invalidate_bp_cache(sis_ctx *ctx);

/* Advances all instances by nsteps MD steps (src/job_md.F90:360-460): per
 * step and instance the displacement-triggered list rebuild, forces, noise
 * and the GJF-2GJ (or Ermak-McCammon) update.  noise == NULL draws Gaussian
 * noise from a counter-based Philox4x32-10 stream; otherwise noise holds
 * [nsteps][n_beads_total][3] doubles in the reference's rnd_bm order. */
int sis_gpu_step(sis_ctx *ctx, int64_t nsteps, const double *noise);

/* set_ele + set_md_coef for one instance at a new temperature / salt
 * (src/set_ele.F90, src/job_md.F90:700-767). */
int sis_gpu_set_condition(sis_ctx *ctx, int32_t inst, double tempK, double ionic_strength);
/* The simulated-annealing update of job_md.F90:597-611 for one instance (or
 * all, inst = -1): the temperature of the noise coefficients (set_md_coef)
 * and of the base-pair free energies dG = dH - T dS moves to tempK; the
 * Debye-Hueckel parameters keep the temperature they were set at, as the
 * reference calls no set_ele there. */
int sis_gpu_set_temperature(sis_ctx *ctx, int32_t inst, double tempK);
/* [Freeze] (set_md_coef, src/job_md.F90:713-729,745-748): beads[n] are
 * 1-based bead numbers of instance inst whose positions stay fixed (the
 * GJF-2GJ position coefficient sqrt(b) h, or the Ermak-McCammon h/gamma and
 * noise, set to zero); the call replaces the instance's earlier set, n = 0
 * frees all.  Under replica exchange every replica must freeze the same
 * beads (the reference freezes by bead number in all replicas). */
int sis_gpu_set_frozen(sis_ctx *ctx, int32_t inst, const int32_t *beads, int32_t n);
/* Base pairs restricted to a given secondary structure (read_ss.F90 sets
 * bp_map from the ct, bpseq or bpl file of [Files.In]; init_bp.F90:207-209
 * then skips every other pair): pairs[2n] are (imp, jmp), 1-based
 * nucleotide numbers of instance inst, after read_ss's checks (chain ends,
 * minimum loop, isolated pairs, known pair types; sis_gb300/inputs.py
 * filter_ss_pairs); the candidate rules of init_bp still apply.  n = 0 lifts
 * the restriction.  The lists are rebuilt at the next call that needs them. */
int sis_gpu_set_ss_pairs(sis_ctx *ctx, int32_t inst, int32_t n, const int32_t *pairs);
/* [Bias_SS] (read_input.F90:1198-1217): on != 0 pulls an allowed pair whose
 * distance lies outside its window toward each other with a constant force
 * (kcal/mol/A; the input's force_pN times 1e-22 J->kcal/mol) in the triplet
 * models 4 and 5 (force_bp_triplet.F90:85-92), and lists every allowed pair
 * whatever its distance (neighbor_list.F90:89-93).  It needs a secondary
 * structure (sis_gpu_set_ss_pairs), as the reference does. */
int sis_gpu_set_bias_ss(sis_ctx *ctx, int32_t on, double force);
/* Caps the magnitude of every bead's total force at fmax (kcal/mol/A) in
 * sis_gpu_step; 0 removes the cap.  An equilibration aid for starting
 * structures with overlapping beads; it has no counterpart in the reference
 * and is off unless set. */
int sis_gpu_set_force_cap(sis_ctx *ctx, double fmax);

/* Optional terms of force.F90:62-75 and energy_sumup.F90:47-52, evaluated in
 * FP64 in both precisions: force term 7 of sis_gpu_force_term, energy slots
 * 7 (stage), 8 (tweezers), 9 (Rg bias) and 10 (restraints).
 * sis_gpu_set_stage: the wall at z = 0 of force_stage.F90 / energy_stage.F90
 * (stage_sigma, stage_eps); sigma = 0 turns it off.
 * sis_gpu_set_rg_bias: the bias on the radius of gyration of force_rg.F90 /
 * energy_rg.F90 for one instance (inst = -1: all); pott 0 off, 1 harmonic,
 * 2 flat-bottomed (no force while Rg <= rg0).
 * sis_gpu_set_bias_items: the sigmoid restraints (force_restraint.F90) and
 * tweezers trap pairs (force_tweezers.F90) of one instance, replacing those
 * set before: kind_ij[n][3] = kind, i, j (1-based beads of the instance);
 * par[n][14].  kind 1 restraint on both beads, 2 restraint on bead i only
 * (Sigmoid-to-bead), par eps, d, s, rcut; kind 3 constant-force trap pair,
 * par the force on bead i (its negative on bead j); kind 4 force-ramp trap
 * pair, par k_i, k_j, trap starts (i xyz, j xyz), trap velocities per step
 * (i xyz, j xyz): the traps sit at start + velocity * istep, istep counting
 * the step being taken (job_md.F90:362), or the steps taken outside one. */
int sis_gpu_set_stage(sis_ctx *ctx, double sigma, double eps);
int sis_gpu_set_rg_bias(sis_ctx *ctx, int32_t inst, int32_t pott, double k, double rg0);
int sis_gpu_set_bias_items(sis_ctx *ctx, int32_t inst, int32_t n, const int32_t *kind_ij, const double *par);
/* per-bead integrator coefficients of instance inst, 4 per bead: GJF-2GJ
 * md_coef(1:3) and md_coef_rep(1) (src/job_md.F90:700-767) */
int sis_gpu_get_md_coef(sis_ctx *ctx, int32_t inst, double *out4);
/* derived per-instance electrostatic values [ele_coef, lambdaD, ele_cutoff, diele] */
int sis_gpu_get_ele(sis_ctx *ctx, int32_t inst, double *out4);

/* Philox step counter of the noise stream (restart files store it in place
 * of the reference's MT19937 state, src/write_rst.F90 PRNG block). */
int sis_gpu_get_step(sis_ctx *ctx, uint64_t *step);
int sis_gpu_set_step(sis_ctx *ctx, uint64_t step);

/* Lanes per bead of the step kernel (1, 2, 4, 8, 16 or 32); 0 (default)
 * lets the autotuner pick it on the first long run (64 steps or more). */
int sis_gpu_set_lanes(sis_ctx *ctx, int32_t lanes);
/* 1 (default): sis_gpu_step runs steady-state steps as captured CUDA graphs
 * (20 steps each); 0: every kernel is launched from the host.  Results are
 * identical; per-kernel profilers see only the second form. */
int sis_gpu_set_graphs(sis_ctx *ctx, int32_t enable);
/* 1: a step's pair forces (WCA, Debye-Hueckel) are computed by a kernel of
 * their own on another stream, concurrently with the bonded and base-pair
 * pass, and the step kernel takes them from a per-bead buffer; 0: the step
 * kernel computes them; -1 (default): the autotuner chooses, with the lanes
 * per bead, on the first long run.  Results are identical. */
int sis_gpu_set_overlap(sis_ctx *ctx, int32_t enable);
/* Per-block kernel of small instances (mixed path): when every instance has
 * at most 2048 beads and an all-pairs list (no cell grid), no base-pair Monte
 * Carlo and no optional term is on, sis_gpu_step runs all its steps in one
 * launch per 1000 steps, each block owning a bucket of whole instances in
 * shared memory (job_md.F90:360-460 for every instance at once).  The
 * buckets and the block width are picked by timing on the first long run.
 * -1 (default): used where eligible; 0: never (the general kernels);
 * 1: as -1.  Trajectories do not depend on the buckets or the block width;
 * they differ from the general kernels' in the order of FP32 sums only. */
int sis_gpu_set_small(sis_ctx *ctx, int32_t mode);

int sis_gpu_get_stats(sis_ctx *ctx, sis_stats *st);
/* Failure-detection self-test (no counterpart in the reference): one block of
 * a cooperative launch never reaches the grid barrier that the
 * trigger/rebuild kernel uses, so the other blocks' bounded waits run out
 * (about a second).  Returns SIS_ERR_TIMEOUT when the kernel reported the
 * timeout; the barrier is then reset, and the context works on. */
int sis_gpu_probe_barrier_timeout(sis_ctx *ctx);
/* Human-readable description of the last error on this context. */
const char *sis_gpu_last_error(const sis_ctx *ctx);

/* Timing on the context's stream (CUDA events), for benchmarks. */
int sis_gpu_event_record(sis_ctx *ctx, int32_t slot);
int sis_gpu_event_elapsed(sis_ctx *ctx, int32_t slot_a, int32_t slot_b, float *ms);
int sis_gpu_synchronize(sis_ctx *ctx);
/* Writes a device buffer larger than L2 on the context's stream. */
int sis_gpu_flush_l2(sis_ctx *ctx);
/* Number of kernels this context has launched so far. */
int64_t sis_gpu_kernel_launches(const sis_ctx *ctx);
/* Like sis_gpu_step (Philox noise), launched kernel by kernel with CUDA
 * events around every kernel group on the context's stream; ms[0..2] receive
 * the summed durations of the bonded and base-pair pass, the step kernel, and
 * the trigger and rebuild kernels (launched every step, early exit when no
 * rebuild is due).  For roofline measurements. */
int sis_gpu_step_profiled(sis_ctx *ctx, int64_t nsteps, float *ms3);

/* Temperature replica exchange on the device (src/replica_exchange.F90,
 * src/energy_replica.F90, src/var_replica.F90:105-259; the reference runs one
 * replica per MPI rank, here every replica is an instance of the context).
 * sis_gpu_remd_init: temps[n_inst] is the ladder by label, strictly
 * ascending; the instances must be replicas of one topology, salt and box,
 * each at a distinct rung (it starts on that label).
 * sis_gpu_remd_exchange: one exchange attempt between the pairs of labels
 * (0,1), (2,3), ... (parity 0, the reference's odd pattern 1-2, 3-4, ...) or
 * (1,2), (3,4), ... (parity 1), on the current coordinates: total potential
 * energies at the own and at the partner temperature (set_ele at the
 * partner's temperature, base-pair energies recomputed), Sugita's criterion
 * delta = ((E_j(T_m) - E_i(T_m))/T_m - (E_j(T_n) - E_i(T_n))/T_n)/k_B, accept
 * if delta < 0 or u <= exp(-delta); an accepted pair swaps labels and
 * temperatures, its velocities are scaled by sqrt(T_n/T_m) (scale_velo) and
 * its noise coefficients follow the new temperature.  uniforms: one per pair
 * in label order (n_inst/2 + 1 values; the reference's random0), or NULL for
 * device Philox uniforms.  rep2lab (out, may be NULL): the label of every
 * instance afterwards; n_accepted (out, may be NULL). */
int sis_gpu_remd_init(sis_ctx *ctx, const double *temps);
/* Replica exchange over any of the reference's replica variables
 * (var_replica.F90 REPT: 1 temperature in K, 2 ionic strength in M,
 * 3 constant trap force magnitude in kcal/mol/A, 4 Rg bias target in A;
 * energy_replica.F90:72-121 sets them to the partner label's values for the
 * partner energy).  kinds[nvar] names the columns of values[n_inst][nvar];
 * row l holds label l's values and replica k starts on label k, taking its
 * values now.  A trap-force variable scales the constant-force pairs of
 * sis_gpu_set_bias_items (their force vectors then give the direction per
 * unit force, twz_DCF_direction); an Rg variable needs the Rg bias on every
 * replica.  Exchanges are sis_gpu_remd_exchange's, with T_m = T_n when the
 * temperature is not a variable (no velocity scaling then). */
int sis_gpu_remd_init_vars(sis_ctx *ctx, int32_t nvar, const int32_t *kinds, const double *values);
int sis_gpu_remd_exchange(sis_ctx *ctx, int32_t parity, const double *uniforms, int32_t *rep2lab, int32_t *n_accepted);

/* Base-pair Monte Carlo removal (src/force_bp_limit_triplet.F90,
 * job_md.F90:364-401), active when sis_params.nstep_bp_mc > 0: every
 * nstep_bp_mc steps and after every list rebuild of an instance, its
 * base-pair evaluation keeps each record's forces, removes pairs until no
 * nucleotide carries more than max_bp_per_nt (the reference's selection,
 * shuffle and Metropolis walk, on device Philox uniforms), scatters the
 * survivors and masks the others until the next pass.  sis_gpu_bp_mc
 * requests a pass at the next force or step evaluation of one instance (or
 * all, inst = -1); draws, if given, are the uniforms it consumes in the
 * reference's order (genrand_double3/double1 values), for exact parity.
 * sis_gpu_get_bp_status: the status of every base-pair record, in the order
 * of sis_gpu_get_list(..., SIS_LIST_BP, ...). */
int sis_gpu_bp_mc(sis_ctx *ctx, int32_t inst, const double *draws, int32_t n_draws);
int sis_gpu_get_bp_status(sis_ctx *ctx, int32_t inst, uint8_t *out, int32_t cap, int32_t *n_out);
/* The energy of every base-pair record cached by the last force or energy
 * evaluation (ene_bp of var_state.F90, zero for records outside the window
 * or above the energy cut), in the order of sis_gpu_get_list(...,
 * SIS_LIST_BP, ...): what write_bp.F90 writes to the .bp/.bpall/.bpe files. */
int sis_gpu_get_bp_energies(sis_ctx *ctx, int32_t inst, double *out, int32_t cap, int32_t *n_out);

/* Serving slots (no counterpart in the reference, whose jobs are separate
 * runs).  Replaces the topology, conditions and state of instance inst by a
 * job of n_chains chains (chain_len, chain_moltype, seq and has_charge as in
 * sis_topology, for the job's beads only) that fits in the instance's bead
 * count; the instance's remaining beads become inert fillers (single-bead
 * chains of sequence D, uncharged, frozen), which no list, bonded or
 * base-pair term includes.  n_chains = 0 empties the slot.  The job's noise
 * stream is `stream` and its step counter starts at the current step, so
 * the job follows the same trajectory as alone in a context of its own with
 * the same seed and stream; init_velocities != 0 draws its velocities as
 * that context's first sis_gpu_init_velocities would, else they are zero.
 * The slot's lists are rebuilt before returning. */
int sis_gpu_load_slot(sis_ctx *ctx, int32_t inst, int32_t n_chains, const int32_t *chain_len, const int32_t *chain_moltype,
                      const int32_t *seq, const uint8_t *has_charge, double tempK, double ionic_strength, uint32_t stream,
                      const double *xyz, int32_t init_velocities);

/* No counterpart in the reference.  sis_gpu_step with host noise (same
 * layout: nsteps x nmp x 3 doubles, step-major), but allocating nothing: it
 * stages one step's noise at a time through a fixed static device buffer
 * of 65,536 beads (1.5 MiB), where sis_gpu_step grows a per-context buffer
 * with cudaMalloc/cudaFree when a call needs more than the last one.
 * Callers that cannot allocate are those whose device memory is already
 * handed out by a fixed budget (a long job that must not fail with an
 * out-of-memory error midway), and those that must not stall other work on
 * the device: cudaFree waits for the whole device, including other
 * contexts' and other threads' work in flight.  Contexts of more than
 * 65,536 beads get SIS_ERR_ARG and a message.  The first call on a device
 * looks the buffer's address up (cudaGetSymbolAddress); the buffer is shared
 * by all contexts on that device, so calls must not overlap in time. */
int sis_gpu_step_noise_static(sis_ctx *ctx, int64_t nsteps, const double *noise);

#ifdef __cplusplus
}
#endif
#endif
