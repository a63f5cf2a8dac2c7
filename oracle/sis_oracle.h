/*
 * sis_oracle.h -- CPU FP64 restatement of the SIS (Hori-Lab/SIS) force and
 * integration hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the correctness oracle and the
 * timed CPU baseline.  Only tests/, __graft_entry__.smoke() and bench.py's
 * CPU-baseline / reference arm may load it.  The product path (libsisgpu.so)
 * never links, loads or calls it.
 *
 * The reference is Fortran and cannot be compiled in this environment (no
 * Fortran compiler, toml-f submodule not vendored), so this file restates its
 * algorithms in C++, routine by routine, each citing the Fortran source it
 * follows.  Arrays keep the reference's layouts: xyz(3,nmp) per replica,
 * pair lists (2,n), bp records (7,n) with 1-based bead indices.
 */
#ifndef SIS_ORACLE_H
#define SIS_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Parameters as read from the input TOML and the .ff file
 * (read_input.F90, read_force_field.F90).  Base-pair parameters are given for
 * the three types the .ff file holds (GC, AU, GU); CG/UA/UG are derived as
 * read_force_field.F90:203-258 does. */
typedef struct or_params {
    /* [potential.bond] */
    double bond_k, bond_r0;
    /* [potential.angle] or [potential.angle_ReB] */
    int32_t angl_reb;
    double angl_k, angl_t0;
    /* 0: no dihedral, 1: [potential.dihedral], 2: [potential.dihedral_exp] */
    int32_t dih_type;
    double dih_k, dih_w, dih_p0;
    /* [potential.wca] */
    double wca_sigma, wca_eps;
    /* [Basepair] */
    int32_t bp_model, bp_min_loop;
    /* 1: reproduce neighbor_list.F90:212 (jmp+1 tested against nmp_chain(ichain)) */
    int32_t bp_jnext_compat;
    double bp_cutoff_energy;
    /* index 0:GC 1:AU 2:GU ; 15 values each in this order:
     * U0 bond_k bond_r angl_k1..4 angl_theta1..4 dihd_k1 dihd_k2 dihd_phi1 dihd_phi2 */
    double bp_ff[3][15];
    double nn_dH[21], nn_dS[21], dH0, dS0;
    int32_t nnend;
    double nnend_dH[6], nnend_dS[6], dHend0, dSend0;
    /* [Electrostatic] */
    int32_t flg_ele, ele_cutoff_type;
    double ele_cutoff_inp, length_per_charge;
    int32_t ele_excl_bond, ele_excl_angle;
    int32_t temp_independent;
    double tempK_ref;
    /* [MD] */
    int32_t integrator; /* 1: GJF-2GJ, 2: Ermak-McCammon */
    double dt, viscosity_Pas, nl_margin;
    /* [Basepair] nstep_MC (0: no Monte Carlo removal), max_bp_per_nt */
    int32_t nstep_bp_mc, max_bp_per_nt;
} or_params;

typedef struct or_system or_system;

/* Topology: nchains chains, chain_len[c] beads each, moltype[c] 1=linear 2=circ,
 * seq[] concatenated (SEQT codes A=0 U=1 G=2 C=3 D=4), has_charge[] per bead.
 * nrep replicas with tempK[r], ionic_strength[r].  pbc_box NULL => no PBC. */
or_system *or_create(int32_t nchains, const int32_t *chain_len, const int32_t *moltype,
                     const int32_t *seq, const uint8_t *has_charge, int32_t nrep,
                     const double *tempK, const double *ionic_strength,
                     const double *pbc_box, const or_params *p);
void or_destroy(or_system *s);
int32_t or_nmp(const or_system *s);

/* state access, xyz(3,nmp) column-major == bead-major xyz triples */
void or_set_xyz(or_system *s, int32_t irep, const double *xyz);
void or_get_xyz(const or_system *s, int32_t irep, double *xyz);
void or_set_velos(or_system *s, int32_t irep, const double *v);
void or_get_velos(const or_system *s, int32_t irep, double *v);
void or_set_accels(or_system *s, int32_t irep, const double *a);
void or_get_accels(const or_system *s, int32_t irep, double *a);

/* neighbor_list.F90 (pbc_wrap + O(N^2) scan) */
void or_neighbor_list(or_system *s, int32_t irep);
/* kind 0: wca (2,n)  1: ele (2,n)  2: bp (7,n) ; returns count, copies min(count,cap) records */
int32_t or_get_list(const or_system *s, int32_t irep, int32_t kind, int32_t *out, int32_t cap);
/* bp_coef(2,n) of the current bp list */
int32_t or_get_bp_coef(const or_system *s, int32_t irep, double *out, int32_t cap);

/* force.F90: forces(3,nmp) */
void or_force(or_system *s, int32_t irep, double *forces);
/* per-term forces, term 1 bond 2 angl 3 dih 4 bp 5 wca 6 ele */
void or_force_term(or_system *s, int32_t irep, int32_t term, double *forces);
/* energy_sumup.F90: energies(0:10) */
void or_energy_sumup(or_system *s, int32_t irep, double tempK, double *energies);
double or_energy_kinetic(const or_system *s, int32_t irep);
double or_rg(const or_system *s, int32_t irep);
/* bp cache flag (flg_bp_energy) */
void or_set_bp_energy_flag(or_system *s, int32_t flag);
/* ene_bp / bp_status of the last force or energy call */
int32_t or_get_bp_state(const or_system *s, int32_t irep, double *ene, uint8_t *status, int32_t cap);

/* set_ele.F90 outputs for replica irep: [ele_coef, lambdaD, ele_cutoff, diele] */
void or_get_ele(const or_system *s, int32_t irep, double *out4);
/* set_md_coef (job_md.F90:700-767): per bead md_coef(1:3), md_coef_rep(1) */
void or_get_md_coef(const or_system *s, int32_t irep, double *out4xN);
/* bp parameters after init_bp: bp_paras(6) as 16 doubles each (cutoff_ddist first), bp_cutoff_dist */
void or_get_bp_paras(const or_system *s, double *out96, double *bp_cutoff_dist);
/* bp3_dH / bp3_dS (468 each) */
void or_get_bp3_tables(const or_system *s, double *dH, double *dS);
void or_set_temperature(or_system *s, int32_t irep, double tempK, double ionic_strength);

/* job_md.F90:360-460 time loop for all replicas: per step, displacement
 * trigger, neighbor_list, force, noise, GJF-2GJ / Ermak-McCammon update.
 * noise: NULL => rnd_boxmuller from the MT stream of each replica;
 *        else noise[step][irep][nmp][3] (reference's rnd_bm order).
 * Returns the number of neighbour-list rebuilds. */
int64_t or_run(or_system *s, int64_t nsteps, const double *noise);
/* initial list build as job_md.F90:196-198 does, and xyz_move reset */
void or_md_init(or_system *s);
void or_init_velocities(or_system *s);
/* step counter and rebuild counter */
int64_t or_nrebuild(const or_system *s);

/* MT19937 stream (mt_stream.F90) and polar Box-Muller (rnd_boxmuller.F90) */
typedef struct or_mt or_mt;
or_mt *or_mt_create(int32_t seed);
void or_mt_destroy(or_mt *m);
uint32_t or_mt_int32(or_mt *m);
double or_mt_double1(or_mt *m);
double or_mt_double3(or_mt *m);
double or_mt_boxmuller(or_mt *m);
/* seed the replica noise streams of a system from one scalar seed (stream 0 for replica 1, ...) */
void or_seed(or_system *s, int32_t seed);
/* the MT stream `base` jumped id * 2^jp outputs ahead (mt_create_stream) */
void or_mt_jump(or_mt *base, int32_t jp, int32_t id, or_mt *that);
/* replica streams as init_mts.F90 derives them from rng_seed */
void or_seed_streams(or_system *s, int32_t seed, int32_t replica_run);

/* physical constants (const_phys.F90) for cross-checks */
double or_const(int32_t which);

/* force_bp_limit_triplet.F90: forces with the base-pair Monte Carlo removal
 * (every record evaluated, then pairs deleted until no nucleotide carries
 * more than max_bp_per_nt); the draws it consumed from the replica's MT
 * stream are kept in order (or_get_mc_draws).  or_get_bp_status: the status
 * of every record of the last force evaluation. */
void or_force_mc(or_system *s, int32_t irep, double *forces);
int32_t or_get_mc_draws(const or_system *s, double *out, int32_t cap);
int32_t or_get_bp_status(const or_system *s, int32_t irep, uint8_t *out, int32_t cap);

/* Optional terms (force.F90:62-75, energy_sumup.F90:47-52), force term 7 and
 * energy slots 7-10.  Stage wall (force_stage.F90): sigma <= 0 turns it off.
 * Rg bias (force_rg.F90): pott 0 off, 1 harmonic, 2 flat-bottomed; rg0 per
 * replica.  Sigmoid restraints (force_restraint.F90): ids3 [n][3] = imp, jmp
 * (1-based), type (1 both beads, 2 subject only); para4 [n][4] = eps, d, s,
 * rcut.  Tweezers (force_tweezers.F90): dual-trap constant force pairs with
 * forces [nrep][ndcf][3], force-ramp pairs with k [nfr][2], trap starts and
 * velocities [nfr][2][3]; the ramps move with the step being taken. */
void or_set_stage(or_system *s, double sigma, double eps);
void or_set_rg_bias(or_system *s, int32_t pott, double k, const double *rg0);
void or_set_restraints(or_system *s, int32_t n, const int32_t *ids3, const double *para4);
void or_set_frozen(or_system *s, int32_t n, const int32_t *beads);
void or_set_tweezers(or_system *s, int32_t ndcf, const int32_t *dcf_pairs, const double *dcf_f, int32_t nfr,
                     const int32_t *fr_pairs, const double *fr_k, const double *fr_init, const double *fr_velo);

#ifdef __cplusplus
}
#endif
#endif
