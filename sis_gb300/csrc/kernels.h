// Kernel launchers of libsisgpu (host side declarations).
#pragma once

#include "common.cuh"

namespace sisg {

// buckets of small instances for k_md_small: bucket b holds the instances
// inst[cta_off[b] .. cta_off[b+1]); cap: beads of the largest bucket;
// sslot: the bonded slot planes in shared memory (set by launch_md_small);
// inner: some instance has kInnerMinBeads beads or more (pair forces over
// inner lists, kernels.cu)
constexpr int kSmallMaxInst = 128;
constexpr int kSmallMaxBeads = 2048;
constexpr int kInnerMinBeads = 256;
// dynamic shared memory of a k_md_small block with the slot planes at most
// (its static shared memory, about 16 KB, comes on top, within the 227 KB
// of a block)
constexpr int kSmallDynMax = 204 * 1024;
struct SmallPlan {
    const int *cta_off;
    const int *inst;
    int n_cta, cap, sslot, inner;
};

struct RebuildPlan {
    const int2 *small_items; // device: (instance, first local bead), 32 beads per item
    int n_small_items, small_grid;
    const int2 *large_items; // device: (instance, first local bead), 256 beads per item
    int n_large_items, large_grid;
};

// device tables of a replica-exchange run (remd.cu)
struct RemdDev {
    InstP *ip;            // the context's instance records (written on a swap)
    InstP *ip2;           // [n_inst] the same records at the partner label's temperature
    const InstP *lab_ip;  // [n_labels] records whose temperature fields are each label's
    double *ene2;         // [n_inst][12] energies at the partner temperature
    int *rep2lab, *lab2rep;
    int *changed;         // [n_inst] 0 kept, 1 velocities times vscale, 2 velocities over vscale
    double *vscale;       // [n_inst]
    int *n_acc;           // [1] accepted swaps of the last exchange
    const double *lab_w;  // [n_labels][n_local] noise coefficient per label and local bead
    int n_local;          // beads per replica
    float *dgf;           // the context's FP32 triplet table [n_inst][469]
    const float *lab_dgf; // [n_labels][469]
};

// trigger != 0: the step kernel's last block decides the displacement trigger
// and advances the step counter (off only in timing passes)
cudaError_t launch_step(int G, const Dev &D, const GlobP &g, int cur, const double *noise, long long noise_step, cudaStream_t st,
                        int trigger);
cudaError_t launch_force(int G, const Dev &D, const GlobP &g, int cur, double *fout, int mask, cudaStream_t st);
int force_kernels(const GlobP &g, int mask); // kernels launch_force launches
// the step split in two: pair forces of every bead into fpair, then the step proper
cudaError_t launch_pairs(int G, const Dev &D, const GlobP &g, int cur, cudaStream_t st);
cudaError_t launch_step_split(int G, const Dev &D, const GlobP &g, int cur, const double *noise, long long ns, cudaStream_t st,
                              int trigger);
cudaError_t launch_pre(const Dev &D, const GlobP &g, int cur, int do_bonded, int do_bp, int test_blocks, int eval_blocks,
                       cudaStream_t st);
int pre_kernels(const GlobP &g, int do_bonded, int do_bp);
cudaError_t launch_bonded(const Dev &D, const GlobP &g, int cur, cudaStream_t st);
// the bonded pass of a step: slot planes (FP64 path) or per-bead forces (fbond, mixed path)
cudaError_t launch_bonded_step(const Dev &D, const GlobP &g, int cur, cudaStream_t st);
// k_bp_test and k_bp_eval
cudaError_t launch_bp(const Dev &D, const GlobP &g, int cur, int test_blocks, int eval_blocks, cudaStream_t st);
int bp_kernels(const GlobP &g);
cudaError_t launch_bp_energy(const Dev &D, const GlobP &g, int cur, double tK, int bp_blocks, cudaStream_t st);
// base-pair Monte Carlo removal of every instance whose pass is due (no-op without it)
cudaError_t launch_bp_mc(const Dev &D, const GlobP &g, cudaStream_t st);
cudaError_t launch_remd_partner_ip(const Dev &D, const RemdDev &R, int n_inst, int parity, cudaStream_t st);
cudaError_t launch_remd_decide(const Dev &D, const RemdDev &R, const GlobP &g, int parity, const double *u, double kB,
                               unsigned long long ctr, cudaStream_t st);
cudaError_t launch_energy(const Dev &D, const GlobP &g, int cur, cudaStream_t st);
// nsteps mixed-path MD steps of every instance in one launch (k_md_small);
// then the cluster lists of the instances it rebuilt (launch_cluster_flagged)
// and launch_small_finish
cudaError_t launch_md_small(const Dev &D, const GlobP &g, int cur, const SmallPlan &sp, int nsteps, const double *noise, int threads,
                            cudaStream_t st);
// dynamic shared memory of a k_md_small block for buckets of cap beads
size_t small_smem_bytes(int cap);
cudaError_t launch_cluster_flagged(const Dev &D, const GlobP &g, cudaStream_t st);
cudaError_t launch_small_finish(const Dev &D, const GlobP &g, unsigned long long nsteps, cudaStream_t st);
cudaError_t launch_rg(const Dev &D, const GlobP &g, int cur, double *out, cudaStream_t st);
// the optional terms' forces into fbp (in_step 1 inside a step, 0 outside)
// and their energies into slots 7-10; nothing when none is on
cudaError_t launch_bias(const Dev &D, const GlobP &g, int cur, int in_step, cudaStream_t st);
int bias_kernels(const GlobP &g);
cudaError_t launch_bias_energy(const Dev &D, const GlobP &g, int cur, cudaStream_t st);
cudaError_t launch_init_velocities(const Dev &D, const GlobP &g, unsigned long long ctr, cudaStream_t st, int only_inst = -1);
cudaError_t launch_mirror(const Dev &D, const GlobP &g, int cur, cudaStream_t st);
// k_trigger_rebuild, one cooperative launch of `grid` blocks (at most
// coop_blocks_per_sm() per SM, and at most kMaxCoopBlocks): after_step, the
// the rebuild of the flagged instances (flagged by the step kernel's trigger
// or by the host); returns at once when none is flagged
cudaError_t launch_rebuild(const Dev &D, const GlobP &g, int cur, const RebuildPlan &pl, int grid, cudaStream_t st);
int coop_blocks_per_sm();
// the grid barrier with block `absent` missing (a self-test of its timeout)
cudaError_t launch_barrier_probe(const Dev &D, int grid, int absent, cudaStream_t st);

} // namespace sisg
