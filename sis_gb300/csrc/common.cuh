// Internal device structures and helpers of libsisgpu (SIS hot path on sm_103a).
//
// Device data layout (n = beads of all instances, flat, instance-major):
//   x[2]      double4   FP64 positions, double-buffered across steps (w unused)
//   mir[2]    uint4     fixed-point mirror of x: per component llrint(x*S) mod 2^32;
//                       the int32 difference of two mirrors is the exact
//                       minimum-image separation in units of 1/S (PBC: S = 2^32/L,
//                       so the box maps onto the 32-bit ring; no PBC: S = 2^20/A)
//   res[2]    float4    residual x*S - llrint(x*S) of each mirror component, for
//                       the rare nearly-collinear terms that need separations
//                       beyond the mirror's resolution
//   v, beta   double4   velocities and GJF-2GJ noise term (reference: velos, accels)
//   move      double4   displacement since the last rebuild (reference: xyz_move)
//   mdc       double4   per-bead integrator coefficients (a, sqrt(b)h/m, sqrt(b)h, noise)
//   fbp       double4   base-pair forces of the current step (atomic scatter
//                       target): FP64 values in the FP64 path; in the mixed path
//                       the same words hold int64 fixed point (units of 2^-32
//                       kcal/mol/A), so that the sum is exact and independent
//                       of the order in which records arrive
//   binfo     int4      (instance, chain start, chain length | circ<<31,
//                        local index | seq<<24 | charge<<28)
//   nbr       int32     per-bead pair list, stride cap: j | WCA<<31 | ELE<<30
//   nnbr      int32     entries per bead
//   cl_*                cluster-pair lists of the mixed path's pair kernel: an
//                       i-cluster is 8 consecutive beads of one instance
//                       (local beads 8c .. 8c+7); for each, the j-clusters
//                       holding its pair-list partners in ascending order, as
//                       the j-cluster's first bead and two 64-bit masks (bit
//                       8a+b: i-bead a with j-bead b is a WCA / an electrostatic
//                       pair of the reference's lists)
//   mir0      uint4     mirror at the last list rebuild (mixed path): the
//                       displacement of the rebuild trigger is the exact
//                       integer difference of the current mirror and this one
//   bps/bps_n int4      base-pair candidates in per-instance segments:
//                       (i, j, type|hash<<8, inst) and neighbour beads
//                       (i-1, j-1, i+1, j+1); a prefix over instance counts
//                       maps a global record index to its segment slot
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace sisg {

constexpr int WCA_BIT = 1 << 31;
constexpr int ELE_BIT = 1 << 30;
constexpr int IDX_MASK = (1 << 30) - 1;
constexpr int MAX_BP_TYPES = 7;

// error flag bits
constexpr int ERR_PAIR_OVERFLOW = 1;
constexpr int ERR_BP_OVERFLOW = 2;
constexpr int ERR_NONFINITE = 4;
constexpr int ERR_TIMEOUT = 8; // a grid barrier wait of k_trigger_rebuild ran out
constexpr int kMaxCoopBlocks = 4096;
// cluster-pair lists: beads per cluster, the per-warp hash table of the
// conversion from per-bead lists, and the largest j-cluster count per i-cluster
constexpr int kCl = 8;
constexpr int kClHash = 512;
constexpr int kClCapMax = 256;

// Fixed-point base-pair force accumulation of the mixed path: one unit is
// 2^-32 kcal/mol/A; contributions of magnitude 2^30 or more are reported as
// non-finite (no physical step survives such a force).
constexpr float FX_LIMIT = 1073741824.0f;
constexpr double FX_UNIT = 1.0 / 4294967296.0;

// round(v * 2^32) for |v| < 2^30 from FP32 and 32-bit integer operations:
// a = v*2^32 is exact; h = trunc(a/2^31) and l = a - h*2^31 are exact, and
// l is rounded to an integer only when |a| < 2^31 (then h = 0).
__device__ __forceinline__ long long fx_of(float v) {
    const float a = v * 4294967296.0f;
    const float h = truncf(a * 4.656612873077392578125e-10f);
    const float l = fmaf(h, -2147483648.0f, a);
    return (long long)__float2int_rz(h) * 2147483648LL + (long long)__float2int_rn(l);
}
__device__ __forceinline__ long long fx_of(double v) { return __double2ll_rn(v * 4294967296.0); }
// exact, order-independent addition of a fixed-point force to bead i
__device__ __forceinline__ void fx_scatter(double4 *fbp, int i, long long fx, long long fy, long long fz) {
    unsigned long long *p = reinterpret_cast<unsigned long long *>(fbp + i);
    atomicAdd(p + 0, (unsigned long long)fx);
    atomicAdd(p + 1, (unsigned long long)fy);
    atomicAdd(p + 2, (unsigned long long)fz);
}
// the fixed-point word as FP32 kcal/mol/A from 32-bit conversions only
// (the high word scaled exactly, the low word rounded once)
__device__ __forceinline__ float fx_float(double word) {
    const long long w = __double_as_longlong(word);
    return fmaf((float)(int)(w >> 32), 1.0f, (float)(unsigned int)w * 2.3283064365386963e-10f);
}
__device__ __forceinline__ double fx_value(double word) { return (double)__double_as_longlong(word) * FX_UNIT; }

struct InstP {
    double box[3];     // PBC box (0 when pbc == 0)
    double half[3];    // box / 2
    double fsc[3];     // fixed-point scale, units per Angstrom
    float finv[3];     // Angstrom per unit
    int pbc;
    int bead_off, n;   // beads [bead_off, bead_off + n)
    int n_act;         // the first n_act of them move; the rest are inert fillers of a slot (sis_gpu_load_slot)
    int cl_off;        // first i-cluster of the instance
    int bp_off, bp_cap;// base-pair staging segment
    double tempK;
    double ele_coef, rcdist, ele_cut, ele_cut2, diele_dTcoef;
    double diele;      // dielectric constant the electrostatic fields were set with
    float ele_coef_f, rcdist_f, ele_cut2_f;
    double wca_nl_cut2, ele_nl_cut2, bp_nl_cut2;
    // cell grid of large PBC instances (large == 0: all-pairs scan)
    int large, cell_base, nc[3];
    double cell_len[3];
    // noise stream of the instance: Philox counter (local bead, step - step0, stream)
    unsigned int stream;
    unsigned long long step0;
    // Rg bias (force_rg.F90): rg_pott 0 off, 1 harmonic, 2 flat-bottomed
    int rg_pott;
    double rg_k, rg0;
    // magnitude of the constant-force trap pairs (kind 3 items carry the force
    // per unit of it; 1 unless the force is a replica-exchange variable,
    // energy_replica.F90:105-107 twz_DCF_forces = value * direction)
    double twz_scale;
    // base pairs only between the pairs of a given secondary structure
    // (read_ss.F90 bp_map): their records come from the partner table ss_*
    int ss_on;
};

struct GlobP {
    int n, n_inst, cap, prec, integrator;
    int n_cl, ccap; // i-clusters of all instances; j-cluster slots per i-cluster
    int angl_reb, dih_type, bp_model, flg_ele, temp_indep;
    int bp_min_loop, bp_jnext_compat, ele_excl_bond, ele_excl_angle;
    double bond_k, bond_r0, angl_k, angl_t0, cos_t0, dih_k, dih_w, dih_p0;
    double wca_sigma, wca_eps, wca_sig2, wca_coef;
    double bp_cutoff_energy, nl_margin;
    float f_bp_cutoff_energy;
    float f_bond_k, f_bond_r0, f_angl_k, f_angl_t0, f_cos_t0, f_dih_k, f_dih_w, f_dih_p0;
    float f_wca_sig2, f_wca_coef, f_wca_sigma, f_wca_eps;
    unsigned long long seed;
    double fcap; // > 0: per-bead force magnitude cap (equilibration only)
    float fcap_f; // the same in FP32 (the mixed path)
    int nstep_mc, max_bp_per_nt; // base-pair Monte Carlo removal (0: none)
    // optional terms (force.F90:62-75): any of them on; stage wall; an Rg
    // bias on some instance; restraint and trap items
    int flg_bias, flg_stage, flg_rg, n_bias;
    double stage_sigma, stage_eps;
    // [Bias_SS] (force_bp_triplet.F90:85-92): a constant pull of an allowed
    // pair outside its distance window; any_ss: some instance has a structure
    int flg_bias_ss, any_ss;
    double bias_ss_force;
};

// One sigmoid restraint or tweezers trap pair (force_restraint.F90,
// force_tweezers.F90).  kind 1: restraint on both beads; 2: restraint on bead
// i only (the reference's Sigmoid-to-bead); 3: constant-force trap pair;
// 4: force-ramp trap pair.  p: 1, 2 eps, d, s, rcut; 3 the force on bead i
// (x, y, z); 4 k_i, k_j, trap starts (i x y z, j x y z), trap velocities
// (i x y z, j x y z).
struct BiasItem {
    int kind, i, j, inst; // global bead indices
    double p[14];
};

// base-pair parameter record (var_potential.F90 basepair_parameters), index 1..6
struct BPP {
    double cutoff_ddist, U0, bond_k, bond_r;
    double angl_k[4], angl_theta[4];
    double dihd_k[2], dihd_phi[2];
};

// FP32 copy of BPP for the mixed path, plus the squared distance window
// (bond_r -+ cutoff_ddist)^2 of the early rejection test
struct BPPf {
    float cutoff_ddist, U0, bond_k, bond_r;
    float angl_k[4], angl_theta[4];
    float dihd_k[2], dihd_phi[2];
    float lo2, hi2;
};

// all device pointers of one context (passed by value to kernels)
struct Dev {
    double4 *x[2];
    uint4 *mir[2];
    float4 *res[2];         // mirror residuals x*S - q (units), w unused
    double4 *v, *beta, *move, *mdc, *fbp;
    int4 *binfo;
    // optional terms: restraint and trap items; per instance the Rg bias
    // centre and force factor, and its energy
    const BiasItem *bias;
    double4 *rgb;
    double *rgv;
    double *mass;
    int *nbr, *nnbr;
    // cluster-pair lists (mixed path): per i-cluster its first bead, its
    // j-cluster count (-1: more than ccap, the pair kernel then walks the
    // per-bead lists of its beads), and ccap slots of (j-cluster first bead,
    // WCA mask, electrostatic mask)
    int *cl_first, *ncl, *cl_j;
    ulonglong2 *cl_m;
    uint4 *mir0;            // [n] mirror at the last rebuild (mixed path)
    // inner pair lists of the per-block kernel (contexts of small instances):
    // each bead's list entries within their cutoff + kInnerMargin at the last
    // refresh, in list order, and the mirror at that refresh; per instance
    // the list rebuilds so far (lgen, counted by every rebuild path) and the
    // rebuild count the inner lists were filtered from (igen)
    int *nbr_in, *nnbr_in;
    uint4 *mir_in;
    int *lgen, *igen;
    // base-pair lists
    int4 *bps, *bps_n;      // per-instance staging segments (records, neighbour beads)
    int *bp_cnt;            // [2*n_inst] staging counts, then their exclusive prefix
    int *bp_total;          // [1] records over all instances
    double *ene_bp;         // per staging slot
    unsigned char *bp_status;
    int *bp_win;            // [staging slots] records inside the distance window this step
    int *bp_nwin;           // [1] their count
    int *bp_fixq;           // [staging slots] records the FP32 pass left to the FP64 one
    int *bp_fixn;           // [1] their count
    const BPP *bpp;         // [7]
    const BPPf *bppf;       // [7]
    void *slot;             // [8][n] bonded forces per term start (float4 or double4)
    void *fpair;            // [n] pair forces of the current step (float4 or double4)
    float4 *fbond;          // [n] mixed path: bonded force of the current step per bead (k_bonded_bead)
    const short *bp3_hash;  // [4097]
    const double *bp3_dH, *bp3_dS; // [469]
    const float *bp_dgf;    // [n_inst][469] FP32 dH - T dS at each instance's
                            // temperature; its sign equals that of the FP64 value
    const InstP *ip;
    // rebuild trigger
    unsigned long long *m1, *m2; // [2][n_inst] top-2 displacement^2 (bit patterns), by step parity
    int *flag;              // [n_inst] rebuild requested
    int *any;               // [1] any flag set
    unsigned int *ticket;   // [3] last-block tickets (step kernel's trigger, unused, base-pair evaluation)
    unsigned int *gbar;     // [2] grid barrier of k_trigger_rebuild: arrivals, generation
    int *gsum;              // [kMaxCoopBlocks] per-block sums of the cell scan
    unsigned long long *step_ctr; // [1] Philox step counter
    int *err;               // [1] error flags
    int *max_need;          // [2] largest pair / bp count seen
    long long *rebuilds;    // [2] instance rebuilds, rebuild passes run by step graphs
    unsigned long long *capped; // [1] bead-steps at which the force cap bound
    // cell lists of large PBC instances
    int *bead_cell, *cell_cnt, *cell_start, *cell_beads;
    int n_cells;
    // energies [n_inst][12] (slots 0..10 + kinetic)
    double *ene;
    // base-pair Monte Carlo removal (force_bp_limit_triplet.F90)
    unsigned char *bp_mask; // per staging slot: survived the last Monte Carlo pass (bp_status_MC)
    long long *bp_frec;     // [slot][18] energy-scaled forces of the 6 beads (fixed point, or FP64 bits)
    int *mc_due;            // [n_inst] the next base-pair evaluation runs the Monte Carlo pass
    int *mc_excess;         // [n] pairs per nucleotide minus max_bp_per_nt
    int *mc_list;           // [n] scratch: nucleotides with excess
    int *mc_seq;            // [staging slots] scratch: pairs of the chosen nucleotide
    unsigned long long *mc_calls; // [n_inst] Monte Carlo passes (Philox counter)
    const double *mc_draws; // caller-supplied uniforms for the next pass, or NULL (Philox)
    int *mc_draw_pos;       // [1] next caller-supplied uniform
    int mc_n_draws;
    // secondary-structure partners: bead i's allowed partners (global bead
    // indices, ascending) are ss_part[ss_start[i] .. ss_start[i+1])
    const int *ss_start, *ss_part;
};

// buffer `cur` of the double-buffered arrays, as a select rather than an
// indexed load, so that a copy of Dev made inside a kernel stays in registers
__device__ __forceinline__ uint4 *mir_at(const Dev &D, int cur) { return cur ? D.mir[1] : D.mir[0]; }
__device__ __forceinline__ float4 *res_at(const Dev &D, int cur) { return cur ? D.res[1] : D.res[0]; }
__device__ __forceinline__ double4 *x_at(const Dev &D, int cur) { return cur ? D.x[1] : D.x[0]; }

// ----------------------------------------------------------------- vectors
template <typename R> struct V3 {
    R x, y, z;
};
template <typename R> __device__ __forceinline__ V3<R> mk(R a, R b, R c) { return V3<R>{a, b, c}; }
template <typename R> __device__ __forceinline__ R dot3(const V3<R> &a, const V3<R> &b) {
    return a.x * b.x + a.y * b.y + a.z * b.z;
}
template <typename R> __device__ __forceinline__ V3<R> cross3(const V3<R> &a, const V3<R> &b) {
    return mk<R>(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
template <typename R> __device__ __forceinline__ V3<R> operator+(V3<R> a, V3<R> b) { return mk<R>(a.x + b.x, a.y + b.y, a.z + b.z); }
template <typename R> __device__ __forceinline__ V3<R> operator-(V3<R> a, V3<R> b) { return mk<R>(a.x - b.x, a.y - b.y, a.z - b.z); }
template <typename R> __device__ __forceinline__ V3<R> operator*(R s, V3<R> a) { return mk<R>(s * a.x, s * a.y, s * a.z); }
template <typename R> __device__ __forceinline__ V3<R> operator-(V3<R> a) { return mk<R>(-a.x, -a.y, -a.z); }

// ------------------------------------------------------- relative position
// FP64: the reference's pbc_vec_d (pbc.F90:140-165), single shift.
__device__ __forceinline__ V3<double> dvec64(const double4 &a, const double4 &b, const InstP &ip) {
    V3<double> v = mk<double>(a.x - b.x, a.y - b.y, a.z - b.z);
    if (ip.pbc) {
        if (v.x > ip.half[0]) v.x = v.x - ip.box[0];
        else if (v.x < -ip.half[0]) v.x = v.x + ip.box[0];
        if (v.y > ip.half[1]) v.y = v.y - ip.box[1];
        else if (v.y < -ip.half[1]) v.y = v.y + ip.box[1];
        if (v.z > ip.half[2]) v.z = v.z - ip.box[2];
        else if (v.z < -ip.half[2]) v.z = v.z + ip.box[2];
    }
    return v;
}
// FP32: from the fixed-point mirror; the wrap of the 32-bit difference is the
// minimum image for PBC instances.
__device__ __forceinline__ V3<float> dvec32(const uint4 &a, const uint4 &b, const InstP &ip) {
    return mk<float>((float)(int)(a.x - b.x) * ip.finv[0], (float)(int)(a.y - b.y) * ip.finv[1],
                     (float)(int)(a.z - b.z) * ip.finv[2]);
}

template <typename R> struct Pos;
template <> struct Pos<double> {
    const double4 *x;
    __device__ __forceinline__ V3<double> d(int a, int b, const InstP &ip) const { return dvec64(x[a], x[b], ip); }
};
template <> struct Pos<float> {
    const uint4 *m;
    __device__ __forceinline__ V3<float> d(int a, int b, const InstP &ip) const { return dvec32(m[a], m[b], ip); }
};

// Mirror component q = round(x*S) mod 2^32 and the residual x*S - q (units of
// 1/S, |r| <= 1/2) that the mirror drops, with one FP64 operation: the
// fused x*S + M, M = 1.5 * 2^40, leaves round(x*S * 2^12) + 2^51 in the low
// 52 mantissa bits of the sum (valid for |x*S| < 2^39), so the integer part
// and the residual (to 2^-12 units) follow from integer arithmetic.  q
// rounds x*S half up after it has been rounded to 2^-12 units; every mirror
// of the library comes from this function, so all agree.  Returns false
// when x*S is out of range or not finite (then q and r are meaningless).
__device__ __forceinline__ bool fixed_mirror(double x, double s, unsigned int &q, float &r) {
    const double u = __fma_rn(x, s, 1649267441664.0); // 1.5 * 2^40
    const long long b = __double_as_longlong(u);
    const long long w = (b & 0xFFFFFFFFFFFFFLL) - (1LL << 51);  // round(t * 2^12)
    const long long qq = (w + 2048) >> 12;
    q = (unsigned int)(unsigned long long)qq;
    r = (float)(int)(w - (qq << 12)) * 0.000244140625f;
    return (b >> 52) == 0x427; // exponent of [2^40, 2^41): |t| < 2^39 and finite
}
__device__ __forceinline__ unsigned int fixed_res(double x, double s, float &r) {
    unsigned int q;
    fixed_mirror(x, s, q, r);
    return q;
}

// 1/d: the hardware approximation refined by one Newton-Raphson step
// (r1 = r0 + r0 (1 - d r0)), within an ulp or so of the rounded quotient
__device__ __forceinline__ float rcp_nr(float d) {
    float r0;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r0) : "f"(d));
    return __fmaf_rn(r0, __fmaf_rn(-d, r0, 1.f), r0);
}

// The displacement trigger of instance k (job_md.F90:376-395): the two
// largest squared displacements since the last rebuild (FP64 bit patterns,
// merged with integer atomics) move the instance by more than the list margin.
__device__ __forceinline__ bool trigger_fires(const GlobP &g, const unsigned long long *m1, const unsigned long long *m2, int k) {
    const double a = __longlong_as_double((long long)__ldcg(m1 + k));
    const double b = __longlong_as_double((long long)__ldcg(m2 + k));
    return sqrt(a) + sqrt(b) > g.nl_margin;
}

// A separation in fixed-point units: the exact mirror difference d (int32,
// the minimum image under PBC) and the residual difference (FP32).
struct FxV {
    int x, y, z;
    float rx, ry, rz;
};
__device__ __forceinline__ FxV fxv(const uint4 *m, const float4 *r, int i, int j) {
    const uint4 a = m[i], b = m[j];
    const float4 ra = r[i], rb = r[j];
    return FxV{(int)(a.x - b.x), (int)(a.y - b.y), (int)(a.z - b.z), ra.x - rb.x, ra.y - rb.y, ra.z - rb.z};
}
// a x b in A^2: the product of the mirror differences is exact in int64 and
// rounded once to FP32; the first-order residual terms are added in FP32
// (the second-order term is below 1 unit^2).  Accurate to a few FP32 ulps of
// |a x b| however nearly parallel a and b are, unlike a cross product of
// FP32 separation vectors, which inherits their ~1e-7 relative rounding.
__device__ __forceinline__ V3<float> cross_fx(const FxV &a, const FxV &b, const InstP &ip) {
    const float ax = (float)a.x, ay = (float)a.y, az = (float)a.z, bx = (float)b.x, by = (float)b.y, bz = (float)b.z;
    const float cx = (float)((long long)a.y * b.z - (long long)a.z * b.y) + ((ay * b.rz - az * b.ry) + (a.ry * bz - a.rz * by));
    const float cy = (float)((long long)a.z * b.x - (long long)a.x * b.z) + ((az * b.rx - ax * b.rz) + (a.rz * bx - a.rx * bz));
    const float cz = (float)((long long)a.x * b.y - (long long)a.y * b.x) + ((ax * b.ry - ay * b.rx) + (a.rx * by - a.ry * bx));
    return mk<float>(cx * (ip.finv[1] * ip.finv[2]), cy * (ip.finv[2] * ip.finv[0]), cz * (ip.finv[0] * ip.finv[1]));
}

// -------------------------------------------------------- bead information
__device__ __forceinline__ int bi_inst(const int4 &b) { return b.x; }
__device__ __forceinline__ int bi_cstart(const int4 &b) { return b.y; }
__device__ __forceinline__ int bi_clen(const int4 &b) { return b.z & 0x7fffffff; }
__device__ __forceinline__ bool bi_circ(const int4 &b) { return (b.z >> 31) & 1; }
__device__ __forceinline__ int bi_lidx(const int4 &b) { return b.w & 0xffffff; }
__device__ __forceinline__ int bi_seq(const int4 &b) { return (b.w >> 24) & 0xf; }
__device__ __forceinline__ bool bi_charge(const int4 &b) { return (b.w >> 28) & 1; }

// bead of local index k of the chain (modular for circular chains); -1 if none
__device__ __forceinline__ int chain_bead(const int4 &b, int k) {
    const int n = bi_clen(b);
    if (bi_circ(b)) {
        k %= n;
        if (k < 0) k += n;
        return bi_cstart(b) + k;
    }
    return (k >= 0 && k < n) ? bi_cstart(b) + k : -1;
}

// ------------------------------------------------------------------ Philox
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11), written from the paper.
__device__ __forceinline__ uint4 philox4x32_10(uint4 c, uint2 k) {
    const unsigned int M0 = 0xD2511F53u, M1 = 0xCD9E8D57u, W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        const unsigned int hi0 = __umulhi(M0, c.x), lo0 = M0 * c.x;
        const unsigned int hi1 = __umulhi(M1, c.z), lo1 = M1 * c.z;
        c = make_uint4(hi1 ^ c.y ^ k.x, lo1, hi0 ^ c.w ^ k.y, lo0);
        k.x += W0;
        k.y += W1;
    }
    return c;
}

} // namespace sisg
