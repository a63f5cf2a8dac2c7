// libsisgpu host side: context, set-up derivations and the C ABI of
// include/sis_gpu.h.
//
// Set-up restates, for the device tables, the reference's init_bp
// (cutoff_ddist, bp_cutoff_dist, the NN triplet table), set_ele (dielectric
// constant, Bjerrum length, ele_coef, Debye length), list_local (the bonded
// topology, here implicit in the per-bead chain information) and the
// friction / mass / GJF-2GJ coefficients of job_md.
#include <cuda_runtime.h>
#include <math.h>
#include <string.h>

#include <algorithm>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/sis_gpu.h"
#include "common.cuh"
#include "kernels.h"

using namespace sisg;

namespace {

// const_phys.F90:5-13
const double PI = 4.0 * atan(1.0);
const double EPS0 = 8.8541878128e-12;
const double ELE = 1.602176634e-19;
const double BOLTZ_J = 1.380649e-23;
const double N_AVO = 6.02214076e23;
const double KCAL2JOUL = 4184.0;
const double JOUL2KCAL_MOL = (1.0 / KCAL2JOUL) * N_AVO;
const double BOLTZ_KCAL_MOL = BOLTZ_J * JOUL2KCAL_MOL;

constexpr int kAllPairsMax = 4096;
constexpr int kEvents = 16;

bool is_comp(int a, int b) {
    return (a == 0 && b == 1) || (a == 1 && (b == 0 || b == 2)) || (a == 2 && (b == 3 || b == 1)) || (a == 3 && b == 2);
}

// NNT index (1..21) of the stack 5'-ij-3'/3'-kl-5' (const_idx.F90 char2nnt, with its aliases)
int nnt_index(int i, int j, int k, int l) {
    static const char C[4] = {'A', 'U', 'G', 'C'};
    static const char *canon[21] = {"GC_CG", "CC_GG", "GA_CU", "CG_GC", "AC_UG", "CA_GU", "AG_UC", "UA_AU", "AU_UA", "AA_UU", "GC_UG",
                                    "CU_GG", "GG_CU", "CG_GU", "AU_UG", "GA_UU", "UG_GU", "UA_GU", "GG_UU", "GU_UG", "AG_UU"};
    static const char *alias[21] = {"",      "GG_CC", "UC_AG", "",      "GU_CA", "UG_AC", "CU_GA", "",      "",      "UU_AA", "GU_CG",
                                    "GG_UC", "UC_GG", "UG_GC", "GU_UA", "UU_AG", "",      "UG_AU", "UU_GG", "",      "UU_GA"};
    char s[6] = {C[i], C[j], '_', C[k], C[l], 0};
    for (int n = 0; n < 21; ++n)
        if (!strcmp(s, canon[n]) || (alias[n][0] && !strcmp(s, alias[n]))) return n + 1;
    return 0;
}

} // namespace

struct sis_ctx {
    int dev = 0; // the CUDA device the context was created on; every entry point runs with it current
    Dev D{};
    GlobP g{};
    sis_params p{};
    int n = 0, n_inst = 0, cur = 0, G = 8;
    int bpb = 2 * 152; // blocks of k_bp_eval and k_bp_energy: two per SM (set from the device at creation)
    int bpt = 8 * 152; // blocks of k_bp_test: the staging capacity, at most eight per SM
    int coop_grid = 0;  // blocks of the cooperative trigger/rebuild kernel (set at creation)
    std::vector<InstP> ip;
    std::vector<int4> binfo;
    std::vector<int> seq;
    std::vector<double> mass;
    std::vector<uint8_t> frozen; // [Freeze] per bead (empty: none)
    std::vector<double> fric;
    std::vector<double> ionic;
    InstP *ip_d = nullptr;
    BPP bpp[MAX_BP_TYPES]{};
    double bp_cutoff_dist = 0.0;
    std::vector<double> bp3_dH, bp3_dS; // triplet free-energy tables [469]
    std::vector<float> dgf;             // [n_inst][469] FP32 dH - T dS
    float *dgf_d = nullptr;
    RebuildPlan plan{};
    int2 *items_d = nullptr;
    cudaStream_t st = nullptr;
    cudaEvent_t ev[kEvents]{};
    bool lists_valid = false, state_set = false, bp_cache = false;
    // instances loaded by sis_gpu_load_slot whose lists the next per-block
    // kernel launch rebuilds (flag set on the device)
    bool stale_lists = false;
    long long launches = 0, steps = 0;
    std::string err;
    double *noise_d = nullptr;
    size_t noise_cap = 0;
    double *fout_d = nullptr;
    void *flush_d = nullptr;
    size_t flush_bytes = 0;
    std::vector<void *> allocs;
    double4 *pin = nullptr; // pinned staging buffer for state transfers (n double4)
    // steady-state step graph (kGraphSteps steps, each ending with the
    // cooperative trigger/rebuild kernel) and the parameters it was captured with
    cudaGraphExec_t gexec = nullptr;
    int graph_cur = -1, graph_G = 0, graph_bpb = 0;
    bool graph_overlap = false;
    GlobP graph_g{};
    bool use_graphs = true;
    // overlap: the step's pair forces (k_pairs) run on st3 concurrently with
    // the bonded and base-pair pass; fork/join events.  overlap_mode -1: the
    // autotuner chooses it with the lanes (until then off); 0 or 1: fixed.
    bool overlap = false;
    int overlap_mode = -1;
    bool lanes_fixed = false;
    cudaStream_t st3 = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    // k_bonded runs on st4 beside the base-pair kernels on st; ev_bond joins it
    cudaStream_t st4 = nullptr;
    cudaEvent_t ev_bond = nullptr;
    // optional terms: restraint and trap items of every instance (global bead
    // indices), uploaded flat to bias_d
    std::vector<std::vector<BiasItem>> bias_items;
    BiasItem *bias_d = nullptr;
    size_t bias_cap = 0;
    double *mc_draws_d = nullptr; // caller-supplied Monte Carlo uniforms
    int mc_draws_cap = 0;
    bool mc_pending = false;      // they apply to the next force or step call
    // temperature replica exchange (remd.cu)
    bool remd_on = false;
    RemdDev remd{};
    double *remd_u = nullptr; // [n_inst / 2 + 1] caller's uniforms
    std::vector<double> remd_lab_ion; // ionic strength of every label
    unsigned long long remd_ctr = 0;
    int n_vel_init = 0;
    bool tuned = false;
    // per-block kernel of small instances (k_md_small): eligible by size and
    // list kind (set at creation), the caller's mode, the bucket plan
    // secondary structure per instance: allowed pairs (global beads, lo < hi)
    std::vector<std::vector<int2>> ss_pairs;
    int *ss_start_d = nullptr, *ss_part_d = nullptr;
    bool small_ok = false;
    int small_mode = -1;
    bool small_tuned = false;
    int small_target = 0;            // bucket count the autotuner chose
    int64_t small_planned = 0;       // steps at the last bucket plan
    int small_threads = 256;
    int *sp_off_d = nullptr, *sp_inst_d = nullptr;
    SmallPlan sp{};
    int sms = 152;
};

namespace {

// Makes the context's device current for the duration of an entry point and
// restores the caller's device afterwards, so that one host thread can drive
// contexts on several GPUs.
struct DevGuard {
    int prev = -1;
    explicit DevGuard(const sis_ctx *c) {
        if (!c) return;
        int d = -1;
        if (cudaGetDevice(&d) == cudaSuccess && d != c->dev && cudaSetDevice(c->dev) == cudaSuccess) prev = d;
    }
    ~DevGuard() {
        if (prev >= 0) cudaSetDevice(prev);
    }
    DevGuard(const DevGuard &) = delete;
    DevGuard &operator=(const DevGuard &) = delete;
};

int fail(sis_ctx *c, int code, const std::string &msg) {
    if (c) c->err = msg;
    return code;
}
#define CK(call)                                                                                                               \
    do {                                                                                                                       \
        cudaError_t e_ = (call);                                                                                               \
        if (e_ != cudaSuccess) return fail(ctx, SIS_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_));             \
    } while (0)

template <typename T> int dalloc(sis_ctx *ctx, T **p, size_t count) {
    void *q = nullptr;
    const size_t bytes = std::max<size_t>(1, count) * sizeof(T);
    if (cudaMalloc(&q, bytes) != cudaSuccess) return fail(ctx, SIS_ERR_NOMEM, "device allocation failed");
    if (cudaMemset(q, 0, bytes) != cudaSuccess) return fail(ctx, SIS_ERR_CUDA, "memset failed");
    ctx->allocs.push_back(q);
    *p = (T *)q;
    return SIS_OK;
}

// set_ele.F90:45-99 (default constants) for instance k
void set_ele_fields(const sis_ctx *ctx, InstP &I, double ionic) {
    const sis_params &p = ctx->p;
    const double MM_A = 87.740, MM_B = -0.40008, MM_C = 9.398e-4, MM_D = -1.410e-6;
    const double T = I.tempK;
    double Tc, diele;
    I.diele_dTcoef = 0.0;
    if (p.temp_independent == 0) {
        Tc = T - 273.15;
        diele = MM_A + MM_B * Tc + MM_C * Tc * Tc + MM_D * Tc * Tc * Tc;
    } else {
        Tc = p.tempK_ref - 273.15;
        diele = MM_A + MM_B * Tc + MM_C * Tc * Tc + MM_D * Tc * Tc * Tc;
        I.diele_dTcoef = 1.0 + p.tempK_ref / diele * (MM_B + 2.0 * MM_C * Tc + 3.0 * MM_D * Tc * Tc);
    }
    const double lb = ELE * ELE / (4.0 * PI * EPS0 * diele * BOLTZ_J * T) * 1.0e10;
    const double Zp = p.length_per_charge / lb;
    double coef = JOUL2KCAL_MOL * 1.0e10 * (ELE * ELE) / (4.0 * PI * EPS0 * diele);
    coef = coef * (Zp * Zp);
    const double lambdaD = 1.0e10 * sqrt((1.0e-3 * EPS0 * diele * BOLTZ_J) / (2.0 * N_AVO * (ELE * ELE))) * sqrt(T / ionic);
    I.ele_coef = coef;
    I.diele = diele;
    I.rcdist = 1.0 / lambdaD;
    I.ele_cut = (p.ele_cutoff_type == 2) ? p.ele_cutoff_inp * lambdaD : p.ele_cutoff_inp;
    I.ele_cut2 = I.ele_cut * I.ele_cut;
    I.ele_coef_f = (float)I.ele_coef;
    I.rcdist_f = (float)I.rcdist;
    I.ele_cut2_f = (float)I.ele_cut2;
    const double m = p.nl_margin;
    I.ele_nl_cut2 = p.flg_ele ? (I.ele_cut + m) * (I.ele_cut + m) : -1.0;
}
void set_ele(sis_ctx *ctx, int k) { set_ele_fields(ctx, ctx->ip[k], ctx->ionic[k]); }

// job_md.F90:94-133 friction and masses, set_md_coef job_md.F90:700-767
double friction_of(const sis_params &p) {
    const double radius = 10.0;
    const double v = (p.integrator == SIS_INTGRT_GJF2GJ) ? p.viscosity_Pas * sqrt(1.0e3 / KCAL2JOUL) * N_AVO * 1.0e-20
                                                          : (JOUL2KCAL_MOL * 1.0e-18) * p.viscosity_Pas;
    return 6.0 * PI * v * radius;
}
// md_coef(4): the noise amplitude, the one coefficient that depends on T
double noise_coef(const sis_params &p, double fric, double m, double T) {
    const double dt = p.dt;
    if (p.integrator == SIS_INTGRT_GJF2GJ) {
        const double c1 = 0.5 * dt * fric / m;
        const double c2 = sqrt(1.0 / (1.0 + c1));
        return 0.5 * c2 / m * sqrt(2.0 * fric * BOLTZ_KCAL_MOL * T * dt);
    }
    return sqrt(2.0 * BOLTZ_KCAL_MOL * T * dt / fric);
}
void md_coefs(sis_ctx *ctx, std::vector<double4> &mdc) {
    const sis_params &p = ctx->p;
    const double fric = friction_of(p);
    mdc.resize(ctx->n);
    ctx->mass.resize(ctx->n);
    for (int i = 0; i < ctx->n; ++i) {
        double m;
        switch (ctx->seq[i]) {
        case 0: m = 328.212; break; // A
        case 2: m = 344.212; break; // G
        case 3: m = 304.182; break; // C
        case 1: m = 305.164; break; // U
        default: m = 320.443; break; // D
        }
        ctx->mass[i] = m;
        const double T = ctx->ip[ctx->binfo[i].x].tempK;
        const double dt = p.dt;
        if (p.integrator == SIS_INTGRT_GJF2GJ) {
            const double c1 = 0.5 * dt * fric / m;
            const double c2 = sqrt(1.0 / (1.0 + c1));
            mdc[i] = make_double4((1.0 - c1) / (1.0 + c1), c2 * dt / m, c2 * dt, noise_coef(p, fric, m, T));
        } else {
            mdc[i] = make_double4(dt / fric, 0.0, 0.0, noise_coef(p, fric, m, T));
        }
        // job_md.F90:713-729,745-748: a frozen bead's position coefficient is
        // zero (GJF-2GJ sqrt(b) h; Ermak-McCammon h/gamma and its noise)
        if (!ctx->frozen.empty() && ctx->frozen[i]) {
            if (p.integrator == SIS_INTGRT_GJF2GJ) {
                mdc[i].z = 0.0;
            } else {
                mdc[i].x = 0.0;
                mdc[i].w = 0.0;
            }
        }
    }
}

// init_bp.F90:39-172 NN triplet tables (model 5)
void bp3_tables(const sis_params &p, std::vector<short> &hash, std::vector<double> &dH, std::vector<double> &dS) {
    hash.assign(4097, 0);
    dH.assign(469, 0.0);
    dS.assign(469, 0.0);
    if (p.bp_model != 5) return;
    auto key = [](int w, int x, int u, int z, int y, int v) {
        if (x < y) return 1 + w + x * 4 + u * 16 + z * 64 + y * 256 + v * 1024;
        return 1 + v + y * 4 + z * 16 + u * 64 + x * 256 + w * 1024;
    };
    auto isAU = [](int a, int b) { return (a == 0 && b == 1) || (a == 1 && b == 0); };
    auto isGC = [](int a, int b) { return (a == 2 && b == 3) || (a == 3 && b == 2); };
    auto isGU = [](int a, int b) { return (a == 2 && b == 1) || (a == 1 && b == 2); };
    int h = 0;
    for (int x = 0; x <= 2; ++x)
        for (int y = x + 1; y <= 3; ++y) {
            if (!is_comp(x, y)) continue;
            for (int w = 0; w <= 3; ++w)
                for (int z = 0; z <= 3; ++z) {
                    const bool cwz = is_comp(w, z);
                    const double h1 = cwz ? 0.5 * (p.nn_dH[nnt_index(w, x, z, y) - 1] - p.dH0) : 0.0;
                    const double s1 = cwz ? 0.5 * (p.nn_dS[nnt_index(w, x, z, y) - 1] - p.dS0) : 0.0;
                    for (int u = 0; u <= 3; ++u)
                        for (int v = 0; v <= 3; ++v) {
                            const bool cuv = is_comp(u, v);
                            if (!cwz && !cuv) continue;
                            ++h;
                            hash[key(w, x, u, z, y, v)] = (short)h;
                            if (cuv) {
                                dH[h] = h1 + 0.5 * (p.nn_dH[nnt_index(x, u, y, v) - 1] - p.dH0);
                                dS[h] = (s1 + 0.5 * (p.nn_dS[nnt_index(x, u, y, v) - 1] - p.dS0)) * 1.0e-3;
                            } else {
                                dH[h] = h1;
                                dS[h] = s1 * 1.0e-3;
                            }
                            if (p.nnend && cwz != cuv) {
                                const int o1 = cwz ? w : u, o2 = cwz ? z : v;
                                int k = 0;
                                if (isAU(x, y)) k = isAU(o1, o2) ? 1 : isGC(o1, o2) ? 2 : isGU(o1, o2) ? 3 : 0;
                                else if (isGU(x, y)) k = isAU(o1, o2) ? 5 : isGC(o1, o2) ? 4 : isGU(o1, o2) ? 6 : 0;
                                if (k) {
                                    dH[h] = dH[h] + p.nnend_dH[k - 1] - p.dHend0;
                                    dS[h] = dS[h] + (p.nnend_dS[k - 1] - p.dSend0) * 1.0e-3;
                                }
                            }
                        }
                }
        }
}

int upload_ip(sis_ctx *ctx) {
    CK(cudaMemcpyAsync(ctx->ip_d, ctx->ip.data(), sizeof(InstP) * ctx->n_inst, cudaMemcpyHostToDevice, ctx->st));
    return SIS_OK;
}

// Row k of the FP32 triplet free-energy table at instance k's temperature.
// dG = dH - T dS is rounded once per operation (as the FP64 kernels and the
// FP64 restatement evaluate it), and the FP32 copy keeps the sign of the FP64
// value, so the dG < 0 test of the mixed path decides as the FP64 path does.
void dgf_row(const sis_ctx *ctx, double T, float *row) {
    for (int h = 0; h < 469; ++h) {
        const double p = T * ctx->bp3_dS[h];
        const double v = ctx->bp3_dH[h] - p;
        float f = (float)v;
        if (v < 0.0 && !(f < 0.f)) f = -1.17549435e-38f;
        if (!(v < 0.0) && !(f >= 0.f)) f = 0.f;
        row[h] = f;
    }
}
int upload_dgf(sis_ctx *ctx, int k) {
    float *row = ctx->dgf.data() + (size_t)k * 469;
    dgf_row(ctx, ctx->ip[k].tempK, row);
    CK(cudaMemcpyAsync(ctx->dgf_d + (size_t)k * 469, row, sizeof(float) * 469, cudaMemcpyHostToDevice, ctx->st));
    return SIS_OK;
}

int ensure_lists(sis_ctx *ctx, bool small_step = false);

int run_rebuild(sis_ctx *ctx) {
    ctx->launches++;
    CK(launch_rebuild(ctx->D, ctx->g, ctx->cur, ctx->plan, ctx->coop_grid, ctx->st));
    return SIS_OK;
}

int flag_all(sis_ctx *ctx, int inst) {
    std::vector<int> f(ctx->n_inst, 0);
    for (int k = 0; k < ctx->n_inst; ++k) f[k] = (inst < 0 || inst == k) ? 1 : 0;
    CK(cudaMemcpyAsync(ctx->D.flag, f.data(), sizeof(int) * ctx->n_inst, cudaMemcpyHostToDevice, ctx->st));
    const int one = 1;
    CK(cudaMemcpyAsync(ctx->D.any, &one, sizeof(int), cudaMemcpyHostToDevice, ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
    return SIS_OK;
}

// The lists current for every instance.  Slots loaded into a context that
// steps through the per-block kernel are rebuilt by that kernel's next
// launch (small_step: the caller launches it); any other caller rebuilds
// them here.
int ensure_lists(sis_ctx *ctx, bool small_step) {
    if (!ctx->state_set) return fail(ctx, SIS_ERR_STATE, "coordinates have not been set");
    if (ctx->stale_lists && !small_step) {
        const int one = 1;
        CK(cudaMemcpyAsync(ctx->D.any, &one, sizeof(int), cudaMemcpyHostToDevice, ctx->st));
        int rc = run_rebuild(ctx);
        if (rc) return rc;
        CK(cudaStreamSynchronize(ctx->st));
        ctx->stale_lists = false;
    }
    if (ctx->lists_valid) return SIS_OK;
    int rc = flag_all(ctx, -1);
    if (rc) return rc;
    rc = run_rebuild(ctx);
    if (rc) return rc;
    ctx->lists_valid = true;
    return SIS_OK;
}

// Reads and clears the device error flags: an error is reported once.
int check_err(sis_ctx *ctx) {
    int e = 0;
    CK(cudaMemcpyAsync(&e, ctx->D.err, sizeof(int), cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
    if (e) CK(cudaMemsetAsync(ctx->D.err, 0, sizeof(int), ctx->st));
    if (e & ERR_TIMEOUT) {
        // blocks left the trigger/rebuild kernel early: start its barrier
        // afresh, clear the cell counters a binning phase may have left
        // partly filled, and rebuild every list at the next call (a rebuild
        // may have stopped half way)
        CK(cudaMemsetAsync(ctx->D.gbar, 0, 2 * sizeof(unsigned int), ctx->st));
        if (ctx->D.n_cells > 0) CK(cudaMemsetAsync(ctx->D.cell_cnt, 0, sizeof(int) * ctx->D.n_cells, ctx->st));
        CK(cudaStreamSynchronize(ctx->st));
        ctx->lists_valid = false;
    }
    if (e & ERR_PAIR_OVERFLOW) return fail(ctx, SIS_ERR_LIST_OVERFLOW, "pair list capacity exceeded");
    if (e & ERR_BP_OVERFLOW) return fail(ctx, SIS_ERR_LIST_OVERFLOW, "base-pair list capacity exceeded");
    if (e & ERR_NONFINITE) return fail(ctx, SIS_ERR_NONFINITE, "non-finite displacement");
    if (e & ERR_TIMEOUT) return fail(ctx, SIS_ERR_TIMEOUT, "grid barrier of the trigger/rebuild kernel timed out");
    return SIS_OK;
}

int inst_range(const sis_ctx *ctx, int inst, int &off, int &cnt) {
    if (inst < -1 || inst >= ctx->n_inst) return SIS_ERR_ARG;
    off = inst < 0 ? 0 : ctx->ip[inst].bead_off;
    cnt = inst < 0 ? ctx->n : ctx->ip[inst].n;
    return SIS_OK;
}

int bp_blocks(const sis_ctx *ctx) { return ctx->g.bp_model > 0 ? ctx->bpb : 0; }
int bp_test_blocks(const sis_ctx *ctx) { return ctx->g.bp_model > 0 ? ctx->bpt : 0; }

// The bonded and base-pair pass of one step at buffer parity `cur`: k_bonded
// on st4 beside k_bp_test, k_bp_eval (+ k_bp_mc) on ctx->st,
// joined on ctx->st.
// The fork event ev_fork is recorded on ctx->st by the caller.
cudaError_t enqueue_pre(sis_ctx *ctx, int cur) {
    cudaError_t e;
    if (ctx->g.bp_model == 0) return launch_bonded_step(ctx->D, ctx->g, cur, ctx->st);
    if ((e = cudaStreamWaitEvent(ctx->st4, ctx->ev_fork, 0)) != cudaSuccess) return e;
    if ((e = launch_bonded_step(ctx->D, ctx->g, cur, ctx->st4)) != cudaSuccess) return e;
    if ((e = cudaEventRecord(ctx->ev_bond, ctx->st4)) != cudaSuccess) return e;
    if ((e = launch_bp(ctx->D, ctx->g, cur, bp_test_blocks(ctx), bp_blocks(ctx), ctx->st)) != cudaSuccess) return e;
    if ((e = launch_bp_mc(ctx->D, ctx->g, ctx->st)) != cudaSuccess) return e;
    return cudaStreamWaitEvent(ctx->st, ctx->ev_bond, 0);
}
int pre_step_kernels(const sis_ctx *ctx) { return 1 + bp_kernels(ctx->g) + (ctx->g.nstep_mc > 0); }

// The forces and update of one step at buffer parity `cur` on ctx->st:
// the bonded and base-pair pass, then k_step; with overlap, k_pairs runs on
// st3 beside that pass and k_step takes its pair forces from fpair.
// The mixed path always takes its pair forces from the cluster-pair kernel:
// beside the pass with overlap, before it on ctx->st without.
cudaError_t enqueue_forces_update(sis_ctx *ctx, int cur, const double *noise, long long ns) {
    cudaError_t e;
    const bool split = ctx->overlap || ctx->g.prec != 0;
    if ((e = cudaEventRecord(ctx->ev_fork, ctx->st)) != cudaSuccess) return e;
    if (ctx->overlap) {
        if ((e = cudaStreamWaitEvent(ctx->st3, ctx->ev_fork, 0)) != cudaSuccess) return e;
        if ((e = launch_pairs(ctx->G, ctx->D, ctx->g, cur, ctx->st3)) != cudaSuccess) return e;
        if ((e = cudaEventRecord(ctx->ev_join, ctx->st3)) != cudaSuccess) return e;
    } else if (split && (e = launch_pairs(ctx->G, ctx->D, ctx->g, cur, ctx->st)) != cudaSuccess) {
        return e;
    }
    if ((e = enqueue_pre(ctx, cur)) != cudaSuccess) return e;
    if ((e = launch_bias(ctx->D, ctx->g, cur, 1, ctx->st)) != cudaSuccess) return e;
    if (!split) return launch_step(ctx->G, ctx->D, ctx->g, cur, noise, ns, ctx->st, 1);
    if (ctx->overlap && (e = cudaStreamWaitEvent(ctx->st, ctx->ev_join, 0)) != cudaSuccess) return e;
    return launch_step_split(ctx->G, ctx->D, ctx->g, cur, noise, ns, ctx->st, 1);
}
int step_kernels(const sis_ctx *ctx) {
    return pre_step_kernels(ctx) + bias_kernels(ctx->g) + 1 + (ctx->overlap || ctx->g.prec != 0 ? 1 : 0);
}

int enqueue_step(sis_ctx *ctx, const double *noise, long long ns) {
    CK(enqueue_forces_update(ctx, ctx->cur, noise, ns));
    ctx->launches += step_kernels(ctx);
    ctx->cur ^= 1;
    return run_rebuild(ctx);
}

// ----------------------------------------------------------- step graphs
// kGraphSteps MD steps captured as one graph: per step k_bonded beside the
// base-pair kernels, k_step and k_trigger_rebuild, which ends at once when no
// instance's trigger fired, so a step without a rebuild runs five kernels and
// nothing else.  An even step count leaves the position buffer parity
// unchanged, so one graph serves every launch.
constexpr int kGraphSteps = 20;

int build_step_graph(sis_ctx *ctx) {
    if (ctx->gexec) cudaGraphExecDestroy(ctx->gexec);
    ctx->gexec = nullptr;
    cudaGraph_t graph = nullptr;
    CK(cudaGraphCreate(&graph, 0));
    cudaError_t e = cudaStreamBeginCaptureToGraph(ctx->st, graph, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed);
    if (e == cudaSuccess) {
        int cur = ctx->cur;
        for (int k = 0; k < kGraphSteps && e == cudaSuccess; ++k) {
            e = enqueue_forces_update(ctx, cur, nullptr, 0);
            cur ^= 1;
            if (e == cudaSuccess)
                e = launch_rebuild(ctx->D, ctx->g, cur, ctx->plan, ctx->coop_grid, ctx->st);
        }
        cudaGraph_t got = nullptr;
        const cudaError_t ee = cudaStreamEndCapture(ctx->st, &got);
        if (e == cudaSuccess) e = ee;
    }
    if (e == cudaSuccess) e = cudaGraphInstantiate(&ctx->gexec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) {
        ctx->gexec = nullptr;
        cudaGetLastError();
        return fail(ctx, SIS_ERR_CUDA, std::string("step graph: ") + cudaGetErrorString(e));
    }
    ctx->graph_cur = ctx->cur;
    ctx->graph_G = ctx->G;
    ctx->graph_bpb = ctx->bpb;
    ctx->graph_g = ctx->g;
    ctx->graph_overlap = ctx->overlap;
    return SIS_OK;
}

// the step graph for the current parameters, captured again when they changed
int ensure_step_graph(sis_ctx *ctx) {
    if (ctx->gexec && ctx->graph_cur == ctx->cur && ctx->graph_G == ctx->G && ctx->graph_bpb == ctx->bpb &&
        ctx->graph_overlap == ctx->overlap && memcmp(&ctx->graph_g, &ctx->g, sizeof(GlobP)) == 0)
        return SIS_OK;
    return build_step_graph(ctx);
}

// Picks the lanes-per-bead width G of the step kernel, and whether its pair
// forces run in k_pairs beside the bonded and base-pair pass (overlap), by
// timing the step kernels of every candidate: four steps captured as a graph
// (without the trigger and rebuild), launched once to warm up and once
// timed.  The step kernels update v, beta and move in place, the
// displacement maxima of blocks that span many instances and the force-cap
// counter; those are saved before and restored after, and the rest of what
// they write (the other position buffer and its mirror, the per-block
// partials, the base-pair forces they consume) is rewritten by the next real
// step.  With the Monte Carlo removal on, the base-pair kernels are left out
// of the timing, since they would consume the pass that is due.
int autotune(sis_ctx *ctx) {
    if (ctx->tuned) return SIS_OK;
    // (the mixed path's step kernel runs one thread per bead whatever G is:
    // only the overlap is tuned there)
    std::vector<int> gs = ctx->g.prec != 0 ? std::vector<int>{1}
                          : ctx->lanes_fixed ? std::vector<int>{ctx->G}
                                             : std::vector<int>{2, 4, 8, 16};
    std::vector<int> ovs = ctx->overlap_mode >= 0 ? std::vector<int>{ctx->overlap_mode} : std::vector<int>{0, 1};
    if (gs.size() * ovs.size() == 1) {
        ctx->G = gs[0];
        ctx->overlap = ovs[0] != 0;
        ctx->tuned = true;
        return SIS_OK;
    }
    const bool with_bp = ctx->g.bp_model > 0 && ctx->g.nstep_mc == 0;
    const size_t n = ctx->n, ni = ctx->n_inst;
    Dev &D = ctx->D;
    double4 *save = nullptr;
    unsigned long long *msave = nullptr;
    if (cudaMalloc(&save, sizeof(double4) * 3 * n) != cudaSuccess ||
        cudaMalloc(&msave, sizeof(unsigned long long) * (4 * ni + 1)) != cudaSuccess) {
        cudaFree(save);
        cudaGetLastError();
        return fail(ctx, SIS_ERR_NOMEM, "autotune scratch");
    }
    auto copy = [&](bool back) -> cudaError_t {
        const cudaMemcpyKind k = cudaMemcpyDeviceToDevice;
        double4 *st[3] = {D.v, D.beta, D.move};
        unsigned long long *ms[3] = {D.m1, D.m2, D.capped};
        const size_t mc[3] = {2 * ni, 2 * ni, 1}, mo[3] = {0, 2 * ni, 4 * ni};
        cudaError_t e = cudaSuccess;
        for (int f = 0; f < 3 && e == cudaSuccess; ++f)
            e = back ? cudaMemcpyAsync(st[f], save + f * n, sizeof(double4) * n, k, ctx->st)
                     : cudaMemcpyAsync(save + f * n, st[f], sizeof(double4) * n, k, ctx->st);
        for (int f = 0; f < 3 && e == cudaSuccess; ++f)
            e = back ? cudaMemcpyAsync(ms[f], msave + mo[f], sizeof(unsigned long long) * mc[f], k, ctx->st)
                     : cudaMemcpyAsync(msave + mo[f], ms[f], sizeof(unsigned long long) * mc[f], k, ctx->st);
        return e;
    };
    const bool mixed = ctx->g.prec != 0;
    auto pass = [&](int G, int ov) -> cudaError_t {
        cudaError_t e;
        if ((e = cudaEventRecord(ctx->ev_fork, ctx->st)) != cudaSuccess) return e;
        if (ov) {
            if ((e = cudaStreamWaitEvent(ctx->st3, ctx->ev_fork, 0)) != cudaSuccess) return e;
            if ((e = launch_pairs(G, D, ctx->g, ctx->cur, ctx->st3)) != cudaSuccess) return e;
            if ((e = cudaEventRecord(ctx->ev_join, ctx->st3)) != cudaSuccess) return e;
        } else if (mixed && (e = launch_pairs(G, D, ctx->g, ctx->cur, ctx->st)) != cudaSuccess) {
            return e;
        }
        if (with_bp) {
            if ((e = cudaStreamWaitEvent(ctx->st4, ctx->ev_fork, 0)) != cudaSuccess) return e;
            if ((e = launch_bonded_step(D, ctx->g, ctx->cur, ctx->st4)) != cudaSuccess) return e;
            if ((e = cudaEventRecord(ctx->ev_bond, ctx->st4)) != cudaSuccess) return e;
            if ((e = launch_bp(D, ctx->g, ctx->cur, bp_test_blocks(ctx), bp_blocks(ctx), ctx->st)) != cudaSuccess) return e;
            if ((e = cudaStreamWaitEvent(ctx->st, ctx->ev_bond, 0)) != cudaSuccess) return e;
        } else if ((e = launch_bonded_step(D, ctx->g, ctx->cur, ctx->st)) != cudaSuccess) {
            return e;
        }
        if (ov && (e = cudaStreamWaitEvent(ctx->st, ctx->ev_join, 0)) != cudaSuccess) return e;
        if (ov || mixed) return launch_step_split(G, D, ctx->g, ctx->cur, nullptr, 0, ctx->st, 0);
        return launch_step(G, D, ctx->g, ctx->cur, nullptr, 0, ctx->st, 0);
    };
    cudaError_t e = copy(false);
    float best = 1e30f;
    int bestG = gs[0], bestOv = ovs[0];
    for (int G : gs)
        for (int ov : ovs) {
            if (e != cudaSuccess) break;
            cudaGraph_t gr = nullptr;
            cudaGraphExec_t ge = nullptr;
            e = cudaStreamBeginCapture(ctx->st, cudaStreamCaptureModeRelaxed);
            for (int r = 0; r < 4 && e == cudaSuccess; ++r) e = pass(G, ov);
            const cudaError_t ee = cudaStreamEndCapture(ctx->st, &gr);
            if (e == cudaSuccess) e = ee;
            if (e == cudaSuccess) e = cudaGraphInstantiate(&ge, gr, 0);
            if (gr) cudaGraphDestroy(gr);
            float ms = 1e30f;
            if (e == cudaSuccess) e = cudaGraphLaunch(ge, ctx->st);
            if (e == cudaSuccess) e = cudaEventRecord(ctx->ev[12], ctx->st);
            if (e == cudaSuccess) e = cudaGraphLaunch(ge, ctx->st);
            if (e == cudaSuccess) e = cudaEventRecord(ctx->ev[13], ctx->st);
            if (e == cudaSuccess) e = cudaEventSynchronize(ctx->ev[13]);
            if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, ctx->ev[12], ctx->ev[13]);
            if (ge) cudaGraphExecDestroy(ge);
            ctx->launches += 8 * (2 + (ov || mixed ? 1 : 0) + (with_bp ? bp_kernels(ctx->g) : 0));
            if (e == cudaSuccess && ms < best) {
                best = ms;
                bestG = G;
                bestOv = ov;
            }
        }
    if (e == cudaSuccess) e = copy(true);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->st);
    cudaFree(save);
    cudaFree(msave);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return fail(ctx, SIS_ERR_CUDA, std::string("autotune: ") + cudaGetErrorString(e));
    }
    ctx->G = bestG;
    ctx->overlap = bestOv != 0;
    ctx->tuned = true;
    return SIS_OK;
}

// ------------------------------------------------------ small instances
bool small_active(const sis_ctx *ctx) {
    return ctx->small_ok && ctx->small_mode != 0 && ctx->g.nstep_mc == 0 && !ctx->g.flg_bias && !ctx->mc_pending;
}

// Buckets of whole instances for k_md_small: costliest first into the
// bucket with the least cost (at most kSmallMaxInst instances and
// kSmallMaxBeads beads each), about `target` buckets; each bucket lists its
// instances in ascending order.
int small_plan(sis_ctx *ctx, int target) {
    const int ni = ctx->n_inst;
    // cost of an instance: its pair-list entries, a per-bead share (the
    // update and bonded terms cost about as much as 90 entries) and its
    // base-pair records; by capacity when slots are loaded in place
    // (sis_gpu_load_slot)
    std::vector<double> cost(ni);
    bool slots = false;
    for (int k = 0; k < ni; ++k) slots |= ctx->ip[k].n_act != ctx->ip[k].n;
    std::vector<int> nn, nbp;
    if (!slots && ctx->lists_valid) {
        nn.resize(ctx->n);
        nbp.resize(ni);
        CK(cudaMemcpyAsync(nn.data(), ctx->D.nnbr, sizeof(int) * ctx->n, cudaMemcpyDeviceToHost, ctx->st));
        CK(cudaMemcpyAsync(nbp.data(), ctx->D.bp_cnt, sizeof(int) * ni, cudaMemcpyDeviceToHost, ctx->st));
        CK(cudaStreamSynchronize(ctx->st));
    }
    for (int k = 0; k < ni; ++k) {
        const InstP &I = ctx->ip[k];
        double c = 90.0 * I.n;
        if (!nn.empty()) {
            for (int i = I.bead_off; i < I.bead_off + I.n; ++i) c += std::min(nn[i], ctx->g.cap);
            c += 8.0 * std::min(nbp[k], I.bp_cap); // base-pair records: a test each
        }
        cost[k] = c;
    }
    std::vector<int> order(ni);
    for (int k = 0; k < ni; ++k) order[k] = k;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return cost[a] > cost[b]; });
    const int nbins = std::max(1, std::min(target, ni));
    std::vector<std::vector<int>> bins(nbins);
    std::vector<int> beads(nbins, 0);
    std::vector<double> load(nbins, 0.0);
    for (int k : order) {
        int best = -1;
        for (int b = 0; b < (int)bins.size(); ++b)
            if ((int)bins[b].size() < kSmallMaxInst && beads[b] + ctx->ip[k].n <= kSmallMaxBeads &&
                (best < 0 || load[b] < load[best]))
                best = b;
        if (best < 0) {
            bins.emplace_back();
            beads.push_back(0);
            load.push_back(0.0);
            best = (int)bins.size() - 1;
        }
        bins[best].push_back(k);
        beads[best] += ctx->ip[k].n;
        load[best] += cost[k];
    }
    std::vector<int> off(1, 0), inst;
    int cap = 1;
    for (size_t b = 0; b < bins.size(); ++b) {
        if (bins[b].empty()) continue;
        std::sort(bins[b].begin(), bins[b].end());
        inst.insert(inst.end(), bins[b].begin(), bins[b].end());
        off.push_back((int)inst.size());
        cap = std::max(cap, beads[b]);
    }
    CK(cudaMemcpyAsync(ctx->sp_off_d, off.data(), sizeof(int) * off.size(), cudaMemcpyHostToDevice, ctx->st));
    CK(cudaMemcpyAsync(ctx->sp_inst_d, inst.data(), sizeof(int) * inst.size(), cudaMemcpyHostToDevice, ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
    ctx->sp.cta_off = ctx->sp_off_d;
    ctx->sp.inst = ctx->sp_inst_d;
    ctx->sp.n_cta = (int)off.size() - 1;
    ctx->sp.cap = cap;
    ctx->sp.inner = 0;
    for (int k = 0; k < ni; ++k) ctx->sp.inner |= ctx->ip[k].n >= kInnerMinBeads ? 1 : 0;
    return SIS_OK;
}

// nsteps steps through k_md_small, at most kSmallChunk per launch; noise: the
// device copy of fed noise (nsteps x n x 3) or NULL
constexpr int kSmallChunk = 1000;
constexpr int64_t kSmallReplan = 2000; // MD steps between bucket plans
int run_small(sis_ctx *ctx, int64_t nsteps, const double *noise) {
    for (int64_t s = 0; s < nsteps;) {
        const int chunk = (int)std::min<int64_t>(kSmallChunk, nsteps - s);
        const double *nz = noise ? noise + (size_t)s * ctx->n * 3 : nullptr;
        CK(launch_md_small(ctx->D, ctx->g, ctx->cur, ctx->sp, chunk, nz, ctx->small_threads, ctx->st));
        CK(launch_cluster_flagged(ctx->D, ctx->g, ctx->st));
        CK(launch_small_finish(ctx->D, ctx->g, (unsigned long long)chunk, ctx->st));
        ctx->launches += 3;
        ctx->cur ^= chunk & 1;
        s += chunk;
        ctx->stale_lists = false;
    }
    return SIS_OK;
}

// Picks the bucket count and the block width of k_md_small by timing real
// steps of each candidate, in two rounds, by each candidate's faster round
// (a list rebuild inside one timed window does not decide the pick); the
// per-bead arithmetic is the same for all, so the steps are part of the
// trajectory.  Returns the steps it took.
int64_t small_autotune(sis_ctx *ctx, int64_t budget, int *rc) {
    *rc = SIS_OK;
    const int sms = ctx->sms;
    std::vector<int> targets;
    for (int f : {1, 2, 3, 4}) {
        const int t = std::min(ctx->n_inst, f * sms);
        if (targets.empty() || targets.back() != t) targets.push_back(t);
    }
    const std::vector<int> widths = {128, 256, 384, 512};
    const int per = 16, rounds = 2;
    const int64_t need = (int64_t)(rounds * targets.size() * widths.size() + 1) * per;
    if (budget < need) {
        if (!ctx->sp.n_cta && (*rc = small_plan(ctx, std::min(ctx->n_inst, 2 * sms)))) return 0;
        return 0;
    }
    std::vector<float> best_ms(targets.size() * widths.size(), 1e30f);
    int64_t taken = 0;
    // the first pass warms up (list state, first-touch), untimed
    if ((*rc = small_plan(ctx, targets[0]))) return taken;
    ctx->small_threads = widths[0];
    if ((*rc = run_small(ctx, per, nullptr))) return taken;
    taken += per;
    for (int r = 0; r < rounds; ++r) {
        for (size_t ti = 0; ti < targets.size(); ++ti) {
            if ((*rc = small_plan(ctx, targets[ti]))) return taken;
            for (size_t wi = 0; wi < widths.size(); ++wi) {
                const int w = widths[wi];
                if (small_smem_bytes(ctx->sp.cap) > 212 * 1024) continue;
                // the 384-thread bound (168 registers, a third of the spills,
                // 12 warps) against 512 (16 warps), by bucket size as measured
                // in steady state: buckets of 64 beads ran 7% faster with 384,
                // of 120 beads as fast, of ~600 beads 13% slower; so 384 only
                // up to 384 beads, and 512 only above 96
                if (w == 384 && ctx->sp.cap > 384) continue;
                if (w == 512 && ctx->sp.cap <= 96) continue;
                ctx->small_threads = w;
                cudaEventRecord(ctx->ev[12], ctx->st);
                if ((*rc = run_small(ctx, per, nullptr))) return taken;
                cudaEventRecord(ctx->ev[13], ctx->st);
                cudaEventSynchronize(ctx->ev[13]);
                float ms = 1e30f;
                cudaEventElapsedTime(&ms, ctx->ev[12], ctx->ev[13]);
                taken += per;
                float &b = best_ms[ti * widths.size() + wi];
                b = std::min(b, ms);
            }
        }
    }
    size_t bi = 0;
    for (size_t k = 1; k < best_ms.size(); ++k)
        if (best_ms[k] < best_ms[bi]) bi = k;
    const int best_t = targets[bi / widths.size()], best_w = widths[bi % widths.size()];
    if ((*rc = small_plan(ctx, best_t))) return taken;
    ctx->small_target = best_t;
    ctx->small_planned = ctx->steps + taken;
    ctx->small_threads = best_w;
    ctx->small_tuned = true;
    return taken;
}

} // namespace

namespace {
bool finite_pos(double v) { return std::isfinite(v) && v > 0.0; }

// Host-side checks of everything that later indexes a device table or
// divides: codes, counts and physical constants.  They run before any CUDA
// call, so a bad input is refused without touching the device.
bool inputs_valid(const sis_topology *top, const sis_params *p) {
    if (!top->inst_chain_off || !top->chain_len || !top->chain_moltype || !top->seq || !top->tempK ||
        !top->ionic_strength)
        return false;
    if (top->inst_chain_off[0] < 0) return false;
    long long nb = 0;
    for (int k = 0; k < top->n_inst; ++k) {
        if (top->inst_chain_off[k + 1] < top->inst_chain_off[k]) return false;
        if (!finite_pos(top->tempK[k])) return false;
        if (p->flg_ele && !finite_pos(top->ionic_strength[k])) return false;
        if (top->box)
            for (int d = 0; d < 3; ++d)
                if (!std::isfinite(top->box[3 * k + d]) || top->box[3 * k + d] < 0.0) return false;
        for (int c = top->inst_chain_off[k]; c < top->inst_chain_off[k + 1]; ++c) {
            const int len = top->chain_len[c];
            if (len < 1 || (top->chain_moltype[c] != 1 && top->chain_moltype[c] != 2)) return false;
            for (int l = 0; l < len; ++l)
                if (top->seq[nb + l] < 0 || top->seq[nb + l] > 4) return false; // SEQT A U G C D
            nb += len;
            if (nb >= (1LL << 30)) return false;
        }
    }
    if (p->precision != SIS_PREC_FP64 && p->precision != SIS_PREC_MIXED) return false;
    if (p->integrator != SIS_INTGRT_GJF2GJ && p->integrator != SIS_INTGRT_BD_EM) return false;
    if (!finite_pos(p->dt) || !finite_pos(p->viscosity_Pas) || !std::isfinite(p->nl_margin) || p->nl_margin < 0.0)
        return false;
    if (p->bp_model < 0 || p->bp_model > 5 || p->nbr_cap < 0 || p->bp_cap < 0 || p->nstep_bp_mc < 0) return false;
    if (p->nstep_bp_mc > 0 && p->max_bp_per_nt < 1) return false;
    if (p->flg_ele && p->ele_cutoff_type != 1 && p->ele_cutoff_type != 2) return false;
    return true;
}
} // namespace

// ====================================================================== API
extern "C" int sis_gpu_create(const sis_topology *top, const sis_params *par, sis_ctx **out) {
    if (!top || !par || !out || top->n_inst <= 0) return SIS_ERR_ARG;
    *out = nullptr;
    if (!inputs_valid(top, par)) return SIS_ERR_ARG;
    sis_ctx *ctx = new sis_ctx();
    *out = nullptr;
    if (cudaGetDevice(&ctx->dev) != cudaSuccess) {
        delete ctx;
        return SIS_ERR_CUDA;
    }
    ctx->p = *par;
    const sis_params &p = ctx->p;
    ctx->n_inst = top->n_inst;
    // ------------------------------------------------ topology and instances
    ctx->ip.resize(ctx->n_inst);
    ctx->ionic.resize(ctx->n_inst);
    int nb = 0;
    for (int k = 0; k < ctx->n_inst; ++k) {
        InstP &I = ctx->ip[k];
        memset(&I, 0, sizeof(InstP));
        I.bead_off = nb;
        for (int c = top->inst_chain_off[k]; c < top->inst_chain_off[k + 1]; ++c) {
            const int len = top->chain_len[c];
            if (len < 1) {
                delete ctx;
                return SIS_ERR_ARG;
            }
            const bool circ = top->chain_moltype[c] == 2;
            for (int l = 0; l < len; ++l) {
                const int i = nb + l;
                const int s = top->seq[i];
                const int q = top->has_charge ? (top->has_charge[i] ? 1 : 0) : 1;
                ctx->binfo.push_back(make_int4(k, nb, len | (circ ? (int)0x80000000u : 0), l | (s << 24) | (q << 28)));
                ctx->seq.push_back(s);
            }
            nb += len;
        }
        I.n = nb - I.bead_off;
        I.n_act = I.n;
        I.stream = top->stream ? top->stream[k] : (unsigned)k;
        I.twz_scale = 1.0;
        I.step0 = 0ull;
        I.tempK = top->tempK[k];
        ctx->ionic[k] = top->ionic_strength[k];
        const double *bx = top->box ? top->box + 3 * k : nullptr;
        I.pbc = bx && bx[0] > 0.0 && bx[1] > 0.0 && bx[2] > 0.0;
        for (int d = 0; d < 3; ++d) {
            I.box[d] = I.pbc ? bx[d] : 0.0;
            I.half[d] = 0.5 * I.box[d];
            I.fsc[d] = I.pbc ? 4294967296.0 / I.box[d] : 1048576.0;
            I.finv[d] = (float)(1.0 / I.fsc[d]);
        }
    }
    ctx->n = nb;
    if (nb <= 0 || nb >= (1 << 30)) {
        delete ctx;
        return SIS_ERR_ARG;
    }
    // ------------------------------------------------------ base pairs
    for (int t = 0; t < 3; ++t) {
        const double *f = p.bp_ff[t];
        BPP b{};
        b.U0 = f[0]; b.bond_k = f[1]; b.bond_r = f[2];
        for (int a = 0; a < 4; ++a) {
            b.angl_k[a] = f[3 + a];
            b.angl_theta[a] = f[7 + a];
        }
        b.dihd_k[0] = f[11]; b.dihd_k[1] = f[12]; b.dihd_phi[0] = f[13]; b.dihd_phi[1] = f[14];
        ctx->bpp[1 + t] = b;
        // read_force_field.F90:203-258: CG/UA/UG swap k1<->k2, k3<->k4, not the angles
        BPP r = b;
        r.angl_k[0] = b.angl_k[1]; r.angl_k[1] = b.angl_k[0];
        r.angl_k[2] = b.angl_k[3]; r.angl_k[3] = b.angl_k[2];
        ctx->bpp[4 + t] = r;
    }
    // init_bp.F90:315-346
    if (fabs(p.bp_cutoff_energy) <= 2.220446049250313e-16) {
        ctx->bp_cutoff_dist = 18.0;
        for (int t = 1; t <= 6; ++t) ctx->bpp[t].cutoff_ddist = ctx->bp_cutoff_dist - 13.8;
    } else {
        ctx->bp_cutoff_dist = 0.0;
        for (int t = 1; t <= 6; ++t) {
            ctx->bpp[t].cutoff_ddist = sqrt(log(fabs(10.0 / p.bp_cutoff_energy)) / ctx->bpp[t].bond_k);
            const double cut = ctx->bpp[t].bond_r + ctx->bpp[t].cutoff_ddist;
            if (cut > ctx->bp_cutoff_dist) ctx->bp_cutoff_dist = cut;
        }
    }
    std::vector<short> hash;
    std::vector<double> dH, dS;
    bp3_tables(p, hash, dH, dS);
    // ---------------------------------------------- per-instance cutoffs
    const double m = p.nl_margin;
    int cap = 32, bp_total_cap = 0, ncells = 0;
    for (int k = 0; k < ctx->n_inst; ++k) {
        InstP &I = ctx->ip[k];
        set_ele(ctx, k);
        I.wca_nl_cut2 = (p.wca_sigma + m) * (p.wca_sigma + m);
        I.bp_nl_cut2 = p.bp_model > 0 ? (ctx->bp_cutoff_dist + m) * (ctx->bp_cutoff_dist + m) : -1.0;
        const int bpc = p.bp_cap > 0 ? p.bp_cap : 12;
        I.bp_off = bp_total_cap;
        I.bp_cap = bpc * I.n + 64;
        bp_total_cap += I.bp_cap;
        I.large = 0;
        if (I.pbc && I.n > kAllPairsMax) {
            double mc2 = std::max(std::max(I.wca_nl_cut2, I.ele_nl_cut2), I.bp_nl_cut2);
            // type-2 cutoffs move with lambdaD; leave room for the largest
            const double lc = sqrt(mc2) * 1.0005;
            int nc[3];
            for (int d = 0; d < 3; ++d) nc[d] = (int)floor(I.box[d] / lc);
            if (nc[0] >= 3 && nc[1] >= 3 && nc[2] >= 3) {
                I.large = 1;
                I.cell_base = ncells;
                for (int d = 0; d < 3; ++d) {
                    I.nc[d] = nc[d];
                    I.cell_len[d] = I.box[d] / nc[d];
                }
                ncells += nc[0] * nc[1] * nc[2];
            }
        }
        const int need = I.large ? 512 : std::min(I.n - 1, 512);
        cap = std::max(cap, need);
    }
    cap = (cap + 31) / 32 * 32;
    if (p.nbr_cap > 0) cap = p.nbr_cap;
    // i-clusters of the mixed path's pair kernel: kCl consecutive beads of an instance
    int n_cl = 0;
    for (int k = 0; k < ctx->n_inst; ++k) {
        ctx->ip[k].cl_off = n_cl;
        n_cl += (ctx->ip[k].n + kCl - 1) / kCl;
    }
    // ------------------------------------------------------ global params
    GlobP &g = ctx->g;
    g.n = ctx->n;
    g.n_inst = ctx->n_inst;
    g.cap = cap;
    g.n_cl = n_cl;
    g.ccap = std::min(kClCapMax, std::max(32, cap / 2));
    g.prec = p.precision;
    g.integrator = p.integrator;
    g.angl_reb = p.angl_reb;
    g.dih_type = p.dih_type;
    g.bp_model = p.bp_model;
    g.flg_ele = p.flg_ele;
    g.temp_indep = p.temp_independent;
    g.bp_min_loop = p.bp_min_loop;
    g.bp_jnext_compat = p.bp_jnext_compat;
    g.ele_excl_bond = p.ele_excl_bond;
    g.ele_excl_angle = p.ele_excl_angle;
    g.bond_k = p.bond_k; g.bond_r0 = p.bond_r0;
    g.angl_k = p.angl_k; g.angl_t0 = p.angl_t0; g.cos_t0 = cos(p.angl_t0);
    g.dih_k = p.dih_k; g.dih_w = p.dih_w; g.dih_p0 = p.dih_p0;
    g.wca_sigma = p.wca_sigma; g.wca_eps = p.wca_eps;
    g.wca_sig2 = p.wca_sigma * p.wca_sigma;
    g.wca_coef = 12.0 * p.wca_eps / g.wca_sig2;
    g.bp_cutoff_energy = p.bp_cutoff_energy;
    g.f_bp_cutoff_energy = (float)p.bp_cutoff_energy;
    g.nstep_mc = (p.bp_model > 0 && p.nstep_bp_mc > 0) ? p.nstep_bp_mc : 0;
    g.max_bp_per_nt = p.max_bp_per_nt > 0 ? p.max_bp_per_nt : 1;
    g.nl_margin = p.nl_margin;
    g.f_bond_k = (float)g.bond_k; g.f_bond_r0 = (float)g.bond_r0;
    g.f_angl_k = (float)g.angl_k; g.f_angl_t0 = (float)g.angl_t0; g.f_cos_t0 = (float)g.cos_t0;
    g.f_dih_k = (float)g.dih_k; g.f_dih_w = (float)g.dih_w; g.f_dih_p0 = (float)g.dih_p0;
    g.f_wca_sig2 = (float)g.wca_sig2; g.f_wca_coef = (float)g.wca_coef;
    g.f_wca_sigma = (float)g.wca_sigma; g.f_wca_eps = (float)g.wca_eps;
    g.seed = p.seed;
    // ----------------------------------------------------------- device
    if (cudaStreamCreateWithFlags(&ctx->st, cudaStreamNonBlocking) != cudaSuccess) {
        delete ctx;
        return SIS_ERR_CUDA;
    }
    for (int e = 0; e < kEvents; ++e) cudaEventCreate(&ctx->ev[e]);
    {
        int dev = 0, sms = 0;
        if (cudaGetDevice(&dev) == cudaSuccess && cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess &&
            sms > 0) {
            ctx->bpb = 2 * sms;
            ctx->sms = sms;
        }
        ctx->bpt = std::max(1, std::min((bp_total_cap + 255) / 256, 8 * (sms > 0 ? sms : 152)));
        // the trigger/rebuild kernel: two blocks per SM (fewer if they do not fit)
        const int per = std::min(2, coop_blocks_per_sm());
        ctx->coop_grid = std::min(kMaxCoopBlocks, std::max(1, per) * (sms > 0 ? sms : 152));
        if (per < 1) ctx->coop_grid = 0;
    }
    Dev &D = ctx->D;
    const int n = ctx->n, ni = ctx->n_inst;
    int rc = 0;
    rc |= dalloc(ctx, &D.x[0], n);
    rc |= dalloc(ctx, &D.x[1], n);
    // the mirrors carry kCl beads of padding: the cluster-pair kernel loads
    // whole j-clusters, past the last bead of the last instance too
    rc |= dalloc(ctx, &D.mir[0], (size_t)n + kCl);
    rc |= dalloc(ctx, &D.mir[1], (size_t)n + kCl);
    if (p.precision != SIS_PREC_FP64) {
        // the per-block kernel of small instances: every instance at most
        // kSmallMaxBeads beads with an all-pairs list
        ctx->small_ok = true;
        for (int k = 0; k < ni; ++k) ctx->small_ok &= ctx->ip[k].n <= kSmallMaxBeads && !ctx->ip[k].large;
        if (ctx->small_ok) {
            rc |= dalloc(ctx, &ctx->sp_off_d, (size_t)ni + 1);
            rc |= dalloc(ctx, &ctx->sp_inst_d, ni);
            // the per-block kernel's inner lists; igen -1: never filtered
            rc |= dalloc(ctx, &D.nbr_in, (size_t)n * cap);
            rc |= dalloc(ctx, &D.nnbr_in, n);
            rc |= dalloc(ctx, &D.mir_in, n);
            rc |= dalloc(ctx, &D.lgen, ni);
            rc |= dalloc(ctx, &D.igen, ni);
            if (!rc && cudaMemset(D.igen, 0xFF, sizeof(int) * ni) != cudaSuccess) rc = SIS_ERR_CUDA;
        }
        rc |= dalloc(ctx, &D.mir0, n);
        rc |= dalloc(ctx, &D.cl_first, n_cl);
        rc |= dalloc(ctx, &D.ncl, n_cl);
        rc |= dalloc(ctx, &D.cl_j, (size_t)n_cl * g.ccap);
        rc |= dalloc(ctx, &D.cl_m, (size_t)n_cl * g.ccap);
    }
    rc |= dalloc(ctx, &D.res[0], n);
    rc |= dalloc(ctx, &D.res[1], n);
    rc |= dalloc(ctx, &D.v, n);
    rc |= dalloc(ctx, &D.beta, n);
    rc |= dalloc(ctx, &D.move, n);
    rc |= dalloc(ctx, &D.mdc, n);
    rc |= dalloc(ctx, &D.fbp, n);
    rc |= dalloc(ctx, &D.binfo, n);
    rc |= dalloc(ctx, &D.mass, n);
    rc |= dalloc(ctx, &D.nbr, (size_t)n * cap);
    rc |= dalloc(ctx, &D.nnbr, n);
    rc |= dalloc(ctx, &D.bps, bp_total_cap);
    rc |= dalloc(ctx, &D.bps_n, bp_total_cap);
    rc |= dalloc(ctx, &D.bp_win, bp_total_cap);
    rc |= dalloc(ctx, &D.bp_nwin, 1);
    rc |= dalloc(ctx, &D.bp_fixq, bp_total_cap);
    rc |= dalloc(ctx, &D.bp_fixn, 1);
    if (g.nstep_mc > 0) {
        rc |= dalloc(ctx, &D.bp_mask, bp_total_cap);
        rc |= dalloc(ctx, &D.bp_frec, (size_t)18 * bp_total_cap);
        rc |= dalloc(ctx, &D.mc_due, ni);
        rc |= dalloc(ctx, &D.mc_excess, n);
        rc |= dalloc(ctx, &D.mc_list, n);
        rc |= dalloc(ctx, &D.mc_seq, bp_total_cap);
        rc |= dalloc(ctx, &D.mc_calls, ni);
        rc |= dalloc(ctx, &D.mc_draw_pos, 1);
    }
    rc |= dalloc(ctx, &D.bp_cnt, 2 * ni);
    rc |= dalloc(ctx, &D.bp_total, 1);
    rc |= dalloc(ctx, &D.ene_bp, bp_total_cap);
    rc |= dalloc(ctx, &D.bp_status, bp_total_cap);
    BPP *bpp_d;
    BPPf *bppf_d;
    short *hash_d;
    double *dH_d, *dS_d;
    rc |= dalloc(ctx, &bpp_d, MAX_BP_TYPES);
    rc |= dalloc(ctx, &bppf_d, MAX_BP_TYPES);
    if (p.precision == SIS_PREC_FP64) {
        double4 *sl;
        rc |= dalloc(ctx, &sl, (size_t)8 * n);
        D.slot = sl;
    } else {
        float4 *sl;
        rc |= dalloc(ctx, &sl, (size_t)8 * n);
        D.slot = sl;
    }
    rc |= dalloc(ctx, &hash_d, 4097);
    rc |= dalloc(ctx, &dH_d, 469);
    rc |= dalloc(ctx, &dS_d, 469);
    rc |= dalloc(ctx, &ctx->dgf_d, (size_t)469 * ni);
    rc |= dalloc(ctx, &ctx->ip_d, ni);
    rc |= dalloc(ctx, &D.m1, 2 * (size_t)ni);
    rc |= dalloc(ctx, &D.m2, 2 * (size_t)ni);
    rc |= dalloc(ctx, &D.gbar, 2);
    rc |= dalloc(ctx, &D.rgb, ni);
    rc |= dalloc(ctx, &D.rgv, ni);
    rc |= dalloc(ctx, &D.gsum, kMaxCoopBlocks);
    rc |= dalloc(ctx, &D.flag, ni);
    rc |= dalloc(ctx, &D.any, 1);
    rc |= dalloc(ctx, &D.ticket, 3);
    rc |= dalloc(ctx, &D.step_ctr, 1);
    rc |= dalloc(ctx, &D.err, 1);
    rc |= dalloc(ctx, &D.max_need, 2);
    rc |= dalloc(ctx, &D.rebuilds, 2); // [0] instance rebuilds, [1] unused
    rc |= dalloc(ctx, &D.capped, 1);
    rc |= dalloc(ctx, &D.bead_cell, n);
    rc |= dalloc(ctx, &D.cell_cnt, ncells);
    rc |= dalloc(ctx, &D.cell_start, ncells + 1);
    rc |= dalloc(ctx, &D.cell_beads, n);
    rc |= dalloc(ctx, &D.ene, (size_t)12 * ni);
    rc |= dalloc(ctx, &ctx->fout_d, (size_t)3 * n);
    {
        double4 *fp = nullptr;
        rc |= dalloc(ctx, &fp, n);
        D.fpair = fp;
    }
    rc |= dalloc(ctx, &D.fbond, n);
    if (cudaStreamCreateWithFlags(&ctx->st3, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&ctx->st4, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->ev_fork, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->ev_join, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->ev_bond, cudaEventDisableTiming) != cudaSuccess)
        rc |= 1;
    if (rc) {
        sis_gpu_destroy(ctx);
        return SIS_ERR_NOMEM;
    }
    if (ctx->coop_grid < 1) {
        sis_gpu_destroy(ctx);
        return SIS_ERR_CUDA;
    }
    D.n_cells = ncells;
    D.bpp = bpp_d;
    D.bppf = bppf_d;
    D.bp3_hash = hash_d;
    D.bp3_dH = dH_d;
    D.bp3_dS = dS_d;
    D.bp_dgf = ctx->dgf_d;
    D.ip = ctx->ip_d;
    std::vector<double4> mdc;
    md_coefs(ctx, mdc);
    // rebuild work items
    std::vector<int2> small, large;
    for (int k = 0; k < ni; ++k) {
        const InstP &I = ctx->ip[k];
        if (I.large)
            for (int l = 0; l < I.n; l += 256) large.push_back(make_int2(k, l));
        else
            for (int l = 0; l < I.n; l += 32) small.push_back(make_int2(k, l));
    }
    std::vector<int2> items(small);
    items.insert(items.end(), large.begin(), large.end());
    if (dalloc(ctx, &ctx->items_d, items.size())) {
        sis_gpu_destroy(ctx);
        return SIS_ERR_NOMEM;
    }
    ctx->plan.small_items = ctx->items_d;
    ctx->plan.n_small_items = (int)small.size();
    ctx->plan.small_grid = std::max(1, std::min((int)small.size(), 4096));
    ctx->plan.large_items = ctx->items_d + small.size();
    ctx->plan.n_large_items = (int)large.size();
    ctx->plan.large_grid = std::max(1, std::min((int)large.size(), 2048));
    // uploads
    bool ok = true;
    ok &= cudaMemcpy(D.binfo, ctx->binfo.data(), sizeof(int4) * n, cudaMemcpyHostToDevice) == cudaSuccess;
    ok &= cudaMemcpy(D.mdc, mdc.data(), sizeof(double4) * n, cudaMemcpyHostToDevice) == cudaSuccess;
    ok &= cudaMemcpy(D.mass, ctx->mass.data(), sizeof(double) * n, cudaMemcpyHostToDevice) == cudaSuccess;
    ok &= cudaMemcpy(bpp_d, ctx->bpp, sizeof(BPP) * MAX_BP_TYPES, cudaMemcpyHostToDevice) == cudaSuccess;
    {
        BPPf bf[MAX_BP_TYPES];
        memset(bf, 0, sizeof(bf));
        for (int t = 1; t < MAX_BP_TYPES; ++t) {
            const BPP &b = ctx->bpp[t];
            BPPf &f = bf[t];
            f.cutoff_ddist = (float)b.cutoff_ddist; f.U0 = (float)b.U0; f.bond_k = (float)b.bond_k; f.bond_r = (float)b.bond_r;
            for (int a = 0; a < 4; ++a) {
                f.angl_k[a] = (float)b.angl_k[a];
                f.angl_theta[a] = (float)b.angl_theta[a];
            }
            for (int a = 0; a < 2; ++a) {
                f.dihd_k[a] = (float)b.dihd_k[a];
                f.dihd_phi[a] = (float)b.dihd_phi[a];
            }
            const double lo = std::max(0.0, b.bond_r - b.cutoff_ddist), hi = b.bond_r + b.cutoff_ddist;
            f.lo2 = (float)(lo * lo);
            f.hi2 = (float)(hi * hi);
        }
        ok &= cudaMemcpy(bppf_d, bf, sizeof(bf), cudaMemcpyHostToDevice) == cudaSuccess;
    }
    ok &= cudaMemcpy(hash_d, hash.data(), sizeof(short) * 4097, cudaMemcpyHostToDevice) == cudaSuccess;
    ok &= cudaMemcpy(dH_d, dH.data(), sizeof(double) * 469, cudaMemcpyHostToDevice) == cudaSuccess;
    ok &= cudaMemcpy(dS_d, dS.data(), sizeof(double) * 469, cudaMemcpyHostToDevice) == cudaSuccess;
    ok &= cudaMemcpy(ctx->ip_d, ctx->ip.data(), sizeof(InstP) * ni, cudaMemcpyHostToDevice) == cudaSuccess;
    ctx->bp3_dH = dH;
    ctx->bp3_dS = dS;
    ctx->dgf.assign((size_t)469 * ni, 0.f);
    for (int k = 0; k < ni && ok; ++k) ok &= upload_dgf(ctx, k) == SIS_OK;
    ok &= cudaStreamSynchronize(ctx->st) == cudaSuccess;
    if (ctx->g.nstep_mc > 0) {
        // job_md.F90:270-273: the first evaluation runs the base-pair Monte Carlo pass
        std::vector<int> due(ni, 1);
        ok &= cudaMemcpy(D.mc_due, due.data(), sizeof(int) * ni, cudaMemcpyHostToDevice) == cudaSuccess;
    }
    if (D.cl_first) {
        std::vector<int> cf;
        cf.reserve(g.n_cl);
        for (int k = 0; k < ni; ++k)
            for (int c = 0; c < ctx->ip[k].n; c += kCl) cf.push_back(ctx->ip[k].bead_off + c);
        ok &= cudaMemcpy(D.cl_first, cf.data(), sizeof(int) * cf.size(), cudaMemcpyHostToDevice) == cudaSuccess;
    }
    ok &= cudaMemcpy(ctx->items_d, items.data(), sizeof(int2) * std::max<size_t>(1, items.size()), cudaMemcpyHostToDevice) ==
          cudaSuccess;
    if (!ok) {
        sis_gpu_destroy(ctx);
        return SIS_ERR_CUDA;
    }
    // lanes per bead from the expected list length
    ctx->G = 8;
    *out = ctx;
    return SIS_OK;
}

extern "C" void sis_gpu_destroy(sis_ctx *ctx) {
    DevGuard dg_(ctx);
    if (!ctx) return;
    if (ctx->st) cudaStreamSynchronize(ctx->st);
    if (ctx->gexec) cudaGraphExecDestroy(ctx->gexec);
    for (void *q : ctx->allocs) cudaFree(q);
    if (ctx->noise_d) cudaFree(ctx->noise_d);
    if (ctx->flush_d) cudaFree(ctx->flush_d);
    if (ctx->pin) cudaFreeHost(ctx->pin);
    for (int e = 0; e < kEvents; ++e)
        if (ctx->ev[e]) cudaEventDestroy(ctx->ev[e]);
    if (ctx->st) cudaStreamDestroy(ctx->st);
    if (ctx->st3) cudaStreamDestroy(ctx->st3);
    if (ctx->st4) cudaStreamDestroy(ctx->st4);
    if (ctx->ev_bond) cudaEventDestroy(ctx->ev_bond);
    if (ctx->ev_fork) cudaEventDestroy(ctx->ev_fork);
    if (ctx->ev_join) cudaEventDestroy(ctx->ev_join);
    if (ctx->mc_draws_d) cudaFree(ctx->mc_draws_d);
    if (ctx->ss_start_d) cudaFree(ctx->ss_start_d);
    if (ctx->ss_part_d) cudaFree(ctx->ss_part_d);
    if (ctx->bias_d) cudaFree(ctx->bias_d);
    delete ctx;
}

extern "C" int sis_gpu_nmp(const sis_ctx *ctx, int32_t inst) {
    if (!ctx || inst < -1 || inst >= ctx->n_inst) return SIS_ERR_ARG;
    return inst < 0 ? ctx->n : ctx->ip[inst].n;
}

extern "C" int sis_gpu_set_state(sis_ctx *ctx, int32_t inst, const double *xyz, const double *velos, const double *accels) {
    DevGuard dg_(ctx);
    if (!ctx) return SIS_ERR_ARG;
    int off, cnt;
    if (inst_range(ctx, inst, off, cnt)) return fail(ctx, SIS_ERR_ARG, "bad instance");
    if (!ctx->pin) CK(cudaMallocHost((void **)&ctx->pin, sizeof(double4) * ctx->n));
    double4 *h = ctx->pin;
    const double *src[3] = {xyz, velos, accels};
    double4 *dst[3] = {ctx->D.x[ctx->cur], ctx->D.v, ctx->D.beta};
    for (int f = 0; f < 3; ++f) {
        if (!src[f]) continue;
        for (int i = 0; i < cnt; ++i) h[i] = make_double4(src[f][3 * i], src[f][3 * i + 1], src[f][3 * i + 2], 0.0);
        CK(cudaMemcpyAsync(dst[f] + off, h, sizeof(double4) * cnt, cudaMemcpyHostToDevice, ctx->st));
        CK(cudaStreamSynchronize(ctx->st));
    }
    if (xyz) {
        CK(launch_mirror(ctx->D, ctx->g, ctx->cur, ctx->st));
        ctx->launches++;
        ctx->lists_valid = false;
        ctx->bp_cache = false;
        if (inst < 0) ctx->state_set = true;
        else ctx->state_set = true;
    }
    return SIS_OK;
}

extern "C" int sis_gpu_get_state(sis_ctx *ctx, int32_t inst, double *xyz, double *velos, double *accels) {
    DevGuard dg_(ctx);
    if (!ctx) return SIS_ERR_ARG;
    int off, cnt;
    if (inst_range(ctx, inst, off, cnt)) return fail(ctx, SIS_ERR_ARG, "bad instance");
    if (!ctx->pin) CK(cudaMallocHost((void **)&ctx->pin, sizeof(double4) * ctx->n));
    double4 *h = ctx->pin;
    double *dst[3] = {xyz, velos, accels};
    const double4 *src[3] = {ctx->D.x[ctx->cur], ctx->D.v, ctx->D.beta};
    for (int f = 0; f < 3; ++f) {
        if (!dst[f]) continue;
        CK(cudaMemcpyAsync(h, src[f] + off, sizeof(double4) * cnt, cudaMemcpyDeviceToHost, ctx->st));
        CK(cudaStreamSynchronize(ctx->st));
        for (int i = 0; i < cnt; ++i) {
            dst[f][3 * i] = h[i].x;
            dst[f][3 * i + 1] = h[i].y;
            dst[f][3 * i + 2] = h[i].z;
        }
    }
    return SIS_OK;
}

extern "C" int sis_gpu_init_velocities(sis_ctx *ctx) {
    DevGuard dg_(ctx);
    if (!ctx) return SIS_ERR_ARG;
    const unsigned long long ctr = (1ull << 62) + 2ull * (unsigned long long)(ctx->n_vel_init++);
    CK(launch_init_velocities(ctx->D, ctx->g, ctr, ctx->st));
    ctx->launches++;
    CK(cudaStreamSynchronize(ctx->st));
    return SIS_OK;
}

extern "C" int sis_gpu_neighbor_list(sis_ctx *ctx, int32_t inst) {
    DevGuard dg_(ctx);
    if (!ctx || inst < -1 || inst >= ctx->n_inst) return SIS_ERR_ARG;
    if (!ctx->state_set) return fail(ctx, SIS_ERR_STATE, "coordinates have not been set");
    if (!ctx->lists_valid) inst = -1;
    int rc = flag_all(ctx, inst);
    if (rc) return rc;
    rc = run_rebuild(ctx);
    if (rc) return rc;
    ctx->lists_valid = true;
    ctx->bp_cache = false;
    CK(cudaStreamSynchronize(ctx->st));
    return check_err(ctx);
}

extern "C" int sis_gpu_get_list(sis_ctx *ctx, int32_t inst, int32_t kind, int32_t *out, int32_t cap, int32_t *n_out) {
    DevGuard dg_(ctx);
    if (!ctx || inst < 0 || inst >= ctx->n_inst || kind < 0 || kind > 4 || !n_out) return SIS_ERR_ARG;
    const bool inner = kind == SIS_LIST_WCA_INNER || kind == SIS_LIST_ELE_INNER;
    if (inner && !ctx->D.nbr_in) return fail(ctx, SIS_ERR_ARG, "get_list: inner lists exist for contexts of small instances only");
    int rc = ensure_lists(ctx);
    if (rc) return rc;
    const InstP &I = ctx->ip[inst];
    const int off = I.bead_off, cnt = I.n;
    std::vector<int> res;
    if (kind != SIS_LIST_BP) {
        std::vector<int> nn(cnt), nb((size_t)cnt * ctx->g.cap);
        CK(cudaMemcpyAsync(nn.data(), (inner ? ctx->D.nnbr_in : ctx->D.nnbr) + off, sizeof(int) * cnt, cudaMemcpyDeviceToHost, ctx->st));
        CK(cudaMemcpyAsync(nb.data(), (inner ? ctx->D.nbr_in : ctx->D.nbr) + (size_t)off * ctx->g.cap, sizeof(int) * nb.size(),
                           cudaMemcpyDeviceToHost, ctx->st));
        CK(cudaStreamSynchronize(ctx->st));
        const int bit = (kind == SIS_LIST_WCA || kind == SIS_LIST_WCA_INNER) ? WCA_BIT : ELE_BIT;
        for (int i = 0; i < cnt; ++i) {
            const int c = std::min(nn[i], ctx->g.cap);
            for (int k = 0; k < c; ++k) {
                const int e = nb[(size_t)i * ctx->g.cap + k];
                const int j = (e & IDX_MASK) - off;
                if ((e & bit) && j > i) {
                    res.push_back(i + 1);
                    res.push_back(j + 1);
                }
            }
        }
        *n_out = (int)(res.size() / 2);
        if (out) memcpy(out, res.data(), sizeof(int) * std::min<size_t>(res.size(), (size_t)cap * 2));
    } else {
        int c = 0;
        CK(cudaMemcpyAsync(&c, ctx->D.bp_cnt + inst, sizeof(int), cudaMemcpyDeviceToHost, ctx->st));
        CK(cudaStreamSynchronize(ctx->st));
        c = std::min(c, I.bp_cap);
        std::vector<int4> r(std::max(c, 1)), q(std::max(c, 1));
        CK(cudaMemcpyAsync(r.data(), ctx->D.bps + I.bp_off, sizeof(int4) * c, cudaMemcpyDeviceToHost, ctx->st));
        CK(cudaMemcpyAsync(q.data(), ctx->D.bps_n + I.bp_off, sizeof(int4) * c, cudaMemcpyDeviceToHost, ctx->st));
        CK(cudaStreamSynchronize(ctx->st));
        for (int k = 0; k < c; ++k) {
            const int rec[7] = {r[k].x - off + 1, r[k].y - off + 1, q[k].x - off + 1, q[k].y - off + 1,
                                q[k].z - off + 1, q[k].w - off + 1, r[k].z & 0xff};
            res.insert(res.end(), rec, rec + 7);
        }
        *n_out = c;
        if (out) memcpy(out, res.data(), sizeof(int) * std::min<size_t>(res.size(), (size_t)cap * 7));
    }
    return SIS_OK;
}

extern "C" int sis_gpu_get_bp_coef(sis_ctx *ctx, int32_t inst, double *out, int32_t cap, int32_t *n_out) {
    DevGuard dg_(ctx);
    if (!ctx || inst < 0 || inst >= ctx->n_inst || !n_out) return SIS_ERR_ARG;
    int rc = ensure_lists(ctx);
    if (rc) return rc;
    const InstP &I = ctx->ip[inst];
    int c = 0;
    CK(cudaMemcpyAsync(&c, ctx->D.bp_cnt + inst, sizeof(int), cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
    c = std::min(c, I.bp_cap);
    std::vector<int4> r(std::max(c, 1));
    std::vector<double> dH(469), dS(469);
    CK(cudaMemcpyAsync(r.data(), ctx->D.bps + I.bp_off, sizeof(int4) * c, cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaMemcpyAsync(dH.data(), ctx->D.bp3_dH, sizeof(double) * 469, cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaMemcpyAsync(dS.data(), ctx->D.bp3_dS, sizeof(double) * 469, cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
    for (int k = 0; k < c && k < cap; ++k) {
        const int h = r[k].z >> 8;
        out[2 * k] = dH[h];
        out[2 * k + 1] = dS[h];
    }
    *n_out = c;
    return SIS_OK;
}

static int force_common(sis_ctx *ctx, int32_t inst, int mask, double *forces) {
    int off, cnt;
    if (inst_range(ctx, inst, off, cnt)) return fail(ctx, SIS_ERR_ARG, "bad instance");
    int rc = ensure_lists(ctx);
    if (rc) return rc;
    const int do_bp = (mask & 8) && ctx->g.bp_model > 0;
    CK(launch_pre(ctx->D, ctx->g, ctx->cur, (mask & 7) != 0, do_bp, bp_test_blocks(ctx), bp_blocks(ctx), ctx->st));
    ctx->launches += pre_kernels(ctx->g, (mask & 7) != 0, do_bp);
    if (do_bp && ctx->g.nstep_mc > 0) {
        CK(launch_bp_mc(ctx->D, ctx->g, ctx->st));
        ctx->launches++;
    }
    if (do_bp) ctx->bp_cache = true;
    if (mask & 128) {
        CK(launch_bias(ctx->D, ctx->g, ctx->cur, 0, ctx->st));
        ctx->launches += bias_kernels(ctx->g);
    }
    CK(launch_force(ctx->G, ctx->D, ctx->g, ctx->cur, ctx->fout_d, mask, ctx->st));
    ctx->launches += force_kernels(ctx->g, mask);
    if (forces) CK(cudaMemcpyAsync(forces, ctx->fout_d + 3 * (size_t)off, sizeof(double) * 3 * cnt, cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
    if (do_bp) {
        ctx->D.mc_draws = nullptr;
        ctx->mc_pending = false;
    }
    return check_err(ctx);
}

extern "C" int sis_gpu_force(sis_ctx *ctx, int32_t inst, double *forces) {
    DevGuard dg_(ctx);
    if (!ctx) return SIS_ERR_ARG;
    return force_common(ctx, inst, 63 | 128, forces);
}

extern "C" int sis_gpu_force_term(sis_ctx *ctx, int32_t inst, int32_t term, double *forces) {
    DevGuard dg_(ctx);
    if (!ctx || term < 1 || term > 7) return SIS_ERR_ARG;
    return force_common(ctx, inst, term == 7 ? 128 : 1 << (term - 1), forces);
}

extern "C" int sis_gpu_rg(sis_ctx *ctx, int32_t inst, double *rg) {
    DevGuard dg_(ctx);
    if (!ctx || !rg || inst < -1 || inst >= ctx->n_inst) return SIS_ERR_ARG;
    if (!ctx->state_set) return fail(ctx, SIS_ERR_STATE, "coordinates have not been set");
    CK(launch_rg(ctx->D, ctx->g, ctx->cur, ctx->fout_d, ctx->st));
    ctx->launches++;
    const int off = inst < 0 ? 0 : inst, cnt = inst < 0 ? ctx->n_inst : 1;
    CK(cudaMemcpyAsync(rg, ctx->fout_d + off, sizeof(double) * cnt, cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
    return SIS_OK;
}

extern "C" int sis_gpu_invalidate_bp_cache(sis_ctx *ctx) {
    DevGuard dg_(ctx);
    if (!ctx) return SIS_ERR_ARG;
    ctx->bp_cache = false;
    return SIS_OK;
}

extern "C" int sis_gpu_energy_sumup(sis_ctx *ctx, int32_t inst, double tempK, double *E) {
    DevGuard dg_(ctx);
    if (!ctx || inst < 0 || inst >= ctx->n_inst || !E) return SIS_ERR_ARG;
    int rc = ensure_lists(ctx);
    if (rc) return rc;
    if (!ctx->bp_cache && ctx->g.bp_model > 0) {
        CK(launch_bp_energy(ctx->D, ctx->g, ctx->cur, tempK, bp_blocks(ctx), ctx->st));
        ctx->launches++;
    }
    CK(cudaMemsetAsync(ctx->D.ene, 0, sizeof(double) * 12 * ctx->n_inst, ctx->st));
    CK(launch_energy(ctx->D, ctx->g, ctx->cur, ctx->st));
    CK(launch_bias_energy(ctx->D, ctx->g, ctx->cur, ctx->st));
    ctx->launches += 2 + (ctx->g.flg_bias ? 1 + ctx->g.flg_rg : 0);
    double h[12];
    CK(cudaMemcpyAsync(h, ctx->D.ene + 12 * (size_t)inst, sizeof(double) * 12, cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
    for (int k = 0; k <= SIS_ENE_MAX; ++k) E[k] = k == 0 ? 0.0 : h[k];
    double tot = 0.0;
    for (int k = 1; k <= SIS_ENE_MAX; ++k) tot += E[k];
    E[0] = tot;
    return SIS_OK;
}

extern "C" int sis_gpu_energy_kinetic(sis_ctx *ctx, int32_t inst, double *ekin) {
    DevGuard dg_(ctx);
    if (!ctx || inst < 0 || inst >= ctx->n_inst || !ekin) return SIS_ERR_ARG;
    int rc = ensure_lists(ctx);
    if (rc) return rc;
    CK(cudaMemsetAsync(ctx->D.ene, 0, sizeof(double) * 12 * ctx->n_inst, ctx->st));
    CK(launch_energy(ctx->D, ctx->g, ctx->cur, ctx->st));
    ctx->launches += 2;
    double h[12];
    CK(cudaMemcpyAsync(h, ctx->D.ene + 12 * (size_t)inst, sizeof(double) * 12, cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
    *ekin = h[11];
    return SIS_OK;
}

extern "C" int sis_gpu_step(sis_ctx *ctx, int64_t nsteps, const double *noise) {
    DevGuard dg_(ctx);
    if (!ctx || nsteps < 0) return SIS_ERR_ARG;
    int rc = ensure_lists(ctx, nsteps > 0 && small_active(ctx));
    if (rc) return rc;
    if (!noise && nsteps >= 64 && !small_active(ctx) && (rc = autotune(ctx))) return rc;
    if (noise) {
        const size_t need = (size_t)nsteps * ctx->n * 3;
        if (need > ctx->noise_cap) {
            if (ctx->noise_d) cudaFree(ctx->noise_d);
            ctx->noise_d = nullptr;
            if (cudaMalloc(&ctx->noise_d, sizeof(double) * need) != cudaSuccess) return fail(ctx, SIS_ERR_NOMEM, "noise buffer");
            ctx->noise_cap = need;
        }
        CK(cudaMemcpyAsync(ctx->noise_d, noise, sizeof(double) * need, cudaMemcpyHostToDevice, ctx->st));
    }
    if (small_active(ctx)) {
        int64_t done = 0;
        if (!noise && !ctx->small_tuned) {
            done = small_autotune(ctx, nsteps, &rc);
            if (rc) return rc;
        } else if (!ctx->sp.n_cta && (rc = small_plan(ctx, std::min(ctx->n_inst, 2 * ctx->sms)))) {
            return rc;
        } else if (ctx->small_tuned && ctx->steps - ctx->small_planned >= kSmallReplan) {
            // the instances' list lengths drift as they fold or unfold: the
            // buckets are balanced again on the current lists (the trajectory
            // does not depend on them)
            if ((rc = small_plan(ctx, ctx->small_target))) return rc;
            ctx->small_planned = ctx->steps;
        }
        if ((rc = run_small(ctx, nsteps - done, noise ? ctx->noise_d + (size_t)done * ctx->n * 3 : nullptr))) return rc;
        ctx->steps += nsteps;
        ctx->bp_cache = true;
        CK(cudaStreamSynchronize(ctx->st));
        ctx->D.mc_draws = nullptr;
        ctx->mc_pending = false;
        return check_err(ctx);
    }
    int64_t s = 0;
    bool graphs = false;
    if (!noise && ctx->use_graphs && !ctx->mc_pending && nsteps >= kGraphSteps) {
        if ((rc = ensure_step_graph(ctx))) return rc;
        for (; s + kGraphSteps <= nsteps; s += kGraphSteps) CK(cudaGraphLaunch(ctx->gexec, ctx->st));
        ctx->launches += (step_kernels(ctx) + 1) * s;
        graphs = true;
    }
    for (; s < nsteps; ++s) {
        rc = enqueue_step(ctx, noise ? ctx->noise_d : nullptr, (long long)s);
        if (rc) return rc;
    }
    ctx->steps += nsteps;
    ctx->bp_cache = true;
    CK(cudaStreamSynchronize(ctx->st));
    ctx->D.mc_draws = nullptr;
    ctx->mc_pending = false;
    (void)graphs;
    return check_err(ctx);
}

extern "C" int sis_gpu_set_condition(sis_ctx *ctx, int32_t inst, double tempK, double ionic) {
    DevGuard dg_(ctx);
    if (!ctx || inst < 0 || inst >= ctx->n_inst || tempK <= 0 || ionic <= 0) return SIS_ERR_ARG;
    ctx->ip[inst].tempK = tempK;
    ctx->ionic[inst] = ionic;
    set_ele(ctx, inst);
    std::vector<double4> mdc;
    md_coefs(ctx, mdc);
    const InstP &I = ctx->ip[inst];
    CK(cudaMemcpyAsync(ctx->D.mdc + I.bead_off, mdc.data() + I.bead_off, sizeof(double4) * I.n, cudaMemcpyHostToDevice, ctx->st));
    int rc = upload_ip(ctx);
    if (!rc) rc = upload_dgf(ctx, inst);
    if (rc) return rc;
    CK(cudaStreamSynchronize(ctx->st));
    return SIS_OK;
}

extern "C" int sis_gpu_set_temperature(sis_ctx *ctx, int32_t inst, double tempK) {
    DevGuard dg_(ctx);
    if (!ctx || inst < -1 || inst >= ctx->n_inst || !(tempK > 0.0)) return SIS_ERR_ARG;
    // the temperature ladder of replica exchange owns the temperatures
    if (ctx->remd_on) return fail(ctx, SIS_ERR_ARG, "set_temperature: replica exchange is on");
    const int k0 = inst < 0 ? 0 : inst, k1 = inst < 0 ? ctx->n_inst : inst + 1;
    for (int k = k0; k < k1; ++k) ctx->ip[k].tempK = tempK;
    std::vector<double4> mdc;
    md_coefs(ctx, mdc);
    for (int k = k0; k < k1; ++k) {
        const InstP &I = ctx->ip[k];
        CK(cudaMemcpyAsync(ctx->D.mdc + I.bead_off, mdc.data() + I.bead_off, sizeof(double4) * I.n, cudaMemcpyHostToDevice,
                           ctx->st));
    }
    int rc = upload_ip(ctx);
    for (int k = k0; k < k1 && !rc; ++k) rc = upload_dgf(ctx, k);
    if (rc) return rc;
    ctx->bp_cache = false;
    CK(cudaStreamSynchronize(ctx->st));
    return SIS_OK;
}

extern "C" int sis_gpu_set_frozen(sis_ctx *ctx, int32_t inst, const int32_t *beads, int32_t n) {
    DevGuard dg_(ctx);
    if (!ctx || inst < 0 || inst >= ctx->n_inst || n < 0 || (n > 0 && !beads)) return SIS_ERR_ARG;
    const InstP &I = ctx->ip[inst];
    for (int q = 0; q < n; ++q)
        if (beads[q] < 1 || beads[q] > I.n) return fail(ctx, SIS_ERR_ARG, "set_frozen: bead number out of range");
    if (ctx->frozen.size() != (size_t)ctx->n) ctx->frozen.assign((size_t)ctx->n, 0);
    std::fill(ctx->frozen.begin() + I.bead_off, ctx->frozen.begin() + I.bead_off + I.n, (uint8_t)0);
    for (int q = 0; q < n; ++q) ctx->frozen[(size_t)I.bead_off + beads[q] - 1] = 1;
    std::vector<double4> mdc;
    md_coefs(ctx, mdc);
    CK(cudaMemcpyAsync(ctx->D.mdc + I.bead_off, mdc.data() + I.bead_off, sizeof(double4) * I.n, cudaMemcpyHostToDevice,
                       ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
    return SIS_OK;
}

// -------------------------------------------------- secondary structure
namespace {
// the partner table of every instance's allowed pairs (CSR over global beads)
int upload_ss(sis_ctx *ctx) {
    std::vector<std::vector<int>> part(ctx->n);
    int any = 0;
    for (int k = 0; k < ctx->n_inst; ++k) {
        ctx->ip[k].ss_on = ctx->ss_pairs[k].empty() ? 0 : 1;
        any |= ctx->ip[k].ss_on;
        for (const int2 &pq : ctx->ss_pairs[k]) {
            part[pq.x].push_back(pq.y);
            part[pq.y].push_back(pq.x);
        }
    }
    std::vector<int> start(ctx->n + 1, 0), flat;
    for (int i = 0; i < ctx->n; ++i) {
        std::sort(part[i].begin(), part[i].end());
        part[i].erase(std::unique(part[i].begin(), part[i].end()), part[i].end());
        start[i + 1] = start[i] + (int)part[i].size();
        flat.insert(flat.end(), part[i].begin(), part[i].end());
    }
    if (ctx->ss_start_d) cudaFree(ctx->ss_start_d);
    if (ctx->ss_part_d) cudaFree(ctx->ss_part_d);
    ctx->ss_start_d = ctx->ss_part_d = nullptr;
    CK(cudaMalloc(&ctx->ss_start_d, sizeof(int) * start.size()));
    CK(cudaMalloc(&ctx->ss_part_d, sizeof(int) * std::max<size_t>(1, flat.size())));
    CK(cudaMemcpy(ctx->ss_start_d, start.data(), sizeof(int) * start.size(), cudaMemcpyHostToDevice));
    if (!flat.empty()) CK(cudaMemcpy(ctx->ss_part_d, flat.data(), sizeof(int) * flat.size(), cudaMemcpyHostToDevice));
    ctx->D.ss_start = ctx->ss_start_d;
    ctx->D.ss_part = ctx->ss_part_d;
    ctx->g.any_ss = any;
    return SIS_OK;
}

// base-pair list cutoff of every instance: (bp_cutoff_dist + margin)^2, or
// with [Bias_SS] the reference's 9999999999.9 (a REAL(4) literal: 1e10)
void bp_list_cut(sis_ctx *ctx) {
    const double m = ctx->p.nl_margin;
    for (int k = 0; k < ctx->n_inst; ++k)
        ctx->ip[k].bp_nl_cut2 = ctx->g.flg_bias_ss ? (double)9999999999.9f : (ctx->bp_cutoff_dist + m) * (ctx->bp_cutoff_dist + m);
}
} // namespace

extern "C" int sis_gpu_set_ss_pairs(sis_ctx *ctx, int32_t inst, int32_t n, const int32_t *pairs) {
    DevGuard dg_(ctx);
    if (!ctx || inst < 0 || inst >= ctx->n_inst || n < 0 || (n > 0 && !pairs)) return SIS_ERR_ARG;
    const InstP &I = ctx->ip[inst];
    std::vector<int2> pq;
    for (int q = 0; q < n; ++q) {
        int i = pairs[2 * q], j = pairs[2 * q + 1];
        if (i < 1 || j < 1 || i > I.n || j > I.n || i == j)
            return fail(ctx, SIS_ERR_ARG, "set_ss_pairs: nucleotide number out of range");
        if (j < i) std::swap(i, j);
        pq.push_back(make_int2(I.bead_off + i - 1, I.bead_off + j - 1));
    }
    if (ctx->ss_pairs.size() != (size_t)ctx->n_inst) ctx->ss_pairs.assign(ctx->n_inst, {});
    ctx->ss_pairs[inst] = pq;
    int rc = upload_ss(ctx);
    if (rc) return rc;
    if ((rc = upload_ip(ctx))) return rc;
    ctx->lists_valid = false;
    return SIS_OK;
}

extern "C" int sis_gpu_set_bias_ss(sis_ctx *ctx, int32_t on, double force) {
    DevGuard dg_(ctx);
    if (!ctx || !std::isfinite(force) || force < 0.0) return SIS_ERR_ARG;
    ctx->g.flg_bias_ss = on ? 1 : 0;
    ctx->g.bias_ss_force = force;
    bp_list_cut(ctx);
    const int rc = upload_ip(ctx);
    if (rc) return rc;
    ctx->lists_valid = false;
    return SIS_OK;
}

// ------------------------------------------------------- optional terms
namespace {
void bias_flags(sis_ctx *ctx) {
    GlobP &g = ctx->g;
    g.flg_rg = 0;
    for (const InstP &I : ctx->ip) g.flg_rg |= I.rg_pott != 0;
    size_t n = 0;
    for (const auto &v : ctx->bias_items) n += v.size();
    g.n_bias = (int)n;
    g.flg_bias = g.flg_stage || g.flg_rg || g.n_bias > 0;
}
} // namespace

extern "C" int sis_gpu_set_stage(sis_ctx *ctx, double sigma, double eps) {
    DevGuard dg_(ctx);
    if (!ctx || !(sigma >= 0.0)) return SIS_ERR_ARG;
    ctx->g.flg_stage = sigma > 0.0;
    ctx->g.stage_sigma = sigma;
    ctx->g.stage_eps = eps;
    bias_flags(ctx);
    return SIS_OK;
}

extern "C" int sis_gpu_set_rg_bias(sis_ctx *ctx, int32_t inst, int32_t pott, double k, double rg0) {
    DevGuard dg_(ctx);
    if (!ctx || inst < -1 || inst >= ctx->n_inst || pott < 0 || pott > 2) return SIS_ERR_ARG;
    for (int q = 0; q < ctx->n_inst; ++q) {
        if (inst >= 0 && q != inst) continue;
        ctx->ip[q].rg_pott = pott;
        ctx->ip[q].rg_k = k;
        ctx->ip[q].rg0 = rg0;
    }
    int rc = upload_ip(ctx);
    if (rc) return rc;
    bias_flags(ctx);
    return SIS_OK;
}

extern "C" int sis_gpu_set_bias_items(sis_ctx *ctx, int32_t inst, int32_t n, const int32_t *kind_ij, const double *par) {
    DevGuard dg_(ctx);
    if (!ctx || inst < 0 || inst >= ctx->n_inst || n < 0 || (n > 0 && (!kind_ij || !par))) return SIS_ERR_ARG;
    if (ctx->bias_items.empty()) ctx->bias_items.resize(ctx->n_inst);
    const InstP &I = ctx->ip[inst];
    std::vector<BiasItem> items((size_t)n);
    for (int q = 0; q < n; ++q) {
        BiasItem &b = items[q];
        b.kind = kind_ij[3 * q];
        const int i = kind_ij[3 * q + 1], j = kind_ij[3 * q + 2];
        if (b.kind < 1 || b.kind > 4 || i < 1 || i > I.n || j < 1 || j > I.n) return fail(ctx, SIS_ERR_ARG, "bad restraint or trap item");
        b.i = I.bead_off + i - 1;
        b.j = I.bead_off + j - 1;
        b.inst = inst;
        for (int k = 0; k < 14; ++k) b.p[k] = par[14 * (size_t)q + k];
        if (b.kind <= 2 && !(b.p[2] != 0.0)) return fail(ctx, SIS_ERR_ARG, "restraint width s must be nonzero");
    }
    ctx->bias_items[inst] = std::move(items);
    std::vector<BiasItem> flat;
    for (const auto &v : ctx->bias_items) flat.insert(flat.end(), v.begin(), v.end());
    if (flat.size() > ctx->bias_cap) {
        if (ctx->bias_d) cudaFree(ctx->bias_d);
        ctx->bias_d = nullptr;
        ctx->bias_cap = 0;
        if (cudaMalloc(&ctx->bias_d, sizeof(BiasItem) * flat.size()) != cudaSuccess) return fail(ctx, SIS_ERR_NOMEM, "bias items");
        ctx->bias_cap = flat.size();
    }
    if (!flat.empty()) {
        CK(cudaMemcpyAsync(ctx->bias_d, flat.data(), sizeof(BiasItem) * flat.size(), cudaMemcpyHostToDevice, ctx->st));
        CK(cudaStreamSynchronize(ctx->st));
    }
    ctx->D.bias = ctx->bias_d;
    bias_flags(ctx);
    return SIS_OK;
}

extern "C" int sis_gpu_set_force_cap(sis_ctx *ctx, double fmax) {
    DevGuard dg_(ctx);
    if (!ctx || fmax < 0.0) return SIS_ERR_ARG;
    ctx->g.fcap = fmax;
    ctx->g.fcap_f = (float)fmax;
    return SIS_OK;
}

extern "C" int sis_gpu_get_md_coef(sis_ctx *ctx, int32_t inst, double *o) {
    DevGuard dg_(ctx);
    if (!ctx || !o) return SIS_ERR_ARG;
    int off, cnt;
    if (inst_range(ctx, inst, off, cnt)) return fail(ctx, SIS_ERR_ARG, "bad instance");
    CK(cudaMemcpyAsync(o, ctx->D.mdc + off, sizeof(double4) * cnt, cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
    return SIS_OK;
}

extern "C" int sis_gpu_get_ele(sis_ctx *ctx, int32_t inst, double *o) {
    DevGuard dg_(ctx);
    if (!ctx || inst < 0 || inst >= ctx->n_inst || !o) return SIS_ERR_ARG;
    const InstP &I = ctx->ip[inst];
    o[0] = I.ele_coef;
    o[1] = 1.0 / I.rcdist;
    o[2] = I.ele_cut;
    o[3] = I.diele;
    return SIS_OK;
}

extern "C" int sis_gpu_get_step(sis_ctx *ctx, uint64_t *step) {
    DevGuard dg_(ctx);
    if (!ctx || !step) return SIS_ERR_ARG;
    unsigned long long v = 0;
    CK(cudaMemcpyAsync(&v, ctx->D.step_ctr, sizeof(v), cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
    *step = v;
    return SIS_OK;
}

extern "C" int sis_gpu_set_step(sis_ctx *ctx, uint64_t step) {
    DevGuard dg_(ctx);
    if (!ctx) return SIS_ERR_ARG;
    unsigned long long v = step;
    CK(cudaMemcpyAsync(ctx->D.step_ctr, &v, sizeof(v), cudaMemcpyHostToDevice, ctx->st));
    // the displacement maxima are kept by step parity: start both afresh
    CK(cudaMemsetAsync(ctx->D.m1, 0, sizeof(unsigned long long) * 2 * ctx->n_inst, ctx->st));
    CK(cudaMemsetAsync(ctx->D.m2, 0, sizeof(unsigned long long) * 2 * ctx->n_inst, ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
    return SIS_OK;
}

extern "C" int sis_gpu_set_lanes(sis_ctx *ctx, int32_t lanes) {
    DevGuard dg_(ctx);
    if (!ctx || !(lanes == 0 || lanes == 1 || lanes == 2 || lanes == 4 || lanes == 8 || lanes == 16 || lanes == 32))
        return SIS_ERR_ARG;
    ctx->lanes_fixed = lanes != 0;
    if (lanes != 0) ctx->G = lanes;
    // the overlap is still the autotuner's to choose unless it was fixed too
    ctx->tuned = ctx->lanes_fixed && ctx->overlap_mode >= 0;
    return SIS_OK;
}

extern "C" int sis_gpu_set_graphs(sis_ctx *ctx, int32_t enable) {
    DevGuard dg_(ctx);
    if (!ctx || (enable != 0 && enable != 1)) return SIS_ERR_ARG;
    ctx->use_graphs = enable != 0;
    return SIS_OK;
}

extern "C" int sis_gpu_set_overlap(sis_ctx *ctx, int32_t enable) {
    DevGuard dg_(ctx);
    if (!ctx || (enable != 0 && enable != 1 && enable != -1)) return SIS_ERR_ARG;
    ctx->overlap_mode = enable;
    if (enable >= 0) ctx->overlap = enable != 0;
    ctx->tuned = ctx->lanes_fixed && ctx->overlap_mode >= 0;
    return SIS_OK;
}

extern "C" int sis_gpu_set_small(sis_ctx *ctx, int32_t mode) {
    DevGuard dg_(ctx);
    if (!ctx || mode < -1 || mode > 1) return SIS_ERR_ARG;
    ctx->small_mode = mode;
    return SIS_OK;
}

extern "C" int sis_gpu_probe_barrier_timeout(sis_ctx *ctx) {
    DevGuard dg_(ctx);
    if (!ctx) return SIS_ERR_ARG;
    CK(launch_barrier_probe(ctx->D, ctx->coop_grid, ctx->coop_grid - 1, ctx->st));
    ctx->launches++;
    return check_err(ctx);
}

extern "C" int sis_gpu_get_stats(sis_ctx *ctx, sis_stats *s) {
    DevGuard dg_(ctx);
    if (!ctx || !s) return SIS_ERR_ARG;
    memset(s, 0, sizeof(*s));
    s->steps = ctx->steps;
    s->n_beads = ctx->n;
    s->n_inst = ctx->n_inst;
    s->lanes_per_bead = ctx->G;
    s->bp_blocks = bp_blocks(ctx);
    s->overlap = ctx->overlap ? 1 : 0;
    s->small_blocks = small_active(ctx) ? ctx->sp.n_cta : 0;
    s->small_threads = small_active(ctx) ? ctx->small_threads : 0;
    long long rb = 0;
    unsigned long long cp = 0;
    int e = 0;
    CK(cudaMemcpyAsync(&rb, ctx->D.rebuilds, sizeof(long long), cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaMemcpyAsync(&cp, ctx->D.capped, sizeof(cp), cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaMemcpyAsync(&e, ctx->D.err, sizeof(int), cudaMemcpyDeviceToHost, ctx->st));
    std::vector<int> nn(ctx->n), bc(ctx->n_inst);
    CK(cudaMemcpyAsync(nn.data(), ctx->D.nnbr, sizeof(int) * ctx->n, cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaMemcpyAsync(bc.data(), ctx->D.bp_cnt, sizeof(int) * ctx->n_inst, cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
    s->rebuilds = rb;
    s->capped = (int64_t)cp;
    s->error_flags = e;
    for (int i = 0; i < ctx->n; ++i) s->pair_entries += std::min(nn[i], ctx->g.cap);
    for (int k = 0; k < ctx->n_inst; ++k) s->bp_pairs += std::min(bc[k], ctx->ip[k].bp_cap);
    if (ctx->g.prec != 0 && ctx->g.n_cl > 0) {
        std::vector<int> nc(ctx->g.n_cl);
        CK(cudaMemcpyAsync(nc.data(), ctx->D.ncl, sizeof(int) * nc.size(), cudaMemcpyDeviceToHost, ctx->st));
        CK(cudaStreamSynchronize(ctx->st));
        for (int c : nc)
            if (c >= 0) {
                s->cluster_pairs += c;
                ++s->i_clusters;
            }
    }
    return SIS_OK;
}

extern "C" const char *sis_gpu_last_error(const sis_ctx *ctx) { return ctx ? ctx->err.c_str() : "null context"; }

extern "C" int sis_gpu_event_record(sis_ctx *ctx, int32_t slot) {
    DevGuard dg_(ctx);
    if (!ctx || slot < 0 || slot >= kEvents) return SIS_ERR_ARG;
    CK(cudaEventRecord(ctx->ev[slot], ctx->st));
    return SIS_OK;
}
extern "C" int sis_gpu_event_elapsed(sis_ctx *ctx, int32_t a, int32_t b, float *ms) {
    DevGuard dg_(ctx);
    if (!ctx || a < 0 || b < 0 || a >= kEvents || b >= kEvents || !ms) return SIS_ERR_ARG;
    CK(cudaEventSynchronize(ctx->ev[b]));
    CK(cudaEventElapsedTime(ms, ctx->ev[a], ctx->ev[b]));
    return SIS_OK;
}
extern "C" int sis_gpu_synchronize(sis_ctx *ctx) {
    DevGuard dg_(ctx);
    if (!ctx) return SIS_ERR_ARG;
    CK(cudaStreamSynchronize(ctx->st));
    return SIS_OK;
}
extern "C" int sis_gpu_flush_l2(sis_ctx *ctx) {
    DevGuard dg_(ctx);
    if (!ctx) return SIS_ERR_ARG;
    if (!ctx->flush_d) {
        ctx->flush_bytes = (size_t)512 << 20;
        if (cudaMalloc(&ctx->flush_d, ctx->flush_bytes) != cudaSuccess) return fail(ctx, SIS_ERR_NOMEM, "flush buffer");
    }
    CK(cudaMemsetAsync(ctx->flush_d, ctx->launches & 0xff, ctx->flush_bytes, ctx->st));
    return SIS_OK;
}
extern "C" int64_t sis_gpu_kernel_launches(const sis_ctx *ctx) { return ctx ? ctx->launches : 0; }

extern "C" int sis_gpu_step_profiled(sis_ctx *ctx, int64_t nsteps, float *ms3) {
    DevGuard dg_(ctx);
    if (!ctx || nsteps < 0 || !ms3) return SIS_ERR_ARG;
    int rc = ensure_lists(ctx);
    if (rc) return rc;
    if ((rc = autotune(ctx))) return rc;
    double acc[3] = {0.0, 0.0, 0.0};
    cudaEvent_t *e = ctx->ev + 8; // events 8..11
    for (int64_t s = 0; s < nsteps; ++s) {
        // the passes one after the other on ctx->st, so that each is timed alone
        CK(cudaEventRecord(e[0], ctx->st));
        CK(cudaEventRecord(ctx->ev_fork, ctx->st));
        CK(enqueue_pre(ctx, ctx->cur));
        CK(launch_bias(ctx->D, ctx->g, ctx->cur, 1, ctx->st));
        ctx->launches += pre_step_kernels(ctx) + bias_kernels(ctx->g);
        CK(cudaEventRecord(e[1], ctx->st));
        if (ctx->overlap || ctx->g.prec != 0) {
            CK(launch_pairs(ctx->G, ctx->D, ctx->g, ctx->cur, ctx->st));
            CK(launch_step_split(ctx->G, ctx->D, ctx->g, ctx->cur, nullptr, 0, ctx->st, 1));
            ctx->launches += 2;
        } else {
            CK(launch_step(ctx->G, ctx->D, ctx->g, ctx->cur, nullptr, 0, ctx->st, 1));
            ctx->launches++;
        }
        ctx->cur ^= 1;
        CK(cudaEventRecord(e[2], ctx->st));
        rc = run_rebuild(ctx);
        if (rc) return rc;
        CK(cudaEventRecord(e[3], ctx->st));
        CK(cudaEventSynchronize(e[3]));
        float t;
        for (int k = 0; k < 3; ++k) {
            CK(cudaEventElapsedTime(&t, e[k], e[k + 1]));
            acc[k] += t;
        }
    }
    ctx->steps += nsteps;
    ctx->bp_cache = true;
    for (int k = 0; k < 3; ++k) ms3[k] = (float)acc[k];
    return check_err(ctx);
}

// ============================================ allocation-free fed-noise step
// sis_gpu_step_noise_static: sis_gpu_step with host noise, staged one step at
// a time through a fixed static device buffer instead of the context's noise
// buffer (which sis_gpu_step grows with cudaMalloc/cudaFree at call time).
// Nothing in the buffer has to start at zero: each step's copy overwrites all
// 3n doubles that step's kernel reads.  The buffer is one per device and
// shared by every context on it, so calls that overlap in time on one device
// race on it; callers serialise them.
constexpr int kStaticNoiseBeads = 65536; // 3 x 65536 doubles = 1.5 MiB
static __device__ __align__(256) double g_noise_scratch[3 * kStaticNoiseBeads];

namespace {

constexpr int kMaxDevices = 64;
std::mutex g_noise_mu;
double *g_noise_addr[kMaxDevices] = {};

// Address of g_noise_scratch on the context's device, looked up once per
// device with that device current (the first call on a device does this
// set-up; a caller that captures its stream should make that first call
// before it starts capturing).
int noise_scratch(sis_ctx *ctx, double **out) {
    const int dev = ctx->dev; // current: the entry point's DevGuard made it so
    if (dev < 0 || dev >= kMaxDevices) return fail(ctx, SIS_ERR_ARG, "sis_gpu_step_noise_static: device index out of range");
    std::lock_guard<std::mutex> lock(g_noise_mu);
    if (!g_noise_addr[dev]) {
        void *p = nullptr;
        CK(cudaGetSymbolAddress(&p, g_noise_scratch));
        g_noise_addr[dev] = static_cast<double *>(p);
    }
    *out = g_noise_addr[dev];
    return SIS_OK;
}

} // namespace

extern "C" int sis_gpu_step_noise_static(sis_ctx *ctx, int64_t nsteps, const double *noise) {
    DevGuard dg_(ctx);
    if (!ctx || nsteps < 0 || (nsteps > 0 && !noise)) return SIS_ERR_ARG;
    if (ctx->n > kStaticNoiseBeads)
        return fail(ctx, SIS_ERR_ARG,
                    "sis_gpu_step_noise_static: " + std::to_string(ctx->n) + " beads exceed the static noise buffer (" +
                        std::to_string(kStaticNoiseBeads) + " beads); use sis_gpu_step");
    double *buf = nullptr;
    int rc = noise_scratch(ctx, &buf);
    if (rc) return rc;
    const bool small = small_active(ctx);
    rc = ensure_lists(ctx, nsteps > 0 && small);
    if (rc) return rc;
    const size_t per = (size_t)ctx->n * 3;
    if (small && !ctx->sp.n_cta && (rc = small_plan(ctx, std::min(ctx->n_inst, 2 * ctx->sms)))) return rc;
    for (int64_t s = 0; s < nsteps; ++s) {
        // stream-ordered: the copy waits for the previous step's kernels
        CK(cudaMemcpyAsync(buf, noise + (size_t)s * per, sizeof(double) * per, cudaMemcpyHostToDevice, ctx->st));
        rc = small ? run_small(ctx, 1, buf) : enqueue_step(ctx, buf, 0);
        if (rc) return rc;
    }
    ctx->steps += nsteps;
    ctx->bp_cache = true;
    CK(cudaStreamSynchronize(ctx->st));
    // caller-supplied Monte Carlo uniforms apply to one call only, as in sis_gpu_step
    ctx->D.mc_draws = nullptr;
    ctx->mc_pending = false;
    return check_err(ctx);
}

// ========================================================= replica exchange
// The replica variables of var_replica.F90 (REPT: 1 temperature, 2 ionic
// strength, 3 constant trap force, 4 Rg bias target).  Labels are the rows
// of `values` ([n_inst][nvar], kinds[v] naming column v); with `assign`,
// replica k starts on label assign[k], else on label k.
namespace {
int remd_setup(sis_ctx *ctx, int nvar, const int *kinds, const double *values, const int *assign) {
    const int ni = ctx->n_inst;
    // replicas of one topology, salt and box
    const InstP &I0 = ctx->ip[0];
    const int nl = I0.n;
    bool has[5] = {false, false, false, false, false};
    for (int v = 0; v < nvar; ++v) {
        if (kinds[v] < 1 || kinds[v] > 4 || has[kinds[v]]) return fail(ctx, SIS_ERR_ARG, "remd: unknown or repeated replica variable");
        has[kinds[v]] = true;
    }
    for (int k = 1; k < ni; ++k) {
        const InstP &I = ctx->ip[k];
        bool same = I.n == nl && (has[2] || ctx->ionic[k] == ctx->ionic[0]) && I.pbc == I0.pbc;
        for (int d = 0; d < 3 && same; ++d) same = I.box[d] == I0.box[d];
        for (int i = 0; i < nl && same; ++i) {
            const int4 a = ctx->binfo[I0.bead_off + i], b = ctx->binfo[I.bead_off + i];
            same = ctx->seq[I0.bead_off + i] == ctx->seq[I.bead_off + i] && a.y - I0.bead_off == b.y - I.bead_off && a.z == b.z &&
                   a.w == b.w;
        }
        if (!same) return fail(ctx, SIS_ERR_ARG, "remd: instances must be replicas of one topology, salt and box");
    }
    if (has[4])
        for (int k = 0; k < ni; ++k)
            if (ctx->ip[k].rg_pott == 0) return fail(ctx, SIS_ERR_ARG, "remd: an Rg replica variable needs the Rg bias on every replica");
    for (int l = 0; l < ni; ++l)
        for (int v = 0; v < nvar; ++v) {
            const double x = values[(size_t)l * nvar + v];
            if (!std::isfinite(x) || ((kinds[v] == 1 || kinds[v] == 2) && !(x > 0.0)))
                return fail(ctx, SIS_ERR_ARG, "remd: a replica variable value is not valid");
        }
    std::vector<int> rep2lab(ni), lab2rep(ni, -1);
    for (int k = 0; k < ni; ++k) {
        rep2lab[k] = assign ? assign[k] : k;
        if (rep2lab[k] < 0 || rep2lab[k] >= ni || lab2rep[rep2lab[k]] >= 0) return fail(ctx, SIS_ERR_ARG, "remd: labels do not form a permutation");
        lab2rep[rep2lab[k]] = k;
    }
    // per-label records: temperature, salt (electrostatic fields), Rg target,
    // trap magnitude; noise coefficient per local bead; FP32 triplet free energies
    auto val = [&](int l, int kind, double dflt) {
        for (int v = 0; v < nvar; ++v)
            if (kinds[v] == kind) return values[(size_t)l * nvar + v];
        return dflt;
    };
    std::vector<InstP> lab_ip(ni, I0);
    std::vector<double> lab_ion(ni);
    std::vector<double> lab_w((size_t)ni * nl);
    std::vector<float> lab_dgf((size_t)ni * 469);
    const double fric = friction_of(ctx->p);
    for (int l = 0; l < ni; ++l) {
        InstP &L = lab_ip[l];
        L.tempK = val(l, 1, I0.tempK);
        lab_ion[l] = val(l, 2, ctx->ionic[0]);
        L.twz_scale = val(l, 3, I0.twz_scale);
        L.rg0 = val(l, 4, I0.rg0);
        set_ele_fields(ctx, L, lab_ion[l]);
        if (I0.large) {
            const double c2 = std::max(std::max(L.wca_nl_cut2, L.ele_nl_cut2), L.bp_nl_cut2);
            for (int d = 0; d < 3; ++d)
                if (I0.cell_len[d] < sqrt(c2) * 1.0005)
                    return fail(ctx, SIS_ERR_ARG, "remd: a label's electrostatic cutoff exceeds the cell grid of the box");
        }
        for (int i = 0; i < nl; ++i) {
            const bool still = ctx->p.integrator != SIS_INTGRT_GJF2GJ && !ctx->frozen.empty() && ctx->frozen[I0.bead_off + i];
            lab_w[(size_t)l * nl + i] = still ? 0.0 : noise_coef(ctx->p, fric, ctx->mass[I0.bead_off + i], L.tempK);
        }
        dgf_row(ctx, L.tempK, lab_dgf.data() + (size_t)l * 469);
    }
    // every replica takes its label's values now (its own record otherwise unchanged)
    bool recut = false;
    for (int k = 0; k < ni; ++k) {
        InstP &I = ctx->ip[k];
        const InstP &L = lab_ip[rep2lab[k]];
        const double cut = I.ele_nl_cut2;
        I.tempK = L.tempK;
        I.twz_scale = L.twz_scale;
        I.rg0 = L.rg0;
        ctx->ionic[k] = lab_ion[rep2lab[k]];
        set_ele(ctx, k);
        recut |= I.ele_nl_cut2 != cut;
    }
    RemdDev &R = ctx->remd;
    if (!ctx->remd_on) {
        int rc = 0;
        InstP *lab_ip_d = nullptr;
        double *lab_w_d = nullptr;
        float *lab_dgf_d = nullptr;
        rc |= dalloc(ctx, &R.ip2, ni);
        rc |= dalloc(ctx, &lab_ip_d, ni);
        rc |= dalloc(ctx, &R.ene2, (size_t)12 * ni);
        rc |= dalloc(ctx, &R.rep2lab, ni);
        rc |= dalloc(ctx, &R.lab2rep, ni);
        rc |= dalloc(ctx, &R.changed, ni);
        rc |= dalloc(ctx, &R.vscale, ni);
        rc |= dalloc(ctx, &R.n_acc, 1);
        rc |= dalloc(ctx, &lab_w_d, (size_t)ni * nl);
        rc |= dalloc(ctx, &lab_dgf_d, (size_t)ni * 469);
        rc |= dalloc(ctx, &ctx->remd_u, ni / 2 + 1);
        if (rc) return SIS_ERR_NOMEM;
        R.lab_ip = lab_ip_d;
        R.lab_w = lab_w_d;
        R.lab_dgf = lab_dgf_d;
        R.ip = ctx->ip_d;
        R.dgf = ctx->dgf_d;
    }
    R.n_local = nl;
    CK(cudaMemcpyAsync((void *)R.lab_ip, lab_ip.data(), sizeof(InstP) * ni, cudaMemcpyHostToDevice, ctx->st));
    CK(cudaMemcpyAsync((void *)R.lab_w, lab_w.data(), sizeof(double) * lab_w.size(), cudaMemcpyHostToDevice, ctx->st));
    CK(cudaMemcpyAsync((void *)R.lab_dgf, lab_dgf.data(), sizeof(float) * lab_dgf.size(), cudaMemcpyHostToDevice, ctx->st));
    CK(cudaMemcpyAsync(R.rep2lab, rep2lab.data(), sizeof(int) * ni, cudaMemcpyHostToDevice, ctx->st));
    CK(cudaMemcpyAsync(R.lab2rep, lab2rep.data(), sizeof(int) * ni, cudaMemcpyHostToDevice, ctx->st));
    int rc = upload_ip(ctx);
    if (rc) return rc;
    // the replicas' noise coefficients and FP32 triplet tables at their labels' temperatures
    std::vector<double4> mdc;
    md_coefs(ctx, mdc);
    CK(cudaMemcpyAsync(ctx->D.mdc, mdc.data(), sizeof(double4) * ctx->n, cudaMemcpyHostToDevice, ctx->st));
    for (int k = 0; k < ni; ++k)
        if ((rc = upload_dgf(ctx, k))) return rc;
    CK(cudaStreamSynchronize(ctx->st));
    if (recut) ctx->lists_valid = false;
    ctx->remd_lab_ion = lab_ion;
    ctx->bp_cache = false;
    ctx->remd_on = true;
    return SIS_OK;
}
} // namespace

extern "C" int sis_gpu_remd_init(sis_ctx *ctx, const double *temps) {
    DevGuard dg_(ctx);
    if (!ctx || !temps || ctx->n_inst < 2) return SIS_ERR_ARG;
    const int ni = ctx->n_inst;
    for (int l = 1; l < ni; ++l)
        if (!(temps[l] > temps[l - 1])) return fail(ctx, SIS_ERR_ARG, "remd: the temperature ladder must be strictly ascending");
    // each replica starts on the label of its temperature
    std::vector<int> rep2lab(ni, -1), lab2rep(ni, -1);
    for (int k = 0; k < ni; ++k) {
        for (int l = 0; l < ni; ++l)
            if (temps[l] == ctx->ip[k].tempK && lab2rep[l] < 0) {
                rep2lab[k] = l;
                lab2rep[l] = k;
                break;
            }
        if (rep2lab[k] < 0) return fail(ctx, SIS_ERR_ARG, "remd: every instance's temperature must be a distinct rung of the ladder");
    }
    const int kind = 1;
    return remd_setup(ctx, 1, &kind, temps, rep2lab.data());
}

extern "C" int sis_gpu_remd_init_vars(sis_ctx *ctx, int32_t nvar, const int32_t *kinds, const double *values) {
    DevGuard dg_(ctx);
    if (!ctx || nvar < 1 || nvar > 4 || !kinds || !values || ctx->n_inst < 2) return SIS_ERR_ARG;
    return remd_setup(ctx, nvar, kinds, values, nullptr);
}

extern "C" int sis_gpu_remd_exchange(sis_ctx *ctx, int32_t parity, const double *uniforms, int32_t *rep2lab, int32_t *n_accepted) {
    DevGuard dg_(ctx);
    if (!ctx || (parity != 0 && parity != 1)) return SIS_ERR_ARG;
    if (!ctx->remd_on) return fail(ctx, SIS_ERR_STATE, "remd: sis_gpu_remd_init has not been called");
    int rc = ensure_lists(ctx);
    if (rc) return rc;
    const int ni = ctx->n_inst;
    const RemdDev &R = ctx->remd;
    // energies at the replicas' own temperatures (energy_replica.F90:54-58)
    if (ctx->g.bp_model > 0) CK(launch_bp_energy(ctx->D, ctx->g, ctx->cur, -1.0, bp_blocks(ctx), ctx->st));
    CK(cudaMemsetAsync(ctx->D.ene, 0, sizeof(double) * 12 * ni, ctx->st));
    CK(launch_energy(ctx->D, ctx->g, ctx->cur, ctx->st));
    CK(launch_bias_energy(ctx->D, ctx->g, ctx->cur, ctx->st));
    // and at their partners' temperatures (energy_replica.F90:72-121)
    CK(launch_remd_partner_ip(ctx->D, R, ni, parity, ctx->st));
    Dev D2 = ctx->D;
    D2.ip = R.ip2;
    D2.ene = R.ene2;
    if (ctx->g.bp_model > 0) CK(launch_bp_energy(D2, ctx->g, ctx->cur, -1.0, bp_blocks(ctx), ctx->st));
    CK(cudaMemsetAsync(R.ene2, 0, sizeof(double) * 12 * ni, ctx->st));
    CK(launch_energy(D2, ctx->g, ctx->cur, ctx->st));
    CK(launch_bias_energy(D2, ctx->g, ctx->cur, ctx->st));
    const double *u = nullptr;
    if (uniforms) {
        CK(cudaMemcpyAsync(ctx->remd_u, uniforms, sizeof(double) * (ni / 2 + 1), cudaMemcpyHostToDevice, ctx->st));
        u = ctx->remd_u;
    }
    CK(launch_remd_decide(ctx->D, R, ctx->g, parity, u, BOLTZ_KCAL_MOL, ctx->remd_ctr++, ctx->st));
    ctx->launches += 2 * (2 + (ctx->g.bp_model > 0) + (ctx->g.flg_bias ? 1 + ctx->g.flg_rg : 0)) + 3;
    // lists of replicas whose electrostatic cutoff moved with the Debye length
    if ((rc = run_rebuild(ctx))) return rc;
    int nacc = 0;
    std::vector<int> r2l(ni);
    CK(cudaMemcpyAsync(r2l.data(), R.rep2lab, sizeof(int) * ni, cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaMemcpyAsync(&nacc, R.n_acc, sizeof(int), cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaMemcpyAsync(ctx->ip.data(), ctx->ip_d, sizeof(InstP) * ni, cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
    for (int k = 0; k < ni; ++k) {
        if (rep2lab) rep2lab[k] = r2l[k];
        ctx->ionic[k] = ctx->remd_lab_ion[r2l[k]];
        if (ctx->g.bp_model == 4 || ctx->g.bp_model == 5) dgf_row(ctx, ctx->ip[k].tempK, ctx->dgf.data() + (size_t)k * 469);
    }
    if (n_accepted) *n_accepted = nacc;
    ctx->bp_cache = false;
    return check_err(ctx);
}

// ===================================================== serving slots
extern "C" int sis_gpu_load_slot(sis_ctx *ctx, int32_t inst, int32_t n_chains, const int32_t *chain_len,
                                 const int32_t *chain_moltype, const int32_t *seq, const uint8_t *has_charge, double tempK,
                                 double ionic, uint32_t stream, const double *xyz, int32_t init_velocities) {
    DevGuard dg_(ctx);
    if (!ctx || inst < 0 || inst >= ctx->n_inst || n_chains < 0 || !(tempK > 0.0) || !(ionic > 0.0)) return SIS_ERR_ARG;
    InstP &I = ctx->ip[inst];
    const int off = I.bead_off, n = I.n;
    int L = 0;
    for (int c = 0; c < n_chains; ++c) {
        if (!chain_len || chain_len[c] < 1) return SIS_ERR_ARG;
        L += chain_len[c];
    }
    if (L > n) return fail(ctx, SIS_ERR_ARG, "load_slot: the job has more beads than the slot");
    if (L > 0 && (!seq || !xyz)) return SIS_ERR_ARG;
    if (!std::isfinite(tempK) || !std::isfinite(ionic)) return SIS_ERR_ARG;
    // every code is checked before the slot is touched, so a refused job
    // leaves the slot as it was
    for (int i = 0; i < L; ++i)
        if (seq[i] < 0 || seq[i] > 4) return fail(ctx, SIS_ERR_ARG, "load_slot: sequence code outside A U G C D");
    for (int c = 0; chain_moltype && c < n_chains; ++c)
        if (chain_moltype[c] != 1 && chain_moltype[c] != 2) return fail(ctx, SIS_ERR_ARG, "load_slot: molecule type");
    // topology: the job's chains, then inert single-bead fillers (sequence D,
    // uncharged: no list, bonded or base-pair term takes them; frozen below)
    int b = off;
    for (int c = 0; c < n_chains; ++c) {
        const int len = chain_len[c];
        const bool circ = chain_moltype && chain_moltype[c] == 2;
        for (int l = 0; l < len; ++l, ++b) {
            const int s = seq[b - off], q = has_charge ? (has_charge[b - off] ? 1 : 0) : 1;
            if (s < 0 || s > 4) return SIS_ERR_ARG;
            ctx->binfo[b] = make_int4(inst, off + (b - off - l), len | (circ ? (int)0x80000000u : 0), l | (s << 24) | (q << 28));
            ctx->seq[b] = s;
        }
    }
    for (; b < off + n; ++b) {
        ctx->binfo[b] = make_int4(inst, b, 1, 4 << 24);
        ctx->seq[b] = 4;
    }
    I.n_act = L;
    // conditions; the noise counter of the job starts at the current step
    I.tempK = tempK;
    ctx->ionic[inst] = ionic;
    set_ele(ctx, inst);
    I.stream = stream;
    unsigned long long sc = 0;
    CK(cudaMemcpyAsync(&sc, ctx->D.step_ctr, sizeof(sc), cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
    I.step0 = sc;
    // a new job starts with no frozen beads
    if (!ctx->frozen.empty()) std::fill(ctx->frozen.begin() + off, ctx->frozen.begin() + off + n, (uint8_t)0);
    std::vector<double4> mdc;
    md_coefs(ctx, mdc);
    for (int i = off + L; i < off + n; ++i) mdc[i] = make_double4(0.0, 0.0, 0.0, 0.0);
    CK(cudaMemcpyAsync(ctx->D.binfo + off, ctx->binfo.data() + off, sizeof(int4) * n, cudaMemcpyHostToDevice, ctx->st));
    CK(cudaMemcpyAsync(ctx->D.mass + off, ctx->mass.data() + off, sizeof(double) * n, cudaMemcpyHostToDevice, ctx->st));
    CK(cudaMemcpyAsync(ctx->D.mdc + off, mdc.data() + off, sizeof(double4) * n, cudaMemcpyHostToDevice, ctx->st));
    int rc = upload_ip(ctx);
    if (!rc) rc = upload_dgf(ctx, inst);
    if (rc) return rc;
    // state: the job's coordinates (fillers on its first bead), zero velocities
    if (!ctx->pin) CK(cudaMallocHost((void **)&ctx->pin, sizeof(double4) * ctx->n));
    CK(cudaStreamSynchronize(ctx->st));
    double4 *h = ctx->pin;
    for (int i = 0; i < n; ++i) {
        const int j = i < L ? i : 0;
        h[i] = L > 0 ? make_double4(xyz[3 * j], xyz[3 * j + 1], xyz[3 * j + 2], 0.0) : make_double4(0.0, 0.0, 0.0, 0.0);
    }
    // both position buffers (and their mirrors): the per-block kernel never
    // moves the fillers, so they stay the same in both
    for (int c = 0; c < 2; ++c) {
        CK(cudaMemcpyAsync(ctx->D.x[c] + off, h, sizeof(double4) * n, cudaMemcpyHostToDevice, ctx->st));
        CK(launch_mirror(ctx->D, ctx->g, c, ctx->st));
    }
    CK(cudaMemsetAsync(ctx->D.v + off, 0, sizeof(double4) * n, ctx->st));
    CK(cudaMemsetAsync(ctx->D.beta + off, 0, sizeof(double4) * n, ctx->st));
    CK(cudaMemsetAsync(ctx->D.move + off, 0, sizeof(double4) * n, ctx->st));
    ctx->launches += 2;
    // velocities as the first sis_gpu_init_velocities of a context would draw them
    if (init_velocities) {
        CK(launch_init_velocities(ctx->D, ctx->g, 1ull << 62, ctx->st, inst));
        ctx->launches++;
    }
    // the slot's lists (with every coordinate set): in a context that steps
    // through the per-block kernel, that kernel's next launch rebuilds them
    // (the slot flagged); otherwise now
    if (ctx->state_set) {
        if (small_active(ctx)) {
            const int one = 1;
            CK(cudaMemcpyAsync(ctx->D.flag + inst, &one, sizeof(int), cudaMemcpyHostToDevice, ctx->st));
            ctx->stale_lists = true;
        } else {
            if ((rc = flag_all(ctx, inst))) return rc;
            if ((rc = run_rebuild(ctx))) return rc;
        }
    }
    ctx->bp_cache = false;
    CK(cudaStreamSynchronize(ctx->st));
    return check_err(ctx);
}

// ============================================== base-pair Monte Carlo pass
extern "C" int sis_gpu_bp_mc(sis_ctx *ctx, int32_t inst, const double *draws, int32_t n_draws) {
    DevGuard dg_(ctx);
    if (!ctx || inst < -1 || inst >= ctx->n_inst || n_draws < 0 || (n_draws > 0 && !draws)) return SIS_ERR_ARG;
    if (ctx->g.nstep_mc <= 0) return fail(ctx, SIS_ERR_STATE, "bp_mc: the context has no base-pair Monte Carlo (nstep_bp_mc = 0)");
    const int one = 1;
    for (int k = inst < 0 ? 0 : inst; k < (inst < 0 ? ctx->n_inst : inst + 1); ++k)
        CK(cudaMemcpy(ctx->D.mc_due + k, &one, sizeof(int), cudaMemcpyHostToDevice));
    if (n_draws > 0) {
        if (n_draws > ctx->mc_draws_cap) {
            if (ctx->mc_draws_d) cudaFree(ctx->mc_draws_d);
            ctx->mc_draws_d = nullptr;
            if (cudaMalloc(&ctx->mc_draws_d, sizeof(double) * n_draws) != cudaSuccess) return fail(ctx, SIS_ERR_NOMEM, "bp_mc draws");
            ctx->mc_draws_cap = n_draws;
        }
        CK(cudaMemcpy(ctx->mc_draws_d, draws, sizeof(double) * n_draws, cudaMemcpyHostToDevice));
        CK(cudaMemset(ctx->D.mc_draw_pos, 0, sizeof(int)));
        ctx->D.mc_draws = ctx->mc_draws_d;
        ctx->D.mc_n_draws = n_draws;
        ctx->mc_pending = true;
    }
    return SIS_OK;
}

extern "C" int sis_gpu_get_bp_energies(sis_ctx *ctx, int32_t inst, double *out, int32_t cap, int32_t *n_out) {
    DevGuard dg_(ctx);
    if (!ctx || inst < 0 || inst >= ctx->n_inst || !n_out) return SIS_ERR_ARG;
    const InstP &I = ctx->ip[inst];
    int c = 0;
    CK(cudaMemcpyAsync(&c, ctx->D.bp_cnt + inst, sizeof(int), cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
    c = std::min(c, I.bp_cap);
    *n_out = c;
    if (out && cap > 0) {
        CK(cudaMemcpyAsync(out, ctx->D.ene_bp + I.bp_off, sizeof(double) * std::min(c, cap), cudaMemcpyDeviceToHost, ctx->st));
        CK(cudaStreamSynchronize(ctx->st));
    }
    return SIS_OK;
}

extern "C" int sis_gpu_get_bp_status(sis_ctx *ctx, int32_t inst, uint8_t *out, int32_t cap, int32_t *n_out) {
    DevGuard dg_(ctx);
    if (!ctx || inst < 0 || inst >= ctx->n_inst || !n_out) return SIS_ERR_ARG;
    const InstP &I = ctx->ip[inst];
    int c = 0;
    CK(cudaMemcpyAsync(&c, ctx->D.bp_cnt + inst, sizeof(int), cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
    c = std::min(c, I.bp_cap);
    *n_out = c;
    if (out && cap > 0) {
        CK(cudaMemcpyAsync(out, ctx->D.bp_status + I.bp_off, std::min(c, cap), cudaMemcpyDeviceToHost, ctx->st));
        CK(cudaStreamSynchronize(ctx->st));
    }
    return SIS_OK;
}
