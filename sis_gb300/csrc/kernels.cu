// Step, force, base-pair and energy kernels of libsisgpu.
//
// One MD step (job_md.F90:360-460) is two kernels:
//   k_bp    base-pair 6-bead terms over the candidate list (force_bp*.F90),
//           scattered into fbp with FP64 atomics (few records pass the
//           distance test, so the scatter is cheap);
//   k_step  one group of G lanes per bead: gathers the WCA and Debye-Hueckel
//           pair forces over the bead's full pair list and the bonded terms
//           touching the bead, adds fbp, and applies the GJF-2GJ (or
//           Ermak-McCammon) update in FP64; its last block evaluates the
//           displacement trigger of every instance (job_md.F90:376-395).
// The list rebuild (k_rebuild in lists.cu) follows and exits at once when no
// instance asked for one.
#include "common.cuh"
#include "kernels.h"
#include "terms.cuh"

namespace sisg {

template <typename R> __device__ __forceinline__ Pos<R> pos_of(const Dev &D, int cur);
template <> __device__ __forceinline__ Pos<double> pos_of<double>(const Dev &D, int cur) { return Pos<double>{D.x[cur]}; }
template <> __device__ __forceinline__ Pos<float> pos_of<float>(const Dev &D, int cur) { return Pos<float>{D.mir[cur]}; }

__device__ __forceinline__ double comp(const V3<double> &a, int c) { return c == 0 ? a.x : (c == 1 ? a.y : a.z); }

// Gaussian deviate of component c of local bead i of a noise stream at step s
// (Box-Muller on one Philox4x32-10 block: components 0,1 share one pair).
template <typename R>
__device__ __forceinline__ double gauss3(unsigned long long seed, int i, unsigned long long s, int c, unsigned stream);
template <> __device__ __forceinline__ double gauss3<float>(unsigned long long seed, int i, unsigned long long s, int c,
                                                            unsigned stream) {
    const uint4 r = philox4x32_10(make_uint4((unsigned)i, (unsigned)s, (unsigned)(s >> 32), stream),
                                  make_uint2((unsigned)seed, (unsigned)(seed >> 32)));
    const unsigned a = c < 2 ? r.x : r.z, b = c < 2 ? r.y : r.w;
    const float u1 = (float)((a >> 8) + 1u) * (1.0f / 16777216.0f);
    const float u2 = (float)(b >> 8) * (1.0f / 16777216.0f);
    float sn, cs;
    sincospif(2.0f * u2, &sn, &cs);
    return (double)(sqrtf(-2.0f * logf(u1)) * (c == 1 ? sn : cs));
}
template <> __device__ __forceinline__ double gauss3<double>(unsigned long long seed, int i, unsigned long long s, int c,
                                                             unsigned stream) {
    const uint4 r = philox4x32_10(make_uint4((unsigned)i, (unsigned)s, (unsigned)(s >> 32), stream),
                                  make_uint2((unsigned)seed, (unsigned)(seed >> 32)));
    const unsigned a = c < 2 ? r.x : r.z, b = c < 2 ? r.y : r.w;
    const double u1 = ((double)a + 1.0) * (1.0 / 4294967296.0);
    const double u2 = (double)b * (1.0 / 4294967296.0);
    double sn, cs;
    sincospi(2.0 * u2, &sn, &cs);
    return sqrt(-2.0 * log(u1)) * (c == 1 ? sn : cs);
}

// ------------------------------------------------------------------ k_step
// MODE 0: full MD step (forces + integration + trigger)
// MODE 1: forces only, written to fout[3*i+c] (terms selected by mask)
template <typename R, int G, int MODE>
__global__ void __launch_bounds__(256) k_step(Dev D, GlobP g, int cur, const double *__restrict__ noise, long long noise_step,
                                              double *__restrict__ fout, int mask) {
    __shared__ unsigned long long s_m1[32], s_m2[32];
    __shared__ int s_lo, s_cnt;
    __shared__ int s_last;
    const int bpb = blockDim.x / G;
    const int i_raw = blockIdx.x * bpb + threadIdx.x / G;
    const int lane = threadIdx.x % G;
    const bool active = i_raw < g.n;
    const int i = active ? i_raw : g.n - 1;
    if (MODE == 0) {
        if (threadIdx.x < 32) {
            s_m1[threadIdx.x] = 0ull;
            s_m2[threadIdx.x] = 0ull;
        }
        if (threadIdx.x == 0) {
            const int i0 = blockIdx.x * bpb;
            const int i1 = min(i0 + bpb - 1, g.n - 1);
            s_lo = D.binfo[i0].x;
            s_cnt = D.binfo[i1].x - s_lo + 1;
        }
        __syncthreads();
    }
    const int4 bi = D.binfo[i];
    const InstP &ip = D.ip[bi.x];
    const Pos<R> P = pos_of<R>(D, cur);
    const double4 *__restrict__ x64 = D.x[cur];

    // non-bonded pair terms over the full list
    V3<R> an = mk<R>(0, 0, 0);
    if (mask & 48) {
        const int cnt = min(D.nnbr[i], g.cap);
        const int *__restrict__ nb = D.nbr + (size_t)i * g.cap;
        const R sig2 = pick<R>(g.wca_sig2, g.f_wca_sig2), wcoef = pick<R>(g.wca_coef, g.f_wca_coef);
        const R ecoef = pick<R>(ip.ele_coef, ip.ele_coef_f), rc = pick<R>(ip.rcdist, ip.rcdist_f);
        const R cut2 = g.flg_ele ? pick<R>(ip.ele_cut2, ip.ele_cut2_f) : R(-1);
        for (int k = lane; k < cnt; k += G) {
            const int e = __ldg(nb + k);
            const int j = e & IDX_MASK;
            const V3<R> v = P.d(i, j, ip);
            const R d2 = dot3(v, v);
            R c;
            if (sizeof(R) == 4)
                c = (R)pair_coef_f(e, (float)d2, (float)sig2, (float)wcoef, (float)ecoef, (float)rc, (float)cut2, mask);
            else
                c = pair_coef<R>(e, d2, sig2, wcoef, ecoef, rc, cut2, mask);
            an = an + c * v;
        }
    }
    // bonded terms touching bead i
    V3<R> ab = mk<R>(0, 0, 0);
    if (mask & 7) {
        for (int t = lane; t < 9; t += G) {
            const int cls = t < 2 ? 1 : (t < 5 ? 2 : 4);
            if (mask & cls) ab = ab + bonded_slot<R>(t, i, bi, P, x64, ip, g);
        }
    }
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1) {
        an.x += __shfl_xor_sync(0xffffffffu, an.x, o);
        an.y += __shfl_xor_sync(0xffffffffu, an.y, o);
        an.z += __shfl_xor_sync(0xffffffffu, an.z, o);
        ab.x += __shfl_xor_sync(0xffffffffu, ab.x, o);
        ab.y += __shfl_xor_sync(0xffffffffu, ab.y, o);
        ab.z += __shfl_xor_sync(0xffffffffu, ab.z, o);
    }
    // per-bead FP64 accumulation
    V3<double> F = mk<double>((double)an.x + (double)ab.x, (double)an.y + (double)ab.y, (double)an.z + (double)ab.z);
    if (mask & 8) {
        const double4 fb = D.fbp[i];
        F = mk<double>(F.x + fb.x, F.y + fb.y, F.z + fb.z);
        __syncwarp();
        if (active && lane == 0) D.fbp[i] = make_double4(0.0, 0.0, 0.0, 0.0);
    }
    if (MODE == 1) {
        if (active)
            for (int c = lane; c < 3; c += G) fout[3 * (size_t)i + c] = comp(F, c);
        return;
    }

    // ---------------------------------------------- GJF-2GJ / Ermak-McCammon
    const int nxt = cur ^ 1;
    const unsigned long long step = *D.step_ctr;
    double mv0 = 0.0, mv1 = 0.0, mv2 = 0.0;
    if (active) {
        const double4 m = D.mdc[i];
        for (int c = lane; c < 3; c += G) {
            const double Fc = comp(F, c);
            const double xi =
                noise ? noise[((size_t)noise_step * g.n + i) * 3 + c]
                      : gauss3<R>(g.seed, i - ip.bead_off, step - ip.step0, c, ip.stream);
            const double xc = ((const double *)(x64 + i))[c];
            double dx;
            if (g.integrator == 1) {
                double *vp = (double *)(D.v + i) + c;
                double *bp = (double *)(D.beta + i) + c;
                const double bn = m.w * xi;
                const double vn = m.x * (*vp) + m.y * Fc + (*bp + bn);
                *bp = bn;
                *vp = vn;
                dx = m.z * vn;
            } else {
                dx = m.x * Fc + m.w * xi;
            }
            const double xn = xc + dx;
            ((double *)(D.x[nxt] + i))[c] = xn;
            double *mp = (double *)(D.move + i) + c;
            const double mn = *mp + dx;
            *mp = mn;
            if (c == 0) mv0 = mn;
            else if (c == 1) mv1 = mn;
            else mv2 = mn;
            ((unsigned int *)(D.mir[nxt] + i))[c] = fixed1(xn, ip.fsc[c]);
        }
    }
    // displacement^2 of the bead (unfused, as dot_product in FP64)
    const int base = (threadIdx.x & 31) - lane;
    const double mx = __shfl_sync(0xffffffffu, mv0, base + (0 % G));
    const double my = __shfl_sync(0xffffffffu, mv1, base + (1 % G));
    const double mz = __shfl_sync(0xffffffffu, mv2, base + (2 % G));
    if (active && lane == 0) {
        const double d2 = __dadd_rn(__dadd_rn(__dmul_rn(mx, mx), __dmul_rn(my, my)), __dmul_rn(mz, mz));
        if (!isfinite(d2)) atomicOr(D.err, ERR_NONFINITE);
        const unsigned long long b = (unsigned long long)__double_as_longlong(d2);
        const int k = bi.x - s_lo;
        if (s_cnt <= 32) {
            const unsigned long long old = atomicMax(&s_m1[k], b);
            atomicMax(&s_m2[k], old < b ? old : b);
        } else {
            const unsigned long long old = atomicMax(&D.m1[bi.x], b);
            atomicMax(&D.m2[bi.x], old < b ? old : b);
        }
    }
    __syncthreads();
    if (s_cnt <= 32 && (int)threadIdx.x < s_cnt) {
        const unsigned long long b1 = s_m1[threadIdx.x], b2 = s_m2[threadIdx.x];
        const int inst = s_lo + threadIdx.x;
        const unsigned long long old = atomicMax(&D.m1[inst], b1);
        const unsigned long long c2 = old < b1 ? old : b1;
        atomicMax(&D.m2[inst], c2 > b2 ? c2 : b2);
    }
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) s_last = (atomicAdd(&D.ticket[0], 1u) == gridDim.x - 1);
    __syncthreads();
    if (s_last) {
        __threadfence();
        int any = 0;
        for (int k = threadIdx.x; k < g.n_inst; k += blockDim.x) {
            const double a = __longlong_as_double((long long)atomicExch(&D.m1[k], 0ull));
            const double b = __longlong_as_double((long long)atomicExch(&D.m2[k], 0ull));
            if (sqrt(a) + sqrt(b) > g.nl_margin) {
                D.flag[k] = 1;
                any = 1;
            }
        }
        if (any) atomicOr(D.any, 1);
        if (threadIdx.x == 0) {
            D.ticket[0] = 0u;
            D.step_ctr[0] = step + 1ull;
        }
    }
}

// -------------------------------------------------------------------- k_bp
// Base-pair records, grid-stride over the candidate list.  The global record
// index is mapped to (instance, slot) by binary search over the per-instance
// prefix counts written by the last list rebuild.
__device__ __forceinline__ bool bp_record(const Dev &D, int r, int n_inst, int &slot) {
    const int total = *D.bp_total;
    if (r >= total) return false;
    int lo = 0, hi = n_inst - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (D.bp_cnt[n_inst + mid] <= r) lo = mid;
        else hi = mid - 1;
    }
    slot = D.ip[lo].bp_off + (r - D.bp_cnt[n_inst + lo]);
    return true;
}

// mode 0: forces (+ cached energies); mode 1: energies only at temperature tK
// (tK < 0: the instance's own temperature)
template <typename R>
__global__ void __launch_bounds__(128) k_bp(Dev D, GlobP g, int cur, int mode, double tK_in) {
    const Pos<R> P = pos_of<R>(D, cur);
    const double4 *__restrict__ x64 = D.x[cur];
    const int total = *D.bp_total;
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < total; r += gridDim.x * blockDim.x) {
        int slot;
        if (!bp_record(D, r, g.n_inst, slot)) break;
        const int4 rec = D.bps[slot];
        const int4 nb = D.bps_n[slot];
        const int i1 = rec.x, i2 = rec.y, type = rec.z & 0xff, h = rec.z >> 8;
        const InstP &ip = D.ip[rec.w];
        const BPP &b = D.bpp[type];
        const bool triplet = g.bp_model == 4 || g.bp_model == 5;
        double ene = 0.0;
        unsigned char st = 0;
        double dG = 1.0;
        bool skip = false;
        if (triplet) {
            double tK = mode == 0 ? ip.tempK : (tK_in < 0 ? ip.tempK : tK_in);
            if (mode == 1 && g.temp_indep) tK = 0.0;
            dG = D.bp3_dH[h] - tK * D.bp3_dS[h];
            if (dG >= 0.0) skip = true;
        }
        if (!skip && mode == 0) {
            V3<R> f[6];
            R u;
            bool nr = false;
            bool ok = bp_force_core<R>(P.d(i1, i2, ip), P.d(i1, nb.x, ip), P.d(i1, nb.z, ip), P.d(nb.y, i2, ip), P.d(nb.w, i2, ip), b,
                                       f, &u, &nr);
            V3<double> fd[6];
            double ud = 0.0;
            if (ok && sizeof(R) == 4 && nr) {
                bool nr2;
                ok = bp_force_core<double>(dvec64(x64[i1], x64[i2], ip), dvec64(x64[i1], x64[nb.x], ip),
                                           dvec64(x64[i1], x64[nb.z], ip), dvec64(x64[nb.y], x64[i2], ip),
                                           dvec64(x64[nb.w], x64[i2], ip), b, fd, &ud, &nr2);
            } else if (ok) {
                for (int q = 0; q < 6; ++q) fd[q] = mk<double>((double)f[q].x, (double)f[q].y, (double)f[q].z);
                ud = (double)u;
            }
            if (ok) {
                const double e = triplet ? b.U0 * dG * exp(-ud) : b.U0 * exp(-ud);
                if (e <= g.bp_cutoff_energy) {
                    ene = e;
                    st = 1;
                    const int ids[6] = {i1, i2, nb.x, nb.y, nb.z, nb.w};
#pragma unroll
                    for (int q = 0; q < 6; ++q) {
                        atomicAdd(&D.fbp[ids[q]].x, e * fd[q].x);
                        atomicAdd(&D.fbp[ids[q]].y, e * fd[q].y);
                        atomicAdd(&D.fbp[ids[q]].z, e * fd[q].z);
                    }
                }
            }
        } else if (!skip) {
            // energy_bp.F90 / energy_bp_triplet.F90 (clamped angles)
            double u = 0.0;
            bool ok;
            if constexpr (sizeof(R) == 8) {
                const V3<double> v = dvec64(x64[i1], x64[i2], ip);
                const double d = sqrt(dot3(v, v)) - b.bond_r;
                ok = fabs(d) <= b.cutoff_ddist;
                if (ok) {
                    u = b.bond_k * (d * d);
                    double th = mp_angle<double>(dvec64(x64[i1], x64[i2], ip), dvec64(x64[nb.y], x64[i2], ip));
                    u = u + b.angl_k[0] * ((th - b.angl_theta[0]) * (th - b.angl_theta[0]));
                    th = mp_angle<double>(dvec64(x64[nb.x], x64[i1], ip), dvec64(x64[i2], x64[i1], ip));
                    u = u + b.angl_k[1] * ((th - b.angl_theta[1]) * (th - b.angl_theta[1]));
                    th = mp_angle<double>(dvec64(x64[i1], x64[i2], ip), dvec64(x64[nb.w], x64[i2], ip));
                    u = u + b.angl_k[2] * ((th - b.angl_theta[2]) * (th - b.angl_theta[2]));
                    th = mp_angle<double>(dvec64(x64[nb.z], x64[i1], ip), dvec64(x64[i2], x64[i1], ip));
                    u = u + b.angl_k[3] * ((th - b.angl_theta[3]) * (th - b.angl_theta[3]));
                    double ph = mp_dihedral<double>(dvec64(x64[nb.x], x64[i1], ip), dvec64(x64[i2], x64[i1], ip),
                                                    dvec64(x64[i2], x64[nb.y], ip));
                    u = u + b.dihd_k[0] * (1.0 + cos(ph + b.dihd_phi[0]));
                    ph = mp_dihedral<double>(dvec64(x64[nb.z], x64[i1], ip), dvec64(x64[i2], x64[i1], ip),
                                             dvec64(x64[i2], x64[nb.w], ip));
                    u = u + b.dihd_k[1] * (1.0 + cos(ph + b.dihd_phi[1]));
                }
            } else {
                const V3<float> v = P.d(i1, i2, ip);
                const float d = sqrtf(dot3(v, v)) - (float)b.bond_r;
                ok = fabsf(d) <= (float)b.cutoff_ddist;
                if (ok) {
                    // angles and dihedrals in FP64 from the FP64 positions
                    double dd = sqrt(dot3(dvec64(x64[i1], x64[i2], ip), dvec64(x64[i1], x64[i2], ip))) - b.bond_r;
                    u = b.bond_k * (dd * dd);
                    double th = mp_angle<double>(dvec64(x64[i1], x64[i2], ip), dvec64(x64[nb.y], x64[i2], ip));
                    u = u + b.angl_k[0] * ((th - b.angl_theta[0]) * (th - b.angl_theta[0]));
                    th = mp_angle<double>(dvec64(x64[nb.x], x64[i1], ip), dvec64(x64[i2], x64[i1], ip));
                    u = u + b.angl_k[1] * ((th - b.angl_theta[1]) * (th - b.angl_theta[1]));
                    th = mp_angle<double>(dvec64(x64[i1], x64[i2], ip), dvec64(x64[nb.w], x64[i2], ip));
                    u = u + b.angl_k[2] * ((th - b.angl_theta[2]) * (th - b.angl_theta[2]));
                    th = mp_angle<double>(dvec64(x64[nb.z], x64[i1], ip), dvec64(x64[i2], x64[i1], ip));
                    u = u + b.angl_k[3] * ((th - b.angl_theta[3]) * (th - b.angl_theta[3]));
                    double ph = mp_dihedral<double>(dvec64(x64[nb.x], x64[i1], ip), dvec64(x64[i2], x64[i1], ip),
                                                    dvec64(x64[i2], x64[nb.y], ip));
                    u = u + b.dihd_k[0] * (1.0 + cos(ph + b.dihd_phi[0]));
                    ph = mp_dihedral<double>(dvec64(x64[nb.z], x64[i1], ip), dvec64(x64[i2], x64[i1], ip),
                                             dvec64(x64[i2], x64[nb.w], ip));
                    u = u + b.dihd_k[1] * (1.0 + cos(ph + b.dihd_phi[1]));
                }
            }
            if (ok) {
                const double e = triplet ? b.U0 * dG * exp(-u) : b.U0 * exp(-u);
                if (e <= g.bp_cutoff_energy) {
                    ene = e;
                    st = 1;
                }
            }
        }
        D.ene_bp[slot] = ene;
        D.bp_status[slot] = st;
    }
}

// --------------------------------------------------------------- energies
// Per-instance energy slots ene[inst*12 + k]: 1 bond 2 angle 3 dihedral
// 5 WCA 6 DH (bp, total and kinetic are added by k_energy_finish).
template <typename R> __global__ void __launch_bounds__(256) k_energy(Dev D, GlobP g, int cur) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= g.n) return;
    const int4 bi = D.binfo[i];
    const InstP &ip = D.ip[bi.x];
    const Pos<R> P = pos_of<R>(D, cur);
    const double4 *x64 = D.x[cur];
    double eb, ea, ed, ew = 0.0, ee = 0.0;
    bonded_energy_owned<R>(i, bi, P, x64, ip, g, &eb, &ea, &ed);
    const int cnt = min(D.nnbr[i], g.cap);
    const int *nb = D.nbr + (size_t)i * g.cap;
    for (int k = 0; k < cnt; ++k) {
        const int e = nb[k];
        const int j = e & IDX_MASK;
        const V3<R> v = P.d(i, j, ip);
        pair_energy<R>(e, dot3(v, v), ip, g, &ew, &ee);
    }
    // every pair appears twice in the full list
    ew *= 0.5;
    ee *= 0.5;
    double *E = D.ene + (size_t)bi.x * 12;
    if (eb != 0.0) atomicAdd(E + 1, eb);
    if (ea != 0.0) atomicAdd(E + 2, ea);
    if (ed != 0.0) atomicAdd(E + 3, ed);
    if (ew != 0.0) atomicAdd(E + 5, ew);
    if (ee != 0.0) atomicAdd(E + 6, ee);
}

// kinetic energy (energy_kinetic.F90) into slot 11 and base-pair sums into slot 4
__global__ void k_energy_finish(Dev D, GlobP g) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < g.n) {
        const double4 v = D.v[i];
        const double e = D.mass[i] * (v.x * v.x + v.y * v.y + v.z * v.z);
        atomicAdd(D.ene + (size_t)D.binfo[i].x * 12 + 11, 0.5 * e);
    }
    // base-pair energies of each instance's staging segment
    if (i < g.n_inst) {
        const InstP &ip = D.ip[i];
        const int c = min(D.bp_cnt[i], ip.bp_cap);
        double s = 0.0;
        for (int k = 0; k < c; ++k) s += D.ene_bp[ip.bp_off + k];
        D.ene[(size_t)i * 12 + 4] = s;
    }
}

// initial velocities and accels from Philox (job_md.F90:214-238)
template <typename R> __global__ void k_init_velocities(Dev D, GlobP g, unsigned long long ctr) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= g.n) return;
    const int4 bi = D.binfo[i];
    const double T = D.ip[bi.x].tempK;
    const double kB = 1.380649e-23 * (1.0 / 4184.0 * 6.02214076e23);
    const double c1 = sqrt(T * kB / D.mass[i]);
    const double4 m = D.mdc[i];
    const InstP &ip = D.ip[bi.x];
    const int li = i - ip.bead_off;
    double4 v, b;
    v.x = c1 * gauss3<double>(g.seed, li, ctr, 0, ip.stream);
    v.y = c1 * gauss3<double>(g.seed, li, ctr, 1, ip.stream);
    v.z = c1 * gauss3<double>(g.seed, li, ctr, 2, ip.stream);
    v.w = 0.0;
    b.x = m.w * gauss3<double>(g.seed, li, ctr + 1, 0, ip.stream);
    b.y = m.w * gauss3<double>(g.seed, li, ctr + 1, 1, ip.stream);
    b.z = m.w * gauss3<double>(g.seed, li, ctr + 1, 2, ip.stream);
    b.w = 0.0;
    D.v[i] = v;
    D.beta[i] = b;
}

// refresh the fixed-point mirror from the FP64 positions
__global__ void k_mirror(Dev D, GlobP g, int cur) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= g.n) return;
    const InstP &ip = D.ip[D.binfo[i].x];
    const double4 x = D.x[cur][i];
    D.mir[cur][i] = make_uint4(fixed1(x.x, ip.fsc[0]), fixed1(x.y, ip.fsc[1]), fixed1(x.z, ip.fsc[2]), 0u);
}

// ------------------------------------------------------------- launchers
template <typename R, int G, int MODE>
static cudaError_t launch_step_g(const Dev &D, const GlobP &g, int cur, const double *noise, long long ns, double *fout, int mask,
                                 cudaStream_t st) {
    const int bpb = 256 / G;
    const int grid = (g.n + bpb - 1) / bpb;
    k_step<R, G, MODE><<<grid, 256, 0, st>>>(D, g, cur, noise, ns, fout, mask);
    return cudaGetLastError();
}

template <typename R, int MODE>
static cudaError_t launch_step_r(int G, const Dev &D, const GlobP &g, int cur, const double *noise, long long ns, double *fout,
                                 int mask, cudaStream_t st) {
    switch (G) {
    case 1: return launch_step_g<R, 1, MODE>(D, g, cur, noise, ns, fout, mask, st);
    case 2: return launch_step_g<R, 2, MODE>(D, g, cur, noise, ns, fout, mask, st);
    case 4: return launch_step_g<R, 4, MODE>(D, g, cur, noise, ns, fout, mask, st);
    case 8: return launch_step_g<R, 8, MODE>(D, g, cur, noise, ns, fout, mask, st);
    case 16: return launch_step_g<R, 16, MODE>(D, g, cur, noise, ns, fout, mask, st);
    default: return launch_step_g<R, 32, MODE>(D, g, cur, noise, ns, fout, mask, st);
    }
}

cudaError_t launch_step(int G, const Dev &D, const GlobP &g, int cur, const double *noise, long long ns, cudaStream_t st) {
    if (g.prec == 0) return launch_step_r<double, 0>(G, D, g, cur, noise, ns, nullptr, 63, st);
    return launch_step_r<float, 0>(G, D, g, cur, noise, ns, nullptr, 63, st);
}

cudaError_t launch_force(int G, const Dev &D, const GlobP &g, int cur, double *fout, int mask, cudaStream_t st) {
    if (g.prec == 0) return launch_step_r<double, 1>(G, D, g, cur, nullptr, 0, fout, mask, st);
    return launch_step_r<float, 1>(G, D, g, cur, nullptr, 0, fout, mask, st);
}

cudaError_t launch_bp(const Dev &D, const GlobP &g, int cur, int mode, double tK, int nblocks, cudaStream_t st) {
    if (g.prec == 0) k_bp<double><<<nblocks, 128, 0, st>>>(D, g, cur, mode, tK);
    else k_bp<float><<<nblocks, 128, 0, st>>>(D, g, cur, mode, tK);
    return cudaGetLastError();
}

cudaError_t launch_energy(const Dev &D, const GlobP &g, int cur, cudaStream_t st) {
    const int grid = (g.n + 255) / 256;
    if (g.prec == 0) k_energy<double><<<grid, 256, 0, st>>>(D, g, cur);
    else k_energy<float><<<grid, 256, 0, st>>>(D, g, cur);
    const int grid2 = (max(g.n, g.n_inst) + 255) / 256;
    k_energy_finish<<<grid2, 256, 0, st>>>(D, g);
    return cudaGetLastError();
}

cudaError_t launch_init_velocities(const Dev &D, const GlobP &g, unsigned long long ctr, cudaStream_t st) {
    k_init_velocities<double><<<(g.n + 255) / 256, 256, 0, st>>>(D, g, ctr);
    return cudaGetLastError();
}

cudaError_t launch_mirror(const Dev &D, const GlobP &g, int cur, cudaStream_t st) {
    k_mirror<<<(g.n + 255) / 256, 256, 0, st>>>(D, g, cur);
    return cudaGetLastError();
}

} // namespace sisg
