// Step, force, base-pair and energy kernels of libsisgpu.
//
// One MD step (job_md.F90:360-460) is these kernels plus the list check:
//   k_bonded  bonded terms, one thread per term start bead, written to
//             per-term force slots (no atomics);
//   k_bp_test, k_bp_eval
//             the base-pair 6-bead terms over the candidate list
//             (force_bp*.F90): one thread per record for the distance
//             window, then one per windowed record, scattered into fbp (FP64
//             atomics in the FP64 path, exact int64 fixed-point atomics in
//             the mixed path); they run beside k_bonded;
//   k_step    one group of G lanes per bead: gathers the WCA and
//             Debye-Hueckel pair forces over the bead's full pair list and
//             the bonded slots touching the bead, adds fbp, and applies the
//             GJF-2GJ (or Ermak-McCammon) update in FP64; per-block partials
//             of the displacement trigger (job_md.F90:376-395) go to
//             k_trigger_rebuild (lists.cu), which merges them and rebuilds
//             the lists of the instances that fired.
#include "common.cuh"
#include "kernels.h"
#include "listcore.cuh"
#include "terms.cuh"

#include <algorithm>

namespace sisg {

template <typename R> __device__ __forceinline__ Pos<R> pos_of(const Dev &D, int cur);
template <> __device__ __forceinline__ Pos<double> pos_of<double>(const Dev &D, int cur) { return Pos<double>{x_at(D, cur)}; }
template <> __device__ __forceinline__ Pos<float> pos_of<float>(const Dev &D, int cur) { return Pos<float>{mir_at(D, cur)}; }

__device__ __forceinline__ double comp(const V3<double> &a, int c) { return c == 0 ? a.x : (c == 1 ? a.y : a.z); }

// Gaussian deviate of component c of local bead i of a noise stream at step s
// (Box-Muller on one Philox4x32-10 block: components 0,1 share one pair).
__device__ __forceinline__ float gauss_f(unsigned long long seed, int i, unsigned long long s, int c, unsigned stream) {
    const uint4 r = philox4x32_10(make_uint4((unsigned)i, (unsigned)s, (unsigned)(s >> 32), stream),
                                  make_uint2((unsigned)seed, (unsigned)(seed >> 32)));
    const unsigned a = c < 2 ? r.x : r.z, b = c < 2 ? r.y : r.w;
    const float u1 = (float)((a >> 8) + 1u) * (1.0f / 16777216.0f);
    const float u2 = (float)(b >> 8) * (1.0f / 16777216.0f);
    float sn, cs;
    sincospif(2.0f * u2, &sn, &cs);
    return sqrtf(-2.0f * logf(u1)) * (c == 1 ? sn : cs);
}
// the three deviates of bead i from one Philox block: gauss_f for c = 0, 1, 2
__device__ __forceinline__ void gauss_f3(unsigned long long seed, int i, unsigned long long s, unsigned stream, float xi[3]) {
    const uint4 r = philox4x32_10(make_uint4((unsigned)i, (unsigned)s, (unsigned)(s >> 32), stream),
                                  make_uint2((unsigned)seed, (unsigned)(seed >> 32)));
    float sn, cs;
    const float ra = sqrtf(-2.0f * logf((float)((r.x >> 8) + 1u) * (1.0f / 16777216.0f)));
    sincospif(2.0f * ((float)(r.y >> 8) * (1.0f / 16777216.0f)), &sn, &cs);
    xi[0] = ra * cs;
    xi[1] = ra * sn;
    const float rb = sqrtf(-2.0f * logf((float)((r.z >> 8) + 1u) * (1.0f / 16777216.0f)));
    sincospif(2.0f * ((float)(r.w >> 8) * (1.0f / 16777216.0f)), &sn, &cs);
    xi[2] = rb * cs;
}
template <typename R>
__device__ __forceinline__ double gauss3(unsigned long long seed, int i, unsigned long long s, int c, unsigned stream);
template <> __device__ __forceinline__ double gauss3<float>(unsigned long long seed, int i, unsigned long long s, int c,
                                                            unsigned stream) {
    return (double)gauss_f(seed, i, s, c, stream);
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

template <typename R> struct Vec4;
template <> struct Vec4<float> {
    using type = float4;
    __device__ static float4 make(const V3<float> &a) { return make_float4(a.x, a.y, a.z, 0.f); }
};
template <> struct Vec4<double> {
    using type = double4;
    __device__ static double4 make(const V3<double> &a) { return make_double4(a.x, a.y, a.z, 0.0); }
};
template <typename V> __device__ __forceinline__ V3<float> v3of(const float4 &a) { return mk<float>(a.x, a.y, a.z); }
__device__ __forceinline__ V3<float> v3(const float4 &a) { return mk<float>(a.x, a.y, a.z); }
__device__ __forceinline__ V3<double> v3(const double4 &a) { return mk<double>(a.x, a.y, a.z); }

// ------------------------------------------------------- k_bonded, k_bp
// Term-parallel passes before the step kernel.
//  * k_bonded: thread s evaluates the bond (s,s+1), the angle (s,s+1,s+2)
//    and the dihedral (s..s+3) of list_local.F90 (all three term types in
//    every thread, so warps do not diverge) and stores their forces in
//    slot[0..7][s]: bond force on s+1; angle forces on s, s+1, s+2;
//    dihedral forces on s..s+3.  Absent terms store zeros.
//  * k_bp_test, k_bp_eval: base-pair records (force_bp*.F90), grid stride;
//    they scatter forces into fbp and cache ene_bp/bp_status (k_bp_energy
//    computes the energies of energy_bp*.F90).
// The global record index is mapped to (instance, slot) by binary search
// over the per-instance prefix counts written by the last list rebuild.
__device__ __forceinline__ bool bp_record(const Dev &D, int r, int total, int n_inst, int &slot) {
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

// Positions of the bonded pass: the mirror (FP32 path) or the FP64 state.
template <typename R> struct PosLd;
template <> struct PosLd<float> {
    using T = uint4;
    __device__ static T ld(const Dev &D, int cur, int i) { return mir_at(D, cur)[i]; }
    __device__ static V3<float> sep(const T &a, const T &b, const InstP &ip) { return dvec32(a, b, ip); }
};
template <> struct PosLd<double> {
    using T = double4;
    __device__ static T ld(const Dev &D, int cur, int i) { return x_at(D, cur)[i]; }
    __device__ static V3<double> sep(const T &a, const T &b, const InstP &ip) { return dvec64(a, b, ip); }
};

// Bonded terms starting at bead s (list_local.F90 order).  The four positions
// are loaded once and the three separations formed from them (the angle's
// x(q1) - x(s) is the exact negation of the bond's x(s) - x(q1) in both
// precisions).  Forces go to the slot planes slot[k][s], k = 0..7, so that a
// warp's stores are contiguous.  In the FP32 path, an angle term with
// |cos| > NEAR_ONE_STRICT, or a dihedral with a flanking angle that close to
// 0 or 180 degrees, is evaluated again from cross products formed exactly
// from the fixed-point mirror and its residuals (cross_fx); only a sine below
// 1e-6 leaves it flagged for the caller's FP64 evaluation.
template <typename R>
__device__ __forceinline__ void bonded_terms_to(const Dev &D, const GlobP &g, int cur, int s, typename Vec4<R>::type *S, size_t pl,
                                                bool *angle_near, bool *dih_near) {
    using L = PosLd<R>;
    const int4 bi = D.binfo[s];
    const InstP &ip = D.ip[bi.x];
    const int l = bi_lidx(bi), n = bi_clen(bi);
    const bool circ = bi_circ(bi);
    const int q1 = chain_bead(bi, l + 1), q2 = chain_bead(bi, l + 2), q3 = chain_bead(bi, l + 3);
    const bool has_b = q1 >= 0 && (!circ || n >= 2);
    const bool has_a = q2 >= 0 && (!circ || n >= 3);
    const bool has_d = g.dih_type != 0 && q3 >= 0 && (!circ || n >= 4);
    const typename L::T p0 = L::ld(D, cur, s), p1 = L::ld(D, cur, q1 >= 0 ? q1 : s), p2 = L::ld(D, cur, q2 >= 0 ? q2 : s),
                        p3 = L::ld(D, cur, q3 >= 0 ? q3 : s);
    const V3<R> v01 = L::sep(p0, p1, ip), v21 = L::sep(p2, p1, ip), v23 = L::sep(p2, p3, ip);
    const V3<R> z = mk<R>(0, 0, 0);
    *angle_near = *dih_near = false;
    // bond (s, s+1)
    const V3<R> fb = has_b ? bond_f<R>(v01, g) : z;
    // angle (s, s+1, s+2)
    V3<R> Fa[3] = {z, z, z};
    if (has_a) {
        R c;
        angle_forces<R>(-v01, v21, g, Fa, &c);
        if (sizeof(R) == 4) *angle_near = fm::fabs(c) > R(NEAR_ONE_STRICT);
    }
    // dihedral (s, s+1, s+2, s+3)
    V3<R> Fd[4] = {z, z, z, z};
    if (has_d) {
        bool nr;
        dih_forces<R>(v01, v21, v23, g, Fd, &nr);
        if (sizeof(R) == 4) *dih_near = nr;
    }
    if constexpr (sizeof(R) == 4) {
        if (*angle_near || *dih_near) {
            const uint4 *mr = mir_at(D, cur);
            const float4 *rr = res_at(D, cur);
            const FxV a01 = fxv(mr, rr, s, q1), a21 = fxv(mr, rr, q2, q1);
            float s2;
            if (*angle_near) {
                angle_forces_cr(-v01, v21, cross_fx(a21, a01, ip), g, Fa, &s2);
                *angle_near = s2 < 1e-12f;
            }
            if (*dih_near) {
                dih_forces_mn(v01, v21, v23, cross_fx(a01, a21, ip), cross_fx(a21, fxv(mr, rr, q2, q3), ip), g, Fd, &s2);
                *dih_near = s2 < 1e-12f;
            }
        }
    }
    S[0] = Vec4<R>::make(fb);
    S[pl] = Vec4<R>::make(Fa[0]);
    S[2 * pl] = Vec4<R>::make(Fa[1]);
    S[3 * pl] = Vec4<R>::make(Fa[2]);
    S[4 * pl] = Vec4<R>::make(Fd[0]);
    S[5 * pl] = Vec4<R>::make(Fd[1]);
    S[6 * pl] = Vec4<R>::make(Fd[2]);
    S[7 * pl] = Vec4<R>::make(Fd[3]);
}

// FP64 re-evaluation of a flagged angle (kind 0) or dihedral (kind 1) term
// starting at bead s; overwrites its FP32 slot forces.
// the terms starting at bead s into the context's slot planes slot[k][s]
template <typename R>
__device__ __forceinline__ void bonded_terms(const Dev &D, const GlobP &g, int cur, int s, bool *angle_near, bool *dih_near) {
    using V4 = typename Vec4<R>::type;
    bonded_terms_to<R>(D, g, cur, s, (V4 *)D.slot + s, (size_t)g.n, angle_near, dih_near);
}

// FP64 forces of the angle (kind 0: F[0..2]) or dihedral (kind 1: F[0..3])
// term starting at bead s, rounded to FP32
__device__ __noinline__ void bonded_fp64_f(const Dev &D, const GlobP &g, int cur, int s, int kind, float4 *F4) {
    const int4 bi = D.binfo[s];
    const InstP &ip = D.ip[bi.x];
    const double4 *x64 = x_at(D, cur); // coherent: the per-block kernel writes x in the same launch
    const int l = bi_lidx(bi);
    const int q1 = chain_bead(bi, l + 1), q2 = chain_bead(bi, l + 2), q3 = chain_bead(bi, l + 3);
    if (kind == 0) {
        V3<double> F[3];
        double c;
        angle_forces<double>(dvec64(x64[q1], x64[s], ip), dvec64(x64[q2], x64[q1], ip), g, F, &c);
        for (int k = 0; k < 3; ++k) F4[k] = make_float4((float)F[k].x, (float)F[k].y, (float)F[k].z, 0.f);
    } else {
        V3<double> F[4];
        bool nr;
        dih_forces<double>(dvec64(x64[s], x64[q1], ip), dvec64(x64[q2], x64[q1], ip), dvec64(x64[q2], x64[q3], ip), g, F, &nr);
        for (int k = 0; k < 4; ++k) F4[k] = make_float4((float)F[k].x, (float)F[k].y, (float)F[k].z, 0.f);
    }
}
// FP64 re-evaluation of a flagged angle (kind 0) or dihedral (kind 1) term
// starting at bead s; overwrites its FP32 slot forces (planes S[k * pl], by
// default the context's slot planes at s).
__device__ __noinline__ void bonded_fp64_to(const Dev &D, const GlobP &g, int cur, int s, int kind, float4 *S, size_t pl) {
    float4 F[4];
    bonded_fp64_f(D, g, cur, s, kind, F);
    for (int k = 0; k < (kind == 0 ? 3 : 4); ++k) S[(kind == 0 ? 1 + k : 4 + k) * pl] = F[k];
}
__device__ __forceinline__ void bonded_fp64(const Dev &D, const GlobP &g, int cur, int s, int kind) {
    bonded_fp64_to(D, g, cur, s, kind, (float4 *)D.slot + s, (size_t)g.n);
}

// The bonded force on bead i of the mixed path, formed by the bead's own
// thread: the nine terms that act on it (bonds starting at l-1 and l,
// angles starting at l-2..l, dihedrals starting at l-3..l, l its chain
// index), each evaluated as bonded_terms evaluates it (the same FP32
// operations, the exact cross products near straight angles, FP64 below a
// sine of 1e-6), its force on bead i summed in the order the slot gather
// (bonded_gather) adds the slot planes.  E supplies the positions (the
// global mirror, or a shared-memory copy), D the FP64 state.  mask: 1 bond,
// 2 angle, 4 dihedral.
__device__ __forceinline__ V3<float> bonded_bead(const Dev &E, const Dev &D, const GlobP &g, int cur, int i, int mask) {
    using L = PosLd<float>;
    const int4 bi = E.binfo[i];
    const InstP &ip = E.ip[bi.x];
    const int l = bi_lidx(bi), n = bi_clen(bi);
    const bool circ = bi_circ(bi);
    // chain beads l-3 .. l+3 (-1: none) and their mirrors
    int q[7];
#pragma unroll
    for (int d = 0; d < 7; ++d) q[d] = d == 3 ? i : chain_bead(bi, l - 3 + d);
    uint4 p[7];
#pragma unroll
    for (int d = 0; d < 7; ++d) p[d] = L::ld(E, cur, q[d] >= 0 ? q[d] : i);
    const V3<float> z = mk<float>(0.f, 0.f, 0.f);
    V3<float> ab = z;
    // bonds (s, s+1) for s = l-1 (force +fb on bead i) and s = l (-fb)
    if (mask & 1) {
#pragma unroll
        for (int t = 0; t < 2; ++t) {
            const int a = 2 + t; // index of the bond's first bead in q
            if (q[a] < 0 || q[a + 1] < 0 || !(!circ || n >= 2)) continue;
            const V3<float> fb = bond_f<float>(L::sep(p[a], p[a + 1], ip), g);
            ab = ab + (t == 0 ? fb : -fb);
        }
    }
    // angles (s, s+1, s+2) for s = l-2, l-1, l: bead i is their k = 2, 1, 0
    if (mask & 2) {
#pragma unroll
        for (int t = 0; t < 3; ++t) {
            const int a = 1 + t, k = 2 - t;
            if (q[a] < 0 || q[a + 1] < 0 || q[a + 2] < 0 || !(!circ || n >= 3)) continue;
            const V3<float> v01 = L::sep(p[a], p[a + 1], ip), v21 = L::sep(p[a + 2], p[a + 1], ip);
            V3<float> Fa[3];
            float c;
            angle_forces<float>(-v01, v21, g, Fa, &c);
            bool near = fabsf(c) > NEAR_ONE_STRICT;
            if (near) {
                const uint4 *mr = mir_at(E, cur);
                const float4 *rr = res_at(E, cur);
                const FxV a01 = fxv(mr, rr, q[a], q[a + 1]), a21 = fxv(mr, rr, q[a + 2], q[a + 1]);
                float s2;
                angle_forces_cr(-v01, v21, cross_fx(a21, a01, ip), g, Fa, &s2);
                near = s2 < 1e-12f;
            }
            if (near) {
                float4 F[4];
                bonded_fp64_f(D, g, cur, q[a], 0, F);
                Fa[k] = mk<float>(F[k].x, F[k].y, F[k].z);
            }
            ab = ab + Fa[k];
        }
    }
    // dihedrals (s .. s+3) for s = l-3 .. l: bead i is their k = 3 .. 0
    if ((mask & 4) && g.dih_type != 0) {
#pragma unroll
        for (int t = 0; t < 4; ++t) {
            const int a = t, k = 3 - t;
            if (q[a] < 0 || q[a + 1] < 0 || q[a + 2] < 0 || q[a + 3] < 0 || !(!circ || n >= 4)) continue;
            const V3<float> v01 = L::sep(p[a], p[a + 1], ip), v21 = L::sep(p[a + 2], p[a + 1], ip),
                            v23 = L::sep(p[a + 2], p[a + 3], ip);
            V3<float> Fd[4];
            bool near;
            dih_forces<float>(v01, v21, v23, g, Fd, &near);
            if (near) {
                const uint4 *mr = mir_at(E, cur);
                const float4 *rr = res_at(E, cur);
                const FxV a01 = fxv(mr, rr, q[a], q[a + 1]), a21 = fxv(mr, rr, q[a + 2], q[a + 1]);
                float s2;
                dih_forces_mn(v01, v21, v23, cross_fx(a01, a21, ip), cross_fx(a21, fxv(mr, rr, q[a + 2], q[a + 3]), ip), g, Fd, &s2);
                near = s2 < 1e-12f;
            }
            if (near) {
                float4 F[4];
                bonded_fp64_f(D, g, cur, q[a], 1, F);
                Fd[k] = mk<float>(F[k].x, F[k].y, F[k].z);
            }
            ab = ab + Fd[k];
        }
    }
    return ab;
}

// window and free-energy test of one record (force mode); returns true when
// the 6-bead term has to be evaluated.  Records that fail are given zero
// energy and status, as force_bp*.F90 zero ene_bp/bp_status before the loop
// (with rec_out; a caller that runs several steps writes them on the last).
template <typename R> __device__ __forceinline__ bool bp_test(const Dev &D, const GlobP &g, int cur, int slot, bool rec_out = true) {
    const int4 rec = D.bps[slot];
    const int type = rec.z & 0xff;
    const InstP &ip = D.ip[rec.w];
    bool pass;
    const bool triplet = g.bp_model == 4 || g.bp_model == 5;
    if (g.nstep_mc > 0 && !D.mc_due[rec.w] && !D.bp_mask[slot]) {
        // removed by the last Monte Carlo pass (force_bp_triplet.F90:64-66)
        pass = false;
    } else if (g.flg_bias_ss && triplet) {
        // [Bias_SS] (force_bp_triplet.F90:78-92, force_bp_limit_triplet.F90:
        // 97-113): dG < 0 first, then the exact distance window, the test the
        // evaluation repeats; outside it, a constant pull of i toward j
        const int h = rec.z >> 8;
        if constexpr (sizeof(R) == 4) pass = D.bp_dgf[rec.w * 469 + h] < 0.f;
        else pass = __dsub_rn(D.bp3_dH[h], __dmul_rn(ip.tempK, D.bp3_dS[h])) < 0.0;
        if (pass) {
            double a12, fx, fy, fz;
            bool out;
            if constexpr (sizeof(R) == 4) {
                const BPPf &bf = D.bppf[type];
                const V3<float> v = dvec32(mir_at(D, cur)[rec.x], mir_at(D, cur)[rec.y], ip);
                const float af = sqrtf(dot3(v, v));
                out = fabsf(af - bf.bond_r) > bf.cutoff_ddist;
                a12 = af;
                fx = v.x, fy = v.y, fz = v.z;
            } else {
                const BPP &b = D.bpp[type];
                const V3<double> v = dvec64(x_at(D, cur)[rec.x], x_at(D, cur)[rec.y], ip);
                a12 = sqrt(dot3(v, v));
                out = fabs(a12 - b.bond_r) > b.cutoff_ddist;
                fx = v.x, fy = v.y, fz = v.z;
            }
            if (out) {
                const double c = g.bias_ss_force / a12;
                fx *= c;
                fy *= c;
                fz *= c;
                if (g.prec == 0) {
                    atomicAdd(&D.fbp[rec.x].x, -fx);
                    atomicAdd(&D.fbp[rec.x].y, -fy);
                    atomicAdd(&D.fbp[rec.x].z, -fz);
                    atomicAdd(&D.fbp[rec.y].x, fx);
                    atomicAdd(&D.fbp[rec.y].y, fy);
                    atomicAdd(&D.fbp[rec.y].z, fz);
                } else if (fabs(fx) < FX_LIMIT && fabs(fy) < FX_LIMIT && fabs(fz) < FX_LIMIT) {
                    fx_scatter(D.fbp, rec.x, -fx_of(fx), -fx_of(fy), -fx_of(fz));
                    fx_scatter(D.fbp, rec.y, fx_of(fx), fx_of(fy), fx_of(fz));
                } else {
                    atomicOr(D.err, ERR_NONFINITE);
                }
                pass = false;
            }
        }
        if (!pass && rec_out) {
            D.ene_bp[slot] = 0.0;
            D.bp_status[slot] = 0;
        }
        return pass;
    } else if constexpr (sizeof(R) == 4) {
        const BPPf &bf = D.bppf[type];
        const V3<float> v = dvec32(mir_at(D, cur)[rec.x], mir_at(D, cur)[rec.y], ip);
        const float d2 = fmaf(v.x, v.x, fmaf(v.y, v.y, v.z * v.z));
        // window widened by 1e-5 relative; the exact test follows
        pass = d2 >= bf.lo2 * 0.99999f && d2 <= bf.hi2 * 1.00001f;
    } else {
        const BPP &b = D.bpp[type];
        const V3<double> v = dvec64(x_at(D, cur)[rec.x], x_at(D, cur)[rec.y], ip);
        pass = fabs(sqrt(dot3(v, v)) - b.bond_r) <= b.cutoff_ddist;
    }
    if (pass && (g.bp_model == 4 || g.bp_model == 5)) {
        const int h = rec.z >> 8;
        if constexpr (sizeof(R) == 4) pass = D.bp_dgf[rec.w * 469 + h] < 0.f;
        else pass = __dsub_rn(D.bp3_dH[h], __dmul_rn(ip.tempK, D.bp3_dS[h])) < 0.0;
    }
    if (!pass && rec_out) {
        D.ene_bp[slot] = 0.0;
        D.bp_status[slot] = 0;
    }
    return pass;
}

// force_bp.F90:44-204 / force_bp_triplet.F90:62-240 for one record that
// passed bp_test: forces scattered into fbp, energy and status cached.
// bp_finish applies the energy cut and the scatter.  In the mixed path,
// contributions with exp(-u) < 2e-9 (u > 20) are not scattered (their forces
// are below the FP32 rounding of the remaining terms) but their energy is
// still cached, and forces go to fbp as fixed point.

__device__ __forceinline__ void bp_finish(const Dev &D, const GlobP &g, int slot, const int4 &rec, const int4 &nb, double dG,
                                          const V3<double> *fd, double ud, bool ok, bool scatter_all, double4 *fbp) {
    const int type = rec.z & 0xff;
    const bool triplet = g.bp_model == 4 || g.bp_model == 5;
    double ene = 0.0;
    unsigned char st = 0;
    if (ok) {
        const BPP &b = D.bpp[type];
        const double e = triplet ? b.U0 * dG * exp(-ud) : b.U0 * exp(-ud);
        if (e <= g.bp_cutoff_energy) {
            ene = e;
            st = 1;
            if (g.nstep_mc > 0 && D.mc_due[rec.w]) {
                // Monte Carlo pass: keep the record's forces until k_bp_mc decides
                long long *fr = D.bp_frec + (size_t)slot * 18;
                for (int q = 0; q < 6; ++q) {
                    const V3<double> c = e * fd[q];
                    const double cc[3] = {c.x, c.y, c.z};
                    for (int k = 0; k < 3; ++k) {
                        long long w;
                        if (g.prec == 0) w = __double_as_longlong(cc[k]);
                        else if (!(scatter_all || ud <= 20.0)) w = 0;
                        else if (fabs(cc[k]) < FX_LIMIT) w = fx_of(cc[k]);
                        else {
                            atomicOr(D.err, ERR_NONFINITE);
                            w = 0;
                        }
                        fr[3 * q + k] = w;
                    }
                }
            } else if (scatter_all || ud <= 20.0) {
                const int ids[6] = {rec.x, rec.y, nb.x, nb.y, nb.z, nb.w};
#pragma unroll
                for (int q = 0; q < 6; ++q) {
                    if (g.prec == 0) {
                        atomicAdd(&fbp[ids[q]].x, e * fd[q].x);
                        atomicAdd(&fbp[ids[q]].y, e * fd[q].y);
                        atomicAdd(&fbp[ids[q]].z, e * fd[q].z);
                    } else {
                        const V3<double> c = e * fd[q];
                        if (!(fabs(c.x) < FX_LIMIT && fabs(c.y) < FX_LIMIT && fabs(c.z) < FX_LIMIT)) {
                            atomicOr(D.err, ERR_NONFINITE);
                            continue;
                        }
                        fx_scatter(fbp, ids[q], fx_of(c.x), fx_of(c.y), fx_of(c.z));
                    }
                }
            }
        }
    }
    D.ene_bp[slot] = ene;
    D.bp_status[slot] = st;
}

__device__ __forceinline__ double bp_dG(const Dev &D, const GlobP &g, const int4 &rec) {
    if (!(g.bp_model == 4 || g.bp_model == 5)) return 1.0;
    const int h = rec.z >> 8;
    return __dsub_rn(D.bp3_dH[h], __dmul_rn(D.ip[rec.w].tempK, D.bp3_dS[h]));
}

// FP64 evaluation (FP64 path, and records flagged near +-1 by the FP32 path)
// fbp: the scatter target (the context's fbp, or a block's shared copy)
__device__ __noinline__ void bp_eval_d(const Dev &D, const GlobP &g, int cur, int slot, double4 *fbp) {
    const double4 *x64 = x_at(D, cur); // coherent: the per-block kernel writes x in the same launch
    const int4 rec = D.bps[slot];
    const int4 nb = D.bps_n[slot];
    const InstP &ip = D.ip[rec.w];
    V3<double> fd[6];
    double ud = 0.0;
    bool nr;
    const bool ok = bp_force_core<double, BPP>(dvec64(x64[rec.x], x64[rec.y], ip), dvec64(x64[rec.x], x64[nb.x], ip),
                                               dvec64(x64[rec.x], x64[nb.z], ip), dvec64(x64[nb.y], x64[rec.y], ip),
                                               dvec64(x64[nb.w], x64[rec.y], ip), D.bpp[rec.z & 0xff], fd, &ud, &nr);
    bp_finish(D, g, slot, rec, nb, bp_dG(D, g, rec), fd, ud, ok, g.prec == 0, fbp);
}

// FP32 evaluation.  A record with a bond angle within 0.03 rad of 0 or 180
// degrees is evaluated again with its four cross products from the exact
// mirror differences and residuals (cross_fx); only if an angle is within
// 1e-6 rad does it return true (writing nothing), so that the caller redoes
// the record in FP64.  rec_out: write the record's energy and status.
__device__ __forceinline__ bool bp_eval_f(const Dev &D, const GlobP &g, int cur, int slot, bool rec_out = true) {
    const uint4 *__restrict__ m = mir_at(D, cur);
    const int4 rec = D.bps[slot];
    const int4 nb = D.bps_n[slot];
    const InstP &ip = D.ip[rec.w];
    V3<float> f[6];
    float u;
    bool nr = false;
    const BPPf &bf = D.bppf[rec.z & 0xff];
    const V3<float> v12 = dvec32(m[rec.x], m[rec.y], ip), v13 = dvec32(m[rec.x], m[nb.x], ip),
                    v15 = dvec32(m[rec.x], m[nb.z], ip), v42 = dvec32(m[nb.y], m[rec.y], ip),
                    v62 = dvec32(m[nb.w], m[rec.y], ip);
    bool ok = bp_force_core_f(v12, v13, v15, v42, v62, bf, nullptr, f, &u, &nr);
    if (ok && nr) {
        const float4 *r = res_at(D, cur);
        const FxV a12 = fxv(m, r, rec.x, rec.y);
        const V3<float> cc[4] = {cross_fx(a12, fxv(m, r, rec.x, nb.x), ip), cross_fx(a12, fxv(m, r, rec.x, nb.z), ip),
                                 cross_fx(fxv(m, r, nb.y, rec.y), a12, ip), cross_fx(fxv(m, r, nb.w, rec.y), a12, ip)};
        ok = bp_force_core_f(v12, v13, v15, v42, v62, bf, cc, f, &u, &nr);
    }
    if (ok && nr) return true;
    float e = 0.f;
    unsigned char st = 0;
    if (ok) {
        const bool triplet = g.bp_model == 4 || g.bp_model == 5;
        const float ex = expf(-u);
        e = triplet ? bf.U0 * D.bp_dgf[rec.w * 469 + (rec.z >> 8)] * ex : bf.U0 * ex;
        st = e <= g.f_bp_cutoff_energy;
        if (!st) {
            e = 0.f;
        } else if (g.nstep_mc > 0 && D.mc_due[rec.w]) {
            // Monte Carlo pass: keep the record's forces until k_bp_mc decides
            long long *fr = D.bp_frec + (size_t)slot * 18;
            for (int q = 0; q < 6; ++q) {
                const float c[3] = {e * f[q].x, e * f[q].y, e * f[q].z};
                for (int k = 0; k < 3; ++k) {
                    long long w = 0;
                    if (u <= 20.f) {
                        if (fabsf(c[k]) < FX_LIMIT) w = fx_of(c[k]);
                        else atomicOr(D.err, ERR_NONFINITE);
                    }
                    fr[3 * q + k] = w;
                }
            }
        } else if (u <= 20.f) {
            const int ids[6] = {rec.x, rec.y, nb.x, nb.y, nb.z, nb.w};
#pragma unroll
            for (int q = 0; q < 6; ++q) {
                const float cx = e * f[q].x, cy = e * f[q].y, cz = e * f[q].z;
                if (!(fabsf(cx) < FX_LIMIT && fabsf(cy) < FX_LIMIT && fabsf(cz) < FX_LIMIT)) {
                    atomicOr(D.err, ERR_NONFINITE);
                    continue;
                }
                fx_scatter(D.fbp, ids[q], fx_of(cx), fx_of(cy), fx_of(cz));
            }
        }
    }
    if (rec_out) {
        D.ene_bp[slot] = (double)e;
        D.bp_status[slot] = st;
    }
    return false;
}

// --------------------------------------------------- bonded and base pairs
// Bonded terms, one start bead per thread; flagged terms are queued in shared
// memory and re-evaluated in FP64 on packed warps.
template <typename R> __global__ void __launch_bounds__(256) k_bonded(Dev D, GlobP g, int cur) {
    __shared__ int qa[256], qd[256];
    __shared__ int na, nd;
    if (threadIdx.x == 0) na = nd = 0;
    __syncthreads();
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s < g.n) {
        bool an, dn;
        bonded_terms<R>(D, g, cur, s, &an, &dn);
        if (an) qa[atomicAdd(&na, 1)] = s;
        if (dn) qd[atomicAdd(&nd, 1)] = s;
    }
    __syncthreads();
    if constexpr (sizeof(R) == 4) {
        for (int k = threadIdx.x; k < na; k += blockDim.x) bonded_fp64(D, g, cur, qa[k], 0);
        for (int k = threadIdx.x; k < nd; k += blockDim.x) bonded_fp64(D, g, cur, qd[k], 1);
    }
}

// The mixed path's bonded pass of a step: the terms starting at the block's
// 256 beads and at the 3 beads before them (k_bonded's evaluation) into
// shared-memory slot planes, then each bead's sum in slot order (the order
// of bonded_gather) into fbond, which k_step_mixed reads as one load.  A
// bead whose terms start outside that range (the wrap of a circular chain)
// forms its sum itself (bonded_bead, the same values).
constexpr int kBondHalo = 3;
__device__ __noinline__ float4 bonded_bead_global(const Dev &D, const GlobP &g, int cur, int i) {
    const V3<float> f = bonded_bead(D, D, g, cur, i, 7);
    return make_float4(f.x, f.y, f.z, 0.f);
}
__global__ void __launch_bounds__(256, 3) k_bonded_fb(const __grid_constant__ Dev D, const __grid_constant__ GlobP g, int cur) {
    __shared__ float4 sS[8][256 + kBondHalo];
    constexpr int pl = 256 + kBondHalo;
    const int b0 = blockIdx.x * 256;
    for (int t = threadIdx.x; t < pl; t += 256) {
        const int s = b0 - kBondHalo + t;
        if (s < 0 || s >= g.n) continue;
        bool an, dn;
        bonded_terms_to<float>(D, g, cur, s, &sS[0][t], pl, &an, &dn);
        if (an) bonded_fp64_to(D, g, cur, s, 0, &sS[0][t], pl);
        if (dn) bonded_fp64_to(D, g, cur, s, 1, &sS[0][t], pl);
    }
    __syncthreads();
    const int i = b0 + threadIdx.x;
    if (i >= g.n) return;
    const int4 bi = D.binfo[i];
    const int l = bi_lidx(bi);
    int qs[9], ks[9];
    bool inside = true;
#pragma unroll
    for (int t = 0; t < 9; ++t) {
        const int start = t < 2 ? l - 1 + t : t < 5 ? l - 2 + (t - 2) : l - 3 + (t - 5);
        ks[t] = t < 2 ? 0 : t < 5 ? 1 + (2 - (t - 2)) : 4 + (3 - (t - 5));
        qs[t] = chain_bead(bi, start);
        const int loc = qs[t] - (b0 - kBondHalo);
        inside &= qs[t] < 0 || (loc >= 0 && loc < pl);
    }
    if (!inside) {
        D.fbond[i] = bonded_bead_global(D, g, cur, i);
        return;
    }
    V3<float> ab = mk<float>(0.f, 0.f, 0.f);
#pragma unroll
    for (int t = 0; t < 9; ++t) {
        if (qs[t] < 0) continue;
        const float4 v = sS[ks[t]][qs[t] - (b0 - kBondHalo)];
        const V3<float> f = mk<float>(v.x, v.y, v.z);
        ab = ab + (t == 1 ? -f : f);
    }
    D.fbond[i] = make_float4(ab.x, ab.y, ab.z, 0.f);
}

// Base-pair records in two passes.  k_bp_test gives every record one thread
// (few registers, so the whole list is resident at once) and appends the
// records inside the distance window to bp_win, about one in ten; k_bp_eval
// then evaluates one windowed record per thread, so the 6-bead term runs on
// full warps.  The FP32 evaluation defers the records with a bond angle
// within 1e-6 rad of 0 or 180 degrees (there are none in ordinary dynamics);
// the last block of k_bp_eval to finish evaluates them in FP64 and resets the
// counts for the next pass.  The order of bp_win does not matter: each record
// writes its own energy and status, and forces add exactly (fixed point) in
// the mixed path.
template <typename R> __device__ __forceinline__ void bp_eval(const Dev &D, const GlobP &g, int cur, int slot) {
    if constexpr (sizeof(R) == 4) {
        if (bp_eval_f(D, g, cur, slot)) D.bp_fixq[atomicAdd(D.bp_fixn, 1)] = slot;
    } else {
        bp_eval_d(D, g, cur, slot, D.fbp);
    }
}

template <typename R> __global__ void __launch_bounds__(256) k_bp_test(Dev D, GlobP g, int cur) {
    const int lane = threadIdx.x & 31;
    const int total = *D.bp_total;
    for (int base = (int)blockIdx.x * 256; base < total; base += (int)gridDim.x * 256) {
        int slot = -1;
        bool pass = false;
        if (bp_record(D, base + (int)threadIdx.x, total, g.n_inst, slot)) pass = bp_test<R>(D, g, cur, slot);
        const unsigned bal = __ballot_sync(0xffffffffu, pass);
        int wb = 0;
        if (lane == 0 && bal) wb = atomicAdd(D.bp_nwin, __popc(bal));
        wb = __shfl_sync(0xffffffffu, wb, 0);
        if (pass) D.bp_win[wb + __popc(bal & ((1u << lane) - 1u))] = slot;
    }
}

// Base-pair records in one pass: one thread per record tests the distance
// window (bp_test); the records inside it, about one in ten, are queued in
// shared memory and evaluated 256 at a time, one per thread, so the 6-bead
// term runs on full warps.  A record the FP32 evaluation hands back (a bond
// angle within 1e-6 rad of 0 or 180 degrees, none in ordinary dynamics) is
// evaluated in FP64 by the same thread.  Each record writes its own energy
// and status, and forces add exactly (fixed point) in the mixed path, so
// the order of evaluation does not matter.
template <typename R> __device__ __forceinline__ void bp_eval_now(const Dev &D, const GlobP &g, int cur, int slot) {
    if constexpr (sizeof(R) == 4) {
        if (bp_eval_f(D, g, cur, slot)) bp_eval_d(D, g, cur, slot, D.fbp);
    } else {
        bp_eval_d(D, g, cur, slot, D.fbp);
    }
}
template <typename R> __global__ void __launch_bounds__(256, 2) k_bp(Dev D, GlobP g, int cur) {
    __shared__ int s_q[512];
    __shared__ int s_n;
    const int lane = threadIdx.x & 31;
    const int total = *D.bp_total;
    if (threadIdx.x == 0) s_n = 0;
    __syncthreads();
    for (int base = (int)blockIdx.x * 256; base < total; base += (int)gridDim.x * 256) {
        int slot = -1;
        bool pass = false;
        if (bp_record(D, base + (int)threadIdx.x, total, g.n_inst, slot)) pass = bp_test<R>(D, g, cur, slot);
        const unsigned bal = __ballot_sync(0xffffffffu, pass);
        int wb = 0;
        if (lane == 0 && bal) wb = atomicAdd(&s_n, __popc(bal));
        wb = __shfl_sync(0xffffffffu, wb, 0);
        if (pass) s_q[wb + __popc(bal & ((1u << lane) - 1u))] = slot;
        __syncthreads();
        const int n = s_n; // at most 511
        if (n >= 256) {
            bp_eval_now<R>(D, g, cur, s_q[threadIdx.x]);
            __syncthreads();
            if ((int)threadIdx.x < n - 256) s_q[threadIdx.x] = s_q[256 + threadIdx.x];
            if (threadIdx.x == 0) s_n = n - 256;
        }
        __syncthreads();
    }
    if ((int)threadIdx.x < s_n) bp_eval_now<R>(D, g, cur, s_q[threadIdx.x]);
}

template <typename R> __global__ void __launch_bounds__(256) k_bp_eval(Dev D, GlobP g, int cur) {
    __shared__ int s_last;
    const int n = *(volatile int *)D.bp_nwin;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) bp_eval<R>(D, g, cur, D.bp_win[k]);
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) s_last = atomicAdd(&D.ticket[2], 1u) == gridDim.x - 1;
    __syncthreads();
    if (!s_last) return;
    __threadfence();
    if constexpr (sizeof(R) == 4) {
        const int nf = *(volatile int *)D.bp_fixn;
        for (int k = threadIdx.x; k < nf; k += blockDim.x) bp_eval_d(D, g, cur, D.bp_fixq[k], D.fbp);
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        *D.bp_fixn = 0;
        *D.bp_nwin = 0;
        D.ticket[2] = 0u;
    }
}

// ------------------------------------------------ base-pair Monte Carlo
// Uniforms of the Monte Carlo pass: the caller's sequence, or Philox blocks
// keyed by (draw, pass counter, tag bit, instance stream), turned into (0,1)
// and [0,1] doubles the way genrand_double3 and genrand_double1 build theirs
// from two 32-bit words (mt_stream.F90:708-769).
__device__ double mc_uniform(const Dev &D, const GlobP &g, const InstP &ip, unsigned long long call, unsigned idx, bool closed) {
    if (D.mc_draws) {
        const int p = atomicAdd(D.mc_draw_pos, 1);
        if (p < D.mc_n_draws) return D.mc_draws[p];
        atomicOr(D.err, ERR_NONFINITE);
        return 0.5;
    }
    const uint4 r = philox4x32_10(make_uint4(idx, (unsigned)call, (unsigned)(call >> 32) | 0x80000000u, ip.stream),
                                  make_uint2((unsigned)g.seed, (unsigned)(g.seed >> 32)));
    if (closed) return ((double)(r.x >> 5) * 67108864.0 + (double)(r.y >> 6)) * (1.0 / 9007199254740991.0);
    return ((double)(r.x >> 6) * 67108864.0 + (double)(r.y >> 6) + 0.5) * (1.0 / 4503599627370496.0);
}

// force_bp_limit_triplet.F90:181-233 for every instance whose pass is due,
// one block per instance: count the pairs of every nucleotide; while some
// nucleotide carries more than max_bp_per_nt, pick one of them uniformly
// (in index order), gather its pairs in the reference's record order (i, j),
// shuffle them with one (0,1) draw per position, walk them keeping the
// candidate with probability exp((E_j - E_keep)/kT) ([0,1] draws) and remove
// the survivor; then scatter the remaining pairs' forces and store the mask.
template <typename R> __global__ void __launch_bounds__(256) k_bp_mc(Dev D, GlobP g) {
    const int k = blockIdx.x;
    if (!D.mc_due[k]) return;
    __shared__ int s_cnt, s_nt, s_m;
    __shared__ int s_warp[8];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const InstP &ip = D.ip[k];
    const int b0 = ip.bead_off, nb = ip.n;
    const int seg = ip.bp_off, cnt = min(D.bp_cnt[k], ip.bp_cap);
    for (int i = tid; i < nb; i += 256) D.mc_excess[b0 + i] = -g.max_bp_per_nt;
    __syncthreads();
    for (int q = tid; q < cnt; q += 256)
        if (D.bp_status[seg + q]) {
            const int4 rec = D.bps[seg + q];
            atomicAdd(&D.mc_excess[rec.x], 1);
            atomicAdd(&D.mc_excess[rec.y], 1);
        }
    __syncthreads();
    const double kB = 1.380649e-23 * ((1.0 / 4184.0) * 6.02214076e23);
    const double beta = 1.0 / (kB * ip.tempK);
    const unsigned long long call = D.mc_calls[k];
    unsigned draw = 0;
    for (;;) {
        // nucleotides with excess pairs, in index order
        if (tid == 0) s_cnt = 0;
        __syncthreads();
        for (int base = 0; base < nb; base += 256) {
            const int i = base + tid;
            const bool f = i < nb && D.mc_excess[b0 + i] > 0;
            const unsigned bal = __ballot_sync(0xffffffffu, f);
            if (lane == 0) s_warp[warp] = __popc(bal);
            __syncthreads();
            int before = s_cnt;
            for (int w = 0; w < warp; ++w) before += s_warp[w];
            if (f) D.mc_list[b0 + before + __popc(bal & ((1u << lane) - 1u))] = b0 + i;
            __syncthreads();
            if (tid == 0)
                for (int w = 0; w < 8; ++w) s_cnt += s_warp[w];
            __syncthreads();
        }
        const int nex = s_cnt;
        if (nex == 0) break;
        if (tid == 0) {
            const double rnd = mc_uniform(D, g, ip, call, draw++, false);
            s_nt = D.mc_list[b0 + (int)ceil(rnd * (double)nex) - 1];
            s_m = 0;
        }
        __syncthreads();
        const int nt = s_nt;
        for (int q = tid; q < cnt; q += 256) {
            const int slot = seg + q;
            if (!D.bp_status[slot]) continue;
            const int4 rec = D.bps[slot];
            if (rec.x == nt || rec.y == nt) D.mc_seq[seg + atomicAdd(&s_m, 1)] = slot;
        }
        __syncthreads();
        if (tid == 0) {
            const int m = s_m;
            int *sq = D.mc_seq + seg;
            for (int a = 1; a < m; ++a) {
                const int v = sq[a];
                const int4 rv = D.bps[v];
                int b = a - 1;
                while (b >= 0) {
                    const int4 rb = D.bps[sq[b]];
                    if (rb.x < rv.x || (rb.x == rv.x && rb.y < rv.y)) break;
                    sq[b + 1] = sq[b];
                    --b;
                }
                sq[b + 1] = v;
            }
            for (int a = 0; a < m; ++a) {
                const double rnd = mc_uniform(D, g, ip, call, draw++, false);
                const int b = (int)ceil(rnd * (double)m) - 1;
                const int t = sq[a];
                sq[a] = sq[b];
                sq[b] = t;
            }
            int del = sq[0];
            for (int a = 1; a < m; ++a) {
                const int j = sq[a];
                const double ratio = exp((D.ene_bp[j] - D.ene_bp[del]) * beta);
                const double rnd = mc_uniform(D, g, ip, call, draw++, true);
                if (rnd < ratio) del = j;
            }
            D.bp_status[del] = 0;
            D.ene_bp[del] = 0.0;
            const int4 rd = D.bps[del];
            D.mc_excess[rd.x] -= 1;
            D.mc_excess[rd.y] -= 1;
        }
        __syncthreads();
    }
    // the survivors: mask of the following steps, and their forces
    for (int q = tid; q < cnt; q += 256) {
        const int slot = seg + q;
        const unsigned char st = D.bp_status[slot];
        D.bp_mask[slot] = st;
        if (!st) continue;
        const int4 rec = D.bps[slot], nb4 = D.bps_n[slot];
        const int ids[6] = {rec.x, rec.y, nb4.x, nb4.y, nb4.z, nb4.w};
        const long long *fr = D.bp_frec + (size_t)slot * 18;
        for (int b = 0; b < 6; ++b) {
            if constexpr (sizeof(R) == 4) {
                fx_scatter(D.fbp, ids[b], fr[3 * b], fr[3 * b + 1], fr[3 * b + 2]);
            } else {
                atomicAdd(&D.fbp[ids[b]].x, __longlong_as_double(fr[3 * b]));
                atomicAdd(&D.fbp[ids[b]].y, __longlong_as_double(fr[3 * b + 1]));
                atomicAdd(&D.fbp[ids[b]].z, __longlong_as_double(fr[3 * b + 2]));
            }
        }
    }
    if (tid == 0) {
        D.mc_due[k] = 0;
        D.mc_calls[k] = call + 1;
    }
}

cudaError_t launch_bp_mc(const Dev &D, const GlobP &g, cudaStream_t st) {
    if (g.nstep_mc <= 0) return cudaSuccess;
    if (g.prec == 0) k_bp_mc<double><<<g.n_inst, 256, 0, st>>>(D, g);
    else k_bp_mc<float><<<g.n_inst, 256, 0, st>>>(D, g);
    return cudaGetLastError();
}

// energy_bp.F90 / energy_bp_triplet.F90 for every record at temperature tK
// (tK < 0: each instance's own): clamped angles, FP64 from the FP64 positions.
__global__ void __launch_bounds__(256) k_bp_energy(Dev D, GlobP g, int cur, double tK_in) {
    const double4 *__restrict__ x64 = x_at(D, cur);
    const int total = *D.bp_total;
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < total; r += gridDim.x * blockDim.x) {
        int slot;
        if (!bp_record(D, r, total, g.n_inst, slot)) break;
        const int4 rec = D.bps[slot];
        const int4 nb = D.bps_n[slot];
        const int i1 = rec.x, i2 = rec.y, type = rec.z & 0xff, h = rec.z >> 8;
        const InstP &ip = D.ip[rec.w];
        const BPP &b = D.bpp[type];
        const bool triplet = g.bp_model == 4 || g.bp_model == 5;
        double ene = 0.0, dG = 1.0;
        unsigned char st = 0;
        // records removed by the last Monte Carlo pass (energy_bp_triplet.F90:40)
        bool skip = g.nstep_mc > 0 && !D.bp_mask[slot];
        if (triplet && !skip) {
            double tK = tK_in < 0 ? ip.tempK : tK_in;
            if (g.temp_indep) tK = 0.0;
            dG = __dsub_rn(D.bp3_dH[h], __dmul_rn(tK, D.bp3_dS[h]));
            skip = dG >= 0.0;
        }
        const V3<double> v = dvec64(x64[i1], x64[i2], ip);
        const double d = sqrt(dot3(v, v)) - b.bond_r;
        if (!skip && fabs(d) <= b.cutoff_ddist) {
            double u = b.bond_k * (d * d);
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
            const double e = triplet ? b.U0 * dG * exp(-u) : b.U0 * exp(-u);
            if (e <= g.bp_cutoff_energy) {
                ene = e;
                st = 1;
            }
        }
        D.ene_bp[slot] = ene;
        D.bp_status[slot] = st;
    }
}

// three Gaussian deviates of one bead from one Philox4x32-10 block
// (Box-Muller on the pairs (r.x, r.y) and (r.z, r.w)); equal to gauss3 for
// components 0, 1, 2

// ------------------------------------------------------------------ k_step
// Phase A (G lanes per bead): WCA + Debye-Hueckel over the bead's full pair
// list and the gather of the bead's bonded slot forces, reduced over the
// lanes; the per-bead sums go to shared memory.
// Phase B (one thread per bead component, packed): FP64 accumulation of the
// force (pair + bonded + base pair) and the GJF-2GJ / Ermak-McCammon update
// (job_md.F90:415-456).  Packing the FP64 work onto whole warps keeps the
// reduced-rate FP64 pipe busy with useful lanes only.
// Phase C (one thread per bead): displacement^2 since the last rebuild and
// its top two per instance; the last block evaluates the rebuild trigger of
// every instance (job_md.F90:376-395).
// MODE 1 computes forces only (terms selected by mask) into fout.

// Phase A of a step: WCA and Debye-Hueckel forces on bead i from its merged
// pair list, lane `lane` of G taking every G-th entry (force_wca.F90:34-67,
// force_ele_DH.F90:39-82); mask bit 16 WCA, bit 32 ele
template <typename R, int G>
__device__ __forceinline__ V3<R> pair_sum(const Dev &D, const GlobP &g, int cur, int i, int lane, const InstP &ip, int mask) {
    V3<R> an = mk<R>(0, 0, 0);
    const int cnt = min(D.nnbr[i], g.cap);
    const int *__restrict__ nb = D.nbr + (size_t)i * g.cap;
    if constexpr (sizeof(R) == 4) {
        const uint4 mi = mir_at(D, cur)[i];
        const uint4 *__restrict__ mir = mir_at(D, cur);
        const float f0 = ip.finv[0], f1 = ip.finv[1], f2 = ip.finv[2];
        const float sig2 = g.f_wca_sig2, wcoef = g.f_wca_coef;
        const float ecoef = ip.ele_coef_f, rc = ip.rcdist_f;
        const float cut2 = g.flg_ele ? ip.ele_cut2_f : -1.f;
#pragma unroll 4
        for (int k = lane; k < cnt; k += G) {
            const int e = __ldg(nb + k);
            const uint4 mj = __ldg(mir + (e & IDX_MASK));
            const float vx = (float)(int)(mi.x - mj.x) * f0;
            const float vy = (float)(int)(mi.y - mj.y) * f1;
            const float vz = (float)(int)(mi.z - mj.z) * f2;
            const float d2 = fmaf(vx, vx, fmaf(vy, vy, vz * vz));
            float c = 0.f;
            if ((e & WCA_BIT) && (mask & 16) && d2 < sig2) {
                const float sq = __fdiv_rn(sig2, d2);
                const float s2 = sq * sq, s4 = s2 * s2;
                c += wcoef * (s4 * s2 * sq - s4);
            }
            if ((e & ELE_BIT) && (mask & 32) && d2 <= cut2) {
                float ri = rsqrtf(d2);
                ri = ri * fmaf(-0.5f * d2 * ri, ri, 1.5f);
                const float r = d2 * ri;
                c += ecoef * ri * ri * (ri + rc) * __expf(-r * rc);
            }
            an.x = fmaf(c, vx, an.x);
            an.y = fmaf(c, vy, an.y);
            an.z = fmaf(c, vz, an.z);
        }
    } else {
        const R sig2 = g.wca_sig2, wcoef = g.wca_coef;
        const R ecoef = ip.ele_coef, rc = ip.rcdist;
        const R cut2 = g.flg_ele ? ip.ele_cut2 : R(-1);
        const Pos<R> P = pos_of<R>(D, cur);
        for (int k = lane; k < cnt; k += G) {
            const int e = __ldg(nb + k);
            const V3<R> v = P.d(i, e & IDX_MASK, ip);
            const R c = pair_coef<R>(e, dot3(v, v), sig2, wcoef, ecoef, rc, cut2, mask);
            an = an + c * v;
        }
    }
    return an;
}

// pair_sum for k_pairs, whose register budget leaves room for the batch
template <typename R, int G>
__device__ __forceinline__ V3<R> pair_sum_b(const Dev &D, const GlobP &g, int cur, int i, int lane, const InstP &ip, int mask) {
    V3<R> an = mk<R>(0, 0, 0);
    const int cnt = min(D.nnbr[i], g.cap);
    const int *__restrict__ nb = D.nbr + (size_t)i * g.cap;
    if constexpr (sizeof(R) == 4) {
        const uint4 mi = mir_at(D, cur)[i];
        const uint4 *__restrict__ mir = mir_at(D, cur);
        const float f0 = ip.finv[0], f1 = ip.finv[1], f2 = ip.finv[2];
        const float sig2 = g.f_wca_sig2, wcoef = g.f_wca_coef;
        const float ecoef = ip.ele_coef_f, rc = ip.rcdist_f;
        const float cut2 = g.flg_ele ? ip.ele_cut2_f : -1.f;
        // batches of B entries per lane: the B list words, then the B mirror
        // gathers, are all issued before any is used, so each lane keeps B
        // gathers in flight; the entries still add in list order, as in
        // pair_sum, so the split step equals the fused one bit for bit
        constexpr int B = 4;
        for (int k0 = lane; k0 < cnt; k0 += B * G) {
            int e[B];
#pragma unroll
            for (int u = 0; u < B; ++u) e[u] = k0 + u * G < cnt ? __ldg(nb + k0 + u * G) : 0;
            uint4 mj[B];
#pragma unroll
            for (int u = 0; u < B; ++u) mj[u] = k0 + u * G < cnt ? __ldg(mir + (e[u] & IDX_MASK)) : mi;
#pragma unroll
            for (int u = 0; u < B; ++u) {
                if (k0 + u * G >= cnt) break;
                const float vx = (float)(int)(mi.x - mj[u].x) * f0;
                const float vy = (float)(int)(mi.y - mj[u].y) * f1;
                const float vz = (float)(int)(mi.z - mj[u].z) * f2;
                const float d2 = fmaf(vx, vx, fmaf(vy, vy, vz * vz));
                float c = 0.f;
                if ((e[u] & WCA_BIT) && (mask & 16) && d2 < sig2) {
                    const float sq = __fdiv_rn(sig2, d2);
                    const float s2 = sq * sq, s4 = s2 * s2;
                    c += wcoef * (s4 * s2 * sq - s4);
                }
                if ((e[u] & ELE_BIT) && (mask & 32) && d2 <= cut2) {
                    float ri = rsqrtf(d2);
                    ri = ri * fmaf(-0.5f * d2 * ri, ri, 1.5f);
                    const float r = d2 * ri;
                    c += ecoef * ri * ri * (ri + rc) * __expf(-r * rc);
                }
                an.x = fmaf(c, vx, an.x);
                an.y = fmaf(c, vy, an.y);
                an.z = fmaf(c, vz, an.z);
            }
        }
    } else {
        const R sig2 = g.wca_sig2, wcoef = g.wca_coef;
        const R ecoef = ip.ele_coef, rc = ip.rcdist;
        const R cut2 = g.flg_ele ? ip.ele_cut2 : R(-1);
        const Pos<R> P = pos_of<R>(D, cur);
        for (int k = lane; k < cnt; k += G) {
            const int e = __ldg(nb + k);
            const V3<R> v = P.d(i, e & IDX_MASK, ip);
            const R c = pair_coef<R>(e, dot3(v, v), sig2, wcoef, ecoef, rc, cut2, mask);
            an = an + c * v;
        }
    }
    return an;
}

// The bonded forces on bead (bi) from the slot planes k_bonded wrote: the 9
// contributions (bond l-1|l, l|l+1; angles starting at l-2, l-1, l;
// dihedrals starting at l-3 .. l), lane `lane` of G taking every G-th
template <typename R>
__device__ __forceinline__ V3<R> bonded_gather_at(const typename Vec4<R>::type *S, size_t pl, int shift, const int4 &bi, int lane,
                                                 int G, int mask) {
    const int l = bi_lidx(bi);
    V3<R> ab = mk<R>(0, 0, 0);
    for (int t = lane; t < 9; t += G) {
        int start, k, cls;
        R sgn = R(1);
        if (t < 2) {
            cls = 1;
            start = l - 1 + t;
            k = 0;
            if (t == 1) sgn = R(-1);
        } else if (t < 5) {
            cls = 2;
            start = l - 2 + (t - 2);
            k = 1 + (2 - (t - 2));
        } else {
            cls = 4;
            start = l - 3 + (t - 5);
            k = 4 + (3 - (t - 5));
        }
        const int q = chain_bead(bi, start);
        if ((mask & cls) && q >= 0) ab = ab + sgn * v3(S[(size_t)k * pl + (q + shift)]);
    }
    return ab;
}
// the same from the context's slot planes (plane pitch n, bead index q)
template <typename R>
__device__ __forceinline__ V3<R> bonded_gather(const Dev &D, const GlobP &g, const int4 &bi, int lane, int G, int mask) {
    return bonded_gather_at<R>((const typename Vec4<R>::type *)D.slot, (size_t)g.n, 0, bi, lane, G, mask);
}

// Pair forces of every bead into fpair (float4 / double4), the step kernel's
// phase A run by itself, so that it can overlap the bonded and base-pair pass
template <typename R, int G> __global__ void __launch_bounds__(256, 5) k_pairs(Dev D, GlobP g, int cur) {
    constexpr int BPB = 256 / G;
    const int b = threadIdx.x / G, lane = threadIdx.x % G;
    const int i_raw = blockIdx.x * BPB + b;
    const int i = i_raw < g.n ? i_raw : g.n - 1;
    const InstP &ip = D.ip[D.binfo[i].x];
    V3<R> an = pair_sum_b<R, G>(D, g, cur, i, lane, ip, 48);
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1) {
        an.x += __shfl_xor_sync(0xffffffffu, an.x, o, G);
        an.y += __shfl_xor_sync(0xffffffffu, an.y, o, G);
        an.z += __shfl_xor_sync(0xffffffffu, an.z, o, G);
    }
    if (lane == 0 && i_raw < g.n) {
        using V4 = typename Vec4<R>::type;
        reinterpret_cast<V4 *>(D.fpair)[i] = Vec4<R>::make(an);
    }
}

// FP32 force coefficient c (F_i = c (x_i - x_j)) of one listed pair at
// squared distance d2: WCA (force_wca.F90:34-67) when the pair is on the WCA
// list and inside sigma, Debye-Hueckel (force_ele_DH.F90:39-82) when it is on
// the electrostatic list and inside the cutoff
struct PairCoef {
    float sig2, wcoef, ecoef, rc, rcl2, cut2; // rcl2: rc log2(e)
};
__device__ __forceinline__ PairCoef pair_coef_of(const GlobP &g, const InstP &ip) {
    PairCoef P;
    P.sig2 = g.f_wca_sig2;
    P.wcoef = g.f_wca_coef;
    P.ecoef = ip.ele_coef_f;
    P.rc = ip.rcdist_f;
    P.rcl2 = ip.rcdist_f * 1.44269504f;
    P.cut2 = g.flg_ele ? ip.ele_cut2_f : -1.f;
    return P;
}
__device__ __forceinline__ float2 rcp_nr2(float2 d2) {
    float2 r0;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r0.x) : "f"(d2.x));
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r0.y) : "f"(d2.y));
    return __ffma2_rn(r0, __ffma2_rn(make_float2(-d2.x, -d2.y), r0, make_float2(1.f, 1.f)), r0);
}
// 2^t by the hardware approximation (exp(-r rc) = 2^(-r rc log2 e))
__device__ __forceinline__ float ex2a(float t) {
    float y;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(t));
    return y;
}
// WCA (force_wca.F90): wcoef ((s/d)^14 - (s/d)^8) with (s/d)^2 = sig2 / d2
__device__ __forceinline__ float wca_c(float d2, const PairCoef &P) {
    const float sq = __fmul_rn(P.sig2, rcp_nr(d2));
    const float s2 = __fmul_rn(sq, sq), s4 = __fmul_rn(s2, s2);
    return __fmul_rn(P.wcoef, __fmaf_rn(__fmul_rn(s4, s2), sq, -s4));
}
__device__ __forceinline__ float2 wca_c2(float2 d2, const PairCoef &P) {
    const float2 sq = __fmul2_rn(make_float2(P.sig2, P.sig2), rcp_nr2(d2));
    const float2 s2 = __fmul2_rn(sq, sq), s4 = __fmul2_rn(s2, s2);
    return __fmul2_rn(make_float2(P.wcoef, P.wcoef), __ffma2_rn(__fmul2_rn(s4, s2), sq, make_float2(-s4.x, -s4.y)));
}
// Debye-Hueckel (force_ele_DH.F90): ecoef ri^2 (ri + rc) exp(-r rc), ri the
// hardware reciprocal square root (relative error below 2^-22), the
// exponential as 2^(-r rc log2 e).  Each term is
// selected by its list bit and distance (pair2: the electrostatic term is
// formed for every pair, the WCA term only when some lane of the warp has a
// pair inside sigma, a warp-uniform branch).
__device__ __forceinline__ float pair_c(bool wca, bool ele, float d2, const PairCoef &P) {
    const float ri = rsqrtf(d2);
    const float rr = __fmul_rn(d2, ri);
    const float ce = __fmul_rn(__fmul_rn(__fmul_rn(P.ecoef, __fmul_rn(ri, ri)), __fadd_rn(ri, P.rc)), ex2a(-rr * P.rcl2));
    const float e = (ele && d2 <= P.cut2) ? ce : 0.f;
    return (wca && d2 < P.sig2) ? __fadd_rn(wca_c(d2, P), e) : e;
}

// Two pairs at once with paired FP32 instructions (FFMA2 and relatives of
// sm_100 and later): the separations v of (i, j) and (i, j') from the mirror
// differences, and the force coefficients c of pair_c, lane by lane the same
// IEEE operations as pair_c.  Called by all 32 lanes of a warp.
struct Pair2 {
    float2 vx, vy, vz, c;
};
__device__ __forceinline__ Pair2 pair2(const uint4 &mi, const uint4 &ma, const uint4 &mb, const float2 f0, const float2 f1,
                                       const float2 f2, bool wa, bool wb, bool ea, bool eb, const PairCoef &P) {
    Pair2 r;
    r.vx = __fmul2_rn(make_float2((float)(int)(mi.x - ma.x), (float)(int)(mi.x - mb.x)), f0);
    r.vy = __fmul2_rn(make_float2((float)(int)(mi.y - ma.y), (float)(int)(mi.y - mb.y)), f1);
    r.vz = __fmul2_rn(make_float2((float)(int)(mi.z - ma.z), (float)(int)(mi.z - mb.z)), f2);
    const float2 d2 = __ffma2_rn(r.vx, r.vx, __ffma2_rn(r.vy, r.vy, __fmul2_rn(r.vz, r.vz)));
    const float2 ri = make_float2(rsqrtf(d2.x), rsqrtf(d2.y));
    const float2 t = __fmul2_rn(__fmul2_rn(d2, ri), make_float2(-P.rcl2, -P.rcl2));
    const float2 ex = make_float2(ex2a(t.x), ex2a(t.y));
    const float2 ce = __fmul2_rn(__fmul2_rn(__fmul2_rn(make_float2(P.ecoef, P.ecoef), __fmul2_rn(ri, ri)),
                                            __fadd2_rn(ri, make_float2(P.rc, P.rc))),
                                 ex);
    r.c.x = (ea && d2.x <= P.cut2) ? ce.x : 0.f;
    r.c.y = (eb && d2.y <= P.cut2) ? ce.y : 0.f;
    const bool w0 = wa && d2.x < P.sig2, w1 = wb && d2.y < P.sig2;
    if (__any_sync(0xffffffffu, w0 || w1)) {
        const float2 cw = wca_c2(d2, P);
        const float2 cs = __fadd2_rn(cw, r.c);
        r.c.x = w0 ? cs.x : r.c.x;
        r.c.y = w1 ? cs.y : r.c.y;
    }
    return r;
}

// 16-byte asynchronous copy global -> shared (cp.async, L1-allocating) and
// the wait for all of a thread's copies
__device__ __forceinline__ void cp_async16(void *smem, const void *gmem) {
    const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

// Pair forces of the mixed path over the cluster-pair lists (lists.cu
// cluster_lists) into fpair: one warp per i-cluster of 8 beads.  The warp
// stages the j-clusters of its list, up to kClChunk at a time, in shared
// memory: lane k loads the k-th cluster record (first bead, WCA and
// electrostatic masks), then the 8 lanes of each group copy the 8 mirrors of
// every 4th cluster (128 contiguous bytes) with cp.async, so the whole
// chunk's mirrors are in flight at once.  Lane (a = lane & 7, q = lane >> 3)
// then takes i-bead a against all 8 j-beads of every 4th j-cluster of the
// list, starting at the q-th, two pairs at a time (pair2).  Sums: even and
// odd partners apart, then added, in list order per lane, then over q (xor
// 8, then 16): a fixed order, and a partner beyond every cutoff adds an
// exact zero.  mask bit 16: WCA, bit 32: electrostatics.  An i-cluster whose
// j-clusters did not fit (count -1) walks its beads' per-bead lists, 4 lanes
// per bead.
constexpr int kClChunk = 32;
__global__ void __launch_bounds__(256, 5) k_pairs_cl(Dev D, GlobP g, int cur, int mask) {
    __shared__ __align__(16) uint4 s_mj[8][kClChunk * kCl];
    __shared__ ulonglong2 s_cm[8][kClChunk];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int ic = blockIdx.x * 8 + w;
    if (ic >= g.n_cl) return;
    const int a = lane & 7, q = lane >> 3;
    const int first = D.cl_first[ic];
    const InstP &ip = D.ip[D.binfo[first].x];
    const int cnt = min(kCl, ip.bead_off + ip.n - first);
    const uint4 *__restrict__ mir = mir_at(D, cur);
    const uint4 mi = mir[first + (a < cnt ? a : 0)];
    const float2 f0 = make_float2(ip.finv[0], ip.finv[0]), f1 = make_float2(ip.finv[1], ip.finv[1]),
                 f2 = make_float2(ip.finv[2], ip.finv[2]);
    const PairCoef P = pair_coef_of(g, ip);
    const unsigned wsel = (mask & 16) ? 0xffu : 0u, esel = (mask & 32) ? 0xffu : 0u;
    float2 ax = make_float2(0.f, 0.f), ay = ax, az = ax;
    const int nc = D.ncl[ic];
    if (nc >= 0) {
        const size_t base = (size_t)ic * g.ccap;
        for (int c0 = 0; c0 < nc; c0 += kClChunk) {
            const int nk = min(kClChunk, nc - c0);
            int j0 = 0;
            if (lane < nk) {
                j0 = __ldg(D.cl_j + base + c0 + lane);
                s_cm[w][lane] = __ldg(D.cl_m + base + c0 + lane);
            }
            for (int t = 0; 4 * t < nk; ++t) {
                const int k = q + 4 * t;
                const int jk = __shfl_sync(0xffffffffu, j0, k & 31);
                if (k < nk) cp_async16(&s_mj[w][k * kCl + a], mir + jk + a);
            }
            cp_async_wait_all();
            __syncwarp();
            for (int k0 = 0; k0 < nk; k0 += 4) {
                // every lane runs every round; a lane past the chunk's end
                // takes cluster 0 with empty masks (exact zeros)
                const int k = k0 + q < nk ? k0 + q : 0;
                const ulonglong2 m = k0 + q < nk ? s_cm[w][k] : make_ulonglong2(0ull, 0ull);
                const unsigned wb = (unsigned)(m.x >> (a * kCl)) & wsel, eb = (unsigned)(m.y >> (a * kCl)) & esel;
                const uint4 *mj = s_mj[w] + k * kCl;
#pragma unroll
                for (int b = 0; b < kCl; b += 2) {
                    const Pair2 pr = pair2(mi, mj[b], mj[b + 1], f0, f1, f2, (wb >> b) & 1u, (wb >> (b + 1)) & 1u, (eb >> b) & 1u,
                                           (eb >> (b + 1)) & 1u, P);
                    ax = __ffma2_rn(pr.c, pr.vx, ax);
                    ay = __ffma2_rn(pr.c, pr.vy, ay);
                    az = __ffma2_rn(pr.c, pr.vz, az);
                }
            }
            __syncwarp();
        }
    } else if (a < cnt) {
        const int gi = first + a;
        const int m = min(D.nnbr[gi], g.cap);
        const int *__restrict__ nb = D.nbr + (size_t)gi * g.cap;
        for (int k = q; k < m; k += 4) {
            const int e = __ldg(nb + k);
            const uint4 mj = __ldg(mir + (e & IDX_MASK));
            const float vx = (float)(int)(mi.x - mj.x) * ip.finv[0];
            const float vy = (float)(int)(mi.y - mj.y) * ip.finv[1];
            const float vz = (float)(int)(mi.z - mj.z) * ip.finv[2];
            const float d2 = fmaf(vx, vx, fmaf(vy, vy, vz * vz));
            const float c = pair_c((e & WCA_BIT) && (mask & 16), (e & ELE_BIT) && (mask & 32), d2, P);
            ax.x = fmaf(c, vx, ax.x);
            ay.x = fmaf(c, vy, ay.x);
            az.x = fmaf(c, vz, az.x);
        }
    }
    float sx = ax.x + ax.y, sy = ay.x + ay.y, sz = az.x + az.y;
#pragma unroll
    for (int o = 8; o <= 16; o <<= 1) {
        sx += __shfl_xor_sync(0xffffffffu, sx, o);
        sy += __shfl_xor_sync(0xffffffffu, sy, o);
        sz += __shfl_xor_sync(0xffffffffu, sz, o);
    }
    if (q == 0 && a < cnt) reinterpret_cast<float4 *>(D.fpair)[first + a] = make_float4(sx, sy, sz, 0.f);
}

// The end of a step kernel: each block merges its per-instance top two
// squared displacements (s_m1/s_m2 for instances s_lo .. s_lo + s_cnt - 1,
// when s_cnt <= 32; otherwise its threads merged them already) into m1/m2 of
// the step's parity (mo).  With decide, the last block to finish decides the
// trigger (job_md.F90:376-395) once every block's top two are merged: it
// flags the instances that fired (clearing their base-pair staging counts)
// for the rebuild kernel that follows, schedules the Monte Carlo pass
// (job_md.F90:364-367), clears m1/m2 of the other parity for the next step
// and advances the Philox step counter (every block read it before).  Called
// by every thread of the block after a barrier.
__device__ __forceinline__ void trigger_merge_decide(const Dev &D, const GlobP &g, const unsigned long long *s_m1,
                                                     const unsigned long long *s_m2, int s_lo, int s_cnt, size_t mo,
                                                     unsigned long long step, bool decide) {
    if (s_cnt <= 32 && (int)threadIdx.x < s_cnt) {
        const unsigned long long b1 = s_m1[threadIdx.x], b2 = s_m2[threadIdx.x];
        const int inst = s_lo + threadIdx.x;
        const unsigned long long old = atomicMax(&D.m1[mo + inst], b1);
        const unsigned long long c2 = old < b1 ? old : b1;
        atomicMax(&D.m2[mo + inst], c2 > b2 ? c2 : b2);
    }
    if (!decide) return;
    __shared__ int s_last;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) s_last = atomicAdd(&D.ticket[0], 1u) == gridDim.x - 1;
    __syncthreads();
    if (!s_last) return;
    __threadfence();
    const unsigned long long *m1 = D.m1 + mo, *m2 = D.m2 + mo;
    unsigned long long *o1 = D.m1 + (mo ? 0 : g.n_inst), *o2 = D.m2 + (mo ? 0 : g.n_inst);
    const bool mc = g.nstep_mc > 0 && (step + 2ull) % (unsigned long long)g.nstep_mc == 0ull;
    int fired = 0;
    for (int k = threadIdx.x; k < g.n_inst; k += blockDim.x) {
        if (trigger_fires(g, m1, m2, k)) {
            D.flag[k] = 1;
            D.bp_cnt[k] = 0;
            fired = 1;
        }
        o1[k] = 0ull;
        o2[k] = 0ull;
        if (mc) D.mc_due[k] = 1;
    }
    fired = __syncthreads_or(fired);
    if (threadIdx.x == 0) {
        if (fired) *D.any = 1;
        *D.step_ctr = step + 1ull;
        D.ticket[0] = 0u;
    }
}

// The mixed path's GJF-2GJ / Ermak-McCammon update of bead ii
// (job_md.F90:415-456) from its loaded state (x, v, beta, coefficients m):
// the force F and the noise xi enter as FP32 increments (cf0, cf1: the force
// and noise coefficients of m in FP32), the velocity and the position
// accumulate in FP64.  Writes the new position, velocity, noise term, mirror
// and residual (buffer cur ^ 1); returns the new mirror (w unused) and, if
// asked, the residual.
__device__ __forceinline__ uint4 mixed_update_core(const Dev &D, const GlobP &g, int cur, int ii, const InstP &jp, const float F[3],
                                                   float cf0, float cf1, const float xi[3], const double4 &x, const double4 &m,
                                                   const double4 &v, const double4 &b, float4 *res_out) {
    double xc[3] = {x.x, x.y, x.z}, vc[3] = {v.x, v.y, v.z}, bc[3] = {b.x, b.y, b.z};
    unsigned int q[3];
    float r[3];
    bool ok = true;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        if (g.integrator == 1) {
            const float bn = cf1 * xi[c];
            const double vn = fma(m.x, vc[c], bc[c]) + (double)fmaf(cf0, F[c], bn);
            bc[c] = (double)bn;
            vc[c] = vn;
            xc[c] = fma(m.z, vn, xc[c]); // x + sqrt(b) h v, one rounding
        } else {
            xc[c] = xc[c] + (double)fmaf(cf0, F[c], cf1 * xi[c]);
        }
        ok &= fixed_mirror(xc[c], jp.fsc[c], q[c], r[c]);
    }
    if (!ok) atomicOr(D.err, ERR_NONFINITE);
    x_at(D, cur ^ 1)[ii] = make_double4(xc[0], xc[1], xc[2], 0.0);
    if (g.integrator == 1) {
        D.v[ii] = make_double4(vc[0], vc[1], vc[2], v.w);
        D.beta[ii] = make_double4(bc[0], bc[1], bc[2], b.w);
    }
    const uint4 mq = make_uint4(q[0], q[1], q[2], 0u);
    const float4 rq = make_float4(r[0], r[1], r[2], 0.f);
    mir_at(D, cur ^ 1)[ii] = mq;
    res_at(D, cur ^ 1)[ii] = rq;
    if (res_out) *res_out = rq;
    return mq;
}
// the noise of bead ii at a step: fed (FP64, rounded to FP32) or Philox
__device__ __forceinline__ void mixed_noise(const GlobP &g, int ii, const InstP &jp, const double *noise, long long noise_step,
                                            unsigned long long step, float xi[3]) {
    if (noise) {
        const double *nz = noise + ((size_t)noise_step * g.n + ii) * 3;
        xi[0] = (float)nz[0];
        xi[1] = (float)nz[1];
        xi[2] = (float)nz[2];
    } else {
        gauss_f3(g.seed, ii - jp.bead_off, step - jp.step0, jp.stream, xi);
    }
}
// The mixed path's step, one thread per bead, after k_pairs_cl: every load
// of the bead's step (pair force, bonded slot planes, base-pair sum, FP64
// state, coefficients, the mirror at the last rebuild) issues before any is
// used; then the force sum (pair + bonded in slot order + base pair), the
// cap, the update (mixed_update_core) and the squared displacement since
// the last rebuild into its instance's top two; the block's top two are
// merged and the last block decides the trigger (mask bit 256).
__global__ void __launch_bounds__(256) k_step_mixed(Dev D, GlobP g, int cur, const double *__restrict__ noise, long long noise_step,
                                                    int mask) {
    __shared__ unsigned long long s_m1[32], s_m2[32];
    __shared__ int s_lo, s_cnt;
    const int i0 = blockIdx.x * blockDim.x;
    const int ii = i0 + threadIdx.x;
    const bool active = ii < g.n;
    const int i = active ? ii : g.n - 1;
    if (threadIdx.x < 32) {
        s_m1[threadIdx.x] = 0ull;
        s_m2[threadIdx.x] = 0ull;
    }
    if (threadIdx.x == 0) {
        const int i1 = min(i0 + (int)blockDim.x - 1, g.n - 1);
        s_lo = D.binfo[i0].x;
        s_cnt = D.binfo[i1].x - s_lo + 1;
    }
    const int4 bi = D.binfo[i];
    const InstP &jp = D.ip[bi.x];
    const float4 fp = reinterpret_cast<const float4 *>(D.fpair)[i];
    const double4 fb = D.fbp[i];
    const double4 x = x_at(D, cur)[i], m = D.mdc[i], v = D.v[i], b = D.beta[i];
    const uint4 m0 = D.mir0[i];
    const unsigned long long step = *D.step_ctr;
    const float4 fbd = D.fbond[i];
    const V3<float> ab = (mask & 7) ? mk<float>(fbd.x, fbd.y, fbd.z) : mk<float>(0.f, 0.f, 0.f);
    float xi[3];
    mixed_noise(g, i, jp, noise, noise_step, step, xi);
    float F[3] = {fp.x + ab.x, fp.y + ab.y, fp.z + ab.z};
    if (mask & 136) {
        F[0] += fx_float(fb.x);
        F[1] += fx_float(fb.y);
        F[2] += fx_float(fb.z);
        if (active) D.fbp[i] = make_double4(0.0, 0.0, 0.0, 0.0);
    }
    if (g.fcap_f > 0.f) {
        const float fm = sqrtf(F[0] * F[0] + F[1] * F[1] + F[2] * F[2]);
        if (fm > g.fcap_f) {
            const float sc = g.fcap_f / fm;
            F[0] *= sc;
            F[1] *= sc;
            F[2] *= sc;
            if (active) atomicAdd(D.capped, 1ull);
        }
    }
    // GJF-2GJ: F -> sqrt(b) h / m, noise -> its amplitude; Ermak-McCammon: F -> h / gamma
    const float cf0 = (float)(g.integrator == 1 ? m.y : m.x), cf1 = (float)m.w;
    uint4 q = m0;
    if (active) q = mixed_update_core(D, g, cur, i, jp, F, cf0, cf1, xi, x, m, v, b, nullptr);
    // the exact integer displacement since the last rebuild
    const float dx = (float)(int)(q.x - m0.x) * jp.finv[0];
    const float dy = (float)(int)(q.y - m0.y) * jp.finv[1];
    const float dz = (float)(int)(q.z - m0.z) * jp.finv[2];
    const unsigned long long bits = (unsigned long long)__double_as_longlong((double)fmaf(dx, dx, fmaf(dy, dy, dz * dz)));
    const size_t mo = (size_t)(step & 1ull) * g.n_inst;
    __syncthreads();
    if (active) {
        if (s_cnt <= 32) {
            const int k = bi.x - s_lo;
            const unsigned long long old = atomicMax(&s_m1[k], bits);
            atomicMax(&s_m2[k], old < bits ? old : bits);
        } else {
            const unsigned long long old = atomicMax(&D.m1[mo + bi.x], bits);
            atomicMax(&D.m2[mo + bi.x], old < bits ? old : bits);
        }
    }
    __syncthreads();
    trigger_merge_decide(D, g, s_m1, s_m2, s_lo, s_cnt, mo, step, mask & 256);
}

template <typename R, int G, int MODE>
__global__ void __launch_bounds__(256, 5) k_step(Dev D, GlobP g, int cur, const double *__restrict__ noise, long long noise_step,
                                              double *__restrict__ fout, int mask) {
    constexpr int BPB = 256 / G;
    __shared__ R sA[3][BPB], sB[3][BPB];
    __shared__ float sScale[BPB];
    __shared__ double sM[3][BPB];
    __shared__ unsigned long long s_m1[32], s_m2[32];
    __shared__ int s_lo, s_cnt;
    const int b = threadIdx.x / G;
    const int lane = threadIdx.x % G;
    const int i0 = blockIdx.x * BPB;
    const int i_raw = i0 + b;
    const bool active = i_raw < g.n;
    const int i = active ? i_raw : g.n - 1;
    if (MODE == 0) {
        if (threadIdx.x < 32) {
            s_m1[threadIdx.x] = 0ull;
            s_m2[threadIdx.x] = 0ull;
        }
        if (threadIdx.x == 0) {
            const int i1 = min(i0 + BPB - 1, g.n - 1);
            s_lo = D.binfo[i0].x;
            s_cnt = D.binfo[i1].x - s_lo + 1;
        }
    }
    const int4 bi = D.binfo[i];
    const InstP &ip = D.ip[bi.x];

    // -------------------------------------------------------------- phase A
    // (mask bit 64: the pair forces were computed by k_pairs)
    V3<R> an = mk<R>(0, 0, 0);
    if (mask & 64) {
        if (lane == 0) {
            using V4 = typename Vec4<R>::type;
            an = v3(reinterpret_cast<const V4 *>(D.fpair)[i]);
        }
    } else if (mask & 48) {
        an = pair_sum<R, G>(D, g, cur, i, lane, ip, mask);
    }
    // bonded: gather of slot forces, 9 contributions spread over the lanes
    V3<R> ab = (mask & 7) ? bonded_gather<R>(D, g, bi, lane, G, mask) : mk<R>(0, 0, 0);
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1) {
        an.x += __shfl_xor_sync(0xffffffffu, an.x, o, G);
        an.y += __shfl_xor_sync(0xffffffffu, an.y, o, G);
        an.z += __shfl_xor_sync(0xffffffffu, an.z, o, G);
        ab.x += __shfl_xor_sync(0xffffffffu, ab.x, o, G);
        ab.y += __shfl_xor_sync(0xffffffffu, ab.y, o, G);
        ab.z += __shfl_xor_sync(0xffffffffu, ab.z, o, G);
    }
    if (lane == 0) {
        sA[0][b] = an.x;
        sA[1][b] = an.y;
        sA[2][b] = an.z;
        sB[0][b] = ab.x;
        sB[1][b] = ab.y;
        sB[2][b] = ab.z;
        float sc = 1.f;
        if (MODE == 0 && g.fcap > 0.0) {
            const double4 fb = D.fbp[i];
            const float bx = sizeof(R) == 4 ? (float)fx_value(fb.x) : (float)fb.x;
            const float by = sizeof(R) == 4 ? (float)fx_value(fb.y) : (float)fb.y;
            const float bz = sizeof(R) == 4 ? (float)fx_value(fb.z) : (float)fb.z;
            const float fx = (float)(an.x + ab.x) + bx, fy = (float)(an.y + ab.y) + by, fz = (float)(an.z + ab.z) + bz;
            const float fm = sqrtf(fx * fx + fy * fy + fz * fz);
            if (fm > (float)g.fcap) {
                sc = (float)g.fcap / fm;
                if (active) atomicAdd(D.capped, 1ull);
            }
        }
        sScale[b] = sc;
    }
    __syncthreads();

    // -------------------------------------------------------------- phase B
    // One thread per (component, bead): the components of the GJF-2GJ /
    // Ermak-McCammon update are independent, and FP64 runs at a small
    // fraction of the FP32 rate on this part, so the block spreads it over
    // 3*BPB threads (whole warps) instead of BPB.
    const unsigned long long step = MODE == 0 ? *D.step_ctr : 0ull;
    for (int t = threadIdx.x; t < 3 * BPB; t += blockDim.x) {
        const int c = t / BPB, bb = t - c * BPB;
        const int ii = i0 + bb;
        if (ii >= g.n) continue;
        double *fp = reinterpret_cast<double *>(D.fbp + ii) + c;
        if constexpr (sizeof(R) == 4) {
            // mixed path, forces only (its step is k_step_mixed): the FP32
            // sums plus the fixed-point base-pair force
            float fb = 0.f;
            if (mask & 136) {
                fb = fx_float(*fp);
                *fp = 0.0;
            }
            fout[3 * (size_t)ii + c] = (double)(sA[c][bb] + sB[c][bb] + fb);
            continue;
        } else {
            double Fc;
            double fb = 0.0;
            if (mask & 136) {
                fb = *fp;
                *fp = 0.0;
            }
            Fc = sA[c][bb] + sB[c][bb] + fb;
            if (MODE == 1) {
                fout[3 * (size_t)ii + c] = Fc;
                continue;
            }
            if (sScale[bb] != 1.f) Fc = Fc * (double)sScale[bb];
            const int4 bj = D.binfo[ii];
            const InstP &jp = D.ip[bj.x];
            const double4 m = D.mdc[ii];
            const double xi = noise ? noise[((size_t)noise_step * g.n + ii) * 3 + c]
                                    : gauss3<R>(g.seed, ii - jp.bead_off, step - jp.step0, c, jp.stream);
            double *vp = reinterpret_cast<double *>(D.v + ii) + c;
            double *bp = reinterpret_cast<double *>(D.beta + ii) + c;
            double *mp = reinterpret_cast<double *>(D.move + ii) + c;
            double dx;
            if (g.integrator == 1) {
                const double bn = m.w * xi;
                const double vn = m.x * *vp + m.y * Fc + (*bp + bn);
                *bp = bn;
                *vp = vn;
                dx = m.z * vn;
            } else {
                dx = m.x * Fc + m.w * xi;
            }
            const double xn = reinterpret_cast<const double *>(x_at(D, cur) + ii)[c] + dx;
            if (!isfinite(xn)) atomicOr(D.err, ERR_NONFINITE);
            const double mc = *mp + dx;
            *mp = mc;
            sM[c][bb] = mc;
            reinterpret_cast<double *>(x_at(D, cur ^ 1) + ii)[c] = xn;
            float r;
            reinterpret_cast<unsigned int *>(mir_at(D, cur ^ 1) + ii)[c] = fixed_res(xn, jp.fsc[c], r);
            reinterpret_cast<float *>(res_at(D, cur ^ 1) + ii)[c] = r;
        }
    }
    if (MODE == 1) return;
    __syncthreads();

    // -------------------------------------------------------------- phase C
    // displacement^2 per bead and its top two per instance (shared memory),
    // merged into m1/m2 of this step's parity (global atomics)
    const size_t mo = (size_t)(step & 1ull) * g.n_inst;
    for (int bb = threadIdx.x; bb < BPB; bb += blockDim.x) {
        const int ii = i0 + bb;
        if (ii >= g.n) continue;
        const double mx = sM[0][bb], my = sM[1][bb], mz = sM[2][bb];
        const double d2 = __dadd_rn(__dadd_rn(__dmul_rn(mx, mx), __dmul_rn(my, my)), __dmul_rn(mz, mz));
        if (!isfinite(d2)) atomicOr(D.err, ERR_NONFINITE);
        const unsigned long long bits = (unsigned long long)__double_as_longlong(d2);
        const int inst = D.binfo[ii].x;
        if (s_cnt <= 32) {
            const int k = inst - s_lo;
            const unsigned long long old = atomicMax(&s_m1[k], bits);
            atomicMax(&s_m2[k], old < bits ? old : bits);
        } else {
            const unsigned long long old = atomicMax(&D.m1[mo + inst], bits);
            atomicMax(&D.m2[mo + inst], old < bits ? old : bits);
        }
    }
    __syncthreads();
    trigger_merge_decide(D, g, s_m1, s_m2, s_lo, s_cnt, mo, step, mask & 256);
}

// ======================================================== small instances
// k_md_small: nsteps MD steps of the mixed path in one launch, for contexts
// whose instances are all small (all-pairs lists, at most kSmallMaxBeads
// beads).  Each block owns a bucket of whole instances (SmallPlan), keeps
// their position mirrors, residuals, base-pair force sums and step forces in
// shared memory, and runs every phase of every step for them with block
// barriers only: base-pair terms (one thread per record), bonded terms (one
// thread per term start), pair forces over the per-bead lists (kSmallLanes
// lanes per bead, partners' mirrors gathered from shared memory), the update
// (one thread per bead), the displacement trigger of each instance and,
// for the instances whose trigger fired, their all-pairs list rebuild (one
// warp per bead).  Blocks never wait on one another.  The per-bead
// arithmetic does not depend on how instances are bucketed or how many
// threads a block has, so every plan gives the same trajectory bit for bit.
// The FP64 state (x, v, beta), the lists and the base-pair records stay in
// global memory, current after every step, for the other entry points.
// Lane l of a bead takes the entries l, l + 8, l + 16, ... of its list; the
// lane sums are reduced over the 8 lanes in a fixed order.
constexpr int kSmallLanes = 8;
// The pair forces of the per-block kernel walk inner lists: the entries of
// the bead's list (whose radius is the cutoff + the list margin) within
// their own cutoff (electrostatic, WCA) + kInnerMargin A.  An instance's
// inner lists are filtered again from its lists when the two largest bead
// displacements since their last filtering sum to more than kInnerMargin
// (no pair can then have come within a cutoff without being listed), when
// its lists were rebuilt, and at the start of a launch whose state moved
// since.  Entries beyond every cutoff add exact zeros, so the inner lists
// leave the forces' terms unchanged.  Instances of fewer than
// kInnerMinBeads moving beads, whose lists hold few such entries, walk
// their lists directly; a context with no instance of that capacity runs
// the kernel without the inner lists (INNER false).
constexpr float kInnerMargin = 2.5f;

// the context as seen by one instance of a bucket: its beads' mirrors,
// residuals and base-pair force sums at their shared-memory slots, addressed
// by global bead index (sb: the instance's first slot, off: its first bead)
// (both buffers name the shared copy: the block keeps one mirror); with
// ipc, the instance record as the shared copy ipc, addressed by the
// instance's global index id, and the base-pair parameters as bpf
__device__ __forceinline__ Dev small_view(const Dev &D, uint4 *s_mir, float4 *s_res, double4 *s_fbp, int sb, int off,
                                          const InstP *ipc, int id, const BPPf *bpf) {
    Dev E = D;
    E.mir[0] = E.mir[1] = s_mir + (sb - off);
    E.res[0] = E.res[1] = s_res + (sb - off);
    E.fbp = s_fbp + (sb - off);
    if (ipc) E.ip = ipc - id;
    E.bppf = bpf;
    return E;
}
// instance records a block keeps in shared memory (blocks of more instances
// read them from global memory)
constexpr int kSmallIpCache = 8;

// bucket-local instance of slot s (s_sb: the instances' first slots, ascending)
__device__ __forceinline__ int small_inst(const int *s_sb, int ni, int s) {
    int lo = 0, hi = ni - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (s_sb[mid] <= s) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// MAXT: the block width bound (512: 128 registers a thread; 384: 168, and a
// third of the register spills, for blocks of up to 384 threads)
template <bool INNER, int MAXT>
__global__ void __launch_bounds__(MAXT) k_md_small(Dev D, GlobP g, int cur, SmallPlan sp, int nsteps, const double *noise) {
    extern __shared__ __align__(16) unsigned char s_dyn[];
    const int cap = sp.cap;
    uint4 *s_mir = (uint4 *)s_dyn;
    float4 *s_res = (float4 *)(s_mir + cap);
    double4 *s_fbp = (double4 *)(s_res + cap);
    float4 *s_F = (float4 *)(s_fbp + cap);   // pair force of the step (xyz)
    double2 *s_cd = (double2 *)(s_F + cap);  // integrator coefficients a, sqrt(b) h (mdc.x, mdc.z)
    // with sp.sslot, the bonded terms' slot planes (8 planes of cap, by the
    // slot of the term's first bead); else the context's slot planes
    const bool sslot = sp.sslot != 0;
    float4 *s_slot = (float4 *)(s_cd + cap);
    float2 *s_cf = (float2 *)(s_slot + (sslot ? 8 * cap : 0)); // FP32 force and noise coefficients of the update
    __shared__ int s_iid[kSmallMaxInst], s_off[kSmallMaxInst], s_n[kSmallMaxInst], s_bpo[kSmallMaxInst];
    __shared__ int s_sb[kSmallMaxInst + 1], s_bp[kSmallMaxInst + 1];
    __shared__ unsigned int s_m1[kSmallMaxInst], s_m2[kSmallMaxInst];
    __shared__ unsigned int s_m3[kSmallMaxInst], s_m4[kSmallMaxInst]; // the same since the inner lists' filtering
    __shared__ int s_fire[kSmallMaxInst], s_ifire[kSmallMaxInst];
    __shared__ int s_any, s_anyi;
    // the next base-pair record chunk and the next pair-force group of the
    // step: warps take them as they become free (a bead's and a record's
    // arithmetic does not depend on the warp that runs it)
    __shared__ int s_rnext, s_pnext;
    __shared__ int2 s_qi[16 * 64]; // per warp: queued base-pair records (2 warp widths)
    __shared__ InstP s_ipc[kSmallIpCache];
    __shared__ BPPf s_bpf[MAX_BP_TYPES];
    const int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, warp = tid >> 5, nwarps = nt >> 5;
    const int k0 = sp.cta_off[blockIdx.x], ni = sp.cta_off[blockIdx.x + 1] - k0;
    if (tid == 0) {
        int sb = 0, nbp = 0;
        for (int q = 0; q < ni; ++q) {
            const int id = sp.inst[k0 + q];
            const InstP &ip = D.ip[id];
            s_iid[q] = id;
            s_off[q] = ip.bead_off;
            s_n[q] = ip.n_act;
            s_bpo[q] = ip.bp_off;
            s_sb[q] = sb;
            s_bp[q] = nbp;
            sb += ip.n_act;
            nbp += min(D.bp_cnt[id], ip.bp_cap);
        }
        s_sb[ni] = sb;
        s_bp[ni] = nbp;
        s_any = s_anyi = 0;
        s_rnext = s_pnext = 0;
    }
    if (tid < ni) s_m1[tid] = s_m2[tid] = s_m3[tid] = s_m4[tid] = 0u;
    __syncthreads();
    const int nb = s_sb[ni];
    // the instance records (when they fit) and the base-pair parameters, as
    // 32-bit words; the view of instance q is view(q)
    const bool ipc_on = ni <= kSmallIpCache;
    if (ipc_on) {
        constexpr int w = (int)(sizeof(InstP) / 4);
        for (int t = tid; t < ni * w; t += nt)
            ((int *)s_ipc)[t] = ((const int *)(D.ip + s_iid[t / w]))[t % w];
    }
    for (int t = tid; t < MAX_BP_TYPES * (int)(sizeof(BPPf) / 4); t += nt) ((int *)s_bpf)[t] = ((const int *)D.bppf)[t];
    auto view = [&](int q) {
        return small_view(D, s_mir, s_res, s_fbp, s_sb[q], s_off[q], ipc_on ? s_ipc + q : nullptr, s_iid[q], s_bpf);
    };
    for (int s = tid; s < nb; s += nt) {
        const int q = small_inst(s_sb, ni, s);
        const int gi = s_off[q] + (s - s_sb[q]);
        s_mir[s] = mir_at(D, cur)[gi];
        s_res[s] = res_at(D, cur)[gi];
        s_fbp[s] = make_double4(0.0, 0.0, 0.0, 0.0);
        // GJF-2GJ: F -> sqrt(b) h / m, noise -> its amplitude; Ermak-McCammon: F -> h / gamma
        const double4 mc = D.mdc[gi];
        s_cd[s] = make_double2(mc.x, mc.z);
        s_cf[s] = make_float2((float)(g.integrator == 1 ? mc.y : mc.x), (float)mc.w);
        // displacement since the inner lists' filtering (state moved between launches)
        if (!INNER || s_n[q] < kInnerMinBeads) continue;
        const uint4 mI = D.mir_in[gi], m = s_mir[s];
        const float *fi = D.ip[s_iid[q]].finv; // (s_ipc is being filled)
        const float dx = (float)(int)(m.x - mI.x) * fi[0], dy = (float)(int)(m.y - mI.y) * fi[1],
                    dz = (float)(int)(m.z - mI.z) * fi[2];
        const unsigned int bits = __float_as_uint(fmaf(dx, dx, fmaf(dy, dy, dz * dz)));
        const unsigned int old = atomicMax(&s_m3[q], bits);
        atomicMax(&s_m4[q], old < bits ? old : bits);
    }
    __syncthreads();
    // the rebuild of the instances with s_fire set (neighbor_list.F90), from
    // the mirrors of buffer c, over their moving beads (a slot's fillers take
    // part in no term: with all_beads, their lists are emptied too); ends
    // with s_any cleared
    auto rebuild = [&](int c, bool all_beads) {
        const int cur = c;
        for (int q = 0; q < ni; ++q) {
            if (!s_fire[q]) continue;
            const int id = s_iid[q], off = s_off[q], na = s_n[q];
            const InstP &ip = D.ip[id];
            const Dev E = view(q);
            const float maxcut2f = scan_cut2f(ip, 1.001f);
            for (int li = warp; li < na; li += nwarps) {
                const int gi = off + li;
                double4 xi_w;
                bead_begin(E, cur, gi, ip, lane, xi_w);
                const int4 bii = D.binfo[gi];
                const uint4 mi = s_mir[s_sb[q] + li];
                int count = 0;
                for (int jb = 0; jb < na; jb += 32) {
                    const int lj = jb + lane;
                    int f = 0;
                    const int gj = off + lj;
                    if (lj < na && lj != li) f = test_pair(E, g, ip, cur, gi, bii, mi, xi_w, gj, maxcut2f, id);
                    warp_append(D, g, gi, lane, f, gj, count);
                }
                bead_end(D, g, gi, lane, count);
            }
            if (all_beads)
                for (int li = na + tid; li < ip.n; li += nt) D.nnbr[off + li] = 0;
        }
        __syncthreads();
        if (g.any_ss)
            for (int q = 0; q < ni; ++q)
                if (s_fire[q] && D.ip[s_iid[q]].ss_on)
                    for (int li = tid; li < s_n[q]; li += nt) ss_records(D, g, cur, s_off[q] + li, s_iid[q]);
        __syncthreads();
        if (tid == 0) {
            int nbp = 0, nfired = 0;
            for (int q = 0; q < ni; ++q) {
                s_bp[q] = nbp;
                nbp += min(__ldcg(D.bp_cnt + s_iid[q]), D.ip[s_iid[q]].bp_cap);
                if (s_fire[q]) {
                    D.flag[s_iid[q]] = 1;
                    ++nfired;
                }
            }
            s_bp[ni] = nbp;
            atomicAdd((unsigned long long *)D.rebuilds, (unsigned long long)nfired);
        }
        __syncthreads();
        if (tid == 0) s_any = 0;
    };
    // the inner lists of the instances with s_ifire set, from their lists and
    // the current mirrors (one warp per bead, kept entries in list order);
    // ends with s_anyi cleared
    auto refresh = [&]() {
        for (int q = 0; q < ni; ++q) {
            if (!s_ifire[q]) continue;
            const int id = s_iid[q], off = s_off[q], sb = s_sb[q], na = s_n[q];
            const InstP &ip = ipc_on ? s_ipc[q] : D.ip[id];
            const float re = g.flg_ele ? sqrtf(ip.ele_cut2_f) : 0.f, rw = sqrtf(g.f_wca_sig2);
            for (int li = warp; li < na; li += nwarps) {
                const int gi = off + li;
                const uint4 mi = s_mir[sb + li];
                const int m = min(D.nnbr[gi], g.cap);
                const int *src = D.nbr + (size_t)gi * g.cap;
                int *dst = D.nbr_in + (size_t)gi * g.cap;
                int cnt = 0;
                for (int k0 = 0; k0 < m; k0 += 32) {
                    const int k = k0 + lane;
                    int e = 0;
                    bool keep = false;
                    if (k < m) {
                        e = src[k];
                        const uint4 mj = s_mir[sb + (e & IDX_MASK) - off];
                        const float dx = (float)(int)(mi.x - mj.x) * ip.finv[0], dy = (float)(int)(mi.y - mj.y) * ip.finv[1],
                                    dz = (float)(int)(mi.z - mj.z) * ip.finv[2];
                        const float d2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
                        const float r = fmaxf((e & ELE_BIT) ? re : 0.f, (e & WCA_BIT) ? rw : 0.f) + kInnerMargin;
                        keep = d2 <= r * r * 1.0001f;
                    }
                    const unsigned bal = __ballot_sync(0xffffffffu, keep);
                    if (keep) dst[cnt + __popc(bal & ((1u << lane) - 1u))] = e;
                    cnt += __popc(bal);
                }
                if (lane == 0) {
                    D.nnbr_in[gi] = cnt;
                    D.mir_in[gi] = mi;
                }
            }
            if (tid == 0) D.igen[id] = __ldcg(D.lgen + id);
        }
        __syncthreads();
        if (tid == 0) s_anyi = 0;
    };
    // the inner lists due at a step's end or at the launch's start (first):
    // the instances whose lists were rebuilt since their filtering (in the
    // launch: rebuilt; before it: their counts differ), or whose two largest
    // displacements since it (s_m3, s_m4) sum to more than the margin
    auto inner_due = [&](int k, bool rebuilt, bool first) {
        const bool f = INNER && s_n[k] >= kInnerMinBeads &&
                       (rebuilt || (first && __ldcg(D.igen + s_iid[k]) != __ldcg(D.lgen + s_iid[k])) ||
                        sqrtf(__uint_as_float(s_m3[k])) + sqrtf(__uint_as_float(s_m4[k])) > kInnerMargin);
        s_ifire[k] = f;
        s_m3[k] = s_m4[k] = 0u;
        if (f) s_anyi = 1;
    };
    // instances flagged before the launch (slots loaded since the last
    // launch): their lists first
    if (tid < ni) {
        const int f = __ldcg(D.flag + s_iid[tid]) != 0;
        s_fire[tid] = f;
        if (f) {
            s_any = 1;
            D.bp_cnt[s_iid[tid]] = 0;
        }
    }
    __syncthreads();
    if (s_any) rebuild(cur, true);
    if (INNER) {
        if (tid < ni) inner_due(tid, false, true);
        __syncthreads();
        if (s_anyi) refresh();
    }
    const unsigned long long step0 = *D.step_ctr;
    for (int st = 0; st < nsteps; ++st) {
        // the base-pair records' energies and statuses are read only after
        // the launch: written on its last step
        const bool rec_out = st == nsteps - 1;
        // Forces.  Base pairs, bonded terms and pair forces need no barrier
        // between them: the base-pair forces add into s_fbp (exact
        // fixed-point atomics), the bonded terms write their slot planes, the
        // pair sums go to s_F, and the update reads all three after one
        // barrier.
        // ------------------------------------------------ base pairs
        if (g.bp_model > 0) {
            // every warp tests 32 records at a time and queues the ones in the
            // distance window (bucket-local instance | slot); a full queue is
            // evaluated by the whole warp, the rest at the end
            int2 *wq = s_qi + warp * 64;
            int wn = 0;
            const int nrec = s_bp[ni];
            for (;;) {
                int r0 = 0;
                if (lane == 0) r0 = atomicAdd(&s_rnext, 32);
                r0 = __shfl_sync(0xffffffffu, r0, 0);
                if (r0 >= nrec) break;
                const int r = r0 + lane;
                bool pass = false;
                int q = 0, slot = 0;
                if (r < nrec) {
                    q = small_inst(s_bp, ni, r);
                    slot = s_bpo[q] + (r - s_bp[q]);
                    const Dev E = view(q);
                    pass = bp_test<float>(E, g, cur, slot, rec_out);
                }
                const unsigned bal = __ballot_sync(0xffffffffu, pass);
                if (pass) wq[wn + __popc(bal & ((1u << lane) - 1u))] = make_int2(q, slot);
                wn += __popc(bal);
                __syncwarp();
                if (wn >= 32) {
                    const int2 w = wq[lane];
                    const Dev E = view(w.x);
                    if (bp_eval_f(E, g, cur, w.y, rec_out)) bp_eval_d(D, g, cur, w.y, E.fbp);
                    __syncwarp();
                    if (lane < wn - 32) wq[lane] = wq[32 + lane];
                    wn -= 32;
                    __syncwarp();
                }
            }
            if (lane < wn) {
                const int2 w = wq[lane];
                const Dev E = view(w.x);
                if (bp_eval_f(E, g, cur, w.y, rec_out)) bp_eval_d(D, g, cur, w.y, E.fbp);
            }
        }
        // ------------------------------------------------ bonded terms
        for (int s = tid; s < nb; s += nt) {
            const int q = small_inst(s_sb, ni, s);
            const int gi = s_off[q] + (s - s_sb[q]);
            const Dev E = view(q);
            bool an, dn;
            float4 *S = sslot ? s_slot + s : (float4 *)D.slot + gi;
            const size_t pl = sslot ? (size_t)cap : (size_t)g.n;
            bonded_terms_to<float>(E, g, cur, gi, S, pl, &an, &dn);
            if (an) bonded_fp64_to(D, g, cur, gi, 0, S, pl);
            if (dn) bonded_fp64_to(D, g, cur, gi, 1, S, pl);
        }
        // ------------------------------------------------ pair forces
        {
            constexpr int BPW = 32 / kSmallLanes; // beads per warp and pass
            const int sub = lane & (kSmallLanes - 1);
            for (;;) {
                int base = 0;
                if (lane == 0) base = atomicAdd(&s_pnext, BPW);
                base = __shfl_sync(0xffffffffu, base, 0);
                if (base >= nb) break;
                // every lane of a warp runs the same passes (shuffles below)
                const int s0 = base + lane / kSmallLanes;
                const int s = min(s0, nb - 1);
                const int q = small_inst(s_sb, ni, s);
                const int off = s_off[q], sb = s_sb[q];
                const int gi = off + (s - sb);
                const InstP &ip = ipc_on ? s_ipc[q] : D.ip[s_iid[q]];
                const uint4 mi = s_mir[s];
                const PairCoef P = pair_coef_of(g, ip);
                const bool inner = INNER && s_n[q] >= kInnerMinBeads;
                const int m = min(inner ? D.nnbr_in[gi] : D.nnbr[gi], g.cap);
                // coherent loads: the launch rewrites the lists
                const int *nbl = (inner ? D.nbr_in : D.nbr) + (size_t)gi * g.cap;
                const float2 f0 = make_float2(ip.finv[0], ip.finv[0]), f1 = make_float2(ip.finv[1], ip.finv[1]),
                             f2 = make_float2(ip.finv[2], ip.finv[2]);
                // lane sub takes entries sub, sub + L, sub + 2L, ... (L =
                // kSmallLanes), two at a time (pair2), in batches of 16
                // entries whose list words load before any is used; a
                // missing entry is the bead itself with no term bit (an
                // exact zero)
                float2 ax = make_float2(0.f, 0.f), ay = ax, az = ax;
                constexpr int L = kSmallLanes;
                // every lane runs the batches of the warp's longest list
                const int mmax = __reduce_max_sync(0xffffffffu, m);
                for (int k0 = sub; k0 - sub < mmax; k0 += 16 * L) {
                    // the batch's 16 list words in flight at once
                    int e[16];
#pragma unroll
                    for (int u = 0; u < 16; ++u) e[u] = k0 + u * L < m ? nbl[k0 + u * L] : gi;
#pragma unroll
                    for (int u = 0; u < 16; u += 2) {
                        if (k0 - sub + u * L >= mmax) break; // warp-uniform: past every lane's list
                        const uint4 ma = s_mir[sb + (e[u] & IDX_MASK) - off], mb = s_mir[sb + (e[u + 1] & IDX_MASK) - off];
                        const Pair2 pr = pair2(mi, ma, mb, f0, f1, f2, e[u] & WCA_BIT, e[u + 1] & WCA_BIT, e[u] & ELE_BIT,
                                               e[u + 1] & ELE_BIT, P);
                        ax = __ffma2_rn(pr.c, pr.vx, ax);
                        ay = __ffma2_rn(pr.c, pr.vy, ay);
                        az = __ffma2_rn(pr.c, pr.vz, az);
                    }
                }
                float fx = ax.x + ax.y, fy = ay.x + ay.y, fz = az.x + az.y;
#pragma unroll
                for (int o = kSmallLanes / 2; o > 0; o >>= 1) {
                    fx += __shfl_xor_sync(0xffffffffu, fx, o, kSmallLanes);
                    fy += __shfl_xor_sync(0xffffffffu, fy, o, kSmallLanes);
                    fz += __shfl_xor_sync(0xffffffffu, fz, o, kSmallLanes);
                }
                if (sub == 0 && s0 < nb) s_F[s] = make_float4(fx, fy, fz, 0.f);
            }
        }
        __syncthreads();
        // ------------------------------------------------ update and trigger (job_md.F90:376-395)
        // the step's force: pair + bonded (its slot planes, in slot order) +
        // base pair (fixed point, cleared for the next step), then the cap
        const unsigned long long step = step0 + (unsigned long long)st;
        for (int s = tid; s < nb; s += nt) {
            const int q = small_inst(s_sb, ni, s);
            const int gi = s_off[q] + (s - s_sb[q]);
            // every global load of the bead's update first
            const bool inner = INNER && s_n[q] >= kInnerMinBeads;
            const uint4 m0 = D.mir0[gi], mI = inner ? D.mir_in[gi] : m0;
            const int4 bi = D.binfo[gi];
            const double4 x = x_at(D, cur)[gi], v = D.v[gi], b = D.beta[gi];
            const InstP &jp = ipc_on ? s_ipc[q] : D.ip[s_iid[q]];
            const V3<float> ab = sslot ? bonded_gather_at<float>(s_slot, (size_t)cap, s_sb[q] - s_off[q], bi, 0, 1, 7)
                                       : bonded_gather<float>(D, g, bi, 0, 1, 7);
            float xi[3];
            mixed_noise(g, gi, jp, noise, st, step, xi);
            const float4 F4 = s_F[s];
            const double4 fb = s_fbp[s];
            s_fbp[s] = make_double4(0.0, 0.0, 0.0, 0.0);
            float F[3] = {F4.x + ab.x + fx_float(fb.x), F4.y + ab.y + fx_float(fb.y), F4.z + ab.z + fx_float(fb.z)};
            if (g.fcap_f > 0.f) {
                const float fm = sqrtf(F[0] * F[0] + F[1] * F[1] + F[2] * F[2]);
                if (fm > g.fcap_f) {
                    const float sc = g.fcap_f / fm;
                    F[0] *= sc;
                    F[1] *= sc;
                    F[2] *= sc;
                    atomicAdd(D.capped, 1ull);
                }
            }
            float4 r4;
            const double2 cd = s_cd[s];
            const float2 cf = s_cf[s];
            const uint4 m1 = mixed_update_core(D, g, cur, gi, jp, F, cf.x, cf.y, xi, x, make_double4(cd.x, 0.0, cd.y, 0.0), v, b, &r4);
            s_mir[s] = m1;
            s_res[s] = r4;
            const float *fi = jp.finv;
            const float dx = (float)(int)(m1.x - m0.x) * fi[0];
            const float dy = (float)(int)(m1.y - m0.y) * fi[1];
            const float dz = (float)(int)(m1.z - m0.z) * fi[2];
            const unsigned int bits = __float_as_uint(fmaf(dx, dx, fmaf(dy, dy, dz * dz)));
            const unsigned int old = atomicMax(&s_m1[q], bits);
            atomicMax(&s_m2[q], old < bits ? old : bits);
            if (inner) {
                const float ix = (float)(int)(m1.x - mI.x) * fi[0], iy = (float)(int)(m1.y - mI.y) * fi[1],
                            iz = (float)(int)(m1.z - mI.z) * fi[2];
                const unsigned int ibits = __float_as_uint(fmaf(ix, ix, fmaf(iy, iy, iz * iz)));
                const unsigned int iold = atomicMax(&s_m3[q], ibits);
                atomicMax(&s_m4[q], iold < ibits ? iold : ibits);
            }
        }
        __syncthreads();
        if (tid == 0) s_rnext = s_pnext = 0;
        if (tid < ni) {
            const bool f = sqrtf(__uint_as_float(s_m1[tid])) + sqrtf(__uint_as_float(s_m2[tid])) > (float)g.nl_margin;
            s_fire[tid] = f;
            s_m1[tid] = s_m2[tid] = 0u;
            if (f) {
                s_any = 1;
                D.bp_cnt[s_iid[tid]] = 0;
            }
            if (INNER) inner_due(tid, f, false);
        }
        __syncthreads();
        cur ^= 1;
        if (s_any) rebuild(cur, false);
        if (INNER && s_anyi) refresh();
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
    const double4 *x64 = x_at(D, cur);
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
// only_inst >= 0: that instance alone.  Frozen beads (all coefficients zero,
// e.g. the inert filler of a serving slot) get zero velocity.
template <typename R> __global__ void k_init_velocities(Dev D, GlobP g, unsigned long long ctr, int only_inst) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= g.n) return;
    const int4 bi = D.binfo[i];
    if (only_inst >= 0 && bi.x != only_inst) return;
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
    if (m.x == 0.0 && m.y == 0.0 && m.z == 0.0 && m.w == 0.0) v = make_double4(0.0, 0.0, 0.0, 0.0);
    D.v[i] = v;
    D.beta[i] = b;
}

// refresh the fixed-point mirror from the FP64 positions
__global__ void k_mirror(Dev D, GlobP g, int cur) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= g.n) return;
    const InstP &ip = D.ip[D.binfo[i].x];
    const double4 x = x_at(D, cur)[i];
    float r[3];
    mir_at(D, cur)[i] = make_uint4(fixed_res(x.x, ip.fsc[0], r[0]), fixed_res(x.y, ip.fsc[1], r[1]), fixed_res(x.z, ip.fsc[2], r[2]), 0u);
    res_at(D, cur)[i] = make_float4(r[0], r[1], r[2], 0.f);
}

// ------------------------------------------------------------- launchers
template <typename R, int G, int MODE>
static cudaError_t launch_step_g(const Dev &D, const GlobP &g, int cur, const double *noise, long long ns, double *fout, int mask,
                                 cudaStream_t st) {
    constexpr int bpb = 256 / G;
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

// (trigger: the last block decides the displacement trigger and advances the
// step counter; off only in the autotuner's timing passes)
static cudaError_t launch_step_mixed(const Dev &D, const GlobP &g, int cur, const double *noise, long long ns, int mask,
                                     cudaStream_t st) {
    k_step_mixed<<<(g.n + 255) / 256, 256, 0, st>>>(D, g, cur, noise, ns, mask);
    return cudaGetLastError();
}
// (the mixed path always takes its pair forces from k_pairs_cl)
cudaError_t launch_step(int G, const Dev &D, const GlobP &g, int cur, const double *noise, long long ns, cudaStream_t st,
                        int trigger) {
    if (g.prec == 0) return launch_step_r<double, 0>(G, D, g, cur, noise, ns, nullptr, 63 | (trigger ? 256 : 0), st);
    return launch_step_mixed(D, g, cur, noise, ns, 63 | 64 | (trigger ? 256 : 0), st);
}

// the step with its pair forces taken from fpair (k_pairs ran before it, with
// the same G, so that every sum is formed in the same order as in one kernel)
cudaError_t launch_step_split(int G, const Dev &D, const GlobP &g, int cur, const double *noise, long long ns, cudaStream_t st,
                              int trigger) {
    const int mask = 63 | 64 | (trigger ? 256 : 0);
    if (g.prec == 0) return launch_step_r<double, 0>(G, D, g, cur, noise, ns, nullptr, mask, st);
    return launch_step_mixed(D, g, cur, noise, ns, mask, st);
}

template <typename R, int G> static cudaError_t launch_pairs_g(const Dev &D, const GlobP &g, int cur, cudaStream_t st) {
    constexpr int bpb = 256 / G;
    k_pairs<R, G><<<(g.n + bpb - 1) / bpb, 256, 0, st>>>(D, g, cur);
    return cudaGetLastError();
}
template <typename R> static cudaError_t launch_pairs_r(int G, const Dev &D, const GlobP &g, int cur, cudaStream_t st) {
    switch (G) {
    case 1: return launch_pairs_g<R, 1>(D, g, cur, st);
    case 2: return launch_pairs_g<R, 2>(D, g, cur, st);
    case 4: return launch_pairs_g<R, 4>(D, g, cur, st);
    case 8: return launch_pairs_g<R, 8>(D, g, cur, st);
    case 16: return launch_pairs_g<R, 16>(D, g, cur, st);
    default: return launch_pairs_g<R, 32>(D, g, cur, st);
    }
}
// pair forces into fpair: per-bead lists in the FP64 path, cluster pairs in the mixed path
cudaError_t launch_pairs(int G, const Dev &D, const GlobP &g, int cur, cudaStream_t st) {
    if (g.prec == 0) return launch_pairs_r<double>(G, D, g, cur, st);
    k_pairs_cl<<<(g.n_cl + 7) / 8, 256, 0, st>>>(D, g, cur, 48);
    return cudaGetLastError();
}

// forces of the terms in mask into fout (MODE 1 of the step kernel); the
// mixed path takes its pair forces from k_pairs_cl
cudaError_t launch_force(int G, const Dev &D, const GlobP &g, int cur, double *fout, int mask, cudaStream_t st) {
    if (g.prec == 0) return launch_step_r<double, 1>(G, D, g, cur, nullptr, 0, fout, mask, st);
    if (mask & 48) {
        k_pairs_cl<<<(g.n_cl + 7) / 8, 256, 0, st>>>(D, g, cur, mask & 48);
        const cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
        mask |= 64;
    }
    return launch_step_r<float, 1>(G, D, g, cur, nullptr, 0, fout, mask, st);
}
int force_kernels(const GlobP &g, int mask) { return 1 + (g.prec != 0 && (mask & 48) ? 1 : 0); }

// bonded terms (if do_bonded) and base-pair forces (if do_bp) of one step
cudaError_t launch_bonded(const Dev &D, const GlobP &g, int cur, cudaStream_t st) {
    if (g.prec == 0) k_bonded<double><<<(g.n + 255) / 256, 256, 0, st>>>(D, g, cur);
    else k_bonded<float><<<(g.n + 255) / 256, 256, 0, st>>>(D, g, cur);
    return cudaGetLastError();
}
cudaError_t launch_bonded_step(const Dev &D, const GlobP &g, int cur, cudaStream_t st) {
    if (g.prec == 0) return launch_bonded(D, g, cur, st);
    k_bonded_fb<<<(g.n + 255) / 256, 256, 0, st>>>(D, g, cur);
    return cudaGetLastError();
}

// test_blocks covers the staging capacity (grid stride beyond it), eval_blocks
// the windowed records of an ordinary step
// (one wave of k_bp, two blocks per SM, each taking a grid-stride share of
// the records: the evaluations of every block then run at once)
cudaError_t launch_bp(const Dev &D, const GlobP &g, int cur, int test_blocks, int eval_blocks, cudaStream_t st) {
    const int blocks = std::max(1, std::min(test_blocks, eval_blocks));
    if (g.prec == 0) k_bp<double><<<blocks, 256, 0, st>>>(D, g, cur);
    else k_bp<float><<<blocks, 256, 0, st>>>(D, g, cur);
    return cudaGetLastError();
}
int bp_kernels(const GlobP &g) { return g.bp_model > 0 ? 1 : 0; }

// bonded terms (if do_bonded) and base-pair forces (if do_bp), one after the
// other on st
cudaError_t launch_pre(const Dev &D, const GlobP &g, int cur, int do_bonded, int do_bp, int test_blocks, int eval_blocks,
                       cudaStream_t st) {
    cudaError_t e = cudaSuccess;
    if (do_bonded) e = launch_bonded(D, g, cur, st);
    if (e == cudaSuccess && do_bp && g.bp_model > 0) e = launch_bp(D, g, cur, test_blocks, eval_blocks, st);
    return e;
}
int pre_kernels(const GlobP &g, int do_bonded, int do_bp) { return (do_bonded ? 1 : 0) + (do_bp ? bp_kernels(g) : 0); }

cudaError_t launch_bp_energy(const Dev &D, const GlobP &g, int cur, double tK, int bp_blocks, cudaStream_t st) {
    k_bp_energy<<<bp_blocks, 256, 0, st>>>(D, g, cur, tK);
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

// energy_rg.F90:17-26: unweighted radius of gyration of each instance's
// coordinates (two passes: centre, then mean squared distance), one block
// per instance with a fixed-order reduction
__device__ __forceinline__ double block_sum(double v, double *s) {
    s[threadIdx.x] = v;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) s[threadIdx.x] += s[threadIdx.x + o];
        __syncthreads();
    }
    const double r = s[0];
    __syncthreads();
    return r;
}
__global__ void __launch_bounds__(256) k_rg(Dev D, int cur, double *out) {
    __shared__ double s[256];
    const InstP &ip = D.ip[blockIdx.x];
    const double4 *x = x_at(D, cur) + ip.bead_off;
    double cx = 0.0, cy = 0.0, cz = 0.0;
    for (int i = threadIdx.x; i < ip.n; i += blockDim.x) {
        cx += x[i].x;
        cy += x[i].y;
        cz += x[i].z;
    }
    cx = block_sum(cx, s) / ip.n;
    cy = block_sum(cy, s) / ip.n;
    cz = block_sum(cz, s) / ip.n;
    double s2 = 0.0;
    for (int i = threadIdx.x; i < ip.n; i += blockDim.x) {
        const double vx = x[i].x - cx, vy = x[i].y - cy, vz = x[i].z - cz;
        s2 += vx * vx + vy * vy + vz * vz;
    }
    s2 = block_sum(s2, s);
    if (threadIdx.x == 0) out[blockIdx.x] = sqrt(s2 / ip.n);
}

// ------------------------------------------------------- optional terms
// force.F90:62-75 and energy_sumup.F90:47-52: stage wall (force_stage.F90),
// tweezers (force_tweezers.F90), Rg bias (force_rg.F90) and sigmoid
// restraints (force_restraint.F90), in FP64 from the FP64 positions in both
// paths (they are O(n) or a handful of pairs).  Forces go to fbp, as the
// base-pair forces do: FP64 atomics in the FP64 path, exact fixed point in
// the mixed path; the step kernel consumes fbp under mask bit 8 or 128.
constexpr double kSmallValue = 2.220446049250313e-16; // const_phys.F90 SMALL_VALUE = epsilon(PI)

__device__ __forceinline__ void bias_scatter(const Dev &D, const GlobP &g, int i, double fx, double fy, double fz) {
    if (g.prec == 0) {
        atomicAdd(&D.fbp[i].x, fx);
        atomicAdd(&D.fbp[i].y, fy);
        atomicAdd(&D.fbp[i].z, fz);
        return;
    }
    if (!(fabs(fx) < FX_LIMIT && fabs(fy) < FX_LIMIT && fabs(fz) < FX_LIMIT)) {
        atomicOr(D.err, ERR_NONFINITE);
        return;
    }
    fx_scatter(D.fbp, i, fx_of(fx), fx_of(fy), fx_of(fz));
}

// force_rg.F90:17-31 / energy_rg.F90: the centre and radius of gyration of
// every instance with an Rg bias (one block each, fixed-order sums), its
// force factor -k (rg - rg0) / (rg n) and its energy
__global__ void __launch_bounds__(256) k_bias_rg(Dev D, GlobP g, int cur) {
    __shared__ double s[256];
    const InstP &ip = D.ip[blockIdx.x];
    if (ip.rg_pott == 0) return;
    const double4 *x = x_at(D, cur) + ip.bead_off;
    double cx = 0.0, cy = 0.0, cz = 0.0;
    for (int i = threadIdx.x; i < ip.n; i += blockDim.x) {
        cx += x[i].x;
        cy += x[i].y;
        cz += x[i].z;
    }
    cx = block_sum(cx, s) / ip.n;
    cy = block_sum(cy, s) / ip.n;
    cz = block_sum(cz, s) / ip.n;
    double s2 = 0.0;
    for (int i = threadIdx.x; i < ip.n; i += blockDim.x) {
        const double vx = x[i].x - cx, vy = x[i].y - cy, vz = x[i].z - cz;
        s2 += vx * vx + vy * vy + vz * vz;
    }
    s2 = block_sum(s2, s);
    if (threadIdx.x == 0) {
        const double rg = sqrt(s2 / ip.n);
        const bool off = ip.rg_pott == 2 && rg <= ip.rg0;
        D.rgb[blockIdx.x] = make_double4(cx, cy, cz, off ? 0.0 : -ip.rg_k * (rg - ip.rg0) / (rg * ip.n));
        D.rgv[blockIdx.x] = off ? 0.0 : 0.5 * ip.rg_k * (rg - ip.rg0) * (rg - ip.rg0);
    }
}

// Threads [0, n): the stage wall and the Rg bias of one bead; then one
// thread per item.  in_step: force ramps place their traps at the
// reference's istep, which counts the step being taken (job_md.F90:362):
// the steps taken plus 1 inside a step, plus 0 outside the MD loop.
__global__ void __launch_bounds__(256) k_bias(Dev D, GlobP g, int cur, int in_step) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const double4 *x = x_at(D, cur);
    if (t < g.n) {
        const int inst = D.binfo[t].x;
        const double4 xi = x[t];
        double fx = 0.0, fy = 0.0, fz = 0.0;
        if (g.flg_stage) {
            double z = xi.z;
            if (z < kSmallValue) z = kSmallValue;
            z = g.stage_sigma / z;
            const double z2 = z * z, z6 = z2 * z2 * z2, z7 = z6 * z, z13 = z6 * z7;
            fz += 24.0 * g.stage_eps / g.stage_sigma * (2.0 * z13 - z7);
        }
        if (g.flg_rg && D.ip[inst].rg_pott != 0) {
            const double4 r = D.rgb[inst];
            fx += r.w * (xi.x - r.x);
            fy += r.w * (xi.y - r.y);
            fz += r.w * (xi.z - r.z);
        }
        if (fx != 0.0 || fy != 0.0 || fz != 0.0) bias_scatter(D, g, t, fx, fy, fz);
        return;
    }
    const int q = t - g.n;
    if (q >= g.n_bias) return;
    const BiasItem b = D.bias[q];
    const InstP &ip = D.ip[b.inst];
    if (b.kind <= 2) {
        const V3<double> v = dvec64(x[b.i], x[b.j], ip);
        const double r = sqrt(dot3(v, v));
        if (r >= b.p[3]) return;
        const double th = tanh((r - b.p[1]) / b.p[2]);
        const double coef = 0.5 * b.p[0] / b.p[2] * (1.0 - th * th) / r;
        bias_scatter(D, g, b.i, -coef * v.x, -coef * v.y, -coef * v.z);
        if (b.kind == 1) bias_scatter(D, g, b.j, coef * v.x, coef * v.y, coef * v.z);
    } else if (b.kind == 3) {
        const double sc = ip.twz_scale;
        bias_scatter(D, g, b.i, sc * b.p[0], sc * b.p[1], sc * b.p[2]);
        bias_scatter(D, g, b.j, -sc * b.p[0], -sc * b.p[1], -sc * b.p[2]);
    } else {
        const double istep = (double)(*D.step_ctr + (unsigned long long)in_step);
        for (int tt = 0; tt < 2; ++tt) {
            const int i = tt ? b.j : b.i;
            const double4 trap = make_double4(b.p[2 + 3 * tt] + b.p[8 + 3 * tt] * istep, b.p[3 + 3 * tt] + b.p[9 + 3 * tt] * istep,
                                              b.p[4 + 3 * tt] + b.p[10 + 3 * tt] * istep, 0.0);
            const V3<double> v = dvec64(trap, x[i], ip);
            bias_scatter(D, g, i, b.p[tt] * v.x, b.p[tt] * v.y, b.p[tt] * v.z);
        }
    }
}

// energy_stage.F90, energy_tweezers.F90, energy_rg.F90, energy_restraint.F90
// into the energy slots 7-10 (k_bias_rg ran first)
__global__ void __launch_bounds__(256) k_bias_energy(Dev D, GlobP g, int cur) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const double4 *x = x_at(D, cur);
    if (t < g.n) {
        if (!g.flg_stage) return;
        const int inst = D.binfo[t].x;
        const double z = g.stage_sigma / x[t].z;
        const double z2 = z * z, z6 = z2 * z2 * z2;
        atomicAdd(D.ene + (size_t)inst * 12 + 7, 4.0 * g.stage_eps * (z6 * z6 - z6));
        return;
    }
    int q = t - g.n;
    if (q < g.n_inst) {
        if (g.flg_rg && D.ip[q].rg_pott != 0) atomicAdd(D.ene + (size_t)q * 12 + 9, D.rgv[q]);
        return;
    }
    q -= g.n_inst;
    if (q >= g.n_bias) return;
    const BiasItem b = D.bias[q];
    const InstP &ip = D.ip[b.inst];
    double *E = D.ene + (size_t)b.inst * 12;
    if (b.kind <= 2) {
        const V3<double> v = dvec64(x[b.i], x[b.j], ip);
        const double r = sqrt(dot3(v, v));
        if (r < b.p[3]) atomicAdd(E + 10, -0.5 * b.p[0] * (1.0 - tanh((r - b.p[1]) / b.p[2])));
    } else if (b.kind == 3) {
        const V3<double> v = dvec64(x[b.i], x[b.j], ip);
        const double sc = ip.twz_scale;
        atomicAdd(E + 8, -(v.x * (sc * b.p[0]) + v.y * (sc * b.p[1]) + v.z * (sc * b.p[2])));
    }
}

cudaError_t launch_bias(const Dev &D, const GlobP &g, int cur, int in_step, cudaStream_t st) {
    if (!g.flg_bias) return cudaSuccess;
    if (g.flg_rg) k_bias_rg<<<g.n_inst, 256, 0, st>>>(D, g, cur);
    k_bias<<<(g.n + g.n_bias + 255) / 256, 256, 0, st>>>(D, g, cur, in_step);
    return cudaGetLastError();
}
int bias_kernels(const GlobP &g) { return g.flg_bias ? 1 + (g.flg_rg ? 1 : 0) : 0; }

cudaError_t launch_bias_energy(const Dev &D, const GlobP &g, int cur, cudaStream_t st) {
    if (!g.flg_bias) return cudaSuccess;
    if (g.flg_rg) k_bias_rg<<<g.n_inst, 256, 0, st>>>(D, g, cur);
    k_bias_energy<<<(g.n + g.n_inst + g.n_bias + 255) / 256, 256, 0, st>>>(D, g, cur);
    return cudaGetLastError();
}

// per bead: mirror, residual, base-pair sum, pair force, coefficients (FP64
// and FP32); then the 8 bonded slot planes when they fit in kSmallDynMax
constexpr size_t kSmallBeadBytes = sizeof(uint4) + sizeof(float4) + sizeof(double4) + sizeof(float4) + sizeof(double2) + sizeof(float2);
bool small_slot_planes(int cap) { return (size_t)cap * (kSmallBeadBytes + 8 * sizeof(float4)) <= (size_t)kSmallDynMax; }
size_t small_smem_bytes(int cap) { return (size_t)cap * (kSmallBeadBytes + (small_slot_planes(cap) ? 8 * sizeof(float4) : 0)); }

cudaError_t launch_md_small(const Dev &D, const GlobP &g, int cur, const SmallPlan &sp, int nsteps, const double *noise, int threads,
                            cudaStream_t st) {
    const size_t smem = small_smem_bytes(sp.cap);
    SmallPlan p = sp;
    p.sslot = small_slot_planes(sp.cap) ? 1 : 0;
    auto kern = sp.inner ? (threads <= 384 ? k_md_small<true, 384> : k_md_small<true, 512>)
                         : (threads <= 384 ? k_md_small<false, 384> : k_md_small<false, 512>);
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    kern<<<p.n_cta, threads, smem, st>>>(D, g, cur, p, nsteps, noise);
    return cudaGetLastError();
}

// the bookkeeping after k_md_small: base-pair prefix counts over the
// instances (as rebuild_finish forms them), the Philox step counter, and the
// rebuild flags (after the cluster lists of the rebuilt instances were formed)
__global__ void __launch_bounds__(256) k_small_finish(Dev D, GlobP g, unsigned long long nsteps) {
    __shared__ int s[256];
    const int n = g.n_inst;
    const int per = (n + 255) / 256;
    const int lo = min(n, (int)threadIdx.x * per), hi = min(n, lo + per);
    int sum = 0;
    for (int k = lo; k < hi; ++k) sum += min(D.bp_cnt[k], D.ip[k].bp_cap);
    s[threadIdx.x] = sum;
    __syncthreads();
    for (int o = 1; o < 256; o <<= 1) {
        const int v = threadIdx.x >= (unsigned)o ? s[threadIdx.x - o] : 0;
        __syncthreads();
        s[threadIdx.x] += v;
        __syncthreads();
    }
    int run = s[threadIdx.x] - sum;
    for (int k = lo; k < hi; ++k) {
        D.bp_cnt[n + k] = run;
        run += min(D.bp_cnt[k], D.ip[k].bp_cap);
        D.flag[k] = 0;
    }
    if (threadIdx.x == 255) *D.bp_total = s[255];
    if (threadIdx.x == 0) *D.step_ctr += nsteps;
}

cudaError_t launch_small_finish(const Dev &D, const GlobP &g, unsigned long long nsteps, cudaStream_t st) {
    k_small_finish<<<1, 256, 0, st>>>(D, g, nsteps);
    return cudaGetLastError();
}

cudaError_t launch_rg(const Dev &D, const GlobP &g, int cur, double *out, cudaStream_t st) {
    k_rg<<<g.n_inst, 256, 0, st>>>(D, cur, out);
    return cudaGetLastError();
}

cudaError_t launch_init_velocities(const Dev &D, const GlobP &g, unsigned long long ctr, cudaStream_t st, int only_inst) {
    k_init_velocities<double><<<(g.n + 255) / 256, 256, 0, st>>>(D, g, ctr, only_inst);
    return cudaGetLastError();
}

cudaError_t launch_mirror(const Dev &D, const GlobP &g, int cur, cudaStream_t st) {
    k_mirror<<<(g.n + 255) / 256, 256, 0, st>>>(D, g, cur);
    return cudaGetLastError();
}

} // namespace sisg
