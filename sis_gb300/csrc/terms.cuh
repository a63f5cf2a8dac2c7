// Force and energy terms of the SIS model, templated on the arithmetic type.
// Each function restates one Fortran routine of the reference; the file:line
// of that routine is given at the function.  FP64 instantiations keep the
// reference's expression order; FP32 instantiations are used by the mixed
// precision path, which re-evaluates angle terms near cos = +-1 in FP64 from
// the FP64 positions.
#pragma once

#include "common.cuh"

namespace sisg {

// Math functions with explicit single/double overloads, so that FP32
// instantiations never promote to the FP64 pipe.
namespace fm {
__device__ __forceinline__ float sqrt(float x) { return sqrtf(x); }
__device__ __forceinline__ double sqrt(double x) { return ::sqrt(x); }
__device__ __forceinline__ float acos(float x) { return acosf(x); }
__device__ __forceinline__ double acos(double x) { return ::acos(x); }
__device__ __forceinline__ float atan2(float y, float x) { return atan2f(y, x); }
__device__ __forceinline__ double atan2(double y, double x) { return ::atan2(y, x); }
__device__ __forceinline__ float sin(float x) { return sinf(x); }
__device__ __forceinline__ double sin(double x) { return ::sin(x); }
__device__ __forceinline__ float cos(float x) { return cosf(x); }
__device__ __forceinline__ double cos(double x) { return ::cos(x); }
__device__ __forceinline__ float exp(float x) { return expf(x); }
__device__ __forceinline__ double exp(double x) { return ::exp(x); }
__device__ __forceinline__ float fabs(float x) { return fabsf(x); }
__device__ __forceinline__ double fabs(double x) { return ::fabs(x); }
__device__ __forceinline__ float copysign(float a, float b) { return copysignf(a, b); }
// a / b: FP32 as a product with the Newton-refined reciprocal (within an ulp
// or so), FP64 as the rounded quotient
__device__ __forceinline__ float div(float a, float b) { return a * rcp_nr(b); }
__device__ __forceinline__ double div(double a, double b) { return a / b; }
__device__ __forceinline__ double copysign(double a, double b) { return ::copysign(a, b); }
} // namespace fm

template <typename R> __device__ __forceinline__ R pick(double d, float f);
template <> __device__ __forceinline__ double pick<double>(double d, float) { return d; }
template <> __device__ __forceinline__ float pick<float>(double, float f) { return f; }

template <typename R> __device__ __forceinline__ V3<R> to(const V3<double> &a) { return mk<R>((R)a.x, (R)a.y, (R)a.z); }

// |cos| above which FP32 angle evaluations are redone in FP64: NEAR_ONE for
// the base-pair angles (acos form), NEAR_ONE_STRICT for the bonded angle and
// dihedral terms, whose FP32 forms are cancellation-free
constexpr float NEAR_ONE = 0.99f;
constexpr float NEAR_ONE_STRICT = 0.9999f;

// ------------------------------------------------------------- bond
// force_bond.F90:33-57: v = x1 - x2, f = k (d - r0)/d v, F1 -= f, F2 += f.
// Returns f (the force on the second bead).
template <typename R> __device__ __forceinline__ V3<R> bond_f(const V3<R> &v, const GlobP &g);
template <> __device__ __forceinline__ V3<double> bond_f<double>(const V3<double> &v, const GlobP &g) {
    const double d = fm::sqrt(dot3(v, v));
    const double delta = d - g.bond_r0;
    return (g.bond_k * delta / d) * v;
}
// FP32: d - r0 cancels; it is formed as (d^2 - r0^2)/(d + r0) with d^2 - r0^2
// accumulated from exact products (fmaf residuals) and error-free sums, so
// that its relative error stays near one float ulp.
__device__ __forceinline__ float two_sum(float a, float b, float &err) {
    const float s = a + b;
    const float bb = s - a;
    err = (a - (s - bb)) + (b - bb);
    return s;
}
template <> __device__ __forceinline__ V3<float> bond_f<float>(const V3<float> &v, const GlobP &g) {
    const float px = v.x * v.x, py = v.y * v.y, pz = v.z * v.z;
    const float ex = fmaf(v.x, v.x, -px), ey = fmaf(v.y, v.y, -py), ez = fmaf(v.z, v.z, -pz);
    float e1, e2;
    const float s1 = two_sum(px, py, e1);
    const float s2 = two_sum(s1, pz, e2);
    const float r0 = g.f_bond_r0;
    const float r0sq = r0 * r0, r0sq_lo = fmaf(r0, r0, -r0sq);
    const float diff = (s2 - r0sq) + ((e1 + e2) + (ex + ey + ez) - r0sq_lo);
    const float d = sqrtf(s2);
    const float delta = diff / (d + r0);
    return (g.f_bond_k * delta / d) * v;
}
template <typename R>
__device__ __forceinline__ V3<R> bond_force(const V3<R> &v, int p, const GlobP &g) {
    const V3<R> f = bond_f<R>(v, g);
    return p == 0 ? -f : f;
}
// energy_bond.F90:17-28
template <typename R> __device__ __forceinline__ R bond_energy(const V3<R> &v, const GlobP &g) {
    const R d = fm::sqrt(dot3(v, v));
    const R dd = d - pick<R>(g.bond_r0, g.f_bond_r0);
    return R(0.5) * pick<R>(g.bond_k, g.f_bond_k) * (dd * dd);
}

// ------------------------------------------------------------- angle
// force_angl.F90:35-83 with v21 = x2 - x1, v32 = x3 - x2; returns the force on
// participant p (0,1,2).  *cos_out receives the cosine before clamping.
template <typename T>
__device__ __forceinline__ V3<T> angle_force_core(const V3<T> &v21, const V3<T> &v32, int p, T k, T t0, T *cos_out) {
    const T d21 = dot3(v21, v21), d32 = dot3(v32, v32), d2132 = dot3(v32, v21);
    T cosine = -d2132 / fm::sqrt(d21 * d32);
    *cos_out = cosine;
    if (fm::fabs(cosine) > T(1)) cosine = fm::copysign(T(1), cosine);
    const T delta = fm::acos(cosine) - t0;
    T t = d21 * d32 - d2132 * d2132;
    if (t <= T(1)) t = T(1);
    const T f = k * delta / fm::sqrt(t);
    const V3<T> f21 = f * ((d2132 / d21) * v21 - v32);
    const V3<T> f32 = f * ((d2132 / d32) * v32 - v21);
    if (p == 0) return -f21;
    if (p == 1) return f21 - f32;
    return f32;
}
// force_angl_ReB.F90:36-74 with v12 = x1 - x2, v32 = x3 - x2
template <typename T>
__device__ __forceinline__ V3<T> angle_reb_force_core(const V3<T> &v12, const V3<T> &v32, int p, T k, T co0, T *cos_out) {
    const T d12 = dot3(v12, v12), d32 = dot3(v32, v32);
    const T a1232 = fm::sqrt(d12 * d32);
    const T cosine = dot3(v12, v32) / a1232;
    *cos_out = cosine;
    const T omc = T(1) - cosine * cosine;
    const T f = -k * (cosine - co0) * (T(1) - cosine * co0) / (omc * omc);
    const V3<T> f1 = f * ((T(1) / a1232) * v32 - (cosine / d12) * v12);
    const V3<T> f3 = f * ((T(1) / a1232) * v12 - (cosine / d32) * v32);
    if (p == 0) return f1;
    if (p == 1) return -(f1 + f3);
    return f3;
}
// a*b - c*d with one rounding (Kahan's difference of products); keeps cross
// products of nearly parallel vectors accurate in FP32
__device__ __forceinline__ float dop(float a, float b, float c, float d) {
    const float w = c * d;
    const float e = fmaf(-c, d, w);
    const float f = fmaf(a, b, -w);
    return f + e;
}
__device__ __forceinline__ V3<float> cross_acc(const V3<float> &a, const V3<float> &b) {
    return mk<float>(dop(a.y, b.z, a.z, b.y), dop(a.z, b.x, a.x, b.z), dop(a.x, b.y, a.y, b.x));
}

// all three forces of one angle term (harmonic or ReB); *c receives the cosine
template <typename T>
__device__ __forceinline__ void angle_forces(const V3<T> &x21, const V3<T> &x32, const GlobP &g, V3<T> F[3], T *c);

// FP32: the angle is atan2(|x21 x x32|, -x21.x32) and t = |x21 x x32|^2
// (Lagrange's identity for the reference's d21*d32 - d2132**2), both free of
// the cancellation that acos and the difference form suffer near 0 and 180
// degrees; the reference's clamps (|cos| <= 1, t >= 1) are kept.
template <>
__device__ __forceinline__ void angle_forces<float>(const V3<float> &x21, const V3<float> &x32, const GlobP &g, V3<float> F[3],
                                                    float *c) {
    const float d21 = dot3(x21, x21), d32 = dot3(x32, x32), d2132 = dot3(x32, x21);
    const V3<float> cr = cross_acc(x21, x32);
    float t = dot3(cr, cr);
    const float cosine = -d2132 * rsqrtf(d21 * d32);
    *c = cosine;
    if (!g.angl_reb) {
        const float delta = atan2f(sqrtf(t), -d2132) - g.f_angl_t0;
        if (t <= 1.f) t = 1.f;
        const float f = g.f_angl_k * delta * rsqrtf(t);
        const V3<float> f21 = f * ((d2132 * rcp_nr(d21)) * x21 - x32);
        const V3<float> f32 = f * ((d2132 * rcp_nr(d32)) * x32 - x21);
        F[0] = -f21;
        F[1] = f21 - f32;
        F[2] = f32;
    } else {
        // v12 = -x21; cos = v12.x32/|v12||x32|; 1 - cos^2 = t/(d12 d32)
        const V3<float> v12 = -x21;
        const float k = g.f_angl_k, co0 = g.f_cos_t0;
        const float ia = rsqrtf(d21 * d32), i21 = rcp_nr(d21), i32 = rcp_nr(d32);
        const float cs = -d2132 * ia;
        const float omc = t * (i21 * i32);
        const float f = -k * (cs - co0) * (1.f - cs * co0) * rcp_nr(omc * omc);
        const V3<float> f1 = f * (ia * x32 - (cs * i21) * v12);
        const V3<float> f3 = f * (ia * v12 - (cs * i32) * x32);
        F[0] = f1;
        F[1] = -(f1 + f3);
        F[2] = f3;
    }
}

template <typename T>
__device__ __forceinline__ void angle_forces(const V3<T> &x21, const V3<T> &x32, const GlobP &g, V3<T> F[3], T *c) {
    // x21 = x2 - x1, x32 = x3 - x2 (FP64: the reference's formulas)
    if (!g.angl_reb) {
        const T d21 = dot3(x21, x21), d32 = dot3(x32, x32), d2132 = dot3(x32, x21);
        T cosine = -d2132 / fm::sqrt(d21 * d32);
        *c = cosine;
        if (fm::fabs(cosine) > T(1)) cosine = fm::copysign(T(1), cosine);
        const T delta = fm::acos(cosine) - pick<T>(g.angl_t0, g.f_angl_t0);
        T t = d21 * d32 - d2132 * d2132;
        if (t <= T(1)) t = T(1);
        const T f = pick<T>(g.angl_k, g.f_angl_k) * delta / fm::sqrt(t);
        const V3<T> f21 = f * ((d2132 / d21) * x21 - x32);
        const V3<T> f32 = f * ((d2132 / d32) * x32 - x21);
        F[0] = -f21;
        F[1] = f21 - f32;
        F[2] = f32;
    } else {
        // v12 = x1 - x2 = -x21, v32 = x3 - x2 = x32
        const V3<T> v12 = -x21;
        const T k = pick<T>(g.angl_k, g.f_angl_k), co0 = pick<T>(g.cos_t0, g.f_cos_t0);
        const T d12 = dot3(v12, v12), d32 = dot3(x32, x32);
        const T a1232 = fm::sqrt(d12 * d32);
        const T cosine = dot3(v12, x32) / a1232;
        *c = cosine;
        const T omc = T(1) - cosine * cosine;
        const T f = -k * (cosine - co0) * (T(1) - cosine * co0) / (omc * omc);
        const V3<T> f1 = f * ((T(1) / a1232) * x32 - (cosine / d12) * v12);
        const V3<T> f3 = f * ((T(1) / a1232) * v12 - (cosine / d32) * x32);
        F[0] = f1;
        F[1] = -(f1 + f3);
        F[2] = f3;
    }
}

// FP32 angle term near 0 or 180 degrees from its cross product
// cr = x21 x x32 accurate to FP32 ulps (cross_fx).  The perpendicular
// vectors of both forms are vector triple products,
//   (d2132/d21) x21 - x32 = (x21 x cr)/d21,  (d2132/d32) x32 - x21 = -(x32 x cr)/d32,
// which cancel nothing, so the forces keep FP32 relative accuracy however
// small the sine.  *sin2 receives |cr|^2 / (d21 d32).
__device__ __forceinline__ void angle_forces_cr(const V3<float> &x21, const V3<float> &x32, const V3<float> &cr, const GlobP &g,
                                                V3<float> F[3], float *sin2) {
    const float d21 = dot3(x21, x21), d32 = dot3(x32, x32), d2132 = dot3(x32, x21);
    float t = dot3(cr, cr);
    *sin2 = t / (d21 * d32);
    const V3<float> p21 = (1.f / d21) * cross3(x21, cr), p32 = (-1.f / d32) * cross3(x32, cr);
    if (!g.angl_reb) {
        const float delta = atan2f(sqrtf(t), -d2132) - g.f_angl_t0;
        if (t <= 1.f) t = 1.f;
        const float f = g.f_angl_k * delta / sqrtf(t);
        const V3<float> f21 = f * p21, f32 = f * p32;
        F[0] = -f21;
        F[1] = f21 - f32;
        F[2] = f32;
    } else {
        const float k = g.f_angl_k, co0 = g.f_cos_t0;
        const float a1232 = sqrtf(d21 * d32);
        const float cs = -d2132 / a1232;
        const float omc = t / (d21 * d32);
        const float f = -k * (cs - co0) * (1.f - cs * co0) / (omc * omc);
        const V3<float> f1 = (-f / a1232) * p21, f3 = (f / a1232) * p32;
        F[0] = f1;
        F[1] = -(f1 + f3);
        F[2] = f3;
    }
}

// energy_angl.F90:18-41 / energy_angl_ReB.F90 with v12 = x1 - x2, v32 = x3 - x2
template <typename T> __device__ __forceinline__ T angle_energy_core(const V3<T> &v12, const V3<T> &v32, const GlobP &g, T *cos_out) {
    T t = dot3(v32, v12) / fm::sqrt(dot3(v12, v12) * dot3(v32, v32));
    *cos_out = t;
    const T k = pick<T>(g.angl_k, g.f_angl_k);
    if (g.angl_reb) {
        const T c0 = pick<T>(g.cos_t0, g.f_cos_t0);
        return T(0.5) * k * ((t - c0) * (t - c0)) / (T(1) - t * t);
    }
    if (t > T(1)) t = T(1);
    else if (t < T(-1)) t = T(-1);
    t = fm::acos(t);
    const T t0 = pick<T>(g.angl_t0, g.f_angl_t0);
    return T(0.5) * k * ((t - t0) * (t - t0));
}

// ---------------------------------------------------------- dihedral
// force_dih_cos.F90:19-60 / force_dih_exp.F90:36-95 with vij = x1 - x2,
// vkj = x3 - x2, vkl = x3 - x4; force on participant p (0..3)
template <typename T>
__device__ __forceinline__ V3<T> dih_force_core(const V3<T> &vij, const V3<T> &vkj, const V3<T> &vkl, int p, const GlobP &g) {
    const V3<T> m = cross3(vij, vkj), n = cross3(vkj, vkl);
    const T akj2 = dot3(vkj, vkj), akj = fm::sqrt(akj2);
    const T dih = fm::atan2(akj * dot3(vij, n), dot3(m, n));
    const T k = pick<T>(g.dih_k, g.f_dih_k), p0 = pick<T>(g.dih_p0, g.f_dih_p0);
    T pre;
    if (g.dih_type == 1) {
        pre = -k * fm::sin(dih + p0) * akj;
    } else {
        const T w = pick<T>(g.dih_w, g.f_dih_w);
        const T dd = dih - p0;
        pre = (k * w) * dd * fm::exp((T(-0.5) * w) * (dd * dd)) * akj;
    }
    const V3<T> fi = (-pre / dot3(m, m)) * m;
    const V3<T> fl = (pre / dot3(n, n)) * n;
    if (p == 0) return fi;
    if (p == 3) return fl;
    const T a = dot3(vij, vkj) / akj2, b = dot3(vkl, vkj) / akj2;
    if (p == 1) return (T(-1) + a) * fi + (-b) * fl;
    return (-a) * fi + (T(-1) + b) * fl;
}
// *near: a flanking bond angle has |cos| > NEAR_ONE (|m| or |n| small)
template <typename T>
__device__ __forceinline__ void dih_forces(const V3<T> &vij, const V3<T> &vkj, const V3<T> &vkl, const GlobP &g, V3<T> F[4],
                                           bool *near) {
    V3<T> m, n;
    if constexpr (sizeof(T) == 4) {
        m = cross_acc(vij, vkj);
        n = cross_acc(vkj, vkl);
    } else {
        m = cross3(vij, vkj);
        n = cross3(vkj, vkl);
    }
    const T akj2 = dot3(vkj, vkj), akj = fm::sqrt(akj2);
    const T s2 = T(1) - T(NEAR_ONE_STRICT) * T(NEAR_ONE_STRICT);
    *near = dot3(m, m) < s2 * dot3(vij, vij) * akj2 || dot3(n, n) < s2 * akj2 * dot3(vkl, vkl);
    const T dih = fm::atan2(akj * dot3(vij, n), dot3(m, n));
    const T k = pick<T>(g.dih_k, g.f_dih_k), p0 = pick<T>(g.dih_p0, g.f_dih_p0);
    T pre;
    if (g.dih_type == 1) {
        pre = -k * fm::sin(dih + p0) * akj;
    } else {
        const T w = pick<T>(g.dih_w, g.f_dih_w);
        const T dd = dih - p0;
        pre = (k * w) * dd * fm::exp((T(-0.5) * w) * (dd * dd)) * akj;
    }
    const V3<T> fi = fm::div(-pre, dot3(m, m)) * m;
    const V3<T> fl = fm::div(pre, dot3(n, n)) * n;
    const T a = fm::div(dot3(vij, vkj), akj2), b = fm::div(dot3(vkl, vkj), akj2);
    F[0] = fi;
    F[1] = (T(-1) + a) * fi + (-b) * fl;
    F[2] = (-a) * fi + (T(-1) + b) * fl;
    F[3] = fl;
}

// FP32 dihedral for a flanking bond angle near 0 or 180 degrees, from
// m = vij x vkj and n = vkj x vkl accurate to FP32 ulps (cross_fx).  The
// sine argument vij.n equals the triple product vkl.m; it is formed with the
// cross product of the straighter flanking angle, since a plain separation
// nearly parallel to vkj would carry its rounding into the other form.
// *sin2 receives the smaller squared sine of the two flanking angles.
__device__ __forceinline__ void dih_forces_mn(const V3<float> &vij, const V3<float> &vkj, const V3<float> &vkl, const V3<float> &m,
                                              const V3<float> &n, const GlobP &g, V3<float> F[4], float *sin2) {
    const float akj2 = dot3(vkj, vkj), akj = sqrtf(akj2);
    const float mm = dot3(m, m), nn = dot3(n, n);
    const float sm = mm / (dot3(vij, vij) * akj2), sn = nn / (akj2 * dot3(vkl, vkl));
    *sin2 = fminf(sm, sn);
    const float y = sm < sn ? dot3(vkl, m) : dot3(vij, n);
    const float dih = atan2f(akj * y, dot3(m, n));
    float pre;
    if (g.dih_type == 1) {
        pre = -g.f_dih_k * sinf(dih + g.f_dih_p0) * akj;
    } else {
        const float w = g.f_dih_w;
        const float dd = dih - g.f_dih_p0;
        pre = (g.f_dih_k * w) * dd * expf((-0.5f * w) * (dd * dd)) * akj;
    }
    const V3<float> fi = (-pre / mm) * m;
    const V3<float> fl = (pre / nn) * n;
    const float a = dot3(vij, vkj) / akj2, b = dot3(vkl, vkj) / akj2;
    F[0] = fi;
    F[1] = (-1.f + a) * fi + (-b) * fl;
    F[2] = (-a) * fi + (-1.f + b) * fl;
    F[3] = fl;
}

// energy_dih_cos.F90:18-39 / energy_dih_exp.F90 (same angle as the force routine)
template <typename T>
__device__ __forceinline__ T dih_energy_core(const V3<T> &vij, const V3<T> &vkj, const V3<T> &vkl, const GlobP &g) {
    const V3<T> m = cross3(vij, vkj), n = cross3(vkj, vkl);
    const T akj = fm::sqrt(dot3(vkj, vkj));
    const T dih = fm::atan2(akj * dot3(vij, n), dot3(m, n));
    const T k = pick<T>(g.dih_k, g.f_dih_k), p0 = pick<T>(g.dih_p0, g.f_dih_p0);
    if (g.dih_type == 1) return k * (T(1) + fm::cos(dih + p0));
    const T w = pick<T>(g.dih_w, g.f_dih_w);
    const T dd = dih - p0;
    return -k * fm::exp((T(-0.5) * w) * (dd * dd));
}

// bonded energies owned by bead i (terms whose first bead is i)
template <typename R>
__device__ void bonded_energy_owned(int i, const int4 &bi, const Pos<R> &P, const double4 *x64, const InstP &ip, const GlobP &g,
                                    double *eb, double *ea, double *ed) {
    const int l = bi_lidx(bi);
    const int n = bi_clen(bi);
    const bool circ = bi_circ(bi);
    *eb = *ea = *ed = 0.0;
    int q[4];
    bool ok = true;
    for (int k = 0; k < 4; ++k) q[k] = chain_bead(bi, l + k);
    if (q[1] >= 0 && (!circ || n >= 2)) *eb = (double)bond_energy<R>(P.d(q[0], q[1], ip), g);
    if (q[1] >= 0 && q[2] >= 0 && (!circ || n >= 3)) {
        R c;
        double e = (double)angle_energy_core<R>(P.d(q[0], q[1], ip), P.d(q[2], q[1], ip), g, &c);
        if (sizeof(R) == 4 && fm::fabs((float)c) > NEAR_ONE) {
            double cd;
            e = angle_energy_core<double>(dvec64(x64[q[0]], x64[q[1]], ip), dvec64(x64[q[2]], x64[q[1]], ip), g, &cd);
        }
        *ea = e;
    }
    for (int k = 0; k < 4; ++k) ok = ok && q[k] >= 0;
    if (g.dih_type != 0 && ok && (!circ || n >= 4))
        *ed = (double)dih_energy_core<R>(P.d(q[0], q[1], ip), P.d(q[2], q[1], ip), P.d(q[2], q[3], ip), g);
}

// -------------------------------------------------------- pair terms
// force_wca.F90:34-67 and force_ele_DH.F90:39-82 folded into one scalar c
// with F_i += c * (x_i - x_j).  The DH force on i is dvdw_dr * (x_i - x_j).
template <typename R>
__device__ __forceinline__ R pair_coef(int e, R d2, R sig2, R wcoef, R ecoef, R rc, R cut2, int mask) {
    R c = R(0);
    if ((e & WCA_BIT) && (mask & 16) && d2 < sig2) {
        const R s = sig2 / d2;
        const R s2 = s * s, s4 = s2 * s2;
        c += wcoef * (s4 * s2 * s - s4);
    }
    if ((e & ELE_BIT) && (mask & 32) && d2 <= cut2) {
        const R r = fm::sqrt(d2);
        const R ri = R(1) / r;
        c += ecoef * ri * ri * (ri + rc) * fm::exp(-r * rc);
    }
    return c;
}
// FP32 variant with a reciprocal square root in place of sqrt and divisions
__device__ __forceinline__ float pair_coef_f(int e, float d2, float sig2, float wcoef, float ecoef, float rc, float cut2, int mask) {
    float c = 0.f;
    const float ri = rsqrtf(d2);
    if ((e & WCA_BIT) && (mask & 16) && d2 < sig2) {
        const float s = sig2 * ri * ri;
        const float s2 = s * s, s4 = s2 * s2;
        c += wcoef * (s4 * s2 * s - s4);
    }
    if ((e & ELE_BIT) && (mask & 32) && d2 <= cut2) {
        const float r = d2 * ri;
        c += ecoef * ri * ri * (ri + rc) * __expf(-r * rc);
    }
    return c;
}
// energy_wca.F90:19-33, energy_ele_DH.F90:20-37 for one (ordered) list entry
template <typename R>
__device__ __forceinline__ void pair_energy(int e, R d2, const InstP &ip, const GlobP &g, double *ew, double *ee) {
    const R d = fm::sqrt(d2);
    if (e & WCA_BIT) {
        const R sg = pick<R>(g.wca_sigma, g.f_wca_sigma);
        if (d < sg) {
            const R s = sg / d;
            const R s6 = s * s * s * s * s * s;
            *ew += (double)(pick<R>(g.wca_eps, g.f_wca_eps) * (s6 * s6 - R(2) * s6 + R(1)));
        }
    }
    if ((e & ELE_BIT) && g.flg_ele) {
        if ((double)d <= ip.ele_cut) {
            const R rc = pick<R>(ip.rcdist, ip.rcdist_f);
            const R coef = pick<R>(ip.ele_coef, ip.ele_coef_f);
            if (g.temp_indep == 0) {
                *ee += (double)(coef / d * fm::exp(-d * rc));
            } else {
                const R rk = d * rc;
                *ee += (double)(coef / d * fm::exp(-rk) * (-(R(1) + R(0.5) * rk) * (R)ip.diele_dTcoef));
            }
        }
    }
}

// ----------------------------------------------------------- base pair
// force_bp.F90:44-204 / force_bp_triplet.F90:62-240 for one record.  Vectors
// v12 = x1-x2, v13 = x1-x3, v15 = x1-x5, v42 = x4-x2, v62 = x6-x2 (bead roles
// 1 imp, 2 jmp, 3 imp-1, 4 jmp-1, 5 imp+1, 6 jmp+1).  Returns false if the
// pair is outside cutoff_ddist.  f[6] receives dU-weighted forces before the
// final multiplication by the energy (as f_bp in the reference); *u_out the
// exponent u; *near is set when an angle cosine is within 1 - NEAR_ONE of +-1
// (FP64 form; the FP32 specialization below uses its own, far tighter, test).
template <typename T, typename P>
__device__ bool bp_force_core(const V3<T> &v12, const V3<T> &v13, const V3<T> &v15, const V3<T> &v42, const V3<T> &v62,
                              const P &b, V3<T> f[6], T *u_out, bool *near) {
    const T d1212 = dot3(v12, v12);
    const T a12 = fm::sqrt(d1212);
    T d = a12 - (T)b.bond_r;
    if (fm::fabs(d) > (T)b.cutoff_ddist) return false;
    *near = false;
    T u = (T)b.bond_k * (d * d);
    V3<T> fi = ((T)2 * (T)b.bond_k * d / a12) * v12, fk, fl;
    f[0] = fi;
    f[1] = -fi;
    const T d1313 = dot3(v13, v13), d4242 = dot3(v42, v42), d1213 = dot3(v12, v13), d1242 = dot3(v12, v42);
    const T d1215 = dot3(v12, v15), d1515 = dot3(v15, v15), d1262 = dot3(v12, v62), d6262 = dot3(v62, v62);
    const T o13 = d1213 / d1212, o42 = d1242 / d1212, o15 = d1215 / d1212, o62 = d1262 / d1212;
    T cosine, pre;
    // 3-1=2 (imp-1 -- imp -- jmp)
    cosine = d1213 / (fm::sqrt(d1313) * a12);
    *near |= fm::fabs((float)cosine) > NEAR_ONE;
    d = fm::acos(cosine) - (T)b.angl_theta[1];
    pre = (T)2 * (T)b.angl_k[1] * d / fm::sqrt(d1313 * d1212 - d1213 * d1213);
    u = u + (T)b.angl_k[1] * (d * d);
    fi = pre * (v12 - (d1213 / d1313) * v13);
    fk = pre * (v13 - o13 * v12);
    f[0] = f[0] - fi - fk;
    f[1] = f[1] + fk;
    f[2] = fi;
    // 1=2-4 (imp -- jmp -- jmp-1)
    cosine = d1242 / (a12 * fm::sqrt(d4242));
    *near |= fm::fabs((float)cosine) > NEAR_ONE;
    d = fm::acos(cosine) - (T)b.angl_theta[0];
    u = u + (T)b.angl_k[0] * (d * d);
    pre = (T)2 * (T)b.angl_k[0] * d / fm::sqrt(d1212 * d4242 - d1242 * d1242);
    fi = -pre * (v42 - o42 * v12);
    fk = -pre * (v12 - (d1242 / d4242) * v42);
    f[0] = f[0] + fi;
    f[1] = f[1] - fi - fk;
    f[3] = fk;
    // 5-1=2 (imp+1 -- imp -- jmp)
    cosine = d1215 / (fm::sqrt(d1515) * a12);
    *near |= fm::fabs((float)cosine) > NEAR_ONE;
    d = fm::acos(cosine) - (T)b.angl_theta[3];
    u = u + (T)b.angl_k[3] * (d * d);
    pre = (T)2 * (T)b.angl_k[3] * d / fm::sqrt(d1515 * d1212 - d1215 * d1215);
    fi = pre * (v12 - (d1215 / d1515) * v15);
    fk = pre * (v15 - o15 * v12);
    f[0] = f[0] - fi - fk;
    f[1] = f[1] + fk;
    f[4] = fi;
    // 1=2-6 (imp -- jmp -- jmp+1)
    cosine = d1262 / (a12 * fm::sqrt(d6262));
    *near |= fm::fabs((float)cosine) > NEAR_ONE;
    d = fm::acos(cosine) - (T)b.angl_theta[2];
    u = u + (T)b.angl_k[2] * (d * d);
    pre = (T)2 * (T)b.angl_k[2] * d / fm::sqrt(d1212 * d6262 - d1262 * d1262);
    fi = -pre * (v62 - o62 * v12);
    fk = -pre * (v12 - (d1262 / d6262) * v62);
    f[0] = f[0] + fi;
    f[1] = f[1] - fi - fk;
    f[5] = fk;
    // dihedral 4-2=1=3
    V3<T> m = cross3(v42, v12), n = cross3(v12, v13);
    T dih = fm::atan2(dot3(v42, n) * a12, dot3(m, n));
    d = dih + (T)b.dihd_phi[0];
    u = u + (T)b.dihd_k[0] * ((T)1 + fm::cos(d));
    pre = -(T)b.dihd_k[0] * fm::sin(d) * a12;
    fi = (pre / dot3(m, m)) * m;
    fl = (-pre / dot3(n, n)) * n;
    f[3] = f[3] + fi;
    f[1] = f[1] + ((T)-1 + o42) * fi - o13 * fl;
    f[0] = f[0] + ((T)-1 + o13) * fl - o42 * fi;
    f[2] = f[2] + fl;
    // dihedral 6-2=1=5
    m = cross3(v62, v12);
    n = cross3(v12, v15);
    dih = fm::atan2(dot3(v62, n) * a12, dot3(m, n));
    d = dih + (T)b.dihd_phi[1];
    u = u + (T)b.dihd_k[1] * ((T)1 + fm::cos(d));
    pre = -(T)b.dihd_k[1] * fm::sin(d) * a12;
    fi = (pre / dot3(m, m)) * m;
    fl = (-pre / dot3(n, n)) * n;
    f[5] = f[5] + fi;
    f[1] = f[1] + ((T)-1 + o62) * fi - o15 * fl;
    f[0] = f[0] + ((T)-1 + o15) * fl - o62 * fi;
    f[4] = f[4] + fl;
    *u_out = u;
    return true;
}

// FP32 form of the same term, free of the cancellation that the acos and
// sqrt(|a|^2 |b|^2 - (a.b)^2) forms suffer near 0 and 180 degrees: each angle
// is atan2(|a x b|, a.b) (Lagrange's identity makes |a x b| the reference's
// square root), and each perpendicular vector a - (a.b / |b|^2) b is formed
// as b x (a x b) / |b|^2 (the vector triple product), which cancels nothing.
// The four cross products v12 x v13, v12 x v15, v42 x v12 and v62 x v12 are
// also the m and n vectors of the two dihedrals, and they alone carry the
// conditioning of the term: both force directions are set by the offsets
// |a| sin(theta).  Without cc they are formed from the FP32 separations,
// whose ~1e-6 A rounding is then amplified by 1/sin(theta), and *near is set
// (nothing else computed) when a bond angle is within 0.03 rad of 0 or 180
// degrees; with cc (cross products from cross_fx, accurate to FP32 ulps)
// only within 1e-6 rad, where the force direction itself is ill-defined.
__device__ __forceinline__ bool bp_force_core_f(const V3<float> &v12, const V3<float> &v13, const V3<float> &v15,
                                                const V3<float> &v42, const V3<float> &v62, const BPPf &b,
                                                const V3<float> *cc, V3<float> f[6], float *u_out, bool *near) {
    const float d1212 = dot3(v12, v12);
    const float a12 = sqrtf(d1212);
    float d = a12 - b.bond_r;
    if (fabsf(d) > b.cutoff_ddist) return false;
    const float d1313 = dot3(v13, v13), d4242 = dot3(v42, v42), d1515 = dot3(v15, v15), d6262 = dot3(v62, v62);
    const V3<float> c13 = cc ? cc[0] : cross_acc(v12, v13), c15 = cc ? cc[1] : cross_acc(v12, v15);
    const V3<float> m42 = cc ? cc[2] : cross_acc(v42, v12), m62 = cc ? cc[3] : cross_acc(v62, v12);
    const float s13 = dot3(c13, c13), s15 = dot3(c15, c15), s42 = dot3(m42, m42), s62 = dot3(m62, m62);
    const float kSin2 = cc ? 1e-12f : 9e-4f;
    *near = s13 < kSin2 * d1212 * d1313 || s15 < kSin2 * d1212 * d1515 || s42 < kSin2 * d1212 * d4242 ||
            s62 < kSin2 * d1212 * d6262;
    if (*near) return true;
    const float d1213 = dot3(v12, v13), d1242 = dot3(v12, v42), d1215 = dot3(v12, v15), d1262 = dot3(v12, v62);
    // quotients as products with reciprocals (rcp_nr, within an ulp or so)
    const float i1212 = rcp_nr(d1212);
    const float o13 = d1213 * i1212, o42 = d1242 * i1212, o15 = d1215 * i1212, o62 = d1262 * i1212;
    float u = b.bond_k * (d * d);
    const V3<float> fb = (2.f * b.bond_k * d * rcp_nr(a12)) * v12;
    V3<float> f0 = fb, f1 = -fb, fi, fk, fl;
    float r, pre;
    // 3-1=2 (imp-1 -- imp -- jmp)
    r = sqrtf(s13);
    d = atan2f(r, d1213) - b.angl_theta[1];
    u += b.angl_k[1] * (d * d);
    pre = 2.f * b.angl_k[1] * d * rcp_nr(r);
    fi = (pre * rcp_nr(d1313)) * cross3(v13, c13);
    fk = (pre * i1212) * cross3(c13, v12);
    f0 = f0 - fi - fk;
    f1 = f1 + fk;
    f[2] = fi;
    // 1=2-4 (imp -- jmp -- jmp-1)
    r = sqrtf(s42);
    d = atan2f(r, d1242) - b.angl_theta[0];
    u += b.angl_k[0] * (d * d);
    pre = 2.f * b.angl_k[0] * d * rcp_nr(r);
    fi = (-pre * i1212) * cross3(v12, m42);
    fk = (-pre * rcp_nr(d4242)) * cross3(m42, v42);
    f0 = f0 + fi;
    f1 = f1 - fi - fk;
    f[3] = fk;
    // 5-1=2 (imp+1 -- imp -- jmp)
    r = sqrtf(s15);
    d = atan2f(r, d1215) - b.angl_theta[3];
    u += b.angl_k[3] * (d * d);
    pre = 2.f * b.angl_k[3] * d * rcp_nr(r);
    fi = (pre * rcp_nr(d1515)) * cross3(v15, c15);
    fk = (pre * i1212) * cross3(c15, v12);
    f0 = f0 - fi - fk;
    f1 = f1 + fk;
    f[4] = fi;
    // 1=2-6 (imp -- jmp -- jmp+1)
    r = sqrtf(s62);
    d = atan2f(r, d1262) - b.angl_theta[2];
    u += b.angl_k[2] * (d * d);
    pre = 2.f * b.angl_k[2] * d * rcp_nr(r);
    fi = (-pre * i1212) * cross3(v12, m62);
    fk = (-pre * rcp_nr(d6262)) * cross3(m62, v62);
    f0 = f0 + fi;
    f1 = f1 - fi - fk;
    f[5] = fk;
    // dihedral 4-2=1=3: m = v42 x v12, n = v12 x v13
    float sn, cs;
    d = atan2f(dot3(v42, c13) * a12, dot3(m42, c13)) + b.dihd_phi[0];
    __sincosf(d, &sn, &cs); // the fast intrinsic: absolute error of order 1e-6 on this range
    u += b.dihd_k[0] * (1.f + cs);
    pre = -b.dihd_k[0] * sn * a12;
    fi = (pre * rcp_nr(s42)) * m42;
    fl = (-pre * rcp_nr(s13)) * c13;
    f[3] = f[3] + fi;
    f1 = f1 + (o42 - 1.f) * fi - o13 * fl;
    f0 = f0 + (o13 - 1.f) * fl - o42 * fi;
    f[2] = f[2] + fl;
    // dihedral 6-2=1=5: m = v62 x v12, n = v12 x v15
    d = atan2f(dot3(v62, c15) * a12, dot3(m62, c15)) + b.dihd_phi[1];
    __sincosf(d, &sn, &cs); // the fast intrinsic: absolute error of order 1e-6 on this range
    u += b.dihd_k[1] * (1.f + cs);
    pre = -b.dihd_k[1] * sn * a12;
    fi = (pre * rcp_nr(s62)) * m62;
    fl = (-pre * rcp_nr(s15)) * c15;
    f[5] = f[5] + fi;
    f1 = f1 + (o62 - 1.f) * fi - o15 * fl;
    f0 = f0 + (o15 - 1.f) * fl - o62 * fi;
    f[4] = f[4] + fl;
    f[0] = f0;
    f[1] = f1;
    *u_out = u;
    return true;
}

// energy_bp.F90 mp_angle (clamped) and mp_dihedral
template <typename T> __device__ __forceinline__ T mp_angle(const V3<T> &v12, const V3<T> &v32) {
    T co = dot3(v32, v12) / fm::sqrt(dot3(v12, v12) * dot3(v32, v32));
    if (co > T(1)) co = T(1);
    else if (co < T(-1)) co = T(-1);
    return fm::acos(co);
}
template <typename T> __device__ __forceinline__ T mp_dihedral(const V3<T> &v12, const V3<T> &v32, const V3<T> &v34) {
    const V3<T> m = cross3(v12, v32), n = cross3(v32, v34);
    return fm::atan2(dot3(v12, n) * fm::sqrt(dot3(v32, v32)), dot3(m, n));
}

} // namespace sisg
