// Device helpers of the neighbour-list rebuild shared by the cooperative
// trigger/rebuild kernel (lists.cu) and the per-block MD kernel of small
// instances (kernels.cu k_md_small): pbc_wrap, the exact FP64 membership
// test of one pair with its list flags and base-pair candidate rules
// (neighbor_list.F90:99-229, init_bp.F90:184-313), the per-bead list append,
// and the conversion of per-bead lists to cluster-pair lists.
#pragma once

#include "common.cuh"

namespace sisg {

__device__ __forceinline__ double wrap1(double x, double L) {
    // pbc_wrap: x - L*(int((x-L)/L)+1) above the box, x + L*(int((0-x)/L)+1) below
    if (x > L) return __dsub_rn(x, __dmul_rn(L, (double)((int)__ddiv_rn(__dsub_rn(x, L), L) + 1)));
    if (x < 0.0) return __dadd_rn(x, __dmul_rn(L, (double)((int)__ddiv_rn(__dsub_rn(0.0, x), L) + 1)));
    return x;
}
__device__ __forceinline__ double4 wrap_pos(const double4 &x, const InstP &ip) {
    if (!ip.pbc) return x;
    return make_double4(wrap1(x.x, ip.box[0]), wrap1(x.y, ip.box[1]), wrap1(x.z, ip.box[2]), x.w);
}
// d2 = dot_product(v,v) of v = pbc_vec_d(x_lo, x_hi), unfused
__device__ __forceinline__ double exact_d2(const double4 &a, const double4 &b, const InstP &ip) {
    const V3<double> v = dvec64(a, b, ip);
    return __dadd_rn(__dadd_rn(__dmul_rn(v.x, v.x), __dmul_rn(v.y, v.y)), __dmul_rn(v.z, v.z));
}

__device__ __forceinline__ bool is_complement(int s1, int s2) {
    // const_idx.F90 is_complement: A-U, U-A, U-G, G-C, G-U, C-G
    return (s1 == 0 && s2 == 1) || (s1 == 1 && (s2 == 0 || s2 == 2)) || (s1 == 2 && (s2 == 3 || s2 == 1)) ||
           (s1 == 3 && s2 == 2);
}
__device__ __forceinline__ int bp3_key(int w, int x, int u, int z, int y, int v) {
    // init_bp.F90:352-378 bp3_hash_key
    if (x < y) return 1 + w + x * 4 + u * 16 + z * 64 + y * 256 + v * 1024;
    return 1 + v + y * 4 + z * 16 + u * 64 + x * 256 + w * 1024;
}

// init_bp.F90:184-313 for the pair lo < hi (global indices, same instance).
// Returns bp3 (0: not a candidate) and the pair type.
static __device__ __forceinline__ int bp_candidate(const Dev &D, const GlobP &g, const int4 &bl, const int4 &bh, int *type_out) {
    *type_out = 0;
    const int model = g.bp_model;
    const int i = bi_lidx(bl) + 1, j = bi_lidx(bh) + 1;
    const int ni = bi_clen(bl), nj = bi_clen(bh);
    const bool ic = bi_circ(bl), jc = bi_circ(bh);
    const bool same = bi_cstart(bl) == bi_cstart(bh);
    int i_pre = i - 1, i_nxt = i + 1, j_pre = j - 1, j_nxt = j + 1;
    if (ic) {
        if (i == 1) i_pre = ni;
        if (i == ni) i_nxt = 1;
    } else if (i == 1 || i == ni) {
        return 0;
    }
    if (jc) {
        if (j == 1) j_pre = nj;
        if (j == nj) j_nxt = 1;
    } else if (j == 1 || j == nj) {
        return 0;
    }
    if (same) {
        if (i + g.bp_min_loop >= j) return 0;
        if (ic && j + g.bp_min_loop >= i + ni) return 0;
    }
    const int si = bi_seq(bl), sj = bi_seq(bh);
    int type = 0;
    if (si == 2 && sj == 3) type = 1;      // GC
    else if (si == 3 && sj == 2) type = 4; // CG
    else if (si == 0 && sj == 1) type = 2; // AU
    else if (si == 1 && sj == 0) type = 5; // UA
    else if (si == 2 && sj == 1) type = 3; // GU
    else if (si == 1 && sj == 2) type = 6; // UG
    if (model != 5 && type == 0) return 0;
    auto sq = [&](const int4 &b, int l) { return bi_seq(D.binfo[bi_cstart(b) + l - 1]); };
    const int s_ipre = sq(bl, i_pre), s_inxt = sq(bl, i_nxt), s_jpre = sq(bh, j_pre), s_jnxt = sq(bh, j_nxt);
    bool pair_ipre_jnxt = is_complement(s_ipre, s_jnxt);
    bool pair_inxt_jpre = is_complement(s_inxt, s_jpre);
    if (!ic && i_pre == 1) pair_ipre_jnxt = false;
    if (!jc && j_nxt == nj) pair_ipre_jnxt = false;
    if (!ic && i_nxt == ni) pair_inxt_jpre = false;
    if (!jc && j_pre == 1) pair_inxt_jpre = false;
    if (same) {
        if (i + 1 + g.bp_min_loop >= j - 1) pair_inxt_jpre = false;
        if (ic && j + 1 + g.bp_min_loop >= i - 1 + ni) pair_ipre_jnxt = false;
    }
    if ((model == 3 || model == 4 || model == 5) && !pair_ipre_jnxt && !pair_inxt_jpre) return 0;
    *type_out = type;
    if (model == 5) {
        int key;
        if (!pair_ipre_jnxt) key = bp3_key(1, si, s_inxt, 1, sj, s_jpre);
        else if (!pair_inxt_jpre) key = bp3_key(s_ipre, si, 1, s_jnxt, sj, 1);
        else key = bp3_key(s_ipre, si, s_inxt, s_jnxt, sj, s_jpre);
        return D.bp3_hash[key];
    }
    return type;
}

// list flags of pair (lo, hi) at squared distance d2 (neighbor_list.F90:99-229)
__device__ __forceinline__ int pair_flags(const GlobP &g, const InstP &ip, const int4 &bl, const int4 &bh, double d2) {
    const int i = bi_lidx(bl) + 1, j = bi_lidx(bh) + 1;
    const bool same = bi_cstart(bl) == bi_cstart(bh);
    const int n = bi_clen(bl);
    int f = 0;
    if (bi_seq(bl) != 4 && bi_seq(bh) != 4 && d2 <= ip.wca_nl_cut2) {
        bool add = true;
        if (same) {
            if (i + 2 >= j) add = false;
            else if (bi_circ(bl) && j + 2 >= i + n) add = false;
        }
        if (add) f |= WCA_BIT;
    }
    if (g.flg_ele && d2 <= ip.ele_nl_cut2 && bi_charge(bl) && bi_charge(bh)) {
        bool add = true;
        if (same) {
            const int eb = g.ele_excl_bond, ea = g.ele_excl_angle;
            if (j == i + 1 && eb) add = false;
            if (j == i + 2 && ea) add = false;
            if (bi_circ(bl)) {
                if (i == 1) {
                    if (j == n && eb) add = false;
                    if (j == n - 1 && ea) add = false;
                } else if (i == 2) {
                    if (j == n && ea) add = false;
                }
            }
        }
        if (add) f |= ELE_BIT;
    }
    return f;
}

// Tests bead gi against candidate gj and appends the results.  Returns the
// list flag word (0 if not listed).
// Tests bead gi against candidate gj and appends base-pair records.  Returns
// the list flag word (0 if not listed).  Membership is decided from the
// float distance when it lies outside a 1e-4 relative band around every
// cutoff (its error is below 1e-6 relative); inside the band the squared
// distance is recomputed exactly as the reference computes it (FP64, wrapped
// coordinates, lower index first, unfused).
// appends the base-pair record of pair (gi < gj) when it is a candidate
// (init_bp.F90:184-313): beads, neighbours (i-1, j-1, i+1, j+1), type and
// nearest-neighbour hash
__device__ __forceinline__ void bp_append(const Dev &D, const GlobP &g, const InstP &ip, int gi, int gj, const int4 &bl,
                                          const int4 &bh, int inst) {
    int type;
    const int bp3 = bp_candidate(D, g, bl, bh, &type);
    if (bp3 <= 0) return;
    const int slot = atomicAdd(&D.bp_cnt[inst], 1);
    if (slot < ip.bp_cap) {
        const int i = bi_lidx(bl) + 1, j = bi_lidx(bh) + 1;
        const int ni = bi_clen(bl), nj = bi_clen(bh);
        const int i3 = (i == 1) ? gi + ni - 1 : gi - 1;
        const int j4 = (j == 1) ? gj + nj - 1 : gj - 1;
        const int i5 = (i == ni) ? gi + 1 - ni : gi + 1;
        const int jend = g.bp_jnext_compat ? ni : nj; // neighbor_list.F90:212
        int j6 = (j == jend) ? gj + 1 - nj : gj + 1;
        if (j6 < ip.bead_off || j6 >= ip.bead_off + ip.n) {
            atomicOr(D.err, ERR_BP_OVERFLOW);
            j6 = gj + 1;
        }
        D.bps[ip.bp_off + slot] = make_int4(gi, gj, type | (bp3 << 8), inst);
        D.bps_n[ip.bp_off + slot] = make_int4(i3, j4, i5, j6);
    } else {
        atomicOr(D.err, ERR_BP_OVERFLOW);
        atomicMax(&D.max_need[1], slot + 1);
    }
}

__device__ __forceinline__ bool near_cut(float d2f, double c2) {
    const float c = (float)c2;
    return d2f > c * 0.9999f && d2f < c * 1.0001f;
}
__device__ __forceinline__ int test_pair(const Dev &D, const GlobP &g, const InstP &ip, int cur, int gi, const int4 &bii,
                                         const uint4 &mi, const double4 &xi_w, int gj, float maxcut2f, int inst) {
    const uint4 mj = mir_at(D, cur)[gj];
    const V3<float> vf = dvec32(mi, mj, ip);
    const float d2f = vf.x * vf.x + vf.y * vf.y + vf.z * vf.z;
    if (!(d2f <= maxcut2f)) return 0;
    const int4 bij = D.binfo[gj];
    const bool ilo = gi < gj;
    double d2 = (double)d2f;
    if (near_cut(d2f, ip.wca_nl_cut2) || near_cut(d2f, ip.ele_nl_cut2) || near_cut(d2f, ip.bp_nl_cut2)) {
        const double4 xj_w = wrap_pos(x_at(D, cur)[gj], ip);
        d2 = ilo ? exact_d2(xi_w, xj_w, ip) : exact_d2(xj_w, xi_w, ip);
    }
    const int4 &bl = ilo ? bii : bij;
    const int4 &bh = ilo ? bij : bii;
    const int f = pair_flags(g, ip, bl, bh, d2);
    // an instance with a given secondary structure takes its base-pair
    // records from ss_records instead
    if (ilo && g.bp_model > 0 && !ip.ss_on && d2 <= ip.bp_nl_cut2) bp_append(D, g, ip, gi, gj, bl, bh, inst);
    return f;
}

// squared list cutoff of the instance's spatial scan (float, with slack):
// base-pair candidates of an instance with a secondary structure come from
// its partner table, so their cutoff does not widen the scan
__device__ __forceinline__ float scan_cut2f(const InstP &ip, float slack) {
    const double c = fmax(ip.wca_nl_cut2, ip.ele_nl_cut2);
    return (float)(ip.ss_on ? c : fmax(c, ip.bp_nl_cut2)) * slack;
}

// The base-pair records of bead gi (lower index of each pair) of an instance
// with a secondary structure: its allowed partners above it, at any place in
// the box, within the base-pair list cutoff (neighbor_list.F90:159-229 with
// bp_map of read_ss.F90; with [Bias_SS] the cutoff is 1e10 A^2, :89-93).
// Positions are wrapped here as the rebuild wraps them (wrapping is
// idempotent, so a position another thread already wrapped reads the same).
__device__ __forceinline__ void ss_records(const Dev &D, const GlobP &g, int cur, int gi, int inst) {
    const InstP &ip = D.ip[inst];
    const double4 xi = wrap_pos(x_at(D, cur)[gi], ip);
    const int4 bi = D.binfo[gi];
    for (int k = D.ss_start[gi]; k < D.ss_start[gi + 1]; ++k) {
        const int gj = D.ss_part[k];
        if (gj <= gi) continue;
        const double4 xj = wrap_pos(x_at(D, cur)[gj], ip);
        if (exact_d2(xi, xj, ip) <= ip.bp_nl_cut2) bp_append(D, g, ip, gi, gj, bi, D.binfo[gj], inst);
    }
}

// appends one warp-chunk of results to bead gi's list
__device__ __forceinline__ void warp_append(const Dev &D, const GlobP &g, int gi, int lane, int f, int gj, int &count) {
    const unsigned bal = __ballot_sync(0xffffffffu, f != 0);
    if (f) {
        const int pos = count + __popc(bal & ((1u << lane) - 1u));
        if (pos < g.cap) D.nbr[(size_t)gi * g.cap + pos] = gj | f;
    }
    count += __popc(bal);
}

__device__ __forceinline__ void bead_begin(const Dev &D, int cur, int gi, const InstP &ip, int lane, double4 &xi_w) {
    xi_w = wrap_pos(x_at(D, cur)[gi], ip);
    if (lane == 0) {
        // one count per rebuild of the instance (its first bead)
        if (D.lgen && gi == ip.bead_off) atomicAdd(D.lgen + D.binfo[gi].x, 1);
        if (ip.pbc) x_at(D, cur)[gi] = xi_w;
        D.move[gi] = make_double4(0.0, 0.0, 0.0, 0.0);
        // the mirror is the same before and after the wrap (the box is 2^32 units)
        if (D.mir0) D.mir0[gi] = mir_at(D, cur)[gi];
    }
}
__device__ __forceinline__ void bead_end(const Dev &D, const GlobP &g, int gi, int lane, int count) {
    if (lane == 0) {
        D.nnbr[gi] = count;
        if (count > g.cap) {
            atomicOr(D.err, ERR_PAIR_OVERFLOW);
            atomicMax(&D.max_need[0], count);
        }
    }
}

__device__ __forceinline__ unsigned cl_hash(int J) { return ((unsigned)J * 2654435761u) >> 23; } // 9 bits: kClHash
__device__ __forceinline__ int cl_find(const int *key, int J) {
    unsigned h = cl_hash(J);
    for (int p = 0; p < kClHash; ++p) {
        if (key[h] == J) return (int)h;
        h = (h + 1) & (kClHash - 1);
    }
    return -1;
}
// The cluster-pair list of i-cluster ic (one warp; key and rank: the warp's
// 2 * kClHash ints of shared memory).
static __device__ void cluster_one(const Dev &D, const GlobP &g, int ic, int *key, int *rank) {
    const int lane = threadIdx.x & 31;
    const int first = D.cl_first[ic];
    const InstP &ip = D.ip[D.binfo[first].x];
    const int cnt = min(kCl, ip.bead_off + ip.n - first);
    for (int h = lane; h < kClHash; h += 32) key[h] = -1;
    __syncwarp();
    // distinct clusters of the entries (the table holds at most kClHash)
    int full = 0;
    for (int a = 0; a < cnt; ++a) {
        const int gi = first + a;
        const int m = min(__ldcg(D.nnbr + gi), g.cap);
        const int *nb = D.nbr + (size_t)gi * g.cap;
        for (int k = lane; k < m; k += 32) {
            const int J = ((__ldcg(nb + k) & IDX_MASK) - ip.bead_off) / kCl;
            unsigned h = cl_hash(J);
            int p = 0;
            for (; p < kClHash; ++p) {
                const int old = atomicCAS(&key[h], -1, J);
                if (old == -1 || old == J) break;
                h = (h + 1) & (kClHash - 1);
            }
            full |= p == kClHash;
        }
    }
    __syncwarp();
    int nu = 0;
    for (int h0 = 0; h0 < kClHash; h0 += 32) nu += __popc(__ballot_sync(0xffffffffu, key[h0 + lane] >= 0));
    full = __any_sync(0xffffffffu, full);
    const size_t base = (size_t)ic * g.ccap;
    if (full || nu > g.ccap) {
        if (lane == 0) D.ncl[ic] = -1;
        __syncwarp();
        return;
    }
    // rank of every distinct cluster: the number of smaller ones
    for (int h = lane; h < kClHash; h += 32) {
        const int v = key[h];
        if (v < 0) continue;
        int r = 0;
        for (int q = 0; q < kClHash; ++q) {
            const int w = key[q];
            r += w >= 0 && w < v;
        }
        rank[h] = r;
        D.cl_j[base + r] = ip.bead_off + v * kCl;
        D.cl_m[base + r] = make_ulonglong2(0ull, 0ull);
    }
    __syncwarp();
    for (int a = 0; a < cnt; ++a) {
        const int gi = first + a;
        const int m = min(__ldcg(D.nnbr + gi), g.cap);
        const int *nb = D.nbr + (size_t)gi * g.cap;
        for (int k = lane; k < m; k += 32) {
            const int e = __ldcg(nb + k);
            const int jl = (e & IDX_MASK) - ip.bead_off;
            const int h = cl_find(key, jl / kCl);
            if (h < 0) continue; // not reached: every cluster was inserted
            const unsigned long long bit = 1ull << (a * kCl + jl % kCl);
            ulonglong2 *dst = D.cl_m + base + rank[h];
            if (e & WCA_BIT) atomicOr(&dst->x, bit);
            if (e & ELE_BIT) atomicOr(&dst->y, bit);
        }
    }
    if (lane == 0) D.ncl[ic] = nu;
    __syncwarp();
}

} // namespace sisg
