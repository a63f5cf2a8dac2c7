// Neighbour-list rebuild of libsisgpu: neighbor_list.F90:1-233 and
// pbc_wrap (pbc.F90:196-226) for the instances whose displacement trigger
// fired (flag[inst] != 0).  Every kernel returns at once when no instance is
// flagged, so the rebuild can be enqueued after every step.
//
// Membership is decided exactly as the reference decides it: the squared
// distance of the pair (lower global index first, pbc_vec_d single shift) is
// evaluated in FP64 without fused multiply-adds and compared with the
// reference's FP64 cutoffs.  A float prefilter on the fixed-point mirror skips
// the FP64 work for pairs that are far outside every cutoff; its relative
// error (< 1e-6) is far inside the prefilter's 1e-3 margin.
//
// Small instances (n <= kAllPairsMax, or PBC boxes with fewer than three
// cells per side) scan all bead pairs of the instance; large PBC instances
// bin beads into cells at least as wide as the largest list cutoff and scan
// the 27 neighbouring cells.
#include "common.cuh"
#include "kernels.h"

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
__device__ int bp_candidate(const Dev &D, const GlobP &g, const int4 &bl, const int4 &bh, int *type_out) {
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
__device__ __forceinline__ bool near_cut(float d2f, double c2) {
    const float c = (float)c2;
    return d2f > c * 0.9999f && d2f < c * 1.0001f;
}
__device__ __forceinline__ int test_pair(const Dev &D, const GlobP &g, const InstP &ip, int cur, int gi, const int4 &bii,
                                         const uint4 &mi, const double4 &xi_w, int gj, float maxcut2f, int inst) {
    const uint4 mj = D.mir[cur][gj];
    const V3<float> vf = dvec32(mi, mj, ip);
    const float d2f = vf.x * vf.x + vf.y * vf.y + vf.z * vf.z;
    if (!(d2f <= maxcut2f)) return 0;
    const int4 bij = D.binfo[gj];
    const bool ilo = gi < gj;
    double d2 = (double)d2f;
    if (near_cut(d2f, ip.wca_nl_cut2) || near_cut(d2f, ip.ele_nl_cut2) || near_cut(d2f, ip.bp_nl_cut2)) {
        const double4 xj_w = wrap_pos(D.x[cur][gj], ip);
        d2 = ilo ? exact_d2(xi_w, xj_w, ip) : exact_d2(xj_w, xi_w, ip);
    }
    const int4 &bl = ilo ? bii : bij;
    const int4 &bh = ilo ? bij : bii;
    const int f = pair_flags(g, ip, bl, bh, d2);
    if (ilo && g.bp_model > 0 && d2 <= ip.bp_nl_cut2) {
        int type;
        const int bp3 = bp_candidate(D, g, bl, bh, &type);
        if (bp3 > 0) {
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
    }
    return f;
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
    xi_w = wrap_pos(D.x[cur][gi], ip);
    if (lane == 0) {
        if (ip.pbc) D.x[cur][gi] = xi_w;
        D.move[gi] = make_double4(0.0, 0.0, 0.0, 0.0);
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

// --------------------------------------------------- all-pairs (small)
// items: (instance, first local bead); 32 beads per item, one warp per bead.
__global__ void __launch_bounds__(256) k_rebuild_small(Dev D, GlobP g, int cur, const int2 *items, int n_items, float slack) {
    if (*(volatile int *)D.any == 0) return;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int it = blockIdx.x; it < n_items; it += gridDim.x) {
        const int2 item = items[it];
        const int inst = item.x;
        if (D.flag[inst] == 0) continue;
        const InstP &ip = D.ip[inst];
        const float maxcut2f = (float)fmax(fmax(ip.wca_nl_cut2, ip.ele_nl_cut2), ip.bp_nl_cut2) * slack;
        for (int li = item.y + warp; li < min(item.y + 32, ip.n); li += 8) {
            const int gi = ip.bead_off + li;
            double4 xi_w;
            bead_begin(D, cur, gi, ip, lane, xi_w);
            const int4 bii = D.binfo[gi];
            const uint4 mi = D.mir[cur][gi];
            int count = 0;
            for (int jb = 0; jb < ip.n; jb += 32) {
                const int lj = jb + lane;
                int f = 0;
                const int gj = ip.bead_off + lj;
                if (lj < ip.n && lj != li) f = test_pair(D, g, ip, cur, gi, bii, mi, xi_w, gj, maxcut2f, inst);
                warp_append(D, g, gi, lane, f, gj, count);
            }
            bead_end(D, g, gi, lane, count);
        }
    }
}

// ------------------------------------------------------- cell list (large)
__device__ __forceinline__ int cell_of(const double4 &xw, const InstP &ip) {
    int c[3];
    const double xs[3] = {xw.x, xw.y, xw.z};
    for (int k = 0; k < 3; ++k) {
        int q = (int)floor(xs[k] / ip.cell_len[k]);
        q = q < 0 ? 0 : (q >= ip.nc[k] ? ip.nc[k] - 1 : q);
        c[k] = q;
    }
    return ip.cell_base + (c[2] * ip.nc[1] + c[1]) * ip.nc[0] + c[0];
}

// bead ranges of large instances: litems = (instance, first local bead), 256 beads each
__global__ void k_cell_bin(Dev D, GlobP g, int cur, const int2 *litems, int n_litems) {
    if (*(volatile int *)D.any == 0) return;
    for (int it = blockIdx.x; it < n_litems; it += gridDim.x) {
        const int2 item = litems[it];
        if (D.flag[item.x] == 0) continue;
        const InstP &ip = D.ip[item.x];
        const int li = item.y + threadIdx.x;
        if (li >= ip.n) continue;
        const int gi = ip.bead_off + li;
        const double4 xw = wrap_pos(D.x[cur][gi], ip);
        const int c = cell_of(xw, ip);
        D.bead_cell[gi] = c;
        atomicAdd(&D.cell_cnt[c], 1);
    }
}

// exclusive scan of cell counts (one block, coalesced tiles of 4096 cells);
// counts are reset to serve as fill cursors
__global__ void __launch_bounds__(1024) k_cell_scan(Dev D) {
    if (*(volatile int *)D.any == 0) return;
    __shared__ int s_warp[32];
    __shared__ int s_carry;
    const int n = D.n_cells;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (threadIdx.x == 0) s_carry = 0;
    __syncthreads();
    for (int base = 0; base < n; base += 4096) {
        const int c0 = base + 4 * threadIdx.x;
        int v[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) v[q] = c0 + q < n ? D.cell_cnt[c0 + q] : 0;
        const int tsum = v[0] + v[1] + v[2] + v[3];
        int incl = tsum;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += y;
        }
        if (lane == 31) s_warp[warp] = incl;
        __syncthreads();
        if (warp == 0) {
            int w = s_warp[lane];
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int y = __shfl_up_sync(0xffffffffu, w, o);
                if (lane >= o) w += y;
            }
            s_warp[lane] = w;
        }
        __syncthreads();
        int run = s_carry + (warp ? s_warp[warp - 1] : 0) + incl - tsum;
#pragma unroll
        for (int q = 0; q < 4; ++q)
            if (c0 + q < n) {
                D.cell_start[c0 + q] = run;
                D.cell_cnt[c0 + q] = 0;
                run += v[q];
            }
        __syncthreads();
        if (threadIdx.x == 1023) s_carry += s_warp[31];
        __syncthreads();
    }
    if (threadIdx.x == 0) D.cell_start[n] = s_carry;
}

__global__ void k_cell_fill(Dev D, GlobP g, const int2 *litems, int n_litems) {
    if (*(volatile int *)D.any == 0) return;
    for (int it = blockIdx.x; it < n_litems; it += gridDim.x) {
        const int2 item = litems[it];
        if (D.flag[item.x] == 0) continue;
        const InstP &ip = D.ip[item.x];
        const int li = item.y + threadIdx.x;
        if (li >= ip.n) continue;
        const int gi = ip.bead_off + li;
        const int c = D.bead_cell[gi];
        const int pos = D.cell_start[c] + atomicAdd(&D.cell_cnt[c], 1);
        D.cell_beads[pos] = gi;
    }
}

// sorts every cell's beads by index so that list order is deterministic:
// one warp per cell ranks up to 256 beads in shared memory (rank = number of
// smaller indices; indices are distinct); larger cells are insertion-sorted
__global__ void __launch_bounds__(256) k_cell_sort(Dev D) {
    if (*(volatile int *)D.any == 0) return;
    constexpr int kCap = 256;
    __shared__ int sb[8][kCap];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int nwarps = gridDim.x * 8;
    for (int c = blockIdx.x * 8 + warp; c < D.n_cells; c += nwarps) {
        const int a = D.cell_start[c], b = D.cell_start[c + 1], m = b - a;
        if (m <= 1) continue;
        if (m <= kCap) {
            for (int k = lane; k < m; k += 32) sb[warp][k] = D.cell_beads[a + k];
            __syncwarp();
            for (int k = lane; k < m; k += 32) {
                const int v = sb[warp][k];
                int r = 0;
                for (int q = 0; q < m; ++q) r += sb[warp][q] < v;
                D.cell_beads[a + r] = v;
            }
            __syncwarp();
        } else if (lane == 0) {
            for (int k = a + 1; k < b; ++k) {
                const int v = D.cell_beads[k];
                int q = k - 1;
                while (q >= a && D.cell_beads[q] > v) {
                    D.cell_beads[q + 1] = D.cell_beads[q];
                    --q;
                }
                D.cell_beads[q + 1] = v;
            }
        }
    }
}

// one warp per bead: the 27 neighbouring cells' beads as candidates
__global__ void __launch_bounds__(256) k_cell_search(Dev D, GlobP g, int cur, const int2 *litems, int n_litems, float slack) {
    if (*(volatile int *)D.any == 0) return;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    // each litem covers 256 beads; 8 warps stride over them
    for (int it = blockIdx.x; it < n_litems; it += gridDim.x) {
        const int2 item = litems[it];
        const int inst = item.x;
        if (D.flag[inst] == 0) continue;
        const InstP &ip = D.ip[inst];
        const float maxcut2f = (float)fmax(fmax(ip.wca_nl_cut2, ip.ele_nl_cut2), ip.bp_nl_cut2) * slack;
        for (int li = item.y + warp; li < min(item.y + 256, ip.n); li += 8) {
            const int gi = ip.bead_off + li;
            double4 xi_w;
            bead_begin(D, cur, gi, ip, lane, xi_w);
            const int4 bii = D.binfo[gi];
            const uint4 mi = D.mir[cur][gi];
            const int c0 = D.bead_cell[gi] - ip.cell_base;
            const int cx = c0 % ip.nc[0], cy = (c0 / ip.nc[0]) % ip.nc[1], cz = c0 / (ip.nc[0] * ip.nc[1]);
            // lane q < 27 owns neighbour cell q; a warp prefix over their
            // counts flattens the 27 ranges into one candidate sequence that
            // every pass consumes 32 at a time (cell order, then bead order)
            int cstart = 0, ccnt = 0;
            if (lane < 27) {
                int qx = cx + lane % 3 - 1, qy = cy + (lane / 3) % 3 - 1, qz = cz + lane / 9 - 1;
                qx = qx < 0 ? qx + ip.nc[0] : (qx >= ip.nc[0] ? qx - ip.nc[0] : qx);
                qy = qy < 0 ? qy + ip.nc[1] : (qy >= ip.nc[1] ? qy - ip.nc[1] : qy);
                qz = qz < 0 ? qz + ip.nc[2] : (qz >= ip.nc[2] ? qz - ip.nc[2] : qz);
                const int c = ip.cell_base + (qz * ip.nc[1] + qy) * ip.nc[0] + qx;
                cstart = D.cell_start[c];
                ccnt = D.cell_start[c + 1] - cstart;
            }
            int incl = ccnt;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int y = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= o) incl += y;
            }
            const int excl = incl - ccnt;
            const int total = __shfl_sync(0xffffffffu, incl, 31);
            int count = 0;
            for (int k0 = 0; k0 < total; k0 += 32) {
                const int k = k0 + lane, kk = min(k, total - 1);
                // owning cell of candidate kk: the last q <= 26 with excl[q] <= kk
                // (that cell is non-empty); every lane runs the same shuffles
                int lo = 0;
#pragma unroll
                for (int step = 16; step > 0; step >>= 1) {
                    const int e = __shfl_sync(0xffffffffu, excl, min(lo + step, 26));
                    if (lo + step <= 26 && e <= kk) lo += step;
                }
                const int cs = __shfl_sync(0xffffffffu, cstart, lo), ce = __shfl_sync(0xffffffffu, excl, lo);
                int f = 0, gj = -1;
                if (k < total) {
                    gj = D.cell_beads[cs + (k - ce)];
                    if (gj != gi) f = test_pair(D, g, ip, cur, gi, bii, mi, xi_w, gj, maxcut2f, inst);
                }
                warp_append(D, g, gi, lane, f, gj, count);
            }
            bead_end(D, g, gi, lane, count);
        }
    }
}

// ------------------------------------------------------------ finish
// One block: base-pair prefix counts, rebuild bookkeeping, reset of flags
// and cell counters.
__global__ void __launch_bounds__(1024) k_rebuild_finish(Dev D, GlobP g, int in_graph) {
    if (*(volatile int *)D.any == 0) return;
    __shared__ int s[1024];
    const int n = g.n_inst;
    const int per = (n + 1023) / 1024;
    const int lo = min(n, (int)threadIdx.x * per), hi = min(n, lo + per);
    int sum = 0, nflag = 0;
    for (int k = lo; k < hi; ++k) {
        const int c = min(D.bp_cnt[k], D.ip[k].bp_cap);
        sum += c;
        nflag += D.flag[k] != 0;
    }
    s[threadIdx.x] = sum;
    __syncthreads();
    for (int o = 1; o < 1024; o <<= 1) {
        const int v = threadIdx.x >= (unsigned)o ? s[threadIdx.x - o] : 0;
        __syncthreads();
        s[threadIdx.x] += v;
        __syncthreads();
    }
    int run = s[threadIdx.x] - sum;
    for (int k = lo; k < hi; ++k) {
        D.bp_cnt[n + k] = run;
        run += min(D.bp_cnt[k], D.ip[k].bp_cap);
        // new records: the next evaluation runs the Monte Carlo pass (job_md.F90:392-394)
        if (D.flag[k] && g.nstep_mc > 0) D.mc_due[k] = 1;
        D.flag[k] = 0;
    }
    if (threadIdx.x == 1023) *D.bp_total = s[1023];
    if (nflag) atomicAdd((unsigned long long *)D.rebuilds, (unsigned long long)nflag);
    for (int c = threadIdx.x; c < D.n_cells; c += blockDim.x) D.cell_cnt[c] = 0;
    __syncthreads();
    if (threadIdx.x == 0) {
        *D.any = 0;
        if (in_graph) atomicAdd((unsigned long long *)(D.rebuilds + 1), 1ull);
    }
}

// Clears the base-pair staging count of flagged instances; first kernel of a rebuild.
__global__ void k_rebuild_begin(Dev D, GlobP g) {
    if (*(volatile int *)D.any == 0) return;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < g.n_inst; k += gridDim.x * blockDim.x)
        if (D.flag[k]) D.bp_cnt[k] = 0;
}

cudaError_t launch_rebuild_body(const Dev &D, const GlobP &g, int cur, const RebuildPlan &pl, int in_graph, cudaStream_t st) {
    const float slack = 1.001f;
    if (pl.n_small_items > 0) k_rebuild_small<<<pl.small_grid, 256, 0, st>>>(D, g, cur, pl.small_items, pl.n_small_items, slack);
    if (pl.n_large_items > 0) {
        k_cell_bin<<<pl.large_grid, 256, 0, st>>>(D, g, cur, pl.large_items, pl.n_large_items);
        k_cell_scan<<<1, 1024, 0, st>>>(D);
        k_cell_fill<<<pl.large_grid, 256, 0, st>>>(D, g, pl.large_items, pl.n_large_items);
        k_cell_sort<<<(D.n_cells + 255) / 256, 256, 0, st>>>(D);
        k_cell_search<<<pl.large_grid, 256, 0, st>>>(D, g, cur, pl.large_items, pl.n_large_items, slack);
    }
    k_rebuild_finish<<<1, 1024, 0, st>>>(D, g, in_graph);
    return cudaGetLastError();
}

int rebuild_body_kernels(const RebuildPlan &pl) { return (pl.n_small_items > 0) + 5 * (pl.n_large_items > 0) + 1; }

cudaError_t launch_rebuild(const Dev &D, const GlobP &g, int cur, const RebuildPlan &pl, int after_step, int nparts,
                           cudaStream_t st) {
    if (after_step) {
        cudaError_t e = launch_trigger(D, g, nparts, st);
        if (e != cudaSuccess) return e;
    } else {
        k_rebuild_begin<<<(g.n_inst + 255) / 256, 256, 0, st>>>(D, g);
    }
    return launch_rebuild_body(D, g, cur, pl, 0, st);
}

} // namespace sisg
