// Displacement trigger and neighbour-list rebuild of libsisgpu:
// job_md.F90:376-395, neighbor_list.F90:1-233 and pbc_wrap (pbc.F90:196-226)
// for the instances whose trigger fired (flag[inst] != 0), in one cooperative
// kernel launched after every step; it ends at once when no instance fired.
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
#include <algorithm>

#include "common.cuh"
#include "kernels.h"
#include "listcore.cuh"

namespace sisg {

// ------------------------------------------------------- grid barrier
// Every block of the cooperative launch is resident at once, so a wait ends
// when the last block arrives.  The wait is bounded all the same: after one
// second of the global timer (or 2^26 polls) the block records ERR_TIMEOUT
// and leaves the kernel.
__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
__device__ bool grid_sync(const Dev &D) {
    __shared__ int s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned int *cnt = D.gbar, *gen = D.gbar + 1;
        const unsigned int g0 = *(volatile unsigned int *)gen;
        __threadfence();
        int ok = 0;
        if (atomicAdd(cnt, 1u) == gridDim.x - 1) {
            *cnt = 0u;
            __threadfence();
            atomicAdd(gen, 1u);
            ok = 1;
        } else {
            const unsigned long long t0 = global_ns();
            for (int it = 0; it < (1 << 26); ++it) {
                if (*(volatile unsigned int *)gen != g0) {
                    ok = 1;
                    break;
                }
                if ((it & 255) == 255 && global_ns() - t0 > 1000000000ull) break;
                __nanosleep(32);
            }
            if (!ok) atomicOr(D.err, ERR_TIMEOUT);
        }
        __threadfence();
        s_ok = ok;
    }
    __syncthreads();
    return s_ok != 0;
}

// --------------------------------------------------- all-pairs (small)
// items: (instance, first local bead); 32 beads per item, one warp per bead.
__device__ void rebuild_small(const Dev &D, const GlobP &g, int cur, const int2 *items, int n_items, float slack) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int it = blockIdx.x; it < n_items; it += gridDim.x) {
        const int2 item = items[it];
        const int inst = item.x;
        if (__ldcg(D.flag + inst) == 0) continue;
        const InstP &ip = D.ip[inst];
        const float maxcut2f = scan_cut2f(ip, slack);
        for (int li = item.y + warp; li < min(item.y + 32, ip.n); li += 8) {
            const int gi = ip.bead_off + li;
            double4 xi_w;
            bead_begin(D, cur, gi, ip, lane, xi_w);
            const int4 bii = D.binfo[gi];
            const uint4 mi = mir_at(D, cur)[gi];
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
// Data that other blocks of the same launch wrote are read with __ldcg (L2),
// never from a possibly stale L1 line.
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
__device__ void cell_bin(const Dev &D, int cur, const int2 *litems, int n_litems) {
    for (int it = blockIdx.x; it < n_litems; it += gridDim.x) {
        const int2 item = litems[it];
        if (__ldcg(D.flag + item.x) == 0) continue;
        const InstP &ip = D.ip[item.x];
        const int li = item.y + threadIdx.x;
        if (li >= ip.n) continue;
        const int gi = ip.bead_off + li;
        const double4 xw = wrap_pos(x_at(D, cur)[gi], ip);
        const int c = cell_of(xw, ip);
        D.bead_cell[gi] = c;
        atomicAdd(&D.cell_cnt[c], 1);
    }
}

// Exclusive scan of the cell counts over the whole grid: block b owns a
// contiguous chunk of cells; first its sum (gsum[b]), then, after a grid
// barrier, its offset (the sum of gsum over lower blocks) and a block scan of
// its chunk in tiles of 4 cells per thread.  Counts are reset to serve as
// fill cursors.
__device__ __forceinline__ int block_sum(int v, int *s_red) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    __syncthreads();
    if (lane == 0) s_red[warp] = v;
    __syncthreads();
    int t = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += s_red[w];
    return t;
}
__device__ __forceinline__ void scan_chunk(const Dev &D, int &lo, int &hi) {
    const int n = D.n_cells;
    const int chunk = (n + gridDim.x - 1) / gridDim.x;
    lo = min(n, (int)blockIdx.x * chunk);
    hi = min(n, lo + chunk);
}
__device__ void cell_scan_sums(const Dev &D, int *s_red) {
    int lo, hi;
    scan_chunk(D, lo, hi);
    int v = 0;
    for (int c = lo + threadIdx.x; c < hi; c += blockDim.x) v += __ldcg(D.cell_cnt + c);
    const int t = block_sum(v, s_red);
    if (threadIdx.x == 0) D.gsum[blockIdx.x] = t;
}
__device__ void cell_scan_write(const Dev &D, int *s_red) {
    __shared__ int s_warp[8];
    __shared__ int s_carry;
    int lo, hi;
    scan_chunk(D, lo, hi);
    int v = 0;
    for (int b = threadIdx.x; b < (int)blockIdx.x; b += blockDim.x) v += __ldcg(D.gsum + b);
    const int offset = block_sum(v, s_red);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (threadIdx.x == 0) s_carry = offset;
    __syncthreads();
    for (int base = lo; base < hi; base += 4 * (int)blockDim.x) {
        const int c0 = base + 4 * threadIdx.x;
        int x[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) x[q] = c0 + q < hi ? __ldcg(D.cell_cnt + c0 + q) : 0;
        const int tsum = x[0] + x[1] + x[2] + x[3];
        int incl = tsum;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += y;
        }
        if (lane == 31) s_warp[warp] = incl;
        __syncthreads();
        int wpre = 0;
        for (int w = 0; w < warp; ++w) wpre += s_warp[w];
        int run = s_carry + wpre + incl - tsum;
#pragma unroll
        for (int q = 0; q < 4; ++q)
            if (c0 + q < hi) {
                D.cell_start[c0 + q] = run;
                D.cell_cnt[c0 + q] = 0;
                run += x[q];
            }
        __syncthreads();
        if (threadIdx.x == 0) {
            int t = 0;
            for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += s_warp[w];
            s_carry += t;
        }
        __syncthreads();
    }
    if (blockIdx.x == gridDim.x - 1 && threadIdx.x == 0) D.cell_start[D.n_cells] = s_carry;
}

__device__ void cell_fill(const Dev &D, const int2 *litems, int n_litems) {
    for (int it = blockIdx.x; it < n_litems; it += gridDim.x) {
        const int2 item = litems[it];
        if (__ldcg(D.flag + item.x) == 0) continue;
        const InstP &ip = D.ip[item.x];
        const int li = item.y + threadIdx.x;
        if (li >= ip.n) continue;
        const int gi = ip.bead_off + li;
        const int c = __ldcg(D.bead_cell + gi);
        const int pos = __ldcg(D.cell_start + c) + atomicAdd(&D.cell_cnt[c], 1);
        D.cell_beads[pos] = gi;
    }
}

// sorts every cell's beads by index so that list order is deterministic:
// one warp per cell ranks up to 256 beads in shared memory (rank = number of
// smaller indices; indices are distinct); larger cells are insertion-sorted
__device__ void cell_sort(const Dev &D) {
    constexpr int kCap = 256;
    __shared__ int sb[8][kCap];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int nwarps = gridDim.x * 8;
    for (int c = blockIdx.x * 8 + warp; c < D.n_cells; c += nwarps) {
        const int a = __ldcg(D.cell_start + c), b = __ldcg(D.cell_start + c + 1), m = b - a;
        if (m <= 1) continue;
        if (m <= kCap) {
            for (int k = lane; k < m; k += 32) sb[warp][k] = __ldcg(D.cell_beads + a + k);
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
                const int v = __ldcg(D.cell_beads + k);
                int q = k - 1;
                while (q >= a && __ldcg(D.cell_beads + q) > v) {
                    D.cell_beads[q + 1] = __ldcg(D.cell_beads + q);
                    --q;
                }
                D.cell_beads[q + 1] = v;
            }
        }
    }
}

// one warp per bead: the 27 neighbouring cells' beads as candidates
__device__ void cell_search(const Dev &D, const GlobP &g, int cur, const int2 *litems, int n_litems, float slack) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    // each litem covers 256 beads; 8 warps stride over them
    for (int it = blockIdx.x; it < n_litems; it += gridDim.x) {
        const int2 item = litems[it];
        const int inst = item.x;
        if (__ldcg(D.flag + inst) == 0) continue;
        const InstP &ip = D.ip[inst];
        const float maxcut2f = scan_cut2f(ip, slack);
        for (int li = item.y + warp; li < min(item.y + 256, ip.n); li += 8) {
            const int gi = ip.bead_off + li;
            double4 xi_w;
            bead_begin(D, cur, gi, ip, lane, xi_w);
            const int4 bii = D.binfo[gi];
            const uint4 mi = mir_at(D, cur)[gi];
            const int c0 = __ldcg(D.bead_cell + gi) - ip.cell_base;
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
                cstart = __ldcg(D.cell_start + c);
                ccnt = __ldcg(D.cell_start + c + 1) - cstart;
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
                    gj = __ldcg(D.cell_beads + cs + (k - ce));
                    if (gj != gi) f = test_pair(D, g, ip, cur, gi, bii, mi, xi_w, gj, maxcut2f, inst);
                }
                warp_append(D, g, gi, lane, f, gj, count);
            }
            bead_end(D, g, gi, lane, count);
        }
    }
}

// ------------------------------------------------------ cluster pairs
// The mixed path's pair kernel walks cluster pairs instead of per-bead lists
// (kernels.cu k_pairs_cl).  For every i-cluster of a rebuilt instance one
// warp gathers the clusters J (local index of the partner / 8) of its beads'
// list entries into a hash table in shared memory, ranks the distinct J in
// ascending order, and ORs each entry's bit 8a+b (a, b: the beads' places in
// their clusters) into the WCA or electrostatic mask of its J (listcore.cuh
// cluster_one).  The order is that of the local indices, so an instance
// gives the same lists alone and in any batch.  An i-cluster with more than
// ccap distinct J gets the count -1, and the pair kernel walks its beads'
// per-bead lists instead.
__device__ void cluster_lists(const Dev &D, const GlobP &g, int *sh) {
    const int warp = threadIdx.x >> 5;
    int *key = sh + warp * 2 * kClHash;
    for (int ic = blockIdx.x * 8 + warp; ic < g.n_cl; ic += gridDim.x * 8) {
        if (__ldcg(D.flag + D.binfo[D.cl_first[ic]].x) == 0) continue;
        cluster_one(D, g, ic, key, key + kClHash);
    }
}

// the cluster lists of the instances flagged by k_md_small
__global__ void __launch_bounds__(256) k_cluster_flagged(Dev D, GlobP g) {
    __shared__ int s_cl[8 * 2 * kClHash];
    cluster_lists(D, g, s_cl);
}
cudaError_t launch_cluster_flagged(const Dev &D, const GlobP &g, cudaStream_t st) {
    if (g.prec == 0 || g.n_cl == 0) return cudaSuccess;
    k_cluster_flagged<<<std::min((g.n_cl + 7) / 8, 4096), 256, 0, st>>>(D, g);
    return cudaGetLastError();
}

// ------------------------------------------------------------ finish
// Block 0: base-pair prefix counts over the instances and rebuild
// bookkeeping; every block: reset of its share of the cell counters.
__device__ void rebuild_finish(const Dev &D, const GlobP &g) {
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < D.n_cells; c += gridDim.x * blockDim.x) D.cell_cnt[c] = 0;
    if (blockIdx.x != 0) return;
    __shared__ int s[256];
    const int n = g.n_inst;
    const int per = (n + 255) / 256;
    const int lo = min(n, (int)threadIdx.x * per), hi = min(n, lo + per);
    int sum = 0, nflag = 0;
    for (int k = lo; k < hi; ++k) {
        const int c = min(__ldcg(D.bp_cnt + k), D.ip[k].bp_cap);
        sum += c;
        nflag += __ldcg(D.flag + k) != 0;
    }
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
        run += min(__ldcg(D.bp_cnt + k), D.ip[k].bp_cap);
        // new records: the next evaluation runs the Monte Carlo pass (job_md.F90:392-394)
        if (__ldcg(D.flag + k) && g.nstep_mc > 0) D.mc_due[k] = 1;
        D.flag[k] = 0;
    }
    if (threadIdx.x == 255) *D.bp_total = s[255];
    if (nflag) atomicAdd((unsigned long long *)D.rebuilds, (unsigned long long)nflag);
    __syncthreads();
    if (threadIdx.x == 0) *D.any = 0;
}

// --------------------------------------------- rebuild kernel
// One cooperative launch after every step, or on request: the rebuild of the
// instances flagged by the step kernel's trigger or by the host (flag, any).
// A step without a rebuild ends at once.  Block 0 clears the flagged
// instances' base-pair staging counts; the rebuild phases follow, separated
// by grid barriers: wrap and cell binning; cell scan; fill; sort; the 27-cell
// search and the all-pairs scan of small instances; finish.
__global__ void __launch_bounds__(256) k_trigger_rebuild(Dev D, GlobP g, int cur, RebuildPlan pl) {
    __shared__ int s_red[8];
    __shared__ int s_cl[8 * 2 * kClHash]; // per warp: cluster hash keys and ranks
    const float slack = 1.001f;
    if (*(volatile int *)D.any == 0) return;
    if (blockIdx.x == 0)
        for (int k = threadIdx.x; k < g.n_inst; k += blockDim.x)
            if (D.flag[k]) D.bp_cnt[k] = 0;
    if (!grid_sync(D)) return;
    if (pl.n_large_items > 0) {
        cell_bin(D, cur, pl.large_items, pl.n_large_items);
        if (!grid_sync(D)) return;
        cell_scan_sums(D, s_red);
        if (!grid_sync(D)) return;
        cell_scan_write(D, s_red);
        if (!grid_sync(D)) return;
        cell_fill(D, pl.large_items, pl.n_large_items);
        if (!grid_sync(D)) return;
        cell_sort(D);
        if (!grid_sync(D)) return;
        cell_search(D, g, cur, pl.large_items, pl.n_large_items, slack);
    }
    if (pl.n_small_items > 0) rebuild_small(D, g, cur, pl.small_items, pl.n_small_items, slack);
    if (g.any_ss) {
        // base-pair records of instances with a given secondary structure
        if (!grid_sync(D)) return;
        for (int gi = blockIdx.x * blockDim.x + threadIdx.x; gi < g.n; gi += gridDim.x * blockDim.x) {
            const int inst = D.binfo[gi].x;
            if (__ldcg(D.flag + inst) && D.ip[inst].ss_on) ss_records(D, g, cur, gi, inst);
        }
    }
    if (g.prec != 0) {
        if (!grid_sync(D)) return;
        cluster_lists(D, g, s_cl);
    }
    if (!grid_sync(D)) return;
    rebuild_finish(D, g);
}

// Self-test of the barrier's bounded wait: block `absent` leaves at once, so
// the wait of every other block runs out, records ERR_TIMEOUT and returns.
__global__ void __launch_bounds__(256) k_barrier_probe(Dev D, int absent) {
    if ((int)blockIdx.x == absent) return;
    grid_sync(D);
}

cudaError_t launch_barrier_probe(const Dev &D, int grid, int absent, cudaStream_t st) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(256);
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, k_barrier_probe, D, absent);
}

int coop_blocks_per_sm() {
    int nb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_trigger_rebuild, 256, 0) != cudaSuccess) return 0;
    return nb;
}

cudaError_t launch_rebuild(const Dev &D, const GlobP &g, int cur, const RebuildPlan &pl, int grid, cudaStream_t st) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(256);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, k_trigger_rebuild, D, g, cur, pl);
}

} // namespace sisg
