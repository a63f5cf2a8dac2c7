// Replica exchange on the device (src/replica_exchange.F90,
// src/energy_replica.F90, src/var_replica.F90:105-259): every replica is one
// instance of the context, all of one topology; a label is one set of
// values of the replica variables (temperature, ionic strength, constant
// trap force, Rg bias target).  An exchange computes each replica's total potential
// energy at its own and at its partner's temperature with the ordinary
// energy kernels (the partner energies through a second set of instance
// records that carry the partner's temperature fields), decides every pair
// in one block, and applies the swaps: labels, temperature fields, velocity
// scaling, noise coefficients and FP32 triplet free energies.
#include <algorithm>

#include "common.cuh"
#include "kernels.h"

namespace sisg {

// the fields of an instance record that a label sets: its temperature, the
// electrostatic fields of its temperature and ionic strength (set_ele), the
// Rg bias target and the constant-force trap magnitude (REPT TEMP, ION, RG,
// TWZDCF of var_replica.F90)
__device__ __forceinline__ void copy_temperature_fields(InstP &d, const InstP &s) {
    d.tempK = s.tempK;
    d.rg0 = s.rg0;
    d.twz_scale = s.twz_scale;
    d.ele_coef = s.ele_coef;
    d.rcdist = s.rcdist;
    d.ele_cut = s.ele_cut;
    d.ele_cut2 = s.ele_cut2;
    d.diele_dTcoef = s.diele_dTcoef;
    d.diele = s.diele;
    d.ele_coef_f = s.ele_coef_f;
    d.rcdist_f = s.rcdist_f;
    d.ele_cut2_f = s.ele_cut2_f;
    d.ele_nl_cut2 = s.ele_nl_cut2;
}

// Partner of (0-based) label l: parity 0 pairs (0,1), (2,3), ... and parity 1
// pairs (1,2), (3,4), ... (the reference's odd and even exchange patterns,
// make_replica_exchange_pair_tb); -1 for an unpaired label.
__device__ __forceinline__ int remd_partner(int l, int parity, int n) {
    if (l - parity < 0) return -1;
    const int p = ((l - parity) & 1) == 0 ? l + 1 : l - 1;
    return p < n ? p : -1;
}

// instance records at the partner label's temperature (energy_replica.F90:95-121)
__global__ void k_remd_partner_ip(Dev D, RemdDev R, int n_inst, int parity) {
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n_inst; k += gridDim.x * blockDim.x) {
        InstP q = D.ip[k];
        const int p = remd_partner(R.rep2lab[k], parity, n_inst);
        if (p >= 0) copy_temperature_fields(q, R.lab_ip[p]);
        R.ip2[k] = q;
    }
}

__device__ __forceinline__ double total_potential(const double *row) {
    double t = 0.0;
    for (int k = 1; k <= 10; ++k) t += row[k];
    return t;
}

// replica_exchange.F90:98-154 for every pair of the pattern, one thread per
// pair (pairs are disjoint).  u: uniforms per pair in label order (the
// reference's random0), or NULL for Philox uniforms keyed by (pair, exchange
// counter).
__global__ void __launch_bounds__(256) k_remd_decide(Dev D, RemdDev R, int n_inst, int parity, const double *u, double kB,
                                                     unsigned long long seed, unsigned long long ctr) {
    for (int k = threadIdx.x; k < n_inst; k += blockDim.x) R.changed[k] = 0;
    if (threadIdx.x == 0) *R.n_acc = 0;
    __syncthreads();
    for (int q = threadIdx.x; 2 * q + parity + 1 < n_inst; q += blockDim.x) {
        const int li = 2 * q + parity, lj = li + 1;
        const int ri = R.lab2rep[li], rj = R.lab2rep[lj];
        const double tm = R.lab_ip[li].tempK, tn = R.lab_ip[lj].tempK;
        const double pot_i_m = total_potential(D.ene + (size_t)ri * 12), pot_i_n = total_potential(R.ene2 + (size_t)ri * 12);
        const double pot_j_n = total_potential(D.ene + (size_t)rj * 12), pot_j_m = total_potential(R.ene2 + (size_t)rj * 12);
        // Sugita, Kitao and Okamoto, J. Chem. Phys. 113, 6042 (2000), eq. 14
        const double delta = ((pot_j_m - pot_i_m) / tm - (pot_j_n - pot_i_n) / tn) / kB;
        double uq;
        if (u) {
            uq = u[q];
        } else {
            const uint4 r = philox4x32_10(make_uint4((unsigned)q, (unsigned)ctr, (unsigned)(ctr >> 32), 0xffffffffu),
                                          make_uint2((unsigned)seed, (unsigned)(seed >> 32)));
            uq = ((double)(((unsigned long long)r.x << 21) ^ (r.y >> 11)) + 1.0) * (1.0 / 9007199254740992.0);
        }
        if (!(delta < 0.0 || uq <= exp(-delta))) continue;
        R.rep2lab[ri] = lj;
        R.rep2lab[rj] = li;
        R.lab2rep[li] = rj;
        R.lab2rep[lj] = ri;
        const double sf = sqrt(tn / tm);
        R.vscale[ri] = sf;
        R.vscale[rj] = sf;
        R.changed[ri] = 1;  // velocities times sf
        R.changed[rj] = 2;  // velocities divided by sf
        InstP &a = R.ip[ri];
        InstP &b = R.ip[rj];
        const double cut_a = a.ele_nl_cut2, cut_b = b.ele_nl_cut2;
        copy_temperature_fields(a, R.lab_ip[lj]);
        copy_temperature_fields(b, R.lab_ip[li]);
        if (a.ele_nl_cut2 != cut_a || b.ele_nl_cut2 != cut_b) {
            // the electrostatic list cutoff follows the Debye length
            D.flag[ri] = 1;
            D.flag[rj] = 1;
            D.bp_cnt[ri] = 0;
            D.bp_cnt[rj] = 0;
            atomicOr(D.any, 1);
        }
        atomicAdd(R.n_acc, 1);
    }
}

// per bead of every swapped replica: velocity scaling (scale_velo,
// replica_exchange.F90:175-209) and the noise coefficient of its new
// temperature; per record of the FP32 triplet table: the new temperature's row
__global__ void k_remd_apply(Dev D, RemdDev R, GlobP g) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < g.n; i += gridDim.x * blockDim.x) {
        const int k = D.binfo[i].x;
        const int c = R.changed[k];
        if (!c) continue;
        const double sf = R.vscale[k];
        double4 v = D.v[i];
        if (c == 1) {
            v.x = sf * v.x;
            v.y = sf * v.y;
            v.z = sf * v.z;
        } else {
            v.x = v.x / sf;
            v.y = v.y / sf;
            v.z = v.z / sf;
        }
        D.v[i] = v;
        const int li = i - D.ip[k].bead_off;
        D.mdc[i].w = R.lab_w[(size_t)R.rep2lab[k] * R.n_local + li];
    }
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < g.n_inst * 469; t += gridDim.x * blockDim.x) {
        const int k = t / 469, h = t - k * 469;
        if (R.changed[k]) R.dgf[t] = R.lab_dgf[(size_t)R.rep2lab[k] * 469 + h];
    }
}

cudaError_t launch_remd_partner_ip(const Dev &D, const RemdDev &R, int n_inst, int parity, cudaStream_t st) {
    k_remd_partner_ip<<<(n_inst + 255) / 256, 256, 0, st>>>(D, R, n_inst, parity);
    return cudaGetLastError();
}

cudaError_t launch_remd_decide(const Dev &D, const RemdDev &R, const GlobP &g, int parity, const double *u, double kB,
                               unsigned long long ctr, cudaStream_t st) {
    k_remd_decide<<<1, 256, 0, st>>>(D, R, g.n_inst, parity, u, kB, g.seed, ctr);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    const int grid = std::max(1, std::min(4 * 152, (std::max(g.n, g.n_inst * 469) + 255) / 256));
    k_remd_apply<<<grid, 256, 0, st>>>(D, R, g);
    return cudaGetLastError();
}

} // namespace sisg
