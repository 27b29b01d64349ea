// mc.cu -- Monte Carlo move cost of one molecule (EnergyCache::move_molecule_cost,
// lumol-core/src/sys/cache.rs:145-220) with the Coulomb GlobalCache costs of
// Ewald (energy/global/ewald.rs:572-613, 758-839) and Wolf (wolf.rs:121-165).
//
// The reference keeps an N x N matrix of pair energies (cache.rs:25, 77) and
// subtracts the cached old energies; here the old pair energies are evaluated
// again from the current positions, which hold the values the cache would
// hold, so no N x N matrix lives on the device.  The moved molecule's atoms
// only interact with atoms of OTHER molecules in this cost, so every bond path
// is BondPath::None (configuration.rs:124-129).
#include "kernels.h"

namespace lg {

constexpr int MC_BLOCK = 256;

// Pair + real-space Coulomb energy change of moving the atoms [mbeg, mbeg + msize)
// to newpos, one thread per other atom j, per-block partial sums.
__global__ void __launch_bounds__(MC_BLOCK) mc_pair_delta_kernel(
    int sys_index, int mbeg, int msize, const double* __restrict__ newpos, const double4_32a* __restrict__ posq,
    const int* __restrict__ kind, const SysDev* __restrict__ sys, const PairDev* __restrict__ ptab,
    uint32_t terms, double* __restrict__ partial) {
    __shared__ double sp[MC_BLOCK], sc[MC_BLOCK];
    const SysDev& s = sys[sys_index];
    int j = s.begin + blockIdx.x * blockDim.x + threadIdx.x;
    double dp = 0.0, dc = 0.0;
    if (j < s.end && !(j >= mbeg && j < mbeg + msize)) {
        double4_32a pj = posq[j];
        int kj = kind[j];
        for (int a = 0; a < msize; a++) {
            int i = mbeg + a;
            double4_32a pi = posq[i];
            const PairDev& p = ptab[s.ptab + kind[i] * s.nk + kj];
            double ox, oy, oz, nx, ny, nz;
            // Configuration::distance(i, j) and UnitCell::distance(r_j, new_i)
            exact_nearest_image(s, pj.x, pj.y, pj.z, pi.x, pi.y, pi.z, ox, oy, oz);
            exact_nearest_image(s, newpos[3 * a], newpos[3 * a + 1], newpos[3 * a + 2], pj.x, pj.y, pj.z, nx, ny,
                                nz);
            double r_old = exact_norm(ox, oy, oz), r_new = exact_norm(nx, ny, nz);
            if ((terms & 1u) && p.type != 0 && !restriction_excluded(p.restriction, 0)) {
                double e, f;
                double e_old = 0.0, e_new = 0.0;
                if (!(r_old >= p.cutoff)) {
                    pair_energy_force(p, r_old, 1.0 / r_old, e, f);
                    e_old = e;
                }
                if (!(r_new >= p.cutoff)) {
                    pair_energy_force(p, r_new, 1.0 / r_new, e, f);
                    e_new = e;
                }
                dp += e_new - e_old;
            }
            double qq = pi.w * pj.w;
            if ((terms & 16u) && s.coul != 0 && qq != 0.0 && !restriction_excluded(s.coul_restr, 0)) {
                double e, fr;
                double e_old = 0.0, e_new = 0.0;
                if (!(r_old > s.coul_rc)) {
                    if (s.coul == 1) ewald_real_pair(s.alpha, false, qq, r_old, 1.0 / r_old, e, fr);
                    else wolf_pair(s, qq, r_old, 1.0 / r_old, e, fr);
                    e_old = e;
                }
                if (!(r_new > s.coul_rc)) {
                    if (s.coul == 1) ewald_real_pair(s.alpha, false, qq, r_new, 1.0 / r_new, e, fr);
                    else wolf_pair(s, qq, r_new, 1.0 / r_new, e, fr);
                    e_new = e;
                }
                dc += e_new - e_old;
            }
        }
    }
    sp[threadIdx.x] = dp;
    sc[threadIdx.x] = dc;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) {
            sp[threadIdx.x] += sp[threadIdx.x + o];
            sc[threadIdx.x] += sc[threadIdx.x + o];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        partial[2 * blockIdx.x] = sp[0];
        partial[2 * blockIdx.x + 1] = sc[0];
    }
}

__device__ __forceinline__ double2 mc_cmul(double2 a, double2 b) {
    return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

// e^{ik.r} of the moved atoms at their new positions (ewald.rs:764-788).
__global__ void mc_new_eikr_kernel(int sys_index, int msize, const double* __restrict__ newpos,
                                   const SysDev* __restrict__ sys, double2* __restrict__ out) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= 3 * msize) return;
    const SysDev& s = sys[sys_index];
    int axis = t / msize, a = t - axis * msize;
    double sn, cs;
    sincos(s.k1[axis] * newpos[3 * a + axis], &sn, &cs);
    double2 e1 = make_double2(cs, sn), v = e1;
    out[(size_t)(0 * 3 + axis) * msize + a] = make_double2(1.0, 0.0);
    out[(size_t)(1 * 3 + axis) * msize + a] = e1;
    for (int q = 2; q <= s.kmax; q++) {
        v = mc_cmul(v, e1);
        out[(size_t)(q * 3 + axis) * msize + a] = v;
    }
}

__device__ __forceinline__ double2 eikr_get(const double2* __restrict__ e, int stride, int q, int axis, int i) {
    if (q >= 0) return e[(size_t)(q * 3 + axis) * stride + i];
    double2 v = e[(size_t)((-q) * 3 + axis) * stride + i];
    return make_double2(v.x, -v.y);
}

// delta rho(k) = sum_a q_a (e^{ik.r_a,new} - e^{ik.r_a,old}) and the k-space
// energy change sum_k f_k (|rho + delta|^2 - |rho|^2) per k (ewald.rs:790-839).
__global__ void mc_delta_rho_kernel(int n, int mbeg, int msize, int kbegin, int nk, const double4_32a* __restrict__ posq,
                                    const KVecDev* __restrict__ kvec, const double2* __restrict__ eikr,
                                    const double2* __restrict__ new_eikr, const double2* __restrict__ rho,
                                    double2* __restrict__ drho, double* __restrict__ dk) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nk) return;
    const KVecDev& kv = kvec[kbegin + k];
    double re = 0.0, im = 0.0;
    for (int a = 0; a < msize; a++) {
        int i = mbeg + a;
        double2 old_phi = mc_cmul(mc_cmul(eikr_get(eikr, n, kv.ikx, 0, i), eikr_get(eikr, n, kv.iky, 1, i)),
                                  eikr_get(eikr, n, kv.ikz, 2, i));
        double2 new_phi = mc_cmul(mc_cmul(eikr_get(new_eikr, msize, kv.ikx, 0, a),
                                          eikr_get(new_eikr, msize, kv.iky, 1, a)),
                                  eikr_get(new_eikr, msize, kv.ikz, 2, a));
        double q = posq[i].w;
        re += q * (new_phi.x - old_phi.x);
        im += q * (new_phi.y - old_phi.y);
    }
    drho[k] = make_double2(re, im);
    double2 r = rho[kbegin + k];
    double nx = r.x + re, ny = r.y + im;
    dk[k] = kv.energy * (nx * nx + ny * ny) - kv.energy * (r.x * r.x + r.y * r.y);
}

// Fixed-order sum of the per-block pair / Coulomb partials and the per-k
// k-space terms: out = {pairs, coulomb real, kspace / (4 pi eps0)}.
__global__ void __launch_bounds__(256) mc_sum_kernel(int nblocks, const double* __restrict__ partial, int nk,
                                                     const double* __restrict__ dk, double* __restrict__ out) {
    __shared__ double s0[256], s1[256], s2[256];
    double a = 0.0, b = 0.0, c = 0.0;
    for (int q = threadIdx.x; q < nblocks; q += blockDim.x) {
        a += partial[2 * q];
        b += partial[2 * q + 1];
    }
    for (int q = threadIdx.x; q < nk; q += blockDim.x) c += dk[q];
    s0[threadIdx.x] = a;
    s1[threadIdx.x] = b;
    s2[threadIdx.x] = c;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) {
            s0[threadIdx.x] += s0[threadIdx.x + o];
            s1[threadIdx.x] += s1[threadIdx.x + o];
            s2[threadIdx.x] += s2[threadIdx.x + o];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        out[0] = s0[0];
        out[1] = s1[0];
        out[2] = s2[0] / FOUR_PI_EPSILON_0;
    }
}

// Accepted move: rho += delta, the molecule's atoms take their new positions
// and their e^{ik.r} are recomputed from them.
__global__ void mc_accept_kernel(int kbegin, int nk, const double2* __restrict__ drho, double2* __restrict__ rho) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nk) return;
    double2 r = rho[kbegin + k], d = drho[k];
    rho[kbegin + k] = make_double2(r.x + d.x, r.y + d.y);
}

__global__ void mc_set_positions_kernel(int n, int mbeg, int msize, int kmax, const double* __restrict__ newpos,
                                        const double* __restrict__ k1, double4_32a* __restrict__ posq,
                                        double2* __restrict__ eikr, int update_eikr) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= 3 * msize) return;
    int axis = t / msize, a = t - axis * msize;
    int i = mbeg + a;
    double x = newpos[3 * a + axis];
    if (axis == 0) posq[i].x = x;
    else if (axis == 1) posq[i].y = x;
    else posq[i].z = x;
    if (!update_eikr) return;
    double sn, cs;
    sincos(k1[axis] * x, &sn, &cs);
    double2 e1 = make_double2(cs, sn), v = e1;
    eikr[(size_t)(0 * 3 + axis) * n + i] = make_double2(1.0, 0.0);
    eikr[(size_t)(1 * 3 + axis) * n + i] = e1;
    for (int q = 2; q <= kmax; q++) {
        v = mc_cmul(v, e1);
        eikr[(size_t)(q * 3 + axis) * n + i] = v;
    }
}

void launch_mc_cost(const Batch& b, int s, const SysDev& sd, int mbeg, int msize, const double* d_newpos,
                    double2* d_new_eikr, double2* d_drho, double* d_partial, double* d_dk, double* d_out,
                    cudaStream_t st) {
    int natoms = sd.end - sd.begin;
    int nblocks = (natoms + MC_BLOCK - 1) / MC_BLOCK;
    if (nblocks > 0)
        mc_pair_delta_kernel<<<nblocks, MC_BLOCK, 0, st>>>(s, mbeg, msize, d_newpos, b.posq, b.kind, b.sys, b.ptab,
                                                          0xffu, d_partial);
    int nk = sd.coul == 1 ? sd.kend - sd.kbegin : 0;
    if (nk > 0 && msize > 0) {
        mc_new_eikr_kernel<<<(3 * msize + 127) / 128, 128, 0, st>>>(s, msize, d_newpos, b.sys, d_new_eikr);
        mc_delta_rho_kernel<<<(nk + 127) / 128, 128, 0, st>>>(b.n, mbeg, msize, sd.kbegin, nk, b.posq, b.kvec, b.eikr,
                                                             d_new_eikr, b.rho, d_drho, d_dk);
    }
    mc_sum_kernel<<<1, 256, 0, st>>>(nblocks, d_partial, nk, d_dk, d_out);
}

void launch_mc_accept(const Batch& b, const SysDev& sd, int mbeg, int msize, const double* d_newpos,
                      const double* d_k1, const double2* d_drho, cudaStream_t st) {
    int nk = sd.coul == 1 ? sd.kend - sd.kbegin : 0;
    if (nk > 0) mc_accept_kernel<<<(nk + 127) / 128, 128, 0, st>>>(sd.kbegin, nk, d_drho, b.rho);
    if (msize > 0)
        mc_set_positions_kernel<<<(3 * msize + 127) / 128, 128, 0, st>>>(b.n, mbeg, msize, sd.kmax, d_newpos, d_k1,
                                                                        b.posq, b.eikr, nk > 0 ? 1 : 0);
}

}  // namespace lg
