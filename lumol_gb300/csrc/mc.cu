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
#include "mixed_common.cuh"

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
    sincos(axis_phase(s, axis, newpos[3 * a], newpos[3 * a + 1], newpos[3 * a + 2]), &sn, &cs);
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
                                        const SysDev* __restrict__ sysp, double4_32a* __restrict__ posq,
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
    sincos(axis_phase(*sysp, axis, newpos[3 * a], newpos[3 * a + 1], newpos[3 * a + 2]), &sn, &cs);
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
                      const SysDev* d_sys, const double2* d_drho, cudaStream_t st) {
    int nk = sd.coul == 1 ? sd.kend - sd.kbegin : 0;
    if (nk > 0) mc_accept_kernel<<<(nk + 127) / 128, 128, 0, st>>>(sd.kbegin, nk, d_drho, b.rho);
    if (msize > 0)
        mc_set_positions_kernel<<<(3 * msize + 127) / 128, 128, 0, st>>>(b.n, mbeg, msize, sd.kmax, d_newpos, d_sys,
                                                                        b.posq, b.eikr, nk > 0 ? 1 : 0);
}

// ---------------------------------------------------------------------------
// Batched Monte Carlo: every system of the batch runs its own Metropolis chain
// of Translate moves (lumol-sim/src/mc/moves/translate.rs:85-125,
// mc/monte_carlo.rs:289-329), one warp per system.  A move's energy change is
// the EnergyCache cost (sys/cache.rs:145-220) of a one-atom molecule, summed
// over the atom's Verlet-list neighbours: the list holds every atom within the
// cutoff of both the old and the new position as long as no atom, the moved
// one included, is farther than skin/2 from where the list was built.  A move
// that would break this stops the chain before it is attempted; the host
// rebuilds the lists and relaunches the remaining moves.
// ---------------------------------------------------------------------------

// SplitMix64 (Steele, Lea & Flood, "Fast splittable pseudorandom number
// generators", OOPSLA 2014): one 64-bit state per chain.
__device__ __forceinline__ uint64_t splitmix64(uint64_t& state) {
    uint64_t z = (state += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
__device__ __forceinline__ double uniform01(uint64_t& state) {
    return (double)(splitmix64(state) >> 11) * (1.0 / 9007199254740992.0);
}

// PairInteraction::energy of the FP64 chains (pairs.rs:185-196): zero at and
// beyond the cutoff, on the exact distance.
__device__ __forceinline__ double mc_pair_energy(const PairDev& p, double dx, double dy, double dz) {
    double r = exact_norm(dx, dy, dz);
    if (r >= p.cutoff) return 0.0;
    double e, f;
    pair_energy_force(p, r, 1.0 / r, e, f);
    return e;
}

__global__ void __launch_bounds__(128) mc_chain_kernel(Batch b, McState* __restrict__ mc) {
    int s = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
    int lane = threadIdx.x & 31;
    if (s >= b.nsys) return;
    McState st = mc[s];
    if (!st.enabled || st.molecular || st.moves_left <= 0 || st.need_rebuild) return;
    const SysDev& sd = b.sys[s];
    int natoms = sd.end - sd.begin;
    if (natoms <= 0) return;
    uint64_t rng = st.rng;
    int64_t left = st.moves_left;
    double energy = st.energy;
    long long accepted = st.accepted, attempted = st.attempted;
    bool rebuild = false;
    while (left > 0) {
        // the move: a random atom (select_molecule) and a displacement in [-delta, delta) per axis
        uint64_t saved = rng;
        int i = sd.begin + min((int)(uniform01(rng) * natoms), natoms - 1);
        double ddx = -st.delta + 2.0 * st.delta * uniform01(rng);
        double ddy = -st.delta + 2.0 * st.delta * uniform01(rng);
        double ddz = -st.delta + 2.0 * st.delta * uniform01(rng);
        double u_accept = uniform01(rng);
        double4_32a old = b.posq[i];
        double nx = old.x + ddx, ny = old.y + ddy, nz = old.z + ddz;
        double4_32a bp = b.pos_build[i];
        double ex = nx - bp.x, ey = ny - bp.y, ez = nz - bp.z;
        ex -= rint(ex * sd.invL[0]) * sd.L[0];
        ey -= rint(ey * sd.invL[1]) * sd.L[1];
        ez -= rint(ez * sd.invL[2]) * sd.L[2];
        if (!(ex * ex + ey * ey + ez * ez <= sd.half_skin2)) {
            rng = saved;  // not attempted: retried after the list rebuild
            rebuild = true;
            break;
        }
        int ki = b.kind[i];
        const PairDev* prow = b.ptab + sd.ptab + ki * sd.nk;
        double de = 0.0;
        // a cell-sorted list (mixed engines) holds sorted positions: map back to atoms
        int row = b.perm ? b.perm[i] : i;
        int cnt = b.nnb[row];
        const int* list = b.nbr + (size_t)row * b.maxnb;
        for (int k = lane; k < cnt; k += 32) {
            int j = b.perm ? b.cell_atoms[list[k]] : list[k];
            double4_32a pj = b.posq[j];
            int kj = b.kind[j];
            const PairDev& p = prow[kj];
            if (p.type == 0 || restriction_excluded(p.restriction, 0)) continue;
            double ox, oy, oz, wx, wy, wz;
            // Configuration::distance(i, j), UnitCell::distance(r_j, new_i)
            exact_nearest_image(sd, pj.x, pj.y, pj.z, old.x, old.y, old.z, ox, oy, oz);
            exact_nearest_image(sd, nx, ny, nz, pj.x, pj.y, pj.z, wx, wy, wz);
            de += mc_pair_energy(p, wx, wy, wz) - mc_pair_energy(p, ox, oy, oz);
        }
        for (int o = 16; o > 0; o >>= 1) de += __shfl_xor_sync(0xffffffffu, de, o);
        attempted++;
        double cost = st.beta * de;
        bool accept = cost <= 0.0 || u_accept < exp(-cost);
        if (accept) {
            // Translate::apply: new position, then Molecule::wrap (UnitCell::wrap_vector)
            if (lane == 0) {
                double w[3] = {nx, ny, nz};
                for (int d = 0; d < 3; d++) w[d] -= floor(w[d] / sd.L[d]) * sd.L[d];
                b.posq[i] = make_double4_32a(w[0], w[1], w[2], old.w);
            }
            energy += de;
            accepted++;
        }
        __syncwarp();
        left--;
    }
    if (lane == 0) {
        mc[s].rng = rng;
        mc[s].moves_left = left;
        mc[s].energy = energy;
        mc[s].accepted = accepted;
        mc[s].attempted = attempted;
        mc[s].need_rebuild = rebuild ? 1 : 0;
    }
}

// Pair energy in FP32 from r^2 (the mixed path's parameters, shift included).
__device__ __forceinline__ float mc_pair_energy_r2(const PairDevF* pp, int type, float4 pq, float shift, float r2) {
    if (!(r2 < pq.w)) return 0.0f;
    if (type == 2) {
        float ir2 = 1.0f / r2;
        float ir6 = ir2 * ir2 * ir2;
        return ir6 * (pq.x * ir6 - pq.y) - shift;
    }
    float inv_r = rsqrtf(r2), fr;
    return pair_mixed(*pp, r2, inv_r * inv_r, inv_r, fr);
}

// Chains of a mixed-precision engine: the same moves and draws as the FP64
// chains, with the energy change evaluated like the mixed MD path: fixed-point
// positions in the cell order of the last list build (a neighbour is one
// gather, its minimum image an integer difference), FP32 pair energies summed
// per lane in FP32 and across lanes in FP64, the Metropolis test with expf.
// An accepted move updates the FP64 position and its fixed-point copy.
__global__ void __launch_bounds__(128) mc_chain_mixed_kernel(Batch b, McState* __restrict__ mc) {
    int s = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
    int lane = threadIdx.x & 31;
    if (s >= b.nsys) return;
    McState st = mc[s];
    if (!st.enabled || st.molecular || st.moves_left <= 0 || st.need_rebuild) return;
    const SysDev& sd = b.sys[s];
    int natoms = sd.end - sd.begin;
    if (natoms <= 0) return;
    const bool single = sd.nk == 1;  // one kind: the parameters once per chain
    const PairDevF* ptab = b.ptabf + sd.ptab;
    int4 ph1 = *reinterpret_cast<const int4*>(ptab);
    float4 pq1 = *(reinterpret_cast<const float4*>(ptab) + 1);
    float shift1 = ptab->shift;
    const float rebuild2 = sd.rebuild2_f;
    uint64_t rng = st.rng;
    int64_t left = st.moves_left;
    double energy = st.energy;
    long long accepted = st.accepted, attempted = st.attempted;
    bool rebuild = false;
    while (left > 0) {
        // the move: a random atom (select_molecule) and a displacement in [-delta, delta) per axis
        uint64_t saved = rng;
        int i = sd.begin + min((int)(uniform01(rng) * natoms), natoms - 1);
        double ddx = -st.delta + 2.0 * st.delta * uniform01(rng);
        double ddy = -st.delta + 2.0 * st.delta * uniform01(rng);
        double ddz = -st.delta + 2.0 * st.delta * uniform01(rng);
        double u_accept = uniform01(rng);
        int t = b.perm[i];
        double4_32a old = b.posq[i];
        uint4 uo = b.posfx[t];
        double4_32a np = make_double4_32a(old.x + ddx, old.y + ddy, old.z + ddz, old.w);
        uint4 un = fixed_position(sd, np);
        if (fixed_dist2(un, b.pfx_build[i], sd.Lq) > rebuild2) {
            rng = saved;  // not attempted: retried after the list rebuild
            rebuild = true;
            break;
        }
        int ki = single ? 0 : b.km[t].x;
        const PairDevF* prow = ptab + ki * sd.nk;
        int cnt = b.nnb[t];
        const int* list = b.nbr + (size_t)t * b.maxnb;
        float de = 0.0f;
        for (int k = lane; k < cnt; k += 32) {
            int js = list[k];
            uint4 pj = b.posfx[js];
            int type = ph1.x;
            float4 pq = pq1;
            float shift = shift1;
            int restr = ph1.y;
            if (!single) {
                const PairDevF* pp = prow + b.km[js].x;
                int4 ph = *reinterpret_cast<const int4*>(pp);
                type = ph.x;
                restr = ph.y;
                pq = *(reinterpret_cast<const float4*>(pp) + 1);
                shift = pp->shift;
            }
            if (type == 0 || restriction_excluded(restr, 0)) continue;
            const PairDevF* pp = single ? ptab : prow + b.km[js].x;
            de += mc_pair_energy_r2(pp, type, pq, shift, fixed_dist2(un, pj, sd.Lq)) -
                  mc_pair_energy_r2(pp, type, pq, shift, fixed_dist2(uo, pj, sd.Lq));
        }
        double ded = (double)de;
        for (int o = 16; o > 0; o >>= 1) ded += __shfl_xor_sync(0xffffffffu, ded, o);
        attempted++;
        double cost = st.beta * ded;
        bool accept = cost <= 0.0 || (float)u_accept < __expf(-(float)cost);
        if (accept) {
            // Translate::apply: new position, then Molecule::wrap (UnitCell::wrap_vector)
            if (lane == 0) {
                double w[3] = {np.x, np.y, np.z};
                for (int d = 0; d < 3; d++) w[d] -= floor(w[d] * sd.invL[d]) * sd.L[d];
                b.posq[i] = make_double4_32a(w[0], w[1], w[2], old.w);
                b.posfx[t] = un;  // the fixed-point copy does not change with the wrap
            }
            energy += ded;
            accepted++;
        }
        __syncwarp();
        left--;
    }
    if (lane == 0) {
        mc[s].rng = rng;
        mc[s].moves_left = left;
        mc[s].energy = energy;
        mc[s].accepted = accepted;
        mc[s].attempted = attempted;
        mc[s].need_rebuild = rebuild ? 1 : 0;
    }
}

// ---------------------------------------------------------------------------
// Molecular chains: MonteCarlo::propagate (mc/monte_carlo.rs:289-330) with
// Translate (mc/moves/translate.rs:84-125) and Rotate (mc/moves/rotate.rs:
// 68-124) of whole rigid molecules, one warp per system, in FP64 on either
// precision.  A move draws, from the chain's SplitMix64 stream: the move
// (the first whose cumulative frequency reaches a uniform number), the
// molecule (uniform), then the displacement (three uniforms in
// [-delta, delta)) or the axis (Marsaglia's 1972 method for a point of the
// unit sphere: two uniforms in [-1, 1) until x1^2 + x2^2 < 1) and the angle
// (uniform in [-theta, theta)), then the Metropolis number.  The energy change
// is EnergyCache::move_molecule_cost (sys/cache.rs:145-220) of the pair
// potentials: each moved atom against its Verlet-list neighbours outside the
// molecule (a rigid move keeps the intramolecular terms).  A move that would
// carry any atom of the molecule past skin / 2 stops the chain before it is
// attempted, as in the single-atom chains.
// ---------------------------------------------------------------------------
struct MolMove {
    bool rotate;
    double d[3];    // Translate: the displacement
    double R[9];    // Rotate: Matrix3::rotation(axis, angle) (matrix.rs:149-168)
    double com[3];  // Rotate: Molecule::center_of_mass (molecules.rs:256-264)
};

__device__ __forceinline__ void mol_new_position(const MolMove& mv, const double4_32a& p, double out[3]) {
    if (!mv.rotate) {
        out[0] = p.x + mv.d[0];
        out[1] = p.y + mv.d[1];
        out[2] = p.z + mv.d[2];
        return;
    }
    // rotate_around_axis (rotate.rs:118-124): com + rotation * (position - com)
    double v[3] = {p.x - mv.com[0], p.y - mv.com[1], p.z - mv.com[2]}, r[3];
    for (int a = 0; a < 3; a++)
        r[a] = __dadd_rn(__dadd_rn(__dmul_rn(mv.R[3 * a], v[0]), __dmul_rn(mv.R[3 * a + 1], v[1])),
                         __dmul_rn(mv.R[3 * a + 2], v[2]));
    for (int a = 0; a < 3; a++) out[a] = mv.com[a] + r[a];
}

// The Ewald k-space energy change of a molecular move (ewald.rs:790-839), this
// lane's share of the system's k-vectors: delta rho(k) = sum_a q_a
// (e^{ik.r_new} - e^{ik.r_old}) with k.r = ikx k_x.r + iky k_y.r + ikz k_z.r
// from the per-axis k-vectors, and sum_k f_k (|rho + delta|^2 - |rho|^2) /
// (4 pi eps0).  With `apply`, rho(k) += delta rho(k) instead (the accepted move).
__device__ double mol_kspace_delta(const Batch& b, const SysDev& sd, const MolMove& mv, int a0, int a1, int lane,
                                   bool apply) {
    double dk = 0.0;
    for (int kk = sd.kbegin + lane; kk < sd.kend; kk += 32) {
        const KVecDev& kv = b.kvec[kk];
        double re = 0.0, im = 0.0;
        for (int a = a0; a < a1; a++) {
            double4_32a p = b.posq[a];
            if (p.w == 0.0) continue;
            double np[3];
            mol_new_position(mv, p, np);
            double po = kv.ikx * axis_phase(sd, 0, p.x, p.y, p.z) + kv.iky * axis_phase(sd, 1, p.x, p.y, p.z) +
                        kv.ikz * axis_phase(sd, 2, p.x, p.y, p.z);
            double pn = kv.ikx * axis_phase(sd, 0, np[0], np[1], np[2]) +
                        kv.iky * axis_phase(sd, 1, np[0], np[1], np[2]) +
                        kv.ikz * axis_phase(sd, 2, np[0], np[1], np[2]);
            double so, co, sn, cn;
            sincos(po, &so, &co);
            sincos(pn, &sn, &cn);
            re += p.w * (cn - co);
            im += p.w * (sn - so);
        }
        double2 r = b.rho[kk];
        if (apply) {
            b.rho[kk] = make_double2(r.x + re, r.y + im);
            continue;
        }
        double nx = r.x + re, ny = r.y + im;
        dk += kv.energy * (nx * nx + ny * ny) - kv.energy * (r.x * r.x + r.y * r.y);
    }
    return dk / FOUR_PI_EPSILON_0;
}

__global__ void __launch_bounds__(128) mc_chain_mol_kernel(Batch b, McState* __restrict__ mc) {
    int s = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
    int lane = threadIdx.x & 31;
    if (s >= b.nsys) return;
    McState st = mc[s];
    if (!st.enabled || !st.molecular || st.moves_left <= 0 || st.need_rebuild) return;
    const SysDev& sd = b.sys[s];
    const int nmol = sd.mol_end - sd.mol_first;
    if (nmol <= 0) return;
    uint64_t rng = st.rng;
    int64_t left = st.moves_left;
    double energy = st.energy;
    long long accepted = st.accepted, attempted = st.attempted;
    bool rebuild = false;
    while (left > 0) {
        uint64_t saved = rng;
        MolMove mv;
        mv.rotate = !(uniform01(rng) <= st.cum_translate);
        const int m = sd.mol_first + min((int)(uniform01(rng) * nmol), nmol - 1);
        const int a0 = b.mol_start[m], a1 = b.mol_start[m + 1];
        if (!mv.rotate) {
            for (int k = 0; k < 3; k++) mv.d[k] = -st.delta + 2.0 * st.delta * uniform01(rng);
        } else {
            double x1 = 0.0, x2 = 0.0, sum = 1.0;
            for (int tries = 0; tries < 64 && !(sum < 1.0); tries++) {
                x1 = -1.0 + 2.0 * uniform01(rng);
                x2 = -1.0 + 2.0 * uniform01(rng);
                sum = x1 * x1 + x2 * x2;
            }
            double axis[3] = {0.0, 0.0, 1.0};
            if (sum < 1.0) {
                double factor = 2.0 * sqrt(1.0 - sum);
                axis[0] = x1 * factor;
                axis[1] = x2 * factor;
                axis[2] = 1.0 - 2.0 * sum;
            }
            double angle = -st.theta + 2.0 * st.theta * uniform01(rng);
            double norm = __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(axis[0], axis[0]), __dmul_rn(axis[1], axis[1])),
                                               __dmul_rn(axis[2], axis[2])));
            double n[3] = {__ddiv_rn(axis[0], norm), __ddiv_rn(axis[1], norm), __ddiv_rn(axis[2], norm)};
            double sn = sin(angle), cs = cos(angle);
            double xs = n[0] * sn, ys = n[1] * sn, zs = n[2] * sn;
            double omc = 1.0 - cs;
            double xy = __dmul_rn(__dmul_rn(n[0], n[1]), omc), xz = __dmul_rn(__dmul_rn(n[0], n[2]), omc),
                   yz = __dmul_rn(__dmul_rn(n[1], n[2]), omc);
            mv.R[0] = __dadd_rn(__dmul_rn(__dmul_rn(n[0], n[0]), omc), cs);
            mv.R[1] = __dadd_rn(xy, zs);
            mv.R[2] = __dsub_rn(xz, ys);
            mv.R[3] = __dsub_rn(xy, zs);
            mv.R[4] = __dadd_rn(__dmul_rn(__dmul_rn(n[1], n[1]), omc), cs);
            mv.R[5] = __dadd_rn(yz, xs);
            mv.R[6] = __dadd_rn(xz, ys);
            mv.R[7] = __dsub_rn(yz, xs);
            mv.R[8] = __dadd_rn(__dmul_rn(__dmul_rn(n[2], n[2]), omc), cs);
            double total = 0.0, c[3] = {0.0, 0.0, 0.0};
            for (int a = a0; a < a1; a++) {
                double4_32a p = b.posq[a];
                double w = b.vel[a].w;
                total = __dadd_rn(total, w);
                c[0] = __dadd_rn(c[0], __dmul_rn(w, p.x));
                c[1] = __dadd_rn(c[1], __dmul_rn(w, p.y));
                c[2] = __dadd_rn(c[2], __dmul_rn(w, p.z));
            }
            for (int k = 0; k < 3; k++) mv.com[k] = __ddiv_rn(c[k], total);
        }
        double u_accept = uniform01(rng);
        // every moved atom stays within skin / 2 of its position at the last build
        bool far = false;
        for (int a = a0 + lane; a < a1; a += 32) {
            double np[3];
            mol_new_position(mv, b.posq[a], np);
            double4_32a bp = b.pos_build[a];
            far = far || !(image_norm2(sd, np[0] - bp.x, np[1] - bp.y, np[2] - bp.z) <= sd.half_skin2);
        }
        if (__any_sync(0xffffffffu, far)) {
            rng = saved;  // not attempted: retried after the list rebuild
            rebuild = true;
            break;
        }
        double de = 0.0;
        const bool coul = sd.coul != 0 && !restriction_excluded(sd.coul_restr, 0);
        for (int a = a0; a < a1; a++) {
            double4_32a old = b.posq[a];
            double np[3];
            mol_new_position(mv, old, np);
            const PairDev* prow = b.ptab + sd.ptab + b.kind[a] * sd.nk;
            int row = b.perm ? b.perm[a] : a;
            int cnt = b.nnb[row];
            const int* list = b.nbr + (size_t)row * b.maxnb;
            for (int k = lane; k < cnt; k += 32) {
                int j = b.perm ? b.cell_atoms[list[k]] : list[k];
                if (b.mol[j] == m) continue;  // (intramolecular terms do not change)
                const PairDev& p = prow[b.kind[j]];
                const bool pair = p.type != 0 && !restriction_excluded(p.restriction, 0);
                double4_32a pj = b.posq[j];
                const double qq = old.w * pj.w;
                if (!pair && !(coul && qq != 0.0)) continue;
                double ox, oy, oz, wx, wy, wz;
                exact_nearest_image(sd, pj.x, pj.y, pj.z, old.x, old.y, old.z, ox, oy, oz);
                exact_nearest_image(sd, np[0], np[1], np[2], pj.x, pj.y, pj.z, wx, wy, wz);
                if (pair) de += mc_pair_energy(p, wx, wy, wz) - mc_pair_energy(p, ox, oy, oz);
                if (coul && qq != 0.0) {  // Ewald real space or Wolf (ewald.rs:387-428, wolf.rs:90-117)
                    const double r_old = exact_norm(ox, oy, oz), r_new = exact_norm(wx, wy, wz);
                    double e, fr, e_old = 0.0, e_new = 0.0;
                    if (!(r_old > sd.coul_rc)) {
                        if (sd.coul == 1) ewald_real_pair(sd.alpha, false, qq, r_old, 1.0 / r_old, e, fr);
                        else wolf_pair(sd, qq, r_old, 1.0 / r_old, e, fr);
                        e_old = e;
                    }
                    if (!(r_new > sd.coul_rc)) {
                        if (sd.coul == 1) ewald_real_pair(sd.alpha, false, qq, r_new, 1.0 / r_new, e, fr);
                        else wolf_pair(sd, qq, r_new, 1.0 / r_new, e, fr);
                        e_new = e;
                    }
                    de += e_new - e_old;
                }
            }
        }
        if (sd.coul == 1) de += mol_kspace_delta(b, sd, mv, a0, a1, lane, false);
        for (int o = 16; o > 0; o >>= 1) de += __shfl_xor_sync(0xffffffffu, de, o);
        attempted++;
        double cost = st.beta * de;
        bool accept = cost <= 0.0 || u_accept < exp(-cost);
        if (accept) {
            // apply: the new positions; a translated molecule is wrapped by its
            // centre of mass (Molecule::wrap, molecules.rs:287-296)
            double shift[3] = {0.0, 0.0, 0.0};
            if (!mv.rotate) {
                double total = 0.0, c[3] = {0.0, 0.0, 0.0};
                for (int a = a0; a < a1; a++) {
                    double np[3];
                    mol_new_position(mv, b.posq[a], np);
                    double w = b.vel[a].w;
                    total = __dadd_rn(total, w);
                    for (int k = 0; k < 3; k++) c[k] = __dadd_rn(c[k], __dmul_rn(w, np[k]));
                }
                double com[3], wc[3];
                for (int k = 0; k < 3; k++) com[k] = wc[k] = __ddiv_rn(c[k], total);
                if (sd.tric) tric_wrap(sd, wc);  // UnitCell::wrap_vector (cells.rs:263-282)
                else
                    for (int k = 0; k < 3; k++)
                        wc[k] = __dsub_rn(wc[k], __dmul_rn(floor(__ddiv_rn(wc[k], sd.L[k])), sd.L[k]));
                for (int k = 0; k < 3; k++) shift[k] = __dsub_rn(wc[k], com[k]);
            }
            // rho(k) += delta rho(k) of the accepted move (ewald.rs:826-830), each
            // lane its own k-vectors, before the positions change
            if (sd.coul == 1) (void)mol_kspace_delta(b, sd, mv, a0, a1, lane, true);
            __syncwarp();  // every lane has read the old positions
            for (int a = a0 + lane; a < a1; a += 32) {
                double4_32a old = b.posq[a];
                double np[3];
                mol_new_position(mv, old, np);
                double4_32a q = make_double4_32a(np[0] + shift[0], np[1] + shift[1], np[2] + shift[2], old.w);
                b.posq[a] = q;
                if (b.perm) b.posfx[b.perm[a]] = fixed_position(sd, q);
            }
            energy += de;
            accepted++;
        }
        __syncwarp();
        left--;
    }
    if (lane == 0) {
        mc[s].rng = rng;
        mc[s].moves_left = left;
        mc[s].energy = energy;
        mc[s].accepted = accepted;
        mc[s].attempted = attempted;
        mc[s].need_rebuild = rebuild ? 1 : 0;
    }
}

void launch_mc_chains(const Batch& b, McState* mc, bool fp64, bool molecular, cudaStream_t st) {
    int warps_per_block = 4;
    int grid = (b.nsys + warps_per_block - 1) / warps_per_block;
    // (each kernel skips the other kind's chains: a chain's draws do not depend on the batch)
    if (molecular) mc_chain_mol_kernel<<<grid, 32 * warps_per_block, 0, st>>>(b, mc);
    if (fp64) mc_chain_kernel<<<grid, 32 * warps_per_block, 0, st>>>(b, mc);
    else mc_chain_mixed_kernel<<<grid, 32 * warps_per_block, 0, st>>>(b, mc);
}

}  // namespace lg
