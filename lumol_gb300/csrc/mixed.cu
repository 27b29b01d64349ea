// mixed.cu -- the mixed-precision force path.
//
// Pair potentials and Ewald real space / Wolf are evaluated in FP32; every
// atom's force is summed with error-free TwoSum steps (a compensated FP32
// sum, rounded once to FP32 at the end); energies and virials are accumulated
// in FP64; the Ewald structure factors rho(k) are accumulated in FP64; the
// integrator keeps FP64 positions and velocities.
//
// Positions reach the kernels as 32-bit fixed-point fractions of the cell
// length (u = floor(frac(x / L) * 2^32)), 16 bytes per atom with the charge:
// the difference of two coordinates, taken as a signed 32-bit integer, wraps
// around exactly like the minimum image of an orthorhombic cell, and its
// resolution (L / 2^32, 1.6e-8 A at L = 70 A) is far below the FP32 rounding
// of the distance itself, so d = int32(u_i - u_j) * L / 2^32 carries a
// relative error of about 6e-8 with no absolute ulp(L) term.
//
// Threads per atom (TPA = 1..32) is a template parameter chosen per workload
// by the autotuner: the TPA lanes of a group walk one atom's neighbour list
// and combine their compensated partial sums with shuffles.
//
// The kernels walk each system's atoms in the cell-sorted order of the last
// list build (rows, list entries, fixed-point positions and (kind, molecule)
// are all in that order), so the neighbours of consecutive atoms share cache
// lines; forces are written back to each atom's own index.
#include "kernels.h"
#include "mixed_common.cuh"

namespace lg {

// LJ1: every system of the batch has one kind and a Lennard-Jones pair (the
// pair type and the one-kind parameters resolved when the kernel is compiled;
// the arithmetic, and so every force bit, is the generic kernel's).
template <int TPA, bool EV, bool GENERAL, bool LJ1 = false, bool NORESTR = false>
__global__ void __launch_bounds__(256, GENERAL && !EV ? 4 : 1) pair_mixed_kernel(
    int n, const uint4* __restrict__ pfx, const int2* __restrict__ km, const int* __restrict__ order,
    const int* __restrict__ sysid, const SysDev* __restrict__ sys,
    const PairDevF* __restrict__ ptab, const int* __restrict__ nbr, const int* __restrict__ nnb, int maxnb,
    const int* __restrict__ spec_off, const int* __restrict__ spec_j, const int8_t* __restrict__ spec_path,
    uint32_t terms, double* __restrict__ force, double* __restrict__ red, const double4_32a* __restrict__ posq) {
    // t walks the cell-sorted order; i is the atom's own index (forces, bond paths)
    int gt = blockIdx.x * blockDim.x + threadIdx.x;
    int t = gt / TPA;
    int sub = gt % TPA;
    bool active = t < n;
    int tt = active ? t : n - 1;
    int i = order[tt];
    const SysDev& s = sys[sysid[tt]];
    uint4 pi = pfx[tt];
    float qi = __uint_as_float(pi.w);
    int2 kmi = km[tt];
    const PairDevF* prow = ptab + s.ptab + kmi.x * s.nk;
    bool coul = GENERAL && (terms & 16u) && s.coul != 0 && qi != 0.0f;
    bool pairs = (terms & 1u) != 0;
    float coul_rc2 = GENERAL ? s.coul_rc2_f : 0.0f;
    float alpha = GENERAL ? (float)s.alpha : 0.0f;
    float pref = qi * (float)(1.0 / FOUR_PI_EPSILON_0);
    MixedAcc A;
    const bool single = LJ1 || s.nk == 1;  // one kind: the pair parameters once per atom
    const int4 ph1 = __ldg(reinterpret_cast<const int4*>(prow));
    const float4 pq1 = __ldg(reinterpret_cast<const float4*>(prow) + 1);
    int cnt = active ? nnb[tt] : 0;
    const int* list = nbr + (size_t)tt * maxnb;
    // (kind, molecule) of a neighbour: not needed for one kind without restrictions
    const bool need_km = GENERAL || !single;
    walk_row<TPA>(
        list, cnt, sub,
        [&](int js, uint4& pj, int2& kmj) {
            pj = pfx[js];
            kmj = need_km ? km[js] : make_int2(0, 0);
        },
        [&](int js, const uint4& pj, const int2& kmj) {
            mixed_entry<EV, GENERAL, LJ1, NORESTR>(A, s, prow, pi, qi, kmi.y, i, tt, js, pj, kmj, order, spec_off, spec_j,
                                     spec_path, pairs, coul, coul_rc2, alpha, pref, single, ph1, pq1, posq);
        });
    // combine the group's compensated sums; one lane converts to FP64
    group_combine<TPA>(A);
    if (EV) {
        A.ep = group_sum_d<TPA>(A.ep);
        A.ec = group_sum_d<TPA>(A.ec);
        A.w0 = group_sum_d<TPA>(A.w0);
        A.w1 = group_sum_d<TPA>(A.w1);
        A.w2 = group_sum_d<TPA>(A.w2);
        A.w3 = group_sum_d<TPA>(A.w3);
        A.w4 = group_sum_d<TPA>(A.w4);
        A.w5 = group_sum_d<TPA>(A.w5);
    }
    if (active && sub == 0) {  // the first force kernel of a step: assigns
        // the compensated sum rounded once to FP32 (one rounding error of the
        // result instead of one per term)
        force[3 * i] = (double)radd(A.fxs, A.fxc);
        force[3 * i + 1] = (double)radd(A.fys, A.fyc);
        force[3 * i + 2] = (double)radd(A.fzs, A.fzc);
        if (EV) {
            double ec = A.ec;
            if (GENERAL && (terms & 16u) && s.coul == 2 && qi != 0.0f) {
                double q = (double)qi;
                ec -= q * q * 0.5 * (s.wolf_ec + s.alpha * FRAC_2_SQRT_PI) / FOUR_PI_EPSILON_0;
            }
            double* rr = red + (size_t)i * RED_STRIDE;
            rr[E_PAIRS] += A.ep;
            rr[E_COUL] += ec;
            double* w = rr + N_ESLOT;
            w[0] += A.w0; w[1] += A.w1; w[2] += A.w2;
            w[3] += A.w1; w[4] += A.w3; w[5] += A.w4;
            w[6] += A.w2; w[7] += A.w4; w[8] += A.w5;
        }
    }
}

template <int TPA, bool GENERAL, bool LJ1 = false, bool NORESTR = false>
void launch_pair_mixed_variant(const Batch& b, uint32_t terms, bool ev, cudaStream_t st) {
    int tb = 256;
    long long threads = (long long)b.n * TPA;
    unsigned grid = (unsigned)((threads + tb - 1) / tb);
    if (ev)
        pair_mixed_kernel<TPA, true, GENERAL, LJ1, NORESTR><<<grid, tb, 0, st>>>(
            b.n, b.posfx, b.km, b.cell_atoms, b.sysid, b.sys, b.ptabf, b.nbr, b.nnb, b.maxnb, b.spec_off, b.spec_j,
            b.spec_path, terms, b.force, b.red, b.posq);
    else
        pair_mixed_kernel<TPA, false, GENERAL, LJ1, NORESTR><<<grid, tb, 0, st>>>(
            b.n, b.posfx, b.km, b.cell_atoms, b.sysid, b.sys, b.ptabf, b.nbr, b.nnb, b.maxnb, b.spec_off, b.spec_j,
            b.spec_path, terms, b.force, b.red, b.posq);
}

template <int TPA>
void launch_pair_mixed_tpa(const Batch& b, uint32_t terms, bool ev, cudaStream_t st) {
    if (b.pair_general && b.norestr) launch_pair_mixed_variant<TPA, true, false, true>(b, terms, ev, st);
    else if (b.pair_general) launch_pair_mixed_variant<TPA, true>(b, terms, ev, st);
    else if (b.lj1) launch_pair_mixed_variant<TPA, false, true>(b, terms, ev, st);
    else launch_pair_mixed_variant<TPA, false>(b, terms, ev, st);
}

void launch_pair_mixed(const Batch& b, uint32_t terms, bool ev, cudaStream_t st) {
    if (b.n == 0) return;
    switch (b.tpa) {
        case 1: launch_pair_mixed_tpa<1>(b, terms, ev, st); break;
        case 2: launch_pair_mixed_tpa<2>(b, terms, ev, st); break;
        case 4: launch_pair_mixed_tpa<4>(b, terms, ev, st); break;
        case 8: launch_pair_mixed_tpa<8>(b, terms, ev, st); break;
        case 16: launch_pair_mixed_tpa<16>(b, terms, ev, st); break;
        default: launch_pair_mixed_tpa<32>(b, terms, ev, st); break;
    }
}

// Fixed-point copy of the wrapped FP64 positions, in the cell-sorted order of
// the mixed path or in atom order (plain path: the FP32 classification of the
// half-list kernel).
__global__ void fixed_positions_kernel(int n, const double4_32a* __restrict__ posq, const int* __restrict__ sysid,
                                       const SysDev* __restrict__ sys, const int* __restrict__ order,
                                       uint4* __restrict__ pfx) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;  // cell-sorted position (atom index without an order)
    if (t >= n) return;
    pfx[t] = fixed_position(sys[sysid[t]], posq[order ? order[t] : t]);
}

void launch_split_positions(const Batch& b, cudaStream_t st) {
    if (b.n && b.posfx)
        fixed_positions_kernel<<<(b.n + 255) / 256, 256, 0, st>>>(b.n, b.posq, b.sysid, b.sys,
                                                                  b.perm ? b.cell_atoms : nullptr, b.posfx);
}

// ---------------------------------------------------------------------------
// Mixed Ewald k-space: FP32 e^{ik.r} with the phase reduced in FP64, FP64
// rho(k) accumulation, FP32 field per chunk of k-vectors.
// ---------------------------------------------------------------------------
__device__ __forceinline__ float2 cmulf(float2 a, float2 b) {
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

__global__ void eikr_mixed_kernel(int n, const double4_32a* __restrict__ posq, const int* __restrict__ sysid,
                                  const SysDev* __restrict__ sys, float2* __restrict__ eikr, float* __restrict__ qf) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= 3 * n) return;
    int axis = t / n, i = t - axis * n;
    const SysDev& s = sys[sysid[i]];
    if (s.coul != 1) return;
    double4_32a p = posq[i];
    if (axis == 0) qf[i] = (float)p.w;  // the charge in FP32, as the real-space pairs use it
    double phase = axis_phase(s, axis, p.x, p.y, p.z);
    phase -= 2.0 * PI * rint(phase * (0.5 / PI));
    float sn, cs;
    sincosf((float)phase, &sn, &cs);
    float2 e1 = make_float2(cs, sn);
    eikr[(size_t)(0 * 3 + axis) * n + i] = make_float2(1.0f, 0.0f);
    eikr[(size_t)(1 * 3 + axis) * n + i] = e1;
    float2 e = e1;
    for (int kk = 2; kk <= s.kmax; kk++) {
        e = cmulf(e, e1);
        eikr[(size_t)(kk * 3 + axis) * n + i] = e;
    }
}

__device__ __forceinline__ float2 eikrf_at(const float2* __restrict__ eikr, int n, int kk, int axis, int i) {
    if (kk >= 0) return eikr[(size_t)(kk * 3 + axis) * n + i];
    float2 v = eikr[(size_t)((-kk) * 3 + axis) * n + i];
    return make_float2(v.x, -v.y);
}

template <bool EV>
__global__ void __launch_bounds__(256) rho_mixed_kernel(int n, const float* __restrict__ qf,
                                                        const SysDev* __restrict__ sys,
                                                        const KVecDev* __restrict__ kvec,
                                                        const float2* __restrict__ eikr, double2* __restrict__ rho,
                                                        float2* __restrict__ rhof, double* __restrict__ kred) {
    __shared__ double sre[256], sim[256];
    int k = blockIdx.x;
    KVecDev kv = kvec[k];
    const SysDev& s = sys[kv.sys];
    // each thread's terms q e^{ik.r} summed in FP32 without rounding error to
    // speak of: the exact product q ph = p + e (e from an FMA), p into a
    // TwoSum, e into its compensation; the threads' sums then meet in FP64.
    // (FP64 arithmetic here ran on GB300's narrow FP64 pipe: four FP64
    // operations a term against about thirty FP32 ones.)
    float rs = 0.f, rc = 0.f, is = 0.f, ic = 0.f;
    for (int i = s.begin + threadIdx.x; i < s.end; i += blockDim.x) {
        float2 ph = cmulf(cmulf(eikrf_at(eikr, n, kv.ikx, 0, i), eikrf_at(eikr, n, kv.iky, 1, i)),
                          eikrf_at(eikr, n, kv.ikz, 2, i));
        const float q = qf[i];
        const float px = __fmul_rn(q, ph.x), py = __fmul_rn(q, ph.y);
        two_sum_acc(rs, rc, px);
        rc = __fadd_rn(rc, __fmaf_rn(q, ph.x, -px));
        two_sum_acc(is, ic, py);
        ic = __fadd_rn(ic, __fmaf_rn(q, ph.y, -py));
    }
    sre[threadIdx.x] = (double)rs + (double)rc;
    sim[threadIdx.x] = (double)is + (double)ic;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) {
            sre[threadIdx.x] += sre[threadIdx.x + o];
            sim[threadIdx.x] += sim[threadIdx.x + o];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        double2 r = make_double2(sre[0], sim[0]);
        rho[k] = r;
        rhof[k] = make_float2((float)r.x, (float)r.y);
        if (EV) {
            double nrm = r.x * r.x + r.y * r.y;
            double* out = kred + (size_t)k * 7;
            out[0] = kv.energy * nrm;
            for (int c = 0; c < 6; c++) out[1 + c] = nrm * kv.virial[c];
        }
    }
}

__global__ void __launch_bounds__(128) field_mixed_kernel(int n, int kchunk, const int* __restrict__ sysid,
                                                          const SysDev* __restrict__ sys,
                                                          const KVecF* __restrict__ kvecf,
                                                          const float2* __restrict__ eikr,
                                                          const float2* __restrict__ rhof,
                                                          double* __restrict__ fpart) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int c = blockIdx.y;
    if (i >= n) return;
    const SysDev& s = sys[sysid[i]];
    float fx = 0.f, fy = 0.f, fz = 0.f;
    if (s.coul == 1) {
        int k0 = s.kbegin + c * kchunk;
        int k1 = min(k0 + kchunk, s.kend);
        for (int k = k0; k < k1; k++) {
            KVecF kv = kvecf[k];
            float2 e = cmulf(cmulf(eikrf_at(eikr, n, kv.ikx, 0, i), eikrf_at(eikr, n, kv.iky, 1, i)),
                             eikrf_at(eikr, n, kv.ikz, 2, i));
            float2 r = rhof[k];
            float imag = e.y * r.x - e.x * r.y;
            fx = fmaf(imag, kv.fx, fx);
            fy = fmaf(imag, kv.fy, fy);
            fz = fmaf(imag, kv.fz, fz);
        }
    }
    double* out = fpart + (size_t)c * 3 * n + 3 * (size_t)i;
    out[0] = fx;
    out[1] = fy;
    out[2] = fz;
}

void launch_kspace_mixed_part(const Batch& b, int part, bool ev, cudaStream_t st) {
    if (b.nkvec == 0 || b.n == 0) return;
    if (part == 0) {
        eikr_mixed_kernel<<<(3 * b.n + 255) / 256, 256, 0, st>>>(b.n, b.posq, b.sysid, b.sys, b.eikrf, b.qf);
    } else if (part == 1) {
        if (ev)
            rho_mixed_kernel<true><<<b.nkvec, 256, 0, st>>>(b.n, b.qf, b.sys, b.kvec, b.eikrf, b.rho, b.rhof,
                                                            b.kred);
        else
            rho_mixed_kernel<false><<<b.nkvec, 256, 0, st>>>(b.n, b.qf, b.sys, b.kvec, b.eikrf, b.rho, b.rhof,
                                                             b.kred);
    } else {
        dim3 grid((b.n + 127) / 128, b.nkchunks);
        field_mixed_kernel<<<grid, 128, 0, st>>>(b.n, b.kchunk, b.sysid, b.sys, b.kvecf, b.eikrf, b.rhof, b.fpart);
        launch_field_reduce(b, st);
    }
}

}  // namespace lg
