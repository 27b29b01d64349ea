// mixed_common.cuh -- device helpers of the mixed-precision pair evaluation,
// shared by the per-step pair kernel (mixed.cu) and the persistent batched MD
// kernel (persist.cu).
#pragma once
#include "kernels.h"

namespace lg {

// FP32 arithmetic with every rounding written out: __fmul_rn / __fadd_rn /
// __fmaf_rn are never contracted into (or split out of) a fused multiply-add
// by the compiler, so an expression rounds the same way in every kernel it is
// inlined into.  The per-step pair kernels, the persistent MD kernel and the
// energy / no-energy variants therefore give each atom the same force bits.
__device__ __forceinline__ float rmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float radd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float rsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float rfma(float a, float b, float c) { return __fmaf_rn(a, b, c); }

// Knuth's TwoSum: s + x = t + err exactly; the error joins the compensation c.
__device__ __forceinline__ void two_sum_acc(float& s, float& c, float x) {
    float t = radd(s, x);
    float bp = rsub(t, s);
    float err = radd(rsub(s, rsub(t, bp)), rsub(x, bp));
    s = t;
    c = radd(c, err);
}

template <int TPA>
__device__ __forceinline__ double group_sum_d(double v) {
#pragma unroll
    for (int o = TPA / 2; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Minimum image of two fixed-point coordinates: signed wrap-around difference.
__device__ __forceinline__ float fixed_image(uint32_t ui, uint32_t uj, float scale) {
    return rmul((float)(int32_t)(ui - uj), scale);
}

// (c12 / r^12 - c6 / r^6): force / r and energy from 1 / r^2 and 1 / r^6.
__device__ __forceinline__ float lj_force_r(float c12, float c6, float ir6, float inv_r2) {
    return rmul(rmul(ir6, rfma(rmul(12.0f, c12), ir6, rmul(-6.0f, c6))), inv_r2);
}
__device__ __forceinline__ float lj_energy(float c12, float c6, float ir6) {
    return rmul(ir6, rfma(c12, ir6, -c6));
}

// Pair potential in FP32: returns energy, writes force / r.
__device__ __forceinline__ float pair_mixed(const PairDevF& p, float r2, float inv_r2, float inv_r, float& fr) {
    switch (p.type) {
        case 2: {  // LJ: c12 / r^12 - c6 / r^6
            float ir6 = rmul(rmul(inv_r2, inv_r2), inv_r2);
            fr = lj_force_r(p.a, p.b, ir6, inv_r2);
            return rsub(lj_energy(p.a, p.b, ir6), p.shift);
        }
        case 3: {  // Buckingham: A exp(-r / rho) - C / r^6
            float r = rmul(r2, inv_r);
            float ex = rmul(p.a, __expf(rmul(-r, p.c)));
            float ir6 = rmul(rmul(inv_r2, inv_r2), inv_r2);
            fr = rfma(rmul(ex, p.c), inv_r, -rmul(rmul(rmul(6.0f, p.b), ir6), inv_r2));
            return rsub(rfma(-p.b, ir6, ex), p.shift);
        }
        case 4: {  // Harmonic k / 2 (r - x0)^2
            float r = rmul(r2, inv_r);
            float dx = rsub(r, p.b);
            fr = rmul(rmul(-p.a, dx), inv_r);
            return rsub(rmul(rmul(rmul(0.5f, p.a), dx), dx), p.shift);
        }
        case 5: {  // BornMayerHuggins: a exp((sigma - r) / rho) - c / r^6 + d / r^8 (c = 1 / rho, e = sigma)
            float r = rmul(r2, inv_r);
            float ex = rmul(p.a, __expf(rmul(rsub(p.e, r), p.c)));
            float ir6 = rmul(rmul(inv_r2, inv_r2), inv_r2);
            float t6 = rmul(rmul(rmul(6.0f, p.b), ir6), inv_r);
            float t8 = rmul(rmul(rmul(rmul(8.0f, p.d), ir6), inv_r2), inv_r);
            fr = rmul(radd(rfma(ex, p.c, -t6), t8), inv_r);
            return rsub(radd(rfma(-p.b, ir6, ex), rmul(rmul(p.d, ir6), inv_r2)), p.shift);
        }
        case 6: {  // Morse: depth (1 - exp(a (x0 - r)))^2, force 2 depth (1 - exp^2) a as the reference
            float r = rmul(r2, inv_r);
            float ex = __expf(rmul(rsub(p.c, r), p.b));
            float rc = rsub(1.0f, ex);
            fr = rmul(rmul(rmul(rmul(2.0f, p.a), rfma(-ex, ex, 1.0f)), p.b), inv_r);
            return rsub(rmul(rmul(p.a, rc), rc), p.shift);
        }
        case 7: {  // Gaussian: -a exp(-b r^2), force 2 b r E
            float e = rmul(-p.a, __expf(rmul(-p.b, r2)));
            fr = rmul(rmul(2.0f, p.b), e);
            return rsub(e, p.shift);
        }
        case 8: {  // Mie: prefactor ((sigma / r)^n - (sigma / r)^m), n = c, m = d
            float sr = rmul(p.b, inv_r);
            float rep = powf(sr, p.c), att = powf(sr, p.d);
            fr = rmul(rmul(p.a, rfma(p.c, rep, -rmul(p.d, att))), inv_r2);
            return rsub(rmul(p.a, rsub(rep, att)), p.shift);
        }
        case PAIR_TABLE: {  // TableComputation (computations.rs:123-144) on FP32 tables
            float r = rmul(r2, inv_r);
            float binf = floorf(rmul(r, p.a));
            if (binf < p.c) {
                int bin = (int)binf;
                float2 t0 = __ldg(p.table + bin), t1 = __ldg(p.table + bin + 1);
                float dx = rfma(-(float)bin, p.b, r);  // r - bin delta (b = delta)
                float e = rfma(dx, rmul(rsub(t1.x, t0.x), p.a), t0.x);
                fr = rmul(rfma(dx, rmul(rsub(t1.y, t0.y), p.a), t0.y), inv_r);
                return rsub(e, p.shift);
            }
            fr = 0.0f;
            return rsub(0.0f, p.shift);
        }
        default:
            fr = 0.0f;
            return 0.0f;
    }
}

// Accumulators of one lane of a pair-kernel group.
struct MixedAcc {
    float fxs = 0.f, fxc = 0.f, fys = 0.f, fyc = 0.f, fzs = 0.f, fzc = 0.f;
    double ep = 0.0, ec = 0.0;
    double w0 = 0, w1 = 0, w2 = 0, w3 = 0, w4 = 0, w5 = 0;
};

// One neighbour-list entry of atom i (sorted position tt): pair potential and
// (GENERAL) restrictions and real-space Coulomb, added to the lane's sums.
// LJ1: a system of one kind with a Lennard-Jones pair (the parameters are
// ph1 / pq1), known when the kernel is compiled; the arithmetic is the same.
// NORESTR: no pair and no Coulomb restriction in the batch (the restriction
// code compiled out; the arithmetic is the same).
template <bool EV, bool GENERAL, bool LJ1 = false, bool NORESTR = false>
__device__ __forceinline__ void mixed_entry(
    MixedAcc& A, const SysDev& s, const PairDevF* __restrict__ prow, uint4 pi, float qi, int mi, int i, int tt,
    int js, uint4 pj, int2 kmj, const int* __restrict__ order, const int* __restrict__ spec_off,
    const int* __restrict__ spec_j, const int8_t* __restrict__ spec_path, bool pairs, bool coul, float coul_rc2,
    float alpha, float pref, bool single, int4 ph1, float4 pq1, const double4_32a* __restrict__ posq) {
    float qj = __uint_as_float(pj.w);
    float dx, dy, dz;
    if (GENERAL && s.tric) {  // (the general kernels only: batches with a triclinic cell take them)
        fixed_delta(s, pi, pj, dx, dy, dz);
    } else {
        dx = fixed_image(pi.x, pj.x, s.Lq[0]);
        dy = fixed_image(pi.y, pj.y, s.Lq[1]);
        dz = fixed_image(pi.z, pj.z, s.Lq[2]);
    }
    float r2 = rfma(dz, dz, rfma(dy, dy, rmul(dx, dx)));
    // the parameters as two 16-byte loads: (type, restriction, -, -) and (a, b, c, rc2);
    // a system with one kind passes them in (loaded once per atom)
    const PairDevF* pp = prow + kmj.x;
    int4 ph;
    float4 pq;
    if (LJ1 || single) {
        ph = ph1;
        pq = pq1;
    } else {
        ph = __ldg(reinterpret_cast<const int4*>(pp));
        pq = __ldg(reinterpret_cast<const float4*>(pp) + 1);
    }
    bool pin = pairs && (LJ1 || ph.x != 0) && r2 < pq.w;
    bool cin = GENERAL && coul && qj != 0.0f && r2 <= coul_rc2;
    if (LJ1 && !EV && !GENERAL) {
        // without a branch: an entry beyond the cutoff adds exact zeros, which
        // leave the compensated sums as they are (r2 >= rc2 > 0 keeps every
        // intermediate finite), and the lanes of a warp never diverge here
        const float inv_r = rsqrtf(r2);
        const float inv_r2 = rmul(inv_r, inv_r);
        const float ir6 = rmul(rmul(inv_r2, inv_r2), inv_r2);
        const float fr = lj_force_r(pq.x, pq.y, ir6, inv_r2);
        two_sum_acc(A.fxs, A.fxc, pin ? rmul(fr, dx) : 0.0f);
        two_sum_acc(A.fys, A.fyc, pin ? rmul(fr, dy) : 0.0f);
        two_sum_acc(A.fzs, A.fzc, pin ? rmul(fr, dz) : 0.0f);
        return;
    }
    if (!(pin || cin)) return;
    float inv_r = rsqrtf(r2);
    float inv_r2 = rmul(inv_r, inv_r);
    float fr = 0.0f;
    float e_pair = 0.0f, e_coul = 0.0f;
    double e_coul_d = 0.0;
    if (!GENERAL) {
        float shift = EV ? __ldg(&pp->shift) : 0.0f;
        if (LJ1 || ph.x == 2) {  // LJ: c12 / r^12 - c6 / r^6
            float ir6 = rmul(rmul(inv_r2, inv_r2), inv_r2);
            fr = lj_force_r(pq.x, pq.y, ir6, inv_r2);
            if (EV) e_pair = rsub(lj_energy(pq.x, pq.y, ir6), shift);
        } else {
            e_pair = pair_mixed(*pp, r2, inv_r2, inv_r, fr);
        }
    } else {
        int path = -1;
        int mj = kmj.y;
        float sc = 1.0f;
        const PairDevF& p = *pp;
        if (!NORESTR && pin && ph.y != 0) {
            path = ph.y <= 2 ? (mi != mj ? 0 : 5) : bond_path(i, order[js], mi, mj, spec_off, spec_j, spec_path);
            if (restriction_excluded(ph.y, path)) pin = false;
            else sc = ph.y == 6 && path == 4 ? p.scale14 : 1.0f;
        }
        if (pin) {
            float f;
            e_pair = rmul(sc, pair_mixed(p, r2, inv_r2, inv_r, f));
            fr = rmul(sc, f);
        }
        if (cin) {
            bool excl = false;
            float csc = 1.0f;
            if (!NORESTR && s.coul_restr != 0) {
                if (path < 0 || (s.coul_restr > 2 && path == 5))
                    path = s.coul_restr <= 2 ? (mi != mj ? 0 : 5)
                                             : bond_path(i, order[js], mi, mj, spec_off, spec_j, spec_path);
                excl = restriction_excluded(s.coul_restr, path);
                if (s.coul_restr == 6 && path == 4) csc = (float)s.coul_scale14;
            }
            float qq = rmul(pref, qj);
            float r = rmul(r2, inv_r);
            float ar = rmul(alpha, r);
            if (s.coul == 1) {
                float g = rmul(rmul(alpha, (float)FRAC_2_SQRT_PI), __expf(rmul(-ar, ar)));
                if (!NORESTR && excl) {
                    // an excluded (bonded) pair's -erf correction (ewald.rs:394-397,
                    // 411-427) in FP64, from the FP64 positions and charges: these
                    // terms (three per water molecule) all have one sign and a
                    // large sum, so FP32 roundings would not average out in the
                    // energy.  The force is then rounded to FP32 like the others.
                    const int j = order[js];
                    const double4_32a a4 = posq[i], b4 = posq[j];
                    double d[3];
                    exact_nearest_image(s, a4.x, a4.y, a4.z, b4.x, b4.y, b4.z, d[0], d[1], d[2]);
                    double rd2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
                    double rd = sqrt(rd2);
                    double ad = s.alpha * rd;
                    double qqd = a4.w * b4.w / FOUR_PI_EPSILON_0;
                    double efd = erf(ad);
                    double gd = s.alpha * FRAC_2_SQRT_PI * exp(-ad * ad);
                    e_coul_d = -qqd * efd / rd;
                    fr = radd(fr, (float)(qqd / rd2 * (gd - efd / rd)));
                    (void)g;
                } else {
                    float ec_ = erfcf(ar);
                    e_coul = rmul(rmul(qq, ec_), inv_r);
                    fr = radd(fr, rmul(rmul(qq, inv_r2), rfma(ec_, inv_r, g)));
                }
            } else if (!excl) {
                float ec_ = erfcf(ar);
                float cq = rmul(csc, qq);
                e_coul = rmul(cq, rfma(ec_, inv_r, -(float)s.wolf_ec));
                float g = rmul(rmul(alpha, (float)FRAC_2_SQRT_PI), __expf(rmul(-ar, ar)));
                float factor = rfma(ec_, inv_r2, rmul(g, inv_r));
                fr = radd(fr, rmul(rmul(cq, rsub(factor, (float)s.wolf_fc)), inv_r));
            }
        }
    }
    float gx = rmul(fr, dx), gy = rmul(fr, dy), gz = rmul(fr, dz);
    // TwoSum-compensated: the lane's sum is (nearly always) the exact sum
    // rounded once, whatever the order of its terms, so a force does not
    // depend on which list build (with entries beyond the cutoff placed
    // differently) its row came from.  (A plain sum measured 4 % faster with
    // the same 1.5e-6 force RMS error, but made trajectories depend on the
    // rebuild history.)
    two_sum_acc(A.fxs, A.fxc, gx);
    two_sum_acc(A.fys, A.fyc, gy);
    two_sum_acc(A.fzs, A.fzc, gz);
    if (EV && js > tt) {  // each unordered pair once (the list is symmetric)
        A.ep += (double)e_pair;
        A.ec += (double)e_coul + e_coul_d;
        A.w0 += (double)rmul(gx, dx);
        A.w1 += (double)rmul(gx, dy);
        A.w2 += (double)rmul(gx, dz);
        A.w3 += (double)rmul(gy, dy);
        A.w4 += (double)rmul(gy, dz);
        A.w5 += (double)rmul(gz, dz);
    }
}

// Combines the compensated force sums of a TPA-lane group (FP32 shuffles, in
// a fixed butterfly order); every lane ends with the group's sums.
template <int TPA>
__device__ __forceinline__ void group_combine(MixedAcc& A) {
#pragma unroll
    for (int o = TPA / 2; o > 0; o >>= 1) {
        float sx = __shfl_xor_sync(0xffffffffu, A.fxs, o), cx = __shfl_xor_sync(0xffffffffu, A.fxc, o);
        float sy = __shfl_xor_sync(0xffffffffu, A.fys, o), cy = __shfl_xor_sync(0xffffffffu, A.fyc, o);
        float sz = __shfl_xor_sync(0xffffffffu, A.fzs, o), cz = __shfl_xor_sync(0xffffffffu, A.fzc, o);
        two_sum_acc(A.fxs, A.fxc, sx);
        A.fxc = radd(A.fxc, cx);
        two_sum_acc(A.fys, A.fyc, sy);
        A.fyc = radd(A.fyc, cy);
        two_sum_acc(A.fzs, A.fzc, sz);
        A.fzc = radd(A.fzc, cz);
    }
}

// Walks one atom's neighbour row for lane `sub` of its TPA-lane group: the
// lane takes pairs of adjacent entries (one 8-byte load of the indices, a
// group of lanes reading contiguous bytes, the next pair's load issued ahead),
// issues both gathers, then evaluates the two entries in order; an odd last
// entry is taken alone.  The
// per-step pair kernel and the persistent kernel both walk rows this way, so
// their force sums run in the same order.  (Blocks of four entries measured
// slower: the extra registers cost occupancy.)
template <int TPA, typename Gather, typename Eval>
__device__ __forceinline__ void walk_row(const int* __restrict__ list, int cnt, int sub, Gather gather, Eval eval) {
    // the lane's pairs start at 2 sub, 2 sub + 2 TPA, ...; the next pair's
    // indices are loaded while this pair is gathered and evaluated
    int k = 2 * sub;
    int2 js = k + 1 < cnt ? *reinterpret_cast<const int2*>(list + k) : make_int2(0, 0);
    while (k + 1 < cnt) {
        const int kn = k + 2 * TPA;
        int2 jn = kn + 1 < cnt ? *reinterpret_cast<const int2*>(list + kn) : js;
        uint4 p0, p1;
        int2 m0, m1;
        gather(js.x, p0, m0);
        gather(js.y, p1, m1);
        eval(js.x, p0, m0);
        eval(js.y, p1, m1);
        js = jn;
        k = kn;
    }
    if (k < cnt) {  // an odd last entry
        int j = list[k];
        uint4 p0;
        int2 m0;
        gather(j, p0, m0);
        eval(j, p0, m0);
    }
}

}  // namespace lg
