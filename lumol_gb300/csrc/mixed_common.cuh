// mixed_common.cuh -- device helpers of the mixed-precision pair evaluation,
// shared by the per-step pair kernel (mixed.cu) and the persistent batched MD
// kernel (persist.cu).
#pragma once
#include "kernels.h"

namespace lg {

__device__ __forceinline__ void two_sum_acc(float& s, float& c, float x) {
    float t = s + x;
    float bp = t - s;
    float err = (s - (t - bp)) + (x - bp);
    s = t;
    c += err;
}

template <int TPA>
__device__ __forceinline__ double group_sum_d(double v) {
#pragma unroll
    for (int o = TPA / 2; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Minimum image of two fixed-point coordinates: signed wrap-around difference.
__device__ __forceinline__ float fixed_image(uint32_t ui, uint32_t uj, float scale) {
    return (float)(int32_t)(ui - uj) * scale;
}

// Pair potential in FP32: returns energy, writes force / r.
__device__ __forceinline__ float pair_mixed(const PairDevF& p, float r2, float inv_r2, float inv_r, float& fr) {
    switch (p.type) {
        case 2: {  // LJ: c12 / r^12 - c6 / r^6
            float ir6 = inv_r2 * inv_r2 * inv_r2;
            float e = ir6 * (p.a * ir6 - p.b);
            fr = ir6 * (12.0f * p.a * ir6 - 6.0f * p.b) * inv_r2;
            return e - p.shift;
        }
        case 3: {  // Buckingham: A exp(-r / rho) - C / r^6
            float r = r2 * inv_r;
            float ex = p.a * __expf(-r * p.c);
            float ir6 = inv_r2 * inv_r2 * inv_r2;
            fr = ex * p.c * inv_r - 6.0f * p.b * ir6 * inv_r2;
            return ex - p.b * ir6 - p.shift;
        }
        case 4: {  // Harmonic k / 2 (r - x0)^2
            float r = r2 * inv_r;
            float dx = r - p.b;
            fr = -p.a * dx * inv_r;
            return 0.5f * p.a * dx * dx - p.shift;
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
template <bool EV, bool GENERAL>
__device__ __forceinline__ void mixed_entry(
    MixedAcc& A, const SysDev& s, const PairDevF* __restrict__ prow, uint4 pi, float qi, int mi, int i, int tt,
    int js, uint4 pj, int2 kmj, const int* __restrict__ order, const int* __restrict__ spec_off,
    const int* __restrict__ spec_j, const int8_t* __restrict__ spec_path, bool pairs, bool coul, float coul_rc2,
    float alpha, float pref, bool single, int4 ph1, float4 pq1) {
    float qj = __uint_as_float(pj.w);
    float dx = fixed_image(pi.x, pj.x, s.Lq[0]);
    float dy = fixed_image(pi.y, pj.y, s.Lq[1]);
    float dz = fixed_image(pi.z, pj.z, s.Lq[2]);
    float r2 = dx * dx + dy * dy + dz * dz;
    // the parameters as two 16-byte loads: (type, restriction, -, -) and (a, b, c, rc2);
    // a system with one kind passes them in (loaded once per atom)
    const PairDevF* pp = prow + kmj.x;
    int4 ph;
    float4 pq;
    if (single) {
        ph = ph1;
        pq = pq1;
    } else {
        ph = __ldg(reinterpret_cast<const int4*>(pp));
        pq = __ldg(reinterpret_cast<const float4*>(pp) + 1);
    }
    bool pin = pairs && ph.x != 0 && r2 < pq.w;
    bool cin = GENERAL && coul && qj != 0.0f && r2 <= coul_rc2;
    if (!(pin || cin)) return;
    float inv_r = rsqrtf(r2);
    float inv_r2 = inv_r * inv_r;
    float fr = 0.0f;
    float e_pair = 0.0f, e_coul = 0.0f;
    if (!GENERAL) {
        float shift = EV ? __ldg(&pp->shift) : 0.0f;
        if (ph.x == 2) {  // LJ: c12 / r^12 - c6 / r^6
            float ir6 = inv_r2 * inv_r2 * inv_r2;
            fr = ir6 * (12.0f * pq.x * ir6 - 6.0f * pq.y) * inv_r2;
            if (EV) e_pair = ir6 * (pq.x * ir6 - pq.y) - shift;
        } else {
            e_pair = pair_mixed(*pp, r2, inv_r2, inv_r, fr);
        }
    } else {
        int path = -1;
        int mj = kmj.y;
        float sc = 1.0f;
        const PairDevF& p = *pp;
        if (pin && ph.y != 0) {
            path = ph.y <= 2 ? (mi != mj ? 0 : 5) : bond_path(i, order[js], mi, mj, spec_off, spec_j, spec_path);
            if (restriction_excluded(ph.y, path)) pin = false;
            else sc = ph.y == 6 && path == 4 ? p.scale14 : 1.0f;
        }
        if (pin) {
            float f;
            e_pair = sc * pair_mixed(p, r2, inv_r2, inv_r, f);
            fr = sc * f;
        }
        if (cin) {
            bool excl = false;
            float csc = 1.0f;
            if (s.coul_restr != 0) {
                if (path < 0 || (s.coul_restr > 2 && path == 5))
                    path = s.coul_restr <= 2 ? (mi != mj ? 0 : 5)
                                             : bond_path(i, order[js], mi, mj, spec_off, spec_j, spec_path);
                excl = restriction_excluded(s.coul_restr, path);
                if (s.coul_restr == 6 && path == 4) csc = (float)s.coul_scale14;
            }
            float qq = pref * qj;
            float r = r2 * inv_r;
            float ar = alpha * r;
            if (s.coul == 1) {
                float g = alpha * (float)FRAC_2_SQRT_PI * __expf(-ar * ar);
                if (excl) {
                    float ef = erff(ar);
                    e_coul = -qq * ef * inv_r;
                    fr += qq * inv_r2 * (g - ef * inv_r);
                } else {
                    float ec_ = erfcf(ar);
                    e_coul = qq * ec_ * inv_r;
                    fr += qq * inv_r2 * (g + ec_ * inv_r);
                }
            } else if (!excl) {
                float ec_ = erfcf(ar);
                e_coul = csc * qq * (ec_ * inv_r - (float)s.wolf_ec);
                float factor = ec_ * inv_r2 + alpha * (float)FRAC_2_SQRT_PI * __expf(-ar * ar) * inv_r;
                fr += csc * qq * (factor - (float)s.wolf_fc) * inv_r;
            }
        }
    }
    float gx = fr * dx, gy = fr * dy, gz = fr * dz;
    two_sum_acc(A.fxs, A.fxc, gx);
    two_sum_acc(A.fys, A.fyc, gy);
    two_sum_acc(A.fzs, A.fzc, gz);
    if (EV && js > tt) {  // each unordered pair once (the list is symmetric)
        A.ep += (double)e_pair;
        A.ec += (double)e_coul;
        A.w0 += (double)(gx * dx);
        A.w1 += (double)(gx * dy);
        A.w2 += (double)(gx * dz);
        A.w3 += (double)(gy * dy);
        A.w4 += (double)(gy * dz);
        A.w5 += (double)(gz * dz);
    }
}

}  // namespace lg
