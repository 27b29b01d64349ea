// forces.cu -- FP64 force / energy / virial kernels of the plain path.
//
// Pair potentials (sys/compute.rs:30-59, sys/energy.rs:32-59, compute.rs:198-231)
// and real-space Coulomb (ewald.rs:383-530, wolf.rs:90-282) run over the
// neighbour list in two passes: each pair is evaluated once (row i, j > i) and
// its force stored, then every atom gathers the forces of its j < i pairs.  No
// force is scattered with atomics, so every atom's force is summed in a fixed
// order and results do not depend on the rest of the batch.  Energies and
// virials go to per-atom slots that a per-system reduction adds up in a fixed
// order.
#include "kernels.h"

namespace lg {

// The reference's decision whether pair (i, j) contributes, for one family,
// shared by the force kernel and the pair-set export so both see the same set.
struct PairDecision {
    bool pair_in;      // pair potential contributes (r < cutoff, not excluded)
    bool coul_in;      // real-space Coulomb contributes
    bool coul_excl;    // Ewald excluded-pair correction (-erf term)
    double pair_scale; // restriction scaling of the pair potential
    double coul_scale; // restriction scaling of Wolf
};

// Restrictions (restrictions.rs:85-115) of a pair whose cutoff tests are
// already decided: pin = the pair potential is within its cutoff, cin = the
// real-space Coulomb term is within its cutoff (both charges non-zero).
__device__ __forceinline__ PairDecision restrict_pair(const SysDev& s, const PairDev& p, bool pin, bool cin,
                                                      int i, int j, int mi, int mj, const int* spec_off,
                                                      const int* spec_j, const int8_t* spec_path) {
    PairDecision d{false, false, false, 1.0, 1.0};
    int path = -1;
    if (pin) {  // pairs.rs:185-218
        if (p.restriction != 0) {
            path = (p.restriction <= 2) ? (mi != mj ? 0 : 5)
                                        : bond_path(i, j, mi, mj, spec_off, spec_j, spec_path);
            if (!restriction_excluded(p.restriction, path)) {
                d.pair_in = true;
                d.pair_scale = restriction_scaling(p.restriction, path, p.scale14);
            }
        } else {
            d.pair_in = true;
        }
    }
    if (cin) {
        bool excl = false;
        if (s.coul_restr != 0) {
            if (path < 0 || (s.coul_restr > 2 && path == 5 && mi == mj))
                path = (s.coul_restr <= 2) ? (mi != mj ? 0 : 5)
                                           : bond_path(i, j, mi, mj, spec_off, spec_j, spec_path);
            excl = restriction_excluded(s.coul_restr, path);
            d.coul_scale = restriction_scaling(s.coul_restr, path, s.coul_scale14);
        }
        if (s.coul == 1) {  // Ewald: excluded pairs get the -erf correction (ewald.rs:390-397)
            d.coul_in = true;
            d.coul_excl = excl;
        } else {  // Wolf: excluded pairs are skipped (wolf.rs:186-189)
            d.coul_in = !excl;
        }
    }
    return d;
}

// The reference's decision with its own cutoff tests on the exact distance r
// (pairs: r >= cutoff is out, pairs.rs:185-218; Coulomb: r > cutoff is out,
// ewald.rs:387-428, wolf.rs:90-117).
__device__ __forceinline__ PairDecision decide_pair(const SysDev& s, const PairDev& p, uint32_t terms,
                                                    int i, int j, int mi, int mj, double qi, double qj,
                                                    double r, const int* spec_off, const int* spec_j,
                                                    const int8_t* spec_path) {
    bool pin = (terms & 1u) && p.type != 0 && !(r >= p.cutoff);
    bool cin = (terms & 16u) && s.coul != 0 && qi != 0.0 && qj != 0.0 && !(r > s.coul_rc);
    return restrict_pair(s, p, pin, cin, i, j, mi, mj, spec_off, spec_j, spec_path);
}

template <int TPA>
__device__ __forceinline__ double group_sum(double v) {
#pragma unroll
    for (int o = TPA / 2; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Relative half-width of the band around a cutoff^2 inside which the FP32
// classification of a pair defers to the reference's exact geometry.  The
// FP32 distance from the fixed-point copies carries a relative error below
// 1e-6, so a pair outside the band is on the same side of the cutoff in FP32
// as in the reference's FP64 test.
constexpr float CUT_BAND = 4.0e-5f;

// Minimum image of an interior pair (|d| well below L / 2, so the nearest
// integer of d / L is never in doubt).
__device__ __forceinline__ double fast_image(double d, double L, double invL) {
    return fma(-rint(d * invL), L, d);
}

// Half-list pair kernel of the plain path: TPA threads per atom (1..32,
// autotuned) walk the j > i tail of atom i's sorted row.  Each entry is first
// classified in FP32 on the fixed-point copies: clearly outside every cutoff
// (skipped, no FP64 work), clearly inside (FP64 arithmetic without the exact
// geometry's fallbacks; LJ from 1 / r^2 without a square root), or near a
// cutoff (the reference's exact geometry and cutoff test, so the pair set is
// the reference's bit for bit).  The pair force is added to atom i's sum and
// stored for atom j, which reads it back in pair_gather_kernel; energies and
// virials count each pair once.  All sums run in a fixed order.
template <int TPA, bool EV, bool GENERAL>
__global__ void __launch_bounds__(256) pair_half_kernel(
    int n, const double4_32a* __restrict__ posq, const uint4* __restrict__ pfx, const int* __restrict__ kind,
    const int* __restrict__ mol, const int* __restrict__ sysid, const SysDev* __restrict__ sys,
    const PairDev* __restrict__ ptab, const int* __restrict__ nbr, const int* __restrict__ nnb,
    const int* __restrict__ nlo, int maxnb, const int* __restrict__ spec_off, const int* __restrict__ spec_j,
    const int8_t* __restrict__ spec_path, uint32_t terms, double* __restrict__ force,
    double4_32a* __restrict__ pf, double* __restrict__ red) {
    int gt = blockIdx.x * blockDim.x + threadIdx.x;
    int i = gt / TPA;
    int sub = gt % TPA;
    bool active = i < n;
    int ii = active ? i : n - 1;
    const SysDev& s = sys[sysid[ii]];
    double4_32a pi = posq[ii];
    uint4 ui = pfx[ii];
    int ki = kind[ii], mi = mol[ii];
    const PairDev* prow = ptab + s.ptab + ki * s.nk;
    bool pairs = (terms & 1u) != 0;
    bool coul_i = GENERAL && (terms & 16u) && s.coul != 0 && pi.w != 0.0;
    float crc2 = s.coul_rc2_f;
    double fx = 0.0, fy = 0.0, fz = 0.0;
    double ep = 0.0, ec = 0.0;
    double wxx = 0.0, wxy = 0.0, wxz = 0.0, wyy = 0.0, wyz = 0.0, wzz = 0.0;
    int cnt = active ? nnb[ii] : 0;
    int k0 = active ? nlo[ii] : 0;
    const int* list = nbr + (size_t)ii * maxnb;
    double4_32a* out = pf + (size_t)ii * maxnb;
    for (int k = k0 + sub; k < cnt; k += TPA) {
        int j = list[k];
        uint4 uj = pfx[j];
        float dxf, dyf, dzf;
        fixed_delta(s, ui, uj, dxf, dyf, dzf);
        float r2f = dxf * dxf + dyf * dyf + dzf * dzf;
        const PairDev& p = prow[kind[j]];
        bool pc = pairs && p.type != 0;
        bool cc = coul_i && __uint_as_float(uj.w) != 0.0f;
        float prc2 = p.cutoff2_f;
        bool band = (pc && fabsf(r2f - prc2) <= CUT_BAND * prc2) || (cc && fabsf(r2f - crc2) <= CUT_BAND * crc2);
        bool pin = pc && r2f < prc2;
        bool cin = cc && r2f < crc2;
        double gx = 0.0, gy = 0.0, gz = 0.0;
        if (band || pin || cin) {
            double4_32a pj = posq[j];
            double dx, dy, dz, r = 0.0, r2 = 0.0;
            PairDecision dec;
            // (a triclinic cell takes the exact geometry for every pair)
            const bool exact = band || s.tric;
            if (exact) {
                exact_nearest_image(s, pi.x, pi.y, pi.z, pj.x, pj.y, pj.z, dx, dy, dz);
                r = exact_norm(dx, dy, dz);
                dec = decide_pair(s, p, terms, i, j, mi, mol[j], pi.w, pj.w, r, spec_off, spec_j, spec_path);
            } else {
                dx = fast_image(pi.x - pj.x, s.L[0], s.invL[0]);
                dy = fast_image(pi.y - pj.y, s.L[1], s.invL[1]);
                dz = fast_image(pi.z - pj.z, s.L[2], s.invL[2]);
                r2 = fma(dx, dx, fma(dy, dy, dz * dz));
                if (GENERAL) dec = restrict_pair(s, p, pin, cin, i, j, mi, mol[j], spec_off, spec_j, spec_path);
                else dec = PairDecision{pin, false, false, 1.0, 1.0};
            }
            double f_over_r = 0.0, e_p = 0.0, e_c = 0.0;
            if (!exact && dec.pair_in && p.type == 2 && !dec.coul_in) {
                // interior LJ: c12 / r^12 - c6 / r^6 from 1 / r^2
                double inv_r2 = __drcp_rn(r2);
                double ir6 = inv_r2 * inv_r2 * inv_r2;
                f_over_r = dec.pair_scale * (ir6 * (12.0 * p.c12 * ir6 - 6.0 * p.c6) * inv_r2);
                if (EV) e_p = dec.pair_scale * (ir6 * (p.c12 * ir6 - p.c6) - p.shift);
            } else if (dec.pair_in || dec.coul_in) {
                if (!exact) r = sqrt(r2);
                double inv_r = 1.0 / r;
                if (dec.pair_in) {
                    double e, f;
                    pair_energy_force(p, r, inv_r, e, f);
                    f_over_r += dec.pair_scale * f * inv_r;
                    e_p = dec.pair_scale * e;
                }
                if (GENERAL && dec.coul_in) {
                    double e, fr;
                    if (s.coul == 1) {
                        ewald_real_pair(s.alpha, dec.coul_excl, pi.w * pj.w, r, inv_r, e, fr);
                    } else {
                        wolf_pair(s, pi.w * pj.w, r, inv_r, e, fr);
                        e *= dec.coul_scale;
                        fr *= dec.coul_scale;
                    }
                    f_over_r += fr;
                    e_c = e;
                }
            }
            gx = f_over_r * dx;
            gy = f_over_r * dy;
            gz = f_over_r * dz;
            fx += gx;
            fy += gy;
            fz += gz;
            if (EV) {
                ep += e_p;
                ec += e_c;
                wxx += gx * dx;
                wxy += gx * dy;
                wxz += gx * dz;
                wyy += gy * dy;
                wyz += gy * dz;
                wzz += gz * dz;
            }
        }
        out[k] = make_double4_32a(gx, gy, gz, 0.0);  // the force on i; j reads it back negated
    }
    fx = group_sum<TPA>(fx);
    fy = group_sum<TPA>(fy);
    fz = group_sum<TPA>(fz);
    if (EV) {
        ep = group_sum<TPA>(ep);
        ec = group_sum<TPA>(ec);
        wxx = group_sum<TPA>(wxx);
        wxy = group_sum<TPA>(wxy);
        wxz = group_sum<TPA>(wxz);
        wyy = group_sum<TPA>(wyy);
        wyz = group_sum<TPA>(wyz);
        wzz = group_sum<TPA>(wzz);
    }
    if (active && sub == 0) {  // the first force kernel of a step: assigns
        force[3 * i] = fx;
        force[3 * i + 1] = fy;
        force[3 * i + 2] = fz;
        if (EV) {
            // Wolf self energy, subtracted once per charged atom (wolf.rs:205)
            if ((terms & 16u) && s.coul == 2 && pi.w != 0.0)
                ec -= pi.w * pi.w * 0.5 * (s.wolf_ec + s.alpha * FRAC_2_SQRT_PI) / FOUR_PI_EPSILON_0;
            double* rr = red + (size_t)i * RED_STRIDE;
            rr[E_PAIRS] += ep;
            rr[E_COUL] += ec;
            double* w = rr + N_ESLOT;
            w[0] += wxx; w[1] += wxy; w[2] += wxz;
            w[3] += wxy; w[4] += wyy; w[5] += wyz;
            w[6] += wxz; w[7] += wyz; w[8] += wzz;
        }
    }
}

// The j < i head of each row: minus the stored forces of pairs (j, i), read
// through the reverse index, added to the atom's force in row order.
template <int TPA>
__global__ void __launch_bounds__(256) pair_gather_kernel(int n, const int* __restrict__ nbr,
                                                          const int* __restrict__ nlo, const int* __restrict__ rev,
                                                          int maxnb, const double4_32a* __restrict__ pf,
                                                          double* __restrict__ force) {
    int gt = blockIdx.x * blockDim.x + threadIdx.x;
    int i = gt / TPA;
    int sub = gt % TPA;
    bool active = i < n;
    int ii = active ? i : n - 1;
    int head = active ? nlo[ii] : 0;
    const int* list = nbr + (size_t)ii * maxnb;
    const int* rrow = rev + (size_t)ii * maxnb;
    double fx = 0.0, fy = 0.0, fz = 0.0;
    for (int k = sub; k < head; k += TPA) {
        double4_32a f = pf[(size_t)list[k] * maxnb + rrow[k]];
        fx -= f.x;
        fy -= f.y;
        fz -= f.z;
    }
    fx = group_sum<TPA>(fx);
    fy = group_sum<TPA>(fy);
    fz = group_sum<TPA>(fz);
    if (active && sub == 0) {
        force[3 * i] += fx;
        force[3 * i + 1] += fy;
        force[3 * i + 2] += fz;
    }
}

template <int TPA, bool EV, bool GENERAL>
void launch_pair_half(const Batch& b, uint32_t terms, unsigned grid, cudaStream_t st) {
    pair_half_kernel<TPA, EV, GENERAL><<<grid, 256, 0, st>>>(b.n, b.posq, b.posfx, b.kind, b.mol, b.sysid, b.sys,
                                                             b.ptab, b.nbr, b.nnb, b.nlo, b.maxnb, b.spec_off,
                                                             b.spec_j, b.spec_path, terms, b.force, b.pf, b.red);
}

template <int TPA>
void launch_pair_fp64_tpa(const Batch& b, uint32_t terms, bool ev, cudaStream_t st) {
    long long threads = (long long)b.n * TPA;
    unsigned grid = (unsigned)((threads + 255) / 256);
    // the pairs-only variant when nothing in the batch needs restrictions or Coulomb
    if (b.pair_general) {
        if (ev) launch_pair_half<TPA, true, true>(b, terms, grid, st);
        else launch_pair_half<TPA, false, true>(b, terms, grid, st);
    } else {
        if (ev) launch_pair_half<TPA, true, false>(b, terms, grid, st);
        else launch_pair_half<TPA, false, false>(b, terms, grid, st);
    }
    pair_gather_kernel<TPA><<<grid, 256, 0, st>>>(b.n, b.nbr, b.nlo, b.rev, b.maxnb, b.pf, b.force);
}

void launch_pair_forces(const Batch& b, uint32_t terms, bool ev, cudaStream_t st) {
    if (b.n == 0) return;
    if (b.precision == 1) {
        launch_pair_mixed(b, terms, ev, st);
        return;
    }
    switch (b.tpa) {
        case 1: launch_pair_fp64_tpa<1>(b, terms, ev, st); break;
        case 2: launch_pair_fp64_tpa<2>(b, terms, ev, st); break;
        case 4: launch_pair_fp64_tpa<4>(b, terms, ev, st); break;
        case 8: launch_pair_fp64_tpa<8>(b, terms, ev, st); break;
        case 16: launch_pair_fp64_tpa<16>(b, terms, ev, st); break;
        default: launch_pair_fp64_tpa<32>(b, terms, ev, st); break;
    }
}

// ---------------------------------------------------------------------------
// Bonds, angles and dihedrals, gathered per atom (compute.rs:62-96, 233-241;
// energy.rs:90-141; UnitCell::angle_and_derivatives, cells.rs:335-362;
// UnitCell::dihedral_and_derivatives, cells.rs:364-411).
// ---------------------------------------------------------------------------
// Energy and force of an angle or dihedral potential at x (par = (k, x0,
// extra, kind), k NaN for NullPotential): Harmonic (functions.rs:135-143),
// CosineHarmonic (functions.rs:198-207), Torsion (functions.rs:244-256).
__device__ __forceinline__ double bonded_energy(const double4_32a& par, double x) {
    if (isnan(par.x)) return 0.0;
    if (par.w == 1.0) {
        double dr = cos(x) - par.z;
        return 0.5 * par.x * dr * dr;
    }
    if (par.w == 2.0) return par.x * (1.0 + cos(par.z * x - par.y));
    if (par.w == 3.0) {  // Morse: depth (1 - exp((x0 - x) a))^2 (functions.rs:415-418)
        double rc = 1.0 - exp((par.y - x) * par.z);
        return par.x * rc * rc;
    }
    double dx = x - par.y;
    return 0.5 * par.x * dx * dx;
}
__device__ __forceinline__ double bonded_force(const double4_32a& par, double x) {
    if (isnan(par.x)) return 0.0;
    if (par.w == 1.0) return par.x * (cos(x) - par.z) * sin(x);
    if (par.w == 2.0) return par.x * par.z * sin(par.z * x - par.y);
    if (par.w == 3.0) {  // Morse's force as functions.rs:420-423 writes it
        double ex = exp((par.y - x) * par.z);
        return 2.0 * par.x * (1.0 - ex * ex) * par.z;
    }
    return par.x * (par.y - x);
}

template <bool EV>
__global__ void bonded_kernel(int n, const double4_32a* __restrict__ posq, const int* __restrict__ sysid,
                              const SysDev* __restrict__ sys, const int* __restrict__ bt_off,
                              const int4* __restrict__ bt, const int* __restrict__ bt_role,
                              const double4_32a* __restrict__ bt_par, uint32_t terms,
                              double* __restrict__ force, double* __restrict__ red) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const SysDev& s = sys[sysid[i]];
    double fx = 0.0, fy = 0.0, fz = 0.0, eb = 0.0, ea = 0.0, ed = 0.0;
    double w[6] = {0, 0, 0, 0, 0, 0};
    for (int t = bt_off[i]; t < bt_off[i + 1]; t++) {
        int4 term = bt[t];
        int role = bt_role[t];
        double4_32a par = bt_par[t];  // (k, x0, extra, kind); k is NaN for a NullPotential
        bool null_pot = isnan(par.x);
        int type = term.x & 3;
        if (type == 0) {
            if (!(terms & 4u)) continue;
            double4_32a pa = posq[term.y], pb = posq[term.z];
            double dx, dy, dz;
            exact_nearest_image(s, pa.x, pa.y, pa.z, pb.x, pb.y, pb.z, dx, dy, dz);
            double r = exact_norm(dx, dy, dz);
            double f = bonded_force(par, r);  // 0 for a NullPotential
            double gx = f * (dx / r), gy = f * (dy / r), gz = f * (dz / r);
            double sgn = role == 0 ? 1.0 : -1.0;
            fx += sgn * gx;
            fy += sgn * gy;
            fz += sgn * gz;
            if (EV && role == 0) {
                eb += bonded_energy(par, r);
                w[0] += gx * dx; w[1] += gx * dy; w[2] += gx * dz;
                w[3] += gy * dy; w[4] += gy * dz; w[5] += gz * dz;
            }
        } else if (type == 1) {
            if (!(terms & 8u)) continue;
            double4_32a p1 = posq[term.y], p2 = posq[term.z], p3 = posq[term.w];
            double ax, ay, az, bx, by, bz;
            exact_nearest_image(s, p1.x, p1.y, p1.z, p2.x, p2.y, p2.z, ax, ay, az);  // r12
            exact_nearest_image(s, p3.x, p3.y, p3.z, p2.x, p2.y, p2.z, bx, by, bz);  // r23
            double n12 = exact_norm(ax, ay, az), n23 = exact_norm(bx, by, bz);
            double ux = ax / n12, uy = ay / n12, uz = az / n12;
            double vx = bx / n23, vy = by / n23, vz = bz / n23;
            double cs = ux * vx + uy * vy + uz * vz;
            double sin_inv = 1.0 / sqrt(1.0 - cs * cs);
            double theta = acos(cs);
            double f = bonded_force(par, theta);
            double gx, gy, gz;
            double d1x = sin_inv * (cs * ux - vx) / n12, d1y = sin_inv * (cs * uy - vy) / n12,
                   d1z = sin_inv * (cs * uz - vz) / n12;
            double d3x = sin_inv * (cs * vx - ux) / n23, d3y = sin_inv * (cs * vy - uy) / n23,
                   d3z = sin_inv * (cs * vz - uz) / n23;
            if (role == 0) {
                gx = d1x; gy = d1y; gz = d1z;
            } else if (role == 2) {
                gx = d3x; gy = d3y; gz = d3z;
            } else {
                gx = -(d1x + d3x); gy = -(d1y + d3y); gz = -(d1z + d3z);
            }
            fx += f * gx;
            fy += f * gy;
            fz += f * gz;
            if (EV && role == 0 && !null_pot) {
                // EnergyEvaluator::angles uses UnitCell::angle (cells.rs:322-330)
                double th = acos((ax * bx + ay * by + az * bz) / (n12 * n23));
                ea += bonded_energy(par, th);
            }
        } else {
            if (!(terms & 128u)) continue;
            double4_32a q1 = posq[term.y], q2 = posq[term.z], q3 = posq[term.w], q4 = posq[term.x >> 2];
            double r12[3], r23[3], r34[3];
            exact_nearest_image(s, q2.x, q2.y, q2.z, q1.x, q1.y, q1.z, r12[0], r12[1], r12[2]);
            exact_nearest_image(s, q3.x, q3.y, q3.z, q2.x, q2.y, q2.z, r23[0], r23[1], r23[2]);
            exact_nearest_image(s, q4.x, q4.y, q4.z, q3.x, q3.y, q3.z, r34[0], r34[1], r34[2]);
            double u[3] = {r12[1] * r23[2] - r12[2] * r23[1], r12[2] * r23[0] - r12[0] * r23[2],
                           r12[0] * r23[1] - r12[1] * r23[0]};
            double v[3] = {r23[1] * r34[2] - r23[2] * r34[1], r23[2] * r34[0] - r23[0] * r34[2],
                           r23[0] * r34[1] - r23[1] * r34[0]};
            double u2 = u[0] * u[0] + u[1] * u[1] + u[2] * u[2];
            double v2 = v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
            double r23_2 = r23[0] * r23[0] + r23[1] * r23[1] + r23[2] * r23[2];
            double r23n = sqrt(r23_2);
            double r23_r34 = r23[0] * r34[0] + r23[1] * r34[1] + r23[2] * r34[2];
            double r12_r23 = r12[0] * r23[0] + r12[1] * r23[1] + r12[2] * r23[2];
            double c1 = -r23n / u2, c4 = r23n / v2;
            double d[3];
            for (int k = 0; k < 3; k++) {
                double d1 = c1 * u[k], d4 = c4 * v[k];
                if (role == 0) d[k] = d1;
                else if (role == 3) d[k] = d4;
                else if (role == 1) d[k] = (-r12_r23 / r23_2 - 1.0) * d1 + (r23_r34 / r23_2) * d4;
                else d[k] = (-r23_r34 / r23_2 - 1.0) * d4 + (r12_r23 / r23_2) * d1;
            }
            double vs[3] = {r23n * v[0], r23n * v[1], r23n * v[2]};
            double phi = atan2(vs[0] * r12[0] + vs[1] * r12[1] + vs[2] * r12[2],
                               u[0] * v[0] + u[1] * v[1] + u[2] * v[2]);
            double f = bonded_force(par, phi);
            fx += f * d[0];
            fy += f * d[1];
            fz += f * d[2];
            if (EV && role == 0) ed += bonded_energy(par, phi);  // dihedral angles add no virial (compute.rs:241)
        }
    }
    force[3 * i] += fx;
    force[3 * i + 1] += fy;
    force[3 * i + 2] += fz;
    if (EV) {
        double* rr = red + (size_t)i * RED_STRIDE;
        rr[E_BONDS] += eb;
        rr[E_ANGLES] += ea;
        rr[E_DIHEDRALS] += ed;
        double* v = rr + N_ESLOT;
        v[0] += w[0]; v[1] += w[1]; v[2] += w[2];
        v[3] += w[1]; v[4] += w[3]; v[5] += w[4];
        v[6] += w[2]; v[7] += w[4]; v[8] += w[5];
    }
}

void launch_bonded(const Batch& b, uint32_t terms, bool ev, cudaStream_t st) {
    if (b.n == 0 || !b.bt_off) return;
    int tb = 128;
    unsigned grid = (b.n + tb - 1) / tb;
    if (ev)
        bonded_kernel<true><<<grid, tb, 0, st>>>(b.n, b.posq, b.sysid, b.sys, b.bt_off, b.bt, b.bt_role,
                                                 b.bt_par, terms, b.force, b.red);
    else
        bonded_kernel<false><<<grid, tb, 0, st>>>(b.n, b.posq, b.sysid, b.sys, b.bt_off, b.bt, b.bt_role,
                                                  b.bt_par, terms, b.force, b.red);
}

// ---------------------------------------------------------------------------
// Ewald k-space (ewald.rs:633-733)
// ---------------------------------------------------------------------------
__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
    return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

// Ewald::eik_dot_r, per-atom part: e^{i k.r} for k = 0..kmax along each axis,
// k = 1 from polar(1, k1 . r) and the others by the same recursion.
__global__ void eikr_kernel(int n, int kdim, const double4_32a* __restrict__ posq,
                            const int* __restrict__ sysid, const SysDev* __restrict__ sys,
                            double2* __restrict__ eikr) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= 3 * n) return;
    int axis = t / n, i = t - axis * n;
    const SysDev& s = sys[sysid[i]];
    if (s.coul != 1) return;
    double4_32a p = posq[i];
    double phi = axis_phase(s, axis, p.x, p.y, p.z);
    double sn, cs;
    sincos(phi, &sn, &cs);
    double2 e1 = make_double2(cs, sn);
    eikr[(size_t)(0 * 3 + axis) * n + i] = make_double2(1.0, 0.0);
    eikr[(size_t)(1 * 3 + axis) * n + i] = e1;
    double2 e = e1;
    for (int kk = 2; kk <= s.kmax; kk++) {
        e = cmul(e, e1);
        eikr[(size_t)(kk * 3 + axis) * n + i] = e;
    }
}

__device__ __forceinline__ double2 eikr_at(const double2* __restrict__ eikr, int n, int kk, int axis, int i) {
    if (kk >= 0) return eikr[(size_t)(kk * 3 + axis) * n + i];
    double2 v = eikr[(size_t)((-kk) * 3 + axis) * n + i];
    return make_double2(v.x, -v.y);
}

// rho(k) = sum_i q_i e^{i k.r_i}: one block per k-vector, fixed-order tree sum.
template <bool EV>
__global__ void __launch_bounds__(256) rho_kernel(int n, const double4_32a* __restrict__ posq,
                                                  const SysDev* __restrict__ sys,
                                                  const KVecDev* __restrict__ kvec,
                                                  const double2* __restrict__ eikr,
                                                  double2* __restrict__ rho, double* __restrict__ kred) {
    __shared__ double sre[256], sim[256];
    int k = blockIdx.x;
    KVecDev kv = kvec[k];
    const SysDev& s = sys[kv.sys];
    double re = 0.0, im = 0.0;
    for (int i = s.begin + threadIdx.x; i < s.end; i += blockDim.x) {
        double2 phi = cmul(cmul(eikr_at(eikr, n, kv.ikx, 0, i), eikr_at(eikr, n, kv.iky, 1, i)),
                           eikr_at(eikr, n, kv.ikz, 2, i));
        double q = posq[i].w;
        re += q * phi.x;
        im += q * phi.y;
    }
    sre[threadIdx.x] = re;
    sim[threadIdx.x] = im;
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
        if (EV) {
            double nrm = r.x * r.x + r.y * r.y;
            double* out = kred + (size_t)k * 7;
            out[0] = kv.energy * nrm;
            for (int c = 0; c < 6; c++) out[1 + c] = nrm * kv.virial[c];
        }
    }
}

// field_i = sum_k Im(e^{i k.r_i} conj(rho_k)) field_k over one chunk of k-vectors.
__global__ void __launch_bounds__(128) field_kernel(int n, int kchunk, const int* __restrict__ sysid,
                                                    const SysDev* __restrict__ sys,
                                                    const KVecDev* __restrict__ kvec,
                                                    const double2* __restrict__ eikr,
                                                    const double2* __restrict__ rho,
                                                    double* __restrict__ fpart) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int c = blockIdx.y;
    if (i >= n) return;
    const SysDev& s = sys[sysid[i]];
    double fx = 0.0, fy = 0.0, fz = 0.0;
    if (s.coul == 1) {
        int k0 = s.kbegin + c * kchunk;
        int k1 = min(k0 + kchunk, s.kend);
        for (int k = k0; k < k1; k++) {
            const KVecDev& kv = kvec[k];
            double2 e = cmul(cmul(eikr_at(eikr, n, kv.ikx, 0, i), eikr_at(eikr, n, kv.iky, 1, i)),
                             eikr_at(eikr, n, kv.ikz, 2, i));
            double2 r = rho[k];
            double imag = e.x * (-r.y) + e.y * r.x;
            fx += imag * kv.field[0];
            fy += imag * kv.field[1];
            fz += imag * kv.field[2];
        }
    }
    double* out = fpart + (size_t)c * 3 * n + 3 * (size_t)i;
    out[0] = fx;
    out[1] = fy;
    out[2] = fz;
}

// force_i += q_i field_i / (4 pi eps0) (ewald.rs:716-719)
__global__ void field_reduce_kernel(int n, int nchunks, const double4_32a* __restrict__ posq,
                                    const int* __restrict__ sysid, const SysDev* __restrict__ sys,
                                    const double* __restrict__ fpart, double* __restrict__ force) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (sys[sysid[i]].coul != 1) return;
    double f[3] = {0.0, 0.0, 0.0};
    for (int c = 0; c < nchunks; c++)
        for (int d = 0; d < 3; d++) f[d] += fpart[(size_t)c * 3 * n + 3 * (size_t)i + d];
    double q = posq[i].w;
    for (int d = 0; d < 3; d++) force[3 * i + d] += q * f[d] / FOUR_PI_EPSILON_0;
}

void launch_kspace(const Batch& b, bool forces, bool ev, cudaStream_t st) {
    if (b.nkvec == 0 || b.n == 0) return;
    if (b.precision == 1) {
        launch_kspace_mixed_part(b, 0, ev, st);
        launch_kspace_mixed_part(b, 1, ev, st);
        if (forces) launch_kspace_mixed_part(b, 2, ev, st);
        return;
    }
    int tb = 256;
    eikr_kernel<<<(3 * b.n + tb - 1) / tb, tb, 0, st>>>(b.n, b.kdim, b.posq, b.sysid, b.sys, b.eikr);
    if (ev)
        rho_kernel<true><<<b.nkvec, 256, 0, st>>>(b.n, b.posq, b.sys, b.kvec, b.eikr, b.rho, b.kred);
    else
        rho_kernel<false><<<b.nkvec, 256, 0, st>>>(b.n, b.posq, b.sys, b.kvec, b.eikr, b.rho, b.kred);
    if (forces) {
        dim3 grid((b.n + 127) / 128, b.nkchunks);
        field_kernel<<<grid, 128, 0, st>>>(b.n, b.kchunk, b.sysid, b.sys, b.kvec, b.eikr, b.rho, b.fpart);
        field_reduce_kernel<<<(b.n + 127) / 128, 128, 0, st>>>(b.n, b.nkchunks, b.posq, b.sysid, b.sys,
                                                               b.fpart, b.force);
    }
}

// One piece of launch_kspace: 0 eikr, 1 rho, 2 field + force.
void launch_kspace_part(const Batch& b, int part, bool ev, cudaStream_t st) {
    if (b.nkvec == 0 || b.n == 0) return;
    if (b.precision == 1) {
        launch_kspace_mixed_part(b, part, ev, st);
        return;
    }
    if (part == 0) {
        eikr_kernel<<<(3 * b.n + 255) / 256, 256, 0, st>>>(b.n, b.kdim, b.posq, b.sysid, b.sys, b.eikr);
    } else if (part == 1) {
        if (ev)
            rho_kernel<true><<<b.nkvec, 256, 0, st>>>(b.n, b.posq, b.sys, b.kvec, b.eikr, b.rho, b.kred);
        else
            rho_kernel<false><<<b.nkvec, 256, 0, st>>>(b.n, b.posq, b.sys, b.kvec, b.eikr, b.rho, b.kred);
    } else {
        dim3 grid((b.n + 127) / 128, b.nkchunks);
        field_kernel<<<grid, 128, 0, st>>>(b.n, b.kchunk, b.sysid, b.sys, b.kvec, b.eikr, b.rho, b.fpart);
        launch_field_reduce(b, st);
    }
}

void launch_field_reduce(const Batch& b, cudaStream_t st) {
    field_reduce_kernel<<<(b.n + 127) / 128, 128, 0, st>>>(b.n, b.nkchunks, b.posq, b.sysid, b.sys, b.fpart,
                                                           b.force);
}

// ---------------------------------------------------------------------------
// Per-system reduction of energies and virials, in a fixed order.
// out[s * RED_STRIDE]: energy of the requested terms, then the virial (9).
// host_const[s * RED_STRIDE]: tail energy, tail virial (trace / 3), Ewald self energy.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) reduce_kernel(const SysDev* __restrict__ sys,
                                                     const double* __restrict__ red,
                                                     const double* __restrict__ kred,
                                                     const double* __restrict__ host_const,
                                                     uint32_t terms, int use_kspace,
                                                     double* __restrict__ out, uint32_t* status,
                                                     uint32_t* sys_status) {
    __shared__ double sh[RED_STRIDE][256];
    int s_idx = blockIdx.x;
    const SysDev& s = sys[s_idx];
    double acc[RED_STRIDE];
    for (int c = 0; c < RED_STRIDE; c++) acc[c] = 0.0;
    for (int i = s.begin + threadIdx.x; i < s.end; i += blockDim.x) {
        const double* rr = red + (size_t)i * RED_STRIDE;
        for (int c = 0; c < RED_STRIDE; c++) acc[c] += rr[c];
    }
    if (use_kspace && s.coul == 1) {
        for (int k = s.kbegin + threadIdx.x; k < s.kend; k += blockDim.x) {
            const double* kk = kred + (size_t)k * 7;
            acc[E_KSPACE] += kk[0];
            const double* v = kk + 1;  // xx xy xz yy yz zz
            acc[N_ESLOT + 0] += v[0] / FOUR_PI_EPSILON_0;
            acc[N_ESLOT + 1] += v[1] / FOUR_PI_EPSILON_0;
            acc[N_ESLOT + 2] += v[2] / FOUR_PI_EPSILON_0;
            acc[N_ESLOT + 3] += v[1] / FOUR_PI_EPSILON_0;
            acc[N_ESLOT + 4] += v[3] / FOUR_PI_EPSILON_0;
            acc[N_ESLOT + 5] += v[4] / FOUR_PI_EPSILON_0;
            acc[N_ESLOT + 6] += v[2] / FOUR_PI_EPSILON_0;
            acc[N_ESLOT + 7] += v[4] / FOUR_PI_EPSILON_0;
            acc[N_ESLOT + 8] += v[5] / FOUR_PI_EPSILON_0;
        }
    }
    for (int c = 0; c < RED_STRIDE; c++) sh[c][threadIdx.x] = acc[c];
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o)
            for (int c = 0; c < RED_STRIDE; c++) sh[c][threadIdx.x] += sh[c][threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        const double* hc = host_const + (size_t)s_idx * RED_STRIDE;
        double e = 0.0;
        if (terms & 1u) e += sh[E_PAIRS][0];
        if (terms & 2u) e += hc[0];
        if (terms & 4u) e += sh[E_BONDS][0];
        if (terms & 8u) e += sh[E_ANGLES][0];
        if (terms & 128u) e += sh[E_DIHEDRALS][0];
        if (terms & 16u) e += sh[E_COUL][0];
        if ((terms & 32u) && s.coul == 1) e += hc[2];
        if ((terms & 64u) && s.coul == 1) e += sh[E_KSPACE][0] / FOUR_PI_EPSILON_0;
        double* o = out + (size_t)s_idx * RED_STRIDE;
        o[0] = e;
        // PotentialEnergy::compute asserts a finite energy (sys/compute.rs:125)
        if (!isfinite(e)) {
            atomicOr(status, ST_NONFINITE);
            if (sys_status) atomicOr(sys_status + s_idx, SYS_NONFINITE);
        }
        for (int c = 0; c < 9; c++) o[1 + c] = sh[N_ESLOT + c][0];
        if (terms & 2u) {
            o[1] += hc[1];
            o[5] += hc[1];
            o[9] += hc[1];
        }
    }
}

void launch_reduce(const Batch& b, uint32_t terms, bool kspace, double* out, cudaStream_t st) {
    if (b.nsys == 0) return;
    reduce_kernel<<<b.nsys, 256, 0, st>>>(b.sys, b.red, b.kred, b.host_const, terms, kspace ? 1 : 0, out,
                                          b.status, b.sys_status);
}

// ---------------------------------------------------------------------------
// Molecular virial (MolecularVirial, sys/compute.rs:278-362).  The centre of
// mass of every molecule (molecules.rs:256-264) is written to each of its
// atoms; then every atom walks the j > i part of its neighbour row and, for
// pairs of different molecules, adds w_ab (r_ab . r_ij) / r_ab^2 with w_ab the
// pair and real-space Coulomb virial of the pair (Ewald ewald.rs:533-571, Wolf
// wolf.rs:285-320) and r_ij the image of the centres' separation; with the
// k-space forces given, it also subtracts F_k,a (x) (x_a - com) (the Ewald
// k-space correction, ewald.rs:736-752).  Each atom assigns its nine slots.
// ---------------------------------------------------------------------------
__global__ void molecule_com_kernel(int nmol, const int* __restrict__ mol_start,
                                    const double4_32a* __restrict__ posq, const double4_32a* __restrict__ vel,
                                    double4_32a* __restrict__ com) {
    int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= nmol) return;
    int a0 = mol_start[m], a1 = mol_start[m + 1];
    double total = 0.0, cx = 0.0, cy = 0.0, cz = 0.0;
    for (int a = a0; a < a1; a++) {
        double4_32a p = posq[a];
        double mass = vel[a].w;
        total += mass;
        cx += mass * p.x;
        cy += mass * p.y;
        cz += mass * p.z;
    }
    double4_32a c = make_double4_32a(cx / total, cy / total, cz / total, 0.0);
    for (int a = a0; a < a1; a++) com[a] = c;
}

__global__ void __launch_bounds__(128) molecular_virial_kernel(
    int n, const double4_32a* __restrict__ posq, const int* __restrict__ kind, const int* __restrict__ mol,
    const int* __restrict__ sysid, const SysDev* __restrict__ sys, const PairDev* __restrict__ ptab,
    const int* __restrict__ nbr, const int* __restrict__ nnb, const int* __restrict__ nlo, int maxnb,
    const int* __restrict__ spec_off, const int* __restrict__ spec_j, const int8_t* __restrict__ spec_path,
    uint32_t terms, const double4_32a* __restrict__ com, const double* __restrict__ kforce,
    const int* __restrict__ perm, const int* __restrict__ cell_atoms, double* __restrict__ red) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const SysDev& s = sys[sysid[i]];
    double4_32a pi = posq[i], ci = com[i];
    int ki = kind[i], mi = mol[i];
    const PairDev* prow = ptab + s.ptab + ki * s.nk;
    double w[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    // a mixed engine's cell-sorted full list: row perm[i], entries are sorted
    // positions, each pair taken once from its lower atom; the plain path's
    // half list: row i from its first j > i
    const int row = perm ? perm[i] : i;
    const int* list = nbr + (size_t)row * maxnb;
    for (int k = perm ? 0 : nlo[i]; k < nnb[row]; k++) {
        int j = list[k];
        if (perm) {
            j = cell_atoms[j];
            if (j <= i) continue;
        }
        if (mol[j] == mi) continue;
        double4_32a pj = posq[j];
        double dx, dy, dz;
        exact_nearest_image(s, pi.x, pi.y, pi.z, pj.x, pj.y, pj.z, dx, dy, dz);
        double r = exact_norm(dx, dy, dz);
        const PairDev& p = prow[kind[j]];
        PairDecision dec = decide_pair(s, p, terms, i, j, mi, mol[j], pi.w, pj.w, r, spec_off, spec_j, spec_path);
        if (!dec.pair_in && !dec.coul_in) continue;
        double inv_r = 1.0 / r;
        double f_over_r = 0.0;
        if (dec.pair_in) {
            double e, f;
            pair_energy_force(p, r, inv_r, e, f);
            f_over_r += dec.pair_scale * f * inv_r;
        }
        if (dec.coul_in) {
            double e, fr;
            if (s.coul == 1) {
                ewald_real_pair(s.alpha, dec.coul_excl, pi.w * pj.w, r, inv_r, e, fr);
            } else {
                wolf_pair(s, pi.w * pj.w, r, inv_r, e, fr);
                fr *= dec.coul_scale;
            }
            f_over_r += fr;
        }
        double4_32a cj = com[j];
        double rx, ry, rz;
        exact_nearest_image(s, ci.x, ci.y, ci.z, cj.x, cj.y, cj.z, rx, ry, rz);
        double scale = f_over_r * (dx * rx + dy * ry + dz * rz) / (dx * dx + dy * dy + dz * dz);
        double gx = scale * dx, gy = scale * dy, gz = scale * dz;
        w[0] += gx * dx; w[1] += gx * dy; w[2] += gx * dz;
        w[3] += gy * dx; w[4] += gy * dy; w[5] += gy * dz;
        w[6] += gz * dx; w[7] += gz * dy; w[8] += gz * dz;
    }
    if (kforce != nullptr && s.coul == 1) {
        double d[3] = {pi.x - ci.x, pi.y - ci.y, pi.z - ci.z};
        for (int a = 0; a < 3; a++)
            for (int b = 0; b < 3; b++) w[3 * a + b] -= kforce[3 * i + a] * d[b];
    }
    double* out = red + (size_t)i * RED_STRIDE + N_ESLOT;
    for (int c = 0; c < 9; c++) out[c] = w[c];
}

void launch_molecular_virial(const Batch& b, uint32_t terms, double4_32a* com, const double* kforce,
                             cudaStream_t st) {
    if (b.n == 0) return;
    molecule_com_kernel<<<(b.nmol + 127) / 128, 128, 0, st>>>(b.nmol, b.mol_start, b.posq, b.vel, com);
    molecular_virial_kernel<<<(b.n + 127) / 128, 128, 0, st>>>(
        b.n, b.posq, b.kind, b.mol, b.sysid, b.sys, b.ptab, b.nbr, b.nnb, b.nlo, b.maxnb, b.spec_off, b.spec_j,
        b.spec_path, terms, com, kforce, b.perm, b.perm ? b.cell_atoms : nullptr, b.red);
}

// ---------------------------------------------------------------------------
// Pair-set export: the (i, j), i < j, that the force kernel counts, decided by
// the same decide_pair().  Order is arbitrary; the host sorts.
// ---------------------------------------------------------------------------
__global__ void pairset_kernel(int n, int family, int a_begin, int a_end, const double4_32a* __restrict__ posq,
                               const int* __restrict__ kind, const int* __restrict__ mol,
                               const int* __restrict__ sysid, const SysDev* __restrict__ sys,
                               const PairDev* __restrict__ ptab, const int* __restrict__ nbr,
                               const int* __restrict__ nnb, int maxnb, const int* __restrict__ spec_off,
                               const int* __restrict__ spec_j, const int8_t* __restrict__ spec_path,
                               const int* __restrict__ perm, const int* __restrict__ cell_atoms,
                               int* __restrict__ out, long long cap, unsigned long long* count) {
    int i = a_begin + blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a_end) return;
    const SysDev& s = sys[sysid[i]];
    double4_32a pi = posq[i];
    int ki = kind[i], mi = mol[i];
    uint32_t terms = family == 0 ? 1u : 16u;
    // a cell-sorted list (mixed engines) holds sorted positions: map back to atoms
    int row = perm ? perm[i] : i;
    for (int k = 0; k < nnb[row]; k++) {
        int j = nbr[(size_t)row * maxnb + k];
        if (perm) j = cell_atoms[j];
        if (j <= i) continue;
        double4_32a pj = posq[j];
        double dx, dy, dz;
        exact_nearest_image(s, pi.x, pi.y, pi.z, pj.x, pj.y, pj.z, dx, dy, dz);
        double r = exact_norm(dx, dy, dz);
        const PairDev& p = ptab[s.ptab + ki * s.nk + kind[j]];
        PairDecision d = decide_pair(s, p, terms, i, j, mi, mol[j], pi.w, pj.w, r, spec_off, spec_j, spec_path);
        bool in = family == 0 ? d.pair_in : d.coul_in;
        if (in) {
            unsigned long long slot = atomicAdd(count, 1ull);
            if ((long long)slot < cap) {
                out[2 * slot] = i - s.begin;
                out[2 * slot + 1] = j - s.begin;
            }
        }
    }
}

void launch_pairset(const Batch& b, int family, int a_begin, int a_end, int* out, long long cap,
                    unsigned long long* count, cudaStream_t st) {
    int tb = 128;
    int na = a_end - a_begin;
    if (na <= 0) return;
    pairset_kernel<<<(na + tb - 1) / tb, tb, 0, st>>>(b.n, family, a_begin, a_end, b.posq, b.kind, b.mol,
                                                      b.sysid, b.sys, b.ptab, b.nbr, b.nnb, b.maxnb,
                                                      b.spec_off, b.spec_j, b.spec_path, b.perm, b.cell_atoms,
                                                      out, cap, count);
}

}  // namespace lg
