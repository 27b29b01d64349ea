// md.cu -- molecular dynamics on device-resident state: the integrators of
// lumol-sim/src/md/integrators.rs (VelocityVerlet, Verlet, LeapFrog), the
// thermostats of md/thermostats.rs (Berendsen, Rescale, CSVR) and the controls
// RemoveTranslation and Rewrap of md/controls.rs, in the order of
// MolecularDynamics::propagate (md/molecular_dynamics.rs:66-76).
//
// One step is: md_first (the previous step's thermostat and controls, the
// integrator's update before the forces, the mixed path's fixed-point
// positions, the neighbour-list displacement test), the force kernels,
// md_second (the integrator's update after the forces, per-chunk kinetic
// energies and momenta).  The per-atom kernels run on tiles of VV_TILE atoms of
// one system, so per-system quantities (the thermostat factor) need no atomics
// and are summed in a fixed order.  All launches have fixed shapes, so a run
// of steps is captured once in a CUDA graph and replayed.
#include "kernels.h"

namespace lg {

// Layout changes between 3 n doubles (x, y, z per atom) and the packed
// double4 state (x, y, z plus the charge or mass, kept): one thread per double
// of the 3 n array, so the 3 n side is read or written in whole contiguous
// lines (it may be a page-locked host buffer reached over the host link).
__global__ void pack3_kernel(int n3, const double* __restrict__ src3, double* __restrict__ dst4) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n3) return;
    int i = t / 3;
    dst4[4 * i + (t - 3 * i)] = src3[t];
}
__global__ void unpack3_kernel(int n3, const double* __restrict__ src4, double* __restrict__ dst3) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n3) return;
    int i = t / 3;
    dst3[t] = src4[4 * i + (t - 3 * i)];
}
void launch_pack3(int n, const double* src3, double4_32a* dst, cudaStream_t st) {
    if (n) pack3_kernel<<<(3 * n + 255) / 256, 256, 0, st>>>(3 * n, src3, reinterpret_cast<double*>(dst));
}
void launch_unpack3(int n, const double4_32a* src, double* dst3, cudaStream_t st) {
    if (n) unpack3_kernel<<<(3 * n + 255) / 256, 256, 0, st>>>(3 * n, reinterpret_cast<const double*>(src), dst3);
}

__global__ void pack_vectors_kernel(int n, const double* __restrict__ src3, double4_32a* __restrict__ dst) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    dst[i] = make_double4_32a(src3[3 * i], src3[3 * i + 1], src3[3 * i + 2], 0.0);
}
void launch_pack_vectors(int n, const double* src3, double4_32a* dst, cudaStream_t st) {
    if (n) pack_vectors_kernel<<<(n + 255) / 256, 256, 0, st>>>(n, src3, dst);
}
void launch_unpack_vectors(int n, const double4_32a* src, double* dst3, cudaStream_t st) {
    launch_unpack3(n, src, dst3, st);
}

void launch_pack_positions(const Batch& b, const double* pos3, cudaStream_t st) { launch_pack3(b.n, pos3, b.posq, st); }
void launch_unpack_positions(const Batch& b, double* pos3, cudaStream_t st) { launch_unpack3(b.n, b.posq, pos3, st); }
void launch_pack_velocities(const Batch& b, const double* vel3, cudaStream_t st) { launch_pack3(b.n, vel3, b.vel, st); }
void launch_unpack_velocities(const Batch& b, double* vel3, cudaStream_t st) {
    launch_unpack3(b.n, b.vel, vel3, st);
}

__global__ void unpack_state_kernel(int n3, const double* __restrict__ pos4, const double* __restrict__ vel4,
                                    double* __restrict__ pos3, double* __restrict__ vel3) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n3) return;
    int i = t / 3;
    int c = 4 * i + (t - 3 * i);
    pos3[t] = pos4[c];
    vel3[t] = vel4[c];
}
__global__ void status_copy_kernel(const uint32_t* __restrict__ src, uint32_t* dst) { *dst = *src; }
void launch_status_copy(const uint32_t* status, uint32_t* dst, cudaStream_t st) {
    status_copy_kernel<<<1, 1, 0, st>>>(status, dst);
}

void launch_unpack_state(const Batch& b, double* pos3, double* vel3, cudaStream_t st) {
    if (b.n)
        unpack_state_kernel<<<(3 * b.n + 255) / 256, 256, 0, st>>>(3 * b.n, reinterpret_cast<const double*>(b.posq),
                                                                  reinterpret_cast<const double*>(b.vel), pos3,
                                                                  vel3);
}

// Marks system si for a list rebuild.  The flag store is idempotent; the
// status word gets one atomic per warp, not one per moved atom.
__device__ __forceinline__ void flag_rebuild(bool moved, int si, uint32_t* status, uint32_t* sys_rebuild) {
    unsigned mask = __ballot_sync(__activemask(), moved);
    if (moved) {
        sys_rebuild[si] = 1u;
        if ((threadIdx.x & 31) == __ffs(mask) - 1) atomicOr(status, ST_REBUILD);
    }
}

// Squared displacement since the last list build on the plain path: FP32 on
// the FP64 differences, minimum image.
__device__ __forceinline__ float plain_displacement2(const SysDev& s, const double4_32a& p, const double4_32a& b) {
    if (s.tric) return (float)image_norm2(s, p.x - b.x, p.y - b.y, p.z - b.z);
    float dx = (float)(p.x - b.x);
    float dy = (float)(p.y - b.y);
    float dz = (float)(p.z - b.z);
    dx -= rintf(dx * s.invLf[0]) * s.Lf[0];
    dy -= rintf(dy * s.invLf[1]) * s.Lf[1];
    dz -= rintf(dz * s.invLf[2]) * s.Lf[2];
    return dx * dx + dy * dy + dz * dz;
}

// The sum of the kinetic energies of gpw consecutive sorted positions in the
// order of a warp butterfly over them (v[j] += v[j + o], o = gpw / 2 ... 1):
// the tree the persistent kernel's force phase sums a chunk's atoms with.
template <int G>
__device__ __forceinline__ double butterfly_tree(const double* a, int cnt) {
    double v[G];
#pragma unroll
    for (int j = 0; j < G; j++) v[j] = j < cnt ? __ldcg(a + j) : 0.0;
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1)
#pragma unroll
        for (int j = 0; j < o; j++) v[j] = v[j] + v[j + o];
    return v[0];
}

// Kinetic energy of a mixed-path system from its atoms' kinetic energies at
// their cell-sorted positions: chunks of G sorted positions summed as the
// persistent kernel sums them, then the chunks as chunk_ke_sum adds them
// (lane-strided, in increasing order, then a butterfly), so both MD paths
// derive the same thermostat factor.  A pass computes 32 / G chunks a lane,
// their loads issued together, and adds them in order: one L2 round trip a
// pass instead of one a chunk.
template <int G>
__device__ double sorted_ke_sum_g(const SysDev& s, const double* ke, int lane) {
    constexpr int U = G >= 32 ? 1 : 32 / G;
    const int n = s.end - s.begin;
    const int nq = (n + G - 1) / G;
    double k = 0.0;
    for (int q0 = lane; q0 < nq; q0 += 32 * U) {
        double c[U];
#pragma unroll
        for (int u = 0; u < U; u++) {
            const int q = q0 + 32 * u;
            c[u] = q < nq ? butterfly_tree<G>(ke + s.begin + (size_t)q * G, min(G, n - q * G)) : 0.0;
        }
#pragma unroll
        for (int u = 0; u < U; u++)
            if (q0 + 32 * u < nq) k += c[u];
    }
    for (int o = 16; o > 0; o >>= 1) k += __shfl_xor_sync(0xffffffffu, k, o);
    return k;
}
// (Not inlined: the tree registers stay out of the integration kernels.)
static __device__ __noinline__ double sorted_ke_sum(const SysDev& s, const double* ke, int gpw, int lane) {
    switch (gpw) {
        case 1: return sorted_ke_sum_g<1>(s, ke, lane);
        case 2: return sorted_ke_sum_g<2>(s, ke, lane);
        case 4: return sorted_ke_sum_g<4>(s, ke, lane);
        case 8: return sorted_ke_sum_g<8>(s, ke, lane);
        case 16: return sorted_ke_sum_g<16>(s, ke, lane);
        default: return sorted_ke_sum_g<32>(s, ke, lane);
    }
}

// The thermostat factor and RemoveTranslation's centre-of-mass velocity of
// every system after a step (adj[4 s] = factor, adj[4 s + 1 .. 3] = the
// centre-of-mass velocity after scaling, controls.rs:29-43, else zero), one
// warp per system, from the sums md_second left: the kinetic energies in the
// persistent kernel's order (mixed path) or per chunk (plain path), the
// momenta per chunk.  Computed once per system and step; the next md_first (or
// md_finalize at the end of a run) applies it.
// RemoveRotation::control (controls.rs:47-71) on the velocities after a step,
// before the thermostat's uniform scaling (which scales the angular momentum
// and so the removed rotation alike): the centre of mass, then the angular
// momentum and the reference's inertia matrix -sum m d (x) d + trace about it,
// angular velocity = inverse(inertia) moment (types/matrix.rs:212-249), and
// v -= (x - com) ^ angular, by one warp over the system's atoms in three passes.
__device__ void remove_rotation(const SysDev& s, const double4_32a* __restrict__ posq,
                                double4_32a* __restrict__ vel, int lane) {
    double c[3] = {0.0, 0.0, 0.0};
    for (int i = s.begin + lane; i < s.end; i += 32) {
        double m = vel[i].w;
        double4_32a p = posq[i];
        c[0] = __dadd_rn(c[0], __dmul_rn(m, p.x));
        c[1] = __dadd_rn(c[1], __dmul_rn(m, p.y));
        c[2] = __dadd_rn(c[2], __dmul_rn(m, p.z));
    }
    double com[3];
    for (int d = 0; d < 3; d++) com[d] = __ddiv_rn(warp_sum(c[d]), s.total_mass);
    double L[3] = {0.0, 0.0, 0.0}, I[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (int i = s.begin + lane; i < s.end; i += 32) {
        double m = vel[i].w;
        double4_32a p = posq[i], v = vel[i];
        double d[3] = {__dsub_rn(p.x, com[0]), __dsub_rn(p.y, com[1]), __dsub_rn(p.z, com[2])};
        double vv[3] = {v.x, v.y, v.z};
        for (int k = 0; k < 3; k++) {  // moment += m (d ^ v)
            int k1 = (k + 1) % 3, k2 = (k + 2) % 3;
            L[k] = __dadd_rn(L[k], __dmul_rn(m, __dsub_rn(__dmul_rn(d[k1], vv[k2]), __dmul_rn(d[k2], vv[k1]))));
        }
        for (int a = 0; a < 3; a++)  // inertia += -m d (x) d
            for (int b = 0; b < 3; b++) I[3 * a + b] = __dadd_rn(I[3 * a + b], __dmul_rn(-m, __dmul_rn(d[a], d[b])));
    }
    for (int k = 0; k < 3; k++) L[k] = warp_sum(L[k]);
    for (int k = 0; k < 9; k++) I[k] = warp_sum(I[k]);
    double tr = __dadd_rn(__dadd_rn(I[0], I[4]), I[8]);
    I[0] = __dadd_rn(I[0], tr);
    I[4] = __dadd_rn(I[4], tr);
    I[8] = __dadd_rn(I[8], tr);
    auto e = [&](int r, int q) { return I[3 * r + q]; };
    auto dif = [&](int a, int b, int c2, int d2) {  // e(a) * e(b) - e(c) * e(d)
        return __dsub_rn(__dmul_rn(I[a], I[b]), __dmul_rn(I[c2], I[d2]));
    };
    double det = __dadd_rn(__dsub_rn(__dmul_rn(e(0, 0), dif(4, 8, 7, 5)), __dmul_rn(e(0, 1), dif(3, 8, 5, 6))),
                           __dmul_rn(e(0, 2), dif(3, 7, 4, 6)));
    double id = __ddiv_rn(1.0, det);
    double inv[9] = {__dmul_rn(dif(4, 8, 7, 5), id), __dmul_rn(dif(2, 7, 1, 8), id), __dmul_rn(dif(1, 5, 2, 4), id),
                     __dmul_rn(dif(5, 6, 3, 8), id), __dmul_rn(dif(0, 8, 2, 6), id), __dmul_rn(dif(3, 2, 0, 5), id),
                     __dmul_rn(dif(3, 7, 6, 4), id), __dmul_rn(dif(6, 1, 0, 7), id), __dmul_rn(dif(0, 4, 3, 1), id)};
    double w[3];
    for (int r = 0; r < 3; r++)
        w[r] = __dadd_rn(__dadd_rn(__dmul_rn(inv[3 * r], L[0]), __dmul_rn(inv[3 * r + 1], L[1])),
                         __dmul_rn(inv[3 * r + 2], L[2]));
    for (int i = s.begin + lane; i < s.end; i += 32) {
        double4_32a p = posq[i], v = vel[i];
        double d[3] = {__dsub_rn(p.x, com[0]), __dsub_rn(p.y, com[1]), __dsub_rn(p.z, com[2])};
        v.x = __dsub_rn(v.x, __dsub_rn(__dmul_rn(d[1], w[2]), __dmul_rn(d[2], w[1])));
        v.y = __dsub_rn(v.y, __dsub_rn(__dmul_rn(d[2], w[0]), __dmul_rn(d[0], w[2])));
        v.z = __dsub_rn(v.z, __dsub_rn(__dmul_rn(d[0], w[1]), __dmul_rn(d[1], w[0])));
        vel[i] = v;
    }
}

__global__ void __launch_bounds__(128) md_adjust_kernel(int nsys, const SysDev* __restrict__ sys,
                                                        const double* __restrict__ kepart,
                                                        const double* __restrict__ mom,
                                                        const unsigned long long* __restrict__ md_count, int gpw,
                                                        int sorted, const double4_32a* __restrict__ posq,
                                                        double4_32a* __restrict__ vel, double* __restrict__ adj) {
    int si = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
    int lane = threadIdx.x & 31;
    if (si >= nsys) return;
    const SysDev& s = sys[si];
    if (s.controls & CTL_REMOVE_ROTATION) remove_rotation(s, posq, vel, lane);
    double k = 0.0;
    if (s.thermostat != TH_NONE)
        k = sorted ? sorted_ke_sum(s, kepart, gpw, lane) : chunk_ke_sum(s, kepart, gpw, lane);
    double f = thermostat_factor(s, k, md_count[si]);
    double c[3] = {0.0, 0.0, 0.0};
    if (s.controls & CTL_REMOVE_TRANSLATION)
        for (int d = 0; d < 3; d++) c[d] = f * chunk_sum(s, mom + d, 3, gpw, lane) / s.total_mass;
    if (lane == 0) {
        adj[4 * si] = f;
        adj[4 * si + 1] = c[0];
        adj[4 * si + 2] = c[1];
        adj[4 * si + 3] = c[2];
    }
}

// v *= factor (the thermostat), then v -= centre-of-mass velocity (RemoveTranslation)
__device__ __forceinline__ void apply_adjust(const SysDev& s, const double* __restrict__ adj, double4_32a& v) {
    double f = adj[0];
    if (s.controls & CTL_REMOVE_TRANSLATION) {
        v.x = __dsub_rn(__dmul_rn(v.x, f), adj[1]);
        v.y = __dsub_rn(__dmul_rn(v.y, f), adj[2]);
        v.z = __dsub_rn(__dmul_rn(v.z, f), adj[3]);
    } else {
        v.x *= f;
        v.y *= f;
        v.z *= f;
    }
}

// The thermostat and controls of step k are computed once per system by
// md_adjust after step k and applied at the start of step k + 1 (the same
// products, in the same order, as right after step k), or by md_finalize at
// the end of a run, which saves a pass over the atoms every step.
//
// md_first: [v *= lambda; v -= v_com]; then the integrator's update before the forces
//   VelocityVerlet  v += dt/2 a; x += v dt      (integrators.rs:44-53)
//   LeapFrog        x += v dt + a dt^2 / 2     (integrators.rs:151-157)
//   Verlet          nothing (its update follows the forces)
// and the neighbour-list displacement test.  Zeroing the forces is left to
// the pair kernel, which assigns.
//
// Plain path (MIXED = false): products and sums rounded separately, as the
// reference (no FMA); the displacement test in FP32 on FP64 differences.
// Mixed path: the same FP64 state updated with fused multiply-adds (FP64
// operations are scarce on this GPU: about 1.7 per SM and clock), the
// fixed-point copy written at the atom's current cell-order slot, and the
// displacement test on fixed-point differences against the copy taken at the
// last build (no FP64 operation).
template <bool MIXED>
__global__ void __launch_bounds__(VV_TILE) md_first_kernel(
    const int2* __restrict__ tiles, const SysDev* __restrict__ sys, double4_32a* __restrict__ posq,
    double4_32a* __restrict__ vel, const double4_32a* __restrict__ acc, const double4_32a* __restrict__ pos_build,
    const uint4* __restrict__ pfx_build, const double* __restrict__ adj, int adjust, const int* __restrict__ perm,
    uint4* __restrict__ posfx, uint32_t* status, uint32_t* sys_rebuild, uint32_t* sys_status) {
    int2 tile = tiles[blockIdx.x];
    const SysDev& s = sys[tile.x];
    int i = tile.y + threadIdx.x;
    if (i >= s.end) return;
    double hdt = s.hdt, dt = s.dt;
    double4_32a v = vel[i], a = acc[i], p = posq[i];
    if (adjust) apply_adjust(s, adj + 4 * tile.x, v);
    if (s.integrator == MD_VERLET) {  // positions move after the forces
        vel[i] = v;
        return;
    }
    const bool leap = s.integrator == MD_LEAP_FROG;
    float r2;
    if (MIXED) {
        if (leap) {
            p.x = fma(v.x, dt, fma(s.hdt2, a.x, p.x));
            p.y = fma(v.y, dt, fma(s.hdt2, a.y, p.y));
            p.z = fma(v.z, dt, fma(s.hdt2, a.z, p.z));
        } else {
            v.x = fma(hdt, a.x, v.x);
            v.y = fma(hdt, a.y, v.y);
            v.z = fma(hdt, a.z, v.z);
            if (s.barostat == 2) {  // AnisoBerendsenBarostat: x = eta x (integrators.rs:302-306)
                baro_scale(s.baro_m, p.x, p.y, p.z);
            } else if (s.barostat) {  // BerendsenBarostat: x *= eta, then x += v dt (integrators.rs:219-225)
                p.x *= s.baro_eta;
                p.y *= s.baro_eta;
                p.z *= s.baro_eta;
            }
            p.x = fma(v.x, dt, p.x);
            p.y = fma(v.y, dt, p.y);
            p.z = fma(v.z, dt, p.z);
        }
        uint4 u = fixed_xyz(s, p);
        store_fixed_xyz(posfx + perm[i], u);  // a rebuild this step rewrites it in the new order
        r2 = fixed_dist2_s(s, u, pfx_build[i]);  // as the persistent kernel
    } else {
        if (leap) {  // (v dt) + ((0.5 a) dt^2)
            p.x = __dadd_rn(p.x, __dadd_rn(__dmul_rn(v.x, dt), __dmul_rn(__dmul_rn(0.5, a.x), s.dt2)));
            p.y = __dadd_rn(p.y, __dadd_rn(__dmul_rn(v.y, dt), __dmul_rn(__dmul_rn(0.5, a.y), s.dt2)));
            p.z = __dadd_rn(p.z, __dadd_rn(__dmul_rn(v.z, dt), __dmul_rn(__dmul_rn(0.5, a.z), s.dt2)));
        } else {
            v.x = __dadd_rn(v.x, __dmul_rn(hdt, a.x));
            v.y = __dadd_rn(v.y, __dmul_rn(hdt, a.y));
            v.z = __dadd_rn(v.z, __dmul_rn(hdt, a.z));
            if (s.barostat == 2) {  // AnisoBerendsenBarostat: x = eta x (integrators.rs:302-306)
                baro_scale(s.baro_m, p.x, p.y, p.z);
            } else if (s.barostat) {  // BerendsenBarostat: x *= eta, then x += v dt (integrators.rs:219-225)
                p.x = __dmul_rn(p.x, s.baro_eta);
                p.y = __dmul_rn(p.y, s.baro_eta);
                p.z = __dmul_rn(p.z, s.baro_eta);
            }
            p.x = __dadd_rn(p.x, __dmul_rn(v.x, dt));
            p.y = __dadd_rn(p.y, __dmul_rn(v.y, dt));
            p.z = __dadd_rn(p.z, __dmul_rn(v.z, dt));
        }
        r2 = plain_displacement2(s, p, pos_build[i]);
        if (posfx) posfx[i] = fixed_position(s, p);  // atom order: the half-list kernel's FP32 classification
    }
    vel[i] = v;
    posq[i] = p;
    flag_nonfinite(p.x, p.y, p.z, tile.x, sys_status, status);
    // against a threshold 1 % below (skin / 2)^2: the FP32 rounding only ever
    // triggers a rebuild early
    flag_rebuild(r2 > s.rebuild2_f, tile.x, status, sys_rebuild);
}

// md_second: the integrator's update after the forces
//   VelocityVerlet  a = F / m; v += dt/2 a                          (integrators.rs:55-68)
//   LeapFrog        a' = F / m; v += (a + a') dt / 2; a = a'        (integrators.rs:159-167)
//   Verlet          x' = 2 x - x_prev + dt^2 / m F; v = (x' - x_prev) / (2 dt);
//                   x_prev = x (held in the acceleration slot)      (integrators.rs:106-122)
// (a Verlet system then writes its fixed-point copy and runs the displacement
// test); with a thermostat, the kinetic energies for the next step's factor
// (mixed path: each atom's at its cell-sorted position, summed as the
// persistent kernel sums them; plain path: chunks of gpw atoms), with
// RemoveTranslation the momenta of chunks of gpw atoms (tiles start at their
// system's first atom in steps of VV_TILE, so a warp holds 32 / gpw whole chunks).  Plain path: the reference's divisions and
// unfused products; mixed path: a = F * (1 / m) in FP32 (the force is an FP32
// value) and fused multiply-adds on the FP64 state.
template <bool MIXED>
__global__ void __launch_bounds__(VV_TILE) md_second_kernel(
    const int2* __restrict__ tiles, const SysDev* __restrict__ sys, const double* __restrict__ force,
    const float* __restrict__ inv_mass, double4_32a* __restrict__ posq, double4_32a* __restrict__ vel,
    double4_32a* __restrict__ acc, const double4_32a* __restrict__ pos_build, const uint4* __restrict__ pfx_build,
    double* __restrict__ kepart, double* __restrict__ mom, unsigned long long* __restrict__ md_count, int gpw,
    const int* __restrict__ perm, uint4* __restrict__ posfx, uint32_t* status, uint32_t* sys_rebuild,
    uint32_t* sys_status) {
    int2 tile = tiles[blockIdx.x];
    const SysDev& s = sys[tile.x];
    int i = tile.y + threadIdx.x;
    double ke = 0.0, mx = 0.0, my = 0.0, mz = 0.0;
    if (i < s.end) {
        double hdt = s.hdt;
        double4_32a v = vel[i];
        double m = v.w;
        double4_32a an;  // F / m
        if (MIXED) {  // the force is an FP32 value (the compensated sum, rounded once): a = F / m in FP32
            float im = inv_mass[i];
            an = make_double4_32a((double)__fmul_rn((float)force[3 * i], im),
                                  (double)__fmul_rn((float)force[3 * i + 1], im),
                                  (double)__fmul_rn((float)force[3 * i + 2], im), 0.0);
        } else {
            an = make_double4_32a(force[3 * i] / m, force[3 * i + 1] / m, force[3 * i + 2] / m, 0.0);
        }
        if (s.integrator == MD_VERLET) {
            double4_32a p = posq[i], prev = acc[i], x = p;
            if (MIXED) {
                x.x = fma(s.dt2, an.x, 2.0 * p.x - prev.x);
                x.y = fma(s.dt2, an.y, 2.0 * p.y - prev.y);
                x.z = fma(s.dt2, an.z, 2.0 * p.z - prev.z);
                v.x = (x.x - prev.x) * s.inv_2dt;
                v.y = (x.y - prev.y) * s.inv_2dt;
                v.z = (x.z - prev.z) * s.inv_2dt;
            } else {  // (2 x - x_prev) + (dt^2 / m) F;  (x' - x_prev) / (2 dt)
                double c = __ddiv_rn(s.dt2, m), two_dt = __dmul_rn(2.0, s.dt);
                x.x = __dadd_rn(__dsub_rn(__dmul_rn(2.0, p.x), prev.x), __dmul_rn(c, force[3 * i]));
                x.y = __dadd_rn(__dsub_rn(__dmul_rn(2.0, p.y), prev.y), __dmul_rn(c, force[3 * i + 1]));
                x.z = __dadd_rn(__dsub_rn(__dmul_rn(2.0, p.z), prev.z), __dmul_rn(c, force[3 * i + 2]));
                v.x = __ddiv_rn(__dsub_rn(x.x, prev.x), two_dt);
                v.y = __ddiv_rn(__dsub_rn(x.y, prev.y), two_dt);
                v.z = __ddiv_rn(__dsub_rn(x.z, prev.z), two_dt);
            }
            acc[i] = make_double4_32a(p.x, p.y, p.z, 0.0);
            posq[i] = x;
            flag_nonfinite(x.x, x.y, x.z, tile.x, sys_status, status);
            float r2;
            if (MIXED) {
                uint4 u = fixed_position(s, x);
                posfx[perm[i]] = u;
                r2 = fixed_dist2_s(s, u, pfx_build[i]);
            } else {
                r2 = plain_displacement2(s, x, pos_build[i]);
                if (posfx) posfx[i] = fixed_position(s, x);
            }
            flag_rebuild(r2 > s.rebuild2_f, tile.x, status, sys_rebuild);
        } else if (s.integrator == MD_LEAP_FROG) {
            double4_32a a = acc[i];
            if (MIXED) {
                v.x = fma(hdt, a.x + an.x, v.x);
                v.y = fma(hdt, a.y + an.y, v.y);
                v.z = fma(hdt, a.z + an.z, v.z);
            } else {  // v + (0.5 (a + a')) dt
                v.x = __dadd_rn(v.x, __dmul_rn(__dmul_rn(0.5, __dadd_rn(a.x, an.x)), s.dt));
                v.y = __dadd_rn(v.y, __dmul_rn(__dmul_rn(0.5, __dadd_rn(a.y, an.y)), s.dt));
                v.z = __dadd_rn(v.z, __dmul_rn(__dmul_rn(0.5, __dadd_rn(a.z, an.z)), s.dt));
            }
            acc[i] = an;
        } else {
            if (MIXED) {
                v.x = fma(hdt, an.x, v.x);
                v.y = fma(hdt, an.y, v.y);
                v.z = fma(hdt, an.z, v.z);
            } else {
                v.x = __dadd_rn(v.x, __dmul_rn(hdt, an.x));
                v.y = __dadd_rn(v.y, __dmul_rn(hdt, an.y));
                v.z = __dadd_rn(v.z, __dmul_rn(hdt, an.z));
            }
            acc[i] = an;
        }
        vel[i] = v;
        flag_nonfinite(v.x, v.y, v.z, tile.x, sys_status, status);
        if (s.thermostat != TH_NONE)
            ke = MIXED ? 0.5 * m * fma(v.x, v.x, fma(v.y, v.y, v.z * v.z))
                       : 0.5 * m * (v.x * v.x + v.y * v.y + v.z * v.z);
        if (s.controls & CTL_REMOVE_TRANSLATION) {
            mx = m * v.x;
            my = m * v.y;
            mz = m * v.z;
        }
    }
    // per-system conditions: every lane of a block belongs to the tile's system
    const bool head = threadIdx.x % gpw == 0 && i < s.end;
    const size_t q = (size_t)s.begin + (i - s.begin) / gpw;
    if (s.thermostat != TH_NONE) {
        if (MIXED) {  // each atom's kinetic energy at its sorted position (the persistent kernel's order)
            if (i < s.end) kepart[perm[i]] = ke;
        } else {
            ke = chunk_butterfly(ke, gpw);
            if (head) kepart[q] = ke;
        }
    }
    if (s.controls & CTL_REMOVE_TRANSLATION) {
        mx = chunk_butterfly(mx, gpw);
        my = chunk_butterfly(my, gpw);
        mz = chunk_butterfly(mz, gpw);
        if (head) {
            mom[3 * q] = mx;
            mom[3 * q + 1] = my;
            mom[3 * q + 2] = mz;
        }
    }
    // the CSVR noise stream of the next thermostat application
    if (s.thermostat == TH_CSVR && threadIdx.x == 0 && tile.y == s.begin) md_count[tile.x] += 1ull;
}

// The pending thermostat and controls at the end of a run.
__global__ void __launch_bounds__(VV_TILE) md_finalize_kernel(const int2* __restrict__ tiles,
                                                              const SysDev* __restrict__ sys,
                                                              const double* __restrict__ adj,
                                                              double4_32a* __restrict__ vel) {
    int2 tile = tiles[blockIdx.x];
    const SysDev& s = sys[tile.x];
    int i = tile.y + threadIdx.x;
    if (i >= s.end) return;
    double4_32a v = vel[i];
    apply_adjust(s, adj + 4 * tile.x, v);
    vel[i] = v;
}

// Rewrap (controls.rs:80-89): each molecule of a system with the control is
// moved by the wrapped centre of mass minus the centre of mass
// (Molecule::wrap, sys/config/molecules.rs:287-296; center_of_mass :256-264;
// UnitCell::wrap_vector, cells.rs:263-270), one thread per molecule, in the
// reference's order of operations.  The fixed-point copies follow.
__global__ void rewrap_kernel(int nmol, const int* __restrict__ mol_start, const int* __restrict__ sysid,
                              const SysDev* __restrict__ sys, double4_32a* __restrict__ posq,
                              const double4_32a* __restrict__ vel, const int* __restrict__ perm,
                              uint4* __restrict__ posfx) {
    int mi = blockIdx.x * blockDim.x + threadIdx.x;
    if (mi >= nmol) return;
    int a0 = mol_start[mi], a1 = mol_start[mi + 1];
    if (a1 <= a0) return;
    const SysDev& s = sys[sysid[a0]];
    if (!(s.controls & CTL_REWRAP)) return;
    double total = 0.0, c[3] = {0.0, 0.0, 0.0};
    for (int a = a0; a < a1; a++) {
        double m = vel[a].w;
        double4_32a p = posq[a];
        total = __dadd_rn(total, m);
        c[0] = __dadd_rn(c[0], __dmul_rn(m, p.x));
        c[1] = __dadd_rn(c[1], __dmul_rn(m, p.y));
        c[2] = __dadd_rn(c[2], __dmul_rn(m, p.z));
    }
    double delta[3];
    if (s.tric) {  // wrap_vector's triclinic branch (cells.rs:271-279)
        double com[3], w[3];
        for (int d = 0; d < 3; d++) com[d] = w[d] = __ddiv_rn(c[d], total);
        tric_wrap(s, w);
        for (int d = 0; d < 3; d++) delta[d] = __dsub_rn(w[d], com[d]);
    } else {
        for (int d = 0; d < 3; d++) {
            double com = __ddiv_rn(c[d], total);
            double wrapped = __dsub_rn(com, __dmul_rn(floor(__ddiv_rn(com, s.L[d])), s.L[d]));
            delta[d] = __dsub_rn(wrapped, com);
        }
    }
    if (delta[0] == 0.0 && delta[1] == 0.0 && delta[2] == 0.0) return;
    for (int a = a0; a < a1; a++) {
        double4_32a p = posq[a];
        p.x = __dadd_rn(p.x, delta[0]);
        p.y = __dadd_rn(p.y, delta[1]);
        p.z = __dadd_rn(p.z, delta[2]);
        posq[a] = p;
        if (perm) posfx[perm[a]] = fixed_position(s, p);
        else if (posfx) posfx[a] = fixed_position(s, p);
    }
}

// Verlet::setup (integrators.rs:92-104): x_prev = x - v dt, in the acceleration slot.
__global__ void verlet_setup_kernel(int begin, int end, const SysDev* __restrict__ sys, int si,
                                    const double4_32a* __restrict__ posq, const double4_32a* __restrict__ vel,
                                    double4_32a* __restrict__ acc) {
    int i = begin + blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= end) return;
    double dt = sys[si].dt;
    double4_32a p = posq[i], v = vel[i];
    acc[i] = make_double4_32a(__dsub_rn(p.x, __dmul_rn(v.x, dt)), __dsub_rn(p.y, __dmul_rn(v.y, dt)),
                              __dsub_rn(p.z, __dmul_rn(v.z, dt)), 0.0);
}

// Displacement test alone, for positions set from the host.
__global__ void check_displacement_kernel(int n, const int* __restrict__ sysid, const SysDev* __restrict__ sys,
                                          const double4_32a* __restrict__ posq,
                                          const double4_32a* __restrict__ pos_build, uint32_t* status,
                                          uint32_t* sys_rebuild) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int si = sysid[i];
    const SysDev& s = sys[si];
    double4_32a p = posq[i], b = pos_build[i];
    flag_rebuild(!(image_norm2(s, p.x - b.x, p.y - b.y, p.z - b.z) <= s.half_skin2), si, status, sys_rebuild);
}

void launch_check_displacement(const Batch& b, cudaStream_t st) {
    if (b.n)
        check_displacement_kernel<<<(b.n + 255) / 256, 256, 0, st>>>(b.n, b.sysid, b.sys, b.posq, b.pos_build,
                                                                   b.status, b.sys_rebuild);
}

__global__ void request_rebuild_kernel(int nsys, uint32_t* status, uint32_t* sys_rebuild) {
    for (int s = threadIdx.x; s < nsys; s += blockDim.x) sys_rebuild[s] = 1u;
    if (threadIdx.x == 0) atomicOr(status, ST_REBUILD);
}

void launch_md_first(const Batch& b, bool adjust, cudaStream_t st) {
    if (!b.ntiles) return;
    int aj = adjust ? 1 : 0;
    if (b.precision == 1)
        md_first_kernel<true><<<b.ntiles, VV_TILE, 0, st>>>(b.tiles, b.sys, b.posq, b.vel, b.acc, b.pos_build,
                                                            b.pfx_build, b.adj, aj, b.perm, b.posfx, b.status,
                                                            b.sys_rebuild, b.sys_status);
    else
        md_first_kernel<false><<<b.ntiles, VV_TILE, 0, st>>>(b.tiles, b.sys, b.posq, b.vel, b.acc, b.pos_build,
                                                             nullptr, b.adj, aj, nullptr, b.posfx, b.status,
                                                             b.sys_rebuild, b.sys_status);
}
void launch_md_second(const Batch& b, cudaStream_t st) {
    if (!b.ntiles) return;
    int gpw = 32 / b.tpa;
    if (b.precision == 1)
        md_second_kernel<true><<<b.ntiles, VV_TILE, 0, st>>>(b.tiles, b.sys, b.force, b.inv_mass, b.posq, b.vel,
                                                             b.acc, b.pos_build, b.pfx_build, b.kepart, b.mom,
                                                             b.md_count, gpw, b.perm, b.posfx, b.status,
                                                             b.sys_rebuild, b.sys_status);
    else
        md_second_kernel<false><<<b.ntiles, VV_TILE, 0, st>>>(b.tiles, b.sys, b.force, nullptr, b.posq, b.vel,
                                                              b.acc, b.pos_build, nullptr, b.kepart, b.mom,
                                                              b.md_count, gpw, nullptr, b.posfx, b.status,
                                                              b.sys_rebuild, b.sys_status);
}
void launch_md_adjust(const Batch& b, cudaStream_t st) {
    if (b.nsys)
        md_adjust_kernel<<<(b.nsys + 3) / 4, 128, 0, st>>>(b.nsys, b.sys, b.kepart, b.mom, b.md_count, 32 / b.tpa,
                                                          b.precision == 1 ? 1 : 0, b.posq, b.vel, b.adj);
}
void launch_md_finalize(const Batch& b, cudaStream_t st) {
    if (b.ntiles) md_finalize_kernel<<<b.ntiles, VV_TILE, 0, st>>>(b.tiles, b.sys, b.adj, b.vel);
}
void launch_rewrap(const Batch& b, cudaStream_t st) {
    if (b.nmol)
        rewrap_kernel<<<(b.nmol + 127) / 128, 128, 0, st>>>(b.nmol, b.mol_start, b.sysid, b.sys, b.posq, b.vel,
                                                            b.precision == 1 ? b.perm : nullptr, b.posfx);
}
void launch_verlet_setup(const Batch& b, int s, int begin, int end, cudaStream_t st) {
    if (end > begin)
        verlet_setup_kernel<<<(end - begin + 255) / 256, 256, 0, st>>>(begin, end, b.sys, s, b.posq, b.vel, b.acc);
}
// KineticEnergy::compute (sys/compute.rs:133-144) of every system at the
// current velocities: one block per system, 0.5 m v.v per atom, a fixed-order
// tree sum.
__global__ void __launch_bounds__(256) kinetic_kernel(const SysDev* __restrict__ sys,
                                                      const double4_32a* __restrict__ vel, double* __restrict__ out) {
    __shared__ double sh[256];
    const SysDev& s = sys[blockIdx.x];
    double k = 0.0;
    for (int i = s.begin + threadIdx.x; i < s.end; i += blockDim.x) {
        double4_32a v = vel[i];
        k += 0.5 * v.w * (v.x * v.x + v.y * v.y + v.z * v.z);
    }
    sh[threadIdx.x] = k;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) out[blockIdx.x] = sh[0];
}
void launch_kinetic(const Batch& b, double* out, cudaStream_t st) {
    if (b.nsys) kinetic_kernel<<<b.nsys, 256, 0, st>>>(b.sys, b.vel, out);
}

// sum_i m_i v_i (x) v_i of each system (Stress, sys/compute.rs:466-480: the
// kinetic part, mass * v.tensorial(v)), a fixed-order tree per system, 9 entries.
__global__ void __launch_bounds__(256) kinetic_tensor_kernel(const SysDev* __restrict__ sys,
                                                             const double4_32a* __restrict__ vel,
                                                             double* __restrict__ out) {
    __shared__ double sh[6][256];
    const SysDev& s = sys[blockIdx.x];
    double k[6] = {0, 0, 0, 0, 0, 0};
    for (int i = s.begin + threadIdx.x; i < s.end; i += blockDim.x) {
        double4_32a v = vel[i];
        const double c[3] = {v.x, v.y, v.z};
        const int ia[6] = {0, 0, 0, 1, 1, 2}, ib[6] = {0, 1, 2, 1, 2, 2};
#pragma unroll
        for (int q = 0; q < 6; q++) k[q] += v.w * (c[ia[q]] * c[ib[q]]);
    }
    for (int q = 0; q < 6; q++) sh[q][threadIdx.x] = k[q];
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o)
            for (int q = 0; q < 6; q++) sh[q][threadIdx.x] += sh[q][threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        double* o9 = out + 9 * blockIdx.x;
        o9[0] = sh[0][0];
        o9[1] = o9[3] = sh[1][0];
        o9[2] = o9[6] = sh[2][0];
        o9[4] = sh[3][0];
        o9[5] = o9[7] = sh[4][0];
        o9[8] = sh[5][0];
    }
}
void launch_kinetic_tensor(const Batch& b, double* out, cudaStream_t st) {
    if (b.nsys) kinetic_tensor_kernel<<<b.nsys, 256, 0, st>>>(b.sys, b.vel, out);
}

// A system's x, y, z (and w unless keep_w: the charge or mass of the new
// description stays) moved to its new offset when the batch changes.
__global__ void carry_vectors_kernel(int n, const double4_32a* __restrict__ src, double4_32a* __restrict__ dst,
                                     int keep_w) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double4_32a v = src[i];
    if (keep_w) v.w = dst[i].w;
    dst[i] = v;
}
void launch_carry_vectors(const double4_32a* src, double4_32a* dst, int n, bool keep_w, cudaStream_t st) {
    if (n > 0) carry_vectors_kernel<<<(n + 255) / 256, 256, 0, st>>>(n, src, dst, keep_w ? 1 : 0);
}

__global__ void identity_order_kernel(int n, int* __restrict__ cell_atoms, int* __restrict__ perm) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    cell_atoms[i] = i;
    if (perm) perm[i] = i;
}
void launch_identity_order(const Batch& b, cudaStream_t st) {
    if (b.n > 0) identity_order_kernel<<<(b.n + 255) / 256, 256, 0, st>>>(b.n, b.cell_atoms, b.perm);
}

__global__ void request_rebuild_flag_kernel(uint32_t* status) { atomicOr(status, ST_REBUILD); }
void launch_request_rebuild_flag(const Batch& b, cudaStream_t st) {
    if (b.status) request_rebuild_flag_kernel<<<1, 1, 0, st>>>(b.status);
}

void launch_request_rebuild(const Batch& b, cudaStream_t st) {
    request_rebuild_kernel<<<1, 256, 0, st>>>(b.nsys, b.status, b.sys_rebuild);
}

}  // namespace lg
