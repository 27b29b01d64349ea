// md.cu -- Velocity-Verlet (lumol-sim/src/md/integrators.rs:22-70) and the
// Berendsen thermostat (md/thermostats.rs:91-121) on device-resident state.
//
// One step is: vv_first (the previous step's Berendsen scaling, half kick,
// drift, the mixed path's fixed-point positions, neighbour-list displacement
// test), the force kernels, vv_second (a = F / m, half kick, per-tile kinetic
// energy).  The per-atom kernels run on tiles of VV_TILE atoms of one system,
// so per-system quantities (the thermostat factor) need no atomics and are
// summed in a fixed order.  All launches have fixed shapes, so a run of steps
// is captured once in a CUDA graph and replayed.
#include "kernels.h"

namespace lg {

__global__ void pack_positions_kernel(int n, const double* __restrict__ pos3, double4_32a* __restrict__ posq) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double4_32a p = posq[i];
    p.x = pos3[3 * i];
    p.y = pos3[3 * i + 1];
    p.z = pos3[3 * i + 2];
    posq[i] = p;
}
__global__ void unpack_positions_kernel(int n, const double4_32a* __restrict__ posq, double* __restrict__ pos3) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double4_32a p = posq[i];
    pos3[3 * i] = p.x;
    pos3[3 * i + 1] = p.y;
    pos3[3 * i + 2] = p.z;
}
__global__ void pack_velocities_kernel(int n, const double* __restrict__ vel3, double4_32a* __restrict__ vel) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double4_32a v = vel[i];
    v.x = vel3[3 * i];
    v.y = vel3[3 * i + 1];
    v.z = vel3[3 * i + 2];
    vel[i] = v;
}
__global__ void unpack_velocities_kernel(int n, const double4_32a* __restrict__ vel, double* __restrict__ vel3) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double4_32a v = vel[i];
    vel3[3 * i] = v.x;
    vel3[3 * i + 1] = v.y;
    vel3[3 * i + 2] = v.z;
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
    if (n) unpack_velocities_kernel<<<(n + 255) / 256, 256, 0, st>>>(n, src, dst3);
}

void launch_pack_positions(const Batch& b, const double* pos3, cudaStream_t st) {
    if (b.n) pack_positions_kernel<<<(b.n + 255) / 256, 256, 0, st>>>(b.n, pos3, b.posq);
}
void launch_unpack_positions(const Batch& b, double* pos3, cudaStream_t st) {
    if (b.n) unpack_positions_kernel<<<(b.n + 255) / 256, 256, 0, st>>>(b.n, b.posq, pos3);
}
void launch_pack_velocities(const Batch& b, const double* vel3, cudaStream_t st) {
    if (b.n) pack_velocities_kernel<<<(b.n + 255) / 256, 256, 0, st>>>(b.n, vel3, b.vel);
}
void launch_unpack_velocities(const Batch& b, double* vel3, cudaStream_t st) {
    if (b.n) unpack_velocities_kernel<<<(b.n + 255) / 256, 256, 0, st>>>(b.n, b.vel, vel3);
}

// v += 0.5 dt a; x += v dt (integrators.rs:48-53), then the displacement
// since the last list build against skin / 2.  Also clears the force buffer
// that the force kernels accumulate into.
// Marks system si for a list rebuild.  The flag store is idempotent; the
// status word gets one atomic per warp, not one per moved atom.
__device__ __forceinline__ void flag_rebuild(bool moved, int si, uint32_t* status, uint32_t* sys_rebuild) {
    unsigned mask = __ballot_sync(__activemask(), moved);
    if (moved) {
        sys_rebuild[si] = 1u;
        if ((threadIdx.x & 31) == __ffs(mask) - 1) atomicOr(status, ST_REBUILD);
    }
}

// The Berendsen factor of a tile's system, computed by its first warp from the
// chunk kinetic energies of the last vv_second (the same sums in every block
// of the system, and the same as the persistent kernel's).
__device__ __forceinline__ void tile_lambda(const SysDev& s, const double* __restrict__ ke, int gpw,
                                            double* s_lambda) {
    if (threadIdx.x < 32) {
        double f = berendsen_factor(s, chunk_ke_sum(s, ke, gpw, threadIdx.x));
        if (threadIdx.x == 0) *s_lambda = f;
    }
    __syncthreads();
}

// The Berendsen scaling of step k is applied at the start of step k + 1 (the
// same products, in the same order, as scaling right after step k), and by
// thermostat_finalize at the end of a run, which saves two launches a step.
// vv_first: [v *= lambda]; v += 0.5 dt a; x += v dt (integrators.rs:45-53);
// the neighbour-list displacement test.  Zeroing the forces is left to the
// pair kernel, which assigns.
//
// Plain path (MIXED = false): products and sums rounded separately, as the
// reference (no FMA); the displacement test in FP32 on FP64 differences.
// Mixed path: the same FP64 state updated with fused multiply-adds (FP64
// operations are scarce on this GPU: about 1.7 per SM and clock), the
// fixed-point copy written at the atom's current cell-order slot, and the
// displacement test on fixed-point differences against the copy taken at the
// last build (no FP64 operation).
template <bool MIXED>
__global__ void __launch_bounds__(VV_TILE) vv_first_kernel(
    const int2* __restrict__ tiles, const SysDev* __restrict__ sys, double4_32a* __restrict__ posq,
    double4_32a* __restrict__ vel, const double4_32a* __restrict__ acc, const double4_32a* __restrict__ pos_build,
    const uint4* __restrict__ pfx_build, const double* __restrict__ kepart, int gpw, int apply_thermostat,
    const int* __restrict__ perm, uint4* __restrict__ posfx, uint32_t* status, uint32_t* sys_rebuild) {
    int2 tile = tiles[blockIdx.x];
    const SysDev& s = sys[tile.x];
    __shared__ double s_lambda;
    if (apply_thermostat) tile_lambda(s, kepart, gpw, &s_lambda);
    int i = tile.y + threadIdx.x;
    if (i >= s.end) return;
    double hdt = s.hdt, dt = s.dt;
    double4_32a v = vel[i], a = acc[i], p = posq[i];
    if (apply_thermostat) {
        double f = s_lambda;
        v.x *= f;
        v.y *= f;
        v.z *= f;
    }
    float r2;
    if (MIXED) {
        v.x = fma(hdt, a.x, v.x);
        v.y = fma(hdt, a.y, v.y);
        v.z = fma(hdt, a.z, v.z);
        p.x = fma(v.x, dt, p.x);
        p.y = fma(v.y, dt, p.y);
        p.z = fma(v.z, dt, p.z);
        uint4 u = fixed_position(s, p);
        posfx[perm[i]] = u;  // a rebuild this step rewrites it in the new order
        r2 = fixed_dist2(u, pfx_build[i], s.Lq);  // as the persistent kernel
    } else {
        v.x = __dadd_rn(v.x, __dmul_rn(hdt, a.x));
        v.y = __dadd_rn(v.y, __dmul_rn(hdt, a.y));
        v.z = __dadd_rn(v.z, __dmul_rn(hdt, a.z));
        p.x = __dadd_rn(p.x, __dmul_rn(v.x, dt));
        p.y = __dadd_rn(p.y, __dmul_rn(v.y, dt));
        p.z = __dadd_rn(p.z, __dmul_rn(v.z, dt));
        double4_32a b = pos_build[i];
        float dx = (float)(p.x - b.x);
        float dy = (float)(p.y - b.y);
        float dz = (float)(p.z - b.z);
        dx -= rintf(dx * s.invLf[0]) * s.Lf[0];
        dy -= rintf(dy * s.invLf[1]) * s.Lf[1];
        dz -= rintf(dz * s.invLf[2]) * s.Lf[2];
        r2 = dx * dx + dy * dy + dz * dz;
        if (posfx) posfx[i] = fixed_position(s, p);  // atom order: the half-list kernel's FP32 classification
    }
    vel[i] = v;
    posq[i] = p;
    // against a threshold 1 % below (skin / 2)^2: the FP32 rounding only ever
    // triggers a rebuild early
    flag_rebuild(r2 > s.rebuild2_f, tile.x, status, sys_rebuild);
}

// a = F / m; v += 0.5 dt a (integrators.rs:55-68); with a thermostat, the
// kinetic energies of the system's chunks of gpw atoms for the next step's
// factor (tiles start at their system's first atom in steps of VV_TILE, so a
// warp holds 32 / gpw whole chunks).
// Plain path: the reference's division and unfused products; mixed path:
// a = F * (1 / m) in FP32 (the force is an FP32 value) and fused multiply-adds
// on the FP64 velocity.
template <bool MIXED>
__global__ void __launch_bounds__(VV_TILE) vv_second_kernel(
    const int2* __restrict__ tiles, const SysDev* __restrict__ sys, const double* __restrict__ force,
    const float* __restrict__ inv_mass, double4_32a* __restrict__ vel, double4_32a* __restrict__ acc,
    double* __restrict__ kepart, int gpw, int thermostat) {
    int2 tile = tiles[blockIdx.x];
    const SysDev& s = sys[tile.x];
    int i = tile.y + threadIdx.x;
    double ke = 0.0;
    if (i < s.end) {
        double hdt = s.hdt;
        double4_32a v = vel[i];
        double m = v.w;
        double4_32a a;
        if (MIXED) {  // the force is an FP32 value (the compensated sum, rounded once): a = F / m in FP32
            float im = inv_mass[i];
            a = make_double4_32a((double)__fmul_rn((float)force[3 * i], im),
                                 (double)__fmul_rn((float)force[3 * i + 1], im),
                                 (double)__fmul_rn((float)force[3 * i + 2], im), 0.0);
            v.x = fma(hdt, a.x, v.x);
            v.y = fma(hdt, a.y, v.y);
            v.z = fma(hdt, a.z, v.z);
            if (thermostat) ke = 0.5 * m * fma(v.x, v.x, fma(v.y, v.y, v.z * v.z));
        } else {  // the reference's force / mass
            a = make_double4_32a(force[3 * i] / m, force[3 * i + 1] / m, force[3 * i + 2] / m, 0.0);
            v.x = __dadd_rn(v.x, __dmul_rn(hdt, a.x));
            v.y = __dadd_rn(v.y, __dmul_rn(hdt, a.y));
            v.z = __dadd_rn(v.z, __dmul_rn(hdt, a.z));
            if (thermostat) ke = 0.5 * m * (v.x * v.x + v.y * v.y + v.z * v.z);
        }
        acc[i] = a;
        vel[i] = v;
    }
    if (thermostat) {
        ke = chunk_butterfly(ke, gpw);
        if (threadIdx.x % gpw == 0 && i < s.end) kepart[s.begin + (i - s.begin) / gpw] = ke;
    }
}

// The pending Berendsen scaling at the end of a run.
__global__ void __launch_bounds__(VV_TILE) thermostat_finalize_kernel(const int2* __restrict__ tiles,
                                                                     const SysDev* __restrict__ sys,
                                                                     const double* __restrict__ kepart, int gpw,
                                                                     double4_32a* __restrict__ vel) {
    int2 tile = tiles[blockIdx.x];
    const SysDev& s = sys[tile.x];
    __shared__ double s_lambda;
    tile_lambda(s, kepart, gpw, &s_lambda);
    int i = tile.y + threadIdx.x;
    if (i >= s.end) return;
    double f = s_lambda;
    double4_32a v = vel[i];
    v.x *= f;
    v.y *= f;
    v.z *= f;
    vel[i] = v;
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
    double dx = p.x - b.x, dy = p.y - b.y, dz = p.z - b.z;
    dx -= rint(dx * s.invL[0]) * s.L[0];
    dy -= rint(dy * s.invL[1]) * s.L[1];
    dz -= rint(dz * s.invL[2]) * s.L[2];
    flag_rebuild(!(dx * dx + dy * dy + dz * dz <= s.half_skin2), si, status, sys_rebuild);
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

void launch_vv_first(const Batch& b, bool apply_thermostat, cudaStream_t st) {
    if (!b.ntiles) return;
    int th = apply_thermostat ? 1 : 0;
    if (b.precision == 1)
        vv_first_kernel<true><<<b.ntiles, VV_TILE, 0, st>>>(b.tiles, b.sys, b.posq, b.vel, b.acc, b.pos_build,
                                                            b.pfx_build, b.kepart, 32 / b.tpa, th, b.perm, b.posfx,
                                                            b.status,
                                                            b.sys_rebuild);
    else
        vv_first_kernel<false><<<b.ntiles, VV_TILE, 0, st>>>(b.tiles, b.sys, b.posq, b.vel, b.acc, b.pos_build,
                                                             nullptr, b.kepart, 32 / b.tpa, th, nullptr, b.posfx,
                                                             b.status,
                                                             b.sys_rebuild);
}
void launch_vv_second(const Batch& b, bool thermostat, cudaStream_t st) {
    if (!b.ntiles) return;
    int th = thermostat ? 1 : 0;
    if (b.precision == 1)
        vv_second_kernel<true><<<b.ntiles, VV_TILE, 0, st>>>(b.tiles, b.sys, b.force, b.inv_mass, b.vel, b.acc,
                                                             b.kepart, 32 / b.tpa, th);
    else
        vv_second_kernel<false><<<b.ntiles, VV_TILE, 0, st>>>(b.tiles, b.sys, b.force, nullptr, b.vel, b.acc,
                                                              b.kepart, 32 / b.tpa, th);
}
void launch_thermostat_finalize(const Batch& b, cudaStream_t st) {
    if (b.ntiles) thermostat_finalize_kernel<<<b.ntiles, VV_TILE, 0, st>>>(b.tiles, b.sys, b.kepart, 32 / b.tpa,
                                                                          b.vel);
}
void launch_request_rebuild(const Batch& b, cudaStream_t st) {
    request_rebuild_kernel<<<1, 256, 0, st>>>(b.nsys, b.status, b.sys_rebuild);
}

}  // namespace lg
