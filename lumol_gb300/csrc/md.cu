// md.cu -- Velocity-Verlet (lumol-sim/src/md/integrators.rs:22-70) and the
// Berendsen thermostat (md/thermostats.rs:91-121) on device-resident state.
//
// One step is: vv_first (half kick + drift + neighbour-list displacement test),
// the force kernels, vv_second (a = F / m, half kick, kinetic energy), and,
// with a thermostat, a per-system reduction of the temperature followed by the
// velocity scaling.  All launches have fixed shapes, so a step is captured once
// in a CUDA graph and replayed.
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

__global__ void vv_first_kernel(int n, const int* __restrict__ sysid, const SysDev* __restrict__ sys,
                                double4_32a* __restrict__ posq, double4_32a* __restrict__ vel,
                                const double4_32a* __restrict__ acc, const double4_32a* __restrict__ pos_build,
                                double* __restrict__ force, uint32_t* status, uint32_t* sys_rebuild) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int si = sysid[i];
    const SysDev& s = sys[si];
    // products and sums rounded separately, as the reference (no FMA)
    double hdt = __dmul_rn(0.5, s.dt);
    double4_32a v = vel[i], a = acc[i], p = posq[i];
    v.x = __dadd_rn(v.x, __dmul_rn(hdt, a.x));
    v.y = __dadd_rn(v.y, __dmul_rn(hdt, a.y));
    v.z = __dadd_rn(v.z, __dmul_rn(hdt, a.z));
    p.x = __dadd_rn(p.x, __dmul_rn(v.x, s.dt));
    p.y = __dadd_rn(p.y, __dmul_rn(v.y, s.dt));
    p.z = __dadd_rn(p.z, __dmul_rn(v.z, s.dt));
    vel[i] = v;
    posq[i] = p;
    force[3 * i] = 0.0;
    force[3 * i + 1] = 0.0;
    force[3 * i + 2] = 0.0;
    // displacement since the list build, in FP32 against a threshold 1 % below
    // (skin / 2)^2: the FP32 rounding only ever triggers a rebuild early
    double4_32a b = pos_build[i];
    float dx = (float)(p.x - b.x), dy = (float)(p.y - b.y), dz = (float)(p.z - b.z);
    dx -= rintf(dx * s.invLf[0]) * s.Lf[0];
    dy -= rintf(dy * s.invLf[1]) * s.Lf[1];
    dz -= rintf(dz * s.invLf[2]) * s.Lf[2];
    flag_rebuild(dx * dx + dy * dy + dz * dz > 0.99f * (float)s.half_skin2, si, status, sys_rebuild);
}

// a = F / m; v += 0.5 dt a (integrators.rs:55-68); kinetic energy per atom
// for the thermostat (compute.rs:133-144).
__global__ void vv_second_kernel(int n, const int* __restrict__ sysid, const SysDev* __restrict__ sys,
                                 const double* __restrict__ force, double4_32a* __restrict__ vel,
                                 double4_32a* __restrict__ acc, double* __restrict__ ke, int thermostat,
                                 int exact_division) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const SysDev& s = sys[sysid[i]];
    double hdt = __dmul_rn(0.5, s.dt);
    double4_32a v = vel[i];
    double m = v.w;
    double4_32a a;
    if (exact_division) {  // the reference's force / mass
        a = make_double4_32a(force[3 * i] / m, force[3 * i + 1] / m, force[3 * i + 2] / m, 0.0);
    } else {  // mixed path: one reciprocal per atom
        double im = 1.0 / m;
        a = make_double4_32a(force[3 * i] * im, force[3 * i + 1] * im, force[3 * i + 2] * im, 0.0);
    }
    v.x = __dadd_rn(v.x, __dmul_rn(hdt, a.x));
    v.y = __dadd_rn(v.y, __dmul_rn(hdt, a.y));
    v.z = __dadd_rn(v.z, __dmul_rn(hdt, a.z));
    acc[i] = a;
    vel[i] = v;
    if (thermostat) ke[i] = 0.5 * m * (v.x * v.x + v.y * v.y + v.z * v.z);
}

// Per-system temperature T = 2 K / (dof kB) and Berendsen factor
// sqrt(1 + (T0 / T - 1) / tau), fixed-order tree sum.
__global__ void __launch_bounds__(256) thermostat_reduce_kernel(const SysDev* __restrict__ sys,
                                                                const double* __restrict__ ke,
                                                                double* __restrict__ lambda) {
    __shared__ double sh[256];
    const SysDev& s = sys[blockIdx.x];
    double acc = 0.0;
    for (int i = s.begin + threadIdx.x; i < s.end; i += blockDim.x) acc += ke[i];
    sh[threadIdx.x] = acc;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        double f = 1.0;
        if (s.thermo_tau > 0.0) {
            double T = 2.0 * sh[0] / (s.dof * K_BOLTZMANN);
            f = sqrt(1.0 + (s.thermo_T / T - 1.0) / s.thermo_tau);
        }
        lambda[blockIdx.x] = f;
    }
}

__global__ void thermostat_scale_kernel(int n, const int* __restrict__ sysid, const double* __restrict__ lambda,
                                        double4_32a* __restrict__ vel) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double f = lambda[sysid[i]];
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

void launch_vv_first(const Batch& b, cudaStream_t st) {
    if (b.n)
        vv_first_kernel<<<(b.n + 255) / 256, 256, 0, st>>>(b.n, b.sysid, b.sys, b.posq, b.vel, b.acc,
                                                         b.pos_build, b.force, b.status, b.sys_rebuild);
}
void launch_vv_second(const Batch& b, bool thermostat, cudaStream_t st) {
    if (b.n)
        vv_second_kernel<<<(b.n + 255) / 256, 256, 0, st>>>(b.n, b.sysid, b.sys, b.force, b.vel, b.acc, b.ke,
                                                          thermostat ? 1 : 0, b.precision == 0 ? 1 : 0);
}
void launch_thermostat(const Batch& b, cudaStream_t st) {
    if (b.n == 0) return;
    thermostat_reduce_kernel<<<b.nsys, 256, 0, st>>>(b.sys, b.ke, b.lambda);
    thermostat_scale_kernel<<<(b.n + 255) / 256, 256, 0, st>>>(b.n, b.sysid, b.lambda, b.vel);
}
void launch_request_rebuild(const Batch& b, cudaStream_t st) {
    request_rebuild_kernel<<<1, 256, 0, st>>>(b.nsys, b.status, b.sys_rebuild);
}

}  // namespace lg
