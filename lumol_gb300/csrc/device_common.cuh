// device_common.cuh -- data layout shared by the host engine and the kernels,
// and the device restatement of the reference's per-pair arithmetic.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace lg {

constexpr double PI = 3.14159265358979323846;
constexpr double FRAC_2_SQRT_PI = 1.12837916709551257390;
// lumol-core/src/consts.rs:9,15
constexpr double K_BOLTZMANN = 8.31446284161522e-7;
constexpr double FOUR_PI_EPSILON_0 = 7.197589831304046;

// Integrators, thermostats and controls of a system's MD (the values of the
// C ABI's LG_INTEGRATOR_*, LG_THERMOSTAT_* and LG_CONTROL_*).
constexpr int MD_VELOCITY_VERLET = 0, MD_VERLET = 1, MD_LEAP_FROG = 2;
constexpr int TH_NONE = 0, TH_BERENDSEN = 1, TH_RESCALE = 2, TH_CSVR = 3;
constexpr uint32_t CTL_REMOVE_TRANSLATION = 1u, CTL_REWRAP = 2u, CTL_REMOVE_ROTATION = 4u;

// Pair potential table entry: one PairInteraction (energy/pairs.rs:57-95).
struct PairDev {
    int32_t type;         // LG_PAIR_*
    int32_t shifted;
    int32_t restriction;  // LG_RESTRICT_*
    int32_t tail;
    double p0, p1, p2;    // LJ: sigma, epsilon; Buckingham: a, c, rho; Harmonic: k, x0
    double cutoff;
    double shift;         // potential.energy(cutoff) when shifted (pairs.rs:86-95)
    double scale14;
    float cutoff2_f;      // mixed path: cutoff^2 in FP32
    float pad_f;
    double c12, c6;       // LJ: 4 eps sigma^12, 4 eps sigma^6 (plain path, interior pairs)
    double p3, p4;        // BMH: sigma, rho; Mie: m
    double aux;           // Mie: energy prefactor
    // a TableComputation (type PAIR_TABLE): (energy, force) at r = i delta, i < tsize
    const double2* table;
    int32_t tsize, tpad;
    double tdelta;
};

// Device type of a pair tabulated with TableComputation (any potential kind).
constexpr int PAIR_TABLE = 9;

// FP32 pair table entry of the mixed path.
//   LJ: a = 4 eps sigma^12, b = 4 eps sigma^6;  Buckingham: a = A, b = C, c = 1 / rho;
//   Harmonic: a = k, b = x0.  shift: energy shift of a shifted interaction.
struct alignas(16) PairDevF {
    int32_t type, restriction, pad0, pad1;
    float a, b, c, rc2, shift, scale14, d, e;  // d, e: BMH d and sigma; Mie m
    const float2* table;  // PAIR_TABLE: (energy, force) at r = i delta, a = 1 / delta, c = tsize - 1
};

// FP32 k-vector of the mixed Ewald field kernel.
struct KVecF {
    int32_t ikx, iky, ikz, sys;
    float fx, fy, fz, energy;
};

// Per-system descriptor (one Lumol System).
struct SysDev {
    double L[3];          // orthorhombic cell lengths (UnitCell::a/b/c)
    double invL[3];       // 1 / L (fast path of the exact minimum image)
    double rlist;         // neighbour-list radius = max cutoff + skin
    double half_skin2;    // (skin / 2)^2: rebuild threshold on displacement
    int32_t begin, end;   // atom range [begin, end) in the batch arrays
    int32_t ptab, nk;     // offset of the pair table and number of kinds
    int32_t coul;         // LG_COULOMB_*
    int32_t coul_restr;   // LG_RESTRICT_*
    double coul_rc;       // Coulomb cutoff
    double alpha;         // Ewald alpha, or Wolf alpha = PI / cutoff
    double wolf_ec, wolf_fc;  // Wolf energy / force constants (wolf.rs:68-84)
    double coul_scale14;
    int32_t kbegin, kend; // Ewald k-vectors [kbegin, kend) in the batch k arrays
    int32_t kmax;
    int32_t ncell[3];     // neighbour cells per dimension
    int32_t cell_begin;   // offset of this system's cells in the batch cell arrays
    int32_t needs_path;   // 1 when a restriction needs bond paths (Exclude*/Scale14)
    double k1[3];         // 2 PI * inv(cell)[d][d]: k-vector of index 1 per axis (cells.rs:224-226)
    // molecular dynamics
    double dt;
    double hdt;                   // 0.5 dt (exact)
    double fxscale[3];            // 2^32 / L: fixed-point units per length (mixed path)
    double thermo_T, thermo_tau;  // thermostat target and time scale (timesteps)
    double dof;                   // 3 N (DegreesOfFreedom::Particles)
    int32_t tile_begin, tile_end; // this system's tiles of the per-atom MD kernels
    float Lf[3], invLf[3];        // FP32 copies for the list build and the mixed path
    float Lq[3];                  // L / 2^32: the length of one fixed-point unit
    float rlist2_f;               // (rlist + margin)^2 in FP32
    float rebuild2_f;             // 0.99 (skin / 2)^2: FP32 displacement threshold (errs towards rebuilding)
    float coul_rc2_f;
    // integrators, thermostats and controls beyond Velocity-Verlet + Berendsen
    // (after the fields the hot kernels read, which keep their offsets)
    double dt2;                   // dt * dt (Verlet, LeapFrog)
    double hdt2;                  // 0.5 dt^2 (mixed LeapFrog)
    double inv_2dt;               // 1 / (2 dt) (mixed Verlet)
    double thermo_tol;            // RescaleThermostat tolerance
    double total_mass;            // sum of the masses in atom order (RemoveTranslation)
    unsigned long long seed;      // CSVR noise
    int32_t integrator;           // MD_*
    int32_t thermostat;           // TH_*
    uint32_t controls;            // CTL_* bits
    int32_t mol_first, mol_end;   // the system's molecules in the batch molecule table (Rewrap)
    double baro_eta;              // BerendsenBarostat: the factor this step scales the positions by
    int32_t barostat;             // 1: BerendsenBarostat (Velocity-Verlet based)
    int32_t baro_pad;
    // CellShape::Triclinic (cells.rs:72-94): the general branches of the
    // geometry.  For an orthorhombic system H and Hi hold the diagonal cell
    // and its inverse, and L / invL / Lf / Lq stay the only fields read.
    int32_t tric;                 // 1: triclinic cell
    int32_t kgen;                 // 1: k-vectors off the axes (an orthorhombic cell with off-diagonal terms)
    double H[9];                  // UnitCell::matrix, row-major; columns are the cell vectors
    double Hi[9];                 // its Matrix3::inverse (matrix.rs:212-227)
    double kax[9];                // k_vector(e_a) = 2 PI Hi e_a (cells.rs:224-226), row a = axis a
    float Hf[9];                  // H in FP32 (mixed path and list builds)
    float tric_padf[3];
    double baro_m[9];             // AnisoBerendsenBarostat: the matrix this step scales the positions by
};

// eta * x (Matrix3 * Vector3D, matrix.rs:389-398) of the anisotropic barostat, in place.
__device__ __forceinline__ void baro_scale(const double* m, double& x, double& y, double& z) {
    double v[3] = {x, y, z}, o[3];
#pragma unroll
    for (int a = 0; a < 3; a++)
        o[a] = __dadd_rn(__dadd_rn(__dmul_rn(m[3 * a], v[0]), __dmul_rn(m[3 * a + 1], v[1])),
                         __dmul_rn(m[3 * a + 2], v[2]));
    x = o[0];
    y = o[1];
    z = o[2];
}

// Matrix3 * Vector3D (matrix.rs:389-398): each row a left-to-right sum of
// unfused products.
__device__ __forceinline__ void mat_vec_exact(const double* m, const double v[3], double out[3]) {
#pragma unroll
    for (int a = 0; a < 3; a++)
        out[a] = __dadd_rn(__dadd_rn(__dmul_rn(m[3 * a], v[0]), __dmul_rn(m[3 * a + 1], v[1])),
                           __dmul_rn(m[3 * a + 2], v[2]));
}

// vector_image of a triclinic cell (cells.rs:292-298): fractional = inv * d,
// each component minus its round (half away from zero), back to Cartesian.
__device__ __forceinline__ void tric_image(const SysDev& s, double d[3]) {
    double f[3];
    mat_vec_exact(s.Hi, d, f);
#pragma unroll
    for (int a = 0; a < 3; a++) f[a] = __dsub_rn(f[a], round(f[a]));
    mat_vec_exact(s.H, f, d);
}

// wrap_vector of a triclinic cell (cells.rs:271-279): the same with floor.
__device__ __forceinline__ void tric_wrap(const SysDev& s, double d[3]) {
    double f[3];
    mat_vec_exact(s.Hi, d, f);
#pragma unroll
    for (int a = 0; a < 3; a++) f[a] = __dsub_rn(f[a], floor(f[a]));
    mat_vec_exact(s.H, f, d);
}

// k_vector(e_axis) * r (cells.rs:224-226, ewald.rs:646-649): the phase of
// e^{i k r} for index 1 along an axis (orthorhombic: the one coordinate).
__device__ __forceinline__ double axis_phase(const SysDev& s, int axis, double x, double y, double z) {
    if (!s.tric && !s.kgen) return s.k1[axis] * (axis == 0 ? x : (axis == 1 ? y : z));
    const double* k = s.kax + 3 * axis;
    return __dadd_rn(__dadd_rn(__dmul_rn(k[0], x), __dmul_rn(k[1], y)), __dmul_rn(k[2], z));
}

// Squared minimum-image length of a displacement (list-rebuild tests).
__device__ __forceinline__ double image_norm2(const SysDev& s, double dx, double dy, double dz) {
    if (s.tric) {
        double d[3] = {dx, dy, dz};
        tric_image(s, d);
        return d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
    }
    dx -= rint(dx * s.invL[0]) * s.L[0];
    dy -= rint(dy * s.invL[1]) * s.L[1];
    dz -= rint(dz * s.invL[2]) * s.L[2];
    return dx * dx + dy * dy + dz * dz;
}

// Fractional coordinates of a position (fused: for the list builds and the
// fixed-point copies, which need consistency, not the reference's roundings).
__device__ __forceinline__ void tric_fractional(const SysDev& s, double x, double y, double z, double f[3]) {
#pragma unroll
    for (int a = 0; a < 3; a++) f[a] = fma(s.Hi[3 * a + 2], z, fma(s.Hi[3 * a + 1], y, s.Hi[3 * a] * x));
}

// Cartesian offset of a fractional offset in FP32 (fractions of the cell
// vectors), each row a fixed sequence of roundings.
__device__ __forceinline__ void tric_cartesian_f(const SysDev& s, float fx, float fy, float fz, float& dx,
                                                 float& dy, float& dz) {
    dx = __fmaf_rn(s.Hf[2], fz, __fmaf_rn(s.Hf[1], fy, __fmul_rn(s.Hf[0], fx)));
    dy = __fmaf_rn(s.Hf[5], fz, __fmaf_rn(s.Hf[4], fy, __fmul_rn(s.Hf[3], fx)));
    dz = __fmaf_rn(s.Hf[8], fz, __fmaf_rn(s.Hf[7], fy, __fmul_rn(s.Hf[6], fx)));
}

// Sum over one system's chunks of a per-chunk value a[stride * (begin + q)]
// (chunk q: atoms begin + q * gpw ..., each chunk summed by a warp butterfly):
// a lane-strided sum over the chunks, then a butterfly over the 32 lanes, so
// every lane gets the same value.  The per-step integrator and the persistent
// kernel both sum kinetic energies this way (L1 bypassed: the chunks may come
// from other SMs of the same launch).
__device__ __forceinline__ double chunk_sum(const SysDev& s, const double* a, int stride, int gpw, int lane) {
    int nq = (s.end - s.begin + gpw - 1) / gpw;
    double k = 0.0;
    for (int q = lane; q < nq; q += 32) k += __ldcg(&a[(size_t)stride * (s.begin + q)]);
    for (int o = 16; o > 0; o >>= 1) k += __shfl_xor_sync(0xffffffffu, k, o);
    return k;
}
__device__ __forceinline__ double chunk_ke_sum(const SysDev& s, const double* ke, int gpw, int lane) {
    return chunk_sum(s, ke, 1, gpw, lane);
}

// SplitMix64 stream of the CSVR noise of one thermostat application: the
// state starts from (seed, count), so every block of a system draws the same
// numbers without shared state.
struct NoiseStream {
    unsigned long long st;
    __device__ __host__ NoiseStream(unsigned long long seed, unsigned long long count)
        : st(seed ^ (count * 0xD1B54A32D192ED03ull)) {}
    __device__ unsigned long long next() {
        unsigned long long z = (st += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    }
    // uniform in (0, 1): the top 53 bits plus one half
    __device__ double uniform() { return ((double)(next() >> 11) + 0.5) * 0x1.0p-53; }
    // standard normal, Box-Muller (cosine branch)
    __device__ double normal() {
        double u1 = uniform(), u2 = uniform();
        return sqrt(-2.0 * log(u1)) * cos(2.0 * PI * u2);
    }
    // Gamma(a, 1) for a >= 1: Marsaglia and Tsang, ACM TOMS 26 (2000) 363-372.
    // The rejection loop accepts with probability above 0.95 per round; after
    // 64 rounds (never reached in practice) it returns the mode d.
    __device__ double gamma(double a) {
        double d = a - 1.0 / 3.0;
        double c = 1.0 / sqrt(9.0 * d);
        for (int it = 0; it < 64; it++) {
            double x = normal();
            double v = 1.0 + c * x;
            if (v <= 0.0) continue;
            v = v * v * v;
            double u = uniform();
            double x2 = x * x;
            if (u < 1.0 - 0.0331 * x2 * x2) return d * v;
            if (log(u) < 0.5 * x2 + d * (1.0 - v + log(v))) return d * v;
        }
        return d;
    }
};

// CSVRThermostat::apply's factor (thermostats.rs:195-210) with the noise of
// CSVRThermostat::sum_noises (thermostats.rs:166-192) for dof - 1 degrees:
// one gaussian rr, and 2 Gamma(n / 2) (n even) or 2 Gamma((n - 1) / 2) + rr^2
// (n odd, the same rr as the reference).
// (Not inlined: a call keeps the sampler's code and stack out of the MD kernels.)
static __device__ __noinline__ double csvr_factor(const SysDev& s, double kinetic, unsigned long long count) {
    double target = K_BOLTZMANN * s.thermo_T / 2.0;  // target_kinetic_per_dof
    double kinetic_factor = target / kinetic;
    double exp_1 = exp(-1.0 / s.thermo_tau);
    double exp_2 = (1.0 - exp_1) * kinetic_factor;
    long long n = (long long)s.dof - 1;
    NoiseStream r(s.seed, count);
    double gauss = 0.0, wiener = 0.0;
    if (n == 1) {
        gauss = r.normal();
        wiener = gauss * gauss;
    } else if (n > 1) {
        gauss = r.normal();
        if (n % 2 == 0) wiener = 2.0 * r.gamma((double)(n / 2));
        else wiener = 2.0 * r.gamma((double)((n - 1) / 2)) + gauss * gauss;
    }
    double scale = exp_1 + exp_2 * (gauss * gauss + wiener) + 2.0 * gauss * sqrt(exp_1 * exp_2);
    return sqrt(scale);
}

// Velocity factor of a system's thermostat at kinetic energy k, with
// T = 2 K / (dof kB) (sys/compute.rs:133-172):
//   Berendsen  sqrt(1 + (T0 / T - 1) / tau)         (thermostats.rs:112-121)
//   Rescale    sqrt(T0 / T) when |T - T0| > tol     (thermostats.rs:66-73, velocities.rs:16-22)
//   CSVR       csvr_factor                          (count: the system's thermostat applications)
__device__ __forceinline__ double berendsen_factor(const SysDev& s, double k) {
    double T = 2.0 * k / (s.dof * K_BOLTZMANN);
    return sqrt(1.0 + (s.thermo_T / T - 1.0) / s.thermo_tau);
}
__device__ __forceinline__ double thermostat_factor(const SysDev& s, double k, unsigned long long count) {
    switch (s.thermostat) {
        case TH_BERENDSEN:
            return berendsen_factor(s, k);
        case TH_RESCALE: {
            double T = 2.0 * k / (s.dof * K_BOLTZMANN);
            return fabs(T - s.thermo_T) > s.thermo_tol ? sqrt(s.thermo_T / T) : 1.0;
        }
        case TH_CSVR:
            return csvr_factor(s, k, count);
        default:
            return 1.0;
    }
}

// Sum of a chunk of gpw lanes (gpw a power of two dividing 32), as a butterfly
// inside the chunk: the same tree as a butterfly over a whole warp whose
// lanes hold one atom's value every 32 / gpw lanes and zeros elsewhere.
__device__ __forceinline__ double chunk_butterfly(double v, int gpw) {
    for (int o = gpw / 2; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Fixed-point copy of a wrapped position for the mixed path: per axis
// u = floor(frac(x / L) * 2^32) (UnitCell::wrap_vector, cells.rs:263-282, as a
// fraction of the cell), and the charge's FP32 bits.
// floor(x 2^32 / L) taken modulo 2^32 is that fraction (two's complement
// wrap-around does the frac).  One FP64 instruction per axis: the fused
// x * scale + 1.5 * 2^52 rounded toward -infinity is floor(x * scale) +
// 1.5 * 2^52 exactly (the unit in the last place there is 1), and the low 32
// bits of its encoding are floor(x * scale) modulo 2^32; this holds for
// |x * scale| < 2^51, i.e. positions within 2^19 cell lengths of the origin.
// (floor of the exact product: no rounding of x * scale first.)
__device__ __forceinline__ uint32_t fixed_coordinate(double x, double scale) {
    return (uint32_t)__double2loint(__fma_rd(x, scale, 6755399441055744.0));
}
// The charge's FP32 copy is never zero for a non-zero charge (a charge below
// the FP32 range keeps the smallest normal value), so "q != 0" tests agree
// with the FP64 charges.
__device__ __forceinline__ float charge_f32(double q) {
    float f = (float)q;
    return (f == 0.0f && q != 0.0) ? (q < 0.0 ? -1.17549435e-38f : 1.17549435e-38f) : f;
}
// (triclinic: u = floor(frac(f) * 2^32) of the fractional coordinates f, so
// the signed 32-bit difference of two atoms is the fractional difference
// minus its nearest integer, as vector_image takes it)
__device__ __forceinline__ uint3 fixed_coordinates(const SysDev& s, double4_32a p) {
    if (s.tric) {
        double f[3];
        tric_fractional(s, p.x, p.y, p.z, f);
        return make_uint3(fixed_coordinate(f[0], 4294967296.0), fixed_coordinate(f[1], 4294967296.0),
                          fixed_coordinate(f[2], 4294967296.0));
    }
    return make_uint3(fixed_coordinate(p.x, s.fxscale[0]), fixed_coordinate(p.y, s.fxscale[1]),
                      fixed_coordinate(p.z, s.fxscale[2]));
}
__device__ __forceinline__ uint4 fixed_position(const SysDev& s, double4_32a p) {
    uint3 u = fixed_coordinates(s, p);
    return make_uint4(u.x, u.y, u.z, __float_as_uint(charge_f32(p.w)));
}
// Orthorhombic only (the persistent kernel, whose batches have no triclinic cell).
__device__ __forceinline__ uint4 fixed_position_ortho(const SysDev& s, double4_32a p) {
    return make_uint4(fixed_coordinate(p.x, s.fxscale[0]), fixed_coordinate(p.y, s.fxscale[1]),
                      fixed_coordinate(p.z, s.fxscale[2]), __float_as_uint(charge_f32(p.w)));
}
// The coordinates alone (w = 0), for the integrators' updates: the charge
// word of an atom's record never changes between list builds, so they store
// x, y, z only (store_fixed_xyz) and skip its FP64 conversion.
__device__ __forceinline__ uint4 fixed_xyz(const SysDev& s, double4_32a p) {
    uint3 u = fixed_coordinates(s, p);
    return make_uint4(u.x, u.y, u.z, 0u);
}
__device__ __forceinline__ uint4 fixed_xyz_ortho(const SysDev& s, double4_32a p) {
    return make_uint4(fixed_coordinate(p.x, s.fxscale[0]), fixed_coordinate(p.y, s.fxscale[1]),
                      fixed_coordinate(p.z, s.fxscale[2]), 0u);
}
__device__ __forceinline__ void store_fixed_xyz(uint4* dst, uint4 u) {
    uint32_t* d = reinterpret_cast<uint32_t*>(dst);
    *reinterpret_cast<uint2*>(d) = make_uint2(u.x, u.y);
    d[2] = u.z;
}

// Squared minimum-image distance of two fixed-point positions in FP32, every
// operation rounded on its own, so the list builds of the per-step and the
// persistent kernels decide every candidate alike.
__device__ __forceinline__ float fixed_dist2(uint4 a, uint4 b, const float* Lq) {
    float dx = __fmul_rn((float)(int32_t)(a.x - b.x), Lq[0]);
    float dy = __fmul_rn((float)(int32_t)(a.y - b.y), Lq[1]);
    float dz = __fmul_rn((float)(int32_t)(a.z - b.z), Lq[2]);
    return __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
}
// Cartesian minimum-image offset of two fixed-point positions in FP32
// (vector_image's image: each fractional difference wrapped into [-1/2, 1/2)).
__device__ __forceinline__ void fixed_delta(const SysDev& s, uint4 a, uint4 b, float& dx, float& dy, float& dz) {
    if (s.tric) {
        const float q = 2.3283064365386963e-10f;  // 2^-32
        tric_cartesian_f(s, __fmul_rn((float)(int32_t)(a.x - b.x), q), __fmul_rn((float)(int32_t)(a.y - b.y), q),
                         __fmul_rn((float)(int32_t)(a.z - b.z), q), dx, dy, dz);
    } else {
        dx = __fmul_rn((float)(int32_t)(a.x - b.x), s.Lq[0]);
        dy = __fmul_rn((float)(int32_t)(a.y - b.y), s.Lq[1]);
        dz = __fmul_rn((float)(int32_t)(a.z - b.z), s.Lq[2]);
    }
}
// fixed_dist2 for any cell shape (the per-step kernels)
__device__ __forceinline__ float fixed_dist2_s(const SysDev& s, uint4 a, uint4 b) {
    if (!s.tric) return fixed_dist2(a, b, s.Lq);
    float dx, dy, dz;
    fixed_delta(s, a, b, dx, dy, dz);
    return __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
}

// Cell of a fixed-point position: u / 2^32 is the wrapped fraction of the
// cell length, so floor(fraction * ncell) is (u * ncell) >> 32.
__device__ __forceinline__ int fixed_cell(const SysDev& s, uint4 u) {
    // the high 32 bits of the 64-bit products u * ncell (__umulhi: the
    // spelled-out (u64)u * n >> 32 lost its z term in one list-build kernel)
    int cx = (int)__umulhi(u.x, (unsigned)s.ncell[0]);
    int cy = (int)__umulhi(u.y, (unsigned)s.ncell[1]);
    int cz = (int)__umulhi(u.z, (unsigned)s.ncell[2]);
    return s.cell_begin + (cz * s.ncell[1] + cy) * s.ncell[0] + cx;
}

// Candidate cells of a list build.  Cells are at least half the list radius
// wide, so every atom within the list radius of an atom in cell (cx, cy, cz)
// lies within two cells of it per dimension (all cells of a dimension with
// fewer than five, each once).  The candidates come as runs of cells that are
// contiguous in memory (one x-row segment each; the periodic wrap splits a
// segment in two): run k = (iz * ny + iy) * 2 + part, at most 5 * 5 * 2 runs.
constexpr int NL_RUNS = 64;

__device__ __forceinline__ int stencil_span(int nc) { return nc >= 5 ? 5 : nc; }
__device__ __forceinline__ int stencil_at(int c, int nc, int k) { return nc >= 5 ? (c + k - 2 + nc) % nc : k; }

// Cells [lo, hi] (system-local indices, hi < lo: empty) of run k.
__device__ __forceinline__ void stencil_run(const SysDev& s, int cx, int cy, int cz, int k, int& lo, int& hi) {
    int ny = stencil_span(s.ncell[1]);
    int iz = k / (2 * ny), iy = (k / 2) % ny, part = k & 1;
    int z = stencil_at(cz, s.ncell[2], iz), y = stencil_at(cy, s.ncell[1], iy);
    int nx = s.ncell[0];
    int xlo, xhi;
    if (nx < 5) {
        xlo = part == 0 ? 0 : 1;
        xhi = part == 0 ? nx - 1 : 0;
    } else if (cx - 2 < 0) {  // wraps below: [cx - 2 + nx, nx - 1], then [0, cx + 2]
        xlo = part == 0 ? cx - 2 + nx : 0;
        xhi = part == 0 ? nx - 1 : cx + 2;
    } else if (cx + 2 >= nx) {  // wraps above: [cx - 2, nx - 1], then [0, cx + 2 - nx]
        xlo = part == 0 ? cx - 2 : 0;
        xhi = part == 0 ? nx - 1 : cx + 2 - nx;
    } else {
        xlo = part == 0 ? cx - 2 : 1;
        xhi = part == 0 ? cx + 2 : 0;
    }
    int row = (z * s.ncell[1] + y) * nx;
    lo = row + xlo;
    hi = row + xhi;
}

__device__ __forceinline__ int stencil_runs(const SysDev& s) {
    return stencil_span(s.ncell[2]) * stencil_span(s.ncell[1]) * 2;
}

// One warp's candidate table for an atom in system cell `local` (system-local
// index) of system si: s_lo[k] = first slot of run k, s_pre[k] = candidates
// before run k, s_pre[nruns] = total.  Returns (nruns, total).
__device__ __forceinline__ int2 stencil_table(const SysDev& s, int si, int local, const int* __restrict__ cell_start,
                                              int lane, int* s_lo, int* s_pre) {
    int cx = local % s.ncell[0];
    int cy = (local / s.ncell[0]) % s.ncell[1];
    int cz = local / (s.ncell[0] * s.ncell[1]);
    int nruns = stencil_runs(s);
    int cnt[2], lo[2];
#pragma unroll
    for (int h = 0; h < 2; h++) {
        int k = lane + 32 * h;
        cnt[h] = 0;
        lo[h] = 0;
        if (k < nruns) {
            int c0, c1;
            stencil_run(s, cx, cy, cz, k, c0, c1);
            if (c1 >= c0) {
                lo[h] = cell_start[s.cell_begin + c0 + si];
                cnt[h] = cell_start[s.cell_begin + c1 + 1 + si] - lo[h];
            }
        }
    }
    int base = 0, total = 0;
#pragma unroll
    for (int h = 0; h < 2; h++) {
        int incl = cnt[h];
        for (int o = 1; o < 32; o <<= 1) {
            int v = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += v;
        }
        int sum = __shfl_sync(0xffffffffu, incl, 31);
        int k = lane + 32 * h;
        if (k < nruns) {
            s_lo[k] = lo[h];
            s_pre[k] = base + incl - cnt[h];
        }
        base += sum;
        total = base;
    }
    if (lane == 0) s_pre[nruns] = total;
    return make_int2(nruns, total);
}

// Slot of candidate q: the run holding it is the last k with s_pre[k] <= q.
__device__ __forceinline__ int stencil_slot(const int* s_lo, const int* s_pre, int nruns, int q) {
    int a = 0, b = nruns - 1;
    while (a < b) {
        int mid = (a + b + 1) >> 1;
        if (s_pre[mid] <= q) a = mid;
        else b = mid - 1;
    }
    return s_lo[a] + (q - s_pre[a]);
}

// One Ewald k-vector with its factors (ewald.rs:102-116).
struct KVecDev {
    int32_t ikx, iky, ikz, sys;
    double energy;      // 4 pi / V exp(-k^2 / (4 alpha^2)) / k^2
    double field[3];    // 2 energy k
    double virial[6];   // energy (1 - 2 (1/k^2 + 1/(4 alpha^2)) k k^T), symmetric xx xy xz yy yz zz
};

// Metropolis chain of one system (batched Monte Carlo).
struct McState {
    double beta;          // 1 / (kB T)
    double delta;         // Translate: delta / sqrt(3), the half width per axis
    double energy;        // EnergyCache energy, updated by the accepted moves
    uint64_t rng;         // SplitMix64 state
    long long moves_left;
    long long accepted, attempted;
    int32_t enabled;
    int32_t need_rebuild;
    // molecular chains (lg_mc_setup_ex): Translate and Rotate of whole molecules
    double theta;          // Rotate: largest angle
    double cum_translate;  // cumulative frequency of Translate (MonteCarlo::normalize_frequencies); 1 without Rotate
    int32_t molecular;     // 1: moves pick molecules (any size) and may rotate them
    int32_t mol_pad;
};

// Status word bits (device -> host).
enum : uint32_t {
    ST_REBUILD = 1u,        // neighbour list must be rebuilt
    ST_OVERFLOW = 2u,       // neighbour list capacity exceeded
    ST_NONFINITE = 4u,      // non-finite energy
    ST_SPECIAL_OVF = 8u,    // bond-path table overflow
    ST_CELL_OVF = 16u,      // cell counts inconsistent with the atoms binned (a cell build was
                            // interrupted): the scatter skipped the write; recount and rebuild
};

// Per-system status bits (Batch::sys_status), read by the host after a run.
enum : uint32_t {
    SYS_NONFINITE = 1u,  // a non-finite velocity, acceleration or energy appeared in the system
};

// A non-finite value in a system's state: the system is flagged (and the
// batch's status word), the others are not affected.
// (the test reads the exponent bits with integer instructions: on GB300 an
// FP64 comparison would take the FP64 pipe, which the integrators saturate)
__device__ __forceinline__ bool nonfinite_bits(double x) {
    return (__double2hiint(x) & 0x7ff00000) == 0x7ff00000;
}
__device__ __forceinline__ void flag_nonfinite(double a, double b, double c, int s, uint32_t* sys_status,
                                               uint32_t* status) {
    if ((nonfinite_bits(a) | nonfinite_bits(b) | nonfinite_bits(c)) && sys_status) {
        atomicOr(sys_status + s, SYS_NONFINITE);
        atomicOr(status, ST_NONFINITE);
    }
}

// Number of energy slots per system in the reduction output:
// [pairs, coulomb real (Ewald real or Wolf), bonds, angles, kspace] then virial 9.
enum { E_PAIRS = 0, E_COUL = 1, E_BONDS = 2, E_ANGLES = 3, E_KSPACE = 4, E_DIHEDRALS = 5, N_ESLOT = 6 };
enum { RED_STRIDE = N_ESLOT + 9 };

// ---------------------------------------------------------------------------
// Exact minimum image (cells.rs:284-301, orthorhombic branch):
//   d -= round(d / L) * L
// with a true division, round half away from zero, and no contraction.  The
// fast path multiplies by 1/L; the result of round() can only differ from the
// reference when d/L is within a few ulps of a half-integer, in which case the
// true division is taken.  The multiply and subtract are rounded separately.
// ---------------------------------------------------------------------------
__device__ __forceinline__ double exact_image(double d, double L, double invL) {
    double t = __dmul_rn(d, invL);
    double rt = round(t);
    if (fabs(__dsub_rn(t, rt)) > 0.4999999999 || fabs(t) > 1.0e5) rt = round(__ddiv_rn(d, L));
    return __dsub_rn(d, __dmul_rn(rt, L));
}

// Vector3D::norm2 then f64::sqrt (types/vectors.rs:102-117), unfused.
__device__ __forceinline__ double exact_norm(double x, double y, double z) {
    double r2 = __dadd_rn(__dadd_rn(__dmul_rn(x, x), __dmul_rn(y, y)), __dmul_rn(z, z));
    return __dsqrt_rn(r2);
}

// Configuration::nearest_image(i, j) = image(r_i - r_j) (configuration.rs:399-403)
__device__ __forceinline__ void exact_nearest_image(const SysDev& s, double xi, double yi, double zi,
                                                    double xj, double yj, double zj, double& dx,
                                                    double& dy, double& dz) {
    if (s.tric) {
        double d[3] = {__dsub_rn(xi, xj), __dsub_rn(yi, yj), __dsub_rn(zi, zj)};
        tric_image(s, d);
        dx = d[0];
        dy = d[1];
        dz = d[2];
        return;
    }
    dx = exact_image(__dsub_rn(xi, xj), s.L[0], s.invL[0]);
    dy = exact_image(__dsub_rn(yi, yj), s.L[1], s.invL[1]);
    dz = exact_image(__dsub_rn(zi, zj), s.L[2], s.invL[2]);
}

// PairRestriction::information (restrictions.rs:85-115).  path: 0 none
// (different molecules), 2 one bond, 3 two bonds, 4 three bonds, 5 far.
__device__ __forceinline__ bool restriction_excluded(int restriction, int path) {
    bool same = path != 0;
    switch (restriction) {
        case 1: return !same;                               // IntraMolecular
        case 2: return same;                                // InterMolecular
        case 3: return path == 2;                           // Exclude12
        case 4: case 6: return path == 2 || path == 3;      // Exclude13, Scale14
        case 5: return path == 2 || path == 3 || path == 4; // Exclude14
        default: return false;                              // None
    }
}
__device__ __forceinline__ double restriction_scaling(int restriction, int path, double s14) {
    return (restriction == 6 && path == 4) ? s14 : 1.0;
}

// f64::powi(x, 6) as LLVM expands it: x^2 * (x^2)^2
__device__ __forceinline__ double powi6(double x) {
    double x2 = x * x;
    return x2 * (x2 * x2);
}

// Potential::energy / force of the pair potentials (functions.rs:85-143, 287-299).
// inv_r = 1 / r.
__device__ __forceinline__ void pair_energy_force(const PairDev& p, double r, double inv_r,
                                                  double& e, double& f) {
    switch (p.type) {
        case 2: {  // LennardJones
            double s6 = powi6(p.p0 * inv_r);
            e = 4.0 * p.p1 * (s6 * s6 - s6);
            f = -24.0 * p.p1 * (s6 - 2.0 * (s6 * s6)) * inv_r;
            break;
        }
        case 3: {  // Buckingham
            double ir3 = inv_r * inv_r * inv_r;
            double ex = exp(-r / p.p2);
            e = p.p0 * ex - p.p1 * (ir3 * ir3);
            f = p.p0 / p.p2 * ex - 6.0 * p.p1 * (ir3 * ir3 * inv_r);
            break;
        }
        case 4: {  // Harmonic
            double dx = r - p.p1;
            e = 0.5 * p.p0 * dx * dx;
            f = p.p0 * (p.p1 - r);
            break;
        }
        case 5: {  // BornMayerHuggins (functions.rs:354-366): a, c, d = p0, p1, p2; sigma, rho = p3, p4
            double r2 = r * r;
            double r6 = r2 * r2 * r2;
            double r7 = r6 * r;
            double ex = exp((p.p3 - r) / p.p4);
            e = p.p0 * ex - p.p1 / r6 + p.p2 / (r6 * r2);
            f = p.p0 / p.p4 * ex - 6.0 * p.p1 / r7 + 8.0 * p.p2 / (r7 * r2);
            break;
        }
        case 6: {  // Morse (functions.rs:415-423, the force as written there): a, x0, depth = p0, p1, p2
            double ex = exp((p.p1 - r) * p.p0);
            double rc = 1.0 - ex;
            e = p.p2 * rc * rc;
            f = 2.0 * p.p2 * (1.0 - ex * ex) * p.p0;
            break;
        }
        case 7: {  // Gaussian (functions.rs:475-481): a, b = p0, p1
            e = -p.p0 * exp(-p.p1 * r * r);
            f = 2.0 * p.p1 * r * e;
            break;
        }
        case 8: {  // Mie (functions.rs:553-565): sigma, n, m = p0, p2, p3; prefactor in aux
            double sr = p.p0 / r;
            double rep = pow(sr, p.p2), att = pow(sr, p.p3);
            e = p.aux * (rep - att);
            f = p.aux * (p.p2 * rep - p.p3 * att) / r;
            break;
        }
        case PAIR_TABLE: {  // Computation::compute_energy / compute_force (computations.rs:123-144)
            double binf = floor(__ddiv_rn(r, p.tdelta));
            if (binf < (double)(p.tsize - 1)) {
                int bin = (int)binf;
                double2 t0 = p.table[bin], t1 = p.table[bin + 1];
                double dx = __dsub_rn(r, __dmul_rn((double)bin, p.tdelta));
                e = __dadd_rn(t0.x, __dmul_rn(dx, __ddiv_rn(__dsub_rn(t1.x, t0.x), p.tdelta)));
                f = __dadd_rn(t0.y, __dmul_rn(dx, __ddiv_rn(__dsub_rn(t1.y, t0.y), p.tdelta)));
            } else {
                e = 0.0;
                f = 0.0;
            }
            break;
        }
        default:
            e = 0.0;
            f = 0.0;
    }
    if (p.shifted) e -= p.shift;
}

// Ewald real-space pair term (ewald.rs:383-428): energy and force / r.
__device__ __forceinline__ void ewald_real_pair(double alpha, bool excluded, double qiqj, double r,
                                                double inv_r, double& e, double& f_over_r) {
    double ar = alpha * r;
    double pref = qiqj * (1.0 / FOUR_PI_EPSILON_0);
    double g = alpha * FRAC_2_SQRT_PI * exp(-ar * ar);
    if (excluded) {
        double erfv = erf(ar);
        e = -pref * erfv * inv_r;
        f_over_r = pref * inv_r * inv_r * (g - erfv * inv_r);
    } else {
        double erfcv = erfc(ar);
        e = pref * erfcv * inv_r;
        f_over_r = pref * inv_r * inv_r * (g + erfcv * inv_r);
    }
}

// Wolf pair term (wolf.rs:90-117): energy and force / r.
__device__ __forceinline__ void wolf_pair(const SysDev& s, double qiqj, double r, double inv_r,
                                          double& e, double& f_over_r) {
    double ar = s.alpha * r;
    double erfcv = erfc(ar);
    e = qiqj * (erfcv * inv_r - s.wolf_ec) * (1.0 / FOUR_PI_EPSILON_0);
    double factor = erfcv * inv_r * inv_r + s.alpha * FRAC_2_SQRT_PI * exp(-ar * ar) * inv_r;
    f_over_r = qiqj * (factor - s.wolf_fc) * inv_r * (1.0 / FOUR_PI_EPSILON_0);
}

// Bond path lookup in the per-atom table of same-molecule pairs closer than
// four bonds.  Returns 0 (different molecules), 2, 3, 4 or 5 (far).
__device__ __forceinline__ int bond_path(int i, int j, int mol_i, int mol_j, const int* spec_off,
                                         const int* spec_j, const int8_t* spec_path) {
    if (mol_i != mol_j) return 0;
    for (int k = spec_off[i]; k < spec_off[i + 1]; k++)
        if (spec_j[k] == j) return spec_path[k];
    return 5;
}

// Warp-level sum of a double.
__device__ __forceinline__ double warp_sum(double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ float warp_sum_f(float v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

}  // namespace lg
