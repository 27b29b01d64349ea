// noalloc.cu -- Ewald k-space forces, energy and virial without any device
// allocation.
//
// Some callers of this library cannot call cudaMalloc: code that runs inside
// another framework whose device memory is owned by its own pool allocator,
// and per-step or per-move loops where cudaMalloc / cudaFree would
// synchronise the device (or fail under a memory cap).  For them this entry
// point computes the same k-space terms as lg_compute(LG_TERM_COUL_KSPACE) on
// device pointers the caller passes, and keeps all of its scratch (k-vector
// factors, e^{ik.r} tables, rho(k), per-k energy and virial terms) in one
// file-scope __device__ array of fixed size.
//
// Limits: at most NA_MAX_ATOMS atoms and kmax <= NA_MAX_KMAX.  The array
// (about 2 MB) is held by every GPU that loads the library, until the process
// exits.  Every call shares it: calls whose work overlaps on the GPU (two
// streams, or two threads) race and corrupt each other's results.  Each call
// writes every scratch slot it reads before reading it, so nothing from the
// previous call leaks into the next one.
//
// The first call on a device looks up the device address of the array
// (cudaGetSymbolAddress) with that device current and keeps it for the life
// of the process; make that first call before any stream capture.  The
// address belongs to the device's primary context: after cudaDeviceReset (or
// anything else that destroys and re-creates the primary context) the array
// can move, so the entry point must not be called again in that process.
#include <algorithm>
#include <mutex>
#include <string>

#include "../../include/lumol_gb300.h"
#include "kernels.h"

namespace lg {
namespace {

constexpr int NA_MAX_ATOMS = LG_NOALLOC_MAX_ATOMS;
constexpr int NA_MAX_KMAX = LG_NOALLOC_MAX_KMAX;
// k-vector candidates of Ewald::prepare's three loops (ewald.rs:146-182) at kmax
constexpr int na_candidates(int kmax) {
    return (kmax - 1) * (2 * kmax) * (2 * kmax) + (kmax - 1) * (2 * kmax) + (kmax - 1);
}
constexpr int NA_MAX_KCAND = na_candidates(NA_MAX_KMAX);
constexpr int NA_KFAC = 12;  // active, energy, field xyz, virial xx xy xz yy yz zz, pad
constexpr size_t NA_OFF_KFAC = 0;
constexpr size_t NA_OFF_EIKR = NA_OFF_KFAC + (size_t)NA_MAX_KCAND * NA_KFAC;
constexpr size_t NA_OFF_RHO = NA_OFF_EIKR + (size_t)(NA_MAX_KMAX + 1) * 3 * NA_MAX_ATOMS * 2;
constexpr size_t NA_OFF_KRED = NA_OFF_RHO + (size_t)NA_MAX_KCAND * 2;
constexpr size_t NA_TOTAL = NA_OFF_KRED + (size_t)NA_MAX_KCAND * 7;

static __device__ __align__(256) double g_noalloc_scratch[NA_TOTAL];

std::mutex g_setup_mutex;
double* g_scratch_address[256] = {nullptr};

__device__ __forceinline__ void na_candidate_index(int c, int kmax, int& ikx, int& iky, int& ikz) {
    int a = (kmax - 1) * (2 * kmax) * (2 * kmax);
    int b = (kmax - 1) * (2 * kmax);
    if (c < a) {
        ikx = 1 + c / (4 * kmax * kmax);
        int r = c % (4 * kmax * kmax);
        iky = -kmax + r / (2 * kmax);
        ikz = -kmax + r % (2 * kmax);
    } else if (c < a + b) {
        int r = c - a;
        ikx = 0;
        iky = 1 + r / (2 * kmax);
        ikz = -kmax + r % (2 * kmax);
    } else {
        ikx = 0;
        iky = 0;
        ikz = 1 + (c - a - b);
    }
}

// k-vector factors of compute_ewald_factors_triclinic (ewald.rs:130-144), one
// thread per candidate; candidates outside the spherical cut are inactive.
__global__ void na_kvec_kernel(double* scratch, int kmax, int ncand, double s0, double s1, double s2,
                               double kmax2, double alpha, double four_pi_v) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= ncand) return;
    int ikx, iky, ikz;
    na_candidate_index(c, kmax, ikx, iky, ikz);
    double k[3] = {s0 * (double)ikx, s1 * (double)iky, s2 * (double)ikz};
    double k2 = k[0] * k[0] + k[1] * k[1] + k[2] * k[2];
    double* f = scratch + NA_OFF_KFAC + (size_t)c * NA_KFAC;
    if (k2 > kmax2) {
        for (int q = 0; q < NA_KFAC; q++) f[q] = 0.0;
        return;
    }
    double a4 = 0.25 / (alpha * alpha);
    double energy = four_pi_v * exp(-k2 * a4) / k2;
    f[0] = 1.0;
    f[1] = energy;
    for (int d = 0; d < 3; d++) f[2 + d] = (2.0 * energy) * k[d];
    double vf = -2.0 * (1.0 / k2 + a4);
    const int ia[6] = {0, 0, 0, 1, 1, 2}, ib[6] = {0, 1, 2, 1, 2, 2};
    for (int q = 0; q < 6; q++) f[5 + q] = energy * ((ia[q] == ib[q] ? 1.0 : 0.0) + vf * (k[ia[q]] * k[ib[q]]));
    f[11] = 0.0;
}

__device__ __forceinline__ double2 na_cmul(double2 a, double2 b) {
    return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

// Ewald::eik_dot_r, per-atom part (ewald.rs:633-662)
__global__ void na_eikr_kernel(double* scratch, const double* __restrict__ pos, int n, int kmax, double k0,
                               double k1, double k2) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= 3 * n) return;
    int axis = t / n, i = t - axis * n;
    double kk1 = axis == 0 ? k0 : (axis == 1 ? k1 : k2);
    double sn, cs;
    sincos(kk1 * pos[3 * i + axis], &sn, &cs);
    double2* e = (double2*)(scratch + NA_OFF_EIKR);
    double2 e1 = make_double2(cs, sn), v = e1;
    e[(size_t)(0 * 3 + axis) * NA_MAX_ATOMS + i] = make_double2(1.0, 0.0);
    e[(size_t)(1 * 3 + axis) * NA_MAX_ATOMS + i] = e1;
    for (int q = 2; q <= kmax; q++) {
        v = na_cmul(v, e1);
        e[(size_t)(q * 3 + axis) * NA_MAX_ATOMS + i] = v;
    }
}

__device__ __forceinline__ double2 na_eikr(const double* scratch, int q, int axis, int i) {
    const double2* e = (const double2*)(scratch + NA_OFF_EIKR);
    if (q >= 0) return e[(size_t)(q * 3 + axis) * NA_MAX_ATOMS + i];
    double2 v = e[(size_t)((-q) * 3 + axis) * NA_MAX_ATOMS + i];
    return make_double2(v.x, -v.y);
}

// rho(k) and the per-k energy / virial terms, one block per candidate.
__global__ void __launch_bounds__(256) na_rho_kernel(double* scratch, const double* __restrict__ charges, int n,
                                                     int kmax) {
    __shared__ double sre[256], sim[256];
    int c = blockIdx.x;
    const double* f = scratch + NA_OFF_KFAC + (size_t)c * NA_KFAC;
    double2* rho = (double2*)(scratch + NA_OFF_RHO);
    double* kred = scratch + NA_OFF_KRED + (size_t)c * 7;
    if (f[0] == 0.0) {
        if (threadIdx.x == 0) {
            rho[c] = make_double2(0.0, 0.0);
            for (int q = 0; q < 7; q++) kred[q] = 0.0;
        }
        return;
    }
    int ikx, iky, ikz;
    na_candidate_index(c, kmax, ikx, iky, ikz);
    double re = 0.0, im = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        double2 ph = na_cmul(na_cmul(na_eikr(scratch, ikx, 0, i), na_eikr(scratch, iky, 1, i)),
                             na_eikr(scratch, ikz, 2, i));
        re += charges[i] * ph.x;
        im += charges[i] * ph.y;
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
        rho[c] = r;
        double nrm = r.x * r.x + r.y * r.y;
        kred[0] = f[1] * nrm;
        for (int q = 0; q < 6; q++) kred[1 + q] = nrm * f[5 + q];
    }
}

// force_i += q_i / (4 pi eps0) sum_k Im(e^{ik.r_i} conj(rho_k)) field_k (ewald.rs:690-720)
__global__ void na_field_kernel(const double* scratch, const double* __restrict__ charges, int n, int kmax,
                                int ncand, double* __restrict__ forces) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double2* rho = (const double2*)(scratch + NA_OFF_RHO);
    double fx = 0.0, fy = 0.0, fz = 0.0;
    for (int c = 0; c < ncand; c++) {
        const double* f = scratch + NA_OFF_KFAC + (size_t)c * NA_KFAC;
        if (f[0] == 0.0) continue;
        int ikx, iky, ikz;
        na_candidate_index(c, kmax, ikx, iky, ikz);
        double2 e = na_cmul(na_cmul(na_eikr(scratch, ikx, 0, i), na_eikr(scratch, iky, 1, i)),
                            na_eikr(scratch, ikz, 2, i));
        double2 r = rho[c];
        double imag = e.x * (-r.y) + e.y * r.x;
        fx += imag * f[2];
        fy += imag * f[3];
        fz += imag * f[4];
    }
    double q = charges[i];
    forces[3 * i] += q * fx / FOUR_PI_EPSILON_0;
    forces[3 * i + 1] += q * fy / FOUR_PI_EPSILON_0;
    forces[3 * i + 2] += q * fz / FOUR_PI_EPSILON_0;
}

// energy = sum_k f_k |rho_k|^2 / (4 pi eps0); virial likewise, fixed order.
__global__ void __launch_bounds__(256) na_reduce_kernel(const double* scratch, int ncand, double* energy,
                                                        double* virial) {
    __shared__ double sh[7][256];
    double acc[7] = {0, 0, 0, 0, 0, 0, 0};
    for (int c = threadIdx.x; c < ncand; c += blockDim.x) {
        const double* kr = scratch + NA_OFF_KRED + (size_t)c * 7;
        for (int q = 0; q < 7; q++) acc[q] += kr[q];
    }
    for (int q = 0; q < 7; q++) sh[q][threadIdx.x] = acc[q];
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o)
            for (int q = 0; q < 7; q++) sh[q][threadIdx.x] += sh[q][threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        if (energy) energy[0] = sh[0][0] / FOUR_PI_EPSILON_0;
        if (virial) {
            const int map[9] = {1, 2, 3, 2, 4, 5, 3, 5, 6};
            for (int q = 0; q < 9; q++) virial[q] = sh[map[q]][0] / FOUR_PI_EPSILON_0;
        }
    }
}

// Errors are reported through lg_last_error(NULL), like those of lg_create.
int na_fail(int code, const std::string& msg) {
    set_global_error(msg);
    return code;
}

}  // namespace
}  // namespace lg

using namespace lg;

extern "C" int lg_ewald_kspace_noalloc(const double* d_positions, const double* d_charges, int64_t n,
                                       const double cell[3], double alpha, int32_t kmax, double* d_forces,
                                       double* d_energy, double* d_virial, void* stream) {
    if (n < 0 || n > NA_MAX_ATOMS)
        return na_fail(LG_ERR_ARGUMENT, "lg_ewald_kspace_noalloc: n = " + std::to_string(n) +
                                            " atoms is outside [0, " + std::to_string(NA_MAX_ATOMS) + "]");
    if (kmax < 1 || kmax > NA_MAX_KMAX)
        return na_fail(LG_ERR_ARGUMENT, "lg_ewald_kspace_noalloc: kmax = " + std::to_string(kmax) +
                                            " is outside [1, " + std::to_string(NA_MAX_KMAX) + "]");
    if (!cell || !(cell[0] > 0.0 && cell[1] > 0.0 && cell[2] > 0.0))
        return na_fail(LG_ERR_ARGUMENT, "lg_ewald_kspace_noalloc: cell lengths must be positive");
    if (!(alpha > 0.0)) return na_fail(LG_ERR_ARGUMENT, "lg_ewald_kspace_noalloc: alpha must be positive");
    if (n > 0 && (!d_positions || !d_charges || !d_forces))
        return na_fail(LG_ERR_ARGUMENT, "lg_ewald_kspace_noalloc: null device pointer");

    // once per device, with that device current: the device address of the scratch array
    int dev = 0;
    cudaError_t ce = cudaGetDevice(&dev);
    if (ce != cudaSuccess) return na_fail(LG_ERR_CUDA, cudaGetErrorString(ce));
    if (dev < 0 || dev >= 256) return na_fail(LG_ERR_ARGUMENT, "lg_ewald_kspace_noalloc: device ordinal too large");
    double* scratch;
    {
        std::lock_guard<std::mutex> lock(g_setup_mutex);
        if (!g_scratch_address[dev]) {
            void* p = nullptr;
            ce = cudaGetSymbolAddress(&p, g_noalloc_scratch);
            if (ce != cudaSuccess)
                return na_fail(LG_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(ce));
            g_scratch_address[dev] = (double*)p;
        }
        scratch = g_scratch_address[dev];
    }
    cudaStream_t st = (cudaStream_t)stream;

    // the reference's k-space setup arithmetic (Matrix3::inverse, Ewald::prepare)
    double L[3] = {cell[0], cell[1], cell[2]};
    double det = L[0] * (L[1] * L[2] - 0.0 * 0.0) - 0.0 * (0.0 * L[2] - 0.0 * 0.0) + 0.0 * (0.0 * 0.0 - L[1] * 0.0);
    double id = 1.0 / det;
    double inv[3] = {(L[1] * L[2] - 0.0 * 0.0) * id, (L[0] * L[2] - 0.0 * 0.0) * id, (L[0] * L[1] - 0.0 * 0.0) * id};
    double s[3] = {(2.0 * PI) * inv[0], (2.0 * PI) * inv[1], (2.0 * PI) * inv[2]};
    double mx = std::max(std::max(s[0], s[1]), s[2]) * (double)kmax;
    double kmax2 = 1.0001 * mx * mx;
    double four_pi_v = 4.0 * PI / (L[0] * L[1] * L[2]);
    int ncand = na_candidates(kmax);

    if (ncand > 0 && n > 0) {
        na_kvec_kernel<<<(ncand + 127) / 128, 128, 0, st>>>(scratch, kmax, ncand, s[0], s[1], s[2], kmax2, alpha,
                                                           four_pi_v);
        na_eikr_kernel<<<(3 * (int)n + 255) / 256, 256, 0, st>>>(scratch, d_positions, (int)n, kmax, s[0], s[1],
                                                                s[2]);
        na_rho_kernel<<<ncand, 256, 0, st>>>(scratch, d_charges, (int)n, kmax);
        na_field_kernel<<<((int)n + 127) / 128, 128, 0, st>>>(scratch, d_charges, (int)n, kmax, ncand, d_forces);
    }
    na_reduce_kernel<<<1, 256, 0, st>>>(scratch, n > 0 ? ncand : 0, d_energy, d_virial);
    ce = cudaGetLastError();
    if (ce != cudaSuccess) return na_fail(LG_ERR_CUDA, cudaGetErrorString(ce));
    return LG_OK;
}
