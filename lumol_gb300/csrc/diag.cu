// diag.cu -- measurement helpers: a dependent-chain DFMA / FFMA throughput
// probe that gives the FP64 and FP32 pipe peaks the force kernels are bounded
// by (the bench reports its kernels against these measured numbers).
#include "kernels.h"

namespace lg {

// Eight independent FMA chains per thread; `iters` rounds.  The result is
// written only if it is non-finite, so the compiler cannot drop the chains.
template <typename T>
__global__ void fma_probe_kernel(int iters, T a, T b, T* sink) {
    T x0 = (T)threadIdx.x, x1 = x0 + (T)1, x2 = x0 + (T)2, x3 = x0 + (T)3;
    T x4 = x0 + (T)4, x5 = x0 + (T)5, x6 = x0 + (T)6, x7 = x0 + (T)7;
    for (int k = 0; k < iters; k++) {
        x0 = x0 * a + b; x1 = x1 * a + b; x2 = x2 * a + b; x3 = x3 * a + b;
        x4 = x4 * a + b; x5 = x5 * a + b; x6 = x6 * a + b; x7 = x7 * a + b;
    }
    T s = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
    if (!(s == s) || s == (T)12345.678) sink[0] = s;
}

// Returns TFLOP/s (2 flops per FMA) of the FP64 (fp64 != 0) or FP32 pipe.
int measure_fma_peak(int fp64, double* tflops) {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    void* sink = nullptr;
    if (cudaMalloc(&sink, 16) != cudaSuccess) return 2;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    int blocks = sms * 8, threads = 256, iters = fp64 ? 2048 : 16384;
    float best = 1e30f;
    for (int rep = 0; rep < 4; rep++) {
        cudaEventRecord(e0);
        if (fp64)
            fma_probe_kernel<double><<<blocks, threads>>>(iters, 0.999999, 1e-7, (double*)sink);
        else
            fma_probe_kernel<float><<<blocks, threads>>>(iters, 0.999999f, 1e-7f, (float*)sink);
        cudaEventRecord(e1);
        cudaEventSynchronize(e1);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (rep > 0 && ms < best) best = ms;
    }
    cudaError_t err = cudaGetLastError();
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(sink);
    if (err != cudaSuccess) return 2;
    double flops = 2.0 * 8.0 * (double)iters * (double)blocks * (double)threads;
    *tflops = flops / (best * 1e-3) / 1e12;
    return 0;
}

}  // namespace lg
