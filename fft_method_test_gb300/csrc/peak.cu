// peak.cu -- FP64 arithmetic throughput of the current device, measured by a
// kernel of independent FMA chains (fp_measure_fp64_rate).  The FP64 apply is
// bound by this rate rather than by HBM on GB300, so its roofline needs the
// measured figure.
#include <cuda_runtime.h>

#include "../../include/fftperm.h"
#include "common.cuh"

namespace fp {
namespace {

constexpr int kChains = 8;

// Each thread runs kChains independent FMA chains of `iters` steps; the
// multiplier keeps the values bounded and the final test keeps the compiler
// from dropping the work.
__global__ void __launch_bounds__(256) k_dfma_rate(int iters, double seed, double* out) {
    double v[kChains];
#pragma unroll
    for (int c = 0; c < kChains; ++c) v[c] = seed + 1e-3 * (threadIdx.x + c);
    const double m = 0.999999, a = 1e-7;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int c = 0; c < kChains; ++c) v[c] = fma(v[c], m, a);
    }
    double s = 0.0;
#pragma unroll
    for (int c = 0; c < kChains; ++c) s += v[c];
    if (s == 12345.678) out[blockIdx.x] = s;  // practically never taken
}

}  // namespace
}  // namespace fp

extern "C" int fp_measure_fp64_rate(double* tflops, double* ms) {
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return FP_ERR_CUDA;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        return FP_ERR_CUDA;
    const int blocks = 8 * sms, threads = 256, iters = 4096, reps = 5;
    double* d_out = nullptr;
    if (cudaMalloc(&d_out, sizeof(double) * blocks) != cudaSuccess) return FP_ERR_NOMEM;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    FP_LAUNCHED();
    fp::k_dfma_rate<<<blocks, threads>>>(iters, 1.0, d_out);  // warm-up
    cudaEventRecord(e0);
    for (int r = 0; r < reps; ++r) {
        FP_LAUNCHED();
        fp::k_dfma_rate<<<blocks, threads>>>(iters, 1.0 + r, d_out);
    }
    cudaEventRecord(e1);
    const cudaError_t e = cudaEventSynchronize(e1);
    float t = 0.f;
    cudaEventElapsedTime(&t, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(d_out);
    if (e != cudaSuccess || t <= 0.f) return FP_ERR_CUDA;
    const double flops = 2.0 * fp::kChains * (double)iters * blocks * threads * reps;
    if (ms) *ms = t / reps;
    if (tflops) *tflops = flops / (t * 1e-3) / 1e12;
    return FP_OK;
}
