// common.cuh -- shared device helpers for the GB300 permeability kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>

namespace fp {

// Process-wide count of this library's kernel launches (all devices and
// streams), read by fp_kernel_launch_count.  Every launch site bumps it.
extern std::atomic<long long> g_kernel_launches;
// The calling thread's own launches (a stream capture subtracts what it
// recorded: other threads keep launching meanwhile).
extern thread_local long long g_thread_launches;
#define FP_LAUNCHED() \
    (++::fp::g_thread_launches, ::fp::g_kernel_launches.fetch_add(1, std::memory_order_relaxed))

// ---- device memory vs graph capture (capi.cu) ----
// cudaMalloc / cudaFree may synchronise the whole device, which invalidates a
// stream capture running in another host thread.  Every allocation or free
// site holds DeviceMemGuard (exclusive, re-entrant within a thread); every
// capture holds CaptureGuard (shared: captures in different threads overlap).
struct DeviceMemGuard {
    DeviceMemGuard();
    ~DeviceMemGuard();
    DeviceMemGuard(const DeviceMemGuard&) = delete;
    DeviceMemGuard& operator=(const DeviceMemGuard&) = delete;
};
struct CaptureGuard {
    CaptureGuard();
    ~CaptureGuard();
    CaptureGuard(const CaptureGuard&) = delete;
    CaptureGuard& operator=(const CaptureGuard&) = delete;
};


template <typename T>
struct Cplx;
template <>
struct Cplx<double> {
    using type = double2;
};
template <>
struct Cplx<float> {
    using type = float2;
};
template <typename T>
using c_t = typename Cplx<T>::type;

template <typename T2>
__device__ __forceinline__ T2 cmk(decltype(T2::x) a, decltype(T2::x) b) {
    T2 r;
    r.x = a;
    r.y = b;
    return r;
}
template <typename T2>
__device__ __forceinline__ T2 cadd(T2 a, T2 b) {
    return cmk<T2>(a.x + b.x, a.y + b.y);
}
template <typename T2>
__device__ __forceinline__ T2 csub(T2 a, T2 b) {
    return cmk<T2>(a.x - b.x, a.y - b.y);
}
template <typename T2>
__device__ __forceinline__ T2 cmul(T2 a, T2 b) {
    return cmk<T2>(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
template <typename T2>
__device__ __forceinline__ T2 cscale(T2 a, decltype(T2::x) s) {
    return cmk<T2>(a.x * s, a.y * s);
}
template <typename T2>
__device__ __forceinline__ T2 cconj(T2 a) {
    return cmk<T2>(a.x, -a.y);
}
// multiply by sign*i:  (sign*i)*(x + iy) = -sign*y + i*sign*x
template <int SIGN, typename T2>
__device__ __forceinline__ T2 cmul_si(T2 a) {
    return SIGN < 0 ? cmk<T2>(a.y, -a.x) : cmk<T2>(-a.y, a.x);
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Deterministic block reduction of NV doubles per thread.  Every thread
// contributes vals[0..NV); thread 0 gets the block totals in out[0..NV).
// scratch: shared array of at least NV * 32 doubles.
template <int NV>
__device__ __forceinline__ void block_sum(double (&vals)[NV], double* scratch, double* out) {
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int nwarp = (blockDim.x + 31) >> 5;
#pragma unroll
    for (int i = 0; i < NV; ++i) {
        double v = warp_sum(vals[i]);
        if (lane == 0) scratch[i * 32 + warp] = v;
    }
    __syncthreads();
    if (warp == 0) {
#pragma unroll
        for (int i = 0; i < NV; ++i) {
            double v = lane < nwarp ? scratch[i * 32 + lane] : 0.0;
            v = warp_sum(v);
            if (lane == 0) out[i] = v;
        }
    }
    __syncthreads();
}

}  // namespace fp
