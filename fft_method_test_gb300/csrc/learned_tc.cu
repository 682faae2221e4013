// learned_tc.cu -- the 3x3x3 convolution of the learned warm start on the
// fifth-generation tensor cores: tcgen05.mma with the accumulator in tensor
// memory (TMEM), operands staged in shared memory.  No counterpart in the
// reference (its MinresSolver::solve takes an initial guess,
// src/solver/MinresSolver.hpp:23, that nothing fills).
//
// Implicit GEMM, one CTA per 128 voxels (the MMA's M):
//   y[v][o] = sum_tap sum_i x[v + sign*dil*off(tap)][i] W[tap][o][i]
// Activations are channels-last BF16 [voxel][channel], weights BF16
// [27][cout][cin] (the data gradient passes the per-tap transposed weights
// and sign -1), periodic wrap, FP32 accumulation.  Per tap the 128 shifted
// input rows (A, 128 x cin) and the tap's weights (B, cout x cin) are
// copied into one of two shared-memory buffers with cp.async, in the
// canonical K-major layout without swizzle: 8 x 16-byte core matrices, the
// two core matrices of a 16-channel chunk side by side (leading byte offset
// 128), 8-row groups 256 bytes apart (stride byte offset).  One thread issues
// cin/16 MMAs of 128 x cout x 16 per tap and commits them to the buffer's
// mbarrier, so the 128 threads gather tap t + 1 while the tensor cores work
// on tap t.  The epilogue reads the accumulator rows back with tcgen05.ld
// (warp w owns TMEM lanes 32w..32w+31 = voxel rows), adds the bias, applies
// ReLU and stores FP32 and/or BF16.
//
// Every wait is bounded (the mbarrier helpers of tma.cuh): on a timeout the
// CTA raises the file-scope error flag (fp_nn_tc_error), frees its TMEM and
// returns.  The dynamic shared memory of a CTA is at least its share of the
// SM for the TMEM columns it holds, so the CTAs resident on an SM never ask
// for more than the 512 TMEM columns there are.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/fftperm.h"
#include "common.cuh"
#include "tma.cuh"

#ifndef FP_TC_LBO
#define FP_TC_LBO 128  // bytes between the two core matrices of a 16-channel chunk
#endif
#ifndef FP_TC_SBO
#define FP_TC_SBO 256  // bytes between 8-row groups
#endif

namespace fp {
namespace {

constexpr int kTcM = 128;  // voxels per CTA = MMA M = TMEM lanes
constexpr int kTcThreads = 128;

__device__ int g_tc_err = 0;

struct TcConv {
    int nx, ny, nz;
    long long n;      // voxels per sample
    long long total;  // voxels of all samples
    int dil, sign;
    const __nv_bfloat16* in;
    int cin;
    const __nv_bfloat16* w;
    const float* bias;
    int relu;
    float* out32;
    __nv_bfloat16* out16;
};

__device__ __forceinline__ void cp_async16_zfill(void* smem, const void* gmem, bool valid) {
    const int n = valid ? 16 : 0;  // src-size 0: the 16 bytes are zero-filled
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(smem_u32(smem)), "l"(gmem),
                 "r"(n)
                 : "memory");
}

// shared-memory matrix descriptor: K-major, no swizzle
__device__ __forceinline__ uint64_t smem_desc(const void* p) {
    const uint32_t a = smem_u32(p);
    return (uint64_t)((a >> 4) & 0x3FFF) | ((uint64_t)((FP_TC_LBO >> 4) & 0x3FFF) << 16) |
           ((uint64_t)((FP_TC_SBO >> 4) & 0x3FFF) << 32) | (1ull << 46);
}

// instruction descriptor of kind::f16: BF16 A and B, FP32 D, K-major both,
// N = cout, M = 128
template <int N>
__device__ __forceinline__ constexpr uint32_t idesc_bf16() {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) |
           ((uint32_t)(kTcM >> 4) << 24);
}

__device__ __forceinline__ void tc_fence_before() {
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

// core-matrix position of element row m, 8-element group q (k = 8q..8q+7)
// inside a tile of `rows` rows: chunk q / 2 of rows * 32 bytes, core matrix
// ((m / 8) * 2 + q % 2) of 128 bytes, row m % 8 of 16 bytes
__device__ __forceinline__ uint32_t core_offset(int m, int q, int rows) {
    return (uint32_t)((q >> 1) * rows * 32 + ((m >> 3) * 2 + (q & 1)) * 128 + (m & 7) * 16);
}

template <int COUT>
__global__ void __launch_bounds__(kTcThreads) k_conv_tc(TcConv p) {
    constexpr int NCOLS = COUT < 32 ? 32 : COUT;  // TMEM columns (power of two, >= 32)
    extern __shared__ __align__(1024) unsigned char sm[];
    uint64_t* bars = reinterpret_cast<uint64_t*>(sm);
    uint32_t* tslot = reinterpret_cast<uint32_t*>(sm + 16);
    const int tid = threadIdx.x;
    const int warp = tid >> 5;
    const int cin = p.cin;
    const int kc = cin / 16;
    const uint32_t abytes = (uint32_t)kTcM * cin * 2;
    const uint32_t bbytes = (uint32_t)COUT * cin * 2;
    unsigned char* buf0 = sm + 1024;
    auto abuf = [&](int b) { return buf0 + (size_t)b * (abytes + bbytes); };
    auto bbuf = [&](int b) { return buf0 + (size_t)b * (abytes + bbytes) + abytes; };

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         smem_u32(tslot)),
                     "r"(NCOLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0) {
        mbar_init(&bars[0], 1);
        mbar_init(&bars[1], 1);
        fence_mbar_init();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tslot;

    // this thread's voxel (A row tid)
    const long long v = (long long)blockIdx.x * kTcM + tid;
    const bool valid = v < p.total;
    const long long vv = valid ? v : 0;
    const long long smp = vv / p.n;
    const long long r = vv - smp * p.n;
    const int x = (int)(r % p.nx);
    const long long q0 = r / p.nx;
    const int y = (int)(q0 % p.ny);
    const int z = (int)(q0 / p.ny);
    const int step = p.sign * p.dil;

    bool ok = true;
    int last = 0;
    for (int tap = 0; tap < 27; ++tap) {
        const int b = tap & 1;
        // the MMAs of tap - 2 read this buffer
        if (tap >= 2 && !tma_pipeline_wait<float2>(bars, tap - 2, b, true, &g_tc_err)) {
            ok = false;
            break;
        }
        // A: the shifted input row of this voxel
        {
            const int dz = tap / 9 - 1, dy = (tap / 3) % 3 - 1, dx = tap % 3 - 1;
            int xx = (x + step * dx) % p.nx, yy = (y + step * dy) % p.ny, zz = (z + step * dz) % p.nz;
            if (xx < 0) xx += p.nx;
            if (yy < 0) yy += p.ny;
            if (zz < 0) zz += p.nz;
            const long long nb = smp * p.n + ((long long)zz * p.ny + yy) * p.nx + xx;
            const __nv_bfloat16* src = p.in + nb * cin;
            unsigned char* a = abuf(b);
            for (int q = 0; q < cin / 8; ++q)
                cp_async16_zfill(a + core_offset(tid, q, kTcM), src + q * 8, valid);
        }
        // B: the tap's weights [cout][cin]
        {
            const int per = cin / 8;
            const __nv_bfloat16* wt = p.w + (size_t)tap * COUT * cin;
            unsigned char* bm = bbuf(b);
            for (int i = tid; i < COUT * per; i += kTcThreads) {
                const int co = i / per;
                const int q = i - co * per;
                cp_async16_zfill(bm + core_offset(co, q, COUT), wt + (size_t)co * cin + q * 8, true);
            }
        }
        asm volatile("cp.async.wait_all;" ::: "memory");
        fence_proxy_async_smem();
        __syncthreads();
        if (tid == 0) {
            tc_fence_after();
            const unsigned char* a = abuf(b);
            const unsigned char* bm = bbuf(b);
            for (int k = 0; k < kc; ++k) {
                const uint64_t ad = smem_desc(a + (size_t)k * kTcM * 32);
                const uint64_t bd = smem_desc(bm + (size_t)k * COUT * 32);
                const uint32_t acc = (tap | k) != 0;
                asm volatile(
                    "{\n"
                    " .reg .pred p;\n"
                    " setp.ne.b32 p, %4, 0;\n"
                    " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n"
                    "}\n" ::"r"(tmem),
                    "l"(ad), "l"(bd), "r"(idesc_bf16<COUT>()), "r"(acc)
                    : "memory");
            }
            asm volatile(
                "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                    smem_u32(&bars[b]))
                : "memory");
        }
        last = tap;
    }
    // the last commit covers every MMA issued before it
    if (ok) ok = tma_pipeline_wait<float2>(bars, last, last & 1, false, &g_tc_err);
    tc_fence_after();
    if (ok) {
        // epilogue: TMEM lanes 32w..32w+31 are the rows of warp w
        const uint32_t trow = tmem + ((uint32_t)(warp * 32) << 16);
#pragma unroll
        for (int c0 = 0; c0 < COUT; c0 += 16) {
            uint32_t rr[16];
            asm volatile(
                "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,"
                "%13,%14,%15}, [%16];"
                : "=r"(rr[0]), "=r"(rr[1]), "=r"(rr[2]), "=r"(rr[3]), "=r"(rr[4]), "=r"(rr[5]),
                  "=r"(rr[6]), "=r"(rr[7]), "=r"(rr[8]), "=r"(rr[9]), "=r"(rr[10]), "=r"(rr[11]),
                  "=r"(rr[12]), "=r"(rr[13]), "=r"(rr[14]), "=r"(rr[15])
                : "r"(trow + (uint32_t)c0));
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
            float f[16];
#pragma unroll
            for (int j = 0; j < 16; ++j) {
                f[j] = __uint_as_float(rr[j]);
                if (p.bias) f[j] += p.bias[c0 + j];
                if (p.relu) f[j] = fmaxf(f[j], 0.f);
            }
            if (valid) {
                if (p.out32) {
                    float4* o = reinterpret_cast<float4*>(p.out32 + v * COUT + c0);
#pragma unroll
                    for (int j = 0; j < 4; ++j)
                        o[j] = make_float4(f[4 * j], f[4 * j + 1], f[4 * j + 2], f[4 * j + 3]);
                }
                if (p.out16) {
                    uint32_t pk[8];
#pragma unroll
                    for (int j = 0; j < 8; ++j) {
                        const uint32_t lo = __bfloat16_as_ushort(__float2bfloat16(f[2 * j]));
                        const uint32_t hi = __bfloat16_as_ushort(__float2bfloat16(f[2 * j + 1]));
                        pk[j] = lo | (hi << 16);
                    }
                    uint4* o = reinterpret_cast<uint4*>(p.out16 + v * COUT + c0);
                    o[0] = make_uint4(pk[0], pk[1], pk[2], pk[3]);
                    o[1] = make_uint4(pk[4], pk[5], pk[6], pk[7]);
                }
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(NCOLS)
                     : "memory");
}

// the largest dynamic shared memory a CTA may use, set once per kernel and device
template <typename K>
void ensure_smem_limit(K kern, std::atomic<unsigned long long>& done) {
    int dev = 0;
    cudaGetDevice(&dev);
    const unsigned long long bit = 1ull << (dev & 63);
    if (!(done.load(std::memory_order_acquire) & bit)) {
        cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, 232448);
        done.fetch_or(bit, std::memory_order_release);
    }
}

// shared memory of one CTA: barriers + two buffers, and at least the CTA's
// share of the SM for its TMEM columns
size_t tc_smem(int cin, int cout) {
    const int ncols = cout < 32 ? 32 : cout;
    const size_t need = 1024 + 2 * ((size_t)kTcM * cin * 2 + (size_t)cout * cin * 2);
    const size_t share = (size_t)233472 * ncols / 512;
    return need > share ? need : share;
}

}  // namespace
}  // namespace fp

extern "C" int fp_nn_conv_tc(int nx, int ny, int nz, int64_t total, int dilation, int sign,
                             const void* in_bf16, int cin, const void* w_bf16, const float* bias,
                             int cout, int relu, float* out_f32, void* out_bf16, void* stream) {
    if (nx <= 0 || ny <= 0 || nz <= 0 || total <= 0 || cin <= 0 || cin % 16 || cin > 128 ||
        !in_bf16 || !w_bf16 || (!out_f32 && !out_bf16))
        return FP_ERR_INVALID;
    if (dilation < 1 || (sign != 1 && sign != -1)) return FP_ERR_INVALID;
    fp::TcConv p{nx, ny, nz, (long long)nx * ny * nz, (long long)total, dilation, sign,
                 static_cast<const __nv_bfloat16*>(in_bf16), cin,
                 static_cast<const __nv_bfloat16*>(w_bf16), bias, relu, out_f32,
                 static_cast<__nv_bfloat16*>(out_bf16)};
    if (p.total % p.n) return FP_ERR_INVALID;
    const long long blocks = (p.total + fp::kTcM - 1) / fp::kTcM;
    if (blocks > 0x7fffffffLL) return FP_ERR_INVALID;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const size_t smem = fp::tc_smem(cin, cout);
    if (smem > 232448) return FP_ERR_INVALID;
#define FP_TC_LAUNCH(C)                                                                           \
    {                                                                                             \
        static std::atomic<unsigned long long> done_{0};                                          \
        fp::ensure_smem_limit(fp::k_conv_tc<C>, done_);                                               \
        FP_LAUNCHED();                                                                            \
        fp::k_conv_tc<C><<<(unsigned)blocks, fp::kTcThreads, smem, s>>>(p);                       \
    }
    switch (cout) {
        case 16: FP_TC_LAUNCH(16) break;
        case 32: FP_TC_LAUNCH(32) break;
        case 64: FP_TC_LAUNCH(64) break;
        case 128: FP_TC_LAUNCH(128) break;
        default: return FP_ERR_INVALID;
    }
#undef FP_TC_LAUNCH
    return cudaGetLastError() == cudaSuccess ? FP_OK : FP_ERR_CUDA;
}

extern "C" int fp_nn_tc_error(int* flag, int reset) {
    int h = 0;
    if (cudaMemcpyFromSymbol(&h, fp::g_tc_err, sizeof(int)) != cudaSuccess) return FP_ERR_CUDA;
    if (flag) *flag = h;
    if (reset) {
        const int z = 0;
        if (cudaMemcpyToSymbol(fp::g_tc_err, &z, sizeof(int)) != cudaSuccess) return FP_ERR_CUDA;
    }
    return FP_OK;
}
