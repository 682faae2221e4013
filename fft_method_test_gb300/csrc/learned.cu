// learned.cu -- kernels of the learned warm start: a small 3-D convolutional
// network that maps a geometry to the interface-force field MINRES starts
// from.  No counterpart in the reference (its MinresSolver::solve takes an
// initial guess, src/solver/MinresSolver.hpp:23, that nothing fills).
//
// Tensors are channels-last: activations [voxel][channel] in BF16 (x fastest
// flat voxel index, samples stacked), weights [tap][out][in] in BF16 with an
// FP32 master copy, tap = (dz+1)*9 + (dy+1)*3 + (dx+1) scaled by the layer's
// dilation, periodic wrap.  Every convolution is an implicit GEMM on the
// tensor cores (mma.sync m16n8k16, BF16 in, FP32 accumulate):
//   forward  y[v][o] = sum_tap sum_i x[v + off(tap)][i] W[tap][o][i]
//   dgrad    dx[u][i] = sum_tap sum_o dy[u - off(tap)][o] W[tap][o][i]
//            (the forward kernel with sign -1 on the offsets and W
//            transposed per tap)
//   wgrad    dW[tap][o][i] = sum_v dy[v][o] x[v + off(tap)][i]
//            (per tap a GEMM over voxels; per-warp partials reduced in a
//            fixed order: deterministic)
// Channel counts: inputs of a convolution a multiple of 16 (the MMA's k),
// outputs a multiple of 8 (its n), at most 64.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/fftperm.h"
#include "common.cuh"

namespace fp {
namespace {

constexpr int kNnWarps = 4;  // warps per CTA; 16 voxels per warp

struct ConvGeom {
    int nx, ny, nz;
    long long n;      // voxels per sample
    long long total;  // voxels of all samples
    int dil;
    int sign;  // +1 forward, -1 data gradient
};

__device__ __forceinline__ long long neighbour(const ConvGeom& g, long long v, int tap) {
    const long long b = v / g.n;
    const long long r = v - b * g.n;
    int x = (int)(r % g.nx);
    const long long q = r / g.nx;
    int y = (int)(q % g.ny);
    int z = (int)(q / g.ny);
    const int dz = tap / 9 - 1, dy = (tap / 3) % 3 - 1, dx = tap % 3 - 1;
    const int s = g.sign * g.dil;
    x = (x + s * dx) % g.nx;
    y = (y + s * dy) % g.ny;
    z = (z + s * dz) % g.nz;
    if (x < 0) x += g.nx;
    if (y < 0) y += g.ny;
    if (z < 0) z += g.nz;
    return b * g.n + ((long long)z * g.ny + y) * g.nx + x;
}

__device__ __forceinline__ void mma_bf16(float c[4], const uint32_t a[4], const uint32_t b[2]) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
        "{%8,%9}, {%0,%1,%2,%3};"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

__device__ __forceinline__ uint32_t ld32(const __nv_bfloat16* p) {
    return *reinterpret_cast<const uint32_t*>(p);
}

__device__ __forceinline__ uint32_t pack2(__nv_bfloat16 lo, __nv_bfloat16 hi) {
    const uint32_t l = (uint32_t)__bfloat16_as_ushort(lo);
    const uint32_t h = (uint32_t)__bfloat16_as_ushort(hi);
    return l | (h << 16);
}

// One warp: 16 consecutive voxels x all COUT output channels.
template <int COUT>
__global__ void __launch_bounds__(32 * kNnWarps) k_conv(ConvGeom g, const __nv_bfloat16* __restrict__ in,
                                                         int cin, const __nv_bfloat16* __restrict__ w,
                                                         const float* __restrict__ bias, int relu,
                                                         float* __restrict__ out32,
                                                         __nv_bfloat16* __restrict__ out16) {
    constexpr int NT = COUT / 8;
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const long long v0 = ((long long)blockIdx.x * kNnWarps + warp) * 16;
    if (v0 >= g.total) return;
    const int grp = lane >> 2;
    const int qd = lane & 3;
    const long long va = v0 + grp, vb = v0 + grp + 8;
    const bool oka = va < g.total, okb = vb < g.total;
    float acc[NT][4];
#pragma unroll
    for (int t = 0; t < NT; ++t) acc[t][0] = acc[t][1] = acc[t][2] = acc[t][3] = 0.f;
    const int kc = cin / 16;
    for (int tap = 0; tap < 27; ++tap) {
        const long long na = oka ? neighbour(g, va, tap) : 0;
        const long long nb = okb ? neighbour(g, vb, tap) : 0;
        for (int k = 0; k < kc; ++k) {
            const int c0 = k * 16 + qd * 2;
            uint32_t a[4];
            a[0] = oka ? ld32(in + na * cin + c0) : 0u;
            a[1] = okb ? ld32(in + nb * cin + c0) : 0u;
            a[2] = oka ? ld32(in + na * cin + c0 + 8) : 0u;
            a[3] = okb ? ld32(in + nb * cin + c0 + 8) : 0u;
#pragma unroll
            for (int t = 0; t < NT; ++t) {
                const __nv_bfloat16* wp = w + ((long long)tap * COUT + t * 8 + grp) * cin + c0;
                uint32_t b[2];
                b[0] = ld32(wp);
                b[1] = ld32(wp + 8);
                mma_bf16(acc[t], a, b);
            }
        }
    }
#pragma unroll
    for (int t = 0; t < NT; ++t) {
        const int o = t * 8 + qd * 2;
        float r[4] = {acc[t][0], acc[t][1], acc[t][2], acc[t][3]};
        if (bias) {
            r[0] += bias[o];
            r[1] += bias[o + 1];
            r[2] += bias[o];
            r[3] += bias[o + 1];
        }
        if (relu)
#pragma unroll
            for (int j = 0; j < 4; ++j) r[j] = fmaxf(r[j], 0.f);
        if (oka) {
            if (out32) {
                out32[va * COUT + o] = r[0];
                out32[va * COUT + o + 1] = r[1];
            }
            if (out16) {
                out16[va * COUT + o] = __float2bfloat16(r[0]);
                out16[va * COUT + o + 1] = __float2bfloat16(r[1]);
            }
        }
        if (okb) {
            if (out32) {
                out32[vb * COUT + o] = r[2];
                out32[vb * COUT + o + 1] = r[3];
            }
            if (out16) {
                out16[vb * COUT + o] = __float2bfloat16(r[2]);
                out16[vb * COUT + o + 1] = __float2bfloat16(r[3]);
            }
        }
    }
}

// Weight gradient partials: warp (tap, chunk) sums over its voxel chunk.
// A = dy^T (rows o, cols voxels), B = x shifted (rows voxels, cols i).
// partial[chunk][tap][cout16][cin] in FP32.
template <int CO16, int CIN>
__global__ void __launch_bounds__(32) k_wgrad(ConvGeom g, const __nv_bfloat16* __restrict__ dy, int cout,
                                               const __nv_bfloat16* __restrict__ x, long long chunk,
                                               float* __restrict__ partial) {
    constexpr int MT = CO16 / 16;
    constexpr int NT = CIN / 8;
    const int tap = blockIdx.y;
    const long long c = blockIdx.x;
    const int lane = threadIdx.x;
    const int grp = lane >> 2;
    const int qd = lane & 3;
    float acc[MT][NT][4];
#pragma unroll
    for (int m = 0; m < MT; ++m)
#pragma unroll
        for (int t = 0; t < NT; ++t) acc[m][t][0] = acc[m][t][1] = acc[m][t][2] = acc[m][t][3] = 0.f;
    const long long v_begin = c * chunk;
    const long long v_end = min(g.total, v_begin + chunk);
    const __nv_bfloat16 zero = __float2bfloat16(0.f);
    for (long long k0 = v_begin; k0 < v_end; k0 += 16) {
        // voxels of this k-step held by this thread: k0 + qd*2 + {0,1} and +8
        long long vk[4];
        bool ok[4];
        long long nk[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            vk[j] = k0 + qd * 2 + (j & 1) + (j >> 1) * 8;
            ok[j] = vk[j] < v_end;
            nk[j] = ok[j] ? neighbour(g, vk[j], tap) : 0;
        }
#pragma unroll
        for (int m = 0; m < MT; ++m) {
            const int oa = m * 16 + grp, ob = oa + 8;
            auto dyv = [&](int j, int o) { return (ok[j] && o < cout) ? dy[vk[j] * cout + o] : zero; };
            uint32_t a[4];
            a[0] = pack2(dyv(0, oa), dyv(1, oa));
            a[1] = pack2(dyv(0, ob), dyv(1, ob));
            a[2] = pack2(dyv(2, oa), dyv(3, oa));
            a[3] = pack2(dyv(2, ob), dyv(3, ob));
#pragma unroll
            for (int t = 0; t < NT; ++t) {
                const int i = t * 8 + grp;
                uint32_t b[2];
                b[0] = pack2(ok[0] ? x[nk[0] * CIN + i] : zero, ok[1] ? x[nk[1] * CIN + i] : zero);
                b[1] = pack2(ok[2] ? x[nk[2] * CIN + i] : zero, ok[3] ? x[nk[3] * CIN + i] : zero);
                mma_bf16(acc[m][t], a, b);
            }
        }
    }
    float* dst = partial + ((c * 27 + tap) * (long long)CO16) * CIN;
#pragma unroll
    for (int m = 0; m < MT; ++m)
#pragma unroll
        for (int t = 0; t < NT; ++t) {
            const int o = m * 16 + grp;
            const int i = t * 8 + qd * 2;
            dst[(long long)o * CIN + i] = acc[m][t][0];
            dst[(long long)o * CIN + i + 1] = acc[m][t][1];
            dst[(long long)(o + 8) * CIN + i] = acc[m][t][2];
            dst[(long long)(o + 8) * CIN + i + 1] = acc[m][t][3];
        }
}

// dW[tap][o][i] (o < cout) = sum over chunks of the partials, in chunk order.
__global__ void k_wgrad_reduce(const float* __restrict__ partial, long long nchunks, int co16, int cin,
                               int cout, float* __restrict__ dw) {
    const long long m = 27LL * cout * cin;
    for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < m;
         e += (long long)gridDim.x * blockDim.x) {
        const long long tap = e / ((long long)cout * cin);
        const long long r = e - tap * cout * cin;
        const long long o = r / cin, i = r - o * cin;
        float s = 0.f;
        for (long long c = 0; c < nchunks; ++c) s += partial[((c * 27 + tap) * co16 + o) * cin + i];
        dw[e] = s;
    }
}

// db[o] = sum_v dy[v][o]   (one CTA per output channel, fixed order)
__global__ void k_bias_grad(const __nv_bfloat16* __restrict__ dy, long long total, int cout, float* db) {
    __shared__ float red[256];
    const int o = blockIdx.x;
    float s = 0.f;
    for (long long v = threadIdx.x; v < total; v += blockDim.x) s += __bfloat162float(dy[v * cout + o]);
    red[threadIdx.x] = s;
    __syncthreads();
    for (int h = blockDim.x / 2; h > 0; h >>= 1) {
        if (threadIdx.x < h) red[threadIdx.x] += red[threadIdx.x + h];
        __syncthreads();
    }
    if (threadIdx.x == 0) db[o] = red[0];
}

// dpre = dpost * (post > 0) into BF16, with channel padding cpad >= c (zeros)
__global__ void k_relu_back(const float* __restrict__ dpost, const __nv_bfloat16* __restrict__ post,
                            long long total, int c, int cpad, __nv_bfloat16* __restrict__ out) {
    const long long m = total * cpad;
    for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < m;
         e += (long long)gridDim.x * blockDim.x) {
        const long long v = e / cpad;
        const int j = (int)(e - v * cpad);
        float d = 0.f;
        if (j < c) {
            d = dpost[v * c + j];
            if (post && !(__bfloat162float(post[v * c + j]) > 0.f)) d = 0.f;
        }
        out[e] = __float2bfloat16(d);
    }
}

// Adam on FP32 masters; refreshes the BF16 forward weights [tap][o][i] and
// the transposed copy [tap][i][o] used by the data gradient.
__global__ void k_adam(float* __restrict__ w, float* __restrict__ m1, float* __restrict__ m2,
                       const float* __restrict__ g, long long count, float lr, float b1, float b2,
                       float eps, float c1, float c2, int cout, int cin,
                       __nv_bfloat16* __restrict__ wf, __nv_bfloat16* __restrict__ wt) {
    for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < count;
         e += (long long)gridDim.x * blockDim.x) {
        const float gr = g[e];
        const float a = b1 * m1[e] + (1.f - b1) * gr;
        const float b = b2 * m2[e] + (1.f - b2) * gr * gr;
        m1[e] = a;
        m2[e] = b;
        const float v = w[e] - lr * (a / c1) / (sqrtf(b / c2) + eps);
        w[e] = v;
        if (wf) {
            const long long tap = e / ((long long)cout * cin);
            const long long r = e - tap * cout * cin;
            const long long o = r / cin, i = r - o * cin;
            wf[e] = __float2bfloat16(v);
            wt[(tap * cin + i) * cout + o] = __float2bfloat16(v);
        }
    }
}

// Per (sample, component): sum of the prediction over the support voxels,
// and the support count (one CTA per sample, fixed order).
__global__ void k_loss_stats(const float* __restrict__ pred, int cstride, const uint8_t* __restrict__ sup,
                             long long n, float* stats) {
    __shared__ float red[4][256];
    const long long b = blockIdx.x;
    float a[4] = {0.f, 0.f, 0.f, 0.f};
    for (long long v = threadIdx.x; v < n; v += blockDim.x) {
        const long long g = b * n + v;
        if (sup[g]) {
            a[0] += pred[g * cstride];
            a[1] += pred[g * cstride + 1];
            a[2] += pred[g * cstride + 2];
            a[3] += 1.f;
        }
    }
    for (int j = 0; j < 4; ++j) red[j][threadIdx.x] = a[j];
    __syncthreads();
    for (int h = blockDim.x / 2; h > 0; h >>= 1) {
        if (threadIdx.x < h)
            for (int j = 0; j < 4; ++j) red[j][threadIdx.x] += red[j][threadIdx.x + h];
        __syncthreads();
    }
    if (threadIdx.x == 0)
        for (int j = 0; j < 4; ++j) stats[4 * b + j] = red[j][0];
}

// Relative squared error per sample, sum_s |P pred - t|^2 / sum_s |t|^2 with
// P the per-component mean removal over the support (the operator's null
// space), and its gradient 2 w (P pred - t) on the support, 0 elsewhere.
// tnorm[b] = sum_s |t|^2; loss[b] receives the per-sample error.
__global__ void k_loss_grad(const float* __restrict__ pred, int cstride, const float* __restrict__ tgt,
                            const uint8_t* __restrict__ sup, long long n, const float* __restrict__ stats,
                            const float* __restrict__ tnorm, float* __restrict__ dpred, float* loss) {
    __shared__ float red[256];
    const long long b = blockIdx.x;
    const float cnt = fmaxf(stats[4 * b + 3], 1.f);
    const float mean[3] = {stats[4 * b] / cnt, stats[4 * b + 1] / cnt, stats[4 * b + 2] / cnt};
    const float w = 1.f / fmaxf(tnorm[b], 1e-30f);
    float acc = 0.f;
    for (long long v = threadIdx.x; v < n; v += blockDim.x) {
        const long long g = b * n + v;
        for (int c = 0; c < cstride; ++c) {
            float d = 0.f;
            if (c < 3 && sup[g]) {
                const float r = pred[g * cstride + c] - mean[c] - tgt[g * 3 + c];
                acc += r * r;
                d = 2.f * w * r;
            }
            dpred[g * cstride + c] = d;
        }
    }
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int h = blockDim.x / 2; h > 0; h >>= 1) {
        if (threadIdx.x < h) red[threadIdx.x] += red[threadIdx.x + h];
        __syncthreads();
    }
    if (threadIdx.x == 0) loss[b] = red[0] * w;
}

int grid_for(long long m, int threads) {
    long long b = (m + threads - 1) / threads;
    if (b > 65535LL * 8) b = 65535LL * 8;
    return (int)(b < 1 ? 1 : b);
}

}  // namespace
}  // namespace fp

using fp::ConvGeom;

// Forward (sign +1) or data-gradient (sign -1) convolution.  total = voxels of
// all samples; n = voxels per sample.  cin % 16 == 0, cout in {8, 16, 32, 64}.
extern "C" int fp_nn_conv(int nx, int ny, int nz, int64_t total, int dilation, int sign,
                          const void* in_bf16, int cin, const void* w_bf16, const float* bias,
                          int cout, int relu, float* out_f32, void* out_bf16, void* stream) {
    if (nx <= 0 || ny <= 0 || nz <= 0 || total <= 0 || cin <= 0 || cin % 16 || !in_bf16 || !w_bf16)
        return FP_ERR_INVALID;
    ConvGeom g{nx, ny, nz, (long long)nx * ny * nz, (long long)total, dilation, sign};
    if (g.total % g.n) return FP_ERR_INVALID;
    const long long warps = (g.total + 15) / 16;
    const int blocks = (int)((warps + fp::kNnWarps - 1) / fp::kNnWarps);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    auto in = static_cast<const __nv_bfloat16*>(in_bf16);
    auto w = static_cast<const __nv_bfloat16*>(w_bf16);
    auto o16 = static_cast<__nv_bfloat16*>(out_bf16);
    switch (cout) {
        case 8: FP_LAUNCHED(); fp::k_conv<8><<<blocks, 32 * fp::kNnWarps, 0, s>>>(g, in, cin, w, bias, relu, out_f32, o16); break;
        case 16: FP_LAUNCHED(); fp::k_conv<16><<<blocks, 32 * fp::kNnWarps, 0, s>>>(g, in, cin, w, bias, relu, out_f32, o16); break;
        case 32: FP_LAUNCHED(); fp::k_conv<32><<<blocks, 32 * fp::kNnWarps, 0, s>>>(g, in, cin, w, bias, relu, out_f32, o16); break;
        case 64: FP_LAUNCHED(); fp::k_conv<64><<<blocks, 32 * fp::kNnWarps, 0, s>>>(g, in, cin, w, bias, relu, out_f32, o16); break;
        default: return FP_ERR_INVALID;
    }
    return cudaGetLastError() == cudaSuccess ? FP_OK : FP_ERR_CUDA;
}

// dW (FP32 [27][cout][cin]) of a forward convolution from its output gradient
// dy (BF16 [total][cout]) and input x (BF16 [total][cin]).  partial: scratch
// of nchunks*27*cout16*cin floats, nchunks = ceil(total / chunk).
extern "C" int fp_nn_wgrad(int nx, int ny, int nz, int64_t total, int dilation, const void* dy_bf16,
                           int cout, const void* x_bf16, int cin, int64_t chunk, float* partial,
                           float* dw, void* stream) {
    if (nx <= 0 || ny <= 0 || nz <= 0 || total <= 0 || chunk <= 0 || chunk % 16 || !dy_bf16 || !x_bf16 ||
        !partial || !dw)
        return FP_ERR_INVALID;
    ConvGeom g{nx, ny, nz, (long long)nx * ny * nz, (long long)total, dilation, +1};
    const long long nchunks = (g.total + chunk - 1) / chunk;
    if (nchunks > 65535) return FP_ERR_INVALID;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    auto dy = static_cast<const __nv_bfloat16*>(dy_bf16);
    auto x = static_cast<const __nv_bfloat16*>(x_bf16);
    const dim3 grid((unsigned)nchunks, 27);
    const int co16 = (cout + 15) / 16 * 16;
#define FP_WG(C16, CI)                                                                  \
    do {                                                                                \
        FP_LAUNCHED();                                                                  \
        fp::k_wgrad<C16, CI><<<grid, 32, 0, s>>>(g, dy, cout, x, (long long)chunk, partial); \
    } while (0)
    if (co16 == 16 && cin == 16) FP_WG(16, 16);
    else if (co16 == 16 && cin == 32) FP_WG(16, 32);
    else if (co16 == 32 && cin == 16) FP_WG(32, 16);
    else if (co16 == 32 && cin == 32) FP_WG(32, 32);
    else if (co16 == 64 && cin == 32) FP_WG(64, 32);
    else if (co16 == 32 && cin == 64) FP_WG(32, 64);
    else if (co16 == 64 && cin == 64) FP_WG(64, 64);
    else return FP_ERR_INVALID;
#undef FP_WG
    FP_LAUNCHED();
    fp::k_wgrad_reduce<<<fp::grid_for(27LL * cout * cin, 256), 256, 0, s>>>(partial, nchunks, co16, cin,
                                                                           cout, dw);
    return cudaGetLastError() == cudaSuccess ? FP_OK : FP_ERR_CUDA;
}

extern "C" int fp_nn_bias_grad(const void* dy_bf16, int64_t total, int cout, float* db, void* stream) {
    if (!dy_bf16 || !db || total <= 0 || cout <= 0) return FP_ERR_INVALID;
    FP_LAUNCHED();
    fp::k_bias_grad<<<cout, 256, 0, static_cast<cudaStream_t>(stream)>>>(
        static_cast<const __nv_bfloat16*>(dy_bf16), (long long)total, cout, db);
    return cudaGetLastError() == cudaSuccess ? FP_OK : FP_ERR_CUDA;
}

extern "C" int fp_nn_relu_back(const float* dpost, const void* post_bf16, int64_t total, int c,
                               int cpad, void* out_bf16, void* stream) {
    if (!dpost || !out_bf16 || total <= 0 || c <= 0 || cpad < c) return FP_ERR_INVALID;
    FP_LAUNCHED();
    fp::k_relu_back<<<fp::grid_for((long long)total * cpad, 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(
        dpost, static_cast<const __nv_bfloat16*>(post_bf16), (long long)total, c, cpad,
        static_cast<__nv_bfloat16*>(out_bf16));
    return cudaGetLastError() == cudaSuccess ? FP_OK : FP_ERR_CUDA;
}

// One Adam step (bias-corrected with c1 = 1 - b1^t, c2 = 1 - b2^t).  For a
// weight tensor (cout, cin > 0) also writes the BF16 forward and transposed
// copies; for a bias pass cout = cin = 0 and null copies.
extern "C" int fp_nn_adam(float* w, float* m1, float* m2, const float* g, int64_t count, float lr,
                          float b1, float b2, float eps, float c1, float c2, int cout, int cin,
                          void* wf_bf16, void* wt_bf16, void* stream) {
    if (!w || !m1 || !m2 || !g || count <= 0) return FP_ERR_INVALID;
    if ((wf_bf16 != nullptr) != (wt_bf16 != nullptr)) return FP_ERR_INVALID;
    if (wf_bf16 && (long long)count != 27LL * cout * cin) return FP_ERR_INVALID;
    FP_LAUNCHED();
    fp::k_adam<<<fp::grid_for((long long)count, 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(
        w, m1, m2, g, (long long)count, lr, b1, b2, eps, c1, c2, cout, cin,
        static_cast<__nv_bfloat16*>(wf_bf16), static_cast<__nv_bfloat16*>(wt_bf16));
    return cudaGetLastError() == cudaSuccess ? FP_OK : FP_ERR_CUDA;
}

// Loss of a batch of `samples` predictions (FP32 [samples*n][cstride],
// channels 0..2 used) against mean-free targets (FP32 [samples*n][3], zero
// off the support): per-sample relative squared error into loss[samples]
// and its gradient into dpred (same layout as pred).  stats: scratch of
// 4*samples floats; tnorm[b] = sum |t|^2 of sample b.
extern "C" int fp_nn_loss(const float* pred, int cstride, const float* tgt, const uint8_t* support,
                          int64_t n, int samples, const float* tnorm, float* stats, float* dpred,
                          float* loss, void* stream) {
    if (!pred || !tgt || !support || !tnorm || !stats || !dpred || !loss || n <= 0 || samples <= 0 ||
        cstride < 3)
        return FP_ERR_INVALID;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    FP_LAUNCHED();
    fp::k_loss_stats<<<samples, 256, 0, s>>>(pred, cstride, support, (long long)n, stats);
    FP_LAUNCHED();
    fp::k_loss_grad<<<samples, 256, 0, s>>>(pred, cstride, tgt, support, (long long)n, stats, tnorm, dpred,
                                            loss);
    return cudaGetLastError() == cudaSuccess ? FP_OK : FP_ERR_CUDA;
}

