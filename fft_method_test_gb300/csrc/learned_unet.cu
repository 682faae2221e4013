// learned_unet.cu -- the multi-level pieces of the warm-start U-Net: 2x
// average pooling, nearest 2x up-sampling with the skip connection added, their
// gradients, and the weight gradient of convolutions whose channel counts the
// tensor-core weight-gradient kernel (learned.cu) does not cover.  No
// counterpart in the reference.
//
// Channels-last tensors [voxel][channel], samples stacked, x fastest.  The
// coarse grid of a fine grid (nx, ny, nz) is (nx/2, ny/2, nz/2); the parent of
// fine voxel (x, y, z) is (x/2, y/2, z/2).
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/fftperm.h"
#include "common.cuh"

namespace fp {
namespace {

int grid_of(long long m, int threads) {
    long long b = (m + threads - 1) / threads;
    if (b > 65535LL * 16) b = 65535LL * 16;
    return (int)(b < 1 ? 1 : b);
}

struct Geo2 {
    int nx, ny, nz;    // fine grid
    long long nf, nc;  // voxels per sample, fine and coarse
};

__device__ __forceinline__ long long parent_of(const Geo2& g, long long v) {
    const long long b = v / g.nf;
    const long long r = v - b * g.nf;
    const int x = (int)(r % g.nx);
    const long long q = r / g.nx;
    const int y = (int)(q % g.ny);
    const int z = (int)(q / g.ny);
    return b * g.nc + ((long long)(z >> 1) * (g.ny >> 1) + (y >> 1)) * (g.nx >> 1) + (x >> 1);
}

// coarse[p][c] = mean of the 8 fine children
__global__ void k_pool2(Geo2 g, long long coarse_total, int c, const __nv_bfloat16* __restrict__ in,
                        __nv_bfloat16* __restrict__ out) {
    const int cx = g.nx >> 1, cy = g.ny >> 1;
    for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < coarse_total * c;
         e += (long long)gridDim.x * blockDim.x) {
        const long long p = e / c;
        const int ch = (int)(e - p * c);
        const long long b = p / g.nc;
        const long long r = p - b * g.nc;
        const int x = (int)(r % cx);
        const long long q = r / cx;
        const int y = (int)(q % cy);
        const int z = (int)(q / cy);
        float s = 0.f;
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const long long f = b * g.nf +
                                ((long long)(2 * z + (k >> 2)) * g.ny + 2 * y + ((k >> 1) & 1)) * g.nx +
                                2 * x + (k & 1);
            s += __bfloat162float(in[f * c + ch]);
        }
        out[e] = __float2bfloat16(0.125f * s);
    }
}

// dfine[v][c] += dcoarse[parent(v)][c] / 8
__global__ void k_pool2_back(Geo2 g, long long fine_total, int c, const float* __restrict__ dcoarse,
                             float* __restrict__ dfine) {
    for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < fine_total * c;
         e += (long long)gridDim.x * blockDim.x) {
        const long long v = e / c;
        const int ch = (int)(e - v * c);
        dfine[e] += 0.125f * dcoarse[parent_of(g, v) * c + ch];
    }
}

// out[v][c] = act(coarse[parent(v)][c] + skip[v][c]), act = ReLU when relu
__global__ void k_up2_add(Geo2 g, long long fine_total, int c, const __nv_bfloat16* __restrict__ coarse,
                          const __nv_bfloat16* __restrict__ skip, int relu,
                          __nv_bfloat16* __restrict__ out) {
    for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < fine_total * c;
         e += (long long)gridDim.x * blockDim.x) {
        const long long v = e / c;
        const int ch = (int)(e - v * c);
        float s = __bfloat162float(coarse[parent_of(g, v) * c + ch]) + __bfloat162float(skip[e]);
        if (relu) s = fmaxf(s, 0.f);
        out[e] = __float2bfloat16(s);
    }
}

// With d = dout masked by ReLU (post > 0): dskip[v] = d[v], and
// dcoarse[p] = sum of d over the 8 children of p (fixed order).
__global__ void k_up2_add_back(Geo2 g, long long coarse_total, int c, const float* __restrict__ dout,
                               const __nv_bfloat16* __restrict__ post, float* __restrict__ dskip,
                               float* __restrict__ dcoarse) {
    const int cx = g.nx >> 1, cy = g.ny >> 1;
    for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < coarse_total * c;
         e += (long long)gridDim.x * blockDim.x) {
        const long long p = e / c;
        const int ch = (int)(e - p * c);
        const long long b = p / g.nc;
        const long long r = p - b * g.nc;
        const int x = (int)(r % cx);
        const long long q = r / cx;
        const int y = (int)(q % cy);
        const int z = (int)(q / cy);
        float s = 0.f;
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const long long f = b * g.nf +
                                ((long long)(2 * z + (k >> 2)) * g.ny + 2 * y + ((k >> 1) & 1)) * g.nx +
                                2 * x + (k & 1);
            float d = dout[f * c + ch];
            if (post && !(__bfloat162float(post[f * c + ch]) > 0.f)) d = 0.f;
            dskip[f * c + ch] = d;
            s += d;
        }
        dcoarse[e] = s;
    }
}

// Weight-gradient partials on the CUDA cores for any channel counts (multiples
// of 16): CTA (chunk, tap, 16 x 16 tile of (o, i)) sums dy[v][o] x[v + off][i]
// over its voxel chunk, 16 voxels at a time through shared memory.
// partial[chunk][tap][cout][cin].
__global__ void __launch_bounds__(256) k_wgrad_cc(int nx, int ny, int nz, long long n, long long total,
                                                  int dil, const __nv_bfloat16* __restrict__ dy,
                                                  int cout, const __nv_bfloat16* __restrict__ x,
                                                  int cin, long long chunk,
                                                  float* __restrict__ partial) {
    __shared__ float sdy[16][17];
    __shared__ float sx[16][17];
    const int tap = blockIdx.y;
    const long long ck = blockIdx.x;
    const int tiles_i = cin / 16;
    const int o0 = (blockIdx.z / tiles_i) * 16;
    const int i0 = (blockIdx.z % tiles_i) * 16;
    const int to = threadIdx.x >> 4, ti = threadIdx.x & 15;
    const int dz = tap / 9 - 1, dyy = (tap / 3) % 3 - 1, dx = tap % 3 - 1;
    const long long vb = ck * chunk, ve = min(total, vb + chunk);
    float acc = 0.f;
    for (long long k0 = vb; k0 < ve; k0 += 16) {
        // thread (to, ti): loads dy[k0 + to][o0 + ti] and x[nb(k0 + to)][i0 + ti]
        const long long v = k0 + to;
        float a = 0.f, bx = 0.f;
        if (v < ve) {
            a = __bfloat162float(dy[v * cout + o0 + ti]);
            const long long smp = v / n;
            const long long r = v - smp * n;
            int xx = (int)(r % nx);
            const long long q = r / nx;
            int yy = (int)(q % ny), zz = (int)(q / ny);
            xx = ((xx + dil * dx) % nx + nx) % nx;
            yy = ((yy + dil * dyy) % ny + ny) % ny;
            zz = ((zz + dil * dz) % nz + nz) % nz;
            const long long nb = smp * n + ((long long)zz * ny + yy) * nx + xx;
            bx = __bfloat162float(x[nb * cin + i0 + ti]);
        }
        sdy[to][ti] = a;
        sx[to][ti] = bx;
        __syncthreads();
#pragma unroll
        for (int j = 0; j < 16; ++j) acc += sdy[j][to] * sx[j][ti];
        __syncthreads();
    }
    partial[((ck * 27 + tap) * (long long)cout + o0 + to) * cin + i0 + ti] = acc;
}

__global__ void k_wgrad_cc_reduce(const float* __restrict__ partial, long long nchunks, int cout, int cin,
                                  float* __restrict__ dw) {
    const long long m = 27LL * cout * cin;
    for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < m;
         e += (long long)gridDim.x * blockDim.x) {
        float s = 0.f;
        for (long long c = 0; c < nchunks; ++c) s += partial[c * m + e];
        dw[e] = s;
    }
}

bool geo2(int nx, int ny, int nz, Geo2* g) {
    if (nx < 2 || ny < 2 || nz < 2 || (nx | ny | nz) & 1) return false;
    g->nx = nx;
    g->ny = ny;
    g->nz = nz;
    g->nf = (long long)nx * ny * nz;
    g->nc = g->nf / 8;
    return true;
}

}  // namespace
}  // namespace fp

extern "C" int fp_nn_pool2(int nx, int ny, int nz, int samples, int c, const void* in_bf16,
                           void* out_bf16, void* stream) {
    fp::Geo2 g;
    if (!fp::geo2(nx, ny, nz, &g) || samples <= 0 || c <= 0 || !in_bf16 || !out_bf16)
        return FP_ERR_INVALID;
    const long long ct = g.nc * samples;
    FP_LAUNCHED();
    fp::k_pool2<<<fp::grid_of(ct * c, 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(
        g, ct, c, static_cast<const __nv_bfloat16*>(in_bf16), static_cast<__nv_bfloat16*>(out_bf16));
    return cudaGetLastError() == cudaSuccess ? FP_OK : FP_ERR_CUDA;
}

extern "C" int fp_nn_pool2_back(int nx, int ny, int nz, int samples, int c, const float* dcoarse,
                                float* dfine, void* stream) {
    fp::Geo2 g;
    if (!fp::geo2(nx, ny, nz, &g) || samples <= 0 || c <= 0 || !dcoarse || !dfine)
        return FP_ERR_INVALID;
    const long long ft = g.nf * samples;
    FP_LAUNCHED();
    fp::k_pool2_back<<<fp::grid_of(ft * c, 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(
        g, ft, c, dcoarse, dfine);
    return cudaGetLastError() == cudaSuccess ? FP_OK : FP_ERR_CUDA;
}

extern "C" int fp_nn_up2_add(int nx, int ny, int nz, int samples, int c, const void* coarse_bf16,
                             const void* skip_bf16, int relu, void* out_bf16, void* stream) {
    fp::Geo2 g;
    if (!fp::geo2(nx, ny, nz, &g) || samples <= 0 || c <= 0 || !coarse_bf16 || !skip_bf16 || !out_bf16)
        return FP_ERR_INVALID;
    const long long ft = g.nf * samples;
    FP_LAUNCHED();
    fp::k_up2_add<<<fp::grid_of(ft * c, 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(
        g, ft, c, static_cast<const __nv_bfloat16*>(coarse_bf16),
        static_cast<const __nv_bfloat16*>(skip_bf16), relu, static_cast<__nv_bfloat16*>(out_bf16));
    return cudaGetLastError() == cudaSuccess ? FP_OK : FP_ERR_CUDA;
}

extern "C" int fp_nn_up2_add_back(int nx, int ny, int nz, int samples, int c, const float* dout,
                                  const void* post_bf16, float* dskip, float* dcoarse, void* stream) {
    fp::Geo2 g;
    if (!fp::geo2(nx, ny, nz, &g) || samples <= 0 || c <= 0 || !dout || !dskip || !dcoarse)
        return FP_ERR_INVALID;
    const long long ct = g.nc * samples;
    FP_LAUNCHED();
    fp::k_up2_add_back<<<fp::grid_of(ct * c, 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(
        g, ct, c, dout, static_cast<const __nv_bfloat16*>(post_bf16), dskip, dcoarse);
    return cudaGetLastError() == cudaSuccess ? FP_OK : FP_ERR_CUDA;
}

extern "C" int fp_nn_wgrad_cc(int nx, int ny, int nz, int64_t total, int dilation, const void* dy_bf16,
                              int cout, const void* x_bf16, int cin, int64_t chunk, float* partial,
                              float* dw, void* stream) {
    if (nx <= 0 || ny <= 0 || nz <= 0 || total <= 0 || chunk <= 0 || cout % 16 || cin % 16 ||
        cout <= 0 || cin <= 0 || !dy_bf16 || !x_bf16 || !partial || !dw)
        return FP_ERR_INVALID;
    const long long n = (long long)nx * ny * nz;
    if (total % n) return FP_ERR_INVALID;
    const long long nchunks = (total + chunk - 1) / chunk;
    if (nchunks > 65535) return FP_ERR_INVALID;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const dim3 grid((unsigned)nchunks, 27, (unsigned)((cout / 16) * (cin / 16)));
    FP_LAUNCHED();
    fp::k_wgrad_cc<<<grid, 256, 0, s>>>(nx, ny, nz, n, (long long)total, dilation,
                                        static_cast<const __nv_bfloat16*>(dy_bf16), cout,
                                        static_cast<const __nv_bfloat16*>(x_bf16), cin, (long long)chunk,
                                        partial);
    FP_LAUNCHED();
    fp::k_wgrad_cc_reduce<<<fp::grid_of(27LL * cout * cin, 256), 256, 0, s>>>(partial, nchunks, cout,
                                                                              cin, dw);
    return cudaGetLastError() == cudaSuccess ? FP_OK : FP_ERR_CUDA;
}
