// fft_passes.cuh -- the kernels of the five apply passes and their launch
// runners.  The kernels are templates on the precision; each runner family is
// compiled in its own translation unit per precision (fft_x*, fft_y*, fft_z*,
// fft_ztma*, selected by FP_DEFINE_{X,Y,Z,ZTMA}_RUNNERS), so the heavy
// unrolled FFT code builds in parallel.  kernels_fft.cu (plans,
// tiling, TMA descriptors, the pass sequence) sees only the declarations.
//
//   P1 forward x (R2C, two real lines per complex FFT) fused with the
//      scatter of the compact support vector (and/or the background force)
//   P2 forward y
//   P3 forward z, Green multiply (3x3 real symmetric), inverse z
//   P4 inverse y
//   P5 inverse x (C2R) fused with the gather to the support, the 1/N scale
//      and per-CTA partial sums used for mean removal and MINRES dots.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

#include "common.cuh"
#include "fft_engine.cuh"
#include "internal.h"
#include "tma.cuh"

namespace fp {

// ---------------------------------------------------------------------------
// kernel argument blocks
// ---------------------------------------------------------------------------

struct XArgs {
    int nx, ny, nz, nxh;
    int ld;        // padded shared-memory line stride
    long long rs;  // row stride of the spectral field (complex elements)
    long long n, nh, nrows;
    int rows_per_cta;
    FftPlanDev plan;
    const int* support;
    const int* row_ptr;
    const uint8_t* mask;
    const double* src;
    const double* src_sum;  // component sums of the compact source (3) or null
    double inv_nb;
    double f0_fluid[3];
    double f0_support[3];
    double* dst;
    const double* dot_with;
    double scale;  // 1/N for the inverse pass
    double* partials;
    void* spec;
    const int* skip;
    int* err;  // bulk-copy pipeline: a bounded wait gave up
};

struct YArgs {
    int ny, nxh, tx, ld, nz;
    long long nh, rs;
    FftPlanDev plan;
    void* spec;
    const int* skip;
    int* err;
};

struct ZArgs {
    int ny, nz, nxh, tz, ld;
    long long nh, rs, plane, gstride;
    FftPlanDev plan;
    const void* green;
    void* spec;
    const int* skip;
    int* err;
};

// Tiling of a persistent TMA-fed pass.
struct TmaTile {
    int ntiles;    // tiles in the pass
    int ntx;       // kx tiles per line of tiles
    int t;         // kx columns per tile
    int nbox;      // TMA boxes along the transform axis
    int box;       // rows per box
    int np;        // component stride of the raw tile in rows: >= nbox * box, padded so
                   // that every component block starts 128-byte aligned
    int bufbytes;  // bytes of one tile buffer (raw tile or padded lines, larger of the two)
    int ld;        // line stride of the padded lines (column_line_stride for t)
};

// ---------------------------------------------------------------------------
// P1: forward x with fused source construction
// ---------------------------------------------------------------------------

template <typename T, int SRC>
__global__ void __launch_bounds__(256, 3) k_xfwd(XArgs a) {
    if (a.skip && *a.skip) return;
    using T2 = c_t<T>;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    T2* lines = reinterpret_cast<T2*>(smem_raw);
    const int nx = a.nx;
    const int ld = a.ld;
    const long long r0 = (long long)blockIdx.x * a.rows_per_cta;
    const int rows = (int)min((long long)a.rows_per_cta, a.nrows - r0);
    const int nreal = 3 * rows;
    const int nq = (nreal + 1) / 2;
    T2* spec = reinterpret_cast<T2*>(a.spec);

    // 1) fill the real lines: real line L = 3*row_local + comp is the real
    //    (L even) or imaginary (L odd) part of complex line L/2.
    const int total = nq * nx;
    for (int t = threadIdx.x; t < total; t += blockDim.x) {
        const int q = t / nx;
        const int x = t - q * nx;
        T vr = 0, vi = 0;
        if (SRC == kSrcDense || SRC == kSrcF0 || SRC == kSrcF0Compact) {
#pragma unroll
            for (int part = 0; part < 2; ++part) {
                const int L = 2 * q + part;
                if (L < nreal) {
                    const int rl = L / 3;
                    const int c = L - 3 * rl;
                    const long long idx = (r0 + rl) * nx + x;
                    double val;
                    if (SRC == kSrcDense) {
                        val = a.src[c * a.n + idx];
                    } else {
                        val = a.mask[idx] ? a.f0_fluid[c] : 0.0;
                    }
                    if (part == 0) vr = (T)val; else vi = (T)val;
                }
            }
        }
        lines[q * ld + pidx<T2>(x)] = cmk<T2>(vr, vi);
    }
    __syncthreads();

    // 2) scatter the compact vector (support voxels are solid: no overlap
    //    with the fluid part of f0).
    if (SRC == kSrcCompact || SRC == kSrcF0 || SRC == kSrcF0Compact) {
        double mean[3] = {0.0, 0.0, 0.0};
        if (SRC != kSrcF0 && a.src_sum) {
            mean[0] = a.src_sum[0] * a.inv_nb;
            mean[1] = a.src_sum[1] * a.inv_nb;
            mean[2] = a.src_sum[2] * a.inv_nb;
        }
        const int s0 = a.row_ptr[r0];
        const int s1 = a.row_ptr[r0 + rows];
        constexpr int U = 4;  // support entries in flight per thread
        for (int sb = s0 + threadIdx.x; sb < s1; sb += U * blockDim.x) {
            int sidx[U];
            double cv[U][3];
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const int s = sb + u * blockDim.x;
                sidx[u] = -1;
#pragma unroll
                for (int c = 0; c < 3; ++c) cv[u][c] = 0.0;
                if (s < s1) {
                    sidx[u] = a.support[s];
                    if (SRC != kSrcF0)
#pragma unroll
                        for (int c = 0; c < 3; ++c) cv[u][c] = a.src[3LL * s + c];
                }
            }
#pragma unroll
            for (int u = 0; u < U; ++u) {
                if (sidx[u] < 0) continue;
                const long long idx = sidx[u];
                const int rl = (int)(idx / nx - r0);
                const int x = (int)(idx - (r0 + rl) * nx);
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    // in the FP32 apply the value is rounded to FP32 anyway:
                    // form it in FP32 (GB300's FP64 pipe is narrow)
                    T val = (T)0;
                    if (SRC != kSrcF0) val = (T)cv[u][c] - (T)mean[c];
                    if (SRC != kSrcCompact) val += (T)a.f0_support[c];
                    const int L = 3 * rl + c;
                    T2* p = &lines[(L >> 1) * ld + pidx<T2>(x)];
                    if (L & 1) p->y = (T)val; else p->x = (T)val;
                }
            }
        }
        __syncthreads();
    }

    // 3) forward FFT of every complex line (shared memory in and out)
    {
        const int tpl = plan_tpl<T2>(a.plan);
        const int q = threadIdx.x / tpl;
        const int lane = threadIdx.x - q * tpl;
        T2* my = lines + (q < nq ? q : 0) * ld;
        fft_lines<-1, kIoSmem, kIoSmem, 1>(&my, a.plan, lane, q < nq, false, NoSrc<T2>{},
                                            NoDst<T2>{});
    }

    // 4) separate the two real spectra and store the half spectrum
    const int nxh = a.nxh;
    const int tot2 = nq * nxh;
    for (int t = threadIdx.x; t < tot2; t += blockDim.x) {
        const int q = t / nxh;
        const int k = t - q * nxh;
        const T2 zk = lines[q * ld + pidx<T2>(k)];
        const int kn = (k == 0) ? 0 : nx - k;
        const T2 zn = lines[q * ld + pidx<T2>(kn)];
        const T2 A = cmk<T2>((T)0.5 * (zk.x + zn.x), (T)0.5 * (zk.y - zn.y));
        const T2 B = cmk<T2>((T)0.5 * (zk.y + zn.y), (T)0.5 * (zn.x - zk.x));
        {
            const int L = 2 * q;
            const int rl = L / 3;
            const int c = L - 3 * rl;
            spec[c * a.nh + (r0 + rl) * a.rs + k] = A;
        }
        const int L = 2 * q + 1;
        if (L < nreal) {
            const int rl = L / 3;
            const int c = L - 3 * rl;
            spec[c * a.nh + (r0 + rl) * a.rs + k] = B;
        }
    }
}

// ---------------------------------------------------------------------------
// P2 / P4: y pass (one z plane, a tile of kx columns, all three components
// per thread; the first stage reads HBM, the last stage writes HBM)
// ---------------------------------------------------------------------------

template <typename T2>
struct ColIo {
    T2* base;          // element (comp 0, y 0) of this thread's column
    long long cstride; // component block stride
    long long estride; // stride between successive elements of the line
    __device__ __forceinline__ T2 operator()(int l, int i) const {
        return base[l * cstride + (long long)i * estride];
    }
    __device__ __forceinline__ void operator()(int l, int i, T2 v) const {
        base[l * cstride + (long long)i * estride] = v;
    }
};

template <typename T, int S>
__device__ __forceinline__ void ypass_body(const YArgs& a) {
    if (a.skip && *a.skip) return;
    using T2 = c_t<T>;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    T2* lines = reinterpret_cast<T2*>(smem_raw);
    const int tx = a.tx;
    const int k0 = blockIdx.x * tx;
    const int c = threadIdx.x % tx;
    const int lane = threadIdx.x / tx;
    const bool active = (k0 + c) < a.nxh;
    const long long z = blockIdx.y;
    ColIo<T2> io;
    io.base = reinterpret_cast<T2*>(a.spec) + z * (long long)a.ny * a.rs + k0 + (active ? c : 0);
    io.cstride = a.nh;
    io.estride = a.rs;
    T2* sl[3];
#pragma unroll
    for (int l = 0; l < 3; ++l) sl[l] = lines + (l * tx + c) * a.ld;
    fft_lines<S, kIoFunc, kIoFunc, 3>(sl, a.plan, lane, active, S > 0, io, io);
}

template <typename T, int S>
__global__ void __launch_bounds__(256) k_ypass(YArgs a) {
    ypass_body<T, S>(a);
}

// The same pass capped at 168 registers: 12 instead of 8 warps of 128-thread
// CTAs per SM, at the price of a few hundred bytes of spills per thread.
// The autotuner chooses between the two.
template <typename T, int S>
__global__ void __maxnreg__(168) k_ypass_lr(YArgs a) {
    ypass_body<T, S>(a);
}

// ---------------------------------------------------------------------------
// P3: z forward, Green multiply in registers, z inverse (one ky, a tile of
// kx columns, three components per thread).  The inverse runs the radices in
// reverse order, so its first stage consumes exactly the elements the
// forward's last stage left in this thread's registers.
// ---------------------------------------------------------------------------

template <int RL, typename T, int IN0, class Src, class Dst>
__device__ __forceinline__ void z_fused(const ZArgs& a, c_t<T>* const* sl, Src& src, Dst& dst,
                                        long long gbase, int lane, bool active) {
    using T2 = c_t<T>;
    const FftPlanDev& p = a.plan;
    const T2* tw = plan_tw<T2>(p);
    const int nst = plan_nstage<T2>(p);
    const int tpl = plan_tpl<T2>(p);
    const int n = p.n;
    NoSrc<T2> nsrc;
    NoDst<T2> ndst;
    // forward stages but the last
    int ns = 1;
    for (int s = 0; s < nst - 1; ++s) {
        const int R = plan_radix<T2>(p, s);
        if (s == 0)
            fft_stage_rt<-1, IN0, kIoSmem, 3>(R, sl, n, ns, lane, tpl, active, tw, src, ndst);
        else
            fft_stage_rt<-1, kIoSmem, kIoSmem, 3>(R, sl, n, ns, lane, tpl, active, tw, nsrc, ndst);
        ns *= R;
    }
    // last forward stage into registers
    constexpr int KM = StageRegs<T2, RL>::KM;
    T2 v[3][KM][RL];
    zero_regs(v);
    if (nst == 1)
        stage_load<RL, kIoFunc, 3>(v, sl, n, lane, tpl, active, src);
    else
        stage_load<RL, kIoSmem, 3>(v, sl, n, lane, tpl, active, nsrc);
    stage_compute<RL, -1, 3>(v, n, ns, lane, tpl, active, tw);
    // Green multiply: output r of butterfly j is kz = j + r * (n / RL)
    const int m = n / RL;
    if (active) {
        const T* g = reinterpret_cast<const T*>(a.green);
#pragma unroll
        for (int kk = 0; kk < KM; ++kk) {
            const int j = lane + kk * tpl;
            if (j < m) {
#pragma unroll
                for (int r = 0; r < RL; ++r) {
                    const long long gi = (long long)(j + r * m) * a.plane + gbase;
                    const T gxx = g[gi], gxy = g[a.gstride + gi], gxz = g[2 * a.gstride + gi];
                    const T gyy = g[3 * a.gstride + gi], gyz = g[4 * a.gstride + gi];
                    const T gzz = g[5 * a.gstride + gi];
                    const int o = out_slot<RL>(r);
                    const T2 ax = v[0][kk][o], ay = v[1][kk][o], az = v[2][kk][o];
                    v[0][kk][o] = cmk<T2>(gxx * ax.x + gxy * ay.x + gxz * az.x, gxx * ax.y + gxy * ay.y + gxz * az.y);
                    v[1][kk][o] = cmk<T2>(gxy * ax.x + gyy * ay.x + gyz * az.x, gxy * ax.y + gyy * ay.y + gyz * az.y);
                    v[2][kk][o] = cmk<T2>(gxz * ax.x + gyz * ay.x + gzz * az.x, gxz * ax.y + gyz * ay.y + gzz * az.y);
                }
            }
        }
    }
    // first inverse stage (radix RL, Ns = 1: no twiddles) on the same registers
    T2 u[3][KM][RL];
    zero_regs(u);
#pragma unroll
    for (int l = 0; l < 3; ++l)
#pragma unroll
        for (int kk = 0; kk < KM; ++kk)
#pragma unroll
            for (int r = 0; r < RL; ++r) u[l][kk][r] = v[l][kk][out_slot<RL>(r)];
    stage_compute<RL, +1, 3>(u, n, 1, lane, tpl, active, tw);
    if (nst == 1) {
        stage_store<RL, kIoFunc, 3>(u, sl, n, 1, lane, tpl, active, dst);
        return;
    }
    __syncthreads();  // every thread has read its last forward inputs
    stage_store<RL, kIoSmem, 3>(u, sl, n, 1, lane, tpl, active, ndst);
    __syncthreads();
    ns = RL;
    for (int s = 1; s < nst; ++s) {
        const int R = plan_radix<T2>(p, nst - 1 - s);
        if (s == nst - 1)
            fft_stage_rt<+1, kIoSmem, kIoFunc, 3>(R, sl, n, ns, lane, tpl, active, tw, nsrc, dst);
        else
            fft_stage_rt<+1, kIoSmem, kIoSmem, 3>(R, sl, n, ns, lane, tpl, active, tw, nsrc, ndst);
        ns *= R;
    }
}

template <typename T, int IN0, class Src, class Dst>
__device__ __forceinline__ void z_fused_rt(const ZArgs& a, c_t<T>* const* sl, Src& src, Dst& dst,
                                           long long gbase, int lane, bool active) {
    using T2 = c_t<T>;
    const int nst = plan_nstage<T2>(a.plan);
    switch (plan_radix<T2>(a.plan, nst - 1)) {
        case 16:
            if constexpr (sizeof(T) == 4) z_fused<16, T, IN0>(a, sl, src, dst, gbase, lane, active);
            break;
        case 8: z_fused<8, T, IN0>(a, sl, src, dst, gbase, lane, active); break;
        case 4: z_fused<4, T, IN0>(a, sl, src, dst, gbase, lane, active); break;
        case 2: z_fused<2, T, IN0>(a, sl, src, dst, gbase, lane, active); break;
        case 3: z_fused<3, T, IN0>(a, sl, src, dst, gbase, lane, active); break;
        default: z_fused<5, T, IN0>(a, sl, src, dst, gbase, lane, active); break;
    }
}

// ZMODE: 0 = forward z, Green multiply, inverse z; 1 = forward z only;
// 2 = inverse z only
template <typename T, int ZMODE>
__device__ __forceinline__ void zgreen_body(const ZArgs& a) {
    if (a.skip && *a.skip) return;
    using T2 = c_t<T>;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    T2* lines = reinterpret_cast<T2*>(smem_raw);
    const int tz = a.tz;
    const int k0 = blockIdx.x * tz;
    const int c = threadIdx.x % tz;
    const int lane = threadIdx.x / tz;
    const bool active = (k0 + c) < a.nxh;
    ColIo<T2> io;
    io.base = reinterpret_cast<T2*>(a.spec) + (long long)blockIdx.y * a.rs + k0 + (active ? c : 0);
    io.cstride = a.nh;
    io.estride = a.plane;
    T2* sl[3];
#pragma unroll
    for (int l = 0; l < 3; ++l) sl[l] = lines + (l * tz + c) * a.ld;
    if (ZMODE == 1) {
        fft_lines<-1, kIoFunc, kIoFunc, 3>(sl, a.plan, lane, active, false, io, io);
    } else if (ZMODE == 2) {
        fft_lines<+1, kIoFunc, kIoFunc, 3>(sl, a.plan, lane, active, false, io, io);
    } else {
        const int nst = plan_nstage<T2>(a.plan);
        if (nst == 0) {  // nz == 1: the z transforms are identities
            if (active && lane == 0) {
                const T* g = reinterpret_cast<const T*>(a.green);
                const long long gi = (long long)blockIdx.y * a.rs + k0 + c;
                const T gxx = g[gi], gxy = g[a.gstride + gi], gxz = g[2 * a.gstride + gi];
                const T gyy = g[3 * a.gstride + gi], gyz = g[4 * a.gstride + gi];
                const T gzz = g[5 * a.gstride + gi];
                const T2 ax = io(0, 0), ay = io(1, 0), az = io(2, 0);
                io(0, 0, cmk<T2>(gxx * ax.x + gxy * ay.x + gxz * az.x, gxx * ax.y + gxy * ay.y + gxz * az.y));
                io(1, 0, cmk<T2>(gxy * ax.x + gyy * ay.x + gyz * az.x, gxy * ax.y + gyy * ay.y + gyz * az.y));
                io(2, 0, cmk<T2>(gxz * ax.x + gyz * ay.x + gzz * az.x, gxz * ax.y + gyz * ay.y + gzz * az.y));
            }
            return;
        }
        z_fused_rt<T, kIoFunc>(a, sl, io, io, (long long)blockIdx.y * a.rs + k0 + c, lane, active);
    }
}

template <typename T, int ZMODE>
__global__ void __launch_bounds__(256) k_zgreen(ZArgs a) {
    zgreen_body<T, ZMODE>(a);
}

// capped at 168 registers (see k_ypass_lr)
template <typename T, int ZMODE>
__global__ void __maxnreg__(168) k_zgreen_lr(ZArgs a) {
    zgreen_body<T, ZMODE>(a);
}

// ---------------------------------------------------------------------------
// Persistent TMA-fed y and z passes.  One CTA per SM walks its tiles; two
// shared-memory buffers alternate so that the TMA loads of tile i+1 (three
// component boxes per tile, completion counted on an mbarrier) run while tile
// i is transformed.  Stage 0 reads the raw TMA tile, later stages exchange
// through padded lines in the same buffer, and the last stage writes HBM
// directly.  Waits are bounded: on a timeout the CTA raises the error flag,
// drains its own prefetch (bounded too) and returns.
// ---------------------------------------------------------------------------

template <typename T2>
struct RawIo {
    const T2* raw;
    int np, t, c;
    __device__ __forceinline__ T2 operator()(int l, int i) const {
        return raw[((long long)l * np + i) * t + c];
    }
};


template <typename T, int S>
__global__ void __launch_bounds__(256) k_ypass_tma(const __grid_constant__ CUtensorMap map, YArgs a,
                                                   TmaTile tt) {
    if (a.skip && *a.skip) return;
    using T2 = c_t<T>;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    uint64_t* bars = reinterpret_cast<uint64_t*>(smem_raw);
    unsigned char* buf0 = smem_raw + 128;
    const int t = tt.t;
    const int c = threadIdx.x % t;
    const int lane = threadIdx.x / t;
    const uint32_t tile_bytes = (uint32_t)(3 * tt.nbox * tt.box * t * sizeof(T2));
    if (threadIdx.x == 0) {
        mbar_init(&bars[0], 1);
        mbar_init(&bars[1], 1);
        fence_mbar_init();
    }
    __syncthreads();
    auto issue = [&](int tile, int b) {
        const int kx0 = (tile % tt.ntx) * t;
        const int z = tile / tt.ntx;
        T2* dst = reinterpret_cast<T2*>(buf0 + (size_t)b * tt.bufbytes);
        mbar_arrive_expect_tx(&bars[b], tile_bytes);
        for (int l = 0; l < 3; ++l)
            for (int yb = 0; yb < tt.nbox; ++yb)
                tma_load_4d(dst + ((size_t)l * tt.np + (size_t)yb * tt.box) * t, &map, 2 * kx0,
                            yb * tt.box, z, l, &bars[b]);
    };
    int tile = blockIdx.x;
    if (threadIdx.x == 0 && tile < tt.ntiles) issue(tile, 0);
    for (int i = 0; tile < tt.ntiles; tile += gridDim.x, ++i) {
        const int b = i & 1;
        const int nt = tile + gridDim.x;
        if (threadIdx.x == 0 && nt < tt.ntiles) {
            fence_proxy_async_smem();
            issue(nt, b ^ 1);
        }
        if (!tma_pipeline_wait<T2>(bars, i, b, nt < tt.ntiles, a.err)) return;
        const int kx0 = (tile % tt.ntx) * t;
        const long long z = tile / tt.ntx;
        const bool active = (kx0 + c) < a.nxh;
        T2* buf = reinterpret_cast<T2*>(buf0 + (size_t)b * tt.bufbytes);
        RawIo<T2> src{buf, tt.np, t, c};
        ColIo<T2> dst;
        dst.base = reinterpret_cast<T2*>(a.spec) + z * (long long)a.ny * a.rs + kx0 + (active ? c : 0);
        dst.cstride = a.nh;
        dst.estride = a.rs;
        T2* sl[3];
#pragma unroll
        for (int l = 0; l < 3; ++l) sl[l] = buf + (l * t + c) * a.ld;
        fft_lines<S, kIoFuncSmem, kIoFunc, 3>(sl, a.plan, lane, active, S > 0, src, dst);
        __syncthreads();  // the buffer is refilled by the prefetch of the next iteration
    }
}

template <typename T>
__global__ void __launch_bounds__(256) k_zgreen_tma(const __grid_constant__ CUtensorMap map, ZArgs a,
                                                    TmaTile tt) {
    if (a.skip && *a.skip) return;
    using T2 = c_t<T>;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    uint64_t* bars = reinterpret_cast<uint64_t*>(smem_raw);
    unsigned char* buf0 = smem_raw + 128;
    const int t = tt.t;
    const int c = threadIdx.x % t;
    const int lane = threadIdx.x / t;
    const uint32_t tile_bytes = (uint32_t)(3 * tt.nbox * tt.box * t * sizeof(T2));
    if (threadIdx.x == 0) {
        mbar_init(&bars[0], 1);
        mbar_init(&bars[1], 1);
        fence_mbar_init();
    }
    __syncthreads();
    auto issue = [&](int tile, int b) {
        const int kx0 = (tile % tt.ntx) * t;
        const int ky = tile / tt.ntx;
        T2* dst = reinterpret_cast<T2*>(buf0 + (size_t)b * tt.bufbytes);
        mbar_arrive_expect_tx(&bars[b], tile_bytes);
        for (int l = 0; l < 3; ++l)
            for (int zb = 0; zb < tt.nbox; ++zb)
                tma_load_4d(dst + ((size_t)l * tt.np + (size_t)zb * tt.box) * t, &map, 2 * kx0, ky,
                            zb * tt.box, l, &bars[b]);
    };
    int tile = blockIdx.x;
    if (threadIdx.x == 0 && tile < tt.ntiles) issue(tile, 0);
    for (int i = 0; tile < tt.ntiles; tile += gridDim.x, ++i) {
        const int b = i & 1;
        const int nt = tile + gridDim.x;
        if (threadIdx.x == 0 && nt < tt.ntiles) {
            fence_proxy_async_smem();
            issue(nt, b ^ 1);
        }
        if (!tma_pipeline_wait<T2>(bars, i, b, nt < tt.ntiles, a.err)) return;
        const int kx0 = (tile % tt.ntx) * t;
        const long long ky = tile / tt.ntx;
        const bool active = (kx0 + c) < a.nxh;
        T2* buf = reinterpret_cast<T2*>(buf0 + (size_t)b * tt.bufbytes);
        RawIo<T2> src{buf, tt.np, t, c};
        ColIo<T2> dst;
        dst.base = reinterpret_cast<T2*>(a.spec) + ky * a.rs + kx0 + (active ? c : 0);
        dst.cstride = a.nh;
        dst.estride = a.plane;
        T2* sl[3];
#pragma unroll
        for (int l = 0; l < 3; ++l) sl[l] = buf + (l * t + c) * a.ld;
        z_fused_rt<T, kIoFuncSmem>(a, sl, src, dst, ky * a.rs + kx0 + c, lane, active);
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// P5: inverse x with fused gather / dense store and partial sums
// ---------------------------------------------------------------------------

// One tile of rows [r0, r0 + rows): Hermitian reconstruction of the complex
// x-lines from the half spectra read through `load(c, row_local, k)`, the C2R
// transform, and the gather / dense store with partial sums into acc.
template <typename T, int DST, class Load>
__device__ __forceinline__ void xinv_tile(const XArgs& a, c_t<T>* lines, long long r0, int rows,
                                          const Load& load, double acc[4]) {
    using T2 = c_t<T>;
    const int nx = a.nx;
    const int nxh = a.nxh;
    const int ld = a.ld;
    const int nreal = 3 * rows;
    const int nq = (nreal + 1) / 2;
    const bool even = (nx % 2) == 0;

    // 1) Z = A + iB on the full line from the two Hermitian half spectra.
    //    Four (A, B) pairs are loaded per thread before any is used, so that
    //    eight independent loads are in flight per thread.
    const int tot = nq * nxh;
    constexpr int U = 4;
    for (int t0 = threadIdx.x; t0 < tot; t0 += U * blockDim.x) {
        T2 A[U], B[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int t = t0 + u * blockDim.x;
            A[u] = cmk<T2>((T)0, (T)0);
            B[u] = cmk<T2>((T)0, (T)0);
            if (t < tot) {
                const int q = t / nxh;
                const int k = t - q * nxh;
                const int La = 2 * q, rla = La / 3, ca = La - 3 * rla;
                A[u] = load(ca, rla, k);
                const int Lb = La + 1;
                if (Lb < nreal) {
                    const int rlb = Lb / 3, cb = Lb - 3 * rlb;
                    B[u] = load(cb, rlb, k);
                }
            }
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int t = t0 + u * blockDim.x;
            if (t < tot) {
                const int q = t / nxh;
                const int k = t - q * nxh;
                T2 Av = A[u], Bv = B[u];
                if (k == 0 || (even && 2 * k == nx)) {  // DC / Nyquist are real for a real line
                    Av.y = 0;
                    Bv.y = 0;
                }
                lines[q * ld + pidx<T2>(k)] = cmk<T2>(Av.x - Bv.y, Av.y + Bv.x);
                const int kn = nx - k;
                if (k > 0 && kn >= nxh) lines[q * ld + pidx<T2>(kn)] = cmk<T2>(Av.x + Bv.y, Bv.x - Av.y);
            }
        }
    }
    __syncthreads();
    {
        const int tpl = plan_tpl<T2>(a.plan);
        const int q = threadIdx.x / tpl;
        const int lane = threadIdx.x - q * tpl;
        T2* my = lines + (q < nq ? q : 0) * ld;
        fft_lines<+1, kIoSmem, kIoSmem, 1>(&my, a.plan, lane, q < nq, false, NoSrc<T2>{},
                                            NoDst<T2>{});
    }
    if (DST == kDstCompact) {
        const int s0 = a.row_ptr[r0];
        const int s1 = a.row_ptr[r0 + rows];
        for (int s = s0 + threadIdx.x; s < s1; s += blockDim.x) {
            const long long idx = a.support[s];
            const int rl = (int)(idx / nx - r0);
            const int x = (int)(idx - (r0 + rl) * nx);
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                const int L = 3 * rl + c;
                const T2 zv = lines[(L >> 1) * ld + pidx<T2>(x)];
                const double val = (double)(((L & 1) ? zv.y : zv.x) * (T)a.scale);
                a.dst[3LL * s + c] = val;
                acc[c] += val;
                if (a.dot_with) acc[3] += a.dot_with[3LL * s + c] * val;
            }
        }
    } else {
        const int total = nreal * nx;
        for (int t = threadIdx.x; t < total; t += blockDim.x) {
            const int L = t / nx;
            const int x = t - L * nx;
            const int rl = L / 3;
            const int c = L - 3 * rl;
            const T2 zv = lines[(L >> 1) * ld + pidx<T2>(x)];
            const double val = (double)(((L & 1) ? zv.y : zv.x) * (T)a.scale);
            a.dst[c * a.n + (r0 + rl) * nx + x] = val;
            acc[c] += val;
        }
    }
}

template <typename T2>
struct GlobalRows {
    const T2* spec;
    long long nh, rs, r0;
    __device__ __forceinline__ T2 operator()(int c, int rl, int k) const {
        return spec[c * nh + (r0 + rl) * rs + k];
    }
};

template <typename T2>
struct SmemRows {
    const T2* raw;  // [3][R][rs]
    int R;
    long long rs;
    __device__ __forceinline__ T2 operator()(int c, int rl, int k) const {
        return raw[((long long)c * R + rl) * rs + k];
    }
};

template <typename T, int DST>
__global__ void __launch_bounds__(256, 3) k_xinv(XArgs a) {
    if (a.skip && *a.skip) return;
    using T2 = c_t<T>;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    T2* lines = reinterpret_cast<T2*>(smem_raw);
    __shared__ double red[4 * 32];
    const long long r0 = (long long)blockIdx.x * a.rows_per_cta;
    const int rows = (int)min((long long)a.rows_per_cta, a.nrows - r0);
    double acc[4] = {0.0, 0.0, 0.0, 0.0};
    GlobalRows<T2> src{reinterpret_cast<const T2*>(a.spec), a.nh, a.rs, r0};
    xinv_tile<T, DST>(a, lines, r0, rows, src, acc);
    double out[4];
    block_sum<4>(acc, red, out);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int i = 0; i < 4; ++i) a.partials[4LL * blockIdx.x + i] = out[i];
    }
}

// Persistent variant: each CTA walks tiles of rows_per_cta rows; the three
// component blocks of tile i+1 (contiguous rows of the half spectrum) arrive
// by 1-D bulk copies into the second raw buffer while tile i is transformed.
// Partial sums are per CTA over all of its tiles (fixed tile order:
// deterministic).  smem: 128 B barriers | raw[2] | lines.
template <typename T, int DST>
__global__ void __launch_bounds__(256, 2) k_xinv_bulk(XArgs a, int raw_bytes) {
    if (a.skip && *a.skip) return;
    using T2 = c_t<T>;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    __shared__ double red[4 * 32];
    uint64_t* bars = reinterpret_cast<uint64_t*>(smem_raw);
    unsigned char* raw0 = smem_raw + 128;
    T2* lines = reinterpret_cast<T2*>(raw0 + 2 * (size_t)raw_bytes);
    const int R = a.rows_per_cta;
    const long long ntiles = (a.nrows + R - 1) / R;
    if (threadIdx.x == 0) {
        mbar_init(&bars[0], 1);
        mbar_init(&bars[1], 1);
        fence_mbar_init();
    }
    __syncthreads();
    const T2* spec = reinterpret_cast<const T2*>(a.spec);
    auto issue = [&](long long tile, int b) {
        const long long r0 = tile * R;
        const int rows = (int)min((long long)R, a.nrows - r0);
        const uint32_t bytes = (uint32_t)((long long)rows * a.rs * sizeof(T2));
        T2* dst = reinterpret_cast<T2*>(raw0 + (size_t)b * raw_bytes);
        mbar_arrive_expect_tx(&bars[b], 3 * bytes);
        for (int c = 0; c < 3; ++c)
            bulk_load(dst + (size_t)c * R * a.rs, spec + c * a.nh + r0 * a.rs, bytes, &bars[b]);
    };
    double acc[4] = {0.0, 0.0, 0.0, 0.0};
    long long tile = blockIdx.x;
    if (threadIdx.x == 0 && tile < ntiles) issue(tile, 0);
    for (int i = 0; tile < ntiles; tile += gridDim.x, ++i) {
        const int b = i & 1;
        const long long nt = tile + gridDim.x;
        if (threadIdx.x == 0 && nt < ntiles) {
            fence_proxy_async_smem();
            issue(nt, b ^ 1);
        }
        if (!tma_pipeline_wait<T2>(bars, i, b, nt < ntiles, a.err)) return;
        const long long r0 = tile * R;
        const int rows = (int)min((long long)R, a.nrows - r0);
        SmemRows<T2> src{reinterpret_cast<const T2*>(raw0 + (size_t)b * raw_bytes), R, a.rs};
        xinv_tile<T, DST>(a, lines, r0, rows, src, acc);
        __syncthreads();  // lines and raw[b] are rewritten by the next iterations
    }
    double out[4];
    block_sum<4>(acc, red, out);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int i = 0; i < 4; ++i) a.partials[4LL * blockIdx.x + i] = out[i];
    }
}

// ---------------------------------------------------------------------------
// launch runners (defined in the pass translation units)
// ---------------------------------------------------------------------------

template <typename T>
cudaError_t run_xfwd(int src_kind, const XArgs& x, int grid, int threads, size_t smem, cudaStream_t s);
template <typename T>
cudaError_t run_xinv(int dst_kind, const XArgs& x, int grid, int threads, size_t smem, cudaStream_t s);
template <typename T>
cudaError_t run_xinv_bulk(int dst_kind, const XArgs& x, int raw_bytes, int grid, int threads,
                          size_t smem, cudaStream_t s);
template <typename T>
cudaError_t run_ypass(int dir, const YArgs& y, dim3 grid, int threads, size_t smem, cudaStream_t s,
                      bool lowreg);
template <typename T>
cudaError_t run_ypass_tma(int dir, const CUtensorMap& map, const YArgs& y, const TmaTile& tt, int grid,
                          int threads, size_t smem, cudaStream_t s);
template <typename T>
cudaError_t run_zgreen(int mode, const ZArgs& z, dim3 grid, int threads, size_t smem, cudaStream_t s,
                       bool lowreg);
template <typename T>
cudaError_t run_zgreen_tma(const CUtensorMap& map, const ZArgs& z, const TmaTile& tt, int grid,
                           int threads, size_t smem, cudaStream_t s);

// The dynamic shared-memory limit is a per-kernel, process-wide attribute.
// Setting it to each launch's own size races between host threads that
// launch one kernel with different sizes (a batch of uneven grids): a launch
// can find the limit lowered under it.  So each kernel gets, once per device,
// the largest limit the device allows next to its static shared memory, and
// launches use what they need below it.
template <typename K>
inline void ensure_max_smem(K kern, std::atomic<unsigned long long>& done) {
    int dev = 0;
    cudaGetDevice(&dev);
    const unsigned long long bit = 1ull << (dev & 63);
    if (!(done.load(std::memory_order_acquire) & bit)) {
        int optin = 0;
        cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
        cudaFuncAttributes fa{};
        cudaFuncGetAttributes(&fa, kern);
        const int limit = optin - (int)fa.sharedSizeBytes;
        if (limit > 0) cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, limit);
        done.fetch_or(bit, std::memory_order_release);
    }
}

#define FP_RUN(kern, grid, threads, smem, s, ...)                 \
    do {                                                          \
        static std::atomic<unsigned long long> smem_set_{0};      \
        ensure_max_smem(kern, smem_set_);                         \
        FP_LAUNCHED();                                            \
        kern<<<grid, threads, smem, s>>>(__VA_ARGS__);            \
    } while (0)

#ifdef FP_DEFINE_X_RUNNERS
template <typename T>
cudaError_t run_xfwd(int src_kind, const XArgs& x, int grid, int threads, size_t smem, cudaStream_t s) {
    switch (src_kind) {
        case kSrcCompact: FP_RUN((k_xfwd<T, kSrcCompact>), grid, threads, smem, s, x); break;
        case kSrcDense: FP_RUN((k_xfwd<T, kSrcDense>), grid, threads, smem, s, x); break;
        case kSrcF0: FP_RUN((k_xfwd<T, kSrcF0>), grid, threads, smem, s, x); break;
        default: FP_RUN((k_xfwd<T, kSrcF0Compact>), grid, threads, smem, s, x); break;
    }
    return cudaGetLastError();
}
template <typename T>
cudaError_t run_xinv(int dst_kind, const XArgs& x, int grid, int threads, size_t smem, cudaStream_t s) {
    if (dst_kind == kDstCompact)
        FP_RUN((k_xinv<T, kDstCompact>), grid, threads, smem, s, x);
    else
        FP_RUN((k_xinv<T, kDstDense>), grid, threads, smem, s, x);
    return cudaGetLastError();
}
template <typename T>
cudaError_t run_xinv_bulk(int dst_kind, const XArgs& x, int raw_bytes, int grid, int threads,
                          size_t smem, cudaStream_t s) {
    if (dst_kind == kDstCompact)
        FP_RUN((k_xinv_bulk<T, kDstCompact>), grid, threads, smem, s, x, raw_bytes);
    else
        FP_RUN((k_xinv_bulk<T, kDstDense>), grid, threads, smem, s, x, raw_bytes);
    return cudaGetLastError();
}
#endif

#ifdef FP_DEFINE_Y_RUNNERS
template <typename T>
cudaError_t run_ypass(int dir, const YArgs& y, dim3 grid, int threads, size_t smem, cudaStream_t s,
                      bool lowreg) {
    if constexpr (sizeof(T) == 4) {
        if (lowreg) {
            if (dir < 0)
                FP_RUN((k_ypass_lr<T, -1>), grid, threads, smem, s, y);
            else
                FP_RUN((k_ypass_lr<T, +1>), grid, threads, smem, s, y);
            return cudaGetLastError();
        }
    }
    if (dir < 0)
        FP_RUN((k_ypass<T, -1>), grid, threads, smem, s, y);
    else
        FP_RUN((k_ypass<T, +1>), grid, threads, smem, s, y);
    return cudaGetLastError();
}
template <typename T>
cudaError_t run_ypass_tma(int dir, const CUtensorMap& map, const YArgs& y, const TmaTile& tt, int grid,
                          int threads, size_t smem, cudaStream_t s) {
    if (dir < 0)
        FP_RUN((k_ypass_tma<T, -1>), grid, threads, smem, s, map, y, tt);
    else
        FP_RUN((k_ypass_tma<T, +1>), grid, threads, smem, s, map, y, tt);
    return cudaGetLastError();
}
#endif

#ifdef FP_DEFINE_Z_RUNNERS
template <typename T>
cudaError_t run_zgreen(int mode, const ZArgs& z, dim3 grid, int threads, size_t smem, cudaStream_t s,
                       bool lowreg) {
    if constexpr (sizeof(T) == 4) {
        if (lowreg && mode == 0) {
            FP_RUN((k_zgreen_lr<T, 0>), grid, threads, smem, s, z);
            return cudaGetLastError();
        }
    }
    switch (mode) {
        case 0: FP_RUN((k_zgreen<T, 0>), grid, threads, smem, s, z); break;
        case 1: FP_RUN((k_zgreen<T, 1>), grid, threads, smem, s, z); break;
        default: FP_RUN((k_zgreen<T, 2>), grid, threads, smem, s, z); break;
    }
    return cudaGetLastError();
}
#endif

#ifdef FP_DEFINE_ZTMA_RUNNERS
template <typename T>
cudaError_t run_zgreen_tma(const CUtensorMap& map, const ZArgs& z, const TmaTile& tt, int grid,
                           int threads, size_t smem, cudaStream_t s) {
    FP_RUN((k_zgreen_tma<T>), grid, threads, smem, s, map, z, tt);
    return cudaGetLastError();
}
#endif

}  // namespace fp
