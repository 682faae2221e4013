// kernels_fft.cu -- the five passes of one Green-operator apply on GB300.
//
//   P1 forward x (R2C, two real lines per complex FFT) fused with the
//      scatter of the compact support vector (and/or the background force)
//   P2 forward y
//   P3 forward z, Green multiply (3x3 real symmetric), inverse z
//   P4 inverse y
//   P5 inverse x (C2R) fused with the gather to the support, the 1/N scale
//      and per-CTA partial sums used for mean removal and MINRES dots.
//
// The spectral field is three component blocks of the half spectrum, each
// laid out [kz][ky][kx] with kx in [0, nx/2] fastest.  This replaces the
// reference's per-component C2C FFTW calls + Green multiply
// (src/bignonnet/GreenOperator.cpp:54-93, src/fft/FFTWBackend.cpp:301-420):
// the reference keeps Re(IFFT(G * FFT f)), whose effective symbol is the
// symmetrised tensor (G(k) + G(-k)) / 2, which is what the Green table holds.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <string>

#include "common.cuh"
#include "fft_engine.cuh"
#include "internal.h"
#include "tma.cuh"

namespace fp {

// ---------------------------------------------------------------------------
// plans
// ---------------------------------------------------------------------------

static int factor_radices(int n, int* radix, int max_log2) {
    int k = 0;
    int e2 = 0;
    while (n % 2 == 0) {
        n /= 2;
        ++e2;
    }
    // split the power of two into ceil(e2/4) stages as evenly as possible
    if (e2 > 0) {
        const int s = (e2 + max_log2 - 1) / max_log2;
        for (int i = 0; i < s; ++i) {
            const int e = e2 / s + (i < e2 % s ? 1 : 0);
            radix[k++] = 1 << e;
        }
    }
    while (n % 3 == 0) {
        n /= 3;
        radix[k++] = 3;
    }
    while (n % 5 == 0) {
        n /= 5;
        radix[k++] = 5;
    }
    return n == 1 ? k : -1;
}

bool fill_plan_radices(int n, FftPlanDev& d) {
    if (n < 1 || n > 640) return false;
    d.n = n;
    const int ns32 = factor_radices(n, d.radix32, 4);
    const int ns64 = factor_radices(n, d.radix64, 3);
    if (ns32 < 0 || ns64 < 0) return false;
    d.nstage32 = ns32;
    d.nstage64 = ns64;
    int r32 = 1, r64 = 1;
    for (int i = 0; i < ns32; ++i) r32 = std::max(r32, d.radix32[i]);
    for (int i = 0; i < ns64; ++i) r64 = std::max(r64, d.radix64[i]);
    d.tpl32 = (n + r32 - 1) / r32;
    d.tpl64 = (n + r64 - 1) / r64;
    return true;
}

bool make_axis_plan(int n, AxisPlan& p, std::string& err) {
    p = AxisPlan{};
    if (n > 640) {
        // the FP64 z pass keeps the three components of one column in one
        // CTA of at most 256 threads
        err = "grid edge " + std::to_string(n) + " exceeds the supported maximum of 640";
        return false;
    }
    p.dev.n = n;
    const int ns32 = factor_radices(n, p.dev.radix32, 4);
    const int ns64 = factor_radices(n, p.dev.radix64, 3);
    if (ns32 < 0 || ns64 < 0) {
        err = "grid edge " + std::to_string(n) + " is not a product of 2, 3 and 5";
        return false;
    }
    p.dev.nstage32 = ns32;
    p.dev.nstage64 = ns64;
    int r32 = 1, r64 = 1;
    for (int i = 0; i < ns32; ++i) r32 = std::max(r32, p.dev.radix32[i]);
    for (int i = 0; i < ns64; ++i) r64 = std::max(r64, p.dev.radix64[i]);
    p.dev.tpl32 = (n + r32 - 1) / r32;
    p.dev.tpl64 = (n + r64 - 1) / r64;
    std::vector<double2> h64(n);
    std::vector<float2> h32(n);
    const double two_pi = 6.283185307179586476925286766559;
    for (int j = 0; j < n; ++j) {
        const double a = two_pi * (double)j / (double)n;
        h64[j] = make_double2(std::cos(a), -std::sin(a));
        h32[j] = make_float2((float)h64[j].x, (float)h64[j].y);
    }
    if (cudaMalloc(&p.tw64, sizeof(double2) * n) != cudaSuccess ||
        cudaMalloc(&p.tw32, sizeof(float2) * n) != cudaSuccess) {
        err = "cudaMalloc failed for FFT twiddles";
        return false;
    }
    cudaMemcpy(p.tw64, h64.data(), sizeof(double2) * n, cudaMemcpyHostToDevice);
    cudaMemcpy(p.tw32, h32.data(), sizeof(float2) * n, cudaMemcpyHostToDevice);
    p.dev.tw64 = p.tw64;
    p.dev.tw32 = p.tw32;
    return true;
}

void free_axis_plan(AxisPlan& p) {
    cudaFree(p.tw64);
    cudaFree(p.tw32);
    p.tw64 = nullptr;
    p.tw32 = nullptr;
}

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
    int np;        // nbox * box: rows of the raw tile in shared memory
    int bufbytes;  // bytes of one tile buffer (raw tile or padded lines, larger of the two)
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
                    double val = 0.0;
                    if (SRC != kSrcF0) val = cv[u][c] - mean[c];
                    if (SRC != kSrcCompact) val += a.f0_support[c];
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
__global__ void __launch_bounds__(256) k_ypass(YArgs a) {
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
__global__ void __launch_bounds__(256) k_zgreen(ZArgs a) {
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

template <typename T2>
__device__ __forceinline__ bool tma_pipeline_wait(uint64_t* bars, int i, int b, bool prefetched,
                                                  int* err) {
    const bool ok = mbar_wait_bounded(&bars[b], (uint32_t)((i >> 1) & 1));
    if (__syncthreads_or(!ok)) {
        if (threadIdx.x == 0) {
            atomicExch(err, 1);
            if (prefetched) mbar_wait_bounded(&bars[b ^ 1], (uint32_t)(((i + 1) >> 1) & 1));
        }
        return false;
    }
    return true;
}

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
    const uint32_t tile_bytes = (uint32_t)(3 * tt.np * t * sizeof(T2));
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
    const uint32_t tile_bytes = (uint32_t)(3 * tt.np * t * sizeof(T2));
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

template <typename T, int DST>
__global__ void __launch_bounds__(256, 3) k_xinv(XArgs a) {
    if (a.skip && *a.skip) return;
    using T2 = c_t<T>;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    T2* lines = reinterpret_cast<T2*>(smem_raw);
    __shared__ double red[4 * 32];
    const int nx = a.nx;
    const int nxh = a.nxh;
    const int ld = a.ld;
    const long long r0 = (long long)blockIdx.x * a.rows_per_cta;
    const int rows = (int)min((long long)a.rows_per_cta, a.nrows - r0);
    const int nreal = 3 * rows;
    const int nq = (nreal + 1) / 2;
    const T2* spec = reinterpret_cast<const T2*>(a.spec);
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
                A[u] = spec[ca * a.nh + (r0 + rla) * a.rs + k];
                const int Lb = La + 1;
                if (Lb < nreal) {
                    const int rlb = Lb / 3, cb = Lb - 3 * rlb;
                    B[u] = spec[cb * a.nh + (r0 + rlb) * a.rs + k];
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
    double acc[4] = {0.0, 0.0, 0.0, 0.0};
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
                const double val = (double)((L & 1) ? zv.y : zv.x) * a.scale;
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
            const double val = (double)((L & 1) ? zv.y : zv.x) * a.scale;
            a.dst[c * a.n + (r0 + rl) * nx + x] = val;
            acc[c] += val;
        }
    }
    double out[4];
    block_sum<4>(acc, red, out);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int i = 0; i < 4; ++i) a.partials[4LL * blockIdx.x + i] = out[i];
    }
}

// ---------------------------------------------------------------------------
// host launcher
// ---------------------------------------------------------------------------

// ---------------------------------------------------------------------------
// TMA descriptors
// ---------------------------------------------------------------------------

using EncodeTiledFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*,
                                   const cuuint64_t*, const cuuint64_t*, const cuuint32_t*,
                                   const cuuint32_t*, CUtensorMapInterleave, CUtensorMapSwizzle,
                                   CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static EncodeTiledFn tma_encoder() {
    static EncodeTiledFn fn = nullptr;
    static bool tried = false;
    if (!tried) {
        tried = true;
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                             &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiledFn>(p);
    }
    return fn;
}

constexpr int kTmaSmemLimit = 227 * 1024;

// Chooses the tiling of the TMA-fed y (axis 0) or z (axis 1) pass and builds
// or reuses its descriptor.  Returns false when the TMA path does not apply.
static bool tma_setup(Problem& P, bool dbl, int axis, int tpl, int ld, TmaTile& tt,
                      const CUtensorMap** map) {
    if (P.tma_off || !tma_encoder()) return false;
    const size_t e = dbl ? sizeof(double) : sizeof(float);
    const size_t e2 = 2 * e;
    const int n = axis == 0 ? P.ny : P.nz;
    if (n < 16) return false;
    TmaCache& cache = axis == 0 ? P.tma_y[dbl ? 0 : 1] : P.tma_z[dbl ? 0 : 1];
    tt.nbox = (n + 255) / 256;
    tt.box = (n + tt.nbox - 1) / tt.nbox;
    tt.np = tt.nbox * tt.box;
    int t = P.tile_yz > 0 ? P.tile_yz : (dbl ? 8 : 16);
    t &= ~1;
    for (; t >= 2; t /= 2) {
        if (t * tpl > 256) continue;
        const size_t raw = (size_t)3 * tt.np * t * e2;
        const size_t lines = (size_t)3 * t * ld * e2;
        const size_t buf = ((raw > lines ? raw : lines) + 127) & ~size_t(127);
        if (128 + 2 * buf > (size_t)kTmaSmemLimit) continue;
        tt.bufbytes = (int)buf;
        break;
    }
    if (t < 2) return false;
    tt.t = t;
    tt.ntx = (P.nxh + t - 1) / t;
    tt.ntiles = tt.ntx * (axis == 0 ? P.nz : P.ny);
    if (!cache.valid || cache.t != t || cache.box != tt.box) {
        const cuuint64_t dims[4] = {(cuuint64_t)(2 * P.nxh), (cuuint64_t)P.ny, (cuuint64_t)P.nz, 3};
        const cuuint64_t strides[3] = {(cuuint64_t)(2 * P.rs * e), (cuuint64_t)(2 * P.rs * P.ny * e),
                                       (cuuint64_t)(2 * P.nh * e)};
        const cuuint32_t box[4] = {(cuuint32_t)(2 * t), axis == 0 ? (cuuint32_t)tt.box : 1u,
                                   axis == 0 ? 1u : (cuuint32_t)tt.box, 1u};
        const cuuint32_t estr[4] = {1, 1, 1, 1};
        const CUresult r = tma_encoder()(
            &cache.map, dbl ? CU_TENSOR_MAP_DATA_TYPE_FLOAT64 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4,
            P.d_spec, dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
            CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
        if (r != CUDA_SUCCESS) return false;
        cache.valid = true;
        cache.t = t;
        cache.box = tt.box;
    }
    *map = &cache.map;
    return true;
}

static int choose_rows_per_cta(const Problem& P, int tpl, int ld, size_t elem) {
    int rows = 1;
    for (int r = 1; r <= 64; ++r) {
        const int nq = (3 * r + 1) / 2;
        if (nq * tpl > 256) break;  // matches __launch_bounds__(256, 3)
        if ((size_t)nq * ld * elem > 72 * 1024) break;
        rows = r;
    }
    if (rows > P.nrows) rows = (int)P.nrows;
    // enough CTAs to fill the machine
    while (rows > 2 && (P.nrows + rows - 1) / rows < 2LL * P.sm_count) rows -= 2;
    return rows;
}

template <typename T>
static cudaError_t apply_impl(Problem& P, const ApplyArgs& aa, int* nparts) {
    using T2 = c_t<T>;
    const size_t elem = sizeof(T2);
    const bool dbl = sizeof(T) == 8;
    const int padsh = dbl ? Prec<double2>::PADSH : Prec<float2>::PADSH;
    const int max_yz = 256;  // matches __launch_bounds__ of the y and z passes
    auto tpl_of = [&](const AxisPlan& ap) { return dbl ? ap.dev.tpl64 : ap.dev.tpl32; };
    const long long rs = P.rs;
    *nparts = 0;

    // ---- x passes
    XArgs x{};
    x.nx = P.nx;
    x.ny = P.ny;
    x.nz = P.nz;
    x.nxh = P.nxh;
    x.ld = line_stride(P.nx, padsh);
    x.rs = rs;
    x.n = P.n;
    x.nh = P.nh;
    x.nrows = P.nrows;
    const int tplx = tpl_of(P.px);
    x.rows_per_cta = choose_rows_per_cta(P, tplx, x.ld, elem);
    x.plan = P.px.dev;
    x.support = P.d_support;
    x.row_ptr = P.d_row_ptr;
    x.mask = P.d_mask;
    x.src = aa.src;
    x.src_sum = aa.src_sum;
    x.inv_nb = P.nb > 0 ? 1.0 / (double)P.nb : 0.0;
    for (int c = 0; c < 3; ++c) {
        x.f0_fluid[c] = aa.f0_fluid[c];
        x.f0_support[c] = aa.f0_support[c];
    }
    x.dst = aa.dst;
    x.dot_with = aa.dot_with;
    x.scale = 1.0 / (double)P.n;
    x.partials = P.d_partials;
    x.spec = P.d_spec;
    x.skip = aa.skip;
    const int nq = (3 * x.rows_per_cta + 1) / 2;
    const int xthreads = std::max(32, ((nq * tplx + 31) / 32) * 32);
    const size_t xsmem = (size_t)nq * x.ld * elem;
    const int xblocks = (int)((P.nrows + x.rows_per_cta - 1) / x.rows_per_cta);

    // ---- y passes: tx columns x 3 components per CTA
    YArgs y{};
    y.ny = P.ny;
    y.nxh = P.nxh;
    y.nh = P.nh;
    y.rs = rs;
    y.plan = P.py.dev;
    y.spec = P.d_spec;
    y.skip = aa.skip;
    y.err = P.d_err;
    y.nz = P.nz;
    y.ld = line_stride(P.ny, padsh);
    const int tply = tpl_of(P.py);
    {
        int tx = P.tile_yz > 0 ? P.tile_yz : (dbl ? 8 : 16);
        while (tx > 1 && (tx * tply > max_yz || (size_t)3 * tx * y.ld * elem > 110 * 1024)) tx /= 2;
        y.tx = tx;
    }
    const int ythreads = y.tx * tply;
    const size_t ysmem = (size_t)3 * y.tx * y.ld * elem;
    dim3 ygrid((P.nxh + y.tx - 1) / y.tx, P.nz);

    // ---- z pass
    ZArgs z{};
    z.ny = P.ny;
    z.nz = P.nz;
    z.nxh = P.nxh;
    z.nh = P.nh;
    z.rs = rs;
    z.plane = (long long)P.ny * rs;
    z.gstride = P.nh;
    z.plan = P.pz.dev;
    z.green = dbl ? (const void*)P.d_green64 : (const void*)P.d_green32;
    z.spec = P.d_spec;
    z.skip = aa.skip;
    z.err = P.d_err;
    z.ld = line_stride(P.nz, padsh);
    const int tplz = tpl_of(P.pz);
    {
        int tz = P.tile_yz > 0 ? P.tile_yz : (dbl ? 8 : 16);
        while (tz > 1 && (tz * tplz > max_yz || (size_t)3 * tz * z.ld * elem > 110 * 1024)) tz /= 2;
        z.tz = tz;
    }
    const int zthreads = z.tz * tplz;
    const size_t zsmem = (size_t)3 * z.tz * z.ld * elem;
    dim3 zgrid((P.nxh + z.tz - 1) / z.tz, P.ny);

    TmaTile tty{}, ttz{};
    const CUtensorMap* mapy = nullptr;
    const CUtensorMap* mapz = nullptr;
    const bool tma_y = P.d_err && tma_setup(P, dbl, 0, tply, y.ld, tty, &mapy);
    const bool tma_z = P.d_err && tma_setup(P, dbl, 1, tplz, z.ld, ttz, &mapz);
    const int ygrid_tma = (int)std::min<long long>(tty.ntiles, P.sm_count);
    const int zgrid_tma = (int)std::min<long long>(ttz.ntiles, P.sm_count);
    const size_t ysmem_tma = 128 + 2 * (size_t)tty.bufbytes;
    const size_t zsmem_tma = 128 + 2 * (size_t)ttz.bufbytes;
    if (tma_y) y.tx = tty.t;
    if (tma_z) z.tz = ttz.t;

#define FP_LAUNCH_TMA(kern, grid, threads, smem, map, args, tt)                                  \
    do {                                                                                          \
        cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)(smem));     \
        FP_LAUNCHED(); kern<<<grid, threads, smem, P.stream>>>(*(map), args, tt);                                \
    } while (0)

#define FP_LAUNCH(kern, grid, threads, smem, args)                                              \
    do {                                                                                          \
        cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)(smem));     \
        FP_LAUNCHED(); kern<<<grid, threads, smem, P.stream>>>(args);                                            \
    } while (0)

    if (aa.stage != kStageInverse) {
        switch (aa.src_kind) {
            case kSrcCompact: FP_LAUNCH((k_xfwd<T, kSrcCompact>), xblocks, xthreads, xsmem, x); break;
            case kSrcDense: FP_LAUNCH((k_xfwd<T, kSrcDense>), xblocks, xthreads, xsmem, x); break;
            case kSrcF0: FP_LAUNCH((k_xfwd<T, kSrcF0>), xblocks, xthreads, xsmem, x); break;
            default: FP_LAUNCH((k_xfwd<T, kSrcF0Compact>), xblocks, xthreads, xsmem, x); break;
        }
        if (tma_y)
            FP_LAUNCH_TMA((k_ypass_tma<T, -1>), ygrid_tma, tty.t * tply, ysmem_tma, mapy, y, tty);
        else if (P.ny > 1)
            FP_LAUNCH((k_ypass<T, -1>), ygrid, ythreads, ysmem, y);
        if (aa.stage == kStageForward) {
            FP_LAUNCH((k_zgreen<T, 1>), zgrid, zthreads, zsmem, z);
            return cudaGetLastError();
        }
        if (tma_z)
            FP_LAUNCH_TMA((k_zgreen_tma<T>), zgrid_tma, ttz.t * tplz, zsmem_tma, mapz, z, ttz);
        else
            FP_LAUNCH((k_zgreen<T, 0>), zgrid, zthreads, zsmem, z);
    } else {
        FP_LAUNCH((k_zgreen<T, 2>), zgrid, zthreads, zsmem, z);
    }
    if (tma_y)
        FP_LAUNCH_TMA((k_ypass_tma<T, +1>), ygrid_tma, tty.t * tply, ysmem_tma, mapy, y, tty);
    else if (P.ny > 1)
        FP_LAUNCH((k_ypass<T, +1>), ygrid, ythreads, ysmem, y);
    if (aa.dst_kind == kDstCompact) {
        FP_LAUNCH((k_xinv<T, kDstCompact>), xblocks, xthreads, xsmem, x);
    } else {
        FP_LAUNCH((k_xinv<T, kDstDense>), xblocks, xthreads, xsmem, x);
    }
#undef FP_LAUNCH
#undef FP_LAUNCH_TMA
    *nparts = xblocks;
    return cudaGetLastError();
}

cudaError_t launch_apply(Problem& P, const ApplyArgs& a, int* nparts) {
    const int prec = a.precision >= 0 ? a.precision : P.precision;
    if (prec == kFP64) return apply_impl<double>(P, a, nparts);
    if (!P.d_green32) return cudaErrorInvalidValue;
    return apply_impl<float>(P, a, nparts);
}

}  // namespace fp
