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

bool make_axis_plan(int n, AxisPlan& p, std::string& err) {
    p = AxisPlan{};
    if (n > 640) {
        // the FP64 z pass keeps the three components of one column in one
        // CTA of at most 256 threads: 3 * ceil(n/8) <= 256
        err = "grid edge " + std::to_string(n) + " exceeds the supported maximum of 640";
        return false;
    }
    p.dev.n = n;
    p.dev.tpl = std::max(1, (n + 7) / 8);
    const int ns = factor_radices(n, p.dev.radix, 4);
    p.dev.nstage64 = factor_radices(n, p.dev.radix64, 3);
    if (ns < 0) {
        err = "grid edge " + std::to_string(n) + " is not a product of 2, 3 and 5";
        return false;
    }
    p.dev.nstage = ns;
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
    int ny, nxh, tx;
    long long nh;
    FftPlanDev plan;
    void* spec;
    const int* skip;
};

struct ZArgs {
    int ny, nz, nxh, tz;
    long long nh;
    FftPlanDev plan;
    const void* green;
    void* spec;
    const int* skip;
};

// ---------------------------------------------------------------------------
// P1: forward x with fused source construction
// ---------------------------------------------------------------------------

template <typename T, int SRC>
__global__ void __launch_bounds__(sizeof(T) == 8 ? 256 : 512) k_xfwd(XArgs a) {
    if (a.skip && *a.skip) return;
    using T2 = c_t<T>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T2* lines = reinterpret_cast<T2*>(smem_raw);
    const int nx = a.nx;
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
        lines[t] = cmk<T2>(vr, vi);
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
        for (int s = s0 + threadIdx.x; s < s1; s += blockDim.x) {
            const long long idx = a.support[s];
            const int rl = (int)(idx / nx - r0);
            const int x = (int)(idx - (r0 + rl) * nx);
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                double val = 0.0;
                if (SRC != kSrcF0) val = a.src[3LL * s + c] - mean[c];
                if (SRC != kSrcCompact) val += a.f0_support[c];
                const int L = 3 * rl + c;
                T2* p = &lines[(L >> 1) * nx + x];
                if (L & 1) p->y = (T)val; else p->x = (T)val;
            }
        }
        __syncthreads();
    }

    // 3) forward FFT of every complex line
    {
        const int tpl = a.plan.tpl;
        const int q = threadIdx.x / tpl;
        const int lane = threadIdx.x - q * tpl;
        fft_line<-1>(q < nq ? lines + q * nx : (T2*)nullptr, a.plan, lane);
    }

    // 4) separate the two real spectra and store the half spectrum
    const int nxh = a.nxh;
    const int tot2 = nq * nxh;
    for (int t = threadIdx.x; t < tot2; t += blockDim.x) {
        const int q = t / nxh;
        const int k = t - q * nxh;
        const T2 zk = lines[q * nx + k];
        const int kn = (k == 0) ? 0 : nx - k;
        const T2 zn = lines[q * nx + kn];
        const T2 A = cmk<T2>((T)0.5 * (zk.x + zn.x), (T)0.5 * (zk.y - zn.y));
        const T2 B = cmk<T2>((T)0.5 * (zk.y + zn.y), (T)0.5 * (zn.x - zk.x));
        {
            const int L = 2 * q;
            const int rl = L / 3;
            const int c = L - 3 * rl;
            spec[c * a.nh + (r0 + rl) * nxh + k] = A;
        }
        const int L = 2 * q + 1;
        if (L < nreal) {
            const int rl = L / 3;
            const int c = L - 3 * rl;
            spec[c * a.nh + (r0 + rl) * nxh + k] = B;
        }
    }
}

// ---------------------------------------------------------------------------
// P2 / P4: y pass (one z plane, a tile of kx columns, one component)
// ---------------------------------------------------------------------------

template <typename T, int S>
__global__ void __launch_bounds__(sizeof(T) == 8 ? 256 : 512) k_ypass(YArgs a) {
    if (a.skip && *a.skip) return;
    using T2 = c_t<T>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T2* lines = reinterpret_cast<T2*>(smem_raw);
    const int ny = a.ny;
    const int k0 = blockIdx.x * a.tx;
    const int tx = min(a.tx, a.nxh - k0);
    const long long z = blockIdx.y;
    const int comp = blockIdx.z;
    T2* base = reinterpret_cast<T2*>(a.spec) + comp * a.nh + z * (long long)ny * a.nxh + k0;
    const int total = ny * tx;
    for (int t = threadIdx.x; t < total; t += blockDim.x) {
        const int y = t / tx;
        const int c = t - y * tx;
        lines[c * ny + y] = base[(long long)y * a.nxh + c];
    }
    __syncthreads();
    {
        const int tpl = a.plan.tpl;
        const int q = threadIdx.x / tpl;
        const int lane = threadIdx.x - q * tpl;
        fft_line<S>(q < tx ? lines + q * ny : (T2*)nullptr, a.plan, lane);
    }
    for (int t = threadIdx.x; t < total; t += blockDim.x) {
        const int y = t / tx;
        const int c = t - y * tx;
        base[(long long)y * a.nxh + c] = lines[c * ny + y];
    }
}

// ---------------------------------------------------------------------------
// P3: z forward, Green multiply, z inverse (one ky, a tile of kx, 3 comps)
// ---------------------------------------------------------------------------

// ZMODE: 0 = forward z, Green multiply, inverse z; 1 = forward z only;
// 2 = inverse z only
template <typename T, int ZMODE>
__global__ void __launch_bounds__(sizeof(T) == 8 ? 256 : 512) k_zgreen(ZArgs a) {
    if (a.skip && *a.skip) return;
    using T2 = c_t<T>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T2* lines = reinterpret_cast<T2*>(smem_raw);
    const int nz = a.nz;
    const int k0 = blockIdx.x * a.tz;
    const int tz = min(a.tz, a.nxh - k0);
    const long long ky = blockIdx.y;
    const long long plane = (long long)a.ny * a.nxh;
    T2* spec = reinterpret_cast<T2*>(a.spec);
    const long long off0 = ky * a.nxh + k0;
    const int total = 3 * nz * tz;
    for (int t = threadIdx.x; t < total; t += blockDim.x) {
        const int c = t % tz;
        const int rest = t / tz;
        const int z = rest % nz;
        const int comp = rest / nz;
        lines[(comp * tz + c) * nz + z] = spec[comp * a.nh + z * plane + off0 + c];
    }
    __syncthreads();
    const int tpl = a.plan.tpl;
    const int q = threadIdx.x / tpl;
    const int lane = threadIdx.x - q * tpl;
    T2* my = q < 3 * tz ? lines + q * nz : (T2*)nullptr;
    if (ZMODE != 2) fft_line<-1>(my, a.plan, lane);
    // Green multiply: u = G f at every (kz, kx)
    const T* g = reinterpret_cast<const T*>(a.green);
    for (int t = threadIdx.x; ZMODE == 0 && t < nz * tz; t += blockDim.x) {
        const int c = t % tz;
        const int z = t / tz;
        const long long gi = z * plane + off0 + c;
        const T gxx = g[gi], gxy = g[a.nh + gi], gxz = g[2 * a.nh + gi];
        const T gyy = g[3 * a.nh + gi], gyz = g[4 * a.nh + gi], gzz = g[5 * a.nh + gi];
        T2* fx = &lines[(0 * tz + c) * nz + z];
        T2* fy = &lines[(1 * tz + c) * nz + z];
        T2* fz = &lines[(2 * tz + c) * nz + z];
        const T2 ax = *fx, ay = *fy, az = *fz;
        *fx = cmk<T2>(gxx * ax.x + gxy * ay.x + gxz * az.x, gxx * ax.y + gxy * ay.y + gxz * az.y);
        *fy = cmk<T2>(gxy * ax.x + gyy * ay.x + gyz * az.x, gxy * ax.y + gyy * ay.y + gyz * az.y);
        *fz = cmk<T2>(gxz * ax.x + gyz * ay.x + gzz * az.x, gxz * ax.y + gyz * ay.y + gzz * az.y);
    }
    __syncthreads();
    if (ZMODE != 1) fft_line<+1>(my, a.plan, lane);
    for (int t = threadIdx.x; t < total; t += blockDim.x) {
        const int c = t % tz;
        const int rest = t / tz;
        const int z = rest % nz;
        const int comp = rest / nz;
        spec[comp * a.nh + z * plane + off0 + c] = lines[(comp * tz + c) * nz + z];
    }
}

// ---------------------------------------------------------------------------
// P5: inverse x with fused gather / dense store and partial sums
// ---------------------------------------------------------------------------

template <typename T, int DST>
__global__ void __launch_bounds__(sizeof(T) == 8 ? 256 : 512) k_xinv(XArgs a) {
    if (a.skip && *a.skip) return;
    using T2 = c_t<T>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T2* lines = reinterpret_cast<T2*>(smem_raw);
    __shared__ double red[4 * 32];
    const int nx = a.nx;
    const int nxh = a.nxh;
    const long long r0 = (long long)blockIdx.x * a.rows_per_cta;
    const int rows = (int)min((long long)a.rows_per_cta, a.nrows - r0);
    const int nreal = 3 * rows;
    const int nq = (nreal + 1) / 2;
    const T2* spec = reinterpret_cast<const T2*>(a.spec);
    const bool even = (nx % 2) == 0;

    // 1) Z = A + iB on the full line from the two Hermitian half spectra
    const int tot = nq * nxh;
    for (int t = threadIdx.x; t < tot; t += blockDim.x) {
        const int q = t / nxh;
        const int k = t - q * nxh;
        T2 A, B;
        {
            const int L = 2 * q;
            const int rl = L / 3;
            const int c = L - 3 * rl;
            A = spec[c * a.nh + (r0 + rl) * nxh + k];
        }
        {
            const int L = 2 * q + 1;
            if (L < nreal) {
                const int rl = L / 3;
                const int c = L - 3 * rl;
                B = spec[c * a.nh + (r0 + rl) * nxh + k];
            } else {
                B = cmk<T2>((T)0, (T)0);
            }
        }
        if (k == 0 || (even && 2 * k == nx)) {  // DC / Nyquist are real for a real line
            A.y = 0;
            B.y = 0;
        }
        lines[q * nx + k] = cmk<T2>(A.x - B.y, A.y + B.x);
        const int kn = nx - k;
        if (k > 0 && kn >= nxh) lines[q * nx + kn] = cmk<T2>(A.x + B.y, B.x - A.y);
    }
    __syncthreads();
    {
        const int tpl = a.plan.tpl;
        const int q = threadIdx.x / tpl;
        const int lane = threadIdx.x - q * tpl;
        fft_line<+1>(q < nq ? lines + q * nx : (T2*)nullptr, a.plan, lane);
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
                const T2 zv = lines[(L >> 1) * nx + x];
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
            const T2 zv = lines[(L >> 1) * nx + x];
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

static int choose_rows_per_cta(const Problem& P, size_t elem, int max_threads) {
    const int tpl = P.px.dev.tpl;
    int rows = 1;
    for (int r = 1; r <= 64; ++r) {
        const int nq = (3 * r + 1) / 2;
        if (nq * tpl > max_threads) break;
        if ((size_t)nq * P.nx * elem > 64 * 1024) break;
        rows = r;
        if (nq * tpl >= max_threads / 2 && (r % 2) == 0) break;
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
    const int max_threads = sizeof(T) == 8 ? 256 : 512;  // matches __launch_bounds__
    XArgs x{};
    x.nx = P.nx;
    x.ny = P.ny;
    x.nz = P.nz;
    x.nxh = P.nxh;
    x.n = P.n;
    x.nh = P.nh;
    x.nrows = P.nrows;
    x.rows_per_cta = choose_rows_per_cta(P, elem, max_threads);
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
    const int xthreads = std::max(32, ((nq * P.px.dev.tpl + 31) / 32) * 32);
    const size_t xsmem = (size_t)nq * P.nx * elem;
    const int xblocks = (int)((P.nrows + x.rows_per_cta - 1) / x.rows_per_cta);

    if (aa.stage != kStageInverse) switch (aa.src_kind) {
        case kSrcCompact:
            cudaFuncSetAttribute(k_xfwd<T, kSrcCompact>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)xsmem);
            k_xfwd<T, kSrcCompact><<<xblocks, xthreads, xsmem, P.stream>>>(x);
            break;
        case kSrcDense:
            cudaFuncSetAttribute(k_xfwd<T, kSrcDense>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)xsmem);
            k_xfwd<T, kSrcDense><<<xblocks, xthreads, xsmem, P.stream>>>(x);
            break;
        case kSrcF0:
            cudaFuncSetAttribute(k_xfwd<T, kSrcF0>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)xsmem);
            k_xfwd<T, kSrcF0><<<xblocks, xthreads, xsmem, P.stream>>>(x);
            break;
        default:
            cudaFuncSetAttribute(k_xfwd<T, kSrcF0Compact>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)xsmem);
            k_xfwd<T, kSrcF0Compact><<<xblocks, xthreads, xsmem, P.stream>>>(x);
            break;
    }

    // y passes
    YArgs y{};
    y.ny = P.ny;
    y.nxh = P.nxh;
    y.nh = P.nh;
    y.plan = P.py.dev;
    y.spec = P.d_spec;
    y.skip = aa.skip;
    {
        int tx = (elem == 16) ? 8 : 16;
        while (tx > 1 && (tx * P.py.dev.tpl > max_threads || (size_t)tx * P.ny * elem > 64 * 1024)) tx /= 2;
        y.tx = tx;
    }
    const int ythreads = std::max(32, ((y.tx * P.py.dev.tpl + 31) / 32) * 32);
    const size_t ysmem = (size_t)y.tx * P.ny * elem;
    dim3 ygrid((P.nxh + y.tx - 1) / y.tx, P.nz, 3);
    cudaFuncSetAttribute(k_ypass<T, -1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ysmem);
    cudaFuncSetAttribute(k_ypass<T, +1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ysmem);
    if (P.ny > 1 && aa.stage != kStageInverse) k_ypass<T, -1><<<ygrid, ythreads, ysmem, P.stream>>>(y);

    // z pass with the Green multiply
    ZArgs z{};
    z.ny = P.ny;
    z.nz = P.nz;
    z.nxh = P.nxh;
    z.nh = P.nh;
    z.plan = P.pz.dev;
    z.green = (sizeof(T) == 8) ? (const void*)P.d_green64 : (const void*)P.d_green32;
    z.spec = P.d_spec;
    z.skip = aa.skip;
    {
        int tz = (elem == 16) ? 4 : 8;
        while (tz > 1 && (3 * tz * P.pz.dev.tpl > max_threads || (size_t)3 * tz * P.nz * elem > 96 * 1024)) tz /= 2;
        z.tz = tz;
    }
    const int zthreads = std::max(32, ((3 * z.tz * P.pz.dev.tpl + 31) / 32) * 32);
    const size_t zsmem = (size_t)3 * z.tz * P.nz * elem;
    dim3 zgrid((P.nxh + z.tz - 1) / z.tz, P.ny);
    if (aa.stage != kStageInverse) {
        if (aa.stage == kStageForward) {
            cudaFuncSetAttribute(k_zgreen<T, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)zsmem);
            k_zgreen<T, 1><<<zgrid, zthreads, zsmem, P.stream>>>(z);
            *nparts = 0;
            return cudaGetLastError();
        }
        cudaFuncSetAttribute(k_zgreen<T, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)zsmem);
        k_zgreen<T, 0><<<zgrid, zthreads, zsmem, P.stream>>>(z);
    } else {
        cudaFuncSetAttribute(k_zgreen<T, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)zsmem);
        k_zgreen<T, 2><<<zgrid, zthreads, zsmem, P.stream>>>(z);
    }

    if (P.ny > 1) k_ypass<T, +1><<<ygrid, ythreads, ysmem, P.stream>>>(y);

    if (aa.dst_kind == kDstCompact) {
        cudaFuncSetAttribute(k_xinv<T, kDstCompact>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)xsmem);
        k_xinv<T, kDstCompact><<<xblocks, xthreads, xsmem, P.stream>>>(x);
    } else {
        cudaFuncSetAttribute(k_xinv<T, kDstDense>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)xsmem);
        k_xinv<T, kDstDense><<<xblocks, xthreads, xsmem, P.stream>>>(x);
    }
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
