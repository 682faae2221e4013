// kernels_fft.cu -- host side of one Green-operator apply on GB300: FFT
// plans, the tiling of each pass, TMA descriptors and the pass sequence.  The
// kernels live in fft_passes.cuh.
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

#include "fft_fast.cuh"
#include "fft_passes.cuh"

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

bool make_axis_plan(int n, AxisPlan& p, std::string& err, cudaStream_t stream) {
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
    if (cudaMallocAsync(reinterpret_cast<void**>(&p.tw64), sizeof(double2) * n, stream) != cudaSuccess ||
        cudaMallocAsync(reinterpret_cast<void**>(&p.tw32), sizeof(float2) * n, stream) != cudaSuccess) {
        err = "device allocation failed for FFT twiddles";
        return false;
    }
    cudaMemcpyAsync(p.tw64, h64.data(), sizeof(double2) * n, cudaMemcpyHostToDevice, stream);
    cudaMemcpyAsync(p.tw32, h32.data(), sizeof(float2) * n, cudaMemcpyHostToDevice, stream);
    cudaStreamSynchronize(stream);  // the host tables must outlive their copies
    p.dev.tw64 = p.tw64;
    p.dev.tw32 = p.tw32;
    return true;
}

void free_axis_plan(AxisPlan& p, cudaStream_t stream) {
    if (p.tw64) cudaFreeAsync(p.tw64, stream);
    if (p.tw32) cudaFreeAsync(p.tw32, stream);
    p.tw64 = nullptr;
    p.tw32 = nullptr;
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

// Resolved once per process; the initialisation of a function-local static
// is thread-safe, and batches call this from several host threads.
static EncodeTiledFn tma_encoder() {
    static const EncodeTiledFn fn = []() -> EncodeTiledFn {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                             &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            return reinterpret_cast<EncodeTiledFn>(p);
        return nullptr;
    }();
    return fn;
}

constexpr int kTmaSmemLimit = 227 * 1024;

// Chooses the tiling of the TMA-fed y (axis 0) or z (axis 1) pass and builds
// or reuses its descriptor.  Returns false when the TMA path does not apply.
static bool tma_setup(Problem& P, bool dbl, int axis, int tpl, int padsh, TmaTile& tt,
                      const CUtensorMap** map) {
    if (P.tma_off || !tma_encoder()) return false;
    const size_t e = dbl ? sizeof(double) : sizeof(float);
    const size_t e2 = 2 * e;
    const int n = axis == 0 ? P.ny : P.nz;
    if (n < 16) return false;
    TmaCache& cache = axis == 0 ? P.tma_y[dbl ? 0 : 1] : P.tma_z[dbl ? 0 : 1];
    tt.nbox = (n + 255) / 256;
    tt.box = (n + tt.nbox - 1) / tt.nbox;
    int t = P.tile_yz > 0 ? P.tile_yz : (dbl ? 8 : 16);
    t &= ~1;
    // A tiled TMA copy writes shared memory from a 128-byte aligned address:
    // each box lands at (component * np + box index * box) * t elements, so
    // box * t * e2 (when there are several boxes) and np * t * e2 must be
    // multiples of 128.  np pads the component stride; the padding rows are
    // neither loaded nor read.
    for (; t >= 2; t /= 2) {
        if (t * tpl > 256) continue;
        if (tt.nbox > 1 && ((size_t)tt.box * t * e2) % 128 != 0) continue;
        tt.np = tt.nbox * tt.box;
        while (((size_t)tt.np * t * e2) % 128 != 0) ++tt.np;
        const size_t raw = (size_t)3 * tt.np * t * e2;
        const int ld = column_line_stride(n, padsh, t, (int)e2);
        tt.ld = ld;
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

bool fast_maps(Problem& P, bool dbl, int tx, const CUtensorMap** spec, const CUtensorMap** green) {
    if (!tma_encoder()) return false;
    const int k = dbl ? 0 : 1;
    const void* g = dbl ? (const void*)P.d_green64 : (const void*)P.d_green32;
    if (!g || P.nz > 256) return false;
    if (!P.fz_valid[k] || P.fz_green_ptr[k] != g) {
        const size_t e = dbl ? sizeof(double) : sizeof(float);
        const CUtensorMapDataType dt = dbl ? CU_TENSOR_MAP_DATA_TYPE_FLOAT64 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32;
        const cuuint32_t estr[4] = {1, 1, 1, 1};
        // the spectral field: interleaved (re, im) reals
        const cuuint64_t sd[4] = {(cuuint64_t)(2 * P.nxh), (cuuint64_t)P.ny, (cuuint64_t)P.nz, 3};
        const cuuint64_t ss[3] = {(cuuint64_t)(2 * P.rs * e), (cuuint64_t)(2 * P.rs * P.ny * e),
                                  (cuuint64_t)(2 * P.nh * e)};
        const cuuint32_t sb[4] = {(cuuint32_t)(2 * tx), 1u, (cuuint32_t)P.nz, 1u};
        CUresult r = tma_encoder()(&P.fz_spec_map[k], dt, 4, P.d_spec, sd, ss, sb, estr,
                                   CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                                   CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
        if (r != CUDA_SUCCESS) return false;
        // the Green table: six real blocks
        const cuuint64_t gd[4] = {(cuuint64_t)P.nxh, (cuuint64_t)P.ny, (cuuint64_t)P.nz, 6};
        const cuuint64_t gs[3] = {(cuuint64_t)(P.rs * e), (cuuint64_t)(P.rs * P.ny * e),
                                  (cuuint64_t)(P.nh * e)};
        const cuuint32_t gb[4] = {(cuuint32_t)tx, 1u, (cuuint32_t)P.nz, 1u};
        r = tma_encoder()(&P.fz_green_map[k], dt, 4, const_cast<void*>(g), gd, gs, gb, estr,
                          CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                          CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
        if (r != CUDA_SUCCESS) return false;
        P.fz_green_ptr[k] = g;
        P.fz_valid[k] = true;
    }
    *spec = &P.fz_spec_map[k];
    *green = &P.fz_green_map[k];
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
    // a tuned cap (fewer rows: smaller CTAs, more of them per SM)
    if (P.x_rows > 0 && P.x_rows < rows) rows = P.x_rows;
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
    x.err = P.d_err;
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
    const int bank_row = 128 / (int)elem;  // elements per shared-memory bank row
    const int tply = tpl_of(P.py);
    {
        const int ld_max = line_stride(P.ny, padsh) + bank_row;
        int tx = P.tile_yz > 0 ? P.tile_yz : (dbl ? 8 : 16);
        while (tx > 1 && (tx * tply > max_yz || (size_t)3 * tx * ld_max * elem > 110 * 1024)) tx /= 2;
        y.tx = tx;
        y.ld = column_line_stride(P.ny, padsh, tx, (int)elem);
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
    const int tplz = tpl_of(P.pz);
    {
        const int ld_max = line_stride(P.nz, padsh) + bank_row;
        int tz = P.tile_yz > 0 ? P.tile_yz : (dbl ? 8 : 16);
        while (tz > 1 && (tz * tplz > max_yz || (size_t)3 * tz * ld_max * elem > 110 * 1024)) tz /= 2;
        z.tz = tz;
        z.ld = column_line_stride(P.nz, padsh, tz, (int)elem);
    }
    const int zthreads = z.tz * tplz;
    const size_t zsmem = (size_t)3 * z.tz * z.ld * elem;
    dim3 zgrid((P.nxh + z.tz - 1) / z.tz, P.ny);

    TmaTile tty{}, ttz{};
    const CUtensorMap* mapy = nullptr;
    const CUtensorMap* mapz = nullptr;
    const bool tma_y = P.d_err && tma_setup(P, dbl, 0, tply, padsh, tty, &mapy);
    const bool tma_z = P.d_err && tma_setup(P, dbl, 1, tplz, padsh, ttz, &mapz);
    const int ygrid_tma = (int)std::min<long long>(tty.ntiles, P.sm_count);
    const int zgrid_tma = (int)std::min<long long>(ttz.ntiles, P.sm_count);
    const size_t ysmem_tma = 128 + 2 * (size_t)tty.bufbytes;
    const size_t zsmem_tma = 128 + 2 * (size_t)ttz.bufbytes;
    // the TMA-fed passes get their own tile width and line stride; the
    // register-fed kernels (also the forward-only / inverse-only z passes)
    // keep the ones their launch shape was computed from
    YArgs yt = y;
    ZArgs zt = z;
    if (tma_y) {
        yt.tx = tty.t;
        yt.ld = tty.ld;
    }
    if (tma_z) {
        zt.tz = ttz.t;
        zt.ld = ttz.ld;
    }

    cudaStream_t st = P.stream;
    cudaError_t e = cudaSuccess;
#define FP_CHECK(call)                       \
    do {                                     \
        e = (call);                          \
        if (e != cudaSuccess) return e;      \
    } while (0)
    if (aa.stage != kStageInverse) {
        FP_CHECK(run_xfwd<T>(aa.src_kind, x, xblocks, xthreads, xsmem, st));
        if (tma_y)
            FP_CHECK(run_ypass_tma<T>(-1, *mapy, yt, tty, ygrid_tma, tty.t * tply, ysmem_tma, st));
        else if (P.ny > 1)
            FP_CHECK(run_ypass<T>(-1, y, ygrid, ythreads, ysmem, st, P.yz_lowreg));
        if (aa.stage == kStageForward) {
            FP_CHECK(run_zgreen<T>(1, z, zgrid, zthreads, zsmem, st, P.yz_lowreg));
            return cudaSuccess;
        }
        if (tma_z)
            FP_CHECK(run_zgreen_tma<T>(*mapz, zt, ttz, zgrid_tma, ttz.t * tplz, zsmem_tma, st));
        else
            FP_CHECK(run_zgreen<T>(0, z, zgrid, zthreads, zsmem, st, P.yz_lowreg));
    } else {
        FP_CHECK(run_zgreen<T>(2, z, zgrid, zthreads, zsmem, st, P.yz_lowreg));
    }
    if (tma_y)
        FP_CHECK(run_ypass_tma<T>(+1, *mapy, yt, tty, ygrid_tma, tty.t * tply, ysmem_tma, st));
    else if (P.ny > 1)
        FP_CHECK(run_ypass<T>(+1, y, ygrid, ythreads, ysmem, st, P.yz_lowreg));
    // inverse x: persistent bulk-copy pipeline when it fits, else one tile per CTA
    XArgs xb = x;
    int raw_bytes = 0;
    size_t bsmem = 0;
    bool bulk = P.x_bulk && P.d_err;
    if (bulk) {
        for (;;) {
            const int nqb = (3 * xb.rows_per_cta + 1) / 2;
            raw_bytes = (int)(((size_t)3 * xb.rows_per_cta * rs * elem + 127) & ~size_t(127));
            bsmem = 128 + 2 * (size_t)raw_bytes + (size_t)nqb * x.ld * elem;
            if (bsmem <= (size_t)kTmaSmemLimit || xb.rows_per_cta == 1) break;
            xb.rows_per_cta -= 1;
        }
        bulk = bsmem <= (size_t)kTmaSmemLimit;
    }
    if (bulk) {
        const long long ntiles = (P.nrows + xb.rows_per_cta - 1) / xb.rows_per_cta;
        const int per_sm = bsmem <= 110 * 1024 ? 2 : 1;
        const int grid = (int)std::min<long long>(ntiles, (long long)per_sm * P.sm_count);
        const int nqb = (3 * xb.rows_per_cta + 1) / 2;
        const int bthreads = std::max(32, ((nqb * tplx + 31) / 32) * 32);
        FP_CHECK(run_xinv_bulk<T>(aa.dst_kind, xb, raw_bytes, grid, bthreads, bsmem, st));
        *nparts = grid;
    } else {
        FP_CHECK(run_xinv<T>(aa.dst_kind, x, xblocks, xthreads, xsmem, st));
        *nparts = xblocks;
    }
#undef FP_CHECK
    return cudaSuccess;
}

cudaError_t launch_apply(Problem& P, const ApplyArgs& a, int* nparts) {
    const int prec = a.precision >= 0 ? a.precision : P.precision;
    if (prec != kFP64 && !P.d_green32) return cudaErrorInvalidValue;
    if (fast_apply_supported(P, prec, a.src_kind, a.dst_kind, a.stage))
        return fast_apply(P, prec, a, nparts);
    if (prec == kFP64) return apply_impl<double>(P, a, nparts);
    return apply_impl<float>(P, a, nparts);
}

}  // namespace fp
