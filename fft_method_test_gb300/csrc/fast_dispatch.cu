// fast_dispatch.cu -- host side of the specialised apply passes
// (fft_fast.cuh): when they apply, launch geometry, and the pass sequence.
#include <cuda_runtime.h>

#include <algorithm>

#include "fft_fast.cuh"

namespace fp {
namespace fast {

// per-edge dispatch to the runners of fast_runners.cuh (instantiated in
// fast32.cu, fast64.cu, fast32n.cu, fast64n.cu)
#define FP_EDGE_SWITCH(n, CALL)                    \
    switch (n) {                                   \
        case 32: return CALL(32);                  \
        case 48: return CALL(48);                  \
        case 64: return CALL(64);                  \
        case 80: return CALL(80);                  \
        case 96: return CALL(96);                  \
        case 128: return CALL(128);                \
        case 160: return CALL(160);                \
        case 256: return CALL(256);                \
        default: break;                            \
    }

template <typename T>
cudaError_t run_xfwd(int n, const FastArgs& a, dim3 grid, int threads, size_t smem, cudaStream_t s) {
#define FP_CALL(N) Passes<T, N>::xfwd(a, grid, threads, smem, s)
    FP_EDGE_SWITCH(n, FP_CALL)
#undef FP_CALL
    return cudaErrorInvalidValue;
}

template <typename T>
cudaError_t run_xinv(int n, const FastArgs& a, int stage_bytes, dim3 grid, int threads, size_t smem,
                     cudaStream_t s) {
#define FP_CALL(N) Passes<T, N>::xinv(a, stage_bytes, grid, threads, smem, s)
    FP_EDGE_SWITCH(n, FP_CALL)
#undef FP_CALL
    return cudaErrorInvalidValue;
}

template <typename T>
cudaError_t run_y(int n, int dir, const FastArgs& a, dim3 grid, cudaStream_t s) {
#define FP_CALL(N) Passes<T, N>::y(dir, a, grid, s)
    FP_EDGE_SWITCH(n, FP_CALL)
#undef FP_CALL
    return cudaErrorInvalidValue;
}

template <typename T>
cudaError_t run_z(int n, int stages, const CUtensorMap& spec_map, const CUtensorMap& green_map,
                  const FastArgs& a, dim3 grid, size_t smem, cudaStream_t s) {
#define FP_CALL(N) Passes<T, N>::z(stages, spec_map, green_map, a, grid, smem, s)
    FP_EDGE_SWITCH(n, FP_CALL)
#undef FP_CALL
    return cudaErrorInvalidValue;
}

template <typename T>
cudaError_t run_z_shared(int n, const FastArgs& a, int grid, size_t smem, cudaStream_t s) {
#define FP_CALL(N) Passes<T, N>::z_shared(a, grid, smem, s)
    FP_EDGE_SWITCH(n, FP_CALL)
#undef FP_CALL
    return cudaErrorInvalidValue;
}

template <typename T>
int z_blocks_per_sm(int n, int stages, size_t smem) {
#define FP_CALL(N) Passes<T, N>::z_per_sm(stages, smem)
    FP_EDGE_SWITCH(n, FP_CALL)
#undef FP_CALL
    return 1;
}

template <typename T>
int x_blocks_per_sm(int n, bool inverse, int threads, size_t smem) {
#define FP_CALL(N) Passes<T, N>::x_per_sm(inverse, threads, smem)
    FP_EDGE_SWITCH(n, FP_CALL)
#undef FP_CALL
    return 1;
}

#undef FP_EDGE_SWITCH

}  // namespace fast

bool fast_apply_supported(const Problem& P, int precision, int src_kind, int dst_kind, int stage) {
    (void)precision;
    if (P.fast_off || P.tma_off || !P.d_err) return false;
    if (src_kind != kSrcCompact || dst_kind != kDstCompact || stage != kStageFull) return false;
    return fast::edge_supported(P.nx) && fast::edge_supported(P.ny) && fast::edge_supported(P.nz);
}

namespace {

// Arguments and launch geometry of one specialised apply.
template <typename T>
struct FastPlan {
    fast::FastArgs a{};
    int xthreads = 0, stage_bytes = 0, xgrid_f = 0, xgrid_i = 0, zstages = 2, zgrid = 0;
    size_t xsmem = 0, xismem = 0, zsmem = 0;
    dim3 ygrid;
    const CUtensorMap* smap = nullptr;
    const CUtensorMap* gmap = nullptr;
};

template <typename T>
cudaError_t fast_plan(Problem& P, const ApplyArgs& aa, FastPlan<T>& pl) {
    using T2 = c_t<T>;
    fast::FastArgs& a = pl.a;
    a = fast::FastArgs{};
    a.nx = P.nx;
    a.ny = P.ny;
    a.nz = P.nz;
    a.nxh = P.nxh;
    a.rs = P.rs;
    a.nh = P.nh;
    a.nrows = P.nrows;
    a.n = P.n;
    a.plane = (long long)P.ny * P.rs;
    a.tw32x = P.px.tw32;
    a.tw32y = P.py.tw32;
    a.tw32z = P.pz.tw32;
    a.tw64x = P.px.tw64;
    a.tw64y = P.py.tw64;
    a.tw64z = P.pz.tw64;
    a.spec = P.d_spec;
    a.green = sizeof(T) == 8 ? (const void*)P.d_green64 : (const void*)P.d_green32;
    a.support = P.d_support;
    a.row_ptr = P.d_row_ptr;
    a.src = aa.src;
    a.src_sum = aa.src_sum;
    a.inv_nb = P.nb > 0 ? 1.0 / (double)P.nb : 0.0;
    a.dst = aa.dst;
    a.dot_with = aa.dot_with;
    a.scale = 1.0 / (double)P.n;
    a.partials = P.d_partials;
    a.skip = aa.skip;
    a.err = P.d_err;

    // x passes: tiles of `rows` grid rows, persistent over the tiles
    // grid rows per tile: the tuned cap when set (even), else about 192 threads
    int rows = P.x_rows > 0 ? std::max(2, P.x_rows & ~1) : fast::x_rows_for(P.nx);
    rows = std::min(rows, 2 * fast::kMaxXLines / 3);
    if (rows > P.nrows) rows = (int)((P.nrows + 1) & ~1LL);
    a.rows = rows;
    a.ntiles = (P.nrows + rows - 1) / rows;
    pl.xthreads = ((3 * rows / 2 * fast::x_tpl(P.nx) + 31) / 32) * 32;
    pl.xsmem = (size_t)(3 * rows / 2) * fast::x_ld_rt<T>(P.nx) * sizeof(T2);
    // inverse x: two stages, each the raw half-spectrum rows of a tile or,
    // after stage A, its padded lines
    const size_t raw = (size_t)3 * rows * P.rs * sizeof(T2);
    pl.stage_bytes = (int)((std::max(raw, pl.xsmem) + 15) & ~size_t(15));
    pl.xismem = 2 * (size_t)pl.stage_bytes;
    const int fwd_per_sm = fast::x_blocks_per_sm<T>(P.nx, false, pl.xthreads, pl.xsmem);
    const int inv_per_sm = fast::x_blocks_per_sm<T>(P.nx, true, pl.xthreads, pl.xismem);
    pl.xgrid_f = (int)std::min<long long>(a.ntiles, (long long)fwd_per_sm * P.sm_count);
    pl.xgrid_i = (int)std::min<long long>(a.ntiles, (long long)inv_per_sm * P.sm_count);
    pl.xgrid_i = std::min(pl.xgrid_i, kMaxPartials);

    // y passes: TX kx columns of one z plane and one component per CTA
    constexpr int TX = fast::col_tx<T>();
    const int ntx = (P.nxh + TX - 1) / TX;
    pl.ygrid = dim3(ntx, P.nz, 3);
    // z pass: persistent, TMA-fed, two pipeline stages per CTA
    constexpr int TZ = fast::z_tx<T>();
    if (!fast_maps(P, sizeof(T) == 8, TZ, &pl.smap, &pl.gmap)) return cudaErrorNotSupported;
    // the tuning flag of the register-capped y/z kernels selects here the
    // single-stage z pass (three CTAs per SM instead of one two-stage CTA)
    pl.zstages = P.yz_lowreg ? 1 : 2;
    pl.zsmem = fast::z_smem_rt<T>(P.nz, pl.zstages);
    const int ntz = (P.nxh + TZ - 1) / TZ;
    pl.zgrid = (int)std::min<long long>(
        (long long)ntz * P.ny,
        (long long)fast::z_blocks_per_sm<T>(P.nz, pl.zstages, pl.zsmem) * P.sm_count);
    return cudaSuccess;
}

// The five passes; `members` > 1 launches the group kernels (a.group set).
// Every member keeps its own grid: the x passes' partial sums are then those
// of a single apply, and the persistent z pass runs the members one after
// another (measured at 256^3: three members in 435 us against 3 x 142 us
// alone; splitting the resident CTAs among the members instead took 706 us).
template <typename T>
cudaError_t fast_run(const Problem& P, const FastPlan<T>& pl, const fast::FastArgs& a, int members) {
    const unsigned G = (unsigned)members;
    const int zgrid = pl.zgrid;
    cudaStream_t st = P.stream;
    cudaError_t e;
    if ((e = fast::run_xfwd<T>(P.nx, a, dim3(pl.xgrid_f, G), pl.xthreads, pl.xsmem, st)) != cudaSuccess)
        return e;
    const dim3 yg(pl.ygrid.x, pl.ygrid.y, 3 * G);
    if ((e = fast::run_y<T>(P.ny, -1, a, yg, st)) != cudaSuccess) return e;
    if (members > 1 && a.share == members && pl.zstages == 2)
        e = fast::run_z_shared<T>(P.nz, a, zgrid, pl.zsmem, st);
    else
        e = fast::run_z<T>(P.nz, pl.zstages, *pl.smap, *pl.gmap, a, dim3(zgrid, G), pl.zsmem, st);
    if (e != cudaSuccess) return e;
    if ((e = fast::run_y<T>(P.ny, +1, a, yg, st)) != cudaSuccess) return e;
    return fast::run_xinv<T>(P.nx, a, pl.stage_bytes, dim3(pl.xgrid_i, G), pl.xthreads, pl.xismem, st);
}

template <typename T>
cudaError_t fast_impl(Problem& P, const ApplyArgs& aa, int* nparts) {
    FastPlan<T> pl;
    cudaError_t e = fast_plan<T>(P, aa, pl);
    if (e != cudaSuccess) return e;
    if ((e = fast_run<T>(P, pl, pl.a, 1)) != cudaSuccess) return e;
    *nparts = pl.xgrid_i;
    return cudaSuccess;
}

template <typename T>
cudaError_t member_impl(Problem& P, const ApplyArgs& aa, fast::FastArgs* args, CUtensorMap* maps,
                        long long* geometry) {
    FastPlan<T> pl;
    cudaError_t e = fast_plan<T>(P, aa, pl);
    if (e != cudaSuccess) return e;
    *args = pl.a;
    maps[0] = *pl.smap;
    maps[1] = *pl.gmap;
    const long long g[kGroupGeometry] = {P.nx, P.ny, P.nz, pl.a.rows, pl.xthreads, pl.stage_bytes,
                                         pl.xgrid_f, pl.xgrid_i, pl.zstages, (long long)pl.zsmem,
                                         pl.zgrid, P.rs};
    for (int i = 0; i < kGroupGeometry; ++i) geometry[i] = g[i];
    return cudaSuccess;
}

template <typename T>
cudaError_t group_impl(Problem& P0, int members, const fast::FastArgs* d_args, const CUtensorMap* d_maps,
                       bool shared_green, int* nparts) {
    FastPlan<T> pl;
    ApplyArgs aa;
    cudaError_t e = fast_plan<T>(P0, aa, pl);
    if (e != cudaSuccess) return e;
    fast::FastArgs a = pl.a;
    a.group = d_args;
    a.group_maps = d_maps;
    a.share = shared_green ? members : 0;
    if ((e = fast_run<T>(P0, pl, a, members)) != cudaSuccess) return e;
    *nparts = pl.xgrid_i;
    return cudaSuccess;
}

}  // namespace

cudaError_t fast_apply(Problem& P, int precision, const ApplyArgs& aa, int* nparts) {
    if (precision == kFP64) return fast_impl<double>(P, aa, nparts);
    return fast_impl<float>(P, aa, nparts);
}

cudaError_t fast_member_args(Problem& P, int precision, const ApplyArgs& aa, fast::FastArgs* args,
                             CUtensorMap* maps, long long* geometry) {
    if (!fast_apply_supported(P, precision, aa.src_kind, aa.dst_kind, aa.stage))
        return cudaErrorNotSupported;
    if (precision == kFP64) return member_impl<double>(P, aa, args, maps, geometry);
    return member_impl<float>(P, aa, args, maps, geometry);
}

cudaError_t fast_apply_group(Problem& P0, int precision, int members, const fast::FastArgs* d_args,
                             const CUtensorMap* d_maps, bool shared_green, int* nparts) {
    if (precision == kFP64) return group_impl<double>(P0, members, d_args, d_maps, shared_green, nparts);
    return group_impl<float>(P0, members, d_args, d_maps, shared_green, nparts);
}

}  // namespace fp
