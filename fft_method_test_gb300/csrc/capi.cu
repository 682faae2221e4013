// capi.cu -- implementation of the C ABI declared in include/fftperm.h.
//
// Each entry point orchestrates device-resident state (internal.h) and the
// kernels of kernels_setup.cu, kernels_fft.cu and kernels_minres.cu.  Host
// buffers are copied in and out at the boundary; the solve paths keep every
// vector on the device between the copies.
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <new>
#include <set>
#include <shared_mutex>
#include <string>
#include <vector>

#include "../../include/fftperm.h"
#include "internal.h"

std::atomic<long long> fp::g_kernel_launches{0};
thread_local long long fp::g_thread_launches = 0;

namespace {
std::shared_mutex g_device_mem_mu;
thread_local int g_device_mem_depth = 0;
}  // namespace

fp::DeviceMemGuard::DeviceMemGuard() {
    if (g_device_mem_depth++ == 0) g_device_mem_mu.lock();
}
fp::DeviceMemGuard::~DeviceMemGuard() {
    if (--g_device_mem_depth == 0) g_device_mem_mu.unlock();
}
fp::CaptureGuard::CaptureGuard() { g_device_mem_mu.lock_shared(); }
fp::CaptureGuard::~CaptureGuard() { g_device_mem_mu.unlock_shared(); }

namespace {

// Pinned scalar blocks are reused across handles: cudaFreeHost synchronises
// the device, so handles hand their block back instead of freeing it.
std::mutex g_pinned_mu;
std::vector<fp::MinresScalars*> g_pinned_free;

fp::MinresScalars* take_pinned() {
    {
        std::lock_guard<std::mutex> lock(g_pinned_mu);
        if (!g_pinned_free.empty()) {
            fp::MinresScalars* p = g_pinned_free.back();
            g_pinned_free.pop_back();
            return p;
        }
    }
    fp::DeviceMemGuard mem_guard;
    void* p = nullptr;
    if (cudaMallocHost(&p, sizeof(fp::MinresScalars)) != cudaSuccess) return nullptr;
    return static_cast<fp::MinresScalars*>(p);
}

void give_pinned(fp::MinresScalars* p) {
    if (!p) return;
    std::lock_guard<std::mutex> lock(g_pinned_mu);
    g_pinned_free.push_back(p);
}

// Freed stream-ordered memory stays in the device's default pool for the
// next handle instead of going back to the driver at each synchronisation.
void keep_pool_memory(int dev) {
    static std::mutex mu;
    static std::set<int> done;
    std::lock_guard<std::mutex> lock(mu);
    if (done.count(dev)) return;
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
        uint64_t threshold = ~0ull;
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &threshold);
    }
    done.insert(dev);
}

}  // namespace

namespace {

using fp::Problem;

int fail(Problem& P, int code, const std::string& msg) {
    P.err = msg;
    return code;
}

int cuda_fail(Problem& P, cudaError_t e, const char* where) {
    P.err = std::string(where) + ": " + cudaGetErrorString(e);
    return FP_ERR_CUDA;
}

#define FP_CUDA(call, where)                          \
    do {                                              \
        cudaError_t e_ = (call);                      \
        if (e_ != cudaSuccess) return cuda_fail(P, e_, where); \
    } while (0)

// Device buffers of a handle are stream-ordered allocations on its stream:
// unlike cudaMalloc / cudaFree they do not synchronise the whole device, so
// handles on other streams (a batch) keep running through one handle's
// set-up and tear-down.
template <typename T>
cudaError_t dalloc(Problem& P, T** p, size_t count) {
    return cudaMallocAsync(reinterpret_cast<void**>(p), sizeof(T) * (count > 0 ? count : 1), P.stream);
}

void dfree(Problem& P, void* p) {
    if (p) cudaFreeAsync(p, P.stream);
}

void free_geometry(Problem& P) {
    fp::release_graphs(P);
    dfree(P, P.d_support);
    dfree(P, P.d_cin);
    dfree(P, P.d_cout);
    dfree(P, P.d_b);
    dfree(P, P.d_x);
    dfree(P, P.d_z);
    dfree(P, P.d_r0);
    dfree(P, P.d_corr);
    P.d_r0 = P.d_corr = nullptr;
    for (auto& v : P.d_v) dfree(P, v), v = nullptr;
    for (auto& w : P.d_w) dfree(P, w), w = nullptr;
    P.d_support = nullptr;
    P.d_cin = nullptr;
    P.d_cout = P.d_b = P.d_x = P.d_z = nullptr;
    P.has_geometry = false;
}

int need_geometry(Problem& P, const char* who) {
    if (!P.has_geometry)
        return fail(P, FP_ERR_STATE, std::string(who) + ": no geometry set (call fp_set_geometry)");
    if (P.nb == 0)
        return fail(P, FP_ERR_STATE, std::string(who) + ": support set is empty");
    return FP_OK;
}

// A TMA pass whose bounded wait gave up leaves the flag set: report it.
int check_device_error(Problem& P) {
    int e = 0;
    FP_CUDA(cudaMemcpyAsync(&e, P.d_err, sizeof(int), cudaMemcpyDeviceToHost, P.stream),
            "error flag copy");
    FP_CUDA(cudaStreamSynchronize(P.stream), "sync");
    if (e) return fail(P, FP_ERR_CUDA, "a TMA wait in an FFT pass timed out");
    return FP_OK;
}

int alloc_dense(Problem& P) {
    if (!P.d_dense_in) FP_CUDA(dalloc(P, &P.d_dense_in, 3 * (size_t)P.n), "cudaMalloc dense");
    if (!P.d_dense_out) FP_CUDA(dalloc(P, &P.d_dense_out, 3 * (size_t)P.n), "cudaMalloc dense");
    return FP_OK;
}

int ensure_green32(Problem& P) {
    if (P.d_green32) return FP_OK;
    FP_CUDA(dalloc(P, &P.d_green32, 6 * (size_t)P.nh), "cudaMalloc green32");
    FP_CUDA(fp::launch_green(P, nullptr, P.d_green32), "green precompute");
    return FP_OK;
}

int ensure_green64(Problem& P) {
    if (P.d_green64) return FP_OK;
    FP_CUDA(dalloc(P, &P.d_green64, 6 * (size_t)P.nh), "cudaMalloc green64");
    FP_CUDA(fp::launch_green(P, P.d_green64, nullptr), "green precompute");
    return FP_OK;
}

// Mixed mode needs both tables: FP32 for the Krylov applies, FP64 for the
// residuals that start and end each refinement segment.  One launch fills both.
int ensure_green_both(Problem& P) {
    if (P.d_green32 && P.d_green64) return FP_OK;
    if (P.d_green32) return ensure_green64(P);
    if (P.d_green64) return ensure_green32(P);
    FP_CUDA(dalloc(P, &P.d_green64, 6 * (size_t)P.nh), "cudaMalloc green64");
    FP_CUDA(dalloc(P, &P.d_green32, 6 * (size_t)P.nh), "cudaMalloc green32");
    FP_CUDA(fp::launch_green(P, P.d_green64, P.d_green32), "green precompute");
    return FP_OK;
}

// y = P_B A_raw P_B x on device compact vectors (src/bignonnet/VariationalOperator.cpp:19-41)
int device_operator_apply(Problem& P, const double* d_x, double* d_y) {
    FP_CUDA(fp::launch_sum3(P, d_x, P.nb, P.d_red), "sum");
    fp::ApplyArgs a;
    a.src = d_x;
    a.src_sum = P.d_red;
    a.dst = d_y;
    a.src_kind = fp::kSrcCompact;
    a.dst_kind = fp::kDstCompact;
    int nparts = 0;
    FP_CUDA(fp::launch_apply(P, a, &nparts), "apply");
    FP_CUDA(fp::launch_reduce4(P, nparts, P.d_red + 4), "reduce");
    FP_CUDA(fp::launch_sub_mean(P, d_y, P.d_red + 4, 1.0), "sub_mean");
    return FP_OK;
}

void f0_coefs(const Problem& P, const double g[3], double cf[3], double cs[3]) {
    // BackgroundForce.cpp:35-36: c_fluid = -1, c_support = -N_F / N_B
    const double c_support = -(double)P.nf / (double)P.nb;
    for (int c = 0; c < 3; ++c) {
        cf[c] = -1.0 * g[c];
        cs[c] = c_support * g[c];
    }
}

// b = -P_B gather(G * f0) on the device (src/bignonnet/VariationalRHS.cpp:15-31)
int device_build_rhs(Problem& P, const double g[3], double* d_b) {
    fp::ApplyArgs a;
    f0_coefs(P, g, a.f0_fluid, a.f0_support);
    a.dst = d_b;
    a.src_kind = fp::kSrcF0;
    a.dst_kind = fp::kDstCompact;
    int nparts = 0;
    FP_CUDA(fp::launch_apply(P, a, &nparts), "apply");
    FP_CUDA(fp::launch_reduce4(P, nparts, P.d_red + 4), "reduce");
    FP_CUDA(fp::launch_sub_mean(P, d_b, P.d_red + 4, -1.0), "sub_mean");
    return FP_OK;
}

// |b - A y| / rhs_norm, A applied at the given precision (kFP64 / kMixed).
int residual_norm(Problem& P, const double* d_b, const double* d_y, int precision, double rhs_norm,
                  double* rel) {
    FP_CUDA(fp::launch_sum3(P, d_y, P.nb, P.d_red), "sum");
    fp::ApplyArgs a;
    a.src = d_y;
    a.src_sum = P.d_red;
    a.dst = P.d_cout;
    a.src_kind = fp::kSrcCompact;
    a.dst_kind = fp::kDstCompact;
    a.precision = precision;
    int nparts = 0;
    FP_CUDA(fp::launch_apply(P, a, &nparts), "apply");
    FP_CUDA(fp::launch_reduce4(P, nparts, P.d_red + 4), "reduce");
    FP_CUDA(fp::launch_sub_mean(P, P.d_cout, P.d_red + 4, 1.0), "sub_mean");
    FP_CUDA(fp::launch_resnorm(P, d_b, P.d_cout, P.d_red + 12), "resnorm");
    double h[4];
    FP_CUDA(cudaMemcpyAsync(h, P.d_red + 12, sizeof(double) * 4, cudaMemcpyDeviceToHost, P.stream),
            "copy");
    FP_CUDA(cudaStreamSynchronize(P.stream), "sync");
    *rel = std::sqrt(h[3] > 0.0 ? h[3] : 0.0) / rhs_norm;
    return FP_OK;
}

int read_scalars(Problem& P) {
    FP_CUDA(cudaMemcpyAsync(P.h_sc, P.d_sc, sizeof(fp::MinresScalars), cudaMemcpyDeviceToHost,
                            P.stream),
            "copy");
    FP_CUDA(cudaStreamSynchronize(P.stream), "sync");
    return FP_OK;
}

// MINRES on device vectors (src/solver/MinresSolver.cpp:46-218); P.d_x
// receives the solution.  hist_host may be null.
//
// FP64 mode runs the reference's recurrence unchanged.
//
// Mixed mode (FP32 operator applies, FP64 Lanczos vectors and scalars) is
// MINRES inside mixed-precision iterative refinement.  Each segment starts
// from the current iterate x0 with the residual r0 = b - A x0 computed with
// the FP64 operator, and runs the reference recurrence on the FP32 operator.
// Every P.reliable_interval iterations the segment's own true residual
// |r0 - A32 (x - x0)| is recomputed (reliable update).  A segment ends when
// the recurrence reports convergence or breakdown, when that true residual is
// below tol, or when the recurrence estimate has run ahead of it (below
// P.ahead_factor = 0.95 of it).  The FP64 residual |b - A x| then decides:
// below tol the solve has converged, otherwise a new segment starts from x.  The reported
// residual is that FP64 residual; the history holds the last segment.
// State of one MINRES solve between chunks of iterations: device_minres runs
// one, group_minres runs several problems of one grid in lockstep.
struct MinresRun {
    Problem* P = nullptr;
    const double* d_b = nullptr;
    double tol = 0.0;
    long long maxit = 0;
    bool mixed = false;
    int chunk = 16;
    const double* seg_x0 = nullptr;  // null: the segment starts from zero
    long long done_its = 0;          // iterations of finished segments
    int restarts = 0;
    double rel64 = -1.0;
    bool converged64 = false;
    bool finished = false;
};

int minres_begin(MinresRun& r, Problem& P, const double* d_b, const double* d_x0, double tol,
                 long long maxit) {
    if (!(tol > 0.0)) return fail(P, FP_ERR_INVALID, "MinresSolver tolerance must be positive");
    if (maxit + 1 > P.hist_cap) {
        fp::release_graphs(P);  // the graphs write the history through the old pointer
        dfree(P, P.d_hist);
        P.d_hist = nullptr;
        FP_CUDA(dalloc(P, &P.d_hist, (size_t)maxit + 1), "cudaMalloc hist");
        P.hist_cap = maxit + 1;
    }
    r = MinresRun{};
    r.P = &P;
    r.d_b = d_b;
    r.tol = tol;
    r.maxit = maxit;
    r.mixed = P.precision == fp::kMixed && P.reliable_interval > 0;
    if (r.mixed) {
        int rc = ensure_green_both(P);
        if (rc) return rc;
    }
    const size_t bytes = sizeof(double) * 3 * (size_t)P.nb;
    // the first segment's r0 uses the FP64 operator in mixed mode
    FP_CUDA(fp::minres_start(P, d_b, d_x0, tol, maxit, r.mixed ? fp::kFP64 : -1), "minres_start");
    r.seg_x0 = d_x0;
    if (r.mixed) {
        FP_CUDA(cudaMemcpyAsync(P.d_r0, P.d_z, bytes, cudaMemcpyDeviceToDevice, P.stream), "copy");
        if (d_x0) {
            FP_CUDA(cudaMemcpyAsync(P.d_corr, d_x0, bytes, cudaMemcpyDeviceToDevice, P.stream),
                    "copy");
            r.seg_x0 = P.d_corr;  // keep the start point (d_x0 may alias P.d_cin)
        }
    }
    r.chunk = r.mixed ? P.reliable_interval : 16;
    return read_scalars(P);
}

// After a chunk of iterations (or none, once the recurrence is done): the
// mixed-mode segment test, FP64 residual and restart; sets r.finished.
int minres_step(MinresRun& r) {
    Problem& P = *r.P;
    constexpr int max_restarts = 20;
    if (!r.mixed) {
        if (P.h_sc->done) r.finished = true;
        return FP_OK;
    }
    const size_t bytes = sizeof(double) * 3 * (size_t)P.nb;
    const fp::MinresScalars s = *P.h_sc;
    const long long total = r.done_its + s.it;
    // the segment's true residual |r0 - A32 (x - x0)| / |b|
    double seg_rel = 0.0;
    if (!s.done || !s.converged) {
        const double* y = P.d_x;
        if (r.seg_x0) {
            FP_CUDA(fp::launch_axpby(P, P.d_cin, 1.0, P.d_x, -1.0, r.seg_x0), "diff");
            y = P.d_cin;
        }
        int rc = residual_norm(P, P.d_r0, y, fp::kMixed, s.rhs_norm, &seg_rel);
        if (rc) return rc;
    }
    const bool seg_end =
        s.done || seg_rel <= P.segment_tol_factor * r.tol || s.rel_res < P.ahead_factor * seg_rel;
    if (!seg_end) return FP_OK;
    int rc = residual_norm(P, r.d_b, P.d_x, fp::kFP64, s.rhs_norm, &r.rel64);
    if (rc) return rc;
    if (r.rel64 <= r.tol) {
        r.converged64 = true;
        r.finished = true;
        return FP_OK;
    }
    if (total >= r.maxit || r.restarts >= max_restarts) {
        r.finished = true;
        return FP_OK;
    }
    // next segment from the current iterate, r0 with the FP64 operator
    FP_CUDA(cudaMemcpyAsync(P.d_corr, P.d_x, bytes, cudaMemcpyDeviceToDevice, P.stream), "copy");
    r.seg_x0 = P.d_corr;
    r.done_its = total;
    ++r.restarts;
    FP_CUDA(fp::minres_start(P, r.d_b, P.d_corr, r.tol, r.maxit - total, fp::kFP64), "minres_start");
    FP_CUDA(cudaMemcpyAsync(P.d_r0, P.d_z, bytes, cudaMemcpyDeviceToDevice, P.stream), "copy");
    return read_scalars(P);
}

int minres_finish(MinresRun& r, double* hist_host, fp_solver_stats* st) {
    Problem& P = *r.P;
    const fp::MinresScalars s = *P.h_sc;
    {
        const int erc = check_device_error(P);
        if (erc) return erc;
    }
    if (hist_host) {
        FP_CUDA(cudaMemcpyAsync(hist_host, P.d_hist, sizeof(double) * (size_t)(s.it + 1),
                                cudaMemcpyDeviceToHost, P.stream),
                "hist copy");
        FP_CUDA(cudaStreamSynchronize(P.stream), "sync");
    }
    if (st) {
        st->iterations = r.done_its + s.it;
        if (r.mixed) {
            st->final_rel_residual = r.rel64;
            st->converged = r.converged64 ? 1 : 0;
        } else {
            st->final_rel_residual = s.rel_res;
            st->converged = s.converged ? 1 : (s.rel_res <= r.tol ? 1 : 0);
        }
        st->refinements = r.restarts;
    }
    return FP_OK;
}

int device_minres(Problem& P, const double* d_b, const double* d_x0, double tol, long long maxit,
                  double* hist_host, fp_solver_stats* st) {
    MinresRun r;
    int rc = minres_begin(r, P, d_b, d_x0, tol, maxit);
    if (rc) return rc;
    while (!r.finished) {
        if (!P.h_sc->done) {
            FP_CUDA(fp::minres_iterations(P, r.chunk), "minres_iteration");
            rc = read_scalars(P);
            if (rc) return rc;
        }
        rc = minres_step(r);
        if (rc) return rc;
    }
    return minres_finish(r, hist_host, st);
}

// Lockstep MINRES of the problems of runs (one grid, one stream): while two
// or more still iterate, each chunk runs through group_iterations (one launch
// per pass for all of them); a lone member takes the single path.  After each
// chunk every unfinished member runs its own segment logic.
int group_minres(std::vector<MinresRun>& runs, fp::GroupTables* tab) {
    for (;;) {
        std::vector<Problem*> act;
        bool any = false;
        int chunk = 0;
        for (auto& r : runs) {
            if (r.finished) continue;
            any = true;
            chunk = r.chunk;
            if (!r.P->h_sc->done) act.push_back(r.P);
        }
        if (!any) return FP_OK;
        if (act.size() == 1) {
            Problem& P = *act[0];
            FP_CUDA(fp::minres_iterations(P, chunk), "minres_iteration");
        } else if (act.size() > 1) {
            Problem& P = *act[0];
            FP_CUDA(fp::group_iterations(act.data(), (int)act.size(), chunk, tab), "group iteration");
        }
        for (Problem* m : act) {
            int rc = read_scalars(*m);
            if (rc) return rc;
        }
        for (auto& r : runs) {
            if (r.finished) continue;
            int rc = minres_step(r);
            if (rc) return rc;
        }
    }
}

// v = G*(f0 + P_B x) - mean_B(...), avg = <v> over the domain
// (src/bignonnet/VelocityRecovery.cpp:12-51).  Leaves U + V' in P.d_dense_out.
int device_recover(Problem& P, const double g[3], const double* d_x, double avg[3], bool keep_field) {
    int rc = alloc_dense(P);
    if (rc) return rc;
    FP_CUDA(fp::launch_sum3(P, d_x, P.nb, P.d_red), "sum");
    fp::ApplyArgs a;
    f0_coefs(P, g, a.f0_fluid, a.f0_support);
    a.src = d_x;
    a.src_sum = P.d_red;
    a.dst = P.d_dense_out;
    a.src_kind = fp::kSrcF0Compact;
    a.dst_kind = fp::kDstDense;
    int nparts = 0;
    FP_CUDA(fp::launch_apply(P, a, &nparts), "apply");
    FP_CUDA(fp::launch_reduce4(P, nparts, P.d_red + 4), "reduce");  // sums over all voxels
    FP_CUDA(fp::launch_gather_sum(P, P.d_dense_out, P.d_red + 8), "gather_sum");
    double h[12];
    FP_CUDA(cudaMemcpyAsync(h, P.d_red, sizeof(double) * 12, cudaMemcpyDeviceToHost, P.stream),
            "copy");
    FP_CUDA(cudaStreamSynchronize(P.stream), "sync");
    double vprime[3];
    for (int c = 0; c < 3; ++c) {
        vprime[c] = -(h[8 + c] / (double)P.nb);
        avg[c] = (h[4 + c] + (double)P.n * vprime[c]) / (double)P.n;
    }
    if (keep_field) {
        double* d_add = P.d_red + 16;
        FP_CUDA(cudaMemcpyAsync(d_add, vprime, sizeof(double) * 3, cudaMemcpyHostToDevice, P.stream),
                "copy");
        FP_CUDA(fp::launch_add_const3(P, P.d_dense_out, d_add), "add");
        FP_CUDA(cudaStreamSynchronize(P.stream), "sync");
    }
    return FP_OK;
}

int finish_geometry(Problem& P, int64_t* nb_out);

double now_s() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch())
        .count();
}

}  // namespace

extern "C" {

int fp_create(int nx, int ny, int nz, double voxel_size, double mu, int p_radius, int precision,
              fp_handle* out) {
    return fp::create_handle(nx, ny, nz, voxel_size, mu, p_radius, precision, true, out);
}

}  // extern "C"

int fp::create_handle(int nx, int ny, int nz, double voxel_size, double mu, int p_radius,
                      int precision, bool with_green, fp_handle* out) {
    if (!out) return FP_ERR_INVALID;
    *out = nullptr;
    fp_problem* h = new (std::nothrow) fp_problem();
    if (!h) return FP_ERR_NOMEM;
    Problem& P = h->P;
    *out = h;
    if (nx <= 0 || ny <= 0 || nz <= 0)
        return fail(P, FP_ERR_INVALID, "Grid dimensions must be positive");
    if (!(mu > 0.0)) return fail(P, FP_ERR_INVALID, "GreenOperator viscosity must be positive");
    if (!(voxel_size > 0.0)) return fail(P, FP_ERR_INVALID, "voxel size must be positive");
    if (precision != FP_PREC_FP64 && precision != FP_PREC_MIXED)
        return fail(P, FP_ERR_INVALID, "unknown precision mode");
    P.nx = nx;
    P.ny = ny;
    P.nz = nz;
    P.n = (long long)nx * ny * nz;
    P.nxh = nx / 2 + 1;
    P.nrows = (long long)ny * nz;
    // a multiple of 4 elements: every FP32 Green row and FP32/FP64 spectral
    // row starts 16-byte aligned (TMA tensor maps need 16-byte strides)
    P.rs = (P.nxh + 3) & ~3LL;
    P.nh = P.rs * P.nrows;
    P.h = voxel_size;
    P.mu = mu;
    P.p_radius = p_radius < 0 ? 0 : p_radius;
    P.precision = precision;
    if (P.n > 2147483647LL) return fail(P, FP_ERR_INVALID, "grid too large (N must fit in int32)");
    int dev = 0;
    FP_CUDA(cudaGetDevice(&dev), "cudaGetDevice");
    FP_CUDA(cudaDeviceGetAttribute(&P.sm_count, cudaDevAttrMultiProcessorCount, dev), "attr");
    FP_CUDA(cudaStreamCreateWithFlags(&P.stream, cudaStreamNonBlocking), "stream");
    keep_pool_memory(dev);
    if (const char* t = std::getenv("FFTPERM_TILE_YZ")) P.tile_yz = std::atoi(t);
    if (const char* t = std::getenv("FFTPERM_NO_TMA")) {
        P.tma_off = std::atoi(t) != 0;  // every TMA / bulk-copy pass off
        P.x_bulk = !P.tma_off;
    }
    if (const char* t = std::getenv("FFTPERM_NO_GRAPHS")) P.use_graphs = std::atoi(t) == 0;
    if (const char* t = std::getenv("FFTPERM_NO_FAST")) P.fast_off = std::atoi(t) != 0;
    if (const char* t = std::getenv("FFTPERM_RELIABLE")) {
        const int k = std::atoi(t);
        if (k > 0) P.reliable_interval = k;
    }
    if (const char* t = std::getenv("FFTPERM_AHEAD")) {
        const double f = std::atof(t);
        if (f > 0.0 && f < 1.0) P.ahead_factor = f;
    }
    if (const char* t = std::getenv("FFTPERM_SEGMENT_TOL")) {
        const double f = std::atof(t);
        if (f > 0.0 && f <= 1.0) P.segment_tol_factor = f;
    }
    std::string err;
    if (!fp::make_axis_plan(nx, P.px, err, P.stream) || !fp::make_axis_plan(ny, P.py, err, P.stream) ||
        !fp::make_axis_plan(nz, P.pz, err, P.stream))
        return fail(P, FP_ERR_UNSUPPORTED, err);
    FP_CUDA(dalloc(P, reinterpret_cast<double2**>(&P.d_spec), 3 * (size_t)P.nh), "cudaMalloc spec");
    const size_t nparts = (size_t)std::max<long long>(fp::kMaxPartials, P.nrows + 64);
    FP_CUDA(dalloc(P, &P.d_partials, 4 * nparts), "cudaMalloc partials");
    FP_CUDA(dalloc(P, &P.d_red, 64), "cudaMalloc red");
    FP_CUDA(cudaMemsetAsync(P.d_red, 0, sizeof(double) * 64, P.stream), "memset red");
    FP_CUDA(dalloc(P, &P.d_sc, 1), "cudaMalloc scalars");
    FP_CUDA(dalloc(P, &P.d_err, 1), "cudaMalloc error flag");
    FP_CUDA(cudaMemsetAsync(P.d_err, 0, sizeof(int), P.stream), "memset");
    P.h_sc = take_pinned();
    if (!P.h_sc) return fail(P, FP_ERR_NOMEM, "cudaMallocHost failed");
    FP_CUDA(dalloc(P, &P.d_row_ptr, (size_t)P.nrows + 1), "cudaMalloc row_ptr");
    FP_CUDA(dalloc(P, &P.d_row_cnt, (size_t)P.nrows + 1), "cudaMalloc row_cnt");
    FP_CUDA(dalloc(P, &P.d_mask, (size_t)P.n), "cudaMalloc mask");
    if (!with_green) return FP_OK;
    int rc = (precision == FP_PREC_MIXED) ? ensure_green_both(P) : ensure_green64(P);
    if (rc) return rc;
    return FP_OK;
}

extern "C" {

int fp_destroy(fp_handle h) {
    if (!h) return FP_OK;
    Problem& P = h->P;
    if (P.stream) cudaStreamSynchronize(P.stream);
    free_geometry(P);
    fp::free_axis_plan(P.px, P.stream);
    fp::free_axis_plan(P.py, P.stream);
    fp::free_axis_plan(P.pz, P.stream);
    dfree(P, P.d_spec);
    dfree(P, P.d_green64);
    dfree(P, P.d_green32);
    dfree(P, P.d_dense_in);
    dfree(P, P.d_dense_out);
    dfree(P, P.d_partials);
    dfree(P, P.d_red);
    dfree(P, P.d_sc);
    dfree(P, P.d_err);
    dfree(P, P.d_hist);
    dfree(P, P.d_row_ptr);
    dfree(P, P.d_row_cnt);
    dfree(P, P.d_mask);
    give_pinned(P.h_sc);
    P.h_sc = nullptr;
    if (P.stream) cudaStreamDestroy(P.stream);
    delete h;
    return FP_OK;
}

const char* fp_last_error(fp_handle h) { return h ? h->P.err.c_str() : "null handle"; }

void* fp_stream(fp_handle h) { return h ? (void*)h->P.stream : nullptr; }

long long fp_kernel_launch_count(void) {
    return fp::g_kernel_launches.load(std::memory_order_relaxed);
}

int fp_synchronize(fp_handle h) {
    if (!h) return FP_ERR_INVALID;
    Problem& P = h->P;
    FP_CUDA(cudaStreamSynchronize(P.stream), "cudaStreamSynchronize");
    return check_device_error(P);
}

int fp_set_precision(fp_handle h, int precision) {
    if (!h) return FP_ERR_INVALID;
    Problem& P = h->P;
    if (precision != FP_PREC_FP64 && precision != FP_PREC_MIXED)
        return fail(P, FP_ERR_INVALID, "unknown precision mode");
    int rc = (precision == FP_PREC_MIXED) ? ensure_green_both(P) : ensure_green64(P);
    if (rc) return rc;
    if (precision != P.precision) fp::release_graphs(P);
    P.precision = precision;
    return FP_OK;
}

int fp_set_geometry(fp_handle h, const uint8_t* fluid_mask, int support_mode, int64_t* nb_out) {
    if (!h) return FP_ERR_INVALID;
    Problem& P = h->P;
    if (!fluid_mask) return fail(P, FP_ERR_INVALID, "BinaryMedium mask must not be null");
    if (support_mode != FP_SUPPORT_INTERFACE && support_mode != FP_SUPPORT_FULLSOLID)
        return fail(P, FP_ERR_INVALID, "unknown support mode");
    free_geometry(P);
    P.support_mode = support_mode;
    FP_CUDA(cudaMemcpyAsync(P.d_mask, fluid_mask, (size_t)P.n, cudaMemcpyHostToDevice, P.stream),
            "mask copy");
    return finish_geometry(P, nb_out);
}

int fp_load_fgeo(fp_handle h, const char* path, uint32_t fluid_id, int support_mode,
                 int64_t* nb_out) {
    if (!h) return FP_ERR_INVALID;
    Problem& P = h->P;
    if (!path) return fail(P, FP_ERR_INVALID, "VoxelIO: path must not be null");
    if (support_mode != FP_SUPPORT_INTERFACE && support_mode != FP_SUPPORT_FULLSOLID)
        return fail(P, FP_ERR_INVALID, "unknown support mode");
    std::FILE* f = std::fopen(path, "rb");
    if (!f) return fail(P, FP_ERR_INVALID, std::string("VoxelIO: cannot open ") + path);
    unsigned char head[32];
    const bool got = std::fread(head, 1, 32, f) == 32;
    if (!got || std::memcmp(head, "FGEO", 4) != 0) {
        std::fclose(f);
        return fail(P, FP_ERR_INVALID, std::string("VoxelIO: invalid .fgeo magic: ") + path);
    }
    if (head[4] != 1 || (head[5] != 1 && head[5] != 2)) {
        std::fclose(f);
        return fail(P, FP_ERR_INVALID, "VoxelIO: unsupported .fgeo version or value type");
    }
    uint64_t dims[3];
    std::memcpy(dims, head + 8, 24);
    if (dims[0] != (uint64_t)P.nx || dims[1] != (uint64_t)P.ny || dims[2] != (uint64_t)P.nz) {
        std::fclose(f);
        return fail(P, FP_ERR_INVALID, "VoxelIO: .fgeo dimensions differ from the grid");
    }
    const int esz = head[5] == 1 ? 4 : 2;
    free_geometry(P);
    P.support_mode = support_mode;
    // the ids stream to the device in chunks; the mask is formed there
    const long long chunk = 1LL << 24;
    void* d_ids = nullptr;
    {
        const cudaError_t e = dalloc(P, reinterpret_cast<unsigned char**>(&d_ids),
                                     (size_t)std::min<long long>(chunk, P.n) * esz);
        if (e != cudaSuccess) {
            std::fclose(f);
            return cuda_fail(P, e, "cudaMalloc ids");
        }
    }
    std::vector<unsigned char> host((size_t)std::min<long long>(chunk, P.n) * esz);
    int rc = FP_OK;
    for (long long i0 = 0; i0 < P.n && rc == FP_OK; i0 += chunk) {
        const long long m = std::min<long long>(chunk, P.n - i0);
        if (std::fread(host.data(), esz, (size_t)m, f) != (size_t)m) {
            rc = fail(P, FP_ERR_INVALID, "VoxelIO: .fgeo payload is truncated");
            break;
        }
        cudaError_t e = cudaMemcpyAsync(d_ids, host.data(), (size_t)m * esz, cudaMemcpyHostToDevice,
                                        P.stream);
        if (e == cudaSuccess) e = fp::launch_ids_to_mask(d_ids, esz, m, fluid_id, P.d_mask + i0, P.stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(P.stream);  // host buffer reused
        if (e != cudaSuccess) rc = cuda_fail(P, e, "ids to mask");
    }
    std::fclose(f);
    dfree(P, d_ids);
    if (rc != FP_OK) return rc;
    return finish_geometry(P, nb_out);
}

int fp_recover_fvel(fp_handle h, const char* path, const double grad[3], const double* x,
                    double porosity, double viscosity) {
    if (!h || !path || !grad || !x) return FP_ERR_INVALID;
    Problem& P = h->P;
    int rc = need_geometry(P, "VelocityRecovery::recover");
    if (rc) return rc;
    const size_t m = 3 * (size_t)P.nb;
    FP_CUDA(cudaMemcpyAsync(P.d_cin, x, sizeof(double) * m, cudaMemcpyHostToDevice, P.stream), "copy");
    double avg[3];
    rc = device_recover(P, grad, P.d_cin, avg, true);
    if (rc) return rc;
    std::FILE* f = std::fopen(path, "wb");
    if (!f) return fail(P, FP_ERR_INVALID, std::string("cannot write velocity file: ") + path);
    bool ok = fp::write_fvel_header(f, P.nx, P.ny, P.nz, porosity, viscosity, grad);
    // the field leaves the device one chunk per component at a time
    const long long chunk = 1LL << 20;
    std::vector<double> comp(3 * (size_t)std::min<long long>(chunk, P.n)), rec(comp.size());
    for (long long i0 = 0; ok && i0 < P.n; i0 += chunk) {
        const long long k = std::min<long long>(chunk, P.n - i0);
        for (int c = 0; c < 3; ++c)
            FP_CUDA(cudaMemcpyAsync(comp.data() + (size_t)c * k, P.d_dense_out + (size_t)c * P.n + i0,
                                    sizeof(double) * k, cudaMemcpyDeviceToHost, P.stream),
                    "copy");
        FP_CUDA(cudaStreamSynchronize(P.stream), "sync");
        for (long long i = 0; i < k; ++i)
            for (int c = 0; c < 3; ++c) rec[3 * i + c] = comp[(size_t)c * k + i];
        ok = std::fwrite(rec.data(), sizeof(double), 3 * (size_t)k, f) == 3 * (size_t)k;
    }
    ok = (std::fclose(f) == 0) && ok;
    return ok ? FP_OK : fail(P, FP_ERR_INVALID, std::string("cannot write velocity file: ") + path);
}

}  // extern "C"

namespace {

int finish_geometry(Problem& P, int64_t* nb_out) {
    FP_CUDA(fp::launch_support(P), "support");
    const size_t m = 3 * (size_t)P.nb;
    FP_CUDA(dalloc(P, &P.d_cin, m), "cudaMalloc");
    FP_CUDA(dalloc(P, &P.d_cout, m), "cudaMalloc");
    FP_CUDA(dalloc(P, &P.d_b, m), "cudaMalloc");
    FP_CUDA(dalloc(P, &P.d_x, m), "cudaMalloc");
    FP_CUDA(dalloc(P, &P.d_z, m), "cudaMalloc");
    FP_CUDA(dalloc(P, &P.d_r0, m), "cudaMalloc");
    FP_CUDA(dalloc(P, &P.d_corr, m), "cudaMalloc");
    for (auto& v : P.d_v) FP_CUDA(dalloc(P, &v, m), "cudaMalloc");
    for (auto& w : P.d_w) FP_CUDA(dalloc(P, &w, m), "cudaMalloc");
    FP_CUDA(cudaStreamSynchronize(P.stream), "sync");
    P.has_geometry = true;
    if (nb_out) *nb_out = P.nb;
    return FP_OK;
}

}  // namespace

extern "C" {

int fp_get_support(fp_handle h, int64_t* out) {
    if (!h || !out) return FP_ERR_INVALID;
    Problem& P = h->P;
    if (!P.has_geometry) return fail(P, FP_ERR_STATE, "fp_get_support: no geometry set");
    std::vector<int> tmp((size_t)P.nb);
    FP_CUDA(cudaMemcpyAsync(tmp.data(), P.d_support, sizeof(int) * tmp.size(), cudaMemcpyDeviceToHost,
                            P.stream),
            "copy");
    FP_CUDA(cudaStreamSynchronize(P.stream), "sync");
    for (size_t i = 0; i < tmp.size(); ++i) out[i] = tmp[i];
    return FP_OK;
}

int fp_get_green(fp_handle h, double* g6) {
    if (!h || !g6) return FP_ERR_INVALID;
    Problem& P = h->P;
    int rc = ensure_green64(P);
    if (rc) return rc;
    FP_CUDA(cudaMemcpy2DAsync(g6, sizeof(double) * P.nxh, P.d_green64, sizeof(double) * P.rs,
                              sizeof(double) * P.nxh, 6 * (size_t)P.nrows, cudaMemcpyDeviceToHost,
                              P.stream),
            "copy");
    FP_CUDA(cudaStreamSynchronize(P.stream), "sync");
    return FP_OK;
}

int fp_green_apply(fp_handle h, const double* force_soa, double* velocity_soa) {
    if (!h || !force_soa || !velocity_soa) return FP_ERR_INVALID;
    Problem& P = h->P;
    int rc = alloc_dense(P);
    if (rc) return rc;
    FP_CUDA(cudaMemcpyAsync(P.d_dense_in, force_soa, sizeof(double) * 3 * (size_t)P.n,
                            cudaMemcpyHostToDevice, P.stream),
            "copy");
    fp::ApplyArgs a;
    a.src = P.d_dense_in;
    a.dst = P.d_dense_out;
    a.src_kind = fp::kSrcDense;
    a.dst_kind = fp::kDstDense;
    int nparts = 0;
    FP_CUDA(fp::launch_apply(P, a, &nparts), "apply");
    FP_CUDA(cudaMemcpyAsync(velocity_soa, P.d_dense_out, sizeof(double) * 3 * (size_t)P.n,
                            cudaMemcpyDeviceToHost, P.stream),
            "copy");
    FP_CUDA(cudaStreamSynchronize(P.stream), "sync");
    return FP_OK;
}

int fp_fft_forward(fp_handle h, const double* real_soa, double* half_spectrum) {
    if (!h || !real_soa || !half_spectrum) return FP_ERR_INVALID;
    Problem& P = h->P;
    int rc = alloc_dense(P);
    if (rc) return rc;
    FP_CUDA(cudaMemcpyAsync(P.d_dense_in, real_soa, sizeof(double) * 3 * (size_t)P.n,
                            cudaMemcpyHostToDevice, P.stream),
            "copy");
    fp::ApplyArgs a;
    a.src = P.d_dense_in;
    a.src_kind = fp::kSrcDense;
    a.stage = fp::kStageForward;
    a.precision = fp::kFP64;
    int nparts = 0;
    FP_CUDA(fp::launch_apply(P, a, &nparts), "forward fft");
    FP_CUDA(cudaMemcpy2DAsync(half_spectrum, sizeof(double2) * P.nxh, P.d_spec, sizeof(double2) * P.rs,
                              sizeof(double2) * P.nxh, 3 * (size_t)P.nrows, cudaMemcpyDeviceToHost,
                              P.stream),
            "copy");
    FP_CUDA(cudaStreamSynchronize(P.stream), "sync");
    return FP_OK;
}

int fp_fft_inverse(fp_handle h, const double* half_spectrum, double* real_soa) {
    if (!h || !real_soa || !half_spectrum) return FP_ERR_INVALID;
    Problem& P = h->P;
    int rc = alloc_dense(P);
    if (rc) return rc;
    FP_CUDA(cudaMemcpy2DAsync(P.d_spec, sizeof(double2) * P.rs, half_spectrum, sizeof(double2) * P.nxh,
                              sizeof(double2) * P.nxh, 3 * (size_t)P.nrows, cudaMemcpyHostToDevice,
                              P.stream),
            "copy");
    fp::ApplyArgs a;
    a.dst = P.d_dense_out;
    a.dst_kind = fp::kDstDense;
    a.stage = fp::kStageInverse;
    a.precision = fp::kFP64;
    int nparts = 0;
    FP_CUDA(fp::launch_apply(P, a, &nparts), "inverse fft");
    FP_CUDA(cudaMemcpyAsync(real_soa, P.d_dense_out, sizeof(double) * 3 * (size_t)P.n,
                            cudaMemcpyDeviceToHost, P.stream),
            "copy");
    FP_CUDA(cudaStreamSynchronize(P.stream), "sync");
    return FP_OK;
}

int fp_background_force(fp_handle h, const double grad[3], double* f0_soa) {
    if (!h || !grad || !f0_soa) return FP_ERR_INVALID;
    Problem& P = h->P;
    int rc = need_geometry(P, "fp_background_force");
    if (rc) return rc;
    rc = alloc_dense(P);
    if (rc) return rc;
    double cf[3], cs[3];
    f0_coefs(P, grad, cf, cs);
    FP_CUDA(fp::launch_background_force(P, cf, cs, P.d_dense_out), "f0");
    FP_CUDA(cudaMemcpyAsync(f0_soa, P.d_dense_out, sizeof(double) * 3 * (size_t)P.n,
                            cudaMemcpyDeviceToHost, P.stream),
            "copy");
    FP_CUDA(cudaStreamSynchronize(P.stream), "sync");
    return FP_OK;
}

int fp_operator_apply(fp_handle h, const double* x, double* y) {
    if (!h || !x || !y) return FP_ERR_INVALID;
    Problem& P = h->P;
    int rc = need_geometry(P, "VariationalOperator::apply");
    if (rc) return rc;
    const size_t bytes = sizeof(double) * 3 * (size_t)P.nb;
    FP_CUDA(cudaMemcpyAsync(P.d_cin, x, bytes, cudaMemcpyHostToDevice, P.stream), "copy");
    rc = device_operator_apply(P, P.d_cin, P.d_cout);
    if (rc) return rc;
    FP_CUDA(cudaMemcpyAsync(y, P.d_cout, bytes, cudaMemcpyDeviceToHost, P.stream), "copy");
    FP_CUDA(cudaStreamSynchronize(P.stream), "sync");
    return check_device_error(P);
}

int fp_operator_apply_device(fp_handle h, const double* d_x, double* d_y) {
    if (!h || !d_x || !d_y) return FP_ERR_INVALID;
    Problem& P = h->P;
    // the vector kernels read two voxels (three double2) per thread
    if ((reinterpret_cast<uintptr_t>(d_x) | reinterpret_cast<uintptr_t>(d_y)) & 15)
        return fail(P, FP_ERR_INVALID, "VariationalOperator::apply: device vectors must be 16-byte aligned");
    int rc = need_geometry(P, "VariationalOperator::apply");
    if (rc) return rc;
    return device_operator_apply(P, d_x, d_y);
}

int fp_build_rhs(fp_handle h, const double grad[3], double* b) {
    if (!h || !grad || !b) return FP_ERR_INVALID;
    Problem& P = h->P;
    int rc = need_geometry(P, "VariationalRHS::build");
    if (rc) return rc;
    rc = device_build_rhs(P, grad, P.d_b);
    if (rc) return rc;
    FP_CUDA(cudaMemcpyAsync(b, P.d_b, sizeof(double) * 3 * (size_t)P.nb, cudaMemcpyDeviceToHost,
                            P.stream),
            "copy");
    FP_CUDA(cudaStreamSynchronize(P.stream), "sync");
    return FP_OK;
}

int fp_minres(fp_handle h, const double* b, const double* x0, double tol, int64_t maxit,
              double* x, double* hist, fp_solver_stats* stats) {
    if (!h || !b || !x) return FP_ERR_INVALID;
    Problem& P = h->P;
    int rc = need_geometry(P, "MinresSolver::solve");
    if (rc) return rc;
    if (maxit < 0) return fail(P, FP_ERR_INVALID, "max_iterations must be non-negative");
    const double t0 = now_s();
    const size_t bytes = sizeof(double) * 3 * (size_t)P.nb;
    FP_CUDA(cudaMemcpyAsync(P.d_b, b, bytes, cudaMemcpyHostToDevice, P.stream), "copy");
    if (x0) FP_CUDA(cudaMemcpyAsync(P.d_cin, x0, bytes, cudaMemcpyHostToDevice, P.stream), "copy");
    rc = device_minres(P, P.d_b, x0 ? P.d_cin : nullptr, tol, maxit, hist, stats);
    if (rc) return rc;
    FP_CUDA(cudaMemcpyAsync(x, P.d_x, bytes, cudaMemcpyDeviceToHost, P.stream), "copy");
    FP_CUDA(cudaStreamSynchronize(P.stream), "sync");
    if (stats) stats->seconds = now_s() - t0;
    return FP_OK;
}

int fp_recover(fp_handle h, const double grad[3], const double* x, double* v_soa, double avg[3]) {
    if (!h || !grad || !x || !avg) return FP_ERR_INVALID;
    Problem& P = h->P;
    int rc = need_geometry(P, "VelocityRecovery::recover");
    if (rc) return rc;
    FP_CUDA(cudaMemcpyAsync(P.d_cin, x, sizeof(double) * 3 * (size_t)P.nb, cudaMemcpyHostToDevice,
                            P.stream),
            "copy");
    rc = device_recover(P, grad, P.d_cin, avg, v_soa != nullptr);
    if (rc) return rc;
    if (v_soa) {
        FP_CUDA(cudaMemcpyAsync(v_soa, P.d_dense_out, sizeof(double) * 3 * (size_t)P.n,
                                cudaMemcpyDeviceToHost, P.stream),
                "copy");
        FP_CUDA(cudaStreamSynchronize(P.stream), "sync");
    }
    return FP_OK;
}

int fp_solve_load_case(fp_handle h, const double grad[3], const double* x0, double tol,
                       int64_t maxit, double avg[3], double* x_out, fp_solver_stats* stats) {
    if (!h || !grad || !avg) return FP_ERR_INVALID;
    Problem& P = h->P;
    int rc = need_geometry(P, "solve_one_direction");
    if (rc) return rc;
    const double t0 = now_s();
    const size_t bytes = sizeof(double) * 3 * (size_t)P.nb;
    if (x0) FP_CUDA(cudaMemcpyAsync(P.d_cin, x0, bytes, cudaMemcpyHostToDevice, P.stream), "copy");
    rc = device_build_rhs(P, grad, P.d_b);
    if (rc) return rc;
    fp_solver_stats st{};
    rc = device_minres(P, P.d_b, x0 ? P.d_cin : nullptr, tol, maxit, nullptr, &st);
    if (rc) return rc;
    rc = device_recover(P, grad, P.d_x, avg, false);
    if (rc) return rc;
    if (x_out) {
        FP_CUDA(cudaMemcpyAsync(x_out, P.d_x, bytes, cudaMemcpyDeviceToHost, P.stream), "copy");
        FP_CUDA(cudaStreamSynchronize(P.stream), "sync");
    }
    st.seconds = now_s() - t0;
    if (stats) *stats = st;
    return FP_OK;
}

int fp_solve_permeability(fp_handle h, double tol, int64_t maxit, double K[9],
                          fp_solver_stats stats[3]) {
    if (!h || !K) return FP_ERR_INVALID;
    Problem& P = h->P;
    int rc = need_geometry(P, "PermeabilityRunner::run");
    if (rc) return rc;
    for (int col = 0; col < 3; ++col) {
        double g[3] = {0.0, 0.0, 0.0};
        g[col] = 1.0;
        double avg[3];
        fp_solver_stats st{};
        rc = fp_solve_load_case(h, g, nullptr, tol, maxit, avg, nullptr, &st);
        if (rc) return rc;
        // colK = -mu <v>; set_column stores -colK (PermeabilityRunner.cpp:772-777,
        // PermeabilityTensor.cpp:16)
        for (int row = 0; row < 3; ++row) K[row * 3 + col] = -(-P.mu * avg[row]);
        if (stats) stats[col] = st;
    }
    return FP_OK;
}

}  // extern "C"

namespace {

// Member i solves load case cols[i] (unit gradient e_col); the members run
// on handles[0]'s stream and iterate in lockstep (group_minres).  avg[i] is
// the member's domain-averaged velocity, st[i] its solver statistics.
int group_solve_cases(int count, fp_handle* handles, const int* cols, double tol, long long maxit,
                      double (*avg)[3], fp_solver_stats* st) {
    Problem& P0 = handles[0]->P;
    std::vector<cudaStream_t> own((size_t)count);
    for (int i = 0; i < count; ++i) {
        Problem& P = handles[i]->P;
        own[(size_t)i] = P.stream;
        FP_CUDA(cudaStreamSynchronize(P.stream), "sync");
        P.stream = P0.stream;
    }
    fp::GroupTables* tab = nullptr;
    auto restore = [&](int rc) {
        cudaStreamSynchronize(P0.stream);
        for (int i = 0; i < count; ++i) handles[i]->P.stream = own[(size_t)i];
        fp::group_tables_destroy(tab);
        return rc;
    };
    const int chunk = P0.precision == fp::kMixed && P0.reliable_interval > 0 ? P0.reliable_interval : 16;
    {
        cudaError_t e = fp::group_tables_create(&tab, count, chunk);
        if (e != cudaSuccess) return restore(cuda_fail(P0, e, "group tables"));
    }
    const double t0 = now_s();
    std::vector<MinresRun> runs((size_t)count);
    for (int i = 0; i < count; ++i) {
        Problem& P = handles[i]->P;
        double g[3] = {0.0, 0.0, 0.0};
        g[cols[i]] = 1.0;
        int rc = device_build_rhs(P, g, P.d_b);
        if (!rc) rc = minres_begin(runs[(size_t)i], P, P.d_b, nullptr, tol, maxit);
        if (rc) return restore(rc);
    }
    int rc = group_minres(runs, tab);
    if (rc) return restore(rc);
    for (int i = 0; i < count; ++i) {
        Problem& P = handles[i]->P;
        double g[3] = {0.0, 0.0, 0.0};
        g[cols[i]] = 1.0;
        st[i] = fp_solver_stats{};
        rc = minres_finish(runs[(size_t)i], nullptr, &st[i]);
        if (!rc) rc = device_recover(P, g, P.d_x, avg[i], false);
        if (rc) return restore(rc);
        st[i].seconds = now_s() - t0;
    }
    return restore(FP_OK);
}

// colK = -mu <v>; set_column stores -colK (PermeabilityRunner.cpp:772-777,
// PermeabilityTensor.cpp:16)
void set_column(double* K, int col, double mu, const double avg[3]) {
    for (int row = 0; row < 3; ++row) K[row * 3 + col] = -(-mu * avg[row]);
}

}  // namespace

extern "C" {

int fp_group_solve_permeability(int count, fp_handle* handles, double tol, int64_t maxit, double* K,
                                fp_solver_stats* stats) {
    if (count < 1 || !handles || !K) return FP_ERR_INVALID;
    for (int i = 0; i < count; ++i)
        if (!handles[i]) return FP_ERR_INVALID;
    Problem& P0 = handles[0]->P;
    for (int i = 0; i < count; ++i) {
        Problem& P = handles[i]->P;
        int rc = need_geometry(P, "PermeabilityRunner::run");
        if (rc) return rc;
        if (P.nx != P0.nx || P.ny != P0.ny || P.nz != P0.nz || P.precision != P0.precision ||
            P.reliable_interval != P0.reliable_interval)
            return fail(P, FP_ERR_INVALID, "group: members must share grid, precision and reliable interval");
        if (P.tile_yz != P0.tile_yz || P.tma_off != P0.tma_off || P.x_bulk != P0.x_bulk ||
            P.x_rows != P0.x_rows || P.yz_lowreg != P0.yz_lowreg || P.fast_off != P0.fast_off)
            return fail(P, FP_ERR_INVALID,
                        "group: members must share the FFT tiling (fp_autotune or fp_set_tiling on each)");
    }
    bool grouped = count > 1;
    for (int i = 0; i < count && grouped; ++i) grouped = fp::group_supported(handles[i]->P);
    if (!grouped) {  // one at a time on the members' own streams
        for (int i = 0; i < count; ++i) {
            int rc = fp_solve_permeability(handles[i], tol, maxit, K + 9 * (size_t)i,
                                           stats ? stats + 3 * (size_t)i : nullptr);
            if (rc) return rc;
        }
        return FP_OK;
    }
    std::vector<int> cols((size_t)count);
    std::vector<std::array<double, 3>> avg((size_t)count);
    std::vector<fp_solver_stats> st((size_t)count);
    for (int col = 0; col < 3; ++col) {
        std::fill(cols.begin(), cols.end(), col);
        int rc = group_solve_cases(count, handles, cols.data(), tol, maxit,
                                   reinterpret_cast<double(*)[3]>(avg.data()), st.data());
        if (rc) return rc;
        for (int i = 0; i < count; ++i) {
            set_column(K + 9 * (size_t)i, col, handles[i]->P.mu, avg[(size_t)i].data());
            if (stats) stats[3 * (size_t)i + col] = st[(size_t)i];
        }
    }
    return FP_OK;
}

int fp_solve_permeability_block(fp_handle h, double tol, int64_t maxit, double K[9],
                                fp_solver_stats stats[3]) {
    if (!h || !K) return FP_ERR_INVALID;
    Problem& P = h->P;
    int rc = need_geometry(P, "PermeabilityRunner::run");
    if (rc) return rc;
    if (!fp::group_supported(P)) return fp_solve_permeability(h, tol, maxit, K, stats);
    // the Green tables the siblings borrow
    rc = P.precision == fp::kMixed ? ensure_green_both(P) : ensure_green64(P);
    if (rc) return rc;
    // two siblings: own vectors, spectral buffer and scalars; the same mask,
    // support, tiling and solver settings; the Green tables of h
    fp_handle sib[2] = {nullptr, nullptr};
    auto drop = [&](int code) {
        for (fp_handle s : sib) {
            if (!s) continue;
            s->P.d_green32 = nullptr;  // borrowed
            s->P.d_green64 = nullptr;
            fp_destroy(s);
        }
        return code;
    };
    for (int k = 0; k < 2; ++k) {
        rc = fp::create_handle(P.nx, P.ny, P.nz, P.h, P.mu, P.p_radius, P.precision, false, &sib[k]);
        if (rc) {
            if (sib[k]) P.err = "block solve: " + sib[k]->P.err;
            return drop(rc);
        }
        Problem& S = sib[k]->P;
        S.support_mode = P.support_mode;
        S.reliable_interval = P.reliable_interval;
        S.ahead_factor = P.ahead_factor;
        S.segment_tol_factor = P.segment_tol_factor;
        S.use_graphs = P.use_graphs;
        S.fast_off = P.fast_off;
        S.tma_off = P.tma_off;
        S.x_bulk = P.x_bulk;
        S.x_rows = P.x_rows;
        S.tile_yz = P.tile_yz;
        S.yz_lowreg = P.yz_lowreg;
        cudaError_t e = cudaStreamSynchronize(P.stream);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(S.d_mask, P.d_mask, (size_t)P.n, cudaMemcpyDeviceToDevice, S.stream);
        if (e != cudaSuccess) return drop(cuda_fail(P, e, "block solve: mask copy"));
        rc = finish_geometry(S, nullptr);
        if (!rc && S.nb != P.nb) rc = fail(S, FP_ERR_STATE, "support size differs");
        if (rc) {
            P.err = "block solve: " + S.err;
            return drop(rc);
        }
        S.d_green32 = P.d_green32;
        S.d_green64 = P.d_green64;
    }
    fp_handle members[3] = {h, sib[0], sib[1]};
    const int cols[3] = {0, 1, 2};
    double avg[3][3];
    fp_solver_stats st[3];
    rc = group_solve_cases(3, members, cols, tol, maxit, avg, st);
    if (rc) {
        for (fp_handle s : sib)
            if (!s->P.err.empty()) P.err = "block solve: " + s->P.err;
        return drop(rc);
    }
    for (int c = 0; c < 3; ++c) {
        set_column(K, c, P.mu, avg[c]);
        if (stats) stats[c] = st[c];
    }
    return drop(FP_OK);
}

}  // extern "C"
