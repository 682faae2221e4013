// batch.cu -- many independent microstructures solved together, and the FFT
// tile autotuner.
//
// Batching.  Each microstructure is a complete permeability solve (three load
// cases) with no data shared with the others, so the batch needs no
// collective: it is a work queue.  The problems are cut into groups of up to
// `max_group` problems of one grid and voxel size; `concurrency` host threads
// each take one group at a time (its own stream) and solve it with
// fp_group_solve_permeability (one lockstep MINRES per load case over the
// group, one launch per pass for all members) or, for a group of one, with
// fp_solve_permeability, whose MINRES iterations are replayed as CUDA graphs
// of 40.  The threads' kernels overlap on the GPU, so the small grids of a
// batch fill the 152 SMs together.  Groups are taken largest first, which
// keeps the tail of the batch short.
//
// Autotuner.  The y and z passes take `tile` kx columns per CTA and have a
// TMA-fed and a register-fed variant; the inverse x pass has a bulk-copy
// pipelined and a one-tile-per-CTA variant; the x passes' rows per CTA can
// be capped (smaller CTAs, more of them per SM).  fp_autotune times the operator apply
// of a handle for each candidate and keeps the fastest; results are cached per
// (grid, precision) for the process.  The batch tunes every distinct grid
// once before the workers start, so that the timings see an idle GPU.
// Tiling changes the schedule and the grouping of the x pass's partial sums;
// each line's transform is the same arithmetic.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <map>
#include <mutex>
#include <string>
#include <thread>
#include <tuple>
#include <vector>

#include "../../include/fftperm.h"
#include "internal.h"

namespace fp {
namespace {

struct TuneKey {
    int nx, ny, nz, precision;
    bool operator<(const TuneKey& o) const {
        return std::tie(nx, ny, nz, precision) < std::tie(o.nx, o.ny, o.nz, o.precision);
    }
};

struct TuneResult {
    int tile = 0;
    bool tma_off = false;
    bool x_bulk = true;
    int x_rows = 0;
    bool yz_lowreg = false;
    double ms = 0.0;
};

std::mutex g_tune_mu;
std::map<TuneKey, TuneResult> g_tune_cache;

thread_local std::string g_batch_error;

void apply_tiling(Problem& P, int tile, bool tma_off, bool x_bulk, int x_rows, bool lowreg) {
    if (P.tile_yz == tile && P.tma_off == tma_off && P.x_bulk == x_bulk && P.x_rows == x_rows &&
        P.yz_lowreg == lowreg)
        return;
    release_graphs(P);
    P.yz_lowreg = lowreg;
    P.tile_yz = tile;
    P.tma_off = tma_off;
    P.x_bulk = x_bulk;
    P.x_rows = x_rows;
    for (auto& c : P.tma_y) c.valid = false;
    for (auto& c : P.tma_z) c.valid = false;
}

// Mean time of `reps` operator applies (compact source when a geometry is
// set, dense otherwise) on the handle's stream, after one warm-up apply.
int time_apply(Problem& P, int reps, double* ms) {
    ApplyArgs a;
    if (P.has_geometry && P.nb > 0) {
        cudaMemsetAsync(P.d_x, 0, sizeof(double) * 3 * (size_t)P.nb, P.stream);
        a.src = P.d_x;
        a.dst = P.d_cout;
        a.src_kind = kSrcCompact;
        a.dst_kind = kDstCompact;
    } else {
        if (!P.d_dense_in && cudaMallocAsync(reinterpret_cast<void**>(&P.d_dense_in),
                                             sizeof(double) * 3 * (size_t)P.n, P.stream) != cudaSuccess)
            return FP_ERR_NOMEM;
        if (!P.d_dense_out && cudaMallocAsync(reinterpret_cast<void**>(&P.d_dense_out),
                                              sizeof(double) * 3 * (size_t)P.n, P.stream) != cudaSuccess)
            return FP_ERR_NOMEM;
        cudaMemsetAsync(P.d_dense_in, 0, sizeof(double) * 3 * (size_t)P.n, P.stream);
        a.src = P.d_dense_in;
        a.dst = P.d_dense_out;
        a.src_kind = kSrcDense;
        a.dst_kind = kDstDense;
    }
    int np = 0;
    if (launch_apply(P, a, &np) != cudaSuccess) return FP_ERR_CUDA;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, P.stream);
    cudaError_t err = cudaSuccess;
    for (int i = 0; i < reps && err == cudaSuccess; ++i) err = launch_apply(P, a, &np);
    cudaEventRecord(e1, P.stream);
    cudaEventSynchronize(e1);
    float t = 0.f;
    cudaEventElapsedTime(&t, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (err != cudaSuccess) return FP_ERR_CUDA;
    int herr = 0;
    cudaMemcpyAsync(&herr, P.d_err, sizeof(int), cudaMemcpyDeviceToHost, P.stream);
    cudaStreamSynchronize(P.stream);
    if (herr) return FP_ERR_CUDA;
    *ms = (double)t / reps;
    return FP_OK;
}

int tune(Problem& P, TuneResult* out) {
    const TuneKey key{P.nx, P.ny, P.nz, P.precision};
    {
        std::lock_guard<std::mutex> lock(g_tune_mu);
        auto it = g_tune_cache.find(key);
        if (it != g_tune_cache.end()) {
            *out = it->second;
            apply_tiling(P, out->tile, out->tma_off, out->x_bulk, out->x_rows, out->yz_lowreg);
            return FP_OK;
        }
    }
    const int tile0 = P.tile_yz;
    const bool tma0 = P.tma_off;
    const bool bulk0 = P.x_bulk;
    const int rows0 = P.x_rows;
    const bool low0 = P.yz_lowreg;
    TuneResult best;
    best.ms = 1e30;
    const int tiles[] = {4, 8, 16, 32};
    const int xrows[] = {0, 4, 2};
    // the register-capped y/z kernels exist for the FP32 register-fed passes
    const int nlow = P.precision == kFP64 ? 1 : 2;
    for (int xr : xrows) {
        for (int xb = 0; xb < 2; ++xb) {
            for (int off = 0; off < 2; ++off) {
                // lowreg: register-capped register-fed y/z passes, or the
                // single-stage z pass of the specialised passes (TMA on)
                for (int lo = 0; lo < nlow; ++lo) {
                    for (int t : tiles) {
                        apply_tiling(P, t, off != 0, xb == 0, xr, lo != 0);
                        double ms = 0.0;
                        const int rc = time_apply(P, 3, &ms);
                        if (rc != FP_OK) {
                            apply_tiling(P, tile0, tma0, bulk0, rows0, low0);
                            return rc;
                        }
                        if (ms < best.ms) {
                            best.ms = ms;
                            best.tile = t;
                            best.tma_off = off != 0;
                            best.x_bulk = xb == 0;
                            best.x_rows = xr;
                            best.yz_lowreg = lo != 0;
                        }
                    }
                }
            }
        }
    }
    apply_tiling(P, best.tile, best.tma_off, best.x_bulk, best.x_rows, best.yz_lowreg);
    {
        std::lock_guard<std::mutex> lock(g_tune_mu);
        g_tune_cache[key] = best;
    }
    *out = best;
    return FP_OK;
}

}  // namespace
}  // namespace fp

extern "C" int fp_time_apply(fp_handle h, int reps, double* ms) {
    if (!h || reps <= 0 || !ms) return FP_ERR_INVALID;
    const int rc = fp::time_apply(h->P, reps, ms);
    if (rc != FP_OK) h->P.err = "fp_time_apply: an operator apply failed";
    return rc;
}

extern "C" int fp_autotune(fp_handle h, int* tile, int* tma_off, int* x_bulk, int* x_rows,
                           int* lowreg, double* apply_ms) {
    using namespace fp;
    if (!h) return FP_ERR_INVALID;
    TuneResult r;
    const int rc = tune(h->P, &r);
    if (rc != FP_OK) {
        h->P.err = "autotune: an operator apply failed";
        return rc;
    }
    if (tile) *tile = r.tile;
    if (tma_off) *tma_off = r.tma_off ? 1 : 0;
    if (x_bulk) *x_bulk = r.x_bulk ? 1 : 0;
    if (x_rows) *x_rows = r.x_rows;
    if (lowreg) *lowreg = r.yz_lowreg ? 1 : 0;
    if (apply_ms) *apply_ms = r.ms;
    return FP_OK;
}

extern "C" int fp_set_tiling(fp_handle h, int tile, int tma_off, int x_bulk, int x_rows, int lowreg) {
    using namespace fp;
    if (!h) return FP_ERR_INVALID;
    if (tile != 0 && tile != 2 && tile != 4 && tile != 8 && tile != 16 && tile != 32) {
        h->P.err = "fp_set_tiling: tile must be 0 (default), 2, 4, 8, 16 or 32";
        return FP_ERR_INVALID;
    }
    apply_tiling(h->P, tile, tma_off != 0, x_bulk != 0, x_rows < 0 ? 0 : x_rows, lowreg != 0);
    return FP_OK;
}

extern "C" const char* fp_batch_last_error(void) { return fp::g_batch_error.c_str(); }

extern "C" int fp_batch_solve_permeability(int count, const int* dims, const uint8_t* const* masks,
                                           const double* voxel_sizes, double mu, int p_radius,
                                           int precision, int support_mode, double tol,
                                           int64_t maxit, int concurrency, int autotune, double* K,
                                           fp_solver_stats* stats, int* status) {
    return fp_batch_solve_grouped(count, dims, masks, voxel_sizes, mu, p_radius, precision, support_mode,
                                  tol, maxit, concurrency, autotune, 1, K, stats, status);
}

extern "C" int fp_batch_solve_grouped(int count, const int* dims, const uint8_t* const* masks,
                                      const double* voxel_sizes, double mu, int p_radius,
                                      int precision, int support_mode, double tol, int64_t maxit,
                                      int concurrency, int autotune, int max_group, double* K,
                                      fp_solver_stats* stats, int* status) {
    using namespace fp;
    g_batch_error.clear();
    if (count < 0 || (count > 0 && (!dims || !masks || !K)) || concurrency < 1 || max_group < 1) {
        g_batch_error = "batch: invalid arguments";
        return FP_ERR_INVALID;
    }
    for (int i = 0; i < count; ++i)
        if (dims[3 * i] <= 0 || dims[3 * i + 1] <= 0 || dims[3 * i + 2] <= 0 || !masks[i]) {
            g_batch_error = "batch: problem " + std::to_string(i) + " has invalid dimensions or mask";
            return FP_ERR_INVALID;
        }
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        g_batch_error = "batch: no CUDA device";
        return FP_ERR_CUDA;
    }
    auto make = [&](int i, fp_handle* h) -> int {
        const double vs = voxel_sizes ? voxel_sizes[i] : 1.0;
        int rc = fp_create(dims[3 * i], dims[3 * i + 1], dims[3 * i + 2], vs, mu, p_radius, precision, h);
        if (rc == FP_OK) rc = fp_set_geometry(*h, masks[i], support_mode, nullptr);
        return rc;
    };
    // 1) tune each distinct grid once, on an otherwise idle GPU
    if (autotune) {
        std::map<TuneKey, int> first;
        for (int i = 0; i < count; ++i) first.emplace(TuneKey{dims[3 * i], dims[3 * i + 1], dims[3 * i + 2], precision}, i);
        for (auto& kv : first) {
            fp_handle h = nullptr;
            int rc = make(kv.second, &h);
            if (rc == FP_OK) {
                TuneResult r;
                rc = tune(h->P, &r);
            }
            if (rc != FP_OK) {
                g_batch_error = "batch: autotune of problem " + std::to_string(kv.second) + ": " +
                                (h ? h->P.err : std::string("create failed"));
                fp_destroy(h);
                return rc;
            }
            fp_destroy(h);
        }
    }
    // 2) jobs: groups of up to max_group problems of one grid and voxel size
    //    (one lockstep solve each), largest total first
    std::map<std::tuple<int, int, int, double>, std::vector<int>> by_grid;
    for (int i = 0; i < count; ++i)
        by_grid[std::make_tuple(dims[3 * i], dims[3 * i + 1], dims[3 * i + 2],
                                voxel_sizes ? voxel_sizes[i] : 1.0)]
            .push_back(i);
    std::vector<std::vector<int>> groups;
    for (auto& kv : by_grid)
        for (size_t k = 0; k < kv.second.size(); k += (size_t)max_group)
            groups.emplace_back(kv.second.begin() + k,
                                kv.second.begin() + std::min(kv.second.size(), k + (size_t)max_group));
    auto voxels = [&](const std::vector<int>& g) {
        long long v = 0;
        for (int i : g) v += (long long)dims[3 * i] * dims[3 * i + 1] * dims[3 * i + 2];
        return v;
    };
    std::stable_sort(groups.begin(), groups.end(),
                     [&](const std::vector<int>& a, const std::vector<int>& b) { return voxels(a) > voxels(b); });
    const int njobs = (int)groups.size();
    std::atomic<int> next{0};
    std::vector<int> rcs((size_t)count, FP_OK);
    std::vector<std::string> errs((size_t)count);
    auto worker = [&]() {
        cudaSetDevice(dev);
        for (;;) {
            const int j = next.fetch_add(1);
            if (j >= njobs) return;
            const std::vector<int>& g = groups[(size_t)j];
            const int G = (int)g.size();
            std::vector<fp_handle> hs((size_t)G, nullptr);
            int rc = FP_OK;
            int bad = g[0];
            for (int k = 0; k < G && rc == FP_OK; ++k) {
                bad = g[(size_t)k];
                rc = make(bad, &hs[(size_t)k]);
                if (rc == FP_OK && autotune) {
                    TuneResult r;
                    rc = tune(hs[(size_t)k]->P, &r);  // a cache hit: sets the tuned tiling
                }
            }
            std::vector<double> Kg((size_t)9 * G);
            std::vector<fp_solver_stats> st((size_t)3 * G);
            if (rc == FP_OK) {
                rc = G == 1 ? fp_solve_permeability(hs[0], tol, maxit, Kg.data(), st.data())
                            : fp_group_solve_permeability(G, hs.data(), tol, maxit, Kg.data(), st.data());
                if (rc != FP_OK) {
                    bad = g[0];
                    for (int k = 0; k < G; ++k)
                        if (!hs[(size_t)k]->P.err.empty()) bad = g[(size_t)k];
                }
            }
            for (int k = 0; k < G; ++k) {
                const int i = g[(size_t)k];
                if (rc == FP_OK) {
                    for (int q = 0; q < 9; ++q) K[9 * (size_t)i + q] = Kg[9 * (size_t)k + q];
                    if (stats)
                        for (int c = 0; c < 3; ++c) stats[3 * (size_t)i + c] = st[3 * (size_t)k + c];
                } else {
                    const int kb = (int)(std::find(g.begin(), g.end(), bad) - g.begin());
                    errs[(size_t)i] = (kb < G && hs[(size_t)kb]) ? hs[(size_t)kb]->P.err
                                                                 : std::string("create failed");
                }
                rcs[(size_t)i] = rc;
            }
            for (fp_handle h : hs) fp_destroy(h);
        }
    };
    const int nthreads = std::min(concurrency, std::max(njobs, 1));
    std::vector<std::thread> pool;
    for (int t = 0; t < nthreads; ++t) pool.emplace_back(worker);
    for (auto& t : pool) t.join();
    int first_rc = FP_OK;
    for (int i = 0; i < count; ++i) {
        if (status) status[i] = rcs[(size_t)i];
        if (rcs[(size_t)i] != FP_OK && first_rc == FP_OK) {
            first_rc = rcs[(size_t)i];
            g_batch_error = "batch: problem " + std::to_string(i) + ": " + errs[(size_t)i];
        }
    }
    return first_rc;
}
