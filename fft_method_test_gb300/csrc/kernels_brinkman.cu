// kernels_brinkman.cu -- the reference's Brinkman-penalisation iteration on
// the GPU (src/brinkman/FluidBrinkman.cpp:282-507), FP64.
//
// One outer iteration (the reference's order):
//   momentum   u* = w (f - grad_c p + mu sum_nbr u) / (alpha + 6 mu) + (1 - w) u
//   divergence div = div_c u*, partial sums of div^2
//   pressure   phi = 0, then 35 Jacobi sweeps phi' = (sum_nbr phi - div) / 6
//   projection u = u* - grad_c phi, p += phi
//   residual   sqrt(sum div^2 / N) < tolerance -> stop; non-finite -> error
// grad_c is the central difference 0.5 (a[+1] - a[-1]) with periodic wrap.
//
// Arithmetic follows the reference expression by expression; this file is
// compiled without FMA contraction (-fmad=false, see build.py), so each field
// value is the reference's value.  The stop test, the non-finite test and the
// iteration counter live on the device, so iterations are queued (and
// graph-captured) without a host round trip per iteration.
#include <cuda_runtime.h>

#include <chrono>
#include <cmath>
#include <cstring>
#include <optional>
#include <string>
#include <vector>

#include "../../include/fftperm.h"
#include "common.cuh"

namespace fp {
namespace {

struct BrState {
    double residual;
    double div_l2;
    int iterations;
    int converged;
    int nonfinite;
    int done;
};

struct BrGrid {
    int nx, ny, nz;
    long long n;
    int nrows;  // ny * nz
};

// Voxel loop of the stencil kernels: CTAs stride over the ny*nz grid rows,
// threads over x, so neighbour indices need no per-voxel integer division.
#define BR_FOR_VOXELS(g, row, x)                                      \
    for (int row = blockIdx.x; row < (g).nrows; row += gridDim.x)     \
        for (int x = threadIdx.x; x < (g).nx; x += blockDim.x)

__device__ __forceinline__ void nbrs(const BrGrid& g, int row, int x, long long& id, long long& xm,
                                     long long& xp, long long& ym, long long& yp, long long& zm,
                                     long long& zp) {
    const int y = row % g.ny;
    const int z = row / g.ny;
    const long long sxy = (long long)g.nx * g.ny;
    const long long base = (long long)row * g.nx;
    id = base + x;
    xm = base + (x == 0 ? g.nx - 1 : x - 1);
    xp = base + (x == g.nx - 1 ? 0 : x + 1);
    const long long rowz = (long long)z * sxy + x;
    ym = rowz + (long long)(y == 0 ? g.ny - 1 : y - 1) * g.nx;
    yp = rowz + (long long)(y == g.ny - 1 ? 0 : y + 1) * g.nx;
    const long long col = (long long)y * g.nx + x;
    zm = (long long)(z == 0 ? g.nz - 1 : z - 1) * sxy + col;
    zp = (long long)(z == g.nz - 1 ? 0 : z + 1) * sxy + col;
}

// FluidBrinkman.cpp:313-369
__global__ void k_br_momentum(BrGrid g, const BrState* st, const uint8_t* __restrict__ fluid,
                              double fluid_mu, double penalty, double relax, double f0, double f1,
                              double f2, const double* __restrict__ ux, const double* __restrict__ uy,
                              const double* __restrict__ uz, const double* __restrict__ p,
                              double* __restrict__ sx, double* __restrict__ sy,
                              double* __restrict__ sz) {
    if (st->done) return;
    BR_FOR_VOXELS(g, row, x) {
        long long id, xm, xp, ym, yp, zm, zp;
        nbrs(g, row, x, id, xm, xp, ym, yp, zm, zp);
        const bool fl = fluid[id] != 0;
        const double mu = fl ? fluid_mu : 1.0;
        const double alpha = fl ? 0.0 : penalty;
        const double lapUx = ux[xm] + ux[xp] + ux[ym] + ux[yp] + ux[zm] + ux[zp];
        const double lapUy = uy[xm] + uy[xp] + uy[ym] + uy[yp] + uy[zm] + uy[zp];
        const double lapUz = uz[xm] + uz[xp] + uz[ym] + uz[yp] + uz[zm] + uz[zp];
        const double dpdx = 0.5 * (p[xp] - p[xm]);
        const double dpdy = 0.5 * (p[yp] - p[ym]);
        const double dpdz = 0.5 * (p[zp] - p[zm]);
        const double denom = alpha + 6.0 * mu;
        const double jx = (f0 - dpdx + mu * lapUx) / denom;
        const double jy = (f1 - dpdy + mu * lapUy) / denom;
        const double jz = (f2 - dpdz + mu * lapUz) / denom;
        sx[id] = relax * jx + (1.0 - relax) * ux[id];
        sy[id] = relax * jy + (1.0 - relax) * uy[id];
        sz[id] = relax * jz + (1.0 - relax) * uz[id];
    }
}

// FluidBrinkman.cpp:371-400, with per-CTA partial sums of div^2
__global__ void k_br_divergence(BrGrid g, const BrState* st, const double* __restrict__ sx,
                                const double* __restrict__ sy, const double* __restrict__ sz,
                                double* __restrict__ div, double* partials) {
    if (st->done) return;
    __shared__ double red[32];
    double acc[1] = {0.0};
    BR_FOR_VOXELS(g, row, x) {
        long long id, xm, xp, ym, yp, zm, zp;
        nbrs(g, row, x, id, xm, xp, ym, yp, zm, zp);
        const double d = 0.5 * (sx[xp] - sx[xm]) + 0.5 * (sy[yp] - sy[ym]) + 0.5 * (sz[zp] - sz[zm]);
        div[id] = d;
        acc[0] += d * d;
    }
    double o[1];
    block_sum<1>(acc, red, o);
    if (threadIdx.x == 0) partials[blockIdx.x] = o[0];
}

// First sweep from phi = 0: (0 + ... + 0 - div) / 6
__global__ void k_br_jacobi0(BrGrid g, const BrState* st, const double* __restrict__ div,
                             double* __restrict__ phin) {
    if (st->done) return;
    for (long long id = (long long)blockIdx.x * blockDim.x + threadIdx.x; id < g.n;
         id += (long long)gridDim.x * blockDim.x)
        phin[id] = (0.0 - div[id]) / 6.0;
}

// FluidBrinkman.cpp:402-433
__global__ void k_br_jacobi(BrGrid g, const BrState* st, const double* __restrict__ phi,
                            const double* __restrict__ div, double* __restrict__ phin) {
    if (st->done) return;
    BR_FOR_VOXELS(g, row, x) {
        long long id, xm, xp, ym, yp, zm, zp;
        nbrs(g, row, x, id, xm, xp, ym, yp, zm, zp);
        const double nb = phi[xm] + phi[xp] + phi[ym] + phi[yp] + phi[zm] + phi[zp];
        phin[id] = (nb - div[id]) / 6.0;
    }
}

// FluidBrinkman.cpp:435-466
__global__ void k_br_project(BrGrid g, const BrState* st, const double* __restrict__ phi,
                             const double* __restrict__ sx, const double* __restrict__ sy,
                             const double* __restrict__ sz, double* __restrict__ ux,
                             double* __restrict__ uy, double* __restrict__ uz,
                             double* __restrict__ p) {
    if (st->done) return;
    BR_FOR_VOXELS(g, row, x) {
        long long id, xm, xp, ym, yp, zm, zp;
        nbrs(g, row, x, id, xm, xp, ym, yp, zm, zp);
        const double gx = 0.5 * (phi[xp] - phi[xm]);
        const double gy = 0.5 * (phi[yp] - phi[ym]);
        const double gz = 0.5 * (phi[zp] - phi[zm]);
        ux[id] = sx[id] - gx;
        uy[id] = sy[id] - gy;
        uz[id] = sz[id] - gz;
        p[id] += phi[id];
    }
}

// FluidBrinkman.cpp:468-497: residual, finiteness, stop test, counter
__global__ void k_br_check(BrState* st, const double* __restrict__ partials, int nparts, long long n,
                           double tol, int maxit) {
    if (st->done) return;
    __shared__ double red[32];
    double acc[1] = {0.0};
    for (int i = threadIdx.x; i < nparts; i += blockDim.x) acc[0] += partials[i];
    double o[1];
    block_sum<1>(acc, red, o);
    if (threadIdx.x != 0) return;
    st->div_l2 = o[0];
    st->iterations += 1;
    const double r = sqrt(o[0] / (double)n);
    st->residual = r;
    if (!isfinite(r)) {
        st->nonfinite = 1;
        st->done = 1;
    } else if (r < tol) {
        st->converged = 1;
        st->done = 1;
    } else if (st->iterations >= maxit) {
        st->done = 1;
    }
}

__global__ void k_br_sum3(BrGrid g, const double* __restrict__ ux, const double* __restrict__ uy,
                          const double* __restrict__ uz, double* partials) {
    __shared__ double red[4 * 32];
    double acc[4] = {0, 0, 0, 0};
    for (long long id = (long long)blockIdx.x * blockDim.x + threadIdx.x; id < g.n;
         id += (long long)gridDim.x * blockDim.x) {
        acc[0] += ux[id];
        acc[1] += uy[id];
        acc[2] += uz[id];
    }
    double o[4];
    block_sum<4>(acc, red, o);
    if (threadIdx.x == 0)
        for (int j = 0; j < 4; ++j) partials[4LL * blockIdx.x + j] = o[j];
}

}  // namespace

void brinkman_set_error(const std::string& m);

}  // namespace fp

using namespace fp;

namespace {

struct BrBuffers {
    double* f = nullptr;  // one allocation: 10 fields of N doubles
    uint8_t* fluid = nullptr;
    double* partials = nullptr;
    BrState* st = nullptr;
    ~BrBuffers() {
        DeviceMemGuard mem_guard;
        cudaFree(f);
        cudaFree(fluid);
        cudaFree(partials);
        cudaFree(st);
    }
};

thread_local std::string g_brinkman_error;

int br_fail(int code, const std::string& m) {
    g_brinkman_error = m;
    return code;
}

}  // namespace

// Shared with kernels_brinkman_fft.cu: both Brinkman entry families report
// through fp_brinkman_last_error.
void fp::brinkman_set_error(const std::string& m) { g_brinkman_error = m; }

extern "C" const char* fp_brinkman_last_error(void) { return g_brinkman_error.c_str(); }

extern "C" int fp_brinkman_solve(int nx, int ny, int nz, const uint32_t* ids, uint32_t fluid_id,
                                 double fluid_mu, double solid_penalty, double relaxation,
                                 double tolerance, int max_iterations, const double force[3],
                                 double* ux_out, double* uy_out, double* uz_out, double* p_out,
                                 double U[3], fp_brinkman_stats* stats) {
    const auto t0 = std::chrono::steady_clock::now();
    g_brinkman_error.clear();
    if (nx <= 0 || ny <= 0 || nz <= 0 || !ids || !force || !U)
        return br_fail(FP_ERR_INVALID, "solveBrinkman: invalid arguments");
    const long long n = (long long)nx * ny * nz;
    // resolvePhaseMask / buildCoefficientFields without phase tags
    // (FluidBrinkman.cpp:98-116, :152-191)
    std::vector<uint8_t> fl((size_t)n);
    long long nfl = 0;
    for (long long i = 0; i < n; ++i) {
        fl[(size_t)i] = ids[i] == fluid_id ? 1 : 0;
        nfl += fl[(size_t)i];
    }
    if (nfl == 0)
        return br_fail(FP_ERR_STATE, "No fluid material ids found. Set phase=fluid or fluid_material_id.");
    if (nfl == n) return br_fail(FP_ERR_STATE, "No solid material ids found for Brinkman solve.");
    BrBuffers b;
    {
        DeviceMemGuard mem_guard;
        if (cudaMalloc(&b.f, sizeof(double) * 10 * (size_t)n) != cudaSuccess ||
            cudaMalloc(&b.fluid, (size_t)n) != cudaSuccess ||
            cudaMalloc(&b.partials, sizeof(double) * 4 * 4096) != cudaSuccess ||
            cudaMalloc(&b.st, sizeof(BrState)) != cudaSuccess)
            return br_fail(FP_ERR_NOMEM, "solveBrinkman: device allocation failed");
    }
    double* ux = b.f;
    double* uy = ux + n;
    double* uz = uy + n;
    double* p = uz + n;
    double* sx = p + n;
    double* sy = sx + n;
    double* sz = sy + n;
    double* div = sz + n;
    double* phi = div + n;
    double* phin = phi + n;
    cudaStream_t s;
    if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess)
        return br_fail(FP_ERR_CUDA, "solveBrinkman: stream creation failed");
    cudaMemsetAsync(b.f, 0, sizeof(double) * 10 * (size_t)n, s);
    cudaMemcpyAsync(b.fluid, fl.data(), (size_t)n, cudaMemcpyHostToDevice, s);
    BrState init{};
    init.done = max_iterations <= 0 ? 1 : 0;
    cudaMemcpyAsync(b.st, &init, sizeof(BrState), cudaMemcpyHostToDevice, s);
    int dev = 0, sms = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    // one CTA walks whole grid rows (threads over x); the flat kernels use
    // the same shape as a grid-stride loop
    int threads = ((nx + 31) / 32) * 32;
    if (threads > 256) threads = 256;
    if (threads < 64) threads = 64;
    const int nrows = ny * nz;
    int blocks = nrows < 16 * sms ? nrows : 16 * sms;
    if (blocks > 4096) blocks = 4096;  // partial-sum slots
    const BrGrid g{nx, ny, nz, n, nrows};

    // one outer iteration, captured once and replayed
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    const long long l0 = g_thread_launches;
    std::optional<CaptureGuard> capture_guard;
    capture_guard.emplace();
    cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
    FP_LAUNCHED(); k_br_momentum<<<blocks, threads, 0, s>>>(g, b.st, b.fluid, fluid_mu, solid_penalty, relaxation,
                                             force[0], force[1], force[2], ux, uy, uz, p, sx, sy, sz);
    FP_LAUNCHED(); k_br_divergence<<<blocks, threads, 0, s>>>(g, b.st, sx, sy, sz, div, b.partials);
    FP_LAUNCHED(); k_br_jacobi0<<<blocks, threads, 0, s>>>(g, b.st, div, phin);
    double* a = phin;  // current phi after sweep 1
    double* c = phi;
    for (int k = 1; k < 35; ++k) {
        FP_LAUNCHED(); k_br_jacobi<<<blocks, threads, 0, s>>>(g, b.st, a, div, c);
        double* t = a;
        a = c;
        c = t;
    }
    FP_LAUNCHED(); k_br_project<<<blocks, threads, 0, s>>>(g, b.st, a, sx, sy, sz, ux, uy, uz, p);
    FP_LAUNCHED(); k_br_check<<<1, 256, 0, s>>>(b.st, b.partials, blocks, n, tolerance, max_iterations);
    cudaError_t e = cudaStreamEndCapture(s, &graph);
    if (e == cudaSuccess) e = cudaGraphInstantiate(&exec, graph, 0);
    capture_guard.reset();
    // the capture ran nothing: count the graph's kernels at each replay
    const long long graph_kernels = g_thread_launches - l0;
    g_kernel_launches.fetch_sub(graph_kernels, std::memory_order_relaxed);
    if (e != cudaSuccess) {
        cudaStreamDestroy(s);
        return br_fail(FP_ERR_CUDA, std::string("solveBrinkman graph: ") + cudaGetErrorString(e));
    }
    BrState* hs = nullptr;
    cudaMallocHost(&hs, sizeof(BrState));
    const int chunk = 8;
    int rc = FP_OK;
    for (;;) {
        cudaMemcpyAsync(hs, b.st, sizeof(BrState), cudaMemcpyDeviceToHost, s);
        e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) {
            rc = br_fail(FP_ERR_CUDA, std::string("solveBrinkman: ") + cudaGetErrorString(e));
            break;
        }
        if (hs->done) break;
        for (int i = 0; i < chunk; ++i) {
            cudaGraphLaunch(exec, s);
            g_kernel_launches.fetch_add(graph_kernels, std::memory_order_relaxed);
        }
    }
    BrState fin = *hs;
    if (rc == FP_OK && fin.nonfinite) {
        rc = br_fail(FP_ERR_NONFINITE, "Brinkman solver became unstable: non-finite residual at iteration " +
                                           std::to_string(fin.iterations));
    }
    // superficial velocity (FluidBrinkman.cpp:233-258)
    if (rc == FP_OK) {
        FP_LAUNCHED(); k_br_sum3<<<blocks, threads, 0, s>>>(g, ux, uy, uz, b.partials);
        std::vector<double> part(4 * (size_t)blocks);
        cudaMemcpyAsync(part.data(), b.partials, sizeof(double) * part.size(), cudaMemcpyDeviceToHost, s);
        cudaStreamSynchronize(s);
        double su[3] = {0, 0, 0};
        for (int i = 0; i < blocks; ++i)
            for (int c3 = 0; c3 < 3; ++c3) su[c3] += part[4 * (size_t)i + c3];
        for (int c3 = 0; c3 < 3; ++c3) U[c3] = su[c3] / (double)n;
        if (!(std::isfinite(U[0]) && std::isfinite(U[1]) && std::isfinite(U[2])))
            rc = br_fail(FP_ERR_NONFINITE, "Brinkman solver produced non-finite macroscopic velocity");
        if (ux_out) cudaMemcpy(ux_out, ux, sizeof(double) * n, cudaMemcpyDeviceToHost);
        if (uy_out) cudaMemcpy(uy_out, uy, sizeof(double) * n, cudaMemcpyDeviceToHost);
        if (uz_out) cudaMemcpy(uz_out, uz, sizeof(double) * n, cudaMemcpyDeviceToHost);
        if (p_out) cudaMemcpy(p_out, p, sizeof(double) * n, cudaMemcpyDeviceToHost);
    }
    if (stats) {
        stats->iterations = fin.iterations;
        stats->residual = fin.residual;
        stats->converged = fin.converged;
        stats->porosity = (double)nfl / (double)n;
        stats->viscosity = fluid_mu;  // mean fluid viscosity: one fluid id
        stats->seconds =
            std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    }
    cudaFreeHost(hs);
    cudaGraphExecDestroy(exec);
    cudaGraphDestroy(graph);
    cudaStreamDestroy(s);
    return rc;
}

// computePermeabilityTensor (FluidBrinkman.cpp:509-553):
// K[i][j] = mu_mean * U_i / f_j * h^2 for unit forcing along each axis.
extern "C" int fp_brinkman_permeability(int nx, int ny, int nz, const uint32_t* ids, uint32_t fluid_id,
                                        double fluid_mu, double solid_penalty, double relaxation,
                                        double tolerance, int max_iterations, double forcing,
                                        double voxel_size, double K[9], fp_brinkman_stats stats[3]) {
    if (!K) return br_fail(FP_ERR_INVALID, "computePermeabilityTensor: K must not be null");
    const double scale = voxel_size * voxel_size;
    for (int j = 0; j < 3; ++j) {
        double f[3] = {0.0, 0.0, 0.0};
        f[j] = forcing;
        double U[3];
        fp_brinkman_stats st{};
        const int rc = fp_brinkman_solve(nx, ny, nz, ids, fluid_id, fluid_mu, solid_penalty, relaxation,
                                         tolerance, max_iterations, f, nullptr, nullptr, nullptr,
                                         nullptr, U, &st);
        if (rc != FP_OK) return rc;
        for (int i = 0; i < 3; ++i) K[i * 3 + j] = st.viscosity * U[i] / f[j] * scale;
        if (stats) stats[j] = st;
    }
    return FP_OK;
}
