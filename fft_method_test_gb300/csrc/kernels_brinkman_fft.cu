// kernels_brinkman_fft.cu -- the Brinkman problem solved to the discrete fixed
// point of the reference's own equations by an FFT-preconditioned projected
// conjugate gradient, FP64.
//
// The reference iteration (src/brinkman/FluidBrinkman.cpp:282-507, on the GPU
// in kernels_brinkman.cu) stops where its momentum relaxation and 35-sweep
// pressure projection are both at rest, i.e. at the solution of
//     (alpha + 6 mu) u - mu sum_nbr u + grad_c p = f,   div_c u = 0
// (momentum :313-369 with u* = u, projection :435-466 with phi = 0), with
// grad_c the periodic central difference 0.5 (a[+1] - a[-1]).  That scheme
// converges like iter^-1.2 and does not reach tolerances of 1e-8.  Here the
// same fixed point is computed directly.  With A = alpha - mu Lap7 and P the
// orthogonal projection onto discretely divergence-free fields, the velocity
// is the solution in range(P) of P A u = P f.  A is symmetric positive
// definite (alpha >= 0, a solid voxel exists), so conjugate gradients apply.
// In Fourier space with s_i = sin(2 pi k_i / n_i) (the symbol of grad_c is
// i s) and lambda = sum 4 sin^2(pi k_i / n_i) (minus the symbol of Lap7):
//     P^(k) = I - s s^T / |s|^2   (I where s = 0: the k_i in {0, n_i/2} modes)
//     M^(k) = P^(k) / (alpha0 + mu lambda)   the preconditioner
// The residual is kept projected, in Fourier space (r^ = P^ F(f - A x)); a
// residual that carries the pressure-gradient part (f - A x unprojected)
// loses accuracy once |P r| << |r|.  One iteration:
//     Ap = A p (7-point stencil), pAp = p . Ap       k_bf_stencil
//     g = rho / pAp                                   k_bf_after_stencil
//     a^ = F(Ap)                                      forward R2C FFT (3 passes)
//     r^ -= g P^ a^,  z^ = r^ / (alpha0 + mu lambda)  k_bf_spectral
//     rho' = <r^, z^> / N, beta = rho' / rho          k_bf_after_spectral
//     z = F^-1(z^)                                    inverse C2R FFT (3 passes)
//     x += g p,  p = z + beta p                       k_bf_update
// Stop: |r^| / |r^_0| <= tol.  At the end the projected residual is
// recomputed from x; if the recurrence ran ahead of it, CG restarts from x.
// Only a uniform viscosity is a symmetric problem: fluid viscosity 1, the
// reference's solid viscosity (other values return FP_ERR_UNSUPPORTED).
#include <cuda_runtime.h>

#include <chrono>
#include <cmath>
#include <string>
#include <vector>

#include "../../include/fftperm.h"
#include "internal.h"

namespace fp {

void brinkman_set_error(const std::string& m);  // kernels_brinkman.cu

namespace {

struct BfScalars {
    double rho;     // <r^, M r^> / N of the current residual
    double pap;     // p . A p
    double g;       // step length
    double beta;    // direction update
    double r0;      // |r^_0| (Parseval-scaled)
    double rel;     // |r^| / r0
    double tol;
    long long it;
    long long maxit;
    int stop;       // set by the reductions; copied to done at the end of the iteration
    int done;       // skips every kernel of later iterations
    int breakdown;  // pAp <= 0 or a non-finite scalar
    int pad;
};

constexpr int kBfThreads = 256;

struct BfGrid {
    int nx, ny, nz;
    long long n;
};

// Ap = (alpha + 6) p - sum_nbr p for the three components (mu = 1), and
// per-block partial sums of p . Ap.
__global__ void __launch_bounds__(kBfThreads) k_bf_stencil(BfGrid g, const BfScalars* sc,
                                                           const uint8_t* __restrict__ fluid,
                                                           double penalty,
                                                           const double* __restrict__ p,
                                                           double* __restrict__ ap, double* partials) {
    __shared__ double red[4 * 32];
    if (sc->done) return;
    double acc[4] = {0, 0, 0, 0};
    const long long n = g.n;
    const long long sxy = (long long)g.nx * g.ny;
    // CTAs stride over grid rows, threads over x: no per-voxel division
    for (int row = blockIdx.x; row < g.ny * g.nz; row += gridDim.x)
        for (int x = threadIdx.x; x < g.nx; x += blockDim.x) {
        const int y = row % g.ny;
        const int z = row / g.ny;
        const long long base = (long long)row * g.nx;
        const long long id = base + x;
        const long long xm = base + (x == 0 ? g.nx - 1 : x - 1);
        const long long xp = base + (x == g.nx - 1 ? 0 : x + 1);
        const long long rowz = (long long)z * sxy + x;
        const long long ym = rowz + (long long)(y == 0 ? g.ny - 1 : y - 1) * g.nx;
        const long long yp = rowz + (long long)(y == g.ny - 1 ? 0 : y + 1) * g.nx;
        const long long col = (long long)y * g.nx + x;
        const long long zm = (long long)(z == 0 ? g.nz - 1 : z - 1) * sxy + col;
        const long long zp = (long long)(z == g.nz - 1 ? 0 : z + 1) * sxy + col;
        const double diag = (fluid[id] ? 0.0 : penalty) + 6.0;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const double* pc = p + c * n;
            const double v = pc[id];
            const double a = diag * v - (pc[xm] + pc[xp] + pc[ym] + pc[yp] + pc[zm] + pc[zp]);
            ap[c * n + id] = a;
            acc[0] += v * a;
        }
    }
    double o[4];
    block_sum<4>(acc, red, o);
    if (threadIdx.x == 0) partials[4LL * blockIdx.x] = o[0];
}

__device__ __forceinline__ bool bad(double v) { return !isfinite(v); }

// g = rho / pAp (deterministic single-block reduction)
__global__ void k_bf_after_stencil(BfScalars* sc, const double* partials, int nparts) {
    __shared__ double red[4 * 32];
    if (sc->done) return;
    double acc[4] = {0, 0, 0, 0};
    for (int i = threadIdx.x; i < nparts; i += blockDim.x) acc[0] += partials[4LL * i];
    double o[4];
    block_sum<4>(acc, red, o);
    if (threadIdx.x == 0) {
        const double pap = o[0];
        sc->pap = pap;
        if (!(pap > 0.0) || bad(pap) || bad(sc->rho)) {
            sc->breakdown = 1;
            sc->stop = 1;
            sc->g = 0.0;
        } else {
            sc->g = sc->rho / pap;
        }
    }
}

struct BfSpecArgs {
    int nx, ny, nz, nxh;
    long long rs, nh, nrows;
    double alpha0;  // preconditioner shift
    double mu;
    const double* sx;  // sin(2 pi k / n) per axis
    const double* sy;
    const double* sz;
    const double* lx;  // 4 sin^2(pi k / n) per axis
    const double* ly;
    const double* lz;
    double2* spec;       // in: F(A p) (iteration) or F(A x) (restart); out: z^
    double2* rhat;       // projected residual
    double fhat0[3];     // F(f) at k = 0 (N f); zero elsewhere for a uniform force
    double* partials;
};

// mode 0 (iteration): r^ -= g P^ a^;  mode 1 (restart): r^ = P^ (F(f) - a^).
// Then z^ = r^ / (alpha0 + mu lambda) into spec; partials {<r^, z^>, |r^|^2}
// with the Hermitian weights of the half spectrum.
template <int MODE>
__global__ void __launch_bounds__(kBfThreads) k_bf_spectral(BfSpecArgs a, const BfScalars* sc) {
    __shared__ double red[4 * 32];
    if (sc->done) return;
    const double g = MODE == 0 ? sc->g : 0.0;
    double acc[4] = {0, 0, 0, 0};
    const bool even = (a.nx & 1) == 0;
    for (int row = blockIdx.x; row < (int)a.nrows; row += gridDim.x)
        for (int kx = threadIdx.x; kx < a.nxh; kx += blockDim.x) {
        const int ky = row % a.ny;
        const int kz = row / a.ny;
        const long long i = (long long)row * a.rs + kx;
        const double s0 = a.sx[kx], s1 = a.sy[ky], s2 = a.sz[kz];
        const double ss = s0 * s0 + s1 * s1 + s2 * s2;
        double2 v0 = a.spec[i], v1 = a.spec[a.nh + i], v2 = a.spec[2 * a.nh + i];
        if (MODE == 1) {
            const bool k0 = (row == 0 && kx == 0);
            v0 = make_double2((k0 ? a.fhat0[0] : 0.0) - v0.x, -v0.y);
            v1 = make_double2((k0 ? a.fhat0[1] : 0.0) - v1.x, -v1.y);
            v2 = make_double2((k0 ? a.fhat0[2] : 0.0) - v2.x, -v2.y);
        }
        if (ss > 0.0) {
            const double inv = 1.0 / ss;
            const double dr = (s0 * v0.x + s1 * v1.x + s2 * v2.x) * inv;
            const double di = (s0 * v0.y + s1 * v1.y + s2 * v2.y) * inv;
            v0.x -= s0 * dr;
            v0.y -= s0 * di;
            v1.x -= s1 * dr;
            v1.y -= s1 * di;
            v2.x -= s2 * dr;
            v2.y -= s2 * di;
        }
        double2 r0, r1, r2;
        if (MODE == 0) {
            r0 = a.rhat[i];
            r1 = a.rhat[a.nh + i];
            r2 = a.rhat[2 * a.nh + i];
            r0.x -= g * v0.x;
            r0.y -= g * v0.y;
            r1.x -= g * v1.x;
            r1.y -= g * v1.y;
            r2.x -= g * v2.x;
            r2.y -= g * v2.y;
        } else {
            r0 = v0;
            r1 = v1;
            r2 = v2;
        }
        a.rhat[i] = r0;
        a.rhat[a.nh + i] = r1;
        a.rhat[2 * a.nh + i] = r2;
        const double lam = a.lx[kx] + a.ly[ky] + a.lz[kz];
        const double d = 1.0 / (a.alpha0 + a.mu * lam);
        a.spec[i] = make_double2(d * r0.x, d * r0.y);
        a.spec[a.nh + i] = make_double2(d * r1.x, d * r1.y);
        a.spec[2 * a.nh + i] = make_double2(d * r2.x, d * r2.y);
        const double w = (kx == 0 || (even && 2 * kx == a.nx)) ? 1.0 : 2.0;
        const double rr = r0.x * r0.x + r0.y * r0.y + r1.x * r1.x + r1.y * r1.y + r2.x * r2.x +
                          r2.y * r2.y;
        acc[0] += w * d * rr;
        acc[1] += w * rr;
    }
    double o[4];
    block_sum<4>(acc, red, o);
    if (threadIdx.x == 0) {
        a.partials[4LL * blockIdx.x] = o[0];
        a.partials[4LL * blockIdx.x + 1] = o[1];
    }
}

// rho', |r^|, beta, the stop test.  restart: beta = 0, the iteration count
// unchanged, and r0 set when it is not yet known.
__global__ void k_bf_after_spectral(BfScalars* sc, const double* partials, int nparts, double inv_n,
                                    int restart) {
    __shared__ double red[4 * 32];
    if (sc->done) return;
    double acc[4] = {0, 0, 0, 0};
    for (int i = threadIdx.x; i < nparts; i += blockDim.x) {
        acc[0] += partials[4LL * i];
        acc[1] += partials[4LL * i + 1];
    }
    double o[4];
    block_sum<4>(acc, red, o);
    if (threadIdx.x == 0) {
        const double rho = o[0] * inv_n;
        const double rn = sqrt(o[1] * inv_n);
        if (restart) {
            if (!(sc->r0 > 0.0)) sc->r0 = rn;
            sc->beta = 0.0;
        } else {
            sc->beta = rho / sc->rho;
            sc->it += 1;
        }
        sc->rho = rho;
        sc->rel = sc->r0 > 0.0 ? rn / sc->r0 : 0.0;
        if (bad(rho) || bad(sc->beta)) {
            sc->breakdown = 1;
            sc->stop = 1;
        }
        if (sc->rel <= sc->tol || sc->it >= sc->maxit) sc->stop = 1;
    }
}

// x += g p; p = z + beta p   (restart: g = 0, beta = 0, so p = z)
template <int RESTART>
__global__ void __launch_bounds__(kBfThreads) k_bf_update(const BfScalars* sc, long long m,
                                                          double* __restrict__ x,
                                                          double* __restrict__ p,
                                                          const double* __restrict__ z) {
    if (sc->done) return;
    const double g = RESTART ? 0.0 : sc->g;
    const double beta = RESTART ? 0.0 : sc->beta;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < m;
         i += (long long)gridDim.x * blockDim.x) {
        const double pv = p[i];
        if (!RESTART) x[i] += g * pv;
        p[i] = RESTART ? z[i] : z[i] + beta * pv;
    }
}

__global__ void k_bf_end(BfScalars* sc) {
    if (threadIdx.x == 0 && blockIdx.x == 0) sc->done = sc->stop;
}

// p^ = -i s . (F(f) - a^) / |s|^2 into component 0 of spec, components 1, 2
// zeroed (pressure gauge: zero on the s = 0 modes).
__global__ void k_bf_pressure(BfSpecArgs a) {
    for (int row = blockIdx.x; row < (int)a.nrows; row += gridDim.x)
        for (int kx = threadIdx.x; kx < a.nxh; kx += blockDim.x) {
        const int ky = row % a.ny;
        const int kz = row / a.ny;
        const long long i = (long long)row * a.rs + kx;
        const double s0 = a.sx[kx], s1 = a.sy[ky], s2 = a.sz[kz];
        const double ss = s0 * s0 + s1 * s1 + s2 * s2;
        const bool k0 = (row == 0 && kx == 0);
        const double2 v0 = a.spec[i], v1 = a.spec[a.nh + i], v2 = a.spec[2 * a.nh + i];
        double2 ph = make_double2(0.0, 0.0);
        if (ss > 0.0) {
            const double inv = 1.0 / ss;
            // q = s . (F(f) - a^)
            const double qr = s0 * ((k0 ? a.fhat0[0] : 0.0) - v0.x) +
                              s1 * ((k0 ? a.fhat0[1] : 0.0) - v1.x) +
                              s2 * ((k0 ? a.fhat0[2] : 0.0) - v2.x);
            const double qi = -(s0 * v0.y + s1 * v1.y + s2 * v2.y);
            ph = make_double2(qi * inv, -qr * inv);  // -i q / |s|^2
        }
        a.spec[i] = ph;
        a.spec[a.nh + i] = make_double2(0.0, 0.0);
        a.spec[2 * a.nh + i] = make_double2(0.0, 0.0);
    }
}

__global__ void k_bf_sum3(long long n, const double* __restrict__ u, double* partials) {
    __shared__ double red[4 * 32];
    double acc[4] = {0, 0, 0, 0};
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        acc[0] += u[i];
        acc[1] += u[n + i];
        acc[2] += u[2 * n + i];
    }
    double o[4];
    block_sum<4>(acc, red, o);
    if (threadIdx.x == 0)
        for (int j = 0; j < 4; ++j) partials[4LL * blockIdx.x + j] = o[j];
}

// sin(2 pi k / n) with exact zeros at k = 0 and k = n/2; 4 sin^2(pi k / n)
void axis_symbols(int n, std::vector<double>& s, std::vector<double>& l) {
    const double kPi = 3.14159265358979323846;
    s.resize(n);
    l.resize(n);
    for (int k = 0; k < n; ++k) {
        s[k] = (2 * k) % n == 0 ? 0.0 : std::sin(2.0 * kPi * (double)k / (double)n);
        const double h = std::sin(kPi * (double)k / (double)n);
        l[k] = 4.0 * h * h;
    }
}

// Device state of one FFT Brinkman problem (one grid, one phase mask).
struct BfSolver {
    fp_handle h = nullptr;
    double* x = nullptr;   // 3N velocity iterate
    double* p = nullptr;   // 3N search direction
    double* w = nullptr;   // 3N: A p, then the inverse transform z
    double2* rhat = nullptr;
    double* tab = nullptr; // sx, sy, sz, lx, ly, lz
    uint8_t* fluid = nullptr;
    BfScalars* sc = nullptr;
    BfScalars* hsc = nullptr;
    int blocks = 0;
    int tx = kBfThreads;  // threads of the x-walking kernels (grid rows)
    int tk = kBfThreads;  // threads of the kx-walking kernels (spectral rows)
    ~BfSolver() {
        DeviceMemGuard mem_guard;
        cudaFree(x);
        cudaFree(p);
        cudaFree(w);
        cudaFree(rhat);
        cudaFree(tab);
        cudaFree(fluid);
        cudaFree(sc);
        if (hsc) cudaFreeHost(hsc);
        if (h) fp_destroy(h);
    }
};

int bf_fail(int code, const std::string& m) {
    brinkman_set_error(m);
    return code;
}

#define BF_CUDA(call, where)                                                                  \
    do {                                                                                      \
        cudaError_t e_ = (call);                                                              \
        if (e_ != cudaSuccess)                                                                \
            return bf_fail(FP_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e_)); \
    } while (0)

int bf_init(BfSolver& S, int nx, int ny, int nz, const uint8_t* fl_host) {
    int rc = create_handle(nx, ny, nz, 1.0, 1.0, 0, FP_PREC_FP64, false, &S.h);
    if (rc != FP_OK) return bf_fail(rc, S.h ? S.h->P.err : std::string("handle creation failed"));
    Problem& P = S.h->P;
    const size_t m = 3 * (size_t)P.n;
    DeviceMemGuard mem_guard;
    BF_CUDA(cudaMalloc(&S.x, sizeof(double) * m), "cudaMalloc");
    BF_CUDA(cudaMalloc(&S.p, sizeof(double) * m), "cudaMalloc");
    BF_CUDA(cudaMalloc(&S.w, sizeof(double) * m), "cudaMalloc");
    BF_CUDA(cudaMalloc(&S.rhat, sizeof(double2) * 3 * (size_t)P.nh), "cudaMalloc");
    BF_CUDA(cudaMalloc(&S.tab, sizeof(double) * 2 * (size_t)(nx + ny + nz)), "cudaMalloc");
    BF_CUDA(cudaMalloc(&S.fluid, (size_t)P.n), "cudaMalloc");
    BF_CUDA(cudaMalloc(&S.sc, sizeof(BfScalars)), "cudaMalloc");
    BF_CUDA(cudaMallocHost(&S.hsc, sizeof(BfScalars)), "cudaMallocHost");
    std::vector<double> t, sx, lx, sy, ly, sz, lz;
    axis_symbols(nx, sx, lx);
    axis_symbols(ny, sy, ly);
    axis_symbols(nz, sz, lz);
    t.insert(t.end(), sx.begin(), sx.end());
    t.insert(t.end(), sy.begin(), sy.end());
    t.insert(t.end(), sz.begin(), sz.end());
    t.insert(t.end(), lx.begin(), lx.end());
    t.insert(t.end(), ly.begin(), ly.end());
    t.insert(t.end(), lz.begin(), lz.end());
    BF_CUDA(cudaMemcpyAsync(S.tab, t.data(), sizeof(double) * t.size(), cudaMemcpyHostToDevice,
                            P.stream),
            "copy");
    BF_CUDA(cudaMemcpyAsync(S.fluid, fl_host, (size_t)P.n, cudaMemcpyHostToDevice, P.stream), "copy");
    BF_CUDA(cudaStreamSynchronize(P.stream), "sync");
    // row-walking kernels: up to 16 CTAs per SM, at most one per grid row,
    // threads rounded up from the row length
    long long b = P.nrows;
    if (b > 16LL * P.sm_count) b = 16LL * P.sm_count;
    S.blocks = (int)b;
    auto fit = [](long long len) {
        long long t = (len + 31) / 32 * 32;
        return (int)(t < 64 ? 64 : (t > kBfThreads ? kBfThreads : t));
    };
    S.tx = fit(P.nx);
    S.tk = fit(P.nxh);
    return FP_OK;
}

BfSpecArgs spec_args(BfSolver& S, const double f[3], double alpha0, double mu) {
    Problem& P = S.h->P;
    BfSpecArgs a{};
    a.nx = P.nx;
    a.ny = P.ny;
    a.nz = P.nz;
    a.nxh = P.nxh;
    a.rs = P.rs;
    a.nh = P.nh;
    a.nrows = P.nrows;
    a.alpha0 = alpha0;
    a.mu = mu;
    a.sx = S.tab;
    a.sy = a.sx + P.nx;
    a.sz = a.sy + P.ny;
    a.lx = a.sz + P.nz;
    a.ly = a.lx + P.nx;
    a.lz = a.ly + P.ny;
    a.spec = static_cast<double2*>(P.d_spec);
    a.rhat = S.rhat;
    for (int c = 0; c < 3; ++c) a.fhat0[c] = (double)P.n * f[c];
    a.partials = P.d_partials;
    return a;
}

cudaError_t fft_forward_dense(Problem& P, const double* src, const int* skip) {
    ApplyArgs a;
    a.src = src;
    a.src_kind = kSrcDense;
    a.stage = kStageForward;
    a.precision = kFP64;
    a.skip = skip;
    int np = 0;
    return launch_apply(P, a, &np);
}

cudaError_t fft_inverse_dense(Problem& P, double* dst, const int* skip) {
    ApplyArgs a;
    a.dst = dst;
    a.dst_kind = kDstDense;
    a.stage = kStageInverse;
    a.precision = kFP64;
    a.skip = skip;
    int np = 0;
    return launch_apply(P, a, &np);
}

// Queue one CG iteration.
cudaError_t bf_iteration(BfSolver& S, const BfSpecArgs& sa, const BfGrid& g, double penalty) {
    Problem& P = S.h->P;
    const int* skip = &S.sc->done;
    FP_LAUNCHED();
    k_bf_stencil<<<S.blocks, S.tx, 0, P.stream>>>(g, S.sc, S.fluid, penalty, S.p, S.w,
                                                         P.d_partials);
    FP_LAUNCHED();
    k_bf_after_stencil<<<1, 256, 0, P.stream>>>(S.sc, P.d_partials, S.blocks);
    cudaError_t e = fft_forward_dense(P, S.w, skip);
    if (e != cudaSuccess) return e;
    FP_LAUNCHED();
    k_bf_spectral<0><<<S.blocks, S.tk, 0, P.stream>>>(sa, S.sc);
    FP_LAUNCHED();
    k_bf_after_spectral<<<1, 256, 0, P.stream>>>(S.sc, P.d_partials, S.blocks, 1.0 / (double)P.n, 0);
    e = fft_inverse_dense(P, S.w, skip);
    if (e != cudaSuccess) return e;
    FP_LAUNCHED();
    k_bf_update<0><<<S.blocks, kBfThreads, 0, P.stream>>>(S.sc, 3 * P.n, S.x, S.p, S.w);
    FP_LAUNCHED();
    k_bf_end<<<1, 32, 0, P.stream>>>(S.sc);
    return cudaGetLastError();
}

// r^ = P^ F(f - A x), z^ = M r^, p = z; sets rho, rel (and r0 when unset).
// Leaves F(A x) overwritten; returns through hsc the new relative residual.
cudaError_t bf_restart(BfSolver& S, const BfSpecArgs& sa, const BfGrid& g, double penalty) {
    Problem& P = S.h->P;
    FP_LAUNCHED();
    k_bf_stencil<<<S.blocks, S.tx, 0, P.stream>>>(g, S.sc, S.fluid, penalty, S.x, S.w,
                                                         P.d_partials);
    cudaError_t e = fft_forward_dense(P, S.w, nullptr);
    if (e != cudaSuccess) return e;
    FP_LAUNCHED();
    k_bf_spectral<1><<<S.blocks, S.tk, 0, P.stream>>>(sa, S.sc);
    FP_LAUNCHED();
    k_bf_after_spectral<<<1, 256, 0, P.stream>>>(S.sc, P.d_partials, S.blocks, 1.0 / (double)P.n, 1);
    e = fft_inverse_dense(P, S.w, nullptr);
    if (e != cudaSuccess) return e;
    FP_LAUNCHED();
    k_bf_update<1><<<S.blocks, kBfThreads, 0, P.stream>>>(S.sc, 3 * P.n, S.x, S.p, S.w);
    return cudaGetLastError();
}

int bf_read(BfSolver& S) {
    Problem& P = S.h->P;
    BF_CUDA(cudaMemcpyAsync(S.hsc, S.sc, sizeof(BfScalars), cudaMemcpyDeviceToHost, P.stream), "copy");
    BF_CUDA(cudaStreamSynchronize(P.stream), "sync");
    return FP_OK;
}

int bf_write(BfSolver& S) {
    Problem& P = S.h->P;
    BF_CUDA(cudaMemcpyAsync(S.sc, S.hsc, sizeof(BfScalars), cudaMemcpyHostToDevice, P.stream), "copy");
    return FP_OK;
}

// One load case on an initialised solver.
int bf_solve(BfSolver& S, double penalty, double tol, long long maxit, const double f[3],
             double* ux, double* uy, double* uz, double* p_out, double U[3],
             fp_brinkman_stats* stats, double* true_rel_out) {
    const auto t0 = std::chrono::steady_clock::now();
    Problem& P = S.h->P;
    const BfGrid g{P.nx, P.ny, P.nz, P.n};
    const double alpha0 = 1.0, mu = 1.0;
    const BfSpecArgs sa = spec_args(S, f, alpha0, mu);
    const long long m = 3 * P.n;
    // x = 0; r^ = P^ F(f) = N f at k = 0; z = f / alpha0 (constant); p = z
    BF_CUDA(cudaMemsetAsync(S.x, 0, sizeof(double) * m, P.stream), "memset");
    *S.hsc = BfScalars{};
    S.hsc->tol = tol;
    S.hsc->maxit = maxit;
    int rc = bf_write(S);
    if (rc) return rc;
    BF_CUDA(bf_restart(S, sa, g, penalty), "FFT Brinkman start");
    rc = bf_read(S);
    if (rc) return rc;
    const int chunk = 25;
    const int max_restarts = 5;
    int restarts = 0;
    double true_rel = S.hsc->rel;
    bool ok = S.hsc->rel <= tol;
    while (!ok) {
        // iterate until the recurrence stops
        while (!S.hsc->stop) {
            for (int i = 0; i < chunk; ++i) BF_CUDA(bf_iteration(S, sa, g, penalty), "FFT Brinkman iteration");
            rc = bf_read(S);
            if (rc) return rc;
        }
        if (S.hsc->breakdown) break;
        // recompute the projected residual from x; restart when it lags
        const long long it = S.hsc->it;
        S.hsc->stop = 0;
        S.hsc->done = 0;
        rc = bf_write(S);
        if (rc) return rc;
        BF_CUDA(bf_restart(S, sa, g, penalty), "FFT Brinkman residual");
        rc = bf_read(S);
        if (rc) return rc;
        true_rel = S.hsc->rel;
        S.hsc->it = it;
        ok = true_rel <= tol;
        if (ok || it >= maxit || restarts >= max_restarts) break;
        ++restarts;
    }
    // device error flag of the TMA passes
    int herr = 0;
    BF_CUDA(cudaMemcpyAsync(&herr, P.d_err, sizeof(int), cudaMemcpyDeviceToHost, P.stream), "copy");
    BF_CUDA(cudaStreamSynchronize(P.stream), "sync");
    if (herr) return bf_fail(FP_ERR_CUDA, "FFT Brinkman: a TMA wait timed out");
    if (S.hsc->breakdown && !ok)
        return bf_fail(FP_ERR_NONFINITE, "FFT Brinkman: conjugate-gradient breakdown (non-finite or "
                                         "non-positive curvature)");
    // superficial velocity: mean of u over all voxels (FluidBrinkman.cpp:233-258)
    FP_LAUNCHED();
    k_bf_sum3<<<S.blocks, kBfThreads, 0, P.stream>>>(P.n, S.x, P.d_partials);
    std::vector<double> part(4 * (size_t)S.blocks);
    BF_CUDA(cudaMemcpyAsync(part.data(), P.d_partials, sizeof(double) * part.size(),
                            cudaMemcpyDeviceToHost, P.stream),
            "copy");
    BF_CUDA(cudaStreamSynchronize(P.stream), "sync");
    double su[3] = {0, 0, 0};
    for (int i = 0; i < S.blocks; ++i)
        for (int c = 0; c < 3; ++c) su[c] += part[4 * (size_t)i + c];
    for (int c = 0; c < 3; ++c) U[c] = su[c] / (double)P.n;
    if (!(std::isfinite(U[0]) && std::isfinite(U[1]) && std::isfinite(U[2])))
        return bf_fail(FP_ERR_NONFINITE, "Brinkman solver produced non-finite macroscopic velocity");
    if (ux) BF_CUDA(cudaMemcpy(ux, S.x, sizeof(double) * P.n, cudaMemcpyDeviceToHost), "copy");
    if (uy) BF_CUDA(cudaMemcpy(uy, S.x + P.n, sizeof(double) * P.n, cudaMemcpyDeviceToHost), "copy");
    if (uz) BF_CUDA(cudaMemcpy(uz, S.x + 2 * P.n, sizeof(double) * P.n, cudaMemcpyDeviceToHost), "copy");
    if (p_out) {
        // pressure from the gradient part of the momentum residual
        S.hsc->done = 0;
        rc = bf_write(S);
        if (rc) return rc;
        FP_LAUNCHED();
        k_bf_stencil<<<S.blocks, S.tx, 0, P.stream>>>(g, S.sc, S.fluid, penalty, S.x, S.w,
                                                             P.d_partials);
        BF_CUDA(fft_forward_dense(P, S.w, nullptr), "pressure FFT");
        FP_LAUNCHED();
        k_bf_pressure<<<S.blocks, S.tk, 0, P.stream>>>(sa);
        BF_CUDA(fft_inverse_dense(P, S.w, nullptr), "pressure FFT");
        BF_CUDA(cudaMemcpyAsync(p_out, S.w, sizeof(double) * P.n, cudaMemcpyDeviceToHost, P.stream),
                "copy");
        BF_CUDA(cudaStreamSynchronize(P.stream), "sync");
    }
    if (true_rel_out) *true_rel_out = true_rel;
    if (stats) {
        stats->iterations = (int32_t)S.hsc->it;
        stats->converged = ok ? 1 : 0;
        stats->residual = true_rel;
        stats->seconds =
            std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    }
    return FP_OK;
}

int bf_prepare(int nx, int ny, int nz, const uint32_t* ids, uint32_t fluid_id, double fluid_mu,
               double solid_penalty, std::vector<uint8_t>& fl, double* porosity) {
    if (nx <= 0 || ny <= 0 || nz <= 0 || !ids)
        return bf_fail(FP_ERR_INVALID, "FFT Brinkman: invalid arguments");
    if (!(solid_penalty >= 0.0) || !std::isfinite(solid_penalty))
        return bf_fail(FP_ERR_INVALID, "FFT Brinkman: solid penalty must be finite and >= 0");
    if (fluid_mu != 1.0)
        return bf_fail(FP_ERR_UNSUPPORTED,
                       "FFT Brinkman: needs a uniform viscosity (fluid viscosity 1, as in the "
                       "solid); use fp_brinkman_solve for other viscosities");
    const long long n = (long long)nx * ny * nz;
    fl.resize((size_t)n);
    long long nfl = 0;
    for (long long i = 0; i < n; ++i) {
        fl[(size_t)i] = ids[i] == fluid_id ? 1 : 0;
        nfl += fl[(size_t)i];
    }
    if (nfl == 0)
        return bf_fail(FP_ERR_STATE, "No fluid material ids found. Set phase=fluid or fluid_material_id.");
    if (nfl == n) return bf_fail(FP_ERR_STATE, "No solid material ids found for Brinkman solve.");
    if (solid_penalty == 0.0)
        return bf_fail(FP_ERR_INVALID, "FFT Brinkman: a zero solid penalty leaves A singular");
    *porosity = (double)nfl / (double)n;
    return FP_OK;
}

}  // namespace
}  // namespace fp

extern "C" int fp_brinkman_fft_solve(int nx, int ny, int nz, const uint32_t* ids, uint32_t fluid_id,
                                     double fluid_mu, double solid_penalty, double tolerance,
                                     int max_iterations, const double force[3], double* ux,
                                     double* uy, double* uz, double* p, double U[3],
                                     fp_brinkman_stats* stats) {
    using namespace fp;
    brinkman_set_error("");
    if (!force || !U) return bf_fail(FP_ERR_INVALID, "FFT Brinkman: invalid arguments");
    if (!(tolerance > 0.0)) return bf_fail(FP_ERR_INVALID, "FFT Brinkman: tolerance must be positive");
    std::vector<uint8_t> fl;
    double porosity = 0.0;
    int rc = bf_prepare(nx, ny, nz, ids, fluid_id, fluid_mu, solid_penalty, fl, &porosity);
    if (rc) return rc;
    BfSolver S;
    rc = bf_init(S, nx, ny, nz, fl.data());
    if (rc) return rc;
    rc = bf_solve(S, solid_penalty, tolerance, max_iterations, force, ux, uy, uz, p, U, stats,
                  nullptr);
    if (rc) return rc;
    if (stats) {
        stats->porosity = porosity;
        stats->viscosity = fluid_mu;
    }
    return FP_OK;
}

extern "C" int fp_brinkman_fft_permeability(int nx, int ny, int nz, const uint32_t* ids,
                                            uint32_t fluid_id, double fluid_mu,
                                            double solid_penalty, double tolerance,
                                            int max_iterations, double forcing, double voxel_size,
                                            double K[9], fp_brinkman_stats stats[3]) {
    using namespace fp;
    brinkman_set_error("");
    if (!K) return bf_fail(FP_ERR_INVALID, "computePermeabilityTensor: K must not be null");
    if (!(tolerance > 0.0)) return bf_fail(FP_ERR_INVALID, "FFT Brinkman: tolerance must be positive");
    if (!(forcing != 0.0) || !std::isfinite(forcing))
        return bf_fail(FP_ERR_INVALID, "computePermeabilityTensor: forcing must be finite and nonzero");
    std::vector<uint8_t> fl;
    double porosity = 0.0;
    int rc = bf_prepare(nx, ny, nz, ids, fluid_id, fluid_mu, solid_penalty, fl, &porosity);
    if (rc) return rc;
    BfSolver S;
    rc = bf_init(S, nx, ny, nz, fl.data());
    if (rc) return rc;
    const double scale = voxel_size * voxel_size;
    for (int j = 0; j < 3; ++j) {
        double f[3] = {0.0, 0.0, 0.0};
        f[j] = forcing;
        double U[3];
        fp_brinkman_stats st{};
        rc = bf_solve(S, solid_penalty, tolerance, max_iterations, f, nullptr, nullptr, nullptr,
                      nullptr, U, &st, nullptr);
        if (rc) return rc;
        st.porosity = porosity;
        st.viscosity = fluid_mu;
        // FluidBrinkman.cpp:532-536: K[i][j] = mu U_i / f_j h^2
        for (int i = 0; i < 3; ++i) K[i * 3 + j] = fluid_mu * U[i] / f[j] * scale;
        if (stats) stats[j] = st;
    }
    return FP_OK;
}
