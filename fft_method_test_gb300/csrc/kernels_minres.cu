// kernels_minres.cu -- MINRES on the device (src/solver/MinresSolver.cpp:46-218).
//
// All Lanczos vectors, inner products and the Givens recurrence stay in FP64
// on the GPU.  One iteration is
//   apply   z_raw = A_raw v, fused partial sums of z_raw and of v . z_raw
//   alpha   one CTA: z mean, alpha = v . (z_raw - mean)
//   zupd    z = (z_raw - mean) - (alpha v + beta v_old), partial |z|^2
//   scalar  one CTA: beta_new, Givens rotation, phi_bar, residual history,
//           stop test (the reference's order of operations)
//   vwupd   v_new = z / beta_new, w_next = (v - eps w_prev - delta w) / rho,
//           x += (cs_new phi_bar) w_next, partial component sums of v_new
//   finish  one CTA: component sums of v_new (the next apply's input mean),
//           iteration counter, stop -> done
// Kernels return at once when the solve is done, so the host can queue
// iterations ahead and read the scalar block only every few iterations.
#include <cuda_runtime.h>

#include <cfloat>
#include <cmath>

#include "common.cuh"
#include "internal.h"

namespace fp {

namespace {

constexpr int kVecThreads = 256;
constexpr double kBreakdownEps = 1e-14;

int vec_blocks(const Problem& P, long long m) {
    long long b = (m + kVecThreads - 1) / kVecThreads;
    const long long cap = 8LL * (P.sm_count > 0 ? P.sm_count : 152);
    if (b > cap) b = cap;
    if (b < 1) b = 1;
    return (int)b;
}

// partial component sums (and with SQUARES the sum of squares; GB300's FP64
// pipe is narrow, so the plain sums skip them) of an AoS vector (three
// components per voxel).  Two voxels (three aligned double2) per thread keep
// the component of every load static; the odd tail voxel goes to the first
// thread of block 0.
template <bool SQUARES>
__global__ void k_sum3(const double* __restrict__ v, long long nb, double* partials) {
    __shared__ double red[4 * 32];
    double acc[4] = {0, 0, 0, 0};
    const long long npair = nb >> 1;
    const double2* v2 = reinterpret_cast<const double2*>(v);
    for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < npair;
         k += (long long)gridDim.x * blockDim.x) {
#pragma unroll
        for (int h = 0; h < 3; ++h) {
            const double2 x = v2[3 * k + h];
            acc[(2 * h) % 3] += x.x;
            acc[(2 * h + 1) % 3] += x.y;
            if (SQUARES) acc[3] += x.x * x.x + x.y * x.y;
        }
    }
    if ((nb & 1) && blockIdx.x == 0 && threadIdx.x == 0) {
        for (int c = 0; c < 3; ++c) {
            const double x = v[3 * (nb - 1) + c];
            acc[c] += x;
            acc[3] += x * x;
        }
    }
    double out[4];
    block_sum<4>(acc, red, out);
    if (threadIdx.x == 0)
        for (int i = 0; i < 4; ++i) partials[4LL * blockIdx.x + i] = out[i];
}

__global__ void k_reduce4(const double* __restrict__ partials, int nparts, double* out) {
    __shared__ double red[4 * 32];
    double acc[4] = {0, 0, 0, 0};
    for (int i = threadIdx.x; i < nparts; i += blockDim.x)
        for (int j = 0; j < 4; ++j) acc[j] += partials[4LL * i + j];
    double o[4];
    block_sum<4>(acc, red, o);
    if (threadIdx.x == 0)
        for (int j = 0; j < 4; ++j) out[j] = o[j];
}

// ---- iteration kernels ------------------------------------------------------

__device__ __forceinline__ void alpha_body(MinresScalars* sc, const double* __restrict__ partials,
                                           int nparts, double inv_nb) {
    if (sc->done) return;
    __shared__ double red[4 * 32];
    double acc[4] = {0, 0, 0, 0};
    for (int i = threadIdx.x; i < nparts; i += blockDim.x)
        for (int j = 0; j < 4; ++j) acc[j] += partials[4LL * i + j];
    double o[4];
    block_sum<4>(acc, red, o);
    if (threadIdx.x == 0) {
        double corr = 0.0;
        for (int c = 0; c < 3; ++c) {
            sc->zmean[c] = o[c] * inv_nb;
            corr += sc->zmean[c] * sc->vsum[c];
        }
        sc->alpha = o[3] - corr;
    }
}

__global__ void k_alpha(MinresScalars* sc, const double* __restrict__ partials, int nparts,
                        double inv_nb) {
    alpha_body(sc, partials, nparts, inv_nb);
}

__device__ void scalar_step(MinresScalars* sc, const double* __restrict__ partials, int nparts,
                            double* hist, double* red);
__device__ void finish_step(MinresScalars* sc, const double* __restrict__ partials, int nparts,
                            double* red);
__device__ __forceinline__ bool last_block(unsigned int* counter, unsigned int nblk);

// Two voxels (six doubles, three aligned double2) per thread: components are
// static, loads are 16-byte vectors.  The odd tail voxel is handled by the
// first thread of block 0.
// blk / nblk: this block and the block count of the member's vector kernels
__device__ __forceinline__ void zupd_body(MinresScalars* sc, double* __restrict__ z,
                                          const double* __restrict__ v, const double* __restrict__ v_old,
                                          long long nb, double* partials, unsigned int* counter,
                                          double* hist, unsigned int blk, unsigned int nblk) {
    if (sc->done) return;
    __shared__ double red[32];
    const double alpha = sc->alpha, beta = sc->beta;
    const double mz[3] = {sc->zmean[0], sc->zmean[1], sc->zmean[2]};
    double acc[1] = {0.0};
    const long long npair = nb >> 1;
    double2* z2 = reinterpret_cast<double2*>(z);
    const double2* v2 = reinterpret_cast<const double2*>(v);
    const double2* o2 = reinterpret_cast<const double2*>(v_old);
    for (long long k = (long long)blk * blockDim.x + threadIdx.x; k < npair;
         k += (long long)nblk * blockDim.x) {
#pragma unroll
        for (int h = 0; h < 3; ++h) {
            const double2 zz = z2[3 * k + h], vv = v2[3 * k + h], oo = o2[3 * k + h];
            const int c0 = (2 * h) % 3, c1 = (2 * h + 1) % 3;
            // z - (mean + alpha v + beta v_old): three FP64 operations per
            // element (GB300's FP64 pipe bounds this kernel)
            const double a0 = zz.x - fma(beta, oo.x, fma(alpha, vv.x, mz[c0]));
            const double a1 = zz.y - fma(beta, oo.y, fma(alpha, vv.y, mz[c1]));
            z2[3 * k + h] = make_double2(a0, a1);
            acc[0] += a0 * a0 + a1 * a1;
        }
    }
    if ((nb & 1) && blk == 0 && threadIdx.x == 0) {
        for (int c = 0; c < 3; ++c) {
            const long long i = 3 * (nb - 1) + c;
            const double a0 = z[i] - fma(beta, v_old[i], fma(alpha, v[i], mz[c]));
            z[i] = a0;
            acc[0] += a0 * a0;
        }
    }
    double o[1];
    block_sum<1>(acc, red, o);
    if (threadIdx.x == 0) partials[blk] = o[0];
    if (last_block(counter, nblk)) scalar_step(sc, partials, (int)nblk, hist, red);
}

__global__ void k_zupd(MinresScalars* sc, double* __restrict__ z, const double* __restrict__ v,
                       const double* __restrict__ v_old, long long nb, double* partials,
                       unsigned int* counter, double* hist) {
    zupd_body(sc, z, v, v_old, nb, partials, counter, hist, blockIdx.x, gridDim.x);
}

// The Givens step of one iteration from the |z|^2 partials, run by one whole
// block (the last block of k_zupd): beta_new, the rotation, phi_bar, the
// residual history and the stop test (MinresSolver.cpp:148-186).
__device__ void scalar_step(MinresScalars* sc, const double* __restrict__ partials, int nparts,
                            double* hist, double* red) {
    double acc[1] = {0.0};
    for (int i = threadIdx.x; i < nparts; i += blockDim.x) acc[0] += __ldcg(partials + i);
    double o[1];
    block_sum<1>(acc, red, o);
    if (threadIdx.x != 0) return;
    const double beta_new = sqrt(o[0] > 0.0 ? o[0] : 0.0);
    const double alpha = sc->alpha;
    const double beta = sc->beta;
    // MinresSolver.cpp:148-186
    const double eps = sc->sn_old * beta;
    const double delta_raw = -sc->cs_old * beta;
    const double delta = sc->cs * delta_raw + sc->sn * alpha;
    const double phi = sc->sn * delta_raw - sc->cs * alpha;
    const double rho = hypot(phi, beta_new);
    double cs_new = 1.0, sn_new = 0.0;
    if (rho > kBreakdownEps) {
        cs_new = phi / rho;
        sn_new = beta_new / rho;
    }
    sc->beta_new = beta_new;
    sc->eps = eps;
    sc->delta = delta;
    sc->rho = rho;
    sc->step = cs_new * sc->phi_bar;
    sc->phi_bar *= sn_new;
    sc->cs_old = sc->cs;
    sc->sn_old = sc->sn;
    sc->cs = cs_new;
    sc->sn = sn_new;
    sc->beta = beta_new;
    const double rel = fabs(sc->phi_bar) / sc->rhs_norm;
    sc->rel_res = rel;
    const long long k = sc->it + 1;
    if (hist) hist[k] = rel;
    if (rel <= sc->tol) {
        sc->converged = 1;
        sc->breakdown = 2;  // stop after this iteration's vector update
    } else if (beta_new < kBreakdownEps) {
        sc->converged = rel <= sc->tol;
        sc->breakdown = 2;
    } else if (k >= sc->maxit) {
        sc->breakdown = 2;
    }
}

__device__ __forceinline__ void vwupd_body(MinresScalars* sc, const double* __restrict__ z,
                                           const double* __restrict__ v, double* __restrict__ v_new,
                                           double* __restrict__ w_prev_to_next,
                                           const double* __restrict__ w, double* __restrict__ x,
                                           long long nb, double* partials, unsigned int* counter,
                                           unsigned int blk, unsigned int nblk) {
    if (sc->done) return;
    __shared__ double red[4 * 32];
    const double beta_new = sc->beta_new, eps = sc->eps, delta = sc->delta, rho = sc->rho;
    const double step = sc->step;
    const bool vb = beta_new > kBreakdownEps;
    const bool rb = rho > kBreakdownEps;
    // one division per CTA: GB300's FP64 pipe is narrow, and per-element
    // divisions made this kernel FP64-bound (x / d becomes x * (1 / d), a
    // difference of at most one rounding)
    const double inv_beta = vb ? 1.0 / beta_new : 0.0;
    const double inv_rho = rb ? 1.0 / rho : 0.0;
    double acc[4] = {0, 0, 0, 0};
    const long long npair = nb >> 1;
    const double2* z2 = reinterpret_cast<const double2*>(z);
    const double2* v2 = reinterpret_cast<const double2*>(v);
    double2* vn2 = reinterpret_cast<double2*>(v_new);
    double2* wp2 = reinterpret_cast<double2*>(w_prev_to_next);
    const double2* w2 = reinterpret_cast<const double2*>(w);
    double2* x2 = reinterpret_cast<double2*>(x);
    for (long long k = (long long)blk * blockDim.x + threadIdx.x; k < npair;
         k += (long long)nblk * blockDim.x) {
#pragma unroll
        for (int h = 0; h < 3; ++h) {
            const long long q = 3 * k + h;
            const double2 zz = z2[q], vo = v2[q], wp = wp2[q], ww = w2[q], xx = x2[q];
            const double vn0 = zz.x * inv_beta;
            const double vn1 = zz.y * inv_beta;
            const double wn0 = (vo.x - eps * wp.x - delta * ww.x) * inv_rho;
            const double wn1 = (vo.y - eps * wp.y - delta * ww.y) * inv_rho;
            vn2[q] = make_double2(vn0, vn1);
            wp2[q] = make_double2(wn0, wn1);
            x2[q] = make_double2(xx.x + step * wn0, xx.y + step * wn1);
            acc[(2 * h) % 3] += vn0;
            acc[(2 * h + 1) % 3] += vn1;
        }
    }
    if ((nb & 1) && blk == 0 && threadIdx.x == 0) {
        for (int c = 0; c < 3; ++c) {
            const long long i = 3 * (nb - 1) + c;
            const double vo = v[i];
            const double vn = z[i] * inv_beta;
            v_new[i] = vn;
            const double wn = (vo - eps * w_prev_to_next[i] - delta * w[i]) * inv_rho;
            w_prev_to_next[i] = wn;
            x[i] += step * wn;
            acc[c] += vn;
        }
    }
    double o[4];
    block_sum<4>(acc, red, o);
    if (threadIdx.x == 0)
        for (int j = 0; j < 4; ++j) partials[4LL * blk + j] = o[j];
    if (last_block(counter, nblk)) finish_step(sc, partials, (int)nblk, red);
}

__global__ void k_vwupd(MinresScalars* sc, const double* __restrict__ z, const double* __restrict__ v,
                        double* __restrict__ v_new, double* __restrict__ w_prev_to_next,
                        const double* __restrict__ w, double* __restrict__ x, long long nb,
                        double* partials, unsigned int* counter) {
    vwupd_body(sc, z, v, v_new, w_prev_to_next, w, x, nb, partials, counter, blockIdx.x, gridDim.x);
}

// ---- group kernels: one launch for several problems (tab[member]) ------------

__global__ void k_alpha_g(const IterArgs* __restrict__ tab) {
    const IterArgs& t = tab[blockIdx.x];
    alpha_body(t.sc, t.partials, t.nparts, t.inv_nb);
}

__global__ void k_zupd_g(const IterArgs* __restrict__ tab) {
    const IterArgs& t = tab[blockIdx.y];
    if (blockIdx.x >= (unsigned)t.nblk) return;
    zupd_body(t.sc, t.z, t.v, t.v_old, t.nb, t.partials, t.tickets, t.hist, blockIdx.x, t.nblk);
}

__global__ void k_vwupd_g(const IterArgs* __restrict__ tab) {
    const IterArgs& t = tab[blockIdx.y];
    if (blockIdx.x >= (unsigned)t.nblk) return;
    vwupd_body(t.sc, t.z, t.v, t.v_new, t.w_prev, t.w, t.x, t.nb, t.partials, t.tickets + 1, blockIdx.x,
               t.nblk);
}

// The end of one iteration, run by one whole block (the last block of
// k_vwupd): component sums of v_new (the next apply's input mean), the
// iteration counter, stop -> done.
__device__ void finish_step(MinresScalars* sc, const double* __restrict__ partials, int nparts,
                            double* red) {
    double acc[4] = {0, 0, 0, 0};
    for (int i = threadIdx.x; i < nparts; i += blockDim.x)
        for (int j = 0; j < 4; ++j) acc[j] += __ldcg(partials + 4LL * i + j);
    double o[4];
    block_sum<4>(acc, red, o);
    if (threadIdx.x == 0) {
        for (int c = 0; c < 3; ++c) sc->vsum[c] = o[c];
        sc->it += 1;
        if (sc->breakdown == 2) sc->done = 1;
    }
}

// true in every thread of the block that finishes last among the nblk blocks
// of one problem (its partial sums are then all in memory); the counter is reset
__device__ __forceinline__ bool last_block(unsigned int* counter, unsigned int nblk) {
    __shared__ bool last;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) {
        const unsigned int t = atomicAdd(counter, 1u);
        last = t == nblk - 1;
        if (last) *counter = 0u;
    }
    __syncthreads();
    return last;
}

// ---- start-up kernels -------------------------------------------------------

__global__ void k_start_norms(MinresScalars* sc, const double* __restrict__ partials, int nparts,
                              int which) {
    __shared__ double red[4 * 32];
    double acc[4] = {0, 0, 0, 0};
    for (int i = threadIdx.x; i < nparts; i += blockDim.x)
        for (int j = 0; j < 4; ++j) acc[j] += partials[4LL * i + j];
    double o[4];
    block_sum<4>(acc, red, o);
    if (threadIdx.x == 0) {
        const double nrm = sqrt(o[3] > 0.0 ? o[3] : 0.0);
        if (which == 0) {
            sc->rhs_norm = nrm;  // raw |b|, clamped below
        } else {
            sc->beta = nrm;  // beta1 = |r0|
        }
    }
}

// r0 = b - (A x0 - mean) when have_x0, else b.
__global__ void k_residual0(const MinresScalars* sc, const double* __restrict__ b,
                            double* __restrict__ z, const double* __restrict__ zmean3,
                            long long m, int have_x0) {
    const double m0 = have_x0 ? zmean3[0] : 0.0, m1 = have_x0 ? zmean3[1] : 0.0,
                 m2 = have_x0 ? zmean3[2] : 0.0;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < m;
         i += (long long)gridDim.x * blockDim.x) {
        if (have_x0) {
            const int c = (int)(i % 3);
            const double mz = c == 0 ? m0 : (c == 1 ? m1 : m2);
            z[i] = b[i] - (z[i] - mz);
        } else {
            z[i] = b[i];
        }
    }
}

__global__ void k_scale_div(const double* __restrict__ z, double* __restrict__ v,
                            const MinresScalars* sc, long long m) {
    const double beta = sc->beta;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < m;
         i += (long long)gridDim.x * blockDim.x)
        v[i] = z[i] / beta;
}

__global__ void k_zmean_from_partials(const double* __restrict__ partials, int nparts,
                                      double inv_nb, double* out3) {
    __shared__ double red[4 * 32];
    double acc[4] = {0, 0, 0, 0};
    for (int i = threadIdx.x; i < nparts; i += blockDim.x)
        for (int j = 0; j < 4; ++j) acc[j] += partials[4LL * i + j];
    double o[4];
    block_sum<4>(acc, red, o);
    if (threadIdx.x == 0)
        for (int c = 0; c < 3; ++c) out3[c] = o[c] * inv_nb;
}

}  // namespace

cudaError_t launch_sum3(Problem& P, const double* v, long long nb, double* out4) {
    const int blocks = vec_blocks(P, (nb + 1) / 2);
    FP_LAUNCHED(); k_sum3<false><<<blocks, kVecThreads, 0, P.stream>>>(v, nb, P.d_partials);
    FP_LAUNCHED(); k_reduce4<<<1, 256, 0, P.stream>>>(P.d_partials, blocks, out4);
    return cudaGetLastError();
}

cudaError_t launch_reduce4(Problem& P, int nparts, double* out4) {
    FP_LAUNCHED(); k_reduce4<<<1, 512, 0, P.stream>>>(P.d_partials, nparts, out4);
    return cudaGetLastError();
}


cudaError_t minres_start(Problem& P, const double* b, const double* x0, double tol,
                         long long maxit, int r0_precision) {
    const long long m = 3 * P.nb;
    MinresScalars init{};
    init.tol = tol;
    init.maxit = maxit;
    init.cs_old = -1.0;
    init.sn_old = 0.0;
    init.cs = -1.0;
    init.sn = 0.0;
    P.queued = 0;
    cudaError_t e = cudaMemcpyAsync(P.d_sc, &init, sizeof(init), cudaMemcpyHostToDevice, P.stream);
    if (e != cudaSuccess) return e;
    const int blocks = vec_blocks(P, m);
    // |b|
    FP_LAUNCHED(); k_sum3<true><<<blocks, kVecThreads, 0, P.stream>>>(b, P.nb, P.d_partials);
    FP_LAUNCHED(); k_start_norms<<<1, 256, 0, P.stream>>>(P.d_sc, P.d_partials, blocks, 0);
    // x = x0 or 0
    if (x0) {
        cudaMemcpyAsync(P.d_x, x0, sizeof(double) * m, cudaMemcpyDeviceToDevice, P.stream);
        // z_raw = A_raw x0 with input mean removal
        launch_sum3(P, P.d_x, P.nb, P.d_red);
        ApplyArgs a;
        a.src = P.d_x;
        a.src_sum = P.d_red;
        a.dst = P.d_z;
        a.src_kind = kSrcCompact;
        a.dst_kind = kDstCompact;
        a.precision = r0_precision;
        int nparts = 0;
        e = launch_apply(P, a, &nparts);
        if (e != cudaSuccess) return e;
        FP_LAUNCHED(); k_zmean_from_partials<<<1, 512, 0, P.stream>>>(P.d_partials, nparts, 1.0 / (double)P.nb,
                                                       P.d_red + 4);
        FP_LAUNCHED(); k_residual0<<<blocks, kVecThreads, 0, P.stream>>>(P.d_sc, b, P.d_z, P.d_red + 4, m, 1);
    } else {
        cudaMemsetAsync(P.d_x, 0, sizeof(double) * m, P.stream);
        FP_LAUNCHED(); k_residual0<<<blocks, kVecThreads, 0, P.stream>>>(P.d_sc, b, P.d_z, nullptr, m, 0);
    }
    // beta1 = |r0|
    FP_LAUNCHED(); k_sum3<true><<<blocks, kVecThreads, 0, P.stream>>>(P.d_z, P.nb, P.d_partials);
    FP_LAUNCHED(); k_start_norms<<<1, 256, 0, P.stream>>>(P.d_sc, P.d_partials, blocks, 1);
    e = cudaMemcpyAsync(P.h_sc, P.d_sc, sizeof(MinresScalars), cudaMemcpyDeviceToHost, P.stream);
    if (e != cudaSuccess) return e;
    e = cudaStreamSynchronize(P.stream);
    if (e != cudaSuccess) return e;
    MinresScalars s = *P.h_sc;
    const double rhs_raw = s.rhs_norm;
    if (rhs_raw == 0.0) {  // MinresSolver.cpp:76-82
        s.rhs_norm = DBL_MIN;
        s.converged = 1;
        s.done = 1;
        s.rel_res = 0.0;
        const double z0 = 0.0;
        if (P.d_hist) cudaMemcpyAsync(P.d_hist, &z0, sizeof(double), cudaMemcpyHostToDevice, P.stream);
        *P.h_sc = s;
        return cudaMemcpyAsync(P.d_sc, P.h_sc, sizeof(MinresScalars), cudaMemcpyHostToDevice, P.stream);
    }
    s.rhs_norm = rhs_raw > DBL_MIN ? rhs_raw : DBL_MIN;
    const double beta1 = s.beta;
    const double rel0 = beta1 / s.rhs_norm;
    s.rel_res = rel0;
    if (P.d_hist) {
        P.h_sc->rel_res = rel0;  // staging through pinned memory
        cudaMemcpyAsync(P.d_hist, &P.h_sc->rel_res, sizeof(double), cudaMemcpyHostToDevice, P.stream);
        cudaStreamSynchronize(P.stream);
    }
    if (rel0 <= tol || beta1 == 0.0) {
        s.converged = 1;
        s.done = 1;
        *P.h_sc = s;
        return cudaMemcpyAsync(P.d_sc, P.h_sc, sizeof(MinresScalars), cudaMemcpyHostToDevice, P.stream);
    }
    s.phi_bar = beta1;
    if (maxit <= 0) s.done = 1;
    *P.h_sc = s;
    cudaMemcpyAsync(P.d_sc, P.h_sc, sizeof(MinresScalars), cudaMemcpyHostToDevice, P.stream);
    // v = r0 / beta1 into V[0]; v_old = V[2] = 0; w = 0
    FP_LAUNCHED(); k_scale_div<<<blocks, kVecThreads, 0, P.stream>>>(P.d_z, P.d_v[0], P.d_sc, m);
    cudaMemsetAsync(P.d_v[2], 0, sizeof(double) * m, P.stream);
    cudaMemsetAsync(P.d_w[0], 0, sizeof(double) * m, P.stream);
    cudaMemsetAsync(P.d_w[1], 0, sizeof(double) * m, P.stream);
    // component sums of v (input mean of the first apply)
    FP_LAUNCHED(); k_sum3<false><<<blocks, kVecThreads, 0, P.stream>>>(P.d_v[0], P.nb, P.d_partials);
    FP_LAUNCHED(); k_reduce4<<<1, 256, 0, P.stream>>>(P.d_partials, blocks, P.d_red + 8);
    // copy the three sums into sc->vsum
    cudaMemcpyAsync(&P.d_sc->vsum[0], P.d_red + 8, sizeof(double) * 3, cudaMemcpyDeviceToDevice,
                    P.stream);
    return cudaGetLastError();
}

// Queue `count` iterations, replaying a CUDA graph of them when graphs are on.
// The buffers rotate with period 6 (three Lanczos vectors, two w vectors), so
// one graph per (start phase, count) serves every chunk.  The kernel launch
// counter counts the graph's kernels at each replay.
cudaError_t minres_iterations(Problem& P, int count) {
    if (!P.use_graphs || count <= 0) {
        for (int i = 0; i < count; ++i) {
            cudaError_t e = minres_iteration(P);
            if (e != cudaSuccess) return e;
        }
        return cudaSuccess;
    }
    const int phase = (int)(P.queued % 6);
    MinresGraph* slot = nullptr;
    for (auto& g : P.graphs)
        if (g.exec && g.phase == phase && g.count == count) slot = &g;
    if (!slot) {
        for (auto& g : P.graphs)
            if (!g.exec) {
                slot = &g;
                break;
            }
        if (!slot) {
            release_graphs(P);
            slot = &P.graphs[0];
        }
        const long long q0 = P.queued;
        CaptureGuard capture_guard;
        const long long l0 = g_thread_launches;
        cudaError_t e = cudaStreamBeginCapture(P.stream, cudaStreamCaptureModeThreadLocal);
        if (e != cudaSuccess) return e;
        cudaError_t le = cudaSuccess;
        for (int i = 0; i < count && le == cudaSuccess; ++i) le = minres_iteration(P);
        cudaGraph_t graph = nullptr;
        e = cudaStreamEndCapture(P.stream, &graph);
        const long long nk = g_thread_launches - l0;
        g_kernel_launches.fetch_sub(nk, std::memory_order_relaxed);  // nothing ran yet
        P.queued = q0;
        if (le != cudaSuccess) {
            if (graph) cudaGraphDestroy(graph);
            return le;
        }
        if (e != cudaSuccess) return e;
        e = cudaGraphInstantiate(&slot->exec, graph, 0);
        cudaGraphDestroy(graph);
        if (e != cudaSuccess) {
            slot->exec = nullptr;
            return e;
        }
        slot->phase = phase;
        slot->count = count;
        slot->kernels = nk;
    }
    cudaError_t e = cudaGraphLaunch(slot->exec, P.stream);
    if (e != cudaSuccess) return e;
    g_kernel_launches.fetch_add(slot->kernels, std::memory_order_relaxed);
    P.queued += count;
    return cudaSuccess;
}

void release_graphs(Problem& P) {
    for (auto& g : P.graphs) {
        if (g.exec) cudaGraphExecDestroy(g.exec);
        g = MinresGraph{};
    }
}

cudaError_t iteration_args(Problem& P, IterArgs* t, ApplyArgs* aa) {
    const long long k = P.queued++;
    double* v = P.d_v[k % 3];
    *aa = ApplyArgs{};
    aa->src = v;
    aa->src_sum = &P.d_sc->vsum[0];
    aa->dst = P.d_z;
    aa->dot_with = v;
    aa->src_kind = kSrcCompact;
    aa->dst_kind = kDstCompact;
    aa->skip = &P.d_sc->done;
    t->sc = P.d_sc;
    t->partials = P.d_partials;
    t->nparts = 0;
    t->nblk = vec_blocks(P, (P.nb + 1) / 2);
    t->inv_nb = 1.0 / (double)P.nb;
    t->nb = P.nb;
    t->z = P.d_z;
    t->v = v;
    t->v_old = P.d_v[(k + 2) % 3];
    t->v_new = P.d_v[(k + 1) % 3];
    t->w_prev = P.d_w[k % 2];
    t->w = P.d_w[(k + 1) % 2];
    t->x = P.d_x;
    t->tickets = reinterpret_cast<unsigned int*>(P.d_red + kTicketSlot);
    t->hist = P.d_hist;
    return cudaSuccess;
}

cudaError_t group_iteration_tail(cudaStream_t s, const IterArgs* d_tab, int members, int max_blocks) {
    FP_LAUNCHED(); k_alpha_g<<<members, 512, 0, s>>>(d_tab);
    FP_LAUNCHED(); k_zupd_g<<<dim3(max_blocks, members), kVecThreads, 0, s>>>(d_tab);
    FP_LAUNCHED(); k_vwupd_g<<<dim3(max_blocks, members), kVecThreads, 0, s>>>(d_tab);
    return cudaGetLastError();
}

cudaError_t minres_iteration(Problem& P) {
    IterArgs t;
    ApplyArgs a;
    iteration_args(P, &t, &a);
    int nparts = 0;
    cudaError_t e = launch_apply(P, a, &nparts);
    if (e != cudaSuccess) return e;
    FP_LAUNCHED(); k_alpha<<<1, 512, 0, P.stream>>>(t.sc, t.partials, nparts, t.inv_nb);
    // the last block of k_zupd runs the Givens step, the last block of
    // k_vwupd the end of the iteration (block-count tickets in d_red)
    FP_LAUNCHED(); k_zupd<<<t.nblk, kVecThreads, 0, P.stream>>>(t.sc, t.z, t.v, t.v_old, t.nb, t.partials,
                                                                 t.tickets, t.hist);
    FP_LAUNCHED(); k_vwupd<<<t.nblk, kVecThreads, 0, P.stream>>>(t.sc, t.z, t.v, t.v_new, t.w_prev, t.w, t.x,
                                                                  t.nb, t.partials, t.tickets + 1);
    return cudaGetLastError();
}

}  // namespace fp

namespace fp {

namespace {

// v = scale * (v - mean), mean = sums[c] * inv_nb (AoS components; two
// voxels per thread as in k_sum3)
template <bool SCALE>
__global__ void k_sub_mean(double* __restrict__ v, long long nb, const double* __restrict__ sums,
                           double inv_nb, double scale) {
    const double mz[3] = {sums[0] * inv_nb, sums[1] * inv_nb, sums[2] * inv_nb};
    const long long npair = nb >> 1;
    double2* v2 = reinterpret_cast<double2*>(v);
    for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < npair;
         k += (long long)gridDim.x * blockDim.x) {
#pragma unroll
        for (int h = 0; h < 3; ++h) {
            double2 x = v2[3 * k + h];
            x.x = x.x - mz[(2 * h) % 3];
            x.y = x.y - mz[(2 * h + 1) % 3];
            if (SCALE) {
                x.x *= scale;
                x.y *= scale;
            }
            v2[3 * k + h] = x;
        }
    }
    if ((nb & 1) && blockIdx.x == 0 && threadIdx.x == 0)
        for (int c = 0; c < 3; ++c) v[3 * (nb - 1) + c] = scale * (v[3 * (nb - 1) + c] - mz[c]);
}

// sums over the support of a dense SoA field, per component
__global__ void k_gather_sum(const double* __restrict__ u, long long n, const int* __restrict__ support,
                             long long nb, double* partials) {
    __shared__ double red[4 * 32];
    double acc[4] = {0, 0, 0, 0};
    for (long long s = (long long)blockIdx.x * blockDim.x + threadIdx.x; s < nb;
         s += (long long)gridDim.x * blockDim.x) {
        const long long v = support[s];
        acc[0] += u[v];
        acc[1] += u[n + v];
        acc[2] += u[2 * n + v];
    }
    double o[4];
    block_sum<4>(acc, red, o);
    if (threadIdx.x == 0)
        for (int j = 0; j < 4; ++j) partials[4LL * blockIdx.x + j] = o[j];
}

// u[c] += add[c] on a dense SoA field
__global__ void k_add_const3(double* __restrict__ u, long long n, const double* __restrict__ add) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < 3 * n;
         i += (long long)gridDim.x * blockDim.x) {
        u[i] += add[i / n];
    }
}

// f0 on a dense SoA field (src/bignonnet/BackgroundForce.cpp:14-60)
__global__ void k_background_force(const uint8_t* __restrict__ mask, long long n,
                                   const int* __restrict__ support, long long nb, double cf0,
                                   double cf1, double cf2, double cs0, double cs1, double cs2,
                                   double* __restrict__ f0) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const bool fl = mask[i] != 0;
        f0[i] = fl ? cf0 : 0.0;
        f0[n + i] = fl ? cf1 : 0.0;
        f0[2 * n + i] = fl ? cf2 : 0.0;
    }
    (void)support;
    (void)nb;
    (void)cs0;
    (void)cs1;
    (void)cs2;
}

__global__ void k_background_force_support(const int* __restrict__ support, long long nb, long long n,
                                           double cs0, double cs1, double cs2, double* __restrict__ f0) {
    for (long long s = (long long)blockIdx.x * blockDim.x + threadIdx.x; s < nb;
         s += (long long)gridDim.x * blockDim.x) {
        const long long v = support[s];
        f0[v] += cs0;
        f0[n + v] += cs1;
        f0[2 * n + v] += cs2;
    }
}

}  // namespace

// sum of (b - ax)^2 over the compact vectors, [blocks][4] partials with the sum in slot 3
__global__ void k_resnorm(const double* __restrict__ b, const double* __restrict__ ax, long long m,
                          double* partials) {
    __shared__ double red[4 * 32];
    double acc[4] = {0, 0, 0, 0};
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < m;
         i += (long long)gridDim.x * blockDim.x) {
        const double r = b[i] - ax[i];
        acc[3] += r * r;
    }
    double o[4];
    block_sum<4>(acc, red, o);
    if (threadIdx.x == 0)
        for (int j = 0; j < 4; ++j) partials[4LL * blockIdx.x + j] = o[j];
}

cudaError_t launch_resnorm(Problem& P, const double* b, const double* ax, double* out4) {
    const long long m = 3 * P.nb;
    const int blocks = vec_blocks(P, m);
    FP_LAUNCHED(); k_resnorm<<<blocks, kVecThreads, 0, P.stream>>>(b, ax, m, P.d_partials);
    FP_LAUNCHED(); k_reduce4<<<1, 512, 0, P.stream>>>(P.d_partials, blocks, out4);
    return cudaGetLastError();
}

static __global__ void k_axpby(double* __restrict__ out, double a, const double* __restrict__ x, double b,
                        const double* __restrict__ y, long long m) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < m;
         i += (long long)gridDim.x * blockDim.x)
        out[i] = a * x[i] + b * y[i];
}

cudaError_t launch_axpby(Problem& P, double* out, double a, const double* x, double b,
                         const double* y) {
    const long long m = 3 * P.nb;
    FP_LAUNCHED(); k_axpby<<<vec_blocks(P, m), kVecThreads, 0, P.stream>>>(out, a, x, b, y, m);
    return cudaGetLastError();
}

cudaError_t launch_sub_mean(Problem& P, double* v, const double* sums, double scale) {
    const int blocks = vec_blocks(P, (P.nb + 1) / 2);
    const double inv_nb = P.nb > 0 ? 1.0 / (double)P.nb : 0.0;
    FP_LAUNCHED();
    if (scale == 1.0)
        k_sub_mean<false><<<blocks, kVecThreads, 0, P.stream>>>(v, P.nb, sums, inv_nb, scale);
    else
        k_sub_mean<true><<<blocks, kVecThreads, 0, P.stream>>>(v, P.nb, sums, inv_nb, scale);
    return cudaGetLastError();
}

cudaError_t launch_gather_sum(Problem& P, const double* u_dense, double* out4) {
    const int blocks = vec_blocks(P, P.nb);
    FP_LAUNCHED(); k_gather_sum<<<blocks, kVecThreads, 0, P.stream>>>(u_dense, P.n, P.d_support, P.nb,
                                                        P.d_partials);
    FP_LAUNCHED(); k_reduce4<<<1, 512, 0, P.stream>>>(P.d_partials, blocks, out4);
    return cudaGetLastError();
}

cudaError_t launch_add_const3(Problem& P, double* u_dense, const double* add3) {
    FP_LAUNCHED(); k_add_const3<<<vec_blocks(P, 3 * P.n), kVecThreads, 0, P.stream>>>(u_dense, P.n, add3);
    return cudaGetLastError();
}

cudaError_t launch_background_force(Problem& P, const double cf[3], const double cs[3],
                                    double* f0) {
    FP_LAUNCHED(); k_background_force<<<vec_blocks(P, P.n), kVecThreads, 0, P.stream>>>(
        P.d_mask, P.n, P.d_support, P.nb, cf[0], cf[1], cf[2], cs[0], cs[1], cs[2], f0);
    FP_LAUNCHED(); k_background_force_support<<<vec_blocks(P, P.nb), kVecThreads, 0, P.stream>>>(
        P.d_support, P.nb, P.n, cs[0], cs[1], cs[2], f0);
    return cudaGetLastError();
}

}  // namespace fp
