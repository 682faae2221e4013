// kernels_setup.cu -- once-per-geometry and once-per-grid kernels:
//   * support extraction (interface voxels or all solid voxels) with a
//     per-row CSR so that the x passes can scatter/gather without a full-grid
//     index map,
//   * the energy-consistent Green tensor on the half spectrum.
#include <cuda_runtime.h>

#include <cfloat>
#include <cmath>
#include <vector>

#include "common.cuh"
#include "internal.h"

namespace fp {

// ---------------------------------------------------------------------------
// Support set (src/geometry/InterfaceVoxels.cpp:7-43,
// src/bignonnet/ForceSupport.cpp:9-25).  A solid voxel (mask == 0) is an
// interface voxel when any of its 26 periodic neighbours is fluid.  The
// reference sorts the list by flat index; the per-row count + scan + ordered
// warp compaction below produces exactly that order.
// ---------------------------------------------------------------------------

__device__ __forceinline__ bool is_support(const uint8_t* __restrict__ mask, int x, int y, int z,
                                           int nx, int ny, int nz, int mode) {
    const long long plane = (long long)nx * ny;
    if (mask[(long long)z * plane + (long long)y * nx + x] != 0) return false;
    if (mode == 1) return true;
    for (int dk = -1; dk <= 1; ++dk) {
        const int zz = (z + dk + nz) % nz;
        for (int dj = -1; dj <= 1; ++dj) {
            const int yy = (y + dj + ny) % ny;
            const uint8_t* row = mask + (long long)zz * plane + (long long)yy * nx;
            for (int di = -1; di <= 1; ++di) {
                if (di == 0 && dj == 0 && dk == 0) continue;
                const int xx = (x + di + nx) % nx;
                if (row[xx] != 0) return true;
            }
        }
    }
    return false;
}

__global__ void k_support_count(const uint8_t* __restrict__ mask, int nx, int ny, int nz,
                                long long nrows, int mode, int* row_cnt, int* row_fluid) {
    const long long r = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (r >= nrows) return;
    const int y = (int)(r % ny);
    const int z = (int)(r / ny);
    int cnt = 0, fl = 0;
    for (int x0 = 0; x0 < nx; x0 += 32) {
        const int x = x0 + lane;
        bool s = false, f = false;
        if (x < nx) {
            f = mask[r * nx + x] != 0;
            s = !f && is_support(mask, x, y, z, nx, ny, nz, mode);
        }
        cnt += __popc(__ballot_sync(0xffffffffu, s));
        fl += __popc(__ballot_sync(0xffffffffu, f));
    }
    if (lane == 0) {
        row_cnt[r] = cnt;
        row_fluid[r] = fl;
    }
}

// Single-block exclusive scan of row counts -> row_ptr[nrows + 1]; also
// totals the fluid counts into *nf.
__global__ void k_scan_rows(const int* __restrict__ cnt, const int* __restrict__ fluid,
                            long long nrows, int* row_ptr, long long* nf) {
    __shared__ long long part[1024];
    __shared__ long long fpart[1024];
    const int t = threadIdx.x;
    const long long chunk = (nrows + blockDim.x - 1) / blockDim.x;
    const long long b = t * chunk;
    const long long e = min(nrows, b + chunk);
    long long s = 0, fs = 0;
    for (long long i = b; i < e; ++i) {
        s += cnt[i];
        fs += fluid[i];
    }
    part[t] = s;
    fpart[t] = fs;
    __syncthreads();
    if (t == 0) {
        long long acc = 0, facc = 0;
        for (int i = 0; i < (int)blockDim.x; ++i) {
            const long long v = part[i];
            part[i] = acc;
            acc += v;
            facc += fpart[i];
        }
        row_ptr[nrows] = (int)acc;
        *nf = facc;
    }
    __syncthreads();
    long long acc = part[t];
    for (long long i = b; i < e; ++i) {
        row_ptr[i] = (int)acc;
        acc += cnt[i];
    }
}

__global__ void k_support_write(const uint8_t* __restrict__ mask, int nx, int ny, int nz,
                                long long nrows, int mode, const int* __restrict__ row_ptr,
                                int* support) {
    const long long r = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (r >= nrows) return;
    const int y = (int)(r % ny);
    const int z = (int)(r / ny);
    int off = row_ptr[r];
    for (int x0 = 0; x0 < nx; x0 += 32) {
        const int x = x0 + lane;
        bool s = false;
        if (x < nx) s = is_support(mask, x, y, z, nx, ny, nz, mode);
        const unsigned bal = __ballot_sync(0xffffffffu, s);
        if (s) support[off + __popc(bal & ((1u << lane) - 1u))] = (int)(r * nx + x);
        off += __popc(bal);
    }
}

cudaError_t launch_support(Problem& P) {
    const int threads = 256;
    const long long warps = P.nrows;
    const int blocks = (int)((warps * 32 + threads - 1) / threads);
    int* d_fluid = nullptr;
    long long* d_nf = nullptr;
    cudaError_t e = cudaMallocAsync(&d_fluid, sizeof(int) * P.nrows, P.stream);
    if (e != cudaSuccess) return e;
    e = cudaMallocAsync(&d_nf, sizeof(long long), P.stream);
    if (e != cudaSuccess) return e;
    k_support_count<<<blocks, threads, 0, P.stream>>>(P.d_mask, P.nx, P.ny, P.nz, P.nrows,
                                                      P.support_mode, P.d_row_cnt, d_fluid);
    k_scan_rows<<<1, 1024, 0, P.stream>>>(P.d_row_cnt, d_fluid, P.nrows, P.d_row_ptr, d_nf);
    int nb = 0;
    long long nf = 0;
    cudaMemcpyAsync(&nb, P.d_row_ptr + P.nrows, sizeof(int), cudaMemcpyDeviceToHost, P.stream);
    cudaMemcpyAsync(&nf, d_nf, sizeof(long long), cudaMemcpyDeviceToHost, P.stream);
    e = cudaStreamSynchronize(P.stream);
    if (e != cudaSuccess) return e;
    P.nb = nb;
    P.nf = nf;
    cudaFreeAsync(d_fluid, P.stream);
    cudaFreeAsync(d_nf, P.stream);
    if (P.d_support) cudaFreeAsync(P.d_support, P.stream);
    e = cudaMallocAsync(&P.d_support, sizeof(int) * (size_t)(nb > 0 ? nb : 1), P.stream);
    if (e != cudaSuccess) return e;
    k_support_write<<<blocks, threads, 0, P.stream>>>(P.d_mask, P.nx, P.ny, P.nz, P.nrows,
                                                      P.support_mode, P.d_row_ptr, P.d_support);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Green tensor (src/bignonnet/GreenOperator.cpp:95-178).
//
// G(k) = sum_{|p_i| <= P} prod_i sinc^2(pi m_i / n_i) (1/(mu q^2)) (I - q q^T / q^2)
// with unshifted m_i = k_i + p_i n_i, k_i in [0, n_i), q_i = 2 pi m_i / L_i,
// L_i = h n_i, terms with zero weight or q^2 <= DBL_EPSILON skipped, G(0) = 0.
// The per-axis factors sinc(pi m/n) and q are tabulated on the host with the
// reference's own expressions; the sums run in the reference's order with
// explicitly rounded operations (no FMA contraction), so each G(k) equals the
// reference's value.  The table stores the symmetrised
// Gs(k) = (G(k) + G(-k)) / 2 on the half spectrum kx in [0, nx/2]: the
// reference keeps only Re(IFFT(G * F)), which is the IFFT of Gs * F.
// ---------------------------------------------------------------------------

struct GreenArgs {
    int nx, ny, nz, nxh, np;  // np = 2P + 1
    double mu;
    const double* sx;  // [nx][np] sinc values
    const double* qx;  // [nx][np]
    const double* sy;
    const double* qy;
    const double* sz;
    const double* qz;
    double* g64;
    float* g32;
    long long nh;
};

__device__ __forceinline__ void green_sum(const GreenArgs& a, int kx, int ky, int kz, double g[6]) {
    for (int i = 0; i < 6; ++i) g[i] = 0.0;
    if (kx == 0 && ky == 0 && kz == 0) return;
    const double* sxr = a.sx + (long long)kx * a.np;
    const double* qxr = a.qx + (long long)kx * a.np;
    const double* syr = a.sy + (long long)ky * a.np;
    const double* qyr = a.qy + (long long)ky * a.np;
    const double* szr = a.sz + (long long)kz * a.np;
    const double* qzr = a.qz + (long long)kz * a.np;
    for (int ix = 0; ix < a.np; ++ix) {
        const double sx = sxr[ix], qx = qxr[ix];
        const double wx = __dmul_rn(sx, sx);
        const double qxx = __dmul_rn(qx, qx);
        for (int iy = 0; iy < a.np; ++iy) {
            const double sy = syr[iy], qy = qyr[iy];
            const double wxy = __dmul_rn(wx, __dmul_rn(sy, sy));
            const double qxy2 = __dadd_rn(qxx, __dmul_rn(qy, qy));
            for (int iz = 0; iz < a.np; ++iz) {
                const double sz = szr[iz], qz = qzr[iz];
                const double weight = __dmul_rn(wxy, __dmul_rn(sz, sz));
                if (weight == 0.0) continue;
                const double q2 = __dadd_rn(qxy2, __dmul_rn(qz, qz));
                if (q2 <= DBL_EPSILON) continue;
                const double inv_mu_q2 = __ddiv_rn(1.0, __dmul_rn(a.mu, q2));
                const double inv_q2 = __ddiv_rn(1.0, q2);
                const double fac = __dmul_rn(weight, inv_mu_q2);
                g[0] = __dadd_rn(g[0], __dmul_rn(fac, __dsub_rn(1.0, __dmul_rn(qxx, inv_q2))));
                g[1] = __dadd_rn(g[1], __dmul_rn(fac, __dmul_rn(__dmul_rn(-qx, qy), inv_q2)));
                g[2] = __dadd_rn(g[2], __dmul_rn(fac, __dmul_rn(__dmul_rn(-qx, qz), inv_q2)));
                g[3] = __dadd_rn(g[3], __dmul_rn(fac, __dsub_rn(1.0, __dmul_rn(__dmul_rn(qy, qy), inv_q2))));
                g[4] = __dadd_rn(g[4], __dmul_rn(fac, __dmul_rn(__dmul_rn(-qy, qz), inv_q2)));
                g[5] = __dadd_rn(g[5], __dmul_rn(fac, __dsub_rn(1.0, __dmul_rn(__dmul_rn(qz, qz), inv_q2))));
            }
        }
    }
}

__global__ void k_green(GreenArgs a) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= a.nh) return;
    const int kx = (int)(t % a.nxh);
    const long long rest = t / a.nxh;
    const int ky = (int)(rest % a.ny);
    const int kz = (int)(rest / a.ny);
    double g[6], gb[6];
    green_sum(a, kx, ky, kz, g);
    const int bx = kx == 0 ? 0 : a.nx - kx;
    const int by = ky == 0 ? 0 : a.ny - ky;
    const int bz = kz == 0 ? 0 : a.nz - kz;
    green_sum(a, bx, by, bz, gb);
    for (int c = 0; c < 6; ++c) {
        const double v = 0.5 * (g[c] + gb[c]);
        if (a.g64) a.g64[c * a.nh + t] = v;
        if (a.g32) a.g32[c * a.nh + t] = (float)v;
    }
}

static double host_sinc(double x) {
    if (std::abs(x) < 1e-12) return 1.0;
    return std::sin(x) / x;
}

cudaError_t launch_green(Problem& P) {
    const int Pr = P.p_radius < 0 ? 0 : P.p_radius;
    const int np = 2 * Pr + 1;
    const double kPi = 3.14159265358979323846;
    auto tab = [&](int n, std::vector<double>& s, std::vector<double>& q) {
        const double L = P.h * (double)n;
        s.resize((size_t)n * np);
        q.resize((size_t)n * np);
        for (int k = 0; k < n; ++k)
            for (int p = -Pr; p <= Pr; ++p) {
                const long long m = (long long)k + (long long)p * n;
                s[(size_t)k * np + (p + Pr)] = host_sinc(kPi * (double)m / (double)n);
                q[(size_t)k * np + (p + Pr)] = (2.0 * kPi * (double)m) / L;
            }
    };
    std::vector<double> hsx, hqx, hsy, hqy, hsz, hqz;
    tab(P.nx, hsx, hqx);
    tab(P.ny, hsy, hqy);
    tab(P.nz, hsz, hqz);
    const size_t tx = hsx.size(), ty = hsy.size(), tz = hsz.size();
    double* d = nullptr;
    cudaError_t e = cudaMalloc(&d, sizeof(double) * 2 * (tx + ty + tz));
    if (e != cudaSuccess) return e;
    double* dsx = d;
    double* dqx = dsx + tx;
    double* dsy = dqx + tx;
    double* dqy = dsy + ty;
    double* dsz = dqy + ty;
    double* dqz = dsz + tz;
    cudaMemcpy(dsx, hsx.data(), sizeof(double) * tx, cudaMemcpyHostToDevice);
    cudaMemcpy(dqx, hqx.data(), sizeof(double) * tx, cudaMemcpyHostToDevice);
    cudaMemcpy(dsy, hsy.data(), sizeof(double) * ty, cudaMemcpyHostToDevice);
    cudaMemcpy(dqy, hqy.data(), sizeof(double) * ty, cudaMemcpyHostToDevice);
    cudaMemcpy(dsz, hsz.data(), sizeof(double) * tz, cudaMemcpyHostToDevice);
    cudaMemcpy(dqz, hqz.data(), sizeof(double) * tz, cudaMemcpyHostToDevice);
    GreenArgs a{};
    a.nx = P.nx;
    a.ny = P.ny;
    a.nz = P.nz;
    a.nxh = P.nxh;
    a.np = np;
    a.mu = P.mu;
    a.sx = dsx;
    a.qx = dqx;
    a.sy = dsy;
    a.qy = dqy;
    a.sz = dsz;
    a.qz = dqz;
    a.g64 = P.d_green64;
    a.g32 = P.d_green32;
    a.nh = P.nh;
    const int threads = 128;
    const long long blocks = (P.nh + threads - 1) / threads;
    k_green<<<(unsigned)blocks, threads, 0, P.stream>>>(a);
    e = cudaGetLastError();
    cudaStreamSynchronize(P.stream);
    cudaFree(d);
    return e;
}

}  // namespace fp
