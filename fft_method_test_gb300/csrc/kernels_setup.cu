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

// mask[i] = (ids[i] == fluid_id) for one chunk of material ids (u16 or u32)
template <typename I>
__global__ void k_ids_to_mask(const I* __restrict__ ids, long long count, uint32_t fluid_id,
                              uint8_t* __restrict__ mask) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < count;
         i += (long long)gridDim.x * blockDim.x)
        mask[i] = (uint32_t)ids[i] == fluid_id ? 1 : 0;
}

cudaError_t launch_ids_to_mask(const void* ids, int id_bytes, long long count, uint32_t fluid_id,
                               uint8_t* mask, cudaStream_t stream) {
    long long blocks = (count + 255) / 256;
    if (blocks > 65535LL * 8) blocks = 65535LL * 8;
    if (blocks < 1) blocks = 1;
    FP_LAUNCHED();
    if (id_bytes == 2)
        k_ids_to_mask<uint16_t><<<(unsigned)blocks, 256, 0, stream>>>(
            static_cast<const uint16_t*>(ids), count, fluid_id, mask);
    else
        k_ids_to_mask<uint32_t><<<(unsigned)blocks, 256, 0, stream>>>(
            static_cast<const uint32_t*>(ids), count, fluid_id, mask);
    return cudaGetLastError();
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
    FP_LAUNCHED(); k_support_count<<<blocks, threads, 0, P.stream>>>(P.d_mask, P.nx, P.ny, P.nz, P.nrows,
                                                      P.support_mode, P.d_row_cnt, d_fluid);
    FP_LAUNCHED(); k_scan_rows<<<1, 1024, 0, P.stream>>>(P.d_row_cnt, d_fluid, P.nrows, P.d_row_ptr, d_nf);
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
    FP_LAUNCHED(); k_support_write<<<blocks, threads, 0, P.stream>>>(P.d_mask, P.nx, P.ny, P.nz, P.nrows,
                                                      P.support_mode, P.d_row_ptr, P.d_support);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Green tensor (src/bignonnet/GreenOperator.cpp:95-178).
//
// G(k) = sum_{|p_i| <= P} prod_i sinc^2(pi m_i / n_i) (1/(mu q^2)) (I - q q^T / q^2)
// with unshifted m_i = k_i + p_i n_i, k_i in [0, n_i), q_i = 2 pi m_i / L_i,
// L_i = h n_i, terms with zero weight or q^2 <= DBL_EPSILON skipped, G(0) = 0.
//
// The table holds the symmetrised Gs(k) = (G(k) + G(-k)) / 2 on the half
// spectrum kx in [0, nx/2]: the reference keeps only Re(IFFT(G * F)), which is
// the IFFT of Gs * F.  Because a term depends on m only through m m^T and
// |m|^2, G(-k) is the sum over the same terms m = k + p n with the window
// p_i in [-P-1, P-1] on every axis where k_i != 0 (and [-P, P] where k_i = 0).
// One loop over the union window [-P-1, P]^3 therefore evaluates each term
// once with coefficient ([p in W^3] + [p in W'^3]) / 2.
// The per-axis factors sinc(pi m/n) and q_i are tabulated on the host with the
// reference's own expressions.
// ---------------------------------------------------------------------------

__global__ void k_green(GreenArgs a) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= a.nh) return;
    const int kx = (int)(t % a.rs);
    const long long rest = t / a.rs;
    if (kx >= a.nxh) {  // row padding
        for (int c = 0; c < 6; ++c) {
            if (a.g64) a.g64[c * a.nh + t] = 0.0;
            if (a.g32) a.g32[c * a.nh + t] = 0.0f;
        }
        return;
    }
    const int ky = (int)(rest % a.ny);
    const int kz = (int)(rest / a.ny);
    double s0 = 0, sxx = 0, syy = 0, szz = 0, sxy = 0, sxz = 0, syz = 0;
    if (!(kx == 0 && ky == 0 && kz == 0)) {
        const int P = a.pr;
        const double* sxr = a.sx + (long long)kx * a.nw;
        const double* qxr = a.qx + (long long)kx * a.nw;
        const double* syr = a.sy + (long long)ky * a.nw;
        const double* qyr = a.qy + (long long)ky * a.nw;
        const double* szr = a.sz + (long long)kz * a.nw;
        const double* qzr = a.qz + (long long)kz * a.nw;
        const double inv_mu = 1.0 / a.mu;
        for (int ix = 0; ix < a.nw; ++ix) {
            const int px = ix - P - 1;
            // membership of p in W = [-P, P] and in W' (shifted where k != 0)
            const int ax = (px >= -P);
            const int bx = kx != 0 ? (px <= P - 1) : ax;
            if (!(ax | bx)) continue;
            const double wx = sxr[ix] * sxr[ix];
            const double qxv = qxr[ix];
            const double qxx = qxv * qxv;
            for (int iy = 0; iy < a.nw; ++iy) {
                const int py = iy - P - 1;
                const int ay = ax & (py >= -P);
                const int by = bx & (ky != 0 ? (py <= P - 1) : (py >= -P));
                if (!(ay | by)) continue;
                const double wxy = wx * (syr[iy] * syr[iy]);
                const double qyv = qyr[iy];
                const double qyy = qyv * qyv;
                const double qxy2 = qxx + qyy;
                const double qxqy = qxv * qyv;
                for (int iz = 0; iz < a.nw; ++iz) {
                    const int pz = iz - P - 1;
                    const int az = ay & (pz >= -P);
                    const int bz = by & (kz != 0 ? (pz <= P - 1) : (pz >= -P));
                    const int cnt = az + bz;
                    if (cnt == 0) continue;
                    const double weight = wxy * (szr[iz] * szr[iz]);
                    if (weight == 0.0) continue;
                    const double qzv = qzr[iz];
                    const double q2 = qxy2 + qzv * qzv;
                    if (q2 <= DBL_EPSILON) continue;
                    const double inv_q2 = __drcp_rn(q2);
                    const double fac = (0.5 * cnt) * weight * inv_q2 * inv_mu;
                    const double f2 = fac * inv_q2;
                    s0 += fac;
                    sxx += f2 * qxx;
                    syy += f2 * qyy;
                    szz += f2 * (qzv * qzv);
                    sxy += f2 * qxqy;
                    sxz += f2 * (qxv * qzv);
                    syz += f2 * (qyv * qzv);
                }
            }
        }
    }
    const double g[6] = {s0 - sxx, -sxy, -sxz, s0 - syy, -syz, s0 - szz};
    for (int c = 0; c < 6; ++c) {
        if (a.g64) a.g64[c * a.nh + t] = g[c];
        if (a.g32) a.g32[c * a.nh + t] = (float)g[c];
    }
}

static double host_sinc(double x) {
    if (std::abs(x) < 1e-12) return 1.0;
    return std::sin(x) / x;
}

cudaError_t launch_green(Problem& P, double* g64, float* g32) {
    const int Pr = P.p_radius < 0 ? 0 : P.p_radius;
    const int nw = 2 * Pr + 2;
    const double kPi = 3.14159265358979323846;
    auto tab = [&](int n, std::vector<double>& s, std::vector<double>& q) {
        const double L = P.h * (double)n;
        s.resize((size_t)n * nw);
        q.resize((size_t)n * nw);
        for (int k = 0; k < n; ++k)
            for (int i = 0; i < nw; ++i) {
                const long long p = i - Pr - 1;
                const long long m = (long long)k + p * n;
                s[(size_t)k * nw + i] = host_sinc(kPi * (double)m / (double)n);
                q[(size_t)k * nw + i] = (2.0 * kPi * (double)m) / L;
            }
    };
    std::vector<double> hsx, hqx, hsy, hqy, hsz, hqz;
    tab(P.nx, hsx, hqx);
    tab(P.ny, hsy, hqy);
    tab(P.nz, hsz, hqz);
    const size_t tx = hsx.size(), ty = hsy.size(), tz = hsz.size();
    double* d = nullptr;
    cudaError_t e = cudaMallocAsync(reinterpret_cast<void**>(&d), sizeof(double) * 2 * (tx + ty + tz),
                                    P.stream);
    if (e != cudaSuccess) return e;
    double* dsx = d;
    double* dqx = dsx + tx;
    double* dsy = dqx + tx;
    double* dqy = dsy + ty;
    double* dsz = dqy + ty;
    double* dqz = dsz + tz;
    cudaMemcpyAsync(dsx, hsx.data(), sizeof(double) * tx, cudaMemcpyHostToDevice, P.stream);
    cudaMemcpyAsync(dqx, hqx.data(), sizeof(double) * tx, cudaMemcpyHostToDevice, P.stream);
    cudaMemcpyAsync(dsy, hsy.data(), sizeof(double) * ty, cudaMemcpyHostToDevice, P.stream);
    cudaMemcpyAsync(dqy, hqy.data(), sizeof(double) * ty, cudaMemcpyHostToDevice, P.stream);
    cudaMemcpyAsync(dsz, hsz.data(), sizeof(double) * tz, cudaMemcpyHostToDevice, P.stream);
    cudaMemcpyAsync(dqz, hqz.data(), sizeof(double) * tz, cudaMemcpyHostToDevice, P.stream);
    GreenArgs a{};
    a.nx = P.nx;
    a.ny = P.ny;
    a.nz = P.nz;
    a.nxh = P.nxh;
    a.rs = P.rs;
    a.nw = nw;
    a.pr = Pr;
    a.mu = P.mu;
    a.sx = dsx;
    a.qx = dqx;
    a.sy = dsy;
    a.qy = dqy;
    a.sz = dsz;
    a.qz = dqz;
    a.g64 = g64;
    a.g32 = g32;
    a.nh = P.nh;
    e = launch_green_kernel(a, P.stream);
    cudaFreeAsync(d, P.stream);
    cudaStreamSynchronize(P.stream);  // the host tables above must outlive their copies
    return e;
}

cudaError_t launch_green_kernel(const GreenArgs& a, cudaStream_t stream) {
    const int threads = 128;
    const long long blocks = (a.nh + threads - 1) / threads;
    FP_LAUNCHED(); k_green<<<(unsigned)blocks, threads, 0, stream>>>(a);
    return cudaGetLastError();
}

}  // namespace fp
