// fast_runners.cuh -- launch runners of the specialised apply passes
// (fft_fast.cuh), one Passes<T, N> per precision and grid edge, instantiated
// by fast32.cu / fast64.cu (powers of two) and fast32n.cu / fast64n.cu (48,
// 80, 96, 160) so that the four build in parallel.
#pragma once

#include <atomic>

#include "fft_fast.cuh"
#include "fft_passes.cuh"

namespace fp {
namespace fast {

template <typename T, int N>
cudaError_t Passes<T, N>::xfwd(const FastArgs& a, int grid, int threads, size_t smem, cudaStream_t s) {
    FP_RUN((k_fx_fwd<T, N>), grid, threads, smem, s, a);
    return cudaGetLastError();
}

template <typename T, int N>
cudaError_t Passes<T, N>::xinv(const FastArgs& a, int stage_bytes, int grid, int threads, size_t smem,
                               cudaStream_t s) {
    FP_RUN((k_fx_inv<T, N>), grid, threads, smem, s, a, stage_bytes);
    return cudaGetLastError();
}

template <typename T, int N>
cudaError_t Passes<T, N>::y(int dir, const FastArgs& a, dim3 grid, cudaStream_t s) {
    constexpr int TX = col_tx<T>();
    if (dir < 0)
        FP_RUN((k_fcol_y<T, N, -1, TX>), grid, TX * Split<N>::TPL, 0, s, a);
    else
        FP_RUN((k_fcol_y<T, N, +1, TX>), grid, TX * Split<N>::TPL, 0, s, a);
    return cudaGetLastError();
}

template <typename T, int N>
cudaError_t Passes<T, N>::z(int stages, const CUtensorMap& spec_map, const CUtensorMap& green_map,
                            const FastArgs& a, dim3 grid, size_t smem, cudaStream_t s) {
    constexpr int TX = z_tx<T>();
    if (stages == 1)
        FP_RUN((k_fz<T, N, TX, 1>), grid, 3 * TX * Split<N>::TPL, smem, s, spec_map, green_map, a);
    else
        FP_RUN((k_fz<T, N, TX, 2>), grid, 3 * TX * Split<N>::TPL, smem, s, spec_map, green_map, a);
    return cudaGetLastError();
}

template <typename T, int N>
int Passes<T, N>::z_per_sm(int stages, size_t smem) {
    constexpr int TX = z_tx<T>();
    static std::atomic<unsigned long long> f1{0}, f2{0};
    int nb = 0;
    if (stages == 1) {
        ensure_max_smem(k_fz<T, N, TX, 1>, f1);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_fz<T, N, TX, 1>, 3 * TX * Split<N>::TPL, smem);
    } else {
        ensure_max_smem(k_fz<T, N, TX, 2>, f2);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_fz<T, N, TX, 2>, 3 * TX * Split<N>::TPL, smem);
    }
    return nb > 0 ? nb : 1;
}

template <typename T, int N>
int Passes<T, N>::x_per_sm(bool inverse, int threads, size_t smem) {
    static std::atomic<unsigned long long> fi{0}, ff{0};
    int nb = 0;
    if (inverse) {
        ensure_max_smem(k_fx_inv<T, N>, fi);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_fx_inv<T, N>, threads, smem);
    } else {
        ensure_max_smem(k_fx_fwd<T, N>, ff);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_fx_fwd<T, N>, threads, smem);
    }
    return nb > 0 ? nb : 1;
}

}  // namespace fast
}  // namespace fp
