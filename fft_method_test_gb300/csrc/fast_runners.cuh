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
cudaError_t Passes<T, N>::xfwd(const FastArgs& a, dim3 grid, int threads, size_t smem, cudaStream_t s) {
    if (a.group)
        FP_RUN((k_fx_fwd<T, N, true>), grid, threads, smem, s, a);
    else
        FP_RUN((k_fx_fwd<T, N, false>), grid, threads, smem, s, a);
    return cudaGetLastError();
}

template <typename T, int N>
cudaError_t Passes<T, N>::xinv(const FastArgs& a, int stage_bytes, dim3 grid, int threads, size_t smem,
                               cudaStream_t s) {
    if (a.group)
        FP_RUN((k_fx_inv<T, N, true>), grid, threads, smem, s, a, stage_bytes);
    else
        FP_RUN((k_fx_inv<T, N, false>), grid, threads, smem, s, a, stage_bytes);
    return cudaGetLastError();
}

template <typename T, int N>
cudaError_t Passes<T, N>::y(int dir, const FastArgs& a, dim3 grid, cudaStream_t s) {
    constexpr int TX = col_tx<T>();
    constexpr int NT = TX * Split<N>::TPL;
    if (a.group) {
        if (dir < 0)
            FP_RUN((k_fcol_y<T, N, -1, TX, true>), grid, NT, 0, s, a);
        else
            FP_RUN((k_fcol_y<T, N, +1, TX, true>), grid, NT, 0, s, a);
    } else {
        if (dir < 0)
            FP_RUN((k_fcol_y<T, N, -1, TX, false>), grid, NT, 0, s, a);
        else
            FP_RUN((k_fcol_y<T, N, +1, TX, false>), grid, NT, 0, s, a);
    }
    return cudaGetLastError();
}

template <typename T, int N>
cudaError_t Passes<T, N>::z(int stages, const CUtensorMap& spec_map, const CUtensorMap& green_map,
                            const FastArgs& a, dim3 grid, size_t smem, cudaStream_t s) {
    constexpr int TX = z_tx<T>();
    constexpr int NT = 3 * TX * Split<N>::TPL;
    if (a.group) {
        if (stages == 1)
            FP_RUN((k_fz<T, N, TX, 1, true>), grid, NT, smem, s, spec_map, green_map, a);
        else
            FP_RUN((k_fz<T, N, TX, 2, true>), grid, NT, smem, s, spec_map, green_map, a);
    } else {
        if (stages == 1)
            FP_RUN((k_fz<T, N, TX, 1, false>), grid, NT, smem, s, spec_map, green_map, a);
        else
            FP_RUN((k_fz<T, N, TX, 2, false>), grid, NT, smem, s, spec_map, green_map, a);
    }
    return cudaGetLastError();
}

template <typename T, int N>
cudaError_t Passes<T, N>::z_shared(const FastArgs& a, int grid, size_t smem, cudaStream_t s) {
    constexpr int TX = z_tx<T>();
    FP_RUN((k_fz_shared<T, N, TX>), grid, 3 * TX * Split<N>::TPL, smem, s, a);
    return cudaGetLastError();
}

template <typename T, int N>
int Passes<T, N>::z_per_sm(int stages, size_t smem) {
    constexpr int TX = z_tx<T>();
    static std::atomic<unsigned long long> f1{0}, f2{0};
    int nb = 0;
    if (stages == 1) {
        ensure_max_smem(k_fz<T, N, TX, 1, false>, f1);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_fz<T, N, TX, 1, false>, 3 * TX * Split<N>::TPL,
                                                      smem);
    } else {
        ensure_max_smem(k_fz<T, N, TX, 2, false>, f2);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_fz<T, N, TX, 2, false>, 3 * TX * Split<N>::TPL,
                                                      smem);
    }
    return nb > 0 ? nb : 1;
}

template <typename T, int N>
int Passes<T, N>::x_per_sm(bool inverse, int threads, size_t smem) {
    static std::atomic<unsigned long long> fi{0}, ff{0};
    int nb = 0;
    if (inverse) {
        ensure_max_smem(k_fx_inv<T, N, false>, fi);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_fx_inv<T, N, false>, threads, smem);
    } else {
        ensure_max_smem(k_fx_fwd<T, N, false>, ff);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_fx_fwd<T, N, false>, threads, smem);
    }
    return nb > 0 ? nb : 1;
}

}  // namespace fast
}  // namespace fp
