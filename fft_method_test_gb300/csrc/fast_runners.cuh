// fast_runners.cuh -- launch runners of the specialised apply passes
// (fft_fast.cuh), instantiated per precision by fast32.cu and fast64.cu so
// that the two build in parallel.
#pragma once

#include "fft_fast.cuh"
#include "fft_passes.cuh"

namespace fp {
namespace fast {

#define FP_FAST_SWITCH(n, CALL)            \
    switch (n) {                           \
        case 32: CALL(32); break;          \
        case 64: CALL(64); break;          \
        case 128: CALL(128); break;        \
        case 256: CALL(256); break;        \
        default: return cudaErrorInvalidValue; \
    }

template <typename T>
cudaError_t run_xfwd(int n, const FastArgs& a, int grid, int threads, size_t smem, cudaStream_t s) {
#define FP_CALL(N) FP_RUN((k_fx_fwd<T, N>), grid, threads, smem, s, a)
    FP_FAST_SWITCH(n, FP_CALL)
#undef FP_CALL
    return cudaGetLastError();
}

template <typename T>
cudaError_t run_xinv(int n, const FastArgs& a, int stage_bytes, int grid, int threads, size_t smem,
                     cudaStream_t s) {
#define FP_CALL(N) FP_RUN((k_fx_inv<T, N>), grid, threads, smem, s, a, stage_bytes)
    FP_FAST_SWITCH(n, FP_CALL)
#undef FP_CALL
    return cudaGetLastError();
}

template <typename T>
cudaError_t run_y(int n, int dir, const FastArgs& a, dim3 grid, cudaStream_t s) {
    constexpr int TX = col_tx<T>();
#define FP_CALL(N)                                                                       \
    if (dir < 0)                                                                         \
        FP_RUN((k_fcol_y<T, N, -1, TX>), grid, TX * Split<N>::R2, 0, s, a);              \
    else                                                                                 \
        FP_RUN((k_fcol_y<T, N, +1, TX>), grid, TX * Split<N>::R2, 0, s, a)
    FP_FAST_SWITCH(n, FP_CALL)
#undef FP_CALL
    return cudaGetLastError();
}

template <typename T>
cudaError_t run_z(int n, int stages, const CUtensorMap& spec_map, const CUtensorMap& green_map,
                  const FastArgs& a, dim3 grid, size_t smem, cudaStream_t s) {
    constexpr int TX = z_tx<T>();
#define FP_CALL(N)                                                                                \
    if (stages == 1)                                                                              \
        FP_RUN((k_fz<T, N, TX, 1>), grid, 3 * TX * Split<N>::R2, smem, s, spec_map, green_map, a); \
    else                                                                                          \
        FP_RUN((k_fz<T, N, TX, 2>), grid, 3 * TX * Split<N>::R2, smem, s, spec_map, green_map, a)
    FP_FAST_SWITCH(n, FP_CALL)
#undef FP_CALL
    return cudaGetLastError();
}

template <typename T>
int z_blocks_per_sm(int n, int stages, size_t smem) {
    constexpr int TX = z_tx<T>();
    int nb = 0;
#define FP_CALL(N)                                                                            \
    {                                                                                         \
        static std::atomic<unsigned long long> f1_{0}, f2_{0};                                \
        if (stages == 1) {                                                                    \
            ensure_max_smem(k_fz<T, N, TX, 1>, f1_);                                          \
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_fz<T, N, TX, 1>,             \
                                                          3 * TX * Split<N>::R2, smem);        \
        } else {                                                                              \
            ensure_max_smem(k_fz<T, N, TX, 2>, f2_);                                          \
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_fz<T, N, TX, 2>,             \
                                                          3 * TX * Split<N>::R2, smem);        \
        }                                                                                     \
    }
    switch (n) {
        case 32: FP_CALL(32); break;
        case 64: FP_CALL(64); break;
        case 128: FP_CALL(128); break;
        case 256: FP_CALL(256); break;
        default: break;
    }
#undef FP_CALL
    return nb > 0 ? nb : 1;
}

template <typename T>
int x_blocks_per_sm(int n, bool inverse, int threads, size_t smem) {
    int nb = 0;
#define FP_CALL(N)                                                                                \
    {                                                                                             \
        static std::atomic<unsigned long long> f_{0}, i_{0};                                      \
        if (inverse) {                                                                            \
            ensure_max_smem(k_fx_inv<T, N>, i_);                                                  \
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_fx_inv<T, N>, threads, smem);    \
        } else {                                                                                  \
            ensure_max_smem(k_fx_fwd<T, N>, f_);                                                  \
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_fx_fwd<T, N>, threads, smem);    \
        }                                                                                         \
    }
    switch (n) {
        case 32: FP_CALL(32); break;
        case 64: FP_CALL(64); break;
        case 128: FP_CALL(128); break;
        case 256: FP_CALL(256); break;
        default: break;
    }
#undef FP_CALL
    return nb > 0 ? nb : 1;
}

#define FP_FAST_INSTANTIATE(T)                                                                      \
    template cudaError_t run_xfwd<T>(int, const FastArgs&, int, int, size_t, cudaStream_t);         \
    template cudaError_t run_xinv<T>(int, const FastArgs&, int, int, int, size_t, cudaStream_t);    \
    template cudaError_t run_y<T>(int, int, const FastArgs&, dim3, cudaStream_t);                   \
    template cudaError_t run_z<T>(int, int, const CUtensorMap&, const CUtensorMap&, const FastArgs&, \
                                  dim3, size_t, cudaStream_t);                                      \
    template int x_blocks_per_sm<T>(int, bool, int, size_t);                                      \
    template int z_blocks_per_sm<T>(int, int, size_t);

}  // namespace fast
}  // namespace fp
