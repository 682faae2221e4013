// fft_y32.cu -- the y passes (P2, P4) in FP32, one translation unit of the
// apply (fft_passes.cuh).
#define FP_DEFINE_Y_RUNNERS
#include "fft_passes.cuh"

namespace fp {
template cudaError_t run_ypass<float>(int, const YArgs&, dim3, int, size_t, cudaStream_t, bool);
template cudaError_t run_ypass_tma<float>(int, const CUtensorMap&, const YArgs&, const TmaTile&, int, int,
                                      size_t, cudaStream_t);
}  // namespace fp
