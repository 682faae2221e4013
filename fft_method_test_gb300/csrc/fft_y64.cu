// fft_y64.cu -- the y passes (P2, P4) in FP64, one translation unit of the
// apply (fft_passes.cuh).
#define FP_DEFINE_Y_RUNNERS
#include "fft_passes.cuh"

namespace fp {
template cudaError_t run_ypass<double>(int, const YArgs&, dim3, int, size_t, cudaStream_t, bool);
template cudaError_t run_ypass_tma<double>(int, const CUtensorMap&, const YArgs&, const TmaTile&, int, int,
                                      size_t, cudaStream_t);
}  // namespace fp
