// fft_x64.cu -- the x passes (P1, P5) in FP64, one translation unit of the
// apply (fft_passes.cuh).
#define FP_DEFINE_X_RUNNERS
#include "fft_passes.cuh"

namespace fp {
template cudaError_t run_xfwd<double>(int, const XArgs&, int, int, size_t, cudaStream_t);
template cudaError_t run_xinv<double>(int, const XArgs&, int, int, size_t, cudaStream_t);
template cudaError_t run_xinv_bulk<double>(int, const XArgs&, int, int, int, size_t, cudaStream_t);
}  // namespace fp
