// fft_z32.cu -- the register-fed z pass (P3; also the forward-only and
// inverse-only z transforms) in FP32, one translation unit of the apply
// (fft_passes.cuh).
#define FP_DEFINE_Z_RUNNERS
#include "fft_passes.cuh"

namespace fp {
template cudaError_t run_zgreen<float>(int, const ZArgs&, dim3, int, size_t, cudaStream_t, bool);
}  // namespace fp
