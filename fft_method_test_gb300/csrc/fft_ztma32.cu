// fft_ztma32.cu -- the TMA-fed z pass (P3) in FP32, one translation unit of
// the apply (fft_passes.cuh).
#define FP_DEFINE_ZTMA_RUNNERS
#include "fft_passes.cuh"

namespace fp {
template cudaError_t run_zgreen_tma<float>(const CUtensorMap&, const ZArgs&, const TmaTile&, int, int,
                                       size_t, cudaStream_t);
}  // namespace fp
