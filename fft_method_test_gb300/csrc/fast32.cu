// fast32.cu -- the specialised apply passes in FP32 (fft_fast.cuh).
#include "fast_runners.cuh"

namespace fp {
namespace fast {
FP_FAST_INSTANTIATE(float)
}  // namespace fast
}  // namespace fp
