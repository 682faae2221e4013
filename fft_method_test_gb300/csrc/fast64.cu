// fast64.cu -- the specialised apply passes in FP64 (fft_fast.cuh).
#include "fast_runners.cuh"

namespace fp {
namespace fast {
FP_FAST_INSTANTIATE(double)
}  // namespace fast
}  // namespace fp
