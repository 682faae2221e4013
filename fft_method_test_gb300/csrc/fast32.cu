// fast32.cu -- the specialised apply passes in FP32 for the power-of-two
// edges (fft_fast.cuh).
#include "fast_runners.cuh"

namespace fp {
namespace fast {
template struct Passes<float, 32>;
template struct Passes<float, 64>;
template struct Passes<float, 128>;
template struct Passes<float, 256>;
}  // namespace fast
}  // namespace fp
