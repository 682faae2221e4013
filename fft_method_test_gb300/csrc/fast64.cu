// fast64.cu -- the specialised apply passes in FP64 for the power-of-two
// edges (fft_fast.cuh).
#include "fast_runners.cuh"

namespace fp {
namespace fast {
template struct Passes<double, 32>;
template struct Passes<double, 64>;
template struct Passes<double, 128>;
template struct Passes<double, 256>;
}  // namespace fast
}  // namespace fp
