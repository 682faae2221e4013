// fast64n.cu -- the specialised apply passes in FP64 for the edges with a
// factor 3 or 5: 48, 80, 96, 160 (fft_fast.cuh).
#include "fast_runners.cuh"

namespace fp {
namespace fast {
template struct Passes<double, 48>;
template struct Passes<double, 80>;
template struct Passes<double, 96>;
template struct Passes<double, 160>;
}  // namespace fast
}  // namespace fp
