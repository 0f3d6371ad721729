// lg_forces_mixed.cu -- mixed-precision force kernel.
#include "lg_common.cuh"
#include "lg_kernels.h"

namespace lg {
bool mixed_available() { return false; }
void launch_forces_mixed(int, const Params &, const StateView &, const PairView &, const BondView &, double, double, int,
                         cudaStream_t) {}
}  // namespace lg
