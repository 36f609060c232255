// Tensor-core (tcgen05) kernels of the mixed-precision path.
#include "lqg_internal.cuh"

namespace lqg {

bool tc_available() { return false; }

void launch_scales_mixed(WaveArgs &, cudaStream_t) {}
void launch_products_mixed(WaveArgs &, cudaStream_t, const int *, int) {}

}  // namespace lqg
