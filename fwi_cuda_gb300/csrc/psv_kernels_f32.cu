// Time-step kernels instantiated for float wavefields.
#include "psv_kernels_impl.cuh"

namespace psv {
PSV_INSTANTIATE_STEP(float)
}  // namespace psv
