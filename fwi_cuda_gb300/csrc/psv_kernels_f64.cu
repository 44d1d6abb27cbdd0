// Time-step kernels instantiated for double wavefields.
#include "psv_kernels_impl.cuh"

namespace psv {
PSV_INSTANTIATE_STEP(double)
}  // namespace psv
