// Survey plan with float wavefields.
#include "psv_plan_impl.cuh"

namespace psv {
std::unique_ptr<PlanIface> make_plan_f32(const Survey &sv, const psv_options &opt, int &status)
{
    return make_plan_t<float>(sv, opt, status);
}
}  // namespace psv
