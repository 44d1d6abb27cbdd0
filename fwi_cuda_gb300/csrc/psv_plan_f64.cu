// Survey plan with double wavefields.
#include "psv_plan_impl.cuh"

namespace psv {
std::unique_ptr<PlanIface> make_plan_f64(const Survey &sv, const psv_options &opt, int &status)
{
    return make_plan_t<double>(sv, opt, status);
}
}  // namespace psv
