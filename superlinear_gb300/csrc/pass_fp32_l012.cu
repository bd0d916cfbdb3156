// FP32-bulk per-atom passes, sh_l_max = 0, 1, 2.
#include "pass_inst.cuh"
namespace sus2g {
SUS2G_INSTANTIATE_PASS(float, 0)
SUS2G_INSTANTIATE_PASS(float, 1)
SUS2G_INSTANTIATE_PASS(float, 2)
}  // namespace sus2g
