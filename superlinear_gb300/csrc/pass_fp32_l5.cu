// FP32-bulk per-atom passes, sh_l_max = 5.
#include "pass_inst.cuh"
namespace sus2g {
SUS2G_INSTANTIATE_PASS(float, 5)
}  // namespace sus2g
