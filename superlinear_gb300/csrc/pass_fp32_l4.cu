// FP32-bulk per-atom passes, sh_l_max = 4.
#include "pass_inst.cuh"
namespace sus2g {
SUS2G_INSTANTIATE_PASS(float, 4)
}  // namespace sus2g
