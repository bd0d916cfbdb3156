// FP64 per-atom passes, sh_l_max = 4.
#include "pass_inst.cuh"
namespace sus2g {
SUS2G_INSTANTIATE_PASS(double, 4)
}  // namespace sus2g
