// FP32-bulk parameter-gradient passes, sh_l_max = 0, 1, 2.
#include "grad_inst.cuh"
namespace sus2g {
SUS2G_INSTANTIATE_GRAD(float, 0)
SUS2G_INSTANTIATE_GRAD(float, 1)
SUS2G_INSTANTIATE_GRAD(float, 2)
}  // namespace sus2g
