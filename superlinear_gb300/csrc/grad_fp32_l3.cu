// FP32-bulk parameter-gradient passes, sh_l_max = 3.
#include "grad_inst.cuh"
namespace sus2g {
SUS2G_INSTANTIATE_GRAD(float, 3)
}  // namespace sus2g
