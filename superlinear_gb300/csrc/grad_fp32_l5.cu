// FP32-bulk parameter-gradient passes, sh_l_max = 5.
#include "grad_inst.cuh"
namespace sus2g {
SUS2G_INSTANTIATE_GRAD(float, 5)
}  // namespace sus2g
