// FP64 parameter-gradient passes, sh_l_max = 3.
#include "grad_inst.cuh"
namespace sus2g {
SUS2G_INSTANTIATE_GRAD(double, 3)
}  // namespace sus2g
