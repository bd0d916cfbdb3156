// FP64 parameter-gradient passes, sh_l_max = 0, 1, 2.
#include "grad_inst.cuh"
namespace sus2g {
SUS2G_INSTANTIATE_GRAD(double, 0)
SUS2G_INSTANTIATE_GRAD(double, 1)
SUS2G_INSTANTIATE_GRAD(double, 2)
}  // namespace sus2g
