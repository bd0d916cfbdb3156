// FP64 parameter-gradient passes, sh_l_max = 5.
#include "grad_inst.cuh"
namespace sus2g {
SUS2G_INSTANTIATE_GRAD(double, 5)
}  // namespace sus2g
