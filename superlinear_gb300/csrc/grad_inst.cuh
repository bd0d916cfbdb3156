// Instantiation body for the parameter-gradient passes; included by grad_fp32.cu and grad_fp64.cu.
#include <algorithm>
#include <stdexcept>
#include <string>

#include "pass_launch.h"

namespace sus2g {

template <>
cudaError_t upload_grad_constants<PASS_REAL>() { return sph_norm_upload(); }

namespace {
constexpr int kGradWarps = 2;
using GradKernel = void (*)(GradArgs<PASS_REAL>);

template <int L>
GradKernel grad_kernel_mode(int mode) {
  constexpr bool kKahan = sizeof(PASS_REAL) == 4;
  switch (mode) {
    case kGradOuter: return grad_pass_kernel<L, PASS_REAL, kGradOuter, kKahan>;
    case kGradGateForward: return grad_pass_kernel<L, PASS_REAL, kGradGateForward, kKahan>;
    case kGradGateReverse: return grad_pass_kernel<L, PASS_REAL, kGradGateReverse, kKahan>;
  }
  throw std::runtime_error("unknown gradient mode");
}

GradKernel grad_kernel(int L, int mode) {
  switch (L) {
    case 0: return grad_kernel_mode<0>(mode);
    case 1: return grad_kernel_mode<1>(mode);
    case 2: return grad_kernel_mode<2>(mode);
    case 3: return grad_kernel_mode<3>(mode);
    case 4: return grad_kernel_mode<4>(mode);
    case 5: return grad_kernel_mode<5>(mode);
  }
  throw std::runtime_error("sh_l_max above 5 is not supported");
}
}  // namespace

template <>
GradLaunch grad_pass_config<PASS_REAL>(int L, int mode, const DevModel<PASS_REAL>& dm, int natoms, int sm_count) {
  if (dm.K > kMaxK) throw std::runtime_error("sh_k_max above " + std::to_string(kMaxK) + " is not supported");
  GradKernel kern = grad_kernel(L, mode);
  const int H = (L + 1) * (L + 1), Lp = L + 1;
  int device = 0, optin = 0;
  cudaGetDevice(&device);
  cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device);
  const size_t table = pass_table_size<PASS_REAL>(dm.C, dm.F, dm.B, dm.nblk);
  const size_t per_warp = grad_warp_size<PASS_REAL>(dm.F, H, dm.M, dm.K);
  // the gate forward pass has no per-edge parameter loop
  const int cols = mode == kGradGateForward
                       ? 0
                       : grad_acc_cols(Lp, dm.B, dm.C, dm.scaling_mode, mode == kGradOuter && dm.gated);
  GradLaunch cfg;
  cfg.warps = kGradWarps;
  cfg.acc_cols = cols;
  auto bytes = [&](int warps, int c) {
    return sizeof(PASS_REAL) * (table + warps * (per_warp + static_cast<size_t>(c) * kAccStride));
  };
  if (bytes(cfg.warps, cols) > static_cast<size_t>(optin)) cfg.warps = 1;
  if (bytes(cfg.warps, cols) > static_cast<size_t>(optin)) { cfg.warps = kGradWarps; cfg.acc_cols = 0; }
  cfg.block = cfg.warps * kWarp;
  cfg.smem = bytes(cfg.warps, cfg.acc_cols);
  cudaError_t err = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(cfg.smem));
  if (err != cudaSuccess) throw std::runtime_error(std::string("gradient shared memory: ") + cudaGetErrorString(err));
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, cfg.block, cfg.smem);
  if (per_sm < 1) throw std::runtime_error("gradient kernel does not fit on an SM (shared memory " + std::to_string(cfg.smem) + " B)");
  const int need = std::max(1, (natoms + cfg.warps - 1) / cfg.warps);
  cfg.grid = std::max(1, std::min(need, per_sm * sm_count));
  return cfg;
}

template <>
int launch_grad_pass<PASS_REAL>(int L, int mode, const GradArgs<PASS_REAL>& a, const GradLaunch& cfg, cudaStream_t s) {
  if (a.natoms == 0) return 0;
  GradKernel kern = grad_kernel(L, mode);
  GradArgs<PASS_REAL> args = a;
  args.acc_cols = cfg.acc_cols;
  kern<<<cfg.grid, cfg.block, cfg.smem, s>>>(args);
  cudaError_t err = cudaGetLastError();
  if (err != cudaSuccess) throw std::runtime_error(std::string("gradient launch: ") + cudaGetErrorString(err));
  return 1;
}

}  // namespace sus2g
