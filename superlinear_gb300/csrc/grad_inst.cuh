// Launch templates of the parameter-gradient passes for one spherical-harmonic order L; explicit
// instantiations in the grad_fp{32,64}_l*.cu units, run-time selection in pass_dispatch.cu.
#pragma once
#include <algorithm>
#include <stdexcept>
#include <string>

#include "pass_launch.h"

namespace sus2g {
namespace grad_detail {

constexpr int kGradMaxWarps = 4;  // warps per block considered by the launch configuration
template <typename Real>
using GradKernel = void (*)(GradArgs<Real>);

// cols: the per-edge parameter contributions go through lane-private shared-memory columns (true)
// or shuffle trees (false); each kernel contains one of the two forms only (a smaller kernel body
// keeps the per-edge loop within the instruction cache).  The gate forward pass has neither.
template <typename Real, int L, int BF, int MODE>
GradKernel<Real> kernel_for_mode(bool cols, int part) {
  constexpr bool kKahan = sizeof(Real) == 4;
  if constexpr (BF == 8) {
    if (part == kGradAtomPart) return grad_pass_kernel<L, Real, MODE, kKahan, BF, false, kGradAtomPart>;
    if (part == kGradEdgePart)
      return cols ? grad_pass_kernel<L, Real, MODE, kKahan, BF, true, kGradEdgePart>
                  : grad_pass_kernel<L, Real, MODE, kKahan, BF, false, kGradEdgePart>;
  }
  if (part != kGradWhole) throw std::runtime_error("split gradient passes are compiled for basis size 8 only");
  return cols ? grad_pass_kernel<L, Real, MODE, kKahan, BF, true, kGradWhole>
              : grad_pass_kernel<L, Real, MODE, kKahan, BF, false, kGradWhole>;
}

// part: GradPart; the split parts exist for basis size 8 (the other sizes run whole)
template <typename Real, int L, int BF>
GradKernel<Real> kernel_for(int mode, bool cols, int part) {
  constexpr bool kKahan = sizeof(Real) == 4;
  switch (mode) {
    case kGradOuter: return kernel_for_mode<Real, L, BF, kGradOuter>(cols, part);
    case kGradGateForward:
      if (part != kGradWhole) throw std::runtime_error("the gate forward gradient pass runs whole");
      return grad_pass_kernel<L, Real, kGradGateForward, kKahan, BF, false, kGradWhole>;
    case kGradGateReverse: return kernel_for_mode<Real, L, BF, kGradGateReverse>(cols, part);
  }
  throw std::runtime_error("unknown gradient mode");
}

template <typename Real, int L>
GradKernel<Real> kernel_for(int mode, int B, bool cols, int part) {
  return B == 8 ? kernel_for<Real, L, 8>(mode, cols, part) : kernel_for<Real, L, 0>(mode, cols, part);
}

}  // namespace grad_detail

template <typename Real, int L>
GradLaunch grad_pass_config_l(int mode, const DevModel<Real>& dm, int natoms, int sm_count, int part) {
  using namespace grad_detail;
  if (dm.K > kMaxK) throw std::runtime_error("sh_k_max above " + std::to_string(kMaxK) + " is not supported");
  constexpr int H = (L + 1) * (L + 1), Lp = L + 1;
  int device = 0, optin = 0;
  cudaGetDevice(&device);
  cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device);
  const size_t table = pass_table_size<Real>(dm.C, dm.F, dm.B, dm.nblk);
  const size_t per_warp = part == kGradEdgePart ? grad_edge_warp_size(dm.K, H)
                                                : grad_warp_size<Real>(dm.F, H, dm.M, dm.K, dm.prog_parts);
  // the gate forward pass and the per-atom part have no per-edge parameter loop
  const int cols = mode == kGradGateForward || part == kGradAtomPart
                       ? 0
                       : grad_acc_cols(Lp, dm.B, dm.C, dm.scaling_mode, mode == kGradOuter && dm.gated);
  GradLaunch cfg;
  cfg.part = part;
  cfg.acc_cols = cols;
  auto bytes = [&](int warps, int c) {
    return sizeof(Real) * (table + warps * (per_warp + static_cast<size_t>(c) * kAccStride));
  };
  if (bytes(1, cols) > static_cast<size_t>(optin)) cfg.acc_cols = 0;  // columns do not fit: shuffle trees
  GradKernel<Real> kern = kernel_for<Real, L>(mode, dm.B, cfg.acc_cols > 0, part);
  cudaError_t err = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
  if (err != cudaSuccess) throw std::runtime_error(std::string("gradient shared memory: ") + cudaGetErrorString(err));
  // warps per block: the most resident warps per SM (registers and shared memory), fewer warps
  // per block on ties (finer work distribution)
  int per_sm = 0, best_warps = 0;
  for (int w = 1; w <= kGradMaxWarps; ++w) {
    const size_t smem = bytes(w, cfg.acc_cols);
    if (smem > static_cast<size_t>(optin)) break;
    int blocks = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, kern, w * kWarp, smem);
    if (blocks * w > per_sm * best_warps) { per_sm = blocks; best_warps = w; }
  }
  if (best_warps == 0 || per_sm < 1)
    throw std::runtime_error("gradient kernel does not fit on an SM (shared memory " + std::to_string(bytes(1, cfg.acc_cols)) + " B)");
  cfg.warps = best_warps;
  cfg.block = cfg.warps * kWarp;
  cfg.smem = bytes(cfg.warps, cfg.acc_cols);
  const int need = std::max(1, (natoms + cfg.warps - 1) / cfg.warps);
  cfg.grid = std::max(1, std::min(need, per_sm * sm_count));
  return cfg;
}

template <typename Real, int L>
int launch_grad_pass_l(int mode, const GradArgs<Real>& a, const GradLaunch& cfg, cudaStream_t s) {
  if (a.natoms == 0) return 0;
  grad_detail::GradKernel<Real> kern = grad_detail::kernel_for<Real, L>(mode, a.dm.B, cfg.acc_cols > 0, cfg.part);
  GradArgs<Real> args = a;
  args.acc_cols = cfg.acc_cols;
  kern<<<cfg.grid, cfg.block, cfg.smem, s>>>(args);
  cudaError_t err = cudaGetLastError();
  if (err != cudaSuccess) throw std::runtime_error(std::string("gradient launch: ") + cudaGetErrorString(err));
  return 1;
}

template <typename Real, int L>
cudaError_t upload_grad_constants_l() { return sph_norm_upload(); }

}  // namespace sus2g

#define SUS2G_INSTANTIATE_GRAD(REAL, L)                                                                  \
  template GradLaunch grad_pass_config_l<REAL, L>(int, const DevModel<REAL>&, int, int, int);            \
  template int launch_grad_pass_l<REAL, L>(int, const GradArgs<REAL>&, const GradLaunch&, cudaStream_t); \
  template cudaError_t upload_grad_constants_l<REAL, L>();
