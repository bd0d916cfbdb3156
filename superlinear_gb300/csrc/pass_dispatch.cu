// Run-time selection of the per-L pass and gradient units (instantiated in pass_fp*_l*.cu and
// grad_fp*_l*.cu); this unit sees only their declarations.
#include <algorithm>
#include <stdexcept>
#include <string>

#include "pass_launch.h"

namespace sus2g {

template <typename Real>
int launch_atom_pass(int L, int mode, const PassArgs<Real>& a, int sm_count, cudaStream_t s, int blocks, bool pdl) {
  if (a.dm.K > kMaxK) throw std::runtime_error("sh_k_max above " + std::to_string(kMaxK) + " is not supported");
  switch (L) {
    case 0: return launch_atom_pass_l<Real, 0>(mode, a, sm_count, s, blocks, pdl);
    case 1: return launch_atom_pass_l<Real, 1>(mode, a, sm_count, s, blocks, pdl);
    case 2: return launch_atom_pass_l<Real, 2>(mode, a, sm_count, s, blocks, pdl);
    case 3: return launch_atom_pass_l<Real, 3>(mode, a, sm_count, s, blocks, pdl);
    case 4: return launch_atom_pass_l<Real, 4>(mode, a, sm_count, s, blocks, pdl);
    case 5: return launch_atom_pass_l<Real, 5>(mode, a, sm_count, s, blocks, pdl);
  }
  throw std::runtime_error("sh_l_max above 5 is not supported");
}

template <typename Real>
GradLaunch grad_pass_config(int L, int mode, const DevModel<Real>& dm, int natoms, int sm_count, int part) {
  switch (L) {
    case 0: return grad_pass_config_l<Real, 0>(mode, dm, natoms, sm_count, part);
    case 1: return grad_pass_config_l<Real, 1>(mode, dm, natoms, sm_count, part);
    case 2: return grad_pass_config_l<Real, 2>(mode, dm, natoms, sm_count, part);
    case 3: return grad_pass_config_l<Real, 3>(mode, dm, natoms, sm_count, part);
    case 4: return grad_pass_config_l<Real, 4>(mode, dm, natoms, sm_count, part);
    case 5: return grad_pass_config_l<Real, 5>(mode, dm, natoms, sm_count, part);
  }
  throw std::runtime_error("sh_l_max above 5 is not supported");
}

template <typename Real>
int launch_grad_pass(int L, int mode, const GradArgs<Real>& a, const GradLaunch& cfg, cudaStream_t s) {
  switch (L) {
    case 0: return launch_grad_pass_l<Real, 0>(mode, a, cfg, s);
    case 1: return launch_grad_pass_l<Real, 1>(mode, a, cfg, s);
    case 2: return launch_grad_pass_l<Real, 2>(mode, a, cfg, s);
    case 3: return launch_grad_pass_l<Real, 3>(mode, a, cfg, s);
    case 4: return launch_grad_pass_l<Real, 4>(mode, a, cfg, s);
    case 5: return launch_grad_pass_l<Real, 5>(mode, a, cfg, s);
  }
  throw std::runtime_error("sh_l_max above 5 is not supported");
}

template <typename Real>
cudaError_t upload_pass_constants() {
  cudaError_t errs[6] = {upload_pass_constants_l<Real, 0>(), upload_pass_constants_l<Real, 1>(),
                         upload_pass_constants_l<Real, 2>(), upload_pass_constants_l<Real, 3>(),
                         upload_pass_constants_l<Real, 4>(), upload_pass_constants_l<Real, 5>()};
  for (cudaError_t e : errs)
    if (e != cudaSuccess) return e;
  return cudaSuccess;
}

template <typename Real>
cudaError_t upload_grad_constants() {
  cudaError_t errs[6] = {upload_grad_constants_l<Real, 0>(), upload_grad_constants_l<Real, 1>(),
                         upload_grad_constants_l<Real, 2>(), upload_grad_constants_l<Real, 3>(),
                         upload_grad_constants_l<Real, 4>(), upload_grad_constants_l<Real, 5>()};
  for (cudaError_t e : errs)
    if (e != cudaSuccess) return e;
  return cudaSuccess;
}

template <typename Real>
int launch_atom_graph(const PassArgs<Real>& a, int sm_count, cudaStream_t s, int gm) {
  if (a.natoms == 0) return 0;
  if (gm < 0 || gm > 2) throw std::runtime_error("graph kernel: unknown pass");
  auto kern = gm == 0 ? atom_graph_kernel<Real, 0> : gm == 1 ? atom_graph_kernel<Real, 1> : atom_graph_kernel<Real, 2>;
  const size_t smem =
      sizeof(Real) * kGraphWarps * static_cast<size_t>(graph_warp_size(a.dm.M, a.dm.prog_parts, a.dm.F, a.dm.Q));
  static size_t configured[3] = {0, 0, 0};
  if (smem > configured[gm]) {
    cudaError_t err = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
    if (err != cudaSuccess) throw std::runtime_error(std::string("graph kernel shared memory: ") + cudaGetErrorString(err));
    configured[gm] = smem;
  }
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kGraphWarps * kWarp, smem);
  if (per_sm < 1) throw std::runtime_error("graph kernel does not fit on an SM");
  const int need = (a.natoms + kGraphWarps - 1) / kGraphWarps;
  const int grid = std::max(1, std::min(need, per_sm * sm_count));
  kern<<<grid, kGraphWarps * kWarp, smem, s>>>(a);
  cudaError_t err = cudaGetLastError();
  if (err != cudaSuccess) throw std::runtime_error(std::string("graph kernel launch: ") + cudaGetErrorString(err));
  return 1;
}

template int launch_atom_graph<float>(const PassArgs<float>&, int, cudaStream_t, int);
template int launch_atom_graph<double>(const PassArgs<double>&, int, cudaStream_t, int);
template int launch_atom_pass<float>(int, int, const PassArgs<float>&, int, cudaStream_t, int, bool);
template int launch_atom_pass<double>(int, int, const PassArgs<double>&, int, cudaStream_t, int, bool);
template GradLaunch grad_pass_config<float>(int, int, const DevModel<float>&, int, int, int);
template GradLaunch grad_pass_config<double>(int, int, const DevModel<double>&, int, int, int);
template int launch_grad_pass<float>(int, int, const GradArgs<float>&, const GradLaunch&, cudaStream_t);
template int launch_grad_pass<double>(int, int, const GradArgs<double>&, const GradLaunch&, cudaStream_t);
template cudaError_t upload_pass_constants<float>();
template cudaError_t upload_pass_constants<double>();
template cudaError_t upload_grad_constants<float>();
template cudaError_t upload_grad_constants<double>();

}  // namespace sus2g
