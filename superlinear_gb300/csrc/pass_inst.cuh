// Instantiation body for launch_atom_pass<Real>; included by pass_fp32.cu and pass_fp64.cu.
#include <stdexcept>
#include <string>

#include "pass_launch.h"

namespace sus2g {

namespace {
constexpr int kPassWarps = 4;

template <int L, int MODE>
int launch_one(const PassArgs<PASS_REAL>& a, int sm_count, cudaStream_t stream) {
  constexpr bool kKahan = sizeof(PASS_REAL) == 4;
  auto kern = atom_pass_kernel<L, PASS_REAL, MODE, kKahan>;
  const auto& dm = a.dm;
  const int H = (L + 1) * (L + 1);
  const size_t smem = sizeof(PASS_REAL) *
      (pass_table_size<PASS_REAL>(dm.C, dm.F, dm.B, dm.nblk) + kPassWarps * pass_warp_size<PASS_REAL>(dm.F, H, dm.M, dm.K));
  static size_t configured = 0;
  if (smem > configured) {
    cudaError_t err = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
    if (err != cudaSuccess) throw std::runtime_error(std::string("pass shared memory: ") + cudaGetErrorString(err));
    configured = smem;
  }
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kPassWarps * kWarp, smem);
  if (per_sm < 1) throw std::runtime_error("pass kernel does not fit on an SM (shared memory " + std::to_string(smem) + " B)");
  const int need = (a.natoms + kPassWarps - 1) / kPassWarps;
  const int grid = std::max(1, std::min(need, per_sm * sm_count));
  if (a.natoms == 0) return 0;
  kern<<<grid, kPassWarps * kWarp, smem, stream>>>(a);
  cudaError_t err = cudaGetLastError();
  if (err != cudaSuccess) throw std::runtime_error(std::string("pass launch: ") + cudaGetErrorString(err));
  return 1;
}

template <int L>
int launch_mode(int mode, const PassArgs<PASS_REAL>& a, int sm_count, cudaStream_t s) {
  switch (mode) {
    case kModeStatic: return launch_one<L, kModeStatic>(a, sm_count, s);
    case kModeGateForward: return launch_one<L, kModeGateForward>(a, sm_count, s);
    case kModeOuter: return launch_one<L, kModeOuter>(a, sm_count, s);
    case kModeGateReverse: return launch_one<L, kModeGateReverse>(a, sm_count, s);
  }
  throw std::runtime_error("unknown pass mode");
}
}  // namespace

template <>
int launch_atom_pass<PASS_REAL>(int L, int mode, const PassArgs<PASS_REAL>& a, int sm_count, cudaStream_t s) {
  if (a.dm.K > kMaxK) throw std::runtime_error("sh_k_max above " + std::to_string(kMaxK) + " is not supported");
  switch (L) {
    case 0: return launch_mode<0>(mode, a, sm_count, s);
    case 1: return launch_mode<1>(mode, a, sm_count, s);
    case 2: return launch_mode<2>(mode, a, sm_count, s);
    case 3: return launch_mode<3>(mode, a, sm_count, s);
    case 4: return launch_mode<4>(mode, a, sm_count, s);
    case 5: return launch_mode<5>(mode, a, sm_count, s);
  }
  throw std::runtime_error("sh_l_max above 5 is not supported");
}

template <>
cudaError_t upload_pass_constants<PASS_REAL>() { return sph_norm_upload(); }

}  // namespace sus2g
