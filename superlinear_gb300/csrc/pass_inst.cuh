// Launch templates of the per-atom passes for one spherical-harmonic order L.  The explicit
// instantiations live in the small pass_fp{32,64}_l*.cu units (one group of L each) so that the
// units compile in parallel; pass_dispatch.cu selects the unit by L at run time.  Each unit owns
// its copy of the spherical-harmonic normalisation table and uploads it through
// upload_pass_constants_l.
#pragma once
#include <algorithm>
#include <stdexcept>
#include <string>

#include "pass_launch.h"

namespace sus2g {
namespace pass_detail {

template <typename Real, int L, int MODE, int BF, int MINB>
int launch_one(const PassArgs<Real>& a, int sm_count, cudaStream_t stream, bool pdl) {
  constexpr bool kKahan = sizeof(Real) == 4;
  auto kern = atom_pass_kernel<L, Real, MODE, kKahan, BF, MINB>;
  const auto& dm = a.dm;
  const int H = (L + 1) * (L + 1);
  const bool h_bulk = MODE == kModeOuterBulk && h_rows_bulk_ok<Real>(dm.F);
  // warps per block: at most the compiled launch bound
  const int wpb = a.block_warps > 0 && a.block_warps < kPassWarps ? a.block_warps : kPassWarps;
  const size_t smem = sizeof(Real) * (efs_table_size(dm.C, dm.F, dm.B, dm.nblk) +
                                      wpb * pass_warp_stride<Real>(dm.F, H, dm.M, dm.K, dm.prog_parts, h_bulk));
  static size_t configured = 0;
  if (smem > configured) {
    cudaError_t err = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
    if (err != cudaSuccess) throw std::runtime_error(std::string("pass shared memory: ") + cudaGetErrorString(err));
    configured = smem;
  }
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, wpb * kWarp, smem);
  if (per_sm < 1) throw std::runtime_error("pass kernel does not fit on an SM (shared memory " + std::to_string(smem) + " B)");
  const int need = (a.natoms + wpb - 1) / wpb;
  const int resident = per_sm * sm_count;
  int grid = std::max(1, std::min(need, resident));
  if (a.grid_mode == 1) {
    // the same number of rounds over the resident warps with the fewest blocks: every warp then
    // takes the same number of centres (to one)
    const int rounds = (need + resident - 1) / resident;
    grid = std::max(1, (need + rounds - 1) / rounds);
  }
  if (a.natoms == 0) return 0;
  cudaError_t err = launch_kernel(pdl, kern, dim3(grid), dim3(wpb * kWarp), smem, stream, a);
  if (err != cudaSuccess) throw std::runtime_error(std::string("pass launch: ") + cudaGetErrorString(err));
  return 1;
}

template <typename Real, int L, int MODE>
constexpr int min_blocks() { return default_min_blocks(L, sizeof(Real) == 4, MODE); }

// B = 8: the register budget min_blocks (3 or 4 resident blocks per SM; 0 = the default);
// other basis sizes: the default only.
template <typename Real, int L, int MODE, int BF>
int launch_budget(int blocks, const PassArgs<Real>& a, int sm_count, cudaStream_t s, bool pdl) {
  if constexpr (BF == 8) {
    if (blocks == 3) return launch_one<Real, L, MODE, BF, 3>(a, sm_count, s, pdl);
    if (blocks == 4) return launch_one<Real, L, MODE, BF, 4>(a, sm_count, s, pdl);
  }
  return launch_one<Real, L, MODE, BF, min_blocks<Real, L, MODE>()>(a, sm_count, s, pdl);
}

template <typename Real, int L, int BF>
int launch_mode(int mode, int blocks, const PassArgs<Real>& a, int sm_count, cudaStream_t s, bool pdl) {
  switch (mode) {
    case kModeStatic: return launch_budget<Real, L, kModeStatic, BF>(blocks, a, sm_count, s, pdl);
    case kModeGateForward: return launch_budget<Real, L, kModeGateForward, BF>(blocks, a, sm_count, s, pdl);
    case kModeOuter:
      // the bulk-copy variant for basis size 8 where the gate-signal rows allow it
      if constexpr (BF == 8)
        if (pass_h_bulk<Real>(mode, a.h_bulk, a.dm.F)) return launch_budget<Real, L, kModeOuterBulk, BF>(blocks, a, sm_count, s, pdl);
      return launch_budget<Real, L, kModeOuter, BF>(blocks, a, sm_count, s, pdl);
    case kModeGateReverse: return launch_budget<Real, L, kModeGateReverse, BF>(blocks, a, sm_count, s, pdl);
    case kModeStaticFwd:
    case kModeStaticRev:
    case kModeOuterFwd:
    case kModeOuterRev:
    case kModeGateFwdEdges:
    case kModeGateRevEdges:
      if constexpr (sizeof(Real) == 4 && BF == 8) {
        switch (mode) {
          case kModeStaticFwd: return launch_budget<Real, L, kModeStaticFwd, BF>(blocks, a, sm_count, s, pdl);
          case kModeStaticRev: return launch_budget<Real, L, kModeStaticRev, BF>(blocks, a, sm_count, s, pdl);
          case kModeOuterFwd: return launch_budget<Real, L, kModeOuterFwd, BF>(blocks, a, sm_count, s, pdl);
          case kModeOuterRev: return launch_budget<Real, L, kModeOuterRev, BF>(blocks, a, sm_count, s, pdl);
          case kModeGateFwdEdges: return launch_budget<Real, L, kModeGateFwdEdges, BF>(blocks, a, sm_count, s, pdl);
          default: return launch_budget<Real, L, kModeGateRevEdges, BF>(blocks, a, sm_count, s, pdl);
        }
      } else {
        throw std::runtime_error("the split passes are compiled for FP32 engines with basis size 8 only");
      }
  }
  throw std::runtime_error("unknown pass mode");
}

}  // namespace pass_detail

// B = 8 (the basis size the reference's model initialisation writes) runs the variant with the
// basis size fixed at compile time; other sizes run the generic variant.
template <typename Real, int L>
int launch_atom_pass_l(int mode, const PassArgs<Real>& a, int sm_count, cudaStream_t s, int blocks, bool pdl) {
  if (a.dm.B == 8) return pass_detail::launch_mode<Real, L, 8>(mode, blocks, a, sm_count, s, pdl);
  return pass_detail::launch_mode<Real, L, 0>(mode, 0, a, sm_count, s, pdl);
}

template <typename Real, int L>
cudaError_t upload_pass_constants_l() { return sph_norm_upload(); }

}  // namespace sus2g

#define SUS2G_INSTANTIATE_PASS(REAL, L)                                                               \
  template int launch_atom_pass_l<REAL, L>(int, const PassArgs<REAL>&, int, cudaStream_t, int, bool); \
  template cudaError_t upload_pass_constants_l<REAL, L>();
