// Launch entry points of the per-atom passes, one translation unit per precision.
#pragma once
#include <cuda_runtime.h>

#include "efs_kernels.cuh"
#include "grad_kernels.cuh"

namespace sus2g {

struct GradLaunch {
  int grid = 0, block = 0, warps = 0;
  int acc_cols = 0;  // lane-private accumulator columns (0: shuffle-tree reductions)
  int part = 0;      // GradPart: the whole pass, or its per-atom or per-edge part
  size_t smem = 0;
};

// Launch shape of grad_pass_kernel<L, Real, mode> or of one part of it (GradPart; grid sized from
// occupancy x SM count).
template <typename Real>
GradLaunch grad_pass_config(int L, int mode, const DevModel<Real>& dm, int natoms, int sm_count, int part = 0);
// Launches it with that shape (a.slots must hold cfg.grid * cfg.warps slices).
template <typename Real>
int launch_grad_pass(int L, int mode, const GradArgs<Real>& a, const GradLaunch& cfg, cudaStream_t stream);

// Launches atom_pass_kernel<L, Real, mode, Kahan = (Real is float)> sized as a multiple of the SM
// count, with the register budget of `blocks` resident blocks per SM (3 or 4; 0 = the default),
// as a programmatic dependent launch when pdl is set (the kernel stages its model tables while
// the previous kernel of the stream drains).  Returns the number of kernels launched (1) or
// throws on a configuration error.
template <typename Real>
int launch_atom_pass(int L, int mode, const PassArgs<Real>& args, int sm_count, cudaStream_t stream,
                     int blocks = 0, bool pdl = false);

// The per-atom graph kernel of a split pass (atom_graph_kernel<Real, gm>: 0 energy pass, 1 gate
// forward, 2 gate reverse): returns 1 or throws.
template <typename Real>
int launch_atom_graph(const PassArgs<Real>& args, int sm_count, cudaStream_t stream, int gm = 0);

// Per-translation-unit constant-table upload (spherical-harmonic normalisation) of every unit.
template <typename Real>
cudaError_t upload_pass_constants();
template <typename Real>
cudaError_t upload_grad_constants();

// Per-L entry points, explicitly instantiated in the pass_fp*_l* / grad_fp*_l* units.
template <typename Real, int L>
int launch_atom_pass_l(int mode, const PassArgs<Real>& a, int sm_count, cudaStream_t s, int blocks, bool pdl);
template <typename Real, int L>
cudaError_t upload_pass_constants_l();
template <typename Real, int L>
GradLaunch grad_pass_config_l(int mode, const DevModel<Real>& dm, int natoms, int sm_count, int part);
template <typename Real, int L>
int launch_grad_pass_l(int mode, const GradArgs<Real>& a, const GradLaunch& cfg, cudaStream_t s);
template <typename Real, int L>
cudaError_t upload_grad_constants_l();

}  // namespace sus2g
