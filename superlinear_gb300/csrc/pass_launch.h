// Launch entry points of the per-atom passes, one translation unit per precision.
#pragma once
#include <cuda_runtime.h>

#include "efs_kernels.cuh"

namespace sus2g {

// Launches atom_pass_kernel<L, Real, mode, Kahan = (Real is float)> sized as a multiple of the SM
// count.  Returns the number of kernels launched (1) or throws on a configuration error.
template <typename Real>
int launch_atom_pass(int L, int mode, const PassArgs<Real>& args, int sm_count, cudaStream_t stream);

// Per-translation-unit constant-table upload (spherical-harmonic normalisation).
template <typename Real>
cudaError_t upload_pass_constants();

}  // namespace sus2g
