// Allocation-free Static E / F / virial entry point (sus2g_static_efs_noalloc).
//
// Who needs it: callers that must not allocate device memory while they run a step -- code that
// records its work into a CUDA stream capture, MD drivers whose device memory is owned by a
// pre-sized arena (Kokkos- or pool-managed host codes), or integrations that forbid driver
// allocations inside their time loop.  The regular entry points grow engine-owned buffers with
// cudaMalloc when a system gets larger; this one instead runs the Static FP32 per-atom pass with
// its scratch (edge records, per-edge dE/dd, per-atom energies and virials, an error flag) in one
// file-scope __device__ array of fixed size, so a call performs no allocation of any kind.
//
// Limits: at most kNoAllocMaxEdges directed edges and kNoAllocMaxAtoms centre atoms per call
// (the array holds 8 MiB of edge records, 6 MiB of dE/dd and 0.9 MiB of per-atom values, and every
// GPU that loads this library keeps it until the process exits).  Calls share the array, so
// calls that overlap on the GPU (different streams, or different host threads on one device)
// race and must be serialised by the caller.
#include <cuda_runtime.h>

#include <cmath>
#include <mutex>
#include <string>

#include "../../include/sus2g.h"
#include "capi_types.h"
#include "device_common.cuh"

namespace sus2g {
namespace {

constexpr long long kNoAllocMaxEdges = 524288;
constexpr int kNoAllocMaxAtoms = 16384;
constexpr size_t kFlagBytes = 256;
constexpr size_t kEdgeRecordBytes = sizeof(EdgeF) * kNoAllocMaxEdges;
constexpr size_t kGradBytes = sizeof(float) * 3 * kNoAllocMaxEdges;
constexpr size_t kSiteBytes = sizeof(double) * kNoAllocMaxAtoms;
constexpr size_t kVirBytes = sizeof(double) * 6 * kNoAllocMaxAtoms;
constexpr size_t kScratchBytes = kFlagBytes + kEdgeRecordBytes + kGradBytes + kSiteBytes + kVirBytes;

// The scratch.  Host code must not use this name as an address: its device address is obtained
// once per device with cudaGetSymbolAddress below.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

std::mutex g_setup_mutex;
void* g_scratch_addr[256] = {nullptr};

void* scratch_on_current_device(int device) {
  if (device < 0 || device >= 256) throw Error(1, "device index out of range");
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (!g_scratch_addr[device]) {
    void* p = nullptr;
    const cudaError_t rc = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (rc != cudaSuccess)
      throw Error(10, std::string("cudaGetSymbolAddress for the allocation-free scratch failed: ") + cudaGetErrorString(rc));
    g_scratch_addr[device] = p;
  }
  return g_scratch_addr[device];
}

// Validates the caller's CSR layout and types, and packs (dx, dy, dz, r) records.
__global__ void k_na_pack(int natoms, int nall, int species, const int* types, const int* row, const int* nbr,
                          const double* vec, long long nedges, EdgeF* d4, int* error) {
  const long long t = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (t < natoms + 1) {
    const int i = static_cast<int>(t);
    if (i == 0 && row[0] != 0) record_error(error, kErrEdgeCapacity);
    if (i == natoms && row[natoms] != nedges) record_error(error, kErrEdgeCapacity);
    if (i < natoms && (row[i] > row[i + 1] || types[i] < 0 || types[i] >= species)) record_error(error, kErrEdgeCapacity);
  }
  if (t < nall && (types[t] < 0 || types[t] >= species)) record_error(error, kErrEdgeCapacity);
  if (t >= nedges) return;
  const int j = nbr[t];
  if (j < 0 || j >= nall) { record_error(error, kErrEdgeCapacity); return; }
  const double x = vec[3 * t], y = vec[3 * t + 1], z = vec[3 * t + 2];
  const double r2 = x * x + y * y + z * z;
  if (!(r2 > 0) || !isfinite(r2)) record_error(error, kErrBadDistance);
  d4[t] = EdgeF{static_cast<float>(x), static_cast<float>(y), static_cast<float>(z), static_cast<float>(sqrt(r2))};
}

// F_i += sum over i's edges of g_e (warp reduction), F_j -= g_e; forces are zeroed beforehand.
__global__ void k_na_forces(int natoms, const int* row, const int* nbr, const float* g, double* forces) {
  const int i = static_cast<int>((static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x) / kWarp);
  const int lane = threadIdx.x & 31;
  if (i >= natoms) return;
  double f[3] = {0, 0, 0};
  for (int e = row[i] + lane; e < row[i + 1]; e += kWarp) {
    const int j = nbr[e];
    for (int c = 0; c < 3; ++c) {
      const double v = g[3 * static_cast<size_t>(e) + c];
      f[c] += v;
      atomicAdd(forces + 3 * static_cast<size_t>(j) + c, -v);
    }
  }
  for (int c = 0; c < 3; ++c) f[c] = warp_sum(f[c]);
  if (lane == 0)
    for (int c = 0; c < 3; ++c) atomicAdd(forces + 3 * static_cast<size_t>(i) + c, f[c]);
}

// Energy and virial: one block, fixed-order reduction into the caller's outputs.
__global__ void k_na_reduce(int natoms, const double* site, const double* vir, double* energy, double* virial,
                            double* site_out) {
  __shared__ double sh[7][256];
  double acc[7] = {0, 0, 0, 0, 0, 0, 0};
  for (int i = threadIdx.x; i < natoms; i += blockDim.x) {
    acc[0] += site[i];
    for (int c = 0; c < 6; ++c) acc[1 + c] += vir[6 * static_cast<size_t>(i) + c];
    if (site_out) site_out[i] = site[i];
  }
  for (int c = 0; c < 7; ++c) sh[c][threadIdx.x] = acc[c];
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s)
      for (int c = 0; c < 7; ++c) sh[c][threadIdx.x] += sh[c][threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    if (energy) *energy = sh[0][0];
    if (virial)
      for (int c = 0; c < 6; ++c) virial[c] = sh[1 + c][0];
  }
}

}  // namespace
}  // namespace sus2g

extern "C" int sus2g_static_efs_noalloc(sus2g_engine e, int natoms, int nall, const int* types, const int* row,
                                        const int* nbr, const double* vec, long long nedges, double* energy,
                                        double* forces, double* virial, double* site_energy) {
  using namespace sus2g;
  try {
    if (!e || natoms < 0 || nall < natoms || nedges < 0) throw Error(1, "invalid argument: engine/layout");
    if (natoms > kNoAllocMaxAtoms)
      throw Error(6, "allocation-free entry point: " + std::to_string(natoms) + " centre atoms exceed the maximum of " +
                         std::to_string(kNoAllocMaxAtoms));
    if (nedges > kNoAllocMaxEdges)
      throw Error(6, "allocation-free entry point: " + std::to_string(nedges) + " edges exceed the maximum of " +
                         std::to_string(kNoAllocMaxEdges));
    if ((natoms > 0 && (!types || !row)) || (nedges > 0 && (!nbr || !vec)))
      throw Error(1, "invalid argument: null device array");
    Engine& eng = *e->engine;
    if (eng.precision() != kFP32 || eng.model().gated)
      throw Error(1, "allocation-free entry point needs a Static model on an FP32 engine");
    cudaError_t rc = cudaSetDevice(eng.device());
    if (rc != cudaSuccess) throw Error(10, std::string("cudaSetDevice: ") + cudaGetErrorString(rc));
    unsigned char* base = static_cast<unsigned char*>(scratch_on_current_device(eng.device()));
    int* err = reinterpret_cast<int*>(base);
    EdgeF* d4 = reinterpret_cast<EdgeF*>(base + kFlagBytes);
    float* g = reinterpret_cast<float*>(base + kFlagBytes + kEdgeRecordBytes);
    double* site = reinterpret_cast<double*>(base + kFlagBytes + kEdgeRecordBytes + kGradBytes);
    double* vir = reinterpret_cast<double*>(base + kFlagBytes + kEdgeRecordBytes + kGradBytes + kSiteBytes);
    cudaStream_t s = eng.stream();
    // The array keeps the previous call's contents: the error flag must start at zero; every other
    // scratch value read below is written first by this call.
    rc = cudaMemsetAsync(err, 0, sizeof(int), s);
    if (rc == cudaSuccess && forces) rc = cudaMemsetAsync(forces, 0, sizeof(double) * 3 * static_cast<size_t>(nall), s);
    if (rc != cudaSuccess) throw Error(10, std::string("cudaMemsetAsync: ") + cudaGetErrorString(rc));
    const long long work = std::max<long long>(std::max<long long>(nedges, natoms + 1), nall);
    if (work > 0)
      k_na_pack<<<static_cast<unsigned>((work + 255) / 256), 256, 0, s>>>(natoms, nall, eng.model().C, types, row, nbr,
                                                                          vec, nedges, d4, err);
    eng.static_pass_external(natoms, types, row, nbr, d4, g, site, vir, err);
    if (forces && natoms)
      k_na_forces<<<static_cast<unsigned>((static_cast<long long>(natoms) * kWarp + 255) / 256), 256, 0, s>>>(
          natoms, row, nbr, g, forces);
    k_na_reduce<<<1, 256, 0, s>>>(natoms, site, vir, energy, virial, site_energy);
    rc = cudaGetLastError();
    if (rc != cudaSuccess) throw Error(10, std::string("kernel launch: ") + cudaGetErrorString(rc));
    int flag = 0;
    rc = cudaMemcpyAsync(&flag, err, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (rc == cudaSuccess) rc = cudaStreamSynchronize(s);
    if (rc != cudaSuccess) throw Error(10, std::string("stream synchronize: ") + cudaGetErrorString(rc));
    if (flag == kErrBadDistance) throw Error(24, "device check failed: zero or non-finite edge length");
    if (flag) throw Error(21, "device check failed: CSR rows, neighbour index or species index out of range");
    return 0;
  } catch (const Error& x) {
    sus2g_set_last_error(x.what());
    return x.code > 0 ? x.code : 1;
  } catch (const std::exception& x) {
    sus2g_set_last_error(x.what());
    return 1;
  }
}
