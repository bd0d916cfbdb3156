// Allocation-free Static E / F / virial entry point (sus2g_static_efs_noalloc).
//
// Who needs it: MD drivers whose device memory is owned by a pre-sized arena (Kokkos- or
// pool-managed host codes) and integrations that forbid driver allocations inside their time
// loop.  The regular entry points grow engine-owned buffers with cudaMalloc when a system gets
// larger; this one instead runs the Static FP32 per-atom pass with all of its scratch (sanitised
// copies of the caller's rows and neighbour indices, edge records, per-edge dE/dd, per-atom
// energies and virials, the incoming-edge lists of the force gather, an error flag) in one
// file-scope __device__ array of fixed size, so a call performs no allocation of any kind.  The
// call synchronises its stream once to report input errors.
//
// Limits: at most kNoAllocMaxEdges directed edges, kNoAllocMaxAtoms centre atoms and
// kNoAllocMaxAll atoms in all (centres plus ghosts) per call.  The array holds about 22 MiB, and
// every GPU that loads this library keeps it until the process exits.  Calls share the array, so
// calls that overlap on the GPU (different streams, or different host threads on one device)
// race and must be serialised by the caller.
//
// Input checks without out-of-range accesses: the first kernel validates the caller's CSR rows,
// neighbour indices and species and records any violation in the error flag, and it writes the
// copies that every later kernel reads with each row clamped to [0, nedges] and each neighbour
// index clamped to [0, nall).  A call with bad input therefore computes garbage inside the
// scratch and the caller's outputs, touches nothing else, and returns the error.
//
// Forces are gathered per atom in a fixed order (outgoing edges, then incoming edges sorted by
// edge index): no floating-point atomics, so results are bitwise reproducible between calls.
#include <cuda_runtime.h>

#include <algorithm>
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
constexpr int kNoAllocMaxAll = 65536;

// Scratch layout (byte offsets, each region 256-byte aligned).
constexpr size_t align256(size_t n) { return (n + 255) & ~size_t(255); }
constexpr size_t kOffFlag = 0;
constexpr size_t kOffD4 = kOffFlag + 256;
constexpr size_t kOffG = kOffD4 + align256(sizeof(EdgeF) * kNoAllocMaxEdges);
constexpr size_t kOffSite = kOffG + align256(sizeof(float) * 3 * kNoAllocMaxEdges);
constexpr size_t kOffVir = kOffSite + align256(sizeof(double) * kNoAllocMaxAtoms);
constexpr size_t kOffRow = kOffVir + align256(sizeof(double) * 6 * kNoAllocMaxAtoms);
constexpr size_t kOffNbr = kOffRow + align256(sizeof(int) * (kNoAllocMaxAtoms + 1));
constexpr size_t kOffInRow = kOffNbr + align256(sizeof(int) * kNoAllocMaxEdges);
constexpr size_t kOffCount = kOffInRow + align256(sizeof(int) * (kNoAllocMaxAll + 1));
constexpr size_t kOffInTmp = kOffCount + align256(sizeof(int) * (kNoAllocMaxAll + 1));
constexpr size_t kOffInEdge = kOffInTmp + align256(sizeof(int) * kNoAllocMaxEdges);
constexpr size_t kScratchBytes = kOffInEdge + align256(sizeof(int) * kNoAllocMaxEdges);

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

// Checks the caller's layout and writes the sanitised copies every later kernel reads:
//   t <= natoms:  row_s[t] = row[t] clamped to [0, nedges]; row[0] = 0, row[natoms] = nedges and
//                 row[t] <= row[t + 1] are checked (kErrEdgeCapacity otherwise);
//   t < nall:     types[t] in [0, C) (kErrBadSpecies);
//   t < nedges:   nbr_s[t] = nbr[t] clamped to [0, nall) (kErrEdgeCapacity when it was not), the
//                 edge record (dx, dy, dz, r) (kErrBadDistance for r = 0 or non-finite), and the
//                 incoming-edge count of the (clamped) neighbour.
__global__ void k_na_pack(int natoms, int nall, int species, const int* types, const int* row, const int* nbr,
                          const double* vec, long long nedges, int* row_s, int* nbr_s, EdgeF* d4, int* in_count,
                          int* error) {
  const long long t = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (t <= natoms) {
    const int i = static_cast<int>(t);
    const int r = row[i];
    bool bad = r < 0 || r > nedges;
    if (i == 0 && r != 0) bad = true;
    if (i == natoms && r != nedges) bad = true;
    if (i < natoms && r > row[i + 1]) bad = true;
    if (bad) record_error(error, kErrEdgeCapacity);
    row_s[i] = static_cast<int>(min(max(static_cast<long long>(r), 0LL), nedges));
  }
  if (t < nall && (types[t] < 0 || types[t] >= species)) record_error(error, kErrBadSpecies);
  if (t >= nedges) return;
  int j = nbr[t];
  if (j < 0 || j >= nall) {
    record_error(error, kErrEdgeCapacity);
    j = 0;
  }
  nbr_s[t] = j;
  atomicAdd(in_count + j, 1);
  const double x = vec[3 * t], y = vec[3 * t + 1], z = vec[3 * t + 2];
  const double r2 = x * x + y * y + z * z;
  if (!(r2 > 0) || !isfinite(r2)) record_error(error, kErrBadDistance);
  d4[t] = EdgeF{static_cast<float>(x), static_cast<float>(y), static_cast<float>(z), static_cast<float>(sqrt(r2))};
}

// Exclusive scan of the n = nall + 1 incoming-edge counts into in_row (one block of kScanThreads
// threads, each over a contiguous chunk); the counts are reset to zero to serve as fill cursors.
constexpr int kScanThreads = 1024;
__global__ void __launch_bounds__(kScanThreads) k_na_scan(int* count, int n, int* in_row) {
  __shared__ int part[kScanThreads];
  const int chunk = (n + kScanThreads - 1) / kScanThreads;
  const int b = threadIdx.x * chunk, e = min(n, b + chunk);
  int s = 0;
  for (int q = b; q < e; ++q) s += count[q];
  part[threadIdx.x] = s;
  __syncthreads();
  // Hillis-Steele inclusive scan of the chunk sums
  for (int o = 1; o < kScanThreads; o <<= 1) {
    const int v = threadIdx.x >= o ? part[threadIdx.x - o] : 0;
    __syncthreads();
    part[threadIdx.x] += v;
    __syncthreads();
  }
  int run = part[threadIdx.x] - s;
  for (int q = b; q < e; ++q) {
    const int c = count[q];
    in_row[q] = run;
    run += c;
    count[q] = 0;
  }
}

// in_tmp[in_row[j] + k] = the edges whose (clamped) neighbour is j, in arrival order.
__global__ void k_na_fill_in(const int* nbr_s, long long nedges, const int* in_row, int* cursor, int* in_tmp) {
  const long long e = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (e >= nedges) return;
  const int j = nbr_s[e];
  in_tmp[in_row[j] + atomicAdd(cursor + j, 1)] = static_cast<int>(e);
}

// Warp per atom: rank sort of the (distinct) edge indices of in(j) into in_edge.
__global__ void k_na_sort_in(const int* in_row, int nall, const int* in_tmp, int* in_edge) {
  const int j = static_cast<int>((static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x) / kWarp);
  const int lane = threadIdx.x & 31;
  if (j >= nall) return;
  const int b = in_row[j], n = in_row[j + 1] - b;
  for (int q = lane; q < n; q += kWarp) {
    const int x = in_tmp[b + q];
    int rank = 0;
    for (int u = 0; u < n; ++u) rank += in_tmp[b + u] < x;
    in_edge[b + rank] = x;
  }
}

// Warp per atom i < nall: F_i = sum over out(i) of g_e - sum over in(i) of g_e, both in a fixed
// order, compensated FP32 with an FP64 result; every force row is written.
__global__ void k_na_forces(int natoms, int nall, const int* row_s, const int* in_row, const int* in_edge,
                            const float* g, double* forces) {
  const int i = static_cast<int>((static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x) / kWarp);
  const int lane = threadIdx.x & 31;
  if (i >= nall) return;
  float hi[3] = {0.f, 0.f, 0.f}, lo[3] = {0.f, 0.f, 0.f};
  if (i < natoms)
    for (int e = row_s[i] + lane; e < row_s[i + 1]; e += kWarp)
      for (int c = 0; c < 3; ++c) csum_add(hi[c], lo[c], g[3 * static_cast<size_t>(e) + c]);
  for (int q = in_row[i] + lane; q < in_row[i + 1]; q += kWarp) {
    const int e = in_edge[q];
    for (int c = 0; c < 3; ++c) csum_add(hi[c], lo[c], -g[3 * static_cast<size_t>(e) + c]);
  }
  double f[3];
  for (int c = 0; c < 3; ++c) f[c] = warp_csum(hi[c], lo[c]);
  if (lane == 0)
    for (int c = 0; c < 3; ++c) forces[3 * static_cast<size_t>(i) + c] = f[c];
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

unsigned blocks_for(long long threads, int block) { return static_cast<unsigned>((threads + block - 1) / block); }

}  // namespace
}  // namespace sus2g

extern "C" int sus2g_static_efs_noalloc(sus2g_engine e, int natoms, int nall, const int* types, const int* row,
                                        const int* nbr, const double* vec, long long nedges, double* energy,
                                        double* forces, double* virial, double* site_energy) {
  using namespace sus2g;
  try {
    if (!e || natoms < 0 || nall < natoms || nedges < 0) throw Error(1, "invalid argument: engine/layout");
    if (natoms == 0 && nedges > 0) throw Error(1, "invalid argument: edges without centre atoms");
    if (natoms > kNoAllocMaxAtoms)
      throw Error(6, "allocation-free entry point: " + std::to_string(natoms) + " centre atoms exceed the maximum of " +
                         std::to_string(kNoAllocMaxAtoms));
    if (nall > kNoAllocMaxAll)
      throw Error(6, "allocation-free entry point: " + std::to_string(nall) + " atoms (centres and ghosts) exceed "
                         "the maximum of " + std::to_string(kNoAllocMaxAll));
    if (nedges > kNoAllocMaxEdges)
      throw Error(6, "allocation-free entry point: " + std::to_string(nedges) + " edges exceed the maximum of " +
                         std::to_string(kNoAllocMaxEdges));
    if ((natoms > 0 && !row) || (nall > 0 && !types) || (nedges > 0 && (!nbr || !vec)))
      throw Error(1, "invalid argument: null device array");
    Engine& eng = *e->engine;
    if (eng.precision() != kFP32 || eng.model().gated)
      throw Error(1, "allocation-free entry point needs a Static model on an FP32 engine");
    cudaError_t rc = cudaSetDevice(eng.device());
    if (rc != cudaSuccess) throw Error(10, std::string("cudaSetDevice: ") + cudaGetErrorString(rc));
    unsigned char* base = static_cast<unsigned char*>(scratch_on_current_device(eng.device()));
    int* err = reinterpret_cast<int*>(base + kOffFlag);
    EdgeF* d4 = reinterpret_cast<EdgeF*>(base + kOffD4);
    float* g = reinterpret_cast<float*>(base + kOffG);
    double* site = reinterpret_cast<double*>(base + kOffSite);
    double* vir = reinterpret_cast<double*>(base + kOffVir);
    int* row_s = reinterpret_cast<int*>(base + kOffRow);
    int* nbr_s = reinterpret_cast<int*>(base + kOffNbr);
    int* in_row = reinterpret_cast<int*>(base + kOffInRow);
    int* count = reinterpret_cast<int*>(base + kOffCount);
    int* in_tmp = reinterpret_cast<int*>(base + kOffInTmp);
    int* in_edge = reinterpret_cast<int*>(base + kOffInEdge);
    cudaStream_t s = eng.stream();
    // The array keeps the previous call's contents: the error flag and the incoming-edge counts
    // must start at zero; every other scratch value read below is written first by this call.
    rc = cudaMemsetAsync(err, 0, sizeof(int), s);
    if (rc == cudaSuccess) rc = cudaMemsetAsync(count, 0, sizeof(int) * (static_cast<size_t>(nall) + 1), s);
    if (rc != cudaSuccess) throw Error(10, std::string("cudaMemsetAsync: ") + cudaGetErrorString(rc));
    if (natoms == 0) {
      // no centres: zero energy and virial, and zero forces on the nall (ghost) atoms
      if (energy) rc = cudaMemsetAsync(energy, 0, sizeof(double), s);
      if (rc == cudaSuccess && virial) rc = cudaMemsetAsync(virial, 0, sizeof(double) * 6, s);
      if (rc == cudaSuccess && forces && nall)
        rc = cudaMemsetAsync(forces, 0, sizeof(double) * 3 * static_cast<size_t>(nall), s);
      if (rc == cudaSuccess) rc = cudaStreamSynchronize(s);
      if (rc != cudaSuccess) throw Error(10, std::string("cudaMemsetAsync: ") + cudaGetErrorString(rc));
      return 0;
    }
    const long long work = std::max<long long>(std::max<long long>(nedges, natoms + 1), nall);
    k_na_pack<<<blocks_for(work, 256), 256, 0, s>>>(natoms, nall, eng.model().C, types, row, nbr, vec, nedges, row_s,
                                                    nbr_s, d4, count, err);
    eng.static_pass_external(natoms, types, row_s, nbr_s, d4, g, site, vir, err);
    if (forces) {
      k_na_scan<<<1, kScanThreads, 0, s>>>(count, nall + 1, in_row);
      if (nedges > 0) {
        k_na_fill_in<<<blocks_for(nedges, 256), 256, 0, s>>>(nbr_s, nedges, in_row, count, in_tmp);
        k_na_sort_in<<<blocks_for(static_cast<long long>(nall) * kWarp, 256), 256, 0, s>>>(in_row, nall, in_tmp,
                                                                                         in_edge);
      }
      k_na_forces<<<blocks_for(static_cast<long long>(nall) * kWarp, 256), 256, 0, s>>>(natoms, nall, row_s, in_row,
                                                                                      in_edge, g, forces);
    }
    k_na_reduce<<<1, 256, 0, s>>>(natoms, site, vir, energy, virial, site_energy);
    rc = cudaGetLastError();
    if (rc != cudaSuccess) throw Error(10, std::string("kernel launch: ") + cudaGetErrorString(rc));
    int flag = 0;
    rc = cudaMemcpyAsync(&flag, err, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (rc == cudaSuccess) rc = cudaStreamSynchronize(s);
    if (rc != cudaSuccess) throw Error(10, std::string("stream synchronize: ") + cudaGetErrorString(rc));
    if (flag == kErrBadDistance) throw Error(24, "device check failed: zero or non-finite edge length");
    if (flag == kErrBadSpecies) throw Error(26, "device check failed: atom species index out of range");
    if (flag) throw Error(21, "device check failed: CSR rows or neighbour index out of range");
    return 0;
  } catch (const Error& x) {
    sus2g_set_last_error(x.what());
    return x.code > 0 ? x.code : 1;
  } catch (const std::exception& x) {
    sus2g_set_last_error(x.what());
    return 1;
  }
}
