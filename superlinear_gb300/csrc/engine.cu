// Host orchestration of the GPU engine: device tables, edge building, pass launches, force gather
// and per-frame reductions.
#include "engine.h"

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <map>
#include <cstring>
#include <numeric>
#include <stdexcept>
#include <string>

#include "neighbors.cuh"
#include "pass_launch.h"

namespace sus2g {

#define SUS2G_CUDA(call)                                                                      \
  do {                                                                                        \
    cudaError_t err__ = (call);                                                               \
    if (err__ != cudaSuccess)                                                                 \
      throw Error(10, std::string("CUDA error: ") + cudaGetErrorString(err__) + " at " #call); \
  } while (0)

void DevBuf::ensure(size_t n) {
  if (n <= bytes && ptr) return;
  release();
  const size_t want = std::max<size_t>(n, 256);
  SUS2G_CUDA(cudaMalloc(&ptr, want));
  bytes = want;
}
void DevBuf::release() {
  if (ptr) cudaFree(ptr);
  ptr = nullptr;
  bytes = 0;
}

// ------------------------------------------------------------------------------------------------
// edge building kernels
// ------------------------------------------------------------------------------------------------
namespace {

// Frame of every atom; with posh / posl (FP32 engines with image-scan frames) also its position
// as double-float parts x = xh + xl, xh = fl32(x), for the image scan's FP32 arithmetic.
__global__ void k_frame_of(const FramePlan* plans, int nframes, int* frame_of, const double* pos, float4* posh,
                           float4* posl) {
  const int f = blockIdx.x;
  if (f >= nframes) return;
  for (int i = plans[f].a0 + threadIdx.x; i < plans[f].a1; i += blockDim.x) {
    frame_of[i] = f;
    if (posh) {
      const double x = pos[3 * i], y = pos[3 * i + 1], z = pos[3 * i + 2];
      const float xh = static_cast<float>(x), yh = static_cast<float>(y), zh = static_cast<float>(z);
      posh[i] = make_float4(xh, yh, zh, 0.f);
      posl[i] = make_float4(static_cast<float>(x - xh), static_cast<float>(y - yh), static_cast<float>(z - zh), 0.f);
    }
  }
}

// Cell-list binning in one pass: per atom the wrapped fractions and integer cell offsets, its bin
// (bins of frame f are bin0 .. bin0 + nb0 nb1 nb2 - 1) and its record in the bin's fixed-capacity
// slots bin bcap .. bin bcap + bcap - 1 (order inside a bin is arbitrary: each centre's edges are
// sorted by (j, image) afterwards).  A bin that receives more than bcap atoms raises *bin_over to
// its count; the host then grows bcap and repeats the step.  With find_frame the atom's frame is
// found here (binary search over the frames' first atoms) and written to frame_of.
__global__ void k_bin_place(const FramePlan* plans, int nframes, bool find_frame, int* frame_of, const double* pos,
                            int natoms, int bcap, int* bin_of, int* rec_of, int* bin_count, AtomFrac* frac,
                            AtomOff* off, BinAtom* bin_rec, BinPos* bin_pos, BinPosF* bin_posf, int* bin_over,
                            int* error, const int* types, int C) {
  pdl_launch_dependents();  // the fill kernel's blocks may become resident while this grid runs
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= natoms) return;
  int f;
  if (find_frame) {
    // last frame whose first atom is <= i (an empty frame shares its first atom with the next one)
    int lo = 0, hi = nframes - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (plans[mid].a0 <= i) lo = mid; else hi = mid - 1;
    }
    f = lo;
    frame_of[i] = f;
  } else {
    f = frame_of[i];
  }
  const FramePlan& fp = plans[f];
  if (types[i] < 0 || types[i] >= C) record_error(error, kErrBadSpecies);
  if (!fp.use_bins) { bin_of[i] = -1; return; }
  const double x = pos[3 * i], y = pos[3 * i + 1], z = pos[3 * i + 2];
  // fractional coordinates, checked before any conversion to an integer: a non-finite coordinate,
  // or one more than 2^30 cells from the home cell, is reported and the atom binned inertly at
  // fraction 0 of bin 0 with non-finite wrapped positions (every distance test then rejects it)
  double sq[3];
  bool finite = true;
  for (int q = 0; q < 3; ++q) {
    sq[q] = x * fp.inv[q] + y * fp.inv[3 + q] + z * fp.inv[6 + q];
    finite = finite && fabs(sq[q]) < 1073741824.0;  // false for NaN and infinities too
  }
  if (!finite) record_error(error, kErrBadPosition);
  int b[3], o[3];
  float w32[3];
  for (int q = 0; q < 3; ++q) {
    const double fl = finite ? floor(sq[q]) : 0.0;
    const double w = finite ? sq[q] - fl : 0.0;
    o[q] = static_cast<int>(fl);
    w32[q] = static_cast<float>(w);
    b[q] = max(0, min(static_cast<int>(w * fp.nb[q]), fp.nb[q] - 1));
  }
  frac[i] = AtomFrac{w32[0], w32[1], w32[2], 0};
  off[i] = AtomOff{o[0], o[1], o[2], 0};
  const int bin = fp.bin0 + (b[0] * fp.nb[1] + b[1]) * fp.nb[2] + b[2];
  bin_of[i] = bin;
  const int slot = atomicAdd(bin_count + bin, 1);
  if (slot >= bcap) { atomicMax(bin_over, slot + 1); rec_of[i] = 0; return; }
  const long long rec = static_cast<long long>(bin) * bcap + slot;
  rec_of[i] = static_cast<int>(rec);
  bin_rec[rec] = BinAtom{w32[0], w32[1], w32[2], i, o[0], o[1], o[2], 0};
  const double* c = fp.cell;
  const double a0 = o[0], a1 = o[1], a2 = o[2];
  const double bad = finite ? 0.0 : nan("");
  const double wx = x - (a0 * c[0] + a1 * c[3] + a2 * c[6]) + bad;
  const double wy = y - (a0 * c[1] + a1 * c[4] + a2 * c[7]) + bad;
  const double wz = z - (a0 * c[2] + a1 * c[5] + a2 * c[8]) + bad;
  bin_pos[rec] = BinPos{wx, wy, wz, i, 0};
  const float hx = static_cast<float>(wx), hy = static_cast<float>(wy), hz = static_cast<float>(wz);
  bin_posf[rec] = BinPosF{hx, hy, hz, i, static_cast<float>(wx - hx), static_cast<float>(wy - hy),
                          static_cast<float>(wz - hz), 0};
}

// One cell-list edge record: components and distance already in the record's precision.
template <typename Real>
__device__ __forceinline__ void write_edge_rec(long long e, int j, int a, int b, int c, Real x, Real y, Real z, Real r,
                                               int* nbr, typename Vec4<Real>::type* d4, unsigned long long* key) {
  nbr[e] = j;
  typename Vec4<Real>::type v;
  v.x = x; v.y = y; v.z = z; v.w = r;
  d4[e] = v;
  key[e] = edge_key(j, a, b, c);
}

template <typename Real>
__device__ __forceinline__ void write_edge(long long e, int j, int a, int b, int c, double x, double y, double z, double r2,
                                           int* nbr, typename Vec4<Real>::type* d4, unsigned long long* key) {
  nbr[e] = j;
  typename Vec4<Real>::type v;
  v.x = Real(x); v.y = Real(y); v.z = Real(z);
  // FP32 records: the distance from the rounded r^2 (an FP32 square root; the FP64 one costs tens
  // of FP64-pipe instructions)
  if constexpr (sizeof(Real) == 4) v.w = sqrtf(static_cast<float>(r2));
  else v.w = sqrt(r2);
  d4[e] = v;
  key[e] = edge_key(j, a, b, c);
}

constexpr int kFillWarps = 8;
constexpr int kFillSortStage = 256;  // keys per warp kept in shared memory for the in-kernel sort
constexpr int kFillSortPer = 4;

// Sorts a centre's n staged edges (slots pad .. pad + n - 1) by key into the final arrays at the
// same slots: each key's rank among the centre's keys (unique within a centre), up to
// kFillSortPer keys per lane per pass with their payloads loaded while the ranks are counted;
// keys from shared memory when the centre has at most kFillSortStage of them.
template <typename Real>
__device__ __forceinline__ void sort_centre_edges(int lane, int n, long long pad, const unsigned long long* skeys,
                                                  const unsigned long long* key, const int* nbr,
                                                  const typename Vec4<Real>::type* d4, unsigned long long* key_out,
                                                  int* nbr_out, typename Vec4<Real>::type* d4_out) {
  const unsigned long long* src = n <= kFillSortStage ? skeys : key + pad;
  for (int q0 = 0; q0 < n; q0 += kFillSortPer * kWarp) {
    unsigned long long kk[kFillSortPer];
    int nb[kFillSortPer], rank[kFillSortPer];
    typename Vec4<Real>::type dd[kFillSortPer];
#pragma unroll
    for (int u = 0; u < kFillSortPer; ++u) {
      const int q = q0 + u * kWarp + lane;
      kk[u] = ~0ull;
      rank[u] = 0;
      if (q < n) {
        kk[u] = src[q];
        nb[u] = nbr[pad + q];
        dd[u] = d4[pad + q];
      }
    }
    for (int t = 0; t < n; ++t) {
      const unsigned long long kt = src[t];
#pragma unroll
      for (int u = 0; u < kFillSortPer; ++u) rank[u] += kt < kk[u];
    }
#pragma unroll
    for (int u = 0; u < kFillSortPer; ++u) {
      if (q0 + u * kWarp + lane < n) {
        key_out[pad + rank[u]] = kk[u];
        nbr_out[pad + rank[u]] = nb[u];
        d4_out[pad + rank[u]] = dd[u];
      }
    }
  }
}

// Cell-list frames: one warp per centre over its 125 stencil bins (warp_bin_edges), one pass.  The
// centre's edges go to its padded slots pad0 + (i - a0) cap .. + cap of the staging buffers; a
// count above cap is clamped to cap and raises *overflow to the full count, which the host reads
// with the step's error check (it then grows the capacity and repeats the step).  With row_end the
// kernel then sorts the centre's edges into the final arrays at the same slots.
template <typename Real>
__global__ void __launch_bounds__(kFillWarps * kWarp, 4)
k_edge_fill_bins(const FramePlan* plans, const int* frame_of, const double* pos, int natoms, double rc2,
                 const int* bin_count, int bin_cap, const BinAtom* bin_rec, const BinPos* bin_pos,
                 const BinPosF* bin_posf, const int* bin_of, const int* rec_of, const AtomFrac* frac, const AtomOff* off,
                 int* counts, int* nbr,
                 typename Vec4<Real>::type* d4, unsigned long long* key, int* overflow, int* error, int* row,
                 int* row_end, unsigned long long* key_out, int* nbr_out, typename Vec4<Real>::type* d4_out) {
  __shared__ int2 queue[kFillWarps][kEdgeQueue];
  __shared__ BinWalk walk[kFillWarps];
  __shared__ unsigned long long skeys[kFillWarps][kFillSortStage];
  pdl_wait();  // the bins and frame map of the previous kernel
  pdl_launch_dependents();
  const int i = static_cast<int>((static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x) / kWarp);
  if (i >= natoms) return;
  const FramePlan& fp = plans[frame_of[i]];
  if (!fp.use_bins) return;
  const int lane = threadIdx.x & 31, w = threadIdx.x / kWarp;
  const unsigned below = (1u << lane) - 1u;
  const long long pad = fp.pad0 + static_cast<long long>(i - fp.a0) * fp.cap;
  const int cap = fp.cap;
  int cursor = 0;
  warp_bin_edges<Real>(i, fp, pos, rc2, bin_count, bin_cap, bin_rec, bin_pos, bin_posf, bin_of, rec_of, frac, off, error,
                       queue[w], walk[w],
                       [&](unsigned mask, bool ok, int j, int a, int b, int c, Real x, Real y, Real z, Real r) {
                         if (ok) {
                           const int k = cursor + __popc(mask & below);
                           if (k < cap) {
                             write_edge_rec<Real>(pad + k, j, a, b, c, x, y, z, r, nbr, d4, key);
                             if (k < kFillSortStage) skeys[w][k] = edge_key(j, a, b, c);
                           }
                         }
                         cursor += __popc(mask);
                       });
  const int n = min(cursor, cap);
  if (lane == 0) {
    counts[i] = n;
    if (cursor > cap) atomicMax(overflow, cursor);
  }
  if (!row_end) return;
  __syncwarp();
  sort_centre_edges<Real>(lane, n, pad, skeys[w], key, nbr, d4, key_out, nbr_out, d4_out);
  if (lane == 0) {
    row[i] = static_cast<int>(pad);
    row_end[i] = static_cast<int>(pad) + n;
  }
}

// Periodic frames too small for cell lists (a perpendicular width below 3 r_c, or at most 512
// atoms): warp per centre i, lanes over the frame's atoms j.  For each j the image range per axis
// is ceil(-f - reach) .. floor(-f + reach), f = (x_j - x_i) . inv(cell), and every image n in it
// is tested exactly in FP64 (r^2 = |x_j + n.cell - x_i|^2 < r_c^2).  Accepted edges take the
// centre's next padded slot (a shared-memory counter) and are then sorted by (j, n) like the
// cell-list edges, so every periodic batch ends in the same padded layout without host
// synchronisation; a count above cap raises *overflow as in the cell-list kernel.
template <typename Real>
__global__ void __launch_bounds__(kFillWarps * kWarp)
k_edge_image_fill(const FramePlan* plans, const int* frame_of, const double* pos, const float4* posh,
                  const float4* posl, const int* types, int C, int natoms, double rc2, int* counts,
                  int* nbr, typename Vec4<Real>::type* d4, unsigned long long* key, int* overflow, int* error, int* row,
                  int* row_end, unsigned long long* key_out, int* nbr_out, typename Vec4<Real>::type* d4_out) {
  __shared__ unsigned long long skeys[kFillWarps][kFillSortStage];
  __shared__ int cursor[kFillWarps];
  pdl_wait();  // the frame map (and, in mixed batches, the cell-list fill) of the previous kernels
  pdl_launch_dependents();
  const int i = static_cast<int>((static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x) / kWarp);
  if (i >= natoms) return;
  const FramePlan& fp = plans[frame_of[i]];
  if (fp.use_bins) return;
  const int lane = threadIdx.x & 31, w = threadIdx.x / kWarp;
  const long long pad = fp.pad0 + static_cast<long long>(i - fp.a0) * fp.cap;
  const int cap = fp.cap;
  if (lane == 0) cursor[w] = 0;
  __syncwarp();
  const double xi = pos[3 * i], yi = pos[3 * i + 1], zi = pos[3 * i + 2];
  // a non-finite centre is reported and gets no edges; a non-finite neighbour is skipped (it
  // reports itself as a centre); image ranges are clamped to the packable [-64, 63] before any
  // conversion to an integer, and a range that reaches past it is reported
  const bool centre_ok = isfinite(xi) && isfinite(yi) && isfinite(zi);
  if (lane == 0 && !centre_ok) record_error(error, kErrBadPosition);
  if (lane == 0 && (types[i] < 0 || types[i] >= C)) record_error(error, kErrBadSpecies);
  const double* c = fp.cell;
  const double* inv = fp.inv;
  float4 cih = make_float4(0.f, 0.f, 0.f, 0.f), cil = cih;
  if (posh) { cih = posh[i]; cil = posl[i]; }
  for (int j = fp.a0 + lane; centre_ok && j < fp.a1; j += kWarp) {
    auto accept = [&](int a, int b, int cc, double vx, double vy, double vz, double r2) {
      const int k = atomicAdd(&cursor[w], 1);
      if (k < cap) {
        write_edge<Real>(pad + k, j, a, b, cc, vx, vy, vz, r2, nbr, d4, key);
        if (k < kFillSortStage) skeys[w][k] = edge_key(j, a, b, cc);
      }
    };
    int lo[3], hi[3];
    if constexpr (sizeof(Real) == 4) {
      // FP32 engines: double-float arithmetic on the (hi, lo) positions, FP64 only near the cutoff.
      //  * dx = x_j - x_i and every image vector v = dx + n . cell are accumulated as double-float
      //    pairs (exact two-sums, m cell_hi split exactly by an FMA): their absolute error is a few
      //    dozen 2^-48 of M, the largest magnitude involved, M = |dx| + sum_r |n_r| |cell_r|.  The
      //    vector is then rounded once to FP32 and r^2 formed in FP32: with M <= 1e6 r_c, r^2 near
      //    r_c^2 errs by well under 1e-6 r_c^2, so r^2 below lo2 = (1 - 1e-4) r_c^2 is inside and
      //    above hi2 = (1 + 1e-4) r_c^2 outside in FP64 too, and the band takes the exact FP64 test.
      //    The accepted set is the FP64 set; accepted vectors are the exact ones rounded once.
      //  * Ranges: f = dx_hi . inv(cell) in FP32 errs by at most ~7 2^-24 S, S = sum |dx_r inv_rq|;
      //    widening reach by 1e-4 + 1e-6 S keeps every image of the FP64 range (extra images are
      //    rejected by the distance test).
      //  Non-finite positions, ranges outside the packable [-64, 63] and larger M take the FP64 loop,
      //  which reports the first two.
      const float4 hj = posh[j], lj = posl[j];
      float xh = hj.x, xl = lj.x, yh = hj.y, yl = lj.y, zh = hj.z, zl = lj.z;
      df_acc(xh, xl, -cih.x, -cil.x);
      df_acc(yh, yl, -cih.y, -cil.y);
      df_acc(zh, zl, -cih.z, -cil.z);
      const float* ch = fp.cellf;
      const float* cl = fp.celll;
      bool fast = true;
      for (int q = 0; q < 3; ++q) {
        const float i0 = fp.invf[q], i1 = fp.invf[3 + q], i2 = fp.invf[6 + q];
        const float f = xh * i0 + yh * i1 + zh * i2;
        const float S = fabsf(xh * i0) + fabsf(yh * i1) + fabsf(zh * i2);
        const float reach = fp.reachf[q] + 1e-4f + 1e-6f * S;
        const float l = ceilf(-f - reach), h = floorf(-f + reach);
        if (!(l >= -64.0f && h <= 63.0f)) { fast = false; break; }
        lo[q] = static_cast<int>(l);
        hi[q] = static_cast<int>(h);
      }
      if (fast) {
        float m = fabsf(xh) + fabsf(yh) + fabsf(zh);
        for (int r = 0; r < 3; ++r)
          m += static_cast<float>(max(abs(lo[r]), abs(hi[r]))) *
               (fabsf(ch[3 * r]) + fabsf(ch[3 * r + 1]) + fabsf(ch[3 * r + 2]));
        fast = m * m <= 1e12f * fp.rc2f;
      }
      if (fast) {
        const float lo2 = fp.lo2, hi2 = fp.hi2;
        for (int a = lo[0]; a <= hi[0]; ++a) {
          float axh = xh, axl = xl, ayh = yh, ayl = yl, azh = zh, azl = zl;
          df_acc_mul(axh, axl, a, ch[0], cl[0]);
          df_acc_mul(ayh, ayl, a, ch[1], cl[1]);
          df_acc_mul(azh, azl, a, ch[2], cl[2]);
          for (int b = lo[1]; b <= hi[1]; ++b) {
            float pxh = axh, pxl = axl, pyh = ayh, pyl = ayl, pzh = azh, pzl = azl;
            df_acc_mul(pxh, pxl, b, ch[3], cl[3]);
            df_acc_mul(pyh, pyl, b, ch[4], cl[4]);
            df_acc_mul(pzh, pzl, b, ch[5], cl[5]);
            for (int cc = lo[2]; cc <= hi[2]; ++cc) {
              float vxh = pxh, vxl = pxl, vyh = pyh, vyl = pyl, vzh = pzh, vzl = pzl;
              df_acc_mul(vxh, vxl, cc, ch[6], cl[6]);
              df_acc_mul(vyh, vyl, cc, ch[7], cl[7]);
              df_acc_mul(vzh, vzl, cc, ch[8], cl[8]);
              const float vx = vxh + vxl, vy = vyh + vyl, vz = vzh + vzl;
              const float r2 = vx * vx + vy * vy + vz * vz;
              if (!(r2 < hi2) || (i == j && a == 0 && b == 0 && cc == 0)) continue;
              if (r2 < lo2) {
                accept(a, b, cc, vx, vy, vz, r2);
              } else {
                const double dx = pos[3 * j] - xi, dy = pos[3 * j + 1] - yi, dz = pos[3 * j + 2] - zi;
                const double ex = dx + a * c[0] + b * c[3] + cc * c[6];
                const double ey = dy + a * c[1] + b * c[4] + cc * c[7];
                const double ez = dz + a * c[2] + b * c[5] + cc * c[8];
                const double d2 = ex * ex + ey * ey + ez * ez;
                if (d2 < rc2) accept(a, b, cc, ex, ey, ez, d2);
              }
            }
          }
        }
        continue;
      }
    }
    // FP64: the exact test of every image (FP64 engines; FP32 engines' fallback)
    const double dx = pos[3 * j] - xi, dy = pos[3 * j + 1] - yi, dz = pos[3 * j + 2] - zi;
    if (!(isfinite(dx) && isfinite(dy) && isfinite(dz))) continue;
    for (int q = 0; q < 3; ++q) {
      const double f = dx * inv[q] + dy * inv[3 + q] + dz * inv[6 + q];
      double l = ceil(-f - fp.reach[q]), h = floor(-f + fp.reach[q]);
      if (l < -64.0 || h > 63.0) {
        record_error(error, kErrImageRange);
        l = fmax(l, -64.0);
        h = fmin(h, 63.0);
      }
      lo[q] = static_cast<int>(l);
      hi[q] = static_cast<int>(fmax(h, l - 1.0));
    }
    for (int a = lo[0]; a <= hi[0]; ++a)
      for (int b = lo[1]; b <= hi[1]; ++b)
        for (int cc = lo[2]; cc <= hi[2]; ++cc) {
          if (i == j && a == 0 && b == 0 && cc == 0) continue;
          const double vx = dx + a * c[0] + b * c[3] + cc * c[6];
          const double vy = dy + a * c[1] + b * c[4] + cc * c[7];
          const double vz = dz + a * c[2] + b * c[5] + cc * c[8];
          const double r2 = vx * vx + vy * vy + vz * vz;
          if (r2 < rc2) accept(a, b, cc, vx, vy, vz, r2);
        }
  }
  __syncwarp();
  const int total = cursor[w], n = min(total, cap);
  if (lane == 0) {
    counts[i] = n;
    if (total > cap) atomicMax(overflow, total);
  }
  sort_centre_edges<Real>(lane, n, pad, skeys[w], key, nbr, d4, key_out, nbr_out, d4_out);
  if (lane == 0) {
    row[i] = static_cast<int>(pad);
    row_end[i] = static_cast<int>(pad) + n;
  }
}

// Sort one centre's edges of a user edge list by key into CSR order (warp per centre, rank sort;
// keys within a centre are unique).  Keys of centres with at most `stage` edges are staged in
// shared memory (the rank loop then reads broadcast shared memory); longer lists rank from global
// memory.  Periodic batches are sorted inside their fill kernels.
constexpr int kSortWarps = 8;
template <typename Real>
__global__ void __launch_bounds__(kSortWarps * kWarp)
k_edge_sort(const int* row, int natoms, int stage, const unsigned long long* key_in, const int* nbr_in,
            const typename Vec4<Real>::type* d4_in, unsigned long long* key_out, int* nbr_out,
            typename Vec4<Real>::type* d4_out) {
  extern __shared__ unsigned long long sort_keys[];
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) / kWarp;
  const int lane = threadIdx.x & 31;
  if (warp >= natoms) return;
  const int e0 = row[warp], n = row[warp + 1] - e0;
  const long long in0 = e0;
  const unsigned long long* K = key_in;
  const int* NB = nbr_in;
  const typename Vec4<Real>::type* D = d4_in;
  const unsigned long long* src = K + in0;
  if (n <= stage) {
    unsigned long long* sk = sort_keys + (threadIdx.x / kWarp) * stage;
    for (int q = lane; q < n; q += kWarp) sk[q] = src[q];
    __syncwarp();
    src = sk;
  }
  // up to kSortPer keys per lane per pass: their payloads load while the ranks are counted
  constexpr int kSortPer = 4;
  for (int q0 = 0; q0 < n; q0 += kSortPer * kWarp) {
    unsigned long long k[kSortPer];
    int nb[kSortPer], rank[kSortPer];
    typename Vec4<Real>::type d[kSortPer];
#pragma unroll
    for (int u = 0; u < kSortPer; ++u) {
      const int q = q0 + u * kWarp + lane;
      k[u] = ~0ull;
      rank[u] = 0;
      if (q < n) {
        k[u] = src[q];
        nb[u] = NB[in0 + q];
        d[u] = D[in0 + q];
      }
    }
    for (int t = 0; t < n; ++t) {
      const unsigned long long kt = src[t];
#pragma unroll
      for (int u = 0; u < kSortPer; ++u) rank[u] += kt < k[u];
    }
#pragma unroll
    for (int u = 0; u < kSortPer; ++u) {
      if (q0 + u * kWarp + lane < n) {
        key_out[e0 + rank[u]] = k[u];
        nbr_out[e0 + rank[u]] = nb[u];
        d4_out[e0 + rank[u]] = d[u];
      }
    }
  }
}

// Reverse edge of every edge (warp per centre i): for e = (i -> j, n) the edge (j -> i, -n) is
// found by binary search in j's sorted keys.
// Up to kRevPer searches per lane run interleaved, so their dependent loads overlap.
// It also clears the first nzero bin counters (their last reader, the fill kernel, is done), so
// that the next step's binning starts from zero without a memset.
__global__ void k_reverse(const int* row, const int* row_end, const unsigned long long* key, int natoms, int* rev,
                          int* error, int* zero, int nzero) {
  constexpr int kRevPer = 4;
  const long long tid = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
  for (long long q = tid; q < nzero; q += static_cast<long long>(gridDim.x) * blockDim.x) zero[q] = 0;
  const int i = static_cast<int>(tid / kWarp);
  const int lane = threadIdx.x & 31;
  if (i >= natoms) return;
  const int end = row_end[i];
  for (int base = row[i]; base < end; base += kRevPer * kWarp) {
    int lo[kRevPer], hi[kRevPer], found[kRevPer];
    unsigned long long want[kRevPer];
#pragma unroll
    for (int u = 0; u < kRevPer; ++u) {
      const int e = base + u * kWarp + lane;
      lo[u] = 0; hi[u] = -1; found[u] = -1; want[u] = 0;
      if (e < end) {
        const unsigned long long k = key[e];
        const int j = static_cast<int>(k >> 21);
        const int n0 = static_cast<int>((k >> 14) & 127) - 64, n1 = static_cast<int>((k >> 7) & 127) - 64,
                  n2 = static_cast<int>(k & 127) - 64;
        want[u] = edge_key(i, -n0, -n1, -n2);
        lo[u] = row[j];
        hi[u] = row_end[j] - 1;
      }
    }
    bool active = true;
    while (active) {
      active = false;
#pragma unroll
      for (int u = 0; u < kRevPer; ++u) {
        if (lo[u] <= hi[u]) {
          const int mid = (lo[u] + hi[u]) >> 1;
          const unsigned long long km = key[mid];
          if (km == want[u]) { found[u] = mid; hi[u] = lo[u] - 1; }
          else if (km < want[u]) lo[u] = mid + 1;
          else hi[u] = mid - 1;
          active = active || lo[u] <= hi[u];
        }
      }
    }
#pragma unroll
    for (int u = 0; u < kRevPer; ++u) {
      const int e = base + u * kWarp + lane;
      if (e < end) {
        if (found[u] < 0) record_error(error, kErrReverseEdge);
        rev[e] = found[u] < 0 ? e : found[u];
      }
    }
  }
}

// F_i = sum over i's edges of (g_e - g_rev(e)), warp per atom: FP64 accumulation for FP64 edge
// gradients, compensated FP32 (two-sum, FP64 result) for FP32 ones.
template <typename Real>
__global__ void k_force_gather(const int* row, const int* row_end, const int* rev, const Real* g, int natoms,
                               double* force) {
  pdl_wait();  // the pass's dE/dd per edge
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) / kWarp;
  const int lane = threadIdx.x & 31;
  if (warp >= natoms) return;
  double f[3] = {0, 0, 0};
  float hi[3] = {0, 0, 0}, lo[3] = {0, 0, 0};
  for (int e = row[warp] + lane; e < row_end[warp]; e += kWarp) {
    const int r = rev[e];
    for (int c = 0; c < 3; ++c) {
      if (sizeof(Real) == 4) {
        csum_add(hi[c], lo[c], float(g[3 * (size_t)e + c]));
        csum_add(hi[c], lo[c], -float(g[3 * (size_t)r + c]));
      } else {
        f[c] += double(g[3 * (size_t)e + c]) - double(g[3 * (size_t)r + c]);
      }
    }
  }
  for (int c = 0; c < 3; ++c) f[c] = sizeof(Real) == 4 ? warp_csum(hi[c], lo[c]) : warp_sum(f[c]);
  if (lane == 0)
    for (int c = 0; c < 3; ++c) force[3 * (size_t)warp + c] = f[c];
}


// Caller edges: incoming lists.  in(j) = the edges whose neighbour is j, sorted by edge index, so
// that per-atom sums over them run in a fixed order (no floating-point atomics).
__global__ void k_count_in(const int* nbr, long long n, int* counts) {
  const long long e = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (e < n) atomicAdd(counts + nbr[e], 1);
}
__global__ void k_fill_in(const int* nbr, long long n, const int* in_row, int* cursor, int* in_tmp) {
  const long long e = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (e >= n) return;
  const int j = nbr[e];
  in_tmp[in_row[j] + atomicAdd(cursor + j, 1)] = static_cast<int>(e);
}
// warp per atom: rank sort of the (unique) edge indices of in(j)
__global__ void k_sort_in(const int* in_row, int nall, const int* in_tmp, int* in_edge) {
  const int j = (blockIdx.x * blockDim.x + threadIdx.x) / kWarp;
  const int lane = threadIdx.x & 31;
  if (j >= nall) return;
  const int b = in_row[j], n = in_row[j + 1] - b;
  for (int q = lane; q < n; q += kWarp) {
    const int x = in_tmp[b + q];
    int rank = 0;
    for (int t = 0; t < n; ++t) rank += in_tmp[b + t] < x;
    in_edge[b + rank] = x;
  }
}

// hbar[j][mu] = sum over in(j), in edge order, of the per-edge contributions hc[e][mu]
// (compensated FP32 for FP32 contributions, FP64 result).
template <typename Real>
__global__ void k_hbar_gather(const int* in_row, const int* in_edge, const Real* hc, int nall, int F, double* hbar) {
  const long long t = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (t >= static_cast<long long>(nall) * F) return;
  const int j = static_cast<int>(t / F), mu = static_cast<int>(t - static_cast<long long>(j) * F);
  double acc = 0.0;
  float hi = 0.f, lo = 0.f;
  for (int q = in_row[j]; q < in_row[j + 1]; ++q) {
    const Real v = hc[static_cast<size_t>(in_edge[q]) * F + mu];
    if (sizeof(Real) == 4) csum_add(hi, lo, float(v));
    else acc += double(v);
  }
  hbar[t] = sizeof(Real) == 4 ? double(hi) + double(lo) : acc;
}

// Caller edges: F_i = sum_{e in out(i)} g_e - sum_{e in in(i)} g_e for every atom (ghosts have
// no out-edges), warp per atom, fixed order.
template <typename Real>
__global__ void k_force_gather_user(const int* row, int nowned, const int* in_row, const int* in_edge, const Real* g,
                                    int nall, double* force) {
  const int i = (blockIdx.x * blockDim.x + threadIdx.x) / kWarp;
  const int lane = threadIdx.x & 31;
  if (i >= nall) return;
  double f[3] = {0, 0, 0};
  float hi[3] = {0, 0, 0}, lo[3] = {0, 0, 0};
  auto add = [&](int e, float sign) {
    for (int c = 0; c < 3; ++c) {
      if (sizeof(Real) == 4) csum_add(hi[c], lo[c], sign * float(g[3 * (size_t)e + c]));
      else f[c] += double(sign) * double(g[3 * (size_t)e + c]);
    }
  };
  if (i < nowned)
    for (int e = row[i] + lane; e < row[i + 1]; e += kWarp) add(e, 1.f);
  for (int q = in_row[i] + lane; q < in_row[i + 1]; q += kWarp) add(in_edge[q], -1.f);
  for (int c = 0; c < 3; ++c) f[c] = sizeof(Real) == 4 ? warp_csum(hi[c], lo[c]) : warp_sum(f[c]);
  if (lane == 0)
    for (int c = 0; c < 3; ++c) force[3 * (size_t)i + c] = f[c];
}

// Row pack / unpack of per-atom vectors for the caller's halo exchange: buf[k][w] = v[atom_k][w]
// (atoms[k], or first + k when atoms is null); mode 0 copies buf into v, mode 1 adds it.
template <typename T>
__global__ void k_rows_pack(const T* v, int width, int n, const int* atoms, int first, double* buf) {
  const long long t = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (t >= static_cast<long long>(n) * width) return;
  const int k = static_cast<int>(t / width), w = static_cast<int>(t - static_cast<long long>(k) * width);
  const int atom = atoms ? atoms[k] : first + k;
  buf[t] = double(v[static_cast<size_t>(atom) * width + w]);
}
template <typename T>
__global__ void k_rows_unpack(T* v, int width, int n, const int* atoms, int first, const double* buf, int add) {
  const long long t = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (t >= static_cast<long long>(n) * width) return;
  const int k = static_cast<int>(t / width), w = static_cast<int>(t - static_cast<long long>(k) * width);
  const int atom = atoms ? atoms[k] : first + k;
  T& dst = v[static_cast<size_t>(atom) * width + w];
  dst = add ? T(double(dst) + buf[t]) : T(buf[t]);
}

__global__ void k_iota(int* v, long long n) {
  const long long e = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (e < n) v[e] = static_cast<int>(e);
}

// Per-frame energy and virial (FP64), one launch: block (f, slice) sums the site energies and
// per-atom virials of its atoms (a fixed strided order per thread, then shuffle trees and the
// block's warps in order) into partial[f][slice][7] and copies the site energies out when asked;
// the block of frame f that arrives last (arrivals[f], reset by that block) adds the frame's
// slices in slice order.  The result does not depend on which block arrives last.
constexpr int kFrameThreads = 256;
__global__ void __launch_bounds__(kFrameThreads)
k_frame_reduce(const FramePlan* plans, int nframes, int S, const double* site, const double* vir_atom,
               double* site_out, double* partial, unsigned* arrivals, double* energy, double* virial) {
  const int f = blockIdx.x, sl = blockIdx.y;
  if (f >= nframes) return;
  double acc[7] = {0, 0, 0, 0, 0, 0, 0};
  for (int i = plans[f].a0 + sl * kFrameThreads + threadIdx.x; i < plans[f].a1; i += S * kFrameThreads) {
    const double e = site[i];
    acc[0] += e;
    if (site_out) site_out[i] = e;
    for (int c = 0; c < 6; ++c) acc[1 + c] += vir_atom[6 * (size_t)i + c];
  }
  __shared__ double sh[kFrameThreads / kWarp][7];
  __shared__ bool last;
  const int lane = threadIdx.x & 31, warp = threadIdx.x / kWarp;
#pragma unroll
  for (int c = 0; c < 7; ++c) {
    double v = acc[c];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane == 0) sh[warp][c] = v;
  }
  __syncthreads();
  if (threadIdx.x < 7) {
    double v = 0.0;
    for (int w = 0; w < kFrameThreads / kWarp; ++w) v += sh[w][threadIdx.x];
    partial[(static_cast<size_t>(f) * S + sl) * 7 + threadIdx.x] = v;
    __threadfence();
  }
  __syncthreads();
  if (threadIdx.x == 0) last = atomicAdd(arrivals + f, 1u) == static_cast<unsigned>(S - 1);
  __syncthreads();
  if (!last) return;
  __threadfence();
  // warp c < 7 sums component c over the S <= 64 slices: lane q holds slices q and q + 32, then a
  // fixed shuffle tree (all loads in flight at once)
  if (warp < 7) {
    const int c = warp;
    const double* pf = partial + static_cast<size_t>(f) * S * 7 + c;
    double v = lane < S ? __ldcg(pf + 7 * lane) : 0.0;
    if (lane + kWarp < S) v += __ldcg(pf + 7 * (lane + kWarp));
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane == 0) {
      if (c == 0) {
        if (energy) energy[f] = v;
      } else if (virial) {
        virial[6 * f + c - 1] = v;
      }
    }
  }
  if (threadIdx.x == 0) arrivals[f] = 0u;
}

// Caller-provided edges (owned centres, LAMMPS layout): count per centre.  An edge with a centre
// or neighbour index out of range is flagged and left out here and by the scatter below alike,
// so that no row keeps an unfilled slot.
__global__ void k_count_centres(const int* ei, const int* ej, long long n, int* counts, int nowned, int nall,
                                int* error) {
  const long long e = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (e >= n) return;
  const int i = ei[e], j = ej[e];
  if (i < 0 || i >= nowned || j < 0 || j >= nall) { record_error(error, kErrEdgeCapacity); return; }
  atomicAdd(counts + i, 1);
}

template <typename Real>
__global__ void k_scatter_user_edges(const int* ei, const int* ej, const double* d, long long n, const int* row,
                                     int* cursor, int* nbr, typename Vec4<Real>::type* d4, unsigned long long* key,
                                     int nowned, int nall, int* error) {
  const long long e = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (e >= n) return;
  const int i = ei[e], j = ej[e];
  if (i < 0 || i >= nowned || j < 0 || j >= nall) { record_error(error, kErrEdgeCapacity); return; }
  const double x = d[3 * e], y = d[3 * e + 1], z = d[3 * e + 2];
  const double r2 = x * x + y * y + z * z;
  if (!(r2 > 0) || !isfinite(r2)) record_error(error, kErrBadDistance);
  const int p = row[i] + atomicAdd(cursor + i, 1);
  nbr[p] = j;
  typename Vec4<Real>::type v;
  v.x = Real(x); v.y = Real(y); v.z = Real(z);
  // FP32 records: the distance from the rounded r^2 (an FP32 square root; the FP64 one costs tens
  // of FP64-pipe instructions)
  if constexpr (sizeof(Real) == 4) v.w = sqrtf(static_cast<float>(r2));
  else v.w = sqrt(r2);
  d4[p] = v;
  // Order key: neighbour, then the caller's edge index (unique, deterministic).
  key[p] = (static_cast<unsigned long long>(j) << 32) | static_cast<unsigned long long>(e & 0xffffffffLL);
}

// Exclusive scan of n counts into row[0..n] on the device (one block; each thread scans a
// contiguous chunk, then the chunk totals are scanned in shared memory).  Totals above 2^31 - 1
// are flagged.
__global__ void k_exclusive_scan(const int* counts, int n, int* row, int* error) {
  __shared__ long long part[1024];
  const int t = threadIdx.x, T = blockDim.x;
  const long long chunk = (static_cast<long long>(n) + T - 1) / T;
  const long long a = t * chunk, b = min(static_cast<long long>(n), a + chunk);
  long long s = 0;
  for (long long i = a; i < b; ++i) s += counts[i];
  part[t] = s;
  __syncthreads();
  for (int off = 1; off < T; off <<= 1) {
    const long long v = t >= off ? part[t - off] : 0;
    __syncthreads();
    part[t] += v;
    __syncthreads();
  }
  long long run = part[t] - s;
  for (long long i = a; i < b; ++i) {
    row[i] = static_cast<int>(run);
    run += counts[i];
  }
  if (t == T - 1) {
    if (part[t] > 2147483647LL) record_error(error, kErrEdgeCapacity);
    row[n] = static_cast<int>(min(part[t], 2147483647LL));
  }
}

void exclusive_scan_host_sync(const int* d_counts, int n, int* d_row, cudaStream_t s, long long* total) {
  std::vector<int> h(n);
  if (n) SUS2G_CUDA(cudaMemcpyAsync(h.data(), d_counts, sizeof(int) * n, cudaMemcpyDeviceToHost, s));
  SUS2G_CUDA(cudaStreamSynchronize(s));
  std::vector<int> r(n + 1);
  long long acc = 0;
  for (int i = 0; i < n; ++i) {
    r[i] = static_cast<int>(acc);
    acc += h[i];
    if (acc > 2000000000LL) throw Error(5, "edge count exceeds 2^31");
  }
  r[n] = static_cast<int>(acc);
  SUS2G_CUDA(cudaMemcpyAsync(d_row, r.data(), sizeof(int) * (n + 1), cudaMemcpyHostToDevice, s));
  SUS2G_CUDA(cudaStreamSynchronize(s));
  *total = acc;
}

void invert3(const double* c, double* inv) {
  // inverse of the row matrix c (rows = lattice vectors)
  const double det = c[0] * (c[4] * c[8] - c[5] * c[7]) - c[1] * (c[3] * c[8] - c[5] * c[6]) + c[2] * (c[3] * c[7] - c[4] * c[6]);
  if (!(std::fabs(det) > 0) || !std::isfinite(det)) throw Error(4, "invalid (singular) cell");
  const double id = 1.0 / det;
  inv[0] = (c[4] * c[8] - c[5] * c[7]) * id;
  inv[1] = (c[2] * c[7] - c[1] * c[8]) * id;
  inv[2] = (c[1] * c[5] - c[2] * c[4]) * id;
  inv[3] = (c[5] * c[6] - c[3] * c[8]) * id;
  inv[4] = (c[0] * c[8] - c[2] * c[6]) * id;
  inv[5] = (c[2] * c[3] - c[0] * c[5]) * id;
  inv[6] = (c[3] * c[7] - c[4] * c[6]) * id;
  inv[7] = (c[1] * c[6] - c[0] * c[7]) * id;
  inv[8] = (c[0] * c[4] - c[1] * c[3]) * id;
}

}  // namespace

// ------------------------------------------------------------------------------------------------
// model tables
// ------------------------------------------------------------------------------------------------
// A pass's graph program on the host (GraphProg, device_common.cuh).  Its structure depends on the
// model topology only and is built once per engine; each upload fills the coefficients: a fixed
// product coefficient, or the current rank weight w[widx] of a contraction row.
struct HostProg {
  std::vector<std::array<int, 4>> steps, comb;
  struct Rec { unsigned ab; int flush; int widx; double cfix; };
  std::vector<Rec> rows;  // [row][kWarp]
  int nfwd = 0, max_parts = 0;
  bool gate = false;
};

namespace {

struct Packer {
  std::vector<int> ints;
  std::vector<double> reals;
  int add_int(const std::vector<int>& v) { int o = static_cast<int>(ints.size()); ints.insert(ints.end(), v.begin(), v.end()); return o; }
  int add_real(const std::vector<double>& v) { int o = static_cast<int>(reals.size()); reals.insert(reals.end(), v.begin(), v.end()); return o; }
};

struct PassOffsets {
  int coeff, scal, wc, ws, wa;
  int ndst, dst_node, dst_begin, dst_src, dst_w, src_begin, src_dst, src_w;
  int levels, level_begin, out_nodes, out_begin, fa, fb, fc, rlevel_begin, in_nodes, in_begin, rout, rother, rc;
};

PassOffsets pack_pass(const Model& m, bool gate, Packer& pk) {
  PassOffsets o{};
  const int C = m.C, F = m.F, B = m.B;
  std::vector<double> coeff(static_cast<size_t>(F) * B);
  const bool own_radial = gate && m.gate_shared_radial;
  for (int mu = 0; mu < F; ++mu)
    for (int b = 0; b < B; ++b)
      coeff[static_cast<size_t>(mu) * B + b] = own_radial ? m.gate_radial[static_cast<size_t>(mu) * B + b]
                                                          : m.radial[static_cast<size_t>(mu) * (B + C) + b];
  o.coeff = pk.add_real(coeff);
  o.scal = pk.add_real(gate && m.gate_decoupled ? m.gate_scal : m.scal);
  std::vector<double> wc(static_cast<size_t>(C) * F), wa(static_cast<size_t>(C) * F, 0.0);
  for (int t = 0; t < C; ++t)
    for (int mu = 0; mu < F; ++mu) {
      const size_t idx = static_cast<size_t>(t) * F + mu;
      wc[idx] = gate ? m.gate_type[idx] : m.radial[static_cast<size_t>(mu) * (B + C) + B + t];
      if (!gate && m.gated) wa[idx] = m.gate_add[idx];
    }
  o.wc = pk.add_real(wc);
  o.ws = o.wc;
  o.wa = pk.add_real(wa);
  // contraction
  const auto& rows = gate ? m.gate_rows : m.outer_rows;
  const auto& w = gate ? m.gate_w : m.outer_w;
  std::vector<int> dsts;
  for (const auto& r : rows) dsts.push_back(r.dst);
  std::sort(dsts.begin(), dsts.end());
  dsts.erase(std::unique(dsts.begin(), dsts.end()), dsts.end());
  std::vector<int> dst_begin{0}, dst_src, src_begin{0}, src_dst;
  std::vector<double> dst_w, src_w;
  for (int d : dsts) {
    for (const auto& r : rows)
      if (r.dst == d) { dst_src.push_back(r.src); dst_w.push_back(r.widx < 0 ? 1.0 : w[r.widx]); }
    dst_begin.push_back(static_cast<int>(dst_src.size()));
  }
  for (int b = 0; b < m.NB; ++b) {
    for (const auto& r : rows)
      if (r.src == b) { src_dst.push_back(r.dst); src_w.push_back(r.widx < 0 ? 1.0 : w[r.widx]); }
    src_begin.push_back(static_cast<int>(src_dst.size()));
  }
  o.ndst = static_cast<int>(dsts.size());
  o.dst_node = pk.add_int(dsts);
  o.dst_begin = pk.add_int(dst_begin);
  o.dst_src = pk.add_int(dst_src);
  o.dst_w = pk.add_real(dst_w);
  o.src_begin = pk.add_int(src_begin);
  o.src_dst = pk.add_int(src_dst);
  o.src_w = pk.add_real(src_w);
  // graph
  const GraphSchedule& g = gate ? m.gate_graph : m.outer_graph;
  o.levels = g.levels;
  o.level_begin = pk.add_int(g.level_begin);
  o.out_nodes = pk.add_int(g.out_nodes);
  o.out_begin = pk.add_int(g.out_begin);
  std::vector<int> fa, fb;
  std::vector<double> fc;
  for (int p : g.fprod) { fa.push_back(m.products[p].a); fb.push_back(m.products[p].b); fc.push_back(m.products[p].c); }
  o.fa = pk.add_int(fa);
  o.fb = pk.add_int(fb);
  o.fc = pk.add_real(fc);
  o.rlevel_begin = pk.add_int(g.rlevel_begin);
  o.in_nodes = pk.add_int(g.in_nodes);
  o.in_begin = pk.add_int(g.in_begin);
  o.rout = pk.add_int(g.rprod_out);
  o.rother = pk.add_int(g.rprod_other);
  o.rc = pk.add_real(g.rprod_c);
  return o;
}

// ---- per-atom graph program (see GraphProg in device_common.cuh) ----
struct ProgGroup {
  int target;
  std::vector<std::array<int, 2>> ab;
  std::vector<double> c;   // fixed coefficient (when widx < 0)
  std::vector<int> widx;   // rank-weight index, or -1
};

// One step: the groups' term lists cut into chunks of about total / 32 terms (at least 4), dealt
// longest first to the least-loaded lane; lists of several chunks sum through partial slots.
// Each lane's chunks become one term stream, stored lane-major and padded with zero terms.
void add_prog_step(HostProg& hp, const std::vector<ProgGroup>& groups, bool reverse, int one) {
  long long total = 0;
  for (const auto& g : groups) total += static_cast<long long>(g.ab.size());
  if (total == 0) return;
  const int T = std::max(4, static_cast<int>((total + kWarp - 1) / kWarp));
  struct Ch { int g, tb, te, flush; };
  std::vector<Ch> chs;
  const int comb_begin = static_cast<int>(hp.comb.size());
  int parts = 0;
  for (size_t gi = 0; gi < groups.size(); ++gi) {
    const int n = static_cast<int>(groups[gi].ab.size());
    if (!n) continue;
    if (n <= T) {
      chs.push_back({static_cast<int>(gi), 0, n, groups[gi].target});
      continue;
    }
    const int k = (n + T - 1) / T, slot0 = parts;
    for (int j = 0; j < k; ++j) chs.push_back({static_cast<int>(gi), j * n / k, (j + 1) * n / k, -(parts++ + 2)});
    hp.comb.push_back({groups[gi].target, slot0, parts, 0});
  }
  std::vector<int> order(chs.size());
  for (size_t i = 0; i < chs.size(); ++i) order[i] = static_cast<int>(i);
  std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return chs[x].te - chs[x].tb > chs[y].te - chs[y].tb; });
  std::vector<int> lane_of(chs.size());
  long long load[kWarp] = {0};
  for (int i : order) {
    int best = 0;
    for (int l = 1; l < kWarp; ++l)
      if (load[l] < load[best]) best = l;
    lane_of[i] = best;
    load[best] += chs[i].te - chs[i].tb;
  }
  // Rows are filled one at a time: each lane takes a term of its current chunk (a chunk's terms
  // may be summed in any order), choosing the one whose two node reads share a shared-memory
  // bank (node index mod 32; equal nodes broadcast) with the fewest other lanes' reads of this
  // row, so that the warp's two loads per row are mostly conflict-free.
  std::vector<std::vector<int>> lane_chunks(kWarp);
  for (size_t i = 0; i < chs.size(); ++i) lane_chunks[lane_of[i]].push_back(static_cast<int>(i));
  std::vector<size_t> next_chunk(kWarp, 0);
  std::vector<std::vector<int>> pool(kWarp);  // remaining term indices of the lane's current chunk
  std::vector<int> cur(kWarp, -1);
  auto refill = [&](int l) {
    if (next_chunk[l] < lane_chunks[l].size()) {
      cur[l] = lane_chunks[l][next_chunk[l]++];
      for (int q = chs[cur[l]].tb; q < chs[cur[l]].te; ++q) pool[l].push_back(q);
    }
  };
  for (int l = 0; l < kWarp; ++l) refill(l);
  const int first = static_cast<int>(hp.rows.size() / kWarp);
  const HostProg::Rec pad{static_cast<unsigned>(one) | (static_cast<unsigned>(one) << 16), kProgNoFlush, -1, 0.0};
  auto seen = [](const std::vector<int>& nodes, int n) { return std::find(nodes.begin(), nodes.end(), n) != nodes.end(); };
  int len = 0;
  for (;;) {
    bool any = false;
    for (int l = 0; l < kWarp; ++l) any = any || !pool[l].empty();
    if (!any) break;
    std::vector<std::vector<int>> bank_a(kWarp), bank_b(kWarp);  // distinct nodes read per bank
    for (int l = 0; l < kWarp; ++l) {
      if (pool[l].empty()) { hp.rows.push_back(pad); continue; }
      const ProgGroup& g = groups[chs[cur[l]].g];
      size_t best = 0;
      int best_cost = 1 << 30;
      for (size_t k = 0; k < pool[l].size(); ++k) {
        const int a = g.ab[pool[l][k]][0], b = g.ab[pool[l][k]][1];
        const int c = (seen(bank_a[a % kWarp], a) ? 0 : static_cast<int>(bank_a[a % kWarp].size())) +
                      (seen(bank_b[b % kWarp], b) ? 0 : static_cast<int>(bank_b[b % kWarp].size()));
        if (c < best_cost) { best_cost = c; best = k; }
      }
      const int q = pool[l][best];
      pool[l].erase(pool[l].begin() + static_cast<long>(best));
      const int a = g.ab[q][0], b = g.ab[q][1];
      if (!seen(bank_a[a % kWarp], a)) bank_a[a % kWarp].push_back(a);
      if (!seen(bank_b[b % kWarp], b)) bank_b[b % kWarp].push_back(b);
      const bool last = pool[l].empty();
      hp.rows.push_back({static_cast<unsigned>(a) | (static_cast<unsigned>(b) << 16), last ? chs[cur[l]].flush : kProgNoFlush,
                         g.widx[q], g.c[q]});
      if (last) refill(l);
    }
    ++len;
  }
  hp.steps.push_back({first, len, comb_begin, (static_cast<int>(hp.comb.size()) << 1) | (reverse ? 1 : 0)});
  hp.max_parts = std::max(hp.max_parts, parts);
}

// The pass's rank contraction and product graph as a program: forward (contraction, graph levels
// 1..L), then reverse (graph levels L-1..0, contraction); node M is the constant 1.
HostProg build_prog(const Model& m, bool gate) {
  if (m.M + 1 > 65535) throw Error(3, "SUS2 model: too many moment nodes for the per-atom program");
  HostProg hp;
  hp.gate = gate;
  const int one = m.M;
  const auto& rows = gate ? m.gate_rows : m.outer_rows;
  const GraphSchedule& g = gate ? m.gate_graph : m.outer_graph;
  std::vector<int> dsts;
  for (const auto& r : rows) dsts.push_back(r.dst);
  std::sort(dsts.begin(), dsts.end());
  dsts.erase(std::unique(dsts.begin(), dsts.end()), dsts.end());
  {
    std::vector<ProgGroup> gs;
    for (int d : dsts) {
      ProgGroup pg{d, {}, {}, {}};
      for (const auto& r : rows)
        if (r.dst == d) { pg.ab.push_back({r.src, one}); pg.c.push_back(1.0); pg.widx.push_back(r.widx); }
      gs.push_back(std::move(pg));
    }
    add_prog_step(hp, gs, false, one);
  }
  for (int lv = 0; lv < g.levels; ++lv) {
    std::vector<ProgGroup> gs;
    for (int q = g.level_begin[lv]; q < g.level_begin[lv + 1]; ++q) {
      ProgGroup pg{g.out_nodes[q], {}, {}, {}};
      for (int p = g.out_begin[q]; p < g.out_begin[q + 1]; ++p) {
        const Product& pr = m.products[g.fprod[p]];
        pg.ab.push_back({pr.a, pr.b});
        pg.c.push_back(pr.c);
        pg.widx.push_back(-1);
      }
      gs.push_back(std::move(pg));
    }
    add_prog_step(hp, gs, false, one);
  }
  hp.nfwd = static_cast<int>(hp.steps.size());
  for (int lv = static_cast<int>(g.rlevel_begin.size()) - 2; lv >= 0; --lv) {
    std::vector<ProgGroup> gs;
    for (int q = g.rlevel_begin[lv]; q < g.rlevel_begin[lv + 1]; ++q) {
      ProgGroup pg{g.in_nodes[q], {}, {}, {}};
      for (int e = g.in_begin[q]; e < g.in_begin[q + 1]; ++e) {
        pg.ab.push_back({g.rprod_out[e], g.rprod_other[e]});
        pg.c.push_back(g.rprod_c[e]);
        pg.widx.push_back(-1);
      }
      gs.push_back(std::move(pg));
    }
    add_prog_step(hp, gs, true, one);
  }
  {
    std::vector<ProgGroup> gs;
    for (int b = 0; b < m.NB; ++b) {
      ProgGroup pg{b, {}, {}, {}};
      for (const auto& r : rows)
        if (r.src == b) { pg.ab.push_back({r.dst, one}); pg.c.push_back(1.0); pg.widx.push_back(r.widx); }
      gs.push_back(std::move(pg));
    }
    add_prog_step(hp, gs, true, one);
  }
  return hp;
}

// Serialises the programs of the passes into one 16-byte aligned device image and binds them.
template <typename Real>
void upload_progs(const Model& m, const std::vector<const HostProg*>& progs, DevBuf& buf, cudaStream_t s,
                  std::vector<GraphProg<Real>>& out) {
  std::vector<unsigned char> img;
  auto put = [&](const void* p, size_t n) {
    const size_t o = (img.size() + 15) & ~size_t(15);
    img.resize(o + n);
    if (n) std::memcpy(img.data() + o, p, n);
    return o;
  };
  struct Off { size_t steps, comb, rows; };
  std::vector<Off> offs;
  for (const HostProg* hp : progs) {
    Off o{};
    o.steps = put(hp->steps.data(), sizeof(int4) * hp->steps.size());
    o.comb = put(hp->comb.data(), sizeof(int4) * hp->comb.size());
    const std::vector<double>& w = hp->gate ? m.gate_w : m.outer_w;
    std::vector<ProgRec<Real>> rows(hp->rows.size());
    for (size_t q = 0; q < rows.size(); ++q) {
      const HostProg::Rec& x = hp->rows[q];
      rows[q] = ProgRec<Real>{};
      rows[q].ab = x.ab;
      rows[q].flush = x.flush;
      rows[q].c = static_cast<Real>(x.widx >= 0 ? w[x.widx] : x.cfix);
    }
    o.rows = put(rows.data(), sizeof(ProgRec<Real>) * rows.size());
    offs.push_back(o);
  }
  if (img.empty()) img.resize(16);
  buf.ensure(img.size());
  SUS2G_CUDA(cudaMemcpyAsync(buf.ptr, img.data(), img.size(), cudaMemcpyHostToDevice, s));
  SUS2G_CUDA(cudaStreamSynchronize(s));
  const unsigned char* base = static_cast<const unsigned char*>(buf.ptr);
  out.clear();
  for (size_t k = 0; k < progs.size(); ++k) {
    GraphProg<Real> g;
    g.nsteps = static_cast<int>(progs[k]->steps.size());
    g.nfwd = progs[k]->nfwd;
    g.max_parts = progs[k]->max_parts;
    g.steps = reinterpret_cast<const int4*>(base + offs[k].steps);
    g.comb = reinterpret_cast<const int4*>(base + offs[k].comb);
    g.rows = reinterpret_cast<const ProgRec<Real>*>(base + offs[k].rows);
    out.push_back(g);
  }
}

template <typename Real>
PassTables<Real> bind_pass(const PassOffsets& o, const int* I, const Real* R) {
  PassTables<Real> t{};
  t.coeff = R + o.coeff; t.scal = R + o.scal; t.wcenter = R + o.wc; t.wsource = R + o.ws; t.wadd = R + o.wa;
  t.ndst = o.ndst; t.dst_node = I + o.dst_node; t.dst_begin = I + o.dst_begin; t.dst_src = I + o.dst_src; t.dst_w = R + o.dst_w;
  t.src_begin = I + o.src_begin; t.src_dst = I + o.src_dst; t.src_w = R + o.src_w;
  t.levels = o.levels; t.level_begin = I + o.level_begin; t.out_nodes = I + o.out_nodes; t.out_begin = I + o.out_begin;
  t.fprod_a = I + o.fa; t.fprod_b = I + o.fb; t.fprod_c = R + o.fc;
  t.rlevel_begin = I + o.rlevel_begin; t.in_nodes = I + o.in_nodes; t.in_begin = I + o.in_begin;
  t.rprod_out = I + o.rout; t.rprod_other = I + o.rother; t.rprod_c = R + o.rc;
  return t;
}

}  // namespace

Engine::Engine(const Model& model, int device, int precision) : model_(model), device_(device), precision_(precision) {
  if (precision != kFP64 && precision != kFP32) throw Error(1, "precision must be 0 (FP64) or 1 (FP32 bulk)");
  pdl_ = default_pdl();
  SUS2G_CUDA(cudaSetDevice(device));
  SUS2G_CUDA(cudaDeviceGetAttribute(&sm_count_, cudaDevAttrMultiProcessorCount, device));
  SUS2G_CUDA(cudaStreamCreateWithFlags(&own_stream_, cudaStreamNonBlocking));
  stream_ = own_stream_;
  // the second stream runs the reverse-edge search beside the first pass: at the most urgent
  // priority, so that its blocks take SM slots ahead of that pass's pending blocks
  int least = 0;
  SUS2G_CUDA(cudaDeviceGetStreamPriorityRange(&least, &urgent_priority_));
  SUS2G_CUDA(cudaStreamCreateWithPriority(&aux_stream_, cudaStreamNonBlocking, urgent_priority_));
  for (cudaEvent_t* e : {&ev_fork_, &ev_rev_, &ev_fork2_, &ev_join2_})
    SUS2G_CUDA(cudaEventCreateWithFlags(e, cudaEventDisableTiming));
  SUS2G_CUDA(upload_pass_constants<float>());
  SUS2G_CUDA(upload_pass_constants<double>());
  SUS2G_CUDA(upload_grad_constants<float>());
  SUS2G_CUDA(upload_grad_constants<double>());
  // scalar readout and gate nodes are written with plain stores; duplicates would race
  auto unique = [](std::vector<int> v) { std::sort(v.begin(), v.end()); return std::adjacent_find(v.begin(), v.end()) == v.end(); };
  if (!unique(model_.scalar_map)) throw Error(3, "SUS2 model: duplicate entries in alpha_moment_mapping");
  if (model_.gated && !unique(model_.gate_nodes)) throw Error(3, "SUS2 model: duplicate gate scalar moments");
  if (model_.K > kMaxK) throw Error(3, "SUS2 model: sh_k_max above 8 is not supported by the GPU engine");
  plans_ = new std::vector<FramePlan>();
  SUS2G_CUDA(cudaMallocHost(&host_total_, 8 * sizeof(int)));
  // [0] error code, [1] cell-list edge capacity overflow (largest count), [2] bin capacity overflow
  error_.ensure(3 * sizeof(int));
  SUS2G_CUDA(cudaMemsetAsync(error_.ptr, 0, 3 * sizeof(int), stream_));
  // the dynamic centre order's counters: zero now; each launch's last warp zeroes its pair again
  work_.ensure(sizeof(int) * kWorkInts);
  SUS2G_CUDA(cudaMemsetAsync(work_.ptr, 0, sizeof(int) * kWorkInts, stream_));
  upload_model();
}

Engine::~Engine() {
  reset_step_graph();
  delete plans_;
  if (host_total_) cudaFreeHost(host_total_);
  if (pinned_) cudaFreeHost(pinned_);
  for (cudaEvent_t e : event_pool_) cudaEventDestroy(e);
  if (precision_ == kFP32) delete static_cast<DevModel<float>*>(dev_model_);
  else delete static_cast<DevModel<double>*>(dev_model_);
  for (cudaEvent_t e : {ev_fork_, ev_rev_, ev_fork2_, ev_join2_})
    if (e) cudaEventDestroy(e);
  if (aux_stream_) cudaStreamDestroy(aux_stream_);
  if (own_stream_) cudaStreamDestroy(own_stream_);
}

// Work on the second stream forks from the engine stream after an event and joins it back
// before the first consumer; the stage timer keeps everything on one stream.
bool Engine::may_fork() const { return !timing_; }

void Engine::wait_reverse() {
  if (!rev_pending_) return;
  SUS2G_CUDA(cudaStreamWaitEvent(stream_, ev_rev_, 0));
  rev_pending_ = false;
}

template <typename Real>
void Engine::upload_tables() {
  const Model& m = model_;
  Packer pk;
  std::vector<int> basic_of(static_cast<size_t>(m.K) * m.H, -1);
  for (int b = 0; b < m.NB; ++b) {
    const auto& q = m.basic[b];
    basic_of[static_cast<size_t>(q[0]) * m.H + q[1] * q[1] + q[1] + q[2]] = b;
  }
  const int o_basic = pk.add_int(basic_of);
  PassOffsets po = pack_pass(m, false, pk);
  PassOffsets pg = m.gated ? pack_pass(m, true, pk) : po;
  const int o_lin = pk.add_real(m.linear);
  const int o_map = pk.add_int(m.scalar_map);
  std::vector<double> wmat;
  std::vector<int> nodes = m.gate_nodes;
  if (m.gated) {
    wmat.resize(static_cast<size_t>(m.F) * m.Q);
    for (int mu = 0; mu < m.F; ++mu)
      for (int q = 0; q < m.Q; ++q) wmat[static_cast<size_t>(mu) * m.Q + q] = m.gate_weight(mu, q);
  }
  const int o_wmat = pk.add_real(wmat);
  const int o_nodes = pk.add_int(nodes);
  // parameter-gradient layout: block offsets in the trainer's order and rank-weight row lists
  std::map<std::string, int> off;
  for (const auto& b : m.layout()) off[b.name] = b.offset;
  auto block = [&](const char* n) { auto it = off.find(n); return it == off.end() ? -1 : it->second; };
  auto weight_rows = [&](const std::vector<ContractionRow>& rows, int nw, int& o_begin, int& o_src, int& o_dst) {
    std::vector<int> begin{0}, src, dst;
    for (int w = 0; w < nw; ++w) {
      for (const auto& r : rows)
        if (r.widx == w) { src.push_back(r.src); dst.push_back(r.dst); }
      begin.push_back(static_cast<int>(src.size()));
    }
    o_begin = pk.add_int(begin);
    o_src = pk.add_int(src);
    o_dst = pk.add_int(dst);
  };
  GradLayout gl{};
  int ow_b = 0, ow_s = 0, ow_d = 0, gw_b = 0, gw_s = 0, gw_d = 0;
  gl.shift_off = block("shift_coeffs");
  gl.species_off = block("species_coeffs");
  gl.linear_off = block("moment_coeffs");
  gl.gate_w_off = block("two_layer_gate_weights");
  gl.nparams = m.param_count();
  gl.outer.coeff_off = block("radial_coeffs");
  gl.outer.coeff_stride = m.B + m.C;
  gl.outer.scal_off = block("scal_coeffs");
  gl.outer.wc_off = block("radial_coeffs") + m.B;
  gl.outer.wc_mu_stride = m.B + m.C;
  gl.outer.wc_t_stride = 1;
  gl.outer.add_off = block("two_layer_gate_additive_coeffs");
  gl.outer.rw_off = block("outer_k_rank1_weights");
  gl.outer.nw = static_cast<int>(m.outer_w.size());
  weight_rows(m.outer_rows, gl.outer.nw, ow_b, ow_s, ow_d);
  if (m.gated) {
    gl.gate.coeff_off = m.gate_shared_radial ? block("two_layer_gate_radial_coeffs") : block("radial_coeffs");
    gl.gate.coeff_stride = m.gate_shared_radial ? m.B : m.B + m.C;
    gl.gate.scal_off = m.gate_decoupled ? block("two_layer_gate_scaling_coeffs") : block("scal_coeffs");
    gl.gate.wc_off = block("two_layer_gate_type_coeffs");
    gl.gate.wc_mu_stride = 1;
    gl.gate.wc_t_stride = m.F;
    gl.gate.add_off = -1;
    gl.gate.rw_off = block("two_layer_gate_k_rank_weights");
    gl.gate.nw = static_cast<int>(m.gate_w.size());
    weight_rows(m.gate_rows, gl.gate.nw, gw_b, gw_s, gw_d);
  }
  std::vector<double> dbl(m.species);
  dbl.insert(dbl.end(), m.shift.begin(), m.shift.end());

  std::vector<Real> reals(pk.reals.begin(), pk.reals.end());
  if (pk.ints.empty()) pk.ints.push_back(0);
  if (reals.empty()) reals.push_back(Real(0));
  tab_int_.ensure(sizeof(int) * pk.ints.size());
  tab_real_.ensure(sizeof(Real) * reals.size());
  tab_dbl_.ensure(sizeof(double) * dbl.size());
  // stream-ordered copies: the engine stream is non-blocking, so a legacy-stream copy would not
  // order against its next kernel; the host vectors die at return, hence the synchronisation
  const cudaStream_t us = stream_ ? stream_ : own_stream_;
  SUS2G_CUDA(cudaMemcpyAsync(tab_int_.ptr, pk.ints.data(), sizeof(int) * pk.ints.size(), cudaMemcpyHostToDevice, us));
  SUS2G_CUDA(cudaMemcpyAsync(tab_real_.ptr, reals.data(), sizeof(Real) * reals.size(), cudaMemcpyHostToDevice, us));
  SUS2G_CUDA(cudaMemcpyAsync(tab_dbl_.ptr, dbl.data(), sizeof(double) * dbl.size(), cudaMemcpyHostToDevice, us));
  SUS2G_CUDA(cudaStreamSynchronize(us));
  const int* I = tab_int_.as<int>();
  const Real* R = tab_real_.as<Real>();
  auto* dm = new DevModel<Real>();
  dm->C = m.C; dm->L = m.L; dm->K = m.K; dm->B = m.B; dm->F = m.F; dm->H = m.H; dm->M = m.M; dm->NB = m.NB;
  dm->S = m.S; dm->Q = m.Q; dm->nblk = m.nblk; dm->scaling_mode = m.scaling_mode;
  dm->rmax = Real(m.max_dist); dm->rang = Real(m.angular); dm->scaling = Real(m.scaling);
  dm->split = m.split; dm->poly = m.poly_cutoff; dm->cutoff_p = m.cutoff_p; dm->gated = m.gated;
  dm->species_readout = m.species_readout;
  dm->basic_of = I + o_basic;
  dm->outer = bind_pass<Real>(po, I, R);
  dm->gate = bind_pass<Real>(pg, I, R);
  {
    // the programs' structure is built once per engine; uploads refresh the rank weights
    if (!prog_[0]) {
      prog_[0].reset(new HostProg(build_prog(m, false)));
      prog_[1].reset(new HostProg(m.gated ? build_prog(m, true) : HostProg{}));
    }
    std::vector<GraphProg<Real>> bound;
    upload_progs<Real>(m, {prog_[0].get(), prog_[1].get()}, tab_prog_, us, bound);
    dm->outer.prog = bound[0];
    dm->gate.prog = m.gated ? bound[1] : bound[0];
    dm->prog_parts = std::max(bound[0].max_parts, m.gated ? bound[1].max_parts : 0);
  }
  dm->linear = R + o_lin;
  dm->species = tab_dbl_.as<double>();
  dm->shift = tab_dbl_.as<double>() + m.C;
  dm->scalar_map = I + o_map;
  dm->gate_wmat = R + o_wmat;
  dm->gate_nodes = I + o_nodes;
  gl.outer.w_begin = I + ow_b; gl.outer.w_src = I + ow_s; gl.outer.w_dst = I + ow_d;
  gl.gate.w_begin = I + gw_b; gl.gate.w_src = I + gw_s; gl.gate.w_dst = I + gw_d;
  dm->grad = gl;
  delete static_cast<DevModel<Real>*>(dev_model_);
  dev_model_ = dm;
}

void Engine::upload_model() {
  SUS2G_CUDA(cudaSetDevice(device_));
  // work already queued on the engine's stream may still read the tables being replaced
  if (stream_) SUS2G_CUDA(cudaStreamSynchronize(stream_));
  reset_step_graph();  // a captured step holds the old tables' values
  if (precision_ == kFP32) upload_tables<float>();
  else upload_tables<double>();
}

long long Engine::nedges() {
  wait_reverse();
  if (!nedges_exact_) {
    // padded layout: the sum of the per-centre counts
    std::vector<int> counts(static_cast<size_t>(std::max(0, ncentres_)));
    if (ncentres_)
      SUS2G_CUDA(cudaMemcpyAsync(counts.data(), counts_.ptr, sizeof(int) * ncentres_, cudaMemcpyDeviceToHost, stream_));
    SUS2G_CUDA(cudaStreamSynchronize(stream_));
    exact_edges_ = 0;
    for (int c : counts) exact_edges_ += c;
    nedges_exact_ = true;
  }
  return exact_edges_;
}

void Engine::copy_edges(long long cap, int* centre, int* neighbour, double* d, long long* count) {
  const long long total = nedges();
  *count = total;
  const int nc = ncentres_;
  std::vector<int> row(static_cast<size_t>(nc) + 1), row_end(static_cast<size_t>(nc));
  std::vector<int> nbr(static_cast<size_t>(std::max<long long>(1, nedges_)));
  const size_t rec = precision_ == kFP32 ? sizeof(EdgeF) : sizeof(EdgeD);
  std::vector<unsigned char> d4(rec * static_cast<size_t>(std::max<long long>(1, nedges_)));
  if (nc) {
    SUS2G_CUDA(cudaMemcpyAsync(row.data(), row_.ptr, sizeof(int) * nc, cudaMemcpyDeviceToHost, stream_));
    SUS2G_CUDA(cudaMemcpyAsync(row_end.data(), d_row_end(), sizeof(int) * nc, cudaMemcpyDeviceToHost, stream_));
  }
  if (nedges_) {
    SUS2G_CUDA(cudaMemcpyAsync(nbr.data(), nbr_.ptr, sizeof(int) * nedges_, cudaMemcpyDeviceToHost, stream_));
    SUS2G_CUDA(cudaMemcpyAsync(d4.data(), d4_.ptr, rec * nedges_, cudaMemcpyDeviceToHost, stream_));
  }
  SUS2G_CUDA(cudaStreamSynchronize(stream_));
  long long k = 0;
  for (int i = 0; i < nc; ++i)
    for (int e = row[i]; e < row_end[i]; ++e, ++k) {
      if (k >= cap) continue;
      if (centre) centre[k] = i;
      if (neighbour) neighbour[k] = nbr[e];
      if (d) {
        if (precision_ == kFP32) {
          const EdgeF& x = reinterpret_cast<const EdgeF*>(d4.data())[e];
          d[3 * k] = x.x; d[3 * k + 1] = x.y; d[3 * k + 2] = x.z;
        } else {
          const EdgeD& x = reinterpret_cast<const EdgeD*>(d4.data())[e];
          d[3 * k] = x.x; d[3 * k + 1] = x.y; d[3 * k + 2] = x.z;
        }
      }
    }
  if (k != total) throw Error(20, "edge rows disagree with the edge count");
}

void* Engine::pinned(size_t bytes) {
  if (bytes > pinned_bytes_) {
    if (pinned_) cudaFreeHost(pinned_);
    pinned_ = nullptr;
    pinned_bytes_ = 0;
    SUS2G_CUDA(cudaMallocHost(&pinned_, bytes));
    pinned_bytes_ = bytes;
  }
  return pinned_;
}

void Engine::check_device_error() {
  enqueue_error_read();
  SUS2G_CUDA(cudaStreamSynchronize(stream_));
  check_error_read();
}

void Engine::enqueue_error_read() {
  wait_reverse();
  SUS2G_CUDA(cudaMemcpyAsync(host_total_ + 4, error_.ptr, 3 * sizeof(int), cudaMemcpyDeviceToHost, stream_));
}

void Engine::check_error_read() {
  const int h = host_total_[4], over = host_total_[5], bin_over = host_total_[6];
  if (over > 0 || bin_over > 0) {
    SUS2G_CUDA(cudaMemsetAsync(error_.ptr, 0, 3 * sizeof(int), stream_));
    if (over > 0) {
      cap_scale_ *= 2.0;
      min_cap_ = std::max(min_cap_, over);
    }
    if (bin_over > 0) {
      bin_cap_scale_ *= 2.0;
      min_bin_cap_ = std::max(min_bin_cap_, bin_over);
    }
    reset_step_graph();
    throw EdgeOverflow();
  }
  if (h) {
    SUS2G_CUDA(cudaMemsetAsync(error_.ptr, 0, sizeof(int), stream_));
    // a warp that left a pass early (a bounded wait that gave up) did not count itself done
    SUS2G_CUDA(cudaMemsetAsync(work_.ptr, 0, sizeof(int) * kWorkInts, stream_));
    static const char* msg[] = {"", "neighbour list capacity or centre index out of range",
                                "periodic image index outside [-64, 63]", "a directed edge has no reverse partner",
                                "zero or non-finite edge length", "non-finite atom coordinate",
                                "atom species index out of range",
                                "a bulk asynchronous copy into shared memory did not complete"};
    throw Error(20 + h, std::string("device check failed: ") + (h > 0 && h < 8 ? msg[h] : "unknown"));
  }
}

cudaEvent_t Engine::take_event() {
  if (event_next_ == event_pool_.size()) {
    cudaEvent_t e;
    SUS2G_CUDA(cudaEventCreate(&e));
    event_pool_.push_back(e);
  }
  return event_pool_[event_next_++];
}

void Engine::mark_begin(int stage) {
  if (!timing_) return;
  open_stage_ = stage;
  open_event_ = take_event();
  SUS2G_CUDA(cudaEventRecord(open_event_, stream_));
}

void Engine::mark_end() {
  if (!timing_ || open_stage_ < 0) return;
  cudaEvent_t e = take_event();
  SUS2G_CUDA(cudaEventRecord(e, stream_));
  marks_.push_back({open_stage_, {open_event_, e}});
  open_stage_ = -1;
}

void Engine::set_timing(bool on) {
  timing_ = on;
  marks_.clear();
  event_next_ = 0;
  for (int i = 0; i < 8; ++i) { stage_ms_[i] = 0; stage_count_[i] = 0; }
}

void Engine::take_stage_times(double* ms, int* counts) {
  SUS2G_CUDA(cudaStreamSynchronize(stream_));
  for (const auto& m : marks_) {
    float t = 0;
    SUS2G_CUDA(cudaEventElapsedTime(&t, m.second.first, m.second.second));
    stage_ms_[m.first] += t;
    stage_count_[m.first] += 1;
  }
  marks_.clear();
  event_next_ = 0;
  for (int i = 0; i < 8; ++i) {
    if (ms) ms[i] = stage_ms_[i];
    if (counts) counts[i] = stage_count_[i];
    stage_ms_[i] = 0;
    stage_count_[i] = 0;
  }
}

void Engine::build_edges(int nframes, const int* frame_natoms, const double* cells, const double* d_pos,
                         const int* d_types) {
  SUS2G_CUDA(cudaSetDevice(device_));
  ++edge_generation_;
  if (nframes < 0) throw Error(1, "negative frame count");
  const double rc = model_.max_dist, rc2 = rc * rc;
  std::vector<FramePlan>& plans = *plans_;
  plans.assign(nframes, FramePlan{});
  int a = 0, bins = 0, bin_cap = min_bin_cap_;
  long long pad_total = 0;
  bins_frames_ = 0;
  for (int f = 0; f < nframes; ++f) {
    FramePlan& fp = plans[f];
    if (frame_natoms[f] < 0) throw Error(1, "negative atom count");
    std::memcpy(fp.cell, cells + 9 * f, sizeof(fp.cell));
    invert3(fp.cell, fp.inv);
    double width[3];
    for (int q = 0; q < 3; ++q) {
      // |column q of inv| = 1 / perpendicular width of the cell along reciprocal direction q
      const double n = std::sqrt(fp.inv[q] * fp.inv[q] + fp.inv[3 + q] * fp.inv[3 + q] + fp.inv[6 + q] * fp.inv[6 + q]);
      fp.reach[q] = rc * n;
      width[q] = 1.0 / n;
    }
    fp.a0 = a;
    fp.a1 = a + frame_natoms[f];
    a = fp.a1;
    fp.use_bins = frame_natoms[f] > 512 && width[0] >= 3 * rc && width[1] >= 3 * rc && width[2] >= 3 * rc;
    fp.bin0 = bins;
    if (fp.use_bins) {
      ++bins_frames_;
      // bins at least r_c / 2 wide (the 5 x 5 x 5 stencil of the fill kernel); widths >= 3 r_c
      // give at least 6 bins per axis, so the periodic stencil never holds a bin twice
      for (int q = 0; q < 3; ++q) fp.nb[q] = std::max(6, std::min(512, static_cast<int>(width[q] / (0.5 * rc))));
      // FP32 prefilter: |error of r^2| <= 2 r_c |error of d|, with |error of d| bounded by the
      // rounding of the wrapped fractions (< 2^-24 each, three terms) times the cell row norms
      double rows = 0;
      for (int q = 0; q < 3; ++q)
        rows += std::sqrt(fp.cell[3 * q] * fp.cell[3 * q] + fp.cell[3 * q + 1] * fp.cell[3 * q + 1] + fp.cell[3 * q + 2] * fp.cell[3 * q + 2]);
      fp.band = 2.0 * rc * (4.0 * 6.0e-8 * rows) * 4.0 + 1e-6;
      fp.screen2 = static_cast<float>(rc2 + fp.band);
      bins += fp.nb[0] * fp.nb[1] * fp.nb[2];
      // bin capacity: twice the frame's mean atoms per bin plus 8 (grown after an overflow)
      const double per_bin = frame_natoms[f] / static_cast<double>(fp.nb[0] * fp.nb[1] * fp.nb[2]);
      bin_cap = std::max(bin_cap, static_cast<int>(std::min(1.0e6, std::ceil(bin_cap_scale_ * per_bin) + 8.0)));
    }
    // FP32 cell rows (hi, lo) and the band of r^2 around r_c^2 that FP32 engines decide in FP64
    // (the cell-list fill's double-float r^2 is within ~1e-6 relative of the exact one, the
    // image scan's FP32 r^2 within ~5e-5)
    for (int q = 0; q < 9; ++q) {
      fp.cellf[q] = static_cast<float>(fp.cell[q]);
      fp.celll[q] = static_cast<float>(fp.cell[q] - static_cast<double>(fp.cellf[q]));
    }
    fp.lo2 = static_cast<float>(rc2 * (1.0 - 1e-4));
    fp.hi2 = static_cast<float>(rc2 * (1.0 + 1e-4));
    for (int q = 0; q < 9; ++q) fp.invf[q] = static_cast<float>(fp.inv[q]);
    for (int q = 0; q < 3; ++q) fp.reachf[q] = static_cast<float>(fp.reach[q]);
    fp.rc2f = static_cast<float>(rc2);
    // padded edge slots of every frame: cap_scale x the mean neighbour count of the frame's density
    // + 64 per centre (grown after an overflow)
    const double vol = std::abs(fp.cell[0] * (fp.cell[4] * fp.cell[8] - fp.cell[5] * fp.cell[7]) -
                                fp.cell[1] * (fp.cell[3] * fp.cell[8] - fp.cell[5] * fp.cell[6]) +
                                fp.cell[2] * (fp.cell[3] * fp.cell[7] - fp.cell[4] * fp.cell[6]));
    const double mean = vol > 0 ? frame_natoms[f] / vol * (4.0 / 3.0) * 3.141592653589793 * rc * rc2 : 0.0;
    fp.cap = std::max(min_cap_, static_cast<int>(std::min(1.0e6, std::ceil(cap_scale_ * mean) + 64.0)));
    fp.pad0 = pad_total;
    pad_total += static_cast<long long>(frame_natoms[f]) * fp.cap;
  }
  natoms_ = ncentres_ = a;
  nframes_ = nframes;
  d_types_ = d_types;
  user_edges_ = false;
  cudaStream_t s = stream_;
  mark_begin(0);
  plan_.ensure(sizeof(FramePlan) * std::max(1, nframes));
  // (a captured step leaves the plans out: they are on the device already, identical by the step key)
  if (nframes && !capturing_)
    SUS2G_CUDA(cudaMemcpyAsync(plan_.ptr, plans.data(), sizeof(FramePlan) * nframes, cudaMemcpyHostToDevice, s));
  frame_of_.ensure(sizeof(int) * std::max(1, a));
  counts_.ensure(sizeof(int) * (a + 1));
  row_.ensure(sizeof(int) * (a + 1));
  {
    // bin counters: zero at the start of a binning pass; the reverse-edge kernel of the previous
    // step cleared the ones it used, so only new or reallocated entries need a memset
    const void* before = bin_count_.ptr;
    bin_count_.ensure(sizeof(int) * (bins + 1));
    if (bin_count_.ptr != before) bin_zeroed_ = 0;
  }
  DevBuf& bin_of = bin_of_;
  bin_of.ensure(sizeof(int) * std::max(1, a));
  // batches with cell lists only: the binning kernel finds each atom's frame itself
  const bool find_frame = bins && bins_frames_ == nframes;
  if (nframes && !find_frame) {
    const bool split = precision_ == kFP32 && bins_frames_ < nframes;
    if (split) posf_.ensure(2 * sizeof(float4) * std::max(1, a));
    k_frame_of<<<nframes, 256, 0, s>>>(plan_.as<FramePlan>(), nframes, frame_of_.as<int>(), d_pos,
                                       split ? posf_.as<float4>() : nullptr, split ? posf_.as<float4>() + a : nullptr);
    ++launches_;
  }
  if (bins) {
    if (bin_zeroed_ < bins + 1) SUS2G_CUDA(cudaMemsetAsync(bin_count_.ptr, 0, sizeof(int) * (bins + 1), s));
    bin_zeroed_ = 0;          // counted into from here on
    bins_used_ = bins + 1;    // cleared again by this step's reverse-edge kernel
    frac_.ensure(sizeof(AtomFrac) * a);
    off_.ensure(sizeof(AtomOff) * a);
    rec_of_.ensure(sizeof(int) * a);
    const size_t slots = static_cast<size_t>(bins) * bin_cap;
    bin_rec_.ensure(sizeof(BinAtom) * slots);
    bin_pos_.ensure(sizeof(BinPos) * slots);
    bin_posf_.ensure(sizeof(BinPosF) * slots);
    // one warp per block: each atom costs ~40 FP64 operations (1/64 of the FP32 rate on this
    // GPU), so small frames are spread over as many SMs as possible (4,096 atoms: 128 SMs)
    k_bin_place<<<(a + kWarp - 1) / kWarp, kWarp, 0, s>>>(plan_.as<FramePlan>(), nframes, find_frame, frame_of_.as<int>(), d_pos, a,
                                               bin_cap, bin_of.as<int>(), rec_of_.as<int>(), bin_count_.as<int>(),
                                               frac_.as<AtomFrac>(),
                                               off_.as<AtomOff>(), bin_rec_.as<BinAtom>(), bin_pos_.as<BinPos>(),
                                               bin_posf_.as<BinPosF>(), error_.as<int>() + 2, error_.as<int>(), d_types,
                                               model_.C);
    ++launches_;
  }
  const unsigned warp_blocks = static_cast<unsigned>((static_cast<long long>(a) * kWarp + 255) / 256);
  const size_t rsz = precision_ == kFP32 ? sizeof(EdgeF) : sizeof(EdgeD);
  const FramePlan* P = plan_.as<FramePlan>();
  const int* FO = frame_of_.as<int>();
  const int* BO = bin_of.as<int>();
  const BinAtom* BR = bin_rec_.as<BinAtom>();
  const BinPos* BP = bin_pos_.as<BinPos>();
  const BinPosF* BPF = bin_posf_.as<BinPosF>();
  const AtomFrac* FR = frac_.as<AtomFrac>();
  const AtomOff* OF = off_.as<AtomOff>();
  int* overflow = error_.as<int>() + 1;
  // every periodic batch: the fill kernels (cell lists and image scan) write each centre's edges
  // to its padded slots and sort them there into the final arrays; no compaction, no host
  // synchronisation.  The edge arrays are sized by the padded capacity, the exact total is the sum
  // of the counts, and an overflow is reported by the step's check_device_error.
  const size_t slots = static_cast<size_t>(std::max<long long>(1, pad_total));
  if (pad_total > 2147483647LL) throw Error(4, "edge build: more than 2^31 - 1 edge slots");
  pad_nbr_.ensure(sizeof(int) * slots);
  pad_d4_.ensure(rsz * slots);
  pad_key_.ensure(sizeof(unsigned long long) * slots);
  nbr_.ensure(sizeof(int) * slots);
  rev_.ensure(sizeof(int) * slots);
  d4_.ensure(rsz * slots);
  key_.ensure(sizeof(unsigned long long) * slots);
  row_end_.ensure(sizeof(int) * std::max(1, a));
  if (a) {
    int* RW = row_.as<int>();
    int* RE = row_end_.as<int>();
    unsigned long long* KO = key_.as<unsigned long long>();
    int* NO = nbr_.as<int>();
    if (bins) {
      if (precision_ == kFP32)
        SUS2G_CUDA(launch_kernel((pdl_ & kPdlFill) != 0, k_edge_fill_bins<float>, dim3(warp_blocks), dim3(kFillWarps * kWarp), 0, s,
            P, FO, d_pos, a, rc2, bin_count_.as<int>(), bin_cap, BR, BP, BPF, BO, rec_of_.as<int>(), FR, OF,
            counts_.as<int>(), pad_nbr_.as<int>(), pad_d4_.as<EdgeF>(), pad_key_.as<unsigned long long>(), overflow,
            error_.as<int>(), RW, RE, KO, NO, d4_.as<EdgeF>()));
      else
        SUS2G_CUDA(launch_kernel((pdl_ & kPdlFill) != 0, k_edge_fill_bins<double>, dim3(warp_blocks), dim3(kFillWarps * kWarp), 0, s,
            P, FO, d_pos, a, rc2, bin_count_.as<int>(), bin_cap, BR, BP, BPF, BO, rec_of_.as<int>(), FR, OF,
            counts_.as<int>(), pad_nbr_.as<int>(), pad_d4_.as<EdgeD>(), pad_key_.as<unsigned long long>(), overflow,
            error_.as<int>(), RW, RE, KO, NO, d4_.as<EdgeD>()));
      ++launches_;
    }
    if (bins_frames_ < nframes) {
      if (precision_ == kFP32)
        SUS2G_CUDA(launch_kernel((pdl_ & kPdlFill) != 0, k_edge_image_fill<float>, dim3(warp_blocks), dim3(kFillWarps * kWarp), 0, s,
            P, FO, d_pos, posf_.as<float4>(), posf_.as<float4>() + a, d_types, model_.C, a, rc2, counts_.as<int>(),
            pad_nbr_.as<int>(), pad_d4_.as<EdgeF>(),
            pad_key_.as<unsigned long long>(), overflow, error_.as<int>(), RW, RE, KO, NO, d4_.as<EdgeF>()));
      else
        SUS2G_CUDA(launch_kernel((pdl_ & kPdlFill) != 0, k_edge_image_fill<double>, dim3(warp_blocks), dim3(kFillWarps * kWarp), 0, s,
            P, FO, d_pos, nullptr, nullptr, d_types, model_.C, a, rc2, counts_.as<int>(), pad_nbr_.as<int>(),
            pad_d4_.as<EdgeD>(),
            pad_key_.as<unsigned long long>(), overflow, error_.as<int>(), RW, RE, KO, NO, d4_.as<EdgeD>()));
      ++launches_;
    }
  }
  nedges_ = pad_total;
  nedges_exact_ = false;
  padded_ = true;
  clear_bins_ = bins > 0;
  finalize_edges();
  mark_end();
}

void Engine::finalize_edges() {
  cudaStream_t s = stream_;
  const int a = ncentres_;
  // (periodic batches were sorted by their fill kernels)
  if (a && !padded_) {
    const int blocks = (a + kSortWarps - 1) / kSortWarps;
    // centres with at most 128 edges rank from shared memory
    constexpr int stage = 128;
    const size_t smem = sizeof(unsigned long long) * kSortWarps * stage;
    if (precision_ == kFP32)
      k_edge_sort<float><<<blocks, kSortWarps * kWarp, smem, s>>>(
          row_.as<int>(), a, stage, tmp_key_.as<unsigned long long>(), tmp_nbr_.as<int>(), tmp_d4_.as<EdgeF>(),
          key_.as<unsigned long long>(), nbr_.as<int>(), d4_.as<EdgeF>());
    else
      k_edge_sort<double><<<blocks, kSortWarps * kWarp, smem, s>>>(
          row_.as<int>(), a, stage, tmp_key_.as<unsigned long long>(), tmp_nbr_.as<int>(), tmp_d4_.as<EdgeD>(),
          key_.as<unsigned long long>(), nbr_.as<int>(), d4_.as<EdgeD>());
    ++launches_;
  }
  if (user_edges_) {
    const int nall = natoms_;
    in_row_.ensure(sizeof(int) * (nall + 1));
    in_edge_.ensure(sizeof(int) * std::max<long long>(1, nedges_));
    counts_.ensure(sizeof(int) * (nall + 1));
    SUS2G_CUDA(cudaMemsetAsync(counts_.ptr, 0, sizeof(int) * (nall + 1), s));
    if (nedges_) {
      const unsigned eb = static_cast<unsigned>((nedges_ + 255) / 256);
      k_iota<<<eb, 256, 0, s>>>(rev_.as<int>(), nedges_);
      k_count_in<<<eb, 256, 0, s>>>(nbr_.as<int>(), nedges_, counts_.as<int>());
      launches_ += 2;
    }
    k_exclusive_scan<<<1, 1024, 0, s>>>(counts_.as<int>(), nall, in_row_.as<int>(), error_.as<int>());
    ++launches_;
    if (nedges_) {
      const unsigned eb = static_cast<unsigned>((nedges_ + 255) / 256);
      SUS2G_CUDA(cudaMemsetAsync(counts_.ptr, 0, sizeof(int) * (nall + 1), s));
      k_fill_in<<<eb, 256, 0, s>>>(nbr_.as<int>(), nedges_, in_row_.as<int>(), counts_.as<int>(), tmp_nbr_.as<int>());
      k_sort_in<<<static_cast<unsigned>((static_cast<long long>(nall) * kWarp + 255) / 256), 256, 0, s>>>(
          in_row_.as<int>(), nall, tmp_nbr_.as<int>(), in_edge_.as<int>());
      launches_ += 2;
    }
  } else if (nedges_ && a) {
    // reverse edges on the second stream: the Static pass and the Effect gate-forward pass do not
    // read them, so they overlap; wait_reverse() joins before the first reader
    // (FP32 engines only: the FP64 pass is long enough that the overlap gains nothing, and its
    // persistent grid loses SMs to the reverse kernel while that runs)
    cudaStream_t rs = s;
    if (may_fork() && precision_ == kFP32) {
      SUS2G_CUDA(cudaEventRecord(ev_fork_, s));
      SUS2G_CUDA(cudaStreamWaitEvent(aux_stream_, ev_fork_, 0));
      rs = aux_stream_;
    }
    SUS2G_CUDA(launch_kernel_priority(rs != s ? urgent_priority_ : 0, k_reverse,
        dim3(static_cast<unsigned>((static_cast<long long>(a) * kWarp + 255) / 256)), dim3(256), 0, rs,
        row_.as<int>(), d_row_end(), key_.as<unsigned long long>(), a, rev_.as<int>(), error_.as<int>(),
        bin_count_.as<int>(), clear_bins_ ? bins_used_ : 0));
    ++launches_;
    if (clear_bins_) bin_zeroed_ = bins_used_;
    if (rs != s) {
      SUS2G_CUDA(cudaEventRecord(ev_rev_, rs));
      rev_pending_ = true;
    }
  }
}

void Engine::set_edges(int nowned, int nall, const int* d_types, int nedges, const int* d_i, const int* d_j, const double* d_d) {
  SUS2G_CUDA(cudaSetDevice(device_));
  ++edge_generation_;
  clear_bins_ = false;
  padded_ = false;
  if (nowned < 0 || nall < nowned || nedges < 0) throw Error(1, "invalid atom layout");
  cudaStream_t s = stream_;
  ncentres_ = nowned;
  natoms_ = nall;
  nframes_ = 1;
  d_types_ = d_types;
  user_edges_ = true;
  std::vector<FramePlan>& plans = *plans_;
  plans.assign(1, FramePlan{});
  plans[0].a0 = 0;
  plans[0].a1 = nowned;
  plan_.ensure(sizeof(FramePlan));
  SUS2G_CUDA(cudaMemcpyAsync(plan_.ptr, plans.data(), sizeof(FramePlan), cudaMemcpyHostToDevice, s));
  counts_.ensure(sizeof(int) * (nowned + 1));
  row_.ensure(sizeof(int) * (nall + 1));
  SUS2G_CUDA(cudaMemsetAsync(counts_.ptr, 0, sizeof(int) * (nowned + 1), s));
  if (nedges) {
    k_count_centres<<<(nedges + 255) / 256, 256, 0, s>>>(d_i, d_j, nedges, counts_.as<int>(), nowned, nall,
                                                         error_.as<int>());
    ++launches_;
  }
  long long total = 0;
  exclusive_scan_host_sync(counts_.as<int>(), nowned, row_.as<int>(), s, &total);
  nedges_ = exact_edges_ = total;
  nedges_exact_ = true;
  const size_t E = std::max<long long>(1, total);
  const size_t rsz = precision_ == kFP32 ? sizeof(EdgeF) : sizeof(EdgeD);
  nbr_.ensure(sizeof(int) * E); tmp_nbr_.ensure(sizeof(int) * E);
  rev_.ensure(sizeof(int) * E);
  d4_.ensure(rsz * E); tmp_d4_.ensure(rsz * E);
  key_.ensure(sizeof(unsigned long long) * E); tmp_key_.ensure(sizeof(unsigned long long) * E);
  DevBuf cursor;
  cursor.ensure(sizeof(int) * (nowned + 1));
  SUS2G_CUDA(cudaMemsetAsync(cursor.ptr, 0, sizeof(int) * (nowned + 1), s));
  if (nedges) {
    if (precision_ == kFP32)
      k_scatter_user_edges<float><<<(nedges + 255) / 256, 256, 0, s>>>(d_i, d_j, d_d, nedges, row_.as<int>(), cursor.as<int>(),
          tmp_nbr_.as<int>(), tmp_d4_.as<EdgeF>(), tmp_key_.as<unsigned long long>(), nowned, nall, error_.as<int>());
    else
      k_scatter_user_edges<double><<<(nedges + 255) / 256, 256, 0, s>>>(d_i, d_j, d_d, nedges, row_.as<int>(), cursor.as<int>(),
          tmp_nbr_.as<int>(), tmp_d4_.as<EdgeD>(), tmp_key_.as<unsigned long long>(), nowned, nall, error_.as<int>());
    ++launches_;
  }
  // rows of ghost atoms are empty
  if (nall > nowned) {
    std::vector<int> tail(nall - nowned, static_cast<int>(total));
    SUS2G_CUDA(cudaMemcpyAsync(row_.as<int>() + nowned + 1, tail.data(), sizeof(int) * tail.size(), cudaMemcpyHostToDevice, s));
    SUS2G_CUDA(cudaStreamSynchronize(s));
  }
  finalize_edges();
}

template <typename Real>
PassArgs<Real> Engine::pass_args() {
  const Model& m = model_;
  const int N = natoms_;
  const size_t E = std::max<long long>(1, nedges_);
  g_.ensure(sizeof(Real) * 3 * E);
  site_.ensure(sizeof(double) * std::max(1, N));
  vir_atom_.ensure(sizeof(double) * 6 * std::max(1, N));
  PassArgs<Real> a{};
  a.dm = *static_cast<DevModel<Real>*>(dev_model_);
  a.moment_mma = moment_mma_ ? 1 : 0;
  a.natoms = ncentres_;
  a.types = d_types_;
  a.row = row_.as<int>();
  a.row_end = d_row_end();
  a.nbr = nbr_.as<int>();
  a.rev = rev_.as<int>();
  a.d4 = static_cast<const typename Vec4<Real>::type*>(d4_.ptr);
  a.g = g_.as<Real>();
  a.site_energy = site_.as<double>();
  a.virial = vir_atom_.as<double>();
  a.desc = desc_out_;
  a.error = error_.as<int>();
  if (m.gated) {
    hsig_.ensure(sizeof(Real) * static_cast<size_t>(std::max(1, N)) * m.F);
    hcontrib_.ensure(sizeof(Real) * E * m.F);
    gmom_.ensure(sizeof(Real) * static_cast<size_t>(std::max(1, N)) * m.M);
    a.hsig = hsig_.as<Real>();
    a.hcontrib = hcontrib_.as<Real>();
    a.gmom = gmom_.as<Real>();
  }
  return a;
}

template <typename Real>
void Engine::run_efs(double* d_energy, double* d_forces, double* d_virial, double* d_site, int stages) {
  const Model& m = model_;
  cudaStream_t s = stream_;
  const int N = natoms_;
  PassArgs<Real> a = pass_args<Real>();
  // stage 1: gate forward (Effect) -- gate signals of the centre atoms
  if (stages & kStageGate) {
    // every centre's site energy, virial and gate signal is written by the passes; only caller
    // layouts with ghosts have rows that must start at zero
    const bool ghosts = user_edges_ && N > ncentres_;
    if (ghosts) {
      SUS2G_CUDA(cudaMemsetAsync(site_.ptr, 0, sizeof(double) * std::max(1, N), s));
      SUS2G_CUDA(cudaMemsetAsync(vir_atom_.ptr, 0, sizeof(double) * 6 * std::max(1, N), s));
    }
    if (m.gated) {
      // ghost rows (caller edges) are filled by the caller's forward exchange
      if (ghosts)
        SUS2G_CUDA(cudaMemsetAsync(hsig_.ptr, 0, sizeof(Real) * static_cast<size_t>(std::max(1, N)) * m.F, s));
      mark_begin(2);
      if (use_gate_split<Real>(0)) launches_ += launch_gate_split<Real>(0, a, (pdl_ & kPdlFirstPass) != 0);
      else launches_ += launch_pass<Real>(kModeGateForward, a, (pdl_ & kPdlFirstPass) != 0);
      mark_end();
    }
  }
  // stage 2: Static pass, or Effect outer pass and the gate-signal adjoint per atom
  if (stages & kStageOuter) {
    if (m.gated) wait_reverse();  // the outer pass writes the gate-signal adjoints at reverse edges
    mark_begin(1);
    const int mode = m.gated ? kModeOuter : kModeStatic;
    if (use_static_split<Real>())
      launches_ += launch_static_split<Real>(a, (pdl_ & (m.gated ? kPdlBetweenPasses : kPdlFirstPass)) != 0);
    else launches_ += launch_pass<Real>(mode, a, (pdl_ & (m.gated ? kPdlBetweenPasses : kPdlFirstPass)) != 0);
    mark_end();
    if (m.gated && user_edges_) {
      hbar_atom_.ensure(sizeof(double) * static_cast<size_t>(std::max(1, N)) * m.F);
      const long long n = static_cast<long long>(N) * m.F;
      if (n) {
        k_hbar_gather<Real><<<static_cast<unsigned>((n + 255) / 256), 256, 0, s>>>(
            in_row_.as<int>(), in_edge_.as<int>(), hcontrib_.as<Real>(), N, m.F, hbar_atom_.as<double>());
        ++launches_;
      }
    }
  }
  // stage 3: Effect gate reverse, forces, per-frame energy and virial
  if (stages & kStageFinish) {
    if (m.gated) {
      if (user_edges_) a.hbar_atom = hbar_atom_.as<double>();
      mark_begin(3);
      if (use_gate_split<Real>(1)) launches_ += launch_gate_split<Real>(1, a, (pdl_ & kPdlBetweenPasses) != 0);
      else launches_ += launch_pass<Real>(kModeGateReverse, a, (pdl_ & kPdlBetweenPasses) != 0);
      mark_end();
    }
    wait_reverse();
    mark_begin(4);
    // frame-reduction buffers first: the arrival counters must be zero before the reduction
    // starts on either stream
    int S = 1;
    if (nframes_) {
      int largest = 0;
      for (const FramePlan& fp : *plans_) largest = std::max(largest, fp.a1 - fp.a0);
      S = std::max(1, std::min(64, (largest + kFrameThreads - 1) / kFrameThreads));
      frame_partial_.ensure(sizeof(double) * 7 * static_cast<size_t>(nframes_) * S);
      if (nframes_ > arrivals_frames_) {
        // arrival counters start at zero; each launch leaves them at zero
        frame_arrivals_.ensure(sizeof(unsigned) * nframes_);
        SUS2G_CUDA(cudaMemsetAsync(frame_arrivals_.ptr, 0, sizeof(unsigned) * nframes_, s));
        arrivals_frames_ = nframes_;
      }
    }
    // the per-frame reduction (site energies and virials) runs on the second stream beside the
    // force gather
    cudaStream_t fs = s;
    if (may_fork() && nframes_ && d_forces && N) {
      SUS2G_CUDA(cudaEventRecord(ev_fork2_, s));
      SUS2G_CUDA(cudaStreamWaitEvent(aux_stream_, ev_fork2_, 0));
      fs = aux_stream_;
    }
    if (d_forces && N) {
      if (user_edges_)
        k_force_gather_user<Real><<<static_cast<unsigned>((static_cast<long long>(N) * kWarp + 255) / 256), 256, 0, s>>>(
            row_.as<int>(), ncentres_, in_row_.as<int>(), in_edge_.as<int>(), g_.as<Real>(), N, d_forces);
      else
        SUS2G_CUDA(launch_kernel((pdl_ & kPdlGather) != 0, k_force_gather<Real>, dim3((N * kWarp + 255) / 256), dim3(256), 0, s,
                                 row_.as<int>(), d_row_end(), rev_.as<int>(), g_.as<Real>(), ncentres_, d_forces));
      ++launches_;
    }
    if (nframes_) {
      k_frame_reduce<<<dim3(nframes_, S), kFrameThreads, 0, fs>>>(
          plan_.as<FramePlan>(), nframes_, S, site_.as<double>(), vir_atom_.as<double>(), d_site,
          frame_partial_.as<double>(), frame_arrivals_.as<unsigned>(), d_energy, d_virial);
      ++launches_;
    } else if (d_site && N) {
      SUS2G_CUDA(cudaMemcpyAsync(d_site, site_.ptr, sizeof(double) * ncentres_, cudaMemcpyDeviceToDevice, s));
    }
    if (fs != s) {
      SUS2G_CUDA(cudaEventRecord(ev_join2_, fs));
      SUS2G_CUDA(cudaStreamWaitEvent(s, ev_join2_, 0));
    }
    mark_end();
  }
}

namespace {
// grad[p] += sum over gradient slices, in two fixed-order levels: block (x, c) sums slices
// c, c + G, c + 2G, ... (G = gridDim.y) of parameters 32 x .. 32 x + 31 in 8 interleaved lanes
// per parameter, combined in shared memory in lane order, into part[c][p]; k_slot_finish adds
// the G partials in order.
constexpr int kSlotGroups = 32;
__global__ void k_slot_partial(const double* slots, int nslots, int nparams, double* part) {
  __shared__ double sh[8][33];
  const int p = blockIdx.x * 32 + threadIdx.x, g = threadIdx.y, c = blockIdx.y, G = gridDim.y;
  double s = 0.0;
  if (p < nparams)
    for (int w = c + G * g; w < nslots; w += 8 * G) s += slots[static_cast<size_t>(w) * nparams + p];
  sh[g][threadIdx.x] = s;
  __syncthreads();
  if (g == 0 && p < nparams) {
    double t = 0.0;
    for (int q = 0; q < 8; ++q) t += sh[q][threadIdx.x];
    part[static_cast<size_t>(c) * nparams + p] = t;
  }
}
__global__ void k_slot_finish(const double* part, int groups, int nparams, double* grad) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= nparams) return;
  double s = 0.0;
  for (int c = 0; c < groups; ++c) s += part[static_cast<size_t>(c) * nparams + p];
  grad[p] += s;
}

// Gate projection weights: dJ/dW[mu][q] = sum_atoms lambda_h[mu] g[node q] + mu_h[mu] gdot[node q],
// a (2F x N) . (N x Q) product reduced over atoms.  Block b takes the atom chunks b, b + grid, ...,
// stages each chunk's lambda / mu rows and gate-node values in shared memory, and adds its partial
// sums into its own slot row (reduced later in fixed order with the other parameter slots), so the
// result is deterministic.  Outputs are taken kGwTile at a time (one per thread and repeat).
constexpr int kGwChunk = 32;
constexpr int kGwThreads = 256;
constexpr int kGwPer = 4;  // outputs per thread per tile
template <typename Real>
__global__ void __launch_bounds__(kGwThreads) k_gate_weight_grad(int natoms, int F, int Q, int M, const int* nodes,
                                                                 const double* lh, const Real* gmom,
                                                                 const Real* gmomd, double* slots, int nparams,
                                                                 int gw_off) {
  // staging and chunk sums in the compute precision (FP32 bulk: the products and each 32-atom
  // chunk's sum in FP32, the chunk partials added in FP64; FP64 plain: FP64 throughout)
  extern __shared__ double gw_sh[];
  Real* sl = reinterpret_cast<Real*>(gw_sh);   // [kGwChunk][2F]
  Real* sg = sl + kGwChunk * 2 * F;            // [kGwChunk][2Q]
  const int FQ = F * Q;
  double* out = slots + static_cast<size_t>(blockIdx.x) * nparams + gw_off;
  for (int tile = 0; tile < FQ; tile += kGwThreads * kGwPer) {
    double acc[kGwPer];
#pragma unroll
    for (int k = 0; k < kGwPer; ++k) acc[k] = 0.0;
    for (int base = blockIdx.x * kGwChunk; base < natoms; base += gridDim.x * kGwChunk) {
      const int n = min(kGwChunk, natoms - base);
      __syncthreads();
      for (int t = threadIdx.x; t < n * 2 * F; t += blockDim.x) sl[t] = Real(lh[static_cast<size_t>(base) * 2 * F + t]);
      for (int t = threadIdx.x; t < n * Q; t += blockDim.x) {
        const int a = t / Q, q = t - a * Q;
        const size_t o = static_cast<size_t>(base + a) * M + nodes[q];
        sg[a * 2 * Q + q] = gmom[o];
        sg[a * 2 * Q + Q + q] = gmomd[o];
      }
      __syncthreads();
#pragma unroll
      for (int k = 0; k < kGwPer; ++k) {
        const int t = tile + k * kGwThreads + threadIdx.x;
        if (t < FQ) {
          const int m = t / Q, q = t - m * Q;
          Real v = Real(0);
          for (int a = 0; a < n; ++a)
            v += sl[a * 2 * F + m] * sg[a * 2 * Q + q] + sl[a * 2 * F + F + m] * sg[a * 2 * Q + Q + q];
          acc[k] += double(v);
        }
      }
    }
#pragma unroll
    for (int k = 0; k < kGwPer; ++k) {
      const int t = tile + k * kGwThreads + threadIdx.x;
      if (t < FQ) out[t] += acc[k];
    }
  }
}
}  // namespace

template <typename Real>
void Engine::run_grad(const double* ew, const double* fw, const double* sw, double* grad,
                      const double* extra_h) {
  const Model& m = model_;
  if (user_edges_) throw Error(1, "the parameter gradient runs on periodic frames (build_edges)");
  if (m.body_combo) throw Error(1, "the parameter gradient of mu-body-linear-combo gates is not implemented");
  cudaStream_t s = stream_;
  const int N = natoms_, P = m.param_count();
  const size_t E = std::max<long long>(1, nedges_);
  const DevModel<Real>& dm = *static_cast<DevModel<Real>*>(dev_model_);
  GradArgs<Real> a{};
  a.dm = dm;
  a.natoms = ncentres_;
  a.types = d_types_;
  a.row = row_.as<int>();
  a.row_end = d_row_end();
  a.nbr = nbr_.as<int>();
  a.rev = rev_.as<int>();
  a.d4 = static_cast<const typename Vec4<Real>::type*>(d4_.ptr);
  a.frame_of = frame_of_.as<int>();
  a.ew = ew;
  a.fw = fw;
  a.sw = sw;
  a.extra_h = extra_h;
  a.error = error_.as<int>();
  // the outer and gate reverse passes whole, or split into their per-atom and per-edge parts
  // (basis size 8) through the moment adjoints in gabar_
  const bool split = grad_split_ && m.B == 8;
  const int part1 = split ? kGradAtomPart : kGradWhole;
  const GradLaunch co = grad_pass_config<Real>(m.L, kGradOuter, dm, ncentres_, sm_count_, part1);
  GradLaunch co2 = co, cf = co, cr = co, cr2 = co;
  if (split) co2 = grad_pass_config<Real>(m.L, kGradOuter, dm, ncentres_, sm_count_, kGradEdgePart);
  if (m.gated) {
    cf = grad_pass_config<Real>(m.L, kGradGateForward, dm, ncentres_, sm_count_);
    cr = grad_pass_config<Real>(m.L, kGradGateReverse, dm, ncentres_, sm_count_, part1);
    cr2 = split ? grad_pass_config<Real>(m.L, kGradGateReverse, dm, ncentres_, sm_count_, kGradEdgePart) : cr;
  }
  const int nslots = std::max({co.grid * co.warps, co2.grid * co2.warps, cf.grid * cf.warps, cr.grid * cr.warps,
                               cr2.grid * cr2.warps});
  if (split) {
    gabar_.ensure(sizeof(Real) * static_cast<size_t>(std::max(1, ncentres_)) * 2 * m.K * (m.L + 1) * (m.L + 1));
    a.abar = gabar_.as<Real>();
  }
  slots_.ensure(sizeof(double) * static_cast<size_t>(nslots) * P);
  SUS2G_CUDA(cudaMemsetAsync(slots_.ptr, 0, sizeof(double) * static_cast<size_t>(nslots) * P, s));
  a.slots = slots_.as<double>();
  if (m.gated) {
    const size_t NF = static_cast<size_t>(std::max(1, N)) * m.F, NM = static_cast<size_t>(std::max(1, N)) * m.M;
    hsig_.ensure(sizeof(Real) * NF);
    hsigd_.ensure(sizeof(Real) * NF);
    gmom_.ensure(sizeof(Real) * NM);
    gmomd_.ensure(sizeof(Real) * NM);
    lhm_.ensure(sizeof(Real) * E * 2 * m.F);
    lh_atom_.ensure(sizeof(double) * 2 * NF);
    a.hsig = hsig_.as<Real>();
    a.hsigd = hsigd_.as<Real>();
    a.gmom = gmom_.as<Real>();
    a.gmomd = gmomd_.as<Real>();
    a.lhm = lhm_.as<Real>();
    a.lh_atom = lh_atom_.as<double>();
    launches_ += launch_grad_pass<Real>(m.L, kGradGateForward, a, cf, s);
    launches_ += launch_grad_pass<Real>(m.L, kGradOuter, a, co, s);
    if (split) launches_ += launch_grad_pass<Real>(m.L, kGradOuter, a, co2, s);
    launches_ += launch_grad_pass<Real>(m.L, kGradGateReverse, a, cr, s);
    if (split) launches_ += launch_grad_pass<Real>(m.L, kGradGateReverse, a, cr2, s);
    const int gw_off = dm.grad.gate_w_off;
    if (N && gw_off >= 0) {
      const int blocks = std::max(1, std::min(nslots, (ncentres_ + kGwChunk - 1) / kGwChunk));
      const size_t smem = sizeof(Real) * kGwChunk * 2 * (m.F + m.Q);
      if (smem > 200 * 1024) throw Error(3, "gate weight gradient: radial functions + gate scalars exceed the shared-memory staging");
      if (smem > 48 * 1024)
        SUS2G_CUDA(cudaFuncSetAttribute(k_gate_weight_grad<Real>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        static_cast<int>(smem)));
      k_gate_weight_grad<Real><<<blocks, kGwThreads, smem, s>>>(ncentres_, m.F, m.Q, m.M, dm.gate_nodes,
                                                                lh_atom_.as<double>(), gmom_.as<Real>(),
                                                                gmomd_.as<Real>(), slots_.as<double>(), P, gw_off);
      ++launches_;
    }
  } else {
    launches_ += launch_grad_pass<Real>(m.L, kGradOuter, a, co, s);
    if (split) launches_ += launch_grad_pass<Real>(m.L, kGradOuter, a, co2, s);
  }
  slot_part_.ensure(sizeof(double) * kSlotGroups * static_cast<size_t>(P));
  k_slot_partial<<<dim3((P + 31) / 32, kSlotGroups), dim3(32, 8), 0, s>>>(slots_.as<double>(), nslots, P,
                                                                         slot_part_.as<double>());
  k_slot_finish<<<(P + 255) / 256, 256, 0, s>>>(slot_part_.as<double>(), kSlotGroups, P, grad);
  launches_ += 2;
}

void Engine::combination_grad(const double* d_ew, const double* d_fw, const double* d_sw, double* d_grad,
                              const double* d_extra_h) {
  SUS2G_CUDA(cudaSetDevice(device_));
  wait_reverse();
  if (precision_ == kFP32) run_grad<float>(d_ew, d_fw, d_sw, d_grad, d_extra_h);
  else run_grad<double>(d_ew, d_fw, d_sw, d_grad, d_extra_h);
}

const void* Engine::d_gate_additive() const {
  if (!model_.gated) return nullptr;
  if (precision_ == kFP32) return static_cast<const DevModel<float>*>(dev_model_)->outer.wadd;
  return static_cast<const DevModel<double>*>(dev_model_)->outer.wadd;
}

int Engine::gate_additive_offset() const {
  if (!model_.gated) return -1;
  if (precision_ == kFP32) return static_cast<const DevModel<float>*>(dev_model_)->grad.outer.add_off;
  return static_cast<const DevModel<double>*>(dev_model_)->grad.outer.add_off;
}

int Engine::static_pass_external(int natoms, const int* types, const int* row, const int* nbr, const void* d4, float* g,
                                 double* site, double* vir, int* error) {
  if (precision_ != kFP32 || model_.gated) throw Error(1, "external Static pass needs a Static model on an FP32 engine");
  PassArgs<float> a{};
  a.dm = *static_cast<DevModel<float>*>(dev_model_);
  a.natoms = natoms;
  a.types = types;
  a.row = row;
  a.row_end = row + 1;
  a.nbr = nbr;
  a.rev = nullptr;
  a.d4 = static_cast<const EdgeF*>(d4);
  a.g = g;
  a.site_energy = site;
  a.virial = vir;
  a.error = error;
  return launch_atom_pass<float>(model_.L, kModeStatic, a, sm_count_, stream_);
}

void Engine::efs(double* d_energy, double* d_forces, double* d_virial, double* d_site) {
  SUS2G_CUDA(cudaSetDevice(device_));
  if (model_.gated && user_edges_ && ncentres_ != natoms_)
    throw Error(1, "Effect models on a ghost layout need the caller's gate-signal exchange: use the staged calls");
  if (precision_ == kFP32) run_efs<float>(d_energy, d_forces, d_virial, d_site, kStageAll);
  else run_efs<double>(d_energy, d_forces, d_virial, d_site, kStageAll);
}

// The energy pass (Static, or the Effect outer pass) split at the per-atom boundary (FP32
// engines, basis size 8): edge->moment forward, per-atom graph kernel, per-edge adjoint -- three
// launches through device moment arrays; the forward and adjoint kernels take the fused pass's
// tile shape.
template <typename Real>
bool Engine::use_static_split() const {
  return static_split_ && sizeof(Real) == 4 && model_.B == 8;
}
template <typename Real>
int Engine::launch_static_split(PassArgs<Real> a, bool pdl) {
  const size_t n = static_cast<size_t>(std::max(1, ncentres_)) * model_.K * model_.H;
  mom_.ensure(sizeof(Real) * n);
  amom_.ensure(sizeof(Real) * n);
  a.mom = mom_.as<Real>();
  a.amom = amom_.as<Real>();
  const int mode = model_.gated ? kModeOuter : kModeStatic;
  a.grid_mode = pass_grid_[mode];
  a.atom_order = pass_order_[mode];
  a.block_warps = pass_wpb_[mode];
  int k = launch_shape<Real>(model_.gated ? kModeOuterFwd : kModeStaticFwd, a, split_blocks_, pdl);
  k += launch_atom_graph<Real>(a, sm_count_, stream_);
  k += launch_shape<Real>(model_.gated ? kModeOuterRev : kModeStaticRev, a, split_blocks_, false);
  return k;
}

// The Effect gate passes split at the per-atom boundary (FP32 engines, basis size 8): which 0 =
// the gate forward pass (edge->moment kernel, then the per-atom gate graph and gate-signal
// projection), 1 = the gate reverse pass (per-atom gather / projection / gate graph reverse,
// then the per-edge adjoint); the per-edge kernels take the fused pass's grid and centre order
// and their own register budget.
template <typename Real>
bool Engine::use_gate_split(int which) const {
  return gate_split_[which] && sizeof(Real) == 4 && model_.B == 8 && model_.gated;
}
template <typename Real>
int Engine::launch_gate_split(int which, PassArgs<Real> a, bool pdl) {
  const size_t n = static_cast<size_t>(std::max(1, ncentres_)) * model_.K * model_.H;
  const int mode = which == 0 ? kModeGateForward : kModeGateReverse;
  a.grid_mode = pass_grid_[mode];
  a.atom_order = pass_order_[mode];
  a.block_warps = pass_wpb_[mode];
  int k = 0;
  if (which == 0) {
    mom_.ensure(sizeof(Real) * n);
    a.mom = mom_.as<Real>();
    k += launch_shape<Real>(kModeGateFwdEdges, a, gate_split_blocks_[0], pdl);
    k += launch_atom_graph<Real>(a, sm_count_, stream_, 1);
  } else {
    amom_.ensure(sizeof(Real) * n);
    a.amom = amom_.as<Real>();
    k += launch_atom_graph<Real>(a, sm_count_, stream_, 2);
    k += launch_shape<Real>(kModeGateRevEdges, a, gate_split_blocks_[1], false);
  }
  return k;
}

// One per-atom pass in the tile shape chosen for its mode (the defaults until autotune runs).
template <typename Real>
int Engine::launch_pass(int mode, PassArgs<Real> a, bool pdl) {
  a.grid_mode = pass_grid_[mode];
  a.atom_order = pass_order_[mode];
  a.h_bulk = pass_stage_[mode];
  a.block_warps = pass_wpb_[mode];
  return launch_shape<Real>(mode, a, pass_blocks_[mode], pdl);
}

// One pass launch in the shape already set in `a` (budget `blocks`); the dynamic centre order
// takes its mode's counter pair.
template <typename Real>
int Engine::launch_shape(int mode, PassArgs<Real> a, int blocks, bool pdl) {
  // the dynamic order's counter pair of this mode (zero between launches: the launch's last
  // warp resets it, so no memset sits between this launch and its predecessor)
  if (a.atom_order == 2) a.work = work_.as<int>() + 2 * mode;
  return launch_atom_pass<Real>(model_.L, mode, a, sm_count_, stream_, blocks, pdl);
}

// Pass-kernel autotuner: on the current layout (the last evaluation's edges), times each pass the
// model runs in every tile shape -- register budget (3 or 4 resident blocks per SM), grid (all
// resident blocks, or the fewest that keep the same centres per warp), centre order (grid-
// strided, contiguous runs per warp, or taken from a device counter) and, for the Effect outer
// pass, the staging of the neighbours' gate-signal rows (plain loads or bulk async copies) --
// `reps` launches each after one warm-up launch, and keeps the fastest shape per pass; then, for
// FP32 models of basis size 8, the pass split at the per-atom boundary in the chosen grid and
// order with either budget, kept where faster.  ms_out[2 mode + (budget - 3)] = the best time of
// each budget (fused).
// The passes read the state the evaluation before them left (gate signals, node adjoints), so a
// full evaluation runs first; the gate reverse pass accumulates into the edge gradients, so the
// next evaluation recomputes them.
template <typename Real>
void Engine::autotune_passes(int reps, int* blocks_out, double* ms_out) {
  const Model& m = model_;
  cudaStream_t s = stream_;
  const int N = natoms_;
  double* scratch = static_cast<double*>(io(7, sizeof(double) * (7 * static_cast<size_t>(std::max(1, nframes_)) +
                                                                  4 * static_cast<size_t>(std::max(1, N)))));
  run_efs<Real>(scratch, scratch + 7 * std::max(1, nframes_), scratch + std::max(1, nframes_), nullptr, kStageAll);
  PassArgs<Real> a = pass_args<Real>();
  const int modes_static[] = {kModeStatic};
  const int modes_gated[] = {kModeGateForward, kModeOuter, kModeGateReverse};
  const int* modes = m.gated ? modes_gated : modes_static;
  const int nmodes = m.gated ? 3 : 1;
  for (int q = 0; q < 4; ++q) { blocks_out[q] = 0; ms_out[2 * q] = ms_out[2 * q + 1] = 0.0; }
  cudaEvent_t e0 = take_event(), e1 = take_event();
  for (int k = 0; k < nmodes; ++k) {
    const int mode = modes[k];
    double best = 0.0;
    int choice = 0, choice_grid = 0, choice_order = 0, choice_stage = 0, choice_wpb = kPassWarps;
    // h_j staging by bulk copies: the outer pass only (basis size 8), where a row is whole
    // 16-byte units
    const int stages = pass_h_bulk<Real>(mode, 1, m.F) && m.B == 8 ? 2 : 1;
    for (int blocks = 3; blocks <= 4; ++blocks)
      for (int grid = 0; grid <= 1; ++grid)
        for (int order = 0; order <= 2; ++order)
          for (int stage = 0; stage < stages; ++stage)
          for (int wpb = 2; wpb <= kPassWarps; wpb += 2) {
            a.grid_mode = grid;
            a.atom_order = order;
            a.h_bulk = stage;
            a.block_warps = wpb;
            launch_shape<Real>(mode, a, blocks, false);
            SUS2G_CUDA(cudaEventRecord(e0, s));
            for (int r = 0; r < reps; ++r) launch_shape<Real>(mode, a, blocks, false);
            SUS2G_CUDA(cudaEventRecord(e1, s));
            SUS2G_CUDA(cudaEventSynchronize(e1));
            float ms = 0.f;
            SUS2G_CUDA(cudaEventElapsedTime(&ms, e0, e1));
            const double per = double(ms) / std::max(1, reps);
            double& slot = ms_out[2 * mode + (blocks - 3)];
            if (slot == 0.0 || per < slot) slot = per;
            if (choice == 0 || per < best) {
              best = per; choice = blocks; choice_grid = grid; choice_order = order; choice_stage = stage;
              choice_wpb = wpb;
            }
          }
    a.h_bulk = 0;
    pass_blocks_[mode] = choice;
    pass_grid_[mode] = choice_grid;
    pass_order_[mode] = choice_order;
    pass_stage_[mode] = choice_stage;
    pass_wpb_[mode] = choice_wpb;
    blocks_out[mode] = choice;
    if ((mode == kModeStatic || mode == kModeOuter) && sizeof(Real) == 4 && m.B == 8) {
      // the fused energy pass (Static, or Effect outer) against its three-kernel split, in the
      // chosen grid and centre order, the split kernels with either register budget
      static_split_ = true;
      double split_best = 0.0;
      int split_choice = 0;
      for (int blocks = 3; blocks <= 4; ++blocks) {
        split_blocks_ = blocks;
        launch_static_split<Real>(a, false);
        SUS2G_CUDA(cudaEventRecord(e0, s));
        for (int r = 0; r < reps; ++r) launch_static_split<Real>(a, false);
        SUS2G_CUDA(cudaEventRecord(e1, s));
        SUS2G_CUDA(cudaEventSynchronize(e1));
        float ms = 0.f;
        SUS2G_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        const double per = double(ms) / std::max(1, reps);
        if (split_choice == 0 || per < split_best) { split_best = per; split_choice = blocks; }
      }
      split_blocks_ = split_choice;
      static_split_ = split_best < best;
    }
    if ((mode == kModeGateForward || mode == kModeGateReverse) && sizeof(Real) == 4 && m.B == 8) {
      // each gate pass against its split (per-edge kernel with either budget, per-atom kernel)
      const int which = mode == kModeGateForward ? 0 : 1;
      gate_split_[which] = true;
      double split_best = 0.0;
      int split_choice = 0;
      for (int blocks = 3; blocks <= 4; ++blocks) {
        gate_split_blocks_[which] = blocks;
        launch_gate_split<Real>(which, a, false);
        SUS2G_CUDA(cudaEventRecord(e0, s));
        for (int r = 0; r < reps; ++r) launch_gate_split<Real>(which, a, false);
        SUS2G_CUDA(cudaEventRecord(e1, s));
        SUS2G_CUDA(cudaEventSynchronize(e1));
        float ms = 0.f;
        SUS2G_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        const double per = double(ms) / std::max(1, reps);
        if (split_choice == 0 || per < split_best) { split_best = per; split_choice = blocks; }
      }
      gate_split_blocks_[which] = split_choice;
      gate_split_[which] = split_best < best;
    }
  }
  event_next_ = 0;
  reset_step_graph();  // a captured step holds the previous budgets
  // graphs captured elsewhere (a trainer's evaluation graph) hold them too: a new edge generation
  // makes their owners rebind and capture again
  ++edge_generation_;
}

void Engine::autotune(int reps, int* blocks_out, double* ms_out) {
  SUS2G_CUDA(cudaSetDevice(device_));
  if (natoms_ <= 0 || ncentres_ <= 0) throw Error(1, "autotune needs an evaluated layout: evaluate once first");
  if (timing_) throw Error(1, "autotune: turn the stage timer off first");
  wait_reverse();
  if (precision_ == kFP32) autotune_passes<float>(reps, blocks_out, ms_out);
  else autotune_passes<double>(reps, blocks_out, ms_out);
  check_device_error();
}

void Engine::set_pass_shape(int mode, int blocks, int grid, int order, int stage, int warps) {
  if (mode < 0 || mode > 3) throw Error(1, "pass shape: mode must be 0 .. 3");
  if (blocks != 0 && blocks != 3 && blocks != 4) throw Error(1, "pass shape: blocks per SM must be 0, 3 or 4");
  if (grid < 0 || grid > 1 || order < 0 || order > 2) throw Error(1, "pass shape: grid 0 .. 1, order 0 .. 2");
  if (stage < 0 || stage > 1) throw Error(1, "pass shape: staging 0 or 1");
  if (warps < 1 || warps > kPassWarps) throw Error(1, "pass shape: warps per block 1 .. 4");
  pass_wpb_[mode] = warps;
  pass_blocks_[mode] = blocks;
  pass_grid_[mode] = grid;
  pass_order_[mode] = order;
  pass_stage_[mode] = stage;
  reset_step_graph();
  ++edge_generation_;  // graphs captured by other owners hold the previous shape
}

void Engine::reset_step_graph() {
  if (step_exec_) cudaGraphExecDestroy(step_exec_);
  if (step_graph_) cudaGraphDestroy(step_graph_);
  step_exec_ = nullptr;
  step_graph_ = nullptr;
  step_key_.clear();
}

void Engine::step_frames(int nframes, const int* frame_natoms, const double* cells, const double* d_pos,
                         const int* d_types, double* d_energy, double* d_forces, double* d_virial, double* d_site) {
  SUS2G_CUDA(cudaSetDevice(device_));
  // layout key: everything the captured launches depend on besides device memory contents
  std::vector<double> key;
  key.reserve(16 + 10 * static_cast<size_t>(std::max(0, nframes)));
  auto ptr = [](const void* p) { return static_cast<double>(reinterpret_cast<uintptr_t>(p)); };
  key.push_back(nframes);
  for (int f = 0; f < nframes; ++f) {
    key.push_back(frame_natoms[f]);
    for (int q = 0; q < 9; ++q) key.push_back(cells[9 * f + q]);
  }
  for (const void* p : {static_cast<const void*>(d_pos), static_cast<const void*>(d_types),
                        static_cast<const void*>(d_energy), static_cast<const void*>(d_forces),
                        static_cast<const void*>(d_virial), static_cast<const void*>(d_site),
                        static_cast<const void*>(stream_)})
    key.push_back(ptr(p));
  key.push_back(cap_scale_);
  key.push_back(min_cap_);
  key.push_back(bin_cap_scale_);
  key.push_back(min_bin_cap_);
  // the same layout as the previous step, with no other edge build, staged call or parameter
  // upload since (those may have regrown the buffers whose addresses a graph holds)
  const bool same = step_graphs_ && !timing_ && key == step_key_ && edge_generation_ == step_gen_;
  if (same && step_exec_) {
    SUS2G_CUDA(cudaGraphLaunch(step_exec_, stream_));
    launches_ += step_launches_;
    step_gen_ = ++edge_generation_;  // the replay rebuilds the edge arrays
    nedges_exact_ = false;
    return;
  }
  // periodic batches build their edges without host synchronisation: the second step of a layout
  // is captured and launched, later ones replay (a one-off layout is never captured)
  if (same && nframes > 0) {
    reset_step_graph();
    const int before = launches_;
    capturing_ = true;
    cudaGraph_t graph = nullptr;
    cudaError_t err = cudaStreamBeginCapture(stream_, cudaStreamCaptureModeRelaxed);
    if (err == cudaSuccess) {
      try {
        build_edges(nframes, frame_natoms, cells, d_pos, d_types);
        efs(d_energy, d_forces, d_virial, d_site);
      } catch (...) {
        capturing_ = false;
        cudaStreamEndCapture(stream_, &graph);
        if (graph) cudaGraphDestroy(graph);
        cudaGetLastError();
        launches_ = before;
        throw;
      }
      err = cudaStreamEndCapture(stream_, &graph);
    }
    capturing_ = false;
    step_launches_ = launches_ - before;
    launches_ = before;  // the capture ran nothing
    if (err == cudaSuccess && graph && cudaGraphInstantiate(&step_exec_, graph, 0) == cudaSuccess) {
      step_graph_ = graph;
      SUS2G_CUDA(cudaGraphLaunch(step_exec_, stream_));
      launches_ += step_launches_;
      step_key_ = key;
      step_gen_ = edge_generation_;
      return;
    }
    // capture refused (e.g. a legacy-stream caller): run this step eagerly and stop capturing
    cudaGetLastError();
    if (graph) cudaGraphDestroy(graph);
    step_exec_ = nullptr;
    step_graphs_ = false;
  } else {
    reset_step_graph();
  }
  build_edges(nframes, frame_natoms, cells, d_pos, d_types);
  efs(d_energy, d_forces, d_virial, d_site);
  step_key_ = key;
  step_gen_ = edge_generation_;
}

void Engine::stage_begin(int nowned, int nall, const int* d_types, int nedges, const int* d_i, const int* d_j,
                         const double* d_d) {
  set_edges(nowned, nall, d_types, nedges, d_i, d_j, d_d);
  if (precision_ == kFP32) run_efs<float>(nullptr, nullptr, nullptr, nullptr, kStageGate);
  else run_efs<double>(nullptr, nullptr, nullptr, nullptr, kStageGate);
  staged_ = 1;
}

void Engine::stage_outer() {
  SUS2G_CUDA(cudaSetDevice(device_));
  if (staged_ != 1) throw Error(1, "staged evaluation: outer() needs begin() first");
  if (precision_ == kFP32) run_efs<float>(nullptr, nullptr, nullptr, nullptr, kStageOuter);
  else run_efs<double>(nullptr, nullptr, nullptr, nullptr, kStageOuter);
  staged_ = 2;
}

void Engine::stage_finish(double* d_energy, double* d_forces, double* d_virial, double* d_site) {
  SUS2G_CUDA(cudaSetDevice(device_));
  if (staged_ != 2) throw Error(1, "staged evaluation: finish() needs outer() first");
  if (precision_ == kFP32) run_efs<float>(d_energy, d_forces, d_virial, d_site, kStageFinish);
  else run_efs<double>(d_energy, d_forces, d_virial, d_site, kStageFinish);
  staged_ = 0;
}

void Engine::stage_rows(int which, int op, int n, const int* d_atoms, int first, double* d_buf) {
  SUS2G_CUDA(cudaSetDevice(device_));
  if (!model_.gated || n <= 0) return;
  const int W = model_.F;
  // forward exchange (h) between begin and outer; reverse exchange (hbar) between outer and finish
  if (which == 0 && staged_ != 1) throw Error(1, "staged evaluation: the gate-signal exchange runs between begin() and outer()");
  if (which == 1 && staged_ != 2) throw Error(1, "staged evaluation: the adjoint exchange runs between outer() and finish()");
  if (!d_atoms && (first < 0 || first + n > natoms_)) throw Error(1, "staged evaluation: atom range outside the layout");
  const long long t = static_cast<long long>(n) * W;
  const unsigned blocks = static_cast<unsigned>((t + 255) / 256);
  cudaStream_t s = stream_;
  if (which == 0) {
    if (op == 0) {
      if (precision_ == kFP32) k_rows_pack<float><<<blocks, 256, 0, s>>>(hsig_.as<float>(), W, n, d_atoms, first, d_buf);
      else k_rows_pack<double><<<blocks, 256, 0, s>>>(hsig_.as<double>(), W, n, d_atoms, first, d_buf);
    } else {
      if (precision_ == kFP32) k_rows_unpack<float><<<blocks, 256, 0, s>>>(hsig_.as<float>(), W, n, d_atoms, first, d_buf, 0);
      else k_rows_unpack<double><<<blocks, 256, 0, s>>>(hsig_.as<double>(), W, n, d_atoms, first, d_buf, 0);
    }
  } else {
    if (op == 0) k_rows_pack<double><<<blocks, 256, 0, s>>>(hbar_atom_.as<double>(), W, n, d_atoms, first, d_buf);
    else k_rows_unpack<double><<<blocks, 256, 0, s>>>(hbar_atom_.as<double>(), W, n, d_atoms, first, d_buf, 1);
  }
  ++launches_;
}

}  // namespace sus2g
