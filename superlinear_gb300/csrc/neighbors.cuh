// Periodic directed-edge builder (CSR by centre) and the small gather / reduction kernels.
//
// Edge set: every (i, j, image n) with |x_j - x_i + n.cell|^2 < r_c^2 except i == j with n = 0,
// i.e. the reference's neighbourhoods including self images in small cells
// (src/neighborhoods.cpp:145-350; the standalone harness enumerates images the same way,
// interfaces/lammps/tests/embedded_efs.cpp:49-66).  Two enumerations produce that set:
//   * image scan (small frames): for each j of the frame the image range
//     ceil(-f - reach) .. floor(-f + reach) per axis, f = (x_j - x_i) . inv(cell),
//     reach_q = r_c |inv(cell)[:, q]|  -- the harness's own bounds;
//   * cell list (frames whose perpendicular widths are all >= 3 r_c): fractional bins of width
//     >= r_c, 27 neighbouring bins with periodic wrap; each (j, n) is found exactly once.
// Afterwards each centre's edges are sorted by (j, n) -- the image-scan order -- and every edge
// gets the index of its reverse edge (j -> i, -n) by binary search, which makes the force gather
// F_i = sum_{e out of i} (g_e - g_rev(e)) atomic-free and deterministic.
#pragma once
#include "device_common.cuh"

namespace sus2g {

struct FramePlan {
  double cell[9];   // rows are lattice vectors
  double inv[9];    // inverse of the row matrix: frac_q = sum_a x_a inv[a][q]
  double reach[3];
  int a0, a1;       // atom range
  int use_bins;
  int nb[3];
  int bin0;         // first bin index of this frame in the global bin arrays
};

__device__ __forceinline__ unsigned long long edge_key(int j, int n0, int n1, int n2) {
  return (static_cast<unsigned long long>(j) << 21) |
         (static_cast<unsigned long long>(n0 + 64) << 14) |
         (static_cast<unsigned long long>(n1 + 64) << 7) |
         static_cast<unsigned long long>(n2 + 64);
}

// Enumerate the edges of centre i; Emit(j, n0, n1, n2, dx, dy, dz, r2) is called in a fixed order.
template <typename Emit>
__device__ __forceinline__ void enumerate_edges(int i, const FramePlan& fp, const double* pos, double rc2,
                                                const int* bin_start, const int* bin_atoms, int* error, Emit&& emit) {
  const double xi = pos[3 * i], yi = pos[3 * i + 1], zi = pos[3 * i + 2];
  const double* c = fp.cell;
  const double* inv = fp.inv;
  if (!fp.use_bins) {
    for (int j = fp.a0; j < fp.a1; ++j) {
      const double dx = pos[3 * j] - xi, dy = pos[3 * j + 1] - yi, dz = pos[3 * j + 2] - zi;
      double f[3];
      int lo[3], hi[3];
      for (int q = 0; q < 3; ++q) {
        f[q] = dx * inv[q] + dy * inv[3 + q] + dz * inv[6 + q];
        lo[q] = static_cast<int>(ceil(-f[q] - fp.reach[q]));
        hi[q] = static_cast<int>(floor(-f[q] + fp.reach[q]));
      }
      for (int a = lo[0]; a <= hi[0]; ++a)
        for (int b = lo[1]; b <= hi[1]; ++b)
          for (int cc = lo[2]; cc <= hi[2]; ++cc) {
            if (i == j && a == 0 && b == 0 && cc == 0) continue;
            const double vx = dx + a * c[0] + b * c[3] + cc * c[6];
            const double vy = dy + a * c[1] + b * c[4] + cc * c[7];
            const double vz = dz + a * c[2] + b * c[5] + cc * c[8];
            const double r2 = vx * vx + vy * vy + vz * vz;
            if (r2 < rc2) {
              if (a < -64 || a > 63 || b < -64 || b > 63 || cc < -64 || cc > 63) { record_error(error, kErrImageRange); continue; }
              emit(j, a, b, cc, vx, vy, vz, r2);
            }
          }
    }
    return;
  }
  double si[3];
  int oi[3], bi[3];
  for (int q = 0; q < 3; ++q) {
    si[q] = xi * inv[q] + yi * inv[3 + q] + zi * inv[6 + q];
    oi[q] = static_cast<int>(floor(si[q]));
    double w = si[q] - oi[q];
    bi[q] = min(static_cast<int>(w * fp.nb[q]), fp.nb[q] - 1);
  }
  for (int d0 = -1; d0 <= 1; ++d0)
    for (int d1 = -1; d1 <= 1; ++d1)
      for (int d2 = -1; d2 <= 1; ++d2) {
        const int raw[3] = {bi[0] + d0, bi[1] + d1, bi[2] + d2};
        int wb[3], W[3];
        for (int q = 0; q < 3; ++q) {
          W[q] = raw[q] < 0 ? -1 : (raw[q] >= fp.nb[q] ? 1 : 0);
          wb[q] = raw[q] - W[q] * fp.nb[q];
        }
        const int bin = fp.bin0 + (wb[0] * fp.nb[1] + wb[1]) * fp.nb[2] + wb[2];
        for (int p = bin_start[bin]; p < bin_start[bin + 1]; ++p) {
          const int j = bin_atoms[p];
          const double xj = pos[3 * j], yj = pos[3 * j + 1], zj = pos[3 * j + 2];
          int n[3];
          for (int q = 0; q < 3; ++q) {
            const double sj = xj * inv[q] + yj * inv[3 + q] + zj * inv[6 + q];
            n[q] = W[q] + oi[q] - static_cast<int>(floor(sj));
          }
          if (i == j && n[0] == 0 && n[1] == 0 && n[2] == 0) continue;
          const double vx = xj - xi + n[0] * c[0] + n[1] * c[3] + n[2] * c[6];
          const double vy = yj - yi + n[0] * c[1] + n[1] * c[4] + n[2] * c[7];
          const double vz = zj - zi + n[0] * c[2] + n[1] * c[5] + n[2] * c[8];
          const double r2 = vx * vx + vy * vy + vz * vz;
          if (r2 < rc2) {
            if (n[0] < -64 || n[0] > 63 || n[1] < -64 || n[1] > 63 || n[2] < -64 || n[2] > 63) { record_error(error, kErrImageRange); continue; }
            emit(j, n[0], n[1], n[2], vx, vy, vz, r2);
          }
        }
      }
}

}  // namespace sus2g
