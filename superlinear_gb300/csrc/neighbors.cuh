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
//     >= r_c / 2, the 125 bins within two of the centre's with periodic wrap; each (j, n) is
//     found exactly once.
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
  int cap;          // cell-list frames: edge slots per centre in the padded staging buffers
  long long pad0;   // cell-list frames: first padded slot of the frame (centre i: pad0 + (i - a0) cap)
  float cellf[9];   // FP32 copy of the cell for the candidate prefilter
  float celll[9];   // cell - cellf: with cellf the double-float form of the cell rows
  double band;      // |r^2 error| bound of the FP32 prefilter; candidates within it get the FP64 test
  float screen2;    // FP32 prefilter threshold r_c^2 + band
  float lo2, hi2;   // FP32 engines: r^2 below lo2 is inside, above hi2 outside, else the FP64 test
  float invf[9], reachf[3], rc2f;  // FP32 copies for the image scan's FP32 ranges and bound
};

// Per-atom wrapped fractional coordinates (FP32, in [0,1)) and the integer cell offsets
// floor(frac) (FP64 arithmetic), written by the binning kernel for cell-list frames.
struct AtomFrac { float x, y, z; int pad; };
struct AtomOff { int x, y, z, pad; };
// One bin slot (atoms grouped by bin): fractional coordinates, the atom's index and its integer
// cell offset, so that a candidate is one 32-byte load.
struct __align__(16) BinAtom { float x, y, z; int j; int ox, oy, oz, pad; };
// The same slot's exact position wrapped into the home cell, x - floor(frac) . cell (FP64), and the
// atom's index: the exact test forms x_j + n.cell - x_i as wrapped x_j + ((w + off_i) . cell - x_i),
// whose second term is one constant per (centre, neighbouring bin).
struct __align__(16) BinPos { double x, y, z; int j, pad; };
// FP32 engines: the wrapped position as double-float parts x = xh + xl (xh = fl32(x)).
struct __align__(16) BinPosF { float xh, yh, zh; int j; float xl, yl, zl; int pad; };

__device__ __forceinline__ unsigned long long edge_key(int j, int n0, int n1, int n2) {
  return (static_cast<unsigned long long>(j) << 21) |
         (static_cast<unsigned long long>(n0 + 64) << 14) |
         (static_cast<unsigned long long>(n1 + 64) << 7) |
         static_cast<unsigned long long>(n2 + 64);
}

// Cell-list frames, one warp per centre i.  Bins are at least r_c / 2 wide, so every neighbour lies
// in the 5 x 5 x 5 bins around the centre's bin (about 2.3x fewer candidates than 27 bins of width
// r_c).  Each lane owns four of those 125 bins and walks their atoms, two candidates per
// iteration (independent loads in flight); candidates that pass the FP32 prefilter are appended
// to a per-warp queue in shared memory (`queue`, 128 entries) and whenever 32 are queued the warp
// tests a full warp of them:
//   * FP64 engines: x_j + n.cell - x_i and r^2 in FP64;
//   * FP32 engines: the same vector from double-float (hi, lo) parts in FP32 arithmetic, with the
//     FP64 test only for the rare entries whose FP32 r^2 lies within 1e-4 relative of r_c^2
//     (FP64 runs at 1/64 of the FP32 rate on this GPU).
// Either way the accepted set is exactly {r^2 < r_c^2} in FP64.  The vector's periodic part
// depends only on the wrap w in {-1, 0, 1}^3 of the neighbouring bin: lane k < 27 holds the shift
// (w_k + off_i) . cell - x_i of wrap k.  Accepted edges of each round are reported through
// Round(mask, lane_accepted, j, n0, n1, n2, x, y, z, r) (Real components and distance), so the
// caller can count or write them with one ballot per round.
constexpr int kEdgeQueue = 128;
constexpr int kBinReach = 2;                       // bins on each side of the centre's bin
constexpr int kBinSpan = 2 * kBinReach + 1;        // 5
constexpr int kBinStencil = kBinSpan * kBinSpan * kBinSpan;  // 125
constexpr int kBinsPerLane = 4;                    // 32 x 4 >= 125
__device__ __forceinline__ int pack_image(int n0, int n1, int n2) {
  return ((n0 + 64) << 14) | ((n1 + 64) << 7) | (n2 + 64);
}

// double-float sum (ah + al) + (bh + bl), rounded to FP32 (two-sum of the high parts)
__device__ __forceinline__ float df_add(float ah, float al, float bh, float bl) {
  const float s = ah + bh;
  const float v = s - ah;
  const float e = (ah - (s - v)) + (bh - v);
  return s + (e + (al + bl));
}

// Double-float accumulation (h, l) += (bh, bl) (Knuth two-sum of the leading parts, the trailing
// parts added once): absolute error a few 2^-48 of the operands' magnitudes.
__device__ __forceinline__ void df_acc(float& h, float& l, float bh, float bl) {
  const float s = h + bh;
  const float v = s - h;
  const float e = (h - (s - v)) + (bh - v) + (l + bl);
  h = s + e;
  l = e - (h - s);
}

// (h, l) += m (ch, cl) for a small integer m (|m| <= 64): m ch is split exactly by an FMA.
__device__ __forceinline__ void df_acc_mul(float& h, float& l, float m, float ch, float cl) {
  const float p = m * ch;
  const float pe = fmaf(m, ch, -p);
  df_acc(h, l, p, fmaf(m, cl, pe));
}

// Per-warp shared tables of the fill: the 27 wrap shifts (FP64 and double-float parts) and the
// lanes' bins (start, length).
// Per wrap w in {-1, 0, 1}^3 of a neighbouring bin (index (w0 + 1) 9 + (w1 + 1) 3 + (w2 + 1)):
// the exact shift (w + off_i) . cell - x_i in FP64 and as double-float parts, the image base
// w + off_i and the FP32 fractional shift w - frac_i of the prefilter.
struct __align__(16) WrapShift {
  double x, y, z;
  float hx, hy, hz, lx, ly, lz;
  int4 nb;      // (w0 + off_i.x, w1 + off_i.y, w2 + off_i.z, -)
  float4 df;    // (w0 - frac_i.x, w1 - frac_i.y, w2 - frac_i.z, -)
};
struct BinWalk {
  WrapShift shift[27];
};

template <typename Real, typename Round>
__device__ __forceinline__ void warp_bin_edges(int i, const FramePlan& fp, const double* pos, double rc2,
                                               const int* bin_count, int bin_cap, const BinAtom* bin_rec,
                                               const BinPos* bin_pos,
                                               const BinPosF* bin_posf, const int* bin_of, const int* rec_of,
                                               const AtomFrac* frac, const AtomOff* off, int* error, int2* queue,
                                               BinWalk& walk, Round&& round) {
  const int lane = threadIdx.x & 31;
  const unsigned below = (1u << lane) - 1u;
  const int local = bin_of[i] - fp.bin0;
  const int bi0 = local / (fp.nb[1] * fp.nb[2]), bi1 = (local / fp.nb[2]) % fp.nb[1], bi2 = local % fp.nb[2];
  const AtomFrac fi = frac[i];
  const AtomOff oi = off[i];
  const double* c = fp.cell;
  const float* cf = fp.cellf;
  const int self_rec = rec_of[i];  // the centre's own bin record
  // lane k < 27: wrap k = (w0 + 1) 9 + (w1 + 1) 3 + (w2 + 1).  Its shift (w + off_i) . cell - x_i =
  // w . cell - (x_i wrapped into the home cell): FP64 engines in FP64; FP32 engines as double-float
  // parts from the cell's and the centre record's (hi, lo) parts in FP32 arithmetic (their exact
  // FP64 shift is formed only for the rare entries near the cutoff)
  if (lane < 27) {
    const int w0 = lane / 9 - 1, w1 = (lane / 3) % 3 - 1, w2 = lane % 3 - 1;
    WrapShift w;
    if constexpr (sizeof(Real) == 8) {
      const double a0 = w0 + oi.x, a1 = w1 + oi.y, a2 = w2 + oi.z;
      w.x = a0 * c[0] + a1 * c[3] + a2 * c[6] - pos[3 * i];
      w.y = a0 * c[1] + a1 * c[4] + a2 * c[7] - pos[3 * i + 1];
      w.z = a0 * c[2] + a1 * c[5] + a2 * c[8] - pos[3 * i + 2];
      w.hx = w.hy = w.hz = w.lx = w.ly = w.lz = 0.f;
    } else {
      const BinPosF me = bin_posf[self_rec];
      const float* cl = fp.celll;
      float h[3], l[3];
#pragma unroll
      for (int q = 0; q < 3; ++q) {
        // w0 row0 + w1 row1 + w2 row2 - x_i, each term an exact (hi, lo) pair
        float sh = -(q == 0 ? me.xh : (q == 1 ? me.yh : me.zh));
        float sl = -(q == 0 ? me.xl : (q == 1 ? me.yl : me.zl));
        const int wq[3] = {w0, w1, w2};
#pragma unroll
        for (int r = 0; r < 3; ++r) {
          const float th = static_cast<float>(wq[r]) * cf[3 * r + q], tl = static_cast<float>(wq[r]) * cl[3 * r + q];
          const float s2 = sh + th, v = s2 - sh;
          const float e = (sh - (s2 - v)) + (th - v);
          const float lo = e + (sl + tl);
          sh = s2 + lo;
          sl = lo - (sh - s2);
        }
        h[q] = sh;
        l[q] = sl;
      }
      w.x = w.y = w.z = 0.0;
      w.hx = h[0]; w.hy = h[1]; w.hz = h[2];
      w.lx = l[0]; w.ly = l[1]; w.lz = l[2];
    }
    w.nb = make_int4(w0 + oi.x, w1 + oi.y, w2 + oi.z, 0);
    w.df = make_float4(static_cast<float>(w0) - fi.x, static_cast<float>(w1) - fi.y, static_cast<float>(w2) - fi.z, 0.f);
    walk.shift[lane] = w;
  }
  // the lane's bins (stencil slots 4 lane + u) laid end to end: record offset start_u - excl_u,
  // exclusive ends excl_1..3 and the wraps packed 5 bits each
  int off0 = 0, off1 = 0, off2 = 0, off3 = 0, ex1 = 0, ex2 = 0, ex3 = 0, kpack = 0, mine = 0;
#pragma unroll
  for (int u = 0; u < kBinsPerLane; ++u) {
    const int sl = kBinsPerLane * lane + u;
    int bstart = 0, blen = 0, wk = 13;
    if (sl < kBinStencil) {
      const int raw0 = bi0 + sl / (kBinSpan * kBinSpan) - kBinReach;
      const int raw1 = bi1 + (sl / kBinSpan) % kBinSpan - kBinReach;
      const int raw2 = bi2 + sl % kBinSpan - kBinReach;
      const int w0 = raw0 < 0 ? -1 : (raw0 >= fp.nb[0] ? 1 : 0);
      const int w1 = raw1 < 0 ? -1 : (raw1 >= fp.nb[1] ? 1 : 0);
      const int w2 = raw2 < 0 ? -1 : (raw2 >= fp.nb[2] ? 1 : 0);
      const int bin = fp.bin0 + ((raw0 - w0 * fp.nb[0]) * fp.nb[1] + (raw1 - w1 * fp.nb[1])) * fp.nb[2] +
                      (raw2 - w2 * fp.nb[2]);
      bstart = bin * bin_cap;
      blen = min(bin_count[bin], bin_cap);
      wk = (w0 + 1) * 9 + (w1 + 1) * 3 + (w2 + 1);
    }
    const int o = bstart - mine;
    if (u == 0) off0 = o;
    if (u == 1) { off1 = o; ex1 = mine; }
    if (u == 2) { off2 = o; ex2 = mine; }
    if (u == 3) { off3 = o; ex3 = mine; }
    kpack |= wk << (5 * u);
    mine += blen;
  }
  int most = mine;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) most = max(most, __shfl_xor_sync(0xffffffffu, most, o));
  // the FP32 cell rows of the prefilter, in registers
  float cr[9];
#pragma unroll
  for (int q = 0; q < 9; ++q) cr[q] = cf[q];
  __syncwarp();
  const float screen = fp.screen2, lo2 = fp.lo2, hi2 = fp.hi2;
  int queued = 0;  // warp-uniform
  // test of queue entries [0, n) (one per lane) and the round callback
  // queue entry: (bin record index, packed image | wrap index k << 21)
  auto drain = [&](int n) {
    bool ok = false;
    int j = 0, n0 = 0, n1 = 0, n2 = 0, k = 0;
    int2 q = make_int2(0, 0);
    if (lane < n) {
      q = queue[lane];
      k = q.y >> 21;
      n0 = ((q.y >> 14) & 127) - 64; n1 = ((q.y >> 7) & 127) - 64; n2 = (q.y & 127) - 64;
    }
    if constexpr (sizeof(Real) == 8) {
      double vx = 0, vy = 0, vz = 0, r2 = 0;
      if (lane < n) {
        const BinPos bp = bin_pos[q.x];
        const WrapShift& w = walk.shift[k];
        j = bp.j;
        vx = bp.x + w.x;
        vy = bp.y + w.y;
        vz = bp.z + w.z;
        r2 = vx * vx + vy * vy + vz * vz;
        ok = r2 < rc2;
      }
      const unsigned mask = __ballot_sync(0xffffffffu, ok);
      round(mask, ok, j, n0, n1, n2, Real(vx), Real(vy), Real(vz), Real(sqrt(r2)));
    } else {
      float vx = 0, vy = 0, vz = 0, r2 = 0;
      if (lane < n) {
        const BinPosF bp = bin_posf[q.x];
        const WrapShift& w = walk.shift[k];
        j = bp.j;
        vx = df_add(bp.xh, bp.xl, w.hx, w.lx);
        vy = df_add(bp.yh, bp.yl, w.hy, w.ly);
        vz = df_add(bp.zh, bp.zl, w.hz, w.lz);
        r2 = vx * vx + vy * vy + vz * vz;
        ok = r2 < lo2;
        if (!ok && r2 < hi2) {
          // near the cutoff: the FP64 test decides, x_j + (w + off_i) . cell - x_i in FP64
          const BinPos bd = bin_pos[q.x];
          const double a0 = k / 9 - 1 + oi.x, a1 = (k / 3) % 3 - 1 + oi.y, a2 = k % 3 - 1 + oi.z;
          const double dx = bd.x + (a0 * c[0] + a1 * c[3] + a2 * c[6] - pos[3 * i]);
          const double dy = bd.y + (a0 * c[1] + a1 * c[4] + a2 * c[7] - pos[3 * i + 1]);
          const double dz = bd.z + (a0 * c[2] + a1 * c[5] + a2 * c[8] - pos[3 * i + 2]);
          const double d2 = dx * dx + dy * dy + dz * dz;
          ok = d2 < rc2;
          vx = static_cast<float>(dx); vy = static_cast<float>(dy); vz = static_cast<float>(dz);
          r2 = static_cast<float>(d2);
        }
      }
      const unsigned mask = __ballot_sync(0xffffffffu, ok);
      round(mask, ok, j, n0, n1, n2, vx, vy, vz, sqrtf(r2));
    }
  };
  // FP32 prefilter of the lane's candidate t (0 <= t < mine, else -1): packed image with the wrap
  // index, and the bin record index
  auto screen_candidate = [&](int t, int& rec_index) -> int {
    if (t >= mine) return -1;
    const int u1 = t >= ex1, u2 = t >= ex2, u3 = t >= ex3;
    rec_index = t + (u3 ? off3 : (u2 ? off2 : (u1 ? off1 : off0)));
    const int k = (kpack >> (5 * (u1 + u2 + u3))) & 31;
    const BinAtom rec = bin_rec[rec_index];
    const float4 df = walk.shift[k].df;
    const float sx32 = rec.x + df.x, sy32 = rec.y + df.y, sz32 = rec.z + df.z;
    const float fx = sx32 * cr[0] + sy32 * cr[3] + sz32 * cr[6];
    const float fy = sx32 * cr[1] + sy32 * cr[4] + sz32 * cr[7];
    const float fz = sx32 * cr[2] + sy32 * cr[5] + sz32 * cr[8];
    if (fx * fx + fy * fy + fz * fz >= screen) return -1;
    const int4 nb = walk.shift[k].nb;
    const int n0 = nb.x - rec.ox, n1 = nb.y - rec.oy, n2 = nb.z - rec.oz;
    if (i == rec.j && n0 == 0 && n1 == 0 && n2 == 0) return -1;
    if (n0 < -64 || n0 > 63 || n1 < -64 || n1 > 63 || n2 < -64 || n2 > 63) {
      record_error(error, kErrImageRange);
      return -1;
    }
    return pack_image(n0, n1, n2) | (k << 21);
  };
  auto push = [&](int packed, int rec_index) {
    const bool pre = packed >= 0;
    const unsigned m = __ballot_sync(0xffffffffu, pre);
    if (pre) queue[queued + __popc(m & below)] = make_int2(rec_index, packed);
    queued += __popc(m);
  };
  // two candidates per lane per iteration (their loads overlap)
  for (int t = 0; t < most; t += 2) {
    int ra = 0, rb = 0;
    const int pa = screen_candidate(t, ra);
    const int pb = screen_candidate(t + 1, rb);
    push(pa, ra);
    push(pb, rb);
    __syncwarp();
    while (queued >= 32) {
      drain(32);
      __syncwarp();
      // move the remainder (< 96 entries) to the front, 32 at a time in order
      for (int q0 = 32; q0 < queued; q0 += 32) {
        int2 rest = make_int2(0, 0);
        const bool have = q0 + lane < queued;
        if (have) rest = queue[q0 + lane];
        __syncwarp();
        if (have) queue[q0 - 32 + lane] = rest;
        __syncwarp();
      }
      queued -= 32;
    }
  }
  if (queued > 0) drain(queued);
  __syncwarp();
}

}  // namespace sus2g
