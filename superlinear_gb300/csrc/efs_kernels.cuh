// Warp-per-atom passes of the SUS2-SH energy / force / virial evaluation.
//
// Algorithm (per centre atom i, edges e = (i -> j, d) sorted by centre):
//   forward   A_i[k,l,m] = sum_e x0(t_i,mu) x3(t_j,mu) R_mu(r_e) Y_lm(d_e),  mu = k (L+1) + l
//             (sus2_sl_kernel.cpp:340-354 forward_moments, :165-216 edge_basis)
//   contract  ranked K -> rank contraction (sus2_sl_kernel.cpp:104-105, 217-221)
//   graph     v[out] += c v[a] v[b] over the pass's product range (:308-313)
//   readout   E_i = species + shift + sum_q rho_q v[map q]            (:556)
//   reverse   adjoint of readout, graph and contraction (:527-528), then per edge
//             g_e = dE/dd_e = sum_b Abar[b] x0 x3 (R'_mu d/r Y_h + R_mu grad Y_h)  (:356-380)
//   Effect    gate pass first (x0 x1 = gate type factors, gate radial / warp), h_i = W g_i
//             (:447-455); outer x3 = tau_j + alpha_j h_j; the outer reverse also emits
//             hbar_j[mu] += Abar x0 alpha R Y (:368), gathered per atom and pushed back through
//             the gate graph (:558-559).
//
// GPU mapping: one warp owns one centre atom at a time.  Lanes take edges (32 per batch); each
// lane evaluates Y_lm and the radial functions of its edge in registers and stages u_mu =
// x0 x3 R_mu and Y_h in shared memory; lanes then switch to owning (k, lm) moment items and
// reduce over the staged edges in a fixed order: a plain sum over each batch of <= 32 edges, then a
// Kahan-compensated add of the batch partial into the atom's moment (FP32 bulk) -- no atomics,
// deterministic.  The rank contraction and the product graph, forward and reverse, run as the
// pass's lane-balanced graph program (GraphProg) over shared-memory node arrays.  The adjoint
// pass recomputes Y and R per edge instead of storing them and writes g_e per edge; forces are
// gathered per atom through the reverse-edge permutation by a separate kernel.
#pragma once
#include <type_traits>

#include "basis.cuh"

namespace sus2g {

enum PassMode : int {
  kModeStatic = 0, kModeGateForward = 1, kModeOuter = 2, kModeGateReverse = 3,
  // the Static pass split at the per-atom boundary into three kernels: the edge->moment forward
  // (moments to a.mom), the per-atom graph (atom_graph_kernel: readout, adjoint moments to
  // a.amom) and the per-edge adjoint (from a.amom)
  kModeStaticFwd = 4, kModeStaticRev = 5,
  // the Effect outer pass compiled with the neighbours' gate-signal rows h_j brought into shared
  // memory by 1-D bulk async copies, one 32-edge batch ahead (a kernel variant of kModeOuter)
  kModeOuterBulk = 6,
  // the Effect outer pass split like the Static pass (forward with h_j, per-atom graph kernel,
  // adjoint writing the hbar contributions)
  kModeOuterFwd = 7, kModeOuterRev = 8,
  // the Effect gate passes split the same way: the gate forward pass's edge->moment part (the
  // per-atom gate graph and gate-signal projection then run in atom_graph_kernel), and the gate
  // reverse pass's per-edge adjoint (after atom_graph_kernel gathered the gate-signal adjoint and
  // ran the gate graph's reverse)
  kModeGateFwdEdges = 9, kModeGateRevEdges = 10
};

template <typename Real>
struct PassArgs {
  DevModel<Real> dm;
  int natoms;
  const int* types;
  const int* row;          // [natoms] first edge of each centre
  const int* row_end;      // [natoms] one past its last edge (row + 1 for CSR layouts)
  const int* nbr;          // [E]
  const int* rev;          // [E] reverse edge
  const typename Vec4<Real>::type* d4;  // [E] (dx, dy, dz, r)
  Real* g;                 // [E][3] dE/dd per edge (written by static/outer, accumulated by gate reverse)
  Real* hsig;              // [natoms][F] gate signal h (written by gate forward)
  Real* hcontrib;          // [E][F] per-edge hbar contributions, stored at the reverse edge
  Real* gmom;              // [natoms][M] gate moment values (gate forward -> gate reverse)
  const double* hbar_atom; // [natoms][F] gate-signal adjoint already summed per atom (caller edges), or null
  double* site_energy;     // [natoms]
  double* virial;          // [natoms][6] (xx, yy, zz, xy, xz, yz), minus d (x) g
  double* desc;            // [natoms][S] scalar moments (descriptors), or null
  Real* mom;               // [natoms][K H] moments (split Static pass: forward -> graph kernel)
  Real* amom;              // [natoms][K H] their adjoints (graph kernel -> per-edge adjoint)
  int* error;
  int moment_mma;          // FP32 engines: 1 = edge->moment batch sums on the tensor cores (3xTF32 mma.sync)
  int atom_order;          // 0: warps take centres grid-strided; 1: each warp a contiguous run of
                           // centres; 2: warps take the next centre from a device counter as they
                           // finish -- dynamic balance for uneven centres
  int* work;               // atom_order 2: {next centre, warps done}, zero at launch; the last warp
                           // to finish zeroes both for the next launch
  int h_bulk;              // Effect outer pass: neighbours' h_j rows staged by bulk async copies (pass_h_bulk)
  int grid_mode;           // 0: all resident blocks; 1: the fewest blocks that keep the same atoms per warp
  int block_warps;         // launch shape: warps per block (1 .. kPassWarps; 0 = kPassWarps); the kernel
                           // reads its block size from blockDim
};

template <typename Real>
__host__ __device__ inline int pass_table_size(int C, int F, int B, int nblk) {
  return F * B + 2 * nblk * C * C + 3 * C * F;
}
__host__ __device__ constexpr int round4(int n) { return (n + 3) & ~3; }
// Staged edge row of the forward reduction: u_mu at [0, F), Y_h at [stage_yoff, + H), padded so
// that rows start on 16-byte boundaries and the row stride in 16-byte units is odd (128-bit row
// stores of a warp then hit distinct bank groups).
__host__ __device__ constexpr int stage_yoff(int F) { return round4(F); }
__host__ __device__ constexpr int stage_stride(int F, int H) {
  return ((round4(stage_yoff(F) + H) / 4) % 2) ? round4(stage_yoff(F) + H) : round4(stage_yoff(F) + H) + 4;
}
// E/F/virial pass tables: radial coefficients [F][B], warp (slope, shift) [2 nblk][C^2], and per
// species pair (t_i, t_j) the products x0(t_i) x1(t_j) and x0(t_i) wadd(t_j) [C^2][F] each.
__host__ __device__ inline int efs_table_size(int C, int F, int B, int nblk) {
  return round4(F * B + 2 * nblk * C * C + 2 * C * C * F);
}
// Per-warp scratch: the staged edge rows, the node values v [M + 1] (v[M] = 1, the graph
// program's constant node), the node adjoints [M + 1] (in the staging rows when they fit: those
// are free once the forward reduction is done), abar [K][H], hbar [F] and the graph program's
// partial slots [parts].
__host__ __device__ constexpr bool adj_in_stage(int F, int H, int M) { return M + 1 <= kWarp * stage_stride(F, H); }
template <typename Real>
__host__ __device__ inline int pass_warp_size(int F, int H, int M, int K, int parts) {
  return round4(kWarp * stage_stride(F, H) + (M + 1) + (adj_in_stage(F, H, M) ? 0 : M + 1) + K * H + F + parts + 4);
}
// Whether the Effect outer pass can stage the neighbours' gate-signal rows h_j with bulk async
// copies: a row must be a whole number of 16-byte units (the copy's size and alignment rule).
// The host launches the kModeOuterBulk variant only then, and sizes its scratch by the same test.
template <typename Real>
__host__ __device__ constexpr bool h_rows_bulk_ok(int F) {
  return (F * static_cast<int>(sizeof(Real))) % 16 == 0;
}
template <typename Real>
__host__ __device__ inline bool pass_h_bulk(int mode, int flag, int F) {
  return (mode == kModeOuter || mode == kModeOuterBulk) && flag != 0 && h_rows_bulk_ok<Real>(F);
}
// Per-warp scratch with the h_j staging area appended: 32 rows of F (one per lane, 16-byte
// aligned) and the warp's mbarrier (4 values, 16 bytes or more).
template <typename Real>
__host__ __device__ inline int pass_warp_stride(int F, int H, int M, int K, int parts, bool h_bulk) {
  return pass_warp_size<Real>(F, H, M, K, parts) + (h_bulk ? kWarp * F + 4 : 0);
}

// Kahan-compensated accumulation for the FP32 bulk form (explicitly rounded steps, never fused
// with the caller's multiplies); plain sums in FP64.
template <typename Real, bool KAHAN>
__device__ __forceinline__ void kadd(Real& s, Real& c, Real x) {
  if constexpr (KAHAN && sizeof(Real) == 4) {
    const float y = __fsub_rn(x, c);
    const float t = __fadd_rn(s, y);
    c = __fsub_rn(__fsub_rn(t, s), y);
    s = t;
  } else if constexpr (KAHAN) {
    const Real y = x - c;
    const Real t = s + y;
    c = (t - s) - y;
    s = t;
  } else {
    s += x;
  }
}

// ---------------------------------------------------------------------------------------------
// Per-edge radial functions of one pass: R_mu and (optionally) dR_mu/dr for all (k, l).
// The warp (slope, shift) depends on (scaling block, t_i, t_j); the Chebyshev part is shared by
// every l of a block and only the envelope differs between l = 0 and l > 0 with two cutoffs.
// ---------------------------------------------------------------------------------------------
// One row of radial coefficients (16-byte aligned when BF > 0: rows of BF = 8 values from an
// aligned table) into registers, with 128-bit loads where the size allows.
template <typename Real, int BF, int NBM>
__device__ __forceinline__ void load_coeff_row(const Real* c, int B, Real (&cc)[NBM]) {
  if constexpr (BF > 0 && sizeof(Real) == 4 && BF % 4 == 0) {
    const float4* c4 = reinterpret_cast<const float4*>(c);
#pragma unroll
    for (int q = 0; q < BF / 4; ++q) {
      const float4 v = c4[q];
      cc[4 * q] = v.x; cc[4 * q + 1] = v.y; cc[4 * q + 2] = v.z; cc[4 * q + 3] = v.w;
    }
  } else if constexpr (BF > 0 && sizeof(Real) == 8 && BF % 2 == 0) {
    const double2* c2 = reinterpret_cast<const double2*>(c);
#pragma unroll
    for (int q = 0; q < BF / 2; ++q) {
      const double2 v = c2[q];
      cc[2 * q] = v.x; cc[2 * q + 1] = v.y;
    }
  } else {
#pragma unroll
    for (int b = 0; b < NBM; ++b) cc[b] = b < B ? c[b] : Real(0);
  }
}

// One edge's inputs: the record (d, r), the neighbour and its species.
template <typename Real>
struct EdgeIn {
  typename Vec4<Real>::type d;
  int j, tj;
};
// (species indices are clamped to [0, C): an index out of range, which the edge build or the
// caller-edge checks report, must not reach the per-species tables within the same step)
__device__ __forceinline__ int species_of(const int* types, int i, int C) { return min(max(types[i], 0), C - 1); }

template <typename Real>
__device__ __forceinline__ EdgeIn<Real> load_edge(const typename Vec4<Real>::type* d4, const int* nbr,
                                                  const int* types, int e, int C) {
  EdgeIn<Real> x;
  x.d = d4[e];
  x.j = nbr[e];
  // one species: no neighbour-type load (it would wait on the neighbour index just loaded)
  x.tj = C == 1 ? 0 : species_of(types, x.j, C);
  return x;
}

// n values between a global row and a shared-memory row, 128-bit accesses when n is a multiple
// of 16 bytes' worth (both rows are then 16-byte aligned: row starts are multiples of n values).
template <typename Real>
__device__ __forceinline__ void copy_row(Real* dst, const Real* src, int n) {
  constexpr int V = 16 / sizeof(Real);
  if (n % V == 0) {
    using W = typename std::conditional<sizeof(Real) == 4, float4, double2>::type;
    for (int q = 0; q < n / V; ++q) reinterpret_cast<W*>(dst)[q] = reinterpret_cast<const W*>(src)[q];
  } else {
    for (int q = 0; q < n; ++q) dst[q] = src[q];
  }
}

// N (a multiple of 4) values to a 16-byte aligned shared-memory row, 128-bit stores for FP32.
template <typename Real, int N>
__device__ __forceinline__ void store_row(Real* dst, const Real (&x)[N]) {
  static_assert(N % 4 == 0, "row length");
  if constexpr (sizeof(Real) == 4) {
#pragma unroll
    for (int q = 0; q < N / 4; ++q)
      reinterpret_cast<float4*>(dst)[q] = make_float4(x[4 * q], x[4 * q + 1], x[4 * q + 2], x[4 * q + 3]);
  } else {
#pragma unroll
    for (int q = 0; q < N / 2; ++q) reinterpret_cast<double2*>(dst)[q] = make_double2(x[2 * q], x[2 * q + 1]);
  }
}

// BF > 0: the basis size is the compile-time constant BF (= dm.B); BF = 0: runtime B <= kMaxB.
template <int L, typename Real, bool DERIV, int BF = 0, typename Body>
__device__ __forceinline__ void radial_loop(const DevModel<Real>& dm, const Real* s_coeff, const Real* s_scal,
                                            int pair, Real r, Body&& body) {
  constexpr int Lp = L + 1;
  constexpr int NBM = BF ? BF : kMaxB;
  const int B = BF ? BF : dm.B, C2 = dm.C * dm.C;
  Real f0, fd0, f1, fd1;
  envelope<Real>(r, dm.rmax, dm.poly, dm.cutoff_p, f0, fd0);
  if (dm.split) envelope<Real>(r, dm.rang, dm.poly, dm.cutoff_p, f1, fd1);
  else { f1 = f0; fd1 = fd0; }
  f0 *= dm.scaling; fd0 *= dm.scaling; f1 *= dm.scaling; fd1 *= dm.scaling;
  const bool angular_on = !(r >= dm.rang);
  for (int k = 0; k < dm.K; ++k) {
    Real Tv[NBM], Td[NBM];
    int sb_prev = -1;
#pragma unroll
    for (int l = 0; l < Lp; ++l) {
      if (l > 0 && !angular_on) break;
      const int sb = scaling_block(dm.scaling_mode, k, l, Lp);
      if (sb != sb_prev) {
        const Real slope = s_scal[2 * sb * C2 + pair], shift = s_scal[(2 * sb + 1) * C2 + pair];
        if (DERIV) cheb_raw<Real, NBM>(r, slope, shift, B, Tv, Td);
        else cheb_raw_values<Real, NBM>(r, slope, shift, B, Tv);
        sb_prev = sb;
      }
      const int mu = k * Lp + l;
      const Real* c = s_coeff + mu * B;
      Real cc[NBM];
      load_coeff_row<Real, BF, NBM>(c, B, cc);
      // two interleaved partial sums per dot product (shorter dependency chains)
      Real a0 = Real(0), a1 = Real(0), d0 = Real(0), d1 = Real(0);
#pragma unroll
      for (int b = 0; b < NBM; ++b) {
        if (b < B) {
          if (b & 1) { a1 += cc[b] * Tv[b]; if (DERIV) d1 += cc[b] * Td[b]; }
          else { a0 += cc[b] * Tv[b]; if (DERIV) d0 += cc[b] * Td[b]; }
        }
      }
      const Real a = a0 + a1, ad = d0 + d1;
      const Real f = l == 0 ? f0 : f1, fd = l == 0 ? fd0 : fd1;
      const Real R = f * a;
      const Real Rd = DERIV ? (fd * a + f * ad) : Real(0);
      body(k, l, mu, R, Rd);
    }
  }
}

// Steps [s0, s1) of a pass's graph program (GraphProg, device_common.cuh) on the warp's node
// arrays: forward steps add into v, reverse steps into adj (DIR 1 / 2: the range holds forward /
// reverse steps only).  Each lane runs its term stream (one
// coalesced row per term), adding chunk sums to their target node or partial slot at the chunk's
// last term; then the lanes combine the partial slots of lists that were cut into several chunks.
template <typename Real, int DIR = 0>
__device__ __forceinline__ void run_prog(const GraphProg<Real>& g, int s0, int s1, Real* v, Real* adj, Real* parts,
                                         int lane) {
  for (int st = s0; st < s1; ++st) {
    const int4 info = g.steps[st];
    const bool rev = DIR == 2 || (DIR == 0 && (info.w & 1));
    Real* T = rev ? adj : v;
    const Real* X = rev ? adj : v;
    const ProgRec<Real>* r = g.rows + static_cast<size_t>(info.x) * kWarp + lane;
    Real acc = Real(0);
#pragma unroll 4
    for (int i = 0; i < info.y; ++i) {
      const ProgRec<Real> p = load_rec<Real>(r + static_cast<size_t>(i) * kWarp);
      acc += p.c * X[p.ab & 0xffffu] * v[p.ab >> 16];
      if (p.flush != kProgNoFlush) {
        if (p.flush >= 0) T[p.flush] += acc;
        else parts[-p.flush - 2] = acc;
        acc = Real(0);
      }
    }
    const int comb_end = info.w >> 1;
    if (comb_end > info.z) {
      __syncwarp();
      for (int q = info.z + lane; q < comb_end; q += kWarp) {
        const int4 e = g.comb[q];
        Real s = Real(0);
        for (int p = e.y; p < e.z; ++p) s += parts[p];
        T[e.x] += s;
      }
    }
    __syncwarp();
  }
}

// ---------------------------------------------------------------------------------------------
// Edge->moment batch sums on the tensor cores (FP32 engines, optional): the batch's staged rows
// form the products D[mu][lm] = sum_q u[q][mu] Y[q][lm] (q < 32 edges), computed as m16n8k8 TF32
// mma.sync tiles with each operand split into a TF32 head and a TF32 tail (3xTF32: head*head +
// head*tail + tail*head, about FP32 accuracy); the entries with l(mu) = l(lm) are the moment
// partials, written to part[k][lm].  Rows past the batch are zero; tile columns past F / H read
// other staged values and are discarded.
// ---------------------------------------------------------------------------------------------
__device__ __forceinline__ unsigned tf32_head(float x) {
  unsigned h;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(h) : "f"(x));
  return h;
}
__device__ __forceinline__ void mma_tf32(float (&d)[4], const unsigned (&a)[4], const unsigned (&b)[2]) {
  asm volatile("mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
               "{%0,%1,%2,%3};"
               : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
               : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}
template <int L>
__device__ __forceinline__ void moments_mma_batch(const float* stage, int sw, int yoff, int F, float* part, int lane) {
  constexpr int Lp = L + 1, H = Lp * Lp;
  const int g = lane >> 2, t = lane & 3;
  const int mtiles = (F + 15) / 16;
  constexpr int ntiles = (H + 7) / 8;
  for (int mt = 0; mt < mtiles; ++mt) {
#pragma unroll
    for (int nt = 0; nt < ntiles; ++nt) {
      float d[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
      for (int ks = 0; ks < kWarp / 8; ++ks) {
        const float* r0 = stage + (8 * ks + t) * sw;
        const float* r4 = r0 + 4 * sw;
        const float av[4] = {r0[16 * mt + g], r0[16 * mt + g + 8], r4[16 * mt + g], r4[16 * mt + g + 8]};
        const float bv[2] = {r0[yoff + 8 * nt + g], r4[yoff + 8 * nt + g]};
        unsigned ah[4], al[4], bh[2], bl[2];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          ah[i] = tf32_head(av[i]);
          al[i] = tf32_head(av[i] - __uint_as_float(ah[i]));
        }
#pragma unroll
        for (int i = 0; i < 2; ++i) {
          bh[i] = tf32_head(bv[i]);
          bl[i] = tf32_head(bv[i] - __uint_as_float(bh[i]));
        }
        mma_tf32(d, al, bh);
        mma_tf32(d, ah, bl);
        mma_tf32(d, ah, bh);
      }
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        const int mu = 16 * mt + g + 8 * (i >> 1), lm = 8 * nt + 2 * t + (i & 1);
        if (mu < F && lm < H) {
          int l = 0;
          while ((l + 1) * (l + 1) <= lm) ++l;
          if (mu % Lp == l) part[(mu / Lp) * H + lm] = d[i];
        }
      }
    }
  }
  __syncwarp();
}

// Readout of one centre and the adjoint seeds: E_i = species + shift + coef sum_q linear_q
// v[map q] into a.site_energy (the sum in compensated FP32 with exact products for the FP32 bulk
// form, FP64 otherwise), the scalar moments into a.desc when requested, adj zeroed and seeded with
// coef linear in Real (the reference's readout, sus2_sl_kernel.cpp:556).
template <typename Real>
__device__ __forceinline__ void readout_seeds(const PassArgs<Real>& a, int atom, int ti, const Real* v, Real* adj,
                                              int lane) {
  const DevModel<Real>& dm = a.dm;
  const int M = dm.M;
  const double coef = dm.species_readout ? 1.0 : dm.species[ti];
  const Real coef_r = Real(coef);
  const int off = dm.species_readout ? ti * dm.S : 0;
  for (int q = lane; q <= M; q += kWarp) adj[q] = Real(0);
  __syncwarp();
  double es64 = 0.0;
  float ehi = 0.f, elo = 0.f;
  for (int q = lane; q < dm.S; q += kWarp) {
    const int node = dm.scalar_map[q];
    const Real lin = dm.linear[off + q], vv = v[node];
    if (sizeof(Real) == 4) csum_add_prod(ehi, elo, float(lin), float(vv));
    else es64 += double(lin) * double(vv);
    adj[node] = coef_r * lin;
    if (a.desc) a.desc[static_cast<size_t>(atom) * dm.S + q] = double(vv);
  }
  const double es = sizeof(Real) == 4 ? warp_csum(ehi, elo) : warp_sum(es64);
  if (lane == 0) a.site_energy[atom] = dm.species[ti] + dm.shift[ti] + coef * es;
  __syncwarp();
}

// ---------------------------------------------------------------------------------------------
// The pass kernel.
// ---------------------------------------------------------------------------------------------
constexpr int kPassWarps = 4;
// Minimum resident blocks per SM (the register budget: 4 blocks = 128 registers, 3 = 168).  Both
// budgets are compiled for the B = 8 passes and the engine's autotuner times them on the caller's
// layout; without tuning: 4 for the FP32 kernels up to L = 3 and the L = 4 gate passes, 3
// otherwise (measured: the L = 4 outer pass spills and runs slower at 128 registers; the FP64
// kernels spill more).
__host__ __device__ constexpr int default_min_blocks(int L, bool fp32, int mode) {
  return (fp32 && (L <= 3 || (L == 4 && mode != kModeOuter && mode != kModeOuterBulk))) ? 4 : 3;
}

template <int L, typename Real, int MODE, bool KAHAN, int BF, int MINB>
__global__ void __launch_bounds__(kPassWarps * kWarp, MINB) atom_pass_kernel(PassArgs<Real> a) {
  constexpr int Lp = L + 1, H = Lp * Lp;
  constexpr int kMaxItems = (kMaxK * H + kWarp - 1) / kWarp;
  using V4 = typename Vec4<Real>::type;
  const DevModel<Real>& dm = a.dm;
  const bool gate_pass = MODE == kModeGateForward || MODE == kModeGateReverse || MODE == kModeGateFwdEdges ||
                         MODE == kModeGateRevEdges;
  // the gate reverse pass adds its edge gradients and virials to the outer pass's
  constexpr bool kGateRev = MODE == kModeGateReverse || MODE == kModeGateRevEdges;
  const PassTables<Real>& pt = gate_pass ? dm.gate : dm.outer;
  const int C = dm.C, F = dm.F, B = BF ? BF : dm.B, K = dm.K, M = dm.M, NB = dm.NB;
  const int warps = blockDim.x / kWarp, warp = threadIdx.x / kWarp, lane = warp_lane();
  // Effect outer pass, bulk variant: the neighbours' h_j rows of a 32-edge batch are brought into
  // hbuf by bulk async copies (one row per lane), issued while the batch before is still being
  // worked on (a constant false in every other variant)
  constexpr bool kBulk = MODE == kModeOuterBulk;
  const bool hb_on = kBulk && h_rows_bulk_ok<Real>(F);

  extern __shared__ __align__(16) unsigned char smem_raw[];
  Real* sm = reinterpret_cast<Real*>(smem_raw);
  Real* s_coeff = sm;
  Real* s_scal = s_coeff + F * B;
  Real* s_pw = s_scal + 2 * dm.nblk * C * C;        // [C^2][F] x0(t_i) x1(t_j)
  Real* s_pa = s_pw + C * C * F;                    // [C^2][F] x0(t_i) wadd(t_j)
  const int wsize = pass_warp_size<Real>(F, H, M, K, dm.prog_parts);
  Real* wbase = sm + efs_table_size(C, F, B, dm.nblk) + pass_warp_stride<Real>(F, H, M, K, dm.prog_parts, hb_on) * warp;
  const int sw = stage_stride(F, H), yoff = stage_yoff(F);
  Real* stage = wbase;                              // [32][sw]: u at [0, F), Y at [yoff, yoff + H)
  Real* v = stage + kWarp * sw;                     // [M + 1], v[M] = 1
  const bool adj_staged = adj_in_stage(F, H, M);
  Real* adj = adj_staged ? stage : v + M + 1;       // [M + 1]
  Real* abar = v + (M + 1) + (adj_staged ? 0 : M + 1);  // [K][H]
  Real* hbar = abar + K * H;                        // [F]
  Real* parts = hbar + F;                           // [prog_parts]
  Real* hbuf = wbase + wsize;                       // [32][F] h_j rows of one batch (hb_on)
  unsigned long long* hb_bar = reinterpret_cast<unsigned long long*>(hbuf + kWarp * F);

  // the next kernel may be scheduled as soon as every block has started; the model tables staged
  // here are written only by host uploads, which completed before the launch chain began, so
  // they are read before the wait for the previous kernel's edges and signals
  pdl_launch_dependents();
  for (int q = threadIdx.x; q < F * B; q += blockDim.x) s_coeff[q] = pt.coeff[q];
  for (int q = threadIdx.x; q < 2 * dm.nblk * C * C; q += blockDim.x) s_scal[q] = pt.scal[q];
  for (int q = threadIdx.x; q < C * C * F; q += blockDim.x) {
    const int pair = q / F, mu = q - pair * F, ti = pair / C, tj = pair - ti * C;
    const Real x0 = pt.wcenter[ti * F + mu];
    s_pw[q] = x0 * pt.wsource[tj * F + mu];
    s_pa[q] = pt.wadd ? x0 * pt.wadd[tj * F + mu] : Real(0);
  }
  __syncthreads();
  pdl_wait();
  const bool effect_outer = MODE == kModeOuter || MODE == kModeOuterBulk || MODE == kModeOuterFwd || MODE == kModeOuterRev;
  // the two per-edge kernels of a split pass: forward only (moments out), adjoint only (moment
  // adjoints in)
  constexpr bool kFwdOnly = MODE == kModeStaticFwd || MODE == kModeOuterFwd || MODE == kModeGateFwdEdges;
  constexpr bool kRevOnly = MODE == kModeStaticRev || MODE == kModeOuterRev || MODE == kModeGateRevEdges;
  // the h_j copies of a batch: lane 0 orders the warp's reads of hbuf before the async writes and
  // announces the bytes, every lane with an edge copies its row; the caller has synchronised the
  // warp after its last reads of hbuf
  unsigned hb_parity = 0;
  if (hb_on) {
    if (lane == 0) mbar_init(hb_bar, 1);
    __syncwarp();
  }
  auto hb_issue = [&](bool has_edge, int j, int nedges) {
    if (lane == 0) {
      fence_proxy_async_smem();
      mbar_arrive_expect(hb_bar, static_cast<unsigned>(nedges * F * sizeof(Real)));
    }
    __syncwarp();
    if (has_edge) bulk_copy_g2s(hbuf + lane * F, a.hsig + (size_t)j * F, F * sizeof(Real), hb_bar);
  };
  // waits for the batch's rows; on a copy that does not complete (bounded wait) records the error,
  // waits once more for the copies in flight and returns false: the warp then leaves the kernel
  auto hb_arrived = [&]() {
    const bool ok = __all_sync(0xffffffffu, mbar_wait_bounded(hb_bar, hb_parity));
    if (!ok) {
      if (lane == 0) record_error(a.error, kErrAsyncCopy);
      mbar_wait_bounded(hb_bar, hb_parity);
    }
    hb_parity ^= 1u;
    return ok;
  };

  // Lane-owned moment items for the forward reduction: item t = lane + 32 s <-> (k, lm); the
  // first nit of the kMaxItems register slots are in use.
  const int nit = (K * H + kWarp - 1) / kWarp;
  int it_u[kMaxItems], it_y[kMaxItems];
#pragma unroll
  for (int s = 0; s < kMaxItems; ++s) {
    const int t = lane + kWarp * s;
    if (t < K * H) {
      const int kk = t / H, lm = t - kk * H;
      int l = 0;
      while ((l + 1) * (l + 1) <= lm) ++l;
      it_u[s] = kk * Lp + l;
      it_y[s] = yoff + lm;
    } else {
      it_u[s] = -1;
      it_y[s] = 0;
    }
  }

  // centres of this warp: grid-strided, one contiguous run (neighbouring centres share their
  // neighbours' rows in L1), or taken one at a time from a device counter
  const int gwarp = blockIdx.x * warps + warp, nwarps = gridDim.x * warps;
  const int per_warp = (a.natoms + nwarps - 1) / nwarps;
  const bool dynamic = a.atom_order == 2;
  auto grab = [&]() {
    int x = 0;
    if (lane == 0) x = atomicAdd(a.work, 1);
    return __shfl_sync(0xffffffffu, x, 0);
  };
  const int atom_first = dynamic ? grab() : (a.atom_order ? gwarp * per_warp : gwarp);
  const int atom_stop = a.atom_order == 1 ? min(a.natoms, atom_first + per_warp) : a.natoms;
  const int atom_step = a.atom_order == 1 ? 1 : nwarps;
  // the dynamic order's reset: every warp counts itself done after its last take (ordered after
  // it by the fence), and the last one zeroes the pair, when no take of this launch is pending
  auto finish_dynamic = [&]() {
    if (dynamic && lane == 0) {
      __threadfence();
      if (atomicAdd(a.work + 1, 1) == nwarps - 1) {
        atomicExch(a.work, 0);
        atomicExch(a.work + 1, 0);
      }
    }
  };
  for (int atom = atom_first; atom < atom_stop; atom = dynamic ? grab() : atom + atom_step) {
    const int ti = C == 1 ? 0 : species_of(a.types, atom, C);
    const int e0 = a.row[atom], e1 = a.row_end[atom];
    // per-atom virial: FP64 for the FP64 form; compensated FP32 (hi, lo) for the FP32 bulk form
    double vir[6] = {0, 0, 0, 0, 0, 0};
    float vhi[6] = {0, 0, 0, 0, 0, 0}, vlo[6] = {0, 0, 0, 0, 0, 0};

    // edge inputs of the lane's edge in the last batch: left by the forward loop, which the
    // per-edge adjoint then starts from (it runs the batches in reverse order)
    EdgeIn<Real> cur{};
    const int nbat = (e1 - e0 + kWarp - 1) / kWarp;
    // the gate reverse pass starts with the per-atom work: its first edge batch loads meanwhile
    if ((MODE == kModeGateReverse || kRevOnly) && nbat > 0 && e0 + (nbat - 1) * kWarp + lane < e1)
      cur = load_edge<Real>(a.d4, a.nbr, a.types, e0 + (nbat - 1) * kWarp + lane, C);
    if (kRevOnly) {
      // ---------------- split pass, per-edge part: adjoint moments from the graph kernel ----------
      for (int t = lane; t < K * H; t += kWarp) abar[t] = a.amom[static_cast<size_t>(atom) * (K * H) + t];
      __syncwarp();
    } else if (MODE != kModeGateReverse) {
      // ---------------- forward moments ----------------
      Real acc[kMaxItems], cmp[kMaxItems];
#pragma unroll
      for (int s = 0; s < kMaxItems; ++s) { acc[s] = Real(0); cmp[s] = Real(0); }
      // the next batch's edge inputs are loaded while the current batch is evaluated
      if (e0 + lane < e1) cur = load_edge<Real>(a.d4, a.nbr, a.types, e0 + lane, C);
      if (hb_on && nbat > 0) hb_issue(e0 + lane < e1, cur.j, min(kWarp, e1 - e0));
      for (int base = e0; base < e1; base += kWarp) {
        const int e = base + lane;
        const bool more = base + kWarp < e1;
        EdgeIn<Real> nxt = cur;
        if (more && e + kWarp < e1) nxt = load_edge<Real>(a.d4, a.nbr, a.types, e + kWarp, C);
        if (hb_on && !hb_arrived()) return;
        Real* row = stage + lane * sw;
        if (e < e1) {
          const V4 dv = cur.d;
          const int j = cur.j;
          const int tj = cur.tj;
          const Real r = dv.w, ir = Real(1) / r;
          Real Y[round4(H)];
          sph_values<L, Real>(dv.x * ir, dv.y * ir, dv.z * ir, Y);
          const bool ang = !(r >= dm.rang);
#pragma unroll
          for (int h = 0; h < round4(H); ++h) Y[h] = (h < H && (h == 0 || ang)) ? Y[h] : Real(0);
          store_row<Real, round4(H)>(row + yoff, Y);
          const int pair = ti * C + tj;
          const Real* pw = s_pw + pair * F;
          const Real* pa = s_pa + pair * F;
          // Effect: the neighbour's gate signal h_j, from the bulk-copied batch rows or staged in
          // the row's u slots (each read once before its u_mu overwrites it)
          const Real* hj = hb_on ? hbuf + lane * F : row;
          if (effect_outer && !hb_on) copy_row<Real>(row, a.hsig + (size_t)j * F, F);
          else if (!effect_outer) for (int mu = 0; mu < F; ++mu) row[mu] = Real(0);
          radial_loop<L, Real, false, BF>(dm, s_coeff, s_scal, pair, r, [&](int k, int l, int mu, Real R, Real) {
            Real w = pw[mu];
            if (effect_outer) w += pa[mu] * hj[mu];
            row[mu] = w * R;
          });
          if (effect_outer && !ang)
            for (int mu = 0; mu < F; ++mu)
              if (mu % Lp != 0) row[mu] = Real(0);
        } else {
          for (int q = 0; q < sw; ++q) row[q] = Real(0);
        }
        __syncwarp();
        // the next batch's h_j rows travel while this batch is reduced
        if (hb_on && more) hb_issue(e + kWarp < e1, nxt.j, min(kWarp, e1 - base - kWarp));
        // plain sum over the batch's (<= 32) staged edges, then a compensated add of the batch
        // partial into the atom's running moment
        const int nb = min(kWarp, e1 - base);
        Real part[kMaxItems];
#pragma unroll
        for (int s = 0; s < kMaxItems; ++s) part[s] = Real(0);
        if (sizeof(Real) == 4 && a.moment_mma) {
          // tensor-core batch sums into the abar rows (free until the reverse), then each lane
          // reads its items
          moments_mma_batch<L>(reinterpret_cast<const float*>(stage), sw, yoff, F, reinterpret_cast<float*>(abar), lane);
#pragma unroll
          for (int s = 0; s < kMaxItems; ++s) {
            if (s >= nit) break;
            if (it_u[s] >= 0) part[s] = abar[lane + kWarp * s];
          }
        } else {
          for (int q = 0; q < nb; ++q) {
            const Real* sr = stage + q * sw;
#pragma unroll
            for (int s = 0; s < kMaxItems; ++s) {
              if (s >= nit) break;  // warp-uniform: only the model's K H items are issued
              if (it_u[s] >= 0) part[s] += sr[it_u[s]] * sr[it_y[s]];
            }
          }
        }
#pragma unroll
        for (int s = 0; s < kMaxItems; ++s) {
          if (s >= nit) break;
          kadd<Real, KAHAN>(acc[s], cmp[s], part[s]);
        }
        __syncwarp();
        if (more) cur = nxt;
      }
      if (kFwdOnly) {
        // split pass, forward part: the moments go to the graph kernel
#pragma unroll
        for (int s = 0; s < kMaxItems; ++s) {
          if (s >= nit) break;
          const int t = lane + kWarp * s;
          if (t < K * H) a.mom[static_cast<size_t>(atom) * (K * H) + t] = acc[s];
        }
        continue;
      }
      for (int q = lane; q <= M; q += kWarp) v[q] = q < M ? Real(0) : Real(1);
      __syncwarp();
#pragma unroll
      for (int s = 0; s < kMaxItems; ++s) {
        const int t = lane + kWarp * s;
        if (t < K * H) {
          const int b = dm.basic_of[t];
          if (b >= 0) v[b] = acc[s];
        }
      }
      __syncwarp();
      run_prog<Real, 1>(pt.prog, 0, pt.prog.nfwd, v, adj, parts, lane);

      if (MODE == kModeGateForward) {
        for (int q = lane; q < M; q += kWarp) a.gmom[(size_t)atom * M + q] = v[q];
        // the gate scalars gathered once into the (here unused) hbar row when they fit, so that
        // each signal's sum reads its weights and the scalars without a node-index load between
        const bool staged = dm.Q <= F;
        if (staged)
          for (int q = lane; q < dm.Q; q += kWarp) hbar[q] = v[dm.gate_nodes[q]];
        __syncwarp();
        for (int mu = lane; mu < F; mu += kWarp) {
          Real h = Real(0);
          for (int q = 0; q < dm.Q; ++q)
            h += dm.gate_wmat[mu * dm.Q + q] * (staged ? hbar[q] : v[dm.gate_nodes[q]]);
          a.hsig[(size_t)atom * F + mu] = h;
        }
        __syncwarp();
        continue;
      }

      // ---------------- readout and seeds ----------------
      readout_seeds<Real>(a, atom, ti, v, adj, lane);
    } else {
      // ---------------- gate reverse: gather hbar, project, load gate values ----------------
      if (!a.hbar_atom && F <= 2 * kWarp) {
        column_sums_2<Real>(a.hcontrib + (size_t)e0 * F, F, e1 - e0, hbar, lane);
      } else {
        for (int mu = lane; mu < F; mu += kWarp) {
          if (a.hbar_atom) {
            hbar[mu] = Real(a.hbar_atom[(size_t)atom * F + mu]);
          } else {
            hbar[mu] = column_sum<Real>(a.hcontrib + (size_t)e0 * F + mu, F, e1 - e0);
          }
        }
      }
      for (int q = lane; q <= M; q += kWarp) {
        v[q] = q < M ? a.gmom[(size_t)atom * M + q] : Real(1);
        adj[q] = Real(0);
      }
      __syncwarp();
      for (int q = lane; q < dm.Q; q += kWarp) {
        Real s = Real(0);
        for (int mu = 0; mu < F; ++mu) s += hbar[mu] * dm.gate_wmat[mu * dm.Q + q];
        adj[dm.gate_nodes[q]] += s;
      }
      __syncwarp();
    }

    // ---------------- reverse graph and contraction ----------------
    if (!kRevOnly) {
      run_prog<Real, 2>(pt.prog, pt.prog.nfwd, pt.prog.nsteps, v, adj, parts, lane);
      for (int t = lane; t < K * H; t += kWarp) {
        const int b = dm.basic_of[t];
        abar[t] = b >= 0 ? adj[b] : Real(0);
      }
      __syncwarp();
    }

    // ---------------- per-edge adjoint ----------------
    // batches in reverse order, the next one's edge inputs loaded while the current one runs
    // (with bulk-copied h_j rows the last forward batch's rows are still in hbuf: the first
    // adjoint batch uses them, and each batch's copies for the one after are issued mid-batch)
    for (int bt = nbat - 1; bt >= 0; --bt) {
      const int e = e0 + bt * kWarp + lane;
      const bool valid = e < e1;
      EdgeIn<Real> nxt = cur;
      if (bt > 0) nxt = load_edge<Real>(a.d4, a.nbr, a.types, e - kWarp, C);
      if (hb_on && bt < nbat - 1 && !hb_arrived()) return;
      if (!hb_on && !valid) { cur = nxt; continue; }
      const V4 dv = cur.d;
      const int j = cur.j;
      const int tj = cur.tj;
      cur = nxt;
      Real r = Real(1), ir = Real(1), ux = Real(0), uy = Real(0), uz = Real(0), s = Real(0);
      bool ang = false;
      // P[h] = sum_k w R_kl(h) abar[k][h] feeds the angular gradient; the radial-derivative term
      // sum_h Qd[h] Y[h], Qd[h] = sum_k w R'_kl(h) abar[k][h], is summed per (k, l) as
      // w R'_kl S_kl with S_kl = sum_{h in l} abar[k][h] Y[h] (no per-h Qd registers)
      Real P[H];
      // Effect: the hbar contributions are written to the lane's row (free after the forward
      // reduction) and go out as one row; h_j comes from the bulk-copied batch rows, or is staged
      // in that row first (each read before its contribution overwrites it)
      Real* hrow = stage + lane * sw;
      if (valid) {
        r = dv.w;
        ir = Real(1) / r;
        ux = dv.x * ir; uy = dv.y * ir; uz = dv.z * ir;
        ang = !(r >= dm.rang);
        Real Y[H];
        sph_values<L, Real>(ux, uy, uz, Y);
#pragma unroll
        for (int h = 0; h < H; ++h) { P[h] = Real(0); if (h > 0 && !ang) Y[h] = Real(0); }
        const Real* hj = hb_on ? hbuf + lane * F : hrow;
        if (effect_outer && !hb_on) copy_row<Real>(hrow, a.hsig + (size_t)j * F, F);
        const int pair = ti * C + tj;
        const Real* pw = s_pw + pair * F;
        const Real* pa = s_pa + pair * F;
        radial_loop<L, Real, true, BF>(dm, s_coeff, s_scal, pair, r, [&](int k, int l, int mu, Real R, Real Rd) {
          Real w = pw[mu], wa = Real(0);
          if (effect_outer) { wa = pa[mu]; w += wa * hj[mu]; }
          const Real wR = w * R;
          const Real* ab = abar + k * H;
          Real S = Real(0);
#pragma unroll
          for (int h = l * l; h < (l + 1) * (l + 1); ++h) {
            const Real av = ab[h];
            P[h] += wR * av;
            S += av * Y[h];
          }
          s += w * Rd * S;
          if (effect_outer) hrow[mu] = wa * R * S;
        });
      }
      // the next (earlier, full) batch's h_j rows travel while this one finishes
      if (hb_on && bt > 0) {
        __syncwarp();
        hb_issue(true, cur.j, kWarp);
      }
      if (!valid) continue;
      if (effect_outer) {
        if (!ang)
          for (int mu = 0; mu < F; ++mu)
            if (mu % Lp != 0) hrow[mu] = Real(0);
        copy_row<Real>(a.hcontrib + (size_t)a.rev[e] * F, hrow, F);
      }
      Real gx = Real(0), gy = Real(0), gz = Real(0);
      if (ang) sph_grad_dot<L, Real>(ux, uy, uz, P, gx, gy, gz);
      const Real ug = ux * gx + uy * gy + uz * gz;
      const Real Gx = ux * s + (gx - ux * ug) * ir;
      const Real Gy = uy * s + (gy - uy * ug) * ir;
      const Real Gz = uz * s + (gz - uz * ug) * ir;
      Real* ge = a.g + (size_t)e * 3;
      if (kGateRev) {
        ge[0] += Gx; ge[1] += Gy; ge[2] += Gz;
      } else {
        ge[0] = Gx; ge[1] = Gy; ge[2] = Gz;
      }
      if (sizeof(Real) == 4) {
        const float dx = float(dv.x), dy = float(dv.y), dz = float(dv.z);
        csum_add_prod(vhi[0], vlo[0], -dx, float(Gx)); csum_add_prod(vhi[1], vlo[1], -dy, float(Gy));
        csum_add_prod(vhi[2], vlo[2], -dz, float(Gz)); csum_add_prod(vhi[3], vlo[3], -dx, float(Gy));
        csum_add_prod(vhi[4], vlo[4], -dx, float(Gz)); csum_add_prod(vhi[5], vlo[5], -dy, float(Gz));
      } else {
        const double dx = dv.x, dy = dv.y, dz = dv.z;
        vir[0] -= dx * double(Gx); vir[1] -= dy * double(Gy); vir[2] -= dz * double(Gz);
        vir[3] -= dx * double(Gy); vir[4] -= dx * double(Gz); vir[5] -= dy * double(Gz);
      }
    }
    // per-atom virial: lane c < 6 writes component c (FP32 bulk: the compensated warp totals of
    // all six components in FP32, then one conversion to FP64 for the whole warp)
    double* vo = a.virial + (size_t)atom * 6;
    if (sizeof(Real) == 4) {
      float h = 0.f, l = 0.f;
#pragma unroll
      for (int c = 0; c < 6; ++c) {
        warp_csum_pair(vhi[c], vlo[c]);
        if (lane == c) { h = vhi[c]; l = vlo[c]; }
      }
      const double vc = double(h) + double(l);
      if (lane < 6) vo[lane] = kGateRev ? vo[lane] + vc : vc;
    } else {
#pragma unroll
      for (int c = 0; c < 6; ++c) vir[c] = warp_sum(vir[c]);
      if (lane == 0) {
        if (kGateRev)
          for (int c = 0; c < 6; ++c) vo[c] += vir[c];
        else
          for (int c = 0; c < 6; ++c) vo[c] = vir[c];
      }
    }
    __syncwarp();
  }
  finish_dynamic();
}

// ---------------------------------------------------------------------------------------------
// The per-atom part of a split pass, warp per centre: for the energy pass (Static or Effect
// outer), moments a.mom -> the graph program forward -> readout (site energy, descriptors) -> the
// program's reverse -> adjoint moments a.amom; for the Effect gate passes, the gate graph forward
// with the gate-signal projection, or the gate-signal adjoint gather and the gate graph reverse.
// Independent of L; several warps of centres in flight per SM hide the program's load latency
// that the fused pass serialises between its edge phases.
// ---------------------------------------------------------------------------------------------
constexpr int kGraphWarps = 4;
__host__ __device__ inline int graph_warp_size(int M, int parts, int F, int Q) {
  return round4(2 * (M + 1) + parts + (F > Q ? F : Q) + 4);
}

// GM: 0 the energy pass (Static or Effect outer tables: readout, adjoint moments to a.amom);
// 1 the gate forward pass (gate tables: gate values to a.gmom, gate signals to a.hsig);
// 2 the gate reverse pass (the gate-signal adjoint gathered per atom, projected onto the gate
// nodes, the gate graph's reverse, adjoint moments to a.amom).

template <typename Real, int GM>
__global__ void __launch_bounds__(kGraphWarps * kWarp) atom_graph_kernel(PassArgs<Real> a) {
  const DevModel<Real>& dm = a.dm;
  const PassTables<Real>& pt = GM == 0 ? dm.outer : dm.gate;
  const int M = dm.M, KH = dm.K * dm.H, C = dm.C, F = dm.F;
  const int warps = blockDim.x / kWarp, warp = threadIdx.x / kWarp, lane = warp_lane();
  extern __shared__ __align__(16) unsigned char smem_raw[];
  Real* v = reinterpret_cast<Real*>(smem_raw) + graph_warp_size(M, dm.prog_parts, F, dm.Q) * warp;
  Real* adj = v + M + 1;
  Real* parts = adj + M + 1;
  Real* hbar = parts + dm.prog_parts;  // [F] (GM 2) or the gate scalars [Q] (GM 1)
  pdl_launch_dependents();
  pdl_wait();
  for (int atom = blockIdx.x * warps + warp; atom < a.natoms; atom += gridDim.x * warps) {
    const int ti = C == 1 ? 0 : species_of(a.types, atom, C);
    if constexpr (GM == 2) {
      // the gate-signal adjoint of the atom: summed over its edges' contributions (stored at the
      // reverse edges by the outer pass), or already summed per atom (caller edges)
      const int e0 = a.row[atom], e1 = a.row_end[atom];
      if (!a.hbar_atom && F <= 2 * kWarp) {
        // both of a lane's columns side by side: the gather is the latency this kernel waits on
        column_sums_2<Real>(a.hcontrib + (size_t)e0 * F, F, e1 - e0, hbar, lane);
      } else {
        for (int mu = lane; mu < F; mu += kWarp)
          hbar[mu] = a.hbar_atom ? Real(a.hbar_atom[(size_t)atom * F + mu])
                                 : column_sum<Real>(a.hcontrib + (size_t)e0 * F + mu, F, e1 - e0);
      }
      for (int q = lane; q <= M; q += kWarp) {
        v[q] = q < M ? a.gmom[(size_t)atom * M + q] : Real(1);
        adj[q] = Real(0);
      }
      __syncwarp();
      for (int q = lane; q < dm.Q; q += kWarp) {
        Real s = Real(0);
        for (int mu = 0; mu < F; ++mu) s += hbar[mu] * dm.gate_wmat[mu * dm.Q + q];
        adj[dm.gate_nodes[q]] += s;
      }
      __syncwarp();
    } else {
      for (int q = lane; q <= M; q += kWarp) v[q] = q < M ? Real(0) : Real(1);
      __syncwarp();
      for (int t = lane; t < KH; t += kWarp) {
        const int b = dm.basic_of[t];
        if (b >= 0) v[b] = a.mom[static_cast<size_t>(atom) * KH + t];
      }
      __syncwarp();
      run_prog<Real, 1>(pt.prog, 0, pt.prog.nfwd, v, adj, parts, lane);
    }
    if constexpr (GM == 1) {
      for (int q = lane; q < M; q += kWarp) a.gmom[(size_t)atom * M + q] = v[q];
      // the gate scalars gathered once, so that each signal's sum reads its weights and the
      // scalars without a node-index load in between
      Real* gs = hbar;
      for (int q = lane; q < dm.Q; q += kWarp) gs[q] = v[dm.gate_nodes[q]];
      __syncwarp();
      for (int mu = lane; mu < F; mu += kWarp) {
        Real h = Real(0);
        for (int q = 0; q < dm.Q; ++q) h += dm.gate_wmat[mu * dm.Q + q] * gs[q];
        a.hsig[(size_t)atom * F + mu] = h;
      }
      __syncwarp();
      continue;
    }
    if constexpr (GM == 0) readout_seeds<Real>(a, atom, ti, v, adj, lane);
    run_prog<Real, 2>(pt.prog, pt.prog.nfwd, pt.prog.nsteps, v, adj, parts, lane);
    for (int t = lane; t < KH; t += kWarp) {
      const int b = dm.basic_of[t];
      a.amom[static_cast<size_t>(atom) * KH + t] = b >= 0 ? adj[b] : Real(0);
    }
    __syncwarp();
  }
}

}  // namespace sus2g
