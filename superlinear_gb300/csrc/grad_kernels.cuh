// Parameter gradient of the SUS2-SH energy model on the GPU (the trainer's
// AccumulateEFSCombinationGrad contract, src/basic_mlip.cpp:421-476, dev_src/mtpr.cpp:9188):
//
//   J(theta) = sum_i eW_i E_i + sum_e w_e . dE/dd_e,     w_e = fW_i - fW_j + S_frame d_e
//
// i.e. the energy weights plus the force / stress weights pulled back to edge vectors.  The
// second term is the directional derivative of the total energy when every edge vector moves
// along w_e, so J is evaluated with forward tangents (dual numbers) through the whole model and
// the parameter gradient follows from one reverse sweep over values and tangents:
//
//   forward   A = sum_e u Y,  Adot = sum_e (udot Y + u Ydot),  u = x0 x3 R,
//             udot = x0 (x3dot R + x3 R' rdot),  rdot = u_e . w_e,  Ydot = grad Y . w_e
//   graph     v[out] += c v_a v_b,  vdot[out] += c (vdot_a v_b + v_a vdot_b)
//   readout   J_i = eW_i E_i + Edot_i  ->  lambda = dJ/dv, mu = dJ/dvdot seeds
//   reverse   lambda_a += c (lambda_out v_b + mu_out vdot_b),  mu_a += c mu_out v_b  (and b)
//   edges     per (k, l): S = sum_m lambda Y, T = sum_m mu Y, U = sum_m mu Ydot,
//             dJ/dR = x0 (x3 (S + U) + x3dot T),  dJ/dR' = x0 x3 rdot T, then the Chebyshev
//             coefficients, the warp (slope, shift) through dxi/ds, dxi/dsigma, and the species /
//             gate factors.
// The Effect gate chain runs the same steps for the gate pass, seeded with
// dJ/dh_j and dJ/dhdot_j gathered per atom (stored at the reverse edge, like the force path).
//
// Reductions are deterministic.  Per-edge contributions to the per-(k, l) parameters (Chebyshev
// coefficients, species factors, warp slope / shift, gate additive factors) go to lane-private
// shared-memory columns (stride 33: conflict-free for a fixed column across lanes and for a fixed
// lane across columns); after each 32-edge batch and radial index k the warp sums every column over
// its 32 lanes in a fixed order (one column per lane) and adds the result to its private FP64
// gradient slice.  Slices are summed in a fixed order by k_slot_reduce.  When the columns do not
// fit in shared memory (many species), the contributions are summed with shuffle trees instead.
#pragma once
#include "efs_kernels.cuh"

namespace sus2g {

enum GradMode : int { kGradOuter = 0, kGradGateForward = 1, kGradGateReverse = 2 };

template <typename Real>
struct GradArgs {
  DevModel<Real> dm;
  int natoms;
  const int* types;
  const int* row;
  const int* row_end;      // one past each centre's last edge (row + 1 for CSR layouts)
  const int* nbr;
  const int* rev;
  const typename Vec4<Real>::type* d4;
  const int* frame_of;
  const double* ew;        // [N] energy weights
  const double* fw;        // [N][3] force weights
  const double* sw;        // [nframes][9] stress weights (row-major)
  Real* hsig;              // [N][F] gate signal h
  Real* hsigd;             // [N][F] tangent of h
  Real* gmom;              // [N][M] gate values
  Real* gmomd;             // [N][M] gate tangents
  Real* lhm;               // [E][2F] dJ/dh, dJ/dhdot contributions stored at the reverse edge
  double* lh_atom;         // [N][2F] gathered per atom (gate reverse)
  const double* extra_h;   // [N][F] additional dJ/dh per atom (objective terms of h), or null
  double* slots;           // [warps in grid][nparams]
  Real* abar;              // [N][2][K][H] adjoints of the moments (values, tangents): the per-atom part
                           // of a split pass writes them, its per-edge part reads them
  int* error;
  int acc_cols;            // lane-private accumulator columns per k (0: shuffle-tree reductions)
};

constexpr int kAccStride = kWarp + 1;

// Per-warp scratch: staged rows [32][2F + 2H + 1], node values and tangents v, vd [M] each, the
// node adjoints lam, mu [M] each (in the staged rows when they fit: those are dead once the forward
// reduction is done, and the per-edge loop recomputes its geometry), abar rows [2][K][H], hbar [2F].
// (v, vd, lam, mu hold M + 1 entries: node M is the graph program's constant 1, tangent 0; the
// program's partial slots take two values each)
__host__ __device__ constexpr bool grad_adj_in_stage(int F, int H, int M) { return 2 * (M + 1) <= kWarp * (2 * F + 2 * H + 1); }
template <typename Real>
__host__ __device__ inline int grad_warp_size(int F, int H, int M, int K, int parts) {
  return kWarp * (2 * F + 2 * H + 1) + 2 * (M + 1) + (grad_adj_in_stage(F, H, M) ? 0 : 2 * (M + 1)) + 2 * K * H +
         2 * F + 2 * parts + 4;
}

// Per-warp scratch of the per-edge part of a split pass: the atom's moment adjoints [2][K][H].
__host__ __device__ inline int grad_edge_warp_size(int K, int H) { return round4(2 * K * H); }

// The parts a pass can run as (GradLaunch::part): the whole pass in one kernel, or split at the
// per-atom boundary into the per-atom part (forward with tangents, readout seeds, reverse sweep;
// moment adjoints to GradArgs::abar) and the per-edge part (parameter contributions per edge from
// those adjoints) -- two smaller kernels whose bodies each fit the instruction cache.
enum GradPart : int { kGradWhole = 0, kGradAtomPart = 1, kGradEdgePart = 2 };

// Accumulator columns per radial index k: Chebyshev coefficients [l][b], species factors [t][l]
// (centre and neighbour factors index the same table), warp slope / shift [sb][t][2] (one warp
// block per k, or one per l for the L and LK maps), gate additive factors [t][l] (Effect outer).
__host__ __device__ inline int grad_acc_nsb(int scaling_mode, int Lp) {
  return (scaling_mode == 1 || scaling_mode == 3) ? Lp : 1;
}
__host__ __device__ inline int grad_acc_cols(int Lp, int B, int C, int scaling_mode, bool effect_outer) {
  return Lp * B + C * Lp + 2 * grad_acc_nsb(scaling_mode, Lp) * C + (effect_outer ? C * Lp : 0);
}

template <typename Real>
__device__ __forceinline__ void slot_add(double* slot, int idx, Real v, int lane) {
  const Real s = warp_sum(v);
  if (lane == 0) slot[idx] += double(s);
}

// Steps [s0, s1) of the pass's graph program (run_prog) on values and tangents (DIR 1: the range
// holds forward steps only, 2: reverse steps only, 0: either -- the kernel compiles only what it
// runs): forward steps
//   v[t] += c v[a] v[b],  vd[t] += c (vd[a] v[b] + v[a] vd[b]),
// reverse steps on the adjoints of values (lam) and tangents (mu):
//   lam[t] += c (lam[a] v[b] + mu[a] vd[b]),  mu[t] += c mu[a] v[b].
template <typename Real, int DIR>
__device__ __forceinline__ void run_prog_dual(const GraphProg<Real>& g, int s0, int s1, Real* v, Real* vd, Real* lam,
                                              Real* mu, Real* parts, int lane) {
  for (int st = s0; st < s1; ++st) {
    const int4 info = g.steps[st];
    const bool rev = DIR == 2 || (DIR == 0 && (info.w & 1));
    Real* T = rev ? lam : v;
    Real* Td = rev ? mu : vd;
    const ProgRec<Real>* r = g.rows + static_cast<size_t>(info.x) * kWarp + lane;
    Real acc = Real(0), accd = Real(0);
    auto flush = [&](int f) {
      if (f >= 0) { T[f] += acc; Td[f] += accd; }
      else { parts[2 * (-f - 2)] = acc; parts[2 * (-f - 2) + 1] = accd; }
      acc = Real(0);
      accd = Real(0);
    };
    if (!rev) {
#pragma unroll 2
      for (int i = 0; i < info.y; ++i) {
        const ProgRec<Real> p = load_rec<Real>(r + static_cast<size_t>(i) * kWarp);
        const int x = p.ab & 0xffffu, y = p.ab >> 16;
        const Real vx = v[x], vy = v[y];
        acc += p.c * vx * vy;
        accd += p.c * (vd[x] * vy + vx * vd[y]);
        if (p.flush != kProgNoFlush) flush(p.flush);
      }
    } else {
#pragma unroll 2
      for (int i = 0; i < info.y; ++i) {
        const ProgRec<Real> p = load_rec<Real>(r + static_cast<size_t>(i) * kWarp);
        const int x = p.ab & 0xffffu, y = p.ab >> 16;
        const Real vy = v[y], mx = mu[x];
        acc += p.c * (lam[x] * vy + mx * vd[y]);
        accd += p.c * mx * vy;
        if (p.flush != kProgNoFlush) flush(p.flush);
      }
    }
    const int comb_end = info.w >> 1;
    if (comb_end > info.z) {
      __syncwarp();
      for (int q = info.z + lane; q < comb_end; q += kWarp) {
        const int4 e = g.comb[q];
        Real s = Real(0), sd = Real(0);
        for (int p = e.y; p < e.z; ++p) { s += parts[2 * p]; sd += parts[2 * p + 1]; }
        T[e.x] += s;
        Td[e.x] += sd;
      }
    }
    __syncwarp();
  }
}

// Rank-weight gradients of the contraction (read before the contraction's reverse step changes
// the basic nodes' adjoints): the per-weight sum of a few products in the compute precision,
// added to the FP64 slice.
template <typename Real>
__device__ __forceinline__ void rank_weight_grad(const PassGradLayout& gl, const Real* v, const Real* vd,
                                                 const Real* lam, const Real* mu, double* slot, int lane) {
  if (gl.rw_off < 0) return;
  for (int w = lane; w < gl.nw; w += kWarp) {
    Real s = Real(0);
    for (int p = gl.w_begin[w]; p < gl.w_begin[w + 1]; ++p) {
      const int src = gl.w_src[p], dst = gl.w_dst[p];
      s += lam[dst] * v[src] + mu[dst] * vd[src];
    }
    slot[gl.rw_off + w] += double(s);
  }
}

// (at most 128 threads per block, chosen by the launch configuration; registers capped for three
// resident blocks for the whole pass, measured 2% faster on the 256-frame training step than the
// uncapped build, and for four for each part of a split pass: 3.66 -> 3.52 ms on that step)
// PART: GradPart (the gate forward pass runs whole: it has no per-edge parameter loop).
template <int L, typename Real, int MODE, bool KAHAN, int BF, bool COLS, int PART>
__global__ void __launch_bounds__(128, PART == kGradWhole ? 3 : 4) grad_pass_kernel(GradArgs<Real> a) {
  constexpr int Lp = L + 1, H = Lp * Lp;
  constexpr int NBM = BF ? BF : kMaxB;
  constexpr int kMaxItems = (kMaxK * H + kWarp - 1) / kWarp;
  using V4 = typename Vec4<Real>::type;
  const DevModel<Real>& dm = a.dm;
  const bool gate_pass = MODE != kGradOuter;
  const PassTables<Real>& pt = gate_pass ? dm.gate : dm.outer;
  const PassGradLayout& gl = gate_pass ? dm.grad.gate : dm.grad.outer;
  const int C = dm.C, F = dm.F, B = BF ? BF : dm.B, K = dm.K, M = dm.M, NB = dm.NB, NP = dm.grad.nparams;
  const int C2 = C * C;
  const bool effect_outer = MODE == kGradOuter && dm.gated;
  const int warps = blockDim.x / kWarp, warp = threadIdx.x / kWarp, lane = warp_lane();

  extern __shared__ __align__(16) unsigned char smem_raw[];
  Real* sm = reinterpret_cast<Real*>(smem_raw);
  Real* s_coeff = sm;
  Real* s_scal = s_coeff + F * B;
  Real* s_w0 = s_scal + 2 * dm.nblk * C2;
  Real* s_w1 = s_w0 + C * F;
  Real* s_wa = s_w1 + C * F;
  const int ncol = COLS ? a.acc_cols : 0;
  const int wsize = PART == kGradEdgePart ? grad_edge_warp_size(K, H) : grad_warp_size<Real>(F, H, M, K, dm.prog_parts);
  Real* wbase = s_wa + C * F + (wsize + ncol * kAccStride) * warp;
  const int sw = 2 * F + 2 * H + 1;
  Real* stage = wbase;
  Real* v = stage + kWarp * sw;    // [M + 1], v[M] = 1
  Real* vd = v + M + 1;            // [M + 1], vd[M] = 0
  const bool adj_staged = grad_adj_in_stage(F, H, M);
  Real* lam = adj_staged ? stage : vd + M + 1;
  Real* mu = lam + M + 1;
  Real* abl = PART == kGradEdgePart ? wbase : vd + M + 1 + (adj_staged ? 0 : 2 * (M + 1));
  Real* abm = abl + K * H;
  Real* hb = abm + K * H;  // [2F]
  Real* parts = hb + 2 * F;  // [2 prog_parts]
  Real* accs = wbase + wsize;  // [ncol][kAccStride]
  const int nsb = grad_acc_nsb(dm.scaling_mode, Lp);
  const int c_wc = Lp * B, c_scal = c_wc + C * Lp, c_add = c_scal + 2 * nsb * C;

  for (int q = threadIdx.x; q < F * B; q += blockDim.x) s_coeff[q] = pt.coeff[q];
  for (int q = threadIdx.x; q < 2 * dm.nblk * C2; q += blockDim.x) s_scal[q] = pt.scal[q];
  for (int q = threadIdx.x; q < C * F; q += blockDim.x) {
    s_w0[q] = pt.wcenter[q];
    s_w1[q] = pt.wsource[q];
    s_wa[q] = pt.wadd ? pt.wadd[q] : Real(0);
  }
  for (int q = lane; q < ncol * kAccStride; q += kWarp) accs[q] = Real(0);
  __syncthreads();
  double* slot = a.slots + static_cast<size_t>(blockIdx.x * warps + warp) * NP;

  const int nit = (K * H + kWarp - 1) / kWarp;  // moment items in use of the kMaxItems slots
  int it_u[kMaxItems], it_y[kMaxItems];
#pragma unroll
  for (int s = 0; s < kMaxItems; ++s) {
    const int t = lane + kWarp * s;
    if (t < K * H) {
      const int kk = t / H, lm = t - kk * H;
      int l = 0;
      while ((l + 1) * (l + 1) <= lm) ++l;
      it_u[s] = kk * Lp + l;
      it_y[s] = 2 * F + lm;
    } else {
      it_u[s] = -1;
      it_y[s] = 0;
    }
  }

  for (int atom = blockIdx.x * warps + warp; atom < a.natoms; atom += gridDim.x * warps) {
    const int ti = C == 1 ? 0 : a.types[atom];
    const int e0 = a.row[atom], e1 = a.row_end[atom];
    const double* Sw = a.sw + 9 * a.frame_of[atom];
    const Real S00 = Real(Sw[0]), S01 = Real(Sw[1]), S02 = Real(Sw[2]), S10 = Real(Sw[3]), S11 = Real(Sw[4]),
               S12 = Real(Sw[5]), S20 = Real(Sw[6]), S21 = Real(Sw[7]), S22 = Real(Sw[8]);
    const double fix = a.fw[3 * atom], fiy = a.fw[3 * atom + 1], fiz = a.fw[3 * atom + 2];

    // geometry, tangent direction and harmonics (values + tangents) of edge e
    auto edge_geometry = [&](int e, int& j, int& tj, Real& r, Real& ux, Real& uy, Real& uz, Real& rdot, Real* Y,
                             Real* Yd, bool& ang) {
      const V4 dv = a.d4[e];
      j = a.nbr[e];
      tj = C == 1 ? 0 : a.types[j];
      r = dv.w;
      const Real ir = Real(1) / r;
      ux = dv.x * ir; uy = dv.y * ir; uz = dv.z * ir;
      const Real wx = Real(fix - a.fw[3 * j]) + S00 * dv.x + S01 * dv.y + S02 * dv.z;
      const Real wy = Real(fiy - a.fw[3 * j + 1]) + S10 * dv.x + S11 * dv.y + S12 * dv.z;
      const Real wz = Real(fiz - a.fw[3 * j + 2]) + S20 * dv.x + S21 * dv.y + S22 * dv.z;
      rdot = ux * wx + uy * wy + uz * wz;
      sph_values<L, Real>(ux, uy, uz, Y);
      sph_tangent<L, Real>(ux, uy, uz, (wx - ux * rdot) * ir, (wy - uy * rdot) * ir, (wz - uz * rdot) * ir, Yd);
      ang = !(r >= dm.rang);
      if (!ang)
#pragma unroll
        for (int h = 1; h < H; ++h) { Y[h] = Real(0); Yd[h] = Real(0); }
    };

    if constexpr (PART == kGradEdgePart) {
      // ---------------- the atom's moment adjoints from the per-atom part ----------------
      const Real* src = a.abar + static_cast<size_t>(atom) * 2 * K * H;
      for (int t = lane; t < 2 * K * H; t += kWarp) abl[t] = src[t];
      __syncwarp();
    } else {
    if (MODE != kGradGateReverse) {
      // ---------------- forward with tangents ----------------
      Real acc[kMaxItems], cmp[kMaxItems], accd[kMaxItems], cmpd[kMaxItems];
#pragma unroll
      for (int s = 0; s < kMaxItems; ++s) { acc[s] = cmp[s] = accd[s] = cmpd[s] = Real(0); }
      for (int base = e0; base < e1; base += kWarp) {
        const int e = base + lane;
        Real* rw = stage + lane * sw;
        for (int q = 0; q < sw; ++q) rw[q] = Real(0);
        if (e < e1) {
          int j, tj;
          Real r, ux, uy, uz, rdot, Y[H], Yd[H];
          bool ang;
          edge_geometry(e, j, tj, r, ux, uy, uz, rdot, Y, Yd, ang);
#pragma unroll
          for (int h = 0; h < H; ++h) { rw[2 * F + h] = Y[h]; rw[2 * F + H + h] = Yd[h]; }
          const Real* hj = effect_outer ? a.hsig + static_cast<size_t>(j) * F : nullptr;
          const Real* hdj = effect_outer ? a.hsigd + static_cast<size_t>(j) * F : nullptr;
          radial_loop<L, Real, true, BF>(dm, s_coeff, s_scal, ti * C + tj, r, [&](int, int, int m_, Real R, Real Rd) {
            const Real x0 = s_w0[ti * F + m_];
            Real x3 = s_w1[tj * F + m_], x3d = Real(0);
            if (effect_outer) {
              x3 += s_wa[tj * F + m_] * hj[m_];
              x3d = s_wa[tj * F + m_] * hdj[m_];
            }
            rw[m_] = x0 * x3 * R;
            rw[F + m_] = x0 * (x3d * R + x3 * Rd * rdot);
          });
        }
        __syncwarp();
        // plain sums over the batch, compensated adds of the batch partials
        const int nb = min(kWarp, e1 - base);
        Real part[kMaxItems], partd[kMaxItems];
#pragma unroll
        for (int s = 0; s < kMaxItems; ++s) { part[s] = Real(0); partd[s] = Real(0); }
        for (int q = 0; q < nb; ++q) {
          const Real* sr = stage + q * sw;
#pragma unroll
          for (int s = 0; s < kMaxItems; ++s) {
            if (s >= nit) break;  // warp-uniform: only the model's K H items are issued
            if (it_u[s] >= 0) {
              const Real uu = sr[it_u[s]], ud = sr[F + it_u[s]], yy = sr[it_y[s]], yd = sr[it_y[s] + H];
              part[s] += uu * yy;
              partd[s] += ud * yy + uu * yd;
            }
          }
        }
#pragma unroll
        for (int s = 0; s < kMaxItems; ++s) {
          kadd<Real, KAHAN>(acc[s], cmp[s], part[s]);
          kadd<Real, KAHAN>(accd[s], cmpd[s], partd[s]);
        }
        __syncwarp();
      }
      for (int q = lane; q <= M; q += kWarp) { v[q] = q < M ? Real(0) : Real(1); vd[q] = Real(0); }
      __syncwarp();
#pragma unroll
      for (int s = 0; s < kMaxItems; ++s) {
        const int t = lane + kWarp * s;
        if (t < K * H) {
          const int b = dm.basic_of[t];
          if (b >= 0) { v[b] = acc[s]; vd[b] = accd[s]; }
        }
      }
      __syncwarp();
      run_prog_dual<Real, 1>(pt.prog, 0, pt.prog.nfwd, v, vd, lam, mu, parts, lane);
      if (MODE == kGradGateForward) {
        for (int q = lane; q < M; q += kWarp) {
          a.gmom[static_cast<size_t>(atom) * M + q] = v[q];
          a.gmomd[static_cast<size_t>(atom) * M + q] = vd[q];
        }
        for (int m_ = lane; m_ < F; m_ += kWarp) {
          Real h = Real(0), hd = Real(0);
          for (int q = 0; q < dm.Q; ++q) {
            h += dm.gate_wmat[m_ * dm.Q + q] * v[dm.gate_nodes[q]];
            hd += dm.gate_wmat[m_ * dm.Q + q] * vd[dm.gate_nodes[q]];
          }
          a.hsig[static_cast<size_t>(atom) * F + m_] = h;
          a.hsigd[static_cast<size_t>(atom) * F + m_] = hd;
        }
        __syncwarp();
        continue;
      }
      // ---------------- readout gradient and seeds ----------------
      const double ewi = a.ew[atom];
      const double coef = dm.species_readout ? 1.0 : dm.species[ti];
      const int off = dm.species_readout ? ti * dm.S : 0;
      for (int q = lane; q <= M; q += kWarp) { lam[q] = Real(0); mu[q] = Real(0); }
      __syncwarp();
      double sp = 0.0;
      for (int q = lane; q < dm.S; q += kWarp) {
        const int node = dm.scalar_map[q];
        const double lin = double(dm.linear[off + q]);
        const double g = ewi * double(v[node]) + double(vd[node]);
        slot[dm.grad.linear_off + off + q] += coef * g;
        if (!dm.species_readout) sp += lin * g;
        lam[node] = Real(ewi * coef * lin);
        mu[node] = Real(coef * lin);
      }
      sp = warp_sum(sp);
      if (lane == 0) {
        slot[dm.grad.shift_off + ti] += ewi;
        slot[dm.grad.species_off + ti] += ewi + sp;
      }
      __syncwarp();
    } else {
      // ---------------- gate reverse seeds from dJ/dh, dJ/dhdot ----------------
      for (int m_ = lane; m_ < 2 * F; m_ += kWarp) {
        const Real s = column_sum<Real>(a.lhm + static_cast<size_t>(e0) * 2 * F + m_, 2 * F, e1 - e0);
        double sd = double(s);
        if (a.extra_h && m_ < F) sd += a.extra_h[static_cast<size_t>(atom) * F + m_];
        hb[m_] = Real(sd);
        a.lh_atom[static_cast<size_t>(atom) * 2 * F + m_] = sd;
      }
      for (int q = lane; q <= M; q += kWarp) {
        v[q] = q < M ? a.gmom[static_cast<size_t>(atom) * M + q] : Real(1);
        vd[q] = q < M ? a.gmomd[static_cast<size_t>(atom) * M + q] : Real(0);
        lam[q] = Real(0);
        mu[q] = Real(0);
      }
      __syncwarp();
      for (int q = lane; q < dm.Q; q += kWarp) {
        Real sl = Real(0), sm_ = Real(0);
        for (int m_ = 0; m_ < F; ++m_) {
          sl += hb[m_] * dm.gate_wmat[m_ * dm.Q + q];
          sm_ += hb[F + m_] * dm.gate_wmat[m_ * dm.Q + q];
        }
        lam[dm.gate_nodes[q]] += sl;
        mu[dm.gate_nodes[q]] += sm_;
      }
      __syncwarp();
    }

    // ---------------- reverse over values and tangents ----------------
    // the contraction's reverse is the program's last step when the pass has a contraction; the
    // rank-weight gradients read the adjoints just before it
    {
      const int last = pt.ndst > 0 ? pt.prog.nsteps - 1 : pt.prog.nsteps;
      run_prog_dual<Real, 2>(pt.prog, pt.prog.nfwd, last, v, vd, lam, mu, parts, lane);
      if (pt.ndst > 0) {
        rank_weight_grad<Real>(gl, v, vd, lam, mu, slot, lane);
        __syncwarp();
        run_prog_dual<Real, 2>(pt.prog, last, pt.prog.nsteps, v, vd, lam, mu, parts, lane);
      }
    }
    if constexpr (PART == kGradAtomPart) {
      Real* dst = a.abar + static_cast<size_t>(atom) * 2 * K * H;
      for (int t = lane; t < K * H; t += kWarp) {
        const int b = dm.basic_of[t];
        dst[t] = b >= 0 ? lam[b] : Real(0);
        dst[K * H + t] = b >= 0 ? mu[b] : Real(0);
      }
      __syncwarp();
      continue;
    }
    for (int t = lane; t < K * H; t += kWarp) {
      const int b = dm.basic_of[t];
      abl[t] = b >= 0 ? lam[b] : Real(0);
      abm[t] = b >= 0 ? mu[b] : Real(0);
    }
    __syncwarp();
    }  // PART != kGradEdgePart

    // ---------------- per-edge parameter contributions ----------------
    for (int base = e0; base < e1; base += kWarp) {
      const int e = base + lane;
      const bool valid = e < e1;
      int j = 0, tj = 0;
      Real r = Real(1), ux = Real(0), uy = Real(0), uz = Real(1), rdot = Real(0), Y[H], Yd[H];
      bool ang = true;
      if (valid) edge_geometry(e, j, tj, r, ux, uy, uz, rdot, Y, Yd, ang);
      else
#pragma unroll
        for (int h = 0; h < H; ++h) { Y[h] = Real(0); Yd[h] = Real(0); }
      Real f0, fd0, f1, fd1;
      envelope<Real>(r, dm.rmax, dm.poly, dm.cutoff_p, f0, fd0);
      if (dm.split) envelope<Real>(r, dm.rang, dm.poly, dm.cutoff_p, f1, fd1);
      else { f1 = f0; fd1 = fd0; }
      f0 *= dm.scaling; fd0 *= dm.scaling; f1 *= dm.scaling; fd1 *= dm.scaling;
      const Real* hj = (effect_outer && valid) ? a.hsig + static_cast<size_t>(j) * F : nullptr;
      const Real* hdj = (effect_outer && valid) ? a.hsigd + static_cast<size_t>(j) * F : nullptr;
      for (int k = 0; k < K; ++k) {
        Real Tv[NBM], D[NBM], DD[NBM];
        WarpVar<Real> wv;
        int sb_prev = -1;
#pragma unroll
        for (int l = 0; l < Lp; ++l) {
          const int sb = scaling_block(dm.scaling_mode, k, l, Lp);
          if (sb != sb_prev) {
            wv = warp_var<Real>(r, s_scal[2 * sb * C2 + ti * C + tj], s_scal[(2 * sb + 1) * C2 + ti * C + tj]);
            cheb_full<Real, NBM>(wv.xi, B, Tv, D, DD);
            sb_prev = sb;
          }
          const int m_ = k * Lp + l;
          const bool on = valid && (l == 0 || ang);
          const Real* c = s_coeff + m_ * B;
          Real cT = Real(0), cD = Real(0), cDD = Real(0);
#pragma unroll
          for (int b = 0; b < NBM; ++b)
            if (b < B) { cT += c[b] * Tv[b]; cD += c[b] * D[b]; cDD += c[b] * DD[b]; }
          const Real f = l == 0 ? f0 : f1, fd = l == 0 ? fd0 : fd1;
          const Real R = f * cT, Rd = fd * cT + f * cD * wv.xr;
          Real Sv = Real(0), Tt = Real(0), Uv = Real(0);
#pragma unroll
          for (int h = l * l; h < (l + 1) * (l + 1); ++h) {
            Sv += abl[k * H + h] * Y[h];
            Tt += abm[k * H + h] * Y[h];
            Uv += abm[k * H + h] * Yd[h];
          }
          const Real x0 = s_w0[ti * F + m_];
          Real x3 = s_w1[tj * F + m_], x3d = Real(0), al = Real(0), hv = Real(0), hdv = Real(0);
          if (effect_outer && valid) {
            al = s_wa[tj * F + m_];
            hv = hj[m_];
            hdv = hdj[m_];
            x3 += al * hv;
            x3d = al * hdv;
          }
          const Real Qv = R * (Sv + Uv) + Rd * rdot * Tt;
          Real dR = on ? x0 * (x3 * (Sv + Uv) + x3d * Tt) : Real(0);
          Real dRd = on ? x0 * x3 * rdot * Tt : Real(0);
          const Real dx0 = on ? x3 * Qv + x3d * R * Tt : Real(0);
          const Real dxj = on ? x0 * Qv : Real(0);
          // warp (slope, shift) of block sb and pair (t_i, t_j)
          const Real ds = wv.xs * (dR * f + dRd * fd) * cD + dRd * f * (wv.xs * wv.xr * cDD + wv.xrs * cD);
          const Real dg = wv.xg * (dR * f + dRd * fd) * cD + dRd * f * (wv.xg * wv.xr * cDD + wv.xrg * cD);
          const Real dal = (effect_outer && on) ? x0 * (Qv * hv + R * Tt * hdv) : Real(0);
          if (COLS) {
            Real* ac = accs + lane;
#pragma unroll
            for (int b = 0; b < NBM; ++b)
              if (b < B) ac[(l * B + b) * kAccStride] += dR * f * Tv[b] + dRd * (fd * Tv[b] + f * D[b] * wv.xr);
            ac[(c_wc + ti * Lp + l) * kAccStride] += dx0;
            ac[(c_wc + tj * Lp + l) * kAccStride] += dxj;
            const int sc = c_scal + 2 * ((nsb > 1 ? l : 0) * C + tj);
            ac[sc * kAccStride] += ds;
            ac[(sc + 1) * kAccStride] += dg;
            if (effect_outer) ac[(c_add + tj * Lp + l) * kAccStride] += dal;
          } else {
            // Chebyshev coefficients of R_mu
            for (int b = 0; b < B; ++b)
              slot_add<Real>(slot, gl.coeff_off + m_ * gl.coeff_stride + b,
                             dR * f * Tv[b] + dRd * (fd * Tv[b] + f * D[b] * wv.xr), lane);
            for (int t = 0; t < C; ++t) {
              slot_add<Real>(slot, gl.scal_off + 2 * sb * C2 + ti * C + t, tj == t ? ds : Real(0), lane);
              slot_add<Real>(slot, gl.scal_off + (2 * sb + 1) * C2 + ti * C + t, tj == t ? dg : Real(0), lane);
            }
            // species factors of the centre and the neighbour
            slot_add<Real>(slot, gl.wc_off + ti * gl.wc_t_stride + m_ * gl.wc_mu_stride, dx0, lane);
            for (int t = 0; t < C; ++t)
              slot_add<Real>(slot, gl.wc_off + t * gl.wc_t_stride + m_ * gl.wc_mu_stride, tj == t ? dxj : Real(0), lane);
            if (effect_outer)
              for (int t = 0; t < C; ++t) slot_add<Real>(slot, gl.add_off + t * F + m_, tj == t ? dal : Real(0), lane);
          }
          if (effect_outer && valid) {
            Real* dst = a.lhm + static_cast<size_t>(a.rev[e]) * 2 * F;
            dst[m_] = on ? x0 * al * Qv : Real(0);
            dst[F + m_] = on ? x0 * al * R * Tt : Real(0);
          }
        }
        if (COLS) {
          // flush the columns of radial index k: column c summed over the 32 lanes in lane order
          __syncwarp();
          for (int c = lane; c < ncol; c += kWarp) {
            Real* col = accs + c * kAccStride;
            Real sum = Real(0);
#pragma unroll 8
            for (int q = 0; q < kWarp; ++q) { sum += col[q]; col[q] = Real(0); }
            int p;
            if (c < c_wc) {
              const int l = c / B, b = c - l * B;
              p = gl.coeff_off + (k * Lp + l) * gl.coeff_stride + b;
            } else if (c < c_scal) {
              const int t = (c - c_wc) / Lp, l = c - c_wc - t * Lp;
              p = gl.wc_off + t * gl.wc_t_stride + (k * Lp + l) * gl.wc_mu_stride;
            } else if (c < c_add) {
              const int idx = c - c_scal, pair = idx >> 1, which = idx & 1;
              const int sbi = pair / C, t = pair - sbi * C;
              const int sb = scaling_block(dm.scaling_mode, k, sbi, Lp);
              p = gl.scal_off + (2 * sb + which) * C2 + ti * C + t;
            } else {
              const int t = (c - c_add) / Lp, l = c - c_add - t * Lp;
              p = gl.add_off + t * F + k * Lp + l;
            }
            slot[p] += double(sum);
          }
          __syncwarp();
        }
      }
    }
    __syncwarp();
  }
}

}  // namespace sus2g
