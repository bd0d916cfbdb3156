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
// deterministic.  The product graph runs level by level over shared-memory node
// arrays; the reverse graph is a gather per consumed node (no write conflicts).  The adjoint
// pass recomputes Y and R per edge instead of storing them and writes g_e per edge; forces are
// gathered per atom through the reverse-edge permutation by a separate kernel.
#pragma once
#include "basis.cuh"

namespace sus2g {

enum PassMode : int { kModeStatic = 0, kModeGateForward = 1, kModeOuter = 2, kModeGateReverse = 3 };

template <typename Real>
struct PassArgs {
  DevModel<Real> dm;
  int natoms;
  const int* types;
  const int* row;          // [natoms + 1] CSR by centre
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
  int* error;
};

template <typename Real>
__host__ __device__ inline int pass_table_size(int C, int F, int B, int nblk) {
  return F * B + 2 * nblk * C * C + 3 * C * F;
}
template <typename Real>
__host__ __device__ inline int pass_warp_size(int F, int H, int M, int K) {
  return kWarp * (F + H + 1) + 2 * M + K * H + F + 4;
}

// Kahan-compensated accumulation for the FP32 bulk form; plain sums in FP64.
template <typename Real, bool KAHAN>
__device__ __forceinline__ void kadd(Real& s, Real& c, Real x) {
  if (KAHAN) {
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
      Real a = Real(0), ad = Real(0);
#pragma unroll
      for (int b = 0; b < NBM; ++b) {
        if (b < B) {
          a += c[b] * Tv[b];
          if (DERIV) ad += c[b] * Td[b];
        }
      }
      const Real f = l == 0 ? f0 : f1, fd = l == 0 ? fd0 : fd1;
      const Real R = f * a;
      const Real Rd = DERIV ? (fd * a + f * ad) : Real(0);
      body(k, l, mu, R, Rd);
    }
  }
}

// ---------------------------------------------------------------------------------------------
// Warp-cooperative per-atom graph helpers on shared-memory node arrays.
// ---------------------------------------------------------------------------------------------
template <typename Real>
__device__ __forceinline__ void contract_forward(const PassTables<Real>& t, Real* v, int lane) {
  for (int q = lane; q < t.ndst; q += kWarp) {
    Real s = Real(0);
    for (int p = t.dst_begin[q]; p < t.dst_begin[q + 1]; ++p) s += t.dst_w[p] * v[t.dst_src[p]];
    v[t.dst_node[q]] += s;
  }
  __syncwarp();
}

template <typename Real>
__device__ __forceinline__ void contract_reverse(const PassTables<Real>& t, int NB, Real* adj, int lane) {
  if (t.ndst == 0) return;
  for (int b = lane; b < NB; b += kWarp) {
    Real s = Real(0);
    for (int p = t.src_begin[b]; p < t.src_begin[b + 1]; ++p) s += t.src_w[p] * adj[t.src_dst[p]];
    adj[b] += s;
  }
  __syncwarp();
}

template <typename Real>
__device__ __forceinline__ void graph_forward(const PassTables<Real>& t, Real* v, int lane) {
  for (int lv = 0; lv < t.levels; ++lv) {
    for (int q = t.level_begin[lv] + lane; q < t.level_begin[lv + 1]; q += kWarp) {
      Real s = Real(0);
      for (int p = t.out_begin[q]; p < t.out_begin[q + 1]; ++p) s += t.fprod_c[p] * v[t.fprod_a[p]] * v[t.fprod_b[p]];
      v[t.out_nodes[q]] += s;
    }
    __syncwarp();
  }
}

template <typename Real>
__device__ __forceinline__ void graph_reverse(const PassTables<Real>& t, const Real* v, Real* adj, int lane) {
  for (int lv = t.levels - 1; lv >= 0; --lv) {
    for (int q = t.rlevel_begin[lv] + lane; q < t.rlevel_begin[lv + 1]; q += kWarp) {
      Real s = Real(0);
      for (int p = t.in_begin[q]; p < t.in_begin[q + 1]; ++p) s += t.rprod_c[p] * adj[t.rprod_out[p]] * v[t.rprod_other[p]];
      adj[t.in_nodes[q]] += s;
    }
    __syncwarp();
  }
}

// ---------------------------------------------------------------------------------------------
// The pass kernel.
// ---------------------------------------------------------------------------------------------
constexpr int kPassWarps = 4;
// Minimum resident blocks per SM: 4 (<= 128 registers) where the FP32 kernels fit without
// spilling (L <= 3), 3 otherwise (measured: the FP64 kernels and L >= 4 run faster at 3).

template <int L, typename Real, int MODE, bool KAHAN, int BF>
__global__ void __launch_bounds__(kPassWarps * kWarp, (L <= 3 && sizeof(Real) == 4) ? 4 : 3) atom_pass_kernel(PassArgs<Real> a) {
  constexpr int Lp = L + 1, H = Lp * Lp;
  constexpr int kMaxItems = (kMaxK * H + kWarp - 1) / kWarp;
  using V4 = typename Vec4<Real>::type;
  const DevModel<Real>& dm = a.dm;
  const bool gate_pass = MODE == kModeGateForward || MODE == kModeGateReverse;
  const PassTables<Real>& pt = gate_pass ? dm.gate : dm.outer;
  const int C = dm.C, F = dm.F, B = BF ? BF : dm.B, K = dm.K, M = dm.M, NB = dm.NB;
  const int warps = blockDim.x / kWarp, warp = threadIdx.x / kWarp, lane = warp_lane();

  extern __shared__ __align__(16) unsigned char smem_raw[];
  Real* sm = reinterpret_cast<Real*>(smem_raw);
  Real* s_coeff = sm;
  Real* s_scal = s_coeff + F * B;
  Real* s_w0 = s_scal + 2 * dm.nblk * C * C;
  Real* s_w1 = s_w0 + C * F;
  Real* s_wa = s_w1 + C * F;
  Real* wbase = s_wa + C * F + pass_warp_size<Real>(F, H, M, K) * warp;
  Real* stage = wbase;                              // [32][F + H + 1]
  Real* v = stage + kWarp * (F + H + 1);            // [M]
  Real* adj = v + M;                                // [M]
  Real* abar = adj + M;                             // [K][H]
  Real* hbar = abar + K * H;                        // [F]
  const int sw = F + H + 1;

  for (int q = threadIdx.x; q < F * B; q += blockDim.x) s_coeff[q] = pt.coeff[q];
  for (int q = threadIdx.x; q < 2 * dm.nblk * C * C; q += blockDim.x) s_scal[q] = pt.scal[q];
  for (int q = threadIdx.x; q < C * F; q += blockDim.x) {
    s_w0[q] = pt.wcenter[q];
    s_w1[q] = pt.wsource[q];
    s_wa[q] = pt.wadd ? pt.wadd[q] : Real(0);
  }
  __syncthreads();
  const bool effect_outer = MODE == kModeOuter;

  // Lane-owned moment items for the forward reduction: item t = lane + 32 s <-> (k, lm).
  int it_u[kMaxItems], it_y[kMaxItems];
#pragma unroll
  for (int s = 0; s < kMaxItems; ++s) {
    const int t = lane + kWarp * s;
    if (t < K * H) {
      const int kk = t / H, lm = t - kk * H;
      int l = 0;
      while ((l + 1) * (l + 1) <= lm) ++l;
      it_u[s] = kk * Lp + l;
      it_y[s] = F + lm;
    } else {
      it_u[s] = -1;
      it_y[s] = 0;
    }
  }

  for (int atom = blockIdx.x * warps + warp; atom < a.natoms; atom += gridDim.x * warps) {
    const int ti = a.types[atom];
    const int e0 = a.row[atom], e1 = a.row[atom + 1];
    // per-atom virial: FP64 for the FP64 form; compensated FP32 (hi, lo) for the FP32 bulk form
    double vir[6] = {0, 0, 0, 0, 0, 0};
    float vhi[6] = {0, 0, 0, 0, 0, 0}, vlo[6] = {0, 0, 0, 0, 0, 0};

    if (MODE != kModeGateReverse) {
      // ---------------- forward moments ----------------
      Real acc[kMaxItems], cmp[kMaxItems];
#pragma unroll
      for (int s = 0; s < kMaxItems; ++s) { acc[s] = Real(0); cmp[s] = Real(0); }
      for (int base = e0; base < e1; base += kWarp) {
        const int e = base + lane;
        Real* row = stage + lane * sw;
        if (e < e1) {
          const V4 dv = a.d4[e];
          const int j = a.nbr[e];
          const int tj = a.types[j];
          const Real r = dv.w, ir = Real(1) / r;
          Real Y[H];
          sph_values<L, Real>(dv.x * ir, dv.y * ir, dv.z * ir, Y);
          const bool ang = !(r >= dm.rang);
#pragma unroll
          for (int h = 0; h < H; ++h) row[F + h] = (h == 0 || ang) ? Y[h] : Real(0);
          const Real* hj = effect_outer ? a.hsig + (size_t)j * F : nullptr;
          for (int mu = 0; mu < F; ++mu) row[mu] = Real(0);
          radial_loop<L, Real, false, BF>(dm, s_coeff, s_scal, ti * C + tj, r, [&](int k, int l, int mu, Real R, Real) {
            Real x3 = s_w1[tj * F + mu];
            if (effect_outer) x3 += s_wa[tj * F + mu] * hj[mu];
            row[mu] = s_w0[ti * F + mu] * x3 * R;
          });
        } else {
          for (int q = 0; q < F; ++q) row[q] = Real(0);
          for (int h = 0; h < H; ++h) row[F + h] = Real(0);
        }
        __syncwarp();
        // plain sum over the batch's (<= 32) staged edges, then a compensated add of the batch
        // partial into the atom's running moment
        const int nb = min(kWarp, e1 - base);
        Real part[kMaxItems];
#pragma unroll
        for (int s = 0; s < kMaxItems; ++s) part[s] = Real(0);
        for (int q = 0; q < nb; ++q) {
          const Real* sr = stage + q * sw;
#pragma unroll
          for (int s = 0; s < kMaxItems; ++s)
            if (it_u[s] >= 0) part[s] += sr[it_u[s]] * sr[it_y[s]];
        }
#pragma unroll
        for (int s = 0; s < kMaxItems; ++s) kadd<Real, KAHAN>(acc[s], cmp[s], part[s]);
        __syncwarp();
      }
      for (int q = lane; q < M; q += kWarp) v[q] = Real(0);
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
      contract_forward<Real>(pt, v, lane);
      graph_forward<Real>(pt, v, lane);

      if (MODE == kModeGateForward) {
        for (int q = lane; q < M; q += kWarp) a.gmom[(size_t)atom * M + q] = v[q];
        for (int mu = lane; mu < F; mu += kWarp) {
          Real h = Real(0);
          for (int q = 0; q < dm.Q; ++q) h += dm.gate_wmat[mu * dm.Q + q] * v[dm.gate_nodes[q]];
          a.hsig[(size_t)atom * F + mu] = h;
        }
        __syncwarp();
        continue;
      }

      // ---------------- readout and seeds ----------------
      const double coef = dm.species_readout ? 1.0 : dm.species[ti];
      const int off = dm.species_readout ? ti * dm.S : 0;
      double es = 0.0;
      for (int q = lane; q < M; q += kWarp) adj[q] = Real(0);
      __syncwarp();
      for (int q = lane; q < dm.S; q += kWarp) {
        const int node = dm.scalar_map[q];
        const double rho = coef * double(dm.linear[off + q]);
        es += rho * double(v[node]);
        adj[node] = Real(rho);
        if (a.desc) a.desc[static_cast<size_t>(atom) * dm.S + q] = double(v[node]);
      }
      es = warp_sum(es);
      if (lane == 0) a.site_energy[atom] = dm.species[ti] + dm.shift[ti] + es;
      __syncwarp();
    } else {
      // ---------------- gate reverse: gather hbar, project, load gate values ----------------
      for (int mu = lane; mu < F; mu += kWarp) {
        if (a.hbar_atom) {
          hbar[mu] = Real(a.hbar_atom[(size_t)atom * F + mu]);
        } else {
          Real s = Real(0);
          for (int e = e0; e < e1; ++e) s += a.hcontrib[(size_t)e * F + mu];
          hbar[mu] = s;
        }
      }
      for (int q = lane; q < M; q += kWarp) {
        v[q] = a.gmom[(size_t)atom * M + q];
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
    graph_reverse<Real>(pt, v, adj, lane);
    contract_reverse<Real>(pt, NB, adj, lane);
    for (int t = lane; t < K * H; t += kWarp) {
      const int b = dm.basic_of[t];
      abar[t] = b >= 0 ? adj[b] : Real(0);
    }
    __syncwarp();

    // ---------------- per-edge adjoint ----------------
    for (int e = e0 + lane; e < e1; e += kWarp) {
      const V4 dv = a.d4[e];
      const int j = a.nbr[e];
      const int tj = a.types[j];
      const Real r = dv.w, ir = Real(1) / r;
      const Real ux = dv.x * ir, uy = dv.y * ir, uz = dv.z * ir;
      const bool ang = !(r >= dm.rang);
      Real Y[H], P[H], Qd[H];
      sph_values<L, Real>(ux, uy, uz, Y);
#pragma unroll
      for (int h = 0; h < H; ++h) { P[h] = Real(0); Qd[h] = Real(0); if (h > 0 && !ang) Y[h] = Real(0); }
      const Real* hj = effect_outer ? a.hsig + (size_t)j * F : nullptr;
      Real* hc = effect_outer ? a.hcontrib + (size_t)a.rev[e] * F : nullptr;
      radial_loop<L, Real, true, BF>(dm, s_coeff, s_scal, ti * C + tj, r, [&](int k, int l, int mu, Real R, Real Rd) {
        const Real x0 = s_w0[ti * F + mu];
        Real x3 = s_w1[tj * F + mu];
        if (effect_outer) x3 += s_wa[tj * F + mu] * hj[mu];
        const Real w = x0 * x3, wR = w * R, wRd = w * Rd;
        const Real* ab = abar + k * H;
        Real S = Real(0);
#pragma unroll
        for (int h = l * l; h < (l + 1) * (l + 1); ++h) {
          const Real av = ab[h];
          P[h] += wR * av;
          Qd[h] += wRd * av;
          if (effect_outer) S += av * Y[h];
        }
        if (effect_outer) hc[mu] = x0 * s_wa[tj * F + mu] * R * S;
      });
      if (effect_outer && !ang)
        for (int mu = 0; mu < F; ++mu)
          if (mu % Lp != 0) hc[mu] = Real(0);
      Real s = Real(0);
#pragma unroll
      for (int h = 0; h < H; ++h) s += Qd[h] * Y[h];
      Real gx = Real(0), gy = Real(0), gz = Real(0);
      if (ang) sph_grad_dot<L, Real>(ux, uy, uz, P, gx, gy, gz);
      const Real ug = ux * gx + uy * gy + uz * gz;
      const Real Gx = ux * s + (gx - ux * ug) * ir;
      const Real Gy = uy * s + (gy - uy * ug) * ir;
      const Real Gz = uz * s + (gz - uz * ug) * ir;
      Real* ge = a.g + (size_t)e * 3;
      if (MODE == kModeGateReverse) {
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
    if (sizeof(Real) == 4) {
#pragma unroll
      for (int c = 0; c < 6; ++c) vir[c] = warp_csum(vhi[c], vlo[c]);
    } else {
#pragma unroll
      for (int c = 0; c < 6; ++c) vir[c] = warp_sum(vir[c]);
    }
    if (lane == 0) {
      double* vo = a.virial + (size_t)atom * 6;
      if (MODE == kModeGateReverse)
        for (int c = 0; c < 6; ++c) vo[c] += vir[c];
      else
        for (int c = 0; c < 6; ++c) vo[c] = vir[c];
    }
    __syncwarp();
  }
}

}  // namespace sus2g
