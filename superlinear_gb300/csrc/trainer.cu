// GPU training step for one engine: labelled frames resident on the device, the energy / force /
// stress objective with its parameter gradient, and an FP64 BFGS on the device.
//
// Objective (NonLinearRegression::AddLoss / AddLossGrad, dev_src/non_linear_regression.cpp:768-1068,
// energy / force / stress terms and the Effect gate-x L2 term; std terms, other penalties and
// regularisers off), summed over the K
// frames and divided by K as the trainer does (dev_src/mtpr_trainer.cpp:4736-4745):
//   d = 0.1, a = <|F0|^2>, s = d / (d + fn a)
//   L_F = wF' s sum |F - F0|^2            dL/dF = 2 wF' s (F - F0)       wF' = wF (/N for "structures")
//   L_S = wS' |S - S0|_F^2 / N            stress weight = -2 wS' (S - S0) / N
//   L_E = wE' s (E - E0)^2 / N            dL/dE = 2 wE' s (E - E0) / N
//   wE' = wE, wS' = wS ("vibrations"), / N ("structures"), * N ("molecules")
// The derivative weights feed Engine::combination_grad (AccumulateEFSCombinationGrad contract).
//
// BFGS (src/common/bfgs.{h,cpp}): dense inverse-Hessian update in FP64 on the device, the
// direction p = -H g on the device, the line search on host scalars with the reference's strong
// Wolfe constants c1 = 0.1, c2 = 0.5 (bfgs.h:384-385).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <limits>
#include <memory>
#include <string>
#include <vector>

#include "../../include/sus2g.h"
#include "capi_types.h"
#include "device_common.cuh"

namespace sus2g {

#define TRAIN_CUDA(call)                                                                      \
  do {                                                                                        \
    cudaError_t err__ = (call);                                                               \
    if (err__ != cudaSuccess)                                                                 \
      throw Error(10, std::string("CUDA error: ") + cudaGetErrorString(err__) + " at " #call); \
  } while (0)

namespace {

struct LossConfig {
  double wE, wF, wS;
  int weighting;  // 0 vibrations, 1 structures, 2 molecules
  int norm_by_forces;
  double gate_x_l2;  // Effect gate-x L2 coefficient (0: off)
};

// One block per frame: loss terms and derivative weights.
__global__ void k_loss(int nframes, const int* fbegin, const double* E, const double* F, const double* V,
                       const double* E0, const double* F0, const double* S0, const int* has, LossConfig c,
                       double* ew, double* fw, double* sw, double* loss_f) {
  const int f = blockIdx.x;
  if (f >= nframes) return;
  const int a0 = fbegin[f], a1 = fbegin[f + 1], n = a1 - a0;
  __shared__ double red[2][256];
  double avef = 0.0, fl = 0.0;
  const bool hasE = has[f] & 1, hasF = has[f] & 2, hasS = has[f] & 4;
  for (int i = a0 + threadIdx.x; i < a1; i += blockDim.x)
    for (int q = 0; q < 3; ++q) avef += F0[3 * static_cast<size_t>(i) + q] * F0[3 * static_cast<size_t>(i) + q];
  red[0][threadIdx.x] = avef;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[0][threadIdx.x] += red[0][threadIdx.x + s];
    __syncthreads();
  }
  avef = n > 0 && hasF ? red[0][0] / n : 0.0;
  const double d = 0.1, scale_fn = d / (d + c.norm_by_forces * avef);
  double wF = c.wF, wE = c.wE, wS = c.wS;
  if (c.weighting == 1 && n > 0) { wF /= n; wE /= n; wS /= n; }
  else if (c.weighting == 2) { wE *= n; wS *= n; }
  const bool useF = c.wF != 0.0 && hasF;
  for (int i = a0 + threadIdx.x; i < a1; i += blockDim.x)
    for (int q = 0; q < 3; ++q) {
      const size_t k = 3 * static_cast<size_t>(i) + q;
      const double delta = F[k] - F0[k];
      if (useF) fl += wF * scale_fn * delta * delta;
      fw[k] = useF ? wF * scale_fn * 2.0 * delta : 0.0;
    }
  __syncthreads();
  red[1][threadIdx.x] = fl;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[1][threadIdx.x] += red[1][threadIdx.x + s];
    __syncthreads();
  }
  double dE = 0.0;
  if (threadIdx.x == 0) {
    double L = red[1][0];
    // virial (xx, yy, zz, xy, xz, yz) -> symmetric 3x3
    const double* v = V + 6 * f;
    const double S[9] = {v[0], v[3], v[4], v[3], v[1], v[5], v[4], v[5], v[2]};
    for (int q = 0; q < 9; ++q) sw[9 * f + q] = 0.0;
    if (wS != 0.0 && hasS && n > 0) {
      for (int q = 0; q < 9; ++q) {
        const double ds = S[q] - S0[9 * f + q];
        L += wS * ds * ds / n;
        sw[9 * f + q] = -2.0 * wS * ds / n;
      }
    }
    if (wE != 0.0 && hasE && n > 0) {
      const double de = E[f] - E0[f];
      L += wE * de * de * scale_fn / n;
      dE = 2.0 * wE * de * scale_fn / n;
    }
    loss_f[f] = L;
    red[0][0] = dE;
  }
  __syncthreads();
  dE = red[0][0];
  for (int i = a0 + threadIdx.x; i < a1; i += blockDim.x) ew[i] = dE;
}

// Effect gate-x L2 term of one frame (block per frame; MLMTPR::AddTwoLayerGateX2Penalty,
// dev_src/mtpr_sh.cpp:5869-6047):  P_f = sum over edges (i -> j) of norm(t_j) sum_mu (alpha(t_j, mu)
// h_j[mu])^2 with norm(t) = coeff / (active types x F x edges whose neighbour type is t).  Edges
// are symmetric, so the edges with neighbour j number deg(j) = row_end[j] - row[j].  Adds P_f to
// loss_f[f]; writes dP/dh_j to extra_h[j] (the gate-chain seed) and the frame's dP/dalpha to
// agrad[f][t F + mu]; fixed-order sums throughout.
template <typename Real>
__global__ void k_gatex_frame(int nframes, const int* fbegin, const int* row, const int* row_end, const int* types,
                              const Real* h,
                              const Real* alpha, int C, int F, double coeff, double* extra_h, double* loss_f,
                              double* agrad) {
  const int f = blockIdx.x;
  if (f >= nframes) return;
  const int a0 = fbegin[f], a1 = fbegin[f + 1];
  __shared__ unsigned long long count[64];
  __shared__ double red[256];
  for (int t = threadIdx.x; t < C; t += blockDim.x) count[t] = 0;
  __syncthreads();
  for (int j = a0 + threadIdx.x; j < a1; j += blockDim.x)
    atomicAdd(&count[types[j]], static_cast<unsigned long long>(row_end[j] - row[j]));
  __syncthreads();
  int active = 0;
  for (int t = 0; t < C; ++t) active += count[t] > 0;
  auto weight = [&](int j) {  // deg(j) norm(t_j)
    const int t = types[j], deg = row_end[j] - row[j];
    return deg > 0 ? coeff * deg / (double(active) * F * double(count[t])) : 0.0;
  };
  double pen = 0.0;
  for (int j = a0 + threadIdx.x; j < a1; j += blockDim.x) {
    const double w = weight(j);
    const int t = types[j];
    for (int mu = 0; mu < F; ++mu) {
      const double al = double(alpha[t * F + mu]), x = al * double(h[static_cast<size_t>(j) * F + mu]);
      pen += w * x * x;
      extra_h[static_cast<size_t>(j) * F + mu] = 2.0 * w * x * al;
    }
  }
  red[threadIdx.x] = pen;
  __syncthreads();
  for (int st = blockDim.x / 2; st > 0; st >>= 1) {
    if (threadIdx.x < st) red[threadIdx.x] += red[threadIdx.x + st];
    __syncthreads();
  }
  if (threadIdx.x == 0) loss_f[f] += red[0];
  for (int q = threadIdx.x; q < C * F; q += blockDim.x) {
    const int t = q / F, mu = q - t * F;
    const double al = double(alpha[q]);
    double g = 0.0;
    for (int j = a0; j < a1; ++j)
      if (types[j] == t) {
        const double hj = double(h[static_cast<size_t>(j) * F + mu]);
        g += 2.0 * weight(j) * al * hj * hj;
      }
    agrad[static_cast<size_t>(f) * C * F + q] = g;
  }
}

// grad[q] += sum over frames of agrad[f][q] (frame order)
__global__ void k_gatex_alpha(int nframes, int n, const double* agrad, double* grad) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  double s = 0.0;
  for (int f = 0; f < nframes; ++f) s += agrad[static_cast<size_t>(f) * n + q];
  grad[q] += s;
}

// Error-metric partial sums of one frame (block per frame), as NonLinearRegression::AddLoss collects
// them (dev_src/non_linear_regression.cpp:781-804): out[f][0..8] = |dE|, dE^2 / N, N (energy
// labelled), sum |dF|, sum dF^2, 3N (forces), sum |dS|, sum dS^2, 6 (stress; components xx, yy,
// zz, yz, xz, xy).
__global__ void k_metrics(int nframes, const int* fbegin, const double* E, const double* F, const double* V,
                          const double* E0, const double* F0, const double* S0, const int* has, double* out) {
  const int f = blockIdx.x;
  if (f >= nframes) return;
  const int a0 = fbegin[f], a1 = fbegin[f + 1], n = a1 - a0;
  __shared__ double red[2][256];
  double fa = 0.0, fs = 0.0;
  if (has[f] & 2)
    for (int i = a0 + threadIdx.x; i < a1; i += blockDim.x)
      for (int q = 0; q < 3; ++q) {
        const double d = F[3 * static_cast<size_t>(i) + q] - F0[3 * static_cast<size_t>(i) + q];
        fa += fabs(d);
        fs += d * d;
      }
  red[0][threadIdx.x] = fa;
  red[1][threadIdx.x] = fs;
  __syncthreads();
  for (int st = blockDim.x / 2; st > 0; st >>= 1) {
    if (threadIdx.x < st) {
      red[0][threadIdx.x] += red[0][threadIdx.x + st];
      red[1][threadIdx.x] += red[1][threadIdx.x + st];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    double* o = out + 9 * static_cast<size_t>(f);
    for (int q = 0; q < 9; ++q) o[q] = 0.0;
    if ((has[f] & 1) && n > 0) {
      const double d = E0[f] - E[f];
      o[0] = fabs(d);
      o[1] = d * d / n;
      o[2] = n;
    }
    if (has[f] & 2) {
      o[3] = red[0][0];
      o[4] = red[1][0];
      o[5] = 3.0 * n;
    }
    if (has[f] & 4) {
      const double* v = V + 6 * f;  // (xx, yy, zz, xy, xz, yz)
      const double* s0 = S0 + 9 * f;
      const double d[6] = {v[0] - s0[0], v[1] - s0[4], v[2] - s0[8], v[5] - s0[5], v[4] - s0[2], v[3] - s0[1]};
      for (int q = 0; q < 6; ++q) { o[6] += fabs(d[q]); o[7] += d[q] * d[q]; }
      o[8] = 6.0;
    }
  }
}

// ---- linear warm-up (MTPR_trainer::TrainLinear, dev_src/mtpr_trainer.cpp:1455) ------------------
// Row layout of the component matrix cm[rows][ncol]: energy rows [0, K), force rows
// [K, K + 3N) in atom order, stress rows [K + 3N, K + 3N + 9K) (a, b row-major per frame).
// Row weights and right-hand sides follow AddToSLAE (mtpr_trainer.cpp:1130-1453).
__global__ void k_lin_rows(int nframes, const int* fbegin, const double* E0, const double* F0, const double* S0,
                           const int* has, LossConfig c, int natoms, double* alpha, double* rhs) {
  const int f = blockIdx.x;
  if (f >= nframes) return;
  const int a0 = fbegin[f], a1 = fbegin[f + 1], n = a1 - a0;
  __shared__ double red[256];
  double avef = 0.0;
  for (int i = a0 + threadIdx.x; i < a1; i += blockDim.x)
    for (int q = 0; q < 3; ++q) avef += F0[3 * static_cast<size_t>(i) + q] * F0[3 * static_cast<size_t>(i) + q];
  red[threadIdx.x] = avef;
  __syncthreads();
  for (int st = blockDim.x / 2; st > 0; st >>= 1) {
    if (threadIdx.x < st) red[threadIdx.x] += red[threadIdx.x + st];
    __syncthreads();
  }
  avef = (has[f] & 2) && n > 0 ? red[0] / n : 0.0;
  const double d = 0.1, scale = d / (d + c.norm_by_forces * avef);
  double we = n > 0 ? c.wE / n : 0.0, wf = c.wF, ws = n > 0 ? c.wS / n : 0.0;
  if (c.weighting == 1 && n > 0) { we /= n; ws /= n; wf /= n; }
  else if (c.weighting == 2) { we *= n; ws *= n; }
  const size_t fr0 = static_cast<size_t>(nframes), sr0 = fr0 + 3 * static_cast<size_t>(natoms);
  if (threadIdx.x == 0) {
    alpha[f] = (has[f] & 1) ? we * scale : 0.0;
    rhs[f] = E0[f];
    for (int q = 0; q < 9; ++q) {
      alpha[sr0 + 9 * f + q] = (c.wS > 0 && (has[f] & 4)) ? ws : 0.0;
      rhs[sr0 + 9 * f + q] = S0[9 * f + q];
    }
  }
  for (int i = a0 + threadIdx.x; i < a1; i += blockDim.x)
    for (int q = 0; q < 3; ++q) {
      const size_t r = fr0 + 3 * static_cast<size_t>(i) + q;
      alpha[r] = (c.wF > 0 && (has[f] & 2)) ? wf * scale : 0.0;
      rhs[r] = F0[3 * static_cast<size_t>(i) + q];
    }
}

// species columns: the frame's count of type t in the energy row (force and stress rows 0)
__global__ void k_lin_species(int nframes, const int* fbegin, const int* types, int C, int ncol, double* cm) {
  const int f = blockIdx.x;
  if (f >= nframes || threadIdx.x >= C) return;
  int count = 0;
  for (int i = fbegin[f]; i < fbegin[f + 1]; ++i) count += types[i] == static_cast<int>(threadIdx.x);
  cm[static_cast<size_t>(f) * ncol + threadIdx.x] = count;
}

// column col from one evaluation: energies, forces, and the virial as a symmetric 3x3
__global__ void k_lin_column(int nframes, int natoms, const double* E, const double* F, const double* V, int ncol,
                             int col, double* cm) {
  const long long t = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
  const long long rows = nframes + 3LL * natoms + 9LL * nframes;
  if (t >= rows) return;
  double v;
  if (t < nframes) {
    v = E[t];
  } else if (t < nframes + 3LL * natoms) {
    v = F[t - nframes];
  } else {
    const long long u = t - nframes - 3LL * natoms;
    const int f = static_cast<int>(u / 9), ab = static_cast<int>(u - 9LL * f);
    const double* w = V + 6 * static_cast<size_t>(f);  // (xx, yy, zz, xy, xz, yz)
    const int map[9] = {0, 3, 4, 3, 1, 5, 4, 5, 2};
    v = w[map[ab]];
  }
  cm[static_cast<size_t>(t) * ncol + col] = v;
}

// A[j][k] = sum_r alpha_r cm[r][j] cm[r][k] (k >= j) and b[j] = sum_r alpha_r rhs_r cm[r][j]: one block
// per output, rows strided over the threads, fixed-order tree (deterministic).  Block index
// < npairs: pair (j, k) in row-major upper-triangle order; then the ncol entries of b.
__global__ void k_lin_normal(long long rows, int ncol, const double* cm, const double* alpha, const double* rhs,
                             double* A, double* b) {
  __shared__ double red[256];
  const int npairs = ncol * (ncol + 1) / 2;
  const int o = blockIdx.x;
  int j = 0, k = -1;
  if (o < npairs) {
    int rem = o;
    while (rem >= ncol - j) { rem -= ncol - j; ++j; }
    k = j + rem;
  } else {
    j = o - npairs;
  }
  double s = 0.0;
  for (long long r = threadIdx.x; r < rows; r += blockDim.x) {
    const double a = alpha[r];
    if (a == 0.0) continue;
    const double x = cm[static_cast<size_t>(r) * ncol + j];
    s += k >= 0 ? a * x * cm[static_cast<size_t>(r) * ncol + k] : a * rhs[r] * x;
  }
  red[threadIdx.x] = s;
  __syncthreads();
  for (int st = blockDim.x / 2; st > 0; st >>= 1) {
    if (threadIdx.x < st) red[threadIdx.x] += red[threadIdx.x + st];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    if (k >= 0) A[static_cast<size_t>(j) * ncol + k] = red[0];
    else b[j] = red[0];
  }
}

// loss = sum_f loss_f / K (fixed order), grad /= K
__global__ void k_loss_finish(int nframes, const double* loss_f, double* loss, double* grad, int nparams) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const double inv = nframes > 0 ? 1.0 / nframes : 0.0;
  if (t == 0) {
    double s = 0.0;
    for (int f = 0; f < nframes; ++f) s += loss_f[f];
    *loss = s * inv;
  }
  if (t < nparams) grad[t] *= inv;
}

// y = A x for a symmetric n x n matrix (row-major), one warp per row.
__global__ void k_symv(int n, const double* A, const double* x, double alpha, double* y) {
  const int row = static_cast<int>((static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x) / kWarp);
  const int lane = threadIdx.x & 31;
  if (row >= n) return;
  double s = 0.0;
  const double* a = A + static_cast<size_t>(row) * n;
  for (int j = lane; j < n; j += kWarp) s += a[j] * x[j];
  s = warp_sum(s);
  if (lane == 0) y[row] = alpha * s;
}

// Fixed-order dot products: out[0] = x . y (one block).
__global__ void k_dot(int n, const double* x, const double* y, double* out) {
  __shared__ double red[256];
  double s = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) s += x[i] * y[i];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int st = blockDim.x / 2; st > 0; st >>= 1) {
    if (threadIdx.x < st) red[threadIdx.x] += red[threadIdx.x + st];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = red[0];
}

// H <- H - rho (Hy s^T + s Hy^T) + (rho^2 y^T H y + rho) s s^T
__global__ void k_bfgs_update(int n, double* H, const double* s, const double* Hy, double rho, double yHy) {
  const long long t = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (t >= static_cast<long long>(n) * n) return;
  const int i = static_cast<int>(t / n), j = static_cast<int>(t - static_cast<long long>(i) * n);
  H[t] += -rho * (Hy[i] * s[j] + s[i] * Hy[j]) + (rho * rho * yHy + rho) * s[i] * s[j];
}

// H <- H + a p p^T + b (p c^T + c p^T)  (UpdateInvHess's three rank-1 updates, bfgs.cpp:470-490)
__global__ void k_bfgs_rank2(int n, double* H, const double* p, const double* c, double a, double b) {
  const long long t = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (t >= static_cast<long long>(n) * n) return;
  const int i = static_cast<int>(t / n), j = static_cast<int>(t - static_cast<long long>(i) * n);
  H[t] += a * p[i] * p[j] + b * (p[i] * c[j] + c[i] * p[j]);
}

__global__ void k_scaled_identity(int n, double* H, double diag) {
  const long long t = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (t >= static_cast<long long>(n) * n) return;
  const int i = static_cast<int>(t / n), j = static_cast<int>(t - static_cast<long long>(i) * n);
  H[t] = i == j ? diag : 0.0;
}

__global__ void k_diagonal_matrix(int n, double* H, const double* diag) {
  const long long t = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (t >= static_cast<long long>(n) * n) return;
  const int i = static_cast<int>(t / n), j = static_cast<int>(t - static_cast<long long>(i) * n);
  H[t] = i == j ? diag[i] : 0.0;
}

__global__ void k_axpy_to(int n, const double* x, double a, const double* p, double* out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = x[i] + a * p[i];
}

__global__ void k_sub(int n, const double* a, const double* b, double* out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = a[i] - b[i];
}

}  // namespace

// One-dimensional search along the BFGS direction in reverse communication, with the decision rules
// of the reference's Linesearch (src/common/bfgs.h:31-290): iterate(f, g) takes the objective and
// its slope at the trial x and sets the next trial.  (lx, lf, lg) is the left bracket end, (rx, rf,
// rg) the right one, (px, pf, pg) the previous trial.  The rules are kept exactly so that the trial
// sequence is the reference's; oracle/oracle.py (RefLineSearch) restates the same rules.
struct RefLineSearch {
  static constexpr double kHuge = 9.9e99;          // HUGE_DOUBLE (src/common/utils.h:24)
  static constexpr double kRightSentinel = 9e99;   // the value bfgs.h:165 compares right_f with
  double x = 0, lx = 0, lf = 0, lg = 0, rx = 1, rf = kHuge, rg = kHuge, px = 0, pf = 0, pg = 0;
  bool stagnated = false;

  void reset(double step = 1.0) {
    stagnated = false;
    x = lx = 0.0;
    rx = step;
    rf = rg = kHuge;
  }
  void reduce_step(double ratio) { x = px + ratio * (x - px); }
  void to_prev(double f, double g) { px = x; pf = f; pg = g; }
  double tolerance() const {
    const double scale = std::max({1.0, std::abs(lx), std::abs(x), std::abs(rx), std::abs(px)});
    return 64.0 * std::numeric_limits<double>::epsilon() * scale;
  }
  double best(double f) const {
    double bx = x, bf = f;
    if (lf < bf) { bx = lx; bf = lf; }
    if (rf < bf) bx = rx;
    return bx;
  }
  bool recover(double f, double g, double tol) {
    if (!(lx < rx)) return false;
    double r = 0.5 * (lx + rx);
    if (std::abs(r - x) <= tol) {
      if (x > lx) {
        const double t = std::nextafter(x, lx);
        if (t != x && t >= lx) r = t;
      }
      if (std::abs(r - x) <= tol && x < rx) {
        const double t = std::nextafter(x, rx);
        if (t != x && t <= rx) r = t;
      }
    }
    if (std::abs(r - x) <= tol) return false;
    to_prev(f, g);
    x = r;
    return true;
  }
  void iterate(double f, double g) {
    if (x == 0) {
      lx = x; lf = f; lg = g;
      if (g > 0) throw Error(5, "BFGS: line search along an increasing direction");
      to_prev(f, g);
      x = rx;
      return;
    }
    const double tol = tolerance();
    if (std::abs(px - x) <= tol) {
      if (recover(f, g, tol)) return;
      if (rx - lx <= tol) {
        stagnated = true;
        x = best(f);
        return;
      }
      throw Error(5, "BFGS: line search stagnated without a distinct step");
    }
    if (x == rx || (x > lx && rf == kRightSentinel)) { rx = x; rf = f; rg = g; }
    if (rg < 0 && rf < lf) {
      if (x > rx) {
        lx = rx; lf = rf; lg = rg;
        rx = x; rf = f; rg = g;
      }
    } else {
      if (g < 0 && f < lf && x > lx) {
        if (x > rx) {
          if (f > rf) {
            to_prev(f, g);
            lx = rx; lf = rf; lg = rg;
            rx = x; rf = f; rg = g;
            x = 0.5 * (lx + rx);
            return;
          }
          rx = x; rf = f; rg = g;
        } else {
          lx = x; lf = f; lg = g;
        }
      }
      if (g > 0 && x < rx) { rx = x; rf = f; rg = g; }
    }
    if (f > lf + 0.1 * lg * (x - lx)) {
      // insufficient decrease: minimiser of a parabola fitted to log(f - f_lin)
      const double slope = -lg * (x - lx), arg = f - lf + slope;
      double nx = lx + 0.5 * (x - lx);
      if (slope > 0.0 && arg > 0.0 && std::isfinite(slope) && std::isfinite(arg)) {
        const double f0 = std::log(slope), g0 = lg / slope, f1 = std::log(arg);
        const double den = f1 - f0 - g0 * (x - lx);
        if (std::isfinite(den) && den != 0.0) nx = lx - 0.5 * g0 * (x - lx) * (x - lx) / den;
      }
      if (nx > rx && rg > 0) nx = lx + 0.5 * (x - lx);
      else if ((nx - lx > 3.0 * rx - 2.0 * lx) && rg < 0) nx = lx + 3.0 * (rx - lx);
      if (!std::isfinite(nx)) nx = lx + 0.5 * (x - lx);
      to_prev(f, g);
      x = nx;
      return;
    }
    if ((g - pg) / (x - px) < 0.0) {
      // negative curvature along the line
      const double nx = rg < 0 ? 3 * rx - 2 * lx : x + 0.5 * (rx - x);
      to_prev(f, g);
      x = nx;
      return;
    }
    // secant step on the slopes
    double nx = x - g * (x - px) / (g - pg);
    if (!std::isfinite(nx)) nx = lx + 0.5 * (rx - lx);
    to_prev(f, g);
    x = nx;
    if (x > rx) {
      if (rg > 0) x = 0.5 * lx + 0.5 * rx;
      else if (x > 3 * rx - 2 * lx) x = 3 * rx - 2 * lx;
      return;
    }
    if (x < lx) {
      to_prev(f, g);
      x = 0.5 * lx + 0.5 * rx;
    }
  }
};

class Trainer {
 public:
  Trainer(Engine& eng, int nframes, const int* natoms, const double* cells, const double* pos, const int* types,
          const double* E0, const double* F0, const double* S0, const int* has, LossConfig cfg)
      : eng_(eng), nframes_(nframes), cfg_(cfg) {
    cudaStream_t s = eng_.stream();
    long long n = 0;
    fbegin_host_.push_back(0);
    for (int f = 0; f < nframes; ++f) { n += natoms[f]; fbegin_host_.push_back(static_cast<int>(n)); }
    natoms_ = static_cast<int>(n);
    nparams_ = eng_.model().param_count();
    natoms_list_.assign(natoms, natoms + nframes);
    cells_.assign(cells, cells + 9 * nframes);
    // host copies: the rescale step builds a trainer on a subset of the frames
    pos_h_.assign(pos, pos + 3 * static_cast<size_t>(n));
    types_h_.assign(types, types + n);
    E0_h_.assign(E0, E0 + nframes);
    F0_h_.assign(F0, F0 + 3 * static_cast<size_t>(n));
    S0_h_.assign(S0, S0 + 9 * static_cast<size_t>(nframes));
    has_h_.assign(has, has + nframes);
    pos_.ensure(sizeof(double) * 3 * std::max(1, natoms_));
    types_.ensure(sizeof(int) * std::max(1, natoms_));
    E0_.ensure(sizeof(double) * std::max(1, nframes));
    F0_.ensure(sizeof(double) * 3 * std::max(1, natoms_));
    S0_.ensure(sizeof(double) * 9 * std::max(1, nframes));
    has_.ensure(sizeof(int) * std::max(1, nframes));
    fbegin_.ensure(sizeof(int) * (nframes + 1));
    TRAIN_CUDA(cudaMemcpyAsync(pos_.ptr, pos, sizeof(double) * 3 * natoms_, cudaMemcpyHostToDevice, s));
    TRAIN_CUDA(cudaMemcpyAsync(types_.ptr, types, sizeof(int) * natoms_, cudaMemcpyHostToDevice, s));
    TRAIN_CUDA(cudaMemcpyAsync(E0_.ptr, E0, sizeof(double) * nframes, cudaMemcpyHostToDevice, s));
    TRAIN_CUDA(cudaMemcpyAsync(F0_.ptr, F0, sizeof(double) * 3 * natoms_, cudaMemcpyHostToDevice, s));
    TRAIN_CUDA(cudaMemcpyAsync(S0_.ptr, S0, sizeof(double) * 9 * nframes, cudaMemcpyHostToDevice, s));
    TRAIN_CUDA(cudaMemcpyAsync(has_.ptr, has, sizeof(int) * nframes, cudaMemcpyHostToDevice, s));
    TRAIN_CUDA(cudaMemcpyAsync(fbegin_.ptr, fbegin_host_.data(), sizeof(int) * (nframes + 1), cudaMemcpyHostToDevice, s));
    // predictions and loss derivatives
    E_.ensure(sizeof(double) * std::max(1, nframes));
    F_.ensure(sizeof(double) * 3 * std::max(1, natoms_));
    V_.ensure(sizeof(double) * 6 * std::max(1, nframes));
    ew_.ensure(sizeof(double) * std::max(1, natoms_));
    fw_.ensure(sizeof(double) * 3 * std::max(1, natoms_));
    sw_.ensure(sizeof(double) * 9 * std::max(1, nframes));
    lossf_.ensure(sizeof(double) * std::max(1, nframes));
    loss_.ensure(sizeof(double) * 8);
    grad_.ensure(sizeof(double) * nparams_);
    const Model& m = eng_.model();
    gatex_ = cfg_.gate_x_l2 > 0.0 && m.gated && natoms_ > 0;
    if (gatex_) {
      if (m.C > 64) throw Error(1, "gate-x term: more than 64 species");
      extra_h_.ensure(sizeof(double) * static_cast<size_t>(natoms_) * m.F);
      agrad_.ensure(sizeof(double) * static_cast<size_t>(std::max(1, nframes)) * m.C * m.F);
    }
    TRAIN_CUDA(cudaMallocHost(&host_scalars_, sizeof(double) * 8));
    bind_edges();
  }

  // The edge set of the fixed frames is built once, and again only when the engine was used for
  // other geometry in between (which also invalidates a captured graph).
  void bind_edges() {
    if (graph_exec_) { cudaGraphExecDestroy(graph_exec_); graph_exec_ = nullptr; }
    if (graph_) { cudaGraphDestroy(graph_); graph_ = nullptr; }
    for (int attempt = 0;; ++attempt) {
      try {
        eng_.build_edges(nframes_, natoms_list_.data(), cells_.data(), pos_.as<double>(), types_.as<int>());
        eng_.check_device_error();
        break;
      } catch (const EdgeOverflow&) {
        if (attempt >= 4) throw;  // the capacity has been grown: build again
      }
    }
    generation_ = eng_.edge_generation();
  }

  ~Trainer() {
    if (graph_exec_) cudaGraphExecDestroy(graph_exec_);
    if (graph_) cudaGraphDestroy(graph_);
    if (host_scalars_) cudaFreeHost(host_scalars_);
  }

  void set_graph(bool on) { use_graph_ = on; }
  int nparams() const { return nparams_; }

  // Enqueues E/F/virial, loss, gradient on the engine stream (device results in loss_/grad_).
  void enqueue_eval() {
    cudaStream_t s = eng_.stream();
    eng_.efs(E_.as<double>(), F_.as<double>(), V_.as<double>(), nullptr);
    if (nframes_)
      k_loss<<<nframes_, 256, 0, s>>>(nframes_, fbegin_.as<int>(), E_.as<double>(), F_.as<double>(), V_.as<double>(),
                                      E0_.as<double>(), F0_.as<double>(), S0_.as<double>(), has_.as<int>(), cfg_,
                                      ew_.as<double>(), fw_.as<double>(), sw_.as<double>(), lossf_.as<double>());
    const Model& m = eng_.model();
    if (gatex_) {
      if (eng_.precision() == kFP32)
        k_gatex_frame<float><<<nframes_, 256, 0, s>>>(nframes_, fbegin_.as<int>(), eng_.d_row(), eng_.d_row_end(),
                                                      types_.as<int>(),
                                                      static_cast<const float*>(eng_.d_gate_signal()),
                                                      static_cast<const float*>(eng_.d_gate_additive()), m.C, m.F,
                                                      cfg_.gate_x_l2, extra_h_.as<double>(), lossf_.as<double>(),
                                                      agrad_.as<double>());
      else
        k_gatex_frame<double><<<nframes_, 256, 0, s>>>(nframes_, fbegin_.as<int>(), eng_.d_row(), eng_.d_row_end(),
                                                       types_.as<int>(),
                                                       static_cast<const double*>(eng_.d_gate_signal()),
                                                       static_cast<const double*>(eng_.d_gate_additive()), m.C, m.F,
                                                       cfg_.gate_x_l2, extra_h_.as<double>(), lossf_.as<double>(),
                                                       agrad_.as<double>());
    }
    TRAIN_CUDA(cudaMemsetAsync(grad_.ptr, 0, sizeof(double) * nparams_, s));
    if (natoms_)
      eng_.combination_grad(ew_.as<double>(), fw_.as<double>(), sw_.as<double>(), grad_.as<double>(),
                            gatex_ ? extra_h_.as<double>() : nullptr);
    if (gatex_)
      k_gatex_alpha<<<(m.C * m.F + 255) / 256, 256, 0, s>>>(nframes_, m.C * m.F, agrad_.as<double>(),
                                                           grad_.as<double>() + eng_.gate_additive_offset());
    k_loss_finish<<<(nparams_ + 255) / 256, 256, 0, s>>>(nframes_, lossf_.as<double>(), loss_.as<double>(),
                                                         grad_.as<double>(), nparams_);
  }

  // Loss and gradient at the parameters already in the engine; results stay on the device.
  void eval_device() {
    if (eng_.edge_generation() != generation_) bind_edges();
    cudaStream_t s = eng_.stream();
    if (!use_graph_) {
      enqueue_eval();
      return;
    }
    if (!graph_exec_) {
      enqueue_eval();  // first evaluation runs eagerly (sizes buffers, configures kernels)
      TRAIN_CUDA(cudaStreamSynchronize(s));
      TRAIN_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeRelaxed));
      enqueue_eval();
      TRAIN_CUDA(cudaStreamEndCapture(s, &graph_));
      TRAIN_CUDA(cudaGraphInstantiate(&graph_exec_, graph_, 0));
      ++graph_builds_;
      return;
    }
    TRAIN_CUDA(cudaGraphLaunch(graph_exec_, s));
  }

  double loss_grad(const double* params, double* grad_host) {
    eng_.set_params(params);
    eval_device();
    cudaStream_t s = eng_.stream();
    TRAIN_CUDA(cudaMemcpyAsync(host_scalars_, loss_.ptr, sizeof(double), cudaMemcpyDeviceToHost, s));
    if (grad_host) TRAIN_CUDA(cudaMemcpyAsync(grad_host, grad_.ptr, sizeof(double) * nparams_, cudaMemcpyDeviceToHost, s));
    TRAIN_CUDA(cudaStreamSynchronize(s));
    eng_.check_device_error();
    return host_scalars_[0];
  }

  // Dense BFGS on the device (BFGS::Iterate / UpdateInvHess, src/common/bfgs.cpp:251-329, 428-502):
  // H starts at the identity, or at the diagonal given by set_inv_hess_diagonal (BFGS::Restart and
  // SetInvHessDiagonal, bfgs.cpp:529-534, bfgs.h:395); p = -H g; a trial x + a p is accepted when
  // the strong Wolfe conditions f <= f0 + c1 a p.g0 and |p.g| <= c2 |p.g0| hold (c1 = 0.1, c2 = 0.5,
  // bfgs.h:384-385), then H takes the rank-2 update with s = a p, y = g - g0, skipped while
  // s.y <= 64 eps.  params (host) in/out; history[max_iter + 1] receives the loss at the start and
  // after each accepted step.  Returns the number of accepted steps; ends early when |g| <= gtol at
  // an accepted point, or when a line search stagnates or runs more than 30 trials (the trainer's
  // stop rule, dev_src/mtpr_trainer.cpp:5328-5333), keeping the last accepted point.
  //
  // Line searches (set_line_search):
  //   kLineSearchReference (default): the reference's Linesearch in reverse communication
  //     (RefLineSearch above), one objective evaluation per BFGS::Iterate call, non-finite
  //     trials backed off by a quarter (ReduceStep(0.25)); every evaluated trial point and its
  //     loss are recorded (trials()).
  //   kLineSearchInterpolating: a bracketing search that interpolates -- lo = the last trial with
  //     sufficient decrease and a negative slope (initially a = 0), hi = the first trial past the
  //     minimum:
  //   * sufficient decrease fails: hi = a; next = the minimiser of the parabola through f(lo),
  //     the slope at lo and f(a), kept within lo + [0.01, 0.5] (a - lo); a non-finite loss takes
  //     a quarter of the step;
  //   * slope still negative and steep: lo = a; inside a bracket as below, else the zero of the
  //     secant through the slopes at the previous lo and a, kept within [2a, 8a];
  //   * slope positive and steep: hi = a; next = the zero of the secant through the slopes at lo
  //     and hi, kept within lo + [0.1, 0.9] (hi - lo) (the parabola again when hi failed the
  //     decrease test).
  //   It takes fewer evaluations per accepted step on the benchmark sets (3.3 on the L5 set) but
  //   does not reproduce the reference's trial sequence.
  void set_inv_hess_diagonal(const double* diag, int n) { h0_diag_.assign(diag, diag + n); }
  enum : int { kLineSearchReference = 0, kLineSearchInterpolating = 1 };
  void set_line_search(int mode) {
    if (mode != kLineSearchReference && mode != kLineSearchInterpolating) throw Error(1, "unknown line search");
    line_search_ = mode;
  }
  // evaluated trial points of the last bfgs call: losses, points [count][nparams], accepted flags
  const std::vector<double>& trial_loss() const { return trial_f_; }
  const std::vector<double>& trial_x() const { return trial_x_; }
  const std::vector<int>& trial_accepted() const { return trial_acc_; }

  int bfgs(double* params, int max_iter, double gtol, double* history) {
    trial_f_.clear();
    trial_x_.clear();
    trial_acc_.clear();
    return line_search_ == kLineSearchReference ? bfgs_reference(params, max_iter, gtol, history)
                                                : bfgs_interpolating(params, max_iter, gtol, history);
  }

  int bfgs_reference(double* params, int max_iter, double gtol, double* history) {
    const int n = nparams_;
    cudaStream_t s = eng_.stream();
    DevBuf H, x, xs, gs, p, dg, yC, sc, dgn;
    H.ensure(sizeof(double) * static_cast<size_t>(n) * n);
    for (DevBuf* b : {&x, &xs, &gs, &p, &dg, &yC}) b->ensure(sizeof(double) * n);
    sc.ensure(sizeof(double) * 8);
    const unsigned nn_blocks = static_cast<unsigned>((static_cast<long long>(n) * n + 255) / 256);
    const unsigned n_blocks = static_cast<unsigned>((n + 255) / 256);
    const unsigned row_blocks = static_cast<unsigned>((static_cast<long long>(n) * kWarp + 255) / 256);
    const double* g = grad_.as<double>();  // gradient of the last evaluation
    auto dot = [&](const double* a, const double* b) {
      k_dot<<<1, 256, 0, s>>>(n, a, b, sc.as<double>());
      TRAIN_CUDA(cudaMemcpyAsync(host_scalars_ + 1, sc.ptr, sizeof(double), cudaMemcpyDeviceToHost, s));
      TRAIN_CUDA(cudaStreamSynchronize(s));
      return host_scalars_[1];
    };
    std::vector<double> xh(params, params + n);
    // Set_x: p = 0, x_start = x, g_start = 0, f_start = p.g_start = HUGE, fresh line search
    TRAIN_CUDA(cudaMemcpyAsync(x.ptr, xh.data(), sizeof(double) * n, cudaMemcpyHostToDevice, s));
    TRAIN_CUDA(cudaMemcpyAsync(xs.ptr, x.ptr, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
    TRAIN_CUDA(cudaMemsetAsync(p.ptr, 0, sizeof(double) * n, s));
    TRAIN_CUDA(cudaMemsetAsync(gs.ptr, 0, sizeof(double) * n, s));
    if (static_cast<int>(h0_diag_.size()) == n && n) {
      dgn.ensure(sizeof(double) * n);
      TRAIN_CUDA(cudaMemcpyAsync(dgn.ptr, h0_diag_.data(), sizeof(double) * n, cudaMemcpyHostToDevice, s));
      k_diagonal_matrix<<<nn_blocks, 256, 0, s>>>(n, H.as<double>(), dgn.as<double>());
    } else {
      k_scaled_identity<<<nn_blocks, 256, 0, s>>>(n, H.as<double>(), 1.0);
    }
    const double c1 = 0.1, c2 = 0.5, floor = 64.0 * std::numeric_limits<double>::epsilon();
    double f_start = RefLineSearch::kHuge, pg_start = RefLineSearch::kHuge;
    RefLineSearch ls;
    std::vector<double> accepted_x(xh);
    int accepted = -1, trials_since = 0;
    // the trial x = x_start + a p, built on the device and read back for the parameter upload
    auto next_trial = [&]() {
      k_axpy_to<<<n_blocks, 256, 0, s>>>(n, xs.as<double>(), ls.x, p.as<double>(), x.as<double>());
      TRAIN_CUDA(cudaMemcpyAsync(xh.data(), x.ptr, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
      TRAIN_CUDA(cudaStreamSynchronize(s));
    };
    while (accepted < max_iter) {
      const double f = loss_grad(xh.data(), nullptr);
      trial_f_.push_back(f);
      trial_x_.insert(trial_x_.end(), xh.begin(), xh.end());
      trial_acc_.push_back(0);
      const double gg = dot(g, g);
      if (!std::isfinite(f) || !std::isfinite(gg)) {
        // a non-finite trial inside a line search backs off (BFGS::Iterate, bfgs.cpp:257-268)
        if (ls.x == 0.0) throw Error(5, "BFGS: non-finite loss or gradient at an accepted point");
        if (++trials_since > 30) break;
        ls.reduce_step(0.25);
        next_trial();
        continue;
      }
      const double pg = dot(g, p.as<double>());
      if (f > f_start + c1 * ls.x * pg_start || std::abs(pg) > c2 * std::abs(pg_start)) {
        ls.iterate(f, pg);
        if (ls.stagnated || ++trials_since > 30) break;
        next_trial();
        continue;
      }
      // accepted: UpdateInvHess (bfgs.cpp:428-502) with the step a p of the finished line search
      trial_acc_.back() = 1;
      accepted_x = xh;
      ++accepted;
      trials_since = 0;
      if (history) history[accepted] = f;
      if (accepted == max_iter || !(std::sqrt(gg) > gtol)) break;
      const double alpha = ls.x;
      k_sub<<<n_blocks, 256, 0, s>>>(n, g, gs.as<double>(), dg.as<double>());
      const double py = alpha * dot(p.as<double>(), dg.as<double>());
      if (!std::isfinite(py)) throw Error(5, "BFGS: non-finite curvature in the inverse-Hessian update");
      if (py > floor) {
        k_symv<<<row_blocks, 256, 0, s>>>(n, H.as<double>(), dg.as<double>(), 1.0, yC.as<double>());
        const double yCy = dot(yC.as<double>(), dg.as<double>());
        if (!std::isfinite(yCy)) throw Error(5, "BFGS: non-finite yHy in the inverse-Hessian update");
        const double foo = (py + yCy) / (py * py);
        if (std::isfinite(foo))
          k_bfgs_rank2<<<nn_blocks, 256, 0, s>>>(n, H.as<double>(), p.as<double>(), yC.as<double>(), alpha * alpha * foo,
                                                 -alpha / py);
      }
      // FormDenseDirection, a fresh line search from this point (SetStart)
      k_symv<<<row_blocks, 256, 0, s>>>(n, H.as<double>(), g, -1.0, p.as<double>());
      const double pgn = dot(g, p.as<double>());
      if (!std::isfinite(pgn)) throw Error(5, "BFGS: non-finite directional derivative");
      ls.reset();
      TRAIN_CUDA(cudaMemcpyAsync(xs.ptr, x.ptr, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
      TRAIN_CUDA(cudaMemcpyAsync(gs.ptr, g, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
      f_start = f;
      pg_start = pgn;
      if (pgn > 0) throw Error(5, "BFGS: search direction is not a descent direction");
      ls.iterate(f, pgn);
      next_trial();
    }
    std::copy(accepted_x.begin(), accepted_x.end(), params);
    eng_.set_params(params);
    return std::max(0, accepted);
  }

  int bfgs_interpolating(double* params, int max_iter, double gtol, double* history) {
    const int n = nparams_;
    cudaStream_t s = eng_.stream();
    DevBuf H, x, g, p, xn, gn, sv, yv, Hy, sc, dg;
    H.ensure(sizeof(double) * static_cast<size_t>(n) * n);
    for (DevBuf* b : {&x, &g, &p, &xn, &gn, &sv, &yv, &Hy}) b->ensure(sizeof(double) * n);
    sc.ensure(sizeof(double) * 8);
    const unsigned nn_blocks = static_cast<unsigned>((static_cast<long long>(n) * n + 255) / 256);
    const unsigned n_blocks = static_cast<unsigned>((n + 255) / 256);
    const unsigned row_blocks = static_cast<unsigned>((static_cast<long long>(n) * kWarp + 255) / 256);
    std::vector<double> xh(params, params + n);
    auto dot = [&](const double* a, const double* b) {
      k_dot<<<1, 256, 0, s>>>(n, a, b, sc.as<double>());
      TRAIN_CUDA(cudaMemcpyAsync(host_scalars_ + 1, sc.ptr, sizeof(double), cudaMemcpyDeviceToHost, s));
      TRAIN_CUDA(cudaStreamSynchronize(s));
      return host_scalars_[1];
    };
    double f = loss_grad(xh.data(), nullptr);
    TRAIN_CUDA(cudaMemcpyAsync(x.ptr, xh.data(), sizeof(double) * n, cudaMemcpyHostToDevice, s));
    TRAIN_CUDA(cudaMemcpyAsync(g.ptr, grad_.ptr, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
    if (static_cast<int>(h0_diag_.size()) == n && n) {
      dg.ensure(sizeof(double) * n);
      TRAIN_CUDA(cudaMemcpyAsync(dg.ptr, h0_diag_.data(), sizeof(double) * n, cudaMemcpyHostToDevice, s));
      k_diagonal_matrix<<<nn_blocks, 256, 0, s>>>(n, H.as<double>(), dg.as<double>());
    } else {
      k_scaled_identity<<<nn_blocks, 256, 0, s>>>(n, H.as<double>(), 1.0);
    }
    if (history) history[0] = f;
    int accepted = 0;
    const double c1 = 0.1, c2 = 0.5, floor = 64.0 * 2.220446049250313e-16;
    for (int it = 0; it < max_iter; ++it) {
      if (!(std::sqrt(dot(g.as<double>(), g.as<double>())) > gtol)) break;
      k_symv<<<row_blocks, 256, 0, s>>>(n, H.as<double>(), g.as<double>(), -1.0, p.as<double>());
      const double gp = dot(g.as<double>(), p.as<double>());
      if (!(gp < 0)) throw Error(5, "BFGS: search direction is not a descent direction");
      double alpha = 1.0, fn = f;
      double lo = 0.0, f_lo = f, g_lo = gp;             // bracket start: sufficient decrease, slope < 0
      double hi = -1.0, f_hi = 0.0, g_hi = 0.0;         // bracket end (hi < 0: none yet)
      bool hi_failed = false;                            // hi failed the sufficient-decrease test
      bool ok = false;
      // the parabola through f(lo), the slope at lo and f(b), minimised, within lo + [0.01, 0.5] (b - lo)
      auto parabola = [&](double b, double fb) {
        const double d = b - lo, den = 2.0 * (fb - f_lo - g_lo * d);
        if (!std::isfinite(fb)) return lo + 0.25 * d;
        double t = den > 0 ? lo - g_lo * d * d / den : lo + 0.5 * d;
        if (!std::isfinite(t)) t = lo + 0.5 * d;
        return std::min(std::max(t, lo + 0.01 * d), lo + 0.5 * d);
      };
      // the zero of the secant through the slopes at lo and hi, within lo + [0.1, 0.9] (hi - lo)
      auto secant = [&]() {
        const double d = hi - lo;
        double t = g_hi > g_lo ? lo - g_lo * d / (g_hi - g_lo) : lo + 0.5 * d;
        if (!std::isfinite(t)) t = lo + 0.5 * d;
        return std::min(std::max(t, lo + 0.1 * d), lo + 0.9 * d);
      };
      for (int ls = 0; ls < 31; ++ls) {
        k_axpy_to<<<n_blocks, 256, 0, s>>>(n, x.as<double>(), alpha, p.as<double>(), xn.as<double>());
        TRAIN_CUDA(cudaMemcpyAsync(xh.data(), xn.ptr, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
        TRAIN_CUDA(cudaStreamSynchronize(s));
        fn = loss_grad(xh.data(), nullptr);
        TRAIN_CUDA(cudaMemcpyAsync(gn.ptr, grad_.ptr, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
        if (!std::isfinite(fn) || fn > f + c1 * alpha * gp) {
          hi = alpha; f_hi = fn; hi_failed = true;
          alpha = parabola(hi, f_hi);
          continue;
        }
        const double gpn = dot(gn.as<double>(), p.as<double>());
        if (std::abs(gpn) <= c2 * std::abs(gp)) { ok = true; break; }
        if (gpn < 0) {
          const double lo_prev = lo, g_prev = g_lo;
          lo = alpha; f_lo = fn; g_lo = gpn;
          if (hi < 0) {
            double t = gpn > g_prev ? alpha - gpn * (alpha - lo_prev) / (gpn - g_prev) : 4.0 * alpha;
            if (!std::isfinite(t)) t = 4.0 * alpha;
            alpha = std::min(std::max(t, 2.0 * alpha), 8.0 * alpha);
            continue;
          }
        } else {
          hi = alpha; f_hi = fn; g_hi = gpn; hi_failed = false;
        }
        alpha = hi_failed ? parabola(hi, f_hi) : secant();
      }
      if (!ok) break;  // line search exhausted: keep the last accepted point
      k_sub<<<n_blocks, 256, 0, s>>>(n, xn.as<double>(), x.as<double>(), sv.as<double>());
      k_sub<<<n_blocks, 256, 0, s>>>(n, gn.as<double>(), g.as<double>(), yv.as<double>());
      const double ys = dot(yv.as<double>(), sv.as<double>());
      if (std::isfinite(ys) && ys > floor) {
        k_symv<<<row_blocks, 256, 0, s>>>(n, H.as<double>(), yv.as<double>(), 1.0, Hy.as<double>());
        const double yHy = dot(yv.as<double>(), Hy.as<double>());
        if (std::isfinite(yHy))
          k_bfgs_update<<<nn_blocks, 256, 0, s>>>(n, H.as<double>(), sv.as<double>(), Hy.as<double>(), 1.0 / ys, yHy);
      }
      TRAIN_CUDA(cudaMemcpyAsync(x.ptr, xn.ptr, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
      TRAIN_CUDA(cudaMemcpyAsync(g.ptr, gn.ptr, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
      f = fn;
      ++accepted;
      if (history) history[accepted] = f;
    }
    TRAIN_CUDA(cudaMemcpyAsync(params, x.ptr, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
    TRAIN_CUDA(cudaStreamSynchronize(s));
    eng_.set_params(params);
    return accepted;
  }

  // The trainer's error metrics at params (E/F/virial only, no gradient): out6 = energy MAE and
  // RMSE (meV/atom), force MAE and RMSE (meV/A), stress MAE and RMSE (eV); 0 where nothing is
  // labelled.  The per-frame partial sums are added on the host in frame order.
  void metrics(const double* params, double* out6) {
    eng_.set_params(params);
    if (eng_.edge_generation() != generation_) bind_edges();
    cudaStream_t s = eng_.stream();
    eng_.efs(E_.as<double>(), F_.as<double>(), V_.as<double>(), nullptr);
    metric_part_.ensure(sizeof(double) * 9 * std::max(1, nframes_));
    if (nframes_)
      k_metrics<<<nframes_, 256, 0, s>>>(nframes_, fbegin_.as<int>(), E_.as<double>(), F_.as<double>(), V_.as<double>(),
                                         E0_.as<double>(), F0_.as<double>(), S0_.as<double>(), has_.as<int>(),
                                         metric_part_.as<double>());
    std::vector<double> part(9 * static_cast<size_t>(nframes_));
    if (nframes_)
      TRAIN_CUDA(cudaMemcpyAsync(part.data(), metric_part_.ptr, sizeof(double) * part.size(), cudaMemcpyDeviceToHost, s));
    TRAIN_CUDA(cudaStreamSynchronize(s));
    eng_.check_device_error();
    double t[9] = {0};
    for (int f = 0; f < nframes_; ++f)
      for (int q = 0; q < 9; ++q) t[q] += part[9 * static_cast<size_t>(f) + q];
    out6[0] = t[2] > 0 ? 1000.0 * t[0] / t[2] : 0.0;
    out6[1] = t[2] > 0 ? 1000.0 * std::sqrt(t[1] / t[2]) : 0.0;
    out6[2] = t[5] > 0 ? 1000.0 * t[3] / t[5] : 0.0;
    out6[3] = t[5] > 0 ? 1000.0 * std::sqrt(t[4] / t[5]) : 0.0;
    out6[4] = t[8] > 0 ? t[6] / t[8] : 0.0;
    out6[5] = t[8] > 0 ? std::sqrt(t[7] / t[8]) : 0.0;
  }

  // Linear warm-up (MTPR_trainer::TrainLinear): normalise the radial Chebyshev rows
  // (MLMTPR::Orthogonalize, dev_src/mtpr.cpp:14110), build the normal equations of the species
  // constants and the scalar readout from one E/F/virial evaluation per readout column (the model
  // with that readout weight 1, centre factors 1 and no constant), add the 1e-13 ridge, solve by
  // Gaussian elimination (SolveSLAE / SolveSLAEGaussian, mtpr_trainer.cpp:971, 282) and apply:
  // centre factor 1, shift = constant - 1, readout = solution.  params (host) in/out.
  void train_linear(double* params) {
    const Model& m = eng_.model();
    const int C = m.C, S = m.S, B = m.B, F = m.F;
    const int heads = m.species_readout ? C : 1, ncol = C + heads * S;
    int o_shift = -1, o_radial = -1, o_species = -1, o_linear = -1;
    for (const auto& blk : m.layout()) {
      if (blk.name == "shift_coeffs") o_shift = blk.offset;
      else if (blk.name == "radial_coeffs") o_radial = blk.offset;
      else if (blk.name == "species_coeffs") o_species = blk.offset;
      else if (blk.name == "moment_coeffs") o_linear = blk.offset;
    }
    std::vector<double> p(params, params + nparams_);
    for (int mu = 0; mu < F; ++mu) {
      double* row = p.data() + o_radial + static_cast<size_t>(mu) * (B + C);
      double norm = 0.0;
      for (int b = 0; b < B; ++b) norm += row[b] * row[b] + 1e-30;
      norm = std::sqrt(norm);
      for (int b = 0; b < B; ++b) row[b] /= norm;
    }
    if (eng_.edge_generation() != generation_) bind_edges();
    cudaStream_t s = eng_.stream();
    const long long rows = nframes_ + 3LL * natoms_ + 9LL * nframes_;
    lin_cm_.ensure(sizeof(double) * static_cast<size_t>(std::max(1LL, rows)) * ncol);
    lin_alpha_.ensure(sizeof(double) * std::max(1LL, rows));
    lin_rhs_.ensure(sizeof(double) * std::max(1LL, rows));
    lin_A_.ensure(sizeof(double) * ncol * ncol);
    lin_b_.ensure(sizeof(double) * ncol);
    TRAIN_CUDA(cudaMemsetAsync(lin_cm_.ptr, 0, sizeof(double) * static_cast<size_t>(std::max(1LL, rows)) * ncol, s));
    TRAIN_CUDA(cudaMemsetAsync(lin_A_.ptr, 0, sizeof(double) * ncol * ncol, s));
    if (nframes_) {
      k_lin_rows<<<nframes_, 256, 0, s>>>(nframes_, fbegin_.as<int>(), E0_.as<double>(), F0_.as<double>(),
                                          S0_.as<double>(), has_.as<int>(), cfg_, natoms_, lin_alpha_.as<double>(),
                                          lin_rhs_.as<double>());
      k_lin_species<<<nframes_, 64, 0, s>>>(nframes_, fbegin_.as<int>(), types_.as<int>(), C, ncol, lin_cm_.as<double>());
    }
    for (int q = 0; q < heads * S; ++q) {
      std::vector<double> pq(p);
      for (int t = 0; t < C; ++t) { pq[o_species + t] = 1.0; pq[o_shift + t] = -1.0; }
      for (int r = 0; r < heads * S; ++r) pq[o_linear + r] = r == q ? 1.0 : 0.0;
      eng_.set_params(pq.data());
      eng_.efs(E_.as<double>(), F_.as<double>(), V_.as<double>(), nullptr);
      if (rows)
        k_lin_column<<<static_cast<unsigned>((rows + 255) / 256), 256, 0, s>>>(
            nframes_, natoms_, E_.as<double>(), F_.as<double>(), V_.as<double>(), ncol, C + q, lin_cm_.as<double>());
    }
    const int outputs = ncol * (ncol + 1) / 2 + ncol;
    k_lin_normal<<<outputs, 256, 0, s>>>(rows, ncol, lin_cm_.as<double>(), lin_alpha_.as<double>(),
                                         lin_rhs_.as<double>(), lin_A_.as<double>(), lin_b_.as<double>());
    std::vector<double> A(static_cast<size_t>(ncol) * ncol), x(ncol);
    TRAIN_CUDA(cudaMemcpyAsync(A.data(), lin_A_.ptr, sizeof(double) * A.size(), cudaMemcpyDeviceToHost, s));
    TRAIN_CUDA(cudaMemcpyAsync(x.data(), lin_b_.ptr, sizeof(double) * ncol, cudaMemcpyDeviceToHost, s));
    TRAIN_CUDA(cudaStreamSynchronize(s));
    eng_.check_device_error();
    for (int i = 0; i < ncol; ++i) {
      for (int j = i + 1; j < ncol; ++j) A[static_cast<size_t>(j) * ncol + i] = A[static_cast<size_t>(i) * ncol + j];
      A[static_cast<size_t>(i) * ncol + i] += 1e-13 * (1.0 + A[static_cast<size_t>(i) * ncol + i]);
    }
    // Gaussian elimination without pivoting (the reference's solver; the ridged matrix is SPD)
    for (int i = 0; i + 1 < ncol; ++i)
      for (int j = i + 1; j < ncol; ++j) {
        const double ratio = A[static_cast<size_t>(j) * ncol + i] / A[static_cast<size_t>(i) * ncol + i];
        for (int c = i; c < ncol; ++c) A[static_cast<size_t>(j) * ncol + c] -= ratio * A[static_cast<size_t>(i) * ncol + c];
        x[j] -= ratio * x[i];
      }
    for (int i = ncol - 1; i >= 0; --i) {
      double t = x[i];
      for (int j = i + 1; j < ncol; ++j) t -= A[static_cast<size_t>(i) * ncol + j] * x[j];
      x[i] = t / A[static_cast<size_t>(i) * ncol + i];
      if (!std::isfinite(x[i])) throw Error(5, "linear warm-up: singular normal equations");
    }
    for (int t = 0; t < C; ++t) { p[o_species + t] = 1.0; p[o_shift + t] = x[t] - 1.0; }
    for (int q = 0; q < heads * S; ++q) p[o_linear + q] = x[C + q];
    std::copy(p.begin(), p.end(), params);
    eng_.set_params(params);
  }

  // Rescale step before the linear solve (Rescale, dev_src/mlp/mtpr_train.cpp:1504-1748): a search
  // over the model's global radial scaling for which the linear warm-up's scalar-readout
  // coefficients sit at a typical magnitude of 1.  On at most five frames (largest, second largest,
  // median, second smallest, smallest by atom count, BuildRescaleSubsetIndices :646) when the set
  // has more than five, else on all: each trial sets the scaling and runs train_linear; the
  // statistics are the median (upper) and RMS spread of log|c| over readout coefficients |c| > 1e-12
  // (ComputeMomentCoeffStats :279).  Bracket the median log at 0 (halve / double the seed, expand in
  // the improving direction, SelectRescaleExpansionDirection, dev_src/rescale_search.h), refine by
  // secant steps in log scaling (up to 6, tolerance 0.15), then try the refined scaling times
  // 1/1.08, 1/1.03, 1, 1.03, 1.08 and keep the trial with the least spread^2 + 3 median^2
  // (RescaleMetric :309).  params (host, in/out) ends as that trial's coefficients; *scaling is
  // set to its scaling and the engine keeps both.  Returns the number of linear solves.
  int rescale(double* params, double* scaling_out) {
    const Model& m = eng_.model();
    const int C = m.C, heads = m.species_readout ? C : 1, nread = heads * m.S;
    int o_linear = -1;
    for (const auto& blk : m.layout())
      if (blk.name == "moment_coeffs") o_linear = blk.offset;
    struct Stats { double center = 0, spread = 0; size_t count = 0; bool valid = false; };
    struct Eval { double scaling = 0; Stats st; std::vector<double> p; bool valid = false; };
    auto stats_of = [&](const std::vector<double>& p) {
      Stats st;
      std::vector<double> logs;
      for (int q = 0; q < nread; ++q) {
        const double a = std::abs(p[o_linear + q]);
        if (a > 1e-12) logs.push_back(std::log(a));
      }
      if (logs.empty()) return st;
      std::sort(logs.begin(), logs.end());
      st.count = logs.size();
      st.center = logs[logs.size() / 2];
      double sq = 0.0;
      for (double v : logs) sq += (v - st.center) * (v - st.center);
      st.spread = std::sqrt(sq / logs.size());
      st.valid = true;
      return st;
    };
    // the frames the trial solves run on
    std::unique_ptr<Trainer> sub;
    if (nframes_ > 5) {
      std::vector<int> order(nframes_);
      for (int f = 0; f < nframes_; ++f) order[f] = f;
      std::stable_sort(order.begin(), order.end(),
                       [&](int a, int b) { return natoms_list_[a] < natoms_list_[b]; });
      std::vector<int> picks;
      auto push = [&](int f) { if (std::find(picks.begin(), picks.end(), f) == picks.end()) picks.push_back(f); };
      const int n = nframes_;
      push(order[n - 1]); push(order[n - 2]); push(order[n / 2]); push(order[1]); push(order[0]);
      std::vector<int> na, hs;
      std::vector<double> cl, ps, e0, f0, s0;
      std::vector<int> ty;
      for (int f : picks) {
        const int a0 = fbegin_host_[f], a1 = fbegin_host_[f + 1];
        na.push_back(a1 - a0);
        cl.insert(cl.end(), cells_.begin() + 9 * f, cells_.begin() + 9 * f + 9);
        ps.insert(ps.end(), pos_h_.begin() + 3 * a0, pos_h_.begin() + 3 * a1);
        ty.insert(ty.end(), types_h_.begin() + a0, types_h_.begin() + a1);
        e0.push_back(E0_h_[f]);
        f0.insert(f0.end(), F0_h_.begin() + 3 * a0, F0_h_.begin() + 3 * a1);
        s0.insert(s0.end(), S0_h_.begin() + 9 * f, S0_h_.begin() + 9 * f + 9);
        hs.push_back(has_h_[f]);
      }
      sub = std::make_unique<Trainer>(eng_, static_cast<int>(picks.size()), na.data(), cl.data(), ps.data(), ty.data(),
                                      e0.data(), f0.data(), s0.data(), hs.data(), cfg_);
    }
    Trainer& T = sub ? *sub : *this;
    std::vector<double> cur(params, params + nparams_);  // coefficients carried from trial to trial
    int solves = 0;
    auto evaluate = [&](double s) {
      Eval r;
      r.scaling = s;
      eng_.set_scaling(s);
      T.train_linear(cur.data());
      ++solves;
      r.p = cur;
      r.st = stats_of(cur);
      r.valid = r.st.valid;
      return r;
    };
    constexpr int kCenterMaxIters = 6, kExpandMaxIters = 6;
    constexpr double kCenterTol = 0.15, kFloor = 1e-12, kBracket = 2.0;
    const double factors[5] = {1.0 / 1.08, 1.0 / 1.03, 1.0, 1.03, 1.08};
    Eval center = evaluate(m.scaling);
    if (!center.valid) {
      // no readout coefficient above the floor: the reference leaves the model as the seed solve
      std::copy(center.p.begin(), center.p.end(), params);
      *scaling_out = center.scaling;
      eng_.set_params(params);
      return solves;
    }
    Eval best = center, pos, neg;
    bool have_pos = false, have_neg = false;
    auto consider = [&](const Eval& e) {
      if (!e.valid) return;
      if (std::abs(e.st.center) < std::abs(best.st.center)) best = e;
      if (e.st.center >= 0.0) {
        if (!have_pos || e.st.center < pos.st.center) pos = e;
        have_pos = true;
      } else {
        if (!have_neg || e.st.center > neg.st.center) neg = e;
        have_neg = true;
      }
    };
    consider(center);
    if (std::abs(center.st.center) >= kCenterTol) {
      Eval lower, upper;
      const double ls = std::max(kFloor, center.scaling / kBracket);
      if (ls < center.scaling) {
        lower = evaluate(ls);
        if (lower.valid) consider(lower);
      }
      if (!(have_pos && have_neg)) {
        const double us = center.scaling * kBracket;
        if (std::isfinite(us)) {
          upper = evaluate(us);
          if (upper.valid) consider(upper);
        }
      }
      if (!(have_pos && have_neg)) {
        // first expansion direction: the probe that improves |median log| most, else none
        int dir = 0;
        double err = std::abs(center.st.center);
        if (lower.valid && std::abs(lower.st.center) < err) { err = std::abs(lower.st.center); dir = -1; }
        if (upper.valid && std::abs(upper.st.center) < err) dir = 1;
        Eval edge = dir < 0 ? lower : upper;
        for (int it = 0; dir != 0 && it < kExpandMaxIters && !(have_pos && have_neg); ++it) {
          const double ts = dir < 0 ? std::max(kFloor, edge.scaling / kBracket) : edge.scaling * kBracket;
          if (!(ts > 0.0) || !std::isfinite(ts) || ts == edge.scaling) break;
          Eval trial = evaluate(ts);
          if (!trial.valid) break;
          const double prev = std::abs(edge.st.center);
          consider(trial);
          edge = trial;
          if (!(have_pos && have_neg) && std::abs(trial.st.center) >= prev) break;
        }
      }
    }
    if (have_pos && have_neg) {
      for (int it = 0; it < kCenterMaxIters; ++it) {
        const double lp = std::log(pos.scaling), ln = std::log(neg.scaling);
        double lt = 0.5 * (lp + ln);
        const double cp = pos.st.center, cn = neg.st.center;
        if (std::abs(cp - cn) > 1e-12) {
          lt = (lp * cn - ln * cp) / (cn - cp);
          lt = std::max(std::min(lt, std::max(lp, ln)), std::min(lp, ln));
          const double span = std::abs(lp - ln);
          if (std::abs(lt - lp) < 0.1 * span || std::abs(lt - ln) < 0.1 * span) lt = 0.5 * (lp + ln);
        }
        Eval trial = evaluate(std::max(kFloor, std::exp(lt)));
        if (!trial.valid) break;
        consider(trial);
        if (std::abs(trial.st.center) < kCenterTol) { best = trial; break; }
      }
    }
    // fine trials around the centred scaling: least spread^2 + 3 median^2
    const double base = best.scaling;
    double best_metric = std::numeric_limits<double>::infinity(), best_scaling = base;
    std::vector<double> best_p = best.p;
    for (int j = 0; j < 5; ++j) {
      Eval trial = evaluate(std::max(kFloor, base * factors[j]));
      if (!trial.valid) continue;
      const double metric = trial.st.spread * trial.st.spread + 3.0 * trial.st.center * trial.st.center;
      if (metric < best_metric) {
        best_metric = metric;
        best_scaling = trial.scaling;
        best_p = trial.p;
      }
    }
    std::copy(best_p.begin(), best_p.end(), params);
    *scaling_out = best_scaling;
    eng_.set_scaling(best_scaling);
    eng_.set_params(params);
    return solves;
  }

  int graph_builds() const { return graph_builds_; }

 private:
  Engine& eng_;
  int nframes_ = 0, natoms_ = 0, nparams_ = 0;
  LossConfig cfg_;
  std::vector<int> fbegin_host_, natoms_list_;
  std::vector<double> cells_;
  std::vector<double> pos_h_, E0_h_, F0_h_, S0_h_;
  std::vector<int> types_h_, has_h_;
  DevBuf pos_, types_, E0_, F0_, S0_, has_, fbegin_;
  DevBuf E_, F_, V_, ew_, fw_, sw_, lossf_, loss_, grad_;
  bool gatex_ = false;
  DevBuf extra_h_, agrad_;  // gate-x term: dP/dh per atom, dP/dalpha per frame
  DevBuf metric_part_;
  DevBuf lin_cm_, lin_alpha_, lin_rhs_, lin_A_, lin_b_;  // linear warm-up
  double* host_scalars_ = nullptr;
  std::vector<double> h0_diag_;  // initial inverse-Hessian diagonal of bfgs (empty: the identity)
  int line_search_ = kLineSearchReference;
  std::vector<double> trial_f_, trial_x_;  // evaluated trials of the last bfgs call
  std::vector<int> trial_acc_;
  bool use_graph_ = true;
  cudaGraph_t graph_ = nullptr;
  cudaGraphExec_t graph_exec_ = nullptr;
  int graph_builds_ = 0;
  unsigned long long generation_ = 0;
};

}  // namespace sus2g

struct sus2g_trainer_s {
  std::unique_ptr<sus2g::Trainer> trainer;
};

namespace {
template <typename F>
int train_guarded(F&& f) {
  try {
    f();
    sus2g_set_last_error("");
    return 0;
  } catch (const sus2g::Error& e) {
    sus2g_set_last_error(e.what());
    return e.code > 0 ? e.code : 1;
  } catch (const std::exception& e) {
    sus2g_set_last_error(e.what());
    return 1;
  }
}
}  // namespace

extern "C" {

int sus2g_trainer_create(sus2g_engine engine, int nframes, const int* natoms, const double* cells,
                         const double* positions, const int* types, const double* energy, const double* forces,
                         const double* stress, const int* has_labels, double wE, double wF, double wS, int weighting,
                         int norm_by_forces, double gate_x_l2, sus2g_trainer* out) {
  return train_guarded([&] {
    if (!engine || !out || nframes < 0 || (nframes && (!natoms || !cells || !energy || !stress || !has_labels)))
      throw sus2g::Error(1, "invalid argument: trainer inputs");
    long long n = 0;
    for (int f = 0; f < nframes; ++f) {
      if (natoms[f] < 0) throw sus2g::Error(1, "invalid argument: natoms");
      n += natoms[f];
    }
    if (n && (!positions || !types || !forces)) throw sus2g::Error(1, "invalid argument: positions/types/forces");
    for (long long i = 0; i < n; ++i)
      if (types[i] < 0 || types[i] >= engine->engine->model().C) throw sus2g::Error(1, "atom species index out of range");
    if (weighting < 0 || weighting > 2) throw sus2g::Error(1, "weighting must be 0 (vibrations), 1 (structures) or 2 (molecules)");
    if (!(gate_x_l2 >= 0.0) || !std::isfinite(gate_x_l2)) throw sus2g::Error(1, "gate_x_l2 must be finite and >= 0");
    sus2g::LossConfig cfg{wE, wF, wS, weighting, norm_by_forces, gate_x_l2};
    auto t = std::make_unique<sus2g_trainer_s>();
    t->trainer = std::make_unique<sus2g::Trainer>(*engine->engine, nframes, natoms, cells, positions, types, energy,
                                                  forces, stress, has_labels, cfg);
    *out = t.release();
  });
}

void sus2g_trainer_free(sus2g_trainer t) { delete t; }

int sus2g_trainer_set_graph(sus2g_trainer t, int enabled) {
  return train_guarded([&] {
    if (!t) throw sus2g::Error(1, "invalid argument: trainer");
    t->trainer->set_graph(enabled != 0);
  });
}

int sus2g_trainer_loss_grad(sus2g_trainer t, const double* params, double* loss, double* grad) {
  return train_guarded([&] {
    if (!t || !params || !loss) throw sus2g::Error(1, "invalid argument: trainer/params/loss");
    *loss = t->trainer->loss_grad(params, grad);
  });
}

int sus2g_trainer_metrics(sus2g_trainer t, const double* params, double* out6) {
  return train_guarded([&] {
    if (!t || !params || !out6) throw sus2g::Error(1, "invalid argument: trainer/params/out");
    t->trainer->metrics(params, out6);
  });
}

int sus2g_trainer_rescale(sus2g_trainer t, double* params, double* scaling, int* solves) {
  return train_guarded([&] {
    if (!t || !params || !scaling) throw sus2g::Error(1, "invalid argument: trainer/params/scaling");
    const int n = t->trainer->rescale(params, scaling);
    if (solves) *solves = n;
  });
}

int sus2g_trainer_train_linear(sus2g_trainer t, double* params) {
  return train_guarded([&] {
    if (!t || !params) throw sus2g::Error(1, "invalid argument: trainer/params");
    t->trainer->train_linear(params);
  });
}

int sus2g_trainer_set_inv_hess_diagonal(sus2g_trainer t, const double* diag, int n) {
  return train_guarded([&] {
    if (!t || n < 0 || (n && !diag)) throw sus2g::Error(1, "invalid argument: trainer/diag/n");
    if (n && n != t->trainer->nparams()) throw sus2g::Error(1, "inverse-Hessian diagonal: length is not the parameter count");
    for (int i = 0; i < n; ++i)
      if (!(std::isfinite(diag[i]) && diag[i] > 0)) throw sus2g::Error(1, "inverse-Hessian diagonal: entries must be finite and positive");
    t->trainer->set_inv_hess_diagonal(diag, n);
  });
}

int sus2g_trainer_set_line_search(sus2g_trainer t, int mode) {
  return train_guarded([&] {
    if (!t) throw sus2g::Error(1, "invalid argument: trainer");
    t->trainer->set_line_search(mode);
  });
}

int sus2g_trainer_bfgs_trials(sus2g_trainer t, int cap, double* loss, double* points, int* accepted, int* count) {
  return train_guarded([&] {
    if (!t || !count || cap < 0) throw sus2g::Error(1, "invalid argument: trainer/count/cap");
    const auto& f = t->trainer->trial_loss();
    const auto& x = t->trainer->trial_x();
    const auto& a = t->trainer->trial_accepted();
    const int n = t->trainer->nparams();
    *count = static_cast<int>(f.size());
    for (int k = 0; k < std::min(cap, *count); ++k) {
      if (loss) loss[k] = f[k];
      if (accepted) accepted[k] = a[k];
      if (points) std::copy(x.begin() + static_cast<size_t>(k) * n, x.begin() + static_cast<size_t>(k + 1) * n,
                            points + static_cast<size_t>(k) * n);
    }
  });
}

int sus2g_trainer_bfgs(sus2g_trainer t, double* params, int max_iter, double gtol, double* history, int* steps) {
  return train_guarded([&] {
    if (!t || !params || max_iter < 0) throw sus2g::Error(1, "invalid argument: trainer/params/max_iter");
    const int k = t->trainer->bfgs(params, max_iter, gtol, history);
    if (steps) *steps = k;
  });
}

}  // extern "C"
