// Per-edge basis functions evaluated in registers: real spherical harmonics Y_lm(d/|d|) and the
// tanh-warped Chebyshev radial basis with its cutoff envelope.
//
// Real Y_lm.  Same convention as the reference engine (interfaces/lammps/ML-SUS2/sus2_sl_kernel.cpp:
// 12-42: orthonormal, Condon-Shortley phase folded so that Y_l,+m ~ +Re (x+iy)^m, index
// h = l*l + l + m).  Formulated here on the unit vector u = d/r:
//     Y_l,0  = N_l0 Pi_l0(u_z)
//     Y_l,+m = sqrt(2) N_lm Pi_lm(u_z) Re (u_x + i u_y)^m,   Y_l,-m = ... Im (u_x + i u_y)^m
// where Pi_mm = (2m-1)!!, Pi_m+1,m = (2m+1) u_z Pi_mm and
//     Pi_lm = ((2l-1) u_z Pi_l-1,m - (l+m-1) Pi_l-2,m) / (l-m)
// is the associated-Legendre recurrence with |u| = 1 substituted, and
// N_lm = sqrt((2l+1)/(4 pi) (l-m)!/(l+m)!).  The gradient with respect to d only needs tangential
// derivatives, so any smooth extension Yhat(u) off the sphere gives
//     dY/dd = (1/r) (I - u u^T) grad_u Yhat(u),
// which the reverse and tangent helpers below use with the polynomial extension above.
//
// Radial basis RBChebyshev_sss (src/radial_basis.cpp:1259, sus2_sl_radial_math.cpp:468-500,
// 1543-1595): xi = tanh(s (r - sigma) / 2), T_0 = 1, T_1 = xi, T_b = 2 xi T_b-1 - T_b-2, times
// scaling * f_c(r) with the legacy envelope f_c = (r - r_c)^2 or the polynomial envelope
// (sus2_sl_radial_math.cpp:256-294).  With two cutoffs the l = 0 functions use max_dist and the
// l > 0 functions use angular_max_dist (RB_CalcForCutoff, sus2_sl_radial_math.cpp:296-336).
#pragma once
#include <cmath>

#include "device_common.cuh"

namespace sus2g {

// N_lm (times sqrt 2 for m > 0), index l*l + l + m for m >= 0, in FP64 and rounded to FP32 (the
// FP32 form reads its own table: converting the FP64 entries at run time would occupy the FP64
// pipe, 1/64 of the FP32 rate on this GPU).  Each translation unit that includes this header owns
// a copy and fills it once per device through sph_norm_upload().
static __constant__ double c_sph_norm[64];
static __constant__ float c_sph_norm_f[64];

static inline cudaError_t sph_norm_upload() {
  double n[64] = {0};
  float nf[64] = {0};
  const double pi = 3.14159265358979323846;
  for (int l = 0; l <= 6; ++l)
    for (int m = 0; m <= l; ++m) {
      double ratio = 1.0;
      for (int a = l - m + 1; a <= l + m; ++a) ratio /= a;
      n[l * l + l + m] = std::sqrt((2 * l + 1) * ratio / (4 * pi)) * (m ? std::sqrt(2.0) : 1.0);
    }
  for (int q = 0; q < 64; ++q) nf[q] = static_cast<float>(n[q]);
  cudaError_t err = cudaMemcpyToSymbol(c_sph_norm, n, sizeof(n));
  if (err != cudaSuccess) return err;
  return cudaMemcpyToSymbol(c_sph_norm_f, nf, sizeof(nf));
}

template <int L> struct Sph { static constexpr int Lp = L + 1, H = Lp * Lp; };

__host__ __device__ constexpr int sh_index(int l, int m) { return l * l + l + m; }

// (2m-1)!! and 1/n as literals of type T: with the unrolled (l, m) loops the argument is a
// compile-time value and these fold to immediates (a constexpr double recursion would be
// evaluated at run time in FP64).
template <typename T>
__device__ __forceinline__ T sph_dfact(int m) {
  switch (m) {
    case 0: case 1: return T(1);
    case 2: return T(3);
    case 3: return T(15);
    case 4: return T(105);
    case 5: return T(945);
    case 6: return T(10395);
    default: return T(135135);
  }
}
template <typename T>
__device__ __forceinline__ T sph_inv(int n) {
  switch (n) {
    case 1: return T(1);
    case 2: return T(0.5);
    case 3: return T(0.33333333333333333333);
    case 4: return T(0.25);
    case 5: return T(0.2);
    case 6: return T(0.16666666666666666667);
    default: return T(0.14285714285714285714);
  }
}

template <typename T> __device__ __forceinline__ T norm_lm(int idx) { return T(c_sph_norm[idx]); }
template <> __device__ __forceinline__ float norm_lm<float>(int idx) { return c_sph_norm_f[idx]; }

// Values Y[h] for h < (L+1)^2 at unit vector (ux, uy, uz).
template <int L, typename T>
__device__ __forceinline__ void sph_values(T ux, T uy, T uz, T* Y) {
  T Cm[L + 1], Sm[L + 1];
  Cm[0] = T(1); Sm[0] = T(0);
#pragma unroll
  for (int m = 1; m <= L; ++m) {
    Cm[m] = ux * Cm[m - 1] - uy * Sm[m - 1];
    Sm[m] = ux * Sm[m - 1] + uy * Cm[m - 1];
  }
#pragma unroll
  for (int m = 0; m <= L; ++m) {
    T p2 = T(0), p1 = T(0), p0 = sph_dfact<T>(m);
#pragma unroll
    for (int l = m; l <= L; ++l) {
      T p;
      if (l == m) p = p0;
      else if (l == m + 1) p = T(2 * m + 1) * uz * p0;
      else p = (T(2 * l - 1) * uz * p1 - T(l + m - 1) * p2) * sph_inv<T>(l - m);
      if (l == m) { p1 = p; }
      else { p2 = p1; p1 = p; }
      const T n = norm_lm<T>(sh_index(l, m)) * p;
      if (m == 0) {
        Y[sh_index(l, 0)] = n;
      } else {
        Y[sh_index(l, m)] = n * Cm[m];
        Y[sh_index(l, -m)] = n * Sm[m];
      }
    }
  }
}

// grad_u of sum_h P[h] Yhat_h(u) (polynomial extension), accumulated into (gx, gy, gz).
template <int L, typename T>
__device__ __forceinline__ void sph_grad_dot(T ux, T uy, T uz, const T* P, T& gx, T& gy, T& gz) {
  T Cm[L + 1], Sm[L + 1];
  Cm[0] = T(1); Sm[0] = T(0);
#pragma unroll
  for (int m = 1; m <= L; ++m) {
    Cm[m] = ux * Cm[m - 1] - uy * Sm[m - 1];
    Sm[m] = ux * Sm[m - 1] + uy * Cm[m - 1];
  }
#pragma unroll
  for (int m = 0; m <= L; ++m) {
    const T pmm = sph_dfact<T>(m);
    T p1 = T(0), p2 = T(0), d1 = T(0), d2 = T(0);
#pragma unroll
    for (int l = m; l <= L; ++l) {
      T p, d;
      if (l == m) { p = pmm; d = T(0); }
      else if (l == m + 1) { p = T(2 * m + 1) * uz * pmm; d = T(2 * m + 1) * pmm; }
      else {
        const T inv = sph_inv<T>(l - m);
        p = (T(2 * l - 1) * uz * p1 - T(l + m - 1) * p2) * inv;
        d = (T(2 * l - 1) * (p1 + uz * d1) - T(l + m - 1) * d2) * inv;
      }
      p2 = p1; p1 = p; d2 = d1; d1 = d;
      const T n = norm_lm<T>(sh_index(l, m));
      if (m == 0) {
        gz += P[sh_index(l, 0)] * n * d;
      } else {
        const T pc = P[sh_index(l, m)] * n, ps = P[sh_index(l, -m)] * n;
        const T mf = T(m);
        // d/dux (Cm, Sm) = m (C_m-1, S_m-1); d/duy (Cm, Sm) = m (-S_m-1, C_m-1)
        gx += p * mf * (pc * Cm[m - 1] + ps * Sm[m - 1]);
        gy += p * mf * (ps * Cm[m - 1] - pc * Sm[m - 1]);
        gz += d * (pc * Cm[m] + ps * Sm[m]);
      }
    }
  }
}

// Tangent of Yhat along a tangential direction t (already projected, divided by r):
// Ydot[h] = t . grad_u Yhat_h.
template <int L, typename T>
__device__ __forceinline__ void sph_tangent(T ux, T uy, T uz, T tx, T ty, T tz, T* Ydot) {
  T Cm[L + 1], Sm[L + 1];
  Cm[0] = T(1); Sm[0] = T(0);
#pragma unroll
  for (int m = 1; m <= L; ++m) {
    Cm[m] = ux * Cm[m - 1] - uy * Sm[m - 1];
    Sm[m] = ux * Sm[m - 1] + uy * Cm[m - 1];
  }
#pragma unroll
  for (int m = 0; m <= L; ++m) {
    const T pmm = sph_dfact<T>(m);
    T p1 = T(0), p2 = T(0), d1 = T(0), d2 = T(0);
#pragma unroll
    for (int l = m; l <= L; ++l) {
      T p, d;
      if (l == m) { p = pmm; d = T(0); }
      else if (l == m + 1) { p = T(2 * m + 1) * uz * pmm; d = T(2 * m + 1) * pmm; }
      else {
        const T inv = sph_inv<T>(l - m);
        p = (T(2 * l - 1) * uz * p1 - T(l + m - 1) * p2) * inv;
        d = (T(2 * l - 1) * (p1 + uz * d1) - T(l + m - 1) * d2) * inv;
      }
      p2 = p1; p1 = p; d2 = d1; d1 = d;
      const T n = norm_lm<T>(sh_index(l, m));
      if (m == 0) {
        Ydot[sh_index(l, 0)] = n * d * tz;
      } else {
        const T mf = T(m);
        Ydot[sh_index(l, m)] = n * (p * mf * (Cm[m - 1] * tx - Sm[m - 1] * ty) + d * Cm[m] * tz);
        Ydot[sh_index(l, -m)] = n * (p * mf * (Sm[m - 1] * tx + Cm[m - 1] * ty) + d * Sm[m] * tz);
      }
    }
  }
}

// Raw Chebyshev values and r-derivatives (envelope 1, scaling 1) for B <= NBM <= kMaxB (NBM is
// the compile-time array bound; with B == NBM known at compile time the loops are exact).
template <typename T, int NBM = kMaxB>
__device__ __forceinline__ void cheb_raw(T r, T slope, T shift, int B, T* Tv, T* Td) {
  const T xi = tanh(slope * (r - shift) * T(0.5));
  const T xr = (T(1) - xi * xi) * slope * T(0.5);
  Tv[0] = T(1); Td[0] = T(0);
  Tv[1] = xi; Td[1] = xr;
#pragma unroll
  for (int b = 2; b < NBM; ++b) {
    if (b < B) {
      Tv[b] = T(2) * xi * Tv[b - 1] - Tv[b - 2];
      Td[b] = T(2) * (xr * Tv[b - 1] + xi * Td[b - 1]) - Td[b - 2];
    }
  }
}

template <typename T, int NBM = kMaxB>
__device__ __forceinline__ void cheb_raw_values(T r, T slope, T shift, int B, T* Tv) {
  const T xi = tanh(slope * (r - shift) * T(0.5));
  Tv[0] = T(1);
  Tv[1] = xi;
#pragma unroll
  for (int b = 2; b < NBM; ++b)
    if (b < B) Tv[b] = T(2) * xi * Tv[b - 1] - Tv[b - 2];
}

// Warp variable and its derivatives for the parameter gradient: xi = tanh(s (r - sigma) / 2).
template <typename T>
struct WarpVar {
  T xi, xr, xs, xg, xrs, xrg;  // xi, d/dr, d/ds, d/dsigma, d2/dr ds, d2/dr dsigma
};

template <typename T>
__device__ __forceinline__ WarpVar<T> warp_var(T r, T slope, T shift) {
  WarpVar<T> w;
  w.xi = tanh(slope * (r - shift) * T(0.5));
  const T e = T(1) - w.xi * w.xi;
  w.xr = e * slope * T(0.5);
  w.xs = e * (r - shift) * T(0.5);
  w.xg = -e * slope * T(0.5);
  w.xrs = e * T(0.5) - w.xi * w.xs * slope;
  w.xrg = -w.xi * w.xg * slope;
  return w;
}

// Chebyshev T_b(xi) with its first and second derivatives in xi, b < B <= NBM <= kMaxB.
template <typename T, int NBM = kMaxB>
__device__ __forceinline__ void cheb_full(T xi, int B, T* Tv, T* D, T* DD) {
  Tv[0] = T(1); D[0] = T(0); DD[0] = T(0);
  Tv[1] = xi; D[1] = T(1); DD[1] = T(0);
#pragma unroll
  for (int b = 2; b < NBM; ++b) {
    if (b < B) {
      Tv[b] = T(2) * xi * Tv[b - 1] - Tv[b - 2];
      D[b] = T(2) * Tv[b - 1] + T(2) * xi * D[b - 1] - D[b - 2];
      DD[b] = T(4) * D[b - 1] + T(2) * xi * DD[b - 1] - DD[b - 2];
    }
  }
}

// Cutoff envelope f_c and its r-derivative (CalcRadialCutoff, sus2_sl_radial_math.cpp:256-294).
template <typename T>
__device__ __forceinline__ void envelope(T r, T rc, int poly, int p, T& f, T& fd) {
  if (r >= rc) { f = T(0); fd = T(0); return; }
  if (!poly) {
    const T dr = r - rc;
    f = dr * dr;
    fd = T(2) * dr;
    return;
  }
  const T x = r / rc, omx = T(1) - x;
  T poly_v = T(0);
  for (int k = p - 1; k >= 0; --k) poly_v = poly_v * x + T(0.5) * T((k + 1) * (k + 2));
  f = omx * omx * omx * poly_v;
  T xp = T(1);
  for (int k = 0; k < p - 1; ++k) xp *= x;
  const T pf = T(p);
  fd = T(-0.5) * pf * (pf + T(1)) * (pf + T(2)) * xp * omx * omx / rc;
}

}  // namespace sus2g
