// CPU FP64 restatement of the SUS2-SH E / F / virial and parameter-gradient path.
// TEST INFRASTRUCTURE ONLY (see sus2_oracle.h): the checker for the GPU engine, pinned against the
// reference's own outputs committed under tests/golden/.
//
// It restates, in plain loops over an explicit edge list:
//   * .sus2 reading and defaults     interfaces/lammps/ML-SUS2/sus2_sl_model.cpp:174-257
//   * periodic image-scan edges      interfaces/lammps/tests/embedded_efs.cpp:49-66
//   * radial basis RBChebyshev_sss   src/radial_basis.cpp:1259-1310 (values, d/dr, d/ds, d/dsigma)
//                                    with the legacy / polynomial envelope sus2_sl_radial_math.cpp:256-336
//   * edge moments                   sus2_sl_kernel.cpp:165-216 (edge_basis), 319-354
//   * rank contraction + CG graph    sus2_sl_kernel.cpp:104-105, 217-221, 308-313
//   * readout, reverse, forces       sus2_sl_kernel.cpp:356-380, 527-562
//   * Effect gate                    sus2_sl_kernel.cpp:447-455, 558-559
//   * parameter gradient             src/basic_mlip.cpp:421-476 (AccumulateEFSCombinationGrad contract):
//       d/dtheta [ sum_i ew_i E_i + sum_e (fw_i - fw_j + sw d_e) . dE/dd_e ]
//     evaluated by forward tangents along the edge weights followed by a reverse sweep.
#include "sus2_oracle.h"

#include <algorithm>
#include <array>
#include <chrono>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <stdexcept>
#include <string>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

using std::vector;
using V3 = std::array<double, 3>;

struct Fail : std::runtime_error { using std::runtime_error::runtime_error; };
void req(bool ok, const std::string& m) { if (!ok) throw Fail(m); }

std::string trim(const std::string& s) {
  const auto a = s.find_first_not_of(" \t\r\n");
  return a == std::string::npos ? "" : s.substr(a, s.find_last_not_of(" \t\r\n") - a + 1);
}

struct Prod { int a, b, out; double c; };

struct Model {
  std::map<std::string, std::string> f;
  int C = 0, L = 0, K = 0, B = 0, F = 0, H = 0, M = 0, NB = 0, P = 0, S = 0, Q = 0, nblk = 0, smode = 3;
  double rmax = 0, rang = 0, scaling = 1;
  bool split = false, poly = false, species_readout = false, gated = false, own_gate_radial = false, decoupled = false;
  int cutoff_p = 5;
  vector<double> shift, scal, radial, species, linear, gate_radial, gate_scal, gate_type, gate_add, gate_w, outer_w, gate_rw;
  vector<std::array<int, 3>> basic;
  vector<Prod> prod;
  vector<int> smap, gnodes;
  int orank = 0, obegin = 0, oprod = 0, grank = 0, gbegin = 0, gpb = 0, gpe = 0;
  // parameter layout offsets (-1 absent)
  int o_shift, o_scal, o_radial, o_grad_radial = -1, o_gscal = -1, o_gadd = -1, o_gtype = -1, o_gw = -1, o_grw = -1,
      o_orw = -1, o_species, o_linear, nparams;

  bool has(const std::string& k) const { return f.count(k) != 0; }
  std::string text(const std::string& k, const std::string& d = "") const { auto it = f.find(k); return it == f.end() ? d : it->second; }
  double real(const std::string& k, double d = 0) const { return has(k) ? std::strtod(text(k).c_str(), nullptr) : d; }
  int integer(const std::string& k, int d = 0) const { return has(k) ? static_cast<int>(std::lround(real(k))) : d; }
  bool boolean(const std::string& k, bool d = false) const { if (!has(k)) return d; auto s = text(k); return s == "true" || s == "1"; }
  vector<double> nums(const std::string& k) const {
    vector<double> out;
    if (!has(k)) return out;
    std::string s = text(k);
    for (char& c : s) if (c == '{' || c == '}' || c == ',') c = ' ';
    const char* p = s.c_str();
    char* end = nullptr;
    while (true) {
      const double x = std::strtod(p, &end);
      if (end == p) break;
      out.push_back(x);
      p = end;
    }
    return out;
  }
  vector<int> ints(const std::string& k) const { vector<int> o; for (double x : nums(k)) o.push_back(static_cast<int>(std::lround(x))); return o; }
  double gate_weight(int mu, int q) const { return gate_w[static_cast<size_t>(mu) * Q + q]; }
};

Model load(const char* path) {
  Model m;
  std::ifstream in(path);
  req(bool(in), std::string("cannot open ") + path);
  std::string line, radial;
  bool in_radial = false, header = false;
  while (std::getline(in, line)) {
    line = trim(line);
    if (line.empty() || line[0] == '#') continue;
    if (!header) { req(line == "MTP", "missing MTP header"); header = true; continue; }
    const auto eq = line.find('=');
    if (eq == std::string::npos) {
      if (line == "radial_coeffs") { in_radial = true; continue; }
      req(in_radial, "unrecognized line " + line);
      if (line == "0-0") continue;
      radial += (radial.empty() ? "" : ",") + line;
      continue;
    }
    in_radial = false;
    std::string key = trim(line.substr(0, eq)), value = trim(line.substr(eq + 1));
    int depth = 0;
    for (char c : value) depth += (c == '{') - (c == '}');
    while (depth > 0 && std::getline(in, line)) { value += " " + trim(line); for (char c : line) depth += (c == '{') - (c == '}'); }
    m.f[key] = value;
  }
  if (!radial.empty()) m.f["radial_coeffs"] = "{" + radial + "}";
  req(m.text("potential_tag") == "SUS2-SH", "not a SUS2-SH model");
  req(m.text("outer_radial_mode", "legacy-plus-mixer") == "legacy-plus-mixer", "only legacy-plus-mixer models");
  req(m.text("radial_basis_type") == "RBChebyshev_sss", "only RBChebyshev_sss");
  m.C = m.integer("species_count"); m.L = m.integer("sh_l_max"); m.K = m.integer("sh_k_max");
  m.B = m.integer("radial_basis_size"); m.F = m.integer("radial_funcs_count"); m.M = m.integer("alpha_moments_count");
  m.S = m.integer("alpha_scalar_moments"); m.H = (m.L + 1) * (m.L + 1);
  m.rmax = m.real("max_dist"); m.rang = m.real("angular_max_dist", m.rmax); m.scaling = m.real("scaling", 1.0);
  m.split = m.rang != m.rmax;
  m.poly = m.text("radial_cutoff_type", "legacy") == "polynomial";
  m.cutoff_p = m.integer("radial_cutoff_p", 5);
  const std::string sm = m.text("scaling_map", "LK");
  m.smode = sm == "pair" ? 0 : sm == "L" ? 1 : sm == "K" ? 2 : 3;
  m.nblk = m.smode == 0 ? 1 : m.smode == 1 ? m.L + 1 : m.smode == 2 ? m.K : m.F;
  const int C = m.C, F = m.F, B = m.B;
  m.radial = m.nums("radial_coeffs");
  if (m.radial.empty()) {
    m.radial.assign(static_cast<size_t>(F) * (B + C), 0.01);
    for (int mu = 0; mu < F; ++mu) for (int t = 0; t < C; ++t) m.radial[mu * (B + C) + B + t] = 2.0;
  }
  m.shift = m.nums("shift_coeffs");
  if (m.shift.empty()) m.shift.assign(C, -1.0);
  m.scal = m.nums("scal_coeffs");
  if (m.scal.empty()) {
    m.scal.assign(2 * C * C * m.nblk, 0.0);
    for (int b = 0; b < m.nblk; ++b)
      for (int t = 0; t < C; ++t)
        for (int u = 0; u < C; ++u) {
          const double x = C == 1 ? .5 : (std::sqrt(t + 1.) + std::sqrt(u + 1.) - 2.) / (2. * std::sqrt(double(C)) - 2.);
          m.scal[2 * b * C * C + t * C + u] = 4.0 - 2.0 * x;
          m.scal[(2 * b + 1) * C * C + t * C + u] = 1.5 + x;
        }
  }
  m.species_readout = m.text("readout_mode", "shared") == "species";
  m.species = m.nums("species_coeffs");
  m.linear = m.nums("moment_coeffs");
  if (m.species.empty()) {
    m.species.assign(C, 0.001);
    m.linear.assign(static_cast<size_t>(m.S) * (m.species_readout ? C : 1), m.species_readout ? 1e-6 : 0.001);
  }
  const auto bv = m.nums("alpha_index_basic");
  for (size_t i = 0; i + 2 < bv.size(); i += 3)
    m.basic.push_back({static_cast<int>(bv[i]), static_cast<int>(bv[i + 1]), static_cast<int>(bv[i + 2])});
  const auto pv = m.nums("sh_products");
  for (size_t i = 0; i + 3 < pv.size(); i += 4)
    m.prod.push_back({static_cast<int>(pv[i]), static_cast<int>(pv[i + 1]), static_cast<int>(pv[i + 2]), pv[i + 3]});
  m.NB = static_cast<int>(m.basic.size());
  m.P = static_cast<int>(m.prod.size());
  m.smap = m.ints("alpha_moment_mapping");
  if (m.boolean("outer_k_rank1_enabled")) {
    m.orank = m.integer("outer_k_rank", 1);
    m.obegin = m.integer("outer_k_rank1_basic_begin");
    m.oprod = m.integer("outer_k_rank1_product_begin");
    m.outer_w = m.nums("outer_k_rank1_weights");
  }
  m.grank = m.integer("two_layer_gate_k_rank");
  m.gbegin = m.integer("two_layer_gate_k_rank_basic_begin");
  m.gpb = m.integer("two_layer_gate_k_rank_product_begin", 0);
  m.gpe = m.grank ? m.integer("two_layer_gate_k_rank_product_end", m.oprod) : m.oprod;
  if (!m.orank && !m.grank) m.gpe = m.P;
  m.gated = m.boolean("two_layer_gate_enabled");
  if (m.gated) {
    req(m.text("two_layer_gate_mode") == "mu-scalar-full", "oracle supports the mu-scalar-full gate");
    m.gnodes = m.ints("two_layer_gate_scalar_moment_indices");
    if (m.gnodes.empty()) for (int q : m.ints("two_layer_gate_scalar_indices")) m.gnodes.push_back(m.smap[q]);
    m.Q = static_cast<int>(m.gnodes.size());
    m.gate_w = m.nums("two_layer_gate_weights");
    m.gate_rw = m.nums("two_layer_gate_k_rank_weights");
    m.own_gate_radial = m.text("two_layer_gate_radial_mode", "base-radial") == "shared-radial";
    m.gate_radial = m.nums("two_layer_gate_radial_coeffs");
    m.decoupled = m.text("two_layer_gate_scaling_mode", "shared-scaling") == "decoupled";
    m.gate_scal = m.nums("two_layer_gate_scaling_coeffs");
    auto expand = [&](const char* key, bool tau) {
      vector<double> v = m.nums(key), o(static_cast<size_t>(C) * F);
      for (int t = 0; t < C; ++t)
        for (int mu = 0; mu < F; ++mu) {
          const size_t i = static_cast<size_t>(t) * F + mu;
          o[i] = i < v.size() ? v[i] : (v.size() == static_cast<size_t>(C) ? v[t] : (v.empty() && tau ? m.radial[mu * (B + C) + B + t] : 1.0));
        }
      return o;
    };
    m.gate_type = expand("two_layer_gate_type_coeffs", true);
    m.gate_add = expand("two_layer_gate_additive_coeffs", false);
  }
  int off = 0;
  auto put = [&](int& o, size_t n) { o = off; off += static_cast<int>(n); };
  put(m.o_shift, m.shift.size()); put(m.o_scal, m.scal.size()); put(m.o_radial, m.radial.size());
  if (m.gated) {
    put(m.o_grad_radial, m.gate_radial.size());
    if (m.decoupled) put(m.o_gscal, m.gate_scal.size());
    put(m.o_gadd, m.gate_add.size()); put(m.o_gtype, m.gate_type.size()); put(m.o_gw, m.gate_w.size());
    if (m.grank) put(m.o_grw, m.gate_rw.size());
  }
  if (m.orank && !m.outer_w.empty()) put(m.o_orw, m.outer_w.size());
  put(m.o_species, m.species.size()); put(m.o_linear, m.linear.size());
  m.nparams = off;
  return m;
}

vector<double>* block(Model& m, int which) {
  vector<double>* all[] = {&m.shift, &m.scal, &m.radial, &m.gate_radial, &m.gate_scal, &m.gate_add, &m.gate_type,
                           &m.gate_w, &m.gate_rw, &m.outer_w, &m.species, &m.linear};
  return all[which];
}
int block_offset(const Model& m, int which) {
  const int o[] = {m.o_shift, m.o_scal, m.o_radial, m.o_grad_radial, m.o_gscal, m.o_gadd, m.o_gtype, m.o_gw, m.o_grw, m.o_orw, m.o_species, m.o_linear};
  return o[which];
}

// ----------------------------------------------------------------------------------------------
// basis functions
// ----------------------------------------------------------------------------------------------
int hidx(int l, int m) { return l * l + l + m; }

// Real Y_lm at d and their gradients wrt d (3H), computed from the polynomial extension on the unit
// vector and projected onto the tangent plane.
void harmonics(const V3& d, int L, vector<double>& Y, vector<double>& dY) {
  const int H = (L + 1) * (L + 1);
  Y.assign(H, 0.0);
  dY.assign(3 * H, 0.0);
  const double r = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
  const double u[3] = {d[0] / r, d[1] / r, d[2] / r};
  const double pi = std::acos(-1.0);
  std::complex<double> w(u[0], u[1]);
  std::complex<double> pw[8];
  pw[0] = 1.0;
  for (int m = 1; m <= L; ++m) pw[m] = pw[m - 1] * w;
  for (int m = 0; m <= L; ++m) {
    double pm2 = 0, pm1 = 0, dm2 = 0, dm1 = 0;
    double pmm = 1;
    for (int k = 1; k <= m; ++k) pmm *= (2 * k - 1);
    for (int l = m; l <= L; ++l) {
      double p, dp;
      if (l == m) { p = pmm; dp = 0; }
      else if (l == m + 1) { p = (2 * m + 1) * u[2] * pmm; dp = (2 * m + 1) * pmm; }
      else {
        p = ((2 * l - 1) * u[2] * pm1 - (l + m - 1) * pm2) / (l - m);
        dp = ((2 * l - 1) * (pm1 + u[2] * dm1) - (l + m - 1) * dm2) / (l - m);
      }
      pm2 = pm1; pm1 = p; dm2 = dm1; dm1 = dp;
      static const std::array<double, 64> norms = [pi] {
        std::array<double, 64> t{};
        for (int ll = 0; ll <= 6; ++ll)
          for (int mm = 0; mm <= ll; ++mm) {
            double ratio = 1;
            for (int a = ll - mm + 1; a <= ll + mm; ++a) ratio /= a;
            t[hidx(ll, mm)] = std::sqrt((2 * ll + 1) * ratio / (4 * pi)) * (mm ? std::sqrt(2.0) : 1.0);
          }
        return t;
      }();
      const double n = norms[hidx(l, m)];
      // extension values and grad_u
      std::complex<double> t = pw[m];
      std::complex<double> tx = m ? double(m) * pw[m - 1] : std::complex<double>(0);   // d/dux (ux+i uy)^m
      std::complex<double> ty = m ? std::complex<double>(0, m) * pw[m - 1] : std::complex<double>(0);
      double g[2][3] = {{n * p * tx.real(), n * p * ty.real(), n * dp * t.real()},
                        {n * p * tx.imag(), n * p * ty.imag(), n * dp * t.imag()}};
      const int idx[2] = {hidx(l, m), hidx(l, -m)};
      const double val[2] = {n * p * t.real(), n * p * t.imag()};
      for (int c = 0; c < (m ? 2 : 1); ++c) {
        Y[idx[c]] = val[c];
        const double ug = u[0] * g[c][0] + u[1] * g[c][1] + u[2] * g[c][2];
        for (int q = 0; q < 3; ++q) dY[3 * idx[c] + q] = (g[c][q] - u[q] * ug) / r;
      }
    }
  }
}

// Chebyshev radial basis with envelope: values v, d/dr, d/dslope, d2/dslope dr, d/dshift, d2/dshift dr.
struct Rad { double v[16], r[16], s[16], sr[16], g[16], gr[16]; };

void radial(const Model& m, double r, double slope, double shift, double rc, Rad& o, bool param_derivs = true) {
  double f, fd;
  if (r >= rc) { f = 0; fd = 0; }
  else if (!m.poly) { f = (r - rc) * (r - rc); fd = 2 * (r - rc); }
  else {
    const double x = r / rc, a = 1 - x;
    double poly = 0;
    for (int k = m.cutoff_p - 1; k >= 0; --k) poly = poly * x + 0.5 * (k + 1) * (k + 2);
    f = a * a * a * poly;
    const double p = m.cutoff_p;
    fd = -0.5 * p * (p + 1) * (p + 2) * std::pow(x, m.cutoff_p - 1) * a * a / rc;
  }
  f *= m.scaling; fd *= m.scaling;
  const double xi = std::tanh(slope * (r - shift) / 2), e = 1 - xi * xi;
  const double xr = e * slope / 2, xs = e * (r - shift) / 2, xg = -e * slope / 2;
  const double xrs = e / 2 - xi * xs * slope, xrg = -xi * xg * slope;
  if (!param_derivs) {  // values and d/dr only (E / F / virial)
    double T0 = 1, T1 = xi, D0 = 0, D1 = 1;
    for (int b = 0; b < m.B; ++b) {
      double T, D;
      if (b == 0) { T = T0; D = D0; }
      else if (b == 1) { T = T1; D = D1; }
      else {
        T = 2 * xi * T1 - T0;
        D = 2 * T1 + 2 * xi * D1 - D0;
        T0 = T1; T1 = T; D0 = D1; D1 = D;
      }
      o.v[b] = f * T;
      o.r[b] = fd * T + f * D * xr;
    }
    return;
  }
  // T_b(xi), T_b', T_b''
  double T[16], D[16], DD[16];
  T[0] = 1; D[0] = 0; DD[0] = 0;
  T[1] = xi; D[1] = 1; DD[1] = 0;
  for (int b = 2; b < m.B; ++b) {
    T[b] = 2 * xi * T[b - 1] - T[b - 2];
    D[b] = 2 * T[b - 1] + 2 * xi * D[b - 1] - D[b - 2];
    DD[b] = 4 * D[b - 1] + 2 * xi * DD[b - 1] - DD[b - 2];
  }
  for (int b = 0; b < m.B; ++b) {
    o.v[b] = f * T[b];
    o.r[b] = fd * T[b] + f * D[b] * xr;
    o.s[b] = f * D[b] * xs;
    o.sr[b] = fd * D[b] * xs + f * (DD[b] * xs * xr + D[b] * xrs);
    o.g[b] = f * D[b] * xg;
    o.gr[b] = fd * D[b] * xg + f * (DD[b] * xg * xr + D[b] * xrg);
  }
}

// ----------------------------------------------------------------------------------------------
// edges and per-atom passes
// ----------------------------------------------------------------------------------------------
struct Edge { int i, j; V3 d; };

vector<Edge> image_edges(int n, const double* cell, const double* pos, double rc) {
  double c[3][3], inv[3][3], det = 0;
  for (int a = 0; a < 3; ++a) for (int b = 0; b < 3; ++b) c[a][b] = cell[3 * a + b];
  for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j)
    inv[j][i] = c[(i + 1) % 3][(j + 1) % 3] * c[(i + 2) % 3][(j + 2) % 3] - c[(i + 1) % 3][(j + 2) % 3] * c[(i + 2) % 3][(j + 1) % 3];
  for (int i = 0; i < 3; ++i) det += c[0][i] * inv[i][0];
  req(std::fabs(det) > 0, "singular cell");
  for (auto& row : inv) for (auto& x : row) x /= det;
  double reach[3];
  for (int q = 0; q < 3; ++q) { double s = 0; for (int a = 0; a < 3; ++a) s += inv[a][q] * inv[a][q]; reach[q] = rc * std::sqrt(s); }
  vector<vector<Edge>> per(n);
#pragma omp parallel for schedule(dynamic, 16)
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) {
      V3 d{}, f{};
      for (int q = 0; q < 3; ++q) d[q] = pos[3 * j + q] - pos[3 * i + q];
      for (int q = 0; q < 3; ++q) for (int a = 0; a < 3; ++a) f[q] += d[a] * inv[a][q];
      int lo[3], hi[3];
      for (int q = 0; q < 3; ++q) { lo[q] = static_cast<int>(std::ceil(-f[q] - reach[q])); hi[q] = static_cast<int>(std::floor(-f[q] + reach[q])); }
      for (int a = lo[0]; a <= hi[0]; ++a)
        for (int b = lo[1]; b <= hi[1]; ++b)
          for (int cc = lo[2]; cc <= hi[2]; ++cc) {
            if (i == j && a == 0 && b == 0 && cc == 0) continue;
            V3 v = d;
            double r2 = 0;
            for (int q = 0; q < 3; ++q) { v[q] += a * c[0][q] + b * c[1][q] + cc * c[2][q]; r2 += v[q] * v[q]; }
            if (r2 < rc * rc) per[i].push_back({i, j, v});
          }
    }
  vector<Edge> out;
  for (auto& p : per) out.insert(out.end(), p.begin(), p.end());
  return out;
}

struct Pass {
  const vector<double>* coeff;  // radial coefficient rows
  int stride;                   // row stride (B or B + C)
  int coeff_off;                // parameter offset of the coefficient block
  const vector<double>* scal;
  int scal_off;
  const vector<double>* wtype;  // C x F centre/source factor
  int wtype_off;                // -1: tau inside radial rows
  int rank, begin, pb, pe;
  const vector<double>* rw;
  int rw_off;
};

Pass outer_pass(const Model& m) {
  return {&m.radial, m.B + m.C, m.o_radial, &m.scal, m.o_scal, nullptr, -1, m.orank, m.obegin, m.oprod, m.P, &m.outer_w, m.o_orw};
}
Pass gate_pass(const Model& m) {
  const bool own = m.own_gate_radial;
  return {own ? &m.gate_radial : &m.radial, own ? m.B : m.B + m.C, own ? m.o_grad_radial : m.o_radial,
          m.decoupled ? &m.gate_scal : &m.scal, m.decoupled ? m.o_gscal : m.o_scal, &m.gate_type, m.o_gtype,
          m.grank, m.gbegin, m.gpb, m.gpe, &m.gate_rw, m.o_grw};
}

// centre / source species factor of radial function mu
double wfac(const Model& m, const Pass& p, int t, int mu) {
  if (p.wtype) return (*p.wtype)[static_cast<size_t>(t) * m.F + mu];
  return m.radial[static_cast<size_t>(mu) * (m.B + m.C) + m.B + t];
}
int wfac_index(const Model& m, const Pass& p, int t, int mu) {
  if (p.wtype) return p.wtype_off + t * m.F + mu;
  return m.o_radial + mu * (m.B + m.C) + m.B + t;
}

int sblock(const Model& m, int k, int l) {
  const int Lp = m.L + 1;
  return m.smode == 2 ? k : m.smode == 1 ? l : m.smode == 0 ? 0 : k * Lp + l;
}

struct EdgeEval {
  double r;
  V3 u;
  vector<double> Y, dY;          // H, 3H
  vector<double> R, Rd;          // F: R_mu and dR_mu/dr
  vector<Rad> rad;               // per mu (raw basis derivatives)
};

void eval_edge(const Model& m, const Pass& p, const Edge& e, int ti, int tj, EdgeEval& ev, bool param_derivs = true) {
  const int Lp = m.L + 1, C = m.C;
  ev.r = std::sqrt(e.d[0] * e.d[0] + e.d[1] * e.d[1] + e.d[2] * e.d[2]);
  for (int q = 0; q < 3; ++q) ev.u[q] = e.d[q] / ev.r;
  harmonics(e.d, m.L, ev.Y, ev.dY);
  const bool ang = ev.r < m.rang;
  if (!ang) {
    for (int h = 1; h < m.H; ++h) { ev.Y[h] = 0; ev.dY[3 * h] = ev.dY[3 * h + 1] = ev.dY[3 * h + 2] = 0; }
  }
  ev.R.assign(m.F, 0.0);
  ev.Rd.assign(m.F, 0.0);
  if (ev.rad.size() != static_cast<size_t>(m.F)) ev.rad.resize(m.F);  // entries are rewritten below when used
  for (int k = 0; k < m.K; ++k)
    for (int l = 0; l < Lp; ++l) {
      if (l > 0 && !ang) continue;
      const int mu = k * Lp + l, sb = sblock(m, k, l), pair = ti * C + tj;
      const double slope = (*p.scal)[2 * sb * C * C + pair], shift = (*p.scal)[(2 * sb + 1) * C * C + pair];
      const double rc = (l > 0 && m.split) ? m.rang : m.rmax;
      radial(m, ev.r, slope, shift, rc, ev.rad[mu], param_derivs);
      double a = 0, ad = 0;
      for (int b = 0; b < m.B; ++b) {
        const double c = (*p.coeff)[static_cast<size_t>(mu) * p.stride + b];
        a += c * ev.rad[mu].v[b];
        ad += c * ev.rad[mu].r[b];
      }
      ev.R[mu] = a;
      ev.Rd[mu] = ad;
    }
}

struct Ctx {
  const Model* m;
  vector<Edge> edges;
  vector<int> row;               // CSR by centre (edges sorted by centre)
  vector<int> types;
  int n = 0;
};

// forward graph of one pass with optional tangents (vd)
void contract_graph_forward(const Model& m, const Pass& p, vector<double>& v, vector<double>* vd) {
  const int H = m.H;
  if (p.rank) {
    for (int a = 0; a < p.rank; ++a)
      for (int b = 0; b < m.NB; ++b) {
        const int k = m.basic[b][0], l = m.basic[b][1], mm = m.basic[b][2];
        const int dst = p.begin + p.rank * (H - (l + 1) * (l + 1)) + (p.rank - 1 - a) * (2 * l + 1) + mm + l;
        const int wi = (l * p.rank + a) * m.K + k;
        const double w = p.rw->empty() ? 1.0 : (*p.rw)[wi];
        v[dst] += w * v[b];
        if (vd) (*vd)[dst] += w * (*vd)[b];
      }
  }
  for (int q = p.pb; q < p.pe; ++q) {
    const Prod& pr = m.prod[q];
    if (vd) (*vd)[pr.out] += pr.c * ((*vd)[pr.a] * v[pr.b] + v[pr.a] * (*vd)[pr.b]);
    v[pr.out] += pr.c * v[pr.a] * v[pr.b];
  }
}

// reverse of the graph and contraction; lam/mu are the adjoints of v and vd; accumulates rank
// weight gradients into grad (if non-null)
void contract_graph_reverse(const Model& m, const Pass& p, const vector<double>& v, const vector<double>* vd,
                            vector<double>& lam, vector<double>* mu, double* grad) {
  const int H = m.H;
  for (int q = p.pe - 1; q >= p.pb; --q) {
    const Prod& pr = m.prod[q];
    const double zl = pr.c * lam[pr.out];
    double zm = 0;
    if (mu) zm = pr.c * (*mu)[pr.out];
    lam[pr.a] += zl * v[pr.b];
    lam[pr.b] += zl * v[pr.a];
    if (mu) {
      lam[pr.a] += zm * (*vd)[pr.b];
      lam[pr.b] += zm * (*vd)[pr.a];
      (*mu)[pr.a] += zm * v[pr.b];
      (*mu)[pr.b] += zm * v[pr.a];
    }
  }
  if (p.rank) {
    for (int a = 0; a < p.rank; ++a)
      for (int b = 0; b < m.NB; ++b) {
        const int k = m.basic[b][0], l = m.basic[b][1], mm = m.basic[b][2];
        const int dst = p.begin + p.rank * (H - (l + 1) * (l + 1)) + (p.rank - 1 - a) * (2 * l + 1) + mm + l;
        const int wi = (l * p.rank + a) * m.K + k;
        const double w = p.rw->empty() ? 1.0 : (*p.rw)[wi];
        lam[b] += w * lam[dst];
        if (mu) (*mu)[b] += w * (*mu)[dst];
        if (grad && !p.rw->empty()) {
          double gsum = lam[dst] * v[b];
          if (mu) gsum += (*mu)[dst] * (*vd)[b];
          grad[p.rw_off + wi] += gsum;
        }
      }
  }
}

int basic_mu(const Model& m, int b) { return m.basic[b][0] * (m.L + 1) + m.basic[b][1]; }
int basic_h(const Model& m, int b) { return hidx(m.basic[b][1], m.basic[b][2]); }

struct Result {
  double energy = 0;
  vector<double> site;
  vector<V3> g;      // per edge dE/dd
  double* desc = nullptr;  // optional [ncentres][S]: the scalar moments v[alpha_moment_mapping[q]]
};

// E / F / virial of the edges in ctx (owned centres are 0..ncentres-1)
void evaluate(const Ctx& cx, int ncentres, Result& res, int threads) {
  const Model& m = *cx.m;
  const int F = m.F, M = m.M;
  const Pass po = outer_pass(m), pg = gate_pass(m);
  const size_t E = cx.edges.size();
  res.site.assign(ncentres, 0.0);
  res.g.assign(E, V3{0, 0, 0});
  vector<double> h(static_cast<size_t>(cx.n) * F, 0.0), gmom, hbar_edge;
  if (m.gated) {
    gmom.assign(static_cast<size_t>(ncentres) * M, 0.0);
    hbar_edge.assign(E * F, 0.0);
  }
  (void)threads;
  // gate pass
  if (m.gated) {
#pragma omp parallel for schedule(dynamic, 4) num_threads(threads)
    for (int i = 0; i < ncentres; ++i) {
      EdgeEval ev;
      vector<double> v(M, 0.0);
      for (int e = cx.row[i]; e < cx.row[i + 1]; ++e) {
        const Edge& ed = cx.edges[e];
        const int ti = cx.types[ed.i], tj = cx.types[ed.j];
        eval_edge(m, pg, ed, ti, tj, ev, false);
        for (int b = 0; b < m.NB; ++b) {
          const int mu = basic_mu(m, b);
          v[b] += wfac(m, pg, ti, mu) * wfac(m, pg, tj, mu) * ev.R[mu] * ev.Y[basic_h(m, b)];
        }
      }
      contract_graph_forward(m, pg, v, nullptr);
      std::copy(v.begin(), v.end(), gmom.begin() + static_cast<size_t>(i) * M);
      for (int mu = 0; mu < F; ++mu) {
        double s = 0;
        for (int q = 0; q < m.Q; ++q) s += m.gate_weight(mu, q) * v[m.gnodes[q]];
        h[static_cast<size_t>(i) * F + mu] = s;
      }
    }
  }
  // outer pass
#pragma omp parallel for schedule(dynamic, 4) num_threads(threads)
  for (int i = 0; i < ncentres; ++i) {
    EdgeEval ev;
    vector<double> v(M, 0.0), lam(M, 0.0);
    const int ti = cx.types[i];
    for (int e = cx.row[i]; e < cx.row[i + 1]; ++e) {
      const Edge& ed = cx.edges[e];
      const int tj = cx.types[ed.j];
      eval_edge(m, po, ed, ti, tj, ev, false);
      for (int b = 0; b < m.NB; ++b) {
        const int mu = basic_mu(m, b);
        double x3 = wfac(m, po, tj, mu);
        if (m.gated) x3 += m.gate_add[tj * F + mu] * h[static_cast<size_t>(ed.j) * F + mu];
        v[b] += wfac(m, po, ti, mu) * x3 * ev.R[mu] * ev.Y[basic_h(m, b)];
      }
    }
    contract_graph_forward(m, po, v, nullptr);
    const double coef = m.species_readout ? 1.0 : m.species[ti];
    const int off = m.species_readout ? ti * m.S : 0;
    double E = m.species[ti] + m.shift[ti];
    for (int q = 0; q < m.S; ++q) {
      E += coef * m.linear[off + q] * v[m.smap[q]];
      lam[m.smap[q]] += coef * m.linear[off + q];
      if (res.desc) res.desc[static_cast<size_t>(i) * m.S + q] = v[m.smap[q]];
    }
    res.site[i] = E;
    contract_graph_reverse(m, po, v, nullptr, lam, nullptr, nullptr);
    for (int e = cx.row[i]; e < cx.row[i + 1]; ++e) {
      const Edge& ed = cx.edges[e];
      const int tj = cx.types[ed.j];
      eval_edge(m, po, ed, ti, tj, ev, false);
      V3 g{0, 0, 0};
      for (int b = 0; b < m.NB; ++b) {
        const int mu = basic_mu(m, b), hh = basic_h(m, b);
        const double x0 = wfac(m, po, ti, mu);
        double x3 = wfac(m, po, tj, mu);
        if (m.gated) {
          const double al = m.gate_add[tj * F + mu];
          x3 += al * h[static_cast<size_t>(ed.j) * F + mu];
          hbar_edge[static_cast<size_t>(e) * F + mu] += lam[b] * x0 * al * ev.R[mu] * ev.Y[hh];
        }
        const double adj = lam[b] * x0 * x3;
        for (int q = 0; q < 3; ++q) g[q] += adj * (ev.Rd[mu] * ev.u[q] * ev.Y[hh] + ev.R[mu] * ev.dY[3 * hh + q]);
      }
      res.g[e] = g;
    }
  }
  if (m.gated) {
    vector<double> hbar(static_cast<size_t>(cx.n) * F, 0.0);
    for (size_t e = 0; e < E; ++e)
      for (int mu = 0; mu < F; ++mu) hbar[static_cast<size_t>(cx.edges[e].j) * F + mu] += hbar_edge[e * F + mu];
#pragma omp parallel for schedule(dynamic, 4) num_threads(threads)
    for (int i = 0; i < ncentres; ++i) {
      EdgeEval ev;
      const int ti = cx.types[i];
      vector<double> v(gmom.begin() + static_cast<size_t>(i) * M, gmom.begin() + static_cast<size_t>(i + 1) * M), lam(M, 0.0);
      for (int q = 0; q < m.Q; ++q) {
        double s = 0;
        for (int mu = 0; mu < F; ++mu) s += hbar[static_cast<size_t>(i) * F + mu] * m.gate_weight(mu, q);
        lam[m.gnodes[q]] += s;
      }
      contract_graph_reverse(m, pg, v, nullptr, lam, nullptr, nullptr);
      for (int e = cx.row[i]; e < cx.row[i + 1]; ++e) {
        const Edge& ed = cx.edges[e];
        const int tj = cx.types[ed.j];
        eval_edge(m, pg, ed, ti, tj, ev, false);
        for (int b = 0; b < m.NB; ++b) {
          const int mu = basic_mu(m, b), hh = basic_h(m, b);
          const double adj = lam[b] * wfac(m, pg, ti, mu) * wfac(m, pg, tj, mu);
          for (int q = 0; q < 3; ++q) res.g[e][q] += adj * (ev.Rd[mu] * ev.u[q] * ev.Y[hh] + ev.R[mu] * ev.dY[3 * hh + q]);
        }
      }
    }
  }
  res.energy = 0;
  for (double x : res.site) res.energy += x;
}

void finish(const Ctx& cx, const Result& res, double* forces, double* virial) {
  if (forces) std::fill(forces, forces + 3 * cx.n, 0.0);
  double w[6] = {0, 0, 0, 0, 0, 0};
  for (size_t e = 0; e < cx.edges.size(); ++e) {
    const Edge& ed = cx.edges[e];
    const V3& g = res.g[e];
    if (forces)
      for (int q = 0; q < 3; ++q) { forces[3 * ed.i + q] += g[q]; forces[3 * ed.j + q] -= g[q]; }
    w[0] -= ed.d[0] * g[0]; w[1] -= ed.d[1] * g[1]; w[2] -= ed.d[2] * g[2];
    w[3] -= ed.d[0] * g[1]; w[4] -= ed.d[0] * g[2]; w[5] -= ed.d[1] * g[2];
  }
  if (virial) std::copy(w, w + 6, virial);
}

void set_err(char* err, int len, const char* msg) {
  if (err && len > 0) { std::strncpy(err, msg, len - 1); err[len - 1] = 0; }
}

// ----------------------------------------------------------------------------------------------
// parameter gradient: forward tangents along the edge weights, then reverse
// ----------------------------------------------------------------------------------------------
struct EdgeTan {
  double rdot;
  vector<double> Ydot;   // H
};

void edge_tangent(const Model& m, const EdgeEval& ev, const V3& w, EdgeTan& t) {
  t.rdot = ev.u[0] * w[0] + ev.u[1] * w[1] + ev.u[2] * w[2];
  t.Ydot.assign(m.H, 0.0);
  for (int h = 0; h < m.H; ++h) t.Ydot[h] = ev.dY[3 * h] * w[0] + ev.dY[3 * h + 1] * w[1] + ev.dY[3 * h + 2] * w[2];
}

// Per-edge parameter contributions for one pass.  dR[mu] = dJ/dR_mu, dRd[mu] = dJ/dR'_mu.
void radial_param_grad(const Model& m, const Pass& p, const EdgeEval& ev, int ti, int tj, const vector<double>& dR,
                       const vector<double>& dRd, double* grad) {
  const int Lp = m.L + 1, C = m.C;
  for (int mu = 0; mu < m.F; ++mu) {
    if (dR[mu] == 0 && dRd[mu] == 0) continue;
    const int k = mu / Lp, l = mu % Lp;
    if (l > 0 && !(ev.r < m.rang)) continue;
    const Rad& rd = ev.rad[mu];
    double ds = 0, dg = 0;
    for (int b = 0; b < m.B; ++b) {
      const double c = (*p.coeff)[static_cast<size_t>(mu) * p.stride + b];
      grad[p.coeff_off + mu * p.stride + b] += dR[mu] * rd.v[b] + dRd[mu] * rd.r[b];
      ds += c * (dR[mu] * rd.s[b] + dRd[mu] * rd.sr[b]);
      dg += c * (dR[mu] * rd.g[b] + dRd[mu] * rd.gr[b]);
    }
    const int sb = sblock(m, k, l), pair = ti * C + tj;
    grad[p.scal_off + 2 * sb * C * C + pair] += ds;
    grad[p.scal_off + (2 * sb + 1) * C * C + pair] += dg;
  }
}

// gate_x > 0 adds the Effect gate-x L2 term of the reference objective for this configuration
// (MLMTPR::AddTwoLayerGateX2Penalty, dev_src/mtpr_sh.cpp:5869-6047, default coefficient 1e-4 in
// NonLinearRegression, non_linear_regression.h:128): P = sum over edges (i -> j) of
// norm(t_j) sum_mu (alpha(t_j, mu) h_j[mu])^2, norm(t) = gate_x / (active types x F x edges whose
// neighbour type is t); *penalty receives P and grad receives dP/dtheta (direct alpha part, and
// dP/dh_j through the gate chain like the outer pass's gate-signal adjoint).
void gradient(const Ctx& cx, const double* ew, const double* fw, const double* sw, double* grad, double gate_x = 0.0,
              double* penalty = nullptr) {
  const Model& m = *cx.m;
  const int F = m.F, M = m.M, N = cx.n, Lp = m.L + 1;
  const Pass po = outer_pass(m), pg = gate_pass(m);
  const size_t E = cx.edges.size();
  vector<V3> wv(E);
  for (size_t e = 0; e < E; ++e) {
    const Edge& ed = cx.edges[e];
    for (int a = 0; a < 3; ++a) {
      wv[e][a] = fw[3 * ed.i + a] - fw[3 * ed.j + a];
      for (int b = 0; b < 3; ++b) wv[e][a] += sw[3 * a + b] * ed.d[b];
    }
  }
  // gate forward with tangents
  vector<double> h(static_cast<size_t>(N) * F, 0.0), hd(static_cast<size_t>(N) * F, 0.0);
  vector<vector<double>> G(N), Gd(N);
  if (m.gated) {
    for (int i = 0; i < N; ++i) {
      EdgeEval ev;
      EdgeTan tn;
      vector<double> v(M, 0.0), vd(M, 0.0);
      for (int e = cx.row[i]; e < cx.row[i + 1]; ++e) {
        const Edge& ed = cx.edges[e];
        const int ti = cx.types[ed.i], tj = cx.types[ed.j];
        eval_edge(m, pg, ed, ti, tj, ev);
        edge_tangent(m, ev, wv[e], tn);
        for (int b = 0; b < m.NB; ++b) {
          const int mu = basic_mu(m, b), hh = basic_h(m, b);
          const double x = wfac(m, pg, ti, mu) * wfac(m, pg, tj, mu);
          v[b] += x * ev.R[mu] * ev.Y[hh];
          vd[b] += x * (ev.Rd[mu] * tn.rdot * ev.Y[hh] + ev.R[mu] * tn.Ydot[hh]);
        }
      }
      contract_graph_forward(m, pg, v, &vd);
      for (int mu = 0; mu < F; ++mu) {
        double s = 0, sd = 0;
        for (int q = 0; q < m.Q; ++q) { s += m.gate_weight(mu, q) * v[m.gnodes[q]]; sd += m.gate_weight(mu, q) * vd[m.gnodes[q]]; }
        h[static_cast<size_t>(i) * F + mu] = s;
        hd[static_cast<size_t>(i) * F + mu] = sd;
      }
      G[i] = v;
      Gd[i] = vd;
    }
  }
  vector<double> lh(static_cast<size_t>(N) * F, 0.0), mh(static_cast<size_t>(N) * F, 0.0);
  // outer forward + reverse per atom
  for (int i = 0; i < N; ++i) {
    EdgeEval ev;
    EdgeTan tn;
    const int ti = cx.types[i];
    vector<double> v(M, 0.0), vd(M, 0.0), lam(M, 0.0), mu_(M, 0.0);
    for (int e = cx.row[i]; e < cx.row[i + 1]; ++e) {
      const Edge& ed = cx.edges[e];
      const int tj = cx.types[ed.j];
      eval_edge(m, po, ed, ti, tj, ev);
      edge_tangent(m, ev, wv[e], tn);
      for (int b = 0; b < m.NB; ++b) {
        const int mu = basic_mu(m, b), hh = basic_h(m, b);
        const double x0 = wfac(m, po, ti, mu);
        double x3 = wfac(m, po, tj, mu), x3d = 0;
        if (m.gated) {
          x3 += m.gate_add[tj * F + mu] * h[static_cast<size_t>(ed.j) * F + mu];
          x3d = m.gate_add[tj * F + mu] * hd[static_cast<size_t>(ed.j) * F + mu];
        }
        v[b] += x0 * x3 * ev.R[mu] * ev.Y[hh];
        vd[b] += x0 * (x3d * ev.R[mu] * ev.Y[hh] + x3 * (ev.Rd[mu] * tn.rdot * ev.Y[hh] + ev.R[mu] * tn.Ydot[hh]));
      }
    }
    contract_graph_forward(m, po, v, &vd);
    const double coef = m.species_readout ? 1.0 : m.species[ti];
    const int off = m.species_readout ? ti * m.S : 0;
    grad[m.o_shift + ti] += ew[i];
    grad[m.o_species + ti] += ew[i];
    for (int q = 0; q < m.S; ++q) {
      const int node = m.smap[q];
      const double rho = coef * m.linear[off + q];
      lam[node] += ew[i] * rho;
      mu_[node] += rho;
      grad[m.o_linear + off + q] += coef * (ew[i] * v[node] + vd[node]);
      if (!m.species_readout) grad[m.o_species + ti] += m.linear[q] * (ew[i] * v[node] + vd[node]);
    }
    contract_graph_reverse(m, po, v, &vd, lam, &mu_, grad);
    for (int e = cx.row[i]; e < cx.row[i + 1]; ++e) {
      const Edge& ed = cx.edges[e];
      const int tj = cx.types[ed.j];
      eval_edge(m, po, ed, ti, tj, ev);
      edge_tangent(m, ev, wv[e], tn);
      vector<double> dR(F, 0.0), dRd(F, 0.0);
      for (int mu = 0; mu < F; ++mu) {
        const int k = mu / Lp, l = mu % Lp;
        double S = 0, T = 0, U = 0;
        for (int mm = -l; mm <= l; ++mm) {
          // basic index of (k, l, mm)
          int b = -1;
          for (int q = 0; q < m.NB; ++q) if (m.basic[q][0] == k && m.basic[q][1] == l && m.basic[q][2] == mm) { b = q; break; }
          if (b < 0) continue;
          const int hh = hidx(l, mm);
          S += lam[b] * ev.Y[hh];
          T += mu_[b] * ev.Y[hh];
          U += mu_[b] * tn.Ydot[hh];
        }
        const double x0 = wfac(m, po, ti, mu);
        double x3 = wfac(m, po, tj, mu), x3d = 0, al = 0, hj = 0, hdj = 0;
        if (m.gated) {
          al = m.gate_add[tj * F + mu];
          hj = h[static_cast<size_t>(ed.j) * F + mu];
          hdj = hd[static_cast<size_t>(ed.j) * F + mu];
          x3 += al * hj;
          x3d = al * hdj;
        }
        const double R = ev.R[mu], Rd = ev.Rd[mu];
        // J_edge = x0 [x3 (R (S + U) + Rd rdot T) + x3d R T]
        const double Qv = R * (S + U) + Rd * tn.rdot * T;
        dR[mu] = x0 * (x3 * (S + U) + x3d * T);
        dRd[mu] = x0 * x3 * tn.rdot * T;
        const double dx0 = x3 * Qv + x3d * R * T;
        const double dtau_j = x0 * Qv;
        grad[wfac_index(m, po, ti, mu)] += dx0;
        grad[wfac_index(m, po, tj, mu)] += dtau_j;
        if (m.gated) {
          grad[m.o_gadd + tj * F + mu] += x0 * (Qv * hj + R * T * hdj);
          lh[static_cast<size_t>(ed.j) * F + mu] += x0 * al * Qv;
          mh[static_cast<size_t>(ed.j) * F + mu] += x0 * al * R * T;
        }
      }
      radial_param_grad(m, po, ev, ti, tj, dR, dRd, grad);
    }
  }
  if (!m.gated) return;
  if (gate_x > 0.0) {
    vector<long long> count(m.C, 0);
    for (size_t e = 0; e < E; ++e) ++count[cx.types[cx.edges[e].j]];
    int active = 0;
    for (long long c : count) active += c > 0;
    double P = 0.0;
    for (size_t e = 0; e < E; ++e) {
      const int j = cx.edges[e].j, t = cx.types[j];
      const double norm = gate_x / (double(active) * F * double(count[t]));
      for (int mu = 0; mu < F; ++mu) {
        const double al = m.gate_add[t * F + mu], hj = h[static_cast<size_t>(j) * F + mu], x = al * hj;
        P += norm * x * x;
        grad[m.o_gadd + t * F + mu] += 2.0 * norm * x * hj;
        lh[static_cast<size_t>(j) * F + mu] += 2.0 * norm * x * al;
      }
    }
    if (penalty) *penalty = P;
  }
  // gate reverse with tangents
  for (int i = 0; i < N; ++i) {
    EdgeEval ev;
    EdgeTan tn;
    const int ti = cx.types[i];
    const vector<double>& v = G[i];
    const vector<double>& vd = Gd[i];
    vector<double> lam(M, 0.0), mu_(M, 0.0);
    for (int q = 0; q < m.Q; ++q) {
      double sl = 0, sm = 0;
      for (int mu = 0; mu < F; ++mu) {
        const double w = m.gate_weight(mu, q);
        sl += lh[static_cast<size_t>(i) * F + mu] * w;
        sm += mh[static_cast<size_t>(i) * F + mu] * w;
        grad[m.o_gw + mu * m.Q + q] += lh[static_cast<size_t>(i) * F + mu] * v[m.gnodes[q]] + mh[static_cast<size_t>(i) * F + mu] * vd[m.gnodes[q]];
      }
      lam[m.gnodes[q]] += sl;
      mu_[m.gnodes[q]] += sm;
    }
    contract_graph_reverse(m, pg, v, &vd, lam, &mu_, grad);
    for (int e = cx.row[i]; e < cx.row[i + 1]; ++e) {
      const Edge& ed = cx.edges[e];
      const int tj = cx.types[ed.j];
      eval_edge(m, pg, ed, ti, tj, ev);
      edge_tangent(m, ev, wv[e], tn);
      vector<double> dR(F, 0.0), dRd(F, 0.0);
      for (int mu = 0; mu < F; ++mu) {
        const int k = mu / Lp, l = mu % Lp;
        double S = 0, T = 0, U = 0;
        for (int mm = -l; mm <= l; ++mm) {
          int b = -1;
          for (int q = 0; q < m.NB; ++q) if (m.basic[q][0] == k && m.basic[q][1] == l && m.basic[q][2] == mm) { b = q; break; }
          if (b < 0) continue;
          const int hh = hidx(l, mm);
          S += lam[b] * ev.Y[hh];
          T += mu_[b] * ev.Y[hh];
          U += mu_[b] * tn.Ydot[hh];
        }
        const double x0 = wfac(m, pg, ti, mu), x1 = wfac(m, pg, tj, mu);
        const double R = ev.R[mu], Rd = ev.Rd[mu];
        const double Qv = R * (S + U) + Rd * tn.rdot * T;
        dR[mu] = x0 * x1 * (S + U);
        dRd[mu] = x0 * x1 * tn.rdot * T;
        grad[wfac_index(m, pg, ti, mu)] += x1 * Qv;
        grad[wfac_index(m, pg, tj, mu)] += x0 * Qv;
      }
      radial_param_grad(m, pg, ev, ti, tj, dR, dRd, grad);
    }
  }
}

Ctx make_ctx(const Model& m, int n, const double* cell, const double* pos, const int* types) {
  Ctx cx;
  cx.m = &m;
  cx.n = n;
  cx.types.assign(types, types + n);
  for (int i = 0; i < n; ++i) req(types[i] >= 0 && types[i] < m.C, "atom species index out of range");
  cx.edges = image_edges(n, cell, pos, m.rmax);
  cx.row.assign(n + 1, 0);
  for (const auto& e : cx.edges) cx.row[e.i + 1]++;
  for (int i = 0; i < n; ++i) cx.row[i + 1] += cx.row[i];
  return cx;
}

}  // namespace

extern "C" {

void* orc_load(const char* path, char* err, int errlen) {
  try {
    return new Model(load(path));
  } catch (const std::exception& e) {
    set_err(err, errlen, e.what());
    return nullptr;
  }
}

void orc_free(void* m) { delete static_cast<Model*>(m); }

int orc_param_count(void* m) { return static_cast<Model*>(m)->nparams; }

int orc_get_params(void* mp, double* out) {
  Model& m = *static_cast<Model*>(mp);
  for (int w = 0; w < 12; ++w) {
    const int o = block_offset(m, w);
    if (o < 0) continue;
    const auto* b = block(m, w);
    std::copy(b->begin(), b->end(), out + o);
  }
  return 0;
}

// The global radial scaling (the .sus2 `scaling` field; MLMTPR::scaling).
double orc_get_scaling(void* mp) { return static_cast<Model*>(mp)->scaling; }
int orc_set_scaling(void* mp, double s) {
  if (!(s > 0) || !std::isfinite(s)) return 1;
  static_cast<Model*>(mp)->scaling = s;
  return 0;
}

int orc_set_params(void* mp, const double* in) {
  Model& m = *static_cast<Model*>(mp);
  for (int w = 0; w < 12; ++w) {
    const int o = block_offset(m, w);
    if (o < 0) continue;
    auto* b = block(m, w);
    std::copy(in + o, in + o + b->size(), b->begin());
  }
  return 0;
}

long long orc_efs(void* mp, int n, const double* cell, const double* pos, const int* types, double* energy,
                  double* forces, double* virial, double* site, int threads, char* err, int errlen) {
  return orc_efs_timed(mp, n, cell, pos, types, energy, forces, virial, site, threads, nullptr, err, errlen);
}

long long orc_efs_timed(void* mp, int n, const double* cell, const double* pos, const int* types, double* energy,
                        double* forces, double* virial, double* site, int threads, double* seconds, char* err,
                        int errlen) {
  try {
    const Model& m = *static_cast<Model*>(mp);
#ifdef _OPENMP
    if (threads <= 0) threads = omp_get_max_threads();
    omp_set_num_threads(threads);
#else
    threads = 1;
#endif
    const auto t0 = std::chrono::steady_clock::now();
    Ctx cx = make_ctx(m, n, cell, pos, types);
    const auto t1 = std::chrono::steady_clock::now();
    Result res;
    evaluate(cx, n, res, threads);
    if (energy) *energy = res.energy;
    if (site) std::copy(res.site.begin(), res.site.end(), site);
    finish(cx, res, forces, virial);
    const auto t2 = std::chrono::steady_clock::now();
    if (seconds) {
      seconds[0] = std::chrono::duration<double>(t1 - t0).count();
      seconds[1] = std::chrono::duration<double>(t2 - t1).count();
    }
    return static_cast<long long>(cx.edges.size());
  } catch (const std::exception& e) {
    set_err(err, errlen, e.what());
    return -1;
  }
}

long long orc_edges(void* mp, int n, const double* cell, const double* pos, long long cap, int* ei, int* ej,
                    double* d, char* err, int errlen) {
  try {
    const Model& m = *static_cast<Model*>(mp);
    const vector<Edge> edges = image_edges(n, cell, pos, m.rmax);
    for (size_t k = 0; k < edges.size() && static_cast<long long>(k) < cap; ++k) {
      if (ei) ei[k] = edges[k].i;
      if (ej) ej[k] = edges[k].j;
      if (d) for (int q = 0; q < 3; ++q) d[3 * k + q] = edges[k].d[q];
    }
    return static_cast<long long>(edges.size());
  } catch (const std::exception& e) {
    set_err(err, errlen, e.what());
    return -1;
  }
}

int orc_efs_edges(void* mp, int nowned, int nall, const int* types, int nedges, const int* ei, const int* ej,
                  const double* d, double* energy, double* forces, double* virial, double* site, char* err, int errlen) {
  try {
    const Model& m = *static_cast<Model*>(mp);
    Ctx cx;
    cx.m = &m;
    cx.n = nall;
    cx.types.assign(types, types + nall);
    vector<int> order(nedges);
    for (int q = 0; q < nedges; ++q) order[q] = q;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return ei[a] < ei[b]; });
    for (int q : order) cx.edges.push_back({ei[q], ej[q], {d[3 * q], d[3 * q + 1], d[3 * q + 2]}});
    cx.row.assign(nall + 1, 0);
    for (const auto& e : cx.edges) { req(e.i >= 0 && e.i < nowned && e.j >= 0 && e.j < nall, "edge index out of range"); cx.row[e.i + 1]++; }
    for (int i = 0; i < nall; ++i) cx.row[i + 1] += cx.row[i];
    Result res;
    req(!m.gated || nowned == nall, "Effect edge lists need all atoms owned");
    evaluate(cx, nowned, res, 1);
    if (energy) *energy = res.energy;
    if (site) std::copy(res.site.begin(), res.site.end(), site);
    finish(cx, res, forces, virial);
    return 0;
  } catch (const std::exception& e) {
    set_err(err, errlen, e.what());
    return -1;
  }
}

int orc_grad(void* mp, int n, const double* cell, const double* pos, const int* types, const double* ew,
             const double* fw, const double* sw, double* grad, char* err, int errlen) {
  try {
    const Model& m = *static_cast<Model*>(mp);
    Ctx cx = make_ctx(m, n, cell, pos, types);
    gradient(cx, ew, fw, sw, grad);
    return 0;
  } catch (const std::exception& e) {
    set_err(err, errlen, e.what());
    return -1;
  }
}

// Per-atom descriptors of one periodic frame: the S scalar moments after the product graph
// (MLMTPR::CalcDescriptors, dev_src/mtpr.cpp:6554: basis_vals[1 + q] per atom), desc[n][S].
int orc_descriptors(void* mp, int n, const double* cell, const double* pos, const int* types, double* desc, char* err,
                    int errlen) {
  try {
    const Model& m = *static_cast<Model*>(mp);
    Ctx cx = make_ctx(m, n, cell, pos, types);
    Result res;
    res.desc = desc;
    evaluate(cx, n, res, 1);
    return 0;
  } catch (const std::exception& e) {
    set_err(err, errlen, e.what());
    return -1;
  }
}

// Dimensions and parameter offsets: out[12] = {C, S, B, F, species_readout, o_shift, o_radial,
// o_species, o_linear, nparams, nblk, K}.
int orc_layout(void* mp, int* out) {
  const Model& m = *static_cast<Model*>(mp);
  const int v[12] = {m.C, m.S, m.B, m.F, m.species_readout ? 1 : 0, m.o_shift, m.o_radial, m.o_species, m.o_linear,
                     m.nparams, m.nblk, m.K};
  for (int q = 0; q < 12; ++q) out[q] = v[q];
  return 0;
}

int orc_grad_gatex(void* mp, int n, const double* cell, const double* pos, const int* types, const double* ew,
                   const double* fw, const double* sw, double gate_x, double* grad, double* penalty, char* err,
                   int errlen) {
  try {
    const Model& m = *static_cast<Model*>(mp);
    Ctx cx = make_ctx(m, n, cell, pos, types);
    *penalty = 0.0;
    gradient(cx, ew, fw, sw, grad, gate_x, penalty);
    return 0;
  } catch (const std::exception& e) {
    set_err(err, errlen, e.what());
    return -1;
  }
}

}  // extern "C"
