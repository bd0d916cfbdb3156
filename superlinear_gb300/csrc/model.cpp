// .sus2 reader, validation and derived per-atom graph schedules (host side).
// Semantics follow interfaces/lammps/ML-SUS2/sus2_sl_model.cpp (Model::load :174-257,
// Model::validate :258-453) and sus2_sl_kernel.cpp:45-106 (Kernel::Kernel), restricted to the
// Static and Effect families; defaults for absent coefficient blocks are the reader's.
#include "model.h"

#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <limits>
#include <set>
#include <sstream>

namespace sus2g {
namespace {

std::string trim(const std::string& s) {
  const auto a = s.find_first_not_of(" \t\r\n");
  return a == std::string::npos ? "" : s.substr(a, s.find_last_not_of(" \t\r\n") - a + 1);
}

void require(bool ok, const std::string& why) {
  if (!ok) throw Error(3, "SUS2 model: " + why);
}

// Brace lists nest arbitrarily; numbers are separated by commas (sus2_sl_model.cpp:103-122).
void list_values(const char*& p, std::vector<double>& out, const std::string& key) {
  while (*p && std::isspace(static_cast<unsigned char>(*p))) ++p;
  require(*p == '{', "expected list in " + key);
  ++p;
  while (true) {
    while (*p && std::isspace(static_cast<unsigned char>(*p))) ++p;
    if (*p == '}') { ++p; return; }
    if (*p == '{') {
      list_values(p, out, key);
    } else {
      char* end = nullptr;
      const double x = std::strtod(p, &end);
      require(end != p && std::isfinite(x), "invalid finite number in " + key);
      out.push_back(x);
      p = end;
    }
    while (*p && std::isspace(static_cast<unsigned char>(*p))) ++p;
    if (*p == '}') { ++p; return; }
    require(*p == ',', "missing list separator in " + key);
    ++p;
  }
}

int exact_int(double x, const std::string& key) {
  require(std::isfinite(x) && std::floor(x) == x && std::fabs(x) < 2e9, "noninteger " + key);
  return static_cast<int>(x);
}

}  // namespace

std::string Model::text(const std::string& k, const std::string& fb) const {
  auto it = fields.find(k);
  return it == fields.end() ? fb : it->second;
}
double Model::real(const std::string& k, double fb) const {
  if (!has(k)) return fb;
  const std::string s = text(k);
  char* end = nullptr;
  const double v = std::strtod(s.c_str(), &end);
  require(end != s.c_str() && trim(end).empty() && std::isfinite(v), "invalid number " + k);
  return v;
}
int Model::integer(const std::string& k, int fb) const { return has(k) ? exact_int(real(k), k) : fb; }
bool Model::boolean(const std::string& k, bool fb) const {
  if (!has(k)) return fb;
  const auto s = text(k);
  require(s == "true" || s == "false" || s == "0" || s == "1", "invalid boolean " + k);
  return s == "true" || s == "1";
}
std::vector<double> Model::numbers(const std::string& k) const {
  if (!has(k)) return {};
  const std::string s = text(k);
  const char* p = s.c_str();
  std::vector<double> out;
  list_values(p, out, k);
  require(trim(p).empty(), "trailing list text in " + k);
  return out;
}
std::vector<int> Model::integers(const std::string& k) const {
  std::vector<int> out;
  for (double x : numbers(k)) out.push_back(exact_int(x, k));
  return out;
}

void Model::load(const std::string& path) {
  *this = Model();
  std::ifstream in(path.c_str());
  if (!in) throw Error(2, "cannot open model " + path);
  std::string line, radial_text;
  bool radial = false, header = false;
  while (std::getline(in, line)) {
    line = trim(line);
    if (line.empty() || line[0] == '#') continue;
    if (!header) { require(line == "MTP", "missing MTP header"); header = true; continue; }
    const size_t eq = line.find('=');
    if (eq == std::string::npos) {
      if (line == "radial_coeffs") {
        require(!radial && radial_text.empty(), "duplicate radial_coeffs");
        radial = true;
        field_order.push_back("radial_coeffs");
        continue;
      }
      require(radial, "unrecognized line: " + line);
      if (line == "0-0") continue;
      require(line[0] == '{', "invalid radial coefficient block");
      if (!radial_text.empty()) radial_text += ",";
      radial_text += line;
      continue;
    }
    radial = false;
    const std::string key = trim(line.substr(0, eq));
    std::string value = trim(line.substr(eq + 1));
    require(!key.empty() && !has(key), "duplicate or empty field " + key);
    int depth = 0;
    for (char c : value) depth += (c == '{') - (c == '}');
    while (depth > 0 && std::getline(in, line)) {
      value += " " + trim(line);
      for (char c : line) depth += (c == '{') - (c == '}');
    }
    require(depth == 0, "unbalanced braces in " + key);
    fields[key] = value;
    field_order.push_back(key);
  }
  require(header, "empty model");
  C = integer("species_count"); L = integer("sh_l_max"); K = integer("sh_k_max");
  B = integer("radial_basis_size"); F = integer("radial_funcs_count");
  M = integer("alpha_moments_count"); S = integer("alpha_scalar_moments");
  min_dist = real("min_dist"); max_dist = real("max_dist");
  angular = real("angular_max_dist", max_dist); scaling = real("scaling", 1);
  require(C > 0 && C <= 64 && B > 0 && B <= 16 && K > 0 && L >= 0 && L <= 5 && F > 0,
          "unsupported species/radial dimensions (C<=64, B<=16, L<=5)");
  H = (L + 1) * (L + 1);
  const std::string sm = text("scaling_map", "LK");
  scaling_mode = sm == "pair" ? 0 : sm == "L" ? 1 : sm == "K" ? 2 : 3;
  nblk = scaling_mode == 0 ? 1 : scaling_mode == 1 ? L + 1 : scaling_mode == 2 ? K : F;
  // Absent coefficient blocks take the reader's defaults (sus2_sl_model.cpp:205-232).
  if (!radial_text.empty()) fields["radial_coeffs"] = "{" + radial_text + "}";
  this->radial = numbers("radial_coeffs");
  if (this->radial.empty()) {
    this->radial.assign(static_cast<size_t>(F) * (B + C), 0.01);
    for (int mu = 0; mu < F; ++mu)
      for (int t = 0; t < C; ++t) this->radial[static_cast<size_t>(mu) * (B + C) + B + t] = 2.0;
  }
  shift = numbers("shift_coeffs");
  if (shift.empty()) shift.assign(C, -1.0);
  scal = numbers("scal_coeffs");
  if (scal.empty()) {
    const int pairs = C * C;
    scal.assign(2 * pairs * nblk, 0.0);
    const double start = text("radial_basis_type").find("RBLaguerre_log1p") == 0 ? 3. : 4.;
    for (int b = 0; b < nblk; ++b)
      for (int t = 0; t < C; ++t)
        for (int u = 0; u < C; ++u) {
          const double x = C == 1 ? .5 : (std::sqrt(t + 1.) + std::sqrt(u + 1.) - 2.) / (2. * std::sqrt(double(C)) - 2.);
          scal[2 * b * pairs + t * C + u] = start + (2. - start) * x;
          scal[(2 * b + 1) * pairs + t * C + u] = 1.5 + x;
        }
  }
  species_readout = text("readout_mode", "shared") == "species";
  species = numbers("species_coeffs");
  linear = numbers("moment_coeffs");
  if (species.empty()) {
    require(linear.empty(), "moment_coeffs without species_coeffs");
    species.assign(C, 0.001);
    linear.assign(static_cast<size_t>(S) * (species_readout ? C : 1), species_readout ? 1e-6 : 0.001);
  }
  {
    const auto v = numbers("alpha_index_basic");
    require(v.size() % 3 == 0, "invalid row width in alpha_index_basic");
    for (size_t i = 0; i < v.size(); i += 3)
      basic.push_back({exact_int(v[i], "basic k"), exact_int(v[i + 1], "basic l"), exact_int(v[i + 2], "basic m")});
  }
  {
    const auto v = numbers("sh_products");
    require(v.size() % 4 == 0, "invalid row width in sh_products");
    for (size_t i = 0; i < v.size(); i += 4)
      products.push_back({exact_int(v[i], "product a"), exact_int(v[i + 1], "product b"), exact_int(v[i + 2], "product out"), v[i + 3]});
  }
  scalar_map = integers("alpha_moment_mapping");
  NB = static_cast<int>(basic.size());
  P = static_cast<int>(products.size());
  validate();
  derive();
}

void Model::validate() {
  const auto ver = text("version");
  static const std::set<std::string> versions = {"1.1.0", "1.2.0", "1.3.0", "1.4.0", "1.5.0", "1.6.0", "1.7.0", "1.8.0"};
  require(versions.count(ver) != 0, "unsupported version " + ver);
  require(text("potential_tag") == "SUS2-SH", "requires a SUS2-SH spherical harmonic model");
  require(integer("L") == L && static_cast<long long>(K) * (L + 1) == F, "inconsistent L/K dimensions");
  require(integer("sh_body_order") >= 2 && integer("sh_body_order") <= 6 && text("sh_parity") == "even",
          "unsupported body order or parity");
  require(max_dist > min_dist && min_dist >= 0 && scaling > 0, "invalid distance or scaling");
  require(std::isfinite(angular) && angular > 0 && angular <= max_dist, "angular_max_dist must be in (0,max_dist]");
  split = angular != max_dist;
  require(text("radial_basis_type") == "RBChebyshev_sss",
          "this engine evaluates the RBChebyshev_sss radial basis only");
  const std::string cut = text("radial_cutoff_type", "legacy");
  require(cut == "legacy" || cut == "polynomial", "radial_cutoff_type should be legacy or polynomial");
  poly_cutoff = cut == "polynomial";
  cutoff_p = integer("radial_cutoff_p", 5);
  require(cutoff_p >= 1 && cutoff_p <= 64, "radial_cutoff_p should be in [1, 64]");
  require(shift.size() == static_cast<size_t>(C) && species.size() == static_cast<size_t>(C), "wrong species coefficient count");
  require(scal.size() == static_cast<size_t>(2) * C * C * nblk, "wrong coefficient count in scal_coeffs");
  require(radial.size() == static_cast<size_t>(F) * (B + C), "wrong radial coefficient count");
  require(M > 0 && NB == integer("alpha_index_basic_count") && M >= NB, "invalid basic graph dimensions");
  require(P == integer("sh_product_count"), "wrong sh_product_count");
  require(integer("alpha_index_times_count") == 0 && numbers("alpha_index_times").empty(), "Cartesian product graph is unsupported");
  for (const auto& b : basic)
    require(b[0] >= 0 && b[0] < K && b[1] >= 0 && b[1] <= L && b[2] >= -b[1] && b[2] <= b[1], "invalid basic (k,l,m)");
  for (const auto& p : products)
    require(p.a >= 0 && p.b >= 0 && p.out >= 0 && p.a < p.out && p.b < p.out && p.out < M, "invalid or cyclic product graph");
  require(scalar_map.size() == static_cast<size_t>(S), "wrong scalar mapping count");
  for (int i : scalar_map) require(i >= 0 && i < M, "scalar mapping out of range");
  require(linear.size() == static_cast<size_t>(S) * (species_readout ? C : 1), "wrong coefficient count in moment_coeffs");
  const std::string outer = text("outer_radial_mode", "legacy-plus-mixer");
  require(outer == "legacy-plus-mixer", "outer_radial_mode " + outer + " is outside this engine (Static/Effect legacy-plus-mixer)");
  require(!has("two_layer_gate_radial_mixing"), "two_layer_gate_radial_mixing is outside this engine");
  require(!boolean("two_layer_residual_enabled") && !boolean("multi_layer_gate_enabled") &&
          !boolean("two_layer_gate_edge_l1_enabled") && !boolean("joint_readout_enabled") &&
          !boolean("zbl_enabled") && !boolean("two_layer_gate_readout_enabled"),
          "residual/multilayer/edge-L1/joint/ZBL/gate-readout variants are outside this engine");
  const std::string channel = text("outer_channel_mode", "cross-channel");
  require(channel == "cross-channel" || channel == "same-channel", "invalid outer_channel_mode");
  if (boolean("outer_k_rank1_enabled")) {
    outer_rank = integer("outer_k_rank", 1);
    outer_begin = integer("outer_k_rank1_basic_begin");
    outer_product = integer("outer_k_rank1_product_begin");
    const int n = integer("outer_k_rank1_basic_count");
    require(outer_rank > 0 && outer_rank <= K, "invalid outer rank");
    require(n == outer_rank * H && outer_begin >= NB && outer_begin + n <= M && outer_product >= 0 && outer_product <= P,
            "invalid outer rank graph segment");
    outer_w = numbers("outer_k_rank1_weights");
    require(outer_w.empty() || outer_w.size() == static_cast<size_t>(L + 1) * outer_rank * K, "invalid outer contraction weights");
  }
  gate_rank = integer("two_layer_gate_k_rank");
  if (gate_rank > 0) {
    gate_begin = integer("two_layer_gate_k_rank_basic_begin");
    const int n = integer("two_layer_gate_k_rank_basic_count");
    gate_product_begin = integer("two_layer_gate_k_rank_product_begin", 0);
    const int end = integer("two_layer_gate_k_rank_product_end");
    require(gate_rank <= K && n == gate_rank * H && gate_begin >= NB && gate_begin + n <= M &&
            gate_product_begin >= 0 && end >= gate_product_begin && end <= P, "invalid gate rank graph segment");
    gate_w = numbers("two_layer_gate_k_rank_weights");
    require(gate_w.size() == static_cast<size_t>(L + 1) * gate_rank * K, "wrong coefficient count in two_layer_gate_k_rank_weights");
  }
  // gate product range (sus2_sl_kernel.cpp:94-95)
  gate_product_begin = integer("two_layer_gate_k_rank_product_begin", 0);
  gate_product_end = gate_rank ? integer("two_layer_gate_k_rank_product_end", outer_product) : outer_product;
  if (!outer_rank && !gate_rank) gate_product_end = P;
  gated = boolean("two_layer_gate_enabled");
  if (gated) {
    require(text("two_layer_gate_site_mode", "neighbor") == "neighbor", "center-gate mode is not implemented");
    const std::string mode = text("two_layer_gate_mode");
    require(mode == "mu-scalar-full" || mode == "mu-body-linear-combo" || mode == "mu-body-order",
            "unsupported gate mode " + mode);
    body_combo = mode == "mu-body-linear-combo";
    gate_nodes = integers("two_layer_gate_scalar_moment_indices");
    if (gate_nodes.empty())
      for (int q : integers("two_layer_gate_scalar_indices")) {
        require(q >= 0 && q < S, "gate scalar index out of range");
        gate_nodes.push_back(scalar_map[q]);
      }
    Q = static_cast<int>(gate_nodes.size());
    require(Q > 0, "empty gate scalar basis");
    for (int x : gate_nodes) require(x >= 0 && x < M, "gate moment out of range");
    gate_body = integers("two_layer_gate_scalar_body_orders");
    body_count = integer("two_layer_gate_body_order_max") - 1;
    gate_weights = numbers("two_layer_gate_weights");
    if (body_combo) {
      body_mix = numbers("two_layer_gate_body_mix_weights");
      require(gate_weights.size() >= static_cast<size_t>(Q) && gate_body.size() == static_cast<size_t>(Q) &&
              body_mix.size() == static_cast<size_t>(F) * body_count, "invalid body-combo gate weights");
    } else {
      require(gate_weights.size() == static_cast<size_t>(F) * Q, "wrong coefficient count in two_layer_gate_weights");
    }
    const std::string radial_mode = text("two_layer_gate_radial_mode", "base-radial");
    gate_shared_radial = radial_mode == "shared-radial";
    gate_radial = numbers("two_layer_gate_radial_coeffs");
    if (gate_shared_radial)
      require(gate_radial.size() == static_cast<size_t>(F) * B, "wrong coefficient count in two_layer_gate_radial_coeffs");
    else
      require(gate_radial.empty(), "gate radial coefficients require shared-radial mode");
    const std::string gs = text("two_layer_gate_scaling_mode", "shared-scaling");
    gate_decoupled = gs == "decoupled";
    gate_scal = numbers("two_layer_gate_scaling_coeffs");
    if (gate_decoupled) require(gate_scal.size() == scal.size(), "wrong coefficient count in two_layer_gate_scaling_coeffs");
    else require(gate_scal.empty(), "independent gate warps require decoupled scaling");
    // Element rows (one value per species) are broadcast to every radial function; missing
    // rows fall back to the outer tau (type) and 1 (additive) as Kernel::Kernel does.
    auto expand = [&](const std::string& key, bool from_tau) {
      std::vector<double> v = numbers(key), out(static_cast<size_t>(C) * F);
      for (int t = 0; t < C; ++t)
        for (int mu = 0; mu < F; ++mu) {
          const size_t idx = static_cast<size_t>(t) * F + mu;
          double x;
          if (idx < v.size()) x = v[idx];
          else if (v.size() == static_cast<size_t>(C) && !v.empty()) x = v[t];
          else if (v.empty() && from_tau) x = radial[static_cast<size_t>(mu) * (B + C) + B + t];
          else x = v.empty() ? 1.0 : (static_cast<size_t>(t) < v.size() ? v[t] : 1.0);
          out[idx] = x;
        }
      return out;
    };
    gate_type = expand("two_layer_gate_type_coeffs", true);
    gate_add = expand("two_layer_gate_additive_coeffs", false);
  }
}

double Model::gate_weight(int mu, int q) const {
  if (!body_combo) return gate_weights.at(static_cast<size_t>(mu) * Q + q);
  return gate_weights.at(q) * body_mix.at(static_cast<size_t>(mu) * body_count + gate_body.at(q) - 2);
}

GraphSchedule build_schedule(const std::vector<Product>& products, int begin, int end, int nodes) {
  GraphSchedule g;
  std::vector<int> level(nodes, 0);
  std::vector<std::vector<int>> by_out(nodes);
  for (int p = begin; p < end; ++p) by_out[products[p].out].push_back(p);
  int maxlevel = 0;
  for (int n = 0; n < nodes; ++n) {
    if (by_out[n].empty()) continue;
    int lv = 0;
    for (int p : by_out[n]) lv = std::max(lv, std::max(level[products[p].a], level[products[p].b]));
    level[n] = lv + 1;
    maxlevel = std::max(maxlevel, lv + 1);
  }
  g.levels = maxlevel;
  // forward lists, levels 1..maxlevel
  g.level_begin.push_back(0);
  g.out_begin.push_back(0);
  for (int lv = 1; lv <= maxlevel; ++lv) {
    for (int n = 0; n < nodes; ++n)
      if (!by_out[n].empty() && level[n] == lv) {
        g.out_nodes.push_back(n);
        for (int p : by_out[n]) g.fprod.push_back(p);
        g.out_begin.push_back(static_cast<int>(g.fprod.size()));
      }
    g.level_begin.push_back(static_cast<int>(g.out_nodes.size()));
  }
  // reverse gather lists, grouped by the level of the consumed node (0..maxlevel-1)
  std::vector<std::vector<int>> consumers(nodes);  // entries index into a flat (out, other, c) list
  std::vector<int> e_out, e_other;
  std::vector<double> e_c;
  for (int p = begin; p < end; ++p) {
    const auto& q = products[p];
    consumers[q.a].push_back(static_cast<int>(e_out.size()));
    e_out.push_back(q.out); e_other.push_back(q.b); e_c.push_back(q.c);
    consumers[q.b].push_back(static_cast<int>(e_out.size()));
    e_out.push_back(q.out); e_other.push_back(q.a); e_c.push_back(q.c);
  }
  g.rlevel_begin.push_back(0);
  g.in_begin.push_back(0);
  for (int lv = 0; lv < std::max(maxlevel, 1); ++lv) {
    for (int n = 0; n < nodes; ++n)
      if (!consumers[n].empty() && level[n] == lv) {
        g.in_nodes.push_back(n);
        for (int e : consumers[n]) {
          g.rprod_out.push_back(e_out[e]);
          g.rprod_other.push_back(e_other[e]);
          g.rprod_c.push_back(e_c[e]);
        }
        g.in_begin.push_back(static_cast<int>(g.rprod_out.size()));
      }
    g.rlevel_begin.push_back(static_cast<int>(g.in_nodes.size()));
  }
  return g;
}

void Model::derive() {
  auto rows = [&](int rank, int begin, const std::vector<double>& w, std::vector<ContractionRow>& out) {
    for (int a = 0; a < rank; ++a)
      for (int b = 0; b < NB; ++b) {
        const int k = basic[b][0], l = basic[b][1], m = basic[b][2];
        const int dst = begin + rank * (H - (l + 1) * (l + 1)) + (rank - 1 - a) * (2 * l + 1) + m + l;
        out.push_back({b, dst, w.empty() ? -1 : (l * rank + a) * K + k});
      }
  };
  if (outer_rank) rows(outer_rank, outer_begin, outer_w, outer_rows);
  if (gated && gate_rank) rows(gate_rank, gate_begin, gate_w, gate_rows);
  outer_graph = build_schedule(products, outer_product, P, M);
  if (gated) gate_graph = build_schedule(products, gate_product_begin, gate_product_end, M);
}

std::vector<Model::Block> Model::layout() const {
  std::vector<Block> out;
  int off = 0;
  auto add = [&](const std::string& n, size_t s) { out.push_back({n, off, static_cast<int>(s)}); off += static_cast<int>(s); };
  add("shift_coeffs", shift.size());
  add("scal_coeffs", scal.size());
  add("radial_coeffs", radial.size());
  if (gated) {
    add("two_layer_gate_radial_coeffs", gate_radial.size());
    if (gate_decoupled) add("two_layer_gate_scaling_coeffs", gate_scal.size());
    add("two_layer_gate_additive_coeffs", gate_add.size());
    add("two_layer_gate_type_coeffs", gate_type.size());
    add("two_layer_gate_weights", gate_weights.size());
    if (body_combo) add("two_layer_gate_body_mix_weights", body_mix.size());
  }
  if (gated && gate_rank) add("two_layer_gate_k_rank_weights", gate_w.size());
  if (outer_rank && !outer_w.empty()) add("outer_k_rank1_weights", outer_w.size());
  add("species_coeffs", species.size());
  add("moment_coeffs", linear.size());
  return out;
}

void Model::set_scaling(double s) {
  if (!(s > 0) || !std::isfinite(s)) throw Error(1, "scaling must be positive and finite");
  scaling = s;
  char buf[64];
  std::snprintf(buf, sizeof(buf), "%.17e", s);
  if (!fields.count("scaling")) {
    auto it = std::find(field_order.begin(), field_order.end(), "version");
    field_order.insert(it == field_order.end() ? field_order.begin() : it + 1, "scaling");
  }
  fields["scaling"] = buf;
}

void Model::save(const std::string& path) const {
  std::map<std::string, std::string> out = fields;
  std::vector<std::string> order = field_order;
  auto place = [&](const std::string& key, const std::string& after) {
    if (std::find(order.begin(), order.end(), key) != order.end()) return;
    auto it = std::find(order.begin(), order.end(), after);
    order.insert(it == order.end() ? order.end() : it + 1, key);
  };
  static const std::map<std::string, std::string> count_keys = {
      {"two_layer_gate_radial_coeffs", "two_layer_gate_radial_coeff_count"},
      {"two_layer_gate_additive_coeffs", "two_layer_gate_additive_coeff_count"},
      {"two_layer_gate_type_coeffs", "two_layer_gate_type_coeff_count"},
      {"two_layer_gate_weights", "two_layer_gate_weight_count"},
      {"two_layer_gate_k_rank_weights", "two_layer_gate_k_rank_weight_count"},
      {"outer_k_rank1_weights", "outer_k_rank1_weight_count"}};
  char buf[64];
  auto fmt = [&](const double* v, size_t n) {
    std::string t = "{";
    for (size_t q = 0; q < n; ++q) {
      std::snprintf(buf, sizeof(buf), "%.17e", v[q]);
      if (q) t += ", ";
      t += buf;
    }
    return t + "}";
  };
  std::string prev = "scal_coeffs";
  for (const Block& b : layout()) {
    const std::vector<double>& v = *const_cast<Model*>(this)->block_ptr(b.name);
    out[b.name] = fmt(v.data(), v.size());
    place(b.name, prev);
    auto ck = count_keys.find(b.name);
    if (ck != count_keys.end()) {
      out[ck->second] = std::to_string(v.size());
      place(ck->second, b.name);
    }
    prev = b.name;
  }
  // the trainer's sequential reader wants the radial block after scal_coeffs (dev_src/mtpr.cpp:5100-5150)
  auto r = std::find(order.begin(), order.end(), "radial_coeffs");
  auto sc = std::find(order.begin(), order.end(), "scal_coeffs");
  if (r != order.end() && sc != order.end() && r < sc) {
    order.erase(r);
    sc = std::find(order.begin(), order.end(), "scal_coeffs");
    order.insert(sc + 1, "radial_coeffs");
  }
  static const std::set<std::string> radial_meta = {"scaling_inner", "min_dist", "max_dist", "angular_max_dist",
                                                    "radial_basis_size", "radial_cutoff_type", "radial_cutoff_p",
                                                    "radial_funcs_count"};
  std::ofstream os(path.c_str());
  if (!os) throw Error(2, "cannot write model " + path);
  os << "MTP\n";
  for (const std::string& key : order) {
    if (key == "radial_coeffs") {
      os << "\tradial_coeffs\n\t\t0-0\n";
      const size_t w = static_cast<size_t>(B + C);
      for (size_t row = 0; row * w < radial.size(); ++row) os << "\t\t\t" << fmt(radial.data() + row * w, w) << "\n";
      continue;
    }
    os << (radial_meta.count(key) ? "\t" : "") << key << " = " << out.at(key) << "\n";
  }
  if (!os) throw Error(2, "cannot write model " + path);
}

std::vector<double>* Model::block_ptr(const std::string& n) {
  if (n == "shift_coeffs") return &shift;
  if (n == "scal_coeffs") return &scal;
  if (n == "radial_coeffs") return &radial;
  if (n == "two_layer_gate_radial_coeffs") return &gate_radial;
  if (n == "two_layer_gate_scaling_coeffs") return &gate_scal;
  if (n == "two_layer_gate_additive_coeffs") return &gate_add;
  if (n == "two_layer_gate_type_coeffs") return &gate_type;
  if (n == "two_layer_gate_weights") return &gate_weights;
  if (n == "two_layer_gate_body_mix_weights") return &body_mix;
  if (n == "two_layer_gate_k_rank_weights") return &gate_w;
  if (n == "outer_k_rank1_weights") return &outer_w;
  if (n == "species_coeffs") return &species;
  if (n == "moment_coeffs") return &linear;
  throw Error(1, "unknown parameter block " + n);
}

int Model::param_count() const {
  int n = 0;
  for (const auto& b : layout()) n += b.size;
  return n;
}

void Model::get_params(double* out) const {
  for (const auto& b : layout()) {
    const auto* v = const_cast<Model*>(this)->block_ptr(b.name);
    std::copy(v->begin(), v->end(), out + b.offset);
  }
}

void Model::set_params(const double* in) {
  for (const auto& b : layout()) {
    auto* v = block_ptr(b.name);
    std::copy(in + b.offset, in + b.offset + b.size, v->begin());
  }
  outer_rows.clear();
  gate_rows.clear();
  derive();
}

}  // namespace sus2g
