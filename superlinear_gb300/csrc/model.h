// SUS2-SH model: .sus2 text -> validated host tables for the GPU engine.
//
// Follows the reference's standalone reader (interfaces/lammps/ML-SUS2/sus2_sl_model.cpp:174-453,
// Model::load / Model::validate) and the engine set-up in sus2_sl_kernel.cpp:45-106
// (Kernel::Kernel) for the two families on this path: Static and Effect
// (outer_radial_mode = legacy-plus-mixer, two_layer_gate_mode = mu-scalar-full or
// mu-body-linear-combo).  Other families are rejected with a clear error.
#pragma once
#include <array>
#include <map>
#include <stdexcept>
#include <string>
#include <vector>

namespace sus2g {

struct Error : std::runtime_error {
  int code;
  Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

// A cell-list centre had more edges than its padded capacity; the engine has already grown the
// capacity, and the step that raised it is to be repeated.
struct EdgeOverflow : Error {
  EdgeOverflow() : Error(9, "edge build: padded neighbour capacity exceeded (capacity grown; repeat the step)") {}
};

struct Product { int a, b, out; double c; };

// One per-atom graph evaluation schedule (forward levels and the reverse gather lists).
struct GraphSchedule {
  // forward: for each level, the output nodes and, per output, its product list
  std::vector<int> level_begin;     // [nlevels+1] offsets into out_nodes
  std::vector<int> out_nodes;       // nodes produced at each level
  std::vector<int> out_begin;       // [out_nodes+1] offsets into fprod (products of that output)
  std::vector<int> fprod;           // product indices grouped by output
  // reverse: nodes whose adjoint receives contributions, per level (reverse order processed)
  std::vector<int> rlevel_begin;    // [nlevels+1] offsets into in_nodes
  std::vector<int> in_nodes;        // nodes consumed by products, grouped by producing level
  std::vector<int> in_begin;        // [in_nodes+1] offsets into rprod
  std::vector<int> rprod_out;       // for each consumer entry: the product's output node
  std::vector<int> rprod_other;     // the other input node
  std::vector<double> rprod_c;      // coefficient (a==b products appear twice: once per input slot)
  int levels = 0;
};

struct ContractionRow { int src, dst, widx; };  // v[dst] += W[widx] * v[src]

struct Model {
  std::map<std::string, std::string> fields;
  std::vector<std::string> field_order;  // keys in file order ("radial_coeffs" at its block)
  // dimensions
  int C = 0, L = 0, K = 0, B = 0, F = 0, H = 0, M = 0, NB = 0, P = 0, S = 0;
  int nblk = 0, scaling_mode = 3;  // 0 pair, 1 L, 2 K, 3 LK
  double min_dist = 0, max_dist = 0, angular = 0, scaling = 1;
  bool split = false;               // angular cutoff below max_dist
  bool poly_cutoff = false;         // radial_cutoff_type polynomial
  int cutoff_p = 5;
  // parameters (reference .sus2 names)
  std::vector<double> shift, scal, radial;  // radial: F x (B + C)
  std::vector<double> species, linear;      // linear: S or C*S
  bool species_readout = false;
  std::vector<std::array<int, 3>> basic;    // (k, l, m)
  std::vector<Product> products;
  std::vector<int> scalar_map;
  // ranked contractions
  int outer_rank = 0, outer_begin = 0, outer_product = 0;
  int gate_rank = 0, gate_begin = 0, gate_product_begin = 0, gate_product_end = 0;
  std::vector<double> outer_w, gate_w;      // (L+1) x rank x K
  std::vector<ContractionRow> outer_rows, gate_rows;
  // Effect gate
  bool gated = false, body_combo = false, gate_decoupled = false, gate_shared_radial = false;
  std::vector<double> gate_radial;          // F x B (shared-radial) or empty -> radial
  std::vector<double> gate_scal;            // decoupled warp or empty -> scal
  std::vector<double> gate_type, gate_add;  // C x F (element rows broadcast)
  std::vector<double> gate_weights;         // F x Q (or body-combo source vectors)
  std::vector<double> body_mix;             // F x (body_max - 1)
  std::vector<int> gate_nodes, gate_body;
  int Q = 0, body_count = 0;
  // derived schedules
  GraphSchedule outer_graph, gate_graph;

  void load(const std::string& path);
  // Writes the model as a .sus2 file with the current parameter vector (MLMTPR::Save,
  // dev_src/mtpr.cpp:6893): the loaded fields in file order, the trainable blocks replaced by the
  // current values (%.17e, which reads back bit-exactly), the radial block after scal_coeffs.
  void save(const std::string& path) const;
  // flat trainable vector in the reference trainer's order (dev_src/mtpr.h, DistributeCoeffs)
  struct Block { std::string name; int offset, size; };
  std::vector<Block> layout() const;
  int param_count() const;
  void get_params(double* out) const;
  void set_params(const double* in);
  // The global radial scaling (the `scaling` field, MLMTPR::scaling): not a trained coefficient,
  // set by the trainer's rescale step and written back by save().
  void set_scaling(double s);
  double gate_weight(int mu, int q) const;  // sus2_sl_kernel.cpp:314-317

 private:
  bool has(const std::string& k) const { return fields.count(k) != 0; }
  std::string text(const std::string& k, const std::string& fb = "") const;
  double real(const std::string& k, double fb = 0) const;
  int integer(const std::string& k, int fb = 0) const;
  bool boolean(const std::string& k, bool fb = false) const;
  std::vector<double> numbers(const std::string& k) const;
  std::vector<int> integers(const std::string& k) const;
  void validate();
  void derive();
  std::vector<double>* block_ptr(const std::string& name);
};

GraphSchedule build_schedule(const std::vector<Product>& products, int begin, int end, int nodes);

}  // namespace sus2g
