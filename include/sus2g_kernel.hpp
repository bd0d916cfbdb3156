/* C++ counterpart of the reference's SUS2SL::Kernel (interfaces/lammps/ML-SUS2/sus2_sl_kernel.h:16-43)
 * over the C ABI of sus2g.h: the same begin / pack_forward / unpack_forward / outer / pack_reverse /
 * add_reverse / finish surface and the same Edge / Result types, so that a pair style written
 * against the reference's Kernel (pair_sus2_embedded.cpp:250-374) compiles against this header
 * and runs the GPU engine.  Header only; link with libsus2g.so.
 *
 * Differences a caller should know:
 *   - the model is loaded from a .sus2 path (the reference takes a parsed Model);
 *   - pack_forward / unpack_forward / pack_reverse / add_reverse take one atom, as the reference's
 *     do, and each such call is one synchronous transfer; the batched overloads (a list of atoms,
 *     or a run of consecutive rows) move a whole halo in one call and are the ones to use in a
 *     production pair style;
 *   - errors are thrown as std::runtime_error carrying sus2g_last_error() (the reference throws
 *     its own exception type at the same points).
 */
#ifndef SUS2G_KERNEL_HPP
#define SUS2G_KERNEL_HPP

#include <array>
#include <stdexcept>
#include <string>
#include <vector>

#include "sus2g.h"

namespace sus2g {

// Directed edge of an owned centre i to atom j (owned or ghost), d = x_j - x_i (sus2_sl_kernel.h:12).
struct Edge {
  int i, j;
  std::array<double, 3> d;
};

// Result of finish(): total energy of the owned atoms, their site energies, forces on every atom
// (ghost contributions included, for the caller's reverse force communication) and the virial
// (xx, yy, zz, xy, xz, yz) (sus2_sl_kernel.h:13-14).
struct Result {
  double energy = 0;
  std::vector<double> site_energy;
  std::vector<std::array<double, 3>> force;
  std::array<double, 6> virial{{0, 0, 0, 0, 0, 0}};
};

class Kernel {
 public:
  // precision: SUS2G_FP64 (plain) or SUS2G_FP32 (FP32 bulk with FP64 reductions)
  explicit Kernel(const std::string& model_path, int device = 0, int precision = SUS2G_FP64) {
    check(sus2g_model_load(model_path.c_str(), &model_));
    const int rc = sus2g_engine_create(model_, device, precision, &engine_);
    if (rc) {
      sus2g_model_free(model_);
      model_ = nullptr;
      check(rc);
    }
  }
  ~Kernel() {
    if (engine_) sus2g_engine_free(engine_);
    if (model_) sus2g_model_free(model_);
  }
  Kernel(const Kernel&) = delete;
  Kernel& operator=(const Kernel&) = delete;

  // doubles per atom in each halo exchange (the Effect gate signal width; 0 for Static models)
  int communication_width() const {
    int w = 0;
    check(sus2g_engine_comm_width(engine_, &w));
    return w;
  }
  double cutoff() const {
    double c = 0;
    check(sus2g_model_cutoff(model_, &c));
    return c;
  }

  // nowned centres (atoms 0 .. nowned - 1) of nall atoms, types[nall], the owned centres' edges
  void begin(int nowned, int nall, const std::vector<int>& types, const std::vector<Edge>& edges) {
    if (static_cast<int>(types.size()) != nall) throw std::runtime_error("sus2g::Kernel::begin: types.size() != nall");
    nowned_ = nowned;
    nall_ = nall;
    std::vector<int> ei(edges.size()), ej(edges.size());
    std::vector<double> d(3 * edges.size());
    for (size_t k = 0; k < edges.size(); ++k) {
      ei[k] = edges[k].i;
      ej[k] = edges[k].j;
      for (int c = 0; c < 3; ++c) d[3 * k + c] = edges[k].d[c];
    }
    check(sus2g_stage_begin(engine_, nowned, nall, types.data(), static_cast<int>(edges.size()), ei.data(),
                            ej.data(), d.data()));
  }
  // forward exchange of the gate signal: rows of owned atoms out, rows of ghosts in
  void pack_forward(int atom, double* buf) const { pack_forward(1, &atom, buf); }
  void pack_forward(int n, const int* atoms, double* buf) const {
    check(sus2g_stage_pack_forward(engine_, n, atoms, buf));
  }
  void unpack_forward(int atom, const double* buf) { unpack_forward(1, atom, buf); }
  void unpack_forward(int n, int first, const double* buf) { check(sus2g_stage_unpack_forward(engine_, n, first, buf)); }
  void outer() { check(sus2g_stage_outer(engine_)); }
  // reverse exchange of the gate-signal adjoint: rows of ghosts out, added to owned atoms
  void pack_reverse(int atom, double* buf) const { pack_reverse(1, atom, buf); }
  void pack_reverse(int n, int first, double* buf) const { check(sus2g_stage_pack_reverse(engine_, n, first, buf)); }
  void add_reverse(int atom, const double* buf) { add_reverse(1, &atom, buf); }
  void add_reverse(int n, const int* atoms, const double* buf) { check(sus2g_stage_add_reverse(engine_, n, atoms, buf)); }
  // valid until the next begin() or finish()
  const Result& finish() {
    result_.site_energy.assign(nowned_, 0.0);
    result_.force.assign(nall_, {{0, 0, 0}});
    check(sus2g_stage_finish(engine_, &result_.energy, result_.site_energy.data(),
                             reinterpret_cast<double*>(result_.force.data()), result_.virial.data()));
    return result_;
  }

  sus2g_engine engine() const { return engine_; }

 private:
  static void check(int rc) {
    if (rc) throw std::runtime_error(std::string("sus2g: ") + sus2g_last_error());
  }
  sus2g_model model_ = nullptr;
  sus2g_engine engine_ = nullptr;
  int nowned_ = 0, nall_ = 0;
  Result result_;
};

}  // namespace sus2g

#endif /* SUS2G_KERNEL_HPP */
