// C++ client of include/sus2g_kernel.hpp (the reference Kernel's surface over the C ABI), linked
// against libsus2g.so by tests/test_gpu_cpp_kernel.py.
//
// Usage: kernel_domains MODEL FRAME DOMAINS PRECISION
//   FRAME: little-endian binary, int32 n, float64 cell[9] (rows are lattice vectors),
//          float64 positions[3 n], int32 types[n].
// Builds the frame's directed edge list (every periodic image within the cutoff, d = x_j + image
// - x_i), splits the atoms over DOMAINS round robin as the reference's standalone harness does
// (interfaces/lammps/tests/embedded_efs.cpp:67-127: each domain owns atoms i % DOMAINS == p and
// sees every other atom as a ghost, the image folded into d), runs begin / forward exchange /
// outer / reverse exchange / finish per domain through sus2g::Kernel (per-atom exchange calls, as
// the reference's pack/unpack are called), sums the domains' results and compares them with the
// periodic evaluation of the whole frame through sus2g_calc_efs_host.  Prints one line
//   RESULT energy_rel force_rel virial_rel
// with errors relative to (1 + max |value|) and exits 0.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <memory>
#include <stdexcept>
#include <vector>

#include "sus2g_kernel.hpp"

namespace {

double rel(double a, double b) { return std::fabs(a - b) / (1.0 + std::max(std::fabs(a), std::fabs(b))); }

std::vector<sus2g::Edge> periodic_edges(int n, const double* cell, const std::vector<double>& x, double rc) {
  // reach per lattice direction from the inverse cell's column norms
  double inv[3][3], det = 0;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j)
      inv[j][i] = cell[3 * ((i + 1) % 3) + (j + 1) % 3] * cell[3 * ((i + 2) % 3) + (j + 2) % 3] -
                  cell[3 * ((i + 1) % 3) + (j + 2) % 3] * cell[3 * ((i + 2) % 3) + (j + 1) % 3];
  for (int i = 0; i < 3; ++i) det += cell[i] * inv[i][0];
  int reach[3];
  for (int q = 0; q < 3; ++q) {
    double s = 0;
    for (int a = 0; a < 3; ++a) s += (inv[a][q] / det) * (inv[a][q] / det);
    reach[q] = static_cast<int>(std::ceil(rc * std::sqrt(s))) + 1;
  }
  std::vector<sus2g::Edge> out;
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j)
      for (int a = -reach[0]; a <= reach[0]; ++a)
        for (int b = -reach[1]; b <= reach[1]; ++b)
          for (int c = -reach[2]; c <= reach[2]; ++c) {
            if (i == j && a == 0 && b == 0 && c == 0) continue;
            std::array<double, 3> d;
            double r2 = 0;
            for (int q = 0; q < 3; ++q) {
              d[q] = x[3 * j + q] - x[3 * i + q] + a * cell[q] + b * cell[3 + q] + c * cell[6 + q];
              r2 += d[q] * d[q];
            }
            if (r2 < rc * rc) out.push_back({i, j, d});
          }
  return out;
}

}  // namespace

int main(int argc, char** argv) {
  if (argc != 5) {
    std::fprintf(stderr, "usage: kernel_domains MODEL FRAME DOMAINS PRECISION\n");
    return 2;
  }
  try {
    std::ifstream in(argv[2], std::ios::binary);
    int32_t n = 0;
    in.read(reinterpret_cast<char*>(&n), 4);
    double cell[9];
    in.read(reinterpret_cast<char*>(cell), sizeof(cell));
    std::vector<double> x(3 * static_cast<size_t>(n));
    in.read(reinterpret_cast<char*>(x.data()), 8 * static_cast<std::streamsize>(x.size()));
    std::vector<int32_t> t32(n);
    in.read(reinterpret_cast<char*>(t32.data()), 4 * static_cast<std::streamsize>(n));
    if (!in) throw std::runtime_error("truncated frame file");
    const std::vector<int> type(t32.begin(), t32.end());
    const int domains = std::atoi(argv[3]);
    const int precision = std::atoi(argv[4]);

    // the periodic reference through the frame entry point
    sus2g::Kernel whole(argv[1], 0, precision);
    double e_ref = 0, v_ref[6];
    std::vector<double> f_ref(3 * static_cast<size_t>(n)), s_ref(n);
    if (sus2g_calc_efs_host(whole.engine(), 1, &n, cell, x.data(), type.data(), &e_ref, f_ref.data(), v_ref,
                            s_ref.data()))
      throw std::runtime_error(sus2g_last_error());

    const auto edges = periodic_edges(n, cell, x, whole.cutoff());
    std::vector<std::vector<int>> map(domains);  // local -> global atom per domain
    std::vector<int> owner(n), owner_local(n), owned(domains, 0);
    std::vector<std::vector<int>> local(domains, std::vector<int>(n));
    std::vector<std::unique_ptr<sus2g::Kernel>> kernels;
    for (int p = 0; p < domains; ++p) {
      for (int i = 0; i < n; ++i)
        if (i % domains == p) { owner[i] = p; owner_local[i] = static_cast<int>(map[p].size()); map[p].push_back(i); }
      owned[p] = static_cast<int>(map[p].size());
      for (int i = 0; i < n; ++i)
        if (i % domains != p) map[p].push_back(i);
      std::vector<int> types(n);
      for (int k = 0; k < n; ++k) { local[p][map[p][k]] = k; types[k] = type[map[p][k]]; }
      std::vector<sus2g::Edge> pe;
      for (auto e : edges)
        if (e.i % domains == p) { e.i = local[p][e.i]; e.j = local[p][e.j]; pe.push_back(e); }
      kernels.emplace_back(new sus2g::Kernel(argv[1], 0, precision));
      kernels.back()->begin(owned[p], n, types, pe);
    }
    const int width = kernels[0]->communication_width();
    std::vector<double> buf(std::max(width, 1));
    for (int p = 0; p < domains; ++p)
      for (int k = owned[p]; k < n; ++k) {
        const int g = map[p][k];
        kernels[owner[g]]->pack_forward(owner_local[g], buf.data());
        kernels[p]->unpack_forward(k, buf.data());
      }
    for (auto& k : kernels) k->outer();
    for (int p = 0; p < domains; ++p)
      for (int k = owned[p]; k < n; ++k) {
        const int g = map[p][k];
        kernels[p]->pack_reverse(k, buf.data());
        kernels[owner[g]]->add_reverse(owner_local[g], buf.data());
      }
    double energy = 0, virial[6] = {0, 0, 0, 0, 0, 0};
    std::vector<double> force(3 * static_cast<size_t>(n), 0.0);
    for (int p = 0; p < domains; ++p) {
      const sus2g::Result& r = kernels[p]->finish();
      energy += r.energy;
      for (int k = 0; k < n; ++k)
        for (int c = 0; c < 3; ++c) force[3 * map[p][k] + c] += r.force[k][c];
      for (int c = 0; c < 6; ++c) virial[c] += r.virial[c];
    }
    double fe = 0, ve = 0;
    for (size_t q = 0; q < force.size(); ++q) fe = std::max(fe, rel(force[q], f_ref[q]));
    for (int c = 0; c < 6; ++c) ve = std::max(ve, rel(virial[c], v_ref[c]));
    std::printf("RESULT %.3e %.3e %.3e\n", rel(energy, e_ref), fe, ve);
  } catch (const std::exception& e) {
    std::fprintf(stderr, "%s\n", e.what());
    return 1;
  }
  return 0;
}
