// Timing driver around the reference's embedded SUS2-SH engine (test infrastructure only).
//
// Usage: ref-time MODEL EDGES REPS
//   EDGES is a little-endian binary file: int32 n, int32 types[n], int64 E, then E records of
//   (int32 i, int32 j, float64 dx, dy, dz) -- directed owned-centre edges with d = x_j - x_i, as
//   the pair style hands them to the engine (interfaces/lammps/ML-SUS2/sus2_sl_kernel.h:12-13).
//   Runs SUS2SL::Kernel begin / outer / finish (sus2_sl_kernel.cpp:381-562) REPS times on one
//   thread and prints one JSON line: seconds per evaluation (mean and best), the energy and the
//   force checksum sum_i |F_i|_1, so that a caller can check it evaluated the same system.
#include "sus2_sl_kernel.h"

#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <fstream>
#include <stdexcept>
#include <vector>

using namespace LAMMPS_NS::SUS2SL;

int main(int argc, char** argv) {
  if (argc != 4) {
    std::fprintf(stderr, "usage: ref-time MODEL EDGES REPS\n");
    return 2;
  }
  try {
    Model model;
    model.load(argv[1]);
    std::ifstream in(argv[2], std::ios::binary);
    if (!in) throw std::runtime_error("cannot open edge file");
    int32_t n = 0;
    in.read(reinterpret_cast<char*>(&n), 4);
    std::vector<int32_t> t32(n);
    in.read(reinterpret_cast<char*>(t32.data()), 4 * static_cast<std::streamsize>(n));
    int64_t ne = 0;
    in.read(reinterpret_cast<char*>(&ne), 8);
    std::vector<Edge> edges(static_cast<size_t>(ne));
    for (int64_t e = 0; e < ne; ++e) {
      int32_t ij[2];
      double d[3];
      in.read(reinterpret_cast<char*>(ij), 8);
      in.read(reinterpret_cast<char*>(d), 24);
      edges[e] = Edge{ij[0], ij[1], {{d[0], d[1], d[2]}}};
    }
    if (!in) throw std::runtime_error("truncated edge file");
    std::vector<int> types(t32.begin(), t32.end());
    const int reps = std::max(1, std::atoi(argv[3]));
    Kernel kernel(model);
    double total = 0, best = 1e300, energy = 0, fsum = 0;
    for (int r = 0; r < reps; ++r) {
      const auto t0 = std::chrono::steady_clock::now();
      kernel.begin(n, n, types, edges);
      kernel.outer();
      const Result& res = kernel.finish();
      const double dt = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
      total += dt;
      best = std::min(best, dt);
      energy = res.energy;
      fsum = 0;
      for (const auto& f : res.force) fsum += std::fabs(f[0]) + std::fabs(f[1]) + std::fabs(f[2]);
    }
    std::printf("{\"atoms\": %d, \"edges\": %lld, \"reps\": %d, \"seconds_mean\": %.9g, \"seconds_best\": %.9g, "
                "\"energy\": %.17g, \"force_abs_sum\": %.17g}\n",
                n, static_cast<long long>(ne), reps, total / reps, best, energy, fsum);
  } catch (const std::exception& e) {
    std::fprintf(stderr, "%s\n", e.what());
    return 1;
  }
  return 0;
}
