// extern "C" boundary (include/sus2g.h): argument checks, host<->device staging, error codes.
#include "../../include/sus2g.h"

#include <cuda_runtime.h>

#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "capi_types.h"

namespace {
thread_local std::string g_error;

template <typename F>
int guarded(F&& f) {
  try {
    f();
    g_error.clear();
    return 0;
  } catch (const sus2g::Error& e) {
    g_error = e.what();
    return e.code > 0 ? e.code : 1;
  } catch (const std::bad_alloc&) {
    g_error = "out of host memory";
    return 9;
  } catch (const std::exception& e) {
    g_error = e.what();
    return 1;
  }
}

void need(bool ok, const char* what) {
  if (!ok) throw sus2g::Error(1, std::string("invalid argument: ") + what);
}

void cuda(cudaError_t e, const char* where) {
  if (e != cudaSuccess) throw sus2g::Error(10, std::string("CUDA error in ") + where + ": " + cudaGetErrorString(e));
}

// Engine-owned, grow-only device staging buffer for host arrays.
struct Slot {
  void* p;
  Slot(sus2g::Engine& e, int slot, size_t n) : p(e.io(slot, n)) {}
  template <typename T> T* as() { return static_cast<T*>(p); }
};

long long total_atoms(int nframes, const int* natoms) {
  long long n = 0;
  for (int f = 0; f < nframes; ++f) {
    need(natoms[f] >= 0, "natoms must be non-negative");
    n += natoms[f];
  }
  need(n < (1LL << 31), "too many atoms");
  return n;
}
}  // namespace

void sus2g_set_last_error(const char* message) { g_error = message ? message : ""; }

extern "C" {

const char* sus2g_last_error(void) { return g_error.c_str(); }
int sus2g_abi_version(void) { return 100; }

int sus2g_model_load(const char* path, sus2g_model* out) {
  return guarded([&] {
    need(path && out, "path/out");
    auto m = std::make_unique<sus2g_model_s>();
    m->model.load(path);
    *out = m.release();
  });
}

void sus2g_model_free(sus2g_model model) { delete model; }

int sus2g_model_dims(sus2g_model h, int* d) {
  return guarded([&] {
    need(h && d, "model/dims");
    const auto& m = h->model;
    const int v[16] = {m.C, m.L, m.K, m.B, m.F, m.M, m.NB, m.P, m.S, m.Q, m.gated ? 1 : 0, m.param_count(),
                       m.outer_rank, m.gate_rank, m.split ? 1 : 0, 0};
    std::memcpy(d, v, sizeof(v));
  });
}

int sus2g_model_cutoff(sus2g_model h, double* c) {
  return guarded([&] { need(h && c, "model/cutoff"); *c = h->model.max_dist; });
}

int sus2g_model_param_count(sus2g_model h, int* n) {
  return guarded([&] { need(h && n, "model/count"); *n = h->model.param_count(); });
}

int sus2g_model_get_params(sus2g_model h, double* out, int n) {
  return guarded([&] {
    need(h && out, "model/out");
    need(n == h->model.param_count(), "parameter count mismatch");
    h->model.get_params(out);
  });
}

int sus2g_model_set_params(sus2g_model h, const double* in, int n) {
  return guarded([&] {
    need(h && in, "model/in");
    need(n == h->model.param_count(), "parameter count mismatch");
    h->model.set_params(in);
  });
}

int sus2g_model_save(sus2g_model h, const char* path) {
  return guarded([&] {
    need(h && path, "model/path");
    h->model.save(path);
  });
}

int sus2g_engine_create(sus2g_model model, int device, int precision, sus2g_engine* out) {
  return guarded([&] {
    need(model && out, "model/out");
    auto e = std::make_unique<sus2g_engine_s>();
    e->engine = std::make_unique<sus2g::Engine>(model->model, device, precision);
    *out = e.release();
  });
}

void sus2g_engine_free(sus2g_engine e) { delete e; }

int sus2g_model_get_scaling(sus2g_model m, double* scaling) {
  return guarded([&] { need(m && scaling, "model/scaling"); *scaling = m->model.scaling; });
}

int sus2g_model_set_scaling(sus2g_model m, double scaling) {
  return guarded([&] { need(m, "model"); m->model.set_scaling(scaling); });
}

int sus2g_engine_update_params(sus2g_engine e, sus2g_model model) {
  return guarded([&] {
    need(e && model, "engine/model");
    need(model->model.param_count() == e->engine->model().param_count(), "model layout differs from the engine's");
    auto fresh = std::make_unique<sus2g::Engine>(model->model, e->engine->device(), e->engine->precision());
    e->engine = std::move(fresh);
  });
}

int sus2g_engine_set_stream(sus2g_engine e, void* stream) {
  return guarded([&] { need(e, "engine"); e->engine->set_stream(static_cast<cudaStream_t>(stream)); });
}

int sus2g_engine_take_launch_count(sus2g_engine e, int* count) {
  return guarded([&] {
    need(e && count, "engine/count");
    *count = e->engine->last_launches();
    e->engine->reset_launch_count();
  });
}

int sus2g_engine_edge_count(sus2g_engine e, long long* count) {
  return guarded([&] { need(e && count, "engine/count"); *count = e->engine->nedges(); });
}

int sus2g_engine_copy_edges(sus2g_engine e, long long cap, int* centre, int* neighbour, double* d,
                            long long* count) {
  return guarded([&] {
    need(e && count && cap >= 0, "engine/count/capacity");
    e->engine->copy_edges(cap, centre, neighbour, d, count);
  });
}

int sus2g_engine_pass_shape(sus2g_engine e, int mode, int* shape4) {
  return guarded([&] {
    need(e && shape4 && mode >= 0 && mode < 4, "engine/mode/shape");
    e->engine->pass_shape(mode, shape4);
  });
}

int sus2g_engine_set_pass_shape(sus2g_engine e, int mode, int blocks, int grid, int order, int stage, int warps) {
  return guarded([&] {
    need(e, "engine");
    e->engine->set_pass_shape(mode, blocks, grid, order, stage, warps);
  });
}

int sus2g_engine_set_grad_split(sus2g_engine e, int enabled) {
  return guarded([&] { need(e, "engine"); e->engine->set_grad_split(enabled != 0); });
}

int sus2g_engine_set_static_split(sus2g_engine e, int enabled) {
  return guarded([&] { need(e, "engine"); e->engine->set_static_split(enabled != 0); });
}

int sus2g_engine_set_moment_mma(sus2g_engine e, int enabled) {
  return guarded([&] { need(e, "engine"); e->engine->set_moment_mma(enabled != 0); });
}

int sus2g_engine_set_timing(sus2g_engine e, int enabled) {
  return guarded([&] { need(e, "engine"); e->engine->set_timing(enabled != 0); });
}

int sus2g_engine_autotune(sus2g_engine e, int reps, int* blocks4, double* ms8) {
  return guarded([&] {
    need(e && reps > 0, "engine/reps");
    int b[4];
    double ms[8];
    e->engine->autotune(reps, b, ms);
    if (blocks4) std::memcpy(blocks4, b, sizeof(b));
    if (ms8) std::memcpy(ms8, ms, sizeof(ms));
  });
}

int sus2g_engine_set_step_graph(sus2g_engine e, int enabled) {
  return guarded([&] { need(e, "engine"); e->engine->set_step_graphs(enabled != 0); });
}

int sus2g_engine_set_pdl(sus2g_engine e, int sites) {
  return guarded([&] {
    need(e && sites >= -1 && sites <= 15, "engine/sites");
    e->engine->set_pdl(sites);
  });
}

int sus2g_engine_take_stage_times(sus2g_engine e, double* ms, int* counts) {
  return guarded([&] { need(e, "engine"); e->engine->take_stage_times(ms, counts); });
}

int sus2g_calc_efs_device(sus2g_engine e, int nframes, const int* natoms, const double* cells,
                          const double* positions, const int* types, double* energy, double* forces,
                          double* virial, double* site_energy) {
  return guarded([&] {
    need(e && nframes >= 0 && (nframes == 0 || (natoms && cells)), "engine/frames");
    const long long n = total_atoms(nframes, natoms);
    need(n == 0 || (positions && types), "positions/types");
    auto& eng = *e->engine;
    for (int attempt = 0;; ++attempt) {
      try {
        eng.step_frames(nframes, natoms, cells, positions, types, energy, forces, virial, site_energy);
        eng.check_device_error();
        break;
      } catch (const sus2g::EdgeOverflow&) {
        if (attempt >= 4) throw;  // the capacity has been grown: repeat the step
      }
    }
  });
}

int sus2g_calc_efs_host(sus2g_engine e, int nframes, const int* natoms, const double* cells,
                        const double* positions, const int* types, double* energy, double* forces,
                        double* virial, double* site_energy) {
  return guarded([&] {
    need(e && nframes >= 0 && (nframes == 0 || (natoms && cells)), "engine/frames");
    const long long n = total_atoms(nframes, natoms);
    need(n == 0 || (positions && types), "positions/types");
    auto& eng = *e->engine;
    for (long long i = 0; i < n; ++i)
      need(types[i] >= 0 && types[i] < eng.model().C, "atom species index out of range");
    cudaStream_t s = eng.stream();
    cuda(cudaSetDevice(eng.device()), "cudaSetDevice");
    // one pinned staging area and one transfer each way: inputs [positions 3n][types n], outputs
    // [energy nf][forces 3n][virial 6 nf][site n] (doubles; types as int after the positions)
    const size_t in_bytes = sizeof(double) * 3 * n + sizeof(int) * n;
    const size_t out_doubles = static_cast<size_t>(nframes) * 7 + 4 * static_cast<size_t>(n);
    char* stage = static_cast<char*>(eng.pinned(std::max(in_bytes, sizeof(double) * out_doubles)));
    Slot in(eng, 0, in_bytes), out(eng, 2, sizeof(double) * out_doubles);
    double* d_pos = in.as<double>();
    int* d_typ = reinterpret_cast<int*>(in.as<char>() + sizeof(double) * 3 * n);
    double* d_e = out.as<double>();
    double* d_f = d_e + nframes;
    double* d_v = d_f + 3 * n;
    double* d_s = d_v + 6 * static_cast<size_t>(nframes);
    if (n) {
      std::memcpy(stage, positions, sizeof(double) * 3 * n);
      std::memcpy(stage + sizeof(double) * 3 * n, types, sizeof(int) * n);
      cuda(cudaMemcpyAsync(in.p, stage, in_bytes, cudaMemcpyHostToDevice, s), "input copy");
    }
    for (int attempt = 0;; ++attempt) {
      eng.step_frames(nframes, natoms, cells, d_pos, d_typ, energy ? d_e : nullptr, forces ? d_f : nullptr,
                      virial ? d_v : nullptr, site_energy ? d_s : nullptr);
      // the outputs and the error words come back together; one synchronisation
      if (out_doubles)
        cuda(cudaMemcpyAsync(stage, out.p, sizeof(double) * out_doubles, cudaMemcpyDeviceToHost, s), "output copy");
      eng.enqueue_error_read();
      cuda(cudaStreamSynchronize(s), "stream synchronize");
      try {
        eng.check_error_read();
        break;
      } catch (const sus2g::EdgeOverflow&) {
        if (attempt >= 4) throw;  // the capacity has been grown: repeat the step
      }
    }
    const double* h = reinterpret_cast<const double*>(stage);
    if (energy && nframes) std::memcpy(energy, h, sizeof(double) * nframes);
    if (forces && n) std::memcpy(forces, h + nframes, sizeof(double) * 3 * n);
    if (virial && nframes) std::memcpy(virial, h + nframes + 3 * n, sizeof(double) * 6 * nframes);
    if (site_energy && n) std::memcpy(site_energy, h + 7 * static_cast<size_t>(nframes) + 3 * n, sizeof(double) * n);
  });
}

int sus2g_calc_descriptors_host(sus2g_engine e, int nframes, const int* natoms, const double* cells,
                                const double* positions, const int* types, double* desc) {
  return guarded([&] {
    need(e && nframes >= 0 && (nframes == 0 || (natoms && cells)), "engine/frames");
    const long long n = total_atoms(nframes, natoms);
    need(n == 0 || (positions && types && desc), "positions/types/desc");
    auto& eng = *e->engine;
    for (long long i = 0; i < n; ++i)
      need(types[i] >= 0 && types[i] < eng.model().C, "atom species index out of range");
    const int S = eng.model().S;
    cudaStream_t s = eng.stream();
    cuda(cudaSetDevice(eng.device()), "cudaSetDevice");
    Slot pos(eng, 0, sizeof(double) * 3 * n), typ(eng, 1, sizeof(int) * n), out(eng, 2, sizeof(double) * n * S);
    if (n) {
      cuda(cudaMemcpyAsync(pos.p, positions, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, s), "positions copy");
      cuda(cudaMemcpyAsync(typ.p, types, sizeof(int) * n, cudaMemcpyHostToDevice, s), "types copy");
    }
    struct Reset {  // the descriptor output is for this call only
      sus2g::Engine& e;
      ~Reset() { e.set_descriptor_output(nullptr); }
    } reset{eng};
    for (int attempt = 0;; ++attempt) {
      try {
        eng.build_edges(nframes, natoms, cells, pos.as<double>(), typ.as<int>());
        eng.set_descriptor_output(out.as<double>());
        eng.efs(nullptr, nullptr, nullptr, nullptr);
        eng.check_device_error();
        break;
      } catch (const sus2g::EdgeOverflow&) {
        if (attempt >= 4) throw;  // the capacity has been grown: repeat the step
      }
    }
    if (n && S) cuda(cudaMemcpyAsync(desc, out.p, sizeof(double) * n * S, cudaMemcpyDeviceToHost, s), "descriptor copy");
    cuda(cudaStreamSynchronize(s), "stream synchronize");
  });
}

int sus2g_efs_combination_grad_host(sus2g_engine e, int nframes, const int* natoms, const double* cells,
                                    const double* positions, const int* types, const double* ene_w,
                                    const double* frc_w, const double* str_w, double* grad) {
  return guarded([&] {
    need(e && nframes >= 0 && (nframes == 0 || (natoms && cells)), "engine/frames");
    const long long n = total_atoms(nframes, natoms);
    need(n == 0 || (positions && types && ene_w && frc_w), "positions/types/weights");
    need(grad && (nframes == 0 || str_w), "grad/stress weights");
    auto& eng = *e->engine;
    for (long long i = 0; i < n; ++i)
      need(types[i] >= 0 && types[i] < eng.model().C, "atom species index out of range");
    const int P = eng.model().param_count();
    cudaStream_t s = eng.stream();
    cuda(cudaSetDevice(eng.device()), "cudaSetDevice");
    Slot pos(eng, 0, sizeof(double) * 3 * n), typ(eng, 1, sizeof(int) * n), ew(eng, 2, sizeof(double) * n),
        fw(eng, 3, sizeof(double) * 3 * n), sw(eng, 4, sizeof(double) * 9 * nframes), g(eng, 5, sizeof(double) * P);
    if (n) {
      cuda(cudaMemcpyAsync(pos.p, positions, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, s), "positions copy");
      cuda(cudaMemcpyAsync(typ.p, types, sizeof(int) * n, cudaMemcpyHostToDevice, s), "types copy");
      cuda(cudaMemcpyAsync(ew.p, ene_w, sizeof(double) * n, cudaMemcpyHostToDevice, s), "weights copy");
      cuda(cudaMemcpyAsync(fw.p, frc_w, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, s), "weights copy");
    }
    if (nframes) cuda(cudaMemcpyAsync(sw.p, str_w, sizeof(double) * 9 * nframes, cudaMemcpyHostToDevice, s), "weights copy");
    for (int attempt = 0;; ++attempt) {
      try {
        cuda(cudaMemcpyAsync(g.p, grad, sizeof(double) * P, cudaMemcpyHostToDevice, s), "grad copy");
        eng.build_edges(nframes, natoms, cells, pos.as<double>(), typ.as<int>());
        if (n) eng.combination_grad(ew.as<double>(), fw.as<double>(), sw.as<double>(), g.as<double>());
        eng.check_device_error();
        break;
      } catch (const sus2g::EdgeOverflow&) {
        if (attempt >= 4) throw;  // the capacity has been grown: repeat the step
      }
    }
    cuda(cudaMemcpyAsync(grad, g.p, sizeof(double) * P, cudaMemcpyDeviceToHost, s), "grad copy");
    cuda(cudaStreamSynchronize(s), "stream synchronize");
  });
}

int sus2g_efs_combination_grad_device(sus2g_engine e, int nframes, const int* natoms, const double* cells,
                                      const double* positions, const int* types, const double* ene_w,
                                      const double* frc_w, const double* str_w, double* grad) {
  return guarded([&] {
    need(e && nframes >= 0 && (nframes == 0 || (natoms && cells)), "engine/frames");
    const long long n = total_atoms(nframes, natoms);
    need(n == 0 || (positions && types && ene_w && frc_w), "positions/types/weights");
    need(grad && (nframes == 0 || str_w), "grad/stress weights");
    auto& eng = *e->engine;
    const int P = eng.model().param_count();
    cudaStream_t s = eng.stream();
    cuda(cudaSetDevice(eng.device()), "cudaSetDevice");
    // the caller's gradient, put back before an attempt repeated after an edge-capacity overflow
    Slot g0(eng, 5, sizeof(double) * P);
    cuda(cudaMemcpyAsync(g0.p, grad, sizeof(double) * P, cudaMemcpyDeviceToDevice, s), "grad copy");
    for (int attempt = 0;; ++attempt) {
      try {
        if (attempt) cuda(cudaMemcpyAsync(grad, g0.p, sizeof(double) * P, cudaMemcpyDeviceToDevice, s), "grad copy");
        eng.build_edges(nframes, natoms, cells, positions, types);
        if (n) eng.combination_grad(ene_w, frc_w, str_w, grad);
        eng.check_device_error();
        break;
      } catch (const sus2g::EdgeOverflow&) {
        if (attempt >= 4) throw;  // the capacity has been grown: repeat the evaluation
      }
    }
  });
}

// Staged evaluation: device staging slots -- 0 types (held from begin to finish), 1..3 edge input
// at begin and outputs at finish, 4 atom indices and 5 row buffers of the exchanges.
namespace {
void check_edges(sus2g::Engine& eng, int nowned, int nall, const int* types, int nedges, const int* ei, const int* ej,
                 const double* d) {
  need(nowned >= 0 && nall >= nowned && nedges >= 0, "engine/layout");
  need(nall == 0 || types, "types");
  need(nedges == 0 || (ei && ej && d), "edges");
  for (int i = 0; i < nall; ++i) need(types[i] >= 0 && types[i] < eng.model().C, "atom species index out of range");
  for (long long q = 0; q < nedges; ++q) {
    need(ei[q] >= 0 && ei[q] < nowned && ej[q] >= 0 && ej[q] < nall, "edge atom index out of range");
    const double r2 = d[3 * q] * d[3 * q] + d[3 * q + 1] * d[3 * q + 1] + d[3 * q + 2] * d[3 * q + 2];
    need(r2 > 0 && r2 < 1e300, "edge with zero or non-finite length");
  }
}

void stage_rows_host(sus2g_engine e, int which, int op, int n, const int* atoms, int first, double* buf) {
  need(e && n >= 0 && (n == 0 || buf), "engine/rows");
  auto& eng = *e->engine;
  const int W = eng.comm_width();
  if (n == 0 || W == 0) return;
  if (atoms)
    for (int k = 0; k < n; ++k) need(atoms[k] >= 0 && atoms[k] < eng.natoms(), "exchange atom index out of range");
  // add_reverse may name one owner several times (its periodic images are distinct ghosts): rows of
  // the same atom are summed here in call order, so each atom is updated once on the device
  std::vector<int> uniq;
  std::vector<double> summed;
  if (which == 1 && op == 1 && atoms) {
    std::vector<int> slot_of(eng.natoms(), -1);
    for (int k = 0; k < n; ++k) {
      int& q = slot_of[atoms[k]];
      if (q < 0) {
        q = static_cast<int>(uniq.size());
        uniq.push_back(atoms[k]);
        summed.insert(summed.end(), buf + static_cast<size_t>(k) * W, buf + static_cast<size_t>(k + 1) * W);
      } else {
        for (int w = 0; w < W; ++w) summed[static_cast<size_t>(q) * W + w] += buf[static_cast<size_t>(k) * W + w];
      }
    }
    n = static_cast<int>(uniq.size());
    atoms = uniq.data();
    buf = summed.data();
  }
  cudaStream_t s = eng.stream();
  cuda(cudaSetDevice(eng.device()), "cudaSetDevice");
  Slot idx(eng, 4, sizeof(int) * n), rows(eng, 5, sizeof(double) * static_cast<size_t>(n) * W);
  if (atoms) cuda(cudaMemcpyAsync(idx.p, atoms, sizeof(int) * n, cudaMemcpyHostToDevice, s), "index copy");
  if (op == 1) cuda(cudaMemcpyAsync(rows.p, buf, sizeof(double) * n * W, cudaMemcpyHostToDevice, s), "row copy");
  eng.stage_rows(which, op, n, atoms ? idx.as<int>() : nullptr, first, rows.as<double>());
  if (op == 0) cuda(cudaMemcpyAsync(buf, rows.p, sizeof(double) * n * W, cudaMemcpyDeviceToHost, s), "row copy");
  eng.check_device_error();
}
}  // namespace

int sus2g_engine_comm_width(sus2g_engine e, int* width) {
  return guarded([&] { need(e && width, "engine/width"); *width = e->engine->comm_width(); });
}

int sus2g_stage_begin(sus2g_engine e, int nowned, int nall, const int* types, int nedges, const int* ei,
                      const int* ej, const double* d) {
  return guarded([&] {
    need(e, "engine");
    auto& eng = *e->engine;
    check_edges(eng, nowned, nall, types, nedges, ei, ej, d);
    cudaStream_t s = eng.stream();
    cuda(cudaSetDevice(eng.device()), "cudaSetDevice");
    Slot typ(eng, 0, sizeof(int) * nall), di(eng, 1, sizeof(int) * nedges), dj(eng, 2, sizeof(int) * nedges),
        dd(eng, 3, sizeof(double) * 3 * nedges);
    if (nall) cuda(cudaMemcpyAsync(typ.p, types, sizeof(int) * nall, cudaMemcpyHostToDevice, s), "types copy");
    if (nedges) {
      cuda(cudaMemcpyAsync(di.p, ei, sizeof(int) * nedges, cudaMemcpyHostToDevice, s), "edge copy");
      cuda(cudaMemcpyAsync(dj.p, ej, sizeof(int) * nedges, cudaMemcpyHostToDevice, s), "edge copy");
      cuda(cudaMemcpyAsync(dd.p, d, sizeof(double) * 3 * nedges, cudaMemcpyHostToDevice, s), "edge copy");
    }
    eng.stage_begin(nowned, nall, typ.as<int>(), nedges, di.as<int>(), dj.as<int>(), dd.as<double>());
    eng.check_device_error();
  });
}

int sus2g_stage_pack_forward(sus2g_engine e, int n, const int* atoms, double* buf) {
  return guarded([&] { need(n == 0 || atoms, "atoms"); stage_rows_host(e, 0, 0, n, atoms, 0, buf); });
}

int sus2g_stage_unpack_forward(sus2g_engine e, int n, int first, const double* buf) {
  return guarded([&] { stage_rows_host(e, 0, 1, n, nullptr, first, const_cast<double*>(buf)); });
}

int sus2g_stage_outer(sus2g_engine e) {
  return guarded([&] {
    need(e, "engine");
    e->engine->stage_outer();
    e->engine->check_device_error();
  });
}

int sus2g_stage_pack_reverse(sus2g_engine e, int n, int first, double* buf) {
  return guarded([&] { stage_rows_host(e, 1, 0, n, nullptr, first, buf); });
}

int sus2g_stage_add_reverse(sus2g_engine e, int n, const int* atoms, const double* buf) {
  return guarded([&] { need(n == 0 || atoms, "atoms"); stage_rows_host(e, 1, 1, n, atoms, 0, const_cast<double*>(buf)); });
}

int sus2g_stage_finish(sus2g_engine e, double* energy, double* site_energy, double* forces, double* virial) {
  return guarded([&] {
    need(e, "engine");
    auto& eng = *e->engine;
    const int nall = eng.natoms(), nowned = eng.ncentres();
    cudaStream_t s = eng.stream();
    cuda(cudaSetDevice(eng.device()), "cudaSetDevice");
    Slot ev(eng, 1, sizeof(double) * 7), out_f(eng, 2, sizeof(double) * 3 * std::max(1, nall)),
        out_s(eng, 3, sizeof(double) * std::max(1, nowned));
    eng.stage_finish(ev.as<double>(), forces ? out_f.as<double>() : nullptr, ev.as<double>() + 1,
                     site_energy ? out_s.as<double>() : nullptr);
    eng.check_device_error();
    double h[7];
    cuda(cudaMemcpyAsync(h, ev.p, sizeof(h), cudaMemcpyDeviceToHost, s), "energy copy");
    if (forces && nall) cuda(cudaMemcpyAsync(forces, out_f.p, sizeof(double) * 3 * nall, cudaMemcpyDeviceToHost, s), "force copy");
    if (site_energy && nowned) cuda(cudaMemcpyAsync(site_energy, out_s.p, sizeof(double) * nowned, cudaMemcpyDeviceToHost, s), "site copy");
    cuda(cudaStreamSynchronize(s), "stream synchronize");
    if (energy) *energy = h[0];
    if (virial) std::memcpy(virial, h + 1, sizeof(double) * 6);
  });
}

int sus2g_efs_edges_host(sus2g_engine e, int nowned, int nall, const int* types, int nedges, const int* ei,
                         const int* ej, const double* d, double* energy, double* site_energy, double* forces,
                         double* virial) {
  return guarded([&] {
    need(e && nowned >= 0 && nall >= nowned && nedges >= 0, "engine/layout");
    need(nall == 0 || types, "types");
    need(nedges == 0 || (ei && ej && d), "edges");
    auto& eng = *e->engine;
    for (int i = 0; i < nall; ++i) need(types[i] >= 0 && types[i] < eng.model().C, "atom species index out of range");
    const double rc2 = eng.model().max_dist * eng.model().max_dist;
    for (long long q = 0; q < nedges; ++q) {
      need(ei[q] >= 0 && ei[q] < nowned && ej[q] >= 0 && ej[q] < nall, "edge atom index out of range");
      const double r2 = d[3 * q] * d[3 * q] + d[3 * q + 1] * d[3 * q + 1] + d[3 * q + 2] * d[3 * q + 2];
      need(r2 > 0 && r2 < 1e300, "edge with zero or non-finite length");
      (void)rc2;
    }
    cudaStream_t s = eng.stream();
    cuda(cudaSetDevice(eng.device()), "cudaSetDevice");
    Slot typ(eng, 0, sizeof(int) * nall), di(eng, 1, sizeof(int) * nedges), dj(eng, 2, sizeof(int) * nedges),
        dd(eng, 3, sizeof(double) * 3 * nedges);
    Slot out_e(eng, 4, sizeof(double)), out_f(eng, 5, sizeof(double) * 3 * nall), out_v(eng, 6, sizeof(double) * 6),
        out_s(eng, 7, sizeof(double) * nowned);
    if (nall) cuda(cudaMemcpyAsync(typ.p, types, sizeof(int) * nall, cudaMemcpyHostToDevice, s), "types copy");
    if (nedges) {
      cuda(cudaMemcpyAsync(di.p, ei, sizeof(int) * nedges, cudaMemcpyHostToDevice, s), "edge copy");
      cuda(cudaMemcpyAsync(dj.p, ej, sizeof(int) * nedges, cudaMemcpyHostToDevice, s), "edge copy");
      cuda(cudaMemcpyAsync(dd.p, d, sizeof(double) * 3 * nedges, cudaMemcpyHostToDevice, s), "edge copy");
    }
    eng.set_edges(nowned, nall, typ.as<int>(), nedges, di.as<int>(), dj.as<int>(), dd.as<double>());
    eng.efs(out_e.as<double>(), forces ? out_f.as<double>() : nullptr, out_v.as<double>(),
            site_energy ? out_s.as<double>() : nullptr);
    eng.check_device_error();
    if (energy) cuda(cudaMemcpyAsync(energy, out_e.p, sizeof(double), cudaMemcpyDeviceToHost, s), "energy copy");
    if (forces && nall) cuda(cudaMemcpyAsync(forces, out_f.p, sizeof(double) * 3 * nall, cudaMemcpyDeviceToHost, s), "force copy");
    if (virial) cuda(cudaMemcpyAsync(virial, out_v.p, sizeof(double) * 6, cudaMemcpyDeviceToHost, s), "virial copy");
    if (site_energy && nowned) cuda(cudaMemcpyAsync(site_energy, out_s.p, sizeof(double) * nowned, cudaMemcpyDeviceToHost, s), "site copy");
    cuda(cudaStreamSynchronize(s), "stream synchronize");
  });
}

}  // extern "C"
