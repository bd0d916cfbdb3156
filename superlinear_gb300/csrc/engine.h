// GPU engine for one SUS2-SH model on one device: owns the device tables, the per-step buffers and
// the CUDA stream work of an E / F / virial (and, for training, parameter-gradient) evaluation.
#pragma once
#include <cuda_runtime.h>

#include <memory>
#include <string>
#include <vector>

#include "model.h"

namespace sus2g {

template <typename Real> struct PassArgs;  // efs_kernels.cuh
struct HostProg;                            // engine.cu: a pass's graph program on the host

enum Precision : int { kFP64 = 0, kFP32 = 1 };

// Grow-only device buffer.
struct DevBuf {
  void* ptr = nullptr;
  size_t bytes = 0;
  void ensure(size_t n);
  void release();
  template <typename T> T* as() const { return static_cast<T*>(ptr); }
  ~DevBuf() { release(); }
};

struct FramePlan;

class Engine {
 public:
  Engine(const Model& model, int device, int precision);
  ~Engine();
  Engine(const Engine&) = delete;
  Engine& operator=(const Engine&) = delete;

  const Model& model() const { return model_; }
  int precision() const { return precision_; }
  int device() const { return device_; }
  cudaStream_t stream() const { return stream_; }
  void set_stream(cudaStream_t s) { stream_ = s ? s : own_stream_; }

  // Re-upload parameters after Model::set_params.
  void upload_model();
  // Replace the engine's parameter vector (trainer order) and re-upload the device tables.
  void set_params(const double* params) { model_.set_params(params); upload_model(); }
  void set_scaling(double s) { model_.set_scaling(s); upload_model(); }
  // Incremented by every build_edges / set_edges: a caller that captured work on this engine's
  // buffers (a CUDA graph) must rebuild it when the generation it recorded has changed, since a
  // rebuild may reallocate the edge and step buffers.
  unsigned long long edge_generation() const { return edge_generation_; }

  // --- geometry -----------------------------------------------------------------------------
  // Periodic frames: cells (row lattice vectors, 9 doubles each) live on the host, positions
  // (double [N][3]) and types (int [N]) on the device.  Builds the CSR edge list on stream().
  void build_edges(int nframes, const int* frame_natoms, const double* cells, const double* d_pos,
                   const int* d_types);
  // Caller-supplied directed edges (LAMMPS-style owned centres; device arrays).  nowned centres,
  // nall atoms; edges need not be sorted; rev is computed from (i, j, d) pairing.
  void set_edges(int nowned, int nall, const int* d_types, int nedges, const int* d_i, const int* d_j,
                 const double* d_d);

  // One E/F/virial step of periodic frames with device positions / types / outputs (build_edges +
  // efs).  For cell-list batches the second consecutive step of a layout -- frame sizes, cells,
  // buffer addresses, stream -- is captured as a CUDA graph and later ones replay it (positions
  // may change: the replay reads them); a layout change, any other edge build, a parameter
  // upload, the stage timer or a capacity overflow makes the next step eager again.
  void step_frames(int nframes, const int* frame_natoms, const double* cells, const double* d_pos, const int* d_types,
                   double* d_energy, double* d_forces, double* d_virial, double* d_site);
  void set_step_graphs(bool on) { step_graphs_ = on; if (!on) reset_step_graph(); }
  // programmatic dependent launch between the kernels of an E/F/virial step, per launch site
  // (kPdl* bits; negative = the model's default); a change drops a captured step graph.
  // Measured on GB300 (graph replay): the Static 4,096-atom step 0.151 ms with no site, 0.145 ms
  // with the fill and first-pass sites; the Effect L4 110,592-atom step 14.22 ms with none,
  // 14.26 ms with the fill site, 14.37 ms with the first-pass site, 14.44 ms with the gather site
  // (the gather site also slows the Static step).  Defaults: Static fill + first pass, Effect fill.
  static constexpr int kPdlFill = 1, kPdlFirstPass = 2, kPdlBetweenPasses = 4, kPdlGather = 8;
  int default_pdl() const { return model_.gated ? kPdlFill : kPdlFill | kPdlFirstPass; }
  void set_pdl(int sites) {
    if (sites < 0) sites = default_pdl();
    if (sites != pdl_) reset_step_graph();
    pdl_ = sites;
  }
  // Pass-kernel autotuner on the current layout (see engine.cu): blocks_out[mode] = the chosen
  // register budget (3 or 4 resident blocks per SM; 0 for passes the model does not run),
  // ms_out[2 mode + (budget - 3)] = the timed milliseconds per launch.
  void autotune(int reps, int* blocks_out, double* ms_out);
  // tile shape of pass `mode` (0 Static, 1 gate forward, 2 outer, 3 gate reverse): register budget
  // (resident blocks per SM; 0 = default), grid shape, centre order + 4 x split (Static pass run
  // as three kernels) + 8 x h_j staging by bulk async copies, warps per block
  void pass_shape(int mode, int* shape4) const {
    shape4[0] = pass_blocks_[mode]; shape4[1] = pass_grid_[mode];
    const bool gate_split = model_.gated && (mode == 1 || mode == 3) && gate_split_[mode == 1 ? 0 : 1];
    const bool split = (static_split_ && mode == (model_.gated ? 2 : 0)) || gate_split;
    if (split) shape4[0] = gate_split ? gate_split_blocks_[mode == 1 ? 0 : 1] : split_blocks_;
    shape4[2] = pass_order_[mode] + (split ? 4 : 0) + (pass_stage_[mode] ? 8 : 0);
    shape4[3] = pass_wpb_[mode];
  }
  // sets the tile shape of pass `mode` as the autotuner would (blocks 0 = default, 3 or 4; grid 0
  // or 1; order 0, 1 or 2; stage 1 = h_j rows by bulk async copies, Effect outer pass): for
  // pinning a shape measured elsewhere
  void set_pass_shape(int mode, int blocks, int grid, int order, int stage, int warps);
  void reset_step_graph();
  // Edge->moment batch sums of the FP32 passes on the tensor cores (3xTF32 mma.sync) instead of
  // CUDA-core FMAs; off by default (measured slower on GB300, see the design notes); a change
  // drops a captured step graph.
  // The per-atom passes split at the per-atom boundary instead of fused (FP32 engines, basis size
  // 8): the energy pass -- Static, or the Effect outer pass -- as three kernels (edge->moment
  // forward, per-atom graph, per-edge adjoint), the Effect gate passes as two each; the
  // autotuner chooses per pass; a change drops a captured step graph.
  void set_static_split(bool on) {
    if (on != static_split_ || on != gate_split_[0] || on != gate_split_[1]) reset_step_graph();
    static_split_ = gate_split_[0] = gate_split_[1] = on;
  }
  bool static_split() const { return static_split_; }
  // The outer and gate reverse parameter-gradient passes as two kernels each (per-atom part,
  // per-edge part; basis size 8) instead of one; a change drops a captured step graph and makes
  // graphs captured by other owners (a trainer) be captured again.
  void set_grad_split(bool on) {
    if (on != grad_split_) { reset_step_graph(); ++edge_generation_; }
    grad_split_ = on;
  }
  void set_moment_mma(bool on) {
    if (on != moment_mma_) reset_step_graph();
    moment_mma_ = on;
  }

  // --- evaluation ---------------------------------------------------------------------------
  // E / F / virial for the current edges.  Outputs (device, double): per-frame energy [nframes],
  // forces [natoms][3], per-frame virial [nframes][6] in (xx, yy, zz, xy, xz, yz), site energies
  // [natoms]; any output may be null.
  void efs(double* d_energy, double* d_forces, double* d_virial, double* d_site);
  // Per-atom descriptors of the next efs() call (device [natoms][S] FP64: the scalar moments the
  // readout weighs, MLMTPR::CalcDescriptors); null turns the output off.
  void set_descriptor_output(double* d_desc) { desc_out_ = d_desc; }

  // --- staged evaluation on caller edges (SUS2SL::Kernel begin / pack_forward / unpack_forward /
  // outer / pack_reverse / add_reverse / finish, sus2_sl_kernel.h:36-42) ---------------------
  // Width of the per-atom halo vectors (the Effect gate signal h and its adjoint): F, or 0.
  int comm_width() const { return model_.gated ? model_.F : 0; }
  // Edges + gate forward pass of the owned centres.
  void stage_begin(int nowned, int nall, const int* d_types, int nedges, const int* d_i, const int* d_j,
                   const double* d_d);
  // Outer (or Static) pass; for Effect models also the per-atom gate-signal adjoint of every atom.
  void stage_outer();
  // Gate reverse pass, forces (all atoms, ghosts included), site energies, energy, virial.
  void stage_finish(double* d_energy, double* d_forces, double* d_virial, double* d_site);
  // Halo rows (device arrays): which 0 = gate signal h (between begin and outer), 1 = its adjoint
  // (between outer and finish); op 0 packs rows into d_buf, op 1 writes (h) / adds (adjoint) them.
  // Rows are d_atoms[k] (distinct atoms), or first + k when d_atoms is null; d_buf is
  // [n][comm_width()] FP64.
  void stage_rows(int which, int op, int n, const int* d_atoms, int first, double* d_buf);

  // Parameter gradient of  sum_i ew_i E_i + sum_e (fw_i - fw_j + sw_frame d_e) . dE/dd_e  for the
  // frames of the last build_edges (AccumulateEFSCombinationGrad).  Device arrays (double):
  // ew [N], fw [N][3], sw [nframes][9] (row-major); the result is ADDED into grad [nparams].
  // d_extra_h [N][F] (Effect, optional): further dJ/dh per atom of objective terms that depend on
  // the gate signal h, pulled back through the gate chain with the rest.
  void combination_grad(const double* d_ew, const double* d_fw, const double* d_sw, double* d_grad,
                        const double* d_extra_h = nullptr);
  // Device views used by objective terms of the gate signal (Effect): h [N][F] of the last
  // evaluation (compute precision), the gate additive factors alpha [C][F] (compute precision) and
  // their offset in the parameter vector.
  const void* d_gate_signal() const { return hsig_.ptr; }
  const void* d_gate_additive() const;
  int gate_additive_offset() const;

  int natoms() const { return natoms_; }
  int ncentres() const { return ncentres_; }
  int nframes() const { return nframes_; }
  // Directed edges of the last build (for cell-list-only batches read back from the device on
  // first request: the build itself does not synchronise).
  long long nedges();
  // Copies the directed edges of the last build to host arrays in centre order, each centre's
  // edges in the engine's order (sorted by neighbour, then image): centre[k], neighbour[k],
  // d[3k..3k+2] = x_j - x_i (the compute precision's record, widened to double).  Writes at most
  // cap edges (any array may be null); *count = the total.  Synchronises the stream.
  void copy_edges(long long cap, int* centre, int* neighbour, double* d, long long* count);
  // number of kernels launched by the last build_edges + efs (for launch accounting)
  int last_launches() const { return launches_; }
  void reset_launch_count() { launches_ = 0; }
  // Raises if a kernel recorded an error (synchronises the stream).
  void check_device_error();

  // Stage timer: when enabled, each stage of build_edges / efs is bracketed by CUDA events on
  // the engine's stream.  Stages: 0 edge build, 1 Static/outer pass, 2 gate forward pass,
  // 3 gate reverse pass, 4 force gather + frame reductions.
  void set_timing(bool on);
  // Synchronises, then adds the elapsed milliseconds and launch counts per stage since the last
  // call into ms[8] / counts[8] and resets them.
  void take_stage_times(double* ms, int* counts);

  // Grow-only device staging buffer `slot` (0..7) of at least `bytes`, owned by the engine, for
  // entry points that copy host arrays in and out.
  void* io(int slot, size_t bytes) { io_[slot].ensure(bytes ? bytes : 1); return io_[slot].ptr; }
  // Pinned host staging of the host-buffer entry points (grows; freed with the engine).
  void* pinned(size_t bytes);
  // check_device_error in two halves: queue the copy of the error words, then (after the caller's
  // own synchronisation of the engine stream) evaluate them.
  void enqueue_error_read();
  void check_error_read();

  // Static FP32 pass on caller / external buffers (used by the allocation-free entry point):
  // natoms centres, CSR edges (row, nbr) with edge records d4 (EdgeF), outputs g[3E], site[natoms],
  // vir[6 natoms]; launches on stream().  Returns the number of kernels launched.
  int static_pass_external(int natoms, const int* types, const int* row, const int* nbr, const void* d4, float* g,
                           double* site, double* vir, int* error);
  int sm_count() const { return sm_count_; }

  // internal buffers exposed for the tests / parameter-gradient pass
  const int* d_row() const { return row_.as<int>(); }
  // one past each centre's last edge: a separate array for cell-list batches (edges in padded
  // per-centre slots), row + 1 for CSR layouts
  const int* d_row_end() const { return padded_ ? row_end_.as<int>() : row_.as<int>() + 1; }
  const int* d_nbr() const { return nbr_.as<int>(); }
  const int* d_rev() const { return rev_.as<int>(); }

 private:
  template <typename Real> void upload_tables();
  template <typename Real> PassArgs<Real> pass_args();
  template <typename Real> void autotune_passes(int reps, int* blocks_out, double* ms_out);
  enum : int { kStageGate = 1, kStageOuter = 2, kStageFinish = 4, kStageAll = 7 };
  template <typename Real>
  void run_efs(double* d_energy, double* d_forces, double* d_virial, double* d_site, int stages);
  int staged_ = 0;  // staged evaluation: 1 after begin, 2 after outer
  double* desc_out_ = nullptr;
  // step graph (step_frames)
  bool step_graphs_ = true, capturing_ = false;
  int pdl_ = -1;  // set from the model in the constructor
  bool moment_mma_ = false;
  int urgent_priority_ = 0;  // the device's most urgent stream priority
  cudaGraph_t step_graph_ = nullptr;
  cudaGraphExec_t step_exec_ = nullptr;
  std::vector<double> step_key_;
  int step_launches_ = 0;
  unsigned long long step_gen_ = ~0ull;
  template <typename Real>
  void run_grad(const double* ew, const double* fw, const double* sw, double* grad, const double* extra_h);
  DevBuf slots_, slot_part_, hsigd_, gmomd_, lhm_, lh_atom_;
  DevBuf gabar_;                // moment adjoints between the parts of a split gradient pass
  bool grad_split_ = true;      // gradient passes split at the per-atom boundary (basis size 8)
  void finalize_edges();

  Model model_;
  int device_ = 0, precision_ = kFP32;
  cudaStream_t own_stream_ = nullptr, stream_ = nullptr;
  int sm_count_ = 0;
  int launches_ = 0;
  unsigned long long edge_generation_ = 0;

  // model tables (both precisions are packed into one buffer each)
  DevBuf tab_int_, tab_real_, tab_dbl_, tab_prog_;
  std::unique_ptr<HostProg> prog_[2];  // outer and gate graph programs (structure built once)
  void* dev_model_ = nullptr;  // host copy of DevModel<Real>

  // geometry
  int natoms_ = 0, nframes_ = 0, ncentres_ = 0, bins_frames_ = 0;
  long long nedges_ = 0;          // edge slots: exact count, or the padded capacity of a deferred build
  long long exact_edges_ = 0;
  bool nedges_exact_ = true;
  int min_cap_ = 0;              // lower bound of the padded capacity after an overflow
  std::vector<FramePlan>* plans_ = nullptr;
  DevBuf plan_, frame_of_, frame_begin_, types_copy_;
  DevBuf counts_, row_, row_end_, nbr_, rev_, d4_, key_, tmp_key_, tmp_d4_, tmp_nbr_;
  bool padded_ = false;         // cell-list batch: edges left in padded per-centre slots (row_end_)
  int bin_zeroed_ = 0;          // leading bin counters known to be zero on the device
  int bins_used_ = 0;           // bin counters used by the current cell-list build
  DevBuf posf_;  // double-float positions of image-scan batches (FP32 engines)
  DevBuf bin_count_, bin_rec_, bin_pos_, bin_posf_, rec_of_;
  const int* d_types_ = nullptr;
  bool user_edges_ = false;     // caller-supplied edges: no reverse partners, scatter instead of gather
  DevBuf hbar_atom_, bin_of_, frac_, off_, in_row_, in_edge_;  // in_*: caller edges grouped by neighbour
  DevBuf pad_nbr_, pad_d4_, pad_key_;  // padded single-pass staging of cell-list frames
  double cap_scale_ = 2.0;      // padded capacity = cap_scale x mean neighbour count + 64 (grows on overflow)
  double bin_cap_scale_ = 2.0;  // bin capacity = bin_cap_scale x mean atoms per bin + 8 (grows on overflow)
  int min_bin_cap_ = 0;          // lower bound of the bin capacity after an overflow
  bool clear_bins_ = false;
  int* host_total_ = nullptr;   // pinned [4]
  // stage timer (cudaEvent pairs per stage, enabled by set_timing)
  bool timing_ = false;
  std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> marks_;
  std::vector<cudaEvent_t> event_pool_;
  size_t event_next_ = 0;
  double stage_ms_[8] = {0};
  int stage_count_[8] = {0};
  cudaEvent_t take_event();
  void mark_begin(int stage);
  void mark_end();
  int open_stage_ = -1;
  cudaEvent_t open_event_ = nullptr;
  // step buffers
  DevBuf g_, hsig_, hcontrib_, gmom_, site_, vir_atom_, error_, frame_partial_, frame_arrivals_;
  int arrivals_frames_ = 0;     // frame_arrivals_ entries known to be zero
  DevBuf scratch_;
  DevBuf io_[8];
  int pass_blocks_[4] = {0, 0, 0, 0};  // register budget per pass mode (0: the default)
  int pass_grid_[4] = {0, 0, 0, 0};    // grid shape per pass mode (PassArgs::grid_mode)
  int pass_order_[4] = {0, 0, 0, 0};   // centre order per pass mode (PassArgs::atom_order)
  int pass_stage_[4] = {0, 0, 0, 0};   // h_j staging per pass mode (PassArgs::h_bulk; outer pass)
  int pass_wpb_[4] = {4, 4, 4, 4};     // warps per block per pass mode (PassArgs::block_warps)
  template <typename Real> int launch_pass(int mode, PassArgs<Real> a, bool pdl);
  template <typename Real> int launch_shape(int mode, PassArgs<Real> a, int blocks, bool pdl);
  static constexpr int kWorkInts = 32;  // work_: (next centre, warps done) per pass mode (< 16)
  DevBuf work_;                 // counters of the dynamic centre order
  template <typename Real> bool use_static_split() const;
  template <typename Real> bool use_gate_split(int which) const;
  template <typename Real> int launch_gate_split(int which, PassArgs<Real> a, bool pdl);
  template <typename Real> int launch_static_split(PassArgs<Real> a, bool pdl);
  bool static_split_ = false;   // energy pass as forward / per-atom graph / adjoint kernels
  int split_blocks_ = 0;        // register budget of the split's per-edge kernels (0 = default)
  bool gate_split_[2] = {false, false};  // Effect gate forward / reverse passes split
  int gate_split_blocks_[2] = {0, 0};    // their per-edge kernels' register budgets
  DevBuf mom_, amom_;           // the split pass's moments and adjoint moments [N][K H]
  // second stream for independent work inside a step (reverse edges beside the first pass, the
  // frame reduction beside the force gather)
  cudaStream_t aux_stream_ = nullptr;
  cudaEvent_t ev_fork_ = nullptr, ev_rev_ = nullptr, ev_fork2_ = nullptr, ev_join2_ = nullptr;
  bool rev_pending_ = false;
  bool may_fork() const;
  void wait_reverse();
  void* pinned_ = nullptr;
  size_t pinned_bytes_ = 0;
};

}  // namespace sus2g
