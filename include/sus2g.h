/*
 * sus2g.h -- C ABI of the GB300 SUS2-SH descriptor -> energy -> force / virial / parameter-gradient
 * engine.  Plain pointers and sizes only; every function returns 0 on success or a positive error
 * code, with the message available from sus2g_last_error() (thread-local).  No C++ exceptions
 * cross this boundary (the reference converts its exceptions to LAMMPS errors at the same seam,
 * interfaces/lammps/ML-SUS2/pair_sus2_embedded.cpp:311-313).
 *
 * Reference interfaces each entry point replaces are cited as file:line within the reference
 * project (hu-yanxiao/superlinear).
 *
 * Units are the reference's (metal): A, eV, eV/A; virial components are ordered
 * (xx, yy, zz, xy, xz, yz) and equal the reference's plus_stress / Result::virial
 * (sus2_sl_kernel.cpp:545-546): W = -sum_edges d (x) dE/dd.
 */
#ifndef SUS2G_H
#define SUS2G_H

#ifdef __cplusplus
extern "C" {
#endif

#define SUS2G_FP64 0 /* plain FP64 evaluation */
#define SUS2G_FP32 1 /* FP32 bulk (radial, Y_lm, moments, contractions) with FP64 reductions */

typedef struct sus2g_model_s* sus2g_model;
typedef struct sus2g_engine_s* sus2g_engine;

/* Message of the last failed call on this thread ("" if none). */
const char* sus2g_last_error(void);
/* ABI version (major * 100 + minor). */
int sus2g_abi_version(void);

/* ---- model (.sus2) --------------------------------------------------------------------------
 * Replaces LAMMPS_NS::SUS2SL::Model::load + Model::validate
 * (interfaces/lammps/ML-SUS2/sus2_sl_model.cpp:174-257, 258-453) and the trainer's
 * MLMTPR::Load (dev_src/mtpr.cpp:4490) for the Static and Effect families. */
int sus2g_model_load(const char* path, sus2g_model* out);
void sus2g_model_free(sus2g_model model);
/* dims[16] = {species C, l_max L, k_max K, basis B, radial funcs F, moments M, basics NB,
 *             products P, scalars S, gate scalars Q, gated, param count, outer rank, gate rank,
 *             split cutoff, 0}.
 * Replaces the Model / Kernel dimension accessors (sus2_sl_model.h:13-18, sus2_sl_kernel.h:24-31). */
int sus2g_model_dims(sus2g_model model, int* dims16);
/* Neighbour cutoff max_dist (Model::cutoff, sus2_sl_model.cpp:154-159; ZBL is outside this path). */
int sus2g_model_cutoff(sus2g_model model, double* cutoff);
/* Trainable parameter vector in the reference trainer's order
 * (MLMTPR::CoeffCount / Coeff, dev_src/mtpr.h:1340-1347; layout DistributeCoeffs, :1358-1470). */
int sus2g_model_param_count(sus2g_model model, int* count);
int sus2g_model_get_params(sus2g_model model, double* out, int n);
int sus2g_model_set_params(sus2g_model model, const double* in, int n);
/* The model's global radial scaling (the .sus2 `scaling` field, MLMTPR::scaling; not part of the
 * parameter vector).  set: positive and finite; an engine picks it up through
 * sus2g_engine_update_params, and sus2g_model_save writes it. */
int sus2g_model_get_scaling(sus2g_model model, double* scaling);
int sus2g_model_set_scaling(sus2g_model model, double scaling);
/* Write the model with its current parameter vector as a .sus2 file the reference loads
 * (replaces MLMTPR::Save, dev_src/mtpr.cpp:6893): the loaded fields in file order, the trainable
 * blocks replaced by the current values in %.17e (bit-exact on reload). */
int sus2g_model_save(sus2g_model model, const char* path);

/* ---- engine -----------------------------------------------------------------------------------
 * Replaces SUS2SL::Kernel(const Model&) (sus2_sl_kernel.cpp:45-106): binds a model to one CUDA
 * device in FP64 (SUS2G_FP64) or FP32-bulk (SUS2G_FP32) form.  The engine snapshots the model's
 * parameters; call sus2g_engine_update_params after sus2g_model_set_params. */
int sus2g_engine_create(sus2g_model model, int device, int precision, sus2g_engine* out);
void sus2g_engine_free(sus2g_engine engine);
int sus2g_engine_update_params(sus2g_engine engine, sus2g_model model);
/* Use a caller CUDA stream (cudaStream_t passed as void*; NULL restores the engine's own). */
int sus2g_engine_set_stream(sus2g_engine engine, void* cuda_stream);
/* Kernels launched by the engine since the last call to this function. */
int sus2g_engine_take_launch_count(sus2g_engine engine, int* count);
/* Number of directed edges of the last evaluation. */
int sus2g_engine_edge_count(sus2g_engine engine, long long* count);
/* The directed edge set of the last evaluation, copied to host arrays in centre order (each centre's
 * edges sorted by neighbour, then periodic image): centre[k], neighbour[k] (atom indices within the
 * batch), d[3k..3k+2] = x_j - x_i in the compute precision's record widened to double.  At most cap
 * edges are written (any array may be NULL); *count receives the total.  Replaces reading the
 * reference's neighbour lists: Neighborhoods::InitNbhs (src/neighborhoods.cpp:358) and the embedded
 * harness's edge list (interfaces/lammps/tests/embedded_efs.cpp:46-66).  Synchronises. */
int sus2g_engine_copy_edges(sus2g_engine engine, long long cap, int* centre, int* neighbour, double* d,
                            long long* count);
/* Stage timer (CUDA events on the engine's stream), the counterpart of the reference's
 * profile_every stage timers and Kernel::outer_profile (pair_sus2_embedded.cpp:261-264,320-361;
 * sus2_sl_kernel.h:33-35).  Stages: 0 edge build, 1 Static/outer pass, 2 gate forward pass,
 * 3 gate reverse pass, 4 force gather + per-frame reductions.  take_stage_times synchronises and
 * returns milliseconds[8] and event-pair counts[8] accumulated since the previous call. */
int sus2g_engine_set_timing(sus2g_engine engine, int enabled);
int sus2g_engine_take_stage_times(sus2g_engine engine, double* ms8, int* counts8);

/* ---- E / F / virial of periodic frames (trainer calc-efs path) ----------------------------------
 * Replaces MLMTPR::CalcEFS(Configuration&) (dev_src/mtpr.cpp:8779-8956) including its
 * Neighborhoods build (src/neighborhoods.cpp:358-415) for a batch of frames.
 *   nframes, natoms[nframes]      frame sizes; atoms of all frames concatenated
 *   cells[9*nframes]              host, rows are the lattice vectors (Configuration::lattice)
 *   positions[3*N], types[N]      Cartesian positions (A) and species 0..C-1
 *   energy[nframes], forces[3*N], virial[6*nframes], site_energy[N]   outputs (any may be NULL)
 * _host: positions/types/outputs are host memory (copied inside the call, synchronous).
 * _device: positions/types/outputs are device memory on the engine's stream (asynchronous). */
int sus2g_calc_efs_host(sus2g_engine engine, int nframes, const int* natoms, const double* cells,
                        const double* positions, const int* types, double* energy, double* forces,
                        double* virial, double* site_energy);
int sus2g_calc_efs_device(sus2g_engine engine, int nframes, const int* natoms, const double* cells,
                          const double* positions, const int* types, double* energy, double* forces,
                          double* virial, double* site_energy);
/* Step graph of the two calls above: when two consecutive calls have the same layout (frame
 * sizes, cells, buffer addresses, stream) of periodic frames, the second is captured
 * as one CUDA graph (edge build + E/F/virial) and later ones replay it -- positions may change
 * between calls, as in an MD run.  Another edge build on the engine, a parameter update, the
 * stage timer or a neighbour-capacity overflow makes the next call eager again.
 * enabled = 1 (default) or 0. */
int sus2g_engine_set_step_graph(sus2g_engine engine, int enabled);
/* Programmatic dependent launch between the kernels of an E/F/virial evaluation: a kernel may be
 * scheduled, and stage its model tables, while the previous kernel of the stream drains.  sites =
 * a bit mask of launch sites: 1 the edge fill (after binning), 2 the first per-atom pass (after
 * the edge fill), 4 the Effect outer and gate-reverse passes (after the previous pass), 8 the
 * force gather (after the last pass); 0 = none, -1 = the model's default (Static 1 | 2, Effect 1:
 * the sites that measured faster on GB300).  Results are identical for every mask. */
int sus2g_engine_set_pdl(sus2g_engine engine, int sites);
/* FP32 engines: sum each 32-edge batch of the edge->moment accumulation on the tensor cores
 * (m16n8k8 TF32 mma.sync, operands split into TF32 head and tail, three products per tile) instead
 * of CUDA-core FMAs (enabled = 1; default 0).  The same sums as the reference's forward_moments
 * (interfaces/lammps/ML-SUS2/sus2_sl_kernel.cpp:340-354); kept as an option because the CUDA-core
 * form measured faster on GB300. */
int sus2g_engine_set_moment_mma(sus2g_engine engine, int enabled);
/* FP32 engines, models with basis size 8: run the energy pass (the Static pass, or the Effect
 * outer pass) as three kernels -- the edge->moment forward, the per-atom contraction / graph /
 * readout / adjoint, and the per-edge adjoint -- through device moment arrays, and the Effect
 * gate passes as two each (edge->moment forward, then the per-atom gate graph and gate-signal
 * projection; the per-atom gate-signal adjoint gather and gate graph reverse, then the per-edge
 * adjoint), instead of one fused kernel per pass (enabled = 1; default 0; the autotuner chooses
 * per pass).  The same
 * arithmetic in the same order as the fused pass, in separately compiled kernels: results agree
 * to FP32 rounding (bit for bit on the Static models tested).  No counterpart in the reference (a
 * launch-shape choice). */
int sus2g_engine_set_static_split(sus2g_engine engine, int enabled);
/* The outer and gate reverse parameter-gradient passes (sus2g_engine_combination_grad and the
 * trainer) as two kernels each -- the per-atom part (forward with tangents, readout seeds, reverse
 * sweep) writing the moment adjoints, then the per-edge parameter contributions -- instead of one
 * (enabled = 1, the default; basis size 8).  The per-warp gradient slices then receive their terms
 * in another order: results agree to the rounding of the precision and repeat bit for bit.  No
 * counterpart in the reference (a kernel-shape choice). */
int sus2g_engine_set_grad_split(sus2g_engine engine, int enabled);
/* Pass-kernel autotuner: on the layout of the engine's last evaluation, times every per-atom pass
 * the model runs in each tile shape -- compiled register budget (3 and 4 resident blocks per SM;
 * basis size 8), grid shape and centre order (sus2g_engine_pass_shape) -- over `reps` launches
 * each and keeps the fastest for later evaluations.  Grid shape and centre order never change a
 * result bit; the two register budgets are separately compiled kernels whose results agree to the
 * rounding of the precision (the compiler may form multiply-adds differently in each).
 * blocks4[mode] (may be NULL) = the chosen budgets per pass (0 Static, 1 gate forward, 2 outer,
 * 3 gate reverse; 0 for passes the model does not run), ms8[2 mode + budget - 3] (may be NULL) =
 * milliseconds per launch of the budget's fastest shape. */
int sus2g_engine_autotune(sus2g_engine engine, int reps, int* blocks4, double* ms8);
/* Tile shape of a per-atom pass (mode 0 Static, 1 gate forward, 2 outer, 3 gate reverse) as the
 * autotuner left it: shape4 = {register budget in resident blocks per SM (0 = default; for a
 * split pass, that of its per-edge kernels, which the autotuner tunes separately), grid
 * (0 all resident blocks, 1 the fewest blocks with the same centres per warp), centre order
 * (0 grid-strided, 1 contiguous runs per warp, 2 taken from a device counter as warps finish;
 * plus 4 when the Static pass runs as three kernels, sus2g_engine_set_static_split; plus 8 when
 * the Effect outer pass brings the neighbours' gate-signal rows into shared memory by 1-D bulk
 * asynchronous copies, one 32-edge batch ahead), warps per block (2 or 4 from the autotuner)}.  No counterpart in the
 * reference (its kernel has no launch shape). */
int sus2g_engine_pass_shape(sus2g_engine engine, int mode, int* shape4);
/* Sets the tile shape of a per-atom pass as the autotuner would: blocks = register budget (0
 * default, 3 or 4), grid 0 / 1 and order 0 / 1 / 2 as in sus2g_engine_pass_shape, stage 1 = the
 * bulk-copy staging of gate-signal rows (the Effect outer pass, when a row is a whole number of
 * 16-byte units; ignored otherwise), warps = warps per block (1 .. 4; the autotuner tries 2 and
 * 4) -- to pin a shape tuned once for a workload without timing it again (results as under
 * sus2g_engine_autotune).  No counterpart in the reference. */
int sus2g_engine_set_pass_shape(sus2g_engine engine, int mode, int blocks, int grid, int order, int stage,
                                int warps);

/* Per-atom descriptors of periodic frames: the S scalar moments the readout weighs, desc[N][S]
 * (host), in the order of the model's alpha_moment_mapping -- replaces MLMTPR::CalcDescriptors
 * (dev_src/mtpr.cpp:6554, the trainer's calc-descriptors command) for Static and Effect models.
 * S = dims[8] of sus2g_model_dims.  Frames as in sus2g_calc_efs_host. */
int sus2g_calc_descriptors_host(sus2g_engine engine, int nframes, const int* natoms, const double* cells,
                                const double* positions, const int* types, double* desc);

/* ---- E / F / virial of a caller edge list (pair_style sus2/embedded compute contract) ----------
 * Replaces SUS2SL::Kernel::begin / outer / finish (sus2_sl_kernel.cpp:381-562) as called by
 * PairSUS2Embedded::compute (pair_sus2_embedded.cpp:250-314) with a single domain: nowned centre
 * atoms 0..nowned-1, nall >= nowned atoms in total, types[nall], directed edges (ei, ej, d = x_j - x_i).
 * Outputs energy (sum of owned site energies), site_energy[nowned], forces[3*nall] (including
 * ghost contributions, to be reverse-communicated by the caller), virial[6].  Host buffers. */
int sus2g_efs_edges_host(sus2g_engine engine, int nowned, int nall, const int* types, int nedges,
                         const int* ei, const int* ej, const double* d, double* energy, double* site_energy,
                         double* forces, double* virial);

/* ---- staged evaluation with a caller halo exchange (multi-domain pair_style sus2/embedded) -------
 * Replaces SUS2SL::Kernel::begin / pack_forward / unpack_forward / outer / pack_reverse /
 * add_reverse / finish (sus2_sl_kernel.h:36-42, sus2_sl_kernel.cpp:381-562) as driven by
 * PairSUS2Embedded::compute and its comm callbacks (pair_sus2_embedded.cpp:289-298, 327-374):
 *   begin         caller edges of the owned centres (as in sus2g_efs_edges_host) + the Effect gate
 *                 pass of the owned atoms;
 *   forward comm  pack_forward(owned atoms by index) -> caller -> unpack_forward(ghost rows
 *                 first .. first + n - 1): the gate signal h, comm_width doubles per atom;
 *   outer         the outer (or Static) pass;
 *   reverse comm  pack_reverse(ghost rows first ..) -> caller -> add_reverse(owned atoms by index):
 *                 the gate-signal adjoint, comm_width doubles per atom;
 *   finish        gate reverse pass; energy (owned site energies), site_energy[nowned],
 *                 forces[3 * nall] (ghost contributions included, for the caller's force reverse
 *                 communication), virial[6].
 * comm_width is 0 for Static models (the exchanges are then empty).  All buffers are host memory;
 * the calls are synchronous.  Results are deterministic (no floating-point atomics). */
int sus2g_engine_comm_width(sus2g_engine engine, int* width);
int sus2g_stage_begin(sus2g_engine engine, int nowned, int nall, const int* types, int nedges, const int* ei,
                      const int* ej, const double* d);
int sus2g_stage_pack_forward(sus2g_engine engine, int n, const int* atoms, double* buf);
int sus2g_stage_unpack_forward(sus2g_engine engine, int n, int first, const double* buf);
int sus2g_stage_outer(sus2g_engine engine);
int sus2g_stage_pack_reverse(sus2g_engine engine, int n, int first, double* buf);
int sus2g_stage_add_reverse(sus2g_engine engine, int n, const int* atoms, const double* buf);
int sus2g_stage_finish(sus2g_engine engine, double* energy, double* site_energy, double* forces, double* virial);

/* ---- parameter gradient (trainer contract) ------------------------------------------------------
 * Replaces AnyLocalMLIP::AccumulateEFSCombinationGrad (src/basic_mlip.cpp:421-476) and
 * MLMTPR::AccumulateEFSCombinationGrad (dev_src/mtpr.cpp:9188) for a batch of periodic frames:
 *   grad += d/dtheta [ sum_i ene_w[i] E_i + sum_(edges i->j) w_ij . dE/dd_ij ],
 *   w_ij = frc_w[i] - frc_w[j] + str_w(frame) d_ij  (str_w row-major, w_a = sum_b S_ab d_b),
 * i.e. the energy / force / stress weights (dL/dE_i, dL/dF, dL/dS of a loss) pulled back onto the
 * parameters in the Coeff() order.  Frames as in sus2g_calc_efs_host; ene_w[N], frc_w[3N],
 * str_w[9 * nframes] and grad[param count] are host arrays (grad is accumulated into). */
int sus2g_efs_combination_grad_host(sus2g_engine engine, int nframes, const int* natoms, const double* cells,
                                    const double* positions, const int* types, const double* ene_w,
                                    const double* frc_w, const double* str_w, double* grad);
/* The same with positions, types, the weights and grad in device memory (natoms and cells on the
 * host), on the engine's stream; returns when the gradient is complete (torch's autograd path
 * for device tensors, superlinear_gb300.autograd.efs_device). */
int sus2g_efs_combination_grad_device(sus2g_engine engine, int nframes, const int* natoms, const double* cells,
                                      const double* positions, const int* types, const double* ene_w,
                                      const double* frc_w, const double* str_w, double* grad);

/* ---- training objective and BFGS --------------------------------------------------------------
 * A trainer holds a fixed set of labelled frames resident on the engine's device (edges built
 * once) and evaluates the energy / force / stress objective with its parameter gradient:
 *   replaces NonLinearRegression::CalcObjectiveFunctionGrad (dev_src/non_linear_regression.cpp:1112)
 *   over AddLoss / AddLossGrad (:768-880, :892-1068) with the energy / force / stress terms and
 *   the Effect gate-x term (std terms, relative force weights, other penalties and regularisers
 *   off), divided by the frame count K as MTPR_trainer::Train does
 *   (dev_src/mtpr_trainer.cpp:4733-4745).
 * Frames as in sus2g_calc_efs_host (host arrays, copied once).  Labels: energy[nframes],
 * forces[3 * natoms], stress[9 * nframes] (row-major 3x3 in the virial convention of the
 * reference's Configuration::stresses); has_labels[f] bit 0 energy, bit 1 forces, bit 2 stress.
 * weighting: 0 "vibrations", 1 "structures", 2 "molecules" (NonLinearRegression::weighting).
 * gate_x_l2: coefficient of the Effect gate-x L2 term (NonLinearRegression::AddGateXRegularization,
 * non_linear_regression.cpp:293-320, MLMTPR::AddTwoLayerGateX2Penalty, mtpr_sh.cpp:5869; the
 * reference's default is 1e-4, non_linear_regression.h:128); ignored for Static models.
 * The trainer keeps a reference to the engine: free the trainer before the engine. */
typedef struct sus2g_trainer_s* sus2g_trainer;
int sus2g_trainer_create(sus2g_engine engine, int nframes, const int* natoms, const double* cells,
                         const double* positions, const int* types, const double* energy, const double* forces,
                         const double* stress, const int* has_labels, double wE, double wF, double wS, int weighting,
                         int norm_by_forces, double gate_x_l2, sus2g_trainer* out);
void sus2g_trainer_free(sus2g_trainer trainer);
/* Loss (and, when grad != NULL, its gradient [param count], host) at params [param count, host,
 * Coeff() order].  The engine's parameters are replaced by params. */
int sus2g_trainer_loss_grad(sus2g_trainer trainer, const double* params, double* loss, double* grad);
/* The trainer's error metrics at params (E/F/virial only): out6 = energy MAE and RMSE (meV/atom),
 * force MAE and RMSE (meV/A), stress MAE and RMSE (eV), as NonLinearRegression collects and reports
 * them (dev_src/non_linear_regression.cpp:781-804, 1150-1184) -- the training-set error report of
 * the reference's calc-errors / train logs.  The engine's parameters are replaced by params. */
int sus2g_trainer_metrics(sus2g_trainer trainer, const double* params, double* out6);
/* Linear warm-up: replaces MTPR_trainer::TrainLinear (dev_src/mtpr_trainer.cpp:1455) with its
 * AddToSLAE rows (:1130-1453) and SolveSLAE (:971) -- the radial Chebyshev rows normalised to unit
 * norm (MLMTPR::Orthogonalize, dev_src/mtpr.cpp:14110), then the least-squares solve of the species
 * constants and the scalar readout against the labels with the trainer's weights, applied as
 * centre factor 1, shift = constant - 1, readout = solution.  params (host) in/out; the engine's
 * parameters become the result. */
int sus2g_trainer_train_linear(sus2g_trainer trainer, double* params);
/* Rescale step before the linear solve, replacing Rescale (dev_src/mlp/mtpr_train.cpp:1504-1748,
 * run by MTPR_trainer when do-lin rescaling is on, dev_src/mtpr_trainer.cpp:4040-4046): a search over
 * the model's global radial `scaling` in which every trial runs the linear warm-up above on at most
 * five of the frames (largest, second largest, median, second smallest, smallest by atom count)
 * and is judged by the median and spread of log|readout coefficient|.  params (host, in/out, the
 * trainer's Coeff() order) becomes the chosen trial's coefficients, *scaling its scaling; the
 * trainer's engine keeps both (sus2g_model_set_scaling puts the scaling into a model to save).
 * *solves (may be NULL) = linear solves run. */
int sus2g_trainer_rescale(sus2g_trainer trainer, double* params, double* scaling, int* solves);
/* Replay the evaluation as one CUDA graph (enabled = 1, default) or launch it eagerly (0). */
int sus2g_trainer_set_graph(sus2g_trainer trainer, int enabled);
/* Dense BFGS from params (in/out) for at most max_iter accepted steps or until |grad| <= gtol:
 * replaces the MTPR_trainer::Train BFGS loop (dev_src/mtpr_trainer.cpp:4985-4997) over
 * BFGS::Iterate / Linesearch::Iterate / UpdateInvHess (src/common/bfgs.cpp:251-329, 428-502,
 * bfgs.h:121-290) on the raw parameter vector; inverse Hessian, direction and update in FP64 on
 * the device.  Ends early, keeping the last accepted point, when a line search stagnates or
 * takes more than 30 trials (dev_src/mtpr_trainer.cpp:5328-5333).  history[max_iter + 1] (may be
 * NULL) receives the loss before the first and after each accepted step; *steps the accepted
 * step count; params the last accepted point. */
int sus2g_trainer_bfgs(sus2g_trainer trainer, double* params, int max_iter, double gtol, double* history,
                       int* steps);
/* Line search of the following sus2g_trainer_bfgs calls: 0 (default) the reference's Linesearch
 * (src/common/bfgs.h:31-290; the trial sequence is the reference's), 1 an interpolating strong-Wolfe
 * search (fewer evaluations per accepted step, not the reference's sequence). */
int sus2g_trainer_set_line_search(sus2g_trainer trainer, int mode);
/* Trial points of the last sus2g_trainer_bfgs call, one per objective evaluation in order: loss[k],
 * points[k * nparams ...] and accepted[k] (1 where BFGS took the point as its new start), at most
 * cap of them (arrays may be NULL); *count = the number recorded.  The record the reference's
 * trainer log gives per step (dev_src/mtpr_trainer.cpp:4640-4830). */
int sus2g_trainer_bfgs_trials(sus2g_trainer trainer, int cap, double* loss, double* points, int* accepted,
                              int* count);

/* Initial inverse Hessian of the following sus2g_trainer_bfgs calls: diag[n] (n = the parameter
 * count; finite, positive) on the diagonal, zero elsewhere; n = 0 restores the identity.  Replaces
 * BFGS::SetInvHessDiagonal (src/common/bfgs.h:395), which the reference trainer calls with its
 * per-coefficient scaling before BFGS (dev_src/mtpr_trainer.cpp:4011-4072). */
int sus2g_trainer_set_inv_hess_diagonal(sus2g_trainer trainer, const double* diag, int n);

/* ---- allocation-free Static E / F / virial ------------------------------------------------------
 * No counterpart in the reference: this entry point exists for callers that cannot allocate device
 * memory during a step -- MD drivers whose device memory comes from a pre-sized arena, and
 * integrations that forbid driver allocations in their time loop.  Every other entry point may
 * grow engine-owned buffers with cudaMalloc; this one allocates nothing: its scratch is a fixed
 * file-scope device array (about 22 MiB, held by every GPU that loads the library until exit).
 *   All array arguments are DEVICE pointers on the engine's device; the engine must hold a Static
 *   model in FP32-bulk form.  natoms centre atoms (0..natoms-1) of nall >= natoms atoms;
 *   types[nall]; edges in CSR by centre: row[natoms + 1] (row[0] = 0, row[natoms] = nedges,
 *   non-decreasing), nbr[nedges] (0..nall-1), vec[3 * nedges] = x_j - x_i (A).  Outputs (device,
 *   any may be NULL): energy[1], forces[3 * nall] (overwritten), virial[6] (xx, yy, zz, xy, xz, yz),
 *   site_energy[natoms].
 *   Limits: natoms <= 16384, nall <= 65536 and nedges <= 524288; larger calls are rejected with an
 *   error (code 6).  Bad rows or neighbour indices return 21, a species outside [0, C) 26, a zero
 *   or non-finite edge length 24; the device reads only sanitised copies of rows and neighbour
 *   indices, so bad input causes no out-of-range access.  Forces are gathered per atom in a fixed
 *   order (no floating-point atomics): results are bitwise reproducible.
 *   The first call on a device looks up the scratch array's device address for that device
 *   (cudaGetSymbolAddress).  Calls share the scratch array: calls that overlap on the GPU race and
 *   must be serialised by the caller.  The call synchronises the engine's stream to report input
 *   errors. */
int sus2g_static_efs_noalloc(sus2g_engine engine, int natoms, int nall, const int* types, const int* row,
                             const int* nbr, const double* vec, long long nedges, double* energy, double* forces,
                             double* virial, double* site_energy);

#ifdef __cplusplus
}
#endif
#endif /* SUS2G_H */
