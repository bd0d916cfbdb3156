"""Python host API over the C ABI: models, engines and E / F / virial evaluation.

Mirrors the reference's call surface for this path:
  * ``Model(path)``                    ~ SUS2SL::Model::load / MLMTPR::Load (.sus2)
  * ``Engine.calc_efs(frames)``        ~ MLMTPR::CalcEFS over a batch of periodic frames (calc-efs)
  * ``Engine.efs_edges(...)``          ~ SUS2SL::Kernel begin/outer/finish as called by
                                         PairSUS2Embedded::compute (sus2/embedded)
  * ``Engine.stage_*`` / ``pack_*``    ~ the same with the pair style's halo exchange between the
                                         stages (pack_forward / unpack_forward / pack_reverse /
                                         add_reverse, pair_sus2_embedded.cpp:327-374)
Errors raise ``Sus2Error`` with the library's message, as the reference raises on invalid input.
"""
from __future__ import annotations

import ctypes

import numpy as np

from ._lib import Sus2Error, check, load

__all__ = ["Model", "Engine", "Sus2Error", "FP64", "FP32"]

FP64 = 0
FP32 = 1
_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)


def _d(a):
    return a.ctypes.data_as(_dp) if a is not None else None


def _i(a):
    return a.ctypes.data_as(_ip) if a is not None else None


def _addr(a):
    """Address of an array for the c_void_p arguments of the per-step entry points.  Unlike
    data_as it holds no reference: the caller keeps ``a`` alive in a local across the call."""
    return a.ctypes.data


DIM_NAMES = ("C", "L", "K", "B", "F", "M", "NB", "P", "S", "Q", "gated", "nparams", "outer_rank", "gate_rank",
             "split", "reserved")


class Model:
    """A loaded ``.sus2`` SUS2-SH model (host tables)."""

    def __init__(self, path: str):
        lib = load()
        h = ctypes.c_void_p()
        check(lib.sus2g_model_load(str(path).encode(), ctypes.byref(h)))
        self._h = h
        self.path = str(path)
        d = (ctypes.c_int * 16)()
        check(lib.sus2g_model_dims(h, d))
        self.dims = dict(zip(DIM_NAMES, list(d)))
        c = ctypes.c_double()
        check(lib.sus2g_model_cutoff(h, ctypes.byref(c)))
        self.cutoff = c.value

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            load().sus2g_model_free(h)
            self._h = None

    @property
    def nparams(self) -> int:
        return self.dims["nparams"]

    def params(self) -> np.ndarray:
        out = np.zeros(self.nparams)
        check(load().sus2g_model_get_params(self._h, _d(out), out.size))
        return out

    def set_params(self, values) -> None:
        v = np.ascontiguousarray(values, dtype=np.float64)
        check(load().sus2g_model_set_params(self._h, _d(v), v.size))

    @property
    def scaling(self) -> float:
        """The global radial scaling (the .sus2 `scaling` field; not a trained parameter)."""
        v = ctypes.c_double()
        check(load().sus2g_model_get_scaling(self._h, ctypes.byref(v)))
        return v.value

    @scaling.setter
    def scaling(self, value: float) -> None:
        check(load().sus2g_model_set_scaling(self._h, float(value)))

    def save(self, path: str) -> None:
        """Write the model with its current parameters as a ``.sus2`` file (MLMTPR::Save)."""
        check(load().sus2g_model_save(self._h, str(path).encode()))


class Engine:
    """A model bound to one CUDA device in FP64 (``FP64``) or FP32-bulk (``FP32``) form."""

    def __init__(self, model: Model, device: int = 0, precision: int = FP32):
        self.model = model
        h = ctypes.c_void_p()
        check(load().sus2g_engine_create(model._h, int(device), int(precision), ctypes.byref(h)))
        self._h = h
        self.precision = precision
        self.device = int(device)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            load().sus2g_engine_free(h)
            self._h = None

    def update_params(self) -> None:
        check(load().sus2g_engine_update_params(self._h, self.model._h))

    def set_stream(self, stream_ptr: int | None) -> None:
        check(load().sus2g_engine_set_stream(self._h, ctypes.c_void_p(stream_ptr or 0)))

    def take_launch_count(self) -> int:
        n = ctypes.c_int()
        check(load().sus2g_engine_take_launch_count(self._h, ctypes.byref(n)))
        return n.value

    def edge_count(self) -> int:
        n = ctypes.c_longlong()
        check(load().sus2g_engine_edge_count(self._h, ctypes.byref(n)))
        return n.value

    PASSES = ("static", "gate_forward", "outer", "gate_reverse")

    def edges(self):
        """Directed edges of the last evaluation: (centre[E], neighbour[E], d[E, 3] = x_j - x_i), in
        centre order, each centre's edges sorted by neighbour, then image."""
        lib = load()
        n = ctypes.c_longlong()
        check(lib.sus2g_engine_copy_edges(self._h, 0, None, None, None, ctypes.byref(n)))
        ci = np.zeros(n.value, np.int32)
        cj = np.zeros(n.value, np.int32)
        d = np.zeros((n.value, 3))
        check(lib.sus2g_engine_copy_edges(self._h, n.value, _i(ci), _i(cj), _d(d), ctypes.byref(n)))
        return ci, cj, d

    def autotune(self, reps: int = 5):
        """Times every tile shape of every pass on the last evaluation's layout -- register budget,
        grid, centre order, warps per block, and (FP32, basis size 8) the split at the per-atom
        boundary and the outer pass's bulk-copy staging -- and keeps the fastest (``pass_shapes()``
        reports it); returns {pass: (chosen blocks per SM of the fused pass, {blocks: best ms per
        launch of the fused pass with that budget})}."""
        b = (ctypes.c_int * 4)()
        ms = (ctypes.c_double * 8)()
        check(load().sus2g_engine_autotune(self._h, int(reps), b, ms))
        return {name: (b[q], {3: ms[2 * q], 4: ms[2 * q + 1]}) for q, name in enumerate(self.PASSES) if b[q]}

    def pass_shapes(self):
        """Tile shape of each pass the model runs: {pass: {"blocks_per_sm", "grid", "order",
        "warps_per_block", "split", "bulk_h"}} (grid "resident" / "balanced", order "strided" /
        "contiguous" / "dynamic"; split: the Static pass as three kernels; bulk_h: the outer pass's
        gate-signal rows by bulk async copies)."""
        out = {}
        shape = (ctypes.c_int * 4)()
        passes = ("gate_forward", "outer", "gate_reverse") if self.model.dims["gated"] else ("static",)
        for q, name in enumerate(self.PASSES):
            if name not in passes:
                continue
            check(load().sus2g_engine_pass_shape(self._h, q, shape))
            out[name] = {"blocks_per_sm": shape[0], "grid": ("resident", "balanced")[shape[1]],
                         "order": ("strided", "contiguous", "dynamic")[shape[2] & 3],
                         "warps_per_block": shape[3], "split": bool(shape[2] & 4),
                         "bulk_h": bool(shape[2] & 8)}
        return out

    def set_pass_shape(self, name: str, blocks_per_sm: int = 0, grid: str = "resident",
                       order: str = "strided", bulk_h: bool = False, warps_per_block: int = 4) -> None:
        """Pins the tile shape of one pass (a name of PASSES) as the autotuner would set it;
        bulk_h: the outer pass's gate-signal rows by bulk async copies."""
        check(load().sus2g_engine_set_pass_shape(self._h, self.PASSES.index(name), int(blocks_per_sm),
                                                 ("resident", "balanced").index(grid),
                                                 ("strided", "contiguous", "dynamic").index(order),
                                                 1 if bulk_h else 0, int(warps_per_block)))

    def set_step_graph(self, on: bool) -> None:
        """Replay repeated periodic steps of an unchanged layout as one CUDA graph (default on)."""
        check(load().sus2g_engine_set_step_graph(self._h, 1 if on else 0))

    def set_grad_split(self, on: bool) -> None:
        """The outer / gate reverse parameter-gradient passes as per-atom + per-edge kernels
        (default on; basis size 8)."""
        check(load().sus2g_engine_set_grad_split(self._h, 1 if on else 0))

    def set_static_split(self, on: bool) -> None:
        """FP32 engines, basis size 8: every per-atom pass split at the per-atom boundary (the
        energy pass as forward / per-atom graph / adjoint kernels, the Effect gate passes as two
        kernels each) instead of fused; the autotuner chooses per pass."""
        check(load().sus2g_engine_set_static_split(self._h, 1 if on else 0))

    def set_moment_mma(self, on: bool) -> None:
        """FP32 engines: edge->moment batch sums on the tensor cores (3xTF32 mma.sync) instead of
        CUDA-core FMAs (off by default)."""
        check(load().sus2g_engine_set_moment_mma(self._h, 1 if on else 0))

    PDL_FILL, PDL_FIRST_PASS, PDL_BETWEEN_PASSES, PDL_GATHER = 1, 2, 4, 8

    def set_pdl(self, sites: int = -1) -> None:
        """Programmatic dependent launch between the kernels of an evaluation, per launch site (a
        mask of the PDL_* bits; 0 none, -1 the model's default)."""
        check(load().sus2g_engine_set_pdl(self._h, int(sites)))

    STAGES = ("edges", "outer", "gate_forward", "gate_reverse", "gather")

    def set_timing(self, on: bool) -> None:
        check(load().sus2g_engine_set_timing(self._h, 1 if on else 0))

    def take_stage_times(self):
        """{stage: (milliseconds, count)} accumulated since the last call (synchronises)."""
        ms = (ctypes.c_double * 8)()
        cnt = (ctypes.c_int * 8)()
        check(load().sus2g_engine_take_stage_times(self._h, ms, cnt))
        return {name: (ms[i], cnt[i]) for i, name in enumerate(self.STAGES)}

    # -- periodic frames ------------------------------------------------------------------------
    @staticmethod
    def pack_frames(frames):
        if len(frames) == 1:
            # one frame: its arrays as they are when they already have the layout of the C ABI
            f = frames[0]
            return (np.array([f.natoms], dtype=np.int32), np.ascontiguousarray(f.cell, dtype=np.float64).reshape(1, 3, 3),
                    np.ascontiguousarray(f.positions, dtype=np.float64), np.ascontiguousarray(f.types, dtype=np.int32))
        natoms = np.array([f.natoms for f in frames], dtype=np.int32)
        cells = np.ascontiguousarray(np.stack([f.cell for f in frames]) if frames else np.zeros((0, 3, 3)),
                                     dtype=np.float64)
        pos = np.ascontiguousarray(np.concatenate([f.positions for f in frames]) if frames else np.zeros((0, 3)),
                                   dtype=np.float64)
        types = np.ascontiguousarray(np.concatenate([f.types for f in frames]) if frames else np.zeros(0),
                                     dtype=np.int32)
        return natoms, cells, pos, types

    def calc_efs(self, frames):
        """Host arrays in and out: returns (energy[nf], forces[N,3], virial[nf,6], site[N])."""
        natoms, cells, pos, types = self.pack_frames(frames)
        nf, n = natoms.size, int(natoms.sum())
        e = np.empty(nf)
        f = np.empty((n, 3))
        v = np.empty((nf, 6))
        s = np.empty(n)
        check(load().sus2g_calc_efs_host(self._h, nf, _addr(natoms), _addr(cells), _addr(pos), _addr(types),
                                         _addr(e), _addr(f), _addr(v), _addr(s)))
        return e, f, v, s

    def calc_descriptors(self, frames) -> np.ndarray:
        """Per-atom descriptors [N, S] (the scalar moments; MLMTPR::CalcDescriptors / calc-descriptors)."""
        natoms, cells, pos, types = self.pack_frames(frames)
        out = np.zeros((int(natoms.sum()), self.model.dims["S"]))
        check(load().sus2g_calc_descriptors_host(self._h, natoms.size, _i(natoms), _d(cells), _d(pos), _i(types),
                                                 _d(out)))
        return out

    def calc_efs_device(self, natoms, cells, pos_ptr: int, types_ptr: int, energy_ptr: int = 0, forces_ptr: int = 0,
                        virial_ptr: int = 0, site_ptr: int = 0) -> None:
        """Device pointers (e.g. ``tensor.data_ptr()``) for positions/types/outputs; host natoms/cells."""
        natoms = np.ascontiguousarray(natoms, dtype=np.int32)
        cells = np.ascontiguousarray(cells, dtype=np.float64)
        check(load().sus2g_calc_efs_device(self._h, natoms.size, _addr(natoms), _addr(cells), pos_ptr or None,
                                           types_ptr or None, energy_ptr or None, forces_ptr or None,
                                           virial_ptr or None, site_ptr or None))

    def combination_grad(self, frames, ene_w, frc_w, str_w, grad=None):
        """d/dtheta of sum_i ene_w_i E_i + sum_e (frc_w_i - frc_w_j + str_w d_e) . dE/dd_e (host arrays).

        ``ene_w`` [N], ``frc_w`` [N, 3], ``str_w`` [nframes, 3, 3]; returns ``grad`` (accumulated into
        when given) in the parameter order of ``Model.params()``."""
        natoms, cells, pos, types = self.pack_frames(frames)
        nf = natoms.size
        ew = np.ascontiguousarray(ene_w, dtype=np.float64).reshape(-1)
        fw = np.ascontiguousarray(frc_w, dtype=np.float64).reshape(-1, 3)
        sw = np.ascontiguousarray(str_w, dtype=np.float64).reshape(nf, 9)
        g = np.zeros(self.model.nparams) if grad is None else np.ascontiguousarray(grad, dtype=np.float64)
        check(load().sus2g_efs_combination_grad_host(self._h, nf, _i(natoms), _d(cells), _d(pos), _i(types), _d(ew),
                                                     _d(fw), _d(sw), _d(g)))
        return g

    def combination_grad_device(self, natoms, cells, pos_ptr: int, types_ptr: int, ene_w_ptr: int, frc_w_ptr: int,
                                str_w_ptr: int, grad_ptr: int) -> None:
        """combination_grad with device pointers (positions, types, weights, grad accumulated
        into; host natoms / cells), on the engine's stream; returns when the gradient is done."""
        natoms = np.ascontiguousarray(natoms, dtype=np.int32)
        cells = np.ascontiguousarray(cells, dtype=np.float64)
        check(load().sus2g_efs_combination_grad_device(self._h, natoms.size, _addr(natoms), _addr(cells),
                                                       pos_ptr or None, types_ptr or None, ene_w_ptr or None,
                                                       frc_w_ptr or None, str_w_ptr or None, grad_ptr or None))

    # -- caller edge list (pair_style sus2/embedded) --------------------------------------------
    def efs_edges(self, nowned: int, types, ei, ej, d):
        types = np.ascontiguousarray(types, dtype=np.int32)
        ei = np.ascontiguousarray(ei, dtype=np.int32)
        ej = np.ascontiguousarray(ej, dtype=np.int32)
        d = np.ascontiguousarray(d, dtype=np.float64).reshape(-1, 3)
        nall = types.size
        e = np.zeros(1)
        s = np.zeros(nowned)
        f = np.zeros((nall, 3))
        v = np.zeros(6)
        check(load().sus2g_efs_edges_host(self._h, int(nowned), nall, _i(types), ei.size, _i(ei), _i(ej), _d(d),
                                          _d(e), _d(s), _d(f), _d(v)))
        return float(e[0]), s, f, v

    # -- staged evaluation with a caller halo exchange (multi-domain sus2/embedded) ---------------
    def comm_width(self) -> int:
        """Doubles per atom in each halo exchange (the Effect gate signal width F; 0 for Static)."""
        w = ctypes.c_int()
        check(load().sus2g_engine_comm_width(self._h, ctypes.byref(w)))
        return w.value

    def stage_begin(self, nowned: int, types, ei, ej, d) -> None:
        types = np.ascontiguousarray(types, dtype=np.int32)
        ei = np.ascontiguousarray(ei, dtype=np.int32)
        ej = np.ascontiguousarray(ej, dtype=np.int32)
        d = np.ascontiguousarray(d, dtype=np.float64).reshape(-1, 3)
        check(load().sus2g_stage_begin(self._h, int(nowned), types.size, _i(types), ei.size, _i(ei), _i(ej), _d(d)))

    def pack_forward(self, atoms) -> np.ndarray:
        atoms = np.ascontiguousarray(atoms, dtype=np.int32)
        buf = np.zeros((atoms.size, self.comm_width()))
        check(load().sus2g_stage_pack_forward(self._h, atoms.size, _i(atoms), _d(buf)))
        return buf

    def unpack_forward(self, first: int, buf) -> None:
        buf = np.ascontiguousarray(buf, dtype=np.float64)
        n = buf.shape[0] if buf.ndim == 2 else 0
        check(load().sus2g_stage_unpack_forward(self._h, n, int(first), _d(buf)))

    def stage_outer(self) -> None:
        check(load().sus2g_stage_outer(self._h))

    def pack_reverse(self, first: int, n: int) -> np.ndarray:
        buf = np.zeros((int(n), self.comm_width()))
        check(load().sus2g_stage_pack_reverse(self._h, int(n), int(first), _d(buf)))
        return buf

    def add_reverse(self, atoms, buf) -> None:
        atoms = np.ascontiguousarray(atoms, dtype=np.int32)
        buf = np.ascontiguousarray(buf, dtype=np.float64)
        check(load().sus2g_stage_add_reverse(self._h, atoms.size, _i(atoms), _d(buf)))

    def stage_finish(self, nowned: int, nall: int):
        """(energy, site_energy[nowned], forces[nall, 3], virial[6])."""
        e = np.zeros(1)
        s = np.zeros(nowned)
        f = np.zeros((nall, 3))
        v = np.zeros(6)
        check(load().sus2g_stage_finish(self._h, _d(e), _d(s), _d(f), _d(v)))
        return float(e[0]), s, f, v
