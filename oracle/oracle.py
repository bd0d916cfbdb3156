"""ctypes wrapper of the CPU FP64 oracle (``oracle/_build/libsus2_oracle.so``).

TEST INFRASTRUCTURE ONLY: used by ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline
leg of ``bench.py`` as the checker / reported baseline.  The product path never imports it.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "libsus2_oracle.so")

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)


def build() -> str:
    """Compile the oracle with the Makefile next to this file (g++, OpenMP)."""
    r = subprocess.run(["make", "-s", "-C", HERE, "port"], capture_output=True, text=True)
    if r.returncode:
        raise RuntimeError("oracle build failed:\n" + r.stdout + r.stderr)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        L = ctypes.CDLL(LIB)
        L.orc_load.restype = ctypes.c_void_p
        L.orc_load.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_int]
        L.orc_free.argtypes = [ctypes.c_void_p]
        L.orc_param_count.argtypes = [ctypes.c_void_p]
        L.orc_get_params.argtypes = [ctypes.c_void_p, _dp]
        L.orc_set_params.argtypes = [ctypes.c_void_p, _dp]
        L.orc_get_scaling.restype = ctypes.c_double
        L.orc_get_scaling.argtypes = [ctypes.c_void_p]
        L.orc_set_scaling.argtypes = [ctypes.c_void_p, ctypes.c_double]
        L.orc_efs.restype = ctypes.c_longlong
        L.orc_efs.argtypes = [ctypes.c_void_p, ctypes.c_int, _dp, _dp, _ip, _dp, _dp, _dp, _dp, ctypes.c_int,
                              ctypes.c_char_p, ctypes.c_int]
        L.orc_efs_timed.restype = ctypes.c_longlong
        L.orc_efs_timed.argtypes = [ctypes.c_void_p, ctypes.c_int, _dp, _dp, _ip, _dp, _dp, _dp, _dp, ctypes.c_int,
                                    _dp, ctypes.c_char_p, ctypes.c_int]
        L.orc_efs_edges.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, _ip, ctypes.c_int, _ip, _ip, _dp,
                                    _dp, _dp, _dp, _dp, ctypes.c_char_p, ctypes.c_int]
        L.orc_edges.restype = ctypes.c_longlong
        L.orc_edges.argtypes = [ctypes.c_void_p, ctypes.c_int, _dp, _dp, ctypes.c_longlong, _ip, _ip, _dp,
                                ctypes.c_char_p, ctypes.c_int]
        L.orc_grad.argtypes = [ctypes.c_void_p, ctypes.c_int, _dp, _dp, _ip, _dp, _dp, _dp, _dp, ctypes.c_char_p,
                               ctypes.c_int]
        L.orc_layout.argtypes = [ctypes.c_void_p, _ip]
        L.orc_descriptors.argtypes = [ctypes.c_void_p, ctypes.c_int, _dp, _dp, _ip, _dp, ctypes.c_char_p,
                                      ctypes.c_int]
        L.orc_grad_gatex.argtypes = [ctypes.c_void_p, ctypes.c_int, _dp, _dp, _ip, _dp, _dp, _dp, ctypes.c_double,
                                     _dp, _dp, ctypes.c_char_p, ctypes.c_int]
        _lib = L
    return _lib


def _d(a):
    return a.ctypes.data_as(_dp)


def _i(a):
    return a.ctypes.data_as(_ip)


class OracleModel:
    """FP64 CPU evaluation of one ``.sus2`` model."""

    def __init__(self, path: str):
        err = ctypes.create_string_buffer(512)
        self._h = lib().orc_load(path.encode(), err, 512)
        if not self._h:
            raise ValueError(err.value.decode())
        self.nparams = lib().orc_param_count(self._h)

    def __del__(self):
        if getattr(self, "_h", None):
            lib().orc_free(self._h)
            self._h = None

    def params(self) -> np.ndarray:
        out = np.zeros(self.nparams)
        lib().orc_get_params(self._h, _d(out))
        return out

    def set_params(self, p) -> None:
        p = np.ascontiguousarray(p, dtype=np.float64)
        assert p.size == self.nparams
        lib().orc_set_params(self._h, _d(p))

    @property
    def scaling(self) -> float:
        return lib().orc_get_scaling(self._h)

    @scaling.setter
    def scaling(self, s: float) -> None:
        if lib().orc_set_scaling(self._h, float(s)) != 0:
            raise ValueError("scaling must be positive and finite")

    def efs(self, cell, pos, types, threads: int = 1):
        """One periodic frame -> (energy, forces[n,3], virial6, site[n], n_edges)."""
        cell = np.ascontiguousarray(cell, dtype=np.float64).reshape(9)
        pos = np.ascontiguousarray(pos, dtype=np.float64).reshape(-1, 3)
        types = np.ascontiguousarray(types, dtype=np.int32)
        n = types.size
        e = np.zeros(1)
        f = np.zeros((n, 3))
        v = np.zeros(6)
        s = np.zeros(n)
        err = ctypes.create_string_buffer(512)
        ne = lib().orc_efs(self._h, n, _d(cell), _d(pos), _i(types), _d(e), _d(f), _d(v), _d(s), threads, err, 512)
        if ne < 0:
            raise RuntimeError(err.value.decode())
        return float(e[0]), f, v, s, int(ne)

    def efs_timed(self, cell, pos, types, threads: int = 0):
        """One frame; returns (energy, n_edges, edge_build_seconds, compute_seconds)."""
        cell = np.ascontiguousarray(cell, dtype=np.float64).reshape(9)
        pos = np.ascontiguousarray(pos, dtype=np.float64).reshape(-1, 3)
        types = np.ascontiguousarray(types, dtype=np.int32)
        n = types.size
        e = np.zeros(1)
        f = np.zeros((n, 3))
        v = np.zeros(6)
        sec = np.zeros(2)
        err = ctypes.create_string_buffer(512)
        ne = lib().orc_efs_timed(self._h, n, _d(cell), _d(pos), _i(types), _d(e), _d(f), _d(v), None, threads,
                                 _d(sec), err, 512)
        if ne < 0:
            raise RuntimeError(err.value.decode())
        return float(e[0]), int(ne), float(sec[0]), float(sec[1])

    def edges(self, cell, pos):
        """The frame's directed edges (centre[E], neighbour[E], d[E, 3] = x_j - x_i), centre order."""
        cell = np.ascontiguousarray(cell, dtype=np.float64).reshape(9)
        pos = np.ascontiguousarray(pos, dtype=np.float64).reshape(-1, 3)
        err = ctypes.create_string_buffer(512)
        n = pos.shape[0]
        ne = lib().orc_edges(self._h, n, _d(cell), _d(pos), 0, None, None, None, err, 512)
        if ne < 0:
            raise RuntimeError(err.value.decode())
        ei = np.zeros(ne, np.int32)
        ej = np.zeros(ne, np.int32)
        d = np.zeros((ne, 3))
        lib().orc_edges(self._h, n, _d(cell), _d(pos), ne, _i(ei), _i(ej), _d(d), err, 512)
        return ei, ej, d

    def efs_edges(self, nowned, types, ei, ej, d):
        types = np.ascontiguousarray(types, dtype=np.int32)
        ei = np.ascontiguousarray(ei, dtype=np.int32)
        ej = np.ascontiguousarray(ej, dtype=np.int32)
        d = np.ascontiguousarray(d, dtype=np.float64).reshape(-1, 3)
        nall = types.size
        e = np.zeros(1)
        f = np.zeros((nall, 3))
        v = np.zeros(6)
        s = np.zeros(nowned)
        err = ctypes.create_string_buffer(512)
        rc = lib().orc_efs_edges(self._h, nowned, nall, _i(types), ei.size, _i(ei), _i(ej), _d(d), _d(e), _d(f),
                                 _d(v), _d(s), err, 512)
        if rc:
            raise RuntimeError(err.value.decode())
        return float(e[0]), f, v, s

    def layout(self) -> dict:
        out = np.zeros(12, dtype=np.int32)
        lib().orc_layout(self._h, _i(out))
        keys = ("C", "S", "B", "F", "species_readout", "o_shift", "o_radial", "o_species", "o_linear", "nparams",
                "nblk", "K")
        return dict(zip(keys, (int(x) for x in out)))

    def descriptors(self, cell, pos, types, nscalars: int) -> np.ndarray:
        """Per-atom scalar moments [n][nscalars] of one frame (MLMTPR::CalcDescriptors)."""
        cell = np.ascontiguousarray(cell, dtype=np.float64).reshape(9)
        pos = np.ascontiguousarray(pos, dtype=np.float64).reshape(-1, 3)
        types = np.ascontiguousarray(types, dtype=np.int32)
        out = np.zeros((types.size, nscalars))
        err = ctypes.create_string_buffer(512)
        if lib().orc_descriptors(self._h, types.size, _d(cell), _d(pos), _i(types), _d(out), err, 512):
            raise RuntimeError(err.value.decode())
        return out

    def grad(self, cell, pos, types, ew, fw, sw, gate_x: float = 0.0) -> np.ndarray:
        """d/dtheta of sum_i ew_i E_i + sum_e (fw_i - fw_j + sw d_e) . dE/dd_e (one frame); with
        gate_x > 0 also of the Effect gate-x L2 term, whose value is left in ``self.last_penalty``."""
        cell = np.ascontiguousarray(cell, dtype=np.float64).reshape(9)
        pos = np.ascontiguousarray(pos, dtype=np.float64).reshape(-1, 3)
        types = np.ascontiguousarray(types, dtype=np.int32)
        ew = np.ascontiguousarray(ew, dtype=np.float64)
        fw = np.ascontiguousarray(fw, dtype=np.float64).reshape(-1, 3)
        sw = np.ascontiguousarray(sw, dtype=np.float64).reshape(9)
        g = np.zeros(self.nparams)
        err = ctypes.create_string_buffer(512)
        if gate_x > 0.0:
            pen = np.zeros(1)
            if lib().orc_grad_gatex(self._h, types.size, _d(cell), _d(pos), _i(types), _d(ew), _d(fw), _d(sw),
                                    float(gate_x), _d(g), _d(pen), err, 512):
                raise RuntimeError(err.value.decode())
            self.last_penalty = float(pen[0])
            return g
        if lib().orc_grad(self._h, types.size, _d(cell), _d(pos), _i(types), _d(ew), _d(fw), _d(sw), _d(g), err, 512):
            raise RuntimeError(err.value.decode())
        return g


def virial6_to_matrix(v):
    """(xx, yy, zz, xy, xz, yz) -> symmetric 3x3 (the reference harness's virial layout)."""
    return np.array([[v[0], v[3], v[4]], [v[3], v[1], v[5]], [v[4], v[5], v[2]]])


def loss_grad(model: "OracleModel", frames, wE: float, wF: float, wS: float, weighting: str = "vibrations",
              norm_by_forces: int = 0, gate_x_l2: float = 0.0):
    """Energy / force / stress MSE objective summed over labelled frames and its parameter gradient,
    restating NonLinearRegression::AddLoss / AddLossGrad (dev_src/non_linear_regression.cpp:768-1068)
    with the std terms, penalties and regularisers off, plus, when gate_x_l2 > 0, the Effect gate-x
    L2 term (AddGateXRegularization, :293-320); the gradient goes through ``grad``."""
    d = 0.1
    loss = 0.0
    grad = np.zeros(model.nparams)
    for fr in frames:
        n = fr.natoms
        e, f, v, _, _ = model.efs(fr.cell, fr.positions, fr.types)
        s = virial6_to_matrix(v)
        avef = float(np.mean(np.sum(fr.forces ** 2, axis=1))) if fr.forces is not None else 0.0
        scale_fn = d / (d + norm_by_forces * avef)
        fw = np.zeros((n, 3))
        if wF != 0 and fr.forces is not None:
            wgt = wF / n if weighting == "structures" else wF
            delta = f - fr.forces
            loss += wgt * scale_fn * float(np.sum(delta ** 2))
            fw = wgt * scale_fn * 2.0 * delta
        we, ws = wE, wS
        if weighting == "structures":
            we, ws = wE / n, wS / n
        elif weighting == "molecules":
            we, ws = wE * n, wS * n
        sw = np.zeros((3, 3))
        if ws != 0 and fr.stress is not None:
            ds = s - fr.stress
            loss += ws * float(np.sum(ds ** 2)) / n
            sw = -2.0 * ws * ds / n
        ew = 0.0
        if we != 0 and fr.energy is not None:
            loss += we * (e - fr.energy) ** 2 * scale_fn / n
            ew = 2.0 * we * (e - fr.energy) * scale_fn / n
        grad += model.grad(fr.cell, fr.positions, fr.types, np.full(n, ew), fw, sw, gate_x=gate_x_l2)
        if gate_x_l2 > 0.0:
            loss += model.last_penalty
    return loss, grad


METRIC_NAMES = ("energy_mae_mev_per_atom", "energy_rmse_mev_per_atom", "force_mae_mev_per_a", "force_rmse_mev_per_a",
                "stress_mae_ev", "stress_rmse_ev")


def error_metrics(model: "OracleModel", frames):
    """The trainer's error metrics over labelled frames, restating the sums NonLinearRegression::AddLoss
    collects (dev_src/non_linear_regression.cpp:781-804) and their reports (:1150-1184): energy
    sum|dE| / sum N and sqrt(sum dE^2/N / sum N) in meV/atom, force component MAE / RMSE in meV/A,
    stress MAE / RMSE over the six components xx, yy, zz, yz, xz, xy in eV."""
    ea = es = fa = fs = sa = ss = 0.0
    en = fn = sn = 0
    for fr in frames:
        n = fr.natoms
        e, f, v, _, _ = model.efs(fr.cell, fr.positions, fr.types)
        if fr.energy is not None:
            d = fr.energy - e
            ea += abs(d)
            es += d * d / n
            en += n
        if fr.forces is not None:
            df = f - fr.forces
            fa += float(np.sum(np.abs(df)))
            fs += float(np.sum(df * df))
            fn += 3 * n
        if fr.stress is not None:
            ds = virial6_to_matrix(v) - fr.stress
            comps = [ds[0, 0], ds[1, 1], ds[2, 2], ds[1, 2], ds[0, 2], ds[0, 1]]
            sa += sum(abs(c) for c in comps)
            ss += sum(c * c for c in comps)
            sn += 6
    vals = (1000.0 * ea / en if en else 0.0, 1000.0 * np.sqrt(es / en) if en else 0.0,
            1000.0 * fa / fn if fn else 0.0, 1000.0 * np.sqrt(fs / fn) if fn else 0.0,
            sa / sn if sn else 0.0, np.sqrt(ss / sn) if sn else 0.0)
    return dict(zip(METRIC_NAMES, (float(x) for x in vals)))


def train_linear(model: "OracleModel", frames, wE: float, wF: float, wS: float, weighting: str = "vibrations",
                 norm_by_forces: int = 0) -> np.ndarray:
    """The linear warm-up solve, restating MTPR_trainer::TrainLinear (dev_src/mtpr_trainer.cpp:1455)
    for Static and Effect models: the radial Chebyshev rows are normalised to unit L2 norm
    (MLMTPR::Orthogonalize, dev_src/mtpr.cpp:14110), the normal equations of the energy / force /
    stress rows (AddToSLAE, mtpr_trainer.cpp:1130-1453) in the species constants and the scalar
    readout are built from one E/F/virial evaluation per readout column, a 1e-13 ridge is added and
    the system is solved by Gaussian elimination (SolveSLAE, :971; SolveSLAEGaussian, :282), and the
    solution is applied as centre factor 1, shift = constant - 1, readout = solution.  Returns the new
    parameter vector (the model keeps it)."""
    lay = model.layout()
    C, S, B, F = lay["C"], lay["S"], lay["B"], lay["F"]
    p = model.params()
    for mu in range(F):                       # Orthogonalize
        row = p[lay["o_radial"] + mu * (B + C): lay["o_radial"] + mu * (B + C) + B]
        norm = np.sqrt(np.sum(row * row + 1e-30))
        p[lay["o_radial"] + mu * (B + C): lay["o_radial"] + mu * (B + C) + B] = row / norm
    heads = C if lay["species_readout"] else 1
    ncol = C + heads * S
    d = 0.1
    # rows and weights per frame
    cols = []
    for q in range(heads * S):
        pq = p.copy()
        pq[lay["o_species"]: lay["o_species"] + C] = 1.0
        pq[lay["o_shift"]: lay["o_shift"] + C] = -1.0
        pq[lay["o_linear"]: lay["o_linear"] + heads * S] = 0.0
        pq[lay["o_linear"] + q] = 1.0
        model.set_params(pq)
        cols.append([model.efs(fr.cell, fr.positions, fr.types) for fr in frames])
    A = np.zeros((ncol, ncol))
    b = np.zeros(ncol)
    for k, fr in enumerate(frames):
        n = fr.natoms
        we, wf, ws = wE / n, wF, wS / n
        if weighting == "structures":
            we, ws, wf = we / n, ws / n, wf / n
        elif weighting == "molecules":
            we, ws = we * n, ws * n
        avef = float(np.mean(np.sum(fr.forces ** 2, axis=1))) if fr.forces is not None else 0.0
        scale = d / (d + norm_by_forces * avef)
        rows, rhs, alpha = [], [], []
        if fr.energy is not None:
            e_row = np.zeros(ncol)
            for t in range(C):
                e_row[t] = float(np.sum(fr.types == t))
            for q in range(heads * S):
                e_row[C + q] = cols[q][k][0]
            rows.append(e_row); rhs.append(fr.energy); alpha.append(we * scale)
        if wF > 0 and fr.forces is not None:
            for i in range(n):
                for a in range(3):
                    r = np.zeros(ncol)
                    for q in range(heads * S):
                        r[C + q] = cols[q][k][1][i, a]
                    rows.append(r); rhs.append(fr.forces[i, a]); alpha.append(wf * scale)
        if wS > 0 and fr.stress is not None:
            for a in range(3):
                for bb in range(3):
                    r = np.zeros(ncol)
                    for q in range(heads * S):
                        r[C + q] = virial6_to_matrix(cols[q][k][2])[a, bb]
                    rows.append(r); rhs.append(fr.stress[a, bb]); alpha.append(ws)
        for r, y, al in zip(rows, rhs, alpha):
            A += al * np.outer(r, r)
            b += al * y * r
    for i in range(ncol):
        A[i, i] += 1e-13 * (1.0 + A[i, i])
    # Gaussian elimination without pivoting, as SolveSLAEGaussian
    M, x = A.copy(), b.copy()
    for i in range(ncol - 1):
        for j in range(i + 1, ncol):
            ratio = M[j, i] / M[i, i]
            M[j, i:] -= ratio * M[i, i:]
            x[j] -= ratio * x[i]
    x[ncol - 1] /= M[ncol - 1, ncol - 1]
    for i in range(ncol - 2, -1, -1):
        x[i] = (x[i] - M[i, i + 1:] @ x[i + 1:]) / M[i, i]
    p[lay["o_species"]: lay["o_species"] + C] = 1.0
    p[lay["o_shift"]: lay["o_shift"] + C] = x[:C] - 1.0
    p[lay["o_linear"]: lay["o_linear"] + heads * S] = x[C:]
    model.set_params(p)
    return p


def rescale_subset(natoms):
    """Frames the rescale step solves on, restating BuildRescaleSubsetIndices
    (dev_src/mlp/mtpr_train.cpp:646-690): all frames when there are at most five, else the largest,
    second largest, median, second smallest and smallest by atom count (stable order), unique."""
    n = len(natoms)
    if n <= 5:
        return list(range(n))
    order = sorted(range(n), key=lambda f: (natoms[f], f))
    picks = []
    for f in (order[n - 1], order[n - 2], order[n // 2], order[1], order[0]):
        if f not in picks:
            picks.append(f)
    return picks


def moment_stats(params, o_linear: int, nread: int):
    """Median (upper) and RMS spread of log|c| over the scalar-readout coefficients |c| > 1e-12,
    restating ComputeMomentCoeffStats (dev_src/mlp/mtpr_train.cpp:279-307); None when empty."""
    logs = sorted(float(np.log(abs(c))) for c in params[o_linear:o_linear + nread] if abs(c) > 1e-12)
    if not logs:
        return None
    center = logs[len(logs) // 2]
    spread = float(np.sqrt(sum((v - center) ** 2 for v in logs) / len(logs)))
    return center, spread


def expansion_direction(seed, lower, upper):
    """First bracket-expansion direction (SelectRescaleExpansionDirection,
    dev_src/rescale_search.h:10-27): -1 / +1 for the probe that improves |median log| most, 0 when
    neither does; a probe is None when invalid."""
    best, d = abs(seed), 0
    if lower is not None and abs(lower) < best:
        best, d = abs(lower), -1
    if upper is not None and abs(upper) < best:
        d = 1
    return d


def rescale(model: "OracleModel", frames, wE: float, wF: float, wS: float, weighting: str = "vibrations",
            norm_by_forces: int = 0):
    """The rescale step around the linear warm-up, restating Rescale
    (dev_src/mlp/mtpr_train.cpp:1504-1748): returns (params, scaling, linear solves); the model keeps
    both.  Each trial sets the scaling and runs train_linear on the subset frames; the search
    brackets the median log coefficient at 0, refines it by secant steps in log scaling and ends
    with five fine trials judged by spread^2 + 3 median^2 (RescaleMetric, :309)."""
    lay = model.layout()
    heads = lay["C"] if lay["species_readout"] else 1
    nread, o_lin = heads * lay["S"], lay["o_linear"]
    sub = [frames[f] for f in rescale_subset([fr.natoms for fr in frames])]
    solves = [0]

    def evaluate(s):
        model.scaling = s
        p = train_linear(model, sub, wE, wF, wS, weighting, norm_by_forces)
        solves[0] += 1
        return {"scaling": s, "p": p, "st": moment_stats(p, o_lin, nread)}

    floor, factors = 1e-12, (1.0 / 1.08, 1.0 / 1.03, 1.0, 1.03, 1.08)
    center = evaluate(model.scaling)
    if center["st"] is None:
        return center["p"], center["scaling"], solves[0]
    state = {"best": center, "pos": None, "neg": None}

    def consider(e):
        if e is None or e["st"] is None:
            return
        c = e["st"][0]
        if abs(c) < abs(state["best"]["st"][0]):
            state["best"] = e
        if c >= 0.0:
            if state["pos"] is None or c < state["pos"]["st"][0]:
                state["pos"] = e
        elif state["neg"] is None or c > state["neg"]["st"][0]:
            state["neg"] = e

    def bracketed():
        return state["pos"] is not None and state["neg"] is not None

    consider(center)
    if abs(center["st"][0]) >= 0.15:
        lower = upper = None
        ls = max(floor, center["scaling"] / 2.0)
        if ls < center["scaling"]:
            lower = evaluate(ls)
            consider(lower)
        if not bracketed():
            us = center["scaling"] * 2.0
            if np.isfinite(us):
                upper = evaluate(us)
                consider(upper)
        if not bracketed():
            lc = lower["st"][0] if lower is not None and lower["st"] is not None else None
            uc = upper["st"][0] if upper is not None and upper["st"] is not None else None
            d = expansion_direction(center["st"][0], lc, uc)
            edge = lower if d < 0 else upper
            for _ in range(6):
                if d == 0 or bracketed():
                    break
                ts = max(floor, edge["scaling"] / 2.0) if d < 0 else edge["scaling"] * 2.0
                if not (ts > 0.0) or not np.isfinite(ts) or ts == edge["scaling"]:
                    break
                trial = evaluate(ts)
                if trial["st"] is None:
                    break
                prev = abs(edge["st"][0])
                consider(trial)
                edge = trial
                if not bracketed() and abs(trial["st"][0]) >= prev:
                    break
    if bracketed():
        for _ in range(6):
            pos, neg = state["pos"], state["neg"]
            lp, ln = np.log(pos["scaling"]), np.log(neg["scaling"])
            lt = 0.5 * (lp + ln)
            cp, cn = pos["st"][0], neg["st"][0]
            if abs(cp - cn) > 1e-12:
                lt = (lp * cn - ln * cp) / (cn - cp)
                lt = max(min(lt, max(lp, ln)), min(lp, ln))
                span = abs(lp - ln)
                if abs(lt - lp) < 0.1 * span or abs(lt - ln) < 0.1 * span:
                    lt = 0.5 * (lp + ln)
            trial = evaluate(max(floor, float(np.exp(lt))))
            if trial["st"] is None:
                break
            consider(trial)
            if abs(trial["st"][0]) < 0.15:
                state["best"] = trial
                break
    base = state["best"]["scaling"]
    best_metric, best_s, best_p = np.inf, base, state["best"]["p"]
    for f in factors:
        trial = evaluate(max(floor, base * f))
        if trial["st"] is None:
            continue
        c, sp = trial["st"]
        metric = sp * sp + 3.0 * c * c
        if metric < best_metric:
            best_metric, best_s, best_p = metric, trial["scaling"], trial["p"]
    model.scaling = best_s
    model.set_params(best_p)
    return best_p, best_s, solves[0]


# ------------------------------------------------------------------------------------------------
# BFGS with the reference's line search (src/common/bfgs.h:31-290 Linesearch, src/common/bfgs.cpp
# BFGS::Iterate :251-329, UpdateInvHess :428-502, FormDenseDirection :174).  The decision rules
# are kept exactly -- the trial sequence must match the reference's -- in this module's own code.
# ------------------------------------------------------------------------------------------------
HUGE = 9.9e99            # the reference's HUGE_DOUBLE (src/common/utils.h:24), initial right_f / f_start
RIGHT_F_SENTINEL = 9e99  # the value Linesearch::Iterate compares right_f with (bfgs.h:165); the
                         # reset value is HUGE, so that clause only fires if a trial returns 9e99
EPS = np.finfo(float).eps


class RefLineSearch:
    """One-dimensional search along the BFGS direction in reverse communication: iterate(f, g)
    takes the objective and its slope at x and sets the next trial x (Linesearch, bfgs.h:31-290).
    (lx, lf, lg) bracket the left end, (rx, rf, rg) the right end, (px, pf, pg) the previous
    trial."""

    def __init__(self):
        self.lf = self.lg = self.px = self.pf = self.pg = 0.0
        self.reset()

    def reset(self, step=1.0):
        self.stagnated = False
        self.x = self.lx = 0.0
        self.rx = step
        self.rf = self.rg = HUGE

    def reduce_step(self, ratio=0.25):
        self.x = self.px + ratio * (self.x - self.px)

    def _tolerance(self):
        return 64.0 * EPS * max(1.0, abs(self.lx), abs(self.x), abs(self.rx), abs(self.px))

    def _best(self, f):
        bx, bf = self.x, f
        if self.lf < bf:
            bx, bf = self.lx, self.lf
        if self.rf < bf:
            bx = self.rx
        return bx

    def _recover(self, f, g, tol):
        if not self.lx < self.rx:
            return False
        r = 0.5 * (self.lx + self.rx)
        if abs(r - self.x) <= tol:
            if self.x > self.lx:
                t = float(np.nextafter(self.x, self.lx))
                if t != self.x and t >= self.lx:
                    r = t
            if abs(r - self.x) <= tol and self.x < self.rx:
                t = float(np.nextafter(self.x, self.rx))
                if t != self.x and t <= self.rx:
                    r = t
        if abs(r - self.x) <= tol:
            return False
        self.px, self.pf, self.pg = self.x, f, g
        self.x = r
        return True

    def _to_prev(self, f, g):
        self.px, self.pf, self.pg = self.x, f, g

    def iterate(self, f, g):
        x = self.x
        if x == 0:
            self.lx, self.lf, self.lg = x, f, g
            if g > 0:
                raise RuntimeError("line search along an increasing direction")
            self._to_prev(f, g)
            self.x = self.rx
            return
        tol = self._tolerance()
        if abs(self.px - x) <= tol:
            if self._recover(f, g, tol):
                return
            if self.rx - self.lx <= tol:
                self.stagnated = True
                self.x = self._best(f)
                return
            raise RuntimeError("line search stagnated: unable to recover a distinct step")
        if x == self.rx or (x > self.lx and self.rf == RIGHT_F_SENTINEL):
            self.rx, self.rf, self.rg = x, f, g
        if self.rg < 0 and self.rf < self.lf:
            if x > self.rx:
                self.lx, self.lf, self.lg = self.rx, self.rf, self.rg
                self.rx, self.rf, self.rg = x, f, g
        else:
            if g < 0 and f < self.lf and x > self.lx:
                if x > self.rx:
                    if f > self.rf:
                        self._to_prev(f, g)
                        self.lx, self.lf, self.lg = self.rx, self.rf, self.rg
                        self.rx, self.rf, self.rg = x, f, g
                        self.x = 0.5 * (self.lx + self.rx)
                        return
                    self.rx, self.rf, self.rg = x, f, g
                else:
                    self.lx, self.lf, self.lg = x, f, g
            if g > 0 and x < self.rx:
                self.rx, self.rf, self.rg = x, f, g
        lx, lf, lg, rx, rg = self.lx, self.lf, self.lg, self.rx, self.rg
        if f > lf + 0.1 * lg * (x - lx):
            # insufficient decrease: the minimiser of a parabola fitted to log(f - f_lin)
            slope = -lg * (x - lx)
            nx = lx + 0.5 * (x - lx)
            arg = f - lf + slope
            if slope > 0.0 and arg > 0.0 and np.isfinite(slope) and np.isfinite(arg):
                f0, g0, f1 = np.log(slope), lg / slope, np.log(arg)
                den = f1 - f0 - g0 * (x - lx)
                if np.isfinite(den) and den != 0.0:
                    nx = lx - 0.5 * g0 * (x - lx) * (x - lx) / den
            if nx > rx and rg > 0:
                nx = lx + 0.5 * (x - lx)
            elif (nx - lx > 3.0 * rx - 2.0 * lx) and rg < 0:
                nx = lx + 3.0 * (rx - lx)
            if not np.isfinite(nx):
                nx = lx + 0.5 * (x - lx)
            self._to_prev(f, g)
            self.x = float(nx)
            return
        if (g - self.pg) / (x - self.px) < 0.0:
            # negative curvature along the line
            self._to_prev(f, g)
            self.x = 3 * rx - 2 * lx if rg < 0 else x + 0.5 * (rx - x)
            return
        # secant step on the slopes
        nx = x - g * (x - self.px) / (g - self.pg) if g != self.pg else float("nan")
        if not np.isfinite(nx):
            nx = lx + 0.5 * (rx - lx)
        self._to_prev(f, g)
        self.x = nx
        if nx > rx:
            if rg > 0:
                self.x = 0.5 * lx + 0.5 * rx
            elif nx > 3 * rx - 2 * lx:
                self.x = 3 * rx - 2 * lx
            return
        if nx < lx:
            self._to_prev(f, g)
            self.x = 0.5 * lx + 0.5 * rx


def bfgs_reference(fg, x0, iterations, inv_hess_diagonal=None, max_evals=400, c1=0.1, c2=0.5):
    """Minimise with BFGS as the reference's engine does (Set_x, optional SetInvHessDiagonal, then
    Iterate once per objective evaluation).  fg(x) -> (f, g).  Returns (trials, x_accepted): every
    evaluated point as (x, f, accepted), up to `iterations` accepted steps beyond the start, and
    the last accepted point."""
    x = np.array(x0, dtype=float)
    n = x.size
    H = np.diag(np.asarray(inv_hess_diagonal, float)) if inv_hess_diagonal is not None else np.eye(n)
    p = np.zeros(n)
    x_start, g_start = x.copy(), np.zeros(n)
    f_start, pg_start = HUGE, HUGE
    ls = RefLineSearch()
    trials, accepted = [], -1
    while accepted < iterations and len(trials) < max_evals:
        f, g = fg(x)
        xe = x.copy()
        if not np.isfinite(f) or not np.all(np.isfinite(g)):
            if ls.x == 0.0:
                raise RuntimeError("non-finite objective outside a line search")
            ls.reduce_step(0.25)
            x = x_start + ls.x * p
            trials.append((xe, f, False))
            continue
        pg = float(g @ p)
        if f > f_start + c1 * ls.x * pg_start or abs(pg) > c2 * abs(pg_start):
            ls.iterate(f, pg)
            if ls.stagnated:
                trials.append((xe, f, False))
                break
            x = x_start + ls.x * p
            trials.append((xe, f, False))
            continue
        # accepted: inverse-Hessian update with s = alpha p, y = g - g_start (skipped while
        # alpha p . y <= 64 eps), new direction p = -H g, a fresh line search from alpha = 1
        alpha = ls.x
        dg = g - g_start
        py = float(np.sum(alpha * p * dg))
        if not np.isfinite(py):
            raise RuntimeError("non-finite curvature")
        if py > 64.0 * EPS:
            yC = H @ dg
            foo = (py + float(yC @ dg)) / (py * py)
            if np.isfinite(foo):
                H += alpha * alpha * foo * np.outer(p, p) - (alpha / py) * (np.outer(p, yC) + np.outer(yC, p))
        p = -(H @ g)
        pg = float(g @ p)
        ls.reset()
        x_start, g_start, f_start, pg_start = x.copy(), g.copy(), f, pg
        if pg > 0:
            raise RuntimeError("BFGS: ascent direction")
        ls.iterate(f, pg)
        x = x_start + ls.x * p
        trials.append((xe, f, True))
        accepted += 1
    return trials, x_start
