"""Training objective over labelled frames resident on the GPU, its gradient, and BFGS.

Mirrors the reference trainer's objective / optimiser surface for this path:
  * ``Trainer.loss_grad(params)``  ~ NonLinearRegression::CalcObjectiveFunctionGrad
                                     (dev_src/non_linear_regression.cpp:1112) with the energy / force /
                                     stress terms of AddLoss / AddLossGrad (:768-1068), divided by the
                                     frame count as MTPR_trainer::Train does (dev_src/mtpr_trainer.cpp:4737-4745)
  * ``Trainer.bfgs(params, ...)``  ~ the dense BFGS loop of MTPR_trainer::Train over BFGS::Iterate
                                     (src/common/bfgs.cpp:251-329)
  * ``Trainer.train_linear(params)`` ~ MTPR_trainer::TrainLinear, the linear warm-up before BFGS
  * ``Trainer.rescale(params)``      ~ Rescale (dev_src/mlp/mtpr_train.cpp:1504), the scaling search
                                       around it
                                     (dev_src/mtpr_trainer.cpp:1455)
  * ``Trainer.metrics(params)``    ~ the trainer's energy / force / stress MAE and RMSE
``weighting`` takes the reference's names: "vibrations", "structures", "molecules".  ``gate_x_l2``
is the coefficient of the Effect gate-x L2 term of the reference objective (its default 1e-4,
dev_src/non_linear_regression.h:128; ignored for Static models).
"""
from __future__ import annotations

import ctypes

import numpy as np

from ._lib import check, load
from .engine import Engine

__all__ = ["Trainer", "WEIGHTINGS"]

WEIGHTINGS = {"vibrations": 0, "structures": 1, "molecules": 2}
_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)


def _d(a):
    return a.ctypes.data_as(_dp) if a is not None else None


class Trainer:
    """Labelled frames (``energy``, ``forces``, ``stress`` attributes, any may be None) bound to an engine."""

    def __init__(self, engine: Engine, frames, wE: float = 1.0, wF: float = 0.01, wS: float = 0.001,
                 weighting: str = "vibrations", norm_by_forces: int = 0, gate_x_l2: float = 1e-4):
        if weighting not in WEIGHTINGS:
            raise ValueError(f"weighting must be one of {sorted(WEIGHTINGS)}")
        self.engine = engine
        natoms, cells, pos, types = Engine.pack_frames(frames)
        nf, n = natoms.size, int(natoms.sum())
        energy = np.zeros(nf)
        forces = np.zeros((n, 3))
        stress = np.zeros((nf, 9))
        has = np.zeros(nf, dtype=np.int32)
        a = 0
        for k, fr in enumerate(frames):
            if fr.energy is not None:
                energy[k] = fr.energy
                has[k] |= 1
            if fr.forces is not None:
                forces[a:a + fr.natoms] = fr.forces
                has[k] |= 2
            if fr.stress is not None:
                stress[k] = np.asarray(fr.stress, dtype=np.float64).reshape(9)
                has[k] |= 4
            a += fr.natoms
        self.nframes = nf
        self.natoms = n
        h = ctypes.c_void_p()
        check(load().sus2g_trainer_create(engine._h, nf, natoms.ctypes.data_as(_ip), _d(cells), _d(pos),
                                          types.ctypes.data_as(_ip), _d(energy), _d(forces), _d(stress),
                                          has.ctypes.data_as(_ip), float(wE), float(wF), float(wS),
                                          WEIGHTINGS[weighting], int(norm_by_forces), float(gate_x_l2),
                                          ctypes.byref(h)))
        self._h = h

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            load().sus2g_trainer_free(h)
            self._h = None

    @property
    def nparams(self) -> int:
        return self.engine.model.nparams

    def set_graph(self, enabled: bool) -> None:
        check(load().sus2g_trainer_set_graph(self._h, 1 if enabled else 0))

    def loss_grad(self, params, want_grad: bool = True):
        """(loss, grad) at ``params`` (Coeff() order); grad is None when ``want_grad`` is False."""
        p = np.ascontiguousarray(params, dtype=np.float64)
        if p.size != self.nparams:
            raise ValueError(f"expected {self.nparams} parameters, got {p.size}")
        loss = ctypes.c_double()
        g = np.zeros(self.nparams) if want_grad else None
        check(load().sus2g_trainer_loss_grad(self._h, _d(p), ctypes.byref(loss), _d(g)))
        return loss.value, g

    METRICS = ("energy_mae_mev_per_atom", "energy_rmse_mev_per_atom", "force_mae_mev_per_a", "force_rmse_mev_per_a",
               "stress_mae_ev", "stress_rmse_ev")

    def metrics(self, params):
        """The reference trainer's error metrics over the labelled frames at ``params``."""
        p = np.ascontiguousarray(params, dtype=np.float64)
        if p.size != self.nparams:
            raise ValueError(f"expected {self.nparams} parameters, got {p.size}")
        out = np.zeros(6)
        check(load().sus2g_trainer_metrics(self._h, _d(p), _d(out)))
        return dict(zip(self.METRICS, (float(x) for x in out)))

    def train_linear(self, params) -> np.ndarray:
        """Linear warm-up (MTPR_trainer::TrainLinear): returns the parameters after the solve."""
        p = np.array(params, dtype=np.float64)
        if p.size != self.nparams:
            raise ValueError(f"expected {self.nparams} parameters, got {p.size}")
        check(load().sus2g_trainer_train_linear(self._h, _d(p)))
        return p

    def rescale(self, params):
        """Rescale step before the linear solve (the reference trainer's Rescale): returns
        (params, scaling, linear solves).  The trainer's engine keeps the new scaling; put it into a
        model to save with ``model.scaling = scaling``."""
        p = np.array(params, dtype=np.float64)
        if p.size != self.nparams:
            raise ValueError(f"expected {self.nparams} parameters, got {p.size}")
        s = ctypes.c_double()
        n = ctypes.c_int()
        check(load().sus2g_trainer_rescale(self._h, _d(p), ctypes.byref(s), ctypes.byref(n)))
        return p, s.value, n.value

    def set_inv_hess_diagonal(self, diag=None) -> None:
        """Initial inverse Hessian of later ``bfgs`` calls: ``diag`` (one finite positive entry per
        parameter) on the diagonal; ``None`` restores the identity (BFGS::SetInvHessDiagonal,
        src/common/bfgs.h:395)."""
        if diag is None:
            check(load().sus2g_trainer_set_inv_hess_diagonal(self._h, None, 0))
            return
        d = np.ascontiguousarray(diag, dtype=np.float64)
        check(load().sus2g_trainer_set_inv_hess_diagonal(self._h, _d(d), int(d.size)))

    LINE_SEARCHES = {"reference": 0, "interpolating": 1}

    def set_line_search(self, mode: str = "reference") -> None:
        """Line search of later ``bfgs`` calls: "reference" (default; the reference's Linesearch,
        src/common/bfgs.h:31-290) or "interpolating" (fewer evaluations, not the reference's
        trial sequence)."""
        check(load().sus2g_trainer_set_line_search(self._h, self.LINE_SEARCHES[mode]))

    def bfgs_trials(self):
        """Every objective evaluation of the last ``bfgs`` call: (losses[k], points[k, nparams],
        accepted[k])."""
        lib = load()
        n = ctypes.c_int()
        check(lib.sus2g_trainer_bfgs_trials(self._h, 0, None, None, None, ctypes.byref(n)))
        f = np.zeros(n.value)
        x = np.zeros((n.value, self.nparams))
        a = np.zeros(n.value, np.int32)
        check(lib.sus2g_trainer_bfgs_trials(self._h, n.value, _d(f), _d(x), a.ctypes.data_as(_ip), ctypes.byref(n)))
        return f, x, a.astype(bool)

    def bfgs(self, params, max_iter: int = 10, gtol: float = 0.0):
        """Runs BFGS from ``params``; returns (last accepted params, loss history)."""
        p = np.array(params, dtype=np.float64)
        hist = np.zeros(max_iter + 1)
        steps = ctypes.c_int()
        check(load().sus2g_trainer_bfgs(self._h, _d(p), int(max_iter), float(gtol), _d(hist), ctypes.byref(steps)))
        return p, hist[:steps.value + 1]
