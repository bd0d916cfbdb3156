"""torch ``autograd.Function`` over the engine: parameters -> (energy, forces, virial).

The backward pass is the engine's parameter gradient (AccumulateEFSCombinationGrad,
src/basic_mlip.cpp:421-476) with the upstream gradients as its weights:
  * energy: ene_w[i] = dL/dE[frame(i)] for every atom i of the frame;
  * forces: frc_w = dL/dF (sum_i frc_w_i . F_i = sum_edges (frc_w_i - frc_w_j) . dE/dd);
  * virial (xx, yy, zz, xy, xz, yz): str_w[b][a] = -dL/dW_ab for the six stored components
    (sum_edges (str_w d) . dE/dd = -sum_ab str_w[b][a] W_ab with W = -sum_edges d (x) dE/dd).
Gradients with respect to positions are not produced (the reference trainer has none either).
"""
from __future__ import annotations

import numpy as np
import torch

from .engine import Engine

__all__ = ["EFSFunction", "efs"]

_VIRIAL_INDEX = ((0, 0), (1, 1), (2, 2), (0, 1), (0, 2), (1, 2))


class EFSFunction(torch.autograd.Function):
    @staticmethod
    def forward(ctx, params: torch.Tensor, engine: Engine, frames):
        p = params.detach().to("cpu", torch.float64).contiguous().numpy()
        engine.model.set_params(p)
        engine.update_params()
        e, f, v, _ = engine.calc_efs(frames)
        ctx.engine = engine
        ctx.frames = frames
        ctx.params = p
        dev = params.device
        return (torch.from_numpy(e).to(dev), torch.from_numpy(f).to(dev), torch.from_numpy(v).to(dev))

    @staticmethod
    def backward(ctx, gE, gF, gV):
        frames = ctx.frames
        natoms = np.array([fr.natoms for fr in frames], dtype=np.int64)
        nf, n = natoms.size, int(natoms.sum())
        ge = gE.detach().to("cpu", torch.float64).numpy() if gE is not None else np.zeros(nf)
        gf = gF.detach().to("cpu", torch.float64).numpy() if gF is not None else np.zeros((n, 3))
        gv = gV.detach().to("cpu", torch.float64).numpy() if gV is not None else np.zeros((nf, 6))
        ene_w = np.repeat(ge, natoms)
        str_w = np.zeros((nf, 3, 3))
        for c, (a, b) in enumerate(_VIRIAL_INDEX):
            str_w[:, b, a] = -gv[:, c]
        engine = ctx.engine
        # the engine may have been re-parameterised since forward
        engine.model.set_params(ctx.params)
        engine.update_params()
        g = engine.combination_grad(frames, ene_w, gf, str_w)
        return torch.from_numpy(g).to(gE.device if gE is not None else "cpu"), None, None


def efs(params: torch.Tensor, engine: Engine, frames):
    """(energy[nframes], forces[N, 3], virial[nframes, 6]) as differentiable functions of ``params``."""
    return EFSFunction.apply(params, engine, frames)
