"""torch ``autograd.Function`` over the engine: parameters -> (energy, forces, virial).

The backward pass is the engine's parameter gradient (AccumulateEFSCombinationGrad,
src/basic_mlip.cpp:421-476) with the upstream gradients as its weights:
  * energy: ene_w[i] = dL/dE[frame(i)] for every atom i of the frame;
  * forces: frc_w = dL/dF (sum_i frc_w_i . F_i = sum_edges (frc_w_i - frc_w_j) . dE/dd);
  * virial (xx, yy, zz, xy, xz, yz): str_w[b][a] = -dL/dW_ab for the six stored components
    (sum_edges (str_w d) . dE/dd = -sum_ab str_w[b][a] W_ab with W = -sum_edges d (x) dE/dd).
Gradients with respect to positions are not produced (the reference trainer has none either).

``efs`` takes host frames; ``efs_device`` takes the frames as device tensors (positions [N, 3]
float64, types [N] int32 on the engine's GPU, natoms and cells on the host) and keeps every
per-atom array on the device: the evaluation and the gradient run on torch's current stream
through sus2g_calc_efs_device / sus2g_efs_combination_grad_device, with only the parameter vector
(model-sized) crossing to the host.
"""
from __future__ import annotations

import numpy as np
import torch

from .engine import Engine

__all__ = ["EFSFunction", "EFSDeviceFunction", "efs", "efs_device"]

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


def _on_torch_stream(engine: Engine, device: torch.device) -> None:
    """Runs the engine's next call on torch's current stream of ``device`` (the engine's own
    non-blocking stream, after torch's pending work, when that is the legacy default stream)."""
    s = torch.cuda.current_stream(device)
    if s.cuda_stream == 0:
        s.synchronize()
    engine.set_stream(s.cuda_stream)


class EFSDeviceFunction(torch.autograd.Function):
    @staticmethod
    def forward(ctx, params: torch.Tensor, engine: Engine, natoms, cells, positions: torch.Tensor,
                types: torch.Tensor):
        if not positions.is_cuda or not types.is_cuda:
            raise ValueError("efs_device: positions and types must be CUDA tensors")
        if positions.device.index != engine.device or types.device.index != engine.device:
            raise ValueError(f"efs_device: tensors must be on the engine's device cuda:{engine.device}")
        natoms = np.ascontiguousarray(natoms, dtype=np.int32).reshape(-1)
        cells = np.ascontiguousarray(cells, dtype=np.float64).reshape(-1, 3, 3)
        pos = positions.detach().to(torch.float64).contiguous()
        typ = types.detach().to(torch.int32).contiguous()
        n, nf = int(natoms.sum()), natoms.size
        if pos.shape != (n, 3) or typ.shape != (n,) or cells.shape[0] != nf:
            raise ValueError("efs_device: positions [N, 3], types [N], cells [nframes, 3, 3] with N = sum(natoms)")
        p = params.detach().to("cpu", torch.float64).contiguous().numpy()
        engine.model.set_params(p)
        engine.update_params()
        dev = pos.device
        e = torch.empty(nf, dtype=torch.float64, device=dev)
        f = torch.empty((n, 3), dtype=torch.float64, device=dev)
        v = torch.empty((nf, 6), dtype=torch.float64, device=dev)
        _on_torch_stream(engine, dev)
        engine.calc_efs_device(natoms, cells, pos.data_ptr(), typ.data_ptr(), e.data_ptr(), f.data_ptr(), v.data_ptr())
        ctx.engine, ctx.natoms, ctx.cells, ctx.params = engine, natoms, cells, p
        ctx.save_for_backward(pos, typ)
        ctx.param_device, ctx.param_dtype = params.device, params.dtype
        return e, f, v

    @staticmethod
    def backward(ctx, gE, gF, gV):
        pos, typ = ctx.saved_tensors
        natoms, cells, engine = ctx.natoms, ctx.cells, ctx.engine
        dev = pos.device
        n, nf = int(natoms.sum()), natoms.size
        counts = torch.as_tensor(natoms.astype(np.int64), device=dev)
        ene_w = (torch.repeat_interleave(gE.to(torch.float64), counts) if gE is not None
                 else torch.zeros(n, dtype=torch.float64, device=dev)).contiguous()
        frc_w = (gF.to(torch.float64) if gF is not None else torch.zeros((n, 3), dtype=torch.float64, device=dev))
        frc_w = frc_w.contiguous()
        str_w = torch.zeros((nf, 3, 3), dtype=torch.float64, device=dev)
        if gV is not None:
            for c, (a, b) in enumerate(_VIRIAL_INDEX):
                str_w[:, b, a] = -gV[:, c].to(torch.float64)
        grad = torch.zeros(engine.model.nparams, dtype=torch.float64, device=dev)
        # the engine may have been re-parameterised since forward
        engine.model.set_params(ctx.params)
        engine.update_params()
        _on_torch_stream(engine, dev)
        engine.combination_grad_device(natoms, cells, pos.data_ptr(), typ.data_ptr(), ene_w.data_ptr(),
                                       frc_w.data_ptr(), str_w.data_ptr(), grad.data_ptr())
        return grad.to(ctx.param_device, ctx.param_dtype), None, None, None, None, None


def efs_device(params: torch.Tensor, engine: Engine, natoms, cells, positions: torch.Tensor, types: torch.Tensor):
    """(energy[nframes], forces[N, 3], virial[nframes, 6]) on the positions' device, differentiable
    in ``params``; natoms [nframes] and cells [nframes, 3, 3] on the host."""
    return EFSDeviceFunction.apply(params, engine, natoms, cells, positions, types)
