"""Config 5 topology (Effect L5/K8/R2/O2, three species) on the GPU.

The reference's model loader rejects sh_l_max > 4, so this topology has no reference values; the
L5 kernels are checked against the oracle (itself checked against finite differences in
tests/test_oracle_config5.py) on frames of the configuration's shapes: uneven sizes drawn
log-uniformly in [16, 512], random fcc/bcc/diamond lattices a in [2.8, 4.5] A, sigma = 0.15 A,
uniform species.  Bars as elsewhere: FP64 plain within 1e-10 relative, FP32 bulk within 1e-5 eV/A
(forces) and 1e-6 eV/atom (energy) of FP64, parameter gradients within 1e-10 (FP64) and 1e-4
(FP32) relative norm; BFGS with the loss + gradient graph lowers the objective in both forms.
"""
import os

import numpy as np
import pytest

from conftest import rel_err
from superlinear_gb300.synth import training_frames

pytestmark = pytest.mark.gpu

MODEL = "effect_l5k8r2o2_c3.sus2"
FP64_TOL = 1e-10


@pytest.fixture(scope="module")
def sg(engine_lib):
    import superlinear_gb300
    return superlinear_gb300


def rel_norm(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def frames_c5(count, seed, nmax=512):
    return training_frames(count, 16, nmax, 2.8, 4.5, 0.15, seed=seed, species=3, log_uniform=True)


def test_config5_efs_matches_oracle(sg, oracle_lib, golden):
    path = os.path.join(golden, "models", MODEL)
    model = sg.Model(path)
    om = oracle_lib.OracleModel(path)
    frames = frames_c5(5, seed=511)
    g64, g32 = sg.Engine(model, 0, sg.FP64), sg.Engine(model, 0, sg.FP32)
    e, f, v, s = g64.calc_efs(frames)
    e32, f32, v32, s32 = g32.calc_efs(frames)
    off = 0
    for k, fr in enumerate(frames):
        sl = slice(off, off + fr.natoms)
        eo, fo, vo, so, ne = om.efs(fr.cell, fr.positions, fr.types, threads=0)
        assert rel_err(e[k], eo) < FP64_TOL and rel_err(f[sl], fo) < FP64_TOL
        assert rel_err(v[k], vo) < FP64_TOL and rel_err(s[sl], so) < FP64_TOL
        assert np.max(np.abs(f32[sl] - f[sl])) <= 1e-5
        assert abs(e32[k] - e[k]) / fr.natoms <= 1e-6
        off += fr.natoms


def test_config5_parameter_gradient_matches_oracle(sg, oracle_lib, golden):
    path = os.path.join(golden, "models", MODEL)
    model = sg.Model(path)
    om = oracle_lib.OracleModel(path)
    frames = frames_c5(3, seed=512, nmax=128)
    rng = np.random.default_rng(6)
    ew = [np.full(fr.natoms, rng.uniform(0.5, 1.5)) for fr in frames]
    fw = [rng.normal(0, 1, (fr.natoms, 3)) for fr in frames]
    sw = [rng.normal(0, 0.2, (3, 3)) for _ in frames]
    ref = np.zeros(model.nparams)
    for fr, a, b, c in zip(frames, ew, fw, sw):
        ref += om.grad(fr.cell, fr.positions, fr.types, a, b, c)
    g64 = sg.Engine(model, 0, sg.FP64).combination_grad(frames, np.concatenate(ew), np.concatenate(fw), np.stack(sw))
    g32 = sg.Engine(model, 0, sg.FP32).combination_grad(frames, np.concatenate(ew), np.concatenate(fw), np.stack(sw))
    assert rel_norm(g64, ref) <= FP64_TOL
    assert rel_norm(g32, ref) <= 1e-4


def test_config5_training_objective_and_bfgs(sg, oracle_lib, golden):
    """Teacher labels from the oracle at perturbed parameters; the objective (energy + force +
    stress MSE, the example profile's weights) against the oracle's, then a few BFGS iterations in
    FP64 and FP32."""
    path = os.path.join(golden, "models", MODEL)
    model = sg.Model(path)
    om = oracle_lib.OracleModel(path)
    p0 = model.params()
    frames = frames_c5(8, seed=513, nmax=96)
    teacher = p0 * (1 + 0.02 * np.random.default_rng(7).normal(size=p0.size))
    om.set_params(teacher)
    for fr in frames:
        e, f, v, s, ne = om.efs(fr.cell, fr.positions, fr.types)
        fr.energy, fr.forces = e, f
        fr.stress = np.array([[v[0], v[3], v[4]], [v[3], v[1], v[5]], [v[4], v[5], v[2]]])
    om.set_params(p0)
    ref_loss, ref_grad = oracle_lib.loss_grad(om, frames, 1.0, 0.01, 0.001, gate_x_l2=1e-4)
    tr64 = sg.Trainer(sg.Engine(model, 0, sg.FP64), frames, 1.0, 0.01, 0.001, gate_x_l2=1e-4)
    loss, grad = tr64.loss_grad(p0)
    assert abs(loss - ref_loss / len(frames)) <= FP64_TOL * abs(ref_loss / len(frames))
    assert rel_norm(grad, ref_grad / len(frames)) <= FP64_TOL
    tr32 = sg.Trainer(sg.Engine(model, 0, sg.FP32), frames, 1.0, 0.01, 0.001, gate_x_l2=1e-4)
    loss32, grad32 = tr32.loss_grad(p0)
    assert abs(loss32 - loss) <= 1e-5 * abs(loss) and rel_norm(grad32, grad) <= 1e-3
    for tr in (tr64, tr32):
        p, hist = tr.bfgs(p0, max_iter=4)
        assert hist.size >= 3 and np.all(np.diff(hist) <= 0.0) and hist[-1] < hist[0]
