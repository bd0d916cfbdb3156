"""GPU parameter gradient (AccumulateEFSCombinationGrad contract) through the C ABI.

Bars: FP64 plain within 1e-10 relative norm of the reference trainer's analytic gradient
(tests/golden/grad) and of the oracle on uneven batches; FP32 bulk within 1e-4 relative norm of
FP64 (the gradient error stated for the bulk form).
"""
import glob
import os

import numpy as np
import pytest

from conftest import load_json
from superlinear_gb300.synth import read_cfg, training_frames, diamond

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-10
FP32_TOL = 1e-4


def rel_norm(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(np.linalg.norm(b), 1e-300))


@pytest.fixture(scope="module")
def sg(engine_lib):
    import superlinear_gb300
    return superlinear_gb300


@pytest.mark.parametrize("path", sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "grad", "*.json"))),
                         ids=os.path.basename)
def test_gradient_matches_reference_trainer(sg, golden, path):
    data = load_json(path)
    model = sg.Model(os.path.join(golden, "models", data["model"]))
    frames = read_cfg(os.path.join(golden, "frames", data["frames"]))
    g64 = sg.Engine(model, 0, sg.FP64)
    g32 = sg.Engine(model, 0, sg.FP32)
    total = np.zeros(model.nparams)
    for fr, w, ref in zip(frames, data["weights"], data["grad"]):
        g = g64.combination_grad([fr], w["energy"], w["force"], [w["stress"]])
        assert rel_norm(g, ref) <= FP64_TOL
        gf = g32.combination_grad([fr], w["energy"], w["force"], [w["stress"]])
        assert rel_norm(gf, ref) <= FP32_TOL
        total += np.asarray(ref)
    # the whole batch at once accumulates the per-frame gradients
    ew = np.concatenate([w["energy"] for w in data["weights"]])
    fw = np.concatenate([np.asarray(w["force"]) for w in data["weights"]])
    sw = np.stack([np.asarray(w["stress"]) for w in data["weights"]])
    g = g64.combination_grad(frames, ew, fw, sw)
    assert rel_norm(g, total) <= FP64_TOL


def test_gradient_uneven_batch_matches_oracle(sg, oracle_lib, golden):
    path = os.path.join(golden, "models", "effect_l3k4r2o2.sus2")
    model = sg.Model(path)
    om = oracle_lib.OracleModel(path)
    frames = training_frames(10, 8, 120, 3.0, 4.2, 0.1, seed=91)
    rng = np.random.default_rng(5)
    ew = [np.full(fr.natoms, rng.uniform(0.5, 1.5)) for fr in frames]
    fw = [rng.normal(0, 1, (fr.natoms, 3)) for fr in frames]
    sw = [rng.normal(0, 0.2, (3, 3)) for _ in frames]
    ref = np.zeros(model.nparams)
    for fr, a, b, c in zip(frames, ew, fw, sw):
        ref += om.grad(fr.cell, fr.positions, fr.types, a, b, c)
    g = sg.Engine(model, 0, sg.FP64).combination_grad(frames, np.concatenate(ew), np.concatenate(fw), np.stack(sw))
    assert rel_norm(g, ref) <= FP64_TOL
    gf = sg.Engine(model, 0, sg.FP32).combination_grad(frames, np.concatenate(ew), np.concatenate(fw), np.stack(sw))
    assert rel_norm(gf, ref) <= FP32_TOL


def test_gradient_static_cell_list_box(sg, oracle_lib, golden):
    """4,096-atom box (cell-list edges) for the Static model, energy and force weights."""
    path = os.path.join(golden, "models", "static_l3k4o2.sus2")
    model = sg.Model(path)
    om = oracle_lib.OracleModel(path)
    fr = diamond(8, sigma=0.08, seed=3)
    rng = np.random.default_rng(6)
    ew = np.full(fr.natoms, 0.7)
    fw = rng.normal(0, 0.1, (fr.natoms, 3))
    sw = rng.normal(0, 0.01, (3, 3))
    ref = om.grad(fr.cell, fr.positions, fr.types, ew, fw, sw)
    g = sg.Engine(model, 0, sg.FP64).combination_grad([fr], ew, fw, [sw])
    assert rel_norm(g, ref) <= FP64_TOL


def test_gradient_accumulates_and_is_deterministic(sg, golden):
    model = sg.Model(os.path.join(golden, "models", "effect_l3k4r2o2.sus2"))
    frames = training_frames(4, 8, 64, 3.0, 4.2, 0.1, seed=17)
    n = sum(f.natoms for f in frames)
    ew, fw, sw = np.ones(n), np.full((n, 3), 0.3), np.tile(np.eye(3) * 0.1, (4, 1, 1))
    for prec in (sg.FP64, sg.FP32):
        eng = sg.Engine(model, 0, prec)
        a = eng.combination_grad(frames, ew, fw, sw)
        b = eng.combination_grad(frames, ew, fw, sw)
        assert np.array_equal(a, b)
        c = eng.combination_grad(frames, ew, fw, sw, grad=a.copy())
        assert np.allclose(c, 2 * a, rtol=1e-14, atol=0)
