"""The CPU oracle is pinned against the reference's own outputs (CPU only).

* two-cutoff FP64 fixtures shipped with the reference (independent PyTorch float64 values),
* the reference embedded engine on the benchmark model families (tests/golden/efs),
* the reference trainer's AccumulateEFSCombinationGrad parameter gradients (tests/golden/grad).
"""
import glob
import os

import numpy as np
import pytest

from conftest import load_json, rel_err, two_cutoff_cases, virial6_to_matrix
from superlinear_gb300.synth import read_cfg


@pytest.mark.parametrize("model,geom,ref", two_cutoff_cases(), ids=lambda p: os.path.basename(p))
def test_two_cutoff_fixtures(oracle_lib, model, geom, ref):
    m = oracle_lib.OracleModel(model)
    frames = read_cfg(geom)
    data = load_json(ref)
    for rec in data["records"]:
        fr = frames[rec["config"]]
        e, f, v, s, _ = m.efs(fr.cell, fr.positions, fr.types)
        assert rel_err(e, rec["energy"]) < 1e-12
        assert rel_err(f, rec["forces"]) < 1e-12
        assert rel_err(virial6_to_matrix(v), rec["plus_stress"]) < 1e-12


def efs_cases():
    return sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "efs", "*.json")))


@pytest.mark.parametrize("path", efs_cases(), ids=os.path.basename)
def test_embedded_engine_goldens(oracle_lib, golden, path):
    data = load_json(path)
    m = oracle_lib.OracleModel(os.path.join(golden, "models", data["model"]))
    frames = read_cfg(os.path.join(golden, "frames", data["frames"]))
    for rec in data["records"]:
        fr = frames[rec["config"]]
        e, f, v, s, _ = m.efs(fr.cell, fr.positions, fr.types)
        assert rel_err(e, rec["energy"]) < 1e-12
        assert rel_err(f, rec["forces"]) < 1e-12
        assert rel_err(virial6_to_matrix(v), rec["virial"]) < 1e-12
        assert rel_err(s, rec["site_energies"]) < 1e-12


def grad_cases():
    return sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "grad", "*.json")))


@pytest.mark.parametrize("path", grad_cases(), ids=os.path.basename)
def test_trainer_gradient_goldens(oracle_lib, golden, path):
    data = load_json(path)
    m = oracle_lib.OracleModel(os.path.join(golden, "models", data["model"]))
    frames = read_cfg(os.path.join(golden, "frames", data["frames"]))
    for fr, w, ref, tr in zip(frames, data["weights"], data["grad"], data["trainer_efs"]):
        g = m.grad(fr.cell, fr.positions, fr.types, w["energy"], w["force"], w["stress"])
        ref = np.asarray(ref)
        assert np.linalg.norm(g - ref) <= 1e-12 * np.linalg.norm(ref)
        e, f, v, s, _ = m.efs(fr.cell, fr.positions, fr.types)
        assert rel_err(e, tr["energy"]) < 1e-12 and rel_err(f, tr["forces"]) < 1e-12


def test_oracle_rejects_missing_model(oracle_lib, tmp_path):
    with pytest.raises(ValueError):
        oracle_lib.OracleModel(str(tmp_path / "missing.sus2"))


def test_oracle_planted_error_is_detected(oracle_lib, golden):
    """A mistake planted in the oracle's inputs (one coefficient) moves the result off the golden."""
    data = load_json(os.path.join(golden, "efs", "static_l3k4o2__diamond64_s05.json"))
    m = oracle_lib.OracleModel(os.path.join(golden, "models", data["model"]))
    p = m.params()
    p[20] += 1e-3
    m.set_params(p)
    fr = read_cfg(os.path.join(golden, "frames", data["frames"]))[0]
    e, f, *_ = m.efs(fr.cell, fr.positions, fr.types)
    assert rel_err(f, data["records"][0]["forces"]) > 1e-9


def loss_cases():
    return sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "loss", "*.json")))


@pytest.mark.parametrize("path", loss_cases(), ids=os.path.basename)
def test_training_objective_goldens(oracle_lib, golden, path):
    """Energy / force / stress objective (and, in the __gatex files, the Effect gate-x L2 term at the
    reference's default coefficient) and its gradient against the reference trainer's
    NonLinearRegression::CalcObjectiveFunctionGrad (summed over configurations)."""
    data = load_json(path)
    m = oracle_lib.OracleModel(os.path.join(golden, "models", data["model"]))
    frames = read_cfg(os.path.join(golden, "frames", data["frames"]))
    assert len(frames) == data["configs"]
    loss, grad = oracle_lib.loss_grad(m, frames, *data["weights"], weighting=data["weighting"],
                                      gate_x_l2=data.get("gate_x_l2", 0.0))
    ref = np.asarray(data["grad"])
    assert abs(loss - data["loss"]) <= 1e-12 * abs(data["loss"])
    assert np.linalg.norm(grad - ref) <= 1e-12 * np.linalg.norm(ref)
    metrics = oracle_lib.error_metrics(m, frames)
    for name, value in data["metrics"].items():
        assert abs(metrics[name] - value) <= 1e-11 * max(abs(value), 1e-300), name


def desc_cases():
    return sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "desc", "*.json")))


@pytest.mark.parametrize("path", desc_cases(), ids=os.path.basename)
def test_descriptor_goldens(oracle_lib, golden, path):
    """Per-atom scalar moments against the reference trainer's calc-descriptors (printed with 16
    significant digits)."""
    data = load_json(path)
    m = oracle_lib.OracleModel(os.path.join(golden, "models", data["model"]))
    frames = read_cfg(os.path.join(golden, "frames", data["frames"]))
    ref = np.asarray(data["descriptors"])
    ours = np.concatenate([m.descriptors(fr.cell, fr.positions, fr.types, ref.shape[1]) for fr in frames])
    assert np.array_equal(np.concatenate([fr.types for fr in frames]), data["types"])
    assert rel_err(ours, ref) < 1e-13


def linear_cases():
    return sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "linear", "*__labelled.json")))


def rescale_cases():
    return sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "linear", "*__rescale.json")))


@pytest.mark.parametrize("path", linear_cases(), ids=os.path.basename)
def test_linear_warmup_goldens(oracle_lib, golden, path):
    """The linear warm-up solve against the reference's MTPR_trainer::TrainLinear."""
    data = load_json(path)
    m = oracle_lib.OracleModel(os.path.join(golden, "models", data["model"]))
    frames = read_cfg(os.path.join(golden, "frames", data["frames"]))
    p = oracle_lib.train_linear(m, frames, *data["weights"], weighting=data["weighting"])
    assert rel_err(p, data["coeffs"]) < 1e-9


@pytest.mark.parametrize("path", rescale_cases(), ids=os.path.basename)
def test_rescale_goldens(oracle_lib, golden, path):
    """The rescale step (scaling search around the linear warm-up) against the reference's Rescale:
    the chosen scaling and the final coefficients (the Effect set's six frames exercise the
    five-frame subset)."""
    data = load_json(path)
    m = oracle_lib.OracleModel(os.path.join(golden, "models", data["model"]))
    frames = read_cfg(os.path.join(golden, "frames", data["frames"]))
    p, s, solves = oracle_lib.rescale(m, frames, *data["weights"], weighting=data["weighting"])
    assert abs(s - data["scaling"]) <= 1e-9 * data["scaling"]
    assert rel_err(p, data["coeffs"]) < 1e-8
    assert solves >= 6 and m.scaling == s


def test_rescale_helpers_known_answers(oracle_lib):
    """Expansion-direction and subset selection known answers: the former from the reference's own
    self-test (dev_src/mlp/dev_self_test.cpp:3033-3053), the latter by its definition."""
    d = oracle_lib.expansion_direction
    assert d(-5.26730719706032, -8.27303159671854, -2.25) == 1
    assert d(5.0, 2.0, 8.0) == -1
    assert d(-1.0, -2.0, -3.0) == 0
    assert d(-4.0, None, -1.0) == 1
    assert oracle_lib.rescale_subset([10, 20, 30]) == [0, 1, 2]
    # sizes 5 3 9 3 7 1 -> stable order 5(1) 1(3) 3(3) 0(5) 4(7) 2(9): max 2, second max 4,
    # median order[3] = 0, second min 1, min 5
    assert oracle_lib.rescale_subset([5, 3, 9, 3, 7, 1]) == [2, 4, 0, 1, 5]
    st = oracle_lib.moment_stats(np.array([0.0, np.e, 1.0, 1e-13, -np.e ** 2]), 1, 4)
    assert st is not None and abs(st[0] - 1.0) < 1e-15
