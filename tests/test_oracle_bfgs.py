"""The oracle's BFGS restatement (oracle.bfgs_reference) against the reference's BFGS engine: every
trial point and objective value of tests/golden/bfgs (ref-grad --bfgs over the raw parameter
vector on the trainer objective loss / K of a labelled set) within 1e-8 relative."""
import os

import numpy as np
import pytest

from conftest import load_json
from superlinear_gb300.synth import read_cfg

BFGS_TOL = 1e-8


@pytest.mark.parametrize("name", ["static_l2k3o2_c2", "effect_l3k4r2o2"])
def test_oracle_bfgs_matches_reference_trials(oracle_lib, golden, name):
    data = load_json(os.path.join(golden, "bfgs", f"{name}__labelled.json"))
    model = oracle_lib.OracleModel(os.path.join(golden, "models", data["model"]))
    frames = read_cfg(os.path.join(golden, "frames", data["frames"]))
    K = len(frames)

    def fg(x):
        model.set_params(x)
        loss, grad = oracle_lib.loss_grad(model, frames, *data["weights"], weighting=data["weighting"])
        return loss / K, grad / K

    x0 = np.asarray(data["trials"][0]["x"])
    trials, x_acc = oracle_lib.bfgs_reference(fg, x0, data["iterations"],
                                              inv_hess_diagonal=np.full(x0.size, data["inv_hess_diagonal"]))
    ref = data["trials"]
    assert len(trials) == len(ref)
    for (x, f, took), r in zip(trials, ref):
        assert took == r["accepted"]
        assert abs(f - r["f"]) <= BFGS_TOL * abs(r["f"])
        assert np.max(np.abs(x - np.asarray(r["x"]))) <= BFGS_TOL * max(1.0, float(np.max(np.abs(r["x"]))))
    last = [r for r in ref if r["accepted"]][-1]
    assert np.max(np.abs(x_acc - np.asarray(last["x"]))) <= BFGS_TOL * max(1.0, float(np.max(np.abs(last["x"]))))
