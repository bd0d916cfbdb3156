"""GPU training objective, its gradient, BFGS and the torch autograd binding, through the C ABI.

Bars: FP64 plain within 1e-10 relative of the reference trainer's objective and gradient
(tests/golden/loss, NonLinearRegression::CalcObjectiveFunctionGrad summed over configurations, with
and without the Effect gate-x L2 term; the trainer reports both divided by the configuration count) and of the oracle's restatement on
weightings / options the goldens do not cover; FP32 bulk within 1e-5 relative (loss) and 1e-4
relative norm (gradient) of FP64.
"""
import glob
import os

import numpy as np
import pytest

from conftest import load_json
from superlinear_gb300.synth import read_cfg, training_frames

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-10


def rel_norm(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(np.linalg.norm(b), 1e-300))


@pytest.fixture(scope="module")
def sg(engine_lib):
    import superlinear_gb300
    return superlinear_gb300


def loss_cases():
    return sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "loss", "*.json")))


@pytest.mark.parametrize("path", loss_cases(), ids=os.path.basename)
def test_objective_matches_reference_trainer(sg, golden, path):
    data = load_json(path)
    model = sg.Model(os.path.join(golden, "models", data["model"]))
    frames = read_cfg(os.path.join(golden, "frames", data["frames"]))
    k = data["configs"]
    ref_loss, ref_grad = data["loss"] / k, np.asarray(data["grad"]) / k
    p = model.params()
    out = {}
    for prec in (sg.FP64, sg.FP32):
        eng = sg.Engine(model, 0, prec)
        tr = sg.Trainer(eng, frames, *data["weights"], weighting=data["weighting"], gate_x_l2=data["gate_x_l2"])
        out[prec] = tr.loss_grad(p)
        del tr
    loss, grad = out[sg.FP64]
    assert abs(loss - ref_loss) <= FP64_TOL * abs(ref_loss)
    metrics = sg.Trainer(sg.Engine(model, 0, sg.FP64), frames, *data["weights"]).metrics(p)
    for name, value in data["metrics"].items():
        assert abs(metrics[name] - value) <= FP64_TOL * abs(value), name
    assert rel_norm(grad, ref_grad) <= FP64_TOL
    loss32, grad32 = out[sg.FP32]
    assert abs(loss32 - loss) <= 1e-5 * abs(loss)
    assert rel_norm(grad32, grad) <= 1e-4


@pytest.mark.parametrize("weighting,nbf,gx", [("molecules", 0, 0.0), ("structures", 1, 0.0), ("vibrations", 1, 1e-4),
                                              ("molecules", 0, 3e-2)])
def test_objective_matches_oracle_other_weightings(sg, oracle_lib, golden, weighting, nbf, gx):
    """Weightings, force normalisation and gate-x coefficients the goldens do not exercise, on a
    ragged batch where some frames lack energy, force or stress labels."""
    path = os.path.join(golden, "models", "effect_l3k4r2o2.sus2")
    frames = read_cfg(os.path.join(golden, "frames", "effect_l3k4r2o2__labelled.cfg"))
    frames[1].energy = None
    frames[2].forces = None
    frames[3].stress = None
    om = oracle_lib.OracleModel(path)
    ref_loss, ref_grad = oracle_lib.loss_grad(om, frames, 1.0, 0.01, 0.001, weighting=weighting,
                                              norm_by_forces=nbf, gate_x_l2=gx)
    model = sg.Model(path)
    tr = sg.Trainer(sg.Engine(model, 0, sg.FP64), frames, 1.0, 0.01, 0.001, weighting=weighting, norm_by_forces=nbf,
                    gate_x_l2=gx)
    loss, grad = tr.loss_grad(model.params())
    assert abs(loss - ref_loss / len(frames)) <= FP64_TOL * abs(ref_loss / len(frames))
    assert rel_norm(grad, ref_grad / len(frames)) <= FP64_TOL


def test_graph_replay_equals_eager_and_tracks_parameters(sg, golden):
    model = sg.Model(os.path.join(golden, "models", "static_l2k3o2_c2.sus2"))
    frames = read_cfg(os.path.join(golden, "frames", "static_l2k3o2_c2__labelled.cfg"))
    p0 = model.params()
    p1 = p0 * (1.0 + 1e-3 * np.cos(np.arange(p0.size)))
    res = {}
    for graph in (False, True):
        tr = sg.Trainer(sg.Engine(model, 0, sg.FP64), frames)
        tr.set_graph(graph)
        # the replayed graph must read the parameter tables re-uploaded between evaluations
        res[graph] = [tr.loss_grad(p) for p in (p0, p1, p0, p1)]
    for (le, ge), (lg, gg) in zip(res[False], res[True]):
        assert le == lg and np.array_equal(ge, gg)
    assert res[True][0][0] == res[True][2][0] and res[True][0][0] != res[True][1][0]


def test_bfgs_decreases_loss(sg, golden):
    model = sg.Model(os.path.join(golden, "models", "static_l2k3o2_c2.sus2"))
    frames = read_cfg(os.path.join(golden, "frames", "static_l2k3o2_c2__labelled.cfg"))
    tr = sg.Trainer(sg.Engine(model, 0, sg.FP64), frames)
    p0 = model.params()
    p, hist = tr.bfgs(p0, max_iter=8)
    assert hist.size >= 3
    assert np.all(np.diff(hist) <= 0.0)
    assert hist[-1] < 0.9 * hist[0]
    loss, _ = tr.loss_grad(p)
    assert abs(loss - hist[-1]) <= 1e-12 * abs(hist[-1])


@pytest.mark.parametrize("name", ["static_l2k3o2_c2", "effect_l3k4r2o2"])
def test_bfgs_matches_reference_trials(sg, golden, name):
    """Device BFGS with the reference line search (the default) against the reference's BFGS engine
    (tests/golden/bfgs: BFGS::Iterate / Linesearch::Iterate / UpdateInvHess over the raw parameter
    vector on the trainer objective, constant initial inverse-Hessian diagonal): every trial point
    and loss, the accepted flags and the final parameters within 1e-8 relative (FP64)."""
    data = load_json(os.path.join(golden, "bfgs", f"{name}__labelled.json"))
    model = sg.Model(os.path.join(golden, "models", data["model"]))
    frames = read_cfg(os.path.join(golden, "frames", data["frames"]))
    tr = sg.Trainer(sg.Engine(model, 0, sg.FP64), frames, *data["weights"], weighting=data["weighting"],
                    gate_x_l2=0.0)
    p0 = np.asarray(data["trials"][0]["x"])
    assert np.array_equal(p0, model.params())
    tr.set_inv_hess_diagonal(np.full(p0.size, data["inv_hess_diagonal"]))
    p, hist = tr.bfgs(p0, max_iter=data["iterations"])
    f, x, acc = tr.bfgs_trials()
    ref = data["trials"]
    assert f.size == len(ref)
    for k, r in enumerate(ref):
        assert bool(acc[k]) == r["accepted"], k
        assert abs(f[k] - r["f"]) <= 1e-8 * abs(r["f"]), k
        rx = np.asarray(r["x"])
        assert np.max(np.abs(x[k] - rx)) <= 1e-8 * max(1.0, float(np.max(np.abs(rx)))), k
    last = np.asarray([r for r in ref if r["accepted"]][-1]["x"])
    assert np.max(np.abs(p - last)) <= 1e-8 * max(1.0, float(np.max(np.abs(last))))
    assert hist.size == data["iterations"] + 1
    assert np.allclose(hist, [r["f"] for r in ref if r["accepted"]], rtol=1e-8, atol=0)


def test_bfgs_interpolating_line_search_descends(sg, golden):
    """The optional interpolating line search: monotone descent, fewer evaluations per step."""
    model = sg.Model(os.path.join(golden, "models", "static_l2k3o2_c2.sus2"))
    frames = read_cfg(os.path.join(golden, "frames", "static_l2k3o2_c2__labelled.cfg"))
    tr = sg.Trainer(sg.Engine(model, 0, sg.FP64), frames)
    tr.set_line_search("interpolating")
    p, hist = tr.bfgs(model.params(), max_iter=8)
    assert hist.size >= 3 and np.all(np.diff(hist) <= 0.0) and hist[-1] < 0.9 * hist[0]
    loss, _ = tr.loss_grad(p)
    assert abs(loss - hist[-1]) <= 1e-12 * abs(hist[-1])


def test_bfgs_initial_inverse_hessian_diagonal(sg, golden):
    """A diagonal of ones is the default start (bit for bit); a scaled diagonal starts elsewhere
    and still descends; bad diagonals are rejected."""
    model = sg.Model(os.path.join(golden, "models", "static_l2k3o2_c2.sus2"))
    frames = read_cfg(os.path.join(golden, "frames", "static_l2k3o2_c2__labelled.cfg"))
    p0 = model.params()
    tr = sg.Trainer(sg.Engine(model, 0, sg.FP64), frames)
    p_ref, h_ref = tr.bfgs(p0, max_iter=5)
    tr.set_inv_hess_diagonal(np.ones(p0.size))
    p_one, h_one = tr.bfgs(p0, max_iter=5)
    assert np.array_equal(h_one, h_ref) and np.array_equal(p_one, p_ref)
    diag = np.full(p0.size, 0.25)
    diag[: p0.size // 2] = 2.0
    tr.set_inv_hess_diagonal(diag)
    p_d, h_d = tr.bfgs(p0, max_iter=5)
    assert h_d.size >= 3 and np.all(np.diff(h_d) <= 0.0) and h_d[-1] < h_d[0]
    assert not np.array_equal(p_d, p_ref)
    tr.set_inv_hess_diagonal(None)
    p_back, h_back = tr.bfgs(p0, max_iter=5)
    assert np.array_equal(h_back, h_ref)
    for bad in (np.ones(p0.size - 1), -np.ones(p0.size), np.full(p0.size, np.nan)):
        with pytest.raises(sg.Sus2Error):
            tr.set_inv_hess_diagonal(bad)


def test_trainer_rejects_invalid_inputs(sg, golden):
    model = sg.Model(os.path.join(golden, "models", "static_l2k3o2_c2.sus2"))
    frames = read_cfg(os.path.join(golden, "frames", "static_l2k3o2_c2__labelled.cfg"))
    eng = sg.Engine(model, 0, sg.FP64)
    with pytest.raises(ValueError):
        sg.Trainer(eng, frames, weighting="atoms")
    bad = read_cfg(os.path.join(golden, "frames", "static_l2k3o2_c2__labelled.cfg"))
    bad[0].types = bad[0].types.copy()
    bad[0].types[0] = 7
    with pytest.raises(sg.Sus2Error):
        sg.Trainer(eng, bad)
    tr = sg.Trainer(eng, frames)
    with pytest.raises(ValueError):
        tr.loss_grad(np.zeros(3))


def test_autograd_function_matches_finite_differences(sg, golden):
    torch = pytest.importorskip("torch")
    from superlinear_gb300.autograd import efs
    model = sg.Model(os.path.join(golden, "models", "effect_l3k4r2o2.sus2"))
    eng = sg.Engine(model, 0, sg.FP64)
    frames = training_frames(3, 8, 40, 3.0, 4.2, 0.1, seed=77, species=2)
    rng = np.random.default_rng(3)
    n = sum(f.natoms for f in frames)
    a = torch.tensor(rng.normal(size=len(frames)), dtype=torch.float64)
    b = torch.tensor(rng.normal(size=(n, 3)), dtype=torch.float64)
    c = torch.tensor(rng.normal(size=(len(frames), 6)), dtype=torch.float64)

    def objective(p):
        e, f, v = efs(p, eng, frames)
        return (a * e).sum() + (b * f).sum() + (c * v).sum()

    p0 = torch.tensor(model.params(), dtype=torch.float64, requires_grad=True)
    objective(p0).backward()
    g = p0.grad.numpy().copy()
    d = rng.normal(size=p0.numel())
    h = 1e-6
    with torch.no_grad():
        fp = objective(p0 + h * torch.from_numpy(d)).item()
        fm = objective(p0 - h * torch.from_numpy(d)).item()
    fd = (fp - fm) / (2 * h)
    assert abs(fd - g @ d) <= 1e-6 * max(1.0, abs(fd))


def test_autograd_device_tensors_match_host_frames(sg, golden):
    """efs_device: frames as CUDA tensors, every per-atom array kept on the device; the values and
    the parameter gradient of a scalar objective match the host-frame function (FP64)."""
    torch = pytest.importorskip("torch")
    from superlinear_gb300.autograd import efs, efs_device
    model = sg.Model(os.path.join(golden, "models", "effect_l3k4r2o2.sus2"))
    eng = sg.Engine(model, 0, sg.FP64)
    frames = training_frames(3, 8, 40, 3.0, 4.2, 0.1, seed=78, species=2)
    natoms = np.array([f.natoms for f in frames], dtype=np.int32)
    cells = np.stack([f.cell for f in frames])
    dev = torch.device("cuda", 0)
    pos = torch.tensor(np.concatenate([f.positions for f in frames]), dtype=torch.float64, device=dev)
    typ = torch.tensor(np.concatenate([f.types for f in frames]), dtype=torch.int32, device=dev)
    rng = np.random.default_rng(5)
    n = int(natoms.sum())
    a = rng.normal(size=len(frames))
    b = rng.normal(size=(n, 3))
    c = rng.normal(size=(len(frames), 6))

    p_host = torch.tensor(model.params(), dtype=torch.float64, requires_grad=True)
    e, f, v = efs(p_host, eng, frames)
    ((torch.from_numpy(a) * e).sum() + (torch.from_numpy(b) * f).sum() + (torch.from_numpy(c) * v).sum()).backward()

    p_dev = torch.tensor(model.params(), dtype=torch.float64, device=dev, requires_grad=True)
    ed, fd, vd = efs_device(p_dev, eng, natoms, cells, pos, typ)
    assert ed.is_cuda and fd.is_cuda and vd.is_cuda
    ta, tb, tc = (torch.from_numpy(x).to(dev) for x in (a, b, c))
    ((ta * ed).sum() + (tb * fd).sum() + (tc * vd).sum()).backward()
    assert p_dev.grad.is_cuda
    for x, y in ((e, ed), (f, fd), (v, vd)):
        assert np.allclose(x.detach().numpy(), y.detach().cpu().numpy(), rtol=1e-12, atol=1e-12)
    g_host, g_dev = p_host.grad.numpy(), p_dev.grad.cpu().numpy()
    assert np.linalg.norm(g_host - g_dev) <= 1e-12 * np.linalg.norm(g_host)
    with pytest.raises(ValueError):
        efs_device(p_dev, eng, natoms, cells, pos.cpu(), typ)


def test_trainer_survives_other_use_of_its_engine(sg, golden):
    """Evaluating other geometry on the trainer's engine rebuilds the trainer's edges (and graph)."""
    model = sg.Model(os.path.join(golden, "models", "static_l2k3o2_c2.sus2"))
    frames = read_cfg(os.path.join(golden, "frames", "static_l2k3o2_c2__labelled.cfg"))
    eng = sg.Engine(model, 0, sg.FP64)
    tr = sg.Trainer(eng, frames)
    p = model.params()
    first = tr.loss_grad(p)
    tr.loss_grad(p)  # graph replay
    eng.calc_efs(training_frames(3, 60, 200, 3.0, 4.2, 0.1, seed=5, species=2))
    again = tr.loss_grad(p)
    assert first[0] == again[0] and np.array_equal(first[1], again[1])


@pytest.mark.parametrize("path", sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "linear",
                                                            "*__labelled.json"))),
                         ids=os.path.basename)
def test_linear_warmup_matches_reference_trainer(sg, golden, path):
    """Trainer.train_linear (GPU components, device normal equations) against the reference's
    MTPR_trainer::TrainLinear; the FP32 bulk form lowers the objective likewise."""
    data = load_json(path)
    model = sg.Model(os.path.join(golden, "models", data["model"]))
    frames = read_cfg(os.path.join(golden, "frames", data["frames"]))
    p0 = model.params()
    tr = sg.Trainer(sg.Engine(model, 0, sg.FP64), frames, *data["weights"], weighting=data["weighting"], gate_x_l2=0.0)
    p = tr.train_linear(p0)
    # the normal equations are ill-conditioned (condition numbers 3.3e11 Static, 1.5e8 Effect):
    # last-bit differences of the FP64 components move the solution by ~1e-9 relative
    assert np.max(np.abs(p - np.asarray(data["coeffs"])) / (1.0 + np.abs(data["coeffs"]))) < 1e-8
    tr32 = sg.Trainer(sg.Engine(model, 0, sg.FP32), frames, *data["weights"], weighting=data["weighting"], gate_x_l2=0.0)
    before, _ = tr32.loss_grad(p0, want_grad=False)
    p32 = tr32.train_linear(p0)
    after, _ = tr32.loss_grad(p32, want_grad=False)
    assert after < before
    ref_after, _ = tr.loss_grad(p, want_grad=False)
    assert abs(after - ref_after) <= 1e-3 * abs(ref_after)


@pytest.mark.parametrize("path", sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "linear",
                                                            "*__rescale.json"))),
                         ids=os.path.basename)
def test_rescale_matches_reference_trainer(sg, golden, path):
    """Trainer.rescale (a linear warm-up on the GPU per trial) against the reference's Rescale: the
    chosen scaling and the final coefficients; the model saves the new scaling."""
    data = load_json(path)
    model = sg.Model(os.path.join(golden, "models", data["model"]))
    frames = read_cfg(os.path.join(golden, "frames", data["frames"]))
    tr = sg.Trainer(sg.Engine(model, 0, sg.FP64), frames, *data["weights"], weighting=data["weighting"], gate_x_l2=0.0)
    p, s, solves = tr.rescale(model.params())
    assert abs(s - data["scaling"]) <= 1e-8 * data["scaling"]
    assert np.max(np.abs(p - np.asarray(data["coeffs"])) / (1.0 + np.abs(data["coeffs"]))) < 1e-7
    assert solves >= 6
    # the trainer keeps evaluating with the new scaling; the model carries it into a saved file
    loss_after, _ = tr.loss_grad(p, want_grad=False)
    model.scaling = s
    model.set_params(p)
    fresh = sg.Trainer(sg.Engine(model, 0, sg.FP64), frames, *data["weights"], weighting=data["weighting"],
                       gate_x_l2=0.0)
    loss_fresh, _ = fresh.loss_grad(p, want_grad=False)
    assert abs(loss_fresh - loss_after) <= 1e-12 * abs(loss_after)


def test_trainer_after_autotune(sg, golden):
    """Tuning the engine's passes on the trainer's layout: the trainer captures its graph again;
    its objective and gradient are unchanged to the precision's rounding (the register budgets
    are separately compiled kernels) and repeat bit for bit."""
    path = os.path.join(golden, "models", "effect_l3k4r2o2.sus2")
    model = sg.Model(path)
    frames = read_cfg(os.path.join(golden, "frames", "effect_l3k4r2o2__labelled.cfg"))
    for prec in (sg.FP64, sg.FP32):
        eng = sg.Engine(model, 0, prec)
        tr = sg.Trainer(eng, frames)
        l0, g0 = tr.loss_grad(model.params())
        choice = eng.autotune(reps=2)
        assert set(choice) == {"gate_forward", "outer", "gate_reverse"}
        l1, g1 = tr.loss_grad(model.params())
        tol = 1e-12 if prec == sg.FP64 else 1e-6
        assert abs(l1 - l0) <= tol * abs(l0)
        assert np.max(np.abs(g1 - g0)) <= tol * (1.0 + np.max(np.abs(g0)))
        l2, g2 = tr.loss_grad(model.params())
        assert l2 == l1 and np.array_equal(g2, g1)


def test_trainer_every_centre_order(sg, golden):
    """The trainer's objective and gradient in each centre order of its passes (grid-strided,
    contiguous runs, taken from a device counter) match the default order bit for bit (one
    register budget: the default)."""
    path = os.path.join(golden, "models", "effect_l3k4r2o2.sus2")
    model = sg.Model(path)
    frames = read_cfg(os.path.join(golden, "frames", "effect_l3k4r2o2__labelled.cfg"))
    for prec in (sg.FP64, sg.FP32):
        eng = sg.Engine(model, 0, prec)
        tr = sg.Trainer(eng, frames)
        l0, g0 = tr.loss_grad(model.params())
        for p in ("gate_forward", "outer", "gate_reverse"):
            for order in ("contiguous", "dynamic"):
                eng.set_pass_shape(p, 0, "resident", order)
                for _ in range(2):
                    l1, g1 = tr.loss_grad(model.params())
                    assert l1 == l0 and np.array_equal(g1, g0), (prec, p, order)
            eng.set_pass_shape(p)
