"""Step graph of the periodic E / F / virial entry points: repeated steps of one layout (an MD
run's positions moving in fixed buffers) replay one captured CUDA graph of the edge build and the
evaluation.  Bars: bitwise identical to the eager steps of a second engine; FP64 within 1e-10
relative of the oracle after the positions moved; correct after a parameter update, a layout
change and a neighbour-capacity overflow found during a replay.
"""
import os

import numpy as np
import pytest

from conftest import rel_err
from superlinear_gb300.synth import Frame, diamond

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-10


@pytest.fixture(scope="module")
def sg(engine_lib):
    import superlinear_gb300
    return superlinear_gb300


class DeviceFrames:
    """Positions / types / outputs of a batch in fixed device buffers (the MD layout)."""

    def __init__(self, frames):
        import torch
        dev = torch.device("cuda", 0)
        self.natoms = np.array([f.natoms for f in frames], np.int32)
        self.cells = np.stack([f.cell for f in frames]).reshape(-1, 9).copy()
        self.pos = torch.tensor(np.concatenate([f.positions for f in frames]), device=dev)
        self.types = torch.tensor(np.concatenate([f.types for f in frames]).astype(np.int32), device=dev)
        n, nf = int(self.natoms.sum()), len(frames)
        self.E = torch.zeros(nf, dtype=torch.float64, device=dev)
        self.F = torch.zeros(n, 3, dtype=torch.float64, device=dev)
        self.V = torch.zeros(nf, 6, dtype=torch.float64, device=dev)
        self.S = torch.zeros(n, dtype=torch.float64, device=dev)

    def step(self, eng):
        import torch
        eng.calc_efs_device(self.natoms, self.cells, self.pos.data_ptr(), self.types.data_ptr(), self.E.data_ptr(),
                            self.F.data_ptr(), self.V.data_ptr(), self.S.data_ptr())
        torch.cuda.synchronize()
        return tuple(x.cpu().numpy().copy() for x in (self.E, self.F, self.V, self.S))


def batch(species):
    return [diamond(6, sigma=0.05, seed=s, species=species) for s in (3, 4)]


@pytest.mark.parametrize("name", ["static_l3k4o2", "effect_l3k4r2o2"])
@pytest.mark.parametrize("precision", ["FP64", "FP32"])
def test_md_steps_replay_bitwise(sg, golden, oracle_lib, name, precision):
    path = os.path.join(golden, "models", f"{name}.sus2")
    m = sg.Model(path)
    prec = getattr(sg, precision)
    graph, eager = sg.Engine(m, 0, prec), sg.Engine(m, 0, prec)
    eager.set_step_graph(False)
    frames = batch(m.dims["C"])
    a, b = DeviceFrames(frames), DeviceFrames(frames)
    rng = np.random.default_rng(5)
    launches = []
    for step in range(5):
        ra, rb = a.step(graph), b.step(eager)
        for x, y in zip(ra, rb):
            assert np.array_equal(x, y), f"step {step}"
        assert graph.edge_count() == eager.edge_count()
        launches.append((graph.take_launch_count(), eager.take_launch_count()))
        d = rng.normal(0, 0.02, tuple(a.pos.shape))
        import torch
        a.pos += torch.tensor(d, device=a.pos.device)
        b.pos += torch.tensor(d, device=b.pos.device)
    # every step reports the kernels it ran, replayed or not
    assert all(x == y and x > 0 for x, y in launches)
    if precision == "FP64":
        om = oracle_lib.OracleModel(path)
        pos = a.pos.cpu().numpy()
        ra = a.step(graph)
        off = 0
        for k, fr in enumerate(frames):
            sl = slice(off, off + fr.natoms)
            eo, fo, vo, so, ne = om.efs(fr.cell, pos[sl], fr.types, threads=0)
            assert rel_err(ra[0][k], eo) < FP64_TOL and rel_err(ra[1][sl], fo) < FP64_TOL
            assert rel_err(ra[2][k], vo) < FP64_TOL and rel_err(ra[3][sl], so) < FP64_TOL
            off += fr.natoms


def test_param_update_and_layout_change(sg, golden):
    path = os.path.join(golden, "models", "effect_l3k4r2o2.sus2")
    m = sg.Model(path)
    graph, eager = sg.Engine(m, 0, sg.FP64), sg.Engine(m, 0, sg.FP64)
    eager.set_step_graph(False)
    frames = batch(2)
    a, b = DeviceFrames(frames), DeviceFrames(frames)
    for _ in range(3):
        a.step(graph), b.step(eager)
    p0 = m.params()
    m.set_params(p0 * (1 + 1e-3 * np.sin(np.arange(p0.size))))
    graph.update_params(), eager.update_params()
    for _ in range(3):
        for x, y in zip(a.step(graph), b.step(eager)):
            assert np.array_equal(x, y)
    # another batch on the same engine, then back to the first one
    c, d = DeviceFrames(frames[:1]), DeviceFrames(frames[:1])
    for x, y in zip(c.step(graph), d.step(eager)):
        assert np.array_equal(x, y)
    for _ in range(3):
        for x, y in zip(a.step(graph), b.step(eager)):
            assert np.array_equal(x, y)
    # the host entry point shares the engine
    h = graph.calc_efs(frames)
    for x, y in zip(h, eager.calc_efs(frames)):
        assert np.array_equal(x, y)
    m.set_params(p0)


def test_overflow_during_replay_is_retried(sg, golden, oracle_lib):
    """Captured on a uniform box, then the atoms gather into a dense cluster in the same buffers:
    the replay overflows the padded neighbour capacity, the call repeats the step eagerly with a
    grown capacity and matches the oracle."""
    import torch
    path = os.path.join(golden, "models", "static_l3k4o2.sus2")
    m = sg.Model(path)
    eng = sg.Engine(m, 0, sg.FP64)
    om = oracle_lib.OracleModel(path)
    rng = np.random.default_rng(9)
    grid = np.stack(np.meshgrid(*[np.arange(9)] * 3, indexing="ij"), -1).reshape(-1, 3)
    spread = Frame(np.eye(3) * 30.0, grid * 3.3 + 0.5 + rng.normal(0, 0.05, grid.shape),
                   np.zeros(len(grid), dtype=np.int32))
    a = DeviceFrames([spread])
    for _ in range(3):
        a.step(eng)
    cluster = grid * 1.2 + 2.0 + rng.normal(0, 0.03, grid.shape)
    a.pos.copy_(torch.tensor(cluster, device=a.pos.device))
    e, f, v, s = a.step(eng)
    eo, fo, vo, so, ne = om.efs(spread.cell, cluster, spread.types, threads=0)
    assert eng.edge_count() == ne and ne > 150 * spread.natoms
    assert rel_err(e[0], eo) < FP64_TOL and rel_err(f, fo) < FP64_TOL and rel_err(v[0], vo) < FP64_TOL
    for _ in range(2):   # captured again at the grown capacity
        e2, f2, v2, s2 = a.step(eng)
        assert e2[0] == e[0] and np.array_equal(f2, f)


def test_stage_timer_runs_eagerly(sg, golden):
    path = os.path.join(golden, "models", "static_l3k4o2.sus2")
    m = sg.Model(path)
    eng = sg.Engine(m, 0, sg.FP32)
    a = DeviceFrames(batch(1))
    ref = a.step(eng)
    eng.set_timing(True)
    for _ in range(3):
        for x, y in zip(a.step(eng), ref):
            assert np.array_equal(x, y)
    times = eng.take_stage_times()
    assert times["edges"][1] == 3 and times["outer"][1] >= 3
    eng.set_timing(False)
    for _ in range(3):
        for x, y in zip(a.step(eng), ref):
            assert np.array_equal(x, y)


@pytest.mark.parametrize("name", ["static_l3k4o2", "effect_l3k4r2o2"])
@pytest.mark.parametrize("precision", ["FP64", "FP32"])
def test_programmatic_launch_matches_serial_launches(sg, golden, name, precision):
    """Programmatic dependent launch between the step's kernels (the default sites, and all sites)
    against plain stream order, bit for bit, eager and replayed: a cell-list frame (4,096 atoms),
    image-scan frames and a mixed batch of both."""
    import torch
    path = os.path.join(golden, "models", f"{name}.sus2")
    m = sg.Model(path)
    prec = getattr(sg, precision)
    C = m.dims["C"]
    big = diamond(8, sigma=0.06, seed=21, species=C)
    small = [diamond(3, sigma=0.05, seed=s, species=C) for s in (22, 23)]
    for frames, level in (([big], -1), ([big], 15), (small, -1), ([small[0], big, small[1]], 15)):
        pdl, serial = sg.Engine(m, 0, prec), sg.Engine(m, 0, prec)
        pdl.set_pdl(level)
        serial.set_pdl(0)
        for graph in (False, True):
            pdl.set_step_graph(graph)
            serial.set_step_graph(graph)
            a, b = DeviceFrames(frames), DeviceFrames(frames)
            rng = np.random.default_rng(8)
            for step in range(4):
                for x, y in zip(a.step(pdl), b.step(serial)):
                    assert np.array_equal(x, y), f"graph={graph} step {step}"
                d = torch.tensor(rng.normal(0, 0.01, tuple(a.pos.shape)), device=a.pos.device)
                a.pos += d
                b.pos += d
        for x, y in zip(pdl.calc_efs(frames), serial.calc_efs(frames)):
            assert np.array_equal(x, y)


@pytest.mark.parametrize("cells", [3, 7])
def test_device_species_out_of_range_raise(sg, golden, cells):
    """Species indices given in device memory are checked by the edge build (image scan at 216
    atoms, cell lists at 2,744); the passes never index their tables with them, and the engine is
    usable afterwards."""
    path = os.path.join(golden, "models", "effect_l3k4r2o2.sus2")
    m = sg.Model(path)
    for prec in (sg.FP64, sg.FP32):
        eng = sg.Engine(m, 0, prec)
        frames = [diamond(cells, sigma=0.05, seed=41, species=2)]
        a = DeviceFrames(frames)
        ref = a.step(eng)
        good = a.types.clone()
        for bad in (2, -1, 1 << 20):
            a.types[frames[0].natoms // 3] = bad
            with pytest.raises(sg.Sus2Error, match="species index out of range"):
                a.step(eng)
            a.types.copy_(good)
        for x, y in zip(a.step(eng), ref):
            assert np.array_equal(x, y)
