"""Staged evaluation with a caller halo exchange (the multi-domain pair_style sus2/embedded path):
begin / pack_forward / unpack_forward / outer / pack_reverse / add_reverse / finish through the
C ABI, against the periodic evaluation of the same frame.

The domains are LAMMPS-style layouts built from a periodic frame: owned atoms first, then one
ghost per (atom, periodic image) that an owned centre sees; the exchanges between the stages are
done here on the host, as the pair style's comm callbacks would (pair_sus2_embedded.cpp:327-374).
Bars: FP64 plain within 1e-10 relative of the periodic FP64 evaluation; bitwise determinism.
"""
import itertools
import os

import numpy as np
import pytest

from conftest import rel_err
from superlinear_gb300.synth import training_frames

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-10


@pytest.fixture(scope="module")
def sg(engine_lib):
    import superlinear_gb300
    return superlinear_gb300


def periodic_edges(fr, rc):
    """All (i, j, image) with |x_j + n.cell - x_i| < rc, excluding i == j at n = 0."""
    inv = np.linalg.inv(fr.cell)
    reach = np.ceil(rc * np.linalg.norm(inv, axis=0)).astype(int) + 1
    out = []
    pos = fr.positions
    for n in itertools.product(*[range(-r, r + 1) for r in reach]):
        shift = np.asarray(n, dtype=np.float64) @ fr.cell
        d = pos[None, :, :] + shift - pos[:, None, :]
        r2 = np.einsum("ijk,ijk->ij", d, d)
        ii, jj = np.nonzero(r2 < rc * rc)
        for i, j in zip(ii, jj):
            if i == j and n == (0, 0, 0):
                continue
            out.append((int(i), int(j), n, d[i, j]))
    return out


def domain_layout(fr, edges, owned):
    """Local layout of one domain: owned atoms (global indices) first, then ghosts (global j, image)."""
    local = {(int(g), (0, 0, 0)): k for k, g in enumerate(owned)}
    ghosts = []
    ei, ej, d = [], [], []
    owned_set = set(int(g) for g in owned)
    for i, j, n, dv in edges:
        if i not in owned_set:
            continue
        key = (j, n)
        if key not in local:
            local[key] = len(owned) + len(ghosts)
            ghosts.append(j)
        ei.append(local[(i, (0, 0, 0))])
        ej.append(local[key])
        d.append(dv)
    glob = list(int(g) for g in owned) + ghosts
    return {"owned": [int(g) for g in owned], "ghost_owner": ghosts, "global": glob,
            "types": fr.types[glob], "ei": np.array(ei), "ej": np.array(ej), "d": np.array(d)}


def staged_run(sg, model, precision, fr, edges, parts, split=False):
    """Runs the staged calls on one engine per domain (with every pass split at the per-atom
    boundary when split is set); returns total energy, forces per global atom (owned + ghost
    contributions), total virial and site energies per global atom."""
    doms = [domain_layout(fr, edges, p) for p in parts]
    where = {}
    for k, dom in enumerate(doms):
        for loc, g in enumerate(dom["owned"]):
            where[g] = (k, loc)
    engs = [sg.Engine(model, 0, precision) for _ in doms]
    for eng in engs:
        eng.set_static_split(split)
    for eng, dom in zip(engs, doms):
        eng.stage_begin(len(dom["owned"]), dom["types"], dom["ei"], dom["ej"], dom["d"])
    width = engs[0].comm_width()

    def by_owner(dom):
        groups = {}
        for q, g in enumerate(dom["ghost_owner"]):
            k, loc = where[g]
            groups.setdefault(k, ([], []))
            groups[k][0].append(q)
            groups[k][1].append(loc)
        return groups

    # forward exchange: gate signals of the owners into the ghost rows
    for eng, dom in zip(engs, doms):
        G = len(dom["ghost_owner"])
        buf = np.zeros((G, width))
        for k, (rows, locs) in by_owner(dom).items():
            buf[rows] = engs[k].pack_forward(locs)
        if G and width:
            eng.unpack_forward(len(dom["owned"]), buf)
    for eng in engs:
        eng.stage_outer()
    # reverse exchange: ghost adjoints added to their owners
    for eng, dom in zip(engs, doms):
        G = len(dom["ghost_owner"])
        if not (G and width):
            continue
        buf = eng.pack_reverse(len(dom["owned"]), G)
        for k, (rows, locs) in by_owner(dom).items():
            engs[k].add_reverse(locs, buf[rows])
    e_tot, v_tot = 0.0, np.zeros(6)
    forces = np.zeros((fr.natoms, 3))
    site = np.zeros(fr.natoms)
    for eng, dom in zip(engs, doms):
        nown, nall = len(dom["owned"]), len(dom["global"])
        e, s, f, v = eng.stage_finish(nown, nall)
        e_tot += e
        v_tot += v
        np.add.at(forces, dom["global"], f)
        site[dom["owned"]] = s
    return e_tot, forces, v_tot, site


def frame_and_model(sg, golden, name, seed):
    model = sg.Model(os.path.join(golden, "models", f"{name}.sus2"))
    fr = training_frames(1, 48, 80, 3.4, 3.8, 0.1, seed=seed, species=model.dims["C"])[0]
    return model, fr


@pytest.mark.parametrize("name", ["effect_l3k4r2o2", "static_l2k3o2_c2"])
@pytest.mark.parametrize("ndomains", [1, 2])
def test_staged_domains_match_periodic(sg, golden, name, ndomains):
    model, fr = frame_and_model(sg, golden, name, seed=61 + ndomains)
    ref = sg.Engine(model, 0, sg.FP64)
    e0, f0, v0, s0 = ref.calc_efs([fr])
    edges = periodic_edges(fr, model.cutoff)
    assert len(edges) == ref.edge_count()
    order = np.argsort(fr.positions[:, 0])
    parts = np.array_split(order, ndomains)
    e, f, v, s = staged_run(sg, model, sg.FP64, fr, edges, parts)
    assert rel_err(e, e0[0]) < FP64_TOL
    assert rel_err(f, f0) < FP64_TOL
    assert rel_err(v, v0[0]) < FP64_TOL
    assert rel_err(s, s0) < FP64_TOL
    if model.dims["gated"]:
        assert ref.comm_width() == model.dims["F"]
    else:
        assert ref.comm_width() == 0


def test_staged_fp32_and_determinism(sg, golden):
    model, fr = frame_and_model(sg, golden, "effect_l3k4r2o2", seed=71)
    edges = periodic_edges(fr, model.cutoff)
    order = np.argsort(fr.positions[:, 1])
    parts = np.array_split(order, 2)
    e1, f1, v1, s1 = staged_run(sg, model, sg.FP32, fr, edges, parts)
    e2, f2, v2, s2 = staged_run(sg, model, sg.FP32, fr, edges, parts)
    assert e1 == e2 and np.array_equal(f1, f2) and np.array_equal(v1, v2) and np.array_equal(s1, s2)
    e0, f0, v0, s0 = sg.Engine(model, 0, sg.FP64).calc_efs([fr])
    assert np.max(np.abs(f1 - f0)) <= 1e-5
    assert abs(e1 - e0[0]) / fr.natoms <= 1e-6


def test_staged_split_passes(sg, golden):
    """The staged calls with every Effect pass split at the per-atom boundary (gate forward into
    its edge->moment and per-atom gate graph kernels, the outer pass into three, the gate reverse
    pass gathering the caller's summed gate-signal adjoints in its per-atom kernel) agree with the
    fused passes to FP32 rounding and keep the FP32 bar against the periodic FP64 evaluation."""
    model, fr = frame_and_model(sg, golden, "effect_l3k4r2o2", seed=73)
    edges = periodic_edges(fr, model.cutoff)
    parts = np.array_split(np.argsort(fr.positions[:, 2]), 2)
    fused = staged_run(sg, model, sg.FP32, fr, edges, parts)
    split = staged_run(sg, model, sg.FP32, fr, edges, parts, split=True)
    for x, y in zip(fused, split):
        assert rel_err(x, y) < 2e-6
    e0, f0, v0, s0 = sg.Engine(model, 0, sg.FP64).calc_efs([fr])
    assert np.max(np.abs(split[1] - f0)) <= 1e-5
    assert abs(split[0] - e0[0]) / fr.natoms <= 1e-6


def test_staged_order_is_enforced(sg, golden):
    model, fr = frame_and_model(sg, golden, "effect_l3k4r2o2", seed=72)
    eng = sg.Engine(model, 0, sg.FP64)
    with pytest.raises(sg.Sus2Error):
        eng.stage_outer()                       # before begin
    dom = domain_layout(fr, periodic_edges(fr, model.cutoff), np.arange(fr.natoms))
    eng.stage_begin(fr.natoms, dom["types"], dom["ei"], dom["ej"], dom["d"])
    with pytest.raises(sg.Sus2Error):
        eng.pack_reverse(fr.natoms, 1)          # adjoint exchange before outer
    with pytest.raises(sg.Sus2Error):
        eng.pack_forward([len(dom["global"]) + 5])   # index outside the layout
    # the one-call entry point refuses an Effect ghost layout (it has no exchange)
    with pytest.raises(sg.Sus2Error):
        eng.efs_edges(fr.natoms, dom["types"], dom["ei"], dom["ej"], dom["d"])
