"""The allocation-free entry point sus2g_static_efs_noalloc, called through the C ABI.

It serves callers that cannot allocate device memory during a step (stream capture, arena-managed
MD codes).  It must give the same E / F / virial as the regular caller-edge entry point
(sus2g_efs_edges_host) within the FP32-bulk tolerance used by the other GPU tests, on two calls
in a row (the scratch array keeps the previous call's contents), and reject sizes above its
stated maximum.  Kept in its own file, collected last.
"""
import ctypes
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FORCE_TOL = 1e-5    # eV/A, as the FP32-bulk bound of the other GPU tests
ENERGY_TOL = 1e-6   # eV/atom


def periodic_edges(frame, cutoff):
    """Directed edges of an orthorhombic box wider than 2 cutoff (minimum image), sorted by centre."""
    L = np.diag(frame.cell)
    x = frame.positions
    ei, ej, d = [], [], []
    for i in range(frame.natoms):
        v = x - x[i]
        v -= L * np.round(v / L)
        r2 = np.einsum("ij,ij->i", v, v)
        idx = np.nonzero((r2 < cutoff * cutoff) & (np.arange(frame.natoms) != i))[0]
        ei.append(np.full(idx.size, i))
        ej.append(idx)
        d.append(v[idx])
    return (np.concatenate(ei).astype(np.int32), np.concatenate(ej).astype(np.int32),
            np.ascontiguousarray(np.concatenate(d)))


@pytest.fixture(scope="module")
def setup(engine_lib, golden):
    torch = pytest.importorskip("torch")
    import superlinear_gb300 as sg
    from superlinear_gb300.synth import diamond
    model = sg.Model(os.path.join(golden, "models", "static_l3k4o2.sus2"))
    engine = sg.Engine(model, 0, sg.FP32)
    return torch, sg, model, engine, diamond


def run_noalloc(torch, lib, engine, n, types, ei, ej, d):
    dev = torch.device("cuda", 0)
    counts = np.bincount(ei, minlength=n)
    row = np.concatenate([[0], np.cumsum(counts)]).astype(np.int32)
    t_types = torch.tensor(types, dtype=torch.int32, device=dev)
    t_row = torch.tensor(row, device=dev)
    t_nbr = torch.tensor(ej, dtype=torch.int32, device=dev)
    t_vec = torch.tensor(d, dtype=torch.float64, device=dev)
    e = torch.zeros(1, dtype=torch.float64, device=dev)
    f = torch.full((n, 3), 7.0, dtype=torch.float64, device=dev)   # must be overwritten
    v = torch.zeros(6, dtype=torch.float64, device=dev)
    s = torch.zeros(n, dtype=torch.float64, device=dev)
    torch.cuda.synchronize()
    vp = ctypes.c_void_p
    rc = lib.sus2g_static_efs_noalloc(engine._h, n, n, vp(t_types.data_ptr()), vp(t_row.data_ptr()),
                                      vp(t_nbr.data_ptr()), vp(t_vec.data_ptr()), ei.size, vp(e.data_ptr()),
                                      vp(f.data_ptr()), vp(v.data_ptr()), vp(s.data_ptr()))
    assert rc == 0, lib.sus2g_last_error().decode()
    torch.cuda.synchronize()
    return float(e.cpu()[0]), f.cpu().numpy(), v.cpu().numpy(), s.cpu().numpy()


@pytest.mark.parametrize("cells,seed", [(4, 31), (8, 32)])
def test_noalloc_matches_regular_entry_point_twice(setup, engine_lib, cells, seed):
    torch, sg, model, engine, diamond = setup
    frame = diamond(cells, sigma=0.08, seed=seed)  # boxes wider than 2 cutoff: minimum image holds
    ei, ej, d = periodic_edges(frame, model.cutoff)
    n = frame.natoms
    e_ref, s_ref, f_ref, v_ref = engine.efs_edges(n, frame.types, ei, ej, d)
    for _ in range(2):
        e, f, v, s = run_noalloc(torch, engine_lib, engine, n, frame.types, ei, ej, d)
        assert np.max(np.abs(f - f_ref)) <= FORCE_TOL
        assert abs(e - e_ref) / n <= ENERGY_TOL
        assert np.max(np.abs(s - s_ref)) <= ENERGY_TOL
        assert np.max(np.abs(v - v_ref)) <= FORCE_TOL * max(1.0, np.max(np.abs(v_ref)))


def test_noalloc_rejects_sizes_above_maximum(setup, engine_lib):
    torch, sg, model, engine, diamond = setup
    dev = torch.device("cuda", 0)
    dummy = torch.zeros(8, dtype=torch.int32, device=dev)
    vec = torch.zeros(24, dtype=torch.float64, device=dev)
    vp = ctypes.c_void_p
    rc = engine_lib.sus2g_static_efs_noalloc(engine._h, 4, 4, vp(dummy.data_ptr()), vp(dummy.data_ptr()),
                                             vp(dummy.data_ptr()), vp(vec.data_ptr()), 524289, None, None, None, None)
    assert rc != 0 and "exceed the maximum" in engine_lib.sus2g_last_error().decode()
    rc = engine_lib.sus2g_static_efs_noalloc(engine._h, 16385, 16385, vp(dummy.data_ptr()), vp(dummy.data_ptr()),
                                             vp(dummy.data_ptr()), vp(vec.data_ptr()), 8, None, None, None, None)
    assert rc != 0 and "exceed the maximum" in engine_lib.sus2g_last_error().decode()
