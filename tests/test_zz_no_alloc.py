"""The allocation-free entry point sus2g_static_efs_noalloc, called through the C ABI.

It serves callers that cannot allocate device memory during a step (MD codes whose device memory
comes from a pre-sized arena, time loops that forbid driver allocations).  It must give the same
E / F / virial as the regular caller-edge entry point (sus2g_efs_edges_host) within the FP32-bulk
tolerance used by the other GPU tests, on two calls in a row (the scratch array keeps the previous
call's contents) and bitwise equal between them, with and without ghost atoms; reject sizes above
its stated maxima; and turn bad rows, neighbour indices and species into error codes.  The bad
inputs below stay within the caller's arrays: the entry point's first kernel reads each of them
only at its own index and records the violation, and every later kernel reads its clamped copies.
Kept in its own file, collected last.
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


def ghost_layout(frame, ei, ej, d):
    """Owned atoms 0..n-1 plus one ghost per edge whose neighbour lies in a shifted image (the
    pair style's layout): returns (types of all atoms, neighbour indices into them)."""
    n = frame.natoms
    x = frame.positions
    direct = np.abs((x[ej] - x[ei]) - d).max(axis=1) < 1e-9
    ghost = np.nonzero(~direct)[0]
    ej2 = ej.copy()
    ej2[ghost] = n + np.arange(ghost.size)
    types = np.concatenate([frame.types, frame.types[ej[ghost]]]).astype(np.int32)
    return types, ej2.astype(np.int32)


def csr_rows(ei, n):
    counts = np.bincount(ei, minlength=n)
    return np.concatenate([[0], np.cumsum(counts)]).astype(np.int32)


def call_noalloc(torch, lib, engine, n, types, row, ej, d):
    """One call with the given (possibly bad) layout; returns (rc, E, F, virial, site energies)."""
    dev = torch.device("cuda", 0)
    nall = len(types)
    t_types = torch.tensor(np.asarray(types, np.int32), device=dev)
    t_row = torch.tensor(np.asarray(row, np.int32), device=dev)
    t_nbr = torch.tensor(np.asarray(ej, np.int32), device=dev)
    t_vec = torch.tensor(np.asarray(d, np.float64).reshape(-1, 3), device=dev)
    e = torch.zeros(1, dtype=torch.float64, device=dev)
    f = torch.full((nall, 3), 7.0, dtype=torch.float64, device=dev)   # must be overwritten
    v = torch.zeros(6, dtype=torch.float64, device=dev)
    s = torch.zeros(max(n, 1), dtype=torch.float64, device=dev)
    torch.cuda.synchronize()
    vp = ctypes.c_void_p
    rc = lib.sus2g_static_efs_noalloc(engine._h, n, nall, vp(t_types.data_ptr()), vp(t_row.data_ptr()),
                                      vp(t_nbr.data_ptr()), vp(t_vec.data_ptr()), len(ej), vp(e.data_ptr()),
                                      vp(f.data_ptr()), vp(v.data_ptr()), vp(s.data_ptr()))
    torch.cuda.synchronize()
    return rc, float(e.cpu()[0]), f.cpu().numpy(), v.cpu().numpy(), s.cpu().numpy()[:n]


def run_noalloc(torch, lib, engine, n, types, ei, ej, d):
    dev = torch.device("cuda", 0)
    row = csr_rows(ei, n)
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
    prev = None
    for _ in range(2):
        e, f, v, s = run_noalloc(torch, engine_lib, engine, n, frame.types, ei, ej, d)
        assert np.max(np.abs(f - f_ref)) <= FORCE_TOL
        assert abs(e - e_ref) / n <= ENERGY_TOL
        assert np.max(np.abs(s - s_ref)) <= ENERGY_TOL
        assert np.max(np.abs(v - v_ref)) <= FORCE_TOL * max(1.0, np.max(np.abs(v_ref)))
        if prev is not None:  # fixed-order gathers: the second call is bitwise equal to the first
            assert prev[0] == e and np.array_equal(prev[1], f) and np.array_equal(prev[2], v)
        prev = (e, f, v)


def test_noalloc_with_ghosts_matches_regular_entry_point(setup, engine_lib):
    torch, sg, model, engine, diamond = setup
    frame = diamond(4, sigma=0.08, seed=35)
    ei, ej, d = periodic_edges(frame, model.cutoff)
    n = frame.natoms
    types, ej2 = ghost_layout(frame, ei, ej, d)
    assert types.size > n
    e_ref, s_ref, f_ref, v_ref = engine.efs_edges(n, types, ei, ej2, d)
    for _ in range(2):
        rc, e, f, v, s = call_noalloc(torch, engine_lib, engine, n, types, csr_rows(ei, n), ej2, d)
        assert rc == 0, engine_lib.sus2g_last_error().decode()
        assert f.shape == f_ref.shape and np.max(np.abs(f - f_ref)) <= FORCE_TOL
        assert abs(e - e_ref) / n <= ENERGY_TOL
        assert np.max(np.abs(v - v_ref)) <= FORCE_TOL * max(1.0, np.max(np.abs(v_ref)))


def test_noalloc_bad_input_returns_error_codes(setup, engine_lib):
    """Out-of-range neighbour indices, non-monotone or inconsistent rows and species outside [0, C)
    are reported as error codes; a good call afterwards is still correct."""
    torch, sg, model, engine, diamond = setup
    frame = diamond(4, sigma=0.08, seed=36)
    ei, ej, d = periodic_edges(frame, model.cutoff)
    n = frame.natoms
    row = csr_rows(ei, n)
    cases = []
    bad = ej.copy(); bad[17] = n + 5; cases.append(("nbr above nall", frame.types, row, bad, 21))
    bad = ej.copy(); bad[-1] = -3; cases.append(("negative nbr", frame.types, row, bad, 21))
    r = row.copy(); r[10], r[11] = r[11] + 40, r[10]; cases.append(("non-monotone row", frame.types, r, ej, 21))
    r = row.copy(); r[n] = row[n] - 1; cases.append(("last row below nedges", frame.types, r, ej, 21))
    r = row.copy(); r[5] = 10 * row[n]; cases.append(("row above nedges", frame.types, r, ej, 21))
    t = frame.types.copy(); t[3] = model.dims["C"] + 2; cases.append(("species above C", t, row, ej, 26))
    t = frame.types.copy(); t[0] = -1; cases.append(("negative species", t, row, ej, 26))
    for name, types, rows, nbr, code in cases:
        rc = call_noalloc(torch, engine_lib, engine, n, types, rows, nbr, d)[0]
        assert rc == code, (name, rc, engine_lib.sus2g_last_error().decode())
    e_ref, _, f_ref, _ = engine.efs_edges(n, frame.types, ei, ej, d)
    rc, e, f, _, _ = call_noalloc(torch, engine_lib, engine, n, frame.types, row, ej, d)
    assert rc == 0 and np.max(np.abs(f - f_ref)) <= FORCE_TOL and abs(e - e_ref) / n <= ENERGY_TOL


def test_noalloc_without_centres_gives_zeros(setup, engine_lib):
    torch, sg, model, engine, diamond = setup
    rc, e, f, v, _ = call_noalloc(torch, engine_lib, engine, 0, np.zeros(3, np.int32), np.zeros(1, np.int32),
                                  np.zeros(0, np.int32), np.zeros((0, 3)))
    assert rc == 0, engine_lib.sus2g_last_error().decode()
    assert e == 0.0 and not f.any() and not v.any()


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
    rc = engine_lib.sus2g_static_efs_noalloc(engine._h, 4, 65537, vp(dummy.data_ptr()), vp(dummy.data_ptr()),
                                             vp(dummy.data_ptr()), vp(vec.data_ptr()), 8, None, None, None, None)
    assert rc != 0 and "exceed the maximum" in engine_lib.sus2g_last_error().decode()
