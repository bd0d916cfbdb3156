"""Host-side logic that needs no GPU: the C ABI exports, .sus2 parsing and validation through the
library's host code, parameter layout, workload generators, and .cfg / .sus2 text round trips."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from superlinear_gb300.sus2_format import read_sus2, write_sus2
from superlinear_gb300.synth import (coeff_layout, diamond, fields_to_vector, read_cfg, training_frames,
                                     vector_to_fields, write_cfg)

MODELS = ("static_l3k4o2", "effect_l3k4r2o2", "effect_l4k8r2o3", "static_l2k3o2_c2")


def test_abi_exports_every_declared_symbol(engine_lib):
    from superlinear_gb300._lib import header_functions
    names = header_functions()
    assert len(names) >= 18
    missing = [n for n in names if not hasattr(engine_lib, n)]
    assert not missing, missing
    assert engine_lib.sus2g_abi_version() == 100


@pytest.mark.parametrize("name", MODELS)
def test_model_dims_and_params(engine_lib, golden, name):
    from superlinear_gb300 import Model
    path = os.path.join(golden, "models", name + ".sus2")
    m = Model(path)
    f = read_sus2(path)
    assert m.dims["M"] == int(f["alpha_moments_count"])
    assert m.dims["P"] == int(f["sh_product_count"])
    assert m.dims["S"] == int(f["alpha_scalar_moments"])
    assert m.nparams == sum(s for _, s in coeff_layout(f))
    assert np.array_equal(m.params(), fields_to_vector(f))


def test_reference_dimensions_of_benchmark_models(engine_lib, golden):
    """The init-sh topologies have the reference's sizes (F, NB, M, P, S, parameters)."""
    from superlinear_gb300 import Model
    expect = {"static_l3k4o2": (16, 64, 208, 436, 60, 246), "effect_l3k4r2o2": (16, 64, 296, 652, 26, 1464),
              "effect_l4k8r2o3": (40, 200, 770, 2630, 60, 5228)}
    for name, dims in expect.items():
        d = Model(os.path.join(golden, "models", name + ".sus2")).dims
        assert (d["F"], d["NB"], d["M"], d["P"], d["S"], d["nparams"]) == dims


def test_set_params_roundtrip(engine_lib, golden):
    from superlinear_gb300 import Model
    m = Model(os.path.join(golden, "models", "effect_l3k4r2o2.sus2"))
    p = m.params()
    q = p + np.linspace(0, 1, p.size)
    m.set_params(q)
    assert np.array_equal(m.params(), q)
    with pytest.raises(RuntimeError):
        m.set_params(q[:-1])


@pytest.mark.parametrize("mutation,needle", [
    (lambda t: t.replace("potential_tag = SUS2-SH", "potential_tag = MTP"), "SUS2-SH"),
    (lambda t: t.replace("version = 1.8.0", "version = 9.9.9"), "version"),
    (lambda t: t.replace("alpha_moments_count = 208", "alpha_moments_count = 20"), ""),
    (lambda t: t.replace("sh_product_count = 436", "sh_product_count = 435"), "sh_product_count"),
    (lambda t: t.replace("outer_radial_mode = legacy-plus-mixer", "outer_radial_mode = adaptive-coefficients"), "outer_radial_mode"),
    (lambda t: t.replace("MTP", "XYZ", 1), "MTP header"),
    (lambda t: t.replace("scal_coeffs = {", "scal_coeffs = {1.0, "), "scal_coeffs"),
])
def test_model_validation_errors(engine_lib, golden, tmp_path, mutation, needle):
    from superlinear_gb300 import Model, Sus2Error
    text = open(os.path.join(golden, "models", "static_l3k4o2.sus2")).read()
    bad = tmp_path / "bad.sus2"
    bad.write_text(mutation(text))
    with pytest.raises(Sus2Error) as info:
        Model(str(bad))
    assert needle in str(info.value)


def test_missing_model_file(engine_lib, tmp_path):
    from superlinear_gb300 import Model, Sus2Error
    with pytest.raises(Sus2Error):
        Model(str(tmp_path / "nope.sus2"))


def test_two_cutoff_fixture_models_load(engine_lib, golden):
    from superlinear_gb300 import Model
    m = Model(os.path.join(golden, "two_cutoff", "fixtures_v2", "effect.mtp"))
    assert m.dims["split"] == 1 and m.dims["gated"] == 1
    s = Model(os.path.join(golden, "two_cutoff", "fixtures_v2", "static.mtp"))
    assert s.dims["outer_rank"] == 0 and s.dims["gated"] == 0


def test_sus2_text_roundtrip(tmp_path, golden):
    for name in MODELS:
        f = read_sus2(os.path.join(golden, "models", name + ".sus2"))
        v = fields_to_vector(f)
        vector_to_fields(f, v * 1.5)
        out = tmp_path / (name + ".sus2")
        write_sus2(str(out), f)
        assert np.allclose(fields_to_vector(read_sus2(str(out))), v * 1.5, rtol=0, atol=0)


def test_cfg_roundtrip(tmp_path):
    frames = training_frames(5, 8, 64, 3.0, 4.2, 0.1, seed=3)
    for k, fr in enumerate(frames):
        fr.energy = float(k)
        fr.forces = np.full((fr.natoms, 3), 0.5)
        fr.stress = np.eye(3) * k
    p = tmp_path / "a.cfg"
    write_cfg(str(p), frames)
    back = read_cfg(str(p))
    assert len(back) == 5
    for a, b in zip(frames, back):
        assert np.array_equal(a.positions, b.positions) and np.array_equal(a.types, b.types)
        assert np.array_equal(a.cell, b.cell) and a.energy == b.energy
        assert np.array_equal(a.forces, b.forces) and np.allclose(a.stress, b.stress)


def test_workload_generators_are_seeded():
    a = diamond(2, sigma=0.08, seed=5)
    b = diamond(2, sigma=0.08, seed=5)
    assert a.natoms == 64 and np.array_equal(a.positions, b.positions)
    fr = training_frames(64, 8, 216, 3.0, 4.2, 0.1, seed=1)
    n = np.array([f.natoms for f in fr])
    assert n.min() >= 8 and n.max() <= 216 and len(set(n.tolist())) > 10
    assert {0, 1} >= set(np.concatenate([f.types for f in fr]).tolist())


@pytest.mark.parametrize("name", ["static_l3k4o2", "effect_l3k4r2o2", "effect_l4k8r2o3", "static_l2k3o2_c2_poly5"])
def test_model_save_reloads_bit_exactly(engine_lib, oracle_lib, golden, tmp_path, name):
    """sus2g_model_save (MLMTPR::Save counterpart): a changed parameter vector written and read back
    through the library, the Python reader, the oracle and -- when it has been built here -- the
    reference trainer, bit for bit."""
    import subprocess

    import superlinear_gb300 as sg
    m = sg.Model(os.path.join(golden, "models", f"{name}.sus2"))
    p = m.params() * (1.0 + 0.125 * np.sin(np.arange(m.nparams))) + 1e-3
    m.set_params(p)
    out = str(tmp_path / "saved.sus2")
    m.save(out)
    assert np.array_equal(sg.Model(out).params(), p)
    assert np.array_equal(fields_to_vector(read_sus2(out)), p)
    assert np.array_equal(oracle_lib.OracleModel(out).params(), p)
    assert sg.Model(out).dims == m.dims
    ref = os.path.join(os.path.dirname(os.path.dirname(__file__)), "oracle", "_ref", "ref-grad")
    if os.path.exists(ref):
        first = subprocess.run([ref, out, "/dev/null"], capture_output=True, text=True, check=True).stdout.splitlines()[0]
        import json
        assert np.array_equal(np.asarray(json.loads(first)["coeffs"]), p)


def test_model_save_rejects_bad_path(engine_lib, golden):
    import superlinear_gb300 as sg
    m = sg.Model(os.path.join(golden, "models", "static_l3k4o2.sus2"))
    with pytest.raises(sg.Sus2Error):
        m.save("/nonexistent-directory/x.sus2")


@pytest.mark.parametrize("name", ["static_l3k4o2", "effect_l4k8r2o3"])
def test_plain_c_client_of_the_abi(engine_lib, golden, tmp_path, name):
    """include/sus2g.h compiled as C99 with warnings as errors, linked against libsus2g.so by a C
    program (tests/c/model_info.c) that loads a model, reads its dimensions, cutoff and
    parameters and checks the error reporting of a missing file: the same values as the Python
    binding reads.  Also compiles both headers as C++17.  Needs no GPU."""
    import superlinear_gb300 as sg
    from superlinear_gb300 import _lib
    cc = shutil.which("gcc") or shutil.which("cc")
    cxx = shutil.which("g++") or shutil.which("c++")
    if cc is None or cxx is None:
        pytest.skip("no C / C++ compiler")
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    inc = os.path.join(root, "include")
    libdir = os.path.dirname(_lib.LIB_PATH)
    exe = str(tmp_path / "model_info")
    r = subprocess.run([cc, "-std=c99", "-Wall", "-Wextra", "-Werror", "-I", inc,
                        os.path.join(root, "tests", "c", "model_info.c"), "-L", libdir, "-lsus2g",
                        f"-Wl,-rpath,{libdir}", "-lm", "-o", exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    hpp = tmp_path / "headers.cpp"
    hpp.write_text('#include "sus2g.h"\n#include "sus2g_kernel.hpp"\nint main() { return 0; }\n')
    r = subprocess.run([cxx, "-std=c++17", "-Wall", "-Werror", "-fsyntax-only", "-I", inc, str(hpp)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]

    path = os.path.join(golden, "models", f"{name}.sus2")
    r = subprocess.run([exe, path], capture_output=True, text=True)
    assert r.returncode == 0, (r.returncode, r.stderr[-2000:])
    fields = r.stdout.split()
    assert fields[0] == "INFO"
    dims = [int(x) for x in fields[1:17]]
    cutoff, count, abs_sum = float(fields[17]), int(fields[18]), float(fields[19])
    m = sg.Model(path)
    p = np.asarray(m.params())
    assert count == p.size == dims[11]
    assert cutoff == m.cutoff
    assert dims == [int(v) for v in m.dims.values()]
    assert abs(abs_sum - float(np.abs(p).sum())) <= 1e-12 * max(1.0, abs_sum)
