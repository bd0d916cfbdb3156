"""The C++ Kernel surface (include/sus2g_kernel.hpp) compiled by g++ into a client program that
links libsus2g.so: one- and two-domain staged runs of a periodic frame, driven as the reference's
standalone harness drives its Kernel (tests/cpp/kernel_domains.cpp), against the periodic
evaluation of the same frame.  Bars: FP64 within 1e-10 relative, FP32 bulk within 1e-5."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from superlinear_gb300.synth import training_frames

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def client(engine_lib, tmp_path_factory):
    from superlinear_gb300 import _lib
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    out = str(tmp_path_factory.mktemp("cpp") / "kernel_domains")
    libdir = os.path.dirname(_lib.LIB_PATH)
    cmd = [cxx, "-O2", "-std=c++17", "-I", os.path.join(ROOT, "include"), os.path.join(ROOT, "tests", "cpp", "kernel_domains.cpp"),
           "-L", libdir, "-lsus2g", f"-Wl,-rpath,{libdir}", "-o", out]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    return out


def write_frame(path, fr):
    with open(path, "wb") as fh:
        fh.write(np.int32(fr.natoms).tobytes())
        fh.write(np.ascontiguousarray(fr.cell, dtype="<f8").tobytes())
        fh.write(np.ascontiguousarray(fr.positions, dtype="<f8").tobytes())
        fh.write(np.ascontiguousarray(fr.types, dtype="<i4").tobytes())


@pytest.mark.parametrize("model", ["static_l2k3o2_c2", "effect_l3k4r2o2"])
@pytest.mark.parametrize("domains", [1, 2])
@pytest.mark.parametrize("precision,tol", [(0, 1e-10), (1, 1e-5)])
def test_cpp_kernel_domains_match_periodic(client, golden, tmp_path, model, domains, precision, tol):
    fr = training_frames(1, 20, 40, 3.4, 4.0, 0.1, seed=61, species=2)[0]
    frame = str(tmp_path / "frame.bin")
    write_frame(frame, fr)
    r = subprocess.run([client, os.path.join(golden, "models", model + ".sus2"), frame, str(domains), str(precision)],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    line = [x for x in r.stdout.splitlines() if x.startswith("RESULT")][-1]
    errs = [float(x) for x in line.split()[1:]]
    assert max(errs) <= tol, (line, r.stdout[-500:])
