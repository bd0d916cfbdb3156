"""Shared fixtures: golden-fixture access and the oracle / engine libraries."""
import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); run with -m gpu")


@pytest.fixture(scope="session")
def golden():
    return GOLDEN


@pytest.fixture(scope="session")
def oracle_lib():
    import oracle as orc
    orc.build()
    return orc


@pytest.fixture(scope="session")
def engine_lib():
    from superlinear_gb300 import build
    build.build()
    from superlinear_gb300 import _lib
    return _lib.load()


def rel_err(a, b):
    """max |a-b| / (1 + max(|a|, |b|)) -- the reference harness's tolerance form
    (interfaces/lammps/tests/embedded_two_cutoff_check.py:30-37)."""
    a = np.asarray(a, dtype=float)
    b = np.asarray(b, dtype=float)
    return float(np.max(np.abs(a - b) / (1.0 + np.maximum(np.abs(a), np.abs(b))))) if a.size else 0.0


def load_json(path):
    with open(path) as fh:
        return json.load(fh)


def virial6_to_matrix(v):
    v = np.asarray(v)
    return np.array([[v[0], v[3], v[4]], [v[3], v[1], v[5]], [v[4], v[5], v[2]]])


def two_cutoff_cases():
    """(model path, geometry frames path, reference json path) of the reference's golden fixtures."""
    out = []
    for sub, names in (("fixtures_v2", ("static", "effect")), ("fixtures_hi_l", ("effect_l3k4r3o3",))):
        for nm in names:
            out.append((os.path.join(GOLDEN, "two_cutoff", sub, nm + ".mtp"),
                        os.path.join(GOLDEN, "two_cutoff", sub, "geometries.cfg"),
                        os.path.join(GOLDEN, "two_cutoff", sub, nm + ".efs.json")))
    return out
