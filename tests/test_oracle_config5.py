"""Config 5 topology (Effect L5/K8/R2/O2, three species) in the oracle.

The reference's model loader rejects sh_l_max > 4, so no reference values exist for this
topology.  The oracle is checked against its own finite differences instead: forces against
-dE/dx, the virial against the energy change under a homogeneous strain, and the parameter
gradient of the energy against central differences in a few parameters of every block type.
"""
import os

import numpy as np
import pytest

from superlinear_gb300.synth import training_frames

MODEL = "effect_l5k8r2o2_c3.sus2"


@pytest.fixture(scope="module")
def case(oracle_lib, golden):
    m = oracle_lib.OracleModel(os.path.join(golden, "models", MODEL))
    fr = training_frames(1, 16, 24, 2.8, 4.5, 0.15, seed=501, species=3, log_uniform=True)[0]
    return m, fr


def test_config5_forces_and_virial_are_energy_derivatives(case):
    m, fr = case
    e, f, v, s, ne = m.efs(fr.cell, fr.positions, fr.types)
    assert ne > 0 and abs(e - s.sum()) < 1e-10 * abs(e)
    h = 1e-5
    rng = np.random.default_rng(3)
    for i in rng.choice(fr.natoms, 4, replace=False):
        for c in range(3):
            p = fr.positions.copy()
            p[i, c] += h
            ep = m.efs(fr.cell, p, fr.types)[0]
            p[i, c] -= 2 * h
            em = m.efs(fr.cell, p, fr.types)[0]
            assert abs(-(ep - em) / (2 * h) - f[i, c]) < 1e-6 * (1 + abs(f[i, c]))
    # virial (xx, yy, zz, xy, xz, yz) = -dE/deps for positions and cell strained by (1 + eps)
    for k, (a, b) in enumerate(((0, 0), (1, 1), (2, 2), (0, 1), (0, 2), (1, 2))):
        vals = []
        for sgn in (1, -1):
            eps = np.eye(3)
            eps[a, b] += sgn * h
            if a != b:
                eps[b, a] += sgn * h
            vals.append(m.efs(fr.cell @ eps, fr.positions @ eps, fr.types)[0])
        dE = (vals[0] - vals[1]) / (2 * h) / (1 if a == b else 2)
        assert abs(-dE - v[k]) < 1e-6 * (1 + abs(v[k]))


def test_config5_parameter_gradient_is_energy_derivative(case):
    m, fr = case
    n = fr.natoms
    g = m.grad(fr.cell, fr.positions, fr.types, np.ones(n), np.zeros((n, 3)), np.zeros((3, 3)))
    p0 = m.params()
    rng = np.random.default_rng(4)
    idx = rng.choice(p0.size, 12, replace=False)
    for q in idx:
        h = 1e-6 * max(1.0, abs(p0[q]))
        p = p0.copy()
        p[q] += h
        m.set_params(p)
        ep = m.efs(fr.cell, fr.positions, fr.types)[0]
        p[q] -= 2 * h
        m.set_params(p)
        em = m.efs(fr.cell, fr.positions, fr.types)[0]
        m.set_params(p0)
        assert abs((ep - em) / (2 * h) - g[q]) < 1e-5 * (1 + abs(g[q])), q
