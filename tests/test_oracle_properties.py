"""Size-independent properties of the CPU oracle on random periodic frames (CPU only): the energy
is invariant under a rigid rotation and a translation of the frame, forces rotate with it and sum
to zero over the periodic frame, the virial is symmetric and rotates as a tensor, and a relabelled
atom order permutes the per-atom outputs only.  Static and Effect models, two species."""
import os

import numpy as np
import pytest

from superlinear_gb300.synth import training_frames

MODELS = ("static_l2k3o2_c2", "effect_l3k4r2o2")


def rotation(seed):
    q = np.random.default_rng(seed).normal(size=4)
    a, b, c, d = q / np.linalg.norm(q)
    return np.array([[a * a + b * b - c * c - d * d, 2 * (b * c - a * d), 2 * (b * d + a * c)],
                     [2 * (b * c + a * d), a * a - b * b + c * c - d * d, 2 * (c * d - a * b)],
                     [2 * (b * d - a * c), 2 * (c * d + a * b), a * a - b * b - c * c + d * d]])


def full_virial(v6):
    xx, yy, zz, xy, xz, yz = v6
    return np.array([[xx, xy, xz], [xy, yy, yz], [xz, yz, zz]])


@pytest.mark.parametrize("name", MODELS)
def test_rigid_motion_and_permutation(oracle_lib, golden, name):
    m = oracle_lib.OracleModel(os.path.join(golden, "models", f"{name}.sus2"))
    fr = training_frames(1, 24, 40, 3.2, 3.8, 0.1, seed=91, species=2)[0]
    e, f, v, s, ne = m.efs(fr.cell, fr.positions, fr.types)
    assert ne > 0
    scale = 1.0 + np.max(np.abs(f))
    # periodic frame: the forces sum to zero; the virial is symmetric
    assert np.max(np.abs(f.sum(axis=0))) <= 1e-10 * scale * fr.natoms
    # a rigid rotation of cell and positions (rows of the cell are the lattice vectors)
    R = rotation(5)
    er, fr_, vr, sr, ner = m.efs(fr.cell @ R.T, fr.positions @ R.T, fr.types)
    assert ner == ne
    assert abs(er - e) <= 1e-10 * (1.0 + abs(e))
    assert np.max(np.abs(fr_ - f @ R.T)) <= 1e-10 * scale
    assert np.max(np.abs(full_virial(vr) - R @ full_virial(v) @ R.T)) <= 1e-9 * (1.0 + np.max(np.abs(v)))
    assert np.max(np.abs(sr - s)) <= 1e-10 * (1.0 + np.max(np.abs(s)))
    # a translation, and a relabelling of the atoms
    et, ft, vt, st, _ = m.efs(fr.cell, fr.positions + np.array([0.37, -1.2, 2.9]), fr.types)
    assert abs(et - e) <= 1e-10 * (1.0 + abs(e)) and np.max(np.abs(ft - f)) <= 1e-10 * scale
    perm = np.random.default_rng(7).permutation(fr.natoms)
    ep, fp, vp, sp, _ = m.efs(fr.cell, fr.positions[perm], fr.types[perm])
    assert abs(ep - e) <= 1e-10 * (1.0 + abs(e))
    assert np.max(np.abs(fp - f[perm])) <= 1e-10 * scale
    assert np.max(np.abs(sp - s[perm])) <= 1e-10 * (1.0 + np.max(np.abs(s)))
    assert np.max(np.abs(vp - v)) <= 1e-10 * (1.0 + np.max(np.abs(v)))


@pytest.mark.parametrize("name", MODELS)
def test_parameter_gradient_is_rotation_invariant(oracle_lib, golden, name):
    """The combination gradient d/dtheta [sum ew E + sum_e (fw_i - fw_j + S d_e) . dE/dd_e] is the
    same for a rotated frame when the force weights rotate as vectors and the stress weights as a
    tensor (S -> R S R^T), and a relabelling of the atoms with their weights leaves it unchanged."""
    m = oracle_lib.OracleModel(os.path.join(golden, "models", f"{name}.sus2"))
    fr = training_frames(1, 20, 32, 3.2, 3.8, 0.1, seed=93, species=2)[0]
    rng = np.random.default_rng(17)
    ew = rng.normal(size=fr.natoms)
    fw = rng.normal(size=(fr.natoms, 3))
    S = rng.normal(size=(3, 3))
    g = m.grad(fr.cell, fr.positions, fr.types, ew, fw, S)
    assert np.linalg.norm(g) > 0
    R = rotation(23)
    gr = m.grad(fr.cell @ R.T, fr.positions @ R.T, fr.types, ew, fw @ R.T, R @ S @ R.T)
    assert np.linalg.norm(gr - g) <= 1e-10 * np.linalg.norm(g)
    perm = np.random.default_rng(29).permutation(fr.natoms)
    gp = m.grad(fr.cell, fr.positions[perm], fr.types[perm], ew[perm], fw[perm], S)
    assert np.linalg.norm(gp - g) <= 1e-10 * np.linalg.norm(g)
