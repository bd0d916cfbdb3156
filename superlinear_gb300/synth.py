"""Seeded synthetic workloads: lattices, training frames, and model parameters.

The reference measures no public dataset for this path; every input here is
generated from a seed with the shapes of the benchmark configurations:

* periodic diamond boxes (a = 3.567 A, n x n x n conventional cells, Gaussian
  displacements) for the E/F/virial step;
* uneven training frames built from random fcc / bcc / diamond supercells;
* model parameters filled block by block in the reference's trainer parameter
  order (``dev_src/mtpr.h:1358-1470``, ``DistributeCoeffs``), so that a vector
  produced here can be written into a ``.sus2`` topology by either loader.
"""
from __future__ import annotations

import numpy as np

from .sus2_format import as_int, format_list, parse_list

__all__ = ["Frame", "diamond", "lattice_frame", "training_frames", "coeff_layout",
           "fields_to_vector", "vector_to_fields", "random_vector", "write_cfg", "read_cfg"]


class Frame:
    """One periodic configuration: ``cell`` rows are lattice vectors (A)."""

    def __init__(self, cell, positions, types, energy=None, forces=None, stress=None):
        self.cell = np.asarray(cell, dtype=np.float64).reshape(3, 3)
        self.positions = np.ascontiguousarray(positions, dtype=np.float64).reshape(-1, 3)
        self.types = np.ascontiguousarray(types, dtype=np.int32).reshape(-1)
        self.energy = energy
        self.forces = forces
        self.stress = stress  # plus-stress (virial, eV), 3x3

    @property
    def natoms(self) -> int:
        return int(self.types.shape[0])


_BASIS = {
    "fcc": np.array([[0, 0, 0], [0, .5, .5], [.5, 0, .5], [.5, .5, 0]], dtype=np.float64),
    "bcc": np.array([[0, 0, 0], [.5, .5, .5]], dtype=np.float64),
    "diamond": np.array([[0, 0, 0], [0, .5, .5], [.5, 0, .5], [.5, .5, 0],
                         [.25, .25, .25], [.25, .75, .75], [.75, .25, .75], [.75, .75, .25]],
                        dtype=np.float64),
}


def lattice_frame(kind: str, reps, a: float, sigma: float, rng, type_prob=None, species=1):
    """A ``reps``-repeated conventional cubic cell of ``kind`` with displacements."""
    basis = _BASIS[kind]
    n1, n2, n3 = (int(x) for x in reps)
    grid = np.stack(np.meshgrid(np.arange(n1), np.arange(n2), np.arange(n3), indexing="ij"), -1)
    frac = (grid.reshape(-1, 1, 3) + basis[None, :, :]).reshape(-1, 3)
    pos = frac * a + rng.normal(0.0, sigma, size=frac.shape)
    cell = np.diag([n1 * a, n2 * a, n3 * a])
    n = pos.shape[0]
    if species <= 1:
        types = np.zeros(n, dtype=np.int32)
    elif type_prob is not None:
        types = (rng.random(n) < type_prob).astype(np.int32)
    else:
        types = rng.integers(0, species, size=n).astype(np.int32)
    return Frame(cell, pos, types)


def diamond(ncell: int, a: float = 3.567, sigma: float = 0.05, seed: int = 0, species: int = 1,
            type_prob: float | None = None) -> Frame:
    """Periodic diamond box of ``8 ncell^3`` atoms (the E/F/virial benchmark geometry)."""
    rng = np.random.default_rng(seed)
    return lattice_frame("diamond", (ncell, ncell, ncell), a, sigma, rng,
                         type_prob=type_prob if species == 2 else None, species=species)


def training_frames(count: int, nmin: int, nmax: int, a_lo: float, a_hi: float, sigma: float,
                    seed: int, species: int = 2, log_uniform: bool = False):
    """Uneven random fcc/bcc/diamond frames with ``nmin <= N <= nmax`` atoms.

    The target size is drawn uniformly (or log-uniformly); the supercell repeats are
    the most cubic factorisation whose atom count is closest to the target.
    """
    rng = np.random.default_rng(seed)
    frames = []
    kinds = ("fcc", "bcc", "diamond")
    for _ in range(count):
        kind = kinds[int(rng.integers(0, 3))]
        nb = _BASIS[kind].shape[0]
        if log_uniform:
            target = float(np.exp(rng.uniform(np.log(nmin), np.log(nmax))))
        else:
            target = float(rng.integers(nmin, nmax + 1))
        best = None
        for n1 in range(1, 8):
            for n2 in range(n1, 8):
                for n3 in range(n2, 8):
                    n = nb * n1 * n2 * n3
                    if n < nmin or n > nmax:
                        continue
                    score = (abs(n - target), n3 - n1)
                    if best is None or score < best[0]:
                        best = (score, (n1, n2, n3))
        reps = best[1] if best else (1, 1, 1)
        reps = tuple(rng.permutation(reps))
        a = float(rng.uniform(a_lo, a_hi))
        frames.append(lattice_frame(kind, reps, a, sigma, rng, type_prob=0.5 if species == 2 else None,
                                    species=species))
    return frames


# --------------------------------------------------------------------------------------------
# Parameter vector layout (the reference trainer's Coeff() order for the supported families)
# --------------------------------------------------------------------------------------------

def _dims(fields):
    C = as_int(fields, "species_count")
    L = as_int(fields, "sh_l_max")
    K = as_int(fields, "sh_k_max")
    B = as_int(fields, "radial_basis_size")
    F = as_int(fields, "radial_funcs_count")
    S = as_int(fields, "alpha_scalar_moments")
    sm = fields.get("scaling_map", "LK")
    nblk = {"pair": 1, "L": L + 1, "K": K}.get(sm, F)
    return C, L, K, B, F, S, nblk


def coeff_layout(fields):
    """Ordered ``[(field_name, size), ...]`` of the trainable parameter vector.

    Static:  shift | scal | radial | [outer rank W] | species | moment readout
    Effect:  shift | scal | radial | gate radial | [gate scal] | gate additive | gate type |
             gate weights | gate rank W | outer rank W | species | moment readout
    """
    C, L, K, B, F, S, nblk = _dims(fields)
    gated = fields.get("two_layer_gate_enabled", "false") in ("true", "1")
    ranked = fields.get("outer_k_rank1_enabled", "false") in ("true", "1")
    O = as_int(fields, "outer_k_rank", 1) if ranked else 0
    G = as_int(fields, "two_layer_gate_k_rank", 0)
    heads = C if fields.get("readout_mode", "shared") == "species" else 1
    out = [("shift_coeffs", C), ("scal_coeffs", 2 * nblk * C * C), ("radial_coeffs", F * (B + C))]
    if gated:
        Q = len(parse_list(fields["two_layer_gate_scalar_indices"]))
        out.append(("two_layer_gate_radial_coeffs", F * B))
        if fields.get("two_layer_gate_scaling_mode", "shared-scaling") == "decoupled":
            out.append(("two_layer_gate_scaling_coeffs", 2 * nblk * C * C))
        out += [("two_layer_gate_additive_coeffs", C * F), ("two_layer_gate_type_coeffs", C * F),
                ("two_layer_gate_weights", F * Q)]
    if G > 0:
        out.append(("two_layer_gate_k_rank_weights", (L + 1) * G * K))
    if O > 0 and as_int(fields, "outer_k_rank1_weight_count", 0) > 0:
        out.append(("outer_k_rank1_weights", (L + 1) * O * K))
    out += [("species_coeffs", C), ("moment_coeffs", heads * S)]
    return out


def fields_to_vector(fields) -> np.ndarray:
    vals = []
    for name, size in coeff_layout(fields):
        v = parse_list(fields[name])
        if len(v) != size:
            raise ValueError(f"{name}: expected {size} values, found {len(v)}")
        vals.extend(v)
    return np.asarray(vals, dtype=np.float64)


def vector_to_fields(fields, vec) -> None:
    """Write ``vec`` (reference parameter order) into ``fields`` in place."""
    off = 0
    vec = np.asarray(vec, dtype=np.float64)
    for name, size in coeff_layout(fields):
        fields[name] = format_list(vec[off:off + size])
        count_key = {"two_layer_gate_radial_coeffs": "two_layer_gate_radial_coeff_count",
                     "two_layer_gate_additive_coeffs": "two_layer_gate_additive_coeff_count",
                     "two_layer_gate_type_coeffs": "two_layer_gate_type_coeff_count",
                     "two_layer_gate_weights": "two_layer_gate_weight_count",
                     "two_layer_gate_k_rank_weights": "two_layer_gate_k_rank_weight_count",
                     "outer_k_rank1_weights": "outer_k_rank1_weight_count"}.get(name)
        if count_key:
            fields[count_key] = str(size)
        off += size
    if off != vec.size:
        raise ValueError("parameter vector length does not match the model layout")


def random_vector(fields, seed: int, radial_scale: float = 1.0, readout_scale: float = 1.0) -> np.ndarray:
    """Seeded O(1)-force parameters for a topology (block by block, reference order).

    Readout weights are drawn ``readout_scale * U(-1, 1)/S`` with unit species
    coefficients and tau ~ U(0.5, 1.5); radial (and gate radial) coefficients
    ``radial_scale * U(-0.5, 0.5)``; warps slope ~ U(2.5, 3.5), shift ~ U(1.5, 2.5);
    gate weights U(-1, 1)/Q; contraction weights U(-1, 1).  The two scales are
    chosen per model so that forces on the benchmark geometries are O(1) eV/A
    rather than the ~1e-8 eV/A of an untrained model.
    """
    C, L, K, B, F, S, nblk = _dims(fields)
    rng = np.random.default_rng(seed)
    parts = []
    for name, size in coeff_layout(fields):
        if name == "shift_coeffs":
            v = rng.uniform(-1.5, -0.5, size)
        elif name in ("scal_coeffs", "two_layer_gate_scaling_coeffs"):
            v = np.empty(size)
            for blk in range(nblk):
                base = 2 * blk * C * C
                v[base:base + C * C] = rng.uniform(2.5, 3.5, C * C)
                v[base + C * C:base + 2 * C * C] = rng.uniform(1.5, 2.5, C * C)
        elif name == "radial_coeffs":
            v = radial_scale * rng.uniform(-0.5, 0.5, (F, B + C))
            v[:, B:] = rng.uniform(0.5, 1.5, (F, C))
            v = v.reshape(-1)
        elif name == "two_layer_gate_radial_coeffs":
            v = radial_scale * rng.uniform(-0.5, 0.5, size)
        elif name == "two_layer_gate_additive_coeffs":
            v = rng.uniform(0.05, 0.15, size)
        elif name == "two_layer_gate_type_coeffs":
            v = rng.uniform(0.5, 1.5, size)
        elif name == "two_layer_gate_weights":
            Q = size // F
            v = rng.uniform(-1.0, 1.0, size) / Q
        elif name in ("two_layer_gate_k_rank_weights", "outer_k_rank1_weights"):
            v = rng.uniform(-1.0, 1.0, size)
        elif name == "species_coeffs":
            v = np.ones(size)
        elif name == "moment_coeffs":
            v = readout_scale * rng.uniform(-1.0, 1.0, size) / S
        else:  # pragma: no cover - layout and generator are kept in step
            raise KeyError(name)
        parts.append(np.asarray(v, dtype=np.float64).reshape(-1))
    return np.concatenate(parts)


# --------------------------------------------------------------------------------------------
# .cfg text (src/configuration.cpp:429-770 reader, :1093 writer)
# --------------------------------------------------------------------------------------------

def write_cfg(path: str, frames) -> None:
    with open(path, "w") as fh:
        for fr in frames:
            fh.write("BEGIN_CFG\n Size\n    %d\n Supercell\n" % fr.natoms)
            for row in fr.cell:
                fh.write("    %.17g %.17g %.17g\n" % tuple(row))
            has_f = fr.forces is not None
            fh.write(" AtomData:  id type cartes_x cartes_y cartes_z%s\n" % (" fx fy fz" if has_f else ""))
            for i in range(fr.natoms):
                p = fr.positions[i]
                line = "  %d %d %.17g %.17g %.17g" % (i + 1, fr.types[i], p[0], p[1], p[2])
                if has_f:
                    line += " %.17g %.17g %.17g" % tuple(fr.forces[i])
                fh.write(line + "\n")
            if fr.energy is not None:
                fh.write(" Energy\n    %.17g\n" % fr.energy)
            if fr.stress is not None:
                s = np.asarray(fr.stress)
                fh.write(" PlusStress:  xx yy zz yz xz xy\n    %.17g %.17g %.17g %.17g %.17g %.17g\n"
                         % (s[0, 0], s[1, 1], s[2, 2], s[1, 2], s[0, 2], s[0, 1]))
            fh.write("END_CFG\n\n")


def read_cfg(path: str):
    frames = []
    with open(path) as fh:
        lines = fh.read().splitlines()
    i = 0
    while i < len(lines):
        if lines[i].strip() != "BEGIN_CFG":
            i += 1
            continue
        n = 0
        cell = np.eye(3) * 1e3
        pos = types = forces = None
        energy = stress = None
        i += 1
        while lines[i].strip() != "END_CFG":
            t = lines[i].strip()
            if t == "Size":
                n = int(lines[i + 1]); i += 2; continue
            if t == "Supercell":
                cell = np.array([[float(x) for x in lines[i + k].split()] for k in (1, 2, 3)]); i += 4; continue
            if t.startswith("AtomData:"):
                keys = t.split(":", 1)[1].split()
                rows = np.array([[float(x) for x in lines[i + 1 + k].split()] for k in range(n)])
                types = rows[:, keys.index("type")].astype(np.int32)
                pos = rows[:, [keys.index("cartes_" + a) for a in "xyz"]]
                if "fx" in keys:
                    forces = rows[:, [keys.index(a) for a in ("fx", "fy", "fz")]]
                i += 1 + n; continue
            if t == "Energy":
                energy = float(lines[i + 1]); i += 2; continue
            if t.startswith("PlusStress:"):
                v = [float(x) for x in lines[i + 1].split()]
                xx, yy, zz, yz, xz, xy = v
                stress = np.array([[xx, xy, xz], [xy, yy, yz], [xz, yz, zz]]); i += 2; continue
            i += 1
        frames.append(Frame(cell, pos, types, energy, forces, stress))
        i += 1
    return frames
