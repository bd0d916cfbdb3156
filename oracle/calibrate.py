"""Speed of the CPU restatement against the reference's own engine, one thread each (test tooling).

The GPU machine receives neither the reference's sources nor binaries built from them, so the
benchmark's CPU arm times the restatement (oracle/sus2_oracle.cpp).  This script measures, where
the reference checkout was compiled (oracle/_ref/ref-time, `make -C oracle _ref/ref-time`), how
the restatement's per-evaluation time compares with the reference's SUS2SL::Kernel
begin / outer / finish on the same edge list, and prints one JSON line per workload:

  python oracle/calibrate.py [--effect]

Workloads: the 4,096-atom Static L3/K4/O2 diamond (8x8x8 cells, sigma 0.08 A) and, with --effect,
the 110,592-atom Effect L4/K8/R2/O3 diamond (24x24x24 cells, sigma 0.1 A, two species 50/50).
Both boxes are cubic and wider than twice the cutoff, so the minimum-image edge list is the full
edge set.  Edge building is excluded on both sides.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)


def min_image_edges(frame, cutoff):
    """Directed edges (i, j, d = x_j - x_i) of a cubic box wider than 2 cutoff, sorted by centre."""
    from scipy.spatial import cKDTree
    L = float(frame.cell[0, 0])
    x = np.mod(frame.positions, L)
    pairs = cKDTree(x, boxsize=L).query_pairs(cutoff, output_type="ndarray")
    i = np.concatenate([pairs[:, 0], pairs[:, 1]])
    j = np.concatenate([pairs[:, 1], pairs[:, 0]])
    d = frame.positions[j] - frame.positions[i]
    d -= L * np.round(d / L)
    keep = np.einsum("ij,ij->i", d, d) < cutoff * cutoff
    i, j, d = i[keep], j[keep], d[keep]
    order = np.lexsort((j, i))
    return i[order].astype(np.int32), j[order].astype(np.int32), np.ascontiguousarray(d[order])


def write_edges(path, types, i, j, d):
    rec = np.zeros(i.size, dtype=[("i", "<i4"), ("j", "<i4"), ("d", "<f8", 3)])
    rec["i"], rec["j"], rec["d"] = i, j, d
    with open(path, "wb") as fh:
        fh.write(np.int32(types.size).tobytes())
        fh.write(np.ascontiguousarray(types, dtype="<i4").tobytes())
        fh.write(np.int64(i.size).tobytes())
        fh.write(rec.tobytes())


def calibrate(name, model_path, frame, cutoff, reps):
    import oracle as orc
    tool = os.path.join(HERE, "_ref", "ref-time")
    if not os.path.exists(tool):
        sys.exit(f"missing {tool}: build it with make -C oracle _ref/ref-time")
    i, j, d = min_image_edges(frame, cutoff)
    with tempfile.TemporaryDirectory() as tmp:
        path = os.path.join(tmp, "edges.bin")
        write_edges(path, frame.types, i, j, d)
        out = subprocess.run([tool, model_path, path, str(reps)], capture_output=True, text=True, check=True)
    ref = json.loads(out.stdout.strip().splitlines()[-1])
    m = orc.OracleModel(model_path)
    port = []
    energy = None
    for _ in range(reps):
        energy, ne, _, tc = m.efs_timed(frame.cell, frame.positions, frame.types, threads=1)
        port.append(tc)
    return {"workload": name, "atoms": frame.natoms, "edges": int(i.size), "oracle_edges": ne, "threads": 1,
            "reference_s": ref["seconds_mean"], "port_s": float(np.mean(port)),
            "port_over_reference_speed": ref["seconds_mean"] / float(np.mean(port)),
            "energy_reference": ref["energy"], "energy_port": energy}


def main():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--effect", action="store_true", help="also the 110,592-atom Effect L4/K8/R2/O3 box")
    ap.add_argument("--reps", type=int, default=3)
    args = ap.parse_args()
    from superlinear_gb300.synth import diamond
    models = os.path.join(ROOT, "tests", "golden", "models")
    print(json.dumps(calibrate("static_l3k4o2_diamond4096", os.path.join(models, "static_l3k4o2.sus2"),
                               diamond(8, a=3.567, sigma=0.08, seed=2), 5.0, args.reps)), flush=True)
    if args.effect:
        fr = diamond(24, a=3.567, sigma=0.1, seed=4, species=2, type_prob=0.5)
        print(json.dumps(calibrate("effect_l4k8r2o3_diamond110592", os.path.join(models, "effect_l4k8r2o3.sus2"),
                                   fr, 5.5, 1)), flush=True)


if __name__ == "__main__":
    main()
