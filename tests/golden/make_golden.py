#!/usr/bin/env python3
"""Regenerate the committed golden fixtures from the reference implementation.

Runs only where the reference checkout and its oracle builds exist
(``make -C oracle ref REF=<reference>`` then ``make -C oracle _ref/ref-grad``).
Everything it writes lands under ``tests/golden/``; the tests and the GPU
checks read those files and never the reference itself.

Outputs
  two_cutoff/        the reference's own FP64 two-cutoff fixtures, copied byte for byte
                     (interfaces/lammps/tests/fixtures/two_cutoff/{fixtures_v2,fixtures_hi_l})
  models/*.sus2      benchmark topologies written by the reference's ``init-sh`` (grouped YAML
                     front end, src/mlp/grouped_input.cpp) with seeded parameters
                     (superlinear_gb300.synth.random_vector) and checked to load back
                     bit-exactly through the reference trainer
  frames/*.cfg       seeded geometries
  efs/*.json         E / F / virial / site energies from the reference embedded engine
                     (interfaces/lammps/tests/embedded_efs.cpp, one domain)
  grad/*.json        dTheta of sum_i eW_i E_i + sum_e w_e . dE/dd_e from the reference trainer's
                     AccumulateEFSCombinationGrad (src/basic_mlip.cpp:421, dev_src/mtpr.cpp:9188)
                     for seeded random weights, plus the trainer's own CalcEFS
"""
from __future__ import annotations

import argparse
import hashlib
import json
import os
import shutil
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

from superlinear_gb300.sus2_format import read_sus2, write_sus2  # noqa: E402
from superlinear_gb300.synth import (diamond, fields_to_vector, random_vector,  # noqa: E402
                                     training_frames, vector_to_fields, write_cfg, lattice_frame)

# (name, yaml model block, (parameter seed, radial scale, readout scale))
MODELS = {
    "static_l3k4o2": ("static-radial", dict(elements="[C]", l_max=3, radial_channels=4, neighbor_cutoff=5.0,
                      interaction=dict(channels=2, body_order=4, channel_coupling="cross")), (11, 3.0, 5.0)),
    "effect_l3k4r2o2": ("coordination-effect", dict(species_count=2, l_max=3, radial_channels=4, neighbor_cutoff=5.0,
                        coordination=dict(channels=2, body_order=4, channel_coupling="cross"),
                        interaction=dict(channels=2, body_order=4, channel_coupling="diagonal")), (12, 5.0, 8.0)),
    "effect_l4k8r2o3": ("coordination-effect", dict(species_count=2, l_max=4, radial_channels=8, neighbor_cutoff=5.5,
                        coordination=dict(channels=2, body_order=4, channel_coupling="cross"),
                        interaction=dict(channels=3, body_order=4, channel_coupling="diagonal")), (13, 3.0, 8.0)),
    # small two-species Static model used by the fast tests
    "static_l2k3o2_c2": ("static-radial", dict(species_count=2, l_max=2, radial_channels=3, neighbor_cutoff=4.5,
                         interaction=dict(channels=2, body_order=4, channel_coupling="cross")), (14, 5.0, 20.0)),
}


def yaml_for(kind, spec, out):
    lines = ["schema_version: 1", "model:", f"  kind: {kind}"]
    for key in ("elements", "species_count", "l_max", "radial_channels", "neighbor_cutoff"):
        if key in spec:
            lines.append(f"  {key}: {spec[key]}")
    lines += ["  radial:", "    basis: chebyshev-sss", "    basis_size: 8", "    warp_sharing: K"]
    for group in ("coordination", "interaction"):
        if group in spec:
            lines.append(f"  {group}:")
            lines += [f"    {k}: {v}" for k, v in spec[group].items()]
    lines += ["  readout:", "    element_mode: per-element", "output:", f"  model: {out}"]
    return "\n".join(lines) + "\n"


def run(cmd, **kw):
    r = subprocess.run(cmd, capture_output=True, text=True, **kw)
    if r.returncode:
        raise RuntimeError(f"{cmd[0]} failed: {r.stderr[-2000:]}")
    return r.stdout


def frames_for(name):
    """Seeded geometries per model: (label, [frames])."""
    if name == "static_l3k4o2":
        return [("diamond64_s05", [diamond(2, sigma=0.05, seed=101)]),
                ("diamond64_s15", [diamond(2, sigma=0.15, seed=102)])]
    if name == "static_l2k3o2_c2":
        rng = np.random.default_rng(103)
        return [("mixed", [lattice_frame("fcc", (2, 2, 1), 3.4, 0.12, rng, type_prob=0.5, species=2),
                           lattice_frame("bcc", (2, 2, 2), 2.9, 0.12, rng, type_prob=0.5, species=2)])]
    if name == "effect_l3k4r2o2":
        return [("train4", training_frames(4, 8, 64, 3.0, 4.2, 0.1, seed=104, species=2))]
    if name == "effect_l4k8r2o3":
        return [("diamond64_c2", [diamond(2, sigma=0.1, seed=105, species=2, type_prob=0.5)])]
    raise KeyError(name)


# (model, frame set) of the descriptor goldens
DESC_CASES = (("static_l3k4o2", "diamond64_s05"), ("static_l2k3o2_c2", "mixed"), ("effect_l3k4r2o2", "train4"))

# (model, radial_cutoff_p): polynomial-envelope variants (sus2_sl_radial_math.cpp:256-294)
POLY_VARIANTS = (("static_l2k3o2_c2", 5), ("effect_l3k4r2o2", 3))


def LOSS_CASES():
    """(model, frames to label, (wE, wF, wS)); loss weights of the reference's example profile."""
    return [("effect_l3k4r2o2", training_frames(6, 8, 64, 3.0, 4.2, 0.1, seed=211, species=2), (1.0, 0.01, 0.001)),
            ("static_l2k3o2_c2", training_frames(4, 8, 48, 3.0, 4.2, 0.1, seed=212, species=2), (1.0, 0.01, 0.001))]


def weights_for(frames, seed):
    """Seeded loss-derivative weights (per-atom energy weight, per-atom force weight, 3x3 stress)."""
    rng = np.random.default_rng(seed)
    out = []
    for fr in frames:
        n = fr.natoms
        ew = np.full(n, rng.uniform(0.5, 1.5))
        fw = rng.normal(0, 1.0, (n, 3))
        sw = rng.normal(0, 0.2, (3, 3))
        out.append((ew, fw, sw))
    return out


def golden_efs_and_grad(name, model, frame_sets, seed, tmp, emb, refgrad):
    """E/F/virial goldens (reference embedded engine, one frame at a time) and parameter-gradient
    goldens (reference trainer, seeded weights) of one model over its labelled frame sets."""
    for label, frames in frame_sets:
        cfg = os.path.join(HERE, "frames", f"{name}__{label}.cfg")
        write_cfg(cfg, frames)
        # 3. embedded engine E/F/virial, one frame at a time
        records = []
        for k, fr in enumerate(frames):
            one = os.path.join(tmp, "one.cfg")
            write_cfg(one, [fr])
            out = run([emb, model, one, "1", "direct"])
            line = next(l for l in out.splitlines() if l.startswith("NATIVE_EFS_JSON"))
            rec = json.loads(line.split(" ", 1)[1])
            rec["config"] = k
            records.append(rec)
        with open(os.path.join(HERE, "efs", f"{name}__{label}.json"), "w") as fh:
            json.dump({"model": f"{name}.sus2", "frames": f"{name}__{label}.cfg",
                       "source": "reference embedded engine (embedded_efs.cpp, domains=1, direct)",
                       "records": records}, fh)
        # 4. trainer gradient for seeded weights
        wts = weights_for(frames, seed + 1000)
        wfile = os.path.join(tmp, "w.txt")
        with open(wfile, "w") as fh:
            for ew, fw, sw in wts:
                fh.write(f"{len(ew)}\n")
                for i in range(len(ew)):
                    fh.write("%.17g %.17g %.17g %.17g\n" % (ew[i], *fw[i]))
                for row in sw:
                    fh.write("%.17g %.17g %.17g\n" % tuple(row))
        lines = [json.loads(l) for l in run([refgrad, model, cfg, wfile]).splitlines()]
        efs = [l for l in lines if "energy" in l]
        grads = [l["grad"] for l in lines if "grad" in l]
        with open(os.path.join(HERE, "grad", f"{name}__{label}.json"), "w") as fh:
            json.dump({"model": f"{name}.sus2", "frames": f"{name}__{label}.cfg",
                       "source": "reference trainer MLMTPR::CalcEFS + AccumulateEFSCombinationGrad",
                       "weights": [{"energy": ew.tolist(), "force": fw.tolist(), "stress": sw.tolist()}
                                   for ew, fw, sw in wts],
                       "trainer_efs": efs, "grad": grads}, fh)
        print(name, label, "frames", len(frames), "atoms", [f.natoms for f in frames])


def main():
    ap = argparse.ArgumentParser(description=__doc__)
    ap.add_argument("--reference", default=os.environ.get("SUS2_REFERENCE", os.path.join(os.path.dirname(os.path.abspath(__file__)), "..", "..", "..", "reference")))
    ap.add_argument("--oracle", default=os.path.join(REPO, "oracle", "_ref"))
    ap.add_argument("--rescale-only", action="store_true", help="only regenerate the rescale-step goldens")
    ap.add_argument("--config5-only", action="store_true", help="only regenerate the L5 (config 5) model")
    ap.add_argument("--bfgs-only", action="store_true", help="only regenerate the BFGS trial goldens")
    args = ap.parse_args()
    emb = os.path.join(args.oracle, "embedded-efs")
    mlp = os.path.join(args.oracle, "mlp-sus2")
    refgrad = os.path.join(args.oracle, "ref-grad")
    for tool in (emb, mlp, refgrad):
        if not os.path.exists(tool):
            sys.exit(f"missing {tool}: build it with make -C oracle ref _ref/ref-grad")
    if args.rescale_only:
        golden_rescale(refgrad)
        return
    if args.config5_only:
        golden_config5(mlp)
        return
    if args.bfgs_only:
        golden_bfgs(refgrad)
        return

    # 1. the reference's own golden fixtures
    src = os.path.join(args.reference, "interfaces/lammps/tests/fixtures/two_cutoff")
    dst = os.path.join(HERE, "two_cutoff")
    manifest = {}
    for sub in ("fixtures_v2", "fixtures_hi_l"):
        os.makedirs(os.path.join(dst, sub), exist_ok=True)
        for fn in sorted(os.listdir(os.path.join(src, sub))):
            if fn.startswith("adaptive"):
                continue  # Adaptive family is outside this path
            shutil.copyfile(os.path.join(src, sub, fn), os.path.join(dst, sub, fn))
            manifest[f"{sub}/{fn}"] = hashlib.sha256(open(os.path.join(dst, sub, fn), "rb").read()).hexdigest()

    for sub in ("models", "frames", "efs", "grad"):
        os.makedirs(os.path.join(HERE, sub), exist_ok=True)

    with tempfile.TemporaryDirectory() as tmp:
        for name, (kind, spec, (seed, rscale, oscale)) in MODELS.items():
            ypath = os.path.join(tmp, f"{name}.yaml")
            topo = os.path.join(tmp, f"{name}.sus2")
            with open(ypath, "w") as fh:
                fh.write(yaml_for(kind, spec, f"{name}.sus2"))
            run([mlp, "init-sh", ypath], cwd=tmp)
            # 2. parameters: reference Save of the topology, then our seeded vector, then verify
            fields = read_sus2(topo)
            vec = random_vector(fields, seed, rscale, oscale)
            vfile = os.path.join(tmp, "v.txt")
            np.savetxt(vfile, vec)
            saved = os.path.join(tmp, f"{name}_saved.sus2")
            run([refgrad, "--write", topo, saved, vfile])
            fields = read_sus2(saved)
            vector_to_fields(fields, vec)
            model = os.path.join(HERE, "models", f"{name}.sus2")
            write_sus2(model, fields)
            back = json.loads(run([refgrad, model, "/dev/null"]).splitlines()[0])["coeffs"]
            assert np.array_equal(np.asarray(back), vec), f"{name}: reference did not load the written vector"
            assert np.array_equal(fields_to_vector(read_sus2(model)), vec)
            manifest[f"models/{name}.sus2"] = hashlib.sha256(open(model, "rb").read()).hexdigest()

            golden_efs_and_grad(name, model, frames_for(name), seed, tmp, emb, refgrad)
        # 4b. polynomial radial cutoff (radial_cutoff_type = polynomial): variants of two models
        for base, p in POLY_VARIANTS:
            seed = MODELS[base][2][0]
            src = os.path.join(HERE, "models", f"{base}.sus2")
            name = f"{base}_poly{p}"
            model = os.path.join(HERE, "models", f"{name}.sus2")
            with open(src) as fh:
                text = fh.read()
            head, sep, rest = text.partition("radial_basis_size = ")
            line, nl, tail = rest.partition("\n")
            with open(model, "w") as fh:
                fh.write(head + sep + line + nl + f"\tradial_cutoff_type = polynomial\n\tradial_cutoff_p = {p}\n" + tail)
            back = json.loads(run([refgrad, model, "/dev/null"]).splitlines()[0])["coeffs"]
            assert np.array_equal(np.asarray(back), fields_to_vector(read_sus2(src))), f"{name}: reference load"
            manifest[f"models/{name}.sus2"] = hashlib.sha256(open(model, "rb").read()).hexdigest()
            golden_efs_and_grad(name, model, [(l, f) for l, f in frames_for(base)], seed, tmp, emb, refgrad)
        # 4c. per-atom descriptors (the S scalar moments) from the reference trainer's calc-descriptors
        os.makedirs(os.path.join(HERE, "desc"), exist_ok=True)
        for name, label in DESC_CASES:
            model = os.path.join(HERE, "models", f"{name}.sus2")
            cfg = os.path.join(HERE, "frames", f"{name}__{label}.cfg")
            out = os.path.join(tmp, "desc.txt")
            run([mlp, "calc-descriptors", model, cfg, out], cwd=tmp)
            types, values = [], []
            with open(out) as fh:
                for line in fh:
                    if line.startswith("#") or not line.strip():
                        continue
                    row = line.split()
                    types.append(int(row[0]))
                    values.append([float(x) for x in row[1:]])
            with open(os.path.join(HERE, "desc", f"{name}__{label}.json"), "w") as fh:
                json.dump({"model": f"{name}.sus2", "frames": f"{name}__{label}.cfg",
                           "source": "reference trainer calc-descriptors (MLMTPR::CalcDescriptors), 16 digits",
                           "types": types, "descriptors": values}, fh)
        # 5. labelled training sets: teacher labels (another seeded parameter vector, evaluated by the
        #    reference embedded engine), student loss + gradient from the reference trainer's
        #    NonLinearRegression::CalcObjectiveFunctionGrad (energy / force / stress MSE terms; for
        #    Effect models also with the gate-x L2 regulariser at its default 1e-4)
        os.makedirs(os.path.join(HERE, "loss"), exist_ok=True)
        for name, frames, weights in LOSS_CASES():
            kind, spec, (seed, rscale, oscale) = MODELS[name]
            model = os.path.join(HERE, "models", f"{name}.sus2")
            teacher = os.path.join(tmp, f"{name}_teacher.sus2")
            fields = read_sus2(model)
            vector_to_fields(fields, random_vector(fields, seed + 500, rscale, oscale))
            write_sus2(teacher, fields)
            for fr in frames:
                one = os.path.join(tmp, "one.cfg")
                write_cfg(one, [fr])
                out = run([emb, teacher, one, "1", "direct"])
                rec = json.loads(next(l for l in out.splitlines() if l.startswith("NATIVE_EFS_JSON")).split(" ", 1)[1])
                fr.energy = rec["energy"]
                fr.forces = np.asarray(rec["forces"])
                fr.stress = np.asarray(rec["virial"])
            cfg = os.path.join(HERE, "frames", f"{name}__labelled.cfg")
            write_cfg(cfg, frames)
            # the MSE terms alone, and (Effect) with the reference's default gate-x L2 coefficient
            cases = [(w, 0.0, "") for w in ("vibrations", "structures")]
            if kind == "coordination-effect":
                cases += [(w, 1e-4, "__gatex") for w in ("vibrations", "structures")]
            for weighting, gx, tag in cases:
                res = json.loads(run([refgrad, "--loss", model, cfg, *(str(w) for w in weights), weighting, repr(gx)]))
                with open(os.path.join(HERE, "loss", f"{name}__{weighting}{tag}.json"), "w") as fh:
                    json.dump({"model": f"{name}.sus2", "frames": f"{name}__labelled.cfg", "weights": weights,
                               "weighting": weighting, "gate_x_l2": gx,
                               "source": "reference NonLinearRegression::CalcObjectiveFunctionGrad (summed over configs)",
                               "loss": res["loss"], "grad": res["grad"], "configs": res["configs"],
                               "metrics": dict(zip(("energy_mae_mev_per_atom", "energy_rmse_mev_per_atom",
                                                    "force_mae_mev_per_a", "force_rmse_mev_per_a", "stress_mae_ev",
                                                    "stress_rmse_ev"), res["metrics"]))}, fh)
            print(name, "labelled frames", len(frames))
    # 6. linear warm-up: MTPR_trainer::TrainLinear on the labelled sets
    os.makedirs(os.path.join(HERE, "linear"), exist_ok=True)
    for name, _, weights in LOSS_CASES():
        model = os.path.join(HERE, "models", f"{name}.sus2")
        cfg = os.path.join(HERE, "frames", f"{name}__labelled.cfg")
        res = json.loads(run([refgrad, "--linear", model, cfg, *(str(w) for w in weights)]))
        with open(os.path.join(HERE, "linear", f"{name}__labelled.json"), "w") as fh:
            json.dump({"model": f"{name}.sus2", "frames": f"{name}__labelled.cfg", "weights": weights,
                       "weighting": "vibrations", "source": "reference MTPR_trainer::TrainLinear",
                       "coeffs": res["coeffs"], "configs": res["configs"]}, fh)
    golden_rescale(refgrad)
    golden_bfgs(refgrad)
    golden_config5(mlp)
    with open(os.path.join(HERE, "manifest.json"), "w") as fh:
        json.dump(manifest, fh, indent=1, sort_keys=True)


# Config 5 topology: Effect L5/K8/R2/O2, three species.  The reference's init-sh writes it, but its
# model loader rejects sh_l_max > 4, so the seeded parameters are written with this package's
# writer (no reference round trip) and the L5 evaluations have no reference values: GPU and oracle
# are checked against each other and against finite differences.
CONFIG5 = ("effect_l5k8r2o2_c3", "coordination-effect",
           dict(species_count=3, l_max=5, radial_channels=8, neighbor_cutoff=5.0,
                coordination=dict(channels=2, body_order=4, channel_coupling="cross"),
                interaction=dict(channels=2, body_order=4, channel_coupling="diagonal")), (15, 3.0, 8.0))


def golden_config5(mlp):
    name, kind, spec, (seed, rscale, oscale) = CONFIG5
    with tempfile.TemporaryDirectory() as tmp:
        ypath = os.path.join(tmp, f"{name}.yaml")
        with open(ypath, "w") as fh:
            fh.write(yaml_for(kind, spec, f"{name}.sus2"))
        run([mlp, "init-sh", ypath], cwd=tmp)
        fields = read_sus2(os.path.join(tmp, f"{name}.sus2"))
        vec = random_vector(fields, seed, rscale, oscale)
        vector_to_fields(fields, vec)
        model = os.path.join(HERE, "models", f"{name}.sus2")
        write_sus2(model, fields)
        assert np.array_equal(fields_to_vector(read_sus2(model)), vec)
    print(name, "written (init-sh topology, seeded parameters)")


def golden_rescale(refgrad):
    """7. rescale step: the reference trainer's Rescale (scaling search around TrainLinear) on the
    labelled sets (the Effect set has six frames, so its five-frame subset is exercised)."""
    for name, _, weights in LOSS_CASES():
        model = os.path.join(HERE, "models", f"{name}.sus2")
        cfg = os.path.join(HERE, "frames", f"{name}__labelled.cfg")
        res = json.loads(run([refgrad, "--rescale", model, cfg, *(str(w) for w in weights)]))
        with open(os.path.join(HERE, "linear", f"{name}__rescale.json"), "w") as fh:
            json.dump({"model": f"{name}.sus2", "frames": f"{name}__labelled.cfg", "weights": weights,
                       "weighting": "vibrations", "source": "reference Rescale (dev_src/mlp/mtpr_train.cpp)",
                       "scaling": res["scaling"], "coeffs": res["coeffs"], "configs": res["configs"]}, fh)


BFGS_CASES = (("static_l2k3o2_c2", 0.1), ("effect_l3k4r2o2", 0.1))


def golden_bfgs(refgrad, iters=5):
    """8. BFGS: the reference's BFGS engine (BFGS::Iterate / Linesearch::Iterate / UpdateInvHess,
    src/common/bfgs.{h,cpp}) over the raw parameter vector on the trainer objective of each labelled
    set, from the model's parameters and a constant initial inverse-Hessian diagonal; every trial
    point, its objective value and whether BFGS accepted it, up to `iters` accepted steps."""
    os.makedirs(os.path.join(HERE, "bfgs"), exist_ok=True)
    weights = {name: w for name, _, w in LOSS_CASES()}
    with tempfile.TemporaryDirectory() as tmp:
        for name, diag in BFGS_CASES:
            model = os.path.join(HERE, "models", f"{name}.sus2")
            cfg = os.path.join(HERE, "frames", f"{name}__labelled.cfg")
            n = len(json.loads(run([refgrad, model, "/dev/null"]).splitlines()[0])["coeffs"])
            dfile = os.path.join(tmp, "diag.txt")
            np.savetxt(dfile, np.full(n, diag))
            out = run([refgrad, "--bfgs", model, cfg, *(str(w) for w in weights[name]), "vibrations", str(iters), dfile])
            trials = [json.loads(line) for line in out.splitlines() if line.strip()]
            assert sum(t["accepted"] for t in trials) == iters + 1, f"{name}: BFGS stopped early"
            with open(os.path.join(HERE, "bfgs", f"{name}__labelled.json"), "w") as fh:
                json.dump({"model": f"{name}.sus2", "frames": f"{name}__labelled.cfg", "weights": weights[name],
                           "weighting": "vibrations", "inv_hess_diagonal": diag, "iterations": iters,
                           "source": "reference BFGS engine (src/common/bfgs.{h,cpp}) driven by ref-grad --bfgs",
                           "trials": [{"f": t["f"], "accepted": t["accepted"], "x": t["x"]} for t in trials]}, fh)
            print(name, "bfgs trials", len(trials))


if __name__ == "__main__":
    main()
