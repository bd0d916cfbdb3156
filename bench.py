#!/usr/bin/env python3
"""Benchmark of the SUS2-SH E / F / virial hot path on one GB300 (one JSON line on stdout).

Workload (the configuration the headline metric is quoted on): Static L3/K4/O2 carbon model,
4,096-atom periodic diamond (8x8x8 conventional cells, a = 3.567 A, seeded Gaussian
displacements sigma = 0.08 A), cutoff 5.0 A.  One step = one MD-step evaluation: build the
directed edge list from positions on the GPU, then energy, forces and virial (FP32 bulk with
FP64 reductions; the FP64 plain path is timed alongside).  Repeated steps of the unchanged layout
replay one CUDA graph of the whole step, as in an MD run; the per-stage times come from separate
eager steps under the stage timer.  The inputs are smaller than L2, so L2 is flushed (a 256 MiB
write) between timed steps, outside the step's events.

The training loss + gradient throughput (frames/s, FP32 bulk vs FP64 plain) over a batch of 256
uneven Effect L3/K4/R2/O2 frames is reported alongside under "train_effect_l3k4r2o2_256", and the
same for 2,048 Effect L5/K8/R2/O2 frames with three species (sizes log-uniform in [16, 512], plus
timed BFGS iterations) under "train_effect_l5k8r2o2_2048".

--impl reference times the CPU reference path on the host cores instead: the FP64 CPU
restatement of the reference algorithm (the reference's own sources do not travel to the GPU
machine), all host threads, E/F/virial per step on the same frame.

Multi-GPU: the path runs on one GPU; with --gpus N each rank runs an independent replica of the
same workload (replicas only, no collective) and rank 0 reports the sum of rank throughputs
timed as max over ranks.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

METRIC = "atom-steps/s E/F/virial; train loss+grad frames/s; FP32-bulk vs FP64, 1 GB300"
MODEL = os.path.join(ROOT, "tests", "golden", "models", "static_l3k4o2.sus2")
EFFECT_MODEL = os.path.join(ROOT, "tests", "golden", "models", "effect_l4k8r2o3.sus2")
TRAIN_MODEL = os.path.join(ROOT, "tests", "golden", "models", "effect_l3k4r2o2.sus2")
C5_MODEL = os.path.join(ROOT, "tests", "golden", "models", "effect_l5k8r2o2_c3.sus2")
TRAIN_WEIGHTS = (1.0, 0.01, 0.001)  # energy + force + stress MSE (the example training profile's weights)
PEAKS = os.path.join(ROOT, "MEASURED_PEAKS.json")
TRAFFIC = os.path.join(ROOT, "profiles", "dram_traffic.txt")


def workload(cells: int = 8):
    from superlinear_gb300.synth import diamond
    return diamond(cells, a=3.567, sigma=0.08, seed=2)


# ------------------------------------------------------------------------------------------------
# algorithmic flop model (per edge and per atom), counting FMA as 2 and tanh / sqrt / div as 1
# ------------------------------------------------------------------------------------------------
def pass_flops(d, edges, atoms):
    """Forward + reverse of one per-atom pass (Static outer pass, or each Effect pass)."""
    H = (d["L"] + 1) ** 2
    K, B, F, NB = d["K"], d["B"], d["F"], d["NB"]
    nblk = K  # warp sharing K in the benchmark models
    fwd = 6 + 12 * H + nblk * (3 * B + 10) + 2 * F * B + 4 * NB
    rev = 6 + 42 * H + nblk * (7 * B + 15) + 4 * F * B + 24 * NB + 18
    per_atom = 2 * 4 * max(d["outer_rank"], 1) * H * K + 9 * d["P"] + 4 * d["S"]
    return edges * (fwd + rev) + atoms * per_atom


def algorithmic_bytes(d, edges, atoms, real_bytes=4):
    """Bytes one Static pass must move: per edge the neighbour index, the edge record (d, r) and
    the written dE/dd; per atom the type, row offsets, site energy and virial."""
    return edges * (4 + 4 * real_bytes + 3 * real_bytes) + atoms * (4 + 4 + 8 + 48)


# ------------------------------------------------------------------------------------------------
class NvmlClocks:
    """Read-only NVML queries through ctypes (SM clock, max SM clock, power, clock-event reasons)."""

    REASONS = {0x4: "sw_power_cap", 0x8: "hw_slowdown", 0x20: "sw_thermal_slowdown", 0x40: "hw_thermal_slowdown",
               0x80: "hw_power_brake_slowdown"}

    def __init__(self, index: int):
        import ctypes
        self.c = ctypes
        self.lib = ctypes.CDLL("libnvidia-ml.so.1")
        if self.lib.nvmlInit_v2() != 0:
            raise OSError("nvmlInit failed")
        self.h = ctypes.c_void_p()
        found = False
        try:  # the CUDA device's UUID, robust to a remapped device order
            import torch
            uuid = "GPU-" + str(torch.cuda.get_device_properties(index).uuid)
            found = self.lib.nvmlDeviceGetHandleByUUID(uuid.encode(), ctypes.byref(self.h)) == 0
        except Exception:
            found = False
        if not found and self.lib.nvmlDeviceGetHandleByIndex_v2(ctypes.c_uint(index), ctypes.byref(self.h)) != 0:
            raise OSError("no NVML device")
        self.reasons_fn = getattr(self.lib, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
            self.lib.nvmlDeviceGetCurrentClocksThrottleReasons

    def sample(self):
        c = self.c
        sm, mx, pw, rs = c.c_uint(), c.c_uint(), c.c_uint(), c.c_ulonglong()
        self.lib.nvmlDeviceGetClockInfo(self.h, 1, c.byref(sm))       # NVML_CLOCK_SM
        self.lib.nvmlDeviceGetMaxClockInfo(self.h, 1, c.byref(mx))
        self.lib.nvmlDeviceGetPowerUsage(self.h, c.byref(pw))
        self.reasons_fn(self.h, c.byref(rs))
        return sm.value, mx.value, pw.value / 1000.0, rs.value


class ClockSampler:
    """SM clocks / clock-event reasons sampled during the timed region: NVML every ~2 ms (plus one
    sample at start and stop), or nvidia-smi every 200 ms when NVML cannot be loaded."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.rows = []      # (sm_mhz, max_mhz, reasons set)
        self.proc = None
        self.nvml = None
        self.stop_flag = threading.Event()
        try:
            self.nvml = NvmlClocks(device)
        except (OSError, AttributeError):
            self.nvml = None

    def _nvml_row(self):
        sm, mx, _, bits = self.nvml.sample()
        return sm, mx, {name for bit, name in NvmlClocks.REASONS.items() if bits & bit}

    def _poll(self):
        while not self.stop_flag.is_set():
            self.rows.append(self._nvml_row())
            time.sleep(0.002)

    def start(self):
        self.stop_flag.clear()
        if self.nvml is not None:
            self.rows.append(self._nvml_row())
            self.thread = threading.Thread(target=self._poll, daemon=True)
            self.thread.start()
            return
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None

    def _read(self):
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9 and parts[1].replace(".", "").isdigit():
                reasons = {n for n, v in zip(names, parts[5:9]) if v.lower() == "active"}
                self.rows.append((float(parts[1]), float(parts[2]), reasons))

    def stop(self):
        if self.nvml is not None:
            self.stop_flag.set()
            self.thread.join(timeout=2)
            self.rows.append(self._nvml_row())
            source = "nvml"
        elif self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.thread.join(timeout=2)
            source = "nvidia-smi"
        else:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["clock query unavailable"], "samples": 0}
        sm = [r[0] for r in self.rows]
        mx = [r[1] for r in self.rows]
        reasons = set().union(*[r[2] for r in self.rows]) if self.rows else set()
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(self.rows), "source": source}


def dist_info():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def max_over_ranks(values, world, device):
    """Per-rank timings -> their maximum over the ranks (replicas: the job is as slow as its slowest
    rank); every rank receives the result."""
    import torch
    t = torch.tensor(list(values), dtype=torch.float64, device=device)
    if world > 1:
        import torch.distributed as dist
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(x) for x in t.cpu()]


def replica_throughput(units_per_rank, world, ms):
    """Whole-job throughput of `world` replicas that each processed units_per_rank in ms."""
    return units_per_rank * world / (ms / 1e3)


def read_traffic(key):
    """DRAM bytes per launch of the dominant kernel from the committed ncu summary, or None."""
    try:
        with open(TRAFFIC) as fh:
            for line in fh:
                parts = line.split()
                if len(parts) >= 2 and parts[0] == key:
                    return float(parts[1])
    except OSError:
        pass
    return None


# ------------------------------------------------------------------------------------------------
def tune(eng, reps):
    """Runs the pass autotuner on the engine's last layout; returns the chosen tile shape per pass."""
    eng.autotune(reps=reps)
    return eng.pass_shapes()


def training_set(sg, nframes=256, seed=31):
    """256 uneven periodic frames (8-216 atoms, fcc/bcc/diamond, a in [3.0, 4.2] A, sigma 0.1 A,
    types Bernoulli(0.5)) labelled by a seeded random-init teacher of the same Effect L3/K4/R2/O2
    topology (FP64 GPU evaluation, outside any timed region)."""
    from superlinear_gb300.sus2_format import read_sus2
    from superlinear_gb300.synth import random_vector, training_frames
    frames = training_frames(nframes, 8, 216, 3.0, 4.2, 0.1, seed=seed, species=2)
    teacher = sg.Model(TRAIN_MODEL)
    teacher.set_params(random_vector(read_sus2(TRAIN_MODEL), seed + 500, 5.0, 8.0))
    e, f, v, _ = sg.Engine(teacher, 0, sg.FP64).calc_efs(frames)
    a = 0
    for k, fr in enumerate(frames):
        fr.energy = float(e[k])
        fr.forces = f[a:a + fr.natoms].copy()
        xx, yy, zz, xy, xz, yz = v[k]
        fr.stress = np.array([[xx, xy, xz], [xy, yy, yz], [xz, yz, zz]])
        a += fr.natoms
    return frames


def bench_training(sg, torch, steps, warmup):
    """Training loss + gradient frames/s over the 256-frame Effect batch, FP32 bulk and FP64 plain:
    one step = one Trainer.loss_grad (parameter upload, the captured loss+gradient CUDA graph,
    loss and gradient read back to the host), as a BFGS iteration calls it."""
    frames = training_set(sg)
    model = sg.Model(TRAIN_MODEL)
    p = model.params()
    out = {"workload": "effect_l3k4r2o2_train256", "frames": len(frames), "atoms": int(sum(f.natoms for f in frames)),
           "weights": {"energy": TRAIN_WEIGHTS[0], "force": TRAIN_WEIGHTS[1], "stress": TRAIN_WEIGHTS[2]}}
    losses = {}
    for prec, key, nsteps in ((sg.FP32, "fp32", steps), (sg.FP64, "fp64", max(5, steps // 2))):
        eng = sg.Engine(model, 0, prec)
        tr = sg.Trainer(eng, frames, *TRAIN_WEIGHTS, gate_x_l2=0.0)
        tr.loss_grad(p)
        out.setdefault("autotune", {})[key] = tune(eng, 2)
        for _ in range(warmup):
            tr.loss_grad(p)
        torch.cuda.synchronize()
        t = []
        for _ in range(nsteps):
            t0 = time.perf_counter()
            loss, g = tr.loss_grad(p)
            t.append(time.perf_counter() - t0)
        ms = 1e3 * float(np.mean(t))
        losses[key] = (loss, g)
        out[key] = {"ms_per_step": ms, "frames_per_s": len(frames) / (ms / 1e3), "edges": eng.edge_count()}
        del tr, eng
    out["fp32_over_fp64"] = out["fp64"]["ms_per_step"] / out["fp32"]["ms_per_step"]
    (l32, g32), (l64, g64) = losses["fp32"], losses["fp64"]
    out["fp32_error"] = {"loss_rel": abs(l32 - l64) / abs(l64),
                         "grad_rel_norm": float(np.linalg.norm(g32 - g64) / np.linalg.norm(g64))}
    return frames, out


def config5_set(sg, nframes=2048, seed=53):
    """2,048 uneven periodic frames (sizes log-uniform in [16, 512], fcc/bcc/diamond, a in
    [2.8, 4.5] A, sigma 0.15 A, three species uniform) labelled by a teacher of the same Effect
    L5/K8/R2/O2 topology at 2% perturbed parameters (FP64 GPU evaluation, outside any timed region)."""
    from superlinear_gb300.synth import training_frames
    frames = training_frames(nframes, 16, 512, 2.8, 4.5, 0.15, seed=seed, species=3, log_uniform=True)
    teacher = sg.Model(C5_MODEL)
    p0 = teacher.params()
    teacher.set_params(p0 * (1 + 0.02 * np.random.default_rng(seed + 1).normal(size=p0.size)))
    e, f, v, _ = sg.Engine(teacher, 0, sg.FP64).calc_efs(frames)
    a = 0
    for k, fr in enumerate(frames):
        fr.energy = float(e[k])
        fr.forces = f[a:a + fr.natoms].copy()
        xx, yy, zz, xy, xz, yz = v[k]
        fr.stress = np.array([[xx, xy, xz], [xy, yy, yz], [xz, yz, zz]])
        a += fr.natoms
    return frames


def bench_config5(sg, torch, steps, warmup, bfgs_iters, cpu_frames=0):
    """Loss + gradient frames/s over the 2,048-frame L5 batch (FP32 bulk and FP64 plain, one step =
    one Trainer.loss_grad as a BFGS iteration calls it), then bfgs_iters BFGS iterations in FP32
    (each: line-search evaluations through the captured loss+gradient graph and the device-side
    inverse-Hessian update)."""
    frames = config5_set(sg)
    model = sg.Model(C5_MODEL)
    p = model.params()
    out = {"workload": "effect_l5k8r2o2_c3_train2048", "frames": len(frames),
           "atoms": int(sum(f.natoms for f in frames)),
           "weights": {"energy": TRAIN_WEIGHTS[0], "force": TRAIN_WEIGHTS[1], "stress": TRAIN_WEIGHTS[2]}}
    losses = {}
    for prec, key, nw, nsteps in ((sg.FP32, "fp32", warmup, steps), (sg.FP64, "fp64", 1, 2)):
        eng = sg.Engine(model, 0, prec)
        tr = sg.Trainer(eng, frames, *TRAIN_WEIGHTS, gate_x_l2=0.0)
        tr.loss_grad(p)
        if prec == sg.FP32:  # (the FP64 passes of this batch take ~0.8 s each: defaults)
            out.setdefault("autotune", {})[key] = tune(eng, 1)
        for _ in range(nw):
            tr.loss_grad(p)
        torch.cuda.synchronize()
        t = []
        for _ in range(nsteps):
            t0 = time.perf_counter()
            loss, g = tr.loss_grad(p)
            t.append(time.perf_counter() - t0)
        ms = 1e3 * float(np.mean(t))
        losses[key] = (loss, g)
        out[key] = {"ms_per_step": ms, "frames_per_s": len(frames) / (ms / 1e3), "edges": eng.edge_count()}
        if prec == sg.FP32 and bfgs_iters > 0:
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            _, hist = tr.bfgs(p, max_iter=bfgs_iters)
            dt = time.perf_counter() - t0
            nev = int(tr.bfgs_trials()[0].size)
            out["bfgs_fp32"] = {"iterations": int(hist.size - 1), "requested": bfgs_iters, "evaluations": nev,
                                "seconds": dt, "ms_per_iteration": 1e3 * dt / max(1, hist.size - 1),
                                "loss_first": float(hist[0]), "loss_last": float(hist[-1]),
                                "line_search": "reference (Linesearch::Iterate)",
                                "timed_region": "the whole sus2g_trainer_bfgs call from the model's parameters "
                                                "(every objective evaluation, direction and inverse-Hessian update)"}
        del tr, eng
    out["fp32_over_fp64"] = out["fp64"]["ms_per_step"] / out["fp32"]["ms_per_step"]
    (l32, g32), (l64, g64) = losses["fp32"], losses["fp64"]
    out["fp32_error"] = {"loss_rel": abs(l32 - l64) / abs(l64),
                         "grad_rel_norm": float(np.linalg.norm(g32 - g64) / np.linalg.norm(g64))}
    if cpu_frames > 0:
        sample = frames[::max(1, len(frames) // cpu_frames)][:cpu_frames]
        nd, tcpu, nw = cpu_train_parallel(sample, C5_MODEL)
        out["cpu_baseline"] = {"value": nd / tcpu, "unit": "frames/s", "cores": nw, "kind": "port",
                               "sample": f"loss + gradient of {nd} frames (every {max(1, len(frames) // cpu_frames)}"
                                         f"th of the batch, {sum(f.natoms for f in sample)} atoms) by the FP64 CPU "
                                         f"restatement, {nw} processes: {tcpu:.2f} s"}
        out["fp32_over_cpu"] = out["fp32"]["frames_per_s"] / out["cpu_baseline"]["value"]
    return out


def _cpu_train_warm(_):
    import oracle as orc
    orc.lib()
    time.sleep(0.2)  # keeps this worker busy so that the warm-up tasks reach every worker
    return 0


def _cpu_train_chunk(job):
    model_path, frames = job
    import oracle as orc
    orc.loss_grad(orc.OracleModel(model_path), frames, *TRAIN_WEIGHTS)
    return len(frames)


def cpu_train_parallel(frames, model_path, workers=None):
    """Loss + gradient of `frames` by the FP64 CPU restatement in `workers` processes (all host
    cores by default), frames dealt round-robin; returns (frames done, wall seconds).  The pool is
    started with spawn and warmed (library loaded in every worker) outside the timed region."""
    import concurrent.futures as cf
    import multiprocessing as mp
    workers = max(1, min(workers or (os.cpu_count() or 1), len(frames)))
    chunks = [frames[k::workers] for k in range(workers)]
    with cf.ProcessPoolExecutor(workers, mp_context=mp.get_context("spawn")) as ex:
        list(ex.map(_cpu_train_warm, range(workers)))
        t0 = time.perf_counter()
        done = sum(ex.map(_cpu_train_chunk, [(model_path, c) for c in chunks]))
        dt = time.perf_counter() - t0
    return done, dt, workers


def cpu_sample(frame, threads, min_seconds=8.0, max_evals=50):
    """Time the oracle port on the frame: E/F/virial compute per evaluation (edge build reported
    separately), repeated until min_seconds of CPU work."""
    import oracle as orc
    m = orc.OracleModel(MODEL)
    evals, compute, edges_t = 0, 0.0, 0.0
    t0 = time.perf_counter()
    while evals == 0 or (evals < max_evals and (time.perf_counter() - t0) < min_seconds):
        _, ne, te, tc = m.efs_timed(frame.cell, frame.positions, frame.types, threads=threads)
        compute += tc
        edges_t += te
        evals += 1
    return evals, compute, edges_t


def run_reference(args):
    rank, world, _ = dist_info()
    if rank != 0:
        return 0
    import oracle as orc
    orc.build()
    frame = workload()
    threads = os.cpu_count() or 1
    # warmup
    for _ in range(max(0, args.warmup)):
        cpu_sample(frame, threads, min_seconds=0.0, max_evals=1)
    times = []
    edge_times = []
    for _ in range(args.steps):
        n, tc, te = cpu_sample(frame, threads, min_seconds=0.0, max_evals=1)
        times.append(tc)
        edge_times.append(te)
    ms = 1e3 * float(np.mean(times))
    value = frame.natoms / (ms / 1e3)
    line = {
        "metric": METRIC, "value": value, "unit": "atom-steps/s", "impl": "reference", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": "static_l3k4o2_diamond4096", "atoms": frame.natoms, "cutoff": 5.0,
                   "cells": "8x8x8", "sigma": 0.08},
        "cpu_baseline": {"value": value, "unit": "atom-steps/s", "cores": threads, "kind": "port",
                         "sample": f"{args.steps} full E/F/virial evaluations of the 4,096-atom frame; "
                                   f"edge build excluded (mean {1e3 * float(np.mean(edge_times)):.1f} ms, O(N^2) "
                                   f"image scan like the reference's Neighborhoods)"},
        "e2e": {"value": value, "unit": "atom-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def pin_order(eng, order, split=False):
    """Pins every pass of the engine's model to one centre order (default budget and grid), and
    splits the passes when asked."""
    eng.set_static_split(split)
    if order:
        for p in (("gate_forward", "outer", "gate_reverse") if eng.model.dims["gated"] else ("static",)):
            eng.set_pass_shape(p, 0, "resident", order)


def run_profile_train(args):
    """FP32 trainer steps only (for ncu launch lists of the training workload)."""
    import torch

    import superlinear_gb300 as sg
    frames = training_set(sg)
    model = sg.Model(TRAIN_MODEL)
    eng = sg.Engine(model, 0, sg.FP32)
    pin_order(eng, args.order, args.split)
    tr = sg.Trainer(eng, frames, *TRAIN_WEIGHTS, gate_x_l2=0.0)
    tr.set_graph(not args.no_graph)
    p = model.params()
    for _ in range(args.warmup + args.steps):
        loss, _ = tr.loss_grad(p)
    torch.cuda.synchronize()
    print(json.dumps({"profile_train": True, "frames": len(frames), "loss": loss}), flush=True)
    return 0


def run_profile_effect(args):
    """FP32 E/F/virial steps of the Effect L4/K8/R2/O3 model on a diamond of --cells cells per edge
    (24 -> the 110,592-atom configuration; smaller boxes for ncu captures)."""
    import torch

    import superlinear_gb300 as sg
    from superlinear_gb300.synth import diamond
    fr = diamond(args.cells, a=3.567, sigma=0.1, seed=4, species=2, type_prob=0.5)
    dev = torch.device("cuda", 0)
    eng = sg.Engine(sg.Model(EFFECT_MODEL), 0, sg.FP32)
    eng.set_moment_mma(args.moment_mma)
    pin_order(eng, args.order, args.split)
    pos = torch.tensor(fr.positions, device=dev)
    typ = torch.tensor(fr.types, device=dev)
    out = torch.zeros(fr.natoms * 3 + 7, dtype=torch.float64, device=dev)
    args_ = (np.array([fr.natoms], np.int32), fr.cell.reshape(1, 9).copy(), pos.data_ptr(), typ.data_ptr(),
             out.data_ptr(), out.data_ptr() + 8, out.data_ptr() + 8 * (1 + 3 * fr.natoms), 0)
    for _ in range(args.warmup + args.steps):
        eng.calc_efs_device(*args_)
    torch.cuda.synchronize()
    eng.set_timing(True)
    eng.take_stage_times()
    eng.calc_efs_device(*args_)
    stages = {k: v[0] for k, v in eng.take_stage_times().items() if v[1]}
    print(json.dumps({"profile_effect": True, "atoms": fr.natoms, "edges": eng.edge_count(), "stages_ms": stages}),
          flush=True)
    return 0


def run_ours(args):
    import torch

    import superlinear_gb300 as sg
    rank, world, local = dist_info()
    device = local if torch.cuda.device_count() > local else 0
    torch.cuda.set_device(device)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", init_method="env://")
    frame = workload(args.cells)
    n = frame.natoms
    dev = torch.device("cuda", device)
    model = sg.Model(MODEL)
    stream = torch.cuda.current_stream()
    pos = torch.tensor(frame.positions, device=dev)
    typ = torch.tensor(frame.types, device=dev)
    E = torch.zeros(1, dtype=torch.float64, device=dev)
    F = torch.zeros(n, 3, dtype=torch.float64, device=dev)
    V = torch.zeros(1, 6, dtype=torch.float64, device=dev)
    natoms = np.array([n], np.int32)
    cells = frame.cell.reshape(1, 9).copy()
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)

    def make(prec):
        eng = sg.Engine(model, device, prec)
        eng.set_stream(stream.cuda_stream)
        return eng

    def step(eng):
        eng.calc_efs_device(natoms, cells, pos.data_ptr(), typ.data_ptr(), E.data_ptr(), F.data_ptr(), V.data_ptr(), 0)

    def stage_times(eng, steps):
        """Per-stage CUDA-event times of separate steps (the stage timer runs the steps eagerly)."""
        eng.set_timing(True)
        eng.take_stage_times()
        for _ in range(steps):
            flush.fill_(1.0)
            step(eng)
        torch.cuda.synchronize()
        stages = eng.take_stage_times()
        eng.set_timing(False)
        return stages

    def timed(eng, steps, warmup, sampler=None):
        for _ in range(warmup):
            step(eng)
        torch.cuda.synchronize()
        eng.take_launch_count()
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()
        if sampler:
            sampler.start()
        # every timed step between its own event pair, queued back to back behind its L2 flush (not
        # timed) so that host submission does not leave the device idle inside a step; one
        # synchronisation at the end
        marks = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
        for a, b in marks:
            flush.fill_(1.0)  # L2 flush between timed steps (not timed)
            a.record(stream)
            step(eng)
            b.record(stream)
        torch.cuda.synchronize()
        total = sum(a.elapsed_time(b) for a, b in marks)
        clocks = sampler.stop() if sampler else None
        launches = eng.take_launch_count()
        return total / steps, stage_times(eng, steps), launches, clocks

    eng32 = make(sg.FP32)
    eng32.set_moment_mma(args.moment_mma)
    if args.profile_only:
        pin_order(eng32, args.order, args.split)
    # pass-kernel autotuner on the workload's layout (after one evaluation), as a user would run it
    # (not in the profiling mode, whose ncu launch offsets count the steps' own launches)
    tuned = {}
    if not args.profile_only:
        step(eng32)
        tuned["fp32"] = tune(eng32, 5)
    sampler = ClockSampler(device) if rank == 0 and not args.profile_only else None
    ms32, st32, launches, clocks = timed(eng32, args.steps, args.warmup, sampler)
    edges = eng32.edge_count()
    if args.profile_only:
        print(json.dumps({"profile_only": True, "atoms": n, "edges": edges, "ms_per_step": ms32,
                          "stages_ms": {k: v[0] / max(1, v[1]) for k, v in st32.items() if v[1]}}), flush=True)
        return 0
    eng64 = make(sg.FP64)
    step(eng64)
    tuned["fp64"] = tune(eng64, 5)
    ms64, st64, _, _ = timed(eng64, max(3, args.steps // 2), args.warmup)

    # e2e through the C ABI with host buffers (copies in and out inside the timed region)
    for _ in range(args.warmup):
        eng32.calc_efs([frame])
    torch.cuda.synchronize()
    calls = []
    for _ in range(args.steps):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        eng32.calc_efs([frame])
        calls.append(time.perf_counter() - t1)
    e2e_ms = 1e3 * float(np.mean(calls))

    # max over ranks
    ms32, ms64, e2e_ms = max_over_ranks([ms32, ms64, e2e_ms], world, dev)
    if rank != 0:
        if world > 1:
            torch.distributed.destroy_process_group()
        return 0

    d = model.dims
    pass_ms = st32["outer"][0] / max(1, st32["outer"][1])
    flops = pass_flops(d, edges, n)
    peaks = {}
    try:
        with open(PEAKS) as fh:
            peaks = json.load(fh)
    except OSError:
        pass
    sm_mhz = (clocks or {}).get("sm_mhz") or peaks.get("sm_max_mhz", 2070.0)
    sm_count = torch.cuda.get_device_properties(device).multi_processor_count
    fp32_peak = sm_count * 128 * 2 * float(peaks.get("sm_max_mhz", 2070.0)) * 1e6 / 1e12
    achieved = flops / (pass_ms / 1e3) / 1e12
    hbm_peak = float(peaks.get("hbm_gbs", 6800.0))
    abytes = algorithmic_bytes(d, edges, n)
    traffic = read_traffic("static_pass_diamond4096_fp32")
    executed = read_traffic("static_pass_diamond4096_fp32_executed_flops")
    # CPU baseline (oracle port, all host cores, bounded sample)
    threads = os.cpu_count() or 1
    nev, tc, te = cpu_sample(frame, threads, min_seconds=10.0, max_evals=40)
    cpu_value = frame.natoms * nev / tc

    # Effect L4/K8/R2/O3 at 110,592 atoms (the large-system configuration), FP32 and FP64
    extra = {}
    if not args.skip_effect:
        from superlinear_gb300.synth import diamond
        fr4 = diamond(24, a=3.567, sigma=0.1, seed=4, species=2, type_prob=0.5)
        m4 = sg.Model(EFFECT_MODEL)
        p4 = torch.tensor(fr4.positions, device=dev)
        t4 = torch.tensor(fr4.types, device=dev)
        F4 = torch.zeros(fr4.natoms, 3, dtype=torch.float64, device=dev)
        c4 = fr4.cell.reshape(1, 9).copy()
        n4 = np.array([fr4.natoms], np.int32)
        results = {}
        for prec, key, reps in ((sg.FP32, "fp32", 5), (sg.FP64, "fp64", 2)):
            e4 = sg.Engine(m4, device, prec)
            e4.set_stream(stream.cuda_stream)
            e4.calc_efs_device(n4, c4, p4.data_ptr(), t4.data_ptr(), E.data_ptr(), F4.data_ptr(), V.data_ptr(), 0)
            tuned[f"effect110k_{key}"] = tune(e4, 2)
            e4.calc_efs_device(n4, c4, p4.data_ptr(), t4.data_ptr(), E.data_ptr(), F4.data_ptr(), V.data_ptr(), 0)
            torch.cuda.synchronize()
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(stream)
            for _ in range(reps):
                e4.calc_efs_device(n4, c4, p4.data_ptr(), t4.data_ptr(), E.data_ptr(), F4.data_ptr(), V.data_ptr(), 0)
            b.record(stream)
            b.synchronize()
            ms = a.elapsed_time(b) / reps
            results[key] = (float(E.cpu()[0]), F4.cpu().numpy().copy())
            extra[key] = {"ms_per_step": ms, "atom_steps_per_s": fr4.natoms / (ms / 1e3), "edges": e4.edge_count()}
            if prec == sg.FP32:
                e4.set_timing(True)
                e4.take_stage_times()
                e4.calc_efs_device(n4, c4, p4.data_ptr(), t4.data_ptr(), E.data_ptr(), F4.data_ptr(), V.data_ptr(), 0)
                extra[key]["stages_ms"] = {k: v[0] for k, v in e4.take_stage_times().items() if v[1]}
                e4.set_timing(False)
            del e4
        extra["fp32_over_fp64"] = extra["fp64"]["ms_per_step"] / extra["fp32"]["ms_per_step"]
        (e32, f32), (e64, f64) = results["fp32"], results["fp64"]
        dfn = np.linalg.norm(f32 - f64, axis=1)
        extra["fp32_error"] = {"against": "FP64 plain GPU path on the same box (pinned to the FP64 oracle at "
                                          "13,824 atoms of the same model and lattice by the GPU tests)",
                               "force_max_ev_per_a": float(np.max(np.abs(f32 - f64))),
                               "force_rms_ev_per_a": float(np.sqrt(np.mean(dfn ** 2))),
                               "energy_ev_per_atom": abs(e32 - e64) / fr4.natoms,
                               "bars": {"force_ev_per_a": 1e-5, "energy_ev_per_atom": 1e-6}}
        if not args.skip_cpu_large:
            # CPU baseline at this size: the FP64 CPU restatement, all host cores, one evaluation
            # (edge build excluded and reported separately)
            import oracle as orc
            om4 = orc.OracleModel(EFFECT_MODEL)
            threads = os.cpu_count() or 1
            _, ne4, te4, tc4 = om4.efs_timed(fr4.cell, fr4.positions, fr4.types, threads=threads)
            cpu4 = fr4.natoms / tc4
            extra["cpu_baseline"] = {"value": cpu4, "unit": "atom-steps/s", "cores": threads, "kind": "port",
                                     "sample": f"one E/F/virial evaluation of the 110,592-atom box ({ne4} edges) by the "
                                               f"FP64 CPU restatement on {threads} threads: {tc4:.2f} s; edge build "
                                               f"excluded ({te4:.2f} s)"}
            extra["fp32_over_cpu"] = extra["fp32"]["atom_steps_per_s"] / cpu4
            extra["fp64_over_cpu"] = extra["fp64"]["atom_steps_per_s"] / cpu4

    # training loss + gradient over the 256-frame Effect L3/K4/R2/O2 batch
    train = None
    if not args.skip_train:
        tframes, train = bench_training(sg, torch, max(3, args.steps // 2), args.warmup)
        nd, tcpu, nw = cpu_train_parallel(tframes, TRAIN_MODEL)
        train["cpu_baseline"] = {"value": nd / tcpu, "unit": "frames/s", "cores": nw, "kind": "port",
                                 "sample": f"loss + gradient of all {nd} frames of the batch by the FP64 CPU "
                                           f"restatement, {nw} processes over interleaved frame shards: {tcpu:.2f} s"}
        train["fp32_over_cpu"] = train["fp32"]["frames_per_s"] / train["cpu_baseline"]["value"]

    # training loss + gradient and BFGS over the 2,048-frame Effect L5/K8/R2/O2 batch
    c5 = None
    if not args.skip_config5:
        c5 = bench_config5(sg, torch, 3, 3, args.bfgs_iters, cpu_frames=128)

    line = {
        "metric": METRIC, "value": replica_throughput(n, world, ms32), "unit": "atom-steps/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms32, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": "static_l3k4o2_diamond4096", "model": "Static L3/K4/O2 (1 species, C)", "atoms": n,
                   "edges": edges, "cutoff": 5.0, "cells": "8x8x8", "a": 3.567, "sigma": 0.08,
                   "step": "GPU edge build + energy/forces/virial", "l2": "flushed (256 MiB write) between steps",
                   "parallelism": f"replicas x{world}" if world > 1 else "single GPU"},
        "fp64_plain": {"ms_per_step": ms64, "value": replica_throughput(n, world, ms64), "fp32_over_fp64": ms64 / ms32},
        "stages_ms_per_step": {k: v[0] / max(1, v[1]) for k, v in st32.items() if v[1]},
        "roofline": {"bound": "fp32", "achieved": achieved, "peak": fp32_peak, "unit": "TFLOP/s",
                     "frac": achieved / fp32_peak,
                     "peak_source": f"nominal FP32 FMA rate {sm_count} SMs x 128 lanes x 2 flop x sm_max_mhz "
                                    "(MEASURED_PEAKS.json holds no FP32 CUDA-core peak)",
                     "kernel": "atom_pass_kernel (Static, forward + adjoint)", "kernel_ms": pass_ms,
                     "flops_per_launch": flops,
                     "hbm": {"achieved": abytes / (pass_ms / 1e3) / 1e9, "peak": hbm_peak, "unit": "GB/s",
                             "frac": abytes / (pass_ms / 1e3) / 1e9 / hbm_peak, "peak_source": "MEASURED_PEAKS.json hbm_gbs (measured)"},
                     "traffic": traffic,
                     # the same launch by executed FP32 flops (2 FFMA + FADD + FMUL, one ncu capture):
                     # the per-edge formula counts ~1.8x the arithmetic this kernel performs
                     "executed": ({"flops_per_launch": executed, "achieved": executed / (pass_ms / 1e3) / 1e12,
                                   "frac": executed / (pass_ms / 1e3) / 1e12 / fp32_peak}
                                  if executed else None)},
        "cpu_baseline": {"value": cpu_value, "unit": "atom-steps/s", "cores": threads, "kind": "port",
                         "sample": f"{nev} E/F/virial evaluations of the same 4,096-atom frame by the FP64 CPU "
                                   f"restatement on {threads} threads, edge build excluded "
                                   f"({1e3 * te / max(nev, 1):.1f} ms each)"},
        "e2e": {"value": replica_throughput(n, world, e2e_ms), "unit": "atom-steps/s",
                "h2d_bytes_per_step": n * 3 * 8 + n * 4 + 9 * 8,
                "d2h_bytes_per_step": 8 + n * 3 * 8 + 6 * 8 + n * 8, "ms_per_step": e2e_ms,
                "api": "sus2g_calc_efs_host (C ABI, host buffers)"},
        "clocks": clocks,
        "gpu_launches": launches,
        "autotune": tuned,
        "effect_l4k8r2o3_110592": extra or None,
        "train_effect_l3k4r2o2_256": train,
        "train_effect_l5k8r2o2_2048": c5,
    }
    print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser(description=__doc__)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--skip-effect", action="store_true", help="skip the 110,592-atom Effect measurement")
    ap.add_argument("--skip-train", action="store_true", help="skip the 256-frame training loss+gradient measurement")
    ap.add_argument("--skip-cpu-large", action="store_true",
                    help="skip the CPU baseline evaluation of the 110,592-atom box")
    ap.add_argument("--profile-only", action="store_true",
                    help="only the FP32 timed steps (for ncu captures); prints a short JSON line")
    ap.add_argument("--cells", type=int, default=8, help="diamond cells per edge (8 -> the 4,096-atom workload)")
    ap.add_argument("--profile-train", action="store_true",
                    help="only FP32 training loss+gradient steps over the 256-frame batch (for ncu launch lists)")
    ap.add_argument("--no-graph", action="store_true", help="with --profile-train: eager launches instead of the graph")
    ap.add_argument("--profile-effect", action="store_true",
                    help="only FP32 Effect L4/K8/R2/O3 steps on a --cells diamond (for ncu captures)")
    ap.add_argument("--order", choices=("strided", "contiguous", "dynamic"), default=None,
                    help="with the profiling modes: pin every pass to this centre order (default budgets and "
                         "grid), as the autotuner's choice would set it, without the autotuner's launches")
    ap.add_argument("--split", action="store_true",
                    help="with the profiling modes: every per-atom pass split at the per-atom boundary")
    ap.add_argument("--moment-mma", action="store_true",
                    help="with --profile-only / --profile-effect: edge->moment sums on the tensor cores (3xTF32)")
    ap.add_argument("--skip-config5", action="store_true",
                    help="skip the 2,048-frame L5 training loss+gradient and BFGS measurement")
    ap.add_argument("--bfgs-iters", type=int, default=100, help="timed FP32 BFGS iterations on the L5 batch")
    ap.add_argument("--config5-only", action="store_true",
                    help="only the 2,048-frame L5 training measurement; prints its JSON object")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)
    if args.profile_train:
        return run_profile_train(args)
    if args.profile_effect:
        return run_profile_effect(args)
    if args.config5_only:
        import torch

        import superlinear_gb300 as sg
        print(json.dumps(bench_config5(sg, torch, 3, 3, args.bfgs_iters)), flush=True)
        return 0
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
