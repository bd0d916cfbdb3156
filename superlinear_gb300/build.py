"""In-tree build of the CUDA engine library ``_build/libsus2g.so`` for sm_103a.

Every translation unit under ``csrc/`` is compiled by ``nvcc`` in parallel (one ``-gencode``,
``-lineinfo``), then linked as a shared library exporting the C ABI of ``include/sus2g.h``.
Objects are rebuilt only when a source or header is newer than them.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libsus2g.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc_path() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _newest(paths) -> float:
    return max((os.path.getmtime(p) for p in paths), default=0.0)


def build(verbose: bool = False, jobs: int | None = None) -> str:
    os.makedirs(BUILD, exist_ok=True)
    nvcc = nvcc_path()
    headers = glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh")) + \
        glob.glob(os.path.join(HERE, "..", "include", "*.h"))
    hdr_time = _newest(headers)
    sources = sorted(glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.cpp")))
    flags = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-fno-fast-math",
             "-Wno-deprecated-gpu-targets"] + ARCH
    # objects built with other flags are rebuilt
    stamp = os.path.join(BUILD, "flags.txt")
    if not os.path.exists(stamp) or open(stamp).read() != " ".join(flags):
        for old in glob.glob(os.path.join(BUILD, "*.o")):
            os.remove(old)
        with open(stamp, "w") as f:
            f.write(" ".join(flags))
    jobs_list = []
    objects = []
    for src in sources:
        obj = os.path.join(BUILD, os.path.basename(src) + ".o")
        objects.append(obj)
        if os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(src), hdr_time):
            continue
        cmd = [nvcc] + flags + ["-c", src, "-o", obj]
        if src.endswith(".cpp"):
            cmd = [nvcc, "-x", "cu"] + flags + ["-c", src, "-o", obj]
        jobs_list.append(cmd)

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode:
            raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stderr[-4000:]}")
        if verbose and r.stderr:
            print(r.stderr, file=sys.stderr)
        return cmd[-1]

    if jobs_list:
        with cf.ThreadPoolExecutor(max_workers=jobs or min(len(jobs_list), os.cpu_count() or 4)) as pool:
            for out in pool.map(run, jobs_list):
                if verbose:
                    print("built", os.path.basename(out))
    if not os.path.exists(LIB) or os.path.getmtime(LIB) < _newest(objects):
        cmd = [nvcc] + ARCH + ["-shared", "-o", LIB] + objects + ["-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode:
            raise RuntimeError(f"link failed: {r.stderr[-4000:]}")
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
