"""Build libmbqc_gb300.so in-tree with nvcc for sm_103a (no cmake, no torch).

    python -m mentpy_gb300.build [--force] [--verbose-ptxas]

Translation units compile in parallel; a unit is rebuilt when any source or
header is newer than its object file or the flags changed.
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import hashlib
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIBDIR = os.path.join(HERE, "lib")
LIB = os.path.join(LIBDIR, "libmbqc_gb300.so")
INCLUDE = os.path.join(ROOT, "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
         "--expt-relaxed-constexpr", "-I", INCLUDE, "-I", CSRC]

SV_REG_WINDOWS = range(1, 11)
SV_ADJ_WINDOWS = range(1, 9)


def units():
    """(source, object, extra flags) for every translation unit."""
    out = []
    for name in ("plan.cu", "sv_api.cu", "adj_api.cu", "adj_noalloc.cu", "dm.cu", "dm_batch.cu", "dm_adj.cu",
                 "sv_stream.cu", "graph_compile.cu", "train.cu", "sv_sampled.cu",
                 "sv_adj_wide.cu"):
        out.append((os.path.join(CSRC, name), os.path.join(BUILD, name[:-3] + ".o"), []))
    for w in SV_REG_WINDOWS:
        out.append((os.path.join(CSRC, "sv_reg.cu"), os.path.join(BUILD, f"sv_reg_w{w}.o"), [f"-DSV_W={w}"]))
    for w in SV_ADJ_WINDOWS:
        out.append((os.path.join(CSRC, "sv_adj.cu"), os.path.join(BUILD, f"sv_adj_w{w}.o"), [f"-DSV_W={w}"]))
    return out


def nvcc():
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(exe):
        raise RuntimeError("nvcc not found: the CUDA 13 toolkit is required to build libmbqc_gb300")
    return exe


def _deps_mtime():
    m = 0.0
    for d in (CSRC, INCLUDE):
        for f in os.listdir(d):
            m = max(m, os.path.getmtime(os.path.join(d, f)))
    return m


def _stamp(flags):
    return hashlib.sha1(" ".join(flags).encode()).hexdigest()


def _compile(src, obj, extra, force, ptxas_v):
    flags = ARCH + FLAGS + extra + (["-Xptxas", "-v"] if ptxas_v else [])
    stamp_file = obj + ".flags"
    fresh = (
        not force
        and os.path.exists(obj)
        and os.path.getmtime(obj) >= _deps_mtime()
        and os.path.exists(stamp_file)
        and open(stamp_file).read() == _stamp(flags)
    )
    if fresh:
        return obj, ""
    cmd = [nvcc()] + flags + ["-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {os.path.basename(obj)}:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    with open(stamp_file, "w") as f:
        f.write(_stamp(flags))
    return obj, r.stderr


def build(force: bool = False, ptxas_verbose: bool = False, jobs: int = 0) -> str:
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    us = units()
    jobs = jobs or min(len(us), os.cpu_count() or 4)
    logs = []
    with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
        futs = [ex.submit(_compile, s, o, e, force, ptxas_verbose) for s, o, e in us]
        objs = []
        for f in futs:
            obj, log = f.result()
            objs.append(obj)
            if log:
                logs.append(f"== {os.path.basename(obj)}\n{log}")
    newest = max(os.path.getmtime(o) for o in objs)
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < newest:
        cmd = [nvcc()] + ARCH + ["-shared", "-cudart", "shared", "-o", LIB] + objs + [
            "-Xlinker", "-rpath=/usr/local/cuda/lib64"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    if ptxas_verbose and logs:
        print("\n".join(logs))
    return LIB


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--force", action="store_true")
    ap.add_argument("--verbose-ptxas", action="store_true")
    ap.add_argument("-j", "--jobs", type=int, default=0)
    a = ap.parse_args()
    print(build(a.force, a.verbose_ptxas, a.jobs))
