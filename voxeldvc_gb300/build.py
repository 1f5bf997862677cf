"""Build recipe of the CUDA library ``libvdvc.so`` (sm_103a only).

Each ``csrc/*.cu`` translation unit is compiled to an object in parallel,
then linked into one shared library next to this file.  The build is
incremental on file modification times.  Run ``python -m
voxeldvc_gb300.build`` or call :func:`build`.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD_DIR = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(HERE, "libvdvc.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + [
    "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
    "--expt-relaxed-constexpr", "-I", INCLUDE, "-I", CSRC,
]
LINK_LIBS = ["-lcufft", "-Xlinker", "-rpath=/usr/local/cuda/lib64"]


def _nvcc() -> str:
    cand = shutil.which("nvcc")
    if cand:
        return cand
    for p in ("/usr/local/cuda/bin/nvcc",):
        if os.path.exists(p):
            return p
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libvdvc.so")


def _sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    hs += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]
    return hs


def _newest(paths):
    return max((os.path.getmtime(p) for p in paths), default=0.0)


def build(verbose: bool = False, force: bool = False, extra_flags=()) -> str:
    """Compile ``libvdvc.so`` if any source is newer than it; return its path."""
    nvcc = _nvcc()
    os.makedirs(BUILD_DIR, exist_ok=True)
    srcs = _sources()
    hdr_time = _newest(_headers())
    objs = []
    jobs = []
    for src in srcs:
        obj = os.path.join(BUILD_DIR, os.path.basename(src)[:-3] + ".o")
        objs.append(obj)
        stale = force or not os.path.exists(obj) or os.path.getmtime(obj) < max(os.path.getmtime(src), hdr_time)
        if stale:
            cmd = [nvcc, *NVCC_FLAGS, *extra_flags, "-c", src, "-o", obj]
            jobs.append(cmd)
    if jobs:
        workers = min(len(jobs), max(1, os.cpu_count() or 1))
        with cf.ThreadPoolExecutor(workers) as ex:
            results = list(ex.map(lambda c: subprocess.run(c, capture_output=True, text=True), jobs))
        failed = [(c, r) for c, r in zip(jobs, results) if r.returncode != 0]
        for c, r in zip(jobs, results):
            if verbose or r.returncode != 0:
                sys.stderr.write(" ".join(c) + "\n" + r.stdout + r.stderr)
        if failed:
            raise RuntimeError("nvcc failed for: " + ", ".join(c[-3] for c, _ in failed))
    if force or jobs or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < _newest(objs):
        tmp = LIB_PATH + ".tmp"
        cmd = [nvcc, *ARCH, "-shared", "-o", tmp, *objs, *LINK_LIBS]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
            raise RuntimeError("link of libvdvc.so failed")
        os.replace(tmp, LIB_PATH)
    return LIB_PATH


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
