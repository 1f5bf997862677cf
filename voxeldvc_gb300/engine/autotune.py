"""Schedule autotuner with a JSON cache.

Knobs, per problem class (the element sizes and meshes of a batch, or of a
single level):
  * pcg_chunk -- PCG iterations per body of the device-driven WHILE graph:
    small bodies stop sooner after convergence, large bodies amortise the
    per-body continue kernel and graph-node overhead;
  * concurrent -- a batch's problems on their own streams (parallel branches
    of one graph) or serialised on one stream.
Each candidate runs one GN iteration with a short PCG from the same start
(U restored before every trial), timed on the host around a synchronised
call; the fastest is cached under a key of GPU name + problem class in
$VDVC_TUNE_CACHE (default ~/.cache/voxeldvc_gb300/tune.json) and reused
without measuring.
"""
from __future__ import annotations

import ctypes as C
import json
import os
import time

import numpy as np

from .. import _device as D
from .. import _lib

CHUNKS = (1, 2, 4, 8)
TRIAL_PCG_ITERS = 16


def cache_path():
    p = os.environ.get("VDVC_TUNE_CACHE")
    if p:
        return p
    return os.path.join(os.path.expanduser("~"), ".cache", "voxeldvc_gb300", "tune.json")


def _gpu():
    try:
        return D.torch().cuda.get_device_name()
    except Exception:  # no device: keys still work, tuning does not
        return "unknown"


def batch_key(items):
    """items: [(h, (Nx, Ny, Nz))] of the batch's problems."""
    parts = sorted(f"h{h}:{m[0]}x{m[1]}x{m[2]}" for h, m in items)
    return f"batch|{_gpu()}|{len(parts)}|" + ";".join(parts)


def _load():
    try:
        with open(cache_path()) as fh:
            return json.load(fh)
    except (OSError, ValueError):
        return {}


def lookup(key):
    v = _load().get(key)
    if not v:
        return None, None
    return int(v["pcg_chunk"]), int(v["concurrent"])


def store(key, value):
    path = cache_path()
    data = _load()
    data[key] = value
    try:
        os.makedirs(os.path.dirname(path), exist_ok=True)
        tmp = path + ".tmp"
        with open(tmp, "w") as fh:
            json.dump(data, fh, indent=1, sort_keys=True)
        os.replace(tmp, path)
    except OSError:
        pass  # a read-only home: the result is used, just not cached


def tune_batch(L, batch, solvers, setups, pcg_max_iter, pcg_tol, key, stream):
    """Measure every (pcg_chunk, concurrent) candidate on the batch's first
    GN iteration and keep the fastest; returns it."""
    n = len(solvers)
    active = np.ones(n, dtype=np.int32)
    out = np.zeros(12 * n, dtype=np.float64)
    it = int(min(pcg_max_iter, TRIAL_PCG_ITERS))
    trials = {}

    def reset():
        for sv, ls in zip(solvers, setups):
            _lib.check(L.vdvc_gn_set_U(sv, ls.U64.data_ptr(), stream), "set_U")

    for conc in (0, 1):
        for chunk in CHUNKS:
            _lib.check(L.vdvc_gn_batch_set_schedule(batch, chunk, conc), "batch_set_schedule")
            times = []
            for rep in range(2):  # the first builds the graph
                reset()
                D.torch().cuda.synchronize()
                t0 = time.perf_counter()
                _lib.check(L.vdvc_gn_batch_iterate(batch, active.ctypes.data, None, it, float(pcg_tol),
                                                   out.ctypes.data, stream), "batch_iterate")
                times.append(time.perf_counter() - t0)
            trials[(chunk, conc)] = times[-1]
    reset()
    best = min(trials, key=trials.get)
    _lib.check(L.vdvc_gn_batch_set_schedule(batch, best[0], best[1]), "batch_set_schedule")
    store(key, {"pcg_chunk": best[0], "concurrent": best[1],
                "trials_ms": {f"{c}/{k}": round(1e3 * t, 3) for (c, k), t in trials.items()}})
    return best
