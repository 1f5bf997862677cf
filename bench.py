#!/usr/bin/env python
"""Benchmark of the GB300 voxelDVC Gauss-Newton path.

Workload (default `necking_512`): the 513^3 float32 pair of a fiber-composite
texture (5000 cylinders) under tensile necking, h = 8 (64^3 elements,
823,875 dof), equilibrium-gap regularizer, 3-level pyramid with FFT seed,
dynamic mask frozen after 4 iterations (the `voxeldvc run` settings).  One
step = one complete plain-FP32 multiscale GN-PCG solve to the reference's
stopping rules.  Data are synthetic and generated on the GPU (seeded);
the inputs (540 MB each) are larger than L2, so no flush is needed.

  value   device-resident solve time (s/solve), CUDA events on the stream
  e2e     the same solve through the public API with host numpy inputs:
          host->device image upload and device->host read of (U, res, dU)
          inside the timed region
  roofline  the matrix-free Hessian matvec at the finest level, timed with
          CUDA events right after the timed solves on the same data
  cpu_baseline  the CPU oracle (NumPy restatement of the reference) per
          operation on a bounded sample, extrapolated to the solve with the
          operation counts of the GPU solve

`--impl reference` times only the CPU oracle leg (the reference has no CPU
solver of its own besides its NumPy execution) and prints the same metric.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "512³ h=8 DVC time to 0.02vx RMS, plain vs mixed/learned; matvec GB/s"

# Operation counts of the FP32 GB300 solve of necking_512 (per level, coarse
# to fine): GN iterations and total PCG iterations.  The CPU leg multiplies
# its measured per-operation times by these; the GPU leg reports its own
# counts next to them in every run.
# DRAM bytes per voxel of one float32 matvec (k_strip_hv_fast<8> + k_gather),
# ncu dram__bytes_read + write on the 257^3 case.
TRAFFIC_B_PER_VOXEL = 14.04

SOLVE_COUNTS = {"necking_512": {"gn": [30, 4, 2], "pcg": [752, 84, 41]},
                "necking_512_eqgap": {"gn": [30, 30, 30], "pcg": [60000, 60000, 60000]},
                "necking_256": {"gn": [8, 6, 3], "pcg": [200, 108, 57]},
                "plain_small": {"gn": [10, 5, 3], "pcg": [200, 100, 60]},
                "large_1024": {"gn": [30, 30, 3, 2], "pcg": [2179, 1388, 140, 95]}}


def parse(argv=None):
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=3)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--workload", default="necking_512")
    p.add_argument("--e2e-steps", type=int, default=1)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--cpu-sample-layers", type=int, default=None,
                   help="element layers per CPU-baseline worker (default: the whole mesh split over the cores)")
    p.add_argument("--no-forms", action="store_true",
                   help="skip the precision / learned-seed form comparison (FP64 reference solve included)")
    p.add_argument("--only", default=None, choices=[None, "matvec", "kernels", "ground-truth", "post", "eh-form", "learned"],
                   help="matvec: time only the finest-level Hessian matvec; kernels: run each hot kernel of the "
                        "plain, precision and learned forms a few times on the 257^3 case (the profiling commands)")
    return p.parse_args(argv)


def matvec_only(args):
    """Generate the workload's reference image, then run `--warmup` + `--steps`
    finest-level Hessian matvecs (vdvc_matvec_H) and print their mean time."""
    import torch
    from voxeldvc_gb300 import _lib, synth
    from voxeldvc_gb300.engine import correlate_gpu as CG
    wl = synth.WORKLOADS[args.workload]()
    Nx, Ny, Nz = wl.mesh
    f = synth.texture(wl.shape, wl.n_cyl)
    grad, mask0 = CG._grad_vox(f, wl.shape, np.float32, 0.0)
    del f
    ndof = 3 * (Nx + 1) * (Ny + 1) * (Nz + 1)
    v = torch.randn(ndof, device="cuda", dtype=torch.float32)
    out = torch.empty_like(v)
    L = _lib.lib()
    nws = L.vdvc_workspace_bytes(_lib.F32, wl.h, Nx, Ny, Nz)
    ws = torch.empty(nws, dtype=torch.uint8, device="cuda")
    s = torch.cuda.current_stream()

    def mv():
        _lib.check(L.vdvc_matvec_H(v.data_ptr(), grad.data_ptr(), mask0.data_ptr(), _lib.F32, wl.h, Nx, Ny, Nz,
                                   out.data_ptr(), ws.data_ptr(), nws, s.cuda_stream))

    for _ in range(args.warmup):
        mv()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(s)
    for _ in range(args.steps):
        mv()
    e1.record(s)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / max(1, args.steps)
    nvox = wl.shape[0] * wl.shape[1] * wl.shape[2]
    print(json.dumps({"workload": wl.name, "matvec_ms": round(ms, 4),
                      "algorithmic_GBs": round((nvox * 13 + ndof * 8) / ms / 1e6, 1)}))


# ---------------------------------------------------------------------------
# clocks during the timed region
# ---------------------------------------------------------------------------

class Clocks:
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.path = tempfile.mktemp(suffix=".csv")
        self.proc = None
        self.gpu = gpu_index

    def __enter__(self):
        try:
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.fh,
                                         stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.fh.close()

    def summary(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        os.unlink(self.path)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------------------
# CPU oracle leg: per-operation times on a bounded sample, extrapolated
# ---------------------------------------------------------------------------

def _timed(fn, *a, **k):
    t0 = time.perf_counter()
    fn(*a, **k)
    return time.perf_counter() - t0


def _cpu_slab_times(job):
    """Per-operation seconds of the oracle on one slab of `nz` element layers
    of every pyramid level (one worker of the CPU baseline)."""
    Nx, Ny, h0, scales, nz, nu, seed = job
    from oracle import dvc_oracle as O
    rng = np.random.default_rng(seed)
    K_lap = O.k_ref_laplacian()
    out = {}
    nd = 3 * (Nx + 1) * (Ny + 1) * (nz + 1)
    v64 = rng.standard_normal(nd)
    out["k"] = _timed(O.matvec_k_ref, v64, K_lap, float(h0), Nx, Ny, nz)
    out["vec"] = _timed(lambda: [v64 * 1.0001 + v64 for _ in range(10)] and float(np.dot(v64, v64)))
    for s in scales:
        h = h0 // 2 ** s
        Nvx, Nvy, Nvz = Nx * h + 1, Ny * h + 1, nz * h + 1
        nvox = Nvx * Nvy * Nvz
        grad = rng.standard_normal((nvox, 3)).astype(np.float32)
        mask = rng.random(nvox) < 0.95
        res = rng.standard_normal(nvox)
        vs = rng.standard_normal(nd)
        gimg = rng.random((Nvx, Nvy, Nvz)).astype(np.float32)
        out[h] = {"mv": _timed(O.matvec_h, vs, grad, mask, h, Nx, Ny, nz),
                  "dg": _timed(O.diag_h, grad, mask, h, Nx, Ny, nz, nd),
                  "b": _timed(O.compute_b, res, mask, grad, h, Nx, Ny, nz, nd),
                  "st": _timed(O.masked_mean_std, res, mask, h, Nx, Ny, nz),
                  "sm": _timed(O.sample_deformed, 0.3 * vs, gimg, h, Nx, Ny, nz, (0, 0, 0), mask)}
    return out


def cpu_workers():
    """Host cores this process may use."""
    try:
        return max(1, len(os.sched_getaffinity(0)))
    except AttributeError:
        return max(1, os.cpu_count() or 1)


def cpu_model(wl, counts, layers=None, procs=None):
    """Seconds of the reference path on this host's cores for one solve.
    The reference's operators loop over element chunks, so the mesh splits
    into z slabs that run on separate cores: `procs` worker processes
    (spawned: the parent may hold a CUDA context; one BLAS/OpenMP thread
    each) time every operation of every pyramid level on their own slabs,
    all at once, so the times include the cores' contention for memory
    bandwidth.  By default the slabs cover the whole mesh (Nz / procs layers
    each) and a full-mesh operation costs the slowest worker's time; with
    `layers` given, each worker times that many layers and the cost is
    extrapolated linearly to Nz / procs layers.  Multiplied by the solve's
    GN and PCG counts."""
    import multiprocessing as mp
    Nx, Ny, Nz = wl.mesh
    procs = max(1, min(procs or cpu_workers(), Nz))
    per = layers or -(-Nz // procs)
    eqgap = wl.solve["reg_type"] == "equilibrium_gap"
    scales = sorted(wl.solve["scales"], reverse=True)
    jobs = [(Nx, Ny, wl.h, scales, per, wl.solve.get("nu", 0.3), p) for p in range(procs)]
    t_start = time.perf_counter()
    if procs > 1:
        keys = ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS", "MKL_NUM_THREADS")
        saved = {k: os.environ.get(k) for k in keys}
        os.environ.update({k: "1" for k in keys})
        try:
            with mp.get_context("spawn").Pool(procs) as pool:
                res = pool.map(_cpu_slab_times, jobs)
        finally:
            for k, v in saved.items():
                if v is None:
                    os.environ.pop(k, None)
                else:
                    os.environ[k] = v
    else:
        res = [_cpu_slab_times(jobs[0])]
    wall = time.perf_counter() - t_start
    layers = per
    scale = (Nz / procs) / per
    slow = lambda key, lvl=None: max((r[lvl][key] if lvl else r[key]) for r in res) * scale  # noqa: E731
    t_k = slow("k")
    t_reg = (3 if eqgap else 1) * t_k          # K P K + eps K_lap  (or K_lap)
    t_reg_diag = (2 * 32 * t_k + t_k) if eqgap else t_k  # Hutchinson (32 probes x K P K) + diag K_lap
    t_vec = slow("vec")
    levels, total = [], 0.0
    for li, s in enumerate(scales):
        h = wl.h // 2 ** s
        t_mv, t_dg, t_b, t_st, t_sm = (slow(k, h) for k in ("mv", "dg", "b", "st", "sm"))
        t_pcg = t_mv + t_reg + t_vec
        t_gn = t_sm + 2 * t_st + t_b + t_reg + t_dg + t_reg_diag + t_st
        n_gn, n_pcg = counts["gn"][li], counts["pcg"][li]
        t_level = n_gn * t_gn + (n_pcg + n_gn) * t_pcg
        total += t_level
        levels.append({"h": h, "matvec_s": round(t_mv, 3), "gn_fixed_s": round(t_gn, 3), "level_s": round(t_level, 1)})
    return total, {"levels": levels, "reg_matvec_s": round(t_k, 3), "sample_wall_s": round(wall, 1),
                   "sample": f"oracle per-op timing by {procs} worker processes at once, each on its own z slab "
                             f"of {layers} element layer(s) of every level (full mesh {Nz} layers; "
                             f"{'whole mesh covered' if layers * procs >= Nz else 'extrapolated in layers'}), "
                             f"slowest worker per op; extrapolated with the solve's GN/PCG counts {counts}",
                   "threads": procs}


def reference_arm(args):
    from voxeldvc_gb300 import synth
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    wl = synth.WORKLOADS[args.workload]()
    counts = SOLVE_COUNTS[args.workload]
    vals = []
    info = None
    # the CPU leg has no warm-up effects worth discarding beyond numpy's first
    # call; each step re-measures every operation on fresh samples
    for _ in range(max(1, args.steps)):
        v, info = cpu_model(wl, counts, args.cpu_sample_layers)
        vals.append(v)
    value = float(np.median(vals))
    line = {"metric": METRIC, "value": round(value, 2), "unit": "s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(value * 1e3, 1), "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 (PCG promoted to f64 as in the reference)",
            "data": "synthetic", "impl": "reference",
            "config": {"workload": wl.name, "mesh": list(wl.mesh), "h": wl.h, "extrapolated": True},
            "cpu_baseline": {"value": round(value, 2), "unit": "s", "cores": info["threads"], "kind": "port",
                             "sample": info["sample"]},
            "e2e": {"value": round(value, 2), "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "detail": info}
    print(json.dumps(line))


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------

def solve_kwargs(wl):
    from voxeldvc_gb300.engine import geometry_dvc as G
    s = wl.solve
    kw = dict(scales=s["scales"], l0=s["l0"], K_ref_laplacian=G.build_K_ref_laplacian(), reg_type=s["reg_type"],
              dynamic_mask=True, freeze_mask_after=4, maxiter=30, eps=1e-3, pcg_tol=1e-6, pcg_max_iter=2000,
              glt=0.0, fft_prealign=True, disp=False)
    if s["reg_type"] == "equilibrium_gap":
        kw["K_ref_elastic"] = G.build_K_ref(s.get("nu", 0.3))
        kw["reg_exponent"] = s.get("reg_exponent", 4)
    for key in ("prealign_affine", "precision"):
        if key in s:
            kw[key] = s[key]
    return kw


def compare_forms(wl, f_pix, g_pix, kw, U_plain, e2e_plain, plain_s):
    """Plain FP32, precision form and learned seed + precision form against
    the FP64 solve of the same inputs (the project's GPU FP64 mode, parity
    checked against the NumPy FP64 oracle at small sizes): wall time of the
    device-resident solve, the same through the public API with host arrays,
    and the nodal RMS difference to the FP64 displacement."""
    import torch
    from voxeldvc_gb300.engine import correlate_gpu as CG
    from voxeldvc_gb300.learned import solve as LS
    Nx, Ny, Nz = wl.mesh

    def timed(fn, reps=3):
        fn()
        ts, out = [], None
        for _ in range(reps):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            out = fn()
            torch.cuda.synchronize()
            ts.append(time.perf_counter() - t0)
        return float(np.median(ts)), out

    t64, (U64, _, _) = timed(lambda: CG.multiscale_correlate_gpu(f_pix, g_pix, Nx, Ny, Nz, wl.h, xp=torch,
                                                                  dtype=np.float64, **kw), reps=1)
    U64 = U64.double()

    def rms(U):
        return float(torch.sqrt(torch.mean((U.double() - U64) ** 2)).item())

    out = {"reference": "GPU FP64 solve of the same inputs", "f64_s": round(t64, 4),
           "target_rms_vx": 0.02, "plain": {"rms_vs_f64_vx": round(rms(U_plain), 6)}}
    tm, (Um, _, _) = timed(lambda: CG.multiscale_correlate_gpu(f_pix, g_pix, Nx, Ny, Nz, wl.h, xp=torch,
                                                                precision="mixed", **kw))
    out["mixed"] = {"s": round(tm, 4), "rms_vs_f64_vx": round(rms(Um), 6)}
    kwl = {k: v for k, v in kw.items() if k not in ("scales", "fft_prealign")}
    try:
        net = LS.default_net()
    except (OSError, KeyError) as e:
        out["learned_mixed"] = {"unavailable": f"no trained seed network ({e})"}
        return out
    stats = []
    tl, (Ul, _, _) = timed(lambda: LS.learned_correlate_gpu(f_pix, g_pix, Nx, Ny, Nz, wl.h, torch, net=net,
                                                            precision="mixed", stats=stats, **kwl))
    last = stats[-1]
    gn = [s for s in stats if "gn_iters" in s]
    out["learned_mixed"] = {"s": round(tl, 4), "rms_vs_f64_vx": round(rms(Ul), 6), "seed": last.get("seed"),
                            "norm_res": last.get("norm_res"), "gn_iters": [s["gn_iters"] for s in gn[-1:]],
                            "pcg_iters": [int(sum(s["pcg_iters"])) for s in gn[-1:]]}
    # the same through the public API with host arrays (as the plain e2e)
    f_host = f_pix.cpu().pin_memory().numpy()
    g_host = g_pix.cpu().pin_memory().numpy()
    te, _ = timed(lambda: LS.learned_correlate_gpu(f_host, g_host, Nx, Ny, Nz, wl.h, np, net=net,
                                                   precision="mixed", **kwl), reps=2)
    out["learned_mixed"]["e2e_s"] = round(te, 4)
    if e2e_plain:
        out["learned_mixed"]["e2e_speedup_vs_plain"] = round(e2e_plain["value"] / te, 3)
    out["learned_mixed"]["speedup_vs_plain_device"] = round(plain_s / tl, 3)
    out["mixed"]["speedup_vs_plain_device"] = round(plain_s / tm, 3)
    return out


def compare_batch():
    """The batched form on the load-series workload (16 problems, one 385^3
    reference, uneven ROIs, h in {8, 12, 16}): the lockstep batch (cached or
    default schedule) against the same solves one after another."""
    import torch
    from voxeldvc_gb300 import synth
    from voxeldvc_gb300.engine import batch as B, correlate_gpu as CG, geometry_dvc as G
    f_pix, gs, problems, fields = synth.series_385()
    Kl = G.build_K_ref_laplacian()
    kw = dict(scales=(2, 1, 0), fft_prealign=True, dynamic_mask=True, freeze_mask_after=4, maxiter=30, eps=1e-3,
              pcg_tol=1e-6, pcg_max_iter=2000, glt=0.0)

    def seq():
        outs = []
        for i, p in enumerate(problems):
            h = p["h"]
            (x0, y0, z0), (Nx, Ny, Nz) = p["origin"], p["mesh"]
            sl = (slice(x0, x0 + Nx * h + 1), slice(y0, y0 + Ny * h + 1), slice(z0, z0 + Nz * h + 1))
            outs.append(CG.multiscale_correlate_gpu(f_pix[sl], gs[i][sl], Nx, Ny, Nz, h, xp=torch, l0=4.5 * h,
                                                    K_ref_laplacian=Kl, disp=False, **kw))
        return outs

    def bat(stats=None):
        return B.batch_multiscale_correlate_gpu(f_pix, gs, problems, torch, l0_factor=4.5, K_ref_laplacian=Kl,
                                                tune=True, stats=stats, **kw)

    res = {}
    for label, fn in (("sequential_s", seq), ("batch_s", bat)):
        fn()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        out = fn()
        torch.cuda.synchronize()
        res[label] = round(time.perf_counter() - t0, 4)
    st = []
    out = bat(st)
    rms = [float(np.sqrt(np.mean((out[i][0].double().cpu().numpy() - synth.true_U_problem(p, fields[i])) ** 2)))
           for i, p in enumerate(problems)]
    res.update(problems=len(problems), hs=[p["h"] for p in problems],
               meshes=[list(p["mesh"]) for p in problems], speedup=round(res["sequential_s"] / res["batch_s"], 3),
               rms_vs_true_field_vx_max=round(max(rms), 5), schedule=[s["schedule"] for s in st])
    return res


def max_over_ranks(value, world, device):
    """The slowest rank's value (replicas: the job ends with its last rank);
    the process group's backend moves the tensor (NCCL on the GPU, gloo in
    the CPU tests)."""
    if world <= 1:
        return value
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def gpu_arm(args):
    import torch
    import torch.distributed as dist
    from voxeldvc_gb300 import _lib, synth
    from voxeldvc_gb300.engine import correlate_gpu as CG
    from voxeldvc_gb300.engine import kernels_dvc as K
    from voxeldvc_gb300.engine import geometry_dvc as G

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl")

    def barrier():
        if world > 1:
            dist.barrier()

    wl = synth.WORKLOADS[args.workload]()
    Nx, Ny, Nz = wl.mesh
    f_pix, g_pix = wl.make()
    torch.cuda.synchronize()
    kw = solve_kwargs(wl)

    def step(stats=None):
        return CG.multiscale_correlate_gpu(f_pix, g_pix, Nx, Ny, Nz, wl.h, xp=torch, stats=stats, **kw)

    # the per-level statistics come from the last warm-up step, so every
    # timed step runs the same code; the host's garbage collector is held
    # off during the timed region (the solve is host-driven per GN iteration)
    level_stats = []
    n_warm = max(1, args.warmup)
    for w in range(n_warm):
        step(level_stats if w == n_warm - 1 else None)
    torch.cuda.synchronize()
    barrier()
    stream = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    n0 = _lib.launch_count()
    import gc
    gc.collect()
    gc.disable()
    try:
        with Clocks(local) as clk:
            torch.cuda.synchronize()
            e0.record(stream)
            for _ in range(args.steps):
                U, res, dU = step()
            e1.record(stream)
            torch.cuda.synchronize()
    finally:
        gc.enable()
    launches = (_lib.launch_count() - n0) // max(1, args.steps)
    ms = e0.elapsed_time(e1) / args.steps
    barrier()
    ms = max_over_ranks(ms, world, "cuda")
    clocks = clk.summary()

    # accuracy vs the analytic field (sanity; the solve's own error), over
    # all nodes and over the nodes at least 4 elements inside the mesh border
    # (near the border the deformed position can leave g: truncated support)
    Uh = U.double().cpu().numpy()
    err = (Uh - wl.true_U()).reshape(-1, 3)
    rms_true = float(np.sqrt(np.mean(err ** 2)))
    nb = np.array(wl.mesh) + 1
    nn = np.arange(int(np.prod(nb)))
    ijk = np.stack([nn % nb[0], (nn // nb[0]) % nb[1], nn // (nb[0] * nb[1])], 1)
    inner = np.all((ijk >= 4) & (ijk <= np.array(wl.mesh) - 4), axis=1)
    rms_inner = float(np.sqrt(np.mean(err[inner] ** 2))) if inner.any() else float("nan")

    # roofline: the finest-level Hessian matvec on the same data
    grad, mask0 = CG._grad_vox(CG.pix_to_vox(f_pix, np.float32)[0], wl.shape, np.float32, 0.0)
    v = torch.randn(3 * (Nx + 1) * (Ny + 1) * (Nz + 1), device="cuda", dtype=torch.float32)
    nvox = wl.shape[0] * wl.shape[1] * wl.shape[2]
    ndof = v.numel()
    out = torch.empty_like(v)
    nws = _lib.lib().vdvc_workspace_bytes(_lib.F32, wl.h, Nx, Ny, Nz)
    ws = torch.empty(nws, dtype=torch.uint8, device="cuda")
    L = _lib.lib()

    def mv():
        _lib.check(L.vdvc_matvec_H(v.data_ptr(), grad.data_ptr(), mask0.data_ptr(), _lib.F32, wl.h, Nx, Ny, Nz,
                                   out.data_ptr(), ws.data_ptr(), nws, stream.cuda_stream))

    for _ in range(5):
        mv()
    reps = 50
    m0, m1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    m0.record(stream)
    for _ in range(reps):
        mv()
    m1.record(stream)
    torch.cuda.synchronize()
    mv_ms = m0.elapsed_time(m1) / reps
    alg_bytes = nvox * 13 + ndof * 8
    peaks = {}
    pp = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(pp):
        peaks = json.load(open(pp))
    peak = peaks.get("hbm_gbs", 6800.0)
    achieved = alg_bytes / (mv_ms * 1e-3) / 1e9
    del grad, mask0, ws

    # e2e through the public API with host arrays
    e2e = None
    if args.e2e_steps > 0 and rank == 0:
        f_host = f_pix.cpu().pin_memory().numpy()
        g_host = g_pix.cpu().pin_memory().numpy()
        t_e2e = []
        # one untimed call: host result buffers are pinned once and reused
        CG.multiscale_correlate_gpu(f_host, g_host, Nx, Ny, Nz, wl.h, xp=np, **kw)
        for _ in range(args.e2e_steps):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            Ue, re, de = CG.multiscale_correlate_gpu(f_host, g_host, Nx, Ny, Nz, wl.h, xp=np, **kw)
            t_e2e.append(time.perf_counter() - t0)
        e2e = {"value": round(float(np.median(t_e2e)), 4), "unit": "s",
               "h2d_bytes_per_step": int(f_host.nbytes + g_host.nbytes),
               "d2h_bytes_per_step": int(Ue.nbytes + re.nbytes + de.nbytes)}

    forms = None
    if rank == 0 and world == 1 and not args.no_forms:
        forms = compare_forms(wl, f_pix, g_pix, kw, U, e2e, ms / 1e3)
        del f_pix, g_pix
        torch.cuda.empty_cache()
        forms["batch"] = compare_batch()

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        counts = {"gn": [s["gn_iters"] for s in level_stats], "pcg": [int(sum(s["pcg_iters"])) for s in level_stats]}
        cv, cinfo = cpu_model(wl, counts, args.cpu_sample_layers)
        cpu = {"value": round(cv, 2), "unit": "s", "cores": cinfo["threads"], "kind": "port", "sample": cinfo["sample"],
               "detail": cinfo["levels"]}

    if rank == 0:
        line = {"metric": METRIC, "value": round(ms / 1e3, 4), "unit": "s", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": round(ms, 2), "higher_is_better": False, "scaling": "weak",
                "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                "config": {"workload": wl.name, "mesh": list(wl.mesh), "h": wl.h, "ndof": ndof,
                           "reg": wl.solve["reg_type"], "scales": list(wl.solve["scales"]),
                           "parallelism": f"replicas x{world}", "l2": "inputs (540 MB each) larger than L2"},
                "gpu_launches": int(launches),
                "solve": {"gn_iters": [s["gn_iters"] for s in level_stats],
                          "pcg_iters": [s["pcg_iters"] for s in level_stats],
                          "level_gn_wall_s": [round(s["gn_wall_s"], 4) for s in level_stats],
                          "rms_vs_true_field_vx": round(rms_true, 5),
                          "rms_vs_true_field_inner_vx": round(rms_inner, 5)},
                "roofline": {"bound": "hbm", "kernel": "matvec_H f32 (k_strip_hv_fast + k_gather)",
                             "achieved": round(achieved, 1), "peak": peak, "peak_source": "MEASURED_PEAKS.json hbm_gbs"
                             if "hbm_gbs" in peaks else "fallback 6800", "unit": "GB/s",
                             "frac": round(achieved / peak, 4),
                             # DRAM bytes per launch from ncu on the 257^3 case (14.04 B per
                             # voxel, profiles/strip_hv_fast_f32_necking257.md), scaled to
                             # this launch's voxel count
                             "traffic": int(TRAFFIC_B_PER_VOXEL * nvox),
                             "algorithmic_bytes": int(alg_bytes), "ms": round(mv_ms, 4)},
                "cpu_baseline": cpu, "e2e": e2e, "forms": forms, "clocks": clocks}
        print(json.dumps(line))
    if world > 1:
        dist.destroy_process_group()


def kernels_only(args):
    """Each hot kernel a few times on the 257^3 necking case (h = 8, 32^3
    elements) and its h = 2 level (65^3 voxels after decimation by 4 ...
    here a 129^3 h = 2 mesh of 64^3 elements): the matrix-free Hessian pass
    (strip, h = 8; thread per element, h = 2), the precision form's element
    Hessian formation and matvec, one GN iteration's sampling and residual
    passes (also at the h = 4 and h = 2 levels), the network's forward
    pass.  Prints one line per group."""
    import torch
    from voxeldvc_gb300 import _lib, synth
    from voxeldvc_gb300.engine import correlate_gpu as CG, kernels_dvc as K, geometry_dvc as G
    from voxeldvc_gb300.learned import solve as LS
    reps = max(1, args.steps)
    wl = synth.WORKLOADS["necking_256"]()
    Nx, Ny, Nz = wl.mesh
    f_pix, g_pix = wl.make()
    f_vox, shape = CG.pix_to_vox(f_pix, np.float32)
    grad, mask0 = CG._grad_vox(f_vox, shape, np.float32, 0.0)
    N, w = G.build_N_stencil(wl.h)
    v = torch.randn(3 * (Nx + 1) * (Ny + 1) * (Nz + 1), device="cuda")
    for _ in range(reps):
        K.matvec_H(v, grad.view(-1, 3), mask0, N, w, wl.h, Nx, Ny, Nz, torch)
        K.matvec_H_mixed(v, grad.view(-1, 3), mask0, N, w, wl.h, Nx, Ny, Nz, torch)
    # h = 2 on 64^3 elements (the coarse level of the 513^3 benchmark)
    f2 = synth.texture((129, 129, 129), 80, seed=4)
    g2, m2 = CG._grad_vox(f2, (129, 129, 129), np.float32, 0.0)
    N2, w2 = G.build_N_stencil(2)
    v2 = torch.randn(3 * 65 ** 3, device="cuda")
    for _ in range(reps):
        K.matvec_H(v2, g2.view(-1, 3), m2, N2, w2, 2, 64, 64, 64, torch)
    # one finest-level GN iteration (sampling, residual, b, diag, PCG)
    CG.correlate_gpu(f_pix, g_pix, Nx, Ny, Nz, wl.h, torch, l0=36.0, K_ref_laplacian=G.build_K_ref_laplacian(),
                     dynamic_mask=True, maxiter=reps, eps=0.0, disp=False)
    # the same at the pyramid's h = 4 and h = 2 levels (images decimated by 2
    # and 4, 32^3 elements): the thread-per-element sampling, residual and
    # Hessian passes
    for s in (1, 2):
        d = 2 ** s
        CG.correlate_gpu(f_pix[::d, ::d, ::d].contiguous(), g_pix[::d, ::d, ::d].contiguous(), Nx, Ny, Nz,
                         wl.h // d, torch, l0=36.0 / d, K_ref_laplacian=G.build_K_ref_laplacian(),
                         dynamic_mask=True, maxiter=reps, eps=0.0, disp=False)
    for _ in range(reps):
        LS.learned_seed(f_pix, g_pix, Nx, Ny, Nz, wl.h)
    torch.cuda.synchronize()
    print(json.dumps({"kernels": "done", "reps": reps, "workload": wl.name}))


def learned_only(args):
    """The learned seed + precision form solve of the workload, --warmup
    untimed and --steps timed runs (device-resident inputs), with the GN
    log of the last run: the command behind the launch-list profile of the
    target form."""
    import torch
    from voxeldvc_gb300 import synth
    from voxeldvc_gb300.learned import solve as LS
    wl = synth.WORKLOADS[args.workload]()
    Nx, Ny, Nz = wl.mesh
    f_pix, g_pix = wl.make()
    kwl = {k: v for k, v in solve_kwargs(wl).items() if k not in ("scales", "fft_prealign")}
    net = LS.default_net()
    ts, st = [], []
    for i in range(args.warmup + args.steps):
        st = []
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        U, _, _ = LS.learned_correlate_gpu(f_pix, g_pix, Nx, Ny, Nz, wl.h, torch, net=net, precision="mixed",
                                           stats=st, **kwl)
        torch.cuda.synchronize()
        if i >= args.warmup:
            ts.append(time.perf_counter() - t0)
    gn = [s for s in st if "gn_iters" in s]
    err = (U.double().cpu().numpy() - wl.true_U()).reshape(-1, 3)
    print(json.dumps({"learned_mixed_s": round(float(np.median(ts)), 4), "workload": wl.name,
                      "gn_iters": [s["gn_iters"] for s in gn], "pcg_iters": [s["pcg_iters"] for s in gn],
                      "rms_vs_true_field_vx": round(float(np.sqrt(np.mean(err ** 2))), 5)}))


def eh_form_only(args):
    """The precision form's Hessian matvec (BF16 conversion + element-Hessian
    formation + matvec + gather) on the workload's finest level with each
    formation: CUDA cores (default) and tcgen05 (VDVC_EH_FORM=tc); wall time
    per call (median of --steps) and the relative difference of the results."""
    import torch
    from voxeldvc_gb300 import synth
    from voxeldvc_gb300.engine import correlate_gpu as CG, kernels_dvc as K, geometry_dvc as G
    wl = synth.WORKLOADS[args.workload]()
    Nx, Ny, Nz = wl.mesh
    f_pix, _ = wl.make()
    f_vox, shape = CG.pix_to_vox(f_pix, np.float32)
    grad, mask0 = CG._grad_vox(f_vox, shape, np.float32, 0.0)
    N, w = G.build_N_stencil(wl.h)
    v = torch.randn(3 * (Nx + 1) * (Ny + 1) * (Nz + 1), device="cuda", generator=torch.Generator("cuda").manual_seed(0))
    res, outs = {}, {}
    old = os.environ.get("VDVC_EH_FORM")
    try:
        for form in ("cuda", "tc"):
            os.environ["VDVC_EH_FORM"] = form
            for _ in range(2):
                K.matvec_H_mixed(v, grad.view(-1, 3), mask0, N, w, wl.h, Nx, Ny, Nz, torch)
            ts = []
            for _ in range(max(3, args.steps)):
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                outs[form] = K.matvec_H_mixed(v, grad.view(-1, 3), mask0, N, w, wl.h, Nx, Ny, Nz, torch)
                torch.cuda.synchronize()
                ts.append(time.perf_counter() - t0)
            res[form] = round(float(np.median(ts)) * 1e3, 3)
    finally:
        if old is None:
            os.environ.pop("VDVC_EH_FORM", None)
        else:
            os.environ["VDVC_EH_FORM"] = old
    d = float(torch.linalg.norm(outs["tc"] - outs["cuda"]) / torch.linalg.norm(outs["cuda"]))
    print(json.dumps({"eh_form_matvec_ms": res, "rel_diff_tc_vs_cuda": d, "workload": wl.name}))


def post_only(args):
    """The post-solve stages of `voxeldvc run` on the 257^3 necking case after
    one plain solve: forward push, ZNCC, active mask, per-element strain and
    quality fields, diagnostic masks, and the ground-truth backward warp;
    CUDA-event time per stage (median of --steps) and its algorithmic bytes."""
    import torch
    from voxeldvc_gb300 import synth
    from voxeldvc_gb300.engine import correlate_gpu as CG, kernels_dvc as K, write_output as W
    from voxeldvc_gb300.ground_truth import prepare_ground_truth as PG
    wl = synth.WORKLOADS["necking_256"]()
    Nx, Ny, Nz = wl.mesh
    h = wl.h
    f_pix, g_pix = wl.make()
    kw = solve_kwargs(wl)
    U, res, dU = CG.multiscale_correlate_gpu(f_pix, g_pix, Nx, Ny, Nz, h, xp=torch, **kw)
    nv = tuple(int(s) for s in f_pix.shape)
    Nvox = nv[0] * nv[1] * nv[2]
    Ne = Nx * Ny * Nz
    U_grid = torch.stack([U[c::3].reshape(Nz + 1, Ny + 1, Nx + 1).permute(2, 1, 0) for c in range(3)], -1).double()
    active = CG.compute_active_mask(U, g_pix, Nx, Ny, Nz, h, torch)
    f64 = f_pix.double()
    u_vox = torch.zeros(nv + (3,), dtype=torch.float64, device="cuda")
    u_vox[..., 2] = 0.5
    stages = {
        "push_reference_forward": (lambda: W.push_reference_forward(f_pix, U, Nx, Ny, Nz, h, xp=torch),
                                   Nvox * (4 + 24 + 4 + 4)),
        "compute_zncc": (lambda: W.compute_zncc(f_pix.reshape(-1), g_pix.reshape(-1), active), Nvox * (8 + 8 + 1) * 2),
        "compute_active_mask": (lambda: CG.compute_active_mask(U, g_pix, Nx, Ny, Nz, h, torch), Nvox * (4 + 1)),
        "principal_strains_cell": (lambda: W.compute_principal_strains_cell(U_grid, h), Ne * (24 + 24)),
        "correlation_quality_cell": (lambda: W.compute_correlation_quality_cell(res, f_pix, h, Nx, Ny, Nz),
                                     Nvox * (8 + 4) + Ne * 16),
        "unsafe_masks": (lambda: K.compute_unsafe_voxel_mask(active, h, Nx, Ny, Nz), Nvox * 2),
        "gt_backward_warp": (lambda: PG.make_deformed_image(f64, u_vox, xp=torch), Nvox * (8 + 24 + 8)),
    }
    out = {}
    for name, (fn, nbytes) in stages.items():
        fn()
        ts = []
        for _ in range(max(3, args.steps)):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            e0.record()
            fn()
            e1.record()
            torch.cuda.synchronize()
            ts.append(e0.elapsed_time(e1))
        ms = float(np.median(ts))
        out[name] = {"ms": round(ms, 3), "algorithmic_bytes": int(nbytes), "gbs": round(nbytes / ms / 1e6, 1)}
    print(json.dumps({"post": out, "workload": wl.name, "voxels": Nvox, "elements": Ne,
                      "note": "host results (xp=numpy) are not requested: device tensors, no copies"}))


def ground_truth_only(args):
    """The known-answer pipeline (prepare -> preprocess -> run -> analyse) on
    the seeded 65^3 stand-ins for the reference's two ground-truth datasets,
    h = 8, l0 = 4.5 h: node RMS error over the recoverable and valid sets and
    the wall time of each stage (the first run of a kind includes one-time
    set-up; the second is reported)."""
    import tempfile
    import contextlib
    import io
    from voxeldvc_gb300 import synth
    from voxeldvc_gb300 import run_ground_truth_pipeline as RG
    from voxeldvc_gb300.ground_truth import analyse_ground_truth as AG
    out = {}
    for kind in synth.GT_KINDS:
        ref, U = synth.gt_stand_in(kind)
        with tempfile.TemporaryDirectory() as tmp:
            np.save(os.path.join(tmp, "ref.npy"), ref)
            np.save(os.path.join(tmp, "U.npy"), U)
            walls = []
            for rep in range(2):
                work = os.path.join(tmp, f"run{rep}")
                t0 = time.perf_counter()
                with contextlib.redirect_stdout(io.StringIO()):
                    RG.main(["--output-dir", work, "--gt-ref-file", os.path.join(tmp, "ref.npy"),
                             "--gt-displacement-file", os.path.join(tmp, "U.npy")])
                walls.append(time.perf_counter() - t0)
            with contextlib.redirect_stdout(io.StringIO()):
                st = AG.analyse(work, os.path.join(work, "gt_input"))
        out[kind] = {"rms_recoverable_vx": round(st["recoverable"][1], 5), "rms_valid_vx": round(st["valid"][1], 5),
                     "nodes_recoverable": st["recoverable"][0], "nodes_valid": st["valid"][0],
                     "rms_voxel_valid_vx": round(st.get("voxel_valid_rms", float("nan")), 5),
                     "pipeline_wall_s": round(walls[-1], 3)}
    print(json.dumps({"ground_truth": out, "data": "seeded 65^3 stand-ins (synth.gt_stand_in)", "h": 8,
                      "l0_factor": 4.5}))


def main():
    args = parse()
    if args.impl == "reference":
        reference_arm(args)
    elif args.only == "matvec":
        matvec_only(args)
    elif args.only == "kernels":
        kernels_only(args)
    elif args.only == "ground-truth":
        ground_truth_only(args)
    elif args.only == "post":
        post_only(args)
    elif args.only == "eh-form":
        eh_form_only(args)
    elif args.only == "learned":
        learned_only(args)
    else:
        gpu_arm(args)


if __name__ == "__main__":
    main()
