#!/usr/bin/env python
"""Benchmark of the GB300 voxelDVC Gauss-Newton path.

Workload (default `necking_512`): the 513^3 float32 pair of a fiber-composite
texture (5000 cylinders) under tensile necking, h = 8 (64^3 elements,
823,875 dof), Laplacian regularizer with l0 = 4.5 h (the `voxeldvc run`
settings; the equilibrium-gap variant is `--workload necking_512_eqgap`),
3-level pyramid with FFT seed, dynamic mask frozen after 4 iterations.  One
step = one complete plain-FP32 multiscale GN-PCG solve to the reference's
stopping rules.  Data are synthetic and generated on the GPU (seeded); the
inputs (540 MB each) are larger than L2, so no flush is needed.

  value   device-resident solve time (s/solve), CUDA events on the stream
  e2e     the same solve through the public API with ordinary (pageable)
          host numpy inputs: host->device image upload and device->host
          read of (U, res, dU) inside the timed region
  roofline  the finest level's Hessian matvec in the form the solve's PCG
          applies it (element Hessians from the float32 gradient at h >= 6),
          timed with CUDA events right after the timed solves on the same
          data; `roofline_matrix_free` the same for the matrix-free pass (the
          reference's formulation); `traffic` is the DRAM bytes of an ncu
          capture of the 257^3 case scaled to this launch's size
  cpu_baseline  the reference's own operators (voxelDVC's engine on NumPy,
          installed unmodified in baseline/_ref) on slabs of this run's
          arrays over all host cores, assembled into a solve time with this
          solve's GN / PCG counts (labelled extrapolated)

`--impl reference` runs only the reference's CPU leg on the same workload
(generated by the seeded NumPy generator, without this package's GPU
library) and prints the same metric.
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

# DRAM bytes per voxel of one float32 matvec (k_strip_hv_fast<8> + k_gather),
# ncu dram__bytes_read + write on the 257^3 case.
TRAFFIC_B_PER_VOXEL = 14.04

# DRAM bytes per element of one element-Hessian apply, ncu dram__bytes_read
# + write of k_eh_matvec_tma on the 513^3 case itself (the gather's element-
# vector reads hit L2).
TRAFFIC_B_PER_ELEMENT_EH = 709.8

# Operation counts (per pyramid level, coarse to fine: GN iterations, total
# PCG iterations) that the reference arm multiplies its measured operation
# times by: those of the GB300 FP32 solve of each workload, which match the
# reference's own solve where it was run (tests/golden/baseline_*.npz: the
# 513^3 necking workload's coarse level takes 30 GN / 733 PCG iterations
# there, 30 / 752 here).  The GPU arm uses the counts of its own solve.
SOLVE_COUNTS = {"necking_512": {"gn": [30, 4, 2], "pcg": [752, 84, 41]},
                "necking_512_eqgap": {"gn": [30, 30, 30], "pcg": [60000, 60000, 60000]},
                "necking_256": {"gn": [30, 6, 3], "pcg": [732, 106, 55]},
                "plain_small": {"gn": [20, 7, 4], "pcg": [372, 138, 81]},
                "large_1024": {"gn": [30, 30, 3, 2], "pcg": [2179, 1388, 140, 95]}}


def parse(argv=None):
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=3)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--workload", default="necking_512")
    p.add_argument("--e2e-steps", type=int, default=5)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--cpu-sample-layers", type=int, default=None,
                   help="element layers each CPU worker times per pyramid level (default 1)")
    p.add_argument("--cpu-procs", type=int, default=None,
                   help="CPU worker processes (default: every host core this process may use)")
    p.add_argument("--no-forms", action="store_true",
                   help="skip the precision / learned-seed form comparison (FP64 reference solve included)")
    p.add_argument("--only", default=None, choices=[None, "matvec", "kernels", "ground-truth", "post", "eh-form", "learned"],
                   help="matvec: time only the finest-level Hessian matvec; kernels: run each hot kernel of the "
                        "plain, precision and learned forms a few times on the 257^3 case (the profiling commands)")
    return p.parse_args(argv)


def _events_ms(fn, warmup, reps, stream):
    """Mean CUDA-event time (ms) of `reps` back-to-back calls on `stream`."""
    import torch
    for _ in range(warmup):
        fn()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(reps):
        fn()
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / max(1, reps)


def matvec_only(args):
    """Generate the workload's reference image, then run `--warmup` + `--steps`
    finest-level Hessian matvecs -- matrix-free (vdvc_matvec_H) and from
    element Hessians formed once (vdvc_eh_apply) -- and print their mean
    times."""
    import torch
    from voxeldvc_gb300 import _lib, synth
    from voxeldvc_gb300.engine import correlate_gpu as CG, kernels_dvc as K
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

    ms = _events_ms(mv, args.warmup, args.steps, s)
    eh = K.ElementHessians(grad, mask0, wl.h, Nx, Ny, Nz)
    ms_eh = _events_ms(lambda: eh.matvec_into(v, out), args.warmup, args.steps, s)
    eh.status()
    nvox = wl.shape[0] * wl.shape[1] * wl.shape[2]
    ne = Nx * Ny * Nz
    print(json.dumps({"workload": wl.name, "matvec_ms": round(ms, 4),
                      "algorithmic_GBs": round((nvox * 13 + ndof * 8) / ms / 1e6, 1),
                      "eh_apply_ms": round(ms_eh, 4),
                      "eh_apply_algorithmic_GBs": round((ne * 648 + ndof * 8) / ms_eh / 1e6, 1)}))


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
# CPU leg: the reference's own operators (voxelDVC engine on NumPy)
# ---------------------------------------------------------------------------

REF_DIR = os.path.join(ROOT, "baseline", "_ref")

# What the CPU leg needs to know of each workload (the reference arm must not
# load this package's native library, so it does not read voxeldvc_gb300's
# workload table): volume edge, element edge, regularizer, l0, pyramid, the
# seeded NumPy generator case (oracle/workload_inputs.py), the analytic field.
CPU_WORKLOADS = {
    "necking_512": dict(name="necking_513^3_h8", n=513, h=8, reg="laplacian", l0=36.0, scales=(2, 1, 0),
                        case="necking_513", field="necking"),
    "necking_256": dict(name="necking_257^3_h8", n=257, h=8, reg="laplacian", l0=36.0, scales=(2, 1, 0),
                        case="necking_257", field="necking"),
    "plain_small": dict(name="plain_small_129^3_h16", n=129, h=16, reg="laplacian", l0=32.0, scales=(2, 1, 0),
                        case="plain_small", field="plain_small"),
}


def ref_engine():
    """The reference's engine modules (voxelDVC src/voxeldvc/engine/*, installed
    unmodified into baseline/_ref); they import only NumPy and SciPy."""
    if not os.path.isdir(os.path.join(REF_DIR, "voxeldvc", "engine")):
        raise FileNotFoundError("the reference is not installed in baseline/_ref")
    if REF_DIR not in sys.path:
        sys.path.insert(0, REF_DIR)
    from voxeldvc.engine import correlate_gpu as RCG, kernels_dvc as RKD, geometry_dvc as RG
    return RCG, RKD, RG


def _level_field(spec, s, X, Y, Z):
    """The workload's analytic displacement at level-s voxel coordinates, in
    level-s voxels (the pyramid's coarse levels see u(s x) / s)."""
    from oracle import workload_inputs as WI
    if spec["field"] == "necking":
        u = WI.field_necking(X * s, Y * s, Z * s, spec["n"])
    else:
        u = WI.field_plain_small(X * s, Y * s, Z * s)
    return [c / s for c in u]


def _ref_slab_job(job):
    """Seconds of each reference operator on one z slab of one pyramid level
    (one worker of the CPU leg): `L` element layers starting at layer z0 of
    the level's (Nx, Ny, Nz) mesh, cut from the level's images (memory-mapped
    .npy files written by the parent).  The operators are the reference's
    functions called as its correlate_gpu calls them (correlate_gpu.py:
    938-960, 1068-1128; kernels_dvc.py:349-583), on the slab's own arrays:
    gradient and erosion, sampling of g at x + u (u = the analytic field at
    the slab's nodes), the masked statistics, the residual, b, the diagonal,
    the Hessian and regularizer matvecs and the PCG's vector work."""
    tmp, s, Nx, Ny, z0, L, spec = job
    RCG, RKD, RG = ref_engine()
    h = spec["h"] // s
    f = np.load(os.path.join(tmp, f"f{s}.npy"), mmap_mode="r")
    g = np.load(os.path.join(tmp, f"g{s}.npy"), mmap_mode="r")
    nvx, nvy, nvz = f.shape
    v0, v1 = z0 * h, (z0 + L) * h + 1
    t = {}
    # per-level set-up: values, gradient (with a plane of context on each
    # side, as in the whole image), mask0 and its erosion, grad zeroed there
    a0, a1 = max(0, v0 - 1), min(nvz, v1 + 1)
    f_ext = np.ascontiguousarray(f[:, :, a0:a1])
    t0 = time.perf_counter()
    f_vox, grad = RCG.image_grad_and_values(np.asarray(f_ext, dtype=np.float32), np, dtype=np.float32)
    mask0 = f_vox > 0.0
    gm = RCG.erode_mask0_vox(mask0, nvx, nvy, a1 - a0, np)
    grad[~gm] = 0
    t["grad"] = time.perf_counter() - t0
    plane = nvx * nvy
    lo, hi = (v0 - a0) * plane, (v1 - a0) * plane
    f_vox, grad, mask0 = f_vox[lo:hi].copy(), grad[lo:hi].copy(), mask0[lo:hi].copy()
    Ndof = 3 * (Nx + 1) * (Ny + 1) * (L + 1)
    N, w = RG.build_N_stencil(h)
    K_lap = RG.build_K_ref_laplacian()
    # nodal U: the analytic field at the slab's nodes (level units)
    nn = np.arange((Nx + 1) * (Ny + 1) * (L + 1))
    X = (nn % (Nx + 1)) * float(h)
    Y = ((nn // (Nx + 1)) % (Ny + 1)) * float(h)
    Z = (nn // ((Nx + 1) * (Ny + 1)) + z0) * float(h)
    U = np.empty(Ndof, np.float32)
    for c, uc in enumerate(_level_field(spec, s, X, Y, Z)):
        U[c::3] = uc
    # g with a margin of planes around the slab (the deformed positions stay
    # within it: |u_z| + 2 planes); g_origin shifts slab coordinates into it
    m = int(np.ceil(np.max(np.abs(U[2::3])))) + 2
    b0, b1 = max(0, v0 - m), min(nvz, v1 + m)
    g_sl = np.ascontiguousarray(g[:, :, b0:b1])
    origin = (0, 0, b0 - v0)
    t0 = time.perf_counter()
    g_vals, mvox = RCG.sample_deformed_field(U, g_sl, N, h, Nx, Ny, L, np, g_origin=origin, mask0_vox=mask0,
                                             glt=0.0)
    t["sample"] = time.perf_counter() - t0
    t0 = time.perf_counter()
    g_mean, std1 = RCG.masked_quadpoint_mean_std(g_vals, mvox, h, Nx, Ny, L, np)
    t["stats"] = time.perf_counter() - t0
    t0 = time.perf_counter()
    g_vals -= g_mean
    g_vals *= -(1.0 / max(std1, 1e-30))
    g_vals += f_vox
    res = g_vals
    res[~mvox] = 0.0
    t["res"] = time.perf_counter() - t0
    t0 = time.perf_counter()
    b = RCG.compute_b_gpu(res, mvox, grad, N, w, h, Nx, Ny, L, Ndof, np)
    t["b"] = time.perf_counter() - t0
    t0 = time.perf_counter()
    RKD.build_diagonal_H(grad, mvox, N, w, h, Nx, Ny, L, Ndof, np)
    t["diag"] = time.perf_counter() - t0
    t0 = time.perf_counter()
    RKD.build_diagonal_K_ref(K_lap, h, Nx, Ny, L, Ndof, np)
    t["diag_reg"] = time.perf_counter() - t0
    v = b.astype(np.float64)
    t0 = time.perf_counter()
    Hv = RKD.matvec_H(v, grad, mvox, N, w, h, Nx, Ny, L, np)
    t["mv"] = time.perf_counter() - t0
    t0 = time.perf_counter()
    Rv = RKD.matvec_K_ref(v, K_lap, E_elem=h, Nx=Nx, Ny=Ny, Nz=L, xp=np)
    t["reg"] = time.perf_counter() - t0
    # the PCG's own vector work per iteration: the reference's pcg with an
    # identity matvec, per iteration
    Mi = 1.0 / (np.abs(Hv + 0.01 * Rv) + 1.0)
    k = 8
    t0 = time.perf_counter()
    RKD.pcg(lambda x: x, v, Mi, np, max_iter=k, tol=0.0)
    t["vec"] = (time.perf_counter() - t0) / (k + 1)
    return t


def cpu_workers():
    """Host cores this process may use."""
    try:
        return max(1, len(os.sched_getaffinity(0)))
    except AttributeError:
        return max(1, os.cpu_count() or 1)


class RefCpuLeg:
    """The reference's own NumPy execution of the path, timed on this host's
    cores.  The reference's operators loop over element chunks of a whole
    mesh on one core; here every pyramid level's mesh is cut into z slabs
    and `procs` spawned worker processes (one BLAS/OpenMP thread each) time
    the reference functions on their own slab, all at once, so the times
    include the cores' contention for memory bandwidth.  A worker times
    `layers` element layers and its time is scaled to its share of the mesh
    (Nz / procs layers); a full-mesh operation costs the slowest worker's
    scaled time.  The solve time is assembled from the operation times with
    the solve's GN and PCG iteration counts (labelled extrapolated)."""

    def __init__(self, spec, f_pix, g_pix, procs=None, layers=1):
        import multiprocessing as mp
        import tempfile as tf
        self.spec = spec
        self.procs = procs or cpu_workers()
        self.layers = layers
        self.dir = tf.TemporaryDirectory(prefix="vdvc_cpu_")
        for sc in spec["scales"]:
            d = 2 ** sc
            np.save(os.path.join(self.dir.name, f"f{d}.npy"), np.ascontiguousarray(f_pix[::d, ::d, ::d]))
            np.save(os.path.join(self.dir.name, f"g{d}.npy"), np.ascontiguousarray(g_pix[::d, ::d, ::d]))
        keys = ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS", "MKL_NUM_THREADS")
        saved = {k: os.environ.get(k) for k in keys}
        os.environ.update({k: "1" for k in keys})
        try:
            self.pool = mp.get_context("spawn").Pool(self.procs)
        finally:
            for k, v in saved.items():
                if v is None:
                    os.environ.pop(k, None)
                else:
                    os.environ[k] = v

    def close(self):
        self.pool.close()
        self.pool.join()
        self.dir.cleanup()

    def sample(self, counts):
        """One bounded sample: every level's operations on `layers` element
        layers per worker; returns (seconds per solve, detail)."""
        spec, n = self.spec, self.spec["n"]
        Nel = (n - 1) // spec["h"]
        Nx = Ny = Nz = Nel
        procs = min(self.procs, Nz)
        share = Nz / procs                     # layers of the mesh per core
        jobs, where = [], []
        for sc in sorted(spec["scales"], reverse=True):
            d = 2 ** sc
            for p in range(procs):
                z0 = min(Nz - self.layers, int(p * share))
                jobs.append((self.dir.name, d, Nx, Ny, z0, self.layers, spec))
                where.append(d)
        t0 = time.perf_counter()
        res = self.pool.map(_ref_slab_job, jobs)
        wall = time.perf_counter() - t0
        scale = share / self.layers
        levels, total = [], 0.0
        for li, sc in enumerate(sorted(spec["scales"], reverse=True)):
            d = 2 ** sc
            rs = [r for r, w in zip(res, where) if w == d]
            op = {k: max(r[k] for r in rs) * scale for k in rs[0]}
            t_pcg = op["mv"] + op["reg"] + op["vec"]
            # per GN iteration: sampling, stats of g, residual, b - ll R U,
            # diag H + ll diag R, the displayed stats of res
            t_gn = op["sample"] + 2 * op["stats"] + op["res"] + op["b"] + op["reg"] + op["diag"] + op["diag_reg"]
            # per level: gradient, mask erosion, stats of f, lambda calibration
            t_setup = op["grad"] + op["stats"] + op["mv"] + op["reg"]
            n_gn, n_pcg = counts["gn"][li], counts["pcg"][li]
            t_level = t_setup + n_gn * t_gn + (n_pcg + n_gn) * t_pcg
            total += t_level
            levels.append({"h": spec["h"] // d, "matvec_H_s": round(op["mv"], 3), "sample_s": round(op["sample"], 3),
                           "gn_fixed_s": round(t_gn, 3), "level_s": round(t_level, 1)})
        info = {"levels": levels, "sample_wall_s": round(wall, 2), "threads": procs,
                "sample": f"the reference's own operators (voxelDVC engine, NumPy, from baseline/_ref) on the "
                          f"workload's arrays: {procs} worker processes at once, each timing {self.layers} element "
                          f"layer(s) of its own z slab of every pyramid level, scaled to its {share:g}-layer share "
                          f"of the {Nz}-layer mesh, slowest worker per operation; solve time extrapolated with the "
                          f"GN/PCG counts {counts}"}
        return total, info


def ref_counts(workload):
    return SOLVE_COUNTS[workload]


def reference_arm(args):
    """`--impl reference`: the reference's own CPU execution of the path on
    the host cores (rank 0 only), on the same workload, metric and units as
    the GB300 arm.  The workload's pair is generated on the host by the
    seeded NumPy generator (oracle/workload_inputs.py); nothing of this
    package's GPU library is loaded."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    spec = CPU_WORKLOADS.get(args.workload)
    base = {"metric": METRIC, "impl": "reference"}
    if spec is None:
        print(json.dumps(dict(base, unavailable=f"no CPU timing plan for workload {args.workload}")))
        return
    try:
        ref_engine()
    except (FileNotFoundError, ImportError) as e:
        print(json.dumps(dict(base, unavailable=str(e))))
        return
    from oracle import workload_inputs as WI
    t0 = time.perf_counter()
    f_pix, g_pix = WI.CASES[spec["case"]]()
    t_gen = time.perf_counter() - t0
    counts = ref_counts(args.workload)
    leg = RefCpuLeg(spec, f_pix, g_pix, procs=args.cpu_procs, layers=args.cpu_sample_layers or 1)
    del f_pix, g_pix
    vals, info = [], None
    try:
        for i in range(max(0, args.warmup) + max(1, args.steps)):
            v, info = leg.sample(counts)
            if i >= args.warmup:
                vals.append(v)
    finally:
        leg.close()
    value = float(np.median(vals))
    line = dict(base, value=round(value, 2), unit="s", n_gpus=args.gpus, steps=args.steps, warmup=args.warmup,
                ms_per_step=round(value * 1e3, 1), higher_is_better=False, scaling="weak", vs_baseline=None,
                dtype="f32 (the reference promotes b and the PCG to f64 when l0 is set)", data="synthetic",
                config={"workload": spec["name"], "mesh": [(spec["n"] - 1) // spec["h"]] * 3, "h": spec["h"],
                        "reg": spec["reg"], "scales": list(spec["scales"]), "extrapolated": True},
                cpu_baseline={"value": round(value, 2), "unit": "s", "cores": info["threads"], "kind": "reference",
                              "sample": info["sample"]},
                e2e={"value": round(value, 2), "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
                detail=dict(info, input_generation_s=round(t_gen, 1)))
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
            # the previous call's results are released first, as a caller
            # that keeps one result at a time does: host results reuse the
            # pooled pinned buffers instead of fresh pageable memory
            out = None
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            out = fn()
            torch.cuda.synchronize()
            ts.append(time.perf_counter() - t0)
        return float(np.median(ts)), out

    t64, (U64, _, _) = timed(lambda: CG.multiscale_correlate_gpu(f_pix, g_pix, Nx, Ny, Nz, wl.h, xp=torch,
                                                                  dtype=np.float64, **kw), reps=1)
    U64 = U64.double()
    from voxeldvc_gb300.engine import write_output as W

    def rms(U):
        return float(torch.sqrt(torch.mean((U.double() - U64) ** 2)).item())

    def strains(U):
        # principal strains at the element centroids (write_output's cell strains)
        Ug = U.double().reshape(Nz + 1, Ny + 1, Nx + 1, 3).permute(2, 1, 0, 3)
        return np.asarray(W.compute_principal_strains_cell(Ug, wl.h))

    ps64 = strains(U64)

    def strain_rms(U):
        return float(np.sqrt(np.mean((strains(U) - ps64) ** 2)))

    out = {"reference": "GPU FP64 solve of the same inputs", "f64_s": round(t64, 4),
           "target_rms_vx": 0.02, "strain_rms_f64": float(np.sqrt(np.mean(ps64 ** 2))),
           "plain": {"rms_vs_f64_vx": round(rms(U_plain), 6), "strain_rms_vs_f64": strain_rms(U_plain)}}
    tm, (Um, _, _) = timed(lambda: CG.multiscale_correlate_gpu(f_pix, g_pix, Nx, Ny, Nz, wl.h, xp=torch,
                                                                precision="mixed", **kw))
    out["mixed"] = {"s": round(tm, 4), "rms_vs_f64_vx": round(rms(Um), 6), "strain_rms_vs_f64": strain_rms(Um)}
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
    out["learned_mixed"] = {"s": round(tl, 4), "rms_vs_f64_vx": round(rms(Ul), 6), "strain_rms_vs_f64": strain_rms(Ul),
                            "seed": last.get("seed"),
                            "norm_res": last.get("norm_res"), "gn_iters": [s["gn_iters"] for s in gn[-1:]],
                            "pcg_iters": [int(sum(s["pcg_iters"])) for s in gn[-1:]]}
    # the same through the public API with host arrays (ordinary numpy
    # arrays, as the plain e2e)
    f_host = np.array(f_pix.cpu().numpy())
    g_host = np.array(g_pix.cpu().numpy())
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
               rms_vs_true_field_vx_max=round(max(rms), 5), schedule=[s["schedule"] for s in st],
               level_setup_s=[round(s["setup_s"], 4) for s in st], level_gn_wall_s=[round(s["gn_wall_s"], 4) for s in st],
               level_gn_iters_max=[max(s["gn_iters"]) for s in st])
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

    # rooflines: the finest level's Hessian matvec on the same data, in the
    # form the solve's PCG applies (element Hessians from the float32
    # gradient at h >= 6) and matrix-free (the reference's formulation)
    grad, mask0 = CG._grad_vox(CG.pix_to_vox(f_pix, np.float32)[0], wl.shape, np.float32, 0.0)
    v = torch.randn(3 * (Nx + 1) * (Ny + 1) * (Nz + 1), device="cuda", dtype=torch.float32)
    nvox = wl.shape[0] * wl.shape[1] * wl.shape[2]
    ndof = v.numel()
    ne = Nx * Ny * Nz
    out = torch.empty_like(v)
    nws = _lib.lib().vdvc_workspace_bytes(_lib.F32, wl.h, Nx, Ny, Nz)
    ws = torch.empty(nws, dtype=torch.uint8, device="cuda")
    L = _lib.lib()

    def mv():
        _lib.check(L.vdvc_matvec_H(v.data_ptr(), grad.data_ptr(), mask0.data_ptr(), _lib.F32, wl.h, Nx, Ny, Nz,
                                   out.data_ptr(), ws.data_ptr(), nws, stream.cuda_stream))

    mv_ms = _events_ms(mv, 5, 50, stream)
    alg_bytes = nvox * 13 + ndof * 8
    peaks = {}
    pp = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(pp):
        peaks = json.load(open(pp))
    peak = peaks.get("hbm_gbs", 6800.0)
    peak_source = "MEASURED_PEAKS.json hbm_gbs" if "hbm_gbs" in peaks else "fallback 6800"
    achieved = alg_bytes / (mv_ms * 1e-3) / 1e9
    roof_mf = {"bound": "hbm", "kernel": "matvec_H f32 matrix-free (k_strip_hv_fast + k_gather)",
               "achieved": round(achieved, 1), "peak": peak, "peak_source": peak_source, "unit": "GB/s",
               "frac": round(achieved / peak, 4), "traffic": int(TRAFFIC_B_PER_VOXEL * nvox),
               "traffic_source": f"ncu dram bytes of the 257^3 case ({TRAFFIC_B_PER_VOXEL} B per "
                                 f"voxel) scaled to this launch's {nvox} voxels",
               "algorithmic_bytes": int(alg_bytes), "ms": round(mv_ms, 4)}
    roof = roof_mf
    if level_stats and level_stats[-1].get("hessian") == "element":
        eh = K.ElementHessians(grad, mask0, wl.h, Nx, Ny, Nz)
        eh_ms = _events_ms(lambda: eh.matvec_into(v, out), 5, 50, stream)
        eh.status()
        eh_bytes = ne * 648 + ndof * 8
        eh_ach = eh_bytes / (eh_ms * 1e-3) / 1e9
        roof = {"bound": "hbm", "kernel": "matvec_H f32 from element Hessians (k_eh_matvec_tma + k_gather), the "
                                          "finest level's PCG operator",
                "achieved": round(eh_ach, 1), "peak": peak, "peak_source": peak_source, "unit": "GB/s",
                "frac": round(eh_ach / peak, 4),
                "traffic": int(TRAFFIC_B_PER_ELEMENT_EH * ne) if TRAFFIC_B_PER_ELEMENT_EH else None,
                "traffic_source": (f"ncu dram bytes of k_eh_matvec_tma on the 513^3 case ({TRAFFIC_B_PER_ELEMENT_EH} "
                                   f"B per element) times this launch's {ne} elements") if TRAFFIC_B_PER_ELEMENT_EH else
                "not captured",
                "algorithmic_bytes": int(eh_bytes), "ms": round(eh_ms, 4),
                "formation": "once per GN iteration until the b mask freezes (k_eh_form, not in this figure)"}
        del eh
    del grad, mask0, ws

    # e2e through the public API with host arrays: ordinary (pageable) numpy
    # arrays, as `voxeldvc run` hands in what np.load returned
    e2e = None
    f_host = g_host = None
    if rank == 0 and (args.e2e_steps > 0 or not args.no_cpu_baseline):
        f_host = np.array(f_pix.cpu().numpy())
        g_host = np.array(g_pix.cpu().numpy())
    if args.e2e_steps > 0 and rank == 0:
        t_e2e = []
        # one untimed call: the pinned host result buffers (reused once the
        # arrays handed out are released) are allocated here, as in any
        # repeated use
        CG.multiscale_correlate_gpu(f_host, g_host, Nx, Ny, Nz, wl.h, xp=np, **kw)
        gc.collect()
        gc.disable()  # as in the device-timed region
        out = None
        try:
            for _ in range(args.e2e_steps):
                # a caller that keeps one result at a time: the previous
                # call's arrays are released first, so every call returns
                # its results in the same pooled pinned buffers
                out = None
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                out = CG.multiscale_correlate_gpu(f_host, g_host, Nx, Ny, Nz, wl.h, xp=np, **kw)
                t_e2e.append(time.perf_counter() - t0)
        finally:
            gc.enable()
        Ue, re, de = out
        del out
        e2e = {"value": round(float(np.median(t_e2e)), 4), "unit": "s", "samples_s": [round(t, 4) for t in t_e2e],
               "h2d_bytes_per_step": int(f_host.nbytes + g_host.nbytes),
               "d2h_bytes_per_step": int(Ue.nbytes + re.nbytes + de.nbytes)}
        del Ue, re, de  # their pooled host buffers serve the forms' end-to-end calls

    forms = None
    if rank == 0 and world == 1 and not args.no_forms:
        forms = compare_forms(wl, f_pix, g_pix, kw, U, e2e, ms / 1e3)
        del f_pix, g_pix
        torch.cuda.empty_cache()
        forms["batch"] = compare_batch()

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        # the reference's own operators on this run's own arrays, with this
        # solve's GN / PCG counts
        spec = CPU_WORKLOADS.get(args.workload)
        try:
            if spec is None:
                raise KeyError(f"no CPU timing plan for workload {args.workload}")
            ref_engine()
            counts = {"gn": [s["gn_iters"] for s in level_stats],
                      "pcg": [int(sum(s["pcg_iters"])) for s in level_stats]}
            leg = RefCpuLeg(spec, f_host, g_host, procs=args.cpu_procs, layers=args.cpu_sample_layers or 1)
            try:
                cv, cinfo = leg.sample(counts)
            finally:
                leg.close()
            cpu = {"value": round(cv, 2), "unit": "s", "cores": cinfo["threads"], "kind": "reference",
                   "sample": cinfo["sample"], "detail": cinfo["levels"]}
        except (KeyError, FileNotFoundError, ImportError) as e:
            cpu = {"value": None, "unit": "s", "kind": "reference", "unavailable": str(e)}

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
                "roofline": roof, "roofline_matrix_free": roof_mf,
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
                      "du": [[float(f"{d:.3e}") for d in s["du"]] for s in gn], "seed": st[-1].get("seed"),
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
