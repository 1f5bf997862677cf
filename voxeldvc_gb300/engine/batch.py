"""Batched DVC: a series of deformed volumes against one reference, each
with its own region of interest and element size, solved together.

The reference correlates one (f, g) pair per call
(engine/correlate_gpu.py:1143-1305, multiscale_correlate_gpu); this runs the
same multiscale Gauss-Newton solve for every problem of a series, level by
level, with all problems' GN iterations in lockstep through one
`vdvc_gn_batch` (include/vdvc.h): one call per GN iteration, the PCG loops
of all problems in one device-driven CUDA graph, one host synchronisation.
Each problem's arithmetic is exactly that of its own multiscale solve; only
the schedule differs.  Problems leave the lockstep as they converge.

A problem is a dict: origin (x0, y0, z0) of its ROI in voxels of f, element
size h, mesh (Nx, Ny, Nz); its ROI is f[x0 : x0 + Nx h + 1, ...] and the same
box of its deformed image.
"""
from __future__ import annotations

import ctypes as C
import time
from concurrent.futures import ThreadPoolExecutor

import numpy as np

from .. import _device as D
from .. import _lib
from . import correlate_gpu as CG
from . import autotune


def _crop(pix, origin, size):
    x0, y0, z0 = origin
    sx, sy, sz = size
    return pix[x0:x0 + sx, y0:y0 + sy, z0:z0 + sz]


def _check_problem(p, fshape):
    h = int(p["h"])
    Nx, Ny, Nz = (int(v) for v in p["mesh"])
    x0, y0, z0 = (int(v) for v in p["origin"])
    size = (Nx * h + 1, Ny * h + 1, Nz * h + 1)
    if min(h, Nx, Ny, Nz) < 1 or min(x0, y0, z0) < 0 or any(o + s > f for o, s, f in zip((x0, y0, z0), size, fshape)):
        raise ValueError(f"problem {p} does not fit the reference volume {tuple(fshape)}")
    return h, (Nx, Ny, Nz), (x0, y0, z0), size


def batch_multiscale_correlate_gpu(f_pix, g_pixs, problems, xp, scales=(2, 1, 0), l0_factor=None,
                                   fft_prealign=True, K_ref_laplacian=None, dynamic_mask=False,
                                   freeze_mask_after=None, maxiter=30, eps=1e-3, pcg_tol=1e-6, pcg_max_iter=2000,
                                   glt=0.0, tune=False, pcg_chunk=None, concurrent=None, stats=None, disp=False):
    """Solve every problem of the series; returns a list of (U, res, dU) in
    the layout of multiscale_correlate_gpu.  l0_factor: Laplacian length
    l0 = l0_factor * h per problem (None: no regularizer).  Schedule: the
    PCG graph's iterations per body and the stream layout come from
    `pcg_chunk` / `concurrent`, else from the autotuner's cache, else (with
    tune=True) are measured once per problem class and cached
    (engine/autotune.py), else default to (4, concurrent)."""
    if len(g_pixs) != len(problems):
        raise ValueError("one deformed image per problem")
    dtype = np.dtype(np.float32)
    fshape = tuple(int(v) for v in f_pix.shape)
    if len(fshape) != 3:
        raise ValueError(f"expected a 3-D reference volume, got shape {fshape}")
    specs = [_check_problem(p, fshape) for p in problems]
    scales = sorted(set(scales), reverse=True)
    for h, mesh, origin, size in specs:
        for isc in scales:
            if h % (2 ** isc):
                raise ValueError(f"h={h} is not divisible by 2**{isc} (scale {isc})")
    n = len(problems)
    U = [None] * n
    res = [None] * n
    dU = [None] * n
    L = _lib.lib()
    level_info = []
    # each problem's ROI of f and of its g in vox layout, once for all levels
    torch = D.torch()
    t_setup = time.perf_counter()
    rois = [(CG.pix_to_vox(_crop(f_pix, origin, size), dtype), CG.pix_to_vox(_crop(g_pixs[i], origin, size), dtype))
            for i, (h, mesh, origin, size) in enumerate(specs)]
    t_layout = time.perf_counter() - t_setup
    rois_ready = torch.cuda.Event()
    rois_ready.record(torch.cuda.current_stream())

    def build(iscale, fft_seed):
        """Every problem's set-up of one level, on the current stream; the
        seed is the FFT shift (coarsest level) or zero (set from the level
        below once it is solved).  Returns (setups, seconds)."""
        t0 = time.perf_counter()
        s = 2 ** iscale
        setups = []
        for i, (h, mesh, origin, size) in enumerate(specs):
            (f_c, fs), (g_c, gs) = rois[i]
            f_i, fs_i = CG._decimate(f_c, fs, s, dtype)
            g_i, gs_i = CG._decimate(g_c, gs, s, dtype)
            h_i = h // s
            U0 = None
            if fft_seed and fft_prealign:
                # the shift stays on the device: no host synchronisation per problem
                d = CG._fft_shift_device(f_i, fs_i, g_i, gs_i, dtype)
                U0 = CG._uniform_U0(d, (mesh[0] + 1) * (mesh[1] + 1) * (mesh[2] + 1), dtype)
            l0_i = None if l0_factor is None else l0_factor * h / s
            ls = CG._setup_level(CG._Level(f_i, fs_i, g_i, gs_i), *mesh, h_i, glt=glt, l0=l0_i,
                                 K_ref_laplacian=K_ref_laplacian, dynamic_mask=dynamic_mask, U0=U0,
                                 maxiter=maxiter, disp=disp, dtype=dtype, defer=True)
            setups.append(ls)
        # every problem's set-up scalars in one read-back (which also waits
        # for the level's set-up work on this stream)
        scal = torch.stack([ls.dsc for ls in setups]).cpu().numpy()
        for ls, v in zip(setups, scal):
            CG._finish_setup(ls, v)
        return setups, time.perf_counter() - t0

    # once the coarsest level is set up, the finer levels' set-ups run one
    # after another on a side stream and a helper thread while the levels
    # iterate: a set-up needs nothing of the level below but the seed, which
    # is set after the join, and the coarse levels' GN iterations leave the
    # GPU mostly idle (the host thread waits in the stream synchronisation,
    # which releases the interpreter lock).  Starting them alongside the
    # coarsest level's set-up was measured slower (0.198 s for the
    # 16-problem series): two set-ups at once contend for the host and the
    # GPU.
    side = torch.cuda.Stream()
    dev = torch.cuda.current_device()

    def build_on_side(iscale):
        torch.cuda.set_device(dev)
        with torch.cuda.stream(side):
            side.wait_event(rois_ready)
            return build(iscale, False)

    pool = ThreadPoolExecutor(max_workers=1)
    try:
        pending = []
        prev_s = None
        for li, iscale in enumerate(scales):
            s = 2 ** iscale
            if li == 0:
                setups, t_setup = build(iscale, True)
                pending = [pool.submit(build_on_side, isc) for isc in scales[1:]]
            else:
                setups, t_setup = pending[li - 1].result()
                torch.cuda.current_stream().wait_stream(side)
                for i, ls in enumerate(setups):
                    # the seed from the level below, read in the solve dtype
                    ls.U64 = (U[i] * (prev_s / s)).to(D.torch_dtype(dtype)).reshape(-1).to(torch.float64)
            info = _solve_batch(L, setups, specs, dynamic_mask, freeze_mask_after, maxiter, eps, pcg_tol,
                                pcg_max_iter, tune, pcg_chunk, concurrent, disp)
            info.update(scale=iscale, setup_s=t_setup, layout_s=t_layout if li == 0 else 0.0)
            level_info.append(info)
            for i, ls in enumerate(setups):
                U[i], res[i], dU[i] = ls.result
            prev_s = s
    finally:
        pool.shutdown(wait=True, cancel_futures=True)
    if stats is not None:
        stats.extend(level_info)
    return [(D.out(U[i], xp), D.out(res[i], xp), D.out(dU[i], xp)) for i in range(n)]


def _solve_batch(L, setups, specs, dynamic_mask, freeze_mask_after, maxiter, eps, pcg_tol, pcg_max_iter, tune,
                 pcg_chunk, concurrent, disp):
    n = len(setups)
    descs = (_lib.GnDesc * n)(*[ls.desc for ls in setups])
    for d in descs:
        # the solvers' own set-up runs on this thread's stream (the set-ups
        # may have been built on the helper thread's side stream, which by
        # now carries the next level's set-up)
        d.stream = D.stream()
    ws = (C.c_void_p * n)(*[ls.ws.data_ptr() for ls in setups])
    wsb = (C.c_size_t * n)(*[ls.nbytes for ls in setups])
    key = autotune.batch_key([(ls.h, specs[i][1]) for i, ls in enumerate(setups)])
    chunk, conc = autotune.lookup(key) if (pcg_chunk is None and concurrent is None) else (None, None)
    cached = chunk is not None
    chunk = pcg_chunk or chunk or 4
    conc = (1 if concurrent is None else int(bool(concurrent))) if conc is None else conc
    batch = C.c_void_p()
    _lib.check(L.vdvc_gn_batch_create(descs, n, ws, wsb, int(chunk), int(conc), C.byref(batch)), "batch_create")
    st = D.stream()
    info = {"n": n, "gn_iters": [0] * n, "pcg_iters": [[] for _ in range(n)], "h": [ls.h for ls in setups]}
    t0 = time.perf_counter()
    try:
        solvers = []
        for i, ls in enumerate(setups):
            sv = C.c_void_p()
            _lib.check(L.vdvc_gn_batch_solver(batch, i, C.byref(sv)), "batch_solver")
            solvers.append(sv)
            _lib.check(L.vdvc_gn_set_U(sv, ls.U64.data_ptr(), st), "set_U")
            if not dynamic_mask:
                _lib.check(L.vdvc_gn_frozen_diag(sv, st), "frozen_diag")
        if tune and not cached and pcg_chunk is None and concurrent is None and maxiter > 0:
            chunk, conc = autotune.tune_batch(L, batch, solvers, setups, pcg_max_iter, pcg_tol, key, st)
        info["schedule"] = {"pcg_chunk": int(chunk), "concurrent": int(conc)}
        active = np.ones(n, dtype=np.int32)
        frozen = np.zeros(n, dtype=bool)
        out = np.zeros(12 * n, dtype=np.float64)
        errs = np.full(n, np.inf)
        for ik in range(maxiter):
            freeze = np.zeros(n, dtype=np.int32)
            if freeze_mask_after is not None and ik >= freeze_mask_after:
                freeze = ((~frozen) & (active != 0)).astype(np.int32)
            _lib.check(L.vdvc_gn_batch_iterate(batch, active.ctypes.data, freeze.ctypes.data, int(pcg_max_iter),
                                               float(pcg_tol), out.ctypes.data, st), "batch_iterate")
            frozen |= freeze.astype(bool)
            o = out.reshape(n, 12)
            for i in np.nonzero(active)[0]:
                if int(o[i, 11]) == _lib.ERR_ZERO_DIVISION:
                    raise ZeroDivisionError(f"problem {i}: float division by zero (std of g over the b mask is 0)")
                info["gn_iters"][i] = ik + 1
                info["pcg_iters"][i].append(int(o[i, 8]))
                with np.errstate(divide="ignore", invalid="ignore"):
                    errs[i] = float(np.sqrt(o[i, 0]) / np.sqrt(o[i, 1]))
                if disp:
                    print(f"[{i}] " + CG._gn_scalars_line(o[i], ik, errs[i], setups[i].Nvox))
                if errs[i] < eps:
                    active[i] = 0
            if not active.any():
                break
        info["converged"] = [bool(e < eps) for e in errs]
        info["norm_res"] = [CG._norm_res(out.reshape(n, 12)[i], setups[i].std0) for i in range(n)]
        for i, ls in enumerate(setups):
            f64 = int(ls.out_dt == np.float64)
            Uo = D.empty(ls.Ndof, ls.out_dt)
            r = D.empty(ls.Nvox, ls.out_dt)
            d = D.empty(ls.Ndof, ls.out_dt)
            _lib.check(L.vdvc_gn_read(solvers[i], _lib.GN_U, Uo.data_ptr(), f64, st), "read")
            _lib.check(L.vdvc_gn_read(solvers[i], _lib.GN_RES, r.data_ptr(), f64, st), "read")
            _lib.check(L.vdvc_gn_read(solvers[i], _lib.GN_DU, d.data_ptr(), f64, st), "read")
            ls.result = (Uo, r, d)
    finally:
        L.vdvc_gn_batch_destroy(batch)
        D.torch().cuda.current_stream().synchronize()
    info["gn_wall_s"] = time.perf_counter() - t0
    return info
