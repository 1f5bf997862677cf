"""DVC solve seeded by the learned initial guess.

The network's displacement, resampled to the mesh nodes, replaces the coarse
pyramid levels and the FFT shift of `multiscale_correlate_gpu`
(engine/correlate_gpu.py:1143-1305 in the reference): only the finest level
is solved, from that seed.  The plain multiscale solve stays the fallback:
it runs when the registered pair's normalised residual
    rho = mean over the live mask of (f^ - g^)^2 / 2  =  1 - ZNCC
(f^, g^ the standardised reference and deformed values) exceeds
`fallback_threshold` (default 0.05), when the seeded solve stops without
meeting its GN tolerance, or when the two images differ in shape.  A
correctly registered pair sits at the noise floor (rho ~ sigma_n^2 /
(2 sigma_f^2), 0.005 for the benchmark textures); a pair left in a wrong
local minimum is near 1 - ZNCC of unrelated textures.
"""
from __future__ import annotations

import time

import numpy as np

from .. import _device as D
from ..engine import correlate_gpu as CG
from .seednet import SeedNet, WEIGHTS_PATH

_NETS = {}

# Network passes averaged into the seed: the pair itself and its mirror
# image along x (seednet.SeedNet.predict_nodes).  On the 513^3 necking pair
# the mean of the two is 15 % closer to the true field than one pass (0.353
# vs 0.416 vx RMS; four passes 0.302) and the seeded solve stops after 3
# instead of 4 GN iterations; the second pass runs on a side stream.
SEED_PASSES = 2


def default_net(path=WEIGHTS_PATH):
    """The trained network shipped with the package (loaded once per device)."""
    key = (path, D.torch().cuda.current_device())
    if key not in _NETS:
        _NETS[key] = SeedNet.load(path)
    return _NETS[key]


def learned_seed(f_pix, g_pix, Nx, Ny, Nz, h, g_origin=(0, 0, 0), net=None, seed_passes=SEED_PASSES):
    """Seed U (float64 CUDA, Ndof) for the mesh from the (f, g) pair."""
    f_vox, fs = CG.pix_to_vox(f_pix, np.float32)
    g_vox, gs = CG.pix_to_vox(g_pix, np.float32)
    return _seed_vox(f_vox, fs, g_vox, gs, Nx, Ny, Nz, h, g_origin, net, seed_passes)


def _seed_vox(f_vox, fs, g_vox, gs, Nx, Ny, Nz, h, g_origin, net, seed_passes=SEED_PASSES, wait=True):
    """The seed (float64 CUDA, Ndof); wait=False: (seed, event or None), the
    network running on side streams until the caller's stream waits on the
    event."""
    net = net or default_net()
    if tuple(fs) != tuple(gs):
        raise ValueError("the learned seed needs f and g of one shape")
    U0, ready = net.predict_nodes(f_vox, g_vox, fs, h, Nx, Ny, Nz, passes=seed_passes, wait=False)
    if any(o != 0 for o in g_origin):
        # the network sees g in its own array frame: u = u_array + g_origin
        torch = D.torch()
        torch.cuda.current_stream().wait_event(ready)
        ready = None
        U0.view(-1, 3).add_(torch.tensor([float(o) for o in g_origin], dtype=torch.float64, device=U0.device))
    if wait:
        if ready is not None:
            D.torch().cuda.current_stream().wait_event(ready)
        return U0
    return U0, ready


def learned_correlate_gpu(f_pix, g_pix, Nx, Ny, Nz, h, xp, g_origin=(0, 0, 0), l0=None, net=None,
                          fallback_threshold=0.05, scales=(2, 1, 0), fft_prealign=True, stats=None,
                          seed_passes=SEED_PASSES, **kwargs):
    """Finest-level GN solve from the learned seed, with the plain
    multiscale solve as fallback.  Same arguments and returns as
    multiscale_correlate_gpu; `stats` (a list) receives the per-level info
    dicts and a final {'seed': 'learned' | 'fallback', ...} entry."""
    dtype = np.dtype(kwargs.get("dtype", np.float32))
    levels = [] if stats is None else stats
    t0 = time.perf_counter()
    reason = None
    # one layout pass per image: the float32 copies feed both the network
    # and (for a float32 solve) the GN level
    f32, fs = CG.pix_to_vox(f_pix, np.float32)
    g32, gs = CG.pix_to_vox(g_pix, np.float32)
    # the network runs on side streams while this stream sets the level up
    # (gradient, masks, statistics, regularization weight); the GN
    # iterations wait for the seed
    try:
        seed = _seed_vox(f32, fs, g32, gs, Nx, Ny, Nz, h, g_origin, net, seed_passes, wait=False)
    except ValueError as e:
        seed, reason = None, str(e)
    seed_s = time.perf_counter() - t0
    if seed is not None:
        if dtype == np.float32:
            f_vox, g_vox = f32, g32
        else:
            f_vox, fs = CG.pix_to_vox(f_pix, dtype)
            g_vox, gs = CG.pix_to_vox(g_pix, dtype)
        # host results: the residual field is written straight into pinned
        # host memory by the read-back (float64 when regularized or float64)
        res_ent = None
        if D.wants_host(xp) and kwargs.get("maxiter", 30) >= 1:
            res_dt = np.dtype(np.float64) if (l0 is not None or dtype == np.float64) else dtype
            res_ent = D.host_result(fs[0] * fs[1] * fs[2], res_dt)
        U, res, dU, info = CG._solve_level(CG._Level(f_vox, fs, g_vox, gs), Nx, Ny, Nz, h, g_origin=g_origin, l0=l0,
                                           U0_async=seed, stats=levels,
                                           res_dst=None if res_ent is None else res_ent[0], **kwargs)
        rho = info.get("norm_res", float("inf"))
        if np.isfinite(rho) and rho <= fallback_threshold and info.get("converged", False):
            levels.append(dict(seed="learned", norm_res=rho, seed_s=seed_s))
            res_out = D.claim_host_result(res_ent) if res_ent is not None else D.out(res, xp)
            return D.out(U, xp), res_out, D.out(dU, xp)
        reason = f"normalised residual {rho:.4f}" if rho > fallback_threshold or not np.isfinite(rho) \
            else "GN tolerance not met"
    U, res, dU = CG.multiscale_correlate_gpu(f_pix, g_pix, Nx, Ny, Nz, h, xp, scales=scales, g_origin=g_origin,
                                             l0=l0, fft_prealign=fft_prealign, stats=levels, **kwargs)
    levels.append(dict(seed="fallback", reason=reason, seed_s=seed_s))
    return U, res, dU
