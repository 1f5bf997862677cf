"""Pre-processing glue of `voxeldvc preprocess` (preprocess.py of the
reference) on the GPU: the affine warp of the deformed volume onto the
reference grid, integer binning, and the n h + 1 crop of the valid overlap.
Same names, arguments, printed lines and returns as the reference; volumes
are numpy pix[x, y, z] arrays (or CUDA tensors), C order.
"""
from __future__ import annotations

import numpy as np

from . import _device as D
from . import _lib

_BIN_TYPES = {np.dtype(np.float32): _lib.F32, np.dtype(np.uint8): _lib.U8, np.dtype(np.uint16): _lib.U16,
              np.dtype(np.int16): _lib.I16}


def _dev_f32(vol):
    return D.to_device(vol, np.float32).contiguous()


def warp_onto_ref_grid(A, t, c, Nf, g_gpu, xp, chunk=30):
    """g sampled on f's voxel grid at x' = A (x - c) + c + t (trilinear, 0
    outside g).  Returns a float32 numpy array of shape Nf (the reference
    returns host memory too); `chunk` is accepted and ignored -- the warp is
    one pass."""
    Nf = tuple(int(n) for n in Nf)
    g = _dev_f32(g_gpu)
    gs = tuple(int(n) for n in g.shape)
    if len(gs) != 3 or len(Nf) != 3:
        raise ValueError("g and Nf must be 3-D")
    out = D.empty(Nf[0] * Nf[1] * Nf[2], np.float32)
    Ah = np.ascontiguousarray(np.asarray(A, np.float64).reshape(3, 3))
    th = np.ascontiguousarray(np.asarray(t, np.float64).reshape(3))
    ch = np.ascontiguousarray(np.asarray(c, np.float64).reshape(3))
    _lib.check(_lib.lib().vdvc_warp_affine(g.data_ptr(), *gs, Ah.ctypes.data_as(_lib.pd), th.ctypes.data_as(_lib.pd),
                                           ch.ctypes.data_as(_lib.pd), *Nf, out.data_ptr(), D.stream()),
               "warp_onto_ref_grid")
    return D.out(out.view(*Nf), np)


def bin_volume(vol, B):
    """Average-bin by the integer factor B along every axis (float32); the
    shape must be divisible by B."""
    dt = D.np_dtype_of(vol) if D.is_tensor(vol) else np.asarray(vol).dtype
    S0, S1, S2 = (int(s) for s in vol.shape)
    assert S0 % B == 0 and S1 % B == 0 and S2 % B == 0, \
        f"Volume shape {tuple(vol.shape)} not divisible by bin factor {B}"
    if dt not in _BIN_TYPES:
        vol, dt = (vol.to(D.torch().float32) if D.is_tensor(vol) else np.asarray(vol, np.float32)), np.dtype(np.float32)
    v = D.to_device(vol).contiguous()
    out = D.empty((S0 // B) * (S1 // B) * (S2 // B), np.float32)
    _lib.check(_lib.lib().vdvc_bin_volume(v.data_ptr(), _BIN_TYPES[dt], S0, S1, S2, int(B), out.data_ptr(),
                                          D.stream()), "bin_volume")
    return D.out(out.view(S0 // B, S1 // B, S2 // B), np)


def compute_crop(f, g_warped, h, glt=0.0):
    """n h + 1 crop of the valid overlap region (f > glt and g_warped > glt):
    bounding box by axis projections, each dimension snapped down to n h + 1
    and re-centred, shifted into f's bounds.  Returns lo, hi (hi exclusive)."""
    fd, gd = _dev_f32(f), _dev_f32(g_warped)
    n0, n1, n2 = (int(s) for s in fd.shape)
    if tuple(gd.shape) != (n0, n1, n2):
        raise ValueError("f and g_warped must have the same shape")
    p = [D.zeros(n, np.uint8) for n in (n0, n1, n2)]
    _lib.check(_lib.lib().vdvc_overlap_projections(fd.data_ptr(), gd.data_ptr(), n0, n1, n2, float(glt), p[0].data_ptr(),
                                                   p[1].data_ptr(), p[2].data_ptr(), D.stream()), "compute_crop")
    idx = [np.nonzero(D.out(q, np))[0] for q in p]
    if idx[0].size == 0:
        raise RuntimeError("No valid overlap region found")
    lo = np.array([idx[0][0], idx[1][0], idx[2][0]])
    hi = np.array([idx[0][-1], idx[1][-1], idx[2][-1]])
    size = hi - lo + 1
    print(f"  valid overlap AABB : lo={lo}  hi={hi}  size={size}")
    snapped = ((size - 1) // h) * h + 1
    n_elems = (snapped - 1) // h
    print(f"  snapped size (h={h}): {snapped}  (n_elements = {n_elems})")
    mid = (lo + hi) // 2
    lo_out = mid - snapped // 2
    hi_out = lo_out + snapped
    Nf = np.array((n0, n1, n2))
    for i in range(3):
        if lo_out[i] < 0:
            shift = -lo_out[i]
            lo_out[i] += shift
            hi_out[i] += shift
        if hi_out[i] > Nf[i]:
            shift = hi_out[i] - Nf[i]
            lo_out[i] -= shift
            hi_out[i] -= shift
    return lo_out, hi_out
