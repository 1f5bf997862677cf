"""Post-solve voxel stages of the `voxeldvc run` outputs
(engine/write_output.py of the reference), on the GPU.

push_field_forward / push_reference_forward (write_output.py:571-625): a
voxel field pushed forward by the recovered displacement, field(x - u(x)),
with u the FE-interpolated displacement (interp_field_vox) and the
map_coordinates order / mode / cval semantics of the reference
(`vdvc_push_field`).  compute_zncc (write_output.py:658-690): the
zero-normalised cross-correlation quality figure (`vdvc_zncc`).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from .. import _device as D
from .. import _lib
from . import correlate_gpu as CG

_MODES = {"nearest": 0, "constant": 1}


def push_field_forward(field, U, Nx_e, Ny_e, Nz_e, h, order=1, mode='nearest', cval=0.0, xp=np):
    """field_pushed(x) = field(x - u(x)) on the (Nvx, Nvy, Nvz) voxel grid.
    order 0 (nearest; for label / mask fields) or 1 (trilinear); mode
    'nearest' clamps out-of-domain lookups to the edge, 'constant' writes
    cval there.  Returns an array of field's shape and dtype."""
    if order not in (0, 1):
        raise ValueError("order must be 0 or 1")
    if mode not in _MODES:
        raise ValueError(f"mode must be one of {sorted(_MODES)}")
    shape = tuple(int(s) for s in (field.shape if hasattr(field, "shape") else np.shape(field)))
    Nvx, Nvy, Nvz = Nx_e * h + 1, Ny_e * h + 1, Nz_e * h + 1
    if shape != (Nvx, Nvy, Nvz):
        raise ValueError(f"field has shape {shape}, expected {(Nvx, Nvy, Nvz)}")
    in_dt = D.np_dtype_of(field) if D.is_tensor(field) else np.asarray(field).dtype
    dt = np.dtype(np.float32) if in_dt == np.float32 else np.dtype(np.float64)
    f_vox, _ = CG.pix_to_vox(field, dt)
    Ud = D.to_device(U, np.float64).reshape(-1)
    u_cf = CG.interp_field_vox(Ud, None, h, Nx_e, Ny_e, Nz_e, D.torch(), channels_first=True)
    out = D.empty(Nvx * Nvy * Nvz, dt)
    _lib.check(_lib.lib().vdvc_push_field(f_vox.data_ptr(), D.code_of(dt), u_cf.data_ptr(), Nvx, Nvy, Nvz, int(order),
                                          _MODES[mode], float(cval), out.data_ptr(), D.stream()), "push_field_forward")
    pushed = out.view(Nvz, Nvy, Nvx).permute(2, 1, 0)
    if in_dt != dt:
        pushed = pushed.to(D.torch_dtype(in_dt))
    return D.out(pushed, xp)


def push_reference_forward(ref, U, Nx_e, Ny_e, Nz_e, h, xp=np):
    """ref(x - u(x)): the reference image on the deformed image's grid
    (order 1, mode 'nearest')."""
    return push_field_forward(ref, U, Nx_e, Ny_e, Nz_e, h, order=1, xp=xp)


def compute_zncc(f_flat, g_warped_flat, mask_vox, xp=np):
    """Zero-normalised cross-correlation of f and the warped g over
    mask_vox, float64 sums; NaN for an empty mask or a zero denominator."""
    f = D.to_device(f_flat, np.float64).reshape(-1)
    g = D.to_device(g_warped_flat, np.float64).reshape(-1)
    m = D.mask_u8(mask_vox).reshape(-1)
    if not (f.numel() == g.numel() == m.numel()):
        raise ValueError("f_flat, g_warped_flat and mask_vox must have the same length")
    ws = D.scratch.get(1 << 16)
    out = C.c_double(0.0)
    _lib.check(_lib.lib().vdvc_zncc(f.data_ptr(), g.data_ptr(), _lib.F64, m.data_ptr(), f.numel(), C.byref(out),
                                    ws.data_ptr(), ws.numel(), D.stream()), "compute_zncc")
    return float(out.value)
