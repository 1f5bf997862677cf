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
    cval there.  Returns an array of field's shape and dtype.
    Reference: engine/write_output.py:571-608."""
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
    if in_dt.kind in "iu" and in_dt != dt:
        # integer fields: scipy's output conversion (round half away from zero)
        cast = D.empty(out.numel(), np.int16 if in_dt == np.uint16 else in_dt)
        _lib.check(_lib.lib().vdvc_cast_round(out.data_ptr(), out.numel(), D.code_of(in_dt), cast.data_ptr(),
                                              D.stream()), "push_field_forward")
        pushed = cast.view(Nvz, Nvy, Nvx).permute(2, 1, 0)
        host = D.out(pushed, np) if D.wants_host(xp) else pushed
        return host.view(np.uint16) if in_dt == np.uint16 and D.wants_host(xp) else host
    pushed = out.view(Nvz, Nvy, Nvx).permute(2, 1, 0)
    if in_dt != dt:
        pushed = pushed.to(D.torch_dtype(in_dt))
    return D.out(pushed, xp)


def push_reference_forward(ref, U, Nx_e, Ny_e, Nz_e, h, xp=np):
    """ref(x - u(x)): the reference image on the deformed image's grid
    (order 1, mode 'nearest').
    Reference: engine/write_output.py:611-622."""
    return push_field_forward(ref, U, Nx_e, Ny_e, Nz_e, h, order=1, xp=xp)


def compute_zncc(f_flat, g_warped_flat, mask_vox, xp=np):
    """Zero-normalised cross-correlation of f and the warped g over
    mask_vox, float64 sums; NaN for an empty mask or a zero denominator.
    Reference: engine/write_output.py:658-690."""
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


# ---- per-element (cell) fields (write_output.py:256-491) ------------------

def _flat_x(a, dtype):
    """x-fastest flat device copy of a voxel or element array: a 1-D array
    is taken as already flat x-fastest, a 3-D [x, y, z] array is flattened
    in Fortran order (the reference's reshape(-1, order='F'))."""
    nd = len(a.shape) if hasattr(a, "shape") else np.ndim(a)
    if nd == 3 and np.dtype(dtype) in (np.float32, np.float64):
        return CG.pix_to_vox(a, dtype)[0]
    t = D.to_device(a)
    if np.dtype(dtype) == np.uint8 and t.dtype != D.torch().uint8:
        t = (t != 0).to(D.torch().uint8)
    elif np.dtype(dtype) != np.uint8:
        t = t.to(D.torch_dtype(dtype))
    if nd == 3:
        t = t.permute(2, 1, 0)
    return t.contiguous().reshape(-1)


def _cell_grid(t, Nx, Ny, Nz, comps=0):
    """x-fastest element (or node) array -> [i, j, k(, c)] host array."""
    if comps:
        return D.out(t.view(Nz, Ny, Nx, comps).permute(2, 1, 0, 3), np)
    return D.out(t.view(Nz, Ny, Nx).permute(2, 1, 0), np)


def _node_major(U_grid):
    """(Nx+1, Ny+1, Nz+1, 3) displacement grid -> node-major flat float64
    (node x-fastest, component fastest within a node)."""
    t = D.to_device(U_grid, np.float64)
    if t.dim() != 4 or t.shape[3] != 3:
        raise ValueError(f"U_grid must have shape (Nx+1, Ny+1, Nz+1, 3), got {tuple(t.shape)}")
    return t.permute(2, 1, 0, 3).contiguous().reshape(-1)


def compute_principal_strains_cell(U_grid, h):
    """Principal small-strain values e1 >= e2 >= e3 at every element
    centroid, from the Hex8 shape-function gradients scaled by 1/h.
    U_grid: (Nx+1, Ny+1, Nz+1, 3); returns (Nx, Ny, Nz, 3) float64.
    Reference: engine/write_output.py:256-281."""
    Nx, Ny, Nz = (int(n) - 1 for n in U_grid.shape[:3])
    U = _node_major(U_grid)
    ps = D.empty(Nx * Ny * Nz * 3, np.float64)
    _lib.check(_lib.lib().vdvc_cell_strains(U.data_ptr(), int(h), Nx, Ny, Nz, ps.data_ptr(), None, D.stream()),
               "compute_principal_strains_cell")
    return _cell_grid(ps, Nx, Ny, Nz, 3)


def compute_equivalent_strain(principal_strains):
    """Von Mises equivalent strain sqrt(2)/3 sqrt((e1-e2)^2 + (e2-e3)^2 +
    (e3-e1)^2) over the last axis; returns principal_strains.shape[:-1].
    Reference: engine/write_output.py:284-306."""
    shape = tuple(int(s) for s in principal_strains.shape)
    if shape[-1] != 3:
        raise ValueError("the last axis must hold the three principal strains")
    p = D.to_device(principal_strains, np.float64).reshape(-1)
    n = p.numel() // 3
    out = D.empty(n, np.float64)
    _lib.check(_lib.lib().vdvc_equivalent_strain(p.data_ptr(), n, out.data_ptr(), D.stream()),
               "compute_equivalent_strain")
    return D.out(out.view(shape[:-1]), np)


def _cell_call(ref, res, unsafe, h, Nx, Ny, Nz, glt=0.0, material=False, safe=False):
    Ne = Nx * Ny * Nz
    Nvox = (Nx * h + 1) * (Ny * h + 1) * (Nz * h + 1)
    rdt = np.dtype(np.float32) if ref is not None and (D.np_dtype_of(ref) if D.is_tensor(ref) else
                                                       np.asarray(ref).dtype) == np.float32 else np.dtype(np.float64)
    rf = _flat_x(ref, rdt) if ref is not None else None
    rs = _flat_x(res, np.float64) if res is not None else None
    us = _flat_x(unsafe, np.uint8) if unsafe is not None else None
    for name, t in (("ref", rf), ("res", rs), ("unsafe_vox", us)):
        if t is not None and t.numel() != Nvox:
            raise ValueError(f"{name} has {t.numel()} voxels, expected {Nvox}")
    o_mat = D.empty(Ne, np.uint8) if material else None
    o_safe = D.empty(Ne, np.uint8) if safe else None
    o_std = D.empty(Ne, np.float64) if res is not None else None
    o_zn = D.empty(Ne, np.float64) if res is not None else None
    _lib.check(_lib.lib().vdvc_cell_fields(D.ptr(rf), D.code_of(rdt),
                                           D.ptr(rs), D.ptr(us), int(h), Nx, Ny, Nz, float(glt), D.ptr(o_mat),
                                           D.ptr(o_safe), D.ptr(o_std), D.ptr(o_zn), D.stream()), "cell fields")
    return o_mat, o_safe, o_std, o_zn


def compute_material_cell_mask(ref, h, Nx, Ny, Nz, glt=0.0):
    """Per-element bool mask: mean reference grey level over the element's
    (h+1)^3 voxels > glt.  Returns (Nx, Ny, Nz).
    Reference: engine/write_output.py:309-333."""
    m, _, _, _ = _cell_call(ref, None, None, h, Nx, Ny, Nz, glt=glt, material=True)
    return _cell_grid(m.view(D.torch().bool), Nx, Ny, Nz)


def compute_material_cell_mask_eroded(material_cell_mask):
    """One-cell erosion, 26-neighbourhood, the mesh border counting as
    material (binary_erosion with border_value=1).
    Reference: engine/write_output.py:336-349."""
    Nx, Ny, Nz = (int(n) for n in material_cell_mask.shape)
    m = _flat_x(material_cell_mask, np.uint8)
    out = D.empty(Nx * Ny * Nz, np.uint8)
    _lib.check(_lib.lib().vdvc_cell_erode(m.data_ptr(), Nx, Ny, Nz, out.data_ptr(), D.stream()),
               "compute_material_cell_mask_eroded")
    return _cell_grid(out.view(D.torch().bool), Nx, Ny, Nz)


def compute_safe_cell_mask(unsafe_vox, h, Nx, Ny, Nz):
    """Per-element mask, True where none of the element's (h+1)^3 voxels is
    flagged in unsafe_vox (flat x-fastest, or an (Nvx, Nvy, Nvz) grid).
    Reference: engine/write_output.py:352-377."""
    _, s, _, _ = _cell_call(None, None, unsafe_vox, h, Nx, Ny, Nz, safe=True)
    return _cell_grid(s.view(D.torch().bool), Nx, Ny, Nz)


def compute_correlation_quality_cell(res, ref, h, Nx, Ny, Nz):
    """(residual_std_cell, zncc_cell), both (Nx, Ny, Nz): the population std
    of res and the ZNCC of ref and ref - res over each element's active
    voxels (res != 0); NaN below 8 active voxels, and zncc NaN for a zero
    denominator.
    Reference: engine/write_output.py:380-447."""
    _, _, s, z = _cell_call(ref, res, None, h, Nx, Ny, Nz)
    return _cell_grid(s, Nx, Ny, Nz), _cell_grid(z, Nx, Ny, Nz)


def compute_gn_convergence_cell(dU, U, Nx, Ny, Nz):
    """||dU|| / ||U|| over each element's 8 corner nodes (24 DOFs); NaN
    where ||U|| = 0.  dU, U: flat node-major (Ndof,).  Returns (Nx, Ny, Nz).
    Reference: engine/write_output.py:450-491."""
    d = D.to_device(dU, np.float64).reshape(-1)
    u = D.to_device(U, np.float64).reshape(-1)
    Ndof = 3 * (Nx + 1) * (Ny + 1) * (Nz + 1)
    if d.numel() != Ndof or u.numel() != Ndof:
        raise ValueError(f"dU and U must have {Ndof} entries")
    out = D.empty(Nx * Ny * Nz, np.float64)
    _lib.check(_lib.lib().vdvc_cell_gn_convergence(d.data_ptr(), u.data_ptr(), Nx, Ny, Nz, out.data_ptr(), D.stream()),
               "compute_gn_convergence_cell")
    return _cell_grid(out, Nx, Ny, Nz)
