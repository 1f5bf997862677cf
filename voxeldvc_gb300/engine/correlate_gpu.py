"""Matrix-free Gauss-Newton DVC correlation on the GPU.

Drop-in counterpart of the reference module engine/correlate_gpu.py: the
same public functions with the same arguments and printed output.  The GN
iteration itself runs in a device-resident solver object of libvdvc.so
(one sample/rhs/pcg/update round per iteration, one host read-back of a
few scalars per iteration); images travel to the GPU once and the pyramid
levels are decimated there.

`xp` chooses the type of the returned arrays (numpy -> numpy, anything else
-> torch CUDA tensors).  Images may be numpy arrays or torch tensors in the
reference's pix[x,y,z] C-order layout.
"""
from __future__ import annotations

import ctypes as C
import threading
import time

import numpy as np

from .. import _device as D
from .. import _lib
from .geometry_dvc import build_N_stencil, build_interior_dof_mask
from . import kernels_dvc as K


# ---------------------------------------------------------------------------
# image layout helpers
# ---------------------------------------------------------------------------

def _pix_code_and_tensor(pix):
    """(device tensor holding pix's bytes, libvdvc element code, shape)."""
    T = D.torch()
    if D.is_tensor(pix):
        t = pix if pix.is_cuda else pix.to(D.device())
        t = t.contiguous()
        npd = D.np_dtype_of(t)
        if npd == np.bool_:
            t = t.to(T.uint8)
            npd = np.dtype(np.uint8)
        if npd == np.int64:
            t = t.to(T.int32)
            npd = np.dtype(np.int32)
        return t, D.code_of(npd), tuple(t.shape)
    a = np.asarray(pix)
    if a.dtype == np.bool_:
        a = a.astype(np.uint8)
    if a.dtype not in (np.float32, np.float64, np.uint8, np.uint16, np.int16, np.int32):
        a = a.astype(np.float64)
    a = np.ascontiguousarray(a)
    shape = a.shape
    raw = T.from_numpy(a.reshape(-1).view(np.uint8)).to(D.device())
    return raw, D.code_of(a.dtype), shape


# Host arrays at least this large are read by the transpose kernel in place
# where the device reads pageable host memory (no staged copy).
_DIRECT_MIN_BYTES = 1 << 20
_direct = {}


def _host_direct():
    dev = D.torch().cuda.current_device()
    if dev not in _direct:
        _direct[dev] = bool(_lib.lib().vdvc_device_reads_pageable(dev))
    return _direct[dev]


def pix_to_vox(pix, dtype=np.float32):
    """Device copy of pix[x,y,z] in vox layout (x fastest), cast to dtype.
    Returns (tensor (Nvox,), shape).  A large host array is read in place by
    the transpose kernel where the device reads pageable host memory
    (vdvc_device_reads_pageable), else staged through a device copy."""
    if _host_readable(pix):
        a = np.asarray(pix)
        nx, ny, nz = a.shape
        out = D.empty(nx * ny * nz, dtype)
        _lib.check(_lib.lib().vdvc_pix_to_vox(a.ctypes.data, D.code_of(a.dtype), nx, ny, nz, out.data_ptr(),
                                              D.code_of(dtype), D.stream()), "pix_to_vox")
        # the kernel reads `a`: finish before the caller may free or change it
        D.torch().cuda.current_stream().synchronize()
        return out, (nx, ny, nz)
    t, code, shape = _pix_code_and_tensor(pix)
    if len(shape) != 3:
        raise ValueError(f"expected a 3-D volume, got shape {shape}")
    nx, ny, nz = shape
    out = D.empty(nx * ny * nz, dtype)
    _lib.check(_lib.lib().vdvc_pix_to_vox(t.data_ptr(), code, nx, ny, nz, out.data_ptr(), D.code_of(dtype),
                                          D.stream()), "pix_to_vox")
    return out, (nx, ny, nz)


def _host_readable(pix):
    """pix is a host array that the layout kernel may read in place."""
    if D.is_tensor(pix):
        return False
    a = np.asarray(pix)
    return (a.ndim == 3 and a.nbytes >= _DIRECT_MIN_BYTES and a.flags.c_contiguous and
            a.dtype in (np.float32, np.float64, np.uint8, np.uint16, np.int16, np.int32) and _host_direct())


def _pix_to_vox_strided_host(a, s, dtype):
    """Vox layout of a[::s, ::s, ::s] read in place from the host array `a`
    (the caller keeps `a` alive until the current stream has finished)."""
    nx, ny, nz = a.shape
    o = ((nx + s - 1) // s, (ny + s - 1) // s, (nz + s - 1) // s)
    out = D.empty(o[0] * o[1] * o[2], dtype)
    _lib.check(_lib.lib().vdvc_pix_to_vox_strided(a.ctypes.data, D.code_of(a.dtype), nx, ny, nz, s, 0,
                                                  out.data_ptr(), D.code_of(dtype), D.stream()), "pix_to_vox_strided")
    return out, o


_LAYOUT_STREAMS = {}
_BACKGROUND_LAYOUT_BLOCKS = 2 * 152  # two 256-thread blocks per SM of a GB300


def _layout_stream():
    torch = D.torch()
    key = torch.cuda.current_device()
    if key not in _LAYOUT_STREAMS:
        _LAYOUT_STREAMS[key] = torch.cuda.Stream()
    return _LAYOUT_STREAMS[key]


def _vox_to_pix_host(vox, shape):
    return D.out(vox, np).reshape(shape[2], shape[1], shape[0]).transpose(2, 1, 0)


def _decimate(vox, shape, s, dtype):
    nx, ny, nz = shape
    if s == 1:
        return vox, shape
    o = ((nx + s - 1) // s, (ny + s - 1) // s, (nz + s - 1) // s)
    out = D.empty(o[0] * o[1] * o[2], dtype)
    _lib.check(_lib.lib().vdvc_decimate(vox.data_ptr(), D.code_of(dtype), nx, ny, nz, s, out.data_ptr(),
                                        D.stream()), "decimate")
    return out, o


def _dot(a, b=None):
    """float64 sum(a*b) or sum(a) on the device (one host sync)."""
    dt = D.np_dtype_of(a)
    ws = D.scratch.get(1 << 16)
    out = C.c_double(0.0)
    _lib.check(_lib.lib().vdvc_dot(a.data_ptr(), D.ptr(b), D.code_of(dt), a.numel(), C.byref(out), ws.data_ptr(),
                                   ws.numel(), D.stream()), "dot")
    return out.value


# ---------------------------------------------------------------------------
# reference-image preparation (correlate_gpu.py:49-157)
# ---------------------------------------------------------------------------

def _grad_vox(f_vox, shape, dtype, glt=None):
    nx, ny, nz = shape
    grad = D.empty(3 * nx * ny * nz, dtype)
    mask0 = D.empty(nx * ny * nz, np.uint8) if glt is not None else None
    _lib.check(_lib.lib().vdvc_image_grad(f_vox.data_ptr(), D.code_of(dtype), nx, ny, nz,
                                          float(glt if glt is not None else 0.0), grad.data_ptr(), D.ptr(mask0),
                                          D.stream()), "image_grad")
    return grad, mask0


def image_grad_and_values(pix, xp, dtype=np.float32):
    """(f_vox (Nvox,), grad_f_vox (Nvox, 3)): values and xp.gradient of the
    image, x-fastest voxel order.
    Reference: engine/correlate_gpu.py:49-72."""
    dtype = np.dtype(dtype)
    f_vox, shape = pix_to_vox(pix, dtype)
    grad, _ = _grad_vox(f_vox, shape, dtype)
    return D.out(f_vox, xp), D.out(grad.reshape(-1, 3), xp)


def erode_mask0_vox(mask0_vox, Nvx, Nvy, Nvz, xp):
    """6-neighbour erosion (minimum filter, mode 'nearest') of a voxel mask.
    Reference: engine/correlate_gpu.py:75-94."""
    m = D.mask_u8(mask0_vox).reshape(-1)
    if m.numel() != Nvx * Nvy * Nvz:
        raise ValueError("mask size does not match (Nvx, Nvy, Nvz)")
    out = D.empty(m.numel(), np.uint8)
    _lib.check(_lib.lib().vdvc_erode_mask(m.data_ptr(), Nvx, Nvy, Nvz, out.data_ptr(), D.stream()), "erode")
    return D.out(out.to(D.torch().bool), xp)


def _stats_sums(field, mask, h, Nx, Ny, Nz, out=None):
    """count, s1, s2 of field over mask (multiplicity-weighted, float64):
    host values, or into the device buffer `out` (3 doubles, no sync)."""
    dt = D.np_dtype_of(field)
    sums = D.empty(3, np.float64) if out is None else out
    ws = D.scratch.get(1 << 16)
    _lib.check(_lib.lib().vdvc_masked_stats(field.data_ptr(), D.code_of(dt), mask.data_ptr(), h, Nx, Ny, Nz,
                                            sums.data_ptr(), ws.data_ptr(), ws.numel(), D.stream()), "masked_stats")
    return sums.cpu().numpy() if out is None else None


def _dot_into(a, b, out):
    """float64 sum(a*b) into the device double `out` (no sync)."""
    dt = D.np_dtype_of(a)
    ws = D.scratch.get(1 << 16)
    _lib.check(_lib.lib().vdvc_dot_device(a.data_ptr(), D.ptr(b), D.code_of(dt), a.numel(), out.data_ptr(),
                                          ws.data_ptr(), ws.numel(), D.stream()), "dot")


def _mean_std(c, s1, s2):
    # engine/correlate_gpu.py:152-157
    if c < 1:
        return 0.0, 0.0
    mean = float(s1) / c
    var = float(s2) / c - mean * mean
    return mean, (var if var > 0.0 else 0.0) ** 0.5


def masked_quadpoint_mean_std(field_vox, mask_vox, h, Nx, Ny, Nz, xp, chunk_size=None):
    """Mean and population std of field_vox over the (element, stencil
    point) array restricted to mask_vox (float64 sums).
    Reference: engine/correlate_gpu.py:113-157."""
    dt = K._float_dtype(field_vox)
    f = D.to_device(field_vox, dt).reshape(-1)
    m = D.mask_u8(mask_vox).reshape(-1)
    c, s1, s2 = _stats_sums(f, m, h, Nx, Ny, Nz)
    return _mean_std(c, s1, s2)


def gather_quadpoint_values(field_vox, h, Nx, Ny, Nz, xp):
    """(Ne*(h+1)^3,) per-(element, stencil point) copy of a voxel field.
    A host-side index gather kept for API compatibility (the solve itself
    never materialises it).
    Reference: engine/correlate_gpu.py:97-110."""
    vals = np.asarray(D.out(D.to_device(field_vox), np)).reshape(-1)
    Ne = Nx * Ny * Nz
    offs = np.asarray(K.get_voxel_offsets(h, Nx, Ny, np))
    org = np.asarray(K.get_elem_voxel_origins(np.arange(Ne, dtype=np.int32), h, Nx, Ny, np))
    out = vals[(org[:, None] + offs[None, :]).reshape(-1)]
    return out if D.wants_host(xp) else D.to_device(out)


def interp_field_vox(U, N_stencil, h, Nx, Ny, Nz, xp, chunk_size=200_000, channels_first=False):
    """u(x) = sum_a N_a U_a at every voxel centre: (Nvox, 3) or (3, Nvox).
    Reference: engine/correlate_gpu.py:160-198."""
    dt = K._float_dtype(U)
    Ud = D.to_device(U, dt).reshape(-1)
    Nvox, Ndof = K._mesh_sizes(h, Nx, Ny, Nz)
    if Ud.numel() != Ndof:
        raise ValueError(f"U has {Ud.numel()} entries, expected {Ndof}")
    out = D.empty(3 * Nvox, dt)
    _lib.check(_lib.lib().vdvc_interp_field(Ud.data_ptr(), D.code_of(dt), h, Nx, Ny, Nz, int(bool(channels_first)),
                                            out.data_ptr(), D.stream()), "interp_field_vox")
    out = out.reshape(3, Nvox) if channels_first else out.reshape(Nvox, 3)
    return D.out(out, xp)


def _sample(U, g_vox, gshape, h, Nx, Ny, Nz, g_origin, mask0, glt, dt):
    Nvox, Ndof = K._mesh_sizes(h, Nx, Ny, Nz)
    g_vals = D.empty(Nvox, dt)
    mask = D.empty(Nvox, np.uint8)
    gx0, gy0, gz0 = g_origin
    _lib.check(_lib.lib().vdvc_sample_deformed(U.data_ptr(), g_vox.data_ptr(), D.code_of(dt), gshape[0], gshape[1],
                                               gshape[2], float(gx0), float(gy0), float(gz0), D.ptr(mask0),
                                               float(glt), h, Nx, Ny, Nz, g_vals.data_ptr(), mask.data_ptr(),
                                               D.stream()), "sample_deformed_field")
    return g_vals, mask


def sample_deformed_field(U, g_pix_x, N_stencil, h, Nx, Ny, Nz, xp, g_origin=(0, 0, 0), mask0_vox=None,
                          chunk_size=None, glt=0.0):
    """(g_vals, mask_vox): g sampled at x + u(x) (order-1, clipped) and the
    active mask in_bounds & mask0 & g > glt.
    Reference: engine/correlate_gpu.py:201-281."""
    dt = K._float_dtype(U)
    Ud = D.to_device(U, dt).reshape(-1)
    g_vox, gshape = pix_to_vox(g_pix_x, dt)
    m0 = None if mask0_vox is None else D.mask_u8(mask0_vox).reshape(-1)
    g_vals, mask = _sample(Ud, g_vox, gshape, h, Nx, Ny, Nz, g_origin, m0, glt, dt)
    return D.out(g_vals, xp), D.out(mask.to(D.torch().bool), xp)


def compute_active_mask(U, g_pix, Nx, Ny, Nz, h, xp, g_origin=(0, 0, 0), mask0_vox=None, glt=0.0):
    """Per-voxel active mask (mask0 & in_bounds(x+u) & g(x+u) > glt).
    Reference: engine/correlate_gpu.py:284-338."""
    _, mask = sample_deformed_field(U, g_pix, None, h, Nx, Ny, Nz, D.torch(), g_origin=g_origin,
                                    mask0_vox=mask0_vox, glt=glt)
    return D.out(mask, xp)


def compute_b_gpu(res_vox, mask_vox, grad_f_vox, N_stencil, w_stencil, h, Nx, Ny, Nz, Ndof, xp, chunk_size=None):
    """b = sum_e P_e^T sum_q w_q m_q res_q N_q (x) grad f_q.
    Reference: engine/correlate_gpu.py:341-378."""
    K._check_stencil(N_stencil, w_stencil, h)
    Nvox, nd = K._mesh_sizes(h, Nx, Ny, Nz)
    dt = K._float_dtype(grad_f_vox)
    cdt = K._float_dtype(grad_f_vox, res_vox)
    g, m = K._grad_mask(grad_f_vox, mask_vox, cdt, Nvox)
    r = D.to_device(res_vox, cdt).reshape(-1)
    out = D.empty(Ndof, cdt)
    ws, n = K._ws(cdt, h, Nx, Ny, Nz)
    _lib.check(_lib.lib().vdvc_compute_b(r.data_ptr(), m.data_ptr(), g.data_ptr(), D.code_of(cdt), h, Nx, Ny, Nz,
                                         out.data_ptr(), ws.data_ptr(), n, D.stream()), "compute_b_gpu")
    if cdt != dt:
        out = out.to(D.torch_dtype(dt))  # the reference accumulates into a grad-dtype array
    return D.out(out, xp)


# ---------------------------------------------------------------------------
# FFT pre-alignment (correlate_gpu.py:381-414)
# ---------------------------------------------------------------------------

def _fft_shift_vox(f_vox, fshape, g_vox, gshape, dt):
    d = (C.c_double * 3)()
    _lib.check(_lib.lib().vdvc_fft_rigid_shift(f_vox.data_ptr(), *fshape, g_vox.data_ptr(), *gshape, D.code_of(dt),
                                               C.cast(d, _lib.pd), D.stream()), "fft_rigid_shift")
    return np.array([d[0], d[1], d[2]], dtype=np.float64)


def _fft_shift_device(f_vox, fshape, g_vox, gshape, dt):
    """The shift as a float64 CUDA tensor of 3, left on the device (no host
    synchronisation)."""
    d = D.empty(3, np.float64)
    _lib.check(_lib.lib().vdvc_fft_rigid_shift_device(f_vox.data_ptr(), *fshape, g_vox.data_ptr(), *gshape,
                                                      D.code_of(dt), d.data_ptr(), D.stream()), "fft_rigid_shift")
    return d


def _uniform_U0(d, n_nodes, dtype):
    """Nodal field equal to the shift d (device, 3) at every node, in dtype."""
    return d.to(D.torch_dtype(dtype)).repeat(n_nodes)


def fft_rigid_shift(f_pix, g_pix, xp):
    """Integer voxel shift d with g(x) ~= f(x - d) by phase correlation.
    Reference: engine/correlate_gpu.py:381-414."""
    f_vox, fs = pix_to_vox(f_pix, np.float64)
    g_vox, gs = pix_to_vox(g_pix, np.float64)
    return _fft_shift_vox(f_vox, fs, g_vox, gs, np.float64)


# ---------------------------------------------------------------------------
# Gauss-Newton solve at one level (correlate_gpu.py:828-1140)
# ---------------------------------------------------------------------------

class _Level:
    """Device inputs of one pyramid level, kept alive for the solver."""

    def __init__(self, f_vox, fshape, g_vox, gshape):
        self.f_vox, self.fshape, self.g_vox, self.gshape = f_vox, fshape, g_vox, gshape


def _plane_wave(Nx, Ny, Nz, h, dtype):
    # V = cos(j h / T 2 pi) on the x components, T = 10 h, evaluated in the
    # solve dtype (correlate_gpu.py:1016-1020)
    T = 10 * h
    nn = (Nx + 1) * (Ny + 1) * (Nz + 1)
    jj = (np.arange(nn) // (Nx + 1)) % (Ny + 1)
    Vs = np.cos(jj.astype(dtype) * h / T * 2 * np.pi)
    V = np.zeros(3 * nn, dtype=dtype)
    V[0::3] = Vs
    return V


# Device copies of the calibration plane wave, per (device, mesh, h, dtype):
# built with NumPy on the host exactly as the reference builds it (a few
# milliseconds for a 65^3-node mesh, at every pyramid level of every solve
# without the cache).
_PLANE_WAVES = {}
_PLANE_WAVES_MAX = 16
_PLANE_WAVES_LOCK = threading.Lock()  # level set-ups may run on two host threads (engine/batch.py)


def _plane_wave_device(Nx, Ny, Nz, h, dtype):
    key = (D.torch().cuda.current_device(), Nx, Ny, Nz, h, np.dtype(dtype).str)
    with _PLANE_WAVES_LOCK:
        V = _PLANE_WAVES.get(key)
        if V is None:
            if len(_PLANE_WAVES) >= _PLANE_WAVES_MAX:
                _PLANE_WAVES.pop(next(iter(_PLANE_WAVES)))
            V = _PLANE_WAVES[key] = D.to_device(_plane_wave(Nx, Ny, Nz, h, dtype))
    return V


class _LevelSetup:
    """Everything one GN solver of a level needs: the descriptor, its
    workspaces, the device arrays it points to (kept alive here), U0 and the
    level's scalars."""


# Element edges the element-Hessian kernels are built for, and the smallest
# edge at which a float32 plain solve takes them by default: from h = 4 an
# element's 162 stored floats (648 B) weigh less than its voxels' gradient
# and mask (13 B x h^3 = 832 B at h = 4), and a PCG applies them ~20 times
# per formation (513^3 benchmark, h = 4 level: 11.8 -> 8.8 ms); at h = 2 the
# matrix-free pass reads 104 B per element from L2.
ELEMENT_H = frozenset((1, 2, 3, 4, 6, 8, 12, 16))
ELEMENT_MIN_H = 4


def _lap_blockdiag(K):
    """K (24x24, dof 3a+c) = one 8x8 block L8 on each displacement
    component, K[3a+c][3b+c'] = (c == c') L8[a][b], exactly."""
    K = np.asarray(K, dtype=np.float64)
    L8 = K[0::3, 0::3]
    ref = np.kron(L8, np.eye(3))
    return K.shape == (24, 24) and bool(np.array_equal(K, ref))


def _setup_level(lv, Nx, Ny, Nz, h, g_origin=(0, 0, 0), glt=0.0, l0=None, K_ref_laplacian=None, reg_exponent=2,
                 c_reg=1.0, reg_type='laplacian', K_ref_elastic=None, eps_reg=1e-3, dynamic_mask=False, U0=None,
                 maxiter=30, disp=True, dtype=np.float32, pcg_chunk=0, precision='plain', mixed_min_h=4,
                 hessian='auto', defer=False):
    """Level set-up of correlate_gpu (engine/correlate_gpu.py:905-1053):
    gradient, masks, reference stats, regularizer and lambda calibration,
    U0, and the solver descriptor.  Returns a _LevelSetup (ls.empty is set
    when maxiter < 1: nothing to solve).

    hessian: how a float32 plain solve applies H in its PCG -- 'matrix_free'
    (from the gradient every step, as kernels_dvc.matvec_H), 'element'
    (element Hessians formed from the same float32 gradient once per GN
    iteration: the same float32 products summed in another order) or 'auto'
    (element Hessians at h >= ELEMENT_MIN_H, where an element's 162 stored
    entries weigh less than its voxels' gradient and mask, 13 B x h^3).

    defer: leave the level's scalars on the device; the caller completes
    the set-up with _finish_setup (the batch reads all problems' at once)."""
    dtype = np.dtype(dtype)
    if precision not in ('plain', 'mixed'):
        raise ValueError("precision must be 'plain' or 'mixed'")
    if precision == 'mixed' and dtype != np.float32:
        raise ValueError("precision='mixed' is a float32 solve (BF16 gradient, FP32 element Hessians)")
    if hessian not in ('auto', 'matrix_free', 'element'):
        raise ValueError("hessian must be 'auto', 'matrix_free' or 'element'")
    # The element-Hessian forms pay where an element's 162 stored entries
    # weigh less than its voxels' gradient and mask (13 B x h^3): h >= 4.
    # Below that the matrix-free FP32 pass moves less data and is kept.
    if precision == 'mixed' and h < mixed_min_h:
        precision = 'plain'
    element = False
    if precision == 'plain' and dtype == np.float32 and h in ELEMENT_H and hessian != 'matrix_free':
        lap_ok = l0 is None or K_ref_laplacian is None or _lap_blockdiag(K_ref_laplacian)
        if hessian == 'element' and not lap_ok:
            raise ValueError("hessian='element' needs K_ref_laplacian = one 8x8 block per displacement component")
        element = lap_ok and (hessian == 'element' or h >= ELEMENT_MIN_H)
    elif hessian == 'element':
        raise ValueError(f"hessian='element' is a float32 plain solve with h in {sorted(ELEMENT_H)}")

    Nvx, Nvy, Nvz = Nx * h + 1, Ny * h + 1, Nz * h + 1
    Ndof = 3 * (Nx + 1) * (Ny + 1) * (Nz + 1)
    Nvox = Nvx * Nvy * Nvz
    if Nvox > np.iinfo(np.int32).max or Ndof > np.iinfo(np.int32).max:
        raise ValueError(
            "Nvox=%d / Ndof=%d exceed int32 range; matrix-free index "
            "arrays assume int32 indices" % (Nvox, Ndof))
    if tuple(lv.fshape) != (Nvx, Nvy, Nvz):
        raise ValueError(f"f_pix has shape {tuple(lv.fshape)}, expected (Nx*h+1, Ny*h+1, Nz*h+1) = "
                         f"{(Nvx, Nvy, Nvz)}")
    L = _lib.lib()
    # the level's scalars are reduced into one device buffer (count, s1, s2
    # of f over mask0; v.Hv and v.Lv of the calibration) and read back once
    # (_finish_setup), so that a batch reads every problem's in one go
    dsc = D.zeros(5, np.float64)
    if dtype == np.float32:
        # gradient, mask0 and the statistics of f over mask0 in one read of f
        grad = D.empty(3 * Nvox, dtype)
        mask0 = D.empty(Nvox, np.uint8)
        ws_ = D.scratch.get(1 << 18)
        _lib.check(L.vdvc_image_grad_stats(lv.f_vox.data_ptr(), Nvx, Nvy, Nvz, float(glt), grad.data_ptr(),
                                           mask0.data_ptr(), h, Nx, Ny, Nz, dsc.data_ptr(), ws_.data_ptr(),
                                           ws_.numel(), D.stream()), "image_grad_stats")
    else:
        grad, mask0 = _grad_vox(lv.f_vox, lv.fshape, dtype, glt)
        _stats_sums(lv.f_vox, mask0, h, Nx, Ny, Nz, out=dsc[0:3])

    N_stencil, w_stencil = build_N_stencil(h)
    if reg_type not in ('laplacian', 'equilibrium_gap'):
        raise ValueError("reg_type must be 'laplacian' or 'equilibrium_gap'")

    interior = None
    diag_eq = None
    if reg_type == 'equilibrium_gap':
        interior = D.to_device(build_interior_dof_mask(Nx, Ny, Nz), dtype)

    reg_code = _lib.REG_NONE
    host_HL = None   # (H0, L0) where they are reduced on the host
    ll_factor = 0.0
    if l0 is not None:
        if K_ref_laplacian is None:
            raise ValueError("K_ref_laplacian is required when l0 is given")
        if reg_type == 'equilibrium_gap' and K_ref_elastic is None:
            raise ValueError("K_ref_elastic is required when l0 is given and "
                             "reg_type='equilibrium_gap'")
        T_ = 10 * h
        if reg_type == 'equilibrium_gap':
            reg_code = _lib.REG_EQUILIBRIUM_GAP
            diag_eq = K.build_diagonal_equilibrium_gap(K_ref_elastic, interior.to(D.torch().float64), h, Nx, Ny, Nz,
                                                       Ndof, D.torch())
            dH = K.build_diagonal_H(grad.reshape(-1, 3), mask0, N_stencil, w_stencil, h, Nx, Ny, Nz, Ndof,
                                    D.torch())
            dlap = K.build_diagonal_K_ref(K_ref_laplacian, h, Nx, Ny, Nz, Ndof, D.torch())
            host_HL = (_dot(dH), _dot(diag_eq) + eps_reg * _dot(dlap))
        else:
            reg_code = _lib.REG_LAPLACIAN
            V = _plane_wave_device(Nx, Ny, Nz, h, dtype)
            Hv = K.matvec_H(V, grad.reshape(-1, 3), mask0, N_stencil, w_stencil, h, Nx, Ny, Nz, D.torch())
            Lv = K.matvec_K_ref(V, K_ref_laplacian, h, Nx, Ny, Nz, D.torch())
            _dot_into(V, Hv, dsc[3:4])
            _dot_into(V, Lv, dsc[4:5])
        ll_factor = c_reg * (l0 / T_) ** reg_exponent

    out_dt = np.dtype(np.float64) if (l0 is not None or dtype == np.float64) else dtype
    # U0 is read in the solve dtype (correlate_gpu.py:1037), kept as float64
    U64 = D.zeros(Ndof, np.float64) if U0 is None else \
        D.to_device(U0, dtype).reshape(-1).to(D.torch().float64)
    if U64.numel() != Ndof:
        raise ValueError(f"U0 has {U64.numel()} entries, expected {Ndof}")
    ls = _LevelSetup()
    ls.h, ls.Nvox, ls.Ndof, ls.out_dt, ls.U64 = h, Nvox, Ndof, out_dt, U64
    ls.precision, ls.dynamic_mask = precision, bool(dynamic_mask)
    ls.hessian = 'element' if (element or precision == 'mixed') else 'matrix_free'
    ls.empty = maxiter < 1
    ls.dsc, ls.host_HL, ls.ll_factor, ls.reg_type, ls.regularized = dsc, host_HL, ll_factor, reg_type, l0 is not None
    ls.disp, ls.desc = disp, None
    if ls.empty:
        if not defer:
            _finish_setup(ls)
        return ls

    Klap = np.ascontiguousarray(K_ref_laplacian if K_ref_laplacian is not None else np.zeros((24, 24)),
                                dtype=np.float64)
    Kel = np.ascontiguousarray(K_ref_elastic if K_ref_elastic is not None else np.zeros((24, 24)), dtype=np.float64)
    desc = _lib.GnDesc()
    desc.dtype = D.code_of(dtype)
    desc.h, desc.Nx, desc.Ny, desc.Nz = h, Nx, Ny, Nz
    desc.gnx, desc.gny, desc.gnz = lv.gshape
    desc.gx0, desc.gy0, desc.gz0 = (float(o) for o in g_origin)
    desc.glt = float(glt)
    desc.reg_type = reg_code
    desc.eps_reg = float(eps_reg)
    desc.K_lap = Klap.ctypes.data_as(_lib.pd)
    desc.K_el = Kel.ctypes.data_as(_lib.pd)
    desc.dynamic_mask = int(bool(dynamic_mask))
    desc.pcg_chunk = int(pcg_chunk)
    desc.f_vox = lv.f_vox.data_ptr()
    desc.g_vox = lv.g_vox.data_ptr()
    desc.grad = grad.data_ptr()
    desc.mask0 = mask0.data_ptr()
    desc.interior = D.ptr(interior)
    desc.diag_eqgap = D.ptr(diag_eq)
    desc.stream = D.stream()
    nbytes = L.vdvc_gn_workspace_bytes(desc.dtype, h, Nx, Ny, Nz)
    ws = D.torch().empty(nbytes, dtype=D.torch().uint8, device=D.device())
    eh_ws = None
    if precision == 'mixed' or element:
        desc.precision = _lib.PREC_MIXED if precision == 'mixed' else _lib.PREC_ELEMENT
        eh_bytes = L.vdvc_gn_eh_workspace_bytes(desc.precision, h, Nx, Ny, Nz)
        eh_ws = D.torch().empty(eh_bytes, dtype=D.torch().uint8, device=D.device())
        desc.eh_ws, desc.eh_ws_bytes = eh_ws.data_ptr(), eh_bytes
    ls.desc, ls.ws, ls.eh_ws, ls.nbytes = desc, ws, eh_ws, nbytes
    # the descriptor holds raw pointers: keep what they point to alive
    ls.keep = (Klap, Kel, grad, mask0, interior, diag_eq, lv)
    if not defer:
        _finish_setup(ls)
    return ls


def _finish_setup(ls, host_scalars=None):
    """The scalars of a level set-up from its device buffer (read here, or
    passed in by a caller that read several set-ups' at once): mean0 and
    std0 of f over mask0, the regularization weight, and the descriptor's
    copies of them."""
    v = ls.dsc.cpu().numpy() if host_scalars is None else host_scalars
    ls.mean0, ls.std0 = _mean_std(v[0], v[1], v[2])
    ls.ll = 0.0
    if ls.regularized:
        H0, L0 = ls.host_HL if ls.host_HL is not None else (float(v[3]), float(v[4]))
        ls.ll = ls.ll_factor * H0 / L0
        if ls.disp:
            print('Regularization: %s with lambda = %2.3e' % (ls.reg_type, ls.ll))
    elif ls.disp:
        print('Regularization: None')
    if ls.desc is not None:
        ls.desc.ll = float(ls.ll)
        ls.desc.mean0, ls.desc.std0 = ls.mean0, ls.std0
    return ls


def _gn_scalars_line(out8, ik, err, Nvox):
    _, stdr = _mean_std(out8[2], out8[3], out8[4])
    n_active = int(out8[5])
    return ("Iter # %2d | std(res)=%2.2f gl | dU/U=%1.2e | active pts=%d/%d (%.1f%%)"
            % (ik + 1, stdr, err, n_active, Nvox, 100 * n_active / Nvox))


def _norm_res(out8, std0):
    # 1 - ZNCC of the registered pair over the live mask, from the last
    # residual: res/std0 = f^ - g^ for the standardised f^, g^ (the
    # residual is built from the centred f, correlate_gpu.py:962, :1094)
    c_l, s2_l = out8[2], out8[4]
    return float(s2_l / c_l / (2.0 * std0 * std0)) if c_l > 0 else float("inf")


def _solve_level(lv, Nx, Ny, Nz, h, g_origin=(0, 0, 0), glt=0.0, l0=None, K_ref_laplacian=None, reg_exponent=2,
                 c_reg=1.0, reg_type='laplacian', K_ref_elastic=None, eps_reg=1e-3, dynamic_mask=False,
                 freeze_mask_after=None, U0=None, maxiter=30, eps=1e-3, pcg_tol=1e-6, pcg_max_iter=2000,
                 disp=True, dtype=np.float32, pcg_chunk=0, stats=None, precision='plain', mixed_min_h=4,
                 hessian='auto', U0_async=None, res_dst=None):
    """One pyramid level: set-up, GN iterations, read-back.  U0_async:
    (U0 float64 CUDA tensor, CUDA event or None) produced on another stream
    -- the set-up is enqueued first and only the iterations wait for it.
    res_dst: a pinned host tensor of the residual's size and output dtype
    that the read-back writes directly (returned as res)."""
    if U0_async is not None and U0 is not None:
        raise ValueError("give U0 or U0_async, not both")
    ls = _setup_level(lv, Nx, Ny, Nz, h, g_origin=g_origin, glt=glt, l0=l0, K_ref_laplacian=K_ref_laplacian,
                      reg_exponent=reg_exponent, c_reg=c_reg, reg_type=reg_type, K_ref_elastic=K_ref_elastic,
                      eps_reg=eps_reg, dynamic_mask=dynamic_mask, U0=U0, maxiter=maxiter, disp=disp, dtype=dtype,
                      pcg_chunk=pcg_chunk, precision=precision, mixed_min_h=mixed_min_h, hessian=hessian)
    if U0_async is not None:
        U0d, ready = U0_async
        if ready is not None:
            D.torch().cuda.current_stream().wait_event(ready)
        if U0d.numel() != ls.Ndof:
            raise ValueError(f"U0 has {U0d.numel()} entries, expected {ls.Ndof}")
        ls.U64 = U0d.reshape(-1).to(D.torch().float64)
    out_dt, Nvox, Ndof, U64 = ls.out_dt, ls.Nvox, ls.Ndof, ls.U64
    if ls.empty:
        return U64.to(D.torch_dtype(out_dt)), D.zeros(Nvox, out_dt), D.zeros(Ndof, out_dt), {}
    L = _lib.lib()
    desc, ws, eh_ws, nbytes, ll, precision = ls.desc, ls.ws, ls.eh_ws, ls.nbytes, ls.ll, ls.precision

    solver = C.c_void_p()
    _lib.check(L.vdvc_gn_create(C.byref(desc), ws.data_ptr(), nbytes, C.byref(solver)), "correlate_gpu")
    info = {"gn_iters": 0, "pcg_iters": [], "pcg_status": [], "du": [], "ll": ll, "h": h, "precision": precision,
            "hessian": ls.hessian}
    t_start = time.perf_counter()
    try:
        st = D.stream()
        _lib.check(L.vdvc_gn_set_U(solver, U64.data_ptr(), st), "set_U")
        if not dynamic_mask:
            _lib.check(L.vdvc_gn_frozen_diag(solver, st), "frozen_diag")
        frozen = False
        out8 = (C.c_double * 12)()
        for ik in range(maxiter):
            freeze_now = freeze_mask_after is not None and not frozen and ik >= freeze_mask_after
            # sample -> rhs -> pcg -> update, one host synchronisation
            _lib.check(L.vdvc_gn_iterate(solver, int(freeze_now), int(pcg_max_iter), float(pcg_tol),
                                         C.cast(out8, _lib.pd), st), "GN iteration")
            frozen = frozen or freeze_now
            info["gn_iters"] = ik + 1
            info["pcg_iters"].append(int(out8[8]))
            info["pcg_status"].append(int(out8[10]))
            dd, uu = out8[0], out8[1]
            with np.errstate(divide='ignore', invalid='ignore'):
                err = float(np.sqrt(np.float64(dd)) / np.sqrt(np.float64(uu)))
            info["du"].append(err)
            if disp:
                print(_gn_scalars_line(out8, ik, err, Nvox))
            if err < eps:
                break
        info["converged"] = bool(err < eps)
        info["norm_res"] = _norm_res(out8, ls.std0)
        Uo = D.empty(Ndof, out_dt)
        res = res_dst if res_dst is not None else D.empty(Nvox, out_dt)
        dU = D.empty(Ndof, out_dt)
        f64 = int(out_dt == np.float64)
        _lib.check(L.vdvc_gn_read(solver, _lib.GN_U, Uo.data_ptr(), f64, st), "read")
        _lib.check(L.vdvc_gn_read(solver, _lib.GN_RES, res.data_ptr(), f64, st), "read")
        _lib.check(L.vdvc_gn_read(solver, _lib.GN_DU, dU.data_ptr(), f64, st), "read")
    finally:
        L.vdvc_gn_destroy(solver)
        D.torch().cuda.current_stream().synchronize()
        del ws, eh_ws
    info["gn_wall_s"] = time.perf_counter() - t_start
    if stats is not None:
        stats.append(info)
    return Uo, res, dU, info


def correlate_gpu(f_pix, g_pix, Nx, Ny, Nz, h, xp, g_origin=(0, 0, 0),
                  glt=0.0,
                  l0=None, K_ref_laplacian=None, reg_exponent=2, c_reg=1.0,
                  reg_type='laplacian', K_ref_elastic=None, eps_reg=1e-3,
                  dynamic_mask=False, freeze_mask_after=None, U0=None,
                  maxiter=30, eps=1e-3, pcg_tol=1e-6, pcg_max_iter=2000,
                  disp=True, dtype=np.float32, **solver_opts):
    """Matrix-free GN-PCG DVC solve of f_pix/g_pix on an (Nx,Ny,Nz) mesh of
    edge h; returns (U, res, dU) as in the reference.
    Reference: engine/correlate_gpu.py:828-1140."""
    dtype = np.dtype(dtype)
    f_vox, fs = pix_to_vox(f_pix, dtype)
    g_vox, gs = pix_to_vox(g_pix, dtype)
    U, res, dU, _ = _solve_level(_Level(f_vox, fs, g_vox, gs), Nx, Ny, Nz, h, g_origin=g_origin, glt=glt, l0=l0,
                                 K_ref_laplacian=K_ref_laplacian, reg_exponent=reg_exponent, c_reg=c_reg,
                                 reg_type=reg_type, K_ref_elastic=K_ref_elastic, eps_reg=eps_reg,
                                 dynamic_mask=dynamic_mask, freeze_mask_after=freeze_mask_after, U0=U0,
                                 maxiter=maxiter, eps=eps, pcg_tol=pcg_tol, pcg_max_iter=pcg_max_iter, disp=disp,
                                 dtype=dtype, **solver_opts)
    return D.out(U, xp), D.out(res, xp), D.out(dU, xp)


def _affine_U0(A_aff, t_aff, c_aff, s, h_i, Nx, Ny, Nz):
    # u_i(X_i) = A (X_i - c_i) + c_i + t_i - X_i at the nodes, c_i = c/s,
    # t_i = t/s (correlate_gpu.py:1264-1281); float64 on the host
    c_i = c_aff / s
    t_i = t_aff / s
    n_nodes = (Nx + 1) * (Ny + 1) * (Nz + 1)
    node = np.arange(n_nodes)
    X = np.stack([node % (Nx + 1), (node // (Nx + 1)) % (Ny + 1), node // ((Nx + 1) * (Ny + 1))],
                 axis=1).astype(np.float64) * h_i
    u = (X - c_i) @ A_aff.T + c_i + t_i - X
    return u.reshape(-1)


def multiscale_correlate_gpu(f_pix, g_pix, Nx, Ny, Nz, h, xp, scales=(2, 1, 0),
                             g_origin=(0, 0, 0), l0=None, fft_prealign=True,
                             prealign_affine=False, ext_affine=None,
                             **kwargs):
    """Coarse-to-fine pyramid of correlate_gpu solves (strided decimation by
    2**iscale, fixed element grid, h_i = h / 2**iscale, U carried between
    levels); returns the finest level's (U, res, dU).
    Reference: engine/correlate_gpu.py:1143-1305."""
    scales = sorted(set(scales), reverse=True)
    dtype = np.dtype(kwargs.get('dtype', np.float32))
    disp = kwargs.get('disp', True)
    # The reference checks each level as it reaches it (correlate_gpu.py:
    # 1248-1254).  Levels run coarsest first and divisibility by 2**i implies
    # it for every smaller i, so the first failing level is always the first
    # level: checking all of them here raises the same error at the same
    # point, before any image reaches the device.
    for iscale in scales:
        s = 2 ** iscale
        if h % s != 0:
            raise ValueError("h=%d not divisible by 2**%d=%d" % (h, iscale, s))
        if any(o % s != 0 for o in g_origin):
            raise ValueError("g_origin=%r not divisible by 2**%d=%d for all "
                             "requested scales" % (g_origin, iscale, s))

    A_aff = t_aff = c_aff = None
    if ext_affine is not None:
        A_aff, t_aff, c_aff = ext_affine
        A_aff = np.asarray(A_aff, dtype=np.float64)
        t_aff = np.asarray(t_aff, dtype=np.float64)
        c_aff = np.asarray(c_aff, dtype=np.float64)
        if disp:
            print("External affine: t = (%.1f, %.1f, %.1f) voxels, "
                  "c = (%.1f, %.1f, %.1f)" % (*t_aff, *c_aff))
    elif prealign_affine:
        A_aff, t_aff, c_aff, aff_info = affine_prealign(f_pix, g_pix, xp)
        if disp:
            rx, ry, rz = (180 / np.pi) * np.array([
                np.arctan2(A_aff[2, 1], A_aff[2, 2]),
                np.arctan2(-A_aff[2, 0], np.hypot(A_aff[2, 1], A_aff[2, 2])),
                np.arctan2(A_aff[1, 0], A_aff[0, 0])])
            sx, sy, sz = np.linalg.norm(A_aff, axis=0)
            print("Affine pre-alignment (full res): rotation (deg) = (%.3f, %.3f, %.3f), "
                  "scale = (%.4f, %.4f, %.4f), t = (%.1f, %.1f, %.1f) voxels "
                  "(1-ZNCC %.4f -> %.4f)"
                  % (rx, ry, rz, sx, sy, sz, t_aff[0], t_aff[1], t_aff[2],
                     aff_info['cost_translation_only'], aff_info['cost_final']))

    # full-resolution images on the device once, vox layout, solve dtype.
    # Host images that the device reads in place: the coarsest level reads
    # its every-s-th voxels straight from them, and the full-resolution
    # layout runs on a side stream under that level's iterations; the finer
    # levels wait for it.
    coarse = {}
    full_ready = None
    if scales[0] > 0 and _host_readable(f_pix) and _host_readable(g_pix):
        torch = D.torch()
        fa, ga = np.asarray(f_pix), np.asarray(g_pix)
        s0 = 2 ** scales[0]
        coarse[s0] = (_pix_to_vox_strided_host(fa, s0, dtype), _pix_to_vox_strided_host(ga, s0, dtype))
        fs, gs = tuple(fa.shape), tuple(ga.shape)
        f_full = D.empty(fa.size, dtype)  # allocated on this stream: the side stream only writes them
        g_full = D.empty(ga.size, dtype)
        main, side = torch.cuda.current_stream(), _layout_stream()
        side.wait_stream(main)
        with torch.cuda.stream(side):
            # a bounded grid: its blocks mostly wait on the host link and
            # would otherwise hold every SM against the level's kernels
            for a, out in ((fa, f_full), (ga, g_full)):
                _lib.check(_lib.lib().vdvc_pix_to_vox_strided(a.ctypes.data, D.code_of(a.dtype), *a.shape, 1,
                                                              _BACKGROUND_LAYOUT_BLOCKS, out.data_ptr(),
                                                              D.code_of(dtype), D.stream()), "pix_to_vox")
            full_ready = torch.cuda.Event()
            full_ready.record(side)
    else:
        f_full, fs = pix_to_vox(f_pix, dtype)
        g_full, gs = pix_to_vox(g_pix, dtype)

    try:
        return _pyramid(f_full, fs, g_full, gs, coarse, full_ready, scales, Nx, Ny, Nz, h, dtype, g_origin, l0, A_aff,
                        t_aff, c_aff, fft_prealign, disp, xp, kwargs)
    finally:
        if full_ready is not None:
            # both streams have finished reading the caller's arrays
            full_ready.synchronize()
            D.torch().cuda.current_stream().synchronize()


def _pyramid(f_full, fs, g_full, gs, coarse, full_ready, scales, Nx, Ny, Nz, h, dtype, g_origin, l0, A_aff, t_aff,
             c_aff, fft_prealign, disp, xp, kwargs):
    U = None
    prev_s = None
    res = dU = None
    for iscale in scales:
        s = 2 ** iscale
        h_i = h // s
        if s in coarse:
            (f_i, fs_i), (g_i, gs_i) = coarse.pop(s)
        else:
            if full_ready is not None:
                D.torch().cuda.current_stream().wait_event(full_ready)
            f_i, fs_i = _decimate(f_full, fs, s, dtype)
            g_i, gs_i = _decimate(g_full, gs, s, dtype)
        g_origin_i = tuple(o // s for o in g_origin)
        l0_i = None if l0 is None else l0 / s

        if U is not None:
            # the reference rescales the promoted U, and the next level
            # re-reads it in the solve dtype (correlate_gpu.py:1263, :1037)
            U = (U * (prev_s / s)).to(D.torch_dtype(dtype))
        elif A_aff is not None:
            U = D.to_device(_affine_U0(A_aff, t_aff, c_aff, s, h_i, Nx, Ny, Nz).astype(dtype))
        elif fft_prealign:
            dd = _fft_shift_device(f_i, fs_i, g_i, gs_i, dtype)
            U = _uniform_U0(dd, (Nx + 1) * (Ny + 1) * (Nz + 1), dtype)
            if disp:
                d = dd.cpu().numpy()
                print("FFT pre-alignment: rigid shift d = (%.1f, %.1f, %.1f) voxels"
                      % (d[0] * s, d[1] * s, d[2] * s))

        if disp:
            print("=== MULTISCALE: scale 2^%d (image decimated by %d, h_i=%d/%d=%d) ==="
                  % (iscale, s, h, s, h_i))
        # host results: the finest level's residual field (the one large
        # output) is converted straight into pinned host memory by the
        # read-back kernel instead of a device copy and a transfer; its
        # dtype follows the level set-up's rule (float64 when regularized
        # or in a float64 solve)
        res_ent = None
        if iscale == scales[-1] and D.wants_host(xp) and kwargs.get('maxiter', 30) >= 1:
            res_dt = np.dtype(np.float64) if (l0 is not None or dtype == np.float64) else dtype
            res_ent = D.host_result(fs_i[0] * fs_i[1] * fs_i[2], res_dt)
        U, res, dU, _ = _solve_level(_Level(f_i, fs_i, g_i, gs_i), Nx, Ny, Nz, h_i, g_origin=g_origin_i, l0=l0_i,
                                     U0=U, res_dst=None if res_ent is None else res_ent[0], **kwargs)
        prev_s = s
    res_out = D.claim_host_result(res_ent) if res_ent is not None else D.out(res, xp)
    return D.out(U, xp), res_out, D.out(dU, xp)


# ---------------------------------------------------------------------------
# affine pre-alignment (correlate_gpu.py:417-825)
# ---------------------------------------------------------------------------

def _ptr3(a):
    a = np.ascontiguousarray(a, dtype=np.float64).reshape(-1)
    return a, a.ctypes.data_as(_lib.pd)


def _zncc_cost(sums):
    """1 - ZNCC from (n, sum f, sum g, sum f^2, sum g^2, sum fg), with the
    reference's guards: fewer than 1000 voxels or a degenerate variance
    give 2.0 (correlate_gpu.py:417-433)."""
    n, sf, sg, sff, sgg, sfg = sums
    if int(n) < 1000:
        return 2.0
    vf = sff - sf * sf / n
    vg = sgg - sg * sg / n
    denom = np.sqrt(max(vf, 0.0) * max(vg, 0.0))
    if denom < 1e-8:
        return 2.0
    return 1.0 - float((sfg - sf * sg / n) / denom)


def _build_affine_matrix(p):
    """A = Rz(rz) Ry(ry) Rx(rx) diag(sx, sy, sz) from p = (rx, ry, rz, sx, sy,
    sz, ...) (correlate_gpu.py:436-448)."""
    rx, ry, rz, sx, sy, sz = (float(v) for v in p[:6])

    def rot(axis, a):
        c, s = np.cos(a), np.sin(a)
        R = np.eye(3)
        i, j = [(1, 2), (0, 2), (0, 1)][axis]
        R[i, i], R[j, j] = c, c
        R[i, j], R[j, i] = -s, s
        if axis == 1:  # rotation about y: R[0,2] = +sin, R[2,0] = -sin
            R[i, j], R[j, i] = s, -s
        return R

    return rot(2, rz) @ rot(1, ry) @ rot(0, rx) @ np.diag([sx, sy, sz])


def affine_prealign(f_pix, g_pix, xp, decimate=4, t0=None, angle_bound=0.3, scale_bound=0.15, maxiter=200,
                    disp=False):
    """9-DOF (rotation, per-axis scale, translation) alignment maximising the
    ZNCC of f(x) and g(A (x - c) + c + t) on copies decimated by `decimate`;
    the cost is evaluated on the GPU, the Powell search runs on the host
    (scipy).  Returns (A, t, c, info) in full-resolution voxel units.
    Reference: engine/correlate_gpu.py:451-567."""
    from scipy.optimize import minimize
    f_full, fs = pix_to_vox(f_pix, np.float32)
    g_full, gs = pix_to_vox(g_pix, np.float32)
    f_d, fsd = _decimate(f_full, fs, decimate, np.float32)
    g_d, gsd = _decimate(g_full, gs, decimate, np.float32)
    del f_full, g_full
    c = np.array([(n - 1) / 2.0 for n in fsd], dtype=np.float64)
    if t0 is None:
        t0_dec = _fft_shift_vox(f_d, fsd, g_d, gsd, np.float32)
    else:
        t0_dec = np.asarray(t0, dtype=np.float64) / decimate
    L = _lib.lib()
    ws = D.torch().empty(L.vdvc_affine_workspace_bytes(), dtype=D.torch().uint8, device=D.device())
    cb, cp = _ptr3(c)
    out6 = (C.c_double * 6)()

    def warp_and_cost(p):
        A, Ap = _ptr3(_build_affine_matrix(p))
        t, tp = _ptr3(p[6:9])
        _lib.check(L.vdvc_affine_zncc_sums(f_d.data_ptr(), *fsd, g_d.data_ptr(), *gsd, Ap, tp, cp,
                                           C.cast(out6, _lib.pd), ws.data_ptr(), ws.numel(), D.stream()),
                   "affine_prealign")
        return _zncc_cost(list(out6))

    p_identity = np.array([0., 0., 0., 1., 1., 1., 0., 0., 0.])
    p_translation_only = p_identity.copy()
    p_translation_only[6:9] = t0_dec
    cost_identity = warp_and_cost(p_identity)
    cost_translation_only = warp_and_cost(p_translation_only)
    bounds = ([(-angle_bound, angle_bound)] * 3 + [(1 - scale_bound, 1 + scale_bound)] * 3 + [(None, None)] * 3)
    result = minimize(warp_and_cost, p_translation_only, method='Powell', bounds=bounds,
                      options={'maxiter': maxiter, 'disp': disp})
    p_opt = result.x
    A = _build_affine_matrix(p_opt)
    info = {'cost_identity': cost_identity, 'cost_translation_only': cost_translation_only,
            'cost_final': float(result.fun), 'nfev': result.nfev, 'p': p_opt}
    return A, p_opt[6:9] * decimate, c * decimate, info


def affine_refine_gn(f_pix, g_pix, xp, A0, t0, c, sigmas=(4.0, 2.0, 1.0, 0.0), max_iter=50, tol=1e-6, patience=3,
                     cval=0.0, chunk_voxels=8_000_000, disp=False):
    """Forward-additive Gauss-Newton refinement of a full 3x3 affine +
    translation in the generative convention def(x) ~ ref(x - M (x - c) - t_r)
    over a Gaussian scale space; each iteration's 12x12 float64 normal
    equations are assembled on the GPU in one pass.  Returns (A, t, info) in
    the affine_prealign convention.  `chunk_voxels` is accepted and ignored.
    Reference: engine/correlate_gpu.py:600-825."""
    T = D.torch()
    f, shape = pix_to_vox(f_pix, np.float32)
    g, gshape = pix_to_vox(g_pix, np.float32)
    if tuple(gshape) != tuple(shape):
        raise ValueError("affine_refine_gn needs f_pix and g_pix of the same shape")
    nx, ny, nz = shape
    n = nx * ny * nz
    I3 = np.eye(3)
    A0 = np.asarray(A0, dtype=np.float64)
    t0 = np.asarray(t0, dtype=np.float64)
    A0inv = np.linalg.inv(A0)
    M = I3 - A0inv
    tr = A0inv @ t0
    c = np.asarray(c, dtype=np.float64)
    L = _lib.lib()
    ws = T.empty(L.vdvc_affine_workspace_bytes(), dtype=T.uint8, device=D.device())
    cb, cp = _ptr3(c)
    tmp = [D.empty(n, np.float32) for _ in range(3)]
    f_s_buf, g_s_buf = D.empty(n, np.float32), D.empty(n, np.float32)
    st = D.stream()

    def _rms(M_, tr_):
        Mb, Mp = _ptr3(M_)
        tb, tp = _ptr3(tr_)
        out2 = (C.c_double * 2)()
        _lib.check(L.vdvc_affine_rms_sums(f.data_ptr(), g.data_ptr(), nx, ny, nz, Mp, tp, cp, float(cval),
                                          C.cast(out2, _lib.pd), ws.data_ptr(), ws.numel(), st), "affine_refine_gn")
        return float(np.sqrt(out2[0] / max(out2[1], 1.0)))

    rms_initial = _rms(M, tr)
    iters = []
    H = np.empty(144)
    b = np.empty(12)
    for sigma in sigmas:
        if sigma > 0:
            _lib.check(L.vdvc_gaussian_filter(f.data_ptr(), f_s_buf.data_ptr(), nx, ny, nz, float(sigma), 0, 0.0,
                                              None, tmp[0].data_ptr(), st), "gaussian_filter")
            _lib.check(L.vdvc_smooth_masked(g.data_ptr(), nx, ny, nz, float(sigma), float(cval), g_s_buf.data_ptr(),
                                            tmp[0].data_ptr(), tmp[1].data_ptr(), tmp[2].data_ptr(), st),
                       "smooth_masked")
            f_s, g_s = f_s_buf, g_s_buf
        else:
            f_s, g_s = f, g
        grad, _ = _grad_vox(f_s, shape, np.float32)
        n_it = 0
        best_step = np.inf
        stall = 0
        for it in range(max_iter):
            Mb, Mp = _ptr3(M)
            tb, tp = _ptr3(tr)
            _lib.check(L.vdvc_affine_normal_equations(f_s.data_ptr(), grad.data_ptr(), g_s.data_ptr(), g.data_ptr(),
                                                      nx, ny, nz, Mp, tp, cp, float(cval), H.ctypes.data_as(_lib.pd),
                                                      b.ctypes.data_as(_lib.pd), ws.data_ptr(), ws.numel(), st),
                       "affine_refine_gn")
            Hm = H.reshape(12, 12).copy()
            Hm += np.eye(12) * (1e-9 * float(np.trace(Hm)) / 12.0 + 1e-30)
            dp = np.linalg.solve(Hm, b)
            M = M + dp[:9].reshape(3, 3)
            tr = tr + dp[9:]
            step = float(np.linalg.norm(dp))
            n_it = it + 1
            if disp:
                print(f"    sigma={sigma:g} iter {it:2d}: ||dp||={step:.3e}", flush=True)
            if step < tol:
                break
            if step < best_step - 1e-12:
                best_step = step
                stall = 0
            else:
                stall += 1
                if stall >= patience:
                    break
        iters.append(n_it)
        del grad
    rms = _rms(M, tr)
    A = np.linalg.inv(I3 - M)
    return A, A @ tr, {'rms_initial': rms_initial, 'rms_final': rms, 'iters': iters}
