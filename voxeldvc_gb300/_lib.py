"""ctypes binding of ``libvdvc.so`` (the C ABI declared in include/vdvc.h).

The library is loaded from the package directory only.  There is no
fallback: if it is missing or fails to load, :func:`lib` raises, so no
operator of this package can silently run anywhere but on the GPU.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libvdvc.so")

# status codes (include/vdvc.h)
OK = 0
ERR_ARG = 1
ERR_INDEX_RANGE = 2
ERR_CUDA = 3
ERR_WORKSPACE = 4
ERR_NONFINITE = 5
ERR_ZERO_DIVISION = 6
ERR_CUFFT = 7
ERR_UNSUPPORTED = 8
ERR_TIMEOUT = 9

# element type codes
F32, F64, U8, U16, I16, I32 = 0, 1, 2, 3, 4, 5

# regularizer kinds
REG_NONE, REG_LAPLACIAN, REG_EQUILIBRIUM_GAP = 0, 1, 2

# Hessian forms of the GN solver (vdvc_gn_desc.precision)
PREC_PLAIN, PREC_MIXED, PREC_ELEMENT = 0, 1, 2

vp = C.c_void_p
ci = C.c_int
cd = C.c_double
cz = C.c_size_t
pd = C.POINTER(C.c_double)
pi = C.POINTER(C.c_int)

# name -> (restype, argtypes); one line per entry point of include/vdvc.h
SIGNATURES = {
    "vdvc_abi_version": (ci, []),
    "vdvc_status_string": (C.c_char_p, [ci]),
    "vdvc_last_error": (C.c_char_p, []),
    "vdvc_launch_count": (C.c_longlong, []),
    "vdvc_workspace_bytes": (cz, [ci, ci, ci, ci, ci]),
    "vdvc_pix_to_vox": (ci, [vp, ci, ci, ci, ci, vp, ci, vp]),
    "vdvc_pix_to_vox_strided": (ci, [vp, ci, ci, ci, ci, ci, ci, vp, ci, vp]),
    "vdvc_decimate": (ci, [vp, ci, ci, ci, ci, ci, vp, vp]),
    "vdvc_image_grad": (ci, [vp, ci, ci, ci, ci, cd, vp, vp, vp]),
    "vdvc_image_grad_stats": (ci, [vp, ci, ci, ci, cd, vp, vp, ci, ci, ci, ci, vp, vp, cz, vp]),
    "vdvc_erode_mask": (ci, [vp, ci, ci, ci, vp, vp]),
    "vdvc_masked_stats": (ci, [vp, ci, vp, ci, ci, ci, ci, vp, vp, cz, vp]),
    "vdvc_matvec_H": (ci, [vp, vp, vp, ci, ci, ci, ci, ci, vp, vp, cz, vp]),
    "vdvc_matvec_H_noalloc": (ci, [vp, vp, vp, ci, ci, ci, ci, vp, vp]),
    "vdvc_matvec_H_noalloc_max_elements": (cz, []),
    "vdvc_selftest_bounded_wait": (ci, [ci, C.c_longlong, vp]),
    "vdvc_matvec_H_mixed": (ci, [vp, vp, vp, ci, ci, ci, ci, vp, vp, cz, vp]),
    "vdvc_eh_workspace_bytes": (cz, [ci, ci, ci, ci]),
    "vdvc_device_reads_pageable": (ci, [ci]),
    "vdvc_gn_eh_workspace_bytes": (cz, [ci, ci, ci, ci, ci]),
    "vdvc_eh_bytes": (cz, [ci, ci, ci, ci]),
    "vdvc_eh_op_workspace_bytes": (cz, [ci, ci, ci, ci]),
    "vdvc_eh_form": (ci, [vp, ci, vp, ci, ci, ci, ci, vp, vp, cz, vp]),
    "vdvc_eh_apply": (ci, [vp, vp, ci, ci, ci, ci, vp, vp, cz, vp]),
    "vdvc_eh_status": (ci, [vp, cz, ci, ci, ci, ci, vp]),
    "vdvc_diag_H": (ci, [vp, vp, ci, ci, ci, ci, ci, vp, vp, cz, vp]),
    "vdvc_compute_b": (ci, [vp, vp, vp, ci, ci, ci, ci, ci, vp, vp, cz, vp]),
    "vdvc_matvec_K_ref": (ci, [vp, ci, pd, vp, cd, ci, ci, ci, vp, vp]),
    "vdvc_diag_K_ref": (ci, [ci, pd, vp, cd, ci, ci, ci, vp, vp]),
    "vdvc_matvec_equilibrium_gap": (ci, [vp, ci, pd, vp, vp, cd, ci, ci, ci, vp, vp, cz, vp]),
    "vdvc_diag_equilibrium_gap": (ci, [vp, ci, pd, vp, vp, cd, ci, ci, ci, vp, vp, cz, vp]),
    "vdvc_sample_deformed": (ci, [vp, vp, ci, ci, ci, ci, cd, cd, cd, vp, cd, ci, ci, ci, ci, vp, vp, vp]),
    "vdvc_interp_field": (ci, [vp, ci, ci, ci, ci, ci, ci, vp, vp]),
    "vdvc_dot": (ci, [vp, vp, ci, C.c_longlong, pd, vp, cz, vp]),
    "vdvc_dot_device": (ci, [vp, vp, ci, C.c_longlong, vp, vp, cz, vp]),
    "vdvc_push_field": (ci, [vp, ci, vp, ci, ci, ci, ci, ci, cd, vp, vp]),
    "vdvc_zncc": (ci, [vp, vp, ci, vp, C.c_longlong, pd, vp, cz, vp]),
    "vdvc_cast_round": (ci, [vp, C.c_longlong, ci, vp, vp]),
    "vdvc_warp_affine": (ci, [vp, ci, ci, ci, pd, pd, pd, ci, ci, ci, vp, vp]),
    "vdvc_bin_volume": (ci, [vp, ci, ci, ci, ci, ci, vp, vp]),
    "vdvc_overlap_projections": (ci, [vp, vp, ci, ci, ci, cd, vp, vp, vp, vp]),
    "vdvc_cell_strains": (ci, [vp, ci, ci, ci, ci, vp, vp, vp]),
    "vdvc_equivalent_strain": (ci, [vp, C.c_longlong, vp, vp]),
    "vdvc_cell_fields": (ci, [vp, ci, vp, vp, ci, ci, ci, ci, cd, vp, vp, vp, vp, vp]),
    "vdvc_cell_erode": (ci, [vp, ci, ci, ci, vp, vp]),
    "vdvc_cell_gn_convergence": (ci, [vp, vp, ci, ci, ci, vp, vp]),
    "vdvc_unsafe_masks_workspace_bytes": (cz, [ci, ci, ci]),
    "vdvc_gt_warp": (ci, [vp, vp, ci, ci, ci, vp, vp]),
    "vdvc_gt_voxel_in_bounds": (ci, [vp, ci, ci, ci, ci, ci, ci, vp, vp]),
    "vdvc_gt_node_oob_fraction": (ci, [vp, ci, ci, ci, ci, ci, ci, ci, C.POINTER(C.c_longlong), vp, vp]),
    "vdvc_unsafe_masks": (ci, [vp, vp, ci, ci, ci, ci, cd, cd, vp, vp, vp, vp, vp, cz, vp]),
    "vdvc_fft_rigid_shift": (ci, [vp, ci, ci, ci, vp, ci, ci, ci, ci, pd, vp]),
    "vdvc_fft_rigid_shift_device": (ci, [vp, ci, ci, ci, vp, ci, ci, ci, ci, vp, vp]),
    "vdvc_pcg_workspace_bytes": (cz, []),
    "vdvc_pcg_begin": (ci, [vp, vp, vp, ci, C.c_longlong, vp, vp, vp, ci, cd, vp, cz, vp]),
    "vdvc_pcg_step": (ci, [vp, vp, ci, C.c_longlong, vp, vp, vp, vp, vp, cz, pd, pi, vp]),
    "vdvc_pcg_direction": (ci, [vp, vp, ci, C.c_longlong, vp, cz, vp]),
    "vdvc_gn_workspace_bytes": (cz, [ci, ci, ci, ci, ci]),
    "vdvc_gn_create": (ci, [vp, vp, cz, C.POINTER(vp)]),
    "vdvc_gn_set_U": (ci, [vp, vp, vp]),
    "vdvc_gn_frozen_diag": (ci, [vp, vp]),
    "vdvc_gn_sample": (ci, [vp, ci, vp]),
    "vdvc_gn_rhs": (ci, [vp, vp]),
    "vdvc_gn_pcg": (ci, [vp, ci, cd, pi, pd, pi, vp]),
    "vdvc_gn_update": (ci, [vp, pd, vp]),
    "vdvc_gn_iterate": (ci, [vp, ci, ci, cd, vp, vp]),
    "vdvc_gn_read": (ci, [vp, ci, vp, ci, vp]),
    "vdvc_gn_destroy": (None, [vp]),
    "vdvc_gn_batch_create": (ci, [vp, ci, vp, vp, ci, ci, C.POINTER(vp)]),
    "vdvc_gn_batch_solver": (ci, [vp, ci, C.POINTER(vp)]),
    "vdvc_gn_batch_iterate": (ci, [vp, vp, vp, ci, cd, vp, vp]),
    "vdvc_gn_batch_set_schedule": (ci, [vp, ci, ci]),
    "vdvc_gn_batch_destroy": (None, [vp]),
    "vdvc_affine_workspace_bytes": (cz, []),
    "vdvc_affine_zncc_sums": (ci, [vp, ci, ci, ci, vp, ci, ci, ci, pd, pd, pd, pd, vp, cz, vp]),
    "vdvc_gaussian_filter": (ci, [vp, vp, ci, ci, ci, cd, ci, cd, vp, vp, vp]),
    "vdvc_smooth_masked": (ci, [vp, ci, ci, ci, cd, cd, vp, vp, vp, vp, vp]),
    "vdvc_affine_normal_equations": (ci, [vp, vp, vp, vp, ci, ci, ci, pd, pd, pd, cd, pd, pd, vp, cz, vp]),
    "vdvc_affine_rms_sums": (ci, [vp, vp, ci, ci, ci, pd, pd, pd, cd, pd, vp, cz, vp]),
    # include/vdvc_synth.h
    "vdvc_synth_workspace_bytes": (cz, [ci, ci, ci]),
    "vdvc_synth_texture": (ci, [vp, ci, ci, ci, C.c_ulonglong, cd, cd, vp, ci, cd, vp, cz, vp]),
    "vdvc_synth_warp": (ci, [vp, ci, ci, ci, ci, pd, ci, cd, C.c_ulonglong, vp, vp]),
    "vdvc_synth_warp_ffd": (ci, [vp, ci, ci, ci, pd, vp, ci, cd, C.c_ulonglong, vp, vp]),
    "vdvc_synth_ffd_inverse_grid": (ci, [pd, vp, ci, ci, ci, ci, ci, ci, ci, cd, ci, vp, vp]),
    "vdvc_synth_field_grid": (ci, [ci, pd, ci, ci, ci, ci, cd, vp, vp]),
    # include/vdvc_cnn.h
    "vdvc_cnn_conv": (ci, [vp, ci, ci, ci, vp, vp, ci, ci, vp, ci, ci, ci, ci, vp, vp]),
    "vdvc_cnn_status": (ci, [vp]),
    "vdvc_cnn_conv_wgrad": (ci, [vp, ci, ci, ci, vp, ci, ci, ci, vp, vp, ci, vp, cz, vp]),
    "vdvc_cnn_wgrad_workspace_bytes": (cz, [ci, ci]),
    "vdvc_cnn_bias_grad": (ci, [vp, ci, ci, ci, C.c_longlong, vp, ci, vp, cz, vp]),
    "vdvc_cnn_relu_bwd": (ci, [vp, vp, C.c_longlong, vp]),
    "vdvc_cnn_upsample2": (ci, [vp, ci, ci, ci, ci, ci, vp, ci, ci, ci, ci, ci, ci, vp]),
    "vdvc_cnn_upsample2_bwd": (ci, [vp, ci, ci, ci, ci, ci, vp, ci, ci, ci, ci, ci, ci, vp]),
    "vdvc_cnn_pool_input": (ci, [vp, vp, ci, ci, ci, pd, vp, vp]),
    "vdvc_cnn_pool_input_mirrored": (ci, [vp, vp, ci, ci, ci, pd, ci, vp, vp]),
    "vdvc_cnn_input_moments": (ci, [vp, vp, C.c_longlong, vp, vp, cz, vp]),
    "vdvc_cnn_pool_input_dev": (ci, [vp, vp, ci, ci, ci, vp, ci, vp, vp]),
    "vdvc_cnn_mirror_input": (ci, [vp, ci, ci, ci, ci, vp, vp]),
    "vdvc_cnn_mse": (ci, [vp, ci, vp, C.c_longlong, vp, vp, ci, cd, vp, cz, vp]),
    "vdvc_cnn_adam": (ci, [vp, vp, vp, vp, C.c_longlong, cd, cd, cd, cd, ci, vp]),
    "vdvc_cnn_pack_weights": (ci, [vp, ci, ci, vp, vp, vp]),
    "vdvc_cnn_seed_nodes": (ci, [vp, ci, ci, ci, ci, ci, ci, ci, ci, vp, vp]),
    "vdvc_cnn_seed_nodes_acc": (ci, [vp, ci, ci, ci, ci, ci, ci, ci, ci, ci, cd, ci, vp, vp]),
}


class ConvGeom(C.Structure):
    """ctypes mirror of vdvc_conv_geom (include/vdvc_cnn.h)."""
    _fields_ = [(n, ci) for n in ("nx", "ny", "nz", "sx", "sy", "sz", "a", "b", "c", "d")]

GN_U, GN_DU, GN_RES, GN_LIVE_MASK = 0, 1, 2, 3


class GnDesc(C.Structure):
    """ctypes mirror of vdvc_gn_desc (include/vdvc.h)."""
    _fields_ = [
        ("dtype", ci), ("h", ci), ("Nx", ci), ("Ny", ci), ("Nz", ci),
        ("gnx", ci), ("gny", ci), ("gnz", ci),
        ("gx0", cd), ("gy0", cd), ("gz0", cd),
        ("glt", cd),
        ("reg_type", ci),
        ("ll", cd), ("eps_reg", cd),
        ("K_lap", pd), ("K_el", pd),
        ("dynamic_mask", ci), ("pcg_chunk", ci),
        ("f_vox", vp), ("g_vox", vp), ("grad", vp), ("mask0", vp),
        ("interior", vp), ("diag_eqgap", vp),
        ("mean0", cd), ("std0", cd),
        ("stream", vp),
        ("precision", ci), ("eh_ws", vp), ("eh_ws_bytes", cz),
    ]

_lock = threading.Lock()
_lib = None


class VdvcError(RuntimeError):
    """A CUDA-side failure reported by libvdvc."""


class VdvcTimeout(VdvcError):
    """A bounded device-side wait ran out (VDVC_ERR_TIMEOUT): the kernel
    returned early, its results are not valid, the CUDA context is usable."""


def lib():
    """The loaded library, with argument types set.  Raises if absent."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH):
                raise ImportError(
                    f"{LIB_PATH} is missing: build it with `python -m voxeldvc_gb300.build` "
                    "(this package has no CPU fallback)")
            L = C.CDLL(LIB_PATH)
            for name, (res, args) in SIGNATURES.items():
                fn = getattr(L, name)
                fn.restype = res
                fn.argtypes = args
            _lib = L
    return _lib


def last_error() -> str:
    return lib().vdvc_last_error().decode(errors="replace")


def check(status: int, what: str = "") -> None:
    """Map a libvdvc status to the exception the reference would raise."""
    if status == OK:
        return
    msg = last_error()
    text = f"{what}: {msg}" if what else msg
    if status in (ERR_ARG, ERR_INDEX_RANGE):
        raise ValueError(text)
    if status == ERR_ZERO_DIVISION:
        raise ZeroDivisionError(text or "float division by zero")
    if status == ERR_UNSUPPORTED:
        raise NotImplementedError(text)
    if status == ERR_NONFINITE:
        raise FloatingPointError(text)
    if status == ERR_TIMEOUT:
        raise VdvcTimeout(f"libvdvc status {status} (device-side wait timed out): {text}")
    raise VdvcError(f"libvdvc status {status} ({lib().vdvc_status_string(status).decode()}): {text}")


def launch_count() -> int:
    return int(lib().vdvc_launch_count())
