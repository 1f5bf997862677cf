"""`voxeldvc preprocess` (preprocess.py of the reference) on the GPU: the
affine warp of the deformed volume onto the reference grid, integer binning,
the n h + 1 crop of the valid overlap, and the command itself (`main`: load,
bin, crop, affine prealign + refine, crop, save the cropped volumes and
affine_prealign.json with the reference's keys).  Same names, arguments,
printed lines and returns as the reference; volumes are numpy pix[x, y, z]
arrays (or CUDA tensors), C order.
"""
from __future__ import annotations

import argparse
import json
import os
import sys

import numpy as np

from . import _device as D
from . import _lib

_BIN_TYPES = {np.dtype(np.float32): _lib.F32, np.dtype(np.uint8): _lib.U8, np.dtype(np.uint16): _lib.U16,
              np.dtype(np.int16): _lib.I16}


def _dev_f32(vol):
    if not D.is_tensor(vol) and np.asarray(vol).dtype == np.uint16:
        vol = np.asarray(vol, np.float32)  # no uint16 device arithmetic in torch
    return D.to_device(vol, np.float32).contiguous()


def warp_onto_ref_grid(A, t, c, Nf, g_gpu, xp, chunk=30):
    """g sampled on f's voxel grid at x' = A (x - c) + c + t (trilinear, 0
    outside g).  Returns a float32 numpy array of shape Nf (the reference
    returns host memory too); `chunk` is accepted and ignored -- the warp is
    one pass.
    Reference: preprocess.py:233-285."""
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
    shape must be divisible by B.
    Reference: preprocess.py:288-312."""
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
    and re-centred, shifted into f's bounds.  Returns lo, hi (hi exclusive).
    Reference: preprocess.py:315-367."""
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


# ---- `voxeldvc preprocess` (preprocess.py:372-695) -------------------------

DEFAULT_H = 8


def load_volume(filepath):
    """.npy volume (or .tif/.tiff through tifffile where it is installed).
    Reference: preprocess.py:72-85."""
    ext = os.path.splitext(filepath)[1].lower()
    if ext == '.npy':
        return np.load(filepath)
    if ext in ('.tif', '.tiff'):
        import tifffile
        return tifffile.imread(filepath)
    raise ValueError(f"Unsupported file format: {ext}")


def rotation_angles_deg(A):
    """Euler angles (deg, x y z) of the rotation R of the polar
    decomposition A = R P, and P's diagonal (the axis-aligned scale).
    Reference: preprocess.py:199-219."""
    Us, _, Vt = np.linalg.svd(A)
    R = Us @ Vt
    if np.linalg.det(R) < 0:
        R = R.copy()
        R[:, -1] *= -1
    angles = (np.degrees(np.arctan2(R[2, 1], R[2, 2])),
              np.degrees(np.arctan2(-R[2, 0], np.hypot(R[2, 1], R[2, 2]))),
              np.degrees(np.arctan2(R[1, 0], R[0, 0])))
    return angles, np.diag(R.T @ A).copy()


def normal_strains(A):
    """diag(I - A^-1): the per-axis normal strain in the reference frame.
    Reference: preprocess.py:222-230."""
    return np.diag(np.eye(3) - np.linalg.inv(A))


def _box(title, rows):
    w = max(len(str(k)) for k, _ in rows)
    print(f"+-- {title} " + "-" * max(4, 60 - len(title)))
    for k, v in rows:
        print(f"| {str(k):<{w}}  {v}")
    print("+" + "-" * (65 if len(title) < 60 else len(title) + 5))


def _affine_rows(A, t, c):
    angles, scales = rotation_angles_deg(A)
    eps = normal_strains(A)
    return [("Rotation  [deg]", "  ".join(f"{a:+.3f}" for a in angles)),
            ("Scale", "  ".join(f"{s:.4f}" for s in scales)),
            ("Normal strain", "  ".join(f"{e:+.5f}" for e in eps)),
            ("Translation [vox]", "  ".join(f"{x:+.3f}" for x in t)),
            ("Center [vox]", "  ".join(f"{x:.2f}" for x in c))]


def _fail(*lines):
    for ln in lines:
        print(ln)
    sys.exit(1)


def parse_args(argv=None):
    p = argparse.ArgumentParser(description="Affine pre-alignment and n*h+1 overlap crop of a reference / "
                                            "deformed volume pair (GB300).")
    p.add_argument('ref_path', type=str, nargs='?', help='Path to reference image (.npy file)')
    p.add_argument('def_path', type=str, nargs='?', help='Path to deformed image (.npy file)')
    p.add_argument('--h', type=int, default=DEFAULT_H, dest='h',
                   help=f'DVC element edge length in voxels (default: {DEFAULT_H}).')
    p.add_argument('--glt', type=float, default=0.0, dest='glt', help='Gray-level threshold (default: 0.0).')
    p.add_argument('--bin', type=int, default=1, dest='bin_factor', help='Spatial binning factor (default: 1).')
    p.add_argument('--decimate', type=int, default=4, dest='decimate',
                   help='Downsampling factor for affine pre-alignment (default: 4).')
    p.add_argument('--no-affine-refine', action='store_true', dest='no_affine_refine',
                   help='Skip the full-resolution Gauss-Newton refinement of the affine.')
    p.add_argument('--output-dir', type=str, required=True, dest='output_dir', help='Output directory (required).')
    p.add_argument('--crop', type=int, nargs=3, default=[0, 0, 0], dest='crop', metavar=('X', 'Y', 'Z'),
                   help='Pixels to crop symmetrically from each axis (default: 0 0 0).')
    return p.parse_args(argv)


def main(argv=None):
    """Same steps, outputs and affine_prealign.json keys as the reference's
    preprocess: load, bin, symmetric crop, affine prealign (+ Gauss-Newton
    refine), warp onto the reference grid, n h + 1 overlap crop, deformed
    bounding box, save.
    Reference: preprocess.py:372-691."""
    from .engine.correlate_gpu import affine_prealign, affine_refine_gn
    args = parse_args(argv)
    if args.ref_path is None:
        _fail("ERROR: Missing required parameter 'ref_path'",
              "Usage: python preprocess.py <ref_path> <def_path> [options]")
    if args.def_path is None:
        _fail("ERROR: Missing required parameter 'def_path'",
              "Usage: python preprocess.py <ref_path> <def_path> [options]")
    h, glt, B, crop_vals, decimate = args.h, args.glt, args.bin_factor, args.crop, args.decimate
    ref_path, def_path = os.path.expanduser(args.ref_path), os.path.expanduser(args.def_path)
    if B < 1:
        _fail("ERROR: Invalid parameter '--bin': must be >= 1", f"       Received: {B}")
    if decimate < 1:
        _fail("ERROR: Invalid parameter '--decimate': must be >= 1", f"       Received: {decimate}")
    if any(cv < 0 for cv in crop_vals):
        _fail("ERROR: Invalid parameter '--crop': all values must be >= 0", f"       Received: {crop_vals}")
    for name, path in (("ref_path", ref_path), ("def_path", def_path)):
        if not os.path.exists(path):
            kind = "Reference" if name == "ref_path" else "Deformed"
            _fail(f"ERROR: {kind} image file not found", f"       Parameter '{name}': {path}")
    output_dir = os.path.expanduser(args.output_dir)
    print()
    _box("Parameters as understood by the program",
         [("ref_path", ref_path), ("def_path", def_path), ("h (element size)", h), ("glt (gray thresh)", glt),
          ("bin_factor", B), ("crop (x,y,z)", crop_vals), ("output_dir", output_dir)])
    print(f"\nElement edge length h = {h}  |  bin factor = {B}")

    print(f"Loading {ref_path}")
    ref = load_volume(ref_path)
    ref_dtype = ref.dtype
    print(f"  ref:      shape={ref.shape}  dtype={ref.dtype}")
    print(f"Loading {def_path}")
    deformed = load_volume(def_path)
    def_dtype = deformed.dtype
    print(f"  deformed: shape={deformed.shape}  dtype={deformed.dtype}")

    if B > 1:
        rt = tuple((s // B) * B for s in ref.shape)
        dt = tuple((s // B) * B for s in deformed.shape)
        ref = bin_volume(np.ascontiguousarray(ref[:rt[0], :rt[1], :rt[2]]), B)
        deformed = bin_volume(np.ascontiguousarray(deformed[:dt[0], :dt[1], :dt[2]]), B)
        print(f"\nAfter binning by {B}:")
        print(f"  ref:      shape={ref.shape}  dtype={ref.dtype}")
        print(f"  deformed: shape={deformed.shape}  dtype={deformed.dtype}")

    if any(cv > 0 for cv in crop_vals):
        lo_c, hi_c = [0, 0, 0], list(ref.shape)
        for i, cv in enumerate(crop_vals):
            if cv > 0:
                lo_c[i] = cv // 2
                hi_c[i] -= cv - cv // 2
                if lo_c[i] >= hi_c[i]:
                    _fail(f"ERROR: crop value {cv} for axis {i} exceeds dimension {ref.shape[i]}")
        ref = ref[lo_c[0]:hi_c[0], lo_c[1]:hi_c[1], lo_c[2]:hi_c[2]]
        deformed = deformed[lo_c[0]:hi_c[0], lo_c[1]:hi_c[1], lo_c[2]:hi_c[2]]
        print("\nAfter additional cropping:")
        print(f"  ref:      shape={ref.shape}  dtype={ref.dtype}")
        print(f"  deformed: shape={deformed.shape}  dtype={deformed.dtype}")

    f_pix = _dev_f32(np.ascontiguousarray(ref))
    g_pix = _dev_f32(np.ascontiguousarray(deformed))
    print(f"\nRunning affine_prealign (decimate={decimate}) …")
    A, t, c, info = affine_prealign(f_pix, g_pix, np, decimate=decimate, disp=True)
    _box("Recovered affine transform (x y z)", _affine_rows(A, t, c))
    c_id, c_tr, c_af = info['cost_identity'], info['cost_translation_only'], info['cost_final']
    imp = (lambda v: "—" if c_id == 0 else f"{100.0 * (c_id - v) / c_id:+.1f}%")
    _box("Alignment quality", [("No alignment (identity)", f"{c_id:.4f}  baseline"),
                               ("+ translation (FFT)", f"{c_tr:.4f}  {imp(c_tr)}"),
                               ("+ full affine", f"{c_af:.4f}  {imp(c_af)}"),
                               ("optimiser evaluations (nfev)", info['nfev'])])
    refine_info = None
    if not args.no_affine_refine:
        print("\nRefining affine by full-resolution Gauss-Newton (coarse-to-fine) …")
        A, t, refine_info = affine_refine_gn(f_pix, g_pix, np, A, t, c, disp=False)
        _box("Recovered affine transform (x y z)", _affine_rows(A, t, c))
        r0, r1 = refine_info['rms_initial'], refine_info['rms_final']
        _box("Affine refinement (Gauss-Newton)",
             [("Coarse prealign", f"{r0:.2f}  baseline"),
              ("+ Gauss-Newton refine", f"{r1:.2f}  " + ("—" if r0 == 0 else f"{100.0 * (r0 - r1) / r0:+.1f}%")),
              ("GN iters/level", refine_info['iters'])])
    del f_pix

    print("\nWarping deformed onto reference grid …")
    g_warped = warp_onto_ref_grid(A, t, c, ref.shape, g_pix, np)
    del g_pix
    print(f"  g_warped: shape={g_warped.shape}  above-glt={100.0 * np.count_nonzero(g_warped > glt) / g_warped.size:.1f}%")
    print("\nFinding overlap crop …")
    lo, hi = compute_crop(ref, g_warped, h, glt)
    del g_warped
    crop_shape = tuple(int(x) for x in (hi - lo))
    print(f"\nFinal crop shape : {crop_shape}")
    print(f"  slice  [{lo[0]}:{hi[0]}, {lo[1]}:{hi[1]}, {lo[2]}:{hi[2]}]")
    print(f"  coverage : ref {100 * np.prod(crop_shape) / ref.size:.1f}%")
    for i, s in enumerate(crop_shape):
        n = (s - 1) // h
        assert s == n * h + 1, f"axis {i}: {s} is not n*{h}+1"
        print(f"  axis {i} : {s} = {n}*{h}+1  ✓")
    ref_crop = ref[lo[0]:hi[0], lo[1]:hi[1], lo[2]:hi[2]]
    def_ref_aligned = deformed[lo[0]:hi[0], lo[1]:hi[1], lo[2]:hi[2]]

    # deformed-image box sampled by the correlation: the crop's 8 corners
    # through the affine, 1 voxel of margin below and 2 above, clamped
    corners = np.array([[lo[0] + dx * (hi[0] - lo[0] - 1), lo[1] + dy * (hi[1] - lo[1] - 1),
                         lo[2] + dz * (hi[2] - lo[2] - 1)] for dx in (0, 1) for dy in (0, 1) for dz in (0, 1)],
                       dtype=np.float64)
    mapped = (corners - c) @ A.T + c + t
    lo_def = np.maximum(np.floor(mapped.min(axis=0)).astype(int) - 1, 0)
    hi_def = np.minimum(np.ceil(mapped.max(axis=0)).astype(int) + 2, np.array(deformed.shape))
    def_crop = deformed[lo_def[0]:hi_def[0], lo_def[1]:hi_def[1], lo_def[2]:hi_def[2]]
    print("\nDeformed bounding box for correlation:")
    print(f"  lo_def = {lo_def.tolist()}  hi_def = {hi_def.tolist()}")
    print(f"  def_preprocessed shape = {def_crop.shape}")

    ref_crop = ref_crop.astype(ref_dtype)
    def_crop = def_crop.astype(def_dtype)
    def_ref_aligned = def_ref_aligned.astype(def_dtype)
    out_ref = os.path.join(output_dir, 'ref_preprocessed.npy')
    out_def = os.path.join(output_dir, 'def_preprocessed.npy')
    out_ali = os.path.join(output_dir, 'def_ref_aligned.npy')
    out_json = os.path.join(output_dir, 'affine_prealign.json')
    os.makedirs(output_dir, exist_ok=True)
    np.save(out_ref, ref_crop)
    np.save(out_def, def_crop)
    np.save(out_ali, def_ref_aligned)
    print(f"\nSaved {out_ref}         shape={ref_crop.shape}  dtype={ref_crop.dtype}")
    print(f"Saved {out_def}         shape={def_crop.shape}  dtype={def_crop.dtype}")
    print(f"Saved {out_ali}  shape={def_ref_aligned.shape}  dtype={def_ref_aligned.dtype}")

    angles, scales = rotation_angles_deg(A)
    meta = {
        "description": (
            "Affine pre-alignment parameters; glt is the gray-level threshold reused by run_dvc. "
            "All spatial quantities (t, c, crop_lo, def_lo) are in binned voxel units; A is dimensionless. "
            "def_preprocessed.npy is the original (non-warped) deformed volume cropped to [def_lo, def_hi); "
            "def_ref_aligned.npy is the deformed volume at the reference crop's index range. "
            "For a DVC node at output position x_out: u_affine = (A-I) @ (x_out + crop_lo - c) + t "
            "[binned voxels]; u_total_fullres = (u_affine + u_dvc) * bin_factor."),
        "h": h, "glt": glt, "bin_factor": B, "additional_crop_xyz": crop_vals,
        "ref_file": ref_path, "def_file": def_path,
        "ref_crop_file": out_ref, "def_crop_file": out_def, "def_ref_aligned_file": out_ali,
        "crop_lo": [int(x) for x in lo], "crop_hi": [int(x) for x in hi], "crop_shape": list(crop_shape),
        "def_lo": [int(x) for x in lo_def], "def_hi": [int(x) for x in hi_def],
        "affine_A": A.tolist(), "affine_t": t.tolist(), "affine_c": c.tolist(),
        "affine_t_fullres": (t * B).tolist(), "affine_c_fullres": (c * B).tolist(),
        "rotation_deg_xyz": [float(a) for a in angles], "scale_xyz": [float(s) for s in scales],
        "normal_strain_xyz": [float(e) for e in normal_strains(A)],
        "cost_identity": float(c_id), "cost_translation_only": float(c_tr), "cost_affine": float(c_af),
        "nfev": int(info['nfev']),
        "affine_refine": (None if refine_info is None else {
            "rms_initial": float(refine_info['rms_initial']), "rms_final": float(refine_info['rms_final']),
            "iters": [int(n) for n in refine_info['iters']]}),
    }
    with open(out_json, 'w') as fh:
        json.dump(meta, fh, indent=2)
    print(f"Saved {out_json}")
    return 0


if __name__ == '__main__':
    sys.exit(main())
