"""Stage 1 of the ground-truth pipeline (ground_truth/prepare_ground_truth.py
of the reference): the reference / deformed image pair for a known
displacement field, with the backward warp on the GPU (`vdvc_gt_warp`).

  --gt-ref-file PATH            reference image .npy, shape (N, N, N)
  --gt-displacement-file PATH   displacement .npy, shape (N+1, N+1, N+1, 3),
                                channels-last, voxel units, sampled at the
                                integer coordinates 0..N
  --tensile-strain STRAIN       instead: u_x = STRAIN x, u_y = u_z = 0
  --output-dir DIR              ref.npy, deformed.npy (float64),
                                u_gt_vox.npy (N, N, N, 3), gt_meta.json

deformed(x) = ref(x - u_gt(x)), trilinear with linear extrapolation past
the image edges (scipy RegularGridInterpolator, fill_value None).
"""
from __future__ import annotations

import argparse
import json
import os
import sys

import numpy as np

from .. import _device as D
from .. import _lib

GT_DIR = os.path.join(os.path.abspath('assets'), 'GT_z+0.01')
DEFAULT_GT_REF_FILE = os.path.join(GT_DIR, 'ref.npy')
DEFAULT_GT_DISPLACEMENT_FILE = os.path.join(GT_DIR, 'U.npy')
DEFAULT_OUTPUT_DIR = os.path.join(os.path.abspath('dvc_elastic_groundtruth'), 'gt_input')


def make_deformed_image(ref, u_gt_vox, xp=np):
    """deformed(x) = ref(x - u(x)) for ref (nx, ny, nz) and u_gt_vox
    (nx, ny, nz, 3), float64; bit-identical to the reference's
    RegularGridInterpolator evaluation.
    Reference: ground_truth/prepare_ground_truth.py:68-90."""
    r = D.to_device(np.ascontiguousarray(ref) if not D.is_tensor(ref) else ref, np.float64)
    u = D.to_device(np.ascontiguousarray(u_gt_vox) if not D.is_tensor(u_gt_vox) else u_gt_vox, np.float64)
    nx, ny, nz = (int(s) for s in r.shape)
    if tuple(u.shape) != (nx, ny, nz, 3):
        raise ValueError(f"u_gt_vox must have shape {(nx, ny, nz, 3)}, got {tuple(u.shape)}")
    out = D.empty(nx * ny * nz, np.float64)
    _lib.check(_lib.lib().vdvc_gt_warp(r.data_ptr(), u.data_ptr(), nx, ny, nz, out.data_ptr(), D.stream()),
               "make_deformed_image")
    return D.out(out.view(nx, ny, nz), xp)


def make_uniaxial_gt(n, strain):
    """(n, n, n, 3) field u_x = strain * x, u_y = u_z = 0 on the integer grid.
    Reference: ground_truth/prepare_ground_truth.py:93-107."""
    u = np.zeros((n, n, n, 3), dtype=np.float64)
    u[..., 0] = strain * np.arange(n, dtype=np.float64)[:, None, None]
    return u


def gt_at_voxels(u_gt, shape):
    """The displacement at the image voxels 0..N-1 of its (N+1)^3 integer
    grid.  The reference interpolates it trilinearly there; at grid points
    the weights are exactly 0 and 1, so that is the grid's own values."""
    nx, ny, nz = shape
    return np.ascontiguousarray(np.asarray(u_gt, dtype=np.float64)[:nx, :ny, :nz])


def parse_args(argv=None):
    """Reference: ground_truth/prepare_ground_truth.py:110-138."""
    p = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    p.add_argument('--gt-ref-file', type=str, default=DEFAULT_GT_REF_FILE, dest='gt_ref_file')
    g = p.add_mutually_exclusive_group()
    g.add_argument('--gt-displacement-file', type=str, default=DEFAULT_GT_DISPLACEMENT_FILE,
                   dest='gt_displacement_file')
    g.add_argument('--tensile-strain', type=float, default=None, dest='tensile_strain')
    p.add_argument('--output-dir', type=str, default=DEFAULT_OUTPUT_DIR, dest='output_dir')
    return p.parse_args(argv)


def main(argv=None):
    """Reference: ground_truth/prepare_ground_truth.py:141-226."""
    args = parse_args(argv)
    out_dir = os.path.expanduser(args.output_dir)
    ref_file = os.path.expanduser(args.gt_ref_file)
    os.makedirs(out_dir, exist_ok=True)
    print("=" * 70)
    print("PREPARE GROUND-TRUTH IMAGE PAIR")
    print("=" * 70)
    ref_raw = np.load(ref_file)
    nx, ny, nz = ref_raw.shape
    assert nx == ny == nz, f"reference image must be cubic (N,N,N), got {ref_raw.shape}"
    if args.tensile_strain is not None:
        print(f"\nImposing synthetic uniaxial tensile strain: du_x/dx = {args.tensile_strain} "
              f"(x direction only, u_y=u_z=0)")
        u_gt = make_uniaxial_gt(nx + 1, args.tensile_strain)
        source = {'type': 'tensile_strain', 'strain': args.tensile_strain}
    else:
        disp_file = os.path.expanduser(args.gt_displacement_file)
        u_gt = np.load(disp_file).astype(np.float64)
        want = (nx + 1, ny + 1, nz + 1)
        assert u_gt.shape[:3] == want and u_gt.shape[3:] == (3,), (
            f"ground-truth displacement field must have shape (N+1,N+1,N+1,3) for an (N,N,N) reference image; "
            f"got reference {ref_raw.shape} vs. displacement {u_gt.shape}, expected {want + (3,)}.")
        source = {'type': 'ct_displacement_field', 'file': disp_file}
    print(f"Reference: {ref_raw.shape} {ref_raw.dtype}  min={ref_raw.min()}  max={ref_raw.max()}")
    print(f"GT displacement: {u_gt.shape} {u_gt.dtype}")
    for c, name in enumerate(['ux', 'uy', 'uz']):
        print(f"  GT {name}: min={u_gt[..., c].min():.4f}  max={u_gt[..., c].max():.4f}")
    u_vox = gt_at_voxels(u_gt, (nx, ny, nz))
    print("\nGT displacement at image voxels (interpolated):")
    for c, name in enumerate(['ux', 'uy', 'uz']):
        print(f"  {name}: min={u_vox[..., c].min():.4f}  max={u_vox[..., c].max():.4f}")
    deformed = make_deformed_image(ref_raw.astype(np.float64), u_vox)
    print(f"\nDeformed image: min={deformed.min():.2f}  max={deformed.max():.2f}")
    paths = {k: os.path.join(out_dir, f) for k, f in
             (('ref', 'ref.npy'), ('def', 'deformed.npy'), ('u', 'u_gt_vox.npy'), ('meta', 'gt_meta.json'))}
    np.save(paths['ref'], ref_raw)
    np.save(paths['def'], deformed)
    np.save(paths['u'], u_vox)
    with open(paths['meta'], 'w') as fh:
        json.dump({'gt_ref_file': ref_file, 'ground_truth_source': source, 'ref_shape': list(ref_raw.shape),
                   'ref_dtype': str(ref_raw.dtype)}, fh, indent=2)
    print(f"\nSaved {paths['ref']}  shape={ref_raw.shape}  dtype={ref_raw.dtype}")
    print(f"Saved {paths['def']}  shape={deformed.shape}  dtype={deformed.dtype}")
    print(f"Saved {paths['u']}  shape={u_vox.shape}  dtype={u_vox.dtype}")
    print(f"Saved {paths['meta']}")
    print("\n✓ PREPARE GROUND-TRUTH COMPLETE")
    return 0


if __name__ == "__main__":
    sys.exit(main())
