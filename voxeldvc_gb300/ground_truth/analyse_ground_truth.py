"""Stage 4 of the ground-truth pipeline (ground_truth/analyse_ground_truth.py
of the reference): score the displacement `voxeldvc run` recovered against
the known field, at the mesh nodes and at every voxel of the reference crop.

  --work-dir DIR   preprocess / run output (affine_prealign.json,
                   U_recovered.npy, ref.npy, and the masks
                   unsafe_voxel_mask.npy / overlap_lost_element_mask.npy)
  --gt-dir DIR     prepare stage output (u_gt_vox.npy, deformed.npy)

U_recovered.npy maps crop-local reference positions to full-image deformed
positions, so crop_lo is subtracted before the comparison.  Nodes whose
support box (voxels within h) maps partly outside the deformed image under
the known field are "truncated"; the "valid" set also drops nodes and voxels
the saved solver masks flag.  The recoverability masks, the support
fractions and the per-voxel FE interpolation run on the GPU
(`vdvc_gt_voxel_in_bounds`, `vdvc_gt_node_oob_fraction`,
`vdvc_interp_field`); the printed statistics are host reductions of the
saved arrays.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import sys

import numpy as np

from .. import _device as D
from .. import _lib
from ..engine.correlate_gpu import interp_field_vox
from ..engine.geometry_dvc import build_N_stencil, build_node_index, element_node_ids
from ..run_dvc import _Tee, mesh_dims

DEFAULT_WORK_DIR = os.path.abspath('dvc_elastic_groundtruth')
DEFAULT_GT_DIR = os.path.join(DEFAULT_WORK_DIR, 'gt_input')


def parse_args(argv=None):
    """Reference: ground_truth/analyse_ground_truth.py:84-91."""
    p = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    p.add_argument('--work-dir', type=str, default=DEFAULT_WORK_DIR, dest='work_dir')
    p.add_argument('--gt-dir', type=str, default=DEFAULT_GT_DIR, dest='gt_dir')
    return p.parse_args(argv)


def grid_to_dofs(U_grid):
    """(nbx, nby, nbz, 3) nodal grid -> flat node-major DOFs U[3 node + c].
    Reference: ground_truth/analyse_ground_truth.py:94-105."""
    return np.ascontiguousarray(np.transpose(np.asarray(U_grid), (2, 1, 0, 3))).reshape(-1)


def _in_bounds_dev(u_gt_vox, g_shape):
    u = D.to_device(np.ascontiguousarray(u_gt_vox) if not D.is_tensor(u_gt_vox) else u_gt_vox, np.float64)
    nx, ny, nz = (int(s) for s in u.shape[:3])
    out = D.empty(nx * ny * nz, np.uint8)
    _lib.check(_lib.lib().vdvc_gt_voxel_in_bounds(u.data_ptr(), nx, ny, nz, *(int(s) for s in g_shape),
                                                  out.data_ptr(), D.stream()), "voxel_in_bounds")
    return out, (nx, ny, nz)


def voxel_in_bounds(u_gt_vox, g_shape):
    """(nx, ny, nz) bool: x + u_gt(x) inside the deformed image (g_origin 0).
    Reference: ground_truth/analyse_ground_truth.py:108-129."""
    out, shape = _in_bounds_dev(u_gt_vox, g_shape)
    return D.out(out.view(D.torch().bool).view(*shape), np)


def node_oob_fraction(u_gt_vox_full, h, nbfx, nbfy, nbfz, g_shape, crop_lo):
    """(nbfx, nbfy, nbfz): per node at crop_lo + (i, j, k) h, the fraction of
    its support box [v - h, v + h] (clamped to the image) whose voxels map
    outside the deformed image under the known field.
    Reference: ground_truth/analyse_ground_truth.py:132-165."""
    inb, (nx, ny, nz) = _in_bounds_dev(u_gt_vox_full, g_shape)
    out = D.empty(nbfx * nbfy * nbfz, np.float64)
    lo = (C.c_longlong * 3)(*(int(x) for x in crop_lo))
    _lib.check(_lib.lib().vdvc_gt_node_oob_fraction(inb.data_ptr(), nx, ny, nz, int(h), nbfx, nbfy, nbfz, lo,
                                                    out.data_ptr(), D.stream()), "node_oob_fraction")
    return D.out(out.view(nbfx, nbfy, nbfz), np)


def load_validity_masks(work_dir, Nx_e, Ny_e, Nz_e):
    """(node_masked_out (nbx, nby, nbz), vox_masked_out (Nvx, Nvy, Nvz)) from
    the saved solver masks, or (None, None) when they are absent: voxels
    flagged in unsafe_voxel_mask.npy, and nodes of any element flagged in
    overlap_lost_element_mask.npy.
    Reference: ground_truth/analyse_ground_truth.py:168-201."""
    elem_path = os.path.join(work_dir, 'overlap_lost_element_mask.npy')
    vox_path = os.path.join(work_dir, 'unsafe_voxel_mask.npy')
    if not (os.path.exists(elem_path) and os.path.exists(vox_path)):
        return None, None
    vox_masked_out = np.load(vox_path).astype(bool)
    ol = np.load(elem_path).astype(bool).flatten(order='F')
    node_idx = build_node_index(Nx_e, Ny_e, Nz_e)
    elem_nodes = element_node_ids(node_idx, Nx_e, Ny_e, Nz_e)
    flat = np.zeros(node_idx.size, dtype=bool)
    flat[elem_nodes[ol].ravel()] = True
    return flat[node_idx], vox_masked_out


def _table_row(name, gt_c, rec_c, err_c):
    return (f"  {name:<10} {gt_c.mean():>10.5f} {gt_c.std():>10.5f} {rec_c.mean():>10.5f} {rec_c.std():>10.5f} "
            f"{np.sqrt(np.mean(err_c ** 2)):>10.5f} {np.max(np.abs(err_c)):>10.5f}")


HEADER = (f"{'Component':<12} {'GT mean':>10} {'GT std':>10} "
          f"{'Rec mean':>10} {'Rec std':>10} {'RMS err':>10} {'Max |err|':>10}")


def analyse(work_dir, gt_dir):
    """The comparison; returns a dict of the headline figures (node RMS
    over the recoverable and valid sets, voxel RMS) besides printing and
    saving what the reference prints and saves."""
    with open(os.path.join(work_dir, 'affine_prealign.json')) as fh:
        meta = json.load(fh)
    h = int(meta['h'])
    crop_lo = np.array(meta['crop_lo'])
    U_rec = np.load(os.path.join(work_dir, 'U_recovered.npy')) - crop_lo
    ref_crop = np.load(os.path.join(work_dir, 'ref.npy'))
    Nx_e, Ny_e, Nz_e = mesh_dims(ref_crop.shape, h)
    nb = (Nx_e + 1, Ny_e + 1, Nz_e + 1)
    assert U_rec.shape[:3] == nb
    print(f"work_dir={work_dir}  mesh: Nx_e={Nx_e}, Ny_e={Ny_e}, Nz_e={Nz_e}  h={h}  crop_lo={crop_lo.tolist()}")
    u_full = np.load(os.path.join(gt_dir, 'u_gt_vox.npy'))
    g_shape = np.load(os.path.join(gt_dir, 'deformed.npy'), mmap_mode='r').shape
    print(f"gt_dir={gt_dir}  u_gt_vox_full shape={u_full.shape}  deformed_full shape={tuple(g_shape)}")

    u_nodes = u_full[np.ix_(*(crop_lo[a] + np.arange(nb[a]) * h for a in range(3)))]
    error = U_rec - u_nodes
    oob = node_oob_fraction(u_full, h, *nb, g_shape, crop_lo)
    truncated = oob > 0
    recoverable = ~truncated
    node_out, vox_out = load_validity_masks(work_dir, Nx_e, Ny_e, Nz_e)
    have = node_out is not None
    node_valid = recoverable & ~node_out if have else None

    print("\n" + "=" * 70)
    print("GROUND-TRUTH COMPARISON (at mesh nodes)")
    print("=" * 70)
    print(HEADER)
    for c, name in enumerate(['ux', 'uy', 'uz']):
        print(_table_row(name, u_nodes[..., c], U_rec[..., c], error[..., c]))

    def region(mask):
        if not np.any(mask):
            return 0, float('nan'), float('nan')
        e = error[mask]
        return int(mask.sum()), float(np.sqrt(np.mean(e ** 2))), float(np.max(np.linalg.norm(e, axis=-1)))

    print("\n  Displacement error by region (truncated nodes reported separately):")
    print(f"  {'Region':<34} {'#nodes':>7} {'RMS err':>10} {'Max |err|':>10}")
    regions = [('recoverable (support in g)', recoverable)]
    if have:
        regions.append(('valid (recoverable & unmasked)', node_valid))
    regions += [('truncated (support clipped)', truncated), ('all nodes', np.ones_like(truncated))]
    stats = {}
    for label, mask in regions:
        n, rms, mx = region(mask)
        stats[label.split(' ')[0]] = (n, rms, mx)
        print(f"  {label:<34} {n:>7d} {rms:>10.5f} {mx:>10.5f}")
    print(f"\n  Truncated nodes: {int(truncated.sum())}/{truncated.size} "
          f"(max support out-of-bounds fraction = {oob.max():.3f})")
    if have:
        print(f"  Masked-out (boundary shell / overlap-lost) among recoverable: "
              f"{int((recoverable & node_out).sum())}/{int(recoverable.sum())}")
    np.save(os.path.join(work_dir, 'U_gt_nodes.npy'), u_nodes)
    np.save(os.path.join(work_dir, 'U_error.npy'), error)
    np.save(os.path.join(work_dir, 'node_truncated_mask.npy'), truncated)
    np.save(os.path.join(work_dir, 'node_oob_fraction.npy'), oob)
    if have:
        np.save(os.path.join(work_dir, 'node_valid_mask.npy'), node_valid)

    Nvx, Nvy, Nvz = ref_crop.shape
    sl = tuple(slice(crop_lo[a], crop_lo[a] + n) for a, n in enumerate((Nvx, Nvy, Nvz)))
    u_gt_vox = u_full[sl]
    N_stencil, _ = build_N_stencil(h)
    u_rec_vox = interp_field_vox(grid_to_dofs(U_rec), N_stencil, h, Nx_e, Ny_e, Nz_e, np)
    u_rec_vox = np.asarray(u_rec_vox).reshape(Nvx, Nvy, Nvz, 3, order='F')
    err_vox = u_rec_vox - u_gt_vox
    vox_rec = voxel_in_bounds(u_full, g_shape)[sl]

    def voxel_table(sel):
        for c, name in enumerate(['ux', 'uy', 'uz']):
            print(_table_row(name, u_gt_vox[..., c][sel], u_rec_vox[..., c][sel], err_vox[..., c][sel]))

    print("\n" + "=" * 70)
    print("GROUND-TRUTH COMPARISON (at every voxel)")
    print("=" * 70)
    print(HEADER)
    voxel_table(vox_rec)
    print(f"  (restricted to recoverable voxels: {int(vox_rec.sum())} -- support in g under the GT field)")
    stats['voxel_recoverable_rms'] = float(np.sqrt(np.mean(err_vox[vox_rec] ** 2)))
    if have:
        vox_valid = vox_rec & ~vox_out
        print("\n" + HEADER)
        voxel_table(vox_valid)
        print(f"  (restricted to VALID voxels: {int(vox_valid.sum())} -- recoverable AND not mask-flagged)")
        stats['voxel_valid_rms'] = float(np.sqrt(np.mean(err_vox[vox_valid] ** 2)))
    np.save(os.path.join(work_dir, 'U_gt_vox.npy'), u_gt_vox)
    np.save(os.path.join(work_dir, 'U_recovered_vox.npy'), u_rec_vox)
    np.save(os.path.join(work_dir, 'U_error_vox.npy'), err_vox)
    np.save(os.path.join(work_dir, 'voxel_recoverable_mask.npy'), vox_rec)
    if have:
        np.save(os.path.join(work_dir, 'voxel_valid_mask.npy'), vox_rec & ~vox_out)
    print("\n✓ GROUND-TRUTH COMPARISON COMPLETE")
    return stats


def analyse_logged(work_dir, gt_dir):
    """analyse() with its report also written to
    <work_dir>/ground_truth_comparison_log.txt; returns analyse()'s figures."""
    log_path = os.path.join(work_dir, 'ground_truth_comparison_log.txt')
    log_file = open(log_path, 'w')
    stdout = sys.stdout
    sys.stdout = _Tee(stdout, log_file)
    try:
        print("=" * 70)
        print("GROUND-TRUTH COMPARISON")
        print("=" * 70)
        stats = analyse(work_dir, gt_dir)
    finally:
        sys.stdout = stdout
        log_file.close()
    print(f"Log written to {log_path}")
    return stats


def main(argv=None):
    """Reference: ground_truth/analyse_ground_truth.py:204-382."""
    args = parse_args(argv)
    analyse_logged(os.path.expanduser(args.work_dir), os.path.expanduser(args.gt_dir))
    return 0


if __name__ == "__main__":
    sys.exit(main())
