"""`voxeldvc run WORK_DIR` on the GB300 engine (reference: src/voxeldvc/run_dvc.py).

Reads the preprocess outputs of WORK_DIR (affine_prealign.json,
ref_preprocessed.npy, def_preprocessed.npy), runs the multiscale GN solve
with the reference's fixed settings (scales (2,1,0), dynamic mask frozen
after 4 iterations, external affine seed adjusted for the crop offsets,
Laplacian regulariser with l0 = l0_factor * h) and writes the solve's
results:

  U_recovered.npy      (Nx+1, Ny+1, Nz+1, 3) nodal displacement to full-image
                        deformed coordinates (def_lo added back)
  U_local.npy          same layout, the displacement minus the affine seed
  residual.npy         (Nvx, Nvy, Nvz) final residual
  dU.npy               (Nx+1, Ny+1, Nz+1, 3) last GN update
  ref.npy, deformed.npy  the reference crop and the deformed volume at the
                        same index range (def_ref_aligned.npy, when present)
  ref_forward_pushed.npy  (Nvx, Nvy, Nvz) reference pushed onto the deformed
                        grid by the local displacement
  principal_strains_cell.npy (Nx, Ny, Nz, 3), equivalent_strain_cell.npy,
  residual_std_cell.npy, zncc_cell.npy, gn_convergence_cell.npy,
  material_cell_mask.npy, material_cell_mask_eroded.npy,
  overlap_lost_element_mask.npy (Nx, Ny, Nz) per-element fields
  unsafe_voxel_mask.npy (Nvx, Nvy, Nvz)
  run_log.txt          the run's printed output

The reference's deformed-configuration remaps (scipy griddata) and VTK
files are not written.
"""
from __future__ import annotations

import argparse
import json
import os
import sys
import time
import warnings

import numpy as np

DEFAULT_L0_FACTOR = 4.5  # dvc_defaults.py:8


class _Tee:
    def __init__(self, *streams):
        self.streams = streams

    def write(self, data):
        for s in self.streams:
            s.write(data)

    def flush(self):
        for s in self.streams:
            s.flush()


def parse_args(argv=None):
    """Reference: run_dvc.py:56-62."""
    p = argparse.ArgumentParser(prog="voxeldvc run")
    p.add_argument('work_dir', type=str)
    p.add_argument('--l0-factor', type=float, default=DEFAULT_L0_FACTOR, dest='l0_factor',
                   help=f"Regularization length l0 = l0_factor * h, in voxels (default: {DEFAULT_L0_FACTOR}).")
    return p.parse_args(argv)


def mesh_dims(shape, h):
    """Largest N per axis with N*h <= shape-1 (write_output.py:228-230)."""
    return tuple((s - 1) // h for s in shape)


def _grid(U, Nx, Ny, Nz):
    # node = i + j(Nx+1) + k(Nx+1)(Ny+1): Fortran order of (Nx+1, Ny+1, Nz+1)
    return np.stack([U[c::3].reshape(Nx + 1, Ny + 1, Nz + 1, order='F') for c in range(3)], axis=-1)


def _dofs(U_grid):
    # inverse of _grid: (Nx+1, Ny+1, Nz+1, 3) -> node-major flat DOFs
    return np.ascontiguousarray(np.transpose(U_grid, (2, 1, 0, 3))).reshape(-1)


def _cell_outputs(work, U, U_grid, dU, res, ref, active, Nx, Ny, Nz, h, glt):
    """Element-scale fields of write_outputs (write_output.py:790-950) and
    the diagnostic masks they gate with (kernels_dvc.py:92-341)."""
    from .engine import write_output as W
    from .engine import kernels_dvc as KD
    Nv = ref.shape
    mask0 = np.ravel(np.asarray(ref), order='F') > glt
    unsafe = KD.compute_unsafe_voxel_mask(active, h, Nx, Ny, Nz)
    safe = W.compute_safe_cell_mask(unsafe, h, Nx, Ny, Nz)
    lost = KD.compute_overlap_lost_element_mask(active, mask0, h, Nx, Ny, Nz).reshape(Nx, Ny, Nz, order='F')
    print(f"Unsafe voxels: {int(unsafe.sum())}/{unsafe.size} ({100 * unsafe.mean():.1f}%)")
    print(f"Safe elements (no unsafe voxel): {int(safe.sum())}/{safe.size} ({100 * safe.mean():.1f}%)")
    print(f"Overlap-lost elements (lost material overlap or <50% material): {int(lost.sum())}/{lost.size} "
          f"({100 * lost.mean():.1f}%)")
    ps = W.compute_principal_strains_cell(U_grid, h)
    for c, name in enumerate(['e1 (max)', 'e2 (mid)', 'e3 (min)']):
        comp = ps[..., c]
        print(f"  cell {name}: mean={comp.mean():.5f}  std={comp.std():.5f}  min={comp.min():.5f}  "
              f"max={comp.max():.5f}")
    eq = W.compute_equivalent_strain(ps)
    print(f"  cell eq. strain: mean={eq.mean():.5f}  std={eq.std():.5f}  min={eq.min():.5f}  max={eq.max():.5f}")
    rstd, zn = W.compute_correlation_quality_cell(res, ref, h, Nx, Ny, Nz)
    gn = W.compute_gn_convergence_cell(dU, U, Nx, Ny, Nz)
    with warnings.catch_warnings():  # all-NaN fields print nan, as the reference's do
        warnings.simplefilter('ignore', RuntimeWarning)
        print(f"  cell residual std: mean={np.nanmean(rstd):.4f}  min={np.nanmin(rstd):.4f}  "
              f"max={np.nanmax(rstd):.4f}")
        print(f"  cell ZNCC: mean={np.nanmean(zn):.5f}  min={np.nanmin(zn):.5f}  max={np.nanmax(zn):.5f}")
        print(f"  cell GN convergence dU/U: mean={np.nanmean(gn):.2e}  min={np.nanmin(gn):.2e}  "
              f"max={np.nanmax(gn):.2e}")
    mat = W.compute_material_cell_mask(ref, h, Nx, Ny, Nz, glt=glt)
    mat_er = W.compute_material_cell_mask_eroded(mat)
    print(f"Material cells (mean reference gray > glt): {int(mat.sum())}/{mat.size} ({100 * mat.mean():.1f}%)")
    for name, arr in (('principal_strains_cell', ps), ('equivalent_strain_cell', eq), ('residual_std_cell', rstd),
                      ('zncc_cell', zn), ('gn_convergence_cell', gn),
                      ('unsafe_voxel_mask', unsafe.reshape(Nv, order='F')),
                      ('overlap_lost_element_mask', lost), ('material_cell_mask', mat),
                      ('material_cell_mask_eroded', mat_er)):
        np.save(os.path.join(work, f'{name}.npy'), arr)
    return unsafe.reshape(Nv, order='F')


def main(argv=None):
    """Reference: run_dvc.py:65-192."""
    from .engine.correlate_gpu import multiscale_correlate_gpu
    from .engine.geometry_dvc import build_K_ref_laplacian

    t_start = time.perf_counter()
    args = parse_args(argv)
    work = os.path.expanduser(args.work_dir)
    log_file = open(os.path.join(work, 'run_log.txt'), 'w')
    stdout = sys.stdout
    sys.stdout = _Tee(stdout, log_file)
    try:
        with open(os.path.join(work, 'affine_prealign.json')) as fh:
            meta = json.load(fh)
        h = int(meta['h'])
        glt = float(meta.get('glt', 0.0))
        A = np.array(meta['affine_A'], dtype=np.float64)
        t = np.array(meta['affine_t'], dtype=np.float64)
        c = np.array(meta['affine_c'], dtype=np.float64)
        crop_lo = np.array(meta['crop_lo'])
        lo_def = np.array(meta['def_lo'])
        # the solve works in def_preprocessed coordinates (run_dvc.py:89-94)
        c_adj = c - crop_lo
        t_adj = t + crop_lo - lo_def

        ref = np.load(os.path.join(work, 'ref_preprocessed.npy'))
        deformed = np.load(os.path.join(work, 'def_preprocessed.npy'))
        Nx, Ny, Nz = mesh_dims(ref.shape, h)
        l0 = args.l0_factor * h
        print("Run configuration")
        for k, v in [("work_dir", work), ("h (element size)", h), ("glt (gray thresh)", glt),
                     ("l0_factor", args.l0_factor), ("l0 [vox]", f"{l0:g}"), ("mesh (Nx,Ny,Nz)", f"{Nx} x {Ny} x {Nz}"),
                     ("ref shape", str(ref.shape)), ("deformed shape", str(deformed.shape))]:
            print(f"  {k:<20} {v}")
        print("\nGPU matrix-free DVC (multiscale, ext_affine U0, original deformed) …")
        t_setup = time.perf_counter()
        U, res, dU = multiscale_correlate_gpu(
            ref, deformed, Nx, Ny, Nz, h, xp=np, scales=(2, 1, 0), l0=l0, glt=glt,
            K_ref_laplacian=build_K_ref_laplacian(), dynamic_mask=True, fft_prealign=False,
            prealign_affine=False, ext_affine=(A, t_adj, c_adj), disp=True, freeze_mask_after=4)
        t_corr = time.perf_counter()
        assert np.all(np.isfinite(U)), "Recovered displacement contains NaN/inf"

        # local displacement = U minus the affine seed field (run_dvc.py:151-159)
        nb = (Nx + 1, Ny + 1, Nz + 1)
        X = np.stack(np.meshgrid(*[np.arange(n) for n in nb], indexing='ij'), axis=-1).astype(np.float64) * h
        u_aff = (X - c_adj) @ A.T + c_adj + t_adj - X
        U_grid = _grid(U, Nx, Ny, Nz)
        U_local = U_grid - u_aff
        U_grid = U_grid + lo_def.reshape(1, 1, 1, 3)  # to full-image deformed coordinates
        np.save(os.path.join(work, 'U_recovered.npy'), U_grid)
        np.save(os.path.join(work, 'U_local.npy'), U_local)
        np.save(os.path.join(work, 'residual.npy'), res.reshape(ref.shape, order='F'))
        np.save(os.path.join(work, 'dU.npy'), _grid(dU, Nx, Ny, Nz))
        np.save(os.path.join(work, 'ref.npy'), ref)
        aligned = os.path.join(work, 'def_ref_aligned.npy')
        if os.path.exists(aligned):
            np.save(os.path.join(work, 'deformed.npy'), np.load(aligned))
        # post-solve voxel stages (engine/write_output.py): the reference
        # pushed onto the deformed grid, and the correlation quality over
        # the active voxels (f and the warped g = f - res)
        from .engine.write_output import push_reference_forward, compute_zncc
        from .engine.correlate_gpu import compute_active_mask
        # pushed with the local displacement (U minus the affine seed), as
        # run_dvc.py:160-172 passes U_push = U_local
        np.save(os.path.join(work, 'ref_forward_pushed.npy'),
                push_reference_forward(ref, _dofs(U_local), Nx, Ny, Nz, h))
        # mask0 & in bounds & g > glt, as write_outputs forms it (write_output.py:766-781)
        active = compute_active_mask(U, deformed, Nx, Ny, Nz, h, np, glt=glt,
                                     mask0_vox=np.ravel(np.asarray(ref), order='F') > glt)
        f_flat = np.ravel(np.asarray(ref, dtype=np.float64), order='F')
        zncc = compute_zncc(f_flat, f_flat - res, active)
        print(f"  ZNCC (active voxels): {zncc:.6f}")
        unsafe_grid = _cell_outputs(work, U, U_grid, dU, res, ref, active, Nx, Ny, Nz, h, glt)
        # the unsafe mask pushed like the reference, nearest-neighbour, and
        # flagged unsafe where its source leaves the reference domain
        # (write_output.py:900-911)
        from .engine.write_output import push_field_forward
        pushed_unsafe = np.asarray(push_field_forward(unsafe_grid.astype(np.uint8), _dofs(U_local), Nx, Ny, Nz, h,
                                                      order=0, mode='constant', cval=1)).astype(bool)
        print(f"Unsafe voxels (forward-pushed to deformed grid): {int(pushed_unsafe.sum())}/{pushed_unsafe.size} "
              f"({100 * pushed_unsafe.mean():.1f}%)")
        np.save(os.path.join(work, 'unsafe_voxel_mask_forward_pushed.npy'), pushed_unsafe)
        for ci, name in enumerate(['ux', 'uy', 'uz']):
            comp = U_grid[..., ci]
            print(f"  {name}: mean={comp.mean():.4f}  std={comp.std():.4f}  min={comp.min():.4f}  max={comp.max():.4f}")
        print("\nDVC COMPLETE")
        t_end = time.perf_counter()
        print("Timing")
        for k, v in [("Setup (load + mesh)", t_setup - t_start), ("Multiscale correlation", t_corr - t_setup),
                     ("Output generation", t_end - t_corr), ("Total", t_end - t_start)]:
            print(f"  {k:<24} {v:8.2f} s")
    finally:
        sys.stdout = stdout
        log_file.close()
    return 0


if __name__ == "__main__":
    sys.exit(main())
