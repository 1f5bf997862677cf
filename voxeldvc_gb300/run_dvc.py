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
  ref_forward_pushed.npy  (Nvx, Nvy, Nvz) reference pushed onto the deformed grid
  run_log.txt          the run's printed output

The derived post-processing fields of the reference's write_outputs (strain,
quality and mask fields, VTK files) are a later stage and not written here.
"""
from __future__ import annotations

import argparse
import json
import os
import sys
import time

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


def main(argv=None):
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
        # post-solve voxel stages (engine/write_output.py): the reference
        # pushed onto the deformed grid, and the correlation quality over
        # the active voxels (f and the warped g = f - res)
        from .engine.write_output import push_reference_forward, compute_zncc
        from .engine.correlate_gpu import compute_active_mask
        np.save(os.path.join(work, 'ref_forward_pushed.npy'),
                push_reference_forward(ref, U, Nx, Ny, Nz, h))
        active = compute_active_mask(U, deformed, Nx, Ny, Nz, h, np, glt=glt)
        f_flat = np.ravel(np.asarray(ref, dtype=np.float64), order='F')
        zncc = compute_zncc(f_flat, f_flat - res, active)
        print(f"  ZNCC (active voxels): {zncc:.6f}")
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
