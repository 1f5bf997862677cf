"""`voxeldvc ground-truth` (run_ground_truth_pipeline.py of the reference):
the known-answer accuracy check end to end through the same stages a real
run uses:

  1. ground_truth.prepare_ground_truth   reference / deformed pair
  2. preprocess                          affine prealign + overlap crop
  3. run_dvc                             multiscale DVC
  4. ground_truth.analyse_ground_truth   recovered vs. known displacement

  --output-dir DIR   stage 1 writes DIR/gt_input, stages 2-4 write DIR
  --gt-ref-file, --gt-displacement-file | --tensile-strain   to stage 1
  --h H              to stage 2 (default 8)
  --l0-factor F      to stage 3 (default 4.5)
  --subprocess       run each stage as `python -m` (as the reference does)
                     instead of in this process (one CUDA context)

In process, `prepare_input` (stage 1) and `solve_and_analyse` (stages 2-4)
are also callable on their own; the latter returns the analysis figures, so
a caller running many configurations on one prepared input (the sweep)
reads them without going back to the saved arrays.
"""
from __future__ import annotations

import argparse
import os
import subprocess
import sys

DEFAULT_H = 8
DEFAULT_L0_FACTOR = 4.5

_STAGES = {
    'prepare': 'voxeldvc_gb300.ground_truth.prepare_ground_truth',
    'preprocess': 'voxeldvc_gb300.preprocess',
    'run': 'voxeldvc_gb300.run_dvc',
    'analyse': 'voxeldvc_gb300.ground_truth.analyse_ground_truth',
}


def _banner(module, args):
    print("\n" + "=" * 70)
    print("STAGE: " + " ".join([sys.executable, '-m', module] + list(args)))
    print("=" * 70)


def run_stage(module, args, in_process=True):
    """One stage as `python -m module args` or its main() in this process.
    Reference: run_ground_truth_pipeline.py:51-56."""
    _banner(module, args)
    if not in_process:
        subprocess.run([sys.executable, '-m', module] + list(args), check=True)
        return
    import importlib
    rc = importlib.import_module(module).main(list(args))
    if rc not in (None, 0):
        raise RuntimeError(f"stage {module} exited with {rc}")


def prepare_input(gt_dir, gt_ref_file=None, gt_displacement_file=None, tensile_strain=None, in_process=True):
    """Stage 1 into gt_dir (ref.npy, deformed.npy, U.npy, ...)."""
    args = ['--output-dir', gt_dir]
    if gt_ref_file is not None:
        args += ['--gt-ref-file', gt_ref_file]
    if gt_displacement_file is not None:
        args += ['--gt-displacement-file', gt_displacement_file]
    if tensile_strain is not None:
        args += ['--tensile-strain', str(tensile_strain)]
    run_stage(_STAGES['prepare'], args, in_process)


def solve_and_analyse(work_dir, gt_dir, h=DEFAULT_H, l0_factor=DEFAULT_L0_FACTOR, in_process=True):
    """Stages 2-4 on a prepared input; returns the analysis figures
    ({'recoverable': (n, rms, max), 'valid': ..., 'truncated': ..., 'all':
    ...}) in process, None with in_process=False."""
    run_stage(_STAGES['preprocess'], [os.path.join(gt_dir, 'ref.npy'), os.path.join(gt_dir, 'deformed.npy'),
                                      '--h', str(h), '--output-dir', work_dir], in_process)
    run_stage(_STAGES['run'], [work_dir, '--l0-factor', str(l0_factor)], in_process)
    if not in_process:
        run_stage(_STAGES['analyse'], ['--work-dir', work_dir, '--gt-dir', gt_dir], False)
        return None
    from .ground_truth import analyse_ground_truth as AG
    _banner(_STAGES['analyse'], ['--work-dir', work_dir, '--gt-dir', gt_dir])
    return AG.analyse_logged(work_dir, gt_dir)


def parse_args(argv=None):
    """Reference: run_ground_truth_pipeline.py:59-84."""
    p = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    p.add_argument('--gt-ref-file', type=str, default=None, dest='gt_ref_file')
    g = p.add_mutually_exclusive_group()
    g.add_argument('--gt-displacement-file', type=str, default=None, dest='gt_displacement_file')
    g.add_argument('--tensile-strain', type=float, default=None, dest='tensile_strain')
    p.add_argument('--h', type=int, default=DEFAULT_H, dest='h')
    p.add_argument('--l0-factor', type=float, default=DEFAULT_L0_FACTOR, dest='l0_factor')
    p.add_argument('--output-dir', type=str, required=True, dest='output_dir')
    p.add_argument('--subprocess', action='store_true', dest='subprocess')
    return p.parse_args(argv)


def main(argv=None):
    """Reference: run_ground_truth_pipeline.py:87-126."""
    args = parse_args(argv)
    out = os.path.abspath(args.output_dir)
    gt = os.path.join(out, 'gt_input')
    inproc = not args.subprocess
    prepare_input(gt, args.gt_ref_file, args.gt_displacement_file, args.tensile_strain, inproc)
    solve_and_analyse(out, gt, args.h, args.l0_factor, inproc)
    print("\n" + "=" * 70)
    print("✓ GROUND-TRUTH PIPELINE COMPLETE")
    print("=" * 70)
    print(f"  gt_input : {gt}")
    print(f"  work_dir : {out}")
    print(f"  logs     : {os.path.join(out, 'run_log.txt')}, {os.path.join(out, 'ground_truth_comparison_log.txt')}")
    return 0


if __name__ == "__main__":
    sys.exit(main())
