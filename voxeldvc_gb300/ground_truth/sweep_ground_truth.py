"""`voxeldvc sweep-ground-truth` (ground_truth/sweep_ground_truth.py of the
reference): the known-answer pipeline once per (h, l0_factor) pair, each in
<output-root>/h<h>_l0f<l0_factor>/, and a table of the node RMS error over
the recoverable and the valid node sets (read back from the U_error.npy and
node masks the analysis stage saves) with the last dU/U of the solve log.

  --gt-ref-file PATH (required), --gt-displacement-file PATH | --tensile-strain S
  --h H_LIST            comma-separated element edges (default 4,8,16)
  --l0-factor LIST      comma-separated l0 factors, l0 = l0_factor h (default 2.25,4.5,9)
  --output-root DIR     (required)
  --csv PATH            also write the table as CSV

A pair whose recoverable RMS exceeds 1 voxel is marked DIVERGED (an
under-regularised solve finishes its iterations with an implausible error
rather than raising).
"""
from __future__ import annotations

import argparse
import csv
import os
import re
import sys

import numpy as np

from .. import run_ground_truth_pipeline

DEFAULT_H_SWEEP = "4,8,16"
DEFAULT_L0_FACTOR_SWEEP = "2.25,4.5,9"
DIVERGED_RMS_THRESHOLD = 1.0  # voxels

_DU_RE = re.compile(r'dU/U=([0-9.eE+-]+)')
FIELDS = ['h', 'l0_factor', 'l0', 'n_recoverable', 'n_total', 'rms', 'max_err', 'n_valid', 'rms_valid',
          'max_err_valid', 'du_final', 'status']


def parse_args(argv=None):
    """Reference: ground_truth/sweep_ground_truth.py:73-99."""
    p = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    p.add_argument('--gt-ref-file', type=str, required=True, dest='gt_ref_file')
    g = p.add_mutually_exclusive_group(required=True)
    g.add_argument('--gt-displacement-file', type=str, default=None, dest='gt_displacement_file')
    g.add_argument('--tensile-strain', type=float, default=None, dest='tensile_strain')
    p.add_argument('--h', type=str, default=DEFAULT_H_SWEEP, dest='h_values')
    p.add_argument('--l0-factor', type=str, default=DEFAULT_L0_FACTOR_SWEEP, dest='l0_factors')
    p.add_argument('--output-root', type=str, required=True, dest='output_root')
    p.add_argument('--csv', type=str, default=None, dest='csv_path')
    return p.parse_args(argv)


def parse_final_du_over_u(run_log_path):
    """The last `dU/U=` value of a solve log (NaN when absent).
    Reference: ground_truth/sweep_ground_truth.py:102-113."""
    try:
        with open(run_log_path) as fh:
            found = _DU_RE.findall(fh.read())
    except OSError:
        return float('nan')
    return float(found[-1]) if found else float('nan')


def _rms_max(error, mask):
    sel = error[mask]
    if sel.size == 0:
        return float('nan'), float('nan')
    return float(np.sqrt(np.mean(sel ** 2))), float(np.max(np.linalg.norm(sel, axis=-1)))


def summarize_combo(work_dir):
    """RMS / max error over the recoverable and valid node sets of one run.
    Reference: ground_truth/sweep_ground_truth.py:126-158."""
    error = np.load(os.path.join(work_dir, 'U_error.npy'))
    truncated = np.load(os.path.join(work_dir, 'node_truncated_mask.npy'))
    rec = ~truncated
    rms, mx = _rms_max(error, rec)
    vpath = os.path.join(work_dir, 'node_valid_mask.npy')
    if os.path.exists(vpath):
        valid = np.load(vpath)
        n_valid = int(valid.sum())
        rms_v, mx_v = _rms_max(error, valid)
    else:
        n_valid, rms_v, mx_v = 0, float('nan'), float('nan')
    return dict(n_recoverable=int(rec.sum()), n_total=int(truncated.size), rms=rms, max_err=mx, n_valid=n_valid,
                rms_valid=rms_v, max_err_valid=mx_v,
                du_final=parse_final_du_over_u(os.path.join(work_dir, 'run_log.txt')), status='ok')


def run_sweep(h_values, l0_factors, gt_ref_file, gt_displacement_file, tensile_strain, output_root):
    """Reference: ground_truth/sweep_ground_truth.py:161-188."""
    results = []
    for h in h_values:
        for lf in l0_factors:
            combo = os.path.join(output_root, f"h{h}_l0f{lf:g}")
            args = ['--h', str(h), '--l0-factor', str(lf), '--output-dir', combo, '--gt-ref-file', gt_ref_file]
            if gt_displacement_file is not None:
                args += ['--gt-displacement-file', gt_displacement_file]
            if tensile_strain is not None:
                args += ['--tensile-strain', str(tensile_strain)]
            print("\n" + "#" * 70)
            print(f"# SWEEP COMBO: h={h}  l0_factor={lf:g}  (l0={lf * h:g} vox)")
            print("#" * 70)
            try:
                run_ground_truth_pipeline.main(args)
                stats = summarize_combo(combo)
            except Exception as exc:  # a failed pair is reported, the sweep goes on
                print(f"!! combo h={h}, l0_factor={lf:g} FAILED: {exc}", file=sys.stderr)
                stats = dict(n_recoverable=0, n_total=0, rms=float('nan'), max_err=float('nan'), n_valid=0,
                             rms_valid=float('nan'), max_err_valid=float('nan'), du_final=float('nan'),
                             status='FAILED')
            results.append(dict(h=h, l0_factor=lf, l0=lf * h, **stats))
    return results


def _best(results, key):
    ok = [r for r in results if r['status'] == 'ok' and not r['rms'] > DIVERGED_RMS_THRESHOLD
          and not np.isnan(r[key])]
    return min(ok, key=lambda r: r[key]) if ok else None


def print_summary_table(results):
    """Reference: ground_truth/sweep_ground_truth.py:204-236."""
    print("\n" + "=" * 104)
    print("SWEEP SUMMARY: node RMS displacement error vs. h, l0_factor "
          "(valid = fair measure; recoverable over-counts the boundary shell)")
    print("=" * 104)
    print(f"{'h':>4} {'l0_factor':>10} {'l0(vox)':>8} {'rec.nodes':>12} {'rec RMS':>10} {'rec max':>10} "
          f"{'val.nodes':>12} {'valid RMS':>10} {'valid max':>10} {'final dU/U':>12}  status")
    for r in results:
        flag = r['status'] if r['status'] != 'ok' else ('DIVERGED' if r['rms'] > DIVERGED_RMS_THRESHOLD else '')
        print(f"{r['h']:>4} {r['l0_factor']:>10g} {r['l0']:>8g} {str(r['n_recoverable']) + '/' + str(r['n_total']):>12} "
              f"{r['rms']:>10.5f} {r['max_err']:>10.5f} {str(r['n_valid']) + '/' + str(r['n_total']):>12} "
              f"{r['rms_valid']:>10.5f} {r['max_err_valid']:>10.5f} {r['du_final']:>12.2e}  {flag}")
    b = _best(results, 'rms')
    if b is not None:
        print(f"\nBest by recoverable RMS (non-diverged): h={b['h']}, l0_factor={b['l0_factor']:g} "
              f"(l0={b['l0']:g} vox) -> RMS={b['rms']:.5f} vox")
    b = _best(results, 'rms_valid')
    if b is not None:
        print(f"Best by valid RMS (non-diverged, fair measure): h={b['h']}, l0_factor={b['l0_factor']:g} "
              f"(l0={b['l0']:g} vox) -> RMS={b['rms_valid']:.5f} vox")


def write_csv(path, results):
    """Reference: ground_truth/sweep_ground_truth.py:239-248."""
    with open(path, 'w', newline='') as fh:
        w = csv.DictWriter(fh, fieldnames=FIELDS)
        w.writeheader()
        for r in results:
            w.writerow({k: r[k] for k in FIELDS})
    print(f"\nSaved sweep summary CSV -> {path}")


def main(argv=None):
    """Reference: ground_truth/sweep_ground_truth.py:251-262."""
    args = parse_args(argv)
    results = run_sweep([int(x) for x in args.h_values.split(',')], [float(x) for x in args.l0_factors.split(',')],
                        args.gt_ref_file, args.gt_displacement_file, args.tensile_strain,
                        os.path.abspath(args.output_root))
    print_summary_table(results)
    if args.csv_path:
        write_csv(args.csv_path, results)
    return 0


if __name__ == "__main__":
    sys.exit(main())
