"""`voxeldvc sweep-ground-truth`: the known-answer accuracy check over a grid
of (element edge h, regularisation length factor l0_factor) pairs, as the
reference's ground_truth/sweep_ground_truth.py offers it: each pair's run
in <output-root>/h<h>_l0f<l0_factor>/, then a table of the node RMS and max
error over the recoverable and the valid node sets with each solve's last
dU/U, the best pairs, and optionally a CSV.

  --gt-ref-file PATH (required), --gt-displacement-file PATH | --tensile-strain S
  --h H_LIST            comma-separated element edges (default 4,8,16)
  --l0-factor LIST      comma-separated l0 factors, l0 = l0_factor h (default 2.25,4.5,9)
  --output-root DIR     (required)
  --csv PATH            also write the table as CSV

How it runs here: the known-answer input (stage 1: reference volume,
deformed volume, true field) depends on none of the swept parameters, so it
is prepared once in <output-root>/gt_input and every pair's directory links
to it; each pair then runs preprocess -> solve -> analysis in this process
(one CUDA context), and its figures come straight from the analysis stage
rather than from re-reading the arrays it saved.  A pair that raises is
reported as FAILED and the sweep goes on; a pair whose recoverable RMS
exceeds 1 voxel is flagged DIVERGED (an under-regularised solve ends its
iterations with an implausible error instead of raising).
"""
from __future__ import annotations

import argparse
import csv
import itertools
import math
import os
import re
import sys
from dataclasses import dataclass, field

from .. import run_ground_truth_pipeline as pipeline

DEFAULT_H_SWEEP = "4,8,16"
DEFAULT_L0_FACTOR_SWEEP = "2.25,4.5,9"
DIVERGED_RMS_THRESHOLD = 1.0  # voxels

# The CSV columns and the solve-log pattern are what downstream tools read.
FIELDS = ['h', 'l0_factor', 'l0', 'n_recoverable', 'n_total', 'rms', 'max_err', 'n_valid', 'rms_valid',
          'max_err_valid', 'du_final', 'status']
DU_PATTERN = re.compile(r'dU/U=([0-9.eE+-]+)')

NAN = float('nan')


@dataclass
class PairOutcome:
    """One (h, l0_factor) run: node counts and errors over the recoverable
    and valid sets ((count, RMS, max |error|) each), the solve's last dU/U
    and 'ok' / 'FAILED'."""
    h: int
    l0_factor: float
    n_total: int = 0
    recoverable: tuple = (0, NAN, NAN)
    valid: tuple = (0, NAN, NAN)
    du_final: float = NAN
    status: str = 'ok'
    error: str = field(default='', repr=False)

    @property
    def l0(self):
        return self.l0_factor * self.h

    @property
    def diverged(self):
        return self.status == 'ok' and self.recoverable[1] > DIVERGED_RMS_THRESHOLD

    def row(self):
        """The CSV / table record (FIELDS)."""
        return dict(h=self.h, l0_factor=self.l0_factor, l0=self.l0, n_recoverable=self.recoverable[0],
                    n_total=self.n_total, rms=self.recoverable[1], max_err=self.recoverable[2],
                    n_valid=self.valid[0], rms_valid=self.valid[1], max_err_valid=self.valid[2],
                    du_final=self.du_final, status=self.status)

    @classmethod
    def from_analysis(cls, h, l0_factor, figures, du_final):
        """From analyse_ground_truth.analyse()'s figures."""
        return cls(h=h, l0_factor=l0_factor, n_total=int(figures['all'][0]),
                   recoverable=tuple(figures['recoverable']),
                   valid=tuple(figures.get('valid', (0, NAN, NAN))), du_final=du_final)


def last_du_over_u(log_text):
    """The last `dU/U=` value a solve log printed (NaN when there is none)."""
    hits = DU_PATTERN.findall(log_text)
    return float(hits[-1]) if hits else NAN


def _read_last_du(work_dir):
    try:
        with open(os.path.join(work_dir, 'run_log.txt')) as fh:
            return last_du_over_u(fh.read())
    except OSError:
        return NAN


def pair_dir(output_root, h, l0_factor):
    return os.path.join(output_root, f"h{h}_l0f{l0_factor:g}")


def run_pair(output_root, gt_dir, h, l0_factor):
    """Stages 2-4 of one pair on the shared prepared input."""
    work = pair_dir(output_root, h, l0_factor)
    os.makedirs(work, exist_ok=True)
    link = os.path.join(work, 'gt_input')
    if not os.path.lexists(link):
        os.symlink(os.path.relpath(gt_dir, work), link)
    print("\n" + "#" * 70)
    print(f"# SWEEP COMBO: h={h}  l0_factor={l0_factor:g}  (l0={l0_factor * h:g} vox)")
    print("#" * 70)
    figures = pipeline.solve_and_analyse(work, gt_dir, h, l0_factor)
    return PairOutcome.from_analysis(h, l0_factor, figures, _read_last_du(work))


def sweep(h_values, l0_factors, output_root, gt_ref_file, gt_displacement_file=None, tensile_strain=None):
    """Prepare the known-answer input once, then run every pair."""
    gt_dir = os.path.join(output_root, 'gt_input')
    pipeline.prepare_input(gt_dir, gt_ref_file, gt_displacement_file, tensile_strain)
    outcomes = []
    for h, lf in itertools.product(h_values, l0_factors):
        try:
            outcomes.append(run_pair(output_root, gt_dir, h, lf))
        except Exception as exc:  # reported in the table; the other pairs still run
            print(f"!! combo h={h}, l0_factor={lf:g} FAILED: {exc}", file=sys.stderr)
            outcomes.append(PairOutcome(h=h, l0_factor=lf, status='FAILED', error=str(exc)))
    return outcomes


def best(outcomes, figure):
    """The non-diverged successful pair with the smallest `figure` RMS
    ('recoverable' or 'valid'), or None."""
    pool = [o for o in outcomes if o.status == 'ok' and not o.diverged and not math.isnan(getattr(o, figure)[1])]
    return min(pool, key=lambda o: getattr(o, figure)[1]) if pool else None


def summary_lines(outcomes):
    """The summary table and the best-pair lines, as printed."""
    rule = "=" * 104
    lines = ["", rule, "SWEEP SUMMARY: node RMS displacement error vs. h, l0_factor "
             "(valid = fair measure; recoverable over-counts the boundary shell)", rule,
             f"{'h':>4} {'l0_factor':>10} {'l0(vox)':>8} {'rec.nodes':>12} {'rec RMS':>10} {'rec max':>10} "
             f"{'val.nodes':>12} {'valid RMS':>10} {'valid max':>10} {'final dU/U':>12}  status"]
    for o in outcomes:
        flag = 'DIVERGED' if o.diverged else ('' if o.status == 'ok' else o.status)
        (nr, rr, mr), (nv, rv, mv) = o.recoverable, o.valid
        lines.append(f"{o.h:>4} {o.l0_factor:>10g} {o.l0:>8g} {f'{nr}/{o.n_total}':>12} {rr:>10.5f} {mr:>10.5f} "
                     f"{f'{nv}/{o.n_total}':>12} {rv:>10.5f} {mv:>10.5f} {o.du_final:>12.2e}  {flag}")
    for figure, text in (('recoverable', "\nBest by recoverable RMS (non-diverged)"),
                         ('valid', "Best by valid RMS (non-diverged, fair measure)")):
        b = best(outcomes, figure)
        if b is not None:
            lines.append(f"{text}: h={b.h}, l0_factor={b.l0_factor:g} (l0={b.l0:g} vox) -> "
                         f"RMS={getattr(b, figure)[1]:.5f} vox")
    return lines


def write_csv(path, outcomes):
    with open(path, 'w', newline='') as fh:
        w = csv.DictWriter(fh, fieldnames=FIELDS)
        w.writeheader()
        w.writerows(o.row() for o in outcomes)
    print(f"\nSaved sweep summary CSV -> {path}")


def parse_args(argv=None):
    """The reference's options (ground_truth/sweep_ground_truth.py:73-99)."""
    p = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    p.add_argument('--gt-ref-file', type=str, required=True, dest='gt_ref_file')
    src = p.add_mutually_exclusive_group(required=True)
    src.add_argument('--gt-displacement-file', type=str, default=None, dest='gt_displacement_file')
    src.add_argument('--tensile-strain', type=float, default=None, dest='tensile_strain')
    p.add_argument('--h', type=str, default=DEFAULT_H_SWEEP, dest='h_values')
    p.add_argument('--l0-factor', type=str, default=DEFAULT_L0_FACTOR_SWEEP, dest='l0_factors')
    p.add_argument('--output-root', type=str, required=True, dest='output_root')
    p.add_argument('--csv', type=str, default=None, dest='csv_path')
    return p.parse_args(argv)


def main(argv=None):
    args = parse_args(argv)
    outcomes = sweep([int(x) for x in args.h_values.split(',')], [float(x) for x in args.l0_factors.split(',')],
                     os.path.abspath(args.output_root), args.gt_ref_file, args.gt_displacement_file,
                     args.tensile_strain)
    print("\n".join(summary_lines(outcomes)))
    if args.csv_path:
        write_csv(args.csv_path, outcomes)
    return 0


if __name__ == "__main__":
    sys.exit(main())
