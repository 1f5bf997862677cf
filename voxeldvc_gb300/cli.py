"""Command-line entry: `python -m voxeldvc_gb300.cli COMMAND ...`.

Mirrors the reference's `voxeldvc` dispatcher (src/voxeldvc/cli.py) for the
solve pipeline: preprocess, run, and the ground-truth accuracy check with
its stages.  The viewers (napari), VTK export and format converters are not
part of this package.
"""
import argparse
import importlib
import sys

_SUBCOMMANDS = {
    "preprocess": ("voxeldvc_gb300.preprocess", "affine pre-alignment + overlap crop"),
    "run": ("voxeldvc_gb300.run_dvc", "multiscale Gauss-Newton DVC solve"),
    "ground-truth": ("voxeldvc_gb300.run_ground_truth_pipeline", "4-stage known-ground-truth accuracy check"),
    "prepare-ground-truth": ("voxeldvc_gb300.ground_truth.prepare_ground_truth",
                             "generate ground-truth reference/deformed image pair"),
    "analyse-ground-truth": ("voxeldvc_gb300.ground_truth.analyse_ground_truth",
                             "compare recovered vs. ground-truth displacement"),
    "sweep-ground-truth": ("voxeldvc_gb300.ground_truth.sweep_ground_truth",
                           "sweep h/l0_factor and score RMS vs. ground truth"),
}


def main(argv=None):
    """Reference: cli.py:31-57."""
    argv = sys.argv[1:] if argv is None else argv
    parser = argparse.ArgumentParser(
        prog="voxeldvc",
        description="voxelDVC Gauss-Newton DVC on GB300.",
        formatter_class=argparse.RawDescriptionHelpFormatter,
        epilog="commands:\n" + "\n".join(f"  {n}  {d}" for n, (_, d) in sorted(_SUBCOMMANDS.items())))
    parser.add_argument("command", choices=sorted(_SUBCOMMANDS), metavar="command")
    parser.add_argument("args", nargs=argparse.REMAINDER, help=argparse.SUPPRESS)
    if not argv:
        parser.print_help()
        return 0
    ns = parser.parse_args(argv)
    module = importlib.import_module(_SUBCOMMANDS[ns.command][0])
    return module.main(ns.args)


if __name__ == "__main__":
    sys.exit(main())
