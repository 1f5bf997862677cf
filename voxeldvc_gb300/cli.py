"""Command-line entry: `python -m voxeldvc_gb300.cli run WORK_DIR [--l0-factor F]`.

Mirrors the `run` subcommand of the reference's `voxeldvc` dispatcher
(src/voxeldvc/cli.py); the other reference subcommands (preprocess glue,
viewers, ground-truth tools) are not part of this package.
"""
import argparse
import importlib
import sys

_SUBCOMMANDS = {
    "run": ("voxeldvc_gb300.run_dvc", "multiscale Gauss-Newton DVC solve"),
}


def main(argv=None):
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
