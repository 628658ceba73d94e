"""Command line: ``python -m diffmpm_gb300 -f deck.toml`` runs a TOML deck
(the reference's ``mpm`` command, diffmpm/cli/mpm.py)."""
import argparse

from .mpm import MPM


def main(argv=None):
    ap = argparse.ArgumentParser(prog="diffmpm_gb300", description="Run an MPM input deck on the GPU.")
    ap.add_argument("-f", "--file", dest="filepath", required=True, help="Input TOML file")
    ap.add_argument("--honor-scheme", action="store_true",
                    help="use the deck's meta.scheme (the reference always runs USF)")
    args = ap.parse_args(argv)
    MPM(args.filepath, honor_scheme=args.honor_scheme).solve()


if __name__ == "__main__":
    main()
