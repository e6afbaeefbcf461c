"""``cupymag`` command line (drop-in for cupymag/cli.py:24-67).

    python -m cupymag_gb300.cli [config.yaml] [--version]

A missing config prints an error and returns 1; exceptions during the run are
printed and return 1, as in the reference.  Unlike the reference, ``--version``
works without a config (the config is read only after argument parsing).
"""
import argparse
import sys
from pathlib import Path

from . import __version__


def main(argv=None):
    parser = argparse.ArgumentParser(
        description="CuPyMag (GB300 kernels): GPU finite-element micromagnetics with magnetostriction")
    parser.add_argument("config_file", nargs="?", default="config.yaml",
                        help="Path to YAML configuration file (default: config.yaml)")
    parser.add_argument("--version", action="version", version=f"CuPyMag v{__version__}")
    args = parser.parse_args(argv)
    config_path = Path(args.config_file).resolve()
    if not config_path.exists():
        print(f"Error: Configuration file '{config_path}' not found.")
        print("Please create a config.yaml file or copy one from the examples/ directory.")
        return 1
    try:
        from .core.Micromagnetics import main as run_simulation
        run_simulation(config_path)
        return 0
    except KeyboardInterrupt:
        print("\nSimulation interrupted by user.")
        return 1
    except Exception as e:  # noqa: BLE001 -- the reference prints and returns 1
        print(f"Error: {e}")
        return 1


if __name__ == "__main__":
    sys.exit(main())
