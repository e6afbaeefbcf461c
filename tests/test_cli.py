"""The ``cupymag`` command line (cupymag/cli.py:24-67, console script of setup.py:56-60)."""
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_console_script_is_declared():
    """pyproject.toml maps the `cupymag` command to cli.main, as the reference's setup.py does."""
    import tomllib
    with open(os.path.join(ROOT, "pyproject.toml"), "rb") as f:
        meta = tomllib.load(f)
    target = meta["project"]["scripts"]["cupymag"]
    assert target == "cupymag_gb300.cli:main"
    mod, fn = target.split(":")
    import importlib
    assert callable(getattr(importlib.import_module(mod), fn))
    from cupymag_gb300 import __version__
    assert meta["project"]["version"] == __version__


def test_missing_config_returns_1(tmp_path, capsys):
    from cupymag_gb300.cli import main
    assert main([str(tmp_path / "nope.yaml")]) == 1
    out = capsys.readouterr().out
    assert "Error: Configuration file" in out and "not found" in out


def test_version_needs_no_config(capsys):
    from cupymag_gb300 import __version__
    from cupymag_gb300.cli import main
    with pytest.raises(SystemExit) as e:
        main(["--version"])
    assert e.value.code == 0
    assert capsys.readouterr().out.strip() == f"CuPyMag v{__version__}"


def test_run_error_is_printed_and_returns_1(tmp_path, capsys):
    """A config that fails to load is reported the reference's way ("Error: ..." and 1)."""
    from cupymag_gb300.cli import main
    p = tmp_path / "bad.yaml"
    p.write_text("physics: {}\n")
    assert main([str(p)]) == 1
    assert capsys.readouterr().out.startswith("Error: ")


def test_module_entry_point_exits_with_main_status(tmp_path):
    r = subprocess.run([sys.executable, "-m", "cupymag_gb300.cli", str(tmp_path / "nope.yaml")], cwd=ROOT,
                       capture_output=True, text=True)
    assert r.returncode == 1
    assert "not found" in r.stdout
