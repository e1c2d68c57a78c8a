"""The reference's call site as plain C against the library (examples/drop_in.c)."""
from __future__ import annotations

import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
SRC = ROOT / "benchmark-sptrsv_gb300" / "examples" / "drop_in.c"
LIBDIR = ROOT / "benchmark-sptrsv_gb300" / "_build"


def _compile(tmp_path) -> Path:
    cc = shutil.which("cc") or shutil.which("gcc")
    if cc is None:
        pytest.skip("no C compiler")
    if not (LIBDIR / "libsptrsv_gb300.so").exists():
        pytest.skip("library not built")
    exe = tmp_path / "drop_in"
    subprocess.run([cc, "-std=c11", "-O2", "-Wall", "-Werror", str(SRC), f"-I{ROOT / 'include'}", f"-L{LIBDIR}",
                    "-lsptrsv_gb300", f"-Wl,-rpath,{LIBDIR}", "-o", str(exe)], check=True, capture_output=True,
                   text=True)
    return exe


def test_drop_in_compiles_against_the_header(tmp_path):
    assert _compile(tmp_path).exists()


@pytest.mark.gpu
def test_drop_in_runs(tmp_path, cuda):
    exe = _compile(tmp_path)
    res = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert res.returncode == 0, res.stdout + res.stderr
    assert "drop-in ok" in res.stdout
    assert res.stdout.count("status 0") == 2
