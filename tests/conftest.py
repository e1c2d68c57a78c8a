"""Shared test setup: import paths, the `gpu` marker, golden fixtures, builds."""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
PKG = ROOT / "benchmark-sptrsv_gb300"
for p in (str(ROOT), str(PKG)):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = ROOT / "tests" / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def golden_names():
    return sorted(p.stem for p in GOLDEN.glob("*.npz"))


def load_golden(name):
    d = np.load(GOLDEN / f"{name}.npz")
    return {k: d[k] for k in d.files}


@pytest.fixture(scope="session")
def oracle_port():
    from oracle import oracle
    return oracle.port()


@pytest.fixture(scope="session")
def built_lib():
    """Builds (if stale) and loads libsptrsv_gb300.so."""
    import build as pkg_build  # benchmark-sptrsv_gb300/build.py
    pkg_build.build()
    from sptrsv_gb300 import _lib
    return _lib.load()


@pytest.fixture(scope="session")
def cuda(built_lib):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    torch.cuda.init()
    return torch
