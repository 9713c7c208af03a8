"""Shared test setup: import paths, the `gpu` marker, helpers."""
import os
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
for p in (ROOT, ROOT / "trixicuda.jl_gb300"):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libtrixi_b200.so")


def rel_err(a, b):
    """Relative error in the 2-norm, the definition of Julia's isapprox that
    the reference's @test_approx uses (test/test_macros.jl:39)."""
    a = np.asarray(a, dtype=np.float64).reshape(-1)
    b = np.asarray(b, dtype=np.float64).reshape(-1)
    scale = max(np.linalg.norm(a), np.linalg.norm(b), 1e-300)
    return float(np.linalg.norm(a - b) / scale)


def rel_err_max(a, b):
    """Pointwise error scaled by the largest value (a stricter, max-norm view)."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def assert_rel(a, b, rtol, what="", max_factor=10.0):
    """2-norm relative error <= rtol, and max-norm relative error <= max_factor*rtol."""
    e = rel_err(a, b)
    assert e <= rtol, f"{what}: relative 2-norm error {e:.3e} > {rtol:.1e}"
    em = rel_err_max(a, b)
    assert em <= max_factor * rtol, f"{what}: relative max-norm error {em:.3e} > {max_factor * rtol:.1e}"


@pytest.fixture(scope="session")
def cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from trixicuda import _lib

    _lib.load(build_if_missing=True)
    return torch
