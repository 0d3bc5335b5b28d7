"""Shared pytest setup: import paths, the ``gpu`` marker and golden-fixture helpers."""

from __future__ import annotations

import sys
from pathlib import Path

import numpy as np
import pytest
import scipy.sparse as sp

ROOT = Path(__file__).resolve().parents[1]
PKG = ROOT / "xkep-cae_gb300"
GOLDEN = ROOT / "tests" / "golden"
for p in (str(ROOT), str(PKG)):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a) and the built extension")


def golden(name: str):
    return np.load(GOLDEN / f"{name}.npz")


def golden_csr(z, prefix: str, n: int) -> sp.csr_matrix:
    return sp.csr_matrix((z[prefix + "_data"], z[prefix + "_indices"], z[prefix + "_indptr"]), shape=(n, n))


def rel_err(a, b) -> float:
    """Max-norm relative error ``max|a-b| / max|b|`` (0 for two empty arrays)."""
    a = np.asarray(a, dtype=float)
    b = np.asarray(b, dtype=float)
    if b.size == 0:
        return 0.0 if a.size == 0 else float("inf")
    m = float(np.max(np.abs(b)))
    d = float(np.max(np.abs(a - b)))
    return d / m if m > 0 else d


def sparse_rel_err(A, B) -> float:
    m = abs(B).max() if B.nnz else 0.0
    d = abs(A - B).max() if (A - B).nnz else 0.0
    return float(d / m) if m > 0 else float(d)


@pytest.fixture
def gold():
    return golden
