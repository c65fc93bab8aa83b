"""Shared pytest configuration: markers, golden-fixture loading, tolerances."""

from __future__ import annotations

import sys
from pathlib import Path

import numpy as np
import pytest

REPO = Path(__file__).resolve().parents[1]
if str(REPO) not in sys.path:
    sys.path.insert(0, str(REPO))

GOLDEN = Path(__file__).resolve().parent / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a) and the built extension")


def load_golden(group: str, precision: str) -> dict:
    with np.load(GOLDEN / f"golden_{group}_{precision}.npz") as z:
        return {k: z[k] for k in z.files}


def real_t_of(precision: str):
    return {"single": np.float32, "double": np.float64}[precision]


def ref_tol(precision: str) -> float:
    """The reference tests' absolute tolerance: 1e3 machine epsilons."""
    real_t = real_t_of(precision)
    return float(real_t(1e3) * np.finfo(real_t).eps)


def rel_l2(a, b) -> float:
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    den = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (den if den > 0 else 1.0))


@pytest.fixture(params=["single", "double"])
def precision(request):
    return request.param
