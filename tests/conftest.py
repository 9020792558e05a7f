"""Shared pytest setup: the `gpu` marker, import paths and small helpers."""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

GOLDEN = ROOT / "tests" / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a); runs the engine's kernels")


@pytest.fixture(scope="session")
def golden():
    def load(name: str):
        return np.load(GOLDEN / f"{name}.npz")
    return load


def fp_tol(a: np.ndarray) -> float:
    """The per-step FP32 tolerance: 1e-5 of the field's range (at least 1e-5 absolute)."""
    r = float(np.max(a) - np.min(a)) if a.size else 0.0
    return max(1e-5 * r, 1e-5)
