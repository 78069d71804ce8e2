"""Shared test setup: import paths, the `gpu` marker, common helpers."""
import os
import sys

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (REPO, os.path.join(REPO, "dwarf-p-ice3_gb300"), os.path.join(REPO, "oracle"),
          os.path.join(REPO, "tests")):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = os.path.join(REPO, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libice3gb.so")


def load_golden(name):
    return dict(np.load(os.path.join(GOLDEN, f"{name}.npz")))


def rel_err(a, b, floor_frac=1e-5):
    """max |a-b| / max(|b|, floor), floor = floor_frac * RMS(b) (per field).

    With floor_frac = 1e-5 a value produced by cancellation (|b| far below the
    field scale) is held to an absolute error of TOL * 1e-5 * RMS(b).

    Non-finite values must sit at the same places with the same value (the
    reference itself produces NaN on some degenerate inputs); inf is returned
    when they do not."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    fa, fb = np.isfinite(a), np.isfinite(b)
    if not np.array_equal(fa, fb):
        return float("inf")
    if not np.array_equal(np.nan_to_num(a[~fa], nan=0.5), np.nan_to_num(b[~fb], nan=0.5)):
        return float("inf")
    a, b = a[fa], b[fb]
    rms = float(np.sqrt(np.mean(b * b))) if b.size else 0.0
    floor = max(floor_frac * rms, 1e-300)
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), floor))) if b.size else 0.0


from parity import assert_parity, sensitivity  # noqa: E402,F401
