"""Shared pytest configuration: markers, import paths, golden-fixture loading."""

import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
GOLDEN = Path(__file__).resolve().parent / "golden"
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a) and the built extension")


def load_fixture(name):
    """Load ``tests/golden/<name>.npz`` as a plain dict of arrays."""
    with np.load(GOLDEN / f"{name}.npz") as z:
        return {k: z[k] for k in z.files}


def fixture_names(prefix):
    return sorted(p.stem for p in GOLDEN.glob(f"{prefix}*.npz"))


def rel_err(a, b):
    """Relative Frobenius error, the metric of the reference's GPU-vs-CPU test
    (tests/regression/test_engine_regression.py:140-149)."""
    b = np.asarray(b)
    d = np.linalg.norm((np.asarray(a) - b).ravel())
    return float(d / max(np.linalg.norm(b.ravel()), 1e-30))


@pytest.fixture
def fixture_loader():
    return load_fixture


def platform_reproduces_order(fx):
    """True when this platform's np.argsort yields the position orders the
    reference recorded (only 'NA' order can differ: it sorts LED distances with
    ties, and NumPy's unstable default sort breaks ties differently on x86 and Arm)."""
    if str(fx.get("meta_order", "")) != "NA" or "in_orders" not in fx:
        return True
    pos = fx["in_positions"]
    rows = pos[:, 0] - np.mean(pos[:, 0])
    cols = pos[:, 1] - np.mean(pos[:, 1])
    here = np.argsort(np.sqrt(rows**2 + cols**2))
    return all(np.array_equal(here, o) for o in fx["in_orders"])
