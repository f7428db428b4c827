"""Shared helpers of the test suite.

Tests marked ``gpu`` need a CUDA GPU and call the product only through its
C ABI (libnufi_gb300.so); the others run on the CPU and cover the oracle
against the reference's golden vectors, the host logic and the C ABI's
exported surface.
"""
import json
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
GOLDEN = ROOT / "tests" / "golden"
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

from numericalflowiteration_gb300.config import Config  # noqa: E402


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a kernels)")


def golden(name: str):
    """(config, dict of arrays) of one golden case produced by the reference."""
    z = np.load(GOLDEN / f"{name}.npz")
    cfg = Config.from_bytes(z["config"].tobytes())
    return cfg, {k: z[k] for k in z.files if k != "config"}


def golden_manifest():
    return json.loads((GOLDEN / "manifest.json").read_text())


def rel_max(a, b):
    """max |a - b| / max |b| — the relative error measure of these tests."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    den = np.max(np.abs(b))
    return float(np.max(np.abs(a - b)) / (den if den > 0 else 1.0))


def energy_tol(g) -> float:
    """Tolerance on max |dW| / max |W| against a run case's golden energy
    history: 1e-12, or 3x the case's FP64 summation floor where that is
    larger.  The floor is the gap between the reference's loop summing rho
    in q order and the same loop summing compensated (make_golden.py); with
    alpha = 1e-3 the field comes from a 1e-3 perturbation of rho ~ -1, and
    the O(sqrt(Nm) eps) rounding of the O(1) sum is ~1e-12 of the energy.
    The reference's own GPU kernel (atomics in arbitrary order) is not
    reproducible below that floor either."""
    return max(1e-12, 3.0 * float(g["summation_floor"]))


@pytest.fixture(scope="session")
def oracle_mod():
    from oracle import oracle
    oracle.build()
    return oracle
