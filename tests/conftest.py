"""pytest setup: import paths, the ``gpu`` marker, shared fixtures.

``-m "not gpu"`` runs the oracle against the golden vectors, the host-side
logic and the C ABI surface (no CUDA device needed); ``-m gpu`` runs the
parity tests of the CUDA path against the oracle.
"""
import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "fock-rs_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU and the built libfock_gb300.so")


@pytest.fixture(scope="session")
def golden_h2o():
    with open(os.path.join(GOLDEN, "h2o_sto3g_ref.json")) as f:
        return json.load(f)


@pytest.fixture(scope="session")
def golden_boys():
    with open(os.path.join(GOLDEN, "boys_mpmath.json")) as f:
        return json.load(f)


@pytest.fixture(scope="session")
def oracle_lib():
    import oracle
    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def gpu_lib():
    """The built CUDA library; builds it when missing (fails loudly on error)."""
    import fock_gb300._lib as L
    if not os.path.exists(L.LIB_PATH):
        sys.path.insert(0, os.path.join(ROOT, "fock-rs_gb300"))
        import build as B
        B.build()
    return L.lib()


def random_density(n, seed=0, nocc=None):
    """A physical-looking symmetric density 2 C_occ C_occ^T from random orbitals."""
    rng = np.random.default_rng(seed)
    nocc = nocc or max(1, n // 3)
    Cm = rng.normal(size=(n, nocc)) / np.sqrt(n)
    return 2.0 * Cm @ Cm.T
