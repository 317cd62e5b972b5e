"""Test configuration: the ``gpu`` marker and a session-wide build of libpn and the oracle.

``-m "not gpu"`` runs here without a GPU: the oracle against the reference's golden vectors,
the host logic, and that libpn loads and exports its C ABI.  ``-m gpu`` runs the parity tests
of the CUDA path through the C ABI on a GB300.
"""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session", autouse=True)
def built():
    from pn_gb300 import build as b
    from oracle import pyoracle as po
    b.build()
    po.build(ref=True)
    yield


@pytest.fixture(scope="session")
def pn():
    import pn_gb300
    return pn_gb300


@pytest.fixture(scope="session")
def oracle():
    from oracle import pyoracle as po
    return po


def golden(name):
    import numpy as np
    path = os.path.join(GOLDEN, name)
    if not os.path.exists(path):
        pytest.skip(f"golden file {name} not generated")
    return np.load(path)


def relerr(a, b):
    """Per-particle normwise relative error |a_i - b_i| / |b_i|."""
    import numpy as np
    return np.linalg.norm(a - b, axis=1) / np.maximum(np.linalg.norm(b, axis=1), 1e-300)


def assert_matches_reference(a, a_ref, a_exact, tol=1e-12):
    """FP64 parity with the reference, particle by particle.

    Every particle must be within tol (normwise relative) of the exact value of the
    reference's formulas (a_exact: the same algorithm in long double).  Against the reference
    itself every particle must be within tol too, except where the reference's own double
    rounding is larger than tol (|a_ref - a_exact| > tol |a_exact|); there the difference must
    stay within that rounding error plus tol."""
    import numpy as np
    e_exact = relerr(a, a_exact)
    assert e_exact.max() <= tol, ("vs exact", int(e_exact.argmax()), float(e_exact.max()))
    e_ref = relerr(a, a_ref)
    own = relerr(a_ref, a_exact)
    bad = e_ref > tol
    assert (own[bad] > tol).all(), ("vs reference where it is accurate",
                                    np.nonzero(bad & (own <= tol))[0][:5])
    na = np.linalg.norm(a_exact, axis=1)
    lim = np.linalg.norm(a_ref - a_exact, axis=1) + tol * na
    assert (np.linalg.norm(a - a_ref, axis=1) <= lim).all()
