"""pn_force_noalloc: the force evaluation for callers that cannot allocate GPU memory.

Callers such as a framework that owns all device memory through its own pool, or a
time-critical loop in which cudaMalloc/cudaFree would stall the device, pass their device
buffers for x, v, m and the result a; every work buffer of the evaluation lives in a fixed,
file-scope device array of the library (PN_NOALLOC_SCRATCH_BYTES, for at most PN_NOALLOC_NMAX
particles).  Its results must be those of the allocating device-pointer entry point
(pn_force_device) and of the oracle, call after call: the array keeps the previous call's
contents, so a sequence of calls -- the largest system first, then smaller ones with other
data, down to a BH alone -- is compared, for the Newtonian sweep (inv_c2 = 0), weak 1PN terms
(inv_c2 = 1e-6) and the reference's c = 1.  Device-side failures are read back by
pn_noalloc_status (a star exactly on the BH gives a non-finite force).

This file is collected last (test_zz_*) and is written to pass alone in a fresh process too.
"""
import ctypes

import numpy as np
import pytest

from conftest import relerr

pytestmark = pytest.mark.gpu

NMAX = 8192  # PN_NOALLOC_NMAX in include/pn.h
EPS = 0.02
# (n, seed) of consecutive calls: larger systems first, so stale contents of the shared array
# (pair sums of more stars, more j-range splits) would show in the later, smaller calls
SEQUENCE = [(NMAX, 1), (3001, 2), (65, 3), (2, 4), (1, 5)]


def _system(n, seed):
    rng = np.random.default_rng(seed)
    x = rng.uniform(-1, 1, (n, 3))
    v = rng.normal(0, 0.3, (n, 3))
    m = rng.uniform(0.5, 1.5, n) / n
    x[0] = rng.normal(0, 0.05, 3)
    v[0] = 0.0
    m[0] = 0.02
    return x, v, m


def _bind(pn):
    L = pn.lib()
    f = L.pn_force_noalloc
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_double,
                  ctypes.c_double, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
    st = L.pn_noalloc_status
    st.restype = ctypes.c_int
    st.argtypes = [ctypes.c_void_p]
    return f, st


def _oracle_force(oracle, x, v, m, ic2):
    if ic2 == 0.0:
        return oracle.force_newton(x, m, EPS)
    if ic2 == 1.0:
        return oracle.force(x, v, m, EPS)
    return None  # the oracle is the reference: c = 1 or the Newtonian sweep only


@pytest.mark.parametrize("ic2", [0.0, 1e-6, 1.0])
@pytest.mark.parametrize("prec", [0, 1])
def test_noalloc_matches_device_entry_point_and_oracle(pn, oracle, prec, ic2):
    torch = pytest.importorskip("torch")
    noalloc, status = _bind(pn)
    for call, (n, seed) in enumerate(SEQUENCE):
        x, v, m = _system(n, seed)
        dx = torch.tensor(x, device="cuda")
        dv = torch.tensor(v, device="cuda")
        dm = torch.tensor(m, device="cuda")
        a_dev = torch.zeros_like(dx)
        with pn.Context(n, eps=EPS, inv_c2=ic2, precision=prec) as c:
            c.force_device(n, ctypes.c_void_p(dx.data_ptr()), ctypes.c_void_p(dv.data_ptr()),
                           ctypes.c_void_p(dm.data_ptr()), ctypes.c_void_p(a_dev.data_ptr()))
            c.sync()
        a = torch.full_like(dx, float("nan"))
        torch.cuda.synchronize()
        rc = noalloc(n, dx.data_ptr(), dv.data_ptr(), dm.data_ptr(), EPS, ic2, prec, a.data_ptr(), None)
        assert rc == 0, f"call {call}: status {rc}"
        assert status(None) == 0, f"call {call}: device status"
        got = a.cpu().numpy()
        if n == 1:
            assert (got == 0).all()  # a BH alone feels nothing (Limit-sticky9.c:36-51)
            continue
        # against the allocating entry point: same algorithm, another launch shape (FP64: the
        # summation order differs; mixed: FP32 pair sums split differently over j)
        e = relerr(got, a_dev.cpu().numpy())
        assert np.isfinite(e).all() and e.max() <= (1e-12 if prec == 0 else 1e-5), (call, float(e.max()))
        ref = _oracle_force(oracle, x, v, m, ic2) if n <= 3001 else None
        if ref is not None:
            e = relerr(got, ref)
            if prec == 0:
                assert e.max() <= 1e-12, (call, float(e.max()))
            else:
                # FP32 pair terms: at c = 1 the Newtonian and 1PN terms cancel on some particles of
                # a uniform random cube, so the bound is on the error relative to the RMS force
                d = np.linalg.norm(got - ref, axis=1)
                rms = np.sqrt((d ** 2).mean() / (np.linalg.norm(ref, axis=1) ** 2).mean())
                assert rms <= 1e-6 and e.max() <= 1e-3, (call, float(rms), float(e.max()))


@pytest.mark.parametrize("prec", [0, 1])
def test_noalloc_status_reports_star_on_bh(pn, prec):
    """Limit-sticky9.c:74 gives 0/0 for a star exactly on the BH: the call itself succeeds on the
    host, pn_noalloc_status reports the non-finite force, and the next call clears it."""
    torch = pytest.importorskip("torch")
    noalloc, status = _bind(pn)
    x = torch.tensor([[0.0, 0, 0], [0.0, 0, 0], [0.5, 0, 0]], dtype=torch.float64, device="cuda")
    v = torch.tensor([[0.0, 0, 0], [0.1, 0, 0], [0, 0.1, 0]], dtype=torch.float64, device="cuda")
    m = torch.tensor([0.01, 1e-3, 1e-3], dtype=torch.float64, device="cuda")
    a = torch.zeros_like(x)
    torch.cuda.synchronize()
    assert noalloc(3, x.data_ptr(), v.data_ptr(), m.data_ptr(), 0.01, 1.0, prec, a.data_ptr(), None) == 0
    assert status(None) == -4  # PN_ERR_NONFINITE
    assert not torch.isfinite(a[0]).all()
    x[1, 0] = 0.25
    assert noalloc(3, x.data_ptr(), v.data_ptr(), m.data_ptr(), 0.01, 1.0, prec, a.data_ptr(), None) == 0
    assert status(None) == 0
    assert torch.isfinite(a).all()


def test_noalloc_rejects_too_many_particles(pn):
    torch = pytest.importorskip("torch")
    noalloc, _ = _bind(pn)
    buf = torch.zeros((NMAX + 1, 3), dtype=torch.float64, device="cuda")
    rc = noalloc(NMAX + 1, buf.data_ptr(), buf.data_ptr(), buf.data_ptr(), 0.01, 1.0, 0,
                 buf.data_ptr(), None)
    assert rc == -1  # PN_ERR_INVALID
