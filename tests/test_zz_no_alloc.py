"""pn_force_noalloc: the force evaluation for callers that cannot allocate GPU memory.

Callers such as a framework that owns all device memory through its own pool, or a
time-critical loop in which cudaMalloc/cudaFree would stall the device, pass their device
buffers for x, v, m and the result a; every work buffer of the evaluation lives in a fixed,
file-scope device array of the library (PN_NOALLOC_SCRATCH_BYTES, for at most PN_NOALLOC_NMAX
particles).  Its results must be those of the allocating device-pointer entry point
(pn_force_device), call after call: the array keeps the previous call's contents, so two calls
in a row -- a larger system, then a smaller one with other data -- are compared.

This file is collected last (test_zz_*) and is written to pass alone in a fresh process too.
"""
import ctypes

import numpy as np
import pytest

from conftest import relerr

pytestmark = pytest.mark.gpu

NMAX = 8192  # PN_NOALLOC_NMAX in include/pn.h


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
    return f


@pytest.mark.parametrize("prec", [0, 1])
def test_noalloc_matches_device_entry_point_twice(pn, prec):
    torch = pytest.importorskip("torch")
    noalloc = _bind(pn)
    eps = 0.02
    tol = 1e-12 if prec == 0 else 1e-5
    for call, (n, seed) in enumerate([(NMAX, 1), (3001, 2)]):
        x, v, m = _system(n, seed)
        dx = torch.tensor(x, device="cuda")
        dv = torch.tensor(v, device="cuda")
        dm = torch.tensor(m, device="cuda")
        a_ref = torch.zeros_like(dx)
        with pn.Context(n, eps=eps, precision=prec) as c:
            c.force_device(n, ctypes.c_void_p(dx.data_ptr()), ctypes.c_void_p(dv.data_ptr()),
                           ctypes.c_void_p(dm.data_ptr()), ctypes.c_void_p(a_ref.data_ptr()))
            c.sync()
        a = torch.full_like(dx, float("nan"))
        torch.cuda.synchronize()
        rc = noalloc(n, dx.data_ptr(), dv.data_ptr(), dm.data_ptr(), eps, 1.0, prec, a.data_ptr(), None)
        assert rc == 0, f"call {call}: status {rc}"
        torch.cuda.synchronize()
        e = relerr(a.cpu().numpy(), a_ref.cpu().numpy())
        assert np.isfinite(e).all() and e.max() <= tol, (call, float(e.max()))


def test_noalloc_rejects_too_many_particles(pn):
    torch = pytest.importorskip("torch")
    noalloc = _bind(pn)
    buf = torch.zeros((NMAX + 1, 3), dtype=torch.float64, device="cuda")
    rc = noalloc(NMAX + 1, buf.data_ptr(), buf.data_ptr(), buf.data_ptr(), 0.01, 1.0, 0,
                 buf.data_ptr(), None)
    assert rc == -1  # PN_ERR_INVALID
