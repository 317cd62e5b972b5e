"""ctypes bindings for the CPU oracle -- TEST INFRASTRUCTURE ONLY.

Two libraries live under ``oracle/``:

* ``_build/libpn_oracle.so`` -- the C restatement (``pn_oracle.c``) of the reference's
  force path (Limit-sticky9.c:21-424 force, :427-714 energies, :841-893 integrator step).
  It is built on every machine by ``oracle/Makefile``.
* ``_ref/libls9ref.so`` -- the unmodified reference functions compiled from their own
  source (``make ref``).  It only exists where the reference source is present; tests that
  need it skip elsewhere.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg import this
module.  The product library never does.

:func:`plummer_bh` samples the Plummer + BH workload with numpy alone (same construction as
libpn's generator, its own random stream), so that the CPU arm of the benchmark builds its input
without loading the GPU library.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "_build", "libpn_oracle.so")
ORACLE_LD_SO = os.path.join(HERE, "_build", "libpn_oracle_ld.so")
REF_SO = os.path.join(HERE, "_ref", "libls9ref.so")

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)


def _ptr(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(_dp)


def build(ref: bool = True) -> None:
    """Build the oracle (and the reference harness when its source exists)."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    if ref and reference_source_present():
        subprocess.run(["make", "-s", "-C", HERE, "ref"], check=True)


def reference_dir() -> str:
    """The reference source tree: $LS9_DIR, else the Makefile's default (``make ls9-dir``)."""
    d = os.environ.get("LS9_DIR")
    if d:
        return d
    r = subprocess.run(["make", "-s", "-C", HERE, "ls9-dir"], capture_output=True, text=True)
    return r.stdout.strip() if r.returncode == 0 else ""


def reference_source_present() -> bool:
    d = reference_dir()
    return bool(d) and os.path.exists(os.path.join(d, "Limit-sticky9.c"))


_lib = None
_ref = None
_ld = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(ORACLE_SO):
            build(ref=False)
        L = ctypes.CDLL(ORACLE_SO)
        L.orc_force.argtypes = [ctypes.c_int, _dp, _dp, _dp, ctypes.c_double, _dp]
        L.orc_force.restype = None
        L.orc_force_newton.argtypes = [ctypes.c_int, _dp, _dp, ctypes.c_double, _dp]
        L.orc_force_newton.restype = None
        L.orc_energy.argtypes = [ctypes.c_int, _dp, _dp, _dp, ctypes.c_double, _dp]
        L.orc_energy.restype = ctypes.c_double
        L.orc_run.argtypes = [ctypes.c_int, _dp, _dp, _dp, ctypes.c_double, ctypes.c_double,
                              ctypes.c_int]
        L.orc_run.restype = ctypes.c_int
        L.orc_force_rows.argtypes = [ctypes.c_int, _dp, _dp, _dp, ctypes.c_double, _ip,
                                     ctypes.c_int, _dp, _dp]
        L.orc_force_rows.restype = ctypes.c_int
        _lib = L
    return _lib


def lib_ld():
    """The long-double build of the restatement (exact reference for rounding checks)."""
    global _ld
    if _ld is None:
        if not os.path.exists(ORACLE_LD_SO):
            build(ref=False)
        L = ctypes.CDLL(ORACLE_LD_SO)
        L.orcld_force_d.argtypes = [ctypes.c_int, _dp, _dp, _dp, ctypes.c_double, _dp]
        L.orcld_force_d.restype = None
        L.orcld_energy_d.argtypes = [ctypes.c_int, _dp, _dp, _dp, ctypes.c_double, _dp]
        L.orcld_energy_d.restype = ctypes.c_double
        _ld = L
    return _ld


def force_exact(x, v, m, eps):
    """force() evaluated in long double, rounded to double at the end."""
    x, v, m = _state(x, v, m)
    a = np.zeros_like(x)
    lib_ld().orcld_force_d(x.shape[0], _ptr(x), _ptr(v), _ptr(m), float(eps), _ptr(a))
    return a


def energy_exact(x, v, m, eps):
    x, v, m = _state(x, v, m)
    out = np.zeros(4)
    lib_ld().orcld_energy_d(x.shape[0], _ptr(x), _ptr(v), _ptr(m), float(eps), _ptr(out))
    return out


def ref_available() -> bool:
    return os.path.exists(REF_SO)


def ref():
    """The unmodified reference functions (only where built)."""
    global _ref
    if _ref is None:
        if not os.path.exists(REF_SO):
            raise FileNotFoundError(REF_SO)
        L = ctypes.CDLL(REF_SO)
        L.ls9_force.argtypes = [_dp, _dp, _dp, ctypes.c_double, _dp, ctypes.c_int]
        L.ls9_force.restype = None
        L.ls9_initial_energy.argtypes = [_dp, _dp, _dp, ctypes.c_int, _dp, ctypes.c_double]
        L.ls9_initial_energy.restype = None
        L.ls9_rk_step.argtypes = [_dp, _dp, _dp, ctypes.c_double, ctypes.c_double, ctypes.c_int,
                                  _dp]
        L.ls9_rk_step.restype = None
        _ref = L
    return _ref


def _big_stack(fn, *args):
    """Run fn on a thread with a 512 MiB stack: the reference keeps NMAX-sized arrays
    (6.5 MB in force(), 4.3 MB in the energy functions) on the stack."""
    out = {}
    old = threading.stack_size()
    threading.stack_size(512 << 20)
    try:
        def run():
            try:
                out["r"] = fn(*args)
            except BaseException as e:  # pragma: no cover - surfaced below
                out["e"] = e
        t = threading.Thread(target=run)
        t.start()
        t.join()
    finally:
        threading.stack_size(old)
    if "e" in out:
        raise out["e"]
    return out.get("r")


def _state(x, v, m):
    x = np.ascontiguousarray(x, dtype=np.float64).reshape(-1, 3)
    v = np.ascontiguousarray(v, dtype=np.float64).reshape(-1, 3)
    m = np.ascontiguousarray(m, dtype=np.float64).reshape(-1)
    assert x.shape == v.shape and x.shape[0] == m.shape[0]
    return x, v, m


def plummer_bh(nstars, seed=1, bh_fraction=0.01):
    """A Plummer sphere of nstars equal-mass stars in Henon units (M = 1, E = -1/4) by the
    Aarseth-Henon-Wielen (1974) method -- radius from the cumulative mass with the outer 0.1 %
    cut, speed ratio q from g(q) = q^2 (1 - q^2)^(7/2) by rejection, isotropic directions,
    centre-of-mass frame -- plus a BH of bh_fraction x the stellar mass at the origin at rest
    (row 0).  numpy's generator, vectorised: the same distribution as libpn's pn_ic_plummer,
    not the same random numbers.  Returns (x, v, m), AoS float64."""
    rng = np.random.default_rng(seed)
    n = int(nstars)

    def iso(r):
        z = (1.0 - 2.0 * rng.random(r.size)) * r
        ph = 2.0 * np.pi * rng.random(r.size)
        rho = np.sqrt(np.maximum(r * r - z * z, 0.0))
        return np.stack([rho * np.cos(ph), rho * np.sin(ph), z], axis=1)

    X1 = np.empty(n)
    todo = np.arange(n)
    while todo.size:
        u = rng.random(todo.size)
        ok = (u > 1e-12) & (u <= 0.999)
        X1[todo[ok]] = u[ok]
        todo = todo[~ok]
    r = 1.0 / np.sqrt(X1 ** (-2.0 / 3.0) - 1.0)
    q = np.empty(n)
    todo = np.arange(n)
    while todo.size:
        X4, X5 = rng.random(todo.size), rng.random(todo.size)
        ok = 0.1 * X5 < X4 * X4 * (1.0 - X4 * X4) ** 3.5
        q[todo[ok]] = X4[ok]
        todo = todo[~ok]
    rscale = 3.0 * np.pi / 16.0
    xs = iso(r) * rscale
    vs = iso(q * np.sqrt(2.0) * (1.0 + r * r) ** -0.25) / np.sqrt(rscale)
    xs -= xs.mean(axis=0)
    vs -= vs.mean(axis=0)
    x = np.zeros((n + 1, 3))
    v = np.zeros((n + 1, 3))
    x[1:], v[1:] = xs, vs
    m = np.full(n + 1, 1.0 / max(n, 1))
    m[0] = bh_fraction
    return x, v, m


# ---------------------------------------------------------------- the C restatement
def force(x, v, m, eps):
    x, v, m = _state(x, v, m)
    a = np.zeros_like(x)
    lib().orc_force(x.shape[0], _ptr(x), _ptr(v), _ptr(m), float(eps), _ptr(a))
    return a


def force_newton(x, m, eps):
    x = np.ascontiguousarray(x, dtype=np.float64).reshape(-1, 3)
    m = np.ascontiguousarray(m, dtype=np.float64)
    a = np.zeros_like(x)
    lib().orc_force_newton(x.shape[0], _ptr(x), _ptr(m), float(eps), _ptr(a))
    return a


def force_rows(x, v, m, eps, rows, with_bh_row=False):
    """Rows of force() for the given star indices; with_bh_row also returns each row's
    share of the BH three-body sum (the work of one full row of force())."""
    x, v, m = _state(x, v, m)
    rows = np.ascontiguousarray(rows, dtype=np.int32)
    a = np.zeros((rows.shape[0], 3))
    b = np.zeros((rows.shape[0], 3)) if with_bh_row else None
    rc = lib().orc_force_rows(x.shape[0], _ptr(x), _ptr(v), _ptr(m), float(eps),
                              rows.ctypes.data_as(_ip), rows.shape[0], _ptr(a),
                              _ptr(b) if b is not None else None)
    if rc != 0:
        raise ValueError("orc_force_rows: bad row index")
    return (a, b) if with_bh_row else a


def time_force_rows(x, v, m, eps, rows, threads=1):
    """Wall time of force() rows (all three O(N^2) sweeps per row) split over host threads
    (ctypes releases the GIL).  Returns seconds."""
    import time
    x, v, m = _state(x, v, m)
    rows = np.ascontiguousarray(rows, dtype=np.int32)
    parts = [p for p in np.array_split(rows, max(1, threads)) if p.size]
    outs = [(np.zeros((p.size, 3)), np.zeros((p.size, 3))) for p in parts]
    L = lib()

    def work(k):
        p = parts[k]
        L.orc_force_rows(x.shape[0], _ptr(x), _ptr(v), _ptr(m), float(eps),
                         p.ctypes.data_as(_ip), p.size, _ptr(outs[k][0]), _ptr(outs[k][1]))
    ths = [threading.Thread(target=work, args=(k,)) for k in range(len(parts))]
    t0 = time.perf_counter()
    for t in ths:
        t.start()
    for t in ths:
        t.join()
    return time.perf_counter() - t0


def energy(x, v, m, eps):
    """Returns (pot_n, kin_n, pot_pn, total) as the reference prints them."""
    x, v, m = _state(x, v, m)
    out = np.zeros(4)
    lib().orc_energy(x.shape[0], _ptr(x), _ptr(v), _ptr(m), float(eps), _ptr(out))
    return out


def run(x, v, m, eps, dt, nsteps):
    x, v, m = _state(x, v, m)
    x = x.copy()
    v = v.copy()
    rc = lib().orc_run(x.shape[0], _ptr(x), _ptr(v), _ptr(m), float(eps), float(dt), int(nsteps))
    if rc != 0:
        raise MemoryError("orc_run")
    return x, v


# ---------------------------------------------------------------- the reference itself
def ref_force(x, v, m, eps):
    x, v, m = _state(x, v, m)
    a = np.zeros_like(x)
    _big_stack(ref().ls9_force, _ptr(x), _ptr(v), _ptr(m), float(eps), _ptr(a), x.shape[0])
    return a


def ref_initial_energy(x, v, m, eps):
    x, v, m = _state(x, v, m)
    e = np.zeros(1)
    _big_stack(ref().ls9_initial_energy, _ptr(x), _ptr(v), _ptr(m), x.shape[0], _ptr(e),
               float(eps))
    return float(e[0])


def ref_run(x, v, m, eps, dt, nsteps):
    x, v, m = _state(x, v, m)
    x = x.copy()
    v = v.copy()
    scratch = np.zeros(33 * x.shape[0])

    def go():
        for _ in range(nsteps):
            ref().ls9_rk_step(_ptr(x), _ptr(v), _ptr(m), float(eps), float(dt), x.shape[0],
                              _ptr(scratch))
    _big_stack(go)
    return x, v
