"""pn_gb300 -- Python view of libpn, the GB300 (sm_103a) direct-summation force path of the
Limit-sticky9 limited-1PN N-body code.

Everything here calls the C ABI declared in ``include/pn.h`` through ctypes; there is no
Python or CPU implementation of the physics in this package, and every entry point raises
when ``pn_gb300/_lib/libpn.so`` is missing or no GPU is present.

Mirrors of the reference's entry points (Limit-sticky9.c):

* :func:`force`           -- ``force()``            (:21-424)
* :func:`initial_energy`  -- ``initial_energy()``   (:566-714), returns the energies
* :func:`energy`          -- ``energy()``           (:427-564), returns the energies and DE

Arrays are AoS ``float64[n, 3]`` with row 0 the black hole (BH), as in the reference.
:class:`Context` is the device-resident API (state on the GPU, whole integration steps).
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libpn.so")

PN_OK = 0
PN_PREC_FP64 = 0
PN_PREC_MIXED = 1
PROBE_F32X2 = 2  # PN_PROBE_F32X2: pn_probe_fma_peak of FP32 as packed two-lane fma.rn.f32x2
PN_PAIR_AUTO, PN_PAIR_SCALAR, PN_PAIR_F32X2, PN_PAIR_F32X2_OCC3, PN_PAIR_F32X2_OCC4 = 0, 1, 2, 3, 4
PN_NMAX = 270000

_STATUS = {0: "PN_OK", -1: "PN_ERR_INVALID", -2: "PN_ERR_CUDA", -3: "PN_ERR_NOMEM",
           -4: "PN_ERR_NONFINITE", -5: "PN_ERR_IO", -6: "PN_ERR_TIMEOUT",
           -7: "PN_ERR_UNSUPPORTED", -8: "PN_ERR_STATE"}


class PNError(RuntimeError):
    def __init__(self, status: int, where: str, detail: str = ""):
        self.status = status
        super().__init__(f"{where}: {_STATUS.get(status, status)} {detail}".strip())


class Params(ctypes.Structure):
    _fields_ = [("eps", ctypes.c_double), ("dt", ctypes.c_double), ("inv_c2", ctypes.c_double),
                ("precision", ctypes.c_int), ("tile_j", ctypes.c_int),
                ("i_per_thread", ctypes.c_int), ("j_split", ctypes.c_int),
                ("grid_split", ctypes.c_int), ("pair_variant", ctypes.c_int),
                ("integrator", ctypes.c_int)]


class Energy(ctypes.Structure):
    _fields_ = [("pot_n", ctypes.c_double), ("kin_n", ctypes.c_double),
                ("pot_pn", ctypes.c_double), ("total", ctypes.c_double)]

    def as_tuple(self):
        return (self.pot_n, self.kin_n, self.pot_pn, self.total)


class Stats(ctypes.Structure):
    _fields_ = [("pair_ms", ctypes.c_double), ("total_ms", ctypes.c_double),
                ("interactions", ctypes.c_double), ("tile_j", ctypes.c_int),
                ("i_per_thread", ctypes.c_int), ("j_split", ctypes.c_int),
                ("grid_split", ctypes.c_int), ("threads", ctypes.c_int),
                ("pair_variant", ctypes.c_int)]


_dp = ctypes.POINTER(ctypes.c_double)
_lib = None

# (name, restype, argtypes) of every function include/pn.h declares
SIGNATURES = [
    ("force", None, [_dp, _dp, _dp, ctypes.c_double, _dp, _dp, ctypes.c_int]),
    ("energy", None, [ctypes.c_double, _dp, _dp, _dp, ctypes.c_int, ctypes.c_double, ctypes.c_double]),
    ("initial_energy", None, [_dp, _dp, _dp, ctypes.c_int, _dp, ctypes.c_double]),
    ("push_velocity", None, [_dp, _dp, ctypes.c_double, ctypes.c_int]),
    ("push_position", None, [_dp, _dp, ctypes.c_double, ctypes.c_int]),
    ("pn_last_error", ctypes.c_int, []),
    ("pn_last_error_message", ctypes.c_char_p, []),
    ("pn_strerror", ctypes.c_char_p, [ctypes.c_int]),
    ("pn_dropin_configure", ctypes.c_int, [ctypes.c_int, ctypes.c_double]),
    ("pn_dropin_release", None, []),
    ("pn_params_default", None, [ctypes.POINTER(Params)]),
    ("pn_create", ctypes.c_int, [ctypes.POINTER(ctypes.c_void_p), ctypes.c_int, ctypes.POINTER(Params)]),
    ("pn_destroy", ctypes.c_int, [ctypes.c_void_p]),
    ("pn_set_state", ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, _dp, _dp, _dp]),
    ("pn_get_state", ctypes.c_int, [ctypes.c_void_p, _dp, _dp]),
    ("pn_force", ctypes.c_int, [ctypes.c_void_p, _dp]),
    ("pn_steps", ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    ("pn_sync", ctypes.c_int, [ctypes.c_void_p]),
    ("pn_energy", ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(Energy)]),
    ("pn_steps_energy", ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(Energy)]),
    ("pn_steps_energy_async", ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    ("pn_energy_result", ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(Energy)]),
    ("pn_snapshot_begin", ctypes.c_int, [ctypes.c_void_p]),
    ("pn_snapshot_end", ctypes.c_int, [ctypes.c_void_p, _dp, _dp]),
    ("pn_time", ctypes.c_double, [ctypes.c_void_p]),
    ("pn_get_stats", ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(Stats)]),
    ("pn_set_params", ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(Params)]),
    ("pn_save_checkpoint", ctypes.c_int, [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_double, ctypes.c_double]),
    ("pn_load_checkpoint", ctypes.c_int, [ctypes.c_void_p, ctypes.c_char_p, _dp, _dp]),
    ("pn_force_device", ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p,
                                       ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                       ctypes.c_void_p]),
    ("pn_force_noalloc", ctypes.c_int, [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                        ctypes.c_double, ctypes.c_double, ctypes.c_int, ctypes.c_void_p,
                                        ctypes.c_void_p]),
    ("pn_noalloc_last_error", ctypes.c_int, []),
    ("pn_noalloc_status", ctypes.c_int, [ctypes.c_void_p]),
    ("pn_force_vjp", ctypes.c_int, [ctypes.c_void_p, _dp, _dp, _dp, _dp]),
    ("pn_adj_forward", ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int]),
    ("pn_adj_backward", ctypes.c_int, [ctypes.c_void_p, _dp, _dp, _dp, _dp, _dp]),
    ("pn_ens_create", ctypes.c_int, [ctypes.POINTER(ctypes.c_void_p), ctypes.c_int,
                                     ctypes.POINTER(ctypes.c_int), _dp, ctypes.POINTER(Params)]),
    ("pn_ens_destroy", ctypes.c_int, [ctypes.c_void_p]),
    ("pn_ens_set_state", ctypes.c_int, [ctypes.c_void_p, _dp, _dp, _dp]),
    ("pn_ens_get_state", ctypes.c_int, [ctypes.c_void_p, _dp, _dp]),
    ("pn_ens_force", ctypes.c_int, [ctypes.c_void_p, _dp]),
    ("pn_ens_steps", ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    ("pn_ens_sync", ctypes.c_int, [ctypes.c_void_p]),
    ("pn_ens_energy", ctypes.c_int, [ctypes.c_void_p, _dp]),
    ("pn_ens_time", ctypes.c_double, [ctypes.c_void_p]),
    ("pn_ens_last_error", ctypes.c_int, []),
    ("pn_ens_bench_steps", ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, _dp]),
    ("pn_ens_autotune", ctypes.c_int, [ctypes.c_void_p]),
    ("pn_ens_set_shape", ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                        ctypes.c_int, ctypes.c_int]),
    ("pn_ens_get_shape", ctypes.c_int, [ctypes.c_void_p, ctypes.c_int] + [ctypes.POINTER(ctypes.c_int)] * 4),
    ("pn_ic_uniform_sphere", ctypes.c_int, [ctypes.c_int, ctypes.c_double, ctypes.c_uint64, _dp, _dp]),
    ("pn_ic_plummer", ctypes.c_int, [ctypes.c_int, ctypes.c_uint64, _dp, _dp]),
    ("pn_read_init", ctypes.c_int, [ctypes.c_char_p, ctypes.c_int, _dp, _dp]),
    ("pn_write_init", ctypes.c_int, [ctypes.c_char_p, ctypes.c_int, _dp, _dp]),
    ("pn_write_snapshot", ctypes.c_int, [ctypes.c_char_p, ctypes.c_int, _dp, _dp, ctypes.c_int]),
    ("pn_autotune", ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, _dp]),
    ("pn_autotune_clear", None, []),
    ("pn_bench_steps", ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, _dp, _dp]),
    ("pn_flops_per_pair", ctypes.c_double, [ctypes.c_int, ctypes.c_int, ctypes.c_int]),
    ("pn_probe_fma_peak", ctypes.c_int, [ctypes.c_int, _dp]),
    ("pn_selftest_wait_timeout", ctypes.c_int, [ctypes.c_void_p, ctypes.c_double]),
    ("pn_device_count", ctypes.c_int, []),
    ("pn_version", ctypes.c_char_p, []),
]


def lib():
    """The loaded libpn (raises if it was not built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"libpn is not built ({LIB_PATH}); run python -m pn_gb300.build")
        L = ctypes.CDLL(LIB_PATH)
        for name, res, args in SIGNATURES:
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _check(rc: int, where: str):
    if rc != PN_OK:
        msg = lib().pn_last_error_message()
        raise PNError(rc, where, msg.decode() if msg else "")


def _require_gpu():
    if lib().pn_device_count() < 1:
        raise PNError(-7, "libpn", "no CUDA device visible")


def _p(a: np.ndarray):
    return a.ctypes.data_as(_dp)


def _aos(a, n=None):
    a = np.ascontiguousarray(a, dtype=np.float64).reshape(-1, 3)
    if n is not None and a.shape[0] != n:
        raise ValueError("array length mismatch")
    return a


# ------------------------------------------------------------------ drop-in mirrors
def configure(precision: int = PN_PREC_FP64, inv_c2: float = 1.0):
    """Precision and 1PN weight of the drop-in entry points."""
    _check(lib().pn_dropin_configure(int(precision), float(inv_c2)), "pn_dropin_configure")


def force(x, v, m, eps):
    """``force(x, v, m, eps, a, pot, n)`` of the reference; returns a[n, 3]."""
    _require_gpu()
    x = _aos(x)
    n = x.shape[0]
    v = _aos(v, n)
    m = np.ascontiguousarray(m, dtype=np.float64)
    a = np.zeros_like(x)
    lib().force(_p(x), _p(v), _p(m), float(eps), _p(a), None, n)
    _check(lib().pn_last_error(), "force")
    return a


def initial_energy(x, v, m, eps):
    """Prints as the reference does and returns the total energy (``*init_ene``)."""
    _require_gpu()
    x = _aos(x)
    n = x.shape[0]
    v = _aos(v, n)
    m = np.ascontiguousarray(m, dtype=np.float64)
    e = np.zeros(1)
    lib().initial_energy(_p(x), _p(v), _p(m), n, _p(e), float(eps))
    _check(lib().pn_last_error(), "initial_energy")
    return float(e[0])


def energy(t, x, v, m, init_ene, eps):
    """Prints the reference's three lines (time, energies, DE)."""
    _require_gpu()
    x = _aos(x)
    n = x.shape[0]
    v = _aos(v, n)
    m = np.ascontiguousarray(m, dtype=np.float64)
    lib().energy(float(t), _p(x), _p(v), _p(m), n, float(init_ene), float(eps))
    _check(lib().pn_last_error(), "energy")


# ------------------------------------------------------------------ device-resident context
def default_params(**kw) -> Params:
    p = Params()
    lib().pn_params_default(ctypes.byref(p))
    for k, val in kw.items():
        if not hasattr(p, k):
            raise KeyError(k)
        setattr(p, k, val)
    return p


class Context:
    """A system resident on the GPU (``pn_ctx``)."""

    def __init__(self, nmax: int, **params):
        _require_gpu()
        self.params = default_params(**params)
        h = ctypes.c_void_p()
        _check(lib().pn_create(ctypes.byref(h), int(nmax), ctypes.byref(self.params)), "pn_create")
        self._h = h
        self.n = 0

    def close(self):
        if getattr(self, "_h", None):
            lib().pn_destroy(self._h)
            self._h = None

    __del__ = close

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def set_params(self, **kw):
        for k, val in kw.items():
            setattr(self.params, k, val)
        _check(lib().pn_set_params(self._h, ctypes.byref(self.params)), "pn_set_params")

    def set_state(self, x, v, m):
        x = _aos(x)
        n = x.shape[0]
        v = _aos(v, n)
        m = np.ascontiguousarray(m, dtype=np.float64)
        _check(lib().pn_set_state(self._h, n, _p(x), _p(v), _p(m)), "pn_set_state")
        self.n = n

    def get_state(self):
        x = np.zeros((self.n, 3))
        v = np.zeros((self.n, 3))
        _check(lib().pn_get_state(self._h, _p(x), _p(v)), "pn_get_state")
        return x, v

    def force(self):
        a = np.zeros((self.n, 3))
        _check(lib().pn_force(self._h, _p(a)), "pn_force")
        return a

    def steps(self, k: int, sync: bool = True):
        _check(lib().pn_steps(self._h, int(k)), "pn_steps")
        if sync:
            self.sync()

    def sync(self):
        _check(lib().pn_sync(self._h), "pn_sync")

    def energy(self):
        e = Energy()
        _check(lib().pn_energy(self._h, ctypes.byref(e)), "pn_energy")
        return e.as_tuple()

    def steps_energy_async(self, k: int):
        _check(lib().pn_steps_energy_async(self._h, int(k)), "pn_steps_energy_async")

    def energy_result(self):
        e = Energy()
        _check(lib().pn_energy_result(self._h, ctypes.byref(e)), "pn_energy_result")
        return e.as_tuple()

    def snapshot_begin(self):
        _check(lib().pn_snapshot_begin(self._h), "pn_snapshot_begin")

    def snapshot_end(self):
        x = np.zeros((self.n, 3))
        v = np.zeros((self.n, 3))
        _check(lib().pn_snapshot_end(self._h, _p(x), _p(v)), "pn_snapshot_end")
        return x, v

    def steps_energy(self, k: int):
        """Energies of the current state (as energy()) from the first force sweep of the next
        k integration steps, which are then run (as steps())."""
        e = Energy()
        _check(lib().pn_steps_energy(self._h, int(k), ctypes.byref(e)), "pn_steps_energy")
        return e.as_tuple()

    @property
    def time(self) -> float:
        return lib().pn_time(self._h)

    def stats(self) -> Stats:
        s = Stats()
        _check(lib().pn_get_stats(self._h, ctypes.byref(s)), "pn_get_stats")
        return s

    def autotune(self, sweeps: int = 1):
        """Tunes the pair-sweep launch shape on the current state; returns the best times (ms)."""
        t = np.zeros(2)
        _check(lib().pn_autotune(self._h, int(sweeps), _p(t)), "pn_autotune")
        return t

    def force_vjp(self, abar):
        """(xbar, vbar, m0bar) = VJP of the force at the current state with adjoint abar."""
        ab = _aos(abar, self.n)
        xb = np.zeros((self.n, 3))
        vb = np.zeros((self.n, 3))
        m0 = np.zeros(1)
        _check(lib().pn_force_vjp(self._h, _p(ab), _p(xb), _p(vb), _p(m0)), "pn_force_vjp")
        return xb, vb, float(m0[0])

    def adjoint_forward(self, nsteps: int, checkpoint_every: int):
        _check(lib().pn_adj_forward(self._h, int(nsteps), int(checkpoint_every)), "pn_adj_forward")

    def adjoint_backward(self, xbar_T, vbar_T):
        """(dL/dx0, dL/dv0, dL/dm0) from dL/dx(T), dL/dv(T) after adjoint_forward."""
        xb = _aos(xbar_T, self.n)
        vb = _aos(vbar_T, self.n)
        x0 = np.zeros((self.n, 3))
        v0 = np.zeros((self.n, 3))
        m0 = np.zeros(1)
        _check(lib().pn_adj_backward(self._h, _p(xb), _p(vb), _p(x0), _p(v0), _p(m0)),
               "pn_adj_backward")
        return x0, v0, float(m0[0])

    def bench_steps(self, k: int, flush_l2: bool = True):
        """Times k integration steps (CUDA events on the context's stream).  Returns
        (step_ms[k], pair_ms[k])."""
        sm = np.zeros(max(k, 1))
        pm = np.zeros(max(k, 1))
        _check(lib().pn_bench_steps(self._h, int(k), int(flush_l2), _p(sm), _p(pm)),
               "pn_bench_steps")
        return sm[:k], pm[:k]

    def force_device(self, n, d_x, d_v, d_m, d_a, stream=None):
        """One evaluation on caller-owned device AoS buffers (raw device pointers)."""
        _check(lib().pn_force_device(self._h, int(n), d_x, d_v, d_m, d_a, stream), "pn_force_device")


class Ensemble:
    """Independent clusters advanced together (``pn_ens``).  ``systems`` is a list of
    :class:`System`; ``eps`` one softening per cluster."""

    def __init__(self, systems, eps, **params):
        _require_gpu()
        self.sizes = [s.x.shape[0] for s in systems]
        self.offsets = np.concatenate([[0], np.cumsum(self.sizes)]).astype(int)
        self.params = default_params(**params)
        n = (ctypes.c_int * len(systems))(*self.sizes)
        e = np.ascontiguousarray(eps, dtype=np.float64)
        h = ctypes.c_void_p()
        rc = lib().pn_ens_create(ctypes.byref(h), len(systems), n, _p(e), ctypes.byref(self.params))
        if rc != PN_OK:
            raise PNError(rc, "pn_ens_create")
        self._h = h
        self.set_state(systems)

    def _ck(self, rc, where):
        if rc != PN_OK:
            raise PNError(rc, where)

    def close(self):
        if getattr(self, "_h", None):
            lib().pn_ens_destroy(self._h)
            self._h = None

    __del__ = close

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def set_state(self, systems):
        x = np.ascontiguousarray(np.concatenate([s.x for s in systems]))
        v = np.ascontiguousarray(np.concatenate([s.v for s in systems]))
        m = np.ascontiguousarray(np.concatenate([s.m for s in systems]))
        self._ck(lib().pn_ens_set_state(self._h, _p(x), _p(v), _p(m)), "pn_ens_set_state")

    def split(self, arr):
        return [arr[self.offsets[c]:self.offsets[c + 1]] for c in range(len(self.sizes))]

    def get_state(self):
        P = int(self.offsets[-1])
        x = np.zeros((P, 3))
        v = np.zeros((P, 3))
        self._ck(lib().pn_ens_get_state(self._h, _p(x), _p(v)), "pn_ens_get_state")
        return self.split(x), self.split(v)

    def force(self):
        a = np.zeros((int(self.offsets[-1]), 3))
        self._ck(lib().pn_ens_force(self._h, _p(a)), "pn_ens_force")
        return self.split(a)

    def steps(self, k, sync=True):
        self._ck(lib().pn_ens_steps(self._h, int(k)), "pn_ens_steps")
        if sync:
            self._ck(lib().pn_ens_sync(self._h), "pn_ens_sync")

    def energy(self):
        out = np.zeros(4 * len(self.sizes))
        self._ck(lib().pn_ens_energy(self._h, _p(out)), "pn_ens_energy")
        return out.reshape(-1, 4)

    def bench_steps(self, k):
        t = np.zeros(max(1, k))
        self._ck(lib().pn_ens_bench_steps(self._h, int(k), _p(t)), "pn_ens_bench_steps")
        return t[:k]

    def autotune(self):
        self._ck(lib().pn_ens_autotune(self._h), "pn_ens_autotune")

    def set_shape(self, ipt=0, js=0, size_class=-1, tile_j=128, tiles_per_item=32):
        self._ck(lib().pn_ens_set_shape(self._h, ipt, js, size_class, tile_j, tiles_per_item),
                 "pn_ens_set_shape")

    def shape(self, size_class):
        v = [ctypes.c_int() for _ in range(4)]
        self._ck(lib().pn_ens_get_shape(self._h, size_class, *[ctypes.byref(q) for q in v]),
                 "pn_ens_get_shape")
        return tuple(q.value for q in v)


# ------------------------------------------------------------------ initial conditions and I/O
def uniform_sphere(nstars: int, radius: float = 1.0, seed: int = 1):
    x = np.zeros((nstars, 3))
    v = np.zeros((nstars, 3))
    _check(lib().pn_ic_uniform_sphere(nstars, radius, seed, _p(x), _p(v)), "pn_ic_uniform_sphere")
    return x, v


def plummer(nstars: int, seed: int = 1):
    x = np.zeros((nstars, 3))
    v = np.zeros((nstars, 3))
    _check(lib().pn_ic_plummer(nstars, seed, _p(x), _p(v)), "pn_ic_plummer")
    return x, v


def read_init(path: str, nstars: int):
    x = np.zeros((nstars, 3))
    v = np.zeros((nstars, 3))
    _check(lib().pn_read_init(path.encode(), nstars, _p(x), _p(v)), "pn_read_init")
    return x, v


def write_init(path: str, x, v):
    x = _aos(x)
    v = _aos(v, x.shape[0])
    _check(lib().pn_write_init(path.encode(), x.shape[0], _p(x), _p(v)), "pn_write_init")


def write_snapshot(path: str, x, v, append: bool = False):
    x = _aos(x)
    v = _aos(v, x.shape[0])
    _check(lib().pn_write_snapshot(path.encode(), x.shape[0], _p(x), _p(v), int(append)),
           "pn_write_snapshot")


@dataclass
class System:
    """BH + stars as the reference lays them out (row 0 = BH)."""
    x: np.ndarray
    v: np.ndarray
    m: np.ndarray


def with_bh(xs, vs, m_star, m_bh, bh_x=(0.0, 0.0, 0.0), bh_v=(0.0, 0.0, 0.0)) -> System:
    """Prepends the BH (Limit-sticky9.c:786-792 places it at the origin at rest)."""
    n = xs.shape[0] + 1
    x = np.zeros((n, 3))
    v = np.zeros((n, 3))
    x[0] = bh_x
    v[0] = bh_v
    x[1:] = xs
    v[1:] = vs
    m = np.empty(n)
    m[0] = m_bh
    m[1:] = m_star
    return System(x, v, m)


def config_uniform_sphere(nstars: int = 10000, seed: int = 1, m_star: float = 1e-4,
                          m_bh: float = 0.01, float_rounded: bool = True) -> System:
    """Cold uniform ball of radius 1 plus a BH at the origin at rest.  With float_rounded the
    positions are rounded to float, as reading them from the reference's input format does
    (Limit-sticky9.c:796-808)."""
    xs, vs = uniform_sphere(nstars, 1.0, seed)
    if float_rounded:
        xs = xs.astype(np.float32).astype(np.float64)
    return with_bh(xs, vs, m_star, m_bh)


def config_plummer(nstars: int, seed: int = 1, bh_fraction: float = 0.01) -> System:
    """Plummer sphere (Henon units, total stellar mass 1) plus a BH of bh_fraction x the
    stellar mass at the origin at rest."""
    xs, vs = plummer(nstars, seed)
    return with_bh(xs, vs, 1.0 / nstars, bh_fraction)


def flops_per_pair(mode: int, precision: int, pair_variant: int = PN_PAIR_SCALAR) -> float:
    return lib().pn_flops_per_pair(int(mode), int(precision), int(pair_variant))


def probe_fma_peak(precision: int) -> float:
    """Measured FMA peak of this GPU in TFLOP/s: FP32 for PN_PREC_MIXED, FP64 for PN_PREC_FP64,
    and FP32 issued as packed two-lane fma.rn.f32x2 instructions for 2 (PROBE_F32X2)."""
    t = np.zeros(1)
    _check(lib().pn_probe_fma_peak(int(precision), _p(t)), "pn_probe_fma_peak")
    return float(t[0])


def plummer_eps(nstars: int) -> float:
    """Softening 0.01 * 4 / N^(1/3) of the Plummer configurations."""
    return 0.01 * 4.0 / nstars ** (1.0 / 3.0)
