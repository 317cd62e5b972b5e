"""libpn's C ABI and host utilities, without a GPU: the library loads, exports every function
include/pn.h declares, reports the absence of a GPU as a status (no abort), and its initial
conditions and text formats behave as the reference's (Limit-sticky9.c:777-826)."""
import ctypes
import os
import re

import numpy as np
import pytest

from conftest import ROOT


def header_functions():
    src = open(os.path.join(ROOT, "include", "pn.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    names = re.findall(r"^[a-z_ ]+?[\s\*]([a-z_0-9]+)\s*\(", src, flags=re.M)
    return sorted(set(names))


def test_header_parsed():
    names = header_functions()
    for must in ("force", "energy", "initial_energy", "pn_create", "pn_steps", "pn_force_device"):
        assert must in names


def test_library_exports_every_declared_function(pn):
    L = pn.lib()
    missing = [n for n in header_functions() if not hasattr(L, n)]
    assert not missing, missing
    bound = {name for name, _, _ in pn.SIGNATURES}
    assert set(header_functions()) <= bound, set(header_functions()) - bound


def test_version_and_status_strings(pn):
    assert b"sm_103a" in pn.lib().pn_version()
    assert pn.lib().pn_strerror(0) == b"ok"
    assert pn.lib().pn_strerror(-4).startswith(b"non-finite")


def test_params_default_match_reference(pn):
    p = pn.default_params()
    assert p.eps == 0.001 and p.dt == 1.0 / 131072.0  # Limit-sticky9.c:770-771
    assert p.inv_c2 == 1.0 and p.precision == pn.PN_PREC_FP64


def test_no_gpu_is_a_status_not_an_abort(pn):
    if pn.lib().pn_device_count() > 0:
        pytest.skip("a GPU is present")
    h = ctypes.c_void_p()
    p = pn.default_params()
    assert pn.lib().pn_create(ctypes.byref(h), 100, ctypes.byref(p)) == -7
    with pytest.raises(pn.PNError):
        pn.force(np.zeros((2, 3)), np.zeros((2, 3)), np.array([0.01, 1e-3]), 0.01)
    # the raw drop-in entry point returns with PN_ERR_UNSUPPORTED and leaves a untouched
    x = np.zeros((2, 3))
    x[1, 0] = 0.5
    a = np.full((2, 3), 7.0)
    m = np.array([0.01, 1e-3])
    pn.lib().force(pn._p(x), pn._p(np.zeros((2, 3))), pn._p(m), 0.01, pn._p(a), None, 2)
    assert pn.lib().pn_last_error() == -7 and (a == 7.0).all()


def test_invalid_arguments(pn):
    h = ctypes.c_void_p()
    p = pn.default_params(eps=-1.0)
    assert pn.lib().pn_create(ctypes.byref(h), 100, ctypes.byref(p)) == -1
    p = pn.default_params(tile_j=48)
    assert pn.lib().pn_create(ctypes.byref(h), 100, ctypes.byref(p)) == -1
    assert pn.lib().pn_create(ctypes.byref(h), 0, None) == -1
    # the peak probes: FP64, FP32, packed FP32x2 (0..2); anything else or no output is invalid
    t = np.zeros(1)
    assert pn.lib().pn_probe_fma_peak(3, pn._p(t)) == -1
    assert pn.lib().pn_probe_fma_peak(-1, pn._p(t)) == -1
    assert pn.lib().pn_probe_fma_peak(pn.PN_PREC_MIXED, None) == -1


def test_uniform_sphere_deterministic(pn):
    x1, v1 = pn.uniform_sphere(5000, 1.0, 7)
    x2, _ = pn.uniform_sphere(5000, 1.0, 7)
    x3, _ = pn.uniform_sphere(5000, 1.0, 8)
    assert np.array_equal(x1, x2) and not np.array_equal(x1, x3)
    r = np.linalg.norm(x1, axis=1)
    assert r.max() <= 1.0 and (v1 == 0).all()
    # uniform in volume: P(r < 0.5) = 1/8
    assert abs((r < 0.5).mean() - 0.125) < 0.02


def test_plummer_henon_units(pn):
    n = 20000
    x, v = pn.plummer(n, 3)
    m = 1.0 / n
    kin = 0.5 * m * (v * v).sum()
    assert kin == pytest.approx(0.25, rel=0.03)  # Henon units: K = 1/4, E = -1/4
    assert np.abs(x.mean(0)).max() < 1e-12 and np.abs(v.mean(0)).max() < 1e-12
    # potential on a sample of 2000 stars (scaled): W = -1/2
    rng = np.random.default_rng(0)
    idx = rng.choice(n, 2000, replace=False)
    xs = x[idx]
    d = np.linalg.norm(xs[:, None] - xs[None], axis=2)
    iu = np.triu_indices(2000, 1)
    w = -(1.0 / 2000) ** 2 * (1.0 / d[iu]).sum()
    assert w == pytest.approx(-0.5, rel=0.05)


def test_init_format_round_trip(pn, tmp_path):
    x, v = pn.uniform_sphere(100, 1.0, 3)
    v = np.random.default_rng(1).normal(size=(100, 3))
    p = str(tmp_path / "init.dat")
    pn.write_init(p, x, v)
    x2, v2 = pn.read_init(p, 100)
    assert np.array_equal(x2, x.astype(np.float32).astype(np.float64))
    assert np.array_equal(v2, v.astype(np.float32).astype(np.float64))
    lines = open(p).read().splitlines()
    assert len(lines) == 200


def test_read_init_rejects_short_file(pn, tmp_path):
    p = tmp_path / "short.dat"
    p.write_text("1 2 3\n4 5 6\n")
    with pytest.raises(pn.PNError):
        pn.read_init(str(p), 2)


def test_reads_reference_format_lines(pn, tmp_path):
    """The reference's own file uses Fortran-style columns and E-notation zeros."""
    p = tmp_path / "f.dat"
    p.write_text("  -4.070518     -0.2571839      -2.165247    \n"
                 "  0.0000000E+00  0.0000000E+00  0.0000000E+00\n")
    x, v = pn.read_init(str(p), 1)
    assert np.array_equal(x[0], np.array([-4.070518, -0.2571839, -2.165247], dtype=np.float32))
    assert (v == 0).all()


def test_snapshot_format(pn, tmp_path):
    x = np.array([[0.0, 0, 0], [1.25, -2.5, 3.0]])
    v = np.array([[0.0, 0, 0], [0.1, 0.2, 0.3]])
    p = str(tmp_path / "snap.dat")
    pn.write_snapshot(p, x, v)
    pn.write_snapshot(p, x, v, append=True)
    lines = open(p).read().split("\n")
    assert lines[1] == "1.250000 -2.500000 3.000000 "  # "%lf %lf %lf \n", Limit-sticky9.c:821
    assert len([ln for ln in lines if ln]) == 8


def test_push_helpers_match_reference_loops(pn):
    """push_velocity / push_position (Limit-sticky9.c:716-738) are plain host loops."""
    v = np.ones((3, 3))
    a = np.full((3, 3), 2.0)
    pn.lib().push_velocity(pn._p(v), pn._p(a), 0.5, 3)
    assert (v == 2.0).all()
    x = np.zeros((3, 3))
    pn.lib().push_position(pn._p(x), pn._p(v), 0.25, 3)
    assert (x == 0.5).all()
