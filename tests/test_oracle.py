"""The CPU oracle (oracle/pn_oracle.c) pinned to the reference.

* against golden vectors generated by the unmodified reference (tests/golden/, made by
  tests/golden/make_golden.py from Limit-sticky9.c compiled by oracle/Makefile): bit-exact;
* against the reference itself (oracle/_ref), where its source is present: bit-exact;
* the reference's behavioural quirks, pinned in the oracle.
"""
import numpy as np
import pytest

from conftest import golden


def test_kat_small_bit_exact(oracle):
    g = golden("kat_small.npz")
    eps, dt = float(g["eps"][0]), float(g["dt"][0])
    for k in ("n2", "n3", "n4"):
        x, v, m = g[k + "_x"], g[k + "_v"], g[k + "_m"]
        assert np.array_equal(oracle.force(x, v, m, eps), g[k + "_a"]), k
        assert oracle.energy(x, v, m, eps)[3] == g[k + "_e"][0], k
        x1, v1 = oracle.run(x, v, m, eps, dt, 1)
        assert np.array_equal(x1, g[k + "_x1"]) and np.array_equal(v1, g[k + "_v1"]), k


def test_random_1001_bit_exact(oracle):
    g = golden("random_1001.npz")
    eps, dt = float(g["eps"][0]), float(g["dt"][0])
    assert np.array_equal(oracle.force(g["x"], g["v"], g["m"], eps), g["a"])
    assert oracle.energy(g["x"], g["v"], g["m"], eps)[3] == g["e"][0]
    x5, v5 = oracle.run(g["x"], g["v"], g["m"], eps, dt, 5)
    assert np.array_equal(x5, g["x5"]) and np.array_equal(v5, g["v5"])


def _init10k_state(g):
    xs = g["xs"].astype(np.float64)
    n = xs.shape[0] + 1
    x = np.zeros((n, 3))
    x[1:] = xs
    v = np.zeros((n, 3))
    m = np.empty(n)
    m[0] = 100.0 / n  # Limit-sticky9.c:813-816
    m[1:] = 1.0 / (n - 1)
    return x, v, m


def test_init10k_bit_exact(oracle):
    g = golden("init10k_2000.npz")
    x, v, m = _init10k_state(g)
    eps, dt = float(g["eps"][0]), float(g["dt"][0])
    assert np.array_equal(oracle.force(x, v, m, eps), g["a"])
    assert oracle.energy(x, v, m, eps)[3] == g["e"][0]
    x10, v10 = oracle.run(x, v, m, eps, dt, 10)
    assert np.array_equal(x10, g["x10"]) and np.array_equal(v10, g["v10"])


def test_config1_force_bit_exact(oracle):
    g = golden("config1.npz")
    n = g["xs"].shape[0] + 1
    x = np.zeros((n, 3))
    x[1:] = g["xs"].astype(np.float64)
    v = np.zeros((n, 3))
    eps = float(g["eps"][0])
    assert np.array_equal(oracle.force(x, v, g["m"], eps), g["a"])
    assert oracle.energy(x, v, g["m"], eps)[3] == g["e0"][0]


@pytest.mark.parametrize("n", [1, 2, 3, 4, 17, 64, 65, 300])
def test_against_reference_live(oracle, n):
    if not oracle.ref_available():
        pytest.skip("reference source not present on this machine")
    rng = np.random.default_rng(100 + n)
    x = rng.uniform(-1, 1, (n, 3))
    v = rng.normal(0, 0.3, (n, 3))
    m = rng.uniform(0.5, 1.5, n) / n
    x[0] = rng.normal(0, 0.05, 3)
    v[0] = 0
    eps = 0.015
    assert np.array_equal(oracle.force(x, v, m, eps), oracle.ref_force(x, v, m, eps))
    assert oracle.energy(x, v, m, eps)[3] == oracle.ref_initial_energy(x, v, m, eps)
    xa, va = oracle.run(x, v, m, eps, 1e-3, 2)
    xb, vb = oracle.ref_run(x, v, m, eps, 1e-3, 2)
    assert np.array_equal(xa, xb) and np.array_equal(va, vb)


def _edge_system(kind, n=40):
    rng = np.random.default_rng(7)
    x = rng.uniform(-1, 1, (n, 3))
    v = rng.normal(0, 0.3, (n, 3))
    m = rng.uniform(0.5, 1.5, n) / n
    m[0] = 0.05
    if kind == "moving_offset_bh":  # the BH away from the origin and moving
        x[0] = [0.4, -0.7, 0.2]
        v[0] = [0.05, 0.02, -0.03]
    elif kind == "coincident_stars":  # star pairs at identical positions (softened, finite)
        x[0] = [0.0, 0.0, 0.1]
        x[5] = x[6] = x[7]
        v[5] = -v[6]
    elif kind == "wide_scales":  # a tight core and a far halo: 1e-4 .. 1e3
        x[0] = 0.0
        x[1:] *= np.exp(rng.uniform(np.log(1e-4), np.log(1e3), (n - 1, 1)))
    elif kind == "mass_ratios":  # stars from 1e-9 to 1e-1 of a heavy BH
        m[0] = 10.0
        m[1:] = np.exp(rng.uniform(np.log(1e-9), np.log(1e-1), n - 1))
    return x, v, m


@pytest.mark.parametrize("kind", ["moving_offset_bh", "coincident_stars", "wide_scales", "mass_ratios"])
def test_against_reference_live_edge_cases(oracle, kind):
    """Bit-exact against the reference compiled from its source, on inputs the reference's own
    loops treat as edge cases: the BH off the origin and moving (every BH-relative term and the
    BH's own 1PN acceleration, Limit-sticky9.c:54-97), coincident stars, 7 decades of radius,
    8 decades of mass."""
    if not oracle.ref_available():
        pytest.skip("reference source not present on this machine")
    x, v, m = _edge_system(kind)
    eps = 0.01
    a = oracle.force(x, v, m, eps)
    assert np.isfinite(a).all()
    assert np.array_equal(a, oracle.ref_force(x, v, m, eps))
    assert oracle.energy(x, v, m, eps)[3] == oracle.ref_initial_energy(x, v, m, eps)
    xa, va = oracle.run(x, v, m, eps, 1e-4, 2)
    xb, vb = oracle.ref_run(x, v, m, eps, 1e-4, 2)
    assert np.array_equal(xa, xb) and np.array_equal(va, vb)


def test_quirk_scheme_is_state_averaging(oracle):
    """Limit-sticky9.c:841-893: three force() calls and an average of the stage STATES, so a
    force-free particle advances by dt*(v+v+v)/6 = v*dt/2 per step (first order)."""
    x = np.array([[0.0, 0, 0], [1e3, 0, 0]])
    v = np.array([[0.0, 0, 0], [0.5, 0, 0]])
    m = np.array([1e-300, 1e-300])  # no force in practice
    x1, v1 = oracle.run(x, v, m, 0.01, 0.1, 1)
    assert x1[1, 0] == pytest.approx(1e3 + 0.5 * 0.1 / 2, rel=0, abs=1e-12)


def test_quirk_a1c_removal_not_exact(oracle):
    """Limit-sticky9.c:176-207 removes the a1c self pair with 1.25*eps (the self-pair limit
    of :139 is 1.25/eps) and the opposite sign of dxb: the BH acceleration of a BH + 1 star
    system therefore differs from the pair-free expression.  The oracle keeps it."""
    x = np.array([[0.0, 0, 0], [0.3, 0, 0]])
    v = np.zeros((2, 3))
    m = np.array([0.01, 1e-3])
    eps = 0.05
    a = oracle.force(x, v, m, eps)
    eps2 = eps * eps
    r2 = 0.09
    R = 1 / np.sqrt(r2 + eps2)
    mr3 = m[1] * R ** 3
    newton = m[1] * 0.3 * R ** 3
    a1 = mr3 * 0.3 * (5 * m[0] * R)
    single = 4 * mr3 * R * m[1] * 0.3
    pair_self = mr3 * m[1] * 0.3 * (4 * R + 1.25 / eps)  # the two 0.25 terms cancel for j = i
    removal = -(mr3 * m[1] * (-0.3) * (4 * R + 1.25 * eps))  # 'removal' adds (sign quirk)
    expect = newton + a1 + single + pair_self + removal
    assert a[0, 0] == pytest.approx(expect, rel=1e-12)


def test_quirk_star_on_bh_is_nan(oracle):
    """Limit-sticky9.c:74 divides by the UNSOFTENED r2: a star exactly on the BH gives 0/0."""
    x = np.array([[0.0, 0, 0], [0.0, 0, 0], [0.5, 0, 0]])
    v = np.array([[0.0, 0, 0], [0.1, 0, 0], [0, 0.1, 0]])
    m = np.array([0.01, 1e-3, 1e-3])
    a = oracle.force(x, v, m, 0.01)
    assert np.isnan(a[0]).all()
    assert np.isfinite(a[2]).all()
