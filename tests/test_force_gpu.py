"""Parity of the CUDA force path with the reference, through libpn's C ABI (GB300).

Tolerances (FP64 mode, per particle, normwise |a_i - a_ref,i| / |a_ref,i|):
  accelerations <= 1e-12, energies <= 1e-12 (relative), trajectories <= 1e-10 (relative to the
  largest coordinate), as the summation order differs from the reference's sequential loops.
  Where the reference's own double rounding exceeds 1e-12 (the BH of a symmetric cluster,
  whose net acceleration is far below the sum of its terms), accelerations are checked against
  the long-double evaluation of the reference's formulas (conftest.assert_matches_reference).
Mixed mode (FP32 pair terms) is checked against the FP64 GPU path and the oracle with the
error bounds stated at each test.
"""
import ctypes

import numpy as np
import pytest

from conftest import assert_matches_reference, golden, relerr

pytestmark = pytest.mark.gpu

TOL_A = 1e-12
TOL_E = 1e-12
TOL_TRAJ = 1e-10


def traj_err(a, b):
    return np.abs(a - b).max() / np.abs(b).max()


def ctx_force(pn, x, v, m, eps, **kw):
    with pn.Context(x.shape[0], eps=eps, **kw) as c:
        c.set_state(x, v, m)
        return c.force()


def random_system(n, seed, v0=0.0):
    rng = np.random.default_rng(seed)
    x = rng.uniform(-1, 1, (n, 3))
    v = rng.normal(0, 0.3, (n, 3))
    m = rng.uniform(0.5, 1.5, n) / n
    x[0] = rng.normal(0, 0.05, 3)
    v[0] = v0 * rng.normal(size=3)
    m[0] = 0.02
    return x, v, m


# ------------------------------------------------------------------ golden vectors (reference)
def test_kat_small(pn):
    g = golden("kat_small.npz")
    eps, dt = float(g["eps"][0]), float(g["dt"][0])
    for k in ("n2", "n3", "n4"):
        x, v, m = g[k + "_x"], g[k + "_v"], g[k + "_m"]
        with pn.Context(x.shape[0], eps=eps, dt=dt) as c:
            c.set_state(x, v, m)
            assert_matches_reference(c.force(), g[k + "_a"], g[k + "_a_exact"], TOL_A)
            assert abs(c.energy()[3] / g[k + "_e"][0] - 1) <= TOL_E, k
            c.steps(1)
            x1, v1 = c.get_state()
        assert traj_err(x1, g[k + "_x1"]) <= TOL_A and traj_err(v1, g[k + "_v1"]) <= TOL_A, k


def test_random_1001(pn):
    g = golden("random_1001.npz")
    eps, dt = float(g["eps"][0]), float(g["dt"][0])
    with pn.Context(1001, eps=eps, dt=dt) as c:
        c.set_state(g["x"], g["v"], g["m"])
        assert_matches_reference(c.force(), g["a"], g["a_exact"], TOL_A)
        assert abs(c.energy()[3] / g["e"][0] - 1) <= TOL_E
        c.steps(5)
        x5, v5 = c.get_state()
    assert traj_err(x5, g["x5"]) <= TOL_TRAJ and traj_err(v5, g["v5"]) <= TOL_TRAJ


def test_init10k_reference_file(pn):
    """The reference's own input (first 2000 stars of Init10k-sphere.dat), its masses and eps."""
    g = golden("init10k_2000.npz")
    xs = g["xs"].astype(np.float64)
    n = xs.shape[0] + 1
    x = np.zeros((n, 3))
    x[1:] = xs
    v = np.zeros((n, 3))
    m = np.empty(n)
    m[0] = 100.0 / n
    m[1:] = 1.0 / (n - 1)
    eps, dt = float(g["eps"][0]), float(g["dt"][0])
    with pn.Context(n, eps=eps, dt=dt) as c:
        c.set_state(x, v, m)
        assert_matches_reference(c.force(), g["a"], g["a_exact"], TOL_A)
        assert abs(c.energy()[3] / g["e"][0] - 1) <= TOL_E
        c.steps(10)
        x10, v10 = c.get_state()
    assert traj_err(x10, g["x10"]) <= TOL_TRAJ and traj_err(v10, g["v10"]) <= TOL_TRAJ


def test_config1_uniform_sphere_100_steps(pn):
    """10 000 stars + BH, eps = 0.01, dt = 1e-3: one force() call, E0, 100 steps, E_end."""
    g = golden("config1.npz")
    n = g["xs"].shape[0] + 1
    x = np.zeros((n, 3))
    x[1:] = g["xs"].astype(np.float64)
    v = np.zeros((n, 3))
    eps, dt = float(g["eps"][0]), float(g["dt"][0])
    # the same input through the reference's input format
    s = pn.config_uniform_sphere(10000, seed=1, m_star=1e-4, m_bh=0.01)
    assert np.array_equal(s.x, x)
    with pn.Context(n, eps=eps, dt=dt) as c:
        c.set_state(x, v, g["m"])
        assert_matches_reference(c.force(), g["a"], g["a_exact"], TOL_A)
        assert abs(c.energy()[3] / g["e0"][0] - 1) <= TOL_E
        c.steps(int(g["nsteps"][0]))
        xT, vT = c.get_state()
        assert abs(c.energy()[3] / g["eT"][0] - 1) <= TOL_E
        assert c.time == pytest.approx(int(g["nsteps"][0]) * dt)
    assert traj_err(xT, g["xT"]) <= TOL_TRAJ and traj_err(vT, g["vT"]) <= TOL_TRAJ


# ------------------------------------------------------------------ against the oracle
SHAPES = [dict(), dict(i_per_thread=1), dict(i_per_thread=4), dict(j_split=2), dict(j_split=4),
          dict(j_split=8), dict(tile_j=32), dict(tile_j=256), dict(grid_split=3),
          dict(grid_split=7, tile_j=32, j_split=4),
          # the packed f32x2 sweep (mixed precision only; FP64 ignores the variant)
          dict(pair_variant=2), dict(pair_variant=2, i_per_thread=1, tile_j=32),
          dict(pair_variant=2, i_per_thread=2, tile_j=256, grid_split=5),
          dict(pair_variant=3, i_per_thread=2, tile_j=128, grid_split=3),
          dict(pair_variant=4, i_per_thread=2, tile_j=256, grid_split=2)]


@pytest.mark.parametrize("n", [1, 2, 3, 33, 64, 65, 129, 257, 1000])
def test_fp64_ragged_sizes(pn, oracle, n):
    x, v, m = random_system(n, n)
    a = ctx_force(pn, x, v, m, 0.02)
    assert relerr(a, oracle.force_exact(x, v, m, 0.02)).max() <= TOL_A


@pytest.mark.parametrize("shape", SHAPES, ids=[str(s) for s in SHAPES])
@pytest.mark.parametrize("prec", [0, 1])
def test_launch_shapes(pn, oracle, shape, prec):
    x, v, m = random_system(777, 5)
    a = ctx_force(pn, x, v, m, 0.02, precision=prec, **shape)
    ax = oracle.force_exact(x, v, m, 0.02)
    e = relerr(a, ax)
    if prec == 0:
        assert e.max() <= TOL_A
    else:
        # c = 1 on a uniform random cube: Newtonian and 1PN terms cancel on many particles, so
        # the error is bounded against the RMS acceleration (per-particle: loose)
        d = np.linalg.norm(a - ax, axis=1)
        assert np.sqrt((d ** 2).mean() / (np.linalg.norm(ax, axis=1) ** 2).mean()) <= 1e-6
        assert e.max() <= 1e-3


def test_energy_with_moving_bh(pn, oracle):
    """energy() uses the BH velocity (Limit-sticky9.c:498-499); force() ignores it."""
    x, v, m = random_system(300, 11, v0=0.05)
    with pn.Context(300, eps=0.02) as c:
        c.set_state(x, v, m)
        e = np.array(c.energy())
    eo = oracle.energy(x, v, m, 0.02)
    assert np.abs(e / eo - 1).max() <= TOL_E


def test_steps_vs_oracle(pn, oracle):
    x, v, m = random_system(257, 3)
    with pn.Context(257, eps=0.02, dt=2e-3) as c:
        c.set_state(x, v, m)
        c.steps(3)
        xg, vg = c.get_state()
    xo, vo = oracle.run(x, v, m, 0.02, 2e-3, 3)
    assert traj_err(xg, xo) <= TOL_A and traj_err(vg, vo) <= TOL_A


def test_step_replay_deterministic(pn):
    """Four steps in one call and four calls of one step replay the same graph."""
    x, v, m = random_system(500, 4)
    out = []
    for batched in (True, False):
        with pn.Context(500, eps=0.02, dt=1e-3) as c:
            c.set_state(x, v, m)
            if batched:
                c.steps(4)
            else:
                for _ in range(4):
                    c.steps(1)
            out.append(c.get_state())
    assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1])


def test_deterministic(pn):
    x, v, m = random_system(3000, 8)
    for prec in (0, 1):
        with pn.Context(3000, eps=0.01, precision=prec) as c:
            c.set_state(x, v, m)
            assert np.array_equal(c.force(), c.force())


@pytest.mark.parametrize("variant", [0, 2])
def test_newtonian_only(pn, oracle, variant):
    """inv_c2 = 0 gives the Newtonian sweep alone (Limit-sticky9.c:36-51)."""
    x, v, m = random_system(700, 9)
    an = oracle.force_newton(x, m, 0.02)
    assert relerr(ctx_force(pn, x, v, m, 0.02, inv_c2=0.0), an).max() <= TOL_A
    e = relerr(ctx_force(pn, x, v, m, 0.02, inv_c2=0.0, precision=1, pair_variant=variant), an)
    assert np.sqrt((e ** 2).mean()) <= 1e-6


@pytest.mark.parametrize("variant", [1, 2])
def test_mixed_energy_sweep(pn, oracle, variant):
    x, v, m = random_system(900, 14, v0=0.05)
    with pn.Context(900, eps=0.02, precision=1, pair_variant=variant) as c:
        c.set_state(x, v, m)
        e = np.array(c.energy())
    assert np.abs(e / oracle.energy(x, v, m, 0.02) - 1).max() <= 1e-6


@pytest.mark.parametrize("cval", [10.0, 1000.0])
def test_inv_c2_rescaling_identity(pn, oracle, cval):
    """With c != 1: a(x, v, m; c) = c^2 a_ref(x, v/c, m/c^2) (the reference has c = 1)."""
    x, v, m = random_system(400, 12)
    a = ctx_force(pn, x, v, m, 0.02, inv_c2=1.0 / cval ** 2)
    aref = cval ** 2 * oracle.force(x, v / cval, m / cval ** 2, 0.02)
    assert relerr(a, aref).max() <= 1e-11


def test_single_particle_bh_only(pn):
    a = ctx_force(pn, np.zeros((1, 3)), np.zeros((1, 3)), np.array([0.01]), 0.01)
    assert (a == 0).all()


def test_star_on_bh_reports_nonfinite(pn):
    """Limit-sticky9.c:74 gives 0/0 for a star exactly on the BH; libpn reports it."""
    x = np.array([[0.0, 0, 0], [0.0, 0, 0], [0.5, 0, 0]])
    v = np.array([[0.0, 0, 0], [0.1, 0, 0], [0, 0.1, 0]])
    m = np.array([0.01, 1e-3, 1e-3])
    with pn.Context(3, eps=0.01) as c:
        c.set_state(x, v, m)
        with pytest.raises(pn.PNError) as ei:
            c.force()
        assert ei.value.status == -4
        # the context stays usable afterwards
        c.set_state(np.array([[0.0, 0, 0], [0.3, 0, 0]]), np.zeros((2, 3)), m[:2])
        assert np.isfinite(c.force()).all()
    a = np.zeros((3, 3))
    pn.lib().force(pn._p(x), pn._p(v), pn._p(m), 0.01, pn._p(a), None, 3)
    assert pn.lib().pn_last_error() == -4 and np.isnan(a[0]).all()


def test_bounded_wait_times_out_cleanly(pn):
    with pn.Context(10, eps=0.01) as c:
        rc = pn.lib().pn_selftest_wait_timeout(c._h, 0.01)
        assert rc == -6
        # the context (and GPU) stay usable
        x, v, m = random_system(10, 1)
        c.set_state(x, v, m)
        assert np.isfinite(c.force()).all()


def test_fma_peak_probes(pn):
    """The roofline denominators: FP32 FMA, the same issued as packed fma.rn.f32x2, and FP64
    (GB300's FP64 rate is a small fraction of FP32's); an unknown probe is rejected."""
    f32 = pn.probe_fma_peak(pn.PN_PREC_MIXED)
    f2 = pn.probe_fma_peak(pn.PROBE_F32X2)
    f64 = pn.probe_fma_peak(pn.PN_PREC_FP64)
    assert f32 > 0 and f2 > 0 and 0 < f64 < 0.25 * f32, (f32, f2, f64)
    assert f2 <= 1.1 * f32, (f32, f2)  # two lanes per instruction, the same FMA units
    t = np.zeros(1)
    assert pn.lib().pn_probe_fma_peak(3, t.ctypes.data_as(ctypes.POINTER(ctypes.c_double))) == -1


# ------------------------------------------------------------------ drop-in entry points
def test_dropin_force_and_energy_output(pn, oracle, capfd):
    x, v, m = random_system(1001, 21)
    pn.configure(pn.PN_PREC_FP64, 1.0)
    a = pn.force(x, v, m, 0.02)
    assert relerr(a, oracle.force(x, v, m, 0.02)).max() <= TOL_A
    e0 = pn.initial_energy(x, v, m, 0.02)
    assert abs(e0 / oracle.energy(x, v, m, 0.02)[3] - 1) <= TOL_E
    pn.energy(0.5, x, v, m, e0, 0.02)
    out = capfd.readouterr().out.splitlines()
    # Limit-sticky9.c:701-703 then :560-563
    assert out[0] == "time = 0"
    assert out[1].startswith("pot = ") and " kin = " in out[1]
    assert out[2].startswith(" pot_pn = ") and out[3].startswith("  total= ")
    assert out[4] == "time = 0.5" and out[-1].startswith(" DE = ") and out[-1].endswith(" 0.5")
    de = float(out[-1].split()[2])
    assert abs(de) < 1e-12


def test_dropin_mixed_precision(pn, oracle):
    x, v, m = random_system(2000, 22)
    pn.configure(pn.PN_PREC_MIXED, 1.0)
    try:
        a = pn.force(x, v, m, 0.02)
    finally:
        pn.configure(pn.PN_PREC_FP64, 1.0)
    ax = oracle.force_exact(x, v, m, 0.02)
    d = np.linalg.norm(a - ax, axis=1)
    assert np.sqrt((d ** 2).mean() / (np.linalg.norm(ax, axis=1) ** 2).mean()) <= 1e-6


def test_force_device_pointers(pn, oracle):
    torch = pytest.importorskip("torch")
    x, v, m = random_system(600, 23)
    dx = torch.tensor(x, device="cuda")
    dv = torch.tensor(v, device="cuda")
    dm = torch.tensor(m, device="cuda")
    da = torch.zeros_like(dx)
    with pn.Context(600, eps=0.02) as c:
        c.force_device(600, ctypes.c_void_p(dx.data_ptr()), ctypes.c_void_p(dv.data_ptr()),
                       ctypes.c_void_p(dm.data_ptr()), ctypes.c_void_p(da.data_ptr()))
        c.sync()
    assert relerr(da.cpu().numpy(), oracle.force(x, v, m, 0.02)).max() <= TOL_A


# ------------------------------------------------------------------ mixed precision on a cluster
def test_mixed_error_plummer(pn):
    """Mixed vs FP64 GPU on a 16k-star Plummer cluster: RMS relative force error <= 1e-6
    (c = 1000, where the 1PN terms are corrections), and with the reference's c = 1 an RMS
    error <= 1e-6 of the RMS acceleration."""
    s = pn.config_plummer(16384, 5)
    eps = pn.plummer_eps(16384)
    for ic2, metric in ((1e-6, "rel"), (1.0, "abs")):
        a64 = ctx_force(pn, s.x, s.v, s.m, eps, inv_c2=ic2)
        a32 = ctx_force(pn, s.x, s.v, s.m, eps, inv_c2=ic2, precision=1)
        if metric == "rel":
            e = relerr(a32, a64)
            assert np.sqrt((e ** 2).mean()) <= 1e-6, np.sqrt((e ** 2).mean())
        else:
            d = np.linalg.norm(a32 - a64, axis=1)
            assert np.sqrt((d ** 2).mean() / (np.linalg.norm(a64, axis=1) ** 2).mean()) <= 1e-6


def pair_term_magnitudes(x, v, m, eps, chunk=512):
    """Per star i: the absolute sums of the pair terms its FP32 sums add up (float64),
    Gabs_i = sum_j m_j Q^3 |d| (the Newtonian sum G) and
    Wabs_i = sum_j |cd_ij| |d| + |cv_ij| |dv| (the velocity- and BH-weighted cross sum W),
    with the pair weights of the force sweep (pn_device.cuh)."""
    s = x[1:] - x[0]
    vs, ms, m0, eps2 = v[1:], m[1:], m[0], eps * eps
    q = (s * s).sum(1)
    R = 1.0 / np.sqrt(q + eps2)
    mu3 = ms * R ** 3
    c1, c3, k35, qe = 1.25 * m0 * R, 0.25 * m0 * R ** 3, 3.5 * m0 * mu3, q + eps2
    n = s.shape[0]
    Gabs, Wabs = np.zeros(n), np.zeros(n)
    for i0 in range(0, n, chunk):
        i1 = min(n, i0 + chunk)
        d = s[None, :, :] - s[i0:i1, None, :]
        dv = vs[None, :, :] - vs[i0:i1, None, :]
        dd = (d * d).sum(2)
        rho = dd + eps2
        Q = 1.0 / np.sqrt(rho)
        mQ3 = ms[None, :] * Q ** 3
        dn = np.sqrt(dd)
        vdj, vdi = (vs[None, :, :] * d).sum(2), (vs[i0:i1, None, :] * d).sum(2)
        dv2 = (dv * dv).sum(2)
        br = c1 + c3 * (rho - qe[i0:i1, None]) + (vs[i0:i1] ** 2).sum(1)[:, None] - 2 * dv2 + 1.5 * vdj ** 2 * Q ** 2
        Gabs[i0:i1] = (mQ3 * dn).sum(1)
        Wabs[i0:i1] = (np.abs(mQ3 * br + k35 * Q) * dn + np.abs(mQ3 * (4 * vdi - 3 * vdj)) * np.sqrt(dv2)).sum(1)
    return Gabs, Wabs


def test_mixed_error_bound_per_particle_at_c1(pn):
    """Mixed precision at the reference's c = 1, particle by particle (N = 8,192 Plummer + BH).

    The FP32 pair sums are accurate to a few units of FP32 rounding (u = 2^-24) of the absolute
    sums of their terms, so the per-particle bound is stated against those:
        |a32_i - a64_i| <= 8 u (Gabs_i + Wabs_i)      (pair_term_magnitudes; N = 16,384 gave 3.8)
    i.e. a relative error of at most 8 u kappa_i with kappa_i = (Gabs_i + Wabs_i) / |a_i|.  At
    c = 1 kappa reaches ~1e3 for halo stars: the W sum of a star far from the cluster picks up
    k35_j Q d terms of the stars around the BH (k35 ~ m0 m R^3) whose sum cancels against the
    BH-mediated terms of the finishing kernel, leaving a net acceleration ~1e-3 of them.  Stars
    without that cancellation (kappa < 10) keep the FP32 level: RMS relative error <= 1e-6."""
    n = 8192
    s = pn.config_plummer(n, 9)
    eps = pn.plummer_eps(n)
    a64 = ctx_force(pn, s.x, s.v, s.m, eps, inv_c2=1.0)
    a32 = ctx_force(pn, s.x, s.v, s.m, eps, inv_c2=1.0, precision=1)
    Gabs, Wabs = pair_term_magnitudes(s.x, s.v, s.m, eps)
    u = 2.0 ** -24
    err = np.linalg.norm(a32 - a64, axis=1)[1:]
    na = np.linalg.norm(a64, axis=1)[1:]
    r = err / (u * (Gabs + Wabs))
    kappa = (Gabs + Wabs) / na
    well = kappa < 10
    rel = err[well] / na[well]
    info = {"max_err_over_u_scale": float(r.max()), "median": float(np.median(r)), "kappa_max": float(kappa.max()),
            "rms_rel_kappa_lt_10": float(np.sqrt((rel ** 2).mean())), "stars_kappa_ge_10": int((~well).sum())}
    assert r.max() <= 8.0, info
    assert np.sqrt((rel ** 2).mean()) <= 1e-6, info


def test_mixed_energy_drift_matches_fp64(pn):
    s = pn.config_plummer(4096, 6)
    eps = pn.plummer_eps(4096)
    drift = []
    for prec in (0, 1):
        with pn.Context(4097, eps=eps, dt=1 / 1024, inv_c2=1e-6, precision=prec) as c:
            c.set_state(s.x, s.v, s.m)
            e0 = c.energy()[3]
            c.steps(50)
            drift.append(c.energy()[3] / e0 - 1)
    assert abs(drift[1] - drift[0]) <= 1e-6 + 0.05 * abs(drift[0])


# ------------------------------------------------------------------ optional classic RK4
def test_rk4_matches_host_rk4_with_oracle_forces(pn, oracle):
    x, v, m = random_system(120, 31)
    eps, h = 0.02, 2e-3

    def f(xx, vv):
        return vv, oracle.force_exact(xx, vv, m, eps)

    xr, vr = x.copy(), v.copy()
    for _ in range(3):
        k1x, k1v = f(xr, vr)
        k2x, k2v = f(xr + 0.5 * h * k1x, vr + 0.5 * h * k1v)
        k3x, k3v = f(xr + 0.5 * h * k2x, vr + 0.5 * h * k2v)
        k4x, k4v = f(xr + h * k3x, vr + h * k3v)
        xr = xr + h / 6 * (k1x + 2 * k2x + 2 * k3x + k4x)
        vr = vr + h / 6 * (k1v + 2 * k2v + 2 * k3v + k4v)
    with pn.Context(120, eps=eps, dt=h, integrator=1) as c:
        c.set_state(x, v, m)
        c.steps(3)
        xg, vg = c.get_state()
    assert traj_err(xg, xr) <= 1e-12 and traj_err(vg, vr) <= 1e-12


def test_rk4_is_fourth_order(pn):
    """Newtonian two-body orbit (inv_c2 = 0): halving dt divides the RK4 error by ~16, while
    the reference's state-averaging scheme is first order (error halves)."""
    x = np.array([[0.0, 0, 0], [1.0, 0, 0]])
    v = np.array([[0.0, 0, 0], [0, 1.0, 0]])
    m = np.array([1.0, 1e-12])

    def end(integrator, dt, steps):
        with pn.Context(2, eps=1e-4, dt=dt, inv_c2=0.0, integrator=integrator) as c:
            c.set_state(x, v, m)
            c.steps(steps)
            return c.get_state()[0][1]

    exact = end(1, 1e-3 / 8, 1600)  # t = 0.2 with a small step as the reference solution
    e1 = np.abs(end(1, 1e-2, 20) - exact).max()
    e2 = np.abs(end(1, 5e-3, 40) - exact).max()
    assert 12 < e1 / e2 < 20


# ------------------------------------------------------------------ energy fused into the force sweep
@pytest.mark.parametrize("prec,variant,integrator,ic2", [
    (0, 0, 0, 1.0), (0, 0, 0, 0.0), (0, 0, 1, 1.0),
    (1, 2, 0, 1.0), (1, 1, 0, 1.0), (1, 2, 1, 1e-6),
])
def test_steps_energy_fused(pn, oracle, prec, variant, integrator, ic2):
    """pn_steps_energy: the energies of the state the steps start from, taken from the first
    force sweep (Limit-sticky9.c:896 energy() then :851 force() at the same state), equal
    pn_energy's (FP64: 1e-12; mixed: 1e-6 of the oracle, as the separate mixed energy sweep),
    and the steps that follow are those of pn_steps (1e-12 of the largest coordinate)."""
    n, k = 1500, 3
    x, v, m = random_system(n, 21, v0=0.05)
    kw = dict(eps=0.02, dt=1e-3, inv_c2=ic2, precision=prec, pair_variant=variant, integrator=integrator)
    with pn.Context(n, **kw) as c:
        c.set_state(x, v, m)
        e_sep = np.array(c.energy())
        c.steps(k)
        xa, va = c.get_state()
    with pn.Context(n, **kw) as c:
        c.set_state(x, v, m)
        e_fused = np.array(c.steps_energy(k))
        assert abs(c.time - k * 1e-3) < 1e-15
        xb, vb = c.get_state()
    # relative to the largest energy (the 1PN energy is exactly 0 when inv_c2 = 0)
    scale = np.abs(e_sep).max()
    if prec == 0:
        assert np.abs(e_fused - e_sep).max() <= TOL_E * scale, (e_fused, e_sep)
    else:
        with pn.Context(n, eps=0.02, inv_c2=ic2) as c:
            c.set_state(x, v, m)
            e_ref = np.array(c.energy())
        if ic2 == 1.0:
            assert np.abs(e_ref / oracle.energy(x, v, m, 0.02) - 1).max() <= TOL_E
        assert np.abs(e_fused - e_ref).max() <= 1e-6 * scale, (e_fused, e_ref)
    assert traj_err(xb, xa) <= 1e-12 and traj_err(vb, va) <= 1e-12


def test_steps_energy_twice_and_rejects_zero_steps(pn):
    """Back-to-back fused calls report the energy at each call's starting state."""
    n = 700
    x, v, m = random_system(n, 22, v0=0.05)
    with pn.Context(n, eps=0.02, dt=1e-3) as c:
        c.set_state(x, v, m)
        e1 = np.array(c.steps_energy(2))
        e_mid = np.array(c.energy())
        e2 = np.array(c.steps_energy(1))
        with pytest.raises(RuntimeError):
            c.steps_energy(0)
    assert np.abs(e2 / e_mid - 1).max() <= TOL_E
    assert np.abs(e1 - e_mid).max() > 0  # the state moved


def test_snapshot_async_is_the_state_it_was_taken_at(pn):
    """pn_snapshot_begin/end: the state at the call, while later steps already run."""
    n = 900
    x, v, m = random_system(n, 23, v0=0.05)
    with pn.Context(n, eps=0.02, dt=1e-3) as c:
        c.set_state(x, v, m)
        c.steps(2)
        x2, v2 = c.get_state()
        c.snapshot_begin()
        c.steps_energy_async(3)
        xs, vs = c.snapshot_end()
        e = np.array(c.energy_result())
        with pytest.raises(RuntimeError):
            c.snapshot_end()
        x5, _ = c.get_state()
        e2 = np.array(c.energy())
    assert np.array_equal(xs, x2) and np.array_equal(vs, v2)
    assert not np.array_equal(x5, x2)
    with pn.Context(n, eps=0.02, dt=1e-3) as c:
        c.set_state(x2, v2, m)
        e_ref = np.array(c.energy())
    assert np.abs(e - e_ref).max() <= TOL_E * np.abs(e_ref).max()
    assert np.abs(e2 - e_ref).max() > 0
