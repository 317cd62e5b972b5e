"""Ensembles of independent clusters (pn_ens): one persistent pair launch for all clusters,
checked cluster by cluster against individual FP64 runs and the oracle."""
import numpy as np
import pytest

from conftest import relerr

pytestmark = pytest.mark.gpu


def clusters(pn, sizes, seed=0):
    """Plummer clusters (BH mass fraction log-uniform in [1e-3, 1e-1]); clusters of fewer than
    16 stars get random positions instead (the centre-of-mass shift would put a single star
    exactly on the BH, where the reference's 1PN term is 0/0)."""
    rng = np.random.default_rng(seed)
    out, eps = [], []
    for k, ns in enumerate(sizes):
        if ns == 0:
            s = pn.System(np.zeros((1, 3)), np.zeros((1, 3)), np.array([0.02]))
        elif ns < 16:
            xs = rng.uniform(-1, 1, (ns, 3))
            vs = rng.normal(0, 0.3, (ns, 3))
            s = pn.with_bh(xs, vs, 1.0 / ns, 0.02)
        else:
            s = pn.config_plummer(ns, seed * 100 + k, bh_fraction=float(10 ** rng.uniform(-3, -1)))
        out.append(s)
        eps.append(0.01)
    return out, eps


def fp64_close(a, ax, tol=1e-12):
    """FP64 agreement per particle, relative to max(|a_i|, 0.1 RMS|a|): at the reference's
    c = 1 the 1PN terms cancel the Newtonian force on some stars of these clusters."""
    n = np.linalg.norm(ax, axis=1)
    floor = 0.1 * np.sqrt((n ** 2).mean())
    return (np.linalg.norm(a - ax, axis=1) <= tol * np.maximum(n, floor)).all()


SIZES = [0, 1, 2, 63, 300, 777, 1500, 4100]


@pytest.mark.parametrize("prec", [0, 1])
def test_ensemble_force_matches_individual(pn, oracle, prec):
    systems, eps = clusters(pn, SIZES, 1)
    with pn.Ensemble(systems, eps, precision=prec, inv_c2=1.0) as e:
        acc = e.force()
    for s, a, ep in zip(systems, acc, eps):
        ax = oracle.force_exact(s.x, s.v, s.m, ep)
        if prec == 0:
            assert fp64_close(a, ax)
        else:
            d = np.linalg.norm(a - ax, axis=1)
            scale = max((np.linalg.norm(ax, axis=1) ** 2).mean(), 1e-300)  # BH-only cluster: a = 0
            assert np.sqrt((d ** 2).mean() / scale) <= 1e-6


def test_ensemble_steps_match_individual_fp64(pn):
    systems, eps = clusters(pn, [5, 200, 900, 2100], 2)
    with pn.Ensemble(systems, eps, precision=0, dt=1 / 1024) as e:
        e.steps(3)
        xs, vs = e.get_state()
        en = e.energy()
    for s, x, v, ep, ee in zip(systems, xs, vs, eps, en):
        with pn.Context(s.x.shape[0], eps=ep, dt=1 / 1024) as c:
            c.set_state(s.x, s.v, s.m)
            c.steps(3)
            xr, vr = c.get_state()
            er = np.array(c.energy())
        assert np.abs(x - xr).max() <= 1e-12 * np.abs(xr).max()
        assert np.abs(v - vr).max() <= 1e-12 * np.abs(vr).max()
        assert np.abs(ee / er - 1).max() <= 1e-12


def test_ensemble_mixed_steps_close_to_fp64(pn):
    systems, eps = clusters(pn, [300, 1200, 3000], 3)
    res = []
    for prec in (0, 1):
        with pn.Ensemble(systems, eps, precision=prec, dt=1 / 1024, inv_c2=1e-6) as e:
            e.steps(10)
            res.append(e.get_state())
    for x64, x32 in zip(res[0][0], res[1][0]):
        assert np.abs(x32 - x64).max() <= 1e-9 * np.abs(x64).max()


def test_ensemble_autotune_keeps_results(pn, oracle):
    systems, eps = clusters(pn, [100, 1000, 2500, 2600], 4)
    with pn.Ensemble(systems, eps, precision=1) as e:
        a0 = e.force()
        e.autotune()
        a1 = e.force()
        ipt, js, tj, tpi = e.shape(11)
        assert tj in (64, 128, 256) and tpi >= 1 and (ipt, js) in ((1, 1), (2, 1), (1, 4))
    for s, x0, x1, ep in zip(systems, a0, a1, eps):
        ax = oracle.force_exact(s.x, s.v, s.m, ep)
        for a in (x0, x1):
            d = np.linalg.norm(a - ax, axis=1)
            assert np.sqrt((d ** 2).mean() / (np.linalg.norm(ax, axis=1) ** 2).mean()) <= 1e-6


def test_ensemble_explicit_shapes(pn, oracle):
    systems, eps = clusters(pn, [64, 700, 1300], 5)
    for ipt, js, tj, tpi in [(1, 1, 32, 1), (2, 1, 256, 4), (1, 4, 64, 2)]:
        with pn.Ensemble(systems, eps, precision=0) as e:
            e.set_shape(ipt, js)
            for k in range(6, 12):
                e.set_shape(0, 0, k, tj, tpi)
            acc = e.force()
        for s, a, ep in zip(systems, acc, eps):
            assert fp64_close(a, oracle.force_exact(s.x, s.v, s.m, ep))


def test_ensemble_256_clusters_persistent_queue(pn, oracle):
    """The ensemble configuration's shape at test size: 256 Plummer + BH clusters, N log-uniform
    in [64, 2048], BH mass fraction log-uniform in [1e-3, 1e-1], eps = 0.01, dt = 1/1024, so the
    persistent queue runs at the real item count.  Every cluster of the FP64 ensemble equals its
    individual FP64 run (1e-12) and every cluster of the tuned mixed ensemble stays close to it
    after 10 steps (positions 1e-8, velocities 1e-6 of the largest); a few clusters' forces at c = 1 are checked against the exact oracle."""
    rng = np.random.default_rng(256)
    nc = 256
    sizes = np.exp(rng.uniform(np.log(64), np.log(2048), nc)).astype(int)
    fracs = np.exp(rng.uniform(np.log(1e-3), np.log(1e-1), nc))
    systems = [pn.config_plummer(int(s), 5000 + k, float(f)) for k, (s, f) in enumerate(zip(sizes, fracs))]
    eps = [0.01] * nc
    nsteps = 10
    states = {}
    for prec in (0, 1):
        with pn.Ensemble(systems, eps, precision=prec, dt=1 / 1024, inv_c2=1e-6) as e:
            if prec == 1:
                e.autotune()
            e.steps(nsteps)
            states[prec] = e.get_state()
    for k, s in enumerate(systems):
        with pn.Context(s.x.shape[0], eps=eps[k], dt=1 / 1024, inv_c2=1e-6) as c:
            c.set_state(s.x, s.v, s.m)
            c.steps(nsteps)
            xr, vr = c.get_state()
        x64, v64 = states[0][0][k], states[0][1][k]
        x32, v32 = states[1][0][k], states[1][1][k]
        assert np.abs(x64 - xr).max() <= 1e-12 * np.abs(xr).max(), k
        assert np.abs(v64 - vr).max() <= 1e-12 * np.abs(vr).max(), k
        # mixed: FP32 pair terms (per-particle force error ~1e-6 at worst) over 30 evaluations
        assert np.abs(x32 - xr).max() <= 1e-8 * np.abs(xr).max(), k
        assert np.abs(v32 - vr).max() <= 1e-6 * np.abs(vr).max(), k
    picks = sorted({int(np.argmin(sizes)), int(np.argmax(sizes))} | {int(q) for q in rng.choice(nc, 3, replace=False)})
    forces = {}
    for prec in (0, 1):
        with pn.Ensemble(systems, eps, precision=prec, inv_c2=1.0) as e:
            forces[prec] = e.force()
    for k in picks:
        s = systems[k]
        ax = oracle.force_exact(s.x, s.v, s.m, eps[k])
        assert fp64_close(forces[0][k], ax), k
        d = np.linalg.norm(forces[1][k] - ax, axis=1)
        assert np.sqrt((d ** 2).mean() / (np.linalg.norm(ax, axis=1) ** 2).mean()) <= 1e-6, k
