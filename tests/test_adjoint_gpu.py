"""The discrete adjoint (pn_force_vjp, pn_adj_forward/backward) against central finite
differences of the reference force (the oracle) and of whole trajectories, and through
torch.autograd.gradcheck with a torch.autograd.Function that calls the C ABI (test harness
only)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def system(n, seed, v0=0.0):
    rng = np.random.default_rng(seed)
    x = rng.uniform(-1, 1, (n, 3))
    v = rng.normal(0, 0.3, (n, 3))
    m = rng.uniform(0.5, 1.5, n) / n
    x[0] = rng.normal(0, 0.05, 3)
    v[0] = 0.0
    m[0] = 0.02
    return x, v, m


def fd_force_directional(oracle, x, v, m, eps, abar, dx, dv, dm0, h=1e-6):
    def f(t):
        mm = m.copy()
        mm[0] += t * dm0
        return (abar * oracle.force_exact(x + t * dx, v + t * dv, mm, eps)).sum()
    return (f(h) - f(-h)) / (2 * h)


@pytest.mark.parametrize("n", [2, 7, 130])
@pytest.mark.parametrize("ic2", [1.0, 0.0])
def test_force_vjp_directional_fd(pn, oracle, n, ic2):
    x, v, m = system(n, n + 7)
    eps = 0.05
    rng = np.random.default_rng(1)
    abar = rng.normal(size=(n, 3))
    with pn.Context(n, eps=eps, inv_c2=ic2) as c:
        c.set_state(x, v, m)
        xb, vb, m0b = c.force_vjp(abar)
    if ic2 == 0.0:
        # the oracle is the reference (c = 1); inv_c2 = 0 is its Newtonian sweep alone
        def f(t, dx, dv, dm):
            mm = m.copy()
            mm[0] += t * dm
            return (abar * oracle.force_newton(x + t * dx, mm, eps)).sum()
        fd = lambda dx, dv, dm: (f(1e-6, dx, dv, dm) - f(-1e-6, dx, dv, dm)) / 2e-6
    else:
        fd = lambda dx, dv, dm: fd_force_directional(oracle, x, v, m, eps, abar, dx, dv, dm)
    for trial in range(3):
        dx = rng.normal(size=(n, 3))
        dv = rng.normal(size=(n, 3))
        got = (xb * dx).sum()
        want = fd(dx, np.zeros_like(dv), 0.0)
        assert abs(got - want) <= 1e-6 * (abs(want) + np.abs(xb).sum() * 1e-3), (got, want)
        got = (vb * dv).sum()
        want = fd(np.zeros_like(dx), dv, 0.0)
        assert abs(got - want) <= 1e-6 * (abs(want) + np.abs(vb).sum() * 1e-3 + 1e-12), (got, want)
    want = fd(np.zeros_like(x), np.zeros_like(v), 1.0)
    assert abs(m0b - want) <= 1e-6 * (abs(want) + 1e-9), (m0b, want)


@pytest.mark.parametrize("n", [2000, 2, 130, 257, 385])
def test_force_vjp_mixed_close_to_fp64(pn, n):
    """The mixed-precision VJP (packed sweep, two rows per thread, ragged last block) against
    the FP64 one: 1e-5 RMS relative."""
    x, v, m = system(n, 3)
    abar = np.random.default_rng(2).normal(size=x.shape)
    out = []
    for prec in (0, 1):
        with pn.Context(n, eps=0.02, precision=prec) as c:
            c.set_state(x, v, m)
            out.append(c.force_vjp(abar))
    for k in (0, 1):
        d = np.linalg.norm(out[1][k] - out[0][k], axis=1)
        ref = np.linalg.norm(out[0][k], axis=1)
        assert np.sqrt((d ** 2).mean() / (ref ** 2).mean()) <= 1e-5
    assert abs(out[1][2] / out[0][2] - 1) <= 1e-5


def test_torch_gradcheck_through_the_c_abi(pn):
    torch = pytest.importorskip("torch")
    n, eps = 5, 0.1
    x0, v0, m = system(n, 11)
    ctx = pn.Context(n, eps=eps)

    class PNForce(torch.autograd.Function):
        @staticmethod
        def forward(fctx, x, v, m0):
            mm = m.copy()
            mm[0] = float(m0)
            ctx.set_state(x.detach().numpy(), v.detach().numpy(), mm)
            fctx.save_for_backward(x, v, m0)
            return torch.from_numpy(ctx.force())

        @staticmethod
        def backward(fctx, abar):
            x, v, m0 = fctx.saved_tensors
            mm = m.copy()
            mm[0] = float(m0)
            ctx.set_state(x.detach().numpy(), v.detach().numpy(), mm)
            xb, vb, m0b = ctx.force_vjp(abar.detach().numpy())
            return torch.from_numpy(xb), torch.from_numpy(vb), torch.tensor(m0b, dtype=torch.float64)

    x = torch.tensor(x0, dtype=torch.float64, requires_grad=True)
    v = torch.tensor(v0, dtype=torch.float64, requires_grad=True)
    m0 = torch.tensor(m[0], dtype=torch.float64, requires_grad=True)
    assert torch.autograd.gradcheck(PNForce.apply, (x, v, m0), eps=1e-6, atol=1e-7, rtol=1e-5)
    ctx.close()


def run_loss(pn, x, v, m, eps, dt, nsteps, xt, vt, prec=0):
    with pn.Context(x.shape[0], eps=eps, dt=dt, precision=prec) as c:
        c.set_state(x, v, m)
        c.steps(nsteps)
        xe, ve = c.get_state()
    return ((xe - xt) ** 2).sum() + ((ve - vt) ** 2).sum()


@pytest.mark.parametrize("K", [1, 4, 7])
def test_trajectory_gradient_fd(pn, K):
    n, eps, dt, nsteps = 64, 0.05, 0.01, 12
    x, v, m = system(n, 21)
    rng = np.random.default_rng(3)
    xt = x + rng.normal(0, 1e-3, x.shape)
    vt = v + rng.normal(0, 1e-3, v.shape)
    with pn.Context(n, eps=eps, dt=dt) as c:
        c.set_state(x, v, m)
        c.adjoint_forward(nsteps, K)
        xe, ve = c.get_state()
        gx, gv, gm = c.adjoint_backward(2 * (xe - xt), 2 * (ve - vt))
        xe2, _ = c.get_state()
    assert np.array_equal(xe, xe2)  # the final state is restored
    h = 1e-6
    idx = rng.choice(n * 3, 6, replace=False)
    for q in idx:
        p, k = divmod(int(q), 3)
        for arr, g in ((x, gx), (v, gv)):
            ap, am = arr.copy(), arr.copy()
            ap[p, k] += h
            am[p, k] -= h
            if arr is x:
                fd = (run_loss(pn, ap, v, m, eps, dt, nsteps, xt, vt) - run_loss(pn, am, v, m, eps, dt, nsteps, xt, vt)) / (2 * h)
            else:
                fd = (run_loss(pn, x, ap, m, eps, dt, nsteps, xt, vt) - run_loss(pn, x, am, m, eps, dt, nsteps, xt, vt)) / (2 * h)
            assert abs(g[p, k] - fd) <= 1e-6 * max(abs(fd), 1e-3), (p, k, g[p, k], fd)
    mp, mm = m.copy(), m.copy()
    mp[0] += h
    mm[0] -= h
    fd = (run_loss(pn, x, v, mp, eps, dt, nsteps, xt, vt) - run_loss(pn, x, v, mm, eps, dt, nsteps, xt, vt)) / (2 * h)
    assert abs(gm - fd) <= 1e-6 * max(abs(fd), 1e-3), (gm, fd)


@pytest.mark.parametrize("n", [2, 129, 300, 1025])
@pytest.mark.parametrize("prec", [0, 1])
def test_symmetric_sweep_equals_ordered_sweep(pn, monkeypatch, n, prec):
    """The symmetric VJP sweep (each unordered pair once, one CTA per pair of 128-star tiles, the
    row sums of q carried lane to lane) against the ordered sweep (each row over every star),
    selected with PN_VJP_SWEEP: the same sums in another order, at ragged sizes (one tile, a
    partial last tile, several tiles), FP64 and mixed, at c = 1 and with the weak 1PN terms."""
    x, v, m = system(n, 40 + n)
    abar = np.random.default_rng(n).normal(size=x.shape)
    for ic2 in (1.0, 1e-6):
        out = {}
        for mode in ("ordered", "symmetric"):
            monkeypatch.setenv("PN_VJP_SWEEP", mode)
            with pn.Context(n, eps=0.02, precision=prec, inv_c2=ic2) as c:
                c.set_state(x, v, m)
                out[mode] = c.force_vjp(abar)
        tol = 1e-12 if prec == 0 else 1e-5
        for k in (0, 1):
            a, b = out["symmetric"][k], out["ordered"][k]
            d = np.linalg.norm(a - b, axis=1)
            ref = np.linalg.norm(b, axis=1)
            assert np.sqrt((d ** 2).mean() / max((ref ** 2).mean(), 1e-300)) <= tol, (ic2, k)
        assert abs(out["symmetric"][2] - out["ordered"][2]) <= tol * abs(out["ordered"][2]) + 1e-300, ic2
