"""The algebra of the adjoint pair sweep (k_pair_vjp, pn_adjoint.cu), checked in float64 on the CPU.

For one ordered pair (i, j) with d = s_j - s_i, dv = v_j - v_i, Q = (|d|^2 + eps^2)^(-1/2), the
pair's contribution to the adjoint-weighted forward sums is
    F = Gbar.(m Q^3 d) + Phibar m Q + S0bar m Q^3 + Ubar mu3 Q + Wbar.(cd d + cv dv)
    cd = m Q^3 br + k35 Q,  cv = m Q^3 (4 v_i.d - 3 v_j.d)
    br = c1 + c3 (|d|^2 + eps^2 - qe_i) + |v_i|^2 - 2 |dv|^2 + 1.5 (v_j.d)^2 Q^2
(the forward pair sums of the force sweep).  The sweep accumulates, per row p, the derivatives of
sum_q F(p, q) (role 1) and sum_q F(q, p) (role 2) with respect to row p's variables, in a
factored form: scalar sums times per-row factors, both roles sharing one vector sum for s-bar and
one for v-bar, the self pair skipped and its mu3 term added per row.  This test checks
  (1) the closed-form pair derivatives against central differences of F itself, and
  (2) the factored row sums against the plain per-pair sums of those derivatives.
"""
import numpy as np

rng = np.random.default_rng(0)
N = 60
EPS2 = 0.01
s = rng.normal(size=(N, 3))
v = rng.normal(size=(N, 3)) * 0.5
m, mu3, c1, c3, k35 = (rng.uniform(0.1, 1, N) for _ in range(5))
qe = rng.uniform(0.5, 2, N)
G, W = rng.normal(size=(N, 3)), rng.normal(size=(N, 3))
Phi, S0, U = rng.normal(size=N), rng.normal(size=N), rng.normal(size=N)


def F(i, j, si, vi, sj, vj, mj, mu3j, c1j, c3j, k35j):
    d = sj - si
    dv = vj - vi
    rho = d @ d + EPS2
    Q = rho ** -0.5
    br = c1j + c3j * (rho - qe[i]) + vi @ vi - 2 * dv @ dv + 1.5 * (vj @ d) ** 2 * Q * Q
    cd = mj * Q ** 3 * br + k35j * Q
    cv = mj * Q ** 3 * (4 * vi @ d - 3 * vj @ d)
    return (G[i] @ (mj * Q ** 3 * d) + Phi[i] * mj * Q + S0[i] * mj * Q ** 3 + U[i] * mu3j * Q
            + W[i] @ (cd * d + cv * dv))


def pair_derivs(i, j):
    """Closed forms: dF/dd, dF/dv_i, dF/dv_j, dF/dqe_i and dF/d(mu3_j, c1_j, c3_j, k35_j)."""
    d = s[j] - s[i]
    dv = v[j] - v[i]
    rho = d @ d + EPS2
    Q = rho ** -0.5
    Q2, Q3 = Q * Q, Q ** 3
    mQ3 = m[j] * Q3
    gd, wd, wdv = G[i] @ d, W[i] @ d, W[i] @ dv
    vdi, vdj = v[i] @ d, v[j] @ d
    br = c1[j] + c3[j] * (rho - qe[i]) + v[i] @ v[i] - 2 * dv @ dv + 1.5 * vdj ** 2 * Q2
    k4 = 4 * vdi - 3 * vdj
    cd = mQ3 * br + k35[j] * Q
    cv = mQ3 * k4
    LQ = (3 * m[j] * Q2 * (gd + S0[i] + br * wd + k4 * wdv) + Phi[i] * m[j] + U[i] * mu3[j]
          + wd * (3 * mQ3 * vdj ** 2 * Q + k35[j]))
    D = (mQ3 * (G[i] + 2 * c3[j] * wd * d + 3 * Q2 * vdj * wd * v[j] + wdv * (4 * v[i] - 3 * v[j]))
         + cd * W[i] - LQ * Q3 * d)
    dvi = mQ3 * wd * (4 * v[j] - 2 * v[i]) + 4 * mQ3 * wdv * d - cv * W[i]
    dvj = mQ3 * wd * (-4 * dv + 3 * Q2 * vdj * d) - 3 * mQ3 * wdv * d + cv * W[i]
    return dict(D=D, dvi=dvi, dvj=dvj, dqe=-c3[j] * mQ3 * wd, dmu3=U[i] * Q, dc1=mQ3 * wd,
                dc3=mQ3 * wd * (rho - qe[i]), dk35=Q * wd)


def test_pair_derivatives_match_finite_differences():
    h = 1e-6
    for i, j in [(0, 1), (5, 17), (33, 2)]:
        der = pair_derivs(i, j)
        args = [s[i], v[i], s[j], v[j], m[j], mu3[j], c1[j], c3[j], k35[j]]

        def num(k, comp=None):
            a, b = [x.copy() if isinstance(x, np.ndarray) else x for x in args], \
                   [x.copy() if isinstance(x, np.ndarray) else x for x in args]
            if comp is None:
                a[k] += h
                b[k] -= h
            else:
                a[k][comp] += h
                b[k][comp] -= h
            return (F(i, j, *a) - F(i, j, *b)) / (2 * h)

        fd_D = np.array([num(2, c) for c in range(3)])  # d/ds_j = dF/dd
        fd_vi = np.array([num(1, c) for c in range(3)])
        fd_vj = np.array([num(3, c) for c in range(3)])
        scale = max(np.abs(fd_D).max(), 1.0)
        assert np.abs(der["D"] - fd_D).max() <= 1e-6 * scale
        assert np.abs(der["dvi"] - fd_vi).max() <= 1e-6 * max(np.abs(fd_vi).max(), 1.0)
        assert np.abs(der["dvj"] - fd_vj).max() <= 1e-6 * max(np.abs(fd_vj).max(), 1.0)
        for key, k in (("dmu3", 5), ("dc1", 6), ("dc3", 7), ("dk35", 8)):
            assert abs(der[key] - num(k)) <= 1e-6 * max(abs(num(k)), 1.0)


def plain_row(p):
    """Row p: derivatives of sum_q F(p, q) and sum_q F(q, p) w.r.t. p's variables (self pair
    included, as the forward sums include it)."""
    sb, vb = np.zeros(3), np.zeros(3)
    out = dict(qe=0.0, mu3=0.0, c1=0.0, c3=0.0, k35=0.0)
    for q in range(N):
        r1, r2 = pair_derivs(p, q), pair_derivs(q, p)
        sb += -r1["D"] + r2["D"]
        vb += r1["dvi"] + r2["dvj"]
        out["qe"] += r1["dqe"]
        for k in ("mu3", "c1", "c3", "k35"):
            out[k] += r2["d" + k]
    return np.concatenate([sb, vb, [out["qe"], out["mu3"], out["c1"], out["c3"], out["k35"]]])


def factored_row(p):
    """The sweep's form: scalar sums times row factors, shared vector sums, self pair skipped."""
    Sacc, Vacc = np.zeros(3), np.zeros(3)
    A = B = Sg = Scv = QE = Sg2 = Sb2 = MU3 = C3 = K35 = S0s = 0.0
    vi2 = (v * v).sum(1)
    cW = (W * v).sum(1)
    for q in range(N):
        if q == p:
            continue
        d = s[q] - s[p]
        rho = d @ d + EPS2
        Q = rho ** -0.5
        Q2, Q3 = Q * Q, Q ** 3
        vdp, vdq, vpq = v[p] @ d, v[q] @ d, v[p] @ v[q]
        dv2 = vi2[p] + vi2[q] - 2 * vpq
        mQ3 = m[q] * Q3
        gd, wd, wdv = G[p] @ d, W[p] @ d, W[p] @ v[q] - cW[p]
        br = c1[q] + c3[q] * (rho - qe[p]) + vi2[p] - 2 * dv2 + 1.5 * vdq ** 2 * Q2
        k4 = 4 * vdp - 3 * vdq
        cd, cv = mQ3 * br + k35[q] * Q, mQ3 * k4
        LQ = (3 * m[q] * Q2 * (gd + S0[p] + br * wd + k4 * wdv) + Phi[p] * m[q] + U[p] * mu3[q]
              + wd * (3 * mQ3 * vdq ** 2 * Q + k35[q]))
        ga, h = mQ3 * wd, mQ3 * wdv
        al = 2 * c3[q] * ga - LQ * Q3
        be = 3 * (Q2 * vdq * ga - h)
        A += h; B += cd; Sg += ga; Scv += cv; QE += c3[q] * ga; S0s += mQ3
        mQ3b = m[p] * Q3
        gq, wq = G[q] @ d, W[q] @ d
        wdv2 = W[q] @ v[p] - cW[q]
        rq = rho - qe[q]
        br2 = c1[p] + c3[p] * rq + vi2[q] - 2 * dv2 + 1.5 * vdp ** 2 * Q2
        k42 = 3 * vdp - 4 * vdq
        cd2, cv2 = mQ3b * br2 + k35[p] * Q, mQ3b * k42
        LQ2 = (3 * m[p] * Q2 * (-gq + S0[q] - br2 * wq + k42 * wdv2) + Phi[q] * m[p] + U[q] * mu3[p]
               - wq * (3 * mQ3b * vdp ** 2 * Q + k35[p]))
        ga2, h2 = -mQ3b * wq, mQ3b * wdv2
        al2 = 2 * c3[p] * ga2 - LQ2 * Q3
        be2 = -3 * (Q2 * vdp * ga2 + h2)
        Sg2 += ga2; Sb2 += be2; MU3 += U[q] * Q; C3 += ga2 * rq; K35 += -Q * wq
        Sacc += -(al + al2) * d + (4 * h2 - be) * v[q] + mQ3b * G[q] + cd2 * W[q]
        Vacc += 4 * (ga + ga2) * v[q] + (4 * h - be2) * d + cv2 * W[q]
    sb = Sacc - G[p] * S0s - 4 * v[p] * A - W[p] * B + v[p] * Sb2
    vb = Vacc - 2 * v[p] * Sg - W[p] * Scv - 4 * v[p] * Sg2
    return np.concatenate([sb, vb, [-QE, MU3 + U[p] / np.sqrt(EPS2), Sg2, C3, K35]])


def test_factored_row_sums_equal_plain_sums():
    for p in (0, 7, 41):
        a, b = plain_row(p), factored_row(p)
        assert np.abs(a - b).max() <= 1e-12 * np.abs(a).max(), (p, np.abs(a - b).argmax())


def _row_out(p, Y):
    """The per-row finish of the factored sums (vjp_row_out), self pair's mu3 term included."""
    Sacc, Vacc = Y[0:3], Y[3:6]
    A, B, Sg, Scv, QE, S0s, Sg2, Sb2, MU3, C3, K35 = Y[6:]
    sb = Sacc - G[p] * S0s - 4 * v[p] * A - W[p] * B + v[p] * Sb2
    vb = Vacc - 2 * v[p] * Sg - W[p] * Scv - 4 * v[p] * Sg2
    return np.concatenate([sb, vb, [-QE, MU3 + U[p] / np.sqrt(EPS2), Sg2, C3, K35]])


def symmetric_rows():
    """The symmetric sweep's form: each unordered pair {p, q} visited once; the intermediates of
    the two pair terms F(p, q) and F(q, p) serve row p (y) and row q (z, the same sums with
    d -> -d and the two terms' roles exchanged)."""
    Y = np.zeros((N, 17))
    vi2 = (v * v).sum(1)
    cW = (W * v).sum(1)
    for p in range(N):
        for q in range(p + 1, N):
            d = s[q] - s[p]
            rho = d @ d + EPS2
            Q = rho ** -0.5
            Q2, Q3 = Q * Q, Q ** 3
            vdp, vdq, vpq = v[p] @ d, v[q] @ d, v[p] @ v[q]
            dv2 = vi2[p] + vi2[q] - 2 * vpq
            rp = rho - qe[p]
            mQ3 = m[q] * Q3
            gd, wd, wdv = G[p] @ d, W[p] @ d, W[p] @ v[q] - cW[p]
            # the kernel's form: -2|v_q|^2 folded into c1v, |v_p|^2 - 2|dv|^2 = -|v_p|^2 - 2|v_q|^2 + 4 v_p.v_q
            br = (c1[q] - 2 * vi2[q]) + c3[q] * rp + (4 * vpq - vi2[p]) + 1.5 * vdq ** 2 * Q2
            k4 = 4 * vdp - 3 * vdq
            cd, cv = mQ3 * br + k35[q] * Q, mQ3 * k4
            inn = gd + S0[p] + br * wd + k4 * wdv
            LQ = 3 * m[q] * Q2 * (inn + wd * vdq ** 2 * Q2) + Phi[p] * m[q] + U[p] * mu3[q] + wd * k35[q]
            ga, h = mQ3 * wd, mQ3 * wdv
            al = 2 * c3[q] * ga - LQ * Q3
            be = 3 * (Q2 * vdq * ga - h)
            mQ3b = m[p] * Q3
            gq, wq = G[q] @ d, W[q] @ d
            wdv2 = W[q] @ v[p] - cW[q]
            rq = rho - qe[q]
            br2 = (c1[p] - 2 * vi2[p]) + c3[p] * rq + (4 * vpq - vi2[q]) + 1.5 * vdp ** 2 * Q2
            k42 = 3 * vdp - 4 * vdq
            cd2, cv2 = mQ3b * br2 + k35[p] * Q, mQ3b * k42
            inn2 = -gq + S0[q] - br2 * wq + k42 * wdv2
            LQ2 = 3 * m[p] * Q2 * (inn2 - wq * vdp ** 2 * Q2) + Phi[q] * m[p] + U[q] * mu3[p] - wq * k35[p]
            ga2, h2 = -mQ3b * wq, mQ3b * wdv2
            al2 = 2 * c3[p] * ga2 - LQ2 * Q3
            be2 = -3 * (Q2 * vdp * ga2 + h2)
            cS, cSv, cV, cVd = -(al + al2), 4 * h2 - be, 4 * (ga + ga2), 4 * h - be2
            y = Y[p]
            y[0:3] += cS * d + cSv * v[q] + mQ3b * G[q] + cd2 * W[q]
            y[3:6] += cV * v[q] + cVd * d + cv2 * W[q]
            y[6:] += [h, cd, ga, cv, c3[q] * ga, mQ3, ga2, be2, U[q] * Q, ga2 * rq, -Q * wq]
            z = Y[q]
            z[0:3] += -cS * d + cVd * v[p] + mQ3 * G[p] + cd * W[p]
            z[3:6] += cV * v[p] - cSv * d + cv * W[p]
            z[6:] += [h2, cd2, ga2, cv2, c3[p] * ga2, mQ3b, ga, be, U[p] * Q, ga * rp, Q * wd]
    return np.array([_row_out(p, Y[p]) for p in range(N)])


def test_symmetric_sweep_equals_plain_sums():
    rows = symmetric_rows()
    for p in (0, 7, 41, N - 1):
        a = plain_row(p)
        assert np.abs(rows[p] - a).max() <= 1e-12 * np.abs(a).max(), (p, np.abs(rows[p] - a).argmax())
