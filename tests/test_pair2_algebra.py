"""The pair sweeps' arithmetic restated in numpy: the packed FP32x2 form (pn_pair2.cuh) and the
scalar form of the FP32 and FP64 sweeps (pn_device.cuh).

The packed sweep evaluates the pair sums of pn_device.cuh (G, Phi, S0, U, W and Psi) from
scaled operands: positions as hi/lo pairs relative to a tile origin, m / K^3, mu3 / K, k35 / K,
w = sqrt(3) v, c1 - 2|v|^2 and c3 (k_prep's paired pack), the i side's 4/sqrt(3) v (or
1/sqrt(3) v), qe and -|v_i|^2 (pair2_block's registers), Newton's step with K-scaled constants
(Q' = K Q), and the per-tile term -0.75 vi* sum ct of the velocity-weighted sum.
Here the same operations, in the same order, run in float64 with K = 1/sqrt(2) and are checked
against the sums written from their definitions (the algebra), and in float32 with the
kernel's K and an emulated FMA (the rounding stays at a few units of FP32 rounding of the
absolute term sums).  The scalar form is checked the same way.  Everything runs on the CPU.
"""
import numpy as np
import pytest

X2_K = 2965821.0 / 4194304.0  # pn_device.cuh
SQRT3 = np.sqrt(3.0)


def _system(n, seed):
    rng = np.random.default_rng(seed)
    s = rng.normal(0.0, 1.0, (n, 3)) * rng.uniform(0.05, 3.0, (n, 1))  # BH-relative positions
    s[:8] *= 40.0  # a few halo stars
    v = rng.normal(0.0, 0.4, (n, 3))
    m = rng.uniform(0.5, 1.5, n) / n
    return s, v, m, 0.7, 0.02  # ..., m0, eps


def _definitions(s, v, m, m0, eps, i):
    """The pair sums of star i from their definitions (pn_device.cuh), float64."""
    eps2 = eps * eps
    d = s - s[i]
    dv = v - v[i]
    rho = (d * d).sum(1) + eps2
    Q = rho ** -0.5
    R = ((s * s).sum(1) + eps2) ** -0.5
    mu3 = m * R ** 3
    c1, c3, k35 = 1.25 * m0 * R, 0.25 * m0 * R ** 3, 3.5 * m0 * mu3
    qe = (s[i] * s[i]).sum() + eps2
    vdj, vdi = (v * d).sum(1), (v[i] * d).sum(1)
    mQ3 = m * Q ** 3
    br = c1 + c3 * (rho - qe) + (v[i] ** 2).sum() - 2 * (dv * dv).sum(1) + 1.5 * vdj ** 2 * Q ** 2
    cd = mQ3 * br + k35 * Q
    cv = mQ3 * (4 * vdi - 3 * vdj)
    out = {"G": (mQ3[:, None] * d).sum(0), "Phi": (m * Q).sum(), "S0": mQ3.sum(), "U": (mu3 * Q).sum(),
           "W": (cd[:, None] * d + cv[:, None] * dv).sum(0),
           "Psi": (m * Q * (7 * (v * v[i]).sum(1) + vdi * vdj * Q ** 2)).sum()}
    absw = (np.abs(cd) + np.abs(cv)) * np.sqrt((d * d).sum(1) + (dv * dv).sum(1))
    scale = {"G": (mQ3 * np.sqrt((d * d).sum(1))).sum(), "Phi": out["Phi"], "S0": out["S0"], "U": out["U"],
             "W": absw.sum(), "Psi": (m * Q * np.abs(7 * (v * v[i]).sum(1) + vdi * vdj * Q ** 2)).sum()}
    return out, scale


class _Arith:
    """Operations of one precision: float64, or float32 with a single-rounding FMA."""

    def __init__(self, dt):
        self.dt = dt

    def c(self, x):
        return np.asarray(x, dtype=np.float64).astype(self.dt)

    def fma(self, a, b, c):
        return (np.float64(1) * a * b + c).astype(self.dt) if self.dt == np.float32 else a * b + c

    def rsqrt(self, x):  # the MUFU estimate (its error is below FP32 rounding plus one ulp)
        return self.c(np.asarray(x, np.float64) ** -0.5)


def _split(x, dt):
    hi = x.astype(dt)
    return hi, (x - hi.astype(np.float64)).astype(dt)


def _packed(s, v, m, m0, eps, i, mode, dt, K=X2_K):
    """pair2_accumulate over all j (one tile whose origin is star 0) plus pair2_block's per-tile
    and final steps, in precision dt."""
    A = _Arith(dt)
    eps2 = eps * eps
    R = ((s * s).sum(1) + eps2) ** -0.5
    mu3 = m * R ** 3
    c1, c3, k35 = 1.25 * m0 * R, 0.25 * m0 * R ** 3, 3.5 * m0 * mu3
    o = s[0]
    # k_prep's paired pack
    hj, lj = _split(s - o, dt)
    jm, jmu3, jk35 = A.c(m / K ** 3), A.c(mu3 / K), A.c(k35 / K)
    w = A.c(SQRT3 * v)
    jc1, jc3 = A.c(c1 - 2 * (v * v).sum(1)), A.c(c3)
    # pair2_block's i registers: (s_i - o) formed in float64 here (the kernel's exact FP32
    # two_diff of the two split values gives the same pair to 2^-48)
    ei, li = _split(s[i] - o, dt)
    vf = v[i].astype(np.float32).astype(np.float64) if dt == np.float32 else v[i]  # the kernel reads FP32 v_i
    vi = A.c((4.0 if mode != "energy" else 1.0) / SQRT3 * vf)
    qe = np.float32((s[i] * s[i]).sum() + eps2) if dt == np.float32 else (s[i] * s[i]).sum() + eps2
    qe = A.c(qe)
    nvi2 = A.c(-(vf * vf).sum())
    e2 = A.c(eps2)

    d = [(hj[:, k] - ei[k]) + (lj[:, k] - li[k]) for k in range(3)]
    rhoe = A.fma(d[2], d[2], A.fma(d[1], d[1], A.fma(d[0], d[0], e2)))
    y = A.rsqrt(rhoe)
    Q = y * A.fma(rhoe * A.c(-0.5 * K), y * y, A.c(1.5 * K))
    Q2 = Q * Q
    mQ = jm * Q
    mQ3 = mQ * Q2
    c7 = A.c(7.0 * K * K)
    sums = {"G": np.array([(mQ3 * d[k]).astype(np.float64).sum() for k in range(3)]),
            "Phi": K * K * mQ.astype(np.float64).sum(), "S0": mQ3.astype(np.float64).sum(),
            "U": (jmu3 * Q).astype(np.float64).sum()}
    vdj = A.fma(w[:, 2], d[2], A.fma(w[:, 1], d[1], w[:, 0] * d[0]))
    vdi = A.fma(vi[2], d[2], A.fma(vi[1], d[1], vi[0] * d[0]))
    if mode == "energy":
        vivj = A.fma(vi[2], w[:, 2], A.fma(vi[1], w[:, 1], vi[0] * w[:, 0]))
        psi = A.fma(mQ, A.fma(c7, vivj, (vdi * vdj) * Q2), 0)
        return {"Phi": sums["Phi"], "Psi": psi.astype(np.float64).sum()}
    vivj = A.fma(vi[2], w[:, 2], A.fma(vi[1], w[:, 1], A.fma(vi[0], w[:, 0], nvi2)))  # 4 vi.vj - vi^2
    br = A.fma(rhoe - qe, jc3, jc1)
    br = br + vivj
    br = A.fma(vdj * vdj, Q2, br)
    cd = A.fma(mQ3, br, jk35 * Q)
    ct = mQ3 * (vdi - vdj)
    W = np.array([A.fma(cd, d[k], ct * w[:, k]).astype(np.float64).sum() for k in range(3)])
    W += -0.75 * ct.astype(np.float64).sum() * vi.astype(np.float64)
    out = dict(sums, W=W)
    if mode == "force_energy":
        psi = A.fma(mQ, A.fma(c7, vivj, (vdi * vdj) * Q2), 0).astype(np.float64).sum()
        out["Psi"] = 0.25 * psi - 1.75 * float(nvi2) * out["Phi"]
    return out


def _scalar(s, v, m, m0, eps, i, mode, dt, K=None):
    """pair_accumulate (pn_device.cuh) over all j, the scalar form of the FP32 and FP64 sweeps:
    unscaled pack (hi, lo, m | mu3 | v, qe | c1, c3, k35), the MUFU rsqrt refined as
    y + (y/2)(1 - x y^2) in FP32 (FP64: rsqrt), cv dv accumulated per pair."""
    A = _Arith(dt)
    eps2 = eps * eps
    R = ((s * s).sum(1) + eps2) ** -0.5
    mu3 = m * R ** 3
    c1, c3, k35 = 1.25 * m0 * R, 0.25 * m0 * R ** 3, 3.5 * m0 * mu3
    o = s[0]
    if dt == np.float32:
        hj, lj = _split(s - o, dt)
        ei, li = _split(s[i] - o, dt)
        d = [(hj[:, k] - ei[k]) + (lj[:, k] - li[k]) for k in range(3)]
    else:
        d = [s[:, k] - s[i, k] for k in range(3)]
    jm, jmu3, jc1, jc3, jk35 = A.c(m), A.c(mu3), A.c(c1), A.c(c3), A.c(k35)
    jv = A.c(v)
    vf = v[i].astype(np.float32).astype(np.float64) if dt == np.float32 else v[i]
    vi = A.c(vf)
    vi2 = A.c((vf * vf).sum())
    qe = A.c((s[i] * s[i]).sum() + eps2)
    e2 = A.c(eps2)
    rhoe = A.fma(d[2], d[2], A.fma(d[1], d[1], A.fma(d[0], d[0], e2)))
    if dt == np.float32:
        y = A.rsqrt(rhoe)
        h = rhoe * y
        Q = A.fma(A.c(0.5) * y, A.fma(-h, y, A.c(1.0)), y)
    else:
        Q = rhoe ** -0.5
    Q2 = Q * Q
    mQ = jm * Q
    vdj = A.fma(jv[:, 2], d[2], A.fma(jv[:, 1], d[1], jv[:, 0] * d[0]))
    vdi = A.fma(vi[2], d[2], A.fma(vi[1], d[1], vi[0] * d[0]))
    if mode == "energy":
        vivj = A.fma(vi[2], jv[:, 2], A.fma(vi[1], jv[:, 1], vi[0] * jv[:, 0]))
        psi = A.fma(mQ, A.fma(A.c(7.0), vivj, (vdi * vdj) * Q2), 0)
        return {"Phi": mQ.astype(np.float64).sum(), "Psi": psi.astype(np.float64).sum()}
    mQ3 = mQ * Q2
    dv = [jv[:, k] - vi[k] for k in range(3)]
    dv2 = A.fma(dv[2], dv[2], A.fma(dv[1], dv[1], dv[0] * dv[0]))
    br = A.fma(rhoe - qe, jc3, jc1)
    br = br + A.fma(A.c(-2.0), dv2, vi2)
    br = A.fma(A.c(1.5), (vdj * vdj) * Q2, br)
    cd = A.fma(mQ3, br, jk35 * Q)
    cv = mQ3 * A.fma(A.c(4.0), vdi, A.c(-3.0) * vdj)
    return {"G": np.array([(mQ3 * d[k]).astype(np.float64).sum() for k in range(3)]),
            "Phi": mQ.astype(np.float64).sum(), "S0": mQ3.astype(np.float64).sum(),
            "U": (jmu3 * Q).astype(np.float64).sum(),
            "W": np.array([A.fma(cd, d[k], cv * dv[k]).astype(np.float64).sum() for k in range(3)])}


FORMS = {"packed": _packed, "scalar": _scalar}


@pytest.mark.parametrize("form,mode", [("packed", "force"), ("packed", "force_energy"), ("packed", "energy"),
                                       ("scalar", "force"), ("scalar", "energy")])
def test_sweep_sums_equal_definitions_in_float64(form, mode):
    s, v, m, m0, eps = _system(300, 1)
    for i in (0, 1, 5, 77, 299):  # the tile-origin star, halo stars, core stars
        ref, scale = _definitions(s, v, m, m0, eps, i)
        got = FORMS[form](s, v, m, m0, eps, i, mode, np.float64, K=np.sqrt(0.5))
        for key, val in got.items():
            err = np.max(np.abs(np.asarray(val) - np.asarray(ref[key])))
            assert err <= 1e-12 * scale[key], (mode, i, key, err, scale[key])


@pytest.mark.parametrize("form", ["packed", "scalar"])
@pytest.mark.parametrize("mode", ["force", "energy"])
def test_sweep_sums_float32_rounding_level(form, mode):
    """In float32 every sum stays within a few units of FP32 rounding (u = 2^-24) of the sum of
    its terms' magnitudes; the velocity inputs are rounded to FP32 as the kernel's are."""
    s, v, m, m0, eps = _system(2048, 2)
    u = 2.0 ** -24
    worst = {}
    for i in range(0, 2048, 97):
        ref, scale = _definitions(s, v.astype(np.float32).astype(np.float64), m, m0, eps, i)
        got = FORMS[form](s, v, m, m0, eps, i, mode, np.float32)
        for key, val in got.items():
            r = np.max(np.abs(np.asarray(val) - np.asarray(ref[key]))) / (u * scale[key])
            worst[key] = max(worst.get(key, 0.0), float(r))
    assert max(worst.values()) <= 16.0, worst
