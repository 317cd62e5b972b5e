"""Generates the golden vectors under tests/golden/ from the UNMODIFIED reference code.

The reference functions (Limit-sticky9.c force / initial_energy, and its integration step)
are compiled from their own source by ``oracle/Makefile`` (target ``ref``) into
``oracle/_ref/libls9ref.so``; this script calls them through ``oracle/pyoracle.py``.  It needs
the reference source tree (``LS9_DIR``, else the default of ``oracle/Makefile``) and only runs
where that exists; the .npz files it writes are committed, so the tests do not need the reference.

    python tests/golden/make_golden.py [case ...]      (cases: kat random init10k config1)

Every case also stores a_exact: force() of the same input evaluated by the oracle's
long-double build (the reference's formulas with a 64-bit significand).  Where the reference's
own double rounding exceeds the test tolerance -- the BH of a symmetric cluster, whose net
acceleration is orders of magnitude below the sum of its terms -- the tests measure against it.

Cases
  kat      hand-placed BH + 1..3 stars with velocities (n = 2, 3, 4): force, energy, 1 step
  random   n = 1001, positions uniform in [-1,1]^3, velocities N(0, 0.3^2), random masses:
           force, energy, 5 steps (dt = 1e-3, eps = 0.02)
  init10k  the reference's own input file Init10k-sphere.dat, first 2000 stars (cold), with
           the reference's mass rule m0 = 100/n, m_i = 1/(n-1) and eps = 0.001
           (Limit-sticky9.c:770, 813-816): force, energy, 10 steps at dt = 1/131072
  config1  10 000 stars uniform in the unit ball (pn_ic_uniform_sphere, seed 1, positions
           rounded to float as the input format does), m = 1e-4, BH 0.01 at rest at the
           origin, eps = 0.01, dt = 1e-3: force, energy, 100 steps and the final energy
"""
from __future__ import annotations

import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import pyoracle as po  # noqa: E402


def _save(name, **arrs):
    path = os.path.join(HERE, name)
    np.savez_compressed(path, **arrs)
    print("wrote", path, os.path.getsize(path), "bytes", flush=True)


def case_kat():
    cases = {
        "n2": (np.array([[0, 0, 0], [0.3, -0.2, 0.1]]),
               np.array([[0, 0, 0], [0.05, 0.2, -0.1]]), np.array([0.01, 1e-3])),
        "n3": (np.array([[0.01, 0, 0], [0.5, 0.1, -0.3], [-0.2, 0.4, 0.25]]),
               np.array([[0, 0, 0], [0.1, -0.05, 0.2], [-0.15, 0.1, 0.05]]),
               np.array([0.02, 1e-3, 2e-3])),
        "n4": (np.array([[0, 0, 0], [1.0, 0, 0], [0, 1.0, 0], [0, 0, 1.0]]),
               np.array([[0, 0, 0], [0, 0.3, 0], [0, 0, 0.3], [0.3, 0, 0]]),
               np.array([0.05, 1e-2, 1e-2, 1e-2])),
    }
    out = {}
    eps, dt = 0.01, 1e-3
    for k, (x, v, m) in cases.items():
        out[k + "_x"], out[k + "_v"], out[k + "_m"] = x, v, m
        out[k + "_a"] = po.ref_force(x, v, m, eps)
        out[k + "_a_exact"] = po.force_exact(x, v, m, eps)
        out[k + "_e"] = np.array([po.ref_initial_energy(x, v, m, eps)])
        x1, v1 = po.ref_run(x, v, m, eps, dt, 1)
        out[k + "_x1"], out[k + "_v1"] = x1, v1
    out["eps"], out["dt"] = np.array([eps]), np.array([dt])
    _save("kat_small.npz", **out)


def case_random():
    rng = np.random.default_rng(20261203)
    n, eps, dt = 1001, 0.02, 1e-3
    x = rng.uniform(-1, 1, (n, 3))
    v = rng.normal(0, 0.3, (n, 3))
    m = rng.uniform(0.5, 1.5, n) / n
    x[0] = rng.normal(0, 0.05, 3)
    v[0] = 0.0
    m[0] = 0.02
    a = po.ref_force(x, v, m, eps)
    e = po.ref_initial_energy(x, v, m, eps)
    x5, v5 = po.ref_run(x, v, m, eps, dt, 5)
    _save("random_1001.npz", x=x, v=v, m=m, a=a, a_exact=po.force_exact(x, v, m, eps),
          e=np.array([e]), x5=x5, v5=v5, eps=np.array([eps]), dt=np.array([dt]))


def case_init10k():
    src = os.path.join(po.reference_dir(), "Init10k-sphere.dat")
    nstars = 2000
    xs = np.zeros((nstars, 3))
    with open(src) as fh:
        for i in range(nstars):
            xs[i] = np.array(fh.readline().split(), dtype=np.float32)
    n = nstars + 1
    x = np.zeros((n, 3))
    x[1:] = xs.astype(np.float32).astype(np.float64)
    v = np.zeros((n, 3))
    m = np.empty(n)
    m[0] = 100.0 / n
    m[1:] = 1.0 / (n - 1)
    eps, dt = 0.001, 1.0 / 131072.0
    a = po.ref_force(x, v, m, eps)
    e = po.ref_initial_energy(x, v, m, eps)
    x10, v10 = po.ref_run(x, v, m, eps, dt, 10)
    _save("init10k_2000.npz", xs=xs.astype(np.float32), a=a, a_exact=po.force_exact(x, v, m, eps),
          e=np.array([e]), x10=x10, v10=v10, eps=np.array([eps]), dt=np.array([dt]))


def case_config1(nsteps=100):
    import pn_gb300 as pn  # host-only IC generator (no GPU needed)
    s = pn.config_uniform_sphere(10000, seed=1, m_star=1e-4, m_bh=0.01, float_rounded=True)
    eps, dt = 0.01, 1e-3
    t0 = time.time()
    a = po.ref_force(s.x, s.v, s.m, eps)
    print("config1 force", time.time() - t0, "s", flush=True)
    e0 = po.ref_initial_energy(s.x, s.v, s.m, eps)
    xT, vT = po.ref_run(s.x, s.v, s.m, eps, dt, nsteps)
    print("config1 run", time.time() - t0, "s", flush=True)
    eT = po.ref_initial_energy(xT, vT, s.m, eps)
    _save("config1.npz", xs=s.x[1:].astype(np.float32), m=s.m, a=a,
          a_exact=po.force_exact(s.x, s.v, s.m, eps), e0=np.array([e0]),
          xT=xT, vT=vT, eT=np.array([eT]), nsteps=np.array([nsteps]), eps=np.array([eps]),
          dt=np.array([dt]))


def case_config1_exact():
    """Adds the long-double force to an existing config1.npz."""
    path = os.path.join(HERE, "config1.npz")
    g = dict(np.load(path))
    n = g["xs"].shape[0] + 1
    x = np.zeros((n, 3))
    x[1:] = g["xs"].astype(np.float64)
    g["a_exact"] = po.force_exact(x, np.zeros((n, 3)), g["m"], float(g["eps"][0]))
    _save("config1.npz", **g)


if __name__ == "__main__":
    po.build(ref=True)
    if not po.ref_available():
        sys.exit("the reference source is not present; golden vectors cannot be regenerated here")
    which = sys.argv[1:] or ["kat", "random", "init10k", "config1"]
    for w in which:
        {"kat": case_kat, "random": case_random, "init10k": case_init10k, "config1": case_config1,
         "config1_exact": case_config1_exact}[w]()
