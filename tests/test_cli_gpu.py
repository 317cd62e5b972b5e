"""pn_run, the command-line equivalent of the reference's main (Limit-sticky9.c:740-920): its
input and snapshot formats, its printed lines and its trajectory (against the oracle), and
resuming from a binary checkpoint."""
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT

pytestmark = pytest.mark.gpu

EXE = os.path.join(ROOT, "pn_gb300", "_lib", "pn_run")


def _run(args, cwd):
    r = subprocess.run([EXE] + args, capture_output=True, text=True, cwd=cwd, timeout=600)
    assert r.returncode == 0, r.stderr
    return r.stdout


def _read_blocks(path, n):
    vals = np.loadtxt(path)
    assert vals.shape[0] % (2 * n) == 0
    return vals.reshape(-1, 2, n, 3)  # [snapshot][x|v][particle][k]


def test_main_loop_equivalent(pn, oracle, tmp_path):
    # a cold shell 1 <= r <= 5 (the reference's own input is a cold shell 1 <= r <= 10); the
    # reference's mass rule m0 = 100/n makes the BH heavy at small n, so stars stay away from it
    nstars, eps, dt = 100, 0.01, 1e-3
    u, _ = pn.uniform_sphere(nstars, 1.0, 9)
    r = np.linalg.norm(u, axis=1, keepdims=True)
    xs = u / r * (1.0 + 4.0 * r)
    vs = np.zeros_like(xs)
    pn.write_init(str(tmp_path / "init.dat"), xs, vs)
    out = _run(["--input", "init.dat", "--output", "snap.dat", "-n", str(nstars + 1), "--eps", str(eps),
                "--dt", str(dt), "--endtime", "0.01", "--deouttime", "0.005"], tmp_path)
    lines = out.splitlines()
    assert lines[0].strip() == "Init" and lines[1].strip() == "start"
    assert lines[2] == "time = 0" and lines[3].startswith("pot = ")
    assert sum(ln.startswith(" DE = ") for ln in lines) == 2
    assert abs(float(lines[-1]) - 0.01) < 1e-12
    snaps = _read_blocks(tmp_path / "snap.dat", nstars + 1)
    assert snaps.shape[0] == 4  # initial, t = 0.005, t = 0.01, final (Limit-sticky9.c:820-916)
    # the oracle from the same (float-rounded) input and the reference's mass rule
    x0, v0 = pn.read_init(str(tmp_path / "init.dat"), nstars)
    n = nstars + 1
    x = np.zeros((n, 3)); v = np.zeros((n, 3))
    x[1:], v[1:] = x0, v0
    m = np.empty(n); m[0] = 100.0 / n; m[1:] = 1.0 / (n - 1)
    xo, vo = oracle.run(x, v, m, eps, dt, 10)
    assert np.isfinite(xo).all() and np.abs(xo).max() < 10  # a physical run
    # snapshots carry 6 decimals ("%lf", Limit-sticky9.c:900-905)
    assert np.abs(snaps[-1, 0] - xo).max() <= 1e-6 and np.abs(snaps[-1, 1] - vo).max() <= 1e-6


def test_checkpoint_resume(pn, tmp_path):
    nstars = 60
    xs, _ = pn.uniform_sphere(nstars, 1.0, 3)
    pn.write_init(str(tmp_path / "init.dat"), xs, np.zeros_like(xs))
    common = ["--input", "init.dat", "-n", str(nstars + 1), "--eps", "0.02", "--dt", "0.001",
              "--deouttime", "0.004", "--lossless"]
    _run(common + ["--output", "full.dat", "--endtime", "0.012"], tmp_path)
    _run(common + ["--output", "a.dat", "--endtime", "0.008", "--checkpoint", "ck.bin"], tmp_path)
    _run(common + ["--output", "b.dat", "--endtime", "0.012", "--resume", "ck.bin"], tmp_path)
    full = _read_blocks(tmp_path / "full.dat", nstars + 1)
    resumed = _read_blocks(tmp_path / "b.dat", nstars + 1)
    assert np.array_equal(full[-1], resumed[-1])  # lossless snapshots, identical arithmetic
