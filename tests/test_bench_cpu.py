"""The benchmark's CPU pieces, run here without a GPU: the reference arm (the oracle port on one
core) loads no part of libpn and prints the same workload config as the GPU arm, and the
oracle's Plummer sampler draws the same distribution as libpn's generator."""
import json
import os
import subprocess
import sys

import numpy as np

from conftest import ROOT


def test_reference_arm_loads_no_libpn():
    code = (
        "import sys, json, argparse; sys.path.insert(0, %r); import bench;"
        "a = argparse.Namespace(steps=1, warmup=0); bench.run_reference(a, 0, 1);"
        "maps = open('/proc/self/maps').read();"
        "print(json.dumps({'pn_gb300': 'pn_gb300' in sys.modules, 'libpn': 'libpn.so' in maps}))" % ROOT)
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr
    lines = [json.loads(ln) for ln in r.stdout.strip().splitlines()]
    line, probe = lines[-2], lines[-1]
    assert probe == {"pn_gb300": False, "libpn": False}
    sys.path.insert(0, ROOT)
    import bench
    assert line["impl"] == "reference" and line["config"] == bench.workload_config()
    assert line["cpu_baseline"]["cores"] == 1 and line["value"] > 0
    assert line["e2e"]["h2d_bytes_per_step"] == 0


def test_oracle_plummer_sampler_matches_libpn_distribution(pn, oracle):
    n = 65536
    x, v, m = oracle.plummer_bh(n, 3, 0.01)
    s = pn.config_plummer(n, 3, 0.01)
    assert x.shape == s.x.shape and m[0] == s.m[0] and np.allclose(m[1:], s.m[1:])
    assert (x[0] == 0).all() and (v[0] == 0).all()
    for a, b in ((x, s.x), (v, s.v)):
        ra, rb = np.linalg.norm(a[1:], axis=1), np.linalg.norm(b[1:], axis=1)
        for q in (0.1, 0.5, 0.9):  # radial / speed quantiles agree to sampling noise
            assert abs(np.quantile(ra, q) / np.quantile(rb, q) - 1) < 0.04
        assert np.abs(a[1:].mean(axis=0)).max() < 1e-12  # centre-of-mass frame
    kin = 0.5 * (m[1:] * (v[1:] ** 2).sum(axis=1)).sum()
    assert abs(kin - 0.25) < 0.01  # Henon units: kinetic energy = -E = 1/4 (virial)
