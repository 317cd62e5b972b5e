"""Benchmark of the Limit-sticky9 force path on GB300: interactions/s of the integration step.

Workload (the configuration the headline metric is quoted on): a Plummer sphere of
N = 262,144 equal-mass stars in Henon units plus a BH of 0.01 x the stellar mass at the origin
at rest (seeded, synthetic), eps = 0.01 * 4 / N^(1/3), dt = 1/1024, c = 1000 (inv_c2 = 1e-6; every
1PN term is evaluated, as small corrections).  A step is one integration step of the reference's scheme
(Limit-sticky9.c:844-893): three force() evaluations and the stage updates.  One interaction
is one Newtonian (i, j) pair, n^2 per force() evaluation (n = N + 1), so a step is 3 n^2
interactions.

  value        mixed precision (FP32 pair terms, FP64 state/O(N) terms), state resident in HBM,
               device time of K steps with CUDA events on the stream the kernels run on; the
               L2 is overwritten (2x its size) before every timed step
  e2e          the same metric through the reference-facing drop-in force() with host arrays,
               as the reference's main loop calls it: per step 3 x (H2D x, v, m; D2H a) and the
               stage updates on the host, wall clock
  fp64         the FP64 path (parity with the reference) on the same workload
  roofline     the pair-sweep kernel against the measured FP32 FMA peak of this GPU
  cpu_baseline the oracle port of the reference (bit-identical to it) on a bounded sample of
               rows of force() on the host cores, scaled to interactions/s

--impl reference times the reference's CPU implementation of the path (the oracle port; the
reference itself cannot be built on the GPU host) on all host cores, a bounded sample per step.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

NSTARS = 262144
SEED = 2026
BH_FRACTION = 0.01
DT = 1.0 / 1024.0
# c = 1000 in these units: the 1PN terms are corrections to the Newtonian force.  (With the
# reference's implicit c = 1 a Hénon-unit Plummer sphere has v/c ~ 1 and its 1PN "corrections"
# are O(1): the energy runs away within a few steps.)  The kernels do the same work for any c.
INV_C2 = 1e-6
METRIC = "interactions/s at N=2^18 (mixed FP32/FP64 integration step)"
UNIT = "interactions/s"


def workload_config(nstars=NSTARS):
    import pn_gb300 as pn
    return {"workload": f"plummer_bh_N{nstars}", "n_particles": nstars + 1,
            "bh_mass_fraction": BH_FRACTION, "eps": pn.plummer_eps(nstars), "dt": DT,
            "inv_c2": INV_C2, "step": "3 force() evaluations + stage updates (Limit-sticky9.c:844-893)",
            "interaction": "one Newtonian (i,j) pair, n^2 per force()",
            "l2": "2x L2 overwritten before each timed step"}


def _measured_hbm_gbs():
    """The HBM copy bandwidth measured on this GPU type, else None."""
    try:
        return float(json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))["hbm_gbs"])
    except (OSError, ValueError, KeyError):
        return None


def dist_init(n_gpus):
    """torchrun env -> (rank, world, torch.distributed or None)."""
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        dist.init_process_group("nccl")
        return rank, world, dist
    return 0, 1, None


def max_over_ranks(val, dist):
    """The slowest rank's time (replicas run independently; the job ends with the last)."""
    if dist is None:
        return val
    import torch
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([val], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(world, steps, units_per_step, slowest_seconds):
    """Whole-job throughput of `world` independent replicas: all units over the slowest time."""
    return world * steps * units_per_step / slowest_seconds


def barrier(dist):
    if dist is not None:
        dist.barrier()


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms while active."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self):
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self, device=0):
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [p.strip() for p in ln.split(",")]
            if len(f) < 9 or not f[0].isdigit() or int(f[0]) != device:
                continue
            try:
                sm.append(float(f[1]))
                mx = max(mx, float(f[2]))
            except ValueError:
                continue
            for nm, val in zip(names, f[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx or None,
                "reasons": sorted(reasons), "samples": len(sm)}


def cpu_baseline(sysm, eps, seconds=12.0, threads=None):
    """The oracle port on a bounded sample of force() rows (all three O(N^2) sweeps of each
    row), timed on the host cores; returns interactions/s and the sample description."""
    from oracle import pyoracle as po
    po.build(ref=False)
    threads = threads or os.cpu_count() or 1
    n = sysm.x.shape[0]
    rng = np.random.default_rng(1)
    rows = np.sort(rng.choice(np.arange(1, n), size=threads * 2, replace=False))
    t = po.time_force_rows(sysm.x, sysm.v, sysm.m, eps, rows, threads)  # calibration
    per_row = t / rows.size * threads
    k = max(threads, int(seconds * threads / max(per_row, 1e-6)))
    k = min(k, n - 1)
    rows = np.sort(rng.choice(np.arange(1, n), size=k, replace=False))
    t = po.time_force_rows(sysm.x, sysm.v, sysm.m, eps, rows, threads)
    rate = rows.size * n / t
    return rate, {"rows": int(rows.size), "seconds": t, "threads": threads,
                  "sample": f"{rows.size} random rows of force() at N={n - 1} (Newtonian row, "
                            f"star cross row and BH cross row each), {threads} threads; "
                            f"interactions = rows x n"}


def run_reference(args, rank, world, dist):
    """--impl reference: the reference's CPU path (oracle port) on all host cores."""
    import pn_gb300 as pn
    if rank != 0:
        return 0
    sysm = pn.config_plummer(NSTARS, SEED, BH_FRACTION)
    eps = pn.plummer_eps(NSTARS)
    threads = os.cpu_count() or 1
    from oracle import pyoracle as po
    po.build(ref=False)
    n = sysm.x.shape[0]
    rng = np.random.default_rng(7)
    rows_per_step = threads * 4
    times = []
    for s in range(args.warmup + args.steps):
        rows = np.sort(rng.choice(np.arange(1, n), size=rows_per_step, replace=False))
        t = po.time_force_rows(sysm.x, sysm.v, sysm.m, eps, rows, threads)
        if s >= args.warmup:
            times.append(t)
    total = sum(times)
    value = args.steps * rows_per_step * n / total
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded Plummer sphere + BH)", "config": workload_config(),
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": f"{rows_per_step} random rows of force() per step "
                                       f"(all three O(N^2) sweeps per row), {threads} threads; "
                                       "the reference source is not on the GPU host, so the "
                                       "bit-identical C port of it runs"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def run_ensemble(args):
    """Configuration 4: 256 Plummer + BH clusters, N log-uniform in [1024, 65536], BH mass
    fraction log-uniform in [1e-3, 1e-1], eps = 0.01, dt = 1/1024, mixed precision, one
    persistent pair launch per force evaluation, each step one CUDA graph.  Times K steps
    (interactions/s = sum n_c^2 per evaluation, 3 per step) and checks a subset of clusters
    against individual FP64 runs."""
    import pn_gb300 as pn
    rng = np.random.default_rng(4)
    nc = args.clusters
    sizes = np.exp(rng.uniform(np.log(1024), np.log(65536), nc)).astype(int)
    fracs = np.exp(rng.uniform(np.log(1e-3), np.log(1e-1), nc))
    systems = [pn.config_plummer(int(s), 1000 + k, float(f)) for k, (s, f) in enumerate(zip(sizes, fracs))]
    eps = [0.01] * nc
    inter = 3.0 * sum(float(s.x.shape[0]) ** 2 for s in systems)
    e = pn.Ensemble(systems, eps, dt=DT, inv_c2=INV_C2, precision=pn.PN_PREC_MIXED)
    t0 = time.perf_counter()
    e.autotune()
    tune_s = time.perf_counter() - t0
    e.bench_steps(args.warmup)
    with ClockSampler() as clk:
        ms = e.bench_steps(args.steps)
    total = float(ms.sum())
    # cluster-by-cluster check: the ensemble (mixed) after the warm-up and timed steps against
    # individual FP64 contexts run for the same number of steps
    nsteps = args.warmup + args.steps
    xs, vs = e.get_state()
    e.close()
    picks = sorted(set([int(np.argmin(sizes)), int(np.argmax(sizes))] + list(rng.choice(nc, 4, replace=False))))
    errs = {}
    for k in picks:
        s = systems[k]
        with pn.Context(s.x.shape[0], eps=eps[k], dt=DT, inv_c2=INV_C2) as c:
            c.set_state(s.x, s.v, s.m)
            c.steps(nsteps)
            xr, vr = c.get_state()
        errs[str(k)] = {"n": int(s.x.shape[0]),
                        "max_pos_err_rel": float(np.abs(xs[k] - xr).max() / np.abs(xr).max()),
                        "max_vel_err_rel": float(np.abs(vs[k] - vr).max() / np.abs(vr).max())}
    line = {"metric": "interactions/s, ensemble of 256 clusters (persistent launch, CUDA graph steps)",
            "value": args.steps * inter / (total * 1e-3), "unit": UNIT, "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
            "config": {"workload": f"ensemble_{nc}_plummer_bh", "n_range": [int(sizes.min()), int(sizes.max())],
                       "particles": int(sum(s.x.shape[0] for s in systems)), "eps": 0.01, "dt": DT,
                       "inv_c2": INV_C2, "autotune_s": tune_s},
            "clocks": clk.summary(), "check_vs_individual_fp64": errs}
    print(json.dumps(line), flush=True)
    return 0


def run_adjoint(args):
    """Configuration 5: N = 16384 Plummer + BH (mass fraction 0.05), 200 steps at dt = 1/1024.
    Loss: squared distance of the final snapshot (x, v) to a target made with the BH mass x 1.1
    and initial positions + N(0, 1e-3^2).  Reports the cost of the adjoint per step against a
    forward step (mixed and FP64) with checkpoints every 20 steps (segments recomputed) and with
    every stage kept (checkpoint interval = steps, no recomputation: 1.2 GB of HBM here).
    The FP64 gradient is checked against central differences (h = 1e-6) on sampled coordinates
    and the BH mass over --fd-steps steps: over 200 steps at this dt the close BH passages make
    the loss too nonlinear in the inputs for any step h to converge (h = 1e-4 .. 1e-7 disagree
    with each other by more than 100 %), over 40 steps the differences converge to the adjoint
    (~1e-9 at h = 1e-6).  The mixed-precision gradient is compared with the FP64 one."""
    import pn_gb300 as pn
    ns, nsteps = args.adj_n, args.adj_steps
    s = pn.config_plummer(ns, 77, 0.05)
    eps = pn.plummer_eps(ns)
    rng = np.random.default_rng(5)
    n = ns + 1

    def final(x, v, m, steps, prec=0):
        with pn.Context(n, eps=eps, dt=DT, inv_c2=INV_C2, precision=prec) as c:
            c.set_state(x, v, m)
            c.steps(steps)
            return c.get_state()

    mt = s.m.copy()
    mt[0] *= 1.1
    xt0 = s.x + rng.normal(0, 1e-3, s.x.shape)
    xt0[0] = s.x[0]

    def gradient(c, steps, K, xT, vT):
        c.set_state(s.x, s.v, s.m)
        c.adjoint_forward(steps, K)
        xe, ve = c.get_state()
        t0 = time.perf_counter()
        g = c.adjoint_backward(2 * (xe - xT), 2 * (ve - vT))
        return g, (time.perf_counter() - t0) / steps

    xT, vT = final(xt0, s.v, mt, nsteps)
    timing = {}
    for prec in (1, 0):
        with pn.Context(n, eps=eps, dt=DT, inv_c2=INV_C2, precision=prec) as c:
            c.set_state(s.x, s.v, s.m)
            c.steps(2)  # warm-up (graph, kernels)
            c.set_state(s.x, s.v, s.m)
            t0 = time.perf_counter()
            c.steps(nsteps)
            fwd = (time.perf_counter() - t0) / nsteps
            r = {"fwd_ms_per_step": fwd * 1e3}
            for K in (20, nsteps):
                _, bwd = gradient(c, nsteps, K, xT, vT)
                r[f"adj_ms_per_step_K{K}"] = bwd * 1e3
                r[f"ratio_K{K}"] = bwd / fwd
            timing["mixed" if prec else "fp64"] = r
    # finite-difference check (FP64) over fd_steps steps
    fs = args.fd_steps
    xTf, vTf = final(xt0, s.v, mt, fs)

    def loss(x, v, m):
        xe, ve = final(x, v, m, fs)
        return float(((xe - xTf) ** 2).sum() + ((ve - vTf) ** 2).sum())

    grads = {}
    for prec in (0, 1):
        with pn.Context(n, eps=eps, dt=DT, inv_c2=INV_C2, precision=prec) as c:
            grads[prec], _ = gradient(c, fs, 20, xTf, vTf)
    gx, gv, gm = grads[0]
    h = 1e-6
    checks = []
    for q in rng.choice(np.arange(3, 6 * n), args.fd_coords, replace=False):
        which, r_ = divmod(int(q), 3 * n)
        p_, k = divmod(r_, 3)
        if p_ == 0:
            continue
        a = (s.x if which == 0 else s.v).copy()
        b = a.copy()
        a[p_, k] += h
        b[p_, k] -= h
        lp = loss(a, s.v, s.m) if which == 0 else loss(s.x, a, s.m)
        lm = loss(b, s.v, s.m) if which == 0 else loss(s.x, b, s.m)
        fd = (lp - lm) / (2 * h)
        g = (gx if which == 0 else gv)[p_, k]
        checks.append(abs(g - fd) / max(abs(fd), 1e-300))
    mp, mm = s.m.copy(), s.m.copy()
    mp[0] += h
    mm[0] -= h
    fdm = (loss(s.x, s.v, mp) - loss(s.x, s.v, mm)) / (2 * h)
    gx1, gv1, gm1 = grads[1]
    dmix = np.sqrt((np.linalg.norm(gx1 - gx) ** 2 + np.linalg.norm(gv1 - gv) ** 2) /
                   (np.linalg.norm(gx) ** 2 + np.linalg.norm(gv) ** 2))
    line = {"metric": f"adjoint backward cost per step / forward step (N={ns}, {nsteps} steps, mixed, "
                      f"every stage kept in HBM)",
            "value": timing["mixed"][f"ratio_K{nsteps}"], "unit": "ratio", "n_gpus": 1, "steps": nsteps,
            "warmup": 2, "higher_is_better": False, "dtype": "f32+f64", "data": "synthetic",
            "config": {"workload": f"plummer_bh_N{ns}_adjoint", "bh_mass_fraction": 0.05, "dt": DT,
                       "checkpoint_every": nsteps, "also_timed_checkpoint_every": 20, "inv_c2": INV_C2},
            "timing": timing,
            "fd_check_fp64": {"steps": fs, "h": h, "coords": len(checks), "max_rel_err": float(max(checks)),
                              "median_rel_err": float(np.median(checks)),
                              "bh_mass_rel_err": float(abs(gm - fdm) / abs(fdm))},
            "mixed_vs_fp64_grad_rel": float(dmix), "mixed_vs_fp64_dm0_rel": float(abs(gm1 / gm - 1))}
    print(json.dumps(line), flush=True)
    return 0


def run_long(args, nstars, precisions, nsteps_by_prec, label):
    """Energy drift and step throughput of device-resident runs (one JSON line)."""
    import pn_gb300 as pn
    s = pn.config_plummer(nstars, SEED, BH_FRACTION)
    eps = pn.plummer_eps(nstars)
    n = nstars + 1
    res = {}
    for prec in precisions:
        with pn.Context(n, eps=eps, dt=DT, inv_c2=INV_C2, precision=0) as c:
            c.set_state(s.x, s.v, s.m)
            e0 = c.energy()[3]  # energies in FP64 for both modes
            k = nsteps_by_prec[prec]
            chunks = [k // 5 + (1 if q < k % 5 else 0) for q in range(5)]
            ms, curve, done = [], [], 0
            with ClockSampler() as clk:
                for kc in chunks:
                    if kc == 0:
                        continue
                    c.set_params(precision=prec)
                    ms.append(c.bench_steps(kc, flush_l2=False)[0])
                    done += kc
                    c.set_params(precision=0)
                    curve.append((done, float(c.energy()[3] / e0 - 1)))
            ms = np.concatenate(ms)
            res["mixed" if prec else "fp64"] = {
                "steps": k, "ms_per_step": float(ms.mean()), "value": 3.0 * n * n / (ms.mean() * 1e-3),
                "energy_drift": curve[-1][1], "drift_curve": curve, "clocks": clk.summary()}
    line = {"metric": label, "unit": UNIT, "n_gpus": 1, "data": "synthetic",
            "config": dict(workload_config(nstars), dt=DT), **res}
    print(json.dumps(line), flush=True)
    return 0


def profile_case(nstars, shape=None):
    """One mixed-precision force evaluation of the bench workload at nstars (ncu target);
    shape = "ipt,tile_j,grid_split" pins the packed sweep's launch shape (e.g. the tuned one)."""
    import pn_gb300 as pn
    sysm = pn.config_plummer(nstars, SEED, BH_FRACTION)
    kw = {}
    if shape:
        ipt, tj, gs = (int(t) for t in shape.split(","))
        kw = dict(i_per_thread=ipt, tile_j=tj, grid_split=gs, pair_variant=2)
    with pn.Context(nstars + 1, eps=pn.plummer_eps(nstars), inv_c2=INV_C2,
                    precision=pn.PN_PREC_MIXED, **kw) as c:
        c.set_state(sysm.x, sysm.v, sysm.m)
        c.force()
        st = c.stats()
        print(json.dumps({"profile_case": nstars, "pair_ms": st.pair_ms, "tile_j": st.tile_j,
                          "i_per_thread": st.i_per_thread, "j_split": st.j_split,
                          "grid_split": st.grid_split, "pair_variant": st.pair_variant}))
    return 0


def host_stage_step(pn, x, v, m, eps, dt):
    """The reference main loop's step around the drop-in force() (Limit-sticky9.c:844-893)."""
    a = pn.force(x, v, m, eps)
    x1 = x + 0.5 * v * dt
    v1 = v + 0.5 * a * dt
    h = x1.copy()
    hv = v1.copy()
    a = pn.force(x1, v1, m, eps)
    x1 = x + 0.5 * v1 * dt
    v1 = v + 0.5 * a * dt
    h += x1
    hv += v1
    a = pn.force(x1, v1, m, eps)
    x3 = x + v1 * dt
    v3 = v + a * dt
    return (x + x3 + 2.0 * h) / 6.0, (v + v3 + 2.0 * hv) / 6.0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=8)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="pn", choices=["pn", "reference"])
    ap.add_argument("--nstars", type=int, default=NSTARS)
    ap.add_argument("--quick", action="store_true", help="skip the FP64, accuracy and CPU legs")
    ap.add_argument("--profile-case", type=int, default=0, metavar="N",
                    help="set up N stars, tune, run one mixed force evaluation and exit (for ncu)")
    ap.add_argument("--ensemble", action="store_true", help="configuration 4 (ensemble) instead")
    ap.add_argument("--clusters", type=int, default=256)
    ap.add_argument("--adjoint", action="store_true", help="configuration 5 (adjoint) instead")
    ap.add_argument("--adj-n", type=int, default=16384)
    ap.add_argument("--adj-steps", type=int, default=200)
    ap.add_argument("--fd-coords", type=int, default=8)
    ap.add_argument("--fd-steps", type=int, default=40)
    ap.add_argument("--shape", default=None, help="--profile-case launch shape: ipt,tile_j,grid_split")
    ap.add_argument("--fp64-run", type=int, default=0, metavar="STEPS",
                    help="Plummer run at N=65536, FP64 and mixed, STEPS steps each (throughput, energy drift)")
    ap.add_argument("--drift", type=int, default=0, metavar="STEPS",
                    help="energy drift of the headline workload, mixed and FP64, STEPS steps each")
    ap.add_argument("--long-mixed", type=int, default=0, metavar="STEPS",
                    help="energy drift of the headline workload in mixed precision over STEPS steps")
    args = ap.parse_args()
    if args.fp64_run:
        return run_long(args, 65536, (0, 1), {0: args.fp64_run, 1: args.fp64_run},
                        "integration at N=65536, FP64 and mixed (interactions/s, energy drift)")
    if args.drift:
        return run_long(args, args.nstars, (1, 0), {1: args.drift, 0: args.drift},
                        "energy drift, mixed vs FP64 (interactions/s per mode)")
    if args.long_mixed:
        return run_long(args, args.nstars, (1,), {1: args.long_mixed},
                        "energy drift of the mixed-precision integration (interactions/s)")
    if args.profile_case:
        return profile_case(args.profile_case, args.shape)
    if args.ensemble:
        return run_ensemble(args)
    if args.adjoint:
        return run_adjoint(args)
    rank, world, dist = dist_init(args.gpus)
    if args.impl == "reference":
        return run_reference(args, rank, world, dist)

    import pn_gb300 as pn
    from pn_gb300 import build as b
    if not os.path.exists(pn.LIB_PATH):
        b.build()
    ns = args.nstars
    n = ns + 1
    sysm = pn.config_plummer(ns, SEED + rank, BH_FRACTION)
    eps = pn.plummer_eps(ns)
    out = {}

    # ---------------- mixed precision, device resident (value)
    ctx = pn.Context(n, eps=eps, dt=DT, inv_c2=INV_C2, precision=pn.PN_PREC_MIXED)
    ctx.set_state(sysm.x, sysm.v, sysm.m)
    ctx.autotune(1)  # setup: launch shape of the pair sweep for this size (not timed)
    ctx.bench_steps(args.warmup, flush_l2=True)
    barrier(dist)
    with ClockSampler() as clk:
        t0 = time.perf_counter()
        step_ms, pair_ms = ctx.bench_steps(args.steps, flush_l2=True)
        wall = time.perf_counter() - t0
    barrier(dist)
    st = ctx.stats()
    total_ms = max_over_ranks(float(step_ms.sum()), dist)
    inter_step = 3.0 * n * n
    value = replica_throughput(world, args.steps, inter_step, total_ms * 1e-3)
    ms_per_step = total_ms / args.steps
    pair_launch_ms = float(pair_ms.mean()) / 3.0
    ctx.close()

    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64",
            "data": "synthetic (seeded Plummer sphere + BH)",
            "config": dict(workload_config(ns), parallelism=f"replicas{world}" if world > 1 else "1 GPU",
                           pair_kernel={"tile_j": st.tile_j, "i_per_thread": st.i_per_thread,
                                        "j_split": st.j_split, "grid_split": st.grid_split,
                                        "threads": st.threads}),
            "gpu_launches": 9 * args.steps,
            "clocks": clk.summary(int(os.environ.get("LOCAL_RANK", "0")))}

    # roofline of the pair sweep against the measured FP32 FMA peak
    if rank == 0:
        flops_pair = pn.flops_per_pair(1, pn.PN_PREC_MIXED, st.pair_variant)
        peak32 = pn.probe_fma_peak(pn.PN_PREC_MIXED)
        pairs = float(ns) * float(ns)
        achieved = pairs * flops_pair / (pair_launch_ms * 1e-3) / 1e12
        kname = "k_pair2<MODE_FORCE> (packed f32x2)" if st.pair_variant == 2 else "k_pair<float, MODE_FORCE>"
        line["roofline"] = {"bound": "fp32", "kernel": kname,
                            "achieved": achieved, "peak": peak32, "unit": "TFLOP/s",
                            "frac": achieved / peak32, "traffic": None,
                            "flops_per_pair": flops_pair,
                            "pair_launch_ms": pair_launch_ms,
                            "peak_source": "measured FP32 FMA throughput of this GPU (pn_probe_fma_peak)",
                            "pair_interactions_per_s": pairs / (pair_launch_ms * 1e-3)}
        prof = os.path.join(ROOT, "profiles", "pair_sweep_traffic.json")
        if os.path.exists(prof) and ns == NSTARS and st.pair_variant == 2:
            try:  # DRAM bytes of one launch at this size and shape, from an ncu capture
                pt = json.load(open(prof))
                line["roofline"]["traffic"] = pt.get("k_pair2_force_f32_N262144_bytes_per_launch")
                line["roofline"]["traffic_shape"] = pt.get("k_pair2_force_f32_N262144_shape")
                line["roofline"]["ncu_fma_pipe_active_pct"] = pt.get("fma_pipe_active_pct_N65536")
            except (OSError, ValueError):
                pass

        # the O(N) kernels (k_prep + k_finish with the fused stage update) per evaluation: the
        # step's time outside the three pair sweeps, against the measured HBM copy bandwidth
        on_ms = max(float(step_ms.mean()) - float(pair_ms.mean()), 0.0) / 3.0
        gs = st.grid_split
        moved = 216 + 56 + 72 * gs + 168  # prep in/out; finish: per-star data, split sums, stage state
        algo = 104 + 144                  # BH-star O(N) terms + one stage update, per star
        peak_hbm = _measured_hbm_gbs()
        line["o_n_kernels"] = {"ms_per_evaluation": on_ms, "bytes_per_star_moved": moved,
                               "bytes_per_star_algorithmic": algo,
                               "moved_gbs": ns * moved / (on_ms * 1e-3) / 1e9 if on_ms > 0 else None,
                               "algorithmic_gbs": ns * algo / (on_ms * 1e-3) / 1e9 if on_ms > 0 else None,
                               "peak_gbs": peak_hbm, "peak_source": "MEASURED_PEAKS.json hbm_gbs"}

    # ---------------- e2e through the drop-in force() with host arrays
    pn.configure(pn.PN_PREC_MIXED, INV_C2)
    x, v = sysm.x.copy(), sysm.v.copy()
    x, v = host_stage_step(pn, x, v, sysm.m, eps, DT)  # warm-up
    e2e_steps = max(1, min(args.steps, 3))
    barrier(dist)
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        x, v = host_stage_step(pn, x, v, sysm.m, eps, DT)
    e2e_s = max_over_ranks(time.perf_counter() - t0, dist)
    pn.configure(pn.PN_PREC_FP64, INV_C2)
    pn.lib().pn_dropin_release()
    line["e2e"] = {"value": replica_throughput(world, e2e_steps, inter_step, e2e_s), "unit": UNIT,
                   "h2d_bytes_per_step": 3 * (2 * 24 + 8) * n, "d2h_bytes_per_step": 3 * 24 * n,
                   "path": "drop-in force() x3 per step with host arrays + host stage updates"}
    line["gpu_launches"] += 9 * e2e_steps

    if rank == 0 and not args.quick:
        # ---------------- FP64 path on the same workload (one step) and mixed accuracy
        c64 = pn.Context(n, eps=eps, dt=DT, inv_c2=INV_C2, precision=pn.PN_PREC_FP64)
        c64.set_state(sysm.x, sysm.v, sysm.m)
        a64 = c64.force()
        sm64, pm64 = c64.bench_steps(1, flush_l2=True)
        c64.close()
        line["fp64"] = {"value": inter_step / (sm64[0] * 1e-3), "unit": UNIT,
                        "ms_per_step": float(sm64[0]),
                        "peak_fp64_tflops": pn.probe_fma_peak(pn.PN_PREC_FP64),
                        "pair_tflops": float(ns) * ns * pn.flops_per_pair(1, 0) / (pm64[0] / 3 * 1e-3) / 1e12}
        line["mixed_over_fp64"] = value / world / line["fp64"]["value"]
        acc = {}
        for ic2 in (INV_C2, 1.0):
            cm = pn.Context(n, eps=eps, inv_c2=ic2, precision=pn.PN_PREC_MIXED)
            cm.set_state(sysm.x, sysm.v, sysm.m)
            a32 = cm.force()
            cm.close()
            if ic2 != INV_C2:
                cd = pn.Context(n, eps=eps, inv_c2=ic2, precision=pn.PN_PREC_FP64)
                cd.set_state(sysm.x, sysm.v, sysm.m)
                ref = cd.force()
                cd.close()
            else:
                ref = a64
            d = np.linalg.norm(a32 - ref, axis=1)
            r = d / np.linalg.norm(ref, axis=1)
            acc[f"inv_c2={ic2:g}"] = {
                "rms_rel": float(np.sqrt((r ** 2).mean())), "max_rel": float(r.max()),
                "rms_abs_over_rms_a": float(np.sqrt((d ** 2).mean() / (np.linalg.norm(ref, axis=1) ** 2).mean()))}
        line["accuracy_vs_fp64"] = acc
        # ---------------- CPU baseline (oracle port), bounded sample
        rate, info = cpu_baseline(sysm, eps)
        rate1, info1 = cpu_baseline(sysm, eps, seconds=4.0, threads=1)  # the reference runs on one core
        line["cpu_baseline"] = {"value": rate, "unit": UNIT, "cores": info["threads"], "kind": "port",
                                "sample": info["sample"], "seconds": info["seconds"],
                                "single_core_value": rate1, "single_core_sample": info1["sample"]}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
