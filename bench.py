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

On one GPU the same JSON line also carries the other configurations of the workload set, each
run within a share of a wall-clock budget (--budget-s, default 25 min for the whole command;
a leg that would overrun stops early and says how far it got):

  config4      256 clusters, N log-uniform in [1024, 65536], in one persistent launch per force
               evaluation (mixed), K timed steps; clusters checked against individual FP64 runs
  config5      the discrete adjoint at N = 16,384 over 200 steps: backward cost per step over a
               forward step with checkpoints every 20 steps and with every stage kept, mixed and
               FP64; the FP64 gradient against central differences (h = 1e-6) on 64 coordinates
               and the BH mass, with a Richardson pair (h/2) on the worst ones
  config2      N = 65,536 Plummer + BH, 500 steps in FP64 and in mixed precision: throughput and
               the two energy-drift curves (every 50 steps)

--impl reference times the reference's CPU implementation of the path (the oracle port; the
reference itself cannot be built on the GPU host) on one core, as the reference runs.
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
T_START = time.monotonic()


class Budget:
    """Wall-clock budget of the whole command (seconds from process start)."""

    def __init__(self, seconds):
        self.end = T_START + seconds

    def left(self):
        return self.end - time.monotonic()


def plummer_eps(nstars):
    """Softening 0.01 * 4 / N^(1/3) of the Plummer configurations."""
    return 0.01 * 4.0 / nstars ** (1.0 / 3.0)


def workload_config(nstars=NSTARS, world=1):
    """The workload both arms time (the same keys and values in both lines)."""
    return {"workload": f"plummer_bh_N{nstars}", "n_particles": nstars + 1,
            "bh_mass_fraction": BH_FRACTION, "eps": plummer_eps(nstars), "dt": DT,
            "inv_c2": INV_C2, "step": "3 force() evaluations + stage updates (Limit-sticky9.c:844-893)",
            "interaction": "one Newtonian (i,j) pair, n^2 per force()",
            "l2": "2x L2 overwritten before each timed step",
            "parallelism": f"replicas{world}" if world > 1 else "1 GPU"}


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


def cpu_baseline(x, v, m, eps, seconds=12.0, threads=None):
    """The oracle port on a bounded sample of force() rows (all three O(N^2) sweeps of each
    row), timed on the host cores; returns interactions/s and the sample description."""
    from oracle import pyoracle as po
    po.build(ref=False)
    threads = threads or os.cpu_count() or 1
    n = x.shape[0]
    rng = np.random.default_rng(1)
    rows = np.sort(rng.choice(np.arange(1, n), size=threads * 2, replace=False))
    t = po.time_force_rows(x, v, m, eps, rows, threads)  # calibration
    per_row = t / rows.size * threads
    k = max(threads, int(seconds * threads / max(per_row, 1e-6)))
    k = min(k, n - 1)
    rows = np.sort(rng.choice(np.arange(1, n), size=k, replace=False))
    t = po.time_force_rows(x, v, m, eps, rows, threads)
    rate = rows.size * n / t
    return rate, {"rows": int(rows.size), "seconds": t, "threads": threads,
                  "sample": f"{rows.size} random rows of force() at N={n - 1} (Newtonian row, "
                            f"star cross row and BH cross row each), {threads} threads; "
                            f"interactions = rows x n"}


def run_reference(args, rank, world):
    """--impl reference: the reference's CPU implementation of the path (the oracle port,
    bit-identical to Limit-sticky9.c's force(); the reference source is not on the GPU host) on
    this host's cores.  The reference is single-threaded as shipped (its OpenMP pragma is
    commented out, Limit-sticky9.c:34), so `value` is one core; the same sample on every host
    thread is reported beside it.  The input is the same Plummer + BH workload, sampled by the
    oracle's own numpy generator: this arm loads no part of libpn."""
    if rank != 0:
        return 0
    from oracle import pyoracle as po
    po.build(ref=False)
    x, v, m = po.plummer_bh(NSTARS, SEED, BH_FRACTION)
    eps = plummer_eps(NSTARS)
    n = x.shape[0]
    rng = np.random.default_rng(7)
    # rows per step: about 0.25 s of one core (calibrated on a few rows)
    t = po.time_force_rows(x, v, m, eps, np.sort(rng.choice(np.arange(1, n), 4, replace=False)), 1)
    rows_per_step = int(min(max(2, 0.25 / max(t / 4, 1e-6)), 4096))
    times = []
    for s_ in range(args.warmup + args.steps):
        rows = np.sort(rng.choice(np.arange(1, n), size=rows_per_step, replace=False))
        t = po.time_force_rows(x, v, m, eps, rows, 1)
        if s_ >= args.warmup:
            times.append(t)
    total = sum(times)
    value = args.steps * rows_per_step * n / total
    threads = os.cpu_count() or 1
    rows = np.sort(rng.choice(np.arange(1, n), size=min(n - 1, rows_per_step * threads * 4), replace=False))
    t_all = po.time_force_rows(x, v, m, eps, rows, threads)
    sample = (f"{rows_per_step} random rows of force() per step (all three O(N^2) sweeps per row, "
              f"n interactions each), 1 thread as the reference runs; the reference source is not "
              f"on the GPU host, so the bit-identical C port of it runs")
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded Plummer sphere + BH)", "config": workload_config(NSTARS, world),
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": 1, "kind": "port", "sample": sample,
                             "all_threads_value": rows.size * n / t_all, "all_threads": threads},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------------------- configuration 4
def ensemble_leg(steps, warmup, nclusters, allowance):
    """256 Plummer + BH clusters, N log-uniform in [1024, 65536], BH mass fraction log-uniform in
    [1e-3, 1e-1], eps = 0.01, dt = 1/1024, mixed precision, one persistent pair launch per force
    evaluation, each step one CUDA graph.  Times `steps` steps (interactions/s = sum n_c^2 per
    evaluation, 3 per step) and checks clusters (the smallest, the largest and random ones)
    against individual FP64 runs of the same number of steps."""
    import pn_gb300 as pn
    t_leg = time.monotonic()
    rng = np.random.default_rng(4)
    nc = nclusters
    sizes = np.exp(rng.uniform(np.log(1024), np.log(65536), nc)).astype(int)
    fracs = np.exp(rng.uniform(np.log(1e-3), np.log(1e-1), nc))
    systems = [pn.config_plummer(int(s), 1000 + k, float(f)) for k, (s, f) in enumerate(zip(sizes, fracs))]
    eps = [0.01] * nc
    inter = 3.0 * sum(float(s.x.shape[0]) ** 2 for s in systems)
    e = pn.Ensemble(systems, eps, dt=DT, inv_c2=INV_C2, precision=pn.PN_PREC_MIXED)
    t0 = time.perf_counter()
    e.autotune()
    tune_s = time.perf_counter() - t0
    e.bench_steps(warmup)
    with ClockSampler() as clk:
        ms = e.bench_steps(steps)
    total = float(ms.sum())
    nsteps = warmup + steps
    xs, vs = e.get_state()
    e.close()
    picks = [int(np.argmin(sizes)), int(np.argmax(sizes))]
    picks += [int(k) for k in rng.choice(nc, 6, replace=False) if int(k) not in picks]
    errs, skipped = {}, []
    for k in picks:
        s = systems[k]
        # an individual FP64 run costs ~n^2 / 1.1e10 s per evaluation on this GPU
        est = 3.0 * nsteps * float(s.x.shape[0]) ** 2 / 1.0e10
        if time.monotonic() - t_leg + est > allowance:
            skipped.append(k)
            continue
        with pn.Context(s.x.shape[0], eps=eps[k], dt=DT, inv_c2=INV_C2) as c:
            c.set_state(s.x, s.v, s.m)
            c.steps(nsteps)
            xr, vr = c.get_state()
        errs[str(k)] = {"n": int(s.x.shape[0]), "bh_fraction": float(fracs[k]),
                        "max_pos_err_rel": float(np.abs(xs[k] - xr).max() / np.abs(xr).max()),
                        "max_vel_err_rel": float(np.abs(vs[k] - vr).max() / np.abs(vr).max())}
    return {"metric": f"interactions/s, ensemble of {nc} clusters (persistent launch, CUDA graph steps)",
            "value": steps * inter / (total * 1e-3), "unit": UNIT, "steps": steps, "warmup": warmup,
            "ms_per_step": total / steps, "dtype": "f32+f64", "gpu_launches": 3 * 3 * steps,
            "config": {"workload": f"ensemble_{nc}_plummer_bh", "n_range": [int(sizes.min()), int(sizes.max())],
                       "particles": int(sum(s.x.shape[0] for s in systems)), "eps": 0.01, "dt": DT,
                       "inv_c2": INV_C2, "autotune_s": tune_s},
            "clocks": clk.summary(),
            "check_vs_individual_fp64": {"steps": nsteps, "clusters": errs, "skipped_for_time": skipped,
                                         "max_pos_err_rel": max((v["max_pos_err_rel"] for v in errs.values()), default=None),
                                         "max_vel_err_rel": max((v["max_vel_err_rel"] for v in errs.values()), default=None)},
            "seconds": time.monotonic() - t_leg}


# ---------------------------------------------------------------------------- configuration 5
def adjoint_leg(ns, nsteps, fd_steps, fd_coords, allowance, richardson=6):
    """N = 16384 Plummer + BH (mass fraction 0.05), 200 steps at dt = 1/1024.  Loss: squared
    distance of the final snapshot (x, v) to a target made with the BH mass x 1.1 and initial
    positions + N(0, 1e-3^2).

    Cost: the backward pass per step over a forward step, mixed and FP64, with checkpoints every
    20 steps (the backward pass recomputes each segment but the last from its checkpoint) and
    with every stage kept (checkpoint interval = steps: nothing recomputed).

    Finite differences (FP64, h = 1e-6) over `fd_steps` steps: over 200 steps at this dt the
    close BH passages make the loss too nonlinear in the inputs for any h to converge (h = 1e-4
    .. 1e-7 disagree by more than 100 %); over 40 steps they converge.  Coordinates: half at
    random among the stars' positions and velocities, half the largest |g|, plus the BH mass.
    Errors are reported normwise, |g_i - fd_i| / max|g| (the adjoint's largest component), and
    per coordinate for the largest-|g| half; the worst coordinates get a second difference at
    h/2 (Richardson pair): truncation error scales as h^2, round-off as 1/h.  The mixed-precision
    gradient is compared with the FP64 one."""
    import pn_gb300 as pn
    t_leg = time.monotonic()
    s = pn.config_plummer(ns, 77, 0.05)
    eps = plummer_eps(ns)
    rng = np.random.default_rng(5)
    n = ns + 1
    mt = s.m.copy()
    mt[0] *= 1.1
    xt0 = s.x + rng.normal(0, 1e-3, s.x.shape)
    xt0[0] = s.x[0]

    def final(c, x, v, m, steps):
        c.set_state(x, v, m)
        c.steps(steps)
        return c.get_state()

    def gradient(c, steps, K, xT, vT):
        c.set_state(s.x, s.v, s.m)
        c.adjoint_forward(steps, K)
        xe, ve = c.get_state()
        t0 = time.perf_counter()
        g = c.adjoint_backward(2 * (xe - xT), 2 * (ve - vT))
        return g, (time.perf_counter() - t0) / steps

    out = {"metric": f"adjoint backward cost per step / forward step (N={ns}, {nsteps} steps, "
                     f"checkpoints every 20 steps, mixed)", "unit": "ratio", "higher_is_better": False,
           "config": {"workload": f"plummer_bh_N{ns}_adjoint", "bh_mass_fraction": 0.05, "dt": DT,
                      "steps": nsteps, "checkpoint_every": 20, "also_timed_checkpoint_every": nsteps,
                      "inv_c2": INV_C2, "loss": "|x(T)-x*(T)|^2 + |v(T)-v*(T)|^2, target: m_BH x 1.1, "
                                                "x0 + N(0, 1e-3^2)"}}
    with pn.Context(n, eps=eps, dt=DT, inv_c2=INV_C2, precision=pn.PN_PREC_MIXED) as c:
        xT, vT = final(c, xt0, s.v, mt, nsteps)  # the target (any precision: it is data)
        xTf, vTf = final(c, xt0, s.v, mt, fd_steps)
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
    out["value"] = timing["mixed"]["ratio_K20"]
    out["timing"] = timing
    # gradients over the finite-difference horizon, FP64 and mixed
    grads = {}
    for prec in (0, 1):
        with pn.Context(n, eps=eps, dt=DT, inv_c2=INV_C2, precision=prec) as c:
            grads[prec], _ = gradient(c, fd_steps, 20, xTf, vTf)
    gx, gv, gm = grads[0]
    gx1, gv1, gm1 = grads[1]
    out["mixed_vs_fp64_grad_rel"] = float(np.sqrt((np.linalg.norm(gx1 - gx) ** 2 + np.linalg.norm(gv1 - gv) ** 2) /
                                                  (np.linalg.norm(gx) ** 2 + np.linalg.norm(gv) ** 2)))
    out["mixed_vs_fp64_dm0_rel"] = float(abs(gm1 / gm - 1))
    gall = np.concatenate([gx[1:].ravel(), gv[1:].ravel()])  # stars' coordinates
    gmax = float(np.abs(gall).max())
    half = fd_coords // 2
    top = np.argsort(-np.abs(gall))[:half]
    rest = np.setdiff1d(np.arange(gall.size), top)
    rnd = rng.choice(rest, fd_coords - half, replace=False)
    h = 1e-6
    with pn.Context(n, eps=eps, dt=DT, inv_c2=INV_C2, precision=pn.PN_PREC_FP64) as c:
        c.set_state(s.x, s.v, s.m)
        c.steps(1)  # warm-up

        def loss(x, v, m):
            xe, ve = final(c, x, v, m, fd_steps)
            return float(((xe - xTf) ** 2).sum() + ((ve - vTf) ** 2).sum())

        def fd_coord(q, hh):
            which, r_ = divmod(int(q), 3 * ns)
            p_, k = divmod(r_, 3)
            p_ += 1  # stars are rows 1..ns
            a = (s.x if which == 0 else s.v).copy()
            b = a.copy()
            a[p_, k] += hh
            b[p_, k] -= hh
            lp = loss(a, s.v, s.m) if which == 0 else loss(s.x, a, s.m)
            lm = loss(b, s.v, s.m) if which == 0 else loss(s.x, b, s.m)
            return (lp - lm) / (2 * hh), ("x" if which == 0 else "v", p_, k)

        def fd_mass(hh):
            mp, mm = s.m.copy(), s.m.copy()
            mp[0] += hh
            mm[0] -= hh
            return (loss(s.x, s.v, mp) - loss(s.x, s.v, mm)) / (2 * hh)

        t1 = time.perf_counter()
        fdm = fd_mass(h)
        per_loss = (time.perf_counter() - t1) / 2
        rows, skipped = [], 0
        for kind, qs in (("top_abs_g", top), ("random", rnd)):
            for q in qs:
                if time.monotonic() - t_leg + 2 * per_loss > allowance:
                    skipped += 1
                    continue
                fd, (var, p_, k) = fd_coord(q, h)
                g = float(gall[q])
                rows.append({"kind": kind, "var": var, "particle": int(p_), "k": int(k), "g": g, "fd": float(fd),
                             "err_normwise": abs(g - fd) / gmax, "err_rel": abs(g - fd) / max(abs(fd), 1e-300), "q": int(q)})
        # Richardson pairs: the worst coordinates (normwise) and the BH mass at h / 2
        worst = sorted(rows, key=lambda r: -r["err_normwise"])[:richardson]
        for r in worst:
            if time.monotonic() - t_leg + 2 * per_loss > allowance:
                break
            fd2, _ = fd_coord(r["q"], h / 2)
            r["fd_h2"] = float(fd2)
            r["err_normwise_h2"] = abs(r["g"] - fd2) / gmax
        fdm2 = fd_mass(h / 2) if time.monotonic() - t_leg + 2 * per_loss <= allowance else None
    tops = [r for r in rows if r["kind"] == "top_abs_g"]
    out["fd_check_fp64"] = {
        "steps": fd_steps, "h": h, "coords": len(rows), "skipped_for_time": skipped, "max_abs_g": gmax,
        "max_err_normwise": max(r["err_normwise"] for r in rows) if rows else None,
        "median_err_normwise": float(np.median([r["err_normwise"] for r in rows])) if rows else None,
        "max_err_rel_top_abs_g": max(r["err_rel"] for r in tops) if tops else None,
        "median_err_rel_top_abs_g": float(np.median([r["err_rel"] for r in tops])) if tops else None,
        "bh_mass": {"g": float(gm), "fd": float(fdm), "err_rel": float(abs(gm - fdm) / abs(fdm)),
                    "fd_h2": None if fdm2 is None else float(fdm2),
                    "err_rel_h2": None if fdm2 is None else float(abs(gm - fdm2) / abs(fdm2))},
        "richardson": [{k: r[k] for k in ("var", "particle", "k", "g", "fd", "fd_h2", "err_normwise",
                                          "err_normwise_h2") if k in r} for r in worst],
        "loss_eval_s": per_loss}
    out["seconds"] = time.monotonic() - t_leg
    return out


# ---------------------------------------------------------------------------- configuration 2
def long_run(nstars, precisions, nsteps, every, allowance, label):
    """Device-resident runs of the Plummer + BH workload at nstars: step throughput and the energy
    drift E(t)/E(0) - 1 every `every` steps (energies in FP64 for both modes), then the largest
    gap between the drift curves.  Stops early (and says so) when the allowance would be
    exceeded."""
    import pn_gb300 as pn
    t_leg = time.monotonic()
    s = pn.config_plummer(nstars, SEED, BH_FRACTION)
    eps = plummer_eps(nstars)
    n = nstars + 1
    res = {}
    for prec in precisions:
        with pn.Context(n, eps=eps, dt=DT, inv_c2=INV_C2, precision=0) as c:
            c.set_state(s.x, s.v, s.m)
            e0 = c.energy()[3]
            ms, curve, done, truncated = [], [(0, 0.0)], 0, False
            with ClockSampler() as clk:
                while done < nsteps:
                    kc = min(every, nsteps - done)
                    if ms:
                        per = float(np.concatenate(ms).mean()) * 1e-3
                        if time.monotonic() - t_leg + kc * per * 1.05 + 1.0 > allowance:
                            truncated = True
                            break
                    c.set_params(precision=prec)
                    ms.append(c.bench_steps(kc, flush_l2=False)[0])
                    done += kc
                    c.set_params(precision=0)
                    curve.append((done, float(c.energy()[3] / e0 - 1)))
            allm = np.concatenate(ms)
            res["mixed" if prec else "fp64"] = {
                "steps": done, "truncated": truncated, "ms_per_step": float(allm.mean()),
                "value": 3.0 * n * n / (allm.mean() * 1e-3), "energy_drift": curve[-1][1],
                "drift_curve": curve, "clocks": clk.summary()}
    out = {"metric": label, "unit": UNIT, "config": dict(workload_config(nstars), steps=nsteps)}
    out.update(res)
    if "mixed" in res and "fp64" in res:
        a = dict(res["mixed"]["drift_curve"])
        b = dict(res["fp64"]["drift_curve"])
        common = sorted(set(a) & set(b))
        out["drift_max_abs_diff"] = max(abs(a[t] - b[t]) for t in common)
        out["mixed_over_fp64"] = res["mixed"]["value"] / res["fp64"]["value"]
    out["seconds"] = time.monotonic() - t_leg
    return out


def profile_case(nstars, shape=None):
    """One mixed-precision force evaluation of the bench workload at nstars (ncu target);
    shape = "ipt,tile_j,grid_split[,pair_variant]" pins the packed sweep's launch shape (e.g. the
    tuned one; pair_variant 3 / 4 = the build for 3 / 4 CTAs per SM)."""
    import pn_gb300 as pn
    sysm = pn.config_plummer(nstars, SEED, BH_FRACTION)
    kw = {}
    if shape:
        f = [int(t) for t in shape.split(",")]
        kw = dict(i_per_thread=f[0], tile_j=f[1], grid_split=f[2], pair_variant=f[3] if len(f) > 3 else 2)
    with pn.Context(nstars + 1, eps=plummer_eps(nstars), inv_c2=INV_C2,
                    precision=pn.PN_PREC_MIXED, **kw) as c:
        c.set_state(sysm.x, sysm.v, sysm.m)
        c.force()
        st = c.stats()
        print(json.dumps({"profile_case": nstars, "pair_ms": st.pair_ms, "tile_j": st.tile_j,
                          "i_per_thread": st.i_per_thread, "j_split": st.j_split,
                          "grid_split": st.grid_split, "pair_variant": st.pair_variant}))
    return 0


def host_stage_step(pn, x, v, m, eps, dt):
    """The reference main loop's step around the drop-in force() (Limit-sticky9.c:844-893), the
    stage arithmetic done in place (the same roundings as the reference's loops: 0.5 dt is exact)."""
    a = pn.force(x, v, m, eps)
    x1 = v * (0.5 * dt)
    x1 += x
    v1 = a * (0.5 * dt)
    v1 += v
    h = x1.copy()
    hv = v1.copy()
    a = pn.force(x1, v1, m, eps)
    np.multiply(v1, 0.5 * dt, out=x1)
    x1 += x
    np.multiply(a, 0.5 * dt, out=v1)
    v1 += v
    h += x1
    hv += v1
    a = pn.force(x1, v1, m, eps)
    # (x + x3 + 2 h) / 6 with x3 = x + v1 dt, and the same for v
    np.multiply(v1, dt, out=x1)
    x1 += x
    x1 += x
    h *= 2.0
    x1 += h
    x1 /= 6.0
    np.multiply(a, dt, out=v1)
    v1 += v
    v1 += v
    hv *= 2.0
    v1 += hv
    v1 /= 6.0
    return x1, v1


# ---------------------------------------------------------------------------- headline
def headline(args, rank, world, dist):
    """Configuration 3 (the metric's workload): the line's value, roofline, e2e, FP64, accuracy
    and CPU baseline."""
    import pn_gb300 as pn
    from pn_gb300 import build as b
    if not os.path.exists(pn.LIB_PATH):
        b.build()
    ns = args.nstars
    n = ns + 1
    sysm = pn.config_plummer(ns, SEED + rank, BH_FRACTION)
    eps = plummer_eps(ns)

    # ---------------- mixed precision, device resident (value)
    ctx = pn.Context(n, eps=eps, dt=DT, inv_c2=INV_C2, precision=pn.PN_PREC_MIXED)
    ctx.set_state(sysm.x, sysm.v, sysm.m)
    ctx.autotune(1)  # setup: launch shape of the pair sweep for this size (not timed)
    ctx.bench_steps(args.warmup, flush_l2=True)
    barrier(dist)
    with ClockSampler() as clk:
        step_ms, pair_ms = ctx.bench_steps(args.steps, flush_l2=True)
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
            "config": workload_config(ns, world),
            "gpu_launches": 9 * args.steps,
            "clocks": clk.summary(int(os.environ.get("LOCAL_RANK", "0")))}
    launch_shape = {"tile_j": st.tile_j, "i_per_thread": st.i_per_thread, "j_split": st.j_split,
                    "grid_split": st.grid_split, "threads": st.threads, "pair_variant": st.pair_variant}

    # roofline of the pair sweep against the measured FP32 FMA peak
    if rank == 0:
        flops_pair = pn.flops_per_pair(1, pn.PN_PREC_MIXED, st.pair_variant)
        peak32 = pn.probe_fma_peak(pn.PN_PREC_MIXED)
        pairs = float(ns) * float(ns)
        achieved = pairs * flops_pair / (pair_launch_ms * 1e-3) / 1e12
        kname = {2: "k_pair2<MODE_FORCE> (packed f32x2)",
                 3: "k_pair2<MODE_FORCE> (packed f32x2, 3 CTAs per SM)",
                 4: "k_pair2<MODE_FORCE> (packed f32x2, 4 CTAs per SM)"}.get(st.pair_variant, "k_pair<float, MODE_FORCE>")
        line["roofline"] = {"bound": "fp32", "kernel": kname,
                            "achieved": achieved, "peak": peak32, "unit": "TFLOP/s",
                            "frac": achieved / peak32, "traffic": None,
                            "flops_per_pair": flops_pair, "launch_shape": launch_shape,
                            "pair_launch_ms": pair_launch_ms,
                            "peak_source": "measured FP32 FMA throughput of this GPU (pn_probe_fma_peak)",
                            "pair_interactions_per_s": pairs / (pair_launch_ms * 1e-3)}
        if st.pair_variant in (2, 3, 4):
            # the same FMA work issued as packed two-lane instructions, as the packed sweep does:
            # the ceiling of a sweep made only of fma.rn.f32x2
            peak2 = pn.probe_fma_peak(pn.PROBE_F32X2)
            line["roofline"]["peak_f32x2"] = peak2
            line["roofline"]["frac_of_f32x2_peak"] = achieved / peak2
        prof = os.path.join(ROOT, "profiles", "pair_sweep_traffic.json")
        if os.path.exists(prof) and ns == NSTARS and st.pair_variant in (2, 3, 4):
            try:  # DRAM bytes of one launch at this size and shape, from an ncu capture
                pt = json.load(open(prof))
                line["roofline"]["traffic"] = pt.get("k_pair2_force_f32_N262144_bytes_per_launch")
                line["roofline"]["traffic_source"] = ("ncu dram__bytes_read.sum + dram__bytes_write.sum of one "
                                                      "launch, committed profile (not this run): "
                                                      + str(pt.get("k_pair2_force_f32_N262144_shape")))
                line["roofline"]["ncu_fma_pipe_active_pct"] = pt.get("fma_pipe_active_pct_N65536")
            except (OSError, ValueError):
                pass

        # the O(N) kernels (k_prep + k_finish with the fused stage update) per evaluation: the
        # step's time outside the three pair sweeps, against the measured HBM copy bandwidth
        on_ms = max(float(step_ms.mean()) - float(pair_ms.mean()), 0.0) / 3.0
        gs = st.grid_split
        # k_prep reads x, v, m (56 B) and writes spos, the paired pack, the i-side pack (96 B; the
        # scalar pack's 64 B too when the scalar sweep runs); k_finish reads v, m, spos (56 B) and
        # the j-range partial sums (9 doubles per split), and reads/writes the stage state (168 B)
        moved = 56 + (96 if st.pair_variant in (2, 3, 4) else 160) + 56 + 72 * gs + 168
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
            na = np.linalg.norm(ref, axis=1)
            r = d / na
            acc[f"inv_c2={ic2:g}"] = {
                "rms_rel": float(np.sqrt((r ** 2).mean())), "max_rel": float(r.max()),
                "rms_abs_over_rms_a": float(np.sqrt((d ** 2).mean() / (na ** 2).mean()))}
            if ic2 == 1.0:
                acc["inv_c2=1"]["note"] = ("per-particle error bounded by 8 u (Gabs + Wabs), the absolute "
                                           "sums of the pair terms (tests/test_force_gpu.py)")
        line["accuracy_vs_fp64"] = acc
        # ---------------- CPU baseline (oracle port), bounded sample
        rate, info = cpu_baseline(sysm.x, sysm.v, sysm.m, eps)
        rate1, info1 = cpu_baseline(sysm.x, sysm.v, sysm.m, eps, seconds=4.0, threads=1)
        line["cpu_baseline"] = {"value": rate, "unit": UNIT, "cores": info["threads"], "kind": "port",
                                "sample": info["sample"], "seconds": info["seconds"],
                                "single_core_value": rate1, "single_core_sample": info1["sample"]}
    return line


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=8)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="pn", choices=["pn", "reference"])
    ap.add_argument("--nstars", type=int, default=NSTARS)
    ap.add_argument("--quick", action="store_true",
                    help="headline only: skip the FP64, accuracy, CPU and other-configuration legs")
    ap.add_argument("--no-configs", action="store_true", help="skip the config2/4/5 legs of the line")
    ap.add_argument("--budget-s", type=float, default=1500.0,
                    help="wall-clock budget of the whole command; the config legs fit inside it")
    ap.add_argument("--profile-case", type=int, default=0, metavar="N",
                    help="set up N stars, tune, run one mixed force evaluation and exit (for ncu)")
    ap.add_argument("--ensemble", action="store_true", help="configuration 4 (ensemble) alone")
    ap.add_argument("--clusters", type=int, default=256)
    ap.add_argument("--adjoint", action="store_true", help="configuration 5 (adjoint) alone")
    ap.add_argument("--adj-n", type=int, default=16384)
    ap.add_argument("--adj-steps", type=int, default=200)
    ap.add_argument("--fd-coords", type=int, default=64)
    ap.add_argument("--fd-steps", type=int, default=40)
    ap.add_argument("--shape", default=None,
                    help="--profile-case launch shape: ipt,tile_j,grid_split[,pair_variant]")
    ap.add_argument("--fp64-run", type=int, default=0, metavar="STEPS",
                    help="configuration 2 alone: N=65536, FP64 and mixed, STEPS steps each")
    ap.add_argument("--drift", type=int, default=0, metavar="STEPS",
                    help="energy drift of the headline workload, mixed and FP64, STEPS steps each")
    ap.add_argument("--long-mixed", type=int, default=0, metavar="STEPS",
                    help="energy drift of the headline workload in mixed precision over STEPS steps")
    args = ap.parse_args()
    budget = Budget(args.budget_s)
    if args.impl == "reference":
        # the reference arm is CPU work on rank 0 only: no process group, no GPU library
        return run_reference(args, int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")))
    if args.fp64_run:
        every = max(1, args.fp64_run // 10)
        r = long_run(65536, (1, 0), args.fp64_run, every, budget.left() - 30,
                     "integration at N=65536, FP64 and mixed (interactions/s, energy drift)")
        print(json.dumps(r), flush=True)
        return 0
    if args.drift:
        r = long_run(args.nstars, (1, 0), args.drift, max(1, args.drift // 5), budget.left() - 30,
                     "energy drift, mixed vs FP64 (interactions/s per mode)")
        print(json.dumps(r), flush=True)
        return 0
    if args.long_mixed:
        r = long_run(args.nstars, (1,), args.long_mixed, max(1, args.long_mixed // 5), budget.left() - 30,
                     "energy drift of the mixed-precision integration (interactions/s)")
        print(json.dumps(r), flush=True)
        return 0
    if args.profile_case:
        return profile_case(args.profile_case, args.shape)
    if args.ensemble:
        print(json.dumps(ensemble_leg(args.steps, args.warmup, args.clusters, budget.left() - 30)), flush=True)
        return 0
    if args.adjoint:
        print(json.dumps(adjoint_leg(args.adj_n, args.adj_steps, args.fd_steps, args.fd_coords,
                                     budget.left() - 30)), flush=True)
        return 0
    rank, world, dist = dist_init(args.gpus)
    line = headline(args, rank, world, dist)
    if rank == 0 and world == 1 and not args.quick and not args.no_configs:
        # the other configurations of the workload set, inside the remaining budget: config 2's
        # FP64 run is the longest and goes last, keeping what the earlier legs leave
        reserve = 30.0
        line["config4"] = ensemble_leg(args.steps, args.warmup, 256, min(240.0, budget.left() - reserve - 1000))
        line["config5"] = adjoint_leg(16384, 200, 40, 64, min(720.0, budget.left() - reserve - 640))
        line["config2"] = long_run(65536, (1, 0), 500, 50, budget.left() - reserve,
                                   "integration at N=65536 over 500 steps, FP64 and mixed "
                                   "(interactions/s, energy drift)")
        line["gpu_launches"] += line["config4"]["gpu_launches"]
    if rank == 0:
        line["wall_s"] = time.monotonic() - T_START
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
