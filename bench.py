#!/usr/bin/env python
"""Replica-sampler step throughput on GB300 (the hot path of ESM-Sampling's `sampler = "replicas"`).

A step is one replica step of one chain (replica_step!, src/replicas.jl:676): the scheduled weather
bursts with their compensated re-initialisation, one operation sweep of every replica (operation_sweep!,
src/local.jl:2401: the local sweep with the plain families; with --storage-ms also the storage
multiscale sweep with probability 1/2 and the long-range storage sweep, as operation_sweep! runs
them), the capacity scores, the replica-averaged Langevin step of the shared capacities and the
dispatch following. The two storage sweeps are also timed on their own and reported as
`storage_ms` and `storage_long`. Workload: 40 nodes, 60 lines, hourly T = 8760, 64 weather replicas
(the "plain method on GPU" configuration), synthetic seeded data.

  value  device throughput: sweeps of all replicas per second from CUDA-event spans on the
         library's stream (inputs resident in HBM; every input is larger than L2)
  e2e    the same metric through the public API with host buffers: the host-driven replica loop
         (gate, weights, schedule) calling the C ABI, host<->device copies of every step included
  --impl reference: the CPU restatement of the reference algorithm (the reference itself is Julia
         and cannot run here) on all host cores, on a bounded sample of the same workload
"""
import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
for _p in (ROOT, os.path.join(ROOT, "esm-sampling_gb300")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import numpy as np  # noqa: E402

WORKLOAD = dict(N=40, L=60, T=8760, R=64, seed=1234)
# a reduced case of the same model (T = 584, 15-hour steps) for profiler captures
SMALL = dict(N=40, L=60, T=584, R=64, seed=1234)
METRIC = "local-move sweeps/s"
UNIT = "sweeps/s"


def rank_info():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class Clocks:
    """nvidia-smi samples every 200 ms during the timed region."""

    def __init__(self):
        self.rows = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "--query-gpu=index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
                 "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
                 "--format=csv,noheader,nounits", "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL,
                text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        dev = os.environ.get("CUDA_VISIBLE_DEVICES", "0").split(",")[0]
        rows = [r for r in self.rows if len(r) >= 9 and (r[0] == dev or len(set(x[0] for x in self.rows)) == 1)]
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower().startswith("active")})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def setup_chain(precision=32, storage_ms=0):
    from esmgb.device import DeviceChain
    from esmgb.model import initial_state, make_model
    w = WORKLOAD
    m = make_model(w["N"], w["L"], w["T"], seed=w["seed"])
    st = initial_state(m, w["R"], seed=7)
    d = DeviceChain(m, w["R"], precision=precision, seed=w["seed"], storage_ms=storage_ms)
    d.upload(st)
    return m, st, d


def schedule(ctl, it, R, rng):
    """Weather bursts of the step (replica_schedule: weather_schedule / replica_weather!,
    src/replicas.jl:571-606)."""
    from esmgb.replicas import replica_schedule
    return replica_schedule(ctl, it, R, WORKLOAD["T"], rng)


def carrier_params(m):
    from esmgb.model import LANGEVIN_KAPPA
    eta = np.full(len(m.carriers), 5e-4)             # langevin_eta (src/run.jl:105)
    ks = np.array([LANGEVIN_KAPPA.get(c, 100.0) for c in m.carriers])
    return eta, ks


def device_loop(d, m, ctl, it0, n, rng, pre, counts=False):
    """The device-resident step: everything on the GPU, host arrays only for the schedule. With
    counts, the move counts of the sweeps (tried and taken per family, guard events) are read after
    each sweep (one more short synchronisation per step: the score call synchronises anyway) and
    returned summed."""
    eta, ks = carrier_params(m)
    w = np.full(d.R, 1.0 / d.R)
    total = None
    for q in range(n):
        it = it0 + q
        moved, theta, window, wstart, _ = pre[q] if pre else schedule(ctl, it, d.R, rng)
        if moved.any():
            d.weather_step(moved, theta, window, wstart, it=it)
        st = d.sweeps(1, sweep0=it, stats=counts)
        if counts:
            total = st if total is None else total + st
        d.scores()
        d.langevin_step(w, eta, ks, ctl.kappa_min, ctl.clip, ctl.box, None, it)
    return total


FAMILIES = ("unit", "pair", "xpair", "xlocc", "xloc", "potential", "cellpair", "cell", "spair", "tpot", "tsoc",
            "atoms")  # the ESM_FAM_* order of the move counts, then the basis atoms


def move_counts(st):
    """The correctness counters of the bench line from esm_operation_sweeps' counts."""
    st = np.asarray(st, np.int64)
    fam = {f: [int(st[2 * i]), int(st[2 * i + 1])] for i, f in enumerate(FAMILIES) if st[2 * i] > 0}
    tried = int(st[:-1:2].sum())
    return {"tried": tried, "taken": int(st[1:-1:2].sum()), "guards": int(st[-1]),
            "guard_rate": int(st[-1]) / max(tried, 1), "by_family": fam,
            "note": "line moves of the timed sweeps, [tried, taken] per family; a guard event is a walk "
                    "beyond the point cap, left at t = 0"}


def e2e_loop(d, m, ctl, R_set, it0, n, rng):
    """The host-driven replica loop through the library's public call, replica_step (replica_step!,
    src/replicas.jl:676-704, over the C ABI); returns the bytes copied per step each way."""
    from esmgb import replicas as RP
    _, ks = carrier_params(m)
    ratio = m.beta_k / m.beta_v
    h2d = d2h = 0
    for q in range(n):
        rec = RP.replica_step(d, R_set, ctl, it0 + q, rng, ks, ratio, m.unit_hi, m.unit_group)
        h2d += rec["h2d"]
        d2h += rec["d2h"]
    return h2d / n, d2h / n


def carrier_totals(m, k):
    """ktot (src/replicas.jl:812): the capacity of every carrier, summed over its units."""
    return np.bincount(np.asarray(m.unit_group), weights=np.asarray(k, float), minlength=len(m.carriers))


def capacity_ess(m, kt, seconds):
    """The metric's capacity ESS/s: the bulk ESS (src/convergence.jl:125) of every carrier total over
    the steps of one chain, the smallest over carriers, per wall second; with the relative MCSE of
    each carrier's mean (src/convergence.jl:141)."""
    from esmgb.convergence import ess_bulk, mcse_rel
    kt = np.asarray(kt)
    ess, mcse = {}, {}
    for i, c in enumerate(m.carriers):
        x = kt[:, i]
        if not np.all(np.isfinite(x)) or np.ptp(x) == 0:   # a carrier that did not move has no samples
            ess[c], mcse[c] = 0.0, float("inf")
        else:
            ess[c], mcse[c] = float(ess_bulk([x])), float(mcse_rel([x]))
    worst = min(ess, key=ess.get)
    nonfinite = int((~np.isfinite(kt)).any(axis=1).sum())
    w = np.log(np.maximum(kt, 1e-300))
    msjd = float(np.mean(np.sum(np.diff(w, axis=0) ** 2, axis=1))) if len(kt) > 1 else 0.0
    return {"value": ess[worst] / seconds, "unit": "ESS/s", "ess_min": ess[worst], "carrier": worst,
            "steps": len(kt), "seconds": seconds, "ess": ess, "mcse_rel": mcse,
            "msjd_log_ktot_per_step": msjd, "nonfinite_steps": nonfinite}


def ess_arms(d, m, ctl, it0, n, arms=("plain", "learned", "da")):
    """Capacity ESS/s of the plain replica step and of the learned capacity steps over n steps each,
    every arm from the same saved chain state and over the same weather schedule; each step is one
    plain evaluation (an operation sweep and the scores). The learned arms use the surrogate of the
    learned-proposal configuration: 3 hidden layers of 512, minibatches of 1024, Adam at 1e-3, 4x the
    plain step; it is trained on the plain arm's pairs before its arms (not timed) and online during
    them.
      plain    the device Langevin step on the replica-averaged score (replica_step!, src/replicas.jl:676)
      learned  SurrogateLangevin: the surrogate's drift at 4x the plain step, judged by the plain scores
      da       DALangevin: 4x proposals, delayed acceptance with the plain estimate as second stage"""
    from esmgb.surrogate import DALangevin, ScoreSurrogate, SurrogateLangevin
    eta, ks = carrier_params(m)
    w = np.full(d.R, 1.0 / d.R)
    rng = np.random.Generator(np.random.PCG64(99))
    sched = [schedule(ctl, it0 + q, d.R, rng) for q in range(n)]
    d.sync(600.0)
    d.state_save()
    out = {}
    pairs = []
    k = d.download_k()
    occ = d.regime_occupancy()
    kt = []
    t0 = time.perf_counter()
    for q in range(n):
        moved, theta, window, wstart, _ = sched[q]
        if moved.any():
            d.weather_step(moved, theta, window, wstart, it=it0 + q)
            occ = d.regime_occupancy()
        d.sweeps(1, sweep0=it0 + q, stats=False)
        sk, _, _ = d.scores()
        pairs.append((k, occ, w @ sk))
        k, _ = d.langevin_step(w, eta, ks, ctl.kappa_min, ctl.clip, ctl.box, None, it0 + q)
        kt.append(carrier_totals(m, k))
    d.sync(600.0)
    out["plain"] = capacity_ess(m, kt, time.perf_counter() - t0)
    learned = [a for a in arms if a != "plain"]
    if not learned:
        d.state_restore()
        return out
    sur = ScoreSurrogate(m, hidden=(512, 512, 512), capacity=8192, batch=1024, lr=1e-3, seed=1,
                         min_pairs=min(16, n))
    for kk, oc, sb in pairs:
        sur.add(kk, oc, sb)
    sur.train(200)
    for arm in learned:
        d.state_restore()
        if arm == "learned":
            stepper = SurrogateLangevin(d, m, sur, eta, ks, ctl.kappa_min, ctl.clip, mult=4.0, seed=3)
        else:
            stepper = DALangevin(d, m, sur, eta, ks, ctl.kappa_min, ctl.clip, mult=4.0, seed=3)
        kt = []
        t0 = time.perf_counter()
        for q in range(n):
            if arm == "learned":
                stepper.step(it0 + q, sched[q])
            else:
                moved, theta, window, wstart, _ = sched[q]
                if moved.any():
                    d.weather_step(moved, theta, window, wstart, it=it0 + q)
                stepper.step(it0 + q)
            kt.append(carrier_totals(m, stepper.k))
        d.sync(600.0)
        out[arm] = capacity_ess(m, kt, time.perf_counter() - t0)
        out[arm]["stats"] = dict(stepper.stats)
        pv = out["plain"]["value"]
        out[arm]["ratio_to_plain"] = out[arm]["value"] / pv if pv > 0 else None
    sur.close()
    d.state_restore()
    return out


def cpu_sample(threads, sweeps=1, R=2, storage_ms=0, warm=1):
    """The oracle on the host cores: `warm` untimed operation sweeps from sweep 1 (a worn state, as
    the GPU chain's), then `sweeps` timed operation sweeps and the scores of R of the replicas; with
    storage_ms, two timed sweeps (the storage multiscale sweep runs with probability 1/2)."""
    if storage_ms:
        sweeps = 2
    from esmgb.model import initial_state, make_model
    from oracle.oracle import Oracle
    w = WORKLOAD
    m = make_model(w["N"], w["L"], w["T"], seed=w["seed"])
    st = initial_state(m, R, seed=7)
    o = Oracle(m, R, seed=w["seed"], threads=threads, storage_ms=storage_ms, storage_long=storage_ms)
    o.set_state(st)
    if warm:
        o.sweeps(warm, 1)
    t0 = time.perf_counter()
    o.sweeps(sweeps, 1 + warm)
    o.scores()
    dt = time.perf_counter() - t0
    return sweeps * (R / w["R"]) / dt, dt


def run_reference(args):
    """The reference arm: the reference's algorithm (the FP64 restatement in oracle/, OpenMP over the
    steps of a colour class) on all host cores, on a bounded sample of the workload -- one chain of 1
    of the 64 replicas of the same model and start state. Its --warmup steps (untimed) wear the
    sample's state as the GPU arm's warm-up wears its chain; each timed step is one operation sweep
    of the sample (the next sweep index; with --storage-ms the storage sweeps as operation_sweep!
    runs them) and its capacity scores. ms_per_step is the measured wall time of a sample step;
    value is the workload's rate that the sample implies (the sample's sweeps/s over the replicas it
    holds: x 64)."""
    rank, world, _ = rank_info()
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    from oracle import oracle as O
    O.build()
    from esmgb.model import initial_state, make_model
    from oracle.oracle import Oracle
    w = WORKLOAD
    nrep = 1
    sm = int(args.storage_ms)
    m = make_model(w["N"], w["L"], w["T"], seed=w["seed"])
    o = Oracle(m, nrep, seed=w["seed"], threads=threads, storage_ms=sm, storage_long=sm)
    o.set_state(initial_state(m, nrep, seed=7))
    sweep = 1
    for _ in range(args.warmup):
        o.sweeps(1, sweep)
        o.scores()
        sweep += 1
    dts = []
    t0 = time.perf_counter()
    for _ in range(args.steps):
        t1 = time.perf_counter()
        o.sweeps(1, sweep)
        o.scores()
        dts.append(time.perf_counter() - t1)
        sweep += 1
    wall = time.perf_counter() - t0
    scale = w["R"] / nrep
    value = len(dts) / (sum(dts) * scale)
    sample = (f"one chain of {nrep} of the {w['R']} replicas (T = {w['T']}), worn by {args.warmup} untimed steps; "
              f"each step one operation sweep{' with the storage sweeps' if sm else ''} and the capacity scores "
              f"of the sample ({1000.0 * sum(dts) / max(len(dts), 1):.0f} ms per step), scaled x{scale:g} to the "
              f"workload's replicas")
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * sum(dts) / max(len(dts), 1),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": config_dict(), "sample_scale": scale,
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "note": ("the reference is a Julia package (no Julia on this machine): its algorithm is timed through "
                     "the FP64 C++ restatement in oracle/, OpenMP over the steps of a colour class; ms_per_step is "
                     "the wall time of a step of the sample, value the workload's rate the sample implies"),
            "wall_s": wall}
    print(json.dumps(line), flush=True)


def profile_case(args):
    """Operation sweeps of the reduced case, for ncu captures of the line-move kernel."""
    from esmgb import build as B
    B.build()
    from esmgb.device import DeviceChain
    from esmgb.model import initial_state, make_model
    w = dict(SMALL)
    if args.T:
        w["T"] = args.T
    if args.N:
        w["N"], w["L"] = args.N, args.L or int(round(1.5 * args.N))
    if args.R:
        w["R"] = args.R
    m = make_model(w["N"], w["L"], w["T"], seed=w["seed"])
    d = DeviceChain(m, w["R"], precision=32, seed=w["seed"])
    d.upload(initial_state(m, w["R"], seed=7))
    grid = None
    d.set_move_schedule(args.schedule)
    if args.grid:
        d.set_move_grid(*(int(x) for x in args.grid.lower().split("x")))
    elif args.autotune:
        grid = d.autotune_moves(sweep=0)[0]
    if args.sep:
        d.set_sep_walk(args.sep)
    d.sweeps(args.warmup, 0, stats=False)
    d.set_timing(True)
    st = d.sweeps(args.steps, args.warmup)
    d.scores()
    kt = d.timing()
    print(json.dumps({"case": "small", "N": w["N"], "T": w["T"], "R": w["R"], "sweeps": args.steps,
                      "grid": list(d.move_grid()[:2]), "schedule": d.move_schedule(), "sep_walk_min_units": args.sep,
                      "kernel_ms": {k: v[0] for k, v in kt.items()}, "launches": {k: v[1] for k, v in kt.items()},
                      "moves_tried": int(st[:-1:2].sum()), "guards": int(st[-1])}), flush=True)


def learned_case(args):
    """Long capacity chains of the plain step and the learned capacity steps on a reduced-T model of
    the learned-proposal configuration (40 nodes, 60 lines, --T steps, default 120, --R replicas,
    default 64; surrogate 3 x 512, minibatches of 1024, Adam 1e-3, 4x the plain step): --warmup plain
    steps that train the surrogate (2 Adam steps per pair), then --ess-steps steps per arm, every arm
    from the same saved state over the same weather schedule, one plain evaluation per step. Per arm:
    the bulk ESS of every carrier total (src/convergence.jl:125) and its minimum per second, the
    mean squared jump of the log carrier totals, the carrier means with their MCSE, and the shift of
    each mean from the plain arm's in MCSE units.
      plain    the plain step (device Langevin step, langevin_update, src/replicas.jl:368)
      plain4   the plain step at 4x its size and clip
      sur1     SurrogateLangevin with its judge (falls back to the plain step where the surrogate
               disagrees with the plain estimates beyond their noise)
      surinf   SurrogateLangevin with the judge off (the surrogate's drift whenever it is trained)"""
    from esmgb import build as B
    B.build()
    from esmgb.convergence import ess_bulk
    from esmgb.device import DeviceChain
    from esmgb.model import LANGEVIN_KAPPA, initial_state, make_model
    from esmgb.replicas import ReplicaCtl, replica_schedule
    from esmgb.surrogate import ScoreSurrogate, SurrogateLangevin
    T, R, N, W = args.T or 120, args.R or 64, args.ess_steps, args.warmup
    m = make_model(40, 60, T, seed=5)
    eta = np.full(len(m.carriers), 5e-4)
    ks = np.array([LANGEVIN_KAPPA.get(c, 100.0) for c in m.carriers])
    ug = np.asarray(m.unit_group)
    d = DeviceChain(m, R, precision=32, seed=3)
    d.upload(initial_state(m, R, seed=7))
    ctl = ReplicaCtl(M=R)
    w = np.full(R, 1.0 / R)
    rng = np.random.Generator(np.random.PCG64(1))
    sched = [replica_schedule(ctl, it, R, T, rng) for it in range(W + N + 1)]
    sur = ScoreSurrogate(m, hidden=(512, 512, 512), capacity=8192, batch=1024, lr=1e-3, seed=1)
    t0 = time.perf_counter()
    for it in range(W):
        mv, th, win, ws, _ = sched[it]
        if mv.any():
            d.weather_step(mv, th, win, ws, it=it)
        d.sweeps(1, sweep0=it, stats=False)
        sk, fk, _ = d.scores()
        sur.add(d.download_k(), d.regime_occupancy(), w @ sk)
        sur.train(2)
        d.langevin_step(w, eta, ks, 1.0, 0.02, True, None, it)
    d.sync(600.0)
    out = {"case": "learned", "workload": f"40 nodes, 60 lines, T={T}, {R} replicas", "warmup_steps": W,
           "warmup_s": time.perf_counter() - t0, "steps_per_arm": N, "arms": {}}
    d.state_save()
    for arm in [a for a in (args.arms or "plain,plain4,sur1,surinf").split(",") if a]:
        d.state_restore()
        kt = []
        t0 = time.perf_counter()
        st = None
        if arm.startswith("plain"):
            mult = 4.0 if arm == "plain4" else 1.0
            for q in range(N):
                it = W + q
                mv, th, win, ws, _ = sched[it]
                if mv.any():
                    d.weather_step(mv, th, win, ws, it=it)
                d.sweeps(1, sweep0=it, stats=False)
                d.scores()
                k, _ = d.langevin_step(w, mult * eta, ks, 1.0, mult * 0.02, True, None, it)
                kt.append(carrier_totals(m, k))
        else:
            tol = {"sur1": 1.0, "surinf": float("inf")}[arm]
            sl = SurrogateLangevin(d, m, sur, eta, ks, 1.0, 0.02, mult=4.0, seed=3, train_steps=2, tol=tol)
            for q in range(N):
                sl.step(W + q, sched[W + q])
                kt.append(carrier_totals(m, sl.k))
            st = dict(sl.stats)
        d.sync(600.0)
        secs = time.perf_counter() - t0
        kt = np.asarray(kt)
        ess = {c: (float(ess_bulk([kt[:, i]])) if np.ptp(kt[:, i]) > 0 and np.all(np.isfinite(kt[:, i])) else 0.0)
               for i, c in enumerate(m.carriers)}
        r = {"seconds": secs, "ess": ess, "ess_min": min(ess.values()), "ess_per_s": min(ess.values()) / secs,
             "msjd_log_ktot": float(np.mean(np.sum(np.diff(np.log(kt), axis=0) ** 2, axis=1))),
             "mean": {c: float(kt[:, i].mean()) for i, c in enumerate(m.carriers)},
             "mcse": {c: float(kt[:, i].std() / np.sqrt(max(ess[c], 1.0))) for i, c in enumerate(m.carriers)}}
        if st:
            r["stats"] = st
        out["arms"][arm] = r
    sur.close()
    p = out["arms"].get("plain")
    if p:
        for arm, r in out["arms"].items():
            if arm != "plain":
                r["shift_mcse"] = {c: (r["mean"][c] - p["mean"][c]) / math.hypot(r["mcse"][c], p["mcse"][c])
                                   for c in m.carriers}
                r["ess_per_s_over_plain"] = r["ess_per_s"] / p["ess_per_s"]
    print(json.dumps(out), flush=True)


def mlp_case(args):
    """The surrogate's training step at the full form's sizes (5 hidden layers of 1024 between the
    256-node model's 1357 capacities plus the 8-dim regime summary and its 1357 scores, minibatches of
    1024), with the tcgen05 GEMMs and with the mma.sync GEMMs: wall time per step and TFLOP/s (the
    forward, backward and weight-gradient GEMMs, 3 x 2 x B x the layers' weights)."""
    from esmgb import build as B
    B.build()
    from esmgb.surrogate import MLP
    dims = [1365, 1024, 1024, 1024, 1024, 1024, 1357]
    flops = 3 * 2 * 1024 * sum(dims[i] * dims[i + 1] for i in range(len(dims) - 1))
    rng = np.random.default_rng(0)
    x = rng.standard_normal((1024, dims[0])).astype(np.float32)
    t = rng.standard_normal((1024, dims[-1])).astype(np.float32)
    out = {"case": "mlp", "dims": dims, "batch": 1024, "flops_per_step": flops}
    for kind, name in ((1, "tcgen05"), (0, "mma_sync")):
        net = MLP(dims, batch_max=1024, seed=1)
        net.set_gemm(kind)
        for _ in range(max(args.warmup, 1)):
            net.train_step(x, t, 1e-3)
        t0 = time.perf_counter()
        for _ in range(args.steps):
            net.train_step(x, t, 1e-3)
        dt = (time.perf_counter() - t0) / args.steps
        out[name] = {"ms": 1000 * dt, "tflops": flops / dt / 1e12}
        net.close()
    print(json.dumps(out), flush=True)


def storage_case(args):
    """One forced storage multiscale sweep after one operation sweep (40 nodes, 64 replicas, T from
    --T, default 8760), for timing and profiler captures of k_plateau."""
    from esmgb import build as B
    B.build()
    from esmgb.device import DeviceChain
    from esmgb.model import initial_state, make_model
    T = args.T or WORKLOAD["T"]
    m = make_model(WORKLOAD["N"], WORKLOAD["L"], T, seed=WORKLOAD["seed"])
    d = DeviceChain(m, WORKLOAD["R"], precision=32, seed=WORKLOAD["seed"])
    d.upload(initial_state(m, WORKLOAD["R"], seed=7))
    d.sweeps(1, 0, stats=False)
    d.sync(600.0)
    d.set_timing(True)
    st = d.storage_ms(1, force=True)
    d.sync(600.0)
    ms_ms = d.timing()["storage"][0]
    sl = d.storage_long(1)
    d.sync(600.0)
    print(json.dumps({"case": "storage", "T": T, "R": WORKLOAD["R"], "multiscale": {"moves": [int(x) for x in st],
                      "ms": ms_ms}, "long_range": {"moves": [int(x) for x in sl], "ms": d.timing()["storage"][0]}}),
          flush=True)


def batch_case(args):
    """Many independent models of uneven size on one GPU (the batching configuration): N ~ U{10..128},
    L = 1.5 N, T in {1460, 2920, 8760}, 16 replicas each (seed-fixed). Default: one esm_batch over
    the models' contexts -- one captured graph per sweep, one line-move launch per move index over
    the tasks of every model, the grid picked by the batch's autotuner (untimed); --batch-mode
    streams: every model's own graph-captured sweep on its own stream, the host enqueuing one sweep
    on every context before waiting for all. The timed region is --steps sweeps of every model."""
    from esmgb import build as B
    B.build()
    from esmgb.device import DeviceBatch, DeviceChain
    from esmgb.model import initial_state, make_model
    rng = np.random.default_rng(2024)
    nm = args.models
    specs = [(int(rng.integers(10, 129)), int(rng.choice([1460, 2920, 8760]))) for _ in range(nm)]
    chains = []
    t0 = time.perf_counter()
    for i, (N, T) in enumerate(specs):
        m = make_model(N, int(round(1.5 * N)), T, seed=1000 + i)
        d = DeviceChain(m, 16, precision=32, seed=1000 + i)
        d.upload(initial_state(m, 16, seed=7))
        if args.grid and args.batch_mode == "streams":
            d.set_move_grid(*(int(x) for x in args.grid.lower().split("x")))
        chains.append((m, d))
    setup = time.perf_counter() - t0
    out = {"case": "batch", "mode": args.batch_mode, "models": nm, "replicas": 16, "sweeps": args.steps}
    moves = sum((sum(len(a.ptr) - 1 for a in m.atoms) + round(4.0 * m.N)) * m.T * 16 for m, _ in chains)
    if args.batch_mode == "batch":
        bt = DeviceBatch([d for _, d in chains])
        t1 = time.perf_counter()
        if args.grid:
            bt.set_grid(*(int(x) for x in args.grid.lower().split("x")))
        else:
            best, cand = bt.autotune(sweep=0)
            out["autotune_ms"] = {f"{a}x{b}": round(v, 2) for (a, b), v in cand.items()}
        out["autotune_s"] = time.perf_counter() - t1
        out["grid"] = list(bt.grid()[:2])
        bt.sweeps(args.warmup, 0, stats=False)           # captures the batch's sweep graph
        l0 = bt.launch_count()
        t0 = time.perf_counter()
        st = bt.sweeps(args.steps, args.warmup)
        dt = time.perf_counter() - t0
        dev = bt.last_ms() / 1e3
        out.update({"model_sweeps_per_s": nm * args.steps / dev, "line_moves_per_s": moves * args.steps / dev,
                    "device_s": dev, "wall_s": dt, "gpu_launches": bt.launch_count() - l0,
                    "guards": int(st[:, -1].sum()), "moves_tried": int(st[:, :-1:2].sum())})
        bt.close()
    else:
        for m, d in chains:                       # warm-up: captures each context's class graphs
            d.sweeps(args.warmup, 0, stats=False)
        for m, d in chains:
            d.sync(600.0)
        t0 = time.perf_counter()
        for s in range(args.steps):
            for m, d in chains:
                d.sweeps(1, args.warmup + s, stats=False)
        for m, d in chains:
            d.sync(600.0)
        dt = time.perf_counter() - t0
        out.update({"model_sweeps_per_s": nm * args.steps / dt, "line_moves_per_s": moves * args.steps / dt,
                    "wall_s": dt})
    out.update({"setup_s": setup, "sizes": {"N": [n for n, _ in specs], "T": [t for _, t in specs]}})
    print(json.dumps(out), flush=True)


def n256_case(args):
    """The full-scale configuration: 256 nodes, 420 lines, hourly T = 8760, 256 replicas, the storage
    sweeps on (the multiscale sweep with probability 1/2, the long-range sweep every sweep, as
    operation_sweep! runs them) and the automatic point cap of the 256-unit state-of-charge atoms
    (1024). Steps as the default bench's (weather, operation sweep, scores, Langevin step), then one
    training step of the 5 x 1024 surrogate on minibatches of 1024 (BF16 tensor cores), timed; the
    oracle on a sample of one replica's moves (the first moves of one colour class), extrapolated to
    the whole sweep of 256 replicas."""
    from esmgb import build as B
    B.build()
    from esmgb import replicas as RP
    from esmgb.device import DeviceChain
    from esmgb.model import initial_state, make_model
    from esmgb.surrogate import MLP
    N, L, T, R = args.N or 256, args.L or 420, args.T or 8760, args.R or 256
    m = make_model(N, L, T, seed=1234)
    d = DeviceChain(m, R, precision=32, seed=1234, storage_ms=1, storage_long=1)
    d.upload(initial_state(m, R, seed=7))
    # the walk buffers of a 256-node model exceed the lanes' local arrays and live in global slabs,
    # sized at creation for at most 1 GB (7 warps per SM here); a single chain on the GPU grows them
    # to the grid: 4-warp blocks at 32 warps per SM (the autotuner's choice at 128 nodes), ~9 GB
    d.set_move_grid(*((int(x) for x in args.grid.lower().split("x")) if args.grid else (4, 32)))
    d.set_move_schedule(args.schedule)
    ctl = RP.ReplicaCtl(M=R)
    rng = np.random.Generator(np.random.PCG64(1))
    t0 = time.perf_counter()
    device_loop(d, m, ctl, 1, args.warmup, rng, None)
    d.sync(3600.0)
    warm_s = time.perf_counter() - t0
    d.set_timing(True)
    st0 = np.zeros(2 * (12) + 1, np.int64)
    t0 = time.perf_counter()
    eta, ks = carrier_params(m)
    w = np.full(R, 1.0 / R)
    for q in range(args.steps):
        it = 1 + args.warmup + q
        moved, theta, window, wstart, _ = schedule(ctl, it, R, rng)
        if moved.any():
            d.weather_step(moved, theta, window, wstart, it=it)
        st0 += d.sweeps(1, sweep0=it)
        d.scores()
        d.langevin_step(w, eta, ks, ctl.kappa_min, ctl.clip, ctl.box, None, it)
    d.sync(3600.0)
    wall = time.perf_counter() - t0
    kt = d.timing()
    dev_ms = sum(v[0] for v in kt.values())
    cls_ms, cls_n = kt["class_pass"]
    alg = 4 * (11 * N + 2 * L) * (T / 2) * R
    per = cls_ms / max(cls_n, 1) / 1000.0
    peak, kind = peaks()
    tried = int(st0[:-1:2].sum())
    out = {"case": "n256", "workload": f"{N} nodes, {L} lines, T={T} hourly, {R} replicas, storage sweeps on",
           "steps": args.steps, "warmup": args.warmup, "warmup_s": warm_s,
           "sweeps_per_s": args.steps / (dev_ms / 1000.0), "wall_s": wall, "ms_per_step": dev_ms / args.steps,
           "kernel_ms_per_step": {k: v[0] / args.steps for k, v in kt.items()},
           "moves_tried": tried, "guards": int(st0[-1]), "guard_rate": int(st0[-1]) / max(tried, 1),
           "max_points": int(d.opts.max_points) or 4 * N,
           "roofline_class_pass": {"bound": "hbm", "achieved": alg / per / 1e9 if per > 0 else 0.0, "peak": peak,
                                   "unit": "GB/s", "frac": (alg / per / 1e9) / peak if per > 0 else 0.0,
                                   "peak_kind": kind},
           "move_grid": list(d.move_grid()[:2])}
    # the surrogate of the full form: 5 hidden layers of 1024, minibatches of 1024
    d_in = m.Kunits + 4 * m.K
    dims = [d_in, 1024, 1024, 1024, 1024, 1024, m.Kunits]
    mlp = MLP(dims, batch_max=1024, seed=1)
    xr = np.random.default_rng(0)
    x = xr.standard_normal((1024, d_in)).astype(np.float32)
    y = xr.standard_normal((1024, m.Kunits)).astype(np.float32)
    for _ in range(3):
        mlp.train_step(x, y, 1e-3)
    ns = 20
    t0 = time.perf_counter()
    for _ in range(ns):
        mlp.train_step(x, y, 1e-3)
    mlp_s = (time.perf_counter() - t0) / ns
    flops = 3 * 2 * 1024 * sum(dims[i] * dims[i + 1] for i in range(len(dims) - 1))
    out["surrogate_train_step"] = {"dims": dims, "batch": 1024, "ms": 1000 * mlp_s, "tflops": flops / mlp_s / 1e12,
                                   "note": "forward + backward + Adam of one minibatch, wall time of the call "
                                           "(host copies of the minibatch included)"}
    mlp.close()
    if not args.no_cpu_baseline:
        from oracle import oracle as O
        from oracle.oracle import Oracle
        O.build()
        st1 = d.download()
        sub = {k: (v if k == "k" else np.ascontiguousarray(v[..., :1])) for k, v in st1.items()}
        o = Oracle(m, 1, seed=1234, threads=os.cpu_count() or 1)
        o.set_state(sub)
        o.rebuild()
        nm = sum(len(a.ptr) - 1 for a in m.atoms) + int(round(4.0 * N))
        lim = min(nm, args.cpu_moves)
        t0 = time.perf_counter()
        o.class_pass_range(1 + args.warmup + args.steps, 0, 0, lim)
        dt = time.perf_counter() - t0
        sweep_s = dt * (nm / lim) * 2 * R
        out["cpu_baseline"] = {"value": 1.0 / sweep_s, "unit": "local sweeps/s", "cores": os.cpu_count() or 1,
                               "kind": "port", "sample": f"the first {lim} of {nm} moves of one colour class of 1 "
                                                         f"replica ({dt:.1f} s), extrapolated to 2 classes and {R} "
                                                         f"replicas (local sweep only)"}
    print(json.dumps(out), flush=True)


def ess_case(args):
    """Capacity ESS/s of the plain and learned capacity steps at the benchmarked configuration over
    longer chains than the default line's: --warmup plain steps (untimed, from the bench's start
    state), then ess_arms with --ess-steps steps per arm from the chain state they reached."""
    from esmgb import build as B
    B.build()
    from esmgb import replicas as RP
    m, st, d = setup_chain(32)
    d.set_move_grid(2, 32)
    ctl = RP.ReplicaCtl(M=d.R)
    rng = np.random.Generator(np.random.PCG64(1))
    t0 = time.perf_counter()
    device_loop(d, m, ctl, 1, args.warmup, rng, None)
    d.sync(3600.0)
    warm = time.perf_counter() - t0
    arms = tuple(a for a in (args.arms or "plain,learned,da").split(",") if a)
    res = ess_arms(d, m, ctl, 1 + args.warmup, args.ess_steps, arms=arms)
    out = {"case": "ess", "workload": config_dict()["workload"], "warmup_steps": args.warmup, "warmup_s": warm,
           "steps_per_arm": args.ess_steps, "capacity_ess_per_s": {a: v["value"] for a, v in res.items()},
           "ratio_to_plain": {a: v.get("ratio_to_plain") for a, v in res.items() if a != "plain"}, "detail": res}
    print(json.dumps(out), flush=True)


def job_rate(pg, world, steps, seconds):
    """Whole-job rate of `world` ranks that each ran `steps` units: world * steps over the slowest
    rank's time (max over ranks, after which every rank holds the same value); (rate, seconds)."""
    if pg:
        import torch
        t = torch.tensor([float(seconds)], dtype=torch.float64)
        pg.all_reduce(t, op=pg.ReduceOp.MAX)
        seconds = float(t[0])
        pg.barrier()
    return world * steps / seconds, seconds


def config_dict():
    w = WORKLOAD
    return {"workload": "plain replica sampler on GPU: 40 nodes, 60 lines, T=8760 hourly, 64 replicas",
            "nodes": w["N"], "lines": w["L"], "T": w["T"], "replicas": w["R"], "chains_per_gpu": 1,
            "l2": "inputs larger than L2 (state arrays 0.9 GB per chain)", "parallelism": "independent chains per GPU"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=8)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-replicas", type=int, default=2)
    ap.add_argument("--T", type=int, default=0, help="--case small: steps (default 584)")
    ap.add_argument("--N", type=int, default=0, help="--case small: nodes (default 40)")
    ap.add_argument("--L", type=int, default=0, help="--case small: lines (default 1.5 N)")
    ap.add_argument("--R", type=int, default=0, help="--case small: replicas (default 64)")
    ap.add_argument("--models", type=int, default=96, help="--case batch: number of models")
    ap.add_argument("--schedule", default="move", choices=["move", "class"],
                    help="line moves of a class pass: one launch per move, or the whole class in one launch")
    ap.add_argument("--batch-mode", default="batch", choices=["batch", "streams"],
                    help="--case batch: one esm_batch (default) or every model on its own stream")
    ap.add_argument("--ess-steps", type=int, default=32,
                    help="steps of each arm of the capacity ESS/s measurement (plain, learned, delayed "
                         "acceptance); 0: none")
    ap.add_argument("--storage-ms", action="store_true",
                    help="operation sweeps include the storage sweeps: multiscale (probability 1/2) and long-range")
    ap.add_argument("--autotune", action="store_true", help="--case small: the autotuner picks the line-move grid")
    ap.add_argument("--grid", default="", help="line-move grid WPBxWPS (warps per block x per SM) instead of "
                                               "the autotuner's choice")
    ap.add_argument("--cpu-moves", type=int, default=64, help="--case n256: moves of the oracle's sample")
    ap.add_argument("--arms", default="", help="the arms measured: --case ess (default plain,learned,da), "
                    "--case learned (default plain,plain4,sur1,surinf)")
    ap.add_argument("--sep", type=int, default=0, help="--case small: cooperative walk of separable moves of "
                                                     "at least this many units (0: off)")
    ap.add_argument("--case", default="full", choices=["full", "small", "batch", "storage", "n256", "ess", "mlp", "learned"],
                    help="small: the reduced profiling case (sweeps only, no JSON contract line)")
    args = ap.parse_args()
    if args.case == "small":
        return profile_case(args)
    if args.case == "batch":
        return batch_case(args)
    if args.case == "storage":
        return storage_case(args)
    if args.case == "n256":
        return n256_case(args)
    if args.case == "ess":
        return ess_case(args)
    if args.case == "mlp":
        return mlp_case(args)
    if args.case == "learned":
        return learned_case(args)
    rank, world, local = rank_info()
    if world > 1 and "CUDA_VISIBLE_DEVICES" not in os.environ:
        os.environ["CUDA_VISIBLE_DEVICES"] = str(local)
    if args.impl == "reference":
        return run_reference(args)
    pg = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo", init_method="env://")
        pg = dist
    from esmgb import build as B
    B.build()
    from esmgb import replicas as RP
    m, st, d = setup_chain(32, storage_ms=int(args.storage_ms))
    if args.storage_ms:
        d.close()
        from esmgb.device import DeviceChain
        d = DeviceChain(m, WORKLOAD["R"], precision=32, seed=WORKLOAD["seed"], storage_ms=1, storage_long=1)
        d.upload(st)
    R = d.R
    # the line-move grid picked by the library's autotuner (one timed colour class per candidate,
    # state restored), untimed setup; --grid WPBxWPS fixes it instead (profiler runs)
    d.set_move_schedule(args.schedule)
    if args.grid:
        wpb, wps = (int(x) for x in args.grid.lower().split("x"))
        d.set_move_grid(wpb, wps)
        grid, grid_ms = d.move_grid()[:2], {}
    else:
        grid, grid_ms = d.autotune_moves(sweep=0)
    ctl = RP.ReplicaCtl(M=R)
    rng = np.random.Generator(np.random.PCG64(rank + 1))
    # iterations placed so that the timed region contains a weather burst (every 40 steps)
    it0 = 40 - args.warmup - args.steps // 2
    it0 = it0 if it0 > 0 else 40 + it0 % 40
    device_loop(d, m, ctl, it0, args.warmup, rng, None)
    pre = [schedule(ctl, it0 + args.warmup + q, R, rng) for q in range(args.steps)]
    d.sync(600.0)
    if pg:
        pg.barrier()
    launches0 = d.launch_count()
    d.set_timing(True)
    clk = Clocks()
    clk.start()
    t0 = time.perf_counter()
    counts = device_loop(d, m, ctl, it0 + args.warmup, args.steps, rng, pre, counts=True)
    d.sync(600.0)
    wall_dev = time.perf_counter() - t0
    clocks = clk.stop()
    kt = d.timing()
    launches = d.launch_count() - launches0
    dev_ms = sum(v[0] for v in kt.values())
    value, dev_s = job_rate(pg, world, args.steps, dev_ms / 1000.0)
    dev_ms = 1000.0 * dev_s
    # end to end through the public API, host driver included
    Rset = RP.ReplicaSet(M=R, eta_w=[5e-4] * len(m.carriers))
    d.sync(600.0)
    t0 = time.perf_counter()
    h2d, d2h = e2e_loop(d, m, ctl, Rset, it0 + args.warmup + args.steps, args.steps, rng)
    d.sync(600.0)
    e2e, e2e_wall = job_rate(pg, world, args.steps, time.perf_counter() - t0)
    # the storage multiscale sweep on its own (one forced sweep, every class pass), device time
    d.sync(600.0)
    d.set_timing(True)
    sms = d.storage_ms(it0 + args.warmup + 2 * args.steps, force=True)
    d.sync(600.0)
    sms_ms = d.timing()["storage"][0]
    sl = d.storage_long(it0 + args.warmup + 2 * args.steps)
    d.sync(600.0)
    sl_ms = d.timing()["storage"][0]
    d.set_timing(False)
    ess = ess_arms(d, m, ctl, it0 + args.warmup + 2 * args.steps + 1, args.ess_steps) if args.ess_steps > 0 else None
    if rank != 0:
        return
    # roofline of the dominant kernels (one colour class: k_prep_moves and one k_move launch per
    # move, timed together as one span): algorithmic bytes of one class pass = the compulsory FP32
    # state traffic of one colour class, 4 (11 N + 2 L) (T/2) R bytes
    N, L, T = m.N, m.L, m.T
    cls_ms, cls_n = kt["class_pass"]
    alg = 4 * (11 * N + 2 * L) * (T / 2) * R
    per = cls_ms / max(cls_n, 1) / 1000.0
    peak, kind = peaks()
    achieved = alg / per / 1e9 if per > 0 else 0.0
    moves = (sum(len(a.ptr) - 1 for a in m.atoms) + round(4.0 * N)) * T * R
    traffic = None
    prof = os.path.join(ROOT, "profiles", "linemove_traffic.json")
    if os.path.exists(prof):
        try:
            traffic = json.load(open(prof)).get("bytes_per_launch_full")
        except Exception:
            traffic = None
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": dev_ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded generator of the configuration)",
            "config": config_dict(),
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic, "peak_kind": kind,
                         "kernel": "k_prep_moves + k_move (the line moves of one colour class, one span)",
                         "note": ("the exact line sampler is latency-bound (per-lane walk scratch, divergent walks): "
                                  "the HBM bytes are the compulsory state; `traffic` is the measured DRAM traffic, "
                                  "mostly walk scratch")},
            "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h)},
            "gpu_launches": int(launches), "clocks": clocks,
            "move_grid": {"warps_per_block": grid[0], "warps_per_sm": grid[1], "schedule": d.move_schedule(),
                          "autotune_ms_per_class": {f"{a}x{b}": round(v, 1) for (a, b), v in grid_ms.items()}},
            "kernel_ms_per_step": {k: v[0] / args.steps for k, v in kt.items()},
            "line_moves_per_s": moves * args.steps / (dev_ms / 1000.0) * world,
            "moves": move_counts(counts),
            "storage_ms": {"ms_per_sweep": sms_ms, "moves": int(sms[0]), "moves_taken": int(sms[1]),
                           "note": "storage multiscale sweep (plateau moves) timed alone; it runs in half of "
                                   "the operation sweeps with --storage-ms"},
            "storage_long": {"ms_per_sweep": sl_ms, "moves": int(sl[0]), "moves_taken": int(sl[1]),
                             "note": "long-range storage sweep timed alone; every operation sweep with "
                                     "--storage-ms"},
            "wall_device_loop_s": wall_dev}
    if ess:
        line["capacity_ess_per_s"] = {
            "plain": ess["plain"]["value"], "learned": ess.get("learned", {}).get("value"),
            "delayed_acceptance": ess.get("da", {}).get("value"),
            "learned_over_plain": ess.get("learned", {}).get("ratio_to_plain"),
            "delayed_acceptance_over_plain": ess.get("da", {}).get("ratio_to_plain"),
            "steps_per_arm": args.ess_steps, "unit": "ESS/s",
            "note": ("min over carriers of the bulk ESS of the carrier totals per wall second, each arm from the same "
                     "chain state (after the timed and end-to-end steps) over the same weather schedule; "
                     "short chains: the ESS is of the steps measured, with the per-carrier detail below"),
            "detail": ess}
    if not args.no_cpu_baseline:
        try:
            from oracle import oracle as O
            O.build()
            threads = os.cpu_count() or 1
            v, dt = cpu_sample(threads, 1, args.cpu_replicas, int(args.storage_ms))
            line["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                                    "sample": f"after one untimed operation sweep from the start state, the next "
                                              f"operation sweep(s) and the scores of {args.cpu_replicas} of the 64 "
                                              f"replicas at T = 8760 ({dt:.1f} s), scaled to 64 replicas"}
        except Exception as e:  # the baseline is reported, never the target
            line["cpu_baseline"] = {"value": None, "unit": UNIT, "cores": 0, "kind": "port", "sample": f"failed: {e}"}
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
