"""Host side of the replica sampler: controls, weather schedule, gate, drift weights and the step
adaptation (src/replicas.jl sections 4-5), mirroring the reference's names and semantics.

These are the pieces the reference keeps on the host in its GPU port as well
(device/src/replica_run.jl:309): scalar bookkeeping per replica and step. The hot path (sweeps,
scores, Langevin step with dispatch following, weather draws) runs in libesmcuda.so through
:mod:`esmgb.device`.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np


@dataclass
class ReplicaCtl:
    """Settings of the replica sampler (``src/replicas.jl:484`` ReplicaCtl, defaults as there)."""
    M: int = 8
    inner: int = 1
    theta: float = 0.0
    burst_every: int = 40
    phi: float = 0.3
    window: int = 60
    window_prob: float = 0.5
    ffbs: bool = False
    comp: bool = True
    gate_min: int = 10
    gate_max: int = 30
    gate_min_window: int = 20
    gate_max_window: int = 60
    gate_win: int = 8
    gate_tol: float = 0.3
    eta_w: list = field(default_factory=list)
    kappa_s: list = field(default_factory=list)
    kappa_min: float = 1.0
    clip: float = 0.02
    box: bool = True
    probe_every: int = 20
    probe_len: int = 30
    probe_tail: int = 15
    probe_win: int = 10
    probe_avg: int = 3
    adapt: bool = True
    gap_hi: float = 0.10
    gap_lo: float = 0.05
    eta_min: float = 2e-5
    eta_max: float = 2e-3
    shrink: float = 0.7
    grow: float = 1.2
    lam: float = 0.0
    Phi: object = None


def weather_schedule(ctl: ReplicaCtl, it: int, j: int):
    """(angle, burst) of replica j (1-based) at step ``it`` (``src/replicas.jl:571``)."""
    nb = ctl.burst_every
    burst = nb > 0 and (it + (j - 1) * (nb // ctl.M)) % nb == 0
    if burst:
        th = math.acos(max(-1.0, min(1.0, math.cos(ctl.theta) * math.cos(ctl.phi)))) if ctl.theta > 0 else ctl.phi
    else:
        th = ctl.theta
    return th, burst


def categorical(p, u):
    """First index k (1-based) with u sum(p) <= sum_{i<=k} p_i (``src/replicas.jl:115``)."""
    t = u * sum(p)
    c = 0.0
    for k, pk in enumerate(p):
        c += pk
        if t <= c:
            return k + 1
    return len(p)


def window_bounds(T0: int, B: int, u: float):
    """Window [a, b] (1-based) of length B with a uniform start (``src/replicas.jl:167``)."""
    a = min(T0, 1 + math.floor(u * T0))
    return a, min(T0, a + B - 1)


def relaxation_indicator(gbuf, win: int):
    """``src/replicas.jl:634``: largest difference of the halves' mean normalised scores."""
    h = win // 2
    if not (len(gbuf) >= 2 * h and h >= 1):
        return math.inf
    n = len(gbuf)
    a = np.mean(np.asarray(gbuf[n - 2 * h:n - h], float), axis=0)
    b = np.mean(np.asarray(gbuf[n - h:n], float), axis=0)
    d = [abs(x - y) for x, y in zip(a, b) if math.isfinite(x) and math.isfinite(y)]
    return 0.0 if not d else max(d)


@dataclass
class ReplicaSet:
    """Per-chain replica bookkeeping (``src/replicas.jl:549``); the states live on the device."""
    M: int
    eta_w: list
    since: list = None
    window: list = None
    active: list = None
    gbuf: list = None
    hist: list = None
    gaps: list = None

    def __post_init__(self):
        self.since = [10 ** 9] * self.M if self.since is None else self.since
        self.window = [False] * self.M if self.window is None else self.window
        self.active = [True] * self.M if self.active is None else self.active
        self.gbuf = [[] for _ in range(self.M)] if self.gbuf is None else self.gbuf
        self.hist = [[] for _ in range(self.M)] if self.hist is None else self.hist
        self.gaps = [] if self.gaps is None else self.gaps
        self.eta_w = list(self.eta_w)


def update_gate(R: ReplicaSet, j: int, g, ctl: ReplicaCtl) -> bool:
    """``src/replicas.jl:651`` update_gate! (j 0-based)."""
    if ctl.burst_every == 0:
        R.active[j] = True
        return True
    if R.active[j]:
        return True
    R.gbuf[j].append(list(g))
    if len(R.gbuf[j]) > ctl.gate_win:
        R.gbuf[j].pop(0)
    gmin, gmax = (ctl.gate_min_window, ctl.gate_max_window) if R.window[j] else (ctl.gate_min, ctl.gate_max)
    if not R.since[j] >= gmin:
        return False
    R.active[j] = R.since[j] >= gmax or relaxation_indicator(R.gbuf[j], ctl.gate_win) < ctl.gate_tol
    if R.active[j]:
        R.gbuf[j].clear()
    return R.active[j]


def tilt_weights(lam: float, Phis, active):
    """``src/replicas.jl:303``: exp(lam Phi_j) over the active replicas, normalised."""
    active = list(active)
    if not any(active):
        active = [True] * len(active)
    a = np.array([lam * P if act else -math.inf for act, P in zip(active, Phis)])
    w = np.exp(a - a.max())
    return w / w.sum()


def uniform_weights(active):
    """``src/replicas.jl:310``: 1/M_active over the active replicas (all if none)."""
    active = list(active)
    if not any(active):
        active = [True] * len(active)
    w = np.array([1.0 if a else 0.0 for a in active])
    return w / w.sum()


def drift_weights(ctl: ReplicaCtl, Phis, active):
    """``src/replicas.jl:664``."""
    return uniform_weights(active) if ctl.Phi is None else tilt_weights(ctl.lam, Phis, active)


def replica_feature_names(m):
    """``src/replicas.jl:277`` replica_feature_names: the order of esm_replica_features' columns."""
    ren = sorted({int(g) for g, k in zip(m.unit_group, m.unit_kind) if k == 0})
    return (["load_GW"] + ["cf_" + m.carriers[g] for g in ren] + ["resload_mean_GW", "resload_peak_GW",
            "resload_7step_GW"] + [f"regime_{k + 1}" for k in range(m.K)] + ["regime_switches"])


def weather_features(m, z, reg, kref):
    """``src/replicas.jl:246`` weather_features and ``:274`` replica_features of one weather path
    (anomalies z [n0, T], regimes reg [T]) on the host, as esm_replica_features computes them on the
    device for every replica: the nodes' loads are series 0 .. N-1, the data map is the model's
    (load (x)+, availability logistic(x)), the residual load is taken at the reference capacities
    kref [K] of the renewable units. Used for the prior statistics of the tilt functional."""
    X = m.xbar + m.wscale[:, None] * np.asarray(z, float)
    D = np.maximum(X[: m.N], 0.0).sum(axis=0)
    kind = np.asarray(m.unit_kind)
    ren = np.flatnonzero(kind == 0)
    A = 1.0 / (1.0 + np.exp(-X[np.asarray(m.unit_series)[ren]]))
    Rs = (np.asarray(kref, float)[ren][:, None] * A).sum(axis=0)
    res = (D - Rs) / 1e3
    T = len(res)
    w7 = max(np.mean(res[np.arange(t, t + 7) % T]) for t in range(T))
    groups = np.asarray(m.unit_group)[ren]
    cf = [float(A[groups == g].mean()) for g in sorted(set(groups.tolist()))]
    reg = np.asarray(reg)
    freq = [float(np.mean(reg == k)) for k in range(m.K)]
    return np.array([D.mean() / 1e3, *cf, res.mean(), res.max(), w7, *freq, float(np.count_nonzero(np.diff(reg)))])


class TiltFunctional:
    """``src/replicas.jl:278`` TiltFunctional: Phi(x) = the annual mean residual load of a replica's
    weather at the fixed reference capacities kref [K], standardised by its prior mean and standard
    deviation, estimated from n exact prior draws (``:291``, stream rng). Called with a chain, it
    evaluates Phi for every replica of the chain (esm_replica_features)."""

    def __init__(self, m, kref, rng, n: int = 200):
        from .model import sample_weather
        self.kref = np.asarray(kref, float).copy()
        self.col = replica_feature_names(m).index("resload_mean_GW")
        v = []
        for _ in range(n):
            reg, z = sample_weather(m, rng)
            v.append(weather_features(m, z, reg, self.kref)[self.col])
        self.mu = float(np.mean(v))
        self.sigma = float(np.std(v, ddof=1))

    def __call__(self, dev):
        return (np.asarray(dev.replica_features(self.kref))[:, self.col] - self.mu) / self.sigma


def adapt_step(R: ReplicaSet, gap, ctl: ReplicaCtl) -> bool:
    """``src/replicas.jl:758`` adapt_step!: shrink/grow eta_w per k field from probe_avg probes."""
    R.gaps.append(list(gap))
    if len(R.gaps) < ctl.probe_avg:
        return False
    for f in range(len(R.eta_w)):
        v = [g[f] for g in R.gaps if math.isfinite(g[f])]
        if not v:
            continue
        gbar = sum(v) / len(v)
        if abs(gbar) > ctl.gap_hi:
            R.eta_w[f] = max(ctl.eta_min, R.eta_w[f] * ctl.shrink)
        elif abs(gbar) < ctl.gap_lo:
            R.eta_w[f] = min(ctl.eta_max, R.eta_w[f] * ctl.grow)
    R.gaps.clear()
    return True


def langevin_drift_w(k, g, eta, kappa_s):
    """``src/replicas.jl:357``: eta ((k + kappa_s) g + 1)."""
    return eta * ((np.asarray(k) + kappa_s) * np.asarray(g) + 1)


def interior_nodes(k, hi, lo=50.0):
    """``src/replicas.jl:475``: capacity above ``lo`` MW and below the box."""
    k = np.asarray(k)
    return (k > lo) & (k < np.asarray(hi) - 1)


def masked_mean(v, mask):
    v = np.asarray(v)
    return float(v[mask].mean()) if mask.any() else math.nan


def _div(a, b):
    """a / b with the IEEE result for every b, a zero of either sign included (the reference's
    Float64 division), not an error."""
    with np.errstate(divide="ignore", invalid="ignore"):
        return float(np.float64(a) / np.float64(b))


def masked_means(v, mask, groups, nfields):
    """``src/replicas.jl:477`` masked_means: per k field (a capacity group of the flat unit vector,
    ``groups`` [K]) the mean of v over its masked units, NaN where none."""
    v = np.asarray(v)
    groups = np.asarray(groups)
    return [masked_mean(v, mask & (groups == f)) for f in range(nfields)]


def record_hist(R: ReplicaSet, j: int, rs, ctl: ReplicaCtl):
    """``src/replicas.jl:690-693``: an active replica's score record r s joins its in-flight window
    of the last ``probe_win`` records."""
    if R.active[j]:
        R.hist[j].append(np.array(rs, float))
        if len(R.hist[j]) > ctl.probe_win:
            R.hist[j].pop(0)


def probe_candidate(R: ReplicaSet, ctl: ReplicaCtl):
    """``src/replicas.jl:717`` probe_candidate (0-based): among the active replicas with a full
    in-flight window (``probe_win`` score records), the one longest after its burst; None if none."""
    cand = [j for j in range(R.M) if R.active[j] and len(R.hist[j]) >= ctl.probe_win]
    if not cand:
        return None
    return max(cand, key=lambda j: (R.since[j], -j))


def probe_sweep0(it: int, ctl: ReplicaCtl) -> int:
    """The first sweep index of the probe at step ``it``: every probe draws from its own sweep
    indices of the probe streams (the reference's probe stream ``prngs[c]`` advances from probe to
    probe, src/replicas.jl:923)."""
    return it * ctl.probe_len


def lag_probe(dev, j: int, hist, ctl: ReplicaCtl, ratio: float, k, hi, it: int, groups=None, nfields=1):
    """``src/replicas.jl:733`` lag_probe at step ``it``: the device runs ``probe_len`` operation
    sweeps of a frozen copy of replica j (esm_lag_probe, sweep indices from probe_sweep0; the chain
    is unchanged) and returns the mean capacity score of the last ``probe_tail``; the gap of the
    in-flight scores (the mean of ``hist``, replica j's records of r s, r = beta_k / beta_v, as
    record_hist keeps them) against it is formed on the interior nodes, per k field (the capacity
    groups ``groups`` of the units; one field over all units without them):
    gap = (<r s_in> - <r s_eq>) / <fk>."""
    sk_eq, fk = dev.lag_probe(j, ctl.probe_len, ctl.probe_tail, probe_sweep0(it, ctl))
    inflight = np.mean(np.asarray(hist, float), axis=0)
    mask = interior_nodes(k, hi)
    if groups is None:
        groups, nfields = np.zeros(len(mask), int), 1
    rs_eq = masked_means(ratio * sk_eq, mask, groups, nfields)
    rs_in = masked_means(inflight, mask, groups, nfields)
    fkm = masked_means(fk, mask, groups, nfields)
    gap = [_div(a - b, c) for a, b, c in zip(rs_in, rs_eq, fkm)]
    return {"gap": gap, "rs_eq": rs_eq, "rs_in": rs_in, "fk": fkm}


def init_replicas(dev, s0, ctl: ReplicaCtl, nsweeps: int, rng, it: int = 0, sweep0: int = 0) -> ReplicaSet:
    """``src/replicas.jl:785`` init_replicas on a chain `dev` (upload / weather_step / sweeps of the
    C ABI): its R replicas start at the capacities and operation of `s0` (its first replica), each
    with a fresh exact weather draw, the compensated initialisation of the dispatch and `nsweeps`
    operation sweeps at fixed k.

    The draw is made in two parts: the regime paths from the prior chain on the host
    (sample_weather_batch, the recursion of sample_weather), then the anomalies from the prior given
    those paths by the device's weather step at pCN angle pi/2 (the rotation keeps a weight of
    cos(pi/2) ~ 6e-17 of the old innovations; replica j's normals come from its stream of step
    `it`). The uploaded anomalies are those of s0, so the weather step's compensate_weather!
    measures the residual change against the residual of s0, as the reference's r0. Returns the
    chain's ReplicaSet."""
    from .model import sample_weather_batch
    m, R = dev.m, dev.R
    get = (lambda k: s0[k]) if isinstance(s0, dict) else (lambda k: getattr(s0, k))
    st = {k: np.repeat(np.asarray(get(k), float)[..., :1], R, axis=-1) for k in ("theta", "g", "e", "z")}
    st["reg"], _ = sample_weather_batch(m, R, rng)
    st["k"] = np.asarray(get("k"), float)
    dev.upload(st)
    dev.weather_step(np.ones(R, np.int32), np.full(R, math.pi / 2), np.zeros(R, np.int32), np.ones(R, np.int32),
                     it=it)
    if nsweeps > 0:
        dev.sweeps(nsweeps, sweep0)
    return ReplicaSet(M=R, eta_w=list(ctl.eta_w))


def replica_schedule(ctl: ReplicaCtl, it: int, M: int, T: int, rng):
    """The weather draws of every replica at step ``it`` (replica_weather!, src/replicas.jl:586-606:
    weather_schedule, the window coin and its start): (moved, angle, window, window start (1-based),
    burst) per replica, as the arrays esm_weather_step takes."""
    moved = np.zeros(M, np.int32)
    theta = np.zeros(M)
    window = np.zeros(M, np.int32)
    wstart = np.ones(M, np.int32)
    bursts = np.zeros(M, bool)
    for j in range(M):
        th, burst = weather_schedule(ctl, it, j + 1)
        regime = (burst or ctl.burst_every == 0) and ctl.window > 0
        win = regime and rng.random() < ctl.window_prob
        theta[j] = th
        bursts[j] = burst
        if th > 0 or win:
            moved[j] = 1
        if win:
            window[j] = ctl.window
            wstart[j] = window_bounds(T, ctl.window, rng.random())[0]
    return moved, theta, window, wstart, bursts


def replica_step(dev, R: ReplicaSet, ctl: ReplicaCtl, it: int, rng, kappa_s, ratio: float, hi, groups,
                 Phis=None):
    """``src/replicas.jl:676`` replica_step! for the chain `dev` (the C ABI's calls): the weather
    step of the replicas the schedule moves (with the gate reset at a burst), ``ctl.inner``
    operation sweeps (sweep indices it·inner …), the capacity scores, per replica its gate and
    in-flight record, the drift weights and one Langevin step of the shared capacities with
    dispatch following (step ``R.eta_w`` per k field, offsets ``kappa_s`` per field). ``ratio`` is
    beta_k / beta_v, ``hi`` the capacity box, ``groups`` the k field of each unit. Returns the
    step's record: moved, scores, prior terms, weights, the capacities before and after, the clip
    count, the masked field means of r s-bar and fk, and the bytes copied each way."""
    M = dev.R
    nf = len(R.eta_w)
    moved, theta, window, wstart, bursts = replica_schedule(ctl, it, M, dev.m.T, rng)
    h2d = d2h = 0
    for j in range(M):
        if bursts[j]:
            R.since[j], R.window[j], R.active[j] = 0, bool(window[j] > 0), False
            R.gbuf[j].clear()
            R.hist[j].clear()
        else:
            R.since[j] += 1
    if moved.any():
        dev.weather_step(moved, theta, window, wstart, it=it)
        h2d += moved.nbytes + theta.nbytes + window.nbytes + wstart.nbytes
    dev.sweeps(ctl.inner, it * ctl.inner, stats=False)
    sk, fk, parts = dev.scores()
    kraw = dev.download_k()
    d2h += sk.nbytes + fk.nbytes + parts.nbytes + kraw.nbytes
    mask = interior_nodes(kraw, hi)
    groups = np.asarray(groups)
    fmask = [mask & (groups == f) for f in range(nf)]
    fkm = [float(fk[fm].mean()) if fm.any() else math.nan for fm in fmask]
    rsk = ratio * sk
    rs_all = np.stack([rsk[:, fm].mean(axis=1) if fm.any() else np.full(M, math.nan) for fm in fmask], axis=1)
    for j in range(M):
        update_gate(R, j, [_div(a, b) for a, b in zip(rs_all[j].tolist(), fkm)], ctl)
        record_hist(R, j, rsk[j], ctl)
    if Phis is None:   # Phi of every replica's weather after its weather step (src/replicas.jl:691)
        Phis = np.zeros(M) if ctl.Phi is None else np.asarray(ctl.Phi(dev), float)
    wts = drift_weights(ctl, Phis, R.active)
    eta = np.asarray(R.eta_w, float)
    ks = np.asarray(kappa_s, float)
    knew, nclip = dev.langevin_step(wts, eta, ks, ctl.kappa_min, ctl.clip, ctl.box, None, it)
    h2d += wts.nbytes + eta.nbytes + ks.nbytes
    d2h += knew.nbytes
    sbar = np.asarray(wts) @ sk
    return {"it": it, "moved": moved.astype(bool), "sk": sk, "fk": fk, "parts": parts, "wts": wts, "Phis": Phis,
            "kraw": kraw,
            "knew": knew, "nclip": nclip, "rs": masked_means(ratio * sbar, mask, groups, nf), "fkm": fkm,
            "h2d": h2d, "d2h": d2h}


LANGEVIN_ETA = 5e-4   # the initial Langevin step of every k field (langevin_eta, src/run.jl:105)


REPLICA_TRACE_KEYS = ("ktot", "capex", "op", "shed", "penalty", "pfcost", "weights", "active", "since", "phi", "rs",
                      "fk", "eta_w", "nclip", "moved", "time", "features")   # src/replicas.jl:807


def replica_record(dev, R: ReplicaSet, rec, kref, groups, nf, t):
    """``src/replicas.jl:811`` replica_record: the per-step record of a chain's replicas, keyed as
    REPLICA_TRACE_KEYS -- the capacity totals per k field, the capex and per replica the operational
    cost, shed, penalty and generation-plus-storage-plus-capex cost (the cost parts of the step's
    score call: capex, op, gen, storage, shed, dump, penalty), the drift weights, gates and Phi, the
    field means, the step sizes, the clip count, the weather moves, the times (since the run's start
    and of the step) and the replicas' weather features at the reference capacities, stacked
    replica by replica."""
    parts = np.asarray(rec["parts"], float)
    knew = np.asarray(rec["knew"], float)
    feats = np.asarray(dev.replica_features(kref), float).reshape(-1)
    return {"ktot": [float(np.sum(knew[groups == f])) for f in range(nf)], "capex": [float(parts[0, 0])],
            "op": parts[:, 1], "shed": parts[:, 4], "penalty": parts[:, 6],
            "pfcost": parts[:, 0] + parts[:, 2] + parts[:, 3], "weights": np.asarray(rec["wts"], float),
            "active": np.asarray(R.active, float), "since": np.minimum(np.asarray(R.since, float), 1e6),
            "phi": np.asarray(rec["Phis"], float), "rs": rec["rs"], "fk": rec["fkm"], "eta_w": list(R.eta_w),
            "nclip": [float(rec["nclip"])], "moved": np.asarray(rec["moved"], float), "time": t, "features": feats}


def run_replicas(dev, s0, ctl: ReplicaCtl, nwarm: int, nprod: int, rng, *, kappa_s, ratio: float, hi, groups,
                 seed: int, init_sweeps: int = 2, snapshot_path=None, snapshot_every: int = 0,
                 tilt_functional=None, tilt_samples: int = 200):
    """``src/replicas.jl:841`` run_replicas for one chain on `dev` (the C ABI's calls; no
    configuration system, logs or output files): resume from ``snapshot_path`` when it holds a
    snapshot of this chain (read_replica_snapshot with its checks), else init_replicas from `s0`;
    then the steps up to nwarm + nprod (replica_step), each recorded by replica_record; every
    ``probe_every`` steps the lag probe of probe_candidate (the chain must be created with the probe
    context) with the step adaptation during the warm-up (adapt_step, ``:921-926``); a snapshot
    every ``snapshot_every`` steps before the last (boundary!). The reference capacities of the
    features and of the tilt are s0's (``:863``); tilt_functional "resload_mean" declares the tilt
    (TiltFunctional from tilt_samples exact draws of the stream seed + 5151, ``:865``; its lambda is
    ctl.lam). Returns (ReplicaSet, step records, probe records), the records as dictionaries of
    per-step vectors, as the snapshot's trace and probe groups keep them."""
    import time as _time

    from . import snapshot as SN
    groups = np.asarray(groups)
    nf = int(groups.max()) + 1
    eta_w = list(ctl.eta_w) if ctl.eta_w else [LANGEVIN_ETA] * nf
    kref = np.asarray(s0["k"] if isinstance(s0, dict) else s0.k, float).copy()
    if tilt_functional is not None:
        if tilt_functional != "resload_mean":
            raise ValueError(f"unknown tilt functional {tilt_functional!r} (the reference's: 'resload_mean')")
        ctl.Phi = TiltFunctional(dev.m, kref, np.random.Generator(np.random.PCG64(seed + 5151)), n=tilt_samples)
    t_start = _time.perf_counter()
    snap = SN.read_replica_snapshot(snapshot_path, seed=seed, shapes=dev.shapes()) if snapshot_path else None
    if snap is not None:
        R = ReplicaSet(M=dev.R, eta_w=eta_w)
        SN.resume_chain(snap["sets"][0], dev, R)
        it0, trace, probes = snap["it"], snap["sets"][0]["trace"], snap["sets"][0]["probe"]
        restarts = snap["restarts"] + 1
    else:
        R = init_replicas(dev, s0, ctl, init_sweeps, rng)
        R.eta_w = eta_w
        it0, trace, probes, restarts = 0, {}, {}, 0
    for it in range(it0 + 1, nwarm + nprod + 1):
        t1 = _time.perf_counter()
        rec = replica_step(dev, R, ctl, it, rng, kappa_s, ratio, hi, groups)
        t2 = _time.perf_counter()
        trace.setdefault("it", []).append(np.asarray([it], float))
        for key, val in replica_record(dev, R, rec, kref, groups, nf, [t2 - t_start, t2 - t1]).items():
            trace.setdefault(key, []).append(np.asarray(val, float))
        if ctl.probe_every > 0 and it % ctl.probe_every == 0:
            j = probe_candidate(R, ctl)
            if j is not None:
                pr = lag_probe(dev, j, R.hist[j], ctl, ratio, rec["knew"], hi, it, groups, nf)
                eta0 = list(R.eta_w)
                adapted = ctl.adapt and it <= nwarm and adapt_step(R, pr["gap"], ctl)
                for key, val in (("it", [it, j]), ("gap", pr["gap"]), ("eta_before", eta0),
                                 ("eta_after", list(R.eta_w)), ("adapted", [float(adapted)])):
                    probes.setdefault(key, []).append(np.asarray(val, float))
        if snapshot_path and snapshot_every > 0 and it % snapshot_every == 0 and it < nwarm + nprod:
            SN.write_replica_snapshot(snapshot_path, [{"chain": dev, "set": R, "trace": trace, "probe": probes}],
                                      it=it, seed=seed, phase="warmup" if it < nwarm else "production",
                                      where=f"step {it}", restarts=restarts)
    return R, trace, probes

