"""run_replicas (src/replicas.jl:841) for one chain over the C ABI's calls, run here on the oracle
behind the same calls: initialisation, steps, lag probes with the step adaptation in the warm-up
only, periodic snapshots and a resume from one."""
import numpy as np

from esmgb import replicas as RP
from esmgb.cabi import probe_seed
from esmgb.model import LANGEVIN_KAPPA, initial_state, make_model
from oracle.oracle import Oracle

SEED = 3


class OracleChain:
    """The device chain's calls on the oracle; the lag probe on a one-replica oracle with the
    probe seed, as esm_lag_probe runs it."""

    def __init__(self, o):
        self.o, self.m, self.R = o, o.m, o.R

    def shapes(self):
        return self.o.shapes()

    def upload(self, st):
        self.o.set_state(st)

    def download(self):
        return self.o.get_state()

    def weather_step(self, *a, **kw):
        self.o.weather_step(*a, **kw)

    def sweeps(self, n, sweep0=0, stats=True):
        return self.o.sweeps(n, sweep0)

    def scores(self):
        return self.o.scores()

    def download_k(self):
        return self.o.get_state()["k"]

    def langevin_step(self, *a, **kw):
        return self.o.langevin_step(*a, **kw)

    def replica_features(self, kref):
        st = self.o.get_state()
        return np.stack([RP.weather_features(self.m, st["z"][:, :, j], st["reg"][:, j], kref) for j in range(self.R)])

    def lag_probe(self, j, nsweeps, tail, sweep0):
        s = self.o.get_state()
        c = Oracle(self.m, 1, seed=probe_seed(SEED))
        c.set_state({k: (v if k == "k" else np.ascontiguousarray(v[..., j:j + 1])) for k, v in s.items()})
        acc = 0.0
        for q in range(nsweeps):
            c.sweeps(1, sweep0 + q)
            if q >= nsweeps - tail:
                sk, fk, _ = c.scores()
                acc = acc + sk[0] / tail
        return acc, fk


def setup(R=4):
    m = make_model(12, 18, 40, seed=4)
    s0 = initial_state(m, 1, seed=2)
    ch = OracleChain(Oracle(m, R, seed=SEED))
    ks = np.array([LANGEVIN_KAPPA.get(c, 100.0) for c in m.carriers])
    kw = dict(kappa_s=ks, ratio=m.beta_k / m.beta_v, hi=m.unit_hi, groups=m.unit_group, seed=SEED, init_sweeps=1)
    return m, s0, ch, kw


def ctl_for(R):
    return RP.ReplicaCtl(M=R, burst_every=0, probe_every=2, probe_len=2, probe_tail=1, probe_win=1, probe_avg=1,
                         gap_lo=1e9, gap_hi=2e9, grow=1.5)


def test_run_replicas_probes_adapt_in_warmup_only(tmp_path):
    m, s0, ch, kw = setup()
    ctl = ctl_for(4)
    R, trace, probes = RP.run_replicas(ch, s0, ctl, 4, 2, np.random.Generator(np.random.PCG64(1)), **kw)
    assert [int(x[0]) for x in trace["it"]] == [1, 2, 3, 4, 5, 6]
    assert len(trace["ktot"][0]) == len(m.carriers)
    its = [int(x[0]) for x in probes["it"]]
    assert its == [2, 4, 6]
    adapted = [bool(x[0]) for x in probes["adapted"]]
    assert adapted == [True, True, False]           # |gap| < gap_lo grows the step, in the warm-up only
    for a, b, g, ad in zip(probes["eta_before"], probes["eta_after"], probes["gap"], adapted):
        fin = np.isfinite(g)
        if ad:
            assert np.all(b[fin] >= a[fin])
        else:
            np.testing.assert_array_equal(a, b)
    np.testing.assert_array_equal(R.eta_w, probes["eta_after"][-1])
    # the per-step record of the reference's driver (replica_record, src/replicas.jl:807-819)
    assert set(RP.REPLICA_TRACE_KEYS) <= set(trace)
    nfeat = len(RP.replica_feature_names(m))
    for key, n in (("capex", 1), ("op", 4), ("shed", 4), ("penalty", 4), ("pfcost", 4), ("weights", 4), ("active", 4),
                   ("since", 4), ("phi", 4), ("moved", 4), ("time", 2), ("features", 4 * nfeat),
                   ("eta_w", len(m.carriers)), ("nclip", 1)):
        assert all(len(v) == n for v in trace[key]), key
    assert all(np.all(v == 0) for v in trace["phi"])          # no tilt declared
    assert all(abs(v.sum() - 1) < 1e-12 for v in trace["weights"])
    k0 = np.asarray(s0.k, float)
    f0 = RP.weather_features(m, ch.o.get_state()["z"][:, :, 0], ch.o.get_state()["reg"][:, 0], k0)
    np.testing.assert_allclose(trace["features"][-1][:nfeat], f0, rtol=1e-12)


def test_run_replicas_declared_tilt():
    """tilt_functional "resload_mean" (src/replicas.jl:865): Phi from the replicas' weather, the
    drift weights exp(lambda Phi) over the active replicas, both recorded."""
    m, s0, ch, kw = setup()
    ctl = ctl_for(4)
    ctl.lam = 1.0
    R, trace, _ = RP.run_replicas(ch, s0, ctl, 2, 1, np.random.Generator(np.random.PCG64(1)),
                                  tilt_functional="resload_mean", tilt_samples=20, **kw)
    assert isinstance(ctl.Phi, RP.TiltFunctional)
    for phi, w, act in zip(trace["phi"], trace["weights"], trace["active"]):
        a = act > 0 if act.any() else np.ones(4, bool)
        e = np.where(a, np.exp(phi - phi[a].max()), 0.0)
        np.testing.assert_allclose(w, e / e.sum(), rtol=1e-13)
    assert np.ptp(trace["phi"][-1]) > 0


def test_run_replicas_snapshot_and_resume(tmp_path):
    m, s0, ch, kw = setup()
    path = str(tmp_path / "snap.npz")
    ctl = ctl_for(4)
    R1, trace1, _ = RP.run_replicas(ch, s0, ctl, 3, 2, np.random.Generator(np.random.PCG64(1)), snapshot_path=path,
                                    snapshot_every=2, **kw)
    from esmgb import snapshot as SN
    snap = SN.read_replica_snapshot(path, seed=SEED)
    assert snap["it"] == 4 and snap["phase"] == "production" and snap["restarts"] == 0
    assert [int(x[0]) for x in snap["sets"][0]["trace"]["it"]] == [1, 2, 3, 4]
    # a second run from the snapshot continues at step 5 with the saved records and step sizes
    ch2 = OracleChain(Oracle(m, 4, seed=SEED))
    R2, trace2, probes2 = RP.run_replicas(ch2, s0, ctl_for(4), 3, 2, np.random.Generator(np.random.PCG64(9)),
                                          snapshot_path=path, snapshot_every=2, **kw)
    assert [int(x[0]) for x in trace2["it"]] == [1, 2, 3, 4, 5]
    np.testing.assert_array_equal(trace2["ktot"][3], trace1["ktot"][3])
