"""replica_step (replica_step!, src/replicas.jl:676-704) and bench.py's end-to-end loop over the
chain calls of the C ABI, run here on the oracle behind the same calls: the schedule's bursts reset
the gates, the active replicas keep their in-flight records, the shared capacities take one
Langevin step, and the bytes each way are those of the arrays copied."""
import math

import numpy as np
import pytest

import bench
from esmgb import replicas as RP
from esmgb.model import LANGEVIN_KAPPA, initial_state, make_model
from oracle.oracle import Oracle


class OracleChain:
    """The calls of the device chain that replica_step makes, on the oracle."""

    def __init__(self, o):
        self.o, self.m, self.R = o, o.m, o.R

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


def chain(R=4, T=40):
    m = make_model(12, 18, T, seed=4)
    o = Oracle(m, R, seed=3)
    o.set_state(initial_state(m, R, seed=2))
    return m, OracleChain(o)


def test_replica_step_gates_records_and_capacities():
    m, ch = chain()
    R = 4
    ctl = RP.ReplicaCtl(M=R, burst_every=4, window=8, probe_win=3)
    Rs = RP.ReplicaSet(M=R, eta_w=[5e-4] * len(m.carriers))
    ks = np.array([LANGEVIN_KAPPA.get(c, 100.0) for c in m.carriers])
    rng = np.random.Generator(np.random.PCG64(5))
    ratio = m.beta_k / m.beta_v
    k_prev = ch.download_k().copy()
    for it in range(1, 6):
        since0 = list(Rs.since)
        h0 = [len(h) for h in Rs.hist]
        rec = RP.replica_step(ch, Rs, ctl, it, rng, ks, ratio, m.unit_hi, m.unit_group)
        for j in range(R):
            burst = (it + j) % 4 == 0          # weather_schedule: (it + (j - 1) * (4 // 4)) mod 4, j 1-based
            assert Rs.since[j] == (0 if burst else since0[j] + 1)
            if burst:                           # moved, gate reset and closed, window emptied
                assert rec["moved"][j] and not Rs.active[j] and len(Rs.hist[j]) == 0
            elif Rs.active[j]:                  # an active replica records its score
                assert len(Rs.hist[j]) == min(h0[j] + 1, ctl.probe_win)
            else:
                assert len(Rs.hist[j]) == h0[j]
        np.testing.assert_array_equal(rec["kraw"], k_prev)
        assert not np.array_equal(rec["knew"], rec["kraw"])   # the capacities moved
        k_prev = rec["knew"]
        np.testing.assert_array_equal(ch.download_k(), rec["knew"])
        assert math.isclose(sum(rec["wts"]), 1.0)
        assert len(rec["rs"]) == len(rec["fkm"]) == len(m.carriers)
        K = m.Kunits
        assert rec["d2h"] == 8 * (R * K + K + 8 * R + K + K)
        nmoved = 4 * R + 8 * R + 4 * R + 4 * R if rec["moved"].any() else 0
        assert rec["h2d"] == nmoved + 8 * R + 8 * len(m.carriers) * 2


def test_bench_e2e_loop_on_the_oracle():
    m, ch = chain()
    ctl = RP.ReplicaCtl(M=4)
    Rs = RP.ReplicaSet(M=4, eta_w=[5e-4] * len(m.carriers))
    h2d, d2h = bench.e2e_loop(ch, m, ctl, Rs, 10, 3, np.random.Generator(np.random.PCG64(1)))
    assert h2d > 0 and d2h == 8 * (4 * m.Kunits + 3 * m.Kunits + 32)


def test_bench_device_loop_counts_on_the_oracle():
    """The bench's timed loop with its correctness counters: the move counts of every sweep, summed,
    in the bench line's layout (tried and taken per family and for the atoms, guard events)."""
    m, ch = chain()
    ctl = RP.ReplicaCtl(M=4)
    st = bench.device_loop(ch, m, ctl, 10, 2, np.random.Generator(np.random.PCG64(1)), None, counts=True)
    mc = bench.move_counts(st)
    assert mc["tried"] == int(np.asarray(st)[:-1:2].sum()) > 0
    assert 0 < mc["taken"] <= mc["tried"] and mc["guards"] == 0
    assert set(mc["by_family"]) <= set(bench.FAMILIES) and "atoms" in mc["by_family"]
    assert sum(v[0] for v in mc["by_family"].values()) == mc["tried"]
    assert bench.device_loop(ch, m, ctl, 12, 1, np.random.Generator(np.random.PCG64(1)), None) is None


def test_weather_features_host():
    """weather_features (src/replicas.jl:246, :274) on the host: the load and residual-load columns
    from the data map directly, the residual load equal to the load without reference capacities,
    the regime frequencies summing to 1, the peak above the worst 7-step mean above the mean."""
    m, ch = chain()
    st = ch.o.get_state()
    z, reg = st["z"][:, :, 1], st["reg"][:, 1]
    names = RP.replica_feature_names(m)
    kref = np.asarray(m.unit_hi, float) * 0.3
    f = RP.weather_features(m, z, reg, kref)
    assert len(f) == len(names)
    X = m.xbar + m.wscale[:, None] * z
    D = np.maximum(X[: m.N], 0).sum(0)
    assert f[names.index("load_GW")] == pytest.approx(D.mean() / 1e3, rel=1e-13)
    f0 = RP.weather_features(m, z, reg, np.zeros(m.Kunits))
    assert f0[names.index("resload_mean_GW")] == pytest.approx(f0[names.index("load_GW")], rel=1e-13)
    i = names.index("resload_mean_GW")
    assert f[i + 1] >= f[i + 2] >= f[i] and f[i] < f0[i]
    freq = [f[names.index(f"regime_{k + 1}")] for k in range(m.K)]
    assert sum(freq) == pytest.approx(1.0) and f[-1] == np.count_nonzero(np.diff(reg))
    cfs = [f[j] for j, nm in enumerate(names) if nm.startswith("cf_")]
    assert len(cfs) >= 2 and all(0 < c < 1 for c in cfs)


def test_replica_step_stress_tilt():
    """replica_step with a declared tilt functional (TiltFunctional, src/replicas.jl:278; the
    reference's check "one step; lambda = 0 is the untilted step bitwise", test/test_replicas.jl:249):
    Phi of every replica from its weather, standardised by the prior statistics; at lambda = 0 the
    weights and the new capacities are those of the untilted step bit for bit; at lambda = 2 the
    weights are exp(lambda Phi) over the active replicas and the capacities move differently."""
    m, _ = chain()
    kref = np.asarray(m.unit_hi, float) * 0.3
    Phi = RP.TiltFunctional(m, kref, np.random.Generator(np.random.PCG64(2)), n=20)
    assert math.isfinite(Phi.mu) and Phi.sigma > 0
    ks = np.array([LANGEVIN_KAPPA.get(c, 100.0) for c in m.carriers])
    out = {}
    for lab, phi, lam in (("none", None, 0.0), ("zero", Phi, 0.0), ("two", Phi, 2.0)):
        _, ch = chain()
        ctl = RP.ReplicaCtl(M=4, burst_every=3, Phi=phi, lam=lam)
        Rs = RP.ReplicaSet(M=4, eta_w=[5e-4] * len(m.carriers))
        rec = RP.replica_step(ch, Rs, ctl, 1, np.random.Generator(np.random.PCG64(5)), ks, m.beta_k / m.beta_v,
                              m.unit_hi, m.unit_group)
        out[lab] = (rec, ch)
    (rn, _), (rz, chz), (r2, _) = out["none"], out["zero"], out["two"]
    assert np.array_equal(rz["wts"], rn["wts"]) and np.array_equal(rz["knew"], rn["knew"])
    assert np.allclose(rz["Phis"], (chz.replica_features(kref)[:, Phi.col] - Phi.mu) / Phi.sigma)
    assert np.all(rn["Phis"] == 0)
    act = rn["wts"] > 0
    w = np.where(act, np.exp(2.0 * r2["Phis"] - (2.0 * r2["Phis"][act]).max()), 0.0)
    np.testing.assert_allclose(r2["wts"], w / w.sum(), rtol=1e-14)
    assert not np.array_equal(r2["wts"], rz["wts"]) and not np.array_equal(r2["knew"], rz["knew"])


def test_lag_probe_per_field():
    class FakeDev:
        def lag_probe(self, j, n, tail, sweep0):
            return np.array([1.0, 2.0, 3.0, 4.0]), np.array([1.0, 1.0, 2.0, 2.0])

    ctl = RP.ReplicaCtl(M=2, probe_len=4, probe_tail=2)
    k = np.array([100.0, 100.0, 100.0, 10.0])
    pr = RP.lag_probe(FakeDev(), 0, [np.array([2.0, 2.0, 8.0, 8.0])], ctl, 1.0, k, np.full(4, 1e4), it=1,
                      groups=np.array([0, 0, 1, 1]), nfields=2)
    # field 0: units 0, 1: rs_in 2, rs_eq 1.5, fk 1; field 1: unit 2 only (unit 3 below 50 MW)
    assert pr["gap"] == [0.5, (8.0 - 3.0) / 2.0]
