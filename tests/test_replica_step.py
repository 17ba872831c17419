"""replica_step (replica_step!, src/replicas.jl:676-704) and bench.py's end-to-end loop over the
chain calls of the C ABI, run here on the oracle behind the same calls: the schedule's bursts reset
the gates, the active replicas keep their in-flight records, the shared capacities take one
Langevin step, and the bytes each way are those of the arrays copied."""
import math

import numpy as np

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
