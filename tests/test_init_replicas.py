"""init_replicas (src/replicas.jl:785) over the chain calls of the C ABI, run here on the oracle:
every replica starts at the operation and capacities of s0 with its own prior regime path and
anomalies, and the dispatchable units take up the residual change against s0's residual
(compensate_weather!, :207) wherever their headroom allows."""
import math

import numpy as np

from esmgb import replicas as RP
from esmgb.model import initial_state, make_model, sample_weather_batch
from oracle.oracle import Oracle


class OracleChain:
    """upload / weather_step / sweeps of the device chain, on the oracle."""

    def __init__(self, o):
        self.o, self.m, self.R = o, o.m, o.R

    def upload(self, st):
        self.o.set_state(st)

    def weather_step(self, *a, **kw):
        self.o.weather_step(*a, **kw)

    def sweeps(self, n, sweep0=0):
        return self.o.sweeps(n, sweep0)


def residual(m, st, R):
    o = Oracle(m, R, seed=1)
    o.set_state(st)
    o.rebuild()
    return o.caches()[0]


def test_init_replicas_fresh_weather_and_compensation():
    m = make_model(16, 24, 40, seed=3)
    s0 = initial_state(m, 1, seed=5)
    R = 6
    o = Oracle(m, R, seed=7)
    ch = OracleChain(o)
    ctl = RP.ReplicaCtl(M=R, eta_w=[1e-3])
    Rset = RP.init_replicas(ch, s0, ctl, 0, np.random.Generator(np.random.PCG64(11)), it=4)
    assert Rset.M == R and Rset.eta_w == [1e-3]
    st = o.get_state()
    reg_want, _ = sample_weather_batch(m, R, np.random.Generator(np.random.PCG64(11)))
    np.testing.assert_array_equal(st["reg"], reg_want)            # the prior regime paths
    for k in ("theta", "e"):                                     # operation of s0 in every replica
        np.testing.assert_array_equal(st[k], np.repeat(getattr(s0, k), R, axis=-1))
    np.testing.assert_array_equal(st["k"], s0.k)
    z = st["z"]
    assert not np.allclose(z[..., 0], z[..., 1])                 # fresh anomalies per replica
    assert not np.allclose(z[..., 0], s0.z[..., 0])
    # compensation against s0's residual: the dispatch moves only where the residual changed, and
    # the residual returns to s0's wherever the units' headroom (or output) covers the change
    r0 = residual(m, s0, 1)
    r_now = residual(m, st, R)
    raw = dict(st, g=np.repeat(s0.g, R, axis=-1))
    r_raw = residual(m, raw, R)                                  # new weather, s0's dispatch
    d_now, d_raw = np.abs(r_now - r0), np.abs(r_raw - r0)
    assert (d_now <= d_raw + 1e-6).all()
    moved = d_raw > 1e-6
    covered = np.mean(d_now[moved] < 1e-6)
    print(f"init: residual entries changed by the weather {moved.mean():.3f}, restored {covered:.3f}")
    assert moved.mean() > 0.5 and covered > 0.2


def test_init_replicas_sweeps():
    m = make_model(12, 18, 24, seed=4)
    s0 = initial_state(m, 1, seed=2)
    o = Oracle(m, 4, seed=7)
    RP.init_replicas(OracleChain(o), s0, RP.ReplicaCtl(M=4), 2, np.random.Generator(np.random.PCG64(1)), it=0,
                     sweep0=10)
    st = o.get_state()
    assert not np.array_equal(st["theta"], np.repeat(s0.theta, 4, axis=-1))   # the sweeps moved the angles
    assert math.isclose(float(np.abs(st["k"] - s0.k).max()), 0.0)              # at fixed k


def test_init_replicas_anomalies_are_prior_draws():
    """The anomalies init_replicas leaves are a draw from the prior given the new regime paths: their
    VAR innovations (src/replicas.jl:29-112, the diagonal VAR of the model) are independent standard
    normals (mean within 4 standard errors of 0, variance within 5 % of 1, lag-one correlation
    within 4 standard errors of 0)."""
    m = make_model(12, 18, 120, seed=3)
    s0 = initial_state(m, 1, seed=5)
    R = 16
    o = Oracle(m, R, seed=7)
    RP.init_replicas(OracleChain(o), s0, RP.ReplicaCtl(M=R), 0, np.random.Generator(np.random.PCG64(2)), it=1)
    st = o.get_state()
    z, reg = st["z"], st["reg"]
    T = m.T
    e = np.empty_like(z)
    e[:, 0, :] = z[:, 0, :] / m.sig0[:, None]
    for t in range(1, T):
        k = reg[t]                                           # [R]
        cs, sn = math.cos(2 * math.pi * (t + 1) / T), math.sin(2 * math.pi * (t + 1) / T)
        mean = (m.phi[k].T * z[:, t - 1, :] + m.mu[k, :, 0].T + cs * m.mu[k, :, 1].T + sn * m.mu[k, :, 2].T)
        e[:, t, :] = (z[:, t, :] - mean) / m.sig[k].T
    x = e.ravel()
    n = x.size
    lag = (e[:, 1:, :] * e[:, :-1, :]).mean()
    print(f"innovations: n {n}, mean {x.mean():.4f}, var {x.var():.4f}, lag-one {lag:.4f}")
    assert abs(x.mean()) < 4 / math.sqrt(n) and abs(x.var() - 1) < 0.05 and abs(lag) < 4 / math.sqrt(n)
