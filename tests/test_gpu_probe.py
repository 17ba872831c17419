"""The lag probe on the CUDA path (esm_lag_probe; lag_probe, src/replicas.jl:733): a frozen copy of
one replica runs operation sweeps in the chain's one-replica probe context, on the probe's own
streams, and the chain is left unchanged.

The probe equals a one-replica chain started from the same replica with the probe seed (the
same kernels on the same state: scores to the round-off of their atomic accumulation, 1e-12 of
the largest score), and in FP64 it follows the oracle's one-replica chain (the reference's
loop of operation_sweep! and capacity_scores over a copy of the replica): units whose scores
differ beyond 1e-9 of the largest, at most 5 % (a flipped segment in one of the two sweeps moves
its unit's score; measured none)."""
import numpy as np
import pytest

from esmgb import replicas as RP
from esmgb.cabi import probe_seed
from esmgb.device import DeviceChain
from oracle.oracle import Oracle
from test_gpu_parity import make

pytestmark = pytest.mark.gpu

J, NSW, TAIL, SW0 = 7, 4, 2, 50


@pytest.fixture(scope="module")
def state():
    """The perturbed start after three oracle operation sweeps (near equilibrium)."""
    m, st = make(T=120)
    o = Oracle(m, 32, seed=21)
    o.set_state(st)
    o.sweeps(3, 100)
    s = o.get_state()
    for k in ("theta", "g", "e", "z", "reg", "k"):
        setattr(st, k, s[k])
    return m, st


def replica(s, j):
    return {k: (v if k == "k" else np.ascontiguousarray(v[..., j:j + 1])) for k, v in s.items()}


def chain_probe(ch, nsweeps, tail, sweep0):
    """The reference's probe loop on a one-replica chain (device or oracle)."""
    acc = 0.0
    for q in range(nsweeps):
        ch.sweeps(1, sweep0 + q)
        if q >= nsweeps - tail:
            sk, fk, _ = ch.scores()
            acc = acc + sk[0] / tail
    return acc, fk


@pytest.mark.parametrize("prec", [64, 32])
def test_probe_is_a_frozen_one_replica_chain(state, prec):
    m, st = state
    d = DeviceChain(m, 32, precision=prec, seed=5, probe=1)
    d.upload(st)
    d.sweeps(1, 0)
    before = d.download()
    sk, fk = d.lag_probe(J, NSW, TAIL, SW0)
    after = d.download()
    for k in before:
        np.testing.assert_array_equal(before[k], after[k], err_msg=k)
    c = DeviceChain(m, 1, precision=prec, seed=probe_seed(5))
    c.upload(replica(before, J))
    sk1, fk1 = chain_probe(c, NSW, TAIL, SW0)
    scale = np.abs(sk1).max() + 1e-30
    assert np.abs(sk - sk1).max() / scale < 1e-12
    np.testing.assert_array_equal(fk, fk1)
    sk2, _ = d.lag_probe(J, NSW, TAIL, SW0)     # the probe is repeatable
    assert np.abs(sk2 - sk).max() / scale < 1e-12


def test_probe_fp64_oracle(state):
    m, st = state
    d = DeviceChain(m, 32, precision=64, seed=5, probe=1)
    d.upload(st)
    s = d.download()
    sk, fk = d.lag_probe(J, 2, 2, SW0)
    o = Oracle(m, 1, seed=probe_seed(5))
    o.set_state(replica(s, J))
    sk0, fk0 = chain_probe(o, 2, 2, SW0)
    np.testing.assert_allclose(fk, fk0, rtol=1e-14)
    rel = np.abs(sk - sk0) / (np.abs(sk0).max() + 1e-30)
    print(f"probe vs oracle FP64: units {rel.size}, median {np.median(rel):.2e}, "
          f"above 1e-9 {np.mean(rel > 1e-9):.3f}, max {rel.max():.2e}")
    assert np.median(rel) < 1e-9
    assert np.mean(rel > 1e-9) <= 0.05          # measured 0 (largest difference 3e-13)


def test_probe_gap_and_errors(state):
    m, st = state
    d = DeviceChain(m, 32, precision=32, seed=5, probe=1)
    d.upload(st)
    ctl = RP.ReplicaCtl(M=32, probe_len=3, probe_tail=2)
    sk, fk, _ = d.scores()
    ratio = m.beta_k / m.beta_v
    hist = [ratio * sk[J], ratio * sk[J]]
    k = d.download_k()
    pr = RP.lag_probe(d, J, hist, ctl, ratio, k, m.unit_hi, it=20)
    assert np.isfinite(pr["gap"][0])
    bare = DeviceChain(m, 32, precision=32, seed=5)
    bare.upload(st)
    with pytest.raises(RuntimeError, match="probe"):
        bare.lag_probe(J)
    with pytest.raises(RuntimeError):
        d.lag_probe(32)
