"""The learned part: the online surrogate of the replica-averaged score (BF16 tensor-core MLP
trained on the plain sampler's pairs) and the delayed-acceptance capacity step. Shows what the
trained network gains over the plain step on a small model: the mean squared jump of the
capacities in w = log(k + kappa_s) per plain evaluation (equal cost per iteration), printed;
asserted are the mechanics (training lowers the loss; a rejected proposal leaves the state as it
was; the bookkeeping adds up)."""
import numpy as np
import pytest

from esmgb.device import DeviceChain
from esmgb.model import LANGEVIN_KAPPA, initial_state, make_model
from esmgb.surrogate import DALangevin, ScoreSurrogate

pytestmark = pytest.mark.gpu


def _setup(T=120, R=16):
    m = make_model(40, 60, T, seed=5)
    eta = np.full(len(m.carriers), 5e-4)
    ks = np.array([LANGEVIN_KAPPA.get(c, 100.0) for c in m.carriers])
    d = DeviceChain(m, R, precision=32, seed=3)
    d.upload(initial_state(m, R, seed=7))
    return m, d, eta, ks


def test_surrogate_learns_and_da_mechanics():
    m, d, eta, ks = _setup()
    ug = np.asarray(m.unit_group)
    mv = eta[ug] > 0
    R = d.R
    w = np.full(R, 1.0 / R)
    sur = ScoreSurrogate(m, hidden=(256, 256), capacity=2048, batch=256, lr=1e-3, seed=1)
    for it in range(160):                                 # plain steps; the surrogate learns from them
        d.sweeps(1, sweep0=it, stats=False)
        sk, fk, _ = d.scores()
        k = d.download_k()
        sur.add(k, d.regime_occupancy(), w @ sk)
        sur.train(4)
        d.langevin_step(w, eta, ks, 1.0, 0.02, True, None, it)
    losses = [x for x in sur.losses if x is not None]
    assert np.mean(losses[-20:]) < np.mean(losses[:20])
    # a proposal rejected at stage 2 restores the saved state exactly
    d.state_save()
    before = d.download()
    knew = before["k"].copy()
    knew[mv] *= 1.01
    d.follow_capacities(knew)
    d.sweeps(1, sweep0=500, stats=False)
    d.state_restore()
    after = d.download()
    for key in ("theta", "g", "e", "z", "k"):
        assert np.array_equal(before[key], after[key]), key
    # plain vs delayed acceptance from the same state, one plain evaluation per iteration each
    d.state_save()
    n = 60
    W = []
    for it in range(n):
        d.sweeps(1, sweep0=1000 + it, stats=False)
        d.scores()
        k, _ = d.langevin_step(w, eta, ks, 1.0, 0.02, True, None, 1000 + it)
        W.append(np.log(k + ks[ug]))
    msj_plain = np.mean(np.sum(np.diff(np.array(W)[:, mv], axis=0) ** 2, axis=1))
    d.state_restore()
    da = DALangevin(d, m, sur, eta, ks, mult=4.0, seed=2, train_steps=2)
    W = []
    for it in range(n):
        da.step(1000 + it)
        W.append(np.log(da.k + ks[ug]))
    msj_da = np.mean(np.sum(np.diff(np.array(W)[:, mv], axis=0) ** 2, axis=1))
    st = da.stats
    print(f"learned vs plain: msjd per plain evaluation {msj_da:.3e} vs {msj_plain:.3e} "
          f"(ratio {msj_da / msj_plain:.3f}); stage-1 passes {st['stage1']}/{st['iters']}, accepted {st['accepted']}")
    assert st["plain_evals"] == st["iters"] == n
    assert st["accepted"] <= st["stage1"] <= st["iters"]
    assert np.isfinite(msj_da) and np.isfinite(msj_plain)
    sur.close()
    d.close()


def test_surrogate_langevin_mixing():
    """SurrogateLangevin (the surrogate's drift at 4x the plain step, judged by the plain scores)
    against the plain step from one saved state, one plain evaluation per iteration each: the mean
    squared jump of w = log(k + kappa_s) per plain evaluation, printed with the share of iterations
    that used the surrogate; asserted: the states stay finite and the bookkeeping adds up."""
    from esmgb.surrogate import SurrogateLangevin
    m, d, eta, ks = _setup()
    ug = np.asarray(m.unit_group)
    mv = eta[ug] > 0
    R = d.R
    w = np.full(R, 1.0 / R)
    sur = ScoreSurrogate(m, hidden=(512, 512, 512), capacity=2048, batch=1024, lr=1e-3, seed=1)
    for it in range(160):
        d.sweeps(1, sweep0=it, stats=False)
        sk, fk, _ = d.scores()
        sur.add(d.download_k(), d.regime_occupancy(), w @ sk)
        sur.train(4)
        d.langevin_step(w, eta, ks, 1.0, 0.02, True, None, it)
    d.state_save()
    n = 60
    W = []
    for it in range(n):
        d.sweeps(1, sweep0=2000 + it, stats=False)
        d.scores()
        k, _ = d.langevin_step(w, eta, ks, 1.0, 0.02, True, None, 2000 + it)
        W.append(np.log(k + ks[ug]))
    msj_plain = np.mean(np.sum(np.diff(np.array(W)[:, mv], axis=0) ** 2, axis=1))
    d.state_restore()
    sl = SurrogateLangevin(d, m, sur, eta, ks, mult=4.0, seed=2, train_steps=2)
    W = []
    for it in range(n):
        sl.step(2000 + it)
        W.append(np.log(sl.k + ks[ug]))
    W = np.array(W)
    msj = np.mean(np.sum(np.diff(W[:, mv], axis=0) ** 2, axis=1))
    st = sl.stats
    print(f"surrogate drift vs plain: msjd per plain evaluation {msj:.3e} vs {msj_plain:.3e} "
          f"(ratio {msj / msj_plain:.3f}); surrogate steps {st['learned']}/{st['iters']}, "
          f"judged discrepancy {np.mean(np.abs(sl.z[mv])):.3f}")
    assert np.all(np.isfinite(W))
    assert st["plain_evals"] == st["iters"] + 1
    sur.close()
    d.close()
