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
    """What the trained network gains, and what it costs. SurrogateLangevin (the surrogate's drift at
    4x the plain step) against the plain step from one saved state, one plain evaluation per
    iteration each. With its judge off the chain uses the surrogate's drift every iteration and its
    capacities move much farther per plain evaluation than the plain step's (asserted: the mean
    squared jump of w = log(k + kappa_s) per plain evaluation is at least twice the plain step's);
    the carrier means it reaches are printed beside the plain chain's (the longer runs of
    bench.py --case learned show them shifted by several MCSE: one sweep per step does not keep the
    replicas' dispatch, on which the plain estimates are taken, in step with 4x faster capacities).
    With its judge on, the surrogate is used only while its drift agrees with the plain estimates
    within their noise (asserted: the bookkeeping of learned and plain iterations adds up)."""
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
    W, KT = [], []
    for it in range(n):
        d.sweeps(1, sweep0=2000 + it, stats=False)
        d.scores()
        k, _ = d.langevin_step(w, eta, ks, 1.0, 0.02, True, None, 2000 + it)
        W.append(np.log(k + ks[ug]))
        KT.append(np.bincount(ug, weights=k, minlength=len(m.carriers)))
    msj_plain = np.mean(np.sum(np.diff(np.array(W)[:, mv], axis=0) ** 2, axis=1))
    kt_plain = np.mean(KT, axis=0)
    out = {}
    for tol in (float("inf"), 1.0):
        d.state_restore()
        sl = SurrogateLangevin(d, m, sur, eta, ks, mult=4.0, seed=2, train_steps=2, tol=tol)
        W, KT = [], []
        for it in range(n):
            sl.step(2000 + it)
            W.append(np.log(sl.k + ks[ug]))
            KT.append(np.bincount(ug, weights=sl.k, minlength=len(m.carriers)))
        W = np.array(W)
        assert np.all(np.isfinite(W))
        msj = np.mean(np.sum(np.diff(W[:, mv], axis=0) ** 2, axis=1))
        st = sl.stats
        assert st["plain_evals"] == st["iters"] + 1 == n + 1
        assert 0 <= st["learned"] <= st["iters"]
        out[tol] = (msj, st["learned"], np.mean(KT, axis=0))
        print(f"surrogate drift (judge tolerance {tol}): msjd per plain evaluation {msj:.3e} vs plain "
              f"{msj_plain:.3e} (ratio {msj / msj_plain:.2f}); surrogate steps {st['learned']}/{st['iters']}; "
              f"carrier means / plain's: {np.round(out[tol][2] / kt_plain, 3).tolist()}")
    msj_free, used_free, _ = out[float("inf")]
    assert used_free >= 0.8 * n        # judge off: the surrogate's drift wherever its prediction is in range
    assert msj_free >= 2.0 * msj_plain
    sur.close()
    d.close()
