"""Parity of the CUDA path (through the C ABI) with the CPU oracle on identical states and the same
Philox streams (the reference's device verification protocol: same prepared moves, same random
numbers, compared exactly or to round-off; docs/system/testing.md).

Tolerances: FP64 kernels against the FP64 oracle 1e-9 relative per element, at most 1 % of
(step, replica) tasks allowed to differ beyond it (discrete flips at a segment boundary from
last-bit differences of the transcendental functions); FP32 kernels 2e-3 relative (4e-3 absolute on
utilisations), at most 5 % of tasks flipped. Scores (both builds form their terms in FP64): 1e-9
relative of the score scale, and bitwise repeatable."""
import numpy as np
import pytest

from esmgb.device import DeviceChain
from esmgb.model import make_model, initial_state
from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu


def _rel(a, b, scale):
    return np.abs(a - b) / (scale + np.abs(b))


def task_flips(sd, so, m, tol_rel, tol_abs):
    """Fraction of (step, replica) entries whose state differs beyond tolerance, and the largest
    difference among the others."""
    bad = np.zeros((m.T, so["g"].shape[2]), bool)
    th = np.nan_to_num(_rel(sd["theta"], so["theta"], 1.0 + np.abs(so["theta"]).max()), nan=np.inf).max(0)
    gg = np.nan_to_num(np.abs(sd["g"] - so["g"]), nan=np.inf).max(0)    # (a non-finite entry is a flip)
    ee = np.nan_to_num(np.abs(sd["e"] - so["e"]), nan=np.inf).max(0)
    bad |= th > tol_rel
    bad |= gg > tol_abs
    bad |= ee > tol_abs
    worst = max(th[~bad].max(initial=0), gg[~bad].max(initial=0), ee[~bad].max(initial=0))
    return bad.mean(), worst


def make(N=40, L=60, T=40, R=32, seed=11):
    """A non-degenerate state: the heuristic start (whose residuals cancel to round-off, so that
    their signs are set by last-bit differences) perturbed at random."""
    m = make_model(N, L, T, seed=seed)
    st = initial_state(m, R, seed=3)
    rng = np.random.Generator(np.random.PCG64(seed))
    st.g = st.g + 0.05 * rng.standard_normal(st.g.shape)
    st.e = rng.uniform(0.05, 0.95, st.e.shape)
    st.theta = 30.0 * rng.standard_normal(st.theta.shape)
    return m, st


@pytest.fixture(scope="module")
def base():
    return make()


@pytest.fixture(scope="module")
def equilibrated():
    """The perturbed state after three oracle sweeps: near equilibrium the line potentials of the
    moves span tens of nats, the regime the FP32 build is designed for (far from it a move's
    potential falls by thousands of nats, and FP32 resolves its minimum to ~1e-7 of that)."""
    m, st = make()
    o = Oracle(m, 32, seed=21)
    o.set_state(st)
    o.sweeps(3, 100)
    s = o.get_state()
    for k in ("theta", "g", "e", "z", "reg", "k"):
        setattr(st, k, s[k])
    return m, st


@pytest.mark.parametrize("prec", [64, 32])
def test_rebuild_caches(base, prec):
    m, st = base
    d = DeviceChain(m, 32, precision=prec, seed=5)
    d.upload(st)
    d.rebuild()
    r, F = d.caches()
    o = Oracle(m, 32, seed=5)
    o.set_state(st)
    o.rebuild()
    r0, F0 = o.caches()
    tol = 1e-12 if prec == 64 else 2e-6
    assert np.abs(r - r0).max() <= tol * (1 + np.abs(r0).max())
    assert np.abs(F - F0).max() <= tol * (1 + np.abs(F0).max())


def test_class_pass_fp64(base):
    """A whole colour class (every move of every task) of the FP64 build against the oracle."""
    m, st = base
    d = DeviceChain(m, 32, precision=64, seed=5)
    d.upload(st)
    d.rebuild()
    o = Oracle(m, 32, seed=5)
    o.set_state(st)
    o.rebuild()
    sd = d.class_pass(3, 0)
    so = o.class_pass(3, 0)
    assert np.array_equal(sd[:-1:2], so[:-1:2])           # the same moves were tried
    assert sd[-1] == so[-1] == 0                          # no guard events
    frac, worst = task_flips(d.download(), o.get_state(), m, 1e-9, 1e-9)
    print(f"FP64 class pass: flipped tasks {frac:.4f}, worst other {worst:.2e}")
    assert frac <= 0.02


@pytest.mark.parametrize("sep", [0, 2, 41])
def test_class_pass_fp64_walk_modes(base, sep):
    """The same class pass with the separable moves walked one task per lane (sep 0 and 41: no
    move has 41 units) or one task per warp (sep 2: every separable move): the same moves tried,
    no guard events, and the oracle's result on all but the flipped tasks."""
    m, st = base
    d = DeviceChain(m, 32, precision=64, seed=5)
    d.upload(st)
    d.set_sep_walk(sep)
    assert d.sep_walk()[0] == sep
    d.rebuild()
    o = Oracle(m, 32, seed=5)
    o.set_state(st)
    o.rebuild()
    sd = d.class_pass(3, 0)
    so = o.class_pass(3, 0)
    assert np.array_equal(sd[:-1:2], so[:-1:2])
    assert sd[-1] == so[-1] == 0
    frac, worst = task_flips(d.download(), o.get_state(), m, 1e-9, 1e-9)
    print(f"FP64 class pass, separable walk from {sep} units: flipped tasks {frac:.4f}, worst other {worst:.2e}")
    assert frac <= 0.02


@pytest.mark.parametrize("sep", [0, 2])
@pytest.mark.parametrize("limit", [1, 20])
def test_moves_fp32_walk_modes(equilibrated, sep, limit):
    """The first moves of every task of the FP32 build with either walk of the separable moves."""
    m, st = equilibrated
    d = DeviceChain(m, 32, precision=32, seed=5)
    d.upload(st)
    d.set_sep_walk(sep)
    d.rebuild()
    o = Oracle(m, 32, seed=5)
    o.set_state(st)
    o.rebuild()
    sd = d.class_pass(3, 1, limit)
    so = o.class_pass(3, 1, limit)
    assert np.array_equal(sd[:-1:2], so[:-1:2])
    frac, worst = task_flips(d.download(), o.get_state(), m, 2e-3, 4e-3)
    print(f"FP32 first {limit} moves, separable walk from {sep} units: flipped {frac:.4f}, worst other {worst:.2e}")
    assert frac <= 0.02


@pytest.mark.parametrize("wpb,wps", [(1, 8), (2, 0), (4, 0), (4, 16)])
def test_class_pass_fp64_grids(base, wpb, wps):
    """The same class pass with every k_move block shape and a reduced grid: the work items are
    taken from a per-move counter, so the grid must not change the result."""
    m, st = base
    d = DeviceChain(m, 32, precision=64, seed=5)
    d.upload(st)
    d.set_move_grid(wpb, wps)
    assert d.move_grid()[0] == wpb
    d.rebuild()
    o = Oracle(m, 32, seed=5)
    o.set_state(st)
    o.rebuild()
    sd = d.class_pass(3, 0)
    so = o.class_pass(3, 0)
    assert np.array_equal(sd[:-1:2], so[:-1:2])
    assert sd[-1] == so[-1] == 0
    frac, worst = task_flips(d.download(), o.get_state(), m, 1e-9, 1e-9)
    assert frac <= 0.02


def test_autotune_keeps_state(base):
    """esm_autotune_moves times candidate grids from the current state and restores it: the chain
    state after tuning equals the state before, and a sweep afterwards matches an untuned chain."""
    m, st = base
    d = DeviceChain(m, 32, precision=64, seed=5)
    d.upload(st)
    before = d.download()
    (wpb, wps), times = d.autotune_moves(sweep=3)
    assert (wpb, wps) in times and len(times) >= 3
    assert d.move_grid()[:2] == (wpb, wps)
    after = d.download()
    for k in ("theta", "g", "e", "z", "k"):
        assert np.array_equal(before[k], after[k]), k
    d2 = DeviceChain(m, 32, precision=64, seed=5)
    d2.upload(st)
    s1, s2 = d.sweeps(1, 4), d2.sweeps(1, 4)
    assert np.array_equal(s1, s2)
    a, b = d.download(), d2.download()
    assert (np.abs(a["g"] - b["g"]).max(0) > 1e-9).mean() <= 0.02


@pytest.mark.parametrize("limit", [1, 5, 20])
def test_moves_fp32(equilibrated, limit):
    """The first `limit` moves of every task of the FP32 build on identical states. A task whose
    state differs beyond tolerance had a discrete flip at one of its moves (the per-move flip rate
    is at most about frac / limit); once flipped, later moves of that task are not comparable."""
    m, st = equilibrated
    d = DeviceChain(m, 32, precision=32, seed=5)
    d.upload(st)
    d.rebuild()
    o = Oracle(m, 32, seed=5)
    o.set_state(st)
    o.rebuild()
    sd = d.class_pass(3, 1, limit)
    so = o.class_pass(3, 1, limit)
    assert np.array_equal(sd[:-1:2], so[:-1:2])
    frac, worst = task_flips(d.download(), o.get_state(), m, 2e-3, 4e-3)
    print(f"FP32 first {limit} moves: flipped tasks {frac:.4f}, worst other {worst:.2e}")
    assert frac <= 0.02


def test_class_pass_fp32_statistics(base):
    """A whole FP32 class pass: tasks diverge after a flip, so compare what the moves did in
    distribution: the mean absolute change of every field agrees with the oracle's to 5 %."""
    m, st = base
    d = DeviceChain(m, 32, precision=32, seed=5)
    d.upload(st)
    o = Oracle(m, 32, seed=5)
    o.set_state(st)
    d.sweeps(1, 0)
    o.sweeps(1, 0)
    a, b = d.download(), o.get_state()
    frac, _ = task_flips(a, b, m, 2e-3, 4e-3)
    print(f"FP32 sweep: tasks still within tolerance {1 - frac:.3f}")
    for k in ("theta", "g", "e"):
        ma = np.abs(a[k] - st.__dict__[k]).mean()
        mb = np.abs(b[k] - st.__dict__[k]).mean()
        assert abs(ma / mb - 1) < 0.05, (k, ma, mb)


def test_sweeps_fp64_odd_T_small_R():
    m, st = make(T=73, R=4)                               # three colour classes; 8 steps per warp
    d = DeviceChain(m, 4, precision=64, seed=9)
    d.upload(st)
    o = Oracle(m, 4, seed=9)
    o.set_state(st)
    sd = d.sweeps(1, 10)
    so = o.sweeps(1, 10)
    assert np.array_equal(sd[:-1:2], so[:-1:2])
    frac, worst = task_flips(d.download(), o.get_state(), m, 1e-9, 1e-9)
    print(f"odd T: flipped {frac:.4f}, worst {worst:.2e}")
    assert frac <= 0.03


def test_class_pass_large_model_global_scratch():
    """A 128-node model: its lane layout exceeds the lanes' local arrays, so the walks use the
    global per-block slabs (interleaved by lane). The first 20 moves of every task of the FP64
    build match the oracle; over a whole class (~1000 moves per task) the tasks diverge more
    often than at 40 nodes, through round-off sign changes of node balances that pro-rata
    compensation holds at zero, which add or drop a (spurious, linear) point; the moves tried
    and the guard events still agree."""
    m, st = make(N=128, L=192, T=24, R=8)
    o = Oracle(m, 8, seed=21)      # one oracle sweep first: node balances at round-off zero (nodes
    o.set_state(st)                # without units in the heuristic start) would flip pro-rata kinks
    o.sweeps(1, 100)
    s = o.get_state()
    for k in ("theta", "g", "e", "z", "reg", "k"):
        setattr(st, k, s[k])
    for limit, grid in ((20, None), (0, None), (20, (4, 0))):
        d = DeviceChain(m, 8, precision=64, seed=5)
        d.upload(st)
        if grid:  # four-warp blocks at their limit: the global scratch grows to the grid
            d.set_move_grid(*grid)
            assert d.move_grid()[0] == 4
        o = Oracle(m, 8, seed=5)
        o.set_state(st)
        sd = d.class_pass(3, 0, limit)
        so = o.class_pass(3, 0, limit)
        assert np.array_equal(sd[:-1:2], so[:-1:2])
        assert sd[-1] == so[-1] == 0                      # no guard events
        frac, worst = task_flips(d.download(), o.get_state(), m, 1e-9, 1e-9)
        print(f"128 nodes, FP64, first {limit or 'all'} moves: flipped tasks {frac:.4f}, worst other {worst:.2e}")
        if limit:
            assert frac <= 0.02
        d.close()


@pytest.mark.parametrize("prec", [64, 32])
def test_capacity_scores(base, prec):
    """The scores against the oracle's FP64 scores of the same state. FP64 build: every term in FP64,
    the sums in another order (1e-9 of the score scale). FP32 build: the terms in FP32 with
    compensated sums; every score and cost part lies within the bound the pass reports for it
    (esm_score_errors), the bounds are below 1e-3 of the score scale and the errors below 1e-5.
    Both builds sum in a fixed order: the same state gives the same scores bit for bit."""
    m, st = base
    d = DeviceChain(m, 32, precision=prec, seed=5)
    d.upload(st)
    d.sweeps(1, 0)
    o = Oracle(m, 32, seed=5)
    o.set_state(d.download())
    sk, fk, parts = d.scores()
    ek, ep = d.score_errors()
    sk0, fk0, parts0 = o.scores()
    scale = np.abs(sk0).max(axis=0) + 1e-3
    err = (np.abs(sk - sk0) / scale).max()
    bnd = (ek / scale).max()
    over = np.abs(sk - sk0) / np.maximum(ek, 1e-300)
    pover = np.abs(parts[:, :7] - parts0[:, :7]) / np.maximum(ep[:, :7], 1e-300)
    print(f"scores FP{prec} against the oracle: {err:.2e} of the score scale; bound {bnd:.2e}; "
          f"error / bound at most {over.max():.3f} (scores), {pover.max():.3f} (parts)")
    assert np.all(np.abs(sk - sk0) <= ek), over.max()
    assert np.all(np.abs(parts[:, :7] - parts0[:, :7]) <= ep[:, :7] + 1e-9), pover.max()
    if prec == 64:
        assert err < 1e-9
        np.testing.assert_allclose(parts[:, :7], parts0[:, :7], rtol=1e-9, atol=1e-6)
    else:
        # the bound is a worst case (every rounding at its extreme: about 1e-4 of the scale where the
        # shed and dump terms of a unit cancel); the error itself is of the order of the FP32 epsilon
        assert bnd < 1e-3 and err < 1e-5
        np.testing.assert_allclose(parts[:, :7], parts0[:, :7], rtol=1e-5, atol=1e-3)
    np.testing.assert_allclose(fk, fk0, rtol=1e-14)
    sk2, fk2, parts2 = d.scores()
    assert np.array_equal(sk, sk2) and np.array_equal(parts, parts2)


def test_langevin_step_fp64(base):
    m, st = base
    R = 32
    d = DeviceChain(m, R, precision=64, seed=5)
    d.upload(st)
    d.sweeps(1, 0)
    o = Oracle(m, R, seed=5)
    o.set_state(d.download())
    d.scores()
    o.scores()
    rng = np.random.Generator(np.random.PCG64(4))
    xi = rng.standard_normal(m.Kunits)
    w = np.full(R, 1.0 / R)
    ng = len(m.carriers)
    eta = np.full(ng, 5e-4)
    ks = np.array([500.0, 200.0, 1000.0, 300.0, 100.0, 100.0])
    kd, ncd = d.langevin_step(w, eta, ks, 1.0, 0.02, True, xi, 1)
    ko, nco = o.langevin_step(w, eta, ks, 1.0, 0.02, True, xi, 1)
    np.testing.assert_allclose(kd, ko, rtol=1e-12)
    assert ncd == nco
    a, b = d.download(), o.get_state()
    assert np.abs(a["g"] - b["g"]).max() < 1e-9
    r, _ = d.caches()
    o.rebuild()
    r0, _ = o.caches()
    assert np.abs(r - r0).max() < 1e-6


def test_langevin_stream_normals(base):
    """Without injected normals the device draws them from its Philox stream; the oracle replays it."""
    m, st = base
    R = 32
    d = DeviceChain(m, R, precision=64, seed=5)
    d.upload(st)
    o = Oracle(m, R, seed=5)
    o.set_state(st)
    d.scores()
    o.scores()
    w = np.full(R, 1.0 / R)
    eta = np.full(len(m.carriers), 5e-4)
    ks = np.full(len(m.carriers), 300.0)
    kd, _ = d.langevin_step(w, eta, ks, it=7)
    ko, _ = o.langevin_step(w, eta, ks, it=7)
    np.testing.assert_allclose(kd, ko, rtol=1e-12)


@pytest.mark.parametrize("prec", [64, 32])
def test_weather_step(base, prec):
    m, st = base
    R = 32
    d = DeviceChain(m, R, precision=prec, seed=5)
    d.upload(st)
    o = Oracle(m, R, seed=5)
    o.set_state(st)
    moved = (np.arange(R) % 3 != 0).astype(np.int32)
    theta = np.where(np.arange(R) % 2 == 0, 0.3, 0.1)
    window = np.where(np.arange(R) % 4 == 1, 12, 0)
    wstart = 1 + (np.arange(R) * 7) % m.T
    d.weather_step(moved, theta, window, wstart, it=4)
    o.weather_step(moved, theta, window, wstart, it=4)
    a, b = d.download(), o.get_state()
    assert np.array_equal(a["reg"], b["reg"])
    tz = 1e-9 if prec == 64 else 2e-5
    assert np.abs(a["z"] - b["z"]).max() < tz * (1 + np.abs(b["z"]).max())
    tg = 1e-8 if prec == 64 else 2e-3
    assert np.abs(a["g"] - b["g"]).max() < tg
