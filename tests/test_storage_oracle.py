"""The oracle's storage multiscale sweep (storage_ms_sweep!, src/flowmoves.jl:255, plateau moves):
its plan of class passes, and the consistency of its moves with the model (the residual cache kept by
the moves equals a rebuild, as the reference's caches after a sweep, src/local.jl:2054)."""
import numpy as np

from esmgb.model import initial_state, make_model
from oracle.oracle import Oracle


def _oracle(T=120, R=4, seed=3):
    m = make_model(12, 18, T, seed=seed)
    o = Oracle(m, R, seed=9, threads=4)
    o.set_state(initial_state(m, R, seed=2))
    return m, o


def test_plan_structure():
    m, o = _oracle()
    plan = o.storage_ms_plan(5)
    lengths = [p[0] for p in plan]
    assert set(lengths) <= {2, 4, 8, 16, 32} and all(L < m.T // 2 for L in lengths)
    for L in set(lengths):  # both block parities of every length, one offset below L
        ps = [p for p in plan if p[0] == L]
        assert sorted(p[2] for p in ps) == [0, 1] and len({p[1] for p in ps}) == 1 and ps[0][1] < L
    # the sweep's coin: the sweep runs with probability 1/2
    ran = sum(1 for s in range(200) if o.storage_ms_plan(s, force=False))
    assert 70 <= ran <= 130


def test_moves_keep_the_caches():
    m, o = _oracle()
    o.sweeps(2, 0)
    s0 = o.get_state()
    st = o.storage_ms(5)
    assert st[0] > 0 and st[1] > 0.5 * st[0] and st[2] == 0
    r1, F1 = o.caches()
    o.rebuild()
    r2, F2 = o.caches()
    assert np.abs(r1 - r2).max() <= 1e-9 * (1 + np.abs(r2).max())
    assert np.array_equal(F1, F2)  # no line is touched
    s1 = o.get_state()
    assert np.array_equal(s0["theta"], s1["theta"])
    assert (s1["e"] != s0["e"]).mean() > 0.5  # most states of charge moved


def test_long_range_plan_and_caches():
    """storage_long_sweep! (src/storage_long.jl:245): the units with at least 24 h of storage, each
    with the level move and 4 cyclic plateaus of length 1 .. T-1; the caches stay consistent."""
    m, o = _oracle()
    o.sweeps(1, 0)
    plan = o.storage_long_plan(3)
    hours = m.unit_hours[m.stor]
    units = sorted({p[0] for p in plan})
    assert units == [j for j in range(m.S) if hours[j] >= 24.0]
    for j in units:
        mv = [p for p in plan if p[0] == j]
        assert len(mv) == 5 and sum(p[1] == m.T for p in mv) == 1
        assert all(1 <= p[1] <= m.T and 0 <= p[2] < m.T for p in mv)
    s0 = o.get_state()
    st = o.storage_long(3)
    assert st[0] == len(plan) * o.R and st[2] == 0
    r1, _ = o.caches()
    o.rebuild()
    r2, _ = o.caches()
    assert np.abs(r1 - r2).max() <= 1e-9 * (1 + np.abs(r2).max())
    s1 = o.get_state()
    moved = np.abs(s1["e"] - s0["e"]).max(axis=(1, 2)) > 0
    assert set(np.flatnonzero(moved)) <= set(units)  # only the long-duration units move
