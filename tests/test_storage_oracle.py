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


def _blocks(m, rng, ntrial):
    """Storage block moves as the sweeps draw them: multiscale plateaus of one unit or of a cell-class
    aggregate over L in {1, 2, 8} inside the year, long-range plateaus of one long-duration unit that
    wrap the year end, and level moves (L = T)."""
    from esmgb.cabi import storage_groups
    sgp, sgu = storage_groups(m)
    longu = [j for j, u in enumerate(m.stor) if m.unit_hours[u] >= 24]
    for trial in range(ntrial):
        kind = trial % 4
        if kind == 0:
            us, L = [int(rng.integers(0, m.S))], int(rng.choice([1, 2, 8]))
            b0 = int(rng.integers(0, m.T - L))
        elif kind == 1:
            g = int(rng.integers(0, len(sgp) - 1))
            us, L = [int(x) for x in sgu[sgp[g]:sgp[g + 1]]], int(rng.choice([1, 2, 8]))
            b0 = int(rng.integers(0, m.T - L))
        elif kind == 2:
            us, L = [int(rng.choice(longu))], int(rng.integers(m.T // 2, m.T - 1))
            b0 = int(rng.integers(m.T // 2, m.T))
        else:
            us, L, b0 = [int(rng.choice(longu))], m.T, 0
        yield trial, kind, us, b0, L


def test_block_moves_exact_reversible_linear():
    """The reference's storage-move checks (test/test_local.jl:227-345, test/test_moves.jl §1-2) on
    the oracle's plateau, long-range and level moves: the cost change a move evaluates equals the
    global change after the commit; the move prepared again at the moved state and moved by -t
    returns to the start with the log-Jacobians cancelling (t on the scale of the first kink, or
    beyond it); the potential is linear between walk points (1e-6 nats)."""
    import copy
    m = make_model(12, 18, 40, seed=4, dispatch=("OCGT", "CCGT"))
    rng = np.random.Generator(np.random.PCG64(41))
    st = initial_state(m, 4, seed=2)
    st = copy.deepcopy(st)
    st.g = st.g + 0.05 * rng.standard_normal(st.g.shape)
    st.e = rng.uniform(0.05, 0.95, st.e.shape)
    o = Oracle(m, 4, seed=9)
    o.set_state(st)
    o.rebuild()
    beta = m.beta_v
    worst_c = worst_r = worst_j = worst_l = 0.0
    counts = [0, 0, 0, 0]
    ncross = 0
    for trial, kind, us, b0, L in _blocks(m, rng, 160):
        rep = int(rng.integers(0, 4))
        ok, _, (Q, g), _ = o.block_at(us, b0, L, rep, 0.0, commit=False)
        if not ok:
            continue
        counts[kind] += 1
        # walk linearity
        w = o.block_walk(us, b0, L, rep)
        if w is not None:
            pts, cs = w
            for j in range(len(pts) - 1):
                if pts[j + 1] > pts[j]:
                    for a in (0.25, 0.5, 0.75):
                        x = pts[j] + a * (pts[j + 1] - pts[j])
                        dc = o.block_at(us, b0, L, rep, x, commit=False)[3]
                        worst_l = max(worst_l, abs(beta * dc - ((1 - a) * cs[j] + a * cs[j + 1])))
        # exactness and reversibility
        if g != 0.0 and abs(Q / g) < 1e5:
            t = 0.3 * rng.standard_normal() * abs(Q / g) if trial % 8 < 4 else -2.0 * Q / g
            ncross += abs(t) > abs(Q / g)
        else:
            t = 0.02 * rng.standard_normal()
        s0 = o.get_state()
        c0 = o.scores()[2][rep, 1]
        _, lj, _, dc = o.block_at(us, b0, L, rep, t)
        c1 = o.scores()[2][rep, 1]
        worst_c = max(worst_c, abs((c1 - c0) - dc) / (1e-12 * abs(c0) + 1e-9 * (1 + abs(dc))))
        _, lj2, _, _ = o.block_at(us, b0, L, rep, -t)
        s1 = o.get_state()
        worst_r = max(worst_r, max(np.abs(s1[k] - s0[k]).max() / (1 + np.abs(s0[k]).max()) for k in ("g", "e")))
        worst_j = max(worst_j, abs(lj + lj2))
    print(f"block moves {counts} (plateau, aggregate, long, level), {ncross} across a kink: cost {worst_c:.2e} "
          f"(of the bound), return {worst_r:.2e}, log-Jacobian sum {worst_j:.2e}, linearity {worst_l:.2e} nats")
    assert min(counts) > 10 and ncross > 5
    assert worst_c <= 1.0
    assert worst_r < 1e-9 and worst_j < 1e-8
    assert worst_l < 1e-6
