"""Synthetic model tables and the oracle's own consistency (the reference's model-dependent checks
restated on the synthetic model: caches after a sweep equal a rebuild, src/local.jl:2054; the score
against finite differences of the cost, test/test_replicas.jl "score against finite differences")."""
import numpy as np
import pytest

from esmgb.model import make_model, initial_state, haar_basis
from oracle.oracle import Oracle


@pytest.fixture(scope="module")
def small():
    m = make_model(40, 60, 40, seed=11)
    st = initial_state(m, 4, seed=3)
    return m, st


def test_haar_atoms_orthonormal(small):
    # test/runtests.jl:83-100: graph Haar bases are orthonormal
    m, _ = small
    for a in m.atoms:
        n = len(a.ptr) - 1
        size = m.N if a.role == 1 else (m.D if a.role == 3 else m.S)
        U = np.zeros((size, n))
        for j in range(n):
            U[a.idx[a.ptr[j]:a.ptr[j + 1]], j] = a.val[a.ptr[j]:a.ptr[j + 1]]
        used = np.flatnonzero(np.abs(U).sum(1) > 0)
        G = U[used].T @ U[used]
        np.testing.assert_allclose(G, np.eye(n), atol=1e-12)
    # theta atoms are orthogonal to the component constants (gauge removed)
    th = m.atoms[0]
    for j in range(len(th.ptr) - 1):
        assert abs(th.val[th.ptr[j]:th.ptr[j + 1]].sum()) < 1e-12


def _dense(cols, n):
    U = np.zeros((n, len(cols)))
    for j, (rows, vals) in enumerate(cols):
        U[rows, j] = vals
    return U


def test_haar_bases_reference_properties():
    """test/test_local.jl:8-41 ("sparse graph Haar field bases") restated: a 30-node path graph
    with three levels (one cell, countries, nodes). The basis is orthonormal with one column per
    level cell beyond its parent; on a 17-node support it stays orthonormal and sparse (at most
    |support| (ceil(log2 |support|) + 3) nonzeros); its first columns up to a level span the fields
    constant on that level's cells; the angle basis without its top level has N - 2 columns, none
    with a component constant."""
    rng = np.random.Generator(np.random.PCG64(11))
    N = 30
    country = rng.integers(1, 6, N)
    parts = [np.ones(N, int), country, np.arange(N)]
    edges = [(i, i + 1, 1.0) for i in range(N - 1)]
    cols, gcounts, _ = haar_basis(parts, np.arange(N), edges=edges)
    U = _dense(cols, N)
    np.testing.assert_allclose(U.T @ U, np.eye(U.shape[1]), atol=1e-12)
    assert gcounts == [1, len(np.unique(country)), N]
    sup = np.sort(rng.permutation(N)[:17])
    bcols, bcounts, _ = haar_basis(parts, sup, edges=edges)
    B = _dense(bcols, len(sup))
    np.testing.assert_allclose(B.T @ B, np.eye(B.shape[1]), atol=1e-12)
    assert B.shape[1] == len(sup)
    assert sum(len(r) for r, _ in bcols) <= len(sup) * (int(np.ceil(np.log2(len(sup)))) + 3)
    for Mq in (1, gcounts[1], N):
        q = max(i for i, g in enumerate(gcounts) if g <= Mq)   # the level of Mq modes
        m = bcounts[q]
        Um = B[:, :m]
        keys = [tuple(int(p[n]) for p in parts[:q + 1]) for n in sup]
        for c in set(keys):
            v = np.array([k == c for k in keys], float)
            np.testing.assert_allclose(Um @ (Um.T @ v), v, atol=1e-12)
    comp = np.array([1 if i < 20 else 2 for i in range(N)])
    tcols, _, _ = haar_basis([comp, country, np.arange(N)], np.arange(N), edges=edges, drop_top=True)
    T = _dense(tcols, N)
    assert T.shape[1] == N - 2
    np.testing.assert_allclose(T.T @ T, np.eye(N - 2), atol=1e-12)
    assert np.linalg.norm(T.T @ (comp == 1)) < 1e-10 and np.linalg.norm(T.T @ (comp == 2)) < 1e-10


def test_move_tables(small):
    m, _ = small
    assert m.units_ptr[-1] == m.D and m.stor_ptr[-1] == m.S
    assert np.isclose(m.qcum[-1], 1.0)
    # xloc templates route a unit dipole: injection +1 at n, -1 at m inside the ball (src/local.jl:122)
    for n in range(m.N):
        for p in range(m.xpart_ptr[n], m.xpart_ptr[n + 1]):
            mm = m.xpart[p]
            th = np.zeros(m.N)
            th[m.xnod[m.xnod_ptr[p]:m.xnod_ptr[p + 1]]] = m.xval[m.xnod_ptr[p]:m.xnod_ptr[p + 1]]
            inj = np.zeros(m.N)
            for e in range(m.L):
                f = m.line_b[e] * (th[m.bus0[e]] - th[m.bus1[e]])
                inj[m.bus0[e]] += f
                inj[m.bus1[e]] -= f
            assert abs(inj[n] - 1) < 1e-12 and abs(inj[mm] + 1) < 1e-12


def test_sweep_caches_equal_rebuild_and_determinism(small):
    m, st = small
    o = Oracle(m, 4, seed=5)
    o.set_state(st)
    stats = o.sweeps(2, 0)
    assert stats[-1] == 0                       # no guard events
    assert stats[:-1:2].sum() > 0
    r1, F1 = o.caches()
    o.rebuild()
    r2, F2 = o.caches()
    assert np.abs(r1 - r2).max() < 1e-8 * (1 + np.abs(r2).max())
    assert np.abs(F1 - F2).max() < 1e-8 * (1 + np.abs(F2).max())
    s1 = o.get_state()
    o2 = Oracle(m, 4, seed=5)
    o2.set_state(st)
    o2.sweeps(2, 0)
    s2 = o2.get_state()
    for k in ("theta", "g", "e"):
        assert np.array_equal(s1[k], s2[k])


def test_score_against_finite_differences(small):
    m, st = small
    # a state whose residuals are away from the balance kink (r = 0), so that a finite difference
    # of the piecewise-linear cost does not cross kinks
    o = Oracle(m, 4, seed=5)
    rng = np.random.Generator(np.random.PCG64(2))
    pert = _with_k({k: getattr(st, k) for k in ("theta", "g", "e", "z", "reg", "k")}, st.k)
    pert.g = st.g + 0.05 * rng.standard_normal(st.g.shape)
    pert.e = np.clip(st.e + 0.2 * rng.standard_normal(st.e.shape), 0.01, 0.99)
    o.set_state(pert)
    sk, fk, parts = o.scores()
    base = {k: getattr(pert, k) for k in ("theta", "g", "e", "z", "reg", "k")}
    h = 0.05
    for u in (0, 45, 100, 130, 170, 200):        # renewables, OCGT, storage units
        vals = []
        for s in (+1, -1):
            k = base["k"].copy()
            k[u] += s * h
            o.set_state(_with_k(base, k))
            _, _, p = o.scores()
            lj = m.T * np.log(k[u] + m.kappa0) if m.unit_kind[u] != 0 else 0.0
            vals.append(-m.beta_v * p[:, 1] + lj)
        fd = (vals[0] - vals[1]) / (2 * h)
        np.testing.assert_allclose(sk[:, u], fd, rtol=1e-5, atol=1e-7)


class _S:
    pass


def _with_k(base, k):
    s = _S()
    for key, v in base.items():
        setattr(s, key, v)
    s.k = k
    return s


def _rates(**on):
    from esmgb.model import FAMILIES
    return tuple(float(on.get(f, 0.0)) for f in FAMILIES)


def _deficit_state(st):
    """Low renewables (weather anomaly -3) and every dispatchable unit at half output: the nodes'
    requirement is positive and the dispatch can follow it inside the box."""
    import copy
    s = copy.deepcopy(st)
    s.z[:] = -3.0
    s.g[:] = 0.5
    return s


def _first_move_of(o, fam, cls=0):
    """A sweep whose class-`cls` move list starts with a draw of family `fam`."""
    for sw in range(400):
        k, _, _ = o.move_list(sw, cls, 0)
        if k[0] == fam:
            return sw
    raise AssertionError("no such sweep")


@pytest.mark.parametrize("fam", ["tpot", "tsoc"])
def test_transport_families_caches_and_counts(small, fam):
    """Sweeps of the compensated transport families only (with the atoms): moves are tried and
    taken (the Jacobian test, with its small log-Jacobians, rejects few) and the caches still equal
    a rebuild."""
    from esmgb.model import FAMILIES
    m, st = small
    o = Oracle(m, 4, seed=5, rates=_rates(**{fam: 1.0}))
    o.set_state(st)
    stats = o.sweeps(2, 0)
    f = FAMILIES.index(fam)
    assert stats[2 * f] > 0 and stats[2 * f + 1] > 0
    assert stats[:2 * f:2].sum() == 0           # no other family was drawn
    assert stats[-1] == 0
    r1, F1 = o.caches()
    o.rebuild()
    r2, F2 = o.caches()
    assert np.abs(r1 - r2).max() < 1e-8 * (1 + np.abs(r2).max())
    assert np.abs(F1 - F2).max() < 1e-8 * (1 + np.abs(F2).max())


def test_tpot_compensation_keeps_the_residuals(small):
    """prep_tpot! (src/local.jl:1741): the angle of node n rises by t, the flows of its lines change
    by b (+-t) and the dispatch at every end node follows the requirement change g t pro rata, so a
    node's residual changes by at most |g t| (a unit or the node leaving the box) and by nothing
    where the compensation stays inside; with the opposite sign it would change by 2 g t."""
    from esmgb.model import FAMILIES
    m, st = small
    o = Oracle(m, 4, seed=5, rates=_rates(tpot=1.0))
    sw = _first_move_of(o, FAMILIES.index("tpot"))
    o.set_state(_deficit_state(st))
    o.rebuild()
    r0, _ = o.caches()
    s0 = o.get_state()
    o.class_pass(sw, 0, limit=1)
    r1, _ = o.caches()
    dth = o.get_state()["theta"] - s0["theta"]
    nodes = np.unique(np.nonzero(dth)[0])
    assert len(nodes) == 1                      # one node for every task of the class
    n = int(nodes[0])
    g = np.zeros(m.N)
    for e in range(m.L):
        a, b = int(m.bus0[e]), int(m.bus1[e])
        if n in (a, b):
            df = m.line_b[e] * ((a == n) - (b == n))
            g[a] += df
            g[b] -= df
    ends = np.flatnonzero(g != 0)
    moved = np.argwhere(dth[n] != 0)            # (step, replica) of the moved tasks
    assert len(moved) > 0
    exact = 0
    for tau, rep in moved:
        t = dth[n, tau, rep]
        dr = r1[:, tau, rep] - r0[:, tau, rep]
        scale = np.abs(g * t).max()
        assert (np.abs(dr[ends]) <= np.abs(g[ends] * t) * (1 + 1e-9) + 1e-9 * scale).all()
        others = np.setdiff1d(np.arange(m.N), ends)
        assert np.abs(dr[others]).max(initial=0) <= 1e-9 * scale
        exact += np.abs(dr).max() <= 1e-9 * scale
    print(f"tpot node {n}: {len(moved)} moved tasks, residuals unchanged in {exact}")
    assert exact >= 0.2 * len(moved)            # measured 27 of 80


def test_tsoc_compensation_direction(small):
    """prep_tsoc! (src/local.jl:1849): the state of charge of one unit at tau rises by t; the
    dispatch at its node follows +kappa_s t at tau - 1 and -kappa_s t at tau (with soc_qadj), so
    the node's residuals change only by the efficiency bend of the storage power (a fraction
    |1/eta_in - 1| or |eta_out - 1| of kappa_s t), not by the whole kappa_s t (or twice it with the
    opposite sign)."""
    from esmgb.model import FAMILIES
    m, st = small
    o = Oracle(m, 4, seed=5, rates=_rates(tsoc=1.0))
    sw = _first_move_of(o, FAMILIES.index("tsoc"))
    o.set_state(_deficit_state(st))
    o.rebuild()
    r0, _ = o.caches()
    s0 = o.get_state()
    o.class_pass(sw, 0, limit=1)
    r1, _ = o.caches()
    de = o.get_state()["e"] - s0["e"]
    units = np.unique(np.nonzero(de)[0])
    assert len(units) == 1
    sj = int(units[0])
    u = int(m.stor[sj])
    n = int(m.unit_bus[u])
    kc = np.clip(s0["k"][u], m.unit_lo[u], m.unit_hi[u])
    ks = kc * m.unit_hours[u] / m.dt
    moved = np.argwhere(de[sj] != 0)
    assert len(moved) > 0
    ratios = []
    for tau, rep in moved:
        t = de[sj, tau, rep]
        taum = (tau - 1) % m.T
        ratios.append(max(abs(r1[n, tau, rep] - r0[n, tau, rep]), abs(r1[n, taum, rep] - r0[n, taum, rep])) /
                      (ks * abs(t)))
    print(f"tsoc unit {sj} at node {n}: {len(moved)} moved tasks, median residual ratio {np.median(ratios):.3f}")
    assert np.median(ratios) < 0.6


@pytest.fixture(scope="module")
def two_dispatch():
    """Two dispatchable units at every node (OCGT and CCGT): the pair and cell-pair selections and
    the Jacobian terms (|S| - 1 = 1) of the compensated moves come into play."""
    m = make_model(12, 18, 40, seed=4, dispatch=("OCGT", "CCGT"))
    return m, initial_state(m, 4, seed=2)


def test_two_dispatch_model_sweeps(two_dispatch):
    """Sweeps with every family (the plain rates and tpot, tsoc at 0.1) on the two-unit model: every
    family is tried and moves, the Jacobian test rejects some compensated moves, and the caches
    equal a rebuild."""
    from esmgb.model import FAMILIES, FAMILY_RATES
    m, st = two_dispatch
    o = Oracle(m, 4, seed=5, rates=tuple(FAMILY_RATES[:9]) + (0.1, 0.1))
    o.set_state(st)
    stats = o.sweeps(2, 0)
    tried, moved = stats[0:2 * len(FAMILIES):2], stats[1:2 * len(FAMILIES):2]
    assert (tried > 0).all() and (moved > 0).all(), dict(zip(FAMILIES, tried))
    comp = [FAMILIES.index(f) for f in ("xlocc", "tpot", "tsoc")]
    assert (tried[comp] - moved[comp]).sum() > 0           # Jacobian rejections
    assert stats[-1] == 0
    r1, F1 = o.caches()
    o.rebuild()
    r2, F2 = o.caches()
    assert np.abs(r1 - r2).max() < 1e-8 * (1 + np.abs(r2).max())
    assert np.abs(F1 - F2).max() < 1e-8 * (1 + np.abs(F2).max())


@pytest.mark.parametrize("model", ["one", "two"])
@pytest.mark.parametrize("state", ["perturbed", "deficit"])
def test_compensated_moves_are_reversible(small, two_dispatch, model, state):
    """test/test_local.jl:285-345 and test/test_moves.jl (2, reversibility) restated for every
    family, the compensated ones (xlocc, tpot, tsoc) with their kinks: a move by t, then the same
    move prepared at the new state and moved by -t, returns to the start (the shares and the
    excess are coordinates of the curve; soc_qadj makes the requirement of tsoc's compensation
    follow the nominal storage injection), and the two log-Jacobians cancel. t is drawn as there:
    on the scale of the first kink, or twice its distance (beyond it); for the families without
    kinks (or with a kink beyond 1e5) over five decades. The line density of the move prepared at
    the moved state is the forward one shifted by t (bound 1e-6 as there)."""
    from esmgb.model import FAMILIES
    import copy
    m, st = small if model == "one" else two_dispatch
    rng = np.random.Generator(np.random.PCG64(17))
    if state == "deficit":
        st = _deficit_state(st)
    else:
        # the start state's dispatch covers the residual exactly (r = 0, so the excess e = 0 and a
        # move that empties the unit leaves P = 0, where prorata! makes no kink on the way back):
        # perturbed dispatch gives generic residuals, as the reference's test states
        st = copy.deepcopy(st)
        st.g = st.g + 0.05 * rng.standard_normal(st.g.shape)
    o = Oracle(m, 4, seed=5)
    o.set_state(st)
    o.rebuild()
    comp = [FAMILIES.index(f) for f in ("xlocc", "tpot", "tsoc")]
    worst = worstj = ljmax = worstd = 0.0
    ncross = nmoves = nplain = 0
    for trial in range(360):
        fam = trial % len(FAMILIES)
        tau, rep = int(rng.integers(0, m.T)), int(rng.integers(0, 4))
        ok, _, (Q, g) = o.move_at(fam, tau, rep, 1, trial, 0.0, commit=False)
        if not ok:
            continue
        s0 = o.get_state()
        if fam in comp and g != 0.0 and abs(Q / g) < 1e5:   # (a leak of round-off size puts the kink far away)
            t = 0.3 * rng.standard_normal() * abs(Q / g) if (trial // len(FAMILIES)) % 2 else -2.0 * Q / g
        else:
            t = float(rng.choice([-1.0, 1.0]) * 10.0 ** rng.uniform(-3.0, 2.5))
            g, Q = 0.0, 0.0
            nplain += 1
        def dens(x):  # the line log-density (up to its constant) of the move prepared now, at x
            _, ljx, _, dcx = o.move_at(fam, tau, rep, 1, trial, x, commit=False, with_cost=True)
            return -m.beta_v * dcx + ljx, abs(m.beta_v * dcx)
        us = (-t, -0.37 * t, 0.61 * t, 1.5 * t)
        f0, m0 = dens(t)
        fwd = [dens(t + u) for u in us]
        _, lj, _ = o.move_at(fam, tau, rep, 1, trial, t)
        fr0 = dens(0.0)[0]
        for u, (fu, mu) in zip(us, fwd):   # the reverse density is the forward one shifted
            wdens = abs((dens(u)[0] - fr0) - (fu - f0)) / (1 + 1e-9 * (mu + m0))
            worstd = max(worstd, wdens)
        _, lj2, _ = o.move_at(fam, tau, rep, 1, trial, -t)
        s1 = o.get_state()
        for k in ("theta", "g", "e"):
            worst = max(worst, np.abs(s1[k] - s0[k]).max() / (1 + np.abs(s0[k]).max()))
        worstj = max(worstj, abs(lj + lj2))
        ljmax = max(ljmax, abs(lj))
        if g != 0.0:
            ncross += abs(t) > abs(Q / g)
            nmoves += 1
    print(f"{model} {state}: {nmoves} compensated moves, {ncross} across the kink, {nplain} others, worst "
          f"{worst:.2e}, largest |log-Jacobian| {ljmax:.2e}, worst sum {worstj:.2e}, reverse density {worstd:.2e}")
    assert worstd < 1e-6
    assert nmoves > 60 and ncross > 10 and nplain > 150
    assert (ljmax > 1e-3) == (model == "two")      # the Jacobian terms vanish with one unit per node
    assert worst < 1e-9
    assert worstj < 1e-8


@pytest.mark.parametrize("model", ["one", "two"])
def test_every_family_cost_change_is_exact(small, two_dispatch, model):
    """test/test_moves.jl (draw consistency): the cost change a move evaluates for its t equals
    the change of the global operational cost (energy_cost, src/energy.jl:551) after the commit,
    for every family, at sites of random step, replica and selection, with t over five decades."""
    import copy
    from esmgb.model import FAMILIES
    m, st = small if model == "one" else two_dispatch
    rng = np.random.Generator(np.random.PCG64(23))
    st = copy.deepcopy(st)
    st.g = st.g + 0.05 * rng.standard_normal(st.g.shape)
    o = Oracle(m, 4, seed=5)
    o.set_state(st)
    o.rebuild()
    made = {f: 0 for f in FAMILIES}
    worst = 0.0
    for trial in range(330):
        fam = trial % len(FAMILIES)
        tau, rep = int(rng.integers(0, m.T)), int(rng.integers(0, 4))
        t = float(rng.choice([-1.0, 1.0]) * 10.0 ** rng.uniform(-3.0, 2.5))
        c0 = o.scores()[2][rep, 1]
        ok, _, _, dc = o.move_at(fam, tau, rep, 2, trial, t, with_cost=True)
        if not ok:
            continue
        c1 = o.scores()[2][rep, 1]
        err = abs((c1 - c0) - dc)
        assert err <= 1e-11 * abs(c0) + 1e-9 * abs(dc), (FAMILIES[fam], t, c1 - c0, dc)
        worst = max(worst, err / (abs(c0) + abs(dc)))
        made[FAMILIES[fam]] += 1
    print(model, made, f"worst {worst:.1e}")
    blocked = {"pair", "cellpair"} if model == "one" else set()
    assert all(v > 0 for f, v in made.items() if f not in blocked)
    r1, F1 = o.caches()
    o.rebuild()
    r2, _ = o.caches()
    assert np.abs(r1 - r2).max() < 1e-8 * (1 + np.abs(r2).max())


@pytest.mark.parametrize("model", ["one", "two"])
def test_every_family_potential_is_linear_between_walk_points(small, two_dispatch, model):
    """test/test_moves.jl 1a: between consecutive points of a move's walk the potential beta
    DeltaC(t) is linear (checked at 1/4, 1/2, 3/4 of every segment, bound 1e-6 nats as there), so
    the walk misses no kink or root of the line's piecewise-linear cost."""
    import copy
    from esmgb.model import FAMILIES
    m, st = small if model == "one" else two_dispatch
    rng = np.random.Generator(np.random.PCG64(29))
    st = copy.deepcopy(st)
    st.g = st.g + 0.05 * rng.standard_normal(st.g.shape)
    o = Oracle(m, 4, seed=5)
    o.set_state(st)
    o.rebuild()
    beta = m.beta_v
    worst, nseg = 0.0, {f: 0 for f in FAMILIES}
    for trial in range(110):
        fam = trial % len(FAMILIES)
        tau, rep = int(rng.integers(0, m.T)), int(rng.integers(0, 4))
        w = o.move_walk(fam, tau, rep, 3, trial)
        if w is None:
            continue
        pts, cs = w
        for j in range(len(pts) - 1):
            if not pts[j + 1] > pts[j]:
                continue
            nseg[FAMILIES[fam]] += 1
            for a in (0.25, 0.5, 0.75):
                t = pts[j] + a * (pts[j + 1] - pts[j])
                _, _, _, dc = o.move_at(fam, tau, rep, 3, trial, t, commit=False, with_cost=True)
                worst = max(worst, abs(beta * dc - ((1 - a) * cs[j] + a * cs[j + 1])))
    print(model, nseg, f"worst {worst:.2e} nats")
    blocked = {"pair", "cellpair"} if model == "one" else set()
    assert all(v > 0 for f, v in nseg.items() if f not in blocked)
    assert worst < 1e-6


def _prorata_coords(m, st, r, kmin=1.0):
    """Shares sigma [D, T, R] and excess e [N, T, R] of the dispatchable units at every node and
    step (prorata_coords of test/test_kop.jl); NaN where a node has no unit or |P| < 1e-6."""
    k = st["k"]
    g = st["g"]
    kap = np.array([m.unit_avail[u] * np.clip(k[u], m.unit_lo[u], m.unit_hi[u]) for u in m.disp])
    use = np.abs(kap) >= kmin
    bus = m.unit_bus[m.disp]
    sig = np.full(g.shape, np.nan)
    e = np.full(r.shape, np.nan)
    for n in range(m.N):
        js = np.flatnonzero((bus == n) & use)
        if len(js) == 0:
            continue
        p = kap[js, None, None] * g[js]
        P = p.sum(0)
        Q = r[n] + (kap[js, None, None] * np.clip(g[js], 0.0, 1.0)).sum(0)
        ok = np.abs(P) >= 1e-6
        e[n] = np.where(ok, P - np.maximum(Q, 0.0), np.nan)
        sig[js] = np.where(ok, p / np.where(ok, P, 1.0), np.nan)
    return sig, e


def test_following_keeps_prorata_coordinates(two_dispatch):
    """follow_capacities! (src/replicas.jl:448) in the oracle's Langevin step, as test/test_kop.jl
    checks it: the dispatchable units keep their output (utilisation scaled by c(k0)/c(k1)), the
    renewable and storage units move along their kop curves at fixed utilisation with the node's
    dispatch following share-preservingly, so the shares and the excess of every node's
    dispatchable units are unchanged (bounds 1e-9 and 1e-6 as there), the storage states and the
    weather are untouched, and the capacities become the Langevin step's."""
    import copy
    m, st = two_dispatch
    rng = np.random.Generator(np.random.PCG64(43))
    st = copy.deepcopy(st)
    st.g = st.g + 0.05 * rng.standard_normal(st.g.shape)
    o = Oracle(m, 4, seed=5)
    o.set_state(st)
    o.rebuild()
    s0 = o.get_state()
    r0, _ = o.caches()
    sig0, e0 = _prorata_coords(m, s0, r0)
    o.scores()
    G = len(m.carriers)
    knew, _ = o.langevin_step(np.full(4, 0.25), np.full(G, 2e-3), np.full(G, 300.0), 1.0, 10.0, True,
                              rng.standard_normal(m.Kunits), 7)
    s1 = o.get_state()
    r1, _ = o.caches()
    np.testing.assert_array_equal(s1["k"], knew)
    assert np.abs(knew - s0["k"]).max() > 1.0                  # the capacities moved
    sig1, e1 = _prorata_coords(m, s1, r1)
    both = ~np.isnan(sig0) & ~np.isnan(sig1)
    esig = np.abs(sig1 - sig0)[both].max()
    bothe = ~np.isnan(e0) & ~np.isnan(e1)
    ee = (np.abs(e1 - e0) / (1 + np.abs(e0)))[bothe].max()
    print(f"following: shares {esig:.2e} over {both.sum()}, excess {ee:.2e} over {bothe.sum()}")
    assert both.mean() > 0.9 and esig < 1e-9 and ee < 1e-6
    # the storage states and the renewable utilisations (weather) are unchanged: fixed utilisations
    np.testing.assert_array_equal(s1["e"], s0["e"])
    np.testing.assert_array_equal(s1["z"], s0["z"])


def test_following_of_dispatchable_capacities_keeps_output(two_dispatch):
    """test/test_replicas.jl "dispatch-following maps": when only the dispatchable capacities move
    (the Langevin step with zero step for every other field), their output c(k) omega is kept at
    every step (rtol 1e-9, atol 1e-6) and the residual with it (1e-6); the other capacities and the
    storage states are untouched."""
    import copy
    m, st = two_dispatch
    rng = np.random.Generator(np.random.PCG64(47))
    st = copy.deepcopy(st)
    st.g = st.g + 0.05 * rng.standard_normal(st.g.shape)
    o = Oracle(m, 4, seed=5)
    o.set_state(st)
    o.rebuild()
    s0 = o.get_state()
    r0, _ = o.caches()
    o.scores()
    G = len(m.carriers)
    dispg = sorted({int(m.unit_group[u]) for u in m.disp})
    eta = np.array([2e-3 if gi in dispg else 0.0 for gi in range(G)])
    knew, _ = o.langevin_step(np.full(4, 0.25), eta, np.full(G, 300.0), 1.0, 10.0, True, rng.standard_normal(m.Kunits), 3)
    s1 = o.get_state()
    r1, _ = o.caches()
    moved = np.abs(knew - s0["k"]) > 0
    assert moved[m.disp].any() and not moved[np.setdiff1d(np.arange(m.Kunits), m.disp)].any()
    for j, u in enumerate(m.disp):
        kc0 = np.clip(s0["k"][u], m.unit_lo[u], m.unit_hi[u])
        kc1 = np.clip(s1["k"][u], m.unit_lo[u], m.unit_hi[u])
        np.testing.assert_allclose(kc1 * s1["g"][j], kc0 * s0["g"][j], rtol=1e-9, atol=1e-6)
    assert np.abs(r1 - r0).max() < 1e-6
    np.testing.assert_array_equal(s1["e"], s0["e"])
