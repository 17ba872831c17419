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
    assert stats[:20:2].sum() > 0
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
