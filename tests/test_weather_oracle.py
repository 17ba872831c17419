"""The weather process of the oracle leaves the prior invariant (the reference's checks of
test/test_replicas.jl:101-160 restated on the synthetic prior): the pCN step keeps the stationary
law of the VAR, the regime window draws the exact conditional (against enumeration), and the step
reads neither the capacities nor the dispatch."""
import itertools
import math

import numpy as np
import pytest

from esmgb.model import initial_state, make_model
from oracle.oracle import Oracle


@pytest.fixture(scope="module")
def tiny():
    m = make_model(8, 10, 24, seed=4, n_off=2, countries=2)
    return m


def test_pcn_keeps_stationary_law(tiny):
    m = tiny
    R = 64
    st = initial_state(m, R, seed=2)
    o = Oracle(m, R, seed=3)
    o.set_state(st)
    moved = np.ones(R, np.int32)
    zs = []
    for it in range(30):
        o.weather_step(moved, np.full(R, 0.8), np.zeros(R), np.ones(R), it=it)
        zs.append(o.get_state()["z"][:, 5:, :].ravel())
    z = np.concatenate(zs)
    ref = initial_state(m, 256, seed=99).z[:, 5:, :].ravel()     # exact prior draws
    assert abs(z.std() / ref.std() - 1) < 0.05
    assert abs(z.mean() - ref.mean()) < 0.1


def test_weather_step_independent_of_dispatch(tiny):
    m = tiny
    R = 4
    st = initial_state(m, R, seed=2)
    args = (np.ones(R), np.full(R, 0.3), np.full(R, 5), np.array([3, 7, 11, 20]))
    o1 = Oracle(m, R, seed=3)
    o1.set_state(st)
    o1.weather_step(*args, it=5)
    st2 = initial_state(m, R, seed=2)
    st2.g = st2.g * 0.5
    st2.k = st2.k * 1.3
    o2 = Oracle(m, R, seed=3)
    o2.set_state(st2)
    o2.weather_step(*args, it=5)
    a, b = o1.get_state(), o2.get_state()
    assert np.array_equal(a["z"], b["z"]) and np.array_equal(a["reg"], b["reg"])


def test_regime_window_against_enumeration(tiny):
    m = tiny
    R = 256
    st = initial_state(m, R, seed=2)
    T = m.T
    reg = np.zeros((T, R), np.int32)
    reg[:, :] = 0
    reg[4, :] = 1                 # the regime after the window (1-based step 5)
    st.reg = reg
    a, B = 3, 2                   # window steps 3, 4 (1-based), regime 1 at step 2 before, 1 at step 5 after
    counts = {}
    for it in range(40):
        o = Oracle(m, R, seed=100 + it)
        o.set_state(st)
        o.weather_step(np.ones(R), np.zeros(R), np.full(R, B), np.full(R, a), it=it)
        rg = o.get_state()["reg"]
        for r in range(R):
            key = (int(rg[2, r]), int(rg[3, r]))
            counts[key] = counts.get(key, 0) + 1
    P = m.Ptr
    w = {}
    for path in itertools.product(range(2), repeat=2):
        w[path] = P[0, path[0]] * P[path[0], path[1]] * P[path[1], 1]
    tot = sum(w.values())
    n = sum(counts.values())
    for path, pw in w.items():
        p = pw / tot
        sd = math.sqrt(p * (1 - p) / n)
        assert abs(counts.get(path, 0) / n - p) < 5 * sd + 1e-3


def test_compensation_follows_headroom_and_output():
    """compensate_weather! (src/replicas.jl:207) in the oracle's weather step, on a model with two
    dispatchable units per node: at every node and step the residual change `need` of the weather
    move is taken up by the dispatchable units, an increase in proportion to their headroom (up to
    it), a decrease in proportion to their output; the rest stays on the residual."""
    import copy
    from esmgb.model import initial_state, make_model
    from oracle.oracle import Oracle
    m = make_model(12, 18, 40, seed=4, dispatch=("OCGT", "CCGT"))
    R = 3
    st = initial_state(m, R, seed=2)
    rng = np.random.Generator(np.random.PCG64(3))
    st.g = np.clip(st.g + 0.1 * rng.standard_normal(st.g.shape), 0.0, 1.0)
    o = Oracle(m, R, seed=5)
    o.set_state(st)
    o.rebuild()
    s0 = o.get_state()
    r0, _ = o.caches()
    o.weather_step(np.ones(R, np.int32), np.full(R, 0.6), np.zeros(R, np.int32), np.ones(R, np.int32), it=2)
    s1 = o.get_state()
    raw = Oracle(m, R, seed=5)
    raw.set_state(dict(s1, g=s0["g"]))
    raw.rebuild()
    need_all = raw.caches()[0] - r0
    k = s0["k"]
    kap = np.array([m.unit_avail[u] * np.clip(k[u], m.unit_lo[u], m.unit_hi[u]) for u in m.disp])
    bus = m.unit_bus[m.disp]
    worst, nchk = 0.0, 0
    for n in range(m.N):
        js = np.flatnonzero(bus == n)
        for t in range(m.T):
            for rep in range(R):
                need = need_all[n, t, rep]
                if abs(need) < 1e-6:
                    continue
                p = kap[js] * np.clip(s0["g"][js, t, rep], 0.0, 1.0)
                wq = np.maximum(kap[js] - p, 0.0) if need > 0 else p
                tot = wq.sum()
                dy = s1["g"][js, t, rep] - s0["g"][js, t, rep]
                if tot <= 1e-9:
                    assert np.abs(dy).max() == 0.0
                    continue
                a = min(need, tot) / tot if need > 0 else max(need, -tot) / tot
                want = a * wq / kap[js]
                worst = max(worst, np.abs(dy - want).max())
                nchk += 1
    print(f"compensation: {nchk} (node, step, replica) entries, worst {worst:.2e}")
    assert nchk > 100 and worst < 1e-12
