"""Parity at the benchmarked configuration: the synthetic 40-node, 60-line model at hourly T = 8760
with 64 replicas, the bench's model seed (1234), start state (seed 7) and Philox seed (1234), worn by
one operation sweep of the device chain. The oracle replays replicas 0 and 1: the lane streams are
keyed by the replica index and the move list is shared by the class, so an oracle of two replicas
draws exactly what the device draws for its first two.

Every task whose draws differ is explained (tests/flipdiag.py) at its first differing draw: the
discrete choice there and the margin by which the oracle's own draw cleared that choice's boundary.
A later draw of a task can differ widely once an earlier one moved its state (a theta move on a flat
potential amplifies a 1e-4 change of a state of charge), so the first draw is the one examined, at
a tight tolerance.
Tolerances: FP64 elements 1e-9, at most 2 % of the tasks flipped, first differing draws (beyond
1e-9 |t| + 1e-12) within 1e-8 of their boundary (relative to the total mass, to maxnats for a stop;
same-segment offsets within 1e-6 of the segment's length); FP32 elements 2e-3 (4e-3 absolute on
utilisations and states of charge), first differing draws (beyond 1e-4 |t| + 1e-6) within 5e-3 of
their boundary -- the FP32 potentials carry round-off up to about 1e-3 nats (4.8e-7 times the summed
magnitudes of a move's terms), so segment masses and end points are known to about that relative
accuracy -- (same-segment offsets: within 2e-2 of the length, or the segment flat to 1e-2 nats:
the FP32 flat-segment threshold is the round-off scale of the segment's end points, about 1e-3 nats
on storage moves; the FP32 build divides with the approximate single-precision division, 2 ulp,
so a breakpoint at t carries about 2.4e-7 |t| of placement error, which within a short segment near
a clamp moves the offset by up to about 1e-2 of the segment's length). The absolute floor of 1e-6 is the FP32 resolution of the state: a state of charge
near 1 has an ulp of 6e-8, so where it sits within 1e-5 of a clamp the clamp's breakpoint is placed
only to about 1e-2 of its distance, and draws below 1e-6 (about 16 ulps of the state through the
atoms' coefficients) differ by that placement, not by a discrete choice."""
import numpy as np
import pytest

from esmgb.device import DeviceChain
from esmgb.model import initial_state, make_model
from oracle.oracle import Oracle

from flipdiag import explain_flips, first_diffs, summary
from test_gpu_parity import task_flips

pytestmark = pytest.mark.gpu

N, L, T, R, SEED = 40, 60, 8760, 64, 1234
NREP = 2          # replicas the oracle replays
SWEEP, CLS = 1, 0
MAXNATS = 40.0


@pytest.fixture(scope="module")
def model():
    return make_model(N, L, T, seed=SEED)


def nmoves(m):
    return sum(len(a.ptr) - 1 for a in m.atoms) + int(round(4.0 * m.N))


def worn(m, prec):
    """The device chain after one operation sweep (sweep 0) from the bench's start state."""
    d = DeviceChain(m, R, precision=prec, seed=SEED)
    d.upload(initial_state(m, R, seed=7))
    st = d.sweeps(1, 0)
    return d, st


def sub(st, n=NREP):
    """Replicas 0 .. n-1 of a downloaded state."""
    out = {}
    for k, v in st.items():
        out[k] = v if k == "k" else np.ascontiguousarray(v[..., :n])
    return out


def oracle_at(m, st):
    o = Oracle(m, NREP, seed=SEED)
    o.set_state(st)
    o.rebuild()
    return o


@pytest.fixture(scope="module")
def fp64_start(model):
    d, st = worn(model, 64)
    s = d.download()
    assert st[-1] <= 1e-6 * st[:-1:2].sum()               # guard events are rare at the default cap
    return d, s


def test_config1_class_pass_fp64(model, fp64_start):
    """A whole colour class of the FP64 build at the benchmarked size against the oracle."""
    m = model
    d, s0 = fp64_start
    st0 = sub(s0)
    nm, ns = nmoves(m), (T + 1 - CLS) // 2
    d.upload(s0)
    d.set_move_log(NREP)
    d.rebuild()
    o = oracle_at(m, st0)
    sd = d.class_pass(SWEEP, CLS)
    tlog = np.full((nm, ns, NREP), np.nan)
    so = o.class_pass_range(SWEEP, CLS, 0, -1, tlog)
    # the same moves were tried (every task tries the class's list: 32x the oracle's two replicas)
    assert np.array_equal(sd[:-1:2], (R // NREP) * so[:-1:2])
    tdev = d.move_log(CLS, nm, ns)
    a, b = sub(d.download()), o.get_state()
    frac, worst = task_flips(a, b, m, 1e-9, 1e-9)
    first = first_diffs(tdev, tlog, 1e-9, 1e-12)
    flips = explain_flips(lambda: oracle_at(m, st0), SWEEP, CLS, first, tdev, MAXNATS)
    print(f"config 1 FP64 class pass: {ns * NREP} tasks, flipped {frac:.4f} (first differing draw in "
          f"{(first >= 0).mean():.4f}), worst other {worst:.2e}, guards device {sd[-1]} oracle {so[-1]}")
    print("flips by kind (count, largest margin):", summary(flips))
    for f in sorted(flips, key=lambda f: -f["margin"])[:5]:
        print({k: f[k] for k in ("q", "rep", "move", "kind", "margin", "fam", "entries", "t", "t_dev")})
    assert frac <= 0.02
    assert all(f["margin"] <= (1e-6 if f["kind"] == "offset" else 1e-8) for f in flips), summary(flips)
    d.set_move_log(0)


@pytest.fixture(scope="module")
def fp32_start(model):
    d, st = worn(model, 32)
    return d, d.download()


@pytest.mark.parametrize("limit", [1, 5, 20])
def test_config1_moves_fp32(model, fp32_start, limit):
    """The first `limit` moves of every task of the FP32 production build at the benchmarked size."""
    m = model
    d, s0 = fp32_start
    st0 = sub(s0)
    nm, ns = nmoves(m), (T + 1 - CLS) // 2
    d.upload(s0)
    d.set_move_log(NREP)
    d.rebuild()
    o = oracle_at(m, st0)
    sd = d.class_pass(SWEEP, CLS, limit)
    tlog = np.full((nm, ns, NREP), np.nan)
    so = o.class_pass_range(SWEEP, CLS, 0, limit, tlog)
    assert np.array_equal(sd[:-1:2], (R // NREP) * so[:-1:2])
    tdev = d.move_log(CLS, nm, ns)
    frac, worst = task_flips(sub(d.download()), o.get_state(), m, 2e-3, 4e-3)
    first = first_diffs(tdev[:limit], tlog[:limit], 1e-4, 1e-6)
    flips = explain_flips(lambda: oracle_at(m, st0), SWEEP, CLS, first, tdev, MAXNATS, fp32=True)
    print(f"config 1 FP32 first {limit} moves: flipped {frac:.4f} (first differing draw in "
          f"{(first >= 0).mean():.4f}), worst other {worst:.2e}; flips by kind:", summary(flips))
    for f in sorted(flips, key=lambda f: -f["margin"])[:5]:
        print({k: f.get(k) for k in ("q", "rep", "move", "kind", "margin", "fam", "entries", "t", "t_dev", "gL", "L")})
    assert frac <= 0.02
    assert all(f["margin"] <= (2e-2 if f["kind"] == "offset" else 5e-3) for f in flips), summary(flips)
    d.set_move_log(0)


def test_config1_sweep_state_finite(model):
    """Every state value stays finite over FP32 sweeps at the benchmarked size (about five of the
    3.6e8 line moves of a sweep draw an offset uniform that rounds to 1 in FP32; they must not make
    an infinite step), and so do the capacity scores."""
    d = DeviceChain(model, R, precision=32, seed=SEED)
    d.upload(initial_state(model, R, seed=7))
    d.sweeps(2, 0)
    s = d.download()
    for k in ("theta", "g", "e"):
        assert np.all(np.isfinite(s[k])), k
    sk, fk, parts = d.scores()
    assert np.all(np.isfinite(sk)) and np.all(np.isfinite(parts))
    d.close()


def test_config1_weather_finite(model):
    """The weather anomalies stay finite over FP32 weather steps of every replica at the benchmarked
    size: a step draws n0 * T * R normals, some of whose uniforms round to 1 in FP32 (a Box-Muller
    radius from log(1 - u) must not become infinite and spread along the VAR recursion)."""
    d = DeviceChain(model, R, precision=32, seed=SEED)
    d.upload(initial_state(model, R, seed=7))
    moved = np.ones(R, np.int32)
    theta = np.full(R, 0.7)
    window = np.zeros(R, np.int32)
    wstart = np.ones(R, np.int32)
    for it in range(1, 9):
        d.weather_step(moved, theta, window, wstart, it=it)
    s = d.download()
    assert np.all(np.isfinite(s["z"])) and np.all(np.isfinite(s["g"]))
    d.close()
