"""Parity of the storage multiscale sweep of the CUDA path (k_plateau through esm_storage_ms) with
the oracle on identical states and Philox streams.

A plateau move changes a replica over a whole block (L + 1 steps), and a discrete flip (a segment
chosen the other way on last-bit differences) carries into the block's later moves and into the
later passes, so parity is measured per (block, replica) task of the first class passes: FP64 1e-9
per element with at most 2 % of the tasks flipped (measured 0), FP32 4e-3 with at most 10 % (a task
runs 8 moves, each over L + 1 steps; measured 5-6 %, about 0.7 % per move, as the 20-move FP32 test
of the line moves). The whole sweep is checked for equal move counts and round-off agreement of the
unflipped entries."""
import numpy as np
import pytest

from esmgb.device import DeviceChain
from oracle.oracle import Oracle
from test_gpu_parity import make, task_flips

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def state():
    """The perturbed start after three oracle operation sweeps with the storage sweep (the regime
    the FP32 build is designed for, as the line-move parity tests)."""
    m, st = make(T=120)
    o = Oracle(m, 32, seed=21, storage_ms=1)
    o.set_state(st)
    o.sweeps(3, 100)
    s = o.get_state()
    for k in ("theta", "g", "e", "z", "reg", "k"):
        setattr(st, k, s[k])
    return m, st


def block_flips(sd, so, plan_pass, T, tol):
    """Fraction of the (block, replica) tasks of one class pass whose states differ beyond tol."""
    L, o, cls = plan_pass
    starts = [b0 for k, b0 in enumerate(range(o, T - L, L)) if k % 2 == cls]
    de = np.abs(sd["e"] - so["e"]).max(0)   # [T, R]
    dg = np.abs(sd["g"] - so["g"]).max(0)
    bad = [(np.maximum(de[b0:b0 + L + 1], dg[b0:b0 + L + 1]) > tol).any(0) for b0 in starts]
    return np.mean(bad), len(starts)


@pytest.mark.parametrize("prec,tol,maxflip", [(64, 1e-9, 0.02), (32, 4e-3, 0.10)])
@pytest.mark.parametrize("npass", [1, 2, 4])
def test_storage_ms_passes(state, prec, tol, maxflip, npass):
    m, st = state
    d = DeviceChain(m, 32, precision=prec, seed=5)
    d.upload(st)
    o = Oracle(m, 32, seed=5)
    o.set_state(st)
    plan = o.storage_ms_plan(7)
    sd, so = d.storage_ms(7, max_passes=npass), o.storage_ms(7, max_passes=npass)
    assert sd[0] == so[0] > 0          # the same moves were tried
    assert sd[2] == so[2] == 0         # no guard events
    a, b = d.download(), o.get_state()
    for p in plan[:npass]:
        frac, nb = block_flips(a, b, p, m.T, tol)
        print(f"storage_ms FP{prec} pass {p}: {nb} blocks x 32 replicas, flipped tasks {frac:.4f}")
        assert frac <= maxflip


def test_storage_ms_sweep(state):
    m, st = state
    d = DeviceChain(m, 32, precision=64, seed=5)
    d.upload(st)
    o = Oracle(m, 32, seed=5)
    o.set_state(st)
    sd, so = d.storage_ms(7), o.storage_ms(7)
    assert sd[0] == so[0] > 0 and sd[2] == so[2] == 0
    frac, worst = task_flips(d.download(), o.get_state(), m, 1e-9, 1e-9)
    print(f"storage_ms FP64 whole sweep: entries differing {frac:.4f}, worst other {worst:.2e}")
    assert worst <= 1e-9 and frac <= 0.5


def test_operation_sweeps_with_storage(state):
    """Operation sweeps with the storage multiscale sweep (its coin drawn per sweep) on both sides."""
    m, st = state
    d = DeviceChain(m, 32, precision=64, seed=5, storage_ms=1)
    d.upload(st)
    o = Oracle(m, 32, seed=5, storage_ms=1)
    o.set_state(st)
    assert any(bool(o.storage_ms_plan(s, force=False)) for s in range(3))
    sd, so = d.sweeps(3, 0), o.sweeps(3, 0)
    assert np.array_equal(sd[:-1:2], so[:-1:2])
    frac, worst = task_flips(d.download(), o.get_state(), m, 1e-9, 1e-9)
    print(f"3 operation sweeps with storage: entries differing {frac:.4f}, worst other {worst:.2e}")
    assert worst <= 1e-8 and frac <= 0.5


@pytest.mark.parametrize("prec,tol,maxflip", [(64, 1e-9, 0.03), (32, 4e-3, 0.10)])
def test_storage_long_sweep(state, prec, tol, maxflip):
    """The long-range storage sweep (storage_long_sweep!, src/storage_long.jl:245): every eligible
    unit's level move and long-range plateaus; parity per (unit, replica) task over the year (5 moves
    per task, each over up to the whole year: measured 1.8 % FP64, 1.2 % FP32 tasks flipped; the FP64
    flips are mirrored draws on segments flat to round-off, test_storage_long_flips_explained)."""
    m, st = state
    d = DeviceChain(m, 32, precision=prec, seed=5)
    d.upload(st)
    o = Oracle(m, 32, seed=5)
    o.set_state(st)
    plan = o.storage_long_plan(9)
    units = sorted({p[0] for p in plan})
    assert units and any(p[1] == m.T for p in plan) and any(p[1] < m.T for p in plan)
    sd, so = d.storage_long(9), o.storage_long(9)
    assert sd[0] == so[0] == len(plan) * 32
    assert sd[2] == so[2] == 0
    a, b = d.download(), o.get_state()
    de = np.abs(a["e"] - b["e"]).max(1)[units]          # [units, R]
    frac = (de > tol).mean()
    print(f"storage_long FP{prec}: {len(units)} units, moves {sd[0]}, taken {sd[1]} / {so[1]}, flipped tasks {frac:.4f}")
    assert frac <= maxflip
    if prec == 64:
        ok = de <= tol
        dg = np.abs(a["g"] - b["g"]).max()
        assert ok.all() or dg > 0  # (the dispatch follows the flipped tasks only)


def test_storage_long_flips_explained(state):
    """Each (unit, replica) task of the FP64 long-range sweep whose draws differ from the oracle's,
    explained at its first differing move (tests/flipdiag.py): the discrete choice there and how near
    its boundary the oracle's own draw was. Every one is a round-off flip: within 1e-8 of a segment,
    stop or Jacobian boundary, or the same segment with an offset within 1e-6 of its length, or a
    segment flat to round-off drawn from the other end (measured: these mirrored draws on flat
    segments of level moves and long plateaus, |g L| about 1e-10 nats, make up the flipped tasks)."""
    from flipdiag import classify, first_diffs, summary
    m, st = state
    R = 32
    d = DeviceChain(m, R, precision=64, seed=5)
    d.upload(st)
    d.set_move_log(R)
    o = Oracle(m, R, seed=5)
    o.set_state(st)
    plan = o.storage_long_plan(9)
    order = []
    for u, _, _ in plan:
        if u not in order:
            order.append(u)
    nu = len(order)
    d.storage_long(9)
    tdev = d.storage_long_log(nu)                       # [unit, move, replica]
    tlog = np.full((nu, 5, R), np.nan)
    o.storage_long_log(9, tlog)
    first = first_diffs(tdev.transpose(1, 0, 2), tlog.transpose(1, 0, 2), 1e-9, 1e-12)   # [unit, replica]
    o2 = Oracle(m, R, seed=5)
    o2.set_state(st)
    o2.rebuild()
    flips = []
    for ui, rep in zip(*np.nonzero(first >= 0)):
        mi = int(first[ui, rep])
        o2.sl_task(9, int(ui), int(rep), 0, mi)
        e = o2.sl_explain(9, int(ui), int(rep), mi, float(np.nan_to_num(tdev[ui, mi, rep])))
        assert e is not None
        e["t_dev"] = float(tdev[ui, mi, rep])
        kind, margin = classify(e, 40.0)
        flips.append(dict(unit=int(ui), rep=int(rep), move=mi, kind=kind, margin=margin, **e))
    print(f"storage_long FP64: {nu} units x {R} replicas, tasks with a differing draw {(first >= 0).mean():.4f};",
          "by kind (count, largest margin):", summary(flips))
    for f in sorted(flips, key=lambda f: -f["margin"])[:6]:
        print({k: f[k] for k in ("unit", "rep", "move", "kind", "margin", "fam", "entries", "t", "t_dev", "seg",
                                 "seg_other", "nseg", "npts_r", "npts_l", "gL", "L")})
    d.set_move_log(0)
    assert all(f["margin"] <= (1e-6 if f["kind"] == "offset" else 1e-8) for f in flips), summary(flips)
