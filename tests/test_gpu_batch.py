"""A batch of chains of uneven sizes (esm_batch_*: one captured graph per sweep, one line-move launch
per move index over the tasks of every chain) against each chain's own context: the batch changes
where a task runs, not its arithmetic, so every chain's state after the batch's sweeps equals,
bit for bit, the state its own esm_operation_sweeps gives, with the same move counts per family.
Covered: chains of different node counts, odd and even T (three and two colour classes), different
replica counts (one class step per warp item, and several), a model whose walk buffers exceed the
lanes' local arrays (the batch's global slabs), both block shapes and both precisions; and the
batch's autotuner leaving every chain as it found it."""
import numpy as np
import pytest

from esmgb.device import DeviceBatch, DeviceChain
from esmgb.model import initial_state, make_model

pytestmark = pytest.mark.gpu

SPECS = [  # (nodes, lines, T, replicas, model seed)
    (10, 15, 73, 16, 101),    # odd T: three colour classes
    (40, 60, 40, 32, 102),
    (24, 36, 30, 8, 103),     # 8 replicas: four class steps per warp item
    (17, 26, 24, 16, 104),
]
BIG = (128, 192, 24, 8, 105)  # lane layout beyond the local arrays (global walk slabs)


def _chains(specs, precision):
    out = []
    for N, L, T, R, seed in specs:
        m = make_model(N, L, T, seed=seed)
        st = initial_state(m, R, seed=7)
        rng = np.random.Generator(np.random.PCG64(seed))
        st.e = rng.uniform(0.05, 0.95, st.e.shape)
        out.append((m, R, seed, st))
    return out


def _pair(spec, precision):
    m, R, seed, st = spec
    a = DeviceChain(m, R, precision=precision, seed=seed)
    b = DeviceChain(m, R, precision=precision, seed=seed)
    a.upload(st)
    b.upload(st)
    return a, b


def _equal(a, b):
    sa, sb = a.download(), b.download()
    return all(np.array_equal(sa[k], sb[k]) for k in ("theta", "g", "e", "z", "reg", "k"))


@pytest.mark.parametrize("precision,wpb", [(64, 1), (32, 1), (32, 2)])
def test_batch_equals_own_contexts(precision, wpb):
    specs = _chains(SPECS + ([BIG] if precision == 64 else []), precision)
    pairs = [_pair(s, precision) for s in specs]
    batch = DeviceBatch([p[0] for p in pairs])
    batch.set_grid(wpb, 0)
    assert batch.grid()[0] == wpb
    st_b = batch.sweeps(2, sweep0=7)
    st_b2 = batch.sweeps(1, sweep0=9)
    for i, (a, b) in enumerate(pairs):
        s1 = b.sweeps(2, sweep0=7)
        s2 = b.sweeps(1, sweep0=9)
        assert np.array_equal(st_b[i], s1), (i, st_b[i], s1)
        assert np.array_equal(st_b2[i], s2), i
        assert st_b[i][:-1:2].sum() > 0
        assert _equal(a, b), f"chain {i} ({specs[i][0].N} nodes, T = {specs[i][0].T}) differs"
    assert batch.launch_count() > 0
    assert batch.last_ms() > 0
    # the chains stay usable on their own after the batch
    a, b = pairs[0]
    a.sweeps(1, 20)
    b.sweeps(1, 20)
    assert _equal(a, b)
    batch.close()
    for a, b in pairs:
        a.close()
        b.close()


def test_batch_autotune_keeps_state():
    specs = _chains(SPECS, 32)
    pairs = [_pair(s, 32) for s in specs]
    batch = DeviceBatch([p[0] for p in pairs])
    best, cand = batch.autotune(sweep=3)
    print(f"batch autotuner: best {best}, candidates {cand}")
    assert best in cand and len(cand) >= 4
    assert batch.grid()[:2] == best
    for a, b in pairs:
        assert _equal(a, b)
    st = batch.sweeps(1, sweep0=4)
    for i, (a, b) in enumerate(pairs):
        assert np.array_equal(st[i], b.sweeps(1, sweep0=4))
        assert _equal(a, b)
    batch.close()


def test_batch_rejects():
    m = make_model(10, 15, 30, seed=1)
    a = DeviceChain(m, 8, precision=32, seed=1)
    b = DeviceChain(m, 8, precision=64, seed=1)
    c = DeviceChain(m, 8, precision=32, seed=1, storage_ms=1)
    for chains in ([a, b], [a, a], [a, c]):
        with pytest.raises(Exception):
            DeviceBatch(chains)
    bt = DeviceBatch([a])
    with pytest.raises(Exception):  # no state uploaded
        bt.sweeps(1)
    with pytest.raises(Exception):
        bt.set_grid(4, 0)
    bt.close()
    for x in (a, b, c):
        x.close()
