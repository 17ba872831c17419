"""The whole-class launch of the line moves (esm_set_move_schedule, ESM_MOVES_PER_CLASS): one
launch per class pass whose warps run an item's next move as soon as its previous one is done,
against the default one launch per move. The tasks of a colour class are independent, so every
task runs the same moves on the same values: the states and the move counts must be equal bit for
bit, in both precisions, with several class steps per warp item (8 replicas), an odd T (three
classes), a model whose walk buffers live in the global slabs (128 nodes), every block shape, a
move limit, and the move log."""
import numpy as np
import pytest

from esmgb.device import DeviceChain
from esmgb.model import initial_state, make_model

pytestmark = pytest.mark.gpu


def _state(m, R, seed):
    st = initial_state(m, R, seed=7)
    rng = np.random.Generator(np.random.PCG64(seed))
    st.e = rng.uniform(0.05, 0.95, st.e.shape)
    st.g = np.clip(st.g + 0.05 * rng.standard_normal(st.g.shape), 0, 1)
    return st


def _equal(a, b):
    sa, sb = a.download(), b.download()
    return all(np.array_equal(sa[k], sb[k]) for k in ("theta", "g", "e", "z", "reg", "k"))


CASES = [  # (nodes, lines, T, replicas, precision, grid)
    (40, 60, 40, 32, 64, (1, 0)),
    (40, 60, 40, 32, 32, (2, 0)),
    (24, 36, 73, 8, 32, (4, 0)),      # odd T, four class steps per item
    (24, 36, 73, 8, 64, (1, 8)),
    (128, 192, 24, 8, 64, (1, 0)),    # global walk slabs
]


@pytest.mark.parametrize("N,L,T,R,precision,grid", CASES)
def test_whole_class_launch_equals_per_move(N, L, T, R, precision, grid):
    m = make_model(N, L, T, seed=N + T)
    st = _state(m, R, N + T)
    a = DeviceChain(m, R, precision=precision, seed=9)
    b = DeviceChain(m, R, precision=precision, seed=9)
    for d in (a, b):
        d.upload(st)
        d.set_move_grid(*grid)
    a.set_move_schedule("class")
    assert a.move_schedule() == "class" and b.move_schedule() == "move"
    sa = a.sweeps(2, 5)
    sb = b.sweeps(2, 5)
    assert np.array_equal(sa, sb), (sa, sb)
    assert sa[:-1:2].sum() > 0
    assert _equal(a, b)
    # a move limit (the first 7 moves of class 1)
    assert np.array_equal(a.class_pass(8, 1, 7), b.class_pass(8, 1, 7))
    assert _equal(a, b)
    # back to per-move launches on the same chain
    a.set_move_schedule("move")
    assert np.array_equal(a.sweeps(1, 9), b.sweeps(1, 9))
    assert _equal(a, b)
    a.close()
    b.close()


def test_whole_class_launch_move_log():
    m = make_model(40, 60, 40, seed=3)
    st = _state(m, 32, 3)
    a = DeviceChain(m, 32, precision=64, seed=4)
    b = DeviceChain(m, 32, precision=64, seed=4)
    for d in (a, b):
        d.upload(st)
        d.set_move_log(2)
    a.set_move_schedule("class")
    nm = sum(len(x.ptr) - 1 for x in m.atoms) + int(round(4.0 * m.N))
    a.class_pass(1, 0)
    b.class_pass(1, 0)
    la = a.move_log(0, nm, m.T // 2)
    lb = b.move_log(0, nm, m.T // 2)
    assert np.array_equal(np.isnan(la), np.isnan(lb))
    assert np.array_equal(np.nan_to_num(la), np.nan_to_num(lb))
    a.close()
    b.close()
