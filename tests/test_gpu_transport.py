"""Parity of the compensated transport families tpot and tsoc (prep_tpot!, prep_tsoc!,
src/local.jl:1741, :1849) on the CUDA path with the oracle, on identical states and Philox streams.

The rates are the plain families' with tpot and tsoc at 0.1 each, as the flow design adds them
(flow_families, src/flowmoves.jl:333), and the two alone. Besides the perturbed start (mostly in
surplus, where the pro-rata compensation is inactive) a deficit state (low renewables, dispatch at
half output) makes the compensation act at every kink node. Bounds as the line-move tests: FP64
1e-9 with at most 2 % of the (step, replica) tasks flipped, FP32 2e-3 / 4e-3 over the first moves."""
import copy

import numpy as np
import pytest

from esmgb.device import DeviceChain
from esmgb.model import FAMILIES, FAMILY_RATES
from oracle.oracle import Oracle
from test_gpu_parity import make, task_flips

pytestmark = pytest.mark.gpu

FLOW = tuple(FAMILY_RATES[:9]) + (0.1, 0.1)
ONLY = (0.0,) * 9 + (1.0, 1.0)
TPOT, TSOC = FAMILIES.index("tpot"), FAMILIES.index("tsoc")


def deficit(st):
    s = copy.deepcopy(st)
    s.z[:] = -3.0
    s.g[:] = 0.5
    return s


@pytest.fixture(scope="module")
def base():
    return make()


@pytest.mark.parametrize("rates", [FLOW, ONLY], ids=["flow", "only"])
@pytest.mark.parametrize("state", ["start", "deficit"])
def test_transport_class_pass_fp64(base, rates, state):
    m, st = base
    st = deficit(st) if state == "deficit" else st
    d = DeviceChain(m, 32, precision=64, seed=5, rates=rates)
    d.upload(st)
    d.rebuild()
    o = Oracle(m, 32, seed=5, rates=rates)
    o.set_state(st)
    o.rebuild()
    sd = d.class_pass(3, 0)
    so = o.class_pass(3, 0)
    assert np.array_equal(sd[:-1:2], so[:-1:2])           # the same moves were tried
    assert sd[-1] == so[-1] == 0
    for f in (TPOT, TSOC):
        assert sd[2 * f] > 0 and sd[2 * f + 1] > 0
    frac, worst = task_flips(d.download(), o.get_state(), m, 1e-9, 1e-9)
    print(f"transport FP64 {state} {'flow' if rates == FLOW else 'only'}: tpot {sd[2 * TPOT + 1]}/{sd[2 * TPOT]}, "
          f"tsoc {sd[2 * TSOC + 1]}/{sd[2 * TSOC]} moved, flipped tasks {frac:.4f}, worst other {worst:.2e}")
    assert frac <= 0.02


@pytest.mark.parametrize("limit", [1, 5])
def test_transport_moves_fp32(base, limit):
    m, st = base
    st = deficit(st)
    d = DeviceChain(m, 32, precision=32, seed=5, rates=ONLY)
    d.upload(st)
    d.rebuild()
    o = Oracle(m, 32, seed=5, rates=ONLY)
    o.set_state(st)
    o.rebuild()
    sd = d.class_pass(3, 1, limit)
    so = o.class_pass(3, 1, limit)
    assert np.array_equal(sd[:-1:2], so[:-1:2])
    frac, worst = task_flips(d.download(), o.get_state(), m, 2e-3, 4e-3)
    print(f"transport FP32 first {limit} moves: flipped tasks {frac:.4f}, worst other {worst:.2e}")
    assert frac <= 0.05
