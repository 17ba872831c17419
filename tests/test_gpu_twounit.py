"""Device parity on the model with two dispatchable units at every node (OCGT and CCGT): there the
`pair` and `cellpair` selections make moves (prep_random!, src/local.jl:1608-1670) and the compensated
moves' Jacobian has |S| - 1 = 1 (logjac, src/local.jl:1868-1887), which the benchmark model (one
dispatchable unit per node) never exercises. The compensated transport families run at their flow
rates (0.1 each) beside the plain families.

Per family: the moves tried equal the oracle's exactly; the moves taken differ by no more than the
tasks whose draws differ; every task whose draws differ is explained at its first differing draw
(tests/flipdiag.py), FP64 within 1e-8 of its boundary (same-segment offsets within 1e-6 of the
length), FP32 (first 5 moves) within 5e-3 (offsets 2e-2)."""
import numpy as np
import pytest

from esmgb.cabi import NFAM
from esmgb.device import DeviceChain
from esmgb.model import initial_state, make_model
from oracle.oracle import Oracle

from flipdiag import explain_flips, first_diffs, summary
from test_gpu_parity import task_flips

pytestmark = pytest.mark.gpu

R, SEED, SWEEP, CLS = 32, 5, 3, 0
FAMS = ["unit", "pair", "xpair", "xlocc", "xloc", "potential", "cellpair", "cell", "spair", "tpot", "tsoc"]


def rates():
    from esmgb.model import FAMILY_RATES
    r = list(FAMILY_RATES)
    r[9] = r[10] = 0.1          # tpot, tsoc at their flow-design rates
    return r


@pytest.fixture(scope="module")
def start():
    m = make_model(40, 60, 40, seed=11, dispatch=("OCGT", "CCGT"))
    st = initial_state(m, R, seed=3)
    rng = np.random.Generator(np.random.PCG64(11))
    st.g = st.g + 0.05 * rng.standard_normal(st.g.shape)
    st.e = rng.uniform(0.05, 0.95, st.e.shape)
    st.theta = 30.0 * rng.standard_normal(st.theta.shape)
    o = Oracle(m, R, seed=21, rates=rates())
    o.set_state(st)
    o.sweeps(2, 100)
    return m, o.get_state()


def nmoves(m):
    return sum(len(a.ptr) - 1 for a in m.atoms) + int(round(4.0 * m.N))


def oracle_at(m, st):
    o = Oracle(m, R, seed=SEED, rates=rates())
    o.set_state(st)
    o.rebuild()
    return o


@pytest.mark.parametrize("prec", [64, 32])
def test_two_unit_class_pass(start, prec):
    m, st = start
    nm, ns = nmoves(m), m.T // 2
    d = DeviceChain(m, R, precision=prec, seed=SEED, rates=rates())
    d.upload(st)
    d.set_move_log(R)
    d.rebuild()
    o = oracle_at(m, st)
    limit = 0 if prec == 64 else 5
    sd = d.class_pass(SWEEP, CLS, limit)
    tlog = np.full((nm, ns, R), np.nan)
    so = o.class_pass_range(SWEEP, CLS, 0, limit if limit else -1, tlog)
    tdev = d.move_log(CLS, nm, ns)
    tried_d, tried_o = sd[:-1:2], so[:-1:2]
    moved_d, moved_o = sd[1:-1:2], so[1:-1:2]
    assert np.array_equal(tried_d, tried_o)
    if prec == 64:      # every family makes moves on this model
        for f in ("pair", "cellpair", "xlocc", "tpot", "tsoc"):
            assert tried_o[FAMS.index(f)] > 0 and moved_o[FAMS.index(f)] > 0, f
    nl = limit if limit else nm
    tol_rel, tol_abs = (1e-9, 1e-12) if prec == 64 else (1e-4, 1e-6)
    first = first_diffs(tdev[:nl], tlog[:nl], tol_rel, tol_abs)
    ndiff = int((first >= 0).sum())
    assert np.all(np.abs(moved_d - moved_o) <= ndiff)
    st_tol = (1e-9, 1e-9) if prec == 64 else (2e-3, 4e-3)
    frac, worst = task_flips(d.download(), o.get_state(), m, *st_tol)
    flips = explain_flips(lambda: oracle_at(m, st), SWEEP, CLS, first, tdev, 40.0, fp32=prec == 32)
    fam_names = FAMS + ["atoms"]
    print(f"two-unit model FP{prec}{'' if limit == 0 else f' first {limit} moves'}: tried/taken per family "
          + ", ".join(f"{fam_names[i]} {tried_o[i]}/{moved_d[i]}:{moved_o[i]}" for i in range(NFAM + 1) if tried_o[i])
          + f"; flipped {frac:.4f}, tasks with a differing draw {(first >= 0).mean():.4f}; by kind:", summary(flips))
    for f in sorted(flips, key=lambda f: -f["margin"])[:4]:
        print({k: f.get(k) for k in ("q", "rep", "move", "kind", "margin", "fam", "entries", "t", "t_dev", "lj", "uj")})
    assert frac <= 0.02
    bound = (lambda f: 1e-6 if f["kind"] == "offset" else 1e-8) if prec == 64 else \
        (lambda f: 2e-2 if f["kind"] == "offset" else 5e-3)
    assert all(f["margin"] <= bound(f) for f in flips), summary(flips)
    d.set_move_log(0)
    d.close()
