"""Chain marginals of the CUDA path (FP32, production) against the CPU oracle (FP64): independent
chains (different seeds) from the same start must agree on the posterior means of the line flows
and dispatch (local sweeps at fixed capacities) and of the carrier capacity totals (the replica
step with the Langevin capacity move) within 2 MCSE, |mean_A - mean_B| <= 2 sqrt(MCSE_A^2 + MCSE_B^2)
(the reference's agreement metric, src/convergence.jl:141). With many marginals a few fall outside
2 MCSE by chance (about 5 % each); the tests require 85 % of them inside and none beyond 4 MCSE.
The flows and dispatch mix slowly (the angles wander where the potential is flat between line
limits): their MCSE comes from the spread of 4 independent chains per side, with the thresholds
of a 4-chain estimate (80 % within 2, none beyond 4.5)."""
import math

import numpy as np
import pytest

from esmgb.convergence import ess_single
from esmgb.device import DeviceChain
from esmgb.model import LANGEVIN_KAPPA, initial_state, make_model
from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu


def _z(a, b):
    """|mean difference| in units of the combined MCSE, per column."""
    out = []
    for j in range(a.shape[1]):
        x, y = a[:, j], b[:, j]
        sx = x.std(ddof=1) / math.sqrt(max(ess_single(x), 1.0))
        sy = y.std(ddof=1) / math.sqrt(max(ess_single(y), 1.0))
        s = math.sqrt(sx ** 2 + sy ** 2)
        out.append(abs(x.mean() - y.mean()) / s if s > 0 else (0.0 if x.mean() == y.mean() else np.inf))
    return np.array(out)


def _check(z, what, min_frac=0.85, max_z=4.0):
    frac = float(np.mean(z <= 2.0))
    print(f"{what}: {frac:.3f} of {len(z)} marginals within 2 MCSE, max {z.max():.2f}")
    assert frac >= min_frac, (what, frac)
    assert z.max() <= max_z, (what, z.max())


def _zk(A, B):
    """Marginals of K independent chains per side: |mean_A - mean_B| over the combined standard
    error of the chain means (between-chain spread: robust to the slow mixing of the flows, whose
    single-chain autocorrelation estimates are unreliable over a few hundred sweeps)."""
    A, B = np.asarray(A), np.asarray(B)            # [K, n, ncols]
    ma, mb = A.mean(axis=1), B.mean(axis=1)        # [K, ncols] chain means
    se = np.sqrt(ma.var(axis=0, ddof=1) / len(ma) + mb.var(axis=0, ddof=1) / len(mb))
    d = np.abs(ma.mean(0) - mb.mean(0))
    return np.where(se > 0, d / np.where(se > 0, se, 1), np.where(d == 0, 0.0, np.inf))


def test_flow_and_dispatch_marginals():
    m = make_model(12, 18, 24, seed=7)
    R = 4
    st = initial_state(m, R, seed=3)
    K, burn, n = 4, 200, 500
    Fd, Fo, Gd, Go = [], [], [], []
    for k in range(K):
        d = DeviceChain(m, R, precision=32, seed=101 + k)
        d.upload(st)
        o = Oracle(m, R, seed=501 + k)
        o.set_state(st)
        fd, fo, gd, go = [], [], [], []
        for s in range(burn + n):
            d.sweeps(1, s, stats=False)
            o.sweeps(1, s)
            if s < burn:
                continue
            d.rebuild()
            fd.append(d.caches()[1].mean(axis=(1, 2)))
            gd.append(d.download()["g"].mean(axis=(1, 2)))
            o.rebuild()
            fo.append(o.caches()[1].mean(axis=(1, 2)))
            go.append(o.get_state()["g"].mean(axis=(1, 2)))
        Fd.append(fd), Fo.append(fo), Gd.append(gd), Go.append(go)
        d.close()
    _check(_zk(Fd, Fo), "line flows (4 chains a side)", min_frac=0.8, max_z=4.5)
    _check(_zk(Gd, Go), "dispatch (4 chains a side)", min_frac=0.8, max_z=4.5)


def test_capacity_marginals():
    m = make_model(12, 18, 24, seed=7)
    R = 4
    st = initial_state(m, R, seed=3)
    eta = np.full(len(m.carriers), 5e-3)                 # faster mixing than production, same on both sides
    ks = np.array([LANGEVIN_KAPPA.get(c, 100.0) for c in m.carriers])
    w = np.full(R, 1.0 / R)
    d = DeviceChain(m, R, precision=32, seed=101)
    d.upload(st)
    o = Oracle(m, R, seed=202)
    o.set_state(st)
    ug = np.asarray(m.unit_group)
    ng = len(m.carriers)
    burn, n = 200, 1200
    Kd, Ko = [], []
    for s in range(burn + n):
        d.sweeps(1, s, stats=False)
        d.scores()
        kd, _ = d.langevin_step(w, eta, ks, 1.0, 0.02, True, None, s)
        o.sweeps(1, s)
        o.scores()
        ko, _ = o.langevin_step(w, eta, ks, 1.0, 0.02, True, None, s)
        if s >= burn:
            Kd.append([kd[ug == g].sum() for g in range(ng)])
            Ko.append([ko[ug == g].sum() for g in range(ng)])
    Kd, Ko = np.array(Kd), np.array(Ko)
    moving = eta > 0
    _check(_z(Kd[:, moving], Ko[:, moving]), "carrier capacity totals")
