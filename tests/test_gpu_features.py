"""The weather features of every replica on the device (esm_replica_features: weather_features /
replica_features, src/replicas.jl:246-276) against their host restatement (replicas.weather_features)
on the chain's own weather, in both precisions: the load, carrier availabilities and residual-load
columns to 1e-12 relative in FP64 (the FP32 build maps its FP32 anomalies in FP32: 1e-5), the
regime frequencies and switches exactly; and the stress tilt of the replica step evaluated on the
device (TiltFunctional, :278): Phi per replica and the tilted drift weights."""
import numpy as np
import pytest

from esmgb import replicas as RP
from esmgb.device import DeviceChain
from esmgb.model import LANGEVIN_KAPPA, initial_state, make_model

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision,T,R", [(64, 120, 16), (32, 120, 16), (32, 8760, 64)])
def test_replica_features_match_host(precision, T, R):
    m = make_model(40, 60, T, seed=5)
    d = DeviceChain(m, R, precision=precision, seed=3)
    d.upload(initial_state(m, R, seed=7))
    ctl = RP.ReplicaCtl(M=R)
    rng = np.random.Generator(np.random.PCG64(4))
    # one weather step of every replica (pCN at angle pi/2 and a regime window): fresh anomalies
    moved = np.ones(R, np.int32)
    theta = np.full(R, np.pi / 2)
    window = np.full(R, min(ctl.window, T // 2), np.int32)
    wstart = np.array([RP.window_bounds(T, int(window[0]), rng.random())[0] for _ in range(R)], np.int32)
    d.weather_step(moved, theta, window, wstart, it=3)
    kref = np.asarray(m.unit_hi, float) * 0.3
    f = d.replica_features(kref)
    names = RP.replica_feature_names(m)
    assert f.shape == (R, len(names))
    st = d.download()
    check = range(R) if T <= 120 else (0, 17, 63)
    rtol, atol = (1e-12, 1e-9) if precision == 64 else (1e-5, 1e-4)   # GW: 0.1 MW in FP32
    nreg = m.K
    for j in check:
        h = RP.weather_features(m, st["z"][:, :, j], st["reg"][:, j], kref)
        np.testing.assert_allclose(f[j, :-nreg - 1], h[:-nreg - 1], rtol=rtol, atol=atol)
        np.testing.assert_array_equal(f[j, -nreg - 1:], h[-nreg - 1:])
    assert np.all(np.isfinite(f))
    # bitwise repeatable
    assert np.array_equal(f, d.replica_features(kref))
    d.close()


def test_tilt_on_the_device():
    m = make_model(40, 60, 120, seed=5)
    R = 16
    d = DeviceChain(m, R, precision=32, seed=3)
    d.upload(initial_state(m, R, seed=7))
    kref = np.asarray(m.unit_hi, float) * 0.3
    Phi = RP.TiltFunctional(m, kref, np.random.Generator(np.random.PCG64(2)), n=30)
    ks = np.array([LANGEVIN_KAPPA.get(c, 100.0) for c in m.carriers])
    ctl = RP.ReplicaCtl(M=R, Phi=Phi, lam=1.5)
    Rs = RP.ReplicaSet(M=R, eta_w=[5e-4] * len(m.carriers))
    rec = RP.replica_step(d, Rs, ctl, 2, np.random.Generator(np.random.PCG64(5)), ks, m.beta_k / m.beta_v,
                          m.unit_hi, m.unit_group)
    phis = rec["Phis"]
    assert phis.shape == (R,) and np.all(np.isfinite(phis)) and np.ptp(phis) > 0
    act = rec["wts"] > 0
    w = np.where(act, np.exp(1.5 * phis - (1.5 * phis[act]).max()), 0.0)
    np.testing.assert_allclose(rec["wts"], w / w.sum(), rtol=1e-14)
    d.close()
