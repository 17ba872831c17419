"""A device chain resumed from a snapshot (write_replica_snapshot / read_replica_snapshot,
src/replicas.jl:1080-1167) continues exactly as the uninterrupted chain: the sweeps rebuild their
caches from the state and draw from streams keyed by the sweep index, so the FP32 state after the
next sweep is bit-identical."""
import numpy as np
import pytest

from esmgb import replicas as RP
from esmgb import snapshot as SN
from esmgb.device import DeviceChain
from test_gpu_parity import make

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("prec", [32, 64])
def test_device_resume_continues_the_chain(tmp_path, prec):
    m, st = make(T=40)
    a = DeviceChain(m, 32, precision=prec, seed=5)
    a.upload(st)
    a.sweeps(2, 0)
    R = RP.ReplicaSet(M=32, eta_w=[1e-3])
    path = str(tmp_path / "snap.npz")
    SN.write_replica_snapshot(path, [{"chain": a, "set": R, "start": "cold"}], it=2, seed=5)
    a.sweeps(1, 2)
    want = a.download()
    b = DeviceChain(m, 32, precision=prec, seed=5)
    snap = SN.read_replica_snapshot(path, seed=5, shapes=b.shapes())
    SN.resume_chain(snap["sets"][0], b, RP.ReplicaSet(M=32, eta_w=[0.0]))
    b.sweeps(1, 2)
    got = b.download()
    for k in SN.STATE_KEYS:
        np.testing.assert_array_equal(got[k], want[k], err_msg=k)
