"""Snapshots of the replica driver (write_replica_snapshot / read_replica_snapshot,
src/replicas.jl:1080-1167) on the CPU, with the oracle standing in for the device chain: a chain
resumed from a snapshot continues exactly as the uninterrupted chain, the bookkeeping round-trips,
and the reference's checks (driver, version, levels, seed, sizes) reject a foreign snapshot."""
import numpy as np
import pytest

from esmgb import replicas as RP
from esmgb import snapshot as SN
from esmgb.model import initial_state, make_model
from oracle.oracle import Oracle


class OracleChain:
    """The two calls of the device chain a snapshot uses, on the oracle."""

    def __init__(self, o):
        self.o, self.R = o, o.R

    def download(self):
        return self.o.get_state()

    def upload(self, st):
        self.o.set_state(st)

    def shapes(self):
        return self.o.shapes()


@pytest.fixture(scope="module")
def small():
    m = make_model(12, 18, 24, seed=4)
    return m, initial_state(m, 4, seed=2)


def test_resume_continues_the_chain(small, tmp_path):
    m, st = small
    a = Oracle(m, 4, seed=9)
    a.set_state(st)
    a.sweeps(2, 0)
    R = RP.ReplicaSet(M=4, eta_w=[1e-3, 2e-3])
    R.since, R.window, R.active = [3, 0, 7, 1], [True, False, False, True], [True, False, True, True]
    R.gbuf[1].append([0.5])
    R.hist[0].append(np.ones(m.Kunits))
    path = str(tmp_path / "snap.npz")
    SN.write_replica_snapshot(path, [{"chain": OracleChain(a), "set": R, "start": "cold",
                                      "Q": [np.arange(3.0), np.arange(3.0) + 1],
                                      "probe": {"gap": [np.array([0.1]), np.array([0.2])]}}],
                              it=2, seed=9, phase="warmup", where="step 2")
    assert not [p for p in tmp_path.iterdir() if p.name.endswith(".tmp") or ".tmp" in p.name]
    a.sweeps(1, 2)
    want = a.get_state()

    b = Oracle(m, 4, seed=9)
    chain = OracleChain(b)
    snap = SN.read_replica_snapshot(path, seed=9, shapes=chain.shapes())
    assert snap["it"] == 2 and snap["phase"] == "warmup" and snap["where"] == "step 2"
    s1 = snap["sets"][0]
    assert s1["start"] == "cold" and s1["replicas"] == 4
    np.testing.assert_array_equal(s1["Q"][1], np.arange(3.0) + 1)
    np.testing.assert_array_equal(s1["probe"]["gap"][1], [0.2])
    R2 = RP.ReplicaSet(M=4, eta_w=[0.0, 0.0])
    SN.resume_chain(s1, chain, R2)
    assert R2.eta_w == R.eta_w and R2.since == R.since and R2.window == R.window and R2.active == R.active
    assert R2.gbuf == [[]] * 4 and R2.hist == [[]] * 4 and R2.gaps == []
    b.sweeps(1, 2)
    got = b.get_state()
    for k in SN.STATE_KEYS:
        np.testing.assert_array_equal(got[k], want[k], err_msg=k)


def test_snapshot_checks(small, tmp_path):
    m, st = small
    o = Oracle(m, 4, seed=9)
    o.set_state(st)
    R = RP.ReplicaSet(M=4, eta_w=[1e-3])
    path = str(tmp_path / "s.npz")
    assert SN.read_replica_snapshot(str(tmp_path / "none.npz"), seed=9) is None
    assert SN.read_replica_snapshot("", seed=9) is None
    SN.write_replica_snapshot(path, [{"chain": OracleChain(o), "set": R}], it=5, seed=9)
    with pytest.raises(SN.SnapshotError, match="seed"):
        SN.read_replica_snapshot(path, seed=10)
    with pytest.raises(SN.SnapshotError, match="levels"):
        SN.read_replica_snapshot(path, seed=9, levels=((1, 0),))
    other = make_model(12, 18, 30, seed=4)
    with pytest.raises(SN.SnapshotError, match="shape"):
        SN.read_replica_snapshot(path, seed=9, shapes=Oracle(other, 4).shapes())
    with np.load(path) as f:
        data = {k: f[k] for k in f.files}
    for key, val, msg in (("driver", np.array("chains"), "not a snapshot"), ("version", np.int64(2), "version")):
        bad = dict(data, **{key: val})
        p2 = str(tmp_path / f"bad_{key}.npz")
        np.savez(p2, **bad)
        with pytest.raises(SN.SnapshotError, match=msg):
            SN.read_replica_snapshot(p2, seed=9)
    snap = SN.read_replica_snapshot(path, seed=9)
    with pytest.raises(SN.SnapshotError, match="replicas"):
        SN.resume_chain(snap["sets"][0], OracleChain(Oracle(m, 2, seed=9)), RP.ReplicaSet(M=2, eta_w=[1e-3]))


def test_atomic_write_leaves_no_partial_file(tmp_path):
    path = str(tmp_path / "x.npz")

    def boom(f):
        f.write(b"partial")
        raise OSError("disk full")

    with pytest.raises(OSError):
        SN.atomic_write(path, boom)
    assert list(tmp_path.iterdir()) == []
    SN.atomic_write(path, lambda f: f.write(b"ok"))
    assert open(path, "rb").read() == b"ok" and len(list(tmp_path.iterdir())) == 1
