"""Snapshots of the replica driver: write_replica_snapshot / read_replica_snapshot
(src/replicas.jl:1080-1167) with the atomic write of src/checkpoint.jl:31.

A snapshot holds what the reference's holds, under the same dataset names: `version`, `driver`
("replicas"), `phase`, `it`, `where`, `restarts`, `written`, `co2_price`, `config/seed`,
`nchains`, and per chain `chains/<c>/` (1-based, as there) `start`, `replicas`, `eta_w`, `since`,
`window`, `active`, the monitored trace `Q` and the record groups `trace/<key>` and `probe/<key>`
(one column per record, record_matrix). Two things differ:
- the container is a NumPy `.npz` archive whose member names are those dataset paths (the HDF5
  library is not part of this build);
- the replica states are the chain's node values as the C ABI holds them (`state/theta`, `g`, `e`,
  `z` as [X, T, R] with the replica fastest, `state/reg` [T, R], `state/k` [K]), not the
  reference's per-replica basis coefficients (`replica/<j>/v`, `w`, `z0`).

The Philox streams of the device path are keyed by the sweep and step indices, so a chain resumed
from a snapshot taken after sweep `it` and continued from sweep `it` + 1 reproduces the
uninterrupted chain.
"""
from __future__ import annotations

import os
import time

import numpy as np

SNAPSHOT_VERSION = 1          # src/checkpoint.jl:110
STATE_KEYS = ("theta", "g", "e", "z", "reg", "k")


def atomic_write(path, write, sync=True):
    """src/checkpoint.jl:31 atomic_write: `write(stream)` into a temporary file beside `path`,
    fsync, then rename over `path`; the temporary file is removed if the writer fails."""
    d = os.path.dirname(os.path.abspath(path))
    os.makedirs(d, exist_ok=True)
    tmp = os.path.join(d, f".{os.path.basename(path)}.tmp{os.getpid()}")
    try:
        with open(tmp, "wb") as f:
            write(f)
            f.flush()
            if sync:
                os.fsync(f.fileno())
        os.replace(tmp, path)
    except BaseException:
        if os.path.exists(tmp):
            os.remove(tmp)
        raise
    return path


def _record_matrix(v):
    """Records (equal-length vectors) as the columns of a matrix (record_matrix)."""
    return np.stack([np.asarray(x, float) for x in v], axis=1)


def write_replica_snapshot(path, chains, *, it, seed, phase="warmup", where="", restarts=0, co2_price=0.0,
                           levels=((0, 0),)):
    """Write the snapshot of `chains`, a list of dicts with keys `chain` (an object with `R` and
    `download()` returning the state arrays: a DeviceChain), `set` (its ReplicaSet), `start` (the
    chain's start kind) and optionally `Q` (monitored trace, a list of vectors), `trace` and
    `probe` (record dictionaries: key -> list of vectors)."""
    data = {
        "version": np.int64(SNAPSHOT_VERSION), "driver": np.array("replicas"), "phase": np.array(str(phase)),
        "it": np.int64(it), "where": np.array(str(where)), "restarts": np.int64(restarts),
        "written": np.float64(time.time()), "co2_price": np.float64(co2_price),
        "config/seed": np.int64(seed), "config/levels": np.array([[a, b] for (a, b) in levels], np.int64).T,
        "nchains": np.int64(len(chains)),
    }
    for c, ch in enumerate(chains, start=1):
        g = f"chains/{c}"
        R = ch["set"]
        data[f"{g}/start"] = np.array(str(ch.get("start", "cold")))
        data[f"{g}/replicas"] = np.int64(ch["chain"].R)
        data[f"{g}/eta_w"] = np.asarray(R.eta_w, float)
        data[f"{g}/since"] = np.asarray(R.since, np.int64)
        data[f"{g}/window"] = np.asarray(R.window, np.int64)
        data[f"{g}/active"] = np.asarray(R.active, np.int64)
        if ch.get("Q"):
            data[f"{g}/Q"] = _record_matrix(ch["Q"])
        for grp in ("trace", "probe"):
            for k, v in (ch.get(grp) or {}).items():
                if len(v):
                    data[f"{g}/{grp}/{k}"] = _record_matrix(v)
        st = ch["chain"].download()
        for k in STATE_KEYS:
            data[f"{g}/state/{k}"] = np.ascontiguousarray(st[k])
    return atomic_write(path, lambda f: np.savez(f, **data))


class SnapshotError(RuntimeError):
    pass


def read_replica_snapshot(path, *, seed, shapes=None, levels=((0, 0),)):
    """Read a snapshot (None if `path` is empty or absent), checking as the reference does the
    driver, the format version, the levels, the seed and, with `shapes` (the state shapes of the
    chains to resume, e.g. DeviceChain.shapes()), the sizes of every chain's state. Returns a dict
    with `it`, `restarts`, `where`, `written`, `co2`, `phase`, and `sets`: per chain `start`,
    `replicas`, `eta_w`, `since`, `window`, `active`, `Q`, `trace`, `probe` and `state`."""
    if not path or not os.path.isfile(path):
        return None
    with np.load(path, allow_pickle=False) as f:
        keys = set(f.files)
        if "driver" not in keys or str(f["driver"]) != "replicas":
            raise SnapshotError(f"snapshot {path} is not a snapshot of the replica driver")
        v = int(f["version"])
        if v != SNAPSHOT_VERSION:
            raise SnapshotError(f"snapshot {path}: format version {v}, the code reads {SNAPSHOT_VERSION}")
        lv = np.array([[a, b] for (a, b) in levels], np.int64).T
        if not np.array_equal(f["config/levels"], lv):
            raise SnapshotError(f"snapshot {path}: levels differ from the configuration")
        if int(f["config/seed"]) != int(seed):
            raise SnapshotError(f"snapshot {path}: seed {int(f['config/seed'])}, the configuration has {seed}")
        sets = []
        for c in range(1, int(f["nchains"]) + 1):
            g = f"chains/{c}"
            st = {k: f[f"{g}/state/{k}"] for k in STATE_KEYS}
            if shapes is not None:
                for k, s in shapes.items():
                    if tuple(st[k].shape) != tuple(s):
                        raise SnapshotError(f"snapshot {path}: chain {c} {k} has shape {st[k].shape}, "
                                            f"the problem {tuple(s)}")
            recs = {}
            for grp in ("trace", "probe"):
                pre = f"{g}/{grp}/"
                recs[grp] = {k[len(pre):]: [f[k][:, j].copy() for j in range(f[k].shape[1])]
                             for k in keys if k.startswith(pre)}
            Q = f[f"{g}/Q"] if f"{g}/Q" in keys else np.zeros((0, 0))
            sets.append({
                "start": str(f[f"{g}/start"]), "replicas": int(f[f"{g}/replicas"]),
                "eta_w": f[f"{g}/eta_w"].astype(float).tolist(), "since": f[f"{g}/since"].astype(int).tolist(),
                "window": f[f"{g}/window"].astype(bool).tolist(), "active": f[f"{g}/active"].astype(bool).tolist(),
                "Q": [Q[:, j].copy() for j in range(Q.shape[1])], "trace": recs["trace"], "probe": recs["probe"],
                "state": st,
            })
        return {"it": int(f["it"]), "restarts": int(f["restarts"]), "where": str(f["where"]),
                "written": float(f["written"]), "co2": float(f["co2_price"]), "phase": str(f["phase"]),
                "sets": sets}


def resume_chain(snap_set, chain, R):
    """Load one chain of a read snapshot (src/replicas.jl:891-901): the state into `chain`
    (upload) and eta_w, since, window and active into the ReplicaSet `R`; its gate buffers,
    in-flight windows and probe gaps start empty, as in the fresh ReplicaSet of the reference's
    resume."""
    if snap_set["replicas"] != chain.R:
        raise SnapshotError(f"snapshot chain has {snap_set['replicas']} replicas, the chain {chain.R}")
    chain.upload(snap_set["state"])
    R.eta_w = list(snap_set["eta_w"])
    R.since = list(snap_set["since"])
    R.window = list(snap_set["window"])
    R.active = list(snap_set["active"])
    R.gbuf = [[] for _ in range(R.M)]
    R.hist = [[] for _ in range(R.M)]
    R.gaps = []
