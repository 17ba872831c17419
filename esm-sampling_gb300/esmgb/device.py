"""ctypes binding of libesmcuda.so (the C ABI of ``include/esmcuda.h``) and the replica-chain object
that drives it. This is the product path: there is no CPU fallback -- if the library cannot be
loaded, or no GPU is present, the calls fail loudly.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from .cabi import NFAM, EsmOpts, ModelBuffers, make_opts
from .model import SynthModel

P_f64 = C.POINTER(C.c_double)
P_i32 = C.POINTER(C.c_int32)
P_i64 = C.POINTER(C.c_int64)
NSTAT = 2 * (NFAM + 1) + 1

# the symbols declared in include/esmcuda.h
EXPORTS = ("esm_create", "esm_destroy", "esm_last_error", "esm_upload_state", "esm_download_state",
           "esm_rebuild_caches", "esm_download_caches", "esm_operation_sweeps", "esm_class_pass",
           "esm_capacity_scores", "esm_langevin_step", "esm_weather_step", "esm_sync", "esm_launch_count",
           "esm_set_timing", "esm_timing", "esm_stream", "esm_capacity_scores_static", "esm_score_errors",
           "esm_follow_capacities", "esm_state_save", "esm_state_restore", "esm_regime_occupancy", "esm_set_move_grid", "esm_move_grid",
           "esm_autotune_moves", "esm_storage_ms", "esm_storage_long", "esm_lag_probe", "esm_set_sep_walk",
           "esm_sep_walk", "esm_set_move_log", "esm_move_log", "esm_batch_create", "esm_batch_destroy",
           "esm_batch_last_error", "esm_batch_sweeps", "esm_batch_set_grid", "esm_batch_grid", "esm_batch_autotune",
           "esm_batch_time", "esm_batch_launch_count", "esm_set_move_schedule", "esm_move_schedule",
           "esm_replica_features")
TUNE_MAX = 16  # ESM_TUNE_MAX
KERNEL_FAMILIES = ("class_pass", "rebuild", "score", "langevin_follow", "weather", "storage")

_lib = None


class EsmError(RuntimeError):
    pass


def lib_path():
    from .build import LIB
    return LIB


def load(build_if_missing=True):
    """Load libesmcuda.so (building it in-tree if it is missing); raises if it cannot be loaded."""
    global _lib
    if _lib is not None:
        return _lib
    path = lib_path()
    if not os.path.exists(path):
        if not build_if_missing:
            raise EsmError(f"{path} is missing: run esmgb.build.build()")
        from .build import build
        build()
    L = C.CDLL(path)
    L.esm_create.restype = C.c_int
    L.esm_create.argtypes = [C.c_void_p, C.c_void_p, C.POINTER(C.c_void_p)]
    L.esm_destroy.argtypes = [C.c_void_p]
    L.esm_last_error.restype = C.c_char_p
    L.esm_last_error.argtypes = [C.c_void_p]
    L.esm_upload_state.argtypes = [C.c_void_p, P_f64, P_f64, P_f64, P_f64, P_i32, P_f64]
    L.esm_download_state.argtypes = [C.c_void_p, P_f64, P_f64, P_f64, P_f64, P_i32, P_f64]
    L.esm_rebuild_caches.argtypes = [C.c_void_p]
    L.esm_download_caches.argtypes = [C.c_void_p, P_f64, P_f64]
    L.esm_operation_sweeps.argtypes = [C.c_void_p, C.c_int32, C.c_int64, P_i64]
    L.esm_class_pass.argtypes = [C.c_void_p, C.c_int64, C.c_int32, C.c_int32, P_i64]
    L.esm_capacity_scores.argtypes = [C.c_void_p, P_f64, P_f64, P_f64]
    L.esm_capacity_scores_static.argtypes = [C.c_void_p, P_f64, P_f64, P_f64]
    L.esm_score_errors.argtypes = [C.c_void_p, P_f64, P_f64]
    L.esm_follow_capacities.argtypes = [C.c_void_p, P_f64, C.c_double, P_f64]
    L.esm_state_save.argtypes = [C.c_void_p]
    L.esm_state_restore.argtypes = [C.c_void_p]
    L.esm_regime_occupancy.argtypes = [C.c_void_p, P_f64]
    L.esm_langevin_step.argtypes = [C.c_void_p, P_f64, P_f64, P_f64, C.c_double, C.c_double, C.c_int32, P_f64,
                                    C.c_int64, P_f64, P_i32]
    L.esm_weather_step.argtypes = [C.c_void_p, P_i32, P_f64, P_i32, P_i32, P_f64, C.c_int64]
    L.esm_sync.argtypes = [C.c_void_p, C.c_double]
    L.esm_set_move_grid.argtypes = [C.c_void_p, C.c_int32, C.c_int32]
    L.esm_storage_ms.argtypes = [C.c_void_p, C.c_int64, C.c_int32, C.c_int32, P_i64]
    L.esm_storage_long.argtypes = [C.c_void_p, C.c_int64, P_i64]
    L.esm_lag_probe.argtypes = [C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_int64, P_f64, P_f64]
    L.esm_move_grid.argtypes = [C.c_void_p, P_i32, P_i32, P_i32]
    L.esm_set_sep_walk.argtypes = [C.c_void_p, C.c_int32]
    L.esm_set_move_log.argtypes = [C.c_void_p, C.c_int32]
    L.esm_move_log.argtypes = [C.c_void_p, C.c_int32, P_f64]
    L.esm_sep_walk.argtypes = [C.c_void_p, P_i32, P_i32]
    L.esm_autotune_moves.argtypes = [C.c_void_p, C.c_int64, P_i32, P_i32, P_f64, P_i32]
    L.esm_launch_count.restype = C.c_int64
    L.esm_launch_count.argtypes = [C.c_void_p]
    L.esm_set_timing.argtypes = [C.c_void_p, C.c_int32]
    L.esm_timing.argtypes = [C.c_void_p, P_f64]
    L.esm_stream.restype = C.c_void_p
    L.esm_stream.argtypes = [C.c_void_p]
    L.esm_replica_features.argtypes = [C.c_void_p, P_f64, P_f64, P_i32]
    L.esm_set_move_schedule.argtypes = [C.c_void_p, C.c_int32]
    L.esm_move_schedule.argtypes = [C.c_void_p, P_i32]
    L.esm_batch_create.argtypes = [C.POINTER(C.c_void_p), C.c_int32, C.POINTER(C.c_void_p)]
    L.esm_batch_destroy.argtypes = [C.c_void_p]
    L.esm_batch_last_error.restype = C.c_char_p
    L.esm_batch_last_error.argtypes = [C.c_void_p]
    L.esm_batch_sweeps.argtypes = [C.c_void_p, C.c_int32, C.c_int64, P_i64]
    L.esm_batch_set_grid.argtypes = [C.c_void_p, C.c_int32, C.c_int32]
    L.esm_batch_grid.argtypes = [C.c_void_p, P_i32, P_i32, P_i32]
    L.esm_batch_autotune.argtypes = [C.c_void_p, C.c_int64, P_i32, P_i32, P_f64, P_i32]
    L.esm_batch_time.argtypes = [C.c_void_p, P_f64]
    L.esm_batch_launch_count.restype = C.c_int64
    L.esm_batch_launch_count.argtypes = [C.c_void_p]
    _lib = L
    return L


def _p(a, t=P_f64):
    return None if a is None else a.ctypes.data_as(t)


class DeviceChain:
    """One chain of R replicas on the GPU (an ``esm_ctx``)."""

    def __init__(self, model: SynthModel, R: int, precision: int = 32, seed: int = 1, extra: float = 4.0,
                 maxnats: float = 40.0, kappa_min: float = 1.0, max_points: int = 0, span: int = 0,
                 storage_ms: int = 0, storage_long: int = 0, probe: int = 0, rates=None):
        self.L = load()
        self.m = model
        self.R = R
        self.buf = ModelBuffers(model)
        kw = {} if rates is None else {"rates": rates}
        self.opts: EsmOpts = make_opts(R, precision, seed, extra, maxnats, kappa_min, max_points, span,
                                       storage_ms=storage_ms, storage_long=storage_long, probe=probe, **kw)
        h = C.c_void_p()
        rc = self.L.esm_create(C.byref(self.buf.struct), C.byref(self.opts), C.byref(h))
        self.h = h
        self._check(rc, "esm_create")

    def _check(self, rc, what):
        if rc != 0:
            msg = self.L.esm_last_error(self.h).decode() if self.h else ""
            raise EsmError(f"{what}: status {rc}: {msg}")

    def close(self):
        if getattr(self, "h", None):
            self.L.esm_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def shapes(self):
        m, R = self.m, self.R
        return {"theta": (m.N, m.T, R), "g": (m.D, m.T, R), "e": (m.S, m.T, R), "z": (m.n0, m.T, R),
                "reg": (m.T, R), "k": (m.Kunits,)}

    def upload(self, st):
        arr = {k: np.ascontiguousarray(getattr(st, k) if not isinstance(st, dict) else st[k],
                                       dtype=np.int32 if k == "reg" else np.float64)
               for k in ("theta", "g", "e", "z", "reg", "k")}
        self._check(self.L.esm_upload_state(self.h, _p(arr["theta"]), _p(arr["g"]), _p(arr["e"]), _p(arr["z"]),
                                            _p(arr["reg"], P_i32), _p(arr["k"])), "esm_upload_state")

    def download(self):
        out = {k: np.zeros(s, dtype=np.int32 if k == "reg" else np.float64) for k, s in self.shapes().items()}
        self._check(self.L.esm_download_state(self.h, _p(out["theta"]), _p(out["g"]), _p(out["e"]), _p(out["z"]),
                                              _p(out["reg"], P_i32), _p(out["k"])), "esm_download_state")
        return out

    def download_k(self):
        k = np.zeros(self.m.Kunits)
        self._check(self.L.esm_download_state(self.h, None, None, None, None, None, _p(k)), "esm_download_state")
        return k

    def rebuild(self):
        self._check(self.L.esm_rebuild_caches(self.h), "esm_rebuild_caches")

    def caches(self):
        m, R = self.m, self.R
        r = np.zeros((m.N, m.T, R))
        F = np.zeros((m.L, m.T, R))
        self._check(self.L.esm_download_caches(self.h, _p(r), _p(F)), "esm_download_caches")
        return r, F

    def class_pass(self, sweep, cls, limit=0):
        st = np.zeros(NSTAT, np.int64)
        self._check(self.L.esm_class_pass(self.h, sweep, cls, limit, _p(st, P_i64)), "esm_class_pass")
        return st

    def sweeps(self, n, sweep0=0, stats=True):
        st = np.zeros(NSTAT, np.int64)
        self._check(self.L.esm_operation_sweeps(self.h, n, sweep0, _p(st, P_i64) if stats else None),
                    "esm_operation_sweeps")
        return st

    def storage_ms(self, sweep, force=True, max_passes=0):
        """The storage multiscale sweep of `sweep` (plateau moves; max_passes > 0: its first class
        passes only); returns (tried, taken, guards)."""
        st = np.zeros(3, np.int64)
        self._check(self.L.esm_storage_ms(self.h, sweep, int(force), int(max_passes), _p(st, P_i64)),
                    "esm_storage_ms")
        return st

    def storage_long(self, sweep):
        """The long-range storage sweep of `sweep`; returns (tried, taken, guards)."""
        st = np.zeros(3, np.int64)
        self._check(self.L.esm_storage_long(self.h, sweep, _p(st, P_i64)), "esm_storage_long")
        return st

    def lag_probe(self, j, nsweeps=30, tail=10, sweep0=0):
        """esm_lag_probe: (mean capacity score of the last `tail` of `nsweeps` operation sweeps of a
        frozen copy of replica j, the last prior term fk); the chain is unchanged."""
        sk = np.zeros(self.m.Kunits)
        fk = np.zeros(self.m.Kunits)
        self._check(self.L.esm_lag_probe(self.h, j, nsweeps, tail, sweep0, _p(sk), _p(fk)), "esm_lag_probe")
        return sk, fk

    def scores(self):
        m, R = self.m, self.R
        sk = np.zeros((R, m.Kunits))
        fk = np.zeros(m.Kunits)
        parts = np.zeros((R, 8))
        self._check(self.L.esm_capacity_scores(self.h, _p(sk), _p(fk), _p(parts)), "esm_capacity_scores")
        return sk, fk, parts

    def scores_static(self):
        """esm_capacity_scores_static: the same scores, accumulated in the library's file-scope
        device scratch (nothing is allocated in the call; overlapping calls race)."""
        m, R = self.m, self.R
        sk = np.zeros((R, m.Kunits))
        fk = np.zeros(m.Kunits)
        parts = np.zeros((R, 8))
        self._check(self.L.esm_capacity_scores_static(self.h, _p(sk), _p(fk), _p(parts)),
                    "esm_capacity_scores_static")
        return sk, fk, parts

    def score_errors(self):
        """esm_score_errors: bounds on the distance of the last scores [R, K] and cost parts [R, 8] from
        the exact sums over the same state."""
        m, R = self.m, self.R
        ek = np.zeros((R, m.Kunits))
        ep = np.zeros((R, 8))
        self._check(self.L.esm_score_errors(self.h, _p(ek), _p(ep)), "esm_score_errors")
        return ek, ep

    def follow_capacities(self, knew, kmin=1.0):
        """esm_follow_capacities: every replica follows the capacities to knew; returns the new k."""
        knew = np.ascontiguousarray(knew, dtype=np.float64)
        out = np.zeros(self.m.Kunits)
        self._check(self.L.esm_follow_capacities(self.h, _p(knew), kmin, _p(out)), "esm_follow_capacities")
        return out

    def state_save(self):
        self._check(self.L.esm_state_save(self.h), "esm_state_save")

    def state_restore(self):
        self._check(self.L.esm_state_restore(self.h), "esm_state_restore")

    def regime_occupancy(self):
        occ = np.zeros(self.m.K * 4)
        self._check(self.L.esm_regime_occupancy(self.h, _p(occ)), "esm_regime_occupancy")
        return occ

    def langevin_step(self, w, eta, kappa_s, kmin=1.0, clip=0.02, box=True, xi=None, it=0):
        w, eta, kappa_s = (np.ascontiguousarray(x, dtype=np.float64) for x in (w, eta, kappa_s))
        xi = None if xi is None else np.ascontiguousarray(xi, dtype=np.float64)
        knew = np.zeros(self.m.Kunits)
        nclip = np.zeros(1, np.int32)
        self._check(self.L.esm_langevin_step(self.h, _p(w), _p(eta), _p(kappa_s), kmin, clip, int(box), _p(xi), it,
                                             _p(knew), _p(nclip, P_i32)), "esm_langevin_step")
        return knew, int(nclip[0])

    def weather_step(self, moved, theta, window, wstart, xi=None, it=0):
        """Weather process of the flagged replicas and the compensated re-initialisation of their
        dispatch (replica_weather!, src/replicas.jl:586); wstart is the 1-based window start."""
        moved = np.ascontiguousarray(moved, dtype=np.int32)
        theta = np.ascontiguousarray(theta, dtype=np.float64)
        window = np.ascontiguousarray(window, dtype=np.int32)
        wstart = np.ascontiguousarray(wstart, dtype=np.int32)
        xi = None if xi is None else np.ascontiguousarray(xi, dtype=np.float64)
        self._check(self.L.esm_weather_step(self.h, _p(moved, P_i32), _p(theta), _p(window, P_i32),
                                            _p(wstart, P_i32), _p(xi), it), "esm_weather_step")

    def set_move_grid(self, warps_per_block=1, warps_per_sm=0):
        """Line-move grid: blocks of 1, 2 or 4 warps, resident warps per SM (0: that shape's limit)."""
        self._check(self.L.esm_set_move_grid(self.h, int(warps_per_block), int(warps_per_sm)), "esm_set_move_grid")

    def replica_features(self, kref):
        """esm_replica_features: the weather features of every replica [R, nfeat] at the reference
        capacities kref [K] (columns: replicas.replica_feature_names)."""
        nf = np.zeros(1, np.int32)
        self._check(self.L.esm_replica_features(self.h, None, None, _p(nf, P_i32)), "esm_replica_features")
        out = np.zeros((self.R, int(nf[0])))
        kr = np.ascontiguousarray(kref, dtype=np.float64)
        self._check(self.L.esm_replica_features(self.h, _p(kr), _p(out), _p(nf, P_i32)), "esm_replica_features")
        return out

    def set_move_schedule(self, schedule):
        """How a class pass launches its line moves: "move" (one launch per move) or "class" (the
        whole pass in one launch, an item's next move as soon as its previous one is done)."""
        code = {"move": 0, "class": 1}[schedule]
        self._check(self.L.esm_set_move_schedule(self.h, code), "esm_set_move_schedule")

    def move_schedule(self):
        v = np.zeros(1, np.int32)
        self._check(self.L.esm_move_schedule(self.h, _p(v, P_i32)), "esm_move_schedule")
        return ("move", "class")[int(v[0])]

    def set_move_log(self, nreps):
        """Record the t of every line move of each class pass for replicas below nreps (0: off)."""
        self._check(self.L.esm_set_move_log(self.h, int(nreps)), "esm_set_move_log")
        self._mlog_nrep = int(nreps)

    def move_log(self, cls, nmoves, nsteps):
        """The move log of the last class pass (class cls): [move, class step, replica], NaN where the
        selection made no move."""
        out = np.zeros(nmoves * nsteps * self._mlog_nrep)
        self._check(self.L.esm_move_log(self.h, int(cls), _p(out)), "esm_move_log")
        return out.reshape(nmoves, nsteps, self._mlog_nrep)

    def storage_long_log(self, nunits):
        """The move log of the last long-range storage sweep: [unit, move (5), replica], NaN where no
        move was made."""
        out = np.zeros(nunits * 5 * self._mlog_nrep)
        self._check(self.L.esm_move_log(self.h, -1, _p(out)), "esm_move_log")
        return out.reshape(nunits, 5, self._mlog_nrep)

    def set_sep_walk(self, min_units):
        """The cooperative walk for separable moves of at least min_units units (0: off)."""
        self._check(self.L.esm_set_sep_walk(self.h, int(min_units)), "esm_set_sep_walk")

    def sep_walk(self):
        """(min_units, warps of the cooperative walk kernel)."""
        a, b = np.zeros(1, np.int32), np.zeros(1, np.int32)
        self._check(self.L.esm_sep_walk(self.h, _p(a, P_i32), _p(b, P_i32)), "esm_sep_walk")
        return int(a[0]), int(b[0])

    def move_grid(self):
        """(warps per block, warps per SM, limits per SM of the 1-, 2- and 4-warp shapes)."""
        b, w, lim = np.zeros(1, np.int32), np.zeros(1, np.int32), np.zeros(3, np.int32)
        self._check(self.L.esm_move_grid(self.h, _p(b, P_i32), _p(w, P_i32), _p(lim, P_i32)), "esm_move_grid")
        return int(b[0]), int(w[0]), tuple(int(x) for x in lim)

    def autotune_moves(self, sweep=0):
        """Pick the line-move grid by timing one colour class per candidate (the state is restored
        after each); returns ((warps per block, warps per SM), {(wpb, wps): ms})."""
        best = np.zeros(2, np.int32)
        cand = np.zeros(2 * TUNE_MAX, np.int32)
        ms = np.zeros(TUNE_MAX)
        n = np.zeros(1, np.int32)
        self._check(self.L.esm_autotune_moves(self.h, sweep, _p(best, P_i32), _p(cand, P_i32), _p(ms), _p(n, P_i32)),
                    "esm_autotune_moves")
        return (int(best[0]), int(best[1])), {(int(cand[2 * i]), int(cand[2 * i + 1])): float(ms[i])
                                              for i in range(int(n[0]))}

    def sync(self, timeout_s=60.0):
        self._check(self.L.esm_sync(self.h, timeout_s), "esm_sync")

    def set_timing(self, on=True):
        self._check(self.L.esm_set_timing(self.h, int(on)), "esm_set_timing")

    def timing(self):
        """Per kernel family: (milliseconds, launches) since the last call (CUDA events on the stream)."""
        out = np.zeros(2 * len(KERNEL_FAMILIES))
        self._check(self.L.esm_timing(self.h, _p(out)), "esm_timing")
        return {k: (out[2 * i], int(out[2 * i + 1])) for i, k in enumerate(KERNEL_FAMILIES)}

    def stream(self):
        return self.L.esm_stream(self.h)

    def launch_count(self):
        return int(self.L.esm_launch_count(self.h))


class DeviceBatch:
    """Chains of any sizes whose operation sweeps run together (an ``esm_batch`` over the chains'
    contexts): one captured graph per sweep, one line-move launch per move index over the tasks of
    every chain. The chains stay usable on their own; they must outlive the batch."""

    def __init__(self, chains):
        self.L = load()
        self.chains = list(chains)
        arr = (C.c_void_p * len(self.chains))(*[c.h for c in self.chains])
        h = C.c_void_p()
        rc = self.L.esm_batch_create(arr, len(self.chains), C.byref(h))
        self.h = h
        self._check(rc, "esm_batch_create")

    def _check(self, rc, what):
        if rc != 0:
            msg = self.L.esm_batch_last_error(self.h).decode() if self.h else ""
            raise EsmError(f"{what}: status {rc}: {msg}")

    def close(self):
        if getattr(self, "h", None):
            self.L.esm_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def sweeps(self, n, sweep0=0, stats=True):
        """n operation sweeps of every chain; the move counts per chain [chains, NSTAT] (or None)."""
        st = np.zeros((len(self.chains), NSTAT), np.int64) if stats else None
        self._check(self.L.esm_batch_sweeps(self.h, n, sweep0, _p(st, P_i64)), "esm_batch_sweeps")
        return st

    def set_grid(self, warps_per_block=1, warps_per_sm=0):
        self._check(self.L.esm_batch_set_grid(self.h, int(warps_per_block), int(warps_per_sm)), "esm_batch_set_grid")

    def grid(self):
        """(warps per block, warps per SM, the resident limit per SM of that block shape)."""
        b, w, lim = np.zeros(1, np.int32), np.zeros(1, np.int32), np.zeros(1, np.int32)
        self._check(self.L.esm_batch_grid(self.h, _p(b, P_i32), _p(w, P_i32), _p(lim, P_i32)), "esm_batch_grid")
        return int(b[0]), int(w[0]), int(lim[0])

    def autotune(self, sweep=0):
        """Pick the grid by timing one sweep of every chain per candidate (the states are restored
        after each); returns ((warps per block, warps per SM), {(wpb, wps): ms})."""
        best = np.zeros(2, np.int32)
        cand = np.zeros(2 * TUNE_MAX, np.int32)
        ms = np.zeros(TUNE_MAX)
        n = np.zeros(1, np.int32)
        self._check(self.L.esm_batch_autotune(self.h, sweep, _p(best, P_i32), _p(cand, P_i32), _p(ms), _p(n, P_i32)),
                    "esm_batch_autotune")
        return (int(best[0]), int(best[1])), {(int(cand[2 * i]), int(cand[2 * i + 1])): float(ms[i])
                                              for i in range(int(n[0]))}

    def last_ms(self):
        """Device time (CUDA events) of the last sweeps call, ms."""
        t = np.zeros(1)
        self._check(self.L.esm_batch_time(self.h, _p(t)), "esm_batch_time")
        return float(t[0])

    def launch_count(self):
        return int(self.L.esm_batch_launch_count(self.h))
