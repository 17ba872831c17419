"""ctypes wrapper of the CPU oracle (``oracle/_build/liboracle_esm.so``) -- TEST INFRASTRUCTURE.

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` use it, as the
checker of the CUDA path; the product never imports it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "liboracle_esm.so")

P_f64 = C.POINTER(C.c_double)
P_i32 = C.POINTER(C.c_int32)
P_i64 = C.POINTER(C.c_int64)
NSTAT = 2 * (11 + 1) + 1  # ESM_NFAM = 11


def build():
    """Compile the oracle with its Makefile (gcc, no other dependency)."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        L = C.CDLL(LIB)
        L.orc_logseg.restype = C.c_double
        L.orc_logseg.argtypes = [C.c_double, C.c_double]
        L.orc_trexp_offset.restype = C.c_double
        L.orc_trexp_offset.argtypes = [C.c_double, C.c_double, C.c_double]
        L.orc_philox4.argtypes = [C.c_uint32] * 6 + [C.POINTER(C.c_uint32)]
        L.orc_normal_at.restype = C.c_double
        L.orc_normal_at.argtypes = [C.c_uint64, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32]
        L.orc_langevin_update.restype = C.c_int
        L.orc_langevin_update.argtypes = [C.c_int, P_f64, P_f64, P_f64, C.c_double, C.c_double, C.c_double,
                                          C.c_double, P_f64, P_f64]
        L.orc_create.restype = C.c_void_p
        L.orc_create.argtypes = [C.c_void_p, C.c_void_p]
        L.orc_destroy.argtypes = [C.c_void_p]
        L.orc_set_state.argtypes = [C.c_void_p, P_f64, P_f64, P_f64, P_f64, P_i32, P_f64]
        L.orc_get_state.argtypes = [C.c_void_p, P_f64, P_f64, P_f64, P_f64, P_i32, P_f64]
        L.orc_rebuild.argtypes = [C.c_void_p, C.c_int]
        L.orc_move_walk.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int64, P_f64, P_f64, C.c_int]
        L.orc_block_at.argtypes = [C.c_void_p, P_i32, C.c_int, C.c_int, C.c_int, C.c_int, C.c_double, C.c_int, P_f64,
                                   P_f64, P_f64, P_f64, P_f64, C.c_int]
        L.orc_move_at.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int64, C.c_double, C.c_int,
                                  P_f64, P_f64, P_f64]
        L.orc_get_caches.argtypes = [C.c_void_p, P_f64, P_f64]
        L.orc_set_caches.argtypes = [C.c_void_p, P_f64, P_f64]
        L.orc_class_pass.argtypes = [C.c_void_p, C.c_int64, C.c_int, C.c_int, P_i64, C.c_int]
        L.orc_storage_ms.argtypes = [C.c_void_p, C.c_int64, C.c_int, C.c_int, P_i64, C.c_int]
        L.orc_storage_ms_plan.argtypes = [C.c_void_p, C.c_int64, C.c_int, P_i32]
        L.orc_storage_ms_plan.restype = C.c_int
        L.orc_storage_long.argtypes = [C.c_void_p, C.c_int64, P_i64, C.c_int]
        L.orc_storage_long_plan.argtypes = [C.c_void_p, C.c_int64, P_i32, C.c_int]
        L.orc_storage_long_plan.restype = C.c_int
        L.orc_sweeps.argtypes = [C.c_void_p, C.c_int, C.c_int64, P_i64, C.c_int]
        L.orc_class_pass_range.argtypes = [C.c_void_p, C.c_int64, C.c_int, C.c_int, C.c_int, P_i64, C.c_int, P_f64]
        L.orc_storage_long_log.argtypes = [C.c_void_p, C.c_int64, P_i64, C.c_int, P_f64]
        L.orc_sl_task.restype = C.c_int
        L.orc_sl_task.argtypes = [C.c_void_p, C.c_int64, C.c_int, C.c_int, C.c_int, C.c_int]
        L.orc_sl_explain.restype = C.c_int
        L.orc_sl_explain.argtypes = [C.c_void_p, C.c_int64, C.c_int, C.c_int, C.c_int, C.c_double, P_f64]
        L.orc_task_moves.restype = C.c_int
        L.orc_task_moves.argtypes = [C.c_void_p, C.c_int64, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int]
        L.orc_explain.restype = C.c_int
        L.orc_explain.argtypes = [C.c_void_p, C.c_int64, C.c_int, C.c_int, C.c_int, C.c_int, C.c_double, P_f64]
        L.orc_atom_walk.restype = C.c_int
        L.orc_atom_walk.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, P_f64, P_f64, C.c_int, P_i32]
        L.orc_class_order.argtypes = [C.c_void_p, C.c_int64, P_i32, P_i32]
        L.orc_scores.argtypes = [C.c_void_p, P_f64, P_f64, P_f64, C.c_int]
        L.orc_langevin_step.restype = C.c_int
        L.orc_langevin_step.argtypes = [C.c_void_p, P_f64, P_f64, P_f64, C.c_double, C.c_double, C.c_int, P_f64,
                                        C.c_int64, P_f64, P_i32, C.c_int]
        L.orc_move_list.restype = C.c_int
        L.orc_move_list.argtypes = [C.c_void_p, C.c_int64, C.c_int, C.c_int, P_i32, P_i32, P_i32, C.c_int]
        L.orc_weather_step.argtypes = [C.c_void_p, P_i32, P_f64, P_i32, P_i32, P_f64, C.c_int64, C.c_int]
        _lib = L
    return _lib


def _p(a, t=P_f64):
    return None if a is None else a.ctypes.data_as(t)


def logseg(L, x):
    return lib().orc_logseg(L, x)


def trexp_offset(u, g, L):
    return lib().orc_trexp_offset(u, g, L)


def philox4(k0, k1, c0, c1, c2, c3):
    out = (C.c_uint32 * 4)()
    lib().orc_philox4(k0, k1, c0, c1, c2, c3, out)
    return list(out)


def langevin_update(k, g, xi, eta, ks, kmin=1.0, clip=np.inf, hi=None):
    k, g, xi = (np.ascontiguousarray(x, dtype=np.float64) for x in (k, g, xi))
    out = np.zeros_like(k)
    hi = None if hi is None else np.ascontiguousarray(hi, dtype=np.float64)
    nc = lib().orc_langevin_update(len(k), _p(k), _p(g), _p(xi), eta, ks, kmin, clip, _p(hi), _p(out))
    return out, nc


class Oracle:
    """FP64 CPU restatement of the replica hot path for one chain of R replicas."""

    def __init__(self, model, R, seed=1, extra=4.0, maxnats=40.0, kappa_min=1.0, max_points=0, span=0,
                 threads=None, storage_ms=0, storage_long=0, rates=None):
        import sys
        sys.path.insert(0, os.path.join(os.path.dirname(HERE), "esm-sampling_gb300"))
        from esmgb.cabi import ModelBuffers, make_opts
        self.m = model
        self.R = R
        self.buf = ModelBuffers(model)
        kw = {} if rates is None else {"rates": rates}
        self.opts = make_opts(R, 64, seed, extra, maxnats, kappa_min, max_points, span, storage_ms=storage_ms,
                              storage_long=storage_long, **kw)
        self.threads = threads or os.cpu_count() or 1
        self.h = lib().orc_create(C.byref(self.buf.struct), C.byref(self.opts))

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_destroy(self.h)
            self.h = None

    def shapes(self):
        m, R = self.m, self.R
        return {"theta": (m.N, m.T, R), "g": (m.D, m.T, R), "e": (m.S, m.T, R), "z": (m.n0, m.T, R),
                "reg": (m.T, R), "k": (m.Kunits,)}

    def set_state(self, st):
        get = (lambda k: st[k]) if isinstance(st, dict) else (lambda k: getattr(st, k))
        arr = {k: np.ascontiguousarray(get(k), dtype=np.int32 if k == "reg" else np.float64)
               for k in ("theta", "g", "e", "z", "reg", "k")}
        self._in = arr
        lib().orc_set_state(self.h, _p(arr["theta"]), _p(arr["g"]), _p(arr["e"]), _p(arr["z"]),
                            _p(arr["reg"], P_i32), _p(arr["k"]))

    def get_state(self):
        sh = self.shapes()
        out = {k: np.zeros(s, dtype=np.int32 if k == "reg" else np.float64) for k, s in sh.items()}
        lib().orc_get_state(self.h, _p(out["theta"]), _p(out["g"]), _p(out["e"]), _p(out["z"]),
                            _p(out["reg"], P_i32), _p(out["k"]))
        return out

    def rebuild(self):
        lib().orc_rebuild(self.h, self.threads)

    def caches(self):
        m, R = self.m, self.R
        r = np.zeros((m.N, m.T, R))
        F = np.zeros((m.L, m.T, R))
        lib().orc_get_caches(self.h, _p(r), _p(F))
        return r, F

    def set_caches(self, r, F):
        r = np.ascontiguousarray(r, dtype=np.float64)
        F = np.ascontiguousarray(F, dtype=np.float64)
        lib().orc_set_caches(self.h, _p(r), _p(F))

    def class_pass(self, sweep, cls, limit=0):
        st = np.zeros(NSTAT, np.int64)
        lib().orc_class_pass(self.h, sweep, cls, limit, _p(st, P_i64), self.threads)
        return st

    def class_pass_range(self, sweep, cls, m0, m1, tlog=None):
        """Moves [m0, m1) of every task of a class pass (m1 < 0: to the end); tlog (float64 array
        [moves, class steps, R], may be None) receives the t of every move of the range."""
        st = np.zeros(NSTAT, np.int64)
        lib().orc_class_pass_range(self.h, sweep, cls, m0, m1, _p(st, P_i64), self.threads,
                                   None if tlog is None else tlog.ctypes.data_as(P_f64))
        return st

    def task_moves(self, sweep, cls, q, rep, m0, m1):
        """Moves [m0, m1) (m1 < 0: to the end) of the one task at the class's q-th step of replica rep."""
        n = lib().orc_task_moves(self.h, sweep, cls, q, rep, m0, m1)
        if n < 0:
            raise ValueError("orc_task_moves: bad index")
        return n

    EXPLAIN = ("t", "t_jac", "nseg", "seg", "seg_other", "cat_margin", "seg_margin", "lj", "uj", "lj_other",
               "stop_r", "stop_l", "near_r", "near_l", "npts_r", "npts_l", "fam", "entries", "walk", "tot",
               "ray_r", "ray_l", "gL", "L")

    def explain(self, sweep, cls, mi, q, rep, t_other):
        """Diagnosis of move mi at the class's q-th step of replica rep on the current state (see
        orc_explain): a dict of EXPLAIN, or None when the selection made no move."""
        out = np.zeros(24)
        rc = lib().orc_explain(self.h, sweep, cls, mi, q, rep, float(t_other), _p(out))
        if rc < 0:
            raise ValueError("orc_explain: bad index")
        return dict(zip(self.EXPLAIN, out.tolist())) if rc else None

    def atom_walk(self, atom, tau, rep, maxn=8192):
        """The walk of an atom move on the current state: (points, potentials, [right points, left
        points, primary breakpoints, ray steps]), or None."""
        pts, cs, info = np.zeros(maxn), np.zeros(maxn), np.zeros(4, np.int32)
        n = lib().orc_atom_walk(self.h, atom, tau, rep, _p(pts), _p(cs), maxn, _p(info, P_i32))
        if n <= 0:
            return None
        return pts[:n].copy(), cs[:n].copy(), info.tolist()

    def sweeps(self, n, sweep0=0):
        st = np.zeros(NSTAT, np.int64)
        lib().orc_sweeps(self.h, n, sweep0, _p(st, P_i64), self.threads)
        return st

    def storage_ms(self, sweep, force=True, max_passes=0):
        """The storage multiscale sweep of `sweep` (src/flowmoves.jl:255, plateau moves; max_passes
        > 0: its first class passes only); returns (moves tried, moves taken, guard events)."""
        st = np.zeros(3, np.int64)
        lib().orc_storage_ms(self.h, sweep, int(force), int(max_passes), _p(st, P_i64), self.threads)
        return st

    def storage_long(self, sweep):
        """The long-range storage sweep of `sweep` (src/storage_long.jl:245); returns (moves tried,
        moves taken, guard events)."""
        st = np.zeros(3, np.int64)
        lib().orc_storage_long(self.h, sweep, _p(st, P_i64), self.threads)
        return st

    def storage_long_log(self, sweep, tlog):
        """The long-range storage sweep with the t of every move logged into tlog (float64 [units,
        5, R], the sweep's eligible units in plan order); returns (tried, taken, guards)."""
        st = np.zeros(3, np.int64)
        lib().orc_storage_long_log(self.h, sweep, _p(st, P_i64), self.threads, tlog.ctypes.data_as(P_f64))
        return st

    def sl_task(self, sweep, ui, rep, m0, m1):
        """Moves [m0, m1) (m1 < 0: to the end) of the long-range task of eligible unit ui, replica rep."""
        n = lib().orc_sl_task(self.h, sweep, ui, rep, m0, m1)
        if n < 0:
            raise ValueError("orc_sl_task: bad index")
        return n

    def sl_explain(self, sweep, ui, rep, mi, t_other):
        """Oracle.explain for move mi of the long-range task of eligible unit ui, replica rep."""
        out = np.zeros(24)
        rc = lib().orc_sl_explain(self.h, sweep, ui, rep, mi, float(t_other), _p(out))
        if rc < 0:
            raise ValueError("orc_sl_explain: bad index")
        return dict(zip(self.EXPLAIN, out.tolist())) if rc else None

    def storage_long_plan(self, sweep, maxn=4096):
        """Its moves: [(unit, length, start)] (length T: the level move)."""
        out = np.zeros(3 * maxn, np.int32)
        n = lib().orc_storage_long_plan(self.h, sweep, _p(out, P_i32), maxn)
        return [tuple(int(x) for x in out[3 * i:3 * i + 3]) for i in range(n)]

    def storage_ms_plan(self, sweep, force=True):
        """Its class passes: [(length, offset, block parity)]."""
        out = np.zeros(3 * 14, np.int32)
        n = lib().orc_storage_ms_plan(self.h, sweep, int(force), _p(out, P_i32))
        return [tuple(int(x) for x in out[3 * i:3 * i + 3]) for i in range(n)]

    def move_list(self, sweep, cls, tile, maxn=4096):
        k, f, a = (np.zeros(maxn, np.int32) for _ in range(3))
        n = lib().orc_move_list(self.h, sweep, cls, tile, _p(k, P_i32), _p(f, P_i32), _p(a, P_i32), maxn)
        return k[:n], f[:n], a[:n]

    def move_at(self, fam, tau, rep, cls, sweep, t, commit=True, with_cost=False):
        """One move of family `fam` at step tau of replica rep (selection from the stream (cls,
        sweep)), moved by t when `commit`: (made, log-Jacobian at t, (Q, g) of its first kink)
        and, with `with_cost`, the cost change the move evaluates at t."""
        lj = np.zeros(1)
        kq = np.zeros(2)
        dc = np.zeros(1)
        ok = lib().orc_move_at(self.h, fam, tau, rep, cls, sweep, t, int(commit), _p(lj), _p(kq), _p(dc))
        out = (bool(ok), float(lj[0]), (float(kq[0]), float(kq[1])))
        return out + (float(dc[0]),) if with_cost else out

    def move_walk(self, fam, tau, rep, cls, sweep, maxn=8192):
        """The walk of that move: (points, potentials beta DeltaC), ascending, with t = 0; None if
        the selection made no move or the walk reached the point cap."""
        pts = np.zeros(maxn)
        cs = np.zeros(maxn)
        n = lib().orc_move_walk(self.h, fam, tau, rep, cls, sweep, _p(pts), _p(cs), maxn)
        if n <= 0:
            return None
        n = min(n, maxn)
        return pts[:n].copy(), cs[:n].copy()

    def block_at(self, units, b0, L, rep, t, commit=True):
        """One storage block move of replica rep (the plateau of `units` over the instants b0+1 ..
        b0+L, cyclic; L = T: the level move of one unit), moved by t when `commit`: (made,
        log-Jacobian at t, (Q, g) of its first kink, the cost change it evaluates at t)."""
        us = np.ascontiguousarray(units, dtype=np.int32)
        lj, kq, dc = np.zeros(1), np.zeros(2), np.zeros(1)
        ok = lib().orc_block_at(self.h, _p(us, P_i32), len(us), b0, L, rep, t, int(commit), _p(lj), _p(kq), _p(dc),
                                None, None, 0)
        return bool(ok), float(lj[0]), (float(kq[0]), float(kq[1])), float(dc[0])

    def block_walk(self, units, b0, L, rep, maxn=8192):
        """The walk of that block move: (points, potentials beta DeltaC), ascending, with t = 0;
        None if there is no move or the walk reached the point cap."""
        us = np.ascontiguousarray(units, dtype=np.int32)
        lj, kq, dc = np.zeros(1), np.zeros(2), np.zeros(1)
        pts, cs = np.zeros(maxn), np.zeros(maxn)
        n = lib().orc_block_at(self.h, _p(us, P_i32), len(us), b0, L, rep, 0.0, 0, _p(lj), _p(kq), _p(dc), _p(pts),
                               _p(cs), maxn)
        if n <= 0:
            return None
        n = min(n, maxn)
        return pts[:n].copy(), cs[:n].copy()

    def class_order(self, sweep):
        o = np.zeros(3, np.int32)
        n = np.zeros(1, np.int32)
        lib().orc_class_order(self.h, sweep, _p(o, P_i32), _p(n, P_i32))
        return list(o[: n[0]])

    def scores(self):
        m, R = self.m, self.R
        sk = np.zeros((R, m.Kunits))
        fk = np.zeros(m.Kunits)
        parts = np.zeros((R, 8))
        lib().orc_scores(self.h, _p(sk), _p(fk), _p(parts), self.threads)
        return sk, fk, parts

    def langevin_step(self, w, eta, kappa_s, kmin=1.0, clip=0.02, box=True, xi=None, it=0):
        w, eta, kappa_s = (np.ascontiguousarray(x, dtype=np.float64) for x in (w, eta, kappa_s))
        xi = None if xi is None else np.ascontiguousarray(xi, dtype=np.float64)
        knew = np.zeros(self.m.Kunits)
        nclip = np.zeros(1, np.int32)
        rc = lib().orc_langevin_step(self.h, _p(w), _p(eta), _p(kappa_s), kmin, clip, int(box), _p(xi), it,
                                     _p(knew), _p(nclip, P_i32), self.threads)
        if rc != 0:
            raise RuntimeError(f"oracle langevin_step: status {rc}")
        return knew, int(nclip[0])

    def weather_step(self, moved, theta, window, wstart, xi=None, it=0):
        moved = np.ascontiguousarray(moved, dtype=np.int32)
        theta = np.ascontiguousarray(theta, dtype=np.float64)
        window = np.ascontiguousarray(window, dtype=np.int32)
        wstart = np.ascontiguousarray(wstart, dtype=np.int32)
        xi = None if xi is None else np.ascontiguousarray(xi, dtype=np.float64)
        lib().orc_weather_step(self.h, _p(moved, P_i32), _p(theta), _p(window, P_i32), _p(wstart, P_i32), _p(xi),
                               it, self.threads)
