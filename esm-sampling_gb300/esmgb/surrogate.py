"""Surrogate of the replica-averaged capacity score and the delayed-acceptance Langevin step.

The surrogate (``libesmcuda.so`` esm_mlp_*: BF16 tensor-core forward/backward, FP32 accumulation,
Adam) is trained online on the pairs (features(k, regimes), replica-averaged score) that the plain
sampler produces every step. It is not in the reference; the reference's plain replica step
(src/replicas.jl:676) stays the second stage and the fallback.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from .device import EsmError, load

EXPORTS = ("esm_mlp_create", "esm_mlp_destroy", "esm_mlp_last_error", "esm_mlp_set_layer", "esm_mlp_get_layer",
           "esm_mlp_forward", "esm_mlp_train_step", "esm_mlp_launch_count")

P_f32 = C.POINTER(C.c_float)
P_f64 = C.POINTER(C.c_double)
P_i32 = C.POINTER(C.c_int32)


def _lib():
    L = load()
    if not getattr(L, "_mlp_bound", False):
        L.esm_mlp_create.argtypes = [C.c_int32, P_i32, C.c_int32, C.c_uint64, C.POINTER(C.c_void_p)]
        L.esm_mlp_destroy.argtypes = [C.c_void_p]
        L.esm_mlp_last_error.restype = C.c_char_p
        L.esm_mlp_last_error.argtypes = [C.c_void_p]
        L.esm_mlp_set_layer.argtypes = [C.c_void_p, C.c_int32, P_f32, P_f32]
        L.esm_mlp_get_layer.argtypes = [C.c_void_p, C.c_int32, P_f32, P_f32]
        L.esm_mlp_forward.argtypes = [C.c_void_p, C.c_int32, P_f32, P_f32]
        L.esm_mlp_train_step.argtypes = [C.c_void_p, C.c_int32, P_f32, P_f32, C.c_float, P_f64, P_f32]
        L.esm_mlp_launch_count.restype = C.c_int64
        L.esm_mlp_launch_count.argtypes = [C.c_void_p]
        L._mlp_bound = True
    return L


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


class MLP:
    """dims[0] -> ... -> dims[-1], SiLU hidden layers, on the GPU."""

    def __init__(self, dims, batch_max=1024, seed=1):
        self.L = _lib()
        self.dims = [int(d) for d in dims]
        d = np.array(self.dims, np.int32)
        h = C.c_void_p()
        rc = self.L.esm_mlp_create(len(dims) - 1, d.ctypes.data_as(P_i32), batch_max, seed, C.byref(h))
        self.h = h
        self._check(rc, "esm_mlp_create")

    def _check(self, rc, what):
        if rc != 0:
            msg = self.L.esm_mlp_last_error(self.h).decode() if self.h else ""
            raise EsmError(f"{what}: status {rc}: {msg}")

    def close(self):
        if getattr(self, "h", None):
            self.L.esm_mlp_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def nlayers(self):
        return len(self.dims) - 1

    def set_layer(self, l, W=None, b=None):
        W = None if W is None else _f32(W)
        b = None if b is None else _f32(b)
        self._check(self.L.esm_mlp_set_layer(self.h, l, None if W is None else W.ctypes.data_as(P_f32),
                                             None if b is None else b.ctypes.data_as(P_f32)), "set_layer")

    def get_layer(self, l):
        W = np.zeros((self.dims[l + 1], self.dims[l]), np.float32)
        b = np.zeros(self.dims[l + 1], np.float32)
        self._check(self.L.esm_mlp_get_layer(self.h, l, W.ctypes.data_as(P_f32), b.ctypes.data_as(P_f32)),
                    "get_layer")
        return W, b

    def forward(self, x):
        x = _f32(x)
        y = np.zeros((x.shape[0], self.dims[-1]), np.float32)
        self._check(self.L.esm_mlp_forward(self.h, x.shape[0], x.ctypes.data_as(P_f32), y.ctypes.data_as(P_f32)),
                    "forward")
        return y

    def train_step(self, x, t, lr=1e-3, grads=False):
        x, t = _f32(x), _f32(t)
        loss = np.zeros(1)
        n = sum(self.dims[l] * self.dims[l + 1] + self.dims[l + 1] for l in range(self.nlayers))
        g = np.zeros(n, np.float32) if grads else None
        self._check(self.L.esm_mlp_train_step(self.h, x.shape[0], x.ctypes.data_as(P_f32), t.ctypes.data_as(P_f32),
                                              lr, loss.ctypes.data_as(P_f64),
                                              None if g is None else g.ctypes.data_as(P_f32)), "train_step")
        if not grads:
            return float(loss[0])
        out, off = [], 0
        for l in range(self.nlayers):
            nw = self.dims[l] * self.dims[l + 1]
            out.append((g[off:off + nw].reshape(self.dims[l + 1], self.dims[l]), g[off + nw:off + nw + self.dims[l + 1]]))
            off += nw + self.dims[l + 1]
        return float(loss[0]), out

    def launch_count(self):
        return int(self.L.esm_mlp_launch_count(self.h))
