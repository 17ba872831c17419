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
           "esm_mlp_forward", "esm_mlp_train_step", "esm_mlp_launch_count", "esm_mlp_set_gemm")

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
        L.esm_mlp_set_gemm.argtypes = [C.c_void_p, C.c_int32]
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

    def set_gemm(self, kind):
        """1: tcgen05 tensor-core GEMMs (default), 0: the mma.sync kernel."""
        self._check(self.L.esm_mlp_set_gemm(self.h, int(kind)), "esm_mlp_set_gemm")


# ---------------------------------------------------------------------------------------------
# online surrogate of the replica-averaged score
# ---------------------------------------------------------------------------------------------
class ScoreSurrogate:
    """MLP from (capacities / upper bound, regime occupancy) to the replica-averaged score s_bar [K],
    trained online on the pairs the plain sampler produces (a replay buffer of the latest
    `capacity` pairs, minibatches of `batch`, Adam at `lr`). Targets are standardised per unit with
    the mean and deviation of the pairs in the buffer, refreshed at every training call (the
    sampler's transient moves the scores by orders of magnitude)."""

    def __init__(self, m, hidden=(512, 512, 512), capacity=8192, batch=1024, lr=1e-3, seed=1, min_pairs=64):
        self.K = m.Kunits
        self.nin = self.K + 4 * m.K
        self.hi = np.maximum(np.asarray(m.unit_hi, float), 1.0)
        self.mlp = MLP([self.nin, *hidden, self.K], batch_max=batch, seed=seed)
        self.X = np.zeros((capacity, self.nin), np.float32)
        self.Y = np.zeros((capacity, self.K), np.float64)
        self.n = self.pos = 0
        self.batch, self.lr, self.min_pairs = batch, lr, min_pairs
        self.mu = np.zeros(self.K)
        self.sd = np.ones(self.K)
        self.rng = np.random.default_rng(seed)
        self.losses = []

    def features(self, k, occ):
        return np.concatenate([np.asarray(k, float) / self.hi, np.asarray(occ, float)]).astype(np.float32)

    def add(self, k, occ, sbar):
        self.X[self.pos] = self.features(k, occ)
        self.Y[self.pos] = np.nan_to_num(np.asarray(sbar, float), nan=0.0, posinf=0.0, neginf=0.0)
        self.pos = (self.pos + 1) % len(self.X)
        self.n = min(self.n + 1, len(self.X))

    @property
    def ready(self):
        return self.n >= self.min_pairs

    def train(self, steps=1):
        if not self.ready:
            return None
        y = self.Y[: self.n]
        self.mu = y.mean(0)
        self.sd = np.maximum(y.std(0), 1e-9 + 1e-6 * np.abs(self.mu))
        loss = None
        for _ in range(steps):
            idx = self.rng.integers(0, self.n, size=min(self.batch, self.n))
            t = (self.Y[idx] - self.mu) / self.sd
            loss = self.mlp.train_step(self.X[idx], t.astype(np.float32), self.lr)
        self.losses.append(loss)
        return loss

    def predict(self, k, occ):
        y = self.mlp.forward(self.features(k, occ)[None])[0].astype(np.float64)
        return y * self.sd + self.mu

    def close(self):
        self.mlp.close()


# ---------------------------------------------------------------------------------------------
# delayed-acceptance Langevin step of the capacities
# ---------------------------------------------------------------------------------------------
class DALangevin:
    """Capacity moves proposed with the surrogate's drift at `mult` times the plain step, accepted in
    two stages (Christen and Fox 2005):

    - stage 1, with the surrogate: the Metropolis-adjusted Langevin ratio in w = log(k + kappa_s),
      the log-density difference taken as the trapezoid path integral of the surrogate gradient
      G_s(w) = (k + kappa_s) g_s + 1, g_s = -fk + (beta_k / beta_v) s_hat;
    - stage 2, with the plain replica estimate: every replica follows the proposed capacities and
      sweeps, the plain scores give G(w'), and the move is kept with probability
      min(1, exp(dU - dU_s)), dU the trapezoid integral of the plain gradient.

    Stage 2 targets what the plain estimate targets; a proposal rejected there restores the state
    saved before it. An iteration that does not reach stage 2 sweeps at the current capacities (as
    the plain step does) and refreshes G(w). Every plain evaluation trains the surrogate. Proposals
    outside [kappa_min, hi] are rejected."""

    def __init__(self, d, m, sur, eta, kappa_s, kmin=1.0, clip=0.02, mult=4.0, weights=None, seed=0,
                 train_steps=1, blocks=False):
        self.d, self.m, self.sur = d, m, sur
        ug = np.asarray(m.unit_group)
        self.eta_u = np.asarray(eta, float)[ug]
        self.ks_u = np.asarray(kappa_s, float)[ug]
        self.moving = self.eta_u > 0
        # blocks: propose one capacity group per iteration (cycled), fewer dimensions per acceptance
        self.groups = [np.flatnonzero((ug == gq) & self.moving) for gq in np.unique(ug)] if blocks else None
        self.groups = [g for g in self.groups if len(g)] if blocks else None
        self.h = mult * self.eta_u
        self.clip = mult * clip
        self.kmin = kmin
        self.hi = np.asarray(m.unit_hi, float)
        self.ratio = m.beta_k / m.beta_v
        self.w = np.full(d.R, 1.0 / d.R) if weights is None else np.asarray(weights, float)
        self.rng = np.random.default_rng(seed)
        self.train_steps = train_steps
        self.k = np.asarray(d.download_k(), float).copy()
        self.G = self.fk = None
        self.stats = {"iters": 0, "stage1": 0, "accepted": 0, "plain_evals": 0}

    def grad_w(self, k, sbar, fk):
        return (k + self.ks_u) * (-fk + self.ratio * sbar) + 1.0

    def _plain(self, it):
        self.d.sweeps(1, sweep0=it, stats=False)
        sk, fk, _ = self.d.scores()
        self.stats["plain_evals"] += 1
        return self.w @ sk, fk

    def step(self, it):
        d = self.d
        if self.groups:
            mv = np.zeros_like(self.moving)
            mv[self.groups[self.stats["iters"] % len(self.groups)]] = True
        else:
            mv = self.moving
        self.stats["iters"] += 1
        occ = d.regime_occupancy()
        if self.G is None or not self.sur.ready:
            sbar, self.fk = self._plain(it)
            self.G = self.grad_w(self.k, sbar, self.fk)
            self.sur.add(self.k, occ, sbar)
            self.sur.train(self.train_steps)
            return False
        h = self.h
        w0 = np.log(self.k + self.ks_u)
        Gs0 = self.grad_w(self.k, self.sur.predict(self.k, occ), self.fk)
        dr0 = np.clip(h * Gs0, -self.clip, self.clip)
        w1 = w0.copy()
        w1[mv] = w0[mv] + dr0[mv] + np.sqrt(2 * h[mv]) * self.rng.standard_normal(mv.sum())
        k1 = self.k.copy()
        k1[mv] = np.exp(w1[mv]) - self.ks_u[mv]
        inside = bool(np.all(k1[mv] >= self.kmin) and np.all(k1[mv] <= self.hi[mv]))
        go = False
        if inside:
            Gs1 = self.grad_w(k1, self.sur.predict(k1, occ), self.fk)
            dr1 = np.clip(h * Gs1, -self.clip, self.clip)
            dw = (w1 - w0)[mv]
            lq_f = -np.sum((dw - dr0[mv]) ** 2 / (4 * h[mv]))
            lq_b = -np.sum((-dw - dr1[mv]) ** 2 / (4 * h[mv]))
            dUs = float(np.sum(dw * (Gs0[mv] + Gs1[mv]) / 2))
            go = np.log(self.rng.random()) < dUs + lq_b - lq_f
        accepted = False
        if go:
            self.stats["stage1"] += 1
            d.state_save()
            d.follow_capacities(k1, self.kmin)
            sbar1, fk1 = self._plain(it)
            G1 = self.grad_w(k1, sbar1, fk1)
            self.sur.add(k1, occ, sbar1)
            dU = float(np.sum(dw * (self.G[mv] + G1[mv]) / 2))
            if np.log(self.rng.random()) < dU - dUs:
                self.k, self.G, self.fk = k1, G1, fk1
                accepted = True
                self.stats["accepted"] += 1
            else:
                d.state_restore()
        else:
            sbar, self.fk = self._plain(it)
            self.G = self.grad_w(self.k, sbar, self.fk)
            self.sur.add(self.k, occ, sbar)
        self.sur.train(self.train_steps)
        return accepted


# ---------------------------------------------------------------------------------------------
# surrogate-drift Langevin step of the capacities
# ---------------------------------------------------------------------------------------------
class SurrogateLangevin:
    """The learned capacity step that keeps the plain step's form: the Langevin update of
    langevin_update (src/replicas.jl:368; w = log(k + kappa_s), w' = w + clamp(h G, +-clip) +
    sqrt(2 h) xi, reflected at w_min and, from below, at the box) at `mult` times the plain step size,
    its drift G = (k + kappa_s)(-fk + (beta_k/beta_v) s) + 1 taken from the surrogate s_hat(k) instead
    of the plain replica estimate s_bar. Every replica then follows the new capacities and sweeps, and
    the plain scores there (one plain evaluation per iteration, as the plain step) train the surrogate
    and judge it: a running mean (decay `decay`) of the discrepancy between the plain estimate and
    the surrogate per capacity, in units of the plain estimate's own noise (the spread of the
    replicas' scores over sqrt(R)). While the surrogate is untrained, or the mean absolute judged
    discrepancy of the moving capacities exceeds `tol`, the iteration is the plain step (the plain
    drift at the plain step size).

    The plain step is a Langevin step on a noisy drift (the replica average of R scores): at a step
    size h its noise adds about h^2 Var(G) per step to the 2h of the injected noise. The surrogate's
    drift averages the plain estimates of many iterations, so a longer step does not carry that
    noise; what it carries instead is the surrogate's error, which the judge bounds."""

    def __init__(self, d, m, sur, eta, kappa_s, kmin=1.0, clip=0.02, mult=4.0, weights=None, seed=0,
                 train_steps=1, tol=1.0, decay=0.9):
        self.d, self.m, self.sur = d, m, sur
        ug = np.asarray(m.unit_group)
        self.eta_u = np.asarray(eta, float)[ug]
        self.ks_u = np.asarray(kappa_s, float)[ug]
        self.moving = self.eta_u > 0
        self.mult, self.clip, self.kmin = mult, clip, kmin
        self.hi = np.asarray(m.unit_hi, float)
        self.ratio = m.beta_k / m.beta_v
        self.w = np.full(d.R, 1.0 / d.R) if weights is None else np.asarray(weights, float)
        self.rng = np.random.default_rng(seed)
        self.train_steps, self.tol, self.decay = train_steps, tol, decay
        self.k = np.asarray(d.download_k(), float).copy()
        self.z = np.zeros(m.Kunits)
        self.G = self.fk = None
        self.occ = None
        self.stats = {"iters": 0, "learned": 0, "plain_evals": 0}

    def grad_w(self, k, sbar, fk):
        return (k + self.ks_u) * (-fk + self.ratio * sbar) + 1.0

    def update(self, k, G, h, clip):
        """langevin_update on the moving capacities (the device's k_langevin, on the host)."""
        mv = self.moving
        ks = self.ks_u[mv]
        w = np.log(k[mv] + ks)
        w1 = w + np.clip(h[mv] * G[mv], -clip, clip) + np.sqrt(2 * h[mv]) * self.rng.standard_normal(mv.sum())
        wmin = np.log(self.kmin + ks)
        w1 = np.where(w1 < wmin, 2 * wmin - w1, w1)
        wmax = np.log(np.maximum(self.hi[mv], self.kmin + 1.0) + ks)
        w1 = np.where((w1 > wmax) & (w <= wmax), np.maximum(2 * wmax - w1, wmin), w1)
        out = k.copy()
        out[mv] = np.exp(w1) - ks
        return out

    def plain(self, it):
        """One plain evaluation at the current capacities: (s_bar, fk, the noise sd of G)."""
        self.d.sweeps(1, sweep0=it, stats=False)
        sk, fk, _ = self.d.scores()
        self.stats["plain_evals"] += 1
        sbar = self.w @ sk
        sd = (self.k + self.ks_u) * self.ratio * sk.std(axis=0) / np.sqrt(len(sk))
        return sbar, fk, sd

    def step(self, it, weather=None):
        """One iteration; weather (optional): the weather draws of the step, applied first."""
        d = self.d
        self.stats["iters"] += 1
        if weather is not None and weather[0].any():
            moved, theta, window, wstart = weather[:4]
            d.weather_step(moved, theta, window, wstart, it=it)
            self.occ = None
        if self.occ is None:
            self.occ = d.regime_occupancy()
        if self.G is None:
            sbar, self.fk, _ = self.plain(it)
            self.G = self.grad_w(self.k, sbar, self.fk)
            self.sur.add(self.k, self.occ, sbar)
        judged = np.mean(np.abs(self.z[self.moving]))
        use = self.sur.ready and judged <= self.tol
        if use:
            s_hat = self.sur.predict(self.k, self.occ)
            # a prediction outside what the buffer has seen (or not finite) is not trusted
            use = bool(np.all(np.isfinite(s_hat)) and
                       np.all(np.abs(s_hat - self.sur.mu) <= 10 * self.sur.sd + 1e-12))
        if use:
            Gs = self.grad_w(self.k, s_hat, self.fk)
            k1 = self.update(self.k, Gs, self.mult * self.eta_u, self.mult * self.clip)
            self.stats["learned"] += 1
        else:
            k1 = self.update(self.k, self.G, self.eta_u, self.clip)
        self.k = d.follow_capacities(k1, self.kmin)
        sbar, self.fk, sd = self.plain(it)
        self.G = self.grad_w(self.k, sbar, self.fk)
        if self.sur.ready:
            Gs1 = self.grad_w(self.k, self.sur.predict(self.k, self.occ), self.fk)
            # the noise scale of the plain drift, floored where the replicas agree to round-off
            scale = np.maximum(sd, 1e-3 * np.abs(self.G) + 1e-6)
            zz = np.nan_to_num((self.G - Gs1) / scale, nan=10.0, posinf=10.0, neginf=-10.0)
            self.z = self.decay * self.z + (1 - self.decay) * np.clip(zz, -10, 10)
        self.sur.add(self.k, self.occ, sbar)
        self.sur.train(self.train_steps)
        return use
