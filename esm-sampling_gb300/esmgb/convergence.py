"""Convergence diagnostics of the capacity traces (src/convergence.jl, src/diagnostics.jl): the ESS
and MCSE behind the capacity ESS/s metric and the 2-MCSE agreement check.
"""
from __future__ import annotations

import math

import numpy as np
from scipy.special import erfcinv
from scipy.stats import rankdata


def _autocov(x):
    """Autocovariance with denominator n (as Stan), lags 0..n-1, via FFT."""
    n = len(x)
    xc = x - x.mean()
    f = np.fft.rfft(xc, 2 * n)
    ac = np.fft.irfft(f * np.conj(f))[:n] / n
    return ac


def split_chains(chains):
    out = []
    for c in chains:
        c = np.asarray(c, float)
        h = len(c) // 2
        out.append(c[:h])
        out.append(c[len(c) - h:])
    return out


def rank_normalize(chains):
    """z = Phi^-1((rank - 3/8)/(S + 1/4)) of the pooled draws, average ranks for ties
    (``src/convergence.jl:19`` rank_normalize)."""
    x = np.concatenate([np.asarray(c, float) for c in chains])
    r = rankdata(x, method="average")
    S = len(x)
    z = -math.sqrt(2) * erfcinv(2 * (r - 0.375) / (S + 0.25))
    out, o = [], 0
    for c in chains:
        out.append(z[o:o + len(c)])
        o += len(c)
    return out


def rhat_basic(chains):
    """Plain R-hat of equal-length chains (``src/convergence.jl:45``)."""
    M = len(chains)
    n = min(len(c) for c in chains)
    if M < 2 or n < 2:
        return math.nan
    ms = [np.mean(c[:n]) for c in chains]
    vs = [np.var(c[:n], ddof=1) for c in chains]
    W = float(np.mean(vs))
    B = n * float(np.var(ms, ddof=1))
    if W == 0:
        return 1.0 if B == 0 else math.inf
    vplus = (n - 1) / n * W + B / n
    return math.sqrt(vplus / W)


def rhat_rank(chains):
    """Rank-normalised split R-hat, max of bulk and folded (``src/convergence.jl:60``)."""
    sc = split_chains(chains)
    bulk = rhat_basic(rank_normalize(sc))
    med = float(np.median(np.concatenate(sc)))
    tail = rhat_basic(rank_normalize([np.abs(c - med) for c in sc]))
    return max(bulk, tail)


def ess_multi(chains):
    """Multi-chain ESS with Geyer's initial monotone sequence (``src/convergence.jl:94`` ess_multi)."""
    M = len(chains)
    n = min(len(c) for c in chains)
    if n < 4:
        return float(M * n)
    cs = [np.asarray(c[:n], float) for c in chains]
    acs = [_autocov(c) for c in cs]
    W = float(np.mean([np.var(c, ddof=1) for c in cs]))
    if W == 0:
        return float(M * n)
    ms = [c.mean() for c in cs]
    vplus = (n - 1) / n * W + (np.var(ms, ddof=1) if M > 1 else 0.0)
    acm = np.mean(acs, axis=0)
    rho = 1 - (W - acm) / vplus
    rho[0] = 1.0
    tau, prev, k = -1.0, math.inf, 0
    while 2 * k + 1 < n:
        Pk = rho[2 * k] + rho[2 * k + 1]
        if Pk <= 0:
            break
        Pk = min(Pk, prev)
        tau += 2 * Pk
        prev = Pk
        k += 1
    tau = max(tau, 1 / math.log10(M * n))
    return M * n / tau


def ess_bulk(chains):
    """Bulk ESS: rank-normalised split chains (``src/convergence.jl:125``)."""
    return ess_multi(rank_normalize(split_chains(chains)))


def mcse_rel(chains):
    """MCSE of the mean relative to the sd: 1/sqrt(ESS) (``src/convergence.jl:141``)."""
    return 1 / math.sqrt(max(ess_multi(split_chains(chains)), 1.0))


def ess_single(x):
    """Single-chain Geyer ESS (``src/diagnostics.jl:8`` ess)."""
    x = np.asarray(x, float)
    n = len(x)
    if n < 4:
        return float(n)
    v = np.sum((x - x.mean()) ** 2) / n
    if v == 0:
        return float(n)
    ac = _autocov(x) / v
    s, prev, k = 0.0, math.inf, 0
    while 2 * k + 1 < n:
        G = ac[2 * k] + ac[2 * k + 1]
        if G <= 0:
            break
        G = min(G, prev)
        s += G
        prev = G
        k += 1
    tau = -1 + 2 * s
    return n / max(tau, 1.0 / n)


def agree(mean_a, mcse_a, mean_b, mcse_b):
    """Marginal agreement within 2 MCSE: |mean_A - mean_B| <= 2 sqrt(MCSE_A^2 + MCSE_B^2)."""
    return abs(mean_a - mean_b) <= 2 * math.sqrt(mcse_a ** 2 + mcse_b ** 2)
