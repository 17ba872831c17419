"""Diagnosis of flipped tasks in the parity tests of the line moves.

A flip is a task whose state leaves the tolerance because one move drew another t. Given the t of
every move on both sides (the device's move log and the oracle's), the first move where a task's
draws differ is located, the oracle replays that task up to the move, and ``Oracle.explain`` gives
the discrete choice that can have gone the other way and how close the oracle's own draw was to its
boundary:
  segment   the categorical draw of the segment: the distance of u = u_cat * tot from the interval
            of the segment holding the device's t, relative to the total mass;
  jacobian  the accept test of a compensated move: |u_j - exp(min(0, log J))|;
  stop      where a walk stops (c - cmin - maxnats at a primary breakpoint), over maxnats;
  offset    the same segment with another offset: the continuous map from u_off to t within the
            segment carries the round-off of the segment's end points (margin |t_dev - t| / L);
            a segment flat to round-off (|g L| below 1e-8 nats in FP64, 1e-2 in FP32) has margin 0:
            there trexp_offset (src/local.jl:1106) draws from the left end (u L) when |g L| is below
            its threshold or g >= 0, and from the right end ((1 - u) L) otherwise, so the round-off
            sign of g picks the mirrored map -- both exact draws of the uniform conditional. Flat
            segments are exact where a move changes no term (a level move of the long-range storage
            sweep while every state stays inside the box), and a year-long move's potential carries
            round-off near the threshold's 1e-10 nats; the FP32 build also draws segments flat to
            its round-off scale (about 1e-3 nats on storage moves) uniformly;
  ray       (FP32 only) one of the two draws lies where its walk took ray steps, past every primary
            breakpoint: the FP32 build probes the ray slope 1e-3 ahead instead of 1e-6, so its ray
            points, and with them the map from the uniforms to t, differ there while the potential
            sampled does not; margin 0.
The smallest margin names the flip. Round-off flips have margins of the order of the arithmetic's
relative error; a structural difference (another point set, another rule) shows as a large margin.
"""
import numpy as np


def first_diffs(tdev, torc, tol_rel, tol_abs=None):
    """tdev, torc [moves, steps, reps] (NaN: no move): per task the first move whose t differs by
    more than tol_rel |t| + tol_abs (tol_abs defaults to tol_rel), or -1."""
    tol_abs = tol_rel if tol_abs is None else tol_abs
    na, nb = np.isnan(tdev), np.isnan(torc)
    diff = (na != nb) | (~na & ~nb & (np.abs(np.nan_to_num(tdev) - np.nan_to_num(torc)) >
                                      tol_rel * np.abs(np.nan_to_num(torc)) + tol_abs))
    anyd = diff.any(axis=0)
    return np.where(anyd, diff.argmax(axis=0), -1)


def in_ray(e, t):
    """Whether t lies in the ray region of its direction's walk."""
    if t > 0 and np.isfinite(e["ray_r"]):
        return t > e["ray_r"]
    if t < 0 and np.isfinite(e["ray_l"]):
        return t < e["ray_l"]
    return False


def classify(e, maxnats, fp32=False):
    """(kind, margin) of one explained flip: the same segment is an offset; otherwise the smallest
    margin among the discrete choices that apply."""
    cands = []
    if fp32 and (in_ray(e, e["t"]) or in_ray(e, e["t_dev"])):
        return ("ray", 0.0)
    if e["seg_other"] == e["seg"]:
        flat = abs(e["gL"]) <= (1e-2 if fp32 else 1e-8)
        return ("offset", 0.0 if flat else abs(e["t_dev"] - e["t"]) / max(e["L"], 1e-300))
    if e["seg_other"] >= 0 and e["seg_other"] != e["seg"]:
        cands.append(("segment", abs(e["cat_margin"])))
    for key in ("lj", "lj_other"):
        if np.isfinite(e[key]):
            cands.append(("jacobian", abs(e["uj"] - np.exp(min(0.0, e[key])))))
    for key in ("stop_r", "stop_l", "near_r", "near_l"):
        if np.isfinite(e[key]):
            cands.append(("stop", abs(e[key]) / maxnats))
    if not cands:
        return ("unknown", np.inf)
    return min(cands, key=lambda x: x[1])


def explain_flips(oracle_factory, sweep, cls, first, tdev, maxnats, limit=None, fp32=False):
    """Explain every flipped task: for each task with a first differing move, a fresh replay of
    that task on `oracle_factory()` (an oracle at the start state) up to the move, then
    Oracle.explain. Returns a list of dicts (q, rep, move, kind, margin, t_dev, t_orc, the explain
    fields)."""
    o = oracle_factory()
    out = []
    for q, rep in zip(*np.nonzero(first >= 0)):
        mi = int(first[q, rep])
        if limit is not None and mi >= limit:
            continue
        o.task_moves(sweep, cls, int(q), int(rep), 0, mi)
        e = o.explain(sweep, cls, mi, int(q), int(rep), float(np.nan_to_num(tdev[mi, q, rep])))
        if e is None:
            out.append(dict(q=int(q), rep=int(rep), move=mi, kind="no move", margin=np.inf))
            continue
        e["t_dev"] = float(tdev[mi, q, rep])
        kind, margin = classify(e, maxnats, fp32)
        out.append(dict(q=int(q), rep=int(rep), move=mi, kind=kind, margin=margin, **e))
    return out


def summary(flips):
    kinds = {}
    for f in flips:
        kinds.setdefault(f["kind"], []).append(f["margin"])
    return {k: (len(v), float(np.max(v))) for k, v in kinds.items()}
