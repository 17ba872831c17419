// Warp-cooperative walk of the separable storage moves (the state-of-charge atoms of a storage field:
// storage units at distinct nodes and nothing else), one (step, replica) task per warp.
//
// The line potential of such a move is a sum of one-dimensional piecewise-linear unit functions,
// each with at most ten kinks in a walking direction: its clamps (0 and 1 of the state of charge,
// the primary breakpoints of walk!, src/local.jl:1294), its storage thresholds and the zero
// crossings of its two node balances (the secondary roots of piece_roots!, :1267). The walk visits
// the union of those points in walking order, stops at the first clamp where the potential stands
// more than maxnats above its minimum, and takes ray steps once every clamp is behind.
//
// Here the lanes own the units. The walk goes window by window, a window ending at the nearest clamp
// still ahead: every lane generates the events of its units up to the window end (the same per-unit
// piece arithmetic as the per-lane walk), the window's events are compacted in unit order and sorted
// in shared memory (bitonic, by time, ties by unit and sequence), and the potential at every event
// follows from three warp scans over the sorted events (slope before the event, potential, running
// minimum). Points, segment masses and the categorical draw (sample_line!, :1501) stay in shared
// memory, so the walk keeps no per-lane scratch and runs without divergence between tasks.
#pragma once
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "esm_common.cuh"

namespace esm {

// events one unit can produce in one window (clamps, six storage thresholds, two node-balance roots)
#define ESM_SEP_EVMAX 12

// per-unit fields of the walk state (shared memory, field-major: field f of unit q at f * nu + q)
enum {
    SF_UT = 0,   // time of the unit's next event (+-inf: none)
    SF_UK,       // its kind: 1 clamp, 0 other, -1 none
    SF_USL,      // the unit's slope up to that event
    SF_UE,       // events of the current piece (3)
    SF_UN = SF_UE + 3,
    SF_UH,       // how the piece ends: 1 clamp, 2 threshold, 0 not at all
    SF_UI,       // next event of the piece
    SF_UFE,      // potential at the piece end (or at a probe beyond the piece start)
    SF_UFN,      // potential at the next event
    SF_USW,      // node balances at the piece end (step tau, step tau - 1)
    SF_USA,
    SF_E0,       // state of charge at tau, tau + 1, tau - 1 and the node balances at tau, tau - 1
    SF_E1,
    SF_EM,
    SF_S0W,
    SF_S0A,
    SF_CL0,      // the clamps still ahead, in walking order, and their count
    SF_CL1,
    SF_NCL,
    SF_N
};

struct SepLayout {
    int nu, maxpts, ev, wb;  // unit capacity, point cap per direction, event slots, sort capacity (power of 2)
    int o_us, o_skey, o_wkey, o_wpay, o_wdsl, o_wdab, o_wcl, o_ucnt, o_pts, o_lm, total;  // byte offsets, bytes
};

template <class real>
__host__ __device__ inline SepLayout sep_layout(int nu, int maxpts) {
    SepLayout L;
    L.nu = nu < 1 ? 1 : nu;
    L.maxpts = maxpts;
    L.ev = L.nu * ESM_SEP_EVMAX;
    int wb = 2;
    while (wb < L.ev) wb <<= 1;
    L.wb = wb;
    int o = 0;
    auto take = [&](int bytes) {
        o = (o + 15) & ~15;
        int r = o;
        o += bytes;
        return r;
    };
    L.o_us = take((int)sizeof(real) * SF_N * L.nu);
    L.o_skey = take((int)sizeof(real) * L.ev);
    L.o_wkey = take((int)sizeof(real) * wb);
    L.o_wpay = take((int)sizeof(int) * wb);
    L.o_wdsl = take((int)sizeof(double) * L.ev);
    L.o_wdab = take((int)sizeof(float) * L.ev);
    L.o_wcl = take(L.ev);
    L.o_ucnt = take((int)sizeof(int) * L.nu);
    L.o_pts = take((int)sizeof(real) * 6 * maxpts);
    L.o_lm = take((int)sizeof(real) * (2 * maxpts + 1));
    L.total = (o + 127) & ~127;
    return L;
}

template <class real>
__device__ inline real warp_min(real v) {
    for (int o = 16; o > 0; o >>= 1) v = fmin(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}
template <class real>
__device__ inline real warp_max(real v) {
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}
template <class T>
__device__ inline T warp_sum(T v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
template <class T>
__device__ inline T warp_incl_sum(T v, int lane) {
    for (int o = 1; o < 32; o <<= 1) {
        T x = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += x;
    }
    return v;
}
__device__ inline double warp_incl_min(double v, int lane) {
    for (int o = 1; o < 32; o <<= 1) {
        double x = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v = fmin(v, x);
    }
    return v;
}

template <class real>
struct SepWalk {
    const DevModel<real> &M;
    const Desc<real> &d;
    const SepLayout &SL;
    char *base;  // this warp's region (shared memory, or its slab of global memory)
    int lane, nu;
    int tau, taum, tau1, rep;

    __device__ SepWalk(const DevModel<real> &M_, const Desc<real> &d_, const SepLayout &SL_, char *base_, int lane_)
        : M(M_), d(d_), SL(SL_), base(base_), lane(lane_) {
        nu = d.hdr[1];
    }

    __device__ inline real &U(int f, int q) const { return ((real *)(base + SL.o_us))[f * SL.nu + q]; }
    __device__ inline size_t ix(int x, int t) const { return sidx(x, t, rep, M.T, M.R); }

    // the task's unit values (state of charge at three steps, node balances at two)
    __device__ void load_units() const {
        for (int q = lane; q < nu; q += 32) {
            int j = d.si[q];
            U(SF_E0, q) = M.e[ix(j, tau)];
            U(SF_E1, q) = M.e[ix(j, tau1)];
            U(SF_EM, q) = M.e[ix(j, taum)];
            U(SF_S0W, q) = M.r[ix(d.nds[d.spos[q]], tau)];
            U(SF_S0A, q) = M.r[ix(d.nda[d.sposa[q]], taum)];
        }
        __syncwarp();
    }

    // beta * (cost change) of unit q at t, with its two node balances (the per-lane walk's unit_val
    // on the cached values: the same arithmetic, so the same events)
    __device__ __noinline__ real unit_val(int q, real t, real *Sw, real *Sa) const {
        int j = d.si[q];
        real x = t * d.sa[q];
        real k = M.kc_s[j], w = k + M.kappa0, dt = M.dt, cv = M.c_viol;
        real djw, dw, dja, da;
        real cw = soc_diff<real>(M.s_hours[j], M.s_qt[j], M.s_etain[j], M.s_etaout[j], M.s_mc[j], k, w, dt, cv,
                                 U(SF_E0, q), U(SF_E1, q), x, real(0), &djw, &dw);
        real ca = soc_diff<real>(M.s_hours[j], M.s_qt[j], M.s_etain[j], M.s_etaout[j], M.s_mc[j], k, w, dt, cv,
                                 U(SF_EM, q), U(SF_E0, q), real(0), x, &dja, &da);
        real S0w = U(SF_S0W, q), S0a = U(SF_S0A, q);
        *Sw = S0w + djw;
        *Sa = S0a + dja;
        real bw = dt * phibal_diff<real>(S0w, djw, M.c_shed, M.c_dump);
        real ba = dt * phibal_diff<real>(S0a, dja, M.c_shed, M.c_dump);
        return M.beta_v * (cw + bw + ca + ba);
    }

    __device__ inline static bool root_of(real a, real b, real lo, real hi, real sgn, real *x) {
        if ((a < 0) != (b < 0) && a != b) {
            real xx = lo + (hi - lo) * a / (a - b);
            if (sgn * (xx - lo) > 0 && sgn * (hi - xx) > 0) {
                *x = xx;
                return true;
            }
        }
        return false;
    }

    // the piece of unit q starting at t0 (node balances Sw0, Sa0 there): its end and the node-balance
    // roots inside it, as the per-lane walk's unit_piece
    __device__ __noinline__ void unit_piece(int q, real t0, real sgn, real Sw0, real Sa0) const {
        int j = d.si[q];
        real a = d.sa[q];
        real e0 = U(SF_E0, q);
        real e1c = clampr<real>(U(SF_E1, q), 0, 1), emc = clampr<real>(U(SF_EM, q), 0, 1);
        real h = M.s_hours[j], qt = M.s_qt[j], ein = M.s_etain[j], eout = M.s_etaout[j], dt = M.dt;
        bool have = false, prim = false;
        real ts = 0;
        auto cand = [&](real x, bool p) {
            real tc = x / a;
            if (!isfinite(tc) || !(sgn * (tc - t0) > 0)) return;
            if (!have || sgn * (tc - ts) < 0) {
                ts = tc;
                prim = p;
                have = true;
            }
        };
        cand(real(0) - e0, true);
        cand(real(1) - e0, true);
        real th[3];
        int nth = 0;
        th[nth++] = 0;
        if (ein > 0) th[nth++] = ein;
        if (eout > 0) th[nth++] = real(-1) / eout;
        for (int i = 0; i < nth; ++i) {
            real xw = e1c - e0 - (th[i] + qt) * dt / h;
            if (e0 + xw >= 0 && e0 + xw <= 1) cand(xw, false);
            real xa = emc - e0 + (th[i] + qt) * dt / h;
            if (e0 + xa >= 0 && e0 + xa <= 1) cand(xa, false);
        }
        real tpb = have ? ts : t0 + sgn * fmax(real(1), fabs(t0));
        real Sw1, Sa1;
        U(SF_UFE, q) = unit_val(q, tpb, &Sw1, &Sa1);
        U(SF_USW, q) = Sw1;
        U(SF_USA, q) = Sa1;
        real r[2];
        int nr = 0;
        real pa[2] = {Sw0, Sa0}, pb[2] = {Sw1, Sa1};
        for (int i = 0; i < 2; ++i) {
            real x;
            if (have) {
                if (root_of(pa[i], pb[i], t0, tpb, sgn, &x)) r[nr++] = x;
            } else if (pa[i] != pb[i]) {
                x = t0 + (tpb - t0) * pa[i] / (pa[i] - pb[i]);
                if (isfinite(x) && sgn * (x - t0) > 0) r[nr++] = x;
            }
        }
        if (nr == 2 && sgn * (r[1] - r[0]) < 0) {
            real x = r[0];
            r[0] = r[1];
            r[1] = x;
        }
        int n = 0;
        for (int i = 0; i < nr; ++i) U(SF_UE + n++, q) = r[i];
        if (have) U(SF_UE + n++, q) = ts;
        U(SF_UN, q) = real(n);
        U(SF_UH, q) = have ? (prim ? real(1) : real(2)) : real(0);
        U(SF_UI, q) = real(0);
    }

    // the next event of unit q after its position t (potential f there), as the per-lane unit_next
    __device__ __noinline__ void unit_next(int q, real t, real f, real sgn) const {
        int i = (int)U(SF_UI, q), n = (int)U(SF_UN, q), hk = (int)U(SF_UH, q);
        real Sw, Sa, tn, fn;
        if (i < n) {
            tn = U(SF_UE + i, q);
            bool end = i == n - 1 && hk != 0;
            fn = end ? U(SF_UFE, q) : unit_val(q, tn, &Sw, &Sa);
            U(SF_UT, q) = tn;
            U(SF_UK, q) = end ? (hk == 1 ? real(1) : real(0)) : real(0);
            U(SF_UFN, q) = fn;
            U(SF_USL, q) = tn != t ? (fn - f) / (tn - t) : real(0);
        } else {
            real tp = t + sgn * fmax(real(1), fabs(t));
            fn = unit_val(q, tp, &Sw, &Sa);
            U(SF_UT, q) = real(INFINITY) * sgn;
            U(SF_UK, q) = real(-1);
            U(SF_USL, q) = (fn - f) / (tp - t);
        }
    }

    __device__ void unit_pass(int q, real t, real sgn) const {
        int i = (int)U(SF_UI, q), n = (int)U(SF_UN, q), hk = (int)U(SF_UH, q);
        real f = U(SF_UFN, q);
        if (i == n - 1 && hk != 0)
            unit_piece(q, t, sgn, U(SF_USW, q), U(SF_USA, q));
        else
            U(SF_UI, q) = real(i + 1);
        unit_next(q, t, f, sgn);
    }

    // sort n (key, payload) pairs ascending by key, then payload (bitonic, padded to a power of 2)
    __device__ void sort_window(real *key, int *pay, int n) const {
        int n2 = 2;
        while (n2 < n) n2 <<= 1;
        for (int i = n + lane; i < n2; i += 32) {
            key[i] = real(INFINITY);
            pay[i] = 0x7fffffff;
        }
        __syncwarp();
        for (int k = 2; k <= n2; k <<= 1)
            for (int j = k >> 1; j > 0; j >>= 1) {
                for (int i = lane; i < (n2 >> 1); i += 32) {
                    int lo = ((i & ~(j - 1)) << 1) | (i & (j - 1));
                    int hi = lo + j;
                    real ka = key[lo], kb = key[hi];
                    int pa = pay[lo], pb = pay[hi];
                    bool up = (lo & k) == 0;
                    bool gt = ka > kb || (ka == kb && pa > pb);
                    if (gt == up) {
                        key[lo] = kb;
                        key[hi] = ka;
                        pay[lo] = pb;
                        pay[hi] = pa;
                    }
                }
                __syncwarp();
            }
    }

    // One direction of walk! (src/local.jl:1294) for the separable move. Returns 1 proper, 0 improper
    // (ray steps exhausted), -1 when the points exceed the cap or a unit its event slots (a guard
    // event). The points, their potentials and (FP32) round-off scales go to P, C, Z; *np their count.
    __device__ __noinline__ int walk(real sgn, real *P, real *C, real *Z, int *np) const {
        real *skey = (real *)(base + SL.o_skey);
        real *wkey = (real *)(base + SL.o_wkey);
        int *wpay = (int *)(base + SL.o_wpay);
        double *wdsl = (double *)(base + SL.o_wdsl);
        float *wdab = (float *)(base + SL.o_wdab);
        unsigned char *wcl = (unsigned char *)(base + SL.o_wcl);
        int *ucnt = (int *)(base + SL.o_ucnt);
        const real INF = real(INFINITY);
        const int maxpts = SL.maxpts;
        double Bl = 0, Al = 0;
        int ncll = 0;
        for (int q = lane; q < nu; q += 32) {
            real a = d.sa[q], e0 = U(SF_E0, q);
            real c0 = (real(0) - e0) / a, c1 = (real(1) - e0) / a;
            bool h0 = isfinite(c0) && sgn * c0 > 0, h1 = isfinite(c1) && sgn * c1 > 0;
            real f0 = h0 ? c0 : c1, f1 = c1;
            if (h0 && h1 && sgn * (c1 - c0) < 0) {
                f0 = c1;
                f1 = c0;
            }
            U(SF_CL0, q) = (h0 || h1) ? f0 : INF * sgn;
            U(SF_CL1, q) = (h0 && h1) ? f1 : INF * sgn;
            U(SF_NCL, q) = real((int)h0 + (int)h1);
            ncll += (int)h0 + (int)h1;
            unit_piece(q, real(0), sgn, U(SF_S0W, q), U(SF_S0A, q));
            unit_next(q, real(0), real(0), sgn);
            Bl += (double)U(SF_USL, q);
            Al += fabs((double)U(SF_USL, q));
        }
        double B = warp_sum(Bl), absB = warp_sum(Al);
        int ncl = warp_sum(ncll);
        int npts = 0;
        double c = 0, cmin = 0;
        real tcur = 0;
        bool over = false;
        while (ncl > 0) {
            // the window ends at the nearest clamp ahead
            real wl = INF;
            for (int q = lane; q < nu; q += 32)
                if (U(SF_NCL, q) > 0) wl = fmin(wl, sgn * U(SF_CL0, q));
            wl = warp_min(wl);
            if (!(wl < INF)) break;  // (no clamp left where the count expects one: ray steps)
            real W = sgn * wl;
            int ncw = 0;
            for (int q = lane; q < nu; q += 32) {
                int cq = 0;
                while (true) {
                    real tq = U(SF_UT, q);
                    if (!isfinite(tq) || !(sgn * tq <= sgn * W)) break;
                    if (cq >= ESM_SEP_EVMAX) {
                        over = true;
                        break;
                    }
                    bool clamp = U(SF_UK, q) == real(1);
                    real old = U(SF_USL, q);
                    unit_pass(q, tq, sgn);
                    real nw = U(SF_USL, q);
                    int slot = q * ESM_SEP_EVMAX + cq;
                    skey[slot] = sgn * tq;
                    wdsl[slot] = (double)nw - (double)old;
                    wdab[slot] = (float)fmax(0.0, fabs((double)nw) - fabs((double)old));
                    wcl[slot] = clamp ? 1 : 0;
                    if (clamp) {
                        ++ncw;
                        U(SF_CL0, q) = U(SF_CL1, q);
                        U(SF_CL1, q) = INF * sgn;
                        U(SF_NCL, q) -= real(1);
                    }
                    ++cq;
                }
                ucnt[q] = cq;
            }
            if (__any_sync(0xffffffffu, over)) return -1;
            __syncwarp();
            // compaction in unit order
            int n = 0;
            for (int q0 = 0; q0 < nu; q0 += 32) {
                int q = q0 + lane;
                int cq = q < nu ? ucnt[q] : 0;
                int incl = warp_incl_sum(cq, lane);
                int pos = n + incl - cq;
                for (int s = 0; s < cq; ++s) {
                    wkey[pos + s] = skey[q * ESM_SEP_EVMAX + s];
                    wpay[pos + s] = q * ESM_SEP_EVMAX + s;
                }
                n += __shfl_sync(0xffffffffu, incl, 31);
            }
            __syncwarp();
            sort_window(wkey, wpay, n);
            ncl -= warp_sum(ncw);
            // the potential along the window's events
            int npw = npts;
            for (int b0 = 0; b0 < n; b0 += 32) {
                int i = b0 + lane;
                bool v = i < n;
                real ti = v ? sgn * wkey[i] : tcur;
                real tp = i == 0 ? tcur : sgn * wkey[(v ? i : n) - 1];
                int slot = v ? wpay[i] : 0;
                double ds = v ? wdsl[slot] : 0.0;
                double da = v ? (double)wdab[slot] : 0.0;
                bool cl = v && wcl[slot];
                double dsi = warp_incl_sum(ds, lane);
                double Bx = B + (dsi - ds);  // the summed slope before the event
                double inc = v ? Bx * (double)(ti - tp) : 0.0;
                double ci = c + warp_incl_sum(inc, lane);
                double cmi = fmin(cmin, warp_incl_min(v ? ci : 1e300, lane));
                double dai = warp_incl_sum(da, lane);
                double Ax = absB + (dai - da);
                bool stop = cl && (ci - cmi > (double)M.maxnats);
                unsigned sb = __ballot_sync(0xffffffffu, stop);
                int last = sb ? __ffs(sb) - 1 : 31;
                bool gd = false;
                if (v && lane <= last) {
                    int k = npw + i;
                    if (k >= maxpts) {
                        gd = true;
                    } else {
                        P[k] = ti;
                        C[k] = (real)ci;
                        if constexpr (sizeof(real) == 4) Z[k] = real(4.8e-7) * (real)(fabs(ci) + Ax * fabs((double)ti));
                    }
                }
                if (__any_sync(0xffffffffu, gd)) return -1;
                int lv = min(last, n - 1 - b0);
                B = __shfl_sync(0xffffffffu, Bx + ds, lv);
                c = __shfl_sync(0xffffffffu, ci, lv);
                cmin = __shfl_sync(0xffffffffu, cmi, lv);
                absB = __shfl_sync(0xffffffffu, Ax + da, lv);
                tcur = __shfl_sync(0xffffffffu, ti, lv);
                if (sb) {
                    __syncwarp();
                    *np = npw + b0 + lv + 1;
                    return 1;
                }
            }
            npts = npw + n;
            __syncwarp();
        }
        // ray steps once every clamp is behind (every unit then sits outside its box, so no events
        // are expected; any left are taken in order)
        real delta = 0;
        int nx = 0;
        auto point = [&](real t) -> bool {
            if (npts >= maxpts) return false;
            if (lane == 0) {
                P[npts] = t;
                C[npts] = (real)c;
                if constexpr (sizeof(real) == 4) Z[npts] = real(4.8e-7) * (real)(fabs(c) + absB * fabs((double)t));
            }
            ++npts;
            cmin = fmin(cmin, c);
            return true;
        };
        // the unit with the nearest pending event: (time, owner lane, unit) -- warp-uniform
        auto nearest = [&](real *tS, int *qS) {
            real best = INF;
            int bq = 0x7fffffff;
            for (int q = lane; q < nu; q += 32) {
                real tq = U(SF_UT, q);
                if (isfinite(tq) && (sgn * tq < best || (sgn * tq == best && q < bq))) {
                    best = sgn * tq;
                    bq = q;
                }
            }
            for (int o = 16; o > 0; o >>= 1) {
                real ob = __shfl_xor_sync(0xffffffffu, best, o);
                int oq = __shfl_xor_sync(0xffffffffu, bq, o);
                if (ob < best || (ob == best && oq < bq)) {
                    best = ob;
                    bq = oq;
                }
            }
            *tS = sgn * best;
            *qS = bq;
        };
        auto pass = [&](int qS, real tS) {
            double ds = 0, da = 0;
            if ((qS & 31) == lane) {
                real old = U(SF_USL, qS);
                unit_pass(qS, tS, sgn);
                real nw = U(SF_USL, qS);
                ds = (double)nw - (double)old;
                da = fmax(0.0, fabs((double)nw) - fabs((double)old));
            }
            B += __shfl_sync(0xffffffffu, ds, qS & 31);
            absB += __shfl_sync(0xffffffffu, da, qS & 31);
        };
        __syncwarp();
        while (true) {
            double sl = (double)sgn * B;
            if (sl > 0)
                delta = fmin(real(2) * M.maxnats / (real)sl, real(1e3) * fmax(fabs(tcur), real(1e-3)));
            else
                delta = delta == 0 ? fmax(fabs(tcur), real(1e-6)) : real(2) * delta;
            real target = tcur + sgn * delta;
            if (++nx > 80) {
                __syncwarp();
                *np = npts;
                return 0;
            }
            while (true) {
                real tS;
                int qS;
                nearest(&tS, &qS);
                if (!isfinite(tS) || !(sgn * (target - tS) > 0)) break;
                c += B * (double)(tS - tcur);
                tcur = tS;
                if (!point(tS)) return -1;
                pass(qS, tS);
            }
            c += B * (double)(target - tcur);
            tcur = target;
            if (!point(target)) return -1;
            while (true) {
                real tS;
                int qS;
                nearest(&tS, &qS);
                if (!(isfinite(tS) && tS == target)) break;
                pass(qS, target);
            }
            if (c - cmin > (double)M.maxnats) {
                __syncwarp();
                *np = npts;
                return 1;
            }
        }
    }

    // sample_line! (src/local.jl:1501) over both walks; *guard when a walk overflowed (t = 0)
    __device__ __noinline__ real sample_line(real ucat, real uoff, bool *guard) const {
        const int mp = SL.maxpts;
        real *pts = (real *)(base + SL.o_pts);
        real *pr = pts, *cr = pts + mp, *zr = pts + 2 * mp, *pl = pts + 3 * mp, *cl = pts + 4 * mp, *zl = pts + 5 * mp;
        real *lm = (real *)(base + SL.o_lm);
        *guard = false;
        int nr = 0, nl = 0;
        int w = walk(real(1), pr, cr, zr, &nr);
        if (w < 0) {
            *guard = true;
            return 0;
        }
        if (w == 0) return 0;
        w = walk(real(-1), pl, cl, zl, &nl);
        if (w < 0) {
            *guard = true;
            return 0;
        }
        if (w == 0) return 0;
        __syncwarp();
        auto Pm = [&](int i) -> real { return i < nl ? pl[nl - 1 - i] : (i == nl ? real(0) : pr[i - nl - 1]); };
        auto Cm = [&](int i) -> real { return i < nl ? cl[nl - 1 - i] : (i == nl ? real(0) : cr[i - nl - 1]); };
        auto Zm = [&](int i) -> real { return i < nl ? zl[nl - 1 - i] : (i == nl ? real(0) : zr[i - nl - 1]); };
        int nseg = nl + nr;
        real mx = -INFINITY;
        for (int j = lane; j < nseg; j += 32) {
            real p0 = Pm(j), p1 = Pm(j + 1), c0 = Cm(j), c1 = Cm(j + 1);
            real L = p1 - p0;
            real v = L > 0 ? -fmin(c0, c1) + Lane<real>::logseg(L, fabs(c1 - c0)) : real(-INFINITY);
            lm[j] = v;
            mx = fmax(mx, v);
        }
        mx = warp_max(mx);
        real totl = 0;
        for (int j = lane; j < nseg; j += 32) {
            real x = exp(lm[j] - mx);
            lm[j] = x;
            totl += x;
        }
        real tot = warp_sum(totl);
        __syncwarp();
        real u = ucat * tot, acc = 0;
        int jj = nseg - 1;
        for (int b0 = 0; b0 < nseg; b0 += 32) {
            int j = b0 + lane;
            real x = j < nseg ? lm[j] : real(0);
            real inc = acc + warp_incl_sum(x, lane);
            unsigned bb = __ballot_sync(0xffffffffu, j < nseg && u <= inc);
            if (bb) {
                jj = b0 + __ffs(bb) - 1;
                break;
            }
            acc = __shfl_sync(0xffffffffu, inc, 31);
        }
        real p0 = Pm(jj), p1 = Pm(jj + 1);
        real L = p1 - p0;
        real g = (Cm(jj + 1) - Cm(jj)) / L;
        real flat = Lane<real>::flat_nats;
        if constexpr (sizeof(real) == 4) {
            auto slope = [&](int j) -> real {
                if (j < 0 || j >= nseg) return 0;
                real Lj = Pm(j + 1) - Pm(j);
                return Lj > 0 ? fabs((Cm(j + 1) - Cm(j)) / Lj) : real(0);
            };
            real gl = slope(jj - 1), gm = slope(jj), gr = slope(jj + 1);
            real z0 = Zm(jj) + real(2.4e-7) * fabs(p0) * fmax(gl, gm);
            real z1 = Zm(jj + 1) + real(2.4e-7) * fabs(p1) * fmax(gm, gr);
            flat = fmax(flat, z0 + z1);
        }
        real t = (g >= 0 || fabs(g * L) < flat) ? p0 + Lane<real>::trexp_offset(uoff, g, L, flat)
                                                : p1 - Lane<real>::trexp_offset(uoff, -g, L, flat);
        __syncwarp();
        return t;
    }

    // commit (apply_step!, src/local.jl:2507): every unit's state of charge and its node balances
    __device__ void commit(real t) const {
        for (int q = lane; q < nu; q += 32) {
            int j = d.si[q];
            real x = t * d.sa[q];
            real k = M.kc_s[j], w = k + M.kappa0;
            real djw, dw, dja, da;
            soc_diff<real>(M.s_hours[j], M.s_qt[j], M.s_etain[j], M.s_etaout[j], M.s_mc[j], k, w, M.dt, M.c_viol,
                           U(SF_E0, q), U(SF_E1, q), x, real(0), &djw, &dw);
            soc_diff<real>(M.s_hours[j], M.s_qt[j], M.s_etain[j], M.s_etaout[j], M.s_mc[j], k, w, M.dt, M.c_viol,
                           U(SF_EM, q), U(SF_E0, q), real(0), x, &dja, &da);
            M.r[ix(d.nda[d.sposa[q]], taum)] += dja;
            M.e[ix(j, tau)] += x;
            M.r[ix(d.nds[d.spos[q]], tau)] += djw;
        }
    }
};

// Whether move descriptor d is separable with at least sepmin units (the cooperative walk's moves).
template <class real>
__device__ inline bool sep_move(const Desc<real> &d, int sepmin) {
    const int *h = d.hdr;
    bool sep = h[1] > 0 && h[0] == 0 && h[2] == 0 && h[3] == 0 && h[4] == 0 && h[6] == 0 && h[8] == 0 &&
               h[5] == h[1] && h[7] == h[1];
    return sepmin > 0 && h[12] >= 0 && sep && h[1] >= sepmin;
}

// Move mi of the class for every (step, replica) task when it is a separable move with at least
// sepmin units (else nothing: k_move runs it): one task per warp, taken from the per-move counter.
// The warps' walk buffers sit in dynamic shared memory after the descriptor (sep_smem = 1) or in
// per-warp slabs of gslab.
template <class real, int WPB>
__global__ void __launch_bounds__(32 * WPB)
    k_move_sep(const __grid_constant__ DevModel<real> M, const int *steps, int nsteps, const uint32_t *sweep_p, int mi,
               const char *descs, size_t stride, int sepmin, int sep_smem, char *gslab, unsigned long long *stats,
               unsigned int *next_item) {
    extern __shared__ __align__(16) char smem[];
    __shared__ Desc<real> sd;
    __shared__ SepLayout sSL;
    int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    if (threadIdx.x == 0) {
        // the header first: most moves are not this kernel's
        Desc<real> g = carve_desc<real>((char *)(descs + (size_t)mi * stride), M, M.natoms + M.nextra);
        sd.hdr = g.hdr;
    }
    __syncthreads();
    if (!sep_move<real>(sd, sepmin)) return;  // grid-uniform
    __syncthreads();
    {
        const int4 *src = (const int4 *)(descs + (size_t)mi * stride);
        int4 *dst = (int4 *)smem;
        for (size_t i = threadIdx.x; i < stride / 16; i += 32 * WPB) dst[i] = src[i];
    }
    if (threadIdx.x == 0) {
        sd = carve_desc<real>(smem, M, M.natoms + M.nextra);
        sSL = sep_layout<real>(M.maxstu, M.maxpts);
    }
    __syncthreads();
    const Desc<real> &d = sd;
    const SepLayout &SL = sSL;
    char *wbase = sep_smem ? smem + stride + (size_t)wib * SL.total
                           : gslab + ((size_t)blockIdx.x * WPB + wib) * (size_t)SL.total;
    SepWalk<real> W(M, d, SL, wbase, lane);
    uint32_t sweep = *sweep_p;
    unsigned long long tried = 0, moved = 0, guards = 0;
    int ntask = nsteps * M.R;
    int T = M.T;
    while (true) {
        unsigned int it = 0;
        if (lane == 0) it = atomicAdd(next_item, 1u);
        int task = (int)__shfl_sync(0xffffffffu, it, 0);
        if (task >= ntask) break;
        int q = task / M.R;
        W.rep = task % M.R;
        W.tau = steps[q];
        W.taum = (W.tau - 1 + T) % T;
        W.tau1 = (W.tau + 1) % T;
        W.load_units();
        double uc, uo;
        uniform2(M.seed, ESM_TAG_LANE, 2 * (uint32_t)mi, (uint32_t)W.tau, (uint32_t)W.rep, sweep, &uc, &uo);
        bool guard;
        real t = W.sample_line(unit_uniform<real>(uc), unit_uniform<real>(uo), &guard);
        if (guard) ++guards;
        if (t != 0) W.commit(t);
        if (M.mlog && W.rep < M.mlog_nrep && lane == 0)
            M.mlog[((size_t)mi * nsteps + q) * M.mlog_nrep + W.rep] = (double)t;
        ++tried;
        if (t != 0) ++moved;
        __syncwarp();
    }
    if (lane == 0) {
        int fi = ESM_NFAM;  // atoms
        if (tried) atomicAdd(&stats[2 * fi], tried);
        if (moved) atomicAdd(&stats[2 * fi + 1], moved);
        if (guards) atomicAdd(&stats[2 * (ESM_NFAM + 1)], guards);
    }
}

}  // namespace esm
