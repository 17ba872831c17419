// Storage multiscale sweep on the device: the plateau moves of storage_ms_sweep!
// (src/flowmoves.jl:255, prep_storage_ms! :187 without a shape). A move raises the state of charge
// of its units (one storage unit, or the units of one carrier in one country cell) by t at the
// instants b0+1 .. b0+L of a dyadic block, i.e. moves energy from step b0 to step b0+L; the power
// changes only at those two end steps, where the dispatch at the units' nodes follows pro rata
// (prorata!, src/local.jl:1782, with the requirement adjustment soc_qadj, :1826), with the Jacobian
// of logjac (:1871). Every step of the block has the units' storage terms and node balances.
//
// Mapping. The blocks of one length and parity are independent (they share no step); a class pass
// is one launch in which every thread takes (block, replica) tasks, replica fastest (coalesced
// state access), and runs the class's 8 moves in order. The move selections are state-independent
// and drawn on the host from the class stream, as the local sweep's move list is.
//
// Interior steps. At an interior step both state-of-charge values of a unit's storage term move by
// t, so while every moved value stays strictly inside (0, 1) the term's cost, injection and
// secondaries are exactly unchanged (clamp_diff keeps the change, d does not move). A unit's
// interior steps are therefore evaluated only outside that interval, whose ends are also the first
// primary breakpoints (the state-of-charge clamps) of the unit; the walk visits the same points
// as walk! over the whole block.
#pragma once
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "esm_common.cuh"
#include "esm_linemove.cuh"

namespace esm {

#define ESM_PLAT_RB 256   // roots between two walk points (beyond: the move is left, a guard event)
#define ESM_PLAT_LOCAL 4096  // reals of a thread's local scratch array; larger layouts use the global slab
#define ESM_PLAT_NACT 8   // listed steps per unit whose state lies outside the box (more: the unit is evaluated whole)

// per-lane scratch layout (reals)
struct PlatLayout {
    int pr, cr, zr, pl, cl, zl, lm, ro, gro;
    int slo, shi;                        // [U] clamp-free interval of the moved states inside the box
    int na, act;                         // [U] count, [U * NACT] interior steps touching a state outside the box
    int kv, kq, kg, kp, ke, knm, kph;    // [2U] compensation kink per (end, unit)
    int ka;                              // [2U * MAXK] kinked coefficient per (end, unit, disp unit)
    int dr;                              // [2U] node-balance change per (end, unit)
    int s3, p3;                          // [2U * 3] end storage secondaries, current / previous
    int sb, pb;                          // [2U] end node balances, current / previous
    int total;
};

__host__ __device__ inline PlatLayout plat_layout(int maxpts, int U) {
    PlatLayout L;
    int o = 0;
    L.pr = o; o += maxpts;
    L.cr = o; o += maxpts;
    L.zr = o; o += maxpts;
    L.pl = o; o += maxpts;
    L.cl = o; o += maxpts;
    L.zl = o; o += maxpts;
    L.lm = o; o += 2 * maxpts + 1;
    L.ro = o; o += ESM_PLAT_RB;
    L.gro = o; o += ESM_PLAT_RB;
    L.slo = o; o += U;
    L.shi = o; o += U;
    L.na = o; o += U;
    L.act = o; o += U * ESM_PLAT_NACT;
    L.kv = o; o += 2 * U;
    L.kq = o; o += 2 * U;
    L.kg = o; o += 2 * U;
    L.kp = o; o += 2 * U;
    L.ke = o; o += 2 * U;
    L.knm = o; o += 2 * U;
    L.kph = o; o += 2 * U;
    L.ka = o; o += 2 * U * ESM_PLAT_MAXK;
    L.dr = o; o += 2 * U;
    L.s3 = o; o += 6 * U;
    L.p3 = o; o += 6 * U;
    L.sb = o; o += 2 * U;
    L.pb = o; o += 2 * U;
    L.total = o;
    return L;
}

// COOP: the 32 lanes of a warp run one task together. Every lane runs the walk on its own copy of
// the scratch (identical contents), and the loops over the block's steps -- the clamp-free interval,
// the interior terms outside it, the breakpoint scan, the commit -- are split over the lanes and
// combined by reductions that every lane receives from lane 0, so the control flow stays uniform.
template <class real, bool COOP = false>
struct PLane {
    const DevModel<real> &M;
    const PlatLayout &LL;
    real *slab;
    int sstride;
    int L, b0, rep, U;
    bool lvl = false;  // the level move of the long-range sweep: every instant of the year rises, no end steps
    const int *uj;  // the move's storage units
    mutable real nzs = 0;
    int lane = 0;
    static constexpr int NL = COOP ? 32 : 1;
    __device__ inline real wsum(real v) const {
        if constexpr (COOP) {
            for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
            return __shfl_sync(0xffffffffu, v, 0);
        }
        return v;
    }
    __device__ inline real wmin(real v) const {
        if constexpr (COOP) {
            for (int o = 16; o > 0; o >>= 1) v = fmin(v, __shfl_xor_sync(0xffffffffu, v, o));
            return __shfl_sync(0xffffffffu, v, 0);
        }
        return v;
    }
    __device__ inline real wmax(real v) const {
        if constexpr (COOP) {
            for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
            return __shfl_sync(0xffffffffu, v, 0);
        }
        return v;
    }

    __device__ PLane(const DevModel<real> &M_, const PlatLayout &LL_, real *slab_, int sstride_)
        : M(M_), LL(LL_), slab(slab_), sstride(sstride_) {}

    __device__ inline real &S(int off, int i) const { return slab[(size_t)(off + i) * sstride]; }
    __device__ inline size_t ix(int x, int t) const { return sidx(x, t, rep, M.T, M.R); }
    __device__ inline int node(int u) const { return M.s_bus[uj[u]]; }
    // block positions: step b0 + q, cyclic (the long-range plateaus wrap); the interior terms (both
    // states raised) are q0() .. q0() + nq() - 1, the raised states q0() .. q0() + ns() - 1
    __device__ inline int cyc(int x) const { return x >= M.T ? x - M.T : x; }
    __device__ inline int stp(int q) const { return cyc(b0 + q); }
    __device__ inline int q0() const { return lvl ? 0 : 1; }
    __device__ inline int nq() const { return lvl ? M.T : L - 1; }
    __device__ inline int ns() const { return lvl ? M.T : L; }
    __device__ inline int tau_end(int s) const { return s == 0 ? stp(0) : stp(L); }
    // an interior term whose two states stay strictly inside (0, 1) at t is exactly unchanged
    __device__ inline bool quiet(int u, int q, real t) const {
        int tau = stp(q);
        real y0 = M.e[ix(uj[u], tau)], y1 = M.e[ix(uj[u], cyc(tau + 1))];
        return y0 > 0 && y0 < 1 && y1 > 0 && y1 < 1 && y0 + t > 0 && y0 + t < 1 && y1 + t > 0 && y1 + t < 1;
    }
    __device__ inline bool inside(int u, real t) const { return t > S(LL.slo, u) && t < S(LL.shi, u); }

    // storage term of unit u at block step q (0..L): the change of its cost; *dj the injection
    // change, *d1 the new d (src/energy.jl:448 soc_cost in difference form)
    __device__ __noinline__ real sterm(int u, int q, real t, real *dj, real *d1) const {
        int j = uj[u];
        int tau = stp(q);
        real k = M.kc_s[j];
        return soc_diff<real>(M.s_hours[j], M.s_qt[j], M.s_etain[j], M.s_etaout[j], M.s_mc[j], k, k + M.kappa0, M.dt,
                              M.c_viol, M.e[ix(j, tau)], M.e[ix(j, cyc(tau + 1))], (lvl || q >= 1) ? t : real(0),
                              (lvl || q + 1 <= L) ? t : real(0), dj, d1);
    }
    __device__ inline void sec3(int u, real d, real out[3]) const {
        real ein = M.s_etain[uj[u]];
        out[0] = d;
        out[1] = ein > 0 ? d - ein : real(1);
        out[2] = -d * M.s_etaout[uj[u]] - real(1);
    }

    // the compensation at the end steps (prorata! with soc_qadj), per (end, unit)
    __device__ __noinline__ void kinks() const {
        for (int s = 0; s < 2; ++s) {
            int tau = tau_end(s), t1 = (tau + 1) % M.T;
            for (int u = 0; u < U; ++u) {
                int i = s * U + u, n = node(u), j = uj[u];
                real ks = M.kc_s[j] * M.s_hours[j] / M.dt;
                real g = s == 0 ? ks : -ks;
                real Pm = 0, Qs = 0;
                int nv = 0, c = 0;
                for (int p = M.up[n]; p < M.up[n + 1] && c < ESM_PLAT_MAXK; ++p, ++c) {
                    int d = M.ua[p];
                    real kap = M.d_avail[d] * M.kc_d[d];
                    if (!(fabs(kap) >= M.kmin)) continue;
                    real om = M.g[ix(d, tau)];
                    Pm += kap * om;
                    Qs += kap * clampr<real>(om, 0, 1);
                    nv += 1;
                }
                bool valid = g != 0 && nv > 0 && !(fabs(Pm) < real(1e-6));
                // soc_qadj: nominal minus actual injection of the unit at its node
                real ye = M.e[ix(j, tau)], ye1 = M.e[ix(j, t1)];
                real ec = clampr<real>(ye, 0, 1), ec1 = clampr<real>(ye1, 0, 1);
                real dd = M.s_hours[j] * (ec1 - ec) / M.dt - M.s_qt[j];
                real pc = 0, mcx = 0;
                if (dd >= 0)
                    pc = M.s_etain[j] > 0 ? dd / M.s_etain[j] : real(0);
                else
                    mcx = fmin(-dd * M.s_etaout[j], real(1));
                real qadj = M.kc_s[j] * M.s_hours[j] * (ye1 - ye) / M.dt - M.kc_s[j] * (pc - mcx);
                real Q = M.r[ix(n, tau)] + Qs + qadj;
                S(LL.kv, i) = valid ? real(1) : real(0);
                S(LL.kq, i) = Q;
                S(LL.kg, i) = g;
                S(LL.kp, i) = valid ? Pm : real(1);
                S(LL.ke, i) = Pm - fmax(Q, real(0));
                S(LL.knm, i) = real(nv - 1);
                c = 0;
                for (int p = M.up[n]; p < M.up[n + 1] && c < ESM_PLAT_MAXK; ++p, ++c) {
                    int d = M.ua[p];
                    real kap = M.d_avail[d] * M.kc_d[d];
                    real ak = 0;
                    if (valid && fabs(kap) >= M.kmin) {
                        real sigma = kap * M.g[ix(d, tau)] / Pm;
                        if (sigma != 0) ak = sigma / kap;
                    }
                    S(LL.ka, i * ESM_PLAT_MAXK + c) = ak;
                }
            }
        }
    }

    // Per unit: the interval of t over which every moved state that lies strictly inside (0, 1)
    // stays inside, and the list of interior steps whose storage term involves a moved state outside
    // the box (a state of charge at or beyond a bound moves the term for every t). While t is in the
    // interval, the other interior terms are exactly unchanged. A unit with more than NACT such
    // steps gets an empty interval (evaluated whole).
    __device__ __noinline__ void intervals() const {
        for (int u = 0; u < U; ++u) {
            int j = uj[u];
            real mn = 2, mx = -1;
            int na = 0;
            bool over = false;
            auto list = [&](int qt) {  // an interior term involving a state outside the box
                for (int i = 0; i < na; ++i)
                    if (S(LL.act, u * ESM_PLAT_NACT + i) == real(qt)) return;
                if (na < ESM_PLAT_NACT)
                    S(LL.act, u * ESM_PLAT_NACT + na++) = real(qt);
                else
                    over = true;
            };
            auto out_state = [&](int q) {  // state q is the end value of term q - 1 and the start of term q
                if (lvl) {
                    list(q == 0 ? M.T - 1 : q - 1);
                    list(q);
                } else {
                    if (q - 1 >= 1) list(q - 1);
                    if (q <= L - 1) list(q);
                }
            };
            for (int base = 0; base < ns(); base += NL) {
                int p = base + lane, qo = -1;
                if (p < ns()) {
                    int q = q0() + p;
                    real y = M.e[ix(j, stp(q))];
                    if (y > 0 && y < 1) {
                        mn = fmin(mn, y);
                        mx = fmax(mx, y);
                    } else {
                        qo = q;
                    }
                }
                if constexpr (COOP) {  // the states outside the box, in step order, listed on every lane
                    unsigned bal = __ballot_sync(0xffffffffu, qo >= 0);
                    while (bal) {
                        int l = __ffs(bal) - 1;
                        bal &= bal - 1;
                        out_state(__shfl_sync(0xffffffffu, qo, l));
                    }
                } else if (qo >= 0) {
                    out_state(qo);
                }
            }
            mn = wmin(mn);
            mx = wmax(mx);
            bool ok = !over && mn <= mx;
            if (!over && mn > mx) {  // every raised state outside the box: no interval, terms listed
                S(LL.slo, u) = real(-INFINITY);
                S(LL.shi, u) = real(INFINITY);
            } else {
                S(LL.slo, u) = ok ? -mn : real(0);
                S(LL.shi, u) = ok ? real(1) - mx : real(0);
            }
            S(LL.na, u) = real(over ? 0 : na);
        }
    }

    // the interior step terms of unit u to evaluate at t: every one outside its interval, else the listed
    __device__ inline int nterms(int u, real t) const { return inside(u, t) ? (int)S(LL.na, u) : nq(); }
    __device__ inline int term_q(int u, real t, int i) const {
        return inside(u, t) ? (int)S(LL.act, u * ESM_PLAT_NACT + i) : q0() + i;
    }

    // mv_eval! of the block (src/local.jl:1219): beta * DeltaC(t); the end steps' secondaries into
    // s3/sb (the interior ones are evaluated where they change, in collect)
    __device__ __noinline__ real eval(real t) const {
        real dt = M.dt, cv = M.c_viol, k0 = M.kappa0;
        real D = 0, A = 0;
        for (int i = 0; i < 2 * U; ++i) {
            real Q = S(LL.kq, i);
            S(LL.kph, i) = S(LL.kv, i) != 0 ? fmax(Q + S(LL.kg, i) * t, real(0)) - fmax(Q, real(0)) : real(0);
            S(LL.dr, i) = 0;
        }
        for (int u = 0; u < U; ++u) {
            int n = node(u);
            for (int s = 0; s < (lvl ? 0 : 2); ++s) {  // end steps: storage term, kinked dispatch, node balance
                int i = s * U + u, q = s == 0 ? 0 : L, tau = tau_end(s);
                real dj, d1;
                real cs = sterm(u, q, t, &dj, &d1);
                D += cs;
                A += fabs(cs);
                real sc[3];
                sec3(u, d1, sc);
                for (int h = 0; h < 3; ++h) S(LL.s3, 3 * i + h) = sc[h];
                real dr = dj;
                real ph = S(LL.kph, i);
                int c = 0;
                for (int p = M.up[n]; p < M.up[n + 1] && c < ESM_PLAT_MAXK; ++p, ++c) {
                    real ak = S(LL.ka, i * ESM_PLAT_MAXK + c);
                    if (ak == 0) continue;
                    int d = M.ua[p];
                    real k = M.kc_d[d], Av = M.d_avail[d];
                    real dyc, dex;
                    clamp_diff<real>(M.g[ix(d, tau)], ak * ph, &dyc, &dex);
                    real dp = Av * k * dyc;
                    real cg = dt * M.d_mc[d] * dp + cv * dt * (k + k0) * dex;
                    D += cg;
                    A += fabs(cg);
                    dr -= dp;
                }
                S(LL.dr, i) = dr;
                real r0 = M.r[ix(n, tau)];
                real cb = dt * phibal_diff<real>(r0, dr, M.c_shed, M.c_dump);
                D += cb;
                A += fabs(cb);
                S(LL.sb, i) = r0 + dr;
            }
            int nt = nterms(u, t);
            bool in = inside(u, t);
            real Di = 0, Ai = 0;
            // interior steps: storage term and node balance (the listed ones on every lane; outside
            // the interval every term, split over the lanes)
            for (int i = in ? 0 : lane; i < nt; i += in ? 1 : NL) {
                int q = term_q(u, t, i);
                if (!in && quiet(u, q, t)) continue;
                real dj, d1;
                real cs = sterm(u, q, t, &dj, &d1);
                real cb = dt * phibal_diff<real>(M.r[ix(n, stp(q))], dj, M.c_shed, M.c_dump);
                Di += cs + cb;
                Ai += fabs(cs) + fabs(cb);
            }
            if (!in) {
                Di = wsum(Di);
                Ai = wsum(Ai);
            }
            D += Di;
            A += Ai;
        }
        if constexpr (sizeof(real) == 4) nzs = M.beta_v * A * real(4.8e-7);
        return M.beta_v * D;
    }

    __device__ __noinline__ void save_prev() const {
        for (int i = 0; i < 6 * U; ++i) S(LL.p3, i) = S(LL.s3, i);
        for (int i = 0; i < 2 * U; ++i) S(LL.pb, i) = S(LL.sb, i);
    }

    __device__ static inline bool root_of(real a, real b, real lo, real hi, real sgn, real *x) {
        if ((a < 0) != (b < 0) && a != b) {
            real xx = lo + (hi - lo) * a / (a - b);
            if (sgn * (xx - lo) > 0 && sgn * (hi - xx) > 0) {
                *x = xx;
                return true;
            }
        }
        return false;
    }
    __device__ inline bool add_root(int off, int *n, real x) const {
        if (*n >= ESM_PLAT_RB) return false;
        S(off, (*n)++) = x;
        return true;
    }

    // sign changes of the secondaries between prev (at lo) and cur (at hi): storage ones into gro
    // (when storage splitting applies), node balances into ro; interior steps of the units whose
    // states leave their interval in [lo, hi]
    __device__ __noinline__ bool collect(real lo, real hi, real sgn, bool want_stor, bool want_other, int *nro, int *ngro) const {
        real x;
        for (int i = 0; i < 2 * U; ++i) {
            if (want_stor)
                for (int h = 0; h < 3; ++h)
                    if (root_of(S(LL.p3, 3 * i + h), S(LL.s3, 3 * i + h), lo, hi, sgn, &x) && !add_root(LL.gro, ngro, x))
                        return false;
            if (want_other && root_of(S(LL.pb, i), S(LL.sb, i), lo, hi, sgn, &x) && !add_root(LL.ro, nro, x))
                return false;
        }
        for (int u = 0; u < U; ++u) {
            bool in = inside(u, lo) && inside(u, hi);
            int n = node(u);
            int nt = in ? (int)S(LL.na, u) : nq();
            // the listed terms on every lane; outside the interval every term, split over the lanes in
            // rounds of NL terms, whose roots every lane adds in term order
            int step = in ? 1 : NL;
            for (int base = 0; base < nt; base += step) {
                int i = in ? base : base + lane;
                real rg[3] = {0, 0, 0}, rr = 0;
                int ng = 0;
                bool hr = false;
                if (i < nt) {
                    int q = in ? (int)S(LL.act, u * ESM_PLAT_NACT + i) : q0() + i;
                    if (in || !(quiet(u, q, lo) && quiet(u, q, hi))) {
                        real dja, d1a, djb, d1b;
                        sterm(u, q, lo, &dja, &d1a);
                        sterm(u, q, hi, &djb, &d1b);
                        if (want_stor) {
                            real a3[3], b3[3];
                            sec3(u, d1a, a3);
                            sec3(u, d1b, b3);
                            for (int h = 0; h < 3; ++h)
                                if (root_of(a3[h], b3[h], lo, hi, sgn, &x)) rg[ng++] = x;
                        }
                        if (want_other) {
                            real r0 = M.r[ix(n, stp(q))];
                            if (root_of(r0 + dja, r0 + djb, lo, hi, sgn, &x)) {
                                rr = x;
                                hr = true;
                            }
                        }
                    }
                }
                bool ok = true;
                if (COOP && !in) {
                    unsigned bal = __ballot_sync(0xffffffffu, ng > 0 || hr);
                    while (bal) {
                        int l = __ffs(bal) - 1;
                        bal &= bal - 1;
                        int nl = __shfl_sync(0xffffffffu, ng, l);
                        for (int h = 0; h < 3; ++h) {
                            real xs = __shfl_sync(0xffffffffu, rg[h], l);
                            if (h < nl) ok = add_root(LL.gro, ngro, xs) && ok;
                        }
                        bool hl = __shfl_sync(0xffffffffu, hr, l);
                        real xr = __shfl_sync(0xffffffffu, rr, l);
                        if (hl) ok = add_root(LL.ro, nro, xr) && ok;
                    }
                } else {
                    for (int h = 0; h < ng; ++h) ok = add_root(LL.gro, ngro, rg[h]) && ok;
                    if (hr) ok = add_root(LL.ro, nro, rr) && ok;
                }
                if (!ok) return false;
            }
        }
        return true;
    }

    __device__ __noinline__ void sort_buf(int off, int n, real sgn) const {
        for (int i = 1; i < n; ++i) {
            real x = S(off, i);
            int j = i - 1;
            while (j >= 0 && (sgn > 0 ? x < S(off, j) : x > S(off, j))) {
                S(off, j + 1) = S(off, j);
                --j;
            }
            S(off, j + 1) = x;
        }
    }

    // next primary breakpoint beyond tp (finalize! of every step, scanned): the kink points, the
    // clamps of the kinked dispatch, the clamps of the moved states of charge
    __device__ __noinline__ bool next_bp(real tp, real sgn, real *out) const {
        bool have = false;
        real best = 0;
        auto consider = [&](real x) {
            if (!isfinite(x)) return;
            if (!(sgn * x > 0)) return;
            if (!(sgn * (x - tp) > 0)) return;
            if (!have || sgn * (x - best) < 0) {
                best = x;
                have = true;
            }
        };
        for (int i = 0; i < (lvl ? 0 : 2 * U); ++i) {
            if (S(LL.kv, i) == 0) continue;
            real g = S(LL.kg, i), Q = S(LL.kq, i);
            consider(-Q / g);
            int u = i % U, s = i / U, n = node(u), tau = tau_end(s);
            int c = 0;
            for (int p = M.up[n]; p < M.up[n + 1] && c < ESM_PLAT_MAXK; ++p, ++c) {
                real ak = S(LL.ka, i * ESM_PLAT_MAXK + c);
                if (ak == 0) continue;
                real y0 = M.g[ix(M.ua[p], tau)];
                real offs[4] = {real(0), real(0), -ak * Q, ak * Q};
                real sls[4] = {ak * g, real(0), real(0), ak * g};
                for (int h = 0; h < 4; ++h) {
                    if (sls[h] == 0) continue;
                    consider((real(0) - y0 - offs[h]) / sls[h]);
                    consider((real(1) - y0 - offs[h]) / sls[h]);
                }
            }
        }
        for (int u = 0; u < U; ++u) {
            int j = uj[u];
            if (tp > S(LL.slo, u) && tp < S(LL.shi, u) && S(LL.slo, u) < S(LL.shi, u)) {
                // the nearest clamp of the states inside the box, then the clamps of the states
                // outside it (each a state of a listed term)
                consider(sgn > 0 ? S(LL.shi, u) : S(LL.slo, u));
                int na = (int)S(LL.na, u);
                for (int i = 0; i < na; ++i) {
                    int q = (int)S(LL.act, u * ESM_PLAT_NACT + i);
                    for (int h = 0; h < 2; ++h) {
                        real y0 = M.e[ix(j, cyc(stp(q) + h))];
                        if (y0 > 0 && y0 < 1) continue;
                        consider(real(0) - y0);
                        consider(real(1) - y0);
                    }
                }
                continue;
            }
            for (int p = lane; p < ns(); p += NL) {
                real y0 = M.e[ix(j, stp(q0() + p))];
                consider(real(0) - y0);
                consider(real(1) - y0);
            }
        }
        if constexpr (COOP) {  // the nearest candidate over the lanes (a sign flip is exact)
            real key = wmin(have ? sgn * best : real(INFINITY));
            have = key < real(INFINITY);
            best = have ? sgn * key : real(0);
        }
        *out = best;
        return have;
    }

    __device__ inline void push(int pofs, int cofs, int *np, real x, real c, real z) const {
        S(pofs, *np) = x;
        S(cofs, *np) = c;
        if constexpr (sizeof(real) == 4) S(pofs == LL.pr ? LL.zr : LL.zl, *np) = z;
        ++*np;
    }

    __device__ __noinline__ bool piece_roots(int pofs, int cofs, int *np, real a, real b, real sgn, real *cmin) const {
        int nro = 0, ngro = 0;
        if (!collect(a, b, sgn, false, true, &nro, &ngro)) return false;
        if (nro == 0) return true;
        sort_buf(LL.ro, nro, sgn);
        for (int i = 0; i < nro; ++i) {
            real x = S(LL.ro, i);
            real cx = eval(x);
            if (*np >= M.maxpts) return false;
            push(pofs, cofs, np, x, cx, nzs);
            *cmin = fmin(*cmin, cx);
        }
        return true;
    }

    // walk! (src/local.jl:1294) with storage splitting; 1 proper, 0 improper, -1 buffer overflow
    __device__ __noinline__ int walk(int pofs, int cofs, int *np, real sgn) const {
        real tp = 0, cmin = 0, delta = 0;
        int nx = 0;
        *np = 0;
        eval(real(0));
        save_prev();
        while (true) {
            real t;
            if (!next_bp(tp, sgn, &t)) {
                real cprev = *np == 0 ? real(0) : S(cofs, *np - 1);
                real hp = real(sizeof(real) == 4 ? 1e-3 : 1e-6) * fmax(real(1), fabs(tp));
                real sl = (eval(tp + sgn * hp) + real(0) - cprev - real(0)) / hp;
                if (sl > 0)
                    delta = fmin(real(2) * M.maxnats / sl, real(1e3) * fmax(fabs(tp), real(1e-3)));
                else
                    delta = delta == 0 ? fmax(fabs(tp), real(1e-6)) : real(2) * delta;
                t = tp + sgn * delta;
                nx += 1;
                if (nx > 80) return 0;
            }
            real c = eval(t), zc = nzs;
            int nro = 0, ngro = 0;
            if (!collect(tp, t, sgn, true, false, &nro, &ngro)) return -1;
            if (ngro > 0) {
                sort_buf(LL.gro, ngro, sgn);
                real a0 = tp;
                for (int i = 0; i < ngro; ++i) {
                    real x = S(LL.gro, i);
                    real cx = eval(x), zx = nzs;
                    if (!piece_roots(pofs, cofs, np, a0, x, sgn, &cmin)) return -1;
                    eval(x);
                    if (*np >= M.maxpts) return -1;
                    push(pofs, cofs, np, x, cx, zx);
                    cmin = fmin(cmin, cx);
                    save_prev();
                    a0 = x;
                }
                eval(t);
                if (!piece_roots(pofs, cofs, np, a0, t, sgn, &cmin)) return -1;
                eval(t);
                save_prev();
            } else {
                if (!collect(tp, t, sgn, false, true, &nro, &ngro)) return -1;
                save_prev();
                if (nro > 0) {
                    sort_buf(LL.ro, nro, sgn);
                    for (int i = 0; i < nro; ++i) {
                        real x = S(LL.ro, i);
                        real cx = eval(x);
                        if (*np >= M.maxpts) return -1;
                        push(pofs, cofs, np, x, cx, nzs);
                        cmin = fmin(cmin, cx);
                    }
                }
            }
            if (*np >= M.maxpts) return -1;
            push(pofs, cofs, np, t, c, zc);
            cmin = fmin(cmin, c);
            if (c + real(0) - cmin > M.maxnats) return 1;
            tp = t;
        }
    }

    __device__ static real logseg(real Ls, real x) {
        if (fabs(x) < real(1e-10)) return log(Ls) - x / 2;
        if (x > 0) return log(Ls) + log(-expm1(-x)) - log(x);
        return log(Ls) - x + log(-expm1(x)) - log(-x);
    }
    __device__ static real trexp_offset(real u, real g, real Ls, real flat) {
        real x = g * Ls;
        if (fabs(x) < flat) return u * Ls;
        if (g > 0) return -log1p(-u * (-expm1(-x))) / g;
        return Ls + log1p(-u * (-expm1(x))) / (-g);
    }
    __device__ inline real P(int i, int nl) const {
        return i < nl ? S(LL.pl, nl - 1 - i) : (i == nl ? real(0) : S(LL.pr, i - nl - 1));
    }
    __device__ inline real Cc(int i, int nl) const {
        return i < nl ? S(LL.cl, nl - 1 - i) : (i == nl ? real(0) : S(LL.cr, i - nl - 1));
    }
    __device__ inline real Zz(int i, int nl) const {
        return i < nl ? S(LL.zl, nl - 1 - i) : (i == nl ? real(0) : S(LL.zr, i - nl - 1));
    }

    // sample_line! (src/local.jl:1501), as Lane::sample_line
    __device__ __noinline__ real sample_line(real ucat, real uoff, bool *guard) const {
        *guard = false;
        int nr = 0, nl = 0;
        int w = walk(LL.pr, LL.cr, &nr, real(1));
        if (w < 0) {
            *guard = true;
            return 0;
        }
        if (w == 0) return 0;
        w = walk(LL.pl, LL.cl, &nl, real(-1));
        if (w < 0) {
            *guard = true;
            return 0;
        }
        if (w == 0) return 0;
        int nseg = nl + nr;
        real mx = -INFINITY;
        for (int j = 0; j < nseg; ++j) {
            real p0 = P(j, nl), p1 = P(j + 1, nl), c0 = Cc(j, nl), c1 = Cc(j + 1, nl);
            real Ls = p1 - p0;
            real lm = Ls > 0 ? -fmin(c0, c1) + logseg(Ls, fabs(c1 - c0)) : real(-INFINITY);
            S(LL.lm, j) = lm;
            mx = fmax(mx, lm);
        }
        real tot = 0;
        for (int j = 0; j < nseg; ++j) tot += exp(S(LL.lm, j) - mx);
        real u = ucat * tot, acc = 0;
        int jj = nseg - 1;
        for (int q = 0; q < nseg; ++q) {
            acc += exp(S(LL.lm, q) - mx);
            if (u <= acc) {
                jj = q;
                break;
            }
        }
        real p0 = P(jj, nl), p1 = P(jj + 1, nl);
        real Ls = p1 - p0;
        real g = (Cc(jj + 1, nl) - Cc(jj, nl)) / Ls;
        real flat = sizeof(real) == 4 ? real(1e-4) : real(1e-10);
        if constexpr (sizeof(real) == 4) {
            auto slope = [&](int j) -> real {
                if (j < 0 || j >= nseg) return 0;
                real Lj = P(j + 1, nl) - P(j, nl);
                return Lj > 0 ? fabs((Cc(j + 1, nl) - Cc(j, nl)) / Lj) : real(0);
            };
            real gl = slope(jj - 1), gm = slope(jj), gr = slope(jj + 1);
            real z0 = Zz(jj, nl) + real(2.4e-7) * fabs(p0) * fmax(gl, gm);
            real z1 = Zz(jj + 1, nl) + real(2.4e-7) * fabs(p1) * fmax(gm, gr);
            flat = fmax(flat, z0 + z1);
        }
        return (g >= 0 || fabs(g * Ls) < flat) ? p0 + trexp_offset(uoff, g, Ls, flat)
                                               : p1 - trexp_offset(uoff, -g, Ls, flat);
    }

    // logjac (src/local.jl:1871) of the compensations, in FP64 in both builds (the log-acceptance
    // ratio is an FP64 quantity; its inputs are the build's values)
    __device__ double logjac(real t, bool *any) const {
        double lj = 0;
        *any = false;
        for (int i = 0; i < (lvl ? 0 : 2 * U); ++i) {
            if (S(LL.kv, i) == 0) continue;
            *any = true;
            double Q = S(LL.kq, i);
            lj += (double)S(LL.knm, i) *
                  log(fabs((fmax(Q + (double)S(LL.kg, i) * (double)t, 0.0) + (double)S(LL.ke, i)) / (double)S(LL.kp, i)));
        }
        return lj;
    }

    // commit_block! (src/local.jl:2495): states of charge, kinked dispatch, node balances (each
    // global write by one lane)
    __device__ __noinline__ void commit(real t) const {
        eval(t);
        for (int u = 0; u < U; ++u) {
            int n = node(u);
            for (int s = 0; s < (lvl ? 0 : 2); ++s) {  // end steps: the compensation and the node balance
                if (lane != 0) break;
                int i = s * U + u, tau = tau_end(s);
                real ph = S(LL.kph, i);
                int c = 0;
                for (int p = M.up[n]; p < M.up[n + 1] && c < ESM_PLAT_MAXK; ++p, ++c) {
                    real ak = S(LL.ka, i * ESM_PLAT_MAXK + c);
                    if (ak != 0) M.g[ix(M.ua[p], tau)] += ak * ph;
                }
                M.r[ix(n, tau)] += S(LL.dr, i);
            }
            int nt = nterms(u, t);  // interior steps whose injection changes
            bool in = inside(u, t);
            for (int i = lane; i < nt; i += NL) {
                int q = term_q(u, t, i);
                if (!in && quiet(u, q, t)) continue;
                real dj, d1;
                sterm(u, q, t, &dj, &d1);
                M.r[ix(n, stp(q))] += dj;
            }
        }
        for (int u = 0; u < U; ++u)
            for (int p = lane; p < ns(); p += NL) M.e[ix(uj[u], stp(q0() + p))] += t;
        if constexpr (COOP) __syncwarp();
    }
};

// One class pass of the storage multiscale sweep: threads take (block, replica) tasks (replica
// fastest) and run the class's moves in order. COOP: one warp per task (long blocks, whose moves
// loop over up to 128 steps and whose passes have few tasks).
template <class real, bool COOP>
__global__ void __launch_bounds__(128, 8) k_plateau(const __grid_constant__ DevModel<real> M,
                                                 const __grid_constant__ PlatMoves mv, uint32_t sweep,
                                                 real *scratch, unsigned long long *stats) {
    PlatLayout LL = plat_layout(M.maxpts, ESM_PLAT_MAXU);
    real local[ESM_PLAT_LOCAL];
    size_t gid = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    size_t nthr = (size_t)gridDim.x * blockDim.x;
    bool loc = LL.total <= ESM_PLAT_LOCAL;
    real *slab = loc ? local : scratch + gid;
    PLane<real, COOP> Ln(M, LL, slab, loc ? 1 : (int)nthr);
    Ln.lane = COOP ? (int)(threadIdx.x & 31) : 0;
    Ln.L = mv.L;
    unsigned long long tried = 0, moved = 0, guards = 0;
    size_t ntask = (size_t)mv.nb * M.R;
    size_t t0 = COOP ? gid >> 5 : gid, ts = COOP ? nthr >> 5 : nthr;
    for (size_t task = t0; task < ntask; task += ts) {
        int k = (int)(task / M.R);
        Ln.rep = (int)(task % M.R);
        Ln.b0 = mv.o + (2 * k + mv.cls) * mv.L;
        for (int m = 0; m < 8; ++m) {
            Ln.U = mv.nu[m];
            Ln.uj = mv.j[m];
            if (Ln.U <= 0) continue;
            Ln.intervals();
            Ln.kinks();
            uint32_t w0 = 2u * (8u * (uint32_t)mv.li + (uint32_t)m);
            double uc, uo, uj, un;
            uniform2(M.seed, ESM_TAG_SML, w0, (uint32_t)Ln.b0, (uint32_t)Ln.rep, sweep, &uc, &uo);
            bool guard;
            real t = Ln.sample_line(unit_uniform<real>(uc), unit_uniform<real>(uo), &guard);
            if (guard) ++guards;
            if (t != 0) {
                bool any;
                double lj = Ln.logjac(t, &any);
                if (any) {
                    uniform2(M.seed, ESM_TAG_SML, w0 + 1, (uint32_t)Ln.b0, (uint32_t)Ln.rep, sweep, &uj, &un);
                    if (uj >= exp(fmin(0.0, lj))) t = 0;
                }
            }
            if (t != 0) Ln.commit(t);
            ++tried;
            if (t != 0) ++moved;
        }
    }
    if (Ln.lane == 0) {
        if (tried) atomicAdd(&stats[0], tried);
        if (moved) atomicAdd(&stats[1], moved);
        if (guards) atomicAdd(&stats[2], guards);
    }
}

// The long-range storage sweep (storage_long_sweep!, src/storage_long.jl:245): threads take (unit,
// replica) tasks and run the unit's moves in order -- the level move (every instant of the year
// rises) and the long-range plateaus (prep_slong!, :77: one unit, the cyclic instants a+1 .. a+L,
// compensation at steps a and a+L). plan: per unit [stor index, moves, (L, a) per move]; L = T is the
// level move. The moves of different units touch different nodes (one unit per node and carrier).
template <class real>
__global__ void __launch_bounds__(128, 8) k_storage_long(const __grid_constant__ DevModel<real> M, const int *plan,
                                                        int nunits, uint32_t sweep, real *scratch,
                                                        unsigned long long *stats) {
    PlatLayout LL = plat_layout(M.maxpts, ESM_PLAT_MAXU);
    real local[ESM_PLAT_LOCAL];
    size_t gid = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    size_t nthr = (size_t)gridDim.x * blockDim.x;
    bool loc = LL.total <= ESM_PLAT_LOCAL;
    real *slab = loc ? local : scratch + gid;
    PLane<real, true> Ln(M, LL, slab, loc ? 1 : (int)nthr);  // one warp per task
    Ln.lane = threadIdx.x & 31;
    unsigned long long tried = 0, moved = 0, guards = 0;
    size_t ntask = (size_t)nunits * M.R;
    for (size_t task = gid >> 5; task < ntask; task += nthr >> 5) {
        const int *pu = plan + (task / M.R) * ESM_SL_STRIDE;
        Ln.rep = (int)(task % M.R);
        Ln.U = 1;
        Ln.uj = pu;
        for (int m = 0; m < pu[1]; ++m) {
            int L = pu[2 + 2 * m], a = pu[3 + 2 * m];
            Ln.lvl = L >= M.T;
            Ln.L = Ln.lvl ? M.T : L;
            Ln.b0 = Ln.lvl ? 0 : a;
            Ln.intervals();
            if (!Ln.lvl) Ln.kinks();
            double uc, uo, uj, un;
            uniform2(M.seed, ESM_TAG_SLL, 2u * (uint32_t)m, (uint32_t)pu[0], (uint32_t)Ln.rep, sweep, &uc, &uo);
            bool guard;
            real t = Ln.sample_line(unit_uniform<real>(uc), unit_uniform<real>(uo), &guard);
            if (guard) ++guards;
            if (t != 0 && !Ln.lvl) {
                bool any;
                double lj = Ln.logjac(t, &any);
                if (any) {
                    uniform2(M.seed, ESM_TAG_SLL, 2u * (uint32_t)m + 1, (uint32_t)pu[0], (uint32_t)Ln.rep, sweep, &uj,
                             &un);
                    if (uj >= exp(fmin(0.0, lj))) t = 0;
                }
            }
            if (t != 0) Ln.commit(t);
            if (M.mlog && Ln.rep < M.mlog_nrep && Ln.lane == 0)
                M.mlog[((task / M.R) * 5 + m) * M.mlog_nrep + Ln.rep] = (double)t;
            ++tried;
            if (t != 0) ++moved;
        }
    }
    if (Ln.lane == 0) {
        if (tried) atomicAdd(&stats[0], tried);
        if (moved) atomicAdd(&stats[1], moved);
        if (guards) atomicAdd(&stats[2], guards);
    }
}

template <class real>
cudaError_t launch_storage_long(const DevModel<real> &M, const int *plan, int nunits, uint32_t sweep, real *scratch,
                                int threads, unsigned long long *stats, cudaStream_t s) {
    size_t nthr = (size_t)nunits * M.R * 32;  // one warp per (unit, replica) task
    int blocks = (int)(((size_t)threads < nthr ? (size_t)threads : nthr) + 127) / 128;
    k_storage_long<real><<<blocks, 128, 0, s>>>(M, plan, nunits, sweep, scratch, stats);
    return cudaGetLastError();
}

// threads of k_plateau resident on the device, and the global scratch it needs per thread (0: the
// local array suffices)
template <class real>
int plateau_threads(const DevModel<real> &M) {
    int nb = 0, dev = 0, nsm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_plateau<real, false>, 128, 0) != cudaSuccess || nb < 1)
        nb = 4;
    return nb * nsm * 128;
}
template <class real>
size_t plateau_scratch_reals(const DevModel<real> &M) {
    PlatLayout LL = plat_layout(M.maxpts, ESM_PLAT_MAXU);
    return LL.total <= ESM_PLAT_LOCAL ? 0 : (size_t)LL.total;
}
template <class real>
cudaError_t launch_plateau(const DevModel<real> &M, const PlatMoves &mv, uint32_t sweep, real *scratch, int threads,
                           unsigned long long *stats, cudaStream_t s) {
    bool coop = mv.L >= 32;  // long blocks: one warp per task
    size_t nthr = (size_t)mv.nb * M.R * (coop ? 32 : 1);
    int blocks = (int)(((size_t)threads < nthr ? (size_t)threads : nthr) + 127) / 128;
    if (coop)
        k_plateau<real, true><<<blocks, 128, 0, s>>>(M, mv, sweep, scratch, stats);
    else
        k_plateau<real, false><<<blocks, 128, 0, s>>>(M, mv, sweep, scratch, stats);
    return cudaGetLastError();
}

}  // namespace esm
