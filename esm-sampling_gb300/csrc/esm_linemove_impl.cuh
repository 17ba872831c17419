// Line-move kernels: the exact line-conditional dispatch moves of one parity class of the local
// sweep (src/local.jl:1927 local_sweep!, the threaded body :1954-2051) for every replica.
//
// Mapping. All (step, replica) tasks of a class run the same move list (the move selection reads
// only capacities and static tables, src/local.jl:14 "selection uses only (k, x)"), so a move's
// structure -- entries, lines, touched nodes, storage terms -- is the same for every task and is
// built once per class pass (k_prep_moves). k_move then runs one move for every task: a warp owns
// 32 tasks of a tile (span consecutive steps x replicas, replica fastest, so that every state
// access of the warp is one coalesced 128-byte line of the (X, T, R) arrays), and each lane walks
// its own piecewise-exponential line conditional (walk!, src/local.jl:1294) and draws t
// (sample_line!, :1501) with its own uniforms. Per-lane walk buffers live in a local array when
// they fit it, else in a per-block global slab interleaved by lane.
#pragma once
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "esm_common.cuh"
#include "esm_linemove.cuh"

namespace esm {

// ---------------------------------------------------------------------------------------------
// shared-memory descriptor of the current move of a warp
// ---------------------------------------------------------------------------------------------
struct Carve {
    char *p;
    __host__ __device__ explicit Carve(char *b) : p(b) {}
    template <class U>
    __host__ __device__ U *take(int n) {
        size_t a = (size_t)p;
        a = (a + 15) & ~(size_t)15;
        U *out = (U *)a;
        p = (char *)(a + sizeof(U) * (size_t)(n > 0 ? n : 1));
        return out;
    }
};

template <class real>
struct Desc {
    int *moves;
    int *hdr;  // [0] ng, [1] nse, [2] nl, [3] nk, [4] nku, [5] nns, [6] nga, [7] nna, [8] nth, [9] valid, [10] fam,
               // [11] nku0 (the kinked units of step tau; those of step tau - 1 follow)
    int *gi, *gpos;
    real *ga;
    int *si, *spos, *sposa;
    real *sa;
    int *thn;
    real *tha;
    int *li, *lpa, *lpb;
    real *ldf;
    int *kn;
    real *kg;
    int *ku, *kk, *kupos;
    real *kda;  // direct coefficient of a kinked unit that the move also moves directly (else 0)
    int *ksd;   // step of a kink: 0 tau, 1 tau - 1
    int *kqs;   // storage unit whose requirement adjustment (soc_qadj) enters the kink, or -1
    int *nds, *nda;
    int *gia, *gposa;
    real *gaa;
    real *dth;
    unsigned char *lmark, *nmarks, *nmarka;
    int *posn_s, *posn_a;  // node -> position in the node lists (-1)
};

template <class real>
__host__ __device__ inline Desc<real> carve_desc(char *base, const DevModel<real> &M, int nmoves) {
    Carve c(base);
    Desc<real> d;
    d.moves = c.take<int>(nmoves);
    d.hdr = c.take<int>(16);
    d.gi = c.take<int>(M.maxe);
    d.gpos = c.take<int>(M.maxe);
    d.ga = c.take<real>(M.maxe);
    d.si = c.take<int>(M.maxstu);
    d.spos = c.take<int>(M.maxstu);
    d.sposa = c.take<int>(M.maxstu);
    d.sa = c.take<real>(M.maxstu);
    d.thn = c.take<int>(M.N);
    d.tha = c.take<real>(M.N);
    d.li = c.take<int>(M.L);
    d.lpa = c.take<int>(M.L);
    d.lpb = c.take<int>(M.L);
    d.ldf = c.take<real>(M.L);
    d.kn = c.take<int>(M.maxk);
    d.kg = c.take<real>(M.maxk);
    d.ku = c.take<int>(M.maxku);
    d.kk = c.take<int>(M.maxku);
    d.kupos = c.take<int>(M.maxku);
    d.kda = c.take<real>(M.maxku);
    d.ksd = c.take<int>(M.maxk);
    d.kqs = c.take<int>(M.maxk);
    d.nds = c.take<int>(M.N);
    d.nda = c.take<int>(M.N);
    d.gia = c.take<int>(4);
    d.gposa = c.take<int>(4);
    d.gaa = c.take<real>(4);
    d.dth = c.take<real>(M.N);
    d.lmark = c.take<unsigned char>(M.L);
    d.nmarks = c.take<unsigned char>(M.N);
    d.nmarka = c.take<unsigned char>(M.N);
    d.posn_s = c.take<int>(M.N);
    d.posn_a = c.take<int>(M.N);
    return d;
}

template <class real>
size_t desc_bytes(const DevModel<real> &M, int nmoves) {
    // size by carving from an aligned base
    char *base = (char *)(uintptr_t)4096;
    Carve c(base);
    c.take<int>(nmoves);
    c.take<int>(16);
    c.take<int>(M.maxe);
    c.take<int>(M.maxe);
    c.take<real>(M.maxe);
    c.take<int>(M.maxstu);
    c.take<int>(M.maxstu);
    c.take<int>(M.maxstu);
    c.take<real>(M.maxstu);
    c.take<int>(M.N);
    c.take<real>(M.N);
    c.take<int>(M.L);
    c.take<int>(M.L);
    c.take<int>(M.L);
    c.take<real>(M.L);
    c.take<int>(M.maxk);
    c.take<real>(M.maxk);
    c.take<int>(M.maxku);
    c.take<int>(M.maxku);
    c.take<int>(M.maxku);
    c.take<real>(M.maxku);
    c.take<int>(M.maxk);
    c.take<int>(M.maxk);
    c.take<int>(M.N);
    c.take<int>(M.N);
    c.take<int>(4);
    c.take<int>(4);
    c.take<real>(4);
    c.take<real>(M.N);
    c.take<unsigned char>(M.L);
    c.take<unsigned char>(M.N);
    c.take<unsigned char>(M.N);
    c.take<int>(M.N);
    c.take<int>(M.N);
    return (size_t)(c.p - base) + 16;
}

// per-lane scratch layout (reals), interleaved by lane within a warp slab
struct LaneLayout {
    int pr, cr, pl, cl, lm, drs, dra, sps, spa, dcs, dca, dps, dpa, ro, gro, kq, ke, kp, knm, kph, kv, kua;
    int ut, uk, usl, ue, un, uh, ui, hk, hu, ufe, ufn, usw, usa, zr, zl, total;
    int maxroots;  // capacity of the root buffers ro and gro
};
// sign changes one segment of a walk can hold: every touched node's balance at both steps and the
// three storage secondaries of every storage term at both steps
template <class real>
__host__ __device__ inline int linemove_maxroots(const DevModel<real> &M) {
    return 2 * M.maxn + 6 * M.maxstu;
}

__host__ __device__ inline LaneLayout lane_layout(int maxpts, int maxn, int maxstu, int maxroots, int maxk, int maxku) {
    LaneLayout L;
    int o = 0;
    L.pr = o; o += maxpts;
    L.cr = o; o += maxpts;
    L.pl = o; o += maxpts;
    L.cl = o; o += maxpts;
    L.lm = o; o += 2 * maxpts + 1;
    L.drs = o; o += maxn;
    L.dra = o; o += maxn;
    L.sps = o; o += maxn;
    L.spa = o; o += maxn;
    L.dcs = o; o += maxstu;
    L.dca = o; o += maxstu;
    L.dps = o; o += maxstu;
    L.dpa = o; o += maxstu;
    L.maxroots = maxroots;
    L.ro = o; o += maxroots;
    L.gro = o; o += maxroots;
    L.kq = o; o += maxk;
    L.ke = o; o += maxk;
    L.kp = o; o += maxk;
    L.knm = o; o += maxk;
    L.kph = o; o += maxk;
    L.kv = o; o += maxk;
    L.kua = o; o += maxku;
    L.ut = o; o += maxstu;
    L.uk = o; o += maxstu;
    L.usl = o; o += maxstu;
    L.ue = o; o += 3 * maxstu;
    L.un = o; o += maxstu;
    L.uh = o; o += maxstu;
    L.ui = o; o += maxstu;
    L.hk = o; o += maxstu;
    L.hu = o; o += maxstu;
    L.ufe = o; o += maxstu;
    L.ufn = o; o += maxstu;
    L.usw = o; o += maxstu;
    L.usa = o; o += maxstu;
    L.zr = o; o += maxpts;
    L.zl = o; o += maxpts;
    L.total = o;
    return L;
}

// reals of a lane's local scratch array (16 KB in FP32); larger layouts use the global slab
#define ESM_LANE_LOCAL 4096

// ---------------------------------------------------------------------------------------------
// per-lane context
// ---------------------------------------------------------------------------------------------
template <class real>
struct Lane {
    const DevModel<real> &M;
    Desc<real> &d;            // the warp's move descriptor (shared memory)
    real *slab;               // this lane's scratch: its local array, or its column of the warp's slab
    int sstride;              // 1 (local array) or 32 (slab interleaved by lane)
    int lane;
    const LaneLayout &LL;     // per-lane scratch layout (shared memory)
    int tau, taum, tau1, rep;
    bool active;
    // FP32 build: the round-off scale (nats) of the last eval, 4 eps times the sum of the magnitudes of
    // its terms (the node-balance terms of a move cancel to far less than their size)
    mutable real nzs = 0;

    __device__ Lane(const DevModel<real> &M_, Desc<real> &d_, real *slab_, int sstride_, int lane_,
                    const LaneLayout &LL_)
        : M(M_), d(d_), slab(slab_), sstride(sstride_), lane(lane_), LL(LL_) {}

    __device__ inline real &S(int off, int i) const { return slab[(size_t)(off + i) * sstride]; }
    __device__ inline size_t ix(int x, int t) const { return sidx(x, t, rep, M.T, M.R); }

    __device__ static inline real nzacc(real v, real &A) {
        A += fabs(v);
        return v;
    }
    // append a walk point (its potential and, in FP32, the round-off scale of that potential)
    __device__ inline void push(int pofs, int cofs, int *np, real x, real c, real z) const {
        S(pofs, *np) = x;
        S(cofs, *np) = c;
        if constexpr (sizeof(real) == 4) S(pofs == LL.pr ? LL.zr : LL.zl, *np) = z;
        ++*np;
    }

    // ------------------------------------------------------------------ evaluation of the move
    // eval_move! (src/local.jl:789) of both steps (the later step first, as mv_eval! of a block
    // move, :1219). Returns beta * DeltaC(t); fills d (storage) and dr (nodes) at t.
    __device__ __noinline__ real eval(real t) const {
        const int *hdr = d.hdr;
        int ng = hdr[0], nse = hdr[1], nl = hdr[2], nk = hdr[3], nku = hdr[4], nns = hdr[5], nga = hdr[6],
            nna = hdr[7], nku0 = hdr[11];
        real dt = M.dt, cv = M.c_viol, k0 = M.kappa0;
        real D = 0, A = 0;
        // kinks (src/local.jl:605 update_kinks!)
        for (int q = 0; q < nk; ++q) {
            real Q = S(LL.kq, q);
            S(LL.kph, q) = fmax(Q + d.kg[q] * t, real(0)) - fmax(Q, real(0));
        }
        // ---- step tau (every term in difference form, see clamp_diff)
        for (int q = 0; q < nns; ++q) S(LL.drs, q) = 0;
        for (int q = 0; q < ng; ++q) {
            int j = d.gi[q];
            real k = M.kc_d[j], av = M.d_avail[j];
            real dyc, dex;
            clamp_diff<real>(M.g[ix(j, tau)], t * d.ga[q], &dyc, &dex);
            real dp = av * k * dyc;
            D += nzacc(dt * M.d_mc[j] * dp + cv * dt * (k + k0) * dex, A);
            S(LL.drs, d.gpos[q]) -= dp;
        }
        for (int q = 0; q < nku0; ++q) {  // kinked entries (prorata!, src/local.jl:1782)
            real ak = S(LL.kua, q), a = d.kda[q];
            if (ak == 0 && a == 0) continue;
            int j = d.ku[q];
            real k = M.kc_d[j], av = M.d_avail[j];
            real dyc, dex;
            clamp_diff<real>(M.g[ix(j, tau)], t * a + ak * S(LL.kph, d.kk[q]), &dyc, &dex);
            real dp = av * k * dyc;
            D += nzacc(dt * M.d_mc[j] * dp + cv * dt * (k + k0) * dex, A);
            S(LL.drs, d.kupos[q]) -= dp;
        }
        for (int q = 0; q < nl; ++q) {
            int e = d.li[q];
            real df = t * d.ldf[q];
            D += nzacc(cv * dt * hinge_diff<real>(M.F[ix(e, tau)], df, M.ls[e]), A);
            S(LL.drs, d.lpa[q]) += df;
            S(LL.drs, d.lpb[q]) -= df;
        }
        for (int q = 0; q < nse; ++q) {
            int j = d.si[q];
            real k = M.kc_s[j];
            real dj, d1;
            D += nzacc(soc_diff<real>(M.s_hours[j], M.s_qt[j], M.s_etain[j], M.s_etaout[j], M.s_mc[j], k, k + k0, dt, cv,
                                M.e[ix(j, tau)], M.e[ix(j, tau1)], t * d.sa[q], real(0), &dj, &d1), A);
            S(LL.drs, d.spos[q]) += dj;
            S(LL.dcs, q) = d1;
        }
        for (int q = 0; q < nns; ++q)
            D += nzacc(dt * phibal_diff<real>(M.r[ix(d.nds[q], tau)], S(LL.drs, q), M.c_shed, M.c_dump), A);
        // ---- step tau - 1 (linked storage terms: the end value moves with step tau)
        for (int q = 0; q < nna; ++q) S(LL.dra, q) = 0;
        for (int q = 0; q < nga; ++q) {
            int j = d.gia[q];
            real k = M.kc_d[j], av = M.d_avail[j];
            real dyc, dex;
            clamp_diff<real>(M.g[ix(j, taum)], t * d.gaa[q], &dyc, &dex);
            real dp = av * k * dyc;
            D += nzacc(dt * M.d_mc[j] * dp + cv * dt * (k + k0) * dex, A);
            S(LL.dra, d.gposa[q]) -= dp;
        }
        for (int q = nku0; q < nku; ++q) {  // kinked entries at tau - 1 (prep_tsoc!, src/local.jl:1849)
            real ak = S(LL.kua, q), a = d.kda[q];
            if (ak == 0 && a == 0) continue;
            int j = d.ku[q];
            real k = M.kc_d[j], av = M.d_avail[j];
            real dyc, dex;
            clamp_diff<real>(M.g[ix(j, taum)], t * a + ak * S(LL.kph, d.kk[q]), &dyc, &dex);
            real dp = av * k * dyc;
            D += nzacc(dt * M.d_mc[j] * dp + cv * dt * (k + k0) * dex, A);
            S(LL.dra, d.kupos[q]) -= dp;
        }
        for (int q = 0; q < nse; ++q) {
            int j = d.si[q];
            real k = M.kc_s[j];
            real dj, d1;
            D += nzacc(soc_diff<real>(M.s_hours[j], M.s_qt[j], M.s_etain[j], M.s_etaout[j], M.s_mc[j], k, k + k0, dt, cv,
                                M.e[ix(j, taum)], M.e[ix(j, tau)], real(0), t * d.sa[q], &dj, &d1), A);
            S(LL.dra, d.sposa[q]) += dj;
            S(LL.dca, q) = d1;
        }
        for (int q = 0; q < nna; ++q)
            D += nzacc(dt * phibal_diff<real>(M.r[ix(d.nda[q], taum)], S(LL.dra, q), M.c_shed, M.c_dump), A);
        if constexpr (sizeof(real) == 4) nzs = M.beta_v * A * real(4.8e-7);
        return M.beta_v * D;
    }

    // secondary quantities at the current point into the "previous" buffers
    __device__ void save_prev() const {
        int nse = d.hdr[1], nns = d.hdr[5], nna = d.hdr[7];
        for (int q = 0; q < nse; ++q) {
            S(LL.dps, q) = S(LL.dcs, q);
            S(LL.dpa, q) = S(LL.dca, q);
        }
        for (int q = 0; q < nns; ++q) S(LL.sps, q) = M.r[ix(d.nds[q], tau)] + S(LL.drs, q);
        for (int q = 0; q < nna; ++q) S(LL.spa, q) = M.r[ix(d.nda[q], taum)] + S(LL.dra, q);
    }

    // the three storage secondaries of a storage term (src/local.jl:885)
    __device__ inline void stor_sec(int j, real dd, real out[3]) const {
        real ein = M.s_etain[j];
        out[0] = dd;
        out[1] = ein > 0 ? dd - ein : real(1);
        out[2] = -dd * M.s_etaout[j] - real(1);
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

    // collect sign changes between prev (at lo) and cur (at hi): storage ones into gro (if
    // storage splitting applies), the others into ro. Returns false on root-buffer overflow.
    __device__ __noinline__ bool collect(real lo, real hi, real sgn, bool stor, bool want_stor, bool want_other, int *nro,
                            int *ngro) const {
        int nse = d.hdr[1], nns = d.hdr[5], nna = d.hdr[7];
        real x;
        if (want_stor || !stor) {
            for (int side = 0; side < 2; ++side)
                for (int q = 0; q < nse; ++q) {
                    real a3[3], b3[3];
                    int j = d.si[q];
                    stor_sec(j, side == 0 ? S(LL.dps, q) : S(LL.dpa, q), a3);
                    stor_sec(j, side == 0 ? S(LL.dcs, q) : S(LL.dca, q), b3);
                    for (int h = 0; h < 3; ++h)
                        if (root_of(a3[h], b3[h], lo, hi, sgn, &x)) {
                            if (stor) {
                                if (*ngro >= LL.maxroots) return false;
                                S(LL.gro, (*ngro)++) = x;
                            } else {
                                if (*nro >= LL.maxroots) return false;
                                S(LL.ro, (*nro)++) = x;
                            }
                        }
                }
        }
        if (want_other) {
            for (int q = 0; q < nns; ++q) {
                real b = M.r[ix(d.nds[q], tau)] + S(LL.drs, q);
                if (root_of(S(LL.sps, q), b, lo, hi, sgn, &x)) {
                    if (*nro >= LL.maxroots) return false;
                    S(LL.ro, (*nro)++) = x;
                }
            }
            for (int q = 0; q < nna; ++q) {
                real b = M.r[ix(d.nda[q], taum)] + S(LL.dra, q);
                if (root_of(S(LL.spa, q), b, lo, hi, sgn, &x)) {
                    if (*nro >= LL.maxroots) return false;
                    S(LL.ro, (*nro)++) = x;
                }
            }
        }
        return true;
    }

    __device__ void sort_buf(int off, int n, real sgn) const {  // insertion sort in walking order
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

    // next primary breakpoint beyond tp in walking direction (finalize!, src/local.jl:656, scanned
    // instead of sorted: the same sequence); returns false if none
    __device__ __noinline__ bool next_bp(real tp, real sgn, real *out) const {
        int ng = d.hdr[0], nse = d.hdr[1], nl = d.hdr[2], nk = d.hdr[3], nku = d.hdr[4], nga = d.hdr[6],
            nku0 = d.hdr[11];
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
        for (int q = 0; q < nk; ++q)
            if (S(LL.kv, q) != 0 && d.kg[q] != 0) consider(-S(LL.kq, q) / d.kg[q]);
        for (int q = 0; q < ng; ++q) {
            real a = d.ga[q];
            real y0 = M.g[ix(d.gi[q], tau)];
            consider((real(0) - y0) / a);
            consider((real(1) - y0) / a);
        }
        for (int q = 0; q < nse; ++q) {
            real a = d.sa[q];
            real y0 = M.e[ix(d.si[q], tau)];
            consider((real(0) - y0) / a);
            consider((real(1) - y0) / a);
        }
        for (int q = 0; q < nku; ++q) {
            real ak = S(LL.kua, q), a = d.kda[q];
            if (ak == 0 && a == 0) continue;
            int kq = d.kk[q];
            real Q = S(LL.kq, kq), gk = d.kg[kq];
            real y0 = M.g[ix(d.ku[q], q < nku0 ? tau : taum)];
            real offs[4] = {real(0), real(0), -ak * Q, ak * Q};
            real sls[4] = {a + ak * gk, a, a, a + ak * gk};
            for (int h = 0; h < 4; ++h) {
                if (sls[h] == 0) continue;
                consider((real(0) - y0 - offs[h]) / sls[h]);
                consider((real(1) - y0 - offs[h]) / sls[h]);
            }
        }
        for (int q = 0; q < nga; ++q) {
            real a = d.gaa[q];
            real y0 = M.g[ix(d.gia[q], taum)];
            consider((real(0) - y0) / a);
            consider((real(1) - y0) / a);
        }
        for (int q = 0; q < nl; ++q) {
            int e = d.li[q];
            real f0 = M.F[ix(e, tau)], df = d.ldf[q], se = M.ls[e];
            consider((real(1) * se - f0) / df);
            consider((real(-1) * se - f0) / df);
        }
        *out = best;
        return have;
    }

    // piece_roots! (src/local.jl:1267) between prev (at a) and cur (at b); evaluates the roots
    __device__ __noinline__ bool piece_roots(int pofs, int cofs, int *np, real a, real b, real sgn, real *cmin) const {
        int nro = 0, ngro = 0;
        if (!collect(a, b, sgn, true, false, true, &nro, &ngro)) return false;
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

    // walk! (src/local.jl:1294), plain model. Returns 1 proper, 0 improper, -1 buffer overflow.
    __device__ __noinline__ int walk(int pofs, int cofs, int *np, real sgn) const {
        bool stor = d.hdr[1] > 0;
        real tp = 0, cmin = 0, delta = 0;
        int nx = 0;
        *np = 0;
        eval(real(0));
        save_prev();
        while (true) {
            real t;
            if (!next_bp(tp, sgn, &t)) {
                real cprev = *np == 0 ? real(0) : S(cofs, *np - 1);
                // the probe step of walk! (1e-6 relative). In FP32 the state values y0 + t a carry
                // an absolute round-off of ~1e-7, as large as a 1e-6 step's increment: the FP32
                // build probes 1e-3 ahead instead. The ray points only place the discretisation
                // (the roots inside a ray step are inserted all the same), so this changes which
                // points are walked, not the conditional that is sampled.
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
            if (!collect(tp, t, sgn, stor, true, !stor, &nro, &ngro)) return -1;
            // when storage splitting applies, the other roots are found per piece below
            if (stor && ngro > 0) {
                sort_buf(LL.gro, ngro, sgn);
                real a0 = tp;
                for (int i = 0; i < ngro; ++i) {
                    real x = S(LL.gro, i);
                    real cx = eval(x), zx = nzs;
                    if (!piece_roots(pofs, cofs, np, a0, x, sgn, &cmin)) return -1;
                    eval(x);  // restore the secondaries at x
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
                if (stor) {  // no storage root: the other secondaries over the whole segment
                    if (!collect(tp, t, sgn, true, false, true, &nro, &ngro)) return -1;
                }
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

    // logseg, trexp_offset (src/local.jl:1099, :1106). For x > 0 the FP32 build takes the log of
    // the product, L (1 - e^-x) / x, whose factors stay inside the FP32 range (the second lies in
    // (0, 1]): one logarithm instead of three, the same value to a few ulp; the FP64 build keeps the
    // reference's sum of logarithms, as the oracle does.
    __device__ static real logseg(real L, real x) {
        if (fabs(x) < real(1e-10)) return log(L) - x / 2;
        if constexpr (sizeof(real) == 4) {
            if (x > 0) return log(L * (-expm1(-x)) / x);
        }
        if (x > 0) return log(L) + log(-expm1(-x)) - log(x);
        return log(L) - x + log(-expm1(x)) - log(-x);
    }
    // A segment whose potential changes by less than this many nats is drawn uniformly from its
    // left end (trexp_offset's 1e-10). In the FP32 build the potential of a flat segment comes out
    // as round-off -- up to ~1e-3 nats next to a node-balance kink on the steep side -- and the
    // sign of that round-off would pick between the left and the mirrored u -> t map: it takes
    // 1e-4, or the round-off scale of the segment's two end points if larger (the density then
    // varies by no more than that across the segment).
    static constexpr real flat_nats = sizeof(real) == 4 ? real(1e-4) : real(1e-10);
    __device__ static real trexp_offset(real u, real g, real L, real flat) {
        real x = g * L;
        if (fabs(x) < flat) return u * L;
        if (g > 0) return -log1p(-u * (-expm1(-x))) / g;
        return L + log1p(-u * (-expm1(x))) / (-g);
    }

    __device__ inline real P(int i, int nl) const {  // merged points: left reversed, 0, right
        if (i < nl) return S(LL.pl, nl - 1 - i);
        if (i == nl) return 0;
        return S(LL.pr, i - nl - 1);
    }
    __device__ inline real Zz(int i, int nl) const {  // FP32 round-off scale of the merged points
        if (i < nl) return S(LL.zl, nl - 1 - i);
        if (i == nl) return 0;
        return S(LL.zr, i - nl - 1);
    }
    __device__ inline real Cc(int i, int nl) const {
        if (i < nl) return S(LL.cl, nl - 1 - i);
        if (i == nl) return 0;
        return S(LL.cr, i - nl - 1);
    }


    // ------------------------------------------------------------ separable storage moves
    // A move whose terms are storage units at distinct nodes and nothing else (the atoms of a
    // state-of-charge field, 97 % of the walk work of a sweep): the line potential is a sum of
    // one-dimensional piecewise-linear functions, one per unit, with at most ten kinks each. The
    // walk visits the points walk! visits -- the units' clamp points (the primary breakpoints),
    // their storage thresholds and the zero crossings of their node balances (the secondary
    // roots) -- event by event, re-evaluating only the unit whose piece changes, and advancing the
    // potential along the summed slopes in between.
    __device__ bool separable() const {
        const int *h = d.hdr;
        return h[1] > 0 && h[0] == 0 && h[2] == 0 && h[3] == 0 && h[4] == 0 && h[6] == 0 && h[8] == 0 &&
               h[5] == h[1] && h[7] == h[1];
    }

    // beta * (cost change) of unit q at t, with its two node balances (tau and tau - 1)
    __device__ __noinline__ real unit_val(int q, real t, real *Sw, real *Sa) const {
        int j = d.si[q];
        real x = t * d.sa[q];
        real k = M.kc_s[j], w = k + M.kappa0, dt = M.dt, cv = M.c_viol;
        real djw, dw, dja, da;
        real cw = soc_diff<real>(M.s_hours[j], M.s_qt[j], M.s_etain[j], M.s_etaout[j], M.s_mc[j], k, w, dt, cv,
                                 M.e[ix(j, tau)], M.e[ix(j, tau1)], x, real(0), &djw, &dw);
        real ca = soc_diff<real>(M.s_hours[j], M.s_qt[j], M.s_etain[j], M.s_etaout[j], M.s_mc[j], k, w, dt, cv,
                                 M.e[ix(j, taum)], M.e[ix(j, tau)], real(0), x, &dja, &da);
        real S0w = M.r[ix(d.nds[d.spos[q]], tau)], S0a = M.r[ix(d.nda[d.sposa[q]], taum)];
        *Sw = S0w + djw;
        *Sa = S0a + dja;
        real bw = dt * phibal_diff<real>(S0w, djw, M.c_shed, M.c_dump);
        real ba = dt * phibal_diff<real>(S0a, dja, M.c_shed, M.c_dump);
        return M.beta_v * (cw + bw + ca + ba);
    }

    // The piece of unit q that starts at t0 (where its node balances are Sw0, Sa0): its end (the
    // next clamp of the state of charge -- a primary breakpoint -- or the next storage threshold,
    // both exact) and the zero crossings of its node balances inside it (linear there, so found
    // by interpolation as piece_roots! does). Stored as an event list in walking order: times in
    // ue[0..un), the end kind in uh (1 clamp, 2 threshold, 0 none: the piece runs to infinity);
    // the unit's potential and node balances at the end (or at a probe beyond t0) in ufe, usw, usa.
    __device__ __noinline__ void unit_piece(int q, real t0, real sgn, real Sw0, real Sa0) const {
        int j = d.si[q];
        real a = d.sa[q];
        real e0 = M.e[ix(j, tau)];
        real e1c = clampr<real>(M.e[ix(j, tau1)], 0, 1), emc = clampr<real>(M.e[ix(j, taum)], 0, 1);
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
        th[nth++] = 0;  // the sign changes of the three storage secondaries (src/local.jl:885)
        if (ein > 0) th[nth++] = ein;
        if (eout > 0) th[nth++] = real(-1) / eout;
        for (int i = 0; i < nth; ++i) {
            real xw = e1c - e0 - (th[i] + qt) * dt / h;  // d at tau crosses th
            if (e0 + xw >= 0 && e0 + xw <= 1) cand(xw, false);
            real xa = emc - e0 + (th[i] + qt) * dt / h;  // d of step tau - 1 crosses th
            if (e0 + xa >= 0 && e0 + xa <= 1) cand(xa, false);
        }
        real tpb = have ? ts : t0 + sgn * fmax(real(1), fabs(t0));
        real Sw1, Sa1;
        S(LL.ufe, q) = unit_val(q, tpb, &Sw1, &Sa1);
        S(LL.usw, q) = Sw1;
        S(LL.usa, q) = Sa1;
        real r[2];
        int nr = 0;
        real pa[2] = {Sw0, Sa0}, pb[2] = {Sw1, Sa1};
        for (int i = 0; i < 2; ++i) {
            real x;
            if (have) {
                if (root_of(pa[i], pb[i], t0, tpb, sgn, &x)) r[nr++] = x;
            } else if (pa[i] != pb[i]) {  // linear to infinity: the crossing anywhere ahead
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
        for (int i = 0; i < nr; ++i) S(LL.ue + 3 * q, n++) = r[i];
        if (have) S(LL.ue + 3 * q, n++) = ts;
        S(LL.un, q) = real(n);
        S(LL.uh, q) = have ? (prim ? real(1) : real(2)) : real(0);
        S(LL.ui, q) = real(0);
    }

    // the next event of unit q after its current position t (where its potential is f): time (ut,
    // +-inf if none), kind (uk: 1 clamp, 0 secondary, -1 none), the potential there (ufn) and the
    // slope to there (usl)
    __device__ __noinline__ void unit_next(int q, real t, real f, real sgn) const {
        int i = (int)S(LL.ui, q), n = (int)S(LL.un, q), hk = (int)S(LL.uh, q);
        real Sw, Sa, tn, fn;
        if (i < n) {
            tn = S(LL.ue + 3 * q, i);
            bool end = i == n - 1 && hk != 0;
            fn = end ? S(LL.ufe, q) : unit_val(q, tn, &Sw, &Sa);
            S(LL.ut, q) = tn;
            S(LL.uk, q) = end ? (hk == 1 ? real(1) : real(0)) : real(0);
            S(LL.ufn, q) = fn;
            S(LL.usl, q) = tn != t ? (fn - f) / (tn - t) : real(0);  // (an event at t itself: no extent)
        } else {  // linear to infinity
            real tp = t + sgn * fmax(real(1), fabs(t));
            fn = unit_val(q, tp, &Sw, &Sa);
            S(LL.ut, q) = real(INFINITY) * sgn;
            S(LL.uk, q) = real(-1);
            S(LL.usl, q) = (fn - f) / (tp - t);
        }
    }

    // move unit q past its current event at t: to the next event of its piece, or into the next piece
    __device__ void unit_pass(int q, real t, real sgn) const {
        int i = (int)S(LL.ui, q), n = (int)S(LL.un, q), hk = (int)S(LL.uh, q);
        real f = S(LL.ufn, q);
        if (i == n - 1 && hk != 0)
            unit_piece(q, t, sgn, S(LL.usw, q), S(LL.usa, q));
        else
            S(LL.ui, q) = real(i + 1);
        unit_next(q, t, f, sgn);
    }

    // A min-heap of the units with a pending event, keyed by sgn * (event time): the next event of
    // the walk is at the top, and passing it costs log2(units) steps instead of a scan of all units.
    __device__ inline void heap_up(int i) const {
        real k = S(LL.hk, i), u = S(LL.hu, i);
        while (i > 0) {
            int p = (i - 1) >> 1;
            real kp = S(LL.hk, p);
            if (!(k < kp)) break;
            S(LL.hk, i) = kp;
            S(LL.hu, i) = S(LL.hu, p);
            i = p;
        }
        S(LL.hk, i) = k;
        S(LL.hu, i) = u;
    }
    __device__ inline void heap_down(int i, int n) const {
        real k = S(LL.hk, i), u = S(LL.hu, i);
        while (true) {
            int l = 2 * i + 1;
            if (l >= n) break;
            int m = l;
            real km = S(LL.hk, l);
            if (l + 1 < n) {
                real kr = S(LL.hk, l + 1);
                if (kr < km) {
                    m = l + 1;
                    km = kr;
                }
            }
            if (!(km < k)) break;
            S(LL.hk, i) = km;
            S(LL.hu, i) = S(LL.hu, m);
            i = m;
        }
        S(LL.hk, i) = k;
        S(LL.hu, i) = u;
    }

    // walk! for a separable move; same returns as walk(). The events of all units -- every
    // unit's clamps (the primary breakpoints), storage thresholds and node-balance roots -- are
    // visited in walking order, one point each; the stop test runs at every clamp (walk!'s test
    // at its primary breakpoints), and once every clamp ahead is passed the walk takes ray steps.
    __device__ __noinline__ int walk_sep(int pofs, int cofs, int *np, real sgn) const {
        int nu = d.hdr[1];
        double B = 0;     // summed slope of the potential at the current position
        double absB = 0;  // the sum of the magnitudes of the units' slopes (round-off scale)
        int nh = 0;       // units in the heap
        int ncl = 0;      // clamps ahead (each unit's 0 and 1 crossings in this direction)
        for (int q = 0; q < nu; ++q) {
            real a = d.sa[q], e0 = M.e[ix(d.si[q], tau)];
            real c0 = (real(0) - e0) / a, c1 = (real(1) - e0) / a;
            ncl += (isfinite(c0) && sgn * c0 > 0) + (isfinite(c1) && sgn * c1 > 0);
            unit_piece(q, real(0), sgn, M.r[ix(d.nds[d.spos[q]], tau)], M.r[ix(d.nda[d.sposa[q]], taum)]);
            unit_next(q, real(0), real(0), sgn);
            B += (double)S(LL.usl, q);
            absB += fabs((double)S(LL.usl, q));
            real tq = S(LL.ut, q);
            if (isfinite(tq)) {
                S(LL.hk, nh) = sgn * tq;
                S(LL.hu, nh) = real(q);
                heap_up(nh);
                ++nh;
            }
        }
        *np = 0;
        double c = 0, cmin = 0;
        real tcur = 0, delta = 0;
        int nx = 0;
        bool ray = ncl == 0;
        // the unit at the top passes its event at t: its next event re-keys it (or it leaves)
        auto pass_top = [&](real t) {
            int q = (int)S(LL.hu, 0);
            real old = S(LL.usl, q);
            unit_pass(q, t, sgn);
            B += (double)S(LL.usl, q) - (double)old;
            absB = fmax(absB, absB + fabs((double)S(LL.usl, q)) - fabs((double)old));
            real tn = S(LL.ut, q);
            if (isfinite(tn)) {
                S(LL.hk, 0) = sgn * tn;
            } else {
                --nh;
                S(LL.hk, 0) = S(LL.hk, nh);
                S(LL.hu, 0) = S(LL.hu, nh);
            }
            if (nh > 0) heap_down(0, nh);
        };
        auto point = [&](real t) -> bool {
            if (*np >= M.maxpts) return false;
            push(pofs, cofs, np, t, (real)c, real(4.8e-7) * (real)(fabs(c) + absB * fabs((double)t)));
            cmin = fmin(cmin, c);
            return true;
        };
        while (true) {
            if (!ray) {
                if (nh == 0) {  // (no event left before the clamps the count expects)
                    ray = true;
                    continue;
                }
                int q = (int)S(LL.hu, 0);
                real tS = S(LL.ut, q);
                bool clamp = S(LL.uk, q) == real(1);
                c += B * (double)(tS - tcur);
                tcur = tS;
                if (!point(tS)) return -1;
                pass_top(tS);
                if (clamp) {
                    --ncl;
                    if (c - cmin > (double)M.maxnats) return 1;
                    if (ncl <= 0) ray = true;
                }
            } else {
                // every clamp is behind: ray steps (the outgoing slope is the summed slope)
                double sl = (double)sgn * B;
                if (sl > 0)
                    delta = fmin(real(2) * M.maxnats / (real)sl, real(1e3) * fmax(fabs(tcur), real(1e-3)));
                else
                    delta = delta == 0 ? fmax(fabs(tcur), real(1e-6)) : real(2) * delta;
                real target = tcur + sgn * delta;
                if (++nx > 80) return 0;
                while (nh > 0) {  // the events before the target
                    real tS = S(LL.ut, (int)S(LL.hu, 0));
                    if (!(sgn * (target - tS) > 0)) break;
                    c += B * (double)(tS - tcur);
                    tcur = tS;
                    if (!point(tS)) return -1;
                    pass_top(tS);
                }
                c += B * (double)(target - tcur);
                tcur = target;
                if (!point(target)) return -1;
                while (nh > 0 && S(LL.ut, (int)S(LL.hu, 0)) == target) pass_top(target);
                if (c - cmin > (double)M.maxnats) return 1;
            }
        }
    }

    // sample_line! (src/local.jl:1501); *guard on buffer overflow (t = 0)
    __device__ __noinline__ real sample_line(real ucat, real uoff, bool *guard) const {
        *guard = false;
        int nr = 0, nl = 0;
        bool sep = separable();
        int w = sep ? walk_sep(LL.pr, LL.cr, &nr, real(1)) : walk(LL.pr, LL.cr, &nr, real(1));
        if (w < 0) {
            *guard = true;
            return 0;
        }
        if (w == 0) return 0;
        w = sep ? walk_sep(LL.pl, LL.cl, &nl, real(-1)) : walk(LL.pl, LL.cl, &nl, real(-1));
        if (w < 0) {
            *guard = true;
            return 0;
        }
        if (w == 0) return 0;
        int npt = nl + 1 + nr;
        int nseg = npt - 1;
        real mx = -INFINITY;
        for (int j = 0; j < nseg; ++j) {
            real p0 = P(j, nl), p1 = P(j + 1, nl), c0 = Cc(j, nl), c1 = Cc(j + 1, nl);
            real L = p1 - p0;
            real lm = L > 0 ? -fmin(c0, c1) + logseg(L, fabs(c1 - c0)) : real(-INFINITY);
            S(LL.lm, j) = lm;
            mx = fmax(mx, lm);
        }
        real tot = 0;
        for (int j = 0; j < nseg; ++j) {  // the masses relative to the largest, kept for the inversion
            real e = exp(S(LL.lm, j) - mx);
            S(LL.lm, j) = e;
            tot += e;
        }
        real u = ucat * tot, acc = 0;
        int jj = nseg - 1;
        for (int q = 0; q < nseg; ++q) {
            acc += S(LL.lm, q);
            if (u <= acc) {
                jj = q;
                break;
            }
        }
        real p0 = P(jj, nl), p1 = P(jj + 1, nl);
        real L = p1 - p0;
        real g = (Cc(jj + 1, nl) - Cc(jj, nl)) / L;
        real flat = flat_nats;
        if constexpr (sizeof(real) == 4) {
            // each end's round-off: that of its terms, and that of placing the point itself (a
            // kink at x lands within ulp(x) of where it is, on either side, where the potential
            // turns by the difference of the neighbouring slopes)
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
        return (g >= 0 || fabs(g * L) < flat) ? p0 + trexp_offset(uoff, g, L, flat)
                                              : p1 - trexp_offset(uoff, -g, L, flat);
    }

    // commit_block! / apply_step! (src/local.jl:2495, :2507)
    __device__ __noinline__ void commit(real t) const {
        eval(t);
        int ng = d.hdr[0], nse = d.hdr[1], nl = d.hdr[2], nku = d.hdr[4], nns = d.hdr[5], nga = d.hdr[6],
            nna = d.hdr[7], nth = d.hdr[8], nku0 = d.hdr[11];
        for (int q = 0; q < nga; ++q) M.g[ix(d.gia[q], taum)] += t * d.gaa[q];
        for (int q = 0; q < nna; ++q) M.r[ix(d.nda[q], taum)] += S(LL.dra, q);
        for (int q = 0; q < ng; ++q) M.g[ix(d.gi[q], tau)] += t * d.ga[q];
        for (int q = 0; q < nku; ++q) {
            real ak = S(LL.kua, q), a = d.kda[q];
            if (ak != 0 || a != 0) M.g[ix(d.ku[q], q < nku0 ? tau : taum)] += t * a + ak * S(LL.kph, d.kk[q]);
        }
        for (int q = 0; q < nse; ++q) M.e[ix(d.si[q], tau)] += t * d.sa[q];
        for (int q = 0; q < nth; ++q) M.theta[ix(d.thn[q], tau)] += t * d.tha[q];
        for (int q = 0; q < nl; ++q) M.F[ix(d.li[q], tau)] += t * d.ldf[q];
        for (int q = 0; q < nns; ++q) M.r[ix(d.nds[q], tau)] += S(LL.drs, q);
    }
};

// ---------------------------------------------------------------------------------------------
// warp-uniform move construction
// ---------------------------------------------------------------------------------------------
struct Stream {  // the class stream (TAG_LIST), every lane holds the same copy
    uint64_t seed;
    uint32_t tile, cls, sweep, j;
    __device__ double next() {
        double u0, u1;
        uniform2(seed, ESM_TAG_LIST, j >> 1, tile, cls, sweep, &u0, &u1);
        double u = (j & 1) ? u1 : u0;
        ++j;
        return u;
    }
    __device__ int pick(int n) {
        int i = (int)floor(next() * n);
        return i >= n ? n - 1 : i;
    }
};

// the move list of a tile (local_sweep!, src/local.jl:1964-1974): atoms, then nextra family draws,
// shuffled (Fisher-Yates). Encoding: atom a -> a, family f -> -(f + 1).
template <class real>
__device__ __noinline__ void build_list(const DevModel<real> &M, Desc<real> &d, Stream &st, int lane) {
    int na = M.natoms, n = na + M.nextra;
    __syncwarp();
    for (int i = lane; i < na; i += 32) d.moves[i] = i;
    __syncwarp();
    // family draws: every lane draws the same numbers; lane 0 writes
    for (int i = 0; i < M.nextra; ++i) {
        double u = st.next();
        int kd = ESM_NFAM - 1;
        for (int q = 0; q < ESM_NFAM; ++q)
            if (M.cumw[q] >= u) {
                kd = q;
                break;
            }
        if (lane == 0) d.moves[na + i] = -(kd + 1);
    }
    __syncwarp();
    for (int i = n - 1; i >= 1; --i) {
        int j = st.pick(i + 1);
        if (lane == 0) {
            int tmp = d.moves[i];
            d.moves[i] = d.moves[j];
            d.moves[j] = tmp;
        }
    }
    __syncwarp();
}

template <class real>
__device__ inline void add_node(Desc<real> &d, int side, int n, int *cnt, int *pos_out) {
    unsigned char *mk = side == 0 ? d.nmarks : d.nmarka;
    int *lst = side == 0 ? d.nds : d.nda;
    int *pos = side == 0 ? d.posn_s : d.posn_a;
    if (!mk[n]) {
        mk[n] = 1;
        pos[n] = *cnt;
        lst[(*cnt)++] = n;
    }
    if (pos_out) *pos_out = pos[n];
}

template <class real>
__device__ inline real kappa_d(const DevModel<real> &M, int j) {
    return M.d_avail[j] * M.kc_d[j];
}

// Build the warp-uniform part of move `mv` (lane 0 writes shared memory). Returns the family
// index for the statistics (ESM_NFAM for atoms) or -1 when the selection rejects the move.
template <class real>
__device__ __noinline__ int prep_move(const DevModel<real> &M, Desc<real> &d, Stream &st, int mv, int lane) {
    int N = M.N;
    int *h = d.hdr;
    // every lane computes the same selection; lane 0 writes (after every lane left the last move)
    bool w0 = lane == 0;
    __syncwarp();
    if (w0)
        for (int i = 0; i < 16; ++i) h[i] = 0;
    __syncwarp();
    int fam = mv >= 0 ? ESM_NFAM : -mv - 1;
    int ng = 0, nse = 0, nth = 0, nk = 0, nku = 0, nga = 0;
    int nku0 = -1;  // kinked units of step tau (-1: all of them)
    real kmin = M.kmin;
    auto nun = [&](int n) { return M.up[n + 1] - M.up[n]; };
    bool ok = true;
    if (mv >= 0) {  // prep_atom! (src/local.jl:1567)
        int f = 0;
        while (f + 1 < M.nfields && M.fap[f + 1] <= mv) ++f;
        int role = M.frole[f];
        for (int q = M.ap[mv] + lane; q < M.ap[mv + 1]; q += 32) {
            int i = q - M.ap[mv];
            if (role == ESM_ROLE_THETA) {
                d.thn[i] = M.ai[q];
                d.tha[i] = M.av[q];
            } else if (role == ESM_ROLE_GEN) {
                d.gi[i] = M.ai[q];
                d.ga[i] = M.av[q];
            } else {
                d.si[i] = M.ai[q];
                d.sa[i] = M.av[q];
            }
        }
        int cnt = M.ap[mv + 1] - M.ap[mv];
        if (role == ESM_ROLE_THETA)
            nth = cnt;
        else if (role == ESM_ROLE_GEN)
            ng = cnt;
        else
            nse = cnt;
    } else {
        switch (fam) {
            case ESM_FAM_UNIT: {
                int n = st.pick(N);
                if (nun(n) == 0) {
                    ok = false;
                    break;
                }
                int j = M.ua[M.up[n] + st.pick(nun(n))];
                if (w0) {
                    d.gi[0] = j;
                    d.ga[0] = 1;
                }
                ng = 1;
                break;
            }
            case ESM_FAM_PAIR:
            case ESM_FAM_XPAIR: {
                int n = st.pick(N);
                int m = fam == ESM_FAM_PAIR ? n : st.pick(N);
                if (fam == ESM_FAM_XPAIR && (m == n || M.comp[m] != M.comp[n])) {
                    ok = false;
                    break;
                }
                if (nun(n) == 0 || nun(m) == 0) {
                    ok = false;
                    break;
                }
                int u1 = M.ua[M.up[n] + st.pick(nun(n))];
                int u2 = M.ua[M.up[m] + st.pick(nun(m))];
                if (u1 == u2) {
                    ok = false;
                    break;
                }
                real k1 = kappa_d(M, u1), k2 = kappa_d(M, u2);
                if (fabs(k1) < kmin || fabs(k2) < kmin) {
                    ok = false;
                    break;
                }
                if (w0) {
                    d.gi[0] = u1;
                    d.ga[0] = real(1) / k1;
                    d.gi[1] = u2;
                    d.ga[1] = real(-1) / k2;
                }
                ng = 2;
                if (fam == ESM_FAM_XPAIR) {  // prep_reroute! (src/local.jl:1592)
                    int c = 0;
                    for (int i = 0; i < N; ++i) {
                        if (M.comp[i] != M.comp[n]) continue;
                        real x = M.Z[(size_t)i * N + n] - M.Z[(size_t)i * N + m];
                        if (fabs(x) < real(1e-15)) continue;
                        if (w0) {
                            d.thn[c] = i;
                            d.tha[c] = x;
                        }
                        ++c;
                    }
                    nth = c;
                }
                break;
            }
            case ESM_FAM_XLOC:
            case ESM_FAM_XLOCC: {
                int n = st.pick(N);
                int np = M.xpp[n + 1] - M.xpp[n];
                if (np == 0) {
                    ok = false;
                    break;
                }
                int pair = M.xpp[n] + st.pick(np);
                int m = M.xp[pair];
                if (nun(n) == 0 || nun(m) == 0) {
                    ok = false;
                    break;
                }
                int u1 = M.ua[M.up[n] + st.pick(nun(n))];
                int u2 = M.ua[M.up[m] + st.pick(nun(m))];
                real k1 = kappa_d(M, u1), k2 = kappa_d(M, u2);
                if (fabs(k1) < kmin || fabs(k2) < kmin) {
                    ok = false;
                    break;
                }
                if (w0) {
                    d.gi[0] = u1;
                    d.ga[0] = real(1) / k1;
                    d.gi[1] = u2;
                    d.ga[1] = real(-1) / k2;
                }
                ng = 2;
                nth = M.xnp[pair + 1] - M.xnp[pair];
                for (int q = lane; q < nth; q += 32) {
                    d.thn[q] = M.xn[M.xnp[pair] + q];
                    d.tha[q] = M.xv[M.xnp[pair] + q];
                }
                if (fam == ESM_FAM_XLOCC) {  // leak compensated pro rata (prorata!, src/local.jl:1782)
                    for (int q = M.xlp[pair]; q < M.xlp[pair + 1]; ++q) {
                        real gq = M.xlg[q];
                        if (gq == 0) continue;
                        int ln = M.xln[q];
                        if (w0) {
                            d.kn[nk] = ln;
                            d.kg[nk] = gq;
                            d.ksd[nk] = 0;
                            d.kqs[nk] = -1;
                        }
                        for (int p = M.up[ln]; p < M.up[ln + 1]; ++p) {
                            int j = M.ua[p];
                            if (!(fabs(kappa_d(M, j)) >= kmin)) continue;
                            if (w0) {
                                d.ku[nku] = j;
                                d.kk[nku] = nk;
                            }
                            ++nku;
                        }
                        ++nk;
                    }
                }
                break;
            }
            case ESM_FAM_POTENTIAL: {
                int n = st.pick(N);
                if (M.theta_nnz[n] == 0) {
                    ok = false;
                    break;
                }
                if (w0) {
                    d.thn[0] = n;
                    d.tha[0] = 1;
                }
                nth = 1;
                break;
            }
            case ESM_FAM_CELLPAIR:
            case ESM_FAM_CELL: {
                double u = st.next();
                int q = M.nlev - 1;
                for (int l = 0; l < M.nlev; ++l)
                    if (M.qcum[l] >= u) {
                        q = l;
                        break;
                    }
                int ncell = M.clp[q + 1] - M.clp[q];
                int cidx = M.clp[q] + st.pick(ncell);
                // distinct injecting groups of the cell, ascending
                int fl[8], nfl = 0;
                for (int p = M.cp[cidx]; p < M.cp[cidx + 1]; ++p) {
                    int gg = M.d_group[M.cu[p]];
                    bool seen = false;
                    for (int i = 0; i < nfl; ++i) seen |= fl[i] == gg;
                    if (!seen && nfl < 8) fl[nfl++] = gg;
                }
                for (int i = 1; i < nfl; ++i)
                    for (int j = i; j > 0 && fl[j] < fl[j - 1]; --j) {
                        int tmp = fl[j];
                        fl[j] = fl[j - 1];
                        fl[j - 1] = tmp;
                    }
                if (nfl == 0) {
                    ok = false;
                    break;
                }
                if (fam == ESM_FAM_CELL) {
                    int f = fl[st.pick(nfl)];
                    int c = 0;
                    for (int p = M.cp[cidx]; p < M.cp[cidx + 1]; ++p)
                        if (M.d_group[M.cu[p]] == f) {
                            if (w0) {
                                d.gi[c] = M.cu[p];
                                d.ga[c] = 1;
                            }
                            ++c;
                        }
                    ng = c;
                    break;
                }
                if (nfl < 2) {
                    ok = false;
                    break;
                }
                int f1 = fl[st.pick(nfl)], f2 = fl[st.pick(nfl)];
                if (f1 == f2) {
                    ok = false;
                    break;
                }
                real K1 = 0, K2 = 0;
                for (int p = M.cp[cidx]; p < M.cp[cidx + 1]; ++p) {
                    int j = M.cu[p];
                    if (M.d_group[j] == f1) K1 += kappa_d(M, j);
                    if (M.d_group[j] == f2) K2 += kappa_d(M, j);
                }
                if (fabs(K1) < kmin || fabs(K2) < kmin) {
                    ok = false;
                    break;
                }
                int c = 0;
                for (int p = M.cp[cidx]; p < M.cp[cidx + 1]; ++p)
                    if (M.d_group[M.cu[p]] == f1) {
                        if (w0) {
                            d.gi[c] = M.cu[p];
                            d.ga[c] = real(1) / K1;
                        }
                        ++c;
                    }
                for (int p = M.cp[cidx]; p < M.cp[cidx + 1]; ++p)
                    if (M.d_group[M.cu[p]] == f2) {
                        if (w0) {
                            d.gi[c] = M.cu[p];
                            d.ga[c] = real(-1) / K2;
                        }
                        ++c;
                    }
                ng = c;
                break;
            }
            case ESM_FAM_SPAIR: {
                int n = st.pick(N);
                int ns = M.sp[n + 1] - M.sp[n];
                if (ns == 0 || nun(n) == 0) {
                    ok = false;
                    break;
                }
                int sj = M.sa[M.sp[n] + st.pick(ns)];
                real ks = M.kc_s[sj] * M.s_hours[sj] / M.dt;
                if (ks < kmin) {
                    ok = false;
                    break;
                }
                int u1 = M.ua[M.up[n] + st.pick(nun(n))];
                int u2 = M.ua[M.up[n] + st.pick(nun(n))];
                real k1 = kappa_d(M, u1), k2 = kappa_d(M, u2);
                if (fabs(k1) < kmin || fabs(k2) < kmin) {
                    ok = false;
                    break;
                }
                if (w0) {
                    d.gia[0] = u1;
                    d.gaa[0] = ks / k1;
                    d.si[0] = sj;
                    d.sa[0] = 1;
                    d.gi[0] = u2;
                    d.ga[0] = -ks / k2;
                }
                nga = 1;
                nse = 1;
                ng = 1;
                break;
            }
            case ESM_FAM_TPOT: {  // prep_tpot! (src/local.jl:1741): the angle of node n rises by t
                int n = st.pick(N);
                if (M.theta_nnz[n] == 0) {
                    ok = false;
                    break;
                }
                if (w0) {
                    d.thn[0] = n;
                    d.tha[0] = 1;
                }
                nth = 1;
                // requirement change per unit t at the ends of n's lines (r[a] += f_e, r[b] -= f_e
                // for a line a -> b), node by node in ascending order, each node's terms summed in
                // line order; the dispatch there follows pro rata
                int last = -1;
                for (;;) {
                    int nx = INT_MAX;
                    for (int p = M.nlp[n]; p < M.nlp[n + 1]; ++p) {
                        int e = M.nl[p], a = M.bus0[e], b = M.bus1[e];
                        if (a > last && a < nx) nx = a;
                        if (b > last && b < nx) nx = b;
                    }
                    if (nx == INT_MAX) break;
                    last = nx;
                    real gm = 0;
                    for (int p = M.nlp[n]; p < M.nlp[n + 1]; ++p) {
                        int e = M.nl[p], a = M.bus0[e], b = M.bus1[e];
                        real df = M.lb[e] * real((a == n) - (b == n));
                        if (a == nx) gm += df;
                        if (b == nx) gm -= df;
                    }
                    if (gm == 0) continue;
                    if (w0) {
                        d.kn[nk] = nx;
                        d.kg[nk] = gm;
                        d.ksd[nk] = 0;
                        d.kqs[nk] = -1;
                    }
                    for (int p = M.up[nx]; p < M.up[nx + 1]; ++p) {
                        int j = M.ua[p];
                        if (!(fabs(kappa_d(M, j)) >= kmin)) continue;
                        if (w0) {
                            d.ku[nku] = j;
                            d.kk[nku] = nk;
                        }
                        ++nku;
                    }
                    ++nk;
                }
                break;
            }
            case ESM_FAM_TSOC: {  // prep_tsoc! (src/local.jl:1849): energy moved from step tau - 1 to tau
                int n = st.pick(N);
                int ns = M.sp[n + 1] - M.sp[n];
                if (ns == 0) {
                    ok = false;
                    break;
                }
                int sj = M.sa[M.sp[n] + st.pick(ns)];
                real ks = M.kc_s[sj] * M.s_hours[sj] / M.dt;
                if (ks < kmin) {
                    ok = false;
                    break;
                }
                if (w0) {
                    d.si[0] = sj;
                    d.sa[0] = 1;
                    // kink 0: node n at tau - 1 (+ks), kink 1: node n at tau (-ks), both with the
                    // unit's requirement adjustment (soc_qadj)
                    d.kn[0] = n;
                    d.kg[0] = ks;
                    d.ksd[0] = 1;
                    d.kqs[0] = sj;
                    d.kn[1] = n;
                    d.kg[1] = -ks;
                    d.ksd[1] = 0;
                    d.kqs[1] = sj;
                }
                nse = 1;
                nk = 2;
                for (int side = 0; side < 2; ++side) {  // the kinked units of step tau first
                    for (int p = M.up[n]; p < M.up[n + 1]; ++p) {
                        int j = M.ua[p];
                        if (!(fabs(kappa_d(M, j)) >= kmin)) continue;
                        if (w0) {
                            d.ku[nku] = j;
                            d.kk[nku] = side == 0 ? 1 : 0;
                        }
                        ++nku;
                    }
                    if (side == 0) nku0 = nku;
                }
                break;
            }
        }
    }
    if (nku0 < 0) nku0 = nku;
    __syncwarp();
    if (!ok) return -1;
    // ---- finalize! (src/local.jl:656): zero tiny coefficients, lines, touched nodes
    if (w0) {
        int c = 0;
        for (int q = 0; q < ng; ++q)
            if (!(fabs(d.ga[q]) < real(1e-14))) {
                d.gi[c] = d.gi[q];
                d.ga[c] = d.ga[q];
                ++c;
            }
        ng = c;
        c = 0;
        for (int q = 0; q < nse; ++q)
            if (!(fabs(d.sa[q]) < real(1e-14))) {
                d.si[c] = d.si[q];
                d.sa[c] = d.sa[q];
                ++c;
            }
        nse = c;
        c = 0;
        for (int q = 0; q < nth; ++q)
            if (!(fabs(d.tha[q]) < real(1e-14))) {
                d.thn[c] = d.thn[q];
                d.tha[c] = d.tha[q];
                ++c;
            }
        nth = c;
        // a unit moved directly and pro rata is one term (add_kentry! adds to the unit's entry,
        // src/local.jl:583): its direct coefficient at the same step moves into the kinked entry
        for (int q = 0; q < nku; ++q) {
            d.kda[q] = 0;
            if (q < nku0) {
                for (int p = 0; p < ng; ++p)
                    if (d.gi[p] == d.ku[q] && d.ga[p] != 0) {
                        d.kda[q] = d.ga[p];
                        d.ga[p] = 0;
                    }
            } else {
                for (int p = 0; p < nga; ++p)
                    if (d.gia[p] == d.ku[q] && d.gaa[p] != 0) {
                        d.kda[q] = d.gaa[p];
                        d.gaa[p] = 0;
                    }
            }
        }
        // node lists: ws entries (gens, storage, kinked units), then line ends; wa entries, linked storage
        int nns = 0, nna = 0;
        for (int q = 0; q < ng; ++q) add_node(d, 0, M.d_bus[d.gi[q]], &nns, &d.gpos[q]);
        for (int q = 0; q < nse; ++q) add_node(d, 0, M.s_bus[d.si[q]], &nns, &d.spos[q]);
        for (int q = 0; q < nku0; ++q) add_node(d, 0, M.d_bus[d.ku[q]], &nns, &d.kupos[q]);
        int nl = 0;
        for (int q = 0; q < nth; ++q) d.dth[d.thn[q]] = d.tha[q];
        for (int q = 0; q < nth; ++q) {
            int n = d.thn[q];
            for (int p = M.nlp[n]; p < M.nlp[n + 1]; ++p) {
                int e = M.nl[p];
                if (d.lmark[e]) continue;
                d.lmark[e] = 1;
                real df = M.lb[e] * (d.dth[M.bus0[e]] - d.dth[M.bus1[e]]);
                if (fabs(df) <= real(1e-14)) continue;
                d.li[nl] = e;
                d.ldf[nl] = df;
                ++nl;
            }
        }
        for (int q = 0; q < nl; ++q) {
            add_node(d, 0, M.bus0[d.li[q]], &nns, &d.lpa[q]);
            add_node(d, 0, M.bus1[d.li[q]], &nns, &d.lpb[q]);
        }
        for (int q = 0; q < nth; ++q) {  // reset the dense marks
            int n = d.thn[q];
            d.dth[n] = 0;
            for (int p = M.nlp[n]; p < M.nlp[n + 1]; ++p) d.lmark[M.nl[p]] = 0;
        }
        for (int q = 0; q < nga; ++q) add_node(d, 1, M.d_bus[d.gia[q]], &nna, &d.gposa[q]);
        for (int q = nku0; q < nku; ++q) add_node(d, 1, M.d_bus[d.ku[q]], &nna, &d.kupos[q]);
        for (int q = 0; q < nse; ++q) add_node(d, 1, M.s_bus[d.si[q]], &nna, &d.sposa[q]);
        for (int q = 0; q < nns; ++q) d.nmarks[d.nds[q]] = 0;
        for (int q = 0; q < nna; ++q) d.nmarka[d.nda[q]] = 0;
        h[0] = ng;
        h[1] = nse;
        h[2] = nl;
        h[3] = nk;
        h[4] = nku;
        h[5] = nns;
        h[6] = nga;
        h[7] = nna;
        h[8] = nth;
        h[9] = (ng + nse + nth + nku) > 0;
        h[10] = fam;
        h[11] = nku0;
    }
    __syncwarp();
    if (!d.hdr[9]) return -1;
    return fam;
}

// soc_qadj (src/local.jl:1826) of storage unit j over the step from state ye to ye1: nominal minus
// actual injection, k h (ye1 - ye) / dt - k (p+ - p-), the power that of soc_power (the clamped
// state-of-charge difference less the standing loss, charged through eta_in or discharged
// through eta_out up to the unit's rating)
template <class real>
__device__ inline real soc_qadj_unit(const DevModel<real> &M, int j, real ye, real ye1) {
    real ec = clampr<real>(ye, 0, 1), ec1 = clampr<real>(ye1, 0, 1);
    real dd = M.s_hours[j] * (ec1 - ec) / M.dt - M.s_qt[j];
    real pc = 0, mcx = 0;
    if (dd >= 0)
        pc = M.s_etain[j] > 0 ? dd / M.s_etain[j] : real(0);
    else
        mcx = fmin(-dd * M.s_etaout[j], real(1));
    return M.kc_s[j] * M.s_hours[j] * (ye1 - ye) / M.dt - M.kc_s[j] * (pc - mcx);
}

// per-lane part of the kinks (prorata!, src/local.jl:1782): Q, e, P per kink node (at its step,
// tau or tau - 1, with the storage adjustment where the move sets one) and the kinked
// coefficients sigma/kappa; a lane without dispatch at a node has no kink there
template <class real>
__device__ __noinline__ void lane_kinks(const Lane<real> &Ln) {
    const DevModel<real> &M = Ln.M;
    const Desc<real> &d = Ln.d;
    int nk = d.hdr[3], nku = d.hdr[4], nku0 = d.hdr[11];
    for (int q = 0; q < nk; ++q) {
        int m = d.kn[q];
        int step = d.ksd[q] ? Ln.taum : Ln.tau;
        real Pm = 0, Qs = 0;
        int nu = 0;
        for (int p = M.up[m]; p < M.up[m + 1]; ++p) {
            int j = M.ua[p];
            real kap = kappa_d(M, j);
            if (!(fabs(kap) >= M.kmin)) continue;
            real om = M.g[Ln.ix(j, step)];
            Pm += kap * om;
            Qs += kap * clampr<real>(om, 0, 1);
            nu += 1;
        }
        bool valid = nu > 0 && !(fabs(Pm) < real(1e-6));
        real qadj = 0;
        int sj = d.kqs[q];
        if (sj >= 0 && M.s_bus[sj] == m) {
            int s1 = d.ksd[q] ? Ln.tau : Ln.tau1;
            qadj = soc_qadj_unit(M, sj, M.e[Ln.ix(sj, step)], M.e[Ln.ix(sj, s1)]);
        }
        real Q = M.r[Ln.ix(m, step)] + Qs + qadj;
        Ln.S(Ln.LL.kq, q) = valid ? Q : real(0);
        Ln.S(Ln.LL.kp, q) = valid ? Pm : real(1);
        Ln.S(Ln.LL.ke, q) = valid ? Pm - fmax(Q, real(0)) : real(0);
        Ln.S(Ln.LL.knm, q) = valid ? real(nu - 1) : real(0);
        Ln.S(Ln.LL.kv, q) = valid ? real(1) : real(0);
        Ln.S(Ln.LL.kph, q) = 0;
    }
    for (int q = 0; q < nku; ++q) {
        int kq = d.kk[q];
        real ak = 0;
        if (Ln.S(Ln.LL.kv, kq) != 0) {
            int j = d.ku[q];
            real kap = kappa_d(M, j);
            real sigma = kap * M.g[Ln.ix(j, q < nku0 ? Ln.tau : Ln.taum)] / Ln.S(Ln.LL.kp, kq);
            if (sigma != 0) ak = sigma / kap;
        }
        Ln.S(Ln.LL.kua, q) = ak;
    }
}

}  // namespace esm

#include "esm_sepwalk.cuh"

namespace esm {

// ---------------------------------------------------------------------------------------------
// the kernel: one colour class of one sweep
// ---------------------------------------------------------------------------------------------
// The move list of a colour class and the descriptor of each of its moves. The list and the
// selection draws come from one stream per (class, sweep) (TAG_LIST with tile word 0), shared by
// every task of the class; the selection reads only capacities and static tables, so every
// descriptor is the same for all tasks and is built once here, by one warp, in stream order.
// Descriptor mi goes to descs + mi * stride; its header word 12 holds the family index (-1: no move).
// The body of k_prep_moves for one model, run by one warp: smem is its descriptor workspace
// (stride bytes), sd the shared Desc that carves it.
template <class real>
__device__ __forceinline__ void prep_class(const DevModel<real> &M, char *smem, Desc<real> &sd, uint32_t sweep, int cls,
                                           int nrun, char *descs, size_t stride, int lane) {
    int nmoves = M.natoms + M.nextra;
    if (lane == 0) sd = carve_desc<real>(smem, M, nmoves);
    __syncwarp();
    Desc<real> &d = sd;
    for (int i = lane; i < M.N; i += 32) {
        d.dth[i] = 0;
        d.nmarks[i] = 0;
        d.nmarka[i] = 0;
    }
    for (int i = lane; i < M.L; i += 32) d.lmark[i] = 0;
    __syncwarp();
    Stream st{M.seed, 0u, (uint32_t)cls, sweep, 0u};
    build_list(M, d, st, lane);
    for (int mi = 0; mi < nrun; ++mi) {
        int fi = prep_move(M, d, st, d.moves[mi], lane);
        if (lane == 0) d.hdr[12] = fi;
        __syncwarp();
        const int4 *src = (const int4 *)smem;
        int4 *dst = (int4 *)(descs + (size_t)mi * stride);
        for (size_t i = lane; i < stride / 16; i += 32) dst[i] = src[i];
        __syncwarp();
    }
}

template <class real>
__global__ void __launch_bounds__(32) k_prep_moves(const __grid_constant__ DevModel<real> M, const uint32_t *sweep_p, int cls,
                                                  int nrun, char *descs, size_t stride) {
    extern __shared__ __align__(16) char smem[];
    __shared__ Desc<real> sd;
    prep_class<real>(M, smem, sd, *sweep_p, cls, nrun, descs, stride, threadIdx.x);
}

// Move mi of the class (its descriptor built by k_prep_moves) for every (step, replica) task. One
// warp per block: a warp copies the descriptor to its shared memory, then takes items (32 tasks of
// a tile: span consecutive steps x replicas, replica fastest) from a per-move counter until none
// is left, and each lane walks and samples its own line conditional. One launch per move keeps
// every warp of the grid in the same code; taking items one at a time balances the warps, whose
// walks differ in length.
// Register bound per block shape (WPB warps per block, so many blocks resident per SM): one-warp
// blocks keep the registers the kernel wants (80, 24 warps per SM), two- and four-warp blocks trade
// registers for resident warps (64 and 48 registers: 32 and 40 warps per SM).
template <int WPB>
struct MoveBounds {
    static constexpr int min_blocks = WPB == 1 ? 24 : WPB == 2 ? 16 : 10;
};

// One task of move mi (family fi) at step tau for the lane's replica (Ln.rep): the kinks, the walk
// and draw of t, the Jacobian test of the compensated families and the commit. Returns the t
// taken (0: not moved); *guard on a walk buffer overflow.
template <class real>
__device__ __forceinline__ real move_task(Lane<real> &Ln, const DevModel<real> &M, const Desc<real> &d,
                                          const LaneLayout &LL, int fi, int mi, int tau, uint32_t sweep, bool *guard) {
    int T = M.T;
    Ln.tau = tau;
    Ln.taum = (Ln.tau - 1 + T) % T;
    Ln.tau1 = (Ln.tau + 1) % T;
    lane_kinks(Ln);
    double uc, uo, uj, un;
    uniform2(M.seed, ESM_TAG_LANE, 2 * (uint32_t)mi, (uint32_t)Ln.tau, (uint32_t)Ln.rep, sweep, &uc, &uo);
    real t = Ln.sample_line(unit_uniform<real>(uc), unit_uniform<real>(uo), guard);
    bool compensated = fi == ESM_FAM_XLOCC || fi == ESM_FAM_TPOT || fi == ESM_FAM_TSOC;
    if (compensated && t != 0) {  // Jacobian (logjac, src/local.jl:1871; :2041), in FP64 in both builds
        int nk = d.hdr[3];
        bool any = false;
        double lj = 0;
        for (int k = 0; k < nk; ++k) {
            if (Ln.S(LL.kv, k) == 0) continue;
            any = true;
            double Q = Ln.S(LL.kq, k);
            lj += (double)Ln.S(LL.knm, k) *
                  log(fabs((fmax(Q + (double)d.kg[k] * (double)t, 0.0) + (double)Ln.S(LL.ke, k)) / (double)Ln.S(LL.kp, k)));
        }
        if (any) {
            uniform2(M.seed, ESM_TAG_LANE, 2 * (uint32_t)mi + 1, (uint32_t)Ln.tau, (uint32_t)Ln.rep, sweep, &uj, &un);
            if (uj >= exp(fmin(0.0, lj))) t = 0;
        }
    }
    if (t != 0) Ln.commit(t);
    return t;
}

template <class real, int WPB>
__global__ void __launch_bounds__(32 * WPB, MoveBounds<WPB>::min_blocks)
    k_move(const __grid_constant__ DevModel<real> M, const int *steps, int nsteps, int ntile, int wpt,
           const uint32_t *sweep_p, int mi, const char *descs, size_t stride, real *scratch,
           unsigned long long *stats, unsigned int *next_item, int sepmin) {
    extern __shared__ __align__(16) char smem[];
    __shared__ Desc<real> sd;
    __shared__ LaneLayout sLL;
    int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    {  // the block's warps share one copy of the descriptor
        const int4 *src = (const int4 *)(descs + (size_t)mi * stride);
        int4 *dst = (int4 *)smem;
        for (size_t i = threadIdx.x; i < stride / 16; i += 32 * WPB) dst[i] = src[i];
    }
    if (threadIdx.x == 0) {
        sd = carve_desc<real>(smem, M, M.natoms + M.nextra);
        sLL = lane_layout(M.maxpts, M.maxn, M.maxstu, linemove_maxroots(M), M.maxk, M.maxku);
    }
    if (WPB == 1)
        __syncwarp();
    else
        __syncthreads();
    Desc<real> &d = sd;
    const LaneLayout &LL = sLL;
    int fi = d.hdr[12];
    if (fi < 0) return;  // not a valid move: nothing to do (grid-uniform)
    if (sep_move<real>(d, sepmin)) return;  // k_move_sep walks it (grid-uniform)
    // per-lane scratch: a local array (cached in L1, written back) when the layout fits it, else
    // the lane's column of this warp's slab in global memory
    real local[ESM_LANE_LOCAL];
    bool loc = LL.total <= ESM_LANE_LOCAL;
    real *slab = loc ? local : scratch + ((size_t)blockIdx.x * WPB + wib) * LL.total * 32 + lane;
    Lane<real> Ln(M, d, slab, loc ? 1 : 32, lane, LL);
    uint32_t sweep = *sweep_p;
    unsigned long long tried = 0, moved = 0, guards = 0;
    int nitems = ntile * wpt;
    while (true) {
        unsigned int it = 0;
        if (lane == 0) it = atomicAdd(next_item, 1u);
        int item = (int)__shfl_sync(0xffffffffu, it, 0);
        if (item >= nitems) break;
        int tile = item / wpt, grp = item % wpt;
        int task = grp * 32 + lane;
        int sit = task / M.R;
        Ln.rep = task % M.R;
        int q = tile * M.span + sit;
        if (!(sit < M.span && q < nsteps)) continue;
        bool guard;
        real t = move_task<real>(Ln, M, d, LL, fi, mi, steps[q], sweep, &guard);
        if (guard) ++guards;
        if (M.mlog && Ln.rep < M.mlog_nrep) M.mlog[((size_t)mi * nsteps + q) * M.mlog_nrep + Ln.rep] = (double)t;
        ++tried;
        if (t != 0) ++moved;
    }
    // per-warp counts (tasks tried / moved, guard events) into the class totals
    for (int o = 16; o > 0; o >>= 1) {
        tried += __shfl_xor_sync(0xffffffffu, tried, o);
        moved += __shfl_xor_sync(0xffffffffu, moved, o);
        guards += __shfl_xor_sync(0xffffffffu, guards, o);
    }
    if (lane == 0) {
        if (tried) atomicAdd(&stats[2 * fi], tried);
        if (moved) atomicAdd(&stats[2 * fi + 1], moved);
        if (guards) atomicAdd(&stats[2 * (ESM_NFAM + 1)], guards);
    }
}

// ---------------------------------------------------------------------------------------------
// the whole class in one launch: items of consecutive moves overlap
// ---------------------------------------------------------------------------------------------
__device__ inline unsigned int ld_acquire_u32(const unsigned int *p) {
    unsigned int v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ inline void st_release_u32(unsigned int *p, unsigned int v) {
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ inline unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// The moves of a class pass take no barrier between them: the tasks of a colour class are
// independent (a move at step tau writes steps tau and tau - 1, which no other task of the class
// reads or writes), so a task's move mi + 1 needs only its own move mi. k_move_wave runs the whole
// class in one launch: its warps take (move, item) pairs from one counter in move-major order,
// wait until the item's previous move is published in done[item] (moves completed), run the 32
// tasks exactly as k_move does (move_task), and publish. A warp waits only on an earlier-taken
// pair, held by a running warp, so the earliest unfinished pair never waits and the pass always
// progresses; the waits are still bounded (a pair whose predecessor is not published within
// ESM_WAVE_WAIT_NS sets *err and every warp leaves). The descriptor of a warp's move is read from
// the descriptor buffer in global memory (read-only during the pass), so warps of one block may
// run different moves. One launch replaces a pass's per-move launches and the idle tail each of
// them ends with (8760 items over ~4900 resident warps at T = 8760, 64 replicas: under two items
// per warp and move).
#define ESM_WAVE_WAIT_NS 2000000000ull
template <class real, int WPB>
__global__ void __launch_bounds__(32 * WPB, MoveBounds<WPB>::min_blocks)
    k_move_wave(const __grid_constant__ DevModel<real> M, const int *steps, int nsteps, int ntile, int wpt,
                const uint32_t *sweep_p, int nrun, const char *descs, size_t stride, real *scratch,
                unsigned long long *stats, unsigned int *next, unsigned int *done, int *err) {
    __shared__ Desc<real> sd[WPB];
    __shared__ LaneLayout sLL;
    int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    if (threadIdx.x == 0) sLL = lane_layout(M.maxpts, M.maxn, M.maxstu, linemove_maxroots(M), M.maxk, M.maxku);
    if (WPB == 1)
        __syncwarp();
    else
        __syncthreads();
    const LaneLayout &LL = sLL;
    real local[ESM_LANE_LOCAL];
    bool loc = LL.total <= ESM_LANE_LOCAL;
    real *slab = loc ? local : scratch + ((size_t)blockIdx.x * WPB + wib) * LL.total * 32 + lane;
    Lane<real> Ln(M, sd[wib], slab, loc ? 1 : 32, lane, LL);
    uint32_t sweep = *sweep_p;
    const unsigned int nitems = (unsigned int)(ntile * wpt);
    const unsigned int total = nitems * (unsigned int)nrun;  // (the host keeps it below 2^32)
    const int nmoves = M.natoms + M.nextra;
    int cur = -1, fi = -1;
    unsigned long long tried = 0, moved = 0, guards = 0;
    while (true) {
        unsigned int g = 0;
        if (lane == 0) g = atomicAdd(next, 1u);
        g = __shfl_sync(0xffffffffu, g, 0);
        bool stop = g >= total || *(volatile int *)err != 0;
        int mi = stop ? cur : (int)(g / nitems);
        if (stop || mi != cur) {  // warp-uniform: add the counts of the previous move
            for (int o = 16; o > 0; o >>= 1) {
                tried += __shfl_xor_sync(0xffffffffu, tried, o);
                moved += __shfl_xor_sync(0xffffffffu, moved, o);
                guards += __shfl_xor_sync(0xffffffffu, guards, o);
            }
            if (lane == 0 && fi >= 0) {
                if (tried) atomicAdd(&stats[2 * fi], tried);
                if (moved) atomicAdd(&stats[2 * fi + 1], moved);
                if (guards) atomicAdd(&stats[2 * (ESM_NFAM + 1)], guards);
            }
            tried = moved = guards = 0;
            if (stop) break;
            if (lane == 0) sd[wib] = carve_desc<real>((char *)descs + (size_t)mi * stride, M, nmoves);
            __syncwarp();
            cur = mi;
            fi = sd[wib].hdr[12];
        }
        unsigned int item = g - (unsigned int)mi * nitems;
        if (mi > 0) {  // the item's previous move, published by the warp that ran it
            bool ok = true;
            if (lane == 0) {
                unsigned long long t0 = 0;
                while (ld_acquire_u32(&done[item]) < (unsigned int)mi) {
                    if (*(volatile int *)err != 0) {
                        ok = false;
                        break;
                    }
                    unsigned long long t = global_ns();
                    if (t0 == 0)
                        t0 = t;
                    else if (t - t0 > ESM_WAVE_WAIT_NS) {
                        atomicExch(err, 1);
                        ok = false;
                        break;
                    }
                    __nanosleep(128);
                }
            }
            // the barrier of the shuffle orders every lane's loads after lane 0's acquire
            ok = __shfl_sync(0xffffffffu, ok, 0);
            if (!ok) break;
        }
        if (fi >= 0) {
            int tile = (int)(item / wpt), grp = (int)(item % wpt);
            int task = grp * 32 + lane;
            int sit = task / M.R;
            int q = tile * M.span + sit;
            if (sit < M.span && q < nsteps) {
                Ln.rep = task % M.R;
                bool guard;
                real t = move_task<real>(Ln, M, sd[wib], LL, fi, mi, steps[q], sweep, &guard);
                if (guard) ++guards;
                if (M.mlog && Ln.rep < M.mlog_nrep)
                    M.mlog[((size_t)mi * nsteps + q) * M.mlog_nrep + Ln.rep] = (double)t;
                ++tried;
                if (t != 0) ++moved;
            }
        }
        __threadfence();  // every lane's state writes before the publish
        __syncwarp();
        if (lane == 0) st_release_u32(&done[item], (unsigned int)mi + 1);
    }
}

// ---------------------------------------------------------------------------------------------
// host launcher
// ---------------------------------------------------------------------------------------------
template <class real>
size_t linemove_scratch_reals(const DevModel<real> &M) {
    LaneLayout LL = lane_layout(M.maxpts, M.maxn, M.maxstu, linemove_maxroots(M), M.maxk, M.maxku);
    return LL.total <= ESM_LANE_LOCAL ? 0 : (size_t)LL.total * 32;  // 0: the lanes' local arrays suffice
}

// bytes of one move descriptor (the per-move buffer stride and the dynamic shared memory of k_move)
template <class real>
size_t linemove_smem_per_warp(const DevModel<real> &M) {
    return (desc_bytes(M, M.natoms + M.nextra) + 15) & ~(size_t)15;
}

// warps of k_move resident per SM with blocks of wpb warps (1, 2 or 4), for the grid and scratch
// of a context
template <class real>
int linemove_blocks_per_sm(const DevModel<real> &M, int wpb) {
    int nb = 0;
    size_t stride = linemove_smem_per_warp(M);
    // (the dynamic shared memory limits are set here, at context creation, so that no later call --
    // possibly under stream capture -- has to)
    cudaFuncSetAttribute(k_prep_moves<real>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    cudaError_t e;
    if (wpb == 4) {
        cudaFuncSetAttribute(k_move<real, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_move<real, 4>, 128, stride);
    } else if (wpb == 2) {
        cudaFuncSetAttribute(k_move<real, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_move<real, 2>, 64, stride);
    } else {
        cudaFuncSetAttribute(k_move<real, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_move<real, 1>, 32, stride);
    }
    if (e != cudaSuccess || nb < 1) nb = 16 / wpb;
    return nb * wpb;
}

// The cooperative walk of the separable moves (k_move_sep, two-warp blocks): its per-warp region,
// and whether two regions and the descriptor fit in a block's shared memory (else global slabs).
template <class real>
size_t sep_region_bytes(const DevModel<real> &M) {
    return (size_t)sep_layout<real>(M.maxstu, M.maxpts).total;
}

template <class real>
int sep_warps_per_sm(const DevModel<real> &M, int *in_smem) {
    size_t stride = linemove_smem_per_warp(M);
    size_t per = sep_region_bytes(M);
    size_t smem = stride + 2 * per;
    *in_smem = smem <= 200 * 1024;
    if (!*in_smem) smem = stride;
    cudaFuncSetAttribute(k_move_sep<real, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    int nb = 0;
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_move_sep<real, 2>, 64, smem);
    if (e != cudaSuccess || nb < 1) nb = 1;
    return 2 * nb;
}

template <class real>
cudaError_t launch_class_pass(const DevModel<real> &M, const int *steps, int nsteps, const uint32_t *sweep, int cls,
                              int limit, real *scratch, int wpb, int max_warps, unsigned long long *stats,
                              char *descs, unsigned int *counters, const SepLaunch &sep, const WaveLaunch &wave,
                              cudaStream_t s) {
    int nmoves = M.natoms + M.nextra;
    int nrun = limit > 0 && limit < nmoves ? limit : nmoves;
    size_t stride = linemove_smem_per_warp(M);
    cudaError_t e = cudaMemsetAsync(counters, 0, sizeof(unsigned int) * nrun, s);
    if (e != cudaSuccess) return e;
    k_prep_moves<real><<<1, 32, stride, s>>>(M, sweep, cls, nrun, descs, stride);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    int ntile = (nsteps + M.span - 1) / M.span;
    int wpt = (M.span * M.R + 31) / 32;
    int items = ntile * wpt;
    int warps = items < max_warps ? items : max_warps;
    int blocks = (warps + wpb - 1) / wpb;
    if (wave.on && sep.min_units == 0 && (size_t)items <= wave.max_items &&
        (unsigned long long)items * nrun < (1ull << 32)) {
        if ((e = cudaMemsetAsync(wave.done, 0, sizeof(unsigned int) * items, s)) != cudaSuccess) return e;
        if (wpb == 4)
            k_move_wave<real, 4><<<blocks, 128, 0, s>>>(M, steps, nsteps, ntile, wpt, sweep, nrun, descs, stride,
                                                       scratch, stats, counters, wave.done, wave.err);
        else if (wpb == 2)
            k_move_wave<real, 2><<<blocks, 64, 0, s>>>(M, steps, nsteps, ntile, wpt, sweep, nrun, descs, stride,
                                                      scratch, stats, counters, wave.done, wave.err);
        else
            k_move_wave<real, 1><<<blocks, 32, 0, s>>>(M, steps, nsteps, ntile, wpt, sweep, nrun, descs, stride,
                                                      scratch, stats, counters, wave.done, wave.err);
        return cudaGetLastError();
    }
    int sepmin = sep.min_units;
    int ntask = nsteps * M.R;
    int swarps = ntask < sep.max_warps ? ntask : sep.max_warps;
    int sblocks = (swarps + 1) / 2;
    size_t ssmem = stride + (sep.in_smem ? 2 * sep_region_bytes(M) : 0);
    for (int mi = 0; mi < nrun; ++mi) {
        if (wpb == 4)
            k_move<real, 4><<<blocks, 128, stride, s>>>(M, steps, nsteps, ntile, wpt, sweep, mi, descs, stride, scratch,
                                                       stats, counters + mi, sepmin);
        else if (wpb == 2)
            k_move<real, 2><<<blocks, 64, stride, s>>>(M, steps, nsteps, ntile, wpt, sweep, mi, descs, stride, scratch,
                                                      stats, counters + mi, sepmin);
        else
            k_move<real, 1><<<blocks, 32, stride, s>>>(M, steps, nsteps, ntile, wpt, sweep, mi, descs, stride, scratch,
                                                      stats, counters + mi, sepmin);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
        if (sepmin > 0 && sblocks > 0) {
            k_move_sep<real, 2><<<sblocks, 64, ssmem, s>>>(M, steps, nsteps, sweep, mi, descs, stride, sepmin,
                                                          sep.in_smem, sep.slab, stats, counters + mi);
            if ((e = cudaGetLastError()) != cudaSuccess) return e;
        }
    }
    return cudaSuccess;
}

// ---------------------------------------------------------------------------------------------
// a batch of models
// ---------------------------------------------------------------------------------------------
// Pass p of every model of a batch: block b builds the descriptors of the class that model b runs
// in pass p of the sweep (its own class order, class_order_of), exactly as k_prep_moves does for
// the model alone; block 0 also writes every model's class of the pass and the pass's item prefix
// over the models (items: the model's tiles of its class x the warps of a tile).
template <class real>
__global__ void __launch_bounds__(32) k_prep_batch(const BatchModel<real> *bm, int nm, const uint32_t *sweep_p, int p,
                                                   int *pass_cls, unsigned int *off) {
    extern __shared__ __align__(16) char smem[];
    __shared__ Desc<real> sd;
    int b = blockIdx.x, lane = threadIdx.x;
    uint32_t sweep = *sweep_p;
    const BatchModel<real> &B = bm[b];
    int order[3], ncls;
    class_order_of(B.M.seed, B.M.T, sweep, order, &ncls);
    if (b == 0 && lane == 0) {
        unsigned int acc = 0;
        off[0] = 0;
        for (int q = 0; q < nm; ++q) {
            const BatchModel<real> &Q = bm[q];
            int oq[3], nq;
            class_order_of(Q.M.seed, Q.M.T, sweep, oq, &nq);
            int c = p < nq ? oq[p] : -1;
            pass_cls[q] = c;
            if (c >= 0 && Q.nsteps[c] > 0) {
                int ntile = (Q.nsteps[c] + Q.M.span - 1) / Q.M.span;
                int wpt = (Q.M.span * Q.M.R + 31) / 32;
                acc += (unsigned int)(ntile * wpt);
            }
            off[q + 1] = acc;
        }
    }
    if (p >= ncls || B.nsteps[order[p]] == 0) return;
    prep_class<real>(B.M, smem, sd, sweep, order[p], B.nmoves, B.descs, B.stride, lane);
}

// Move mi of the current pass for every task of the first nact models of the batch. A warp takes
// items from the launch's counter; an item (32 tasks of one model's tile, as in k_move) belongs to
// the model b with off[b] <= item < off[b + 1]. When a warp's item comes from another model than
// its last one, the warp copies that model's tables and layout into its shared memory and points
// its descriptor at the model's descriptor mi in global memory (read-only during the move), after
// adding its counts so far to the previous model's statistics. Each task then runs exactly the
// arithmetic of k_move (move_task), so a model's state after a batch pass is the state its own
// class pass gives. The cooperative walk of separable moves is not used in a batch.
template <class real, int WPB>
__global__ void __launch_bounds__(32 * WPB, MoveBounds<WPB>::min_blocks)
    k_move_batch(const BatchModel<real> *bm, int nact, const int *pass_cls, const unsigned int *off,
                 const uint32_t *sweep_p, int mi, real *scratch, size_t scratch_per_warp, unsigned int *next_item) {
    __shared__ DevModel<real> sM[WPB];
    __shared__ Desc<real> sd[WPB];
    __shared__ LaneLayout sLL[WPB];
    int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    uint32_t sweep = *sweep_p;
    unsigned int total = off[nact];
    real local[ESM_LANE_LOCAL];
    int cur = -1, fi = -1, cls = 0, nsteps = 0;
    const int *steps = nullptr;
    unsigned long long tried = 0, moved = 0, guards = 0;
    while (true) {
        unsigned int it = 0;
        if (lane == 0) it = atomicAdd(next_item, 1u);
        unsigned int item = __shfl_sync(0xffffffffu, it, 0);
        bool done = item >= total;
        int b = cur;
        if (!done) {  // the last model whose prefix is <= item
            int lo = 0, hi = nact - 1;
            while (lo < hi) {
                int mid = (lo + hi + 1) >> 1;
                if (off[mid] <= item)
                    lo = mid;
                else
                    hi = mid - 1;
            }
            b = lo;
        }
        if (done || b != cur) {  // warp-uniform
            for (int o = 16; o > 0; o >>= 1) {
                tried += __shfl_xor_sync(0xffffffffu, tried, o);
                moved += __shfl_xor_sync(0xffffffffu, moved, o);
                guards += __shfl_xor_sync(0xffffffffu, guards, o);
            }
            if (lane == 0 && cur >= 0 && fi >= 0) {
                unsigned long long *st = bm[cur].stats;
                if (tried) atomicAdd(&st[2 * fi], tried);
                if (moved) atomicAdd(&st[2 * fi + 1], moved);
                if (guards) atomicAdd(&st[2 * (ESM_NFAM + 1)], guards);
            }
            tried = moved = guards = 0;
            if (done) break;
            const unsigned int *src = (const unsigned int *)&bm[b].M;
            unsigned int *dst = (unsigned int *)&sM[wib];
            for (int i = lane; i < (int)(sizeof(DevModel<real>) / 4); i += 32) dst[i] = src[i];
            __syncwarp();
            if (lane == 0) {
                sd[wib] = carve_desc<real>(bm[b].descs + (size_t)mi * bm[b].stride, sM[wib], bm[b].nmoves);
                const DevModel<real> &Mb = sM[wib];
                sLL[wib] = lane_layout(Mb.maxpts, Mb.maxn, Mb.maxstu, linemove_maxroots(Mb), Mb.maxk, Mb.maxku);
            }
            __syncwarp();
            cur = b;
            fi = sd[wib].hdr[12];
            cls = pass_cls[b];
            nsteps = cls >= 0 ? bm[b].nsteps[cls] : 0;
            steps = cls >= 0 ? bm[b].steps[cls] : nullptr;
        }
        if (fi < 0) continue;  // the model's move mi is not a valid move: its tasks do nothing
        const DevModel<real> &M = sM[wib];
        const LaneLayout &LL = sLL[wib];
        unsigned int li = item - off[b];
        int wpt = (M.span * M.R + 31) / 32;
        int tile = (int)(li / wpt), grp = (int)(li % wpt);
        int task = grp * 32 + lane;
        int sit = task / M.R;
        int q = tile * M.span + sit;
        if (!(sit < M.span && q < nsteps)) continue;
        bool loc = LL.total <= ESM_LANE_LOCAL;
        real *slab = loc ? local : scratch + ((size_t)blockIdx.x * WPB + wib) * scratch_per_warp + lane;
        Lane<real> Ln(M, sd[wib], slab, loc ? 1 : 32, lane, LL);
        Ln.rep = task % M.R;
        bool guard;
        real t = move_task<real>(Ln, M, sd[wib], LL, fi, mi, steps[q], sweep, &guard);
        if (guard) ++guards;
        ++tried;
        if (t != 0) ++moved;
    }
}

template <class real>
int batch_warps_per_sm(int wpb) {
    int nb = 0;
    cudaError_t e;
    cudaFuncSetAttribute(k_prep_batch<real>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    if (wpb == 2)
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_move_batch<real, 2>, 64, 0);
    else
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_move_batch<real, 1>, 32, 0);
    if (e != cudaSuccess || nb < 1) nb = 16 / wpb;
    return nb * wpb;
}

template <class real>
cudaError_t launch_batch_passes(const BatchModel<real> *bm, const BatchLaunch &bl, const uint32_t *sweep,
                                cudaStream_t s) {
    cudaError_t e = cudaMemsetAsync(bl.counters, 0, sizeof(unsigned int) * bl.maxpass * bl.maxmoves, s);
    if (e != cudaSuccess) return e;
    int blocks = (bl.warps + bl.wpb - 1) / bl.wpb;
    for (int p = 0; p < bl.npass; ++p) {
        int *pc = bl.pass_cls + (size_t)p * bl.nm;
        unsigned int *off = bl.off + (size_t)p * (bl.nm + 1);
        k_prep_batch<real><<<bl.nm, 32, bl.prep_smem, s>>>(bm, bl.nm, sweep, p, pc, off);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
        for (int mi = 0; mi < bl.nmove; ++mi) {
            unsigned int *ctr = bl.counters + (size_t)p * bl.maxmoves + mi;
            if (bl.wpb == 2)
                k_move_batch<real, 2><<<blocks, 64, 0, s>>>(bm, bl.nact[mi], pc, off, sweep, mi, (real *)bl.scratch,
                                                           bl.scratch_per_warp, ctr);
            else
                k_move_batch<real, 1><<<blocks, 32, 0, s>>>(bm, bl.nact[mi], pc, off, sweep, mi, (real *)bl.scratch,
                                                           bl.scratch_per_warp, ctr);
            if ((e = cudaGetLastError()) != cudaSuccess) return e;
        }
    }
    return cudaSuccess;
}

}  // namespace esm
