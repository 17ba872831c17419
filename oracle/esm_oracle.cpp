/*
 * CPU ORACLE of the replica-sampler hot path -- TEST INFRASTRUCTURE ONLY.
 *
 * A plain FP64 restatement of the reference's algorithms (FHell/ESM-Sampling, Julia), function by
 * function, for the synthetic model of this repository (no losses, soft limits, links, unit
 * commitment, vintages or weather entries: the cacheable "plain model" of src/local.jl:984).
 * It is the checker of the CUDA library and the timed CPU baseline; nothing in the product links
 * or calls it. Random numbers follow the Philox stream contract of philox.h, so that the CUDA
 * path can be replayed move by move.
 *
 * Reference files cited as path:line within the reference project.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include "../include/esmcuda.h"
#include "philox.h"

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

using std::vector;

// ------------------------------------------------------------------------------------------
// model copy
// ------------------------------------------------------------------------------------------
struct Model {
    int N, L, T, K, D, S, n0, nreg, nfields, nlev;
    double dt, c_shed, c_dump, c_viol, gamma_k, kappa0, beta_v, beta_k;
    bool physical;
    vector<int> bus0, bus1;
    vector<double> lb, ls;
    vector<int> ukind, ugroup, ubus, useries;
    vector<double> umc, ucapex, ulo, uhi, uavail, uhours, uetain, uetaout, uqt;
    vector<int> disp, stor;
    vector<int> sfield, snode;
    vector<double> xbar, wscale, Ptr, pi0, phi, mu, sig, sig0;
    vector<int> frole, fap, ap, ai;
    vector<double> av;
    vector<int> nlp, nl, up, ua, sp, sa;
    vector<double> qcum;
    vector<int> clp, cp, cu;
    vector<int> xpp, xp, xnp, xn, xlp, xln;
    vector<double> xv, xlg, Z;
    vector<int> comp;
    vector<int> sgp, sgu;   // storage groups (country cell, carrier) -> indices into stor
    vector<int> theta_nnz;  // theta atoms touching node n
    vector<int> disp_of_unit, stor_of_unit;
};

template <class T>
static vector<T> cp_(const T *p, size_t n) {
    return p ? vector<T>(p, p + n) : vector<T>(n, T(0));
}

struct Opts {
    int R, max_points, span;
    uint64_t seed;
    double extra, maxnats, kmin;
    double rates[ESM_NFAM];
    int storage_ms, storage_long;
};

struct Ctx {
    Model m;
    Opts o;
    // state (X, T, R), replica fastest
    vector<double> theta, g, e, z, k, r, F;
    vector<int> reg;
    vector<double> sk_last, fk_last;  // scores of the last capacity_scores call
    bool has_scores = false;
    int64_t sms_stats[3] = {0, 0, 0};  // storage multiscale moves of orc_sweeps: tried, taken, guards
};

static inline size_t ix(const Ctx &c, int x, int t, int rep) {
    return ((size_t)x * c.m.T + t) * c.o.R + rep;
}
static inline double clampd(double x, double lo, double hi) { return x < lo ? lo : (x > hi ? hi : x); }
static inline double kcl(const Ctx &c, int u) { return clampd(c.k[u], c.m.ulo[u], c.m.uhi[u]); }

// weather data map (src/energy.jl:515 datamap; the logistic availability map is the builder
// decision of the synthetic model)
static inline double wraw(const Ctx &c, int s, int t, int rep) {
    return c.m.xbar[(size_t)s * c.m.T + t] + c.m.wscale[s] * c.z[ix(c, s, t, rep)];
}
static inline double avail_map(double x) { return 1.0 / (1.0 + exp(-x)); }
static inline double load_map(double x) { return x > 0.0 ? x : 0.0; }

// ------------------------------------------------------------------------------------------
// cost pieces (src/local.jl:760 gen_cost, src/energy.jl:448 soc_cost, src/local.jl:773 phibal)
// ------------------------------------------------------------------------------------------
static inline double gen_cost(double mc, double A, double k, double w, double dt, double cv, double y, double *p) {
    double yc = clampd(y, 0.0, 1.0);
    *p = A * k * yc;
    return dt * mc * (*p) + cv * dt * w * fabs(y - yc);
}

static inline double soc_cost(const Model &m, int u, double k, double w, double dt, double cv, double ye, double ye1,
                              double *dout, double *jout) {
    double ec = clampd(ye, 0.0, 1.0), ec1 = clampd(ye1, 0.0, 1.0);
    double h = m.uhours[u];
    double d = h * (ec1 - ec) / dt - m.uqt[u];
    double eta = m.uetain[u];
    double pc, mcx;
    if (d >= 0) {
        pc = eta > 0 ? d / eta : 0.0;
        mcx = 0.0;
    } else {
        pc = 0.0;
        mcx = std::min(-d * m.uetaout[u], 1.0);
    }
    double c = dt * m.umc[u] * k * (pc + mcx) + cv * w * h * fabs(ye - ec);
    if (pc > 1) c += cv * dt * w * (pc - 1);
    if (d < 0 && m.uqt[u] <= 0) {
        double ex = -d * m.uetaout[u] - 1.0;
        if (ex > 0) c += cv * dt * w * ex;
    }
    if (d >= 0 && eta <= 0) c += cv * dt * w * d;
    *dout = d;
    *jout = k * (pc - mcx);
    return c;
}

// soc_power (src/energy.jl:437)
static inline void soc_power(const Model &m, int u, double dt, double ec, double ec1, double *pc, double *mcx) {
    double d = m.uhours[u] * (ec1 - ec) / dt - m.uqt[u];
    if (d >= 0) {
        *pc = m.uetain[u] > 0 ? d / m.uetain[u] : 0.0;
        *mcx = 0.0;
    } else {
        *pc = 0.0;
        *mcx = std::min(-d * m.uetaout[u], 1.0);
    }
}

static inline double phibal(const Model &m, double x) { return x > 0 ? m.c_shed * x : -m.c_dump * x; }

// logseg (src/local.jl:1099), trexp_offset (src/local.jl:1106) with the uniform given
static inline double logseg(double L, double x) {
    if (fabs(x) < 1e-10) return log(L) - x / 2;
    if (x > 0) return log(L) + log(-expm1(-x)) - log(x);
    return log(L) - x + log(-expm1(x)) - log(-x);
}
static inline double trexp_offset(double u, double g, double L) {
    double x = g * L;
    if (fabs(x) < 1e-10) return u * L;
    if (g > 0) return -log1p(-u * (-expm1(-x))) / g;
    return L + log1p(-u * (-expm1(x))) / (-g);
}

// ------------------------------------------------------------------------------------------
// caches: LocalCost / rebuild_step! (src/local.jl:313-374)
// ------------------------------------------------------------------------------------------
static void rebuild_step(Ctx &c, int t, int rep) {
    const Model &m = c.m;
    int T = m.T;
    for (int n = 0; n < m.N; ++n) c.r[ix(c, n, t, rep)] = load_map(wraw(c, n, t, rep));
    for (int e = 0; e < m.L; ++e) {
        int a = m.bus0[e], b = m.bus1[e];
        double fl = m.lb[e] * (c.theta[ix(c, a, t, rep)] - c.theta[ix(c, b, t, rep)]);
        c.F[ix(c, e, t, rep)] = fl;
        c.r[ix(c, a, t, rep)] += fl + 0.5 * 0.0;
        c.r[ix(c, b, t, rep)] += -fl + 0.5 * 0.0;
    }
    for (int u = 0; u < m.K; ++u) {  // generators in group order (renewables, dispatchable)
        if (m.ukind[u] == ESM_UNIT_STOR) continue;
        double A, y;
        if (m.ukind[u] == ESM_UNIT_REN) {
            A = avail_map(wraw(c, m.useries[u], t, rep));
            y = 1.0;
        } else {
            A = m.uavail[u];
            y = clampd(c.g[ix(c, m.disp_of_unit[u], t, rep)], 0.0, 1.0);
        }
        c.r[ix(c, m.ubus[u], t, rep)] -= A * kcl(c, u) * y;
    }
    for (int j = 0; j < m.S; ++j) {
        int u = m.stor[j];
        double pc, mcx;
        soc_power(m, u, m.dt, clampd(c.e[ix(c, j, t, rep)], 0.0, 1.0), clampd(c.e[ix(c, j, (t + 1) % T, rep)], 0.0, 1.0),
                  &pc, &mcx);
        c.r[ix(c, m.ubus[u], t, rep)] += kcl(c, u) * (pc - mcx);
    }
}

static void rebuild(Ctx &c, int nthreads) {
    int T = c.m.T, R = c.o.R;
#pragma omp parallel for schedule(static) num_threads(nthreads)
    for (int q = 0; q < T * R; ++q) rebuild_step(c, q / R, q % R);
}

// ------------------------------------------------------------------------------------------
// move workspace (MoveWS, src/local.jl:451) restricted to the plain model
// ------------------------------------------------------------------------------------------
enum { EK_THETA = 0, EK_GEN = 1, EK_SE = 2 };
struct Ent {
    int kind, idx;
    double a, ak;
    int kid;
};
struct Kink {
    double Q, g, phi, Pm, e, nm;
};
struct WS {
    int tau;
    vector<Ent> ent;
    vector<int> pos[3];  // entry position per (kind, idx), -1 none
    vector<Kink> kinks;
    vector<int> lines;
    vector<char> lmark;
    vector<double> dfl;
    vector<int> nodes;
    vector<char> nmark;
    vector<double> dr;
    vector<int> stu;
    vector<char> smark;
    vector<double> bps, sec;
    void init(const Model &m) {
        pos[0].assign(m.N, -1);
        pos[1].assign(m.D, -1);
        pos[2].assign(m.S, -1);
        lmark.assign(m.L, 0);
        dfl.assign(m.L, 0.0);
        nmark.assign(m.N, 0);
        dr.assign(m.N, 0.0);
        smark.assign(m.S, 0);
    }
    void clear() {  // clear! (src/local.jl:536)
        for (auto &en : ent) pos[en.kind][en.idx] = -1;
        ent.clear();
        kinks.clear();
        for (int e : lines) lmark[e] = 0;
        lines.clear();
        for (int n : nodes) {
            nmark[n] = 0;
            dr[n] = 0.0;
        }
        nodes.clear();
        for (int s : stu) smark[s] = 0;
        stu.clear();
        bps.clear();
        sec.clear();
    }
    double dy(int kind, int idx) const {
        int p = pos[kind][idx];
        return p < 0 ? 0.0 : ent[p].a;
    }
    Ent *find_or_add(int kind, int idx) {
        int &p = pos[kind][idx];
        if (p < 0) {
            p = (int)ent.size();
            ent.push_back(Ent{kind, idx, 0.0, 0.0, -1});
        }
        return &ent[p];
    }
    void add_entry(int kind, int idx, double a) {  // add_entry! (src/local.jl:558)
        if (a == 0.0) return;
        find_or_add(kind, idx)->a += a;
    }
    void add_kentry(int j, double a, int kid) {  // add_kentry! (src/local.jl:583)
        if (a == 0.0) return;
        Ent *en = find_or_add(EK_GEN, j);
        en->kid = kid;
        en->ak += a;
    }
    void touch(int n) {
        if (nmark[n]) return;
        nmark[n] = 1;
        nodes.push_back(n);
    }
};

static inline double yval(const Ctx &c, int kind, int idx, int t, int rep) {
    if (kind == EK_THETA) return c.theta[ix(c, idx, t, rep)];
    if (kind == EK_GEN) return c.g[ix(c, idx, t, rep)];
    return c.e[ix(c, idx, t, rep)];
}
static inline int ent_bus(const Model &m, int kind, int idx) {
    if (kind == EK_THETA) return idx;
    if (kind == EK_GEN) return m.ubus[m.disp[idx]];
    return m.ubus[m.stor[idx]];
}

// finalize! (src/local.jl:656), plain model
static void finalize_ws(const Ctx &c, WS &w, int rep) {
    const Model &m = c.m;
    int t = w.tau;
    for (auto &k : w.kinks)
        if (k.g != 0.0) w.bps.push_back(-k.Q / k.g);
    for (auto &en : w.ent) {
        double a = en.a, ak = en.ak;
        if (fabs(a) < 1e-14) {
            en.a = 0.0;
            a = 0.0;
        }
        if (a == 0.0 && ak == 0.0) continue;
        double y0 = yval(c, en.kind, en.idx, t, rep);
        if (ak != 0.0) {
            w.touch(ent_bus(m, en.kind, en.idx));
            const Kink &k = w.kinks[en.kid];
            double Q = k.Q, gk = k.g;
            double offs[4][2] = {{0.0, a + ak * gk}, {0.0, a}, {-ak * Q, a}, {ak * Q, a + ak * gk}};
            for (auto &os : offs) {
                double off = os[0], sl = os[1];
                if (sl == 0.0) continue;
                w.bps.push_back((0.0 - y0 - off) / sl);
                w.bps.push_back((1.0 - y0 - off) / sl);
            }
            continue;
        }
        if (en.kind == EK_THETA) {
            for (int q = m.nlp[en.idx]; q < m.nlp[en.idx + 1]; ++q) {
                int e = m.nl[q];
                if (!w.lmark[e]) {
                    w.lmark[e] = 1;
                    w.lines.push_back(e);
                }
            }
            continue;
        }
        w.bps.push_back((0.0 - y0) / a);
        w.bps.push_back((1.0 - y0) / a);
        if (en.kind == EK_GEN) {
            w.touch(ent_bus(m, en.kind, en.idx));
        } else {
            if (!w.smark[en.idx]) {
                w.smark[en.idx] = 1;
                w.stu.push_back(en.idx);
            }
            w.touch(ent_bus(m, en.kind, en.idx));
        }
    }
    size_t keep = 0;
    for (size_t q = 0; q < w.lines.size(); ++q) {
        int e = w.lines[q];
        int a = m.bus0[e], b = m.bus1[e];
        double df = m.lb[e] * (w.dy(EK_THETA, a) - w.dy(EK_THETA, b));
        if (fabs(df) <= 1e-14) {
            w.lmark[e] = 0;
            continue;
        }
        w.lines[keep++] = e;
        w.dfl[e] = df;
        w.touch(a);
        w.touch(b);
        double f0 = c.F[ix(c, e, t, rep)];
        double se = m.ls[e];
        w.bps.push_back((1.0 * se - f0) / df);
        w.bps.push_back((-1.0 * se - f0) / df);
    }
    w.lines.resize(keep);
}

// link_soc! (src/local.jl:630)
static void link_soc(const Model &m, WS &wa, const WS &wb) {
    for (auto &en : wb.ent) {
        if (en.kind != EK_SE) continue;
        if (en.a == 0.0) continue;
        if (!wa.smark[en.idx]) {
            wa.smark[en.idx] = 1;
            wa.stu.push_back(en.idx);
        }
        wa.touch(m.ubus[m.stor[en.idx]]);
    }
}

// eval_move! / eval_cached! (src/local.jl:789, :926) for one step workspace
static double eval_ws(const Ctx &c, WS &w, int rep, double t, const WS *next, vector<double> &sec) {
    const Model &m = c.m;
    int tau = w.tau, T = m.T;
    double dt = m.dt, cv = m.c_viol, k0 = m.kappa0;
    double D = 0.0;
    for (int n : w.nodes) w.dr[n] = 0.0;
    for (auto &k : w.kinks) k.phi = std::max(k.Q + k.g * t, 0.0) - std::max(k.Q, 0.0);
    for (auto &en : w.ent) {
        if (en.kind != EK_GEN) continue;
        if (en.a == 0.0 && en.kid < 0) continue;
        int u = m.disp[en.idx];
        double y0 = c.g[ix(c, en.idx, tau, rep)];
        double k = kcl(c, u), A = m.uavail[u];
        double y1 = y0 + (t * en.a + (en.kid >= 0 ? en.ak * w.kinks[en.kid].phi : 0.0));
        double p0, p1;
        double c0 = gen_cost(m.umc[u], A, k, k + k0, dt, cv, y0, &p0);
        double c1 = gen_cost(m.umc[u], A, k, k + k0, dt, cv, y1, &p1);
        D += c1 - c0;
        w.dr[m.ubus[u]] -= p1 - p0;
    }
    for (int e : w.lines) {
        double df = w.dfl[e];
        double f0 = c.F[ix(c, e, tau, rep)], f1 = f0 + t * df;
        double se = m.ls[e];
        D += cv * dt * (std::max(fabs(f1) - se, 0.0) - std::max(fabs(f0) - se, 0.0));
        w.dr[m.bus0[e]] += f1 - f0;
        w.dr[m.bus1[e]] -= f1 - f0;
    }
    int t1 = (tau + 1) % T;
    for (int j : w.stu) {
        int u = m.stor[j];
        double k = kcl(c, u), ww = k + k0;
        double ye = c.e[ix(c, j, tau, rep)], ye1 = c.e[ix(c, j, t1, rep)];
        double dye1 = next ? next->dy(EK_SE, j) : 0.0;
        double d0, j0, d1, j1;
        double c0 = soc_cost(m, u, k, ww, dt, cv, ye, ye1, &d0, &j0);
        double c1 = soc_cost(m, u, k, ww, dt, cv, ye + t * w.dy(EK_SE, j), ye1 + t * dye1, &d1, &j1);
        D += c1 - c0;
        w.dr[m.ubus[u]] += j1 - j0;
        sec.push_back(d1);
        sec.push_back(m.uetain[u] > 0 ? d1 - m.uetain[u] : 1.0);
        sec.push_back(-d1 * m.uetaout[u] - 1.0);
    }
    for (int n : w.nodes) {  // balance cells = nodes at the complete level
        double S0 = c.r[ix(c, n, tau, rep)];
        double S1 = S0 + (0.0 + w.dr[n]);
        D += dt * 1 * (phibal(m, S1 / 1) - phibal(m, S0 / 1));
        sec.push_back(S1);
    }
    return D;
}

// a prepared block move over consecutive steps (BlockMove, src/local.jl:1196), steps in time
// order: (tau-1, tau) for the local families, b0 .. b0+L for a storage plateau
struct Mover {
    const Ctx *c;
    vector<WS *> w;
    int rep;
    double beta;
    vector<double> sec;
    bool cyclic = false;  // the steps cover the whole year: the last step's end value is the first's
    double eval(double t) {  // mv_eval! (src/local.jl:1219): later steps first
        sec.clear();
        double D = 0.0;
        int n = (int)w.size();
        for (int q = n - 1; q >= 0; --q)
            D += eval_ws(*c, *w[q], rep, t, q + 1 < n ? w[q + 1] : (cyclic ? w[0] : nullptr), sec);
        return D;
    }
    bool hasstor() const {
        for (const WS *x : w)
            if (!x->stu.empty()) return true;
        return false;
    }
    void mask(vector<char> &g) const {  // storage_mask! (src/local.jl:1244), in evaluation order
        g.clear();
        for (int q = (int)w.size() - 1; q >= 0; --q) {
            for (size_t j = 0; j < w[q]->stu.size() * 3; ++j) g.push_back(1);
            for (size_t j = 0; j < w[q]->nodes.size(); ++j) g.push_back(0);
        }
    }
};

static inline bool wlt(double a, double b, double s) { return s > 0 ? a < b : a > b; }
static void sort_walk(vector<double> &v, double s) {
    std::stable_sort(v.begin(), v.end(), [s](double a, double b) { return wlt(a, b, s); });
}

struct Walk {
    vector<double> pts, cs;
    int cap;
    bool full = false;
    int nprim = 0, nray = 0;  // primary breakpoints and ray steps visited (diagnostics)
    // the stop test's margins (diagnostics): c - cmin - maxnats where the walk stopped, and the
    // largest value it took at an earlier primary breakpoint or ray point (how near a stop came)
    double stop = NAN, near_ = -INFINITY;
    double ray_from = NAN;  // where the ray steps began (the last primary breakpoint, or 0)
    void push(double x, double cx) {
        if ((int)pts.size() >= cap) {
            full = true;
            return;
        }
        pts.push_back(x);
        cs.push_back(cx);
    }
};

// piece_roots! (src/local.jl:1267)
static double piece_roots(Walk &W, Mover &mv, double cmin, const vector<double> &A, const vector<double> &B, double a,
                          double b, const vector<char> &gmask, double sgn) {
    vector<double> sroots;
    for (size_t j = 0; j < B.size(); ++j) {
        if (gmask[j]) continue;
        double u = A[j], v = B[j];
        if ((u < 0) != (v < 0) && u != v) {
            double x = a + (b - a) * u / (u - v);
            if (sgn * (x - a) > 0 && sgn * (b - x) > 0) sroots.push_back(x);
        }
    }
    if (sroots.empty()) return cmin;
    sort_walk(sroots, sgn);
    for (double x : sroots) {
        double cx = mv.beta * mv.eval(x);
        W.push(x, cx);
        cmin = std::min(cmin, cx);
    }
    return cmin;
}

// walk! (src/local.jl:1294) for the plain model (no requirement-tracking kinks, no Gaussian part)
// returns 1 proper, 0 improper (ray steps exhausted)
static int walk(Walk &W, Mover &mv, vector<double> &bp, double sgn, double maxnats, const vector<double> &sec0) {
    double tp = 0.0;
    vector<double> secprev = sec0, secB, secE, roots, groots;
    bool stor = mv.hasstor();
    vector<char> gmask;
    if (stor) mv.mask(gmask);
    double cmin = 0.0;
    size_t idx = 0;
    double delta = 0.0;
    int nx = 0;
    sort_walk(bp, sgn);
    while (true) {
        double t;
        if (idx < bp.size()) {
            t = bp[idx++];
            if (t == tp) continue;
            W.nprim += 1;
        } else {
            if (W.nray == 0) W.ray_from = tp;
            W.nray += 1;
            double cprev = W.cs.empty() ? 0.0 : W.cs.back();
            double hp = 1e-6 * std::max(1.0, fabs(tp));
            double sl = (mv.beta * mv.eval(tp + sgn * hp) + 0.0 - cprev - 0.0) / hp;
            if (sl > 0)
                delta = std::min(2 * maxnats / sl, 1e3 * std::max(fabs(tp), 1e-3));
            else
                delta = delta == 0.0 ? std::max(fabs(tp), 1e-6) : 2 * delta;
            t = tp + sgn * delta;
            nx += 1;
            if (nx > 80) return 0;
        }
        double cval = mv.beta * mv.eval(t);
        vector<double> sec = mv.sec;
        roots.clear();
        groots.clear();
        for (size_t j = 0; j < sec.size(); ++j) {
            double a = secprev[j], b = sec[j];
            if ((a < 0) != (b < 0) && a != b) {
                double x = tp + (t - tp) * a / (a - b);
                if (sgn * (x - tp) > 0 && sgn * (t - x) > 0) {
                    if (stor && gmask[j])
                        groots.push_back(x);
                    else
                        roots.push_back(x);
                }
            }
        }
        if (stor && !groots.empty()) {
            secE = sec;
            sort_walk(groots, sgn);
            double a0 = tp;
            for (double x : groots) {
                double cx = mv.beta * mv.eval(x);
                secB = mv.sec;
                cmin = piece_roots(W, mv, cmin, secprev, secB, a0, x, gmask, sgn);
                W.push(x, cx);
                cmin = std::min(cmin, cx);
                secprev = secB;
                a0 = x;
            }
            cmin = piece_roots(W, mv, cmin, secprev, secE, a0, t, gmask, sgn);
            secprev = secE;
        } else {
            secprev = sec;
            if (!roots.empty()) {
                sort_walk(roots, sgn);
                for (double x : roots) {
                    double cx = mv.beta * mv.eval(x);
                    W.push(x, cx);
                    cmin = std::min(cmin, cx);
                }
            }
        }
        W.push(t, cval);
        cmin = std::min(cmin, cval);
        if (cval + 0.0 - cmin > maxnats) {
            W.stop = cval - cmin - maxnats;
            return 1;
        }
        W.near_ = std::max(W.near_, cval - cmin - maxnats);
        if (W.full) return 1;
        tp = t;
    }
}

// sample_line! (src/local.jl:1501) with the uniforms (u_cat, u_off) given; *guard set when the
// walk exceeded the point cap (the move is then not taken)
static double sample_line(Mover &mv, double maxnats, int cap, double u_cat, double u_off, bool *guard) {
    vector<double> right, left;
    for (const WS *w : mv.w)
        for (double x : w->bps) {
            if (!std::isfinite(x)) continue;
            if (x > 0.0)
                right.push_back(x);
            else if (x < 0.0)
                left.push_back(x);
        }
    mv.eval(0.0);
    vector<double> sec0 = mv.sec;
    Walk Wr, Wl;
    Wr.cap = Wl.cap = cap;
    *guard = false;
    if (!walk(Wr, mv, right, 1.0, maxnats, sec0)) return 0.0;
    if (Wr.full) {
        *guard = true;
        return 0.0;
    }
    if (!walk(Wl, mv, left, -1.0, maxnats, sec0)) return 0.0;
    if (Wl.full) {
        *guard = true;
        return 0.0;
    }
    vector<double> pts, cs;
    for (int j = (int)Wl.pts.size() - 1; j >= 0; --j) {
        pts.push_back(Wl.pts[j]);
        cs.push_back(Wl.cs[j]);
    }
    pts.push_back(0.0);
    cs.push_back(0.0);
    pts.insert(pts.end(), Wr.pts.begin(), Wr.pts.end());
    cs.insert(cs.end(), Wr.cs.begin(), Wr.cs.end());
    int nseg = (int)pts.size() - 1;
    vector<double> lm(nseg);
    double mx = -INFINITY;
    for (int j = 0; j < nseg; ++j) {
        double L = pts[j + 1] - pts[j];
        lm[j] = L > 0 ? -std::min(cs[j], cs[j + 1]) + logseg(L, fabs(cs[j + 1] - cs[j])) : -INFINITY;
        mx = std::max(mx, lm[j]);
    }
    double tot = 0.0;
    for (int j = 0; j < nseg; ++j) tot += exp(lm[j] - mx);
    double u = u_cat * tot, acc = 0.0;
    int jj = nseg - 1;
    for (int q = 0; q < nseg; ++q) {
        acc += exp(lm[q] - mx);
        if (u <= acc) {
            jj = q;
            break;
        }
    }
    double L = pts[jj + 1] - pts[jj];
    double g = (cs[jj + 1] - cs[jj]) / L;
    return (g >= 0 || fabs(g * L) < 1e-10) ? pts[jj] + trexp_offset(u_off, g, L)
                                          : pts[jj + 1] - trexp_offset(u_off, -g, L);
}

// commit_block! / apply_step! (src/local.jl:2495, :2507)
static void commit(Ctx &c, Mover &mv, double t) {
    if (t == 0.0) return;
    mv.eval(t);
    const Model &m = c.m;
    for (WS *w : mv.w) {
        int tau = w->tau;
        for (auto &en : w->ent) {
            double d = t * en.a + (en.kid >= 0 ? en.ak * w->kinks[en.kid].phi : 0.0);
            if (en.kind == EK_THETA)
                c.theta[ix(c, en.idx, tau, mv.rep)] += d;
            else if (en.kind == EK_GEN)
                c.g[ix(c, en.idx, tau, mv.rep)] += d;
            else
                c.e[ix(c, en.idx, tau, mv.rep)] += d;
        }
        for (int e : w->lines) c.F[ix(c, e, tau, mv.rep)] += t * w->dfl[e];
        for (int n : w->nodes) c.r[ix(c, n, tau, mv.rep)] += w->dr[n];
    }
    (void)m;
}

// ------------------------------------------------------------------------------------------
// move selection (src/local.jl:1567-1900), with the tile stream of philox.h
// ------------------------------------------------------------------------------------------
struct TileStream {
    uint64_t seed;
    uint32_t tile, cls, sweep, j = 0;
    double next() {
        double u0, u1;
        orc_uniform2(seed, ESM_TAG_LIST, j >> 1, tile, cls, sweep, &u0, &u1);
        double u = (j & 1) ? u1 : u0;
        ++j;
        return u;
    }
    int pick(int n) {
        int i = (int)floor(next() * n);
        return i >= n ? n - 1 : i;
    }
};

struct MoveRef {
    int kind;  // -1 atom, else family
    int field, atom;
};

static void move_list(const Ctx &c, TileStream &ts, vector<MoveRef> &out) {
    const Model &m = c.m;
    out.clear();
    for (int f = 0; f < m.nfields; ++f)
        for (int a = m.fap[f]; a < m.fap[f + 1]; ++a) out.push_back(MoveRef{-1, f, a});
    int nextra = (int)nearbyint(c.o.extra * m.N);
    double cum[ESM_NFAM], tot = 0.0;
    for (int q = 0; q < ESM_NFAM; ++q) {
        tot += c.o.rates[q];
        cum[q] = tot;
    }
    for (int q = 0; q < ESM_NFAM; ++q) cum[q] /= tot;
    for (int i = 0; i < nextra; ++i) {
        double u = ts.next();
        int kd = ESM_NFAM - 1;
        for (int q = 0; q < ESM_NFAM; ++q)
            if (cum[q] >= u) {
                kd = q;
                break;
            }
        out.push_back(MoveRef{kd, -1, -1});
    }
    for (int i = (int)out.size() - 1; i >= 1; --i) {  // Fisher-Yates
        int j = ts.pick(i + 1);
        std::swap(out[i], out[j]);
    }
}

static inline double kappa_unit(const Ctx &c, int j) {  // kappa_unit (src/local.jl:1585), dispatchable j
    int u = c.m.disp[j];
    return c.m.uavail[u] * kcl(c, u);
}

// prorata! (src/local.jl:1782), plain model (no tracking kinks)
static bool prorata(const Ctx &c, WS &w, int rep, int mnode, double g, vector<Kink> *jac, double qadj = 0.0) {
    const Model &m = c.m;
    if (g == 0.0) return false;
    int tau = w.tau;
    double Pm = 0.0, Qs = 0.0;
    int nu = 0;
    for (int q = m.up[mnode]; q < m.up[mnode + 1]; ++q) {
        int j = m.ua[q];
        double kap = kappa_unit(c, j);
        if (!(fabs(kap) >= c.o.kmin)) continue;
        double om = c.g[ix(c, j, tau, rep)];
        Pm += kap * om;
        Qs += kap * clampd(om, 0.0, 1.0);
        nu += 1;
    }
    if (nu == 0) return false;
    if (fabs(Pm) < 1e-6) return false;
    double Q = c.r[ix(c, mnode, tau, rep)] + Qs + qadj;
    double e = Pm - std::max(Q, 0.0);
    double nm = (double)(nu - 1);
    w.kinks.push_back(Kink{Q, g, 0.0, Pm, e, nm});
    int kid = (int)w.kinks.size() - 1;
    for (int q = m.up[mnode]; q < m.up[mnode + 1]; ++q) {
        int j = m.ua[q];
        double kap = kappa_unit(c, j);
        if (!(fabs(kap) >= c.o.kmin)) continue;
        double sigma = kap * c.g[ix(c, j, tau, rep)] / Pm;
        if (sigma == 0.0) continue;
        w.add_kentry(j, sigma / kap, kid);
    }
    jac->push_back(w.kinks.back());
    return true;
}

static double soc_qadj(const Ctx &c, const vector<int> &us, int mnode, int tau, int rep);

// prep_random!, prep_xloc!, prep_spair!, prep_tpot!, prep_tsoc! (src/local.jl:1608, :1672, :1708,
// :1741, :1849)
static bool prep_family(const Ctx &c, TileStream &ts, int fam, WS &ws, WS &wa, int rep, vector<Kink> *jac) {
    const Model &m = c.m;
    int N = m.N;
    double kmin = c.o.kmin;
    auto nunits = [&](int n) { return m.up[n + 1] - m.up[n]; };
    switch (fam) {
        case ESM_FAM_UNIT: {
            int n = ts.pick(N);
            if (nunits(n) == 0) return false;
            int j = m.ua[m.up[n] + ts.pick(nunits(n))];
            ws.add_entry(EK_GEN, j, 1.0);
            return true;
        }
        case ESM_FAM_PAIR:
        case ESM_FAM_XPAIR: {
            int n = ts.pick(N);
            int mm = fam == ESM_FAM_PAIR ? n : ts.pick(N);
            if (fam == ESM_FAM_XPAIR && (mm == n || m.comp[mm] != m.comp[n])) return false;
            if (nunits(n) == 0 || nunits(mm) == 0) return false;
            int u1 = m.ua[m.up[n] + ts.pick(nunits(n))];
            int u2 = m.ua[m.up[mm] + ts.pick(nunits(mm))];
            if (u1 == u2) return false;
            double k1 = kappa_unit(c, u1), k2 = kappa_unit(c, u2);
            if (fabs(k1) < kmin || fabs(k2) < kmin) return false;
            ws.add_entry(EK_GEN, u1, 1 / k1);
            ws.add_entry(EK_GEN, u2, -1 / k2);
            if (fam == ESM_FAM_XPAIR) {  // prep_reroute! (src/local.jl:1592)
                for (int i = 0; i < N; ++i) {
                    if (m.comp[i] != m.comp[n]) continue;
                    double x = m.Z[(size_t)i * N + n] - m.Z[(size_t)i * N + mm];
                    if (fabs(x) < 1e-15) continue;
                    ws.add_entry(EK_THETA, i, x);
                }
            }
            return true;
        }
        case ESM_FAM_XLOC:
        case ESM_FAM_XLOCC: {
            int n = ts.pick(N);
            int np = m.xpp[n + 1] - m.xpp[n];
            if (np == 0) return false;
            int jp = ts.pick(np);
            int pair = m.xpp[n] + jp;
            int mm = m.xp[pair];
            if (nunits(n) == 0 || nunits(mm) == 0) return false;
            int u1 = m.ua[m.up[n] + ts.pick(nunits(n))];
            int u2 = m.ua[m.up[mm] + ts.pick(nunits(mm))];
            double k1 = kappa_unit(c, u1), k2 = kappa_unit(c, u2);
            if (fabs(k1) < kmin || fabs(k2) < kmin) return false;
            jac->clear();
            ws.add_entry(EK_GEN, u1, 1 / k1);
            ws.add_entry(EK_GEN, u2, -1 / k2);
            for (int q = m.xnp[pair]; q < m.xnp[pair + 1]; ++q) ws.add_entry(EK_THETA, m.xn[q], m.xv[q]);
            if (fam == ESM_FAM_XLOCC)
                for (int q = m.xlp[pair]; q < m.xlp[pair + 1]; ++q) prorata(c, ws, rep, m.xln[q], m.xlg[q], jac);
            return true;
        }
        case ESM_FAM_POTENTIAL: {
            int n = ts.pick(N);
            if (m.theta_nnz[n] == 0) return false;
            ws.add_entry(EK_THETA, n, 1.0);
            return true;
        }
        case ESM_FAM_CELLPAIR:
        case ESM_FAM_CELL: {
            double u = ts.next();
            int q = m.nlev - 1;
            for (int l = 0; l < m.nlev; ++l)
                if (m.qcum[l] >= u) {
                    q = l;
                    break;
                }
            int ncell = m.clp[q + 1] - m.clp[q];
            int cidx = m.clp[q] + ts.pick(ncell);
            // injecting fields present in the cell, in field (group) order
            vector<int> fl;
            for (int p = m.cp[cidx]; p < m.cp[cidx + 1]; ++p) {
                int gidx = m.ugroup[m.disp[m.cu[p]]];
                if (std::find(fl.begin(), fl.end(), gidx) == fl.end()) fl.push_back(gidx);
            }
            std::sort(fl.begin(), fl.end());
            if (fl.empty()) return false;
            if (fam == ESM_FAM_CELL) {
                int f = fl[ts.pick((int)fl.size())];
                for (int p = m.cp[cidx]; p < m.cp[cidx + 1]; ++p)
                    if (m.ugroup[m.disp[m.cu[p]]] == f) ws.add_entry(EK_GEN, m.cu[p], 1.0);
                return true;
            }
            if (fl.size() < 2) return false;
            int f1 = fl[ts.pick((int)fl.size())];
            int f2 = fl[ts.pick((int)fl.size())];
            if (f1 == f2) return false;
            double K1 = 0.0, K2 = 0.0;
            for (int p = m.cp[cidx]; p < m.cp[cidx + 1]; ++p) {
                int j = m.cu[p];
                if (m.ugroup[m.disp[j]] == f1) K1 += kappa_unit(c, j);
                if (m.ugroup[m.disp[j]] == f2) K2 += kappa_unit(c, j);
            }
            if (fabs(K1) < kmin || fabs(K2) < kmin) return false;
            for (int p = m.cp[cidx]; p < m.cp[cidx + 1]; ++p)
                if (m.ugroup[m.disp[m.cu[p]]] == f1) ws.add_entry(EK_GEN, m.cu[p], 1 / K1);
            for (int p = m.cp[cidx]; p < m.cp[cidx + 1]; ++p)
                if (m.ugroup[m.disp[m.cu[p]]] == f2) ws.add_entry(EK_GEN, m.cu[p], -1 / K2);
            return true;
        }
        case ESM_FAM_SPAIR: {
            int n = ts.pick(N);
            int ns = m.sp[n + 1] - m.sp[n];
            if (ns == 0 || nunits(n) == 0) return false;
            int sj = m.sa[m.sp[n] + ts.pick(ns)];
            int su = m.stor[sj];
            double ks = kcl(c, su) * m.uhours[su] / m.dt;
            if (ks < kmin) return false;
            int u1 = m.ua[m.up[n] + ts.pick(nunits(n))];
            int u2 = m.ua[m.up[n] + ts.pick(nunits(n))];
            double k1 = kappa_unit(c, u1), k2 = kappa_unit(c, u2);
            if (fabs(k1) < kmin || fabs(k2) < kmin) return false;
            wa.add_entry(EK_GEN, u1, ks / k1);
            ws.add_entry(EK_SE, sj, 1.0);
            ws.add_entry(EK_GEN, u2, -ks / k2);
            return true;
        }
        case ESM_FAM_TPOT: {  // prep_tpot! (src/local.jl:1741): the angle of node n rises by t
            int n = ts.pick(N);
            if (m.theta_nnz[n] == 0) return false;
            jac->clear();
            ws.add_entry(EK_THETA, n, 1.0);
            // requirement change per unit t: r[a] += f_e, r[b] -= f_e for each line a -> b of n
            vector<double> g(N, 0.0);
            vector<int> gn;
            for (int p = m.nlp[n]; p < m.nlp[n + 1]; ++p) {
                int e = m.nl[p], a = m.bus0[e], b = m.bus1[e];
                double df = m.lb[e] * (double)((a == n) - (b == n));
                g[a] += df;
                g[b] -= df;
                gn.push_back(a);
                gn.push_back(b);
            }
            std::sort(gn.begin(), gn.end());
            gn.erase(std::unique(gn.begin(), gn.end()), gn.end());
            for (int mm : gn)
                if (g[mm] != 0.0) prorata(c, ws, rep, mm, g[mm], jac);
            return true;
        }
        case ESM_FAM_TSOC: {  // prep_tsoc! (src/local.jl:1849): energy moved from step tau-1 to tau
            int n = ts.pick(N);
            int ns = m.sp[n + 1] - m.sp[n];
            if (ns == 0) return false;
            int sj = m.sa[m.sp[n] + ts.pick(ns)];
            int su = m.stor[sj];
            double ks = kcl(c, su) * m.uhours[su] / m.dt;
            if (ks < kmin) return false;
            jac->clear();
            ws.add_entry(EK_SE, sj, 1.0);
            vector<int> us{sj};
            prorata(c, wa, rep, n, ks, jac, soc_qadj(c, us, n, wa.tau, rep));
            prorata(c, ws, rep, n, -ks, jac, soc_qadj(c, us, n, ws.tau, rep));
            return true;
        }
    }
    return false;
}

// the moves of one (replica, step) task: the body of the threaded loop of local_sweep!
// (src/local.jl:1954-2051)
static void run_task(Ctx &c, const vector<MoveRef> &moves, TileStream ts0, int tau, int rep, uint32_t sweep,
                     int64_t *stats, WS &ws, WS &wa, int limit, int m0 = 0, double *tlog = nullptr,
                     size_t tlog_stride = 0, size_t tlog_at = 0) {
    const Model &m = c.m;
    int T = m.T;
    int taum = (tau - 1 + T) % T;
    TileStream ts = ts0;  // the selection draws continue after the list draws
    vector<Kink> jac;
    Mover mv{&c, {&wa, &ws}, rep, m.beta_v, {}};
    size_t nrun = limit > 0 && (size_t)limit < moves.size() ? (size_t)limit : moves.size();
    for (size_t mi = 0; mi < nrun; ++mi) {
        ws.clear();
        wa.clear();
        ws.tau = tau;
        wa.tau = taum;
        jac.clear();
        const MoveRef &mr = moves[mi];
        int fi;
        if ((int)mi < m0) {  // before the range: only the selection draws, to keep the stream position
            if (mr.kind >= 0) prep_family(c, ts, mr.kind, ws, wa, rep, &jac);
            continue;
        }
        if (mr.kind < 0) {  // prep_atom! (src/local.jl:1567)
            int role = m.frole[mr.field];
            int kind = role == ESM_ROLE_THETA ? EK_THETA : (role == ESM_ROLE_GEN ? EK_GEN : EK_SE);
            for (int q = m.ap[mr.atom]; q < m.ap[mr.atom + 1]; ++q) ws.add_entry(kind, m.ai[q], m.av[q]);
            fi = ESM_NFAM;
        } else {
            if (!prep_family(c, ts, mr.kind, ws, wa, rep, &jac)) continue;
            fi = mr.kind;
        }
        finalize_ws(c, ws, rep);
        if (ws.ent.empty()) continue;
        finalize_ws(c, wa, rep);
        link_soc(m, wa, ws);
        double uc, uo, uj, un;
        orc_uniform2(c.o.seed, ESM_TAG_LANE, 2 * (uint32_t)mi, (uint32_t)tau, (uint32_t)rep, sweep, &uc, &uo);
        orc_uniform2(c.o.seed, ESM_TAG_LANE, 2 * (uint32_t)mi + 1, (uint32_t)tau, (uint32_t)rep, sweep, &uj, &un);
        bool guard = false;
        double t = sample_line(mv, c.o.maxnats, c.o.max_points, uc, uo, &guard);
        if (guard) stats[2 * (ESM_NFAM + 1)] += 1;
        bool compensated = mr.kind == ESM_FAM_XLOCC || mr.kind == ESM_FAM_TPOT || mr.kind == ESM_FAM_TSOC;
        if (compensated && t != 0.0 && !jac.empty()) {
            double lj = 0.0;  // logjac (src/local.jl:1871)
            for (auto &k : jac) lj += k.nm * log(fabs((std::max(k.Q + k.g * t, 0.0) + k.e) / k.Pm));
            if (uj >= exp(std::min(0.0, lj))) t = 0.0;
        }
        commit(c, mv, t);
        if (tlog) tlog[mi * tlog_stride + tlog_at] = t;
        stats[2 * fi] += 1;
        stats[2 * fi + 1] += t != 0.0;
    }
    ws.clear();
    wa.clear();
}

static void class_steps(int T, int cls, vector<int> &out) {
    out.clear();
    if (T % 2 == 1) {
        if (cls == 0)
            for (int t = 0; t < T - 1; t += 2) out.push_back(t);
        else if (cls == 1)
            for (int t = 1; t < T - 1; t += 2) out.push_back(t);
        else
            out.push_back(T - 1);
    } else {
        for (int t = cls; t < T; t += 2) out.push_back(t);
    }
}

static int span_of(const Ctx &c) { return c.o.span > 0 ? c.o.span : std::max(1, 32 / c.o.R); }

static void class_pass(Ctx &c, uint32_t sweep, int cls, int64_t *stats, int nthreads, int limit = 0, int m0 = 0,
                       double *tlog = nullptr) {
    vector<int> steps;
    class_steps(c.m.T, cls, steps);
    int span = span_of(c);
    int ntile = ((int)steps.size() + span - 1) / span;
    int R = c.o.R;
    int nst = 2 * (ESM_NFAM + 1) + 1;
    // one move list per (class, sweep), shared by every task of the class (the stream's tile word is 0)
    TileStream ts0{c.o.seed, 0u, (uint32_t)cls, sweep};
    vector<MoveRef> moves;
    move_list(c, ts0, moves);
#pragma omp parallel num_threads(nthreads)
    {
        vector<int64_t> loc(nst, 0);
        WS ws, wa;
        ws.init(c.m);
        wa.init(c.m);
#pragma omp for schedule(dynamic, 1)
        for (int tile = 0; tile < ntile; ++tile) {
            for (int q = tile * span; q < std::min((int)steps.size(), (tile + 1) * span); ++q)
                for (int rep = 0; rep < R; ++rep)
                    run_task(c, moves, ts0, steps[q], rep, sweep, loc.data(), ws, wa, limit, m0, tlog,
                             steps.size() * (size_t)R, (size_t)q * R + rep);
        }
#pragma omp critical
        for (int i = 0; i < nst; ++i) stats[i] += loc[i];
    }
}

static void class_order(const Ctx &c, uint32_t sweep, int order[3], int *ncls) {
    double u0, u1;
    orc_uniform2(c.o.seed, ESM_TAG_SWEEP, 0, 0, 0, sweep, &u0, &u1);
    if (c.m.T % 2 == 0) {
        *ncls = 2;
        order[0] = u0 < 0.5 ? 0 : 1;
        order[1] = 1 - order[0];
    } else {
        *ncls = 3;
        order[0] = 0;
        order[1] = 1;
        order[2] = 2;
        int j = std::min(2, (int)floor(u0 * 3));
        std::swap(order[2], order[j]);
        j = std::min(1, (int)floor(u1 * 2));
        std::swap(order[1], order[j]);
    }
}

// ------------------------------------------------------------------------------------------
// storage multiscale sweep (storage_ms_sweep!, src/flowmoves.jl:255) in its plateau form (the
// shapes need the flow basis, src/flowmoves.jl:302): energy of one storage unit, or of the units
// of one carrier in one country cell, moved from step b0 to step b0 + L of a dyadic block
// ------------------------------------------------------------------------------------------
struct PStream {  // sequential uniforms of one Philox stream (tag, words 1-3)
    uint64_t seed;
    uint32_t tag, w1, w2, w3, j = 0;
    double next() {
        double u0, u1;
        orc_uniform2(seed, tag, j >> 1, w1, w2, w3, &u0, &u1);
        double u = (j & 1) ? u1 : u0;
        ++j;
        return u;
    }
    int pick(int n) {
        int i = (int)floor(next() * n);
        return i >= n ? n - 1 : i;
    }
};

struct SmsPass {
    int li, L, o, cls;
};

// The class passes of the storage multiscale sweep of one operation sweep: its coin (probability
// 1/2, operation_sweep!, src/local.jl:2417; skipped with force), the lengths 2, 4, ..., 128 below
// T/2 in random order, per length a random offset and the order of the two block parities.
static int sms_plan(uint64_t seed, int T, uint32_t sweep, bool force, SmsPass *out) {
    PStream st{seed, ESM_TAG_SMS, 0u, 0u, sweep};
    bool run = st.next() < 0.5;
    if (!run && !force) return 0;
    int lens[7], nl = 0;
    for (int L = 2; L <= 128; L *= 2)
        if (L < T / 2) lens[nl++] = L;
    for (int i = nl - 1; i >= 1; --i) {
        int j = st.pick(i + 1);
        std::swap(lens[i], lens[j]);
    }
    int n = 0;
    for (int q = 0; q < nl; ++q) {
        int L = lens[q];
        int o = st.pick(L);
        bool swap01 = st.next() >= 0.5;
        int nb = 0;
        for (int b0 = o; b0 + L <= T - 1; b0 += L) ++nb;
        if (nb < 2) continue;
        int li = 0;
        while ((2 << li) < L) ++li;
        out[n++] = SmsPass{li, L, o, swap01 ? 1 : 0};
        out[n++] = SmsPass{li, L, o, swap01 ? 0 : 1};
    }
    return n;
}

// soc_qadj (src/local.jl:1826): nominal minus actual injection of the moved storage units at node
// mnode and step tau
static double soc_qadj(const Ctx &c, const vector<int> &us, int mnode, int tau, int rep) {
    const Model &m = c.m;
    int t1 = (tau + 1) % m.T;
    double q = 0.0;
    for (int j : us) {
        int u = m.stor[j];
        if (m.ubus[u] != mnode) continue;
        double ye = c.e[ix(c, j, tau, rep)], ye1 = c.e[ix(c, j, t1, rep)];
        double k = kcl(c, u), pc, mcx;
        soc_power(m, u, m.dt, clampd(ye, 0.0, 1.0), clampd(ye1, 0.0, 1.0), &pc, &mcx);
        q += k * m.uhours[u] * (ye1 - ye) / m.dt - k * (pc - mcx);
    }
    return q;
}

// prep_storage_ms! (src/flowmoves.jl:187), plateau: the state of charge of the units rises by t at
// the instants b0+1 .. b0+L; the power changes at steps b0 (+kappa_s t) and b0+L (-kappa_s t) and
// the dispatch at those nodes follows pro rata (prorata! with soc_qadj)
static bool prep_plateau(const Ctx &c, vector<WS> &wss, int b0, int L, const vector<int> &us, int rep,
                         vector<Kink> *jac) {
    const Model &m = c.m;
    int n = L + 1;
    for (int q = 0; q < n; ++q) {  // the steps b0 .. b0 + L, cyclic (the long-range plateaus wrap)
        wss[q].clear();
        wss[q].tau = (b0 + q) % m.T;
    }
    jac->clear();
    for (int j : us)
        for (int jj = 1; jj <= L; ++jj) wss[jj].add_entry(EK_SE, j, 1.0);
    for (int q = 0; q < n; ++q) {
        vector<int> gn;
        vector<double> gv;
        for (int j : us) {
            int u = m.stor[j];
            double ks = kcl(c, u) * m.uhours[u] / m.dt;
            double e0 = q == 0 ? 0.0 : 1.0, e1 = q + 1 <= L ? 1.0 : 0.0;
            double dg = ks * (e1 - e0);
            if (dg == 0.0) continue;
            int node = m.ubus[u];
            size_t p = std::find(gn.begin(), gn.end(), node) - gn.begin();
            if (p == gn.size()) {
                gn.push_back(node);
                gv.push_back(0.0);
            }
            gv[p] += dg;
        }
        for (size_t p = 0; p < gn.size(); ++p)
            prorata(c, wss[q], rep, gn[p], gv[p], jac, soc_qadj(c, us, gn[p], wss[q].tau, rep));
    }
    bool nonempty = false;
    for (int q = 0; q < n; ++q) {
        finalize_ws(c, wss[q], rep);
        nonempty |= !wss[q].ent.empty();
    }
    for (int q = 0; q + 1 < n; ++q) link_soc(m, wss[q], wss[q + 1]);
    return nonempty;
}

// the 8 move selections of a class (shared by its blocks and replicas: selection reads only k and
// the static tables): a cell-class aggregate with probability 1/2, else one unit
static void sms_moves(const Ctx &c, uint32_t sweep, const SmsPass &ps, vector<vector<int>> &moves) {
    const Model &m = c.m;
    PStream st{c.o.seed, ESM_TAG_SMS, 1u + (uint32_t)ps.li, 2u + (uint32_t)ps.cls, sweep};
    int ng = (int)m.sgp.size() - 1;
    moves.assign(8, {});
    for (int q = 0; q < 8; ++q) {
        if (st.next() < 0.5 && ng > 0) {
            int gi = st.pick(ng);
            for (int p = m.sgp[gi]; p < m.sgp[gi + 1]; ++p) moves[q].push_back(m.sgu[p]);
        } else {
            moves[q].push_back(st.pick(m.S));
        }
    }
}

// one class pass: every block of the class parity, every replica, the 8 moves in order
static void sms_pass(Ctx &c, uint32_t sweep, const SmsPass &ps, int64_t *stats3, int nthreads) {
    const Model &m = c.m;
    int T = m.T, R = c.o.R, L = ps.L;
    vector<int> blocks;
    int k = 0;
    for (int b0 = ps.o; b0 + L <= T - 1; b0 += L, ++k)
        if (k % 2 == ps.cls) blocks.push_back(b0);
    vector<vector<int>> moves;
    sms_moves(c, sweep, ps, moves);
    int nb = (int)blocks.size();
#pragma omp parallel num_threads(nthreads)
    {
        int64_t loc[3] = {0, 0, 0};
        vector<WS> wss(L + 1);
        for (auto &w : wss) w.init(m);
        vector<Kink> jac;
#pragma omp for schedule(dynamic, 1)
        for (int q = 0; q < nb * R; ++q) {
            int b0 = blocks[q / R], rep = q % R;
            for (int mi = 0; mi < 8; ++mi) {
                if (!prep_plateau(c, wss, b0, L, moves[mi], rep, &jac)) continue;
                Mover mv{&c, {}, rep, m.beta_v, {}};
                for (auto &w : wss) mv.w.push_back(&w);
                uint32_t w0 = 2u * (8u * (uint32_t)ps.li + (uint32_t)mi);
                double uc, uo, uj, un;
                orc_uniform2(c.o.seed, ESM_TAG_SML, w0, (uint32_t)b0, (uint32_t)rep, sweep, &uc, &uo);
                orc_uniform2(c.o.seed, ESM_TAG_SML, w0 + 1, (uint32_t)b0, (uint32_t)rep, sweep, &uj, &un);
                bool guard = false;
                double t = sample_line(mv, c.o.maxnats, c.o.max_points, uc, uo, &guard);
                if (guard) loc[2] += 1;
                if (t != 0.0 && !jac.empty()) {  // logjac (src/local.jl:1871)
                    double lj = 0.0;
                    for (auto &kk : jac) lj += kk.nm * log(fabs((std::max(kk.Q + kk.g * t, 0.0) + kk.e) / kk.Pm));
                    if (uj >= exp(std::min(0.0, lj))) t = 0.0;
                }
                commit(c, mv, t);
                loc[0] += 1;
                loc[1] += t != 0.0;
            }
        }
        for (auto &w : wss) w.clear();
#pragma omp critical
        for (int i = 0; i < 3; ++i) stats3[i] += loc[i];
    }
}

// the storage multiscale sweep of one operation sweep (caches rebuilt first, as LocalCost at the
// sweep's start, src/flowmoves.jl:261)
static void sms_sweep(Ctx &c, uint32_t sweep, bool force, int64_t *stats3, int nthreads, int max_passes = 0) {
    SmsPass ps[14];
    int n = sms_plan(c.o.seed, c.m.T, sweep, force, ps);
    if (max_passes > 0 && max_passes < n) n = max_passes;
    if (n == 0 || c.m.S == 0) return;
    rebuild(c, nthreads);
    for (int i = 0; i < n; ++i) sms_pass(c, sweep, ps[i], stats3, nthreads);
}

// ------------------------------------------------------------------------------------------
// long-range storage sweep (storage_long_sweep!, src/storage_long.jl:245): for every storage unit
// with at least 24 h of storage and kappa_s >= kappa_min, a level move (every instant of the year
// rises, no power change inside the box) and 4 long-range plateaus (prep_slong!, :77: the state of
// charge rises at the cyclic instants a+1 .. a+L, energy moved from step a to step a+L with pro-rata
// compensation at both), in random order
// ------------------------------------------------------------------------------------------
struct SlMove {
    int L, a;  // length (T: the level move), start step a (0-based)
};

// the eligible units and their move lists of one sweep (the same streams as the device host side)
static void sl_plan(const Ctx &c, uint32_t sweep, vector<int> &units, vector<vector<SlMove>> &moves) {
    const Model &m = c.m;
    int T = m.T;
    units.clear();
    moves.clear();
    for (int j = 0; j < m.S; ++j) {
        int u = m.stor[j];
        if (!(m.uhours[u] >= 24.0 && kcl(c, u) * m.uhours[u] / m.dt >= c.o.kmin)) continue;
        PStream st{c.o.seed, ESM_TAG_SLG, (uint32_t)j, 0u, sweep};
        vector<SlMove> mv;
        if (st.next() < 1.0) mv.push_back(SlMove{T, 0});  // the level move (p_level = 1)
        for (int q = 0; q < 4; ++q) mv.push_back(SlMove{1 + st.pick(T - 1), 0});
        for (int i = (int)mv.size() - 1; i >= 1; --i) std::swap(mv[i], mv[st.pick(i + 1)]);
        for (auto &x : mv) x.a = st.pick(T);
        units.push_back(j);
        moves.push_back(mv);
    }
}

// the level move (L = T): every instant of unit j rises by t; every step's term sees the next step's
static bool prep_level(const Ctx &c, vector<WS> &wss, int j, int rep) {
    const Model &m = c.m;
    int T = m.T;
    for (int q = 0; q < T; ++q) {
        wss[q].clear();
        wss[q].tau = q;
        wss[q].add_entry(EK_SE, j, 1.0);
    }
    for (int q = 0; q < T; ++q) finalize_ws(c, wss[q], rep);
    for (int q = 0; q < T; ++q) link_soc(m, wss[q], wss[(q + 1) % T]);
    return true;
}

// the moves [m0, m1) (m1 < 0: all) of one (unit, replica) task of the long-range storage sweep:
// unit j (the ui-th eligible unit), its move list ms; tlog (may be NULL): the t of move mi at
// [(ui * 5 + mi) * R + rep]
static void sl_task(Ctx &c, uint32_t sweep, int ui, int j, int rep, const vector<SlMove> &ms, int m0, int m1,
                    vector<WS> &wss, vector<Kink> &jac, int64_t *loc, double *tlog) {
    const Model &m = c.m;
    int T = m.T, R = c.o.R;
    int mend = m1 < 0 ? (int)ms.size() : std::min(m1, (int)ms.size());
    for (int mi = m0; mi < mend; ++mi) {
        const SlMove &sm = ms[mi];
        bool level = sm.L == T;
        jac.clear();
        if (level)
            prep_level(c, wss, j, rep);
        else if (!prep_plateau(c, wss, sm.a, sm.L, {j}, rep, &jac))
            continue;
        Mover mv{&c, {}, rep, m.beta_v, {}};
        mv.cyclic = level;
        int n = level ? T : sm.L + 1;
        for (int k = 0; k < n; ++k) mv.w.push_back(&wss[k]);
        double uc, uo, uj, un;
        orc_uniform2(c.o.seed, ESM_TAG_SLL, 2u * (uint32_t)mi, (uint32_t)j, (uint32_t)rep, sweep, &uc, &uo);
        orc_uniform2(c.o.seed, ESM_TAG_SLL, 2u * (uint32_t)mi + 1, (uint32_t)j, (uint32_t)rep, sweep, &uj, &un);
        bool guard = false;
        double t = sample_line(mv, c.o.maxnats, c.o.max_points, uc, uo, &guard);
        if (guard) loc[2] += 1;
        if (t != 0.0 && !jac.empty()) {
            double lj = 0.0;
            for (auto &kk : jac) lj += kk.nm * log(fabs((std::max(kk.Q + kk.g * t, 0.0) + kk.e) / kk.Pm));
            if (uj >= exp(std::min(0.0, lj))) t = 0.0;
        }
        commit(c, mv, t);
        if (tlog) tlog[((size_t)ui * 5 + mi) * R + rep] = t;
        loc[0] += 1;
        loc[1] += t != 0.0;
    }
}

static void sl_sweep(Ctx &c, uint32_t sweep, int64_t *stats3, int nthreads, double *tlog = nullptr) {
    const Model &m = c.m;
    int T = m.T, R = c.o.R;
    vector<int> units;
    vector<vector<SlMove>> moves;
    sl_plan(c, sweep, units, moves);
    if (units.empty()) return;
    rebuild(c, nthreads);  // LocalCost at the start (src/storage_long.jl:250)
    int nu = (int)units.size();
#pragma omp parallel num_threads(nthreads)
    {
        int64_t loc[3] = {0, 0, 0};
        vector<WS> wss(T);
        for (auto &w : wss) w.init(m);
        vector<Kink> jac;
#pragma omp for schedule(dynamic, 1)
        for (int q = 0; q < nu * R; ++q) {
            int ui = q / R, rep = q % R;
            sl_task(c, sweep, ui, units[ui], rep, moves[ui], 0, -1, wss, jac, loc, tlog);
        }
        for (auto &w : wss) w.clear();
#pragma omp critical
        for (int i = 0; i < 3; ++i) stats3[i] += loc[i];
    }
}

// ------------------------------------------------------------------------------------------
// energy cost with the capacity gradient (src/energy.jl:551-757) and capacity_scores
// (src/replicas.jl:329)
// ------------------------------------------------------------------------------------------
static void scores(Ctx &c, double *sk, double *fk, double *parts, int nthreads) {
    const Model &m = c.m;
    int T = m.T, R = c.o.R, K = m.K;
    double dt = m.dt, cv = m.c_viol, k0 = m.kappa0;
#pragma omp parallel for schedule(static) num_threads(nthreads)
    for (int rep = 0; rep < R; ++rep) {
        vector<double> dk(K, 0.0);
        vector<double> rr(m.N);
        vector<double> Gr((size_t)m.N * T);
        double cgen = 0, cst = 0, pen = 0, shed = 0, dump = 0;
        // residual and the balance gradient per step
        for (int t = 0; t < T; ++t) {
            for (int n = 0; n < m.N; ++n) rr[n] = load_map(wraw(c, n, t, rep));
            for (int e = 0; e < m.L; ++e) {
                int a = m.bus0[e], b = m.bus1[e];
                double fe = m.lb[e] * (c.theta[ix(c, a, t, rep)] - c.theta[ix(c, b, t, rep)]);
                rr[a] += fe + 0.5 * 0.0;
                rr[b] += -fe + 0.5 * 0.0;
                pen += cv * dt * (m.ls[e] * std::max(fabs(fe) / m.ls[e] - 1.0, 0.0));
            }
            for (int u = 0; u < K; ++u) {
                if (m.ukind[u] == ESM_UNIT_STOR) continue;
                double A, Y, Yc;
                if (m.ukind[u] == ESM_UNIT_REN) {
                    A = avail_map(wraw(c, m.useries[u], t, rep));
                    Y = Yc = 1.0;
                } else {
                    A = m.uavail[u];
                    Y = c.g[ix(c, m.disp_of_unit[u], t, rep)];
                    Yc = clampd(Y, 0.0, 1.0);
                }
                double kv = kcl(c, u);
                double p = A * kv * Yc;
                cgen += dt * (m.umc[u] * p);
                rr[m.ubus[u]] -= p;
                if (m.ukind[u] == ESM_UNIT_DISP) {
                    double ex = fabs(Y - Yc);
                    if (ex > 0) pen += cv * dt * (kv + k0) * ex;
                }
            }
            for (int j = 0; j < m.S; ++j) {
                int u = m.stor[j];
                double kv = kcl(c, u);
                double ye = c.e[ix(c, j, t, rep)], ye1 = c.e[ix(c, j, (t + 1) % T, rep)];
                double d, jj;
                double cc = soc_cost(m, u, kv, kv + k0, dt, cv, ye, ye1, &d, &jj);
                double pc, mcx;
                soc_power(m, u, dt, clampd(ye, 0.0, 1.0), clampd(ye1, 0.0, 1.0), &pc, &mcx);
                cst += dt * m.umc[u] * kv * (pc + mcx);
                pen += cc - dt * m.umc[u] * kv * (pc + mcx);
                rr[m.ubus[u]] += jj;
            }
            for (int n = 0; n < m.N; ++n) {
                double x = rr[n];
                if (x > 0)
                    shed += dt * x;
                else
                    dump -= dt * x;
                Gr[(size_t)n * T + t] = dt * (x > 0 ? m.c_shed : (x < 0 ? -m.c_dump : 0.0));
            }
        }
        // generators (gen_grad, src/energy.jl:835)
        for (int t = 0; t < T; ++t)
            for (int u = 0; u < K; ++u) {
                if (m.ukind[u] == ESM_UNIT_STOR) continue;
                double A, Y, Yc;
                bool compf;
                if (m.ukind[u] == ESM_UNIT_REN) {
                    A = avail_map(wraw(c, m.useries[u], t, rep));
                    Y = Yc = 1.0;
                    compf = true;
                } else {
                    A = m.uavail[u];
                    Y = c.g[ix(c, m.disp_of_unit[u], t, rep)];
                    Yc = clampd(Y, 0.0, 1.0);
                    compf = false;
                }
                double kv = kcl(c, u);
                double Gn = Gr[(size_t)m.ubus[u] * T + t];
                if (!(compf || (0.0 < Y && Y < 1.0))) dk[u] += cv * dt * fabs(Y - Yc);
                double dck = m.umc[u] * A * Yc;
                dk[u] += dt * dck - A * Yc * Gn;
                (void)kv;
            }
        // storage (soc_grad, src/energy.jl:466)
        for (int t = 0; t < T; ++t)
            for (int j = 0; j < m.S; ++j) {
                int u = m.stor[j];
                int t1 = (t + 1) % T;
                double h = m.uhours[u];
                double Ec = clampd(c.e[ix(c, j, t, rep)], 0.0, 1.0), Ec1 = clampd(c.e[ix(c, j, t1, rep)], 0.0, 1.0);
                double d = h * (Ec1 - Ec) / dt - m.uqt[u];
                double g = Gr[(size_t)m.ubus[u] * T + t];
                if (d >= 0 && m.uetain[u] <= 0) {
                    dk[u] += cv * dt * d;
                } else if (d >= 0) {
                    double pc = d / m.uetain[u];
                    dk[u] += dt * m.umc[u] * pc + g * pc + (pc > 1 ? cv * dt * (pc - 1) : 0.0);
                } else {
                    double mcx = -d * m.uetaout[u];
                    double mcc = std::min(mcx, 1.0);
                    dk[u] += dt * m.umc[u] * mcc - g * mcc + ((mcx > 1 && m.uqt[u] <= 0) ? cv * dt * (mcx - 1) : 0.0);
                }
            }
        for (int t = 0; t < T; ++t)
            for (int j = 0; j < m.S; ++j) {
                int u = m.stor[j];
                double y = c.e[ix(c, j, t, rep)];
                if (!(0.0 < y && y < 1.0)) dk[u] += cv * m.uhours[u] * fabs(y - clampd(y, 0.0, 1.0));
            }
        // score: -beta_v mask dk + log measure gradient (src/replicas.jl:334, src/energy.jl:811)
        for (int u = 0; u < K; ++u) {
            double y = c.k[u];
            bool in = m.ulo[u] < y && y < m.uhi[u];
            double s = -m.beta_v * ((in ? 1.0 : 0.0) * dk[u]);
            double lm = 0.0;
            if (m.physical && m.ukind[u] != ESM_UNIT_REN && in) lm = (double)T / (y + k0);
            sk[(size_t)rep * K + u] = s + lm;
        }
        if (parts) {
            double capex = 0.0;
            for (int u = 0; u < K; ++u) {
                double kc = kcl(c, u);
                capex += m.ucapex[u] * c.k[u] + m.gamma_k * m.ucapex[u] * fabs(c.k[u] - kc);
            }
            double *P = parts + (size_t)rep * 8;
            P[0] = capex;
            P[1] = cgen + cst + (m.c_shed * shed + m.c_dump * dump) + pen;
            P[2] = cgen;
            P[3] = cst;
            P[4] = shed;
            P[5] = dump;
            P[6] = pen;
            P[7] = 0.0;
        }
    }
    for (int u = 0; u < K; ++u) {
        double ex = c.k[u] - kcl(c, u);
        double sg = ex > 0 ? 1.0 : (ex < 0 ? -1.0 : 0.0);
        fk[u] = m.beta_k * (m.ucapex[u] + m.gamma_k * m.ucapex[u] * sg);
    }
}

// ------------------------------------------------------------------------------------------
// Langevin step and dispatch following (src/replicas.jl:357-473, src/kop.jl)
// ------------------------------------------------------------------------------------------
static double langevin_one(double k, double g, double xi, double eta, double ks, double kmin, double clip, bool box,
                           double hi, int *nclip) {
    double w = log(k + ks);
    double dw0 = eta * ((k + ks) * g + 1);
    if (fabs(dw0) > clip) *nclip += 1;
    double w1 = w + clampd(dw0, -clip, clip) + sqrt(2 * eta) * xi;
    double wmin = log(kmin + ks);
    w1 = w1 < wmin ? 2 * wmin - w1 : w1;
    if (box) {
        double wmax = log(std::max(hi, kmin + 1.0) + ks);
        if (w1 > wmax && w <= wmax) w1 = std::max(2 * wmax - w1, wmin);
    }
    return exp(w1) - ks;
}

// set_dispatchable_capacity! (src/replicas.jl:412) for every replica
static void follow_disp(Ctx &c, const vector<double> &kold, const vector<double> &knew) {
    const Model &m = c.m;
    for (int j = 0; j < m.D; ++j) {
        int u = m.disp[j];
        double kc0 = clampd(kold[u], m.ulo[u], m.uhi[u]), kc1 = clampd(knew[u], m.ulo[u], m.uhi[u]);
        double sc = kc0 == kc1 ? 1.0 : kc0 / kc1;  // kc_ratio (src/local.jl:2119)
        if (sc == 1.0) continue;
        for (int t = 0; t < m.T; ++t)
            for (int rep = 0; rep < c.o.R; ++rep) {
                double &y = c.g[ix(c, j, t, rep)];
                y = y + y * (sc - 1);
            }
    }
}

// kop_prepare / kop_term / kop_eval(commit) (src/kop.jl:79-160, :223) for one unit, one replica;
// c.k[u] still holds the raw k0, the caller sets the new capacity afterwards
static void kop_unit(Ctx &c, int u, double k1, int rep, bool follow) {
    const Model &m = c.m;
    int T = m.T, n = m.ubus[u];
    double k0raw = c.k[u];
    double kc0 = clampd(k0raw, m.ulo[u], m.uhi[u]);
    double dt = m.dt;
    for (int t = 0; t < T; ++t) {
        double jinj;
        if (m.ukind[u] == ESM_UNIT_REN) {
            jinj = avail_map(wraw(c, m.useries[u], t, rep));
        } else {
            int sj = m.stor_of_unit[u];
            double pc, mcx;
            soc_power(m, u, dt, clampd(c.e[ix(c, sj, t, rep)], 0.0, 1.0), clampd(c.e[ix(c, sj, (t + 1) % T, rep)], 0.0, 1.0),
                      &pc, &mcx);
            jinj = mcx - pc;
        }
        double Pt = 0.0, Qs = 0.0;
        int nu = 0;
        for (int q = m.up[n]; q < m.up[n + 1]; ++q) {
            int j = m.ua[q];
            double kap = kappa_unit(c, j);
            if (!(fabs(kap) >= c.o.kmin)) continue;
            double om = c.g[ix(c, j, t, rep)];
            Pt += kap * om;
            Qs += kap * clampd(om, 0.0, 1.0);
            nu += 1;
        }
        double kc1 = clampd(k1, m.ulo[u], m.uhi[u]);
        double dkc = kc1 - kc0;
        double dinj = jinj * dkc;
        double dS = -dinj;
        // below kmin the capacity moves alone (src/replicas.jl:461): the residual takes the change
        if (follow && !(nu == 0 || fabs(Pt) < 1e-6)) {
            double Q = c.r[ix(c, n, t, rep)] + Qs;
            double e = Pt - std::max(Q, 0.0);
            double P1 = std::max(Q - dinj, 0.0) + e;
            for (int q = m.up[n]; q < m.up[n + 1]; ++q) {
                int j = m.ua[q];
                double kap = kappa_unit(c, j);
                if (!(fabs(kap) >= c.o.kmin)) continue;
                double y0 = c.g[ix(c, j, t, rep)];
                double sigma = kap * y0 / Pt;
                double y1 = sigma * P1 / kap;
                dS -= kap * (clampd(y1, 0.0, 1.0) - clampd(y0, 0.0, 1.0));
                c.g[ix(c, j, t, rep)] = y1;
            }
        }
        c.r[ix(c, n, t, rep)] += dS;
    }
}

static void langevin_step(Ctx &c, const double *w, const double *eta, const double *kappa_s, double kmin, double clip,
                          int box, const double *xi, int64_t it, double *knew_out, int *nclip_out, int nthreads) {
    const Model &m = c.m;
    int K = m.K, R = c.o.R;
    const vector<double> &sk = c.sk_last, &fk = c.fk_last;
    double ratio = m.beta_k / m.beta_v;
    vector<double> knew = c.k;
    int nclip = 0;
    int ngroups = 0;
    for (int u = 0; u < K; ++u) ngroups = std::max(ngroups, m.ugroup[u] + 1);
    for (int gidx = 0; gidx < ngroups; ++gidx) {
        if (eta[gidx] == 0) continue;
        int jj = 0;
        for (int u = 0; u < K; ++u) {
            if (m.ugroup[u] != gidx) continue;
            double sbar = 0.0;
            for (int rep = 0; rep < R; ++rep) sbar += w[rep] * sk[(size_t)rep * K + u];
            double g = -fk[u] + ratio * sbar;
            double x = xi ? xi[u] : orc_normal(c.o.seed, ESM_TAG_LGV, (uint32_t)jj, (uint32_t)gidx, (uint32_t)it, 0);
            knew[u] = langevin_one(c.k[u], g, x, eta[gidx], kappa_s[gidx], kmin, clip, box != 0, m.uhi[u], &nclip);
            ++jj;
        }
    }
    // follow_capacities! (src/replicas.jl:448)
    vector<double> kold = c.k;
    follow_disp(c, kold, knew);
    for (int u = 0; u < K; ++u)
        if (m.ukind[u] == ESM_UNIT_DISP) c.k[u] = knew[u];
    rebuild(c, nthreads);
#pragma omp parallel for schedule(static) num_threads(nthreads)
    for (int rep = 0; rep < R; ++rep)
        for (int u = 0; u < K; ++u) {
            if (m.ukind[u] == ESM_UNIT_DISP) continue;
            if (kold[u] >= kmin)
                kop_unit(c, u, kold[u] * exp(log(knew[u] / kold[u])), rep, true);
            else
                kop_unit(c, u, knew[u], rep, false);
        }
    for (int u = 0; u < K; ++u) {
        if (m.ukind[u] == ESM_UNIT_DISP) continue;
        c.k[u] = kold[u] >= kmin ? kold[u] * exp(log(knew[u] / kold[u])) : knew[u];
    }
    rebuild(c, nthreads);
    if (knew_out)
        for (int u = 0; u < K; ++u) knew_out[u] = c.k[u];
    if (nclip_out) *nclip_out = nclip;
}

// ------------------------------------------------------------------------------------------
// weather process of one replica (src/replicas.jl:49-112 pCN in the VAR innovations, :131-167
// regime window, :207 compensate_weather!), for the diagonal single-level VAR of the model
// ------------------------------------------------------------------------------------------
static inline double var_mean(const Model &m, int k, int i, double zprev, int t) {
    double tau = t + 1;  // harmonics(tau, T0) with the reference's 1-based step (src/weather.jl:47)
    double cs = cos(2 * M_PI * tau / m.T), sn = sin(2 * M_PI * tau / m.T);
    const double *mu = &m.mu[((size_t)k * m.n0 + i) * 3];
    return m.phi[(size_t)k * m.n0 + i] * zprev + 1.0 * mu[0] + cs * mu[1] + sn * mu[2];
}

// innovations of series i at regimes regA, rotated by theta (if > 0), rebuilt at regimes regB
static void series_pass(Ctx &c, int i, int rep, const int *regA, const int *regB, double theta, const double *xi,
                        int64_t it) {
    const Model &m = c.m;
    double zpo = 0, zpn = 0;
    double ct = cos(theta), st = sin(theta);
    for (int t = 0; t < m.T; ++t) {
        double zo = c.z[ix(c, i, t, rep)];
        int ka = regA[t], kb = regB[t];
        double e = t == 0 ? zo / m.sig0[i] : (zo - var_mean(m, ka, i, zpo, t)) / m.sig[(size_t)ka * m.n0 + i];
        if (theta > 0) {
            double x = xi ? xi[(size_t)t * m.n0 + i]
                          : orc_normal(c.o.seed, ESM_TAG_WTH, (uint32_t)((size_t)t * m.n0 + i), 0, (uint32_t)rep,
                                       (uint32_t)it);
            e = ct * e + st * x;
        }
        double zn = t == 0 ? m.sig0[i] * e : var_mean(m, kb, i, zpn, t) + m.sig[(size_t)kb * m.n0 + i] * e;
        c.z[ix(c, i, t, rep)] = zn;
        zpo = zo;
        zpn = zn;
    }
}

// regime_window (src/replicas.jl:131-163) with the uniforms of the stream; a is 1-based
static void regime_window(const Ctx &c, const vector<int> &reg, int a, int b, int rep, int64_t it, vector<int> &out) {
    const Model &m = c.m;
    int K = m.nreg, T0 = m.T, B = b - a + 1;
    out = reg;
    vector<double> beta((size_t)K * B, 1.0);
    if (b < T0) {
        for (int q = 0; q < K; ++q) beta[(size_t)q * B + (B - 1)] = m.Ptr[(size_t)q * K + reg[b]];
        for (int tau = b - 1; tau >= a; --tau) {
            int col = tau - a, nxt = tau - a + 1;
            for (int q = 0; q < K; ++q) {
                double s = 0.0;
                for (int p = 0; p < K; ++p) s += m.Ptr[(size_t)q * K + p] * beta[(size_t)p * B + nxt];
                beta[(size_t)q * B + col] = s;
            }
        }
    }
    for (int tau = a; tau <= b; ++tau) {
        double u, u2;
        int j = tau - a;
        orc_uniform2(c.o.seed, ESM_TAG_WTH, (uint32_t)(j >> 1), 1, (uint32_t)rep, (uint32_t)it, &u, &u2);
        if (j & 1) u = u2;
        vector<double> p(K);
        double tot = 0.0;
        for (int q = 0; q < K; ++q) {
            double pr = tau == 1 ? m.pi0[q] : m.Ptr[(size_t)out[tau - 2] * K + q];
            p[q] = pr * beta[(size_t)q * B + (tau - a)];
            tot += p[q];
        }
        double tt = u * tot, cc = 0.0;
        int kk = K - 1;
        for (int q = 0; q < K; ++q) {
            cc += p[q];
            if (tt <= cc) {
                kk = q;
                break;
            }
        }
        out[tau - 1] = kk;
    }
}

// compensate_weather! (src/replicas.jl:207) of one replica from the residual r0 before the change
static void compensate(Ctx &c, int rep, const vector<double> &r0) {
    const Model &m = c.m;
    for (int n = 0; n < m.N; ++n)
        for (int t = 0; t < m.T; ++t) {
            double need = c.r[ix(c, n, t, rep)] - r0[(size_t)n * m.T + t];
            if (fabs(need) < 1e-6) continue;
            int nu = m.up[n + 1] - m.up[n];
            if (nu == 0) continue;
            vector<double> ks(nu), wq(nu);
            double tot = 0.0;
            for (int q = 0; q < nu; ++q) {
                int j = m.ua[m.up[n] + q];
                ks[q] = kappa_unit(c, j);
                double ps = ks[q] * clampd(c.g[ix(c, j, t, rep)], 0.0, 1.0);
                wq[q] = need > 0 ? std::max(ks[q] - ps, 0.0) : ps;
                tot += wq[q];
            }
            if (!(tot > 1e-9)) continue;
            double a = need > 0 ? std::min(need, tot) / tot : std::max(need, -tot) / tot;
            for (int q = 0; q < nu; ++q) {
                if (fabs(ks[q]) < 1e-9) continue;
                double dy = a * wq[q] / ks[q];
                if (dy == 0.0) continue;
                c.g[ix(c, m.ua[m.up[n] + q], t, rep)] += dy;
            }
        }
}

// weather_process_step + compensation for the flagged replicas; wstart is the 1-based window start
static void weather_step(Ctx &c, const int *moved, const double *theta, const int *window, const int *wstart,
                         const double *xi, int64_t it, int nthreads) {
    const Model &m = c.m;
    int R = c.o.R, T = m.T;
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads)
    for (int rep = 0; rep < R; ++rep) {
        if (!moved[rep]) continue;
        for (int t = 0; t < T; ++t) rebuild_step(c, t, rep);
        vector<double> r0((size_t)m.N * T);
        for (int n = 0; n < m.N; ++n)
            for (int t = 0; t < T; ++t) r0[(size_t)n * T + t] = c.r[ix(c, n, t, rep)];
        vector<int> reg(T);
        for (int t = 0; t < T; ++t) reg[t] = c.reg[(size_t)t * R + rep];
        const double *xr = xi ? xi + (size_t)rep * m.n0 * T : nullptr;
        if (theta[rep] > 0)
            for (int i = 0; i < m.n0; ++i) series_pass(c, i, rep, reg.data(), reg.data(), theta[rep], xr, it);
        if (window[rep] > 0) {
            int a = std::max(1, std::min(T, wstart[rep]));
            int b = std::min(T, a + window[rep] - 1);
            vector<int> reg2;
            regime_window(c, reg, a, b, rep, it, reg2);
            for (int i = 0; i < m.n0; ++i) series_pass(c, i, rep, reg.data(), reg2.data(), 0.0, nullptr, it);
            for (int t = 0; t < T; ++t) c.reg[(size_t)t * R + rep] = reg2[t];
        }
        for (int t = 0; t < T; ++t) rebuild_step(c, t, rep);
        compensate(c, rep, r0);
        for (int t = 0; t < T; ++t) rebuild_step(c, t, rep);
    }
}

}  // namespace

// ============================================================================================
// C entry points of the oracle (ctypes)
// ============================================================================================
extern "C" {

double orc_logseg(double L, double x) { return logseg(L, x); }
double orc_trexp_offset(double u, double g, double L) { return trexp_offset(u, g, L); }
void orc_philox4(uint32_t k0, uint32_t k1, uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint32_t *out) {
    orc_philox(k0, k1, c0, c1, c2, c3, out);
}
double orc_normal_at(uint64_t seed, uint32_t tag, uint32_t j, uint32_t c1, uint32_t c2, uint32_t c3) {
    return orc_normal(seed, tag, j, c1, c2, c3);
}

// langevin_update (src/replicas.jl:368) on one field
int orc_langevin_update(int n, const double *k, const double *g, const double *xi, double eta, double ks, double kmin,
                        double clip, const double *hi, double *out) {
    int nclip = 0;
    for (int i = 0; i < n; ++i)
        out[i] = langevin_one(k[i], g[i], xi[i], eta, ks, kmin, clip, hi != nullptr, hi ? hi[i] : 0.0, &nclip);
    return nclip;
}

void *orc_create(const esm_model *em, const esm_opts *eo) {
    Ctx *c = new Ctx();
    Model &m = c->m;
    m.N = em->N;
    m.L = em->L;
    m.T = em->T;
    m.K = em->K;
    m.D = em->D;
    m.S = em->S;
    m.n0 = em->n0;
    m.nreg = em->nreg;
    m.nfields = em->nfields;
    m.nlev = em->nlev;
    m.dt = em->dt;
    m.c_shed = em->c_shed;
    m.c_dump = em->c_dump;
    m.c_viol = em->c_viol;
    m.gamma_k = em->gamma_k;
    m.kappa0 = em->kappa0;
    m.beta_v = em->beta_v;
    m.beta_k = em->beta_k;
    m.physical = em->physical != 0;
    int N = m.N, L = m.L, K = m.K;
    m.bus0 = cp_(em->bus0, L);
    m.bus1 = cp_(em->bus1, L);
    m.lb = cp_(em->line_b, L);
    m.ls = cp_(em->line_s, L);
    m.ukind = cp_(em->unit_kind, K);
    m.ugroup = cp_(em->unit_group, K);
    m.ubus = cp_(em->unit_bus, K);
    m.useries = cp_(em->unit_series, K);
    m.umc = cp_(em->unit_mc, K);
    m.ucapex = cp_(em->unit_capex, K);
    m.ulo = cp_(em->unit_lo, K);
    m.uhi = cp_(em->unit_hi, K);
    m.uavail = cp_(em->unit_avail, K);
    m.uhours = cp_(em->unit_hours, K);
    m.uetain = cp_(em->unit_eta_in, K);
    m.uetaout = cp_(em->unit_eta_out, K);
    m.uqt = cp_(em->unit_qt, K);
    m.disp = cp_(em->disp, m.D);
    m.stor = cp_(em->stor, m.S);
    m.sfield = cp_(em->series_field, m.n0);
    m.snode = cp_(em->series_node, m.n0);
    m.xbar = cp_(em->xbar, (size_t)m.n0 * m.T);
    m.wscale = cp_(em->wscale, m.n0);
    m.Ptr = cp_(em->Ptr, (size_t)m.nreg * m.nreg);
    m.pi0 = cp_(em->pi0, m.nreg);
    m.phi = cp_(em->phi, (size_t)m.nreg * m.n0);
    m.mu = cp_(em->mu, (size_t)m.nreg * m.n0 * 3);
    m.sig = cp_(em->sig, (size_t)m.nreg * m.n0);
    m.sig0 = cp_(em->sig0, m.n0);
    m.frole = cp_(em->field_role, m.nfields);
    m.fap = cp_(em->field_atom_ptr, m.nfields + 1);
    int natoms = m.fap[m.nfields];
    m.ap = cp_(em->atom_ptr, natoms + 1);
    m.ai = cp_(em->atom_idx, m.ap[natoms]);
    m.av = cp_(em->atom_val, m.ap[natoms]);
    m.nlp = cp_(em->nodelines_ptr, N + 1);
    m.nl = cp_(em->nodelines, m.nlp[N]);
    m.up = cp_(em->units_ptr, N + 1);
    m.ua = cp_(em->units_at, m.up[N]);
    m.sp = cp_(em->stor_ptr, N + 1);
    m.sa = cp_(em->stor_at, m.sp[N]);
    m.qcum = cp_(em->qcum, m.nlev);
    m.clp = cp_(em->cell_level_ptr, m.nlev + 1);
    int ncell = m.clp[m.nlev];
    m.cp = cp_(em->cell_ptr, ncell + 1);
    m.cu = cp_(em->cell_units, m.cp[ncell]);
    m.xpp = cp_(em->xpart_ptr, N + 1);
    int npair = m.xpp[N];
    m.xp = cp_(em->xpart, npair);
    m.xnp = cp_(em->xnod_ptr, npair + 1);
    m.xn = cp_(em->xnod, m.xnp[npair]);
    m.xv = cp_(em->xval, m.xnp[npair]);
    m.xlp = cp_(em->xlk_ptr, npair + 1);
    m.xln = cp_(em->xlkn, m.xlp[npair]);
    m.xlg = cp_(em->xlkg, m.xlp[npair]);
    m.Z = cp_(em->reroute, (size_t)N * N);
    m.comp = cp_(em->comp, N);
    m.sgp = cp_(em->sgroup_ptr, (size_t)em->nsgroups + 1);
    m.sgu = cp_(em->sgroup_units, (size_t)m.sgp[em->nsgroups]);
    m.theta_nnz.assign(N, 0);
    for (int f = 0; f < m.nfields; ++f) {
        if (m.frole[f] != ESM_ROLE_THETA) continue;
        for (int a = m.fap[f]; a < m.fap[f + 1]; ++a)
            for (int q = m.ap[a]; q < m.ap[a + 1]; ++q) m.theta_nnz[m.ai[q]] += 1;
    }
    m.disp_of_unit.assign(K, -1);
    m.stor_of_unit.assign(K, -1);
    for (int j = 0; j < m.D; ++j) m.disp_of_unit[m.disp[j]] = j;
    for (int j = 0; j < m.S; ++j) m.stor_of_unit[m.stor[j]] = j;
    Opts &o = c->o;
    o.R = eo->R;
    o.max_points = eo->max_points;
    if (o.max_points == 0) {  // automatic, as esm_auto_max_points
        int mx = 1;
        for (int f = 0; f < m.nfields; ++f)
            if (m.frole[f] == ESM_ROLE_SE)
                for (int a = m.fap[f]; a < m.fap[f + 1]; ++a) mx = std::max(mx, m.ap[a + 1] - m.ap[a]);
        o.max_points = esm_auto_max_points(mx);
    }
    o.span = eo->span;
    o.seed = eo->seed;
    o.extra = eo->extra;
    o.maxnats = eo->maxnats;
    o.kmin = eo->kappa_min;
    for (int q = 0; q < ESM_NFAM; ++q) o.rates[q] = eo->family_rates[q];
    o.storage_ms = eo->storage_ms;
    o.storage_long = eo->storage_long;
    size_t TR = (size_t)m.T * o.R;
    c->theta.assign(N * TR, 0.0);
    c->g.assign(m.D * TR, 0.0);
    c->e.assign(m.S * TR, 0.0);
    c->z.assign(m.n0 * TR, 0.0);
    c->reg.assign(TR, 0);
    c->k.assign(K, 0.0);
    c->r.assign(N * TR, 0.0);
    c->F.assign(L * TR, 0.0);
    return c;
}

void orc_destroy(void *p) { delete (Ctx *)p; }

void orc_set_state(void *p, const double *theta, const double *g, const double *e, const double *z, const int32_t *reg,
                   const double *k) {
    Ctx *c = (Ctx *)p;
    if (theta) std::copy(theta, theta + c->theta.size(), c->theta.begin());
    if (g) std::copy(g, g + c->g.size(), c->g.begin());
    if (e) std::copy(e, e + c->e.size(), c->e.begin());
    if (z) std::copy(z, z + c->z.size(), c->z.begin());
    if (reg) std::copy(reg, reg + c->reg.size(), c->reg.begin());
    if (k) std::copy(k, k + c->k.size(), c->k.begin());
}

void orc_get_state(void *p, double *theta, double *g, double *e, double *z, int32_t *reg, double *k) {
    Ctx *c = (Ctx *)p;
    if (theta) std::copy(c->theta.begin(), c->theta.end(), theta);
    if (g) std::copy(c->g.begin(), c->g.end(), g);
    if (e) std::copy(c->e.begin(), c->e.end(), e);
    if (z) std::copy(c->z.begin(), c->z.end(), z);
    if (reg) std::copy(c->reg.begin(), c->reg.end(), reg);
    if (k) std::copy(c->k.begin(), c->k.end(), k);
}

void orc_rebuild(void *p, int nthreads) { rebuild(*(Ctx *)p, nthreads); }

void orc_get_caches(void *p, double *r, double *F) {
    Ctx *c = (Ctx *)p;
    if (r) std::copy(c->r.begin(), c->r.end(), r);
    if (F) std::copy(c->F.begin(), c->F.end(), F);
}

void orc_set_caches(void *p, const double *r, const double *F) {
    Ctx *c = (Ctx *)p;
    if (r) std::copy(r, r + c->r.size(), c->r.begin());
    if (F) std::copy(F, F + c->F.size(), c->F.begin());
}

// one class of one sweep (caches must be current)
void orc_class_pass(void *p, int64_t sweep, int cls, int limit, int64_t *stats, int nthreads) {
    class_pass(*(Ctx *)p, (uint32_t)sweep, cls, stats, nthreads, limit);
}

// n sweeps: caches rebuilt at each sweep start (LocalCost, src/local.jl:1940), classes in the
// sweep's order
// Moves [m0, m1) of every task of class cls of sweep `sweep` (m1 < 0: to the end of the list); the
// selection draws of the earlier moves are replayed, so the range continues a pass that ran [0, m0).
// tlog (may be NULL): the t of every move of the range, at [(move * nsteps + q) * R + rep] for the
// class's q-th step (entries of moves that made no move are left as they are).
void orc_class_pass_range(void *p, int64_t sweep, int cls, int m0, int m1, int64_t *stats, int nthreads,
                          double *tlog) {
    Ctx *c = (Ctx *)p;
    if (m1 >= 0 && m1 <= m0) return;
    class_pass(*c, (uint32_t)sweep, cls, stats, nthreads, m1 > 0 ? m1 : 0, m0, tlog);
}

// Moves [m0, m1) (m1 < 0: to the end) of one task of a class pass: the class's q-th step of replica
// rep (the tasks of a class are independent, so this advances that task alone). Returns the number
// of moves in the class list.
int orc_task_moves(void *p, int64_t sweep, int cls, int q, int rep, int m0, int m1) {
    Ctx &c = *(Ctx *)p;
    vector<int> steps;
    class_steps(c.m.T, cls, steps);
    if (q < 0 || q >= (int)steps.size() || rep < 0 || rep >= c.o.R) return -1;
    TileStream ts0{c.o.seed, 0u, (uint32_t)cls, (uint32_t)sweep};
    vector<MoveRef> moves;
    move_list(c, ts0, moves);
    WS ws, wa;
    ws.init(c.m);
    wa.init(c.m);
    vector<int64_t> st(2 * (ESM_NFAM + 1) + 1, 0);
    if (m1 >= 0 && m1 <= m0) return (int)moves.size();
    run_task(c, moves, ts0, steps[q], rep, (uint32_t)sweep, st.data(), ws, wa, m1 > 0 ? m1 : 0, m0);
    return (int)moves.size();
}

void orc_sweeps(void *p, int n, int64_t sweep0, int64_t *stats, int nthreads) {
    Ctx *c = (Ctx *)p;
    for (int s = 0; s < n; ++s) {
        uint32_t sw = (uint32_t)(sweep0 + s);
        rebuild(*c, nthreads);
        int order[3], ncls;
        class_order(*c, sw, order, &ncls);
        for (int q = 0; q < ncls; ++q) class_pass(*c, sw, order[q], stats, nthreads);
        if (c->o.storage_ms) {
            int64_t s3[3] = {0, 0, 0};
            sms_sweep(*c, sw, false, s3, nthreads);
            for (int i = 0; i < 3; ++i) c->sms_stats[i] += s3[i];
        }
        if (c->o.storage_long) {
            int64_t s3[3] = {0, 0, 0};
            sl_sweep(*c, sw, s3, nthreads);
        }
    }
}

// the storage multiscale sweep of sweep `sweep` (with force, whatever its coin; max_passes > 0: its
// first class passes only); stats3 += (moves tried, moves taken, guard events)
void orc_storage_ms(void *p, int64_t sweep, int force, int max_passes, int64_t *stats3, int nthreads) {
    sms_sweep(*(Ctx *)p, (uint32_t)sweep, force != 0, stats3, nthreads, max_passes);
}

// the long-range storage sweep of sweep `sweep`; stats3 += (moves tried, moves taken, guard events)
void orc_storage_long(void *p, int64_t sweep, int64_t *stats3, int nthreads) {
    sl_sweep(*(Ctx *)p, (uint32_t)sweep, stats3, nthreads);
}

// the same with the t of every move of the eligible units' tasks logged at [(ui * 5 + m) * R + rep]
// (ui the unit's place among the eligible units, m its move; moves that made no move are left as
// they are)
void orc_storage_long_log(void *p, int64_t sweep, int64_t *stats3, int nthreads, double *tlog) {
    sl_sweep(*(Ctx *)p, (uint32_t)sweep, stats3, nthreads, tlog);
}

// Moves [m0, m1) (m1 < 0: to the end) of one task of the long-range sweep: the ui-th eligible unit,
// replica rep (no cache rebuild: call after a sweep or orc_rebuild). Returns the moves of its list.
int orc_sl_task(void *p, int64_t sweep, int ui, int rep, int m0, int m1) {
    Ctx &c = *(Ctx *)p;
    vector<int> units;
    vector<vector<SlMove>> moves;
    sl_plan(c, (uint32_t)sweep, units, moves);
    if (ui < 0 || ui >= (int)units.size() || rep < 0 || rep >= c.o.R) return -1;
    vector<WS> wss(c.m.T);
    for (auto &w : wss) w.init(c.m);
    vector<Kink> jac;
    int64_t loc[3] = {0, 0, 0};
    if (!(m1 >= 0 && m1 <= m0)) sl_task(c, (uint32_t)sweep, ui, units[ui], rep, moves[ui], m0, m1, wss, jac, loc, nullptr);
    return (int)moves[ui].size();
}

static void explain_mover(Ctx &c, Mover &mv, vector<Kink> &jac, bool compensated, double uc, double uo, double uj,
                          double t_other, double *out);

// orc_explain for move mi of the ui-th eligible unit's task (replica rep) of the long-range sweep on
// the current state; out as orc_explain (16: -2 a level move, -3 a long-range plateau; 17: its
// length). Returns 1, 0 when the move makes no move, -1 on a bad index.
int orc_sl_explain(void *p, int64_t sweep, int ui, int rep, int mi, double t_other, double *out) {
    Ctx &c = *(Ctx *)p;
    const Model &m = c.m;
    int T = m.T;
    vector<int> units;
    vector<vector<SlMove>> moves;
    sl_plan(c, (uint32_t)sweep, units, moves);
    if (ui < 0 || ui >= (int)units.size() || rep < 0 || rep >= c.o.R) return -1;
    if (mi < 0 || mi >= (int)moves[ui].size()) return -1;
    for (int i = 0; i < 24; ++i) out[i] = NAN;
    vector<WS> wss(T);
    for (auto &w : wss) w.init(m);
    vector<Kink> jac;
    int j = units[ui];
    const SlMove &sm = moves[ui][mi];
    bool level = sm.L == T;
    if (level)
        prep_level(c, wss, j, rep);
    else if (!prep_plateau(c, wss, sm.a, sm.L, {j}, rep, &jac))
        return 0;
    Mover mv{&c, {}, rep, m.beta_v, {}};
    mv.cyclic = level;
    int n = level ? T : sm.L + 1;
    for (int k = 0; k < n; ++k) mv.w.push_back(&wss[k]);
    double uc, uo, uj, un;
    orc_uniform2(c.o.seed, ESM_TAG_SLL, 2u * (uint32_t)mi, (uint32_t)j, (uint32_t)rep, (uint32_t)sweep, &uc, &uo);
    orc_uniform2(c.o.seed, ESM_TAG_SLL, 2u * (uint32_t)mi + 1, (uint32_t)j, (uint32_t)rep, (uint32_t)sweep, &uj, &un);
    out[16] = level ? -2.0 : -3.0;
    out[17] = sm.L;
    explain_mover(c, mv, jac, !level, uc, uo, uj, t_other, out);
    for (auto &w : wss) w.clear();
    return 1;
}

// its plan: per eligible unit (stor index) its moves (length, start); returns the number of moves
int orc_storage_long_plan(void *p, int64_t sweep, int32_t *out, int maxn) {
    Ctx *c = (Ctx *)p;
    vector<int> units;
    vector<vector<SlMove>> moves;
    sl_plan(*c, (uint32_t)sweep, units, moves);
    int n = 0;
    for (size_t u = 0; u < units.size(); ++u)
        for (auto &x : moves[u])
            if (n < maxn) {
                out[3 * n] = units[u];
                out[3 * n + 1] = x.L;
                out[3 * n + 2] = x.a;
                ++n;
            }
    return n;
}

// the class passes of the storage multiscale sweep of a sweep: (length, offset, parity) each
int orc_storage_ms_plan(void *p, int64_t sweep, int force, int32_t *out) {
    Ctx *c = (Ctx *)p;
    SmsPass ps[14];
    int n = sms_plan(c->o.seed, c->m.T, (uint32_t)sweep, force != 0, ps);
    for (int i = 0; i < n; ++i) {
        out[3 * i] = ps[i].L;
        out[3 * i + 1] = ps[i].o;
        out[3 * i + 2] = ps[i].cls;
    }
    return n;
}

// the move list of a tile (diagnostics): kind (-1 atom, else family), field, atom
int orc_move_list(void *p, int64_t sweep, int cls, int tile, int *kinds, int *fields, int *atoms, int maxn) {
    Ctx *c = (Ctx *)p;
    (void)tile;  // the list is shared by all tiles of the class
    TileStream ts{c->o.seed, 0u, (uint32_t)cls, (uint32_t)sweep};
    vector<MoveRef> moves;
    move_list(*c, ts, moves);
    int n = (int)moves.size() < maxn ? (int)moves.size() : maxn;
    for (int i = 0; i < n; ++i) {
        kinds[i] = moves[i].kind;
        fields[i] = moves[i].field;
        atoms[i] = moves[i].atom;
    }
    return (int)moves.size();
}

// One move of family `fam` at 0-based step tau of replica rep, its selection drawn from a fresh
// stream (seed, tile 0, cls, sweep), moved by t (commit != 0) or only prepared: returns 1 if the
// selection made a move, the log-Jacobian at t (logjac, src/local.jl:1871) in *lj and the first
// kink's requirement and slope in kq[0], kq[1] (0 and 0 without kinks), and the cost change the
// move evaluates at t (mv_eval!) in *dc. The checks of the reference's reversibility and
// exactness tests (test/test_local.jl:285-345, test/test_moves.jl) call it.
int orc_move_at(void *p, int fam, int tau, int rep, int cls, int64_t sweep, double t, int commit_it, double *lj,
                double *kq, double *dc) {
    Ctx &c = *(Ctx *)p;
    const Model &m = c.m;
    WS ws, wa;
    ws.init(m);
    wa.init(m);
    ws.tau = tau;
    wa.tau = (tau - 1 + m.T) % m.T;
    vector<Kink> jac;
    TileStream ts{c.o.seed, 0u, (uint32_t)cls, (uint32_t)sweep};
    *lj = 0.0;
    *dc = 0.0;
    kq[0] = kq[1] = 0.0;
    if (!prep_family(c, ts, fam, ws, wa, rep, &jac)) return 0;
    finalize_ws(c, ws, rep);
    if (ws.ent.empty()) return 0;
    finalize_ws(c, wa, rep);
    link_soc(m, wa, ws);
    for (auto &k : jac) *lj += k.nm * log(fabs((std::max(k.Q + k.g * t, 0.0) + k.e) / k.Pm));
    if (!jac.empty()) {
        kq[0] = jac[0].Q;
        kq[1] = jac[0].g;
    }
    Mover mv{&c, {&wa, &ws}, rep, m.beta_v, {}};
    *dc = mv.eval(t);
    if (commit_it) commit(c, mv, t);
    return 1;
}

// The walk of the same move (both directions, merged in ascending order with t = 0): points in
// pts and potentials beta * DeltaC in cs, at most maxn; returns their number, 0 if the selection
// made no move, -1 at the point cap. For the reference's walk-linearity check (test/test_moves.jl
// 1a: the potential is linear between consecutive points).
int orc_move_walk(void *p, int fam, int tau, int rep, int cls, int64_t sweep, double *pts, double *cs, int maxn) {
    Ctx &c = *(Ctx *)p;
    const Model &m = c.m;
    WS ws, wa;
    ws.init(m);
    wa.init(m);
    ws.tau = tau;
    wa.tau = (tau - 1 + m.T) % m.T;
    vector<Kink> jac;
    TileStream ts{c.o.seed, 0u, (uint32_t)cls, (uint32_t)sweep};
    if (!prep_family(c, ts, fam, ws, wa, rep, &jac)) return 0;
    finalize_ws(c, ws, rep);
    if (ws.ent.empty()) return 0;
    finalize_ws(c, wa, rep);
    link_soc(m, wa, ws);
    Mover mv{&c, {&wa, &ws}, rep, m.beta_v, {}};
    vector<double> right, left;
    for (const WS *w : mv.w)
        for (double x : w->bps) {
            if (!std::isfinite(x)) continue;
            if (x > 0.0)
                right.push_back(x);
            else if (x < 0.0)
                left.push_back(x);
        }
    mv.eval(0.0);
    vector<double> sec0 = mv.sec;
    Walk Wr, Wl;
    Wr.cap = Wl.cap = c.o.max_points > 0 ? c.o.max_points : 4096;
    if (!walk(Wr, mv, right, 1.0, c.o.maxnats, sec0) || Wr.full) return -1;
    if (!walk(Wl, mv, left, -1.0, c.o.maxnats, sec0) || Wl.full) return -1;
    int n = 0;
    auto put = [&](double x, double cx) {
        if (n < maxn) {
            pts[n] = x;
            cs[n] = cx;
        }
        ++n;
    };
    for (int j = (int)Wl.pts.size() - 1; j >= 0; --j) put(Wl.pts[j], Wl.cs[j]);
    put(0.0, 0.0);
    for (size_t j = 0; j < Wr.pts.size(); ++j) put(Wr.pts[j], Wr.cs[j]);
    return n;
}

// Diagnosis of one move of a class pass (test infrastructure): move mi of the class list of
// (cls, sweep) at the class's q-th step, replica rep, prepared on the current state (call it after
// orc_class_pass_range ran moves [0, mi)), with its walks and draws; t_other is the t another
// implementation drew for the same move. out[0..19]:
//   0 t drawn (before the Jacobian test), 1 t after it, 2 segments, 3 the drawn segment jj,
//   4 the segment holding t_other (-1 outside the walks, -2 t_other = 0), 5 how far u = u_cat tot
//   lies from that segment's cumulative-mass interval, relative to tot (0 inside), 6 the distance of
//   u from the nearer end of jj's interval, relative to tot, 7 log-Jacobian at t, 8 the Jacobian
//   uniform, 9 log-Jacobian at t_other, 10/11 the stop margins of the right and left walks
//   (c - cmin - maxnats where they stopped), 12/13 the largest c - cmin - maxnats at an earlier
//   primary breakpoint or ray point (how near an earlier stop came), 14/15 their points, 16 the
//   family (-1 atom), 17 the move's entries, 18 0 proper walks, 1 improper, 2 point cap, 19 tot,
//   20/21 where the right and left walks began their ray steps (NaN: none), 22 |g L| of the drawn
//   segment (the potential's change across it, nats), 23 its length L.
// Returns 1, 0 when the selection made no move, -1 on a bad index.
// the explanation of one prepared move (its Mover, Jacobian kinks and uniforms) for orc_explain and
// orc_sl_explain: out[0..23] as orc_explain describes (16 and 17 are set by the caller)
static void explain_mover(Ctx &c, Mover &mv, vector<Kink> &jac, bool compensated, double uc, double uo, double uj,
                          double t_other, double *out) {
    out[8] = uj;
    vector<double> right, left;
    for (const WS *w : mv.w)
        for (double x : w->bps) {
            if (!std::isfinite(x)) continue;
            if (x > 0.0)
                right.push_back(x);
            else if (x < 0.0)
                left.push_back(x);
        }
    mv.eval(0.0);
    vector<double> sec0 = mv.sec;
    Walk Wr, Wl;
    Wr.cap = Wl.cap = c.o.max_points;
    int okr = walk(Wr, mv, right, 1.0, c.o.maxnats, sec0);
    int okl = okr && !Wr.full ? walk(Wl, mv, left, -1.0, c.o.maxnats, sec0) : 0;
    out[10] = Wr.stop;
    out[11] = Wl.stop;
    out[12] = Wr.near_;
    out[13] = Wl.near_;
    out[14] = (double)Wr.pts.size();
    out[15] = (double)Wl.pts.size();
    out[20] = Wr.ray_from;
    out[21] = Wl.ray_from;
    auto ljac = [&](double t) {
        double lj = 0.0;
        for (auto &k : jac) lj += k.nm * log(fabs((std::max(k.Q + k.g * t, 0.0) + k.e) / k.Pm));
        return lj;
    };
    if (Wr.full || Wl.full) {
        out[18] = 2;
        out[0] = out[1] = 0.0;
        return;
    }
    if (!okr || !okl) {
        out[18] = 1;
        out[0] = out[1] = 0.0;
        return;
    }
    out[18] = 0;
    vector<double> pts, cs;
    for (int j = (int)Wl.pts.size() - 1; j >= 0; --j) {
        pts.push_back(Wl.pts[j]);
        cs.push_back(Wl.cs[j]);
    }
    pts.push_back(0.0);
    cs.push_back(0.0);
    pts.insert(pts.end(), Wr.pts.begin(), Wr.pts.end());
    cs.insert(cs.end(), Wr.cs.begin(), Wr.cs.end());
    int nseg = (int)pts.size() - 1;
    vector<double> lm(nseg), A(nseg + 1, 0.0);
    double mx = -INFINITY;
    for (int j = 0; j < nseg; ++j) {
        double L = pts[j + 1] - pts[j];
        lm[j] = L > 0 ? -std::min(cs[j], cs[j + 1]) + logseg(L, fabs(cs[j + 1] - cs[j])) : -INFINITY;
        mx = std::max(mx, lm[j]);
    }
    double tot = 0.0;
    for (int j = 0; j < nseg; ++j) tot += exp(lm[j] - mx);
    double u = uc * tot, acc = 0.0;
    int jj = nseg - 1;
    bool found = false;
    for (int k = 0; k < nseg; ++k) {
        acc += exp(lm[k] - mx);
        A[k + 1] = acc;
        if (!found && u <= acc) {
            jj = k;
            found = true;
        }
    }
    double L = pts[jj + 1] - pts[jj];
    double g = (cs[jj + 1] - cs[jj]) / L;
    double t = (g >= 0 || fabs(g * L) < 1e-10) ? pts[jj] + trexp_offset(uo, g, L) : pts[jj + 1] - trexp_offset(uo, -g, L);
    out[0] = t;
    out[22] = fabs(g * L);
    out[23] = L;
    out[2] = nseg;
    out[3] = jj;
    out[19] = tot;
    out[6] = std::min(u - A[jj], A[jj + 1] - u) / tot;
    double t1 = t;
    if (compensated && t != 0.0 && !jac.empty()) {
        double lj = ljac(t);
        out[7] = lj;
        if (uj >= exp(std::min(0.0, lj))) t1 = 0.0;
    }
    out[1] = t1;
    if (compensated && !jac.empty() && t_other != 0.0) out[9] = ljac(t_other);
    int jo = -1;
    if (t_other == 0.0)
        jo = -2;
    else
        for (int j = 0; j < nseg; ++j)
            if (pts[j] <= t_other && t_other <= pts[j + 1]) {
                jo = j;
                break;
            }
    out[4] = jo;
    if (jo >= 0) out[5] = jo > jj ? (A[jo] - u) / tot : (jo < jj ? (u - A[jo + 1]) / tot : 0.0);
}

int orc_explain(void *p, int64_t sweep, int cls, int mi, int q, int rep, double t_other, double *out) {
    Ctx &c = *(Ctx *)p;
    const Model &m = c.m;
    vector<int> steps;
    class_steps(m.T, cls, steps);
    if (q < 0 || q >= (int)steps.size() || rep < 0 || rep >= c.o.R) return -1;
    int tau = steps[q], T = m.T, taum = (tau - 1 + T) % T;
    TileStream ts0{c.o.seed, 0u, (uint32_t)cls, (uint32_t)sweep};
    vector<MoveRef> moves;
    move_list(c, ts0, moves);
    if (mi < 0 || mi >= (int)moves.size()) return -1;
    TileStream ts = ts0;
    WS ws, wa;
    ws.init(m);
    wa.init(m);
    vector<Kink> jac;
    for (int k = 0; k <= mi; ++k) {
        ws.clear();
        wa.clear();
        ws.tau = tau;
        wa.tau = taum;
        jac.clear();
        if (k < mi) {
            if (moves[k].kind >= 0) prep_family(c, ts, moves[k].kind, ws, wa, rep, &jac);
        }
    }
    const MoveRef &mr = moves[mi];
    for (int i = 0; i < 24; ++i) out[i] = NAN;
    if (mr.kind < 0) {
        int role = m.frole[mr.field];
        int kind = role == ESM_ROLE_THETA ? EK_THETA : (role == ESM_ROLE_GEN ? EK_GEN : EK_SE);
        for (int k = m.ap[mr.atom]; k < m.ap[mr.atom + 1]; ++k) ws.add_entry(kind, m.ai[k], m.av[k]);
    } else if (!prep_family(c, ts, mr.kind, ws, wa, rep, &jac)) {
        return 0;
    }
    finalize_ws(c, ws, rep);
    if (ws.ent.empty()) return 0;
    finalize_ws(c, wa, rep);
    link_soc(m, wa, ws);
    out[16] = mr.kind < 0 ? -1.0 : (double)mr.kind;
    out[17] = (double)(ws.ent.size() + wa.ent.size());
    Mover mv{&c, {&wa, &ws}, rep, m.beta_v, {}};
    double uc, uo, uj, un;
    orc_uniform2(c.o.seed, ESM_TAG_LANE, 2 * (uint32_t)mi, (uint32_t)tau, (uint32_t)rep, (uint32_t)sweep, &uc, &uo);
    orc_uniform2(c.o.seed, ESM_TAG_LANE, 2 * (uint32_t)mi + 1, (uint32_t)tau, (uint32_t)rep, (uint32_t)sweep, &uj,
                 &un);
    bool compensated = mr.kind == ESM_FAM_XLOCC || mr.kind == ESM_FAM_TPOT || mr.kind == ESM_FAM_TSOC;
    explain_mover(c, mv, jac, compensated, uc, uo, uj, t_other, out);
    return 1;
}

// The walk of atom `atom` (index into the model's atoms) at 0-based step tau of replica rep on the
// current state, without committing: the points (ascending, with t = 0) and their potentials into
// pts, cs (up to maxn), and in info[0..3] the points of the right and left walks and the primary
// breakpoints and ray steps the two walks visited. Returns the number of points, -1 when a walk
// reached the point cap or ran out of ray steps. A diagnostic of the walk lengths.
int orc_atom_walk(void *p, int atom, int tau, int rep, double *pts, double *cs, int maxn, int *info) {
    Ctx &c = *(Ctx *)p;
    const Model &m = c.m;
    WS ws, wa;
    ws.init(m);
    wa.init(m);
    ws.tau = tau;
    wa.tau = (tau - 1 + m.T) % m.T;
    int f = 0;
    while (f + 1 < (int)m.fap.size() - 1 && m.fap[f + 1] <= atom) ++f;
    int role = m.frole[f];
    int kind = role == ESM_ROLE_THETA ? EK_THETA : (role == ESM_ROLE_GEN ? EK_GEN : EK_SE);
    for (int q = m.ap[atom]; q < m.ap[atom + 1]; ++q) ws.add_entry(kind, m.ai[q], m.av[q]);
    finalize_ws(c, ws, rep);
    if (ws.ent.empty()) return 0;
    finalize_ws(c, wa, rep);
    link_soc(m, wa, ws);
    Mover mv{&c, {&wa, &ws}, rep, m.beta_v, {}};
    vector<double> right, left;
    for (const WS *w : mv.w)
        for (double x : w->bps) {
            if (!std::isfinite(x)) continue;
            if (x > 0.0)
                right.push_back(x);
            else if (x < 0.0)
                left.push_back(x);
        }
    mv.eval(0.0);
    vector<double> sec0 = mv.sec;
    Walk Wr, Wl;
    Wr.cap = Wl.cap = c.o.max_points > 0 ? c.o.max_points : 4096;
    int okr = walk(Wr, mv, right, 1.0, c.o.maxnats, sec0);
    int okl = walk(Wl, mv, left, -1.0, c.o.maxnats, sec0);
    if (info) {
        info[0] = (int)Wr.pts.size();
        info[1] = (int)Wl.pts.size();
        info[2] = Wr.nprim + Wl.nprim;
        info[3] = Wr.nray + Wl.nray;
    }
    if (!okr || !okl || Wr.full || Wl.full) return -1;
    int n = 0;
    auto put = [&](double x, double cx) {
        if (n < maxn) {
            pts[n] = x;
            cs[n] = cx;
        }
        ++n;
    };
    for (int j = (int)Wl.pts.size() - 1; j >= 0; --j) put(Wl.pts[j], Wl.cs[j]);
    put(0.0, 0.0);
    for (size_t j = 0; j < Wr.pts.size(); ++j) put(Wr.pts[j], Wr.cs[j]);
    return n;
}

// One storage block move of replica rep: the plateau of the storage units us[0..nus) over the
// instants b0+1 .. b0+L (cyclic; prep_storage_ms! / prep_slong!) or, with L = T and one unit, its
// level move; moved by t when commit_it. Outputs as orc_move_at, and with pts/cs (maxn > 0) its
// walk as orc_move_walk (the return is then the number of points, -1 at the point cap). For the
// reference's storage-move checks (test/test_local.jl:227-345).
int orc_block_at(void *p, const int *us, int nus, int b0, int L, int rep, double t, int commit_it, double *lj,
                 double *kq, double *dc, double *pts, double *cs, int maxn) {
    Ctx &c = *(Ctx *)p;
    const Model &m = c.m;
    int T = m.T;
    bool level = L == T;
    int n = level ? T : L + 1;
    vector<WS> wss(n);
    for (auto &w : wss) w.init(m);
    vector<Kink> jac;
    vector<int> uv(us, us + nus);
    *lj = 0.0;
    *dc = 0.0;
    kq[0] = kq[1] = 0.0;
    if (level) {
        if (nus != 1) return 0;
        prep_level(c, wss, uv[0], rep);
    } else if (!prep_plateau(c, wss, b0, L, uv, rep, &jac)) {
        return 0;
    }
    Mover mv{&c, {}, rep, m.beta_v, {}};
    mv.cyclic = level;
    for (auto &w : wss) mv.w.push_back(&w);
    for (auto &k : jac) *lj += k.nm * log(fabs((std::max(k.Q + k.g * t, 0.0) + k.e) / k.Pm));
    if (!jac.empty()) {
        kq[0] = jac[0].Q;
        kq[1] = jac[0].g;
    }
    if (maxn > 0) {
        vector<double> right, left;
        for (const WS *w : mv.w)
            for (double x : w->bps) {
                if (!std::isfinite(x)) continue;
                if (x > 0.0)
                    right.push_back(x);
                else if (x < 0.0)
                    left.push_back(x);
            }
        mv.eval(0.0);
        vector<double> sec0 = mv.sec;
        Walk Wr, Wl;
        Wr.cap = Wl.cap = c.o.max_points > 0 ? c.o.max_points : 4096;
        if (!walk(Wr, mv, right, 1.0, c.o.maxnats, sec0) || Wr.full) return -1;
        if (!walk(Wl, mv, left, -1.0, c.o.maxnats, sec0) || Wl.full) return -1;
        int k = 0;
        auto put = [&](double x, double cx) {
            if (k < maxn) {
                pts[k] = x;
                cs[k] = cx;
            }
            ++k;
        };
        for (int j = (int)Wl.pts.size() - 1; j >= 0; --j) put(Wl.pts[j], Wl.cs[j]);
        put(0.0, 0.0);
        for (size_t j = 0; j < Wr.pts.size(); ++j) put(Wr.pts[j], Wr.cs[j]);
        return k;
    }
    *dc = mv.eval(t);
    if (commit_it) commit(c, mv, t);
    return 1;
}

void orc_class_order(void *p, int64_t sweep, int *order, int *ncls) {
    class_order(*(Ctx *)p, (uint32_t)sweep, order, ncls);
}

void orc_scores(void *p, double *sk, double *fk, double *parts, int nthreads) {
    Ctx *c = (Ctx *)p;
    c->sk_last.assign((size_t)c->o.R * c->m.K, 0.0);
    c->fk_last.assign(c->m.K, 0.0);
    scores(*c, c->sk_last.data(), c->fk_last.data(), parts, nthreads);
    c->has_scores = true;
    if (sk) std::copy(c->sk_last.begin(), c->sk_last.end(), sk);
    if (fk) std::copy(c->fk_last.begin(), c->fk_last.end(), fk);
}

int orc_langevin_step(void *p, const double *w, const double *eta, const double *kappa_s, double kmin, double clip,
                      int box, const double *xi, int64_t it, double *knew_out, int *nclip_out, int nthreads) {
    if (!((Ctx *)p)->has_scores) return -5;
    langevin_step(*(Ctx *)p, w, eta, kappa_s, kmin, clip, box, xi, it, knew_out, nclip_out, nthreads);
    ((Ctx *)p)->has_scores = false;
    return 0;
}

void orc_weather_step(void *p, const int32_t *moved, const double *theta, const int32_t *window,
                      const int32_t *wstart, const double *xi, int64_t it, int nthreads) {
    weather_step(*(Ctx *)p, moved, theta, window, wstart, xi, it, nthreads);
}

}  // extern "C"
