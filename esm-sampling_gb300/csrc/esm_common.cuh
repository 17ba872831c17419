// Shared device definitions of libesmcuda: Philox streams, the device model, cost pieces.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/esmcuda.h"

// TAG_SWEEP (0, 0, 0, sweep) class order; TAG_LIST (j/2, tile, class, sweep) move list and selection;
// TAG_LANE (2 move + h, step, replica, sweep) a line move's uniforms; TAG_LGV (j/2, group, it, 0)
// Langevin normals; TAG_WTH (j/2, t, replica, it) weather; TAG_SMS / TAG_SML the storage multiscale
// sweep's plan and block uniforms; TAG_SLG / TAG_SLL the long-range storage sweep's plan and uniforms
#define ESM_TAG_SWEEP 0x53574550u
#define ESM_TAG_LIST 0x4C495354u
#define ESM_TAG_LANE 0x4C414E45u
#define ESM_TAG_LGV 0x4C475600u
#define ESM_TAG_WTH 0x57544800u
#define ESM_TAG_SMS 0x534D5300u
#define ESM_TAG_SML 0x534D4C00u
#define ESM_TAG_SLG 0x534C4700u
#define ESM_TAG_SLL 0x534C4C00u

namespace esm {

// ---------------------------------------------------------------------------------------------
// Philox4x32-10 (Salmon et al., SC11); key (seed low word, seed high word ^ tag), one call per
// counter (w0, w1, w2, w3) gives two 53-bit uniforms; the tags and counter words of every stream
// are listed with the ESM_TAG_* constants below
// ---------------------------------------------------------------------------------------------
__host__ __device__ inline void philox(uint32_t k0, uint32_t k1, uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3,
                                       uint32_t out[4]) {
#pragma unroll
    for (int r = 0; r < 10; ++r) {
#ifdef __CUDA_ARCH__
        uint32_t lo0 = 0xD2511F53u * c0, hi0 = __umulhi(0xD2511F53u, c0);
        uint32_t lo1 = 0xCD9E8D57u * c2, hi1 = __umulhi(0xCD9E8D57u, c2);
#else
        uint64_t p0 = (uint64_t)0xD2511F53u * c0, p1 = (uint64_t)0xCD9E8D57u * c2;
        uint32_t lo0 = (uint32_t)p0, hi0 = (uint32_t)(p0 >> 32), lo1 = (uint32_t)p1, hi1 = (uint32_t)(p1 >> 32);
#endif
        uint32_t n0 = hi1 ^ c1 ^ k0, n2 = hi0 ^ c3 ^ k1;
        c0 = n0;
        c1 = lo1;
        c2 = n2;
        c3 = lo0;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    out[0] = c0;
    out[1] = c1;
    out[2] = c2;
    out[3] = c3;
}

__host__ __device__ inline double u53(uint32_t a, uint32_t b) {
    return ((double)(a >> 5) * 67108864.0 + (double)(b >> 6)) * (1.0 / 9007199254740992.0);
}

__host__ __device__ inline void uniform2(uint64_t seed, uint32_t tag, uint32_t c0, uint32_t c1, uint32_t c2,
                                         uint32_t c3, double *u0, double *u1) {
    uint32_t x[4];
    philox((uint32_t)seed, (uint32_t)(seed >> 32) ^ tag, c0, c1, c2, c3, x);
    *u0 = u53(x[0], x[1]);
    *u1 = u53(x[2], x[3]);
}

// The order of the colour classes in a sweep (local_sweep!, src/local.jl:1934: the parity
// classes in random order, three of them when T is odd): order[0..ncls) from the sweep's stream.
__host__ __device__ inline void class_order_of(uint64_t seed, int T, uint32_t sweep, int order[3], int *ncls) {
    double u0, u1;
    uniform2(seed, ESM_TAG_SWEEP, 0, 0, 0, sweep, &u0, &u1);
    if (T % 2 == 0) {
        *ncls = 2;
        order[0] = u0 < 0.5 ? 0 : 1;
        order[1] = 1 - order[0];
        order[2] = 2;
    } else {
        *ncls = 3;
        order[0] = 0;
        order[1] = 1;
        order[2] = 2;
        int j = (int)floor(u0 * 3);
        j = j < 2 ? j : 2;
        int x = order[2];
        order[2] = order[j];
        order[j] = x;
        j = (int)floor(u1 * 2);
        j = j < 1 ? j : 1;
        x = order[1];
        order[1] = order[j];
        order[j] = x;
    }
}

__host__ __device__ inline double normal_at(uint64_t seed, uint32_t tag, uint32_t j, uint32_t c1, uint32_t c2,
                                            uint32_t c3) {
    double u0, u1;
    uniform2(seed, tag, j >> 1, c1, c2, c3, &u0, &u1);
    double rr = sqrt(-2.0 * log(1.0 - u0));
    double a = 6.283185307179586 * u1;
    return (j & 1) ? rr * sin(a) : rr * cos(a);
}

// A uniform of [0, 1) in the working precision. The 53-bit uniforms round up to 1 in FP32 when they
// lie within 2^-25 of it (3e-8 of the draws), and u = 1 is outside the domain of the inverse-CDF
// maps: the truncated exponential of a steep segment, -log1p(-u (1 - e^-gL)) / g, is infinite at
// u = 1 once 1 - e^-gL rounds to 1. Such a draw is taken to the largest value below 1 instead.
template <class real>
__host__ __device__ inline real unit_uniform(double u) {
    real v = (real)u;
    if constexpr (sizeof(real) == 4)
        return v < 1.0f ? v : 0.99999994f;
    return v;
}

template <class real>
__host__ __device__ inline real clampr(real x, real lo, real hi) {
    return x < lo ? lo : (x > hi ? hi : x);
}

// ---------------------------------------------------------------------------------------------
// device model: static tables and the state of one chain (R replicas), (X, T, R) layouts
// ---------------------------------------------------------------------------------------------
template <class real>
struct DevModel {
    int N, L, T, R, K, D, S, n0, nreg, nfields, nlev, natoms, nextra, span, maxpts;
    int maxe, maxl, maxn, maxk, maxku, maxstu;   // descriptor capacities per move
    real dt, c_shed, c_dump, c_viol, kappa0, beta_v, maxnats, kmin;
    uint64_t seed;
    double cumw[ESM_NFAM];   // family and cell-level draws compare in FP64 in both precisions
    // network
    const int *bus0, *bus1;
    const real *lb, *ls;
    const int *nlp, *nl;
    const int *comp, *theta_nnz;
    const real *Z;
    // dispatchable units (index j in 0..D-1) and storage units (0..S-1)
    const int *d_bus, *d_group;
    const real *d_avail, *d_mc;
    const real *kc_d;                 // clamped capacities of the dispatchable units
    const int *s_bus;
    const real *s_hours, *s_etain, *s_etaout, *s_qt, *s_mc;
    const real *kc_s;
    // move tables
    const int *frole, *fap, *ap, *ai;
    const real *av;
    const int *up, *ua, *sp, *sa;
    const double *qcum;
    const int *clp, *cp, *cu;
    const int *xpp, *xp, *xnp, *xn, *xlp, *xln;
    const real *xv, *xlg;
    // renewable units (0..Nren-1) and the weather
    int Nren;
    const int *r_bus, *r_series;
    const real *r_mc, *kc_r;
    const real *xbar, *wscale;   // [n0*T], [n0]; load of node n is series n
    // flat units (0..K-1): kind, index within its kind, and the units of every node (CSR)
    const int *u_kind, *u_loc;
    const int *nu_ptr, *nu_unit;
    // lines by their first bus (CSR), for node-parallel passes
    const int *lb0_ptr, *lb0_line;
    // state
    real *theta, *g, *e, *r, *F, *z;
    // move log (diagnostics, NULL: off): the t every line move of a class pass took for replicas
    // below mlog_nrep, at [(move * nsteps + q) * mlog_nrep + replica] for the class's q-th step
    double *mlog;
    int mlog_nrep;
};

__host__ __device__ inline size_t sidx(int x, int t, int rep, int T, int R) { return ((size_t)x * T + t) * R + rep; }

// cost pieces (src/local.jl:760 gen_cost, src/energy.jl:448 soc_cost, src/local.jl:773 phibal)
template <class real>
__device__ inline real gen_cost(real mc, real A, real k, real w, real dt, real cv, real y, real *p) {
    real yc = clampr<real>(y, 0, 1);
    *p = A * k * yc;
    return dt * mc * (*p) + cv * dt * w * fabs(y - yc);
}

template <class real>
__device__ inline real soc_cost(real h, real qt, real etain, real etaout, real mc, real k, real w, real dt, real cv,
                                real ye, real ye1, real *dout, real *jout) {
    real ec = clampr<real>(ye, 0, 1), ec1 = clampr<real>(ye1, 0, 1);
    real d = h * (ec1 - ec) / dt - qt;
    real pc, mcx;
    if (d >= 0) {
        pc = etain > 0 ? d / etain : real(0);
        mcx = 0;
    } else {
        pc = 0;
        mcx = fmin(-d * etaout, real(1));
    }
    real c = dt * mc * k * (pc + mcx) + cv * w * h * fabs(ye - ec);
    if (pc > 1) c += cv * dt * w * (pc - 1);
    if (d < 0 && qt <= 0) {
        real ex = -d * etaout - real(1);
        if (ex > 0) c += cv * dt * w * ex;
    }
    if (d >= 0 && etain <= 0) c += cv * dt * w * d;
    *dout = d;
    *jout = k * (pc - mcx);
    return c;
}

template <class real>
__device__ inline real phibal(real x, real cs, real cd) {
    return x > 0 ? cs * x : -cd * x;
}

// ---------------------------------------------------------------------------------------------
// Difference forms of the cost pieces. A line move changes each term by a small amount on top of
// a large value (a generator cost of 1e8 EUR changes by 1e2); the reference evaluates c(t) - c(0),
// which in FP32 leaves ~10 EUR of rounding, i.e. 1e-3 nats of noise on the line potential. These
// forms compute the change itself from the move's increments, exactly where the term stays on one
// linear piece and by the plain difference only across a kink (where both values are small).
// ---------------------------------------------------------------------------------------------

// change of cl(y) = clamp(y, 0, 1) and of the box excess |y - cl(y)| when y0 moves by dy
template <class real>
__device__ inline void clamp_diff(real y0, real dy, real *dyc, real *dex) {
    real y1 = y0 + dy;
    if (y0 > 0 && y0 < 1 && y1 > 0 && y1 < 1) {
        *dyc = dy;
        *dex = 0;
    } else if (y0 >= 1 && y1 >= 1) {
        *dyc = 0;
        *dex = dy;
    } else if (y0 <= 0 && y1 <= 0) {
        *dyc = 0;
        *dex = -dy;
    } else {
        real c0 = clampr<real>(y0, 0, 1), c1 = clampr<real>(y1, 0, 1);
        *dyc = c1 - c0;
        *dex = fabs(y1 - c1) - fabs(y0 - c0);
    }
}

// change of max(|f| - s, 0) when f0 moves by df
template <class real>
__device__ inline real hinge_diff(real f0, real df, real s) {
    real f1 = f0 + df;
    if (fabs(f0) <= s && fabs(f1) <= s) return 0;
    if (f0 > s && f1 > s) return df;
    if (f0 < -s && f1 < -s) return -df;
    return fmax(fabs(f1) - s, real(0)) - fmax(fabs(f0) - s, real(0));
}

// change of phibal(S) when S0 moves by dS
template <class real>
__device__ inline real phibal_diff(real S0, real dS, real cs, real cd) {
    real S1 = S0 + dS;
    if (S0 > 0 && S1 > 0) return cs * dS;
    if (S0 < 0 && S1 < 0) return -cd * dS;
    return phibal<real>(S1, cs, cd) - phibal<real>(S0, cs, cd);
}

// state-of-charge storage term (src/energy.jl:448 soc_cost) as functions of d: the injection per
// unit capacity pc - mc, the running part pc + mc and the penalty part (charging beyond the
// rating, discharging beyond it without inflow, charging a unit that cannot charge)
template <class real>
__device__ inline void soc_parts(real d, real etain, real etaout, real qt, real *inj, real *run, real *pen) {
    if (d >= 0) {
        real pc = etain > 0 ? d / etain : real(0);
        *inj = pc;
        *run = pc;
        *pen = (pc > 1 ? pc - 1 : real(0)) + (etain <= 0 ? d : real(0));
    } else {
        real x = -d * etaout;
        real mc = fmin(x, real(1));
        *inj = -mc;
        *run = mc;
        *pen = (qt <= 0 && x - 1 > 0) ? x - 1 : real(0);
    }
}

template <class real>
__device__ inline int soc_piece(real d, real etain, real etaout) {
    if (d >= 0) return (etain > 0 && d / etain > 1) ? 1 : 0;
    return (-d * etaout >= 1) ? 3 : 2;
}

// change of the storage term when the start value ye moves by a and the end value ye1 by b.
// Returns the cost change; *dj the injection change, *d1 the new d.
template <class real>
__device__ inline real soc_diff(real h, real qt, real etain, real etaout, real mc, real k, real w, real dt, real cv,
                                real ye, real ye1, real a, real b, real *dj, real *d1) {
    real dc0, dex0, dc1, dex1;
    clamp_diff<real>(ye, a, &dc0, &dex0);
    clamp_diff<real>(ye1, b, &dc1, &dex1);
    real ec = clampr<real>(ye, 0, 1), ec1 = clampr<real>(ye1, 0, 1);
    real d0 = h * (ec1 - ec) / dt - qt;
    real dd = h * (dc1 - dc0) / dt;
    real dn = d0 + dd;
    real dinj, drun, dpen;
    int p0 = soc_piece<real>(d0, etain, etaout), p1 = soc_piece<real>(dn, etain, etaout);
    if (p0 == p1) {
        real si, sr, sp;
        if (p0 == 0) {
            si = etain > 0 ? real(1) / etain : real(0);
            sr = si;
            sp = etain <= 0 ? real(1) : real(0);
        } else if (p0 == 1) {
            si = real(1) / etain;
            sr = si;
            sp = si;
        } else if (p0 == 2) {
            si = etaout;
            sr = -etaout;
            sp = 0;
        } else {
            si = 0;
            sr = 0;
            sp = qt <= 0 ? -etaout : real(0);
        }
        dinj = si * dd;
        drun = sr * dd;
        dpen = sp * dd;
    } else {
        real i0, r0, q0, i1, r1, q1;
        soc_parts<real>(d0, etain, etaout, qt, &i0, &r0, &q0);
        soc_parts<real>(dn, etain, etaout, qt, &i1, &r1, &q1);
        dinj = i1 - i0;
        drun = r1 - r0;
        dpen = q1 - q0;
    }
    *dj = k * dinj;
    *d1 = dn;
    return dt * mc * k * drun + cv * dt * w * dpen + cv * w * h * dex0;
}

}  // namespace esm
