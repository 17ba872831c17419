// HBM-bound node-parallel passes of the replica step: cache rebuild, energy and capacity score,
// Langevin step, dispatch following. One thread per (node, step, replica) or (node, step-chunk,
// replica), the replica index fastest so that every load is coalesced over a warp.
#pragma once
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "esm_common.cuh"

namespace esm {

template <class real>
__device__ inline real wraw(const DevModel<real> &M, int s, int t, int rep) {
    return M.xbar[(size_t)s * M.T + t] + M.wscale[s] * M.z[sidx(s, t, rep, M.T, M.R)];
}
template <class real>
__device__ inline real avail_map(real x) {  // logistic availability map (builder decision of the synthetic model)
    return real(1) / (real(1) + exp(-x));
}

// ---------------------------------------------------------------------------------------------
// LocalCost rebuild (src/local.jl:313, rebuild_step! :332): residual per node, flows per line.
// Accumulation order per node as the reference: load, lines, generators, storage.
// ---------------------------------------------------------------------------------------------
template <class real>
__global__ void k_rebuild(DevModel<real> M) {
    size_t TR = (size_t)M.T * M.R;
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (size_t)M.N * TR) return;
    int n = (int)(i / TR);
    size_t tr = i % TR;
    int t = (int)(tr / M.R), rep = (int)(tr % M.R);
    int T = M.T, R = M.R;
    real x = wraw(M, n, t, rep);
    real r = x > 0 ? x : real(0);
    for (int p = M.nlp[n]; p < M.nlp[n + 1]; ++p) {
        int e = M.nl[p];
        int a = M.bus0[e], b = M.bus1[e];
        real fl = M.lb[e] * (M.theta[sidx(a, t, rep, T, R)] - M.theta[sidx(b, t, rep, T, R)]);
        if (a == n) {
            M.F[sidx(e, t, rep, T, R)] = fl;
            r += fl + real(0.5) * real(0);
        } else {
            r += -fl + real(0.5) * real(0);
        }
    }
    for (int p = M.nu_ptr[n]; p < M.nu_ptr[n + 1]; ++p) {
        int u = M.nu_unit[p], j = M.u_loc[u];
        int kd = M.u_kind[u];
        if (kd == ESM_UNIT_REN) {
            real A = avail_map<real>(wraw(M, M.r_series[j], t, rep));
            r -= A * M.kc_r[j] * real(1);
        } else if (kd == ESM_UNIT_DISP) {
            real y = clampr<real>(M.g[sidx(j, t, rep, T, R)], 0, 1);
            r -= M.d_avail[j] * M.kc_d[j] * y;
        }
    }
    for (int p = M.nu_ptr[n]; p < M.nu_ptr[n + 1]; ++p) {
        int u = M.nu_unit[p], j = M.u_loc[u];
        if (M.u_kind[u] != ESM_UNIT_STOR) continue;
        real ec = clampr<real>(M.e[sidx(j, t, rep, T, R)], 0, 1);
        real ec1 = clampr<real>(M.e[sidx(j, (t + 1) % T, rep, T, R)], 0, 1);
        real d = M.s_hours[j] * (ec1 - ec) / M.dt - M.s_qt[j];
        real pc, mcx;
        if (d >= 0) {
            pc = M.s_etain[j] > 0 ? d / M.s_etain[j] : real(0);
            mcx = 0;
        } else {
            pc = 0;
            mcx = fmin(-d * M.s_etaout[j], real(1));
        }
        r += M.kc_s[j] * (pc - mcx);
    }
    M.r[i] = r;
}

// ---------------------------------------------------------------------------------------------
// Energy cost and capacity gradient (src/energy.jl:551-757: gen_grad :835, soc_grad :466) in one
// pass over the state: the residual of every (node, step) and the flows of its lines by the
// rebuild's arithmetic (k_rebuild, in its order), then the cost and gradient terms of the node's
// units, so no cache is read. Thread (replica lane, node slot) of block (replica tile, node group of
// ESM_SCORE_NSLOT nodes, step chunk) sums its node's terms over the chunk's steps. Every (chunk,
// replica, unit) partial of the gradient has one writer (the thread of the unit's node); the cost
// parts are summed over the block's node slots in slot order, and k_score_reduce sums the chunks in
// chunk order: the scores are the same from run to run, bit for bit.
// Two builds of the pass:
//   k_scores_fused<S>  every term in FP64 from the state S (the FP64 parity state);
//   k_scores_f32       the FP32 production build: FP32 state and parameters, terms in FP32, summed
//                      with Neumaier's compensated summation. The one discontinuity of the terms is
//                      the sign of a node balance (shed or dump price); where the FP32 balance lies
//                      within its rounding bound of 0 the sign is taken from the FP64 balance, so
//                      every term is the FP64 term's continuous function of FP32-rounded inputs.
// Each output carries a bound on its distance from the exact value of the same sums over the same
// state (running error analysis: every term's rounding bound, in units of its precision's epsilon,
// summed beside the term; then the summation's own).
//   partial: [values | bounds], each nchunk x (R*K gradient | ngroups*R*5 cost parts: gen, storage,
//   shed, dump, penalty); sums: [dk R*K | parts R*8 | dk bounds R*K | parts bounds R*8]
// ---------------------------------------------------------------------------------------------
#define ESM_SCORE_NSLOT 8
#define ESM_SCORE_MAXU 8
#define ESM_U64 1.1102230246251565e-16  // 2^-53
#define ESM_U32 5.9604645e-8f           // 2^-24

// Neumaier's compensated summation (Neumaier 1974): the running FP32 sum and the rounding error
// that its additions dropped
struct NSum {
    float s = 0.f, c = 0.f;
    __device__ inline void add(float x) {
        float t = s + x;
        c += fabsf(s) >= fabsf(x) ? (s - t) + x : (x - t) + s;
        s = t;
    }
    __device__ inline double value() const { return (double)s + (double)c; }
};

// the FP64 residual of node n at step t from the state S (k_rebuild's order: load, lines,
// generation, storage); *pen, when given, gains the overload penalty of the lines leaving n
template <class S>
__device__ inline double node_residual64(const DevModel<double> &M, const S *theta, const S *gv, const S *ev,
                                         const S *zv, int n, int t, int rep, double *pen) {
    int T = M.T, R = M.R;
    double dt = M.dt, cv = M.c_viol;
    auto wr = [&](int s_) { return M.xbar[(size_t)s_ * T + t] + M.wscale[s_] * (double)zv[sidx(s_, t, rep, T, R)]; };
    double x = wr(n);
    double rr = x > 0 ? x : 0.0;
    for (int p = M.nlp[n]; p < M.nlp[n + 1]; ++p) {
        int e = M.nl[p];
        int a = M.bus0[e], b = M.bus1[e];
        double fl = M.lb[e] * ((double)theta[sidx(a, t, rep, T, R)] - (double)theta[sidx(b, t, rep, T, R)]);
        if (a == n) {
            rr += fl + 0.5 * 0.0;
            if (pen) *pen += cv * dt * (M.ls[e] * fmax(fabs(fl) / M.ls[e] - 1.0, 0.0));
        } else {
            rr += -fl + 0.5 * 0.0;
        }
    }
    for (int p = M.nu_ptr[n]; p < M.nu_ptr[n + 1]; ++p) {
        int u = M.nu_unit[p], j = M.u_loc[u];
        int kd = M.u_kind[u];
        if (kd == ESM_UNIT_REN)
            rr -= avail_map<double>(wr(M.r_series[j])) * M.kc_r[j] * 1.0;
        else if (kd == ESM_UNIT_DISP)
            rr -= M.d_avail[j] * M.kc_d[j] * clampr<double>((double)gv[sidx(j, t, rep, T, R)], 0, 1);
    }
    for (int p = M.nu_ptr[n]; p < M.nu_ptr[n + 1]; ++p) {
        int u = M.nu_unit[p], j = M.u_loc[u];
        if (M.u_kind[u] != ESM_UNIT_STOR) continue;
        double ec = clampr<double>((double)ev[sidx(j, t, rep, T, R)], 0, 1);
        double ec1 = clampr<double>((double)ev[sidx(j, (t + 1) % T, rep, T, R)], 0, 1);
        double d = M.s_hours[j] * (ec1 - ec) / M.dt - M.s_qt[j];
        double pc, mcx;
        if (d >= 0) {
            pc = M.s_etain[j] > 0 ? d / M.s_etain[j] : 0.0;
            mcx = 0;
        } else {
            pc = 0;
            mcx = fmin(-d * M.s_etaout[j], 1.0);
        }
        rr += M.kc_s[j] * (pc - mcx);
    }
    return rr;
}

template <class S>
__global__ void __launch_bounds__(32 * ESM_SCORE_NSLOT)
    k_scores_fused(const __grid_constant__ DevModel<double> M, const S *theta, const S *gv, const S *ev, const S *zv,
                   int tchunk, double *partial) {
    __shared__ double sp[ESM_SCORE_NSLOT][32][10];
    int lane = threadIdx.x, slot = threadIdx.y;
    int rep = blockIdx.x * 32 + lane;
    int n = blockIdx.y * ESM_SCORE_NSLOT + slot;
    int c = blockIdx.z, nchunk = gridDim.z, ng = gridDim.y;
    int T = M.T, R = M.R, K = M.K;
    size_t nrk = (size_t)R * K, half = (size_t)nchunk * (nrk + (size_t)ng * R * 5);
    double part[5] = {0, 0, 0, 0, 0};  // gen, storage, shed, dump, penalty
    double pmag[5] = {0, 0, 0, 0, 0};  // the sums of their terms' magnitudes
    if (rep < R && n < M.N) {
        int t0 = c * tchunk, t1 = min(T, t0 + tchunk);
        double dt = M.dt, cv = M.c_viol, k0 = M.kappa0;
        const int MAXU = ESM_SCORE_MAXU;
        double dk[MAXU], dkbox[MAXU], dmag[MAXU];
        int nu = M.nu_ptr[n + 1] - M.nu_ptr[n];
        for (int q = 0; q < MAXU; ++q) dk[q] = dkbox[q] = dmag[q] = 0;
        auto wr = [&](int s_, int t) {
            return M.xbar[(size_t)s_ * T + t] + M.wscale[s_] * (double)zv[sidx(s_, t, rep, T, R)];
        };
        for (int t = t0; t < t1; ++t) {
            double p4 = part[4];
            double rr = node_residual64<S>(M, theta, gv, ev, zv, n, t, rep, &part[4]);
            pmag[4] += part[4] - p4;  // (the line penalties are not negative)
            // the terms of the cost and of its gradient
            double Gn = dt * (rr > 0 ? M.c_shed : (rr < 0 ? -M.c_dump : 0.0));
            if (rr > 0)
                part[2] += dt * rr;
            else
                part[3] -= dt * rr;
            pmag[rr > 0 ? 2 : 3] += fabs(dt * rr);
            for (int q = 0; q < nu && q < MAXU; ++q) {
                int u = M.nu_unit[M.nu_ptr[n] + q], j = M.u_loc[u];
                int kd = M.u_kind[u];
                if (kd == ESM_UNIT_REN) {
                    double A = avail_map<double>(wr(M.r_series[j], t));
                    double g0 = dt * (M.r_mc[j] * (A * M.kc_r[j] * 1.0));
                    part[0] += g0;
                    pmag[0] += fabs(g0);
                    double a1 = dt * (M.r_mc[j] * A * 1.0), a2 = A * 1.0 * Gn;
                    dk[q] += a1 - a2;
                    dmag[q] += fabs(a1) + fabs(a2);
                } else if (kd == ESM_UNIT_DISP) {
                    double A = M.d_avail[j], kv = M.kc_d[j];
                    double Y = (double)gv[sidx(j, t, rep, T, R)];
                    double Yc = clampr<double>(Y, 0, 1);
                    double g0 = dt * (M.d_mc[j] * (A * kv * Yc));
                    part[0] += g0;
                    pmag[0] += fabs(g0);
                    double exs = fabs(Y - Yc);
                    if (exs > 0) {
                        part[4] += cv * dt * (kv + k0) * exs;
                        pmag[4] += cv * dt * (kv + k0) * exs;
                    }
                    if (!(0.0 < Y && Y < 1.0)) {
                        dk[q] += cv * dt * fabs(Y - Yc);
                        dmag[q] += cv * dt * fabs(Y - Yc);
                    }
                    double a1 = dt * (M.d_mc[j] * A * Yc), a2 = A * Yc * Gn;
                    dk[q] += a1 - a2;
                    dmag[q] += fabs(a1) + fabs(a2);
                } else {
                    double kv = M.kc_s[j], h = M.s_hours[j];
                    double ye = (double)ev[sidx(j, t, rep, T, R)], ye1 = (double)ev[sidx(j, (t + 1) % T, rep, T, R)];
                    double dd, jj;
                    double cc = soc_cost<double>(h, M.s_qt[j], M.s_etain[j], M.s_etaout[j], M.s_mc[j], kv, kv + k0, dt,
                                                 cv, ye, ye1, &dd, &jj);
                    double Ec = clampr<double>(ye, 0, 1), Ec1 = clampr<double>(ye1, 0, 1);
                    double d = h * (Ec1 - Ec) / dt - M.s_qt[j];
                    double pc, mcx;
                    if (d >= 0) {
                        pc = M.s_etain[j] > 0 ? d / M.s_etain[j] : 0.0;
                        mcx = 0;
                    } else {
                        pc = 0;
                        mcx = fmin(-d * M.s_etaout[j], 1.0);
                    }
                    double run = dt * M.s_mc[j] * kv * (pc + mcx);
                    part[1] += run;
                    part[4] += cc - run;
                    // d's rounding (its cancellation) times the slopes in d
                    double sd = fmax(fmax(M.s_etain[j] > 0 ? 1.0 / M.s_etain[j] : 0.0, M.s_etaout[j]), 1.0);
                    double bd = 4.0 * fabs(h * (Ec1 - Ec) / dt) + fabs(M.s_qt[j]) + 4.0 * fabs(d);
                    pmag[1] += fabs(run) + dt * M.s_mc[j] * kv * sd * bd;
                    pmag[4] += fabs(cc) + fabs(run) + dt * (M.s_mc[j] * kv + 2.0 * cv * (kv + k0)) * sd * bd;
                    double a;
                    if (d >= 0 && M.s_etain[j] <= 0) {  // soc_grad (src/energy.jl:470-491)
                        a = cv * dt * d;
                    } else if (d >= 0) {
                        double pcc = d / M.s_etain[j];
                        a = dt * M.s_mc[j] * pcc + Gn * pcc + (pcc > 1 ? cv * dt * (pcc - 1) : 0.0);
                    } else {
                        double mc_ = -d * M.s_etaout[j];
                        double mcc = fmin(mc_, 1.0);
                        a = dt * M.s_mc[j] * mcc - Gn * mcc + ((mc_ > 1 && M.s_qt[j] <= 0) ? cv * dt * (mc_ - 1) : 0.0);
                    }
                    dk[q] += a;
                    dmag[q] += fabs(a) + fabs(Gn) * (pc + mcx) + (dt * M.s_mc[j] + fabs(Gn) + cv * dt) * sd * bd;
                    if (!(0.0 < ye && ye < 1.0)) dkbox[q] += cv * h * fabs(ye - Ec);
                    dmag[q] += cv * h * fabs(ye - Ec);
                }
            }
        }
        double sc = (double)(t1 - t0 + 16) * ESM_U64;
        for (int q = 0; q < nu && q < MAXU; ++q) {
            int u = M.nu_unit[M.nu_ptr[n] + q];
            partial[((size_t)c * R + rep) * K + u] = dk[q] + dkbox[q];
            partial[half + ((size_t)c * R + rep) * K + u] = sc * dmag[q];
        }
        for (int i = 0; i < 5; ++i) pmag[i] *= sc;
    }
    for (int i = 0; i < 5; ++i) {
        sp[slot][lane][i] = part[i];
        sp[slot][lane][5 + i] = pmag[i];
    }
    __syncthreads();
    if (slot == 0 && rep < R) {
        double acc[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
        for (int s2 = 0; s2 < ESM_SCORE_NSLOT; ++s2)
            for (int i = 0; i < 10; ++i) acc[i] += sp[s2][lane][i];
        size_t o = (size_t)nchunk * nrk + (((size_t)c * ng + blockIdx.y) * R + rep) * 5;
        for (int i = 0; i < 5; ++i) {
            partial[o + i] = acc[i];
            partial[half + o + i] = acc[5 + i] + 8.0 * ESM_U64 * fabs(acc[i]);
        }
    }
}

// The FP32 build of the pass (see above). Bounds are summed in units of 2^-24 beside the terms:
// a product or quotient of rounded inputs contributes a few units of its magnitude; the logistic
// availability contributes its weather value's rounding (the sum of the magnitudes of its two
// parts) on top; a storage term contributes the rounding of its flow d (4|Q| + |qt| + 2|d|, Q the
// energy change per hour) times its slope in d.
static __global__ void __launch_bounds__(32 * ESM_SCORE_NSLOT)
    k_scores_f32(const __grid_constant__ DevModel<float> M, const __grid_constant__ DevModel<double> Md, int tchunk,
                 double *partial) {
    __shared__ double sp[ESM_SCORE_NSLOT][32][10];
    int lane = threadIdx.x, slot = threadIdx.y;
    int rep = blockIdx.x * 32 + lane;
    int n = blockIdx.y * ESM_SCORE_NSLOT + slot;
    int c = blockIdx.z, nchunk = gridDim.z, ng = gridDim.y;
    int T = M.T, R = M.R, K = M.K;
    size_t nrk = (size_t)R * K, half = (size_t)nchunk * (nrk + (size_t)ng * R * 5);
    NSum part[5];
    float pe[5] = {0, 0, 0, 0, 0};
    if (rep < R && n < M.N) {
        int t0 = c * tchunk, t1 = min(T, t0 + tchunk);
        const float dt = M.dt, cv = M.c_viol, k0 = M.kappa0, csh = M.c_shed, cdu = M.c_dump;
        const float *th = M.theta, *gv = M.g, *ev = M.e, *zv = M.z;
        int p0 = M.nu_ptr[n], p1 = M.nu_ptr[n + 1];
        int nu = min(p1 - p0, ESM_SCORE_MAXU);
        NSum dk[ESM_SCORE_MAXU];
        float de[ESM_SCORE_MAXU];
#pragma unroll
        for (int q = 0; q < ESM_SCORE_MAXU; ++q) de[q] = 0;
        for (int t = t0; t < t1; ++t) {
            // the weather value of series s and its rounding bound
            auto wr = [&](int s_, float *b) {
                float xb = M.xbar[(size_t)s_ * T + t], wz = M.wscale[s_] * zv[sidx(s_, t, rep, T, R)];
                *b = 2.f * (fabsf(xb) + fabsf(wz));
                return xb + wz;
            };
            // the residual, with the sum of its terms' magnitudes (ab) and their rounding bounds (br)
            float bx;
            float x = wr(n, &bx);
            float rr = x > 0 ? x : 0.f;
            float ab = rr, br = bx;
            int nt = 1;
            for (int p = M.nlp[n]; p < M.nlp[n + 1]; ++p) {
                int e = M.nl[p];
                int a = M.bus0[e], b = M.bus1[e];
                float fl = M.lb[e] * (th[sidx(a, t, rep, T, R)] - th[sidx(b, t, rep, T, R)]);
                float afl = fabsf(fl);
                ab += afl;
                br += 2.f * afl;
                ++nt;
                if (a == n) {
                    rr += fl;
                    float ls = M.ls[e];
                    float pen = cv * dt * (ls * fmaxf(afl / ls - 1.f, 0.f));
                    part[4].add(pen);
                    pe[4] += 6.f * pen + (afl >= 0.999f * ls ? 3.f * cv * dt * afl : 0.f);
                } else {
                    rr -= fl;
                }
            }
            for (int p = p0; p < p1; ++p) {
                int u = M.nu_unit[p], j = M.u_loc[u];
                int kd = M.u_kind[u];
                float v = 0, bv = 0;
                if (kd == ESM_UNIT_REN) {
                    float bs;
                    v = -(avail_map<float>(wr(M.r_series[j], &bs)) * M.kc_r[j]);
                    bv = (8.f + bs) * fabsf(v);
                } else if (kd == ESM_UNIT_DISP) {
                    v = -(M.d_avail[j] * M.kc_d[j] * clampr<float>(gv[sidx(j, t, rep, T, R)], 0, 1));
                    bv = 4.f * fabsf(v);
                } else {
                    float ec = clampr<float>(ev[sidx(j, t, rep, T, R)], 0, 1);
                    float ec1 = clampr<float>(ev[sidx(j, (t + 1) % T, rep, T, R)], 0, 1);
                    float Q = M.s_hours[j] * (ec1 - ec) / dt, d = Q - M.s_qt[j];
                    float ein = M.s_etain[j], eout = M.s_etaout[j];
                    float pc = 0, mcx = 0;
                    if (d >= 0)
                        pc = ein > 0 ? d / ein : 0.f;
                    else
                        mcx = fminf(-d * eout, 1.f);
                    v = M.kc_s[j] * (pc - mcx);
                    float sd = fmaxf(ein > 0 ? 1.f / ein : 0.f, eout);
                    bv = M.kc_s[j] * sd * (4.f * fabsf(Q) + fabsf(M.s_qt[j]) + 4.f * fabsf(d)) + 3.f * fabsf(v);
                }
                rr += v;
                ab += fabsf(v);
                br += bv;
                ++nt;
            }
            br += (float)nt * ab;  // the additions
            // the sign of the balance: FP64 where the FP32 one is within its bound of 0
            int sg = rr > 0 ? 1 : (rr < 0 ? -1 : 0);
            float rb = br;
            if (fabsf(rr) <= 2.f * ESM_U32 * br) {
                double r64 = node_residual64<float>(Md, th, gv, ev, zv, n, t, rep, nullptr);
                sg = r64 > 0 ? 1 : (r64 < 0 ? -1 : 0);
                rr = (float)r64;
                rb = fabsf(rr);
            }
            float Gn = sg > 0 ? dt * csh : (sg < 0 ? -(dt * cdu) : 0.f);
            float gb = 2.f * fabsf(Gn);  // (its product and the rounded prices)
            if (sg > 0) {
                part[2].add(dt * rr);
                pe[2] += dt * (rb + 2.f * fabsf(rr));
            } else {
                part[3].add(-(dt * rr));
                pe[3] += dt * (rb + 2.f * fabsf(rr));
            }
#pragma unroll
            for (int q = 0; q < ESM_SCORE_MAXU; ++q) {
                if (q >= nu) break;
                int u = M.nu_unit[p0 + q], j = M.u_loc[u];
                int kd = M.u_kind[u];
                if (kd == ESM_UNIT_REN) {
                    float bs;
                    float A = avail_map<float>(wr(M.r_series[j], &bs));
                    float wA = 8.f + bs;  // A's bound relative to A
                    float g0 = dt * (M.r_mc[j] * (A * M.kc_r[j]));
                    part[0].add(g0);
                    pe[0] += (wA + 4.f) * fabsf(g0);
                    float a1 = dt * (M.r_mc[j] * A), a2 = A * Gn;
                    dk[q].add(a1 - a2);
                    de[q] += (wA + 4.f) * (fabsf(a1) + fabsf(a2)) + A * gb;
                } else if (kd == ESM_UNIT_DISP) {
                    float A = M.d_avail[j], kv = M.kc_d[j];
                    float Y = gv[sidx(j, t, rep, T, R)];
                    float Yc = clampr<float>(Y, 0, 1);
                    float g0 = dt * (M.d_mc[j] * (A * kv * Yc));
                    part[0].add(g0);
                    pe[0] += 6.f * fabsf(g0);
                    float exs = fabsf(Y - Yc);
                    if (exs > 0) {
                        float p4 = cv * dt * (kv + k0) * exs;
                        part[4].add(p4);
                        pe[4] += 7.f * p4;
                    }
                    if (!(0.f < Y && Y < 1.f)) {
                        float a0 = cv * dt * exs;
                        dk[q].add(a0);
                        de[q] += 5.f * a0;
                    }
                    float a1 = dt * (M.d_mc[j] * A * Yc), a2 = A * Yc * Gn;
                    dk[q].add(a1 - a2);
                    de[q] += 6.f * (fabsf(a1) + fabsf(a2)) + A * Yc * gb;
                } else {
                    float kv = M.kc_s[j], h = M.s_hours[j], qt = M.s_qt[j], ein = M.s_etain[j], eout = M.s_etaout[j];
                    float mc = M.s_mc[j];
                    float ye = ev[sidx(j, t, rep, T, R)], ye1 = ev[sidx(j, (t + 1) % T, rep, T, R)];
                    float dd, jj;
                    float cc = soc_cost<float>(h, qt, ein, eout, mc, kv, kv + k0, dt, cv, ye, ye1, &dd, &jj);
                    float Ec = clampr<float>(ye, 0, 1), Ec1 = clampr<float>(ye1, 0, 1);
                    float Q = h * (Ec1 - Ec) / dt, d = Q - qt;
                    float sd = fmaxf(ein > 0 ? 1.f / ein : 0.f, eout);
                    float bd = 4.f * fabsf(Q) + fabsf(qt) + 4.f * fabsf(d);  // d's rounding bound
                    float pc = 0, mcx = 0;
                    if (d >= 0)
                        pc = ein > 0 ? d / ein : 0.f;
                    else
                        mcx = fminf(-d * eout, 1.f);
                    float run = dt * mc * kv * (pc + mcx);
                    part[1].add(run);
                    pe[1] += dt * mc * kv * sd * bd + 6.f * fabsf(run);
                    part[4].add(cc - run);
                    pe[4] += (dt * (mc * kv + cv * (kv + k0)) * sd + (ein <= 0 ? cv * dt * (kv + k0) : 0.f)) * bd +
                             9.f * (fabsf(cc) + fabsf(run));
                    float a;
                    if (d >= 0 && ein <= 0) {  // soc_grad (src/energy.jl:470-491)
                        a = cv * dt * d;
                    } else if (d >= 0) {
                        float pcc = d / ein;
                        a = dt * mc * pcc + Gn * pcc + (pcc > 1 ? cv * dt * (pcc - 1) : 0.f);
                    } else {
                        float mc_ = -d * eout;
                        float mcc = fminf(mc_, 1.f);
                        a = dt * mc * mcc - Gn * mcc + ((mc_ > 1 && qt <= 0) ? cv * dt * (mc_ - 1) : 0.f);
                    }
                    dk[q].add(a);
                    de[q] += (dt * mc + fabsf(Gn) + cv * dt) * fmaxf(sd, 1.f) * bd + 6.f * fabsf(a) +
                             (pc + mcx) * (gb + 6.f * fabsf(Gn));
                    if (!(0.f < ye && ye < 1.f)) {
                        float bx2 = cv * h * fabsf(ye - Ec);
                        dk[q].add(bx2);
                        de[q] += 5.f * bx2;
                    }
                }
            }
        }
        // the terms' bounds, Neumaier's (2 |sum| + the second-order term) and the conversion to FP64
        float nsq = (float)(t1 - t0) * ESM_U32;
#pragma unroll
        for (int q = 0; q < ESM_SCORE_MAXU; ++q) {
            if (q >= nu) break;
            int u = M.nu_unit[p0 + q];
            double v = dk[q].value();
            partial[((size_t)c * R + rep) * K + u] = v;
            partial[half + ((size_t)c * R + rep) * K + u] =
                (double)ESM_U32 * ((double)de[q] * (1.0 + (double)nsq) + 2.0 * fabs(v));
        }
#pragma unroll
        for (int i = 0; i < 5; ++i) pe[i] *= 1.f + nsq;
    }
    for (int i = 0; i < 5; ++i) {
        double v = part[i].value();
        sp[slot][lane][i] = v;
        sp[slot][lane][5 + i] = (double)ESM_U32 * ((double)pe[i] + 2.0 * fabs(v));
    }
    __syncthreads();
    if (slot == 0 && rep < R) {
        double acc[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
        for (int s2 = 0; s2 < ESM_SCORE_NSLOT; ++s2)
            for (int i = 0; i < 10; ++i) acc[i] += sp[s2][lane][i];
        size_t o = (size_t)nchunk * nrk + (((size_t)c * ng + blockIdx.y) * R + rep) * 5;
        for (int i = 0; i < 5; ++i) {
            partial[o + i] = acc[i];
            partial[half + o + i] = acc[5 + i] + 8.0 * ESM_U64 * fabs(acc[i]);
        }
    }
}

// the chunk partials summed in chunk order: the gradient dk [R*K] and the cost parts [R*8] (slots
// 2-6) with their bounds (the partials' bounds and the FP64 summation's)
static __global__ void k_score_reduce(int R, int K, int nchunk, int ngroups, const double *partial, double *sums) {
    size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    size_t nrk = (size_t)R * K, half = (size_t)nchunk * (nrk + (size_t)ngroups * R * 5);
    double *dk = sums, *parts = sums + nrk, *dkb = parts + (size_t)R * 8, *pb = dkb + nrk;
    double a = 0, m = 0, b = 0;
    if (i < nrk) {
        for (int c = 0; c < nchunk; ++c) {
            double v = partial[(size_t)c * nrk + i];
            a += v;
            m += fabs(v);
            b += partial[half + (size_t)c * nrk + i];
        }
        dk[i] = a;
        dkb[i] = b + (double)(nchunk + 1) * ESM_U64 * m;
    } else if (i < nrk + (size_t)R * 5) {
        size_t k = i - nrk;
        int rep = (int)(k / 5), f = (int)(k % 5);
        const double *pp = partial + (size_t)nchunk * nrk;
        for (int c = 0; c < nchunk; ++c)
            for (int g = 0; g < ngroups; ++g) {
                size_t o = (((size_t)c * ngroups + g) * R + rep) * 5 + f;
                a += pp[o];
                m += fabs(pp[o]);
                b += pp[half + o];
            }
        parts[(size_t)rep * 8 + 2 + f] = a;
        pb[(size_t)rep * 8 + 2 + f] = b + (double)(nchunk * ngroups + 1) * ESM_U64 * m;
    }
}

// capacity_scores (src/replicas.jl:329): sk = -beta_v mask dk + log-measure gradient; fk = beta_k dK/dk;
// parts: capex and op. One thread per (replica, unit); k_raw in FP64. The bounds follow: sk_err =
// beta_v mask dk_bound; the op total's bound from its parts' bounds.
template <class real>
__global__ void k_score_finish(DevModel<real> M, const double *k_raw, const double *u_lo, const double *u_hi,
                               const double *u_capex, double gamma_k, double beta_k, int physical, double *sums,
                               double *sk, double *sk_err, double *fk) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int K = M.K;
    size_t nrk = (size_t)M.R * K;
    double *dk = sums, *parts = sums + nrk, *dkb = parts + (size_t)M.R * 8, *pb = dkb + nrk;
    if (i < M.R * K) {
        int u = i % K;
        double y = k_raw[u];
        bool in = u_lo[u] < y && y < u_hi[u];
        double s = -(double)M.beta_v * ((in ? 1.0 : 0.0) * dk[i]);
        double lm = 0.0;
        if (physical && M.u_kind[u] != ESM_UNIT_REN && in) lm = (double)M.T / (y + (double)M.kappa0);
        sk[i] = s + lm;
        sk_err[i] = fabs((double)M.beta_v) * (in ? dkb[i] : 0.0) + 4.0 * ESM_U64 * (fabs(s) + fabs(lm));
    }
    if (i < K) {
        double kc = fmin(fmax(k_raw[i], u_lo[i]), u_hi[i]);
        double ex = k_raw[i] - kc;
        double sg = ex > 0 ? 1.0 : (ex < 0 ? -1.0 : 0.0);
        fk[i] = beta_k * (u_capex[i] + gamma_k * u_capex[i] * sg);
    }
    if (i < M.R) {
        double capex = 0.0, cm = 0.0;
        for (int u = 0; u < K; ++u) {
            double kc = fmin(fmax(k_raw[u], u_lo[u]), u_hi[u]);
            double v = u_capex[u] * k_raw[u] + gamma_k * u_capex[u] * fabs(k_raw[u] - kc);
            capex += v;
            cm += fabs(v);
        }
        double *P = parts + (size_t)i * 8, *B = pb + (size_t)i * 8;
        double cs = (double)M.c_shed, cd = (double)M.c_dump;
        P[0] = capex;
        P[1] = P[2] + P[3] + (cs * P[4] + cd * P[5]) + P[6];
        P[7] = 0.0;
        B[0] = (double)(K + 4) * ESM_U64 * cm;
        B[1] = B[2] + B[3] + cs * B[4] + cd * B[5] + B[6] +
               8.0 * ESM_U64 * (fabs(P[2]) + fabs(P[3]) + fabs(cs * P[4]) + fabs(cd * P[5]) + fabs(P[6]));
        B[7] = 0.0;
    }
}

// set_dispatchable_capacity! (src/replicas.jl:412): utilisations scaled by c(k0)/c(k1) at every step
template <class real>
__global__ void k_follow_disp(DevModel<real> M, const int *disp, const double *kold, const double *knew,
                              const double *u_lo, const double *u_hi) {
    size_t TR = (size_t)M.T * M.R;
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (size_t)M.D * TR) return;
    int j = (int)(i / TR);
    int u = disp[j];
    double kc0 = fmin(fmax(kold[u], u_lo[u]), u_hi[u]), kc1 = fmin(fmax(knew[u], u_lo[u]), u_hi[u]);
    double sc = kc0 == kc1 ? 1.0 : kc0 / kc1;  // kc_ratio (src/local.jl:2119)
    if (sc == 1.0) return;
    real y = M.g[i];
    M.g[i] = y + y * (real)(sc - 1);
}

// kop curve of the renewable and storage units of one node (kop_term / kop_eval with commit,
// src/kop.jl:79-160; follow_capacities! src/replicas.jl:456-470), per (node, step, replica), units in
// flat order. kold/knew raw capacities (FP64); kc of the dispatchable units already updated.
template <class real>
__global__ void k_kop(DevModel<real> M, const double *kold, const double *k1v, const double *u_lo,
                      const double *u_hi, double kmin) {
    size_t TR = (size_t)M.T * M.R;
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (size_t)M.N * TR) return;
    int n = (int)(i / TR);
    size_t tr = i % TR;
    int t = (int)(tr / M.R), rep = (int)(tr % M.R);
    int T = M.T, R = M.R;
    for (int p = M.nu_ptr[n]; p < M.nu_ptr[n + 1]; ++p) {
        int u = M.nu_unit[p], j = M.u_loc[u];
        int kd = M.u_kind[u];
        if (kd == ESM_UNIT_DISP) continue;
        double k0raw = kold[u];
        double kc0 = fmin(fmax(k0raw, u_lo[u]), u_hi[u]);
        double kc1 = fmin(fmax(k1v[u], u_lo[u]), u_hi[u]);
        real jinj;
        if (kd == ESM_UNIT_REN) {
            jinj = avail_map<real>(wraw(M, M.r_series[j], t, rep));
        } else {
            real ec = clampr<real>(M.e[sidx(j, t, rep, T, R)], 0, 1);
            real ec1 = clampr<real>(M.e[sidx(j, (t + 1) % T, rep, T, R)], 0, 1);
            real d = M.s_hours[j] * (ec1 - ec) / M.dt - M.s_qt[j];
            real pc, mcx;
            if (d >= 0) {
                pc = M.s_etain[j] > 0 ? d / M.s_etain[j] : real(0);
                mcx = 0;
            } else {
                pc = 0;
                mcx = fmin(-d * M.s_etaout[j], real(1));
            }
            jinj = mcx - pc;
        }
        real dkc = (real)(kc1 - kc0);
        real dinj = jinj * dkc;
        real dS = -dinj;
        if (k0raw >= kmin) {  // below kmin: the capacity alone, no following (src/replicas.jl:461)
            real Pt = 0, Qs = 0;
            int nu = 0;
            for (int q = M.up[n]; q < M.up[n + 1]; ++q) {
                int jd = M.ua[q];
                real kap = M.d_avail[jd] * M.kc_d[jd];
                if (!(fabs(kap) >= (real)kmin)) continue;
                real om = M.g[sidx(jd, t, rep, T, R)];
                Pt += kap * om;
                Qs += kap * clampr<real>(om, 0, 1);
                nu += 1;
            }
            if (!(nu == 0 || fabs(Pt) < real(1e-6))) {
                real Q = M.r[i] + Qs;
                real e = Pt - fmax(Q, real(0));
                real P1 = fmax(Q - dinj, real(0)) + e;
                for (int q = M.up[n]; q < M.up[n + 1]; ++q) {
                    int jd = M.ua[q];
                    real kap = M.d_avail[jd] * M.kc_d[jd];
                    if (!(fabs(kap) >= (real)kmin)) continue;
                    size_t gi = sidx(jd, t, rep, T, R);
                    real y0 = M.g[gi];
                    real sigma = kap * y0 / Pt;
                    real y1 = sigma * P1 / kap;
                    dS -= kap * (clampr<real>(y1, 0, 1) - clampr<real>(y0, 0, 1));
                    M.g[gi] = y1;
                }
            }
        }
        M.r[i] += dS;
    }
}

// refresh the clamped capacities (real) from the raw FP64 capacities
template <class real>
__global__ void k_set_kc(int K, const double *k_raw, const double *u_lo, const double *u_hi, const int *u_kind,
                         const int *u_loc, real *kc_d, real *kc_s, real *kc_r) {
    int u = blockIdx.x * blockDim.x + threadIdx.x;
    if (u >= K) return;
    real kc = (real)fmin(fmax(k_raw[u], u_lo[u]), u_hi[u]);
    int j = u_loc[u];
    if (u_kind[u] == ESM_UNIT_DISP)
        kc_d[j] = kc;
    else if (u_kind[u] == ESM_UNIT_STOR)
        kc_s[j] = kc;
    else
        kc_r[j] = kc;
}

#ifdef ESM_COMMON_KERNELS

// regime_window (src/replicas.jl:131-163), one thread per replica; a is 1-based; beta scratch [R*K*T]
__global__ void k_regime_window(int T, int R, int K, const double *Ptr, const double *pi0, const int *moved,
                                const int *window, const int *wstart, const int *reg, int *reg2, double *beta,
                                uint64_t seed, uint32_t it) {
    int rep = blockIdx.x * blockDim.x + threadIdx.x;
    if (rep >= R) return;
    for (int t = 0; t < T; ++t) reg2[(size_t)t * R + rep] = reg[(size_t)t * R + rep];
    if (!moved[rep] || window[rep] <= 0) return;
    int a = min(T, max(1, wstart[rep]));
    int b = min(T, a + window[rep] - 1);
    int B = b - a + 1;
    double *bt = beta + (size_t)rep * K * T;
    for (int q = 0; q < K * B; ++q) bt[q] = 1.0;
    if (b < T) {
        int mb = reg[(size_t)b * R + rep];
        for (int q = 0; q < K; ++q) bt[(size_t)q * B + (B - 1)] = Ptr[(size_t)q * K + mb];
        for (int tau = b - 1; tau >= a; --tau) {
            int col = tau - a, nxt = col + 1;
            for (int q = 0; q < K; ++q) {
                double s = 0.0;
                for (int p = 0; p < K; ++p) s += Ptr[(size_t)q * K + p] * bt[(size_t)p * B + nxt];
                bt[(size_t)q * B + col] = s;
            }
        }
    }
    for (int tau = a; tau <= b; ++tau) {
        int j = tau - a;
        double u, u2;
        uniform2(seed, ESM_TAG_WTH, (uint32_t)(j >> 1), 1, (uint32_t)rep, it, &u, &u2);
        if (j & 1) u = u2;
        double tot = 0.0;
        for (int q = 0; q < K; ++q) {
            double pr = tau == 1 ? pi0[q] : Ptr[(size_t)reg2[(size_t)(tau - 2) * R + rep] * K + q];
            tot += pr * bt[(size_t)q * B + j];
        }
        double tt = u * tot, cc = 0.0;
        int kk = K - 1;
        for (int q = 0; q < K; ++q) {
            double pr = tau == 1 ? pi0[q] : Ptr[(size_t)reg2[(size_t)(tau - 2) * R + rep] * K + q];
            cc += pr * bt[(size_t)q * B + j];
            if (tt <= cc) {
                kk = q;
                break;
            }
        }
        reg2[(size_t)(tau - 1) * R + rep] = kk;
    }
}
// ---------------------------------------------------------------------------------------------
// Langevin step of the shared capacities (langevin_capacities / langevin_update,
// src/replicas.jl:368-403), FP64, one thread per unit; replica average in replica order (:697)
// ---------------------------------------------------------------------------------------------
__global__ void k_langevin(int K, int R, const int *u_group, const int *u_gidx, const double *k_raw, const double *sk,
                           const double *fk, const double *w, const double *eta, const double *kappa_s, double ratio,
                           double kmin, double clip, int box, const double *u_hi, const double *xi, uint64_t seed,
                           uint32_t it, double *knew, int *nclip) {
    int u = blockIdx.x * blockDim.x + threadIdx.x;
    if (u >= K) return;
    int gidx = u_group[u];
    double k = k_raw[u];
    if (eta[gidx] == 0) {
        knew[u] = k;
        return;
    }
    double sbar = 0.0;
    for (int rep = 0; rep < R; ++rep) sbar += w[rep] * sk[(size_t)rep * K + u];
    double g = -fk[u] + ratio * sbar;
    double x = xi ? xi[u] : normal_at(seed, ESM_TAG_LGV, (uint32_t)u_gidx[u], (uint32_t)gidx, it, 0);
    double ks = kappa_s[gidx], et = eta[gidx];
    double wv = log(k + ks);
    double dw0 = et * ((k + ks) * g + 1);
    if (fabs(dw0) > clip) atomicAdd(nclip, 1);
    // clamp (src/replicas.jl:368) by comparisons, as the reference's clamp: a non-finite drift stays
    // non-finite (fmin/fmax would turn NaN into -clip and hide a broken score)
    double w1 = wv + (dw0 > clip ? clip : (dw0 < -clip ? -clip : dw0)) + sqrt(2 * et) * x;
    double wmin = log(kmin + ks);
    w1 = w1 < wmin ? 2 * wmin - w1 : w1;
    if (box) {
        double wmax = log(fmax(u_hi[u], kmin + 1.0) + ks);
        if (w1 > wmax && wv <= wmax) w1 = fmax(2 * wmax - w1, wmin);
    }
    knew[u] = exp(w1) - ks;
}

// k after following: renewables and storage k0 exp(log(k'/k0)) (kop_commit!, src/kop.jl:254),
// or k' when k0 < kmin; dispatchable k'
__global__ void k_kop_capacity(int K, const int *u_kind, const double *kold, const double *knew, double kmin,
                               double *k1) {
    int u = blockIdx.x * blockDim.x + threadIdx.x;
    if (u >= K) return;
    if (u_kind[u] == ESM_UNIT_DISP || kold[u] < kmin)
        k1[u] = knew[u];
    else
        k1[u] = kold[u] * exp(log(knew[u] / kold[u]));
}

#endif

// ---------------------------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------------------------
template <class real>
cudaError_t launch_rebuild(const DevModel<real> &M, cudaStream_t s) {
    size_t n = (size_t)M.N * M.T * M.R;
    k_rebuild<real><<<(unsigned)((n + 255) / 256), 256, 0, s>>>(M);
    return cudaGetLastError();
}


// step chunks of the fused score pass: one per 64 steps, fewer where the partials (and the R*(K+8)
// final sums) would not fit the static score scratch of 2^20 doubles, so that both score entry
// points sum in the same order
// step chunks of the score pass: 64 steps a chunk, fewer chunks where the partials (values and
// bounds) and the sums would not fit 2^20 doubles (the static scratch)
__host__ inline int score_chunks(int T, int R, int K, int N) {
    int ng = (N + ESM_SCORE_NSLOT - 1) / ESM_SCORE_NSLOT;
    long long room = (1LL << 20) - 2LL * R * (K + 8);
    long long nmax = room > 0 ? room / (2LL * R * (K + 5 * ng)) : 0;
    int n = (T + 63) / 64;
    if (nmax >= 1 && n > nmax) n = (int)nmax;
    return n < 1 ? 1 : n;
}
__host__ inline size_t score_partial_doubles(int T, int R, int K, int N) {
    int ng = (N + ESM_SCORE_NSLOT - 1) / ESM_SCORE_NSLOT;
    return 2 * (size_t)score_chunks(T, R, K, N) * R * (K + 5 * (size_t)ng);
}
// the sums: dk [R*K], parts [R*8], and their bounds
__host__ inline size_t score_sum_doubles(int R, int K) { return 2 * (size_t)R * (K + 8); }

template <class S>
cudaError_t launch_scores_fused(const DevModel<double> &M, const S *theta, const S *g, const S *e, const S *z,
                                double *partial, double *sums, cudaStream_t s) {
    int nchunk = score_chunks(M.T, M.R, M.K, M.N);
    int ng = (M.N + ESM_SCORE_NSLOT - 1) / ESM_SCORE_NSLOT;
    int tchunk = (M.T + nchunk - 1) / nchunk;
    dim3 grid((M.R + 31) / 32, ng, nchunk), block(32, ESM_SCORE_NSLOT);
    k_scores_fused<S><<<grid, block, 0, s>>>(M, theta, g, e, z, tchunk, partial);
    cudaError_t err = cudaGetLastError();
    if (err != cudaSuccess) return err;
    size_t n = (size_t)M.R * M.K + (size_t)M.R * 5;
    k_score_reduce<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(M.R, M.K, nchunk, ng, partial, sums);
    return cudaGetLastError();
}

// the FP32 build (launched from the FP32 translation unit, esm_f32.cu)
template <int I>
cudaError_t launch_scores_f32_t(const DevModel<float> &Mf, const DevModel<double> &Md, double *partial, double *sums,
                                cudaStream_t s) {
    int nchunk = score_chunks(Mf.T, Mf.R, Mf.K, Mf.N);
    int ng = (Mf.N + ESM_SCORE_NSLOT - 1) / ESM_SCORE_NSLOT;
    int tchunk = (Mf.T + nchunk - 1) / nchunk;
    dim3 grid((Mf.R + 31) / 32, ng, nchunk), block(32, ESM_SCORE_NSLOT);
    k_scores_f32<<<grid, block, 0, s>>>(Mf, Md, tchunk, partial);
    cudaError_t err = cudaGetLastError();
    if (err != cudaSuccess) return err;
    size_t n = (size_t)Mf.R * Mf.K + (size_t)Mf.R * 5;
    k_score_reduce<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(Mf.R, Mf.K, nchunk, ng, partial, sums);
    return cudaGetLastError();
}
template <int I>
cudaError_t preload_scores_f32_t() {
    cudaFuncAttributes a;
    cudaError_t e = cudaFuncGetAttributes(&a, k_scores_f32);
    if (e != cudaSuccess) return e;
    return cudaFuncGetAttributes(&a, k_score_reduce);
}

template <class real>
cudaError_t launch_score_finish(const DevModel<real> &M, const double *k_raw, const double *lo, const double *hi,
                                const double *capex, double gamma_k, double beta_k, int physical, double *sums,
                                double *sk, double *sk_err, double *fk, cudaStream_t s) {
    int n = M.R * M.K;
    if (n < M.K) n = M.K;
    k_score_finish<real><<<(n + 127) / 128, 128, 0, s>>>(M, k_raw, lo, hi, capex, gamma_k, beta_k, physical, sums, sk,
                                                          sk_err, fk);
    return cudaGetLastError();
}

template <class real>
cudaError_t launch_follow_disp(const DevModel<real> &M, const int *disp, const double *kold, const double *knew,
                               const double *lo, const double *hi, cudaStream_t s) {
    size_t n = (size_t)M.D * M.T * M.R;
    k_follow_disp<real><<<(unsigned)((n + 255) / 256), 256, 0, s>>>(M, disp, kold, knew, lo, hi);
    return cudaGetLastError();
}

template <class real>
cudaError_t launch_kop(const DevModel<real> &M, const double *kold, const double *k1, const double *lo,
                       const double *hi, double kmin, cudaStream_t s) {
    size_t n = (size_t)M.N * M.T * M.R;
    k_kop<real><<<(unsigned)((n + 255) / 256), 256, 0, s>>>(M, kold, k1, lo, hi, kmin);
    return cudaGetLastError();
}

template <class real>
cudaError_t launch_set_kc(int K, const double *k_raw, const double *lo, const double *hi, const int *u_kind,
                          const int *u_loc, real *kc_d, real *kc_s, real *kc_r, cudaStream_t s) {
    k_set_kc<real><<<(K + 127) / 128, 128, 0, s>>>(K, k_raw, lo, hi, u_kind, u_loc, kc_d, kc_s, kc_r);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------------------------
// weather process (src/replicas.jl:49-112 pCN in the VAR innovations; :131-163 regime window;
// :207 compensate_weather!) for the diagonal single-level VAR; the recursion runs in FP64
// ---------------------------------------------------------------------------------------------
// the seasonal regressors of step t: cos and sin of 2 pi tau / T at tau = t + 1 (src/weather.jl:50),
// tabulated once per model
static __global__ void k_season(int T, double *season) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= T) return;
    double tau = t + 1;
    season[2 * t] = cos(2 * 3.141592653589793 * tau / T);
    season[2 * t + 1] = sin(2 * 3.141592653589793 * tau / T);
}

template <class real>
__device__ inline double var_mean(const DevModel<real> &M, const double *phi, const double *mu, const double *season,
                                  int k, int i, double zprev, int t) {
    double cs = season[2 * t], sn = season[2 * t + 1];
    const double *m3 = mu + ((size_t)k * M.n0 + i) * 3;
    return phi[(size_t)k * M.n0 + i] * zprev + 1.0 * m3[0] + cs * m3[1] + sn * m3[2];
}

template <class real>
__device__ inline double weather_normal(uint64_t seed, uint32_t j, uint32_t rep, uint32_t it) {
    double u0, u1;
    uniform2(seed, ESM_TAG_WTH, j >> 1, 0, rep, it, &u0, &u1);
    real rr = sqrt(real(-2) * log((real)(1.0 - u0)));   // 1 - u0 >= 2^-53 before the cast: never log(0)
    real a = real(6.283185307179586) * (real)u1;
    return (double)((j & 1) ? rr * sin(a) : rr * cos(a));
}

// one pass over series i of replica rep: innovations at regA, rotation by theta (> 0), rebuilt at regB
template <class real>
__global__ void k_weather_z(DevModel<real> M, const double *phi, const double *mu, const double *season,
                            const double *sig, const double *sig0, const int *moved, const double *theta, const int *regA,
                            const int *regB, const double *xi, uint64_t seed, uint32_t it, int use_theta) {
    int rep = blockIdx.y * blockDim.x + threadIdx.x;
    int i = blockIdx.x;
    if (rep >= M.R || i >= M.n0) return;
    if (!moved[rep]) return;
    double th = use_theta ? theta[rep] : 0.0;
    if (use_theta && !(th > 0)) return;
    double ct = cos(th), st = sin(th);
    double zpo = 0, zpn = 0;
    int T = M.T, R = M.R;
    for (int t = 0; t < T; ++t) {
        size_t zi = sidx(i, t, rep, T, R);
        double zo = (double)M.z[zi];
        int ka = regA[(size_t)t * R + rep], kb = regB[(size_t)t * R + rep];
        double e = t == 0 ? zo / sig0[i] : (zo - var_mean(M, phi, mu, season, ka, i, zpo, t)) / sig[(size_t)ka * M.n0 + i];
        if (use_theta) {
            double x = xi ? xi[(size_t)rep * M.n0 * T + (size_t)t * M.n0 + i]
                          : weather_normal<real>(seed, (uint32_t)((size_t)t * M.n0 + i), (uint32_t)rep, it);
            e = ct * e + st * x;
        }
        double zn = t == 0 ? sig0[i] * e : var_mean(M, phi, mu, season, kb, i, zpn, t) + sig[(size_t)kb * M.n0 + i] * e;
        M.z[zi] = (real)zn;
        zpo = zo;
        zpn = zn;
    }
}

// compensate_weather! (src/replicas.jl:207) per (node, step, replica) of the moved replicas
template <class real>
__global__ void k_compensate(DevModel<real> M, const int *moved, const real *r0) {
    size_t TR = (size_t)M.T * M.R;
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (size_t)M.N * TR) return;
    int n = (int)(i / TR);
    size_t tr = i % TR;
    int t = (int)(tr / M.R), rep = (int)(tr % M.R);
    if (!moved[rep]) return;
    real need = M.r[i] - r0[i];
    if (fabs(need) < real(1e-6)) return;
    int nu = M.up[n + 1] - M.up[n];
    if (nu == 0) return;
    real tot = 0;
    for (int q = 0; q < nu; ++q) {
        int j = M.ua[M.up[n] + q];
        real ks = M.d_avail[j] * M.kc_d[j];
        real ps = ks * clampr<real>(M.g[sidx(j, t, rep, M.T, M.R)], 0, 1);
        tot += need > 0 ? fmax(ks - ps, real(0)) : ps;
    }
    if (!(tot > real(1e-9))) return;
    real a = need > 0 ? fmin(need, tot) / tot : fmax(need, -tot) / tot;
    for (int q = 0; q < nu; ++q) {
        int j = M.ua[M.up[n] + q];
        real ks = M.d_avail[j] * M.kc_d[j];
        if (fabs(ks) < real(1e-9)) continue;
        size_t gi = sidx(j, t, rep, M.T, M.R);
        real ps = ks * clampr<real>(M.g[gi], 0, 1);
        real w = need > 0 ? fmax(ks - ps, real(0)) : ps;
        real dy = a * w / ks;
        if (dy == 0) continue;
        M.g[gi] += dy;
    }
}

template <class real>
cudaError_t launch_weather_z(const DevModel<real> &M, const double *phi, const double *mu, const double *season,
                             const double *sig, const double *sig0, const int *moved, const double *theta,
                             const int *regA, const int *regB, const double *xi, uint64_t seed, uint32_t it,
                             int use_theta, cudaStream_t s) {
    int bx = M.R < 64 ? M.R : 64;
    dim3 grid(M.n0, (M.R + bx - 1) / bx);
    k_weather_z<real><<<grid, bx, 0, s>>>(M, phi, mu, season, sig, sig0, moved, theta, regA, regB, xi, seed, it,
                                          use_theta);
    return cudaGetLastError();
}

template <class real>
cudaError_t launch_compensate(const DevModel<real> &M, const int *moved, const real *r0, cudaStream_t s) {
    size_t n = (size_t)M.N * M.T * M.R;
    k_compensate<real><<<(unsigned)((n + 255) / 256), 256, 0, s>>>(M, moved, r0);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------------------------
// Weather features of every replica (weather_features / replica_features, src/replicas.jl:246-276):
// the system load D_t = sum_n (load of node n)+, the availability of every weather-dependent
// carrier, and the residual load D_t - sum_j kref_j A_j,t at fixed reference capacities of the
// renewable units, from the replica's weather X = xbar + s z and the data map (k_rebuild's).
// Pass 1, one thread per (step, replica): per step the load and residual load in GW and the
// carriers' summed availabilities, into buf [(2 + C) x T x R] (replica fastest). Pass 2, one block
// per replica: the means over the year, the residual load's peak and worst cyclic 7-step mean, the
// regime frequencies and the number of regime switches, every sum in a fixed order (bitwise
// repeatable).
// ---------------------------------------------------------------------------------------------
template <class real>
__global__ void k_wfeat_steps(DevModel<real> M, const double *kref_r, const int *carrier_r, int C, double *buf) {
    size_t TR = (size_t)M.T * M.R;
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= TR) return;
    int t = (int)(i / M.R), rep = (int)(i % M.R);
    double D = 0;
    for (int n = 0; n < M.N; ++n) {
        double x = (double)wraw(M, n, t, rep);
        D += x > 0 ? x : 0.0;
    }
    double Rs = 0;
    for (int c = 0; c < C; ++c) buf[(size_t)(2 + c) * TR + i] = 0;
    for (int j = 0; j < M.Nren; ++j) {
        double A = (double)avail_map<real>(wraw(M, M.r_series[j], t, rep));
        Rs += kref_r[j] * A;
        int c = carrier_r[j];
        buf[(size_t)(2 + c) * TR + i] += A;
    }
    buf[i] = D / 1e3;
    buf[TR + i] = (D - Rs) / 1e3;
}

#define ESM_WFEAT_THREADS 256
template <class real>
__global__ void __launch_bounds__(ESM_WFEAT_THREADS) k_wfeat_reduce(int T, int R, int C, const int *ncar,
                                                                   const double *buf, const int32_t *reg, int nreg,
                                                                   double *out) {
    __shared__ double sh[ESM_WFEAT_THREADS];
    int rep = blockIdx.x, tid = threadIdx.x;
    size_t TR = (size_t)T * R;
    int nf = 5 + C + nreg;
    double *o = out + (size_t)rep * nf;
    // a fixed-order block sum (each thread's strided steps in order, then a tree) of f(t)
    auto bsum = [&](auto f) -> double {
        double a = 0;
        for (int t = tid; t < T; t += ESM_WFEAT_THREADS) a += f(t);
        sh[tid] = a;
        __syncthreads();
        for (int w = ESM_WFEAT_THREADS / 2; w > 0; w >>= 1) {
            if (tid < w) sh[tid] += sh[tid + w];
            __syncthreads();
        }
        double v = sh[0];
        __syncthreads();
        return v;
    };
    auto bmax = [&](auto f) -> double {
        double a = -INFINITY;
        for (int t = tid; t < T; t += ESM_WFEAT_THREADS) a = fmax(a, f(t));
        sh[tid] = a;
        __syncthreads();
        for (int w = ESM_WFEAT_THREADS / 2; w > 0; w >>= 1) {
            if (tid < w) sh[tid] = fmax(sh[tid], sh[tid + w]);
            __syncthreads();
        }
        double v = sh[0];
        __syncthreads();
        return v;
    };
    auto at = [&](int f, int t) { return buf[(size_t)f * TR + (size_t)t * R + rep]; };
    double load = bsum([&](int t) { return at(0, t); });
    double res = bsum([&](int t) { return at(1, t); });
    double peak = bmax([&](int t) { return at(1, t); });
    double w7 = bmax([&](int t) {
        double a = 0;
        for (int q = 0; q < 7; ++q) a += at(1, (t + q) % T);
        return a / 7.0;
    });
    if (tid == 0) {
        o[0] = load / T;
        o[1 + C] = res / T;
        o[2 + C] = peak;
        o[3 + C] = w7;
    }
    for (int c = 0; c < C; ++c) {
        double a = bsum([&](int t) { return at(2 + c, t); });
        if (tid == 0) o[1 + c] = ncar[c] > 0 ? a / ((double)T * ncar[c]) : 0.0;
    }
    for (int k = 0; k < nreg; ++k) {
        double a = bsum([&](int t) { return reg[(size_t)t * R + rep] == k ? 1.0 : 0.0; });
        if (tid == 0) o[4 + C + k] = a / T;
    }
    double sw = bsum([&](int t) { return t + 1 < T && reg[(size_t)(t + 1) * R + rep] != reg[(size_t)t * R + rep] ? 1.0 : 0.0; });
    if (tid == 0) o[4 + C + nreg] = sw;
}

template <class real>
cudaError_t launch_weather_features(const DevModel<real> &M, const double *kref_r, const int *carrier_r, int C,
                                    const int *ncar, const int32_t *reg, double *buf, double *out, cudaStream_t s) {
    size_t TR = (size_t)M.T * M.R;
    k_wfeat_steps<real><<<(unsigned)((TR + 255) / 256), 256, 0, s>>>(M, kref_r, carrier_r, C, buf);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    k_wfeat_reduce<real><<<M.R, ESM_WFEAT_THREADS, 0, s>>>(M.T, M.R, C, ncar, buf, reg, M.nreg, out);
    return cudaGetLastError();
}

}  // namespace esm
