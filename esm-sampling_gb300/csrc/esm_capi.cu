// C ABI of libesmcuda.so (include/esmcuda.h): context, uploads, and the replica-step entry points.
#define ESM_COMMON_KERNELS
#include <cuda_runtime.h>
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <string>
#include <mutex>
#include <thread>
#include <vector>

#include "../../include/esmcuda.h"
#include "esm_common.cuh"
#include "esm_kernels_impl.cuh"
#include "esm_launch.cuh"

using std::vector;

namespace {

// disp -> knew, others -> kold: the capacities after set_dispatchable_capacity!, before the kop moves
__global__ void k_mix(int K, const int *u_kind, const double *kold, const double *knew, double *kmid) {
    int u = blockIdx.x * blockDim.x + threadIdx.x;
    if (u >= K) return;
    kmid[u] = u_kind[u] == ESM_UNIT_DISP ? knew[u] : kold[u];
}

struct DevBuf {
    void *p = nullptr;
    size_t n = 0;
};

}  // namespace

// device buffers of esm_state_save
struct esm_snap {
    void *theta = nullptr, *g = nullptr, *e = nullptr, *z = nullptr;
    int32_t *reg = nullptr;
    double *k = nullptr;
};

struct esm_ctx {
    int precision = 32;
    int R = 0;
    cudaStream_t stream = nullptr;
    std::string err;
    int64_t launches = 0;
    bool has_state = false, has_scores = false;
    int move_wpb = 1;           // k_move block shape: warps per block (1, 2 or 4)
    int max_warps = 0;          // k_move warps launched per move: the resident limit or a tuned count
    // the cooperative walk of the separable moves (k_move_sep): moves with at least sep_min units
    // (0: off), its grid and where its per-warp walk buffers live
    int sep_min = ESM_SEP_MIN_DEFAULT, sep_max_warps = 0, sep_in_smem = 1;
    int sl_nunits = 0;  // eligible units of the last long-range storage sweep (its move log)
    int device = -1;                   // the device the context was created on
    double *score_scratch = nullptr;   // device address of the static score scratch on that device
    char *d_sep_slab = nullptr;
    int warps_cap[3] = {0, 0, 0};  // the resident limit per block shape (1, 2, 4 warps per block)
    int nsm = 0;
    esm::DevModel<float> Mf;
    esm::DevModel<double> Md;
    vector<void *> allocs;
    // host copies needed by the entry points
    int N, L, T, K, D, S, n0, nreg, ngroups;
    double dt, gamma_k, beta_k, beta_v, kappa0;
    int physical;
    uint64_t seed;
    vector<int> class_len;      // steps per class
    int ncls;
    // device (precision-independent)
    int *d_steps[3] = {nullptr, nullptr, nullptr};
    int *d_disp = nullptr, *d_ugroup = nullptr, *d_ugidx = nullptr, *d_ukind = nullptr, *d_uloc = nullptr;
    double *d_lo = nullptr, *d_hi = nullptr, *d_capex = nullptr;
    double *d_k = nullptr, *d_kold = nullptr, *d_knew = nullptr, *d_k1 = nullptr, *d_kmid = nullptr;
    double *d_sums = nullptr, *d_sk = nullptr, *d_fk = nullptr, *d_sk_err = nullptr;
    double *d_score_part = nullptr;  // the chunk partials of the fused score pass
    const double *last_sums = nullptr;  // the sums (and bounds) of the last score call
    double *d_w = nullptr, *d_eta = nullptr, *d_kappa = nullptr, *d_xi = nullptr;
    int *d_nclip = nullptr;
    unsigned long long *d_stats = nullptr;
    int32_t *d_reg = nullptr, *d_reg2 = nullptr;
    void *d_scratch = nullptr;
    char *d_descs = nullptr;  // the move descriptors of the current class pass
    esm_snap *snap = nullptr;  // esm_state_save buffers (device memory in allocs)
    bool has_snap = false;
    unsigned long long *d_occ = nullptr;
    unsigned int *d_item_ctr = nullptr;  // per move: the next item of the class pass
    int move_schedule = ESM_MOVES_PER_MOVE;  // one launch per move, or the whole class per launch
    unsigned int *d_wave_done = nullptr;     // per work item: moves completed (whole-class launch)
    int *d_wave_err = nullptr;               // set when a wait of the whole-class launch ran out
    size_t wave_items = 0;
    // weather features of the replicas (esm_replica_features): the renewable units' flat indices and
    // carriers (their groups, numbered in increasing group order), and lazily allocated buffers
    std::vector<int> ren_unit, ren_car, car_units;
    double *d_wf_kref = nullptr, *d_wf_buf = nullptr, *d_wf_out = nullptr;
    int *d_wf_car = nullptr, *d_wf_ncar = nullptr;
    uint32_t *d_sweep = nullptr;         // the sweep index of the current class pass
    // storage multiscale sweep
    int storage_ms = 0, storage_long = 0;
    std::vector<int> sgp, sgu;           // storage groups (host copies)
    std::vector<int> stor;               // flat unit of every storage unit (host copies of the model)
    std::vector<double> ulo, uhi, uhours;
    double kappa_min = 1.0;
    int *d_sl_plan = nullptr;            // the long-range sweep's per-unit move lists
    esm_ctx *probe = nullptr;            // one-replica context of the lag probe (esm_opts.probe)
    int sms_threads = 0;
    size_t sms_per = 0;                  // reals of global scratch per storage-kernel thread (0: local arrays)
    void *d_sms_scratch = nullptr;
    int scratch_warps = 0;               // line-move warps the global scratch holds (0: no global scratch needed)
    unsigned long long *d_sms_stats = nullptr;
    cudaGraphExec_t graph[3] = {nullptr, nullptr, nullptr};  // a whole class pass, per class
    // weather
    double *d_season = nullptr;  // cos, sin of the seasonal phase per step
    double *d_phi = nullptr, *d_mu = nullptr, *d_sig = nullptr, *d_sig0 = nullptr, *d_Ptr = nullptr, *d_pi0 = nullptr;
    double *d_wbeta = nullptr, *d_wtheta = nullptr, *d_wxi = nullptr;
    int *d_moved = nullptr, *d_window = nullptr, *d_wstart = nullptr, *d_wflag = nullptr;
    void *d_r0 = nullptr;
    // precision-dependent state pointers (aliases into Mf / Md)
    void *theta = nullptr, *g = nullptr, *e = nullptr, *r = nullptr, *F = nullptr, *z = nullptr;
    void *kc_d = nullptr, *kc_s = nullptr, *kc_r = nullptr;
    // device timing
    bool timing = false;
    struct Mark {
        int kind;
        cudaEvent_t a, b;
    };
    vector<Mark> marks;
    vector<cudaEvent_t> pool;
    double acc_ms[ESM_KT_N] = {};
    double acc_n[ESM_KT_N] = {};
};

namespace {

cudaEvent_t ev_get(esm_ctx *c) {
    if (!c->pool.empty()) {
        cudaEvent_t e = c->pool.back();
        c->pool.pop_back();
        return e;
    }
    cudaEvent_t e;
    cudaEventCreate(&e);
    return e;
}

// bracket the launches of one kernel family with events when timing is on
struct Span {
    esm_ctx *c;
    int kind;
    cudaEvent_t a = nullptr;
    Span(esm_ctx *c_, int k) : c(c_), kind(k) {
        if (c->timing) {
            a = ev_get(c);
            cudaEventRecord(a, c->stream);
        }
    }
    ~Span() {
        if (a) {
            cudaEvent_t b = ev_get(c);
            cudaEventRecord(b, c->stream);
            c->marks.push_back({kind, a, b});
        }
    }
};

int fail(esm_ctx *c, int code, const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    if (c) c->err = buf;
    return code;
}

#define CK(call)                                                                                 \
    do {                                                                                         \
        cudaError_t e_ = (call);                                                                 \
        if (e_ != cudaSuccess)                                                                   \
            return fail(c, e_ == cudaErrorMemoryAllocation ? ESM_ENOMEM : ESM_ECUDA, "%s: %s (%s:%d)", #call, \
                        cudaGetErrorString(e_), __FILE__, __LINE__);                             \
    } while (0)

template <class T>
int dalloc(esm_ctx *c, T **p, size_t n) {
    void *q = nullptr;
    cudaError_t e = cudaMalloc(&q, sizeof(T) * (n ? n : 1));
    if (e != cudaSuccess) return fail(c, ESM_ENOMEM, "cudaMalloc of %zu bytes: %s", sizeof(T) * n, cudaGetErrorString(e));
    c->allocs.push_back(q);
    *p = (T *)q;
    return ESM_OK;
}

template <class T>
int upload(esm_ctx *c, T **p, const T *h, size_t n) {
    int rc = dalloc(c, p, n);
    if (rc) return rc;
    if (n && h) CK(cudaMemcpyAsync(*p, h, sizeof(T) * n, cudaMemcpyHostToDevice, c->stream));
    return ESM_OK;
}

template <class real>
int upload_real(esm_ctx *c, const real **p, const double *h, size_t n) {
    vector<real> tmp(n ? n : 1);
    for (size_t i = 0; i < n; ++i) tmp[i] = (real)h[i];
    real *q;
    int rc = dalloc(c, &q, n);
    if (rc) return rc;
    CK(cudaMemcpy(q, tmp.data(), sizeof(real) * n, cudaMemcpyHostToDevice));
    *p = q;
    return ESM_OK;
}

template <class real>
int upload_real_vec(esm_ctx *c, const real **p, const vector<double> &h) {
    return upload_real<real>(c, p, h.data(), h.size());
}

void class_steps(int T, int cls, vector<int> &out) {
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

template <class real>
esm::DevModel<real> &dm(esm_ctx *c);
template <>
esm::DevModel<float> &dm<float>(esm_ctx *c) { return c->Mf; }
template <>
esm::DevModel<double> &dm<double>(esm_ctx *c) { return c->Md; }

// build the device model of one precision
template <class real>
int build_model(esm_ctx *c, const esm_model *m, const esm_opts *o) {
    esm::DevModel<real> &M = dm<real>(c);
    memset(&M, 0, sizeof M);
    int N = m->N, L = m->L, K = m->K, D = m->D, S = m->S;
    M.N = N;
    M.L = L;
    M.T = m->T;
    M.R = o->R;
    M.K = K;
    M.D = D;
    M.S = S;
    M.n0 = m->n0;
    M.nreg = m->nreg;
    M.nfields = m->nfields;
    M.nlev = m->nlev;
    M.natoms = m->field_atom_ptr[m->nfields];
    M.nextra = (int)nearbyint(o->extra * N);
    M.span = o->span > 0 ? o->span : std::max(1, 32 / o->R);
    M.maxpts = o->max_points;
    M.dt = (real)m->dt;
    M.c_shed = (real)m->c_shed;
    M.c_dump = (real)m->c_dump;
    M.c_viol = (real)m->c_viol;
    M.kappa0 = (real)m->kappa0;
    M.beta_v = (real)m->beta_v;
    M.maxnats = (real)o->maxnats;
    M.kmin = (real)o->kappa_min;
    M.seed = o->seed;
    double tot = 0;
    for (int q = 0; q < ESM_NFAM; ++q) tot += o->family_rates[q];
    double cum = 0;
    for (int q = 0; q < ESM_NFAM; ++q) {
        cum += o->family_rates[q];
        M.cumw[q] = cum / tot;
    }
    int rc;
    // network
    vector<int> nlp(N + 1, 0), nl;
    {
        vector<vector<int>> lst(N);
        for (int e = 0; e < L; ++e) {
            lst[m->bus0[e]].push_back(e);
            lst[m->bus1[e]].push_back(e);
        }
        for (int n = 0; n < N; ++n) {
            nlp[n + 1] = nlp[n] + (int)lst[n].size();
            nl.insert(nl.end(), lst[n].begin(), lst[n].end());
        }
    }
    vector<int> lbp(N + 1, 0), lbl;
    {
        vector<vector<int>> lst(N);
        for (int e = 0; e < L; ++e) lst[m->bus0[e]].push_back(e);
        for (int n = 0; n < N; ++n) {
            lbp[n + 1] = lbp[n] + (int)lst[n].size();
            lbl.insert(lbl.end(), lst[n].begin(), lst[n].end());
        }
    }
    int *ip;
#define UPI(field, src, n)                          \
    if ((rc = upload(c, &ip, (src), (size_t)(n)))) \
        return rc;                                  \
    M.field = ip;
    UPI(bus0, m->bus0, L);
    UPI(bus1, m->bus1, L);
    UPI(nlp, nlp.data(), N + 1);
    UPI(nl, nl.data(), nl.size());
    UPI(lb0_ptr, lbp.data(), N + 1);
    UPI(lb0_line, lbl.data(), lbl.size());
    UPI(comp, m->comp, N);
    if ((rc = upload_real<real>(c, &M.lb, m->line_b, L))) return rc;
    if ((rc = upload_real<real>(c, &M.ls, m->line_s, L))) return rc;
    if ((rc = upload_real<real>(c, &M.Z, m->reroute, (size_t)N * N))) return rc;
    // units
    vector<int> u_loc(K, -1), r_bus, r_series, d_bus, d_group, s_bus;
    vector<double> r_mc, d_avail, d_mc, s_h, s_ei, s_eo, s_q, s_mc;
    int nren = 0;
    for (int u = 0; u < K; ++u) {
        if (m->unit_kind[u] == ESM_UNIT_REN) {
            u_loc[u] = nren++;
            r_bus.push_back(m->unit_bus[u]);
            r_series.push_back(m->unit_series[u]);
            r_mc.push_back(m->unit_mc[u]);
        }
    }
    for (int j = 0; j < D; ++j) {
        int u = m->disp[j];
        u_loc[u] = j;
        d_bus.push_back(m->unit_bus[u]);
        d_group.push_back(m->unit_group[u]);
        d_avail.push_back(m->unit_avail[u]);
        d_mc.push_back(m->unit_mc[u]);
    }
    for (int j = 0; j < S; ++j) {
        int u = m->stor[j];
        u_loc[u] = j;
        s_bus.push_back(m->unit_bus[u]);
        s_h.push_back(m->unit_hours[u]);
        s_ei.push_back(m->unit_eta_in[u]);
        s_eo.push_back(m->unit_eta_out[u]);
        s_q.push_back(m->unit_qt[u]);
        s_mc.push_back(m->unit_mc[u]);
    }
    M.Nren = nren;
    UPI(r_bus, r_bus.data(), nren);
    UPI(r_series, r_series.data(), nren);
    UPI(d_bus, d_bus.data(), D);
    UPI(d_group, d_group.data(), D);
    UPI(s_bus, s_bus.data(), S);
    UPI(u_kind, m->unit_kind, K);
    UPI(u_loc, u_loc.data(), K);
    if ((rc = upload_real_vec<real>(c, &M.r_mc, r_mc))) return rc;
    if ((rc = upload_real_vec<real>(c, &M.d_avail, d_avail))) return rc;
    if ((rc = upload_real_vec<real>(c, &M.d_mc, d_mc))) return rc;
    if ((rc = upload_real_vec<real>(c, &M.s_hours, s_h))) return rc;
    if ((rc = upload_real_vec<real>(c, &M.s_etain, s_ei))) return rc;
    if ((rc = upload_real_vec<real>(c, &M.s_etaout, s_eo))) return rc;
    if ((rc = upload_real_vec<real>(c, &M.s_qt, s_q))) return rc;
    if ((rc = upload_real_vec<real>(c, &M.s_mc, s_mc))) return rc;
    // node -> flat units (ascending)
    vector<int> nup(N + 1, 0), nuu;
    {
        vector<vector<int>> lst(N);
        for (int u = 0; u < K; ++u) lst[m->unit_bus[u]].push_back(u);
        for (int n = 0; n < N; ++n) {
            if (lst[n].size() > 8) return fail(c, ESM_EINVAL, "node %d has %zu units (at most 8)", n, lst[n].size());
            nup[n + 1] = nup[n] + (int)lst[n].size();
            nuu.insert(nuu.end(), lst[n].begin(), lst[n].end());
        }
    }
    UPI(nu_ptr, nup.data(), N + 1);
    UPI(nu_unit, nuu.data(), nuu.size());
    // weather
    if ((rc = upload_real<real>(c, &M.xbar, m->xbar, (size_t)m->n0 * m->T))) return rc;
    if ((rc = upload_real<real>(c, &M.wscale, m->wscale, m->n0))) return rc;
    // move tables
    int natoms = M.natoms;
    UPI(frole, m->field_role, m->nfields);
    UPI(fap, m->field_atom_ptr, m->nfields + 1);
    UPI(ap, m->atom_ptr, natoms + 1);
    UPI(ai, m->atom_idx, m->atom_ptr[natoms]);
    if ((rc = upload_real<real>(c, &M.av, m->atom_val, m->atom_ptr[natoms]))) return rc;
    UPI(up, m->units_ptr, N + 1);
    UPI(ua, m->units_at, m->units_ptr[N]);
    UPI(sp, m->stor_ptr, N + 1);
    UPI(sa, m->stor_at, m->stor_ptr[N]);
    {
        double *qp;
        if ((rc = upload(c, &qp, m->qcum, m->nlev))) return rc;
        M.qcum = qp;
    }
    int ncell = m->cell_level_ptr[m->nlev];
    UPI(clp, m->cell_level_ptr, m->nlev + 1);
    UPI(cp, m->cell_ptr, ncell + 1);
    UPI(cu, m->cell_units, m->cell_ptr[ncell]);
    int npair = m->xpart_ptr[N];
    UPI(xpp, m->xpart_ptr, N + 1);
    UPI(xp, m->xpart, npair);
    UPI(xnp, m->xnod_ptr, npair + 1);
    UPI(xn, m->xnod, m->xnod_ptr[npair]);
    if ((rc = upload_real<real>(c, &M.xv, m->xval, m->xnod_ptr[npair]))) return rc;
    UPI(xlp, m->xlk_ptr, npair + 1);
    UPI(xln, m->xlkn, m->xlk_ptr[npair]);
    if ((rc = upload_real<real>(c, &M.xlg, m->xlkg, m->xlk_ptr[npair]))) return rc;
    vector<int> tnnz(N, 0);
    for (int f = 0; f < m->nfields; ++f) {
        if (m->field_role[f] != ESM_ROLE_THETA) continue;
        for (int a = m->field_atom_ptr[f]; a < m->field_atom_ptr[f + 1]; ++a)
            for (int q = m->atom_ptr[a]; q < m->atom_ptr[a + 1]; ++q) tnnz[m->atom_idx[q]] += 1;
    }
    UPI(theta_nnz, tnnz.data(), N);
#undef UPI
    // descriptor capacities
    int maxatom = 0, maxstu = 1;
    for (int f = 0; f < m->nfields; ++f)
        for (int a = m->field_atom_ptr[f]; a < m->field_atom_ptr[f + 1]; ++a) {
            int nz = m->atom_ptr[a + 1] - m->atom_ptr[a];
            maxatom = std::max(maxatom, nz);
            if (m->field_role[f] == ESM_ROLE_SE) maxstu = std::max(maxstu, nz);
        }
    int maxcell = 0;
    for (int q = 0; q < ncell; ++q) maxcell = std::max(maxcell, m->cell_ptr[q + 1] - m->cell_ptr[q]);
    int maxunits = 1;
    for (int n = 0; n < N; ++n) maxunits = std::max(maxunits, m->units_ptr[n + 1] - m->units_ptr[n]);
    // kinks of one move: the leak nodes of an xlocc pair, the two steps of a tsoc move, a tpot
    // node and the far ends of its lines
    int maxleak = 2;
    for (int p = 0; p < npair; ++p) maxleak = std::max(maxleak, m->xlk_ptr[p + 1] - m->xlk_ptr[p]);
    for (int n = 0; n < N; ++n) maxleak = std::max(maxleak, nlp[n + 1] - nlp[n] + 1);
    M.maxe = std::max(std::max(maxatom, maxcell), 4) + 4;
    M.maxl = L;
    M.maxn = N;
    M.maxk = maxleak;
    M.maxku = maxleak * maxunits;
    M.maxstu = maxstu;
    if (M.maxpts == 0) M.maxpts = esm_auto_max_points(maxstu);
    return ESM_OK;
}

template <class real>
int alloc_state(esm_ctx *c) {
    esm::DevModel<real> &M = dm<real>(c);
    size_t TR = (size_t)M.T * M.R;
    real *p;
    int rc;
#define AL(field, n)                          \
    if ((rc = dalloc(c, &p, (size_t)(n)))) \
        return rc;                            \
    M.field = p;                              \
    c->field = p;
    AL(theta, M.N * TR);
    AL(g, M.D * TR);
    AL(e, M.S * TR);
    AL(r, M.N * TR);
    AL(F, M.L * TR);
    AL(z, M.n0 * TR);
#undef AL
    real *q;
    if ((rc = dalloc(c, &q, M.D))) return rc;
    M.kc_d = q;
    c->kc_d = q;
    if ((rc = dalloc(c, &q, M.S))) return rc;
    M.kc_s = q;
    c->kc_s = q;
    if ((rc = dalloc(c, &q, std::max(M.Nren, 1)))) return rc;
    M.kc_r = q;
    c->kc_r = q;
    // line-move grid (resident one-warp blocks) and, when the lane layout exceeds the local arrays,
    // one global scratch slab per block
    int dev = 0, nsm = 0;
    CK(cudaGetDevice(&dev));
    CK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    int wmax = 0;
    for (int i = 0; i < 3; ++i) {
        c->warps_cap[i] = std::max(4, nsm * esm::linemove_blocks_per_sm<real>(M, 1 << i));
        wmax = std::max(wmax, c->warps_cap[i]);
    }
    c->nsm = nsm;
    c->move_wpb = 1;
    c->max_warps = c->warps_cap[0];
    // the global scratch, when the layout needs one, is first sized for the larger grids only up to
    // 1 GB (never fewer warps than the one-warp blocks' limit): many contexts share one GPU;
    // esm_set_move_grid grows it when a larger grid is set
    size_t per = esm::linemove_scratch_reals<real>(M);
    size_t wscr = (size_t)wmax;
    if (per > 0) {
        size_t fit = ((size_t)1 << 30) / (per * sizeof(real));
        wscr = std::max((size_t)c->warps_cap[0], std::min(wscr, fit));
        c->scratch_warps = (int)wscr;
    }
    if ((rc = dalloc(c, &q, per * wscr))) return rc;
    c->d_scratch = q;
    // the cooperative walk: resident warps of k_move_sep and, when two walk regions and the
    // descriptor do not fit a block's shared memory, one global region per warp (at most 1 GB)
    {
        int in_smem = 1;
        int wps = esm::sep_warps_per_sm<real>(M, &in_smem);
        size_t reg = esm::sep_region_bytes<real>(M);
        size_t sw = (size_t)nsm * wps;
        if (!in_smem) sw = std::max<size_t>(64, std::min(sw, ((size_t)1 << 30) / reg));
        c->sep_max_warps = (int)(sw & ~(size_t)1);
        c->sep_in_smem = in_smem;
        if (!in_smem) {
            char *sl;
            if ((rc = dalloc(c, &sl, reg * (size_t)c->sep_max_warps))) return rc;
            c->d_sep_slab = sl;
        }
    }
    // the move descriptors of a class pass
    char *dp;
    if ((rc = dalloc(c, &dp, esm::linemove_smem_per_warp<real>(M) * (size_t)(M.natoms + M.nextra)))) return rc;
    c->d_descs = dp;
    unsigned int *ctr;
    if ((rc = dalloc(c, &ctr, (size_t)(M.natoms + M.nextra)))) return rc;
    c->d_item_ctr = ctr;
    if ((rc = dalloc(c, &c->d_sweep, 1))) return rc;
    // storage sweeps: resident threads of their kernels; the global scratch they need when the lane
    // layout exceeds the local arrays is allocated at their first use (sms_scratch)
    c->sms_threads = esm::plateau_threads<real>(M);
    c->sms_per = esm::plateau_scratch_reals<real>(M);
    if ((rc = dalloc(c, &c->d_sms_stats, 3))) return rc;
    return ESM_OK;
}

// FP32 build: the FP64 clamped capacities of the FP64 model (its tables and parameters) that the
// capacity scores are computed with. The scores weigh every node balance by the shed or the dump
// price according to its sign, and near equilibrium many balances sit within FP32 round-off of zero:
// the fused score pass therefore forms every balance and term in FP64 from the FP32 state.
int alloc_shadow(esm_ctx *c) {
    esm::DevModel<double> &M = c->Md;
    double *p;
    int rc;
#define AL(field, n)                       \
    if ((rc = dalloc(c, &p, (size_t)(n)))) \
        return rc;                         \
    M.field = p;
    AL(kc_d, M.D);
    AL(kc_s, M.S);
    AL(kc_r, std::max(M.Nren, 1));
#undef AL
    return ESM_OK;
}

// the capacity scores of the current state: the fused pass (partials in `partial`, sums in dk and
// parts) and the finish into the context's sk and fk
// the score pass into partial and sums (esm::score_sum_doubles: dk, parts and their bounds), then
// the scores and their bounds into d_sk, d_sk_err
int scores_any(esm_ctx *c, double *partial, double *sums) {
    Span sp(c, ESM_KT_SCORE);
    if (c->precision == 64) {
        CK(esm::launch_scores_fused<double>(c->Md, c->Md.theta, c->Md.g, c->Md.e, c->Md.z, partial, sums, c->stream));
    } else {
        // the FP64 capacities of the balances recomputed in FP64 near 0
        CK(esm::launch_set_kc<double>(c->K, c->d_k, c->d_lo, c->d_hi, c->d_ukind, c->d_uloc, (double *)c->Md.kc_d,
                                      (double *)c->Md.kc_s, (double *)c->Md.kc_r, c->stream));
        CK(esm::launch_scores_f32(c->Mf, c->Md, partial, sums, c->stream));
        c->launches += 1;
    }
    CK(esm::launch_score_finish<double>(c->Md, c->d_k, c->d_lo, c->d_hi, c->d_capex, c->gamma_k, c->beta_k,
                                        c->physical, sums, c->d_sk, c->d_sk_err, c->d_fk, c->stream));
    c->launches += 3;
    c->last_sums = sums;
    return ESM_OK;
}

template <class real>
int set_kc(esm_ctx *c, const double *k) {
    CK(esm::launch_set_kc<real>(c->K, k, c->d_lo, c->d_hi, c->d_ukind, c->d_uloc, (real *)c->kc_d, (real *)c->kc_s,
                                (real *)c->kc_r, c->stream));
    c->launches += 1;
    return ESM_OK;
}

int set_kc_any(esm_ctx *c, const double *k) { return c->precision == 64 ? set_kc<double>(c, k) : set_kc<float>(c, k); }

template <class real>
int up_state(esm_ctx *c, void *dst, const double *h, size_t n) {
    if (!h) return ESM_OK;
    vector<real> tmp(n);
    for (size_t i = 0; i < n; ++i) tmp[i] = (real)h[i];
    CK(cudaMemcpyAsync(dst, tmp.data(), sizeof(real) * n, cudaMemcpyHostToDevice, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return ESM_OK;
}

template <class real>
int down_state(esm_ctx *c, const void *src, double *h, size_t n) {
    if (!h) return ESM_OK;
    vector<real> tmp(n);
    CK(cudaMemcpyAsync(tmp.data(), src, sizeof(real) * n, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    for (size_t i = 0; i < n; ++i) h[i] = (double)tmp[i];
    return ESM_OK;
}

int rebuild_any(esm_ctx *c) {
    Span sp(c, ESM_KT_REBUILD);
    CK(c->precision == 64 ? esm::launch_rebuild<double>(c->Md, c->stream) : esm::launch_rebuild<float>(c->Mf, c->stream));
    c->launches += 1;
    return ESM_OK;
}

__global__ void k_set_word(uint32_t *p, uint32_t v) { *p = v; }

int class_pass_launch(esm_ctx *c, int cls, int limit) {
    int ns = c->class_len[cls];
    esm::SepLaunch sep{c->sep_min, c->sep_max_warps, c->sep_in_smem, c->d_sep_slab};
    esm::WaveLaunch wave{c->move_schedule == ESM_MOVES_PER_CLASS, c->d_wave_done, c->d_wave_err, c->wave_items};
    if (c->precision == 64)
        CK(esm::launch_class_pass<double>(c->Md, c->d_steps[cls], ns, c->d_sweep, cls, limit, (double *)c->d_scratch,
                                          c->move_wpb, c->max_warps, c->d_stats, c->d_descs, c->d_item_ctr, sep,
                                          wave, c->stream));
    else
        CK(esm::launch_class_pass<float>(c->Mf, c->d_steps[cls], ns, c->d_sweep, cls, limit, (float *)c->d_scratch,
                                         c->move_wpb, c->max_warps, c->d_stats, c->d_descs, c->d_item_ctr, sep,
                                         wave, c->stream));
    return ESM_OK;
}

// the error flag of the whole-class launch: a wait that ran out leaves the pass incomplete
int wave_check(esm_ctx *c) {
    if (c->move_schedule != ESM_MOVES_PER_CLASS || !c->d_wave_err) return ESM_OK;
    int h = 0;
    CK(cudaMemcpy(&h, c->d_wave_err, sizeof(int), cudaMemcpyDeviceToHost));
    if (h) {
        CK(cudaMemset(c->d_wave_err, 0, sizeof(int)));
        return fail(c, ESM_ETIMEOUT, "a line move of the whole-class launch waited beyond its limit for the "
                                     "previous move of its item; the class pass is incomplete");
    }
    return ESM_OK;
}

// One colour class. A whole class (no move limit) runs as a CUDA graph captured at its first use:
// the per-move launches (a few hundred) then cost one graph launch; the sweep index is the only
// argument that changes and is written to the device first.
int class_pass_any(esm_ctx *c, uint32_t sweep, int cls, int limit = 0) {
    int ns = c->class_len[cls];
    if (ns == 0) return ESM_OK;
    Span sp(c, ESM_KT_CLASS);
    k_set_word<<<1, 1, 0, c->stream>>>(c->d_sweep, sweep);
    CK(cudaGetLastError());
    int nmoves = c->precision == 64 ? c->Md.natoms + c->Md.nextra : c->Mf.natoms + c->Mf.nextra;
    int nrun = limit > 0 && limit < nmoves ? limit : nmoves;
    c->launches += 2 + nrun;
    if (limit > 0) return class_pass_launch(c, cls, limit);
    if (!c->graph[cls]) {
        cudaGraph_t g = nullptr;
        CK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
        int rc = class_pass_launch(c, cls, 0);
        cudaError_t e = cudaStreamEndCapture(c->stream, &g);
        if (rc) {
            if (g) cudaGraphDestroy(g);
            return rc;
        }
        CK(e);
        e = cudaGraphInstantiate(&c->graph[cls], g, 0);
        cudaGraphDestroy(g);
        CK(e);
    }
    CK(cudaGraphLaunch(c->graph[cls], c->stream));
    return ESM_OK;
}

void class_order(const esm_ctx *c, uint32_t sweep, int order[3], int *ncls) {
    esm::class_order_of(c->seed, c->T, sweep, order, ncls);
}

int stats_out(esm_ctx *c, int64_t *stats) {
    if (!stats) return ESM_OK;
    unsigned long long h[2 * (ESM_NFAM + 1) + 1];
    CK(cudaMemcpyAsync(h, c->d_stats, sizeof h, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    for (int i = 0; i < 2 * (ESM_NFAM + 1) + 1; ++i) stats[i] += (int64_t)h[i];
    return wave_check(c);
}

}  // namespace

// =============================================================================================
extern "C" {

namespace {
int static_scores_setup(esm_ctx *c);
}

int esm_create(const esm_model *m, const esm_opts *o, esm_ctx **out) {
    if (!out) return ESM_EINVAL;
    *out = nullptr;
    if (!m || !o) return ESM_EINVAL;
    esm_ctx *c = new esm_ctx();
    *out = c;
    if (o->precision != 32 && o->precision != 64) return fail(c, ESM_EINVAL, "precision must be 32 or 64");
    if (o->R < 1 || m->N < 2 || m->T < 2 || m->K < 1) return fail(c, ESM_EINVAL, "bad sizes");
    if (o->max_points != 0 && o->max_points < 8) return fail(c, ESM_EINVAL, "max_points must be 0 (automatic) or >= 8");
    c->precision = o->precision;
    c->R = o->R;
    c->N = m->N;
    c->L = m->L;
    c->T = m->T;
    c->K = m->K;
    c->D = m->D;
    c->S = m->S;
    c->n0 = m->n0;
    c->nreg = m->nreg;
    c->dt = m->dt;
    c->gamma_k = m->gamma_k;
    c->beta_k = m->beta_k;
    c->beta_v = m->beta_v;
    c->kappa0 = m->kappa0;
    c->physical = m->physical;
    c->seed = o->seed;
    CK(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
    int rc = c->precision == 64 ? build_model<double>(c, m, o) : build_model<float>(c, m, o);
    if (rc) return rc;
    rc = c->precision == 64 ? alloc_state<double>(c) : alloc_state<float>(c);
    if (rc) return rc;
    if (c->precision == 32) {  // the FP64 model and state the capacity scores are computed on
        if ((rc = build_model<double>(c, m, o))) return rc;
        if ((rc = alloc_shadow(c))) return rc;
    }
    // storage multiscale sweep: the groups and the limits of its kernel
    c->storage_ms = o->storage_ms != 0;
    c->storage_long = o->storage_long != 0;
    c->stor.assign(m->stor, m->stor + m->S);
    c->ulo.assign(m->unit_lo, m->unit_lo + m->K);
    c->uhi.assign(m->unit_hi, m->unit_hi + m->K);
    c->uhours.assign(m->unit_hours, m->unit_hours + m->K);
    c->kappa_min = o->kappa_min;
    if ((rc = dalloc(c, &c->d_sl_plan, (size_t)std::max(m->S, 1) * ESM_SL_STRIDE))) return rc;
    if (m->nsgroups > 0 && m->sgroup_ptr && m->sgroup_units) {
        c->sgp.assign(m->sgroup_ptr, m->sgroup_ptr + m->nsgroups + 1);
        c->sgu.assign(m->sgroup_units, m->sgroup_units + c->sgp[m->nsgroups]);
    }
    for (size_t g = 0; g + 1 < c->sgp.size(); ++g)
        if (c->sgp[g + 1] - c->sgp[g] > ESM_PLAT_MAXU)
            return fail(c, ESM_EINVAL, "a storage group has more than %d units", ESM_PLAT_MAXU);
    for (int n = 0; n < m->N; ++n)
        if (m->units_ptr[n + 1] - m->units_ptr[n] > ESM_PLAT_MAXK)
            return fail(c, ESM_EINVAL, "a node has more than %d dispatchable units", ESM_PLAT_MAXK);
    // classes
    c->ncls = c->T % 2 ? 3 : 2;
    c->class_len.assign(3, 0);
    vector<int> st;
    for (int q = 0; q < c->ncls; ++q) {
        class_steps(c->T, q, st);
        c->class_len[q] = (int)st.size();
        if ((rc = upload(c, &c->d_steps[q], st.data(), st.size()))) return rc;
    }
    {  // the per-item progress words of the whole-class launch (k_move_wave) and its error flag
        int span = c->precision == 64 ? c->Md.span : c->Mf.span;
        size_t wpt = ((size_t)span * c->R + 31) / 32, mx = 1;
        for (int q = 0; q < c->ncls; ++q) mx = std::max(mx, (size_t)((c->class_len[q] + span - 1) / span) * wpt);
        if ((rc = dalloc(c, &c->d_wave_done, mx))) return rc;
        c->wave_items = mx;
        if ((rc = dalloc(c, &c->d_wave_err, 1))) return rc;
        CK(cudaMemset(c->d_wave_err, 0, sizeof(int)));
    }
    // unit tables (FP64)
    int K = c->K;
    vector<int> gidx(K, 0), cnt(64, 0);
    int ng = 0;
    for (int u = 0; u < K; ++u) {
        int gq = m->unit_group[u];
        if (gq < 0 || gq >= 64) return fail(c, ESM_EINVAL, "unit group out of range");
        gidx[u] = cnt[gq]++;
        ng = std::max(ng, gq + 1);
    }
    c->ngroups = ng;
    {  // the renewable units (their order is the kernels' renewable index) and their carriers
        std::vector<int> gmap(64, -1);
        int nc = 0;
        for (int u = 0; u < K; ++u)
            if (m->unit_kind[u] == ESM_UNIT_REN && gmap[m->unit_group[u]] < 0) gmap[m->unit_group[u]] = 0;
        for (int gq = 0; gq < 64; ++gq)
            if (gmap[gq] == 0) gmap[gq] = nc++;
        c->car_units.assign(nc, 0);
        for (int u = 0; u < K; ++u)
            if (m->unit_kind[u] == ESM_UNIT_REN) {
                c->ren_unit.push_back(u);
                c->ren_car.push_back(gmap[m->unit_group[u]]);
                c->car_units[gmap[m->unit_group[u]]] += 1;
            }
    }
    vector<int> uloc(K, -1);
    {
        int nr = 0;
        for (int u = 0; u < K; ++u)
            if (m->unit_kind[u] == ESM_UNIT_REN) uloc[u] = nr++;
        for (int j = 0; j < m->D; ++j) uloc[m->disp[j]] = j;
        for (int j = 0; j < m->S; ++j) uloc[m->stor[j]] = j;
    }
    if ((rc = upload(c, &c->d_disp, m->disp, m->D))) return rc;
    if ((rc = upload(c, &c->d_ugroup, m->unit_group, K))) return rc;
    if ((rc = upload(c, &c->d_ugidx, gidx.data(), K))) return rc;
    if ((rc = upload(c, &c->d_ukind, m->unit_kind, K))) return rc;
    if ((rc = upload(c, &c->d_uloc, uloc.data(), K))) return rc;
    if ((rc = upload(c, &c->d_lo, m->unit_lo, K))) return rc;
    if ((rc = upload(c, &c->d_hi, m->unit_hi, K))) return rc;
    if ((rc = upload(c, &c->d_capex, m->unit_capex, K))) return rc;
    double *dp;
    for (double **pp : {&c->d_k, &c->d_kold, &c->d_knew, &c->d_k1, &c->d_kmid, &c->d_fk, &c->d_xi}) {
        if ((rc = dalloc(c, &dp, K))) return rc;
        *pp = dp;
    }
    if ((rc = dalloc(c, &c->d_score_part, esm::score_partial_doubles(c->T, c->R, c->K, c->N)))) return rc;
    for (double **pp : {&c->d_sk, &c->d_sk_err}) {
        if ((rc = dalloc(c, &dp, (size_t)c->R * K))) return rc;
        *pp = dp;
    }
    if ((rc = dalloc(c, &c->d_sums, esm::score_sum_doubles(c->R, K)))) return rc;
    if ((rc = dalloc(c, &c->d_w, c->R))) return rc;
    if ((rc = dalloc(c, &c->d_eta, 64))) return rc;
    if ((rc = dalloc(c, &c->d_kappa, 64))) return rc;
    if ((rc = dalloc(c, &c->d_nclip, 1))) return rc;
    if ((rc = dalloc(c, &c->d_stats, 2 * (ESM_NFAM + 1) + 1))) return rc;
    if ((rc = dalloc(c, &c->d_reg, (size_t)c->T * c->R))) return rc;
    if ((rc = dalloc(c, &c->d_reg2, (size_t)c->T * c->R))) return rc;
    // weather prior (FP64)
    size_t n0 = m->n0, nr = m->nreg;
    if ((rc = upload(c, &c->d_phi, m->phi, nr * n0))) return rc;
    if ((rc = upload(c, &c->d_mu, m->mu, nr * n0 * 3))) return rc;
    if ((rc = upload(c, &c->d_sig, m->sig, nr * n0))) return rc;
    if ((rc = upload(c, &c->d_sig0, m->sig0, n0))) return rc;
    if ((rc = dalloc(c, &c->d_season, 2 * (size_t)c->T))) return rc;
    esm::k_season<<<(c->T + 255) / 256, 256, 0, c->stream>>>(c->T, c->d_season);
    CK(cudaGetLastError());
    if ((rc = upload(c, &c->d_Ptr, m->Ptr, nr * nr))) return rc;
    if ((rc = upload(c, &c->d_pi0, m->pi0, nr))) return rc;
    if ((rc = dalloc(c, &c->d_wbeta, (size_t)c->R * nr * c->T))) return rc;
    if ((rc = dalloc(c, &c->d_wtheta, c->R))) return rc;
    if ((rc = dalloc(c, &c->d_moved, c->R))) return rc;
    if ((rc = dalloc(c, &c->d_window, c->R))) return rc;
    if ((rc = dalloc(c, &c->d_wstart, c->R))) return rc;
    if ((rc = dalloc(c, &c->d_wflag, c->R))) return rc;
    {
        size_t rbytes = (c->precision == 64 ? sizeof(double) : sizeof(float)) * (size_t)c->N * c->T * c->R;
        char *q;
        if ((rc = dalloc(c, &q, rbytes))) return rc;
        c->d_r0 = q;
    }
    CK(cudaStreamSynchronize(c->stream));
    if (o->probe) {  // the lag probe's one-replica context, with its own streams
        esm_opts po = *o;
        po.R = 1;
        po.span = 0;
        po.probe = 0;
        po.seed = esm_probe_seed(o->seed);
        int prc = esm_create(m, &po, &c->probe);
        if (prc) {
            std::string msg = c->probe ? esm_last_error(c->probe) : "";
            return fail(c, prc, "probe context: %s", msg.c_str());
        }
    }
    if ((rc = static_scores_setup(c))) return rc;
    return ESM_OK;
}

int esm_destroy(esm_ctx *c) {
    if (!c) return ESM_OK;
    if (c->stream) cudaStreamSynchronize(c->stream);
    for (auto &mk : c->marks) {
        cudaEventDestroy(mk.a);
        cudaEventDestroy(mk.b);
    }
    for (cudaEvent_t e : c->pool) cudaEventDestroy(e);
    for (auto &g : c->graph)
        if (g) cudaGraphExecDestroy(g);
    for (void *p : c->allocs) cudaFree(p);
    if (c->stream) cudaStreamDestroy(c->stream);
    if (c->probe) esm_destroy(c->probe);
    delete c->snap;
    delete c;
    return ESM_OK;
}

const char *esm_last_error(const esm_ctx *c) { return c ? c->err.c_str() : "no context"; }

int esm_upload_state(esm_ctx *c, const double *theta, const double *g, const double *e, const double *z,
                     const int32_t *reg, const double *k) {
    if (!c) return ESM_EINVAL;
    size_t TR = (size_t)c->T * c->R;
    int rc;
    bool f64 = c->precision == 64;
    rc = f64 ? up_state<double>(c, c->theta, theta, c->N * TR) : up_state<float>(c, c->theta, theta, c->N * TR);
    if (rc) return rc;
    rc = f64 ? up_state<double>(c, c->g, g, c->D * TR) : up_state<float>(c, c->g, g, c->D * TR);
    if (rc) return rc;
    rc = f64 ? up_state<double>(c, c->e, e, c->S * TR) : up_state<float>(c, c->e, e, c->S * TR);
    if (rc) return rc;
    rc = f64 ? up_state<double>(c, c->z, z, c->n0 * TR) : up_state<float>(c, c->z, z, c->n0 * TR);
    if (rc) return rc;
    if (reg) CK(cudaMemcpy(c->d_reg, reg, sizeof(int32_t) * TR, cudaMemcpyHostToDevice));
    if (k) {
        CK(cudaMemcpy(c->d_k, k, sizeof(double) * c->K, cudaMemcpyHostToDevice));
        if ((rc = set_kc_any(c, c->d_k))) return rc;
    }
    c->has_state = true;
    c->has_scores = false;
    CK(cudaStreamSynchronize(c->stream));
    return ESM_OK;
}

int esm_download_state(esm_ctx *c, double *theta, double *g, double *e, double *z, int32_t *reg, double *k) {
    if (!c) return ESM_EINVAL;
    size_t TR = (size_t)c->T * c->R;
    bool f64 = c->precision == 64;
    int rc;
    rc = f64 ? down_state<double>(c, c->theta, theta, c->N * TR) : down_state<float>(c, c->theta, theta, c->N * TR);
    if (rc) return rc;
    rc = f64 ? down_state<double>(c, c->g, g, c->D * TR) : down_state<float>(c, c->g, g, c->D * TR);
    if (rc) return rc;
    rc = f64 ? down_state<double>(c, c->e, e, c->S * TR) : down_state<float>(c, c->e, e, c->S * TR);
    if (rc) return rc;
    rc = f64 ? down_state<double>(c, c->z, z, c->n0 * TR) : down_state<float>(c, c->z, z, c->n0 * TR);
    if (rc) return rc;
    if (reg) CK(cudaMemcpy(reg, c->d_reg, sizeof(int32_t) * TR, cudaMemcpyDeviceToHost));
    if (k) CK(cudaMemcpy(k, c->d_k, sizeof(double) * c->K, cudaMemcpyDeviceToHost));
    return ESM_OK;
}

int esm_rebuild_caches(esm_ctx *c) {
    if (!c) return ESM_EINVAL;
    if (!c->has_state) return fail(c, ESM_ESTATE, "no state uploaded");
    return rebuild_any(c);
}

int esm_download_caches(esm_ctx *c, double *r, double *F) {
    if (!c) return ESM_EINVAL;
    size_t TR = (size_t)c->T * c->R;
    bool f64 = c->precision == 64;
    int rc = f64 ? down_state<double>(c, c->r, r, c->N * TR) : down_state<float>(c, c->r, r, c->N * TR);
    if (rc) return rc;
    return f64 ? down_state<double>(c, c->F, F, c->L * TR) : down_state<float>(c, c->F, F, c->L * TR);
}

int esm_class_pass(esm_ctx *c, int64_t sweep, int32_t cls, int32_t move_limit, int64_t *stats) {
    if (!c) return ESM_EINVAL;
    if (!c->has_state) return fail(c, ESM_ESTATE, "no state uploaded");
    if (cls < 0 || cls >= c->ncls) return fail(c, ESM_EINVAL, "class %d out of range", cls);
    CK(cudaMemsetAsync(c->d_stats, 0, sizeof(unsigned long long) * (2 * (ESM_NFAM + 1) + 1), c->stream));
    double *mlog = c->precision == 64 ? c->Md.mlog : c->Mf.mlog;
    if (mlog) {  // entries of moves that made no move (and beyond the limit) read NaN
        size_t nmoves = c->precision == 64 ? c->Md.natoms + c->Md.nextra : c->Mf.natoms + c->Mf.nextra;
        CK(cudaMemsetAsync(mlog, 0xff, sizeof(double) * nmoves * c->class_len[cls] * c->Md.mlog_nrep, c->stream));
    }
    int rc = class_pass_any(c, (uint32_t)sweep, cls, move_limit);
    if (rc) return rc;
    c->has_scores = false;
    return stats_out(c, stats);
}

namespace {
// sequential uniforms of one Philox stream (the oracle's PStream)
struct HStream {
    uint64_t seed;
    uint32_t tag, w1, w2, w3, j = 0;
    double next() {
        double u0, u1;
        esm::uniform2(seed, tag, j >> 1, w1, w2, w3, &u0, &u1);
        double u = (j & 1) ? u1 : u0;
        ++j;
        return u;
    }
    int pick(int n) {
        int i = (int)floor(next() * n);
        return i >= n ? n - 1 : i;
    }
};

// The class passes of the storage multiscale sweep of one operation sweep (storage_ms_sweep!,
// src/flowmoves.jl:255): its coin (probability 1/2, operation_sweep!, src/local.jl:2417; skipped
// with force), the lengths 2 .. 128 below T/2 in random order, per length a random offset and the
// order of the two block parities; then the 8 move selections of every pass (a cell-class aggregate
// with probability 1/2, else one unit). The oracle draws the same streams.
int sms_plan(const esm_ctx *c, uint32_t sweep, bool force, std::vector<esm::PlatMoves> &out) {
    out.clear();
    HStream st{c->seed, ESM_TAG_SMS, 0u, 0u, sweep};
    bool run = st.next() < 0.5;
    if ((!run && !force) || c->S == 0) return 0;
    int lens[7], nl = 0;
    for (int L = 2; L <= 128; L *= 2)
        if (L < c->T / 2) lens[nl++] = L;
    for (int i = nl - 1; i >= 1; --i) std::swap(lens[i], lens[st.pick(i + 1)]);
    int ng = (int)c->sgp.size() - 1;
    for (int q = 0; q < nl; ++q) {
        int L = lens[q];
        int o = st.pick(L);
        bool swap01 = st.next() >= 0.5;
        int nb = 0;
        for (int b0 = o; b0 + L <= c->T - 1; b0 += L) ++nb;
        if (nb < 2) continue;
        int li = 0;
        while ((2 << li) < L) ++li;
        for (int h = 0; h < 2; ++h) {
            esm::PlatMoves mv{};
            mv.L = L;
            mv.o = o;
            mv.cls = swap01 ? 1 - h : h;
            mv.li = li;
            mv.nb = (nb - mv.cls + 1) / 2;
            HStream ms{c->seed, ESM_TAG_SMS, 1u + (uint32_t)li, 2u + (uint32_t)mv.cls, sweep};
            for (int k = 0; k < 8; ++k) {
                if (ms.next() < 0.5 && ng > 0) {
                    int gi = ms.pick(ng);
                    mv.nu[k] = c->sgp[gi + 1] - c->sgp[gi];
                    for (int p = 0; p < mv.nu[k]; ++p) mv.j[k][p] = c->sgu[c->sgp[gi] + p];
                } else {
                    mv.nu[k] = 1;
                    mv.j[k][0] = ms.pick(c->S);
                }
            }
            out.push_back(mv);
        }
    }
    return (int)out.size();
}

// the storage kernels' global scratch (layouts beyond the local arrays only), at their first use:
// at most 256 MB, the grid capped to the threads it holds
int sms_scratch(esm_ctx *c) {
    if (c->sms_per == 0 || c->d_sms_scratch) return ESM_OK;
    size_t rb = c->precision == 64 ? sizeof(double) : sizeof(float);
    size_t fit = ((size_t)256 << 20) / (c->sms_per * rb);
    int thr = (int)std::min((size_t)c->sms_threads, std::max((size_t)128, fit / 128 * 128));
    char *q;
    int rc = dalloc(c, &q, c->sms_per * rb * (size_t)thr);
    if (rc) return rc;
    c->d_sms_scratch = q;
    c->sms_threads = thr;
    return ESM_OK;
}

// the storage multiscale sweep of one operation sweep: caches rebuilt (LocalCost at the start of
// storage_ms_sweep!, src/flowmoves.jl:261), then one launch per class pass
int sms_sweep_any(esm_ctx *c, uint32_t sweep, bool force, int max_passes = 0) {
    std::vector<esm::PlatMoves> plan;
    if (sms_plan(c, sweep, force, plan) == 0) return ESM_OK;
    if (max_passes > 0 && (size_t)max_passes < plan.size()) plan.resize(max_passes);
    int rc = sms_scratch(c);
    if (rc) return rc;
    if ((rc = rebuild_any(c))) return rc;
    if (rc) return rc;
    Span sp(c, ESM_KT_STORAGE);
    for (auto &mv : plan) {
        if (c->precision == 64)
            CK(esm::launch_plateau<double>(c->Md, mv, sweep, (double *)c->d_sms_scratch, c->sms_threads,
                                           c->d_sms_stats, c->stream));
        else
            CK(esm::launch_plateau<float>(c->Mf, mv, sweep, (float *)c->d_sms_scratch, c->sms_threads,
                                          c->d_sms_stats, c->stream));
        c->launches += 1;
    }
    return ESM_OK;
}
// The long-range storage sweep's plan (storage_long_sweep!, src/storage_long.jl:245): the storage
// units with at least 24 h of storage and kappa_s >= kappa_min, each with the level move (p_level
// = 1) and 4 long-range plateaus of length uniform on 1 .. T-1, in random order, each with a start
// uniform on the year. The oracle draws the same streams.
int sl_plan(esm_ctx *c, uint32_t sweep, std::vector<int> &plan) {
    plan.clear();
    std::vector<double> k(c->K);
    CK(cudaMemcpyAsync(k.data(), c->d_k, sizeof(double) * c->K, cudaMemcpyDeviceToHost, c->stream));
    int rc = esm_sync(c, 600.0);
    if (rc) return rc;
    int T = c->T;
    for (int j = 0; j < c->S; ++j) {
        int u = c->stor[j];
        double kc = std::min(std::max(k[u], c->ulo[u]), c->uhi[u]);
        if (!(c->uhours[u] >= 24.0 && kc * c->uhours[u] / c->dt >= c->kappa_min)) continue;
        HStream st{c->seed, ESM_TAG_SLG, (uint32_t)j, 0u, sweep};
        int L[5], a[5], n = 0;
        if (st.next() < 1.0) L[n++] = T;
        for (int q = 0; q < 4; ++q) L[n++] = 1 + st.pick(T - 1);
        for (int i = n - 1; i >= 1; --i) std::swap(L[i], L[st.pick(i + 1)]);
        for (int i = 0; i < n; ++i) a[i] = st.pick(T);
        plan.push_back(j);
        plan.push_back(n);
        for (int i = 0; i < 5; ++i) {
            plan.push_back(i < n ? L[i] : 0);
            plan.push_back(i < n ? a[i] : 0);
        }
    }
    return ESM_OK;
}

int sl_sweep_any(esm_ctx *c, uint32_t sweep) {
    std::vector<int> plan;
    int rc = sl_plan(c, sweep, plan);
    if (rc) return rc;
    int nu = (int)plan.size() / ESM_SL_STRIDE;
    if (nu == 0) return ESM_OK;
    if ((rc = sms_scratch(c))) return rc;
    if ((rc = rebuild_any(c))) return rc;  // LocalCost at the start (src/storage_long.jl:250)
    CK(cudaMemcpyAsync(c->d_sl_plan, plan.data(), sizeof(int) * plan.size(), cudaMemcpyHostToDevice, c->stream));
    c->sl_nunits = nu;
    double *mlog = c->precision == 64 ? c->Md.mlog : c->Mf.mlog;
    if (mlog) CK(cudaMemsetAsync(mlog, 0xff, sizeof(double) * nu * 5 * c->Md.mlog_nrep, c->stream));
    Span sp(c, ESM_KT_STORAGE);
    if (c->precision == 64)
        CK(esm::launch_storage_long<double>(c->Md, c->d_sl_plan, nu, sweep, (double *)c->d_sms_scratch, c->sms_threads,
                                            c->d_sms_stats, c->stream));
    else
        CK(esm::launch_storage_long<float>(c->Mf, c->d_sl_plan, nu, sweep, (float *)c->d_sms_scratch, c->sms_threads,
                                           c->d_sms_stats, c->stream));
    c->launches += 1;
    return esm_sync(c, 600.0);  // (the host plan buffer is reused by the next call)
}
}  // namespace

int esm_storage_long(esm_ctx *c, int64_t sweep, int64_t *stats) {
    if (!c) return ESM_EINVAL;
    if (!c->has_state) return fail(c, ESM_ESTATE, "no state uploaded");
    CK(cudaMemsetAsync(c->d_sms_stats, 0, sizeof(unsigned long long) * 3, c->stream));
    int rc = sl_sweep_any(c, (uint32_t)sweep);
    if (rc) return rc;
    c->has_scores = false;
    if (stats) {
        unsigned long long h[3];
        CK(cudaMemcpyAsync(h, c->d_sms_stats, sizeof h, cudaMemcpyDeviceToHost, c->stream));
        if ((rc = esm_sync(c, 600.0))) return rc;
        for (int i = 0; i < 3; ++i) stats[i] += (int64_t)h[i];
    }
    return ESM_OK;
}

int esm_storage_ms(esm_ctx *c, int64_t sweep, int32_t force, int32_t max_passes, int64_t *stats) {
    if (!c) return ESM_EINVAL;
    if (!c->has_state) return fail(c, ESM_ESTATE, "no state uploaded");
    CK(cudaMemsetAsync(c->d_sms_stats, 0, sizeof(unsigned long long) * 3, c->stream));
    int rc = sms_sweep_any(c, (uint32_t)sweep, force != 0, max_passes);
    if (rc) return rc;
    c->has_scores = false;
    if (stats) {
        unsigned long long h[3];
        CK(cudaMemcpyAsync(h, c->d_sms_stats, sizeof h, cudaMemcpyDeviceToHost, c->stream));
        if ((rc = esm_sync(c, 600.0))) return rc;
        for (int i = 0; i < 3; ++i) stats[i] += (int64_t)h[i];
    }
    return ESM_OK;
}

int esm_operation_sweeps(esm_ctx *c, int32_t n, int64_t sweep0, int64_t *stats) {
    if (!c) return ESM_EINVAL;
    if (!c->has_state) return fail(c, ESM_ESTATE, "no state uploaded");
    CK(cudaMemsetAsync(c->d_stats, 0, sizeof(unsigned long long) * (2 * (ESM_NFAM + 1) + 1), c->stream));
    for (int s = 0; s < n; ++s) {
        uint32_t sw = (uint32_t)(sweep0 + s);
        int rc = rebuild_any(c);
        if (rc) return rc;
        int order[3], nc;
        class_order(c, sw, order, &nc);
        for (int q = 0; q < nc; ++q)
            if ((rc = class_pass_any(c, sw, order[q]))) return rc;
        if (c->storage_ms && (rc = sms_sweep_any(c, sw, false))) return rc;
        if (c->storage_long && (rc = sl_sweep_any(c, sw))) return rc;
    }
    c->has_scores = false;
    return stats_out(c, stats);
}

int esm_capacity_scores(esm_ctx *c, double *sk, double *fk, double *parts) {
    if (!c) return ESM_EINVAL;
    if (!c->has_state) return fail(c, ESM_ESTATE, "no state uploaded");
    int rc = scores_any(c, c->d_score_part, c->d_sums);
    if (rc) return rc;
    if (sk) CK(cudaMemcpyAsync(sk, c->d_sk, sizeof(double) * c->R * c->K, cudaMemcpyDeviceToHost, c->stream));
    if (fk) CK(cudaMemcpyAsync(fk, c->d_fk, sizeof(double) * c->K, cudaMemcpyDeviceToHost, c->stream));
    if (parts)
        CK(cudaMemcpyAsync(parts, c->d_sums + (size_t)c->R * c->K, sizeof(double) * c->R * 8, cudaMemcpyDeviceToHost,
                           c->stream));
    CK(cudaStreamSynchronize(c->stream));
    c->has_scores = true;
    return ESM_OK;
}

int esm_score_errors(esm_ctx *c, double *sk_err, double *parts_err) {
    if (!c) return ESM_EINVAL;
    if (!c->has_scores || !c->last_sums) return fail(c, ESM_ESTATE, "no scores computed since the last state change");
    size_t RK = (size_t)c->R * c->K;
    if (sk_err) CK(cudaMemcpyAsync(sk_err, c->d_sk_err, sizeof(double) * RK, cudaMemcpyDeviceToHost, c->stream));
    if (parts_err)
        CK(cudaMemcpyAsync(parts_err, c->last_sums + 2 * RK + (size_t)c->R * 8, sizeof(double) * c->R * 8,
                           cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return ESM_OK;
}

// follow_capacities! (src/replicas.jl:448) from d_k to d_knew: the dispatchable units at fixed
// output, rebuild, the kop curve, rebuild; d_k becomes the followed capacities
int follow_any(esm_ctx *c, double kappa_min) {
    int K = c->K, rc;
    {
    Span sp(c, ESM_KT_LANGEVIN);
    CK(cudaMemcpyAsync(c->d_kold, c->d_k, sizeof(double) * K, cudaMemcpyDeviceToDevice, c->stream));
    if (c->precision == 64)
        CK(esm::launch_follow_disp<double>(c->Md, c->d_disp, c->d_kold, c->d_knew, c->d_lo, c->d_hi, c->stream));
    else
        CK(esm::launch_follow_disp<float>(c->Mf, c->d_disp, c->d_kold, c->d_knew, c->d_lo, c->d_hi, c->stream));
    k_mix<<<(K + 127) / 128, 128, 0, c->stream>>>(K, c->d_ukind, c->d_kold, c->d_knew, c->d_kmid);
    CK(cudaGetLastError());
    }
    if ((rc = set_kc_any(c, c->d_kmid))) return rc;
    if ((rc = rebuild_any(c))) return rc;
    {
    Span sp(c, ESM_KT_LANGEVIN);
    esm::k_kop_capacity<<<(K + 127) / 128, 128, 0, c->stream>>>(K, c->d_ukind, c->d_kold, c->d_knew, kappa_min,
                                                                 c->d_k1);
    CK(cudaGetLastError());
    if (c->precision == 64)
        CK(esm::launch_kop<double>(c->Md, c->d_kold, c->d_k1, c->d_lo, c->d_hi, kappa_min, c->stream));
    else
        CK(esm::launch_kop<float>(c->Mf, c->d_kold, c->d_k1, c->d_lo, c->d_hi, kappa_min, c->stream));
    }
    CK(cudaMemcpyAsync(c->d_k, c->d_k1, sizeof(double) * K, cudaMemcpyDeviceToDevice, c->stream));
    if ((rc = set_kc_any(c, c->d_k))) return rc;
    if ((rc = rebuild_any(c))) return rc;
    c->launches += 4;
    return ESM_OK;
}

// ---------------------------------------------------------------------------------------------
// Capacity scores whose call allocates nothing. For callers that must not allocate device memory
// in the call: a caller whose device memory is owned by a caching allocator (PyTorch's, a memory
// pool with a hard cap) -- cudaMalloc behind its back fails or fragments once the pool holds the
// device -- and a caller whose step must not stall, as cudaMalloc/cudaFree can synchronise the
// device. The score accumulators (the R x K score sums, the R x 8 cost parts and their bounds) live
// in one file-scope device array instead of buffers of the context.
//   Limit: the fused pass's chunk partials (esm::score_partial_doubles, which takes fewer chunks to
//   fit) and the 2 * R * (K + 8) sums within ESM_SCORE_SCRATCH_DOUBLES (8 MiB); larger contexts get
//   ESM_EINVAL.
//   Set-up: esm_create, which allocates anyway, resolves the array's address on the context's
//   device (cudaGetSymbolAddress, with that device current) and loads the score kernels, so the
//   call itself places nothing on the device. The call must be made with the context's device
//   current (else ESM_EINVAL). A cudaDeviceReset ends the contexts on that device, and with them
//   the addresses they hold.
//   The array is shared by every context on the device: overlapping calls (two streams, two
//   threads, two contexts) race on it and must be serialised by the caller.
// ---------------------------------------------------------------------------------------------
static __device__ __align__(256) double g_score_scratch[ESM_SCORE_SCRATCH_DOUBLES];

namespace {
// esm_create's set-up of the static score path: the context's device, the scratch array's address
// there, the kernels of the path loaded and the error buffer reserved
int static_scores_setup(esm_ctx *c) {
    CK(cudaGetDevice(&c->device));
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_score_scratch);
    if (e != cudaSuccess || !p)
        return fail(c, ESM_ECUDA, "cudaGetSymbolAddress of the score scratch: %s", cudaGetErrorString(e));
    c->score_scratch = (double *)p;
    CK(esm::preload_score_kernels());
    c->err.reserve(512);
    return ESM_OK;
}
}  // namespace

int esm_capacity_scores_static(esm_ctx *c, double *sk, double *fk, double *parts) {
    if (!c) return ESM_EINVAL;
    if (!c->has_state) return fail(c, ESM_ESTATE, "no state uploaded");
    size_t R = c->R, K = c->K;
    size_t npart = esm::score_partial_doubles(c->T, c->R, c->K, c->N), nsum = esm::score_sum_doubles(c->R, c->K);
    size_t need = npart + nsum;
    if (need > (size_t)ESM_SCORE_SCRATCH_DOUBLES)
        return fail(c, ESM_EINVAL, "%zu doubles of score scratch needed (2*R*(K+8) = %zu), the static scratch holds %d",
                    need, nsum, ESM_SCORE_SCRATCH_DOUBLES);
    int dev = -1, rc;
    CK(cudaGetDevice(&dev));
    if (dev != c->device || !c->score_scratch)
        return fail(c, ESM_EINVAL, "device %d is current, the context was created on device %d", dev, c->device);
    // the partials, then the summed gradient, the cost parts and their bounds; every element is
    // written by the pass before it is read, so nothing carries over from an earlier call
    double *part = c->score_scratch, *sums = part + npart, *pd = sums + R * K;
    if ((rc = scores_any(c, part, sums))) return rc;
    if (sk) CK(cudaMemcpyAsync(sk, c->d_sk, sizeof(double) * R * K, cudaMemcpyDeviceToHost, c->stream));
    if (fk) CK(cudaMemcpyAsync(fk, c->d_fk, sizeof(double) * K, cudaMemcpyDeviceToHost, c->stream));
    if (parts) CK(cudaMemcpyAsync(parts, pd, sizeof(double) * R * 8, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    c->has_scores = true;
    return ESM_OK;
}

int esm_langevin_step(esm_ctx *c, const double *w, const double *eta, const double *kappa_s, double kappa_min,
                      double clip, int32_t box, const double *xi, int64_t it, double *knew_out, int32_t *nclip_out) {
    if (!c) return ESM_EINVAL;
    if (!c->has_scores) return fail(c, ESM_ESTATE, "esm_capacity_scores must precede esm_langevin_step");
    if (!w || !eta || !kappa_s) return fail(c, ESM_EINVAL, "w, eta and kappa_s are required");
    int K = c->K, rc;
    CK(cudaMemcpyAsync(c->d_w, w, sizeof(double) * c->R, cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync(c->d_eta, eta, sizeof(double) * c->ngroups, cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync(c->d_kappa, kappa_s, sizeof(double) * c->ngroups, cudaMemcpyHostToDevice, c->stream));
    if (xi) CK(cudaMemcpyAsync(c->d_xi, xi, sizeof(double) * K, cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemsetAsync(c->d_nclip, 0, sizeof(int), c->stream));
    CK(cudaMemcpyAsync(c->d_kold, c->d_k, sizeof(double) * K, cudaMemcpyDeviceToDevice, c->stream));
    {
    Span sp(c, ESM_KT_LANGEVIN);
    esm::k_langevin<<<(K + 127) / 128, 128, 0, c->stream>>>(K, c->R, c->d_ugroup, c->d_ugidx, c->d_kold, c->d_sk,
                                                            c->d_fk, c->d_w, c->d_eta, c->d_kappa,
                                                            c->beta_k / c->beta_v, kappa_min, clip, box,
                                                            c->d_hi, xi ? c->d_xi : nullptr, c->seed, (uint32_t)it,
                                                            c->d_knew, c->d_nclip);
    CK(cudaGetLastError());
    }
    if ((rc = follow_any(c, kappa_min))) return rc;
    if (knew_out) CK(cudaMemcpyAsync(knew_out, c->d_k, sizeof(double) * K, cudaMemcpyDeviceToHost, c->stream));
    int nclip = 0;
    CK(cudaMemcpyAsync(&nclip, c->d_nclip, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    if (nclip_out) *nclip_out = nclip;
    c->has_scores = false;
    return ESM_OK;
}

int esm_weather_step(esm_ctx *c, const int32_t *moved, const double *theta, const int32_t *window,
                     const int32_t *wstart, const double *xi, int64_t it) {
    if (!c) return ESM_EINVAL;
    if (!c->has_state) return fail(c, ESM_ESTATE, "no state uploaded");
    if (!moved || !theta || !window || !wstart) return fail(c, ESM_EINVAL, "moved, theta, window, wstart are required");
    int R = c->R, rc;
    bool any = false, anyw = false, anyt = false;
    for (int r = 0; r < R; ++r) {
        any |= moved[r] != 0;
        anyw |= moved[r] && window[r] > 0;
        anyt |= moved[r] && theta[r] > 0;
    }
    if (!any) return ESM_OK;
    CK(cudaMemcpyAsync(c->d_moved, moved, sizeof(int) * R, cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync(c->d_wtheta, theta, sizeof(double) * R, cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync(c->d_window, window, sizeof(int) * R, cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync(c->d_wstart, wstart, sizeof(int) * R, cudaMemcpyHostToDevice, c->stream));
    vector<int> wflag(R);
    for (int r = 0; r < R; ++r) wflag[r] = moved[r] && window[r] > 0;
    CK(cudaMemcpyAsync(c->d_wflag, wflag.data(), sizeof(int) * R, cudaMemcpyHostToDevice, c->stream));
    const double *dxi = nullptr;
    if (xi) {
        size_t n = (size_t)R * c->n0 * c->T;
        if (!c->d_wxi && (rc = dalloc(c, &c->d_wxi, n))) return rc;
        CK(cudaMemcpyAsync(c->d_wxi, xi, sizeof(double) * n, cudaMemcpyHostToDevice, c->stream));
        dxi = c->d_wxi;
    }
    // residual before the change (compensate_weather!, src/replicas.jl:207 r0)
    if ((rc = rebuild_any(c))) return rc;
    size_t rbytes = (c->precision == 64 ? sizeof(double) : sizeof(float)) * (size_t)c->N * c->T * R;
    CK(cudaMemcpyAsync(c->d_r0, c->r, rbytes, cudaMemcpyDeviceToDevice, c->stream));
    {
    Span sp(c, ESM_KT_WEATHER);
    if (anyt) {  // pCN in the innovations at the current regimes
        if (c->precision == 64)
            CK(esm::launch_weather_z<double>(c->Md, c->d_phi, c->d_mu, c->d_season, c->d_sig, c->d_sig0, c->d_moved, c->d_wtheta,
                                             c->d_reg, c->d_reg, dxi, c->seed, (uint32_t)it, 1, c->stream));
        else
            CK(esm::launch_weather_z<float>(c->Mf, c->d_phi, c->d_mu, c->d_season, c->d_sig, c->d_sig0, c->d_moved, c->d_wtheta,
                                            c->d_reg, c->d_reg, dxi, c->seed, (uint32_t)it, 1, c->stream));
        c->launches += 1;
    }
    if (anyw) {  // regime window, then z rebuilt from its innovations at the new regimes
        esm::k_regime_window<<<(R + 63) / 64, 64, 0, c->stream>>>(c->T, R, c->nreg, c->d_Ptr, c->d_pi0, c->d_moved,
                                                                  c->d_window, c->d_wstart, c->d_reg, c->d_reg2,
                                                                  c->d_wbeta, c->seed, (uint32_t)it);
        CK(cudaGetLastError());
        if (c->precision == 64)
            CK(esm::launch_weather_z<double>(c->Md, c->d_phi, c->d_mu, c->d_season, c->d_sig, c->d_sig0, c->d_wflag, c->d_wtheta,
                                             c->d_reg, c->d_reg2, nullptr, c->seed, (uint32_t)it, 0, c->stream));
        else
            CK(esm::launch_weather_z<float>(c->Mf, c->d_phi, c->d_mu, c->d_season, c->d_sig, c->d_sig0, c->d_wflag, c->d_wtheta,
                                            c->d_reg, c->d_reg2, nullptr, c->seed, (uint32_t)it, 0, c->stream));
        CK(cudaMemcpyAsync(c->d_reg, c->d_reg2, sizeof(int32_t) * c->T * R, cudaMemcpyDeviceToDevice, c->stream));
        c->launches += 2;
    }
    }
    if ((rc = rebuild_any(c))) return rc;
    {
    Span sp(c, ESM_KT_WEATHER);
    if (c->precision == 64)
        CK(esm::launch_compensate<double>(c->Md, c->d_moved, (const double *)c->d_r0, c->stream));
    else
        CK(esm::launch_compensate<float>(c->Mf, c->d_moved, (const float *)c->d_r0, c->stream));
    }
    c->launches += 1;
    if ((rc = rebuild_any(c))) return rc;
    c->has_scores = false;
    CK(cudaStreamSynchronize(c->stream));
    return ESM_OK;
}

int esm_sync(esm_ctx *c, double timeout_s) {
    if (!c) return ESM_EINVAL;
    auto t0 = std::chrono::steady_clock::now();
    while (true) {
        cudaError_t e = cudaStreamQuery(c->stream);
        if (e == cudaSuccess) return wave_check(c);
        if (e != cudaErrorNotReady) return fail(c, ESM_ECUDA, "stream: %s", cudaGetErrorString(e));
        double el = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        if (el > timeout_s) return fail(c, ESM_ETIMEOUT, "stream not idle after %.1f s", timeout_s);
        std::this_thread::sleep_for(std::chrono::microseconds(200));
    }
}

int64_t esm_launch_count(const esm_ctx *c) { return c ? c->launches : 0; }

int esm_set_timing(esm_ctx *c, int32_t on) {
    if (!c) return ESM_EINVAL;
    CK(cudaStreamSynchronize(c->stream));
    for (auto &mk : c->marks) {
        c->pool.push_back(mk.a);
        c->pool.push_back(mk.b);
    }
    c->marks.clear();
    for (int i = 0; i < ESM_KT_N; ++i) c->acc_ms[i] = c->acc_n[i] = 0;
    c->timing = on != 0;
    return ESM_OK;
}

int esm_timing(esm_ctx *c, double *out) {
    if (!c || !out) return ESM_EINVAL;
    CK(cudaStreamSynchronize(c->stream));
    for (auto &mk : c->marks) {
        float ms = 0;
        CK(cudaEventElapsedTime(&ms, mk.a, mk.b));
        c->acc_ms[mk.kind] += ms;
        c->acc_n[mk.kind] += 1;
        c->pool.push_back(mk.a);
        c->pool.push_back(mk.b);
    }
    c->marks.clear();
    for (int i = 0; i < ESM_KT_N; ++i) {
        out[2 * i] = c->acc_ms[i];
        out[2 * i + 1] = c->acc_n[i];
        c->acc_ms[i] = c->acc_n[i] = 0;
    }
    return ESM_OK;
}

void *esm_stream(esm_ctx *c) { return c ? (void *)c->stream : nullptr; }

}  // extern "C"

// ---------------------------------------------------------------------------------------------
// delayed-acceptance support: capacities set to given values (with following), state snapshots,
// regime occupancy
// ---------------------------------------------------------------------------------------------
int esm_follow_capacities(esm_ctx *c, const double *knew, double kappa_min, double *k_out) {
    if (!c || !knew) return ESM_EINVAL;
    if (!c->has_state) return fail(c, ESM_ESTATE, "no state uploaded");
    CK(cudaMemcpyAsync(c->d_knew, knew, sizeof(double) * c->K, cudaMemcpyHostToDevice, c->stream));
    int rc = follow_any(c, kappa_min);
    if (rc) return rc;
    if (k_out) CK(cudaMemcpyAsync(k_out, c->d_k, sizeof(double) * c->K, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    c->has_scores = false;
    return ESM_OK;
}

namespace {
size_t state_bytes(const esm_ctx *c, int which) {
    size_t TR = (size_t)c->T * c->R, w = c->precision == 64 ? 8 : 4;
    switch (which) {
        case 0: return w * c->N * TR;
        case 1: return w * c->D * TR;
        case 2: return w * c->S * TR;
        default: return w * c->n0 * TR;
    }
}
int snap_copy(esm_ctx *c, bool save) {
    esm_snap &sn = *c->snap;
    void *live[4] = {c->theta, c->g, c->e, c->z};
    void *back[4] = {sn.theta, sn.g, sn.e, sn.z};
    for (int i = 0; i < 4; ++i) {
        size_t n = state_bytes(c, i);
        if (n) CK(cudaMemcpyAsync(save ? back[i] : live[i], save ? live[i] : back[i], n, cudaMemcpyDeviceToDevice,
                                  c->stream));
    }
    size_t TR = (size_t)c->T * c->R;
    CK(cudaMemcpyAsync(save ? sn.reg : c->d_reg, save ? c->d_reg : sn.reg, sizeof(int32_t) * TR,
                       cudaMemcpyDeviceToDevice, c->stream));
    CK(cudaMemcpyAsync(save ? sn.k : c->d_k, save ? c->d_k : sn.k, sizeof(double) * c->K, cudaMemcpyDeviceToDevice,
                       c->stream));
    return ESM_OK;
}
}  // namespace

int esm_state_save(esm_ctx *c) {
    if (!c) return ESM_EINVAL;
    if (!c->has_state) return fail(c, ESM_ESTATE, "no state uploaded");
    int rc;
    if (!c->snap) {
        esm_snap *sn = new esm_snap();
        c->snap = sn;
        char *p;
        for (int i = 0; i < 4; ++i) {
            if ((rc = dalloc(c, &p, std::max<size_t>(state_bytes(c, i), 1)))) return rc;
            (i == 0 ? sn->theta : i == 1 ? sn->g : i == 2 ? sn->e : sn->z) = p;
        }
        if ((rc = dalloc(c, &sn->reg, (size_t)c->T * c->R))) return rc;
        if ((rc = dalloc(c, &sn->k, (size_t)c->K))) return rc;
    }
    if ((rc = snap_copy(c, true))) return rc;
    c->has_snap = true;
    return ESM_OK;
}

int esm_state_restore(esm_ctx *c) {
    if (!c) return ESM_EINVAL;
    if (!c->has_snap) return fail(c, ESM_ESTATE, "no saved state");
    int rc = snap_copy(c, false);
    if (rc) return rc;
    if ((rc = set_kc_any(c, c->d_k))) return rc;
    if ((rc = rebuild_any(c))) return rc;
    CK(cudaStreamSynchronize(c->stream));
    c->has_scores = false;
    return ESM_OK;
}

namespace {
template <class T>
__global__ void k_gather_replica(const T *src, T *dst, size_t n, int R, int j) {
    size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i < n) dst[i] = src[i * R + j];
}
template <class T>
int gather_replica(esm_ctx *c, const void *src, void *dst, size_t n, int j) {
    if (n == 0) return ESM_OK;
    k_gather_replica<T><<<(unsigned)((n + 255) / 256), 256, 0, c->stream>>>((const T *)src, (T *)dst, n, c->R, j);
    CK(cudaGetLastError());
    return ESM_OK;
}
template <class real>
int probe_copy(esm_ctx *c, int j) {  // replica j of c into the probe context (its single replica)
    esm_ctx *p = c->probe;
    size_t T = (size_t)c->T;
    int rc;
    if ((rc = gather_replica<real>(c, c->theta, p->theta, c->N * T, j))) return rc;
    if ((rc = gather_replica<real>(c, c->g, p->g, c->D * T, j))) return rc;
    if ((rc = gather_replica<real>(c, c->e, p->e, c->S * T, j))) return rc;
    if ((rc = gather_replica<real>(c, c->z, p->z, c->n0 * T, j))) return rc;
    if ((rc = gather_replica<int32_t>(c, c->d_reg, p->d_reg, T, j))) return rc;
    CK(cudaMemcpyAsync(p->d_k, c->d_k, sizeof(double) * c->K, cudaMemcpyDeviceToDevice, c->stream));
    return esm_sync(c, 600.0);
}
}  // namespace

int esm_lag_probe(esm_ctx *c, int32_t j, int32_t nsweeps, int32_t tail, int64_t sweep0, double *sk_mean,
                  double *fk) {
    if (!c) return ESM_EINVAL;
    if (!c->probe) return fail(c, ESM_ESTATE, "no probe context (esm_opts.probe = 0)");
    if (!c->has_state) return fail(c, ESM_ESTATE, "no state uploaded");
    if (j < 0 || j >= c->R || nsweeps < 1 || tail < 1 || tail > nsweeps)
        return fail(c, ESM_EINVAL, "bad probe arguments");
    int rc = esm_sync(c, 600.0);
    if (rc) return rc;
    rc = c->precision == 64 ? probe_copy<double>(c, j) : probe_copy<float>(c, j);
    if (rc) return rc;
    esm_ctx *p = c->probe;
    if ((rc = set_kc_any(p, p->d_k))) return fail(c, rc, "probe: %s", p->err.c_str());
    p->has_state = true;
    p->has_scores = false;
    std::vector<double> sk(c->K), f(c->K);
    if (sk_mean) std::fill(sk_mean, sk_mean + c->K, 0.0);
    for (int q = 0; q < nsweeps; ++q) {
        if ((rc = esm_operation_sweeps(p, 1, sweep0 + q, nullptr))) return fail(c, rc, "probe: %s", p->err.c_str());
        if (q < nsweeps - tail) continue;
        if ((rc = esm_capacity_scores(p, sk.data(), f.data(), nullptr))) return fail(c, rc, "probe: %s", p->err.c_str());
        if (sk_mean)
            for (int i = 0; i < c->K; ++i) sk_mean[i] += sk[i] / tail;
    }
    if (fk) std::copy(f.begin(), f.end(), fk);
    return ESM_OK;
}

int esm_set_move_grid(esm_ctx *c, int32_t warps_per_block, int32_t warps_per_sm) {
    if (!c) return ESM_EINVAL;
    int wi = warps_per_block == 1 ? 0 : warps_per_block == 2 ? 1 : warps_per_block == 4 ? 2 : -1;
    if (wi < 0) return fail(c, ESM_EINVAL, "warps_per_block must be 1, 2 or 4");
    if (warps_per_sm < 0) return fail(c, ESM_EINVAL, "warps_per_sm must be >= 0");
    int cap = c->warps_cap[wi];
    int w = warps_per_sm == 0 ? cap : std::min(cap, std::max(4, warps_per_sm * c->nsm));
    if (w == c->max_warps && warps_per_block == c->move_wpb) return ESM_OK;
    int rc = esm_sync(c, 600.0);  // the captured class passes hold the old grid: drop them
    if (rc) return rc;
    if (c->scratch_warps > 0 && w > c->scratch_warps) {  // the global scratch grows to the grid
        size_t per = c->precision == 64 ? esm::linemove_scratch_reals<double>(c->Md) * sizeof(double)
                                        : esm::linemove_scratch_reals<float>(c->Mf) * sizeof(float);
        char *q;
        if ((rc = dalloc(c, &q, per * (size_t)w))) return rc;
        auto it = std::find(c->allocs.begin(), c->allocs.end(), c->d_scratch);
        if (it != c->allocs.end()) {
            cudaFree(*it);
            c->allocs.erase(it);
        }
        c->d_scratch = q;
        c->scratch_warps = w;
    }
    for (auto &g : c->graph)
        if (g) {
            CK(cudaGraphExecDestroy(g));
            g = nullptr;
        }
    c->move_wpb = warps_per_block;
    c->max_warps = w;
    return ESM_OK;
}

int esm_set_move_schedule(esm_ctx *c, int32_t schedule) {
    if (!c) return ESM_EINVAL;
    if (schedule != ESM_MOVES_PER_MOVE && schedule != ESM_MOVES_PER_CLASS)
        return fail(c, ESM_EINVAL, "schedule must be ESM_MOVES_PER_MOVE or ESM_MOVES_PER_CLASS");
    if (schedule == c->move_schedule) return ESM_OK;
    int rc = esm_sync(c, 600.0);  // the captured class passes hold the old schedule: drop them
    if (rc) return rc;
    for (auto &g : c->graph)
        if (g) {
            CK(cudaGraphExecDestroy(g));
            g = nullptr;
        }
    c->move_schedule = schedule;
    return ESM_OK;
}

int esm_move_schedule(const esm_ctx *c, int32_t *schedule) {
    if (!c || !schedule) return ESM_EINVAL;
    *schedule = c->move_schedule;
    return ESM_OK;
}

int esm_set_move_log(esm_ctx *c, int32_t nreps) {
    if (!c) return ESM_EINVAL;
    if (nreps < 0 || nreps > c->R) return fail(c, ESM_EINVAL, "nreps must be in 0 .. R");
    int rc = esm_sync(c, 600.0);  // the captured class passes hold the old setting: drop them
    if (rc) return rc;
    for (auto &g : c->graph)
        if (g) {
            CK(cudaGraphExecDestroy(g));
            g = nullptr;
        }
    double *p = nullptr;
    if (nreps > 0) {
        size_t nmoves = c->precision == 64 ? c->Md.natoms + c->Md.nextra : c->Mf.natoms + c->Mf.nextra;
        size_t ns = 0;
        for (int k = 0; k < c->ncls; ++k) ns = std::max(ns, (size_t)c->class_len[k]);
        if ((rc = dalloc(c, &p, nmoves * ns * (size_t)nreps))) return rc;
        CK(cudaMemsetAsync(p, 0xff, sizeof(double) * nmoves * ns * nreps, c->stream));
    }
    c->Mf.mlog = c->Md.mlog = p;
    c->Mf.mlog_nrep = c->Md.mlog_nrep = nreps;
    return ESM_OK;
}

int esm_move_log(esm_ctx *c, int32_t cls, double *out) {
    if (!c || !out) return ESM_EINVAL;
    if (!c->Md.mlog && !c->Mf.mlog) return fail(c, ESM_ESTATE, "the move log is off (esm_set_move_log)");
    if (cls < -1 || cls >= c->ncls) return fail(c, ESM_EINVAL, "class %d out of range", cls);
    size_t nmoves = c->precision == 64 ? c->Md.natoms + c->Md.nextra : c->Mf.natoms + c->Mf.nextra;
    size_t n = cls < 0 ? (size_t)c->sl_nunits * 5 * (size_t)c->Md.mlog_nrep
                       : nmoves * (size_t)c->class_len[cls] * (size_t)c->Md.mlog_nrep;
    double *src = c->precision == 64 ? c->Md.mlog : c->Mf.mlog;
    CK(cudaMemcpyAsync(out, src, sizeof(double) * n, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return ESM_OK;
}

int esm_set_sep_walk(esm_ctx *c, int32_t min_units) {
    if (!c) return ESM_EINVAL;
    if (min_units < 0) return fail(c, ESM_EINVAL, "min_units must be >= 0");
    if (min_units == c->sep_min) return ESM_OK;
    int rc = esm_sync(c, 600.0);  // the captured class passes hold the old choice: drop them
    if (rc) return rc;
    for (auto &g : c->graph)
        if (g) {
            CK(cudaGraphExecDestroy(g));
            g = nullptr;
        }
    c->sep_min = min_units;
    if (c->probe) return esm_set_sep_walk(c->probe, min_units);
    return ESM_OK;
}

int esm_sep_walk(const esm_ctx *c, int32_t *min_units, int32_t *warps) {
    if (!c) return ESM_EINVAL;
    if (min_units) *min_units = c->sep_min;
    if (warps) *warps = c->sep_max_warps;
    return ESM_OK;
}

int esm_move_grid(const esm_ctx *c, int32_t *warps_per_block, int32_t *warps_per_sm, int32_t *limits_per_sm) {
    if (!c || c->nsm < 1) return ESM_EINVAL;
    if (warps_per_block) *warps_per_block = c->move_wpb;
    if (warps_per_sm) *warps_per_sm = (c->max_warps + c->nsm - 1) / c->nsm;
    if (limits_per_sm)
        for (int i = 0; i < 3; ++i) limits_per_sm[i] = (c->warps_cap[i] + c->nsm - 1) / c->nsm;
    return ESM_OK;
}

int esm_autotune_moves(esm_ctx *c, int64_t sweep, int32_t *best, int32_t *cand, double *ms, int32_t *ncand) {
    if (!c) return ESM_EINVAL;
    if (!c->has_state) return fail(c, ESM_ESTATE, "no state uploaded");
    int list[ESM_TUNE_MAX][2], n = 0;
    for (int wi = 0; wi < 3; ++wi) {
        int lim = (c->warps_cap[wi] + c->nsm - 1) / c->nsm;
        for (int w : {8, 16, 24, 32, 40})
            if (w < lim && w % (1 << wi) == 0 && n < ESM_TUNE_MAX - 3 + wi) {
                list[n][0] = 1 << wi;
                list[n++][1] = w;
            }
        list[n][0] = 1 << wi;
        list[n++][1] = lim;
    }
    int rc;
    if ((rc = esm_state_save(c))) return rc;
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    int bw = c->move_wpb, bs = (c->max_warps + c->nsm - 1) / c->nsm;
    double tbest = 1e300;
    for (int i = 0; i < n && !rc; ++i) {
        if ((rc = esm_set_move_grid(c, list[i][0], list[i][1]))) break;
        // one untimed pass captures the class graph for this grid, then one timed pass from the same state
        if ((rc = class_pass_any(c, (uint32_t)sweep, 0))) break;
        if ((rc = esm_state_restore(c))) break;
        if (cudaEventRecord(e0, c->stream) != cudaSuccess) rc = fail(c, ESM_ECUDA, "event record");
        if (!rc) rc = class_pass_any(c, (uint32_t)sweep, 0);
        if (!rc && cudaEventRecord(e1, c->stream) != cudaSuccess) rc = fail(c, ESM_ECUDA, "event record");
        if (!rc) rc = esm_sync(c, 600.0);
        float t = 0;
        if (!rc && cudaEventElapsedTime(&t, e0, e1) != cudaSuccess) rc = fail(c, ESM_ECUDA, "event time");
        if (!rc) rc = esm_state_restore(c);
        if (rc) break;
        if (cand) {
            cand[2 * i] = list[i][0];
            cand[2 * i + 1] = list[i][1];
        }
        if (ms) ms[i] = t;
        if (t < tbest) {
            tbest = t;
            bw = list[i][0];
            bs = list[i][1];
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc) return rc;
    if (ncand) *ncand = n;
    if (best) {
        best[0] = bw;
        best[1] = bs;
    }
    return esm_set_move_grid(c, bw, bs);
}

namespace {
// occupancy of (regime, season) over the steps and replicas: season of 0-based step t with steps
// of h hours, season (src/weather.jl:50) on the 1-based step
__global__ void k_occupancy(int T, int R, int nreg, double h, const int32_t *reg, unsigned long long *cnt) {
    size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i >= (size_t)T * R) return;
    int t = (int)(i / R);
    long day = (long)((double)t * h / 24.0) + 1;
    int sea = (day >= 335 || day <= 59) ? 0 : day <= 151 ? 1 : day <= 243 ? 2 : 3;
    int k = reg[i];
    if (k >= 0 && k < nreg) atomicAdd(&cnt[k * 4 + sea], 1ull);
}
}  // namespace

int esm_replica_features(esm_ctx *c, const double *kref, double *out, int32_t *nfeat) {
    if (!c) return ESM_EINVAL;
    int C = (int)c->car_units.size(), nren = (int)c->ren_unit.size();
    int nf = 5 + C + c->nreg;
    if (nfeat) *nfeat = nf;
    if (!out) return ESM_OK;
    if (!kref) return fail(c, ESM_EINVAL, "kref is required");
    if (!c->has_state) return fail(c, ESM_ESTATE, "no state uploaded");
    int rc;
    size_t TR = (size_t)c->T * c->R;
    if (!c->d_wf_buf) {
        if ((rc = dalloc(c, &c->d_wf_kref, (size_t)std::max(nren, 1)))) return rc;
        if ((rc = dalloc(c, &c->d_wf_car, (size_t)std::max(nren, 1)))) return rc;
        if ((rc = dalloc(c, &c->d_wf_ncar, (size_t)std::max(C, 1)))) return rc;
        if ((rc = dalloc(c, &c->d_wf_buf, (size_t)(2 + C) * TR))) return rc;
        if ((rc = dalloc(c, &c->d_wf_out, (size_t)c->R * nf))) return rc;
        if (nren) CK(cudaMemcpy(c->d_wf_car, c->ren_car.data(), sizeof(int) * nren, cudaMemcpyHostToDevice));
        if (C) CK(cudaMemcpy(c->d_wf_ncar, c->car_units.data(), sizeof(int) * C, cudaMemcpyHostToDevice));
    }
    std::vector<double> kr(std::max(nren, 1), 0.0);
    for (int j = 0; j < nren; ++j) kr[j] = kref[c->ren_unit[j]];
    CK(cudaMemcpyAsync(c->d_wf_kref, kr.data(), sizeof(double) * kr.size(), cudaMemcpyHostToDevice, c->stream));
    if (c->precision == 64)
        CK(esm::launch_weather_features<double>(c->Md, c->d_wf_kref, c->d_wf_car, C, c->d_wf_ncar, c->d_reg, c->d_wf_buf,
                                                c->d_wf_out, c->stream));
    else
        CK(esm::launch_weather_features<float>(c->Mf, c->d_wf_kref, c->d_wf_car, C, c->d_wf_ncar, c->d_reg, c->d_wf_buf,
                                               c->d_wf_out, c->stream));
    c->launches += 2;
    CK(cudaMemcpyAsync(out, c->d_wf_out, sizeof(double) * c->R * nf, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return ESM_OK;
}

int esm_regime_occupancy(esm_ctx *c, double *occ) {
    if (!c || !occ) return ESM_EINVAL;
    if (!c->has_state) return fail(c, ESM_ESTATE, "no state uploaded");
    int n = c->nreg * 4;
    if (!c->d_occ) {
        int rc = dalloc(c, &c->d_occ, (size_t)n);
        if (rc) return rc;
    }
    CK(cudaMemsetAsync(c->d_occ, 0, sizeof(unsigned long long) * n, c->stream));
    size_t TR = (size_t)c->T * c->R;
    k_occupancy<<<(unsigned)((TR + 255) / 256), 256, 0, c->stream>>>(c->T, c->R, c->nreg, c->dt, c->d_reg, c->d_occ);
    CK(cudaGetLastError());
    c->launches += 1;
    std::vector<unsigned long long> h(n);
    CK(cudaMemcpyAsync(h.data(), c->d_occ, sizeof(unsigned long long) * n, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    for (int i = 0; i < n; ++i) occ[i] = (double)h[i] / (double)TR;
    return ESM_OK;
}

// =============================================================================================
// A batch of chains whose operation sweeps run together (esm_batch_*)
// =============================================================================================
struct esm_batch {
    int n = 0, precision = 32;
    std::string err;
    std::vector<esm_ctx *> ctx;   // in launch order: decreasing move count
    std::vector<int> pos;         // pos[i]: the caller's index of ctx[i]
    cudaStream_t stream = nullptr;
    cudaEvent_t ev = nullptr, t0 = nullptr, t1 = nullptr;
    std::vector<int> nact;        // per move index: the models that have it
    esm::BatchLaunch bl{};
    void *d_models = nullptr;     // BatchModel<real>[n]
    uint32_t *d_sweep = nullptr;
    int nsm = 0, cap[2] = {0, 0};
    int scratch_warps = 0;        // warps the global walk slabs hold
    cudaGraphExec_t graph = nullptr;
    float last_ms = 0;
    int64_t launches = 0;         // kernels launched by the batch's sweeps
    std::vector<void *> allocs;
};

namespace {
int bfail(esm_batch *b, int code, const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    if (b) b->err = buf;
    return code;
}

#define BCK(call)                                                                                \
    do {                                                                                         \
        cudaError_t e_ = (call);                                                                 \
        if (e_ != cudaSuccess)                                                                   \
            return bfail(b, e_ == cudaErrorMemoryAllocation ? ESM_ENOMEM : ESM_ECUDA, "%s: %s (%s:%d)", #call, \
                         cudaGetErrorString(e_), __FILE__, __LINE__);                            \
    } while (0)

template <class T>
int balloc(esm_batch *b, T **p, size_t n) {
    void *q = nullptr;
    cudaError_t e = cudaMalloc(&q, sizeof(T) * (n ? n : 1));
    if (e != cudaSuccess) return bfail(b, ESM_ENOMEM, "cudaMalloc of %zu bytes: %s", sizeof(T) * n, cudaGetErrorString(e));
    b->allocs.push_back(q);
    *p = (T *)q;
    return ESM_OK;
}

template <class real>
const esm::DevModel<real> &ctx_model(const esm_ctx *c);
template <>
const esm::DevModel<float> &ctx_model<float>(const esm_ctx *c) { return c->Mf; }
template <>
const esm::DevModel<double> &ctx_model<double>(const esm_ctx *c) { return c->Md; }

// the batch's device tables, grid limits and walk slabs
template <class real>
int batch_setup(esm_batch *b) {
    int n = b->n, rc;
    std::vector<esm::BatchModel<real>> hm(n);
    size_t maxstride = 0, maxlane = 0;
    b->bl.maxpass = 0;
    for (int i = 0; i < n; ++i) {
        esm_ctx *c = b->ctx[i];
        esm::BatchModel<real> &m = hm[i];
        m.M = ctx_model<real>(c);
        m.M.mlog = nullptr;
        m.M.mlog_nrep = 0;
        for (int k = 0; k < 3; ++k) {
            m.steps[k] = c->d_steps[k];
            m.nsteps[k] = k < (int)c->class_len.size() ? c->class_len[k] : 0;
        }
        m.nmoves = m.M.natoms + m.M.nextra;
        m.descs = c->d_descs;
        m.stride = esm::linemove_smem_per_warp<real>(m.M);
        m.stats = c->d_stats;
        maxstride = std::max(maxstride, m.stride);
        maxlane = std::max(maxlane, esm::linemove_scratch_reals<real>(m.M));
        b->bl.maxpass = std::max(b->bl.maxpass, c->ncls);
    }
    if ((rc = balloc(b, (esm::BatchModel<real> **)&b->d_models, (size_t)n))) return rc;
    BCK(cudaMemcpy(b->d_models, hm.data(), sizeof(esm::BatchModel<real>) * n, cudaMemcpyHostToDevice));
    b->bl.nm = n;
    b->bl.maxmoves = hm[0].nmoves;
    b->bl.npass = b->bl.maxpass;
    b->bl.nmove = b->bl.maxmoves;
    b->nact.assign(b->bl.maxmoves, 0);
    for (int mi = 0; mi < b->bl.maxmoves; ++mi)
        while (b->nact[mi] < n && hm[b->nact[mi]].nmoves > mi) ++b->nact[mi];
    b->bl.nact = b->nact.data();
    b->bl.prep_smem = maxstride;
    int dev = 0;
    BCK(cudaGetDevice(&dev));
    BCK(cudaDeviceGetAttribute(&b->nsm, cudaDevAttrMultiProcessorCount, dev));
    for (int i = 0; i < 2; ++i) b->cap[i] = std::max(4, b->nsm * esm::batch_warps_per_sm<real>(1 << i));
    b->bl.wpb = 1;
    b->bl.warps = b->cap[0];
    b->bl.scratch_per_warp = maxlane;
    b->scratch_warps = 0;
    if (maxlane > 0) {  // slabs for the largest grid, at most 1 GB (never fewer than the one-warp limit)
        size_t fit = ((size_t)1 << 30) / (maxlane * sizeof(real));
        size_t w = std::max((size_t)b->cap[0], std::min((size_t)std::max(b->cap[0], b->cap[1]), fit));
        real *q;
        if ((rc = balloc(b, &q, maxlane * w))) return rc;
        b->bl.scratch = q;
        b->scratch_warps = (int)w;
    }
    if ((rc = balloc(b, &b->bl.pass_cls, (size_t)b->bl.maxpass * n))) return rc;
    if ((rc = balloc(b, &b->bl.off, (size_t)b->bl.maxpass * (n + 1)))) return rc;
    if ((rc = balloc(b, &b->bl.counters, (size_t)b->bl.maxpass * b->bl.maxmoves))) return rc;
    if ((rc = balloc(b, &b->d_sweep, 1))) return rc;
    return ESM_OK;
}

// the rebuilds of every chain, then its passes: all of them (a sweep), or the first npass passes
// with their first nmove moves each
template <class real>
int batch_record(esm_batch *b, int npass, int nmove) {
    for (esm_ctx *c : b->ctx) BCK(esm::launch_rebuild<real>(ctx_model<real>(c), b->stream));
    esm::BatchLaunch bl = b->bl;
    bl.npass = npass;
    bl.nmove = nmove;
    BCK(esm::launch_batch_passes<real>((const esm::BatchModel<real> *)b->d_models, bl, b->d_sweep, b->stream));
    return ESM_OK;
}

int batch_sweep(esm_batch *b, uint32_t sweep) {
    k_set_word<<<1, 1, 0, b->stream>>>(b->d_sweep, sweep);
    BCK(cudaGetLastError());
    if (!b->graph) {
        cudaGraph_t g = nullptr;
        BCK(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
        int np = b->bl.maxpass, nm = b->bl.maxmoves;
        int rc = b->precision == 64 ? batch_record<double>(b, np, nm) : batch_record<float>(b, np, nm);
        cudaError_t e = cudaStreamEndCapture(b->stream, &g);
        if (rc) {
            if (g) cudaGraphDestroy(g);
            return rc;
        }
        BCK(e);
        e = cudaGraphInstantiate(&b->graph, g, 0);
        cudaGraphDestroy(g);
        BCK(e);
    }
    BCK(cudaGraphLaunch(b->graph, b->stream));
    b->launches += 1 + b->n + b->bl.maxpass * (1 + b->bl.maxmoves);
    return ESM_OK;
}

int batch_wait(esm_batch *b, double timeout_s) {
    auto t0 = std::chrono::steady_clock::now();
    while (true) {
        cudaError_t e = cudaStreamQuery(b->stream);
        if (e == cudaSuccess) return ESM_OK;
        if (e != cudaErrorNotReady) return bfail(b, ESM_ECUDA, "stream: %s", cudaGetErrorString(e));
        double el = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        if (el > timeout_s) return bfail(b, ESM_ETIMEOUT, "batch stream not idle after %.1f s", timeout_s);
        std::this_thread::sleep_for(std::chrono::microseconds(200));
    }
}

// the batch stream after every context's work so far
int batch_join_in(esm_batch *b) {
    for (esm_ctx *c : b->ctx) {
        BCK(cudaEventRecord(b->ev, c->stream));
        BCK(cudaStreamWaitEvent(b->stream, b->ev, 0));
    }
    return ESM_OK;
}

// every context's later work after the batch's
int batch_join_out(esm_batch *b) {
    BCK(cudaEventRecord(b->ev, b->stream));
    for (esm_ctx *c : b->ctx) BCK(cudaStreamWaitEvent(c->stream, b->ev, 0));
    return ESM_OK;
}
}  // namespace

int esm_batch_create(esm_ctx *const *ctxs, int32_t n, esm_batch **out) {
    if (!out) return ESM_EINVAL;
    *out = nullptr;
    if (!ctxs || n < 1) return ESM_EINVAL;
    esm_batch *b = new esm_batch();
    *out = b;
    b->n = n;
    std::vector<int> idx(n);
    for (int i = 0; i < n; ++i) {
        esm_ctx *c = ctxs[i];
        if (!c) return bfail(b, ESM_EINVAL, "context %d is NULL", i);
        if (c->precision != ctxs[0]->precision) return bfail(b, ESM_EINVAL, "contexts of different precisions");
        if (c->storage_ms || c->storage_long) return bfail(b, ESM_EINVAL, "context %d has the storage sweeps on", i);
        for (int j = 0; j < i; ++j)
            if (ctxs[j] == c) return bfail(b, ESM_EINVAL, "context %d appears twice", i);
        idx[i] = i;
    }
    b->precision = ctxs[0]->precision;
    auto nmv = [&](int i) {
        const esm_ctx *c = ctxs[i];
        return c->precision == 64 ? c->Md.natoms + c->Md.nextra : c->Mf.natoms + c->Mf.nextra;
    };
    std::stable_sort(idx.begin(), idx.end(), [&](int a, int c) { return nmv(a) > nmv(c); });
    for (int i = 0; i < n; ++i) {
        b->ctx.push_back(ctxs[idx[i]]);
        b->pos.push_back(idx[i]);
    }
    BCK(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking));
    BCK(cudaEventCreateWithFlags(&b->ev, cudaEventDisableTiming));
    BCK(cudaEventCreate(&b->t0));
    BCK(cudaEventCreate(&b->t1));
    int rc = b->precision == 64 ? batch_setup<double>(b) : batch_setup<float>(b);
    if (rc) return rc;
    BCK(cudaDeviceSynchronize());
    return ESM_OK;
}

int esm_batch_destroy(esm_batch *b) {
    if (!b) return ESM_OK;
    if (b->stream) cudaStreamSynchronize(b->stream);
    if (b->graph) cudaGraphExecDestroy(b->graph);
    for (void *p : b->allocs) cudaFree(p);
    if (b->ev) cudaEventDestroy(b->ev);
    if (b->t0) cudaEventDestroy(b->t0);
    if (b->t1) cudaEventDestroy(b->t1);
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
    return ESM_OK;
}

const char *esm_batch_last_error(const esm_batch *b) { return b ? b->err.c_str() : "no batch"; }

int esm_batch_sweeps(esm_batch *b, int32_t n, int64_t sweep0, int64_t *stats) {
    if (!b) return ESM_EINVAL;
    if (n < 0) return bfail(b, ESM_EINVAL, "n must be >= 0");
    for (esm_ctx *c : b->ctx)
        if (!c->has_state) return bfail(b, ESM_ESTATE, "a context has no state uploaded");
    int rc;
    if ((rc = batch_join_in(b))) return rc;
    const size_t ns = 2 * (ESM_NFAM + 1) + 1;
    for (esm_ctx *c : b->ctx) BCK(cudaMemsetAsync(c->d_stats, 0, sizeof(unsigned long long) * ns, b->stream));
    BCK(cudaEventRecord(b->t0, b->stream));
    int rs = 0;
    for (int s = 0; s < n && !rs; ++s) rs = batch_sweep(b, (uint32_t)(sweep0 + s));
    if (!rs) BCK(cudaEventRecord(b->t1, b->stream));
    // the contexts' later work waits for what the batch enqueued, also after a failed sweep
    if ((rc = batch_join_out(b))) return rc;
    if (rs) return rs;
    for (esm_ctx *c : b->ctx) c->has_scores = false;
    if ((rc = batch_wait(b, 3600.0))) return rc;
    BCK(cudaEventElapsedTime(&b->last_ms, b->t0, b->t1));
    if (stats) {
        std::vector<unsigned long long> h(ns);
        for (int i = 0; i < b->n; ++i) {
            BCK(cudaMemcpy(h.data(), b->ctx[i]->d_stats, sizeof(unsigned long long) * ns, cudaMemcpyDeviceToHost));
            for (size_t k = 0; k < ns; ++k) stats[(size_t)b->pos[i] * ns + k] = (int64_t)h[k];
        }
    }
    return ESM_OK;
}

int esm_batch_set_grid(esm_batch *b, int32_t warps_per_block, int32_t warps_per_sm) {
    if (!b) return ESM_EINVAL;
    int wi = warps_per_block == 1 ? 0 : warps_per_block == 2 ? 1 : -1;
    if (wi < 0) return bfail(b, ESM_EINVAL, "warps_per_block must be 1 or 2");
    if (warps_per_sm < 0) return bfail(b, ESM_EINVAL, "warps_per_sm must be >= 0");
    int cap = b->cap[wi];
    int w = warps_per_sm == 0 ? cap : std::min(cap, std::max(4, warps_per_sm * b->nsm));
    if (b->scratch_warps > 0) w = std::min(w, b->scratch_warps);
    if (w == b->bl.warps && warps_per_block == b->bl.wpb) return ESM_OK;
    int rc = batch_wait(b, 600.0);  // the captured sweep holds the old grid: drop it
    if (rc) return rc;
    if (b->graph) {
        BCK(cudaGraphExecDestroy(b->graph));
        b->graph = nullptr;
    }
    b->bl.wpb = warps_per_block;
    b->bl.warps = w;
    return ESM_OK;
}

int esm_batch_grid(const esm_batch *b, int32_t *warps_per_block, int32_t *warps_per_sm, int32_t *limit_per_sm) {
    if (!b || b->nsm < 1) return ESM_EINVAL;
    if (warps_per_block) *warps_per_block = b->bl.wpb;
    if (warps_per_sm) *warps_per_sm = (b->bl.warps + b->nsm - 1) / b->nsm;
    if (limit_per_sm) *limit_per_sm = (b->cap[b->bl.wpb == 2 ? 1 : 0] + b->nsm - 1) / b->nsm;
    return ESM_OK;
}

int64_t esm_batch_launch_count(const esm_batch *b) { return b ? b->launches : 0; }

int esm_batch_time(const esm_batch *b, double *ms) {
    if (!b || !ms) return ESM_EINVAL;
    *ms = b->last_ms;
    return ESM_OK;
}

int esm_batch_autotune(esm_batch *b, int64_t sweep, int32_t *best, int32_t *cand, double *ms, int32_t *ncand) {
    if (!b) return ESM_EINVAL;
    for (esm_ctx *c : b->ctx)
        if (!c->has_state) return bfail(b, ESM_ESTATE, "a context has no state uploaded");
    int list[ESM_TUNE_MAX][2], n = 0;
    for (int wi = 0; wi < 2; ++wi) {
        int lim = (b->cap[wi] + b->nsm - 1) / b->nsm;
        for (int w : {8, 16, 24, 32})
            if (w < lim && w % (1 << wi) == 0 && n < ESM_TUNE_MAX - 2 + wi) {
                list[n][0] = 1 << wi;
                list[n++][1] = w;
            }
        list[n][0] = 1 << wi;
        list[n++][1] = lim;
    }
    int rc = 0;
    for (esm_ctx *c : b->ctx)
        if ((rc = esm_state_save(c))) return bfail(b, rc, "state save: %s", c->err.c_str());
    if ((rc = batch_join_in(b))) return rc;
    int bw = b->bl.wpb, bs = (b->bl.warps + b->nsm - 1) / b->nsm;
    int nmove = std::min(b->bl.maxmoves, ESM_BATCH_TUNE_MOVES);
    double tbest = 1e300;
    for (int i = 0; i < n && !rc; ++i) {
        if ((rc = esm_batch_set_grid(b, list[i][0], list[i][1]))) break;
        float t = 0;
        for (int rep = 0; rep < 2 && !rc; ++rep) {  // the first run loads and warms, the second is timed
            k_set_word<<<1, 1, 0, b->stream>>>(b->d_sweep, (uint32_t)sweep);
            if (cudaGetLastError() != cudaSuccess) rc = bfail(b, ESM_ECUDA, "launch");
            if (!rc && cudaEventRecord(b->t0, b->stream) != cudaSuccess) rc = bfail(b, ESM_ECUDA, "event record");
            if (!rc) rc = b->precision == 64 ? batch_record<double>(b, 1, nmove) : batch_record<float>(b, 1, nmove);
            if (!rc && cudaEventRecord(b->t1, b->stream) != cudaSuccess) rc = bfail(b, ESM_ECUDA, "event record");
            if (!rc) rc = batch_wait(b, 600.0);
            if (!rc && cudaEventElapsedTime(&t, b->t0, b->t1) != cudaSuccess) rc = bfail(b, ESM_ECUDA, "event time");
            if (!rc) rc = batch_join_out(b);
            for (esm_ctx *c : b->ctx)
                if (!rc && (rc = esm_state_restore(c))) rc = bfail(b, rc, "state restore: %s", c->err.c_str());
            if (!rc) rc = batch_join_in(b);
        }
        if (rc) break;
        if (cand) {
            cand[2 * i] = list[i][0];
            cand[2 * i + 1] = list[i][1];
        }
        if (ms) ms[i] = t;
        if (t < tbest) {
            tbest = t;
            bw = list[i][0];
            bs = list[i][1];
        }
    }
    if (rc) return rc;
    if (ncand) *ncand = n;
    if (best) {
        best[0] = bw;
        best[1] = bs;
    }
    return esm_batch_set_grid(b, bw, bs);
}
