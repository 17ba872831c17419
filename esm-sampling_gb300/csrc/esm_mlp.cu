// Surrogate of the replica-averaged capacity score: a small MLP trained online on (capacity,
// sampled score) pairs with hand-written BF16 tensor-core kernels (tcgen05.mma with the accumulator
// in tensor memory, esm_tc_gemm.cuh; the warp-level mma.sync m16n8k16 kernel below stays selectable
// as its check, esm_mlp_set_gemm), FP32 accumulation, SiLU hidden layers, mean-squared loss and
// Adam with FP32 master weights.
// The learned part is not in the reference (it is this repository's addition); its CPU check is
// the oracle's FP32 MLP on the same BF16-rounded operands.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include <string>
#include <vector>

#include "../../include/esmcuda.h"
#include "esm_tc_gemm.cuh"

using std::vector;

namespace {

// ---------------------------------------------------------------------------------------------
// generic GEMM C[M,N] (+)= sum_k A(m,k) B(k,n), A and B in BF16 with arbitrary strides, C in FP32.
// 64x64x32 tiles, 4 warps (2x2), each warp a 32x32 block of m16n8k16 BF16 mma.sync fragments.
// Epilogue: optional bias (per n), SiLU, FP32 and BF16 outputs.
// ---------------------------------------------------------------------------------------------
struct GemmArgs {
    int M, N, K;
    const __nv_bfloat16 *A;
    long long sam, sak;  // A(m, k) at A[m*sam + k*sak]
    const __nv_bfloat16 *B;
    long long sbk, sbn;  // B(k, n) at B[k*sbk + n*sbn]
    float *C;            // C(m, n) at C[m*ldc + n] (may be null)
    int ldc;
    int accumulate;      // C += result
    const float *bias;   // per n (may be null)
    int silu;            // apply SiLU in the epilogue (pre-activation kept in C)
    __nv_bfloat16 *Cb;   // BF16 copy of the (activated) output (may be null)
    int ldcb;
};

#define BM 64
#define BN 64
#define BK 32
#define PAD 8

__device__ inline uint32_t pack2(__nv_bfloat16 lo, __nv_bfloat16 hi) {
    uint32_t a = (uint32_t)__bfloat16_as_ushort(lo), b = (uint32_t)__bfloat16_as_ushort(hi);
    return a | (b << 16);
}

__global__ void __launch_bounds__(128) k_gemm_bf16(GemmArgs g) {
    __shared__ __nv_bfloat16 sA[BM][BK + PAD];  // (m, k)
    __shared__ __nv_bfloat16 sB[BN][BK + PAD];  // (n, k)
    int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
    int wm = (warp >> 1) * 32, wn = (warp & 1) * 32;
    int gq = lane >> 2, tq = lane & 3;
    float acc[2][4][4];
    for (int i = 0; i < 2; ++i)
        for (int j = 0; j < 4; ++j)
            for (int r = 0; r < 4; ++r) acc[i][j][r] = 0.f;
    __nv_bfloat16 zero = __float2bfloat16(0.f);
    for (int k0 = 0; k0 < g.K; k0 += BK) {
        for (int e = tid; e < BM * BK; e += 128) {
            int mm = e / BK, kk = e % BK;
            int m = m0 + mm, k = k0 + kk;
            sA[mm][kk] = (m < g.M && k < g.K) ? g.A[(long long)m * g.sam + (long long)k * g.sak] : zero;
        }
        for (int e = tid; e < BN * BK; e += 128) {
            int nn = e / BK, kk = e % BK;
            int n = n0 + nn, k = k0 + kk;
            sB[nn][kk] = (n < g.N && k < g.K) ? g.B[(long long)k * g.sbk + (long long)n * g.sbn] : zero;
        }
        __syncthreads();
#pragma unroll
        for (int ks = 0; ks < BK; ks += 16) {
            uint32_t af[2][4], bf[4][2];
#pragma unroll
            for (int i = 0; i < 2; ++i) {
                int r = wm + i * 16 + gq;
                int c = ks + tq * 2;
                af[i][0] = pack2(sA[r][c], sA[r][c + 1]);
                af[i][1] = pack2(sA[r + 8][c], sA[r + 8][c + 1]);
                af[i][2] = pack2(sA[r][c + 8], sA[r][c + 9]);
                af[i][3] = pack2(sA[r + 8][c + 8], sA[r + 8][c + 9]);
            }
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                int n = wn + j * 8 + gq;
                int c = ks + tq * 2;
                bf[j][0] = pack2(sB[n][c], sB[n][c + 1]);
                bf[j][1] = pack2(sB[n][c + 8], sB[n][c + 9]);
            }
#pragma unroll
            for (int i = 0; i < 2; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    float *d = acc[i][j];
                    asm volatile(
                        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
                        "{%8,%9}, {%0,%1,%2,%3};\n"
                        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
                        : "r"(af[i][0]), "r"(af[i][1]), "r"(af[i][2]), "r"(af[i][3]), "r"(bf[j][0]), "r"(bf[j][1]));
                }
        }
        __syncthreads();
    }
    // epilogue
    for (int i = 0; i < 2; ++i)
        for (int j = 0; j < 4; ++j)
            for (int r = 0; r < 4; ++r) {
                int m = m0 + wm + i * 16 + gq + (r >= 2 ? 8 : 0);
                int n = n0 + wn + j * 8 + tq * 2 + (r & 1);
                if (m >= g.M || n >= g.N) continue;
                float v = acc[i][j][r];
                if (g.bias) v += g.bias[n];
                if (g.C) {
                    float *cp = g.C + (long long)m * g.ldc + n;
                    if (g.accumulate)
                        *cp += v;
                    else
                        *cp = v;
                }
                if (g.Cb) {
                    float o = g.silu ? v / (1.f + expf(-v)) : v;
                    g.Cb[(long long)m * g.ldcb + n] = __float2bfloat16(o);
                }
            }
}

// delta of a hidden layer: d_z = d_a * SiLU'(z)
__global__ void k_silu_back(int n, const float *z, const float *da, float *dz, __nv_bfloat16 *dzb) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float s = 1.f / (1.f + expf(-z[i]));
    float v = da[i] * (s * (1.f + z[i] * (1.f - s)));
    dz[i] = v;
    dzb[i] = __float2bfloat16(v);
}

// output delta of the mean-squared loss: d = (y - t) / B (masked columns beyond d_out are zero);
// per-row squared error accumulated into loss
__global__ void k_loss(int B, int dout, const float *y, const float *t, float *d, __nv_bfloat16 *db, double *loss) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= B * dout) return;
    float e = y[i] - t[i];
    d[i] = e / (float)B;
    db[i] = __float2bfloat16(e / (float)B);
    atomicAdd(loss, 0.5 * (double)e * (double)e / (double)B);
}

// column sums (bias gradient): out[n] = sum_m d[m, n]
__global__ void k_colsum(int M, int N, const float *d, float *out) {
    int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= N) return;
    float s = 0.f;
    for (int m = 0; m < M; ++m) s += d[(long long)m * N + n];
    out[n] = s;
}

// Adam (Kingma and Ba 2015) on FP32 master weights; refresh the BF16 copy and its transpose
__global__ void k_adam(int n, int rows, int cols, float *w, float *m, float *v, const float *g, float lr, float b1,
                       float b2, float eps, float c1, float c2, __nv_bfloat16 *wb, __nv_bfloat16 *wt) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float gi = g[i];
    float mi = b1 * m[i] + (1.f - b1) * gi;
    float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    float wi = w[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    w[i] = wi;
    if (wb) wb[i] = __float2bfloat16(wi);
    if (wt) {
        int r = i / cols, c = i % cols;
        wt[(long long)c * rows + r] = __float2bfloat16(wi);
    }
    (void)rows;
}

__global__ void k_to_bf16(int n, const float *x, __nv_bfloat16 *y) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) y[i] = __float2bfloat16(x[i]);
}

}  // namespace

// ---------------------------------------------------------------------------------------------
// the surrogate context
// ---------------------------------------------------------------------------------------------
struct esm_mlp {
    int nl = 0;                 // layers (hidden + output)
    vector<int> dims;           // d_0 .. d_nl
    int Bmax = 0;
    cudaStream_t stream = nullptr;
    std::string err;
    int64_t launches = 0, steps = 0;
    float lr = 1e-3f, b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    vector<float *> W, b, mW, vW, mb, vb, gW, gb;  // FP32 master, Adam moments, gradients
    vector<__nv_bfloat16 *> Wb, Wt;               // BF16 copies [out, in] and transposed [in, out]
    vector<float *> Z;                             // pre-activations per layer [B, d_{l+1}]
    vector<__nv_bfloat16 *> Ab;                    // activations BF16 per layer [B, d_l] (Ab[0] = input)
    float *dA = nullptr, *dZ = nullptr, *target = nullptr;
    __nv_bfloat16 *dZb = nullptr;
    float *xin = nullptr;
    double *loss = nullptr;
    vector<void *> allocs;
    int gemm_kind = 1;                             // 1: tcgen05 (k_gemm_tc), 0: mma.sync (k_gemm_bf16)
    __nv_bfloat16 *tA = nullptr, *tB = nullptr;    // K-major copies of the weight-gradient operands
    int *tc_err = nullptr;                         // set by k_gemm_tc when a wait ran out
};

namespace {

int mfail(esm_mlp *c, int code, const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    if (c) c->err = buf;
    return code;
}

#define MK(call)                                                                                   \
    do {                                                                                           \
        cudaError_t e_ = (call);                                                                   \
        if (e_ != cudaSuccess)                                                                     \
            return mfail(c, e_ == cudaErrorMemoryAllocation ? ESM_ENOMEM : ESM_ECUDA, "%s: %s", #call, \
                         cudaGetErrorString(e_));                                                  \
    } while (0)

template <class T>
int malloc_(esm_mlp *c, T **p, size_t n) {
    void *q = nullptr;
    cudaError_t e = cudaMalloc(&q, sizeof(T) * (n ? n : 1));
    if (e != cudaSuccess) return mfail(c, ESM_ENOMEM, "cudaMalloc: %s", cudaGetErrorString(e));
    cudaMemsetAsync(q, 0, sizeof(T) * (n ? n : 1), c->stream);
    c->allocs.push_back(q);
    *p = (T *)q;
    return ESM_OK;
}

int gemm_tc(esm_mlp *c, const GemmArgs &g, const __nv_bfloat16 *A, int lda, const __nv_bfloat16 *B, int ldb) {
    tc::GemmTC t{};
    t.M = g.M;
    t.N = g.N;
    t.K = g.K;
    t.A = A;
    t.lda = lda;
    t.B = B;
    t.ldb = ldb;
    t.C = g.C;
    t.ldc = g.ldc;
    t.accumulate = g.accumulate;
    t.bias = g.bias;
    t.silu = g.silu;
    t.Cb = g.Cb;
    t.ldcb = g.ldcb;
    t.err = c->tc_err;
    dim3 grid((g.N + TC_BN - 1) / TC_BN, (g.M + TC_BM - 1) / TC_BM);
    tc::k_gemm_tc<<<grid, 128, TC_SMEM, c->stream>>>(t);
    c->launches += 1;
    MK(cudaGetLastError());
    return ESM_OK;
}

// K-major copy of a BF16 operand given by strides: out[r*ld + k] = X(r, k), X(r, k) at X[r*sr + k*sk]
// with sr == 1 (the row index fastest: a transpose of the row-major [k, r] matrix)
int kmajor(esm_mlp *c, const __nv_bfloat16 *X, int rows, int K, long long sk, __nv_bfloat16 *out) {
    dim3 grid((rows + 31) / 32, (K + 31) / 32), block(32, 8);
    tc::k_transpose_bf16<<<grid, block, 0, c->stream>>>(K, rows, X, (int)sk, out, K);
    c->launches += 1;
    MK(cudaGetLastError());
    return ESM_OK;
}

int gemm(esm_mlp *c, GemmArgs g) {
    if (c->gemm_kind == 1) {
        // the tensor-core path takes K-major operands: A(m, k) rows of A, B(k, n) rows of B indexed by n
        bool ak = g.sak == 1, bk = g.sbk == 1;
        const __nv_bfloat16 *A = g.A, *B = g.B;
        int lda = (int)g.sam, ldb = (int)g.sbn;
        int rc;
        if (!ak) {
            if (g.sam != 1) return mfail(c, ESM_EINVAL, "GEMM operand A with neither stride 1");
            if ((rc = kmajor(c, g.A, g.M, g.K, g.sak, c->tA))) return rc;
            A = c->tA;
            lda = g.K;
        }
        if (!bk) {
            if (g.sbn != 1) return mfail(c, ESM_EINVAL, "GEMM operand B with neither stride 1");
            if ((rc = kmajor(c, g.B, g.N, g.K, g.sbk, c->tB))) return rc;
            B = c->tB;
            ldb = g.K;
        }
        return gemm_tc(c, g, A, lda, B, ldb);
    }
    dim3 grid((g.N + BN - 1) / BN, (g.M + BM - 1) / BM);
    k_gemm_bf16<<<grid, 128, 0, c->stream>>>(g);
    c->launches += 1;
    MK(cudaGetLastError());
    return ESM_OK;
}

// a wait of the tensor-core GEMM ran out: the stream's results are not to be used
int tc_check(esm_mlp *c) {
    if (c->gemm_kind != 1) return ESM_OK;
    int e = 0;
    MK(cudaMemcpyAsync(&e, c->tc_err, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    MK(cudaStreamSynchronize(c->stream));
    if (e) return mfail(c, ESM_ETIMEOUT, "a tensor-core GEMM wait ran out");
    return ESM_OK;
}

// forward pass on B rows already in Ab[0]
int forward(esm_mlp *c, int B) {
    for (int l = 0; l < c->nl; ++l) {
        int din = c->dims[l], dout = c->dims[l + 1];
        bool hidden = l + 1 < c->nl;
        GemmArgs g{};
        g.M = B;
        g.N = dout;
        g.K = din;
        g.A = c->Ab[l];
        g.sam = din;
        g.sak = 1;
        g.B = c->Wb[l];  // B(k, n) = W[n, k]
        g.sbk = 1;
        g.sbn = din;
        g.C = c->Z[l];
        g.ldc = dout;
        g.bias = c->b[l];
        g.silu = hidden ? 1 : 0;
        g.Cb = hidden ? c->Ab[l + 1] : nullptr;
        g.ldcb = dout;
        int rc = gemm(c, g);
        if (rc) return rc;
    }
    return ESM_OK;
}

}  // namespace

extern "C" {

int esm_mlp_create(int32_t nlayers, const int32_t *dims, int32_t batch_max, uint64_t seed, esm_mlp **out) {
    if (!out) return ESM_EINVAL;
    *out = nullptr;
    esm_mlp *c = new esm_mlp();
    *out = c;
    if (nlayers < 1 || !dims || batch_max < 1) return mfail(c, ESM_EINVAL, "bad sizes");
    c->nl = nlayers;
    c->dims.assign(dims, dims + nlayers + 1);
    for (int d : c->dims)
        if (d < 1) return mfail(c, ESM_EINVAL, "bad layer width");
    c->Bmax = batch_max;
    MK(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
    int rc;
    int dmax = 0;
    for (int d : c->dims) dmax = d > dmax ? d : dmax;
    c->W.resize(nlayers);
    c->b.resize(nlayers);
    c->mW.resize(nlayers);
    c->vW.resize(nlayers);
    c->mb.resize(nlayers);
    c->vb.resize(nlayers);
    c->gW.resize(nlayers);
    c->gb.resize(nlayers);
    c->Wb.resize(nlayers);
    c->Wt.resize(nlayers);
    c->Z.resize(nlayers);
    c->Ab.resize(nlayers + 1);
    for (int l = 0; l < nlayers; ++l) {
        size_t nw = (size_t)c->dims[l] * c->dims[l + 1], nb = c->dims[l + 1];
        for (float **p : {&c->W[l], &c->mW[l], &c->vW[l], &c->gW[l]})
            if ((rc = malloc_(c, p, nw))) return rc;
        for (float **p : {&c->b[l], &c->mb[l], &c->vb[l], &c->gb[l]})
            if ((rc = malloc_(c, p, nb))) return rc;
        if ((rc = malloc_(c, &c->Wb[l], nw))) return rc;
        if ((rc = malloc_(c, &c->Wt[l], nw))) return rc;
        if ((rc = malloc_(c, &c->Z[l], (size_t)batch_max * c->dims[l + 1]))) return rc;
    }
    for (int l = 0; l <= nlayers; ++l)
        if ((rc = malloc_(c, &c->Ab[l], (size_t)batch_max * c->dims[l]))) return rc;
    if ((rc = malloc_(c, &c->dA, (size_t)batch_max * dmax))) return rc;
    if ((rc = malloc_(c, &c->dZ, (size_t)batch_max * dmax))) return rc;
    if ((rc = malloc_(c, &c->dZb, (size_t)batch_max * dmax))) return rc;
    if ((rc = malloc_(c, &c->target, (size_t)batch_max * c->dims[nlayers]))) return rc;
    if ((rc = malloc_(c, &c->xin, (size_t)batch_max * c->dims[0]))) return rc;
    if ((rc = malloc_(c, &c->loss, 1))) return rc;
    if ((rc = malloc_(c, &c->tA, (size_t)batch_max * dmax))) return rc;
    if ((rc = malloc_(c, &c->tB, (size_t)batch_max * dmax))) return rc;
    if ((rc = malloc_(c, &c->tc_err, 1))) return rc;
    MK(cudaFuncSetAttribute(tc::k_gemm_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, TC_SMEM));
    // He-style initialisation from a fixed LCG stream (host), zero biases
    uint64_t st = seed * 6364136223846793005ull + 1442695040888963407ull;
    for (int l = 0; l < nlayers; ++l) {
        size_t nw = (size_t)c->dims[l] * c->dims[l + 1];
        vector<float> w(nw);
        float sc = sqrtf(2.f / (float)c->dims[l]) * (l + 1 == nlayers ? 0.1f : 1.f);
        for (size_t i = 0; i < nw; ++i) {
            st = st * 6364136223846793005ull + 1442695040888963407ull;
            double u1 = ((st >> 11) + 0.5) / 9007199254740992.0;
            st = st * 6364136223846793005ull + 1442695040888963407ull;
            double u2 = ((st >> 11) + 0.5) / 9007199254740992.0;
            w[i] = (float)(sc * sqrt(-2.0 * log(u1)) * cos(6.283185307179586 * u2));
        }
        int r2 = esm_mlp_set_layer(c, l, w.data(), nullptr);
        if (r2) return r2;
    }
    MK(cudaStreamSynchronize(c->stream));
    return ESM_OK;
}

int esm_mlp_destroy(esm_mlp *c) {
    if (!c) return ESM_OK;
    if (c->stream) cudaStreamSynchronize(c->stream);
    for (void *p : c->allocs) cudaFree(p);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
    return ESM_OK;
}

const char *esm_mlp_last_error(const esm_mlp *c) { return c ? c->err.c_str() : "no context"; }

int esm_mlp_set_layer(esm_mlp *c, int32_t l, const float *w, const float *bias) {
    if (!c || l < 0 || l >= c->nl) return ESM_EINVAL;
    int rows = c->dims[l + 1], cols = c->dims[l];
    size_t nw = (size_t)rows * cols;
    if (w) {
        MK(cudaMemcpyAsync(c->W[l], w, sizeof(float) * nw, cudaMemcpyHostToDevice, c->stream));
        // BF16 copy and transpose through a zero-rate Adam pass (lr 0 leaves the weights unchanged)
        MK(cudaMemsetAsync(c->gW[l], 0, sizeof(float) * nw, c->stream));
        k_adam<<<(unsigned)((nw + 255) / 256), 256, 0, c->stream>>>((int)nw, rows, cols, c->W[l], c->mW[l], c->vW[l],
                                                                     c->gW[l], 0.f, 0.f, 0.f, 1.f, 1.f, 1.f,
                                                                     c->Wb[l], c->Wt[l]);
        MK(cudaGetLastError());
        c->launches += 1;
    }
    if (bias) MK(cudaMemcpyAsync(c->b[l], bias, sizeof(float) * rows, cudaMemcpyHostToDevice, c->stream));
    MK(cudaStreamSynchronize(c->stream));
    return ESM_OK;
}

int esm_mlp_get_layer(esm_mlp *c, int32_t l, float *w, float *bias) {
    if (!c || l < 0 || l >= c->nl) return ESM_EINVAL;
    int rows = c->dims[l + 1], cols = c->dims[l];
    if (w) MK(cudaMemcpyAsync(w, c->W[l], sizeof(float) * rows * cols, cudaMemcpyDeviceToHost, c->stream));
    if (bias) MK(cudaMemcpyAsync(bias, c->b[l], sizeof(float) * rows, cudaMemcpyDeviceToHost, c->stream));
    MK(cudaStreamSynchronize(c->stream));
    return ESM_OK;
}

int esm_mlp_forward(esm_mlp *c, int32_t B, const float *x, float *y) {
    if (!c || !x || B < 1 || B > c->Bmax) return c ? mfail(c, ESM_EINVAL, "batch %d out of range", B) : ESM_EINVAL;
    int din = c->dims[0], dout = c->dims[c->nl];
    MK(cudaMemcpyAsync(c->xin, x, sizeof(float) * B * din, cudaMemcpyHostToDevice, c->stream));
    k_to_bf16<<<(B * din + 255) / 256, 256, 0, c->stream>>>(B * din, c->xin, c->Ab[0]);
    MK(cudaGetLastError());
    c->launches += 1;
    int rc = forward(c, B);
    if (rc) return rc;
    if (y) MK(cudaMemcpyAsync(y, c->Z[c->nl - 1], sizeof(float) * B * dout, cudaMemcpyDeviceToHost, c->stream));
    MK(cudaStreamSynchronize(c->stream));
    return tc_check(c);
}

// One Adam step on a minibatch (x [B, d0], target [B, d_out]); gradients of the mean-squared loss
// (1/2B) sum (y - t)^2. grads_out (may be null): the gradients of layer 0..nl-1, W then b, FP32.
int esm_mlp_train_step(esm_mlp *c, int32_t B, const float *x, const float *target, float lr, double *loss_out,
                       float *grads_out) {
    if (!c || !x || !target || B < 1 || B > c->Bmax)
        return c ? mfail(c, ESM_EINVAL, "bad training batch") : ESM_EINVAL;
    int nl = c->nl, din = c->dims[0], dout = c->dims[nl];
    MK(cudaMemcpyAsync(c->xin, x, sizeof(float) * B * din, cudaMemcpyHostToDevice, c->stream));
    MK(cudaMemcpyAsync(c->target, target, sizeof(float) * B * dout, cudaMemcpyHostToDevice, c->stream));
    MK(cudaMemsetAsync(c->loss, 0, sizeof(double), c->stream));
    k_to_bf16<<<(B * din + 255) / 256, 256, 0, c->stream>>>(B * din, c->xin, c->Ab[0]);
    int rc = forward(c, B);
    if (rc) return rc;
    k_loss<<<(B * dout + 255) / 256, 256, 0, c->stream>>>(B, dout, c->Z[nl - 1], c->target, c->dZ, c->dZb, c->loss);
    c->launches += 2;
    MK(cudaGetLastError());
    for (int l = nl - 1; l >= 0; --l) {
        int di = c->dims[l], dn = c->dims[l + 1];
        // dW[n, k] = sum_b dZ[b, n] A[b, k]
        GemmArgs g{};
        g.M = dn;
        g.N = di;
        g.K = B;
        g.A = c->dZb;
        g.sam = 1;
        g.sak = dn;
        g.B = c->Ab[l];
        g.sbk = di;
        g.sbn = 1;
        g.C = c->gW[l];
        g.ldc = di;
        if ((rc = gemm(c, g))) return rc;
        k_colsum<<<(dn + 127) / 128, 128, 0, c->stream>>>(B, dn, c->dZ, c->gb[l]);
        c->launches += 1;
        if (l > 0) {
            // dA[b, k] = sum_n dZ[b, n] W[n, k]
            GemmArgs h{};
            h.M = B;
            h.N = di;
            h.K = dn;
            h.A = c->dZb;
            h.sam = dn;
            h.sak = 1;
            h.B = c->Wt[l];  // B(k=n, n=k): Wt[k, n] = W[n, k]
            h.sbk = 1;
            h.sbn = dn;
            h.C = c->dA;
            h.ldc = di;
            if ((rc = gemm(c, h))) return rc;
            k_silu_back<<<(B * di + 255) / 256, 256, 0, c->stream>>>(B * di, c->Z[l - 1], c->dA, c->dZ, c->dZb);
            c->launches += 1;
            MK(cudaGetLastError());
        }
        // the deltas of layer l are consumed: dZ now holds the layer below (computed above)
        if (grads_out) {
            size_t off = 0;
            for (int q = 0; q < l; ++q) off += (size_t)c->dims[q] * c->dims[q + 1] + c->dims[q + 1];
            MK(cudaMemcpyAsync(grads_out + off, c->gW[l], sizeof(float) * dn * di, cudaMemcpyDeviceToHost, c->stream));
            MK(cudaMemcpyAsync(grads_out + off + (size_t)dn * di, c->gb[l], sizeof(float) * dn, cudaMemcpyDeviceToHost,
                               c->stream));
        }
    }
    c->steps += 1;
    float c1 = 1.f - powf(c->b1, (float)c->steps), c2 = 1.f - powf(c->b2, (float)c->steps);
    for (int l = 0; l < nl; ++l) {
        int rows = c->dims[l + 1], cols = c->dims[l];
        int nw = rows * cols;
        k_adam<<<(nw + 255) / 256, 256, 0, c->stream>>>(nw, rows, cols, c->W[l], c->mW[l], c->vW[l], c->gW[l], lr,
                                                         c->b1, c->b2, c->eps, c1, c2, c->Wb[l], c->Wt[l]);
        k_adam<<<(rows + 255) / 256, 256, 0, c->stream>>>(rows, 1, rows, c->b[l], c->mb[l], c->vb[l], c->gb[l], lr,
                                                           c->b1, c->b2, c->eps, c1, c2, nullptr, nullptr);
        c->launches += 2;
    }
    MK(cudaGetLastError());
    double L = 0;
    MK(cudaMemcpyAsync(&L, c->loss, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    MK(cudaStreamSynchronize(c->stream));
    if (loss_out) *loss_out = L;
    return tc_check(c);
}

int64_t esm_mlp_launch_count(const esm_mlp *c) { return c ? c->launches : 0; }

int esm_mlp_set_gemm(esm_mlp *c, int32_t kind) {
    if (!c) return ESM_EINVAL;
    if (kind != 0 && kind != 1) return mfail(c, ESM_EINVAL, "GEMM kind must be 0 (mma.sync) or 1 (tcgen05)");
    MK(cudaStreamSynchronize(c->stream));
    c->gemm_kind = kind;
    return ESM_OK;
}

}  // extern "C"
