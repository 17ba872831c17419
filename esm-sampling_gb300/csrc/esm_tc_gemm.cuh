// BF16 GEMM on the 5th-generation tensor cores (tcgen05) for the surrogate MLP: C[M,N] (+)=
// A[M,K] B[N,K]^T with A and B K-major in BF16, the FP32 accumulator in tensor memory (TMEM).
//
// One CTA of 4 warps per 128 x 64 tile of C. Operands are staged through shared memory in the
// canonical no-swizzle K-major layout of tcgen05 (core matrices of 8 rows x 16 bytes; along K the
// core matrices of a row group are 128 bytes apart (the leading-dimension offset), row groups 1024
// bytes apart (the stride-dimension offset)), two stages deep: while the tensor core multiplies
// stage s, the threads load stage s + 1 from global memory into registers. One elected thread issues
// tcgen05.mma (M = 128, N = 64, K = 16, kind::f16, BF16 x BF16 -> FP32) and commits each stage to an
// mbarrier that releases the stage's shared memory. The epilogue reads the accumulator with
// tcgen05.ld (32 lanes x 32 bits, each warp its 32 rows), adds the bias, applies SiLU and writes
// FP32 and BF16 outputs. Every mbarrier wait is bounded: on time-out the kernel sets *err, frees its
// tensor memory and returns.
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace tc {

#define TC_BM 128
#define TC_BN 64
#define TC_BK 64
#define TC_STAGE_A (TC_BM * TC_BK * 2)  // bytes of one A stage
#define TC_STAGE_B (TC_BN * TC_BK * 2)
#define TC_SMEM (2 * (TC_STAGE_A + TC_STAGE_B) + 1024)
#define TC_WAIT_LIMIT (1 << 24)

struct GemmTC {
    int M, N, K;
    const __nv_bfloat16 *A;  // A(m, k) at A[m*lda + k]
    int lda;
    const __nv_bfloat16 *B;  // B(n, k) at B[n*ldb + k]
    int ldb;
    float *C;  // C(m, n) at C[m*ldc + n] (may be null)
    int ldc;
    int accumulate;
    const float *bias;  // per n (may be null)
    int silu;
    __nv_bfloat16 *Cb;  // BF16 copy of the (activated) output (may be null)
    int ldcb;
    int *err;  // set to 1 when a wait ran out
};

__device__ inline uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// shared-memory matrix descriptor: start address, leading- and stride-dimension byte offsets (all
// in units of 16 bytes), the descriptor version 1 of this architecture, no swizzle
__device__ inline uint64_t sdesc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr & 0x3FFFF) >> 4);
    d |= (uint64_t)((lbo & 0x3FFFF) >> 4) << 16;
    d |= (uint64_t)((sbo & 0x3FFFF) >> 4) << 32;
    d |= (uint64_t)1 << 46;
    return d;
}

// instruction descriptor of kind::f16: FP32 accumulator, BF16 A and B, both K-major, M x N
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ inline bool mbar_wait(uint32_t bar, uint32_t parity) {
    for (int it = 0; it < TC_WAIT_LIMIT; ++it) {
        uint32_t ok;
        asm volatile(
            "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}\n"
            : "=r"(ok)
            : "r"(bar), "r"(parity)
            : "memory");
        if (ok) return true;
    }
    return false;
}

// the 16-byte chunk c of a 128-row x 64-column (or 64-row) K-major tile: row and K chunk, and its
// offset in the canonical layout
__device__ inline uint32_t tile_off(int row, int kc) { return (uint32_t)((row >> 3) * 1024 + kc * 128 + (row & 7) * 16); }

__device__ inline uint4 load_chunk(const __nv_bfloat16 *X, int ld, int rows, int K, int r, int k) {
    uint4 v = make_uint4(0, 0, 0, 0);
    if (r >= rows || k >= K) return v;
    const __nv_bfloat16 *p = X + (size_t)r * ld + k;
    if (k + 8 <= K && ((ld & 7) == 0) && ((((uintptr_t)p) & 15) == 0)) return *(const uint4 *)p;
    __nv_bfloat16 t[8];
    for (int i = 0; i < 8; ++i) t[i] = (k + i < K) ? p[i] : __float2bfloat16(0.f);
    return *(const uint4 *)t;
}

__global__ void __launch_bounds__(128, 1) k_gemm_tc(GemmTC g) {
    extern __shared__ uint8_t smraw[];
    __shared__ __align__(8) uint64_t mbar[2];
    __shared__ uint32_t tmem_s;
    __shared__ int bad_s;
    uint8_t *sm = (uint8_t *)(((uintptr_t)smraw + 1023) & ~(uintptr_t)1023);
    uint8_t *sA[2] = {sm, sm + TC_STAGE_A};
    uint8_t *sB[2] = {sm + 2 * TC_STAGE_A, sm + 2 * TC_STAGE_A + TC_STAGE_B};
    int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    int m0 = blockIdx.y * TC_BM, n0 = blockIdx.x * TC_BN;
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_s)),
                     "r"(TC_BN)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0) {
        bad_s = 0;
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&mbar[0])) : "memory");
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&mbar[1])) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    uint32_t tmem = tmem_s;
    const uint32_t idesc = idesc_bf16(TC_BM, TC_BN);
    int nk = (g.K + TC_BK - 1) / TC_BK;
    uint32_t phase[2] = {0, 0};
    uint4 ra[8], rb[4];
    auto fetch = [&](int t) {  // tile t into registers: A 1024 chunks, B 512 chunks over 128 threads
        int k0 = t * TC_BK;
        for (int i = 0; i < 8; ++i) {
            int c = tid + i * 128, r = c >> 3, kc = c & 7;
            ra[i] = load_chunk(g.A, g.lda, g.M, g.K, m0 + r, k0 + kc * 8);
        }
        for (int i = 0; i < 4; ++i) {
            int c = tid + i * 128, r = c >> 3, kc = c & 7;
            rb[i] = load_chunk(g.B, g.ldb, g.N, g.K, n0 + r, k0 + kc * 8);
        }
    };
    auto store = [&](int s) {
        for (int i = 0; i < 8; ++i) {
            int c = tid + i * 128, r = c >> 3, kc = c & 7;
            *(uint4 *)(sA[s] + tile_off(r, kc)) = ra[i];
        }
        for (int i = 0; i < 4; ++i) {
            int c = tid + i * 128, r = c >> 3, kc = c & 7;
            *(uint4 *)(sB[s] + tile_off(r, kc)) = rb[i];
        }
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    };
    bool ok = true;
    if (nk > 0) fetch(0);
    for (int t = 0; t < nk && ok; ++t) {
        int s = t & 1;
        if (t >= 2) {  // the stage's previous multiplications (tile t - 2) must have read it
            if (!mbar_wait(smem_u32(&mbar[s]), phase[s])) ok = false;
            phase[s] ^= 1;
        }
        if (__syncthreads_or(!ok)) {
            ok = false;
            break;
        }
        store(s);
        __syncthreads();
        if (tid == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            uint32_t a0 = smem_u32(sA[s]), b0 = smem_u32(sB[s]);
            for (int kk = 0; kk < TC_BK / 16; ++kk) {
                uint64_t ad = sdesc(a0 + kk * 256, 128, 1024);
                uint64_t bd = sdesc(b0 + kk * 256, 128, 1024);
                uint32_t acc = (t > 0 || kk > 0) ? 1u : 0u;
                asm volatile(
                    "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\ttcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(
                        tmem),
                    "l"(ad), "l"(bd), "r"(idesc), "r"(acc)
                    : "memory");
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                             smem_u32(&mbar[s]))
                         : "memory");
        }
        if (t + 1 < nk) fetch(t + 1);
    }
    // the last stages' multiplications: their commits complete the accumulator
    if (ok) {
        for (int t = nk - 2 < 0 ? 0 : nk - 2; t < nk; ++t) {
            int s = t & 1;
            if (!mbar_wait(smem_u32(&mbar[s]), phase[s])) ok = false;
            phase[s] ^= 1;
        }
    }
    if (!ok) bad_s = 1;
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (!bad_s && nk > 0) {
        int row = m0 + warp * 32 + lane;
        for (int cc = 0; cc < TC_BN; cc += 16) {
            uint32_t r[16];
            uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)cc;
            asm volatile(
                "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, "
                "%14, %15}, [%16];"
                : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                  "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
                : "r"(taddr));
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
            if (row < g.M)
                for (int j = 0; j < 16; ++j) {
                    int n = n0 + cc + j;
                    if (n >= g.N) break;
                    float v = __uint_as_float(r[j]);
                    if (g.bias) v += g.bias[n];
                    if (g.C) {
                        float *cp = g.C + (size_t)row * g.ldc + n;
                        if (g.accumulate)
                            *cp += v;
                        else
                            *cp = v;
                    }
                    if (g.Cb) {
                        float o = g.silu ? v / (1.f + expf(-v)) : v;
                        g.Cb[(size_t)row * g.ldcb + n] = __float2bfloat16(o);
                    }
                }
        }
    }
    if (bad_s && tid == 0 && g.err) atomicExch(g.err, 1);
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TC_BN) : "memory");
}

// B[n, k] (K-major) from a row-major [k, n] BF16 matrix: out[n*ldo + k] = in[k*ldi + n]
__global__ void k_transpose_bf16(int rows, int cols, const __nv_bfloat16 *in, int ldi, __nv_bfloat16 *out, int ldo) {
    __shared__ __nv_bfloat16 tile[32][33];
    int c0 = blockIdx.x * 32, r0 = blockIdx.y * 32;
    for (int i = threadIdx.y; i < 32; i += blockDim.y) {
        int r = r0 + i, c = c0 + threadIdx.x;
        tile[i][threadIdx.x] = (r < rows && c < cols) ? in[(size_t)r * ldi + c] : __float2bfloat16(0.f);
    }
    __syncthreads();
    for (int i = threadIdx.y; i < 32; i += blockDim.y) {
        int c = c0 + i, r = r0 + threadIdx.x;
        if (c < cols && r < rows) out[(size_t)c * ldo + r] = tile[threadIdx.x][i];
    }
}

}  // namespace tc
