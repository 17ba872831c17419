/*
 * Philox4x32-10 counter-based generator (Salmon et al., "Parallel random numbers: as easy as
 * 1, 2, 3", SC11) and the stream layout shared by the CPU oracle and the CUDA path.
 *
 * ORACLE / TEST INFRASTRUCTURE: this header belongs to the CPU oracle; the CUDA library has its
 * own implementation of the same published algorithm.
 *
 * Stream contract (the device path follows the same layout):
 *   key   = (seed_lo32, seed_hi32 ^ tag)
 *   uniform53(x0, x1) = ((x0 >> 5) * 2^26 + (x1 >> 6)) * 2^-53   in [0, 1)
 *   one Philox call gives two uniforms: (x0, x1) and (x2, x3)
 *   TAG_SWEEP  counter (0, 0, 0, sweep)                class order of a sweep
 *   TAG_LIST   counter (j >> 1, tile, cls, sweep)      uniform j of a move-list tile
 *   TAG_LANE   counter (2 mi + h, tau, rep, sweep)     per replica-step draws of move mi:
 *              h = 0: (u_cat, u_off), h = 1: (u_jac, -)
 *   TAG_LGV    counter (j >> 1, group, it, 0)          Langevin normals (Box-Muller)
 *   TAG_WTH    counter (j >> 1, t, rep, it)            weather normals / uniforms
 *   TAG_SMS    counter (j >> 1, 0, 0, sweep)           storage multiscale sweep of a sweep: its coin,
 *                                                       the order of the lengths, offsets, class order
 *              counter (j >> 1, 1 + li, 2 + cls, sweep) the 8 move selections of a class of length 2^(li+1)
 *   TAG_SML    counter (2 (8 li + m) + h, b0, rep, sweep)  per block-replica draws of move m:
 *              h = 0: (u_cat, u_off), h = 1: (u_jac, -)
 *   TAG_SLG    counter (j >> 1, unit, 0, sweep)        long-range storage sweep: a unit's move list
 *   TAG_SLL    counter (2 m + h, unit, rep, sweep)     per unit-replica draws of its move m
 */
#ifndef ESM_ORACLE_PHILOX_H
#define ESM_ORACLE_PHILOX_H
#include <stdint.h>
#include <math.h>

#define ESM_TAG_SWEEP 0x53574550u
#define ESM_TAG_LIST 0x4C495354u
#define ESM_TAG_LANE 0x4C414E45u
#define ESM_TAG_LGV 0x4C475600u
#define ESM_TAG_WTH 0x57544800u
#define ESM_TAG_SMS 0x534D5300u
#define ESM_TAG_SML 0x534D4C00u
#define ESM_TAG_SLG 0x534C4700u
#define ESM_TAG_SLL 0x534C4C00u

static inline void orc_philox(uint32_t k0, uint32_t k1, uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3,
                              uint32_t out[4]) {
    for (int r = 0; r < 10; ++r) {
        uint64_t p0 = (uint64_t)0xD2511F53u * c0;
        uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
        uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        uint32_t n0 = hi1 ^ c1 ^ k0, n1 = lo1, n2 = hi0 ^ c3 ^ k1, n3 = lo0;
        c0 = n0; c1 = n1; c2 = n2; c3 = n3;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

static inline double orc_u53(uint32_t a, uint32_t b) {
    return ((double)(a >> 5) * 67108864.0 + (double)(b >> 6)) * (1.0 / 9007199254740992.0);
}

/* two uniforms of one call */
static inline void orc_uniform2(uint64_t seed, uint32_t tag, uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3,
                                double *u0, double *u1) {
    uint32_t x[4];
    orc_philox((uint32_t)seed, (uint32_t)(seed >> 32) ^ tag, c0, c1, c2, c3, x);
    *u0 = orc_u53(x[0], x[1]);
    *u1 = orc_u53(x[2], x[3]);
}

/* standard normal number j of a stream (Box-Muller on the pair j >> 1: cos for even j, sin for odd) */
static inline double orc_normal(uint64_t seed, uint32_t tag, uint32_t j, uint32_t c1, uint32_t c2, uint32_t c3) {
    double u0, u1;
    orc_uniform2(seed, tag, j >> 1, c1, c2, c3, &u0, &u1);
    double rr = sqrt(-2.0 * log(1.0 - u0));
    double a = 6.283185307179586 * u1;
    return (j & 1) ? rr * sin(a) : rr * cos(a);
}
#endif
