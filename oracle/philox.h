/* Test infrastructure only (oracle side).
 *
 * Philox4x32-10 counter-based generator (J. K. Salmon, M. A. Moraes,
 * R. O. Dror, D. E. Shaw, "Parallel random numbers: as easy as 1, 2, 3",
 * SC'11), restated in plain C, and the integer -> uniform conversions shared
 * with the CUDA sampler.  Known-answer vectors are checked in
 * tests/test_oracle_rng.py. */
#ifndef ISS_ORACLE_PHILOX_H
#define ISS_ORACLE_PHILOX_H
#include <stdint.h>

static inline void orc_philox4x32_10(const uint32_t ctr_in[4], const uint32_t key_in[2],
                                     uint32_t out[4]) {
    uint32_t c0 = ctr_in[0], c1 = ctr_in[1], c2 = ctr_in[2], c3 = ctr_in[3];
    uint32_t k0 = key_in[0], k1 = key_in[1];
    for (int round = 0; round < 10; round++) {
        const uint64_t p0 = (uint64_t)0xD2511F53u * c0;
        const uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
        const uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        const uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        c0 = hi1 ^ c1 ^ k0;
        c1 = lo1;
        c2 = hi0 ^ c3 ^ k1;
        c3 = lo0;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

/* [0, 1) with 23-bit resolution: (x >> 9) 2^-23, the GPU's float built
 * from those bits as a mantissa in [1, 2) minus 1 (exact in float and double) */
static inline double orc_u01(uint32_t x) { return (double)(x >> 9) * (1.0 / 8388608.0); }
/* (0, 1] with 23-bit resolution, safe for log(): 1 - (x >> 9) 2^-23 */
static inline double orc_u01_pos(uint32_t x) {
    return (double)(8388608u - (x >> 9)) * (1.0 / 8388608.0);
}
/* [0, 1) with 53-bit resolution from two words */
static inline double orc_u53(uint32_t a, uint32_t b) {
    return ((double)(a >> 5) * 67108864.0 + (double)(b >> 6)) * (1.0 / 9007199254740992.0);
}

/* Stream tags (bits 16..31 of counter word 3). */
enum { ORC_TAG_CELL = 1, ORC_TAG_TRY = 2, ORC_TAG_COUNT = 3 };

#endif
