/*
 * dmd_rng.h -- random streams and the logarithm used by the event engine.
 *
 * The reference draws every random number from the Intel runtime's drandm
 * (code/main.F90:171-174, 412, 998, 1009-1026, 1041, 1510, 1537, 1564),
 * whose algorithm is not published.  The engine replaces it with the
 * counter-based generator Philox4x32-10 (Salmon, Moraes, Dror, Shaw,
 * "Parallel random numbers: as easy as 1, 2, 3", SC'11), so that a draw is a
 * pure function of (seed, stream, index, draw number) and does not depend on
 * how events are batched or which thread commits them.
 *
 * dmd_log is a logarithm written from its mathematical definition: split
 * x = m * 2^e with m in [sqrt(1/2), sqrt(2)), then
 * log(m) = 2 atanh(s) = 2 (s + s^3/3 + s^5/5 + ...) with s = (m-1)/(m+1)
 * (|s| <= 0.1716, 12 odd terms), and log(x) = e*ln2 + log(m) with ln2 split
 * into a high and a low part.  It uses only IEEE +, -, *, / so the host and
 * the device produce identical bits when compiled without FMA contraction.
 *
 * This header is the specification of the random streams shared by the
 * CUDA engine and the CPU restatement used to check it.
 */
#ifndef DMD_RNG_H
#define DMD_RNG_H

#include <stdint.h>
#include <string.h>

#ifdef __CUDACC__
#define DMD_HD __host__ __device__ __forceinline__
#else
#define DMD_HD static inline
#endif

/* Stream identifiers. */
#define DMD_STREAM_GHOST0  1u  /* first ghost time (code/main.F90:408-415) */
#define DMD_STREAM_GHOST   2u  /* ghost event g: bead, velocities, next time */
#define DMD_STREAM_CAPTURE 3u  /* terminal-bead capture draw of event coll */

typedef struct { uint32_t v[4]; } dmd_u32x4;

DMD_HD void dmd_mulhilo32(uint32_t a, uint32_t b, uint32_t *hi, uint32_t *lo) {
    uint64_t p = (uint64_t)a * (uint64_t)b;
    *hi = (uint32_t)(p >> 32);
    *lo = (uint32_t)p;
}

/* Philox4x32 with 10 rounds. */
DMD_HD dmd_u32x4 dmd_philox4x32_10(dmd_u32x4 ctr, uint32_t k0, uint32_t k1) {
    const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
    const uint32_t W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
    for (int r = 0; r < 10; ++r) {
        uint32_t hi0, lo0, hi1, lo1;
        dmd_mulhilo32(M0, ctr.v[0], &hi0, &lo0);
        dmd_mulhilo32(M1, ctr.v[2], &hi1, &lo1);
        dmd_u32x4 n;
        n.v[0] = hi1 ^ ctr.v[1] ^ k0;
        n.v[1] = lo1;
        n.v[2] = hi0 ^ ctr.v[3] ^ k1;
        n.v[3] = lo0;
        ctr = n;
        k0 += W0;
        k1 += W1;
    }
    return ctr;
}

/* Uniform double in [0,1) with 53 random bits: draw number k of
 * (stream, index) under key seed.  Two draws come from one Philox block. */
DMD_HD double dmd_uniform(uint64_t seed, uint32_t stream, uint64_t index, uint32_t k) {
    dmd_u32x4 c;
    c.v[0] = k >> 1;
    c.v[1] = (uint32_t)index;
    c.v[2] = (uint32_t)(index >> 32);
    c.v[3] = stream;
    dmd_u32x4 o = dmd_philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
    uint64_t w = (k & 1u) ? (((uint64_t)o.v[3] << 32) | o.v[2])
                          : (((uint64_t)o.v[1] << 32) | o.v[0]);
    return (double)(w >> 11) * (1.0 / 9007199254740992.0);
}

/* Natural logarithm for finite x > 0 (see the header comment). */
DMD_HD double dmd_log(double x) {
    uint64_t b;
    memcpy(&b, &x, sizeof b);
    int e = (int)((b >> 52) & 0x7ff);
    if (e == 0) {               /* subnormal: scale into the normal range */
        x = x * 18014398509481984.0;  /* 2^54 */
        memcpy(&b, &x, sizeof b);
        e = (int)((b >> 52) & 0x7ff) - 54;
    }
    e -= 1023;
    b = (b & 0x000fffffffffffffull) | 0x3ff0000000000000ull;  /* m in [1,2) */
    double m;
    memcpy(&m, &b, sizeof m);
    if (m > 1.4142135623730951) { m = m * 0.5; e += 1; }
    double s = (m - 1.0) / (m + 1.0);
    double s2 = s * s;
    /* 2*atanh(s) = 2 s (1 + s2/3 + s2^2/5 + ... + s2^11/23), Horner form */
    double p = 1.0 / 23.0;
    p = p * s2 + 1.0 / 21.0;
    p = p * s2 + 1.0 / 19.0;
    p = p * s2 + 1.0 / 17.0;
    p = p * s2 + 1.0 / 15.0;
    p = p * s2 + 1.0 / 13.0;
    p = p * s2 + 1.0 / 11.0;
    p = p * s2 + 1.0 / 9.0;
    p = p * s2 + 1.0 / 7.0;
    p = p * s2 + 1.0 / 5.0;
    p = p * s2 + 1.0 / 3.0;
    double lm = 2.0 * s + (2.0 * s) * (s2 * p);
    /* ln 2 = ln2_hi + ln2_lo with ln2_hi = ln 2 rounded to 24 bits, so that
     * e * ln2_hi is exact for every exponent of a double. */
    const double ln2_hi = 0.693147182464599609375;
    const double ln2_lo = -1.904654299957768e-09;
    double de = (double)e;
    return (de * ln2_hi + (lm + de * ln2_lo));
}

#endif /* DMD_RNG_H */
