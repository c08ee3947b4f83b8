/*
 * philox.h -- oracle side of the shared random stream (test infrastructure).
 *
 * Philox-4x32-10 (Salmon, Moraes, Dror & Shaw, "Parallel random numbers: as
 * easy as 1, 2, 3", SC'11): a counter-based generator. The stream protocol
 * that both the oracle and the GPU engine implement is:
 *
 *   key     = (seed low 32 bits, seed high 32 bits)
 *   counter = (block, domain, event id low 32 bits, event id high 32 bits)
 *
 * Draw n of an event in a domain uses block n / 2; the four 32-bit outputs
 * (x0, x1, x2, x3) of a block give the 64-bit words w0 = x1:x0 (even n) and
 * w1 = x3:x2 (odd n). A word w maps to the uniform double
 *
 *   u = ((w >> 12) + 0.5) * 2^-52,  in ]0, 1[,
 *
 * which is exact in IEEE double arithmetic. Domain 0 feeds the transport
 * (the reference's `context->random`, pumas.h:551), domain 1 the sampling of
 * initial states, so that the latter never shifts transport draws.
 *
 * This copy is part of the oracle and is only used by tests and by the
 * CPU baseline; the GPU engine has its own implementation.
 */
#ifndef ORACLE_PHILOX_H
#define ORACLE_PHILOX_H

#include <stdint.h>

#define ORACLE_PHILOX_M0 0xD2511F53u
#define ORACLE_PHILOX_M1 0xCD9E8D57u
#define ORACLE_PHILOX_W0 0x9E3779B9u
#define ORACLE_PHILOX_W1 0xBB67AE85u

static inline void oracle_philox4x32_10(
    const uint32_t ctr_in[4], const uint32_t key_in[2], uint32_t out[4])
{
        uint32_t c0 = ctr_in[0], c1 = ctr_in[1], c2 = ctr_in[2],
                 c3 = ctr_in[3];
        uint32_t k0 = key_in[0], k1 = key_in[1];
        int round;
        for (round = 0; round < 10; round++) {
                const uint64_t p0 = (uint64_t)ORACLE_PHILOX_M0 * c0;
                const uint64_t p1 = (uint64_t)ORACLE_PHILOX_M1 * c2;
                const uint32_t hi0 = (uint32_t)(p0 >> 32),
                               lo0 = (uint32_t)p0;
                const uint32_t hi1 = (uint32_t)(p1 >> 32),
                               lo1 = (uint32_t)p1;
                c0 = hi1 ^ c1 ^ k0;
                c1 = lo1;
                c2 = hi0 ^ c3 ^ k1;
                c3 = lo0;
                k0 += ORACLE_PHILOX_W0;
                k1 += ORACLE_PHILOX_W1;
        }
        out[0] = c0;
        out[1] = c1;
        out[2] = c2;
        out[3] = c3;
}

static inline double oracle_word_to_uniform(uint64_t w)
{
        return ((double)(w >> 12) + 0.5) * (1.0 / 4503599627370496.0);
}

/* Draw n of (seed, domain, event). */
static inline double oracle_uniform(
    uint64_t seed, uint32_t domain, uint64_t event, uint64_t n)
{
        const uint64_t block = n >> 1;
        const uint32_t ctr[4] = { (uint32_t)block, domain, (uint32_t)event,
                (uint32_t)(event >> 32) };
        const uint32_t key[2] = { (uint32_t)seed, (uint32_t)(seed >> 32) };
        uint32_t x[4];
        oracle_philox4x32_10(ctr, key, x);
        const uint64_t w = (n & 1) ?
            (((uint64_t)x[3] << 32) | x[2]) :
            (((uint64_t)x[1] << 32) | x[0]);
        return oracle_word_to_uniform(w);
}

/* Sequential stream of one event, caching the second word of a block. */
struct oracle_stream {
        uint64_t seed;
        uint64_t event;
        uint64_t n;
        double next;
};

/* Continue the stream at draw n (the position a previous transport call of
 * the same event left it at). */
static inline void oracle_stream_seek(struct oracle_stream * s, uint64_t n)
{
        s->n = n;
        s->next = 0.;
        if (n & 1) s->next = oracle_uniform(s->seed, 0u, s->event, n);
}

static inline double oracle_stream_draw(struct oracle_stream * s)
{
        double u;
        if (s->n & 1) {
                u = s->next;
        } else {
                const uint64_t block = s->n >> 1;
                const uint32_t ctr[4] = { (uint32_t)block, 0u,
                        (uint32_t)s->event, (uint32_t)(s->event >> 32) };
                const uint32_t key[2] = { (uint32_t)s->seed,
                        (uint32_t)(s->seed >> 32) };
                uint32_t x[4];
                oracle_philox4x32_10(ctr, key, x);
                u = oracle_word_to_uniform(((uint64_t)x[1] << 32) | x[0]);
                s->next =
                    oracle_word_to_uniform(((uint64_t)x[3] << 32) | x[2]);
        }
        s->n++;
        return u;
}

#endif
