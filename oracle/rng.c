/*
 * RNG restatements. TEST INFRASTRUCTURE ONLY (CPU oracle).
 *
 * PCG32: O'Neill 2014, "PCG: A Family of Simple Fast Space-Efficient Statistically Good
 * Algorithms for Random Number Generation" -- XSH-RR output, 64-bit LCG state, odd stream
 * increment, srandom(initstate, initseq) seeding and Brown-style O(log n) jump-ahead. Not part of
 * the reference; it is the project RNG behind the benchmark workloads.
 *
 * xxhash32 / lcg / rnd: the reference's shader RNG pair, restated from
 * shaders/slang/utils/hash.slang:47-56 (xxhash32 mixing of two words, Jarzynski & Olano 2020) and
 * shaders/slang/utils/random.slang:27-36 (Numerical-Recipes LCG, 24-bit float).
 */
#include "oracle.h"

#define PCG_MULT 6364136223846793005ull

uint32_t orc_pcg32_next(orc_pcg32 *g)
{
    uint64_t old = g->state;
    g->state = old * PCG_MULT + g->inc;
    uint32_t xs = (uint32_t)(((old >> 18u) ^ old) >> 27u);
    uint32_t rot = (uint32_t)(old >> 59u);
    return (xs >> rot) | (xs << ((0u - rot) & 31u));
}

void orc_pcg32_seed(orc_pcg32 *g, uint64_t initstate, uint64_t initseq)
{
    g->state = 0u;
    g->inc = (initseq << 1u) | 1u;
    orc_pcg32_next(g);
    g->state += initstate;
    orc_pcg32_next(g);
}

void orc_pcg32_advance(orc_pcg32 *g, uint64_t delta)
{
    uint64_t cur_mult = PCG_MULT, cur_plus = g->inc;
    uint64_t acc_mult = 1u, acc_plus = 0u;
    while(delta > 0)
    {
        if(delta & 1u)
        {
            acc_mult *= cur_mult;
            acc_plus = acc_plus * cur_mult + cur_plus;
        }
        cur_plus = (cur_mult + 1u) * cur_plus;
        cur_mult *= cur_mult;
        delta >>= 1u;
    }
    g->state = acc_mult * g->state + acc_plus;
}

/* uniform float in [0, 1): the top 24 bits scaled by 2^-24 (exact) */
float orc_u01(uint32_t x) { return (float)(x >> 8) * 0x1p-24f; }

void orc_pcg32_fill(uint64_t initstate, uint64_t initseq, uint64_t skip, uint32_t n, uint32_t *out)
{
    orc_pcg32 g;
    orc_pcg32_seed(&g, initstate, initseq);
    orc_pcg32_advance(&g, skip);
    for(uint32_t i = 0; i < n; ++i) out[i] = orc_pcg32_next(&g);
}

/* hash.slang:47-56 */
uint32_t orc_xxhash32(uint32_t lhs, uint32_t rhs)
{
    const uint32_t P2 = 2246822519u, P3 = 3266489917u, P4 = 668265263u, P5 = 374761393u;
    uint32_t h = lhs + P5 + rhs * P3;
    h = P4 * ((h << 17) | (h >> (32 - 17)));
    h = P2 * (h ^ (h >> 15));
    h = P3 * (h ^ (h >> 13));
    return h ^ (h >> 16);
}

/* random.slang:27-33 */
uint32_t orc_lcg(uint32_t *prev)
{
    *prev = 1664525u * *prev + 1013904223u;
    return *prev & 0x00FFFFFFu;
}

/* random.slang:36 */
float orc_rnd(uint32_t *prev) { return (float)orc_lcg(prev) / (float)0x01000000; }
