/*
 * gen_host.c — the seeded draws of spira_gb300/gen.py in C, for host-side
 * test and CPU-baseline inputs too large for numpy temporaries.
 * TEST INFRASTRUCTURE ONLY (part of liboracle.so).
 * draw(seed, stream, i) = splitmix64(i ^ splitmix64(seed * 0xD1B54A32D192ED03 + stream)).
 */
#include <stdint.h>

static uint64_t splitmix64(uint64_t x) {
    uint64_t z = x + 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

/* kind 0: uint32 below(bound); 1: double in [-1, 1); 2: double in [0, 1) */
void orc_gen_draw(uint64_t seed, uint64_t stream, uint64_t c0, uint64_t n, int kind, uint64_t bound, void *out) {
    const uint64_t key = splitmix64(seed * 0xD1B54A32D192ED03ull + stream);
    for (uint64_t i = 0; i < n; ++i) {
        const uint64_t h = splitmix64((c0 + i) ^ key);
        if (kind == 0) {
            ((uint32_t *)out)[i] = (uint32_t)(((h >> 32) * bound) >> 32);
        } else {
            const double u = (double)(h >> 11) * 0x1.0p-53;
            ((double *)out)[i] = kind == 1 ? 2.0 * u - 1.0 : u;
        }
    }
}

/* rows[o_r .. o_r + len[r]) = r */
void orc_gen_expand_rows(const int64_t *len, uint64_t n_rows, uint32_t *rows) {
    uint64_t k = 0;
    for (uint64_t r = 0; r < n_rows; ++r)
        for (int64_t j = 0; j < len[r]; ++j) rows[k++] = (uint32_t)r;
}
