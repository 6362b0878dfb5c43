/*
 * spg_gen.h — device-side seeded draws for synthetic workloads (benchmark and
 * test inputs). Not part of Spira's interface: Spira has no generators, its
 * benchmark draws inputs with std::mt19937 on the host
 * (bench/spira_bench.cpp:57-104). These entry points produce, on the GPU,
 * exactly the values spira_gb300/gen.py draws on the host: every draw is
 * splitmix64(counter ^ splitmix64(seed * 0xD1B54A32D192ED03 + stream)).
 */
#ifndef SPG_GEN_H
#define SPG_GEN_H

#include <stdint.h>

#include "spg.h"

#ifdef __cplusplus
extern "C" {
#endif

enum spg_gen_kind {
    SPG_GEN_BELOW_U32 = 0, /* uint32 in [0, bound): ((h >> 32) * bound) >> 32 */
    SPG_GEN_SYM_F64 = 1,   /* double in [-1, 1): 2 * ((h >> 11) * 2^-53) - 1 */
    SPG_GEN_UNIT_F64 = 2   /* double in [0, 1) */
};

/* out[i] = draw(seed, stream, counter0 + i) for i < n, on the context stream. */
int spg_gen_draw(spg_ctx *ctx, uint64_t seed, uint64_t stream, uint64_t counter0, uint64_t n, int kind,
                 uint64_t bound, void *d_out);

/* Row ids of a CSR-shaped staging batch: for row r with length lengths[r]
 * (device int64, n_rows entries), writes r into rows[o_r .. o_r + lengths[r])
 * where o_r is the exclusive prefix sum. *total receives sum(lengths). */
int spg_gen_expand_rows(spg_ctx *ctx, const int64_t *d_lengths, uint64_t n_rows, uint32_t *d_rows,
                        uint64_t *total);

#ifdef __cplusplus
}
#endif
#endif /* SPG_GEN_H */
