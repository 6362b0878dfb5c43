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

/* Matrix families of the selector corpus and the batched workload. */
enum spg_gen_family {
    SPG_FAM_BANDED = 0,     /* p = bandwidth: cols r - p/2 .. r + p/2 (clipped) */
    SPG_FAM_BLOCKDIAG = 1,  /* p = block size: dense diagonal blocks */
    SPG_FAM_POWERLAW = 2,   /* lengths min(cap, max(1, rint(Z * scale))), Z ~ table d_cdf[p] */
    SPG_FAM_UNIFORM = 3,    /* p uniform columns per row */
    SPG_FAM_STENCIL2D = 4,  /* p = grid side (n = p^2): 5-point stencil */
    SPG_FAM_STENCIL3D = 5,  /* p = grid side (n = p^3): 7-point stencil */
    SPG_FAM_POISSON = 6     /* lengths ~ Poisson(lambda), uniform columns */
};

/* Staged inserts (rows, cols, vals) of one family member, row by row; random
 * columns may repeat within a row (lock() keeps the last write). Two calls:
 * with d_rows == NULL only *m (the number of inserts) is computed. d_cdf
 * (device, p doubles, cumulative) is read by SPG_FAM_POWERLAW only. Values
 * are uniform in [-1, 1) (stencils: the diagonal is the stencil size minus
 * one, off-diagonals -1). */
int spg_gen_family(spg_ctx *ctx, int family, uint64_t n_rows, uint64_t p, double lambda_or_scale,
                   const double *d_cdf, uint64_t seed, uint32_t *d_rows, uint32_t *d_cols, double *d_vals,
                   uint64_t *m);

#ifdef __cplusplus
}
#endif
#endif /* SPG_GEN_H */
