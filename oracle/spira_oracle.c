/*
 * spira_oracle.c — CPU restatement of Spira's sparse hot path.
 *
 * TEST INFRASTRUCTURE ONLY. This file is the reference the GPU engine is
 * compared against and the CPU baseline bench.py times beside it. The
 * product (libspg.so) never links, loads or calls it.
 *
 * Each function restates one Spira algorithm (file:line inside the Spira
 * source tree). Pinned against Spira itself: tests/test_oracle_pin.py runs
 * these functions and Spira's own code (compiled from its sources by
 * oracle/Makefile into oracle/_ref/) on the same seeded inputs, and
 * tests/golden/ holds fixtures Spira produced.
 *
 * Floating point: compile with -ffp-contract=off; every fused multiply-add
 * that Spira's compiled code may emit is written out as fma() and selected
 * by a `fused` flag, so results are identical on x86-64 and aarch64.
 */
#define _POSIX_C_SOURCE 200809L /* clock_gettime under -std=c11 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#define ORC_OK 0
#define ORC_ERR_ALLOC 4
#define ORC_ERR_RANGE 3

typedef struct {
    uint64_t n_rows, n_cols, nnz, capacity;
    uint64_t *off;  /* n_rows + 1; NULL = never locked */
    uint32_t *cols; /* capacity */
    double *vals;   /* capacity */
} orc_csr;

/* traits.hpp:73-80 — floating point is_zero(x) is abs(x) <= 0: +-0 are zero, NaN is not. */
static int is_zero(double v) { return fabs(v) <= 0.0; }

void orc_csr_free(orc_csr *A) {
    free(A->off);
    free(A->cols);
    free(A->vals);
    A->off = NULL;
    A->cols = NULL;
    A->vals = NULL;
    A->nnz = A->capacity = 0;
}

/* ------------------------------------------------------------------------
 * lock(): aos_array_buffer.hpp:76-101 (sort_and_dedup_keep_zeros),
 * csr_build.hpp:32-98 (build_csr), csr_build.hpp:126-488 (merge_csr),
 * driven as matrix.hpp:277-342.
 * ---------------------------------------------------------------------- */
typedef struct {
    uint32_t col;
    uint64_t seq; /* insertion order */
    double val;
} orc_ent;

/* reverse + stable_sort by column, first of each run = the last write:
 * the same order as sorting by (col ascending, seq descending). */
static int ent_cmp(const void *a, const void *b) {
    const orc_ent *x = (const orc_ent *)a, *y = (const orc_ent *)b;
    if (x->col != y->col) return x->col < y->col ? -1 : 1;
    if (x->seq != y->seq) return x->seq > y->seq ? -1 : 1;
    return 0;
}

int orc_lock(orc_csr *A, const uint32_t *rows, const uint32_t *cols, const double *vals, uint64_t m) {
    const uint64_t n = A->n_rows;
    for (uint64_t i = 0; i < m; ++i)
        if ((uint64_t)rows[i] >= n || (uint64_t)cols[i] >= A->n_cols) return ORC_ERR_RANGE;
    /* Row buffers in insertion order (counting sort by row keeps order). */
    uint64_t *bstart = (uint64_t *)calloc(n + 1, sizeof(uint64_t));
    orc_ent *ents = (orc_ent *)malloc((m ? m : 1) * sizeof(orc_ent));
    uint64_t *cursor = (uint64_t *)malloc((n + 1) * sizeof(uint64_t));
    if (!bstart || !ents || !cursor) return ORC_ERR_ALLOC;
    for (uint64_t i = 0; i < m; ++i) bstart[rows[i] + 1]++;
    for (uint64_t r = 0; r < n; ++r) bstart[r + 1] += bstart[r];
    memcpy(cursor, bstart, (n + 1) * sizeof(uint64_t));
    for (uint64_t i = 0; i < m; ++i) {
        orc_ent e = {cols[i], i, vals[i]};
        ents[cursor[rows[i]]++] = e;
    }
    /* sort_and_dedup_keep_zeros per row: blen[r] = deduplicated length */
    uint64_t *blen = (uint64_t *)calloc(n ? n : 1, sizeof(uint64_t));
    if (!blen) return ORC_ERR_ALLOC;
    for (uint64_t r = 0; r < n; ++r) {
        orc_ent *b = ents + bstart[r];
        const uint64_t k = bstart[r + 1] - bstart[r];
        if (k > 1) qsort(b, k, sizeof(orc_ent), ent_cmp);
        uint64_t w = 0;
        for (uint64_t i = 0; i < k; ++i)
            if (w == 0 || b[i].col != b[w - 1].col) b[w++] = b[i];
        blen[r] = w;
    }
    int rc = ORC_OK;
    if (!A->off) {
        /* build_csr: count non-zeros, prefix, fill (csr_build.hpp:41-95). */
        uint64_t *off = (uint64_t *)malloc((n + 1) * sizeof(uint64_t));
        uint64_t total = 0;
        off[0] = 0;
        for (uint64_t r = 0; r < n; ++r) {
            const orc_ent *b = ents + bstart[r];
            for (uint64_t i = 0; i < blen[r]; ++i)
                if (!is_zero(b[i].val)) ++total;
            off[r + 1] = total;
        }
        uint32_t *oc = (uint32_t *)malloc((total ? total : 1) * sizeof(uint32_t));
        double *ov = (double *)malloc((total ? total : 1) * sizeof(double));
        uint64_t k = 0;
        for (uint64_t r = 0; r < n; ++r) {
            const orc_ent *b = ents + bstart[r];
            for (uint64_t i = 0; i < blen[r]; ++i)
                if (!is_zero(b[i].val)) {
                    oc[k] = b[i].col;
                    ov[k] = b[i].val;
                    ++k;
                }
        }
        A->off = off;
        A->cols = oc;
        A->vals = ov;
        A->nnz = total;
        A->capacity = total;
    } else {
        /* merge_csr: capacity rule (csr_build.hpp:139-145), per-row two
         * pointer merge on dirty rows, copy on clean rows (csr_build.hpp:
         * 195-212, 268-303). Reuse and grow paths produce the same arrays;
         * only the capacity differs. */
        uint64_t total_ub = A->nnz;
        for (uint64_t r = 0; r < n; ++r) total_ub += blen[r];
        const uint64_t cap = (total_ub <= A->capacity) ? A->capacity : total_ub + total_ub / 2;
        uint64_t *off = (uint64_t *)malloc((n + 1) * sizeof(uint64_t));
        uint32_t *oc = (uint32_t *)malloc((cap ? cap : 1) * sizeof(uint32_t));
        double *ov = (double *)malloc((cap ? cap : 1) * sizeof(double));
        uint64_t wp = 0;
        off[0] = 0;
        for (uint64_t r = 0; r < n; ++r) {
            const uint64_t ob = A->off[r], oe = A->off[r + 1];
            const int dirty = bstart[r + 1] != bstart[r];
            if (!dirty) {
                for (uint64_t k = ob; k < oe; ++k) {
                    oc[wp] = A->cols[k];
                    ov[wp] = A->vals[k];
                    ++wp;
                }
                off[r + 1] = wp;
                continue;
            }
            const orc_ent *b = ents + bstart[r];
            uint64_t oi = ob, bi = 0;
            while (oi < oe && bi < blen[r]) {
                const uint32_t occ = A->cols[oi], bc = b[bi].col;
                if (occ < bc) {
                    if (!is_zero(A->vals[oi])) { oc[wp] = occ; ov[wp] = A->vals[oi]; ++wp; }
                    ++oi;
                } else if (bc < occ) {
                    if (!is_zero(b[bi].val)) { oc[wp] = bc; ov[wp] = b[bi].val; ++wp; }
                    ++bi;
                } else {
                    if (!is_zero(b[bi].val)) { oc[wp] = bc; ov[wp] = b[bi].val; ++wp; }
                    ++oi;
                    ++bi;
                }
            }
            for (; oi < oe; ++oi)
                if (!is_zero(A->vals[oi])) { oc[wp] = A->cols[oi]; ov[wp] = A->vals[oi]; ++wp; }
            for (; bi < blen[r]; ++bi)
                if (!is_zero(b[bi].val)) { oc[wp] = b[bi].col; ov[wp] = b[bi].val; ++wp; }
            off[r + 1] = wp;
        }
        free(A->off);
        free(A->cols);
        free(A->vals);
        A->off = off;
        A->cols = oc;
        A->vals = ov;
        A->nnz = wp;
        A->capacity = cap;
    }
    free(bstart);
    free(ents);
    free(cursor);
    free(blen);
    return rc;
}

/* ------------------------------------------------------------------------
 * SpMV
 * ---------------------------------------------------------------------- */

/* serial/spmv.hpp:44-55 and dot_scalar.cpp:4-11: acc += x[col] * val in CSR
 * order; fused = 1 is the same loop under FMA contraction. */
void orc_spmv_scalar(const uint64_t *off, const uint32_t *cols, const double *vals, uint64_t n_rows,
                     const double *x, double *y, int fused) {
    for (uint64_t i = 0; i < n_rows; ++i) {
        double acc = 0.0;
        for (uint64_t k = off[i]; k < off[i + 1]; ++k)
            acc = fused ? fma(x[cols[k]], vals[k], acc) : acc + x[cols[k]] * vals[k];
        y[i] = acc;
    }
}

/* kernel::sparse_dot_double in its SIMD shape: 4 accumulators of `lanes`
 * lanes, a 4*lanes main loop, a lanes-wide second loop into accumulator 0,
 * (a0+a1)+(a2+a3), a horizontal tree reduce (lane i + lane i+h, h halving),
 * then a scalar tail.  lanes = 2: dot_neon.cpp:27-76 (GCC contracts the tail
 * into fma on aarch64: tail_fused = 1); lanes = 8: dot_avx512.cpp:7-56 (that
 * file is built without -mfma, its tail stays mul + add: tail_fused = 0).
 * Pinned bit-exact against Spira's AVX-512 build by tests/test_oracle_pin.py. */
static double dot_blocked(const double *vals, const uint32_t *cols, const double *x, uint64_t n, int lanes,
                          int tail_fused) {
    double a[4][8];
    for (int q = 0; q < 4; ++q)
        for (int l = 0; l < lanes; ++l) a[q][l] = 0.0;
    uint64_t i = 0;
    for (; i + 4 * (uint64_t)lanes <= n; i += 4 * (uint64_t)lanes)
        for (int q = 0; q < 4; ++q)
            for (int l = 0; l < lanes; ++l) {
                const uint64_t k = i + (uint64_t)q * lanes + l;
                a[q][l] = fma(vals[k], x[cols[k]], a[q][l]);
            }
    for (; i + (uint64_t)lanes <= n; i += lanes)
        for (int l = 0; l < lanes; ++l) a[0][l] = fma(vals[i + l], x[cols[i + l]], a[0][l]);
    double v[8];
    for (int l = 0; l < lanes; ++l) v[l] = (a[0][l] + a[1][l]) + (a[2][l] + a[3][l]);
    for (int h = lanes / 2; h >= 1; h /= 2)
        for (int l = 0; l < h; ++l) v[l] = v[l] + v[l + h];
    double acc = v[0];
    for (; i < n; ++i) acc = tail_fused ? fma(x[cols[i]], vals[i], acc) : acc + x[cols[i]] * vals[i];
    return acc;
}

void orc_spmv_blocked(const uint64_t *off, const uint32_t *cols, const double *vals, uint64_t n_rows,
                      const double *x, double *y, int lanes, int tail_fused) {
    for (uint64_t r = 0; r < n_rows; ++r)
        y[r] = dot_blocked(vals + off[r], cols + off[r], x, off[r + 1] - off[r], lanes, tail_fused);
}

/* parallel/algorithms/spmv.hpp:125-161 on parallel_matrix's static row
 * partitions row_start = t*n/T (parallel_matrix.hpp:300-301), one pthread
 * per partition, sparse_dot_double per row. */
typedef struct {
    const uint64_t *off;
    const uint32_t *cols;
    const double *vals;
    const double *x;
    double *y;
    uint64_t r0, r1;
    int lanes, tail_fused;
} orc_par_arg;

static void *par_worker(void *p) {
    orc_par_arg *a = (orc_par_arg *)p;
    for (uint64_t r = a->r0; r < a->r1; ++r)
        a->y[r] = dot_blocked(a->vals + a->off[r], a->cols + a->off[r], a->x, a->off[r + 1] - a->off[r], a->lanes,
                              a->tail_fused);
    return NULL;
}

int orc_spmv_parallel(const uint64_t *off, const uint32_t *cols, const double *vals, uint64_t n_rows,
                      const double *x, double *y, int n_threads, int lanes, int tail_fused) {
    if (n_threads < 1) n_threads = 1;
    pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * (size_t)n_threads);
    orc_par_arg *args = (orc_par_arg *)malloc(sizeof(orc_par_arg) * (size_t)n_threads);
    if (!th || !args) return ORC_ERR_ALLOC;
    for (int t = 0; t < n_threads; ++t) {
        args[t].off = off;
        args[t].cols = cols;
        args[t].vals = vals;
        args[t].x = x;
        args[t].y = y;
        args[t].r0 = (uint64_t)t * n_rows / (uint64_t)n_threads;
        args[t].r1 = (uint64_t)(t + 1) * n_rows / (uint64_t)n_threads;
        args[t].lanes = lanes;
        args[t].tail_fused = tail_fused;
    }
    for (int t = 1; t < n_threads; ++t) pthread_create(&th[t], NULL, par_worker, &args[t]);
    par_worker(&args[0]);
    for (int t = 1; t < n_threads; ++t) pthread_join(th[t], NULL);
    free(th);
    free(args);
    return ORC_OK;
}

/* Compensated (Neumaier) row sums of the exact products' rounded values plus
 * their error terms (TwoProduct via fma), giving y to ~2 ulp; scale[r] =
 * sum |a_rk x_k|, the condition-aware denominator of the parity bound. */
void orc_spmv_compensated(const uint64_t *off, const uint32_t *cols, const double *vals, uint64_t n_rows,
                          const double *x, double *y, double *scale) {
    for (uint64_t r = 0; r < n_rows; ++r) {
        double s = 0.0, c = 0.0, a = 0.0;
        for (uint64_t k = off[r]; k < off[r + 1]; ++k) {
            const double p = vals[k] * x[cols[k]];
            const double pe = fma(vals[k], x[cols[k]], -p);
            const double t = s + p;
            if (fabs(s) >= fabs(p)) c += (s - t) + p;
            else c += (p - t) + s;
            s = t;
            c += pe;
            a += fabs(p);
        }
        y[r] = s + c;
        if (scale) scale[r] = a;
    }
}

/* ------------------------------------------------------------------------
 * SpGEMM — serial/spgemm.hpp:12-53: Gustavson row by row, acc[j] += a_ik *
 * b_kj with k ascending along A's row, entries with v != 0 inserted, then
 * C.lock() (one insert per (i, j): sorted, nothing to dedup, build keeps
 * non-zeros). The hash map's iteration order only permutes inserts that
 * lock() sorts again, so a dense accumulator with a touched list is the
 * same computation.
 * ---------------------------------------------------------------------- */
int orc_spgemm(const orc_csr *A, const orc_csr *B, orc_csr *C, int fused) {
    const uint64_t m = A->n_rows, n = B->n_cols;
    double *acc = (double *)malloc((n ? n : 1) * sizeof(double));
    unsigned char *seen = (unsigned char *)calloc(n ? n : 1, 1);
    uint32_t *touched = (uint32_t *)malloc((n ? n : 1) * sizeof(uint32_t));
    uint64_t cap = 1024, nnz = 0;
    uint32_t *cc = (uint32_t *)malloc(cap * sizeof(uint32_t));
    double *cv = (double *)malloc(cap * sizeof(double));
    uint64_t *off = (uint64_t *)malloc((m + 1) * sizeof(uint64_t));
    if (!acc || !seen || !touched || !cc || !cv || !off) return ORC_ERR_ALLOC;
    off[0] = 0;
    for (uint64_t i = 0; i < m; ++i) {
        uint64_t nt = 0;
        for (uint64_t ka = A->off[i]; ka < A->off[i + 1]; ++ka) {
            const uint32_t k = A->cols[ka];
            const double a = A->vals[ka];
            for (uint64_t kb = B->off[k]; kb < B->off[k + 1]; ++kb) {
                const uint32_t j = B->cols[kb];
                if (!seen[j]) {
                    seen[j] = 1;
                    acc[j] = 0.0;
                    touched[nt++] = j;
                }
                acc[j] = fused ? fma(a, B->vals[kb], acc[j]) : acc[j] + a * B->vals[kb];
            }
        }
        /* sort touched columns (insertion order differs, lock() sorts) */
        for (uint64_t p = 1; p < nt; ++p) {
            uint32_t v = touched[p];
            uint64_t q = p;
            while (q > 0 && touched[q - 1] > v) {
                touched[q] = touched[q - 1];
                --q;
            }
            touched[q] = v;
        }
        for (uint64_t p = 0; p < nt; ++p) {
            const uint32_t j = touched[p];
            seen[j] = 0;
            if (acc[j] != 0.0) { /* spgemm.hpp:44 v != V{} */
                if (nnz == cap) {
                    cap *= 2;
                    cc = (uint32_t *)realloc(cc, cap * sizeof(uint32_t));
                    cv = (double *)realloc(cv, cap * sizeof(double));
                    if (!cc || !cv) return ORC_ERR_ALLOC;
                }
                cc[nnz] = j;
                cv[nnz] = acc[j];
                ++nnz;
            }
        }
        off[i + 1] = nnz;
    }
    free(acc);
    free(seen);
    free(touched);
    C->n_rows = m;
    C->n_cols = n;
    C->off = off;
    C->cols = cc;
    C->vals = cv;
    C->nnz = nnz;
    C->capacity = nnz;
    return ORC_OK;
}

/* Number of products sum_i sum_{k in A_i} nnz(B_k) (the SpGEMM work). */
uint64_t orc_spgemm_products(const orc_csr *A, const orc_csr *B) {
    uint64_t p = 0;
    for (uint64_t ka = 0; ka < A->nnz; ++ka) {
        const uint32_t k = A->cols[ka];
        p += B->off[k + 1] - B->off[k];
    }
    return p;
}

/* ------------------------------------------------------------------------
 * Transpose — serial/transpose.hpp:35-156: histogram of columns, prefix,
 * row-ordered cursor scatter (ascending source row in every output row).
 * ---------------------------------------------------------------------- */
int orc_transpose(const orc_csr *A, orc_csr *T) {
    const uint64_t r = A->n_rows, c = A->n_cols, nnz = A->nnz;
    uint64_t *off = (uint64_t *)calloc(c + 1, sizeof(uint64_t));
    uint64_t *cur = (uint64_t *)malloc((c + 1) * sizeof(uint64_t));
    uint32_t *tc = (uint32_t *)malloc((nnz ? nnz : 1) * sizeof(uint32_t));
    double *tv = (double *)malloc((nnz ? nnz : 1) * sizeof(double));
    if (!off || !cur || !tc || !tv) return ORC_ERR_ALLOC;
    for (uint64_t k = 0; k < nnz; ++k) off[A->cols[k] + 1]++;
    for (uint64_t j = 0; j < c; ++j) off[j + 1] += off[j];
    memcpy(cur, off, (c + 1) * sizeof(uint64_t));
    for (uint64_t i = 0; i < r; ++i)
        for (uint64_t k = A->off[i]; k < A->off[i + 1]; ++k) {
            const uint64_t p = cur[A->cols[k]]++;
            tc[p] = (uint32_t)i;
            tv[p] = A->vals[k];
        }
    free(cur);
    T->n_rows = c;
    T->n_cols = r;
    T->off = off;
    T->cols = tc;
    T->vals = tv;
    T->nnz = nnz;
    T->capacity = nnz;
    return ORC_OK;
}

/* ------------------------------------------------------------------------
 * Matrix addition — serial/matrix_addition.hpp:34-110: per row a two-pointer
 * merge of A's and B's slices; equal columns give a + b, inserted unless the
 * sum is zero; other entries are inserted as they are; the output matrix is
 * then locked, and build_csr drops every zero value (csr_build.hpp:49,71).
 * ---------------------------------------------------------------------- */
int orc_add(const orc_csr *A, const orc_csr *B, orc_csr *C) {
    const uint64_t n = A->n_rows, cap = A->nnz + B->nnz;
    uint64_t *off = (uint64_t *)calloc(n + 1, sizeof(uint64_t));
    uint32_t *cc = (uint32_t *)malloc((cap ? cap : 1) * sizeof(uint32_t));
    double *cv = (double *)malloc((cap ? cap : 1) * sizeof(double));
    if (!off || !cc || !cv) return ORC_ERR_ALLOC;
    uint64_t w = 0;
    for (uint64_t r = 0; r < n; ++r) {
        uint64_t i = A->off ? A->off[r] : 0, ie = A->off ? A->off[r + 1] : 0;
        uint64_t j = B->off ? B->off[r] : 0, je = B->off ? B->off[r + 1] : 0;
        while (i < ie || j < je) {
            uint32_t col;
            double v;
            if (j >= je || (i < ie && A->cols[i] < B->cols[j])) {
                col = A->cols[i];
                v = A->vals[i++];
            } else if (i >= ie || B->cols[j] < A->cols[i]) {
                col = B->cols[j];
                v = B->vals[j++];
            } else {
                col = A->cols[i];
                v = A->vals[i++] + B->vals[j++];
            }
            if (!is_zero(v)) { /* the sum test of the merge, and the lock's zero drop */
                cc[w] = col;
                cv[w] = v;
                ++w;
            }
        }
        off[r + 1] = w;
    }
    C->n_rows = n;
    C->n_cols = A->n_cols;
    C->off = off;
    C->cols = cc;
    C->vals = cv;
    C->nnz = w;
    C->capacity = w;
    return ORC_OK;
}

/* ------------------------------------------------------------------------
 * Scalar multiply / divide — serial/scalars.hpp:22-35 and 51-67 (copy path):
 * every value times (or over) the scalar, inserted into a fresh matrix that
 * is then locked (zero results dropped).
 * ---------------------------------------------------------------------- */
int orc_scale(const orc_csr *A, double s, int divide, orc_csr *C) {
    const uint64_t n = A->n_rows, m = A->nnz;
    uint64_t *off = (uint64_t *)calloc(n + 1, sizeof(uint64_t));
    uint32_t *cc = (uint32_t *)malloc((m ? m : 1) * sizeof(uint32_t));
    double *cv = (double *)malloc((m ? m : 1) * sizeof(double));
    if (!off || !cc || !cv) return ORC_ERR_ALLOC;
    uint64_t w = 0;
    for (uint64_t r = 0; r < n; ++r) {
        for (uint64_t k = A->off[r]; k < A->off[r + 1]; ++k) {
            const double v = divide ? A->vals[k] / s : A->vals[k] * s;
            if (!is_zero(v)) {
                cc[w] = A->cols[k];
                cv[w] = v;
                ++w;
            }
        }
        off[r + 1] = w;
    }
    C->n_rows = n;
    C->n_cols = A->n_cols;
    C->off = off;
    C->cols = cc;
    C->vals = cv;
    C->nnz = w;
    C->capacity = w;
    return ORC_OK;
}

/* Row sums of a locked matrix — csr_storage_soa.hpp:114-120 via
 * row.hpp:208-216: acc += v in CSR order from 0. */
void orc_row_sums(const uint64_t *off, const double *vals, uint64_t n_rows, double *out) {
    for (uint64_t r = 0; r < n_rows; ++r) {
        double acc = 0.0;
        for (uint64_t k = off[r]; k < off[r + 1]; ++k) acc += vals[k];
        out[r] = acc;
    }
}

/* nnz-balanced boundaries — parallel/partition.hpp:78-126, with the row nnz
 * prefix taken from the CSR offsets: bounds[t] = lower_bound(prefix from
 * bounds[t - 1], max(1, t * nnz / T)), clamped to n; uniform when nnz == 0;
 * {0, n, ..., n} for T <= 1 or no rows. */
void orc_partition(const uint64_t *off, uint64_t n_rows, uint64_t T, uint64_t *bounds) {
    bounds[0] = 0;
    for (uint64_t t = 1; t <= T; ++t) bounds[t] = n_rows;
    if (T <= 1 || n_rows == 0) return;
    const uint64_t total = off[n_rows];
    if (total == 0) {
        for (uint64_t t = 1; t < T; ++t) bounds[t] = t * n_rows / T;
        return;
    }
    for (uint64_t t = 1; t < T; ++t) {
        uint64_t target = t * total / T;
        if (target < 1) target = 1;
        uint64_t lo = bounds[t - 1], hi = n_rows + 1;
        while (lo < hi) {
            const uint64_t mid = lo + (hi - lo) / 2;
            if (off[mid] < target) lo = mid + 1;
            else hi = mid;
        }
        bounds[t] = lo < n_rows ? lo : n_rows;
    }
}

/* ------------------------------------------------------------------------
 * Parallel forms, for the multi-core CPU baseline of lock, SpGEMM and
 * transpose: parallel_matrix's static row partitions row_start = t*n/T
 * (parallel_matrix.hpp:300-301), one pthread per partition.
 * ---------------------------------------------------------------------- */
static double orc_now(void) {
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

static uint64_t part_of(const uint64_t *bounds, int T, uint64_t r) {
    int lo = 0, hi = T; /* last t with bounds[t] <= r */
    while (hi - lo > 1) {
        const int mid = (lo + hi) / 2;
        if (bounds[mid] <= r) lo = mid;
        else hi = mid;
    }
    return (uint64_t)lo;
}

/* lock(): parallel_matrix::lock (parallel_matrix.hpp:321-405) locks each
 * partition's own matrix on its own thread. insert() already routed every
 * triple to its partition's buffers (parallel_matrix.hpp:581-602), so that
 * routing is done here before the clock starts. */
typedef struct {
    orc_csr part;
    uint32_t *rows, *cols;
    double *vals;
    uint64_t m;
    int rc;
} orc_lock_part;

static void *lock_worker(void *p) {
    orc_lock_part *q = (orc_lock_part *)p;
    q->rc = orc_lock(&q->part, q->rows, q->cols, q->vals, q->m);
    return NULL;
}

/* Locks n_epochs epochs of staged inserts into an n_rows x n_cols matrix
 * kept as T partitions; seconds[e] = wall time of epoch e's parallel lock;
 * *nnz = stored entries after the last epoch. */
int orc_lock_parallel_time(uint64_t n_rows, uint64_t n_cols, int T, int n_epochs, const uint32_t *const *rows,
                           const uint32_t *const *cols, const double *const *vals, const uint64_t *ms,
                           double *seconds, uint64_t *nnz) {
    if (T < 1) T = 1;
    uint64_t *bounds = (uint64_t *)malloc(sizeof(uint64_t) * (size_t)(T + 1));
    orc_lock_part *parts = (orc_lock_part *)calloc((size_t)T, sizeof(orc_lock_part));
    pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * (size_t)T);
    uint64_t *cnt = (uint64_t *)malloc(sizeof(uint64_t) * (size_t)T);
    if (!bounds || !parts || !th || !cnt) return ORC_ERR_ALLOC;
    for (int t = 0; t <= T; ++t) bounds[t] = (uint64_t)t * n_rows / (uint64_t)T;
    for (int t = 0; t < T; ++t) {
        parts[t].part.n_rows = bounds[t + 1] - bounds[t];
        parts[t].part.n_cols = n_cols;
    }
    int rc = ORC_OK;
    for (int e = 0; e < n_epochs && rc == ORC_OK; ++e) {
        const uint64_t m = ms[e];
        for (int t = 0; t < T; ++t) cnt[t] = 0;
        for (uint64_t i = 0; i < m; ++i) {
            if ((uint64_t)rows[e][i] >= n_rows || (uint64_t)cols[e][i] >= n_cols) return ORC_ERR_RANGE;
            cnt[part_of(bounds, T, rows[e][i])]++;
        }
        for (int t = 0; t < T; ++t) {
            parts[t].rows = (uint32_t *)malloc((cnt[t] ? cnt[t] : 1) * sizeof(uint32_t));
            parts[t].cols = (uint32_t *)malloc((cnt[t] ? cnt[t] : 1) * sizeof(uint32_t));
            parts[t].vals = (double *)malloc((cnt[t] ? cnt[t] : 1) * sizeof(double));
            if (!parts[t].rows || !parts[t].cols || !parts[t].vals) return ORC_ERR_ALLOC;
            parts[t].m = 0;
        }
        for (uint64_t i = 0; i < m; ++i) { /* insertion order kept within each partition */
            const uint64_t t = part_of(bounds, T, rows[e][i]);
            orc_lock_part *q = &parts[t];
            q->rows[q->m] = (uint32_t)(rows[e][i] - bounds[t]);
            q->cols[q->m] = cols[e][i];
            q->vals[q->m] = vals[e][i];
            ++q->m;
        }
        const double t0 = orc_now();
        for (int t = 1; t < T; ++t) pthread_create(&th[t], NULL, lock_worker, &parts[t]);
        lock_worker(&parts[0]);
        for (int t = 1; t < T; ++t) pthread_join(th[t], NULL);
        seconds[e] = orc_now() - t0;
        for (int t = 0; t < T; ++t) {
            if (parts[t].rc != ORC_OK) rc = parts[t].rc;
            free(parts[t].rows);
            free(parts[t].cols);
            free(parts[t].vals);
        }
    }
    uint64_t total = 0;
    for (int t = 0; t < T; ++t) {
        total += parts[t].part.nnz;
        orc_csr_free(&parts[t].part);
    }
    *nnz = total;
    free(bounds);
    free(parts);
    free(th);
    free(cnt);
    return rc;
}

/* SpGEMM: parallel/algorithms/spgemm.hpp:27-69 — each partition's rows of A
 * computed by its own thread (Gustavson, ascending k, drop zero sums, as
 * orc_spgemm), then the partitions' rows assembled into C. */
typedef struct {
    const orc_csr *A, *B;
    uint64_t r0, r1;
    int fused;
    orc_csr out; /* rows r0..r1-1 of C */
    int rc;
} orc_gemm_part;

static void *gemm_worker(void *p) {
    orc_gemm_part *q = (orc_gemm_part *)p;
    orc_csr sub = *q->A;
    sub.n_rows = q->r1 - q->r0;
    sub.off = q->A->off + q->r0; /* offsets stay absolute: cols / vals are shared */
    q->rc = orc_spgemm(&sub, q->B, &q->out, q->fused);
    return NULL;
}

int orc_spgemm_parallel(const orc_csr *A, const orc_csr *B, orc_csr *C, int T, int fused) {
    if (T < 1) T = 1;
    orc_gemm_part *parts = (orc_gemm_part *)calloc((size_t)T, sizeof(orc_gemm_part));
    pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * (size_t)T);
    if (!parts || !th) return ORC_ERR_ALLOC;
    const uint64_t m = A->n_rows;
    for (int t = 0; t < T; ++t) {
        parts[t].A = A;
        parts[t].B = B;
        parts[t].r0 = (uint64_t)t * m / (uint64_t)T;
        parts[t].r1 = (uint64_t)(t + 1) * m / (uint64_t)T;
        parts[t].fused = fused;
    }
    for (int t = 1; t < T; ++t) pthread_create(&th[t], NULL, gemm_worker, &parts[t]);
    gemm_worker(&parts[0]);
    for (int t = 1; t < T; ++t) pthread_join(th[t], NULL);
    uint64_t nnz = 0;
    int rc = ORC_OK;
    for (int t = 0; t < T; ++t) {
        if (parts[t].rc != ORC_OK) rc = parts[t].rc;
        nnz += parts[t].out.nnz;
    }
    uint64_t *off = (uint64_t *)malloc((m + 1) * sizeof(uint64_t));
    uint32_t *cc = (uint32_t *)malloc((nnz ? nnz : 1) * sizeof(uint32_t));
    double *cv = (double *)malloc((nnz ? nnz : 1) * sizeof(double));
    if (!off || !cc || !cv) return ORC_ERR_ALLOC;
    uint64_t base = 0;
    off[0] = 0;
    for (int t = 0; t < T; ++t) {
        const orc_csr *o = &parts[t].out;
        if (rc == ORC_OK) {
            for (uint64_t r = 0; r < o->n_rows; ++r) off[parts[t].r0 + r + 1] = base + o->off[r + 1];
            memcpy(cc + base, o->cols, o->nnz * sizeof(uint32_t));
            memcpy(cv + base, o->vals, o->nnz * sizeof(double));
            base += o->nnz;
        }
        orc_csr_free(&parts[t].out);
    }
    free(parts);
    free(th);
    C->n_rows = m;
    C->n_cols = B->n_cols;
    C->off = off;
    C->cols = cc;
    C->vals = cv;
    C->nnz = nnz;
    C->capacity = nnz;
    return rc;
}

/* Transpose: parallel/algorithms/transpose.hpp:36-70 — output partition t
 * (rows of A^T = columns of A in [c0, c1)) scans every entry of A in row
 * order and keeps those of its columns (O(T nnz) reads, as Spira's); the
 * partitions' rows are then assembled. Within an output row the source rows
 * arrive ascending. */
typedef struct {
    const orc_csr *A;
    uint64_t c0, c1;
    uint64_t *off; /* c1 - c0 + 1, local */
    uint32_t *tc;
    double *tv;
    int rc;
} orc_tr_part;

static void *tr_worker(void *p) {
    orc_tr_part *q = (orc_tr_part *)p;
    const orc_csr *A = q->A;
    const uint64_t w = q->c1 - q->c0;
    q->off = (uint64_t *)calloc(w + 1, sizeof(uint64_t));
    uint64_t *cur = (uint64_t *)malloc((w + 1) * sizeof(uint64_t));
    if (!q->off || !cur) {
        q->rc = ORC_ERR_ALLOC;
        return NULL;
    }
    for (uint64_t k = 0; k < A->nnz; ++k) {
        const uint64_t c = A->cols[k];
        if (c >= q->c0 && c < q->c1) q->off[c - q->c0 + 1]++;
    }
    for (uint64_t j = 0; j < w; ++j) q->off[j + 1] += q->off[j];
    memcpy(cur, q->off, (w + 1) * sizeof(uint64_t));
    const uint64_t n = q->off[w];
    q->tc = (uint32_t *)malloc((n ? n : 1) * sizeof(uint32_t));
    q->tv = (double *)malloc((n ? n : 1) * sizeof(double));
    if (!q->tc || !q->tv) {
        q->rc = ORC_ERR_ALLOC;
        free(cur);
        return NULL;
    }
    for (uint64_t i = 0; i < A->n_rows; ++i)
        for (uint64_t k = A->off[i]; k < A->off[i + 1]; ++k) {
            const uint64_t c = A->cols[k];
            if (c >= q->c0 && c < q->c1) {
                const uint64_t p2 = cur[c - q->c0]++;
                q->tc[p2] = (uint32_t)i;
                q->tv[p2] = A->vals[k];
            }
        }
    free(cur);
    q->rc = ORC_OK;
    return NULL;
}

int orc_transpose_parallel(const orc_csr *A, orc_csr *Tr, int T) {
    if (T < 1) T = 1;
    orc_tr_part *parts = (orc_tr_part *)calloc((size_t)T, sizeof(orc_tr_part));
    pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * (size_t)T);
    if (!parts || !th) return ORC_ERR_ALLOC;
    const uint64_t c = A->n_cols;
    for (int t = 0; t < T; ++t) {
        parts[t].A = A;
        parts[t].c0 = (uint64_t)t * c / (uint64_t)T;
        parts[t].c1 = (uint64_t)(t + 1) * c / (uint64_t)T;
    }
    for (int t = 1; t < T; ++t) pthread_create(&th[t], NULL, tr_worker, &parts[t]);
    tr_worker(&parts[0]);
    for (int t = 1; t < T; ++t) pthread_join(th[t], NULL);
    int rc = ORC_OK;
    for (int t = 0; t < T; ++t)
        if (parts[t].rc != ORC_OK) rc = parts[t].rc;
    uint64_t *off = (uint64_t *)malloc((c + 1) * sizeof(uint64_t));
    uint32_t *tc = (uint32_t *)malloc((A->nnz ? A->nnz : 1) * sizeof(uint32_t));
    double *tv = (double *)malloc((A->nnz ? A->nnz : 1) * sizeof(double));
    if (!off || !tc || !tv) return ORC_ERR_ALLOC;
    uint64_t base = 0;
    off[0] = 0;
    for (int t = 0; t < T; ++t) {
        orc_tr_part *q = &parts[t];
        if (rc == ORC_OK) {
            const uint64_t w = q->c1 - q->c0, n = q->off[w];
            for (uint64_t j = 0; j < w; ++j) off[q->c0 + j + 1] = base + q->off[j + 1];
            memcpy(tc + base, q->tc, n * sizeof(uint32_t));
            memcpy(tv + base, q->tv, n * sizeof(double));
            base += n;
        }
        free(q->off);
        free(q->tc);
        free(q->tv);
    }
    free(parts);
    free(th);
    Tr->n_rows = c;
    Tr->n_cols = A->n_rows;
    Tr->off = off;
    Tr->cols = tc;
    Tr->vals = tv;
    Tr->nnz = A->nnz;
    Tr->capacity = A->nnz;
    return rc;
}
