/*
 * spg.h — C ABI of the GB300 sparse engine (libspg.so).
 *
 * This is the drop-in boundary for Spira's sparse hot path. Spira itself is a
 * header-only C++23 template library with no C ABI; each entry point below
 * names the Spira interface (file:line inside the Spira source tree) whose
 * behaviour it carries. The C++23 facade in include/spira_gb300/ maps these
 * calls back onto Spira's own class and function names and turns status codes
 * into Spira's exception types.
 *
 * Conventions
 *   - Plain C: opaque handles, plain pointers and sizes, int status codes.
 *   - Device-resident CSR, Spira's SoA layout: uint64 offsets[n_rows+1]
 *     (Spira uses std::size_t), uint32 cols[capacity], double vals[capacity]
 *     (csr_storage_soa.hpp:17-77).
 *   - `stream` arguments are cudaStream_t passed as void*; NULL selects the
 *     context's own stream. Calls with a `stream` argument are asynchronous
 *     on that stream; every other call returns after its work is complete.
 *   - Handles are not thread-safe; use one context per host thread.
 *   - No call falls back to the CPU: without a usable GB300 every compute
 *     call fails with SPG_ERR_CUDA.
 */
#ifndef SPG_H
#define SPG_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes; the facade maps them to Spira's exceptions ---------- */
enum spg_status {
    SPG_OK = 0,
    SPG_ERR_INVALID_ARGUMENT = 1, /* std::invalid_argument: shape/size mismatch, malformed CSR */
    SPG_ERR_LOGIC = 2,            /* std::logic_error: wrong mode (e.g. spmv before lock) */
    SPG_ERR_OUT_OF_RANGE = 3,     /* std::out_of_range: row/col index beyond the shape */
    SPG_ERR_NO_MEMORY = 4,        /* std::bad_alloc: device allocation failed */
    SPG_ERR_CUDA = 5,             /* CUDA runtime error (no device, launch failure, ...) */
    SPG_ERR_DEVICE_TIMEOUT = 6,   /* a bounded device-side wait gave up; context stays usable */
    SPG_ERR_UNSUPPORTED = 7,      /* valid request that libspg does not serve */
    SPG_ERR_DOMAIN = 8            /* std::domain_error: division by a zero scalar */
};

/* ---- SpMV variants (spg_spmv `variant`) --------------------------------- */
enum spg_spmv_variant {
    SPG_SPMV_AUTO = -1,     /* learned selector, exhaustive-autotune fallback */
    SPG_SPMV_SCALAR = 0,    /* one thread per row, CSR order (the plain path) */
    SPG_SPMV_VECTOR2 = 1,   /* 2 lanes per row, shuffle reduction */
    SPG_SPMV_VECTOR4 = 2,
    SPG_SPMV_VECTOR8 = 3,
    SPG_SPMV_VECTOR16 = 4,
    SPG_SPMV_VECTOR32 = 5,  /* one warp per row, 16-byte vector loads */
    SPG_SPMV_STREAM = 6,    /* CTA row blocks: coalesced nnz staging in shared memory */
    SPG_SPMV_MERGE = 7,     /* merge-path: equal (rows + nnz) per CTA, carry fix-up */
    SPG_SPMV_ADAPTIVE = 8,  /* warp per 1024 nonzeros, 32 consecutive per lane in one
                               FMA chain, rows closed at a row-start bitmap, segmented
                               combine across lanes and chunks */
    SPG_SPMV_ADAPTIVE16 = 9, /* the same with 16 nonzeros per lane */
    SPG_SPMV_INTERLEAVED = 10, /* ADAPTIVE16's arithmetic over a copy of cols/vals stored
                                  lane-interleaved per 512-nonzero chunk, so every load is
                                  one contiguous warp access; the copy costs 12 B per
                                  nonzero of device memory while cached; 2-entry
                                  sub-batches, 8 blocks of 256 threads per SM */
    /* Tiles of the chunk kernels: the same variant's arithmetic and bits with
     * another sub-batch depth (nonzeros whose loads and gathers a lane issues
     * before their FMAs) and residency (blocks of 256 threads per SM). */
    SPG_SPMV_INTERLEAVED_S4 = 11, /* INTERLEAVED, 4-entry sub-batches, 5 blocks per SM */
    SPG_SPMV_INTERLEAVED_S8 = 12, /* INTERLEAVED, 8-entry sub-batches, 4 blocks per SM */
    SPG_SPMV_ADAPTIVE16_S4 = 13,  /* ADAPTIVE16, 4-entry sub-batches, 6 blocks per SM
                                     (ADAPTIVE16 itself: 8-entry, 4 blocks) */
    SPG_SPMV_ADAPTIVE_S16 = 14,   /* ADAPTIVE, 16-entry sub-batches, 2 blocks per SM
                                     (ADAPTIVE itself: 8-entry, 4 blocks) */
    SPG_SPMV_N_VARIANTS = 15
};

typedef struct spg_ctx spg_ctx; /* one device + one stream + memory pool */
typedef struct spg_csr spg_csr; /* a device-resident CSR matrix */

typedef struct spg_csr_info {
    uint64_t n_rows;
    uint64_t n_cols;
    uint64_t nnz;
    uint64_t capacity; /* Spira's csr_storage::capacity (>= nnz) */
    int built;         /* 0 until the first lock / load */
} spg_csr_info;

/* ---- errors / library --------------------------------------------------- */
const char *spg_strerror(int status);
/* Detail message of the last failing call on this host thread. */
const char *spg_last_error(void);
/* ABI version, major*10000 + minor*100 + patch. */
int spg_version(void);

/* ---- context ------------------------------------------------------------ */
int spg_ctx_create(int device, spg_ctx **out);
int spg_ctx_destroy(spg_ctx *ctx);
/* The context's own stream (cudaStream_t as void*). */
int spg_ctx_stream(spg_ctx *ctx, void **stream);
/* Waits for the context stream; SPG_ERR_DEVICE_TIMEOUT if a kernel's bounded
 * wait gave up since the last check (the context stays usable). */
int spg_ctx_sync(spg_ctx *ctx);
/* Device time of operations that synchronise internally (lock, transpose,
 * SpGEMM, addition, scaling: their output sizes are data-dependent). Between
 * spg_ctx_timer_start and spg_ctx_timer_stop, every stretch of work on the
 * context stream up to one of those synchronisations is timed with CUDA
 * events and added up; the host round trips at the synchronisations are not
 * counted. No Spira counterpart (a measurement aid). */
int spg_ctx_timer_start(spg_ctx *ctx);
int spg_ctx_timer_stop(spg_ctx *ctx, double *device_ms);
/* Self-test of the device-side waits (SpGEMM's ordered scan of tile counts):
 * runs one wait whose predecessor never publishes, bounded by wait_cycles SM
 * clocks (1 .. 2^31). The kernel gives up, sets the context's status word
 * and returns, so the next spg_ctx_sync reports SPG_ERR_DEVICE_TIMEOUT and
 * the context stays usable; *gave_up = 1 when the wait gave up as designed.
 * No Spira counterpart. */
int spg_selftest_wait_timeout(spg_ctx *ctx, long long wait_cycles, int *gave_up);
/* Bytes of the context's device memory pool (the device's default
 * stream-ordered pool, from which every device buffer of libspg comes) that
 * live buffers hold, and that the pool holds from the driver (freed buffers
 * stay cached in it). Either pointer may be NULL. No Spira counterpart
 * (Spira's memory is host memory). */
int spg_ctx_pool_used(spg_ctx *ctx, uint64_t *used_bytes, uint64_t *reserved_bytes);

/* ---- CSR handles ---------------------------------------------------------
 * spg_csr_create: an unbuilt n_rows x n_cols matrix (matrix.hpp:197-209). */
int spg_csr_create(spg_ctx *ctx, uint64_t n_rows, uint64_t n_cols, spg_csr **out);
int spg_csr_destroy(spg_csr *A);
int spg_csr_info_get(const spg_csr *A, spg_csr_info *info);
/* Device pointers of the CSR arrays (valid until the next lock of A). */
int spg_csr_device_arrays(const spg_csr *A, const uint64_t **offsets,
                          const uint32_t **cols, const double **vals);
/* Copy the CSR to host arrays sized n_rows+1 / nnz / nnz; NULL skips an array
 * (matrix.hpp:88-91 csr()). */
int spg_csr_download(spg_ctx *ctx, const spg_csr *A, uint64_t *offsets,
                     uint32_t *cols, double *vals);
/* Validate and install a host CSR (matrix.hpp:520-605 load_csr): offsets[0]
 * == 0, offsets[n_rows] == nnz, non-decreasing, in-range and strictly
 * ascending columns per row; SPG_ERR_INVALID_ARGUMENT otherwise. */
int spg_csr_load(spg_ctx *ctx, spg_csr *A, const uint64_t *offsets,
                 const uint32_t *cols, const double *vals, uint64_t nnz);
/* Deep copy into dst (reshaped to src's shape); tight, capacity == nnz
 * (csr_storage_soa.hpp:44-56). */
int spg_csr_copy(spg_ctx *ctx, const spg_csr *src, spg_csr *dst);
/* Locked-mode point lookup (row.hpp:192-206 via csr_slice::binary_search,
 * csr_storage_soa.hpp:94-104). */
int spg_csr_get(spg_ctx *ctx, const spg_csr *A, uint64_t row, uint32_t col,
                double *value, int *found);
/* [begin, end) of one row in the CSR arrays (matrix.hpp row_nnz). */
int spg_csr_row_range(spg_ctx *ctx, const spg_csr *A, uint64_t row,
                      uint64_t *begin, uint64_t *end);

/* ---- lock(): merge one epoch of staged inserts ---------------------------
 * rows/cols/vals are the epoch's inserts in insertion order. Per (row, col)
 * the last insert wins; a last value of +-0.0 deletes the entry; NaN is kept.
 * First lock builds the CSR, later locks merge into it (matrix.hpp:277-342,
 * aos_array_buffer.hpp:76-101, csr_build.hpp:32-98 and 126-488). Indices are
 * range-checked on the device: SPG_ERR_OUT_OF_RANGE leaves A unchanged. */
int spg_lock(spg_ctx *ctx, spg_csr *A, const uint32_t *rows,
             const uint32_t *cols, const double *vals, uint64_t n_staged);
/* Same with device-resident staging arrays. */
int spg_lock_device(spg_ctx *ctx, spg_csr *A, const uint32_t *d_rows,
                    const uint32_t *d_cols, const double *d_vals,
                    uint64_t n_staged);

/* ---- SpMV y = A x ----------------------------------------------------------
 * spg_spmv: device x[n_cols], y[n_rows]; asynchronous on `stream`
 * (serial/spmv.hpp:141-186, parallel/algorithms/spmv.hpp:125-161,
 * kernel::sparse_dot_double kernels.h:5). SPG_ERR_LOGIC before the first lock. */
int spg_spmv(spg_ctx *ctx, const spg_csr *A, const double *d_x, double *d_y,
             int variant, void *stream);
/* Host vectors with their lengths, as spmv(mat, x, y) takes std::vector:
 * copies x in, runs, copies y out. x_len != n_cols or y_len != n_rows gives
 * SPG_ERR_INVALID_ARGUMENT (serial/spmv.hpp:150-155). */
int spg_spmv_host(spg_ctx *ctx, const spg_csr *A, const double *x,
                  uint64_t x_len, double *y, uint64_t y_len, int variant);
/* The same from pinned host x and y (SPG_ERR_INVALID_ARGUMENT otherwise),
 * enqueued on `stream` and returning at once: the copies and kernels of
 * different matrices can then overlap (one matrix's upload with another's
 * SpMV or download). y is complete once `stream` is; spg_ctx_sync reports a
 * device-side timeout. Calls on the same matrix must be ordered (one stream):
 * each matrix stages x and y in its own device buffers. */
int spg_spmv_host_async(spg_ctx *ctx, const spg_csr *A, const double *x, uint64_t x_len, double *y,
                        uint64_t y_len, int variant, void *stream);
/* n (<= 4) distinct matrices' SpMVs from pinned host buffers xs[i] (n_cols
 * of mats[i]) into ys[i] (n_rows), as one recorded graph enqueued on `stream`
 * (returns at once; y complete once the stream is). variants may be NULL
 * (SPG_SPMV_AUTO for all). The uploads are ordered — matrices whose SpMV
 * reads x anywhere first, largest x first — so that matrix's x does not share
 * the host link with the others while the rest upload, compute and download
 * during its SpMV. No Spira counterpart (one spmv call per matrix there). */
int spg_spmv_host_multi(spg_ctx *ctx, uint32_t n, const spg_csr *const *mats, const double *const *xs,
                        double *const *ys, const int *variants, void *stream);
/* SpMV that allocates no device memory at all. No counterpart in Spira.
 * For callers that cannot call cudaMalloc (or let this library call it):
 * code whose device memory is all owned by another allocator or a fixed
 * arena sized at start-up, and latency-critical loops where an allocation
 * could stall other work on the device. It runs the MERGE variant with its
 * scratch (tile starts and carry-outs) in a fixed array of about 2 MiB
 * compiled into libspg.so, which every device that loads the library keeps
 * until the process exits. Limit: rows + nonzeros <= spg_spmv_noalloc_max()
 * (117 440 512); larger matrices get SPG_ERR_INVALID_ARGUMENT. Every
 * spg_ctx_create looks up the array's device address for its device (this
 * may also load the library's GPU code; a context created after
 * cudaDeviceReset gets the new address), and a call finding none looks it up
 * itself: create the context, or make that first call, before any stream
 * capture.
 * Every call shares the one array: calls that overlap on the GPU (different
 * streams, or several host threads) race, and the caller must serialize
 * them. Each call rewrites all the scratch it reads. Device x, y; asynchronous
 * on `stream`. */
int spg_spmv_noalloc(spg_ctx *ctx, const spg_csr *A, const double *d_x, double *d_y, void *stream);
uint64_t spg_spmv_noalloc_max(void);

/* The variant SPG_SPMV_AUTO resolves to for A. */
int spg_spmv_selected(spg_ctx *ctx, const spg_csr *A, int *variant);
/* Number of kernel launches one spg_spmv of A with `variant` issues (plans
 * are built beforehand and not counted). */
int spg_spmv_launches(spg_ctx *ctx, const spg_csr *A, int variant, int *n_launches);

/* ---- SpMV variant choice ----------------------------------------------------
 * No Spira counterpart: Spira has a single SpMV code path per type
 * combination (serial/spmv.hpp:141-186). These choose which of this engine's
 * kernels computes it; the arithmetic is the same whichever is chosen.
 * SPG_SPMV_AUTO follows the context's policy (per matrix, cached until the
 * next lock): SPG_POLICY_SELECTOR uses the learned selector when one is
 * loaded and the exhaustive autotuner otherwise; SPG_POLICY_AUTOTUNE always
 * autotunes; SPG_POLICY_FIXED takes SPG_SPMV_ADAPTIVE16 without measuring. */
#define SPG_SELECT_FEATURES 40 /* 32-bin log2 row-length histogram + 8 shape stats */
#define SPG_SELECT_HIDDEN 64   /* MLP 40 -> 64 -> 64 -> K, FP32, ReLU */
enum spg_spmv_policy { SPG_POLICY_SELECTOR = 0, SPG_POLICY_AUTOTUNE = 1, SPG_POLICY_FIXED = 2 };

int spg_set_spmv_policy(spg_ctx *ctx, int policy);
/* The 40 selector features of A (host array). */
int spg_spmv_features(spg_ctx *ctx, const spg_csr *A, float *features);
/* Times every variant (median of `reps` warm runs, CUDA events): times_ms
 * [SPG_SPMV_N_VARIANTS] (may be NULL) and the fastest in *best (may be NULL). */
int spg_spmv_autotune(spg_ctx *ctx, const spg_csr *A, int reps, float *times_ms, int *best);
/* Device probe, no Spira counterpart: the rate (gathers per second, median of
 * 5 timed runs after 2 warm-up runs) of random 8-byte reads from an n_x-entry
 * double vector (n_x a power of two; 2^22 = 32 MB stays in L2), n_gathers
 * reads per run, 16 per thread at hashed positions. It is the ceiling of SpMV
 * on matrices with randomly spread columns, where every nonzero's x read hits
 * its own L2 sector. */
int spg_probe_gather_rate(spg_ctx *ctx, uint64_t n_x, uint64_t n_gathers, double *gathers_per_s);
/* The same random reads with their shape as parameters, to show whether the
 * rate above is the device's ceiling: blocks_per_sm x SMs blocks of 256
 * threads (fewer may be resident; *resident_blocks_per_sm, may be NULL, says
 * how many) walk n_gathers / per_thread items of per_thread independent reads
 * (1, 2, 4, ..., 64 in flight per thread). No Spira counterpart. */
int spg_probe_gather_rate_cfg(spg_ctx *ctx, uint64_t n_x, uint64_t n_gathers, int per_thread, int blocks_per_sm,
                              double *gathers_per_s, int *resident_blocks_per_sm);
/* Device probe, no Spira counterpart: the FP64 fused multiply-add rate (FMAs
 * per second, median of 5 timed runs after 2 warm-up runs) of a launch of 8
 * CTAs of 256 threads per SM, each thread running 8 independent FMA chains of
 * `iters` steps. It is the ceiling of the batched multi-RHS SpMV, where every
 * (nonzero, right-hand side) pair is one FP64 FMA and the FP64 pipe, not
 * memory, is the bound. */
int spg_probe_fp64_rate(spg_ctx *ctx, uint32_t iters, double *fma_per_s);
/* Installs a trained selector (NULL blob removes it). Blob layout, FP32:
 * mean[40] scale[40] W1[64][40] b1[64] W2[64][64] b2[64] W3[K][64] b3[K];
 * output k predicts log(time of variant k / fastest time). */
int spg_selector_load(spg_ctx *ctx, const float *blob, uint64_t n_floats, int n_outputs);
/* Number of MLP parameters (W1..b3) for K outputs. */
uint64_t spg_mlp_param_count(int n_outputs);
/* Batched inference of the loaded selector on device features [B][40]. */
int spg_selector_predict(spg_ctx *ctx, const float *d_features, uint32_t B, float *d_out, void *stream);
/* Training kernels on device buffers (FP32). d_act holds [B][2*64]
 * activations from forward for backward; d_grad has the parameter layout. */
int spg_mlp_forward(spg_ctx *ctx, const float *d_params, int n_outputs, const float *d_x, uint32_t B,
                    float *d_act, float *d_out, void *stream);
int spg_mlp_backward(spg_ctx *ctx, const float *d_params, int n_outputs, const float *d_x, uint32_t B,
                     const float *d_act, const float *d_dout, float *d_grad, void *stream);
/* Mean squared error over n outputs: d_dpred = 2 (pred - target) / n; the
 * loss is added to *d_loss when d_loss is not NULL. */
int spg_mlp_mse(spg_ctx *ctx, const float *d_pred, const float *d_target, uint64_t n, float *d_dpred,
                float *d_loss, void *stream);
int spg_mlp_adam(spg_ctx *ctx, float *d_params, const float *d_grad, float *d_m, float *d_v, uint64_t n,
                 float lr, float beta1, float beta2, float eps, uint32_t step, void *stream);
int spg_mlp_argmin(spg_ctx *ctx, const float *d_pred, uint32_t B, int n_outputs, int *d_best, void *stream);

/* ---- batched multi-RHS SpMV ------------------------------------------------
 * No Spira counterpart as a call: each item is Spira's SpMV
 * (serial/spmv.hpp:141-186) applied to the k columns of a row-major X
 * (n_cols x k, X[c * k + j]) into Y (n_rows x k). spg_batch_create builds the
 * work list of (matrix, row tile) items and captures one persistent launch in
 * a CUDA graph; config < 0 autotunes the tile size and CTAs per SM on the
 * batch (runs it a few times), config 0..7 picks one directly. For k < 32 it
 * also records a row order (rows by length inside windows of 256) so the
 * rows sharing a warp are of near-equal length; each Y row is still the same
 * FMA chain over its row. k must be a power of two <= 32. Matrices and
 * vectors must outlive the batch and keep their device arrays (no lock in
 * between). */
typedef struct spg_batch spg_batch;
int spg_batch_create(spg_ctx *ctx, uint32_t n, const spg_csr *const *mats, const double *const *d_X,
                     double *const *d_Y, const uint32_t *k, int config, spg_batch **out);
int spg_batch_config(const spg_batch *batch, int *config, uint32_t *n_items);
/* Replays the graph (one persistent kernel) on `stream`. */
int spg_batch_run(spg_ctx *ctx, spg_batch *batch, void *stream);
/* The comparison path: one plain SpMV launch per matrix per right-hand side. */
int spg_batch_run_plain(spg_ctx *ctx, spg_batch *batch, void *stream);
int spg_batch_destroy(spg_batch *batch);

/* ---- element-wise operations and queries -----------------------------------
 * spg_csr_add: C <- A + B. Per row a merge of the two CSR slices: equal
 * columns give a + b (one IEEE add) and are kept unless the sum is +-0, other
 * entries are copied, stored zeros are dropped; C is reshaped to A's shape
 * with tight capacity (serial/matrix_addition.hpp:34-110,
 * parallel/algorithms/matrix_addition.hpp:24-99). A and B of different shapes
 * give SPG_ERR_INVALID_ARGUMENT, an unlocked A or B SPG_ERR_LOGIC; C must not
 * be A or B. */
int spg_csr_add(spg_ctx *ctx, const spg_csr *A, const spg_csr *B, spg_csr *C);
/* spg_csr_scale: C <- A * scalar (divide == 0) or A / scalar (divide != 0),
 * every committed value once (IEEE multiply / divide), results that are +-0
 * dropped (serial/scalars.hpp:10-67). C may be A (in place; Spira's in-place
 * form stages the scaled values and the next lock installs them, which ends
 * in the same CSR). Division by +-0 gives SPG_ERR_DOMAIN, checked first; an
 * unlocked A gives SPG_ERR_LOGIC. */
int spg_csr_scale(spg_ctx *ctx, spg_csr *A, spg_csr *C, double scalar, int divide);
/* spg_csr_row_sums: d_out[r] = sum of row r's values in CSR order from 0.0,
 * one IEEE add per entry (matrix.hpp:438-443, row.hpp:208-216,
 * csr_storage_soa.hpp:114-120: a locked row's accumulate()). Asynchronous on
 * `stream`. */
int spg_csr_row_sums(spg_ctx *ctx, const spg_csr *A, double *d_out, void *stream);
/* The same for rows [row0, row0 + n) into host out[n]; returns when done.
 * Rows beyond n_rows give SPG_ERR_OUT_OF_RANGE. */
int spg_csr_row_sums_host(spg_ctx *ctx, const spg_csr *A, uint64_t row0, uint64_t n, double *out);
/* spg_csr_lookup: n point queries (d_rows[i], d_cols[i]) against the
 * committed CSR, binary search per query (row.hpp:190-204, locked rows):
 * d_vals[i] = the stored value or 0.0, d_found[i] = 1 or 0 (either output may
 * be NULL). Queries outside the shape report not found. Asynchronous on
 * `stream`. */
int spg_csr_lookup(spg_ctx *ctx, const spg_csr *A, uint64_t n, const uint64_t *d_rows, const uint32_t *d_cols,
                   double *d_vals, uint8_t *d_found, void *stream);
/* spg_csr_partition: nnz-balanced row boundaries for n_parts partitions into
 * host bounds[n_parts + 1]: bounds[t] = first row whose nnz prefix reaches
 * max(1, t * nnz / n_parts), a uniform row split when nnz == 0, {0, n, ...}
 * for one part or no rows (parallel/partition.hpp:78-126, the boundaries
 * parallel_matrix::rebalance installs, parallel_matrix.hpp:434-452). */
int spg_csr_partition(spg_ctx *ctx, const spg_csr *A, uint64_t n_parts, uint64_t *bounds);

/* ---- binary CSR files (no Spira counterpart) --------------------------------
 * Little-endian; each section starts on an 8-byte boundary:
 *   64-byte header: magic "SPGCSR\0\0", u64 version (1), n_rows, n_cols, nnz,
 *                   flags (bit 0: values may hold explicit +-0), checksum, 0
 *   u64 offsets[n_rows + 1]; u32 cols[nnz] zero-padded to 8 bytes; f64 vals[nnz]
 * checksum = sum over the payload's 64-bit words w_i (i from 0 at the first
 * offsets word) of splitmix64_finaliser(w_i ^ (i * 0x9E3779B97F4A7C15)),
 * modulo 2^64 (computed on the device).
 * spg_csr_save writes a locked A (SPG_ERR_LOGIC otherwise). spg_csr_load_file
 * reshapes A to the file's shape after checking the header against the file
 * size, the checksum and load_csr's CSR rules (matrix.hpp:524-575); any
 * failure gives SPG_ERR_INVALID_ARGUMENT and leaves A unchanged.
 * spg_csr_file_info reads and checks only the header (no device needed). */
int spg_csr_save(spg_ctx *ctx, const spg_csr *A, const char *path);
int spg_csr_load_file(spg_ctx *ctx, spg_csr *A, const char *path);
int spg_csr_file_info(const char *path, uint64_t *n_rows, uint64_t *n_cols, uint64_t *nnz);

/* ---- transpose / SpGEMM ----------------------------------------------------
 * spg_transpose: AT <- A^T (AT is reshaped to n_cols x n_rows, capacity ==
 * nnz); each output row lists its source rows in ascending order
 * (serial/transpose.hpp:35-156, parallel/algorithms/transpose.hpp:36-70).
 * SPG_ERR_LOGIC before A's first lock. */
int spg_transpose(spg_ctx *ctx, const spg_csr *A, spg_csr *AT);
/* spg_spgemm: C <- A * B (C reshaped to A.n_rows x B.n_cols). Each C(i, j)
 * is the left-to-right sum over ascending k of the rounded products
 * a_ik * b_kj from 0.0; exact-zero sums are dropped (serial/spgemm.hpp:12-53,
 * parallel/algorithms/spgemm.hpp:27-69). A.n_cols != B.n_rows gives
 * SPG_ERR_INVALID_ARGUMENT, an unlocked A or B SPG_ERR_LOGIC. The kernel
 * path is SPG_SPGEMM_AUTO's choice (below); every path computes the same C. */
int spg_spgemm(spg_ctx *ctx, const spg_csr *A, const spg_csr *B, spg_csr *C);

/* ---- SpGEMM variants and their choice ----------------------------------------
 * No Spira counterpart: Spira has one SpGEMM code path (serial/spgemm.hpp:
 * 28-48). These choose which of this engine's kernels computes it; C is the
 * same bits whichever runs. */
enum spg_spgemm_variant {
    SPG_SPGEMM_AUTO = -1,        /* the context's policy, as for SpMV */
    SPG_SPGEMM_ROWMERGE = 0,     /* a thread per row merges the row's B rows (k-way, by
                                    column); rows with > 32 A entries or > 4096 products
                                    go through expand-sort-compress; a compaction pass */
    SPG_SPGEMM_ESC = 1,          /* expand every product, one global radix sort by
                                    (row, column), left-to-right run sums */
    SPG_SPGEMM_WARPSORT_64 = 2,  /* tiles of consecutive rows: a warp sorts each row's
                                    (column, product) pairs in registers (bitonic, rows of
                                    <= 64 products; heavier rows expand-sort-compress) and
                                    sums each run of equal columns in the run's first lane,
                                    each tile writes C in place after an ordered scan of the
                                    tiles' counts; tiles of <= 1024 products */
    SPG_SPGEMM_WARPSORT_128 = 3, /* the same for rows of <= 128 products, 2048-product tiles */
    SPG_SPGEMM_WARPSORT_256 = 4, /* the same for rows of <= 256 products, 4096-product tiles */
    SPG_SPGEMM_N_VARIANTS = 5
};
/* C <- A * B with a given variant (SPG_SPGEMM_AUTO: as spg_spgemm). */
int spg_spgemm_variant(spg_ctx *ctx, const spg_csr *A, const spg_csr *B, spg_csr *C, int variant);
/* The variant SPG_SPGEMM_AUTO resolves to for A * B. */
int spg_spgemm_selected(spg_ctx *ctx, const spg_csr *A, const spg_csr *B, int *variant);
/* The 40 SpGEMM selector features of A * B (host array): 32-bin log2
 * histogram of the products per row of A, then log sizes (rows, B's
 * columns, nnz of A, products), mean / spread / maximum products per row and
 * the column spread of A (mean |col / n_cols - row / n_rows| over the first
 * and last entry of sampled rows: small for banded, block and stencil
 * patterns, whose products collapse onto few columns). */
int spg_spgemm_features(spg_ctx *ctx, const spg_csr *A, const spg_csr *B, float *features);
/* Times every SpGEMM variant on A * B (median of `reps` runs after one
 * warm-up, wall clock around the complete call: the calls synchronise):
 * times_ms[SPG_SPGEMM_N_VARIANTS] (may be NULL) and the fastest in *best (may
 * be NULL). */
int spg_spgemm_autotune(spg_ctx *ctx, const spg_csr *A, const spg_csr *B, int reps, float *times_ms, int *best);
/* Installs a trained SpGEMM selector (same blob layout as spg_selector_load;
 * output k predicts log(time of SpGEMM variant k / fastest time)); NULL
 * removes it. The context loads spg_spgemm_selector.bin from beside the
 * library (or $SPG_SPGEMM_SELECTOR_MODEL) when it is created. */
int spg_spgemm_selector_load(spg_ctx *ctx, const float *blob, uint64_t n_floats, int n_outputs);
/* Batched inference of the loaded SpGEMM selector on device features [B][40]. */
int spg_spgemm_selector_predict(spg_ctx *ctx, const float *d_features, uint32_t B, float *d_out, void *stream);
/* SPG_SPGEMM_AUTO's policy: SPG_POLICY_SELECTOR (the selector if loaded, else
 * the autotuner), SPG_POLICY_AUTOTUNE, SPG_POLICY_FIXED (SPG_SPGEMM_WARPSORT_128
 * without measuring). The selector never picks a WARPSORT variant that a
 * smaller one does the same work for: when every row of A * B has at most 64
 * products and A entries, _128 and _256 are skipped; up to 128, _256. The
 * choice is cached per (A, B) until either changes. */
int spg_set_spgemm_policy(spg_ctx *ctx, int policy);

#ifdef __cplusplus
}
#endif
#endif /* SPG_H */
