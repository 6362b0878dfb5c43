// spg_internal.cuh — shared internals of libspg.so: handles, error plumbing,
// device buffers and the device-wide primitives (scan, radix sort) that the
// lock / transpose / SpGEMM kernels are built from.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cstdarg>
#include <cstdio>
#include <string>
#include <utility>
#include <atomic>
#include <vector>

#include "../../include/spg.h"

namespace spg {

// ---------------------------------------------------------------------------
// Errors. Every C entry point returns a status; the detail text goes to a
// thread-local string read back by spg_last_error().
// ---------------------------------------------------------------------------
int set_error(int code, const char *fmt, ...);
void clear_error();

struct Status {
    int code = SPG_OK;
    bool ok() const { return code == SPG_OK; }
};

#define SPG_CUDA_TRY(expr)                                                          \
    do {                                                                            \
        cudaError_t _e = (expr);                                                    \
        if (_e != cudaSuccess) {                                                    \
            if (_e == cudaErrorMemoryAllocation) {                                  \
                cudaGetLastError();                                                 \
                return ::spg::set_error(SPG_ERR_NO_MEMORY, "%s: %s (%s:%d)", #expr, \
                                        cudaGetErrorString(_e), __FILE__, __LINE__); \
            }                                                                       \
            return ::spg::set_error(SPG_ERR_CUDA, "%s: %s (%s:%d)", #expr,          \
                                    cudaGetErrorString(_e), __FILE__, __LINE__);    \
        }                                                                           \
    } while (0)

#define SPG_TRY(expr)                      \
    do {                                   \
        int _s = (expr);                   \
        if (_s != SPG_OK) return _s;       \
    } while (0)

#define SPG_LAUNCH_CHECK() SPG_CUDA_TRY(cudaPeekAtLastError())

// ---------------------------------------------------------------------------
// Handles
// ---------------------------------------------------------------------------
struct Ctx;

// Stream-ordered device buffer from the context's memory pool.
struct DevBuf {
    void *ptr = nullptr;
    size_t bytes = 0;
    cudaStream_t stream = nullptr;
    DevBuf() = default;
    DevBuf(const DevBuf &) = delete;
    DevBuf &operator=(const DevBuf &) = delete;
    DevBuf(DevBuf &&o) noexcept { *this = std::move(o); }
    DevBuf &operator=(DevBuf &&o) noexcept {
        if (this != &o) {
            release();
            ptr = o.ptr; bytes = o.bytes; stream = o.stream;
            o.ptr = nullptr; o.bytes = 0;
        }
        return *this;
    }
    ~DevBuf() { release(); }
    int alloc(size_t n, cudaStream_t s);
    void release();
    template <class T> T *as() const { return static_cast<T *>(ptr); }
};

// Cached SpMV plan (row blocks for the stream / merge variants).
struct SpmvPlan {
    int kind = -1;           // variant the plan belongs to
    uint64_t n_items = 0;    // number of work items (blocks / tiles / chunks)
    uint64_t count1 = 0;     // variant-specific count
    DevBuf items;            // variant-specific item descriptors
    DevBuf aux;              // variant-specific scratch (carry-outs)
    DevBuf extra0, extra1, extra2;
    DevBuf extra3, extra4;
    // Host-side block split for the pipelined host SpMV (adaptive variants):
    // host_rows[b] = first row of block b, host_rows[host_nb] = n_rows.
    int host_nb = 0;
    std::vector<uint64_t> host_rows;
};

struct Csr;
struct Batch;
void batch_orphan(Batch *b);  // spg_batch.cu

struct Ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    cudaMemPool_t pool = nullptr;
    // Live handles created on this context. Destroying the context releases
    // their device memory and orphans them; an orphaned handle can still be
    // destroyed, every other call on it returns SPG_ERR_LOGIC.
    std::vector<Csr *> live_csrs;
    std::vector<Batch *> live_batches;
    int n_sms = 0;
    size_t l2_bytes = 0;
    // Status word written by kernels whose bounded waits ran out; 0 = ok.
    // Mapped pinned memory: h_status is the host view, d_status the device one.
    unsigned int *h_status = nullptr;
    unsigned int *d_status = nullptr;
    // Returns SPG_ERR_DEVICE_TIMEOUT (and clears the word) if a kernel flagged
    // one since the last check; call after a stream synchronisation.
    int take_status() {
        const unsigned v = h_status ? *(volatile unsigned *)h_status : 0u;
        if (!v) return SPG_OK;
        *(volatile unsigned *)h_status = 0;
        return set_error(SPG_ERR_DEVICE_TIMEOUT, "a device-side wait gave up (status 0x%x)", v);
    }
    // Pinned host staging for the *_host entry points.
    void *pinned = nullptr;
    size_t pinned_bytes = 0;
    int ensure_pinned(size_t bytes);
    // Device vectors reused by spg_spmv_host, the stream that copies y back
    // while later row blocks compute, and the events between the two.
    DevBuf xbuf, ybuf;
    cudaStream_t copy_stream = nullptr, upload_stream = nullptr;
    static constexpr int N_HOST_EVENTS = 8;
    cudaEvent_t host_events[N_HOST_EVENTS] = {};
    cudaEvent_t upload_events[N_HOST_EVENTS] = {};
    // Host SpMVs of several matrices in one call (spg_host_multi.cu): per
    // matrix lane a compute, an upload and a download stream and events,
    // created at first use; the recorded graph and what it was recorded for.
    static constexpr int MULTI_MAX = 4;
    cudaStream_t multi_stream[MULTI_MAX][3] = {};
    cudaEvent_t multi_event[MULTI_MAX][2 * N_HOST_EVENTS] = {};
    cudaGraphExec_t multi_graph = nullptr;
    std::vector<uintptr_t> multi_key;
    void drop_multi() {
        if (multi_graph) cudaGraphExecDestroy(multi_graph);
        multi_graph = nullptr;
        multi_key.clear();
    }
    // SpMV variant choice: policy and the loaded selector (spg_tune.cu).
    int spmv_policy = SPG_POLICY_SELECTOR;
    DevBuf model;  // FP32 selector blob
    int model_k = 0;
    // The same for SpGEMM.
    int spgemm_policy = SPG_POLICY_SELECTOR;
    DevBuf gemm_model;
    int gemm_model_k = 0;
    // Device-time accounting of operations that synchronise internally
    // (spg_ctx_timer_start / _stop): each stretch of work on the context
    // stream between two host synchronisations is one phase, timed by an
    // event pair; the host round trips between phases are not counted.
    bool timer_on = false;
    double timer_ms = 0.0;
    cudaEvent_t timer_ev[2] = {nullptr, nullptr};
    // Waits for `s` (the operations' synchronisation point); closes and opens
    // a timed phase when the timer runs on this stream.
    int phase_sync(cudaStream_t s);
};

struct Csr {
    Ctx *ctx = nullptr;
    uint64_t n_rows = 0, n_cols = 0;
    uint64_t nnz = 0, capacity = 0;
    bool built = false;
    // True when load_csr installed explicit +-0.0 values (only load_csr can:
    // lock and SpGEMM never store zeros). The merge then drops them from the
    // rows it touches, as csr_build.hpp:274-301 does.
    bool may_have_zeros = false;
    DevBuf off;   // uint64_t[n_rows + 1]
    DevBuf cols;  // uint32_t[capacity]
    DevBuf vals;  // double[capacity]
    // The longest row, computed lazily by csr_max_row.
    bool stats_valid = false;
    uint64_t max_row = 0;
    int selected_spmv = -1;
    // SpGEMM variant chosen for this matrix times gemm_sel_b (at its epoch).
    int gemm_selected = -1;
    const Csr *gemm_sel_b = nullptr;
    uint64_t gemm_sel_b_epoch = 0;
    SpmvPlan plan_stream, plan_merge, plan_adaptive, plan_inter;
    // For the host-buffer SpMV of row-parallel variants: the largest column
    // each of host_reach.size() equal row blocks reads (-1: empty block), so a
    // block can start once the part of x up to that column has arrived.
    std::vector<int64_t> host_reach;
    // The pipelined host SpMV recorded as a CUDA graph for one pinned (x, y)
    // pair and variant, replayed while the same pair comes back.
    cudaGraphExec_t host_graph = nullptr;
    const double *host_gx = nullptr;  // the pair, the variant and the device staging it was recorded with
    double *host_gy = nullptr;
    const void *host_gdx = nullptr, *host_gdy = nullptr;
    int host_gvariant = -1;
    // Device staging of x and y for host-buffer SpMVs from pinned memory (the
    // matrix's own, so SpMVs of different matrices can be in flight at once).
    DevBuf stage_x, stage_y;
    void drop_host_graph() {
        if (host_graph) cudaGraphExecDestroy(host_graph);
        host_graph = nullptr;
        host_gx = nullptr;
        host_gy = nullptr;
        host_gdx = host_gdy = nullptr;
        host_gvariant = -1;
    }
    ~Csr() { drop_host_graph(); }
    // Renewed whenever the CSR changes, unique across all matrices of the
    // process (keys graphs recorded over the matrix).
    uint64_t epoch = 0;
    static uint64_t next_epoch() {
        static std::atomic<uint64_t> counter{0};
        return ++counter;
    }
    void invalidate_derived() {
        epoch = next_epoch();
        stats_valid = false;
        selected_spmv = -1;
        gemm_selected = -1;
        gemm_sel_b = nullptr;
        plan_stream = SpmvPlan{};
        plan_merge = SpmvPlan{};
        plan_adaptive = SpmvPlan{};
        plan_inter = SpmvPlan{};
        host_reach.clear();
        drop_host_graph();
    }
    const uint64_t *d_off() const { return off.as<uint64_t>(); }
    const uint32_t *d_cols() const { return cols.as<uint32_t>(); }
    const double *d_vals() const { return vals.as<double>(); }
    // Frees the device arrays while the owning context's stream still exists.
    void orphan() {
        invalidate_derived();
        off.release();
        cols.release();
        vals.release();
        stage_x.release();  // every device buffer goes while the context's stream exists
        stage_y.release();
        built = false;
        nnz = capacity = 0;
        ctx = nullptr;
    }
};

// Checks that a handle still belongs to a live context.
#define SPG_CHECK_LIVE(A)                                                                              \
    do {                                                                                               \
        if ((A)->ctx == nullptr)                                                                       \
            return ::spg::set_error(SPG_ERR_LOGIC, "the matrix's context was destroyed");             \
    } while (0)

inline cudaStream_t pick_stream(Ctx *c, void *s) {
    return s ? static_cast<cudaStream_t>(s) : c->stream;
}

inline int bits_for(uint64_t n) {  // bits needed to represent 0..n-1
    int b = 0;
    while (b < 64 && (n - 1) >> b) ++b;
    return n <= 1 ? 0 : b;
}

// Elements to allocate for CSR cols/vals of a given capacity: rounded up to a
// multiple of 16 plus 16 more, so kernels that read whole 16-aligned chunks of
// 16 entries (SPG_SPMV_ADAPTIVE) never touch memory past the allocation.
inline uint64_t csr_alloc_elems(uint64_t cap) { return ((cap + 15) & ~15ull) + 16; }
// Entries to allocate for CSR offsets of n rows: n + 1 plus 2 spare, so a
// 16-byte bulk copy of offsets [r0 & ~1, r1 + 1] rounded to an even count
// stays inside the allocation.
inline uint64_t csr_off_elems(uint64_t n_rows) { return n_rows + 3; }

// Ascending bitonic sort of the 32 * E keys a warp holds, key[e] of lane l
// being element 32 e + l. Partners 32 or more apart share a lane (registers),
// nearer ones are exchanged by shuffles.
// k0 > 2 (warp-uniform) skips the stages below k0: the caller guarantees
// that every block of k0 / 2 network positions is already sorted, ascending
// where (position & k0 / 2) == 0 and descending elsewhere.
template <int E, class K>
__device__ __forceinline__ void warp_bitonic(K (&key)[E], int lane, int k0 = 2) {
#pragma unroll
    for (int k = 2; k <= 32 * E; k <<= 1) {
        if (k < k0) continue;
#pragma unroll
        for (int j = k >> 1; j > 0; j >>= 1) {
            if (j >= 32) {
                const int jj = j >> 5;
#pragma unroll
                for (int e = 0; e < E; ++e) {
                    if ((e & jj) == 0) {
                        const int f = e | jj;
                        const bool up = ((32 * e) & k) == 0;  // k >= 64: the item decides
                        const K a = key[e], b = key[f];
                        const bool sw = up ? (a > b) : (a < b);
                        key[e] = sw ? b : a;
                        key[f] = sw ? a : b;
                    }
                }
            } else {
#pragma unroll
                for (int e = 0; e < E; ++e) {
                    const K o = __shfl_xor_sync(0xffffffffu, key[e], j);
                    const int i = 32 * e + lane;
                    const bool keep_min = (((i & k) == 0) == ((i & j) == 0));
                    key[e] = keep_min ? (o < key[e] ? o : key[e]) : (o > key[e] ? o : key[e]);
                }
            }
        }
    }
}

// Spira's ValueTraits<double>::is_zero (traits.hpp:73-80): +0 and -0 are
// zero, NaN is not; also exactly Spira's SpGEMM drop test `v != V{}`
// (spgemm.hpp:44) negated. Tested on the bit pattern (every bit but the sign
// clear): integer ALU work instead of an FP64 compare, which costs as much
// FP64 pipe time as a multiply on GB300.
__device__ __forceinline__ bool is_zero(double v) { return (__double_as_longlong(v) << 1) == 0; }

// Lanes of the (full) warp whose NB-bit value d (a radix digit, or 256 for
// "no key" when NB = 9) equals this lane's: NB ballots on the ALU pipe,
// cheaper on GB300 than match.any, which issues on the narrow
// address-divergence unit.
template <int NB = 9>
__device__ __forceinline__ unsigned warp_match_digit(unsigned d) {
    unsigned peers = 0xffffffffu;
#pragma unroll
    for (int b = 0; b < NB; ++b) {
        const unsigned bit = (d >> b) & 1u;
        const unsigned bal = __ballot_sync(0xffffffffu, bit);
        peers &= bit ? bal : ~bal;
    }
    return peers;
}

inline unsigned grid_for(uint64_t n, unsigned block, unsigned cap = 1u << 30) {
    uint64_t g = (n + block - 1) / block;
    if (g == 0) g = 1;
    if (g > cap) g = cap;
    return static_cast<unsigned>(g);
}

// ---------------------------------------------------------------------------
// Device-wide primitives (spg_prims.cu)
// ---------------------------------------------------------------------------
// Exclusive scan of n uint64 values in place; writes the total to *d_total
// (device pointer, may be null). Temporary memory from the context pool.
int exclusive_scan_u64(Ctx *c, uint64_t *d_data, uint64_t n, uint64_t *d_total,
                       cudaStream_t s);
// Exclusive scan of int64 (signed) values in place.
int exclusive_scan_i64(Ctx *c, int64_t *d_data, uint64_t n, cudaStream_t s);
// Stable LSD radix sort of 64-bit keys carrying a 32-bit payload, on the low
// `key_bits` bits. Inputs are consumed; results land in (keys, vals) again.
int radix_sort_pairs_u64(Ctx *c, uint64_t *d_keys, uint32_t *d_vals, uint64_t n,
                         int key_bits, cudaStream_t s);
// Stable (row, col) order of m pairs whose rows are non-decreasing, sorted
// row by row on chip (rows of up to 32 entries in registers, longer ones in
// shared memory): keys_out = row << cbits | col, idx_out = input position.
// s_off[r] = first position of row r (n_rows + 1 entries). *done = false when
// a row has more than 12 288 entries or columns need more than 26 bits; the
// outputs are then undefined.
// The first lock of row-grouped inserts in one pass of the same sort: every
// row's last write per column, unless zero, in column order at the row's
// first input positions (out_cols / out_vals[s_off[r] + k], k < kept[r]);
// kept[r] for every row r < n_rows. *done as for sort_grouped_rows.
int dedup_grouped_rows(Ctx *c, const uint32_t *cols, const double *vals, const uint64_t *s_off, uint64_t m,
                       uint64_t n_rows, int cbits, uint32_t *out_cols, double *out_vals, uint64_t *kept, bool *done,
                       cudaStream_t s);
int sort_grouped_rows(Ctx *c, const uint32_t *rows, const uint32_t *cols, const uint64_t *s_off, uint64_t m,
                      uint64_t n_rows, int cbits, uint64_t *keys_out, uint32_t *idx_out, bool *done, cudaStream_t s);

// SpGEMM pieces shared by its variants (spg_spgemm.cu, spg_spgemm_sort.cu).
// Expand - sort - compress output: kept entries in (row, column) order.
struct EscOut {
    DevBuf crow, ccol, cval;
    uint64_t n = 0;
};
int spgemm_esc(Ctx *c, const Csr *A, const Csr *B, const uint64_t *hp, uint64_t HP, int rbits, int cbits,
               EscOut *out, cudaStream_t s);
void spgemm_install(Csr *Cm, uint64_t m, uint64_t n, DevBuf &&off, DevBuf &&cols, DevBuf &&vals, uint64_t nnz);
uint64_t read_u64(Ctx *c, const uint64_t *d, cudaStream_t s, int *rc);
int spgemm_warpsort(Ctx *c, const Csr *A, const Csr *B, Csr *Cm, int variant, cudaStream_t s);
int spgemm_run(Ctx *c, const Csr *A, const Csr *B, Csr *Cm, int variant, cudaStream_t s);
// SPG_SPGEMM_AUTO resolved by the context's policy (spg_tune.cu).
int spgemm_resolve_auto(Ctx *c, const Csr *A, const Csr *B, int *variant);

// CSR helpers used by several ops (spg_lock.cu).
int csr_alloc(Csr *A, uint64_t capacity, cudaStream_t s);

// SpMV dispatch (spg_spmv.cu).
int spmv_launch(Ctx *c, Csr *A, const double *x, double *y, int variant,
                cudaStream_t s);
int spmv_resolve_auto(Ctx *c, Csr *A, int *variant);
// Loads spg_selector.bin from beside libspg.so (or $SPG_SELECTOR_MODEL) if any.
int selector_load_default(Ctx *c);
// Looks up the device address of spg_spmv_noalloc's scratch array for the
// current device again (spg_spmv.cu); spg_ctx_create calls it.
void noalloc_refresh(int device);
// SPG_SPMV_ADAPTIVE, SPG_SPMV_ADAPTIVE16 and SPG_SPMV_INTERLEAVED
// (spg_spmv_adaptive.cu); each builds and caches its plan on first use.
int spmv_adaptive(Ctx *c, Csr *A, const double *x, double *y, int variant, cudaStream_t s);
int build_adaptive_plan(Ctx *c, Csr *A, int variant, cudaStream_t s);
// Pipelined form for the host entry point: splits the chunks into at most nb
// blocks (fewer if a row could outrun the one-block look-ahead of the fix-up)
// and returns the first row of each block (rows->back() = n_rows). Stage i
// (0 <= i <= blocks) enqueues block i's chunks (i < blocks) and block i-1's
// fix-up (i >= 1): after stage i, rows [rows[i-1], rows[i]) are final.
int spmv_adaptive_blocks(Ctx *c, Csr *A, int variant, int nb, std::vector<uint64_t> *rows, cudaStream_t s);
int spmv_adaptive_stage(Ctx *c, Csr *A, const double *x, double *y, int variant, int i, cudaStream_t s);
// Rows [r0, r1) of a row-parallel variant (SCALAR, VECTOR*); others give
// SPG_ERR_UNSUPPORTED.
int spmv_launch_rows(Ctx *c, Csr *A, const double *x, double *y, int variant, uint64_t r0, uint64_t r1,
                     cudaStream_t s);
// A->host_reach for nb equal row blocks (cached until the next lock).
int spmv_row_block_reach(Ctx *c, Csr *A, int nb, cudaStream_t s);
// Fills A->max_row (the longest row) once per CSR; `known` false while `s`
// is being captured (the count needs a synchronisation).
int csr_max_row(Ctx *c, Csr *A, cudaStream_t s, bool *known);
// Builds whatever plan `variant` needs, so that a later spmv_launch only
// enqueues work (plans synchronise: callers that record a CUDA graph call it
// before the recording).
int spmv_prepare(Ctx *c, Csr *A, int variant, cudaStream_t s);
// Shape of a chunk-kernel variant (ADAPTIVE, ADAPTIVE16, INTERLEAVED and
// their tiles): nonzeros per lane, sub-batch depth, interleaved copy, blocks
// of 256 threads per SM. items == 0 for every other variant.
struct SegShape {
    int items, sub;
    bool inter;
    int minb;
};
inline SegShape seg_shape(int variant) {
    switch (variant) {
        case SPG_SPMV_ADAPTIVE: return {32, 8, false, 4};
        case SPG_SPMV_ADAPTIVE16: return {16, 8, false, 4};
        case SPG_SPMV_INTERLEAVED: return {16, 2, true, 8};
        case SPG_SPMV_INTERLEAVED_S4: return {16, 4, true, 5};
        case SPG_SPMV_INTERLEAVED_S8: return {16, 8, true, 4};
        case SPG_SPMV_ADAPTIVE16_S4: return {16, 4, false, 6};
        case SPG_SPMV_ADAPTIVE_S16: return {32, 16, false, 2};
        default: return {0, 0, false, 0};
    }
}
inline bool spmv_is_seg(int variant) { return seg_shape(variant).items != 0; }
// The cached plan slot of one of those variants (tiles share their base's).
inline SpmvPlan &adaptive_plan_of(Csr *A, int variant) {
    return seg_shape(variant).inter ? A->plan_inter : A->plan_adaptive;
}

}  // namespace spg

// Opaque C handle types are the internal structs.
struct spg_ctx : spg::Ctx {};
struct spg_csr : spg::Csr {};
