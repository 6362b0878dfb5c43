// spg_batch.cu — many independent CSR matrices, each with k right-hand sides
// (k in 1..32), in one persistent launch replayed from a CUDA graph.
//
// No Spira counterpart: Spira multiplies one matrix by one vector per call
// (serial/spmv.hpp:141-186); a batch item here is exactly that SpMV repeated
// over the k columns of a row-major X (n_cols x k) into Y (n_rows x k), and
// the plain comparison path issues it that way, one launch per matrix per
// right-hand side.
//
// Work items are (matrix, row tile) pairs sized to roughly equal nnz * k and
// handed out through a global atomic counter (reset by a memset node of the
// same graph), so one launch balances matrices of very uneven size. A warp
// maps its 32 lanes to (row slot, right-hand side) = (32 / k rows) x k: every
// lane runs one FMA chain over its row, the k lanes of a row read the same
// column index and value and k consecutive X entries (coalesced). FP64: one
// FMA per (nonzero, right-hand side). Tile size and CTAs per SM come from a
// small autotuner run on the batch itself.
#include <algorithm>
#include <vector>

#include "spg_internal.cuh"

struct spg_batch;

namespace spg {
namespace {

struct BatchMat {
    const uint64_t *off;
    const uint32_t *cols;
    const double *vals;
    const double *X;
    double *Y;
    const uint32_t *perm;  // rows in ascending length (k < 32), or null: rows in order
    uint32_t n_rows;
    uint32_t k;
};

struct BatchItem {
    uint32_t mat;
    uint32_t row0;
    uint32_t row1;
    uint32_t pad;
};

constexpr int BT = 256;

__global__ void __launch_bounds__(BT)
batch_persistent(const BatchMat *__restrict__ mats, const BatchItem *__restrict__ items, uint32_t n_items,
                 unsigned *__restrict__ counter) {
    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    __shared__ uint32_t s_item[BT / 32];
    for (;;) {
        if (lane == 0) s_item[wib] = atomicAdd(counter, 1u);
        __syncwarp();
        const uint32_t it = s_item[wib];
        __syncwarp();
        if (it >= n_items) return;
        const BatchItem itm = items[it];
        const BatchMat M = mats[itm.mat];
        const uint32_t k = M.k;  // power of two, 1..32
        const uint32_t slots = 32u / k;
        const uint32_t slot = (uint32_t)lane / k, j = (uint32_t)lane % k;
        for (uint32_t p = itm.row0 + slot; p < itm.row1; p += slots) {
            // With k < 32 a warp pass runs 32 / k rows side by side and issues
            // FP64 work for the longest; visiting rows in ascending length
            // keeps the rows of a pass nearly equal (a masked FP64 lane costs
            // the same issue slot as a busy one).
            const uint32_t r = M.perm ? M.perm[p] : p;
            const uint64_t b = M.off[r], e = M.off[r + 1];
            // One FMA chain in column order (Spira's scalar order with fused
            // multiply-adds): the FP64 pipe, not FMA latency, bounds this
            // loop, so a second accumulator would only add a final DADD per
            // row. Pairs keep two gathers in flight per lane.
            double acc = 0.0;
            uint64_t q = b;
            for (; q + 1 < e; q += 2) {
                const uint32_t c0 = M.cols[q], c1 = M.cols[q + 1];
                const double v0 = M.vals[q], v1 = M.vals[q + 1];
                const double x0 = __ldg(M.X + (uint64_t)c0 * k + j), x1 = __ldg(M.X + (uint64_t)c1 * k + j);
                acc = fma(v1, x1, fma(v0, x0, acc));
            }
            if (q < e) acc = fma(M.vals[q], __ldg(M.X + (uint64_t)M.cols[q] * k + j), acc);
            M.Y[(uint64_t)r * k + j] = acc;
        }
    }
}

// Row order for the k < 32 matrices: rows sorted by length (ties by index)
// inside windows of WIN consecutive rows. Windows keep the rows a warp
// touches close together (row offsets and Y stay in the same L2 lines)
// while the rows of one warp pass come out with nearly equal lengths.
constexpr int WIN = 256;

// Block per window; win_base[m] = first window of matrix m (n + 1 entries),
// perm + row_base[m] = matrix m's permutation.
__global__ void __launch_bounds__(WIN)
batch_window_sort(const BatchMat *__restrict__ mats, const uint64_t *__restrict__ win_base,
                  const uint64_t *__restrict__ row_base, uint32_t n, uint32_t *__restrict__ perm) {
    __shared__ uint32_t s_len[WIN];
    const uint64_t w = blockIdx.x;
    uint32_t lo = 0, hi = n - 1;  // matrix m with win_base[m] <= w < win_base[m + 1]
    while (lo < hi) {
        const uint32_t mid = (lo + hi + 1) >> 1;
        if (win_base[mid] <= w) lo = mid;
        else hi = mid - 1;
    }
    const BatchMat M = mats[lo];
    const uint32_t r0 = (uint32_t)(w - win_base[lo]) * WIN;
    const uint32_t cnt = min((uint32_t)WIN, M.n_rows - r0);
    const uint32_t i = threadIdx.x;
    uint32_t len = 0xFFFFFFFFu;
    if (i < cnt) {
        const uint64_t l = M.off[r0 + i + 1] - M.off[r0 + i];
        len = l < 0xFFFFFFFEull ? (uint32_t)l : 0xFFFFFFFEu;
    }
    s_len[i] = len;
    __syncthreads();
    if (i < cnt) {
        uint32_t rank = 0;
        for (uint32_t j = 0; j < cnt; ++j) {
            const uint32_t lj = s_len[j];
            rank += (lj < len) || (lj == len && j < i);
        }
        perm[row_base[lo] + r0 + rank] = r0 + i;
    }
}

// Plain path: one launch per matrix per right-hand side, thread per row.
__global__ void batch_plain_column(const uint64_t *__restrict__ off, const uint32_t *__restrict__ cols,
                                   const double *__restrict__ vals, const double *__restrict__ X,
                                   double *__restrict__ Y, uint32_t n_rows, uint32_t k, uint32_t j) {
    const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n_rows) return;
    double acc = 0.0;
    for (uint64_t q = off[r]; q < off[r + 1]; ++q) acc = fma(vals[q], __ldg(X + (uint64_t)cols[q] * k + j), acc);
    Y[(uint64_t)r * k + j] = acc;
}

}  // namespace

struct Batch {
    Ctx *ctx = nullptr;
    uint32_t n_mats = 0;
    std::vector<BatchMat> host_mats;
    std::vector<uint64_t> mat_nnz;
    DevBuf d_mats, d_items, d_counter, d_perm;
    uint32_t n_items = 0;
    int tile_nnzk = 0;  // target nnz * k per work item
    int ctas_per_sm = 0;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    void release() {
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
        exec = nullptr;
        graph = nullptr;
        d_mats.release();
        d_items.release();
        d_counter.release();
        d_perm.release();
    }
    ~Batch() { release(); }
};

void batch_orphan(Batch *b) {
    b->release();
    b->ctx = nullptr;
}

static int batch_build_items(Batch *B, int tile_nnzk, cudaStream_t s) {
    std::vector<BatchItem> items;
    for (uint32_t m = 0; m < B->n_mats; ++m) {
        const BatchMat &M = B->host_mats[m];
        if (!M.n_rows) continue;
        const double per_row = std::max(1.0, (double)B->mat_nnz[m] / M.n_rows) * M.k;
        uint32_t rows = (uint32_t)std::max(1.0, tile_nnzk / per_row);
        const uint32_t slots = 32u / M.k;
        rows = ((rows + slots - 1) / slots) * slots;  // whole warp passes
        for (uint32_t r = 0; r < M.n_rows; r += rows) items.push_back({m, r, std::min(M.n_rows, r + rows), 0});
    }
    B->n_items = (uint32_t)items.size();
    SPG_TRY(B->d_items.alloc(std::max<size_t>(1, items.size()) * sizeof(BatchItem), s));
    if (!items.empty())
        SPG_CUDA_TRY(cudaMemcpyAsync(B->d_items.ptr, items.data(), items.size() * sizeof(BatchItem),
                                     cudaMemcpyHostToDevice, s));
    SPG_CUDA_TRY(cudaStreamSynchronize(s));
    B->tile_nnzk = tile_nnzk;
    return SPG_OK;
}

static int batch_capture(Batch *B, cudaStream_t s) {
    if (B->exec) cudaGraphExecDestroy(B->exec);
    if (B->graph) cudaGraphDestroy(B->graph);
    B->exec = nullptr;
    B->graph = nullptr;
    Ctx *c = B->ctx;
    const unsigned grid = (unsigned)std::max(1, B->ctas_per_sm * c->n_sms);
    cudaStream_t cs;
    SPG_CUDA_TRY(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
    cudaError_t e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) e = cudaMemsetAsync(B->d_counter.ptr, 0, sizeof(unsigned), cs);
    if (e == cudaSuccess && B->n_items) {
        batch_persistent<<<grid, BT, 0, cs>>>(B->d_mats.as<BatchMat>(), B->d_items.as<BatchItem>(), B->n_items,
                                              B->d_counter.as<unsigned>());
        e = cudaPeekAtLastError();
    }
    cudaGraph_t g = nullptr;
    const cudaError_t e2 = cudaStreamEndCapture(cs, &g);
    if (e == cudaSuccess) e = e2;
    if (e == cudaSuccess) e = cudaGraphInstantiate(&B->exec, g, 0);
    cudaStreamDestroy(cs);
    B->graph = g;
    if (e != cudaSuccess) return set_error(SPG_ERR_CUDA, "batch graph capture: %s", cudaGetErrorString(e));
    (void)s;
    return SPG_OK;
}

static int batch_time(Batch *B, cudaStream_t s, int reps, float *ms) {
    cudaEvent_t e0, e1;
    SPG_CUDA_TRY(cudaEventCreate(&e0));
    SPG_CUDA_TRY(cudaEventCreate(&e1));
    SPG_CUDA_TRY(cudaGraphLaunch(B->exec, s));  // warm-up
    std::vector<float> t(reps);
    for (int r = 0; r < reps; ++r) {
        cudaEventRecord(e0, s);
        cudaGraphLaunch(B->exec, s);
        cudaEventRecord(e1, s);
        cudaEventSynchronize(e1);
        cudaEventElapsedTime(&t[r], e0, e1);
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    SPG_CUDA_TRY(cudaGetLastError());
    std::sort(t.begin(), t.end());
    *ms = t[t.size() / 2];
    return SPG_OK;
}

}  // namespace spg

struct spg_batch : spg::Batch {};

using namespace spg;

extern "C" {

int spg_batch_create(spg_ctx *c, uint32_t n, const spg_csr *const *mats, const double *const *d_X,
                     double *const *d_Y, const uint32_t *k, int config, spg_batch **out) {
    if (!c || !out || (n && (!mats || !d_X || !d_Y || !k)))
        return set_error(SPG_ERR_INVALID_ARGUMENT, "spg_batch_create: null argument");
    *out = nullptr;
    SPG_CUDA_TRY(cudaSetDevice(c->device));
    cudaStream_t s = c->stream;
    spg_batch *B = new spg_batch();
    B->ctx = c;
    B->n_mats = n;
    for (uint32_t m = 0; m < n; ++m) {
        const spg_csr *A = mats[m];
        const uint32_t km = k[m];
        if (!A || !A->built) {
            delete B;
            return set_error(SPG_ERR_LOGIC, "spg_batch_create: matrix %u is not locked", m);
        }
        if (km == 0 || km > 32 || (km & (km - 1))) {
            delete B;
            return set_error(SPG_ERR_INVALID_ARGUMENT, "spg_batch_create: k[%u] = %u is not a power of two <= 32", m,
                             km);
        }
        if (A->n_rows > 0xFFFFFFFFull || ((A->n_rows || A->n_cols) && (!d_X[m] || !d_Y[m]))) {
            delete B;
            return set_error(SPG_ERR_INVALID_ARGUMENT, "spg_batch_create: bad matrix %u", m);
        }
        B->host_mats.push_back(
            {A->d_off(), A->d_cols(), A->d_vals(), d_X[m], d_Y[m], nullptr, (uint32_t)A->n_rows, km});
        B->mat_nnz.push_back(A->nnz);
    }
    // length-sorted row windows for the matrices that share a warp pass
    std::vector<uint64_t> row_base(n + 1, 0), win_base(n + 1, 0);
    for (uint32_t m = 0; m < n; ++m) {
        const BatchMat &M = B->host_mats[m];
        const uint64_t rows = M.k < 32 ? M.n_rows : 0;
        row_base[m + 1] = row_base[m] + rows;
        win_base[m + 1] = win_base[m] + (rows + WIN - 1) / WIN;
    }
    int rc = SPG_OK;
    DevBuf d_bases;
    if (win_base[n]) {
        rc = B->d_perm.alloc(row_base[n] * sizeof(uint32_t), s);
        if (rc == SPG_OK) rc = d_bases.alloc(2 * (n + 1) * sizeof(uint64_t), s);
        if (rc == SPG_OK)
            for (uint32_t m = 0; m < n; ++m)
                if (row_base[m + 1] > row_base[m]) B->host_mats[m].perm = B->d_perm.as<uint32_t>() + row_base[m];
    }
    if (rc == SPG_OK) rc = B->d_mats.alloc(std::max<size_t>(1, n) * sizeof(BatchMat), s);
    if (rc == SPG_OK && n)
        rc = cudaMemcpyAsync(B->d_mats.ptr, B->host_mats.data(), n * sizeof(BatchMat), cudaMemcpyHostToDevice, s) ==
                     cudaSuccess
                 ? SPG_OK
                 : set_error(SPG_ERR_CUDA, "spg_batch_create: copy failed");
    if (rc == SPG_OK && win_base[n]) {
        uint64_t *bases = d_bases.as<uint64_t>();
        if (cudaMemcpyAsync(bases, win_base.data(), (n + 1) * sizeof(uint64_t), cudaMemcpyHostToDevice, s) !=
                cudaSuccess ||
            cudaMemcpyAsync(bases + n + 1, row_base.data(), (n + 1) * sizeof(uint64_t), cudaMemcpyHostToDevice, s) !=
                cudaSuccess)
            rc = set_error(SPG_ERR_CUDA, "spg_batch_create: copy failed");
        if (rc == SPG_OK) {
            batch_window_sort<<<(unsigned)win_base[n], WIN, 0, s>>>(B->d_mats.as<BatchMat>(), bases, bases + n + 1, n,
                                                                  B->d_perm.as<uint32_t>());
            if (cudaPeekAtLastError() != cudaSuccess) rc = set_error(SPG_ERR_CUDA, "spg_batch_create: row sort failed");
        }
        // the bases must outlive the sort: host vectors back the copies
        if (rc == SPG_OK && cudaStreamSynchronize(s) != cudaSuccess)
            rc = set_error(SPG_ERR_CUDA, "spg_batch_create: row sort failed");
    }
    if (rc == SPG_OK) rc = B->d_counter.alloc(sizeof(unsigned), s);
    if (rc != SPG_OK) {
        delete B;
        return rc;
    }
    static const int tiles[] = {2048, 4096, 8192, 16384};
    static const int ctas[] = {4, 8};
    if (config >= 0) {
        const int ti = config % 4, ci = (config / 4) % 2;
        B->ctas_per_sm = ctas[ci];
        rc = batch_build_items(B, tiles[ti], s);
        if (rc == SPG_OK) rc = batch_capture(B, s);
    } else {
        // autotune the tile size and CTAs per SM on the batch itself
        float best = 0.0f;
        int best_cfg = 0;
        for (int cfg = 0; cfg < 8 && rc == SPG_OK; ++cfg) {
            B->ctas_per_sm = ctas[cfg / 4];
            rc = batch_build_items(B, tiles[cfg % 4], s);
            if (rc == SPG_OK) rc = batch_capture(B, s);
            float ms = 0.0f;
            if (rc == SPG_OK) rc = batch_time(B, s, 3, &ms);
            if (rc == SPG_OK && (cfg == 0 || ms < best)) {
                best = ms;
                best_cfg = cfg;
            }
        }
        if (rc == SPG_OK) {
            B->ctas_per_sm = ctas[best_cfg / 4];
            rc = batch_build_items(B, tiles[best_cfg % 4], s);
            if (rc == SPG_OK) rc = batch_capture(B, s);
        }
        config = best_cfg;
    }
    if (rc != SPG_OK) {
        delete B;
        return rc;
    }
    c->live_batches.push_back(B);
    *out = B;
    return SPG_OK;
}

int spg_batch_config(const spg_batch *B, int *config, uint32_t *n_items) {
    if (!B) return set_error(SPG_ERR_INVALID_ARGUMENT, "spg_batch_config: null batch");
    if (config) {
        const int ti = B->tile_nnzk == 2048 ? 0 : B->tile_nnzk == 4096 ? 1 : B->tile_nnzk == 8192 ? 2 : 3;
        *config = ti + 4 * (B->ctas_per_sm == 8 ? 1 : 0);
    }
    if (n_items) *n_items = B->n_items;
    return SPG_OK;
}

int spg_batch_run(spg_ctx *c, spg_batch *B, void *stream) {
    if (!c || !B) return set_error(SPG_ERR_INVALID_ARGUMENT, "spg_batch_run: null argument");
    if (!B->ctx) return set_error(SPG_ERR_LOGIC, "the batch's context was destroyed");
    SPG_CUDA_TRY(cudaSetDevice(c->device));
    SPG_CUDA_TRY(cudaGraphLaunch(B->exec, pick_stream(c, stream)));
    return SPG_OK;
}

int spg_batch_run_plain(spg_ctx *c, spg_batch *B, void *stream) {
    if (!c || !B) return set_error(SPG_ERR_INVALID_ARGUMENT, "spg_batch_run_plain: null argument");
    if (!B->ctx) return set_error(SPG_ERR_LOGIC, "the batch's context was destroyed");
    SPG_CUDA_TRY(cudaSetDevice(c->device));
    cudaStream_t s = pick_stream(c, stream);
    for (const BatchMat &M : B->host_mats) {
        if (!M.n_rows) continue;
        for (uint32_t j = 0; j < M.k; ++j)
            batch_plain_column<<<grid_for(M.n_rows, 256), 256, 0, s>>>(M.off, M.cols, M.vals, M.X, M.Y, M.n_rows, M.k,
                                                                      j);
    }
    SPG_LAUNCH_CHECK();
    return SPG_OK;
}

int spg_batch_destroy(spg_batch *B) {
    if (!B) return SPG_OK;
    if (Ctx *c = B->ctx) {
        cudaSetDevice(c->device);
        auto &v = c->live_batches;
        v.erase(std::remove(v.begin(), v.end(), static_cast<Batch *>(B)), v.end());
    }
    delete B;
    return SPG_OK;
}

}  // extern "C"
