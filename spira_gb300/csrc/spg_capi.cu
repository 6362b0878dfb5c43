// spg_capi.cu — the extern "C" surface of libspg.so: contexts, CSR handles,
// host<->device transfer, load_csr validation, point lookup and SpMV entry
// points. Lock lives in spg_lock.cu; kernels in spg_spmv.cu.
#include <algorithm>
#include <cstring>
#include <new>
#include <string>

#include "spg_internal.cuh"

namespace spg {

static thread_local std::string g_last_error;

int set_error(int code, const char *fmt, ...) {
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return code;
}

void clear_error() { g_last_error.clear(); }

int Ctx::phase_sync(cudaStream_t s) {
    const bool timed = timer_on && s == stream;
    if (timed) SPG_CUDA_TRY(cudaEventRecord(timer_ev[1], s));
    SPG_CUDA_TRY(cudaStreamSynchronize(s));
    if (timed) {
        float ms = 0.0f;
        SPG_CUDA_TRY(cudaEventElapsedTime(&ms, timer_ev[0], timer_ev[1]));
        timer_ms += ms;
        SPG_CUDA_TRY(cudaEventRecord(timer_ev[0], s));  // the next phase starts with the next work
    }
    return SPG_OK;
}

int Ctx::ensure_pinned(size_t bytes) {
    if (pinned_bytes >= bytes) return SPG_OK;
    if (pinned) cudaFreeHost(pinned);
    pinned = nullptr;
    pinned_bytes = 0;
    SPG_CUDA_TRY(cudaMallocHost(&pinned, bytes));
    pinned_bytes = bytes;
    return SPG_OK;
}

int csr_alloc(Csr *A, uint64_t capacity, cudaStream_t s) {
    SPG_TRY(A->cols.alloc(csr_alloc_elems(capacity) * sizeof(uint32_t), s));
    SPG_TRY(A->vals.alloc(csr_alloc_elems(capacity) * sizeof(double), s));
    A->capacity = capacity;
    return SPG_OK;
}

namespace {

__global__ void csr_get_kernel(const uint64_t *__restrict__ off, const uint32_t *__restrict__ cols,
                               const double *__restrict__ vals, uint64_t row, uint32_t col,
                               double *out_val, int *out_found) {
    // csr_slice::binary_search (csr_storage_soa.hpp:94-104): lower_bound on
    // the row's strictly ascending columns.
    uint64_t lo = off[row], hi = off[row + 1];
    while (lo < hi) {
        const uint64_t mid = (lo + hi) >> 1;
        if (cols[mid] < col) lo = mid + 1;
        else hi = mid;
    }
    const bool found = lo < off[row + 1] && cols[lo] == col;
    *out_found = found ? 1 : 0;
    *out_val = found ? vals[lo] : 0.0;
}

}  // namespace

// True for page-locked (pinned or registered) host memory.
static bool host_pinned(const void *p) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeHost;
}

}  // namespace spg

using namespace spg;

extern "C" {

const char *spg_strerror(int status) {
    switch (status) {
        case SPG_OK: return "ok";
        case SPG_ERR_INVALID_ARGUMENT: return "invalid argument";
        case SPG_ERR_LOGIC: return "logic error (wrong mode)";
        case SPG_ERR_OUT_OF_RANGE: return "index out of range";
        case SPG_ERR_NO_MEMORY: return "out of device memory";
        case SPG_ERR_CUDA: return "CUDA runtime error";
        case SPG_ERR_DEVICE_TIMEOUT: return "device-side wait timed out";
        case SPG_ERR_UNSUPPORTED: return "unsupported";
        case SPG_ERR_DOMAIN: return "domain error";
        default: return "unknown status";
    }
}

const char *spg_last_error(void) { return g_last_error.c_str(); }

int spg_version(void) { return 10000; }

int spg_ctx_create(int device, spg_ctx **out) {
    if (!out) return set_error(SPG_ERR_INVALID_ARGUMENT, "spg_ctx_create: out is null");
    *out = nullptr;
    int n = 0;
    SPG_CUDA_TRY(cudaGetDeviceCount(&n));
    if (device < 0 || device >= n)
        return set_error(SPG_ERR_INVALID_ARGUMENT, "spg_ctx_create: device %d of %d", device, n);
    SPG_CUDA_TRY(cudaSetDevice(device));
    cudaDeviceProp prop;
    SPG_CUDA_TRY(cudaGetDeviceProperties(&prop, device));
    if (prop.major < 10)
        return set_error(SPG_ERR_UNSUPPORTED, "spg_ctx_create: device %d is sm_%d%d; libspg targets sm_103a",
                         device, prop.major, prop.minor);
    spg_ctx *c = new (std::nothrow) spg_ctx();
    if (!c) return set_error(SPG_ERR_NO_MEMORY, "spg_ctx_create: host allocation failed");
    c->device = device;
    c->n_sms = prop.multiProcessorCount;
    c->l2_bytes = prop.l2CacheSize;
    cudaError_t e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->copy_stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->upload_stream, cudaStreamNonBlocking);
    for (int i = 0; i < Ctx::N_HOST_EVENTS && e == cudaSuccess; ++i) {
        e = cudaEventCreateWithFlags(&c->host_events[i], cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->upload_events[i], cudaEventDisableTiming);
    }
    if (e == cudaSuccess) e = cudaDeviceGetDefaultMemPool(&c->pool, device);
    if (e == cudaSuccess) {
        uint64_t thr = UINT64_MAX;  // keep freed blocks cached in the pool
        e = cudaMemPoolSetAttribute(c->pool, cudaMemPoolAttrReleaseThreshold, &thr);
    }
    // Status word in mapped pinned memory: kernels flag timeouts there and the
    // host reads it after a synchronisation without an extra copy.
    if (e == cudaSuccess) e = cudaHostAlloc(reinterpret_cast<void **>(&c->h_status), sizeof(unsigned),
                                            cudaHostAllocMapped);
    if (e == cudaSuccess) {
        *c->h_status = 0;
        e = cudaHostGetDevicePointer(reinterpret_cast<void **>(&c->d_status), c->h_status, 0);
    }
    if (e != cudaSuccess) {
        if (c->stream) cudaStreamDestroy(c->stream);
        if (c->copy_stream) cudaStreamDestroy(c->copy_stream);
        if (c->upload_stream) cudaStreamDestroy(c->upload_stream);
        for (int i = 0; i < Ctx::N_HOST_EVENTS; ++i) {
            if (c->host_events[i]) cudaEventDestroy(c->host_events[i]);
            if (c->upload_events[i]) cudaEventDestroy(c->upload_events[i]);
        }
        if (c->h_status) cudaFreeHost(c->h_status);
        delete c;
        return set_error(SPG_ERR_CUDA, "spg_ctx_create: %s", cudaGetErrorString(e));
    }
    noalloc_refresh(device);
    selector_load_default(c);
    *out = c;
    return SPG_OK;
}

int spg_ctx_destroy(spg_ctx *c) {
    if (!c) return SPG_OK;
    cudaSetDevice(c->device);
    cudaStreamSynchronize(c->stream);
    for (Batch *b : c->live_batches) batch_orphan(b);
    c->live_batches.clear();
    for (Csr *A : c->live_csrs) A->orphan();
    c->live_csrs.clear();
    c->model.release();
    c->gemm_model.release();
    c->xbuf.release();
    c->ybuf.release();
    cudaStreamSynchronize(c->stream);
    cudaStreamSynchronize(c->copy_stream);
    cudaStreamSynchronize(c->upload_stream);
    if (c->pinned) cudaFreeHost(c->pinned);
    if (c->h_status) cudaFreeHost(c->h_status);
    for (int i = 0; i < Ctx::N_HOST_EVENTS; ++i) {
        if (c->host_events[i]) cudaEventDestroy(c->host_events[i]);
        if (c->upload_events[i]) cudaEventDestroy(c->upload_events[i]);
    }
    for (cudaEvent_t e : c->timer_ev)
        if (e) cudaEventDestroy(e);
    c->drop_multi();
    for (int l = 0; l < Ctx::MULTI_MAX; ++l) {
        for (cudaStream_t &st : c->multi_stream[l])
            if (st) cudaStreamSynchronize(st), cudaStreamDestroy(st);
        for (cudaEvent_t &ev : c->multi_event[l])
            if (ev) cudaEventDestroy(ev);
    }
    cudaStreamDestroy(c->upload_stream);
    cudaStreamDestroy(c->copy_stream);
    cudaStreamDestroy(c->stream);
    delete c;
    return SPG_OK;
}

int spg_ctx_stream(spg_ctx *c, void **stream) {
    if (!c || !stream) return set_error(SPG_ERR_INVALID_ARGUMENT, "spg_ctx_stream: null argument");
    *stream = c->stream;
    return SPG_OK;
}

int spg_ctx_timer_start(spg_ctx *c) {
    if (!c) return set_error(SPG_ERR_INVALID_ARGUMENT, "spg_ctx_timer_start: null context");
    SPG_CUDA_TRY(cudaSetDevice(c->device));
    for (cudaEvent_t &e : c->timer_ev)
        if (!e) SPG_CUDA_TRY(cudaEventCreate(&e));
    SPG_CUDA_TRY(cudaStreamSynchronize(c->stream));
    c->timer_ms = 0.0;
    c->timer_on = true;
    SPG_CUDA_TRY(cudaEventRecord(c->timer_ev[0], c->stream));
    return SPG_OK;
}

int spg_ctx_timer_stop(spg_ctx *c, double *device_ms) {
    if (!c || !device_ms) return set_error(SPG_ERR_INVALID_ARGUMENT, "spg_ctx_timer_stop: null argument");
    if (!c->timer_on) return set_error(SPG_ERR_LOGIC, "spg_ctx_timer_stop: the timer is not running");
    SPG_CUDA_TRY(cudaSetDevice(c->device));
    const int rc = c->phase_sync(c->stream);
    c->timer_on = false;
    SPG_TRY(rc);
    *device_ms = c->timer_ms;
    return SPG_OK;
}

int spg_ctx_pool_used(spg_ctx *c, uint64_t *used_bytes, uint64_t *reserved_bytes) {
    if (!c) return set_error(SPG_ERR_INVALID_ARGUMENT, "spg_ctx_pool_used: null context");
    SPG_CUDA_TRY(cudaSetDevice(c->device));
    if (used_bytes) {
        uint64_t v = 0;  // the attribute is a 64-bit unsigned count
        SPG_CUDA_TRY(cudaMemPoolGetAttribute(c->pool, cudaMemPoolAttrUsedMemCurrent, &v));
        *used_bytes = v;
    }
    if (reserved_bytes) {
        uint64_t v = 0;  // the attribute is a 64-bit unsigned count
        SPG_CUDA_TRY(cudaMemPoolGetAttribute(c->pool, cudaMemPoolAttrReservedMemCurrent, &v));
        *reserved_bytes = v;
    }
    return SPG_OK;
}

int spg_ctx_sync(spg_ctx *c) {
    if (!c) return set_error(SPG_ERR_INVALID_ARGUMENT, "spg_ctx_sync: null context");
    SPG_CUDA_TRY(cudaStreamSynchronize(c->stream));
    return c->take_status();
}

int spg_csr_create(spg_ctx *c, uint64_t n_rows, uint64_t n_cols, spg_csr **out) {
    if (!c || !out) return set_error(SPG_ERR_INVALID_ARGUMENT, "spg_csr_create: null argument");
    if (n_rows > 0xFFFFFFFFull || n_cols > 0xFFFFFFFFull + 1ull)
        return set_error(SPG_ERR_INVALID_ARGUMENT,
                         "spg_csr_create: %llu x %llu exceeds uint32 row/column indices",
                         (unsigned long long)n_rows, (unsigned long long)n_cols);
    spg_csr *A = new (std::nothrow) spg_csr();
    if (!A) return set_error(SPG_ERR_NO_MEMORY, "spg_csr_create: host allocation failed");
    A->ctx = c;
    A->n_rows = n_rows;
    A->n_cols = n_cols;
    c->live_csrs.push_back(A);
    *out = A;
    return SPG_OK;
}

int spg_csr_destroy(spg_csr *A) {
    if (!A) return SPG_OK;
    if (Ctx *c = A->ctx) {  // still owned: unregister, free on the context's stream
        cudaSetDevice(c->device);
        auto &v = c->live_csrs;
        v.erase(std::remove(v.begin(), v.end(), static_cast<Csr *>(A)), v.end());
    }
    delete A;
    return SPG_OK;
}

int spg_csr_info_get(const spg_csr *A, spg_csr_info *info) {
    if (!A || !info) return set_error(SPG_ERR_INVALID_ARGUMENT, "spg_csr_info_get: null argument");
    info->n_rows = A->n_rows;
    info->n_cols = A->n_cols;
    info->nnz = A->nnz;
    info->capacity = A->capacity;
    info->built = A->built ? 1 : 0;
    return SPG_OK;
}

int spg_csr_device_arrays(const spg_csr *A, const uint64_t **offsets, const uint32_t **cols,
                          const double **vals) {
    if (!A) return set_error(SPG_ERR_INVALID_ARGUMENT, "spg_csr_device_arrays: null matrix");
    if (offsets) *offsets = A->d_off();
    if (cols) *cols = A->d_cols();
    if (vals) *vals = A->d_vals();
    return SPG_OK;
}

int spg_csr_download(spg_ctx *c, const spg_csr *A, uint64_t *offsets, uint32_t *cols, double *vals) {
    if (!c || !A) return set_error(SPG_ERR_INVALID_ARGUMENT, "spg_csr_download: null argument");
    if (!A->built) return set_error(SPG_ERR_LOGIC, "spg_csr_download: CSR not built (lock first)");
    SPG_CUDA_TRY(cudaSetDevice(c->device));
    cudaStream_t s = c->stream;
    if (offsets)
        SPG_CUDA_TRY(cudaMemcpyAsync(offsets, A->d_off(), (A->n_rows + 1) * sizeof(uint64_t),
                                     cudaMemcpyDeviceToHost, s));
    if (cols && A->nnz)
        SPG_CUDA_TRY(cudaMemcpyAsync(cols, A->d_cols(), A->nnz * sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
    if (vals && A->nnz)
        SPG_CUDA_TRY(cudaMemcpyAsync(vals, A->d_vals(), A->nnz * sizeof(double), cudaMemcpyDeviceToHost, s));
    SPG_CUDA_TRY(cudaStreamSynchronize(s));
    return SPG_OK;
}

int spg_csr_load(spg_ctx *c, spg_csr *A, const uint64_t *offsets, const uint32_t *cols,
                 const double *vals, uint64_t nnz) {
    if (!c || !A) return set_error(SPG_ERR_INVALID_ARGUMENT, "spg_csr_load: null handle");
    SPG_CHECK_LIVE(A);
    // Validation in the order of matrix::load_csr (matrix.hpp:524-575).
    if (!offsets) return set_error(SPG_ERR_INVALID_ARGUMENT, "spira::matrix::load_csr: CSR offsets array is null");
    if (offsets[0] != 0)
        return set_error(SPG_ERR_INVALID_ARGUMENT, "spira::matrix::load_csr: CSR offsets[0] must be zero");
    if (offsets[A->n_rows] != nnz)
        return set_error(SPG_ERR_INVALID_ARGUMENT,
                         "spira::matrix::load_csr: CSR offsets[n_rows] does not equal nnz");
    if (nnz && (!cols || !vals))
        return set_error(SPG_ERR_INVALID_ARGUMENT, "spg_csr_load: cols/vals null with nnz > 0");
    bool has_zero = false;
    for (uint64_t i = 0; i < A->n_rows; ++i) {
        const uint64_t beg = offsets[i], end = offsets[i + 1];
        if (beg > end)
            return set_error(SPG_ERR_INVALID_ARGUMENT,
                             "spira::matrix::load_csr: CSR offsets are not non-decreasing");
        if (end > nnz)
            return set_error(SPG_ERR_INVALID_ARGUMENT,
                             "spira::matrix::load_csr: CSR offsets are not non-decreasing");
        for (uint64_t k = beg; k < end; ++k) {
            if ((uint64_t)cols[k] >= A->n_cols)
                return set_error(SPG_ERR_INVALID_ARGUMENT,
                                 "spira::matrix::load_csr: column index out of bounds");
            if (k > beg && cols[k] <= cols[k - 1])
                return set_error(SPG_ERR_INVALID_ARGUMENT,
                                 "spira::matrix::load_csr: CSR row entries are not strictly sorted by column");
            if (vals[k] == 0.0) has_zero = true;
        }
    }
    SPG_CUDA_TRY(cudaSetDevice(c->device));
    cudaStream_t s = c->stream;
    DevBuf off, cb, vb;
    SPG_TRY(off.alloc(csr_off_elems(A->n_rows) * sizeof(uint64_t), s));
    SPG_TRY(cb.alloc(csr_alloc_elems(nnz) * sizeof(uint32_t), s));
    SPG_TRY(vb.alloc(csr_alloc_elems(nnz) * sizeof(double), s));
    SPG_CUDA_TRY(cudaMemcpyAsync(off.ptr, offsets, (A->n_rows + 1) * sizeof(uint64_t), cudaMemcpyHostToDevice, s));
    if (nnz) {
        SPG_CUDA_TRY(cudaMemcpyAsync(cb.ptr, cols, nnz * sizeof(uint32_t), cudaMemcpyHostToDevice, s));
        SPG_CUDA_TRY(cudaMemcpyAsync(vb.ptr, vals, nnz * sizeof(double), cudaMemcpyHostToDevice, s));
    }
    SPG_CUDA_TRY(cudaStreamSynchronize(s));
    A->invalidate_derived();
    A->off = std::move(off);
    A->cols = std::move(cb);
    A->vals = std::move(vb);
    A->nnz = nnz;
    A->capacity = nnz;
    A->built = true;
    A->may_have_zeros = has_zero;
    return SPG_OK;
}

int spg_csr_copy(spg_ctx *c, const spg_csr *src, spg_csr *dst) {
    if (!c || !src || !dst) return set_error(SPG_ERR_INVALID_ARGUMENT, "spg_csr_copy: null handle");
    SPG_CHECK_LIVE(src);
    SPG_CHECK_LIVE(dst);
    if (src == dst) return SPG_OK;
    SPG_CUDA_TRY(cudaSetDevice(c->device));
    cudaStream_t s = c->stream;
    dst->invalidate_derived();
    dst->n_rows = src->n_rows;
    dst->n_cols = src->n_cols;
    dst->built = src->built;
    dst->nnz = src->nnz;
    dst->may_have_zeros = src->may_have_zeros;
    if (!src->built) {
        dst->off.release();
        dst->cols.release();
        dst->vals.release();
        dst->capacity = 0;
        return SPG_OK;
    }
    DevBuf off, cb, vb;
    SPG_TRY(off.alloc(csr_off_elems(src->n_rows) * sizeof(uint64_t), s));
    SPG_TRY(cb.alloc(csr_alloc_elems(src->nnz) * sizeof(uint32_t), s));
    SPG_TRY(vb.alloc(csr_alloc_elems(src->nnz) * sizeof(double), s));
    SPG_CUDA_TRY(cudaMemcpyAsync(off.ptr, src->d_off(), (src->n_rows + 1) * sizeof(uint64_t),
                                 cudaMemcpyDeviceToDevice, s));
    if (src->nnz) {
        SPG_CUDA_TRY(cudaMemcpyAsync(cb.ptr, src->d_cols(), src->nnz * sizeof(uint32_t), cudaMemcpyDeviceToDevice, s));
        SPG_CUDA_TRY(cudaMemcpyAsync(vb.ptr, src->d_vals(), src->nnz * sizeof(double), cudaMemcpyDeviceToDevice, s));
    }
    SPG_CUDA_TRY(cudaStreamSynchronize(s));
    dst->off = std::move(off);
    dst->cols = std::move(cb);
    dst->vals = std::move(vb);
    dst->capacity = src->nnz;
    return SPG_OK;
}

int spg_csr_get(spg_ctx *c, const spg_csr *A, uint64_t row, uint32_t col, double *value, int *found) {
    if (!c || !A || !value || !found) return set_error(SPG_ERR_INVALID_ARGUMENT, "spg_csr_get: null argument");
    if (row >= A->n_rows) return set_error(SPG_ERR_OUT_OF_RANGE, "spira::matrix: row_index out of range");
    if ((uint64_t)col >= A->n_cols) return set_error(SPG_ERR_OUT_OF_RANGE, "spira::matrix: col_index out of range");
    if (!A->built) {
        *value = 0.0;
        *found = 0;
        return SPG_OK;
    }
    SPG_CUDA_TRY(cudaSetDevice(c->device));
    cudaStream_t s = c->stream;
    DevBuf out;
    SPG_TRY(out.alloc(16, s));
    csr_get_kernel<<<1, 1, 0, s>>>(A->d_off(), A->d_cols(), A->d_vals(), row, col, out.as<double>(),
                                   reinterpret_cast<int *>(out.as<char>() + 8));
    SPG_LAUNCH_CHECK();
    char h[16];
    SPG_CUDA_TRY(cudaMemcpyAsync(h, out.ptr, 16, cudaMemcpyDeviceToHost, s));
    SPG_CUDA_TRY(cudaStreamSynchronize(s));
    memcpy(value, h, 8);
    memcpy(found, h + 8, 4);
    return SPG_OK;
}

int spg_csr_row_range(spg_ctx *c, const spg_csr *A, uint64_t row, uint64_t *begin, uint64_t *end) {
    if (!c || !A || !begin || !end) return set_error(SPG_ERR_INVALID_ARGUMENT, "spg_csr_row_range: null argument");
    if (row >= A->n_rows) return set_error(SPG_ERR_OUT_OF_RANGE, "spira::matrix: row_index out of range");
    if (!A->built) {
        *begin = *end = 0;
        return SPG_OK;
    }
    SPG_CUDA_TRY(cudaSetDevice(c->device));
    uint64_t h[2];
    SPG_CUDA_TRY(cudaMemcpyAsync(h, A->d_off() + row, 2 * sizeof(uint64_t), cudaMemcpyDeviceToHost, c->stream));
    SPG_CUDA_TRY(cudaStreamSynchronize(c->stream));
    *begin = h[0];
    *end = h[1];
    return SPG_OK;
}

int spg_spmv(spg_ctx *c, const spg_csr *Ac, const double *d_x, double *d_y, int variant, void *stream) {
    if (!c || !Ac) return set_error(SPG_ERR_INVALID_ARGUMENT, "spg_spmv: null handle");
    SPG_CHECK_LIVE(Ac);
    spg_csr *A = const_cast<spg_csr *>(Ac);  // plans are cached on the handle
    if (!A->built) return set_error(SPG_ERR_LOGIC, "spmv: matrix must be locked");
    if ((A->n_cols && !d_x) || (A->n_rows && !d_y))
        return set_error(SPG_ERR_INVALID_ARGUMENT, "spg_spmv: null vector");
    if (variant < SPG_SPMV_AUTO || variant >= SPG_SPMV_N_VARIANTS)
        return set_error(SPG_ERR_INVALID_ARGUMENT, "spg_spmv: unknown variant %d", variant);
    SPG_CUDA_TRY(cudaSetDevice(c->device));
    if (variant == SPG_SPMV_AUTO) SPG_TRY(spmv_resolve_auto(c, A, &variant));
    return spmv_launch(c, A, d_x, d_y, variant, pick_stream(c, stream));
}

// Host-buffer SpMV; `async` (pinned x and y only) enqueues everything on
// `ls` and returns without waiting.
static int spmv_host_impl(spg_ctx *c, const spg_csr *Ac, const double *x, uint64_t x_len, double *y, uint64_t y_len,
                          int variant, bool async, void *user_stream) {
    const char *who = async ? "spg_spmv_host_async" : "spg_spmv_host";
    if (!c || !Ac) return set_error(SPG_ERR_INVALID_ARGUMENT, "%s: null handle", who);
    SPG_CHECK_LIVE(Ac);
    // Checks in the order of serial/spmv.hpp:150-158.
    if (x_len != Ac->n_cols)
        return set_error(SPG_ERR_INVALID_ARGUMENT,
                         "The size of the input vector x does not match the number of columns of the matrix");
    if (y_len != Ac->n_rows)
        return set_error(SPG_ERR_INVALID_ARGUMENT,
                         "The size of the output vector y does not match the number of rows of the matrix");
    if (!Ac->built) return set_error(SPG_ERR_LOGIC, "spmv: matrix must be locked");
    if ((x_len && !x) || (y_len && !y)) return set_error(SPG_ERR_INVALID_ARGUMENT, "%s: null vector", who);
    spg_csr *A = const_cast<spg_csr *>(Ac);
    SPG_CUDA_TRY(cudaSetDevice(c->device));
    cudaStream_t s = c->stream;
    const bool pinned = host_pinned(x) && host_pinned(y);
    if (async && !pinned)
        return set_error(SPG_ERR_INVALID_ARGUMENT, "spg_spmv_host_async: x and y must be pinned host memory");
    const cudaStream_t ls = async ? pick_stream(c, user_stream) : s;  // where the SpMV is enqueued
    if (variant == SPG_SPMV_AUTO) SPG_TRY(spmv_resolve_auto(c, A, &variant));
    if (variant < 0 || variant >= SPG_SPMV_N_VARIANTS)
        return set_error(SPG_ERR_INVALID_ARGUMENT, "%s: unknown variant %d", who, variant);
    SPG_TRY(spmv_prepare(c, A, variant, s));  // plans synchronise: not inside the recorded graph
    // pinned buffers stage through the matrix's own device vectors (recorded
    // graphs stay valid across calls, matrices can overlap); pageable ones
    // through the context's
    DevBuf &bx = pinned ? A->stage_x : c->xbuf, &by = pinned ? A->stage_y : c->ybuf;
    if (bx.bytes < x_len * sizeof(double)) SPG_TRY(bx.alloc(x_len * sizeof(double), s));
    if (by.bytes < y_len * sizeof(double)) SPG_TRY(by.alloc(y_len * sizeof(double), s));
    if (ls != s) {  // the buffers were (re)allocated in s's order
        cudaEvent_t ready = c->host_events[Ctx::N_HOST_EVENTS - 3];
        SPG_CUDA_TRY(cudaEventRecord(ready, s));
        SPG_CUDA_TRY(cudaStreamWaitEvent(ls, ready, 0));
    }
    const double *dx = bx.as<double>();
    double *dy = by.as<double>();
    // Large matrices: compute y in row blocks and copy each block back on a
    // second stream while the next block computes (the host link, ~200 GB/s,
    // otherwise idles during the SpMV).
    constexpr uint64_t PIPELINE_MIN_NNZ = 4u << 20;
    constexpr int NB = 4;  // the last block's copy and the one-block fix-up look-ahead stay exposed;
                           // 2 and 8 blocks measured slower (per-block launch and tail costs)
    static_assert(NB + 1 <= Ctx::N_HOST_EVENTS - 3, "a stage event per block, plus fork, join and ready");
    const bool row_parallel = variant == SPG_SPMV_SCALAR || (variant >= SPG_SPMV_VECTOR2 && variant <= SPG_SPMV_VECTOR32);
    const bool adaptive = spmv_is_seg(variant);
    std::vector<uint64_t> rows;
    if (A->nnz >= PIPELINE_MIN_NNZ && y_len && (row_parallel || adaptive)) {
        if (row_parallel) {
            rows.resize(NB + 1);
            for (int b = 0; b <= NB; ++b) rows[b] = y_len * (uint64_t)b / NB;
        } else {
            SPG_TRY(spmv_adaptive_blocks(c, A, variant, NB, &rows, s));
        }
    }
    const int nb = rows.empty() ? 0 : (int)rows.size() - 1;
    if (nb < 2) {
        if (x_len)
            SPG_CUDA_TRY(cudaMemcpyAsync(const_cast<double *>(dx), x, x_len * sizeof(double), cudaMemcpyHostToDevice,
                                         ls));
        SPG_TRY(spmv_launch(c, A, dx, dy, variant, ls));
        if (y_len) SPG_CUDA_TRY(cudaMemcpyAsync(y, dy, y_len * sizeof(double), cudaMemcpyDeviceToHost, ls));
        if (async) return SPG_OK;
        SPG_CUDA_TRY(cudaStreamSynchronize(s));
        return c->take_status();
    }
    // Row-parallel variants: x also goes up in nb column pieces on a third
    // stream, and a row block starts once the pieces up to the largest column
    // it reads have arrived (banded and stencil matrices overlap all three:
    // upload, compute, download). Other variants read x anywhere: whole upload.
    const uint64_t xc = (x_len + nb - 1) / (uint64_t)nb;  // columns per piece
    if (row_parallel && x_len) SPG_TRY(spmv_row_block_reach(c, A, nb, s));
    cudaEvent_t fork = c->host_events[Ctx::N_HOST_EVENTS - 1], copy_join = c->host_events[Ctx::N_HOST_EVENTS - 2];
    cudaEvent_t upload_join = c->upload_events[Ctx::N_HOST_EVENTS - 1];
    // everything on s, with the side streams forked from and joined back to it
    auto enqueue = [&]() -> int {
        SPG_CUDA_TRY(cudaEventRecord(fork, s));  // the staging buffers are ordered on s
        SPG_CUDA_TRY(cudaStreamWaitEvent(c->copy_stream, fork, 0));
        SPG_CUDA_TRY(cudaStreamWaitEvent(c->upload_stream, fork, 0));
        if (row_parallel && x_len) {
            for (int j = 0; j < nb; ++j) {
                const uint64_t c0 = std::min(x_len, xc * j), c1 = std::min(x_len, xc * (j + 1));
                if (c1 > c0)
                    SPG_CUDA_TRY(cudaMemcpyAsync(const_cast<double *>(dx) + c0, x + c0, (c1 - c0) * sizeof(double),
                                                 cudaMemcpyHostToDevice, c->upload_stream));
                SPG_CUDA_TRY(cudaEventRecord(c->upload_events[j], c->upload_stream));
            }
        } else if (x_len) {
            SPG_CUDA_TRY(cudaMemcpyAsync(const_cast<double *>(dx), x, x_len * sizeof(double), cudaMemcpyHostToDevice,
                                         s));
        }
        // stage i makes rows [rows[i-1], rows[i]) final (row-parallel: stage i
        // computes block i, so its rows are [rows[i], rows[i+1]))
        const int stages = row_parallel ? nb : nb + 1;
        for (int i = 0; i < stages; ++i) {
            uint64_t r0, r1;
            if (row_parallel) {
                r0 = rows[i];
                r1 = rows[i + 1];
                if (x_len) {
                    const int64_t reach = A->host_reach[i];
                    const int piece = reach < 0 ? 0 : (int)std::min<uint64_t>(nb - 1, (uint64_t)reach / xc);
                    SPG_CUDA_TRY(cudaStreamWaitEvent(s, c->upload_events[piece], 0));
                }
                SPG_TRY(spmv_launch_rows(c, A, dx, dy, variant, r0, r1, s));
            } else {
                SPG_TRY(spmv_adaptive_stage(c, A, dx, dy, variant, i, s));
                if (i == 0) continue;
                r0 = rows[i - 1];
                r1 = rows[i];
            }
            if (r1 <= r0) continue;
            cudaEvent_t ev = c->host_events[i];
            SPG_CUDA_TRY(cudaEventRecord(ev, s));
            SPG_CUDA_TRY(cudaStreamWaitEvent(c->copy_stream, ev, 0));
            SPG_CUDA_TRY(cudaMemcpyAsync(y + r0, dy + r0, (r1 - r0) * sizeof(double), cudaMemcpyDeviceToHost,
                                         c->copy_stream));
        }
        SPG_CUDA_TRY(cudaEventRecord(copy_join, c->copy_stream));
        SPG_CUDA_TRY(cudaEventRecord(upload_join, c->upload_stream));
        SPG_CUDA_TRY(cudaStreamWaitEvent(s, copy_join, 0));
        SPG_CUDA_TRY(cudaStreamWaitEvent(s, upload_join, 0));
        return SPG_OK;
    };
    // With pinned x and y the whole sequence is recorded once as a CUDA graph
    // and replayed while the same buffers come back: one launch instead of a
    // few dozen API calls, whose host time otherwise exceeds the transfers of
    // a matrix this size.
    if (pinned) {
        if (!(A->host_graph && A->host_gx == x && A->host_gy == y && A->host_gvariant == variant &&
              A->host_gdx == dx && A->host_gdy == dy)) {
            A->drop_host_graph();
            cudaGraph_t g = nullptr;
            SPG_CUDA_TRY(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
            const int rc = enqueue();
            cudaError_t ec = cudaStreamEndCapture(s, &g);
            cudaGraphExec_t ex = nullptr;
            if (rc == SPG_OK && ec == cudaSuccess) ec = cudaGraphInstantiate(&ex, g, 0);
            if (g) cudaGraphDestroy(g);
            if (rc == SPG_OK && ec == cudaSuccess) {
                A->host_graph = ex;
                A->host_gx = x;
                A->host_gy = y;
                A->host_gdx = dx;
                A->host_gdy = dy;
                A->host_gvariant = variant;
            } else {
                cudaGetLastError();  // not recordable: run the sequence directly below
            }
        }
        if (A->host_graph) {
            SPG_CUDA_TRY(cudaGraphLaunch(A->host_graph, ls));
            if (async) return SPG_OK;
            SPG_CUDA_TRY(cudaStreamSynchronize(s));
            return c->take_status();
        }
    }
    // not recorded: the sequence runs on the context's stream (an
    // asynchronous call then waits for it here)
    if (ls != s) {
        cudaEvent_t before = c->host_events[Ctx::N_HOST_EVENTS - 3];
        SPG_CUDA_TRY(cudaEventRecord(before, ls));
        SPG_CUDA_TRY(cudaStreamWaitEvent(s, before, 0));
    }
    SPG_TRY(enqueue());
    SPG_CUDA_TRY(cudaStreamSynchronize(s));
    return c->take_status();
}

// Several matrices' host-buffer SpMVs as one recorded graph. Each matrix
// gets a lane (compute, upload and download streams). The uploads are
// chained in priority order — matrices whose SpMV reads x anywhere (so waits
// for all of it), largest x first, then the row-parallel ones, whose blocks
// start on the first pieces of theirs — so the first matrix's x is not slowed
// by the others sharing the host link, and the other matrices' transfers and
// kernels proceed while it computes.
struct MultiPlan {
    spg_csr *A;
    const double *x;
    double *y;
    const double *dx;
    double *dy;
    int variant;
    bool row_parallel;
    std::vector<uint64_t> rows;  // row blocks (nb + 1 bounds), empty: one block
    uint64_t xc;                 // columns per x piece (row-parallel)
};

static int multi_lane_resources(Ctx *c, int n) {
    for (int l = 0; l < n; ++l) {
        for (cudaStream_t &st : c->multi_stream[l])
            if (!st) SPG_CUDA_TRY(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
        for (cudaEvent_t &ev : c->multi_event[l])
            if (!ev) SPG_CUDA_TRY(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    }
    return SPG_OK;
}

static int multi_enqueue(Ctx *c, std::vector<MultiPlan> &P, const std::vector<int> &order, cudaStream_t s) {
    constexpr int NE = Ctx::N_HOST_EVENTS;
    cudaEvent_t fork = c->host_events[NE - 1];
    SPG_CUDA_TRY(cudaEventRecord(fork, s));
    cudaEvent_t gate = nullptr;  // the previous lane's last upload
    for (int l = 0; l < (int)order.size(); ++l) {
        MultiPlan &p = P[order[l]];
        cudaStream_t comp = c->multi_stream[l][0], up = c->multi_stream[l][1], copy = c->multi_stream[l][2];
        cudaEvent_t *ev = c->multi_event[l];  // [0, NE): block done; [NE, 2 NE): x piece up
        const uint64_t x_len = p.A->n_cols, y_len = p.A->n_rows;
        for (cudaStream_t st : {comp, up, copy}) SPG_CUDA_TRY(cudaStreamWaitEvent(st, fork, 0));
        if (gate) SPG_CUDA_TRY(cudaStreamWaitEvent(up, gate, 0));
        const int nb = p.rows.empty() ? 1 : (int)p.rows.size() - 1;
        const int pieces = p.row_parallel && nb > 1 ? nb : 1;
        for (int j = 0; j < pieces; ++j) {
            const uint64_t c0 = pieces == 1 ? 0 : std::min(x_len, p.xc * j);
            const uint64_t c1 = pieces == 1 ? x_len : std::min(x_len, p.xc * (j + 1));
            if (c1 > c0)
                SPG_CUDA_TRY(cudaMemcpyAsync(const_cast<double *>(p.dx) + c0, p.x + c0, (c1 - c0) * sizeof(double),
                                             cudaMemcpyHostToDevice, up));
            SPG_CUDA_TRY(cudaEventRecord(ev[NE + j], up));
        }
        gate = ev[NE + pieces - 1];
        if (p.rows.empty()) {  // one block: whole x, one launch, whole y
            SPG_CUDA_TRY(cudaStreamWaitEvent(comp, gate, 0));
            SPG_TRY(spmv_launch(c, p.A, p.dx, p.dy, p.variant, comp));
            SPG_CUDA_TRY(cudaEventRecord(ev[0], comp));
            SPG_CUDA_TRY(cudaStreamWaitEvent(copy, ev[0], 0));
            if (y_len) SPG_CUDA_TRY(cudaMemcpyAsync(p.y, p.dy, y_len * sizeof(double), cudaMemcpyDeviceToHost, copy));
        } else {
            const int stages = p.row_parallel ? nb : nb + 1;
            if (!p.row_parallel) SPG_CUDA_TRY(cudaStreamWaitEvent(comp, gate, 0));
            for (int i = 0; i < stages; ++i) {
                uint64_t r0, r1;
                if (p.row_parallel) {
                    r0 = p.rows[i];
                    r1 = p.rows[i + 1];
                    if (x_len) {
                        const int64_t reach = p.A->host_reach[i];
                        const int piece = reach < 0 ? 0 : (int)std::min<uint64_t>(nb - 1, (uint64_t)reach / p.xc);
                        SPG_CUDA_TRY(cudaStreamWaitEvent(comp, ev[NE + piece], 0));
                    }
                    SPG_TRY(spmv_launch_rows(c, p.A, p.dx, p.dy, p.variant, r0, r1, comp));
                } else {
                    SPG_TRY(spmv_adaptive_stage(c, p.A, p.dx, p.dy, p.variant, i, comp));
                    if (i == 0) continue;
                    r0 = p.rows[i - 1];
                    r1 = p.rows[i];
                }
                if (r1 <= r0) continue;
                SPG_CUDA_TRY(cudaEventRecord(ev[i], comp));
                SPG_CUDA_TRY(cudaStreamWaitEvent(copy, ev[i], 0));
                SPG_CUDA_TRY(cudaMemcpyAsync(p.y + r0, p.dy + r0, (r1 - r0) * sizeof(double), cudaMemcpyDeviceToHost,
                                             copy));
            }
        }
        // join the lane back to s
        for (cudaStream_t st : {comp, up, copy}) {
            SPG_CUDA_TRY(cudaEventRecord(ev[NE - 1], st));
            SPG_CUDA_TRY(cudaStreamWaitEvent(s, ev[NE - 1], 0));
        }
    }
    return SPG_OK;
}

int spg_spmv_host_multi(spg_ctx *c, uint32_t n, const spg_csr *const *mats, const double *const *xs,
                        double *const *ys, const int *variants, void *stream) {
    if (!c || (n && (!mats || !xs || !ys))) return set_error(SPG_ERR_INVALID_ARGUMENT, "spg_spmv_host_multi: null argument");
    if (n > (uint32_t)Ctx::MULTI_MAX)
        return set_error(SPG_ERR_INVALID_ARGUMENT, "spg_spmv_host_multi: at most %d matrices", Ctx::MULTI_MAX);
    if (!n) return SPG_OK;
    SPG_CUDA_TRY(cudaSetDevice(c->device));
    cudaStream_t s = c->stream;
    std::vector<MultiPlan> P(n);
    for (uint32_t i = 0; i < n; ++i) {
        spg_csr *A = const_cast<spg_csr *>(mats[i]);
        if (!A) return set_error(SPG_ERR_INVALID_ARGUMENT, "spg_spmv_host_multi: null matrix %u", i);
        SPG_CHECK_LIVE(A);
        if (!A->built) return set_error(SPG_ERR_LOGIC, "spmv: matrix must be locked");
        for (uint32_t j = 0; j < i; ++j)
            if (mats[j] == mats[i]) return set_error(SPG_ERR_INVALID_ARGUMENT, "spg_spmv_host_multi: matrix %u repeated", i);
        if ((A->n_cols && !xs[i]) || (A->n_rows && !ys[i]) || !host_pinned(xs[i]) || !host_pinned(ys[i]))
            return set_error(SPG_ERR_INVALID_ARGUMENT, "spg_spmv_host_multi: x and y must be pinned host memory");
        int v = variants ? variants[i] : SPG_SPMV_AUTO;
        if (v == SPG_SPMV_AUTO) SPG_TRY(spmv_resolve_auto(c, A, &v));
        if (v < 0 || v >= SPG_SPMV_N_VARIANTS)
            return set_error(SPG_ERR_INVALID_ARGUMENT, "spg_spmv_host_multi: unknown variant %d", v);
        SPG_TRY(spmv_prepare(c, A, v, s));  // before the graph is recorded
        if (A->stage_x.bytes < A->n_cols * sizeof(double)) SPG_TRY(A->stage_x.alloc(A->n_cols * sizeof(double), s));
        if (A->stage_y.bytes < A->n_rows * sizeof(double)) SPG_TRY(A->stage_y.alloc(A->n_rows * sizeof(double), s));
        MultiPlan &p = P[i];
        p.A = A;
        p.x = xs[i];
        p.y = ys[i];
        p.dx = A->stage_x.as<double>();
        p.dy = A->stage_y.as<double>();
        p.variant = v;
        p.row_parallel = v == SPG_SPMV_SCALAR || (v >= SPG_SPMV_VECTOR2 && v <= SPG_SPMV_VECTOR32);
        const bool adaptive = spmv_is_seg(v);
        constexpr uint64_t PIPELINE_MIN_NNZ = 4u << 20;
        constexpr int NB = 4;
        static_assert(NB + 1 <= Ctx::N_HOST_EVENTS - 1, "a stage event per block, plus the join event");
        if (A->nnz >= PIPELINE_MIN_NNZ && A->n_rows && (p.row_parallel || adaptive)) {
            if (p.row_parallel) {
                p.rows.resize(NB + 1);
                for (int b = 0; b <= NB; ++b) p.rows[b] = A->n_rows * (uint64_t)b / NB;
            } else {
                SPG_TRY(spmv_adaptive_blocks(c, A, v, NB, &p.rows, s));
            }
            if (p.rows.size() < 3) p.rows.clear();
        }
        const int nb = p.rows.empty() ? 1 : (int)p.rows.size() - 1;
        p.xc = (A->n_cols + nb - 1) / (uint64_t)nb;
        if (p.row_parallel && nb > 1 && A->n_cols) SPG_TRY(spmv_row_block_reach(c, A, nb, s));
    }
    // priority: matrices that wait for all of x (largest x first), then the row-parallel ones
    std::vector<int> order(n);
    for (uint32_t i = 0; i < n; ++i) order[i] = (int)i;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
        const bool wa = !(P[a].row_parallel && !P[a].rows.empty()), wb = !(P[b].row_parallel && !P[b].rows.empty());
        if (wa != wb) return wa;
        return P[a].A->n_cols > P[b].A->n_cols;
    });
    std::vector<uintptr_t> key;
    for (int i : order) {
        const MultiPlan &p = P[i];
        for (uintptr_t k : {(uintptr_t)p.A, (uintptr_t)p.A->epoch, (uintptr_t)p.x, (uintptr_t)p.y,
                            (uintptr_t)p.dx, (uintptr_t)p.dy, (uintptr_t)p.variant})
            key.push_back(k);
    }
    if (!(c->multi_graph && c->multi_key == key)) {
        c->drop_multi();
        SPG_TRY(multi_lane_resources(c, (int)n));
        cudaGraph_t g = nullptr;
        SPG_CUDA_TRY(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
        const int rc = multi_enqueue(c, P, order, s);
        cudaError_t ec = cudaStreamEndCapture(s, &g);
        cudaGraphExec_t ex = nullptr;
        if (rc == SPG_OK && ec == cudaSuccess) ec = cudaGraphInstantiate(&ex, g, 0);
        if (g) cudaGraphDestroy(g);
        if (rc != SPG_OK) return rc;
        if (ec != cudaSuccess) return set_error(SPG_ERR_CUDA, "spg_spmv_host_multi: graph: %s", cudaGetErrorString(ec));
        c->multi_graph = ex;
        c->multi_key = key;
    }
    const cudaStream_t ls = pick_stream(c, stream);
    if (ls != s) {  // staging was (re)allocated in s's order
        cudaEvent_t ready = c->host_events[Ctx::N_HOST_EVENTS - 3];
        SPG_CUDA_TRY(cudaEventRecord(ready, s));
        SPG_CUDA_TRY(cudaStreamWaitEvent(ls, ready, 0));
    }
    SPG_CUDA_TRY(cudaGraphLaunch(c->multi_graph, ls));
    return SPG_OK;
}

int spg_spmv_host(spg_ctx *c, const spg_csr *Ac, const double *x, uint64_t x_len, double *y, uint64_t y_len,
                  int variant) {
    return spmv_host_impl(c, Ac, x, x_len, y, y_len, variant, false, nullptr);
}

int spg_spmv_host_async(spg_ctx *c, const spg_csr *Ac, const double *x, uint64_t x_len, double *y, uint64_t y_len,
                        int variant, void *stream) {
    return spmv_host_impl(c, Ac, x, x_len, y, y_len, variant, true, stream);
}

int spg_spmv_launches(spg_ctx *c, const spg_csr *Ac, int variant, int *n) {
    if (!c || !Ac || !n) return set_error(SPG_ERR_INVALID_ARGUMENT, "spg_spmv_launches: null argument");
    if (!Ac->built) return set_error(SPG_ERR_LOGIC, "spmv: matrix must be locked");
    SPG_CUDA_TRY(cudaSetDevice(c->device));
    spg_csr *A = const_cast<spg_csr *>(Ac);
    if (variant == SPG_SPMV_AUTO) SPG_TRY(spmv_resolve_auto(c, A, &variant));
    if (variant < 0 || variant >= SPG_SPMV_N_VARIANTS)
        return set_error(SPG_ERR_INVALID_ARGUMENT, "spg_spmv_launches: unknown variant %d", variant);
    if (A->n_rows == 0) {
        *n = 0;
        return SPG_OK;
    }
    switch (variant) {
        case SPG_SPMV_MERGE:
            *n = 2;
            break;
        case SPG_SPMV_STREAM:
            *n = 1;
            break;
        default:
            if (spmv_is_seg(variant)) {
                SPG_TRY(build_adaptive_plan(c, A, variant, c->stream));
                const SpmvPlan &P = adaptive_plan_of(A, variant);
                *n = (P.n_items ? 2 : 0) + (P.count1 ? 1 : 0);
            } else {
                *n = 1;
            }
    }
    return SPG_OK;
}

int spg_spmv_selected(spg_ctx *c, const spg_csr *Ac, int *variant) {
    if (!c || !Ac || !variant) return set_error(SPG_ERR_INVALID_ARGUMENT, "spg_spmv_selected: null argument");
    if (!Ac->built) return set_error(SPG_ERR_LOGIC, "spmv: matrix must be locked");
    SPG_CUDA_TRY(cudaSetDevice(c->device));
    return spmv_resolve_auto(c, const_cast<spg_csr *>(Ac), variant);
}

}  // extern "C"
