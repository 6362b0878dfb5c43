// spg_transpose.cu — A^T as a stable counting sort by column.
//
// Spira (serial/transpose.hpp:35-156) histograms the column indices, prefix-
// sums them into the output offsets and scatters row by row through per-
// column cursors, so every output row lists its source rows in ascending
// order; the result is installed with load_csr (capacity == nnz).
//
// Here the same histogram (device atomics) and prefix sum give the output
// offsets; the scatter runs in parallel through atomic per-column cursors, so
// inside an output row the source rows arrive in any order, and the row-
// grouped on-chip sort (sort_grouped_rows) then orders every output row by
// source row. Source rows are distinct within a column, so the result is
// unique: Spira's. An output row too long for the on-chip sort (more than
// ~10 000 entries in one column) falls back to a stable LSD radix sort of the
// column index with the entry index as payload (entries enter in row-major
// order, stability keeps ascending source rows). Integer work and value
// copies only: bit-exact.
#include "spg_internal.cuh"

namespace spg {
namespace {

constexpr int TB = 256;

// key[k] = column of entry k; idx[k] = k; rowid[k] = source row (warp per row).
__global__ void tr_expand(const uint64_t *__restrict__ off, const uint32_t *__restrict__ cols, uint64_t n_rows,
                          uint64_t *__restrict__ key, uint32_t *__restrict__ idx, uint32_t *__restrict__ rowid) {
    const uint64_t w = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (w >= n_rows) return;
    const uint64_t b = off[w], e = off[w + 1];
    for (uint64_t k = b + lane; k < e; k += 32) {
        key[k] = cols[k];
        idx[k] = (uint32_t)k;
        rowid[k] = (uint32_t)w;
    }
}

__global__ void tr_gather(const uint64_t *__restrict__ key, const uint32_t *__restrict__ perm,
                          const uint32_t *__restrict__ rowid, const double *__restrict__ vals, uint64_t nnz,
                          uint32_t *__restrict__ out_cols, double *__restrict__ out_vals,
                          uint32_t *__restrict__ out_rowkey) {
    for (uint64_t p = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; p < nnz;
         p += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t k = perm[p];
        out_cols[p] = rowid[k];
        out_vals[p] = vals[k];
        out_rowkey[p] = (uint32_t)key[p];
    }
}

__global__ void tr_offsets(const uint32_t *__restrict__ srows, uint64_t u, uint64_t n_rows,
                           uint64_t *__restrict__ off) {
    for (uint64_t r = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; r <= n_rows;
         r += (uint64_t)gridDim.x * blockDim.x) {
        uint64_t lo = 0, hi = u;
        while (lo < hi) {
            const uint64_t mid = (lo + hi) >> 1;
            if ((uint64_t)srows[mid] < r) lo = mid + 1;
            else hi = mid;
        }
        off[r] = lo;
    }
}

__global__ void tr_count(const uint32_t *__restrict__ cols, uint64_t nnz, unsigned long long *__restrict__ cnt) {
    for (uint64_t k = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; k < nnz; k += (uint64_t)gridDim.x * blockDim.x)
        atomicAdd(cnt + cols[k], 1ull);
}

// Thread per source row: entry (w, c) goes to toff[c] + (a cursor of column c).
__global__ void tr_scatter(const uint64_t *__restrict__ off, const uint32_t *__restrict__ cols,
                           const double *__restrict__ vals, uint64_t m, const uint64_t *__restrict__ toff,
                           unsigned *__restrict__ cursor, uint32_t *__restrict__ trow, uint32_t *__restrict__ tsrc,
                           double *__restrict__ tval) {
    const uint64_t w = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (w >= m) return;
    for (uint64_t k = off[w]; k < off[w + 1]; ++k) {
        const uint32_t col = cols[k];
        const uint64_t p = toff[col] + atomicAdd(cursor + col, 1u);
        trow[p] = col;
        tsrc[p] = (uint32_t)w;
        tval[p] = vals[k];
    }
}

__global__ void tr_finish(const uint64_t *__restrict__ keys, const uint32_t *__restrict__ idx, uint64_t nnz,
                          int rbits, const double *__restrict__ tval, uint32_t *__restrict__ out_cols,
                          double *__restrict__ out_vals) {
    const uint64_t mask = rbits ? ((1ull << rbits) - 1) : 0;
    for (uint64_t p = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; p < nnz; p += (uint64_t)gridDim.x * blockDim.x) {
        out_cols[p] = (uint32_t)(keys[p] & mask);
        out_vals[p] = tval[idx[p]];
    }
}

}  // namespace

// Histogram + atomic scatter + on-chip per-row sort; *done = false if an
// output row is too long for the on-chip sort (nothing is installed then).
static int transpose_grouped(Ctx *c, const Csr *A, Csr *T, bool *done, cudaStream_t s) {
    const uint64_t nnz = A->nnz, m = A->n_rows, n = A->n_cols;
    const unsigned gmax = (unsigned)c->n_sms * 32;
    DevBuf out_off, out_cols, out_vals, cursor, trow, tsrc, tval, keys, idx;
    SPG_TRY(out_off.alloc(csr_off_elems(n) * sizeof(uint64_t), s));
    SPG_CUDA_TRY(cudaMemsetAsync(out_off.ptr, 0, csr_off_elems(n) * sizeof(uint64_t), s));
    SPG_TRY(out_cols.alloc(csr_alloc_elems(nnz) * sizeof(uint32_t), s));
    SPG_TRY(out_vals.alloc(csr_alloc_elems(nnz) * sizeof(double), s));
    *done = true;
    if (nnz) {
        tr_count<<<grid_for(nnz, TB, gmax), TB, 0, s>>>(A->d_cols(), nnz,
                                                       reinterpret_cast<unsigned long long *>(out_off.ptr));
        SPG_LAUNCH_CHECK();
        SPG_TRY(exclusive_scan_u64(c, out_off.as<uint64_t>(), n + 1, nullptr, s));
        SPG_TRY(cursor.alloc((n ? n : 1) * sizeof(unsigned), s));
        SPG_CUDA_TRY(cudaMemsetAsync(cursor.ptr, 0, (n ? n : 1) * sizeof(unsigned), s));
        SPG_TRY(trow.alloc(nnz * sizeof(uint32_t), s));
        SPG_TRY(tsrc.alloc(nnz * sizeof(uint32_t), s));
        SPG_TRY(tval.alloc(nnz * sizeof(double), s));
        tr_scatter<<<grid_for(m, TB), TB, 0, s>>>(A->d_off(), A->d_cols(), A->d_vals(), m,
                                                      out_off.as<uint64_t>(), cursor.as<unsigned>(),
                                                      trow.as<uint32_t>(), tsrc.as<uint32_t>(), tval.as<double>());
        SPG_LAUNCH_CHECK();
        SPG_TRY(keys.alloc(nnz * sizeof(uint64_t), s));
        SPG_TRY(idx.alloc(nnz * sizeof(uint32_t), s));
        const int rbits = bits_for(m);
        SPG_TRY(sort_grouped_rows(c, trow.as<uint32_t>(), tsrc.as<uint32_t>(), out_off.as<uint64_t>(), nnz, n, rbits,
                                  keys.as<uint64_t>(), idx.as<uint32_t>(), done, s));
        if (!*done) return SPG_OK;
        tr_finish<<<grid_for(nnz, TB, gmax), TB, 0, s>>>(keys.as<uint64_t>(), idx.as<uint32_t>(), nnz, rbits,
                                                        tval.as<double>(), out_cols.as<uint32_t>(),
                                                        out_vals.as<double>());
        SPG_LAUNCH_CHECK();
    }
    SPG_CUDA_TRY(cudaStreamSynchronize(s));
    T->invalidate_derived();
    T->n_rows = n;
    T->n_cols = m;
    T->off = std::move(out_off);
    T->cols = std::move(out_cols);
    T->vals = std::move(out_vals);
    T->nnz = nnz;
    T->capacity = nnz;
    T->built = true;
    T->may_have_zeros = A->may_have_zeros;
    return SPG_OK;
}

int transpose_impl(Ctx *c, const Csr *A, Csr *T, cudaStream_t s) {
    const uint64_t nnz = A->nnz, m = A->n_rows, n = A->n_cols;
    if (nnz >= (1ull << 32))
        return set_error(SPG_ERR_UNSUPPORTED, "transpose: nnz %llu exceeds 2^32-1", (unsigned long long)nnz);
    bool done = false;
    SPG_TRY(transpose_grouped(c, A, T, &done, s));
    if (done) return SPG_OK;
    DevBuf key, idx, rowid, out_off, out_cols, out_vals, rk;
    SPG_TRY(out_off.alloc(csr_off_elems(n) * sizeof(uint64_t), s));
    SPG_TRY(out_cols.alloc(csr_alloc_elems(nnz) * sizeof(uint32_t), s));
    SPG_TRY(out_vals.alloc(csr_alloc_elems(nnz) * sizeof(double), s));
    if (nnz) {
        SPG_TRY(key.alloc(nnz * sizeof(uint64_t), s));
        SPG_TRY(idx.alloc(nnz * sizeof(uint32_t), s));
        SPG_TRY(rowid.alloc(nnz * sizeof(uint32_t), s));
        SPG_TRY(rk.alloc(nnz * sizeof(uint32_t), s));
        tr_expand<<<grid_for(m * 32, TB), TB, 0, s>>>(A->d_off(), A->d_cols(), m, key.as<uint64_t>(),
                                                     idx.as<uint32_t>(), rowid.as<uint32_t>());
        SPG_LAUNCH_CHECK();
        SPG_TRY(radix_sort_pairs_u64(c, key.as<uint64_t>(), idx.as<uint32_t>(), nnz, bits_for(n), s));
        tr_gather<<<grid_for(nnz, TB, (unsigned)c->n_sms * 32), TB, 0, s>>>(
            key.as<uint64_t>(), idx.as<uint32_t>(), rowid.as<uint32_t>(), A->d_vals(), nnz, out_cols.as<uint32_t>(),
            out_vals.as<double>(), rk.as<uint32_t>());
        SPG_LAUNCH_CHECK();
    }
    tr_offsets<<<grid_for(n + 1, TB, (unsigned)c->n_sms * 32), TB, 0, s>>>(rk.as<uint32_t>(), nnz, n,
                                                                         out_off.as<uint64_t>());
    SPG_LAUNCH_CHECK();
    SPG_CUDA_TRY(cudaStreamSynchronize(s));
    T->invalidate_derived();
    T->n_rows = n;
    T->n_cols = m;
    T->off = std::move(out_off);
    T->cols = std::move(out_cols);
    T->vals = std::move(out_vals);
    T->nnz = nnz;
    T->capacity = nnz;
    T->built = true;
    T->may_have_zeros = A->may_have_zeros;
    return SPG_OK;
}

}  // namespace spg

using namespace spg;

extern "C" int spg_transpose(spg_ctx *c, const spg_csr *A, spg_csr *T) {
    if (!c || !A || !T) return set_error(SPG_ERR_INVALID_ARGUMENT, "spg_transpose: null handle");
    SPG_CHECK_LIVE(A);
    SPG_CHECK_LIVE(T);
    if (!A->built) return set_error(SPG_ERR_LOGIC, "transpose: matrix must be locked");
    if (A == T) return set_error(SPG_ERR_INVALID_ARGUMENT, "spg_transpose: output aliases input");
    SPG_CUDA_TRY(cudaSetDevice(c->device));
    return transpose_impl(c, A, T, c->stream);
}
