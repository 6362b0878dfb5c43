// spg_transpose.cu — A^T as a stable counting sort by column.
//
// Spira (serial/transpose.hpp:35-156) histograms the column indices, prefix-
// sums them into the output offsets and scatters row by row through per-
// column cursors, so every output row lists its source rows in ascending
// order; the result is installed with load_csr (capacity == nnz). Here the
// same permutation comes from a stable LSD radix sort of the column index with
// the entry index as payload: entries enter in row-major order, and stability
// keeps ascending source rows within each column. Offsets are lower_bound of
// each output row in the sorted column keys. Integer work and value copies
// only: bit-exact. HBM-bound: 12 B/nnz + 8 B/row read and written, plus the
// sort passes.
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

}  // namespace

int transpose_impl(Ctx *c, const Csr *A, Csr *T, cudaStream_t s) {
    const uint64_t nnz = A->nnz, m = A->n_rows, n = A->n_cols;
    if (nnz >= (1ull << 32))
        return set_error(SPG_ERR_UNSUPPORTED, "transpose: nnz %llu exceeds 2^32-1", (unsigned long long)nnz);
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
