// spg_transpose.cu — A^T as a stable counting sort by column.
//
// Spira (serial/transpose.hpp:35-156) histograms the column indices, prefix-
// sums them into the output offsets and scatters row by row through per-
// column cursors, so every output row lists its source rows in ascending
// order; the result is installed with load_csr (capacity == nnz).
//
// Here the same histogram (device atomics) and prefix sum give the output
// offsets; the scatter runs in parallel through atomic per-column cursors, so
// inside an output row the source rows arrive in any order, and each output
// row is then put in source-row order: rows of up to 32 entries by a sorting
// network (in one thread's registers, or across a warp's lanes), and when
// any row is longer, all rows by the row-grouped on-chip sort
// (sort_grouped_rows). Source rows are distinct within a column, so the result is
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

// Thread per source row: entry (w, c) goes to toff[c] + (a cursor of column
// c). A row's entries are handled SB at a time with their loads and cursor
// atomics all issued before any result is used (the atomics' round trips
// overlap instead of queueing one after another).
constexpr int SB = 8;

// The sorting-network path runs before the host has seen the longest output
// row: its kernels take the device-side longest row and do nothing when it
// is above 32 (the grouped-sort path then runs instead).
constexpr unsigned long long NET_MAX = 32;

template <bool WRITE_ROW>
__global__ void tr_scatter(const uint64_t *__restrict__ off, const uint32_t *__restrict__ cols,
                           const double *__restrict__ vals, uint64_t m, const uint64_t *__restrict__ toff,
                           unsigned *__restrict__ cursor, uint32_t *__restrict__ trow, uint32_t *__restrict__ tsrc,
                           double *__restrict__ tval, const unsigned long long *__restrict__ longest) {
    const uint64_t w = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (w >= m) return;
    if (longest && *longest > NET_MAX) return;
    const uint64_t e = off[w + 1];
    for (uint64_t k = off[w]; k < e; k += SB) {
        uint32_t col[SB];
        double v[SB];
        uint64_t base[SB];
        unsigned slot[SB];
#pragma unroll
        for (int j = 0; j < SB; ++j) {
            col[j] = k + j < e ? cols[k + j] : 0u;
            v[j] = k + j < e ? vals[k + j] : 0.0;
        }
#pragma unroll
        for (int j = 0; j < SB; ++j)
            if (k + j < e) {
                slot[j] = atomicAdd(cursor + col[j], 1u);
                base[j] = toff[col[j]];
            }
#pragma unroll
        for (int j = 0; j < SB; ++j)
            if (k + j < e) {
                const uint64_t p = base[j] + slot[j];
                if (WRITE_ROW) trow[p] = col[j];  // only the per-tile sort reads it
                tsrc[p] = (uint32_t)w;
                tval[p] = v[j];
            }
    }
}

// Longest output row (for the choice of sort), from the scanned offsets.
__global__ void tr_max_len(const uint64_t *__restrict__ toff, uint64_t n, unsigned long long *__restrict__ mx) {
    unsigned long long v = 0;
    for (uint64_t c = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; c < n; c += (uint64_t)gridDim.x * blockDim.x)
        v = max(v, (unsigned long long)(toff[c + 1] - toff[c]));
#pragma unroll
    for (int o = 16; o; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
    __shared__ unsigned long long s_v[TB / 32];
    if ((threadIdx.x & 31) == 0) s_v[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < TB / 32; ++w) v = max(v, s_v[w]);
        atomicMax(mx, v);
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

// Per output row, the scattered entries (source row, value) put in source-row
// order directly when the row is short: rows of at most 16 entries by one
// thread with a bitonic network in registers (source rows are distinct in a
// column, so the order is unique and the network's instability does not
// matter) and rows of 17..32 entries listed for tr_sort_mid. Used when no
// output row is longer than 32.
template <int N>
__device__ __forceinline__ void bitonic_regs(uint32_t (&k)[N], double (&v)[N]) {
#pragma unroll
    for (int size = 2; size <= N; size <<= 1)
#pragma unroll
        for (int stride = size >> 1; stride > 0; stride >>= 1)
#pragma unroll
            for (int i = 0; i < N; ++i) {
                const int j = i ^ stride;
                if (j > i) {
                    const bool up = (i & size) == 0;
                    if ((k[i] > k[j]) == up) {
                        const uint32_t tk = k[i];
                        k[i] = k[j];
                        k[j] = tk;
                        const double tv = v[i];
                        v[i] = v[j];
                        v[j] = tv;
                    }
                }
            }
}

template <int N>
__device__ __forceinline__ void sort_row_regs(const uint32_t *__restrict__ tsrc, const double *__restrict__ tval,
                                              uint64_t b, uint32_t L, uint32_t *__restrict__ out_cols,
                                              double *__restrict__ out_vals) {
    uint32_t k[N];
    double v[N];
#pragma unroll
    for (int i = 0; i < N; ++i) {
        k[i] = (uint32_t)i < L ? tsrc[b + i] : 0xFFFFFFFFu;
        v[i] = (uint32_t)i < L ? tval[b + i] : 0.0;
    }
    bitonic_regs<N>(k, v);
#pragma unroll
    for (int i = 0; i < N; ++i)
        if ((uint32_t)i < L) {
            out_cols[b + i] = k[i];
            out_vals[b + i] = v[i];
        }
}

__global__ void __launch_bounds__(TB)
tr_sort_short(const uint64_t *__restrict__ toff, uint64_t n, const uint32_t *__restrict__ tsrc,
              const double *__restrict__ tval, uint32_t *__restrict__ out_cols, double *__restrict__ out_vals,
              unsigned long long *__restrict__ n_mid, uint32_t *__restrict__ mid,
              const unsigned long long *__restrict__ longest) {
    if (*longest > NET_MAX) return;
    for (uint64_t c = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; c < n; c += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t b = toff[c];
        const uint64_t L = toff[c + 1] - b;
        if (L <= 1) {
            if (L == 1) {
                out_cols[b] = tsrc[b];
                out_vals[b] = tval[b];
            }
        } else if (L <= 8) {
            sort_row_regs<8>(tsrc, tval, b, (uint32_t)L, out_cols, out_vals);
        } else if (L <= 16) {
            sort_row_regs<16>(tsrc, tval, b, (uint32_t)L, out_cols, out_vals);
        } else {  // 17..32 (longer rows never reach this kernel)
            mid[atomicAdd(n_mid, 1ull)] = (uint32_t)c;
        }
    }
}

// Rows of 17..32 entries: a warp per row, one entry per lane, bitonic sort
// across the lanes by source row.
__global__ void __launch_bounds__(TB)
tr_sort_mid(const uint64_t *__restrict__ toff, const uint32_t *__restrict__ mid,
            const unsigned long long *__restrict__ n_mid, const uint32_t *__restrict__ tsrc,
            const double *__restrict__ tval, uint32_t *__restrict__ out_cols, double *__restrict__ out_vals,
            const unsigned long long *__restrict__ longest) {
    if (*longest > NET_MAX) return;
    const unsigned lane = threadIdx.x & 31;
    const uint64_t n_warps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    const uint64_t cnt = *n_mid;
    for (uint64_t w = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5; w < cnt; w += n_warps) {
        const uint32_t c = mid[w];
        const uint64_t b = toff[c], L = toff[c + 1] - b;
        uint32_t k = lane < L ? tsrc[b + lane] : 0xFFFFFFFFu;
        double v = lane < L ? tval[b + lane] : 0.0;
#pragma unroll
        for (unsigned size = 2; size <= 32; size <<= 1)
#pragma unroll
            for (unsigned stride = size >> 1; stride > 0; stride >>= 1) {
                const uint32_t pk = __shfl_xor_sync(0xffffffffu, k, stride);
                const double pv = __shfl_xor_sync(0xffffffffu, v, stride);
                const bool up = (lane & size) == 0, lower = (lane & stride) == 0;
                // the lower lane of an ascending pair keeps the smaller key
                const bool keep_small = lower == up;
                const bool take = keep_small ? (pk < k) : (pk > k);
                if (take) {
                    k = pk;
                    v = pv;
                }
            }
        if (lane < L) {
            out_cols[b + lane] = k;
            out_vals[b + lane] = v;
        }
    }
}

}  // namespace

// Histogram + atomic scatter + per-row sort: output rows of at most 32
// entries are sorted by tr_sort_short / tr_sort_mid; when some row is longer,
// the row-grouped on-chip sort orders all rows instead. *done = false if an
// output row is too long for that sort too (nothing is installed then).
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
        // the longest output row decides the sort: up to 32 entries, sorting
        // networks per row (and the scatter need not record output rows).
        // That path is enqueued at once, its kernels checking the longest row
        // on the device, so the common case costs no host round trip before
        // the final one; a longer row sends every row through the grouped
        // sort afterwards.
        DevBuf meta, midbuf;
        SPG_TRY(meta.alloc(16, s));  // [longest row (8 bytes)] [rows of 17..32 entries (8 bytes)]
        SPG_CUDA_TRY(cudaMemsetAsync(meta.ptr, 0, 16, s));
        unsigned long long *mx = meta.as<unsigned long long>(), *n_mid = mx + 1;
        tr_max_len<<<grid_for(n, TB, (unsigned)c->n_sms * 8), TB, 0, s>>>(out_off.as<uint64_t>(), n, mx);
        SPG_LAUNCH_CHECK();
        SPG_TRY(cursor.alloc((n ? n : 1) * sizeof(unsigned), s));
        SPG_CUDA_TRY(cudaMemsetAsync(cursor.ptr, 0, (n ? n : 1) * sizeof(unsigned), s));
        SPG_TRY(tsrc.alloc(nnz * sizeof(uint32_t), s));
        SPG_TRY(tval.alloc(nnz * sizeof(double), s));
        unsigned long long longest = NET_MAX + 1;
        if (m < 0xFFFFFFFFull) {  // source rows below the networks' padding key
            SPG_TRY(midbuf.alloc((n ? n : 1) * sizeof(uint32_t), s));
            tr_scatter<false><<<grid_for(m, TB), TB, 0, s>>>(A->d_off(), A->d_cols(), A->d_vals(), m,
                                                             out_off.as<uint64_t>(), cursor.as<unsigned>(), nullptr,
                                                             tsrc.as<uint32_t>(), tval.as<double>(), mx);
            tr_sort_short<<<grid_for(n, TB, gmax), TB, 0, s>>>(out_off.as<uint64_t>(), n, tsrc.as<uint32_t>(),
                                                               tval.as<double>(), out_cols.as<uint32_t>(),
                                                               out_vals.as<double>(), n_mid, midbuf.as<uint32_t>(),
                                                               mx);
            tr_sort_mid<<<(unsigned)c->n_sms * 8, TB, 0, s>>>(out_off.as<uint64_t>(), midbuf.as<uint32_t>(), n_mid,
                                                             tsrc.as<uint32_t>(), tval.as<double>(),
                                                             out_cols.as<uint32_t>(), out_vals.as<double>(), mx);
            SPG_LAUNCH_CHECK();
            SPG_CUDA_TRY(cudaMemcpyAsync(&longest, mx, 8, cudaMemcpyDeviceToHost, s));
            SPG_TRY(c->phase_sync(s));
        }
        if (longest > NET_MAX) {  // the networks' kernels did nothing; cursors are still zero
            SPG_TRY(trow.alloc(nnz * sizeof(uint32_t), s));
            tr_scatter<true><<<grid_for(m, TB), TB, 0, s>>>(A->d_off(), A->d_cols(), A->d_vals(), m,
                                                            out_off.as<uint64_t>(), cursor.as<unsigned>(),
                                                            trow.as<uint32_t>(), tsrc.as<uint32_t>(),
                                                            tval.as<double>(), nullptr);
            SPG_LAUNCH_CHECK();
            SPG_TRY(keys.alloc(nnz * sizeof(uint64_t), s));
            SPG_TRY(idx.alloc(nnz * sizeof(uint32_t), s));
            const int rbits = bits_for(m);
            SPG_TRY(sort_grouped_rows(c, trow.as<uint32_t>(), tsrc.as<uint32_t>(), out_off.as<uint64_t>(), nnz, n,
                                      rbits, keys.as<uint64_t>(), idx.as<uint32_t>(), done, s));
            if (!*done) return SPG_OK;
            tr_finish<<<grid_for(nnz, TB, gmax), TB, 0, s>>>(keys.as<uint64_t>(), idx.as<uint32_t>(), nnz, rbits,
                                                            tval.as<double>(), out_cols.as<uint32_t>(),
                                                            out_vals.as<double>());
            SPG_LAUNCH_CHECK();
        }
    }
    SPG_TRY(c->phase_sync(s));
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
    SPG_TRY(c->phase_sync(s));
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
