// spg_spgemm.cu — C = A * B with Spira's exact structure and FP64 values.
//
// Spira (serial/spgemm.hpp:12-53, parallel/algorithms/spgemm.hpp:27-69) is a
// row-wise Gustavson product: for row i, for each a_ik in A's row (ascending
// k), for each b_kj in B's row k: acc[j] += a_ik * b_kj; entries with
// acc != 0 are inserted into C, and C.lock() sorts them. So each C(i, j) is
// the left-to-right sum over ascending k of the rounded products, starting
// from 0.0, and exact-zero sums are dropped.
//
// GPU formulation (expand - sort - compress):
//   1. products per row of A, scanned into per-row product offsets;
//   2. expand every product (key = i << cbits | j, value = a_ik * b_kj
//      rounded) in (row, A-entry, B-entry) order;
//   3. stable radix sort of the keys with the product index as payload:
//      equal (i, j) keep ascending k;
//   4. sum each run left to right with separate round-to-nearest multiply and
//      add (__dmul_rn / __dadd_rn, never contracted), drop zero sums, compact.
// Values match Spira built without FMA contraction (its x86-64 build) bit for
// bit; structure is exact.
#include "spg_internal.cuh"

namespace spg {
namespace {

constexpr int GB = 256;

__global__ void sg_row_products(const uint64_t *__restrict__ aoff, const uint32_t *__restrict__ acols,
                                const uint64_t *__restrict__ boff, uint64_t m, uint64_t *__restrict__ cnt) {
    const uint64_t w = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (w > m) return;
    if (w == m) {
        if (lane == 0) cnt[m] = 0;
        return;
    }
    uint64_t s = 0;
    for (uint64_t ka = aoff[w] + lane; ka < aoff[w + 1]; ka += 32) {
        const uint32_t k = acols[ka];
        s += boff[k + 1] - boff[k];
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) cnt[w] = s;
}

__global__ void sg_expand(const uint64_t *__restrict__ aoff, const uint32_t *__restrict__ acols,
                          const double *__restrict__ avals, const uint64_t *__restrict__ boff,
                          const uint32_t *__restrict__ bcols, const double *__restrict__ bvals, uint64_t m,
                          int cbits, const uint64_t *__restrict__ pofs, uint64_t *__restrict__ key,
                          uint32_t *__restrict__ idx, double *__restrict__ pval) {
    const uint64_t w = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (w >= m) return;
    uint64_t base = pofs[w];
    const uint64_t rk = w << cbits;
    for (uint64_t ka = aoff[w]; ka < aoff[w + 1]; ++ka) {
        const uint32_t k = acols[ka];
        const double a = avals[ka];
        const uint64_t bb = boff[k], be = boff[k + 1];
        for (uint64_t kb = bb + lane; kb < be; kb += 32) {
            const uint64_t p = base + (kb - bb);
            key[p] = rk | bcols[kb];
            idx[p] = (uint32_t)p;
            pval[p] = __dmul_rn(a, bvals[kb]);
        }
        base += be - bb;
    }
}

__global__ void sg_run_flags(const uint64_t *__restrict__ key, uint64_t P, uint64_t *__restrict__ flag) {
    for (uint64_t p = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; p < P; p += (uint64_t)gridDim.x * blockDim.x)
        flag[p] = (p == 0 || key[p] != key[p - 1]) ? 1 : 0;
}

__global__ void sg_run_begins(const uint64_t *__restrict__ key, const uint64_t *__restrict__ rid, uint64_t P,
                              uint64_t U, uint64_t *__restrict__ begin) {
    for (uint64_t p = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; p < P; p += (uint64_t)gridDim.x * blockDim.x)
        if (p == 0 || key[p] != key[p - 1]) begin[rid[p]] = p;
    if (blockIdx.x == 0 && threadIdx.x == 0) begin[U] = P;
}

__global__ void sg_run_sums(const uint64_t *__restrict__ begin, const uint32_t *__restrict__ perm,
                            const double *__restrict__ pval, uint64_t U, double *__restrict__ sum,
                            uint64_t *__restrict__ keep) {
    for (uint64_t u = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; u < U; u += (uint64_t)gridDim.x * blockDim.x) {
        double acc = 0.0;  // ValueTraits zero; acc[j] default-constructs to V{}
        for (uint64_t q = begin[u]; q < begin[u + 1]; ++q) acc = __dadd_rn(acc, pval[perm[q]]);
        sum[u] = acc;
        keep[u] = (acc != 0.0) ? 1 : 0;  // spgemm.hpp:44: v != V{}
    }
}

__global__ void sg_write(const uint64_t *__restrict__ begin, const uint64_t *__restrict__ key,
                         const double *__restrict__ sum, const uint64_t *__restrict__ pos, uint64_t U, int cbits,
                         uint32_t *__restrict__ ccols, double *__restrict__ cvals, uint32_t *__restrict__ crow) {
    const uint64_t cmask = cbits ? ((1ull << cbits) - 1) : 0;
    for (uint64_t u = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; u < U; u += (uint64_t)gridDim.x * blockDim.x) {
        if (pos[u + 1] == pos[u]) continue;  // dropped
        const uint64_t kk = key[begin[u]];
        const uint64_t d = pos[u];
        ccols[d] = (uint32_t)(kk & cmask);
        cvals[d] = sum[u];
        crow[d] = (uint32_t)(kk >> cbits);
    }
}

__global__ void sg_offsets(const uint32_t *__restrict__ srows, uint64_t u, uint64_t n_rows,
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

uint64_t read_u64(const uint64_t *d, cudaStream_t s, int *rc) {
    uint64_t h = 0;
    cudaError_t e = cudaMemcpyAsync(&h, d, 8, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) *rc = set_error(SPG_ERR_CUDA, "spgemm: %s", cudaGetErrorString(e));
    return h;
}

}  // namespace

int spgemm_impl(Ctx *c, const Csr *A, const Csr *B, Csr *Cm, cudaStream_t s) {
    const uint64_t m = A->n_rows, n = B->n_cols;
    const int cbits = bits_for(n), rbits = bits_for(m);
    const unsigned gmax = (unsigned)c->n_sms * 32;
    int rc = SPG_OK;
    DevBuf pofs;
    SPG_TRY(pofs.alloc((m + 1) * sizeof(uint64_t), s));
    sg_row_products<<<grid_for((m + 1) * 32, GB), GB, 0, s>>>(A->d_off(), A->d_cols(), B->d_off(), m,
                                                             pofs.as<uint64_t>());
    SPG_LAUNCH_CHECK();
    SPG_TRY(exclusive_scan_u64(c, pofs.as<uint64_t>(), m + 1, nullptr, s));
    const uint64_t P = read_u64(pofs.as<uint64_t>() + m, s, &rc);
    SPG_TRY(rc);
    if (P >= (1ull << 32))
        return set_error(SPG_ERR_UNSUPPORTED, "spgemm: %llu products exceed 2^32-1", (unsigned long long)P);
    DevBuf key, idx, pval, flag, begin, sum, keep, out_off, out_cols, out_vals, crow;
    uint64_t U = 0, nnz = 0;
    if (P) {
        SPG_TRY(key.alloc(P * sizeof(uint64_t), s));
        SPG_TRY(idx.alloc(P * sizeof(uint32_t), s));
        SPG_TRY(pval.alloc(P * sizeof(double), s));
        sg_expand<<<grid_for(m * 32, GB), GB, 0, s>>>(A->d_off(), A->d_cols(), A->d_vals(), B->d_off(),
                                                     B->d_cols(), B->d_vals(), m, cbits, pofs.as<uint64_t>(),
                                                     key.as<uint64_t>(), idx.as<uint32_t>(), pval.as<double>());
        SPG_LAUNCH_CHECK();
        SPG_TRY(radix_sort_pairs_u64(c, key.as<uint64_t>(), idx.as<uint32_t>(), P, rbits + cbits, s));
        SPG_TRY(flag.alloc((P + 1) * sizeof(uint64_t), s));
        sg_run_flags<<<grid_for(P, GB, gmax), GB, 0, s>>>(key.as<uint64_t>(), P, flag.as<uint64_t>());
        SPG_LAUNCH_CHECK();
        SPG_TRY(exclusive_scan_u64(c, flag.as<uint64_t>(), P, flag.as<uint64_t>() + P, s));
        U = read_u64(flag.as<uint64_t>() + P, s, &rc);
        SPG_TRY(rc);
        SPG_TRY(begin.alloc((U + 1) * sizeof(uint64_t), s));
        sg_run_begins<<<grid_for(P, GB, gmax), GB, 0, s>>>(key.as<uint64_t>(), flag.as<uint64_t>(), P, U,
                                                          begin.as<uint64_t>());
        SPG_LAUNCH_CHECK();
        SPG_TRY(sum.alloc(U * sizeof(double), s));
        SPG_TRY(keep.alloc((U + 1) * sizeof(uint64_t), s));
        sg_run_sums<<<grid_for(U, GB, gmax), GB, 0, s>>>(begin.as<uint64_t>(), idx.as<uint32_t>(),
                                                        pval.as<double>(), U, sum.as<double>(), keep.as<uint64_t>());
        SPG_LAUNCH_CHECK();
        SPG_TRY(exclusive_scan_u64(c, keep.as<uint64_t>(), U, keep.as<uint64_t>() + U, s));
        nnz = read_u64(keep.as<uint64_t>() + U, s, &rc);
        SPG_TRY(rc);
    }
    SPG_TRY(out_off.alloc(csr_off_elems(m) * sizeof(uint64_t), s));
    SPG_TRY(out_cols.alloc(csr_alloc_elems(nnz) * sizeof(uint32_t), s));
    SPG_TRY(out_vals.alloc(csr_alloc_elems(nnz) * sizeof(double), s));
    SPG_TRY(crow.alloc((nnz ? nnz : 1) * sizeof(uint32_t), s));
    if (U) {
        sg_write<<<grid_for(U, GB, gmax), GB, 0, s>>>(begin.as<uint64_t>(), key.as<uint64_t>(), sum.as<double>(),
                                                     keep.as<uint64_t>(), U, cbits, out_cols.as<uint32_t>(),
                                                     out_vals.as<double>(), crow.as<uint32_t>());
        SPG_LAUNCH_CHECK();
    }
    sg_offsets<<<grid_for(m + 1, GB, gmax), GB, 0, s>>>(crow.as<uint32_t>(), nnz, m, out_off.as<uint64_t>());
    SPG_LAUNCH_CHECK();
    SPG_CUDA_TRY(cudaStreamSynchronize(s));
    Cm->invalidate_derived();
    Cm->n_rows = m;
    Cm->n_cols = n;
    Cm->off = std::move(out_off);
    Cm->cols = std::move(out_cols);
    Cm->vals = std::move(out_vals);
    Cm->nnz = nnz;
    Cm->capacity = nnz;
    Cm->built = true;
    Cm->may_have_zeros = false;
    return SPG_OK;
}

}  // namespace spg

using namespace spg;

extern "C" int spg_spgemm(spg_ctx *c, const spg_csr *A, const spg_csr *B, spg_csr *Cm) {
    if (!c || !A || !B || !Cm) return set_error(SPG_ERR_INVALID_ARGUMENT, "spg_spgemm: null handle");
    SPG_CHECK_LIVE(A);
    SPG_CHECK_LIVE(B);
    SPG_CHECK_LIVE(Cm);
    // Checks in the order of serial/spgemm.hpp:14-21.
    if (A->n_cols != B->n_rows) return set_error(SPG_ERR_INVALID_ARGUMENT, "A.cols must equal B.rows");
    if (!A->built) return set_error(SPG_ERR_LOGIC, "spgemm: A must be locked");
    if (!B->built) return set_error(SPG_ERR_LOGIC, "spgemm: B must be locked");
    if (Cm == A || Cm == B) return set_error(SPG_ERR_INVALID_ARGUMENT, "spg_spgemm: output aliases an input");
    SPG_CUDA_TRY(cudaSetDevice(c->device));
    return spgemm_impl(c, A, B, Cm, c->stream);
}
