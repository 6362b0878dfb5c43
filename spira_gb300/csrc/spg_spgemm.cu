// spg_spgemm.cu — C = A * B with Spira's exact structure and FP64 values.
//
// Spira (serial/spgemm.hpp:12-53, parallel/algorithms/spgemm.hpp:27-69) is a
// row-wise Gustavson product: for row i, for each a_ik in A's row (ascending
// k), for each b_kj in B's row k: acc[j] += a_ik * b_kj; entries with
// acc != 0 are inserted into C, and C.lock() sorts them. So each C(i, j) is
// the left-to-right sum over ascending k of the rounded products, starting
// from 0.0, and exact-zero sums are dropped.
//
// GPU formulation. Products per row of A are counted and scanned. Three
// variants compute the same C (the autotuner and the learned selector choose
// among them, spg_tune.cu):
//
//   SPG_SPGEMM_ROWMERGE: every row owns a scratch region of its product
//   count. Light rows (at most MG_RMAX entries in A's row and MG_PMAX
//   products): one thread merges the row's B rows (each sorted by column) as
//   a k-way merge on the column, taking equal columns in ascending A-entry
//   order, so every C(i, j) is summed in Spira's order. Heavy rows go through
//   expand - sort - compress (below). A final pass compacts the regions.
//
//   SPG_SPGEMM_ESC: expand - sort - compress for every row: expand the
//   products (key = i << cbits | j) in (row, A-entry, B-entry) order, stable
//   radix sort with the product index as payload (equal (i, j) keep
//   ascending k), sum each run left to right; the kept runs are C in order.
//
//   SPG_SPGEMM_WARPSORT_*: tiles of consecutive rows, a warp bitonic sort of
//   each row's (column, product) pairs in registers, a thread per row summing
//   the runs, and the output written in place through an ordered scan
//   (spg_spgemm_sort.cu).
//
// All use separate round-to-nearest multiply and add (__dmul_rn / __dadd_rn,
// never contracted) and drop exact-zero sums. Structure is exact; values
// match, bit for bit, Spira built for a target without FMA instructions
// (generic x86-64, as the oracle's recipe builds it). A Spira build that
// contracts acc[j] += a * b into fma(a, b, acc) — GCC's default
// -ffp-contract=fast on aarch64, or x86-64 with FMA enabled — differs in the
// last bits; the tests bound the difference to that order within 1e-12.
#include "spg_internal.cuh"

namespace spg {
namespace {

constexpr int GB = 256;

// Products per row of A (thread per row); entry m is 0.
__global__ void sg_row_products(const uint64_t *__restrict__ aoff, const uint32_t *__restrict__ acols,
                                const uint64_t *__restrict__ boff, uint64_t m, uint64_t *__restrict__ cnt) {
    const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (i > m) return;
    uint64_t s = 0;
    if (i < m)
        for (uint64_t ka = aoff[i]; ka < aoff[i + 1]; ++ka) {
            const uint32_t k = acols[ka];
            s += boff[k + 1] - boff[k];
        }
    cnt[i] = s;
}

constexpr int MG_RSMALL = 8;      // light rows: <= 8 A entries (cursors in registers) ...
constexpr int MG_RMAX = 32;       // ... or <= 32 (cursors in local memory)
constexpr uint64_t MG_PMAX = 4096;  // and at most this many products

__device__ __forceinline__ bool mg_light(uint64_t r, uint64_t p) { return r <= MG_RMAX && p <= MG_PMAX; }

// Product counts of the rows the row merge leaves to expand - sort -
// compress (0 for light rows); entry m is 0.
__global__ void sg_heavy_products(const uint64_t *__restrict__ aoff, const uint64_t *__restrict__ pofs, uint64_t m,
                                  uint64_t *__restrict__ hp) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i <= m; i += (uint64_t)gridDim.x * blockDim.x) {
        if (i == m) {
            hp[m] = 0;
            continue;
        }
        const uint64_t p = pofs[i + 1] - pofs[i];
        hp[i] = mg_light(aoff[i + 1] - aoff[i], p) ? 0 : p;
    }
}

// Light rows, one thread per row: k-way merge of the B rows named by the
// row's A entries. Each B row is strictly increasing in column, so every list
// holds at most one product of a given column; taking the smallest head
// column and then the lists whose head equals it in ascending list (= A
// entry = k) order sums C(i, j) exactly as Spira's acc[j] += a_ik * b_kj.
// Kept entries go to the row's scratch region at pofs[i]; rowcnt[i] = count.
// R = MG_RSMALL handles rows with r <= R and sets rowcnt = 0 for every other
// row; R = MG_RMAX handles MG_RSMALL < r <= MG_RMAX.
template <int R>
__global__ void __launch_bounds__(128)
sg_merge_rows(const uint64_t *__restrict__ aoff, const uint32_t *__restrict__ acols, const double *__restrict__ avals,
              const uint64_t *__restrict__ boff, const uint32_t *__restrict__ bcols, const double *__restrict__ bvals,
              uint64_t m, const uint64_t *__restrict__ pofs, uint32_t *__restrict__ tcols,
              double *__restrict__ tvals, uint64_t *__restrict__ rowcnt) {
    const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (i >= m) return;
    const uint64_t ab = aoff[i], r = aoff[i + 1] - ab;
    const uint64_t base = pofs[i], P = pofs[i + 1] - base;
    const bool mine = mg_light(r, P) && (R == MG_RSMALL ? r <= (uint64_t)R : r > (uint64_t)MG_RSMALL);
    if (!mine) {
        if (R == MG_RSMALL) rowcnt[i] = 0;
        return;
    }
    // per list: cursor, entries left, and the head's column and value (loaded
    // one step ahead, so a step waits for at most one round of loads; a
    // second register stage for the entry after the head measured slower:
    // 124 registers, four blocks per SM instead of five)
    constexpr bool PF = R <= MG_RSMALL;  // head values in registers (the wide version would spill)
    uint64_t cur[R];
    uint32_t left[R], head[R];
    double a[R], hv[PF ? R : 1];
#pragma unroll
    for (int t = 0; t < R; ++t) {
        cur[t] = 0;
        left[t] = 0;
        head[t] = 0;
        a[t] = 0.0;
        if constexpr (PF) hv[t] = 0.0;
        if ((uint64_t)t < r) {
            const uint32_t k = acols[ab + t];
            const uint64_t b0 = boff[k];
            cur[t] = b0;
            left[t] = (uint32_t)(boff[k + 1] - b0);
            a[t] = avals[ab + t];
            if (left[t]) {
                head[t] = bcols[b0];
                if constexpr (PF) hv[t] = bvals[b0];
            }
        }
    }
    constexpr uint64_t NONE = 1ull << 32;
    uint64_t cnt = 0;
    while (true) {
        uint64_t j = NONE;
#pragma unroll
        for (int t = 0; t < R; ++t)
            if (left[t] && head[t] < j) j = head[t];
        if (j == NONE) break;
        double acc = 0.0;  // ValueTraits zero; acc[j] default-constructs to V{}
        if constexpr (PF) {
            // One multiply and one add per contribution, issued for the whole
            // warp: pick the lowest list whose head is j, add its product,
            // advance it, repeat. (An add per list and per step, masked to the
            // lanes that need it, kept the FP64 pipe busy with idle lanes:
            // a warp FP64 instruction costs the same whatever its mask.)
            while (true) {
                int sel = -1;
                double av = 0.0, bv = 0.0;
#pragma unroll
                for (int t = R - 1; t >= 0; --t) {
                    if (left[t] && head[t] == j) {
                        sel = t;
                        av = a[t];
                        bv = hv[t];
                    }
                }
                if (sel < 0) break;
                acc = __dadd_rn(acc, __dmul_rn(av, bv));
#pragma unroll
                for (int t = 0; t < R; ++t) {
                    if (t == sel) {
                        ++cur[t];
                        if (--left[t]) {
                            head[t] = bcols[cur[t]];
                            hv[t] = bvals[cur[t]];
                        }
                    }
                }
            }
        } else {
#pragma unroll
            for (int t = 0; t < R; ++t) {
                if (left[t] && head[t] == j) {
                    acc = __dadd_rn(acc, __dmul_rn(a[t], bvals[cur[t]]));
                    ++cur[t];
                    if (--left[t]) head[t] = bcols[cur[t]];
                }
            }
        }
        if (!is_zero(acc)) {  // spgemm.hpp:44: v != V{}
            tcols[base + cnt] = (uint32_t)j;
            tvals[base + cnt] = acc;
            ++cnt;
        }
    }
    rowcnt[i] = cnt;
}

// Heavy rows' results (compacted, sorted by (row, col)) into their rows'
// scratch regions; the first entry of each row sets its count.
__global__ void sg_place_heavy(const uint32_t *__restrict__ crow, const uint32_t *__restrict__ ccol,
                               const double *__restrict__ cval, uint64_t nh, const uint64_t *__restrict__ pofs,
                               uint32_t *__restrict__ tcols, double *__restrict__ tvals,
                               uint64_t *__restrict__ rowcnt) {
    for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < nh; e += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t i = crow[e];
        uint64_t lo = 0, hi = e;  // first entry of row i
        while (lo < hi) {
            const uint64_t mid = (lo + hi) >> 1;
            if (crow[mid] < i) lo = mid + 1;
            else hi = mid;
        }
        const uint64_t rank = e - lo;
        tcols[pofs[i] + rank] = ccol[e];
        tvals[pofs[i] + rank] = cval[e];
        if (rank == 0) {
            uint64_t l2 = e, h2 = nh;  // one past the last entry of row i
            while (l2 < h2) {
                const uint64_t mid = (l2 + h2) >> 1;
                if (crow[mid] <= i) l2 = mid + 1;
                else h2 = mid;
            }
            rowcnt[i] = l2 - e;
        }
    }
}

// C from the scratch regions. Block b writes C positions [coff[r0], coff[r1])
// of its rows r0..r1-1 with consecutive threads on consecutive positions; a
// position's row is found by binary search in the block's copy of coff.
constexpr int CP_ROWS = 256;

__global__ void __launch_bounds__(CP_ROWS)
sg_compact(const uint64_t *__restrict__ pofs, const uint64_t *__restrict__ coff, uint64_t m,
           const uint32_t *__restrict__ tcols, const double *__restrict__ tvals, uint32_t *__restrict__ ccols,
           double *__restrict__ cvals) {
    __shared__ uint64_t soff[CP_ROWS + 1], ssrc[CP_ROWS];
    const uint64_t r0 = (uint64_t)blockIdx.x * CP_ROWS;
    const int nr = (int)min((uint64_t)CP_ROWS, m - r0);
    for (int t = threadIdx.x; t <= nr; t += blockDim.x) soff[t] = coff[r0 + t];
    for (int t = threadIdx.x; t < nr; t += blockDim.x) ssrc[t] = pofs[r0 + t];
    __syncthreads();
    const uint64_t q1 = soff[nr];
    for (uint64_t q = soff[0] + threadIdx.x; q < q1; q += blockDim.x) {
        int lo = 0, hi = nr;  // last t with soff[t] <= q
        while (hi - lo > 1) {
            const int mid = (lo + hi) >> 1;
            if (soff[mid] <= q) lo = mid;
            else hi = mid;
        }
        const uint64_t src = ssrc[lo] + (q - soff[lo]);
        ccols[q] = tcols[src];
        cvals[q] = tvals[src];
    }
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
    if (pofs[w + 1] == base) return;  // no products here (or a row handled by the merge path)
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
        keep[u] = is_zero(acc) ? 0 : 1;  // spgemm.hpp:44: v != V{}
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


}  // namespace

// One uint64 read back from the device (synchronises the stream).
uint64_t read_u64(Ctx *c, const uint64_t *d, cudaStream_t s, int *rc) {
    uint64_t h = 0;
    const cudaError_t e = cudaMemcpyAsync(&h, d, 8, cudaMemcpyDeviceToHost, s);
    if (e != cudaSuccess) *rc = set_error(SPG_ERR_CUDA, "spgemm: %s", cudaGetErrorString(e));
    else *rc = c->phase_sync(s);
    return h;
}

// Expand - sort - compress over the rows whose entries of `hp` (the scanned
// product counts of the selected rows, 0 for the others; hp[m] = HP, their
// total) select: products in (row, A entry, B entry) order, a stable radix
// sort by (row, column) carrying the product index, each run summed left to
// right from 0.0, kept sums compacted in (row, column) order into out.
int spgemm_esc(Ctx *c, const Csr *A, const Csr *B, const uint64_t *hp, uint64_t HP, int rbits, int cbits,
               EscOut *out, cudaStream_t s) {
    const uint64_t m = A->n_rows;
    const unsigned gmax = (unsigned)c->n_sms * 32;
    int rc = SPG_OK;
    out->n = 0;
    if (HP == 0) return SPG_OK;
    const uint64_t P = HP;
    DevBuf key, idx, pval, flag, begin, sum, keep;
    SPG_TRY(key.alloc(P * sizeof(uint64_t), s));
    SPG_TRY(idx.alloc(P * sizeof(uint32_t), s));
    SPG_TRY(pval.alloc(P * sizeof(double), s));
    sg_expand<<<grid_for(m * 32, GB), GB, 0, s>>>(A->d_off(), A->d_cols(), A->d_vals(), B->d_off(), B->d_cols(),
                                                 B->d_vals(), m, cbits, hp, key.as<uint64_t>(), idx.as<uint32_t>(),
                                                 pval.as<double>());
    SPG_LAUNCH_CHECK();
    SPG_TRY(radix_sort_pairs_u64(c, key.as<uint64_t>(), idx.as<uint32_t>(), P, rbits + cbits, s));
    SPG_TRY(flag.alloc((P + 1) * sizeof(uint64_t), s));
    sg_run_flags<<<grid_for(P, GB, gmax), GB, 0, s>>>(key.as<uint64_t>(), P, flag.as<uint64_t>());
    SPG_LAUNCH_CHECK();
    SPG_TRY(exclusive_scan_u64(c, flag.as<uint64_t>(), P, flag.as<uint64_t>() + P, s));
    const uint64_t U = read_u64(c, flag.as<uint64_t>() + P, s, &rc);
    SPG_TRY(rc);
    SPG_TRY(begin.alloc((U + 1) * sizeof(uint64_t), s));
    sg_run_begins<<<grid_for(P, GB, gmax), GB, 0, s>>>(key.as<uint64_t>(), flag.as<uint64_t>(), P, U,
                                                      begin.as<uint64_t>());
    SPG_LAUNCH_CHECK();
    SPG_TRY(sum.alloc(U * sizeof(double), s));
    SPG_TRY(keep.alloc((U + 1) * sizeof(uint64_t), s));
    sg_run_sums<<<grid_for(U, GB, gmax), GB, 0, s>>>(begin.as<uint64_t>(), idx.as<uint32_t>(), pval.as<double>(), U,
                                                    sum.as<double>(), keep.as<uint64_t>());
    SPG_LAUNCH_CHECK();
    SPG_TRY(exclusive_scan_u64(c, keep.as<uint64_t>(), U, keep.as<uint64_t>() + U, s));
    const uint64_t nh = read_u64(c, keep.as<uint64_t>() + U, s, &rc);
    SPG_TRY(rc);
    out->n = nh;
    if (nh == 0) return SPG_OK;
    // cols / vals padded like a CSR's, so the ESC variant can install them as C
    SPG_TRY(out->crow.alloc(nh * sizeof(uint32_t), s));
    SPG_TRY(out->ccol.alloc(csr_alloc_elems(nh) * sizeof(uint32_t), s));
    SPG_TRY(out->cval.alloc(csr_alloc_elems(nh) * sizeof(double), s));
    sg_write<<<grid_for(U, GB, gmax), GB, 0, s>>>(begin.as<uint64_t>(), key.as<uint64_t>(), sum.as<double>(),
                                                 keep.as<uint64_t>(), U, cbits, out->ccol.as<uint32_t>(),
                                                 out->cval.as<double>(), out->crow.as<uint32_t>());
    SPG_LAUNCH_CHECK();
    return SPG_OK;
}

namespace {

// Row merge's heavy rows: expand - sort - compress, results placed in the
// rows' scratch regions with their counts.
int spgemm_heavy_rows(Ctx *c, const Csr *A, const Csr *B, const uint64_t *pofs, uint32_t *tcols, double *tvals,
                      uint64_t *rowcnt, int rbits, int cbits, cudaStream_t s) {
    const uint64_t m = A->n_rows;
    const unsigned gmax = (unsigned)c->n_sms * 32;
    int rc = SPG_OK;
    DevBuf hp;
    SPG_TRY(hp.alloc((m + 1) * sizeof(uint64_t), s));
    sg_heavy_products<<<grid_for(m + 1, GB, gmax), GB, 0, s>>>(A->d_off(), pofs, m, hp.as<uint64_t>());
    SPG_LAUNCH_CHECK();
    SPG_TRY(exclusive_scan_u64(c, hp.as<uint64_t>(), m + 1, nullptr, s));
    const uint64_t P = read_u64(c, hp.as<uint64_t>() + m, s, &rc);
    SPG_TRY(rc);
    EscOut eo;
    SPG_TRY(spgemm_esc(c, A, B, hp.as<uint64_t>(), P, rbits, cbits, &eo, s));
    if (eo.n == 0) return SPG_OK;
    sg_place_heavy<<<grid_for(eo.n, GB, gmax), GB, 0, s>>>(eo.crow.as<uint32_t>(), eo.ccol.as<uint32_t>(),
                                                          eo.cval.as<double>(), eo.n, pofs, tcols, tvals, rowcnt);
    SPG_LAUNCH_CHECK();
    return SPG_OK;
}

// Row counts of ESC's compacted output (crow sorted): cnt[crow[e]] += 1.
__global__ void sg_count_rows(const uint32_t *__restrict__ crow, uint64_t n, unsigned long long *__restrict__ cnt) {
    for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < n; e += (uint64_t)gridDim.x * blockDim.x)
        atomicAdd(cnt + crow[e], 1ull);
}

}  // namespace

// C's arrays installed into Cm (reshaped to m x n).
void spgemm_install(Csr *Cm, uint64_t m, uint64_t n, DevBuf &&off, DevBuf &&cols, DevBuf &&vals, uint64_t nnz) {
    Cm->invalidate_derived();
    Cm->n_rows = m;
    Cm->n_cols = n;
    Cm->off = std::move(off);
    Cm->cols = std::move(cols);
    Cm->vals = std::move(vals);
    Cm->nnz = nnz;
    Cm->capacity = nnz;
    Cm->built = true;
    Cm->may_have_zeros = false;
}

// Products per row of A (pofs[i], scanned in place; pofs[m] = P) and P.
int spgemm_products(Ctx *c, const Csr *A, const Csr *B, DevBuf *pofs, uint64_t *P, cudaStream_t s) {
    const uint64_t m = A->n_rows;
    int rc = SPG_OK;
    SPG_TRY(pofs->alloc((m + 1) * sizeof(uint64_t), s));
    sg_row_products<<<grid_for(m + 1, GB), GB, 0, s>>>(A->d_off(), A->d_cols(), B->d_off(), m,
                                                             pofs->as<uint64_t>());
    SPG_LAUNCH_CHECK();
    SPG_TRY(exclusive_scan_u64(c, pofs->as<uint64_t>(), m + 1, nullptr, s));
    *P = read_u64(c, pofs->as<uint64_t>() + m, s, &rc);
    SPG_TRY(rc);
    if (*P >= (1ull << 32))
        return set_error(SPG_ERR_UNSUPPORTED, "spgemm: %llu products exceed 2^32-1", (unsigned long long)*P);
    return SPG_OK;
}

// SPG_SPGEMM_ESC: expand - sort - compress for every row; its compacted
// output is C in CSR order.
int spgemm_esc_all(Ctx *c, const Csr *A, const Csr *B, Csr *Cm, cudaStream_t s) {
    const uint64_t m = A->n_rows, n = B->n_cols;
    const int cbits = bits_for(n), rbits = bits_for(m);
    DevBuf pofs;
    uint64_t P = 0;
    SPG_TRY(spgemm_products(c, A, B, &pofs, &P, s));
    EscOut eo;
    SPG_TRY(spgemm_esc(c, A, B, pofs.as<uint64_t>(), P, rbits, cbits, &eo, s));
    DevBuf off;
    SPG_TRY(off.alloc(csr_off_elems(m) * sizeof(uint64_t), s));
    SPG_CUDA_TRY(cudaMemsetAsync(off.ptr, 0, csr_off_elems(m) * sizeof(uint64_t), s));
    if (eo.n) {
        sg_count_rows<<<grid_for(eo.n, GB, (unsigned)c->n_sms * 32), GB, 0, s>>>(
            eo.crow.as<uint32_t>(), eo.n, reinterpret_cast<unsigned long long *>(off.as<uint64_t>()));
        SPG_LAUNCH_CHECK();
    }
    SPG_TRY(exclusive_scan_u64(c, off.as<uint64_t>(), m + 1, nullptr, s));
    if (!eo.n) {
        SPG_TRY(eo.ccol.alloc(csr_alloc_elems(0) * sizeof(uint32_t), s));
        SPG_TRY(eo.cval.alloc(csr_alloc_elems(0) * sizeof(double), s));
    }
    SPG_TRY(c->phase_sync(s));
    spgemm_install(Cm, m, n, std::move(off), std::move(eo.ccol), std::move(eo.cval), eo.n);
    return SPG_OK;
}

// SPG_SPGEMM_ROWMERGE.
int spgemm_rowmerge(Ctx *c, const Csr *A, const Csr *B, Csr *Cm, cudaStream_t s) {
    const uint64_t m = A->n_rows, n = B->n_cols;
    const int cbits = bits_for(n), rbits = bits_for(m);
    int rc = SPG_OK;
    DevBuf pofs;
    uint64_t P = 0;
    SPG_TRY(spgemm_products(c, A, B, &pofs, &P, s));
    // out_off holds the per-row kept counts, then (scanned) C's offsets
    DevBuf tcols, tvals, out_off, out_cols, out_vals;
    SPG_TRY(out_off.alloc(csr_off_elems(m) * sizeof(uint64_t), s));
    SPG_CUDA_TRY(cudaMemsetAsync(out_off.ptr, 0, csr_off_elems(m) * sizeof(uint64_t), s));
    if (P) {
        SPG_TRY(tcols.alloc(P * sizeof(uint32_t), s));
        SPG_TRY(tvals.alloc(P * sizeof(double), s));
        sg_merge_rows<MG_RSMALL><<<grid_for(m, 128), 128, 0, s>>>(
            A->d_off(), A->d_cols(), A->d_vals(), B->d_off(), B->d_cols(), B->d_vals(), m, pofs.as<uint64_t>(),
            tcols.as<uint32_t>(), tvals.as<double>(), out_off.as<uint64_t>());
        SPG_LAUNCH_CHECK();
        sg_merge_rows<MG_RMAX><<<grid_for(m, 128), 128, 0, s>>>(
            A->d_off(), A->d_cols(), A->d_vals(), B->d_off(), B->d_cols(), B->d_vals(), m, pofs.as<uint64_t>(),
            tcols.as<uint32_t>(), tvals.as<double>(), out_off.as<uint64_t>());
        SPG_LAUNCH_CHECK();
        SPG_TRY(spgemm_heavy_rows(c, A, B, pofs.as<uint64_t>(), tcols.as<uint32_t>(), tvals.as<double>(),
                                  out_off.as<uint64_t>(), rbits, cbits, s));
    }
    SPG_TRY(exclusive_scan_u64(c, out_off.as<uint64_t>(), m + 1, nullptr, s));
    const uint64_t nnz = read_u64(c, out_off.as<uint64_t>() + m, s, &rc);
    SPG_TRY(rc);
    SPG_TRY(out_cols.alloc(csr_alloc_elems(nnz) * sizeof(uint32_t), s));
    SPG_TRY(out_vals.alloc(csr_alloc_elems(nnz) * sizeof(double), s));
    if (nnz) {
        sg_compact<<<grid_for(m, CP_ROWS), CP_ROWS, 0, s>>>(pofs.as<uint64_t>(), out_off.as<uint64_t>(), m,
                                                           tcols.as<uint32_t>(), tvals.as<double>(),
                                                           out_cols.as<uint32_t>(), out_vals.as<double>());
        SPG_LAUNCH_CHECK();
    }
    SPG_TRY(c->phase_sync(s));
    spgemm_install(Cm, m, n, std::move(out_off), std::move(out_cols), std::move(out_vals), nnz);
    return SPG_OK;
}

int spgemm_run(Ctx *c, const Csr *A, const Csr *B, Csr *Cm, int variant, cudaStream_t s) {
    switch (variant) {
        case SPG_SPGEMM_ROWMERGE: return spgemm_rowmerge(c, A, B, Cm, s);
        case SPG_SPGEMM_ESC: return spgemm_esc_all(c, A, B, Cm, s);
        case SPG_SPGEMM_WARPSORT_64:
        case SPG_SPGEMM_WARPSORT_128:
        case SPG_SPGEMM_WARPSORT_256: return spgemm_warpsort(c, A, B, Cm, variant, s);
        default: return set_error(SPG_ERR_INVALID_ARGUMENT, "spgemm: unknown variant %d", variant);
    }
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
    int v = SPG_SPGEMM_AUTO;
    SPG_TRY(spgemm_resolve_auto(c, A, B, &v));
    return spgemm_run(c, A, B, Cm, v, c->stream);
}

extern "C" int spg_spgemm_variant(spg_ctx *c, const spg_csr *A, const spg_csr *B, spg_csr *Cm, int variant) {
    if (!c || !A || !B || !Cm) return set_error(SPG_ERR_INVALID_ARGUMENT, "spg_spgemm_variant: null handle");
    SPG_CHECK_LIVE(A);
    SPG_CHECK_LIVE(B);
    SPG_CHECK_LIVE(Cm);
    if (A->n_cols != B->n_rows) return set_error(SPG_ERR_INVALID_ARGUMENT, "A.cols must equal B.rows");
    if (!A->built) return set_error(SPG_ERR_LOGIC, "spgemm: A must be locked");
    if (!B->built) return set_error(SPG_ERR_LOGIC, "spgemm: B must be locked");
    if (Cm == A || Cm == B) return set_error(SPG_ERR_INVALID_ARGUMENT, "spg_spgemm: output aliases an input");
    if (variant < SPG_SPGEMM_AUTO || variant >= SPG_SPGEMM_N_VARIANTS)
        return set_error(SPG_ERR_INVALID_ARGUMENT, "spg_spgemm_variant: unknown variant %d", variant);
    SPG_CUDA_TRY(cudaSetDevice(c->device));
    if (variant == SPG_SPGEMM_AUTO) SPG_TRY(spgemm_resolve_auto(c, A, B, &variant));
    return spgemm_run(c, A, B, Cm, variant, c->stream);
}
