// spg_spmv.cu — FP64 CSR SpMV y = A x on sm_103a.
//
// Spira computes each row as a sparse dot product over the row's CSR slice
// (serial/spmv.hpp:44-55 scalar loop, serial/spmv.hpp:141-186 and
// parallel/algorithms/spmv.hpp:125-161 through kernel::sparse_dot_double,
// whose SIMD bodies keep 4 blocked accumulators, dot_avx512.cpp:7-56,
// dot_neon.cpp:7-56). The kernels below compute the same row sums with GPU
// reduction trees; the per-row result agrees with Spira's within the FP64
// reassociation bound, not bit for bit (bit-exact only for SCALAR, which
// keeps Spira's left-to-right order with fused multiply-adds).
//
// Variants (one family each for the row-, warp- and merge-path shapes):
//   SCALAR     one thread per row (the plain path);
//   VECTOR<G>  G lanes per row, shuffle reduction; G = 32 uses 16-byte
//              (double2 / uint2) loads of vals / cols;
//   STREAM     row blocks of <= 2047 nnz (or one long row) per CTA; the block's
//              vals/cols/x products are staged in shared memory with coalesced
//              loads and reduced with an adaptive number of lanes per row;
//   MERGE      merge-path split of (row ends + nnz) into equal CTA tiles,
//              carry-out fix-up in tile order (deterministic).
// All bandwidth-bound; the roofline is HBM (12 B/nnz + 8 B/row offsets +
// 8 B/col x + 8 B/row y).
#include "spg_internal.cuh"

namespace spg {
namespace {

constexpr int BLOCK = 256;

__device__ __forceinline__ double ldx(const double *__restrict__ x, uint32_t c) { return __ldg(x + c); }

// ---------------------------------------------------------------------------
// SCALAR: thread per row, fma chain in CSR order (Spira's scalar order with
// contraction: acc = fma(x[c], v, acc)).
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(BLOCK)
spmv_scalar(const uint64_t *__restrict__ off, const uint32_t *__restrict__ cols,
            const double *__restrict__ vals, const double *__restrict__ x,
            double *__restrict__ y, uint64_t n_rows) {
  for (uint64_t r = (uint64_t)blockIdx.x * BLOCK + threadIdx.x; r < n_rows; r += (uint64_t)gridDim.x * BLOCK) {
    const uint64_t b = off[r], e = off[r + 1];
    double acc = 0.0;
    uint64_t k = b;
    // four entries' loads and gathers issued before their FMAs (the chain
    // itself stays in CSR order)
    for (; k + 4 <= e; k += 4) {
        const uint32_t c0 = cols[k], c1 = cols[k + 1], c2 = cols[k + 2], c3 = cols[k + 3];
        const double v0 = vals[k], v1 = vals[k + 1], v2 = vals[k + 2], v3 = vals[k + 3];
        const double x0 = ldx(x, c0), x1 = ldx(x, c1), x2 = ldx(x, c2), x3 = ldx(x, c3);
        acc = fma(x0, v0, acc);
        acc = fma(x1, v1, acc);
        acc = fma(x2, v2, acc);
        acc = fma(x3, v3, acc);
    }
    for (; k < e; ++k) acc = fma(ldx(x, cols[k]), vals[k], acc);
    y[r] = acc;
  }
}

// Dot over [b, e) by NL cooperating lanes (lane in [0, NL)), lane-strided,
// 16-byte loads over the even-aligned interior, scalar head/tail.
template <int NL>
__device__ __forceinline__ double seg_dot_vec2(const uint32_t *__restrict__ cols,
                                               const double *__restrict__ vals,
                                               const double *__restrict__ x, uint64_t b,
                                               uint64_t e, int lane) {
    double acc = 0.0, acc1 = 0.0;
    uint64_t a = (b + 1) & ~1ull;
    if (a > e) a = e;
    const uint64_t ae = e & ~1ull;
    if (b < a && lane == 0) acc = fma(ldx(x, cols[b]), vals[b], acc);
    uint64_t i = a + 2ull * lane;
    // 4 pairs in flight per lane: all loads issue before the gathers.
    for (; i + 6ull * NL < ae; i += 8ull * NL) {
        double2 v[4];
        uint2 c[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            v[u] = *reinterpret_cast<const double2 *>(vals + i + 2ull * NL * u);
            c[u] = *reinterpret_cast<const uint2 *>(cols + i + 2ull * NL * u);
        }
        double g[8];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            g[2 * u] = ldx(x, c[u].x);
            g[2 * u + 1] = ldx(x, c[u].y);
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            acc = fma(g[2 * u], v[u].x, acc);
            acc1 = fma(g[2 * u + 1], v[u].y, acc1);
        }
    }
    for (; i < ae; i += 2ull * NL) {
        const double2 v = *reinterpret_cast<const double2 *>(vals + i);
        const uint2 c = *reinterpret_cast<const uint2 *>(cols + i);
        acc = fma(ldx(x, c.x), v.x, acc);
        acc1 = fma(ldx(x, c.y), v.y, acc1);
    }
    if (ae < e && ae >= a && lane == NL - 1) acc = fma(ldx(x, cols[ae]), vals[ae], acc);
    return acc + acc1;
}

template <int G>
__device__ __forceinline__ double group_reduce(double v) {
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o, G);
    return v;
}

// ---------------------------------------------------------------------------
// VECTOR<G>: G lanes per row.
// ---------------------------------------------------------------------------
template <int G>
__global__ void __launch_bounds__(BLOCK)
spmv_vector(const uint64_t *__restrict__ off, const uint32_t *__restrict__ cols,
            const double *__restrict__ vals, const double *__restrict__ x,
            double *__restrict__ y, uint64_t n_rows) {
    const uint64_t t = (uint64_t)blockIdx.x * BLOCK + threadIdx.x;
    const uint64_t r = t / G;
    const int lane = (int)(t % G);
    // Whole groups are inside or outside the range (BLOCK % G == 0), so the
    // shuffles below never miss a partner.
    if (r >= n_rows) return;
    const uint64_t b = off[r], e = off[r + 1];
    double acc;
    if (G == 32) {
        acc = seg_dot_vec2<32>(cols, vals, x, b, e, lane);
    } else {
        acc = 0.0;
        double acc1 = 0.0;
        uint64_t k = b + lane;
        for (; k + G < e; k += 2 * G) {
            const uint32_t c0 = cols[k], c1 = cols[k + G];
            const double v0 = vals[k], v1 = vals[k + G];
            acc = fma(ldx(x, c0), v0, acc);
            acc1 = fma(ldx(x, c1), v1, acc1);
        }
        if (k < e) acc = fma(ldx(x, cols[k]), vals[k], acc);
        acc += acc1;
    }
    acc = group_reduce<G>(acc);
    if (lane == 0) y[r] = acc;
}

// ---------------------------------------------------------------------------
// STREAM: plan of row blocks.
// A row r starts a block iff r == 0, r % ROWCAP == 0, its start offset falls in
// a different BIN-sized nnz bin than row r-1's, or r or r-1 is a long row
// (> LONG nnz). Hence a block is either one long row or <= ROWCAP short rows
// whose starts share a bin: nnz <= (BIN - 1) + LONG.
// ---------------------------------------------------------------------------
constexpr int ST_LOG_BIN = 10;
constexpr uint64_t ST_BIN = 1ull << ST_LOG_BIN;
constexpr uint64_t ST_LONG = 1024;
constexpr int ST_ROWCAP = 1024;
constexpr int ST_MAX_NNZ = (int)(ST_BIN - 1 + ST_LONG);  // 2047

__global__ void stream_plan_flags(const uint64_t *__restrict__ off, uint64_t n_rows,
                                  uint64_t *__restrict__ flag) {
    const uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n_rows) return;
    bool f = (r == 0) || (r % ST_ROWCAP == 0);
    if (!f) {
        const uint64_t o0 = off[r - 1], o1 = off[r], o2 = off[r + 1];
        f = ((o0 >> ST_LOG_BIN) != (o1 >> ST_LOG_BIN)) || (o1 - o0 > ST_LONG) || (o2 - o1 > ST_LONG);
    }
    flag[r] = f ? 1 : 0;
}

__global__ void stream_plan_scatter(const uint64_t *__restrict__ pos, uint64_t n_rows,
                                    uint64_t *__restrict__ blk) {
    const uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n_rows) return;
    const uint64_t p = pos[r];
    const uint64_t q = pos[r + 1];  // pos has n_rows + 1 entries (total at the end)
    if (q != p) blk[p] = r;
    if (r == n_rows - 1) blk[q] = n_rows;
}

__device__ __forceinline__ double block_reduce_sum(double v, double *red) {
    v = group_reduce<32>(v);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) red[warp] = v;
    __syncthreads();
    double s = 0.0;
    if (warp == 0) {
        s = (lane < BLOCK / 32) ? red[lane] : 0.0;
        s = group_reduce<32>(s);
    }
    return s;  // valid in thread 0
}

__global__ void __launch_bounds__(BLOCK)
spmv_stream(const uint64_t *__restrict__ off, const uint32_t *__restrict__ cols,
            const double *__restrict__ vals, const double *__restrict__ x,
            double *__restrict__ y, const uint64_t *__restrict__ blk) {
    __shared__ double prod[ST_MAX_NNZ + 1];
    __shared__ uint32_t soff[ST_ROWCAP + 1];
    __shared__ double red[BLOCK / 32];
    const uint64_t r0 = blk[blockIdx.x], r1 = blk[blockIdx.x + 1];
    const uint64_t k0 = off[r0], k1 = off[r1];
    const uint32_t nrows = (uint32_t)(r1 - r0);
    const uint64_t nz = k1 - k0;
    if (nz > (uint64_t)ST_MAX_NNZ) {  // a single long row
        double acc = seg_dot_vec2<BLOCK>(cols, vals, x, k0, k1, threadIdx.x);
        acc = block_reduce_sum(acc, red);
        if (threadIdx.x == 0) y[r0] = acc;
        return;
    }
    for (uint32_t i = threadIdx.x; i <= nrows; i += BLOCK) soff[i] = (uint32_t)(off[r0 + i] - k0);
    {
        // ST_ITEMS loads per thread issued before any gather (coalesced).
        constexpr int ST_ITEMS = (ST_MAX_NNZ + BLOCK) / BLOCK;
        double v[ST_ITEMS];
        uint32_t c[ST_ITEMS];
#pragma unroll
        for (int u = 0; u < ST_ITEMS; ++u) {
            const uint32_t i = u * BLOCK + threadIdx.x;
            if (i < nz) {
                v[u] = vals[k0 + i];
                c[u] = cols[k0 + i];
            }
        }
#pragma unroll
        for (int u = 0; u < ST_ITEMS; ++u) {
            const uint32_t i = u * BLOCK + threadIdx.x;
            if (i < nz) prod[i] = v[u] * ldx(x, c[u]);
        }
    }
    __syncthreads();
    // lanes per row: as many as fit, power of two, <= 32
    int L = 1;
    while (L < 32 && (uint32_t)(L * 2) * nrows <= BLOCK) L *= 2;
    const int lane = threadIdx.x % L;
    const uint32_t grp = threadIdx.x / L, ngrp = BLOCK / L;
    for (uint32_t base = 0; base < nrows; base += ngrp) {
        const uint32_t rr = base + grp;  // all lanes of a group share rr
        double acc = 0.0;
        if (rr < nrows) {
            const uint32_t b = soff[rr], e = soff[rr + 1];
            for (uint32_t k = b + lane; k < e; k += L) acc += prod[k];
        }
        // reduce within the group of L lanes (L is block-uniform)
        for (int o = L / 2; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o, L);
        if (rr < nrows && lane == 0) y[r0 + rr] = acc;
    }
}

// ---------------------------------------------------------------------------
// MERGE: merge-path over the two sorted lists A = row end offsets
// (off[1..n]) and B = nnz indices (0..nnz-1). Diagonal d splits at (i, j) with
// i + j = d; tile t covers diagonals [t*TILE, (t+1)*TILE). Each thread walks
// ITEMS consecutive path steps sequentially (rows it finishes are written
// directly), its trailing partial row is combined across threads with a
// segmented block scan, and the tile's last partial row goes to a carry-out
// fixed up in tile order by a second kernel.
// ---------------------------------------------------------------------------
constexpr int MG_ITEMS = 7;
constexpr int MG_TILE = BLOCK * MG_ITEMS;

__device__ __forceinline__ void merge_path_search(uint64_t diag, const uint64_t *__restrict__ row_end,
                                                  uint64_t n_rows, uint64_t nnz, uint64_t &ri,
                                                  uint64_t &ki) {
    // Find the first i such that row_end[i] > diag - i - 1 ... standard form:
    // largest i in [lo, hi] with row_end[i-1] <= diag - i  (A items consumed first on ties)
    uint64_t lo = diag > nnz ? diag - nnz : 0;
    uint64_t hi = diag < n_rows ? diag : n_rows;
    while (lo < hi) {
        const uint64_t mid = (lo + hi) >> 1;
        // A[mid] = row_end[mid] (end offset of row mid); B[diag - mid - 1] = diag - mid - 1
        if (row_end[mid] <= diag - mid - 1) lo = mid + 1;
        else hi = mid;
    }
    ri = lo;
    ki = diag - lo;
}

__global__ void merge_tile_starts(const uint64_t *__restrict__ off, uint64_t n_rows, uint64_t nnz,
                                  uint64_t n_tiles, uint64_t *__restrict__ starts /* 2*(n_tiles+1) */) {
    const uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t > n_tiles) return;
    uint64_t diag = t * MG_TILE;
    const uint64_t total = n_rows + nnz;
    if (diag > total) diag = total;
    uint64_t ri, ki;
    merge_path_search(diag, off + 1, n_rows, nnz, ri, ki);
    starts[2 * t] = ri;
    starts[2 * t + 1] = ki;
}

struct Carry {
    uint64_t row;
    double val;
};

// Block-wide exclusive segmented scan of (head, value) pairs in thread
// order: a head starts a new segment at that thread's value. Returns the
// exclusive result; *incl_last receives the inclusive result of the last
// thread (the tile's carry-out value). Fixed tree: deterministic.
__device__ __forceinline__ double block_seg_excl_scan(bool head, double v, double *incl_last) {
    __shared__ double w_val[BLOCK / 32];
    __shared__ int w_head[BLOCK / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int h = head;
    double p = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int hh = __shfl_up_sync(0xffffffffu, h, o);
        const double pp = __shfl_up_sync(0xffffffffu, p, o);
        if (lane >= o) {
            if (!h) p = pp + p;
            h |= hh;
        }
    }
    if (lane == 31) {
        w_val[warp] = p;
        w_head[warp] = h;
    }
    __syncthreads();
    // carry into this warp from the warps before it, in order
    double wc = 0.0;
    for (int w = 0; w < warp; ++w) wc = w_head[w] ? w_val[w] : wc + w_val[w];
    double incl = h ? p : wc + p;
    double excl = __shfl_up_sync(0xffffffffu, incl, 1);
    if (lane == 0) excl = wc;
    if (threadIdx.x == BLOCK - 1) *incl_last = incl;
    return excl;
}

__global__ void __launch_bounds__(BLOCK)
spmv_merge(const uint64_t *__restrict__ off, const uint32_t *__restrict__ cols,
           const double *__restrict__ vals, const double *__restrict__ x, double *__restrict__ y,
           uint64_t n_rows, const uint64_t *__restrict__ starts, Carry *__restrict__ carry) {
    __shared__ uint64_t s_rowend[MG_TILE];
    __shared__ double s_prod[MG_TILE];
    __shared__ double s_carry_val;
    const uint64_t t = blockIdx.x;
    const uint64_t r_begin = starts[2 * t], k_begin = starts[2 * t + 1];
    const uint64_t r_end = starts[2 * t + 2], k_end = starts[2 * t + 3];
    const uint32_t nr = (uint32_t)(r_end - r_begin), nk = (uint32_t)(k_end - k_begin);
    {
        double v[MG_ITEMS];
        uint32_t c[MG_ITEMS];
        uint64_t re[MG_ITEMS];
#pragma unroll
        for (int u = 0; u < MG_ITEMS; ++u) {
            const uint32_t i = u * BLOCK + threadIdx.x;
            if (i < nk) {
                v[u] = vals[k_begin + i];
                c[u] = cols[k_begin + i];
            }
            if (i < nr) re[u] = off[r_begin + i + 1];
        }
#pragma unroll
        for (int u = 0; u < MG_ITEMS; ++u) {
            const uint32_t i = u * BLOCK + threadIdx.x;
            if (i < nk) s_prod[i] = v[u] * ldx(x, c[u]);
            if (i < nr) s_rowend[i] = re[u];
        }
    }
    __syncthreads();
    // This thread's start on the tile's merge path (diagonal d).
    const uint32_t tile_len = nr + nk;
    const uint32_t d = min((uint32_t)threadIdx.x * MG_ITEMS, tile_len);
    uint32_t lo = d > nk ? d - nk : 0, hi = min(d, nr);
    while (lo < hi) {
        const uint32_t mid = (lo + hi) >> 1;
        if (s_rowend[mid] <= k_begin + (d - mid - 1)) lo = mid + 1;
        else hi = mid;
    }
    const uint32_t ri0 = lo;
    uint32_t ri = lo, ki = d - lo;
    const uint32_t dend = min(d + (uint32_t)MG_ITEMS, tile_len);
    double acc = 0.0, first = 0.0;
    for (uint32_t step = d; step < dend; ++step) {
        if (ri < nr && s_rowend[ri] <= k_begin + ki) {  // row ri ends here
            if (ri == ri0) first = acc;
            else y[r_begin + ri] = acc;
            acc = 0.0;
            ++ri;
        } else {
            acc += s_prod[ki];
            ++ki;
        }
    }
    const bool head = (ri != ri0);
    // the value this thread contributes to the segment it ends in
    const double carry_in = block_seg_excl_scan(head, acc, &s_carry_val);
    if (head) y[r_begin + ri0] = carry_in + first;
    __syncthreads();
    if (threadIdx.x == BLOCK - 1) {
        carry[t].row = r_begin + ri;
        carry[t].val = s_carry_val;
    }
}

// Adds each tile's carry-out to its row. A run of consecutive tiles carrying
// into the same row (a row spanning tiles) is summed by the run's first tile
// in tile order, so the result is deterministic.
__global__ void merge_fixup(const Carry *__restrict__ carry, uint64_t n_tiles, uint64_t n_rows,
                            double *__restrict__ y) {
    const uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n_tiles) return;
    const uint64_t r = carry[t].row;
    if (r >= n_rows) return;
    if (t > 0 && carry[t - 1].row == r) return;
    double s = carry[t].val;
    for (uint64_t u = t + 1; u < n_tiles && carry[u].row == r; ++u) s += carry[u].val;
    y[r] += s;
}

}  // namespace

// ---------------------------------------------------------------------------
// Plans
// ---------------------------------------------------------------------------
static int build_stream_plan(Ctx *c, Csr *A, cudaStream_t s) {
    if (A->plan_stream.kind == SPG_SPMV_STREAM) return SPG_OK;
    const uint64_t n = A->n_rows;
    DevBuf flag;
    SPG_TRY(flag.alloc((n + 1) * sizeof(uint64_t), s));
    stream_plan_flags<<<grid_for(n, 256), 256, 0, s>>>(A->d_off(), n, flag.as<uint64_t>());
    SPG_LAUNCH_CHECK();
    DevBuf total;
    SPG_TRY(total.alloc(sizeof(uint64_t), s));
    SPG_TRY(exclusive_scan_u64(c, flag.as<uint64_t>(), n, flag.as<uint64_t>() + n, s));
    uint64_t nb = 0;
    SPG_CUDA_TRY(cudaMemcpyAsync(&nb, flag.as<uint64_t>() + n, sizeof(uint64_t),
                                 cudaMemcpyDeviceToHost, s));
    SPG_CUDA_TRY(cudaStreamSynchronize(s));
    SpmvPlan p;
    SPG_TRY(p.items.alloc((nb + 1) * sizeof(uint64_t), s));
    stream_plan_scatter<<<grid_for(n, 256), 256, 0, s>>>(flag.as<uint64_t>(), n, p.items.as<uint64_t>());
    SPG_LAUNCH_CHECK();
    p.kind = SPG_SPMV_STREAM;
    p.n_items = nb;
    A->plan_stream = std::move(p);
    return SPG_OK;
}

static int build_merge_plan(Ctx *c, Csr *A, cudaStream_t s) {
    if (A->plan_merge.kind == SPG_SPMV_MERGE) return SPG_OK;
    const uint64_t total = A->n_rows + A->nnz;
    const uint64_t n_tiles = (total + MG_TILE - 1) / MG_TILE;
    SpmvPlan p;
    SPG_TRY(p.items.alloc(2 * (n_tiles + 1) * sizeof(uint64_t), s));
    SPG_TRY(p.aux.alloc((n_tiles ? n_tiles : 1) * sizeof(Carry), s));
    merge_tile_starts<<<grid_for(n_tiles + 1, 256), 256, 0, s>>>(A->d_off(), A->n_rows, A->nnz, n_tiles,
                                                                 p.items.as<uint64_t>());
    SPG_LAUNCH_CHECK();
    p.kind = SPG_SPMV_MERGE;
    p.n_items = n_tiles;
    A->plan_merge = std::move(p);
    (void)c;
    return SPG_OK;
}

namespace {
// reach[b] = largest column of the rows of block b, blocks [n b / nb, n (b+1) / nb)
__global__ void row_block_reach(const uint64_t *__restrict__ off, const uint32_t *__restrict__ cols, uint64_t n,
                                int nb, long long *__restrict__ reach) {
    for (uint64_t r = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; r < n; r += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t b0 = off[r], b1 = off[r + 1];
        if (b1 == b0) continue;
        int b = 0;
        while (b + 1 < nb && r >= n * (uint64_t)(b + 1) / (uint64_t)nb) ++b;
        atomicMax(reach + b, (long long)cols[b1 - 1]);  // columns ascend within a row
    }
}
}  // namespace

namespace {
__global__ void max_row_len(const uint64_t *__restrict__ off, uint64_t n, unsigned long long *__restrict__ mx) {
    unsigned long long m = 0;
    for (uint64_t r = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; r < n; r += (uint64_t)gridDim.x * blockDim.x)
        m = max(m, (unsigned long long)(off[r + 1] - off[r]));
#pragma unroll
    for (int o = 16; o; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
    __shared__ unsigned long long s_m[BLOCK / 32];
    if ((threadIdx.x & 31) == 0) s_m[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < BLOCK / 32; ++w) m = max(m, s_m[w]);
        atomicMax(mx, m);
    }
}

// Rows no longer than this count as balanced for SCALAR.
constexpr uint64_t SCALAR_BALANCED_ROW = 64;
}  // namespace

// The matrix's longest row, computed once per CSR (needs a synchronisation,
// so not while `s` is being captured: then `known` stays false).
int csr_max_row(Ctx *c, Csr *A, cudaStream_t s, bool *known) {
    *known = A->stats_valid;
    if (A->stats_valid) return SPG_OK;
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    SPG_CUDA_TRY(cudaStreamIsCapturing(s, &cs));
    if (cs != cudaStreamCaptureStatusNone) return SPG_OK;
    DevBuf mx;
    SPG_TRY(mx.alloc(sizeof(unsigned long long), s));
    SPG_CUDA_TRY(cudaMemsetAsync(mx.ptr, 0, sizeof(unsigned long long), s));
    if (A->n_rows) {
        max_row_len<<<grid_for(A->n_rows, BLOCK, (unsigned)c->n_sms * 8), BLOCK, 0, s>>>(
            A->d_off(), A->n_rows, mx.as<unsigned long long>());
        SPG_LAUNCH_CHECK();
    }
    unsigned long long h = 0;
    SPG_CUDA_TRY(cudaMemcpyAsync(&h, mx.ptr, sizeof(h), cudaMemcpyDeviceToHost, s));
    SPG_CUDA_TRY(cudaStreamSynchronize(s));
    A->max_row = h;
    A->stats_valid = true;
    *known = true;
    return SPG_OK;
}

// SCALAR's grid: on matrices whose rows are all short (balanced work per
// thread) one wave of blocks striding over the rows, which saves the block
// ramp and tail of a one-block-per-256-rows grid (2D Laplacian: 34.8 -> 33.6
// us); on others (a long row holds up its block) a block per 256 rows.
static unsigned scalar_grid(Ctx *c, Csr *A, uint64_t n, cudaStream_t s) {
    bool known = false;
    if (csr_max_row(c, A, s, &known) != SPG_OK) {
        cudaGetLastError();
        known = false;
    }
    const bool balanced = known && A->max_row <= SCALAR_BALANCED_ROW;
    return grid_for(n, BLOCK, balanced ? (unsigned)c->n_sms * 8 : (1u << 30));
}

int spmv_row_block_reach(Ctx *c, Csr *A, int nb, cudaStream_t s) {
    bool known = false;
    SPG_TRY(csr_max_row(c, A, s, &known));  // before any capture of the row blocks
    if ((int)A->host_reach.size() == nb) return SPG_OK;
    DevBuf d;
    SPG_TRY(d.alloc(nb * sizeof(long long), s));
    std::vector<long long> h(nb, -1);
    SPG_CUDA_TRY(cudaMemcpyAsync(d.ptr, h.data(), nb * sizeof(long long), cudaMemcpyHostToDevice, s));
    if (A->n_rows) {
        row_block_reach<<<grid_for(A->n_rows, BLOCK, (unsigned)c->n_sms * 8), BLOCK, 0, s>>>(
            A->d_off(), A->d_cols(), A->n_rows, nb, d.as<long long>());
        SPG_LAUNCH_CHECK();
    }
    SPG_CUDA_TRY(cudaMemcpyAsync(h.data(), d.ptr, nb * sizeof(long long), cudaMemcpyDeviceToHost, s));
    SPG_CUDA_TRY(cudaStreamSynchronize(s));
    A->host_reach.assign(h.begin(), h.end());
    return SPG_OK;
}

int spmv_launch_rows(Ctx *c, Csr *A, const double *x, double *y, int variant, uint64_t r0, uint64_t r1,
                     cudaStream_t s) {
    (void)c;
    if (r1 <= r0) return SPG_OK;
    const uint64_t n = r1 - r0;
    const uint64_t *off = A->d_off() + r0;  // offsets stay absolute positions in cols / vals
    const uint32_t *cols = A->d_cols();
    const double *vals = A->d_vals();
    double *yb = y + r0;
    switch (variant) {
        case SPG_SPMV_SCALAR:
            spmv_scalar<<<scalar_grid(c, A, n, s), BLOCK, 0, s>>>(off, cols, vals, x, yb, n);
            break;
#define SPG_VEC_CASE(ID, G)                                                                  \
    case ID:                                                                                 \
        spmv_vector<G><<<grid_for(n * G, BLOCK), BLOCK, 0, s>>>(off, cols, vals, x, yb, n);  \
        break;
        SPG_VEC_CASE(SPG_SPMV_VECTOR2, 2)
        SPG_VEC_CASE(SPG_SPMV_VECTOR4, 4)
        SPG_VEC_CASE(SPG_SPMV_VECTOR8, 8)
        SPG_VEC_CASE(SPG_SPMV_VECTOR16, 16)
        SPG_VEC_CASE(SPG_SPMV_VECTOR32, 32)
#undef SPG_VEC_CASE
        default:
            return SPG_ERR_UNSUPPORTED;
    }
    SPG_LAUNCH_CHECK();
    return SPG_OK;
}

int spmv_prepare(Ctx *c, Csr *A, int variant, cudaStream_t s) {
    switch (variant) {
        case SPG_SPMV_SCALAR: {  // the longest row picks SCALAR's grid
            bool known = false;
            return csr_max_row(c, A, s, &known);
        }
        case SPG_SPMV_STREAM:
            return build_stream_plan(c, A, s);
        case SPG_SPMV_MERGE:
            return build_merge_plan(c, A, s);
        default:
            return spmv_is_seg(variant) ? build_adaptive_plan(c, A, variant, s) : SPG_OK;
    }
}

int spmv_launch(Ctx *c, Csr *A, const double *x, double *y, int variant, cudaStream_t s) {
    const uint64_t n = A->n_rows;
    if (n == 0) return SPG_OK;
    const uint64_t *off = A->d_off();
    const uint32_t *cols = A->d_cols();
    const double *vals = A->d_vals();
    switch (variant) {
        case SPG_SPMV_SCALAR:
            spmv_scalar<<<scalar_grid(c, A, n, s), BLOCK, 0, s>>>(off, cols, vals, x, y, n);
            break;
#define SPG_VEC_CASE(ID, G)                                                                   \
    case ID:                                                                                  \
        spmv_vector<G><<<grid_for(n * G, BLOCK), BLOCK, 0, s>>>(off, cols, vals, x, y, n);    \
        break;
        SPG_VEC_CASE(SPG_SPMV_VECTOR2, 2)
        SPG_VEC_CASE(SPG_SPMV_VECTOR4, 4)
        SPG_VEC_CASE(SPG_SPMV_VECTOR8, 8)
        SPG_VEC_CASE(SPG_SPMV_VECTOR16, 16)
        SPG_VEC_CASE(SPG_SPMV_VECTOR32, 32)
#undef SPG_VEC_CASE
        case SPG_SPMV_STREAM: {
            SPG_TRY(build_stream_plan(c, A, s));
            const uint64_t nb = A->plan_stream.n_items;
            if (nb == 0) break;
            spmv_stream<<<(unsigned)nb, BLOCK, 0, s>>>(off, cols, vals, x, y,
                                                       A->plan_stream.items.as<uint64_t>());
            break;
        }
        case SPG_SPMV_MERGE: {
            SPG_TRY(build_merge_plan(c, A, s));
            const uint64_t nt = A->plan_merge.n_items;
            if (nt == 0) break;
            spmv_merge<<<(unsigned)nt, BLOCK, 0, s>>>(off, cols, vals, x, y, n,
                                                      A->plan_merge.items.as<uint64_t>(),
                                                      A->plan_merge.aux.as<Carry>());
            SPG_LAUNCH_CHECK();
            merge_fixup<<<grid_for(nt, 256), 256, 0, s>>>(A->plan_merge.aux.as<Carry>(), nt, n, y);
            break;
        }
        default:
            if (spmv_is_seg(variant)) return spmv_adaptive(c, A, x, y, variant, s);
            return set_error(SPG_ERR_INVALID_ARGUMENT, "spmv: unknown variant %d", variant);
    }
    SPG_LAUNCH_CHECK();
    return SPG_OK;
}

}  // namespace spg

// ---------------------------------------------------------------------------
// SpMV without any device allocation: the MERGE variant with its scratch (the
// tiles' merge-path starts and carry-outs) in a fixed array compiled into the
// library, for callers that must not allocate device memory.
// ---------------------------------------------------------------------------
namespace spg {
namespace {

constexpr uint64_t NOALLOC_MAX_TILES = 65536;  // rows + nonzeros <= 65536 * MG_TILE
constexpr size_t NOALLOC_STARTS_BYTES = 2 * (NOALLOC_MAX_TILES + 1) * sizeof(uint64_t);
constexpr size_t NOALLOC_BYTES = NOALLOC_STARTS_BYTES + NOALLOC_MAX_TILES * sizeof(Carry);

// Every device that loads libspg.so holds these ~2 MiB until the process exits.
static __device__ __align__(256) unsigned char g_spmv_noalloc_scratch[NOALLOC_BYTES];

constexpr int NOALLOC_MAX_DEVICES = 64;
// Per device, the array's device address. Host threads with their own
// contexts may look it up at the same time, hence atomics (they all store the
// same value).
std::atomic<void *> g_noalloc_addr[NOALLOC_MAX_DEVICES] = {};

int noalloc_lookup(int device, void **out) {
    void *p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_spmv_noalloc_scratch);
    if (e != cudaSuccess || !p)
        return set_error(SPG_ERR_CUDA, "spg_spmv_noalloc: cudaGetSymbolAddress failed: %s", cudaGetErrorString(e));
    g_noalloc_addr[device].store(p, std::memory_order_release);
    *out = p;
    return SPG_OK;
}

// Device address of the scratch array for `device` (the current device). The
// host-side symbol is only a stand-in and must never be handed to a kernel.
int noalloc_scratch(int device, void **out) {
    if (device < 0 || device >= NOALLOC_MAX_DEVICES)
        return set_error(SPG_ERR_UNSUPPORTED, "spg_spmv_noalloc: device %d beyond %d", device, NOALLOC_MAX_DEVICES);
    void *p = g_noalloc_addr[device].load(std::memory_order_acquire);
    if (p) {
        *out = p;
        return SPG_OK;
    }
    return noalloc_lookup(device, out);
}

}  // namespace

// Called by spg_ctx_create with `device` current: the address is looked up
// again for every new context, so a context created after cudaDeviceReset
// (which ends the CUDA context the cached address belonged to) sees the new
// one. Failures are left to the first spg_spmv_noalloc call to report.
void noalloc_refresh(int device) {
    if (device < 0 || device >= NOALLOC_MAX_DEVICES) return;
    void *p = nullptr;
    if (noalloc_lookup(device, &p) != SPG_OK) {
        g_noalloc_addr[device].store(nullptr, std::memory_order_release);
        clear_error();
    }
}

}  // namespace spg

extern "C" uint64_t spg_spmv_noalloc_max(void) { return spg::NOALLOC_MAX_TILES * (uint64_t)spg::MG_TILE; }

extern "C" int spg_spmv_noalloc(spg_ctx *c, const spg_csr *A, const double *d_x, double *d_y, void *stream) {
    using namespace spg;
    if (!c || !A) return set_error(SPG_ERR_INVALID_ARGUMENT, "spg_spmv_noalloc: null handle");
    SPG_CHECK_LIVE(A);
    if (!A->built) return set_error(SPG_ERR_LOGIC, "spmv: matrix must be locked");
    if ((A->n_cols && !d_x) || (A->n_rows && !d_y))
        return set_error(SPG_ERR_INVALID_ARGUMENT, "spg_spmv_noalloc: null vector");
    const uint64_t total = A->n_rows + A->nnz;
    if (total > spg_spmv_noalloc_max())
        return set_error(SPG_ERR_INVALID_ARGUMENT,
                         "spg_spmv_noalloc: rows + nonzeros = %llu exceeds the fixed scratch limit of %llu "
                         "(use spg_spmv)",
                         (unsigned long long)total, (unsigned long long)spg_spmv_noalloc_max());
    SPG_CUDA_TRY(cudaSetDevice(c->device));
    if (A->n_rows == 0) return SPG_OK;
    void *scratch = nullptr;
    SPG_TRY(noalloc_scratch(c->device, &scratch));
    uint64_t *starts = static_cast<uint64_t *>(scratch);
    Carry *carry = reinterpret_cast<Carry *>(static_cast<unsigned char *>(scratch) + NOALLOC_STARTS_BYTES);
    const uint64_t nt = (total + MG_TILE - 1) / MG_TILE;
    cudaStream_t s = pick_stream(c, stream);
    // Every call rewrites all tile starts and carries it reads, so nothing
    // left from an earlier call is used.
    merge_tile_starts<<<grid_for(nt + 1, 256), 256, 0, s>>>(A->d_off(), A->n_rows, A->nnz, nt, starts);
    SPG_LAUNCH_CHECK();
    spmv_merge<<<(unsigned)nt, BLOCK, 0, s>>>(A->d_off(), A->d_cols(), A->d_vals(), d_x, d_y, A->n_rows, starts, carry);
    SPG_LAUNCH_CHECK();
    merge_fixup<<<grid_for(nt, 256), 256, 0, s>>>(carry, nt, A->n_rows, d_y);
    SPG_LAUNCH_CHECK();
    return SPG_OK;
}
