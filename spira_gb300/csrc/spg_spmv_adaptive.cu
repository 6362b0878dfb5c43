// spg_spmv_adaptive.cu — SPG_SPMV_ADAPTIVE, the FP64 SpMV shaped for GB300.
//
// GB300 executes FP64 at 2 fused multiply-adds per clock per SM (ncu:
// sm__sass_thread_inst_executed_op_dfma_pred_on.peak_sustained = 2), so at
// ~12 B/nnz the FP64 pipe and HBM finish a SpMV in about the same time: any
// FP64 instruction beyond one FMA per nonzero, and any FP64 lane left idle by
// divergence, shows up directly in the runtime. This variant is built so that
// every nonzero costs one DFMA lane and nothing else:
//
//  * short rows (<= AD_LONG nnz) are cut into row-aligned tiles of at most
//    AD_BLOCK * ITEMS - ITEMS nnz. Thread t of a tile owns the 16-aligned
//    chunk of ITEMS consecutive nonzeros [a0 + ITEMS t, a0 + ITEMS (t+1)),
//    loads it with 16-byte vector loads (vals and cols are allocated to a
//    multiple of 16 entries, so an aligned chunk never leaves the
//    allocation), issues all its x gathers, then runs one FMA chain across
//    the chunk, closing a row whenever the row's end offset (staged in shared
//    memory) is passed. A row that straddles chunks is completed by the
//    thread that ends it, adding the straddled threads' tail partials in
//    thread order (rows are <= AD_LONG, so at most AD_LONG/ITEMS + 1 pieces);
//  * long rows (> AD_LONG nnz) get one warp each: every lane runs an FMA chain
//    over strided aligned chunks, then 5 shuffle additions.
// Both paths are deterministic. The tile list and the long-row list form the
// plan, built on the device once per lock and cached on the matrix.
#include "spg_internal.cuh"

namespace spg {
namespace {

constexpr int AD_BLOCK = 256;
constexpr uint64_t AD_LONG = 128;
constexpr int AD_ROWCAP = 1024;

template <int ITEMS>
struct AdGeom {
    static constexpr uint64_t BIN = (uint64_t)AD_BLOCK * ITEMS - ITEMS - AD_LONG;  // tile nnz <= BIN-1+AD_LONG
};

__device__ __forceinline__ double ldx(const double *__restrict__ x, uint32_t c) { return __ldg(x + c); }

// ---------------------------------------------------------------- plan
// brk[r]: row r starts a tile or is long; lng[r]: row r is long.
__global__ void ad_flags(const uint64_t *__restrict__ off, uint64_t n, uint64_t bin, uint64_t *__restrict__ brk,
                         uint64_t *__restrict__ lng) {
    const uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    const uint64_t o1 = off[r], o2 = off[r + 1];
    const bool L = (o2 - o1) > AD_LONG;
    bool b = L || r == 0 || (r % AD_ROWCAP) == 0;
    if (!b) {
        const uint64_t o0 = off[r - 1];
        b = (o1 - o0) > AD_LONG || (o0 / bin) != (o1 / bin);
    }
    brk[r] = b ? 1 : 0;
    lng[r] = L ? 1 : 0;
}

__global__ void ad_scatter(const uint64_t *__restrict__ bpos, const uint64_t *__restrict__ lpos, uint64_t n,
                           uint32_t *__restrict__ B, uint32_t *__restrict__ Lrows) {
    const uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    if (bpos[r + 1] != bpos[r]) B[bpos[r]] = (uint32_t)r;
    if (lpos[r + 1] != lpos[r]) Lrows[lpos[r]] = (uint32_t)r;
    if (r == n - 1) B[bpos[n]] = (uint32_t)n;
}

// tflag[j] = 1 iff break j starts a short tile.
__global__ void ad_tile_flags(const uint32_t *__restrict__ B, const uint64_t *__restrict__ lpos, uint64_t nb,
                              uint64_t *__restrict__ tflag) {
    const uint64_t j = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= nb) return;
    const uint32_t r = B[j];
    tflag[j] = (lpos[r + 1] == lpos[r]) ? 1 : 0;
}

__global__ void ad_tile_scatter(const uint32_t *__restrict__ B, const uint64_t *__restrict__ tpos, uint64_t nb,
                                uint2 *__restrict__ tiles) {
    const uint64_t j = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= nb) return;
    if (tpos[j + 1] != tpos[j]) tiles[tpos[j]] = make_uint2(B[j], B[j + 1]);
}

// ---------------------------------------------------------------- chunk loads
template <int ITEMS>
__device__ __forceinline__ void load_chunk(const uint32_t *__restrict__ cols, const double *__restrict__ vals,
                                           uint64_t ca, double (&v)[ITEMS], uint32_t (&c)[ITEMS]) {
#pragma unroll
    for (int u = 0; u < ITEMS; u += 2) {
        const double2 t = *reinterpret_cast<const double2 *>(vals + ca + u);
        v[u] = t.x;
        v[u + 1] = t.y;
    }
#pragma unroll
    for (int u = 0; u < ITEMS; u += 4) {
        const uint4 t = *reinterpret_cast<const uint4 *>(cols + ca + u);
        c[u] = t.x;
        c[u + 1] = t.y;
        c[u + 2] = t.z;
        c[u + 3] = t.w;
    }
}

// ---------------------------------------------------------------- short-row tiles
template <int ITEMS>
__global__ void __launch_bounds__(AD_BLOCK)
spmv_ad_tiles(const uint64_t *__restrict__ off, const uint32_t *__restrict__ cols, const double *__restrict__ vals,
              const double *__restrict__ x, double *__restrict__ y, const uint2 *__restrict__ tiles) {
    __shared__ uint32_t s_end[AD_ROWCAP];  // row end offsets relative to the tile's first nonzero
    __shared__ double s_tail[AD_BLOCK];
    __shared__ uint32_t s_tail_row[AD_BLOCK];
    const uint2 tl = tiles[blockIdx.x];
    const uint32_t r0 = tl.x, nr = tl.y - tl.x;
    const uint64_t k0 = off[r0], k1 = off[tl.y];
    for (uint32_t i = threadIdx.x; i < nr; i += AD_BLOCK) s_end[i] = (uint32_t)(off[r0 + i + 1] - k0);
    const uint64_t a0 = k0 & ~(uint64_t)(ITEMS - 1);
    const uint64_t ca = a0 + (uint64_t)ITEMS * threadIdx.x;
    const uint64_t lo = ca > k0 ? ca : k0;
    const uint64_t hi = (ca + ITEMS < k1) ? ca + ITEMS : k1;
    const bool has_items = lo < hi;
    double v[ITEMS];
    uint32_t c[ITEMS];
    if (has_items) load_chunk<ITEMS>(cols, vals, ca, v, c);
    __syncthreads();
    if (k1 == k0) {  // only empty rows
        for (uint32_t i = threadIdx.x; i < nr; i += AD_BLOCK) y[r0 + i] = 0.0;
        return;
    }
    uint32_t row = 0;
    bool head = false;
    double head_val = 0.0, acc = 0.0;
    uint32_t head_row = 0xFFFFFFFFu;
    if (has_items) {
        const uint32_t plo = (uint32_t)(lo - k0), phi = (uint32_t)(hi - k0);
        // first row this thread may close: the row containing item plo
        // (thread with the tile's first item starts at row 0 to close
        // leading empty rows).
        if (plo > 0) {
            uint32_t l = 0, h = nr - 1;  // smallest r with end > plo
            while (l < h) {
                const uint32_t m = (l + h) >> 1;
                if (s_end[m] > plo) h = m;
                else l = m + 1;
            }
            row = l;
            head = (row == 0 ? 0u : s_end[row - 1]) < plo;  // row started before this chunk
        }
        double g[ITEMS];
#pragma unroll
        for (int u = 0; u < ITEMS; ++u) {
            const uint64_t it = ca + u;
            g[u] = 0.0;
            if (it >= lo && it < hi) g[u] = ldx(x, c[u]);  // only in-tile columns are read
        }
        const uint32_t rfirst = row;
#pragma unroll
        for (int u = 0; u < ITEMS; ++u) {
            const uint64_t it = ca + u;
            if (it < lo || it >= hi) continue;
            const uint32_t p = (uint32_t)(it - k0);
            while (s_end[row] <= p) {  // row closes before item p
                if (head && row == rfirst) {
                    head_val = acc;
                    head_row = row;
                } else {
                    y[r0 + row] = acc;
                }
                acc = 0.0;
                ++row;
            }
            acc = fma(g[u], v[u], acc);
        }
        while (row < nr && s_end[row] <= phi) {  // rows ending at the chunk end (and empty rows there)
            if (head && row == rfirst) {
                head_val = acc;
                head_row = row;
            } else {
                y[r0 + row] = acc;
            }
            acc = 0.0;
            ++row;
        }
    }
    s_tail[threadIdx.x] = acc;
    s_tail_row[threadIdx.x] = (has_items && row < nr) ? row : 0xFFFFFFFFu;
    __syncthreads();
    if (head_row != 0xFFFFFFFFu) {
        int j = (int)threadIdx.x - 1;
        while (j >= 0 && s_tail_row[j] == head_row) --j;
        double s = 0.0;
        for (int q = j + 1; q < (int)threadIdx.x; ++q) s += s_tail[q];
        y[r0 + head_row] = s + head_val;
    }
}

// ---------------------------------------------------------------- long rows
template <int ITEMS>
__global__ void __launch_bounds__(AD_BLOCK)
spmv_ad_long(const uint64_t *__restrict__ off, const uint32_t *__restrict__ cols, const double *__restrict__ vals,
             const double *__restrict__ x, double *__restrict__ y, const uint32_t *__restrict__ rows,
             uint64_t n_long) {
    const uint64_t w = ((uint64_t)blockIdx.x * AD_BLOCK + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (w >= n_long) return;
    const uint32_t r = rows[w];
    const uint64_t b = off[r], e = off[r + 1];
    const uint64_t a0 = b & ~(uint64_t)(ITEMS - 1);
    double acc = 0.0;
    for (uint64_t ca = a0 + (uint64_t)ITEMS * lane; ca < e; ca += (uint64_t)ITEMS * 32) {
        double v[ITEMS];
        uint32_t c[ITEMS];
        load_chunk<ITEMS>(cols, vals, ca, v, c);
        double g[ITEMS];
#pragma unroll
        for (int u = 0; u < ITEMS; ++u) {
            const uint64_t it = ca + u;
            g[u] = 0.0;
            if (it >= b && it < e) g[u] = ldx(x, c[u]);  // only in-row columns are read
        }
#pragma unroll
        for (int u = 0; u < ITEMS; ++u) {
            const uint64_t it = ca + u;
            if (it >= b && it < e) acc = fma(g[u], v[u], acc);
        }
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) y[r] = acc;
}

}  // namespace

int build_adaptive_plan(Ctx *c, Csr *A, int items, cudaStream_t s) {
    if (A->plan_adaptive.kind == SPG_SPMV_ADAPTIVE * 100 + items) return SPG_OK;
    const uint64_t n = A->n_rows;
    const uint64_t bin = (items == 8) ? AdGeom<8>::BIN : AdGeom<16>::BIN;
    DevBuf brk, lng, B, L;
    SPG_TRY(brk.alloc((n + 1) * sizeof(uint64_t), s));
    SPG_TRY(lng.alloc((n + 1) * sizeof(uint64_t), s));
    ad_flags<<<grid_for(n, 256), 256, 0, s>>>(A->d_off(), n, bin, brk.as<uint64_t>(), lng.as<uint64_t>());
    SPG_LAUNCH_CHECK();
    SPG_TRY(exclusive_scan_u64(c, brk.as<uint64_t>(), n, brk.as<uint64_t>() + n, s));
    SPG_TRY(exclusive_scan_u64(c, lng.as<uint64_t>(), n, lng.as<uint64_t>() + n, s));
    uint64_t h[2];
    SPG_CUDA_TRY(cudaMemcpyAsync(&h[0], brk.as<uint64_t>() + n, 8, cudaMemcpyDeviceToHost, s));
    SPG_CUDA_TRY(cudaMemcpyAsync(&h[1], lng.as<uint64_t>() + n, 8, cudaMemcpyDeviceToHost, s));
    SPG_CUDA_TRY(cudaStreamSynchronize(s));
    const uint64_t nb = h[0], nl = h[1];
    SPG_TRY(B.alloc((nb + 1) * sizeof(uint32_t), s));
    SpmvPlan p;
    SPG_TRY(p.aux.alloc((nl ? nl : 1) * sizeof(uint32_t), s));
    ad_scatter<<<grid_for(n, 256), 256, 0, s>>>(brk.as<uint64_t>(), lng.as<uint64_t>(), n, B.as<uint32_t>(),
                                                 p.aux.as<uint32_t>());
    SPG_LAUNCH_CHECK();
    DevBuf tpos;
    SPG_TRY(tpos.alloc((nb + 1) * sizeof(uint64_t), s));
    ad_tile_flags<<<grid_for(nb, 256), 256, 0, s>>>(B.as<uint32_t>(), lng.as<uint64_t>(), nb, tpos.as<uint64_t>());
    SPG_LAUNCH_CHECK();
    SPG_TRY(exclusive_scan_u64(c, tpos.as<uint64_t>(), nb, tpos.as<uint64_t>() + nb, s));
    uint64_t nt = 0;
    SPG_CUDA_TRY(cudaMemcpyAsync(&nt, tpos.as<uint64_t>() + nb, 8, cudaMemcpyDeviceToHost, s));
    SPG_CUDA_TRY(cudaStreamSynchronize(s));
    SPG_TRY(p.items.alloc((nt ? nt : 1) * sizeof(uint2), s));
    ad_tile_scatter<<<grid_for(nb, 256), 256, 0, s>>>(B.as<uint32_t>(), tpos.as<uint64_t>(), nb,
                                                      p.items.as<uint2>());
    SPG_LAUNCH_CHECK();
    p.kind = SPG_SPMV_ADAPTIVE * 100 + items;
    p.n_items = nt;
    A->plan_adaptive = std::move(p);
    A->adaptive_long_rows = nl;
    return SPG_OK;
}

int spmv_adaptive(Ctx *c, Csr *A, const double *x, double *y, int items, cudaStream_t s) {
    SPG_TRY(build_adaptive_plan(c, A, items, s));
    const uint64_t nt = A->plan_adaptive.n_items, nl = A->adaptive_long_rows;
    const uint2 *tiles = A->plan_adaptive.items.as<uint2>();
    const uint32_t *lrows = A->plan_adaptive.aux.as<uint32_t>();
    if (items == 8) {
        if (nt) spmv_ad_tiles<8><<<(unsigned)nt, AD_BLOCK, 0, s>>>(A->d_off(), A->d_cols(), A->d_vals(), x, y, tiles);
        SPG_LAUNCH_CHECK();
        if (nl)
            spmv_ad_long<8><<<grid_for(nl * 32, AD_BLOCK), AD_BLOCK, 0, s>>>(A->d_off(), A->d_cols(), A->d_vals(), x, y,
                                                                            lrows, nl);
    } else {
        if (nt) spmv_ad_tiles<16><<<(unsigned)nt, AD_BLOCK, 0, s>>>(A->d_off(), A->d_cols(), A->d_vals(), x, y, tiles);
        SPG_LAUNCH_CHECK();
        if (nl)
            spmv_ad_long<16><<<grid_for(nl * 32, AD_BLOCK), AD_BLOCK, 0, s>>>(A->d_off(), A->d_cols(), A->d_vals(), x,
                                                                             y, lrows, nl);
    }
    SPG_LAUNCH_CHECK();
    return SPG_OK;
}

}  // namespace spg
