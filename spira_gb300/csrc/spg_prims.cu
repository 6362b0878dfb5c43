// spg_prims.cu — device-wide building blocks: exclusive scan (reduce-then-
// scan, recursive over tile sums) and a stable LSD radix sort of 64-bit keys
// with a 32-bit payload. The lock, transpose and SpGEMM paths are built on
// these; the stability of the sort is what carries Spira's "last write wins"
// and "ascending source row" orders onto the GPU.
#include "spg_internal.cuh"

namespace spg {

// ---------------------------------------------------------------------------
// Device buffers
// ---------------------------------------------------------------------------
int DevBuf::alloc(size_t n, cudaStream_t s) {
    release();
    stream = s;
    bytes = n;
    if (n == 0) return SPG_OK;
    cudaError_t e = cudaMallocAsync(&ptr, n, s);
    if (e != cudaSuccess) {
        cudaGetLastError();
        ptr = nullptr;
        bytes = 0;
        return set_error(e == cudaErrorMemoryAllocation ? SPG_ERR_NO_MEMORY : SPG_ERR_CUDA,
                         "device allocation of %zu bytes failed: %s", n, cudaGetErrorString(e));
    }
    return SPG_OK;
}

void DevBuf::release() {
    if (ptr) cudaFreeAsync(ptr, stream);
    ptr = nullptr;
    bytes = 0;
}

// ---------------------------------------------------------------------------
// Exclusive scan
// ---------------------------------------------------------------------------
namespace {

constexpr int SCAN_BLOCK = 256;
constexpr int SCAN_ITEMS = 8;
constexpr int SCAN_TILE = SCAN_BLOCK * SCAN_ITEMS;

template <typename T>
__device__ __forceinline__ T warp_inclusive_scan(T v) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        T o = __shfl_up_sync(0xffffffffu, v, d);
        if (lane >= d) v += o;
    }
    return v;
}

// Block-wide exclusive scan of one value per thread; returns the exclusive
// prefix and the block total.
template <typename T>
__device__ __forceinline__ T block_exclusive_scan(T v, T &total) {
    constexpr int NW = SCAN_BLOCK / 32;
    __shared__ T warp_tot[NW];
    __shared__ T block_total;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    T inc = warp_inclusive_scan(v);
    if (lane == 31) warp_tot[warp] = inc;
    __syncthreads();
    if (warp == 0) {
        T w = (lane < NW) ? warp_tot[lane] : T(0);
        T wi = warp_inclusive_scan(w);
        if (lane < NW) warp_tot[lane] = wi - w;
        if (lane == NW - 1) block_total = wi;
    }
    __syncthreads();
    T res = warp_tot[warp] + inc - v;
    total = block_total;
    __syncthreads();
    return res;
}

template <typename T>
__global__ void scan_tile_reduce(const T *__restrict__ d, uint64_t n, T *__restrict__ tile_sums) {
    const uint64_t base = (uint64_t)blockIdx.x * SCAN_TILE;
    T s = 0;
#pragma unroll
    for (int i = 0; i < SCAN_ITEMS; ++i) {
        uint64_t k = base + (uint64_t)i * SCAN_BLOCK + threadIdx.x;
        if (k < n) s += d[k];
    }
    T total;
    block_exclusive_scan(s, total);
    if (threadIdx.x == 0) tile_sums[blockIdx.x] = total;
}

// Scan each tile (blocked arrangement: thread t owns items t*ITEMS..), adding
// the tile's exclusive prefix. Loads go through shared memory to stay
// coalesced; the shared tile is padded by one element every 16 so the
// blocked reads and writes (thread stride ITEMS) do not pile onto a few banks.
__device__ __forceinline__ int scan_pad(int j) { return j + (j >> 4); }

template <typename T>
__global__ void scan_tile_apply(T *__restrict__ d, uint64_t n, const T *__restrict__ tile_prefix,
                                T *__restrict__ d_total) {
    __shared__ T tile[SCAN_TILE + SCAN_TILE / 16];
    const uint64_t base = (uint64_t)blockIdx.x * SCAN_TILE;
#pragma unroll
    for (int i = 0; i < SCAN_ITEMS; ++i) {
        int j = i * SCAN_BLOCK + threadIdx.x;
        uint64_t k = base + j;
        tile[scan_pad(j)] = (k < n) ? d[k] : T(0);
    }
    __syncthreads();
    T v[SCAN_ITEMS];
    T s = 0;
#pragma unroll
    for (int i = 0; i < SCAN_ITEMS; ++i) {
        v[i] = tile[scan_pad(threadIdx.x * SCAN_ITEMS + i)];
        s += v[i];
    }
    T total;
    T pre = block_exclusive_scan(s, total) + (tile_prefix ? tile_prefix[blockIdx.x] : T(0));
#pragma unroll
    for (int i = 0; i < SCAN_ITEMS; ++i) {
        tile[scan_pad(threadIdx.x * SCAN_ITEMS + i)] = pre;
        pre += v[i];
    }
    __syncthreads();
#pragma unroll
    for (int i = 0; i < SCAN_ITEMS; ++i) {
        int j = i * SCAN_BLOCK + threadIdx.x;
        uint64_t k = base + j;
        if (k < n) d[k] = tile[scan_pad(j)];
    }
    if (d_total && blockIdx.x == gridDim.x - 1 && threadIdx.x == SCAN_BLOCK - 1) {
        // last thread of last tile: its running prefix after all items
        *d_total = pre;
    }
}

template <typename T>
int exclusive_scan_impl(Ctx *c, T *d, uint64_t n, T *d_total, cudaStream_t s) {
    if (n == 0) {
        if (d_total) SPG_CUDA_TRY(cudaMemsetAsync(d_total, 0, sizeof(T), s));
        return SPG_OK;
    }
    const uint64_t tiles = (n + SCAN_TILE - 1) / SCAN_TILE;
    if (tiles == 1) {
        scan_tile_apply<T><<<1, SCAN_BLOCK, 0, s>>>(d, n, nullptr, d_total);
        SPG_LAUNCH_CHECK();
        return SPG_OK;
    }
    DevBuf sums;
    SPG_TRY(sums.alloc(tiles * sizeof(T), s));
    scan_tile_reduce<T><<<(unsigned)tiles, SCAN_BLOCK, 0, s>>>(d, n, sums.as<T>());
    SPG_LAUNCH_CHECK();
    SPG_TRY(exclusive_scan_impl<T>(c, sums.as<T>(), tiles, nullptr, s));
    scan_tile_apply<T><<<(unsigned)tiles, SCAN_BLOCK, 0, s>>>(d, n, sums.as<T>(), d_total);
    SPG_LAUNCH_CHECK();
    return SPG_OK;
}

}  // namespace

int exclusive_scan_u64(Ctx *c, uint64_t *d, uint64_t n, uint64_t *d_total, cudaStream_t s) {
    return exclusive_scan_impl<unsigned long long>(c, reinterpret_cast<unsigned long long *>(d), n,
                                                   reinterpret_cast<unsigned long long *>(d_total), s);
}

int exclusive_scan_i64(Ctx *c, int64_t *d, uint64_t n, cudaStream_t s) {
    return exclusive_scan_impl<long long>(c, reinterpret_cast<long long *>(d), n, nullptr, s);
}

// ---------------------------------------------------------------------------
// Stable LSD radix sort (8-bit digits, reduce-then-scan per pass)
//
// Tile of 4096 keys = 8 warps x 16 iterations x 32 lanes. Warp w owns keys
// [w*512, w*512+512) of the tile and walks them in order (iteration-major,
// lane-minor), so the within-tile rank of every key is its order among equal
// digits: stability follows, and with it the insertion-order tie-break.
// The upsweep counts digits with shared-memory atomics; the scatter ranks
// equal digits within a warp with ballots. The scatter first places the tile in shared memory in digit order, then
// writes each digit's run to its global position with consecutive threads
// on consecutive addresses, so the writes coalesce.
// ---------------------------------------------------------------------------
namespace {

constexpr int RS_WARPS = 8;
constexpr int RS_BLOCK = RS_WARPS * 32;
constexpr int RS_RADIX = 256;
// Keys per thread: 16 (tiles of 4096) for large sorts; small sorts use
// shorter tiles so that enough blocks run.

__device__ __forceinline__ unsigned lanemask_lt() {
    unsigned m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

template <int RS_ITERS>
__global__ void __launch_bounds__(RS_BLOCK)
radix_upsweep(const uint64_t *__restrict__ keys, uint64_t n, int shift, unsigned n_tiles,
              unsigned *__restrict__ hist /* [RADIX][n_tiles] */) {
    constexpr int RS_TILE = RS_BLOCK * RS_ITERS;
    __shared__ unsigned cnt[RS_WARPS][RS_RADIX];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int i = threadIdx.x; i < RS_WARPS * RS_RADIX; i += RS_BLOCK) (&cnt[0][0])[i] = 0;
    __syncthreads();
    const uint64_t base = (uint64_t)blockIdx.x * RS_TILE + (uint64_t)warp * (RS_ITERS * 32);
    unsigned dig[RS_ITERS];
#pragma unroll
    for (int j = 0; j < RS_ITERS; ++j) {
        const uint64_t k = base + j * 32 + lane;
        dig[j] = (k < n) ? (unsigned)((keys[k] >> shift) & 0xFF) : RS_RADIX;
    }
    // counts only: shared-memory atomics, with one add for a warp whose 32
    // digits agree (sorted or skewed inputs would otherwise serialise)
#pragma unroll
    for (int j = 0; j < RS_ITERS; ++j) {
        const unsigned d = dig[j];
        const unsigned d0 = __shfl_sync(0xffffffffu, d, 0);
        if (__all_sync(0xffffffffu, d == d0)) {
            if (lane == 0 && d0 < RS_RADIX) cnt[warp][d0] += 32;
        } else if (d < RS_RADIX) {
            atomicAdd(&cnt[warp][d], 1u);
        }
        __syncwarp();
    }
    __syncthreads();
    for (int d = threadIdx.x; d < RS_RADIX; d += RS_BLOCK) {
        unsigned s = 0;
#pragma unroll
        for (int w = 0; w < RS_WARPS; ++w) s += cnt[w][d];
        hist[(uint64_t)d * n_tiles + blockIdx.x] = s;
    }
}

// Shared memory of radix_scatter (dynamic: above the 48 KB static limit).
template <int RS_TILE>
struct ScatterSmem {
    uint64_t key[RS_TILE];
    uint32_t val[RS_TILE];
    unsigned long long gbase[RS_RADIX];  // global start of each digit's run of this tile
    unsigned cnt[RS_WARPS][RS_RADIX];    // per-warp digit counts, then per-warp offsets
    unsigned loc[RS_RADIX];              // tile-local start of each digit's run
    unsigned wsum[RS_WARPS];
};

static_assert(RS_BLOCK == RS_RADIX, "one thread per digit in the tile-local scan");

template <int RS_ITERS>
__global__ void __launch_bounds__(RS_BLOCK)
radix_scatter(const uint64_t *__restrict__ keys_in, const uint32_t *__restrict__ vals_in,
              uint64_t *__restrict__ keys_out, uint32_t *__restrict__ vals_out, uint64_t n,
              int shift, unsigned n_tiles, const unsigned long long *__restrict__ offs /* scanned */) {
    constexpr int RS_TILE = RS_BLOCK * RS_ITERS;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    ScatterSmem<RS_TILE> &S = *reinterpret_cast<ScatterSmem<RS_TILE> *>(smem_raw);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int t = threadIdx.x;
    for (int i = t; i < RS_WARPS * RS_RADIX; i += RS_BLOCK) (&S.cnt[0][0])[i] = 0;
    S.gbase[t] = offs[(uint64_t)t * n_tiles + blockIdx.x];
    __syncthreads();

    const uint64_t tile0 = (uint64_t)blockIdx.x * RS_TILE;
    const uint64_t base = tile0 + (uint64_t)warp * (RS_ITERS * 32);
    uint64_t key[RS_ITERS];
    unsigned rank[RS_ITERS];
#pragma unroll
    for (int j = 0; j < RS_ITERS; ++j) {
        const uint64_t k = base + j * 32 + lane;
        key[j] = (k < n) ? keys_in[k] : 0;
    }
    // rank of each key among the equal digits before it in the warp's order
#pragma unroll
    for (int j = 0; j < RS_ITERS; ++j) {
        const uint64_t k = base + j * 32 + lane;
        const bool ok = k < n;
        const unsigned valid = __ballot_sync(0xffffffffu, ok);
        rank[j] = 0;
        if (!valid) continue;
        const unsigned d = ok ? (unsigned)((key[j] >> shift) & 0xFF) : RS_RADIX;
        const unsigned peers = warp_match_digit(d) & valid;
        unsigned before = 0;
        if (ok) before = S.cnt[warp][d];
        __syncwarp();
        rank[j] = before + __popc(peers & lanemask_lt());
        if (ok && (peers & lanemask_lt()) == 0) S.cnt[warp][d] = before + __popc(peers);
        __syncwarp();
    }
    __syncthreads();
    // digit t: exclusive prefix over warps (warp order = key order), then an
    // exclusive scan of the tile's digit totals
    unsigned tot = 0;
#pragma unroll
    for (int w = 0; w < RS_WARPS; ++w) {
        const unsigned c = S.cnt[w][t];
        S.cnt[w][t] = tot;
        tot += c;
    }
    unsigned inc = tot;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned v = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += v;
    }
    if (lane == 31) S.wsum[warp] = inc;
    __syncthreads();
    unsigned wpre = 0;
    for (int w = 0; w < warp; ++w) wpre += S.wsum[w];
    S.loc[t] = wpre + inc - tot;
    __syncthreads();
    // place the tile in digit order in shared memory
#pragma unroll
    for (int j = 0; j < RS_ITERS; ++j) {
        const uint64_t k = base + j * 32 + lane;
        if (k < n) {
            const unsigned d = (unsigned)((key[j] >> shift) & 0xFF);
            const unsigned p = S.loc[d] + S.cnt[warp][d] + rank[j];
            S.key[p] = key[j];
            S.val[p] = vals_in[k];
        }
    }
    __syncthreads();
    // write each digit's run to its global position: consecutive threads,
    // consecutive addresses
    const unsigned tile_n = (unsigned)min((uint64_t)RS_TILE, n - tile0);
    for (unsigned i = t; i < tile_n; i += RS_BLOCK) {
        const uint64_t kk = S.key[i];
        const unsigned d = (unsigned)((kk >> shift) & 0xFF);
        const unsigned long long pos = S.gbase[d] + (i - S.loc[d]);
        keys_out[pos] = kk;
        vals_out[pos] = S.val[i];
    }
}

__global__ void scan_u32_to_u64_copy(const unsigned *in, unsigned long long *out, uint64_t n) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x)
        out[i] = in[i];
}

}  // namespace

namespace {

template <int RS_ITERS>
int radix_sort_impl(Ctx *c, uint64_t *d_keys, uint32_t *d_vals, uint64_t n, int key_bits, cudaStream_t s) {
    constexpr int RS_TILE = RS_BLOCK * RS_ITERS;
    const unsigned n_tiles = (unsigned)((n + RS_TILE - 1) / RS_TILE);
    const uint64_t hist_n = (uint64_t)RS_RADIX * n_tiles;
    DevBuf kalt, valt, hist, offs;
    SPG_TRY(kalt.alloc(n * sizeof(uint64_t), s));
    SPG_TRY(valt.alloc(n * sizeof(uint32_t), s));
    SPG_TRY(hist.alloc(hist_n * sizeof(unsigned), s));
    SPG_TRY(offs.alloc(hist_n * sizeof(unsigned long long), s));
    uint64_t *kin = d_keys, *kout = kalt.as<uint64_t>();
    uint32_t *vin = d_vals, *vout = valt.as<uint32_t>();
    const int passes = (key_bits + 7) / 8;
    constexpr size_t smem = sizeof(ScatterSmem<RS_TILE>);
    SPG_CUDA_TRY(cudaFuncSetAttribute(radix_scatter<RS_ITERS>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)smem));
    for (int p = 0; p < passes; ++p) {
        const int shift = p * 8;
        radix_upsweep<RS_ITERS><<<n_tiles, RS_BLOCK, 0, s>>>(kin, n, shift, n_tiles, hist.as<unsigned>());
        SPG_LAUNCH_CHECK();
        scan_u32_to_u64_copy<<<grid_for(hist_n, 256, 4096), 256, 0, s>>>(
            hist.as<unsigned>(), offs.as<unsigned long long>(), hist_n);
        SPG_LAUNCH_CHECK();
        SPG_TRY(exclusive_scan_u64(c, offs.as<uint64_t>(), hist_n, nullptr, s));
        radix_scatter<RS_ITERS><<<n_tiles, RS_BLOCK, smem, s>>>(kin, vin, kout, vout, n, shift, n_tiles,
                                                                offs.as<unsigned long long>());
        SPG_LAUNCH_CHECK();
        std::swap(kin, kout);
        std::swap(vin, vout);
    }
    if (kin != d_keys) {
        SPG_CUDA_TRY(cudaMemcpyAsync(d_keys, kin, n * sizeof(uint64_t), cudaMemcpyDeviceToDevice, s));
        SPG_CUDA_TRY(cudaMemcpyAsync(d_vals, vin, n * sizeof(uint32_t), cudaMemcpyDeviceToDevice, s));
    }
    return SPG_OK;
}

}  // namespace

int radix_sort_pairs_u64(Ctx *c, uint64_t *d_keys, uint32_t *d_vals, uint64_t n, int key_bits,
                         cudaStream_t s) {
    if (n <= 1 || key_bits <= 0) return SPG_OK;
    if (n >= (1ull << 32))
        return set_error(SPG_ERR_UNSUPPORTED, "radix sort of %llu keys exceeds 2^32-1",
                         (unsigned long long)n);
    // at least ~4 tiles per SM
    const uint64_t want = 4ull * (uint64_t)c->n_sms;
    if (n >= want * RS_BLOCK * 16) return radix_sort_impl<16>(c, d_keys, d_vals, n, key_bits, s);
    if (n >= want * RS_BLOCK * 4) return radix_sort_impl<4>(c, d_keys, d_vals, n, key_bits, s);
    return radix_sort_impl<1>(c, d_keys, d_vals, n, key_bits, s);
}

// ---------------------------------------------------------------------------
// Row-grouped sort: pairs (row, col) whose rows are already non-decreasing
// (rows[i] <= rows[i+1]) are put in stable (row, col) order by sorting each
// row's entries by column in shared memory, tile by tile. Tile t holds the
// rows whose first entry lies in [t*TS_SPAN, (t+1)*TS_SPAN): its entries
// [start_t, start_{t+1}) are contiguous and already in row order, so sorting
// inside the tile by (row, column), stably, puts them in their final global
// places. The sort is an LSD radix sort (8-bit digits) of 32-bit composite
// keys (row - first row of the tile, column) with 16-bit tile indices,
// ping-ponged in shared memory. Warp w owns positions [512 w, 512 w + 512) of
// every pass (16 warps of 256 measured slower); each scatter also counts, per
// destination slice, the digit of the next pass, so a pass is one sweep.
// Tiles of at most TS_SMALL entries (three blocks per SM) and tiles of up to
// TS_MAX (one holding a long row; one block per SM) run as two launches over
// a tile plan. A tile longer than
// TS_MAX (a row of more than ~10 000 entries) or whose key needs more than 32
// bits makes the sort report failure; callers then sort globally.
// ---------------------------------------------------------------------------
namespace {

constexpr int TS_SPAN = 2048;
constexpr int TS_SMALL = 4096, TS_SLICE_SMALL = 512;  // 8 warps
constexpr int TS_MAX = 12288, TS_SLICE_LARGE = 512;   // 24 warps

template <int MAXE, int SLICE>
struct TileSortSmem {
    uint32_t key[2][MAXE];
    uint16_t idx[2][MAXE];
    unsigned cnt[2][MAXE / SLICE][256];
    unsigned wsum[8];
};

__device__ __forceinline__ uint64_t first_row_at_or_after(const uint64_t *__restrict__ s_off, uint64_t n,
                                                          uint64_t pos) {
    uint64_t lo = 0, hi = n;  // first r in [0, n] with s_off[r] >= pos
    while (lo < hi) {
        const uint64_t mid = (lo + hi) >> 1;
        if (s_off[mid] < pos) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

// First row of every tile (entry n_tiles: n_rows), and the tiles sorted into
// a list of small ones (<= TS_SMALL entries) and a list of large ones (<=
// TS_MAX); *overflow = 1 if a tile is longer. List order does not matter: the
// tiles are independent.
__global__ void tile_plan(const uint64_t *__restrict__ s_off, uint64_t n_rows, uint64_t n_tiles,
                          uint64_t *__restrict__ tile_r0, unsigned *__restrict__ small_list,
                          unsigned *__restrict__ large_list, unsigned *__restrict__ counts /* [2] */,
                          unsigned *__restrict__ overflow) {
    const uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (t > n_tiles) return;
    const uint64_t r0 = t == n_tiles ? n_rows : first_row_at_or_after(s_off, n_rows, t * TS_SPAN);
    tile_r0[t] = r0;
    if (t == n_tiles) return;
    const uint64_t r1 = first_row_at_or_after(s_off, n_rows, (t + 1) * TS_SPAN);
    const uint64_t E = s_off[r1] - s_off[r0];
    if (E == 0) return;
    if (E <= (uint64_t)TS_SMALL) small_list[atomicAdd(counts, 1u)] = (unsigned)t;
    else if (E <= (uint64_t)TS_MAX) large_list[atomicAdd(counts + 1, 1u)] = (unsigned)t;
    else *overflow = 1u;
}

// Sorts the tiles of `list` (each of at most MAXE entries); one warp per
// TS_SLICE entries.
template <int MAXE, int TS_SLICE>
__global__ void __launch_bounds__(MAXE / TS_SLICE * 32)
grouped_tile_sort(const uint32_t *__restrict__ rows, const uint32_t *__restrict__ cols,
                  const uint64_t *__restrict__ s_off, const uint64_t *__restrict__ tile_r0,
                  const unsigned *__restrict__ list, int cbits, uint64_t *__restrict__ keys_out,
                  uint32_t *__restrict__ idx_out, unsigned *__restrict__ overflow) {
    constexpr int W = MAXE / TS_SLICE, T = W * 32;
    extern __shared__ __align__(16) unsigned char ts_raw[];
    TileSortSmem<MAXE, TS_SLICE> &S = *reinterpret_cast<TileSortSmem<MAXE, TS_SLICE> *>(ts_raw);
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    const unsigned tile = list[blockIdx.x];
    const uint64_t r0 = tile_r0[tile], r1 = tile_r0[tile + 1];
    const uint64_t start = s_off[r0], end = s_off[r1];
    const uint64_t E64 = end - start;
    if (E64 == 0 || E64 > (uint64_t)MAXE) return;  // (the plan never lists such tiles)
    const int E = (int)E64;
    const unsigned span = (unsigned)(r1 - r0 - 1);  // largest row offset inside the tile
    const int bits = (span ? 32 - __clz(span) : 0) + cbits;
    if (bits > 32 || cbits >= 32) {
        if (t == 0) *overflow = 1u;
        return;
    }
    const int passes = (bits + 7) / 8;
    for (int e = t; e < E; e += T) {
        S.key[0][e] = ((rows[start + e] - (uint32_t)r0) << cbits) | cols[start + e];
        S.idx[0][e] = (uint16_t)e;
    }
    for (int i = t; i < 2 * W * 256; i += T) (&S.cnt[0][0][0])[i] = 0;
    __syncthreads();
    const int q0 = warp * TS_SLICE, q1 = min(E, q0 + TS_SLICE);
    // digit counts of the first pass, per warp slice
    for (int q = q0; q < q1 && passes > 0; q += 32) {
        const int qq = q + lane;
        const bool ok = qq < q1;
        const unsigned valid = __ballot_sync(0xffffffffu, ok);
        const unsigned d = ok ? (S.key[0][qq] & 0xFFu) : 0u;
        const unsigned peers = warp_match_digit<8>(d) & valid;
        if (ok && (peers & lanemask_lt()) == 0) S.cnt[0][warp][d] += __popc(peers);
        __syncwarp();
    }
    __syncthreads();
    int cur = 0;
    for (int p = 0; p < passes; ++p) {
        const int c = p & 1, shift = 8 * p;
        // digit t: start of each warp slice's run, then across digits
        unsigned excl = 0;
        if (t < 256) {
            unsigned tot = 0;
            for (int w = 0; w < W; ++w) {
                const unsigned v = S.cnt[c][w][t];
                S.cnt[c][w][t] = tot;
                tot += v;
            }
            unsigned inc = tot;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const unsigned v = __shfl_up_sync(0xffffffffu, inc, o);
                if (lane >= o) inc += v;
            }
            if (lane == 31) S.wsum[warp] = inc;
            excl = inc - tot;
        }
        for (int i = t; i < W * 256; i += T) (&S.cnt[c ^ 1][0][0])[i] = 0;  // next pass's counts
        __syncthreads();
        if (t < 256) {
            unsigned pre = 0;
            for (int w = 0; w < warp; ++w) pre += S.wsum[w];
            const unsigned base = excl + pre;
            for (int w = 0; w < W; ++w) S.cnt[c][w][t] += base;
        }
        __syncthreads();
        // stable scatter; count the next pass's digits per destination slice
        for (int q = q0; q < q1; q += 32) {
            const int qq = q + lane;
            const bool ok = qq < q1;
            const unsigned valid = __ballot_sync(0xffffffffu, ok);
            const uint32_t k = ok ? S.key[cur][qq] : 0u;
            const unsigned d = (k >> shift) & 0xFFu;
            const unsigned peers = warp_match_digit<8>(d) & valid;
            unsigned before = 0;
            if (ok) before = S.cnt[c][warp][d];
            __syncwarp();
            if (ok) {
                const unsigned lt = peers & lanemask_lt();
                const unsigned pos = before + __popc(lt);
                S.key[cur ^ 1][pos] = k;
                S.idx[cur ^ 1][pos] = S.idx[cur][qq];
                if (lt == 0) S.cnt[c][warp][d] = before + __popc(peers);
                if (p + 1 < passes) atomicAdd(&S.cnt[c ^ 1][pos / TS_SLICE][(k >> (shift + 8)) & 0xFFu], 1u);
            }
            __syncwarp();
        }
        __syncthreads();
        cur ^= 1;
    }
    for (int q = t; q < E; q += T) {
        keys_out[start + q] = ((uint64_t)r0 << cbits) + S.key[cur][q];
        idx_out[start + q] = (uint32_t)(start + S.idx[cur][q]);
    }
}

}  // namespace

int sort_grouped_rows(Ctx *c, const uint32_t *rows, const uint32_t *cols, const uint64_t *s_off, uint64_t m,
                      uint64_t n_rows, int cbits, uint64_t *keys_out, uint32_t *idx_out, bool *done, cudaStream_t s) {
    *done = false;
    if (m == 0) {
        *done = true;
        return SPG_OK;
    }
    const uint64_t n_tiles = (m + TS_SPAN - 1) / TS_SPAN;
    DevBuf tile_r0, lists, flags;
    SPG_TRY(tile_r0.alloc((n_tiles + 1) * sizeof(uint64_t), s));
    SPG_TRY(lists.alloc(2 * n_tiles * sizeof(unsigned), s));
    SPG_TRY(flags.alloc(3 * sizeof(unsigned), s));  // overflow, small tiles, large tiles
    SPG_CUDA_TRY(cudaMemsetAsync(flags.ptr, 0, 3 * sizeof(unsigned), s));
    unsigned *small_list = lists.as<unsigned>(), *large_list = small_list + n_tiles;
    unsigned *overflow = flags.as<unsigned>();
    tile_plan<<<grid_for(n_tiles + 1, 256), 256, 0, s>>>(s_off, n_rows, n_tiles, tile_r0.as<uint64_t>(), small_list,
                                                        large_list, overflow + 1, overflow);
    SPG_LAUNCH_CHECK();
    unsigned h[3] = {1u, 0u, 0u};
    SPG_CUDA_TRY(cudaMemcpyAsync(h, overflow, 3 * sizeof(unsigned), cudaMemcpyDeviceToHost, s));
    SPG_TRY(c->phase_sync(s));
    if (h[0]) return SPG_OK;
    constexpr size_t small_smem = sizeof(TileSortSmem<TS_SMALL, TS_SLICE_SMALL>);
    constexpr size_t large_smem = sizeof(TileSortSmem<TS_MAX, TS_SLICE_LARGE>);
    constexpr unsigned small_threads = TS_SMALL / TS_SLICE_SMALL * 32;
    constexpr unsigned large_threads = TS_MAX / TS_SLICE_LARGE * 32;
    auto small_k = grouped_tile_sort<TS_SMALL, TS_SLICE_SMALL>;
    auto large_k = grouped_tile_sort<TS_MAX, TS_SLICE_LARGE>;
    SPG_CUDA_TRY(cudaFuncSetAttribute(small_k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)small_smem));
    SPG_CUDA_TRY(cudaFuncSetAttribute(large_k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)large_smem));
    if (h[1]) {
        small_k<<<h[1], small_threads, small_smem, s>>>(rows, cols, s_off, tile_r0.as<uint64_t>(), small_list, cbits,
                                                        keys_out, idx_out, overflow);
        SPG_LAUNCH_CHECK();
    }
    if (h[2]) {
        large_k<<<h[2], large_threads, large_smem, s>>>(rows, cols, s_off, tile_r0.as<uint64_t>(), large_list, cbits,
                                                        keys_out, idx_out, overflow);
        SPG_LAUNCH_CHECK();
    }
    SPG_CUDA_TRY(cudaMemcpyAsync(h, overflow, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
    SPG_TRY(c->phase_sync(s));
    *done = h[0] == 0;
    return SPG_OK;
}

}  // namespace spg
