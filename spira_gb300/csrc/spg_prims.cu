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
// (rows[i] <= rows[i+1], so row r's entries are [s_off[r], s_off[r+1])) are
// put in stable (row, col) order by sorting every row by column on its own.
// Rows are sorted by length class:
//   * one entry: written through by the planning pass;
//   * 2..32 entries: a bitonic network in registers, 32 / P rows of padded
//     length P (2, 4, 8, 16, 32) per warp, keys (col << 5 | position), so the
//     network's order is the stable order;
//   * 33..SEG_SPAN entries: grouped by the span of SEG_SPAN input positions
//     their first entry lies in (at most 63 such rows start in one span, as
//     they lie 33 or more positions apart; together < 2 SEG_SPAN entries) and
//     sorted tile by tile in shared memory: an LSD radix sort (8-bit digits)
//     of 32-bit keys (rank of the row in the tile, col) with 16-bit tile
//     positions, ping-ponged in shared memory; warp w owns positions
//     [512 w, 512 w + 512) of every pass, and each scatter also counts, per
//     destination slice, the digit of the next pass, so a pass is one sweep;
//   * SEG_SPAN+1..TS_MAX entries: a tile of its own, sorted the same way (no
//     rank bits: ceil(cbits / 8) passes); rows up to TS_SMALL entries in the
//     kernel of the span tiles (three blocks per SM), longer ones in a kernel
//     of one block per SM.
// A tile's key needs rank bits (at most 6) + cbits <= 32, so columns of more
// than 26 bits, and a row longer than TS_MAX, make the sort report failure;
// callers then sort globally. Work lists are filled with atomics, in no
// particular order: every row's output places are fixed by s_off, so the
// result does not depend on that order.
// ---------------------------------------------------------------------------
namespace {

constexpr int SEG_SPAN = 2048;
constexpr int SEG_TILE_ROWS = 64;  // medium rows starting in one span: at most 63
constexpr int TS_SMALL = 4096, TS_SLICE_SMALL = 512;  // 8 warps; a span's medium rows: < 2 SEG_SPAN
constexpr int TS_MAX = 12288, TS_SLICE_LARGE = 512;   // 24 warps
constexpr int SEG_MAX_CBITS = 26;
constexpr uint64_t SEG_ROW_JOB = 1ull << 63;  // large job naming one row (else a span tile)

// counters (unsigned) of the plan
enum : int {
    SC_SHORT = 0,       // [1..5]: rows of padded length 2^c
    SC_SMALL = 6,       // small jobs: span tiles, rows of SEG_SPAN+1..TS_SMALL entries
    SC_LARGE = 7,       // large jobs: rows of TS_SMALL+1..TS_MAX entries
    SC_OVERFLOW = 8,    // a row or a tile the on-chip sort cannot take
    SC_CURSOR = 9,      // [9 + c]: fill cursors of the short classes
    SC_N = 16
};

// 0: nothing to sort (0 or 1 entry), 1..5: short of padded length 2^c,
// 6: medium (span tile), 7: a small job of its own, 8: a large job of its
// own, 9: too long.
__device__ __forceinline__ int seg_class(uint64_t L) {
    if (L <= 1) return 0;
    if (L <= 32) return 32 - __clz((unsigned)(L - 1));
    if (L <= (uint64_t)SEG_SPAN) return 6;
    if (L <= (uint64_t)TS_SMALL) return 7;
    if (L <= (uint64_t)TS_MAX) return 8;
    return 9;
}

// Counts the short rows of every class.
__global__ void __launch_bounds__(256) seg_count(const uint64_t *__restrict__ s_off, uint64_t n_rows,
                                                 unsigned *__restrict__ ctr) {
    __shared__ unsigned sc[6];
    if (threadIdx.x < 6) sc[threadIdx.x] = 0;
    __syncthreads();
    for (uint64_t r = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; r < n_rows;
         r += (uint64_t)gridDim.x * blockDim.x) {
        const int c = seg_class(s_off[r + 1] - s_off[r]);
        if (c >= 1 && c <= 5) atomicAdd(&sc[c], 1u);
    }
    __syncthreads();
    if (threadIdx.x >= 1 && threadIdx.x <= 5 && sc[threadIdx.x]) atomicAdd(&ctr[SC_SHORT + threadIdx.x], sc[threadIdx.x]);
}

// Writes single-entry rows through, lists short rows by class (class c in
// short_rows[base_c ...], base_c = rows of the classes below), medium rows by
// span tile (tile_rows[t * SEG_TILE_ROWS + k], tile_len[t] = their entries)
// and longer rows as small or large jobs of their own.
__global__ void __launch_bounds__(256) seg_place(const uint32_t *__restrict__ cols, const uint64_t *__restrict__ s_off,
                                                 uint64_t n_rows, int cbits, unsigned *__restrict__ ctr,
                                                 uint32_t *__restrict__ short_rows, unsigned *__restrict__ tile_cnt,
                                                 unsigned *__restrict__ tile_len, uint32_t *__restrict__ tile_rows,
                                                 uint64_t *__restrict__ small_jobs,
                                                 uint64_t *__restrict__ large_jobs, uint64_t *__restrict__ keys_out,
                                                 uint32_t *__restrict__ idx_out) {
    __shared__ unsigned sc[8], sbase[8];
    unsigned base[6];
    base[0] = 0;
#pragma unroll
    for (int c = 1; c <= 5; ++c) base[c] = base[c - 1] + (c > 1 ? ctr[SC_SHORT + c - 1] : 0u);
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    const uint64_t n_iter = (n_rows + stride - 1) / stride;  // the same for every thread: block-wide syncs below
    for (uint64_t it = 0; it < n_iter; ++it) {
        const uint64_t r = it * stride + blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
        if (threadIdx.x < 8) sc[threadIdx.x] = 0;
        __syncthreads();
        int c = 0;
        unsigned slot = 0;
        uint64_t b = 0, L = 0;
        if (r < n_rows) {
            b = s_off[r];
            L = s_off[r + 1] - b;
            c = seg_class(L);
            if (L == 1) {
                keys_out[b] = ((uint64_t)r << cbits) | cols[b];
                idx_out[b] = (uint32_t)b;
            } else if (c >= 1 && c <= 5) {
                slot = atomicAdd(&sc[c], 1u);
            } else if (c == 7 || c == 8) {
                slot = atomicAdd(&sc[c - 1], 1u);  // sc[6]: small, sc[7]: large
            } else if (c == 6) {
                const uint64_t t = b / SEG_SPAN;
                const unsigned k = atomicAdd(&tile_cnt[t], 1u);
                if (k < SEG_TILE_ROWS) {
                    tile_rows[t * SEG_TILE_ROWS + k] = (uint32_t)r;
                    atomicAdd(&tile_len[t], (unsigned)L);
                } else {
                    atomicOr(&ctr[SC_OVERFLOW], 1u);  // (not reachable: rows of > 32 entries start 33 apart)
                }
            } else if (c == 9) {
                atomicOr(&ctr[SC_OVERFLOW], 1u);
            }
        }
        __syncthreads();
        if (threadIdx.x >= 1 && threadIdx.x <= 5 && sc[threadIdx.x])
            sbase[threadIdx.x] = atomicAdd(&ctr[SC_CURSOR + threadIdx.x], sc[threadIdx.x]);
        if (threadIdx.x == 6 && sc[6]) sbase[6] = atomicAdd(&ctr[SC_SMALL], sc[6]);
        if (threadIdx.x == 7 && sc[7]) sbase[7] = atomicAdd(&ctr[SC_LARGE], sc[7]);
        __syncthreads();
        if (r < n_rows) {
            if (c >= 1 && c <= 5) short_rows[base[c] + sbase[c] + slot] = (uint32_t)r;
            else if (c == 7) small_jobs[sbase[6] + slot] = SEG_ROW_JOB | r;
            else if (c == 8) large_jobs[sbase[7] + slot] = SEG_ROW_JOB | r;
        }
        __syncthreads();
    }
}

// Span tiles holding medium rows onto the small job list (one atomic per warp).
__global__ void seg_tiles(const unsigned *__restrict__ tile_len, uint64_t n_spans, unsigned *__restrict__ ctr,
                          uint64_t *__restrict__ small_jobs) {
    const uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    const unsigned E = t < n_spans ? tile_len[t] : 0u;
    if (E > (unsigned)TS_SMALL) atomicOr(&ctr[SC_OVERFLOW], 1u);  // (not reachable: < 2 SEG_SPAN)
    const bool take = E != 0 && E <= (unsigned)TS_SMALL;
    const unsigned want = __ballot_sync(0xffffffffu, take);
    if (!want) return;
    const int lane = threadIdx.x & 31, leader = __ffs(want) - 1;
    unsigned base = 0;
    if (lane == leader) base = atomicAdd(&ctr[SC_SMALL], (unsigned)__popc(want));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (take) small_jobs[base + __popc(want & ((1u << lane) - 1u))] = t;
}

// Bitonic sort of aligned P-lane segments of the warp, ascending in every
// segment (P a power of two, <= 32).
template <int P>
__device__ __forceinline__ uint32_t segment_bitonic(uint32_t key, int lane) {
#pragma unroll
    for (int k = 2; k <= P; k <<= 1) {
#pragma unroll
        for (int j = k >> 1; j > 0; j >>= 1) {
            const uint32_t other = __shfl_xor_sync(0xffffffffu, key, j);
            const bool up = k == P || (lane & k) == 0;  // direction of this lane's k-block
            const bool low = (lane & j) == 0;           // lower partner keeps the smaller in an up block
            key = (low == up) ? min(key, other) : max(key, other);
        }
    }
    return key;
}

template <int P>
__device__ __forceinline__ void sort_short_group(const uint32_t *__restrict__ cols, const uint64_t *__restrict__ s_off,
                                                 const uint32_t *__restrict__ list, unsigned n_list, unsigned group,
                                                 int cbits, uint64_t *__restrict__ keys_out,
                                                 uint32_t *__restrict__ idx_out, int lane) {
    const unsigned i = group * (32 / P) + lane / P;
    const int j = lane % P;
    uint32_t key = 0xFFFFFFFFu;  // real keys stay below 2^31: cbits <= 26
    uint64_t b = 0, L = 0, r = 0;
    if (i < n_list) {
        r = list[i];
        b = s_off[r];
        L = s_off[r + 1] - b;
        if ((uint64_t)j < L) key = (cols[b + j] << 5) | (uint32_t)j;
    }
    key = segment_bitonic<P>(key, lane);
    if ((uint64_t)j < L) {
        keys_out[b + j] = (r << cbits) | (key >> 5);
        idx_out[b + j] = (uint32_t)(b + (key & 31u));
    }
}

// Short rows: warp job g of class c sorts rows [g * 32 / P, (g + 1) * 32 / P)
// of that class's list; jobs of all classes in one grid-stride sweep.
__global__ void __launch_bounds__(256) seg_short_sort(const uint32_t *__restrict__ cols,
                                                      const uint64_t *__restrict__ s_off,
                                                      const uint32_t *__restrict__ short_rows,
                                                      const unsigned *__restrict__ ctr, int cbits,
                                                      uint64_t *__restrict__ keys_out, uint32_t *__restrict__ idx_out) {
    unsigned cnt[6], base[6], jobs_end[6];
    cnt[0] = base[0] = jobs_end[0] = 0;
#pragma unroll
    for (int c = 1; c <= 5; ++c) {
        cnt[c] = ctr[SC_SHORT + c];
        base[c] = base[c - 1] + cnt[c - 1];
        const unsigned per = 32u >> c;  // rows per warp
        jobs_end[c] = jobs_end[c - 1] + (cnt[c] + per - 1) / per;
    }
    const int lane = threadIdx.x & 31;
    const unsigned warps = gridDim.x * (blockDim.x >> 5);
    for (unsigned job = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); job < jobs_end[5]; job += warps) {
        int c = 1;
        while (job >= jobs_end[c]) ++c;  // warp-uniform
        const unsigned g = job - jobs_end[c - 1];
        const uint32_t *list = short_rows + base[c];
        switch (c) {
            case 1: sort_short_group<2>(cols, s_off, list, cnt[1], g, cbits, keys_out, idx_out, lane); break;
            case 2: sort_short_group<4>(cols, s_off, list, cnt[2], g, cbits, keys_out, idx_out, lane); break;
            case 3: sort_short_group<8>(cols, s_off, list, cnt[3], g, cbits, keys_out, idx_out, lane); break;
            case 4: sort_short_group<16>(cols, s_off, list, cnt[4], g, cbits, keys_out, idx_out, lane); break;
            default: sort_short_group<32>(cols, s_off, list, cnt[5], g, cbits, keys_out, idx_out, lane); break;
        }
    }
}

template <int MAXE, int SLICE>
struct TileSortSmem {
    uint32_t key[2][MAXE];
    uint16_t idx[2][MAXE];
    unsigned cnt[2][MAXE / SLICE][256];
    unsigned wsum[8];
    uint64_t start[SEG_TILE_ROWS];  // first input position of the tile's rows, by rank
    uint32_t row[SEG_TILE_ROWS];
    unsigned pref[SEG_TILE_ROWS + 1];  // tile position of each rank's first entry
    unsigned n_rows;
};

// Sorts the tiles of a job list (MAXE entries at most): a span tile's medium
// rows, or (jobs with SEG_ROW_JOB set) one long row. Persistent blocks take
// jobs in a grid-stride loop; one warp per SLICE entries.
template <int MAXE, int SLICE>
__global__ void __launch_bounds__(MAXE / SLICE * 32)
seg_tile_sort(const uint32_t *__restrict__ cols, const uint64_t *__restrict__ s_off,
              const unsigned *__restrict__ tile_cnt, const uint32_t *__restrict__ tile_rows,
              const uint64_t *__restrict__ jobs, const unsigned *__restrict__ n_jobs, int cbits,
              uint64_t *__restrict__ keys_out, uint32_t *__restrict__ idx_out, unsigned *__restrict__ overflow) {
    constexpr int W = MAXE / SLICE, T = W * 32;
    extern __shared__ __align__(16) unsigned char ts_raw[];
    TileSortSmem<MAXE, SLICE> &S = *reinterpret_cast<TileSortSmem<MAXE, SLICE> *>(ts_raw);
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    const unsigned nj = *n_jobs;
    for (unsigned jb = blockIdx.x; jb < nj; jb += gridDim.x) {
        const uint64_t job = jobs[jb];
        if (job & SEG_ROW_JOB) {
            if (t == 0) {
                S.n_rows = 1;
                S.row[0] = (uint32_t)(job & ~SEG_ROW_JOB);
            }
        } else {
            const unsigned nr = min(tile_cnt[job], (unsigned)SEG_TILE_ROWS);
            if (t == 0) S.n_rows = nr;
            if (t < (int)nr) S.row[t] = tile_rows[job * SEG_TILE_ROWS + t];
        }
        __syncthreads();
        const unsigned nr = S.n_rows;
        if (t < (int)nr) {
            const uint32_t r = S.row[t];
            S.start[t] = s_off[r];
            S.pref[t + 1] = (unsigned)(s_off[r + 1] - s_off[r]);
        }
        __syncthreads();
        if (t == 0) {
            S.pref[0] = 0;
            for (unsigned i = 1; i <= nr; ++i) S.pref[i] += S.pref[i - 1];
        }
        __syncthreads();
        const int E = (int)S.pref[nr];
        const int rbits = nr > 1 ? 32 - __clz(nr - 1) : 0;
        const int bits = rbits + cbits;
        if (E > MAXE || bits > 32) {  // (the plan never lists such tiles; cbits <= 26 is checked before)
            if (t == 0) atomicOr(overflow, 1u);
            __syncthreads();
            continue;
        }
        const int passes = (bits + 7) / 8;
        for (int e = t; e < E; e += T) {
            unsigned lo = 0, hi = nr - 1;  // rank: last i with pref[i] <= e
            while (lo < hi) {
                const unsigned mid = (lo + hi + 1) >> 1;
                if (S.pref[mid] <= (unsigned)e) lo = mid;
                else hi = mid - 1;
            }
            S.key[0][e] = (lo << cbits) | cols[S.start[lo] + (e - S.pref[lo])];
            S.idx[0][e] = (uint16_t)e;
        }
        for (int i = t; i < 2 * W * 256; i += T) (&S.cnt[0][0][0])[i] = 0;
        __syncthreads();
        const int q0 = warp * SLICE, q1 = min(E, q0 + SLICE);
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
                    if (p + 1 < passes) atomicAdd(&S.cnt[c ^ 1][pos / SLICE][(k >> (shift + 8)) & 0xFFu], 1u);
                }
                __syncwarp();
            }
            __syncthreads();
            cur ^= 1;
        }
        const uint32_t cmask = (uint32_t)((1ull << cbits) - 1);
        for (int q = t; q < E; q += T) {
            const uint32_t k = S.key[cur][q];
            const unsigned i = cbits < 32 ? (k >> cbits) : 0u;
            const uint64_t out = S.start[i] + (unsigned)(q - S.pref[i]);
            keys_out[out] = ((uint64_t)S.row[i] << cbits) | (k & cmask);
            idx_out[out] = (uint32_t)(S.start[i] + (S.idx[cur][q] - S.pref[i]));
        }
        __syncthreads();  // shared state is rebuilt by the next job
    }
}

}  // namespace

int sort_grouped_rows(Ctx *c, const uint32_t *rows, const uint32_t *cols, const uint64_t *s_off, uint64_t m,
                      uint64_t n_rows, int cbits, uint64_t *keys_out, uint32_t *idx_out, bool *done, cudaStream_t s) {
    (void)rows;  // the rows are s_off's
    *done = false;
    if (m == 0) {
        *done = true;
        return SPG_OK;
    }
    if (cbits > SEG_MAX_CBITS || m > 0xFFFFFFFFull) return SPG_OK;
    const uint64_t n_spans = (m + SEG_SPAN - 1) / SEG_SPAN;
    const uint64_t n_small = n_spans + m / (SEG_SPAN + 1) + 1, n_large = m / (TS_SMALL + 1) + 1;
    DevBuf ctr_b, tiles_b, tile_rows_b, short_b, jobs_b;
    SPG_TRY(ctr_b.alloc(SC_N * sizeof(unsigned), s));
    SPG_TRY(tiles_b.alloc(2 * n_spans * sizeof(unsigned), s));  // tile_cnt, tile_len
    SPG_TRY(tile_rows_b.alloc(n_spans * SEG_TILE_ROWS * sizeof(uint32_t), s));
    SPG_TRY(short_b.alloc(n_rows * sizeof(uint32_t), s));
    SPG_TRY(jobs_b.alloc((n_small + n_large) * sizeof(uint64_t), s));
    SPG_CUDA_TRY(cudaMemsetAsync(ctr_b.ptr, 0, SC_N * sizeof(unsigned), s));
    SPG_CUDA_TRY(cudaMemsetAsync(tiles_b.ptr, 0, 2 * n_spans * sizeof(unsigned), s));
    unsigned *ctr = ctr_b.as<unsigned>(), *tile_cnt = tiles_b.as<unsigned>(), *tile_len = tile_cnt + n_spans;
    uint64_t *small_jobs = jobs_b.as<uint64_t>(), *large_jobs = small_jobs + n_small;
    const unsigned gr = grid_for(n_rows, 256, (unsigned)c->n_sms * 8);
    seg_count<<<gr, 256, 0, s>>>(s_off, n_rows, ctr);
    SPG_LAUNCH_CHECK();
    seg_place<<<gr, 256, 0, s>>>(cols, s_off, n_rows, cbits, ctr, short_b.as<uint32_t>(), tile_cnt, tile_len,
                                 tile_rows_b.as<uint32_t>(), small_jobs, large_jobs, keys_out, idx_out);
    SPG_LAUNCH_CHECK();
    seg_tiles<<<grid_for(n_spans, 256), 256, 0, s>>>(tile_len, n_spans, ctr, small_jobs);
    SPG_LAUNCH_CHECK();
    seg_short_sort<<<(unsigned)c->n_sms * 8, 256, 0, s>>>(cols, s_off, short_b.as<uint32_t>(), ctr, cbits, keys_out,
                                                          idx_out);
    SPG_LAUNCH_CHECK();
    constexpr size_t small_smem = sizeof(TileSortSmem<TS_SMALL, TS_SLICE_SMALL>);
    constexpr size_t large_smem = sizeof(TileSortSmem<TS_MAX, TS_SLICE_LARGE>);
    constexpr unsigned small_threads = TS_SMALL / TS_SLICE_SMALL * 32;
    constexpr unsigned large_threads = TS_MAX / TS_SLICE_LARGE * 32;
    auto small_k = seg_tile_sort<TS_SMALL, TS_SLICE_SMALL>;
    auto large_k = seg_tile_sort<TS_MAX, TS_SLICE_LARGE>;
    SPG_CUDA_TRY(cudaFuncSetAttribute(small_k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)small_smem));
    SPG_CUDA_TRY(cudaFuncSetAttribute(large_k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)large_smem));
    // persistent blocks over the job lists, whose lengths stay on the device
    const unsigned small_grid = (unsigned)std::min<uint64_t>(n_small, (uint64_t)c->n_sms * 3);
    const unsigned large_grid = (unsigned)std::min<uint64_t>(n_large, (uint64_t)c->n_sms);
    small_k<<<small_grid, small_threads, small_smem, s>>>(cols, s_off, tile_cnt, tile_rows_b.as<uint32_t>(),
                                                          small_jobs, ctr + SC_SMALL, cbits, keys_out, idx_out,
                                                          ctr + SC_OVERFLOW);
    SPG_LAUNCH_CHECK();
    large_k<<<large_grid, large_threads, large_smem, s>>>(cols, s_off, tile_cnt, tile_rows_b.as<uint32_t>(),
                                                          large_jobs, ctr + SC_LARGE, cbits, keys_out, idx_out,
                                                          ctr + SC_OVERFLOW);
    SPG_LAUNCH_CHECK();
    unsigned h = 1u;
    SPG_CUDA_TRY(cudaMemcpyAsync(&h, ctr + SC_OVERFLOW, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
    SPG_TRY(c->phase_sync(s));
    *done = h == 0;
    return SPG_OK;
}

}  // namespace spg
