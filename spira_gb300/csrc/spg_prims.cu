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
              unsigned long long *__restrict__ hist /* [RADIX][n_tiles], scanned in place next */) {
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

}  // namespace

namespace {

template <int RS_ITERS>
int radix_sort_impl(Ctx *c, uint64_t *d_keys, uint32_t *d_vals, uint64_t n, int key_bits, cudaStream_t s) {
    constexpr int RS_TILE = RS_BLOCK * RS_ITERS;
    const unsigned n_tiles = (unsigned)((n + RS_TILE - 1) / RS_TILE);
    const uint64_t hist_n = (uint64_t)RS_RADIX * n_tiles;
    DevBuf kalt, valt, offs;
    SPG_TRY(kalt.alloc(n * sizeof(uint64_t), s));
    SPG_TRY(valt.alloc(n * sizeof(uint32_t), s));
    SPG_TRY(offs.alloc(hist_n * sizeof(unsigned long long), s));
    uint64_t *kin = d_keys, *kout = kalt.as<uint64_t>();
    uint32_t *vin = d_vals, *vout = valt.as<uint32_t>();
    const int passes = (key_bits + 7) / 8;
    constexpr size_t smem = sizeof(ScatterSmem<RS_TILE>);
    SPG_CUDA_TRY(cudaFuncSetAttribute(radix_scatter<RS_ITERS>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)smem));
    for (int p = 0; p < passes; ++p) {
        const int shift = p * 8;
        radix_upsweep<RS_ITERS><<<n_tiles, RS_BLOCK, 0, s>>>(kin, n, shift, n_tiles, offs.as<unsigned long long>());
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
//     length P (2, 4, 8, 16, 32) per warp, keys (col << 5 | position); a warp
//     takes 32 consecutive rows (their offsets in one coalesced read) and
//     sorts each class present among them in turn;
//   * 33..SEG_MEDIUM entries: one warp per row, a bitonic network over the
//     row padded to a power of two, 2..16 keys (col << 9 | position) to a
//     lane; 32-bit keys while the columns need at most 22 bits, else 64-bit;
//   * SEG_MEDIUM+1..TS_MAX entries: a block per row, in shared memory: an
//     LSD radix sort of the 32-bit columns carrying 16-bit row positions,
//     with 6-bit digits ranked the way Merrill and Grimshaw's block radix
//     sort ranks them: every thread holds I consecutive entries (so thread
//     order is input order), counts its digits in its own column of packed
//     16-bit counters (two digits per word: d and d + 32), one raking scan
//     over all counters in (digit, thread) order turns them into exclusive
//     prefixes, and each entry's rank is its digit's prefix plus the count
//     of the same digit before it in its thread: a stable scatter with no
//     per-digit warp votes. Counters and the exchange arrays share memory,
//     padded one word in 33 so that column and raking accesses and the
//     blocked reads are free of bank conflicts. Three kernels sized to the
//     rows (128 x 16, 256 x 16 and 768 x 16 entries) keep few threads idle.
// In every network the key carries the entry's position in its row, so the
// sorted order is the stable order. Columns of more than 26 bits, or a row
// longer than TS_MAX, make the sort report failure; callers then sort
// globally. Work lists are filled with atomics, in no particular order: every
// row's output places are fixed by s_off, so the result does not depend on
// that order.
// ---------------------------------------------------------------------------
namespace {

constexpr int SEG_MEDIUM = 512;   // rows of 33..SEG_MEDIUM entries: a warp each
constexpr int TS0_T = 128, TS0_I = 16;   // rows up to 2048 entries (256 x 8 measured 29 % slower)
constexpr int TS1_T = 256, TS1_I = 16;   // rows up to 4096
constexpr int TS2_T = 768, TS2_I = 16;   // rows up to TS_MAX
constexpr int TS0 = TS0_T * TS0_I, TS1 = TS1_T * TS1_I, TS_MAX = TS2_T * TS2_I;
constexpr int RS_DBITS = 6, RS_DIGITS = 1 << RS_DBITS, RS_WORDS = RS_DIGITS / 2;
constexpr int SEG_MAX_CBITS = 26;

// counters (unsigned) of the plan
enum : int {
    SC_LIST = 0,        // [1..6]: rows of padded length 2^c (1..5), medium rows (6)
    SC_JOBS = 7,        // [7..9]: rows of tile kernel 0, 1, 2
    SC_OVERFLOW = 10,   // a row the on-chip sort cannot take
    SC_N = 16
};

// 0: nothing to sort (0 or 1 entry), 1..5: short of padded length 2^c,
// 6: medium, 7..9: tile kernel 0..2, 10: too long.
__device__ __forceinline__ int seg_class(uint64_t L) {
    if (L <= 1) return 0;
    if (L <= 32) return 32 - __clz((unsigned)(L - 1));
    if (L <= (uint64_t)SEG_MEDIUM) return 6;
    if (L <= (uint64_t)TS0) return 7;
    if (L <= (uint64_t)TS1) return 8;
    if (L <= (uint64_t)TS_MAX) return 9;
    return 10;
}

// Where the sort puts a row's entries. Key mode (DEDUP = false): keys[p] =
// row << cbits | col and idx[p] = input position, p over the row's input
// positions in sorted order. Dedup mode (a first lock): the row's last write
// per column, unless zero, in column order at the row's first input
// positions (cols[s_off[r] + k], vals[s_off[r] + k]) and kept[r] = their
// number.
struct SegOut {
    uint64_t *keys;
    uint32_t *idx;
    const double *in_vals;
    uint32_t *cols;
    double *vals;
    uint64_t *kept;
};

// The rows of every class c (ctr[SC_LIST + c]; classes 6..9 are listed).
__global__ void __launch_bounds__(256) seg_count(const uint64_t *__restrict__ s_off, uint64_t n_rows,
                                                 unsigned *__restrict__ ctr) {
    __shared__ unsigned sc[10];
    if (threadIdx.x < 10) sc[threadIdx.x] = 0;
    __syncthreads();
    for (uint64_t r = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; r < n_rows;
         r += (uint64_t)gridDim.x * blockDim.x) {
        const int c = seg_class(s_off[r + 1] - s_off[r]);
        if (c >= 1 && c <= 9) atomicAdd(&sc[c], 1u);
        else if (c == 10) atomicOr(&ctr[SC_OVERFLOW], 1u);
    }
    __syncthreads();
    if (threadIdx.x >= 1 && threadIdx.x <= 9 && sc[threadIdx.x]) atomicAdd(&ctr[SC_LIST + threadIdx.x], sc[threadIdx.x]);
}

// Writes single-entry rows through and lists the rows of classes 6..9:
// lists[base_c + k] for class c (base_c = the rows of the listed classes
// below it; classes 7..9 are the tile kernels' lists). cur[c]: fill cursors.
template <bool DEDUP>
__global__ void __launch_bounds__(256) seg_place(const uint32_t *__restrict__ cols, const uint64_t *__restrict__ s_off,
                                                 uint64_t n_rows, int cbits, const unsigned *__restrict__ ctr,
                                                 unsigned *__restrict__ cur, uint32_t *__restrict__ lists, SegOut o) {
    __shared__ unsigned sc[10], sbase[10], base[10];
    if (threadIdx.x == 0) {
        base[6] = 0;
        for (int c = 7; c <= 9; ++c) base[c] = base[c - 1] + ctr[SC_LIST + c - 1];
    }
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    const uint64_t n_iter = (n_rows + stride - 1) / stride;  // the same for every thread: block-wide syncs below
    for (uint64_t it = 0; it < n_iter; ++it) {
        const uint64_t r = it * stride + blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
        if (threadIdx.x < 10) sc[threadIdx.x] = 0;
        __syncthreads();
        int c = 0;
        unsigned slot = 0;
        if (r < n_rows) {
            const uint64_t b = s_off[r], L = s_off[r + 1] - b;
            c = seg_class(L);
            if (L == 1) {
                if constexpr (DEDUP) {
                    const double v = o.in_vals[b];
                    o.cols[b] = cols[b];
                    o.vals[b] = v;
                    o.kept[r] = is_zero(v) ? 0 : 1;
                } else {
                    o.keys[b] = ((uint64_t)r << cbits) | cols[b];
                    o.idx[b] = (uint32_t)b;
                }
            } else if (L == 0) {
                if constexpr (DEDUP) o.kept[r] = 0;
            } else if (c >= 6 && c <= 9) {
                slot = atomicAdd(&sc[c], 1u);
            }
        }
        __syncthreads();
        if (threadIdx.x >= 6 && threadIdx.x <= 9 && sc[threadIdx.x])
            sbase[threadIdx.x] = atomicAdd(&cur[threadIdx.x], sc[threadIdx.x]);
        __syncthreads();
        if (r < n_rows && c >= 6 && c <= 9) lists[base[c] + sbase[c] + slot] = (uint32_t)r;
        __syncthreads();
    }
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

// Rows (b, L, r) of one class, one per P-lane segment (L = 0: no row).
template <int P, bool DEDUP>
__device__ __forceinline__ void sort_short_group(const uint32_t *__restrict__ cols, uint64_t b, uint64_t L,
                                                 uint64_t r, int cbits, const SegOut &o, int lane) {
    const int j = lane % P;
    uint32_t key = 0xFFFFFFFFu;  // real keys stay below 2^31: cbits <= 26
    double v_in = 0.0;
    {
        if ((uint64_t)j < L) {
            key = (cols[b + j] << 5) | (uint32_t)j;
            if constexpr (DEDUP) v_in = o.in_vals[b + j];  // in input order: coalesced
        }
    }
    key = segment_bitonic<P>(key, lane);
    if constexpr (!DEDUP) {
        if ((uint64_t)j < L) {
            o.keys[b + j] = (r << cbits) | (key >> 5);
            o.idx[b + j] = (uint32_t)(b + (key & 31u));
        }
    } else {
        // the last of a run of equal columns is the last write; kept unless
        // zero. Its value comes from the lane that loaded it.
        const uint32_t nxt = __shfl_down_sync(0xffffffffu, key, 1);
        const double v = __shfl_sync(0xffffffffu, v_in, (lane & ~(P - 1)) | (int)(key & (uint32_t)(P - 1)));
        bool keep = false;
        if ((uint64_t)j < L && ((uint64_t)(j + 1) == L || (nxt >> 5) != (key >> 5))) keep = !is_zero(v);
        const unsigned seg = P == 32 ? 0xffffffffu : ((1u << (P & 31)) - 1u) << (lane & ~(P - 1));
        const unsigned bal = __ballot_sync(0xffffffffu, keep) & seg;
        if (keep) {
            const uint64_t w = b + (uint64_t)__popc(bal & ((1u << lane) - 1u));
            o.cols[w] = key >> 5;
            o.vals[w] = v;
        }
        if (j == 0 && L) o.kept[r] = (uint64_t)__popc(bal);
    }
}

// Short rows: warp w takes rows [32 w, 32 w + 32) (grid-stride), reads
// their offsets in one coalesced access, and sorts the rows of each short
// class among them, 32 / P at a time (segment g of P lanes takes the class's
// g-th remaining row).
template <bool DEDUP>
__global__ void __launch_bounds__(256) seg_short_sort(const uint32_t *__restrict__ cols,
                                                      const uint64_t *__restrict__ s_off, uint64_t n_rows, int cbits,
                                                      SegOut o) {
    const int lane = threadIdx.x & 31;
    const uint64_t warps = (uint64_t)gridDim.x * (blockDim.x >> 5);
    for (uint64_t w = blockIdx.x * (uint64_t)(blockDim.x >> 5) + (threadIdx.x >> 5); w * 32 < n_rows; w += warps) {
        const uint64_t r = w * 32 + lane;
        uint64_t b = 0, L = 0;
        if (r < n_rows) {
            b = s_off[r];
            L = s_off[r + 1] - b;
        }
        const int c = (L >= 2 && L <= 32) ? 32 - __clz((unsigned)(L - 1)) : 0;
#pragma unroll
        for (int cls = 1; cls <= 5; ++cls) {
            unsigned mask = __ballot_sync(0xffffffffu, c == cls);
            const int P = 1 << cls, per = 32 >> cls;
            while (mask) {
                const int g = lane >> cls;  // this lane's segment
                const unsigned src = __fns(mask, 0, g + 1);  // the segment's row: g-th set lane of mask
                const int sl = src < 32 ? (int)src : 0;
                const uint64_t gb = __shfl_sync(0xffffffffu, b, sl), gL = __shfl_sync(0xffffffffu, L, sl);
                const uint64_t gr = w * 32 + (uint64_t)sl;
                const uint64_t len = src < 32 ? gL : 0;
                switch (cls) {
                    case 1: sort_short_group<2, DEDUP>(cols, gb, len, gr, cbits, o, lane); break;
                    case 2: sort_short_group<4, DEDUP>(cols, gb, len, gr, cbits, o, lane); break;
                    case 3: sort_short_group<8, DEDUP>(cols, gb, len, gr, cbits, o, lane); break;
                    case 4: sort_short_group<16, DEDUP>(cols, gb, len, gr, cbits, o, lane); break;
                    default: sort_short_group<32, DEDUP>(cols, gb, len, gr, cbits, o, lane); break;
                }
                (void)P;
                for (int k = 0; k < per && mask; ++k) mask &= mask - 1;  // drop the rows just sorted
            }
        }
    }
}

// Compare-exchange of key[e] and key[e | JJ] (elements 32 JJ apart, in one
// lane's registers) in a bitonic stage of block size k.
template <int E, int JJ, class K>
__device__ __forceinline__ void cx_registers(K (&key)[E], int k) {
    if constexpr (JJ < E) {
#pragma unroll
        for (int e = 0; e < E; ++e) {
            if ((e & JJ) == 0) {
                const int f = e | JJ;
                const bool up = ((32 * e) & k) == 0;
                const K a = key[e], b = key[f];
                const bool sw = up ? (a > b) : (a < b);
                key[e] = sw ? b : a;
                key[f] = sw ? a : b;
            }
        }
    }
}

// warp_bitonic's network with the stages in a loop rather than unrolled: the
// same order, a few hundred instructions of code instead of thousands (the
// unrolled kernel stalled on instruction fetch).
template <int E, class K>
__device__ __forceinline__ void warp_bitonic_looped(K (&key)[E], int lane) {
    for (int k = 2; k <= 32 * E; k <<= 1) {
        for (int jj = k >> 6; jj >= 1; jj >>= 1) {  // partners 32 jj apart: registers
            if (jj >= 8) cx_registers<E, 8>(key, k);
            else if (jj == 4) cx_registers<E, 4>(key, k);
            else if (jj == 2) cx_registers<E, 2>(key, k);
            else cx_registers<E, 1>(key, k);
        }
        for (int j = min(k >> 1, 16); j >= 1; j >>= 1) {  // nearer partners: shuffles
#pragma unroll
            for (int e = 0; e < E; ++e) {
                const K o = __shfl_xor_sync(0xffffffffu, key[e], j);
                const int i = 32 * e + lane;
                const bool keep_min = (((i & k) == 0) == ((i & j) == 0));
                key[e] = keep_min ? (o < key[e] ? o : key[e]) : (o > key[e] ? o : key[e]);
            }
        }
    }
}

// One medium row (33..32 E entries), one warp: element 32 e + lane in
// key[e] = col << 9 | position (padding above every key), sorted, written.
// (Holding E consecutive elements per lane instead, so that near partners
// meet in registers, measured 2.6x slower: strided loads and stores, and
// twice the registers.)
template <int E, class K, bool DEDUP>
__device__ __forceinline__ void sort_medium_row(const uint32_t *__restrict__ cols, uint64_t b, uint32_t L, uint64_t r,
                                                int cbits, const SegOut &o, int lane) {
    K key[E];
#pragma unroll
    for (int e = 0; e < E; ++e) {
        const uint32_t p = 32u * e + lane;
        key[e] = p < L ? (((K)cols[b + p] << 9) | (K)p) : ~(K)0;
    }
    warp_bitonic_looped<E, K>(key, lane);
    if constexpr (!DEDUP) {
#pragma unroll
        for (int e = 0; e < E; ++e) {
            const uint32_t p = 32u * e + lane;
            if (p < L) {
                o.keys[b + p] = (r << cbits) | (uint64_t)(key[e] >> 9);
                o.idx[b + p] = (uint32_t)(b + (uint32_t)(key[e] & 511u));
            }
        }
    } else {
        uint32_t kept = 0;
        const unsigned lt = (1u << lane) - 1u;
#pragma unroll
        for (int e = 0; e < E; ++e) {
            const uint32_t p = 32u * e + lane;
            // the next element: lane + 1 of the same register, or lane 0 of the next
            K nx = __shfl_down_sync(0xffffffffu, key[e], 1);
            if (e + 1 < E) {
                const K f = __shfl_sync(0xffffffffu, key[e + 1 < E ? e + 1 : e], 0);
                if (lane == 31) nx = f;
            }
            bool keep = false;
            double v = 0.0;
            if (p < L && (p + 1 == L || (nx >> 9) != (key[e] >> 9))) {  // last write of its column
                v = o.in_vals[b + (uint32_t)(key[e] & 511u)];
                keep = !is_zero(v);
            }
            const unsigned bal = __ballot_sync(0xffffffffu, keep);
            if (keep) {
                const uint64_t w = b + kept + (uint32_t)__popc(bal & lt);
                o.cols[w] = (uint32_t)(key[e] >> 9);
                o.vals[w] = v;
            }
            kept += (uint32_t)__popc(bal);
        }
        if (lane == 0) o.kept[r] = kept;
    }
}

// Medium rows: a warp per row from the class-6 list.
template <class K, bool DEDUP>
__global__ void __launch_bounds__(256, sizeof(K) == 8 ? 2 : 4) seg_medium_sort(const uint32_t *__restrict__ cols,
                                                       const uint64_t *__restrict__ s_off,
                                                       const uint32_t *__restrict__ lists,
                                                       const unsigned *__restrict__ ctr, int cbits, SegOut o) {
    const unsigned n = ctr[SC_LIST + 6];  // class 6 heads the lists
    const int lane = threadIdx.x & 31;
    const unsigned warps = gridDim.x * (blockDim.x >> 5);
    for (unsigned k = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); k < n; k += warps) {
        const uint64_t r = lists[k];
        const uint64_t b = s_off[r];
        const uint32_t L = (uint32_t)(s_off[r + 1] - b);
        if (L <= 64) sort_medium_row<2, K, DEDUP>(cols, b, L, r, cbits, o, lane);
        else if (L <= 128) sort_medium_row<4, K, DEDUP>(cols, b, L, r, cbits, o, lane);
        else if (L <= 256) sort_medium_row<8, K, DEDUP>(cols, b, L, r, cbits, o, lane);
        else sort_medium_row<16, K, DEDUP>(cols, b, L, r, cbits, o, lane);
    }
}

constexpr uint16_t IDX_ZERO = 0x8000;  // row positions are < 2^14

// Shared-memory index with one pad word per 32: threads of a warp reading
// word j of their own 32-word segment (the raking scan), or their k-th of 16
// consecutive entries, hit distinct banks.
__device__ __forceinline__ uint32_t pad33(uint32_t p) { return p + (p >> 5); }

template <int T, int I, bool DEDUP>
struct TileSmem {
    static constexpr int MAXE = T * I;
    static constexpr int NCTR = RS_WORDS * T;
    static constexpr bool VSTAGE = DEDUP && MAXE <= 4096;  // values staged in shared memory
    union {  // the counters live only inside a radix pass, the exchange arrays between passes
        uint32_t ctr[NCTR + NCTR / 32];  // counter word w of thread t at pad33(w T + t)
        struct {
            uint32_t key[MAXE + MAXE / 32];
            uint16_t idx[MAXE + MAXE / 32];  // row position; dedup mode: | IDX_ZERO if the value is zero
            uint32_t ex[MAXE + MAXE / 32 + 2];  // dedup mode: kept entries before each position
        } x;
    } u;
    double val[VSTAGE ? MAXE : 1];  // dedup mode: values by row position, kept through every pass
    uint32_t wsum[T / 32];
};

// Rows of tile kernel KI's list (class 7 + KI, T * I entries at most), a
// block per row; persistent blocks take rows in a grid-stride loop.
template <int T, int I, bool DEDUP>
__global__ void __launch_bounds__(T, T <= 128 ? 6 : T <= 256 ? 3 : 1)
seg_tile_sort(const uint32_t *__restrict__ cols, const uint64_t *__restrict__ s_off,
              const uint32_t *__restrict__ lists, const unsigned *__restrict__ ctr, int ki, int cbits, SegOut o,
              unsigned *__restrict__ overflow) {
    using Sm = TileSmem<T, I, DEDUP>;
    constexpr int W = T / 32;
    extern __shared__ __align__(16) unsigned char ts_raw[];
    Sm &S = *reinterpret_cast<Sm *>(ts_raw);
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    unsigned lbase = 0;
    for (int c = 6; c < 7 + ki; ++c) lbase += ctr[SC_LIST + c];
    const uint32_t *list = lists + lbase;
    const unsigned nj = ctr[SC_JOBS + ki];
    for (unsigned jb = blockIdx.x; jb < nj; jb += gridDim.x) {
        const uint32_t r = list[jb];
        const uint64_t b = s_off[r];
        const int E = (int)(s_off[r + 1] - b);
        if (E > Sm::MAXE) {  // (the plan never lists such rows)
            if (t == 0) atomicOr(overflow, 1u);
            continue;
        }
        const int passes = (cbits + RS_DBITS - 1) / RS_DBITS;
        // coalesced load in input order into the exchange arrays (dedup mode:
        // each value read once; its zero test rides in the position's top bit)
        for (int e = t; e < E; e += T) {
            S.u.x.key[pad33(e)] = cols[b + e];
            uint16_t ix = (uint16_t)e;
            if constexpr (DEDUP) {
                const double v = o.in_vals[b + e];
                if (is_zero(v)) ix |= IDX_ZERO;
                if constexpr (Sm::VSTAGE) S.val[e] = v;
            }
            S.u.x.idx[pad33(e)] = ix;
        }
        __syncthreads();
        // thread t holds positions [t I, t I + I): thread order is input order.
        // v[i] = row position << 16 | rank (16 bits each: E <= 12288)
        const int nv = max(0, min(I, E - t * I));
        uint32_t key[I], v[I];
#pragma unroll
        for (int i = 0; i < I; ++i) {
            if (i < nv) {
                key[i] = S.u.x.key[pad33(t * I + i)];
                v[i] = (uint32_t)S.u.x.idx[pad33(t * I + i)] << 16;
            }
        }
        constexpr uint32_t kColStride = T + T / 32;  // pad33(w T + t) = w kColStride + pad33(t)
        const uint32_t col0 = pad33(t), rake0 = 33u * t;  // pad33(RS_WORDS t + j) = 33 t + j
        for (int p = 0; p < passes; ++p) {
            const int shift = p * RS_DBITS;
            __syncthreads();  // the exchange arrays are read: the counters take their place
            // this thread's column of counters: zeroed and counted by it alone
#pragma unroll 4
            for (int w = 0; w < RS_WORDS; ++w) S.u.ctr[col0 + w * kColStride] = 0;
            // (shared atomics on the thread's own column: no contention, and
            // unlike a load / add / store chain the items' updates pipeline)
#pragma unroll
            for (int i = 0; i < I; ++i) {
                if (i < nv) {
                    const uint32_t d = (key[i] >> shift) & (RS_DIGITS - 1);
                    const uint32_t a = col0 + (d & (RS_WORDS - 1)) * kColStride;
                    const uint32_t sh = (d / RS_WORDS) * 16;  // digits d and d + 32 share a word
                    const uint32_t cv = atomicAdd(&S.u.ctr[a], 1u << sh);
                    v[i] = (v[i] & 0xFFFF0000u) | ((cv >> sh) & 0xFFFFu);  // same digit earlier in this thread
                }
            }
            __syncthreads();
            // raking exclusive scan in (word, thread) order: thread t owns
            // flat counters [RS_WORDS t, RS_WORDS (t + 1)); both 16-bit halves
            // add independently (totals < 2^16)
            uint32_t sum = 0;
#pragma unroll 8
            for (int j = 0; j < RS_WORDS; ++j) sum += S.u.ctr[rake0 + j];
            uint32_t inc = sum;
#pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
                const uint32_t x = __shfl_up_sync(0xffffffffu, inc, d);
                if (lane >= d) inc += x;
            }
            if (lane == 31) S.wsum[warp] = inc;
            __syncthreads();
            uint32_t run = inc - sum, total = 0;
#pragma unroll
            for (int w = 0; w < W; ++w) {
                const uint32_t x = S.wsum[w];
                if (w < warp) run += x;
                total += x;
            }
#pragma unroll
            for (int j0 = 0; j0 < RS_WORDS; j0 += 8) {  // 8 loads in flight, then 8 stores
                uint32_t x[8];
#pragma unroll
                for (int j = 0; j < 8; ++j) x[j] = S.u.ctr[rake0 + j0 + j];
#pragma unroll
                for (int j = 0; j < 8; ++j) {
                    S.u.ctr[rake0 + j0 + j] = run;
                    run += x[j];
                }
            }
            const uint32_t low_total = total & 0xFFFFu;  // entries whose digit is below RS_WORDS
            __syncthreads();
#pragma unroll
            for (int i = 0; i < I; ++i) {
                if (i < nv) {
                    const uint32_t d = (key[i] >> shift) & (RS_DIGITS - 1);
                    const uint32_t a = col0 + (d & (RS_WORDS - 1)) * kColStride;
                    const uint32_t hi = d / RS_WORDS;
                    v[i] += ((S.u.ctr[a] >> (16 * hi)) & 0xFFFFu) + (hi ? low_total : 0u);
                }
            }
            __syncthreads();  // counters read: the exchange arrays take their place
#pragma unroll
            for (int i = 0; i < I; ++i) {
                if (i < nv) {
                    const uint32_t q = pad33(v[i] & 0xFFFFu);
                    S.u.x.key[q] = key[i];
                    S.u.x.idx[q] = (uint16_t)(v[i] >> 16);
                }
            }
            __syncthreads();
            if (p + 1 < passes) {
#pragma unroll
                for (int i = 0; i < I; ++i) {
                    if (i < nv) {
                        key[i] = S.u.x.key[pad33(t * I + i)];
                        v[i] = (uint32_t)S.u.x.idx[pad33(t * I + i)] << 16;
                    }
                }
            }
        }
        if constexpr (!DEDUP) {
            for (int q = t; q < E; q += T) {
                o.keys[b + q] = ((uint64_t)r << cbits) | S.u.x.key[pad33(q)];
                o.idx[b + q] = (uint32_t)(b + S.u.x.idx[pad33(q)]);
            }
        } else {
            // keep = last of a run of equal columns (the last write) and not
            // zero; ex = exclusive count of kept entries
            uint32_t keepm = 0, cnt = 0;
#pragma unroll
            for (int i = 0; i < I; ++i) {
                const int q = t * I + i;
                if (q < E) {
                    const uint32_t k = S.u.x.key[pad33(q)];
                    if ((q + 1 == E || S.u.x.key[pad33(q + 1)] != k) && !(S.u.x.idx[pad33(q)] & IDX_ZERO)) {
                        keepm |= 1u << i;
                        ++cnt;
                    }
                }
            }
            uint32_t inc = cnt;
#pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
                const uint32_t x = __shfl_up_sync(0xffffffffu, inc, d);
                if (lane >= d) inc += x;
            }
            if (lane == 31) S.wsum[warp] = inc;
            __syncthreads();
            uint32_t run = inc - cnt, total = 0;
#pragma unroll
            for (int w = 0; w < W; ++w) {
                const uint32_t x = S.wsum[w];
                if (w < warp) run += x;
                total += x;
            }
#pragma unroll
            for (int i = 0; i < I; ++i) {
                const int q = t * I + i;
                if (q < E) {
                    S.u.x.ex[pad33(q)] = run;
                    run += (keepm >> i) & 1u;
                }
            }
            if (t == 0) {
                S.u.x.ex[pad33(E)] = total;
                o.kept[r] = total;
            }
            __syncthreads();
            for (int q = t; q < E; q += T) {
                const uint32_t e0 = S.u.x.ex[pad33(q)];
                if (S.u.x.ex[pad33(q + 1)] != e0) {
                    const unsigned tp = S.u.x.idx[pad33(q)] & ~IDX_ZERO;
                    o.cols[b + e0] = S.u.x.key[pad33(q)];
                    if constexpr (Sm::VSTAGE) o.vals[b + e0] = S.val[tp];
                    else o.vals[b + e0] = o.in_vals[b + tp];
                }
            }
        }
        __syncthreads();  // shared state is rebuilt by the next row
    }
}

template <int T, int I, bool DEDUP>
int launch_tile_sort(Ctx *c, const uint32_t *cols, const uint64_t *s_off, const uint32_t *lists, const unsigned *ctr,
                     int ki, uint64_t max_rows, int cbits, const SegOut &o, unsigned *overflow, cudaStream_t s) {
    auto k = seg_tile_sort<T, I, DEDUP>;
    constexpr size_t smem = sizeof(TileSmem<T, I, DEDUP>);
    SPG_CUDA_TRY(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int per_sm = 0;
    SPG_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, T, smem));
    // persistent blocks over a list whose length stays on the device
    const uint64_t grid = std::min<uint64_t>(max_rows, (uint64_t)c->n_sms * (uint64_t)std::max(per_sm, 1));
    if (grid == 0) return SPG_OK;
    k<<<(unsigned)grid, T, smem, s>>>(cols, s_off, lists, ctr, ki, cbits, o, overflow);
    SPG_LAUNCH_CHECK();
    return SPG_OK;
}

template <bool DEDUP>
int seg_sort(Ctx *c, const uint32_t *cols, const uint64_t *s_off, uint64_t m, uint64_t n_rows, int cbits,
             const SegOut &o, bool *done, cudaStream_t s) {
    *done = false;
    if (cbits > SEG_MAX_CBITS || m > 0xFFFFFFFFull) return SPG_OK;
    DevBuf ctr_b, lists_b;
    SPG_TRY(ctr_b.alloc(2 * SC_N * sizeof(unsigned), s));  // counters, then the fill cursors
    SPG_TRY(lists_b.alloc(n_rows * sizeof(uint32_t), s));
    SPG_CUDA_TRY(cudaMemsetAsync(ctr_b.ptr, 0, 2 * SC_N * sizeof(unsigned), s));
    unsigned *ctr = ctr_b.as<unsigned>(), *cur = ctr + SC_N, *ovf = ctr + SC_OVERFLOW;
    uint32_t *lists = lists_b.as<uint32_t>();
    const unsigned gr = grid_for(n_rows, 256, (unsigned)c->n_sms * 8);
    seg_count<<<gr, 256, 0, s>>>(s_off, n_rows, ctr);
    SPG_LAUNCH_CHECK();
    seg_place<DEDUP><<<gr, 256, 0, s>>>(cols, s_off, n_rows, cbits, ctr, cur, lists, o);
    SPG_LAUNCH_CHECK();
    seg_short_sort<DEDUP><<<grid_for((n_rows + 31) / 32, 8, (unsigned)c->n_sms * 16), 256, 0, s>>>(cols, s_off, n_rows,
                                                                                                cbits, o);
    SPG_LAUNCH_CHECK();
    // (8 blocks per SM: twice what fits at once, which balanced rows of
    // unequal length better than one wave)
    if (cbits <= 22) seg_medium_sort<uint32_t, DEDUP><<<(unsigned)c->n_sms * 8, 256, 0, s>>>(cols, s_off, lists, ctr, cbits, o);
    else seg_medium_sort<uint64_t, DEDUP><<<(unsigned)c->n_sms * 8, 256, 0, s>>>(cols, s_off, lists, ctr, cbits, o);
    SPG_LAUNCH_CHECK();
    SPG_TRY((launch_tile_sort<TS0_T, TS0_I, DEDUP>(c, cols, s_off, lists, ctr, 0, m / (SEG_MEDIUM + 1) + 1, cbits,
                                                   o, ovf, s)));
    SPG_TRY((launch_tile_sort<TS1_T, TS1_I, DEDUP>(c, cols, s_off, lists, ctr, 1, m / (TS0 + 1) + 1, cbits, o, ovf,
                                                   s)));
    SPG_TRY((launch_tile_sort<TS2_T, TS2_I, DEDUP>(c, cols, s_off, lists, ctr, 2, m / (TS1 + 1) + 1, cbits, o, ovf,
                                                   s)));
    unsigned h = 1u;
    SPG_CUDA_TRY(cudaMemcpyAsync(&h, ovf, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
    SPG_TRY(c->phase_sync(s));
    *done = h == 0;
    return SPG_OK;
}

}  // namespace

int sort_grouped_rows(Ctx *c, const uint32_t *rows, const uint32_t *cols, const uint64_t *s_off, uint64_t m,
                      uint64_t n_rows, int cbits, uint64_t *keys_out, uint32_t *idx_out, bool *done, cudaStream_t s) {
    (void)rows;  // the rows are s_off's
    if (m == 0) {
        *done = true;
        return SPG_OK;
    }
    SegOut o{};
    o.keys = keys_out;
    o.idx = idx_out;
    return seg_sort<false>(c, cols, s_off, m, n_rows, cbits, o, done, s);
}

int dedup_grouped_rows(Ctx *c, const uint32_t *cols, const double *vals, const uint64_t *s_off, uint64_t m,
                       uint64_t n_rows, int cbits, uint32_t *out_cols, double *out_vals, uint64_t *kept, bool *done,
                       cudaStream_t s) {
    SegOut o{};
    o.in_vals = vals;
    o.cols = out_cols;
    o.vals = out_vals;
    o.kept = kept;
    if (m == 0) {
        SPG_CUDA_TRY(cudaMemsetAsync(kept, 0, n_rows * sizeof(uint64_t), s));
        *done = true;
        return SPG_OK;
    }
    return seg_sort<true>(c, cols, s_off, m, n_rows, cbits, o, done, s);
}

}  // namespace spg
