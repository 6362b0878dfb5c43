// spg_spgemm_sort.cu — SPG_SPGEMM_WARPSORT_{64,128,256}: C = A * B with
// Spira's Gustavson order (serial/spgemm.hpp:28-48: for row i, for each a_ik
// in ascending k, acc[j] += a_ik * b_kj; keep acc != 0) from a per-row sort
// instead of a k-way merge.
//
// Rows are cut into tiles of consecutive rows (at most 128 rows and a
// product budget; rows with more than HB products or HB A entries are
// "heavy" and form one-row tiles whose results come from expand - sort -
// compress, spg_spgemm.cu). A block of four warps takes tiles in launch
// order (a ticket from an atomic counter) and, per tile:
//
//   1. per row, one warp: the row's products are expanded over the lanes
//      (slot s = position in (A entry, B entry) order), multiplied
//      (__dmul_rn, all lanes busy), and their keys (column << SB | slot)
//      bitonic-sorted in registers. Column order with slot order inside a
//      column is exactly ascending k for each (i, j). A row of at most 32 A
//      entries whose B rows fit power-of-two blocks of the network places
//      each B row (already sorted) in its own block and starts the network
//      at the first merging stage; other rows take the A entry owning a
//      slot from a max-scan of the entries' first slots;
//   2. the same warp: runs of equal columns are found from the neighbours'
//      columns (shuffles). If the row has none longer than one product (a
//      warp vote), every product is its own sum; otherwise the sorted
//      (column, product) pairs go to the tile's shared memory and the lane
//      holding a run's first product sums it left to right (__dadd_rn from
//      the run's first product: +0.0 + p1 = p1 whenever the sum can be
//      kept, so starting at p1 changes no kept value). The kept sums (not
//      +-0) are ranked with ballots and compacted in place, and the row's
//      kept count goes to the tile;
//   3. the tile's kept count goes through an ordered scan (decoupled
//      look-back over the tiles' published counts, 32 predecessors per step
//      by one warp, every wait bounded), and the tile writes its rows'
//      offsets and entries (a warp per row) straight into C, so no
//      compaction pass and no second scan follow.
//
// A wait that runs out (about a second) sets a bit in the context's status
// word and poisons the tile, so later tiles stop too; the call then returns
// SPG_ERR_DEVICE_TIMEOUT and C is not installed. Tickets follow launch order,
// so every tile a block waits for belongs to a block that already runs.
#include "spg_internal.cuh"

namespace spg {
namespace {

constexpr int SGS_WARPS = 4;
constexpr int SGS_THREADS = 32 * SGS_WARPS;
constexpr uint32_t SGS_RB = SGS_THREADS;  // rows per tile at most: one thread each in the block scan
constexpr unsigned SGS_STATUS_TIMEOUT = 0x10u;
constexpr long long SGS_WAIT_CYCLES = 1ll << 31;  // ~1 s at 2 GHz

constexpr unsigned long long LB_AGG = 1ull << 62;      // tile published its own count
constexpr unsigned long long LB_PREFIX = 2ull << 62;   // tile published its inclusive prefix
constexpr unsigned long long LB_POISON = 3ull << 62;   // tile gave up: everything after stops
constexpr unsigned long long LB_VALUE = (1ull << 62) - 1;

struct SgsArgs {
    const uint64_t *aoff;
    const uint32_t *acols;
    const double *avals;
    const uint64_t *boff;
    const uint32_t *bcols;
    const double *bvals;
    uint64_t m;
    const uint64_t *pofs;        // products per row, scanned (pofs[m] = P)
    const uint64_t *tile_start;  // first row of each tile, [n_tiles + 1]
    const uint64_t *n_tiles;     // device scalar
    const uint64_t *hbeg;        // heavy rows: first entry in (hcol, hval) ...
    const uint32_t *hcnt;        // ... and kept count (0 for other rows)
    const uint32_t *hcol;
    const double *hval;
    unsigned long long *tstate;  // look-back words, one per tile, zeroed
    unsigned long long *ticket;  // zeroed
    uint64_t *coff;
    uint32_t *ccols;
    double *cvals;
    unsigned int *status;
    uint32_t tpb;                // product budget of a tile (shared memory)
    long long wait_cycles;       // bound of every look-back wait
    uint64_t fixed_rows;         // nonzero: no heavy rows; tile t = rows [t F, t F + F), pofs = raw counts
};

__device__ __forceinline__ bool sgs_heavy(const uint64_t *aoff, const uint64_t *pofs, uint64_t i, uint32_t hb) {
    return pofs[i + 1] - pofs[i] > hb || aoff[i + 1] - aoff[i] > hb;
}

// Products per row (pofs[i]) and the products of heavy rows only (hp[i], 0
// for the others); entry m of both is 0; *n_heavy counts heavy rows and
// *p_total sums the products (one atomic per block each).
__global__ void __launch_bounds__(256) sgs_products(const uint64_t *__restrict__ aoff,
                                                    const uint32_t *__restrict__ acols,
                                                    const uint64_t *__restrict__ boff, uint64_t m, uint32_t hb,
                                                    uint64_t *__restrict__ pofs, uint64_t *__restrict__ hp,
                                                    unsigned long long *__restrict__ n_heavy,
                                                    unsigned long long *__restrict__ p_total) {
    __shared__ unsigned long long s_p[8], s_h[8];
    const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    uint64_t p = 0;
    bool heavy = false;
    if (i < m) {
        const uint64_t a0 = aoff[i], a1 = aoff[i + 1];
        for (uint64_t ka = a0; ka < a1; ++ka) {
            const uint32_t k = acols[ka];
            p += boff[k + 1] - boff[k];
        }
        heavy = p > hb || a1 - a0 > hb;
        pofs[i] = p;
        hp[i] = heavy ? p : 0;
    } else if (i == m) {
        pofs[m] = 0;
        hp[m] = 0;
    }
    unsigned long long sp = p, sh = heavy ? 1ull : 0ull;
#pragma unroll
    for (int o = 16; o; o >>= 1) {
        sp += __shfl_xor_sync(0xffffffffu, sp, o);
        sh += __shfl_xor_sync(0xffffffffu, sh, o);
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) {
        s_p[warp] = sp;
        s_h[warp] = sh;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long bp = 0, bh = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
            bp += s_p[w];
            bh += s_h[w];
        }
        if (bp) atomicAdd(p_total, bp);
        if (bh) atomicAdd(n_heavy, bh);
    }
}

// Row i starts a tile: every SGS_RB-th row, heavy rows and the rows after
// them, and the first row whose product offset enters a new window of W
// products (so a tile holds fewer than W + hb products).
__device__ __forceinline__ bool sgs_tile_start(const uint64_t *aoff, const uint64_t *pofs, uint64_t i, uint32_t hb,
                                               uint64_t W) {
    if (i % SGS_RB == 0) return true;
    if (sgs_heavy(aoff, pofs, i, hb) || sgs_heavy(aoff, pofs, i - 1, hb)) return true;
    return pofs[i] / W != pofs[i - 1] / W;
}

__global__ void sgs_tile_flags(const uint64_t *__restrict__ aoff, const uint64_t *__restrict__ pofs, uint64_t m,
                               uint32_t hb, uint64_t W, uint64_t *__restrict__ flag) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < m; i += (uint64_t)gridDim.x * blockDim.x)
        flag[i] = sgs_tile_start(aoff, pofs, i, hb, W) ? 1 : 0;
}

// pos: the flags' exclusive scan; tile_start[n_tiles] = m.
__global__ void sgs_tile_scatter(const uint64_t *__restrict__ aoff, const uint64_t *__restrict__ pofs, uint64_t m,
                                 uint32_t hb, uint64_t W, const uint64_t *__restrict__ pos,
                                 const uint64_t *__restrict__ n_tiles, uint64_t *__restrict__ tile_start) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < m; i += (uint64_t)gridDim.x * blockDim.x) {
        if (sgs_tile_start(aoff, pofs, i, hb, W)) tile_start[pos[i]] = i;
        if (i == 0) tile_start[*n_tiles] = m;
    }
}

// Heavy rows' entries in expand - sort - compress's output (sorted by row).
__global__ void sgs_heavy_index(const uint32_t *__restrict__ crow, uint64_t n, uint64_t *__restrict__ hbeg,
                                uint32_t *__restrict__ hcnt) {
    for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < n; e += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t r = crow[e];
        if (e == 0 || crow[e - 1] != r) hbeg[r] = e;
        atomicAdd(hcnt + r, 1u);
    }
}

// One row, one warp: expand, multiply, sort, sum the runs of equal columns
// and compact; leaves the row's kept (column, sum) pairs at s_col / s_prod
// [reg, reg + kept) and returns kept (the same in every lane). Uses the
// warp's w_a / w_b / w_own (HB entries each). P <= 32 E, A's row has <= HB
// entries.
template <int E, int SB, class K>
__device__ __forceinline__ uint32_t sgs_row(const SgsArgs &g, uint64_t i, uint32_t reg, uint32_t P, uint32_t *s_col, double *s_prod,
                            double *w_a, int64_t *w_b, uint16_t *w_own, int lane) {
    const uint64_t ab = g.aoff[i];
    const uint32_t r = (uint32_t)(g.aoff[i + 1] - ab);
    // A entries: slot ranges [ex, ex + L) by a warp scan of their B row
    // lengths. Up to 32 entries sit one per lane; then, if r blocks of
    // 2^lg >= every L fit the network, entry t's products (already ascending
    // in column: B's rows are sorted) fill block t, reversed in odd blocks,
    // so every block is sorted in the direction the network's stage 2^lg
    // leaves it and the sort starts at stage 2^(lg+1).
    uint32_t L1 = 0, ex1 = 0;
    uint64_t bs1 = 0;
    double a1 = 0.0;
    int lg = 0;
    bool runs = false;
    if (r <= 32) {
        if ((uint32_t)lane < r) {
            const uint32_t k = g.acols[ab + lane];
            a1 = g.avals[ab + lane];
            bs1 = g.boff[k];
            L1 = (uint32_t)(g.boff[k + 1] - bs1);
        }
        uint32_t incl = L1;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t v = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += v;
        }
        ex1 = incl - L1;
        const uint32_t lmax = __reduce_max_sync(0xffffffffu, L1);
        lg = lmax <= 1u ? 0 : 32 - __clz((int)(lmax - 1u));
        runs = lg >= 1 && (r << lg) <= 32u * E;
        if (!runs) {
            for (uint32_t s = lane; s < P; s += 32) w_own[s] = 0;
            __syncwarp();
        }
        if ((uint32_t)lane < r) {
            w_a[lane] = a1;
            w_b[lane] = (int64_t)bs1 - (int64_t)ex1;  // B entry of slot s = w_b[t] + s
            if (!runs && L1) w_own[ex1] = (uint16_t)lane;
        }
    } else {
        for (uint32_t s = lane; s < P; s += 32) w_own[s] = 0;
        __syncwarp();
        uint32_t base = 0;
        for (uint32_t t0 = 0; t0 < r; t0 += 32) {
            const uint32_t t = t0 + lane;
            uint32_t L = 0;
            uint64_t bs = 0;
            double a = 0.0;
            if (t < r) {
                const uint32_t k = g.acols[ab + t];
                a = g.avals[ab + t];
                bs = g.boff[k];
                L = (uint32_t)(g.boff[k + 1] - bs);
            }
            uint32_t incl = L;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t v = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= o) incl += v;
            }
            const uint32_t ex = base + incl - L;
            if (t < r) {
                w_a[t] = a;
                w_b[t] = (int64_t)bs - (int64_t)ex;
                if (L) w_own[ex] = (uint16_t)t;  // distinct: entries with products start at distinct slots
            }
            base += __shfl_sync(0xffffffffu, incl, 31);
        }
    }
    __syncwarp();
    K key[E];
    if (runs) {
        const uint32_t bm = (1u << lg) - 1u;
#pragma unroll
        for (int e = 0; e < E; ++e) {
            const uint32_t q = 32u * e + lane;
            const uint32_t t = q >> lg;  // < 32 as E is minimal for P; t >= r (padding) in any case
            const uint32_t u = (t & 1u) ? bm - (q & bm) : (q & bm);
            const uint32_t ext = __shfl_sync(0xffffffffu, ex1, (int)(t & 31u));
            const uint32_t Lt = __shfl_sync(0xffffffffu, L1, (int)(t & 31u));
            if (t < r && u < Lt) {
                const uint32_t s = ext + u;
                const uint64_t bi = (uint64_t)(w_b[t] + (int64_t)s);
                const uint32_t col = g.bcols[bi];
                s_prod[reg + s] = __dmul_rn(w_a[t], g.bvals[bi]);
                key[e] = ((K)col << SB) | (K)s;
            } else {
                key[e] = ~(K)0;  // above every real key: padding sorts last
            }
        }
    } else {
        // slots: element 32 e + lane; owner = last entry starting at or before it
        uint32_t carry = 0;
#pragma unroll
        for (int e = 0; e < E; ++e) {
            const uint32_t s = 32u * e + lane;
            uint32_t o = s < P ? (uint32_t)w_own[s] : 0u;
#pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
                const uint32_t v = __shfl_up_sync(0xffffffffu, o, d);
                if (lane >= d) o = max(o, v);
            }
            o = max(o, carry);
            carry = __shfl_sync(0xffffffffu, o, 31);
            if (s < P) {
                const uint64_t bi = (uint64_t)(w_b[o] + (int64_t)s);
                const uint32_t col = g.bcols[bi];
                s_prod[reg + s] = __dmul_rn(w_a[o], g.bvals[bi]);
                key[e] = ((K)col << SB) | (K)s;
            } else {
                key[e] = ~(K)0;  // above every real key: padding sorts last
            }
        }
    }
    warp_bitonic<E, K>(key, lane, runs ? 2 << lg : 2);
    __syncwarp();
    // products in sorted order; a run of equal columns starts at a head
    // element (its predecessor's column differs) and continues while the
    // successor's column is the same: neighbours' columns by shuffles
    double pv[E];
    uint32_t col[E];
    bool head[E], cont = false;
#pragma unroll
    for (int e = 0; e < E; ++e) {
        const uint32_t q = 32u * e + lane;
        pv[e] = q < P ? s_prod[reg + (uint32_t)(key[e] & (K)((1u << SB) - 1u))] : 0.0;
        col[e] = (uint32_t)(key[e] >> SB);
    }
#pragma unroll
    for (int e = 0; e < E; ++e) {
        const uint32_t q = 32u * e + lane;
        uint32_t pc = __shfl_up_sync(0xffffffffu, col[e], 1);
        uint32_t nc = __shfl_down_sync(0xffffffffu, col[e], 1);
        if (e > 0) {
            const uint32_t v = __shfl_sync(0xffffffffu, col[e > 0 ? e - 1 : 0], 31);
            if (lane == 0) pc = v;
        }
        if (e + 1 < E) {
            const uint32_t v = __shfl_sync(0xffffffffu, col[e + 1 < E ? e + 1 : e], 0);
            if (lane == 31) nc = v;
        }
        head[e] = q < P && (q == 0 || pc != col[e]);
        cont = cont || (q + 1 < P && nc == col[e]);
    }
    bool keep[E];
    if (__any_sync(0xffffffffu, cont)) {
        // some run is longer than one product: the head lane sums it in slot
        // order (Spira's order) from the sorted copy in shared memory
        __syncwarp();  // every gather done before the sorted copy lands
#pragma unroll
        for (int e = 0; e < E; ++e) {
            const uint32_t q = 32u * e + lane;
            if (q < P) {
                s_col[reg + q] = col[e];
                s_prod[reg + q] = pv[e];
            }
        }
        __syncwarp();
#pragma unroll
        for (int e = 0; e < E; ++e) {
            const uint32_t q = 32u * e + lane;
            keep[e] = false;
            if (head[e]) {
                double acc = pv[e];
                for (uint32_t r = q + 1; r < P && s_col[reg + r] == col[e]; ++r) acc = __dadd_rn(acc, s_prod[reg + r]);
                pv[e] = acc;
                keep[e] = !is_zero(acc);  // spgemm.hpp:44: v != V{}
            }
        }
    } else {
        // every run is one product: its sum is the product itself
#pragma unroll
        for (int e = 0; e < E; ++e) keep[e] = head[e] && !is_zero(pv[e]);  // spgemm.hpp:44
    }
    __syncwarp();  // every gather and run read before the compacted writes land
    uint32_t kept = 0;
    const unsigned lt = (1u << lane) - 1u;
#pragma unroll
    for (int e = 0; e < E; ++e) {
        const unsigned bal = __ballot_sync(0xffffffffu, keep[e]);
        if (keep[e]) {
            const uint32_t w = reg + kept + (uint32_t)__popc(bal & lt);
            s_col[w] = col[e];
            s_prod[w] = pv[e];
        }
        kept += (uint32_t)__popc(bal);
    }
    __syncwarp();
    return kept;
}

// Ordered scan of the tiles' counts, by one warp: lane l reads the word of
// tile p - l, so each step covers 32 predecessors. (Reading 8 words per lane,
// 256 per step, measured slower: 0.73 against 0.43 ms on the 200k x 8
// product with 2048-product tiles.) Returns false if the tile had to give up
// (timeout, or an earlier tile gave up). Lane 0 publishes.
__device__ bool sgs_lookback(const SgsArgs &g, uint64_t t, uint64_t total, uint64_t *base, int lane) {
    if (t == 0) {
        if (lane == 0) atomicExch(g.tstate, LB_PREFIX | total);
        *base = 0;
        return true;
    }
    if (lane == 0) atomicExch(g.tstate + t, LB_AGG | total);
    uint64_t excl = 0;
    int64_t p = (int64_t)t - 1;  // nearest predecessor of the window
    const long long t0 = clock64();
    while (true) {
        const int64_t q = p - lane;
        const unsigned long long v = q >= 0 ? *(volatile unsigned long long *)(g.tstate + q) : 0ull;
        const unsigned long long st = v & ~LB_VALUE;
        const unsigned pref = __ballot_sync(0xffffffffu, q >= 0 && st == LB_PREFIX);
        // lanes up to the nearest prefix (tile 0 always publishes one, so a
        // window reaching q < 0 holds it at a lower lane)
        const unsigned need = pref ? (pref & (0u - pref)) * 2u - 1u : 0xffffffffu;
        const unsigned waiting = __ballot_sync(0xffffffffu, q >= 0 && st == 0) & need;
        const unsigned poison = __ballot_sync(0xffffffffu, q >= 0 && st == LB_POISON) & need;
        if (poison) {
            if (lane == 0) atomicExch(g.tstate + t, LB_POISON);
            return false;
        }
        if (waiting) {
            if (clock64() - t0 > g.wait_cycles) {
                if (lane == 0) {
                    atomicOr(g.status, SGS_STATUS_TIMEOUT);
                    atomicExch(g.tstate + t, LB_POISON);
                }
                return false;
            }
            __nanosleep(32);
            continue;
        }
        unsigned long long add = ((need >> lane) & 1u) ? (v & LB_VALUE) : 0ull;
#pragma unroll
        for (int o = 16; o; o >>= 1) add += __shfl_xor_sync(0xffffffffu, add, o);
        excl += add;
        if (pref) break;
        p -= 32;
    }
    if (lane == 0) atomicExch(g.tstate + t, LB_PREFIX | (excl + total));
    *base = excl;
    return true;
}

template <int HB, class K>
__global__ void __launch_bounds__(SGS_THREADS) sgs_tiles(SgsArgs g) {
    constexpr int SB = HB == 64 ? 6 : HB == 128 ? 7 : 8;
    static_assert((1 << SB) == HB, "HB is a power of two");
    extern __shared__ __align__(16) unsigned char sgs_smem[];
    // row j of the tile keeps its products at [pofs - p0 + j, + P): one slot of
    // skew per row, so rows of equal length do not all start in the same
    // shared-memory bank
    const uint32_t slots = g.tpb + SGS_RB;
    double *s_prod = reinterpret_cast<double *>(sgs_smem);
    uint32_t *s_col = reinterpret_cast<uint32_t *>(s_prod + slots);
    double *w_a_all = reinterpret_cast<double *>(s_col + slots);  // slots is even: 8-byte aligned
    int64_t *w_b_all = reinterpret_cast<int64_t *>(w_a_all + SGS_WARPS * HB);
    uint16_t *w_own_all = reinterpret_cast<uint16_t *>(w_b_all + SGS_WARPS * HB);
    __shared__ uint64_t sh_tile, sh_base;
    __shared__ uint32_t sh_reg[SGS_RB];
    __shared__ uint32_t sh_excl[SGS_RB + 1];
    __shared__ uint32_t sh_kept[SGS_RB];
    __shared__ uint32_t sh_P[32];  // fixed tiles: products of each row
    __shared__ uint32_t sh_wsum[SGS_WARPS];
    __shared__ int sh_ok;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (tid == 0) sh_tile = atomicAdd(g.ticket, 1ull);
    __syncthreads();
    const uint64_t t = sh_tile;
    const bool fixed = g.fixed_rows != 0;
    if (t >= (fixed ? (g.m + g.fixed_rows - 1) / g.fixed_rows : *g.n_tiles)) return;
    uint64_t row0, row1, p0 = 0;
    if (fixed) {
        row0 = t * g.fixed_rows;
        row1 = min(g.m, row0 + g.fixed_rows);
    } else {
        row0 = g.tile_start[t];
        row1 = g.tile_start[t + 1];
        p0 = g.pofs[row0];
    }
    const uint32_t nr = (uint32_t)(row1 - row0);
    const bool heavy_tile = !fixed && nr == 1 && sgs_heavy(g.aoff, g.pofs, row0, HB);
    if (fixed) {  // the rows' regions: an exclusive scan of their products (at most 32 rows)
        if (warp == 0) {
            const uint32_t P = (uint32_t)lane < nr ? (uint32_t)g.pofs[row0 + lane] : 0u;
            uint32_t inc = P;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t v = __shfl_up_sync(0xffffffffu, inc, o);
                if (lane >= o) inc += v;
            }
            if ((uint32_t)lane < nr) {
                sh_P[lane] = P;
                sh_reg[lane] = inc - P + (uint32_t)lane;
            }
        }
        __syncthreads();
    }
    uint32_t cnt = 0;
    if (!heavy_tile) {
        double *w_a = w_a_all + warp * HB;
        int64_t *w_b = w_b_all + warp * HB;
        uint16_t *w_own = w_own_all + warp * HB;
        for (uint32_t j = warp; j < nr; j += SGS_WARPS) {
            const uint64_t i = row0 + j;
            const uint32_t reg = fixed ? sh_reg[j] : (uint32_t)(g.pofs[i] - p0) + j;
            const uint32_t P = fixed ? sh_P[j] : (uint32_t)(g.pofs[i + 1] - g.pofs[i]);
            uint32_t kept = 0;
            if (P == 0) kept = 0;
            else if (P <= 32) kept = sgs_row<1, SB, K>(g, i, reg, P, s_col, s_prod, w_a, w_b, w_own, lane);
            else if (P <= 64) kept = sgs_row<2, SB, K>(g, i, reg, P, s_col, s_prod, w_a, w_b, w_own, lane);
            else if constexpr (HB >= 128) {
                if (P <= 128) kept = sgs_row<4, SB, K>(g, i, reg, P, s_col, s_prod, w_a, w_b, w_own, lane);
                else if constexpr (HB >= 256) kept = sgs_row<8, SB, K>(g, i, reg, P, s_col, s_prod, w_a, w_b, w_own, lane);
            }
            __syncwarp();
            if (lane == 0) {
                sh_kept[j] = kept;
                sh_reg[j] = reg;
            }
        }
        __syncthreads();
        if ((uint32_t)tid < nr) cnt = sh_kept[tid];
    } else if (tid == 0) {
        cnt = g.hcnt[row0];
    }
    // block exclusive scan of the rows' kept counts
    uint32_t incl = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t v = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += v;
    }
    if (lane == 31) sh_wsum[warp] = incl;
    __syncthreads();
    uint32_t before = 0, total = 0;
#pragma unroll
    for (int w = 0; w < SGS_WARPS; ++w) {
        if (w < warp) before += sh_wsum[w];
        total += sh_wsum[w];
    }
    const uint32_t excl = before + incl - cnt;
    if ((uint32_t)tid < nr) sh_excl[tid] = excl;
    if (warp == 0) {
        uint64_t b = 0;
        const bool ok = sgs_lookback(g, t, total, &b, lane);
        if (lane == 0) {
            sh_excl[nr] = total;
            sh_ok = ok ? 1 : 0;
            sh_base = b;
        }
    }
    __syncthreads();
    if (!sh_ok) return;
    const uint64_t base = sh_base;
    if ((uint32_t)tid < nr) g.coff[row0 + tid] = base + excl;
    if (tid == 0 && row1 == g.m) g.coff[g.m] = base + total;
    if (!heavy_tile) {
        // a warp per row, lanes over its kept entries (no search for the row)
        for (uint32_t j = warp; j < nr; j += SGS_WARPS) {
            const uint32_t e0 = sh_excl[j], n = sh_excl[j + 1] - e0, src = sh_reg[j];
            for (uint32_t q = lane; q < n; q += 32) {
                g.ccols[base + e0 + q] = s_col[src + q];
                g.cvals[base + e0 + q] = s_prod[src + q];
            }
        }
    } else {
        const uint64_t hb0 = total ? g.hbeg[row0] : 0;
        for (uint32_t q = tid; q < total; q += SGS_THREADS) {
            g.ccols[base + q] = g.hcol[hb0 + q];
            g.cvals[base + q] = g.hval[hb0 + q];
        }
    }
}

// Self-test of the bounded wait: tile 1 looks back at a tile 0 that never
// publishes (its word stays zero), so the wait runs out after wait_cycles;
// out[0] = 1 if the look-back gave up, out[1] = the poison word it left.
__global__ void sgs_wait_selftest(SgsArgs g, unsigned long long *out) {
    const int lane = threadIdx.x & 31;
    uint64_t base = 0;
    const bool ok = sgs_lookback(g, 1, 5, &base, lane);
    if (lane == 0) {
        out[0] = ok ? 0ull : 1ull;
        out[1] = *(volatile unsigned long long *)(g.tstate + 1);
    }
}

struct SortConfig {
    uint32_t hb;   // products (and A entries) per warp-sorted row at most
    uint32_t tpb;  // products per tile at most (shared memory)
};

SortConfig sort_config(int variant) {
    switch (variant) {
        case SPG_SPGEMM_WARPSORT_64: return {64, 1024};
        case SPG_SPGEMM_WARPSORT_128: return {128, 2048};
        default: return {256, 4096};
    }
}

size_t sgs_smem_bytes(const SortConfig &cf) {
    return (size_t)(cf.tpb + SGS_RB) * (sizeof(double) + sizeof(uint32_t)) +
           (size_t)SGS_WARPS * cf.hb * (sizeof(double) + sizeof(int64_t) + sizeof(uint16_t));
}

template <int HB, class K>
int launch_tiles(const SgsArgs &g, unsigned grid, size_t smem, cudaStream_t s) {
    SPG_CUDA_TRY(cudaFuncSetAttribute(sgs_tiles<HB, K>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    sgs_tiles<HB, K><<<grid, SGS_THREADS, smem, s>>>(g);
    SPG_LAUNCH_CHECK();
    return SPG_OK;
}

}  // namespace

int spgemm_warpsort(Ctx *c, const Csr *A, const Csr *B, Csr *Cm, int variant, cudaStream_t s) {
    const SortConfig cf = sort_config(variant);
    const uint64_t m = A->n_rows, n = B->n_cols;
    const unsigned gmax = (unsigned)c->n_sms * 32;
    int rc = SPG_OK;
    DevBuf pofs, hp, nh_dev;
    SPG_TRY(pofs.alloc((m + 1) * sizeof(uint64_t), s));
    SPG_TRY(hp.alloc((m + 1) * sizeof(uint64_t), s));
    SPG_TRY(nh_dev.alloc(3 * sizeof(uint64_t), s));
    SPG_CUDA_TRY(cudaMemsetAsync(nh_dev.ptr, 0, 3 * sizeof(uint64_t), s));
    unsigned long long *nh = reinterpret_cast<unsigned long long *>(nh_dev.as<uint64_t>());
    sgs_products<<<grid_for(m + 1, 256), 256, 0, s>>>(A->d_off(), A->d_cols(), B->d_off(), m, cf.hb,
                                                     pofs.as<uint64_t>(), hp.as<uint64_t>(), nh, nh + 1);
    SPG_LAUNCH_CHECK();
    uint64_t h[3] = {0, 0, 0};  // heavy rows, products, heavy products
    SPG_CUDA_TRY(cudaMemcpyAsync(h, nh_dev.ptr, 2 * sizeof(uint64_t), cudaMemcpyDeviceToHost, s));
    SPG_TRY(c->phase_sync(s));
    // No heavy row: tiles of F consecutive rows (F rows of at most hb products fill a tile's budget
    // at most), their regions scanned inside the kernel: no scan, no tile plan.
    const uint64_t F = h[0] ? 0 : cf.tpb / cf.hb;
    if (h[0]) {  // heavy rows: the row offsets for the tile plan, and the heavy rows' products
        SPG_TRY(exclusive_scan_u64(c, pofs.as<uint64_t>(), m + 1, nh_dev.as<uint64_t>() + 1, s));
        SPG_TRY(exclusive_scan_u64(c, hp.as<uint64_t>(), m + 1, nh_dev.as<uint64_t>() + 2, s));
        SPG_CUDA_TRY(cudaMemcpyAsync(h + 2, nh_dev.as<uint64_t>() + 2, sizeof(uint64_t), cudaMemcpyDeviceToHost, s));
        SPG_TRY(c->phase_sync(s));
    }
    const uint64_t n_heavy = h[0], P = h[1], HP = h[2];
    if (P >= (1ull << 32))
        return set_error(SPG_ERR_UNSUPPORTED, "spgemm: %llu products exceed 2^32-1", (unsigned long long)P);
    DevBuf off, cols, vals;
    SPG_TRY(off.alloc(csr_off_elems(m) * sizeof(uint64_t), s));
    if (m == 0 || P == 0) {  // no products: every row empty
        SPG_CUDA_TRY(cudaMemsetAsync(off.ptr, 0, csr_off_elems(m) * sizeof(uint64_t), s));
        SPG_TRY(cols.alloc(csr_alloc_elems(0) * sizeof(uint32_t), s));
        SPG_TRY(vals.alloc(csr_alloc_elems(0) * sizeof(double), s));
        SPG_TRY(c->phase_sync(s));
        spgemm_install(Cm, m, n, std::move(off), std::move(cols), std::move(vals), 0);
        return SPG_OK;
    }
    // heavy rows: expand - sort - compress, indexed by row
    EscOut eo;
    DevBuf hbeg, hcnt;
    if (n_heavy) {
        SPG_TRY(spgemm_esc(c, A, B, hp.as<uint64_t>(), HP, bits_for(m), bits_for(n), &eo, s));
        SPG_TRY(hbeg.alloc(m * sizeof(uint64_t), s));
        SPG_TRY(hcnt.alloc(m * sizeof(uint32_t), s));
        SPG_CUDA_TRY(cudaMemsetAsync(hcnt.ptr, 0, m * sizeof(uint32_t), s));
        if (eo.n) {
            sgs_heavy_index<<<grid_for(eo.n, 256, gmax), 256, 0, s>>>(eo.crow.as<uint32_t>(), eo.n,
                                                                     hbeg.as<uint64_t>(), hcnt.as<uint32_t>());
            SPG_LAUNCH_CHECK();
        }
    }
    hp.release();
    // tiles
    const uint64_t W = cf.tpb - cf.hb;
    const uint64_t t_max = F ? (m + F - 1) / F : (m + SGS_RB - 1) / SGS_RB + P / W + 2 * n_heavy + 3;
    DevBuf flag, tile_start, tstate, ticket;
    SPG_TRY(tstate.alloc(t_max * sizeof(unsigned long long), s));
    SPG_TRY(ticket.alloc(2 * sizeof(uint64_t), s));  // [0] ticket counter, [1] tile count
    SPG_CUDA_TRY(cudaMemsetAsync(tstate.ptr, 0, t_max * sizeof(unsigned long long), s));
    SPG_CUDA_TRY(cudaMemsetAsync(ticket.ptr, 0, 2 * sizeof(uint64_t), s));
    if (!F) {
        SPG_TRY(flag.alloc((m + 1) * sizeof(uint64_t), s));
        SPG_TRY(tile_start.alloc((t_max + 1) * sizeof(uint64_t), s));
        sgs_tile_flags<<<grid_for(m, 256, gmax), 256, 0, s>>>(A->d_off(), pofs.as<uint64_t>(), m, cf.hb, W,
                                                             flag.as<uint64_t>());
        SPG_LAUNCH_CHECK();
        SPG_TRY(exclusive_scan_u64(c, flag.as<uint64_t>(), m, ticket.as<uint64_t>() + 1, s));
        sgs_tile_scatter<<<grid_for(m, 256, gmax), 256, 0, s>>>(A->d_off(), pofs.as<uint64_t>(), m, cf.hb, W,
                                                               flag.as<uint64_t>(), ticket.as<uint64_t>() + 1,
                                                               tile_start.as<uint64_t>());
        SPG_LAUNCH_CHECK();
    }
    // C at the products' upper bound (kept entries <= products)
    SPG_TRY(cols.alloc(csr_alloc_elems(P) * sizeof(uint32_t), s));
    SPG_TRY(vals.alloc(csr_alloc_elems(P) * sizeof(double), s));
    SgsArgs g;
    g.aoff = A->d_off();
    g.acols = A->d_cols();
    g.avals = A->d_vals();
    g.boff = B->d_off();
    g.bcols = B->d_cols();
    g.bvals = B->d_vals();
    g.m = m;
    g.pofs = pofs.as<uint64_t>();
    g.tile_start = tile_start.as<uint64_t>();
    g.n_tiles = ticket.as<uint64_t>() + 1;
    g.hbeg = hbeg.as<uint64_t>();
    g.hcnt = hcnt.as<uint32_t>();
    g.hcol = eo.ccol.as<uint32_t>();
    g.hval = eo.cval.as<double>();
    g.tstate = reinterpret_cast<unsigned long long *>(tstate.ptr);
    g.ticket = reinterpret_cast<unsigned long long *>(ticket.as<uint64_t>());
    g.coff = off.as<uint64_t>();
    g.ccols = cols.as<uint32_t>();
    g.cvals = vals.as<double>();
    g.status = c->d_status;
    g.tpb = cf.tpb;
    g.wait_cycles = SGS_WAIT_CYCLES;
    g.fixed_rows = F;
    const size_t smem = sgs_smem_bytes(cf);
    const unsigned grid = (unsigned)t_max;
    // keys: column << log2(hb) | slot, in 32 bits while the columns allow
    const bool k32 = n < (1ull << (32 - (cf.hb == 64 ? 6 : cf.hb == 128 ? 7 : 8)));
    int lrc;
    if (cf.hb == 64) lrc = k32 ? launch_tiles<64, uint32_t>(g, grid, smem, s) : launch_tiles<64, uint64_t>(g, grid, smem, s);
    else if (cf.hb == 128)
        lrc = k32 ? launch_tiles<128, uint32_t>(g, grid, smem, s) : launch_tiles<128, uint64_t>(g, grid, smem, s);
    else lrc = k32 ? launch_tiles<256, uint32_t>(g, grid, smem, s) : launch_tiles<256, uint64_t>(g, grid, smem, s);
    SPG_TRY(lrc);
    const uint64_t nnz = read_u64(c, off.as<uint64_t>() + m, s, &rc);
    SPG_TRY(rc);
    SPG_TRY(c->take_status());
    spgemm_install(Cm, m, n, std::move(off), std::move(cols), std::move(vals), nnz);
    return SPG_OK;
}

}  // namespace spg

using namespace spg;

// Runs the SpGEMM tiles' bounded wait against a predecessor that never
// publishes, with a wait of `wait_cycles` SM clocks; the kernel gives up,
// flags the context's status word and returns. *gave_up = 1 when it did.
extern "C" int spg_selftest_wait_timeout(spg_ctx *c, long long wait_cycles, int *gave_up) {
    if (!c || !gave_up) return set_error(SPG_ERR_INVALID_ARGUMENT, "spg_selftest_wait_timeout: null argument");
    if (wait_cycles < 1 || wait_cycles > SGS_WAIT_CYCLES)
        return set_error(SPG_ERR_INVALID_ARGUMENT, "spg_selftest_wait_timeout: wait_cycles out of range");
    SPG_CUDA_TRY(cudaSetDevice(c->device));
    cudaStream_t s = c->stream;
    DevBuf tstate, out;
    SPG_TRY(tstate.alloc(2 * sizeof(unsigned long long), s));
    SPG_TRY(out.alloc(2 * sizeof(unsigned long long), s));
    SPG_CUDA_TRY(cudaMemsetAsync(tstate.ptr, 0, 2 * sizeof(unsigned long long), s));
    SPG_CUDA_TRY(cudaMemsetAsync(out.ptr, 0, 2 * sizeof(unsigned long long), s));
    SgsArgs g{};
    g.tstate = reinterpret_cast<unsigned long long *>(tstate.ptr);
    g.status = c->d_status;
    g.wait_cycles = wait_cycles;
    sgs_wait_selftest<<<1, 32, 0, s>>>(g, reinterpret_cast<unsigned long long *>(out.ptr));
    SPG_LAUNCH_CHECK();
    unsigned long long h[2] = {0, 0};
    SPG_CUDA_TRY(cudaMemcpyAsync(h, out.ptr, sizeof(h), cudaMemcpyDeviceToHost, s));
    SPG_CUDA_TRY(cudaStreamSynchronize(s));
    *gave_up = (h[0] == 1 && h[1] == LB_POISON) ? 1 : 0;
    return SPG_OK;  // the timeout itself is reported by the next spg_ctx_sync
}
