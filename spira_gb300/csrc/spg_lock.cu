// spg_lock.cu — lock(): merge one epoch of staged inserts into the CSR.
//
// Spira's lock (matrix.hpp:277-342) sorts and dedups every row buffer keeping
// the last write and keeping zeros (aos_array_buffer.hpp:76-101: reverse +
// stable_sort + first-of-run), then either builds the CSR dropping zeros
// (csr_build.hpp:32-98) or two-pointer-merges each dirty row with its old CSR
// slice, the buffer winning on equal columns and a zero deleting
// (csr_build.hpp:126-488). The GPU formulation computes the same CSR:
//
//   1. keys (row << cbits | col) with the staging index as payload go through
//      a stable LSD radix sort; the last element of each equal-key run is the
//      last write (stability keeps insertion order within a run);
//   2. the deduplicated delta D (sorted by row, col; zeros kept) gets row
//      offsets doff by lower_bound per row;
//   3. every delta entry j finds its insertion point ins[j] in its old row and
//      whether it collides; contrib[j] = +1 (new non-zero), -1 (zero that
//      deletes an old entry) or 0; P = exclusive scan of contrib;
//   4. new row counts = old count + P[doff[r+1]] - P[doff[r]]; scan -> offsets;
//   5. old entry (row r, position p, column c): dropped if D holds (r, c),
//      else written to new_off[r] + p + (P[j] - P[doff[r]]) with j the first
//      delta entry of row r with column >= c; delta entry j (non-zero) to
//      new_off[r] + ins[j] + (P[j] - P[doff[r]]).
// Everything is integer work or a copy of the value bits, so structure and
// values are bit-exact against Spira. The first lock is the same pass with an
// empty old CSR. Capacity follows Spira's rule: the first build is tight;
// a merge keeps the old capacity when old nnz + |D| fits, else grows to 1.5x
// that bound (csr_build.hpp:139-145).
#include "spg_internal.cuh"

namespace spg {
namespace {

constexpr int LB = 256;


__global__ void lock_make_keys(const uint32_t *__restrict__ rows, const uint32_t *__restrict__ cols,
                               uint64_t m, int cbits, uint64_t *__restrict__ keys,
                               uint32_t *__restrict__ idx) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < m;
         i += (uint64_t)gridDim.x * blockDim.x) {
        keys[i] = ((uint64_t)rows[i] << cbits) | cols[i];
        idx[i] = (uint32_t)i;
    }
}

// One pass over the staged inserts: keys and staging indices, plus
// stats[0] = max row, stats[1] = max column (range check), stats[2] = 1 if
// some key is greater than its successor (not sorted), stats[3] = 1 if some
// row is (rows not grouped), stats[4] = 1 if some key is not below its
// successor (not strictly increasing: duplicates or unsorted).
// Runs of more than GAP_LONG row offsets with one value (empty rows) are
// listed for offsets_fill_gaps (up to GAP_SLOTS of them) rather than written
// by one thread.
constexpr uint64_t GAP_LONG = 4096;
constexpr unsigned GAP_SLOTS = 1024;

struct RowGap {
    uint64_t lo, hi, pos;
};

// (Writing the staged rows' offsets in this pass as well, speculatively, was
// tried and removed: on inserts in random order every rising step between
// neighbours would write its whole gap of rows, ~m n / 3 stores.)
// VEC: rows and cols 16-byte aligned; each thread reads 4 rows and 4
// columns per step in two 16-byte loads (the successor of its last pair
// comes from the next lane, or one more load at the warp's edge).
template <bool VEC>
__global__ void lock_prepare(const uint32_t *__restrict__ rows, const uint32_t *__restrict__ cols, uint64_t m,
                             int cbits, unsigned *__restrict__ stats) {
    unsigned mr = 0, mc = 0;
    bool d = false, g = false, e = false;
    if constexpr (VEC) {
        const uint64_t n4 = m / 4;  // whole groups of 4; the tail below
        const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
        const uint64_t n_iter = (n4 + stride - 1) / stride;  // warp-uniform: shuffles below
        for (uint64_t it = 0; it < n_iter; ++it) {
            const uint64_t q = it * stride + blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
            const bool ok = q < n4;
            uint4 r4 = make_uint4(0, 0, 0, 0), c4 = make_uint4(0, 0, 0, 0);
            if (ok) {
                r4 = reinterpret_cast<const uint4 *>(rows)[q];
                c4 = reinterpret_cast<const uint4 *>(cols)[q];
            }
            uint32_t rn = __shfl_down_sync(0xffffffffu, r4.x, 1), cn = __shfl_down_sync(0xffffffffu, c4.x, 1);
            const bool have_next = ok && 4 * q + 4 < m;
            if (have_next && ((threadIdx.x & 31) == 31 || q + 1 >= n4)) {
                rn = rows[4 * q + 4];
                cn = cols[4 * q + 4];
            }
            if (ok) {
                const uint32_t rr[5] = {r4.x, r4.y, r4.z, r4.w, rn}, cc[5] = {c4.x, c4.y, c4.z, c4.w, cn};
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    mr = max(mr, rr[k]);
                    mc = max(mc, cc[k]);
                    if (k < 3 || have_next) {
                        const uint64_t k1 = ((uint64_t)rr[k] << cbits) | cc[k];
                        const uint64_t k2 = ((uint64_t)rr[k + 1] << cbits) | cc[k + 1];
                        d |= k1 > k2;
                        e |= k1 >= k2;
                        g |= rr[k] > rr[k + 1];
                    }
                }
            }
        }
    }
    for (uint64_t i = (VEC ? (m & ~3ull) : 0) + blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < m;
         i += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t r = rows[i], c = cols[i];
        const uint64_t k = ((uint64_t)r << cbits) | c;
        mr = max(mr, r);
        mc = max(mc, c);
        if (i + 1 < m) {
            const uint32_t r2 = rows[i + 1];
            const uint64_t k2 = ((uint64_t)r2 << cbits) | cols[i + 1];
            d |= k > k2;
            e |= k >= k2;
            g |= r > r2;
        }
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) {
        mr = max(mr, __shfl_xor_sync(0xffffffffu, mr, o));
        mc = max(mc, __shfl_xor_sync(0xffffffffu, mc, o));
    }
    const unsigned flags = (__any_sync(0xffffffffu, d) ? 1u : 0u) | (__any_sync(0xffffffffu, g) ? 2u : 0u) |
                           (__any_sync(0xffffffffu, e) ? 4u : 0u);
    // one set of atomics per block: per-warp atomics on the same two words
    // serialise at L2 and cost more than the pass itself
    __shared__ unsigned s_mr[LB / 32], s_mc[LB / 32], s_fl[LB / 32];
    const int w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) {
        s_mr[w] = mr;
        s_mc[w] = mc;
        s_fl[w] = flags;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned bm = 0, bc = 0, bf = 0;
        for (int i = 0; i < (int)(blockDim.x >> 5); ++i) {
            bm = max(bm, s_mr[i]);
            bc = max(bc, s_mc[i]);
            bf |= s_fl[i];
        }
        atomicMax(stats, bm);
        atomicMax(stats + 1, bc);
        if (bf & 1u) stats[2] = 1u;
        if (bf & 2u) stats[3] = 1u;
        if (bf & 4u) stats[4] = 1u;
    }
}

// Moves the kept entries of a row-grouped first lock from their rows' input
// positions (row r's at [s_off[r], s_off[r] + kept)) to their CSR positions
// (off: the exclusive scan of the kept counts). The staged rows name each
// position's row, as the rows are grouped.
__global__ void first_grouped_compact(const uint32_t *__restrict__ rows, const uint64_t *__restrict__ s_off,
                                      const uint64_t *__restrict__ off, const uint32_t *__restrict__ scols,
                                      const double *__restrict__ svals, uint64_t m, uint32_t *__restrict__ ocols,
                                      double *__restrict__ ovals) {
    // four positions per thread, their loads issued together: the row, the
    // entry and then the row's offsets are a chain of dependent loads
    constexpr int U = 4;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t e0 = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e0 < m; e0 += U * stride) {
        uint32_t r[U], c[U];
        double v[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const uint64_t e = e0 + u * stride;
            if (e < m) {
                r[u] = rows[e];
                c[u] = scols[e];
                v[u] = svals[e];
            }
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const uint64_t e = e0 + u * stride;
            if (e < m) {
                const uint64_t k = e - s_off[r[u]], o0 = off[r[u]];
                if (k < off[r[u] + 1] - o0) {
                    ocols[o0 + k] = c[u];
                    ovals[o0 + k] = v[u];
                }
            }
        }
    }
}

// First lock of inserts in strictly increasing (row, col) order: the CSR is
// the staged arrays themselves unless a value is zero (*zero = 1; then the
// caller takes the general path).
__global__ void first_direct_copy(const uint32_t *__restrict__ cols, const double *__restrict__ vals, uint64_t m,
                                  uint32_t *__restrict__ out_cols, double *__restrict__ out_vals,
                                  unsigned *__restrict__ zero) {
    bool z = false;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < m;
         i += (uint64_t)gridDim.x * blockDim.x) {
        const double v = vals[i];
        z |= is_zero(v);
        out_cols[i] = cols[i];
        out_vals[i] = v;
    }
    if (__any_sync(0xffffffffu, z) && (threadIdx.x & 31) == 0) *zero = 1u;
}

// flags[0] = 1 if some key is greater than its successor (not sorted);
// flags[1] = 1 if some row is greater than its successor (rows not grouped).
__global__ void keys_descent(const uint64_t *__restrict__ keys, uint64_t m, int cbits, unsigned *__restrict__ flags) {
    bool d = false, g = false;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i + 1 < m;
         i += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t a = keys[i], b = keys[i + 1];
        d |= a > b;
        g |= (a >> cbits) > (b >> cbits);
    }
    const bool wd = __any_sync(0xffffffffu, d), wg = __any_sync(0xffffffffu, g);
    if ((threadIdx.x & 31) == 0) {
        if (wd) flags[0] = 1u;
        if (wg) flags[1] = 1u;
    }
}

// flag[i] = 1 iff sorted key i is the last of its run (the last write).
__global__ void lock_last_flags(const uint64_t *__restrict__ keys, uint64_t m, uint64_t *__restrict__ flag) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < m;
         i += (uint64_t)gridDim.x * blockDim.x)
        flag[i] = (i + 1 == m || keys[i] != keys[i + 1]) ? 1 : 0;
}

__global__ void lock_gather_delta(const uint64_t *__restrict__ keys, const uint32_t *__restrict__ idx,
                                  const uint64_t *__restrict__ pos, uint64_t m, int cbits,
                                  const double *__restrict__ vals, uint32_t *__restrict__ drow,
                                  uint32_t *__restrict__ dcol, double *__restrict__ dval) {
    const uint64_t cmask = cbits ? ((1ull << cbits) - 1) : 0;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < m;
         i += (uint64_t)gridDim.x * blockDim.x) {
        if (i + 1 == m || keys[i] != keys[i + 1]) {
            const uint64_t j = pos[i];
            drow[j] = (uint32_t)(keys[i] >> cbits);
            dcol[j] = (uint32_t)(keys[i] & cmask);
            dval[j] = vals[idx[i]];
        }
    }
}

// off[r] = lower_bound(sorted_rows[0..u), r) for r in [0, n_rows], from the
// row boundaries: position i (i == u standing for row n_rows) is the first
// position of rows srows[i - 1] + 1 .. srows[i], so it writes those offsets.
// One pass over the rows, coalesced, no searches. Runs of up to GAP_LONG
// empty rows are written by the thread at their boundary; longer ones are
// listed in `gaps` (up to GAP_SLOTS of them) for offsets_fill_gaps to spread
// over the grid, and written by their thread once the list is full. A
// decreasing step (never in the sorted input) writes nothing, so every write
// stays inside [0, n_rows].

constexpr int OFF_T = 256, OFF_E = 8, OFF_TILE = OFF_T * OFF_E;  // positions per block step

// Block steps over tiles of OFF_TILE positions: the tile's rows (and the one
// before it) are staged in shared memory with coalesced loads, then thread t
// checks positions t, t + OFF_T, ... against their predecessors, so a
// position costs a few instructions and only row boundaries write.
__global__ void __launch_bounds__(OFF_T)
offsets_from_sorted_rows(const uint32_t *__restrict__ srows, uint64_t u, uint64_t n_rows,
                         uint64_t *__restrict__ off, RowGap *__restrict__ gaps, unsigned *__restrict__ n_gaps) {
    __shared__ uint32_t s_row[OFF_TILE + 1];  // s_row[j] = row at position tile + j - 1 (when < u)
    for (uint64_t tile = blockIdx.x * (uint64_t)OFF_TILE; tile <= u; tile += (uint64_t)gridDim.x * OFF_TILE) {
        // all loads of a thread issued before any is stored (HBM needs many
        // bytes in flight per SM)
        uint32_t v[OFF_E + 1];
#pragma unroll
        for (int k = 0; k <= OFF_E; ++k) {
            const int j = threadIdx.x + k * OFF_T;
            const uint64_t p = tile + j - 1;  // tile == 0, j == 0: never read
            v[k] = (j <= OFF_TILE && tile + j >= 1 && p < u) ? srows[p] : 0u;
        }
#pragma unroll
        for (int k = 0; k <= OFF_E; ++k) {
            const int j = threadIdx.x + k * OFF_T;
            if (j <= OFF_TILE) s_row[j] = v[k];
        }
        __syncthreads();
        const int lim = (int)min((uint64_t)OFF_TILE, u + 1 - tile);  // positions tile .. u of this tile
#pragma unroll
        for (int k = 0; k < OFF_E; ++k) {
            const int j = threadIdx.x + k * OFF_T;
            if (j >= lim) break;
            const uint64_t i = tile + j;
            const bool at_end = i == u;
            // inside a row: same row as the position before (32-bit fast path)
            if (i != 0 && !at_end && s_row[j + 1] == s_row[j]) continue;
            const uint64_t cur = at_end ? n_rows : min((uint64_t)s_row[j + 1], n_rows);
            const uint64_t lo = i == 0 ? 0 : (uint64_t)s_row[j] + 1;  // rows [lo, cur] start at position i
            if (cur + 1 <= lo) continue;  // a decreasing step (never in sorted input): nothing
            const uint64_t hi = cur + 1;
            if (hi - lo > GAP_LONG) {
                const unsigned slot = atomicAdd(n_gaps, 1u);
                if (slot < GAP_SLOTS) {
                    gaps[slot] = {lo, hi, i};
                    continue;  // listed: written by offsets_fill_gaps
                }
            }
            for (uint64_t r = lo; r < hi; ++r) off[r] = i;
        }
        __syncthreads();
    }
}

// The listed long stretches of empty rows, each spread over the whole grid.
__global__ void offsets_fill_gaps(const RowGap *__restrict__ gaps, const unsigned *__restrict__ n_gaps,
                                  uint64_t *__restrict__ off) {
    const unsigned n = min(*n_gaps, GAP_SLOTS);
    const uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x, nt = (uint64_t)gridDim.x * blockDim.x;
    for (unsigned g = 0; g < n; ++g) {
        const RowGap G = gaps[g];
        for (uint64_t r = G.lo + t; r < G.hi; r += nt) off[r] = G.pos;
    }
}

// off[0..n_rows] from the non-decreasing rows srows[0..u) (stream-ordered).
int launch_row_offsets(Ctx *c, const uint32_t *srows, uint64_t u, uint64_t n_rows, uint64_t *off, cudaStream_t s) {
    DevBuf scratch;  // [counter (16 bytes)] [GAP_SLOTS gaps]
    SPG_TRY(scratch.alloc(16 + GAP_SLOTS * sizeof(RowGap), s));
    unsigned *n_gaps = scratch.as<unsigned>();
    RowGap *gaps = reinterpret_cast<RowGap *>(scratch.as<char>() + 16);
    SPG_CUDA_TRY(cudaMemsetAsync(n_gaps, 0, sizeof(unsigned), s));
    offsets_from_sorted_rows<<<grid_for(u + 1, OFF_TILE, (unsigned)c->n_sms * 8), OFF_T, 0, s>>>(srows, u, n_rows, off,
                                                                                            gaps, n_gaps);
    offsets_fill_gaps<<<c->n_sms * 4, LB, 0, s>>>(gaps, n_gaps, off);
    SPG_LAUNCH_CHECK();
    return SPG_OK;
}

// Step 3: insertion point / collision / contribution of every delta entry.
__global__ void merge_delta_probe(const uint64_t *__restrict__ off, const uint32_t *__restrict__ cols,
                                  bool has_old, const uint32_t *__restrict__ drow,
                                  const uint32_t *__restrict__ dcol, const double *__restrict__ dval,
                                  uint64_t u, uint32_t *__restrict__ ins, int64_t *__restrict__ contrib) {
    for (uint64_t j = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; j < u;
         j += (uint64_t)gridDim.x * blockDim.x) {
        const bool z = is_zero(dval[j]);
        bool coll = false;
        uint64_t p = 0;
        if (has_old) {
            const uint64_t b = off[drow[j]], e = off[drow[j] + 1];
            const uint32_t c = dcol[j];
            uint64_t lo = b, hi = e;
            while (lo < hi) {
                const uint64_t mid = (lo + hi) >> 1;
                if (cols[mid] < c) lo = mid + 1;
                else hi = mid;
            }
            coll = lo < e && cols[lo] == c;
            p = lo - b;
        }
        ins[j] = (uint32_t)p;
        contrib[j] = (!z && !coll) ? 1 : ((z && coll) ? -1 : 0);
    }
}

// Step 4 (before the scan): new row counts; cnt[n_rows] = 0.
__global__ void merge_row_counts(const uint64_t *__restrict__ off, bool has_old,
                                 const uint64_t *__restrict__ doff, const int64_t *__restrict__ P,
                                 uint64_t n_rows, uint64_t *__restrict__ cnt) {
    for (uint64_t r = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; r <= n_rows;
         r += (uint64_t)gridDim.x * blockDim.x) {
        if (r == n_rows) {
            cnt[r] = 0;
            continue;
        }
        const int64_t old_cnt = has_old ? (int64_t)(off[r + 1] - off[r]) : 0;
        cnt[r] = (uint64_t)(old_cnt + (P[doff[r + 1]] - P[doff[r]]));
    }
}

// Step 5a: old entries, CTA chunks of MO_CHUNK; the row of each entry is found
// by binary search inside the chunk's row window.
constexpr int MO_CHUNK = 2048;

__device__ __forceinline__ uint64_t row_of(const uint64_t *__restrict__ off, uint64_t lo, uint64_t hi,
                                           uint64_t k) {
    // largest r in [lo, hi] with off[r] <= k
    while (lo < hi) {
        const uint64_t mid = (lo + hi + 1) >> 1;
        if (off[mid] <= k) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// Rows of a chunk whose offsets fit in shared memory; chunks spanning more
// rows (long runs of empty rows) search the global arrays instead.
constexpr int MO_WIN = 1536;

// Rows of the first and last entry of every chunk (thread per chunk: the
// searches run in parallel instead of serialising each block's start).
__global__ void merge_windows(const uint64_t *__restrict__ off, uint64_t n_rows, uint64_t nnz_old,
                              uint64_t n_chunks, uint64_t *__restrict__ win) {
    const uint64_t ch = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (ch >= n_chunks) return;
    const uint64_t k0 = ch * MO_CHUNK, k1 = min(k0 + (uint64_t)MO_CHUNK, nnz_old);
    const uint64_t lo = row_of(off, 0, n_rows, k0);
    win[2 * ch] = lo;
    win[2 * ch + 1] = row_of(off, lo, n_rows, k1 - 1);
}

__global__ void __launch_bounds__(LB)
merge_write_old(const uint64_t *__restrict__ off, const uint32_t *__restrict__ cols,
                const double *__restrict__ vals, const uint64_t *__restrict__ win, uint64_t nnz_old,
                const uint64_t *__restrict__ doff, const uint32_t *__restrict__ dcol,
                const int64_t *__restrict__ P, const uint64_t *__restrict__ new_off,
                uint32_t *__restrict__ out_cols, double *__restrict__ out_vals) {
    __shared__ uint64_t s_off[MO_WIN + 1], s_new[MO_WIN + 1], s_doff[MO_WIN + 1];
    __shared__ uint16_t s_row[MO_CHUNK];  // row of each entry of the chunk, relative to rlo
    const uint64_t k0 = (uint64_t)blockIdx.x * MO_CHUNK;
    const uint64_t k1 = min(k0 + (uint64_t)MO_CHUNK, nnz_old);
    const uint64_t rlo = win[2 * blockIdx.x], rhi = win[2 * blockIdx.x + 1];
    const bool local = rhi - rlo < (uint64_t)MO_WIN;
    if (local) {
        for (uint64_t t = threadIdx.x; t <= rhi - rlo + 1; t += LB) {
            s_off[t] = off[rlo + t];
            s_new[t] = new_off[rlo + t];
            s_doff[t] = doff[rlo + t];
        }
        for (int t = threadIdx.x; t < MO_CHUNK; t += LB) s_row[t] = 0;
        __syncthreads();
        // label the chunk's entries with their rows: every non-empty row starting
        // inside the chunk marks its first entry, then an inclusive max-scan
        // carries each mark over the row's entries (a warp per row left most
        // lanes idle on short rows)
        for (uint64_t rr = threadIdx.x + 1; rr <= rhi - rlo; rr += LB) {
            const uint64_t b = s_off[rr];
            if (b >= k0 && b < k1 && s_off[rr + 1] > b) s_row[b - k0] = (uint16_t)rr;
        }
        __syncthreads();
        constexpr int PT = MO_CHUNK / LB;  // positions per thread, blocked
        const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
        uint16_t lab[PT];
        uint16_t run = 0;
#pragma unroll
        for (int i = 0; i < PT; ++i) {
            run = max(run, s_row[threadIdx.x * PT + i]);
            lab[i] = run;
        }
        uint16_t inc = run;  // inclusive max over threads 0..t
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint16_t v = (uint16_t)__shfl_up_sync(0xffffffffu, (unsigned)inc, o);
            if (lane >= o) inc = max(inc, v);
        }
        __shared__ uint16_t s_wmax[LB / 32];
        if (lane == 31) s_wmax[warp] = inc;
        __syncthreads();
        uint16_t carry = (uint16_t)__shfl_up_sync(0xffffffffu, (unsigned)inc, 1);
        if (lane == 0) carry = 0;
        for (int w = 0; w < warp; ++w) carry = max(carry, s_wmax[w]);
#pragma unroll
        for (int i = 0; i < PT; ++i) s_row[threadIdx.x * PT + i] = max(carry, lab[i]);
    }
    __syncthreads();
    // consecutive threads on consecutive entries (coalesced); a thread's
    // loads for all its entries are issued before any is used
    constexpr int MI = MO_CHUNK / LB;
    uint32_t cs[MI];
    double vs[MI];
#pragma unroll
    for (int q = 0; q < MI; ++q) {
        const uint64_t k = k0 + threadIdx.x + (uint64_t)q * LB;
        cs[q] = k < k1 ? cols[k] : 0u;
        vs[q] = k < k1 ? vals[k] : 0.0;
    }
#pragma unroll
    for (int q = 0; q < MI; ++q) {
        const uint64_t k = k0 + threadIdx.x + (uint64_t)q * LB;
        if (k >= k1) break;
        uint64_t p, ds, de, nb;
        if (local) {
            const int lo = s_row[k - k0];
            p = k - s_off[lo];
            ds = s_doff[lo];
            de = s_doff[lo + 1];
            nb = s_new[lo];
        } else {
            const uint64_t r = row_of(off, rlo, rhi, k);
            p = k - off[r];
            ds = doff[r];
            de = doff[r + 1];
            nb = new_off[r];
        }
        const uint32_t c = cs[q];
        uint64_t dst = nb + p;
        if (ds != de) {
            uint64_t lo = ds, hi = de;
            while (lo < hi) {
                const uint64_t mid = (lo + hi) >> 1;
                if (dcol[mid] < c) lo = mid + 1;
                else hi = mid;
            }
            if (lo < de && dcol[lo] == c) continue;  // replaced or deleted by the delta
            dst += (uint64_t)(P[lo] - P[ds]);
        }
        out_cols[dst] = c;
        out_vals[dst] = vs[q];
    }
}

// Step 5b: non-zero delta entries.
__global__ void merge_write_delta(const uint32_t *__restrict__ drow, const uint32_t *__restrict__ dcol,
                                  const double *__restrict__ dval, const uint32_t *__restrict__ ins,
                                  const uint64_t *__restrict__ doff, const int64_t *__restrict__ P, uint64_t u,
                                  const uint64_t *__restrict__ new_off, uint32_t *__restrict__ out_cols,
                                  double *__restrict__ out_vals) {
    for (uint64_t j = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; j < u;
         j += (uint64_t)gridDim.x * blockDim.x) {
        const double v = dval[j];
        if (is_zero(v)) continue;
        const uint32_t r = drow[j];
        const uint64_t dst = new_off[r] + ins[j] + (uint64_t)(P[j] - P[doff[r]]);
        out_cols[dst] = dcol[j];
        out_vals[dst] = v;
    }
}

// Explicit zeros of a loaded CSR inside rows the delta touches: Spira's merge
// drops them (csr_build.hpp:274-276, 292-296). They become synthetic zero
// inserts placed before the real ones, so a real insert on the same column
// still wins the last-write dedup.
__global__ void zero_entries_in_dirty_rows(const uint64_t *__restrict__ off, const uint32_t *__restrict__ cols,
                                           const double *__restrict__ vals, uint64_t n_rows,
                                           const uint64_t *__restrict__ doff, uint64_t *__restrict__ flag,
                                           uint32_t *__restrict__ zrow, uint32_t *__restrict__ zcol,
                                           const uint64_t *__restrict__ pos, int pass) {
    for (uint64_t r = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; r < n_rows;
         r += (uint64_t)gridDim.x * blockDim.x) {
        const bool dirty = doff[r] != doff[r + 1];
        for (uint64_t k = off[r]; k < off[r + 1]; ++k) {
            const bool z = dirty && is_zero(vals[k]);
            if (pass == 0) {
                flag[k] = z ? 1 : 0;
            } else if (z) {
                zrow[pos[k]] = (uint32_t)r;
                zcol[pos[k]] = cols[k];
            }
        }
    }
}

__global__ void fill_f64(double *p, uint64_t n, double v) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x)
        p[i] = v;
}

// Delta arrays (sorted by (row, col), one entry per key, zeros kept).
struct Delta {
    uint64_t u = 0;
    DevBuf row, col, val;
};

// First lock (build_csr, csr_build.hpp:32-98): the CSR is the last write of
// every key with zeros dropped. flag[i] = 1 iff sorted entry i is kept.
// First lock, general path: the sorted entries are compacted in two passes
// over tiles of KTILE entries, without a per-entry position array. Entry i
// is kept when it is the last of its key run (the last write) and its value
// is not +-0. Pass 1 counts the kept entries of every tile; after a scan of
// the counts, pass 2 recomputes the flags, ranks them inside the tile
// (entries k * KT + t, k-major: ballots per warp, warp totals in shared
// memory) and writes row, column and value at tile prefix + rank.
constexpr int KT = 256, KI = 8, KTILE = KT * KI;

__device__ __forceinline__ unsigned lane_lt_mask() {
    unsigned m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

__device__ __forceinline__ void keep_flags_of_tile(const uint64_t *__restrict__ keys, const uint32_t *__restrict__ idx,
                                                   const double *__restrict__ vals, uint64_t m, uint64_t base,
                                                   bool (&f)[KI], uint64_t (&key)[KI], double (&val)[KI]) {
    uint32_t ix[KI];
    uint64_t nxt[KI];
#pragma unroll
    for (int k = 0; k < KI; ++k) {  // loads of all items first
        const uint64_t i = base + (uint64_t)k * KT + threadIdx.x;
        key[k] = i < m ? keys[i] : 0;
        nxt[k] = i + 1 < m ? keys[i + 1] : ~0ull;
        ix[k] = i < m ? idx[i] : 0;
    }
#pragma unroll
    for (int k = 0; k < KI; ++k) {
        const uint64_t i = base + (uint64_t)k * KT + threadIdx.x;
        const bool last = i < m && (i + 1 == m || key[k] != nxt[k]);
        val[k] = last ? vals[ix[k]] : 0.0;
        f[k] = last && !is_zero(val[k]);
    }
}

__global__ void __launch_bounds__(KT)
first_keep_count(const uint64_t *__restrict__ keys, const uint32_t *__restrict__ idx, const double *__restrict__ vals,
                 uint64_t m, uint64_t *__restrict__ tile_counts) {
    bool f[KI];
    uint64_t key[KI];
    double val[KI];
    keep_flags_of_tile(keys, idx, vals, m, blockIdx.x * (uint64_t)KTILE, f, key, val);
    unsigned c = 0;
#pragma unroll
    for (int k = 0; k < KI; ++k) c += f[k];
#pragma unroll
    for (int o = 16; o; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
    __shared__ unsigned s_c[KT / 32];
    if ((threadIdx.x & 31) == 0) s_c[threadIdx.x >> 5] = c;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned t = 0;
        for (int w = 0; w < KT / 32; ++w) t += s_c[w];
        tile_counts[blockIdx.x] = t;
    }
}

__global__ void __launch_bounds__(KT)
first_keep_gather(const uint64_t *__restrict__ keys, const uint32_t *__restrict__ idx, const double *__restrict__ vals,
                  uint64_t m, int cbits, const uint64_t *__restrict__ tile_prefix, uint32_t *__restrict__ orow,
                  uint32_t *__restrict__ ocol, double *__restrict__ oval) {
    bool f[KI];
    uint64_t key[KI];
    double val[KI];
    keep_flags_of_tile(keys, idx, vals, m, blockIdx.x * (uint64_t)KTILE, f, key, val);
    __shared__ unsigned s_w[KI][KT / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    unsigned rank[KI];
#pragma unroll
    for (int k = 0; k < KI; ++k) {
        const unsigned b = __ballot_sync(0xffffffffu, f[k]);
        rank[k] = __popc(b & lane_lt_mask());
        if (lane == 0) s_w[k][warp] = __popc(b);
    }
    __syncthreads();
    if (threadIdx.x == 0) {  // exclusive prefix over (k, warp): the tile's entry order
        unsigned run = 0;
        for (int k = 0; k < KI; ++k)
            for (int w = 0; w < KT / 32; ++w) {
                const unsigned v = s_w[k][w];
                s_w[k][w] = run;
                run += v;
            }
    }
    __syncthreads();
    const uint64_t base = tile_prefix[blockIdx.x];
    const uint64_t cmask = cbits ? ((1ull << cbits) - 1) : 0;
#pragma unroll
    for (int k = 0; k < KI; ++k) {
        if (!f[k]) continue;
        const uint64_t j = base + s_w[k][warp] + rank[k];
        orow[j] = (uint32_t)(key[k] >> cbits);
        ocol[j] = (uint32_t)(key[k] & cmask);
        oval[j] = val[k];
    }
}

// Keys (row << cbits | col) of the staged inserts sorted stably, with their
// staging indices.
// Keys, indices and order flags of a staged epoch, made once by lock_prepare
// alongside the range check.
struct Prepared {
    unsigned unsorted = 1, ungrouped = 1, not_strict = 1;
    bool ready = false;
};

int sort_keys(Ctx *c, const uint32_t *rows, const uint32_t *cols, uint64_t m, uint64_t n_rows, uint64_t n_cols,
              DevBuf &keys, DevBuf &idx, Prepared *pre, cudaStream_t s) {
    const int cbits = bits_for(n_cols), rbits = bits_for(n_rows);
    const unsigned g = grid_for(m, LB, (unsigned)c->n_sms * 16);
    // Inserts staged already in (row, col) order (row by row, ascending
    // columns: how stencils and most assemblies insert) need no sort: the
    // stable sort of a non-decreasing sequence is the identity. Inserts staged
    // row by row with columns in any order are sorted row by row on chip.
    unsigned f[2] = {1u, 1u};
    SPG_TRY(keys.alloc(m * sizeof(uint64_t), s));
    SPG_TRY(idx.alloc(m * sizeof(uint32_t), s));
    bool have_keys = false;
    auto make_keys = [&]() -> int {
        if (have_keys) return SPG_OK;
        lock_make_keys<<<g, LB, 0, s>>>(rows, cols, m, cbits, keys.as<uint64_t>(), idx.as<uint32_t>());
        SPG_LAUNCH_CHECK();
        have_keys = true;
        return SPG_OK;
    };
    if (pre && pre->ready) {
        f[0] = pre->unsorted;
        f[1] = pre->ungrouped;
    } else {
        SPG_TRY(make_keys());
        DevBuf flag;  // [0] keys unsorted, [1] rows not grouped
        SPG_TRY(flag.alloc(2 * sizeof(unsigned), s));
        SPG_CUDA_TRY(cudaMemsetAsync(flag.ptr, 0, 2 * sizeof(unsigned), s));
        keys_descent<<<g, LB, 0, s>>>(keys.as<uint64_t>(), m, cbits, flag.as<unsigned>());
        SPG_LAUNCH_CHECK();
        SPG_CUDA_TRY(cudaMemcpyAsync(f, flag.ptr, 2 * sizeof(unsigned), cudaMemcpyDeviceToHost, s));
        SPG_TRY(c->phase_sync(s));
    }
    if (!f[0]) return make_keys();  // already sorted: the keys in input order
    if (!f[1]) {  // the row-grouped sort reads rows and columns directly
        DevBuf s_off, keys2, idx2;
        SPG_TRY(s_off.alloc((n_rows + 1) * sizeof(uint64_t), s));
        SPG_TRY(launch_row_offsets(c, rows, m, n_rows, s_off.as<uint64_t>(), s));
        SPG_TRY(keys2.alloc(m * sizeof(uint64_t), s));
        SPG_TRY(idx2.alloc(m * sizeof(uint32_t), s));
        bool done = false;
        SPG_TRY(sort_grouped_rows(c, rows, cols, s_off.as<uint64_t>(), m, n_rows, cbits, keys2.as<uint64_t>(),
                                  idx2.as<uint32_t>(), &done, s));
        if (done) {
            keys = std::move(keys2);
            idx = std::move(idx2);
            return SPG_OK;
        }
    }
    SPG_TRY(make_keys());
    SPG_TRY(radix_sort_pairs_u64(c, keys.as<uint64_t>(), idx.as<uint32_t>(), m, rbits + cbits, s));
    return SPG_OK;
}

int sort_dedup(Ctx *c, const uint32_t *rows, const uint32_t *cols, const double *vals, uint64_t m,
               uint64_t n_rows, uint64_t n_cols, Delta &D, Prepared *pre, cudaStream_t s) {
    const int cbits = bits_for(n_cols);
    const unsigned g = grid_for(m, LB, (unsigned)c->n_sms * 16);
    DevBuf keys, idx, pos;
    SPG_TRY(sort_keys(c, rows, cols, m, n_rows, n_cols, keys, idx, pre, s));
    SPG_TRY(pos.alloc((m + 1) * sizeof(uint64_t), s));
    lock_last_flags<<<g, LB, 0, s>>>(keys.as<uint64_t>(), m, pos.as<uint64_t>());
    SPG_LAUNCH_CHECK();
    SPG_TRY(exclusive_scan_u64(c, pos.as<uint64_t>(), m, pos.as<uint64_t>() + m, s));
    uint64_t u = 0;
    SPG_CUDA_TRY(cudaMemcpyAsync(&u, pos.as<uint64_t>() + m, sizeof(uint64_t), cudaMemcpyDeviceToHost, s));
    SPG_TRY(c->phase_sync(s));
    D.u = u;
    SPG_TRY(D.row.alloc(u * sizeof(uint32_t), s));
    SPG_TRY(D.col.alloc(u * sizeof(uint32_t), s));
    SPG_TRY(D.val.alloc(u * sizeof(double), s));
    lock_gather_delta<<<g, LB, 0, s>>>(keys.as<uint64_t>(), idx.as<uint32_t>(), pos.as<uint64_t>(), m, cbits,
                                       vals, D.row.as<uint32_t>(), D.col.as<uint32_t>(), D.val.as<double>());
    SPG_LAUNCH_CHECK();
    return SPG_OK;
}

int row_offsets(Ctx *c, const uint32_t *srows, uint64_t u, uint64_t n_rows, DevBuf &doff, cudaStream_t s) {
    SPG_TRY(doff.alloc((n_rows + 1) * sizeof(uint64_t), s));
    SPG_TRY(launch_row_offsets(c, srows, u, n_rows, doff.as<uint64_t>(), s));
    return SPG_OK;
}

// First lock: sort, keep the last write of every key unless it is zero, and
// take the offsets from the kept rows.
int first_lock(Ctx *c, Csr *A, const uint32_t *rows, const uint32_t *cols, const double *vals, uint64_t m,
               Prepared *pre, cudaStream_t s) {
    const uint64_t n = A->n_rows;
    const int cbits = bits_for(A->n_cols);
    DevBuf keys, idx, pos, orow, out_cols, out_vals, new_off;
    uint64_t nnz = 0;
    if (m && pre && pre->ready && !pre->not_strict) {
        // strictly increasing keys: no duplicates to resolve, nothing to sort;
        // unless a value is zero, the staged arrays are the CSR
        const unsigned g = grid_for(m, LB, (unsigned)c->n_sms * 16);
        DevBuf zero;
        SPG_TRY(zero.alloc(sizeof(unsigned), s));
        SPG_CUDA_TRY(cudaMemsetAsync(zero.ptr, 0, sizeof(unsigned), s));
        SPG_TRY(out_cols.alloc(csr_alloc_elems(m) * sizeof(uint32_t), s));
        SPG_TRY(out_vals.alloc(csr_alloc_elems(m) * sizeof(double), s));
        first_direct_copy<<<g, LB, 0, s>>>(cols, vals, m, out_cols.as<uint32_t>(), out_vals.as<double>(),
                                           zero.as<unsigned>());
        SPG_LAUNCH_CHECK();
        // the offsets go out before the zero check comes back: one host sync
        SPG_TRY(new_off.alloc(csr_off_elems(n) * sizeof(uint64_t), s));
        SPG_TRY(launch_row_offsets(c, rows, m, n, new_off.as<uint64_t>(), s));
        unsigned hz = 1;
        SPG_CUDA_TRY(cudaMemcpyAsync(&hz, zero.ptr, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
        SPG_TRY(c->phase_sync(s));
        if (!hz) {
            A->invalidate_derived();
            A->off = std::move(new_off);
            A->cols = std::move(out_cols);
            A->vals = std::move(out_vals);
            A->nnz = m;
            A->capacity = m;  // build_csr: exact
            A->built = true;
            A->may_have_zeros = false;
            return SPG_OK;
        }
        new_off.release();
        out_cols.release();
        out_vals.release();
    }
    if (m && pre && pre->ready && pre->unsorted && !pre->ungrouped) {
        // Row-grouped inserts (rows non-decreasing, columns in any order, as
        // row-by-row assembly stages them): every row is sorted, its last
        // write per column kept unless zero, and compacted on chip in one
        // pass, in place at the row's input positions; a scan of the kept
        // counts gives the offsets, and entries move only if some were dropped.
        DevBuf s_off, kept, scols, svals;
        SPG_TRY(s_off.alloc((n + 1) * sizeof(uint64_t), s));
        SPG_TRY(launch_row_offsets(c, rows, m, n, s_off.as<uint64_t>(), s));
        SPG_TRY(kept.alloc(csr_off_elems(n) * sizeof(uint64_t), s));
        SPG_TRY(scols.alloc(csr_alloc_elems(m) * sizeof(uint32_t), s));
        SPG_TRY(svals.alloc(csr_alloc_elems(m) * sizeof(double), s));
        bool done = false;
        SPG_TRY(dedup_grouped_rows(c, cols, vals, s_off.as<uint64_t>(), m, n, cbits, scols.as<uint32_t>(),
                                   svals.as<double>(), kept.as<uint64_t>(), &done, s));
        if (done) {
            SPG_TRY(exclusive_scan_u64(c, kept.as<uint64_t>(), n, kept.as<uint64_t>() + n, s));
            SPG_CUDA_TRY(cudaMemcpyAsync(&nnz, kept.as<uint64_t>() + n, 8, cudaMemcpyDeviceToHost, s));
            SPG_TRY(c->phase_sync(s));
            if (nnz == m) {  // nothing dropped: the staging arrays are the CSR
                out_cols = std::move(scols);
                out_vals = std::move(svals);
            } else {
                SPG_TRY(out_cols.alloc(csr_alloc_elems(nnz) * sizeof(uint32_t), s));
                SPG_TRY(out_vals.alloc(csr_alloc_elems(nnz) * sizeof(double), s));
                first_grouped_compact<<<grid_for(m, LB, (unsigned)c->n_sms * 16), LB, 0, s>>>(
                    rows, s_off.as<uint64_t>(), kept.as<uint64_t>(), scols.as<uint32_t>(), svals.as<double>(), m,
                    out_cols.as<uint32_t>(), out_vals.as<double>());
                SPG_LAUNCH_CHECK();
            }
            A->invalidate_derived();
            A->off = std::move(kept);
            A->cols = std::move(out_cols);
            A->vals = std::move(out_vals);
            A->nnz = nnz;
            A->capacity = nnz;  // build_csr: exact
            A->built = true;
            A->may_have_zeros = false;
            SPG_TRY(c->phase_sync(s));
            return SPG_OK;
        }
    }
    if (m) {
        const unsigned g = grid_for(m, LB, (unsigned)c->n_sms * 16);
        SPG_TRY(sort_keys(c, rows, cols, m, n, A->n_cols, keys, idx, pre, s));
        const uint64_t tiles = (m + KTILE - 1) / KTILE;
        SPG_TRY(pos.alloc((tiles + 1) * sizeof(uint64_t), s));  // kept entries per tile, then their prefix
        first_keep_count<<<(unsigned)tiles, KT, 0, s>>>(keys.as<uint64_t>(), idx.as<uint32_t>(), vals, m,
                                                        pos.as<uint64_t>());
        SPG_LAUNCH_CHECK();
        SPG_TRY(exclusive_scan_u64(c, pos.as<uint64_t>(), tiles, pos.as<uint64_t>() + tiles, s));
        SPG_CUDA_TRY(cudaMemcpyAsync(&nnz, pos.as<uint64_t>() + tiles, 8, cudaMemcpyDeviceToHost, s));
        SPG_TRY(c->phase_sync(s));
        SPG_TRY(out_cols.alloc(csr_alloc_elems(nnz) * sizeof(uint32_t), s));
        SPG_TRY(out_vals.alloc(csr_alloc_elems(nnz) * sizeof(double), s));
        SPG_TRY(orow.alloc((nnz ? nnz : 1) * sizeof(uint32_t), s));
        first_keep_gather<<<(unsigned)tiles, KT, 0, s>>>(keys.as<uint64_t>(), idx.as<uint32_t>(), vals, m, cbits,
                                                         pos.as<uint64_t>(), orow.as<uint32_t>(),
                                                         out_cols.as<uint32_t>(), out_vals.as<double>());
        SPG_LAUNCH_CHECK();
    } else {
        SPG_TRY(out_cols.alloc(csr_alloc_elems(0) * sizeof(uint32_t), s));
        SPG_TRY(out_vals.alloc(csr_alloc_elems(0) * sizeof(double), s));
    }
    SPG_TRY(new_off.alloc(csr_off_elems(n) * sizeof(uint64_t), s));
    SPG_TRY(launch_row_offsets(c, orow.as<uint32_t>(), nnz, n, new_off.as<uint64_t>(), s));
    A->invalidate_derived();
    A->off = std::move(new_off);
    A->cols = std::move(out_cols);
    A->vals = std::move(out_vals);
    A->nnz = nnz;
    A->capacity = nnz;  // build_csr: exact
    A->built = true;
    A->may_have_zeros = false;
    SPG_TRY(c->phase_sync(s));
    return SPG_OK;
}

}  // namespace

// The lock proper, on device-resident staging arrays.
static int lock_device_impl(Ctx *c, Csr *A, const uint32_t *rows, const uint32_t *cols, const double *vals,
                            uint64_t m, cudaStream_t s) {
    if (m >= (1ull << 32))
        return set_error(SPG_ERR_UNSUPPORTED, "lock: %llu staged inserts exceed 2^32-1 per epoch",
                         (unsigned long long)m);
    // Range checks first: a failure leaves A untouched (matrix.hpp:161-171).
    // The same pass builds the sort keys and tells whether they are already
    // in order.
    Prepared pre;
    if (m) {
        DevBuf stats;
        SPG_TRY(stats.alloc(5 * sizeof(unsigned), s));
        SPG_CUDA_TRY(cudaMemsetAsync(stats.ptr, 0, 5 * sizeof(unsigned), s));
        if (((uintptr_t)rows | (uintptr_t)cols) % 16 == 0)
            lock_prepare<true><<<grid_for((m + 3) / 4, LB, (unsigned)c->n_sms * 16), LB, 0, s>>>(
                rows, cols, m, bits_for(A->n_cols), stats.as<unsigned>());
        else
            lock_prepare<false><<<grid_for(m, LB, (unsigned)c->n_sms * 16), LB, 0, s>>>(
                rows, cols, m, bits_for(A->n_cols), stats.as<unsigned>());
        SPG_LAUNCH_CHECK();
        unsigned h[5] = {0u, 0u, 1u, 1u, 1u};
        SPG_CUDA_TRY(cudaMemcpyAsync(h, stats.ptr, 5 * sizeof(unsigned), cudaMemcpyDeviceToHost, s));
        SPG_TRY(c->phase_sync(s));
        if ((uint64_t)h[0] >= A->n_rows)
            return set_error(SPG_ERR_OUT_OF_RANGE, "spira::matrix: row_index out of range (%u >= %llu)", h[0],
                             (unsigned long long)A->n_rows);
        if ((uint64_t)h[1] >= A->n_cols)
            return set_error(SPG_ERR_OUT_OF_RANGE, "spira::matrix: col_index out of range (%u >= %llu)", h[1],
                             (unsigned long long)A->n_cols);
        pre.unsorted = h[2];
        pre.ungrouped = h[3];
        pre.not_strict = h[4];
        pre.ready = true;
    }
    const uint64_t n = A->n_rows;
    const bool has_old = A->built;
    if (has_old && m == 0) return SPG_OK;  // no dirty row: Spira's merge leaves the CSR as it is
    if (!has_old) return first_lock(c, A, rows, cols, vals, m, &pre, s);

    Delta D;
    if (m) SPG_TRY(sort_dedup(c, rows, cols, vals, m, n, A->n_cols, D, &pre, s));
    DevBuf doff;
    SPG_TRY(row_offsets(c, D.row.as<uint32_t>(), D.u, n, doff, s));

    if (has_old && A->may_have_zeros && A->nnz) {
        // Fold explicit old zeros of dirty rows into the delta as deletes.
        DevBuf zpos;
        SPG_TRY(zpos.alloc((A->nnz + 1) * sizeof(uint64_t), s));
        const unsigned gz = grid_for(n, LB, (unsigned)c->n_sms * 32);
        zero_entries_in_dirty_rows<<<gz, LB, 0, s>>>(A->d_off(), A->d_cols(), A->d_vals(), n, doff.as<uint64_t>(),
                                                     zpos.as<uint64_t>(), nullptr, nullptr, nullptr, 0);
        SPG_LAUNCH_CHECK();
        SPG_TRY(exclusive_scan_u64(c, zpos.as<uint64_t>(), A->nnz, zpos.as<uint64_t>() + A->nnz, s));
        uint64_t nz = 0;
        SPG_CUDA_TRY(cudaMemcpyAsync(&nz, zpos.as<uint64_t>() + A->nnz, 8, cudaMemcpyDeviceToHost, s));
        SPG_TRY(c->phase_sync(s));
        if (nz) {
            const uint64_t m2 = nz + D.u;
            DevBuf r2, c2, v2;
            SPG_TRY(r2.alloc(m2 * sizeof(uint32_t), s));
            SPG_TRY(c2.alloc(m2 * sizeof(uint32_t), s));
            SPG_TRY(v2.alloc(m2 * sizeof(double), s));
            zero_entries_in_dirty_rows<<<gz, LB, 0, s>>>(A->d_off(), A->d_cols(), A->d_vals(), n,
                                                         doff.as<uint64_t>(), nullptr, r2.as<uint32_t>(),
                                                         c2.as<uint32_t>(), zpos.as<uint64_t>(), 1);
            SPG_LAUNCH_CHECK();
            fill_f64<<<grid_for(nz, LB, 4096), LB, 0, s>>>(v2.as<double>(), nz, 0.0);
            SPG_LAUNCH_CHECK();
            if (D.u) {
                SPG_CUDA_TRY(cudaMemcpyAsync(r2.as<uint32_t>() + nz, D.row.ptr, D.u * 4, cudaMemcpyDeviceToDevice, s));
                SPG_CUDA_TRY(cudaMemcpyAsync(c2.as<uint32_t>() + nz, D.col.ptr, D.u * 4, cudaMemcpyDeviceToDevice, s));
                SPG_CUDA_TRY(cudaMemcpyAsync(v2.as<double>() + nz, D.val.ptr, D.u * 8, cudaMemcpyDeviceToDevice, s));
            }
            Delta D2;
            SPG_TRY(sort_dedup(c, r2.as<uint32_t>(), c2.as<uint32_t>(), v2.as<double>(), m2, n, A->n_cols, D2,
                               nullptr, s));
            D = std::move(D2);
            SPG_TRY(row_offsets(c, D.row.as<uint32_t>(), D.u, n, doff, s));
        }
    }

    const uint64_t u = D.u;
    DevBuf ins, P;
    SPG_TRY(ins.alloc((u ? u : 1) * sizeof(uint32_t), s));
    SPG_TRY(P.alloc((u + 1) * sizeof(int64_t), s));
    SPG_CUDA_TRY(cudaMemsetAsync(P.as<int64_t>() + u, 0, sizeof(int64_t), s));
    if (u) {
        merge_delta_probe<<<grid_for(u, LB, (unsigned)c->n_sms * 32), LB, 0, s>>>(
            A->d_off(), A->d_cols(), has_old, D.row.as<uint32_t>(), D.col.as<uint32_t>(), D.val.as<double>(), u,
            ins.as<uint32_t>(), P.as<int64_t>());
        SPG_LAUNCH_CHECK();
    }
    SPG_TRY(exclusive_scan_i64(c, P.as<int64_t>(), u + 1, s));

    DevBuf new_off;
    SPG_TRY(new_off.alloc(csr_off_elems(n) * sizeof(uint64_t), s));
    merge_row_counts<<<grid_for(n + 1, LB, (unsigned)c->n_sms * 32), LB, 0, s>>>(
        A->d_off(), has_old, doff.as<uint64_t>(), P.as<int64_t>(), n, new_off.as<uint64_t>());
    SPG_LAUNCH_CHECK();
    SPG_TRY(exclusive_scan_u64(c, new_off.as<uint64_t>(), n + 1, nullptr, s));
    uint64_t new_nnz = 0;
    SPG_CUDA_TRY(cudaMemcpyAsync(&new_nnz, new_off.as<uint64_t>() + n, 8, cudaMemcpyDeviceToHost, s));
    SPG_TRY(c->phase_sync(s));

    uint64_t cap;
    if (!has_old) {
        cap = new_nnz;  // build_csr: exact
    } else {
        const uint64_t total_ub = A->nnz + u;
        cap = (total_ub <= A->capacity) ? A->capacity : total_ub + total_ub / 2;
    }
    DevBuf out_cols, out_vals;
    SPG_TRY(out_cols.alloc(csr_alloc_elems(cap) * sizeof(uint32_t), s));
    SPG_TRY(out_vals.alloc(csr_alloc_elems(cap) * sizeof(double), s));
    if (has_old && A->nnz) {
        const uint64_t chunks = (A->nnz + MO_CHUNK - 1) / MO_CHUNK;
        DevBuf win;
        SPG_TRY(win.alloc(2 * chunks * sizeof(uint64_t), s));
        merge_windows<<<grid_for(chunks, LB), LB, 0, s>>>(A->d_off(), n, A->nnz, chunks, win.as<uint64_t>());
        SPG_LAUNCH_CHECK();
        merge_write_old<<<(unsigned)chunks, LB, 0, s>>>(A->d_off(), A->d_cols(), A->d_vals(), win.as<uint64_t>(),
                                                        A->nnz, doff.as<uint64_t>(), D.col.as<uint32_t>(),
                                                        P.as<int64_t>(), new_off.as<uint64_t>(),
                                                        out_cols.as<uint32_t>(), out_vals.as<double>());
        SPG_LAUNCH_CHECK();
    }
    if (u) {
        merge_write_delta<<<grid_for(u, LB, (unsigned)c->n_sms * 32), LB, 0, s>>>(
            D.row.as<uint32_t>(), D.col.as<uint32_t>(), D.val.as<double>(), ins.as<uint32_t>(), doff.as<uint64_t>(),
            P.as<int64_t>(), u, new_off.as<uint64_t>(), out_cols.as<uint32_t>(), out_vals.as<double>());
        SPG_LAUNCH_CHECK();
    }
    A->invalidate_derived();
    A->off = std::move(new_off);
    A->cols = std::move(out_cols);
    A->vals = std::move(out_vals);
    A->nnz = new_nnz;
    A->capacity = cap;
    A->built = true;
    // Zeros of dirty rows were consumed; clean rows may still hold loaded zeros.
    SPG_TRY(c->phase_sync(s));
    return SPG_OK;
}

}  // namespace spg

using namespace spg;

extern "C" {

int spg_lock_device(spg_ctx *c, spg_csr *A, const uint32_t *d_rows, const uint32_t *d_cols, const double *d_vals,
                    uint64_t n_staged) {
    if (!c || !A) return set_error(SPG_ERR_INVALID_ARGUMENT, "spg_lock_device: null handle");
    SPG_CHECK_LIVE(A);
    if (n_staged && (!d_rows || !d_cols || !d_vals))
        return set_error(SPG_ERR_INVALID_ARGUMENT, "spg_lock_device: null staging array");
    SPG_CUDA_TRY(cudaSetDevice(c->device));
    return lock_device_impl(c, A, d_rows, d_cols, d_vals, n_staged, c->stream);
}

int spg_lock(spg_ctx *c, spg_csr *A, const uint32_t *rows, const uint32_t *cols, const double *vals,
             uint64_t n_staged) {
    if (!c || !A) return set_error(SPG_ERR_INVALID_ARGUMENT, "spg_lock: null handle");
    SPG_CHECK_LIVE(A);
    if (n_staged && (!rows || !cols || !vals))
        return set_error(SPG_ERR_INVALID_ARGUMENT, "spg_lock: null staging array");
    SPG_CUDA_TRY(cudaSetDevice(c->device));
    cudaStream_t s = c->stream;
    DevBuf r, cl, v;
    if (n_staged) {
        SPG_TRY(r.alloc(n_staged * sizeof(uint32_t), s));
        SPG_TRY(cl.alloc(n_staged * sizeof(uint32_t), s));
        SPG_TRY(v.alloc(n_staged * sizeof(double), s));
        SPG_CUDA_TRY(cudaMemcpyAsync(r.ptr, rows, n_staged * sizeof(uint32_t), cudaMemcpyHostToDevice, s));
        SPG_CUDA_TRY(cudaMemcpyAsync(cl.ptr, cols, n_staged * sizeof(uint32_t), cudaMemcpyHostToDevice, s));
        SPG_CUDA_TRY(cudaMemcpyAsync(v.ptr, vals, n_staged * sizeof(double), cudaMemcpyHostToDevice, s));
    }
    return lock_device_impl(c, A, r.as<uint32_t>(), cl.as<uint32_t>(), v.as<double>(), n_staged, s);
}

}  // extern "C"
