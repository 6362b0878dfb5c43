// spg_spmv_adaptive.cu — SPG_SPMV_ADAPTIVE(16), the FP64 SpMV shaped for GB300.
//
// Two limits meet on GB300: FP64 runs at 2 fused multiply-adds per clock per
// SM (ncu: sm__sass_thread_inst_executed_op_dfma_pred_on.peak_sustained = 2),
// and each SM sub-partition issues one warp instruction per clock. At ~12 B
// per nonzero HBM, the FP64 pipe and the issue slots all finish a SpMV in
// about the same time, so a kernel must spend one DFMA lane and only a few
// instructions per nonzero, whatever the row-length distribution.
//
// Plan (built on the device once per lock, cached on the matrix):
//   bitmap     bit p set iff nonzero p is the first of its row;
//   chunk_base number of row starts before each chunk of 32 * ITEMS nonzeros;
//   nzrow      index of the i-th non-empty row (only if empty rows exist) and
//              the list of empty rows (their y is 0).
// Kernel: one warp per chunk. Lane l owns the ITEMS consecutive nonzeros
// [32 ITEMS w + ITEMS l, + ITEMS): it loads them with 16-byte vector loads
// (the CSR arrays are padded so these never leave their allocations), issues
// its x gathers, and runs one FMA chain, closing a row at every bitmap bit.
// Rows that start and end inside a lane are written directly. The piece a
// lane holds of a row started in an earlier lane is combined with a warp
// segmented scan of the lanes' tail pieces (shuffles only when every lane
// starts a row, the common case for short rows); rows crossing a chunk
// boundary leave a (row, partial) record per chunk, summed in chunk order by
// a second small kernel. Deterministic for a given matrix and variant.
//
// SPG_SPMV_INTERLEAVED runs the same kernel over a copy of cols and vals
// stored lane-interleaved within each 512-nonzero chunk, both in pairs: the
// k-th pair of nonzeros of every lane lies side by side (16 bytes of values,
// 8 bytes of columns per lane). A lane still owns 16 consecutive nonzeros and
// sums them in the same order, so y is bit-identical to SPG_SPMV_ADAPTIVE16,
// but each warp load is one contiguous 512-byte (values) or 256-byte
// (columns) access instead of 32 strided pieces, and every 128-byte line is
// requested once. On random-column matrices the x gathers saturate the L1 to
// L2 request path; the strided loads of the in-place layout cost about as
// many L1 wavefronts again, the interleaved ones an eighth of that.
#include "spg_internal.cuh"

namespace spg {
namespace {

constexpr uint32_t NONE = 0xFFFFFFFFu;

struct Rec {
    uint32_t row;
    uint32_t pad;
    double val;
};

__device__ __forceinline__ double ldx(const double *__restrict__ x, uint32_t c) { return __ldg(x + c); }

__device__ __forceinline__ unsigned lanemask_lt() {
    unsigned m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// ---------------------------------------------------------------- plan
__global__ void seg_row_starts(const uint64_t *__restrict__ off, uint64_t n, unsigned *__restrict__ bitmap,
                               uint64_t *__restrict__ ne) {
    const uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    const uint64_t b = off[r], e = off[r + 1];
    ne[r] = (e > b) ? 1 : 0;
    if (e > b) atomicOr(bitmap + (b >> 5), 1u << (b & 31));
}

__global__ void seg_word_popc(const unsigned *__restrict__ bitmap, uint64_t n_words, uint64_t *__restrict__ pc) {
    const uint64_t w = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (w < n_words) pc[w] = __popc(bitmap[w]);
}

__global__ void seg_chunk_base(const uint64_t *__restrict__ pc_scan, uint64_t n_chunks, int words_per_chunk,
                               uint32_t *__restrict__ base) {
    const uint64_t c = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c < n_chunks) base[c] = (uint32_t)pc_scan[c * words_per_chunk];
}

__global__ void seg_row_maps(const uint64_t *__restrict__ ne_scan, uint64_t n, uint32_t *__restrict__ nzrow,
                             uint32_t *__restrict__ empty) {
    const uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    const uint64_t i = ne_scan[r];
    if (ne_scan[r + 1] != i) nzrow[i] = (uint32_t)r;
    else empty[r - i] = (uint32_t)r;
}

// ---------------------------------------------------------------- SpMV
// ITEMS nonzeros per lane, handled in sub-batches of SUB (loads, gathers, FMAs)
// to keep registers low enough for MINB CTAs of 256 threads per SM. INTER: cols
// and vals are the lane-interleaved copies (ITEMS == 16). The sub-batch size
// does not change the FMA order. INTERLEAVED runs SUB = 2 at 32 registers, 8
// CTAs (64 warps) per SM: on the random-column Zipf matrix its gathers are
// latency-bound, and more warps with 2 gathers each in flight beat fewer with
// 8 (4M rows: 0.268 ms against 0.289-0.299 with SUB = 8 at 4 CTAs, 0.276 with
// SUB = 4 at 5 CTAs).
template <int ITEMS, int SUB, bool INTER, int MINB = 4>
__global__ void __launch_bounds__(256, MINB)
spmv_seg(const uint32_t *__restrict__ cols, const double *__restrict__ vals, const double *__restrict__ x,
         double *__restrict__ y, uint64_t nnz, const unsigned *__restrict__ bitmap,
         const uint32_t *__restrict__ chunk_base, const uint32_t *__restrict__ nzrow, Rec *__restrict__ recs,
         uint64_t c0, uint64_t c1) {  // chunks [c0, c1)
    const uint64_t w = c0 + (((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    if (w >= c1) return;
    static_assert(INTER ? SUB % 2 == 0 : SUB % 4 == 0, "loads come in 16-byte pieces (interleaved: pairs)");
    const uint64_t p0 = w * (32ull * ITEMS) + (uint64_t)lane * ITEMS;
    unsigned word = 0;
    if (p0 < nnz) {
        word = bitmap[p0 >> 5] >> (p0 & 31);
        if constexpr (ITEMS < 32) word &= (1u << ITEMS) - 1u;
        if (nnz - p0 < (uint64_t)ITEMS) word &= (1u << (unsigned)(nnz - p0)) - 1u;
    }
    // row starts before my first item
    const int pc = __popc(word);
    int incl = pc;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += t;
    }
    const uint32_t sb = chunk_base[w] + (uint32_t)(incl - pc);
    uint32_t cur = sb - 1u;  // row in progress at my first item (NONE before the first row)
    double acc = 0.0, head = 0.0;
    bool seen = false;
#pragma unroll
    for (int h = 0; h < ITEMS / SUB; ++h) {
        const uint64_t base = p0 + (uint64_t)SUB * h;
        const uint32_t nv = base < nnz ? (uint32_t)min(nnz - base, (uint64_t)SUB) : 0u;
        double v[SUB], g[SUB];
        uint32_t c[SUB];
        if (nv) {
            if constexpr (INTER) {
                // pair k of lane l sits at chunk + 64 k + 2 l (vals and cols alike)
                const uint64_t cb = w * (32ull * ITEMS);
#pragma unroll
                for (int u = 0; u < SUB; u += 2) {
                    const double2 t = __ldcs(reinterpret_cast<const double2 *>(
                        vals + cb + 64u * (unsigned)((SUB * h + u) >> 1) + 2u * (unsigned)lane));
                    v[u] = t.x;
                    v[u + 1] = t.y;
                }
#pragma unroll
                for (int u = 0; u < SUB; u += 2) {
                    const uint2 q = __ldcs(reinterpret_cast<const uint2 *>(
                        cols + cb + 64u * (unsigned)((SUB * h + u) >> 1) + 2u * (unsigned)lane));
                    c[u] = q.x;
                    c[u + 1] = q.y;
                }
            } else {
#pragma unroll
                for (int u = 0; u < SUB; u += 2) {
                    const double2 t = *reinterpret_cast<const double2 *>(vals + base + u);
                    v[u] = t.x;
                    v[u + 1] = t.y;
                }
#pragma unroll
                for (int u = 0; u < SUB; u += 4) {
                    const uint4 t = *reinterpret_cast<const uint4 *>(cols + base + u);
                    c[u] = t.x;
                    c[u + 1] = t.y;
                    c[u + 2] = t.z;
                    c[u + 3] = t.w;
                }
            }
        }
#pragma unroll
        for (int u = 0; u < SUB; ++u) {
            g[u] = 0.0;
            if ((uint32_t)u < nv) g[u] = ldx(x, c[u]);  // only real columns are read
            else v[u] = 0.0;
        }
#pragma unroll
        for (int u = 0; u < SUB; ++u) {
            if ((word >> (SUB * h + u)) & 1u) {  // a row starts at this nonzero: close the previous one
                if (!seen) {
                    head = acc;
                    seen = true;
                } else {
                    y[nzrow ? nzrow[cur] : cur] = acc;
                }
                acc = 0.0;
                ++cur;
            }
            acc = fma(g[u], v[u], acc);
        }
    }
    // acc: tail piece of row `cur`; head: piece of row sb-1 before my first start.
    const bool has = word != 0;
    const unsigned hasmask = __ballot_sync(0xffffffffu, has);
    double carry_in;  // sum of the earlier lanes' pieces of the row I receive
    if (hasmask == 0xffffffffu) {
        carry_in = __shfl_up_sync(0xffffffffu, acc, 1);
        if (lane == 0) carry_in = 0.0;
    } else {
        // segmented inclusive scan of tail pieces; a lane with a start opens a segment
        double v = acc;
        bool f = has;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const double tv = __shfl_up_sync(0xffffffffu, v, o);
            const bool tf = __shfl_up_sync(0xffffffffu, f, o);
            if (lane >= o && !f) v += tv;
            if (lane >= o) f = f || tf;
        }
        carry_in = __shfl_up_sync(0xffffffffu, v, 1);
        if (lane == 0) carry_in = 0.0;
    }
    const bool started_in_chunk = (hasmask & lanemask_lt()) != 0;
    if (has) {
        const double total = carry_in + head;
        if (started_in_chunk) {
            y[nzrow ? nzrow[sb - 1u] : sb - 1u] = total;
        } else {
            // first lane with a start: the piece of the row entering the chunk
            Rec r;
            r.row = (lane == 0 && (word & 1u)) ? NONE : sb - 1u;
            r.pad = 0;
            r.val = total;
            recs[2 * w] = r;
        }
    }
    if (lane == 31) {
        const double out = has ? acc : carry_in + acc;  // inclusive value at the chunk end
        Rec r;
        r.pad = 0;
        r.val = out;
        if (hasmask == 0) {  // the entering row runs through the whole chunk
            r.row = cur;
            recs[2 * w] = r;
            r.row = NONE;
            r.val = 0.0;
            recs[2 * w + 1] = r;
        } else {
            r.row = cur;
            recs[2 * w + 1] = r;
        }
    }
}

// Lane-interleaved copy for SPG_SPMV_INTERLEAVED: nonzero p = 512 w + 16 l + u
// (chunk w, lane l, item u) goes to 512 w + 64 (u / 2) + 2 l + u % 2 in vals and
// cols alike; the tail of the last chunk is zero.
__global__ void seg_interleave(const uint32_t *__restrict__ cols, const double *__restrict__ vals, uint64_t nnz,
                               uint64_t n_slots, uint32_t *__restrict__ icols, double *__restrict__ ivals) {
    for (uint64_t p = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; p < n_slots;
         p += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t w = p >> 9;
        const unsigned q = (unsigned)(p & 511), l = q >> 4, u = q & 15;
        const bool real = p < nnz;
        ivals[(w << 9) + 64u * (u >> 1) + 2u * l + (u & 1u)] = real ? vals[p] : 0.0;
        icols[(w << 9) + 64u * (u >> 1) + 2u * l + (u & 1u)] = real ? cols[p] : 0u;
    }
}

// Rows crossing chunk boundaries: each run of records with the same row
// (at most one NONE record between two of them) is summed in chunk order by
// the thread holding its first record.
// Runs starting at records [q0, q1) are summed (a run may read on up to
// n_recs).
__global__ void seg_fixup(const Rec *__restrict__ recs, uint64_t q0, uint64_t q1, uint64_t n_recs,
                          const uint32_t *__restrict__ nzrow, double *__restrict__ y) {
    const uint64_t q = q0 + (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= q1) return;
    const uint32_t row = recs[q].row;
    if (row == NONE) return;
    if (q > 0) {
        uint64_t p = q - 1;
        if (recs[p].row == NONE && p > 0) --p;
        if (recs[p].row == row) return;  // not the first record of this row
    }
    double s = recs[q].val;
    uint64_t k = q + 1;
    while (k < n_recs) {
        uint32_t r = recs[k].row;
        if (r == NONE && k + 1 < n_recs) {
            ++k;
            r = recs[k].row;
        }
        if (r != row) break;
        s += recs[k].val;
        ++k;
    }
    y[nzrow ? nzrow[row] : row] = s;
}

__global__ void seg_empty_rows(const uint32_t *__restrict__ empty, uint64_t n_empty, double *__restrict__ y) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n_empty) y[empty[i]] = 0.0;
}

}  // namespace

// Plan layout (Csr::plan_adaptive, or Csr::plan_inter for the interleaved
// variant): items = bitmap, extra0 = chunk_base, aux = chunk records,
// extra1 = nzrow, extra2 = empty rows, count1 = #empty; interleaved only:
// extra3 = cols, extra4 = vals in lane-interleaved order.
int build_adaptive_plan(Ctx *c, Csr *A, int variant, cudaStream_t s) {
    const SegShape sh = seg_shape(variant);
    const int items = sh.items;
    const bool inter = sh.inter;
    if (!items) return set_error(SPG_ERR_INVALID_ARGUMENT, "adaptive plan: variant %d", variant);
    SpmvPlan &slot = adaptive_plan_of(A, variant);
    const int kind = 2 * items + (inter ? 1 : 0);  // tiles of one variant share its plan
    if (slot.kind == kind) return SPG_OK;
    const uint64_t n = A->n_rows, nnz = A->nnz;
    const uint64_t chunk = 32ull * items;
    const uint64_t n_chunks = (nnz + chunk - 1) / chunk;
    const uint64_t n_words = (nnz + 31) / 32 + 1;
    if (n_chunks >= (1ull << 31)) return set_error(SPG_ERR_UNSUPPORTED, "adaptive plan: too many chunks");
    SpmvPlan P;
    DevBuf bm, cb, ne, recs, nzrow, empty, pc;
    SPG_TRY(bm.alloc(n_words * sizeof(unsigned), s));
    SPG_CUDA_TRY(cudaMemsetAsync(bm.ptr, 0, n_words * sizeof(unsigned), s));
    SPG_TRY(ne.alloc((n + 1) * sizeof(uint64_t), s));
    if (n) {
        seg_row_starts<<<grid_for(n, 256), 256, 0, s>>>(A->d_off(), n, bm.as<unsigned>(), ne.as<uint64_t>());
        SPG_LAUNCH_CHECK();
    }
    SPG_TRY(exclusive_scan_u64(c, ne.as<uint64_t>(), n, ne.as<uint64_t>() + n, s));
    uint64_t n_ne = 0;
    SPG_CUDA_TRY(cudaMemcpyAsync(&n_ne, ne.as<uint64_t>() + n, 8, cudaMemcpyDeviceToHost, s));
    SPG_TRY(pc.alloc((n_words + 1) * sizeof(uint64_t), s));
    seg_word_popc<<<grid_for(n_words, 256), 256, 0, s>>>(bm.as<unsigned>(), n_words, pc.as<uint64_t>());
    SPG_LAUNCH_CHECK();
    SPG_TRY(exclusive_scan_u64(c, pc.as<uint64_t>(), n_words, pc.as<uint64_t>() + n_words, s));
    SPG_TRY(cb.alloc((n_chunks ? n_chunks : 1) * sizeof(uint32_t), s));
    if (n_chunks) {
        seg_chunk_base<<<grid_for(n_chunks, 256), 256, 0, s>>>(pc.as<uint64_t>(), n_chunks, items, cb.as<uint32_t>());
        SPG_LAUNCH_CHECK();
    }
    SPG_CUDA_TRY(cudaStreamSynchronize(s));
    const uint64_t n_empty = n - n_ne;
    if (n_empty) {
        SPG_TRY(nzrow.alloc((n_ne ? n_ne : 1) * sizeof(uint32_t), s));
        SPG_TRY(empty.alloc(n_empty * sizeof(uint32_t), s));
        seg_row_maps<<<grid_for(n, 256), 256, 0, s>>>(ne.as<uint64_t>(), n, nzrow.as<uint32_t>(),
                                                      empty.as<uint32_t>());
        SPG_LAUNCH_CHECK();
    }
    SPG_TRY(recs.alloc((2 * n_chunks + 1) * sizeof(Rec), s));
    if (inter && n_chunks) {
        const uint64_t n_slots = n_chunks * chunk;
        SPG_TRY(P.extra3.alloc(n_slots * sizeof(uint32_t), s));
        SPG_TRY(P.extra4.alloc(n_slots * sizeof(double), s));
        seg_interleave<<<grid_for(n_slots, 256, (unsigned)c->n_sms * 16), 256, 0, s>>>(
            A->d_cols(), A->d_vals(), nnz, n_slots, P.extra3.as<uint32_t>(), P.extra4.as<double>());
        SPG_LAUNCH_CHECK();
    }
    P.kind = kind;
    P.n_items = n_chunks;
    P.items = std::move(bm);
    P.aux = std::move(recs);
    P.extra0 = std::move(cb);
    P.extra1 = std::move(nzrow);
    P.extra2 = std::move(empty);
    P.count1 = n_empty;
    slot = std::move(P);
    return SPG_OK;
}

namespace {

// The chunk kernel over chunks [c0, c1).
int launch_seg(const SpmvPlan &P, const Csr *A, const double *x, double *y, int variant, uint64_t c0, uint64_t c1,
               cudaStream_t s) {
    if (c1 <= c0) return SPG_OK;
    const uint32_t *nzrow = P.count1 ? P.extra1.as<uint32_t>() : nullptr;
    const unsigned grid = grid_for((c1 - c0) * 32, 256);
    const uint32_t *ic = P.extra3.as<uint32_t>(), *cc = A->d_cols();
    const double *iv = P.extra4.as<double>(), *cv = A->d_vals();
    const unsigned *bm = P.items.as<unsigned>();
    const uint32_t *cb = P.extra0.as<uint32_t>();
    Rec *rc = P.aux.as<Rec>();
    const uint64_t nnz = A->nnz;
    switch (variant) {
        case SPG_SPMV_INTERLEAVED:
            spmv_seg<16, 2, true, 8><<<grid, 256, 0, s>>>(ic, iv, x, y, nnz, bm, cb, nzrow, rc, c0, c1);
            break;
        case SPG_SPMV_INTERLEAVED_S4:
            spmv_seg<16, 4, true, 5><<<grid, 256, 0, s>>>(ic, iv, x, y, nnz, bm, cb, nzrow, rc, c0, c1);
            break;
        case SPG_SPMV_INTERLEAVED_S8:
            spmv_seg<16, 8, true, 4><<<grid, 256, 0, s>>>(ic, iv, x, y, nnz, bm, cb, nzrow, rc, c0, c1);
            break;
        case SPG_SPMV_ADAPTIVE16:
            spmv_seg<16, 8, false, 4><<<grid, 256, 0, s>>>(cc, cv, x, y, nnz, bm, cb, nzrow, rc, c0, c1);
            break;
        case SPG_SPMV_ADAPTIVE16_S4:
            spmv_seg<16, 4, false, 6><<<grid, 256, 0, s>>>(cc, cv, x, y, nnz, bm, cb, nzrow, rc, c0, c1);
            break;
        case SPG_SPMV_ADAPTIVE:
            spmv_seg<32, 8, false, 4><<<grid, 256, 0, s>>>(cc, cv, x, y, nnz, bm, cb, nzrow, rc, c0, c1);
            break;
        case SPG_SPMV_ADAPTIVE_S16:
            spmv_seg<32, 16, false, 2><<<grid, 256, 0, s>>>(cc, cv, x, y, nnz, bm, cb, nzrow, rc, c0, c1);
            break;
        default:
            return set_error(SPG_ERR_INVALID_ARGUMENT, "spmv: variant %d is not a chunk kernel", variant);
    }
    SPG_LAUNCH_CHECK();
    return SPG_OK;
}

// The fix-up of the runs starting at records of chunks [c0, c1).
int launch_fixup(const SpmvPlan &P, double *y, uint64_t c0, uint64_t c1, cudaStream_t s) {
    if (c1 <= c0) return SPG_OK;
    const uint32_t *nzrow = P.count1 ? P.extra1.as<uint32_t>() : nullptr;
    seg_fixup<<<grid_for(2 * (c1 - c0), 256), 256, 0, s>>>(P.aux.as<Rec>(), 2 * c0, 2 * c1, 2 * P.n_items, nzrow, y);
    SPG_LAUNCH_CHECK();
    return SPG_OK;
}

int launch_empty_rows(const SpmvPlan &P, double *y, cudaStream_t s) {
    if (!P.count1) return SPG_OK;
    seg_empty_rows<<<grid_for(P.count1, 256), 256, 0, s>>>(P.extra2.as<uint32_t>(), P.count1, y);
    SPG_LAUNCH_CHECK();
    return SPG_OK;
}

}  // namespace

int spmv_adaptive(Ctx *c, Csr *A, const double *x, double *y, int variant, cudaStream_t s) {
    SPG_TRY(build_adaptive_plan(c, A, variant, s));
    const SpmvPlan &P = adaptive_plan_of(A, variant);
    SPG_TRY(launch_seg(P, A, x, y, variant, 0, P.n_items, s));
    SPG_TRY(launch_fixup(P, y, 0, P.n_items, s));
    SPG_TRY(launch_empty_rows(P, y, s));
    return SPG_OK;
}

int spmv_adaptive_blocks(Ctx *c, Csr *A, int variant, int nb, std::vector<uint64_t> *rows, cudaStream_t s) {
    SPG_TRY(build_adaptive_plan(c, A, variant, s));
    SpmvPlan &P = adaptive_plan_of(A, variant);
    const uint64_t nch = P.n_items;
    if (P.host_nb == nb && (int)P.host_rows.size() == nb + 1) {
        *rows = P.host_rows;
        return SPG_OK;
    }
    // Blocks must be long enough that a row starting in block b ends by the
    // end of block b + 1 (the fix-up of block b reads ahead one block).
    bool known = false;
    SPG_TRY(csr_max_row(c, A, s, &known));
    const uint64_t max_row = known ? A->max_row : A->nnz;  // no row is longer than nnz
    const uint64_t chunk_nnz = 32ull * seg_shape(variant).items;
    while (nb > 1 && (nch / nb) * chunk_nnz < max_row + 2 * chunk_nnz) --nb;
    if (nb < 1) nb = 1;
    // first (actual) row starting at or after each block's first chunk
    rows->assign(nb + 1, 0);
    const uint64_t n_nonempty = A->n_rows - P.count1;
    for (int b = 1; b < nb; ++b) {
        const uint64_t ch = nch * (uint64_t)b / (uint64_t)nb;  // < nch
        uint32_t v = 0;  // non-empty rows starting before chunk ch = index of the first one at or after it
        SPG_CUDA_TRY(cudaMemcpyAsync(&v, P.extra0.as<uint32_t>() + ch, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
        SPG_CUDA_TRY(cudaStreamSynchronize(s));
        uint64_t r = A->n_rows;
        if (v < n_nonempty) {
            r = v;
            if (P.count1) {  // map to the actual row
                uint32_t a = 0;
                SPG_CUDA_TRY(cudaMemcpyAsync(&a, P.extra1.as<uint32_t>() + v, sizeof(uint32_t),
                                             cudaMemcpyDeviceToHost, s));
                SPG_CUDA_TRY(cudaStreamSynchronize(s));
                r = a;
            }
        }
        (*rows)[b] = r;
    }
    (*rows)[0] = 0;
    (*rows)[nb] = A->n_rows;
    P.host_nb = nb;
    P.host_rows = *rows;
    return SPG_OK;
}

int spmv_adaptive_stage(Ctx *c, Csr *A, const double *x, double *y, int variant, int i, cudaStream_t s) {
    (void)c;
    const SpmvPlan &P = adaptive_plan_of(A, variant);
    const int nb = P.host_nb;
    const uint64_t nch = P.n_items;
    auto cb = [&](int b) { return nch * (uint64_t)b / (uint64_t)nb; };
    if (i == 0) SPG_TRY(launch_empty_rows(P, y, s));
    if (i < nb) SPG_TRY(launch_seg(P, A, x, y, variant, cb(i), cb(i + 1), s));
    if (i >= 1) SPG_TRY(launch_fixup(P, y, cb(i - 1), cb(i), s));
    return SPG_OK;
}

}  // namespace spg
