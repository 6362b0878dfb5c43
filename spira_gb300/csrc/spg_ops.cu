// spg_ops.cu — element-wise CSR operations and queries around the hot path:
// C = A + B, C = A * s and A / s, row sums, batched point lookups and
// nnz-balanced row partitions.
//
//   add      serial/matrix_addition.hpp:34-110, parallel/algorithms/
//            matrix_addition.hpp:24-99: per row a two-pointer merge of A's
//            and B's CSR slices; equal columns give a + b (one IEEE add),
//            kept unless the sum is +-0; other entries are copied; the result
//            is locked, which drops every stored zero (csr_build.hpp:49,71).
//   scale    serial/scalars.hpp:10-67: val * s or val / s for every committed
//            entry, zeros dropped by the lock that follows; division by a zero
//            scalar is a domain error.
//   row sums matrix.hpp:438-443, row.hpp:208-216, csr_storage_soa.hpp:114-120:
//            a locked row's sum, acc += v left to right from 0.0.
//   lookup   row.hpp:190-204 (locked rows): binary search of the CSR slice.
//   bounds   parallel/partition.hpp:78-126: first row whose nnz prefix
//            reaches max(1, t * nnz / T); a uniform split when nnz == 0.
//
// Addition on the GPU, entry-parallel with no per-row loop (any row-length
// mix balances): every entry of A finds by binary search the first entry of
// B's row at or after its column (and whether it collides), every entry of B
// the same in A's row. Keep flags of A (sum or own value non-zero) and of B
// (no collision, value non-zero) are scanned separately into SA and SB. With
// ja the absolute position found in B for A entry e, and ib the one found in
// A for B entry f:
//     position of A entry e in C = SA[e] + SB[ja]
//     position of B entry f in C = SB[f] + SA[ib]
//     C offsets: off_C[r] = SA[off_A[r]] + SB[off_B[r]]
// since the kept entries before e in C are the kept A entries before e plus
// the kept B entries of earlier rows and of e's row below its column. Values
// are copied or summed once (__dadd_rn), so C is bit-exact.
#include <algorithm>
#include <vector>

#include "spg_internal.cuh"

namespace spg {
namespace {

constexpr int OB = 256;
constexpr uint64_t COLLIDE = 1ull << 63;  // high bit of a found position: the columns are equal


// Row holding entry e: the last r with off[r] <= e (rows before it end at or
// before e, empty rows share their successor's offset).
__device__ __forceinline__ uint64_t row_of(const uint64_t *__restrict__ off, uint64_t n_rows, uint64_t e) {
    uint64_t lo = 0, hi = n_rows - 1;
    while (lo < hi) {
        const uint64_t mid = (lo + hi + 1) >> 1;
        if (off[mid] <= e) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// First position in [b, e) whose column is >= c.
__device__ __forceinline__ uint64_t lower_col(const uint32_t *__restrict__ cols, uint64_t b, uint64_t e, uint32_t c) {
    while (b < e) {
        const uint64_t mid = (b + e) >> 1;
        if (cols[mid] < c) b = mid + 1;
        else e = mid;
    }
    return b;
}

// Keep flag and partner position of every entry of X against Y's rows; for X
// = A the kept value is the sum on a collision, for X = B a collision drops
// the entry (A's side holds the sum). A block takes a tile of PT consecutive
// entries: two searches find the rows of its first and last entry, the
// offsets of the rows in between go to shared memory (when they fit), and
// every entry finds its row there.
constexpr int PT = 2048, PROWS = 2048;

template <bool X_IS_A>
__global__ void __launch_bounds__(OB)
add_probe(const uint64_t *__restrict__ xoff, const uint32_t *__restrict__ xcols, const double *__restrict__ xvals,
          uint64_t nx, const uint64_t *__restrict__ yoff, const uint32_t *__restrict__ ycols,
          const double *__restrict__ yvals, uint64_t n_rows, uint64_t *__restrict__ keep,
          uint64_t *__restrict__ partner) {
    __shared__ uint64_t s_off[PROWS + 1];
    __shared__ uint64_t s_win[2];
    for (uint64_t e0 = blockIdx.x * (uint64_t)PT; e0 < nx; e0 += (uint64_t)gridDim.x * PT) {
        const uint64_t e1 = min(nx, e0 + PT);
        if (threadIdx.x == 0) s_win[0] = row_of(xoff, n_rows, e0);
        if (threadIdx.x == 32) s_win[1] = row_of(xoff, n_rows, e1 - 1);
        __syncthreads();
        const uint64_t r_lo = s_win[0], r_hi = s_win[1];
        const bool in_smem = r_hi - r_lo < PROWS;
        if (in_smem)
            for (uint64_t j = threadIdx.x; j <= r_hi - r_lo + 1; j += OB) s_off[j] = xoff[r_lo + j];
        __syncthreads();
        for (uint64_t e = e0 + threadIdx.x; e < e1; e += OB) {
            uint64_t r;
            if (in_smem) {  // last j with s_off[j] <= e
                uint64_t lo = 0, hi = r_hi - r_lo;
                while (lo < hi) {
                    const uint64_t mid = (lo + hi + 1) >> 1;
                    if (s_off[mid] <= e) lo = mid;
                    else hi = mid - 1;
                }
                r = r_lo + lo;
            } else {
                uint64_t lo = r_lo, hi = r_hi;
                while (lo < hi) {
                    const uint64_t mid = (lo + hi + 1) >> 1;
                    if (xoff[mid] <= e) lo = mid;
                    else hi = mid - 1;
                }
                r = lo;
            }
            const uint32_t c = xcols[e];
            const uint64_t yb = yoff[r], ye = yoff[r + 1];
            const uint64_t p = lower_col(ycols, yb, ye, c);
            const bool coll = p < ye && ycols[p] == c;
            bool k;
            if (X_IS_A) k = !is_zero(coll ? __dadd_rn(xvals[e], yvals[p]) : xvals[e]);
            else k = !coll && !is_zero(xvals[e]);
            keep[e] = k ? 1u : 0u;
            partner[e] = p | (coll ? COLLIDE : 0);
        }
        __syncthreads();
    }
}

__global__ void add_offsets(const uint64_t *__restrict__ aoff, const uint64_t *__restrict__ boff,
                            const uint64_t *__restrict__ sa, const uint64_t *__restrict__ sb, uint64_t n_rows,
                            uint64_t *__restrict__ coff) {
    for (uint64_t r = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; r <= n_rows;
         r += (uint64_t)gridDim.x * blockDim.x)
        coff[r] = sa[aoff[r]] + sb[boff[r]];
}

// Writes X's kept entries into C. sx = X's scanned keep flags (nx + 1
// entries), sy = Y's; X = A sums on a collision. A thread handles SI entries
// per step with their loads issued together.
template <bool X_IS_A>
__global__ void __launch_bounds__(OB)
add_scatter(const uint32_t *__restrict__ xcols, const double *__restrict__ xvals, uint64_t nx,
            const double *__restrict__ yvals, const uint64_t *__restrict__ sx, const uint64_t *__restrict__ sy,
            const uint64_t *__restrict__ partner, uint32_t *__restrict__ ccols, double *__restrict__ cvals) {
    constexpr int SI = 4;
    for (uint64_t e0 = blockIdx.x * (uint64_t)(OB * SI); e0 < nx; e0 += (uint64_t)gridDim.x * OB * SI) {
        uint64_t s0[SI], s1[SI], pp[SI];
#pragma unroll
        for (int q = 0; q < SI; ++q) {
            const uint64_t e = e0 + threadIdx.x + (uint64_t)q * OB;
            s0[q] = e < nx ? sx[e] : 0;
            s1[q] = e < nx ? sx[e + 1] : 0;
            pp[q] = e < nx ? partner[e] : 0;
        }
        uint64_t pos[SI];
        double v[SI], yv[SI];
        uint32_t c[SI];
#pragma unroll
        for (int q = 0; q < SI; ++q) {
            const uint64_t e = e0 + threadIdx.x + (uint64_t)q * OB;
            const bool kept = e < nx && s1[q] != s0[q];
            const uint64_t p = pp[q] & ~COLLIDE;
            pos[q] = kept ? s0[q] + sy[p] : 0;
            c[q] = kept ? xcols[e] : 0u;
            v[q] = kept ? xvals[e] : 0.0;
            yv[q] = (kept && X_IS_A && (pp[q] & COLLIDE)) ? yvals[p] : 0.0;
        }
#pragma unroll
        for (int q = 0; q < SI; ++q) {
            const uint64_t e = e0 + threadIdx.x + (uint64_t)q * OB;
            if (e >= nx || s1[q] == s0[q]) continue;  // dropped
            double val = v[q];
            if (X_IS_A && (pp[q] & COLLIDE)) val = __dadd_rn(val, yv[q]);
            ccols[pos[q]] = c[q];
            cvals[pos[q]] = val;
        }
    }
}

// scale: v * s or v / s into out (may alias vals); zero results counted per
// block into *zeros.
__global__ void scale_values(const double *vals, uint64_t n, double s, int divide,
                             double *out, unsigned long long *__restrict__ zeros) {
    unsigned long long z = 0;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const double v = divide ? __ddiv_rn(vals[i], s) : __dmul_rn(vals[i], s);
        out[i] = v;
        z += is_zero(v);
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) z += __shfl_xor_sync(0xffffffffu, z, o);
    __shared__ unsigned long long s_z[OB / 32];
    if ((threadIdx.x & 31) == 0) s_z[threadIdx.x >> 5] = z;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < OB / 32; ++w) z += s_z[w];
        if (z) atomicAdd(zeros, z);
    }
}

__global__ void nonzero_flags(const double *__restrict__ v, uint64_t n, uint64_t *__restrict__ keep) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        keep[i] = is_zero(v[i]) ? 0u : 1u;
}

__global__ void compact_offsets(const uint64_t *__restrict__ off, const uint64_t *__restrict__ sk, uint64_t n_rows,
                                uint64_t *__restrict__ out) {
    for (uint64_t r = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; r <= n_rows;
         r += (uint64_t)gridDim.x * blockDim.x)
        out[r] = sk[off[r]];
}

__global__ void compact_entries(const uint32_t *__restrict__ cols, const double *__restrict__ v, uint64_t n,
                                const uint64_t *__restrict__ sk, uint32_t *__restrict__ ocols,
                                double *__restrict__ ovals) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t p = sk[i];
        if (sk[i + 1] == p) continue;
        ocols[p] = cols[i];
        ovals[p] = v[i];
    }
}

// Row sums in CSR order: each sum is one left-to-right chain of __dadd_rn,
// as the CPU loop adds it, so a row is never split and a lane owns a row.
// A warp FP64 instruction costs the FP64 pipe the same whether one lane or
// 32 are active, so lanes must carry rows of similar length: rows of at most
// RS_SHORT entries are summed where they lie (thread per row), longer rows
// are bucketed by length (bucket b holds lengths in (32 << b, 64 << b]) and
// summed bucket by bucket, a lane per row, each loading RS_BATCH values
// ahead of its adds.
constexpr int RS_SHORT = 32, RS_BUCKETS = 10, RS_BATCH = 8;

__device__ __forceinline__ int rs_bucket(uint64_t len) {  // len > RS_SHORT
    const int b = 63 - __clzll((long long)(len - 1)) - 5;  // (32, 64] -> 0, (64, 128] -> 1, ...
    return b < RS_BUCKETS - 1 ? b : RS_BUCKETS - 1;
}

__device__ __forceinline__ double row_chain(const double *__restrict__ vals, uint64_t k, uint64_t e) {
    double acc = 0.0;
    for (; k + RS_BATCH <= e; k += RS_BATCH) {
        double v[RS_BATCH];
#pragma unroll
        for (int j = 0; j < RS_BATCH; ++j) v[j] = vals[k + j];
#pragma unroll
        for (int j = 0; j < RS_BATCH; ++j) acc = __dadd_rn(acc, v[j]);
    }
    for (; k < e; ++k) acc = __dadd_rn(acc, vals[k]);
    return acc;
}

// The same chain for long rows, software-pipelined: four batches of
// RS_BATCH values are in flight while one is added, so a lane's chain runs
// at the FP64 latency instead of waiting on memory every batch.
__device__ __forceinline__ void rs_load(double (&r)[RS_BATCH], const double *__restrict__ vals, uint64_t p,
                                        uint64_t e) {
#pragma unroll
    for (int j = 0; j < RS_BATCH; ++j) r[j] = p + j < e ? vals[p + j] : 0.0;
}

__device__ __forceinline__ void rs_add(double &acc, const double (&r)[RS_BATCH], uint64_t p, uint64_t e) {
#pragma unroll
    for (int j = 0; j < RS_BATCH; ++j)
        if (p + j < e) acc = __dadd_rn(acc, r[j]);
}

__device__ __forceinline__ double row_chain_long(const double *__restrict__ vals, uint64_t k, uint64_t e) {
    constexpr uint64_t B = RS_BATCH;
    double acc = 0.0, r0[RS_BATCH], r1[RS_BATCH], r2[RS_BATCH], r3[RS_BATCH];
    rs_load(r0, vals, k, e);
    rs_load(r1, vals, k + B, e);
    rs_load(r2, vals, k + 2 * B, e);
    rs_load(r3, vals, k + 3 * B, e);
    for (; k < e; k += 4 * B) {
        rs_add(acc, r0, k, e);
        rs_load(r0, vals, k + 4 * B, e);
        rs_add(acc, r1, k + B, e);
        rs_load(r1, vals, k + 5 * B, e);
        rs_add(acc, r2, k + 2 * B, e);
        rs_load(r2, vals, k + 6 * B, e);
        rs_add(acc, r3, k + 3 * B, e);
        rs_load(r3, vals, k + 7 * B, e);
    }
    return acc;
}

// Pass 1: short rows summed; long rows counted per bucket (fill == false)
// or placed in their bucket's list (fill == true; cursor[b] starts at the
// bucket's first slot).
template <bool FILL>
__global__ void __launch_bounds__(OB)
row_sums_split(const uint64_t *__restrict__ off, const double *__restrict__ vals, uint64_t n_rows,
               double *__restrict__ out, unsigned long long *__restrict__ cnt, uint32_t *__restrict__ list) {
    __shared__ unsigned s_cnt[RS_BUCKETS];
    if (!FILL) {
        for (int i = threadIdx.x; i < RS_BUCKETS; i += OB) s_cnt[i] = 0;
        __syncthreads();
    }
    for (uint64_t r = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; r < n_rows;
         r += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t b = off[r], e = off[r + 1];
        if (e - b <= RS_SHORT) {
            if (!FILL) out[r] = row_chain(vals, b, e);
        } else if (FILL) {
            list[atomicAdd(&cnt[rs_bucket(e - b)], 1ull)] = (uint32_t)r;
        } else {
            atomicAdd(&s_cnt[rs_bucket(e - b)], 1u);
        }
    }
    if (!FILL) {
        __syncthreads();
        for (int i = threadIdx.x; i < RS_BUCKETS; i += OB)
            if (s_cnt[i]) atomicAdd(&cnt[i], (unsigned long long)s_cnt[i]);
    }
}

// cnt[0..B) counts -> base[]: the buckets laid out longest first, base[b]
// = first slot of bucket b, base[B] = total; cnt becomes the fill cursors.
__global__ void row_sums_buckets(unsigned long long *__restrict__ cnt, unsigned long long *__restrict__ base) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        unsigned long long run = 0;
        for (int i = RS_BUCKETS - 1; i >= 0; --i) {
            base[i] = run;
            run += cnt[i];
            cnt[i] = base[i];
        }
        base[RS_BUCKETS] = run;
    }
}

// Pass 2: the long rows, longest first, a lane per row. A warp FP64
// instruction occupies its scheduler's FP64 unit for 64 cycles, so a row's
// chain advances one value per 64 cycles at best, and only if its warp is
// the sole FP64 user of that scheduler: the launch is one block of RS_LW
// warps per SM (a warp per scheduler), and list entry i goes to warp
// i % W, lane (i / W) % 32, so the heaviest rows land in different warps
// and each warp's lanes carry rows of falling length.
constexpr int RS_LW = 4;

__global__ void __launch_bounds__(RS_LW * 32)
row_sums_long(const uint64_t *__restrict__ off, const double *__restrict__ vals, const uint32_t *__restrict__ list,
              const unsigned long long *__restrict__ base, double *__restrict__ out) {
    const uint64_t W = (uint64_t)gridDim.x * RS_LW;
    const uint64_t w = blockIdx.x * (uint64_t)RS_LW + (threadIdx.x >> 5), lane = threadIdx.x & 31;
    const uint64_t total = base[RS_BUCKETS];
    for (uint64_t i = w + W * lane; i < total; i += W * 32) {
        const uint32_t r = list[i];
        out[r] = row_chain_long(vals, off[r], off[r + 1]);
    }
}

int row_sums_impl(Ctx *c, const uint64_t *off, const double *vals, uint64_t n_rows, uint64_t nnz, double *out,
                  cudaStream_t s) {
    const unsigned cap = (unsigned)c->n_sms * 16;
    const uint64_t max_long = nnz / (RS_SHORT + 1) + 1;
    DevBuf meta, list;
    SPG_TRY(meta.alloc((2 * RS_BUCKETS + 1) * sizeof(unsigned long long), s));
    SPG_TRY(list.alloc(max_long * sizeof(uint32_t), s));
    unsigned long long *cnt = meta.as<unsigned long long>(), *base = cnt + RS_BUCKETS;
    SPG_CUDA_TRY(cudaMemsetAsync(cnt, 0, RS_BUCKETS * sizeof(unsigned long long), s));
    row_sums_split<false><<<grid_for(n_rows, OB, cap), OB, 0, s>>>(off, vals, n_rows, out, cnt, nullptr);
    row_sums_buckets<<<1, 32, 0, s>>>(cnt, base);
    row_sums_split<true><<<grid_for(n_rows, OB, cap), OB, 0, s>>>(off, vals, n_rows, out, cnt, list.as<uint32_t>());
    row_sums_long<<<(unsigned)c->n_sms, RS_LW * 32, 0, s>>>(off, vals, list.as<uint32_t>(), base, out);
    SPG_LAUNCH_CHECK();
    return SPG_OK;
}

// Point lookups: found[i] = 1 and vals_out[i] = A(r, c) when stored; queries
// outside the shape or on absent entries give found 0 and 0.0.
__global__ void lookup_kernel(const uint64_t *__restrict__ off, const uint32_t *__restrict__ cols,
                              const double *__restrict__ vals, uint64_t n_rows, uint64_t n_cols, uint64_t n,
                              const uint64_t *__restrict__ qr, const uint32_t *__restrict__ qc,
                              double *__restrict__ vals_out, uint8_t *__restrict__ found) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t r = qr[i];
        const uint32_t c = qc[i];
        double v = 0.0;
        uint8_t f = 0;
        if (r < n_rows && (uint64_t)c < n_cols) {
            const uint64_t e = off[r + 1];
            const uint64_t p = lower_col(cols, off[r], e, c);
            if (p < e && cols[p] == c) {
                v = vals[p];
                f = 1;
            }
        }
        if (vals_out) vals_out[i] = v;
        if (found) found[i] = f;
    }
}

// bounds[t] for t in [1, T): the first row r with off[r] >= max(1, t * nnz / T)
// (lower_bound over off[0..n_rows], clamped to n_rows); uniform when nnz == 0.
__global__ void partition_kernel(const uint64_t *__restrict__ off, uint64_t n_rows, uint64_t T,
                                 uint64_t *__restrict__ bounds) {
    const uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (t > T) return;
    if (t == 0) {
        bounds[0] = 0;
        return;
    }
    if (t == T) {
        bounds[T] = n_rows;
        return;
    }
    const uint64_t total = off[n_rows];
    if (total == 0) {
        bounds[t] = t * n_rows / T;
        return;
    }
    uint64_t target = t * total / T;
    if (target < 1) target = 1;
    uint64_t lo = 0, hi = n_rows + 1;  // first index in [0, n_rows] with off >= target
    while (lo < hi) {
        const uint64_t mid = (lo + hi) >> 1;
        if (off[mid] < target) lo = mid + 1;
        else hi = mid;
    }
    bounds[t] = lo < n_rows ? lo : n_rows;
}

int read_word(Ctx *c, const uint64_t *d, cudaStream_t s, uint64_t *h) {
    SPG_CUDA_TRY(cudaMemcpyAsync(h, d, sizeof(uint64_t), cudaMemcpyDeviceToHost, s));
    return c->phase_sync(s);
}

// Installs (off, cols, vals, nnz) as the CSR of C; capacity defaults to nnz
// (tight, as a lock after an empty matrix builds it).
void install(Csr *C, uint64_t n_rows, uint64_t n_cols, DevBuf &off, DevBuf &cols, DevBuf &vals, uint64_t nnz,
             uint64_t capacity = ~0ull) {
    C->invalidate_derived();
    C->n_rows = n_rows;
    C->n_cols = n_cols;
    C->off = std::move(off);
    C->cols = std::move(cols);
    C->vals = std::move(vals);
    C->nnz = nnz;
    C->capacity = capacity == ~0ull ? nnz : capacity;
    C->built = true;
    C->may_have_zeros = false;
}

int add_impl(Ctx *c, const Csr *A, const Csr *B, Csr *Cm, cudaStream_t s) {
    const uint64_t n = A->n_rows, na = A->nnz, nb = B->nnz;
    const unsigned cap = (unsigned)c->n_sms * 16;
    DevBuf ka, kb, pa, pb, off, cols, vals;
    SPG_TRY(ka.alloc((na + 1) * sizeof(uint64_t), s));
    SPG_TRY(kb.alloc((nb + 1) * sizeof(uint64_t), s));
    SPG_TRY(pa.alloc(std::max<uint64_t>(na, 1) * sizeof(uint64_t), s));
    SPG_TRY(pb.alloc(std::max<uint64_t>(nb, 1) * sizeof(uint64_t), s));
    if (na)
        add_probe<true><<<grid_for(na, PT, cap), OB, 0, s>>>(A->d_off(), A->d_cols(), A->d_vals(), na, B->d_off(),
                                                             B->d_cols(), B->d_vals(), n, ka.as<uint64_t>(),
                                                             pa.as<uint64_t>());
    if (nb)
        add_probe<false><<<grid_for(nb, PT, cap), OB, 0, s>>>(B->d_off(), B->d_cols(), B->d_vals(), nb, A->d_off(),
                                                              A->d_cols(), A->d_vals(), n, kb.as<uint64_t>(),
                                                              pb.as<uint64_t>());
    SPG_LAUNCH_CHECK();
    if (na) SPG_TRY(exclusive_scan_u64(c, ka.as<uint64_t>(), na, ka.as<uint64_t>() + na, s));
    else SPG_CUDA_TRY(cudaMemsetAsync(ka.ptr, 0, sizeof(uint64_t), s));
    if (nb) SPG_TRY(exclusive_scan_u64(c, kb.as<uint64_t>(), nb, kb.as<uint64_t>() + nb, s));
    else SPG_CUDA_TRY(cudaMemsetAsync(kb.ptr, 0, sizeof(uint64_t), s));
    SPG_TRY(off.alloc(csr_off_elems(n) * sizeof(uint64_t), s));
    add_offsets<<<grid_for(n + 1, OB, cap), OB, 0, s>>>(A->d_off(), B->d_off(), ka.as<uint64_t>(), kb.as<uint64_t>(),
                                                        n, off.as<uint64_t>());
    SPG_LAUNCH_CHECK();
    uint64_t nnz = 0;
    SPG_TRY(read_word(c, off.as<uint64_t>() + n, s, &nnz));
    SPG_TRY(cols.alloc(csr_alloc_elems(nnz) * sizeof(uint32_t), s));
    SPG_TRY(vals.alloc(csr_alloc_elems(nnz) * sizeof(double), s));
    if (na)
        add_scatter<true><<<grid_for(na, OB * 4, cap), OB, 0, s>>>(A->d_cols(), A->d_vals(), na, B->d_vals(),
                                                               ka.as<uint64_t>(), kb.as<uint64_t>(), pa.as<uint64_t>(),
                                                               cols.as<uint32_t>(), vals.as<double>());
    if (nb)
        add_scatter<false><<<grid_for(nb, OB * 4, cap), OB, 0, s>>>(B->d_cols(), B->d_vals(), nb, A->d_vals(),
                                                                kb.as<uint64_t>(), ka.as<uint64_t>(),
                                                                pb.as<uint64_t>(), cols.as<uint32_t>(),
                                                                vals.as<double>());
    SPG_LAUNCH_CHECK();
    SPG_TRY(c->phase_sync(s));
    install(Cm, n, A->n_cols, off, cols, vals, nnz);
    return SPG_OK;
}

// In place, Spira stages every committed entry's scaled value and the next
// lock merges them: a merge of |D| = nnz unique entries, so the capacity
// follows the merge rule (csr_build.hpp:139-145): kept while old nnz + |D|
// fits, else 1.5 x (old nnz + |D|).
int scale_impl(Ctx *c, Csr *A, Csr *Cm, double sc, int divide, cudaStream_t s) {
    const uint64_t n = A->n_rows, m = A->nnz;
    const unsigned cap = (unsigned)c->n_sms * 16;
    const bool in_place = A == Cm;
    uint64_t out_cap = m;  // copy path: a fresh matrix locked once, tight
    if (in_place) {
        const uint64_t ub = 2 * m;
        out_cap = ub <= A->capacity ? A->capacity : ub + ub / 2;
    }
    const bool same_arrays = in_place && out_cap == A->capacity;  // values rewritten where they are
    DevBuf zc, off, cols, vals;
    SPG_TRY(zc.alloc(sizeof(unsigned long long), s));
    SPG_CUDA_TRY(cudaMemsetAsync(zc.ptr, 0, sizeof(unsigned long long), s));
    double *out = nullptr;
    if (same_arrays) {
        out = A->vals.as<double>();
    } else {
        SPG_TRY(vals.alloc(csr_alloc_elems(out_cap) * sizeof(double), s));
        out = vals.as<double>();
    }
    if (m)
        scale_values<<<grid_for(m, OB, cap), OB, 0, s>>>(A->d_vals(), m, sc, divide, out,
                                                         zc.as<unsigned long long>());
    SPG_LAUNCH_CHECK();
    uint64_t zeros = 0;
    SPG_TRY(read_word(c, zc.as<uint64_t>(), s, &zeros));
    if (zeros == 0) {
        if (same_arrays) {
            A->invalidate_derived();  // cached plans hold copies of the values
            return SPG_OK;
        }
        SPG_TRY(off.alloc(csr_off_elems(n) * sizeof(uint64_t), s));
        SPG_TRY(cols.alloc(csr_alloc_elems(out_cap) * sizeof(uint32_t), s));
        SPG_CUDA_TRY(cudaMemcpyAsync(off.ptr, A->d_off(), (n + 1) * sizeof(uint64_t), cudaMemcpyDeviceToDevice, s));
        if (m)
            SPG_CUDA_TRY(cudaMemcpyAsync(cols.ptr, A->d_cols(), m * sizeof(uint32_t), cudaMemcpyDeviceToDevice, s));
        SPG_TRY(c->phase_sync(s));
        install(Cm, n, A->n_cols, off, cols, vals, m, out_cap);
        return SPG_OK;
    }
    // some results are +-0: compact them away (the lock after the scaled
    // inserts deletes those entries)
    const double *scaled = out;
    DevBuf keep, ncols, nvals;
    SPG_TRY(keep.alloc((m + 1) * sizeof(uint64_t), s));
    nonzero_flags<<<grid_for(m, OB, cap), OB, 0, s>>>(scaled, m, keep.as<uint64_t>());
    SPG_LAUNCH_CHECK();
    SPG_TRY(exclusive_scan_u64(c, keep.as<uint64_t>(), m, keep.as<uint64_t>() + m, s));
    const uint64_t nnz = m - zeros;
    if (!in_place) out_cap = nnz;
    SPG_TRY(off.alloc(csr_off_elems(n) * sizeof(uint64_t), s));
    SPG_TRY(ncols.alloc(csr_alloc_elems(out_cap) * sizeof(uint32_t), s));
    SPG_TRY(nvals.alloc(csr_alloc_elems(out_cap) * sizeof(double), s));
    compact_offsets<<<grid_for(n + 1, OB, cap), OB, 0, s>>>(A->d_off(), keep.as<uint64_t>(), n, off.as<uint64_t>());
    compact_entries<<<grid_for(m, OB, cap), OB, 0, s>>>(A->d_cols(), scaled, m, keep.as<uint64_t>(),
                                                        ncols.as<uint32_t>(), nvals.as<double>());
    SPG_LAUNCH_CHECK();
    SPG_TRY(c->phase_sync(s));
    install(Cm, n, A->n_cols, off, ncols, nvals, nnz, out_cap);
    return SPG_OK;
}

}  // namespace
}  // namespace spg

using namespace spg;

extern "C" {

int spg_csr_add(spg_ctx *c, const spg_csr *A, const spg_csr *B, spg_csr *Cm) {
    if (!c || !A || !B || !Cm) return set_error(SPG_ERR_INVALID_ARGUMENT, "spg_csr_add: null handle");
    SPG_CHECK_LIVE(A);
    SPG_CHECK_LIVE(B);
    SPG_CHECK_LIVE(Cm);
    // checks in the order of serial/matrix_addition.hpp:89-97
    if (A->n_rows != B->n_rows || A->n_cols != B->n_cols)
        return set_error(SPG_ERR_INVALID_ARGUMENT, "Matrices aren't the same size");
    if (!A->built) return set_error(SPG_ERR_LOGIC, "MatrixAddition: A must be locked");
    if (!B->built) return set_error(SPG_ERR_LOGIC, "MatrixAddition: B must be locked");
    if (Cm == A || Cm == B) return set_error(SPG_ERR_INVALID_ARGUMENT, "spg_csr_add: output aliases an input");
    SPG_CUDA_TRY(cudaSetDevice(c->device));
    return add_impl(c, A, B, Cm, c->stream);
}

int spg_csr_scale(spg_ctx *c, spg_csr *A, spg_csr *Cm, double scalar, int divide) {
    if (!c || !A || !Cm) return set_error(SPG_ERR_INVALID_ARGUMENT, "spg_csr_scale: null handle");
    SPG_CHECK_LIVE(A);
    SPG_CHECK_LIVE(Cm);
    // serial/scalars.hpp:39-41, 54-56: the zero check comes first
    if (divide && fabs(scalar) <= 0.0) return set_error(SPG_ERR_DOMAIN, "Divison by zero");
    if (!A->built)
        return set_error(SPG_ERR_LOGIC, divide ? "division_scaler: input matrix must be locked"
                                               : "multiplication_scaler: input matrix must be locked");
    SPG_CUDA_TRY(cudaSetDevice(c->device));
    return scale_impl(c, A, Cm, scalar, divide, c->stream);
}

int spg_csr_row_sums(spg_ctx *c, const spg_csr *A, double *d_out, void *stream) {
    if (!c || !A || (!d_out && A->n_rows)) return set_error(SPG_ERR_INVALID_ARGUMENT, "spg_csr_row_sums: null argument");
    SPG_CHECK_LIVE(A);
    if (!A->built) return set_error(SPG_ERR_LOGIC, "spg_csr_row_sums: matrix must be locked");
    if (!A->n_rows) return SPG_OK;
    SPG_CUDA_TRY(cudaSetDevice(c->device));
    return row_sums_impl(c, A->d_off(), A->d_vals(), A->n_rows, A->nnz, d_out, pick_stream(c, stream));
}

int spg_csr_row_sums_host(spg_ctx *c, const spg_csr *A, uint64_t row0, uint64_t n, double *out) {
    if (!c || !A || (n && !out)) return set_error(SPG_ERR_INVALID_ARGUMENT, "spg_csr_row_sums_host: null argument");
    SPG_CHECK_LIVE(A);
    if (row0 > A->n_rows || n > A->n_rows - row0)
        return set_error(SPG_ERR_OUT_OF_RANGE, "Row does not exist in matrix");
    if (!A->built) return set_error(SPG_ERR_LOGIC, "spg_csr_row_sums_host: matrix must be locked");
    if (!n) return SPG_OK;
    SPG_CUDA_TRY(cudaSetDevice(c->device));
    cudaStream_t s = c->stream;
    DevBuf d;
    SPG_TRY(d.alloc(n * sizeof(double), s));
    SPG_TRY(row_sums_impl(c, A->d_off() + row0, A->d_vals(), n, A->nnz, d.as<double>(), s));
    SPG_CUDA_TRY(cudaMemcpyAsync(out, d.ptr, n * sizeof(double), cudaMemcpyDeviceToHost, s));
    SPG_CUDA_TRY(cudaStreamSynchronize(s));
    return SPG_OK;
}

int spg_csr_lookup(spg_ctx *c, const spg_csr *A, uint64_t n, const uint64_t *d_rows, const uint32_t *d_cols,
                   double *d_vals, uint8_t *d_found, void *stream) {
    if (!c || !A || (n && (!d_rows || !d_cols || (!d_vals && !d_found))))
        return set_error(SPG_ERR_INVALID_ARGUMENT, "spg_csr_lookup: null argument");
    SPG_CHECK_LIVE(A);
    if (!n) return SPG_OK;
    SPG_CUDA_TRY(cudaSetDevice(c->device));
    cudaStream_t s = pick_stream(c, stream);
    if (!A->built) {  // nothing committed: every query misses
        if (d_vals) SPG_CUDA_TRY(cudaMemsetAsync(d_vals, 0, n * sizeof(double), s));
        if (d_found) SPG_CUDA_TRY(cudaMemsetAsync(d_found, 0, n, s));
        return SPG_OK;
    }
    lookup_kernel<<<grid_for(n, OB, (unsigned)c->n_sms * 16), OB, 0, s>>>(
        A->d_off(), A->d_cols(), A->d_vals(), A->n_rows, A->n_cols, n, d_rows, d_cols, d_vals, d_found);
    SPG_LAUNCH_CHECK();
    return SPG_OK;
}

int spg_csr_partition(spg_ctx *c, const spg_csr *A, uint64_t n_parts, uint64_t *bounds) {
    if (!c || !A || !bounds || n_parts == 0)
        return set_error(SPG_ERR_INVALID_ARGUMENT, "spg_csr_partition: null argument or zero parts");
    SPG_CHECK_LIVE(A);
    const uint64_t n = A->n_rows;
    // partition.hpp:84-88: {0, n, n, ...} for one part or no rows
    if (n_parts == 1 || n == 0 || !A->built) {
        if (!A->built && n_parts > 1 && n) {  // nothing committed: nnz == 0, uniform split
            for (uint64_t t = 0; t <= n_parts; ++t) bounds[t] = t * n / n_parts;
            return SPG_OK;
        }
        bounds[0] = 0;
        for (uint64_t t = 1; t <= n_parts; ++t) bounds[t] = n;
        return SPG_OK;
    }
    SPG_CUDA_TRY(cudaSetDevice(c->device));
    cudaStream_t s = c->stream;
    DevBuf d;
    SPG_TRY(d.alloc((n_parts + 1) * sizeof(uint64_t), s));
    partition_kernel<<<grid_for(n_parts + 1, OB), OB, 0, s>>>(A->d_off(), n, n_parts, d.as<uint64_t>());
    SPG_LAUNCH_CHECK();
    SPG_CUDA_TRY(cudaMemcpyAsync(bounds, d.ptr, (n_parts + 1) * sizeof(uint64_t), cudaMemcpyDeviceToHost, s));
    SPG_CUDA_TRY(cudaStreamSynchronize(s));
    return SPG_OK;
}

}  // extern "C"
