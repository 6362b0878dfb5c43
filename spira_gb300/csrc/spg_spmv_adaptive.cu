// spg_spmv_adaptive.cu — SPG_SPMV_ADAPTIVE(16), the FP64 SpMV shaped for GB300.
//
// GB300 executes FP64 at 2 fused multiply-adds per clock per SM (ncu:
// sm__sass_thread_inst_executed_op_dfma_pred_on.peak_sustained = 2), so at
// ~12 B/nnz the FP64 pipe and HBM finish a SpMV in about the same time: any
// FP64 instruction beyond one FMA per nonzero, and any FP64 lane left idle by
// divergence, shows up in the runtime. This variant spends one DFMA lane per
// nonzero and keeps HBM busy with bulk asynchronous copies:
//
//  * short rows (<= AD_LONG nnz) are cut into row-aligned tiles of at most
//    AD_BLOCK * ITEMS - 17 nnz and <= AD_ROWCAP rows. A persistent CTA walks
//    its tiles (tile = blockIdx.x + i * gridDim.x) through an NSTAGE-deep
//    ring in shared memory: one thread issues cp.async.bulk copies of the
//    tile's vals, cols and row offsets (16-byte aligned windows; the CSR
//    arrays carry padding so the windows never leave their allocations) and
//    an mbarrier completes when the bytes land, NSTAGE - 1 tiles ahead of the
//    tile being computed. Thread t owns the ITEMS consecutive nonzeros
//    [a0 + ITEMS t, a0 + ITEMS (t+1)) of the 16-aligned window, issues its x
//    gathers, then runs one FMA chain across them, closing a row whenever the
//    row's end offset is passed. A row straddling threads is finished by the
//    thread that ends it, adding the straddled threads' tail partials in
//    thread order (rows are <= AD_LONG, so few pieces);
//  * long rows (> AD_LONG nnz) get one warp each: lane-strided 16-byte loads,
//    four pairs in flight per lane, one FMA per nonzero, 5 shuffle additions.
// Both paths are deterministic. Every mbarrier wait is bounded: on timeout the
// CTA sets bit 0 of the context status word, waits (bounded) for its copies
// in flight and returns. The tile and long-row lists form the plan, built on
// the device once per lock and cached on the matrix.
#include "spg_internal.cuh"

namespace spg {
namespace {

constexpr int AD_BLOCK = 256;
constexpr uint64_t AD_LONG = 128;
constexpr int AD_ROWCAP = 1024;
constexpr uint32_t AD_WAIT_LIMIT = 1u << 22;

struct TileDesc {
    uint32_t r0, r1;
    uint64_t k0, k1;
};

template <int ITEMS>
struct AdGeom {
    static constexpr int T = AD_BLOCK * ITEMS;                   // nonzeros per window
    static constexpr uint64_t BIN = (uint64_t)T - 16 - AD_LONG;  // tile nnz <= BIN - 1 + AD_LONG
    static constexpr size_t VAL_B = (size_t)T * 8;
    static constexpr size_t COL_B = (size_t)T * 4;
    static constexpr size_t OFF_B = (((size_t)AD_ROWCAP + 2) * 8 + 127) & ~(size_t)127;
    static constexpr size_t STAGE_B = VAL_B + COL_B + OFF_B;
};

__device__ __forceinline__ double ldx(const double *__restrict__ x, uint32_t c) { return __ldg(x + c); }

// ---------------------------------------------------------------- PTX wrappers
__device__ __forceinline__ uint32_t smem_addr(const void *p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_init_fence() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, uint32_t parity) {
    for (uint32_t i = 0; i < AD_WAIT_LIMIT; ++i)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}
// Orders this thread's earlier generic-proxy accesses to shared memory before
// later async-proxy (bulk copy) writes to it.
__device__ __forceinline__ void fence_proxy_async() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_addr(dst)),
        "l"(src), "r"(bytes), "r"(smem_addr(bar))
        : "memory");
}

// ---------------------------------------------------------------- plan
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

__global__ void ad_tile_flags(const uint32_t *__restrict__ B, const uint64_t *__restrict__ lpos, uint64_t nb,
                              uint64_t *__restrict__ tflag) {
    const uint64_t j = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= nb) return;
    const uint32_t r = B[j];
    tflag[j] = (lpos[r + 1] == lpos[r]) ? 1 : 0;
}

__global__ void ad_tile_scatter(const uint32_t *__restrict__ B, const uint64_t *__restrict__ tpos,
                                const uint64_t *__restrict__ off, uint64_t nb, TileDesc *__restrict__ tiles) {
    const uint64_t j = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= nb) return;
    if (tpos[j + 1] != tpos[j]) {
        TileDesc d;
        d.r0 = B[j];
        d.r1 = B[j + 1];
        d.k0 = off[d.r0];
        d.k1 = off[d.r1];
        tiles[tpos[j]] = d;
    }
}

// ---------------------------------------------------------------- short-row tiles
template <int ITEMS, int NSTAGE>
__global__ void __launch_bounds__(AD_BLOCK)
spmv_ad_tiles(const uint64_t *__restrict__ off, const uint32_t *__restrict__ cols, const double *__restrict__ vals,
              const double *__restrict__ x, double *__restrict__ y, const TileDesc *__restrict__ tiles,
              uint32_t n_tiles, unsigned *__restrict__ status) {
    using Gm = AdGeom<ITEMS>;
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ __align__(8) uint64_t bars[NSTAGE];
    __shared__ double s_tail[AD_BLOCK];
    __shared__ uint32_t s_tail_row[AD_BLOCK];
    __shared__ int s_abort;
    const uint32_t tid = threadIdx.x;
    const uint32_t G = gridDim.x;

    // thread 0's bookkeeping of stages with copies in flight
    uint32_t pending = 0, issued_parity = 0;
    auto issue = [&](uint32_t tile, int s) {
        const TileDesc d = tiles[tile];
        const uint64_t a0 = d.k0 & ~15ull;
        const uint32_t span = (uint32_t)(((d.k1 + 15) & ~15ull) - a0);
        const uint32_t ro = d.r0 & ~1u;
        const uint32_t nro = ((d.r1 + 1 - ro) + 1) & ~1u;
        unsigned char *st = smem + (size_t)s * Gm::STAGE_B;
        mbar_expect_tx(&bars[s], span * 12u + nro * 8u);
        if (span) {
            bulk_g2s(st, vals + a0, span * 8u, &bars[s]);
            bulk_g2s(st + Gm::VAL_B, cols + a0, span * 4u, &bars[s]);
        }
        bulk_g2s(st + Gm::VAL_B + Gm::COL_B, off + ro, nro * 8u, &bars[s]);
        pending |= 1u << s;
        issued_parity ^= 1u << s;
    };

    if (tid == 0) {
        for (int s = 0; s < NSTAGE; ++s) mbar_init(&bars[s], 1);
        mbar_init_fence();
        s_abort = 0;
    }
    __syncthreads();
    if (tid == 0)
        for (int s = 0; s < NSTAGE; ++s) {
            const uint32_t t = blockIdx.x + (uint32_t)s * G;
            if (t < n_tiles) issue(t, s);
        }

    for (uint32_t it = 0;; ++it) {
        const uint32_t tile = blockIdx.x + it * G;
        if (tile >= n_tiles) break;
        const int s = (int)(it % NSTAGE);
        const uint32_t par = (it / NSTAGE) & 1u;
        if (!mbar_wait_bounded(&bars[s], par)) s_abort = 1;
        __syncthreads();
        if (s_abort) break;
        if (tid == 0) pending &= ~(1u << s);

        const TileDesc d = tiles[tile];
        const unsigned char *st = smem + (size_t)s * Gm::STAGE_B;
        const double *sv = reinterpret_cast<const double *>(st);
        const uint32_t *sc = reinterpret_cast<const uint32_t *>(st + Gm::VAL_B);
        const uint64_t *so = reinterpret_cast<const uint64_t *>(st + Gm::VAL_B + Gm::COL_B) + (d.r0 & 1u);
        // so[i] = off[r0 + i]; row i of the tile ends at so[i + 1] - k0
        const uint32_t nr = d.r1 - d.r0;
        const uint64_t k0 = d.k0, k1 = d.k1;
        const uint64_t a0 = k0 & ~15ull;
        const uint64_t ca = a0 + (uint64_t)ITEMS * tid;
        const uint64_t lo = ca > k0 ? ca : k0;
        const uint64_t hi = (ca + ITEMS < k1) ? ca + ITEMS : k1;
        const bool has_items = lo < hi;
        double acc = 0.0, head_val = 0.0;
        uint32_t row = 0, head_row = 0xFFFFFFFFu;
        if (k1 == k0) {
            for (uint32_t i = tid; i < nr; i += AD_BLOCK) y[d.r0 + i] = 0.0;
        } else if (has_items) {
            const uint32_t plo = (uint32_t)(lo - k0), phi = (uint32_t)(hi - k0);
            bool head = false;
            if (plo > 0) {
                uint32_t l = 0, h = nr - 1;  // smallest row with end > plo
                while (l < h) {
                    const uint32_t m = (l + h) >> 1;
                    if ((uint32_t)(so[m + 1] - k0) > plo) h = m;
                    else l = m + 1;
                }
                row = l;
                head = (uint32_t)(so[row] - k0) < plo;
            }
            const uint32_t base = (uint32_t)(ca - a0);
            double g[ITEMS], v[ITEMS];
#pragma unroll
            for (int u = 0; u < ITEMS; ++u) {
                const uint64_t itm = ca + u;
                g[u] = 0.0;
                v[u] = sv[base + u];
                if (itm >= lo && itm < hi) g[u] = ldx(x, sc[base + u]);  // only in-tile columns are read
            }
            const uint32_t rfirst = row;
            uint32_t rend = (uint32_t)(so[row + 1] - k0);
#pragma unroll
            for (int u = 0; u < ITEMS; ++u) {
                const uint64_t itm = ca + u;
                if (itm < lo || itm >= hi) continue;
                const uint32_t p = (uint32_t)(itm - k0);
                while (rend <= p) {  // row closes before item p
                    if (head && row == rfirst) {
                        head_val = acc;
                        head_row = row;
                    } else {
                        y[d.r0 + row] = acc;
                    }
                    acc = 0.0;
                    ++row;
                    rend = (uint32_t)(so[row + 1] - k0);
                }
                acc = fma(g[u], v[u], acc);
            }
            while (row < nr && rend <= phi) {  // rows ending at the chunk end, empty rows there
                if (head && row == rfirst) {
                    head_val = acc;
                    head_row = row;
                } else {
                    y[d.r0 + row] = acc;
                }
                acc = 0.0;
                ++row;
                if (row < nr) rend = (uint32_t)(so[row + 1] - k0);
            }
        }
        s_tail[tid] = acc;
        s_tail_row[tid] = (has_items && k1 != k0 && row < nr) ? row : 0xFFFFFFFFu;
        __syncthreads();
        if (head_row != 0xFFFFFFFFu) {
            int j = (int)tid - 1;
            while (j >= 0 && s_tail_row[j] == head_row) --j;
            double sum = 0.0;
            for (int q = j + 1; q < (int)tid; ++q) sum += s_tail[q];
            y[d.r0 + head_row] = sum + head_val;
        }
        __syncthreads();  // stage s and the tail arrays are free again
        if (tid == 0) {
            const uint32_t next = tile + (uint32_t)NSTAGE * G;
            if (next < n_tiles) {
                fence_proxy_async();
                issue(next, s);
            }
        }
    }
    if (tid == 0 && s_abort) {
        atomicOr(status, 1u);
        // wait (bounded) for the copies still in flight before leaving
        for (int s = 0; s < NSTAGE; ++s)
            if (pending & (1u << s)) mbar_wait_bounded(&bars[s], ((issued_parity >> s) & 1u) ^ 1u);
    }
}

// ---------------------------------------------------------------- long rows
__global__ void __launch_bounds__(AD_BLOCK)
spmv_ad_long(const uint64_t *__restrict__ off, const uint32_t *__restrict__ cols, const double *__restrict__ vals,
             const double *__restrict__ x, double *__restrict__ y, const uint32_t *__restrict__ rows,
             uint64_t n_long) {
    const uint64_t w = ((uint64_t)blockIdx.x * AD_BLOCK + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (w >= n_long) return;
    const uint32_t r = rows[w];
    const uint64_t b = off[r], e = off[r + 1];
    // lane-strided 16-byte pairs over the even-aligned interior; scalar head / tail
    double acc = 0.0, acc1 = 0.0;
    const uint64_t a = (b + 1) & ~1ull;
    const uint64_t ae = e & ~1ull;
    if (b < a && lane == 0) acc = fma(ldx(x, cols[b]), vals[b], acc);
    uint64_t i = a + 2ull * lane;
    for (; i + 6ull * 32 < ae; i += 8ull * 32) {
        double2 v[4];
        uint2 c[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            v[u] = *reinterpret_cast<const double2 *>(vals + i + 64ull * u);
            c[u] = *reinterpret_cast<const uint2 *>(cols + i + 64ull * u);
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
    for (; i < ae; i += 64ull) {
        const double2 v = *reinterpret_cast<const double2 *>(vals + i);
        const uint2 c = *reinterpret_cast<const uint2 *>(cols + i);
        acc = fma(ldx(x, c.x), v.x, acc);
        acc1 = fma(ldx(x, c.y), v.y, acc1);
    }
    if (ae < e && ae >= a && lane == 31) acc = fma(ldx(x, cols[ae]), vals[ae], acc);
    acc += acc1;
#pragma unroll
    for (int o = 16; o; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) y[r] = acc;
}

template <int ITEMS, int NSTAGE>
int launch_tiles(Ctx *c, Csr *A, const double *x, double *y, cudaStream_t s) {
    using Gm = AdGeom<ITEMS>;
    static bool attr_set[64] = {};
    const size_t dyn = (size_t)NSTAGE * Gm::STAGE_B;
    auto kern = spmv_ad_tiles<ITEMS, NSTAGE>;
    if (!attr_set[c->device & 63]) {
        SPG_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn));
        attr_set[c->device & 63] = true;
    }
    int per_sm = 0;
    SPG_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, AD_BLOCK, dyn));
    if (per_sm < 1) per_sm = 1;
    const uint64_t nt = A->plan_adaptive.n_items;
    const uint64_t g = std::min<uint64_t>(nt, (uint64_t)per_sm * c->n_sms);
    kern<<<(unsigned)g, AD_BLOCK, dyn, s>>>(A->d_off(), A->d_cols(), A->d_vals(), x, y,
                                            A->plan_adaptive.items.as<TileDesc>(), (uint32_t)nt, c->d_status);
    SPG_LAUNCH_CHECK();
    return SPG_OK;
}

}  // namespace

int build_adaptive_plan(Ctx *c, Csr *A, int items, cudaStream_t s) {
    if (A->plan_adaptive.kind == SPG_SPMV_ADAPTIVE * 100 + items) return SPG_OK;
    const uint64_t n = A->n_rows;
    const uint64_t bin = (items == 8) ? AdGeom<8>::BIN : AdGeom<16>::BIN;
    DevBuf brk, lng, B;
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
    if (nt >= (1ull << 32)) return set_error(SPG_ERR_UNSUPPORTED, "adaptive plan: too many tiles");
    SPG_TRY(p.items.alloc((nt ? nt : 1) * sizeof(TileDesc), s));
    ad_tile_scatter<<<grid_for(nb, 256), 256, 0, s>>>(B.as<uint32_t>(), tpos.as<uint64_t>(), A->d_off(), nb,
                                                      p.items.as<TileDesc>());
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
    if (nt) {
        if (items == 8) SPG_TRY((launch_tiles<8, 3>(c, A, x, y, s)));
        else SPG_TRY((launch_tiles<16, 2>(c, A, x, y, s)));
    }
    if (nl) {
        spmv_ad_long<<<grid_for(nl * 32, AD_BLOCK), AD_BLOCK, 0, s>>>(A->d_off(), A->d_cols(), A->d_vals(), x, y,
                                                                     A->plan_adaptive.aux.as<uint32_t>(), nl);
        SPG_LAUNCH_CHECK();
    }
    return SPG_OK;
}

}  // namespace spg
