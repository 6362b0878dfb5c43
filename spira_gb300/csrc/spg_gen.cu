// spg_gen.cu — seeded synthetic draws on the device (include/spg_gen.h).
// Bit-identical to spira_gb300/gen.py: same splitmix64 finaliser, same
// stream keying, same integer / double conversions.
#include "../../include/spg_gen.h"
#include "spg_internal.cuh"

namespace spg {
namespace {

__host__ __device__ __forceinline__ uint64_t splitmix64(uint64_t x) {
    uint64_t z = x + 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

__global__ void gen_draw_kernel(uint64_t key, uint64_t c0, uint64_t n, int kind, uint64_t bound, void *out) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t h = splitmix64((c0 + i) ^ key);
        if (kind == SPG_GEN_BELOW_U32) {
            static_cast<uint32_t *>(out)[i] = (uint32_t)(((h >> 32) * bound) >> 32);
        } else {
            const double u = (double)(h >> 11) * 0x1.0p-53;
            static_cast<double *>(out)[i] = (kind == SPG_GEN_SYM_F64) ? 2.0 * u - 1.0 : u;
        }
    }
}

__global__ void expand_rows_kernel(const uint64_t *__restrict__ start, uint64_t n_rows, uint32_t *__restrict__ rows) {
    // one warp per row: rows are written with coalesced stores
    const uint64_t w = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (w >= n_rows) return;
    const uint64_t b = start[w], e = start[w + 1];
    for (uint64_t k = b + lane; k < e; k += 32) rows[k] = (uint32_t)w;
}

__device__ __forceinline__ uint64_t fam_key(uint64_t seed, uint64_t stream) {
    return splitmix64(seed * 0xD1B54A32D192ED03ull + stream);
}

__device__ __forceinline__ double fam_unit(uint64_t key, uint64_t k) {
    return (double)(splitmix64(k ^ key) >> 11) * 0x1.0p-53;
}

// Row length of row r for the family (also the number of stencil neighbours).
__device__ uint64_t fam_length(int fam, uint64_t r, uint64_t n, uint64_t p, double ls, const double *cdf,
                               uint64_t seed) {
    switch (fam) {
        case SPG_FAM_BANDED: {
            const uint64_t h = p / 2;
            const uint64_t lo = r > h ? r - h : 0, hi = min(n - 1, r + h);
            return hi - lo + 1;
        }
        case SPG_FAM_BLOCKDIAG: {
            const uint64_t b0 = (r / p) * p;
            return min(p, n - b0);
        }
        case SPG_FAM_POWERLAW: {
            const double u = fam_unit(fam_key(seed, 3), r);
            uint64_t lo = 0, hi = p;  // first index with cdf > u
            while (lo < hi) {
                const uint64_t mid = (lo + hi) >> 1;
                if (cdf[mid] > u) hi = mid;
                else lo = mid + 1;
            }
            const double z = (double)min(lo + 1, p);
            const double L = rint(z * ls);
            return (uint64_t)fmin((double)p, fmax(1.0, L));
        }
        case SPG_FAM_UNIFORM:
            return p;
        case SPG_FAM_STENCIL2D: {
            const uint64_t x = r % p, y = r / p;
            return 1 + (x > 0) + (x + 1 < p) + (y > 0) + (y + 1 < p);
        }
        case SPG_FAM_STENCIL3D: {
            const uint64_t x = r % p, y = (r / p) % p, z = r / (p * p);
            return 1 + (x > 0) + (x + 1 < p) + (y > 0) + (y + 1 < p) + (z > 0) + (z + 1 < p);
        }
        default: {  // Poisson(ls) by inversion of the CDF
            const double u = fam_unit(fam_key(seed, 3), r);
            double pk = exp(-ls), cum = pk;
            uint64_t k = 0;
            while (u > cum && k < 1024) {
                ++k;
                pk *= ls / (double)k;
                cum += pk;
            }
            return k;
        }
    }
}

__global__ void fam_lengths_kernel(int fam, uint64_t n, uint64_t p, double ls, const double *cdf, uint64_t seed,
                                   uint64_t *len) {
    for (uint64_t r = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; r < n; r += (uint64_t)gridDim.x * blockDim.x)
        len[r] = fam_length(fam, r, n, p, ls, cdf, seed);
}

// warp per row: entry j of row r at start[r] + j
__global__ void fam_fill_kernel(int fam, uint64_t n, uint64_t p, uint64_t seed, const uint64_t *__restrict__ start,
                                uint32_t *__restrict__ rows, uint32_t *__restrict__ cols, double *__restrict__ vals) {
    const uint64_t r = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (r >= n) return;
    const uint64_t b = start[r], e = start[r + 1];
    const uint64_t kc = fam_key(seed, 4), kv = fam_key(seed, 5);
    for (uint64_t k = b + lane; k < e; k += 32) {
        const uint64_t j = k - b;
        uint64_t c = 0;
        double v = 2.0 * fam_unit(kv, k) - 1.0;
        if (fam == SPG_FAM_BANDED) {
            const uint64_t h = p / 2;
            c = (r > h ? r - h : 0) + j;
        } else if (fam == SPG_FAM_BLOCKDIAG) {
            c = (r / p) * p + j;
        } else if (fam == SPG_FAM_STENCIL2D || fam == SPG_FAM_STENCIL3D) {
            // neighbours in ascending column order; the j-th valid one
            const bool is3 = fam == SPG_FAM_STENCIL3D;
            const uint64_t x = r % p, y = (r / p) % p, z = is3 ? r / (p * p) : 0;
            const uint64_t gg = p * p;
            uint64_t cand[7];
            int nc = 0;
            if (is3 && z > 0) cand[nc++] = r - gg;
            if (y > 0) cand[nc++] = r - p;
            if (x > 0) cand[nc++] = r - 1;
            cand[nc++] = r;
            if (x + 1 < p) cand[nc++] = r + 1;
            if (y + 1 < p) cand[nc++] = r + p;
            if (is3 && z + 1 < p) cand[nc++] = r + gg;
            c = cand[j < (uint64_t)nc ? j : 0];
            v = (c == r) ? (double)(nc - 1) : -1.0;
        } else {
            c = (uint64_t)(((splitmix64(k ^ kc) >> 32) * n) >> 32);
        }
        rows[k] = (uint32_t)r;
        cols[k] = (uint32_t)c;
        vals[k] = v;
    }
}

__global__ void copy_i64_to_u64(const int64_t *in, uint64_t *out, uint64_t n) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x)
        out[i] = in[i] > 0 ? (uint64_t)in[i] : 0;
}

}  // namespace
}  // namespace spg

using namespace spg;

extern "C" {

int spg_gen_draw(spg_ctx *c, uint64_t seed, uint64_t stream, uint64_t counter0, uint64_t n, int kind, uint64_t bound,
                 void *d_out) {
    if (!c || (n && !d_out)) return set_error(SPG_ERR_INVALID_ARGUMENT, "spg_gen_draw: null argument");
    if (kind < 0 || kind > 2) return set_error(SPG_ERR_INVALID_ARGUMENT, "spg_gen_draw: unknown kind %d", kind);
    if (kind == SPG_GEN_BELOW_U32 && (bound == 0 || bound > 0xFFFFFFFFull + 1))
        return set_error(SPG_ERR_INVALID_ARGUMENT, "spg_gen_draw: bound must be in [1, 2^32]");
    if (!n) return SPG_OK;
    SPG_CUDA_TRY(cudaSetDevice(c->device));
    const uint64_t key = splitmix64(seed * 0xD1B54A32D192ED03ull + stream);
    gen_draw_kernel<<<grid_for(n, 256, (unsigned)c->n_sms * 32), 256, 0, c->stream>>>(key, counter0, n, kind, bound,
                                                                                      d_out);
    SPG_LAUNCH_CHECK();
    return SPG_OK;
}

int spg_gen_expand_rows(spg_ctx *c, const int64_t *d_lengths, uint64_t n_rows, uint32_t *d_rows, uint64_t *total) {
    if (!c || !total) return set_error(SPG_ERR_INVALID_ARGUMENT, "spg_gen_expand_rows: null argument");
    SPG_CUDA_TRY(cudaSetDevice(c->device));
    cudaStream_t s = c->stream;
    DevBuf start;
    SPG_TRY(start.alloc((n_rows + 1) * sizeof(uint64_t), s));
    if (n_rows) {
        copy_i64_to_u64<<<grid_for(n_rows, 256, 4096), 256, 0, s>>>(d_lengths, start.as<uint64_t>(), n_rows);
        SPG_LAUNCH_CHECK();
    }
    SPG_TRY(exclusive_scan_u64(c, start.as<uint64_t>(), n_rows, start.as<uint64_t>() + n_rows, s));
    SPG_CUDA_TRY(cudaMemcpyAsync(total, start.as<uint64_t>() + n_rows, sizeof(uint64_t), cudaMemcpyDeviceToHost, s));
    if (n_rows && d_rows) {
        expand_rows_kernel<<<grid_for(n_rows * 32, 256), 256, 0, s>>>(start.as<uint64_t>(), n_rows, d_rows);
        SPG_LAUNCH_CHECK();
    }
    SPG_CUDA_TRY(cudaStreamSynchronize(s));
    return SPG_OK;
}

int spg_gen_family(spg_ctx *c, int family, uint64_t n_rows, uint64_t p, double ls, const double *d_cdf, uint64_t seed,
                   uint32_t *d_rows, uint32_t *d_cols, double *d_vals, uint64_t *m) {
    if (!c || !m) return set_error(SPG_ERR_INVALID_ARGUMENT, "spg_gen_family: null argument");
    if (family < 0 || family > SPG_FAM_POISSON)
        return set_error(SPG_ERR_INVALID_ARGUMENT, "spg_gen_family: unknown family %d", family);
    if (family != SPG_FAM_POISSON && p == 0) return set_error(SPG_ERR_INVALID_ARGUMENT, "spg_gen_family: p == 0");
    if (family == SPG_FAM_POWERLAW && !d_cdf) return set_error(SPG_ERR_INVALID_ARGUMENT, "spg_gen_family: no cdf");
    if (n_rows > 0xFFFFFFFFull) return set_error(SPG_ERR_INVALID_ARGUMENT, "spg_gen_family: too many rows");
    SPG_CUDA_TRY(cudaSetDevice(c->device));
    cudaStream_t s = c->stream;
    DevBuf start;
    SPG_TRY(start.alloc((n_rows + 1) * sizeof(uint64_t), s));
    if (n_rows) {
        fam_lengths_kernel<<<grid_for(n_rows, 256, (unsigned)c->n_sms * 32), 256, 0, s>>>(
            family, n_rows, p, ls, d_cdf, seed, start.as<uint64_t>());
        SPG_LAUNCH_CHECK();
    }
    SPG_TRY(exclusive_scan_u64(c, start.as<uint64_t>(), n_rows, start.as<uint64_t>() + n_rows, s));
    SPG_CUDA_TRY(cudaMemcpyAsync(m, start.as<uint64_t>() + n_rows, sizeof(uint64_t), cudaMemcpyDeviceToHost, s));
    SPG_CUDA_TRY(cudaStreamSynchronize(s));
    if (d_rows && d_cols && d_vals && n_rows) {
        fam_fill_kernel<<<grid_for(n_rows * 32, 256), 256, 0, s>>>(family, n_rows, p, seed, start.as<uint64_t>(),
                                                                  d_rows, d_cols, d_vals);
        SPG_LAUNCH_CHECK();
        SPG_CUDA_TRY(cudaStreamSynchronize(s));
    }
    return SPG_OK;
}

}  // extern "C"
