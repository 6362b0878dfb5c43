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

}  // extern "C"
