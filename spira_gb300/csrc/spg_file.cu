// spg_file.cu — a binary CSR file format for device matrices (no Spira
// counterpart: Spira has no on-disk format).
//
// Layout, little-endian, every section starting on an 8-byte boundary:
//   header   64 bytes: magic "SPGCSR\0\0", u64 version (1), n_rows, n_cols,
//            nnz, flags (bit 0: the values may hold explicit +-0, as
//            load_csr can install), checksum, reserved 0
//   offsets  u64[n_rows + 1]
//   cols     u32[nnz], zero-padded to a multiple of 8 bytes
//   vals     f64[nnz]
// The checksum is order-independent, so the GPU computes it with one
// reduction: the payload read as 64-bit words w_i (i counting from the first
// offsets word), checksum = sum over i of mix(w_i ^ (i * 0x9E3779B97F4A7C15))
// modulo 2^64, mix being the splitmix64 finaliser.
//
// Saving copies the device arrays through two pinned staging buffers while
// the file is written; loading reads the file in chunks into the same
// buffers and uploads each while the next is read. A loaded file is checked
// against its header sizes, its checksum and the CSR rules of load_csr
// (matrix.hpp:524-575) on the device before it replaces the matrix.
#include <cstdio>
#include <cstring>
#include <vector>

#include "spg_internal.cuh"

namespace spg {
namespace {

constexpr char MAGIC[8] = {'S', 'P', 'G', 'C', 'S', 'R', 0, 0};
constexpr uint64_t VERSION = 1;
constexpr uint64_t FLAG_ZEROS = 1;
constexpr size_t CHUNK = 32u << 20;  // staging buffer bytes
constexpr int FB = 256;

struct FileHeader {
    char magic[8];
    uint64_t version, n_rows, n_cols, nnz, flags, checksum, reserved;
};
static_assert(sizeof(FileHeader) == 64, "header is 64 bytes");

__device__ __forceinline__ uint64_t mix64(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// Adds the words of one section (word i of the payload at index base + i)
// to *sum. n_bytes may end inside a word: the rest of that word counts as 0.
__global__ void __launch_bounds__(FB)
checksum_words(const unsigned char *__restrict__ p, uint64_t n_bytes, uint64_t base,
               unsigned long long *__restrict__ sum) {
    const uint64_t n_words = (n_bytes + 7) / 8;
    unsigned long long acc = 0;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n_words;
         i += (uint64_t)gridDim.x * blockDim.x) {
        uint64_t w;
        if (8 * i + 8 <= n_bytes) {
            w = reinterpret_cast<const uint64_t *>(p)[i];  // sections start 8-byte aligned
        } else {
            w = 0;
            for (uint64_t b = 8 * i; b < n_bytes; ++b) w |= (uint64_t)p[b] << (8 * (b - 8 * i));
        }
        acc += mix64(w ^ ((base + i) * 0x9E3779B97F4A7C15ull));
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    __shared__ unsigned long long s[FB / 32];
    if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < FB / 32; ++w) acc += s[w];
        atomicAdd(sum, acc);
    }
}

// CSR rules, flags: bit 0 offsets[0] != 0, bit 1 not non-decreasing (or past
// nnz), bit 2 column out of range, bit 3 columns not strictly ascending in a
// row, bit 4 a +-0 value (allowed; reported for the zeros flag).
__global__ void validate_csr(const uint64_t *__restrict__ off, const uint32_t *__restrict__ cols,
                             const double *__restrict__ vals, uint64_t n_rows, uint64_t n_cols, uint64_t nnz,
                             unsigned *__restrict__ flags) {
    unsigned f = 0;
    const uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x, nt = (uint64_t)gridDim.x * blockDim.x;
    if (t == 0 && off[0] != 0) f |= 1u;
    for (uint64_t r = t; r < n_rows; r += nt)
        if (off[r] > off[r + 1] || off[r + 1] > nnz) f |= 2u;
    for (uint64_t k = t; k < nnz; k += nt) {
        if ((uint64_t)cols[k] >= n_cols) f |= 4u;
        if (fabs(vals[k]) <= 0.0) f |= 16u;
    }
    if (f) atomicOr(flags, f);
}

// Strict ascent inside rows, checked once offsets are known to be sound.
__global__ void validate_rows(const uint64_t *__restrict__ off, const uint32_t *__restrict__ cols, uint64_t n_rows,
                              unsigned *__restrict__ flags) {
    for (uint64_t r = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; r < n_rows;
         r += (uint64_t)gridDim.x * blockDim.x) {
        for (uint64_t k = off[r] + 1; k < off[r + 1]; ++k)
            if (cols[k] <= cols[k - 1]) {
                atomicOr(flags, 8u);
                break;
            }
    }
}

uint64_t pad8(uint64_t b) { return (b + 7) & ~7ull; }

int device_checksum(Ctx *c, const uint64_t *off, const uint32_t *cols, const double *vals, uint64_t n_rows,
                    uint64_t nnz, cudaStream_t s, uint64_t *out) {
    DevBuf sum;
    SPG_TRY(sum.alloc(sizeof(unsigned long long), s));
    SPG_CUDA_TRY(cudaMemsetAsync(sum.ptr, 0, sizeof(unsigned long long), s));
    const unsigned cap = (unsigned)c->n_sms * 8;
    const uint64_t ob = (n_rows + 1) * 8, cb = nnz * 4, vb = nnz * 8;
    unsigned long long *d = sum.as<unsigned long long>();
    checksum_words<<<grid_for((ob + 7) / 8, FB, cap), FB, 0, s>>>(reinterpret_cast<const unsigned char *>(off), ob, 0,
                                                                 d);
    if (cb)
        checksum_words<<<grid_for((cb + 7) / 8, FB, cap), FB, 0, s>>>(reinterpret_cast<const unsigned char *>(cols),
                                                                     cb, ob / 8, d);
    if (vb)
        checksum_words<<<grid_for(vb / 8, FB, cap), FB, 0, s>>>(reinterpret_cast<const unsigned char *>(vals), vb,
                                                               ob / 8 + pad8(cb) / 8, d);
    SPG_LAUNCH_CHECK();
    SPG_CUDA_TRY(cudaMemcpyAsync(out, d, 8, cudaMemcpyDeviceToHost, s));
    SPG_CUDA_TRY(cudaStreamSynchronize(s));
    return SPG_OK;
}

struct File {
    FILE *f = nullptr;
    ~File() {
        if (f) fclose(f);
    }
};

// Two pinned staging buffers for chunked transfers.
struct Staging {
    void *buf[2] = {nullptr, nullptr};
    cudaEvent_t ev[2] = {nullptr, nullptr};
    ~Staging() {
        for (int i = 0; i < 2; ++i) {
            if (ev[i]) cudaEventSynchronize(ev[i]), cudaEventDestroy(ev[i]);
            if (buf[i]) cudaFreeHost(buf[i]);
        }
    }
    int init() {
        for (int i = 0; i < 2; ++i) {
            SPG_CUDA_TRY(cudaMallocHost(&buf[i], CHUNK));
            SPG_CUDA_TRY(cudaEventCreateWithFlags(&ev[i], cudaEventDisableTiming));
        }
        return SPG_OK;
    }
};

int write_section(FILE *f, const void *dev, uint64_t bytes, Staging &st, cudaStream_t s) {
    for (uint64_t done = 0, k = 0; done < bytes; done += CHUNK, ++k) {
        const uint64_t n = std::min<uint64_t>(CHUNK, bytes - done);
        const int b = (int)(k & 1);
        SPG_CUDA_TRY(cudaMemcpyAsync(st.buf[b], static_cast<const char *>(dev) + done, n, cudaMemcpyDeviceToHost, s));
        SPG_CUDA_TRY(cudaEventRecord(st.ev[b], s));
        SPG_CUDA_TRY(cudaEventSynchronize(st.ev[b]));
        if (fwrite(st.buf[b], 1, n, f) != n) return set_error(SPG_ERR_INVALID_ARGUMENT, "spg_csr_save: write failed");
    }
    const uint64_t pad = pad8(bytes) - bytes;
    static const char zeros[8] = {};
    if (pad && fwrite(zeros, 1, pad, f) != pad) return set_error(SPG_ERR_INVALID_ARGUMENT, "spg_csr_save: write failed");
    return SPG_OK;
}

// Reads `bytes` from the file into device memory, chunk k+1 read while
// chunk k uploads.
int read_section(FILE *f, void *dev, uint64_t bytes, Staging &st, cudaStream_t s) {
    for (uint64_t done = 0, k = 0; done < bytes; done += CHUNK, ++k) {
        const uint64_t n = std::min<uint64_t>(CHUNK, bytes - done);
        const int b = (int)(k & 1);
        SPG_CUDA_TRY(cudaEventSynchronize(st.ev[b]));  // the upload that last used this buffer is done
        if (fread(st.buf[b], 1, n, f) != n) return set_error(SPG_ERR_INVALID_ARGUMENT, "spg_csr_load_file: file truncated");
        SPG_CUDA_TRY(cudaMemcpyAsync(static_cast<char *>(dev) + done, st.buf[b], n, cudaMemcpyHostToDevice, s));
        SPG_CUDA_TRY(cudaEventRecord(st.ev[b], s));
    }
    const uint64_t pad = pad8(bytes) - bytes;
    char tmp[8];
    if (pad && fread(tmp, 1, pad, f) != pad) return set_error(SPG_ERR_INVALID_ARGUMENT, "spg_csr_load_file: file truncated");
    return SPG_OK;
}

int read_header(const char *path, FileHeader *h, uint64_t *file_bytes) {
    File fl;
    fl.f = fopen(path, "rb");
    if (!fl.f) return set_error(SPG_ERR_INVALID_ARGUMENT, "spg_csr_file: cannot open %s", path);
    if (fread(h, 1, sizeof(FileHeader), fl.f) != sizeof(FileHeader))
        return set_error(SPG_ERR_INVALID_ARGUMENT, "spg_csr_file: file shorter than its header");
    if (memcmp(h->magic, MAGIC, 8) != 0) return set_error(SPG_ERR_INVALID_ARGUMENT, "spg_csr_file: not a CSR file");
    if (h->version != VERSION)
        return set_error(SPG_ERR_UNSUPPORTED, "spg_csr_file: version %llu", (unsigned long long)h->version);
    if (fseek(fl.f, 0, SEEK_END) != 0) return set_error(SPG_ERR_INVALID_ARGUMENT, "spg_csr_file: cannot seek");
    const long end = ftell(fl.f);
    if (end < 0) return set_error(SPG_ERR_INVALID_ARGUMENT, "spg_csr_file: cannot seek");
    *file_bytes = (uint64_t)end;
    // sizes must describe exactly the file (and not overflow)
    if (h->n_rows >= (1ull << 40) || h->nnz >= (1ull << 40) || h->n_cols > (1ull << 32))
        return set_error(SPG_ERR_INVALID_ARGUMENT, "spg_csr_file: sizes out of range");
    const uint64_t want = sizeof(FileHeader) + (h->n_rows + 1) * 8 + pad8(h->nnz * 4) + h->nnz * 8;
    if (want != *file_bytes) return set_error(SPG_ERR_INVALID_ARGUMENT, "spg_csr_file: file size does not match its header");
    return SPG_OK;
}

}  // namespace
}  // namespace spg

using namespace spg;

extern "C" {

int spg_csr_file_info(const char *path, uint64_t *n_rows, uint64_t *n_cols, uint64_t *nnz) {
    if (!path) return set_error(SPG_ERR_INVALID_ARGUMENT, "spg_csr_file_info: null path");
    FileHeader h;
    uint64_t bytes = 0;
    SPG_TRY(read_header(path, &h, &bytes));
    if (n_rows) *n_rows = h.n_rows;
    if (n_cols) *n_cols = h.n_cols;
    if (nnz) *nnz = h.nnz;
    return SPG_OK;
}

int spg_csr_save(spg_ctx *c, const spg_csr *A, const char *path) {
    if (!c || !A || !path) return set_error(SPG_ERR_INVALID_ARGUMENT, "spg_csr_save: null argument");
    SPG_CHECK_LIVE(A);
    if (!A->built) return set_error(SPG_ERR_LOGIC, "spg_csr_save: matrix must be locked");
    SPG_CUDA_TRY(cudaSetDevice(c->device));
    cudaStream_t s = c->stream;
    FileHeader h{};
    memcpy(h.magic, MAGIC, 8);
    h.version = VERSION;
    h.n_rows = A->n_rows;
    h.n_cols = A->n_cols;
    h.nnz = A->nnz;
    h.flags = A->may_have_zeros ? FLAG_ZEROS : 0;
    SPG_TRY(device_checksum(c, A->d_off(), A->d_cols(), A->d_vals(), A->n_rows, A->nnz, s, &h.checksum));
    Staging st;
    SPG_TRY(st.init());
    File fl;
    fl.f = fopen(path, "wb");
    if (!fl.f) return set_error(SPG_ERR_INVALID_ARGUMENT, "spg_csr_save: cannot create %s", path);
    if (fwrite(&h, 1, sizeof(h), fl.f) != sizeof(h)) return set_error(SPG_ERR_INVALID_ARGUMENT, "spg_csr_save: write failed");
    SPG_TRY(write_section(fl.f, A->d_off(), (A->n_rows + 1) * 8, st, s));
    SPG_TRY(write_section(fl.f, A->d_cols(), A->nnz * 4, st, s));
    SPG_TRY(write_section(fl.f, A->d_vals(), A->nnz * 8, st, s));
    if (fflush(fl.f) != 0) return set_error(SPG_ERR_INVALID_ARGUMENT, "spg_csr_save: write failed");
    return SPG_OK;
}

int spg_csr_load_file(spg_ctx *c, spg_csr *A, const char *path) {
    if (!c || !A || !path) return set_error(SPG_ERR_INVALID_ARGUMENT, "spg_csr_load_file: null argument");
    SPG_CHECK_LIVE(A);
    FileHeader h;
    uint64_t bytes = 0;
    SPG_TRY(read_header(path, &h, &bytes));
    SPG_CUDA_TRY(cudaSetDevice(c->device));
    cudaStream_t s = c->stream;
    const uint64_t n = h.n_rows, nnz = h.nnz;
    DevBuf off, cols, vals;
    SPG_TRY(off.alloc(csr_off_elems(n) * sizeof(uint64_t), s));
    SPG_TRY(cols.alloc(csr_alloc_elems(nnz) * sizeof(uint32_t), s));
    SPG_TRY(vals.alloc(csr_alloc_elems(nnz) * sizeof(double), s));
    {
        Staging st;
        SPG_TRY(st.init());
        File fl;
        fl.f = fopen(path, "rb");
        if (!fl.f) return set_error(SPG_ERR_INVALID_ARGUMENT, "spg_csr_load_file: cannot open %s", path);
        if (fseek(fl.f, (long)sizeof(FileHeader), SEEK_SET) != 0)
            return set_error(SPG_ERR_INVALID_ARGUMENT, "spg_csr_load_file: cannot seek");
        SPG_TRY(read_section(fl.f, off.ptr, (n + 1) * 8, st, s));
        SPG_TRY(read_section(fl.f, cols.ptr, nnz * 4, st, s));
        SPG_TRY(read_section(fl.f, vals.ptr, nnz * 8, st, s));
        SPG_CUDA_TRY(cudaStreamSynchronize(s));
    }
    uint64_t sum = 0;
    SPG_TRY(device_checksum(c, off.as<uint64_t>(), cols.as<uint32_t>(), vals.as<double>(), n, nnz, s, &sum));
    if (sum != h.checksum) return set_error(SPG_ERR_INVALID_ARGUMENT, "spg_csr_load_file: checksum mismatch");
    DevBuf fl;
    SPG_TRY(fl.alloc(sizeof(unsigned), s));
    SPG_CUDA_TRY(cudaMemsetAsync(fl.ptr, 0, sizeof(unsigned), s));
    const unsigned cap = (unsigned)c->n_sms * 8;
    validate_csr<<<grid_for(std::max(n, nnz), FB, cap), FB, 0, s>>>(off.as<uint64_t>(), cols.as<uint32_t>(),
                                                                    vals.as<double>(), n, h.n_cols, nnz,
                                                                    fl.as<unsigned>());
    SPG_LAUNCH_CHECK();
    unsigned f = 0;
    SPG_CUDA_TRY(cudaMemcpyAsync(&f, fl.ptr, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
    SPG_CUDA_TRY(cudaStreamSynchronize(s));
    if (f & 1u) return set_error(SPG_ERR_INVALID_ARGUMENT, "spira::matrix::load_csr: CSR offsets[0] must be zero");
    uint64_t last = 0;
    SPG_CUDA_TRY(cudaMemcpyAsync(&last, off.as<uint64_t>() + n, 8, cudaMemcpyDeviceToHost, s));
    SPG_CUDA_TRY(cudaStreamSynchronize(s));
    if (last != nnz)
        return set_error(SPG_ERR_INVALID_ARGUMENT, "spira::matrix::load_csr: CSR offsets[n_rows] does not equal nnz");
    if (f & 2u)
        return set_error(SPG_ERR_INVALID_ARGUMENT, "spira::matrix::load_csr: CSR offsets are not non-decreasing");
    if (f & 4u) return set_error(SPG_ERR_INVALID_ARGUMENT, "spira::matrix::load_csr: column index out of bounds");
    validate_rows<<<grid_for(n, FB, cap), FB, 0, s>>>(off.as<uint64_t>(), cols.as<uint32_t>(), n, fl.as<unsigned>());
    SPG_LAUNCH_CHECK();
    SPG_CUDA_TRY(cudaMemcpyAsync(&f, fl.ptr, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
    SPG_CUDA_TRY(cudaStreamSynchronize(s));
    if (f & 8u)
        return set_error(SPG_ERR_INVALID_ARGUMENT,
                         "spira::matrix::load_csr: CSR row entries are not strictly sorted by column");
    A->invalidate_derived();
    A->n_rows = n;
    A->n_cols = h.n_cols;
    A->off = std::move(off);
    A->cols = std::move(cols);
    A->vals = std::move(vals);
    A->nnz = nnz;
    A->capacity = nnz;
    A->built = true;
    A->may_have_zeros = (f & 16u) != 0;
    return SPG_OK;
}

}  // extern "C"
