// spg_tune.cu — variant choice for SpMV: the exhaustive autotuner, the
// matrix features, and the learned selector (a 40 -> 64 -> 64 -> K FP32 MLP
// with hand-written forward, backward and Adam kernels).
//
// Spira has a single SpMV code path per type combination (serial/spmv.hpp,
// parallel/algorithms/spmv.hpp), so none of this has a Spira counterpart; it
// decides which of this engine's kernels computes Spira's SpMV. The
// arithmetic of the SpMV kernels is the same whichever is chosen.
//
// Policy for SPG_SPMV_AUTO (per matrix, cached until the next lock):
//   a selector model is installed -> features + MLP inference on the device,
//                                    argmin of the predicted log-times;
//   otherwise                      -> exhaustive autotune (every variant timed
//                                    with CUDA events), fastest wins.
#include <dlfcn.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdlib>
#include <string>
#include <vector>

#include "spg_internal.cuh"

namespace spg {
namespace {

// ---------------------------------------------------------------- gather probe
// The ceiling of SpMV on matrices whose columns are spread at random: random
// 8-byte reads of an L2-resident x. Each thread makes 16 independent reads at
// hashed positions (32-bit "lowbias32" finaliser), so every warp request
// touches ~32 different sectors, as the x gathers of such a matrix do.
constexpr uint64_t GATHER_PER_THREAD = 16;

__device__ __forceinline__ uint32_t mix32(uint32_t a) {
    a ^= a >> 16;
    a *= 0x7feb352dU;
    a ^= a >> 15;
    a *= 0x846ca68bU;
    a ^= a >> 16;
    return a;
}

__global__ void gather_probe(const double *__restrict__ x, uint32_t mask, double *__restrict__ out, uint64_t n_thr) {
    const uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (t >= n_thr) return;
    // the values are combined with integer XOR: the probe times gathers alone,
    // with no FP64 work beside them (an FP64 add per gather measured the same)
    unsigned long long a = 0;
#pragma unroll
    for (uint32_t j = 0; j < GATHER_PER_THREAD; ++j)
        a ^= (unsigned long long)__double_as_longlong(
            __ldg(x + (mix32((uint32_t)t * (uint32_t)GATHER_PER_THREAD + j) & mask)));
    out[t] = __longlong_as_double((long long)a);
}

// The same reads with the number in flight and the occupancy as parameters:
// a grid of blocks_per_sm x SMs blocks of 256 threads walks n_iter work items
// of PER independent gathers each (grid-stride), so each thread has PER reads
// in flight and an SM at most blocks x 256 x PER. Sweeping both shows whether
// the rate above is a hardware ceiling or a latency limit of one shape.
template <int PER>
__global__ void __launch_bounds__(256) gather_probe_cfg(const double *__restrict__ x, uint32_t mask,
                                                        double *__restrict__ out, uint64_t n_iter) {
    const uint64_t t0 = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    const uint64_t nt = (uint64_t)gridDim.x * blockDim.x;
    unsigned long long a = 0;
    for (uint64_t it = t0; it < n_iter; it += nt) {
#pragma unroll
        for (uint32_t j = 0; j < (uint32_t)PER; ++j)
            a ^= (unsigned long long)__double_as_longlong(__ldg(x + (mix32((uint32_t)it * (uint32_t)PER + j) & mask)));
    }
    out[t0] = __longlong_as_double((long long)a);
}

// FP64 FMA rate: 8 independent chains per thread (enough warps and chains to
// cover the pipe's latency); a = a * m + c with |m| < 1 stays bounded. m and c
// are arguments, so nothing folds at compile time.
constexpr int FMA_CHAINS = 8;

__global__ void __launch_bounds__(256) fma_probe(double m, double c, uint32_t iters, double *__restrict__ out) {
    double a[FMA_CHAINS];
#pragma unroll
    for (int i = 0; i < FMA_CHAINS; ++i) a[i] = (double)(threadIdx.x + i);
    for (uint32_t it = 0; it < iters; ++it) {
#pragma unroll
        for (int i = 0; i < FMA_CHAINS; ++i) a[i] = fma(a[i], m, c);
    }
    double s = 0.0;
#pragma unroll
    for (int i = 0; i < FMA_CHAINS; ++i) s += a[i];
    out[blockIdx.x * (uint64_t)blockDim.x + threadIdx.x] = s;
}

// ---------------------------------------------------------------- features
// acc layout (doubles): [0..31] histogram, 32 sum L, 33 sum L^2, 34 max L,
// 35 empty rows, 36 sum of |col/n_cols - row/n_rows| over sampled nonzeros,
// 37 sampled nonzeros.
__global__ void feat_rows(const uint64_t *__restrict__ off, const uint32_t *__restrict__ cols, uint64_t n_rows,
                          uint64_t n_cols, double *__restrict__ acc) {
    __shared__ double s[38];
    for (int i = threadIdx.x; i < 38; i += blockDim.x) s[i] = 0.0;
    __syncthreads();
    double sl = 0, sl2 = 0, mx = 0, emp = 0, spread = 0, cnt = 0;
    for (uint64_t r = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; r < n_rows;
         r += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t b = off[r], e = off[r + 1];
        const uint64_t L = e - b;
        int bin = 0;
        if (L) {
            bin = 1 + (63 - __clzll((long long)L));
            if (bin > 31) bin = 31;
        } else {
            emp += 1;
        }
        atomicAdd(&s[bin], 1.0);
        sl += (double)L;
        sl2 += (double)L * (double)L;
        mx = fmax(mx, (double)L);
        if ((r & 15) == 0 && L) {  // spread proxy on every 16th row, first and last entry
            const double rr = (double)r / (double)n_rows;
            spread += fabs((double)cols[b] / (double)n_cols - rr) + fabs((double)cols[e - 1] / (double)n_cols - rr);
            cnt += 2;
        }
    }
    atomicAdd(&s[32], sl);
    atomicAdd(&s[33], sl2);
    atomicAdd(&s[35], emp);
    atomicAdd(&s[36], spread);
    atomicAdd(&s[37], cnt);
    // max via integer atomic on the bit pattern (non-negative doubles order as integers)
    atomicMax(reinterpret_cast<unsigned long long *>(&s[34]), __double_as_longlong(mx));
    __syncthreads();
    for (int i = threadIdx.x; i < 38; i += blockDim.x) {
        if (i == 34) atomicMax(reinterpret_cast<unsigned long long *>(&acc[34]), __double_as_longlong(s[34]));
        else atomicAdd(&acc[i], s[i]);
    }
}

// SpGEMM features of A * B. acc layout (doubles): [0..31] histogram of the
// products per row (bin 0: none, else 1 + floor(log2 p), capped at 31),
// 32 sum p, 33 sum p^2, 34 max p, 35 sum of |col / n_cols - row / m| over the
// first and last entry of every 16th non-empty row of A, 36 their number,
// 37 the longest row of A (entries).
// The spread tells local patterns (banded, block-diagonal, stencils: a row's
// products fall on few columns, the output is several times smaller than
// the products) from scattered ones (products mostly distinct), which the
// counts alone do not: uniform rows of 8 and 8 x 8 diagonal blocks both give
// 64 products per row, and the fastest variant differs.
__global__ void feat_gemm_rows(const uint64_t *__restrict__ aoff, const uint32_t *__restrict__ acols,
                               const uint64_t *__restrict__ boff, uint64_t m, uint64_t n_cols_a,
                               double *__restrict__ acc) {
    __shared__ double s[38];
    for (int i = threadIdx.x; i < 38; i += blockDim.x) s[i] = 0.0;
    __syncthreads();
    double sp = 0, sp2 = 0, mx = 0, spread = 0, cnt = 0, mxa = 0;
    for (uint64_t r = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; r < m; r += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t a0 = aoff[r], a1 = aoff[r + 1];
        uint64_t p = 0;
        for (uint64_t ka = a0; ka < a1; ++ka) {
            const uint32_t k = acols[ka];
            p += boff[k + 1] - boff[k];
        }
        int bin = 0;
        if (p) {
            bin = 1 + (63 - __clzll((long long)p));
            if (bin > 31) bin = 31;
        }
        atomicAdd(&s[bin], 1.0);
        sp += (double)p;
        sp2 += (double)p * (double)p;
        mx = fmax(mx, (double)p);
        mxa = fmax(mxa, (double)(a1 - a0));
        if ((r & 15) == 0 && a1 > a0) {
            const double rr = (double)r / (double)m;
            spread += fabs((double)acols[a0] / (double)n_cols_a - rr) + fabs((double)acols[a1 - 1] / (double)n_cols_a - rr);
            cnt += 2;
        }
    }
    atomicAdd(&s[32], sp);
    atomicAdd(&s[33], sp2);
    atomicMax(reinterpret_cast<unsigned long long *>(&s[34]), __double_as_longlong(mx));
    atomicAdd(&s[35], spread);
    atomicAdd(&s[36], cnt);
    atomicMax(reinterpret_cast<unsigned long long *>(&s[37]), __double_as_longlong(mxa));
    __syncthreads();
    for (int i = threadIdx.x; i < 38; i += blockDim.x) {
        if (i == 34 || i == 37) atomicMax(reinterpret_cast<unsigned long long *>(&acc[i]), __double_as_longlong(s[i]));
        else atomicAdd(&acc[i], s[i]);
    }
}

// ---------------------------------------------------------------- MLP
// Parameter layout (floats): W1[H][F] b1[H] W2[H][H] b2[H] W3[K][H] b3[K];
// a selector blob is [mean[F] scale[F] params...]: x_norm = (x - mean) * scale.
constexpr int F = SPG_SELECT_FEATURES;
constexpr int H = SPG_SELECT_HIDDEN;

__host__ __device__ constexpr uint64_t n_params(int K) {
    return (uint64_t)H * F + H + (uint64_t)H * H + H + (uint64_t)K * H + K;
}

// layer: out[b][j] = act(sum_i W[j][i] in[b][i] + bias[j]); one thread per (b, j)
__global__ void mlp_dense(const float *__restrict__ W, const float *__restrict__ bias, const float *__restrict__ in,
                          int n_in, int n_out, uint32_t B, int relu, float *__restrict__ out) {
    const uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (uint64_t)B * n_out) return;
    const uint32_t b = (uint32_t)(t / n_out);
    const int j = (int)(t % n_out);
    const float *w = W + (uint64_t)j * n_in;
    const float *x = in + (uint64_t)b * n_in;
    float s = bias[j];
    for (int i = 0; i < n_in; ++i) s = fmaf(w[i], x[i], s);
    out[t] = relu ? fmaxf(s, 0.0f) : s;
}

__global__ void mlp_normalize(const float *__restrict__ X, const float *__restrict__ mean,
                              const float *__restrict__ scale, uint32_t B, float *__restrict__ out) {
    const uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (uint64_t)B * F) return;
    const int i = (int)(t % F);
    out[t] = (X[t] - mean[i]) * scale[i];
}

// dIn[b][i] = sum_j dOut[b][j] * W[j][i], masked by the ReLU of `act_in` when given
__global__ void mlp_back_input(const float *__restrict__ W, const float *__restrict__ dout, int n_in, int n_out,
                               uint32_t B, const float *__restrict__ act_in, float *__restrict__ din) {
    const uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (uint64_t)B * n_in) return;
    const uint32_t b = (uint32_t)(t / n_in);
    const int i = (int)(t % n_in);
    float s = 0.0f;
    for (int j = 0; j < n_out; ++j) s = fmaf(dout[(uint64_t)b * n_out + j], W[(uint64_t)j * n_in + i], s);
    if (act_in && act_in[t] <= 0.0f) s = 0.0f;
    din[t] = s;
}

// dW[j][i] = sum_b dOut[b][j] in[b][i]; dbias[j] = sum_b dOut[b][j]; one thread per weight
__global__ void mlp_back_weights(const float *__restrict__ dout, const float *__restrict__ in, int n_in, int n_out,
                                 uint32_t B, float *__restrict__ dW, float *__restrict__ db) {
    const uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const uint64_t nw = (uint64_t)n_out * n_in;
    if (t < nw) {
        const int j = (int)(t / n_in), i = (int)(t % n_in);
        float s = 0.0f;
        for (uint32_t b = 0; b < B; ++b) s = fmaf(dout[(uint64_t)b * n_out + j], in[(uint64_t)b * n_in + i], s);
        dW[t] = s;
    } else if (t < nw + n_out) {
        const int j = (int)(t - nw);
        float s = 0.0f;
        for (uint32_t b = 0; b < B; ++b) s += dout[(uint64_t)b * n_out + j];
        db[j] = s;
    }
}

// loss = mean over (b, k) of (pred - target)^2; dpred = 2 (pred - target) / (B K)
__global__ void mlp_mse_grad(const float *__restrict__ pred, const float *__restrict__ target, uint64_t n,
                             float *__restrict__ dpred, float *__restrict__ loss_acc) {
    const uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    float l = 0.0f;
    if (t < n) {
        const float d = pred[t] - target[t];
        dpred[t] = 2.0f * d / (float)n;
        l = d * d / (float)n;
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) l += __shfl_xor_sync(0xffffffffu, l, o);
    if ((threadIdx.x & 31) == 0 && loss_acc) atomicAdd(loss_acc, l);
}

__global__ void mlp_adam(float *__restrict__ w, const float *__restrict__ g, float *__restrict__ m,
                         float *__restrict__ v, uint64_t n, float lr, float b1, float b2, float eps, float c1,
                         float c2) {
    const uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const float gt = g[t];
    const float mt = b1 * m[t] + (1.0f - b1) * gt;
    const float vt = b2 * v[t] + (1.0f - b2) * gt * gt;
    m[t] = mt;
    v[t] = vt;
    w[t] -= lr * (mt / c1) / (sqrtf(vt / c2) + eps);
}

__global__ void mlp_argmin(const float *__restrict__ pred, uint32_t B, int K, int *__restrict__ best) {
    const uint32_t b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= B) return;
    int bi = 0;
    float bv = pred[(uint64_t)b * K];
    for (int k = 1; k < K; ++k) {
        const float v = pred[(uint64_t)b * K + k];
        if (v < bv) {
            bv = v;
            bi = k;
        }
    }
    best[b] = bi;
}

struct Layers {
    const float *W1, *b1, *W2, *b2, *W3, *b3;
};

Layers layers(const float *P, int K) {
    Layers L;
    L.W1 = P;
    L.b1 = L.W1 + (uint64_t)H * F;
    L.W2 = L.b1 + H;
    L.b2 = L.W2 + (uint64_t)H * H;
    L.W3 = L.b2 + H;
    L.b3 = L.W3 + (uint64_t)K * H;
    return L;
}

// act workspace per sample: h1[H], h2[H]
int forward(const float *P, int K, const float *Xn, uint32_t B, float *act, float *out, cudaStream_t s) {
    const Layers L = layers(P, K);
    float *h1 = act, *h2 = act + (uint64_t)B * H;
    mlp_dense<<<grid_for((uint64_t)B * H, 256), 256, 0, s>>>(L.W1, L.b1, Xn, F, H, B, 1, h1);
    mlp_dense<<<grid_for((uint64_t)B * H, 256), 256, 0, s>>>(L.W2, L.b2, h1, H, H, B, 1, h2);
    mlp_dense<<<grid_for((uint64_t)B * K, 256), 256, 0, s>>>(L.W3, L.b3, h2, H, K, B, 0, out);
    SPG_LAUNCH_CHECK();
    return SPG_OK;
}

}  // namespace

// ---------------------------------------------------------------- host side
int spmv_features(Ctx *c, Csr *A, float *f) {
    cudaStream_t s = c->stream;
    DevBuf acc;
    SPG_TRY(acc.alloc(38 * sizeof(double), s));
    SPG_CUDA_TRY(cudaMemsetAsync(acc.ptr, 0, 38 * sizeof(double), s));
    if (A->n_rows) {
        feat_rows<<<grid_for(A->n_rows, 256, (unsigned)c->n_sms * 8), 256, 0, s>>>(A->d_off(), A->d_cols(), A->n_rows,
                                                                                    A->n_cols ? A->n_cols : 1,
                                                                                    acc.as<double>());
        SPG_LAUNCH_CHECK();
    }
    double h[38];
    SPG_CUDA_TRY(cudaMemcpyAsync(h, acc.ptr, sizeof(h), cudaMemcpyDeviceToHost, s));
    SPG_CUDA_TRY(cudaStreamSynchronize(s));
    const double n = (double)(A->n_rows ? A->n_rows : 1);
    for (int i = 0; i < 32; ++i) f[i] = (float)(h[i] / n);
    const double mean = h[32] / n;
    const double var = std::max(0.0, h[33] / n - mean * mean);
    f[32] = (float)(std::log2((double)A->n_rows + 1.0) / 32.0);
    f[33] = (float)(std::log2((double)A->n_cols + 1.0) / 32.0);
    f[34] = (float)(std::log2((double)A->nnz + 1.0) / 40.0);
    f[35] = (float)(std::log2(mean + 1.0) / 16.0);
    f[36] = (float)(std::log2(std::sqrt(var) + 1.0) / 16.0);
    f[37] = (float)(std::log2(h[34] + 1.0) / 32.0);
    f[38] = (float)(h[35] / n);
    f[39] = (float)(h[37] > 0 ? h[36] / h[37] : 0.0);
    return SPG_OK;
}

int spmv_autotune(Ctx *c, Csr *A, int reps, float *times_ms, int *best) {
    cudaStream_t s = c->stream;
    if (reps < 1) reps = 1;
    if (c->xbuf.bytes < A->n_cols * sizeof(double)) SPG_TRY(c->xbuf.alloc(A->n_cols * sizeof(double), s));
    if (c->ybuf.bytes < A->n_rows * sizeof(double)) SPG_TRY(c->ybuf.alloc(A->n_rows * sizeof(double), s));
    // x = 1.0 everywhere (timing does not depend on the values)
    if (A->n_cols) {
        std::vector<double> ones(std::min<uint64_t>(A->n_cols, 1u << 20), 1.0);
        for (uint64_t o = 0; o < A->n_cols; o += ones.size()) {
            const uint64_t m = std::min<uint64_t>(ones.size(), A->n_cols - o);
            SPG_CUDA_TRY(cudaMemcpyAsync(c->xbuf.as<double>() + o, ones.data(), m * sizeof(double),
                                         cudaMemcpyHostToDevice, s));
            SPG_CUDA_TRY(cudaStreamSynchronize(s));
        }
    }
    cudaEvent_t e0, e1;
    SPG_CUDA_TRY(cudaEventCreate(&e0));
    SPG_CUDA_TRY(cudaEventCreate(&e1));
    int bi = 0;
    float bt = 0.0f;
    int rc = SPG_OK;
    for (int v = 0; v < SPG_SPMV_N_VARIANTS && rc == SPG_OK; ++v) {
        rc = spmv_launch(c, A, c->xbuf.as<double>(), c->ybuf.as<double>(), v, s);  // builds plans, warms up
        if (rc != SPG_OK) break;
        std::vector<float> ts(reps);
        for (int r = 0; r < reps && rc == SPG_OK; ++r) {
            cudaEventRecord(e0, s);
            rc = spmv_launch(c, A, c->xbuf.as<double>(), c->ybuf.as<double>(), v, s);
            cudaEventRecord(e1, s);
            if (cudaEventSynchronize(e1) != cudaSuccess) rc = set_error(SPG_ERR_CUDA, "autotune: event sync failed");
            cudaEventElapsedTime(&ts[r], e0, e1);
        }
        std::sort(ts.begin(), ts.end());
        const float t = ts[ts.size() / 2];
        if (times_ms) times_ms[v] = t;
        if (v == 0 || t < bt) {
            bt = t;
            bi = v;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    SPG_TRY(rc);
    SPG_TRY(c->take_status());
    if (best) *best = bi;
    return SPG_OK;
}

int selector_predict_dev(const DevBuf &model, int K, const float *d_x, uint32_t B, float *d_out, cudaStream_t s) {
    const float *mean = model.as<float>();
    const float *scale = mean + F;
    const float *P = scale + F;
    DevBuf xn, act;
    SPG_TRY(xn.alloc((uint64_t)B * F * sizeof(float), s));
    SPG_TRY(act.alloc((uint64_t)B * 2 * H * sizeof(float), s));
    mlp_normalize<<<grid_for((uint64_t)B * F, 256), 256, 0, s>>>(d_x, mean, scale, B, xn.as<float>());
    SPG_LAUNCH_CHECK();
    return forward(P, K, xn.as<float>(), B, act.as<float>(), d_out, s);
}

int spmv_resolve_auto(Ctx *c, Csr *A, int *variant) {
    if (A->selected_spmv >= 0) {
        *variant = A->selected_spmv;
        return SPG_OK;
    }
    int v = SPG_SPMV_ADAPTIVE;
    if (c->spmv_policy == SPG_POLICY_FIXED) {
        v = SPG_SPMV_ADAPTIVE16;
    } else if (c->spmv_policy == SPG_POLICY_SELECTOR && c->model_k > 0) {
        float f[F];
        SPG_TRY(spmv_features(c, A, f));
        cudaStream_t s = c->stream;
        DevBuf df, dout, db;
        SPG_TRY(df.alloc(F * sizeof(float), s));
        SPG_TRY(dout.alloc(c->model_k * sizeof(float), s));
        SPG_TRY(db.alloc(sizeof(int), s));
        SPG_CUDA_TRY(cudaMemcpyAsync(df.ptr, f, sizeof(f), cudaMemcpyHostToDevice, s));
        SPG_TRY(selector_predict_dev(c->model, c->model_k, df.as<float>(), 1, dout.as<float>(), s));
        mlp_argmin<<<1, 32, 0, s>>>(dout.as<float>(), 1, c->model_k, db.as<int>());
        SPG_LAUNCH_CHECK();
        SPG_CUDA_TRY(cudaMemcpyAsync(&v, db.ptr, sizeof(int), cudaMemcpyDeviceToHost, s));
        SPG_CUDA_TRY(cudaStreamSynchronize(s));
        if (v < 0 || v >= SPG_SPMV_N_VARIANTS) v = SPG_SPMV_ADAPTIVE;
    } else {
        SPG_TRY(spmv_autotune(c, A, 5, nullptr, &v));
    }
    A->selected_spmv = v;
    *variant = v;
    return SPG_OK;
}

// A trained selector shipped beside the library (`file` in the directory of
// libspg.so) or named by the environment variable `env`; absent or malformed
// files leave the context on the autotuner for that operation.
int selector_load_file(Ctx *c, const char *env, const char *file, int max_k, DevBuf *model, int *model_k) {
    std::string path;
    if (const char *e = getenv(env)) {
        path = e;
    } else {
        Dl_info info;
        if (dladdr(reinterpret_cast<void *>(&selector_load_file), &info) && info.dli_fname) {
            path = info.dli_fname;
            const size_t slash = path.rfind('/');
            path = (slash == std::string::npos ? std::string(".") : path.substr(0, slash)) + "/" + file;
        }
    }
    if (path.empty()) return SPG_OK;
    FILE *fp = fopen(path.c_str(), "rb");
    if (!fp) return SPG_OK;
    std::vector<float> blob;
    float buf[4096];
    size_t got;
    while ((got = fread(buf, sizeof(float), 4096, fp)) > 0) blob.insert(blob.end(), buf, buf + got);
    fclose(fp);
    const long long base = 2LL * F + (long long)n_params(0);
    const long long per_k = H + 1;
    const long long rest = (long long)blob.size() - base;
    if (rest <= 0 || rest % per_k) return SPG_OK;
    const int K = (int)(rest / per_k);
    if (K < 1 || K > max_k) return SPG_OK;
    if (model->alloc(blob.size() * sizeof(float), c->stream) != SPG_OK) {
        clear_error();
        return SPG_OK;
    }
    if (cudaMemcpyAsync(model->ptr, blob.data(), blob.size() * sizeof(float), cudaMemcpyHostToDevice, c->stream) !=
            cudaSuccess ||
        cudaStreamSynchronize(c->stream) != cudaSuccess) {
        model->release();
        return SPG_OK;
    }
    *model_k = K;
    return SPG_OK;
}

int selector_load_default(Ctx *c) {
    selector_load_file(c, "SPG_SELECTOR_MODEL", "spg_selector.bin", SPG_SPMV_N_VARIANTS, &c->model, &c->model_k);
    selector_load_file(c, "SPG_SPGEMM_SELECTOR_MODEL", "spg_spgemm_selector.bin", SPG_SPGEMM_N_VARIANTS,
                       &c->gemm_model, &c->gemm_model_k);
    return SPG_OK;
}

// ---------------------------------------------------------------- SpGEMM choice
// max_products / max_a (may be null): the most products and A entries of any row.
int spgemm_features(Ctx *c, const Csr *A, const Csr *B, float *f, double *max_products = nullptr,
                    double *max_a = nullptr) {
    cudaStream_t s = c->stream;
    DevBuf acc;
    SPG_TRY(acc.alloc(38 * sizeof(double), s));
    SPG_CUDA_TRY(cudaMemsetAsync(acc.ptr, 0, 38 * sizeof(double), s));
    if (A->n_rows) {
        feat_gemm_rows<<<grid_for(A->n_rows, 256, (unsigned)c->n_sms * 8), 256, 0, s>>>(
            A->d_off(), A->d_cols(), B->d_off(), A->n_rows, A->n_cols ? A->n_cols : 1, acc.as<double>());
        SPG_LAUNCH_CHECK();
    }
    double h[38];
    SPG_CUDA_TRY(cudaMemcpyAsync(h, acc.ptr, sizeof(h), cudaMemcpyDeviceToHost, s));
    SPG_CUDA_TRY(cudaStreamSynchronize(s));
    if (max_products) *max_products = h[34];
    if (max_a) *max_a = h[37];
    const double m = (double)(A->n_rows ? A->n_rows : 1);
    for (int i = 0; i < 32; ++i) f[i] = (float)(h[i] / m);
    const double mean = h[32] / m;
    const double var = std::max(0.0, h[33] / m - mean * mean);
    f[32] = (float)(std::log2((double)A->n_rows + 1.0) / 32.0);
    f[33] = (float)(std::log2((double)B->n_cols + 1.0) / 32.0);
    f[34] = (float)(std::log2((double)A->nnz + 1.0) / 40.0);
    f[35] = (float)(std::log2(h[32] + 1.0) / 40.0);
    f[36] = (float)(std::log2(mean + 1.0) / 16.0);
    f[37] = (float)(std::log2(std::sqrt(var) + 1.0) / 16.0);
    f[38] = (float)(std::log2(h[34] + 1.0) / 32.0);
    f[39] = (float)(h[36] > 0 ? h[35] / h[36] : 0.0);
    return SPG_OK;
}

int spgemm_autotune(Ctx *c, const Csr *A, const Csr *B, int reps, float *times_ms, int *best) {
    cudaStream_t s = c->stream;
    if (reps < 1) reps = 1;
    int bi = 0;
    double bt = 0.0;
    for (int v = 0; v < SPG_SPGEMM_N_VARIANTS; ++v) {
        std::vector<double> ts;
        for (int r = 0; r <= reps; ++r) {  // run 0 warms up
            Csr tmp;
            tmp.ctx = c;
            SPG_CUDA_TRY(cudaStreamSynchronize(s));
            const auto t0 = std::chrono::steady_clock::now();
            SPG_TRY(spgemm_run(c, A, B, &tmp, v, s));
            SPG_CUDA_TRY(cudaStreamSynchronize(s));
            const auto t1 = std::chrono::steady_clock::now();
            if (r) ts.push_back(std::chrono::duration<double, std::milli>(t1 - t0).count());
        }
        std::sort(ts.begin(), ts.end());
        const double t = ts[ts.size() / 2];
        if (times_ms) times_ms[v] = (float)t;
        if (v == 0 || t < bt) {
            bt = t;
            bi = v;
        }
    }
    if (best) *best = bi;
    return SPG_OK;
}

int spgemm_resolve_auto(Ctx *c, const Csr *A, const Csr *B, int *variant) {
    Csr *Am = const_cast<Csr *>(A);
    if (Am->gemm_selected >= 0 && Am->gemm_sel_b == B && Am->gemm_sel_b_epoch == B->epoch) {
        *variant = Am->gemm_selected;
        return SPG_OK;
    }
    int v = SPG_SPGEMM_WARPSORT_128;
    if (c->spgemm_policy == SPG_POLICY_SELECTOR && c->gemm_model_k == SPG_SPGEMM_N_VARIANTS) {
        float f[F];
        double maxp = 0.0, maxa = 0.0;
        SPG_TRY(spgemm_features(c, A, B, f, &maxp, &maxa));
        cudaStream_t s = c->stream;
        DevBuf df, dout;
        SPG_TRY(df.alloc(F * sizeof(float), s));
        SPG_TRY(dout.alloc(SPG_SPGEMM_N_VARIANTS * sizeof(float), s));
        SPG_CUDA_TRY(cudaMemcpyAsync(df.ptr, f, sizeof(f), cudaMemcpyHostToDevice, s));
        SPG_TRY(selector_predict_dev(c->gemm_model, c->gemm_model_k, df.as<float>(), 1, dout.as<float>(), s));
        float sc[SPG_SPGEMM_N_VARIANTS];
        SPG_CUDA_TRY(cudaMemcpyAsync(sc, dout.ptr, sizeof(sc), cudaMemcpyDeviceToHost, s));
        SPG_CUDA_TRY(cudaStreamSynchronize(s));
        // Dominated by construction, never chosen: when every row has at most 64 products and 64 A
        // entries, the WARPSORT variants for 128 and 256 do WARPSORT_64's work row for row with more
        // shared memory per tile (fewer tiles resident); likewise 256 against 128 up to 128.
        if (maxp <= 64.0 && maxa <= 64.0) sc[SPG_SPGEMM_WARPSORT_128] = sc[SPG_SPGEMM_WARPSORT_256] = INFINITY;
        else if (maxp <= 128.0 && maxa <= 128.0) sc[SPG_SPGEMM_WARPSORT_256] = INFINITY;
        v = 0;
        for (int k = 1; k < SPG_SPGEMM_N_VARIANTS; ++k)
            if (sc[k] < sc[v]) v = k;
    } else if (c->spgemm_policy != SPG_POLICY_FIXED) {
        SPG_TRY(spgemm_autotune(c, A, B, 3, nullptr, &v));
    }
    Am->gemm_selected = v;
    Am->gemm_sel_b = B;
    Am->gemm_sel_b_epoch = B->epoch;
    *variant = v;
    return SPG_OK;
}

}  // namespace spg

using namespace spg;

extern "C" {

int spg_spmv_features(spg_ctx *c, const spg_csr *A, float *features) {
    if (!c || !A || !features) return set_error(SPG_ERR_INVALID_ARGUMENT, "spg_spmv_features: null argument");
    if (!A->built) return set_error(SPG_ERR_LOGIC, "spmv: matrix must be locked");
    SPG_CUDA_TRY(cudaSetDevice(c->device));
    return spmv_features(c, const_cast<spg_csr *>(A), features);
}

int spg_spmv_autotune(spg_ctx *c, const spg_csr *A, int reps, float *times_ms, int *best) {
    if (!c || !A) return set_error(SPG_ERR_INVALID_ARGUMENT, "spg_spmv_autotune: null argument");
    if (!A->built) return set_error(SPG_ERR_LOGIC, "spmv: matrix must be locked");
    SPG_CUDA_TRY(cudaSetDevice(c->device));
    return spmv_autotune(c, const_cast<spg_csr *>(A), reps, times_ms, best);
}

int spg_spgemm_features(spg_ctx *c, const spg_csr *A, const spg_csr *B, float *features) {
    if (!c || !A || !B || !features) return set_error(SPG_ERR_INVALID_ARGUMENT, "spg_spgemm_features: null argument");
    if (A->n_cols != B->n_rows) return set_error(SPG_ERR_INVALID_ARGUMENT, "A.cols must equal B.rows");
    if (!A->built) return set_error(SPG_ERR_LOGIC, "spgemm: A must be locked");
    if (!B->built) return set_error(SPG_ERR_LOGIC, "spgemm: B must be locked");
    SPG_CUDA_TRY(cudaSetDevice(c->device));
    return spgemm_features(c, A, B, features);
}

int spg_spgemm_autotune(spg_ctx *c, const spg_csr *A, const spg_csr *B, int reps, float *times_ms, int *best) {
    if (!c || !A || !B) return set_error(SPG_ERR_INVALID_ARGUMENT, "spg_spgemm_autotune: null argument");
    if (A->n_cols != B->n_rows) return set_error(SPG_ERR_INVALID_ARGUMENT, "A.cols must equal B.rows");
    if (!A->built) return set_error(SPG_ERR_LOGIC, "spgemm: A must be locked");
    if (!B->built) return set_error(SPG_ERR_LOGIC, "spgemm: B must be locked");
    SPG_CUDA_TRY(cudaSetDevice(c->device));
    return spgemm_autotune(c, A, B, reps, times_ms, best);
}

int spg_spgemm_selected(spg_ctx *c, const spg_csr *A, const spg_csr *B, int *variant) {
    if (!c || !A || !B || !variant) return set_error(SPG_ERR_INVALID_ARGUMENT, "spg_spgemm_selected: null argument");
    if (A->n_cols != B->n_rows) return set_error(SPG_ERR_INVALID_ARGUMENT, "A.cols must equal B.rows");
    if (!A->built) return set_error(SPG_ERR_LOGIC, "spgemm: A must be locked");
    if (!B->built) return set_error(SPG_ERR_LOGIC, "spgemm: B must be locked");
    SPG_CUDA_TRY(cudaSetDevice(c->device));
    return spgemm_resolve_auto(c, A, B, variant);
}

int spg_set_spgemm_policy(spg_ctx *c, int policy) {
    if (!c) return set_error(SPG_ERR_INVALID_ARGUMENT, "spg_set_spgemm_policy: null context");
    if (policy < SPG_POLICY_SELECTOR || policy > SPG_POLICY_FIXED)
        return set_error(SPG_ERR_INVALID_ARGUMENT, "spg_set_spgemm_policy: unknown policy %d", policy);
    c->spgemm_policy = policy;
    return SPG_OK;
}

int spg_spgemm_selector_load(spg_ctx *c, const float *blob, uint64_t n_floats, int n_outputs) {
    if (!c) return set_error(SPG_ERR_INVALID_ARGUMENT, "spg_spgemm_selector_load: null context");
    SPG_CUDA_TRY(cudaSetDevice(c->device));
    if (!blob) {
        c->gemm_model.release();
        c->gemm_model_k = 0;
        return SPG_OK;
    }
    if (n_outputs < 1 || n_outputs > SPG_SPGEMM_N_VARIANTS || n_floats != 2 * F + n_params(n_outputs))
        return set_error(SPG_ERR_INVALID_ARGUMENT, "spg_spgemm_selector_load: blob of %llu floats does not fit K=%d",
                         (unsigned long long)n_floats, n_outputs);
    SPG_TRY(c->gemm_model.alloc(n_floats * sizeof(float), c->stream));
    SPG_CUDA_TRY(
        cudaMemcpyAsync(c->gemm_model.ptr, blob, n_floats * sizeof(float), cudaMemcpyHostToDevice, c->stream));
    SPG_CUDA_TRY(cudaStreamSynchronize(c->stream));
    c->gemm_model_k = n_outputs;
    return SPG_OK;
}

int spg_spgemm_selector_predict(spg_ctx *c, const float *d_features, uint32_t B, float *d_out, void *stream) {
    if (!c || (B && (!d_features || !d_out)))
        return set_error(SPG_ERR_INVALID_ARGUMENT, "spg_spgemm_selector_predict: null");
    if (c->gemm_model_k <= 0) return set_error(SPG_ERR_LOGIC, "spg_spgemm_selector_predict: no selector loaded");
    SPG_CUDA_TRY(cudaSetDevice(c->device));
    if (!B) return SPG_OK;
    return selector_predict_dev(c->gemm_model, c->gemm_model_k, d_features, B, d_out, pick_stream(c, stream));
}

int spg_set_spmv_policy(spg_ctx *c, int policy) {
    if (!c) return set_error(SPG_ERR_INVALID_ARGUMENT, "spg_set_spmv_policy: null context");
    if (policy < SPG_POLICY_SELECTOR || policy > SPG_POLICY_FIXED)
        return set_error(SPG_ERR_INVALID_ARGUMENT, "spg_set_spmv_policy: unknown policy %d", policy);
    c->spmv_policy = policy;
    return SPG_OK;
}

int spg_selector_load(spg_ctx *c, const float *blob, uint64_t n_floats, int n_outputs) {
    if (!c) return set_error(SPG_ERR_INVALID_ARGUMENT, "spg_selector_load: null context");
    SPG_CUDA_TRY(cudaSetDevice(c->device));
    if (!blob) {
        c->model.release();
        c->model_k = 0;
        return SPG_OK;
    }
    if (n_outputs < 1 || n_outputs > SPG_SPMV_N_VARIANTS || n_floats != 2 * F + n_params(n_outputs))
        return set_error(SPG_ERR_INVALID_ARGUMENT, "spg_selector_load: blob of %llu floats does not fit K=%d",
                         (unsigned long long)n_floats, n_outputs);
    SPG_TRY(c->model.alloc(n_floats * sizeof(float), c->stream));
    SPG_CUDA_TRY(cudaMemcpyAsync(c->model.ptr, blob, n_floats * sizeof(float), cudaMemcpyHostToDevice, c->stream));
    SPG_CUDA_TRY(cudaStreamSynchronize(c->stream));
    c->model_k = n_outputs;
    return SPG_OK;
}

uint64_t spg_mlp_param_count(int n_outputs) { return n_params(n_outputs); }

int spg_selector_predict(spg_ctx *c, const float *d_features, uint32_t B, float *d_out, void *stream) {
    if (!c || (B && (!d_features || !d_out))) return set_error(SPG_ERR_INVALID_ARGUMENT, "spg_selector_predict: null");
    if (c->model_k <= 0) return set_error(SPG_ERR_LOGIC, "spg_selector_predict: no selector loaded");
    SPG_CUDA_TRY(cudaSetDevice(c->device));
    if (!B) return SPG_OK;
    return selector_predict_dev(c->model, c->model_k, d_features, B, d_out, pick_stream(c, stream));
}

int spg_mlp_forward(spg_ctx *c, const float *d_params, int n_outputs, const float *d_x, uint32_t B, float *d_act,
                    float *d_out, void *stream) {
    if (!c || !d_params || (B && (!d_x || !d_act || !d_out)))
        return set_error(SPG_ERR_INVALID_ARGUMENT, "spg_mlp_forward: null argument");
    SPG_CUDA_TRY(cudaSetDevice(c->device));
    if (!B) return SPG_OK;
    return forward(d_params, n_outputs, d_x, B, d_act, d_out, pick_stream(c, stream));
}

int spg_mlp_backward(spg_ctx *c, const float *d_params, int n_outputs, const float *d_x, uint32_t B,
                     const float *d_act, const float *d_dout, float *d_grad, void *stream) {
    if (!c || !d_params || !d_grad || (B && (!d_x || !d_act || !d_dout)))
        return set_error(SPG_ERR_INVALID_ARGUMENT, "spg_mlp_backward: null argument");
    SPG_CUDA_TRY(cudaSetDevice(c->device));
    cudaStream_t s = pick_stream(c, stream);
    const int K = n_outputs;
    const Layers L = layers(d_params, K);
    float *gW1 = d_grad, *gb1 = gW1 + (uint64_t)H * F, *gW2 = gb1 + H, *gb2 = gW2 + (uint64_t)H * H,
          *gW3 = gb2 + H, *gb3 = gW3 + (uint64_t)K * H;
    const float *h1 = d_act, *h2 = d_act + (uint64_t)B * H;
    DevBuf d2, d1;
    SPG_TRY(d2.alloc((uint64_t)(B ? B : 1) * H * sizeof(float), s));
    SPG_TRY(d1.alloc((uint64_t)(B ? B : 1) * H * sizeof(float), s));
    mlp_back_weights<<<grid_for((uint64_t)K * H + K, 256), 256, 0, s>>>(d_dout, h2, H, K, B, gW3, gb3);
    mlp_back_input<<<grid_for((uint64_t)B * H, 256), 256, 0, s>>>(L.W3, d_dout, H, K, B, h2, d2.as<float>());
    mlp_back_weights<<<grid_for((uint64_t)H * H + H, 256), 256, 0, s>>>(d2.as<float>(), h1, H, H, B, gW2, gb2);
    mlp_back_input<<<grid_for((uint64_t)B * H, 256), 256, 0, s>>>(L.W2, d2.as<float>(), H, H, B, h1, d1.as<float>());
    mlp_back_weights<<<grid_for((uint64_t)H * F + H, 256), 256, 0, s>>>(d1.as<float>(), d_x, F, H, B, gW1, gb1);
    SPG_LAUNCH_CHECK();
    return SPG_OK;
}

int spg_mlp_mse(spg_ctx *c, const float *d_pred, const float *d_target, uint64_t n, float *d_dpred, float *d_loss,
                void *stream) {
    if (!c || (n && (!d_pred || !d_target || !d_dpred)))
        return set_error(SPG_ERR_INVALID_ARGUMENT, "spg_mlp_mse: null argument");
    SPG_CUDA_TRY(cudaSetDevice(c->device));
    if (!n) return SPG_OK;
    mlp_mse_grad<<<grid_for(n, 256), 256, 0, pick_stream(c, stream)>>>(d_pred, d_target, n, d_dpred, d_loss);
    SPG_LAUNCH_CHECK();
    return SPG_OK;
}

int spg_mlp_adam(spg_ctx *c, float *d_params, const float *d_grad, float *d_m, float *d_v, uint64_t n, float lr,
                 float beta1, float beta2, float eps, uint32_t step, void *stream) {
    if (!c || !d_params || !d_grad || !d_m || !d_v || step == 0)
        return set_error(SPG_ERR_INVALID_ARGUMENT, "spg_mlp_adam: bad argument");
    SPG_CUDA_TRY(cudaSetDevice(c->device));
    const float c1 = 1.0f - std::pow(beta1, (float)step), c2 = 1.0f - std::pow(beta2, (float)step);
    mlp_adam<<<grid_for(n, 256), 256, 0, pick_stream(c, stream)>>>(d_params, d_grad, d_m, d_v, n, lr, beta1, beta2,
                                                                    eps, c1, c2);
    SPG_LAUNCH_CHECK();
    return SPG_OK;
}

int spg_mlp_argmin(spg_ctx *c, const float *d_pred, uint32_t B, int n_outputs, int *d_best, void *stream) {
    if (!c || (B && (!d_pred || !d_best))) return set_error(SPG_ERR_INVALID_ARGUMENT, "spg_mlp_argmin: null");
    SPG_CUDA_TRY(cudaSetDevice(c->device));
    if (!B) return SPG_OK;
    mlp_argmin<<<grid_for(B, 256), 256, 0, pick_stream(c, stream)>>>(d_pred, B, n_outputs, d_best);
    SPG_LAUNCH_CHECK();
    return SPG_OK;
}

int spg_probe_gather_rate(spg_ctx *c, uint64_t n_x, uint64_t n_gathers, double *gathers_per_s) {
    if (!c || !gathers_per_s) return set_error(SPG_ERR_INVALID_ARGUMENT, "spg_probe_gather_rate: null argument");
    if (n_x == 0 || (n_x & (n_x - 1)) || n_x > (1ull << 32))
        return set_error(SPG_ERR_INVALID_ARGUMENT, "spg_probe_gather_rate: n_x must be a power of two <= 2^32");
    const uint64_t n_thr = n_gathers / GATHER_PER_THREAD;
    if (n_thr == 0 || n_thr > (1ull << 32))
        return set_error(SPG_ERR_INVALID_ARGUMENT, "spg_probe_gather_rate: n_gathers out of range");
    SPG_CUDA_TRY(cudaSetDevice(c->device));
    cudaStream_t s = c->stream;
    DevBuf x, out;
    SPG_TRY(x.alloc(n_x * sizeof(double), s));
    SPG_TRY(out.alloc(n_thr * sizeof(double), s));
    SPG_CUDA_TRY(cudaMemsetAsync(x.ptr, 0, n_x * sizeof(double), s));
    cudaEvent_t e0, e1;
    SPG_CUDA_TRY(cudaEventCreate(&e0));
    SPG_CUDA_TRY(cudaEventCreate(&e1));
    std::vector<float> ts;
    int rc = SPG_OK;
    for (int r = 0; r < 7 && rc == SPG_OK; ++r) {
        cudaEventRecord(e0, s);
        gather_probe<<<grid_for(n_thr, 256), 256, 0, s>>>(x.as<double>(), (uint32_t)(n_x - 1), out.as<double>(),
                                                          n_thr);
        cudaEventRecord(e1, s);
        if (cudaEventSynchronize(e1) != cudaSuccess) rc = set_error(SPG_ERR_CUDA, "gather probe: event sync failed");
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (r >= 2) ts.push_back(ms);  // two warm-up runs
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    SPG_TRY(rc);
    SPG_LAUNCH_CHECK();
    std::sort(ts.begin(), ts.end());
    *gathers_per_s = (double)(n_thr * GATHER_PER_THREAD) / (ts[ts.size() / 2] * 1e-3);
    return SPG_OK;
}

int spg_probe_gather_rate_cfg(spg_ctx *c, uint64_t n_x, uint64_t n_gathers, int per_thread, int blocks_per_sm,
                              double *gathers_per_s, int *resident_blocks_per_sm) {
    if (!c || !gathers_per_s) return set_error(SPG_ERR_INVALID_ARGUMENT, "spg_probe_gather_rate_cfg: null argument");
    if (n_x == 0 || (n_x & (n_x - 1)) || n_x > (1ull << 32))
        return set_error(SPG_ERR_INVALID_ARGUMENT, "spg_probe_gather_rate_cfg: n_x must be a power of two <= 2^32");
    if (blocks_per_sm < 1 || blocks_per_sm > 64)
        return set_error(SPG_ERR_INVALID_ARGUMENT, "spg_probe_gather_rate_cfg: blocks_per_sm must be in [1, 64]");
    const void *fn = nullptr;
    switch (per_thread) {
        case 1: fn = (const void *)gather_probe_cfg<1>; break;
        case 2: fn = (const void *)gather_probe_cfg<2>; break;
        case 4: fn = (const void *)gather_probe_cfg<4>; break;
        case 8: fn = (const void *)gather_probe_cfg<8>; break;
        case 16: fn = (const void *)gather_probe_cfg<16>; break;
        case 32: fn = (const void *)gather_probe_cfg<32>; break;
        case 64: fn = (const void *)gather_probe_cfg<64>; break;
        default:
            return set_error(SPG_ERR_INVALID_ARGUMENT, "spg_probe_gather_rate_cfg: per_thread must be 1, 2, ..., 64");
    }
    const uint64_t n_iter = n_gathers / (uint64_t)per_thread;
    if (n_iter == 0 || n_iter > (1ull << 32))
        return set_error(SPG_ERR_INVALID_ARGUMENT, "spg_probe_gather_rate_cfg: n_gathers out of range");
    SPG_CUDA_TRY(cudaSetDevice(c->device));
    int resident = 0;
    SPG_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&resident, fn, 256, 0));
    if (resident_blocks_per_sm) *resident_blocks_per_sm = std::min(resident, blocks_per_sm);
    cudaStream_t s = c->stream;
    const unsigned grid = (unsigned)(blocks_per_sm * c->n_sms);
    DevBuf x, out;
    SPG_TRY(x.alloc(n_x * sizeof(double), s));
    SPG_TRY(out.alloc((uint64_t)grid * 256 * sizeof(double), s));
    SPG_CUDA_TRY(cudaMemsetAsync(x.ptr, 0, n_x * sizeof(double), s));
    const double *xp = x.as<double>();
    uint32_t mask = (uint32_t)(n_x - 1);
    double *op = out.as<double>();
    void *args[] = {(void *)&xp, (void *)&mask, (void *)&op, (void *)&n_iter};
    cudaEvent_t e0, e1;
    SPG_CUDA_TRY(cudaEventCreate(&e0));
    SPG_CUDA_TRY(cudaEventCreate(&e1));
    std::vector<float> ts;
    int rc = SPG_OK;
    for (int r = 0; r < 7 && rc == SPG_OK; ++r) {
        cudaEventRecord(e0, s);
        if (cudaLaunchKernel(fn, dim3(grid), dim3(256), args, 0, s) != cudaSuccess)
            rc = set_error(SPG_ERR_CUDA, "gather probe: launch failed");
        cudaEventRecord(e1, s);
        if (rc == SPG_OK && cudaEventSynchronize(e1) != cudaSuccess)
            rc = set_error(SPG_ERR_CUDA, "gather probe: event sync failed");
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (r >= 2) ts.push_back(ms);  // two warm-up runs
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    SPG_TRY(rc);
    SPG_LAUNCH_CHECK();
    std::sort(ts.begin(), ts.end());
    *gathers_per_s = (double)(n_iter * (uint64_t)per_thread) / (ts[ts.size() / 2] * 1e-3);
    return SPG_OK;
}

int spg_probe_fp64_rate(spg_ctx *c, uint32_t iters, double *fma_per_s) {
    if (!c || !fma_per_s) return set_error(SPG_ERR_INVALID_ARGUMENT, "spg_probe_fp64_rate: null argument");
    if (iters < 16 || iters > (1u << 20))
        return set_error(SPG_ERR_INVALID_ARGUMENT, "spg_probe_fp64_rate: iters must be in [16, 2^20]");
    SPG_CUDA_TRY(cudaSetDevice(c->device));
    cudaStream_t s = c->stream;
    const unsigned grid = (unsigned)(8 * c->n_sms);
    DevBuf out;
    SPG_TRY(out.alloc((uint64_t)grid * 256 * sizeof(double), s));
    cudaEvent_t e0, e1;
    SPG_CUDA_TRY(cudaEventCreate(&e0));
    SPG_CUDA_TRY(cudaEventCreate(&e1));
    std::vector<float> ts;
    int rc = SPG_OK;
    for (int r = 0; r < 7 && rc == SPG_OK; ++r) {
        cudaEventRecord(e0, s);
        fma_probe<<<grid, 256, 0, s>>>(0.999999, 1e-3, iters, out.as<double>());
        cudaEventRecord(e1, s);
        if (cudaEventSynchronize(e1) != cudaSuccess) rc = set_error(SPG_ERR_CUDA, "fp64 probe: event sync failed");
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (r >= 2) ts.push_back(ms);  // two warm-up runs
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    SPG_TRY(rc);
    SPG_LAUNCH_CHECK();
    std::sort(ts.begin(), ts.end());
    *fma_per_s = (double)grid * 256.0 * FMA_CHAINS * iters / (ts[ts.size() / 2] * 1e-3);
    return SPG_OK;
}

}  // extern "C"
