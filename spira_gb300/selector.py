"""The learned variant selectors (SpMV and SpGEMM).

A small FP32 MLP (40 -> 64 -> 64 -> K) reads 40 features of a locked matrix
(SpMV: 32-bin log2 row-length histogram + 8 shape statistics; SpGEMM of
A * A: 32-bin log2 histogram of the products per row + 8 statistics; both
computed on the device) and predicts, for each of the K candidates — SpMV
(variant, tile) pairs or SpGEMM variants — log(time / fastest time).
SPG_SPMV_AUTO / SPG_SPGEMM_AUTO then take the argmin. The networks are
trained on the GPU with libspg's own forward / backward / Adam kernels on
timings that the exhaustive autotuners (spg_spmv_autotune,
spg_spgemm_autotune) measure on a generated corpus; the autotuners stay the
fallback and the yardstick (regret is reported against them).

Corpus: five families (banded with bandwidth 3..201, block-diagonal with
blocks 4..64, power-law with Zipf alpha 1.5..2.5, uniform-random with
4..64 nonzeros per row, 2D / 3D stencils), row counts log-uniform in
[1e3, 4e6], nonzeros capped per matrix (NNZ_CAP for SpMV, GEMM_NNZ_CAP for
SpGEMM, whose products grow with the row lengths; rows are scaled down to
fit), FP64 values. Matrix i of a corpus is a pure function of (seed, i).
"""
from __future__ import annotations

import math
import time
from dataclasses import dataclass

import numpy as np

from . import (FAM_BANDED, FAM_BLOCKDIAG, FAM_POWERLAW, FAM_STENCIL2D, FAM_STENCIL3D, FAM_UNIFORM, N_FEATURES,
               N_HIDDEN, SPGEMM_VARIANTS, SPMV_VARIANTS, Context, Csr, Mlp, gen_family)
from . import gen

K = len(SPMV_VARIANTS)
K_GEMM = len(SPGEMM_VARIANTS)
NNZ_CAP = 64_000_000
GEMM_NNZ_CAP = 2_000_000
# fixed variants "without the selector": the comparison a gain is measured against
DEFAULT_SPMV = SPMV_VARIANTS["adaptive16"]
DEFAULT_SPGEMM = SPGEMM_VARIANTS["rowmerge"]
FAMILY_NAMES = ["banded", "blockdiag", "powerlaw", "uniform", "stencil"]


@dataclass
class Spec:
    family: int
    n_rows: int
    p: int
    ls: float = 0.0
    alpha: float = 0.0
    seed: int = 0

    @property
    def name(self) -> str:
        return f"{self.family}:{self.n_rows}:{self.p}:{self.alpha:.3f}"


def corpus_spec(i: int, seed: int, nnz_cap: int = NNZ_CAP) -> Spec:
    """Matrix i of the corpus drawn with `seed`."""
    u = gen.unit(gen.hash3(seed, 50 + i % 7, np.arange(i * 8, i * 8 + 8, dtype=np.uint64)))
    fam = int(u[0] * 5)
    n = int(round(math.exp(math.log(1e3) + u[1] * (math.log(4e6) - math.log(1e3)))))
    s = int(gen.hash3(seed, 60, np.array([i], np.uint64))[0] & np.uint64(0x7FFFFFFF))
    if fam == 0:
        bw = 3 + 2 * int(u[2] * 100)  # 3..201, odd
        n = max(bw, min(n, nnz_cap // bw))
        return Spec(FAM_BANDED, n, bw, seed=s)
    if fam == 1:
        b = 4 + int(u[2] * 61)  # 4..64
        n = max(b, min(n, nnz_cap // b))
        return Spec(FAM_BLOCKDIAG, n, b, seed=s)
    if fam == 2:
        alpha = 1.5 + u[2]  # 1.5..2.5
        cap = 10_000
        mean_target = 4.0 + u[3] * 28.0
        n = min(n, int(nnz_cap / mean_target))
        return Spec(FAM_POWERLAW, max(n, 16), cap, ls=mean_target, alpha=float(alpha), seed=s)
    if fam == 3:
        k = 4 + int(u[2] * 61)  # 4..64
        n = max(k, min(n, nnz_cap // k))
        return Spec(FAM_UNIFORM, n, k, seed=s)
    if u[2] < 0.5:  # 2D 5-point on side g
        g = max(4, int(round(math.sqrt(min(n, nnz_cap // 5)))))
        return Spec(FAM_STENCIL2D, g * g, g, seed=s)
    g = max(3, int(round(min(n, nnz_cap // 7) ** (1.0 / 3.0))))
    return Spec(FAM_STENCIL3D, g ** 3, g, seed=s)


def gemm_corpus_spec(i: int, seed: int) -> Spec:
    """Matrix i of the SpGEMM corpus (C = A * A): the same families with
    nonzeros capped at GEMM_NNZ_CAP."""
    return corpus_spec(i, seed, GEMM_NNZ_CAP)


def build(ctx: Context, spec: Spec) -> Csr:
    """Generate the staged inserts on the device and lock them into a CSR."""
    import torch
    cdf_t = None
    ls = spec.ls
    if spec.family == FAM_POWERLAW:
        k = np.arange(1, spec.p + 1, dtype=np.float64)
        pk = k ** (-spec.alpha)
        cdf = np.cumsum(pk) / pk.sum()
        ls = spec.ls / float((k * pk).sum() / pk.sum())  # scale so that the mean length is spec.ls
        cdf_t = torch.from_numpy(cdf).cuda()
        torch.cuda.synchronize()
    m = gen_family(ctx, spec.family, spec.n_rows, spec.p, ls, cdf_t, spec.seed)
    rows = torch.empty(max(m, 1), dtype=torch.int32, device="cuda")
    cols = torch.empty(max(m, 1), dtype=torch.int32, device="cuda")
    vals = torch.empty(max(m, 1), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    gen_family(ctx, spec.family, spec.n_rows, spec.p, ls, cdf_t, spec.seed, rows, cols, vals)
    A = Csr(ctx, spec.n_rows, spec.n_rows)
    A.lock_device(rows, cols, vals, m)
    return A


def collect(ctx: Context, indices, seed: int, reps: int = 3, log_every: int = 0, op: str = "spmv",
            time_cap_s: float | None = None):
    """(features [n, 40] float32, times [n, K] float32, specs) for corpus
    matrices `indices`, labelled by the exhaustive autotuner of `op`
    ("spmv": the SpMV (variant, tile) candidates of A; "spgemm": the SpGEMM
    variants of A * A). Stops early once time_cap_s seconds have passed."""
    X, T, S = [], [], []
    t0 = time.time()
    for j, i in enumerate(indices):
        if time_cap_s is not None and time.time() - t0 > time_cap_s:
            break
        spec = corpus_spec(int(i), seed) if op == "spmv" else gemm_corpus_spec(int(i), seed)
        A = build(ctx, spec)
        if op == "spmv":
            X.append(A.features())
            t, _ = A.autotune(reps)
        else:
            X.append(A.spgemm_features(A))
            t, _ = A.spgemm_autotune(A, reps)
        T.append(t)
        S.append(spec)
        A.close()
        if log_every and (j + 1) % log_every == 0:
            print(f"  corpus {j + 1}/{len(indices)}  {time.time() - t0:.1f}s", flush=True)
    return np.array(X, np.float32).reshape(-1, N_FEATURES), np.array(T, np.float32), S


def features_of(ctx: Context, indices, seed: int, op: str = "spmv") -> np.ndarray:
    """Features [n, 40] of corpus matrices `indices` (no timing)."""
    X = []
    for i in indices:
        A = build(ctx, corpus_spec(int(i), seed) if op == "spmv" else gemm_corpus_spec(int(i), seed))
        X.append(A.features() if op == "spmv" else A.spgemm_features(A))
        A.close()
    return np.array(X, np.float32).reshape(-1, N_FEATURES)


def targets(times: np.ndarray) -> np.ndarray:
    """log(t_k / min_k t_k) per matrix."""
    t = np.maximum(times, 1e-6)
    return np.log(t / t.min(axis=1, keepdims=True)).astype(np.float32)


def init_params(n_outputs: int, seed: int = 0) -> np.ndarray:
    rng = np.random.default_rng(seed)
    F, H = N_FEATURES, N_HIDDEN

    def he(o, i):
        return (rng.standard_normal((o, i)) * math.sqrt(2.0 / i)).astype(np.float32)

    parts = [he(H, F), np.zeros(H, np.float32), he(H, H), np.zeros(H, np.float32),
             he(n_outputs, H) * 0.1, np.zeros(n_outputs, np.float32)]
    return np.concatenate([p.ravel() for p in parts])


def normalization(X: np.ndarray):
    mean = X.mean(axis=0)
    sd = X.std(axis=0)
    scale = np.where(sd > 1e-6, 1.0 / np.maximum(sd, 1e-6), 1.0)
    return mean.astype(np.float32), scale.astype(np.float32)


def train(ctx: Context, X: np.ndarray, T: np.ndarray, epochs: int = 400, batch: int = 512, lr: float = 3e-3,
          seed: int = 0, log_every: int = 0):
    """Train on the GPU with libspg's kernels (K = T's columns); returns
    (blob, loss history)."""
    import torch
    K = T.shape[1]
    mlp = Mlp(ctx, K)
    mean, scale = normalization(X)
    Xn = ((X - mean) * scale).astype(np.float32)
    Y = targets(T)
    dev = "cuda"
    Xd = torch.from_numpy(Xn).to(dev)
    Yd = torch.from_numpy(Y).to(dev)
    P = torch.from_numpy(init_params(K, seed)).to(dev)
    G = torch.zeros_like(P)
    Mo = torch.zeros_like(P)
    Vo = torch.zeros_like(P)
    n = len(Xn)
    bmax = min(batch, n)
    act = torch.empty(bmax * 2 * N_HIDDEN, dtype=torch.float32, device=dev)
    out = torch.empty(bmax * K, dtype=torch.float32, device=dev)
    dout = torch.empty_like(out)
    loss = torch.zeros(1, dtype=torch.float32, device=dev)
    rng = np.random.default_rng(seed + 1)
    hist = []
    step = 0
    torch.cuda.synchronize()
    for ep in range(epochs):
        perm = torch.from_numpy(rng.permutation(n)).to(dev)
        loss.zero_()
        nb = 0
        for b0 in range(0, n, bmax):
            idx = perm[b0:b0 + bmax]
            B = len(idx)
            xb = Xd[idx].contiguous()
            yb = Yd[idx].contiguous()
            torch.cuda.synchronize()
            mlp.forward(P, xb, act, out, B)
            mlp.mse(out, yb, B * K, dout, loss)
            mlp.backward(P, xb, act, dout, G, B)
            step += 1
            mlp.adam(P, G, Mo, Vo, lr, step)
            ctx.sync()
            nb += 1
        hist.append(float(loss.item()) / nb)
        if log_every and (ep + 1) % log_every == 0:
            print(f"  epoch {ep + 1}: loss {hist[-1]:.4f}", flush=True)
    blob = np.concatenate([mean, scale, P.cpu().numpy()]).astype(np.float32)
    return blob, hist


def blob_outputs(blob: np.ndarray) -> int:
    """K of a selector blob [mean, scale, W1, b1, W2, b2, W3, b3]."""
    base = 2 * N_FEATURES + N_HIDDEN * N_FEATURES + N_HIDDEN + N_HIDDEN * N_HIDDEN + N_HIDDEN
    return (len(blob) - base) // (N_HIDDEN + 1)


def predict(ctx: Context, blob: np.ndarray, X: np.ndarray, op: str = "spmv") -> np.ndarray:
    """Predicted log-time ratios [n, K] via the loaded-selector inference path
    (installs the blob as the context's `op` selector)."""
    import torch
    from . import _check, _ptr, lib
    Kb = blob_outputs(blob)
    if op == "spmv":
        ctx.load_selector(blob, Kb)
    else:
        ctx.load_spgemm_selector(blob, Kb)
    Xd = torch.from_numpy(np.ascontiguousarray(X, np.float32)).cuda()
    out = torch.empty(max(len(X), 1) * Kb, dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    fn = lib().spg_selector_predict if op == "spmv" else lib().spg_spgemm_selector_predict
    _check(fn(ctx.h, _ptr(Xd), len(X), _ptr(out), None))
    ctx.sync()
    return out.cpu().numpy()[:len(X) * Kb].reshape(len(X), Kb)


def evaluate(T: np.ndarray, choice: np.ndarray, default: int) -> dict:
    """Regret of `choice` against the exhaustive-autotune best on timings T,
    and of the fixed `default` (the method without the selector)."""
    n = len(T)
    best = T.min(axis=1)
    t_choice = T[np.arange(n), choice]
    t_default = T[:, default]
    return {
        "n": int(n),
        "top1": float(np.mean(choice == T.argmin(axis=1))),
        "mean_regret": float(np.mean(t_choice / best - 1.0)),
        "p95_regret": float(np.quantile(t_choice / best - 1.0, 0.95)),
        "total_time_ratio": float(t_choice.sum() / best.sum()),        # learned vs exhaustive
        "default_total_time_ratio": float(t_default.sum() / best.sum()),  # fixed default vs exhaustive
        "default_mean_regret": float(np.mean(t_default / best - 1.0)),
    }


# ---------------------------------------------------------------- FP64 reference
def forward_ref(params: np.ndarray, X: np.ndarray, n_outputs: int):
    """FP64 forward of the same network (for gradient checks)."""
    F, H, Kk = N_FEATURES, N_HIDDEN, n_outputs
    p = params.astype(np.float64)
    o = 0
    W1 = p[o:o + H * F].reshape(H, F); o += H * F
    b1 = p[o:o + H]; o += H
    W2 = p[o:o + H * H].reshape(H, H); o += H * H
    b2 = p[o:o + H]; o += H
    W3 = p[o:o + Kk * H].reshape(Kk, H); o += Kk * H
    b3 = p[o:o + Kk]
    z1 = X @ W1.T + b1
    h1 = np.maximum(z1, 0)
    z2 = h1 @ W2.T + b2
    h2 = np.maximum(z2, 0)
    out = h2 @ W3.T + b3
    return out, (W1, W2, W3, h1, h2, z1, z2)


def backward_ref(params: np.ndarray, X: np.ndarray, dout: np.ndarray, n_outputs: int) -> np.ndarray:
    out, (W1, W2, W3, h1, h2, z1, z2) = forward_ref(params, X, n_outputs)
    gW3 = dout.T @ h2
    gb3 = dout.sum(axis=0)
    d2 = (dout @ W3) * (z2 > 0)
    gW2 = d2.T @ h1
    gb2 = d2.sum(axis=0)
    d1 = (d2 @ W2) * (z1 > 0)
    gW1 = d1.T @ X
    gb1 = d1.sum(axis=0)
    return np.concatenate([gW1.ravel(), gb1, gW2.ravel(), gb2, gW3.ravel(), gb3])
