"""The learned selector: FP64 reference gradients (CPU), libspg's FP32 MLP
kernels against them (GPU), features, the autotuner, and a small end-to-end
training run showing what the trained network gains over the fixed default."""
from __future__ import annotations

import numpy as np
import pytest

from spira_gb300 import selector as S

K = S.K


def test_fp64_reference_gradient_is_the_derivative():
    rng = np.random.default_rng(0)
    P = S.init_params(K, seed=1).astype(np.float64)
    X = rng.standard_normal((7, 40))
    T = rng.standard_normal((7, K))

    def loss(p):
        out, _ = S.forward_ref(p, X, K)
        return np.mean((out - T) ** 2)

    out, _ = S.forward_ref(P, X, K)
    dout = 2 * (out - T) / out.size
    g = S.backward_ref(P, X, dout, K)
    for idx in rng.choice(len(P), 40, replace=False):
        e = np.zeros_like(P)
        e[idx] = 1e-6
        fd = (loss(P + e) - loss(P - e)) / 2e-6
        assert abs(fd - g[idx]) <= 1e-6 + 1e-5 * abs(fd), (idx, fd, g[idx])


def test_corpus_specs_are_deterministic_and_bounded():
    for i in range(200):
        a, b = S.corpus_spec(i, 7), S.corpus_spec(i, 7)
        assert a == b
        assert 1 <= a.n_rows <= 4_000_000
    fams = {S.corpus_spec(i, 7).family for i in range(200)}
    assert len(fams) >= 5


@pytest.mark.gpu
def test_mlp_kernels_match_fp64(ctx):
    import torch
    import spira_gb300 as sg
    rng = np.random.default_rng(3)
    B = 37
    P = S.init_params(K, seed=2)
    P[-K:] = rng.standard_normal(K).astype(np.float32) * 0.1  # non-zero output biases
    X = rng.standard_normal((B, 40)).astype(np.float32)
    Y = rng.standard_normal((B, K)).astype(np.float32)
    mlp = sg.Mlp(ctx, K)
    Pd, Xd, Yd = (torch.from_numpy(a).cuda() for a in (P, X.ravel(), Y.ravel()))
    act = torch.empty(B * 128, device="cuda")
    out = torch.empty(B * K, device="cuda")
    dout = torch.empty(B * K, device="cuda")
    G = torch.empty_like(Pd)
    loss = torch.zeros(1, device="cuda")
    torch.cuda.synchronize()
    mlp.forward(Pd, Xd, act, out, B)
    mlp.mse(out, Yd, B * K, dout, loss)
    mlp.backward(Pd, Xd, act, dout, G, B)
    ctx.sync()
    ref_out, _ = S.forward_ref(P, X.astype(np.float64), K)
    np.testing.assert_allclose(out.cpu().numpy().reshape(B, K), ref_out, rtol=1e-4, atol=1e-5)
    ref_dout = 2 * (ref_out - Y) / ref_out.size
    np.testing.assert_allclose(dout.cpu().numpy().reshape(B, K), ref_dout, rtol=1e-4, atol=1e-7)
    assert abs(loss.item() - np.mean((ref_out - Y) ** 2)) <= 1e-4 * np.mean((ref_out - Y) ** 2)
    g_ref = S.backward_ref(P, X.astype(np.float64), ref_dout, K)
    g = G.cpu().numpy()
    scale = np.abs(g_ref).max()
    assert np.max(np.abs(g - g_ref)) <= 1e-4 * scale


@pytest.mark.gpu
def test_adam_step_matches_numpy(ctx):
    import torch
    import spira_gb300 as sg
    rng = np.random.default_rng(4)
    mlp = sg.Mlp(ctx, K)
    n = mlp.n_params
    w = rng.standard_normal(n).astype(np.float32)
    g = rng.standard_normal(n).astype(np.float32)
    m = np.zeros(n, np.float32)
    v = np.zeros(n, np.float32)
    wd, gd, md, vd = (torch.from_numpy(a.copy()).cuda() for a in (w, g, m, v))
    torch.cuda.synchronize()
    mlp.adam(wd, gd, md, vd, 1e-2, 1)
    ctx.sync()
    m1 = 0.1 * g
    v1 = 0.001 * g * g
    w1 = w - 1e-2 * (m1 / 0.1) / (np.sqrt(v1 / 0.001) + 1e-8)
    np.testing.assert_allclose(wd.cpu().numpy(), w1, rtol=1e-5, atol=1e-6)


@pytest.mark.gpu
def test_features_match_host(ctx):
    import spira_gb300 as sg
    from spira_gb300 import gen
    r, c, v = gen.zipf_rows(30_000, seed=5)
    A = sg.Csr(ctx, 30_000, 30_000)
    A.lock(r, c, v)
    f = A.features()
    H = A.download()
    L = np.diff(H.off.astype(np.int64))
    hist = np.zeros(32)
    for Lr in L:
        b = 0 if Lr == 0 else min(31, 1 + int(np.floor(np.log2(Lr))))
        hist[b] += 1
    np.testing.assert_allclose(f[:32], hist / len(L), atol=1e-6)
    assert abs(f[35] - np.log2(L.mean() + 1) / 16) < 1e-5
    assert abs(f[37] - np.log2(L.max() + 1) / 32) < 1e-5


@pytest.mark.gpu
def test_autotune_reports_every_variant(ctx):
    import spira_gb300 as sg
    from spira_gb300 import gen
    r, c, v = gen.laplacian_2d(300)
    A = sg.Csr(ctx, 90_000, 90_000)
    A.lock(r, c, v)
    t, best = A.autotune(3)
    assert len(t) == K and np.all(t > 0) and best == int(np.argmin(t))


@pytest.mark.gpu
def test_small_training_run_beats_fixed_default(ctx):
    """Trains on a small corpus; on held-out matrices the variants the trained
    network picks must take strictly less total time than the fixed default
    (the method without the network)."""
    import spira_gb300 as sg
    X, T, specs = S.collect(ctx, range(120), seed=11, reps=2)
    blob, hist = S.train(ctx, X[:100], T[:100], epochs=150, batch=64, lr=3e-3)
    assert hist[-1] < hist[0]
    pred = S.predict(ctx, blob, X[100:])
    ev = S.evaluate(T[100:], pred.argmin(axis=1), S.DEFAULT_SPMV)
    assert ev["total_time_ratio"] < ev["default_total_time_ratio"], ev
    # AUTO through the installed selector picks a valid variant
    A = S.build(ctx, specs[100])
    ctx.set_spmv_policy(sg.POLICY_SELECTOR)
    assert 0 <= A.selected_spmv() < K
    ctx.load_selector(None, 0)


@pytest.mark.gpu
def test_small_spgemm_training_run_beats_fixed_default(ctx):
    """The same for the SpGEMM selector (C = A * A on the SpGEMM corpus)."""
    import spira_gb300 as sg
    X, T, specs = S.collect(ctx, range(90), seed=13, reps=1, op="spgemm")
    assert T.shape == (90, S.K_GEMM)
    blob, hist = S.train(ctx, X[:70], T[:70], epochs=150, batch=32, lr=3e-3)
    assert hist[-1] < hist[0]
    pred = S.predict(ctx, blob, X[70:], op="spgemm")
    ev = S.evaluate(T[70:], pred.argmin(axis=1), S.DEFAULT_SPGEMM)
    assert ev["total_time_ratio"] < ev["default_total_time_ratio"], ev
    A = S.build(ctx, S.gemm_corpus_spec(70, 13))
    ctx.set_spgemm_policy(sg.POLICY_SELECTOR)
    assert 0 <= A.spgemm_selected(A) < S.K_GEMM
    ctx.load_spgemm_selector(None, 0)


@pytest.mark.gpu
@pytest.mark.parametrize("op, first, n, bound", [("spmv", 20_000, 60, 1.05), ("spgemm", 4_000, 40, 1.10)])
def test_shipped_selector_on_unseen_matrices(ctx, op, first, n, bound):
    """The shipped model, on corpus matrices past its training range: total
    time within `bound` of exhaustive autotuning, and below the fixed
    default's."""
    import spira_gb300 as sg
    path = sg._PKG / ("spg_selector.bin" if op == "spmv" else "spg_spgemm_selector.bin")
    blob = np.fromfile(path, dtype=np.float32)
    assert S.blob_outputs(blob) == (S.K if op == "spmv" else S.K_GEMM)
    X, T, _ = S.collect(ctx, range(first, first + n), seed=7, reps=2, op=op)
    ev = S.evaluate(T, S.predict(ctx, blob, X, op=op).argmin(axis=1),
                    S.DEFAULT_SPMV if op == "spmv" else S.DEFAULT_SPGEMM)
    assert ev["total_time_ratio"] <= bound, ev
    assert ev["total_time_ratio"] < ev["default_total_time_ratio"], ev


@pytest.mark.gpu
def test_spgemm_selector_skips_dominated_variants(ctx):
    """SPG_SPGEMM_AUTO with the shipped model never picks a WARPSORT variant
    whose rows a smaller one takes with less shared memory: uniform rows of 8
    (64 products per row) rule out _128 and _256, rows of 10 (up to 100) _256."""
    import spira_gb300 as sg
    from spira_gb300 import gen
    for k, ruled_out in ((8, {sg.SPGEMM_VARIANTS["warpsort_128"], sg.SPGEMM_VARIANTS["warpsort_256"]}),
                         (10, {sg.SPGEMM_VARIANTS["warpsort_256"]})):
        n = 50_000
        r, c, v = gen.uniform_rows(n, n, k, seed=77 + k)
        A = sg.Csr(ctx, n, n)
        A.lock(r, c, v)
        assert A.spgemm_selected(A) not in ruled_out
        A.close()
