"""SpMV on the GPU, every variant, against the oracle and Spira's golden
outputs. FP64 tolerance (written here, the project's stated FP64 bound): per row
|y - y_ref| <= 1e-12 * sum_k |a_rk x_k|; the compensated oracle gives y_ref
to ~2 ulp, and Spira's own SIMD path is held to the same bound."""
from __future__ import annotations

import json
from pathlib import Path

import numpy as np
import pytest

import oracle
import spira_gb300 as sg
from spira_gb300 import gen
from conftest import SPMV_TOL, spmv_rel_err

pytestmark = pytest.mark.gpu

GOLD = json.loads((Path(__file__).parent / "golden" / "golden.json").read_text())
GOLD_Y = np.load(Path(__file__).parent / "golden" / "golden_y.npz")
VARIANTS = list(sg.SPMV_VARIANTS.items()) + [("auto", sg.SPMV_AUTO)]


def build(ctx, n_rows, n_cols, epochs):
    A = sg.Csr(ctx, n_rows, n_cols)
    for r, c, v in epochs:
        A.lock(r, c, v)
    return A


def check_all_variants(A, x, host=None):
    host = host or A.download()
    y_ref, scale = oracle.spmv_compensated(host, x)
    errs = {}
    for name, v in VARIANTS:
        y = A.spmv_host(x, variant=v)
        errs[name] = spmv_rel_err(y, y_ref, scale)
        assert errs[name] <= SPMV_TOL, (name, errs[name])
    return errs


def _csr_from_rows(lengths, n_cols, seed):
    lengths = np.asarray(lengths, np.int64)
    rows = np.repeat(np.arange(len(lengths), dtype=np.uint32), lengths)
    ctr = np.arange(len(rows), dtype=np.uint64)
    cols = gen.below(gen.hash3(seed, 1, ctr), n_cols)
    vals = gen.sym_unit(gen.hash3(seed, 2, ctr))
    return rows, cols, vals


@pytest.mark.parametrize("lengths", [
    [0],
    [1],
    [0, 0, 0, 5, 0],
    [3] * 1000,
    [5000],                                  # one long row
    [1023, 1024, 1025, 2046, 2047, 2048, 2049, 1, 0, 7],  # around the STREAM thresholds
    [0] * 5000 + [40_000] + [0] * 5000,      # a long row between empty stretches
    list(range(0, 3000, 7)),                 # ramp
    [1] * 3000 + [10_000] * 3 + [2] * 3000,
])
def test_spmv_edge_shapes(ctx, lengths):
    n_cols = 70_000
    r, c, v = _csr_from_rows(lengths, n_cols, seed=len(lengths))
    A = build(ctx, len(lengths), n_cols, [(r, c, v)])
    x = gen.dense_x(n_cols, 1)
    check_all_variants(A, x)


def test_spmv_empty_rows_give_exact_zero(ctx):
    r, c, v = _csr_from_rows([0, 3, 0, 0, 2, 0], 10, seed=3)
    A = build(ctx, 6, 10, [(r, c, v)])
    for name, var in VARIANTS:
        y = A.spmv_host(np.full(10, 2.5), variant=var)
        assert y[0] == 0.0 and y[2] == 0.0 and y[3] == 0.0 and y[5] == 0.0, name


@pytest.mark.parametrize("rec", GOLD["workloads"], ids=[w["name"] for w in GOLD["workloads"]])
def test_spmv_matches_spira_golden(ctx, rec):
    """Against y produced by Spira's own sparse_dot_double path."""
    from test_oracle_pin import _workloads
    name, nr, nc, ep, x = _workloads()[rec["name"]]
    A = build(ctx, nr, nc, ep)
    host = A.download()
    assert oracle.csr_digest(host) == rec["csr_sha256"]
    y_spira = GOLD_Y[rec["name"] + "__y"]
    _, scale = oracle.spmv_compensated(host, x)
    for vname, v in VARIANTS:
        y = A.spmv_host(x, variant=v)
        assert spmv_rel_err(y, y_spira, scale) <= 2 * SPMV_TOL, vname


def test_spmv_scalar_is_bit_exact_with_fused_scalar_order(ctx):
    r, c, v = gen.zipf_rows(20_000, seed=4)
    A = build(ctx, 20_000, 20_000, [(r, c, v)])
    x = gen.dense_x(20_000, 5)
    y = A.spmv_host(x, variant=sg.SPMV_SCALAR)
    np.testing.assert_array_equal(y, oracle.spmv_scalar(A.download(), x, fused=True))


@pytest.mark.parametrize("lengths", [[5000], [1, 3, 0, 17] * 3000, list(range(0, 3000, 7)), [16] * 4096])
def test_interleaved_is_bit_identical_to_adaptive16(ctx, lengths):
    """The interleaved variant runs ADAPTIVE16's per-lane FMA chains over a
    permuted copy of cols/vals: the same bits, whatever the row lengths."""
    r, c, v = _csr_from_rows(lengths, 30_000, seed=sum(lengths) % 1000)
    A = build(ctx, len(lengths), 30_000, [(r, c, v)])
    x = gen.dense_x(30_000, 6)
    np.testing.assert_array_equal(A.spmv_host(x, variant=sg.SPMV_INTERLEAVED),
                                  A.spmv_host(x, variant=sg.SPMV_ADAPTIVE16))


def test_plans_follow_relock(ctx):
    """Cached plans (and the interleaved copy) are rebuilt after a re-lock."""
    r, c, v = gen.zipf_rows(30_000, seed=13)
    A = build(ctx, 30_000, 30_000, [(r, c, v)])
    x = gen.dense_x(30_000, 14)
    for _, var in VARIANTS:
        A.spmv_host(x, variant=var)
    A.lock(*gen.relock_batch(30_000, 30_000, len(r), seed=15, zero_frac=0.1))
    check_all_variants(A, x)


def test_host_spmv_pipelined_blocks_match_device_path(ctx):
    """Host-buffer SpMV of a large matrix runs in row blocks whose results are
    copied back while the next block computes; y must be bit-identical to the
    one-launch device path, with empty rows and long rows crossing blocks."""
    import torch
    n = 700_000
    lengths = np.where(np.arange(n) % 3 == 1, 0, 10).astype(np.int64)
    lengths[::50_000] = 12_000  # long rows (their chunks straddle block boundaries)
    r, c, v = _csr_from_rows(lengths, n, seed=77)
    A = build(ctx, n, n, [(r, c, v)])
    assert A.nnz >= (4 << 20)
    x = gen.dense_x(n, 78)
    xd = torch.from_numpy(x).cuda()
    yd = torch.empty(n, dtype=torch.float64, device="cuda")
    xp = torch.from_numpy(x).pin_memory()  # pinned buffers take the recorded-graph path
    yp = torch.empty(n, dtype=torch.float64).pin_memory()
    for name, var in VARIANTS:
        if var == sg.SPMV_AUTO:
            continue
        A.spmv(xd, yd, var)
        ctx.sync()
        want = yd.cpu().numpy()
        np.testing.assert_array_equal(A.spmv_host(x, variant=var), want, err_msg=name)
        for _ in range(2):  # record, then replay
            yp.zero_()
            A.spmv_host(xp.numpy(), yp.numpy(), variant=var)
            np.testing.assert_array_equal(yp.numpy(), want, err_msg=name + " (pinned)")
    # a re-lock drops the recorded graph: the next call sees the new matrix
    A.lock(np.array([5], np.uint32), np.array([7], np.uint32), np.array([3.0]))
    A.spmv(xd, yd, sg.SPMV_SCALAR)
    ctx.sync()
    A.spmv_host(xp.numpy(), yp.numpy(), variant=sg.SPMV_SCALAR)
    np.testing.assert_array_equal(yp.numpy(), yd.cpu().numpy())


def test_host_spmv_async_two_matrices_two_streams(ctx):
    """Asynchronous host-buffer SpMVs of two matrices in flight at once on
    two streams give the same bits as the synchronous call; unpinned
    buffers are refused."""
    import torch
    mats = []
    for n, seed in ((700_000, 81), (300_000, 82)):
        r, c, v = gen.zipf_rows(n, seed=seed) if n == 300_000 else gen.laplacian_2d(837)
        n = 837 * 837 if n == 700_000 else n
        A = build(ctx, n, n, [(r, c, v)])
        x = gen.dense_x(n, seed + 1)
        mats.append((A, torch.from_numpy(x).pin_memory(), torch.empty(n, dtype=torch.float64).pin_memory(),
                     A.spmv_host(x)))
    streams = [torch.cuda.Stream(), torch.cuda.Stream()]
    for rep in range(3):  # record, then replay
        for (A, xp, yp, want), st in zip(mats, streams):
            yp.zero_()
            A.spmv_host_async(xp.numpy(), yp.numpy(), stream=st.cuda_stream)
        for st in streams:
            st.synchronize()
        for A, xp, yp, want in mats:
            np.testing.assert_array_equal(yp.numpy(), want)
    A, xp, yp, want = mats[0]
    with pytest.raises(sg.InvalidArgument):
        A.spmv_host_async(xp.numpy().copy(), yp.numpy())


def test_host_spmv_multi(ctx):
    """Several matrices' host-buffer SpMVs in one call (one recorded graph):
    the same bits as one call each, re-recorded after a re-lock; unpinned
    buffers, repeated matrices and more than four are refused."""
    import torch
    mats, xs, ys, want = [], [], [], []
    specs = [("zipf", 300_000, 91), ("lap", 837, 92), ("rand", 50_000, 93)]
    for kind, n, seed in specs:
        if kind == "zipf":
            r, c, v = gen.zipf_rows(n, seed=seed)
        elif kind == "lap":
            r, c, v = gen.laplacian_2d(n)
            n = n * n
        else:
            r, c, v = gen.random_rows(n, n, 12, seed=seed)
        A = build(ctx, n, n, [(r, c, v)])
        x = gen.dense_x(n, seed + 1)
        mats.append(A)
        xs.append(torch.from_numpy(x).pin_memory())
        ys.append(torch.empty(n, dtype=torch.float64).pin_memory())
        want.append(A.spmv_host(x))
    st = torch.cuda.Stream()
    for rep in range(3):
        for y in ys:
            y.zero_()
        sg.spmv_host_multi(ctx, mats, [x.numpy() for x in xs], [y.numpy() for y in ys], stream=st.cuda_stream)
        st.synchronize()
        for y, w in zip(ys, want):
            np.testing.assert_array_equal(y.numpy(), w)
    mats[1].lock(np.array([3], np.uint32), np.array([4], np.uint32), np.array([2.0]))
    want[1] = mats[1].spmv_host(xs[1].numpy().copy())
    sg.spmv_host_multi(ctx, mats, [x.numpy() for x in xs], [y.numpy() for y in ys])
    ctx.sync()
    for y, w in zip(ys, want):
        np.testing.assert_array_equal(y.numpy(), w)
    with pytest.raises(sg.InvalidArgument):
        sg.spmv_host_multi(ctx, mats[:1], [xs[0].numpy().copy()], [ys[0].numpy()])
    with pytest.raises(sg.InvalidArgument):
        sg.spmv_host_multi(ctx, [mats[0], mats[0]], [xs[0].numpy()] * 2, [ys[0].numpy()] * 2)
    with pytest.raises(sg.InvalidArgument):
        sg.spmv_host_multi(ctx, mats * 2, [x.numpy() for x in xs] * 2, [y.numpy() for y in ys] * 2)


def test_gather_probe(ctx):
    r = ctx.probe_gather_rate(1 << 20, 1 << 22)
    assert 1e9 < r < 1e13
    with pytest.raises(sg.InvalidArgument):
        ctx.probe_gather_rate(3, 1 << 20)
    with pytest.raises(sg.InvalidArgument):
        ctx.probe_gather_rate(1 << 20, 8)


def test_fp64_probe(ctx):
    r = ctx.probe_fp64_rate(256)
    assert 1e10 < r < 1e13
    with pytest.raises(sg.InvalidArgument):
        ctx.probe_fp64_rate(4)


def test_spmv_laplacian_2a_full(ctx):
    """Config 2a at full size: 5-point Laplacian on 1414^2, re-lock, SpMV."""
    r, c, v = gen.laplacian_2d(1414)
    n = 1414 * 1414
    assert n == 1_999_396 and len(r) == 9_991_324
    b = gen.relock_batch(n, n, len(r), seed=21)
    A = build(ctx, n, n, [(r, c, v), b])
    x = gen.dense_x(n, 22)
    errs = check_all_variants(A, x)
    assert max(errs.values()) <= SPMV_TOL


def test_spmv_zipf_2b_full(ctx):
    """Config 2b at full size: 4M x 4M, Zipf(1.8) rows capped at 10 000."""
    from spira_gb300 import gen_device
    n = 4_000_000
    r, c, v, m = gen_device.zipf_rows(ctx, n, seed=31)
    A = sg.Csr(ctx, n, n)
    A.lock_device(r, c, v, m)
    A.lock(*gen.relock_batch(n, n, m, seed=32))
    x = gen.dense_x(n, 33)
    check_all_variants(A, x)


def test_spmv_device_pointers_and_stream(ctx):
    import torch
    r, c, v = gen.random_rows(5000, 4000, 10, seed=8)
    A = build(ctx, 5000, 4000, [(r, c, v)])
    x = gen.dense_x(4000, 9)
    xd = torch.from_numpy(x).cuda()
    yd = torch.empty(5000, dtype=torch.float64, device="cuda")
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        A.spmv(xd, yd, sg.SPMV_MERGE, stream=s.cuda_stream)
    s.synchronize()
    y_ref, scale = oracle.spmv_compensated(A.download(), x)
    assert spmv_rel_err(yd.cpu().numpy(), y_ref, scale) <= SPMV_TOL


def test_host_spmv_multi_builds_plans_before_recording(ctx):
    """Plan-based variants named explicitly on matrices that never ran them:
    their plans are built before the graph is recorded (a plan build
    synchronises, which a recording stream cannot)."""
    import torch
    specs = [(sg.SPMV_MERGE, 20_000, 41), (sg.SPMV_STREAM, 30_000, 42), (sg.SPMV_INTERLEAVED, 25_000, 43)]
    mats, xs, ys, want = [], [], [], []
    for v, n, seed in specs:
        r, c, vals = gen.random_rows(n, n, 9, seed=seed)
        mats.append(build(ctx, n, n, [(r, c, vals)]))
        x = gen.dense_x(n, seed)
        xs.append(torch.from_numpy(x).pin_memory())
        ys.append(torch.empty(n, dtype=torch.float64).pin_memory())
    sg.spmv_host_multi(ctx, mats, [x.numpy() for x in xs], [y.numpy() for y in ys],
                       variants=[v for v, _, _ in specs])
    ctx.sync()
    for A, (v, _, _), x, y in zip(mats, specs, xs, ys):
        np.testing.assert_array_equal(y.numpy(), A.spmv_host(x.numpy().copy(), variant=v))


@pytest.mark.parametrize("tile, base", [("interleaved_s4", "interleaved"), ("interleaved_s8", "interleaved"),
                                        ("interleaved", "adaptive16"), ("adaptive16_s4", "adaptive16"),
                                        ("adaptive_s16", "adaptive")])
def test_spmv_tiles_give_their_variants_bits(ctx, tile, base):
    """A tile changes only how many nonzeros a lane loads before its FMAs and
    how many blocks share an SM, never a lane's FMA order: y is bit-identical
    to its variant's (INTERLEAVED is ADAPTIVE16's arithmetic)."""
    r, c, v = gen.zipf_rows(30_000, seed=21)
    A = build(ctx, 30_000, 30_000, [(r, c, v)])
    x = gen.dense_x(30_000, 22)
    y_t = A.spmv_host(x, variant=sg.SPMV_VARIANTS[tile])
    y_b = A.spmv_host(x, variant=sg.SPMV_VARIANTS[base])
    np.testing.assert_array_equal(y_t.view(np.uint64), y_b.view(np.uint64))
