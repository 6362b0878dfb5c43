"""FP64 CSR SpMV benchmark on one GB300 (Spira's sparse hot path).

Workload: the large lock/merge + SpMV configuration -
  (a) 5-point 2D Laplacian on a 1414 x 1414 grid (n = 1 999 396, nnz = 9 991 324),
  (b) 4M x 4M power-law matrix, row lengths Zipf(1.8) capped at 10 000 and
      scaled to mean 16 (L = min(10000, max(1, round(Z * 16 / E[Z])))),
      uniform columns, values uniform[-1, 1);
each built by insert -> lock(), then 1 % of nnz new entries inserted into a
random 10 % of rows and lock() again (the merge). One step = one SpMV
y = A x on each of (a) and (b). Inputs are synthetic (seeded generators).

metric: GB/s on Spira's own SpMV byte model (bench/spira_bench.cpp:297-307 with
8-byte offsets): 12 nnz + 8 (n_rows + 1) + 8 n_cols + 8 n_rows per matrix,
summed over both matrices, divided by the step time.

    python bench.py [--gpus 1] [--steps K] [--warmup W] [--impl ours|reference]
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "FP64 SpMV GB/s & % HBM roofline: learned/autotuned vs plain, 1 GB300"
WORKLOAD = "spmv_lock_merge_2d_laplacian_1414sq_plus_zipf1.8_4M"
GRID = 1414
ZIPF_N = 4_000_000


# DRAM bytes (read + write) per launch of the dominant kernel from one ncu
# capture of dram__bytes_read.sum + dram__bytes_write.sum on the first-lock
# 4M-row Zipf matrix: (bytes, nonzeros of the captured matrix); scaled to the
# bench matrix by its nonzero count.
NCU_TRAFFIC = {("zipf4m", "interleaved"): (817.1e6, 63_247_590)}


def spmv_bytes(n_rows, n_cols, nnz):
    return 12 * nnz + 8 * (n_rows + 1) + 8 * n_cols + 8 * n_rows


def workload_config(meta):
    """The `config` both arms print: the same matrices (name, shape, nonzeros
    after the re-lock) and the same bytes per step. meta: [(name, n_rows,
    n_cols, nnz)]."""
    mats = [{"name": nm, "n_rows": int(r), "n_cols": int(c), "nnz": int(z), "bytes_per_spmv": spmv_bytes(r, c, z)}
            for nm, r, c, z in meta]
    return {"workload": WORKLOAD, "matrices": mats, "bytes_per_step": int(sum(m["bytes_per_spmv"] for m in mats)),
            "l2": "no flush: each step streams 1.03 GB (> 129 MB L2)"}


# What the CPU arm runs where Spira's own sources are absent (kind "port"):
# the oracle's C restatement of parallel::algorithms::spmv
# (parallel/algorithms/spmv.hpp:125-161) over parallel_matrix's t*n/T row
# partitions, each row in sparse_dot_double's SIMD order (4 accumulators x
# lanes, tree reduce, tail) written as scalar fma() loops.
CPU_PORT_BUILD = ("oracle/spira_oracle.c: gcc -O2 -ffp-contract=off, scalar fma() loops in the SIMD dot's "
                  "order (NEON shape on aarch64: 2 lanes x 4 accumulators, fused tail; AVX-512 shape on x86-64), "
                  "pthreads over t*n/T row partitions")
CPU_REF_BUILD = ("Spira compiled from its sources (oracle/Makefile `ref`: -std=gnu++23 -O3, per-file SIMD flags), "
                 "parallel::algorithms::spmv on parallel_matrix<soa_tag, uint32_t, double>")


class Replicas:
    """One process per GPU under torchrun: every rank runs the same workload
    on its own GPU (the path does not shard: replicas only), timed regions are
    bracketed by barriers and the slowest rank's time is the job's. Scalars
    travel over gloo; there is no data-path collective."""

    def __init__(self):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        if self.world > 1:
            import torch.distributed as dist
            if not dist.is_initialized():
                dist.init_process_group("gloo")

    def barrier(self):
        if self.world > 1:
            import torch.distributed as dist
            dist.barrier()

    def max(self, v: float) -> float:
        if self.world == 1:
            return v
        import torch
        import torch.distributed as dist
        t = torch.tensor([float(v)], dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t.item())


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def make_inputs(zipf_rows=None):
    """[(name, n_rows, n_cols, epochs, x)]; epochs[0] of the Zipf matrix comes
    from `zipf_rows(n, seed)` (device or host generator), the rest from the
    host generators of spira_gb300.gen."""
    from spira_gb300 import gen
    out = []
    r, c, v = gen.laplacian_2d(GRID)
    n = GRID * GRID
    out.append(("laplacian2d", n, n, [(r, c, v), gen.relock_batch(n, n, len(r), seed=21)], gen.dense_x(n, 22)))
    first = zipf_rows(ZIPF_N, 31)
    m = first[3] if len(first) == 4 else len(first[0])
    out.append(("zipf4m", ZIPF_N, ZIPF_N, [first, gen.relock_batch(ZIPF_N, ZIPF_N, m, seed=32)],
                gen.dense_x(ZIPF_N, 33)))
    return out


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device=0):
        self.device = device
        self.p = None
        self.out = None

    def start(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                                       "--format=csv,noheader,nounits", "-lms", "100"],
                                      stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.p = None

    def stop(self):
        if not self.p:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        self.p.terminate()
        try:
            txt, _ = self.p.communicate(timeout=5)
        except Exception:
            self.p.kill()
            txt = ""
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in txt.strip().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for nm, val in zip(names, f[5:9]):
                if val.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(mx)), "reasons": sorted(reasons),
                "samples": len(sm)}


def run_ours(args):
    import torch

    import spira_gb300 as sg

    rep = Replicas()
    dev = rep.local
    torch.cuda.set_device(dev)
    ctx = sg.Context(dev)
    stream = torch.cuda.ExternalStream(ctx.stream)
    from spira_gb300 import gen_device

    mats = []
    for name, nr, nc, epochs, x in make_inputs(lambda n, seed: gen_device.zipf_rows(ctx, n, seed=seed)):
        A = sg.Csr(ctx, nr, nc)
        for ep in epochs:
            if len(ep) == 4:  # device-resident staging (rows, cols, vals, m)
                A.lock_device(ep[0], ep[1], ep[2], ep[3])
            else:
                A.lock(*ep)
        epochs = None
        nnz = A.nnz
        xd = torch.from_numpy(x).to(f"cuda:{dev}")
        yd = torch.empty(nr, dtype=torch.float64, device=f"cuda:{dev}")
        mats.append({"name": name, "A": A, "x": x, "xd": xd, "yd": yd, "n_rows": nr, "n_cols": nc, "nnz": nnz,
                     "bytes": spmv_bytes(nr, nc, nnz)})
    ctx.sync()
    total_bytes = sum(m["bytes"] for m in mats)

    for m in mats:
        m["selected"] = m["A"].selected_spmv()  # SPMV_AUTO: the learned selector's pick
        t_all, best = m["A"].autotune(5)  # exhaustive autotuner: the yardstick of the selector
        m["autotuned"] = best
        m["autotune_ms"] = t_all

    side = torch.cuda.Stream()

    def step(variant_of):
        # the two matrices are independent: their SpMVs run on two streams (the
        # Laplacian's HBM-bound kernel fills in beside the Zipf matrix's
        # L2-bound one), joined before the next step
        side.wait_stream(stream)
        for i, m in enumerate(mats):
            st = side if i == 0 else stream
            m["A"].spmv(m["xd"], m["yd"], variant_of(m), stream=st.cuda_stream)
        stream.wait_stream(side)

    def timed(variant_of, steps, warmup):
        """ms per step over `steps` steps (events only at the two ends of the
        timed region), and each matrix's mean SpMV time from a separate pass
        with events around every launch (one stream)."""
        with torch.cuda.stream(stream):
            for _ in range(warmup):
                step(variant_of)
            torch.cuda.synchronize()
            rep.barrier()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(steps):
                step(variant_of)
            e1.record(stream)
            torch.cuda.synchronize()
            rep.barrier()
            total_ms = rep.max(float(e0.elapsed_time(e1)))
            k = min(steps, 200)
            ev = [[torch.cuda.Event(enable_timing=True) for _ in range(2 * len(mats))] for _ in range(k)]
            for s in range(k):
                for i, m in enumerate(mats):
                    ev[s][2 * i].record(stream)
                    m["A"].spmv(m["xd"], m["yd"], variant_of(m), stream=ctx.stream)
                    ev[s][2 * i + 1].record(stream)
            torch.cuda.synchronize()
        per = np.array([[ev[s][2 * i].elapsed_time(ev[s][2 * i + 1]) for i in range(len(mats))] for s in range(k)])
        return total_ms / steps, per.mean(axis=0)

    def b2b(m, reps=100):
        """ms per SpMV over `reps` back-to-back SpMVs of one matrix (each one
        streams more than the L2 holds), events only at the ends."""
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            for _ in range(3):
                m["A"].spmv(m["xd"], m["yd"], m["selected"], stream=ctx.stream)
            e0.record(stream)
            for _ in range(reps):
                m["A"].spmv(m["xd"], m["yd"], m["selected"], stream=ctx.stream)
            e1.record(stream)
            torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps

    clk = ClockSampler(dev)
    clk.start()
    ms_sel, per_sel = timed(lambda m: m["selected"], args.steps, args.warmup)
    ms_plain, per_plain = timed(lambda m: sg.SPMV_SCALAR, args.steps, args.warmup)
    ms_auto, per_auto = timed(lambda m: m["autotuned"], max(args.steps // 4, 10), args.warmup)
    ms_b2b = [b2b(m) for m in mats]
    clocks = clk.stop()
    batched = None if (args.no_batched or rep.rank != 0) else run_batched(ctx, stream)
    selector = None if (args.no_selector or rep.rank != 0) else run_selector(ctx)

    # parity check of the measured configuration against the compensated oracle
    import oracle
    host = [m["A"].download() for m in mats]
    max_err = 0.0
    for m, h in zip(mats, host):
        y = m["yd"].cpu().numpy()
        y_ref, sc = oracle.spmv_compensated(h, m["x"])
        d = np.abs(y - y_ref) / np.where(sc > 0, sc, 1.0)
        max_err = max(max_err, float(d.max()))

    # end to end through the C ABI with host (pinned) buffers: each step
    # uploads both x, runs both SpMVs and reads both y back; the two
    # matrices' calls go out asynchronously on two streams, so one matrix's
    # transfers overlap the other's (the host link is the bound)
    xs = [torch.from_numpy(m["x"]).pin_memory() for m in mats]
    ys = [torch.empty(m["n_rows"], dtype=torch.float64).pin_memory() for m in mats]
    e2e_streams = [torch.cuda.Stream() for _ in mats]
    e2e_steps = max(10, min(args.steps, 200))

    # one spg_spmv_host_multi call per step: the Zipf matrix's x goes up first
    # (its SpMV reads x anywhere), the Laplacian's transfers and SpMV run
    # during the Zipf SpMV
    xh = [x.numpy() for x in xs]
    yh = [y.numpy() for y in ys]
    e2e_variants = [m["selected"] for m in mats]

    def e2e_step():
        sg.spmv_host_multi(ctx, [m["A"] for m in mats], xh, yh, e2e_variants, e2e_streams[0].cuda_stream)
        e2e_streams[0].synchronize()

    for _ in range(3):
        e2e_step()
    rep.barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        e2e_step()
    e2e_ms = rep.max((time.perf_counter() - t0) * 1e3 / e2e_steps)
    rep.barrier()
    ctx.sync()  # reports a device-side timeout, if any

    peak, peak_kind = peaks()
    ops = None if (args.no_ops or rep.rank != 0) else run_ops(ctx, peak)
    dom = int(np.argmax(per_sel))
    dm = mats[dom]
    achieved = dm["bytes"] / (per_sel[dom] * 1e-3) / 1e9
    gpu_launches = rep.world * args.steps * sum(m["A"].spmv_launches(m["selected"]) for m in mats)
    # The second ceiling of a random-column matrix: requests from L1 to L2.
    # Every x read is its own request (one 32-byte sector); the 12 B/nnz matrix
    # stream arrives in coalesced 128-byte requests. The probe's random reads
    # (one request each), swept over reads in flight per thread and blocks per
    # SM, measure the rate; its maximum is the ceiling.
    g_best, g_pts = ctx.gather_ceiling_sweep(1 << 22, 1 << 26)
    gather_rate = g_best["gathers_per_s"]
    g_rates = [p["gathers_per_s"] for p in g_pts]
    # one request per x read, the matrix stream in 128-byte requests, one write request per row of y
    # (ncu on the 1M-row case: 17.01 M read requests against 17.2 M modelled, plus 1.0 M writes)
    l1_l2_requests = dm["nnz"] * (1 + 12 / 128) + dm["n_rows"]
    floor_ms = l1_l2_requests / gather_rate * 1e3
    cap = NCU_TRAFFIC.get((dm["name"], sg.SPMV_NAMES[dm["selected"]]))
    traffic = round(cap[0] * dm["nnz"] / cap[1]) if cap else None

    if rep.rank != 0:  # the other replicas only contribute their timings
        return
    cpu = cpu_baseline(host, [m["x"] for m in mats], total_bytes)
    W = rep.world  # every replica moves the step's bytes
    line = {
        "metric": METRIC,
        "value": round(W * total_bytes / (ms_sel * 1e-3) / 1e9, 2),
        "unit": "GB/s",
        "n_gpus": W,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(ms_sel, 5),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic (seeded generators: 2D Laplacian 1414^2 and Zipf(1.8) 4M rows)",
        "config": workload_config([(m["name"], m["n_rows"], m["n_cols"], m["nnz"]) for m in mats]),
        "execution": "the two SpMVs of a step on two streams, joined per step",
        "per_matrix": [
            {"name": m["name"], "variant": sg.SPMV_NAMES[m["selected"]],
             "ms_selected": round(float(per_sel[i]), 5), "ms_plain": round(float(per_plain[i]), 5),
             "gbs_selected": round(m["bytes"] / (per_sel[i] * 1e-3) / 1e9, 1),
             "gbs_plain": round(m["bytes"] / (per_plain[i] * 1e-3) / 1e9, 1),
             "ms_100_back_to_back": round(ms_b2b[i], 5),
             "gbs_100_back_to_back": round(m["bytes"] / (ms_b2b[i] * 1e-3) / 1e9, 1),
             "frac_100_back_to_back": round(m["bytes"] / (ms_b2b[i] * 1e-3) / 1e9 / peak, 4)}
            for i, m in enumerate(mats)],
        "plain": {"variant": "scalar (one thread per row)", "value": round(W * total_bytes / (ms_plain * 1e-3) / 1e9, 2),
                  "ms_per_step": round(ms_plain, 5)},
        "autotuned": {"value": round(W * total_bytes / (ms_auto * 1e-3) / 1e9, 2), "ms_per_step": round(ms_auto, 5),
                      "variants": [sg.SPMV_NAMES[m["autotuned"]] for m in mats],
                      "learned_over_autotuned_time": round(ms_sel / ms_auto, 4),
                      "autotune_ms_per_variant": {m["name"]: {sg.SPMV_NAMES[v]: round(float(t), 4)
                                                             for v, t in enumerate(m["autotune_ms"])}
                                                  for m in mats}},
        "batched": batched,
        "selector": selector,
        "ops": ops,
        "roofline": {"bound": "hbm", "kernel": f"spmv[{dm['name']}:{sg.SPMV_NAMES[dm['selected']]}]",
                     "achieved": round(achieved, 1), "peak": peak, "peak_kind": peak_kind, "unit": "GB/s",
                     "frac": round(achieved / peak, 4), "traffic": traffic,
                     "algorithmic_bytes": dm["bytes"],
                     "gather_ceiling": {"random_8B_gathers_per_s": round(gather_rate, -6),
                                        "probe": "spg_probe_gather_rate_cfg(2^22 doubles, 2^26 reads): maximum "
                                                 "over 2..64 reads in flight per thread x 2..16 blocks of 256 "
                                                 "per SM",
                                        "sweep_min_max": [round(min(g_rates), -6), round(max(g_rates), -6)],
                                        "best_shape": {k: g_best[k] for k in ("per_thread", "blocks_per_sm",
                                                                              "resident_blocks_per_sm")},
                                        "l1_to_l2_requests_per_launch": round(l1_l2_requests),
                                        "model": "one request per x read + matrix stream / 128 B + one y write per row",
                                        "floor_ms": round(floor_ms, 5),
                                        "frac_of_ceiling": round(floor_ms / per_sel[dom], 4)}},
        "parity": {"max_err_vs_compensated_oracle": max_err, "tolerance": 1e-12,
                   "bound": "|y-y_ref| <= tol * sum|a x| per row"},
        "e2e": {"value": round(W * total_bytes / (e2e_ms * 1e-3) / 1e9, 2), "unit": "GB/s",
                "ms_per_step": round(e2e_ms, 4),
                "h2d_bytes_per_step": int(sum(8 * m["n_cols"] for m in mats)),
                "d2h_bytes_per_step": int(sum(8 * m["n_rows"] for m in mats)),
                "path": "spg_spmv_host_multi (C ABI): both matrices per call, from pinned host x to pinned host y"},
        "gpu_launches": gpu_launches,
        "clocks": clocks,
        "cpu_baseline": cpu,
    }
    print(json.dumps(line))


def run_batched(ctx, stream, n_mats=4096, seed=2024):
    """Batched multi-RHS workload: 4 096 matrices (rows log-uniform in
    [100, 200 000], Poisson(12) nnz per row, k in {1..32}); one persistent
    launch from a CUDA graph (tiles autotuned) vs one plain launch per matrix
    per right-hand side."""
    import torch

    import spira_gb300 as sg
    from spira_gb300 import batched as bt
    t0 = time.time()
    mats, Xs, Ys, ks, nnz = bt.build(ctx, n_mats, seed)
    t_build = time.time() - t0
    B = sg.Batch(ctx, mats, Xs, Ys, ks, config=-1)
    cfg, n_items = B.config()
    by = bt.bytes_per_run(mats, ks, nnz)

    def time_it(fn, reps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        fn()
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(reps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps

    ms_graph = time_it(lambda: B.run(ctx.stream), 20)
    ms_plain = time_it(lambda: B.run_plain(ctx.stream), 3)
    # every (nonzero, right-hand side) pair is one FP64 FMA: the FP64 pipe is
    # this workload's bound, measured by the FMA-rate probe in the same run
    fmas = sum(int(z) * int(k) for z, k in zip(nnz, ks))
    fp64_peak = ctx.probe_fp64_rate(4096)
    # spot-check 3 matrices against the compensated oracle
    import oracle
    worst = 0.0
    B.run(ctx.stream)
    ctx.sync()
    for i in (0, n_mats // 2, n_mats - 1):
        H = mats[i].download()
        k = ks[i]
        Xh = Xs[i].cpu().numpy().reshape(H.n_cols, k)
        Yh = Ys[i].cpu().numpy().reshape(H.n_rows, k)
        for j in range(k):
            yr, sc = oracle.spmv_compensated(H, Xh[:, j].copy())
            worst = max(worst, float((np.abs(Yh[:, j] - yr) / np.where(sc > 0, sc, 1.0)).max()))
    out = {
        "workload": f"{n_mats} CSR matrices, rows log-uniform [100, 200000], Poisson(12) nnz/row, k in 1..32",
        "total_nnz": int(sum(nnz)), "total_rows": int(sum(A.n_rows for A in mats)),
        "rhs_total": int(sum(ks)), "bytes_per_run": int(by),
        "persistent_graph": {"ms": round(ms_graph, 4), "gbs": round(by / (ms_graph * 1e-3) / 1e9, 1),
                             "launches": 1, "config": cfg, "work_items": n_items},
        "fp64_roofline": {"fmas_per_run": fmas, "achieved_fma_per_s": round(fmas / (ms_graph * 1e-3) / 1e9, 1),
                          "peak_fma_per_s": round(fp64_peak / 1e9, 1), "unit": "G FMA/s",
                          "peak": "FMA-rate probe (8 chains x 256 threads x 8 CTAs per SM), same run",
                          "frac": round(fmas / (ms_graph * 1e-3) / fp64_peak, 3)},
        "plain_per_matrix_per_rhs": {"ms": round(ms_plain, 3), "gbs": round(by / (ms_plain * 1e-3) / 1e9, 1),
                                     "launches": int(sum(ks))},
        "speedup": round(ms_plain / ms_graph, 2),
        "max_err_vs_compensated_oracle_sampled": worst,
        "setup_s": round(t_build, 1),
    }
    B.close()
    for A in mats:
        A.close()
    del Xs, Ys
    torch.cuda.empty_cache()
    return out


# The shipped selectors were trained on corpus matrices 0 .. n-1 drawn with
# seed 7 (SpMV: n = 20 000, SpGEMM: n = 4 000; the last 10 % of each held out
# during training). The bench scores them on matrices from index n on, which
# neither training nor its held-out check has seen.
SELECTOR_HELD_OUT = {"spmv": (20_000, 3), "spgemm": (4_000, 2)}  # first index, autotune reps


def run_selector(ctx, budget_s=75.0):
    """Held-out regret of the shipped learned selectors against exhaustive
    autotuning (every candidate timed) and against the fixed default
    (ADAPTIVE16 for SpMV, ROWMERGE for SpGEMM: the method without the
    selector), on a time-capped slice of the corpus the selectors never saw."""
    import spira_gb300 as sg
    from spira_gb300 import selector as S
    out = {}
    models = {"spmv": sg._PKG / "spg_selector.bin", "spgemm": sg._PKG / "spg_spgemm_selector.bin"}
    share = {"spmv": 0.55, "spgemm": 0.45}
    for op, (first, reps) in SELECTOR_HELD_OUT.items():
        path = models[op]
        if not path.exists():
            out[op] = {"unavailable": f"no shipped model ({path.name})"}
            continue
        blob = np.fromfile(path, dtype=np.float32)
        t0 = time.time()
        X, T, _ = S.collect(ctx, range(first, first + 100_000), seed=7, reps=reps, op=op,
                            time_cap_s=budget_s * share[op])
        secs = time.time() - t0
        choice = S.predict(ctx, blob, X, op=op).argmin(axis=1)
        default = S.DEFAULT_SPMV if op == "spmv" else S.DEFAULT_SPGEMM
        ev = S.evaluate(T, choice, default)
        names = sg.SPMV_NAMES if op == "spmv" else sg.SPGEMM_NAMES
        ev.update({"corpus_indices": [first, first + len(X)], "seed": 7, "seconds": round(secs, 1),
                   "candidates": len(names), "default": names[default],
                   "exhaustive_best_histogram": {names[k]: int(c) for k, c in
                                                 enumerate(np.bincount(T.argmin(axis=1), minlength=len(names)))
                                                 if c}})
        out[op] = ev  # (predict installed the shipped model, which the context had loaded anyway)
    return out


def lock_bytes(n_rows, staged, nnz_old, nnz_new):
    """Algorithmic bytes of one lock(): read the staged triples (u32 row, u32
    column, f64 value) and the old CSR, write the new CSR."""
    old = 12 * nnz_old + 8 * (n_rows + 1) if nnz_old else 0
    return 16 * staged + old + 12 * nnz_new + 8 * (n_rows + 1)


def csr_bytes(n_rows, nnz):
    return 12 * nnz + 8 * (n_rows + 1)


def run_ops(ctx, peak):
    """lock() (first build and 1 % re-lock merge), transpose and SpGEMM (every
    variant and the selected one) on the GPU at their full configuration
    sizes. Each GPU figure is the median of 3 calls, twice: wall time around
    the C-ABI call with the stream synchronised on both sides (the calls
    synchronise internally: their output sizes are data-dependent), and
    device time (spg_ctx_timer: the stream's work between those internal
    synchronisations, host round trips excluded). CPU: the oracle's C port of
    Spira's parallel paths on all host cores (parallel_matrix partitions
    t*n/T: per-partition lock, row-partitioned Gustavson SpGEMM, transpose by
    output partitions each scanning all of A), and of the serial path on one
    core."""
    import torch

    import oracle
    import spira_gb300 as sg
    from spira_gb300 import gen, gen_device

    nthr = os.cpu_count() or 1

    def wall(fn, reps=3, setup=None):
        ts, ds = [], []
        for _ in range(reps):
            if setup:
                setup()
            ctx.sync()
            t0 = time.perf_counter()
            fn()
            ctx.sync()
            ts.append(time.perf_counter() - t0)
        for _ in range(reps):
            if setup:
                setup()
            ctx.sync()
            ds.append(ctx.device_ms(fn))
        return float(np.median(ts)) * 1e3, float(np.median(ds))

    def cpu(fn):
        t0 = time.perf_counter()
        out = fn()
        return (time.perf_counter() - t0) * 1e3, out

    def rec(name, gpu, by, cpu_ms, cpu_serial_ms=None, **kw):
        gpu_ms, dev_ms = gpu
        d = {"case": name, "gpu_ms": round(gpu_ms, 3), "gpu_device_ms": round(dev_ms, 3), "bytes": int(by),
             "gbs": round(by / (gpu_ms * 1e-3) / 1e9, 1), "frac_of_hbm": round(by / (gpu_ms * 1e-3) / 1e9 / peak, 4),
             "device_gbs": round(by / (dev_ms * 1e-3) / 1e9, 1),
             "device_frac_of_hbm": round(by / (dev_ms * 1e-3) / 1e9 / peak, 4)}
        if cpu_ms is not None:
            d.update({"cpu_ms": round(cpu_ms, 1), "cpu_kind": "port", "cpu_cores": nthr,
                      "speedup_vs_cpu": round(cpu_ms / gpu_ms, 1)})
        if cpu_serial_ms is not None:
            d.update({"cpu_serial_ms": round(cpu_serial_ms, 1), "cpu_serial_cores": 1,
                      "speedup_vs_cpu_serial": round(cpu_serial_ms / gpu_ms, 1)})
        d.update(kw)
        return d

    out = {"lock": [], "transpose": [], "spgemm": [],
           "cpu": f"oracle C port of Spira's parallel paths, {nthr} threads (serial path on 1 core beside it)"}
    dev = "cuda:0"

    def to_dev(r, c, v):
        return (torch.from_numpy(r.view(np.int32)).to(dev), torch.from_numpy(c.view(np.int32)).to(dev),
                torch.from_numpy(v).to(dev))

    # ---- lock: 2D Laplacian (2a) and Zipf 4M (2b), first lock + 1 % re-lock
    g2 = GRID * GRID
    r, c, v = gen.laplacian_2d(GRID)
    b = gen.relock_batch(g2, g2, len(r), seed=21)
    cases = [("laplacian2d", g2, (r, c, v), b, True)]
    zr, zc, zv, zm = gen_device.zipf_rows(ctx, ZIPF_N, seed=31)
    cases.append(("zipf4m", ZIPF_N, (zr, zc, zv, zm), gen.relock_batch(ZIPF_N, ZIPF_N, zm, seed=32), False))
    for name, n, first, delta, host_first in cases:
        d_first = to_dev(*first) + (len(first[0]),) if host_first else first
        m = d_first[3]
        holder = []

        def do_first():
            A = sg.Csr(ctx, n, n)
            A.lock_device(*d_first)
            holder.append(A)

        t_first = wall(do_first)
        A = holder[-1]
        nnz0 = A.nnz
        for h in holder[:-1]:
            h.close()
        pristine = sg.Csr(ctx, n, n)
        pristine.copy_from(A)
        t_relock = wall(lambda: A.lock(*delta), setup=lambda: A.copy_from(pristine))
        nnz1 = A.nnz
        t_e2e = None
        cpu_first = cpu_relock = ser_first = ser_relock = None
        if host_first:
            def do_host():
                B = sg.Csr(ctx, n, n)
                B.lock(*first)
                B.close()
            t_e2e = wall(do_host)[0]
            # each epoch timed on its own inside the port (the second epoch's
            # time is the relock alone); one thread is Spira's serial path
            secs1, _ = oracle.lock_parallel_time(n, n, [first, delta], 1)
            ser_first, ser_relock = secs1[0] * 1e3, secs1[1] * 1e3
            host_epochs = [first, delta]
        else:
            # the same first epoch, copied back from the device; the serial
            # path is skipped here (it alone would take most of a minute)
            host_epochs = [(d_first[0][:m].cpu().numpy().view(np.uint32), d_first[1][:m].cpu().numpy().view(np.uint32),
                            d_first[2][:m].cpu().numpy()), delta]
        secs, _ = oracle.lock_parallel_time(n, n, host_epochs, nthr)
        cpu_first, cpu_relock = secs[0] * 1e3, secs[1] * 1e3
        del host_epochs
        out["lock"].append(rec(f"{name}_first", t_first, lock_bytes(n, m, 0, nnz0), cpu_first, ser_first,
                               staged=int(m), nnz=int(nnz0), staging="device",
                               **({"e2e_ms_host_staging": round(t_e2e, 3)} if t_e2e else {})))
        out["lock"].append(rec(f"{name}_relock", t_relock, lock_bytes(n, len(delta[0]), nnz0, nnz1), cpu_relock,
                               ser_relock, staged=int(len(delta[0])), nnz=int(nnz1), staging="host"))
        A.close()
        pristine.close()
        del d_first
    del zr, zc, zv
    torch.cuda.empty_cache()

    # ---- transpose and SpGEMM: 3D Laplacian 100^3 (3a), uniform 200k x 8 (3b)
    for name, n, (r, c, v) in [("laplacian3d_100", 100 ** 3, gen.laplacian_3d(100)),
                               ("uniform200k_8", 200_000, gen.uniform_rows(200_000, 200_000, 8, seed=77))]:
        A = sg.Csr(ctx, n, n)
        A.lock(r, c, v)
        H = A.download()
        res = {}

        def do_t():
            if "T" in res:
                res["T"].close()
            res["T"] = A.transpose()

        t_t = wall(do_t)
        ser_t, T_ref = cpu(lambda: oracle.transpose(H))
        cpu_t, _ = cpu(lambda: oracle.transpose_parallel(H, nthr))
        T = res["T"]
        same_t = oracle.csr_digest(T.download()) == oracle.csr_digest(T_ref)
        out["transpose"].append(rec(name, t_t, 2 * csr_bytes(n, A.nnz), cpu_t, ser_t, nnz=int(A.nnz),
                                    bit_exact=same_t))
        T.close()
        res.clear()
        ser_g, C_ref = cpu(lambda: oracle.spgemm(H, H))
        cpu_g, _ = cpu(lambda: oracle.spgemm_parallel(H, H, nthr))
        ref_digest = oracle.csr_digest(C_ref)
        prods = int(oracle.spgemm_products(H, H))
        by = 2 * csr_bytes(n, A.nnz) + csr_bytes(n, len(C_ref.cols))
        per_variant = {}
        for vname, vid in sg.SPGEMM_VARIANTS.items():
            def do_g():
                if "C" in res:
                    res["C"].close()
                res["C"] = A.spgemm(A, vid)

            tv = wall(do_g)
            per_variant[vname] = {"gpu_ms": round(tv[0], 3), "gpu_device_ms": round(tv[1], 3),
                                  "bit_exact": oracle.csr_digest(res["C"].download()) == ref_digest}
            res["C"].close()
            res.clear()
        sel = A.spgemm_selected(A)

        def do_auto():
            if "C" in res:
                res["C"].close()
            res["C"] = A.spgemm(A)

        t_g = wall(do_auto)
        Cm = res["C"]
        same_g = oracle.csr_digest(Cm.download()) == ref_digest
        best = min(per_variant, key=lambda k: per_variant[k]["gpu_ms"])
        out["spgemm"].append(rec(name, t_g, by, cpu_g, ser_g, nnz_a=int(A.nnz), nnz_c=int(Cm.nnz), products=prods,
                                 gproducts_per_s=round(prods / (t_g[0] * 1e-3) / 1e9, 2), bit_exact=same_g,
                                 selected=sg.SPGEMM_NAMES[sel], fastest=best,
                                 selected_over_fastest=round(t_g[0] / per_variant[best]["gpu_ms"], 4),
                                 variants=per_variant))
        Cm.close()
        A.close()

    # ---- element-wise: A + B, A * s (copy and in place), row sums on the 2a
    # Laplacian and the 2b Zipf matrix, B = A after the 1 % re-lock
    out["elementwise"] = []
    r, c, v = gen.laplacian_2d(GRID)
    zr, zc, zv, zm = gen_device.zipf_rows(ctx, ZIPF_N, seed=31)
    for name, n in (("laplacian2d", GRID * GRID), ("zipf4m", ZIPF_N)):
        A = sg.Csr(ctx, n, n)
        if name == "laplacian2d":
            A.lock(r, c, v)
        else:
            A.lock_device(zr, zc, zv, zm)
        B = sg.Csr(ctx, n, n)
        B.copy_from(A)
        B.lock(*gen.relock_batch(n, n, A.nnz, seed=21 if name == "laplacian2d" else 32))
        HA, HB = A.download(), B.download()
        res = {}

        def do_add():
            if "C" in res:
                res["C"].close()
            res["C"] = A.add(B)

        t_add = wall(do_add)
        cpu_add, C_ref = cpu(lambda: oracle.add(HA, HB))
        Cm = res["C"]
        by = csr_bytes(n, A.nnz) + csr_bytes(n, B.nnz) + csr_bytes(n, Cm.nnz)
        out["elementwise"].append(rec(f"add_{name}", t_add, by, None, cpu_add, nnz_a=int(A.nnz), nnz_b=int(B.nnz),
                                      nnz_c=int(Cm.nnz),
                                      bit_exact=oracle.csr_digest(Cm.download()) == oracle.csr_digest(C_ref)))
        Cm.close()
        res.clear()

        def do_scale():
            if "S" in res:
                res["S"].close()
            res["S"] = A.scaled(2.5)

        t_sc = wall(do_scale)
        cpu_sc, S_ref = cpu(lambda: oracle.scale(HA, 2.5))
        out["elementwise"].append(rec(f"scale_copy_{name}", t_sc, 2 * csr_bytes(n, A.nnz), None, cpu_sc, nnz=int(A.nnz),
                                      bit_exact=oracle.csr_digest(res["S"].download()) == oracle.csr_digest(S_ref)))
        res["S"].close()
        t_ip = wall(lambda: A.scale_(-1.0))  # exact: six sign flips, A as before
        out["elementwise"].append(rec(f"scale_in_place_{name}", t_ip, 16 * A.nnz, None, nnz=int(A.nnz)))
        sums = torch.empty(n, dtype=torch.float64, device=dev)
        t_rs = wall(lambda: A.row_sums(sums))
        cpu_rs, rs_ref = cpu(lambda: oracle.row_sums(A.download()))
        out["elementwise"].append(rec(f"row_sums_{name}", t_rs, 8 * A.nnz + 8 * (n + 1) + 8 * n, None, cpu_rs,
                                      bit_exact=bool(np.array_equal(sums.cpu().numpy().view(np.uint64),
                                                                    rs_ref.view(np.uint64)))))
        A.close()
        B.close()
        del sums
    del zr, zc, zv
    torch.cuda.empty_cache()
    return out


def _cpu_spmv_seconds(host, xs, nthr, kind, budget_s):
    """Mean seconds of one SpMV per matrix on the host cores."""
    import oracle
    out = []
    per_budget = budget_s / max(len(host), 1)
    for h, x in zip(host, xs):
        if kind == "reference":
            t1, _ = oracle.ref_spmv_parallel_time(h, x, nthr, reps=1)
            reps = int(max(1, min(200, per_budget / max(t1, 1e-6))))
            t, _ = oracle.ref_spmv_parallel_time(h, x, nthr, reps=reps)
        else:
            y = np.empty(h.n_rows)
            oracle.spmv_parallel(h, x, nthr, y=y)
            t0 = time.perf_counter()
            reps = 0
            while reps < 200 and time.perf_counter() - t0 < per_budget:
                oracle.spmv_parallel(h, x, nthr, y=y)
                reps += 1
            t = (time.perf_counter() - t0) / max(reps, 1)
        out.append((t, reps))
    return out


def cpu_baseline(host, xs, total_bytes, budget_s=12.0):
    """Spira's threaded SIMD SpMV path on the host cores: Spira itself where
    its sources were compiled (oracle/_ref), else the oracle's port of it."""
    import oracle
    nthr = os.cpu_count() or 1
    kind = "reference" if oracle.ref_available() else "port"
    per = _cpu_spmv_seconds(host, xs, nthr, kind, budget_s)
    dt = sum(t for t, _ in per)
    return {"value": round(total_bytes / dt / 1e9, 3), "unit": "GB/s", "cores": nthr, "kind": kind,
            "sample": f"full SpMVs of both matrices ({', '.join(str(r) for _, r in per)} reps), "
                      f"{nthr} threads, parallel_matrix partitions t*n/T",
            "build": CPU_REF_BUILD if kind == "reference" else CPU_PORT_BUILD}


def run_reference(args):
    """The reference arm: Spira's threaded SIMD CPU SpMV on the host cores,
    on the same matrices (built by the oracle's restatement of lock())."""
    import oracle
    nthr = os.cpu_count() or 1
    host, xs, meta = [], [], []
    for name, nr, nc, epochs, x in make_inputs(lambda n, seed: oracle.zipf_rows_host(n, seed=seed)):
        host.append(oracle.lock_epochs(nr, nc, epochs))
        xs.append(x)
        meta.append((name, nr, nc, len(host[-1].cols)))
    total_bytes = sum(spmv_bytes(h.n_rows, h.n_cols, len(h.cols)) for h in host)
    kind = "reference" if oracle.ref_available() else "port"
    _cpu_spmv_seconds(host, xs, nthr, kind, budget_s=1.0)  # warm-up
    per = _cpu_spmv_seconds(host, xs, nthr, kind, budget_s=min(60.0, 0.02 * max(args.steps, 1) + 5.0))
    dt = sum(t for t, _ in per)
    v = round(total_bytes / dt / 1e9, 3)
    sample = (f"{min(r for _, r in per)}+ full SpMVs per matrix (time-capped sample of the {args.steps} steps), "
              f"{nthr} threads")
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": v, "unit": "GB/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(dt * 1e3, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": workload_config(meta),
        "cpu_baseline": {"value": v, "unit": "GB/s", "cores": nthr, "kind": kind, "sample": sample,
                         "build": CPU_REF_BUILD if kind == "reference" else CPU_PORT_BUILD},
        "e2e": {"value": v, "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }))


PROFILE_CASES = {
    # name: (rows, kind); zipf1m is a quarter-size Zipf matrix (~16M nonzeros,
    # ~220 MB: larger than L2, small enough for multi-pass ncu captures)
    "laplacian2d": (GRID * GRID, "laplacian"),
    "zipf1m": (1_000_000, "zipf"),
    "zipf4m": (ZIPF_N, "zipf"),
    # lock / transpose / SpGEMM: `--reps` calls of the operation
    "lock_zipf1m": (1_000_000, "lock"),
    "lock_zipf4m": (ZIPF_N, "lock"),
    "lock_laplacian2d": (GRID * GRID, "lock"),
    "relock_zipf1m": (1_000_000, "relock"),
    "relock_laplacian2d": (GRID * GRID, "relock"),
    "batched256": (256, "batched"),  # the batched workload's first 256 matrices
    "transpose_laplacian3d": (100 ** 3, "transpose"),
    "spgemm_laplacian3d": (100 ** 3, "spgemm"),
    "spgemm_uniform200k": (200_000, "spgemm"),
    "add_zipf1m": (1_000_000, "add"),  # A + (A after a 1 % re-lock)
}


def run_profile_op(ctx, case, n, kind, reps, variants=""):
    """lock / transpose / SpGEMM cases of run_profile_case (SpGEMM: each
    variant named in `variants`, else the selected one)."""
    import spira_gb300 as sg
    from spira_gb300 import gen, gen_device
    ms = []
    if kind == "batched":
        import torch
        from spira_gb300 import batched as bt
        mats, Xs, Ys, ks, nz = bt.build(ctx, n, 2024)
        B = sg.Batch(ctx, mats, Xs, Ys, ks, config=-1)
        B.run(ctx.stream)
        for _ in range(reps):
            ctx.sync()
            t0 = time.perf_counter()
            B.run(ctx.stream)
            ctx.sync()
            ms.append((time.perf_counter() - t0) * 1e3)
        print(json.dumps({"profile_case": case, "matrices": n, "nnz": int(sum(nz)), "config": B.config(),
                          "ms_per_call": [round(t, 3) for t in ms]}))
        return
    if kind == "add":
        r, c, v, m = gen_device.zipf_rows(ctx, n, seed=31)
        A = sg.Csr(ctx, n, n)
        A.lock_device(r, c, v, m)
        del r, c, v
        B = sg.Csr(ctx, n, n)
        B.copy_from(A)
        B.lock(*gen.relock_batch(n, n, A.nnz, seed=32))
        for _ in range(reps + 1):
            ctx.sync()
            t0 = time.perf_counter()
            Cm = A.add(B)
            ctx.sync()
            ms.append((time.perf_counter() - t0) * 1e3)
            nnz = Cm.nnz
            Cm.close()
        print(json.dumps({"profile_case": case, "n_rows": n, "nnz": nnz, "ms_per_call": [round(t, 3) for t in ms]}))
        return
    if kind == "relock":
        import torch
        if case == "relock_laplacian2d":  # the bench's 2a re-lock: 1 % new entries into 10 % of the rows
            hr, hc, hv = gen.laplacian_2d(GRID)
            A = sg.Csr(ctx, n, n)
            A.lock(hr, hc, hv)
            dr, dc, dv = gen.relock_batch(n, n, A.nnz, seed=21)
        else:
            r, c, v, m = gen_device.zipf_rows(ctx, n, seed=31)
            A = sg.Csr(ctx, n, n)
            A.lock_device(r, c, v, m)
            del r, c, v
            dr, dc, dv = gen.relock_batch(n, n, A.nnz, seed=32)
        d = (torch.from_numpy(dr.view(np.int32)).cuda(), torch.from_numpy(dc.view(np.int32)).cuda(),
             torch.from_numpy(dv).cuda())
        pristine = sg.Csr(ctx, n, n)
        pristine.copy_from(A)
        for _ in range(reps + 1):
            A.copy_from(pristine)
            ctx.sync()
            t0 = time.perf_counter()
            A.lock_device(d[0], d[1], d[2], len(dr))
            ctx.sync()
            ms.append((time.perf_counter() - t0) * 1e3)
        nnz = A.nnz
    elif kind == "lock":
        if case == "lock_laplacian2d":
            import torch
            hr, hc, hv = gen.laplacian_2d(GRID)
            r, c, v = (torch.from_numpy(hr.view(np.int32)).cuda(), torch.from_numpy(hc.view(np.int32)).cuda(),
                       torch.from_numpy(hv).cuda())
            m = len(hr)
        else:
            r, c, v, m = gen_device.zipf_rows(ctx, n, seed=31)
        for _ in range(reps + 1):
            A = sg.Csr(ctx, n, n)
            ctx.sync()
            t0 = time.perf_counter()
            A.lock_device(r, c, v, m)
            ctx.sync()
            ms.append((time.perf_counter() - t0) * 1e3)
            nnz = A.nnz
            A.close()
    else:
        r, c, v = gen.laplacian_3d(100) if n == 100 ** 3 else gen.uniform_rows(n, n, 8, seed=77)
        A = sg.Csr(ctx, n, n)
        A.lock(r, c, v)
        nnz = A.nnz
        names = [v for v in variants.split(",") if v in sg.SPGEMM_VARIANTS] if kind == "spgemm" else []
        per = {}
        for name in (names or ["auto"]):
            vid = sg.SPGEMM_VARIANTS.get(name, sg.SPGEMM_AUTO)
            ms = []
            for _ in range(reps + 1):
                ctx.sync()
                t0 = time.perf_counter()
                B = A.transpose() if kind == "transpose" else A.spgemm(A, vid)
                ctx.sync()
                ms.append((time.perf_counter() - t0) * 1e3)
                B.close()
            per[name] = [round(t, 3) for t in ms]
        print(json.dumps({"profile_case": case, "n_rows": n, "nnz": nnz, "ms_per_call": per}))
        return
    print(json.dumps({"profile_case": case, "n_rows": n, "nnz": nnz, "ms_per_call": [round(t, 3) for t in ms]}))


def run_profile_case(args):
    """One matrix, a few SpMVs per listed variant: the program ncu captures.
    Prints the per-SpMV CUDA-event times (not a bench value)."""
    import torch

    import spira_gb300 as sg
    from spira_gb300 import gen, gen_device
    ctx = sg.Context(0)
    stream = torch.cuda.ExternalStream(ctx.stream)
    n, kind = PROFILE_CASES[args.profile_case]
    if kind in ("lock", "relock", "transpose", "spgemm", "batched", "add"):
        run_profile_op(ctx, args.profile_case, n, kind, args.reps, args.variants)
        return
    if kind == "zipf":
        r, c, v, m = gen_device.zipf_rows(ctx, n, seed=31)
        A = sg.Csr(ctx, n, n)
        A.lock_device(r, c, v, m)
        del r, c, v
    else:
        r, c, v = gen.laplacian_2d(GRID)
        A = sg.Csr(ctx, n, n)
        A.lock(r, c, v)
    x = torch.from_numpy(gen.dense_x(n, 3)).to("cuda:0")
    y = torch.empty(n, dtype=torch.float64, device="cuda:0")
    ctx.sync()
    out = {}
    if args.host:  # host-buffer SpMV through the C ABI (pinned x and y), wall time per call
        xh = torch.from_numpy(gen.dense_x(n, 3)).pin_memory()
        yh = torch.empty(n, dtype=torch.float64).pin_memory()
        for name in args.variants.split(","):
            vid = sg.SPMV_VARIANTS[name]
            A.spmv_host(xh.numpy(), yh.numpy(), variant=vid)
            ts = []
            for _ in range(args.reps):
                t0 = time.perf_counter()
                A.spmv_host(xh.numpy(), yh.numpy(), variant=vid)
                ts.append((time.perf_counter() - t0) * 1e3)
            out[name] = [round(t, 4) for t in ts]
        print(json.dumps({"profile_case": args.profile_case, "host": True, "n_rows": n, "nnz": A.nnz,
                          "ms_per_call": out}))
        return
    with torch.cuda.stream(stream):
        for name in args.variants.split(","):
            vid = sg.SPMV_VARIANTS[name]
            A.spmv(x, y, vid, stream=ctx.stream)  # builds the variant's plan
            ev = [torch.cuda.Event(enable_timing=True) for _ in range(args.reps + 1)]
            ev[0].record(stream)
            for i in range(args.reps):
                A.spmv(x, y, vid, stream=ctx.stream)
                ev[i + 1].record(stream)
            torch.cuda.synchronize()
            out[name] = [round(ev[i].elapsed_time(ev[i + 1]), 5) for i in range(args.reps)]
    print(json.dumps({"profile_case": args.profile_case, "n_rows": n, "nnz": A.nnz,
                      "bytes_per_spmv": spmv_bytes(n, n, A.nnz), "ms_per_spmv": out}))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--profile-case", choices=sorted(PROFILE_CASES),
                    help="run a few SpMVs of one matrix (for ncu captures) instead of the bench")
    ap.add_argument("--variants", default="adaptive16", help="with --profile-case: comma-separated variant names")
    ap.add_argument("--reps", type=int, default=2, help="with --profile-case: SpMVs per variant after one warm-up")
    ap.add_argument("--host", action="store_true", help="with --profile-case: time host-buffer SpMV calls")
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-batched", action="store_true", help="skip the batched multi-RHS section")
    ap.add_argument("--no-ops", action="store_true", help="skip the lock / transpose / SpGEMM section")
    ap.add_argument("--no-selector", action="store_true", help="skip the selectors' held-out regret section")
    args = ap.parse_args()
    if args.profile_case:
        run_profile_case(args)
        return
    rank = int(os.environ.get("RANK", "0"))
    if args.impl == "reference":
        if rank == 0:
            run_reference(args)
        return
    # N > 1 (torchrun): every rank runs an independent replica on its GPU
    # (replicas only: the path does not shard), rank 0 prints the job's line
    run_ours(args)


if __name__ == "__main__":
    main()
