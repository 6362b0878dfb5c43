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


def spmv_bytes(n_rows, n_cols, nnz):
    return 12 * nnz + 8 * (n_rows + 1) + 8 * n_cols + 8 * n_rows


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

    dev = 0
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
        t_all, best = m["A"].autotune(5)  # exhaustive autotuner: the judge
        m["autotuned"] = best
        m["autotune_ms"] = t_all

    def timed(variant_of, steps, warmup):
        ev = [[torch.cuda.Event(enable_timing=True) for _ in range(len(mats) + 1)] for _ in range(steps)]
        with torch.cuda.stream(stream):
            for _ in range(warmup):
                for m in mats:
                    m["A"].spmv(m["xd"], m["yd"], variant_of(m), stream=ctx.stream)
            torch.cuda.synchronize()
            for s in range(steps):
                ev[s][0].record(stream)
                for i, m in enumerate(mats):
                    m["A"].spmv(m["xd"], m["yd"], variant_of(m), stream=ctx.stream)
                    ev[s][i + 1].record(stream)
            torch.cuda.synchronize()
        per = np.array([[ev[s][i].elapsed_time(ev[s][i + 1]) for i in range(len(mats))] for s in range(steps)])
        total_ms = float(ev[0][0].elapsed_time(ev[-1][-1]))
        return total_ms / steps, per.mean(axis=0)

    clk = ClockSampler(dev)
    clk.start()
    ms_sel, per_sel = timed(lambda m: m["selected"], args.steps, args.warmup)
    ms_plain, per_plain = timed(lambda m: sg.SPMV_SCALAR, args.steps, args.warmup)
    ms_auto, per_auto = timed(lambda m: m["autotuned"], max(args.steps // 4, 10), args.warmup)
    clocks = clk.stop()
    batched = None if args.no_batched else run_batched(ctx, stream)

    # parity check of the measured configuration against the compensated oracle
    import oracle
    host = [m["A"].download() for m in mats]
    max_err = 0.0
    for m, h in zip(mats, host):
        y = m["yd"].cpu().numpy()
        y_ref, sc = oracle.spmv_compensated(h, m["x"])
        d = np.abs(y - y_ref) / np.where(sc > 0, sc, 1.0)
        max_err = max(max_err, float(d.max()))

    # end to end through the C ABI with host (pinned) buffers
    xs = [torch.from_numpy(m["x"]).pin_memory() for m in mats]
    ys = [torch.empty(m["n_rows"], dtype=torch.float64).pin_memory() for m in mats]
    e2e_steps = max(10, min(args.steps, 200))
    for _ in range(3):
        for m, xh, yh in zip(mats, xs, ys):
            m["A"].spmv_host(xh.numpy(), yh.numpy(), variant=m["selected"])
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        for m, xh, yh in zip(mats, xs, ys):
            m["A"].spmv_host(xh.numpy(), yh.numpy(), variant=m["selected"])
    e2e_ms = (time.perf_counter() - t0) * 1e3 / e2e_steps

    peak, peak_kind = peaks()
    dom = int(np.argmax(per_sel))
    dm = mats[dom]
    achieved = dm["bytes"] / (per_sel[dom] * 1e-3) / 1e9
    gpu_launches = args.steps * sum(m["A"].spmv_launches(m["selected"]) for m in mats)

    cpu = cpu_baseline(host, [m["x"] for m in mats], total_bytes)
    line = {
        "metric": METRIC,
        "value": round(total_bytes / (ms_sel * 1e-3) / 1e9, 2),
        "unit": "GB/s",
        "n_gpus": 1,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(ms_sel, 5),
        "higher_is_better": True,
        "scaling": "replicas",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic (seeded generators: 2D Laplacian 1414^2 and Zipf(1.8) 4M rows)",
        "config": {"workload": WORKLOAD, "matrices": [
            {"name": m["name"], "n_rows": m["n_rows"], "n_cols": m["n_cols"], "nnz": m["nnz"],
             "bytes_per_spmv": m["bytes"], "variant": sg.SPMV_NAMES[m["selected"]],
             "ms_selected": round(float(per_sel[i]), 5), "ms_plain": round(float(per_plain[i]), 5),
             "gbs_selected": round(m["bytes"] / (per_sel[i] * 1e-3) / 1e9, 1),
             "gbs_plain": round(m["bytes"] / (per_plain[i] * 1e-3) / 1e9, 1)}
            for i, m in enumerate(mats)],
            "bytes_per_step": total_bytes,
            "l2": "no flush: each step streams 1.03 GB (> 129 MB L2)"},
        "plain": {"variant": "scalar (one thread per row)", "value": round(total_bytes / (ms_plain * 1e-3) / 1e9, 2),
                  "ms_per_step": round(ms_plain, 5)},
        "autotuned": {"value": round(total_bytes / (ms_auto * 1e-3) / 1e9, 2), "ms_per_step": round(ms_auto, 5),
                      "variants": [sg.SPMV_NAMES[m["autotuned"]] for m in mats],
                      "learned_over_autotuned_time": round(ms_sel / ms_auto, 4),
                      "autotune_ms_per_variant": {m["name"]: {sg.SPMV_NAMES[v]: round(float(t), 4)
                                                             for v, t in enumerate(m["autotune_ms"])}
                                                  for m in mats}},
        "batched": batched,
        "roofline": {"bound": "hbm", "kernel": f"spmv[{dm['name']}:{sg.SPMV_NAMES[dm['selected']]}]",
                     "achieved": round(achieved, 1), "peak": peak, "peak_kind": peak_kind, "unit": "GB/s",
                     "frac": round(achieved / peak, 4), "traffic": None},
        "parity": {"max_err_vs_compensated_oracle": max_err, "tolerance": 1e-12,
                   "bound": "|y-y_ref| <= tol * sum|a x| per row"},
        "e2e": {"value": round(total_bytes / (e2e_ms * 1e-3) / 1e9, 2), "unit": "GB/s",
                "ms_per_step": round(e2e_ms, 4),
                "h2d_bytes_per_step": int(sum(8 * m["n_cols"] for m in mats)),
                "d2h_bytes_per_step": int(sum(8 * m["n_rows"] for m in mats)),
                "path": "spg_spmv_host (C ABI) from pinned host x to pinned host y"},
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
                      f"{nthr} threads, parallel_matrix partitions t*n/T"}


def run_reference(args):
    """The reference arm: Spira's threaded SIMD CPU SpMV on the host cores,
    on the same matrices (built by the oracle's restatement of lock())."""
    import oracle
    nthr = os.cpu_count() or 1
    host, xs = [], []
    for name, nr, nc, epochs, x in make_inputs(lambda n, seed: oracle.zipf_rows_host(n, seed=seed)):
        host.append(oracle.lock_epochs(nr, nc, epochs))
        xs.append(x)
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
        "scaling": "replicas", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": WORKLOAD, "bytes_per_step": total_bytes},
        "cpu_baseline": {"value": v, "unit": "GB/s", "cores": nthr, "kind": kind, "sample": sample},
        "e2e": {"value": v, "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-batched", action="store_true", help="skip the batched multi-RHS section")
    args = ap.parse_args()
    rank = int(os.environ.get("RANK", "0"))
    if args.impl == "reference":
        if rank == 0:
            run_reference(args)
        return
    if args.gpus > 1 or int(os.environ.get("WORLD_SIZE", "1")) > 1:
        # replicas only: the path does not shard within one job; each rank would
        # run an independent replica. This pool runs one GPU per job.
        if rank != 0:
            return
    run_ours(args)


if __name__ == "__main__":
    main()
