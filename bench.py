#!/usr/bin/env python
"""Benchmark of the implicitly restarted Lanczos solver on one GB300.

One step = one complete eigen-solve (start vector to converged Ritz pairs)
of the workload.  Default workload: 3-D 7-point Dirichlet Laplacian on a
160^3 grid (n = 4,096,000, nnz = 28,518,400) plus a diagonal shift
uniform[0, 0.1) per row from seed 1, CSR int32/FP64, nev = 20, ncv = 60,
largest algebraic, tolerance 1e-10, start vector uniform[-1, 1) from seed 0.
Metric: converged eigenpairs per second; a step counts only if every
returned pair has ||A v - lambda v|| <= 1e-10 ||A||_inf.

    value   device-resident: CSR already in HBM, outputs to device buffers,
            CUDA events on the solver's stream around K solves
    e2e     through the C ABI with pinned host buffers: dcsrmv_operator_gpu
            construction (CSR host->device) + ds_solver_gpu writing host
            values/vectors (+ operator teardown), wall clock per solve
    roofline  the dominant kernel class of one profiled solve (CUDA events
            around every launch): algorithmic bytes / time vs the measured
            HBM peak, and FP64 flops / time vs the live FP64 probe

`--impl reference` times the oracle's C restatement of the reference CPU
solver (oracle/, OpenMP over all host cores) on the same workload: each step
is one restart cycle's worth of Lanczos steps, extrapolated to the SpMV
count of the full solve.  Multi-GPU runs are independent replicas (the
reference path does not shard a solve): value sums every rank's rate.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

from hlanc_gb300 import generators as G  # noqa: E402

# SpMV calls of a full solve of each workload, measured with this library on
# GB300 (the algorithm's count; the CPU baseline extrapolates its sampled
# per-step time with it).
WORKLOADS = {
    "lap3d_160": dict(desc="3-D Laplacian 160^3 + U[0,0.1) diagonal shift (seed 1)",
                      gen=lambda: G.laplacian_3d(160, shift_seed=1), nev=20, ncv=60, tol=1e-10),
    "lap3d_100": dict(desc="3-D Laplacian 100^3 + U[0,0.1) diagonal shift (seed 1)",
                      gen=lambda: G.laplacian_3d(100, shift_seed=1), nev=20, ncv=60, tol=1e-10),
    "lap3d_64": dict(desc="3-D Laplacian 64^3 + U[0,0.1) diagonal shift (seed 1)",
                     gen=lambda: G.laplacian_3d(64, shift_seed=1), nev=20, ncv=60, tol=1e-10),
    "lap2d_100": dict(desc="2-D Laplacian 100^2 (reference tolerance dlamch('E'))",
                      gen=lambda: G.laplacian_2d(100), nev=10, ncv=30, tol=0.0),
    "chunglu_22": dict(desc="normalised adjacency of a Chung-Lu graph, n = 2^22, exponent 2.5, mean degree 32 "
                            "(seed 2); FP32 SpMV + FP64 refinement",
                       gen=lambda: G.chung_lu_normalized(1 << 22, seed=2), nev=16, ncv=48, tol=1e-10, mixed=True),
    "chunglu_22_fp64": dict(desc="normalised adjacency of a Chung-Lu graph, n = 2^22 (seed 2); plain FP64",
                            gen=lambda: G.chung_lu_normalized(1 << 22, seed=2), nev=16, ncv=48, tol=1e-10),
}
FULL_SOLVE_SPMV = {"lap3d_160": 3460, "lap3d_100": None, "lap3d_64": 1312, "lap2d_100": 1375,
                   "chunglu_22": None, "chunglu_22_fp64": None}


def _env_int(k, d):
    try:
        return int(os.environ.get(k, d))
    except ValueError:
        return d


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:  # noqa: BLE001
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for name, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def cgs_fp64_share(kind: str, nev: int, ncv: int) -> float:
    """Fraction of a CGS kernel's columns run as FP64 FMAs by the hybrid
    kernels (kernels_step.cu), over the column counts c = nev+1 .. ncv of one
    restart cycle: projection panels of 8 split 5 + 3 (tails 1,1,2,2,3,3,4 of
    1..7), the update runs whole groups of 8 (about c/2) in FP64."""
    tail = [0, 1, 1, 2, 2, 3, 3, 4]
    f = t = 0
    for c in range(nev + 1, ncv + 1):
        if kind == "cgs_proj":
            f += 5 * (c // 8) + tail[c % 8]
        else:
            f += c if c < 8 else ((c + 8) >> 4) << 3
        t += c
    return f / t


def read_traffic_ratio(kernel_class: str):
    """DRAM bytes / algorithmic bytes of a kernel class from the committed ncu
    summary (profiles/*.txt line 'traffic_ratio_dram_over_algorithmic <class> <r>');
    the traffic of a launch here is that ratio times its algorithmic bytes
    (traffic grows in proportion to the rows and columns a launch streams)."""
    d = os.path.join(ROOT, "profiles")
    if not os.path.isdir(d):
        return None
    for fn in sorted(os.listdir(d)):
        if not fn.endswith(".txt"):
            continue
        with open(os.path.join(d, fn)) as f:
            for line in f:
                p = line.split()
                if len(p) == 3 and p[0] == "traffic_ratio_dram_over_algorithmic" and p[1] == kernel_class:
                    return float(p[2])
    return None


def dist_setup(ngpus):
    rank, world = _env_int("RANK", 0), _env_int("WORLD_SIZE", 1)
    local = _env_int("LOCAL_RANK", 0)
    pg = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo", init_method="env://")
        pg = dist
    return rank, world, local, pg


def barrier(pg):
    if pg is not None:
        pg.barrier()


def allmax(pg, x):
    if pg is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


def replica_value(world: int, nev: int, max_ms: float) -> float:
    """Whole-job eigenpairs/s of `world` independent replicas, each solving
    nev pairs per step, timed by the slowest rank (max over ranks)."""
    return world * nev / (max_ms / 1e3)


def cpu_sample(m, wl, threads, full_spmv):
    """Oracle port, first restart cycle of the same solve; extrapolated."""
    import oracle
    oracle.build()
    x0 = G.start_vector(m.n, 0)
    t = time.perf_counter()
    rc, vals, vecs, st = oracle.solve_csr(m.row_ptr, m.col, m.val, m.ncols, False, wl["nev"], wl["ncv"], x0,
                                          tol=wl["tol"], max_iter=1, threads=threads)
    dt = time.perf_counter() - t
    per_spmv = dt / max(st["spmv_calls"], 1)
    est = per_spmv * full_spmv
    return dict(value=wl["nev"] / est, unit="eigenpairs/s", cores=threads, kind="port",
                sample=(f"first restart cycle ({st['spmv_calls']} Lanczos steps, {dt:.2f} s) of the same solve "
                        f"on {threads} threads, extrapolated to the full solve's {full_spmv} SpMV steps"),
                seconds_per_step=per_spmv)


def run_reference(args, wl, m):
    rank = _env_int("RANK", 0)
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    full = FULL_SOLVE_SPMV.get(args.workload) or args.full_spmv
    for _ in range(args.warmup):
        cpu_sample(m, wl, threads, full)
    vals = [cpu_sample(m, wl, threads, full) for _ in range(args.steps)]
    v = statistics.median(x["value"] for x in vals)
    secs = wl["nev"] / v
    line = {"metric": "converged eigenpairs/s (resid <= 1e-10 ||A||)", "value": v, "unit": "eigenpairs/s",
            "impl": "reference", "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": secs * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic (seeded generator)",
            "config": config_of(args, wl, m),
            "cpu_baseline": {"value": v, "unit": "eigenpairs/s", "cores": threads, "kind": "port",
                             "sample": vals[0]["sample"]},
            "e2e": {"value": v, "unit": "eigenpairs/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def batch_problems(count, seed=3):
    """The batched workload: `count` symmetric banded-random matrices, n
    log-uniform in [2000, 200000], half-bandwidth uniform in {2..16}, 10% of
    rows with 1-8 extra off-band entries, N(0,1) entries, diagonal N(0, 4)."""
    ns, bws = G.batched_problem_sizes(count, 2000, 200000, 2, 16, seed=seed)
    return [G.banded_random(int(n), int(b), seed=seed, problem=i) for i, (n, b) in enumerate(zip(ns, bws))]


def run_batch(args):
    """Batched form vs the plain FP64 drop-in run one problem at a time."""
    import torch

    import hlanc_gb300 as H
    from hlanc_gb300 import build
    build.build()
    mats = batch_problems(args.batch_count)
    nev, ncv = 8, 24
    out = {}
    for mode, prec in (("fp64", H.HLANC_PREC_FP64), ("fp32_refine", H.HLANC_PREC_FP32_REFINE)):
        ops = [H.dcsrmv_operator_gpu(m, precision=prec) for m in mats]
        vals = [torch.zeros(ncv, dtype=torch.float64, device="cuda") for _ in mats]
        vecs = [torch.zeros((ncv, m.n), dtype=torch.float64, device="cuda") for m in mats]
        times = []
        for rep in range(args.warmup + args.steps):
            b = H.Batch(ops, nev, ncv, precision=prec, tol=1e-10)
            torch.cuda.synchronize()
            t = time.perf_counter()
            status, st = b.run([v.data_ptr() for v in vals], [x.data_ptr() for x in vecs])
            torch.cuda.synchronize()
            dt = time.perf_counter() - t
            b.close()
            if rep >= args.warmup:
                times.append(dt)
        ok = int((status == 0).sum())
        worst = 0.0
        for m, op, v, x in zip(mats, ops, vals, vecs):
            r, _ = H.residuals_device(op, nev, v.data_ptr(), x.data_ptr(), m.n)
            worst = max(worst, float(r.max()) / float(np.abs(G.to_scipy(m)).sum(axis=1).max()))
        t = statistics.median(times)
        out[f"batched_{mode}"] = {"seconds": t, "eigenpairs_per_s": ok * nev / t, "converged": ok,
                                  "max_residual_over_normA": worst, "spmv_calls": st["spmv_calls"]}
        if mode == "fp64":
            # plain FP64 drop-in, one solve after another (same GPU, same problems)
            torch.cuda.synchronize()
            t = time.perf_counter()
            okp = 0
            for m, op, v, x in zip(mats, ops, vals, vecs):
                stp = H.solve_device(op, nev, ncv, v.data_ptr(), x.data_ptr(), m.n, tol=1e-10)
                okp += stp["rc"] == 0
            torch.cuda.synchronize()
            tp = time.perf_counter() - t
            out["plain_fp64_one_at_a_time"] = {"seconds": tp, "eigenpairs_per_s": okp * nev / tp, "converged": okp}
        del ops
    best = max(out["batched_fp64"]["eigenpairs_per_s"], out["batched_fp32_refine"]["eigenpairs_per_s"])
    line = {"metric": "converged eigenpairs/s (resid <= 1e-10 ||A||), batched", "value":
            out["batched_fp32_refine"]["eigenpairs_per_s"], "unit": "eigenpairs/s", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "dtype": "f64 (fp32 SpMV)",
            "data": "synthetic (seeded generator)",
            "config": {"workload": f"batch{args.batch_count}", "nev": nev, "ncv": ncv, "tol": 1e-10,
                       "matrices": "banded random, n log-uniform [2000,200000], half-bandwidth U{2..16}, seed 3"},
            "results": out, "speedup_vs_plain_fp64": best / out["plain_fp64_one_at_a_time"]["eigenpairs_per_s"]}
    print(json.dumps(line), flush=True)


def serve_requests(count, seed=4, rate=200.0, n_lo=1000, n_hi=200000):
    """Poisson request stream: exponential inter-arrival times (mean 1/rate)
    from seed, n log-uniform in [n_lo, n_hi], generator uniform over the
    workloads' families, nev uniform in {4, 8, 16}, ncv = 3 nev, 70% FP32-SpMV
    + refinement and 30% plain FP64."""
    u = G.uniform01(seed, 40, 6 * count).reshape(count, 6)
    arrivals = np.cumsum(-np.log(1.0 - u[:, 0]) / rate)
    reqs = []
    for i in range(count):
        n = int(np.exp(np.log(n_lo) + u[i, 1] * (np.log(n_hi) - np.log(n_lo))))
        fam = int(u[i, 2] * 4)
        if fam == 0:
            nx = max(int(round(np.sqrt(n))), 8)
            m = G.laplacian_2d(nx)
        elif fam == 1:
            N = max(int(round(n ** (1 / 3))), 6)
            m = G.laplacian_3d(N, shift_seed=seed + i)
        elif fam == 2:
            m = G.banded_random(n, 2 + int(u[i, 5] * 15), seed=seed, problem=1000 + i)
        else:
            m = G.chung_lu_normalized(max(n, 1024), seed=seed + i)
        nev = (4, 8, 16)[min(int(u[i, 3] * 3), 2)]
        mixed = u[i, 4] < 0.7
        reqs.append(dict(t=float(arrivals[i]), m=m, nev=nev, ncv=3 * nev, mixed=bool(mixed), fam=fam))
    return reqs


def run_serve(args):
    """Continuous-batching server vs the plain FP64 solver serving the same
    stream one request at a time (FIFO); latency = completion - arrival.
    The server also runs the stream with every request in FP64, to separate
    the engine's gain from the precision mix."""
    import hlanc_gb300 as H
    from hlanc_gb300 import build
    build.build()
    reqs = serve_requests(args.serve_count, n_hi=args.serve_nmax)
    for r in reqs:
        prec = H.HLANC_PREC_FP32_REFINE if r["mixed"] else H.HLANC_PREC_FP64
        r["op"] = H.dcsrmv_operator_gpu(r["m"], precision=prec)
    # warm-up: a few solves to load kernels
    for r in reqs[:3]:
        H.solve(r["op"], r["nev"], r["ncv"], tol=1e-10)

    def stats(lat, t_total, ok_pairs, ok):
        lat = np.sort(np.array(lat))
        return {"requests": len(lat), "converged": ok, "seconds": t_total, "eigenpairs_per_s": ok_pairs / t_total,
                "p50_s": float(np.percentile(lat, 50)), "p95_s": float(np.percentile(lat, 95)),
                "p99_s": float(np.percentile(lat, 99))}

    def serve(all_fp64):
        srv = H.Server(mem_budget_bytes=150 << 30, max_slots=args.serve_slots, lanes=args.serve_lanes)
        t0 = time.perf_counter()
        nxt, ids, done, lat, pairs, ok = 0, {}, set(), [], 0, 0
        while len(done) < len(reqs):
            now = time.perf_counter() - t0
            while nxt < len(reqs) and reqs[nxt]["t"] <= now:
                r = reqs[nxt]
                mixed = r["mixed"] and not all_fp64
                kw = dict(tol=1e-10, precision=H.HLANC_PREC_FP32_REFINE if mixed else H.HLANC_PREC_FP64)
                ids[srv.submit(r["op"], r["nev"], r["ncv"], **kw)] = nxt
                nxt += 1
            active, waiting = srv.step()
            for rid, i in list(ids.items()):
                if i in done:
                    continue
                res = srv.poll(rid)
                if res is not None:
                    done.add(i)
                    lat.append(time.perf_counter() - t0 - reqs[i]["t"])
                    pairs += reqs[i]["nev"] if res[0] == 0 else 0
                    ok += res[0] == 0
            if active == 0 and waiting == 0 and nxt < len(reqs):
                time.sleep(max(0.0, reqs[nxt]["t"] - (time.perf_counter() - t0)))
        out = stats(lat, time.perf_counter() - t0, pairs, ok)
        out["engine"] = srv.stats()
        srv.close()
        return out

    served = serve(False)
    served_fp64 = serve(True)
    # plain FP64, one at a time, FIFO over the same arrivals
    t0 = time.perf_counter()
    lat, pairs, ok = [], 0, 0
    for r in reqs:
        now = time.perf_counter() - t0
        if r["t"] > now:
            time.sleep(r["t"] - now)
        rc, _, _, _ = H.solve(r["op"], r["nev"], r["ncv"], tol=1e-10)
        lat.append(time.perf_counter() - t0 - r["t"])
        pairs += r["nev"] if rc == 0 else 0
        ok += rc == 0
    plain = stats(lat, time.perf_counter() - t0, pairs, ok)
    line = {"metric": "serving throughput (eigenpairs/s) and latency", "value": served["eigenpairs_per_s"],
            "unit": "eigenpairs/s", "n_gpus": 1, "higher_is_better": True, "dtype": "f64 (70% fp32 SpMV)",
            "data": "synthetic (seeded generators)",
            "config": {"workload": f"serve{args.serve_count}", "arrivals": "Poisson, mean 200 req/s, seed 4",
                       "n": f"log-uniform [1000, {args.serve_nmax}]", "nev": "{4,8,16}, ncv = 3 nev",
                       "mix": "70% fp32+refine", "tol": 1e-10, "max_restarts": 200,
                       "slots": args.serve_slots, "lanes": args.serve_lanes or 2, "mem_budget_GB": 150},
            "server": served, "server_all_fp64": served_fp64, "plain_fp64_one_at_a_time": plain,
            "throughput_ratio": served["eigenpairs_per_s"] / plain["eigenpairs_per_s"],
            "throughput_ratio_all_fp64": served_fp64["eigenpairs_per_s"] / plain["eigenpairs_per_s"],
            "p99_ratio_plain_over_server": plain["p99_s"] / served["p99_s"]}
    print(json.dumps(line), flush=True)


def config_of(args, wl, m):
    return {"workload": args.workload, "description": wl["desc"], "n": m.n, "nnz": m.nnz, "nev": wl["nev"],
            "ncv": wl["ncv"], "tol": wl["tol"] or "dlamch(E)", "which": "largest algebraic",
            "start": "uniform[-1,1) seed 0",
            "precision": "fp32 SpMV + fp64 refinement" if wl.get("mixed") else "fp64",
            "l2": "inputs larger than L2 (CSR + basis >> 129 MB); no flush needed",
            "parallelism": "replicas"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="lap3d_160", choices=sorted(WORKLOADS))
    ap.add_argument("--e2e-steps", type=int, default=1)
    ap.add_argument("--full-spmv", type=int, default=0, help="SpMV count of a full solve (CPU extrapolation)")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--batch", action="store_true", help="batched form (512 banded problems)")
    ap.add_argument("--batch-count", type=int, default=512)
    ap.add_argument("--serve", action="store_true", help="serving form (Poisson request stream)")
    ap.add_argument("--serve-count", type=int, default=100)
    ap.add_argument("--serve-slots", type=int, default=32)
    ap.add_argument("--serve-lanes", type=int, default=0, help="server launch lanes (0 = library default)")
    ap.add_argument("--serve-nmax", type=int, default=200000, help="largest n of the request stream")
    args = ap.parse_args()
    if args.batch:
        run_batch(args)
        return
    if args.serve:
        run_serve(args)
        return
    wl = WORKLOADS[args.workload]
    m = wl["gen"]()
    if args.impl == "reference":
        run_reference(args, wl, m)
        return

    import torch

    import hlanc_gb300 as H
    from hlanc_gb300 import build
    rank, world, local, pg = dist_setup(args.gpus)
    torch.cuda.set_device(local)
    build.build()
    dev = local
    nev, ncv, tol = wl["nev"], wl["ncv"], wl["tol"]
    prec = H.HLANC_PREC_FP32_REFINE if wl.get("mixed") else H.HLANC_PREC_FP64
    op = H.dcsrmv_operator_gpu(m, dev=dev, precision=prec)
    stream = torch.cuda.Stream()
    vals = torch.zeros(ncv, dtype=torch.float64, device="cuda")
    vecs = torch.zeros((ncv, m.n), dtype=torch.float64, device="cuda")
    norm_a = float(np.abs(G.to_scipy(m)).sum(axis=1).max())

    def solve_dev(**kw):
        return H.solve_device(op, nev, ncv, vals.data_ptr(), vecs.data_ptr(), m.n, dev=dev, tol=tol,
                              stream=stream.cuda_stream, precision=prec, **kw)

    for _ in range(args.warmup):
        st = solve_dev()
    torch.cuda.synchronize()
    barrier(pg)
    launches0 = H.kernel_launches()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    stats = []
    with ClockSampler(dev) as clk:
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(args.steps):
            stats.append(solve_dev())
        e1.record(stream)
        torch.cuda.synchronize()
    launches = H.kernel_launches() - launches0
    ms = e0.elapsed_time(e1) / args.steps
    ms = allmax(pg, ms)
    barrier(pg)
    res, rdiff = H.residuals_device(op, nev, vals.data_ptr(), vecs.data_ptr(), m.n)
    valid = all(s["rc"] == 0 and s["nconv"] >= nev for s in stats) and float(res.max()) <= 1e-10 * norm_a
    value = replica_value(world, nev, ms) if valid else 0.0
    mixed_cmp = None
    if prec == H.HLANC_PREC_FP32_REFINE:
        # per-eigenpair comparison of the mixed-precision pairs with a plain FP64 solve
        vals64 = torch.zeros(ncv, dtype=torch.float64, device="cuda")
        vecs64 = torch.zeros((ncv, m.n), dtype=torch.float64, device="cuda")
        H.solve_device(op, nev, ncv, vals64.data_ptr(), vecs64.data_ptr(), m.n, dev=dev, tol=tol,
                       stream=stream.cuda_stream, precision=H.HLANC_PREC_FP64)
        torch.cuda.synchronize()
        l_mix, l_64 = vals[:nev].double().cpu().numpy(), vals64[:nev].double().cpu().numpy()
        dots = torch.abs((vecs[:nev] * vecs64[:nev]).sum(dim=1)).cpu().numpy()
        mixed_cmp = {"eigenvalue_rel_diff": [float(abs(a - b) / abs(b)) for a, b in zip(l_mix, l_64)],
                     "residual_over_normA": [float(r / norm_a) for r in res],
                     "abs_dot_with_fp64_vector": [float(d) for d in dots],
                     "note": "pair i of the FP32-SpMV + FP64-refinement solve against pair i of a plain FP64 solve "
                             "(same start vector); |<v, v64>| near 1 where the eigenvalue is simple"}

    # end to end through the C ABI with host buffers in pinned memory: the
    # operator is built from host CSR arrays, the solve returns its pairs to
    # host arrays, both copies inside the timed region
    def pinned(a):
        t = torch.empty(a.shape, dtype=torch.from_numpy(a[:1]).dtype, pin_memory=True)
        t.numpy()[...] = a
        return t.numpy()

    class HostCSR:
        pass
    hc = HostCSR()
    hc.n, hc.ncols = m.n, m.ncols
    hc.row_ptr, hc.col, hc.val = pinned(np.asarray(m.row_ptr, np.int32)), pinned(np.asarray(m.col, np.int32)), \
        pinned(np.asarray(m.val, np.float64))
    values_h = torch.zeros(ncv, dtype=torch.float64, pin_memory=True).numpy()
    vectors_h = torch.zeros(m.n * ncv, dtype=torch.float64, pin_memory=True).numpy()
    e2e_ms, e2e_parts = [], []
    for _ in range(args.e2e_steps):
        torch.cuda.synchronize()
        t = time.perf_counter()
        op2 = H.dcsrmv_operator_gpu(hc, dev=dev, precision=prec)
        t1 = time.perf_counter()
        st2: dict = {}
        rc = H.ds_solver_gpu(m.n, nev, ncv, values_h, vectors_h, m.n, op2, dev, opts_=H.opts(tol=tol, precision=prec),
                             stats=st2)
        t2 = time.perf_counter()
        op2.close()
        t3 = time.perf_counter()
        e2e_ms.append((t3 - t) * 1e3)
        e2e_parts.append({"operator_create_ms": (t1 - t) * 1e3, "solve_and_copy_out_ms": (t2 - t1) * 1e3,
                          "operator_destroy_ms": (t3 - t2) * 1e3})
        valid = valid and rc == 0
    e2e_ms = allmax(pg, statistics.median(e2e_ms))
    h2d = 4 * (m.n + 1) + 12 * m.nnz
    d2h = 8 * nev + 8 * m.n * ncv

    # the SpMV kernel alone (dcsrmv_operator_gpu::operator() on device vectors)
    xs = torch.rand(m.n, dtype=torch.float64, device="cuda")
    ys = torch.zeros_like(xs)
    for _ in range(3):
        op.spmv_async(xs.data_ptr(), ys.data_ptr(), stream.cuda_stream)
    reps = 20
    f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    f0.record(stream)
    for _ in range(reps):
        op.spmv_async(xs.data_ptr(), ys.data_ptr(), stream.cuda_stream)
    f1.record(stream)
    torch.cuda.synchronize()
    spmv_ms = f0.elapsed_time(f1) / reps
    # the same with L2 flushed (a 256 MB write) before each call, timed one by one
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    flushed = []
    for rep in range(8):
        with torch.cuda.stream(stream):
            flush.fill_(rep)
        g0, g1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        g0.record(stream)
        op.spmv_async(xs.data_ptr(), ys.data_ptr(), stream.cuda_stream)
        g1.record(stream)
        torch.cuda.synchronize()
        flushed.append(g0.elapsed_time(g1))
    spmv_flushed_ms = statistics.median(flushed[2:])
    nnz_g = op.nnz_general()
    spmv_bytes = 12.0 * nnz_g + 4.0 * (m.n + 1) + 16.0 * m.n
    del xs, ys, flush

    # roofline: one profiled solve
    pst = solve_dev(profile=True)
    prof = H.last_profile()
    kernel_classes = ["spmv", "cgs_proj", "cgs_apply", "basis", "ritz"]
    dom = max(kernel_classes, key=lambda k: prof[k]["ms"])
    total_kernel_ms = sum(prof[k]["ms"] for k in kernel_classes + ["aux"])
    peak, peak_src = measured_peaks()
    fp64_peak = H.fp64_peak_tflops(dev)
    d = prof[dom]
    achieved = d["bytes"] / (d["ms"] * 1e-3) / 1e9 if d["ms"] else 0.0
    ratio = read_traffic_ratio(dom)
    traffic = ratio * d["bytes"] / max(d["launches"], 1) if ratio else None
    # share of the dominant kernel's multiply-adds issued as FP64 FMAs: the
    # hybrid CGS kernels run 5 of every 8 projection columns and about half
    # of the update columns in FP64, the rest as exact integer products
    hybrid = m.n >= H.CGS_HYBRID_MIN_ROWS and dom in ("cgs_proj", "cgs_apply")
    fp64_share = cgs_fp64_share(dom, nev, ncv) if hybrid else 1.0
    roofline = {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "peak_source": f"{peak_src} (MEASURED_PEAKS.json hbm_gbs)",
                "traffic": traffic, "traffic_source": "ncu dram bytes / algorithmic bytes (profiles/) x "
                                                          "algorithmic bytes per launch" if ratio else None,
                "bytes_per_launch": d["bytes"] / max(d["launches"], 1),
                "avg_launch_ms": d["ms"] / max(d["launches"], 1),
                "cgs_kernels": "hybrid FP64 + exact integer" if hybrid else "fp64",
                "fp64": {"achieved_tflops": fp64_share * d["flops"] / (d["ms"] * 1e-3) / 1e12 if d["ms"] else 0.0,
                         "peak_tflops": fp64_peak,
                         "frac": (fp64_share * d["flops"] / (d["ms"] * 1e-3) / 1e12) / fp64_peak if d["ms"] else 0.0,
                         "fp64_share_of_flops": fp64_share,
                         "peak_source": "measured live (hlanc_diag_fp64_tflops)"},
                "time_share": {k: prof[k]["ms"] / total_kernel_ms for k in kernel_classes + ["aux"]},
                "host_restart_ms": prof["host_restart"]["ms"]}
    line = {"metric": "converged eigenpairs/s (resid <= 1e-10 ||A||)", "value": value, "unit": "eigenpairs/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64 (fp32 SpMV)" if wl.get("mixed") else "f64",
            "data": "synthetic (seeded generator)", "config": config_of(args, wl, m),
            "valid": bool(valid), "max_residual_over_normA": float(res.max()) / norm_a,
            "solve": {"spmv_calls": stats[-1]["spmv_calls"], "restarts": stats[-1]["restarts"],
                      "cgs_passes": stats[-1]["cgs_passes"], "nconv": stats[-1]["nconv"]},
            "e2e": {"value": world * nev / (e2e_ms / 1e3) if valid else 0.0, "unit": "eigenpairs/s",
                    "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h, "ms_per_step": e2e_ms,
                    "host_buffers": "pinned", "breakdown": e2e_parts[-1]},
            "roofline": roofline, "gpu_launches": launches, "clocks": clk.summary(),
            **({"mixed_vs_fp64": mixed_cmp} if mixed_cmp else {}),
            "spmv": {"us_per_call": spmv_ms * 1e3, "bytes_per_call": spmv_bytes,
                     "achieved_gbs": spmv_bytes / (spmv_ms * 1e-3) / 1e9,
                     "frac_of_hbm": spmv_bytes / (spmv_ms * 1e-3) / 1e9 / measured_peaks()[0],
                     "us_per_call_l2_flushed": spmv_flushed_ms * 1e3,
                     "frac_of_hbm_l2_flushed": spmv_bytes / (spmv_flushed_ms * 1e-3) / 1e9 / measured_peaks()[0],
                     "note": "FP64 CSR SpMV alone, algorithmic bytes 12 nnz + 4(n+1) + 16 n; back-to-back calls "
                             "(the CSR arrays exceed L2, x/y may stay in it) and, separately, each call after a "
                             "256 MB L2 flush"}}
    if rank == 0 and world == 1 and not args.no_cpu:
        full = FULL_SOLVE_SPMV.get(args.workload) or stats[-1]["spmv_calls"]
        line["cpu_baseline"] = cpu_sample(m, wl, os.cpu_count() or 1, full)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if pg is not None:
        pg.destroy_process_group()


if __name__ == "__main__":
    main()
