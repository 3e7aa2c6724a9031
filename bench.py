"""Benchmark: CommonNN fit points/s on the 200,000 x 3 MD-like workload.

One step = one complete fit of 200,000 points in 3D float64 (20
anisotropic Gaussians + 5 % background, mean degree ~215): cell-grid
radius search (r = 0.1) -> CSR, common-neighbour check (c = 10) +
union-find, canonical labels, sort_by_size (member_cutoff = 50).

* ``value``  -- points/s with the points already resident in HBM (device
  pointers through the C ABI), CUDA events around each step on the
  library's stream; L2 is flushed (a 256 MiB write) between steps,
  outside the timed events.
* ``e2e``    -- the same fit through the C ABI with HOST buffers: the
  H2D copy of the points, labels and consider and the D2H copy of labels
  and consider are inside the timed region (pinned host memory).
* ``roofline`` -- the dominant kernel's algorithmic bytes per launch over
  its CUDA-event time (library stage events, same stream).
* ``cpu_baseline`` -- the oracle port of the reference path on this
  host's cores (1 thread, like the reference).

``--impl reference`` times the reference's CPU path instead (the oracle
port: grid-restated neighbour lists on all host threads, then the
reference's BFS with the sorted-merge check on one thread, then
sort_by_size), one full fit per step.

With torchrun (N > 1) every rank fits its own replica of the workload on
its own GPU (the fit does not shard); value = points of all ranks / the
slowest rank's time.
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

WORKLOADS = {
    # the headline workload: 200,000 x 3, cell-grid search
    "md3d-200k": dict(name="md3d-200k", n=200_000, d=3, radius_cutoff=0.1, cnn_cutoff=10, member_cutoff=50,
                      gen=("md3d", {})),
    # 5,000 x 2 blobs (the reference's own brute-force recipe is timed beside it)
    "blobs2d-5k": dict(name="blobs2d-5k", n=5000, d=2, radius_cutoff=0.3, cnn_cutoff=5, member_cutoff=10,
                       gen=("blobs2d", {})),
    # 500,000 x 64 feature vectors, tensor-core Gram search (mean degree ~100)
    "features-500k-d64": dict(name="features-500k-d64", n=500_000, d=64, radius_cutoff=2.9, cnn_cutoff=8,
                              member_cutoff=None, gen=("features", {})),
    # 1,000,000 x 3 float32 nested blobs: 8 radii x 8 cnn_cutoffs in one batched sweep
    "nested3d-1m-sweep": dict(name="nested3d-1m-sweep", n=1_000_000, d=3, radius_cutoff=0.15, cnn_cutoff=None,
                              member_cutoff=None, gen=("nested3d", {}), kind="sweep",
                              radii=[float(r) for r in np.linspace(0.03, 0.15, 8)],
                              cuts=[2, 5, 10, 20, 40, 80, 120, 160]),
    # served request stream: Poisson arrivals of jobs of uneven size and dimension
    "serve-stream": dict(name="serve-stream", n=None, d=None, radius_cutoff=None, cnn_cutoff=None,
                         member_cutoff=10, gen=None, kind="serve", n_jobs=2000, rates=[10.0, 100.0, 500.0]),
    # the same generator at 100,000 points (small enough for a full ncu capture)
    "features-100k-d64": dict(name="features-100k-d64", n=100_000, d=64, radius_cutoff=2.9, cnn_cutoff=8,
                              member_cutoff=None, gen=("features", {})),
}
WORKLOAD = WORKLOADS["md3d-200k"]
METRIC = "CommonNN fit points/s (bit-exact labels)"
UNIT = "points/s"


def fpmode_name() -> str:
    """The float64 accumulation both arms use: the reference as built on this
    host (fused multiply-add on aarch64, separate on x86-64)."""
    from commonnnclustering_gb300 import _abi
    return "fused" if _abi.host_fpmode() == _abi.FP_FUSED else "separate"


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def init_dist(world):
    if world <= 1:
        return None
    import torch.distributed as dist
    os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
    dist.init_process_group("gloo")
    return dist


def reduce_max(dist, v: float) -> float:
    if dist is None:
        return v
    import torch
    t = torch.tensor([v], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(dist):
    if dist is not None:
        dist.barrier()


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.samples = []
        self._stop = threading.Event()
        self._th = None

    def _run(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                                      "--format=csv,noheader,nounits"], capture_output=True, text=True,
                                     timeout=5).stdout.strip()
                if out:
                    self.samples.append([c.strip() for c in out.split(",")])
            except Exception:
                pass
            self._stop.wait(0.2)

    def __enter__(self):
        self._th = threading.Thread(target=self._run, daemon=True)
        self._th.start()
        return self

    def __exit__(self, *a):
        self._stop.set()
        if self._th:
            self._th.join(timeout=6)

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        mx = [float(s[2]) for s in self.samples if s[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4)
                          if len(s) > 5 + i and s[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


def make_points():
    from commonnnclustering_gb300 import workloads
    name, kw = WORKLOAD["gen"]
    return getattr(workloads, name)(n=WORKLOAD["n"], **kw)


def roofline_entry(stats_list, nnz, n, peaks):
    """Dominant kernel by mean stage time; algorithmic bytes per launch."""
    d = WORKLOAD["d"]
    if d >= 16:  # tensor-core Gram kernel: FLOPs of the 128 x 128 tiles it actually computed
        ms = statistics.mean(s["ms_gram"] for s in stats_list)
        nblk = (n + 127) // 128
        all_pairs = nblk * (nblk + 1) // 2 * 128 * 128
        pairs = statistics.mean(s["n_candidates"] for s in stats_list)  # tiles left after pruning x 128^2
        dp = (d + 63) // 64 * 64
        useful = 2.0 * pairs * dp
        issued = 6.0 * useful  # three-way bf16 split: hi.hi + hi.mid + mid.hi + hi.lo + lo.hi + mid.mid
        peak = peaks.get("bf16_tflops")
        achieved = issued / (ms * 1e-3) / 1e12 if ms > 0 else None
        return {
            "kernel": "gram_search_kernel (tcgen05, three-way bf16 split)", "bound": "tensor", "achieved": achieved, "peak": peak,
            "unit": "TFLOP/s", "frac": (achieved / peak) if (achieved and peak) else None, "traffic": None,
            "algorithmic_flops_issued": issued, "algorithmic_flops_useful": useful,
            "tile_pairs_computed": pairs, "tile_pairs_unpruned": all_pairs,
            "useful_tflops": useful / (ms * 1e-3) / 1e12 if ms > 0 else None, "ms_per_launch": ms,
            "peak_source": "MEASURED_PEAKS.json bf16_tflops (measured burst)" if peak else "fallback",
            "stage_ms": {k: round(statistics.mean(s[k] for s in stats_list), 4)
                         for k in ("ms_count", "ms_gram", "ms_check", "ms_label", "ms_sort")},
        }
    stages = {
        # stage -> (kernel name, algorithmic bytes per launch)
        # one pass into per-row slots: float4 coordinates read, rows, lengths and slot starts written
        "ms_count": ("grid_unit_kernel<slots>", 16 * n + 4 * nnz + 4 * n + 8 * n),
        # slots -> compact CSR: rows read and written, offsets read
        "ms_fill": ("compact_rows_kernel", 8 * nnz + 16 * (n + 1)),
        "ms_check": ("check_union_kernel", 4 * nnz + 8 * (n + 1) + n + 8 * n),
        "ms_cells": ("cell binning (assign, scan, place)", 4 * 8 * n),
        "ms_label": ("labelling", 24 * n),
        "ms_sort": ("sort_by_size", 32 * n),
    }
    means = {k: statistics.mean(s[k] for s in stats_list) for k in stages}
    top = max(means, key=means.get)
    kname, bytes_ = stages[top]
    ms = means[top]
    achieved = bytes_ / (ms * 1e-3) / 1e9 if ms > 0 else None
    peak = peaks.get("hbm_gbs")
    traffic = None
    tpath = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(tpath):
        try:
            with open(tpath) as f:
                traffic = json.load(f).get(kname)
        except Exception:
            traffic = None
    return {
        "kernel": kname, "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
        "frac": (achieved / peak) if (achieved and peak) else None, "traffic": traffic,
        "algorithmic_bytes": bytes_, "ms_per_launch": ms,
        "peak_source": "MEASURED_PEAKS.json hbm_gbs (measured)" if "hbm_gbs" in peaks else "fallback 6800",
        "stage_ms": {k: round(v, 4) for k, v in means.items()},
        "other_stage_ms": {k: round(statistics.mean(s.get(k, 0.0) for s in stats_list), 4)
                           for k in ("ms_bbox", "ms_scan", "ms_nodes")},
    }


def cpu_baseline(x, budget_s=25.0):
    from oracle import cnn_oracle
    W = WORKLOAD
    if W["d"] >= 16:
        # all-pairs float64 rows on 1 thread for a sample of query points; the
        # full fit would take hours, so the rate is per query row, stated as such
        rng = np.random.default_rng(0)
        k = 64
        idx = rng.choice(x.shape[0], k, replace=False)
        t = time.perf_counter()
        r2 = W["radius_cutoff"] ** 2
        for i in idx:
            cnn_oracle.neighbour_row(x, int(i), r2)
        dt = time.perf_counter() - t
        per_row = dt / k
        return {"value": 1.0 / per_row, "unit": "query rows/s (neighbour search only)", "cores": 1, "kind": "port",
                "sample": f"{k} brute-force float64 neighbour rows of {W['name']} against all {x.shape[0]} points "
                          f"(oracle restatement of the reference getter), {dt:.1f} s; a full fit needs "
                          f"{x.shape[0]} rows (~{per_row * x.shape[0] / 3600:.1f} h on 1 thread)"}
    if W["name"] == "blobs2d-5k":
        t = time.perf_counter()
        cnn_oracle.clustering_fit(x, W["radius_cutoff"], W["cnn_cutoff"], member_cutoff=W["member_cutoff"],
                                  brute_force=True)
        dt = time.perf_counter() - t
        return {"value": W["n"] / dt, "unit": UNIT, "cores": 1, "kind": "port",
                "sample": f"1 full fit of {W['name']} with the reference's default recipe restated "
                          f"(brute-force getter per query + BFS), {dt:.2f} s"}
    t0 = time.perf_counter()
    times = []
    while True:
        t = time.perf_counter()
        cnn_oracle.clustering_fit(x, W["radius_cutoff"], W["cnn_cutoff"], member_cutoff=W["member_cutoff"],
                                  nthreads=1)
        times.append(time.perf_counter() - t)
        if time.perf_counter() - t0 + times[-1] > budget_s or len(times) >= 3:
            break
    best = min(times)
    return {"value": W["n"] / best, "unit": UNIT, "cores": 1, "kind": "port",
            "sample": f"{len(times)} full fits of {W['name']} (oracle restatement: grid neighbour lists + "
                      f"BFS with sorted-merge check + sort_by_size, 1 thread), best {best:.2f} s"}


def run_gpu(args):
    import torch
    from commonnnclustering_gb300 import _abi

    rank, world, local = dist_env()
    dist = init_dist(world)
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    W = WORKLOAD
    x = make_points()
    n = x.shape[0]
    stream = torch.cuda.Stream(device=dev)
    ctx = _abi.Context(local, stream=int(stream.cuda_stream))
    ctx.set_timing(True)
    xt = torch.from_numpy(x).to(dev)
    labels = torch.zeros(n, dtype=torch.int64, device=dev)
    consider = torch.ones(n, dtype=torch.uint8, device=dev)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    r2 = W["radius_cutoff"] ** 2
    sc, nm = W["cnn_cutoff"] + 2, W["cnn_cutoff"] + 1
    sort_cutoff = W["member_cutoff"] if W["member_cutoff"] is not None else 2  # Labels.sort_by_size default
    torch.cuda.synchronize()

    def step():
        with torch.cuda.stream(stream):
            labels.zero_()
            consider.fill_(1)
        ctx.set_points(xt)
        ctx.build_neighbours(r2)
        ctx.fit(sc, nm, 1, consider, labels)
        ctx.sort_by_size(labels, sort_cutoff, None)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    launches0 = ctx.stats()["n_launches"]
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    stats_list = []
    barrier(dist)
    torch.cuda.synchronize()
    t_wall = time.perf_counter()
    with ClockSampler(local) as clocks:
        for i in range(args.steps):
            with torch.cuda.stream(stream):
                flush.zero_()  # 256 MiB write: evicts L2 between steps
            ev[i][0].record(stream)
            step()
            ev[i][1].record(stream)
            stats_list.append(ctx.stats())
        torch.cuda.synchronize()
    t_wall = time.perf_counter() - t_wall
    barrier(dist)
    step_ms = [a.elapsed_time(b) for a, b in ev]
    mean_ms = statistics.mean(step_ms)
    max_ms = reduce_max(dist, mean_ms)
    launches = (stats_list[-1]["n_launches"] - launches0) // max(args.steps, 1)
    nnz = stats_list[-1]["n_nonzero"]
    check_labels = labels.cpu().numpy()

    # e2e: host buffers through the C ABI (pinned), copies inside the timed region
    x_host = torch.from_numpy(x).pin_memory().numpy()
    lab_host = torch.zeros(n, dtype=torch.int64).pin_memory().numpy()
    con_host = torch.ones(n, dtype=torch.uint8).pin_memory().numpy()
    e2e_ctx = _abi.Context(local)

    def e2e_step():
        lab_host[:] = 0
        con_host[:] = 1
        e2e_ctx.set_points(x_host)
        e2e_ctx.build_neighbours(r2)
        e2e_ctx.fit(sc, nm, 1, con_host, lab_host)
        e2e_ctx.sort_by_size(lab_host, sort_cutoff, None)

    for _ in range(max(1, args.warmup)):
        e2e_step()
    e2e_times = []
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t = time.perf_counter()
        e2e_step()
        e2e_times.append(time.perf_counter() - t)
    e2e_max = reduce_max(dist, statistics.mean(e2e_times))
    if not np.array_equal(lab_host, check_labels):
        raise SystemExit("bench: host-buffer and device-buffer fits disagree")
    h2d = n * W["d"] * 8 + n * 8 * 2 + n      # points, labels (fit + sort), consider
    d2h = n * 8 * 2 + n                       # labels (fit + sort), consider

    if rank != 0:
        return
    peaks = {}
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peaks = json.load(f)
    except Exception:
        peaks = {"hbm_gbs": 6800.0}
    line = {
        "metric": METRIC, "value": world * n / (max_ms * 1e-3), "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": max_ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": f"synthetic (seeded {WORKLOAD['gen'][0]} generator)",
        "config": {"workload": W["name"], "n_points": n, "n_dim": W["d"], "radius_cutoff": W["radius_cutoff"],
                   "cnn_cutoff": W["cnn_cutoff"], "member_cutoff": W["member_cutoff"],
                   "neighbour_pairs": nnz, "l2": "flushed between steps (256 MiB write)",
                   "parallelism": "replicas" if world > 1 else "single", "fpmode": fpmode_name()},
        "e2e": {"value": world * n / e2e_max, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "gpu_launches": int(launches) * args.steps,
        "gpu_launches_per_step": int(launches),
        "clocks": clocks.summary(),
        "roofline": roofline_entry(stats_list, nnz, n, peaks),
        "wall_s_timed_region": t_wall,
        "fit_stats": {k: stats_list[-1][k] for k in ("n_nodes", "n_checks", "n_accepted", "n_exact",
                                                     "n_candidates", "n_clusters", "filter_band", "max_abs_err",
                                                     "search_kind")},
    }
    if world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(x)
    print(json.dumps(line), flush=True)


def run_sweep(args):
    """Batched sweep vs the same 64 fits run one by one (both on the GPU)."""
    import torch
    from commonnnclustering_gb300 import _abi

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    W = WORKLOAD
    x = make_points()  # float32, widened exactly inside the library
    n = x.shape[0]
    radii, cuts = W["radii"], W["cuts"]
    r2 = [r * r for r in radii]
    cut_pairs = [(c + 2, c + 1) for c in cuts]
    stream = torch.cuda.Stream(device=dev)
    ctx = _abi.Context(local, stream=int(stream.cuda_stream))
    xt = torch.from_numpy(x).to(dev)
    out = torch.empty((len(radii), len(cuts), n), dtype=torch.int64, device=dev)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)

    def batched():
        ctx.set_points(xt)
        ctx.sweep(r2, cut_pairs, member_cutoff=2, labels_out=out)

    lab = torch.zeros(n, dtype=torch.int64, device=dev)
    con = torch.ones(n, dtype=torch.uint8, device=dev)

    def one_by_one(check=None):
        for k, rr in enumerate(r2):
            for j, (sc, nm) in enumerate(cut_pairs):
                with torch.cuda.stream(stream):
                    lab.zero_()
                    con.fill_(1)
                ctx.set_points(xt)
                ctx.build_neighbours(rr)
                ctx.fit(sc, nm, 1, con, lab)
                ctx.sort_by_size(lab, 2, None)
                if check is not None:
                    stream.synchronize()  # the library writes lab on its own stream
                if check is not None and not torch.equal(lab, check[k, j]):
                    raise SystemExit(f"bench: sweep differs from the separate fit at r={radii[k]}, c={cuts[j]}")

    def timed(fn, steps):
        ts = []
        for _ in range(steps):
            with torch.cuda.stream(stream):
                flush.zero_()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            fn()
            b.record(stream)
            torch.cuda.synchronize()
            ts.append(a.elapsed_time(b))
        return statistics.mean(ts)

    for _ in range(args.warmup):
        batched()
    one_by_one(check=out)  # also the parity check: every pair equals its separate fit
    with ClockSampler(local) as clocks:
        ms_batched = timed(batched, args.steps)
        ms_plain = timed(one_by_one, max(1, min(args.steps, 2)))
    fits = len(radii) * len(cuts)
    st = ctx.stats()
    if rank != 0:
        return
    line = {
        "metric": METRIC, "value": n * fits / (ms_batched * 1e-3), "unit": "points/s (summed over the fits)",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_batched,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded nested3d generator, float32-stored)",
        "config": {"workload": W["name"], "n_points": n, "n_dim": 3, "radii": radii, "cnn_cutoffs": cuts,
                   "member_cutoff": 2, "fits_per_step": fits, "l2": "flushed between steps (256 MiB write)",
                   "largest_radius_pairs": st["n_nonzero"]},
        "plain_one_by_one_ms": ms_plain, "speedup_vs_one_by_one": ms_plain / ms_batched,
        "fits_per_s": fits / (ms_batched * 1e-3), "clocks": clocks.summary(),
        "gpu_launches_per_step": None,
    }
    print(json.dumps(line), flush=True)


def run_serve(args):
    """Served stream: continuous batching vs one job at a time, per arrival rate."""
    import torch
    from commonnnclustering_gb300 import serve, workloads

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    W = WORKLOAD
    results = []
    t_gen = time.perf_counter()
    raw = workloads.job_stream(n_jobs=W["n_jobs"], rate=1.0, seed=11)
    t_gen = time.perf_counter() - t_gen
    # arrival gaps of the trace at rate 1; each rate rescales them
    base = np.array([j["arrival"] for j in raw])
    srv = serve.Server(n_slots=args.slots, device=local)
    try:
        # warm-up: every slot sees the largest jobs once (device workspaces grown)
        big = sorted(raw, key=lambda j: -j["points"].shape[0] * j["points"].shape[1])[: 2 * args.slots]
        srv.serve([serve.Job(job_id=-1 - i, **dict(j, arrival=0.0)) for i, j in enumerate(big)], realtime=False)
        srv.done.clear()
        for rate in W["rates"]:
            n_jobs = W["n_jobs"] if rate >= 100 else min(W["n_jobs"], int(rate * 60))  # <= 60 s of arrivals
            jobs = [serve.Job(job_id=i, **dict(raw[i], arrival=float(base[i] / rate))) for i in range(n_jobs)]
            srv.done.clear()
            srv.serve(jobs, realtime=True)
            batched = serve.latency_summary(jobs)
            plain_jobs = [serve.Job(job_id=i, **dict(raw[i], arrival=float(base[i] / rate))) for i in range(n_jobs)]
            serve.serve_one_at_a_time(plain_jobs, device=local, realtime=True)
            plain = serve.latency_summary(plain_jobs)
            differ = [(a, b) for a, b in zip(jobs, plain_jobs)
                      if a.labels is None or b.labels is None or not np.array_equal(a.labels, b.labels)]
            detail = []
            for a, b in differ[:5]:
                from commonnnclustering_gb300 import _abi
                c = _abi.Context(local)
                alone = serve.run_job_alone(c, a)  # a fresh context decides which side is off
                c.close()
                detail.append({"job": a.job_id, "n": int(a.points.shape[0]), "d": int(a.points.shape[1]),
                               "radius_cutoff": a.radius_cutoff, "cnn_cutoff": a.cnn_cutoff,
                               "error_mix": a.error, "error_alone": b.error,
                               "mix_equals_fresh": a.labels is not None and bool(np.array_equal(a.labels, alone)),
                               "alone_equals_fresh": b.labels is not None and bool(np.array_equal(b.labels, alone))})
            results.append({"rate_jobs_per_s": rate, "jobs": n_jobs, "continuous_batching": batched,
                            "one_at_a_time": plain, "identical_labels": not differ,
                            "jobs_differing": len(differ), "differing": detail,
                            "max_jobs_in_flight": srv.max_in_flight})
    finally:
        srv.close()
    if rank != 0:
        return
    top = results[-1]
    line = {
        "metric": "served CommonNN fits: jobs/s and p50/p99 latency", "value": top["continuous_batching"]["jobs_per_s"],
        "unit": "jobs/s", "n_gpus": world, "steps": len(results), "warmup": 1, "ms_per_step": None,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded job stream: lognormal sizes, d in {2,3,16,64}, Poisson arrivals)",
        "config": {"workload": W["name"], "n_jobs": W["n_jobs"], "rates": W["rates"], "slots": args.slots,
                   "trace_generation_s": t_gen},
        "per_rate": results,
    }
    print(json.dumps(line), flush=True)


def run_reference(args):
    rank, world, local = dist_env()
    if rank != 0:
        return
    from oracle import cnn_oracle
    W = WORKLOAD
    x = make_points()
    n = x.shape[0]
    cores = max(1, len(os.sched_getaffinity(0)))
    if W["d"] >= 16:
        # the reference's brute-force getter over all pairs is hours per fit
        # here; each step times a bounded sample of query rows on all cores
        base = cpu_baseline(x)
        rows_per_s = base["value"] * cores
        line = {
            "impl": "reference", "metric": METRIC, "value": rows_per_s, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * n / rows_per_s,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded features generator)",
            "config": {"workload": W["name"], "n_points": n, "n_dim": W["d"], "radius_cutoff": W["radius_cutoff"],
                       "cnn_cutoff": W["cnn_cutoff"]},
            "cpu_baseline": {"value": rows_per_s, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": base["sample"] + f"; scaled to {cores} threads; neighbour search only "
                                       "(an upper bound on the fit rate)"},
            "e2e": {"value": rows_per_s, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        }
        print(json.dumps(line), flush=True)
        return

    def step():
        cnn_oracle.clustering_fit(x, W["radius_cutoff"], W["cnn_cutoff"], member_cutoff=W["member_cutoff"],
                                  nthreads=cores)

    for _ in range(args.warmup):
        step()
    times = []
    for _ in range(args.steps):
        t = time.perf_counter()
        step()
        times.append(time.perf_counter() - t)
    mean_s = statistics.mean(times)
    value = n / mean_s
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": mean_s * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": f"synthetic (seeded {WORKLOAD['gen'][0]} generator)",
        "config": {"workload": W["name"], "n_points": n, "n_dim": W["d"], "radius_cutoff": W["radius_cutoff"],
                   "cnn_cutoff": W["cnn_cutoff"], "member_cutoff": W["member_cutoff"], "fpmode": fpmode_name()},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": f"full {W['name']} fit per step: neighbour lists restated on {cores} threads, "
                                   "the reference's BFS + sorted-merge check on 1 thread, sort_by_size"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--workload", default="md3d-200k", choices=sorted(WORKLOADS))
    ap.add_argument("--slots", type=int, default=4, help="concurrent jobs of the served stream")
    args = ap.parse_args()
    global WORKLOAD
    WORKLOAD = WORKLOADS[args.workload]
    if args.warmup < 3 and args.impl != "reference":
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    elif WORKLOAD.get("kind") == "sweep":
        run_sweep(args)
    elif WORKLOAD.get("kind") == "serve":
        run_serve(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
