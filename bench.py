"""Benchmark: CommonNN fit points/s, headline on the 200,000 x 3 MD-like workload.

One step of the headline = one complete fit of 200,000 points in 3D float64
(20 anisotropic Gaussians + 5 % background, mean degree ~215): cell-grid
radius search (r = 0.1) -> neighbour graph, common-neighbour check (c = 10)
+ union-find, canonical labels, sort_by_size (member_cutoff = 50).

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
* ``workloads`` -- the other four workloads, each with its own value, e2e,
  roofline, clocks and CPU baseline: ``blobs2d-5k`` (5,000 x 2),
  ``features-500k-d64`` (tensor-core search, beside the plain float32
  all-pairs search on the same points), ``nested3d-1m-sweep`` (64 (r, c)
  fits in one batched call, beside the same fits one by one) and
  ``serve-stream`` (continuous batching of a job stream, beside one job at
  a time).  ``--headline-only`` skips them; ``--workload NAME`` runs one
  workload as the only line.

``--impl reference`` times the reference's CPU path instead (the oracle
port: grid-restated neighbour lists on all host threads, then the
reference's BFS with the sorted-merge check on one thread, then
sort_by_size), one full fit of the headline workload per step.

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
                              member_cutoff=None, gen=("features", {}), max_steps=5),
    # 1,000,000 x 3 float32 nested blobs: 8 radii x 8 cnn_cutoffs in one batched sweep
    "nested3d-1m-sweep": dict(name="nested3d-1m-sweep", n=1_000_000, d=3, radius_cutoff=0.15, cnn_cutoff=None,
                              member_cutoff=None, gen=("nested3d", {}), kind="sweep", max_steps=3,
                              radii=[float(r) for r in np.linspace(0.03, 0.15, 8)],
                              cuts=[2, 5, 10, 20, 40, 80, 120, 160], cpu_subsample=20),
    # served request stream: Poisson arrivals of jobs of uneven size and dimension
    "serve-stream": dict(name="serve-stream", n=None, d=None, radius_cutoff=None, cnn_cutoff=None,
                         member_cutoff=10, gen=None, kind="serve", n_jobs=2000, rates=[10.0, 100.0, 500.0]),
    # the same stream shortened for the default run: 400 jobs at 100 and 500 jobs/s
    "serve-stream-short": dict(name="serve-stream", n=None, d=None, radius_cutoff=None, cnn_cutoff=None,
                               member_cutoff=10, gen=None, kind="serve", n_jobs=400, rates=[100.0, 500.0]),
    # the same generator at 100,000 points (small enough for a full ncu capture)
    "features-100k-d64": dict(name="features-100k-d64", n=100_000, d=64, radius_cutoff=2.9, cnn_cutoff=8,
                              member_cutoff=None, gen=("features", {})),
}
HEADLINE = "md3d-200k"
SUB_WORKLOADS = ["blobs2d-5k", "features-500k-d64", "nested3d-1m-sweep", "serve-stream-short"]
METRIC = "CommonNN fit points/s (bit-exact labels)"
INTERSECTIONS = {"auto": 0, "merge": 1, "bitset": 2}  # cnn_intersection
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


def load_peaks() -> dict:
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f)
    except Exception:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "_fallback": True}


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


def make_points(W):
    from commonnnclustering_gb300 import workloads
    name, kw = W["gen"]
    return getattr(workloads, name)(n=W["n"], **kw)


# ---------------------------------------------------------------------------
# rooflines
# ---------------------------------------------------------------------------
def tensor_roofline(W, stats_list, n, peaks):
    """Gram kernel: FLOPs of the 128 x 128 tiles it computed (useful and issued)."""
    d = W["d"]
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
        "kernel": "gram_search_kernel (tcgen05, three-way bf16 split)", "bound": "tensor", "achieved": achieved,
        "peak": peak, "unit": "TFLOP/s", "frac": (achieved / peak) if (achieved and peak) else None, "traffic": None,
        "algorithmic_flops_issued": issued, "algorithmic_flops_useful": useful,
        "tile_pairs_computed": pairs, "tile_pairs_unpruned": all_pairs,
        "useful_tflops": useful / (ms * 1e-3) / 1e12 if ms > 0 else None,
        "useful_frac": (useful / (ms * 1e-3) / 1e12 / peak) if (ms > 0 and peak) else None,
        "ms_per_launch": ms,
        "peak_source": "MEASURED_PEAKS.json bf16_tflops (measured burst)" if not peaks.get("_fallback") else "fallback",
        "stage_ms": {k: round(statistics.mean(s[k] for s in stats_list), 4)
                     for k in ("ms_count", "ms_gram", "ms_check", "ms_label", "ms_sort")},
    }


def hbm_roofline(stats_list, nnz, n, peaks, workload=None):
    """Dominant stage by mean CUDA-event time; algorithmic bytes per launch.
    `traffic` comes from the committed ncu capture, which holds one
    workload's launches: other workloads report null."""
    stages = {
        # stage -> (kernel name, algorithmic bytes per launch)
        # one pass into per-row slots: float4 coordinates read, rows, lengths and slot starts written
        "ms_count": ("grid_unit_kernel<slots>", 16 * n + 4 * nnz + 4 * n + 8 * n),
        # rows left in their slots (a public build): each row's end and split
        # point -- start and length read, end and split written, ~8 entries
        # bisected per row; the compaction to CSR runs only when asked for
        "ms_fill": ("row_split_kernel", 8 * n + 4 * n + 8 * n + 4 * n + 32 * n),
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
                tj = json.load(f)
            if tj.get("_workload") == workload:
                traffic = tj.get(kname)
        except Exception:
            traffic = None
    return {
        "kernel": kname, "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
        "frac": (achieved / peak) if (achieved and peak) else None, "traffic": traffic,
        "algorithmic_bytes": bytes_, "ms_per_launch": ms,
        "peak_source": "MEASURED_PEAKS.json hbm_gbs (measured)" if not peaks.get("_fallback") else "fallback 6800",
        "stage_ms": {k: round(v, 4) for k, v in means.items()},
        "other_stage_ms": {k: round(statistics.mean(s.get(k, 0.0) for s in stats_list), 4)
                           for k in ("ms_bbox", "ms_scan", "ms_nodes")},
    }


def issue_roofline(roof, workload, sm_count, clocks):
    """The dominant kernel against the SM issue rate, for a kernel that is
    issue-bound rather than HBM-bound (the cell-grid search): warp
    instructions of one launch from the committed ncu capture of this
    workload, over the live launch time, against 4 warp instructions per SM
    per cycle at the median SM clock sampled during the run."""
    tpath = os.path.join(ROOT, "profiles", "traffic.json")
    try:
        with open(tpath) as f:
            tj = json.load(f)
    except Exception:
        return None
    if tj.get("_workload") != workload:
        return None
    inst = (tj.get("_issue") or {}).get(roof.get("kernel"))
    mhz = (clocks or {}).get("sm_mhz") or (clocks or {}).get("sm_max_mhz")
    ms = roof.get("ms_per_launch")
    if not inst or not mhz or not ms or not sm_count:
        return None
    achieved = inst / (ms * 1e-3)
    peak = 4.0 * sm_count * mhz * 1e6
    return {"warp_instructions": inst, "achieved": achieved, "peak": peak, "unit": "warp instructions/s",
            "frac": achieved / peak, "source": tj.get("_issue_source")}


# ---------------------------------------------------------------------------
# CPU baselines (the oracle port of the reference path; bounded samples)
# ---------------------------------------------------------------------------
def cpu_baseline(W, x, budget_s=25.0):
    from oracle import cnn_oracle
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


# ---------------------------------------------------------------------------
# one fit per step (md3d-200k, blobs2d-5k, features-500k-d64)
# ---------------------------------------------------------------------------
def fit_record(W, args, peaks, dist=None, world=1, local=0, rank=0, cpu=True):
    import torch
    from commonnnclustering_gb300 import _abi

    dev = torch.device("cuda", local)
    steps = min(args.steps, W.get("max_steps", args.steps))
    x = make_points(W)
    n = x.shape[0]
    stream = torch.cuda.Stream(device=dev)
    ctx = _abi.Context(local, stream=int(stream.cuda_stream))
    ctx.set_timing(True)
    ctx.set_intersection(INTERSECTIONS[args.intersection])
    xt = torch.from_numpy(x).to(dev)
    labels = torch.zeros(n, dtype=torch.int64, device=dev)
    consider = torch.ones(n, dtype=torch.uint8, device=dev)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    r2 = W["radius_cutoff"] ** 2
    sc, nm = W["cnn_cutoff"] + 2, W["cnn_cutoff"] + 1
    sort_cutoff = W["member_cutoff"] if W["member_cutoff"] is not None else 2  # Labels.sort_by_size default
    torch.cuda.synchronize()

    def step():
        # the search, then Clustering.fit from fresh labels + sort_by_size
        # as one library call (cnn_fit_fresh: fresh arrays made on the device)
        ctx.set_points(xt)
        ctx.build_neighbours(r2)
        ctx.fit_fresh(sc, nm, True, sort_cutoff, None, labels=labels, consider=consider)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    launches0 = ctx.stats()["n_launches"]
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    stats_list = []
    barrier(dist)
    torch.cuda.synchronize()
    t_wall = time.perf_counter()
    with ClockSampler(local) as clocks:
        for i in range(steps):
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
    launches = (stats_list[-1]["n_launches"] - launches0) // max(steps, 1)
    nnz = stats_list[-1]["n_nonzero"]
    check_labels = labels.cpu().numpy()

    # the plain float32 all-pairs search on the same points (tensor-core workloads)
    plain = None
    if W["d"] >= 16:
        ctx.set_search(_abi.SEARCH_ALL_PAIRS)
        plain_labels = torch.zeros(n, dtype=torch.int64, device=dev)
        plain_cons = torch.ones(n, dtype=torch.uint8, device=dev)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            flush.zero_()
        a.record(stream)
        ctx.set_points(xt)
        ctx.build_neighbours(r2)
        ctx.fit(sc, nm, 1, plain_cons, plain_labels)
        ctx.sort_by_size(plain_labels, sort_cutoff, None)
        b.record(stream)
        torch.cuda.synchronize()
        pst = ctx.stats()
        ctx.set_search(_abi.SEARCH_AUTO)
        plain_ms = a.elapsed_time(b)
        plain = {"search": "tiled all-pairs float32 + float64 band (tile_search_kernel)", "ms_per_fit": plain_ms,
                 "search_kind": pst["search_kind"], "identical_labels": bool(torch.equal(plain_labels, labels)),
                 "identical_neighbour_count": pst["n_nonzero"] == nnz,
                 "speedup_of_tensor_core_path": plain_ms / mean_ms}

    # e2e: host buffers through the C ABI (pinned), copies inside the timed region
    x_host = torch.from_numpy(x).pin_memory().numpy()
    lab_host = torch.zeros(n, dtype=torch.int64).pin_memory().numpy()
    con_host = torch.ones(n, dtype=torch.uint8).pin_memory().numpy()
    e2e_ctx = _abi.Context(local)
    e2e_ctx.set_intersection(INTERSECTIONS[args.intersection])

    def e2e_step():
        # Clustering.fit with fresh labels + sort_by_size: one library call
        # after the search (cnn_fit_fresh), labels and consider back on the host
        e2e_ctx.set_points(x_host)
        e2e_ctx.build_neighbours(r2)
        e2e_ctx.fit_fresh(sc, nm, True, sort_cutoff, None, labels=lab_host, consider=con_host)

    for _ in range(max(1, min(args.warmup, 3))):
        e2e_step()
    e2e_times = []
    for _ in range(steps):
        flush.zero_()
        torch.cuda.synchronize()
        t = time.perf_counter()
        e2e_step()
        e2e_times.append(time.perf_counter() - t)
    e2e_max = reduce_max(dist, statistics.mean(e2e_times))
    if not np.array_equal(lab_host, check_labels):
        raise SystemExit(f"bench: host-buffer and device-buffer fits of {W['name']} disagree")
    e2e_ctx.close()
    h2d = n * W["d"] * 8                      # points (fresh labels and consider are made on the device)
    d2h = n * 8                               # labels (consider is all 0 after the fit: set on the host)
    ctx.close()
    if rank != 0:
        return None
    rec = {
        "metric": METRIC, "value": world * n / (max_ms * 1e-3), "unit": UNIT, "n_gpus": world,
        "steps": steps, "warmup": args.warmup, "ms_per_step": max_ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": f"synthetic (seeded {W['gen'][0]} generator)",
        "config": {"workload": W["name"], "n_points": n, "n_dim": W["d"], "radius_cutoff": W["radius_cutoff"],
                   "cnn_cutoff": W["cnn_cutoff"], "member_cutoff": W["member_cutoff"],
                   "neighbour_pairs": nnz, "l2": "flushed between steps (256 MiB write)",
                   "parallelism": "replicas" if world > 1 else "single", "fpmode": fpmode_name()},
        "e2e": {"value": world * n / e2e_max, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "gpu_launches": int(launches) * steps,
        "gpu_launches_per_step": int(launches),
        "clocks": clocks.summary(),
        "roofline": (tensor_roofline(W, stats_list, n, peaks) if W["d"] >= 16
                     else hbm_roofline(stats_list, nnz, n, peaks, W["name"])),
        "wall_s_timed_region": t_wall,
        "fit_stats": {k: stats_list[-1][k] for k in ("n_nodes", "n_checks", "n_accepted", "n_exact",
                                                     "n_candidates", "n_clusters", "filter_band", "max_abs_err",
                                                     "search_kind")},
        "intersection": {"requested": args.intersection,
                         "used": {1: "merge", 2: "bitset"}.get(stats_list[-1]["intersection"], "none")},
    }
    if W["d"] < 16:
        sm_count = torch.cuda.get_device_properties(dev).multi_processor_count
        issue = issue_roofline(rec["roofline"], W["name"], sm_count, rec["clocks"])
        if issue:
            rec["roofline"]["issue"] = issue
    if W["d"] >= 16:
        rec["fit_stats"]["recheck_fraction"] = (stats_list[-1]["n_exact"] / stats_list[-1]["n_candidates"]
                                                if stats_list[-1]["n_candidates"] else None)
    if plain is not None:
        rec["plain_gpu"] = plain
    if cpu and world == 1 and not args.no_cpu_baseline:
        rec["cpu_baseline"] = cpu_baseline(W, x)
    return rec


# ---------------------------------------------------------------------------
# batched sweep: 64 (radius, cut) fits per step
# ---------------------------------------------------------------------------
def sweep_cpu_baseline(W, x):
    """The reference's way of scanning the 64 pairs (one full fit each) on a
    documented subsample: every k-th point, oracle fits on 1 thread."""
    from oracle import cnn_oracle
    k = W["cpu_subsample"]
    xs = np.ascontiguousarray(x[::k], dtype=np.float64)
    t = time.perf_counter()
    fits = 0
    for r in W["radii"]:
        for c in W["cuts"]:
            if time.perf_counter() - t > 30.0:
                break
            cnn_oracle.clustering_fit(xs, r, c, member_cutoff=2, nthreads=1)
            fits += 1
    dt = time.perf_counter() - t
    return {"value": xs.shape[0] * fits / dt, "unit": "points/s (summed over the fits)", "cores": 1, "kind": "port",
            "sample": f"{fits} of the 64 (r, c) fits on every {k}th point ({xs.shape[0]} points, the same box, so "
                      f"1/{k} of the density) with the oracle restatement (grid neighbour lists + BFS + "
                      f"sort_by_size, 1 thread), {dt:.1f} s; not extrapolated to 1,000,000 points"}


def sweep_record(W, args, peaks, dist=None, world=1, local=0, rank=0, cpu=True):
    """Batched sweep vs the same 64 fits run one by one (both on the GPU)."""
    import torch
    from commonnnclustering_gb300 import _abi

    dev = torch.device("cuda", local)
    steps = min(args.steps, W.get("max_steps", args.steps))
    x = make_points(W)  # float32, widened exactly inside the library
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
    nnz_by_radius = {}

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
                    nnz_by_radius[k] = ctx.neighbour_count()
                    if not torch.equal(lab, check[k, j]):
                        raise SystemExit(f"bench: sweep differs from the separate fit at r={radii[k]}, c={cuts[j]}")

    def timed(fn, nsteps):
        ts = []
        for _ in range(nsteps):
            with torch.cuda.stream(stream):
                flush.zero_()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            fn()
            b.record(stream)
            torch.cuda.synchronize()
            ts.append(a.elapsed_time(b))
        return statistics.mean(ts)

    for _ in range(max(1, min(args.warmup, 3))):
        batched()
    torch.cuda.synchronize()
    l0 = ctx.stats()["n_launches"]
    batched()
    torch.cuda.synchronize()
    sw = ctx.stats()  # this sweep's kernels and the CUDA graphs its fits ran as
    kernels_per_step = int(sw["n_launches"] - l0)
    one_by_one(check=out)  # also the parity check: every pair equals its separate fit
    with ClockSampler(local) as clocks:
        ms_batched = timed(batched, steps)
        ms_plain = timed(one_by_one, 1)
    ms_batched = reduce_max(dist, ms_batched)
    fits = len(radii) * len(cuts)
    st = ctx.stats()

    # e2e: host points in, host labels out (pinned buffers), through the
    # public sweep call
    e2e_ctx = _abi.Context(local)
    x_host = torch.from_numpy(x).pin_memory().numpy()
    got = torch.empty((len(radii), len(cuts), n), dtype=torch.int64).pin_memory().numpy()
    e2e_ctx.set_points(x_host)
    e2e_ctx.sweep(r2, cut_pairs, member_cutoff=2, labels_out=got)
    e2e_times = []
    for _ in range(steps):
        flush.zero_()
        torch.cuda.synchronize()
        t = time.perf_counter()
        e2e_ctx.set_points(x_host)
        e2e_ctx.sweep(r2, cut_pairs, member_cutoff=2, labels_out=got)
        e2e_times.append(time.perf_counter() - t)
    if not np.array_equal(got, out.cpu().numpy()):
        raise SystemExit("bench: host-buffer and device-buffer sweeps disagree")
    e2e_ctx.close()
    e2e_s = reduce_max(dist, statistics.mean(e2e_times))
    ctx.close()
    if rank != 0:
        return None
    # whole-step algorithmic bytes: the largest-radius graph written once,
    # every smaller radius's graph written once, and one pass of each fit
    # over its graph (int32 entries + per-point offsets, flags and labels)
    nnz_max = nnz_by_radius[len(radii) - 1]
    bytes_step = 4 * nnz_max + sum(4 * nnz_by_radius[k] for k in range(len(radii) - 1)) + \
        sum(len(cuts) * (4 * nnz_by_radius[k] + 24 * n) for k in range(len(radii)))
    achieved = bytes_step / (ms_batched * 1e-3) / 1e9
    peak = peaks.get("hbm_gbs")
    rec = {
        "metric": METRIC, "value": world * n * fits / (ms_batched * 1e-3), "unit": "points/s (summed over the fits)",
        "n_gpus": world, "steps": steps, "warmup": args.warmup, "ms_per_step": ms_batched,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded nested3d generator, float32-stored)",
        "config": {"workload": W["name"], "n_points": n, "n_dim": 3, "radii": radii, "cnn_cutoffs": cuts,
                   "member_cutoff": 2, "fits_per_step": fits, "l2": "flushed between steps (256 MiB write)",
                   "largest_radius_pairs": nnz_max, "pairs_by_radius": [nnz_by_radius[k] for k in range(len(radii))],
                   "fpmode": fpmode_name()},
        "e2e": {"value": world * n * fits / e2e_s, "unit": "points/s (summed over the fits)",
                "h2d_bytes_per_step": n * 3 * 4, "d2h_bytes_per_step": fits * n * 8},
        "gpu_launches": kernels_per_step * steps,
        "gpu_launches_per_step": kernels_per_step,
        "cuda_graph": {"graphs_per_step": sw["graphs"], "nodes_per_step": sw["graph_nodes"],
                       "ms_capture_and_instantiate": round(sw["ms_graph_build"], 3),
                       "note": "the 64 fits (with their sorts and open-pair lists) run as captured graphs; "
                               "the searches, radius buckets and graph fills before them are plain launches"},
        "e2e_ms_steps": [round(1e3 * t, 2) for t in e2e_times],
        "plain_gpu": {"path": "the same 64 fits one by one (search + fit + sort_by_size each)",
                      "ms_per_step": ms_plain, "speedup_of_batched_sweep": ms_plain / ms_batched},
        "fits_per_s": fits / (ms_batched * 1e-3),
        "clocks": clocks.summary(),
        "roofline": {"kernel": "whole sweep step (search at r_max, radius buckets, graphs of all radii, 64 fits)",
                     "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak if peak else None, "traffic": None,
                     "algorithmic_bytes": bytes_step, "ms_per_launch": ms_batched,
                     "peak_source": "MEASURED_PEAKS.json hbm_gbs (measured)"},
        "last_fit_stats": {k: st[k] for k in ("n_nodes", "n_checks", "n_accepted", "n_clusters")},
    }
    if cpu and world == 1 and not args.no_cpu_baseline:
        rec["cpu_baseline"] = sweep_cpu_baseline(W, x)
    return rec


# ---------------------------------------------------------------------------
# served stream
# ---------------------------------------------------------------------------
def serve_cpu_baseline(raw, budget_s=20.0):
    """Sequential per-job reference fits: the oracle restatement, neighbour
    lists on all host threads and the BFS on one, as the reference arm runs
    the headline workload."""
    from oracle import cnn_oracle
    cores = max(1, len(os.sched_getaffinity(0)))
    t = time.perf_counter()
    done, pts = 0, 0
    for j in raw:
        if time.perf_counter() - t > budget_s:
            break
        x = j["points"]
        if x.shape[1] >= 16:
            # the rows of a d >= 16 job come from the pivot-pruned exact scan;
            # the reference itself would run its O(n^2) getter
            csr = cnn_oracle.neighbourhoods(x, j["radius_cutoff"] ** 2, grid="pivot", nthreads=cores)
        else:
            csr = cnn_oracle.neighbourhoods(x, j["radius_cutoff"] ** 2, nthreads=cores)
        cnn_oracle.clustering_fit(x, j["radius_cutoff"], j["cnn_cutoff"], member_cutoff=j["member_cutoff"],
                                  neighbours=csr)
        done += 1
        pts += x.shape[0]
    dt = time.perf_counter() - t
    return {"value": done / dt, "unit": "jobs/s", "cores": cores, "kind": "port",
            "sample": f"the first {done} jobs of the stream ({pts} points) fitted one after another by the "
                      f"oracle restatement (grid or pivot-pruned neighbour lists on {cores} threads, BFS + "
                      f"sort_by_size on 1), {dt:.1f} s; {pts / dt:.0f} points/s"}


def serve_record(W, args, peaks, dist=None, world=1, local=0, rank=0, cpu=True):
    """Served stream: continuous batching vs one job at a time, per arrival rate."""
    from commonnnclustering_gb300 import serve, workloads

    results = []
    t_gen = time.perf_counter()
    raw = workloads.job_stream(n_jobs=W["n_jobs"], rate=1.0, seed=11)
    t_gen = time.perf_counter() - t_gen
    # arrival gaps of the trace at rate 1; each rate rescales them
    base = np.array([j["arrival"] for j in raw])
    srv = serve.Server(n_slots=args.slots, device=local)
    clocks = ClockSampler(local)
    try:
        # warm-up: every slot sees the largest jobs once (device workspaces grown)
        big = sorted(raw, key=lambda j: -j["points"].shape[0] * j["points"].shape[1])[: 2 * args.slots]
        srv.serve([serve.Job(job_id=-1 - i, **dict(j, arrival=0.0)) for i, j in enumerate(big)], realtime=False)
        with clocks:
            for rate in W["rates"]:
                n_jobs = W["n_jobs"] if rate >= 100 else min(W["n_jobs"], int(rate * 60))  # <= 60 s of arrivals
                jobs = [serve.Job(job_id=i, **dict(raw[i], arrival=float(base[i] / rate))) for i in range(n_jobs)]
                srv.serve(jobs, realtime=True)
                batched = serve.latency_summary(jobs)
                plain_jobs = [serve.Job(job_id=i, **dict(raw[i], arrival=float(base[i] / rate)))
                              for i in range(n_jobs)]
                serve.serve_one_at_a_time(plain_jobs, device=local, realtime=True)
                plain = serve.latency_summary(plain_jobs)
                differ = [(a, b) for a, b in zip(jobs, plain_jobs)
                          if a.labels is None or b.labels is None or not np.array_equal(a.labels, b.labels)]
                results.append({"rate_jobs_per_s": rate, "jobs": n_jobs, "continuous_batching": batched,
                                "one_at_a_time": plain, "identical_labels": not differ,
                                "jobs_differing": len(differ),
                                "errors": sorted({a.error for a, _ in differ if a.error} |
                                                 {b.error for _, b in differ if b.error})[:3],
                                "max_jobs_in_flight": srv.max_in_flight,
                                "server": {k: srv.stats[k] for k in ("budget_bytes", "peak_held_bytes", "requeued",
                                                                     "released", "failed")}})
    finally:
        srv.close()
    if rank != 0:
        return None
    top = results[-1]
    sizes = np.array([j["points"].shape[0] for j in raw])
    dims = np.array([j["points"].shape[1] for j in raw])
    rec = {
        "metric": "served CommonNN fits: jobs/s and p50/p99 latency", "value": top["continuous_batching"]["jobs_per_s"],
        "unit": "jobs/s", "n_gpus": world, "steps": len(results), "warmup": 1, "ms_per_step": None,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded job stream: lognormal sizes, d in {2,3,16,64}, Poisson arrivals)",
        "config": {"workload": W["name"], "n_jobs": W["n_jobs"], "rates": W["rates"], "slots": args.slots,
                   "trace_generation_s": t_gen, "points_per_job_median": float(np.median(sizes)),
                   "points_per_job_max": int(sizes.max()),
                   "jobs_by_dim": {str(d): int((dims == d).sum()) for d in (2, 3, 16, 64)},
                   "fpmode": fpmode_name()},
        # jobs arrive as host arrays and leave as host labels: the value is already end to end
        "e2e": {"value": top["continuous_batching"]["jobs_per_s"], "unit": "jobs/s",
                "h2d_bytes_per_step": int(sum(j["points"].nbytes for j in raw[:top["jobs"]])),
                "d2h_bytes_per_step": int(sum(8 * j["points"].shape[0] for j in raw[:top["jobs"]]))},
        "p50_ms": top["continuous_batching"]["p50_ms"], "p99_ms": top["continuous_batching"]["p99_ms"],
        "plain_gpu": {"path": "one job at a time on one context", "jobs_per_s": top["one_at_a_time"]["jobs_per_s"],
                      "p50_ms": top["one_at_a_time"]["p50_ms"], "p99_ms": top["one_at_a_time"]["p99_ms"],
                      "speedup_of_continuous_batching": (top["continuous_batching"]["jobs_per_s"] /
                                                         top["one_at_a_time"]["jobs_per_s"])},
        "per_rate": results,
        "clocks": clocks.summary(),
        "roofline": None,
        "roofline_note": "a mix of jobs of every size and dimension; the kernels' rooflines are those of the fit "
                         "workloads",
    }
    if cpu and world == 1 and not args.no_cpu_baseline:
        rec["cpu_baseline"] = serve_cpu_baseline(raw)
    return rec


def record_for(name, args, peaks, **kw):
    W = WORKLOADS[name]
    kind = W.get("kind")
    if kind == "sweep":
        return sweep_record(W, args, peaks, **kw)
    if kind == "serve":
        return serve_record(W, args, peaks, **kw)
    return fit_record(W, args, peaks, **kw)


def run_gpu(args):
    import torch

    rank, world, local = dist_env()
    dist = init_dist(world)
    torch.cuda.set_device(local)
    peaks = load_peaks()
    name = args.workload or HEADLINE
    line = record_for(name, args, peaks, dist=dist, world=world, local=local, rank=rank)
    if args.workload is None and not args.headline_only and world == 1:
        subs = {}
        for sub in SUB_WORKLOADS:
            key = WORKLOADS[sub]["name"]
            t = time.perf_counter()
            try:
                subs[key] = record_for(sub, args, peaks, dist=dist, world=world, local=local, rank=rank)
            except SystemExit:
                raise
            except Exception as e:  # a failing sub-workload is reported; the headline still stands
                subs[key] = {"error": f"{type(e).__name__}: {e}"}
            if subs[key] is not None:
                subs[key]["bench_wall_s"] = time.perf_counter() - t
        if line is not None:
            line["workloads"] = subs
    if line is not None:
        print(json.dumps(line), flush=True)


def run_reference(args):
    rank, world, local = dist_env()
    if rank != 0:
        return
    from oracle import cnn_oracle
    W = WORKLOADS[args.workload or HEADLINE]
    if W.get("kind"):
        print(json.dumps({"impl": "reference", "unavailable": f"the reference arm times the fit workloads; "
                                                              f"{W['name']} reports its CPU baseline in its own "
                                                              f"record"}), flush=True)
        return
    x = make_points(W)
    n = x.shape[0]
    cores = max(1, len(os.sched_getaffinity(0)))
    if W["d"] >= 16:
        # the reference's brute-force getter over all pairs is hours per fit
        # here; each step times a bounded sample of query rows on all cores
        base = cpu_baseline(W, x)
        rows_per_s = base["value"] * cores
        line = {
            "impl": "reference", "metric": METRIC, "value": rows_per_s, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * n / rows_per_s,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded features generator)",
            "config": {"workload": W["name"], "n_points": n, "n_dim": W["d"], "radius_cutoff": W["radius_cutoff"],
                       "cnn_cutoff": W["cnn_cutoff"], "fpmode": fpmode_name()},
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
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": f"synthetic (seeded {W['gen'][0]} generator)",
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
    ap.add_argument("--headline-only", action="store_true", help="skip the other workloads' sub-records")
    ap.add_argument("--workload", default=None, choices=sorted(WORKLOADS),
                    help="run this workload alone as the only line (default: the headline plus sub-records)")
    ap.add_argument("--slots", type=int, default=4, help="concurrent jobs of the served stream")
    ap.add_argument("--intersection", default="auto", choices=sorted(INTERSECTIONS),
                    help="intersection strategy of the fit workloads (auto: the library's tuner picks)")
    args = ap.parse_args()
    if args.warmup < 3 and args.impl != "reference":
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
