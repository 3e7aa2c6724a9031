"""A served stream of clustering jobs with continuous batching.

Jobs (points + radius_cutoff, cnn_cutoff, member_cutoff) arrive over time.
The library's job server (cnn_server_create / cnn_submit / cnn_wait, in
csrc/server.cu) owns ``n_slots`` contexts, each with its own CUDA stream,
device-resident workspace that persists across jobs, and a native worker
thread.  It admits a waiting job as soon as a slot is free AND its
reservation fits the budget -- the oldest job first, and when the oldest does
not fit yet, any later job that does (backfill, bounded by aging), so small
jobs keep flowing past a large one.  A running job's context cannot grow
past its reservation, so the budget bounds the device memory really held,
not an estimate.  Admitted jobs run concurrently on their slots' streams.

Each job is one ``Clustering.fit`` (fresh labels, current_start 1, then
sort_by_size) through the C ABI with host buffers, so its result does not
depend on what else is running: ``tests/test_gpu_serve.py`` checks every
job alone against the same job in the mix.
"""
from __future__ import annotations

import time
from dataclasses import dataclass
from typing import Callable, List, Optional

import numpy as np

from . import _abi


@dataclass
class Job:
    job_id: int
    points: np.ndarray
    radius_cutoff: float
    cnn_cutoff: int
    member_cutoff: Optional[int] = 10
    arrival: float = 0.0             # seconds from the start of the stream
    expected_degree: float = 300.0   # for the footprint estimate
    labels: Optional[np.ndarray] = None
    t_admit: Optional[float] = None
    t_done: Optional[float] = None
    slot: Optional[int] = None
    error: Optional[str] = None

    @property
    def latency(self) -> Optional[float]:
        if self.t_done is None:
            return None
        return self.t_done - self.arrival


def footprint_bytes(n: int, d: int, expected_degree: float) -> int:
    """Device bytes a fit of n x d points needs (upper estimate)."""
    pts = n * d * 8
    graph = int(n * expected_degree * 4 * 1.25) + n * 48
    work = n * 64
    if d >= 16:  # bf16 split, float norms, key and band lists of the tensor-core search
        dp = (d + 63) // 64 * 64
        graph += n * dp * 4 + n * 256 * 8 + n * 64 * 12
    elif d > 3:
        graph += n * d * 4
    else:
        graph += n * 32 + min(64 * n, 1 << 26) * 12
    return pts + graph + work


def run_job_alone(ctx: _abi.Context, job: Job) -> np.ndarray:
    """One job as Clustering.fit runs it from fresh labels, then
    sort_by_size (host buffers; cnn_fit_fresh, the call the server makes)."""
    x = np.ascontiguousarray(job.points)
    ctx.set_points(x)
    ctx.build_neighbours(job.radius_cutoff ** 2)
    return ctx.fit_fresh(job.cnn_cutoff + 2, job.cnn_cutoff + 1, True,
                         2 if job.member_cutoff is None else job.member_cutoff, None)


class Server:
    """Continuous batching through the library's job server (cnn_submit /
    cnn_wait): ``n_slots`` contexts with their own streams and native worker
    threads; admission under ``hbm_budget_bytes``, which bounds the device
    bytes the slots' workspaces really hold (a job that outgrows its
    estimate runs again alone with the whole budget)."""

    def __init__(self, n_slots: int = 4, hbm_budget_bytes: Optional[int] = None, device: int = 0,
                 backfill: bool = True):
        if hbm_budget_bytes is None:
            try:
                import torch
                free, _ = torch.cuda.mem_get_info(device)
                hbm_budget_bytes = int(free * 0.6)
            except Exception:
                hbm_budget_bytes = 32 << 30
        self.budget = int(hbm_budget_bytes)
        self.backfill = backfill  # the library always backfills (bounded by aging)
        self.native = _abi.NativeServer(device, n_slots, self.budget)
        self.max_in_flight = 0
        self.stats = {}

    def serve(self, jobs: List[Job], realtime: bool = True, on_done: Optional[Callable] = None) -> List[Job]:
        """Feed jobs at their arrival times; return them when all are done."""
        jobs = sorted(jobs, key=lambda j: j.arrival)
        t0 = time.perf_counter()
        ids = []
        for job in jobs:
            if realtime:
                delay = job.arrival - (time.perf_counter() - t0)
                if delay > 0:
                    time.sleep(delay)
            else:
                job.arrival = time.perf_counter() - t0
            x = np.ascontiguousarray(job.points)
            ids.append(self.native.submit(
                x, job.radius_cutoff ** 2, job.cnn_cutoff + 2, job.cnn_cutoff + 1,
                member_cutoff=2 if job.member_cutoff is None else job.member_cutoff,
                reserve_bytes=footprint_bytes(x.shape[0], x.shape[1], job.expected_degree)))
        for job, jid in zip(jobs, ids):
            try:
                job.labels, info = self.native.wait(jid)
            except _abi.CNNError as e:  # the job fails alone; the server keeps going
                job.error = str(e)
                info = e.info
            # the library's clock: start and end relative to the submission
            job.slot = info.get("slot")
            job.t_admit = job.arrival + (info["t_start"] - info["t_submit"])
            job.t_done = job.arrival + (info["t_done"] - info["t_submit"])
            if on_done is not None:
                on_done(job)
        self.stats = self.native.stats()
        self.max_in_flight = self.stats["max_running"]
        return jobs

    def close(self):
        self.native.close()


def serve_one_at_a_time(jobs: List[Job], device: int = 0, realtime: bool = True) -> List[Job]:
    """The plain path: one context, jobs strictly in arrival order."""
    ctx = _abi.Context(device)
    t0 = time.perf_counter()
    for job in sorted(jobs, key=lambda j: j.arrival):
        if realtime:
            delay = job.arrival - (time.perf_counter() - t0)
            if delay > 0:
                time.sleep(delay)
        job.t_admit = time.perf_counter() - t0
        job.labels = run_job_alone(ctx, job)
        job.t_done = time.perf_counter() - t0
    ctx.close()
    return jobs


def latency_summary(jobs: List[Job]) -> dict:
    lat = np.array([j.latency for j in jobs if j.latency is not None])
    span = max(j.t_done for j in jobs) - min(j.arrival for j in jobs)
    return {"jobs": len(jobs), "p50_ms": float(np.percentile(lat, 50) * 1e3),
            "p99_ms": float(np.percentile(lat, 99) * 1e3), "mean_ms": float(lat.mean() * 1e3),
            "jobs_per_s": len(jobs) / span if span > 0 else None,
            "points_per_s": sum(j.points.shape[0] for j in jobs) / span if span > 0 else None}


__all__ = ["Job", "Server", "footprint_bytes", "run_job_alone", "serve_one_at_a_time", "latency_summary"]
