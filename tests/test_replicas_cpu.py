"""bench.py's multi-rank path on CPU (gloo, world_size 2): the fit does not
shard, so N ranks run N replicas; the job time is the slowest rank's and
only rank 0 reports.  No GPU is touched here."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def rank_main(rank, world, port, out):
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    import bench
    r, w, local = bench.dist_env()
    d = bench.init_dist(w)
    bench.barrier(d)
    slowest = bench.reduce_max(d, 1.0 + rank)  # each rank's own step time
    out.put((r, w, local, slowest))
    bench.barrier(d)
    dist.destroy_process_group()


def test_two_ranks_take_the_slowest_time():
    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    port = free_port()
    procs = [ctx.Process(target=rank_main, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted(out.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert got == [(0, 2, 0, 2.0), (1, 2, 1, 2.0)]


def reference_rank_main(rank, world, port, out):
    import contextlib
    import io
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    import bench
    args = type("A", (), {"steps": 1, "warmup": 0, "workload": "blobs2d-5k", "intersection": "auto"})()
    buf = io.StringIO()
    with contextlib.redirect_stdout(buf):
        bench.run_reference(args)
    out.put((rank, buf.getvalue()))


def test_reference_arm_reports_on_rank_zero_only():
    import json
    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    port = free_port()
    procs = [ctx.Process(target=reference_rank_main, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    got = dict(out.get(timeout=300) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert got[1] == ""
    line = json.loads(got[0].strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["n_gpus"] == 2 and line["value"] > 0
    assert line["e2e"]["h2d_bytes_per_step"] == 0
