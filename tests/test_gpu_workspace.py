"""Workspace hygiene: stale or garbage device workspace never changes a result.

Contexts keep their device buffers between calls (grow-only), so every
kernel must initialise what it reads.  CNN_DEBUG_POISON=<byte> makes a new
context fill each fresh allocation with that byte; results must be equal
for every fill and for contexts that ran other, larger jobs before.
"""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def mods():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from commonnnclustering_gb300 import _abi, serve, workloads
    return _abi, serve, workloads


def make_jobs(serve, workloads):
    rng = np.random.default_rng(7)
    jobs = []
    for i, (n, d, k) in enumerate([(20000, 3, 30), (6000, 2, 8), (8000, 5, 12), (9000, 16, 10), (7000, 64, 6),
                                   (30000, 3, 120), (1500, 64, 3), (3000, 2, 1)]):
        x = workloads.mixture(n, d, k, seed=100 + i)
        r = workloads.degree_radius(x, float(rng.uniform(40, 200)), seed=i)
        jobs.append(serve.Job(job_id=i, points=x, radius_cutoff=r, cnn_cutoff=int(rng.integers(2, 30)),
                              member_cutoff=int(rng.integers(2, 12))))
    return jobs


def contexts_with_poison(_abi, byte):
    old = os.environ.get("CNN_DEBUG_POISON")
    os.environ["CNN_DEBUG_POISON"] = str(byte)
    try:
        return _abi.Context(0)
    finally:
        if old is None:
            del os.environ["CNN_DEBUG_POISON"]
        else:
            os.environ["CNN_DEBUG_POISON"] = old


def test_results_do_not_depend_on_workspace_contents(mods):
    _abi, serve, workloads = mods
    jobs = make_jobs(serve, workloads)
    ref = []
    ctx = _abi.Context(0)
    for j in jobs:
        ref.append(serve.run_job_alone(ctx, j))
    ctx.close()
    for byte in (0x00, 0xFF, 0xA5, 0x7F):
        ctx = contexts_with_poison(_abi, byte)
        for j, want in zip(jobs, ref):
            got = serve.run_job_alone(ctx, j)
            assert np.array_equal(got, want), (byte, j.job_id)
        ctx.close()


def test_results_do_not_depend_on_job_history(mods):
    _abi, serve, workloads = mods
    jobs = make_jobs(serve, workloads)
    fresh = []
    for j in jobs:
        ctx = contexts_with_poison(_abi, 0xFF)
        fresh.append(serve.run_job_alone(ctx, j))
        ctx.close()
    # one context, the jobs in two different orders: buffers hold the previous job's data
    for order in (list(range(len(jobs))), list(reversed(range(len(jobs))))):
        ctx = _abi.Context(0)
        for i in order:
            assert np.array_equal(serve.run_job_alone(ctx, jobs[i]), fresh[i]), (order[0], i)
        ctx.close()
