"""Served stream: every job's result in the concurrent mix equals the job run alone."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def serve():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from commonnnclustering_gb300 import serve
    return serve


def make_jobs(serve_mod, n_jobs, rate, seed):
    from commonnnclustering_gb300 import workloads
    raw = workloads.job_stream(n_jobs=n_jobs, rate=rate, seed=seed, pool=8, max_points=30000)
    return [serve_mod.Job(job_id=i, **j) for i, j in enumerate(raw)]


def test_jobs_in_the_mix_equal_jobs_alone(serve):
    from commonnnclustering_gb300 import _abi
    jobs = make_jobs(serve, 40, rate=400.0, seed=3)
    srv = serve.Server(n_slots=4, hbm_budget_bytes=8 << 30)
    try:
        srv.serve(jobs, realtime=True)
    finally:
        srv.close()
    assert all(j.error is None for j in jobs), [j.error for j in jobs if j.error]
    assert srv.max_in_flight > 1  # the jobs really overlapped
    ctx = _abi.Context(0)
    for j in jobs:
        alone = serve.run_job_alone(ctx, j)
        assert np.array_equal(alone, j.labels), j.job_id
    ctx.close()
    s = serve.latency_summary(jobs)
    assert s["p99_ms"] >= s["p50_ms"] > 0


def test_admission_respects_the_memory_budget(serve):
    jobs = make_jobs(serve, 12, rate=1000.0, seed=4)
    biggest = max(serve.footprint_bytes(j.points.shape[0], j.points.shape[1], j.expected_degree) for j in jobs)
    srv = serve.Server(n_slots=4, hbm_budget_bytes=biggest)  # room for about one job at a time
    try:
        srv.serve(jobs, realtime=False)
    finally:
        srv.close()
    assert all(j.error is None and j.labels is not None for j in jobs)
    assert srv.in_use == 0


def test_gram_searches_of_different_widths_in_threads(serve):
    """Concurrent contexts whose tensor-core searches need different
    dynamic shared memory (n_dim 16 to 128) all succeed and match the same
    searches run one after another."""
    import threading
    from commonnnclustering_gb300 import _abi
    rng = np.random.default_rng(8)
    cases = []
    for t in range(16):
        d = (16, 32, 64, 128)[t % 4]
        centres = rng.normal(0, 3.0, size=(6, d))
        x = np.vstack([c + rng.normal(0, 0.4, size=(700, d)) for c in centres])
        cases.append((x, (0.35 * np.sqrt(2.0 * d)) ** 2))
    ctx = _abi.Context(0)
    want = []
    for x, r2 in cases:
        ctx.set_points(x)
        ctx.build_neighbours(r2)
        assert ctx.stats()["search_kind"] == 3  # the tensor-core path
        want.append(ctx.get_neighbours())
    ctx.close()
    got = [None] * len(cases)
    errors = []

    def worker(w):
        c = _abi.Context(0)
        try:
            for _ in range(3):
                for i in range(w, len(cases), 4):
                    x, r2 = cases[i]
                    c.set_points(x)
                    c.build_neighbours(r2)
                    got[i] = c.get_neighbours()
        except Exception as e:  # reported below
            errors.append(repr(e))
        finally:
            c.close()

    threads = [threading.Thread(target=worker, args=(w,)) for w in range(4)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    assert not errors, errors
    for (wo, wi), (go, gi) in zip(want, got):
        assert np.array_equal(wo, go) and np.array_equal(wi, gi)
