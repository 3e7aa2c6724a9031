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
    """The budget bounds the device bytes the slots' workspaces really hold
    (the library's own accounting of its allocations), not an estimate."""
    jobs = make_jobs(serve, 12, rate=1000.0, seed=4)
    biggest = max(serve.footprint_bytes(j.points.shape[0], j.points.shape[1], j.expected_degree) for j in jobs)
    # room for one or two jobs at a time; a job whose real need passes its
    # estimate runs again alone
    srv = serve.Server(n_slots=4, hbm_budget_bytes=2 * biggest)
    try:
        srv.serve(jobs, realtime=False)
    finally:
        srv.close()
    assert all(j.error is None and j.labels is not None for j in jobs), [j.error for j in jobs if j.error]
    st = srv.stats
    assert st["done"] == 12 and st["failed"] == 0 and st["running"] == 0 and st["queued"] == 0
    assert 0 < st["peak_held_bytes"] <= st["budget_bytes"]
    assert st["committed_bytes"] <= st["budget_bytes"]


def test_job_that_outgrows_its_reservation_runs_again(serve):
    """A job whose first reservation is far too small hits the workspace
    limit before any allocation past it, is queued again with a larger
    reservation, and ends with the same labels as run alone; the bytes held
    never exceed the budget."""
    from commonnnclustering_gb300 import _abi, workloads
    rng = np.random.default_rng(12)
    xs = [workloads.blobs2d(n=int(n), seed=int(s)) for n, s in zip(rng.integers(3000, 9000, 6), range(6))]
    budget = 256 << 20
    srv = _abi.NativeServer(0, 3, budget)
    try:
        ids = [srv.submit(x, 0.3 ** 2, 7, 6, member_cutoff=5, reserve_bytes=(1 << 20) if i == 2 else 0)
               for i, x in enumerate(xs)]
        got = [srv.wait(i) for i in ids]
        st = srv.stats()
    finally:
        srv.close()
    assert got[2][1]["attempts"] >= 2 and got[2][1]["reserved_bytes"] > (1 << 20)
    assert st["requeued"] >= 1 and st["failed"] == 0
    assert 0 < st["peak_held_bytes"] <= budget
    ctx = _abi.Context(0)
    try:
        for x, (labels, info) in zip(xs, got):
            ctx.set_points(x)
            ctx.build_neighbours(0.3 ** 2)
            want = np.zeros(x.shape[0], dtype=np.int64)
            ctx.fit(7, 6, 1, np.ones(x.shape[0], dtype=np.uint8), want)
            ctx.sort_by_size(want, 5, None)
            assert np.array_equal(labels, want)
    finally:
        ctx.close()


def test_job_larger_than_the_whole_budget_fails_alone(serve):
    """A job that does not fit even the whole budget fails with
    CNN_ERR_OOM; the jobs around it complete."""
    from commonnnclustering_gb300 import _abi, workloads
    small = workloads.blobs2d(n=2000, seed=1)
    big = workloads.blobs2d(n=400000, seed=2)
    srv = _abi.NativeServer(0, 2, 64 << 20)
    try:
        a = srv.submit(small, 0.3 ** 2, 7, 6)
        b = srv.submit(big, 0.3 ** 2, 7, 6)
        c = srv.submit(small, 0.3 ** 2, 7, 6)
        la, _ = srv.wait(a)
        with pytest.raises(_abi.CNNError) as e:
            srv.wait(b)
        assert e.value.status == _abi.CNN_ERR_OOM
        lc, _ = srv.wait(c)
        assert np.array_equal(la, lc)
        assert srv.stats()["peak_held_bytes"] <= 64 << 20
    finally:
        srv.close()


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


def test_job_states_wait_timeout_and_release(serve):
    """cnn_poll / cnn_wait / cnn_job_release semantics: a job is QUEUED or
    RUNNING until DONE, a zero wait limit returns CNN_ERR_TIMEOUT or the
    done job, a job cannot be released before it is done and its id is
    invalid after."""
    import ctypes
    from commonnnclustering_gb300 import _abi, workloads
    srv = _abi.NativeServer(0, 1, 8 << 30)
    try:
        xs = [workloads.md3d(n=60000, seed=s) for s in range(3)]
        ids = [srv.submit(x, 0.1 ** 2, 12, 11, member_cutoff=50) for x in xs]
        states = [srv.poll(i)["state"] for i in ids]
        assert all(s in (_abi.JOB_QUEUED, _abi.JOB_RUNNING, _abi.JOB_DONE) for s in states)
        info = _abi.cnn_job_info()
        st = srv._lib.cnn_wait(srv._h, ids[-1], 0, ctypes.byref(info))
        assert st in (_abi.CNN_OK, _abi.CNN_ERR_TIMEOUT)
        if st == _abi.CNN_ERR_TIMEOUT:
            assert info.state != _abi.JOB_DONE
            assert srv._lib.cnn_job_release(srv._h, ids[-1]) == _abi.CNN_ERR_STATE
        assert srv._lib.cnn_wait(srv._h, ids[-1], -1, ctypes.byref(info)) == _abi.CNN_OK
        assert info.state == _abi.JOB_DONE and info.result == _abi.CNN_OK
        assert info.t_submit <= info.t_start <= info.t_done
        for i in ids[:-1]:
            labels, inf = srv.wait(i)      # waits, then releases the record
            assert inf["state"] == _abi.JOB_DONE
            assert srv._lib.cnn_poll(srv._h, i, ctypes.byref(info)) == _abi.CNN_ERR_INVALID_ARG
        assert srv._lib.cnn_job_release(srv._h, ids[-1]) == _abi.CNN_OK
        assert srv._lib.cnn_job_release(srv._h, ids[-1]) == _abi.CNN_ERR_INVALID_ARG
        st = srv.stats()
        assert st["done"] == 3 and st["failed"] == 0 and st["max_running"] == 1
    finally:
        srv._keep.clear()
        srv.close()
