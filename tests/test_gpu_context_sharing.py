"""Several users of one library context (the per-thread default context).

Clusterings, ``sweep()`` and ``Labels.sort_by_size`` all run on the same
per-thread, per-device context.  A fitter that keeps its neighbour graph on
the device between fits must notice when someone else replaced the graph of
the context, and the fit must never write more labels than the caller's
arrays hold: every labelling here is compared with the oracle.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import commonnnclustering_gb300 as cnn
    from oracle import cnn_oracle
    return torch, cnn, cnn_oracle


def test_two_device_clusterings_on_one_context(env):
    torch, cnn, oracle = env
    from commonnnclustering_gb300 import workloads
    xa = workloads.md3d(n=30000, seed=8, centre_spread=2.0)   # A larger than B: a stale graph
    xb = workloads.blobs2d(n=5000, seed=3)                    # of B could not overrun A's labels
    a = cnn.Clustering(torch.from_numpy(xa).cuda())
    b = cnn.Clustering(torch.from_numpy(xb).cuda())
    want_a, _ = oracle.clustering_fit(xa, 0.12, 8, member_cutoff=10)
    want_b, _ = oracle.clustering_fit(xb, 0.3, 5, member_cutoff=10)
    for cl, want, (r, c) in ((a, want_a, (0.12, 8)), (b, want_b, (0.3, 5)), (a, want_a, (0.12, 8)),
                             (b, want_b, (0.3, 5))):
        cl.fit(r, c, member_cutoff=10, v=False)
        assert cl.labels.shape[0] == want.shape[0]
        assert np.array_equal(cl.labels.cpu().numpy(), want)
    assert a.fitter.context_for() is b.fitter.context_for()  # the case under test: one shared context


def test_sweep_and_sort_by_size_between_fits(env):
    torch, cnn, oracle = env
    from commonnnclustering_gb300 import sweep, workloads
    xa = workloads.md3d(n=20000, seed=9, centre_spread=2.0)
    a = cnn.Clustering(torch.from_numpy(xa).cuda())
    want, _ = oracle.clustering_fit(xa, 0.12, 6, member_cutoff=10)
    a.fit(0.12, 6, member_cutoff=10, v=False)
    assert np.array_equal(a.labels.cpu().numpy(), want)
    # another graph on the same context: a sweep over other points
    xs = workloads.blobs2d(n=4000, seed=1)
    out = sweep(torch.from_numpy(xs).cuda(), [0.25, 0.3], [5], member_cutoff=10)
    for k, r in enumerate((0.25, 0.3)):
        w, _ = oracle.clustering_fit(xs, r, 5, member_cutoff=10)
        assert np.array_equal(out[k, 0].cpu().numpy() if hasattr(out, "cpu") else out[k, 0], w)
    a.fit(0.12, 6, member_cutoff=10, v=False)
    assert np.array_equal(a.labels.cpu().numpy(), want)
    # Labels.sort_by_size of unrelated labels on the same context
    other = cnn.Labels(torch.tensor([3, 3, 1, 0, 1, 3], dtype=torch.int64, device="cuda"))
    other.sort_by_size(member_cutoff=1)
    assert other.labels.cpu().tolist() == [1, 1, 2, 0, 2, 1]
    a.fit(0.12, 6, member_cutoff=10, v=False)
    assert np.array_equal(a.labels.cpu().numpy(), want)


def test_fit_rejects_labels_of_another_length(env):
    torch, cnn, oracle = env
    from commonnnclustering_gb300 import _abi, workloads
    x = workloads.blobs2d(n=3000, seed=4)
    ctx = _abi.Context(0)
    ctx.set_points(x)
    ctx.build_neighbours(0.09)
    short = np.zeros(2999, dtype=np.int64)
    with pytest.raises(ValueError):
        ctx.fit(7, 6, 1, np.ones(2999, dtype=np.uint8), short)
    # the C entry point itself rejects a wrong count before touching anything
    lab = np.zeros(4000, dtype=np.int64)
    con = np.ones(4000, dtype=np.uint8)
    st = ctx._lib.cnn_fit(ctx._h, 7, 6, 1, con.ctypes.data, lab.ctypes.data, 4000, _abi.MEM_HOST)
    assert st == 1 and not lab.any() and con.all()
    ctx.close()
