"""Batched (radius, cnn_cutoff) sweep: every result must equal a separate fit."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def cnn():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import commonnnclustering_gb300 as cnn
    return cnn


def separate_fit(cnn, x, r, c, member_cutoff):
    cl = cnn.Clustering(cnn.InputDataGPUComponents(x))
    cl.fit(r, c, member_cutoff=member_cutoff, v=False)
    return np.asarray(cl.labels)


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_sweep_equals_separate_fits(cnn, dtype):
    from commonnnclustering_gb300 import workloads
    x = workloads.nested3d(n=30000, seed=2, n_parents=6, box=3.0).astype(dtype)
    radii = [0.03, 0.06, 0.09, 0.12]
    cuts = [2, 5, 20, 60]
    got = cnn.sweep(x, radii, cuts, member_cutoff=5)
    assert got.shape == (4, 4, x.shape[0])
    for k, r in enumerate(radii):
        for j, c in enumerate(cuts):
            assert np.array_equal(got[k, j], separate_fit(cnn, x, r, c, 5)), (r, c)


def test_sweep_against_oracle(cnn):
    from commonnnclustering_gb300 import workloads
    from oracle import cnn_oracle
    x = workloads.nested3d(n=8000, seed=5, n_parents=3, box=2.0).astype(np.float64)
    radii, cuts = [0.05, 0.1], [3, 10]
    got = cnn.sweep(x, radii, cuts, member_cutoff=2)
    for k, r in enumerate(radii):
        for j, c in enumerate(cuts):
            want, _ = cnn_oracle.clustering_fit(x, r, c, member_cutoff=2)
            assert np.array_equal(got[k, j], want), (r, c)


def test_sweep_without_grid_searches_each_radius(cnn):
    rng = np.random.default_rng(3)
    x = np.vstack([rng.normal(0, 1, size=(1500, 5)), rng.normal(4, 0.5, size=(1500, 5))])
    radii, cuts = [0.6, 0.9], [2, 8]
    got = cnn.sweep(x, radii, cuts, member_cutoff=2)
    for k, r in enumerate(radii):
        for j, c in enumerate(cuts):
            assert np.array_equal(got[k, j], separate_fit(cnn, x, r, c, 2)), (r, c)


def test_sweep_rejects_descending_radii(cnn):
    ctx = cnn.Context(0)
    ctx.set_points(np.random.default_rng(0).normal(size=(50, 2)))
    with pytest.raises(cnn.CNNError):
        ctx.sweep([0.04, 0.01], [(3, 2)])
    ctx.close()


def fit_pair(cnn, ctx, x, rc, sim, nmem, member_cutoff):
    labels = np.zeros(x.shape[0], dtype=np.int64)
    consider = np.ones(x.shape[0], dtype=np.uint8)
    ctx.set_points(x)
    ctx.build_neighbours(rc)
    ctx.fit(sim, nmem, 1, consider, labels)
    ctx.sort_by_size(labels, member_cutoff, None)
    return labels


@pytest.mark.parametrize("d", [3, 5])
def test_sweep_unordered_cut_pairs(cnn, d):
    # (similarity_cutoff, n_member_cutoff) pairs in no particular order,
    # including 0 (every pair passes) and -1 (no pair passes): fits may only
    # start from fits that refine them
    rng = np.random.default_rng(11 + d)
    centres = rng.uniform(-3, 3, size=(12, d))
    x = np.vstack([c + rng.normal(0, 0.25, size=(1500, d)) for c in centres])
    rcs = [0.04, 0.09, 0.16] if d == 3 else [0.3, 0.5]
    cuts = [(5, 2), (3, 8), (0, 4), (-1, 3), (7, 7), (5, 9), (12, 1), (3, 8)]
    ctx = cnn.Context(0)
    ctx.set_points(x)
    got = ctx.sweep(rcs, cuts, member_cutoff=3)
    alone = cnn.Context(0)
    for k, rc in enumerate(rcs):
        for j, (sim, nmem) in enumerate(cuts):
            assert np.array_equal(got[k, j], fit_pair(cnn, alone, x, rc, sim, nmem, 3)), (rc, sim, nmem)
    ctx.close()
    alone.close()


def test_radius_by_radius_equals_all_radii_at_once(cnn, monkeypatch):
    """The sweep builds every smaller radius's graph in one pass when they fit
    in its memory budget, else one radius at a time: both give the same labels."""
    from commonnnclustering_gb300 import workloads
    x = workloads.nested3d(n=20000, seed=7, n_parents=5, box=3.0).astype(np.float64)
    radii, cuts = [0.03, 0.06, 0.1], [2, 10, 40]
    at_once = cnn.sweep(x, radii, cuts, member_cutoff=3)
    monkeypatch.setenv("CNN_SWEEP_GRAPH_BUDGET", "0")
    one_by_one = cnn.sweep(x, radii, cuts, member_cutoff=3)
    assert np.array_equal(at_once, one_by_one)
    for k, r in enumerate(radii):
        assert np.array_equal(at_once[k, 1], separate_fit(cnn, x, r, cuts[1], 3)), r


@pytest.mark.parametrize("max_clusters", [None, 3])
def test_sweep_as_cuda_graph_equals_plain_launches(cnn, monkeypatch, max_clusters):
    """The sweep's fits run as captured CUDA graphs (the sort of each fit
    enqueues the same work whatever the labels hold); with capture switched
    off (CNN_SWEEP_GRAPH=0 at context creation) the same labels come out."""
    from commonnnclustering_gb300 import _abi, workloads
    x = workloads.nested3d(n=40000, seed=8, n_parents=8, box=3.0).astype(np.float64)
    x2 = workloads.nested3d(n=40000, seed=11, n_parents=5, box=3.0).astype(np.float64)
    r2 = [r * r for r in (0.03, 0.05, 0.08, 0.11)]
    cuts = [(c + 2, c + 1) for c in (2, 5, 20, 60)]
    out = {}
    for graph in ("1", "0"):
        monkeypatch.setenv("CNN_SWEEP_GRAPH", graph)
        ctx = _abi.Context(0)
        try:
            # the second sweep on the same context reuses the instantiated
            # graph with updated parameters (other points, other graph sizes)
            for key, pts in ((graph, x), (graph + "b", x2)):
                ctx.set_points(pts)
                out[key] = ctx.sweep(r2, cuts, member_cutoff=5, max_clusters=max_clusters)
                st = ctx.stats()
                if graph == "1":
                    assert st["graphs"] >= 1 and st["graph_nodes"] > 100
                else:
                    assert st["graphs"] == 0
        finally:
            ctx.close()
    assert np.array_equal(out["1"], out["0"])
    assert np.array_equal(out["1b"], out["0b"])
    # and each equals a plain fit + sort_by_size on the same context type
    ctx = _abi.Context(0)
    try:
        ctx.set_points(x)
        for k, rc in enumerate(r2):
            ctx.build_neighbours(rc)
            for j, (sc, nm) in enumerate(cuts):
                labels = np.zeros(x.shape[0], dtype=np.int64)
                ctx.fit(sc, nm, 1, np.ones(x.shape[0], dtype=np.uint8), labels)
                ctx.sort_by_size(labels, 5, max_clusters)
                assert np.array_equal(out["1"][k, j], labels), (k, j)
    finally:
        ctx.close()
