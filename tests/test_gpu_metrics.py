"""GPU: the periodic metric and precomputed distances (square and linear)
against the reference's fixtures and the oracle."""
import hashlib

import numpy as np
import pytest

from conftest import load_golden, pairwise_distances
from oracle import cnn_oracle as o

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def cnn():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import commonnnclustering_gb300 as cnn
    return cnn


def digest(offsets, indices):
    h = hashlib.sha256()
    h.update(np.ascontiguousarray(offsets, dtype=np.int64).tobytes())
    h.update(np.ascontiguousarray(indices, dtype=np.int32).tobytes())
    return h.hexdigest()


def periodic_clustering(cnn, x, bounds, fpmode="separate"):
    metric = cnn.MetricGPUEuclideanPeriodicReduced(bounds)
    getter = cnn.NeighboursGetterGPUGrid(cnn.DistanceGetterGPUMetric(metric), fpmode=fpmode)
    return cnn.Clustering(x, fitter=cnn.FitterGPU(getter))


def test_periodic_matches_reference(cnn):
    g = load_golden("periodic_dihedrals.npz")
    for k in range(int(g["n_cases"])):
        r, c, mc = g[f"params_{k}"]
        cl = periodic_clustering(cnn, g["points"], g["bounds"])
        cl.fit(r, int(c), member_cutoff=int(mc), v=False)
        assert np.array_equal(np.asarray(cl.labels), g[f"labels_{k}"])
        ctx = cl.fitter.context_for(None)
        off, idx = ctx.get_neighbours()
        assert digest(off, idx) == str(g[f"csr_sha256_{k}"])


def test_periodic_recipe_keywords(cnn):
    g = load_golden("periodic_dihedrals.npz")
    metric = (cnn.MetricGPUEuclideanPeriodicReduced, (g["bounds"],), {})
    cl = cnn.Clustering(g["points"], fitter__getter__dgetter__metric=metric)
    r, c, mc = g["params_0"]
    cl.fit(r, int(c), member_cutoff=int(mc), v=False)
    assert np.array_equal(np.asarray(cl.labels), g["labels_0"])


@pytest.mark.parametrize("fpmode", ["separate", "fused"])
@pytest.mark.parametrize("d", [1, 3, 5])
def test_periodic_against_oracle(cnn, d, fpmode):
    rng = np.random.default_rng(90 + d)
    bounds = np.array([10.0, 0.0, 7.5, 12.0, 3.0][:d])  # one dimension not periodic
    x = rng.uniform(-12, 15, size=(2500, d))
    x[:800] = (rng.normal(0, 0.6, size=(800, d)) + 9.9)  # a cluster across the box edge
    r = 0.6 if d <= 3 else 1.2
    off, idx = o.periodic_neighbourhoods(x, bounds, r * r, 1 if fpmode == "fused" else 0)
    want = o.fit_from_neighbourhoods(off, idx, 4, member_cutoff=3)
    cl = periodic_clustering(cnn, x, bounds, fpmode)
    cl.fit(r, 4, member_cutoff=3, v=False)
    assert np.array_equal(np.asarray(cl.labels), want)
    got_off, got_idx = cl.fitter.context_for(None).get_neighbours()
    assert np.array_equal(got_off, off) and np.array_equal(got_idx, idx)


def test_periodic_needs_bounds(cnn):
    ctx = cnn.Context(0)
    ctx.set_points(np.zeros((10, 2)))
    ctx.set_periodic_bounds([1.0])  # wrong length
    with pytest.raises(cnn.CNNError):
        ctx.build_neighbours(0.1, metric=3)
    ctx.close()


def test_precomputed_square_and_linear_match_reference(cnn):
    import torch
    g = load_golden("precomputed_distances.npz")
    dist = pairwise_distances(g["points"])
    r, c, mc = float(g["radius_cutoff"]), int(g["cnn_cutoff"]), int(g["member_cutoff"])
    cl = cnn.Clustering(dist, recipe="distances")
    cl.fit(r, c, member_cutoff=mc, v=False)
    assert np.array_equal(np.asarray(cl.labels), g["labels_square"])
    iu = np.triu_indices(dist.shape[0], 1)
    lin = cnn.InputDataGPUDistancesLinear(dist[iu])
    getter = cnn.NeighboursGetterGPUGrid(cnn._types.DistanceGetterGPULookup())
    cl = cnn.Clustering(lin, fitter=cnn.FitterGPU(getter))
    cl.fit(r, c, member_cutoff=mc, v=False)
    assert np.array_equal(np.asarray(cl.labels), g["labels_linear"])
    # device-resident square matrix
    dt = torch.from_numpy(dist).cuda()
    cl = cnn.Clustering(cnn.InputDataGPUDistances(dt), recipe="distances")
    cl.fit(r, c, member_cutoff=mc, v=False)
    assert np.array_equal(cl.labels.cpu().numpy(), g["labels_square"])


def test_precomputed_rows_against_oracle(cnn):
    rng = np.random.default_rng(5)
    x = rng.normal(size=(900, 3))
    dist = pairwise_distances(x)
    dist[3, 7] = dist[7, 3] = np.nan  # NaN never admits a pair
    ctx = cnn.Context(0)
    for linear in (False, True):
        if linear:
            iu = np.triu_indices(dist.shape[0], 1)
            ctx.set_distances(dist[iu], layout=1)
            want = o.distance_neighbourhoods(dist[iu], 0.4, linear=True)
        else:
            ctx.set_distances(dist)
            want = o.distance_neighbourhoods(dist, 0.4)
        ctx.build_neighbours(0.4, metric=2)
        off, idx = ctx.get_neighbours()
        assert np.array_equal(off, want[0]) and np.array_equal(idx, want[1])
    # a sweep over precomputed distances equals separate fits
    ctx.set_distances(dist)
    got = ctx.sweep([0.2, 0.4], [(4, 3), (7, 6)], metric=2)
    for k, rc in enumerate([0.2, 0.4]):
        for j, (sim, nmem) in enumerate([(4, 3), (7, 6)]):
            off, idx = o.distance_neighbourhoods(dist, rc)
            labels = np.zeros(900, dtype=np.int64)
            o.fit_bfs_csr(off, idx, sim, nmem, 1, np.ones(900, dtype=np.uint8), labels)
            o.sort_by_size(labels, 2)
            assert np.array_equal(got[k, j], labels)
    ctx.close()


def test_periodic_predict_against_oracle(cnn):
    rng = np.random.default_rng(14)
    bounds = np.array([360.0, 360.0])
    centres = np.array([[-175.0, 0.0], [90.0, 90.0]])
    x = np.vstack([cc + rng.normal(0, 12, size=(400, 2)) for cc in centres])
    x = (x + 180) % 360 - 180
    y = np.vstack([cc + rng.normal(0, 14, size=(300, 2)) for cc in centres])
    y = (y + 180) % 360 - 180
    r, c = 10.0, 5
    off, idx = o.periodic_neighbourhoods(x, bounds, r * r)
    labels = o.fit_from_neighbourhoods(off, idx, c, member_cutoff=5)
    clusters = sorted(set(labels.tolist()) - {0})
    want, _ = o.predict_firstmatch(x, labels, y, r * r, c + 2, c + 1, clusters, periodic_bounds=bounds)
    metric = cnn.MetricGPUEuclideanPeriodicReduced(bounds)
    getter = cnn.NeighboursGetterGPUGrid(cnn.DistanceGetterGPUMetric(metric))
    cl = cnn.Clustering(x, predictor=cnn.PredictorFirstmatchGPU(getter))
    cl.labels = labels
    other = cnn.Clustering(y)
    cl.predict(other._bundle, r, c)
    assert np.array_equal(np.asarray(other.labels), want)


@pytest.mark.parametrize("fpmode", ["separate", "fused"])
def test_periodic_wrapped_grid_against_oracle(cnn, fpmode):
    """The periodic metric runs on a wrapped cell grid (n_dim <= 3, at least 3
    cells per periodic dimension): coordinates far outside the box, points
    on the box edges and at half a box, and a lattice whose minimum-image
    distances hit the cutoff exactly give the oracle's neighbour sets."""
    from commonnnclustering_gb300 import _abi
    rng = np.random.default_rng(7)
    bounds = np.array([360.0, 360.0])
    x = rng.uniform(-900.0, 900.0, size=(12000, 2))            # several box lengths out
    x[:3000] = rng.normal(0.0, 8.0, size=(3000, 2)) + 180.0     # a cluster across the +-180 edge
    x[3000:3010] = [[0, 0], [360, 0], [-360, 360], [180, -180], [540, 180],
                    [-180, 0], [179.999999, 0], [-179.999999, 0], [720, 720], [0, 180]]
    lat = np.stack(np.meshgrid(np.arange(-180.0, 180.0, 10.0), np.arange(-180.0, 180.0, 10.0)), -1).reshape(-1, 2)
    x = np.vstack([x, lat])
    fp = 1 if fpmode == "fused" else 0
    for r in (10.0, 14.0):  # the lattice spacing: ties s == r^2 at r = 10
        off, idx = o.periodic_neighbourhoods(x, bounds, r * r, fp)
        ctx = _abi.Context(0)
        try:
            ctx.set_points(x)
            ctx.set_periodic_bounds(bounds)
            ctx.build_neighbours(r * r, metric=_abi.METRIC_EUCLIDEAN_PERIODIC_REDUCED, fpmode=fp)
            assert ctx.stats()["search_kind"] == 1  # the wrapped grid
            got_off, got_idx = ctx.get_neighbours()
            assert np.array_equal(got_off, off) and np.array_equal(got_idx, idx)
        finally:
            ctx.close()


def test_periodic_mixed_dimensions_on_the_grid(cnn):
    """3-D with one dimension not periodic and two periodic ones of
    different box lengths; a box too small for 3 cells falls back to the
    all-pairs search with the same sets."""
    from commonnnclustering_gb300 import _abi
    rng = np.random.default_rng(8)
    x = rng.uniform(-20.0, 20.0, size=(15000, 3))
    for bounds, kind in ((np.array([10.0, 0.0, 7.5]), 1), (np.array([1.5, 10.0, 10.0]), 2)):
        off, idx = o.periodic_neighbourhoods(x, bounds, 0.6 ** 2, 0)
        ctx = _abi.Context(0)
        try:
            ctx.set_points(x)
            ctx.set_periodic_bounds(bounds)
            ctx.build_neighbours(0.6 ** 2, metric=_abi.METRIC_EUCLIDEAN_PERIODIC_REDUCED, fpmode=0)
            assert ctx.stats()["search_kind"] == kind
            got_off, got_idx = ctx.get_neighbours()
            assert np.array_equal(got_off, off) and np.array_equal(got_idx, idx)
        finally:
            ctx.close()
