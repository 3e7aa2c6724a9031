"""GPU: step lists (cnn_sweep_pairs), HierarchicalFitterRepeatGPU and
PredictorFirstmatchGPU against the reference's fixtures and the oracle."""
import numpy as np
import pytest

from conftest import bundle_tree, golden_tree, load_golden, predict_cases
from oracle import cnn_oracle as o

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def cnn():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import commonnnclustering_gb300 as cnn
    return cnn


def separate(ctx, x, rc, sim, nmem, member_cutoff, sort=True):
    labels = np.zeros(x.shape[0], dtype=np.int64)
    consider = np.ones(x.shape[0], dtype=np.uint8)
    ctx.set_points(x)
    ctx.build_neighbours(rc)
    ctx.fit(sim, nmem, 1, consider, labels)
    if sort:
        ctx.sort_by_size(labels, member_cutoff, None)
    return labels


@pytest.mark.parametrize("d", [2, 3, 8])
@pytest.mark.parametrize("sort", [True, False])
def test_step_list_equals_separate_fits(cnn, d, sort):
    rng = np.random.default_rng(40 + d)
    centres = rng.uniform(-3, 3, size=(10, d))
    x = np.vstack([c + rng.normal(0, 0.3, size=(700, d)) for c in centres])
    base = 0.03 if d <= 3 else 0.5
    # unordered steps with a repeated pair and repeated radii
    steps = [(base * 2.0, 5, 6), (base, 3, 4), (base * 2.0, 5, 6), (base * 3.0, 0, 2), (base, 8, 2),
             (base * 3.0, -1, 3), (base * 1.5, 4, 9)]
    ctx = cnn.Context(0)
    ctx.set_points(x)
    got = ctx.sweep_pairs([s[0] for s in steps], [(s[1], s[2]) for s in steps], member_cutoff=4, sort=sort)
    alone = cnn.Context(0)
    for i, (rc, sim, nmem) in enumerate(steps):
        assert np.array_equal(got[i], separate(alone, x, rc, sim, nmem, 4, sort)), steps[i]
    ctx.close()
    alone.close()


def test_step_list_more_than_16_radii(cnn):
    rng = np.random.default_rng(9)
    x = rng.normal(size=(3000, 2))
    radii = list(np.linspace(0.002, 0.04, 20))
    ctx = cnn.Context(0)
    ctx.set_points(x)
    got = ctx.sweep_pairs(radii, [(4, 3)] * len(radii), member_cutoff=2)
    alone = cnn.Context(0)
    for i, rc in enumerate(radii):
        assert np.array_equal(got[i], separate(alone, x, rc, 4, 3, 2))
    ctx.close()
    alone.close()


def test_hierarchical_repeat_matches_reference(cnn):
    g = load_golden("hierarchy_repeat.npz")
    cl = cnn.Clustering(g["points"], hierarchical_fitter="repeat")
    cl.fit_hierarchical(radius_cutoff=list(g["radii"]), cnn_cutoff=list(g["cuts"]),
                        member_cutoff=int(g["member_cutoff"]), v=False)
    want = golden_tree(g)
    got = bundle_tree(cl._bundle)
    assert set(got) == set(want)
    for path, (lab, root, parent) in want.items():
        assert np.array_equal(got[path][0], lab), path
        assert np.array_equal(got[path][1], root), path
    cl.reel()
    assert np.array_equal(np.asarray(cl.labels), g["reeled"])


def test_hierarchical_repeat_against_oracle(cnn):
    x = cnn_points = load_golden("blobs2d_5k.npz")["points"]
    radii, cuts = [0.12, 0.06, 0.03], [5, 8, 5]
    cl = cnn.Clustering(cnn_points, hierarchical_fitter="repeat")
    cl.fit_hierarchical(radius_cutoff=radii, cnn_cutoff=cuts, member_cutoff=10, v=False)
    steps = o.repeat_step_labels(x, radii, cuts, member_cutoff=10)
    assert np.array_equal(np.asarray(cl.labels), steps[0])
    for label, child in cl.children.items():
        assert np.array_equal(np.asarray(child.labels), steps[1][child.root_indices])


@pytest.mark.parametrize("case", [0, 1, 2])
def test_predict_matches_reference(cnn, case):
    x, labels, y, r, c, clusters, want = predict_cases(load_golden("predict_firstmatch.npz"))[case]
    cl = cnn.Clustering(x, predictor="firstmatch")
    cl.labels = labels
    other = cnn.Clustering(y)
    cl.predict(other._bundle, r, c, clusters=clusters)
    assert np.array_equal(np.asarray(other.labels), want)
    assert other._bundle._labels.meta["frozen"]


@pytest.mark.parametrize("d,fpmode", [(2, 0), (3, 1), (5, 0), (16, 0)])
def test_predict_against_oracle(cnn, d, fpmode):
    rng = np.random.default_rng(70 + d)
    centres = rng.uniform(-3, 3, size=(4, d))
    x = np.vstack([cc + rng.normal(0, 0.5, size=(300, d)) for cc in centres])
    y = np.vstack([cc + rng.normal(0, 0.6, size=(250, d)) for cc in centres])
    r = 0.5 if d <= 3 else (1.1 if d == 5 else 2.4)
    prm = o.make_parameters(r, 4, 0)
    ref_labels, _ = o.clustering_fit(x, r, 4, member_cutoff=3, fpmode=fpmode)
    clusters = sorted(set(ref_labels.tolist()) - {0})[:3]
    # some other points already decided: they keep their label
    start = np.zeros(y.shape[0], dtype=np.int64)
    cons = np.ones(y.shape[0], dtype=np.uint8)
    start[::17] = 99
    cons[::17] = 0
    want, want_cons = o.predict_firstmatch(x, ref_labels, y, prm["radius_cutoff"], prm["similarity_cutoff"],
                                           prm["n_member_cutoff"], clusters, start, cons, fpmode=fpmode)
    ctx = cnn.Context(0)
    ctx.set_points(x)
    got, got_cons = start.copy(), cons.copy()
    ctx.predict(y, ref_labels, clusters, prm["radius_cutoff"], prm["similarity_cutoff"], prm["n_member_cutoff"],
                got, got_cons, fpmode=fpmode)
    assert np.array_equal(got, want)
    assert np.array_equal(got_cons, want_cons)
    # device arrays, float32 other points widened exactly
    import torch
    yt = torch.from_numpy(y.astype(np.float32)).cuda()
    want32, _ = o.predict_firstmatch(x, ref_labels, y.astype(np.float32).astype(np.float64), prm["radius_cutoff"],
                                     prm["similarity_cutoff"], prm["n_member_cutoff"], clusters, fpmode=fpmode)
    lt = torch.zeros(y.shape[0], dtype=torch.int64, device="cuda")
    ct = torch.ones(y.shape[0], dtype=torch.uint8, device="cuda")
    ctx.set_points(torch.from_numpy(x).cuda())
    ctx.predict(yt, torch.from_numpy(ref_labels).cuda(), clusters, prm["radius_cutoff"], prm["similarity_cutoff"],
                prm["n_member_cutoff"], lt, ct, fpmode=fpmode)
    torch.cuda.synchronize()
    assert np.array_equal(lt.cpu().numpy(), want32)
    ctx.close()


def test_predict_edge_cases(cnn):
    ctx = cnn.Context(0)
    x = np.random.default_rng(3).normal(size=(200, 2))
    ctx.set_points(x)
    labels = np.ones(200, dtype=np.int64)
    # no other points
    ctx.predict(np.zeros((0, 2)), labels, [1], 0.25, 3, 2, np.zeros(0, dtype=np.int64), np.zeros(0, dtype=np.uint8))
    # empty consider set: nothing is assigned
    out, cons = np.zeros(10, dtype=np.int64), np.ones(10, dtype=np.uint8)
    ctx.predict(x[:10], labels, [], 0.25, 3, 2, out, cons)
    assert not out.any() and cons.all()
    # similarity cutoff 0 takes the first labelled neighbour with enough neighbours
    ctx.predict(x[:10], labels, [1], 0.25, 0, 2, out, cons)
    want, _ = o.predict_firstmatch(x, labels, x[:10], 0.25, 0, 2, [1])
    assert np.array_equal(out, want)
    with pytest.raises(cnn.CNNError):
        ctx.predict(np.zeros((3, 3)), labels, [1], 0.25, 3, 2, np.zeros(3, dtype=np.int64),
                    np.ones(3, dtype=np.uint8))
    ctx.close()


@pytest.mark.parametrize("d", [1, 2, 3])
def test_predict_on_the_cell_grid_against_oracle(cnn, d):
    """Other points binned into this set's cell grid (n_dim <= 3): points
    far outside the grid, just outside its edge, non-finite ones and
    duplicates of clustered points get the oracle's labels."""
    rng = np.random.default_rng(300 + d)
    centres = rng.uniform(-3, 3, size=(5, d))
    x = np.vstack([cc + rng.normal(0, 0.45, size=(3000, d)) for cc in centres])
    y = np.vstack([cc + rng.normal(0, 0.6, size=(2500, d)) for cc in centres])
    lo, hi = x.min(0), x.max(0)
    y[:20] = hi + 0.1                      # just outside the grid's edge
    y[20:40] = lo - 0.15
    y[40:60] = hi + 50.0                   # far outside
    y[60:80] = x[100:120]                  # duplicates of clustered points
    y[80, 0] = np.nan
    y[81, -1] = np.inf
    r = 0.35 if d > 1 else 0.02
    prm = o.make_parameters(r, 4, 0)
    ref_labels, _ = o.clustering_fit(x, r, 4, member_cutoff=3)
    clusters = sorted(set(ref_labels.tolist()) - {0})
    want, want_cons = o.predict_firstmatch(x, ref_labels, y, prm["radius_cutoff"], prm["similarity_cutoff"],
                                           prm["n_member_cutoff"], clusters)
    ctx = cnn.Context(0)
    try:
        ctx.set_points(x)
        got = np.zeros(y.shape[0], dtype=np.int64)
        got_cons = np.ones(y.shape[0], dtype=np.uint8)
        ctx.predict(y, ref_labels, clusters, prm["radius_cutoff"], prm["similarity_cutoff"], prm["n_member_cutoff"],
                    got, got_cons)
        assert ctx.stats()["search_kind"] == 1  # this set's graph (and the cross rows) on the grid
        assert np.array_equal(got, want)
        assert np.array_equal(got_cons, want_cons)
    finally:
        ctx.close()
