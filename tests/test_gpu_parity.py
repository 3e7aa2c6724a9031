"""GPU parity: the CUDA path against the reference's golden fixtures and
against the oracle, through the C ABI (libcnngpu.so).

Integer/index results are compared bit-exactly: neighbour lists (CSR),
labels, consider flags.
"""
import numpy as np
import pytest

from conftest import FIT_CASES, fit_kwargs, load_golden

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def cnn():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import commonnnclustering_gb300 as cnn
    return cnn


@pytest.fixture(scope="module")
def oracle():
    from oracle import cnn_oracle
    return cnn_oracle


def gpu_csr(cnn, x, radius_cutoff, metric=0, fpmode=0):
    ctx = cnn.Context(0)
    ctx.set_points(np.ascontiguousarray(x))
    ctx.build_neighbours(radius_cutoff, metric, fpmode)
    off, idx = ctx.get_neighbours(x.shape[0])
    st = ctx.stats()
    ctx.close()
    return off, idx, st


@pytest.mark.parametrize("name", FIT_CASES)
def test_golden_neighbourhoods(cnn, name):
    import hashlib
    g = load_golden(name)
    r = float(g["radius_cutoff"])
    off, idx, _ = gpu_csr(cnn, g["points"], r * r)
    assert np.array_equal(np.diff(off), g["degrees"])
    h = hashlib.sha256()
    h.update(off.astype(np.int64).tobytes())
    h.update(idx.astype(np.int32).tobytes())
    assert h.hexdigest() == str(g["csr_sha256"])


@pytest.mark.parametrize("name", FIT_CASES)
def test_golden_fit_labels(cnn, name):
    g = load_golden(name)
    kw = fit_kwargs(g)
    cl = cnn.Clustering(g["points"])
    cl.fit(float(g["radius_cutoff"]), int(g["cnn_cutoff"]), v=False, **kw)
    assert np.array_equal(np.asarray(cl.labels), g["labels"])


def test_readme_quickstart(cnn):
    data = [[0, 0], [1, 1], [1, 0], [0, -1], [0.5, -0.5], [2, 1.5], [2.5, -0.5], [4, 2], [4.5, 2.5],
            [5, -1], [5.5, -0.5], [5.5, -1.5]]
    cl = cnn.Clustering(data)
    cl.fit(radius_cutoff=1.5, cnn_cutoff=1, v=False)
    assert cl.labels.tolist() == [1, 1, 1, 1, 1, 0, 0, 0, 0, 2, 2, 2]


def test_golden_euclidean_sqrt_metric(cnn):
    g = load_golden("euclidean_sqrt.npz")
    r = float(g["radius_cutoff"])
    off, idx, _ = gpu_csr(cnn, g["points"], r, metric=1)
    assert np.array_equal(off, g["offsets"]) and np.array_equal(idx, g["indices"])
    b = cnn.recipes.Builder("coordinates", **{"fitter.ngetter.dgetter.metric": "euclidean"})
    cl = cnn.Clustering(g["points"], fitter=b.make_component("fitter"))
    cl.fit(r, int(g["cnn_cutoff"]), member_cutoff=int(g["member_cutoff"]), v=False)
    assert np.array_equal(np.asarray(cl.labels), g["labels"])


def test_golden_frozen_refit(cnn):
    g = load_golden("frozen_refit.npz")
    cl = cnn.Clustering(g["points"])
    cl.fit(float(g["r1"]), int(g["c1"]), member_cutoff=int(g["m1"]), v=False)
    assert np.array_equal(np.asarray(cl.labels), g["first_labels"])
    cl._bundle._labels.meta["frozen"] = True
    cl._bundle._labels.consider[:] = g["consider"]
    cl.fit(float(g["r2"]), int(g["c2"]), member_cutoff=int(g["m2"]), v=False)
    assert np.array_equal(np.asarray(cl.labels), g["second_labels"])


def test_golden_sort_by_size(cnn):
    g = load_golden("sort_by_size.npz")
    for i in range(int(g["n_cases"])):
        lab = cnn.Labels(g[f"in_{i}"].copy())
        mc, mx = int(g["member_cutoff"][i]), int(g["max_clusters"][i])
        lab.sort_by_size(None if mc < 0 else mc, None if mx < 0 else mx)
        assert np.array_equal(lab.labels, g[f"out_{i}"]), i


def test_golden_check_truth_table(cnn):
    g = load_golden("check_table.npz")
    ctx = cnn.default_context(0)
    pa = pb = 0
    for k in range(g["c"].shape[0]):
        a = g["a"][pa:pa + g["len_a"][k]]
        b = g["b"][pb:pb + g["len_b"][k]]
        pa += g["len_a"][k]
        pb += g["len_b"][k]
        assert ctx.check_lists(a, b, int(g["c"][k])) == bool(g["expected"][k]), k


@pytest.mark.parametrize("d", [1, 2, 3, 5, 16, 64])
@pytest.mark.parametrize("fpmode", [0, 1])
def test_random_csr_against_oracle(cnn, oracle, d, fpmode):
    rng = np.random.default_rng(100 + d)
    n = 3000 if d <= 3 else 1500
    x = np.vstack([rng.normal(0, 1, size=(n // 2, d)), rng.normal(3, 0.5, size=(n - n // 2, d))])
    # radius giving ~30 neighbours
    sub = x[rng.choice(n, 64, replace=False)]
    dd = np.sort(((sub[:, None, :] - x[None]) ** 2).sum(-1), axis=1)[:, 30]
    r2 = float(np.median(dd))
    want = oracle.neighbourhoods(x, r2, fpmode=fpmode, grid=True)
    off, idx, st = gpu_csr(cnn, x, r2, fpmode=fpmode)
    assert np.array_equal(off, want[0]) and np.array_equal(idx, want[1])


def test_boundary_ties_on_lattice(cnn, oracle):
    # integer lattice: many squared distances equal r**2 exactly
    g = np.array([[i, j, k] for i in range(12) for j in range(12) for k in range(12)], dtype=np.float64)
    for r2 in (1.0, 2.0, 3.0, 4.0):
        want = oracle.neighbourhoods(g, r2)
        off, idx, _ = gpu_csr(cnn, g, r2)
        assert np.array_equal(off, want[0]) and np.array_equal(idx, want[1]), r2


def test_nonfinite_points_have_no_neighbours(cnn, oracle):
    rng = np.random.default_rng(3)
    x = rng.normal(size=(500, 3))
    x[7, 1] = np.nan
    x[11, 0] = np.inf
    x[12, 0] = np.inf
    want = oracle.neighbourhoods(x, 0.25, grid=False)
    off, idx, _ = gpu_csr(cnn, x, 0.25)
    assert np.array_equal(off, want[0]) and np.array_equal(idx, want[1])
    assert off[8] - off[7] == 0


def test_degenerate_radius(cnn, oracle):
    rng = np.random.default_rng(4)
    x = np.round(rng.normal(size=(300, 2)), 1)  # many duplicates
    for r2 in (0.0, -1.0, float("nan"), float("inf")):
        want = oracle.neighbourhoods(x, r2, grid=False)
        off, idx, _ = gpu_csr(cnn, x, r2)
        assert np.array_equal(off, want[0]) and np.array_equal(idx, want[1]), r2


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_random_fit_against_oracle(cnn, oracle, seed):
    from commonnnclustering_gb300 import workloads
    rng = np.random.default_rng(seed)
    x = workloads.md3d(n=20000, seed=seed, centre_spread=2.0)
    r = 0.12
    for c, mc in ((0, 2), (3, 5), (10, 10), (40, 2)):
        want, _ = oracle.clustering_fit(x, r, c, member_cutoff=mc)
        cl = cnn.Clustering(x)
        cl.fit(r, c, member_cutoff=mc, v=False)
        assert np.array_equal(np.asarray(cl.labels), want), (seed, c)


def test_fit_unsorted_and_raw_numbering(cnn, oracle):
    from commonnnclustering_gb300 import workloads
    x = workloads.blobs2d()
    want, _ = oracle.clustering_fit(x, 0.3, 5, sort=False)
    cl = cnn.Clustering(x)
    cl.fit(0.3, 5, sort_by_size=False, v=False)
    assert np.array_equal(np.asarray(cl.labels), want)


def test_abi_fit_consider_and_current_start(cnn, oracle):
    from commonnnclustering_gb300 import workloads
    x = workloads.blobs2d(n=3000, seed=5)
    p = oracle.make_parameters(0.3, 4, 7)
    off, idx = oracle.neighbourhoods(x, p["radius_cutoff"])
    rng = np.random.default_rng(9)
    consider = (rng.random(x.shape[0]) < 0.8).astype(np.uint8)
    labels0 = np.where(consider == 0, 3, 0).astype(np.int64)
    want_l, want_c = labels0.copy(), consider.copy()
    oracle.fit_bfs_csr(off, idx, p["similarity_cutoff"], p["n_member_cutoff"], 7, want_c, want_l)
    ctx = cnn.Context(0)
    ctx.set_points(x)
    ctx.build_neighbours(p["radius_cutoff"])
    got_l, got_c = labels0.copy(), consider.copy()
    ctx.fit(p["similarity_cutoff"], p["n_member_cutoff"], 7, got_c, got_l)
    assert np.array_equal(got_l, want_l) and np.array_equal(got_c, want_c)


def test_precomputed_neighbourhoods_recipe(cnn):
    g = load_golden("moons_1500.npz")
    off, idx = g["offsets"], g["indices"]
    rng = np.random.default_rng(0)
    rows = [rng.permutation(idx[off[i]:off[i + 1]]) for i in range(off.shape[0] - 1)]  # unsorted rows
    cl = cnn.Clustering(rows, recipe="neighbourhoods")
    cl.fit(float(g["radius_cutoff"]), int(g["cnn_cutoff"]), v=False)
    assert np.array_equal(np.asarray(cl.labels), g["labels"])


def test_device_tensor_input_and_graph_reuse(cnn, oracle):
    import torch
    from commonnnclustering_gb300 import workloads
    x = workloads.blobs2d()
    xt = torch.from_numpy(x).cuda()
    cl = cnn.Clustering(xt)
    for r, c in ((0.3, 5), (0.3, 8), (0.25, 5)):
        cl.fit(r, c, member_cutoff=10, v=False)
        want, _ = oracle.clustering_fit(x, r, c, member_cutoff=10)
        assert cl.labels.is_cuda
        assert np.array_equal(cl.labels.cpu().numpy(), want)


def test_float32_input_widened_exactly(cnn, oracle):
    from commonnnclustering_gb300 import workloads
    x32 = workloads.nested3d(n=20000, seed=1, n_parents=4)
    x64 = x32.astype(np.float64)
    want, _ = oracle.clustering_fit(x64, 0.06, 5, member_cutoff=10)
    cl = cnn.Clustering(cnn.InputDataGPUComponents(x32))
    cl.fit(0.06, 5, member_cutoff=10, v=False)
    assert np.array_equal(np.asarray(cl.labels), want)


def test_repeated_fits_are_identical(cnn):
    from commonnnclustering_gb300 import workloads
    x = workloads.md3d(n=50000, seed=3)
    outs = []
    for _ in range(3):
        cl = cnn.Clustering(x)
        cl.fit(0.1, 10, member_cutoff=50, v=False)
        outs.append(np.asarray(cl.labels).copy())
    assert all(np.array_equal(outs[0], o) for o in outs[1:])


def test_empty_and_single_point(cnn):
    cl = cnn.Clustering(np.zeros((1, 3)))
    cl.fit(0.5, 0, v=False)
    assert cl.labels.tolist() == [0]
    ctx = cnn.Context(0)
    ctx.set_points(np.zeros((0, 2)))
    ctx.build_neighbours(0.25)
    assert ctx.neighbour_count() == 0
    ctx.fit(2, 1, 1, np.zeros(0, dtype=np.uint8), np.zeros(0, dtype=np.int64))


def test_errors_are_reported(cnn):
    ctx = cnn.Context(0)
    with pytest.raises(cnn.CNNError):
        ctx.fit(2, 1, 1, np.ones(3, dtype=np.uint8), np.zeros(3, dtype=np.int64))  # no graph yet
    with pytest.raises(cnn.CNNError):
        ctx.set_neighbours(np.array([0, 2, 3], dtype=np.int64), np.array([0, 5, 1], dtype=np.int32))


@pytest.mark.parametrize("d", [16, 64])
def test_tensor_core_search_against_oracle(cnn, oracle, d):
    """n_dim >= 16 takes the tcgen05 Gram path; the CSR must equal the oracle's."""
    from commonnnclustering_gb300 import workloads
    x = workloads.features(n=12000, d=d, seed=31, n_clusters=12)
    rng = np.random.default_rng(5)
    sub = x[rng.choice(x.shape[0], 64, replace=False)]
    dd = np.sort(((sub[:, None, :] - x[None]) ** 2).sum(-1), axis=1)[:, 60]
    r2 = float(np.median(dd))
    for fpmode in (0, 1):
        want = oracle.neighbourhoods(x, r2, fpmode=fpmode, grid=False)
        off, idx, st = gpu_csr(cnn, x, r2, fpmode=fpmode)
        assert st["search_kind"] == 3, st
        assert np.array_equal(off, want[0]) and np.array_equal(idx, want[1])


def test_tensor_core_fit_labels(cnn, oracle):
    from commonnnclustering_gb300 import workloads
    x = workloads.features(n=8000, d=64, seed=32, n_clusters=8)
    want, info = oracle.clustering_fit(x, 3.1, 5)
    cl = cnn.Clustering(x)
    cl.fit(3.1, 5, v=False)
    assert np.array_equal(np.asarray(cl.labels), want)


def test_tensor_core_wait_timeout_stops_cleanly(cnn, oracle):
    """A barrier wait of the tensor-core search that runs out (limit 1 ns)
    ends the kernel through its bounded-wait path: the call returns
    CNN_ERR_TIMEOUT, and the same context then searches correctly with the
    default limit (copies drained, tensor memory freed)."""
    from commonnnclustering_gb300 import workloads
    x = workloads.features(n=16000, d=64, seed=33, n_clusters=12)
    r2 = 3.1 ** 2
    want = oracle.neighbourhoods(x, r2, fpmode=0, grid=False)
    ctx = cnn.Context(0)
    ctx.set_points(x)
    ctx.set_wait_limit(1)
    with pytest.raises(cnn.CNNError) as err:
        ctx.build_neighbours(r2)
    assert err.value.status == 4  # CNN_ERR_TIMEOUT
    ctx.set_wait_limit(0)
    for _ in range(2):
        ctx.build_neighbours(r2)
        assert ctx.stats()["search_kind"] == 3
        off, idx = ctx.get_neighbours(x.shape[0])
        assert np.array_equal(off, want[0]) and np.array_equal(idx, want[1])
    ctx.close()


def test_search_preference_changes_the_search_not_the_sets(cnn, oracle):
    """SEARCH_ALL_PAIRS (the plain float32 all-pairs search) and the
    automatic choice (tensor cores at n_dim 16, the cell grid at 3) give the
    oracle's neighbour sets."""
    from commonnnclustering_gb300 import _abi, workloads
    for x, r2, auto_kind in ((workloads.features(n=6000, d=16, seed=35, n_clusters=6), 1.6 ** 2, 3),
                             (workloads.md3d(n=20000, seed=5, centre_spread=2.0), 0.1 ** 2, 1)):
        want = oracle.neighbourhoods(x, r2, grid=x.shape[1] <= 3)
        ctx = cnn.Context(0)
        ctx.set_points(x)
        for pref, kind in ((_abi.SEARCH_ALL_PAIRS, 2), (_abi.SEARCH_AUTO, auto_kind)):
            ctx.set_search(pref)
            ctx.build_neighbours(r2)
            assert ctx.stats()["search_kind"] == kind
            off, idx = ctx.get_neighbours(x.shape[0])
            assert np.array_equal(off, want[0]) and np.array_equal(idx, want[1])
        ctx.close()


@pytest.mark.parametrize("n_values,span", [(3000, 1), (20000, 1), (24576, 1), (40000, 1), (5000, 1000)])
def test_sort_by_size_many_label_values(cnn, oracle, n_values, span):
    """sort_by_size over label ranges on both sides of the one-block ranking
    (<= 24,576 values) and sparse label values (a span far above n)."""
    rng = np.random.default_rng(n_values)
    n = 200_000
    values = (np.arange(1, n_values + 1, dtype=np.int64) * span)
    sizes = rng.zipf(1.6, size=n_values).clip(1, 500)
    lab = np.repeat(values, sizes)[:n]
    lab = np.concatenate([lab, np.zeros(max(0, n - lab.shape[0]), dtype=np.int64)])
    lab = lab[rng.permutation(lab.shape[0])]
    for mc, mx in ((2, None), (5, 100), (1, None)):
        want = lab.copy()
        oracle.sort_by_size(want, mc, mx)
        got = cnn.Labels(lab.copy())
        got.sort_by_size(mc, mx)
        assert np.array_equal(np.asarray(got.labels), want), (mc, mx)


@pytest.mark.parametrize("d", [1, 2, 3])
def test_grid_reach_two_gives_the_same_sets(cnn, oracle, monkeypatch, d):
    """Cells of edge R/2 with a 5-cell stencil per dimension (CNN_GRID_REACH=2,
    read when a context is created) scan fewer candidates and give the
    oracle's neighbour sets and labels."""
    from commonnnclustering_gb300 import _abi, workloads
    monkeypatch.setenv("CNN_GRID_REACH", "2")
    x = np.ascontiguousarray(workloads.md3d(n=20000, seed=9, centre_spread=2.0)[:, :d])
    r2 = 0.1 ** 2 if d == 3 else 0.02 ** 2
    want = oracle.neighbourhoods(x, r2, grid=True)
    ctx = cnn.Context(0)
    try:
        ctx.set_points(x)
        ctx.build_neighbours(r2)
        assert ctx.stats()["search_kind"] == 1
        off, idx = ctx.get_neighbours(x.shape[0])
        assert np.array_equal(off, want[0]) and np.array_equal(idx, want[1])
        labels = np.zeros(x.shape[0], dtype=np.int64)
        consider = np.ones(x.shape[0], dtype=np.uint8)
        ctx.fit(7, 6, 1, consider, labels)
        ref_labels = np.zeros(x.shape[0], dtype=np.int64)
        oracle.fit_bfs_csr(want[0], want[1], 7, 6, 1, np.ones(x.shape[0], dtype=np.uint8), ref_labels)
        assert np.array_equal(labels, ref_labels)
    finally:
        ctx.close()


@pytest.mark.parametrize("mem", ["host", "device"])
@pytest.mark.parametrize("strategy", ["auto", "merge", "bitset"])
def test_fit_fresh_equals_fit_then_sort(cnn, mem, strategy):
    """cnn_fit_fresh (fresh labels made on the device, the sort reading the
    cluster count there) gives the labels of cnn_fit + cnn_sort_by_size on
    fresh arrays, with the intersection tuner's calibration fit, either
    strategy, a cluster limit and no sort."""
    import torch
    from commonnnclustering_gb300 import _abi, workloads
    x = workloads.md3d(n=30000, seed=13, centre_spread=2.0)
    ctx = cnn.Context(0)
    try:
        ctx.set_intersection({"auto": _abi.INTERSECT_AUTO, "merge": _abi.INTERSECT_MERGE,
                              "bitset": _abi.INTERSECT_BITSET}[strategy])
        ctx.set_points(x)
        for (sc, nm, mc, mx, sort) in ((12, 11, 5, None, True), (7, 6, 2, 3, True), (12, 11, 5, None, False)):
            ctx.build_neighbours(0.1 ** 2)
            want = np.zeros(x.shape[0], dtype=np.int64)
            cons = np.ones(x.shape[0], dtype=np.uint8)
            ctx.fit(sc, nm, 1, cons, want)
            if sort:
                ctx.sort_by_size(want, mc, mx)
            ctx.build_neighbours(0.1 ** 2)
            if mem == "host":
                got_cons = np.ones(x.shape[0], dtype=np.uint8)
                got = ctx.fit_fresh(sc, nm, sort, mc, mx, consider=got_cons)
                assert not got_cons.any()
            else:
                lt = torch.full((x.shape[0],), -5, dtype=torch.int64, device="cuda")
                ctx.fit_fresh(sc, nm, sort, mc, mx, labels=lt)
                torch.cuda.synchronize()
                got = lt.cpu().numpy()
            assert np.array_equal(got, want), (sc, nm, mc, mx, sort)
    finally:
        ctx.close()


@pytest.mark.parametrize("n_blobs", [3000, 9000])
def test_fit_fresh_many_clusters(cnn, n_blobs):
    """Thousands of small clusters (beyond the 4,096 labels ranked in shared
    memory for 9,000 blobs): the fresh fit's label counts, taken from the
    component sizes of its union-find, order the clusters as cnn_sort_by_size
    counting the labels does, with a member cutoff that drops some and a
    cluster limit."""
    rng = np.random.default_rng(31)
    centres = rng.uniform(0, 1000, size=(n_blobs, 3))
    sizes = rng.integers(3, 12, size=n_blobs)
    x = np.ascontiguousarray(np.vstack([c + rng.normal(0, 0.05, size=(k, 3)) for c, k in zip(centres, sizes)]))
    x = x[rng.permutation(x.shape[0])]
    ctx = cnn.Context(0)
    try:
        ctx.set_points(x)
        for (mc, mx) in ((2, None), (6, None), (2, n_blobs // 3)):
            ctx.build_neighbours(0.3 ** 2)
            want = np.zeros(x.shape[0], dtype=np.int64)
            ctx.fit(2, 1, 1, np.ones(x.shape[0], dtype=np.uint8), want)
            assert want.max() > 2000
            ctx.sort_by_size(want, mc, mx)
            ctx.build_neighbours(0.3 ** 2)
            got = ctx.fit_fresh(2, 1, True, mc, mx)
            assert np.array_equal(got, want), (mc, mx)
    finally:
        ctx.close()


def test_rows_left_in_their_slots(cnn, oracle):
    """A public cell-grid build leaves the rows where the search wrote them;
    the pair count (cnn_neighbour_count, the statistics), a fit on the slots,
    the exported CSR (made on request) and a fit after it all agree with the
    oracle, and with each other."""
    from commonnnclustering_gb300 import _abi, workloads
    x = workloads.md3d(n=40000, seed=17, centre_spread=2.0)
    r2 = 0.1 ** 2
    want_off, want_idx = oracle.neighbourhoods(x, r2, grid=True)
    ref = np.zeros(x.shape[0], dtype=np.int64)
    oracle.fit_bfs_csr(want_off, want_idx, 12, 11, 1, np.ones(x.shape[0], dtype=np.uint8), ref)
    ctx = cnn.Context(0)
    try:
        ctx.set_intersection(_abi.INTERSECT_MERGE)
        ctx.set_points(x)
        ctx.build_neighbours(r2)
        assert ctx.neighbour_count() == want_idx.shape[0]
        assert ctx.stats()["n_nonzero"] == want_idx.shape[0]
        first = np.zeros(x.shape[0], dtype=np.int64)
        ctx.fit(12, 11, 1, np.ones(x.shape[0], dtype=np.uint8), first)  # on the slots
        assert np.array_equal(first, ref)
        off, idx = ctx.get_neighbours(x.shape[0])  # the CSR, made now
        assert np.array_equal(off, want_off) and np.array_equal(idx, want_idx)
        again = np.zeros(x.shape[0], dtype=np.int64)
        ctx.fit(12, 11, 1, np.ones(x.shape[0], dtype=np.uint8), again)  # on the CSR
        assert np.array_equal(again, ref)
        ctx.build_neighbours(r2)
        got = ctx.fit_fresh(12, 11, True, 2, None)
        sorted_ref = ref.copy()
        ctx.sort_by_size(sorted_ref, 2, None)
        assert np.array_equal(got, sorted_ref)
    finally:
        ctx.close()


def test_stage_times_belong_to_the_last_call(cnn):
    """With timing on, a stage the last build or fit did not run reports 0,
    not an earlier call's time: a fit without its sort after one with it, a
    build that leaves the rows in their slots (no row-offset scan, no fit yet)
    after one whose CSR was made."""
    from commonnnclustering_gb300 import _abi, workloads
    x = workloads.md3d(n=20000, seed=23, centre_spread=2.0)
    ctx = cnn.Context(0)
    try:
        ctx.set_timing(True)
        ctx.set_intersection(_abi.INTERSECT_MERGE)
        ctx.set_points(x)
        ctx.build_neighbours(0.1 ** 2)
        ctx.get_neighbours(x.shape[0])  # the CSR, made on request
        ctx.fit_fresh(12, 11, True, 2, None)
        st = ctx.stats()
        assert st["ms_sort"] > 0 and st["ms_check"] > 0
        ctx.fit_fresh(12, 11, False, 2, None)
        st = ctx.stats()
        assert st["ms_sort"] == 0 and st["ms_check"] > 0
        ctx.build_neighbours(0.1 ** 2)
        st = ctx.stats()
        assert st["ms_count"] > 0 and st["ms_scan"] == 0 and st["ms_check"] == 0
    finally:
        ctx.close()


def test_fit_fresh_on_other_graphs(cnn):
    """cnn_fit_fresh after the tensor-core search (n_dim 16, the graph in the
    search's pivot-grouped order), after precomputed neighbourhoods
    (cnn_set_neighbours) and with only noise: the labels of cnn_fit +
    cnn_sort_by_size."""
    from commonnnclustering_gb300 import workloads
    x = workloads.features(n=6000, d=16, seed=21, n_clusters=6)
    ctx = cnn.Context(0)
    try:
        ctx.set_points(x)
        for r2, sc, nm in ((1.6 ** 2, 7, 6), (1.6 ** 2, 2000, 1999)):  # the second: no node, all noise
            ctx.build_neighbours(r2)
            assert ctx.stats()["search_kind"] == 3
            want = np.zeros(x.shape[0], dtype=np.int64)
            ctx.fit(sc, nm, 1, np.ones(x.shape[0], dtype=np.uint8), want)
            ctx.sort_by_size(want, 5, None)
            ctx.build_neighbours(r2)
            got = ctx.fit_fresh(sc, nm, True, 5, None)
            assert np.array_equal(got, want), (sc, nm)
        off, idx = ctx.get_neighbours()
        ctx.set_neighbours(off, idx)
        want = np.zeros(x.shape[0], dtype=np.int64)
        ctx.fit(7, 6, 1, np.ones(x.shape[0], dtype=np.uint8), want)
        ctx.sort_by_size(want, 3, 4)
        got = ctx.fit_fresh(7, 6, True, 3, 4)
        assert np.array_equal(got, want)
    finally:
        ctx.close()
