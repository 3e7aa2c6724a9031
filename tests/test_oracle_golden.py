"""Pins the oracle to the reference's own outputs (golden fixtures).

The fixtures were produced by running cnnclustering 0.5.0 itself
(tests/golden/make_golden.py).  If the oracle disagrees with any of them,
no GPU parity claim built on the oracle holds.
"""
import hashlib

import numpy as np
import pytest

from conftest import FIT_CASES, fit_kwargs, load_golden
from oracle import cnn_oracle as o


def digest(offsets, indices):
    h = hashlib.sha256()
    h.update(np.ascontiguousarray(offsets, dtype=np.int64).tobytes())
    h.update(np.ascontiguousarray(indices, dtype=np.int32).tobytes())
    return h.hexdigest()


@pytest.mark.parametrize("name", FIT_CASES)
@pytest.mark.parametrize("grid", [False, True])
def test_oracle_neighbourhoods_match_reference(name, grid):
    g = load_golden(name)
    r = float(g["radius_cutoff"])
    off, idx = o.neighbourhoods(g["points"], r * r, grid=grid)
    assert np.array_equal(np.diff(off), g["degrees"])
    assert digest(off, idx) == str(g["csr_sha256"])
    if "indices" in g:
        assert np.array_equal(idx, g["indices"])


@pytest.mark.parametrize("name", FIT_CASES)
def test_oracle_fit_matches_reference(name):
    g = load_golden(name)
    kw = fit_kwargs(g)
    sort = kw.pop("sort_by_size", True)
    labels, _ = o.clustering_fit(g["points"], float(g["radius_cutoff"]), int(g["cnn_cutoff"]),
                                 sort=sort, **kw)
    assert np.array_equal(labels, g["labels"])


@pytest.mark.parametrize("name", ["quickstart.npz", "moons_1500.npz", "edge_3d.npz"])
def test_oracle_bruteforce_fit_matches_reference(name):
    g = load_golden(name)
    kw = fit_kwargs(g)
    sort = kw.pop("sort_by_size", True)
    labels, _ = o.clustering_fit(g["points"], float(g["radius_cutoff"]), int(g["cnn_cutoff"]),
                                 sort=sort, brute_force=True, **kw)
    assert np.array_equal(labels, g["labels"])


def test_oracle_quickstart_readme_vector():
    g = load_golden("quickstart.npz")
    assert g["labels"].tolist() == [1, 1, 1, 1, 1, 0, 0, 0, 0, 2, 2, 2]
    labels, _ = o.clustering_fit(g["points"], 1.5, 1)
    assert labels.tolist() == [1, 1, 1, 1, 1, 0, 0, 0, 0, 2, 2, 2]


def test_oracle_euclidean_sqrt_metric():
    g = load_golden("euclidean_sqrt.npz")
    r = float(g["radius_cutoff"])
    off, idx = o.neighbourhoods(g["points"], r, metric=o.METRIC_EUCLIDEAN)
    assert np.array_equal(off, g["offsets"]) and np.array_equal(idx, g["indices"])
    labels, _ = o.clustering_fit(g["points"], r, int(g["cnn_cutoff"]),
                                 member_cutoff=int(g["member_cutoff"]), metric=o.METRIC_EUCLIDEAN)
    assert np.array_equal(labels, g["labels"])


def test_oracle_frozen_refit():
    g = load_golden("frozen_refit.npz")
    first, _ = o.clustering_fit(g["points"], float(g["r1"]), int(g["c1"]), member_cutoff=int(g["m1"]))
    assert np.array_equal(first, g["first_labels"])
    second, _ = o.clustering_fit(g["points"], float(g["r2"]), int(g["c2"]), member_cutoff=int(g["m2"]),
                                 labels=first, consider=g["consider"], frozen=True)
    assert np.array_equal(second, g["second_labels"])


def test_oracle_sort_by_size_vectors():
    g = load_golden("sort_by_size.npz")
    for i in range(int(g["n_cases"])):
        lab = g[f"in_{i}"].copy()
        mc = int(g["member_cutoff"][i])
        mx = int(g["max_clusters"][i])
        o.sort_by_size(lab, None if mc < 0 else mc, None if mx < 0 else mx)
        assert np.array_equal(lab, g[f"out_{i}"]), i


def test_oracle_check_truth_table():
    g = load_golden("check_table.npz")
    pa = pb = 0
    for k in range(g["c"].shape[0]):
        a = g["a"][pa:pa + g["len_a"][k]]
        b = g["b"][pb:pb + g["len_b"][k]]
        pa += g["len_a"][k]
        pb += g["len_b"][k]
        assert o.check_sorted(a, b, int(g["c"][k])) == bool(g["expected"][k]), k


def test_oracle_fused_mode_differs_only_by_rounding():
    # The fused mode is the reference compiled with FMA contraction; no
    # build of the reference here uses it, so it is checked by construction:
    # same sets except pairs whose squared distance lies within a few ulps
    # of the cutoff.
    rng = np.random.default_rng(0)
    x = rng.normal(size=(3000, 3))
    r2 = 0.3 ** 2
    a = o.neighbourhoods(x, r2, fpmode=o.FP_SEPARATE)
    b = o.neighbourhoods(x, r2, fpmode=o.FP_FUSED)
    da, db = np.diff(a[0]), np.diff(b[0])
    assert np.abs(da - db).sum() <= 4


def test_oracle_predict_firstmatch_matches_reference():
    from conftest import predict_cases
    for x, labels, y, r, c, clusters, want in predict_cases(load_golden("predict_firstmatch.npz")):
        prm = o.make_parameters(r, c, 0)
        if clusters is None:
            clusters = set(np.unique(labels).tolist()) - {0}
        got, cons = o.predict_firstmatch(x, labels, y, prm["radius_cutoff"], prm["similarity_cutoff"],
                                         prm["n_member_cutoff"], clusters)
        assert np.array_equal(got, want)
        assert np.array_equal(cons == 0, got != 0)


def test_oracle_repeat_steps_match_reference_tree():
    from conftest import golden_tree
    g = load_golden("hierarchy_repeat.npz")
    steps = o.repeat_step_labels(g["points"], g["radii"], g["cuts"], member_cutoff=int(g["member_cutoff"]))
    tree = golden_tree(g)
    checked = 0
    for path, (lab, root, _) in tree.items():
        depth = len(path)
        if depth >= steps.shape[0]:
            assert lab.shape[0] == 0  # leaves of the last step carry no labels
            continue
        idx = np.arange(g["points"].shape[0]) if depth == 0 else root
        assert np.array_equal(lab, steps[depth][idx]), path
        checked += 1
    assert checked > 5


def test_oracle_periodic_metric_matches_reference():
    g = load_golden("periodic_dihedrals.npz")
    for k in range(int(g["n_cases"])):
        r, c, mc = g[f"params_{k}"]
        off, idx = o.periodic_neighbourhoods(g["points"], g["bounds"], r * r)
        assert digest(off, idx) == str(g[f"csr_sha256_{k}"])
        labels = o.fit_from_neighbourhoods(off, idx, int(c), member_cutoff=int(mc))
        assert np.array_equal(labels, g[f"labels_{k}"])


def test_oracle_precomputed_distances_match_reference():
    from conftest import pairwise_distances
    g = load_golden("precomputed_distances.npz")
    dist = pairwise_distances(g["points"])
    iu = np.triu_indices(dist.shape[0], 1)
    r, c, mc = float(g["radius_cutoff"]), int(g["cnn_cutoff"]), int(g["member_cutoff"])
    sq = o.fit_from_neighbourhoods(*o.distance_neighbourhoods(dist, r), c, member_cutoff=mc)
    lin = o.fit_from_neighbourhoods(*o.distance_neighbourhoods(dist[iu], r, linear=True), c, member_cutoff=mc)
    assert np.array_equal(sq, g["labels_square"])
    assert np.array_equal(lin, g["labels_linear"])
