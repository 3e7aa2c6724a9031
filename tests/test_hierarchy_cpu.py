"""Hierarchy bookkeeping of HierarchicalFitterRepeatGPU, isolate() and reel()
against the tree the reference built (tests/golden/hierarchy_repeat.npz).

The per-step labels come from the oracle here (no GPU); the tree, the
reference indices and reel() are this package's host code.
"""
import numpy as np
import pytest

from conftest import bundle_tree, golden_tree, load_golden
from oracle import cnn_oracle as o


@pytest.fixture()
def hierarchy(monkeypatch):
    import commonnnclustering_gb300 as cnn
    g = load_golden("hierarchy_repeat.npz")

    def oracle_steps(self, bundle, params, member_cutoff, max_clusters, sort_by_size):
        return o.repeat_step_labels(bundle._input_data.data, [p.radius_cutoff for p in params],
                                    [p.similarity_cutoff for p in params], member_cutoff=member_cutoff,
                                    max_clusters=max_clusters, sort=sort_by_size)

    monkeypatch.setattr(cnn.HierarchicalFitterRepeatGPU, "step_labels", oracle_steps)
    cl = cnn.Clustering(g["points"], hierarchical_fitter="repeat")
    cl.fit_hierarchical(radius_cutoff=list(g["radii"]), cnn_cutoff=list(g["cuts"]),
                        member_cutoff=int(g["member_cutoff"]), v=False)
    return cnn, g, cl


def test_parameters_pass_through_unadjusted():
    import commonnnclustering_gb300 as cnn
    p = cnn.HierarchicalFitterRepeatGPU().make_parameters(0.5, 4, 1)
    assert (p.radius_cutoff, p.similarity_cutoff, p.n_member_cutoff) == (0.5, 4, 4)


def test_tree_matches_reference(hierarchy):
    cnn, g, cl = hierarchy
    want = golden_tree(g)
    got = bundle_tree(cl._bundle)
    assert set(got) == set(want)
    for path, (lab, root, parent) in want.items():
        glab, groot, gparent = got[path]
        assert np.array_equal(glab, lab), path
        assert np.array_equal(groot, root), path
        assert np.array_equal(gparent, parent), path
    child = cl[list(want)[-1]]
    assert child.hierarchy_level == len(list(want)[-1])
    assert cl._bundle.get_child(".".join(str(p) for p in list(want)[-1])) is child


def test_reel_matches_reference(hierarchy):
    cnn, g, cl = hierarchy
    cl.reel()
    assert np.array_equal(np.asarray(cl.labels), g["reeled"])


def test_isolate_attaches_subsets_and_parts():
    import commonnnclustering_gb300 as cnn
    x = np.arange(20, dtype=np.float64).reshape(10, 2)
    cl = cnn.Clustering([x[:4], x[4:]])  # two parts: meta edges [4, 6]
    cl.labels = np.array([1, 2, 1, 0, 2, 2, 1, 0, 0, 2])
    cl.isolate()
    assert list(cl.children) == [1, 2]  # order of first occurrence
    one = cl.children[1]
    assert np.array_equal(one.parent_indices, [0, 2, 6])
    assert np.array_equal(one.input_data, x[[0, 2, 6]])
    assert one._input_data.meta["edges"] == [2, 1]
    assert cl.children[2]._input_data.meta["edges"] == [1, 3]
    assert one.alias == "rootroot - 1"  # the reference appends to the child's default alias "root"


def test_trim_trivial_leafs():
    import commonnnclustering_gb300 as cnn
    cl = cnn.Clustering(np.zeros((4, 2)))
    cl.labels = np.array([1, 1, 2, 2])
    cl.isolate()
    cl.children[1].labels = np.array([0, 0])
    cl.trim_trivial_leafs()
    assert cl.children[1]._labels is None


def nonnested_points():
    rng = np.random.default_rng(2024)
    parents = rng.uniform(-6, 6, size=(6, 2))
    kids = (parents[:, None, :] + rng.normal(0, 0.6, size=(6, 4, 2))).reshape(-1, 2)
    x = np.vstack([k + rng.normal(0, 0.15, size=(90, 2)) for k in kids])
    return np.ascontiguousarray(x[rng.permutation(x.shape[0])])


NONNESTED = dict(radius_cutoff=[0.03, 0.1, 0.4, 0.9], cnn_cutoff=[10, 8, 5, 3], member_cutoff=5)


def test_nonnested_step_list_raises_like_the_reference(monkeypatch):
    """Step lists whose later clusters merge earlier ones (radius growing):
    a step-k cluster spans several step-(k-1) clusters.  The reference's
    repeat fitter then fails inside Bundle.isolate with an IndexError, and so
    does this package's (the same isolate bookkeeping) -- the order in which
    the parents are walked never shows in a result."""
    import os
    import sys
    import commonnnclustering_gb300 as cnn
    from conftest import ROOT
    x = nonnested_points()

    def oracle_steps(self, bundle, params, member_cutoff, max_clusters, sort_by_size):
        return o.repeat_step_labels(bundle._input_data.data, [p.radius_cutoff for p in params],
                                    [p.similarity_cutoff for p in params], member_cutoff=member_cutoff,
                                    max_clusters=max_clusters, sort=sort_by_size)

    monkeypatch.setattr(cnn.HierarchicalFitterRepeatGPU, "step_labels", oracle_steps)
    cl = cnn.Clustering(x, hierarchical_fitter="repeat")
    with pytest.raises(IndexError):
        cl.fit_hierarchical(v=False, **NONNESTED)
    ref = os.path.join(ROOT, "baseline", "_ref")
    if not os.path.isdir(os.path.join(ref, "cnnclustering")):
        pytest.skip("reference package not installed here")
    sys.path.insert(0, ref)
    try:
        ref_cluster = pytest.importorskip("cnnclustering.cluster")
        recipe = {"input_data": "components_mview", "preparation_hook": "points_from_parts",
                  "hierarchical_fitter": "repeat", "hierarchical_fitter.fitter": "bfs",
                  "hierarchical_fitter.fitter.ngetter": "brute_force", "hierarchical_fitter.fitter.na": "vuset",
                  "hierarchical_fitter.fitter.checker": "switch", "hierarchical_fitter.fitter.queue": "fifo",
                  "hierarchical_fitter.fitter.ngetter.dgetter": "metric",
                  "hierarchical_fitter.fitter.ngetter.dgetter.metric": "euclidean_r"}
        rcl = ref_cluster.Clustering(x, recipe=recipe)
        with pytest.raises(IndexError):
            rcl.fit_hierarchical(v=False, **NONNESTED)
    finally:
        sys.path.remove(ref)
