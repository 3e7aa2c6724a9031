"""Host-side logic that needs no GPU: recipes, parameters, input
preparation, records; and registration with the reference package when
it is importable here."""
import os
import sys

import numpy as np
import pytest

from conftest import ROOT
from commonnnclustering_gb300 import (ClusterParameters, FitterGPU, Labels, MetricGPUEuclidean, recipes)
from commonnnclustering_gb300.report import Record, Summary


def test_default_recipe_builds_gpu_fitter():
    f = recipes.Builder().make_component("fitter")
    assert isinstance(f, FitterGPU)
    assert f._neighbours_getter.is_selfcounting


@pytest.mark.parametrize("r,c,cs", [(0.3, 5, 1), (1.5, 0, 4), (2.0, 10, 1)])
def test_make_parameters_matches_reference_rule(r, c, cs):
    # _fit.pyx:130-161: r -> r**2 (reduced metric); self-counting: +1 / +2
    p = recipes.Builder().make_component("fitter").make_parameters(r, c, cs)
    assert p.radius_cutoff == r ** 2
    assert p.n_member_cutoff == c + 1 and p.similarity_cutoff == c + 2 and p.current_start == cs


def test_make_parameters_euclidean_metric_keeps_radius():
    b = recipes.Builder(recipes.get_registered_recipe("coordinates"),
                        **{"fitter.ngetter.dgetter.metric": MetricGPUEuclidean})
    p = b.make_component("fitter").make_parameters(0.7, 3, 1)
    assert p.radius_cutoff == 0.7


def test_recipe_aliases_and_dunder_keys():
    b = recipes.Builder("coordinates", fitter__ngetter__dgetter__metric="euclidean")
    assert "fitter.neighbours_getter.distance_getter.metric" in b.recipe
    f = b.make_component("fitter")
    assert isinstance(f._neighbours_getter._distance_getter._metric, MetricGPUEuclidean)


def test_prepare_points_from_parts():
    (data,), kw = recipes.prepare_points_from_parts([[[0, 0], [1, 1]], [[2, 2], [3, 3]]])
    assert data.shape == (4, 2) and kw["meta"]["edges"] == [2, 2]
    (data,), kw = recipes.prepare_points_from_parts([[0, 0], [1, 1], [2, 2]])
    assert data.shape == (3, 2) and data.dtype == np.float64
    (data,), kw = recipes.prepare_points_from_parts([1.0, 2.0, 3.0])
    assert data.shape == (1, 3)


def test_prepare_neighbourhoods_to_csr():
    (off, idx), _ = recipes.prepare_neighbourhoods([[0, 1], [1, 0, 2], [2]])
    assert off.tolist() == [0, 2, 5, 6] and idx.tolist() == [0, 1, 1, 0, 2, 2]


def test_cluster_parameters_defaults():
    p = ClusterParameters(0.5, 3)
    assert p.n_member_cutoff == 3 and p.current_start == 1
    assert set(p.to_dict()) == {"radius_cutoff", "similarity_cutoff", "similarity_cutoff_continuous",
                                "n_member_cutoff", "current_start"}


def test_labels_host_bookkeeping():
    L = Labels(np.array([1, 1, 2, 2, 0, 1], dtype=np.int64))
    assert L.to_set() == {0, 1, 2}
    assert dict(L.to_mapping()) == {0: [4], 1: [0, 1, 5], 2: [2, 3]}
    assert L.consider.dtype == np.uint8 and L.consider.tolist() == [1] * 6
    with pytest.raises(ValueError):
        Labels(np.zeros(3, dtype=np.int64), consider=np.ones(2, dtype=np.uint8))


def test_record_and_summary():
    s = Summary()
    s.append(Record(100, 0.3, 5, 10, None, 3, 0.5, 0.1, 0.25))
    assert len(s) == 1 and "#points" in str(s[0])
    with pytest.raises(TypeError):
        s.append(1)


def test_register_with_reference_package():
    ref = os.path.join(ROOT, "baseline", "_ref")
    if not os.path.isdir(os.path.join(ref, "cnnclustering")):
        pytest.skip("reference package not installed here")
    sys.path.insert(0, ref)
    try:
        pytest.importorskip("cnnclustering")
        from cnnclustering import cluster as ref_cluster
        from cnnclustering import _fit as ref_fit
        from commonnnclustering_gb300 import interop
        interop.register_with_reference()
        cl = ref_cluster.Clustering(np.zeros((4, 2)), recipe="gpu")
        assert isinstance(cl._fitter, FitterGPU)
        assert isinstance(cl._fitter, ref_fit.Fitter)
        p = cl._fitter.make_parameters(0.5, 2, 1)
        assert p.radius_cutoff == 0.25 and p.similarity_cutoff == 4
    finally:
        sys.path.remove(ref)


def test_context_fit_rejects_arrays_of_another_length_before_calling_the_library():
    """Context.fit checks labels/consider against the graph's point count on
    the host; nothing reaches the library (it is not even loaded here)."""
    import numpy as np
    from commonnnclustering_gb300 import _abi
    ctx = object.__new__(_abi.Context)   # no device: only the Python check runs
    ctx._lib = None
    ctx._h = None
    ctx._n_points = 100
    ctx._points_set = True
    with pytest.raises(ValueError):
        ctx.fit(7, 6, 1, np.ones(100, dtype=np.uint8), np.zeros(99, dtype=np.int64))
    with pytest.raises(ValueError):
        ctx.fit(7, 6, 1, np.ones(101, dtype=np.uint8), np.zeros(101, dtype=np.int64))
    with pytest.raises(ValueError):
        ctx.fit(7, 6, 1, np.ones(99, dtype=np.uint8), np.zeros(100, dtype=np.int64))


def test_fitter_graph_key_follows_the_context_generation():
    """FitterGPU reuses a device graph only while the context's graph
    generation is the one recorded at its own build."""
    from commonnnclustering_gb300 import _fit

    class FakeCtx:
        def __init__(self):
            self.gen, self.builds, self.device, self.stream = 0, 0, 0, None

        def graph_generation(self):
            return self.gen

        def set_points(self, data):
            self.gen += 1

        def build_neighbours(self, *a):
            self.gen += 1
            self.builds += 1

    class FakeTensor:
        _version = 0
        shape = (10, 3)
        __cuda_array_interface__ = {"data": (1234, False), "shape": (10, 3), "typestr": "<f8"}

        def data_ptr(self):
            return 1234

    class Inp:
        data = FakeTensor()
        meta = {}

    ctx = FakeCtx()
    f = _fit.FitterGPU(context=ctx)
    f._sync_stream = lambda c, a: None
    p = _fit.ClusterParameters(0.01, 12, 12, 11, 1)
    f.prepare(Inp(), p)
    f.prepare(Inp(), p)
    assert ctx.builds == 1           # reused: nothing else touched the context
    ctx.gen += 1                     # another user replaced the graph
    f.prepare(Inp(), p)
    assert ctx.builds == 2


class _OracleContext:
    """Stands in for the library context on a machine without a GPU: the
    calls FitterGPU makes, computed by the oracle on the same arrays."""

    def __init__(self):
        self.device, self.stream, self._gen, self.x = 0, None, 0, None

    def graph_generation(self):
        return self._gen

    def set_points(self, data):
        self.x = np.asarray(data, dtype=np.float64)
        self._gen += 1

    def build_neighbours(self, radius_cutoff, metric=0, fpmode=None):
        from oracle import cnn_oracle
        self.csr = cnn_oracle.neighbourhoods(self.x, radius_cutoff, metric, fpmode)
        self._gen += 1

    def fit(self, similarity_cutoff, n_member_cutoff, current_start, consider, labels):
        from oracle import cnn_oracle
        cnn_oracle.fit_bfs_csr(self.csr[0], self.csr[1], similarity_cutoff, n_member_cutoff, current_start,
                               np.asarray(consider), np.asarray(labels))


def test_reference_clustering_fit_runs_through_the_gpu_fitter(monkeypatch):
    """The reference's own Clustering.fit (cluster.pyx:256-392) with the
    "gpu" recipe: its orchestration -- make_parameters through FitterGPU's
    getter, fresh and frozen labels, cnn_offset, sort_by_size -- drives
    FitterGPU.fit, whose library calls are answered by the oracle here.  The
    labels equal the reference's default recipe on the same points."""
    ref = os.path.join(ROOT, "baseline", "_ref")
    if not os.path.isdir(os.path.join(ref, "cnnclustering")):
        pytest.skip("reference package not installed here")
    sys.path.insert(0, ref)
    try:
        pytest.importorskip("cnnclustering")
        from cnnclustering import cluster as ref_cluster
        from commonnnclustering_gb300 import _abi, interop, workloads
        interop.register_with_reference()
        fake = _OracleContext()
        monkeypatch.setattr(_abi, "default_context", lambda device=0: fake)
        x = workloads.blobs2d(n=1500, seed=4)
        for kw in ({"member_cutoff": 10}, {"member_cutoff": 5, "cnn_offset": 2}, {"sort_by_size": False}):
            gpu = ref_cluster.Clustering(x, recipe="gpu")
            gpu.fit(0.3, 5, v=False, **kw)
            plain = ref_cluster.Clustering(x)
            plain.fit(0.3, 5, v=False, **kw)
            assert isinstance(gpu._fitter, FitterGPU)
            assert np.array_equal(np.asarray(gpu.labels), np.asarray(plain.labels)), kw
    finally:
        sys.path.remove(ref)
