"""Plug the GPU fitter into the reference package itself.

``register_with_reference()`` makes the GPU components usable from
cnnclustering's own ``Clustering`` and recipe registry (when cnnclustering
is importable):

* ``FitterGPU`` becomes a virtual subclass of ``cnnclustering._fit.Fitter``
  (the reference registers its Ext types the same way,
  src/cnnclustering/_types.pyx:1279-1282), so ``Clustering`` accepts it;
* the names ``"gpu"`` (fitter), ``"grid"`` (neighbours getter),
  ``"gpu"`` (similarity checker) and ``"union_find"`` (queue) are added to
  ``cnnclustering.recipes.COMPONENT_NAME_TYPE_MAP``, and a ``"gpu"``
  recipe to ``REGISTERED_RECIPES``.

After that, ``cluster.Clustering(X, recipe="gpu").fit(r, c)`` runs the
reference's orchestration with the GPU fit.  FitterGPU reads the
reference's InputDataExtComponentsMemoryview (``.data``) and writes the
reference's Labels (``.labels``/``.consider`` views) in place.
"""
from __future__ import annotations

from . import _fit, _types

GPU_RECIPE = {
    "input_data": "components_mview",
    "preparation_hook": "points_from_parts",
    "fitter": "gpu",
    "fitter.ngetter": "grid",
    "fitter.na": "gpu",
    "fitter.checker": "gpu",
    "fitter.queue": "union_find",
    "fitter.ngetter.dgetter": "gpu_metric",
    "fitter.ngetter.dgetter.metric": "gpu_euclidean_r",
}


def reference_fitter_type():
    """FitterGPU as the reference's Clustering needs it: the reference types
    the parameters argument of its fit (``ClusterParameters cluster_params``,
    src/cnnclustering/cluster.pyx:250-254), so make_parameters must hand out
    the reference's own ClusterParameters; everything else is FitterGPU."""
    import cnnclustering._types as ref_types

    class FitterGPUForReference(_fit.FitterGPU):
        def make_parameters(self, radius_cutoff, cnn_cutoff, current_start):
            p = super().make_parameters(radius_cutoff, cnn_cutoff, current_start)
            return ref_types.ClusterParameters(p.radius_cutoff, p.similarity_cutoff, p.similarity_cutoff_continuous,
                                               p.n_member_cutoff, p.current_start)

    return FitterGPUForReference


def register_with_reference():
    """Register the GPU components with an importable cnnclustering."""
    import cnnclustering._fit as ref_fit
    import cnnclustering.recipes as ref_recipes

    fitter_type = reference_fitter_type()
    ref_fit.Fitter.register(fitter_type)
    m = ref_recipes.COMPONENT_NAME_TYPE_MAP
    m["fitter"]["gpu"] = fitter_type
    m["neighbours_getter"]["grid"] = _types.NeighboursGetterGPUGrid
    m["neighbours"]["gpu"] = _types.NeighboursGPU
    m["similarity_checker"]["gpu"] = _types.SimilarityCheckerGPU
    m.setdefault("queue", {})["union_find"] = _types.QueueGPUUnionFind
    m["distance_getter"]["gpu_metric"] = _types.DistanceGetterGPUMetric
    m["metric"]["gpu_euclidean_r"] = _types.MetricGPUEuclideanReduced
    m["metric"]["gpu_euclidean"] = _types.MetricGPUEuclidean
    ref_recipes.REGISTERED_RECIPES["gpu"] = dict(GPU_RECIPE)
    return ref_recipes.REGISTERED_RECIPES["gpu"]
