"""Recipes: named component sets and the Builder that assembles them.

Same recipe language as the reference (src/cnnclustering/recipes.py:
181-313, 316-445): dotted keys (``"fitter.ngetter.dgetter.metric"``),
``__`` accepted for ``.``, short aliases (``ngetter``, ``na``,
``checker`` ...), values given as registered names, types, or
``(type_or_name, args, kwargs)`` tuples, and types that list their own
sub-components through ``get_builder_kwargs``.  The registered recipes
name GPU components; ``"coordinates"`` (the reference's default name) is
the GPU cell-grid fit.
"""
from __future__ import annotations

from collections.abc import Iterable

import numpy as np

from . import _fit, _mst, _predict, _types

P_AINDEX = _types.P_AINDEX
P_AVALUE = _types.P_AVALUE


def prepare_pass(data):
    return (data,), {}


def prepare_points_from_parts(data):
    """Stack point parts into one [n, d] float64 array (meta["edges"] holds
    the part lengths), accepting one point, a 2D sequence or a sequence of
    2D parts (src/cnnclustering/recipes.py:52-147).  CUDA tensors pass
    through unchanged."""
    from . import _abi
    if _abi.is_device_array(data):
        return (data,), {"meta": {"edges": [int(data.shape[0])]}}
    if isinstance(data, np.ndarray) and data.ndim == 2:
        return (np.ascontiguousarray(data, dtype=P_AVALUE),), {"meta": {"edges": [data.shape[0]]}}
    if len(data) == 0:
        parts = [np.zeros((0, 0))]
    else:
        try:
            d2 = [len(x) for x in data]
        except TypeError:
            parts = [np.array([data], dtype=P_AVALUE)]
        else:
            try:
                d3 = [len(y) for x in data for y in x]
            except TypeError:
                if len(set(d2)) != 1:
                    raise ValueError("Dimension mismatch")
                parts = [np.asarray(data, dtype=P_AVALUE)]
            else:
                if len(set(d3)) != 1:
                    raise ValueError("Dimension mismatch")
                parts = [np.asarray(x, dtype=P_AVALUE) for x in data]
    meta = {"edges": [x.shape[0] for x in parts]}
    stacked = np.vstack(parts) if parts[0].size or len(parts) > 1 else parts[0]
    return (np.asarray(stacked, order="C", dtype=P_AVALUE),), {"meta": meta}


def prepare_neighbourhoods(data):
    """Neighbourhood sequences -> CSR arrays (offsets int64, indices int32)."""
    inp = _types.InputDataGPUNeighbourhoods.from_sequence(list(data))
    return inp.data, {"meta": {}}


class Builder:
    default_recipe = "coordinates"
    default_preparation_hook = staticmethod(prepare_pass)

    def __init__(self, recipe=None, **kwargs):
        if recipe is None:
            recipe = self.default_recipe
        if isinstance(recipe, str):
            recipe = get_registered_recipe(recipe)
        recipe = dict(recipe)
        recipe.update(kwargs)
        recipe = {k.replace("__", "."): v for k, v in recipe.items()}
        self.recipe = {".".join(COMPONENT_ALT_KW_MAP.get(kw, kw) for kw in k.split(".")): v
                       for k, v in recipe.items()}

    def make_component(self, component_kw, alternative=None, prev_kw=None):
        prev_kw = [] if prev_kw is None else prev_kw
        full_kw = ".".join([*prev_kw, component_kw])
        if alternative is not None:
            alternative = full_kw.rsplit(".", 1)[0] + f".{alternative}"
        if full_kw in self.recipe:
            details = self.recipe[full_kw]
        elif alternative is not None and alternative in self.recipe:
            details = self.recipe[alternative]
        else:
            return object
        if details is None:
            return None
        kw_type = COMPONENT_KW_TYPE_ALIAS_MAP.get(component_kw, component_kw)
        args, kwargs = (), {}
        if isinstance(details, str):
            component_type = COMPONENT_NAME_TYPE_MAP[kw_type][details]
        elif isinstance(details, tuple):
            component_type, args, kwargs = details
            kwargs = dict(kwargs)
            if isinstance(component_type, str):
                component_type = COMPONENT_NAME_TYPE_MAP[kw_type][component_type]
        else:
            component_type = details
        if hasattr(component_type, "get_builder_kwargs"):
            for sub_kw, alt in component_type.get_builder_kwargs():
                sub = self.make_component(sub_kw, alt, prev_kw=full_kw.split("."))
                if sub is not object:
                    kwargs[sub_kw] = sub
        return component_type(*args, **kwargs)

    def make_input_data(self, data, preparation_hook=None, details=None):
        if preparation_hook is None:
            preparation_hook = self.recipe.get("preparation_hook", self.default_preparation_hook)
            if isinstance(preparation_hook, str):
                preparation_hook = COMPONENT_NAME_TYPE_MAP["preparation_hook"][preparation_hook]
        if details is None:
            try:
                details = self.recipe["input_data"]
            except KeyError:
                raise LookupError("Input data type details not found")
        args, kwargs = (), {}
        if isinstance(details, str):
            component_type = COMPONENT_NAME_TYPE_MAP["input_data"][details]
        elif isinstance(details, tuple):
            component_type, args, kwargs = details
            kwargs = dict(kwargs)
            if isinstance(component_type, str):
                component_type = COMPONENT_NAME_TYPE_MAP["input_data"][component_type]
        else:
            component_type = details
        data_args, data_kwargs = preparation_hook(data)
        args = (*data_args, *args)
        data_kwargs.setdefault("meta", {})
        data_kwargs["meta"].update(kwargs.get("meta", {}))
        kwargs.update(data_kwargs)
        return component_type(*args, **kwargs)


_GPU_POINTS = {
    "input_data": "components_gpu",
    "preparation_hook": "points_from_parts",
    "fitter": "gpu",
    "fitter.ngetter": "grid",
    "fitter.na": "gpu",
    "fitter.checker": "gpu",
    "fitter.queue": "union_find",
    "fitter.ngetter.dgetter": "metric",
    "fitter.ngetter.dgetter.metric": "euclidean_r",
}

REGISTERED_RECIPES = {
    "none": {},
    "coordinates": dict(_GPU_POINTS),
    "gpu_coordinates": dict(_GPU_POINTS),
    "distances": {
        "input_data": "components_mview",
        "preparation_hook": "points_from_parts",
        "fitter": "gpu",
        "fitter.ngetter": "grid",
        "fitter.na": "gpu",
        "fitter.checker": "gpu",
        "fitter.queue": "union_find",
        "fitter.ngetter.dgetter": "metric",
        "fitter.ngetter.dgetter.metric": "precomputed",
    },
    "neighbourhoods": {
        "input_data": "neighbourhoods_gpu",
        "preparation_hook": "neighbourhoods",
        "fitter": "gpu",
        "fitter.ngetter": "lookup",
        "fitter.na": "gpu",
        "fitter.checker": "gpu",
        "fitter.queue": "union_find",
    },
    "sorted_neighbourhoods": {
        "input_data": "neighbourhoods_gpu",
        "preparation_hook": "neighbourhoods",
        "fitter": "gpu",
        "fitter.ngetter": ("lookup", (), {"is_sorted": True}),
        "fitter.na": "gpu",
        "fitter.checker": "gpu",
        "fitter.queue": "union_find",
    },
}


def get_registered_recipe(key):
    return REGISTERED_RECIPES[key.lower()]


COMPONENT_ALT_KW_MAP = {
    "prep": "preparation_hook", "input": "input_data", "data": "input_data", "n": "neighbours",
    "na": "neighbours", "nb": "neighbour_neighbours", "getter": "neighbours_getter",
    "ogetter": "neighbours_getter_other", "ngetter": "neighbours_getter",
    "ongetter": "neighbours_getter_other", "dgetter": "distance_getter", "checker": "similarity_checker",
    "q": "queue", "pq": "priority_queue", "prioq": "priority_queue", "hfitter": "hierarchical_fitter",
}

COMPONENT_KW_TYPE_ALIAS_MAP = {
    "neighbour_neighbours": "neighbours",
    "neighbour_getter_other": "neighbours_getter",
}

COMPONENT_NAME_TYPE_MAP = {
    "preparation_hook": {"points_from_parts": prepare_points_from_parts, "neighbourhoods": prepare_neighbourhoods,
                         "pass": prepare_pass},
    "input_data": {"components_gpu": _types.InputDataGPUComponents,
                   "components_mview": _types.InputDataGPUComponents,
                   "distances_gpu": _types.InputDataGPUDistances,
                   "distances_linear_gpu": _types.InputDataGPUDistancesLinear,
                   "neighbourhoods_gpu": _types.InputDataGPUNeighbourhoods,
                   "neighbourhoods_mview": _types.InputDataGPUNeighbourhoods},
    "neighbours_getter": {"grid": _types.NeighboursGetterGPUGrid, "brute_force": _types.NeighboursGetterGPUGrid,
                          "lookup": _types.NeighboursGetterGPULookup},
    "distance_getter": {"metric": _types.DistanceGetterGPUMetric, "lookup": _types.DistanceGetterGPULookup},
    "neighbours": {"gpu": _types.NeighboursGPU, "vector": _types.NeighboursGPU, "vuset": _types.NeighboursGPU},
    "metric": {"euclidean": _types.MetricGPUEuclidean, "euclidean_r": _types.MetricGPUEuclideanReduced,
               "euclidean_reduced": _types.MetricGPUEuclideanReduced, "precomputed": _types.MetricGPUPrecomputed,
               "euclidean_periodic_r": _types.MetricGPUEuclideanPeriodicReduced,
               "euclidean_periodic_reduced": _types.MetricGPUEuclideanPeriodicReduced},
    "similarity_checker": {"gpu": _types.SimilarityCheckerGPU, "screen": _types.SimilarityCheckerGPU,
                           "switch": _types.SimilarityCheckerGPU, "contains": _types.SimilarityCheckerGPU},
    "queue": {"union_find": _types.QueueGPUUnionFind, "fifo": _types.QueueGPUUnionFind},
    "fitter": {"gpu": _fit.FitterGPU, "bfs": _fit.FitterGPU},
    "hierarchical_fitter": {"repeat": _fit.HierarchicalFitterRepeatGPU, "mst": _mst.HierarchicalFitterMSTPrimGPU},
    "priority_queue": {"maxheap": _mst.PriorityQueueMaxHeapGPU},
    "predictor": {"firstmatch": _predict.PredictorFirstmatchGPU},
}


def _is_iterable(x):
    return isinstance(x, Iterable)
