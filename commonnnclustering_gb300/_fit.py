"""Fitter interface and the GPU fitter.

``Fitter`` mirrors the reference's ABC (src/cnnclustering/_fit.pyx:43-85):
``fit(input_data, labels, cluster_params)`` plus ``make_parameters``,
which turns (r, c) into the ClusterParameters the getter compares with:
r -> metric.adjust_radius(r) and, for a self-counting getter,
n_member_cutoff = c + 1 and similarity_cutoff = c + 2.

``FitterGPU`` is the drop-in for ``FitterExtBFS`` (_fit.pyx:356-504): one
call builds (or takes) the neighbour graph on the device and clusters it;
labels and consider are written in place exactly as the reference's
fitter writes them.
"""
from __future__ import annotations

from abc import ABC, abstractmethod
from typing import Optional

import numpy as np

from . import _abi
from ._types import (ClusterParameters, InputDataGPUDistances, InputDataGPUDistancesLinear,
                     InputDataGPUNeighbourhoods, NeighboursGetterGPUGrid, NeighboursGetterGPULookup,
                     SimilarityCheckerGPU, QueueGPUUnionFind, NeighboursGPU, _device_of)


class Fitter(ABC):
    """Fitter interface (src/cnnclustering/_fit.pyx:43-85)."""

    @abstractmethod
    def fit(self, input_data, labels, cluster_params):
        """Generic clustering"""

    def make_parameters(self, radius_cutoff: float, cnn_cutoff: int,
                        current_start: int) -> ClusterParameters:
        try:
            used_metric = self._neighbours_getter._distance_getter._metric
        except AttributeError:
            pass
        else:
            radius_cutoff = used_metric.adjust_radius(radius_cutoff)

        n_member_cutoff = cnn_cutoff
        try:
            is_selfcounting = self._neighbours_getter.is_selfcounting
        except AttributeError:
            pass
        else:
            if is_selfcounting:
                n_member_cutoff += 1
                cnn_cutoff += 2

        return ClusterParameters(radius_cutoff, cnn_cutoff, cnn_cutoff, n_member_cutoff, current_start)


def _distance_layout(input_data, metric_code: int):
    """DIST_SQUARE / DIST_LINEAR for distance input, None for coordinates."""
    if isinstance(input_data, InputDataGPUDistancesLinear):
        return _abi.DIST_LINEAR
    if isinstance(input_data, InputDataGPUDistances):
        return _abi.DIST_SQUARE
    meta = getattr(input_data, "meta", None) or {}
    if meta.get("access_distances", False) or metric_code == _abi.METRIC_PRECOMPUTED:
        shape = tuple(getattr(input_data.data, "shape", ()))
        return _abi.DIST_LINEAR if len(shape) == 1 else _abi.DIST_SQUARE
    return None


def load_input(ctx: _abi.Context, input_data, neighbours_getter, metric_code: int) -> int:
    """Points or distances of ``input_data`` onto the context; returns the
    metric code the neighbour search uses."""
    layout = _distance_layout(input_data, metric_code)
    if layout is not None:
        ctx.set_distances(input_data.data, layout, n_points=input_data.n_points)
        return _abi.METRIC_PRECOMPUTED
    ctx.set_points(input_data.data)
    if metric_code == _abi.METRIC_EUCLIDEAN_PERIODIC_REDUCED:
        ctx.set_periodic_bounds(neighbours_getter._distance_getter._metric.bounds)
    return metric_code


def _is_neighbourhood_input(input_data) -> bool:
    if isinstance(input_data, InputDataGPUNeighbourhoods):
        return True
    meta = getattr(input_data, "meta", None) or {}
    return bool(meta.get("access_neighbours", False)) and not bool(meta.get("access_coords", False))


class FitterGPU(Fitter):
    """CommonNN fit on the GPU.

    Args mirror ``FitterExtBFS``'s constructor (neighbours getter,
    neighbour containers, similarity checker, queue); only the getter's
    metric, self-counting flag and fpmode influence the result.

    Keyword args:
        device: CUDA device index.
        context: an explicit ``_abi.Context`` (default: one per thread and
            device).
        reuse_graph: keep the neighbour graph on the device between fits
            when the input is a CUDA tensor that has not been modified
            (torch version counter), the radius, metric and fpmode are
            unchanged, and nothing else has replaced the graph of the
            context since (the context's graph generation, which every other
            user of a shared context changes).  Host (numpy) inputs are
            always re-uploaded.
    """

    def __init__(self, neighbours_getter=None, neighbours=None, neighbour_neighbours=None,
                 similarity_checker=None, queue=None, *, device: Optional[int] = None,
                 context: Optional[_abi.Context] = None, reuse_graph: bool = True):
        self._neighbours_getter = neighbours_getter if neighbours_getter is not None else NeighboursGetterGPUGrid()
        self._neighbours = neighbours if neighbours is not None else NeighboursGPU()
        self._neighbour_neighbours = neighbour_neighbours if neighbour_neighbours is not None else NeighboursGPU()
        self._similarity_checker = similarity_checker if similarity_checker is not None else SimilarityCheckerGPU()
        self._queue = queue if queue is not None else QueueGPUUnionFind()
        self._device = device
        self._context = context
        self.reuse_graph = reuse_graph
        self._graph_key = None  # (input identity, parameters, context, graph generation) of the last build
        self.last_stats: dict = {}

    def __str__(self):
        attr_str = ", ".join([
            f"ngetter={self._neighbours_getter}",
            f"na={self._neighbours}",
            f"nb={self._neighbour_neighbours}",
            f"checker={self._similarity_checker}",
            f"queue={self._queue}",
        ])
        return f"{type(self).__name__}({attr_str})"

    @classmethod
    def get_builder_kwargs(cls):
        return [
            ("neighbours_getter", None),
            ("neighbours", None),
            ("neighbour_neighbours", "neighbours"),
            ("similarity_checker", None),
            ("queue", None),
        ]

    def context_for(self, array=None) -> _abi.Context:
        if self._context is None:
            dev = self._device if self._device is not None else _device_of(array) if array is not None else 0
            self._context = _abi.default_context(dev)
        return self._context

    def _metric_code(self) -> int:
        try:
            return int(self._neighbours_getter._distance_getter._metric.code)
        except AttributeError:
            return _abi.METRIC_EUCLIDEAN_REDUCED

    def _fpmode_code(self) -> int:
        return getattr(self._neighbours_getter, "fpmode_code", _abi.host_fpmode())

    def prepare(self, input_data, cluster_params: ClusterParameters) -> _abi.Context:
        """Put the neighbour graph of ``input_data`` on the device."""
        if _is_neighbourhood_input(input_data):
            if isinstance(input_data, InputDataGPUNeighbourhoods):
                offsets, indices = input_data.data
            else:  # the reference's padded neighbourhood input
                offsets, indices = InputDataGPUNeighbourhoods.from_sequence(list(input_data.data)).data
            ctx = self.context_for(offsets)
            self._sync_stream(ctx, offsets)
            ctx.set_neighbours(offsets, indices)
            self._graph_key = None
            return ctx
        data = input_data.data
        ctx = self.context_for(data)
        self._sync_stream(ctx, data)
        key = None
        if (self.reuse_graph and _abi.is_device_array(data) and hasattr(data, "_version")
                and _distance_layout(input_data, self._metric_code()) is None
                and self._metric_code() != _abi.METRIC_EUCLIDEAN_PERIODIC_REDUCED):
            key = (id(data), int(data.data_ptr()), tuple(data.shape), int(data._version),
                   float(cluster_params.radius_cutoff), self._metric_code(), self._fpmode_code())
        if (key is not None and self._graph_key is not None and self._graph_key[0] == key
                and self._graph_key[1] is ctx and self._graph_key[2] == ctx.graph_generation()):
            return ctx
        self._graph_key = None
        metric = load_input(ctx, input_data, self._neighbours_getter, self._metric_code())
        ctx.build_neighbours(cluster_params.radius_cutoff, metric, self._fpmode_code())
        if key is not None:
            self._graph_key = (key, ctx, ctx.graph_generation())
        return ctx

    @staticmethod
    def _sync_stream(ctx: _abi.Context, array):
        """Run on torch's current stream when the data lives in torch."""
        if _abi.is_device_array(array):
            st = _abi.current_torch_stream(ctx.device)
            if st is not None and st != ctx.stream:
                ctx.set_stream(st)

    def fit(self, input_data, labels, cluster_params):
        """Cluster ``input_data``; ``labels.labels``/``labels.consider`` in place."""
        ctx = self.prepare(input_data, cluster_params)
        ctx.fit(cluster_params.similarity_cutoff, cluster_params.n_member_cutoff,
                cluster_params.current_start, labels.consider, labels.labels)


class FitterGPUNeighbourhoods(FitterGPU):
    """The GPU fitter preset for precomputed neighbourhood input."""

    def __init__(self, neighbours_getter=None, *args, **kwargs):
        if neighbours_getter is None:
            neighbours_getter = NeighboursGetterGPULookup(is_sorted=False, is_selfcounting=True)
        super().__init__(neighbours_getter, *args, **kwargs)


class HierarchicalFitter(ABC):
    """Hierarchical fitter interface (src/cnnclustering/_fit.pyx:88-126).

    ``make_parameters`` reads ``self._neighbours_getter`` like the
    reference's; a hierarchical fitter without that attribute (the repeat
    fitter) passes (radius_cutoff, cnn_cutoff) through unchanged.
    """

    @abstractmethod
    def fit(self, bundle, **kwargs):
        """Generic hierarchical clustering"""

    make_parameters = Fitter.make_parameters


class HierarchicalFitterRepeatGPU(HierarchicalFitter):
    """Drop-in for ``HierarchicalFitterRepeat`` (src/cnnclustering/_fit.pyx:1014-1187).

    Every step (radius_cutoff[i], cnn_cutoff[i]) is a complete fit of all
    points of the bundle from fresh labels; the labels of step i become
    the labels of the step-(i-1) clusters' children, which are isolated
    into child bundles.  With a ``FitterGPU`` on coordinates all steps run
    as one batched device call (one largest-radius search per 16 radii,
    fits seeded along the (radius, cut) lattice, ``cnn_sweep_pairs``);
    any other fitter is called step by step.  The hierarchy bookkeeping
    (:1146-1184) is host work.

    As in the reference, the parameters come from this object's
    ``make_parameters``: it has no neighbours getter, so the radius is not
    adjusted by the metric and no self-counting offsets are added.
    """

    def __init__(self, fitter=None):
        self._fitter = fitter if fitter is not None else FitterGPU()

    def __str__(self):
        return f"{type(self).__name__}(fitter={self._fitter})"

    @classmethod
    def get_builder_kwargs(cls):
        return [("fitter", None)]

    def fit(self, bundle, **kwargs):
        self._fit(bundle, kwargs["radius_cutoff"], kwargs["cnn_cutoff"], kwargs.get("member_cutoff"),
                  kwargs.get("max_clusters"), kwargs.get("cnn_offset"), kwargs.get("sort_by_size", True),
                  kwargs.get("info", True), kwargs.get("v", True))

    def step_labels(self, bundle, params, member_cutoff, max_clusters, sort_by_size):
        """Labels of every step, shape [n_steps, n_points] (host)."""
        from ._types import Labels
        input_data = bundle._input_data
        fitter = self._fitter
        if isinstance(fitter, FitterGPU) and not _is_neighbourhood_input(input_data):
            data = input_data.data
            ctx = fitter.context_for(data)
            fitter._sync_stream(ctx, data)
            metric = load_input(ctx, input_data, fitter._neighbours_getter, fitter._metric_code())
            fitter._graph_key = None
            out = ctx.sweep_pairs([p.radius_cutoff for p in params],
                                  [(p.similarity_cutoff, p.n_member_cutoff) for p in params],
                                  member_cutoff=2 if member_cutoff is None else int(member_cutoff),
                                  max_clusters=max_clusters, sort=sort_by_size, metric=metric,
                                  fpmode=fitter._fpmode_code())
            return np.asarray(out)
        n = input_data.n_points
        rows = []
        for p in params:
            labels = Labels(np.zeros(n, order="C", dtype=np.int64))
            fitter.fit(input_data, labels, p)
            if sort_by_size:
                labels.sort_by_size(member_cutoff, max_clusters)
            rows.append(np.array(labels._host(), dtype=np.int64))
        return np.stack(rows) if rows else np.zeros((0, n), dtype=np.int64)

    def _fit(self, bundle, radius_cutoff, cnn_cutoff, member_cutoff=None, max_clusters=None, cnn_offset=None,
             sort_by_size=True, info=True, v=True):
        import weakref
        from collections.abc import Iterable
        from ._types import Labels

        if not isinstance(radius_cutoff, Iterable):
            radius_cutoff = [radius_cutoff]
        radius_cutoff = [float(x) for x in radius_cutoff]
        if not isinstance(cnn_cutoff, Iterable):
            cnn_cutoff = [cnn_cutoff]
        cnn_cutoff = [int(x) for x in cnn_cutoff]
        if len(radius_cutoff) == 1:
            radius_cutoff *= len(cnn_cutoff)
        if len(cnn_cutoff) == 1:
            cnn_cutoff *= len(radius_cutoff)
        n_steps = len(radius_cutoff)
        assert n_steps == len(cnn_cutoff)
        if cnn_offset is None:
            cnn_offset = 0
        params = [self.make_parameters(radius_cutoff[i], cnn_cutoff[i] - cnn_offset, 1) for i in range(n_steps)]
        if v:
            for i in range(n_steps):
                print(f"Running step {i:<5} (r = {radius_cutoff[i]}, c = {cnn_cutoff[i]})")
        all_labels = self.step_labels(bundle, params, member_cutoff, max_clusters, sort_by_size)

        n_points = bundle._input_data.n_points
        previous = np.ones(n_points, dtype=np.int64)
        terminal = {1: bundle}
        for step in range(n_steps):
            current = all_labels[step]
            new_terminal = {}
            # points of every parent cluster, in point order; parents in
            # ascending label order
            order = np.argsort(previous, kind="stable")
            sorted_prev = previous[order]
            values, starts = np.unique(sorted_prev, return_index=True)
            ends = np.append(starts[1:], sorted_prev.shape[0])
            for p_label, a, b in zip(values.tolist(), starts.tolist(), ends.tolist()):
                if p_label == 0:
                    continue
                parent_clustering = terminal[p_label]
                parent_clustering._labels = Labels.from_sequence(current[order[a:b]])
                if info:
                    label_params = {k: (radius_cutoff[step], cnn_cutoff[step])
                                    for k in parent_clustering._labels.to_set() if k != 0}
                    parent_clustering._labels.meta.update({"params": label_params,
                                                           "reference": weakref.proxy(parent_clustering),
                                                           "origin": "fit"})
                parent_clustering.isolate(isolate_input_data=False)
                for c_label, child in parent_clustering._children.items():
                    if c_label == 0:
                        continue
                    new_terminal[c_label] = child
            terminal = new_terminal
            previous = current


__all__ = ["Fitter", "FitterGPU", "FitterGPUNeighbourhoods", "HierarchicalFitter", "HierarchicalFitterRepeatGPU",
           "np"]
