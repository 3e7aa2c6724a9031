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
from ._types import (ClusterParameters, InputDataGPUNeighbourhoods, NeighboursGetterGPUGrid,
                     NeighboursGetterGPULookup, SimilarityCheckerGPU, QueueGPUUnionFind, NeighboursGPU,
                     _device_of)


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
            (torch version counter) and the radius, metric and fpmode are
            unchanged.  Host (numpy) inputs are always re-uploaded.
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
        self._graph_key = None
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
        return getattr(self._neighbours_getter, "fpmode_code", _abi.FP_SEPARATE)

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
        if self.reuse_graph and _abi.is_device_array(data) and hasattr(data, "_version"):
            key = (id(data), int(data.data_ptr()), tuple(data.shape), int(data._version),
                   float(cluster_params.radius_cutoff), self._metric_code(), self._fpmode_code())
        if key is not None and key == self._graph_key:
            return ctx
        ctx.set_points(data)
        ctx.build_neighbours(cluster_params.radius_cutoff, self._metric_code(), self._fpmode_code())
        self._graph_key = key
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


__all__ = ["Fitter", "FitterGPU", "FitterGPUNeighbourhoods", "np"]
