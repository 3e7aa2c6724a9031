"""Cluster label prediction for other points.

``Predictor`` mirrors the reference's interface (src/cnnclustering/_fit.pyx:
164-213) and ``PredictorFirstmatchGPU`` is the drop-in for
``PredictorFirstmatch`` (:1194-1291): every other point takes the label of
the first of its neighbours among the clustered points (index order) whose
label is in the consider set, which has enough neighbours itself and which
shares enough neighbours with it.  ``Clustering.predict`` (cluster.pyx:
558-655) orchestrates it; the prediction itself is one ``cnn_predict``
call (cross-set radius search, this set's graph, first-match kernel).
"""
from __future__ import annotations

import time
import weakref
from abc import ABC, abstractmethod

import numpy as np

from . import _abi
from ._fit import Fitter
from ._types import (Labels, NeighboursGetterGPUGrid, NeighboursGPU, P_AINDEX, SimilarityCheckerGPU,
                     _device_of)


class Predictor(ABC):
    """Predictor interface (src/cnnclustering/_fit.pyx:164-213)."""

    @abstractmethod
    def predict(self, input_data, predictand_input_data, labels, predictand_labels, cluster_params):
        """Generic cluster label prediction"""

    make_parameters = Fitter.make_parameters


class PredictorFirstmatchGPU(Predictor):
    """First-match label prediction on the GPU.

    Constructor arguments mirror ``PredictorFirstmatch``; the getter's metric,
    self-counting flag and fpmode set the comparison, the other components
    only name the reference's containers.
    """

    def __init__(self, neighbours_getter=None, neighbours_getter_other=None, neighbours=None,
                 neighbour_neighbours=None, similarity_checker=None, *, device=None, context=None):
        self._neighbours_getter = neighbours_getter if neighbours_getter is not None else NeighboursGetterGPUGrid()
        self._neighbours_getter_other = (neighbours_getter_other if neighbours_getter_other is not None
                                         else self._neighbours_getter)
        self._neighbours = neighbours if neighbours is not None else NeighboursGPU()
        self._neighbour_neighbours = neighbour_neighbours if neighbour_neighbours is not None else NeighboursGPU()
        self._similarity_checker = similarity_checker if similarity_checker is not None else SimilarityCheckerGPU()
        self._device = device
        self._context = context

    def __str__(self):
        attr_str = ", ".join([f"ngetter={self._neighbours_getter}", f"ngetter_other={self._neighbours_getter_other}",
                              f"na={self._neighbours}", f"nb={self._neighbour_neighbours}",
                              f"checker={self._similarity_checker}"])
        return f"{type(self).__name__}({attr_str})"

    @classmethod
    def get_builder_kwargs(cls):
        return [("neighbours_getter", None), ("neighbours_getter_other", "neighbours_getter"),
                ("neighbours", None), ("neighbour_neighbours", "neighbours"), ("similarity_checker", None)]

    def _metric_code(self) -> int:
        try:
            return int(self._neighbours_getter._distance_getter._metric.code)
        except AttributeError:
            return _abi.METRIC_EUCLIDEAN_REDUCED

    def predict(self, input_data, predictand_input_data, labels, predictand_labels, cluster_params):
        """Labels of ``predictand_input_data`` in place (labels and consider)."""
        data = input_data.data
        other = predictand_input_data.data
        if self._context is None:
            dev = self._device if self._device is not None else _device_of(data)
            self._context = _abi.Context(dev)
        ctx = self._context
        if _abi.is_device_array(data):
            st = _abi.current_torch_stream(ctx.device)
            if st is not None and st != ctx.stream:
                ctx.set_stream(st)
        metric = self._metric_code()
        ctx.set_points(data)
        if metric == _abi.METRIC_EUCLIDEAN_PERIODIC_REDUCED:
            ctx.set_periodic_bounds(self._neighbours_getter._distance_getter._metric.bounds)
        ctx.predict(other, labels.labels, predictand_labels.consider_set, cluster_params.radius_cutoff,
                    cluster_params.similarity_cutoff, cluster_params.n_member_cutoff, predictand_labels.labels,
                    predictand_labels.consider, metric=metric,
                    fpmode=getattr(self._neighbours_getter, "fpmode_code", _abi.host_fpmode()))


def predict_into(clustering, bundle, other, radius_cutoff, cnn_cutoff, clusters=None, cnn_offset=None, info=True,
                 record=True, record_time=True, v=True, purge=False):
    """``Clustering.predict`` (src/cnnclustering/cluster.pyx:558-655): ``other``
    is a Bundle (or a Clustering) whose labels are predicted in place."""
    if hasattr(other, "_bundle"):
        other = other._bundle
    if cnn_offset is None:
        cnn_offset = 0
    cnn_cutoff -= cnn_offset
    assert cnn_cutoff >= 0
    if other._labels is None or purge or not other._labels.meta.get("frozen", False):
        other._labels = Labels(np.zeros(other._input_data.n_points, order="C", dtype=P_AINDEX))
    predictor = clustering._predictor
    cluster_params = predictor.make_parameters(radius_cutoff, cnn_cutoff, 0)
    if clusters is None:
        clusters = bundle._labels.to_set() - {0}
    other._labels.consider_set = clusters
    go = time.time()
    predictor.predict(bundle._input_data, other._input_data, bundle._labels, other._labels, cluster_params)
    execution_time = time.time() - go if record_time else None
    if info:
        params = {k: (radius_cutoff, cnn_cutoff) for k in clusters if k != 0}
        old_params = other._labels.meta.get("params", {})
        old_params.update(params)
        other._labels.meta.update({"params": old_params, "reference": weakref.proxy(bundle), "origin": "predict"})
    other._labels.meta["frozen"] = True
    return execution_time


__all__ = ["Predictor", "PredictorFirstmatchGPU", "predict_into"]
