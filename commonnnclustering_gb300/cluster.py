"""``Clustering``: the user-facing object, mirroring the reference's
fit orchestration (src/cnnclustering/cluster.pyx:102-392).

``fit(radius_cutoff, cnn_cutoff, member_cutoff, max_clusters, cnn_offset,
sort_by_size, info, record, record_time, v, purge)`` does what the
reference does around its fitter -- cnn_offset, fresh or frozen labels,
``make_parameters``, the timed fit, meta["params"], ``sort_by_size`` and a
``Record`` -- with the fit and the sort on the GPU.
"""
from __future__ import annotations

import functools
import time
import weakref
from collections import Counter
from typing import Optional

import numpy as np

from . import recipes
from ._fit import Fitter
from ._types import InputData, Labels, P_AINDEX
from .report import Record, Summary


class Bundle:
    """Input data, labels and fit records of one clustering
    (the subset of src/cnnclustering/_bundle.pyx:20-272 the fit uses)."""

    def __init__(self, input_data=None, labels=None, summary=None):
        self._input_data = input_data
        self._labels = labels
        self._summary = Summary() if summary is None else summary
        self._children = None

    @property
    def labels(self):
        return None if self._labels is None else self._labels.labels

    @labels.setter
    def labels(self, value):
        self._labels = value if isinstance(value, Labels) else Labels.from_sequence(value)


def timed(function):
    @functools.wraps(function)
    def wrapper(*args, **kwargs):
        go = time.time()
        out = function(*args, **kwargs)
        return out, time.time() - go
    return wrapper


class Clustering:
    def __init__(self, data=None, *, fitter=None, bundle_kwargs=None, recipe=None, **recipe_kwargs):
        builder = recipes.Builder(recipe, **recipe_kwargs)
        bundle_kwargs = {} if bundle_kwargs is None else bundle_kwargs
        if data is None:
            self._bundle = None
        elif isinstance(data, Bundle):
            self._bundle = data
        elif isinstance(data, InputData):
            self._bundle = Bundle(data, **bundle_kwargs)
        else:
            self._bundle = Bundle(builder.make_input_data(data), **bundle_kwargs)
        if isinstance(fitter, Fitter):
            self._fitter = fitter
        else:
            if fitter is not None:
                builder.recipe["fitter"] = fitter
            made = builder.make_component("fitter")
            self._fitter = None if made is object else made

    @property
    def labels(self):
        if self._bundle is None or self._bundle._labels is None:
            return None
        return self._bundle._labels.labels

    @labels.setter
    def labels(self, value):
        if self._bundle is None:
            raise ValueError("Can't set labels because there is no root bundle")
        self._bundle.labels = value

    @property
    def input_data(self):
        if self._bundle is None or self._bundle._input_data is None:
            return None
        return self._bundle._input_data.data

    @property
    def fitter(self):
        return self._fitter

    @fitter.setter
    def fitter(self, value):
        if value is not None and not isinstance(value, Fitter):
            raise TypeError(f"Can't use object of type {type(value).__name__} as fitter.")
        self._fitter = value

    @property
    def summary(self):
        return self._bundle._summary

    def __str__(self):
        inp = None if self._bundle is None else self._bundle._input_data
        return f"{type(self).__name__}(input_data={inp}, fitter={self._fitter})"

    def _fit(self, cluster_params, bundle=None):
        bundle = self._bundle if bundle is None else bundle
        self._fitter.fit(bundle._input_data, bundle._labels, cluster_params)

    def fit(self, radius_cutoff: float, cnn_cutoff: int, member_cutoff: Optional[int] = None,
            max_clusters: Optional[int] = None, cnn_offset: Optional[int] = None, sort_by_size: bool = True,
            info: bool = True, record: bool = True, record_time: bool = True, v: bool = True,
            purge: bool = False, bundle=None) -> None:
        bundle = self._bundle if bundle is None else bundle
        if cnn_offset is None:
            cnn_offset = 0
        cnn_cutoff -= cnn_offset
        assert cnn_cutoff >= 0
        n = bundle._input_data.n_points
        if bundle._labels is None or purge or not bundle._labels.meta.get("frozen", False):
            data = bundle._input_data.data
            from . import _abi
            if _abi.is_device_array(data):
                import torch
                lab = torch.zeros(n, dtype=torch.int64, device=data.device)
            else:
                lab = np.zeros(n, order="C", dtype=P_AINDEX)
            bundle._labels = Labels(lab)
            old_label_set = set()
            current_start = 1
        else:
            old_label_set = bundle._labels.to_set()
            current_start = max(old_label_set) + 1
        cluster_params = self._fitter.make_parameters(radius_cutoff, cnn_cutoff, current_start)
        if record_time:
            _, execution_time = timed(self._fitter.fit)(bundle._input_data, bundle._labels, cluster_params)
        else:
            self._fitter.fit(bundle._input_data, bundle._labels, cluster_params)
            execution_time = None
        if info:
            new_label_set = bundle._labels.to_set()
            params = {k: (radius_cutoff, cnn_cutoff) for k in new_label_set - old_label_set if k != 0}
            old_params = bundle._labels.meta.get("params", {})
            old_params.update(params)
            bundle._labels.meta.update({"params": old_params, "reference": weakref.proxy(bundle),
                                        "origin": "fit"})
        if sort_by_size:
            bundle._labels.sort_by_size(member_cutoff, max_clusters)
        if record:
            host = bundle._labels._host()
            freq = Counter(host.tolist())
            n_noise = freq.pop(0, 0)
            n_largest = freq.most_common(1)[0][1] if freq else 0
            rec = Record(n, radius_cutoff, cnn_cutoff, member_cutoff, max_clusters, len(set(freq)),
                         n_largest / n if n else 0.0, n_noise / n if n else 0.0, execution_time)
            if v:
                print(rec)
            bundle._summary.append(rec)
