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
from ._bundle import Bundle, bfs_leafs
from ._fit import Fitter, HierarchicalFitter
from ._types import InputData, Labels, P_AINDEX
from .report import Record, Summary


def timed(function):
    @functools.wraps(function)
    def wrapper(*args, **kwargs):
        go = time.time()
        out = function(*args, **kwargs)
        return out, time.time() - go
    return wrapper


class Clustering:
    def __init__(self, data=None, *, fitter=None, hierarchical_fitter=None, predictor=None, bundle_kwargs=None,
                 recipe=None, **recipe_kwargs):
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
        from ._predict import Predictor
        for kw, component_kw, kw_type in ((fitter, "fitter", Fitter),
                                          (hierarchical_fitter, "hierarchical_fitter", HierarchicalFitter),
                                          (predictor, "predictor", Predictor)):
            if isinstance(kw, kw_type):
                setattr(self, f"_{component_kw}", kw)
                continue
            if kw is not None:
                builder.recipe[component_kw] = kw
            made = builder.make_component(component_kw)
            setattr(self, f"_{component_kw}", None if made is object else made)

    @property
    def root(self):
        return self._bundle

    @property
    def children(self):
        return self._bundle._children

    def __getitem__(self, value):
        return self._bundle.get_child(value)

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

    @property
    def hierarchical_fitter(self):
        return self._hierarchical_fitter

    @property
    def predictor(self):
        return self._predictor

    def __str__(self):
        inp = None if self._bundle is None else self._bundle._input_data
        return (f"{type(self).__name__}(input_data={inp}, fitter={self._fitter}, "
                f"hfitter={self._hierarchical_fitter}, predictor={self._predictor})")

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

    # -- hierarchy (src/cnnclustering/cluster.pyx:394-552) ------------------------------
    def fit_hierarchical(self, purge=True, bundle=None, **fitter_kwargs):
        """Run the hierarchical fitter (e.g. ``HierarchicalFitterRepeatGPU``) on a bundle."""
        bundle = self._bundle if bundle is None else bundle
        if purge or bundle._children is None:
            bundle._children = {}
        self._hierarchical_fitter.fit(bundle, **fitter_kwargs)

    def isolate(self, purge: bool = True, isolate_input_data: bool = True, bundle=None):
        """One child bundle per cluster label."""
        bundle = self._bundle if bundle is None else bundle
        bundle.isolate(purge, isolate_input_data)

    def trim_shrinking_leafs(self, bundle=None):
        bundle = self._bundle if bundle is None else bundle

        def _trim_shrinking(b, new=True):
            if not b._children:
                splits = will_split = False
            else:
                label_set = b._labels.set
                label_set.discard(0)
                splits = len(label_set) > 1
                will_split = any([_trim_shrinking(child, new=splits) for child in b._children.values()])
            keep = new or will_split or splits
            if not keep:
                b._labels = None
                b._children = {}
            return keep

        _trim_shrinking(bundle)

    def trim_trivial_leafs(self, bundle=None):
        """Reset labels and children of every all-noise clustering."""
        bundle = self._bundle if bundle is None else bundle

        def _trim_trivial(b):
            if b._labels is None:
                return
            if b._labels.set == {0}:
                b._labels = None
                b._children = {}
                return
            for child in b._children.values():
                _trim_trivial(child)

        _trim_trivial(bundle)

    def reel(self, depth: Optional[int] = None, bundle=None) -> None:
        """Fold the labels of lower levels into their parents' labels."""
        bundle = self._bundle if bundle is None else bundle
        if depth is not None:
            assert depth > 0

        def _reel(parent, depth):
            if not parent._children:
                return
            if depth is not None:
                depth -= 1
            parent._labels.meta["origin"] = "reel"
            parent_labels = parent._labels.labels
            for label, child in parent._children.items():
                if child._labels is None:
                    continue
                if depth is None or depth > 0:
                    _reel(child, depth)
                n_clusters = int(max(parent_labels))
                child_labels = np.asarray(child._labels.labels)
                new = np.where(child_labels == 0, 0, child_labels + n_clusters)
                parent_labels[np.asarray(child.parent_indices)] = new
                parent._labels.meta.get("params", {}).pop(label, None)
                for old_label, p in child._labels.meta.get("params", {}).items():
                    parent._labels.meta.setdefault("params", {})[old_label + n_clusters] = p

        _reel(bundle, depth)

    def predict(self, other, radius_cutoff: float, cnn_cutoff: int, clusters=None, cnn_offset=None,
                info: bool = True, record: bool = True, record_time: bool = True, v: bool = True,
                purge: bool = False, bundle=None):
        """Labels for the points of ``other`` from this clustering (see ``PredictorFirstmatchGPU``)."""
        from ._predict import predict_into
        bundle = self._bundle if bundle is None else bundle
        return predict_into(self, bundle, other, radius_cutoff, cnn_cutoff, clusters, cnn_offset, info, record,
                            record_time, v, purge)


__all__ = ["Bundle", "Clustering", "bfs_leafs", "timed"]
