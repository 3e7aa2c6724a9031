"""``Bundle``: one node of the clustering hierarchy.

Mirrors src/cnnclustering/_bundle.pyx:20-402 -- input data, labels, the
children created from those labels (``isolate``), the reference indices
that map a child's points back to its parent and to the root, and the
traversal helpers.  All of it is host bookkeeping; the fits that produce
the labels run on the GPU.
"""
from __future__ import annotations

import weakref
from collections import deque
from collections.abc import Iterable, MutableMapping, MutableSequence

import numpy as np

from ._types import InputData, Labels
from .report import Summary


class ReferenceIndices:
    """Point indices of a child in its root and in its parent
    (the reference keeps the same pair, src/cnnclustering/_types.pyx:289-302)."""

    def __init__(self, root_indices, parent_indices):
        self.root = np.asarray(root_indices, dtype=np.intp)
        self.parent = np.asarray(parent_indices, dtype=np.intp)


class Bundle:
    def __init__(self, input_data=None, graph=None, labels=None, reference_indices=None, children=None,
                 alias=None, parent=None, meta=None, summary=None, hierarchy_level=0):
        self.input_data = input_data
        self._graph = graph
        self.labels = labels
        self._reference_indices = reference_indices
        self.children = children
        self.alias = "root" if alias is None else str(alias)
        if parent is not None:
            self._parent = weakref.proxy(parent)
            self.hierarchy_level = parent.hierarchy_level + 1
        else:
            self._parent = None
            self.hierarchy_level = hierarchy_level
        self.meta = {} if meta is None else meta
        self.summary = summary
        self._lambda = -np.inf

    # -- properties (src/cnnclustering/_bundle.pyx:57-147) -----------------------
    @property
    def labels(self):
        return None if self._labels is None else self._labels.labels

    @labels.setter
    def labels(self, value):
        if value is not None and not isinstance(value, Labels):
            value = Labels(value) if hasattr(value, "shape") else Labels.from_sequence(value)
        self._labels = value

    @property
    def root_indices(self):
        return None if self._reference_indices is None else self._reference_indices.root

    @property
    def parent_indices(self):
        return None if self._reference_indices is None else self._reference_indices.parent

    @property
    def input_data(self):
        return None if self._input_data is None else self._input_data.data

    @input_data.setter
    def input_data(self, value):
        if value is not None and not isinstance(value, InputData):
            raise TypeError(f"Can't use object of type {type(value).__name__} as input data. "
                            f"Expected type {InputData.__name__}.")
        self._input_data = value

    @property
    def children(self):
        return self._children

    @children.setter
    def children(self, value):
        if value is None:
            value = {}
        if not isinstance(value, MutableMapping):
            raise TypeError("Expected a mutable mapping")
        self._children = value

    @property
    def hierarchy_level(self):
        return self._hierarchy_level

    @hierarchy_level.setter
    def hierarchy_level(self, value):
        self._hierarchy_level = int(value)

    @property
    def summary(self):
        return self._summary

    @summary.setter
    def summary(self, value):
        if value is None:
            value = Summary()
        if not isinstance(value, MutableSequence):
            raise TypeError("Expected a mutable sequence")
        self._summary = value

    def info(self):
        access = []
        if self._input_data is not None:
            meta = self._input_data.meta or {}
            for kind, check in (("coordinates", "access_coords"), ("distances", "access_distances"),
                                ("neighbours", "access_neighbours")):
                if meta.get(check, False):
                    access.append(kind)
        if not access:
            access = ["unknown"]
        n_points = self._input_data.n_points if self._input_data is not None else None
        return "\n".join([f"alias: {self.alias!r}", f"hierarchy_level: {self._hierarchy_level}",
                          f"access: {', '.join(access)}", f"points: {n_points}",
                          f"children: {len(self.children)}"])

    # -- children (src/cnnclustering/_bundle.pyx:148-272) ---------------------------
    @staticmethod
    def _as_path(label):
        if isinstance(label, str):
            label = label.split(".")
        if isinstance(label, Iterable):
            label = [int(x) for x in label]
            if len(label) == 1:
                label = label[0]
        return label

    def get_child(self, label):
        label = self._as_path(label)
        if isinstance(label, (int, np.integer)):
            try:
                return self._children[int(label)]
            except KeyError:
                raise KeyError(f"Clustering {self.alias!r} has no child with label {label}")
        next_label, *rest = label
        try:
            return self._children[next_label].get_child(rest)
        except KeyError:
            raise KeyError(f"Clustering {self.alias!r} has no child with label {next_label}")

    def add_child(self, label, bundle=None):
        if bundle is None:
            bundle = type(self)(parent=self)
        assert isinstance(bundle, Bundle)
        label = self._as_path(label)
        if isinstance(label, (int, np.integer)):
            self._children[int(label)] = bundle
            return
        *rest, last = label
        self.get_child(rest)._children[last] = bundle

    def __getitem__(self, key):
        return self.get_child(key)

    def __setitem__(self, key, value):
        self.add_child(key, value)

    def isolate(self, purge: bool = True, isolate_input_data: bool = True):
        """Create a child for each cluster label (src/cnnclustering/_bundle.pyx:275-352)."""
        isolate(self, purge, isolate_input_data)


def isolate(bundle: Bundle, purge: bool = True, isolate_input_data: bool = True):
    if purge or bundle._children is None:
        bundle._children = {}
    labels = np.asarray(bundle._labels._host())
    order = np.argsort(labels, kind="stable")  # indices of every label, ascending
    sorted_labels = labels[order]
    values, starts = np.unique(sorted_labels, return_index=True)
    ends = np.append(starts[1:], sorted_labels.shape[0])
    # the reference walks Labels.mapping, a dict filled in point order:
    # labels in order of their first occurrence
    first = [int(order[s]) for s in starts]
    for idx in np.argsort(first, kind="stable"):
        label = int(values[idx])
        if label == 0:
            continue
        parent_indices = np.asarray(order[starts[idx]:ends[idx]], dtype=np.intp)
        root = bundle._reference_indices
        root_indices = parent_indices if root is None else root.root[parent_indices]
        child = Bundle(parent=bundle)
        child._reference_indices = ReferenceIndices(root_indices, parent_indices)
        child.alias += f"{bundle.alias if bundle.alias is not None else ''} - {label}"
        bundle._children[label] = child
        if not isolate_input_data:
            continue
        child._input_data = bundle._input_data.get_subset(parent_indices)
        meta = bundle._input_data.meta or {}
        edges = meta.get("edges", None)
        if edges is None:
            continue
        child_edges = []
        child._input_data.meta["edges"] = child_edges
        if not edges:
            continue
        # points per part of the child (the parts of the parent, in order)
        bounds = np.cumsum(np.asarray(edges, dtype=np.int64))
        part_of = np.searchsorted(bounds, parent_indices, side="right")
        counts = np.bincount(part_of, minlength=len(edges))[:len(edges)]
        last = int(part_of[-1]) if parent_indices.shape[0] else 0
        child_edges.extend(int(c) for c in counts[:last + 1])
        while len(child_edges) < len(edges):
            child_edges.append(0)


def bfs_leafs(root: Bundle):
    """Every bundle of the hierarchy, breadth first (src/cnnclustering/_bundle.pyx:393-402)."""
    yield root
    q = deque([root])
    while q:
        bundle = q.popleft()
        for child in bundle._children.values():
            yield child
            q.append(child)


__all__ = ["Bundle", "ReferenceIndices", "isolate", "bfs_leafs"]
