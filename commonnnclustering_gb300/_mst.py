"""``HierarchicalFitterMSTPrimGPU``: the cluster hierarchy of a maximum
spanning forest of the common-neighbour graph.

Mirrors ``HierarchicalFitterMSTPrim`` (src/cnnclustering/_fit.pyx:733-1011):

* every neighbour pair (a, b) is weighted by the full common-neighbour count
  |N(a) & N(b)| (SimilarityCheckerExtScreensorted._get, _types.pyx:
  2708-2753) -- computed for all pairs at once on the GPU;
* Prim's algorithm grows a maximum spanning forest from every unvisited
  point in index order with a max-heap keyed (-weight, (a, b)) -- run by
  the library's host code on those weights, so that ties resolve as in the
  reference (``cnn_mst_prim``);
* the tree edges, strongest first, merge single-linkage style into bundles
  whose ``_lambda`` is the merge weight; merges at one weight are folded
  together and children smaller than ``member_cutoff`` are dropped
  (``check_children``, _bundle.pyx:355-390) -- host bookkeeping here.

Bundles carry a light weighted graph (``WeightedGraph``) with the part of
networkx's Graph interface the hierarchy uses (``len``, ``nodes``,
``edges(data=True)``, ``add_edges_from``).
"""
from __future__ import annotations

import weakref
from collections import deque
from typing import Iterable, Optional

import numpy as np

from . import _abi
from ._bundle import Bundle
from ._fit import HierarchicalFitter
from ._types import (Labels, NeighboursGetterGPUGrid, NeighboursGPU, P_AINDEX, SimilarityCheckerGPU, _device_of)


class WeightedGraph:
    """Undirected weighted edges and their nodes."""

    def __init__(self, edges: Optional[Iterable] = None):
        self._adj_nodes: dict = {}
        self._edges: dict = {}
        if edges is not None:
            for e in edges:
                u, v = int(e[0]), int(e[1])
                w = e[2]["weight"] if isinstance(e[2], dict) else e[2]
                self.add_edge(u, v, w)

    def add_edge(self, u: int, v: int, weight):
        self._adj_nodes.setdefault(u, None)
        self._adj_nodes.setdefault(v, None)
        self._edges[(u, v) if u <= v else (v, u)] = weight

    def add_edges_from(self, edges):
        for u, v, data in edges:
            self.add_edge(int(u), int(v), data["weight"] if isinstance(data, dict) else data)

    def edges(self, data: bool = False):
        if data:
            return [(u, v, {"weight": w}) for (u, v), w in self._edges.items()]
        return list(self._edges)

    @property
    def nodes(self):
        return list(self._adj_nodes)

    def __len__(self):
        return len(self._adj_nodes)

    def __iter__(self):
        return iter(self._adj_nodes)


def check_children(bundle: Bundle, member_cutoff: int, needs_folding: bool = False):
    """src/cnnclustering/_bundle.pyx:355-390: fold children that merged at the
    bundle's own weight, drop children with fewer than member_cutoff points,
    and replace a single child by its children."""
    if needs_folding:
        leafs = []
        queue = deque()
        for child in bundle._children.values():
            (queue if child._lambda == bundle._lambda else leafs).append(child)
        while queue:
            candidate = queue.popleft()
            for child in candidate._children.values():
                (queue if child._lambda == bundle._lambda else leafs).append(child)
        bundle._children = {count: child for count, child in enumerate(leafs, 1)}
    # numbered before filtering, as the reference does
    bundle._children = {k: v for k, v in enumerate(bundle._children.values(), 1) if len(v._graph) >= member_cutoff}
    if len(bundle._children) == 1:
        child = bundle._children.popitem()[1]
        for label, grandchild in enumerate(child._children.values(), 1):
            bundle._children[label] = grandchild
            bundle._lambda = child._lambda
    for child in bundle._children.values():
        child._parent = weakref.proxy(bundle)


def build_mst_hierarchy(bundle: Bundle, edges, n_points: int, member_cutoff: int):
    """The bundle tree from the tree edges in pop order (_fit.pyx:901-1011)."""
    parent = np.arange(n_points, dtype=np.int64)
    root_label = np.arange(n_points, dtype=np.int64)

    def get_root(p):
        # the root only (link order as the reference's parent indicator);
        # path compression leaves every root unchanged
        r = p
        while parent[r] != r:
            r = parent[r]
        while parent[p] != r:
            parent[p], p = r, parent[p]
        return r

    top_bundles: dict = {}
    checked = np.zeros(max(n_points - 1, 0), dtype=bool)
    current_weight = np.inf
    needs_folding = False
    i = -1
    for i, (a, b, weight) in enumerate(edges):
        a, b = int(a), int(b)
        ra, rb = get_root(a), get_root(b)
        la, lb = int(root_label[ra]), int(root_label[rb])
        if weight < current_weight:
            for index, top in top_bundles.items():
                if checked[index]:
                    continue
                check_children(top, member_cutoff, needs_folding)
                checked[index] = True
            needs_folding = False
        else:
            needs_folding = True
        top = top_bundles[i] = Bundle(graph=WeightedGraph([(a, b, {"weight": weight})]))
        top._lambda = weight
        label = 1
        if la >= n_points:
            left = top_bundles.pop(la - n_points)
            top._graph.add_edges_from(left._graph.edges(data=True))
            top._children[label] = left
            label += 1
        if lb >= n_points:
            right = top_bundles.pop(lb - n_points)
            top._graph.add_edges_from(right._graph.edges(data=True))
            top._children[label] = right
        parent[ra] = rb
        root_label[rb] = i + n_points
        current_weight = weight
    for index, top in top_bundles.items():
        if checked[index]:
            continue
        check_children(top, member_cutoff, needs_folding)
    if i < n_points - 2:
        bundle._lambda = -np.inf
        bundle._graph = WeightedGraph()
        count = 1
        for top in top_bundles.values():
            if len(top._graph) >= member_cutoff:
                bundle._children[count] = top
                count += 1
        for child in bundle._children.values():
            child._parent = weakref.proxy(bundle)
    else:
        top = top_bundles[n_points - 2]
        bundle._graph = top._graph
        bundle._lambda = top._lambda


class PriorityQueueMaxHeapGPU:
    """Names the reference's max-heap component (PriorityQueueMaxHeap,
    src/cnnclustering/_types.pyx:2825-2851); the heap itself runs inside
    cnn_mst_prim with the same (-weight, (a, b)) order."""

    def __str__(self):
        return f"{type(self).__name__}"


class HierarchicalFitterMSTPrimGPU(HierarchicalFitter):
    """Drop-in for ``HierarchicalFitterMSTPrim`` (constructor arguments mirror
    it; the getter's metric and fpmode set the neighbourhoods)."""

    def __init__(self, neighbours_getter=None, neighbours=None, neighbour_neighbours=None, similarity_checker=None,
                 priority_queue=None, priority_queue_tree=None, *, device=None, context=None):
        self._neighbours_getter = neighbours_getter if neighbours_getter is not None else NeighboursGetterGPUGrid()
        self._neighbours = neighbours if neighbours is not None else NeighboursGPU()
        self._neighbour_neighbours = neighbour_neighbours if neighbour_neighbours is not None else NeighboursGPU()
        self._similarity_checker = similarity_checker if similarity_checker is not None else SimilarityCheckerGPU()
        self._priority_queue = priority_queue
        self._priority_queue_tree = priority_queue_tree
        self._device = device
        self._context = context

    def __str__(self):
        attr_str = ", ".join([f"ngetter={self._neighbours_getter}", f"na={self._neighbours}",
                              f"nb={self._neighbour_neighbours}", f"checker={self._similarity_checker}",
                              f"prioq={self._priority_queue}", f"prioq (tree)={self._priority_queue_tree}"])
        return f"{type(self).__name__}({attr_str})"

    @classmethod
    def get_builder_kwargs(cls):
        return [("neighbours_getter", None), ("neighbours", None), ("neighbour_neighbours", "neighbours"),
                ("similarity_checker", None), ("priority_queue", None), ("priority_queue_tree", "priority_queue")]

    def _metric_code(self) -> int:
        try:
            return int(self._neighbours_getter._distance_getter._metric.code)
        except AttributeError:
            return _abi.METRIC_EUCLIDEAN_REDUCED

    def tree_edges(self, input_data, radius_cutoff: float):
        """(a, b, weight) of the maximum spanning forest in the tree queue's pop order."""
        from ._fit import load_input
        data = input_data.data
        if self._context is None:
            dev = self._device if self._device is not None else _device_of(data)
            self._context = _abi.Context(dev)
        ctx = self._context
        metric = load_input(ctx, input_data, self._neighbours_getter, self._metric_code())
        a, b, w = ctx.mst_prim(radius_cutoff, metric=metric,
                               fpmode=getattr(self._neighbours_getter, "fpmode_code", _abi.host_fpmode()))
        return list(zip(a.tolist(), b.tolist(), w.tolist()))

    def fit(self, bundle, **kwargs):
        self._fit(bundle, kwargs["radius_cutoff"], kwargs.get("member_cutoff"), kwargs.get("max_clusters"),
                  kwargs.get("cnn_offset"), kwargs.get("sort_by_size", True), kwargs.get("info", True),
                  kwargs.get("v", True))

    def _fit(self, bundle, radius_cutoff: float, member_cutoff: Optional[int] = None, max_clusters=None,
             cnn_offset=None, sort_by_size: bool = True, info: bool = True, v: bool = True):
        from ._fit import Fitter
        n_points = bundle._input_data.n_points
        labels = Labels(np.ones(n_points, order="C", dtype=P_AINDEX))
        bundle._labels = labels
        cluster_params = Fitter.make_parameters(self, radius_cutoff, 0, 1)
        if member_cutoff is None:
            member_cutoff = 10
        edges = self.tree_edges(bundle._input_data, cluster_params.radius_cutoff)
        labels.consider[:] = 0  # Prim visits every point
        build_mst_hierarchy(bundle, edges, n_points, member_cutoff)


__all__ = ["HierarchicalFitterMSTPrimGPU", "PriorityQueueMaxHeapGPU", "WeightedGraph", "build_mst_hierarchy",
           "check_children"]
