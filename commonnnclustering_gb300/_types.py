"""Component types mirroring cnnclustering's plugin API, backed by the GPU.

The reference composes a fitter from InputData / NeighboursGetter /
DistanceGetter / Metric / Neighbours / SimilarityChecker / Queue objects
with per-point C methods (src/cnnclustering/_types.pxd:119-565).  A
per-point GPU call would be useless, so here the whole fit is one call
(see ``_fit.FitterGPU``); the component objects keep the reference's
attributes and methods so that ``Fitter.make_parameters``, recipes and
per-point inspection behave the same:

* ``ClusterParameters``       -- src/cnnclustering/_types.pyx:22-85
* ``Labels``                  -- src/cnnclustering/_types.pyx:88-286
* ``InputDataGPUComponents``  -- InputDataExtComponentsMemoryview,
                                 src/cnnclustering/_types.pyx:1034-1109
* ``InputDataGPUNeighbourhoods`` -- InputDataExtNeighbourhoodsMemoryview,
                                 src/cnnclustering/_types.pyx:1153-1217
* ``NeighboursGetterGPUGrid`` -- NeighboursGetterExtBruteForce,
                                 src/cnnclustering/_types.pyx:1658-1735
* ``NeighboursGetterGPULookup`` -- NeighboursGetterExtLookup,
                                 src/cnnclustering/_types.pyx:1791-1832
* ``DistanceGetterGPUMetric`` -- DistanceGetterExtMetric, :1966-2017
* ``MetricGPUEuclideanReduced`` / ``MetricGPUEuclidean``
                              -- MetricExtEuclideanReduced :2250-2287,
                                 MetricExtEuclidean :2170-2207
* ``NeighboursGPU``           -- NeighboursExtVector, :1377-1424
* ``SimilarityCheckerGPU``    -- SimilarityCheckerExtScreensorted, :2637-2753
* ``QueueGPUUnionFind``       -- stands where QueueExtFIFOQueue
                                 (:2802-2819) stood; the GPU fitter grows
                                 clusters with union-find, not a queue.
"""
from __future__ import annotations

from abc import ABC, abstractmethod
from collections import defaultdict
from typing import Optional

import numpy as np

from . import _abi

P_AINDEX = np.intp
P_AVALUE = np.float64
P_ABOOL = np.uint8


class ClusterParameters:
    """Input parameters of one fit (same fields as the reference)."""

    __slots__ = ("radius_cutoff", "similarity_cutoff", "similarity_cutoff_continuous",
                 "n_member_cutoff", "current_start")

    def __init__(self, radius_cutoff: float, similarity_cutoff: int = 0,
                 similarity_cutoff_continuous: float = 0.0, n_member_cutoff: Optional[int] = None,
                 current_start: int = 1):
        if n_member_cutoff is None:
            n_member_cutoff = similarity_cutoff
        self.radius_cutoff = float(radius_cutoff)
        self.similarity_cutoff = int(similarity_cutoff)
        self.similarity_cutoff_continuous = float(similarity_cutoff_continuous)
        self.n_member_cutoff = int(n_member_cutoff)
        self.current_start = int(current_start)

    def to_dict(self):
        return {k: getattr(self, k) for k in self.__slots__}

    def __repr__(self):
        return f"{self.to_dict()!r}"

    __str__ = __repr__


class Labels:
    """Cluster label assignments (int64) with the uint8 ``consider`` mask.

    ``labels``/``consider`` may be numpy arrays or CUDA tensors; the GPU
    fitter reads and writes them in place either way.
    """

    def __init__(self, labels, *, consider=None, meta=None):
        self._labels = labels
        if consider is None:
            if _abi.is_device_array(labels):
                import torch
                consider = torch.ones(labels.shape[0], dtype=torch.uint8, device=labels.device)
            else:
                consider = np.ones(np.asarray(labels).shape[0], dtype=P_ABOOL)
        elif len(consider) != len(labels):
            raise ValueError("'labels' and 'consider' must have the same length")
        self._consider = consider
        self.meta = {} if meta is None else meta
        self._consider_set = set()

    @classmethod
    def from_sequence(cls, labels, *, consider=None, meta=None):
        labels = np.array(labels, order="C", dtype=P_AINDEX)
        if consider is not None:
            consider = np.array(consider, order="C", dtype=P_ABOOL)
        return cls(labels, consider=consider, meta=meta)

    @classmethod
    def from_length(cls, n: int, meta=None):
        return cls(np.zeros(n, order="C", dtype=P_AINDEX), meta=meta)

    @property
    def labels(self):
        return self._labels

    @property
    def consider(self):
        return self._consider

    @property
    def n_points(self):
        return int(self._labels.shape[0])

    @property
    def consider_set(self):
        return self._consider_set

    @consider_set.setter
    def consider_set(self, value):
        self._consider_set = value

    def _host(self):
        if _abi.is_device_array(self._labels):
            return self._labels.cpu().numpy()
        return np.asarray(self._labels)

    @property
    def mapping(self):
        return self.to_mapping()

    @property
    def set(self):
        return self.to_set()

    def to_mapping(self):
        mapping = defaultdict(list)
        for index, label in enumerate(self._host().tolist()):
            mapping[label].append(index)
        return mapping

    def to_set(self):
        return set(np.unique(self._host()).tolist())

    def __repr__(self):
        return f"{type(self).__name__}({list(self._host())!s})"

    def __str__(self):
        return f"{self._host()!s}"

    def sort_by_size(self, member_cutoff: Optional[int] = None, max_clusters: Optional[int] = None,
                     bundle=None, context: Optional[_abi.Context] = None):
        """Renumber clusters by size on the GPU (Labels.sort_by_size)."""
        if member_cutoff is None:
            member_cutoff = 2
        if self.n_points == 0:
            return
        before = self._host().copy() if (self.meta.get("params") or bundle is not None) else None
        ctx = context if context is not None else _abi.default_context(_device_of(self._labels))
        ctx.sort_by_size(self._labels, member_cutoff, max_clusters)
        if before is not None:
            reassign = _reassign_map(before, self._host())
            params = self.meta.get("params", {})
            self.meta["params"] = {reassign[k]: v for k, v in params.items()
                                   if k in reassign and reassign[k] != 0}
            if bundle is not None and getattr(bundle, "_children", None) is not None:
                bundle._children = {reassign[k]: c for k, c in bundle._children.items()
                                    if reassign.get(k, 0) != 0}


def _reassign_map(before: np.ndarray, after: np.ndarray) -> dict:
    uniq, idx = np.unique(before, return_index=True)
    return {int(u): int(after[i]) for u, i in zip(uniq, idx)}


def _device_of(a) -> int:
    if _abi.is_device_array(a):
        dev = getattr(a, "device", None)
        idx = getattr(dev, "index", None)
        return int(idx) if idx is not None else 0
    return 0


# ---------------------------------------------------------------------------
# Input data
# ---------------------------------------------------------------------------
class InputData(ABC):
    """Input data interface (src/cnnclustering/_types.pyx:305-389)."""

    @property
    @abstractmethod
    def n_points(self) -> int:
        ...

    @property
    def meta(self):
        return self._meta


class InputDataGPUComponents(InputData):
    """Point coordinates [n_points, n_dim] (float64, or float32 widened
    exactly to float64), as a numpy array or a CUDA tensor."""

    def __init__(self, data, *, meta=None):
        if not _abi.is_device_array(data):
            data = np.asarray(data)
            if data.ndim == 1:
                data = data.reshape(-1, 1)
            if data.dtype != np.float32:
                data = np.ascontiguousarray(data, dtype=P_AVALUE)
        self._data = data
        self._meta = {} if meta is None else meta
        self._meta.setdefault("access_coords", True)

    @property
    def data(self):
        return self._data

    @property
    def n_points(self) -> int:
        return int(self._data.shape[0])

    @property
    def n_dim(self) -> int:
        return int(self._data.shape[1])

    def get_component(self, point: int, dimension: int) -> float:
        return float(self._data[point, dimension])

    def get_subset(self, indices) -> "InputDataGPUComponents":
        """The rows `indices` (src/cnnclustering/_types.pyx:1064-1086, coordinates)."""
        idx = np.asarray(indices, dtype=np.int64)
        if _abi.is_device_array(self._data):
            import torch
            return type(self)(self._data[torch.as_tensor(idx, device=self._data.device)].contiguous())
        return type(self)(np.ascontiguousarray(self._data[idx]))

    def __str__(self):
        return f"{type(self).__name__}"


class InputDataGPUDistances(InputData):
    """Precomputed distances as a square [n_points, n_points] float64 matrix
    (the "distances" recipe's input, src/cnnclustering/recipes.py:329-339)."""

    def __init__(self, data, *, meta=None):
        if not _abi.is_device_array(data):
            data = np.ascontiguousarray(data, dtype=P_AVALUE)
        if len(data.shape) != 2 or data.shape[0] != data.shape[1]:
            raise ValueError("distances must be a square [n_points, n_points] matrix")
        self._data = data
        self._meta = {"access_distances": True}
        if meta:
            self._meta.update(meta)

    @property
    def data(self):
        return self._data

    @property
    def n_points(self) -> int:
        return int(self._data.shape[0])

    def get_distance(self, a: int, b: int) -> float:
        return float(self._data[a, b])

    def get_subset(self, indices) -> "InputDataGPUDistances":
        idx = np.asarray(indices, dtype=np.int64)
        if _abi.is_device_array(self._data):
            import torch
            t = torch.as_tensor(idx, device=self._data.device)
            return type(self)(self._data[t][:, t].contiguous())
        return type(self)(np.ascontiguousarray(self._data[np.ix_(idx, idx)]))


class InputDataGPUDistancesLinear(InputData):
    """Precomputed distances as the upper triangle by rows, n(n-1)/2 values
    (InputDataExtDistancesLinearMemoryview, src/cnnclustering/_types.pyx:1112-1150)."""

    def __init__(self, data, *, n_points=None, meta=None):
        if not _abi.is_device_array(data):
            data = np.ascontiguousarray(data, dtype=P_AVALUE).reshape(-1)
        self._data = data
        size = int(data.shape[0])
        self._n_points = int(n_points) if n_points is not None else int(0.5 * (np.sqrt(8 * size + 1) + 1))
        self._meta = {"access_distances": True}
        if meta:
            self._meta.update(meta)

    @property
    def data(self):
        return self._data

    @property
    def n_points(self) -> int:
        return self._n_points

    def get_distance(self, a: int, b: int) -> float:
        if a == b:
            return 0.0
        a, b = min(a, b), max(a, b)
        return float(self._data[a * (self._n_points - 1) - (a * a - a) // 2 + b - a - 1])


class InputDataGPUNeighbourhoods(InputData):
    """Precomputed neighbourhoods as CSR (offsets int64[n+1], indices int32)."""

    def __init__(self, offsets, indices, *, meta=None):
        self._offsets = offsets
        self._indices = indices
        self._meta = {} if meta is None else meta

    @classmethod
    def from_sequence(cls, neighbourhoods, meta=None):
        lens = np.array([len(s) for s in neighbourhoods], dtype=np.int64)
        offsets = np.zeros(lens.shape[0] + 1, dtype=np.int64)
        np.cumsum(lens, out=offsets[1:])
        indices = (np.concatenate([np.asarray(s, dtype=np.int32) for s in neighbourhoods])
                   if len(neighbourhoods) else np.zeros(0, dtype=np.int32))
        return cls(offsets, indices.astype(np.int32), meta=meta)

    @property
    def data(self):
        return self._offsets, self._indices

    @property
    def n_points(self) -> int:
        return int(self._offsets.shape[0]) - 1

    def get_n_neighbours(self, point: int) -> int:
        return int(self._offsets[point + 1] - self._offsets[point])

    def get_neighbour(self, point: int, member: int) -> int:
        return int(self._indices[self._offsets[point] + member])

    def get_subset(self, indices) -> "InputDataGPUNeighbourhoods":
        """Rows `indices`, each keeping only members in `indices`, member
        values unchanged (src/cnnclustering/_types.pyx:1199-1217)."""
        idx = np.asarray(indices, dtype=np.int64)
        off, ind = (np.asarray(a) for a in (self._offsets, self._indices))
        keep = np.zeros(max(self.n_points, int(ind.max()) + 1 if ind.size else 0), dtype=bool)
        keep[idx] = True
        rows = [ind[off[i]:off[i + 1]] for i in idx]
        return type(self).from_sequence([r[keep[r]] for r in rows], meta=dict(self._meta))


# ---------------------------------------------------------------------------
# Metric / distance getter / neighbours getter
# ---------------------------------------------------------------------------
class MetricGPUEuclideanReduced:
    """Squared Euclidean distance; the radius is compared squared."""

    code = _abi.METRIC_EUCLIDEAN_REDUCED

    def adjust_radius(self, radius_cutoff: float) -> float:
        return radius_cutoff ** 2

    def __str__(self):
        return f"{type(self).__name__}"


class MetricGPUEuclidean:
    """Euclidean distance (square root of the same sum)."""

    code = _abi.METRIC_EUCLIDEAN

    def adjust_radius(self, radius_cutoff: float) -> float:
        return radius_cutoff

    def __str__(self):
        return f"{type(self).__name__}"


class MetricGPUPrecomputed:
    """Distances given as input (MetricExtPrecomputed, src/cnnclustering/_types.pyx:
    2108-2127): the stored value is compared with the radius as given."""

    code = _abi.METRIC_PRECOMPUTED

    def adjust_radius(self, radius_cutoff: float) -> float:
        return radius_cutoff

    def __str__(self):
        return f"{type(self).__name__}"


class MetricGPUEuclideanPeriodicReduced:
    """Squared Euclidean distance with minimum images in a periodic box
    (MetricExtEuclideanPeriodicReduced, src/cnnclustering/_types.pyx:2290-2348);
    ``bounds`` per dimension, 0 = not periodic."""

    code = _abi.METRIC_EUCLIDEAN_PERIODIC_REDUCED

    def __init__(self, bounds):
        self._bounds = np.ascontiguousarray(bounds, dtype=P_AVALUE).reshape(-1)

    @property
    def bounds(self):
        return self._bounds

    def adjust_radius(self, radius_cutoff: float) -> float:
        return radius_cutoff ** 2

    def __str__(self):
        return f"{type(self).__name__}(bounds={self._bounds.tolist()})"


class DistanceGetterGPULookup:
    """Distances read from the input (DistanceGetterExtLookup,
    src/cnnclustering/_types.pyx:2019-2037), e.g. InputDataGPUDistancesLinear."""

    _metric = MetricGPUPrecomputed()

    @classmethod
    def get_builder_kwargs(cls):
        return []

    def __str__(self):
        return f"{type(self).__name__}"


class DistanceGetterGPUMetric:
    def __init__(self, metric=None):
        self._metric = metric if metric is not None else MetricGPUEuclideanReduced()

    @classmethod
    def get_builder_kwargs(cls):
        return [("metric", None)]

    def __str__(self):
        return f"{type(self).__name__}(metric={self._metric})"


class NeighboursGetterGPUGrid:
    """Radius neighbourhoods of all points on the GPU, self included, each
    list ascending (cell grid for n_dim <= 3, tiled all-pairs otherwise).

    ``fpmode`` selects how the float64 sum of squares is accumulated:
    ``"separate"`` (multiply, then add: the reference as GCC builds it on
    x86-64), ``"fused"`` (one fused multiply-add per term: the reference as
    GCC builds it on aarch64, e.g. a GB300's Grace host) or ``"auto"`` (the
    default): the mode of the reference built on this host
    (``_abi.host_fpmode``, ``CNN_FPMODE`` overrides it).
    """

    def __init__(self, distance_getter=None, fpmode: str = "auto"):
        self.is_sorted = True
        self.is_selfcounting = True
        self._distance_getter = distance_getter if distance_getter is not None else DistanceGetterGPUMetric()
        if fpmode not in ("separate", "fused", "auto"):
            raise ValueError("fpmode must be 'separate', 'fused' or 'auto'")
        if fpmode == "auto":
            fpmode = "fused" if _abi.host_fpmode() == _abi.FP_FUSED else "separate"
        self.fpmode = fpmode

    @classmethod
    def get_builder_kwargs(cls):
        return [("distance_getter", None)]

    @property
    def fpmode_code(self) -> int:
        return _abi.FP_FUSED if self.fpmode == "fused" else _abi.FP_SEPARATE

    def __str__(self):
        return (f"{type(self).__name__}(dgetter={self._distance_getter}, sorted={self.is_sorted}, "
                f"selfcounting={self.is_selfcounting})")


class NeighboursGetterGPULookup:
    """Neighbourhoods taken from precomputed lists (InputDataGPUNeighbourhoods)."""

    def __init__(self, is_sorted: bool = False, is_selfcounting: bool = True):
        self.is_sorted = is_sorted
        self.is_selfcounting = is_selfcounting

    def __str__(self):
        return f"{type(self).__name__}(sorted={self.is_sorted}, selfcounting={self.is_selfcounting})"


class NeighboursGPU:
    """One neighbour list (for per-point inspection), ascending members."""

    def __init__(self, initial_size: int = 1, neighbours=None):
        self._neighbours = [] if neighbours is None else list(neighbours)

    @property
    def n_points(self) -> int:
        return len(self._neighbours)

    @property
    def neighbours(self):
        return np.asarray(self._neighbours, dtype=P_AINDEX)

    def assign(self, member: int):
        self._neighbours.append(int(member))

    def reset(self):
        self._neighbours = []

    def enough(self, member_cutoff: int) -> bool:
        """Strict: more than member_cutoff members (_types.pyx:1408-1411)."""
        return len(self._neighbours) > member_cutoff

    def get_member(self, index: int) -> int:
        return self._neighbours[index]

    def contains(self, member: int) -> bool:
        return member in self._neighbours


class SimilarityCheckerGPU:
    """Common-neighbour check on the GPU (sorted-merge semantics)."""

    def __init__(self, context: Optional[_abi.Context] = None):
        self._context = context

    def check(self, neighbours_a, neighbours_b, cluster_params) -> bool:
        a = np.sort(np.asarray(neighbours_a.neighbours, dtype=np.int32))
        b = np.sort(np.asarray(neighbours_b.neighbours, dtype=np.int32))
        ctx = self._context if self._context is not None else _abi.default_context()
        return ctx.check_lists(a, b, cluster_params.similarity_cutoff)

    def __str__(self):
        return f"{type(self).__name__}"


class QueueGPUUnionFind:
    """Placeholder for the BFS queue slot of a recipe: the GPU fitter joins
    clusters with a lock-free union-find, whose result does not depend on
    visiting order (FIFO and LIFO queues give the same labels)."""

    def __str__(self):
        return f"{type(self).__name__}"
