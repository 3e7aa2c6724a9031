"""Oracle for the CommonNN fit path (TEST INFRASTRUCTURE ONLY).

This module is the checker the CUDA library is compared against.  Only the
tests, ``__graft_entry__.smoke()`` and the CPU-baseline legs of ``bench.py``
import it; the library itself never imports, links or falls back to it.

It wraps the C restatement in ``cnn_oracle.c`` (compiled by ``build.py``)
and restates the pure-Python parts of the reference with numpy:

* ``make_parameters``    -- ``Fitter.make_parameters``
                            (src/cnnclustering/_fit.pyx:51-85, 130-161)
* ``sort_by_size``       -- ``Labels.sort_by_size``
                            (src/cnnclustering/_types.pyx:212-286)
* ``clustering_fit``     -- ``Clustering.fit`` orchestration: cnn_offset,
                            label initialisation / frozen labels,
                            parameters, fit, sort_by_size
                            (src/cnnclustering/cluster.pyx:256-392)
* ``repeat_step_labels`` -- the step loop of HierarchicalFitterRepeat._fit
                            (src/cnnclustering/_fit.pyx:1060-1144)
* ``predict_firstmatch`` -- PredictorFirstmatch.predict
                            (src/cnnclustering/_fit.pyx:1235-1291)
* ``periodic_neighbourhoods`` / ``distance_neighbourhoods`` -- the brute-force
                            getter over MetricExtEuclideanPeriodicReduced and
                            over precomputed distances (square or linear)
                            (src/cnnclustering/_types.pyx:1692-1710, 2290-2348,
                            2108-2127, 2019-2037, 1127-1143)
"""
from __future__ import annotations

import ctypes
import os
from typing import Optional

import numpy as np

from . import build as _build

METRIC_EUCLIDEAN_REDUCED = 0
METRIC_EUCLIDEAN = 1
FP_SEPARATE = 0
FP_FUSED = 1


def host_fpmode(fpmode=None) -> int:
    """The float64 accumulation a call uses; None: the reference's as built
    on this host.

    The reference compiles ``total += cpow(a - b, 2)`` (_types.pyx:2253-2267)
    with its setup.py flags; measured with ``oracle/fma_probe.py``, GCC on
    x86-64 (no FMA in the baseline ISA) keeps two roundings and GCC on aarch64
    fuses each term into one FMA.  ``CNN_FPMODE=separate|fused`` in the
    environment overrides the host's mode (the golden fixtures were made on
    x86-64, so tests that compare with them set "separate").
    """
    if fpmode is not None:
        return int(fpmode)
    env = os.environ.get("CNN_FPMODE", "").strip().lower()
    if env in ("separate", "fused"):
        return FP_FUSED if env == "fused" else FP_SEPARATE
    import platform
    return FP_FUSED if platform.machine().lower() in ("aarch64", "arm64") else FP_SEPARATE

_lib = None


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        L = ctypes.CDLL(path)
        i64, i32, dbl, i = ctypes.c_int64, ctypes.c_int32, ctypes.c_double, ctypes.c_int
        p = ctypes.c_void_p
        L.oracle_sqdist.restype = dbl
        L.oracle_sqdist.argtypes = [p, p, i32, i]
        for name in ("oracle_neighbour_counts", "oracle_neighbour_counts_grid"):
            f = getattr(L, name)
            f.restype = i
            f.argtypes = [p, i64, i32, dbl, i, i, i, p]
        for name in ("oracle_neighbour_fill", "oracle_neighbour_fill_grid"):
            f = getattr(L, name)
            f.restype = i
            f.argtypes = [p, i64, i32, dbl, i, i, i, p, p]
        L.oracle_pivot_run.restype = i64
        L.oracle_pivot_run.argtypes = [p, i64, i32, dbl, i, i, i]
        L.oracle_pivot_take.restype = i
        L.oracle_pivot_take.argtypes = [p, p]
        L.oracle_neighbour_row.restype = i64
        L.oracle_neighbour_row.argtypes = [p, i64, i32, p, dbl, i, i, p]
        L.oracle_check_sorted.restype = i
        L.oracle_check_sorted.argtypes = [p, i64, p, i64, i64]
        L.oracle_count_common_sorted.restype = i64
        L.oracle_count_common_sorted.argtypes = [p, i64, p, i64]
        L.oracle_fit_bfs_csr.restype = i64
        L.oracle_fit_bfs_csr.argtypes = [p, p, i64, i64, i64, i64, p, p]
        L.oracle_fit_bfs_points.restype = i64
        L.oracle_fit_bfs_points.argtypes = [p, i64, i32, dbl, i, i, i64, i64, i64, p, p]
        L.oracle_periodic_sqdist.restype = dbl
        L.oracle_periodic_sqdist.argtypes = [p, p, i32, p, i]
        L.oracle_periodic_row.restype = i64
        L.oracle_periodic_row.argtypes = [p, i64, i32, p, p, dbl, i, p]
        _lib = L
    return _lib


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


def _nthreads(nthreads: Optional[int]) -> int:
    if nthreads is None:
        return max(1, len(os.sched_getaffinity(0)))
    return max(1, int(nthreads))


def sqdist(xa, xb, fpmode=None) -> float:
    xa = np.ascontiguousarray(xa, dtype=np.float64)
    xb = np.ascontiguousarray(xb, dtype=np.float64)
    return lib().oracle_sqdist(_ptr(xa), _ptr(xb), xa.shape[0], host_fpmode(fpmode))


def neighbourhoods(x, radius_cutoff: float, metric=METRIC_EUCLIDEAN_REDUCED,
                   fpmode=None, nthreads=None, grid=True):
    """Sorted CSR neighbourhoods (self included) of every point.

    ``radius_cutoff`` is the adjusted value the getter compares with
    (r**2 for the reduced metric).  ``grid``: True = cell grid (n_dim <= 3),
    False = plain brute force, "pivot" = brute force with the exact pivot
    prune (large sets in high dimension).  Returns (offsets int64[n+1],
    indices int32[nnz]).
    """
    x = np.ascontiguousarray(x, dtype=np.float64)
    if x.ndim == 1:
        x = x.reshape(-1, 1)
    n, d = x.shape
    counts = np.zeros(n, dtype=np.int64)
    L = lib()
    nt = _nthreads(nthreads)
    fp = host_fpmode(fpmode)
    if grid == "pivot":
        nnz = L.oracle_pivot_run(_ptr(x), n, d, float(radius_cutoff), metric, fp, nt)
        if nnz >= 0:
            offsets = np.zeros(n + 1, dtype=np.int64)
            indices = np.empty(max(int(nnz), 1), dtype=np.int32)
            if L.oracle_pivot_take(_ptr(offsets), _ptr(indices)) != 0:
                raise MemoryError("oracle pivot rows lost")
            return offsets, indices[:int(nnz)]
        if nnz == -1:
            raise MemoryError("oracle pivot search failed")
        grid = False  # non-finite coordinates: the plain scan
    fc = L.oracle_neighbour_counts_grid if grid else L.oracle_neighbour_counts
    ff = L.oracle_neighbour_fill_grid if grid else L.oracle_neighbour_fill
    if fc(_ptr(x), n, d, float(radius_cutoff), metric, fp, nt, _ptr(counts)) != 0:
        raise MemoryError("oracle neighbour count failed")
    offsets = np.zeros(n + 1, dtype=np.int64)
    np.cumsum(counts, out=offsets[1:])
    indices = np.empty(int(offsets[-1]), dtype=np.int32)
    if ff(_ptr(x), n, d, float(radius_cutoff), metric, fp, nt, _ptr(offsets), _ptr(indices)) != 0:
        raise MemoryError("oracle neighbour fill failed")
    return offsets, indices


def neighbour_row(x, i: int, radius_cutoff: float, metric=METRIC_EUCLIDEAN_REDUCED,
                  fpmode=None) -> np.ndarray:
    """Ascending neighbour indices of point i (self included), brute force."""
    x = np.ascontiguousarray(x, dtype=np.float64)
    n, d = x.shape
    q = np.ascontiguousarray(x[i], dtype=np.float64)
    out = np.empty(n, dtype=np.int32)
    c = lib().oracle_neighbour_row(_ptr(x), n, d, _ptr(q), float(radius_cutoff), metric, host_fpmode(fpmode),
                                   _ptr(out))
    return out[:c].copy()


def check_sorted(a, b, c: int) -> bool:
    a = np.ascontiguousarray(a, dtype=np.int32)
    b = np.ascontiguousarray(b, dtype=np.int32)
    return bool(lib().oracle_check_sorted(_ptr(a), a.shape[0], _ptr(b), b.shape[0], int(c)))


def count_common_sorted(a, b) -> int:
    a = np.ascontiguousarray(a, dtype=np.int32)
    b = np.ascontiguousarray(b, dtype=np.int32)
    return int(lib().oracle_count_common_sorted(_ptr(a), a.shape[0], _ptr(b), b.shape[0]))


def make_parameters(radius_cutoff: float, cnn_cutoff: int, current_start: int = 1,
                    metric=METRIC_EUCLIDEAN_REDUCED, is_selfcounting: bool = True):
    """Fitter.make_parameters (src/cnnclustering/_fit.pyx:130-161)."""
    if metric == METRIC_EUCLIDEAN_REDUCED:
        radius_cutoff = radius_cutoff ** 2
    n_member_cutoff = cnn_cutoff
    similarity_cutoff = cnn_cutoff
    if is_selfcounting:
        n_member_cutoff += 1
        similarity_cutoff += 2
    return {"radius_cutoff": float(radius_cutoff), "similarity_cutoff": int(similarity_cutoff),
            "n_member_cutoff": int(n_member_cutoff), "current_start": int(current_start)}


def fit_bfs_csr(offsets, indices, similarity_cutoff, n_member_cutoff, current_start,
                consider, labels) -> int:
    """FitterExtBFS._fit over sorted CSR lists; updates labels/consider in place."""
    assert consider.dtype == np.uint8 and consider.flags.c_contiguous
    assert labels.dtype == np.int64 and labels.flags.c_contiguous
    offsets = np.ascontiguousarray(offsets, dtype=np.int64)
    indices = np.ascontiguousarray(indices, dtype=np.int32)
    n = offsets.shape[0] - 1
    r = lib().oracle_fit_bfs_csr(_ptr(offsets), _ptr(indices), n, int(similarity_cutoff),
                                 int(n_member_cutoff), int(current_start), _ptr(consider),
                                 _ptr(labels))
    if r < 0:
        raise MemoryError("oracle fit failed")
    return int(r)


def fit_bfs_points(x, radius_cutoff, similarity_cutoff, n_member_cutoff, current_start,
                   consider, labels, metric=METRIC_EUCLIDEAN_REDUCED, fpmode=None) -> int:
    """FitterExtBFS._fit with the brute-force getter (default recipe)."""
    x = np.ascontiguousarray(x, dtype=np.float64)
    n, d = x.shape
    r = lib().oracle_fit_bfs_points(_ptr(x), n, d, float(radius_cutoff), metric, host_fpmode(fpmode),
                                    int(similarity_cutoff), int(n_member_cutoff),
                                    int(current_start), _ptr(consider), _ptr(labels))
    if r < 0:
        raise MemoryError("oracle fit failed")
    return int(r)


def sort_by_size(labels: np.ndarray, member_cutoff: Optional[int] = None,
                 max_clusters: Optional[int] = None) -> dict:
    """Labels.sort_by_size in place (src/cnnclustering/_types.pyx:212-286).

    ``Counter.most_common`` orders by count, descending, and keeps the
    insertion (first occurrence) order for ties.  Returns the reassign map.
    """
    if member_cutoff is None:
        member_cutoff = 2
    uniq, first, counts = np.unique(labels, return_index=True, return_counts=True)
    keep = uniq != 0
    uniq, first, counts = uniq[keep], first[keep], counts[keep]
    if uniq.shape[0] == 0:
        return {}
    if max_clusters is None:
        max_clusters = uniq.shape[0]
    order = np.lexsort((first, -counts))
    reassign = {0: 0}
    new_label = 1
    for cluster_count, k in enumerate(order, 1):
        old = int(uniq[k])
        if cluster_count > max_clusters:
            reassign[old] = 0
            continue
        if counts[k] >= member_cutoff:
            reassign[old] = new_label
            new_label += 1
            continue
        reassign[old] = 0
    keys = np.array(list(reassign.keys()), dtype=np.int64)
    vals = np.array(list(reassign.values()), dtype=np.int64)
    srt = np.argsort(keys)
    pos = np.searchsorted(keys[srt], labels)
    labels[:] = vals[srt][pos]
    return reassign


def clustering_fit(x, radius_cutoff: float, cnn_cutoff: int, member_cutoff=None,
                   max_clusters=None, cnn_offset=None, sort: bool = True,
                   metric=METRIC_EUCLIDEAN_REDUCED, fpmode=None,
                   labels=None, consider=None, frozen: bool = False,
                   neighbours=None, brute_force: bool = False, nthreads=None):
    """Clustering.fit (src/cnnclustering/cluster.pyx:256-392) on the oracle.

    Returns (labels, info) where info holds the CSR and counters.
    """
    x = np.ascontiguousarray(x, dtype=np.float64)
    if x.ndim == 1:
        x = x.reshape(-1, 1)
    n = x.shape[0]
    if cnn_offset is None:
        cnn_offset = 0
    cnn_cutoff -= cnn_offset
    assert cnn_cutoff >= 0
    if labels is None or not frozen:
        labels = np.zeros(n, dtype=np.int64)
        consider = np.ones(n, dtype=np.uint8)
        current_start = 1
    else:
        labels = np.array(labels, dtype=np.int64)
        consider = (np.ones(n, dtype=np.uint8) if consider is None
                    else np.array(consider, dtype=np.uint8))
        current_start = int(labels.max()) + 1 if n else 1
    params = make_parameters(radius_cutoff, cnn_cutoff, current_start, metric)
    info = {"params": params}
    if brute_force:
        info["n_checks"] = fit_bfs_points(x, params["radius_cutoff"], params["similarity_cutoff"],
                                          params["n_member_cutoff"], current_start, consider,
                                          labels, metric, fpmode)
    else:
        if neighbours is None:
            neighbours = neighbourhoods(x, params["radius_cutoff"], metric, fpmode, nthreads)
        offsets, indices = neighbours
        info["offsets"], info["indices"] = offsets, indices
        info["n_checks"] = fit_bfs_csr(offsets, indices, params["similarity_cutoff"],
                                       params["n_member_cutoff"], current_start, consider, labels)
    if sort:
        sort_by_size(labels, member_cutoff, max_clusters)
    return labels, info


def other_row(x, q, radius_cutoff: float, metric=METRIC_EUCLIDEAN_REDUCED, fpmode=None) -> np.ndarray:
    """Ascending indices of the points of x within the cutoff of the point q
    (NeighboursGetterExtBruteForce._get_other, src/cnnclustering/_types.pyx:1712-1731)."""
    x = np.ascontiguousarray(x, dtype=np.float64)
    n, d = x.shape
    q = np.ascontiguousarray(q, dtype=np.float64).reshape(-1)
    out = np.empty(n, dtype=np.int32)
    c = lib().oracle_neighbour_row(_ptr(x), n, d, _ptr(q), float(radius_cutoff), metric, host_fpmode(fpmode),
                                   _ptr(out))
    return out[:c].copy()


def predict_firstmatch(x, labels, y, radius_cutoff: float, similarity_cutoff: int, n_member_cutoff: int,
                       clusters, other_labels=None, other_consider=None, metric=METRIC_EUCLIDEAN_REDUCED,
                       fpmode=None, periodic_bounds=None):
    """PredictorFirstmatch.predict (src/cnnclustering/_fit.pyx:1235-1291) with
    brute-force getters; parameters as Predictor.make_parameters gives them.
    With ``periodic_bounds`` the clustered points' rows use the periodic
    metric while the other points' rows use the plain sum of squares, as
    MetricExtEuclideanPeriodicReduced._calc_distance_other does
    (_types.pyx:2327-2345).  Returns (other_labels, other_consider)."""
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.ascontiguousarray(y, dtype=np.float64)
    m = y.shape[0]
    out = np.zeros(m, dtype=np.int64) if other_labels is None else np.array(other_labels, dtype=np.int64)
    cons = np.ones(m, dtype=np.uint8) if other_consider is None else np.array(other_consider, dtype=np.uint8)
    clusters = set(int(c) for c in clusters)
    if periodic_bounds is not None:
        offsets, indices = periodic_neighbourhoods(x, periodic_bounds, radius_cutoff, fpmode)
    else:
        offsets, indices = neighbourhoods(x, radius_cutoff, metric, fpmode, grid=False)
    for p in range(m):
        if cons[p] == 0:
            continue
        row = other_row(x, y[p], radius_cutoff, metric, fpmode)
        if not row.shape[0] > n_member_cutoff:
            continue
        for i in row:
            label = int(labels[i])
            if label not in clusters:
                continue
            nb = indices[offsets[i]:offsets[i + 1]]
            if not nb.shape[0] > n_member_cutoff:
                continue
            if check_sorted(row, nb, similarity_cutoff):
                cons[p] = 0
                out[p] = label
                break
    return out, cons


def repeat_step_labels(x, radius_cutoffs, cnn_cutoffs, member_cutoff=None, max_clusters=None, cnn_offset=None,
                       sort: bool = True, metric=METRIC_EUCLIDEAN_REDUCED, fpmode=None):
    """Labels of every step of HierarchicalFitterRepeat._fit
    (src/cnnclustering/_fit.pyx:1060-1144).  Its make_parameters finds no
    neighbours getter on the hierarchical fitter, so each step compares with
    radius_cutoff itself and uses similarity = n_member = cnn_cutoff."""
    x = np.ascontiguousarray(x, dtype=np.float64)
    radius_cutoffs = [float(r) for r in np.atleast_1d(radius_cutoffs)]
    cnn_cutoffs = [int(c) for c in np.atleast_1d(cnn_cutoffs)]
    if len(radius_cutoffs) == 1:
        radius_cutoffs *= len(cnn_cutoffs)
    if len(cnn_cutoffs) == 1:
        cnn_cutoffs *= len(radius_cutoffs)
    offset = 0 if cnn_offset is None else cnn_offset
    rows = []
    for r, c in zip(radius_cutoffs, cnn_cutoffs):
        c -= offset
        labels = np.zeros(x.shape[0], dtype=np.int64)
        consider = np.ones(x.shape[0], dtype=np.uint8)
        off, ind = neighbourhoods(x, r, metric, fpmode)
        fit_bfs_csr(off, ind, c, c, 1, consider, labels)
        if sort:
            sort_by_size(labels, member_cutoff, max_clusters)
        rows.append(labels)
    return np.stack(rows)


def _rows_to_csr(rows):
    offsets = np.zeros(len(rows) + 1, dtype=np.int64)
    offsets[1:] = np.cumsum([r.shape[0] for r in rows])
    indices = np.concatenate(rows).astype(np.int32) if rows else np.zeros(0, dtype=np.int32)
    return offsets, indices


def periodic_neighbourhoods(x, bounds, radius_cutoff: float, fpmode=None):
    """Brute-force rows (self included, ascending) under the periodic metric;
    radius_cutoff as compared (r**2)."""
    x = np.ascontiguousarray(x, dtype=np.float64)
    n, d = x.shape
    b = np.ascontiguousarray(bounds, dtype=np.float64).reshape(-1)
    out = np.empty(n, dtype=np.int32)
    L = lib()
    rows = []
    for i in range(n):
        c = L.oracle_periodic_row(_ptr(x), n, d, _ptr(b), _ptr(np.ascontiguousarray(x[i])), float(radius_cutoff),
                                  host_fpmode(fpmode), _ptr(out))
        rows.append(out[:c].copy())
    return _rows_to_csr(rows)


def linear_distance(data, n: int, a: int, b: int) -> float:
    """InputDataExtDistancesLinearMemoryview._get_distance (_types.pyx:1127-1143)."""
    if a == b:
        return 0.0
    a, b = min(a, b), max(a, b)
    return float(data[a * (n - 1) - (a * a - a) // 2 + b - a - 1])


def distance_neighbourhoods(dist, radius_cutoff: float, linear: bool = False, n_points=None):
    """Rows {j : distance(i, j) <= radius_cutoff} (ascending) from a square
    matrix or the linear upper triangle."""
    if linear:
        dist = np.asarray(dist, dtype=np.float64).reshape(-1)
        n = int(n_points) if n_points is not None else int(0.5 * (np.sqrt(8 * dist.shape[0] + 1) + 1))
        sq = np.zeros((n, n), dtype=np.float64)
        iu = np.triu_indices(n, 1)  # row-major upper triangle, the linear order
        sq[iu] = dist
        sq[(iu[1], iu[0])] = dist
    else:
        sq = np.asarray(dist, dtype=np.float64)
    rows = [np.nonzero(sq[i] <= radius_cutoff)[0].astype(np.int32) for i in range(sq.shape[0])]
    return _rows_to_csr(rows)


def fit_from_neighbourhoods(offsets, indices, cnn_cutoff: int, member_cutoff=None, max_clusters=None,
                            is_selfcounting: bool = True):
    """Clustering.fit on given rows: parameters (c+2, c+1), fresh labels, sort_by_size."""
    n = offsets.shape[0] - 1
    labels = np.zeros(n, dtype=np.int64)
    consider = np.ones(n, dtype=np.uint8)
    sim = cnn_cutoff + 2 if is_selfcounting else cnn_cutoff
    nmem = cnn_cutoff + 1 if is_selfcounting else cnn_cutoff
    fit_bfs_csr(offsets, indices, sim, nmem, 1, consider, labels)
    sort_by_size(labels, member_cutoff, max_clusters)
    return labels


def mst_prim_edges(x, radius_cutoff: float, metric=METRIC_EUCLIDEAN_REDUCED, fpmode=None, neighbours=None):
    """Tree edges of HierarchicalFitterMSTPrim._fit (src/cnnclustering/_fit.pyx:
    820-899) in the order its tree queue pops them: Prim's algorithm over the
    neighbour graph from every unvisited point in index order, weights = the
    full common-neighbour count (SimilarityCheckerExtScreensorted._get,
    _types.pyx:2708-2753), a max-heap keyed (-weight, (a, b)).
    ``radius_cutoff`` as compared (r**2 for the reduced metric).
    Returns a list of (a, b, weight)."""
    import heapq
    x = np.ascontiguousarray(x, dtype=np.float64)
    n = x.shape[0]
    if neighbours is None:
        neighbours = neighbourhoods(x, radius_cutoff, metric, fpmode)
    off, idx = neighbours
    rows = [idx[off[i]:off[i + 1]] for i in range(n)]
    visited = np.zeros(n, dtype=bool)
    heap, tree = [], []
    for point in range(n):
        if visited[point]:
            continue
        visited[point] = True
        for member in rows[point]:
            if not visited[member]:
                heapq.heappush(heap, (-count_common_sorted(rows[point], rows[member]), (point, int(member))))
        while heap:
            w, (a, b) = heapq.heappop(heap)
            if visited[b]:
                continue
            visited[b] = True
            heapq.heappush(tree, (w, (a, b)))
            for member in rows[b]:
                if not visited[member]:
                    heapq.heappush(heap, (-count_common_sorted(rows[b], rows[member]), (b, int(member))))
    out = []
    while tree:
        w, (a, b) = heapq.heappop(tree)
        out.append((a, b, -w))
    return out
