"""ctypes binding of libcnngpu.so (the C ABI declared in include/cnngpu.h).

The library is the only compute path: if it cannot be loaded, every entry
point raises.  There is no CPU fallback.

Arrays handed to the library are numpy arrays (host memory, copied by the
library) or CUDA device arrays: torch tensors on a CUDA device or any
object exposing ``__cuda_array_interface__`` (used in place, on the
context's stream).
"""
from __future__ import annotations

import ctypes
import os
import threading
from typing import Optional

import numpy as np

from . import _build

CNN_OK = 0
CNN_ERR_INVALID_ARG, CNN_ERR_OOM, CNN_ERR_CUDA, CNN_ERR_TIMEOUT, CNN_ERR_UNSUPPORTED, CNN_ERR_STATE = 1, 2, 3, 4, 5, 6
_STATUS = {1: "invalid argument", 2: "out of memory", 3: "CUDA error", 4: "timeout",
           5: "unsupported", 6: "bad state"}

METRIC_EUCLIDEAN_REDUCED = 0
METRIC_EUCLIDEAN = 1
METRIC_PRECOMPUTED = 2
METRIC_EUCLIDEAN_PERIODIC_REDUCED = 3
DIST_SQUARE = 0
DIST_LINEAR = 1
FP_SEPARATE = 0
FP_FUSED = 1
DTYPE_F64 = 0
DTYPE_F32 = 1
MEM_HOST = 0
MEM_DEVICE = 1
SEARCH_AUTO = 0
SEARCH_GRID = 1
SEARCH_ALL_PAIRS = 2
SEARCH_TENSOR = 3
INTERSECT_AUTO = 0
INTERSECT_MERGE = 1
INTERSECT_BITSET = 2


def host_fpmode(fpmode: Optional[int] = None) -> int:
    """The float64 accumulation of the distance sum; None: the one the
    reference reproduces when it is built on this host.

    The reference sums ``total += cpow(a - b, 2)`` (src/cnnclustering/
    _types.pyx:2253-2267) and is compiled with its setup.py flags.  GCC on
    x86-64 (no FMA in the baseline ISA) keeps the multiply and the add
    (FP_SEPARATE); GCC on aarch64 (the GB300's Grace host) fuses each term
    into one FMA (FP_FUSED), with the same flags.  ``CNN_FPMODE=separate`` or
    ``fused`` in the environment chooses explicitly.
    """
    if fpmode is not None:
        return int(fpmode)
    env = os.environ.get("CNN_FPMODE", "").strip().lower()
    if env in ("separate", "fused"):
        return FP_FUSED if env == "fused" else FP_SEPARATE
    import platform
    return FP_FUSED if platform.machine().lower() in ("aarch64", "arm64") else FP_SEPARATE


class CNNError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{_STATUS.get(status, status)}: {message}")
        self.status = status


class cnn_stats(ctypes.Structure):
    _fields_ = [
        ("n_points", ctypes.c_int64), ("n_nonzero", ctypes.c_int64), ("n_nodes", ctypes.c_int64),
        ("n_checks", ctypes.c_int64), ("n_accepted", ctypes.c_int64), ("n_exact", ctypes.c_int64),
        ("n_candidates", ctypes.c_int64), ("n_clusters", ctypes.c_int64),
        ("search_kind", ctypes.c_int32), ("filter_enabled", ctypes.c_int32), ("filter_band", ctypes.c_double),
        ("ms_bbox", ctypes.c_float), ("ms_cells", ctypes.c_float), ("ms_count", ctypes.c_float),
        ("ms_scan", ctypes.c_float), ("ms_fill", ctypes.c_float), ("ms_nodes", ctypes.c_float),
        ("ms_check", ctypes.c_float), ("ms_label", ctypes.c_float), ("ms_sort", ctypes.c_float),
        ("n_launches", ctypes.c_int64), ("ms_gram", ctypes.c_float), ("max_abs_err", ctypes.c_float),
        ("intersection", ctypes.c_int32), ("tuned", ctypes.c_int32), ("tune_ms_merge", ctypes.c_float),
        ("tune_ms_bitset", ctypes.c_float), ("ms_weights", ctypes.c_float),
        ("graphs", ctypes.c_int32), ("graph_nodes", ctypes.c_int64), ("ms_graph_build", ctypes.c_float),
    ]

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}


# every symbol include/cnngpu.h declares, with its ctypes signature
_P = ctypes.c_void_p
_I64 = ctypes.c_int64
_I32 = ctypes.c_int32
_INT = ctypes.c_int
class cnn_job(ctypes.Structure):
    _fields_ = [
        ("points", ctypes.c_void_p), ("dtype", ctypes.c_int), ("n_points", ctypes.c_int64),
        ("n_dim", ctypes.c_int32), ("metric", ctypes.c_int), ("fpmode", ctypes.c_int),
        ("radius_cutoff", ctypes.c_double), ("similarity_cutoff", ctypes.c_int64),
        ("n_member_cutoff", ctypes.c_int64), ("member_cutoff", ctypes.c_int64), ("max_clusters", ctypes.c_int64),
        ("labels", ctypes.c_void_p), ("reserve_bytes", ctypes.c_int64),
    ]


class cnn_job_info(ctypes.Structure):
    _fields_ = [
        ("state", ctypes.c_int), ("result", ctypes.c_int), ("slot", ctypes.c_int32), ("attempts", ctypes.c_int32),
        ("reserved_bytes", ctypes.c_int64), ("t_submit", ctypes.c_double), ("t_start", ctypes.c_double),
        ("t_done", ctypes.c_double),
    ]

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}


class cnn_server_stats(ctypes.Structure):
    _fields_ = [
        ("submitted", ctypes.c_int64), ("done", ctypes.c_int64), ("failed", ctypes.c_int64),
        ("requeued", ctypes.c_int64), ("released", ctypes.c_int64), ("running", ctypes.c_int32),
        ("queued", ctypes.c_int32), ("max_running", ctypes.c_int32), ("budget_bytes", ctypes.c_int64),
        ("committed_bytes", ctypes.c_int64), ("held_bytes", ctypes.c_int64), ("peak_held_bytes", ctypes.c_int64),
    ]

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}


JOB_QUEUED, JOB_RUNNING, JOB_DONE = 0, 1, 2

SIGNATURES = {
    "cnn_abi_version": (_INT, []),
    "cnn_create": (_INT, [ctypes.POINTER(_P), _INT, _P]),
    "cnn_destroy": (_INT, [_P]),
    "cnn_set_stream": (_INT, [_P, _P]),
    "cnn_last_error": (ctypes.c_char_p, [_P]),
    "cnn_set_timing": (_INT, [_P, _INT]),
    "cnn_get_stats": (_INT, [_P, ctypes.POINTER(cnn_stats)]),
    "cnn_set_wait_limit": (_INT, [_P, _I64]),
    "cnn_set_search": (_INT, [_P, _INT]),
    "cnn_set_intersection": (_INT, [_P, _INT]),
    "cnn_set_points": (_INT, [_P, _P, _INT, _I64, _I32, _INT]),
    "cnn_build_neighbours": (_INT, [_P, ctypes.c_double, _INT, _INT]),
    "cnn_set_neighbours": (_INT, [_P, _P, _P, _I64, _INT]),
    "cnn_neighbour_count": (_INT, [_P, ctypes.POINTER(_I64)]),
    "cnn_get_neighbours": (_INT, [_P, _P, _P, _INT]),
    "cnn_fit": (_INT, [_P, _I64, _I64, _I64, _P, _P, _I64, _INT]),
    "cnn_fit_fresh": (_INT, [_P, _I64, _I64, _I32, _I64, _I64, _P, _P, _I64, _INT]),
    "cnn_graph_generation": (_INT, [_P, ctypes.POINTER(_I64)]),
    "cnn_sort_by_size": (_INT, [_P, _P, _I64, _I64, _I64, _INT]),
    "cnn_check_lists": (_INT, [_P, _P, _I64, _P, _I64, _I64, _P, _INT]),
    "cnn_fit_csr_noalloc": (_INT, [_P, _P, _I64, _I64, _I64, _I64, _P, _P, _P]),
    "cnn_sweep": (_INT, [_P, _P, _I32, _P, _P, _I32, _INT, _INT, _I64, _I64, _P, _INT]),
    "cnn_sweep_pairs": (_INT, [_P, _P, _P, _P, _I32, _INT, _INT, _I32, _I64, _I64, _P, _INT]),
    "cnn_set_distances": (_INT, [_P, _P, _INT, _I64, _INT]),
    "cnn_mst_prim": (_INT, [_P, ctypes.c_double, _INT, _INT, _P, _P, _P, _I64, ctypes.POINTER(_I64)]),
    "cnn_set_periodic_bounds": (_INT, [_P, _P, _I32]),
    "cnn_predict": (_INT, [_P, _P, _INT, _I64, _I32, _P, _P, _I64, ctypes.c_double, _INT, _INT, _I64, _I64, _P, _P,
                           _INT]),
    "cnn_server_create": (_INT, [ctypes.POINTER(_P), _INT, _I32, _I64]),
    "cnn_server_destroy": (_INT, [_P]),
    "cnn_submit": (_INT, [_P, ctypes.POINTER(cnn_job), ctypes.POINTER(_I64)]),
    "cnn_poll": (_INT, [_P, _I64, ctypes.POINTER(cnn_job_info)]),
    "cnn_wait": (_INT, [_P, _I64, _I64, ctypes.POINTER(cnn_job_info)]),
    "cnn_job_error": (_INT, [_P, _I64, ctypes.c_char_p, _I64]),
    "cnn_job_release": (_INT, [_P, _I64]),
    "cnn_server_get_stats": (_INT, [_P, ctypes.POINTER(cnn_server_stats)]),
}

_lib = None
_lib_lock = threading.Lock()


def lib_path() -> str:
    return _build.LIB


ABI_VERSION = 2  # CNN_ABI_VERSION of include/cnngpu.h


def load(build_if_missing: bool = True):
    """Load libcnngpu.so (building it first when it is missing or stale)."""
    global _lib
    with _lib_lock:
        if _lib is None:
            path = _build.LIB
            if build_if_missing:
                _build.build()
            if not os.path.exists(path):
                raise ImportError(f"libcnngpu.so not found at {path}; build it with "
                                  "python -c 'import __graft_entry__ as g; g.build()'")
            L = ctypes.CDLL(path)
            for name, (res, args) in SIGNATURES.items():
                f = getattr(L, name)
                f.restype = res
                f.argtypes = args
            if L.cnn_abi_version() != ABI_VERSION:  # the structs below mirror this version's header
                raise ImportError(f"{path} has ABI version {L.cnn_abi_version()}, this binding expects "
                                  f"{ABI_VERSION}: rebuild it")
            _lib = L
    return _lib


# ---------------------------------------------------------------------------
# array helpers
# ---------------------------------------------------------------------------
def _torch():
    try:
        import torch
        return torch
    except ImportError:  # pragma: no cover
        return None


def is_device_array(a) -> bool:
    t = _torch()
    if t is not None and isinstance(a, t.Tensor):
        return a.is_cuda
    return hasattr(a, "__cuda_array_interface__")


def device_pointer(a, dtype, writable=False) -> int:
    """Pointer of a contiguous CUDA array of the given numpy dtype."""
    t = _torch()
    if t is not None and isinstance(a, t.Tensor):
        want = {np.float64: t.float64, np.float32: t.float32, np.int64: t.int64,
                np.int32: t.int32, np.uint8: t.uint8}[np.dtype(dtype).type]
        if a.dtype != want:
            raise TypeError(f"expected a {want} tensor, got {a.dtype}")
        if not a.is_contiguous():
            raise ValueError("device tensors must be contiguous")
        return int(a.data_ptr())
    cai = a.__cuda_array_interface__
    if np.dtype(cai["typestr"]) != np.dtype(dtype):
        raise TypeError(f"expected {np.dtype(dtype)}, got {cai['typestr']}")
    if cai.get("strides") not in (None,):
        exp = np.empty(cai["shape"], dtype=dtype).strides
        if tuple(cai["strides"]) != tuple(exp):
            raise ValueError("device arrays must be C-contiguous")
    if writable and cai["data"][1]:
        raise ValueError("device array is read-only")
    return int(cai["data"][0])


def host_array(a, dtype, writable=False) -> np.ndarray:
    arr = np.asarray(a)
    if arr.dtype != np.dtype(dtype) or not arr.flags.c_contiguous:
        if writable:
            raise TypeError(f"in-place arrays must be C-contiguous {np.dtype(dtype)}")
        arr = np.ascontiguousarray(arr, dtype=dtype)
    if writable and not arr.flags.writeable:
        raise ValueError("array is read-only")
    return arr


def current_torch_stream(device: int) -> Optional[int]:
    t = _torch()
    if t is None or not t.cuda.is_available():
        return None
    return int(t.cuda.current_stream(device).cuda_stream)


class Context:
    """One library context: device workspace, neighbour graph, stream."""

    def __init__(self, device: int = 0, stream: Optional[int] = None):
        self._lib = load()
        h = ctypes.c_void_p()
        st = self._lib.cnn_create(ctypes.byref(h), int(device), ctypes.c_void_p(stream) if stream else None)
        if st != CNN_OK:
            raise CNNError(st, f"cnn_create(device={device}) failed (is a CUDA device visible?)")
        self._h = h
        self.device = int(device)
        self.stream = stream
        self._n_points = 0
        self._points_set = False  # without points the library itself reports the missing graph

    def close(self):
        if getattr(self, "_h", None):
            self._lib.cnn_destroy(self._h)
            self._h = None

    def __del__(self):  # pragma: no cover
        try:
            self.close()
        except Exception:
            pass

    def _check(self, st: int, what: str):
        if st != CNN_OK:
            msg = self._lib.cnn_last_error(self._h)
            raise CNNError(st, f"{what}: {msg.decode() if msg else ''}")

    # -- configuration -------------------------------------------------------
    def set_stream(self, stream: Optional[int]):
        self._check(self._lib.cnn_set_stream(self._h, ctypes.c_void_p(stream) if stream else None),
                    "cnn_set_stream")
        self.stream = stream

    def set_timing(self, enabled: bool):
        self._check(self._lib.cnn_set_timing(self._h, 1 if enabled else 0), "cnn_set_timing")

    def set_search(self, search: int):
        """Search preference of the following builds (SEARCH_AUTO,
        SEARCH_GRID, SEARCH_ALL_PAIRS, SEARCH_TENSOR); same neighbour sets."""
        self._check(self._lib.cnn_set_search(self._h, int(search)), "cnn_set_search")

    def set_intersection(self, strategy: int):
        """Intersection strategy of cell-grid fits (INTERSECT_AUTO: tuned per
        workload profile, INTERSECT_MERGE: sorted lists, INTERSECT_BITSET:
        bit masks); same labels."""
        self._check(self._lib.cnn_set_intersection(self._h, int(strategy)), "cnn_set_intersection")

    def set_wait_limit(self, limit_ns: int):
        """Limit of the kernels' bounded waits (ns); <= 0: the default 2 s."""
        self._check(self._lib.cnn_set_wait_limit(self._h, int(limit_ns)), "cnn_set_wait_limit")

    def stats(self) -> dict:
        s = cnn_stats()
        self._check(self._lib.cnn_get_stats(self._h, ctypes.byref(s)), "cnn_get_stats")
        return s.as_dict()

    # -- neighbour graph -------------------------------------------------------
    def set_distances(self, distances, layout: int = DIST_SQUARE, n_points: Optional[int] = None):
        """Precomputed distances (float64): [n, n] (DIST_SQUARE) or the
        n(n-1)/2 upper triangle by rows (DIST_LINEAR)."""
        if is_device_array(distances):
            ptr, mem, keep = device_pointer(distances, np.float64), MEM_DEVICE, distances
            size = int(np.prod(tuple(distances.shape)))
        else:
            arr = host_array(distances, np.float64)
            ptr, mem, keep, size = arr.ctypes.data, MEM_HOST, arr, arr.size
        if layout == DIST_SQUARE:
            n = int(distances.shape[0])
        else:
            n = int(n_points) if n_points is not None else int(0.5 * (np.sqrt(8 * size + 1) + 1))
        self._check(self._lib.cnn_set_distances(self._h, ctypes.c_void_p(ptr), int(layout), n, mem),
                    "cnn_set_distances")
        self._points_ref = keep
        self._n_points = n
        self._points_set = True

    def set_periodic_bounds(self, bounds):
        b = np.ascontiguousarray(bounds, dtype=np.float64).reshape(-1)
        self._check(self._lib.cnn_set_periodic_bounds(self._h, ctypes.c_void_p(b.ctypes.data), b.shape[0]),
                    "cnn_set_periodic_bounds")

    def set_points(self, points):
        """points: [n, d] float64/float32 numpy array or CUDA array."""
        if is_device_array(points):
            shape = tuple(points.shape)
            dt = np.float32 if "float32" in str(points.dtype) else np.float64
            ptr = device_pointer(points, dt)
            mem, keep = MEM_DEVICE, points
        else:
            arr = np.asarray(points)
            dt = np.float32 if arr.dtype == np.float32 else np.float64
            arr = host_array(arr, dt)
            shape = arr.shape
            ptr, mem, keep = arr.ctypes.data, MEM_HOST, arr
        if len(shape) == 1:
            shape = (shape[0], 1)
        if len(shape) != 2:
            raise ValueError("points must be a 2D array [n_points, n_dim]")
        self._check(self._lib.cnn_set_points(self._h, ctypes.c_void_p(ptr), DTYPE_F32 if dt == np.float32 else DTYPE_F64,
                                             int(shape[0]), int(shape[1]), mem), "cnn_set_points")
        self._points_ref = keep
        self._n_points = int(shape[0])
        self._points_set = True
        return shape

    def build_neighbours(self, radius_cutoff: float, metric: int = METRIC_EUCLIDEAN_REDUCED,
                         fpmode: Optional[int] = None):
        self._check(self._lib.cnn_build_neighbours(self._h, float(radius_cutoff), int(metric), host_fpmode(fpmode)),
                    "cnn_build_neighbours")

    def set_neighbours(self, offsets, indices):
        if is_device_array(offsets):
            n = int(offsets.shape[0]) - 1
            self._check(self._lib.cnn_set_neighbours(
                self._h, ctypes.c_void_p(device_pointer(offsets, np.int64)),
                ctypes.c_void_p(device_pointer(indices, np.int32)), n, MEM_DEVICE), "cnn_set_neighbours")
            self._points_ref = (offsets, indices)
        else:
            off = host_array(offsets, np.int64)
            idx = host_array(indices, np.int32)
            n = off.shape[0] - 1
            self._check(self._lib.cnn_set_neighbours(self._h, ctypes.c_void_p(off.ctypes.data),
                                                     ctypes.c_void_p(idx.ctypes.data), n, MEM_HOST),
                        "cnn_set_neighbours")
        self._n_points = n
        self._points_set = True

    def neighbour_count(self) -> int:
        v = ctypes.c_int64()
        self._check(self._lib.cnn_neighbour_count(self._h, ctypes.byref(v)), "cnn_neighbour_count")
        return int(v.value)

    def get_neighbours(self, n_points: Optional[int] = None):
        """Sorted CSR (offsets int64[n+1], indices int32[nnz]) as numpy arrays."""
        if n_points is None:
            n_points = int(self._n_points)
        nnz = self.neighbour_count()
        off = np.empty(n_points + 1, dtype=np.int64)
        idx = np.empty(max(nnz, 1), dtype=np.int32)
        self._check(self._lib.cnn_get_neighbours(self._h, ctypes.c_void_p(off.ctypes.data),
                                                 ctypes.c_void_p(idx.ctypes.data), MEM_HOST),
                    "cnn_get_neighbours")
        return off, idx[:nnz]

    def graph_generation(self) -> int:
        """Changes whenever this context's points, distances, neighbourhoods
        or neighbour graph are replaced (by any caller of the context)."""
        v = ctypes.c_int64()
        self._check(self._lib.cnn_graph_generation(self._h, ctypes.byref(v)), "cnn_graph_generation")
        return int(v.value)

    # -- fit -------------------------------------------------------------------
    def fit(self, similarity_cutoff: int, n_member_cutoff: int, current_start: int, consider, labels):
        """Cluster the current graph; labels/consider updated in place.

        labels and consider must hold exactly one entry per point of the
        current graph (ValueError otherwise, before the library is called).
        """
        n_lab, n_con = int(labels.shape[0]), int(consider.shape[0])
        if n_lab != n_con or (self._points_set and n_lab != int(self._n_points)):
            raise ValueError(f"labels ({n_lab}) and consider ({n_con}) must have one entry per point of the "
                             f"current neighbour graph ({int(self._n_points)})")
        if is_device_array(labels):
            lp = device_pointer(labels, np.int64, writable=True)
            cp = device_pointer(consider, np.uint8, writable=True)
            mem = MEM_DEVICE
        else:
            lab = host_array(labels, np.int64, writable=True)
            con = host_array(consider, np.uint8, writable=True)
            lp, cp, mem = lab.ctypes.data, con.ctypes.data, MEM_HOST
        self._check(self._lib.cnn_fit(self._h, int(similarity_cutoff), int(n_member_cutoff), int(current_start),
                                      ctypes.c_void_p(cp), ctypes.c_void_p(lp), n_lab, mem), "cnn_fit")

    def fit_fresh(self, similarity_cutoff: int, n_member_cutoff: int, sort: bool = True, member_cutoff: int = 2,
                  max_clusters: Optional[int] = None, labels=None, consider=None):
        """Clustering.fit from fresh labels (current_start 1), then
        sort_by_size when ``sort``, in one library call (cnn_fit_fresh).
        ``labels``: output array (host or CUDA, one int64 per point), a new
        host array when None; ``consider``: optional output (all 0 after).
        Returns labels."""
        n = int(self._n_points)
        if labels is None:
            labels = np.empty(n, dtype=np.int64)
        if int(labels.shape[0]) != n or (consider is not None and int(consider.shape[0]) != n):
            raise ValueError(f"labels/consider must have one entry per point of the current neighbour graph ({n})")
        mx = -1 if max_clusters is None else int(max_clusters)
        if mx < -1:
            mx = 0  # a negative limit keeps no cluster (every rank exceeds it)
        if is_device_array(labels):
            lp = device_pointer(labels, np.int64, writable=True)
            cp = device_pointer(consider, np.uint8, writable=True) if consider is not None else 0
            mem = MEM_DEVICE
        else:
            lab = host_array(labels, np.int64, writable=True)
            con = host_array(consider, np.uint8, writable=True) if consider is not None else None
            lp, cp, mem = lab.ctypes.data, (con.ctypes.data if con is not None else 0), MEM_HOST
        self._check(self._lib.cnn_fit_fresh(self._h, int(similarity_cutoff), int(n_member_cutoff), 1 if sort else 0,
                                            int(member_cutoff), mx, ctypes.c_void_p(lp), ctypes.c_void_p(cp or None),
                                            n, mem), "cnn_fit_fresh")
        return labels

    def sort_by_size(self, labels, member_cutoff: int, max_clusters: Optional[int]):
        mx = -1 if max_clusters is None else int(max_clusters)
        if mx < -1:
            mx = 0  # a negative limit keeps no cluster (every rank exceeds it)
        if is_device_array(labels):
            lp, mem, n = device_pointer(labels, np.int64, writable=True), MEM_DEVICE, int(labels.shape[0])
        else:
            lab = host_array(labels, np.int64, writable=True)
            lp, mem, n = lab.ctypes.data, MEM_HOST, lab.shape[0]
        self._check(self._lib.cnn_sort_by_size(self._h, ctypes.c_void_p(lp), n, int(member_cutoff), mx, mem),
                    "cnn_sort_by_size")

    def sweep(self, radius_cutoffs, cuts, member_cutoff: int = 2, max_clusters: Optional[int] = None,
              metric: int = METRIC_EUCLIDEAN_REDUCED, fpmode: Optional[int] = None, labels_out=None):
        """Fits for every (radius, cut) pair on the current points.

        radius_cutoffs: adjusted cutoffs, ascending.  cuts: sequence of
        (similarity_cutoff, n_member_cutoff).  Returns labels of shape
        [n_radii, n_cuts, n_points]: labels_out when given (a CUDA tensor,
        or a C-contiguous int64 host array of that shape, e.g. in pinned
        memory), else a new host numpy array.
        """
        rc = np.ascontiguousarray(radius_cutoffs, dtype=np.float64)
        sc = np.ascontiguousarray([c[0] for c in cuts], dtype=np.int64)
        nm = np.ascontiguousarray([c[1] for c in cuts], dtype=np.int64)
        mx = -1 if max_clusters is None else int(max_clusters)
        n = int(self._n_points)
        if labels_out is not None and is_device_array(labels_out):
            ptr, mem, out = device_pointer(labels_out, np.int64, writable=True), MEM_DEVICE, labels_out
        elif labels_out is not None:
            out = labels_out
            if (not isinstance(out, np.ndarray) or out.dtype != np.int64 or not out.flags.c_contiguous
                    or not out.flags.writeable or out.shape != (rc.shape[0], sc.shape[0], n)):
                raise ValueError(f"labels_out: a writable C-contiguous int64 array of shape "
                                 f"{(rc.shape[0], sc.shape[0], n)} is needed")
            ptr, mem = out.ctypes.data, MEM_HOST
        else:
            out = np.empty((rc.shape[0], sc.shape[0], n), dtype=np.int64)
            ptr, mem = out.ctypes.data, MEM_HOST
        self._check(self._lib.cnn_sweep(self._h, ctypes.c_void_p(rc.ctypes.data), rc.shape[0],
                                        ctypes.c_void_p(sc.ctypes.data), ctypes.c_void_p(nm.ctypes.data),
                                        sc.shape[0], int(metric), host_fpmode(fpmode), int(member_cutoff), mx,
                                        ctypes.c_void_p(ptr), mem), "cnn_sweep")
        return out

    def sweep_pairs(self, radius_cutoffs, cuts, member_cutoff: int = 2, max_clusters: Optional[int] = None,
                    sort: bool = True, metric: int = METRIC_EUCLIDEAN_REDUCED, fpmode: Optional[int] = None,
                    labels_out=None):
        """Fits for a list of steps on the current points.

        radius_cutoffs: adjusted cutoff per step (any order, repeats allowed).
        cuts: (similarity_cutoff, n_member_cutoff) per step.  Returns labels
        of shape [n_steps, n_points] (host numpy array unless a CUDA tensor is
        given as labels_out); row i equals the separate fit of step i.
        """
        rc = np.ascontiguousarray(radius_cutoffs, dtype=np.float64).reshape(-1)
        if len(cuts) != rc.shape[0]:
            raise ValueError("need one (similarity_cutoff, n_member_cutoff) per radius cutoff")
        sc = np.ascontiguousarray([c[0] for c in cuts], dtype=np.int64)
        nm = np.ascontiguousarray([c[1] for c in cuts], dtype=np.int64)
        mx = -1 if max_clusters is None else int(max_clusters)
        n = int(self._n_points)
        if labels_out is not None and is_device_array(labels_out):
            ptr, mem, out = device_pointer(labels_out, np.int64, writable=True), MEM_DEVICE, labels_out
        else:
            out = np.empty((rc.shape[0], n), dtype=np.int64)
            ptr, mem = out.ctypes.data, MEM_HOST
        self._check(self._lib.cnn_sweep_pairs(self._h, ctypes.c_void_p(rc.ctypes.data),
                                              ctypes.c_void_p(sc.ctypes.data), ctypes.c_void_p(nm.ctypes.data),
                                              rc.shape[0], int(metric), host_fpmode(fpmode), 1 if sort else 0,
                                              int(member_cutoff), mx, ctypes.c_void_p(ptr), mem), "cnn_sweep_pairs")
        return out

    def predict(self, other_points, labels, clusters, radius_cutoff: float, similarity_cutoff: int,
                n_member_cutoff: int, other_labels, other_consider, metric: int = METRIC_EUCLIDEAN_REDUCED,
                fpmode: Optional[int] = None):
        """First-match labels for other points from the current points' labels.

        other_points: [m, n_dim] float64/float32; labels: [n_points] int64 of
        the current points; clusters: labels that may be handed out.
        other_labels (int64 [m]) and other_consider (uint8 [m]) are updated in
        place.  All arrays on the host, or all CUDA tensors.
        """
        dev = is_device_array(other_points)
        if dev:
            dt = np.float32 if "float32" in str(other_points.dtype) else np.float64
            shape = tuple(other_points.shape)
            xp = device_pointer(other_points, dt)
            lab_p = device_pointer(labels, np.int64)
            out_l = device_pointer(other_labels, np.int64, writable=True)
            out_c = device_pointer(other_consider, np.uint8, writable=True)
            t = _torch()
            cl = t.as_tensor(sorted({int(c) for c in clusters}), dtype=t.int64, device=other_points.device)
            cl_p, n_cl, mem, keep = device_pointer(cl, np.int64), int(cl.shape[0]), MEM_DEVICE, cl
        else:
            xo = np.asarray(other_points)
            dt = np.float32 if xo.dtype == np.float32 else np.float64
            xo = host_array(xo.reshape(xo.shape[0], -1) if xo.ndim == 1 else xo, dt)
            shape = xo.shape
            lab = host_array(labels, np.int64)
            ol = host_array(other_labels, np.int64, writable=True)
            oc = host_array(other_consider, np.uint8, writable=True)
            cl = np.ascontiguousarray(sorted({int(c) for c in clusters}), dtype=np.int64)
            xp, lab_p, out_l, out_c = xo.ctypes.data, lab.ctypes.data, ol.ctypes.data, oc.ctypes.data
            cl_p, n_cl, mem, keep = cl.ctypes.data, int(cl.shape[0]), MEM_HOST, (xo, lab, cl)
        self._check(self._lib.cnn_predict(self._h, ctypes.c_void_p(xp), DTYPE_F32 if dt == np.float32 else DTYPE_F64,
                                          int(shape[0]), int(shape[1]), ctypes.c_void_p(lab_p), ctypes.c_void_p(cl_p),
                                          n_cl, float(radius_cutoff), int(metric), host_fpmode(fpmode),
                                          int(similarity_cutoff), int(n_member_cutoff), ctypes.c_void_p(out_l),
                                          ctypes.c_void_p(out_c), mem), "cnn_predict")
        del keep

    def mst_prim(self, radius_cutoff: float, metric: int = METRIC_EUCLIDEAN_REDUCED, fpmode: Optional[int] = None):
        """Maximum spanning forest edges (a, b, weight) in Prim's tree-queue order."""
        cap = max(int(self._n_points) - 1, 1)
        a = np.empty(cap, dtype=np.int64)
        b = np.empty(cap, dtype=np.int64)
        w = np.empty(cap, dtype=np.int64)
        ne = ctypes.c_int64()
        self._check(self._lib.cnn_mst_prim(self._h, float(radius_cutoff), int(metric), host_fpmode(fpmode),
                                           ctypes.c_void_p(a.ctypes.data), ctypes.c_void_p(b.ctypes.data),
                                           ctypes.c_void_p(w.ctypes.data), cap, ctypes.byref(ne)), "cnn_mst_prim")
        k = int(ne.value)
        return a[:k], b[:k], w[:k]

    def check_lists(self, a, b, c: int) -> bool:
        a = host_array(a, np.int32)
        b = host_array(b, np.int32)
        r = np.zeros(1, dtype=np.int32)
        self._check(self._lib.cnn_check_lists(self._h, ctypes.c_void_p(a.ctypes.data), a.shape[0],
                                              ctypes.c_void_p(b.ctypes.data), b.shape[0], int(c),
                                              ctypes.c_void_p(r.ctypes.data), MEM_HOST), "cnn_check_lists")
        return bool(r[0])


class NativeServer:
    """The library's job server (cnn_server_*): n_slots contexts with their
    own streams and worker threads, admission under a device-memory budget
    that bounds the bytes the workspaces really hold."""

    def __init__(self, device: int = 0, n_slots: int = 4, budget_bytes: int = 32 << 30):
        self._lib = load()
        h = ctypes.c_void_p()
        st = self._lib.cnn_server_create(ctypes.byref(h), int(device), int(n_slots), int(budget_bytes))
        if st != CNN_OK:
            raise CNNError(st, f"cnn_server_create(device={device}, n_slots={n_slots}) failed")
        self._h = h
        self._keep = {}  # job id -> the host arrays the job reads and writes

    def submit(self, points, radius_cutoff: float, similarity_cutoff: int, n_member_cutoff: int,
               member_cutoff: int = 2, max_clusters: Optional[int] = None, metric: int = METRIC_EUCLIDEAN_REDUCED,
               fpmode: Optional[int] = None, reserve_bytes: int = 0, labels=None) -> int:
        x = np.ascontiguousarray(points)
        if x.dtype not in (np.float64, np.float32):
            x = x.astype(np.float64)
        if x.ndim != 2:
            raise ValueError("points: a 2-D array [n_points, n_dim] is needed")
        n = x.shape[0]
        lab = np.empty(n, dtype=np.int64) if labels is None else labels
        if lab.dtype != np.int64 or lab.shape != (n,) or not lab.flags.c_contiguous:
            raise ValueError("labels: a C-contiguous int64 array of n_points entries is needed")
        job = cnn_job(points=x.ctypes.data, dtype=DTYPE_F64 if x.dtype == np.float64 else DTYPE_F32, n_points=n,
                      n_dim=x.shape[1], metric=int(metric), fpmode=host_fpmode(fpmode),
                      radius_cutoff=float(radius_cutoff), similarity_cutoff=int(similarity_cutoff),
                      n_member_cutoff=int(n_member_cutoff), member_cutoff=int(member_cutoff),
                      max_clusters=-1 if max_clusters is None else int(max_clusters),
                      labels=lab.ctypes.data, reserve_bytes=int(reserve_bytes))
        jid = ctypes.c_int64()
        st = self._lib.cnn_submit(self._h, ctypes.byref(job), ctypes.byref(jid))
        if st != CNN_OK:
            raise CNNError(st, "cnn_submit: invalid job")
        self._keep[jid.value] = (x, lab)
        return jid.value

    def poll(self, job_id: int) -> dict:
        info = cnn_job_info()
        st = self._lib.cnn_poll(self._h, int(job_id), ctypes.byref(info))
        if st != CNN_OK:
            raise CNNError(st, f"cnn_poll({job_id})")
        return info.as_dict()

    def wait(self, job_id: int, timeout_s: Optional[float] = None):
        """Blocks until the job is done; returns (labels, info).  A failed
        job raises CNNError with its message."""
        info = cnn_job_info()
        ns = -1 if timeout_s is None else int(timeout_s * 1e9)
        st = self._lib.cnn_wait(self._h, int(job_id), ns, ctypes.byref(info))
        if st != CNN_OK:
            raise CNNError(st, f"cnn_wait({job_id})")
        d = info.as_dict()
        if d["result"] != CNN_OK:
            buf = ctypes.create_string_buffer(512)
            self._lib.cnn_job_error(self._h, int(job_id), buf, 512)
            self._lib.cnn_job_release(self._h, int(job_id))
            self._keep.pop(job_id, None)
            err = CNNError(d["result"], f"job {job_id}: {buf.value.decode()}")
            err.info = d  # the job's times and slot
            raise err
        _, lab = self._keep.pop(job_id)
        self._lib.cnn_job_release(self._h, int(job_id))
        return lab, d

    def stats(self) -> dict:
        s = cnn_server_stats()
        st = self._lib.cnn_server_get_stats(self._h, ctypes.byref(s))
        if st != CNN_OK:
            raise CNNError(st, "cnn_server_get_stats")
        return s.as_dict()

    def close(self):
        if getattr(self, "_h", None):
            self._lib.cnn_server_destroy(self._h)
            self._h = None
            self._keep.clear()

    def __del__(self):  # pragma: no cover
        try:
            self.close()
        except Exception:
            pass


_tls = threading.local()


def default_context(device: int = 0) -> Context:
    """A per-thread, per-device context (contexts are not thread-safe)."""
    ctxs = getattr(_tls, "ctxs", None)
    if ctxs is None:
        ctxs = _tls.ctxs = {}
    ctx = ctxs.get(device)
    if ctx is None:
        ctx = ctxs[device] = Context(device)
    return ctx
