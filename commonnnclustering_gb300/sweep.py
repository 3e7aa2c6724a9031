"""Batched fits over (radius_cutoff, cnn_cutoff) pairs.

The reference scans parameter pairs with ``HierarchicalFitterRepeat``
(src/cnnclustering/_fit.pyx:1014-1187), running one complete fit per step
(:1131-1141) -- every neighbourhood recomputed each time.  ``sweep`` runs
the neighbour search once at the largest radius, derives each smaller
radius's neighbourhoods from it exactly, and fits every pair on the GPU.
Each returned labelling equals ``Clustering(points).fit(r, c,
member_cutoff, max_clusters)`` for that pair.
"""
from __future__ import annotations

from typing import Optional, Sequence

import numpy as np

from . import _abi
from ._types import InputDataGPUComponents, MetricGPUEuclidean, MetricGPUEuclideanReduced


def sweep(points, radius_cutoffs: Sequence[float], cnn_cutoffs: Sequence[int],
          member_cutoff: Optional[int] = None, max_clusters: Optional[int] = None,
          metric=None, fpmode: str = "auto", is_selfcounting: bool = True,
          context: Optional[_abi.Context] = None, labels_out=None):
    """Labels of every (radius, cnn_cutoff) pair, shape [n_radii, n_cuts, n].

    ``points`` is a numpy array or a CUDA tensor ([n, d], float64 or
    float32).  Radii are sorted ascending (the result follows that order).
    """
    metric = metric if metric is not None else MetricGPUEuclideanReduced()
    radii = sorted(float(r) for r in radius_cutoffs)
    adjusted = [metric.adjust_radius(r) for r in radii]
    cuts = []
    for c in cnn_cutoffs:
        c = int(c)
        cuts.append((c + 2, c + 1) if is_selfcounting else (c, c))
    if member_cutoff is None:
        member_cutoff = 2
    data = InputDataGPUComponents(points).data
    dev = 0
    if _abi.is_device_array(data):
        idx = getattr(getattr(data, "device", None), "index", None)
        dev = int(idx) if idx is not None else 0
    ctx = context if context is not None else _abi.default_context(dev)
    if _abi.is_device_array(data):
        st = _abi.current_torch_stream(ctx.device)
        if st is not None and st != ctx.stream:
            ctx.set_stream(st)
    ctx.set_points(data)
    code = _abi.METRIC_EUCLIDEAN if isinstance(metric, MetricGPUEuclidean) else _abi.METRIC_EUCLIDEAN_REDUCED
    fp = _abi.host_fpmode() if fpmode == "auto" else _abi.FP_FUSED if fpmode == "fused" else _abi.FP_SEPARATE
    return ctx.sweep(adjusted, cuts, member_cutoff=member_cutoff, max_clusters=max_clusters, metric=code,
                     fpmode=fp, labels_out=labels_out)


__all__ = ["sweep", "np"]
