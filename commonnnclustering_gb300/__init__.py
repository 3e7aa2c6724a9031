"""GB300-native CommonNN clustering fit.

Drop-in GPU components for cnnclustering's fit hot path (radius neighbour
search, common-neighbour check, cluster assignment, sort_by_size), with
the compute in hand-written sm_103a CUDA kernels behind the C ABI of
``libcnngpu.so`` (include/cnngpu.h).  Quick start::

    from commonnnclustering_gb300 import Clustering
    clustering = Clustering(points)            # numpy array or CUDA tensor
    clustering.fit(radius_cutoff=0.3, cnn_cutoff=5, member_cutoff=10)
    clustering.labels
"""
from ._abi import CNNError, Context, default_context
from ._bundle import ReferenceIndices, bfs_leafs, isolate
from ._fit import Fitter, FitterGPU, FitterGPUNeighbourhoods, HierarchicalFitter, HierarchicalFitterRepeatGPU
from ._mst import HierarchicalFitterMSTPrimGPU, WeightedGraph
from ._predict import Predictor, PredictorFirstmatchGPU
from ._types import (ClusterParameters, DistanceGetterGPULookup, DistanceGetterGPUMetric, InputData,
                     InputDataGPUComponents, InputDataGPUDistances, InputDataGPUDistancesLinear,
                     InputDataGPUNeighbourhoods, Labels, MetricGPUEuclidean, MetricGPUEuclideanPeriodicReduced,
                     MetricGPUEuclideanReduced, MetricGPUPrecomputed, NeighboursGetterGPUGrid,
                     NeighboursGetterGPULookup, NeighboursGPU, QueueGPUUnionFind, SimilarityCheckerGPU)
from .cluster import Bundle, Clustering
from .report import Record, Summary
from .sweep import sweep

__version__ = "0.1.0"

__all__ = [
    "CNNError", "Context", "default_context", "Fitter", "FitterGPU", "FitterGPUNeighbourhoods",
    "ClusterParameters", "DistanceGetterGPUMetric", "InputData", "InputDataGPUComponents",
    "InputDataGPUNeighbourhoods", "Labels", "MetricGPUEuclidean", "MetricGPUEuclideanReduced",
    "NeighboursGetterGPUGrid", "NeighboursGetterGPULookup", "NeighboursGPU", "QueueGPUUnionFind",
    "SimilarityCheckerGPU", "Bundle", "Clustering", "Record", "Summary", "sweep", "HierarchicalFitter",
    "HierarchicalFitterRepeatGPU", "Predictor", "PredictorFirstmatchGPU", "ReferenceIndices", "bfs_leafs",
    "isolate", "DistanceGetterGPULookup", "InputDataGPUDistances", "InputDataGPUDistancesLinear",
    "MetricGPUEuclideanPeriodicReduced", "MetricGPUPrecomputed", "HierarchicalFitterMSTPrimGPU", "WeightedGraph",
]
