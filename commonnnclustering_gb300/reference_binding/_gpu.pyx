# cython: language_level=3
# distutils: language = c++
# _gpu.pyx -- the GPU fitter as a module of cnnclustering itself (what a
# cnnclustering maintainer adds next to src/cnnclustering/_fit.pyx).  It
# binds libcnngpu.so through include/cnngpu.h and fits where
# FitterExtBFS._fit does (src/cnnclustering/_fit.pyx:408-491): the labels
# and consider arrays of the reference's Labels are written in place.
# Register it with the recipes as COMPONENT_NAME_TYPE_MAP["fitter"]["gpu"].
from libc.stdint cimport int32_t, int64_t, uint8_t

from cnnclustering._primitive_types cimport AINDEX, AVALUE, ABOOL
from cnnclustering._types cimport ClusterParameters, Labels, InputDataExtComponentsMemoryview
from cnnclustering._fit cimport FitterExtInterface

from cnnclustering._fit import Fitter

cdef extern from "cnngpu.h":
    ctypedef struct cnn_context:
        pass
    ctypedef enum cnn_status:
        CNN_OK
    ctypedef enum cnn_dtype:
        CNN_DTYPE_F64
    ctypedef enum cnn_memspace:
        CNN_MEM_HOST
    ctypedef enum cnn_metric:
        CNN_METRIC_EUCLIDEAN_REDUCED
    ctypedef enum cnn_fpmode:
        CNN_FP_SEPARATE
        CNN_FP_FUSED
    cnn_status cnn_create(cnn_context **out, int device, void *stream)
    cnn_status cnn_destroy(cnn_context *ctx)
    const char *cnn_last_error(const cnn_context *ctx)
    cnn_status cnn_set_points(cnn_context *ctx, const void *points, cnn_dtype dtype,
                              int64_t n_points, int32_t n_dim, cnn_memspace mem)
    cnn_status cnn_build_neighbours(cnn_context *ctx, double radius_cutoff,
                                    cnn_metric metric, cnn_fpmode fpmode)
    cnn_status cnn_fit(cnn_context *ctx, int64_t similarity_cutoff,
                       int64_t n_member_cutoff, int64_t current_start,
                       uint8_t *consider, int64_t *labels, int64_t n_points,
                       cnn_memspace mem)

cdef class FitterExtGPU(FitterExtInterface):
    """FitterExtBFS's place in a recipe, the fit on the GPU.  fpmode: the
    float64 accumulation of the reference build whose labels are to be
    reproduced (0 separate multiply and add, 1 fused)."""
    cdef cnn_context *_ctx
    cdef cnn_fpmode _fpmode
    cdef public object _neighbours_getter  # make_parameters reads the metric and self-counting

    def __cinit__(self, neighbours_getter, *args, fpmode=0, **kwargs):
        self._neighbours_getter = neighbours_getter
        self._fpmode = CNN_FP_FUSED if fpmode else CNN_FP_SEPARATE
        self._ctx = NULL

    def __dealloc__(self):
        if self._ctx != NULL:
            cnn_destroy(self._ctx)

    cdef cnn_context *_context(self) except NULL:
        if self._ctx == NULL and cnn_create(&self._ctx, 0, NULL) != CNN_OK:
            self._ctx = NULL
            raise RuntimeError("cnn_create: no usable CUDA device")
        return self._ctx

    def fit(self, InputDataExtComponentsMemoryview input_data, Labels labels,
            ClusterParameters cluster_params):
        cdef cnn_context *ctx = self._context()
        cdef AVALUE[:, ::1] x = input_data._data
        cdef AINDEX n = x.shape[0]
        if n == 0:
            return
        if (cnn_set_points(ctx, &x[0, 0], CNN_DTYPE_F64, n, <int32_t>x.shape[1], CNN_MEM_HOST) != CNN_OK or
                cnn_build_neighbours(ctx, cluster_params.radius_cutoff, CNN_METRIC_EUCLIDEAN_REDUCED, self._fpmode) != CNN_OK or
                cnn_fit(ctx, cluster_params.similarity_cutoff, cluster_params.n_member_cutoff,
                        cluster_params.current_start, <uint8_t *>&labels._consider[0],
                        <int64_t *>&labels._labels[0], n, CNN_MEM_HOST) != CNN_OK):
            raise RuntimeError(cnn_last_error(ctx).decode())


Fitter.register(FitterExtGPU)
