/*
 * cnngpu.h -- C ABI of the GB300 CommonNN fit library (libcnngpu.so).
 *
 * The library replaces the hot path of cnnclustering 0.5.0's
 * Clustering.fit: radius neighbour search, the common-neighbour similarity
 * check and the BFS cluster growth, plus Labels.sort_by_size.  All entry
 * points take plain pointers and sizes; arrays may live on the host or on
 * the device (cnn_memspace).  Nothing here depends on torch.
 *
 * Reference interfaces each entry point stands in for (paths relative to
 * the reference project root):
 *
 *   cnn_set_points        InputDataExtComponentsMemoryview.__cinit__
 *                           src/cnnclustering/_types.pyx:1040-1048
 *   cnn_build_neighbours  NeighboursGetterExtBruteForce._get for every point
 *                           src/cnnclustering/_types.pyx:1692-1710 with
 *                           MetricExtEuclideanReduced._calc_distance
 *                           :2253-2267 / MetricExtEuclidean :2173-2187
 *   cnn_set_neighbours    InputDataExtNeighbourhoodsMemoryview +
 *                           NeighboursGetterExtLookup._get
 *                           src/cnnclustering/_types.pyx:1159-1171, 1806-1817
 *   cnn_get_neighbours    the per-point lists those getters return, as CSR
 *   cnn_fit               FitterExtBFS._fit (with _enough and _check)
 *                           src/cnnclustering/_fit.pyx:408-491,
 *                           _types.pyx:1408-1411, 2580-2610, 2654-2706
 *   cnn_sort_by_size      Labels.sort_by_size
 *                           src/cnnclustering/_types.pyx:212-286
 *   cnn_fit_fresh         Clustering.fit with fresh labels + sort_by_size
 *                           src/cnnclustering/cluster.pyx:316-364
 *   cnn_check_lists       SimilarityCheckerExtScreensorted._check
 *                           src/cnnclustering/_types.pyx:2654-2706
 *
 * Threading: a context is not thread-safe; use one per host thread.  All
 * device work of a context runs on its stream, in order.  Calls that
 * return host-visible results synchronise that stream.
 *
 * Errors: every call returns a cnn_status; cnn_last_error() gives the
 * message of the last failure on that context.  No C++ exception crosses
 * this boundary.
 */
#ifndef CNNGPU_H
#define CNNGPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define CNN_API __attribute__((visibility("default")))
#else
#define CNN_API
#endif

#define CNN_ABI_VERSION 2

typedef struct cnn_context cnn_context;

typedef enum cnn_status {
    CNN_OK = 0,
    CNN_ERR_INVALID_ARG = 1,
    CNN_ERR_OOM = 2,
    CNN_ERR_CUDA = 3,
    CNN_ERR_TIMEOUT = 4,
    CNN_ERR_UNSUPPORTED = 5,
    CNN_ERR_STATE = 6
} cnn_status;

/* Which distance the getter compares with radius_cutoff. */
typedef enum cnn_metric {
    CNN_METRIC_EUCLIDEAN_REDUCED = 0, /* sum of squares <= radius_cutoff (= r*r) */
    CNN_METRIC_EUCLIDEAN = 1,         /* sqrt(sum of squares) <= radius_cutoff (= r) */
    CNN_METRIC_PRECOMPUTED = 2,       /* stored distance <= radius_cutoff (= r), cnn_set_distances
                                         (MetricExtPrecomputed, _types.pyx:2108-2127, and the
                                         lookup getter, :2019-2037) */
    CNN_METRIC_EUCLIDEAN_PERIODIC_REDUCED = 3 /* sum of squared minimum-image differences
                                         <= radius_cutoff (= r*r), bounds from
                                         cnn_set_periodic_bounds (_types.pyx:2290-2348) */
} cnn_metric;

/* Layout of precomputed distances (cnn_set_distances). */
typedef enum cnn_dist_layout {
    CNN_DIST_SQUARE = 0, /* [n][n] row-major: the "distances" recipe's
                            InputDataExtComponentsMemoryview (_types.pyx:1034-1062) */
    CNN_DIST_LINEAR = 1  /* upper triangle by rows, n(n-1)/2 values:
                            InputDataExtDistancesLinearMemoryview (_types.pyx:1112-1150) */
} cnn_dist_layout;

/* How each term of the float64 distance sum is accumulated:
 * SEPARATE: total = total + (t*t), two roundings (reference built for
 *           x86-64 without FMA);
 * FUSED:    total = fma(t, t, total), one rounding (reference built with
 *           FMA contraction, e.g. GCC's default on aarch64). */
typedef enum cnn_fpmode {
    CNN_FP_SEPARATE = 0,
    CNN_FP_FUSED = 1
} cnn_fpmode;

typedef enum cnn_dtype {
    CNN_DTYPE_F64 = 0,
    CNN_DTYPE_F32 = 1 /* widened to float64 exactly before any compare */
} cnn_dtype;

typedef enum cnn_memspace {
    CNN_MEM_HOST = 0,
    CNN_MEM_DEVICE = 1
} cnn_memspace;

/* Per-context counters and stage times of the most recent calls.  Times
 * are milliseconds between CUDA events recorded on the context stream
 * (0 when timing is off). */
typedef struct cnn_stats {
    int64_t n_points;
    int64_t n_nonzero;        /* neighbour pairs stored (self included) */
    int64_t n_nodes;          /* core points with consider == 1 */
    int64_t n_checks;         /* similarity checks executed */
    int64_t n_accepted;       /* checks that passed */
    int64_t n_exact;          /* candidate pairs decided in float64 */
    int64_t n_candidates;     /* candidate pairs tested by the search */
    int64_t n_clusters;       /* clusters found by the last fit */
    int32_t search_kind;      /* 1 = cell grid (d <= 3), 2 = tiled all-pairs float32,
                                 3 = tensor-core Gram (d >= 16), 4 = precomputed distances,
                                 0 = precomputed neighbourhoods */
    int32_t filter_enabled;   /* 1 when the float32 prefilter was usable */
    double filter_band;       /* half-width of the float64 recheck band on d^2 */
    float ms_bbox, ms_cells, ms_count, ms_scan, ms_fill;   /* neighbour build */
    float ms_nodes, ms_check, ms_label;                    /* fit */
    float ms_sort;                                         /* sort_by_size */
    int64_t n_launches;       /* kernels launched by this context since creation */
    float ms_gram;            /* tensor-core distance kernel alone (n_dim >= 16) */
    float max_abs_err;        /* max |d^2 tensor-core - d^2 float64| over rechecked pairs */
    int32_t intersection;     /* strategy of the last fit: CNN_INTERSECT_MERGE or _BITSET */
    int32_t tuned;            /* 1: the last fit timed both strategies for the tuner */
    float tune_ms_merge;      /* those times (search + fit), 0 otherwise */
    float tune_ms_bitset;
    float ms_weights;         /* cnn_mst_prim: the pair weights (full counts) */
    int32_t graphs;           /* cnn_sweep / cnn_sweep_pairs: CUDA graphs the fits ran as
                                 (0: launched one by one) */
    int64_t graph_nodes;      /* kernels, copies and memsets in those graphs */
    float ms_graph_build;     /* host time to capture and instantiate them */
} cnn_stats;

CNN_API int cnn_abi_version(void);

/* Which neighbour search cnn_build_neighbours runs (a preference: a search
 * that does not apply to the points or the metric falls back to the
 * automatic choice).  AUTO: cell grid for n_dim <= 3, tensor-core Gram
 * search for n_dim >= 16, tiled all-pairs float32 otherwise; ALL_PAIRS: the
 * tiled all-pairs float32 search with the float64 band for any n_dim (the
 * plain GPU path the others are measured against).  The neighbour sets are
 * the same whichever runs. */
typedef enum cnn_search {
    CNN_SEARCH_AUTO = 0,
    CNN_SEARCH_GRID = 1,
    CNN_SEARCH_ALL_PAIRS = 2,
    CNN_SEARCH_TENSOR = 3
} cnn_search;

/* How the common-neighbour counts of cell-grid graphs (n_dim <= 3) are
 * taken.  MERGE: sorted neighbour lists, warp-wide merge with early exit;
 * BITSET: rows stored as bit masks over each cell's stencil candidates,
 * counts by AND + popcount of the overlapping runs; AUTO (default): the
 * library's tuner times both on the first fit of each workload profile
 * (point count and candidates per point) and keeps the faster for later
 * graphs of that profile (per process).  Results are identical. */
typedef enum cnn_intersection {
    CNN_INTERSECT_AUTO = 0,
    CNN_INTERSECT_MERGE = 1,
    CNN_INTERSECT_BITSET = 2
} cnn_intersection;

/* Create a context on `device`.  `stream` is a cudaStream_t (may be NULL:
 * the context creates its own non-blocking stream). */
CNN_API cnn_status cnn_create(cnn_context **out, int device, void *stream);
CNN_API cnn_status cnn_destroy(cnn_context *ctx);
CNN_API cnn_status cnn_set_stream(cnn_context *ctx, void *stream);
CNN_API const char *cnn_last_error(const cnn_context *ctx);
CNN_API cnn_status cnn_set_timing(cnn_context *ctx, int enabled);
CNN_API cnn_status cnn_get_stats(const cnn_context *ctx, cnn_stats *out);

/* Limit, in nanoseconds, of every bounded wait inside the context's
 * pipelined kernels (the tensor-core search's barrier waits); <= 0 restores
 * the default of 2 s.  A wait that runs out stops the kernel cleanly (its
 * copies drained, its tensor memory freed) and the call returns
 * CNN_ERR_TIMEOUT; the context stays usable.  No reference counterpart: a
 * testing and watchdog knob. */
CNN_API cnn_status cnn_set_wait_limit(cnn_context *ctx, int64_t limit_ns);

/* The search preference of the following cnn_build_neighbours calls (see
 * cnn_search); no reference counterpart: the reference has one brute-force
 * getter. */
CNN_API cnn_status cnn_set_search(cnn_context *ctx, cnn_search search);

/* The intersection strategy of the following cnn_build_neighbours +
 * cnn_fit calls (see cnn_intersection); no reference counterpart. */
CNN_API cnn_status cnn_set_intersection(cnn_context *ctx, cnn_intersection intersection);

/* Points, row-major [n_points x n_dim].  Device arrays are used in place
 * (they must stay alive and unchanged until the next cnn_set_points);
 * host arrays are copied. */
CNN_API cnn_status cnn_set_points(cnn_context *ctx, const void *points, cnn_dtype dtype,
                                  int64_t n_points, int32_t n_dim, cnn_memspace mem);

/* Radius neighbourhoods of every point (self included) for the adjusted
 * radius_cutoff the reference's getter compares with (r*r for the reduced
 * metric, r for the Euclidean metric).  The graph stays on the device. */
CNN_API cnn_status cnn_build_neighbours(cnn_context *ctx, double radius_cutoff,
                                        cnn_metric metric, cnn_fpmode fpmode);

/* Precomputed neighbourhoods in CSR form (offsets int64[n+1], indices
 * int32[nnz]); rows are sorted on the device, so any order is accepted.
 * Replaces the points of the context. */
CNN_API cnn_status cnn_set_neighbours(cnn_context *ctx, const int64_t *offsets,
                                      const int32_t *indices, int64_t n_points,
                                      cnn_memspace mem);

/* Number of stored neighbour pairs of the current graph.  After a cell-grid
 * cnn_build_neighbours the count is read back here (a stream sync) or by
 * cnn_get_stats: the build itself does not wait for it. */
CNN_API cnn_status cnn_neighbour_count(cnn_context *ctx, int64_t *nnz);

/* The current graph as CSR in point-index order with ascending rows:
 * offsets int64[n+1], indices int32[nnz].  A cell-grid cnn_build_neighbours
 * leaves each row in the slot the search wrote it to (cnn_fit walks them
 * there); the first call here makes the CSR (a scan and a compaction). */
CNN_API cnn_status cnn_get_neighbours(cnn_context *ctx, int64_t *offsets, int32_t *indices,
                                      cnn_memspace mem);

/* Cluster the current graph.  Semantics of FitterExtBFS._fit: points with
 * more than n_member_cutoff neighbours and consider == 1 are nodes; two
 * nodes that are neighbours and share at least similarity_cutoff
 * neighbours are joined; each connected set of nodes gets one label,
 * numbered from current_start in the order of its lowest point index.
 * labels[] of nodes and consider[] of every visited point are written in
 * place as the reference does; other entries are left as they are.
 * n_points is the length of labels[] and consider[]: it must equal the
 * point count of the current graph (the reference writes exactly
 * input_data.n_points labels), else CNN_ERR_INVALID_ARG is returned
 * before anything is copied or launched. */
CNN_API cnn_status cnn_fit(cnn_context *ctx, int64_t similarity_cutoff, int64_t n_member_cutoff,
                           int64_t current_start, uint8_t *consider, int64_t *labels,
                           int64_t n_points, cnn_memspace mem);

/* Clustering.fit from fresh labels (src/cnnclustering/cluster.pyx:316-364
 * with no labels yet: labels 0, consider 1, current_start 1), then, when
 * sort != 0, Labels.sort_by_size(member_cutoff, max_clusters) -- in one
 * call: the fresh arrays are made on the device and the sort reads the
 * cluster count there, so nothing is copied in and only labels[n] (and
 * consider[n], all 0 afterwards, if not NULL) come back.  Same labels as
 * cnn_fit + cnn_sort_by_size on fresh arrays.  n_points as for cnn_fit. */
CNN_API cnn_status cnn_fit_fresh(cnn_context *ctx, int64_t similarity_cutoff, int64_t n_member_cutoff,
                                 int32_t sort, int64_t member_cutoff, int64_t max_clusters,
                                 int64_t *labels, uint8_t *consider, int64_t n_points,
                                 cnn_memspace mem);

/* A counter of the graphs this context has held: it changes whenever the
 * points, distances or neighbourhoods are replaced or a neighbour graph is
 * built (cnn_set_points, cnn_set_distances, cnn_set_neighbours,
 * cnn_build_neighbours, and the calls that build a graph on their own:
 * cnn_sweep, cnn_sweep_pairs, cnn_predict, cnn_mst_prim).  A caller that
 * keeps a graph for later fits compares it to tell whether the context still
 * holds that graph. */
CNN_API cnn_status cnn_graph_generation(const cnn_context *ctx, int64_t *generation);

/* Labels.sort_by_size on labels[n] in place: renumber clusters by size
 * (descending, ties by first occurrence), zero clusters with fewer than
 * member_cutoff members and all clusters after the first max_clusters
 * (max_clusters < 0: no limit).  Label 0 stays 0. */
CNN_API cnn_status cnn_sort_by_size(cnn_context *ctx, int64_t *labels, int64_t n,
                                    int64_t member_cutoff, int64_t max_clusters,
                                    cnn_memspace mem);

/* Similarity check of two ascending member lists: *result = 1 when they
 * share at least c members (c == 0: always 1; an empty list: 0). */
CNN_API cnn_status cnn_check_lists(cnn_context *ctx, const int32_t *a, int64_t na,
                                   const int32_t *b, int64_t nb, int64_t c, int32_t *result,
                                   cnn_memspace mem);

/* Batched fits over n_radii x n_cuts (radius, cut) pairs on the current
 * points -- the scan HierarchicalFitterRepeat performs
 * (src/cnnclustering/_fit.pyx:1014-1187, one full fit per step at
 * :1131-1141) -- with the neighbour search run once at the largest radius.
 * radius_cutoffs: adjusted cutoffs, ascending (<= 16).  Cut j is
 * (similarity_cutoffs[j], n_member_cutoffs[j]) as make_parameters gives them.
 * Every pair is fitted from fresh labels (current_start 1) and sorted with
 * (member_cutoff, max_clusters < 0: no limit); labels_out[(k * n_cuts + j) *
 * n_points + i] then equals what cnn_fit + cnn_sort_by_size give at radius
 * k and cut j.  The context keeps the largest-radius graph afterwards.
 * The fits (with their sorts) enqueue no host round trip and run as one
 * CUDA graph captured on the context's stream (kept by the context and
 * updated for the next sweep of the same shape); CNN_SWEEP_GRAPH=0 in the
 * environment at cnn_create runs them as plain launches.  cnn_stats.graphs,
 * graph_nodes and ms_graph_build report it. */
CNN_API cnn_status cnn_sweep(cnn_context *ctx, const double *radius_cutoffs, int32_t n_radii,
                             const int64_t *similarity_cutoffs, const int64_t *n_member_cutoffs,
                             int32_t n_cuts, cnn_metric metric, cnn_fpmode fpmode,
                             int64_t member_cutoff, int64_t max_clusters, int64_t *labels_out,
                             cnn_memspace mem);

/* Precomputed distances instead of points (layout above); device arrays
 * are used in place.  The neighbour graph is then built with
 * cnn_build_neighbours(ctx, radius_cutoff, CNN_METRIC_PRECOMPUTED, ...):
 * N(i) = {j : distance(i, j) <= radius_cutoff}, the diagonal of the linear
 * layout being 0, as NeighboursGetterExtBruteForce._get
 * (src/cnnclustering/_types.pyx:1692-1710) collects them. */
CNN_API cnn_status cnn_set_distances(cnn_context *ctx, const double *distances, cnn_dist_layout layout,
                                     int64_t n_points, cnn_memspace mem);

/* Box lengths per dimension for CNN_METRIC_EUCLIDEAN_PERIODIC_REDUCED
 * (MetricExtEuclideanPeriodicReduced(bounds), _types.pyx:2290-2348): per
 * dimension d = |a - b|, and when bound > 0, d = fmod(d, bound) and
 * d = bound - d if d > bound / 2.  Host array of n_dim values. */
CNN_API cnn_status cnn_set_periodic_bounds(cnn_context *ctx, const double *bounds, int32_t n_dim);

/* The step list of HierarchicalFitterRepeat._fit
 * (src/cnnclustering/_fit.pyx:1131-1141): step i fits (radius_cutoffs[i],
 * similarity_cutoffs[i], n_member_cutoffs[i]) from fresh labels
 * (current_start 1) and, when sort != 0, sorts with (member_cutoff,
 * max_clusters < 0: no limit), as :1143-1144 do.  Steps may come in any
 * order and repeat; labels_out[i * n_points + p] equals the separate fit of
 * step i.  Distinct radii share largest-radius searches (16 radii per
 * search); fits are seeded along the (radius, cut) lattice as in cnn_sweep. */
CNN_API cnn_status cnn_sweep_pairs(cnn_context *ctx, const double *radius_cutoffs,
                                   const int64_t *similarity_cutoffs, const int64_t *n_member_cutoffs,
                                   int32_t n_steps, cnn_metric metric, cnn_fpmode fpmode, int32_t sort,
                                   int64_t member_cutoff, int64_t max_clusters, int64_t *labels_out,
                                   cnn_memspace mem);

/* Labels for other points from the clustering of the current points:
 * PredictorFirstmatch.predict (src/cnnclustering/_fit.pyx:1235-1291) with
 * NeighboursGetter.get_other (_types.pyx:1712-1731).  labels: the current
 * points' labels [n_points]; clusters: the consider set (labels that may be
 * handed out; any order).  radius_cutoff and the cutoffs as
 * Predictor.make_parameters gives them.  For every other point p with
 * other_consider[p] == 1 and more than n_member_cutoff neighbours among the
 * current points, the first neighbour (in index order) whose label is in
 * the set, whose own neighbourhood has more than n_member_cutoff members and
 * that shares at least similarity_cutoff neighbours with p (0: always, < 0:
 * never) gives p its label, and other_consider[p] becomes 0; other points
 * keep their label.  other_points, labels, clusters, other_labels and
 * other_consider all live in `mem`.  The current points' graph at this
 * radius stays in the context afterwards. */
CNN_API cnn_status cnn_predict(cnn_context *ctx, const void *other_points, cnn_dtype dtype, int64_t n_other,
                               int32_t n_dim, const int64_t *labels, const int64_t *clusters, int64_t n_clusters,
                               double radius_cutoff, cnn_metric metric, cnn_fpmode fpmode,
                               int64_t similarity_cutoff, int64_t n_member_cutoff, int64_t *other_labels,
                               uint8_t *other_consider, cnn_memspace mem);

/* Maximum spanning forest of the common-neighbour graph, as
 * HierarchicalFitterMSTPrim._fit builds it (src/cnnclustering/_fit.pyx:
 * 820-899): neighbourhoods at radius_cutoff (as compared: r*r for the
 * reduced metric), every pair weighted by its full common-neighbour count
 * (_types.pyx:2708-2753), Prim's algorithm from every unvisited point in
 * index order with the reference's max-heap order (-weight, (a, b)).
 * Output host arrays (capacity >= n_points - 1): the tree edges (a, b,
 * weight) in the order the reference's tree queue pops them (weight
 * descending, then a, then b).  The neighbour graph stays in the context. */
CNN_API cnn_status cnn_mst_prim(cnn_context *ctx, double radius_cutoff, cnn_metric metric, cnn_fpmode fpmode,
                                int64_t *edges_a, int64_t *edges_b, int64_t *weights, int64_t capacity,
                                int64_t *n_edges);

/* ---------------------------------------------------------------------
 * Fit without device memory allocation.  This entry point has no
 * counterpart in the reference.
 *
 * For callers that must not allocate device memory while they run: a
 * serving loop whose memory budget is fixed at start-up, a plug-in inside
 * a framework whose caching allocator already holds the free memory, or a
 * latency-critical loop that cannot afford cudaMalloc/cudaFree (either may
 * synchronise the whole device).  The caller passes inputs and outputs;
 * the only other memory used is a fixed scratch block compiled into the
 * library (about 1.9 MB per GPU, held by every GPU that loads the library
 * until the process exits).
 *
 * All pointers are device pointers.  The graph must be what
 * cnn_get_neighbours produces: offsets int64[n_points + 1] from 0, rows of
 * `indices` strictly ascending with values in [0, n_points), and the
 * neighbour relation symmetric; for such a graph the labels equal those of
 * cnn_set_neighbours + cnn_fit.  The offsets and rows are checked on the GPU
 * before they are used; a graph that fails (decreasing offsets, an index out
 * of range, a row out of order) is not fitted and labels and consider stay
 * as they were -- a fitted call always leaves every consider entry 0.
 * Symmetry is not checked: an asymmetric graph gives undefined labels.
 * Work is queued on `stream` (a cudaStream_t, NULL = legacy default stream)
 * on the current device; the call returns before it finishes.
 *
 * Limits and sharing: n_points above CNN_NOALLOC_MAX_POINTS returns
 * CNN_ERR_INVALID_ARG without touching the GPU; a CUDA error already
 * pending when the call starts returns CNN_ERR_CUDA and is left pending.
 * All calls share the one scratch block, so calls whose GPU work overlaps
 * (other streams, other host threads) race and must be serialised by the
 * caller.  The first call on a device looks up the scratch block's device
 * address once (with that device current); make that first call before any
 * stream capture, and do not call this entry point again after
 * cudaDeviceReset in the same process. */
#define CNN_NOALLOC_MAX_POINTS 65536

CNN_API cnn_status cnn_fit_csr_noalloc(const int64_t *offsets, const int32_t *indices,
                                       int64_t n_points, int64_t similarity_cutoff,
                                       int64_t n_member_cutoff, int64_t current_start,
                                       uint8_t *consider, int64_t *labels, void *stream);

/* ---- Served job stream (continuous batching) ------------------------------
 * A server runs many Clustering.fit jobs concurrently on one device
 * (src/cnnclustering/cluster.pyx:256-392 per job, fresh labels): n_slots
 * contexts, each with its own stream and workspace kept between jobs, and
 * one host worker thread per slot.  cnn_submit queues a job and returns at
 * once; jobs start oldest first as slots free up, and later jobs pass one
 * that does not fit the memory budget yet (up to 64 times, then it waits at
 * the head until it fits).  Each job's labels equal cnn_set_points +
 * cnn_build_neighbours + cnn_fit (fresh labels, current_start 1) +
 * cnn_sort_by_size run alone.
 *
 * Memory: the device bytes the slots' workspaces hold never exceed
 * budget_bytes.  A running job holds a reservation its context cannot grow
 * past (checked before any allocation): what its slot already holds plus
 * the job's need; idle slots count with what they hold and are released
 * when a waiting job needs the room.  The need starts from
 * job->reserve_bytes (or an estimate from n_points and n_dim when 0),
 * scaled by what earlier jobs of the same kind (n_dim <= 3, < 16, >= 16)
 * needed beyond their estimates.  A job that outgrows its reservation is
 * queued again at the head with at least twice the need
 * (cnn_job_info.attempts counts the starts); once the need reaches the
 * budget the job runs alone, and fails with CNN_ERR_OOM only if the whole
 * budget is too small.
 *
 * Host buffers: points and labels are host memory owned by the caller and
 * must stay valid until the job is done; labels[n_points] is written by the
 * job.  Threads: every entry point may be called from any thread. */
typedef struct cnn_server cnn_server;

typedef struct cnn_job {
    const void *points;          /* host, row-major [n_points x n_dim] */
    cnn_dtype dtype;
    int64_t n_points;
    int32_t n_dim;
    cnn_metric metric;           /* EUCLIDEAN_REDUCED or EUCLIDEAN */
    cnn_fpmode fpmode;
    double radius_cutoff;        /* adjusted, as make_parameters gives it */
    int64_t similarity_cutoff;   /* as make_parameters gives them */
    int64_t n_member_cutoff;
    int64_t member_cutoff;       /* sort_by_size; < 0: labels left unsorted */
    int64_t max_clusters;        /* sort_by_size; < 0: no limit */
    int64_t *labels;             /* host [n_points], written when the job is done */
    int64_t reserve_bytes;       /* first reservation; 0: estimated */
} cnn_job;

typedef enum cnn_job_state {
    CNN_JOB_QUEUED = 0,
    CNN_JOB_RUNNING = 1,
    CNN_JOB_DONE = 2
} cnn_job_state;

typedef struct cnn_job_info {
    cnn_job_state state;
    cnn_status result;           /* of a done job */
    int32_t slot;                /* of the last start, -1 before */
    int32_t attempts;            /* starts: 2 when the job outgrew its first reservation */
    int64_t reserved_bytes;      /* reservation of the last start */
    double t_submit, t_start, t_done;  /* seconds since cnn_server_create */
} cnn_job_info;

typedef struct cnn_server_stats {
    int64_t submitted, done, failed;
    int64_t requeued;            /* jobs that outgrew their first reservation */
    int64_t released;            /* idle workspaces released to make room */
    int32_t running, queued, max_running;
    int64_t budget_bytes;
    int64_t committed_bytes;     /* running reservations + idle holdings, now */
    int64_t held_bytes;          /* device bytes the slots' workspaces hold, now */
    int64_t peak_held_bytes;     /* largest held_bytes seen (at job ends and here) */
} cnn_server_stats;

CNN_API cnn_status cnn_server_create(cnn_server **out, int device, int32_t n_slots,
                                     int64_t budget_bytes);
/* Waits for every submitted job, then frees the server. */
CNN_API cnn_status cnn_server_destroy(cnn_server *srv);
CNN_API cnn_status cnn_submit(cnn_server *srv, const cnn_job *job, int64_t *job_id);
CNN_API cnn_status cnn_poll(cnn_server *srv, int64_t job_id, cnn_job_info *info);
/* Blocks until the job is done (timeout_ns < 0: no limit); CNN_ERR_TIMEOUT
 * when the limit passes first (info then holds the current state). */
CNN_API cnn_status cnn_wait(cnn_server *srv, int64_t job_id, int64_t timeout_ns,
                            cnn_job_info *info);
/* The message of a failed job (empty when it succeeded). */
CNN_API cnn_status cnn_job_error(cnn_server *srv, int64_t job_id, char *buf, int64_t size);
/* Forgets a done job (its id is invalid afterwards). */
CNN_API cnn_status cnn_job_release(cnn_server *srv, int64_t job_id);
CNN_API cnn_status cnn_server_get_stats(cnn_server *srv, cnn_server_stats *out);

#ifdef __cplusplus
}
#endif

#endif /* CNNGPU_H */
