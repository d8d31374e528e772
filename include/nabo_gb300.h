/* nabo_gb300.h -- C ABI of the GB300 kNN search library.
 *
 * A drop-in for the k-nearest-neighbour path of libnabo 1.1.2
 * (Nabo::NearestNeighbourSearch<T>, nabo/nabo.h:257-441): the same build
 * and search semantics, run on one NVIDIA GB300 (sm_103a). Plain pointers
 * and sizes only; no C++ or framework types cross this boundary.
 *
 * Matrices use the reference's Eigen layout: a cloud or a query set is
 * `rows x n`, column-major, one point per column, consecutive points
 * `colStride` elements apart (colStride >= rows). Results are `k x nq`
 * column-major: indices (int32) and squared distances (T) of the k
 * neighbours of query i are at [i*k, i*k + k), ascending by distance.
 * Unfound slots hold index -1 and distance +inf (nabo/nabo.h:216-226).
 *
 * Error handling: every function returns 0 on success or a NABO_CUDA_ERR_*
 * code; nabo_cuda_last_error() returns the calling thread's message. The
 * argument checks and their messages are those of the reference
 * (nabo/nabo.cpp:102-131, :134-179; nabo/kdtree_cpu.cpp:234-251), which
 * the C++ front end rethrows as exceptions.
 */
#ifndef NABO_GB300_H
#define NABO_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define NABO_GB300_VERSION "0.1.0"
#define NABO_GB300_REFERENCE_VERSION "1.1.2"

/* Status codes. */
#define NABO_CUDA_OK 0
#define NABO_CUDA_ERR_ARGUMENT 1    /* the reference throws Nabo::runtime_error */
#define NABO_CUDA_ERR_CUDA 2        /* CUDA runtime error (no GPU, out of memory, ...) */
#define NABO_CUDA_ERR_UNSUPPORTED 3 /* valid for the reference, outside this library's limits */
#define NABO_CUDA_ERR_INTERNAL 4

/* Scalar types. */
#define NABO_CUDA_FLOAT32 0
#define NABO_CUDA_FLOAT64 1

/* Search types: the reference's enum (nabo/nabo.h:290-299) extended with
 * the CUDA types, placed after BRUTE_FORCE_CL. Only the CUDA types are
 * implemented here; the CPU and OpenCL types stay in libnabo. */
#define NABO_SEARCH_BRUTE_FORCE 0
#define NABO_SEARCH_KDTREE_LINEAR_HEAP 1
#define NABO_SEARCH_KDTREE_TREE_HEAP 2
#define NABO_SEARCH_KDTREE_CL_PT_IN_NODES 3
#define NABO_SEARCH_KDTREE_CL_PT_IN_LEAVES 4
#define NABO_SEARCH_BRUTE_FORCE_CL 5
#define NABO_SEARCH_KDTREE_CUDA 6
#define NABO_SEARCH_BRUTE_FORCE_CUDA 7
#define NABO_SEARCH_TYPE_COUNT 8

/* Creation flags (nabo/nabo.h:302-305) and search flags (:308-312). */
#define NABO_TOUCH_STATISTICS 1u
#define NABO_ALLOW_SELF_MATCH 1u
#define NABO_SORT_RESULTS 2u

/* Additional parameters, the typed form of Nabo::Parameters
 * (nabo/nabo.h:231-254). Initialise with nabo_cuda_params_init(). */
typedef struct nabo_cuda_params {
  uint32_t struct_size;   /* sizeof(nabo_cuda_params) */
  uint32_t bucketSize;    /* "bucketSize", default 8 (nabo/kdtree_cpu.cpp:230) */
  int32_t queryOrdering;  /* 1 (default): reorder the queries of large
                             searches along a Morton curve (by leaf for more
                             than 3 dimensions): from about 2^18 queries at
                             k = 10 in 3-D, fewer for larger k or more
                             dimensions; smaller searches keep the given
                             order, the sort costing more than it saves
                             there; 0: keep the given order */
  int32_t traversal;      /* kd-tree search order. 0 (default) or 1: the
                             reference's visit order (nabo/kdtree_cpu.cpp:
                             367-447), one query per thread; 2: the warp
                             packet -- the 32 queries of a warp walk one node
                             sequence, each pruning for itself -- for exact
                             searches (epsilon 0) without TOUCH_STATISTICS
                             and k <= 32 (larger k use the reference order) */
  int32_t threadsPerBlock; /* batched search kernel block size: 32, 64 or 128
                              (0 = 128); chosen by the autotuner */
  int32_t pipelineChunks;  /* host-buffer searches of 2^18 queries or more
                              with page-locked result buffers: searched in
                              this many chunks of shrinking size whose
                              downloads overlap the next chunk's search
                              (0 = default, 1 = one search then one
                              download; at most 64); for a batch, the cloud
                              groups of nabo_cuda_batch_run_host */
  int32_t splitRule;       /* kd-tree split. 0 (default): the reference's
                              sliding midpoint (nabo/kdtree_cpu.cpp:134-190),
                              the reference's tree node for node; 1: the
                              median of the cell's widest dimension -- a
                              balanced tree with the same node layout (the
                              balanced trees of nabo/kdtree_opencl.cpp:474-514
                              with buckets), an autotuner candidate for
                              callers that need neither the reference's tree
                              nor its TOUCH_STATISTICS counts (refused with
                              NABO_TOUCH_STATISTICS); exact results */
  int32_t lanesPerQuery;   /* batched search with k <= 32: 1 (0 = default):
                              one thread per query; 8: a group of 8 lanes
                              per query (one traversal, the top-k spread
                              over the group's registers); chosen by the
                              autotuner, same results */
} nabo_cuda_params;

typedef struct nabo_cuda_search nabo_cuda_search; /* opaque */

/* Fills `p` with the defaults. */
void nabo_cuda_params_init(nabo_cuda_params* p);

/* Builds a search object on the current CUDA device.
 * Replaces NearestNeighbourSearch<T>::create (nabo/nabo.h:360,
 * nabo/nabo.cpp:134-155) for the CUDA search types, and the constructors
 * KDTreeUnbalancedPtInLeavesImplicitBoundsStackOpt (nabo/kdtree_cpu.cpp:
 * 227-272) and BruteForceSearch (nabo/brute_force_cpu.cpp:44-60).
 * `cloud` is HOST memory; it is copied to the device and not referenced
 * after the call returns. `dim` is clamped to `rows` as in the reference.
 * `params` may be NULL. */
int nabo_cuda_create(int dtype, const void* cloud, int rows, int64_t n, int64_t colStride, int dim, int searchType,
                     unsigned creationFlags, const nabo_cuda_params* params, nabo_cuda_search** out);

/* Same, with `cloud` in DEVICE memory (read during the call only). */
int nabo_cuda_create_device(int dtype, const void* cloud, int rows, int64_t n, int64_t colStride, int dim,
                            int searchType, unsigned creationFlags, const nabo_cuda_params* params,
                            nabo_cuda_search** out);

/* Releases the object and its device memory. Accepts NULL.
 * Replaces the virtual destructor (nabo/nabo.h:427). */
int nabo_cuda_destroy(nabo_cuda_search* s);

/* k-nearest-neighbour search with HOST buffers.
 * Replaces NearestNeighbourSearch<T>::knn (nabo/nabo.h:338) when
 * maxRadii == NULL (radius = maxRadius for every query) and the per-query
 * radii overload (nabo/nabo.h:351) when maxRadii != NULL (nq values).
 * query: qRows x nq column-major, column stride qStride (>= qRows).
 * indices: k*nq int32; dists2: k*nq of the object's scalar type.
 * touched (may be NULL): receives the TOUCH_STATISTICS count (points
 * examined in visited leaves; nq*n for brute force) when the object was
 * created with NABO_TOUCH_STATISTICS, else 0. Neighbours at equal distance
 * are ranked by index (the lower index first, whatever the visit order), so
 * a far subtree is visited when its box distance is <= the current k-th
 * distance, where the reference requires < (nabo/kdtree_cpu.cpp:416-417):
 * the count equals the reference's except when a box distance exactly
 * equals the k-th distance at that moment (it then counts that subtree's
 * points too; about 20 of 104 M points on a 1.15 M-point lidar scan).
 * Results are always sorted ascending (SORT_RESULTS is accepted).
 * k up to 32 runs one query per thread, k from 33 to 1024 a group of lanes
 * per query (same results); larger k returns NABO_CUDA_ERR_UNSUPPORTED.
 * kd-trees of any height are searched: those taller than 256 levels (the
 * split rule gives such trees on geometrically spaced coordinates) with
 * their traversal stacks in global memory, taken from the scratch pool. */
int nabo_cuda_knn(const nabo_cuda_search* s, const void* query, int qRows, int64_t nq, int64_t qStride, int k,
                  double epsilon, unsigned optionFlags, double maxRadius, const void* maxRadii, int32_t* indices,
                  void* dists2, uint64_t* touched);

/* Same search with DEVICE buffers, stream-ordered on `stream` (a
 * cudaStream_t; NULL = legacy default stream). Does not synchronise.
 * touched (may be NULL) is a DEVICE uint64 to which the count is ADDED. */
int nabo_cuda_knn_device(const nabo_cuda_search* s, const void* query, int qRows, int64_t nq, int64_t qStride,
                         int k, double epsilon, unsigned optionFlags, double maxRadius, const void* maxRadii,
                         int32_t* indices, void* dists2, uint64_t* touched, void* stream);

/* Search that allocates no device memory (no counterpart in the reference,
 * whose CPU search needs no device memory at all).
 *
 * nabo_cuda_knn_device takes its query-ordering scratch from a memory
 * pool, which may call into the CUDA allocator. Some callers must not do
 * that once they are running: a robot's real-time perception loop (for
 * example ICP registering every lidar scan) that fixes its GPU memory at
 * start-up because allocation can block or synchronise the device, and
 * applications whose device memory is owned by their own arena. For them
 * this entry point takes its scratch from a fixed array inside the library,
 * NABO_CUDA_NOALLOC_SCRATCH_BYTES (3.25 MiB) per GPU, held by every GPU
 * that loads the library until the process exits. The caller passes device
 * inputs and outputs exactly as for nabo_cuda_knn_device; the results are
 * identical.
 *
 * Limits and rules:
 *  - nq <= NABO_CUDA_NOALLOC_MAX_QUERIES per call; larger requests fail
 *    with NABO_CUDA_ERR_ARGUMENT (split the batch);
 *  - the first call on a device looks up the array's device address
 *    (cudaGetSymbolAddress); make that first call before any stream
 *    capture;
 *  - every call on a device shares the one array: calls whose work
 *    overlaps on the GPU (different streams or threads without ordering
 *    between them) race and corrupt each other's results. Order them on
 *    one stream or synchronise between them. */
#define NABO_CUDA_NOALLOC_MAX_QUERIES 262144
#define NABO_CUDA_NOALLOC_SCRATCH_BYTES 3407872
int nabo_cuda_knn_device_noalloc(const nabo_cuda_search* s, const void* query, int qRows, int64_t nq,
                                 int64_t qStride, int k, double epsilon, unsigned optionFlags, double maxRadius,
                                 const void* maxRadii, int32_t* indices, void* dists2, uint64_t* touched,
                                 void* stream);

/* ---------------------------------------------------------------------
 * Learned search radius (no counterpart in the reference; it feeds the
 * reference's per-query radius overload, nabo/nabo.h:351).
 *
 * A radius model is a small network (inputs padded to 16: the normalised
 * coordinates, plus for 3-D clouds the occupancy of the voxel holding the
 * query at 8 octave scales; two hidden layers of 64 SiLU units; BF16
 * weights, FP32 sums) trained on the GPU to predict log(d_k), the log
 * distance of a query's k-th neighbour, from training queries whose d_k the
 * exact kd-tree search computes. A learned search runs the kd-tree search
 * with the per-query radius safety * exp(prediction + calibrated margin)
 * (capped at maxRadius) and
 * searches again without it every query that found fewer than k
 * neighbours inside its radius, so results equal nabo_cuda_knn's. */
typedef struct nabo_cuda_radius_model nabo_cuda_radius_model; /* opaque */
#define NABO_CUDA_RADIUS_MODEL_INPUTS 16
#define NABO_CUDA_RADIUS_MODEL_PARAMS 5313 /* W1[64][16] b1[64] W2[64][64] b2[64] w3[64] b3 */

typedef struct nabo_cuda_train_params {
  uint32_t struct_size;
  int32_t epochs;  /* passes over the training queries, default 30 */
  int32_t batch;   /* minibatch, default 4096 */
  float lr;        /* Adam learning rate (cosine-decayed), default 3e-3 */
  float safety;    /* radius = safety * exp(prediction), default 1.2 */
  float targetMissRate; /* after training, widen the radius until about this
                           fraction of the training queries would fall outside
                           it (default 0.01: on lidar scans every fallback
                           costs a whole second search while a wider radius
                           costs little; 0 keeps the plain safety factor) */
  uint64_t seed;   /* weight initialisation and shuffling, default 1234 */
  int32_t reserved[4];
} nabo_cuda_train_params;

void nabo_cuda_train_params_init(nabo_cuda_train_params* p);

/* Trains a model for k-NN searches of `s` (a KDTREE_CUDA object) from
 * `n` training queries in DEVICE memory (qRows x n, column stride qStride).
 * Training queries without k neighbours within maxRadius are left out. */
int nabo_cuda_radius_model_train(const nabo_cuda_search* s, const void* trainQueries, int qRows, int64_t n,
                                 int64_t qStride, int k, unsigned optionFlags, double maxRadius,
                                 const nabo_cuda_train_params* params, nabo_cuda_radius_model** out);
int nabo_cuda_radius_model_destroy(nabo_cuda_radius_model* m);

/* Per-query radii (DEVICE; the search object's scalar type), capped at
 * maxRadius; `raw` (DEVICE float, may be NULL) receives the standardised
 * network outputs. Stream-ordered. */
int nabo_cuda_radius_model_predict_device(const nabo_cuda_radius_model* m, const void* query, int qRows, int64_t nq,
                                          int64_t qStride, double maxRadius, void* radii, float* raw, void* stream);

/* Learned search with DEVICE buffers (stream-ordered, no host sync).
 * Same arguments and results as nabo_cuda_knn_device; `fallbacks` (DEVICE
 * int32, may be NULL) receives the number of queries searched again. With
 * TOUCH_STATISTICS, `touched` accumulates the points examined by both
 * searches (not the reference's count for an unbounded search). */
int nabo_cuda_knn_learned_device(const nabo_cuda_search* s, const nabo_cuda_radius_model* m, const void* query,
                                 int qRows, int64_t nq, int64_t qStride, int k, double epsilon, unsigned optionFlags,
                                 double maxRadius, int32_t* indices, void* dists2, uint64_t* touched,
                                 int32_t* fallbacks, void* stream);
/* Same with HOST buffers; `fallbacks` is a host int64. */
int nabo_cuda_knn_learned(const nabo_cuda_search* s, const nabo_cuda_radius_model* m, const void* query, int qRows,
                          int64_t nq, int64_t qStride, int k, double epsilon, unsigned optionFlags, double maxRadius,
                          int32_t* indices, void* dists2, uint64_t* touched, int64_t* fallbacks);

/* Network inputs of queries (DEVICE float, nq x 16), for checks. */
int nabo_cuda_radius_model_features_device(const nabo_cuda_radius_model* m, const void* query, int qRows, int64_t nq,
                                           int64_t qStride, float* features, void* stream);
/* Gradient (HOST, NABO_CUDA_RADIUS_MODEL_PARAMS floats) of the mean squared
 * error of the network over n samples: features (DEVICE float, n x 16) and
 * standardised targets (DEVICE float, n); `loss` (HOST) receives the summed
 * squared error. For gradient checks against an independent computation. */
int nabo_cuda_radius_model_gradients(const nabo_cuda_radius_model* m, const float* features, const float* targets,
                                     int64_t n, float* grad, float* loss);
/* Save / load: params (HOST, NABO_CUDA_RADIUS_MODEL_PARAMS FP32 master
 * weights) and meta (HOST, 16 floats: mu, sigma, safety, k, final training
 * loss, training samples, inputs used, calibrated margin, finest voxel
 * size, 7 zeros); either may be NULL. set() takes mu, sigma, safety, the
 * margin and the voxel size (rebuilding the voxel tables) from meta. */
int nabo_cuda_radius_model_get(const nabo_cuda_radius_model* m, float* params, float* meta);
int nabo_cuda_radius_model_set(nabo_cuda_radius_model* m, const float* params, const float* meta);

/* ---------------------------------------------------------------------
 * Batches of clouds (no counterpart in the reference, which builds one
 * tree per object). The clouds of a batch are stored back to back (cloud c
 * = columns [sum of earlier counts, + pointCounts[c]) of a dim x total
 * column-major array, stride dim); their kd-trees -- each the tree the
 * reference builds for that cloud alone -- are built together, and all
 * their queries are searched by one kernel launch, each in its cloud's
 * tree with the k given for that cloud. Self matches are not allowed
 * (k <= points - 1 per cloud). Results of cloud c's queries follow those
 * of the earlier clouds (k_c x nq_c, column-major per cloud), with indices
 * local to the cloud. */
typedef struct nabo_cuda_batch nabo_cuda_batch; /* opaque */

/* maxLevels: levels of the level-synchronous top build (segments of more
 * than 256 points), run without host synchronisation (0 = 48). A tree
 * needing more is reported by nabo_cuda_batch_status. params: bucketSize
 * and threadsPerBlock (may be NULL). */
int nabo_cuda_batch_create(int dtype, int dim, int nClouds, const int64_t* pointCounts,
                           const nabo_cuda_params* params, int maxLevels, nabo_cuda_batch** out);
int nabo_cuda_batch_destroy(nabo_cuda_batch* b);
/* Queries per cloud and k per cloud (HOST arrays, nClouds each). */
int nabo_cuda_batch_set_queries(nabo_cuda_batch* b, const int64_t* queryCounts, const int32_t* k);
/* Builds all trees from `clouds` (DEVICE); stream-ordered, no host sync. */
int nabo_cuda_batch_build_device(nabo_cuda_batch* b, const void* clouds, void* stream);
/* Searches all queries (DEVICE, dim x total queries, stride dim); results
 * into DEVICE arrays of sum(k_c * nq_c) entries. Stream-ordered. */
int nabo_cuda_batch_knn_device(nabo_cuda_batch* b, const void* queries, double epsilon, unsigned optionFlags,
                               double maxRadius, int32_t* indices, void* dists2, void* stream);
/* The same search with a radius per query (DEVICE, nq values of the
 * batch's scalar type, in query order): the reference's per-query radius
 * overload (nabo/nabo.h:351, nabo/kdtree_cpu.cpp:306-336) for every cloud.
 * A query whose radius is below maxRadius and that finds fewer than its
 * cloud's k neighbours inside it is searched again with maxRadius alone
 * (the learned-radius form's exact fallback); `fallbacks` (DEVICE int32,
 * may be NULL) receives how many were. With radii >= maxRadius it is the
 * plain per-query radius search. Stream-ordered. */
int nabo_cuda_batch_knn_radii_device(nabo_cuda_batch* b, const void* queries, const void* maxRadii, double epsilon,
                                     unsigned optionFlags, double maxRadius, int32_t* indices, void* dists2,
                                     int32_t* fallbacks, void* stream);
/* Batched learned radius: one model per (dimension, scalar type) serves
 * every cloud of batches of that kind. Its 8 inputs are taken from each
 * query's own cloud and tree -- the query descends its tree to its home
 * leaf (the search's first descent); the logs of the nearest, root-mean-
 * square and farthest distances to that leaf's points and of their count,
 * the log of the cloud's size and of its k, the leaf's depth and the mean
 * log extent of its cell -- so the network sees local density rather than
 * coordinates. Train with training queries laid out by the batch's current
 * query plan (nabo_cuda_batch_set_queries) and their exact results (dists2
 * of nabo_cuda_batch_knn_device); DEVICE buffers. Training as
 * nabo_cuda_radius_model_train (targets log d_k, safety, calibrated
 * margin). */
int nabo_cuda_batch_radius_model_train(nabo_cuda_batch* b, const void* queries, const void* dists2,
                                       const nabo_cuda_train_params* params, nabo_cuda_radius_model** out);
/* Learned batched search: the model's radius per query (capped at
 * maxRadius), then nabo_cuda_batch_knn_radii_device, so results equal the
 * plain batched search's; `fallbacks` (DEVICE int32, may be NULL) receives
 * the number of queries searched again. The model must be a batched model
 * of the batch's dimension and scalar type. Stream-ordered. */
int nabo_cuda_batch_knn_learned_device(nabo_cuda_batch* b, const nabo_cuda_radius_model* m, const void* queries,
                                       double epsilon, unsigned optionFlags, double maxRadius, int32_t* indices,
                                       void* dists2, int32_t* fallbacks, void* stream);
/* A batched model's radii (DEVICE, nq values of the batch's scalar type,
 * capped at maxRadius) and, if `raw` (DEVICE float) is given, standardised
 * outputs, for the queries of the current plan; and its network inputs
 * (DEVICE float, nq x 16), for checks. Stream-ordered. */
int nabo_cuda_batch_radius_model_predict_device(nabo_cuda_batch* b, const nabo_cuda_radius_model* m,
                                                const void* queries, double maxRadius, void* radii, float* raw,
                                                void* stream);
int nabo_cuda_batch_radius_model_features_device(nabo_cuda_batch* b, const nabo_cuda_radius_model* m,
                                                 const void* queries, float* features, void* stream);
/* Build + search as one CUDA graph: captured on the first call for these
 * buffers and arguments, replayed by later calls with the same ones (new
 * coordinates written into the same buffers). */
int nabo_cuda_batch_run(nabo_cuda_batch* b, const void* clouds, const void* queries, double epsilon,
                        unsigned optionFlags, double maxRadius, int32_t* indices, void* dists2, void* stream);
/* Build + search from HOST buffers (clouds, queries) into HOST result
 * arrays; returns when the results are there. The device copies are the
 * batch's own, allocated on first use. When all four buffers are
 * page-locked, one CUDA graph (captured as for nabo_cuda_batch_run) uploads
 * the queries during the build and searches the clouds in
 * params.pipelineChunks groups (0 = 8) of about equal result size, each
 * group's results downloaded while the next group is searched; otherwise
 * plain copies surround the device run. Results equal
 * nabo_cuda_batch_run's. Device calls on this batch still running on
 * other streams must have finished. */
int nabo_cuda_batch_run_host(nabo_cuda_batch* b, const void* clouds, const void* queries, double epsilon,
                             unsigned optionFlags, double maxRadius, int32_t* indices, void* dists2);
/* Synchronises the device, then info[0] = status bits (1 non-finite input,
 * 2 capacity or level limit exceeded, 4 a tree taller than the search
 * kernels' 256-level stacks -- not an error: its queries are searched again
 * with stacks in global memory, inside the same launch sequence -- and 8
 * one such stack did not fit the batch's stack memory, so those queries'
 * results are not written), [1] total nodes, [2] tallest tree, [3] top
 * levels run, [4] result entries, [5] queries, [6] points, [7] clouds. */
int nabo_cuda_batch_status(nabo_cuda_batch* b, int64_t info[8]);
/* One cloud's tree (indices local to the cloud), as nabo_cuda_export_tree;
 * with cutDim NULL only *nodeCount is set. */
int nabo_cuda_batch_export_tree(nabo_cuda_batch* b, int cloud, int64_t* nodeCount, int32_t* cutDim, void* cutVal,
                                uint32_t* right, uint32_t* bucketStart, uint32_t* bucketSize, int32_t* buckets);

/* Object properties: the reference's public members dim, minBound,
 * maxBound, creationOptionFlags (nabo/nabo.h:274-282) plus build facts.
 * info[0]=dim info[1]=n info[2]=dtype info[3]=searchType
 * info[4]=creationFlags info[5]=bucketSize info[6]=nodeCount
 * info[7]=tree height (inner nodes on the longest root-to-leaf path). */
int nabo_cuda_get_info(const nabo_cuda_search* s, int64_t info[8]);
/* minBound/maxBound, `dim` values of the object's scalar type. */
int nabo_cuda_get_bounds(const nabo_cuda_search* s, void* minBound, void* maxBound);

/* Copies the kd-tree to host arrays (nodeCount entries each, pre-order):
 * cutDim (-1 for a leaf), cutVal (scalar type), right child index,
 * bucket start, bucket size; and `buckets` (n point indices in leaf
 * order). Any pointer may be NULL. For parity checks against the
 * reference's node array (nabo/nabo_private.h:138-177). */
int nabo_cuda_export_tree(const nabo_cuda_search* s, int32_t* cutDim, void* cutVal, uint32_t* right,
                          uint32_t* bucketStart, uint32_t* bucketSize, int32_t* buckets);

/* Profiling aid (no reference counterpart; the reference times whole
 * calls, tests/knnbench.cpp:134-169): when enabled, every later
 * nabo_cuda_knn_device call on `s` records a pair of CUDA events right
 * around its search kernel, and nabo_cuda_last_kernel_ms() waits for the
 * second and returns the kernel's duration in milliseconds. Meant for
 * single-threaded benchmarking; concurrent calls on one object overwrite
 * each other's events. */
int nabo_cuda_profile(nabo_cuda_search* s, int enable);
int nabo_cuda_last_kernel_ms(const nabo_cuda_search* s, float* ms);

/* Last error message of the calling thread ("" if none). */
const char* nabo_cuda_last_error(void);

/* Library version string. */
const char* nabo_cuda_version(void);

/* Measured fused-multiply-add throughput of the current GPU in flop/s (two
 * flops per FMA) for NABO_CUDA_FLOAT32 or NABO_CUDA_FLOAT64: the denominator
 * of the brute-force search's roofline, which is bound by the arithmetic
 * pipes rather than by memory. Runs a short kernel (a few milliseconds). */
int nabo_cuda_measure_fma_peak(int dtype, double* flops);

#ifdef __cplusplus
}
#endif

#endif /* NABO_GB300_H */
