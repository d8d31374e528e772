// internal.cuh -- declarations shared by the build, search and C-ABI units.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "common.cuh"
#include "nabo_gb300.h"

struct nabo_cuda_search;
struct nabo_cuda_batch;

namespace nabo_gb300 {

// Status codes (mirrored in include/nabo_gb300.h).
enum Status : int {
  kOk = 0,
  kErrArgument = 1,
  kErrCuda = 2,
  kErrUnsupported = 3,
  kErrInternal = 4,
};

// Sets the calling thread's last-error message; returns `code`.
int set_error(int code, const std::string& msg);
int cuda_error(cudaError_t e, const char* what);

#define NABO_CUDA_TRY(expr)                                        \
  do {                                                             \
    cudaError_t e__ = (expr);                                      \
    if (e__ != cudaSuccess) return ::nabo_gb300::cuda_error(e__, #expr); \
  } while (0)

// Stream-ordered scratch from a library-owned memory pool of the current
// device. The pool keeps freed memory mapped (release threshold: unlimited)
// so repeated searches do not remap their scratch after every
// synchronisation; it is separate from the device's default pool, so other
// users of cudaMallocAsync are unaffected.
cudaError_t scratch_alloc(void** p, size_t bytes, cudaStream_t stream);
cudaError_t scratch_free(void* p, cudaStream_t stream);
// Consecutive query chunks of a pipelined search: chunk c is the queries
// [c ? end[c-1] : 0, end[c]).
constexpr int kMaxQueryChunks = 64;
struct QueryChunks {
  int n = 0;
  int64_t end[kMaxQueryChunks] = {};
};
// n chunks of shrinking size (weights n, n-1, ..., 1), so that the last
// chunk's results, downloaded after every search has finished, are few.
QueryChunks shrinking_chunks(int64_t nq, int n);

// Launches a kernel that begins with pdl_begin() with programmatic stream
// serialization, so that it is scheduled while the kernel before it drains.
template <typename... KArgs, typename... Args>
cudaError_t launch_pdl(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t stream,
                       Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = stream;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kernel, static_cast<KArgs>(args)...);
}

// While set (calling thread only), scratch_alloc uses cudaMallocAsync so the
// allocations can be captured into a CUDA graph.
void set_capture_allocations(bool on);

// Device-resident kd-tree (or, for brute force, the packed cloud only).
struct DeviceCloud {
  int dtype = 0;        // 0 = f32, 1 = f64
  int dim = 0;          // dimensions searched (<= cloud rows)
  int dpad = 0;         // compiled record dimension (>= dim)
  int64_t n = 0;        // points
  unsigned bucketSize = 8;
  int splitRule = 0;      // 0: the reference's sliding midpoint; 1: median (balanced)
  void* recs = nullptr;   // Rec<T,dpad>[n], leaf order (kd-tree) or cloud order (brute force)
  void* nodes = nullptr;  // Node<T>[nodeCount] (kd-tree only)
  int64_t nodeCount = 0;
  int height = 0;         // max inner nodes on a root-to-leaf path
  double lo[kMaxDim];     // true per-dimension bounds of the points (for query ordering)
  double hi[kMaxDim];
  // f64 kd-trees: float copies of recs (same order) and the largest
  // coordinate magnitude (device float), for the search's float pre-filter
  void* recs32 = nullptr;
  float* coordMax = nullptr;
};

struct BuildStats {
  int topLevels = 0;
  int64_t topNodes = 0;
  int64_t smallSegments = 0;
};

// Builds the kd-tree of `n` points (dim coordinates each, column stride
// `stride` elements) held in device memory at `dCloud`. Produces the same
// tree as the reference's KDTreeUnbalancedPtInLeavesImplicitBoundsStackOpt
// constructor (nabo/kdtree_cpu.cpp:109-272): same nodes, cut values and
// bucket order. `rootMin/rootMax` receive the root box the reference uses
// (with its max-bound initialisation), as doubles.
// splitRule 1 cuts at the median of the widest dimension instead (a
// balanced tree, not the reference's; see nabo_cuda_params::splitRule).
template <typename T, int D>
int build_kdtree(const T* dCloud, int64_t n, int64_t stride, int dim, unsigned bucketSize, cudaStream_t stream,
                 DeviceCloud* out, double* rootMin, double* rootMax, BuildStats* stats, int splitRule = 0);

// Output buffers of a forest build (all device memory, allocated by the
// caller): records (n), nodes (2n), nodeOffset (nClouds+1), root boxes
// (nClouds x kMaxDim each, scalar type), status (4 ints).
struct ForestOut {
  void* recs = nullptr;
  void* nodes = nullptr;
  int64_t nodeCap = 0;  // entries of `nodes`
  int64_t* nodeOffset = nullptr;
  void* rootLo = nullptr;
  void* rootHi = nullptr;
  int* status = nullptr;
};

// A batched search over a forest (batch.cu).
// Register top-k sizes compiled; a request for k uses the smallest K >= k.
#define NABO_K_LIST(X) X(1) X(2) X(5) X(8) X(10) X(16) X(32)
constexpr int kMaxK = 32;

inline int round_k(int k) {
#define NABO_ROUND(KK) \
  if (k <= KK) return KK;
  NABO_K_LIST(NABO_ROUND)
#undef NABO_ROUND
  return -1;
}

// Queries of a batch grouped by the top-k size compiled for their cloud's k
// (1, 2, 5, 8, 10, 16 or 32): one search launch per group, so a k = 1 cloud
// does not carry a 16-slot heap because another cloud wants 16. A group
// lists its clouds that have queries ("runs", by cloud id); runPrefix holds
// the running query count over all runs, group after group, so group g's
// launch covers positions [runPrefix[runBegin[g]], runPrefix[runBegin[g+1]])
// of that count, and run r's queries sit at leaf-order positions
// [qOffset[c], qOffset[c+1]) of cloud c = runCloud[r].
struct BatchClassPlan {
  int groups = 0;
  std::vector<int> K;                 // [groups]
  std::vector<int> runBegin;          // [groups + 1]
  std::vector<int32_t> runCloud;      // host copy
  std::vector<int64_t> runPrefix;     // host copy, [runs + 1]
  int32_t* dRunCloud = nullptr;       // device copies
  int64_t* dRunPrefix = nullptr;
};

struct BatchArgs {
  const void* nodes;
  const void* recs;
  int dim;
  int nClouds;
  int64_t nodeCap;              // hist entries (>= total nodes)
  const int64_t* nodeOffset;    // device, nClouds+1
  const int64_t* qOffset;       // device, nClouds+1
  const int64_t* outOffset;     // device, nClouds+1 (result entries)
  const int32_t* kOf;           // device, nClouds
  int kMax;
  const void* query;            // device, dim rows x nq, stride qStride
  int64_t nq;
  int64_t qStride;
  double eps;
  unsigned optionFlags;
  double maxRadius;
  int32_t* indices;             // device, concatenated per cloud
  void* dists2;
  int32_t* order;               // scratch
  uint32_t* hist;
  uint32_t* cell;
  uint32_t* rank;
  int blockSize;                // threads per block of the search kernel
  const void* recs32;           // f64: float copies of recs, or null
  const float* coordMax;        // f64: device float, largest coordinate magnitude
  // Trees taller than the search kernels' stacks (256 levels), which only
  // the device knows of (*heightDev: the tallest tree): the search is then
  // run by the deep kernel with stacks in `slab`; *deepFail is set to -1 if
  // one stack does not fit the slab.
  void* slab;
  int64_t slabBytes;
  const int* heightDev;
  int32_t* deepFail;
  // Optional per-query radii (device, nq values in query order, the batch's
  // scalar type), the reference's maxRadii overload (nabo/nabo.h:351) for
  // every cloud; a query whose radius is below maxRadius and that finds
  // fewer than its cloud's k neighbours inside it searches again with
  // maxRadius, counted in *fallbacks (may be null).
  const void* maxRadii;
  int32_t* fallbacks;
  int lanesPerQuery;            // 1: one thread per query; 8: a lane group (k <= 32)
  const BatchClassPlan* classes;  // null or no groups: one launch sized for the largest k
  const int64_t* hQOffset;        // host copy of qOffset (to map a position range to clouds)
  // streams and events for running the groups' launches side by side (all
  // null: one after the other on the caller's stream)
  cudaStream_t aux[2];
  cudaEvent_t evFork;
  cudaEvent_t evJoin[2];
};
template <typename T, int D>
int knn_batch(const BatchArgs& b, cudaStream_t stream);
// knn_batch in two steps: the leaf order of all queries, then the search
// of order positions [begin, end).
template <typename T, int D>
int order_batch(const BatchArgs& b, cudaStream_t stream);
template <typename T, int D>
int search_batch(const BatchArgs& b, int64_t begin, int64_t end, cudaStream_t stream);

// Float copies of double records and their largest coordinate magnitude
// (recs32 holds n Rec<float, D>; coordMax one device float).
template <int D>
int narrow_records(const void* recs, int64_t n, int dim, void* recs32, float* coordMax, cudaStream_t stream);

template <typename T, int D>
int build_forest(const T* dCloud, int64_t n, int64_t stride, int dim, unsigned bucketSize, const int64_t* dOff,
                 int nClouds, int maxLevels, cudaStream_t stream, ForestOut* f, int splitRule = 0);

// Packs the cloud into records in cloud order (brute force) and computes
// its true bounds.
template <typename T, int D>
int pack_cloud(const T* dCloud, int64_t n, int64_t stride, int dim, cudaStream_t stream, DeviceCloud* out);

struct KnnArgs {
  const void* query = nullptr;  // device, dim rows x nq, column stride qStride
  int64_t nq = 0;
  int64_t qStride = 0;
  int k = 1;
  double eps = 0.0;
  unsigned optionFlags = 0;
  bool touchStats = false;
  double maxRadius = 0.0;        // used when maxRadii == nullptr
  const void* maxRadii = nullptr;  // device, nq values, or nullptr
  int32_t* indices = nullptr;    // device, k x nq column-major
  void* dists2 = nullptr;        // device, k x nq column-major
  unsigned long long* touched = nullptr;  // device counter (accumulated), may be null
  bool sortQueries = true;       // reorder queries along a space-filling curve
  int32_t* found = nullptr;      // optional device output: neighbours found per query
  int traversal = 0;             // 0 auto, 1 reference order, 2 warp packet (exact search only)
  const int32_t* nqDevice = nullptr;  // optional device count: only the first *nqDevice of nq run
  // With maxRadii: a query whose bounded search found fewer than k
  // neighbours although its radius was below fallbackRadius searches again
  // with maxRadius (in the same thread) and is counted in *fallbacks.
  double fallbackRadius = -1.0;
  int32_t* fallbacks = nullptr;
  cudaEvent_t evStart = nullptr; // optional: recorded right before / after the search kernel
  cudaEvent_t evStop = nullptr;
  // Optional device memory for the traversal stacks of a kd-tree taller than
  // the compiled stacks (256 levels); without it such a search takes them
  // from the scratch pool.
  void* stackSlab = nullptr;
  size_t stackSlabBytes = 0;
};

// Whether a search runs its queries in a sorted order. The sort costs about
// 130 us almost whatever the size, so it pays only for enough work: measured
// on GB300, 3-D lidar scans at k = 10 gained from 2^18 queries (440 vs
// 470 us) and lost below (131 k: 346 vs 260 us), while 8-D clustered clouds
// at k = 32 gained 30 % at 200 k queries (16.7 vs 23.9 ms). The rule weighs
// the queries by k and by the dimension.
inline bool worth_sorting(int64_t nq, int k, int dim) {
  const double work = (double)nq * (k + 10) / 20.0 * (dim > 3 ? 8.0 : 1.0);
  return work >= (double)(int64_t(1) << 18);
}
template <typename T, int D>
int knn_kdtree(const DeviceCloud& c, const KnnArgs& a, cudaStream_t stream);
template <typename T, int D>
int knn_bruteforce(const DeviceCloud& c, const KnnArgs& a, cudaStream_t stream);

template <typename T, int D>
int knn_kdtree_given_order(const DeviceCloud& c, const KnnArgs& a, const int32_t* order, cudaStream_t stream);
template <typename T, int D>
int knn_chunk_order(const DeviceCloud& c, const void* query, int64_t nq, int64_t qStride, const QueryChunks& chunks,
                    int32_t* order, cudaStream_t stream, void* copyOut = nullptr);
template <typename T, int D>
int knn_leaf_order(const DeviceCloud& c, const void* query, int64_t nq, int64_t qStride, int32_t* order,
                   cudaStream_t stream);

// Read access to a search object for the allocation-free entry point, and
// the search-argument checks every entry point applies.
struct HandleView {
  const DeviceCloud* cloud;
  int searchType;
  unsigned creationFlags;
  int device;
  int traversal;
  bool sortQueries;     // the object's queryOrdering parameter
  cudaEvent_t evStart;  // profiling events (null when profiling is off)
  cudaEvent_t evStop;
};
HandleView handle_view(const struct ::nabo_cuda_search* s);
int handle_check_knn(const struct ::nabo_cuda_search* s, int qRows, int64_t nq, int64_t qStride, int k,
                     unsigned optionFlags, const void* maxRadii);

// Read access to a batch for the learned batched form (learned.cu).
struct BatchView {
  int dtype, dim, dpad, nClouds, kMax, device;
  int64_t nq;
  const void* nodes;
  const void* recs;
  const int64_t* pointOff;   // device, nClouds+1: the clouds' point offsets
  const int64_t* nodeOffset; // device, nClouds+1
  const void* rootLo;        // device, nClouds x kMaxDim (scalar type)
  const void* rootHi;
  const int64_t* qOffset;    // device, nClouds+1 (current query plan)
  const int64_t* outOffset;  // device, nClouds+1
  const int32_t* kOf;        // device, nClouds
};
int batch_view(const struct ::nabo_cuda_batch* b, BatchView* out);

// Learned search radius (learned.cu).
struct RadiusModel;
int radius_model_train(const struct ::nabo_cuda_search* s, const void* dTrain, int64_t nTrain, int64_t qStride, int k,
                       unsigned optionFlags, double maxRadius, const nabo_cuda_train_params& tp, RadiusModel** out,
                       cudaStream_t st);
void radius_model_free(RadiusModel* m);
int radius_model_predict(const RadiusModel& m, const void* query, int64_t nq, int64_t qStride, double maxRadius,
                         void* radii, float* raw, cudaStream_t st);
int knn_learned(const struct ::nabo_cuda_search* s, const RadiusModel& m, const KnnArgs& base, int32_t* dFallbacks,
                cudaStream_t st);
int radius_model_gradients(const RadiusModel& m, const float* dX, const float* dY, int64_t n, float* hGrad,
                           float* hLoss, cudaStream_t st);
int radius_model_features(const RadiusModel& m, const void* query, int64_t nq, int64_t qStride, float* dX,
                          cudaStream_t st);
int radius_model_get(const RadiusModel& m, float* params, float* meta);
int radius_model_set(RadiusModel& m, const float* params, const float* meta);
const void* radius_model_owner(const RadiusModel& m);
int radius_model_k(const RadiusModel& m);

// Query ordering: writes a permutation of [0, nq) grouping nearby queries
// (a stable sort by Morton code). With chunks (n > 1) the permutation is
// chunk-major: chunk c's queries come before those of chunk c+1, in Morton
// order among themselves (the chunk number takes the top bits of a 32-bit
// key, so more chunks leave a coarser curve). With copyOut, the first dim
// coordinates of each query row are also written there at the same
// offsets (dQuery may then be a device-mapped page-locked host buffer).
template <typename T>
int order_queries(const T* dQuery, int64_t nq, int64_t qStride, int dim, const double* lo, const double* hi,
                  int32_t* dOrder, cudaStream_t stream, const QueryChunks* chunks = nullptr, T* copyOut = nullptr);

// Counting-sort placement: dHist holds per-cell counts (turned into offsets
// in place), dCell/dRank each query's cell and rank inside it. With binsDev
// only the first min(bins, *binsDev) cells (a count the device holds) are
// scanned; every cell at or past it must be empty.
int order_by_cells(const uint32_t* dCell, const uint32_t* dRank, uint32_t* dHist, int64_t bins, int64_t nq,
                   int32_t* dOrder, cudaStream_t stream, const int64_t* binsDev = nullptr);

// Zeroes the first min(n, *nDev) entries (all n when nDev is null).
int zero_u32(uint32_t* data, int64_t n, const int64_t* nDev, cudaStream_t stream);

// Stable sort of element indices 0..n-1 (or of dVals, when given) by the
// low `bits` bits of dKeys, written to dOrder; dKeys is clobbered.
int sort_order_u32(uint32_t* dKeys, int64_t n, int bits, int32_t* dOrder, cudaStream_t stream,
                   const uint32_t* dVals = nullptr);

// Device-wide exclusive scan of uint32 values (in place), returns total via
// a device pointer. Scratch is stream-ordered.
int scan_exclusive_u32(uint32_t* data, int64_t n, uint32_t* dTotal, cudaStream_t stream,
                       const int64_t* nDev = nullptr);

}  // namespace nabo_gb300
