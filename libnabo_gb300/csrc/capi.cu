// capi.cu -- the extern "C" boundary (include/nabo_gb300.h).
//
// Argument checks follow the reference in order and wording:
//   create:  nabo/nabo.cpp:137-138 (dim <= 0), :76-79 (empty cloud),
//            nabo/kdtree_cpu.cpp:234-235 (bucket size), :245-251 (node count)
//   knn:     nabo/nabo.cpp:102-131 (checkSizesKnn)
// so the C++ front end can rethrow them as the reference's exceptions.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <mutex>
#include <limits>
#include <string>
#include <vector>

#include "internal.cuh"
#include "nabo_gb300.h"

namespace nabo_gb300 {

namespace {
thread_local std::string g_lastError;
thread_local cudaError_t g_lastCudaError = cudaSuccess;  // the code behind the last kErrCuda
}

int set_error(int code, const std::string& msg) {
  g_lastError = msg;
  return code;
}

namespace {
std::mutex g_poolMutex;
cudaMemPool_t g_pools[64] = {};
}  // namespace

static cudaError_t library_pool(cudaMemPool_t* pool) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(g_poolMutex);
  if (!g_pools[dev]) {
    cudaMemPoolProps props = {};
    props.allocType = cudaMemAllocationTypePinned;
    props.handleTypes = cudaMemHandleTypeNone;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = dev;
    cudaMemPool_t p;
    e = cudaMemPoolCreate(&p, &props);
    if (e != cudaSuccess) return e;
    uint64_t keep = ~0ull;
    e = cudaMemPoolSetAttribute(p, cudaMemPoolAttrReleaseThreshold, &keep);
    if (e != cudaSuccess) {
      cudaMemPoolDestroy(p);
      return e;
    }
    g_pools[dev] = p;
  }
  *pool = g_pools[dev];
  return cudaSuccess;
}

namespace {
thread_local bool g_captureAllocations = false;
}

void set_capture_allocations(bool on) { g_captureAllocations = on; }

cudaError_t scratch_alloc(void** p, size_t bytes, cudaStream_t stream) {
  // while a CUDA graph is being captured, allocations become graph memory
  // nodes of the device's default pool
  if (g_captureAllocations) return cudaMallocAsync(p, bytes, stream);
  cudaMemPool_t pool;
  const cudaError_t e = library_pool(&pool);
  if (e != cudaSuccess) return e;
  return cudaMallocFromPoolAsync(p, bytes, pool, stream);
}

cudaError_t scratch_free(void* p, cudaStream_t stream) { return cudaFreeAsync(p, stream); }

int cuda_error(cudaError_t e, const char* what) {
  g_lastCudaError = e;
  g_lastError = std::string("CUDA error in ") + what + ": " + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ")";
  return kErrCuda;
}

}  // namespace nabo_gb300

using namespace nabo_gb300;

namespace nabo_gb300 {
constexpr int kPipelineMaxChunks = kMaxQueryChunks;  // nabo_cuda_params::pipelineChunks

// The arguments a pipelined call's CUDA graph was captured with (compared
// bytewise; made with make_pipe_key so that padding is zero).
struct PipeKey {
  const void* query;
  const void* maxRadii;
  const void* indices;
  const void* dists2;
  int64_t nq;
  int64_t qStride;
  double epsilon;
  double maxRadius;
  int qRows;
  int k;
  unsigned optionFlags;
  int nChunks;
};

inline PipeKey make_pipe_key(const void* query, const void* maxRadii, const void* indices, const void* dists2,
                             int64_t nq, int64_t qStride, double epsilon, double maxRadius, int qRows, int k,
                             unsigned optionFlags, int nChunks) {
  PipeKey key;
  std::memset(&key, 0, sizeof(key));
  key.query = query;
  key.maxRadii = maxRadii;
  key.indices = indices;
  key.dists2 = dists2;
  key.nq = nq;
  key.qStride = qStride;
  key.epsilon = epsilon;
  key.maxRadius = maxRadius;
  key.qRows = qRows;
  key.k = k;
  key.optionFlags = optionFlags;
  key.nChunks = nChunks;
  return key;
}

inline bool same_key(const PipeKey& a, const PipeKey& b) { return std::memcmp(&a, &b, sizeof(PipeKey)) == 0; }

// Two compute streams, a copy stream and the events that order them; the
// main stream, a page-locked touched-count slot and the CUDA graph of a
// repeated call.
struct PipeRes {
  cudaStream_t comp[2] = {};
  cudaStream_t copy = nullptr;
  cudaStream_t main = nullptr;
  cudaEvent_t ready = nullptr, copied = nullptr;
  cudaEvent_t compDone[2] = {};
  cudaEvent_t searched[kPipelineMaxChunks] = {};
  unsigned long long* hostTouched = nullptr;
  cudaGraphExec_t exec = nullptr;
  PipeKey graphKey = {};
  PipeKey lastKey = {};
  bool hasLast = false;
  bool noGraph = false;  // a capture failed once: direct calls only
  bool made = false;
};

inline void destroy_pipe(PipeRes& p) {
  if (p.exec) cudaGraphExecDestroy(p.exec);
  if (p.main) cudaStreamDestroy(p.main);
  if (p.hostTouched) cudaFreeHost(p.hostTouched);
  for (int i = 0; i < 2; ++i) {
    if (p.comp[i]) cudaStreamDestroy(p.comp[i]);
    if (p.compDone[i]) cudaEventDestroy(p.compDone[i]);
  }
  for (int i = 0; i < kPipelineMaxChunks; ++i)
    if (p.searched[i]) cudaEventDestroy(p.searched[i]);
  if (p.copy) cudaStreamDestroy(p.copy);
  if (p.ready) cudaEventDestroy(p.ready);
  if (p.copied) cudaEventDestroy(p.copied);
  p = PipeRes();
}

inline cudaError_t make_pipe(PipeRes& p) {
  cudaError_t e = cudaStreamCreateWithFlags(&p.copy, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&p.main, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaHostAlloc((void**)&p.hostTouched, sizeof(unsigned long long), cudaHostAllocDefault);
  for (int i = 0; i < 2 && e == cudaSuccess; ++i) e = cudaStreamCreateWithFlags(&p.comp[i], cudaStreamNonBlocking);
  for (int i = 0; i < 2 && e == cudaSuccess; ++i) e = cudaEventCreateWithFlags(&p.compDone[i], cudaEventDisableTiming);
  for (int i = 0; i < kPipelineMaxChunks && e == cudaSuccess; ++i)
    e = cudaEventCreateWithFlags(&p.searched[i], cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&p.ready, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&p.copied, cudaEventDisableTiming);
  if (e != cudaSuccess)
    destroy_pipe(p);
  else
    p.made = true;
  return e;
}
}  // namespace nabo_gb300

struct nabo_cuda_search {
  DeviceCloud c;
  int searchType = 0;
  unsigned creationFlags = 0;
  int rows = 0;
  int device = 0;
  int queryOrdering = 1;
  int traversal = 0;
  int pipelineChunks = 0;
  double minBound[kMaxDim];
  double maxBound[kMaxDim];
  cudaEvent_t evStart = nullptr;  // profiling: bracket the search kernel
  cudaEvent_t evStop = nullptr;
  // Staging for small host-buffer calls: one pinned host block and one
  // device block with the same layout, so a call is one upload, the search
  // and one download. Taken with try_lock; a concurrent call on the same
  // object uses the general path instead.
  mutable std::mutex stageLock;
  mutable void* stageHost = nullptr;
  mutable void* stageDev = nullptr;
  mutable size_t stageBytes = 0;  // size of each block, grown by powers of two
  // a staged call that repeats the previous one's sizes and arguments
  // replays a CUDA graph of its upload, search and download
  mutable cudaStream_t stageStream = nullptr;
  mutable cudaGraphExec_t stageExec = nullptr;
  mutable PipeKey stageGraphKey = {};
  mutable PipeKey stageLastKey = {};
  mutable bool stageHasLast = false;
  mutable bool stageNoGraph = false;  // a capture failed once: direct calls only
  // Streams and events of the pipelined large-call path, made on first use
  // and kept (a call made while another holds them makes its own).
  mutable std::mutex pipeLock;
  mutable PipeRes pipe;
};

namespace {

// Runs `body` with the object's device current, restoring the caller's.
struct DeviceGuard {
  int prev = -1;
  bool ok = true;
  explicit DeviceGuard(int dev) {
    if (cudaGetDevice(&prev) != cudaSuccess) {
      ok = false;
      return;
    }
    if (prev != dev && cudaSetDevice(dev) != cudaSuccess) ok = false;
  }
  ~DeviceGuard() {
    int cur = -1;
    if (prev >= 0 && cudaGetDevice(&cur) == cudaSuccess && cur != prev) cudaSetDevice(prev);
  }
};

int pad_dim(int dim) {
  if (dim <= 2) return 2;
  if (dim == 3) return 3;
  if (dim == 4) return 4;
  if (dim <= 8) return 8;
  if (dim <= 16) return 16;
  return -1;
}

#define NABO_DISPATCH(dtype, dpad, CALL)                         \
  do {                                                           \
    if ((dtype) == NABO_CUDA_FLOAT32) {                          \
      using T = float;                                           \
      switch (dpad) {                                            \
        case 2: { constexpr int D = 2; return CALL; }            \
        case 3: { constexpr int D = 3; return CALL; }            \
        case 4: { constexpr int D = 4; return CALL; }            \
        case 8: { constexpr int D = 8; return CALL; }            \
        case 16: { constexpr int D = 16; return CALL; }          \
      }                                                          \
    } else {                                                     \
      using T = double;                                          \
      switch (dpad) {                                            \
        case 2: { constexpr int D = 2; return CALL; }            \
        case 3: { constexpr int D = 3; return CALL; }            \
        case 4: { constexpr int D = 4; return CALL; }            \
        case 8: { constexpr int D = 8; return CALL; }            \
        case 16: { constexpr int D = 16; return CALL; }          \
      }                                                          \
    }                                                            \
    return set_error(kErrInternal, "bad dispatch");              \
  } while (0)

// The same dispatch, storing the result in `rc` instead of returning it.
#define NABO_DISPATCH_RC(rc, dtype, dpad, CALL)                  \
  do {                                                           \
    bool hit_ = true;                                            \
    if ((dtype) == NABO_CUDA_FLOAT32) {                          \
      using T = float;                                           \
      switch (dpad) {                                            \
        case 2: { constexpr int D = 2; rc = CALL; break; }       \
        case 3: { constexpr int D = 3; rc = CALL; break; }       \
        case 4: { constexpr int D = 4; rc = CALL; break; }       \
        case 8: { constexpr int D = 8; rc = CALL; break; }       \
        case 16: { constexpr int D = 16; rc = CALL; break; }     \
        default: hit_ = false;                                   \
      }                                                          \
    } else {                                                     \
      using T = double;                                          \
      switch (dpad) {                                            \
        case 2: { constexpr int D = 2; rc = CALL; break; }       \
        case 3: { constexpr int D = 3; rc = CALL; break; }       \
        case 4: { constexpr int D = 4; rc = CALL; break; }       \
        case 8: { constexpr int D = 8; rc = CALL; break; }       \
        case 16: { constexpr int D = 16; rc = CALL; break; }     \
        default: hit_ = false;                                   \
      }                                                          \
    }                                                            \
    if (!hit_) rc = set_error(kErrInternal, "bad dispatch");     \
  } while (0)

uint32_t storage_bit_count(uint32_t v) {
  for (uint32_t i = 0; i < 64; ++i) {
    if (v == 0) return i;
    v >>= 1;
  }
  return 64;
}

// Float copies of a double kd-tree's records for the search's pre-filter.
template <int D>
int narrow_cloud_d(DeviceCloud& c, cudaStream_t st) {
  NABO_CUDA_TRY(cudaMalloc(&c.recs32, (size_t)c.n * sizeof(Rec<float, D>)));
  NABO_CUDA_TRY(cudaMalloc((void**)&c.coordMax, sizeof(float)));
  return narrow_records<D>(c.recs, c.n, c.dim, c.recs32, c.coordMax, st);
}

int narrow_cloud(DeviceCloud& c, cudaStream_t st) {
  switch (c.dpad) {
    case 2: return narrow_cloud_d<2>(c, st);
    case 3: return narrow_cloud_d<3>(c, st);
    case 4: return narrow_cloud_d<4>(c, st);
    case 8: return narrow_cloud_d<8>(c, st);
    default: return narrow_cloud_d<16>(c, st);
  }
}

int build_any(nabo_cuda_search* h, const void* dCloud, int64_t stride, cudaStream_t st) {
  double rootMin[kMaxDim], rootMax[kMaxDim];
  if (h->searchType == NABO_SEARCH_KDTREE_CUDA) {
    int rc = kOk;
    NABO_DISPATCH_RC(rc, h->c.dtype, h->c.dpad,
                     (build_kdtree<T, D>(static_cast<const T*>(dCloud), h->c.n, stride, h->c.dim, h->c.bucketSize,
                                         st, &h->c, rootMin, rootMax, nullptr, h->c.splitRule)));
    if (rc == kOk && h->c.dtype == NABO_CUDA_FLOAT64) rc = narrow_cloud(h->c, st);
    return rc;
  }
  NABO_DISPATCH(h->c.dtype, h->c.dpad, (pack_cloud<T, D>(static_cast<const T*>(dCloud), h->c.n, stride, h->c.dim, st, &h->c)));
}

int knn_any(const nabo_cuda_search* h, const KnnArgs& a, cudaStream_t st) {
  if (h->searchType == NABO_SEARCH_KDTREE_CUDA) {
    NABO_DISPATCH(h->c.dtype, h->c.dpad, (knn_kdtree<T, D>(h->c, a, st)));
  }
  NABO_DISPATCH(h->c.dtype, h->c.dpad, (knn_bruteforce<T, D>(h->c, a, st)));
}

int knn_given_order_any(const nabo_cuda_search* h, const KnnArgs& a, const int32_t* order, cudaStream_t st) {
  NABO_DISPATCH(h->c.dtype, h->c.dpad, (knn_kdtree_given_order<T, D>(h->c, a, order, st)));
}

int chunk_order_any(const nabo_cuda_search* h, const void* query, int64_t nq, int64_t qStride,
                    const QueryChunks& chunks, int32_t* order, cudaStream_t st, void* copyOut) {
  NABO_DISPATCH(h->c.dtype, h->c.dpad,
                (knn_chunk_order<T, D>(h->c, query, nq, qStride, chunks, order, st, copyOut)));
}

void free_events(nabo_cuda_search* s) {
  if (s->evStart) cudaEventDestroy(s->evStart);
  if (s->evStop) cudaEventDestroy(s->evStop);
  s->evStart = s->evStop = nullptr;
}

void free_stage(nabo_cuda_search* s) {
  if (s->stageExec) cudaGraphExecDestroy(s->stageExec);
  if (s->stageStream) cudaStreamDestroy(s->stageStream);
  if (s->stageHost) cudaFreeHost(s->stageHost);
  if (s->stageDev) cudaFree(s->stageDev);
  s->stageExec = nullptr;
  s->stageStream = nullptr;
  s->stageHasLast = false;
  s->stageHost = s->stageDev = nullptr;
  s->stageBytes = 0;
}

void free_cloud(DeviceCloud& c) {
  if (c.recs) cudaFree(c.recs);
  if (c.nodes) cudaFree(c.nodes);
  if (c.recs32) cudaFree(c.recs32);
  if (c.coordMax) cudaFree(c.coordMax);
  c.recs = nullptr;
  c.nodes = nullptr;
  c.recs32 = nullptr;
  c.coordMax = nullptr;
}

int create_impl(int dtype, const void* cloud, bool cloudOnDevice, int rows, int64_t n, int64_t colStride, int dimIn,
                int searchType, unsigned creationFlags, const nabo_cuda_params* params, nabo_cuda_search** out) {
  if (!out) return set_error(kErrArgument, "output handle pointer is NULL");
  *out = nullptr;
  if (dtype != NABO_CUDA_FLOAT32 && dtype != NABO_CUDA_FLOAT64) return set_error(kErrArgument, "unknown scalar type");
  nabo_cuda_params p;
  nabo_cuda_params_init(&p);
  if (params) {
    p.bucketSize = params->bucketSize;
    p.queryOrdering = params->queryOrdering;
    p.traversal = params->traversal;
    p.pipelineChunks = params->pipelineChunks;
    p.splitRule = params->splitRule;
  }
  if (p.pipelineChunks < 0 || p.pipelineChunks > kPipelineMaxChunks)
    return set_error(kErrArgument, "pipelineChunks must be between 0 and 64");
  if (p.splitRule != 0 && p.splitRule != 1) return set_error(kErrArgument, "splitRule must be 0 or 1");
  if (p.splitRule == 1 && (creationFlags & NABO_TOUCH_STATISTICS))
    return set_error(kErrArgument, "the median-split tree is not the reference's tree: TOUCH_STATISTICS would not "
                                   "count what the reference counts (use splitRule 0)");
  // NearestNeighbourSearch::create (nabo/nabo.cpp:137-138)
  if (dimIn <= 0) return set_error(kErrArgument, "Your space must have at least one dimension");
  if (searchType < 0 || searchType >= NABO_SEARCH_TYPE_COUNT) return set_error(kErrArgument, "Unknown search type");
  if (searchType != NABO_SEARCH_KDTREE_CUDA && searchType != NABO_SEARCH_BRUTE_FORCE_CUDA)
    return set_error(kErrUnsupported,
                     "this library provides only the CUDA search types (KDTREE_CUDA, BRUTE_FORCE_CUDA); "
                     "the CPU and OpenCL types are provided by libnabo");
  // base constructor (nabo/nabo.cpp:69-80)
  if (n == 0) return set_error(kErrArgument, "Cloud has no points");
  if (rows == 0) return set_error(kErrArgument, "Cloud has 0 dimensions");
  if (n < 0 || rows < 0) return set_error(kErrArgument, "negative cloud size");
  if (!cloud) return set_error(kErrArgument, "cloud pointer is NULL");
  if (colStride < rows) return set_error(kErrArgument, "cloud column stride is smaller than its row count");
  const int dim = std::min(dimIn, rows);
  if (searchType == NABO_SEARCH_KDTREE_CUDA) {
    // nabo/kdtree_cpu.cpp:234-251
    if (p.bucketSize < 2)
      return set_error(kErrArgument,
                       "Requested bucket size " + std::to_string(p.bucketSize) + ", but must be larger than 2");
    if (n > (int64_t)p.bucketSize) {
      const uint32_t dimBitCount = storage_bit_count((uint32_t)dim);
      const uint64_t maxNodeCount = (0x1ULL << (32 - dimBitCount)) - 1;
      const uint64_t estimatedNodeCount = (uint64_t)n / (p.bucketSize / 2);
      if (estimatedNodeCount > maxNodeCount)
        return set_error(kErrArgument, "Cloud has a risk to have more nodes (" + std::to_string(estimatedNodeCount) +
                                           ") than the kd-tree allows (" + std::to_string(maxNodeCount) +
                                           "). The kd-tree has " + std::to_string(dimBitCount) +
                                           " bits for dimensions and " + std::to_string(32 - dimBitCount) +
                                           " bits for node indices");
    }
  }
  const int dpad = pad_dim(dim);
  if (dpad < 0) return set_error(kErrUnsupported, "the CUDA search types support at most 16 dimensions");
  if (n > (int64_t)std::numeric_limits<int32_t>::max())
    return set_error(kErrUnsupported, "clouds are indexed with int (nabo/nabo.h:267): at most 2^31-1 points");
  if (searchType == NABO_SEARCH_KDTREE_CUDA && std::min<int64_t>(n, p.bucketSize) > (int64_t)kMaxNodeIndex)
    return set_error(kErrUnsupported, "bucket size too large for the device node layout");

  nabo_cuda_search* h = new nabo_cuda_search();
  h->searchType = searchType;
  h->creationFlags = creationFlags;
  h->rows = rows;
  h->queryOrdering = p.queryOrdering;
  h->traversal = p.traversal;
  h->pipelineChunks = p.pipelineChunks;
  h->c.splitRule = searchType == NABO_SEARCH_KDTREE_CUDA ? p.splitRule : 0;
  if (p.traversal < 0 || p.traversal > 2) {
    delete h;
    return set_error(kErrArgument, "traversal must be 0, 1 or 2");
  }
  h->c.dtype = dtype;
  h->c.dim = dim;
  h->c.dpad = dpad;
  h->c.n = n;
  h->c.bucketSize = p.bucketSize;
  if (cudaGetDevice(&h->device) != cudaSuccess) {
    const cudaError_t e = cudaGetLastError();
    delete h;
    return cuda_error(e, "cudaGetDevice");
  }
  cudaStream_t st = cudaStreamPerThread;
  const size_t es = dtype == NABO_CUDA_FLOAT32 ? 4 : 8;
  const size_t bytes = (size_t)((n - 1) * colStride + rows) * es;
  const void* dCloud = cloud;
  void* tmp = nullptr;
  int rc = kOk;
  if (!cloudOnDevice) {
    cudaError_t e = scratch_alloc(&tmp, bytes, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(tmp, cloud, bytes, cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) rc = cuda_error(e, "cloud upload");
    dCloud = tmp;
  }
  if (rc == kOk) rc = build_any(h, dCloud, colStride, st);
  if (tmp) scratch_free(tmp, st);
  if (rc == kOk) {
    const cudaError_t e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) rc = cuda_error(e, "create");
  }
  if (rc != kOk) {
    cudaStreamSynchronize(st);
    free_cloud(h->c);
    delete h;
    return rc;
  }
  // Public bounds (nabo/nabo.h:280-282): brute force stores the true
  // bounds (nabo/brute_force_cpu.cpp:48-50); the kd-tree leaves the base
  // constructor's initial values when the cloud fits one bucket
  // (nabo/kdtree_cpu.cpp:236-243), else min over points and
  // max(numeric_limits<T>::min(), max over points) (nabo/nabo.cpp:73-74).
  for (int d = 0; d < kMaxDim; ++d) {
    h->minBound[d] = h->c.lo[d];
    h->maxBound[d] = h->c.hi[d];
  }
  if (searchType == NABO_SEARCH_KDTREE_CUDA) {
    const double tmin = dtype == NABO_CUDA_FLOAT32 ? (double)std::numeric_limits<float>::min()
                                                   : std::numeric_limits<double>::min();
    const double tmax = dtype == NABO_CUDA_FLOAT32 ? (double)std::numeric_limits<float>::max()
                                                   : std::numeric_limits<double>::max();
    for (int d = 0; d < dim; ++d) {
      if (n <= (int64_t)p.bucketSize) {
        h->minBound[d] = tmax;
        h->maxBound[d] = tmin;
      } else {
        h->maxBound[d] = std::max(h->maxBound[d], tmin);
      }
    }
  }
  *out = h;
  return kOk;
}

int check_knn(const nabo_cuda_search* h, int qRows, int64_t nq, int64_t qStride, int k, unsigned optionFlags,
              const void* maxRadii) {
  const bool allowSelf = optionFlags & NABO_ALLOW_SELF_MATCH;
  const int64_t cols = h->c.n;
  // nabo/nabo.cpp:105-115
  if (allowSelf) {
    if (k > cols)
      return set_error(kErrArgument, "Requesting more points (" + std::to_string(k) + ") than available in cloud (" +
                                         std::to_string(cols) + ")");
  } else {
    if (k > cols - 1)
      return set_error(kErrArgument, "Requesting more points (" + std::to_string(k) +
                                         ") than available in cloud minus 1 (" + std::to_string(cols - 1) +
                                         ") (as self match is forbidden)");
  }
  // nabo/nabo.cpp:116-117
  if (qRows < h->c.dim)
    return set_error(kErrArgument, "Query has less dimensions (" + std::to_string(qRows) +
                                       ") than requested for cloud (" + std::to_string(h->c.dim) + ")");
  // nabo/nabo.cpp:128-130
  const unsigned maxFlags = NABO_ALLOW_SELF_MATCH | NABO_SORT_RESULTS;
  if (optionFlags > maxFlags)
    return set_error(kErrArgument, "OR-ed value of option flags (" + std::to_string(optionFlags) +
                                       ") is larger than maximal valid value (" + std::to_string(maxFlags) + ")");
  (void)maxRadii;
  if (k < 1) return set_error(kErrArgument, "k must be at least 1");
  if (nq < 0) return set_error(kErrArgument, "negative query count");
  if (qStride < qRows) return set_error(kErrArgument, "query column stride is smaller than its row count");
  if (nq > (int64_t)std::numeric_limits<int32_t>::max())
    return set_error(kErrUnsupported, "at most 2^31-1 queries per call");
  return kOk;
}

}  // namespace

namespace nabo_gb300 {
HandleView handle_view(const nabo_cuda_search* s) {
  HandleView v;
  v.cloud = &s->c;
  v.searchType = s->searchType;
  v.creationFlags = s->creationFlags;
  v.device = s->device;
  v.traversal = s->traversal;
  v.sortQueries = s->queryOrdering != 0;
  v.evStart = s->evStart;
  v.evStop = s->evStop;
  return v;
}

int handle_check_knn(const nabo_cuda_search* s, int qRows, int64_t nq, int64_t qStride, int k, unsigned optionFlags,
                     const void* maxRadii) {
  return check_knn(s, qRows, nq, qStride, k, optionFlags, maxRadii);
}
}  // namespace nabo_gb300

extern "C" {

void nabo_cuda_params_init(nabo_cuda_params* p) {
  if (!p) return;
  std::memset(p, 0, sizeof(*p));
  p->struct_size = sizeof(nabo_cuda_params);
  p->bucketSize = 8;
  p->queryOrdering = 1;
}

int nabo_cuda_create(int dtype, const void* cloud, int rows, int64_t n, int64_t colStride, int dim, int searchType,
                     unsigned creationFlags, const nabo_cuda_params* params, nabo_cuda_search** out) {
  return create_impl(dtype, cloud, false, rows, n, colStride, dim, searchType, creationFlags, params, out);
}

int nabo_cuda_create_device(int dtype, const void* cloud, int rows, int64_t n, int64_t colStride, int dim,
                            int searchType, unsigned creationFlags, const nabo_cuda_params* params,
                            nabo_cuda_search** out) {
  return create_impl(dtype, cloud, true, rows, n, colStride, dim, searchType, creationFlags, params, out);
}

int nabo_cuda_destroy(nabo_cuda_search* s) {
  if (!s) return kOk;
  DeviceGuard g(s->device);
  free_events(s);
  free_stage(s);
  destroy_pipe(s->pipe);
  free_cloud(s->c);
  delete s;
  return kOk;
}

}  // extern "C"

namespace {

constexpr size_t kStageBytes = size_t(4) << 20;  // largest call staged
constexpr size_t kStageMinBytes = size_t(64) << 10;

size_t align16(size_t x) { return (x + 15) & ~size_t(15); }

void knn_args_common(const nabo_cuda_search* s, KnnArgs& a, int64_t nq, int k, double epsilon, unsigned optionFlags,
                     double maxRadius) {
  a.nq = nq;
  a.k = k;
  a.eps = epsilon;
  a.optionFlags = optionFlags;
  a.touchStats = (s->creationFlags & NABO_TOUCH_STATISTICS) != 0;
  a.maxRadius = maxRadius;
  a.sortQueries = s->queryOrdering != 0;
  a.traversal = s->traversal;
}

uint64_t touched_result(const nabo_cuda_search* s, int64_t nq, unsigned long long counted) {
  if (!(s->creationFlags & NABO_TOUCH_STATISTICS)) return 0;
  if (s->searchType == NABO_SEARCH_BRUTE_FORCE_CUDA) return (uint64_t)nq * (uint64_t)s->c.n;  // nabo/brute_force_cpu.cpp:99-100
  return counted;
}

// The host-buffer search through the object's staging blocks, laid out as
// [query (packed columns) | radii | touched | indices | dists2]: the upload
// covers query..touched (touched uploaded as 0), the download
// touched..dists2. Returns -1 when the call does not fit or the staging is
// in use by another thread.
int knn_staged(const nabo_cuda_search* s, const void* query, int qRows, int64_t nq, int64_t qStride, int k,
               double epsilon, unsigned optionFlags, double maxRadius, const void* maxRadii, int32_t* indices,
               void* dists2, uint64_t* touched) {
  const size_t es = s->c.dtype == NABO_CUDA_FLOAT32 ? 4 : 8;
  const size_t outN = (size_t)nq * (size_t)k;
  const size_t rowBytes = (size_t)qRows * es;
  const size_t offRadii = align16((size_t)nq * rowBytes);
  const size_t offTouched = align16(offRadii + (maxRadii ? (size_t)nq * es : 0));
  const size_t offIdx = offTouched + 16;
  const size_t offD2 = align16(offIdx + outN * sizeof(int32_t));
  const size_t total = align16(offD2 + outN * es);
  if (total > kStageBytes) return -1;
  std::unique_lock<std::mutex> lock(s->stageLock, std::try_to_lock);
  if (!lock.owns_lock()) return -1;
  cudaError_t e = cudaSuccess;
  if (s->stageBytes < total) {  // the blocks fit the calls seen so far: page-locked memory is scarce
    size_t bytes = std::max(kStageMinBytes, s->stageBytes);
    while (bytes < total) bytes *= 2;
    free_stage(const_cast<nabo_cuda_search*>(s));
    e = cudaMallocHost(&s->stageHost, bytes);
    if (e == cudaSuccess) e = cudaMalloc(&s->stageDev, bytes);
    if (e == cudaSuccess) s->stageBytes = bytes;
    if (e != cudaSuccess) {
      free_stage(const_cast<nabo_cuda_search*>(s));
      return cuda_error(e, "knn staging buffers");
    }
  }
  unsigned char* h = static_cast<unsigned char*>(s->stageHost);
  unsigned char* d = static_cast<unsigned char*>(s->stageDev);
  const unsigned char* q = static_cast<const unsigned char*>(query);
  if (qStride == qRows)
    std::memcpy(h, q, (size_t)nq * rowBytes);
  else
    for (int64_t i = 0; i < nq; ++i) std::memcpy(h + (size_t)i * rowBytes, q + (size_t)i * qStride * es, rowBytes);
  if (maxRadii) std::memcpy(h + offRadii, maxRadii, (size_t)nq * es);
  std::memset(h + offTouched, 0, 16);
  // upload, search, download on `st`
  auto enqueue = [&](cudaStream_t st) {
    cudaError_t ee = cudaMemcpyAsync(d, h, offTouched + 16, cudaMemcpyHostToDevice, st);
    if (ee != cudaSuccess) return cuda_error(ee, "knn upload");
    KnnArgs a;
    knn_args_common(s, a, nq, k, epsilon, optionFlags, maxRadius);
    a.query = d;
    a.qStride = qRows;
    a.maxRadii = maxRadii ? d + offRadii : nullptr;
    a.indices = reinterpret_cast<int32_t*>(d + offIdx);
    a.dists2 = d + offD2;
    a.touched = reinterpret_cast<unsigned long long*>(d + offTouched);
    int r = knn_any(s, a, st);
    if (r == kOk) {
      ee = cudaMemcpyAsync(h + offTouched, d + offTouched, total - offTouched, cudaMemcpyDeviceToHost, st);
      if (ee != cudaSuccess) r = cuda_error(ee, "knn download");
    }
    return r;
  };
  // the staging blocks are the graph's only buffers, so sizes and arguments
  // identify a call
  const PipeKey key = make_pipe_key(h, maxRadii ? h + offRadii : nullptr, d, nullptr, nq, qRows, epsilon, maxRadius,
                                    qRows, k, optionFlags, 0);
  const bool replay = !s->stageNoGraph && s->stageExec && same_key(s->stageGraphKey, key);
  bool capture = !s->stageNoGraph && !replay && s->stageHasLast && same_key(s->stageLastKey, key);
  s->stageLastKey = key;
  s->stageHasLast = true;
  if (capture) {
    if (s->stageExec) cudaGraphExecDestroy(s->stageExec);
    s->stageExec = nullptr;
    cudaError_t ce = s->stageStream ? cudaSuccess : cudaStreamCreateWithFlags(&s->stageStream, cudaStreamNonBlocking);
    int crc = kOk;
    if (ce == cudaSuccess) {
      set_capture_allocations(true);
      ce = cudaStreamBeginCapture(s->stageStream, cudaStreamCaptureModeThreadLocal);
      if (ce == cudaSuccess) {
        crc = enqueue(s->stageStream);
        cudaGraph_t graph = nullptr;
        ce = cudaStreamEndCapture(s->stageStream, &graph);
        if (crc == kOk && ce == cudaSuccess) ce = cudaGraphInstantiate(&s->stageExec, graph, 0);
        if (graph) cudaGraphDestroy(graph);
      }
      set_capture_allocations(false);
    }
    if (crc != kOk || ce != cudaSuccess) {  // not capturable here: direct calls from now on
      cudaGetLastError();
      if (s->stageExec) cudaGraphExecDestroy(s->stageExec);
      s->stageExec = nullptr;
      s->stageNoGraph = true;
      capture = false;
    } else {
      s->stageGraphKey = key;
    }
  }
  int rc = kOk;
  cudaStream_t st = cudaStreamPerThread;
  if (replay || capture) {
    st = s->stageStream;
    e = cudaGraphLaunch(s->stageExec, st);
    if (e != cudaSuccess) rc = cuda_error(e, "cudaGraphLaunch");
  } else {
    rc = enqueue(st);
  }
  e = cudaStreamSynchronize(st);
  if (rc == kOk && e != cudaSuccess) rc = cuda_error(e, "knn");
  if (rc != kOk) return rc;
  std::memcpy(indices, h + offIdx, outN * sizeof(int32_t));
  std::memcpy(dists2, h + offD2, outN * es);
  if (touched) {
    unsigned long long ht;
    std::memcpy(&ht, h + offTouched, sizeof(ht));
    *touched = touched_result(s, nq, ht);
  }
  return kOk;
}

// Errors by which the runtime refuses a stream capture or a graph as such
// (as opposed to a capture that some concurrent work invalidated).
bool capture_refused(cudaError_t e) {
  switch (e) {
    case cudaErrorStreamCaptureUnsupported:
    case cudaErrorStreamCaptureUnmatched:
    case cudaErrorStreamCaptureUnjoined:
    case cudaErrorStreamCaptureIsolation:
    case cudaErrorStreamCaptureImplicit:
    case cudaErrorStreamCaptureWrongThread:
    case cudaErrorNotSupported:
      return true;
    default:
      return false;
  }
}

bool is_pinned(const void* p) {
  cudaPointerAttributes attr;
  if (cudaPointerGetAttributes(&attr, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return attr.type == cudaMemoryTypeHost;
}

// The device address of a page-locked host buffer mapped into the device's
// address space, else nullptr.
const void* mapped_host(const void* p) {
  cudaPointerAttributes attr;
  if (cudaPointerGetAttributes(&attr, p) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  return attr.type == cudaMemoryTypeHost ? attr.devicePointer : nullptr;
}

// Large host-buffer searches whose result buffers are pinned: the queries
// are uploaded and ordered once, then searched in pipelineChunks
// consecutive chunks of shrinking size (the last chunk's download is the
// part that no search hides), one launch each on alternating streams, and a
// copy stream downloads each chunk's result rows as soon as its search is
// done, while the next chunk searches. With query ordering the order is
// chunk-major (each chunk's queries along the Morton curve), so a chunk's
// launch covers a contiguous part of one order. Results are those of one
// call: each query's result goes to its own column and the touched counter
// sums over the chunks. Returns -1 when the call is too small, a result
// buffer is not pinned, or the cloud has more than 3 dimensions with
// query ordering on.
constexpr int64_t kPipelineMin = int64_t(1) << 18;
constexpr int kPipelineChunks = 5;  // default

// The pipelined call's work (see knn_pipelined), enqueued on `main` and the
// streams of `pr`: upload, query order, one search launch per chunk, each
// chunk's download, the touched count into *hostTouched. Joins the other
// streams back into `main` even after an error; does not synchronise.
int pipeline_enqueue(const nabo_cuda_search* s, const PipeRes* pr, cudaStream_t main, const void* query, int qRows,
                     int64_t nq, int64_t qStride, int k, double epsilon, unsigned optionFlags, double maxRadius,
                     const void* maxRadii, int32_t* indices, void* dists2, const QueryChunks& chunks, bool ordered,
                     unsigned long long* hostTouched) {
  const size_t es = s->c.dtype == NABO_CUDA_FLOAT32 ? 4 : 8;
  const size_t qBytes = (size_t)((nq - 1) * qStride + qRows) * es;
  const size_t outN = (size_t)nq * (size_t)k;
  unsigned char *dq = nullptr, *dr = nullptr, *dd = nullptr;
  int32_t *di = nullptr, *order = nullptr;
  unsigned long long* dt = nullptr;
  int rc = kOk;
  cudaError_t e = cudaSuccess;
  const cudaStream_t* const comp = pr->comp;
  cudaStream_t copy = pr->copy;
  cudaEvent_t ready = pr->ready, copied = pr->copied;
  const cudaEvent_t* const searched = pr->searched;
  const cudaEvent_t* const compDone = pr->compDone;
  if (e == cudaSuccess) e = scratch_alloc((void**)&dq, qBytes, main);
  if (e == cudaSuccess && maxRadii) e = scratch_alloc((void**)&dr, (size_t)nq * es, main);
  if (e == cudaSuccess) e = scratch_alloc((void**)&di, outN * sizeof(int32_t), main);
  if (e == cudaSuccess) e = scratch_alloc((void**)&dd, outN * es, main);
  if (e == cudaSuccess) e = scratch_alloc((void**)&dt, sizeof(unsigned long long), main);
  if (e == cudaSuccess && ordered) e = scratch_alloc((void**)&order, (size_t)nq * sizeof(int32_t), main);
  // With query ordering and a device-mapped page-locked query buffer, the
  // Morton kernel reads the queries over the host link and writes them to
  // the device copy as it goes: the upload and the key pass in one.
  const void* hostQuery = ordered ? mapped_host(query) : nullptr;
  if (e == cudaSuccess && !hostQuery) e = cudaMemcpyAsync(dq, query, qBytes, cudaMemcpyHostToDevice, main);
  if (e == cudaSuccess && maxRadii) e = cudaMemcpyAsync(dr, maxRadii, (size_t)nq * es, cudaMemcpyHostToDevice, main);
  if (e == cudaSuccess) e = cudaMemsetAsync(dt, 0, sizeof(unsigned long long), main);
  if (e != cudaSuccess) rc = cuda_error(e, "knn pipeline setup");
  if (rc == kOk && ordered)
    rc = hostQuery ? chunk_order_any(s, hostQuery, nq, qStride, chunks, order, main, dq)
                   : chunk_order_any(s, dq, nq, qStride, chunks, order, main, nullptr);
  if (rc == kOk && cudaEventRecord(ready, main) != cudaSuccess) rc = cuda_error(cudaGetLastError(), "knn pipeline");
  for (int c = 0; c < chunks.n && rc == kOk; ++c) {
    const int64_t c0 = c ? chunks.end[c - 1] : 0, c1 = chunks.end[c];
    const int64_t m = c1 - c0;
    if (m <= 0) continue;
    cudaStream_t cs = comp[c & 1];
    e = cudaStreamWaitEvent(cs, ready, 0);
    if (e != cudaSuccess) {
      rc = cuda_error(e, "knn pipeline");
      break;
    }
    KnnArgs a;
    knn_args_common(s, a, m, k, epsilon, optionFlags, maxRadius);
    a.touched = dt;
    a.qStride = qStride;
    if (ordered) {  // the chunk's part of the order holds global query indices
      a.query = dq;
      a.maxRadii = dr;
      a.indices = di;
      a.dists2 = dd;
      rc = knn_given_order_any(s, a, order + c0, cs);
    } else {
      a.query = dq + (size_t)c0 * qStride * es;
      a.maxRadii = maxRadii ? dr + (size_t)c0 * es : nullptr;
      a.indices = di + (size_t)c0 * k;
      a.dists2 = dd + (size_t)c0 * k * es;
      rc = knn_any(s, a, cs);
    }
    if (rc != kOk) break;
    e = cudaEventRecord(searched[c], cs);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(copy, searched[c], 0);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(indices + (size_t)c0 * k, di + (size_t)c0 * k, (size_t)m * k * sizeof(int32_t),
                          cudaMemcpyDeviceToHost, copy);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(static_cast<unsigned char*>(dists2) + (size_t)c0 * k * es, dd + (size_t)c0 * k * es,
                          (size_t)m * k * es, cudaMemcpyDeviceToHost, copy);
    if (e != cudaSuccess) rc = cuda_error(e, "knn chunk download");
  }
  // the main stream waits for the compute and copy streams before the frees
  for (int i = 0; i < 2; ++i)
    if (comp[i] && cudaEventRecord(compDone[i], comp[i]) == cudaSuccess) cudaStreamWaitEvent(main, compDone[i], 0);
  if (copy && cudaEventRecord(copied, copy) == cudaSuccess) cudaStreamWaitEvent(main, copied, 0);
  if (rc == kOk) {
    e = cudaMemcpyAsync(hostTouched, dt, sizeof(*hostTouched), cudaMemcpyDeviceToHost, main);
    if (e != cudaSuccess) rc = cuda_error(e, "knn touched count");
  }
  for (void* p : {(void*)dq, (void*)dr, (void*)di, (void*)dd, (void*)dt, (void*)order})
    if (p) scratch_free(p, main);
  return rc;
}

int knn_pipelined(const nabo_cuda_search* s, const void* query, int qRows, int64_t nq, int64_t qStride, int k,
                  double epsilon, unsigned optionFlags, double maxRadius, const void* maxRadii, int32_t* indices,
                  void* dists2, uint64_t* touched) {
  const int nChunks = s->pipelineChunks > 0 ? s->pipelineChunks : kPipelineChunks;
  if (nq < kPipelineMin || nChunks < 2) return -1;
  if (!is_pinned(indices) || !is_pinned(dists2)) return -1;
  const bool ordered =
      s->searchType == NABO_SEARCH_KDTREE_CUDA && s->queryOrdering != 0 && worth_sorting(nq, k, s->c.dim);
  if (ordered && s->c.dim > 3) return -1;
  const QueryChunks chunks = shrinking_chunks(nq, nChunks);
  // the object's streams and events, or this call's own while another call holds them
  PipeRes own;
  PipeRes* pr = &own;
  std::unique_lock<std::mutex> lock(s->pipeLock, std::try_to_lock);
  if (lock.owns_lock() && (s->pipe.made || make_pipe(s->pipe) == cudaSuccess)) pr = &s->pipe;
  if (pr == &own) {
    const cudaError_t e = make_pipe(own);
    if (e != cudaSuccess) return cuda_error(e, "knn pipeline setup");
  }
  int rc = kOk;
  unsigned long long ht = 0;
  // A call that repeats the previous one (same page-locked buffers, same
  // arguments) runs as one CUDA graph of the whole call, captured on the
  // first repeat and replayed after; its copies read and write the buffers'
  // current contents.
  const PipeKey key = make_pipe_key(query, maxRadii, indices, dists2, nq, qStride, epsilon, maxRadius, qRows, k,
                                    optionFlags, nChunks);
  const bool graphable =
      pr == &s->pipe && !pr->noGraph && is_pinned(query) && (!maxRadii || is_pinned(maxRadii));
  const bool replay = graphable && pr->exec && same_key(pr->graphKey, key);
  bool capture = graphable && !replay && pr->hasLast && same_key(pr->lastKey, key);
  if (graphable) {
    pr->lastKey = key;
    pr->hasLast = true;
  }
  if (capture) {
    if (pr->exec) cudaGraphExecDestroy(pr->exec);
    pr->exec = nullptr;
    set_capture_allocations(true);
    g_lastCudaError = cudaSuccess;
    cudaError_t e = cudaStreamBeginCapture(pr->main, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) {
      rc = cuda_error(e, "cudaStreamBeginCapture");
    } else {
      rc = pipeline_enqueue(s, pr, pr->main, query, qRows, nq, qStride, k, epsilon, optionFlags, maxRadius,
                            maxRadii, indices, dists2, chunks, ordered, pr->hostTouched);
      cudaGraph_t graph = nullptr;
      e = cudaStreamEndCapture(pr->main, &graph);
      if (rc == kOk && e != cudaSuccess) rc = cuda_error(e, "cudaStreamEndCapture");
      if (rc == kOk) {
        e = cudaGraphInstantiate(&pr->exec, graph, 0);
        if (e != cudaSuccess) {
          pr->exec = nullptr;
          rc = cuda_error(e, "cudaGraphInstantiate");
        }
      }
      if (graph) cudaGraphDestroy(graph);
    }
    set_capture_allocations(false);
    if (rc == kOk) {
      pr->graphKey = key;
    } else {
      // This call runs directly instead (a real error recurs there). A
      // capture the runtime refuses (capture or graph not supported here)
      // turns graphs off for this object; any other failure, for example
      // another thread's legacy-stream work invalidating the capture, only
      // drops this graph, and a later repeat captures again.
      cudaGetLastError();
      if (pr->exec) cudaGraphExecDestroy(pr->exec);
      pr->exec = nullptr;
      pr->hasLast = false;
      if (capture_refused(g_lastCudaError)) pr->noGraph = true;
      capture = false;
      rc = kOk;
      g_lastError.clear();
    }
  }
  if (rc == kOk && (replay || capture)) {
    cudaError_t e = cudaGraphLaunch(pr->exec, pr->main);
    if (e == cudaSuccess) e = cudaStreamSynchronize(pr->main);
    if (e != cudaSuccess) rc = cuda_error(e, "knn");
    ht = *pr->hostTouched;
  } else if (rc == kOk) {
    cudaStream_t main = cudaStreamPerThread;
    rc = pipeline_enqueue(s, pr, main, query, qRows, nq, qStride, k, epsilon, optionFlags, maxRadius, maxRadii,
                          indices, dists2, chunks, ordered, &ht);
    const cudaError_t e = cudaStreamSynchronize(main);
    if (rc == kOk && e != cudaSuccess) rc = cuda_error(e, "knn");
  }
  if (pr == &own) destroy_pipe(own);
  if (rc == kOk && touched) *touched = touched_result(s, nq, ht);
  return rc;
}

}  // namespace

extern "C" {

int nabo_cuda_knn(const nabo_cuda_search* s, const void* query, int qRows, int64_t nq, int64_t qStride, int k,
                  double epsilon, unsigned optionFlags, double maxRadius, const void* maxRadii, int32_t* indices,
                  void* dists2, uint64_t* touched) {
  if (!s) return set_error(kErrArgument, "search object is NULL");
  int rc = check_knn(s, qRows, nq, qStride, k, optionFlags, maxRadii);
  if (rc != kOk) return rc;
  if (touched) *touched = 0;
  if (nq == 0) return kOk;
  if (!query || !indices || !dists2) return set_error(kErrArgument, "NULL query or result buffer");
  DeviceGuard g(s->device);
  if (!g.ok) return cuda_error(cudaGetLastError(), "cudaSetDevice");
  rc = knn_staged(s, query, qRows, nq, qStride, k, epsilon, optionFlags, maxRadius, maxRadii, indices, dists2,
                  touched);
  if (rc != -1) return rc;
  rc = knn_pipelined(s, query, qRows, nq, qStride, k, epsilon, optionFlags, maxRadius, maxRadii, indices, dists2,
                     touched);
  if (rc != -1) return rc;
  rc = kOk;
  cudaStream_t st = cudaStreamPerThread;
  const size_t es = s->c.dtype == NABO_CUDA_FLOAT32 ? 4 : 8;
  const size_t qBytes = (size_t)((nq - 1) * qStride + qRows) * es;
  const size_t outN = (size_t)nq * (size_t)k;
  void *dq = nullptr, *dr = nullptr, *dd = nullptr;
  int32_t* di = nullptr;
  unsigned long long* dt = nullptr;
  cudaError_t e = scratch_alloc(&dq, qBytes, st);
  if (e == cudaSuccess && maxRadii) e = scratch_alloc(&dr, (size_t)nq * es, st);
  if (e == cudaSuccess) e = scratch_alloc((void**)&di, outN * sizeof(int32_t), st);
  if (e == cudaSuccess) e = scratch_alloc(&dd, outN * es, st);
  if (e == cudaSuccess) e = scratch_alloc((void**)&dt, sizeof(unsigned long long), st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dq, query, qBytes, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess && maxRadii) e = cudaMemcpyAsync(dr, maxRadii, (size_t)nq * es, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemsetAsync(dt, 0, sizeof(unsigned long long), st);
  if (e != cudaSuccess) rc = cuda_error(e, "knn setup");
  if (rc == kOk) {
    KnnArgs a;
    knn_args_common(s, a, nq, k, epsilon, optionFlags, maxRadius);
    a.query = dq;
    a.qStride = qStride;
    a.maxRadii = dr;
    a.indices = di;
    a.dists2 = dd;
    a.touched = dt;
    rc = knn_any(s, a, st);
  }
  unsigned long long ht = 0;
  if (rc == kOk) {
    e = cudaMemcpyAsync(indices, di, outN * sizeof(int32_t), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dists2, dd, outN * es, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&ht, dt, sizeof(ht), cudaMemcpyDeviceToHost, st);
    if (e != cudaSuccess) rc = cuda_error(e, "knn results");
  }
  if (dq) scratch_free(dq, st);
  if (dr) scratch_free(dr, st);
  if (di) scratch_free(di, st);
  if (dd) scratch_free(dd, st);
  if (dt) scratch_free(dt, st);
  e = cudaStreamSynchronize(st);
  if (rc == kOk && e != cudaSuccess) rc = cuda_error(e, "knn");
  if (rc == kOk && touched) *touched = touched_result(s, nq, ht);
  return rc;
}

int nabo_cuda_knn_device(const nabo_cuda_search* s, const void* query, int qRows, int64_t nq, int64_t qStride,
                         int k, double epsilon, unsigned optionFlags, double maxRadius, const void* maxRadii,
                         int32_t* indices, void* dists2, uint64_t* touched, void* stream) {
  if (!s) return set_error(kErrArgument, "search object is NULL");
  int rc = check_knn(s, qRows, nq, qStride, k, optionFlags, maxRadii);
  if (rc != kOk) return rc;
  if (nq == 0) return kOk;
  if (!query || !indices || !dists2) return set_error(kErrArgument, "NULL query or result buffer");
  DeviceGuard g(s->device);
  if (!g.ok) return cuda_error(cudaGetLastError(), "cudaSetDevice");
  KnnArgs a;
  a.query = query;
  a.nq = nq;
  a.qStride = qStride;
  a.k = k;
  a.eps = epsilon;
  a.optionFlags = optionFlags;
  a.touchStats = (s->creationFlags & NABO_TOUCH_STATISTICS) != 0 && s->searchType == NABO_SEARCH_KDTREE_CUDA;
  a.maxRadius = maxRadius;
  a.maxRadii = maxRadii;
  a.indices = indices;
  a.dists2 = dists2;
  a.touched = reinterpret_cast<unsigned long long*>(touched);
  a.sortQueries = s->queryOrdering != 0;
  a.traversal = s->traversal;
  a.evStart = s->evStart;
  a.evStop = s->evStop;
  return knn_any(s, a, static_cast<cudaStream_t>(stream));
}

int nabo_cuda_profile(nabo_cuda_search* s, int enable) {
  if (!s) return set_error(kErrArgument, "search object is NULL");
  DeviceGuard g(s->device);
  free_events(s);
  if (enable) {
    cudaError_t e = cudaEventCreate(&s->evStart);
    if (e == cudaSuccess) e = cudaEventCreate(&s->evStop);
    if (e != cudaSuccess) {
      free_events(s);
      return cuda_error(e, "cudaEventCreate");
    }
  }
  return kOk;
}

int nabo_cuda_last_kernel_ms(const nabo_cuda_search* s, float* ms) {
  if (!s || !ms) return set_error(kErrArgument, "NULL argument");
  if (!s->evStart) return set_error(kErrArgument, "profiling is not enabled on this search object");
  DeviceGuard g(s->device);
  cudaError_t e = cudaEventSynchronize(s->evStop);
  if (e == cudaSuccess) e = cudaEventElapsedTime(ms, s->evStart, s->evStop);
  if (e != cudaSuccess) return cuda_error(e, "kernel timing");
  return kOk;
}

int nabo_cuda_get_info(const nabo_cuda_search* s, int64_t info[8]) {
  if (!s || !info) return set_error(kErrArgument, "NULL argument");
  info[0] = s->c.dim;
  info[1] = s->c.n;
  info[2] = s->c.dtype;
  info[3] = s->searchType;
  info[4] = s->creationFlags;
  info[5] = s->c.bucketSize;
  info[6] = s->c.nodeCount;
  info[7] = s->c.height;
  return kOk;
}

int nabo_cuda_get_bounds(const nabo_cuda_search* s, void* minBound, void* maxBound) {
  if (!s) return set_error(kErrArgument, "search object is NULL");
  for (int d = 0; d < s->c.dim; ++d) {
    if (s->c.dtype == NABO_CUDA_FLOAT32) {
      if (minBound) static_cast<float*>(minBound)[d] = (float)s->minBound[d];
      if (maxBound) static_cast<float*>(maxBound)[d] = (float)s->maxBound[d];
    } else {
      if (minBound) static_cast<double*>(minBound)[d] = s->minBound[d];
      if (maxBound) static_cast<double*>(maxBound)[d] = s->maxBound[d];
    }
  }
  return kOk;
}

int nabo_cuda_export_tree(const nabo_cuda_search* s, int32_t* cutDim, void* cutVal, uint32_t* right,
                          uint32_t* bucketStart, uint32_t* bucketSize, int32_t* buckets) {
  if (!s) return set_error(kErrArgument, "search object is NULL");
  if (s->searchType != NABO_SEARCH_KDTREE_CUDA) return set_error(kErrArgument, "not a kd-tree search object");
  DeviceGuard g(s->device);
  const bool f32 = s->c.dtype == NABO_CUDA_FLOAT32;
  const size_t nodeBytes = f32 ? 8 : 16;
  std::vector<unsigned char> nodes((size_t)s->c.nodeCount * nodeBytes);
  cudaError_t e = cudaMemcpy(nodes.data(), s->c.nodes, nodes.size(), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_error(e, "export nodes");
  for (int64_t i = 0; i < s->c.nodeCount; ++i) {
    const unsigned char* p = nodes.data() + i * nodeBytes;
    uint32_t meta, start;
    std::memcpy(&meta, p, 4);
    std::memcpy(&start, p + 4, 4);
    const bool leaf = node_is_leaf(meta);
    if (cutDim) cutDim[i] = leaf ? -1 : (int32_t)node_dim(meta);
    if (right) right[i] = leaf ? 0u : node_payload(meta);
    if (bucketStart) bucketStart[i] = leaf ? start : 0u;
    if (bucketSize) bucketSize[i] = leaf ? node_payload(meta) : 0u;
    if (cutVal) {
      if (f32) {
        float v = 0.0f;
        if (!leaf) std::memcpy(&v, p + 4, 4);
        static_cast<float*>(cutVal)[i] = v;
      } else {
        double v = 0.0;
        if (!leaf) std::memcpy(&v, p + 8, 8);
        static_cast<double*>(cutVal)[i] = v;
      }
    }
  }
  if (buckets) {
    const size_t es = f32 ? 4 : 8;
    const size_t recBytes = ((size_t)s->c.dpad * es + 4 + 15) / 16 * 16;
    std::vector<unsigned char> recs((size_t)s->c.n * recBytes);
    e = cudaMemcpy(recs.data(), s->c.recs, recs.size(), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_error(e, "export buckets");
    for (int64_t i = 0; i < s->c.n; ++i) std::memcpy(buckets + i, recs.data() + i * recBytes + s->c.dpad * es, 4);
  }
  return kOk;
}

const char* nabo_cuda_last_error(void) { return g_lastError.c_str(); }

const char* nabo_cuda_version(void) { return NABO_GB300_VERSION; }

}  // extern "C"
