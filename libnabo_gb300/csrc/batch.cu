// batch.cu -- many clouds of uneven sizes built and searched together.
//
// The clouds of a batch are stored back to back; their trees are built in
// one forest build (all segments of all clouds share each level's kernels;
// a fixed number of levels runs with no host synchronisation) and all their
// queries are searched by one launch of the kd-tree kernel, each query in
// its own cloud's tree with that cloud's k. nabo_cuda_batch_run captures
// build + search into a CUDA graph on first use and replays it afterwards,
// so a new batch of the same shape (new coordinates written to the same
// buffers) costs one graph launch. nabo_cuda_batch_run_host does the same
// from host buffers; page-locked ones are copied inside the graph, on a
// branch that overlaps the copies with the work (see capture_host).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <type_traits>
#include <vector>

#include "internal.cuh"
#include "nabo_gb300.h"

using namespace nabo_gb300;

struct nabo_cuda_batch {
  int dtype = 0;
  int dim = 0;
  int dpad = 0;
  int nClouds = 0;
  int64_t nTotal = 0;
  unsigned bucketSize = 8;
  int splitRule = 0;  // 0: the reference's sliding midpoint; 1: median
  int lanesPerQuery = 1;
  int maxLevels = 48;
  int blockSize = 128;
  int device = 0;
  int64_t* dOff = nullptr;
  void* recs = nullptr;
  void* nodes = nullptr;
  int64_t* nodeOffset = nullptr;
  void* rootBox = nullptr;
  int* status = nullptr;
  void* recs32 = nullptr;    // f64: float copies of recs for the search's pre-filter
  float* coordMax = nullptr;
  // query plan
  int64_t nq = 0;
  int kMax = 0;
  int64_t outTotal = 0;
  int64_t* dQOff = nullptr;
  int64_t* dOutOff = nullptr;
  int32_t* dK = nullptr;
  int32_t* order = nullptr;
  uint32_t* hist = nullptr;
  uint32_t* cell = nullptr;
  uint32_t* rank = nullptr;
  // trees taller than the search kernels' stacks: the deep search's stacks
  int64_t nMax = 0;  // points of the largest cloud
  void* slab = nullptr;
  int64_t slabBytes = 0;
  // captured graph and the arguments it was captured with
  cudaGraphExec_t exec = nullptr;
  const void* gClouds = nullptr;
  const void* gQuery = nullptr;
  int32_t* gIdx = nullptr;
  void* gD2 = nullptr;
  double gEps = 0.0, gRadius = 0.0;
  unsigned gFlags = 0;
  // host-buffer runs: the plan's offsets on the host, device copies of the
  // inputs and results, two streams and the graph of the last page-locked call
  std::vector<int64_t> hQOff, hOutOff;
  BatchClassPlan plan;  // search launches by compiled top-k size
  // two more streams and their events, for the plan's groups side by side
  cudaStream_t aux[2] = {nullptr, nullptr};
  cudaEvent_t evFork = nullptr;
  cudaEvent_t evJoin[2] = {nullptr, nullptr};
  int groups = 8;
  void* devClouds = nullptr;
  void* devQueries = nullptr;
  int32_t* devIdx = nullptr;
  void* devD2 = nullptr;
  cudaStream_t hostStream = nullptr;
  cudaStream_t copyStream = nullptr;
  cudaGraphExec_t hostExec = nullptr;
  const void* hClouds = nullptr;
  const void* hQuery = nullptr;
  int32_t* hIdx = nullptr;
  void* hD2 = nullptr;
  double hEps = 0.0, hRadius = 0.0;
  unsigned hFlags = 0;
};

namespace {

struct Guard {
  int prev = -1;
  explicit Guard(int dev) {
    if (cudaGetDevice(&prev) == cudaSuccess && prev != dev) cudaSetDevice(dev);
  }
  ~Guard() {
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

void drop_graph(nabo_cuda_batch* b) {
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->hostExec) cudaGraphExecDestroy(b->hostExec);
  b->exec = nullptr;
  b->hostExec = nullptr;
}

void free_query_plan(nabo_cuda_batch* b) {
  for (void* p : {(void*)b->dQOff, (void*)b->dOutOff, (void*)b->dK, (void*)b->order, (void*)b->hist,
                  (void*)b->cell, (void*)b->rank, b->devQueries, (void*)b->devIdx, b->devD2, b->slab})
    if (p) cudaFree(p);
  b->slab = nullptr;
  b->slabBytes = 0;
  b->dQOff = b->dOutOff = nullptr;
  b->dK = b->order = nullptr;
  b->hist = b->cell = b->rank = nullptr;
  b->devQueries = b->devD2 = nullptr;
  b->devIdx = nullptr;
  b->hQOff.clear();
  b->hOutOff.clear();
  for (void* p : {(void*)b->plan.dRunCloud, (void*)b->plan.dRunPrefix})
    if (p) cudaFree(p);
  b->plan = BatchClassPlan();
}

// Groups the clouds by the top-k size compiled for their k (k <= 32; a
// batch with a larger k searches all queries by lane groups instead).
cudaError_t make_class_plan(nabo_cuda_batch* b, const std::vector<int32_t>& ks,
                            const std::vector<int64_t>& qoff) {
  BatchClassPlan& p = b->plan;
  p = BatchClassPlan();
  if (b->kMax > kMaxK) return cudaSuccess;
  std::vector<int> sizes;
  for (int32_t k : ks) sizes.push_back(round_k(k));
  std::sort(sizes.begin(), sizes.end());
  sizes.erase(std::unique(sizes.begin(), sizes.end()), sizes.end());
  p.runPrefix.push_back(0);
  for (int K : sizes) {
    const int first = (int)p.runCloud.size();
    for (int c = 0; c < b->nClouds; ++c) {
      const int64_t cnt = qoff[(size_t)c + 1] - qoff[(size_t)c];
      if (round_k(ks[(size_t)c]) != K || cnt == 0) continue;
      p.runCloud.push_back(c);
      p.runPrefix.push_back(p.runPrefix.back() + cnt);
    }
    if ((int)p.runCloud.size() == first) continue;
    p.K.push_back(K);
    p.runBegin.push_back(first);
  }
  p.groups = (int)p.K.size();
  p.runBegin.push_back((int)p.runCloud.size());
  if (p.groups == 0) return cudaSuccess;
  cudaError_t e = cudaMalloc((void**)&p.dRunCloud, p.runCloud.size() * sizeof(int32_t));
  if (e == cudaSuccess) e = cudaMalloc((void**)&p.dRunPrefix, p.runPrefix.size() * sizeof(int64_t));
  if (e == cudaSuccess)
    e = cudaMemcpy(p.dRunCloud, p.runCloud.data(), p.runCloud.size() * sizeof(int32_t), cudaMemcpyHostToDevice);
  if (e == cudaSuccess)
    e = cudaMemcpy(p.dRunPrefix, p.runPrefix.data(), p.runPrefix.size() * sizeof(int64_t), cudaMemcpyHostToDevice);
  return e;
}

// f(T(), std::integral_constant<int, D>()) for the batch's scalar type and
// compiled record dimension.
template <typename F>
int dispatch(const nabo_cuda_batch* b, F&& f) {
  using std::integral_constant;
  if (b->dtype == NABO_CUDA_FLOAT32) {
    switch (b->dpad) {
      case 2: return f(float(), integral_constant<int, 2>());
      case 3: return f(float(), integral_constant<int, 3>());
      case 4: return f(float(), integral_constant<int, 4>());
      case 8: return f(float(), integral_constant<int, 8>());
      case 16: return f(float(), integral_constant<int, 16>());
    }
  } else {
    switch (b->dpad) {
      case 2: return f(double(), integral_constant<int, 2>());
      case 3: return f(double(), integral_constant<int, 3>());
      case 4: return f(double(), integral_constant<int, 4>());
      case 8: return f(double(), integral_constant<int, 8>());
      case 16: return f(double(), integral_constant<int, 16>());
    }
  }
  return set_error(kErrInternal, "bad dispatch");
}

int build(nabo_cuda_batch* b, const void* clouds, cudaStream_t st) {
  ForestOut f;
  f.recs = b->recs;
  f.nodes = b->nodes;
  f.nodeCap = 2 * b->nTotal;
  f.nodeOffset = b->nodeOffset;
  const size_t es = b->dtype == NABO_CUDA_FLOAT32 ? 4 : 8;
  f.rootLo = b->rootBox;
  f.rootHi = static_cast<unsigned char*>(b->rootBox) + (size_t)b->nClouds * kMaxDim * es;
  f.status = b->status;
  // status[4]: the deep search's failure flag, cleared with each build
  const cudaError_t e = cudaMemsetAsync(b->status + 4, 0, sizeof(int), st);
  if (e != cudaSuccess) return cuda_error(e, "batch status");
#define NABO_B_CASE(TT, DD)                                                                                \
  if (b->dpad == DD) {                                                                                     \
    const int rc = build_forest<TT, DD>(static_cast<const TT*>(clouds), b->nTotal, b->dim, b->dim,        \
                                        b->bucketSize, b->dOff, b->nClouds, b->maxLevels, st, &f,          \
                                        b->splitRule);                                                     \
    if (rc != kOk || !b->recs32) return rc;                                                                \
    return narrow_records<DD>(b->recs, b->nTotal, b->dim, b->recs32, b->coordMax, st);                   \
  }
  if (b->dtype == NABO_CUDA_FLOAT32) {
    NABO_B_CASE(float, 2) NABO_B_CASE(float, 3) NABO_B_CASE(float, 4) NABO_B_CASE(float, 8) NABO_B_CASE(float, 16)
  } else {
    NABO_B_CASE(double, 2) NABO_B_CASE(double, 3) NABO_B_CASE(double, 4) NABO_B_CASE(double, 8)
    NABO_B_CASE(double, 16)
  }
#undef NABO_B_CASE
  return set_error(kErrInternal, "bad dispatch");
}

BatchArgs batch_args(const nabo_cuda_batch* b, const void* query, double eps, unsigned flags, double maxRadius,
                     int32_t* indices, void* dists2) {
  BatchArgs a;
  a.nodes = b->nodes;
  a.recs = b->recs;
  a.dim = b->dim;
  a.nClouds = b->nClouds;
  a.nodeCap = 2 * b->nTotal;
  a.nodeOffset = b->nodeOffset;
  a.qOffset = b->dQOff;
  a.outOffset = b->dOutOff;
  a.kOf = b->dK;
  a.kMax = b->kMax;
  a.query = query;
  a.nq = b->nq;
  a.qStride = b->dim;
  a.eps = eps;
  a.optionFlags = flags;
  a.maxRadius = maxRadius;
  a.indices = indices;
  a.dists2 = dists2;
  a.order = b->order;
  a.hist = b->hist;
  a.cell = b->cell;
  a.rank = b->rank;
  a.blockSize = b->blockSize;
  a.recs32 = b->recs32;
  a.coordMax = b->coordMax;
  a.slab = b->slab;
  a.slabBytes = b->slabBytes;
  a.heightDev = b->status + 2;
  a.deepFail = b->status + 4;
  a.maxRadii = nullptr;
  a.fallbacks = nullptr;
  a.lanesPerQuery = b->lanesPerQuery;
  a.classes = &b->plan;
  a.hQOffset = b->hQOff.empty() ? nullptr : b->hQOff.data();
  a.aux[0] = b->aux[0];
  a.aux[1] = b->aux[1];
  a.evFork = b->evFork;
  a.evJoin[0] = b->evJoin[0];
  a.evJoin[1] = b->evJoin[1];
  return a;
}

int search(nabo_cuda_batch* b, const void* query, double eps, unsigned flags, double maxRadius, int32_t* indices,
           void* dists2, cudaStream_t st, const void* radii = nullptr, int32_t* fallbacks = nullptr) {
  BatchArgs a = batch_args(b, query, eps, flags, maxRadius, indices, dists2);
  a.maxRadii = radii;
  a.fallbacks = fallbacks;
  return dispatch(b, [&](auto t, auto d) { return knn_batch<decltype(t), decltype(d)::value>(a, st); });
}

size_t elem_bytes(const nabo_cuda_batch* b) { return b->dtype == NABO_CUDA_FLOAT32 ? 4 : 8; }

// Bytes one tree level takes in a deep search's stack: the one-thread
// search's entry (rd, the offsets and the node in 16-byte chunks) or the
// group search's (the same without padding), whichever is larger.
int64_t stack_level_bytes(const nabo_cuda_batch* b) {
  const int64_t tw = (int64_t)elem_bytes(b) / 4;
  const int64_t words = tw * (b->dpad + 1) + 1;
  const int64_t one = (words + 3) / 4 * 16;
  const int64_t group = (b->dpad + 1) * (int64_t)elem_bytes(b) + 4;
  return std::max(one, group);
}

// Device copies of a host run's inputs and results, streams; made on first use.
int host_buffers(nabo_cuda_batch* b) {
  const size_t es = elem_bytes(b);
  cudaError_t e = cudaSuccess;
  if (!b->hostStream) e = cudaStreamCreateWithFlags(&b->hostStream, cudaStreamNonBlocking);
  if (e == cudaSuccess && !b->copyStream) e = cudaStreamCreateWithFlags(&b->copyStream, cudaStreamNonBlocking);
  if (e == cudaSuccess && !b->devClouds) e = cudaMalloc(&b->devClouds, (size_t)b->nTotal * b->dim * es);
  if (e == cudaSuccess && !b->devQueries) e = cudaMalloc(&b->devQueries, (size_t)std::max<int64_t>(b->nq, 1) * b->dim * es);
  if (e == cudaSuccess && !b->devIdx) e = cudaMalloc((void**)&b->devIdx, (size_t)std::max<int64_t>(b->outTotal, 1) * 4);
  if (e == cudaSuccess && !b->devD2) e = cudaMalloc(&b->devD2, (size_t)std::max<int64_t>(b->outTotal, 1) * es);
  return e == cudaSuccess ? kOk : cuda_error(e, "batch host-run buffers");
}

// True if [p, p + bytes) starts and ends in page-locked host memory.
bool pinned_range(const void* p, size_t bytes) {
  if (bytes == 0) return true;
  for (const void* q : {p, (const void*)(static_cast<const unsigned char*>(p) + bytes - 1)}) {
    cudaPointerAttributes attr;
    if (cudaPointerGetAttributes(&attr, q) != cudaSuccess) {
      cudaGetLastError();
      return false;
    }
    if (attr.type != cudaMemoryTypeHost) return false;
  }
  return true;
}

// Download groups: runs of whole clouds [cuts[i], cuts[i+1]) of about
// outTotal / groups result entries each (a cloud's results are contiguous
// only as a whole; see order_batch).
std::vector<int> group_cuts(const nabo_cuda_batch* b) {
  std::vector<int> cuts{0};
  for (int g = 1; g < b->groups; ++g) {
    const int64_t target = b->outTotal * g / b->groups;
    int c = cuts.back();
    while (c < b->nClouds && b->hOutOff[(size_t)c] < target) ++c;
    if (c > cuts.back() && c < b->nClouds) cuts.push_back(c);
  }
  cuts.push_back(b->nClouds);
  return cuts;
}

// The page-locked host run as one graph with two branches. Copy branch:
// clouds up, queries up (during the build), then each group's results down
// as soon as its search is done. Work branch: forest build once the clouds
// are in, query order once the queries are in, then one search launch per
// group of clouds, so downloads overlap the remaining searches.
int capture_host(nabo_cuda_batch* b, const void* clouds, const void* queries, double eps, unsigned flags,
                 double maxRadius, int32_t* indices, void* dists2) {
  const size_t es = elem_bytes(b);
  cudaStream_t st = b->hostStream, cp = b->copyStream;
  int rc = kOk;
  auto check = [&](cudaError_t e, const char* what) {
    if (rc == kOk && e != cudaSuccess) rc = cuda_error(e, what);
    return rc == kOk;
  };
  // events for the links between the branches, made before the capture
  std::vector<cudaEvent_t> events((size_t)b->groups + 4, nullptr);
  for (cudaEvent_t& ev : events) check(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming), "cudaEventCreate");
  size_t used = 0;
  // `to` waits for the work enqueued so far on `from` (tried even after an
  // error, so that the copy branch is always joined before the capture ends)
  auto link = [&](cudaStream_t from, cudaStream_t to) {
    if (used >= events.size() || !events[used]) return;
    cudaEvent_t ev = events[used++];
    cudaError_t e = cudaEventRecord(ev, from);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(to, ev, 0);
    check(e, "stream link");
  };
  const BatchArgs a = batch_args(b, b->devQueries, eps, flags, maxRadius, b->devIdx, b->devD2);
  set_capture_allocations(true);
  if (rc == kOk && check(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal), "cudaStreamBeginCapture")) {
    link(st, cp);
    if (rc == kOk)
      check(cudaMemcpyAsync(b->devClouds, clouds, (size_t)b->nTotal * b->dim * es, cudaMemcpyHostToDevice, cp),
            "cloud upload");
    link(cp, st);
    if (rc == kOk) rc = build(b, b->devClouds, st);
    if (rc == kOk && b->nq > 0) {
      check(cudaMemcpyAsync(b->devQueries, queries, (size_t)b->nq * b->dim * es, cudaMemcpyHostToDevice, cp),
            "query upload");
      link(cp, st);
      if (rc == kOk)
        rc = dispatch(b, [&](auto t, auto d) { return order_batch<decltype(t), decltype(d)::value>(a, st); });
      const std::vector<int> cuts = group_cuts(b);
      for (size_t g = 0; rc == kOk && g + 1 < cuts.size(); ++g) {
        const int64_t q0 = b->hQOff[(size_t)cuts[g]], q1 = b->hQOff[(size_t)cuts[g + 1]];
        const int64_t o0 = b->hOutOff[(size_t)cuts[g]], o1 = b->hOutOff[(size_t)cuts[g + 1]];
        rc = dispatch(b, [&](auto t, auto d) {
          return search_batch<decltype(t), decltype(d)::value>(a, q0, q1, st);
        });
        link(st, cp);
        if (rc == kOk && o1 > o0) {
          check(cudaMemcpyAsync(indices + o0, b->devIdx + o0, (size_t)(o1 - o0) * 4, cudaMemcpyDeviceToHost, cp),
                "index download");
          check(cudaMemcpyAsync(static_cast<unsigned char*>(dists2) + o0 * es,
                                static_cast<unsigned char*>(b->devD2) + o0 * es, (size_t)(o1 - o0) * es,
                                cudaMemcpyDeviceToHost, cp),
                "distance download");
        }
      }
    }
    link(cp, st);  // join the copy branch
    cudaGraph_t graph = nullptr;
    const cudaError_t e = cudaStreamEndCapture(st, &graph);
    check(e, "cudaStreamEndCapture");
    if (rc == kOk) check(cudaGraphInstantiate(&b->hostExec, graph, 0), "cudaGraphInstantiate");
    if (graph) cudaGraphDestroy(graph);
  }
  set_capture_allocations(false);
  for (cudaEvent_t ev : events)
    if (ev) cudaEventDestroy(ev);
  if (rc != kOk) b->hostExec = nullptr;
  return rc;
}

}  // namespace

namespace nabo_gb300 {
int batch_view(const nabo_cuda_batch* b, BatchView* v) {
  if (!b) return set_error(kErrArgument, "NULL batch");
  if (!b->dQOff) return set_error(kErrArgument, "call nabo_cuda_batch_set_queries first");
  v->dtype = b->dtype;
  v->dim = b->dim;
  v->dpad = b->dpad;
  v->nClouds = b->nClouds;
  v->kMax = b->kMax;
  v->device = b->device;
  v->nq = b->nq;
  v->nodes = b->nodes;
  v->recs = b->recs;
  v->pointOff = b->dOff;
  v->nodeOffset = b->nodeOffset;
  v->rootLo = b->rootBox;
  v->rootHi = static_cast<const unsigned char*>(b->rootBox) + (size_t)b->nClouds * kMaxDim * elem_bytes(b);
  v->qOffset = b->dQOff;
  v->outOffset = b->dOutOff;
  v->kOf = b->dK;
  return kOk;
}
}  // namespace nabo_gb300

extern "C" {

int nabo_cuda_batch_create(int dtype, int dim, int nClouds, const int64_t* pointCounts,
                           const nabo_cuda_params* params, int maxLevels, nabo_cuda_batch** out) {
  if (!out || !pointCounts) return set_error(kErrArgument, "NULL argument");
  *out = nullptr;
  if (dtype != NABO_CUDA_FLOAT32 && dtype != NABO_CUDA_FLOAT64) return set_error(kErrArgument, "unknown scalar type");
  if (dim <= 0) return set_error(kErrArgument, "Your space must have at least one dimension");
  if (nClouds < 1) return set_error(kErrArgument, "a batch needs at least one cloud");
  const int dpad = pad_dim(dim);
  if (dpad < 0) return set_error(kErrUnsupported, "the CUDA search types support at most 16 dimensions");
  nabo_cuda_params p;
  nabo_cuda_params_init(&p);
  if (params) {
    p.bucketSize = params->bucketSize;
    p.threadsPerBlock = params->threadsPerBlock;
    p.pipelineChunks = params->pipelineChunks;
    p.splitRule = params->splitRule;
    p.lanesPerQuery = params->lanesPerQuery;
  }
  if (p.pipelineChunks < 0 || p.pipelineChunks > 64)
    return set_error(kErrArgument, "pipelineChunks must be between 0 and 64");
  if (p.splitRule != 0 && p.splitRule != 1) return set_error(kErrArgument, "splitRule must be 0 or 1");
  if (p.lanesPerQuery != 0 && p.lanesPerQuery != 1 && p.lanesPerQuery != 8)
    return set_error(kErrArgument, "lanesPerQuery must be 1 or 8");
  if (p.bucketSize < 2)
    return set_error(kErrArgument, "Requested bucket size " + std::to_string(p.bucketSize) + ", but must be larger than 2");
  int64_t total = 0;
  for (int c = 0; c < nClouds; ++c) {
    if (pointCounts[c] <= 0) return set_error(kErrArgument, "Cloud has no points");
    total += pointCounts[c];
  }
  if (total > (int64_t)1 << 30) return set_error(kErrUnsupported, "a batch holds at most 2^30 points");
  nabo_cuda_batch* b = new nabo_cuda_batch();
  b->dtype = dtype;
  b->dim = dim;
  b->dpad = dpad;
  b->nClouds = nClouds;
  b->nTotal = total;
  b->bucketSize = p.bucketSize;
  b->maxLevels = maxLevels > 0 ? maxLevels : 48;
  b->blockSize = p.threadsPerBlock > 0 ? p.threadsPerBlock : 128;
  b->splitRule = p.splitRule;
  b->lanesPerQuery = p.lanesPerQuery == 8 ? 8 : 1;
  // 8 groups: host run of 512 clouds, 22 M queries, median of 10 calls, each
  // group searching with one launch per compiled top-k size side by side:
  // 2 groups 25.05 ms, 4 23.46, 8 23.00, 16 23.29 (those launches one after
  // another: 25.65, 24.40, 24.67, 25.83)
  b->groups = p.pipelineChunks > 0 ? p.pipelineChunks : 8;
  if (b->blockSize != 32 && b->blockSize != 64 && b->blockSize != 128) {
    delete b;
    return set_error(kErrArgument, "threads per block must be 32, 64 or 128");
  }
  cudaGetDevice(&b->device);
  const size_t es = dtype == NABO_CUDA_FLOAT32 ? 4 : 8;
  const size_t recBytes = ((size_t)dpad * es + 4 + 15) / 16 * 16;
  const size_t nodeBytes = dtype == NABO_CUDA_FLOAT32 ? 8 : 16;
  std::vector<int64_t> off((size_t)nClouds + 1, 0);
  for (int c = 0; c < nClouds; ++c) {
    off[(size_t)c + 1] = off[(size_t)c] + pointCounts[c];
    b->nMax = std::max<int64_t>(b->nMax, pointCounts[c]);
  }
  cudaError_t e = cudaMalloc((void**)&b->dOff, off.size() * sizeof(int64_t));
  if (e == cudaSuccess) e = cudaMalloc(&b->recs, (size_t)total * recBytes);
  if (e == cudaSuccess) e = cudaMalloc(&b->nodes, (size_t)2 * total * nodeBytes);
  if (e == cudaSuccess) e = cudaMalloc((void**)&b->nodeOffset, off.size() * sizeof(int64_t));
  if (e == cudaSuccess) e = cudaMalloc(&b->rootBox, (size_t)2 * nClouds * kMaxDim * es);
  if (e == cudaSuccess) e = cudaMalloc((void**)&b->status, 8 * sizeof(int));
  if (e == cudaSuccess && dtype == NABO_CUDA_FLOAT64) {
    const size_t rec32 = ((size_t)dpad * 4 + 4 + 15) / 16 * 16;  // sizeof(Rec<float, dpad>)
    e = cudaMalloc(&b->recs32, (size_t)total * rec32);
    if (e == cudaSuccess) e = cudaMalloc((void**)&b->coordMax, sizeof(float));
  }
  if (e == cudaSuccess) e = cudaMemcpy(b->dOff, off.data(), off.size() * sizeof(int64_t), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemset(b->status, 0, 8 * sizeof(int));
  if (e != cudaSuccess) {
    nabo_cuda_batch_destroy(b);
    return cuda_error(e, "batch allocation");
  }
  *out = b;
  return kOk;
}

int nabo_cuda_batch_destroy(nabo_cuda_batch* b) {
  if (!b) return kOk;
  Guard g(b->device);
  drop_graph(b);
  free_query_plan(b);
  for (void* p : {(void*)b->dOff, b->recs, b->nodes, (void*)b->nodeOffset, b->rootBox, (void*)b->status, b->recs32,
                  (void*)b->coordMax, b->devClouds})
    if (p) cudaFree(p);
  for (cudaStream_t st : {b->hostStream, b->copyStream, b->aux[0], b->aux[1]})
    if (st) cudaStreamDestroy(st);
  for (cudaEvent_t ev : {b->evFork, b->evJoin[0], b->evJoin[1]})
    if (ev) cudaEventDestroy(ev);
  delete b;
  return kOk;
}

int nabo_cuda_batch_set_queries(nabo_cuda_batch* b, const int64_t* queryCounts, const int32_t* k) {
  if (!b || !queryCounts || !k) return set_error(kErrArgument, "NULL argument");
  Guard g(b->device);
  int64_t nq = 0, outTotal = 0;
  int kMax = 0;
  std::vector<int64_t> qoff((size_t)b->nClouds + 1, 0), ooff((size_t)b->nClouds + 1, 0);
  std::vector<int32_t> ks((size_t)b->nClouds);
  std::vector<int64_t> counts((size_t)b->nClouds);
  std::vector<int64_t> hoff((size_t)b->nClouds + 1);
  cudaError_t e = cudaMemcpy(hoff.data(), b->dOff, hoff.size() * sizeof(int64_t), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_error(e, "batch offsets");
  for (int c = 0; c < b->nClouds; ++c) {
    const int64_t pts = hoff[(size_t)c + 1] - hoff[(size_t)c];
    if (queryCounts[c] < 0) return set_error(kErrArgument, "negative query count");
    // nabo/nabo.cpp:105-115, self match forbidden: k <= points - 1
    if (k[c] < 1 || k[c] > pts - 1)
      return set_error(kErrArgument, "Requesting more points (" + std::to_string(k[c]) +
                                         ") than available in cloud minus 1 (" + std::to_string(pts - 1) +
                                         ") (as self match is forbidden)");
    if (k[c] > 1024)
      return set_error(kErrUnsupported, "k larger than 1024 is not supported by the CUDA search types");
    ks[(size_t)c] = k[c];
    kMax = std::max(kMax, k[c]);
    qoff[(size_t)c + 1] = qoff[(size_t)c] + queryCounts[c];
    ooff[(size_t)c + 1] = ooff[(size_t)c] + queryCounts[c] * k[c];
  }
  nq = qoff.back();
  outTotal = ooff.back();
  if (nq > (int64_t)1 << 30) return set_error(kErrUnsupported, "a batch searches at most 2^30 queries");
  drop_graph(b);
  free_query_plan(b);
  b->nq = nq;
  b->kMax = kMax;
  b->outTotal = outTotal;
  e = cudaMalloc((void**)&b->dQOff, qoff.size() * sizeof(int64_t));
  if (e == cudaSuccess) e = cudaMalloc((void**)&b->dOutOff, ooff.size() * sizeof(int64_t));
  if (e == cudaSuccess) e = cudaMalloc((void**)&b->dK, ks.size() * sizeof(int32_t));
  if (e == cudaSuccess) e = cudaMalloc((void**)&b->order, (size_t)std::max<int64_t>(nq, 1) * sizeof(int32_t));
  if (e == cudaSuccess) e = cudaMalloc((void**)&b->cell, (size_t)std::max<int64_t>(nq, 1) * sizeof(uint32_t));
  if (e == cudaSuccess) e = cudaMalloc((void**)&b->rank, (size_t)std::max<int64_t>(nq, 1) * sizeof(uint32_t));
  if (e == cudaSuccess) e = cudaMalloc((void**)&b->hist, (size_t)2 * b->nTotal * sizeof(uint32_t));
  if (e == cudaSuccess) {
    // the deep search's stacks: room for one stack as tall as the largest
    // cloud (a tree's height is below its point count), 16 MiB at least so
    // that several queries search at once, 256 MiB at most
    b->slabBytes = std::min<int64_t>(int64_t(256) << 20, std::max<int64_t>(int64_t(16) << 20,
                                                                           (b->nMax + 2) * stack_level_bytes(b)));
    e = cudaMalloc(&b->slab, (size_t)b->slabBytes);
  }
  if (e == cudaSuccess) e = cudaMemcpy(b->dQOff, qoff.data(), qoff.size() * sizeof(int64_t), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(b->dOutOff, ooff.data(), ooff.size() * sizeof(int64_t), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(b->dK, ks.data(), ks.size() * sizeof(int32_t), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    free_query_plan(b);
    return cuda_error(e, "batch query plan");
  }
  e = make_class_plan(b, ks, qoff);
  if (e == cudaSuccess && b->plan.groups > 1 && !b->evFork) {
    // made once per batch, kept until it is destroyed
    for (int i = 0; i < 2 && e == cudaSuccess; ++i) {
      e = cudaStreamCreateWithFlags(&b->aux[i], cudaStreamNonBlocking);
      if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->evJoin[i], cudaEventDisableTiming);
    }
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->evFork, cudaEventDisableTiming);
  }
  if (e != cudaSuccess) {
    free_query_plan(b);
    return cuda_error(e, "batch query groups");
  }
  b->hQOff = std::move(qoff);
  b->hOutOff = std::move(ooff);
  return kOk;
}

int nabo_cuda_batch_build_device(nabo_cuda_batch* b, const void* clouds, void* stream) {
  if (!b || !clouds) return set_error(kErrArgument, "NULL argument");
  Guard g(b->device);
  return build(b, clouds, static_cast<cudaStream_t>(stream));
}

int nabo_cuda_batch_knn_device(nabo_cuda_batch* b, const void* queries, double epsilon, unsigned optionFlags,
                               double maxRadius, int32_t* indices, void* dists2, void* stream) {
  if (!b) return set_error(kErrArgument, "NULL batch");
  if (!b->dQOff) return set_error(kErrArgument, "call nabo_cuda_batch_set_queries first");
  if (optionFlags & NABO_ALLOW_SELF_MATCH)
    return set_error(kErrUnsupported, "batched searches forbid self matches (the plan checks k <= points - 1)");
  if (optionFlags > 3) return set_error(kErrArgument, "OR-ed value of option flags is larger than maximal valid value (3)");
  if (b->nq == 0) return kOk;
  if (!queries || !indices || !dists2) return set_error(kErrArgument, "NULL query or result buffer");
  Guard g(b->device);
  return search(b, queries, epsilon, optionFlags, maxRadius, indices, dists2, static_cast<cudaStream_t>(stream));
}


int nabo_cuda_batch_knn_radii_device(nabo_cuda_batch* b, const void* queries, const void* maxRadii, double epsilon,
                                     unsigned optionFlags, double maxRadius, int32_t* indices, void* dists2,
                                     int32_t* fallbacks, void* stream) {
  if (!b) return set_error(kErrArgument, "NULL batch");
  if (!b->dQOff) return set_error(kErrArgument, "call nabo_cuda_batch_set_queries first");
  if (optionFlags & NABO_ALLOW_SELF_MATCH)
    return set_error(kErrUnsupported, "batched searches forbid self matches (the plan checks k <= points - 1)");
  if (optionFlags > 3) return set_error(kErrArgument, "OR-ed value of option flags is larger than maximal valid value (3)");
  if (b->nq == 0) return kOk;
  if (!queries || !maxRadii || !indices || !dists2) return set_error(kErrArgument, "NULL query, radii or result buffer");
  Guard g(b->device);
  return search(b, queries, epsilon, optionFlags, maxRadius, indices, dists2, static_cast<cudaStream_t>(stream),
                maxRadii, fallbacks);
}

int nabo_cuda_batch_run(nabo_cuda_batch* b, const void* clouds, const void* queries, double epsilon,
                        unsigned optionFlags, double maxRadius, int32_t* indices, void* dists2, void* stream) {
  if (!b || !clouds) return set_error(kErrArgument, "NULL argument");
  if (!b->dQOff) return set_error(kErrArgument, "call nabo_cuda_batch_set_queries first");
  if (optionFlags & NABO_ALLOW_SELF_MATCH)
    return set_error(kErrUnsupported, "batched searches forbid self matches (the plan checks k <= points - 1)");
  if (b->nq > 0 && (!queries || !indices || !dists2)) return set_error(kErrArgument, "NULL query or result buffer");
  Guard g(b->device);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const bool same = b->exec && b->gClouds == clouds && b->gQuery == queries && b->gIdx == indices &&
                    b->gD2 == dists2 && b->gEps == epsilon && b->gFlags == optionFlags && b->gRadius == maxRadius;
  if (!same) {
    if (b->exec) cudaGraphExecDestroy(b->exec);
    b->exec = nullptr;
    cudaStream_t cap;
    cudaError_t e = cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking);
    if (e != cudaSuccess) return cuda_error(e, "capture stream");
    set_capture_allocations(true);
    e = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal);
    int rc = e == cudaSuccess ? kOk : cuda_error(e, "cudaStreamBeginCapture");
    if (rc == kOk) rc = build(b, clouds, cap);
    if (rc == kOk && b->nq > 0) rc = search(b, queries, epsilon, optionFlags, maxRadius, indices, dists2, cap);
    cudaGraph_t graph = nullptr;
    e = cudaStreamEndCapture(cap, &graph);
    set_capture_allocations(false);
    if (rc == kOk && e != cudaSuccess) rc = cuda_error(e, "cudaStreamEndCapture");
    if (rc == kOk) {
      e = cudaGraphInstantiate(&b->exec, graph, 0);
      if (e != cudaSuccess) rc = cuda_error(e, "cudaGraphInstantiate");
    }
    if (graph) cudaGraphDestroy(graph);
    cudaStreamDestroy(cap);
    if (rc != kOk) {
      b->exec = nullptr;
      return rc;
    }
    b->gClouds = clouds;
    b->gQuery = queries;
    b->gIdx = indices;
    b->gD2 = dists2;
    b->gEps = epsilon;
    b->gFlags = optionFlags;
    b->gRadius = maxRadius;
  }
  const cudaError_t e = cudaGraphLaunch(b->exec, st);
  if (e != cudaSuccess) return cuda_error(e, "cudaGraphLaunch");
  return kOk;
}

int nabo_cuda_batch_run_host(nabo_cuda_batch* b, const void* clouds, const void* queries, double epsilon,
                             unsigned optionFlags, double maxRadius, int32_t* indices, void* dists2) {
  if (!b || !clouds) return set_error(kErrArgument, "NULL argument");
  if (!b->dQOff) return set_error(kErrArgument, "call nabo_cuda_batch_set_queries first");
  if (optionFlags & NABO_ALLOW_SELF_MATCH)
    return set_error(kErrUnsupported, "batched searches forbid self matches (the plan checks k <= points - 1)");
  if (optionFlags > 3) return set_error(kErrArgument, "OR-ed value of option flags is larger than maximal valid value (3)");
  if (b->nq > 0 && (!queries || !indices || !dists2)) return set_error(kErrArgument, "NULL query or result buffer");
  Guard g(b->device);
  int rc = host_buffers(b);
  if (rc != kOk) return rc;
  const size_t es = elem_bytes(b);
  const size_t cBytes = (size_t)b->nTotal * b->dim * es, qBytes = (size_t)b->nq * b->dim * es;
  const size_t oEntries = (size_t)b->outTotal;
  cudaStream_t st = b->hostStream;
  cudaError_t e;
  if (pinned_range(clouds, cBytes) && pinned_range(queries, qBytes) && pinned_range(indices, oEntries * 4) &&
      pinned_range(dists2, oEntries * es)) {
    const bool same = b->hostExec && b->hClouds == clouds && b->hQuery == queries && b->hIdx == indices &&
                      b->hD2 == dists2 && b->hEps == epsilon && b->hFlags == optionFlags && b->hRadius == maxRadius;
    if (!same) {
      if (b->hostExec) cudaGraphExecDestroy(b->hostExec);
      b->hostExec = nullptr;
      rc = capture_host(b, clouds, queries, epsilon, optionFlags, maxRadius, indices, dists2);
      if (rc != kOk) return rc;
      b->hClouds = clouds;
      b->hQuery = queries;
      b->hIdx = indices;
      b->hD2 = dists2;
      b->hEps = epsilon;
      b->hFlags = optionFlags;
      b->hRadius = maxRadius;
    }
    e = cudaGraphLaunch(b->hostExec, st);
    if (e != cudaSuccess) return cuda_error(e, "cudaGraphLaunch");
  } else {
    // pageable buffers: plain copies around the device run
    e = cudaMemcpyAsync(b->devClouds, clouds, cBytes, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess && qBytes) e = cudaMemcpyAsync(b->devQueries, queries, qBytes, cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return cuda_error(e, "batch upload");
    rc = nabo_cuda_batch_run(b, b->devClouds, b->devQueries, epsilon, optionFlags, maxRadius, b->devIdx, b->devD2, st);
    if (rc != kOk) return rc;
    if (oEntries) {
      e = cudaMemcpyAsync(indices, b->devIdx, oEntries * 4, cudaMemcpyDeviceToHost, st);
      if (e == cudaSuccess) e = cudaMemcpyAsync(dists2, b->devD2, oEntries * es, cudaMemcpyDeviceToHost, st);
      if (e != cudaSuccess) return cuda_error(e, "batch download");
    }
  }
  e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return cuda_error(e, "batch host run");
  return kOk;
}

int nabo_cuda_batch_status(nabo_cuda_batch* b, int64_t info[8]) {
  if (!b || !info) return set_error(kErrArgument, "NULL argument");
  Guard g(b->device);
  int hs[8];
  int64_t total = 0;
  cudaError_t e = cudaDeviceSynchronize();
  if (e == cudaSuccess) e = cudaMemcpy(hs, b->status, sizeof(hs), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess)
    e = cudaMemcpy(&total, b->nodeOffset + b->nClouds, sizeof(int64_t), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_error(e, "batch status");
  // a tree taller than the search kernels' stacks (256) is searched with
  // stacks in global memory (bit 4); bit 8: one such stack did not fit
  info[0] = (hs[0] ? 1 : 0) | (hs[1] ? 2 : 0) | (hs[2] > 256 ? 4 : 0) | (hs[4] ? 8 : 0);
  info[1] = total;
  info[2] = hs[2];
  info[3] = hs[3];
  info[4] = b->outTotal;
  info[5] = b->nq;
  info[6] = b->nTotal;
  info[7] = b->nClouds;
  return kOk;
}

int nabo_cuda_batch_export_tree(nabo_cuda_batch* b, int cloud, int64_t* nodeCount, int32_t* cutDim, void* cutVal,
                                uint32_t* right, uint32_t* bucketStart, uint32_t* bucketSize, int32_t* buckets) {
  if (!b || cloud < 0 || cloud >= b->nClouds || !nodeCount) return set_error(kErrArgument, "bad argument");
  Guard g(b->device);
  int64_t noff[2], poff[2];
  cudaError_t e = cudaDeviceSynchronize();
  if (e == cudaSuccess) e = cudaMemcpy(noff, b->nodeOffset + cloud, sizeof(noff), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(poff, b->dOff + cloud, sizeof(poff), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_error(e, "batch export");
  const int64_t cnt = noff[1] - noff[0];
  if (!cutDim) {
    *nodeCount = cnt;
    return kOk;
  }
  if (*nodeCount < cnt) return set_error(kErrArgument, "arrays too small");
  *nodeCount = cnt;
  const bool f32 = b->dtype == NABO_CUDA_FLOAT32;
  const size_t nodeBytes = f32 ? 8 : 16;
  std::vector<unsigned char> nodes((size_t)cnt * nodeBytes);
  e = cudaMemcpy(nodes.data(), static_cast<unsigned char*>(b->nodes) + noff[0] * nodeBytes, nodes.size(),
                 cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_error(e, "batch export nodes");
  for (int64_t i = 0; i < cnt; ++i) {
    const unsigned char* p = nodes.data() + i * nodeBytes;
    uint32_t meta, start;
    std::memcpy(&meta, p, 4);
    std::memcpy(&start, p + 4, 4);
    const bool leaf = node_is_leaf(meta);
    cutDim[i] = leaf ? -1 : (int32_t)node_dim(meta);
    if (right) right[i] = leaf ? 0u : node_payload(meta) - (uint32_t)noff[0];
    if (bucketStart) bucketStart[i] = leaf ? start - (uint32_t)poff[0] : 0u;
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
    const size_t recBytes = ((size_t)b->dpad * es + 4 + 15) / 16 * 16;
    const int64_t n = poff[1] - poff[0];
    std::vector<unsigned char> recs((size_t)n * recBytes);
    e = cudaMemcpy(recs.data(), static_cast<unsigned char*>(b->recs) + poff[0] * recBytes, recs.size(),
                   cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_error(e, "batch export buckets");
    for (int64_t i = 0; i < n; ++i) std::memcpy(buckets + i, recs.data() + i * recBytes + b->dpad * es, 4);
  }
  return kOk;
}

}  // extern "C"
