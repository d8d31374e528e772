// noalloc.cu -- kNN search that allocates no device memory.
//
// The regular device search (nabo_cuda_knn_device) orders its queries with
// scratch taken from a memory pool. This entry point is for callers that
// must not reach the CUDA allocator once running -- a real-time robot
// perception loop that fixed its GPU memory at start-up, or an application
// whose device memory is owned by its own arena: the same search, with the
// query-ordering scratch in one fixed array that lives in this file.
//
// The array holds, for up to kMaxQueries queries, the query order, each
// query's cell and its rank inside the cell, plus a kBins-entry cell
// histogram. Queries are grouped by a Morton (Z-order) cell of the cloud's
// bounding box, counted, scanned and placed, then the kd-tree search kernel
// runs with that order. Queries are ordered under the same rule as the
// regular search (the object's queryOrdering parameter, and enough work for
// the order to pay). A kd-tree taller than the search kernels' stacks (256
// levels) is searched unordered with its traversal stacks in the array
// instead. Every call on a device reuses the array: the histogram is
// cleared at the start of each call, and calls that overlap on the GPU race.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <mutex>
#include <string>

#include "internal.cuh"
#include "nabo_gb300.h"

namespace nabo_gb300 {
namespace {

constexpr int64_t kMaxQueries = NABO_CUDA_NOALLOC_MAX_QUERIES;
constexpr int kBinsLog2 = 16;
constexpr int kBins = 1 << kBinsLog2;
constexpr size_t kScratchBytes = (size_t)kMaxQueries * 3 * sizeof(uint32_t) + (size_t)kBins * sizeof(uint32_t);
static_assert(kScratchBytes == NABO_CUDA_NOALLOC_SCRATCH_BYTES, "scratch size must match the header");

// The scratch itself. In host code this name is only a stand-in for the
// symbol; the device address comes from cudaGetSymbolAddress below.
static __device__ __align__(256) unsigned char g_noallocScratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_addrMutex;
unsigned char* g_addr[kMaxDevices] = {};

// Device address of the scratch on the current device. It is looked up on
// every call made outside a stream capture, so that it follows the module
// if the device's context is torn down and made again (cudaDeviceReset);
// a call made while `stream` is capturing uses the address of the last call
// outside capture, because the lookup may load the module. So the first
// call on a device comes before any capture, and after a cudaDeviceReset
// one call outside capture comes before capturing again.
int scratch_address(int device, cudaStream_t stream, unsigned char** out) {
  if (device < 0 || device >= kMaxDevices) return set_error(kErrUnsupported, "device ordinal out of range");
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  cudaError_t e = cudaStreamIsCapturing(stream, &cs);
  if (e != cudaSuccess) return cuda_error(e, "cudaStreamIsCapturing");
  std::lock_guard<std::mutex> lock(g_addrMutex);
  if (cs == cudaStreamCaptureStatusNone) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noallocScratch);
    if (e != cudaSuccess) return cuda_error(e, "cudaGetSymbolAddress(no-alloc scratch)");
    g_addr[device] = static_cast<unsigned char*>(p);
  } else if (!g_addr[device]) {
    return set_error(kErrArgument, "nabo_cuda_knn_device_noalloc: the first call on a device must come before "
                                   "any stream capture");
  }
  *out = g_addr[device];
  return kOk;
}

struct Layout {
  int32_t* order;
  uint32_t* cell;
  uint32_t* rank;
  uint32_t* hist;
};

Layout layout(unsigned char* base) {
  Layout l;
  l.order = reinterpret_cast<int32_t*>(base);
  l.cell = reinterpret_cast<uint32_t*>(base + (size_t)kMaxQueries * 4);
  l.rank = reinterpret_cast<uint32_t*>(base + (size_t)kMaxQueries * 8);
  l.hist = reinterpret_cast<uint32_t*>(base + (size_t)kMaxQueries * 12);
  return l;
}

// Levels the search kernels' own stacks hold (taller trees search with
// their stacks in the array).
constexpr int kSearchStackLevels = 256;

constexpr int kCellDims = 10;
struct CellGrid {
  float lo[kCellDims];
  float scale[kCellDims];
  int dims;
  int bits;
  int shift;
};

__global__ void k_na_clear(uint32_t* hist) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < kBins; i += gridDim.x * blockDim.x) hist[i] = 0u;
}

template <typename T>
__global__ void k_na_cells(const T* __restrict__ q, int64_t nq, int64_t qStride, CellGrid g, uint32_t* cell,
                           uint32_t* rank, uint32_t* hist) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= nq) return;
  const float maxc = (float)((1u << g.bits) - 1u);
  uint32_t c[kCellDims];
#pragma unroll
  for (int d = 0; d < kCellDims; ++d) {
    c[d] = 0u;
    if (d < g.dims) {
      const float v = fminf(fmaxf(((float)q[i * qStride + d] - g.lo[d]) * g.scale[d], 0.0f), maxc);
      c[d] = (uint32_t)v;
    }
  }
  uint32_t key = 0;
  for (int b = g.bits - 1; b >= 0; --b)
    for (int d = 0; d < g.dims; ++d) key = (key << 1) | ((c[d] >> b) & 1u);
  const uint32_t cl = key >> g.shift;  // < kBins
  cell[i] = cl;
  rank[i] = atomicAdd(hist + cl, 1u);
}

// Exclusive scan of the kBins histogram by one block of 1024 threads.
__global__ void __launch_bounds__(1024) k_na_scan(uint32_t* hist) {
  __shared__ uint32_t warpSums[32];
  __shared__ uint32_t carry;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (threadIdx.x == 0) carry = 0u;
  __syncthreads();
  for (int base = 0; base < kBins; base += 1024) {
    const uint32_t v = hist[base + threadIdx.x];
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) warpSums[warp] = x;
    __syncthreads();
    if (warp == 0) {
      uint32_t w = warpSums[lane];
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
        if (lane >= o) w += y;
      }
      warpSums[lane] = w;
    }
    __syncthreads();
    const uint32_t prefix = carry + (warp > 0 ? warpSums[warp - 1] : 0u) + x - v;
    hist[base + threadIdx.x] = prefix;
    __syncthreads();
    if (threadIdx.x == 0) carry += warpSums[31];
    __syncthreads();
  }
}

__global__ void k_na_place(const uint32_t* __restrict__ cell, const uint32_t* __restrict__ rank,
                           const uint32_t* __restrict__ start, int64_t nq, int32_t* order) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= nq) return;
  order[start[cell[i]] + rank[i]] = (int32_t)i;
}

CellGrid make_grid(const DeviceCloud& c) {
  CellGrid g;
  g.dims = std::min(c.dim, kCellDims);
  g.bits = std::max(1, kBinsLog2 / g.dims);
  g.shift = std::max(0, g.bits * g.dims - kBinsLog2);
  for (int d = 0; d < kCellDims; ++d) {
    g.lo[d] = 0.0f;
    g.scale[d] = 0.0f;
    if (d < g.dims) {
      const double ext = c.hi[d] - c.lo[d];
      g.lo[d] = (float)c.lo[d];
      g.scale[d] = (ext > 0.0 && std::isfinite(ext)) ? (float)(((1u << g.bits) - 1u) / ext) : 0.0f;
    }
  }
  return g;
}

template <typename T>
int order_in_scratch(const DeviceCloud& c, const T* q, int64_t nq, int64_t qStride, const Layout& l,
                     cudaStream_t st) {
  k_na_clear<<<kBins / 1024, 1024, 0, st>>>(l.hist);
  k_na_cells<T><<<ceil_div(nq, 256), 256, 0, st>>>(q, nq, qStride, make_grid(c), l.cell, l.rank, l.hist);
  k_na_scan<<<1, 1024, 0, st>>>(l.hist);
  k_na_place<<<ceil_div(nq, 256), 256, 0, st>>>(l.cell, l.rank, l.hist, nq, l.order);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_error(e, "no-alloc query ordering");
  return kOk;
}

template <typename T, int D>
int search_noalloc(const DeviceCloud& c, const KnnArgs& a, const Layout* l, cudaStream_t st) {
  const int32_t* order = nullptr;
  if (l) {
    const int rc = order_in_scratch<T>(c, static_cast<const T*>(a.query), a.nq, a.qStride, *l, st);
    if (rc != kOk) return rc;
    order = l->order;
  }
  // a.stackSlab (set for tall trees) keeps this from allocating stacks
  return knn_kdtree_given_order<T, D>(c, a, order, st);
}

int dispatch(const DeviceCloud& c, const KnnArgs& a, const Layout* l, cudaStream_t st) {
#define NABO_NA_CASE(TT, DD) \
  if (c.dpad == DD) return search_noalloc<TT, DD>(c, a, l, st);
  if (c.dtype == NABO_CUDA_FLOAT32) {
    NABO_NA_CASE(float, 2)
    NABO_NA_CASE(float, 3)
    NABO_NA_CASE(float, 4)
    NABO_NA_CASE(float, 8)
    NABO_NA_CASE(float, 16)
  } else {
    NABO_NA_CASE(double, 2)
    NABO_NA_CASE(double, 3)
    NABO_NA_CASE(double, 4)
    NABO_NA_CASE(double, 8)
    NABO_NA_CASE(double, 16)
  }
#undef NABO_NA_CASE
  return set_error(kErrInternal, "bad dispatch");
}

}  // namespace
}  // namespace nabo_gb300

using namespace nabo_gb300;

extern "C" int nabo_cuda_knn_device_noalloc(const nabo_cuda_search* s, const void* query, int qRows, int64_t nq,
                                            int64_t qStride, int k, double epsilon, unsigned optionFlags,
                                            double maxRadius, const void* maxRadii, int32_t* indices, void* dists2,
                                            uint64_t* touched, void* stream) {
  if (!s) return set_error(kErrArgument, "search object is NULL");
  int rc = handle_check_knn(s, qRows, nq, qStride, k, optionFlags, maxRadii);
  if (rc != kOk) return rc;
  if (nq > kMaxQueries)
    return set_error(kErrArgument, "nabo_cuda_knn_device_noalloc: " + std::to_string(nq) +
                                       " queries exceed its fixed scratch (at most " +
                                       std::to_string(kMaxQueries) + " per call); split the batch");
  if (nq == 0) return kOk;
  if (!query || !indices || !dists2) return set_error(kErrArgument, "NULL query or result buffer");
  const HandleView h = handle_view(s);
  int prev = -1;
  cudaError_t e = cudaGetDevice(&prev);
  if (e != cudaSuccess) return cuda_error(e, "cudaGetDevice");
  if (prev != h.device && (e = cudaSetDevice(h.device)) != cudaSuccess) return cuda_error(e, "cudaSetDevice");
  KnnArgs a;
  a.query = query;
  a.nq = nq;
  a.qStride = qStride;
  a.k = k;
  a.eps = epsilon;
  a.optionFlags = optionFlags;
  a.maxRadius = maxRadius;
  a.maxRadii = maxRadii;
  a.indices = indices;
  a.dists2 = dists2;
  a.traversal = h.traversal;
  a.evStart = h.evStart;
  a.evStop = h.evStop;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (h.searchType == NABO_SEARCH_KDTREE_CUDA) {
    a.touchStats = (h.creationFlags & NABO_TOUCH_STATISTICS) != 0;
    a.touched = reinterpret_cast<unsigned long long*>(touched);
    unsigned char* base = nullptr;
    rc = scratch_address(h.device, st, &base);
    if (rc == kOk) {
      const Layout l = layout(base);
      const bool tall = h.cloud->height > kSearchStackLevels;
      if (tall) {  // the whole array holds the traversal stacks; no ordering
        a.stackSlab = base;
        a.stackSlabBytes = kScratchBytes;
      }
      const bool ordered = !tall && h.sortQueries && worth_sorting(nq, k, h.cloud->dim);
      rc = dispatch(*h.cloud, a, ordered ? &l : nullptr, st);
    }
  } else {
    rc = set_error(kErrArgument, "nabo_cuda_knn_device_noalloc serves kd-tree objects; "
                                 "the brute-force search already allocates nothing (use nabo_cuda_knn_device)");
  }
  if (prev >= 0 && prev != h.device) cudaSetDevice(prev);
  return rc;
}
