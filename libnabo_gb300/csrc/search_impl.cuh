// search_impl.cuh -- host-side dispatch of the kNN kernels for one (T, D).
// Included by one translation unit per (T, D) so they compile in parallel.
#pragma once

#include "internal.cuh"
#include "search.cuh"
#include "search_wide.cuh"

#include <algorithm>
#include <cstring>
#include <string>

namespace nabo_gb300 {

// Traversal stack depths compiled; the tree's height selects one.
constexpr int kStackSmall = 64;
constexpr int kStackLarge = 256;

// k above kMaxK: a group of lanes per query holding K slots (K compiled
// below): 8 lanes for K = 64 and 128 (four queries share a warp's traversal
// instructions), a whole warp beyond. Measured on lidar scans (kernel ms):
// K = 64 9.50 by warps, 6.05 by 8 lanes; K = 128 15.5 by 16 lanes, 14.9 by
// 8; K = 256 43.7 by warps, 44.6 by 16 lanes, 52.3 by 8; K = 512 165 by
// warps, 200 by 16 lanes.
#define NABO_WIDE_LIST(X) X(64) X(128) X(256) X(512) X(1024)
constexpr int kMaxWideK = 1024;
constexpr int kWideThreads = 128;  // threads per block of the kd-tree kernel
constexpr int kWideBfWarps = 8;    // queries per block of the brute force

template <int KK>
struct WideShape {
  static constexpr int G = KK <= 128 ? 8 : 32;
  static constexpr int M = KK / G;
};

inline int wide_k(int k) {
#define NABO_ROUND(KK) \
  if (k <= KK) return KK;
  NABO_WIDE_LIST(NABO_ROUND)
#undef NABO_ROUND
  return -1;
}

inline int k_unsupported() {
  return set_error(kErrUnsupported, "k larger than 1024 is not supported by the CUDA search types");
}

// Shared memory the wide kernel's stacks may take per block; trees too tall
// for one warp's stacks there search with the stacks in global memory.
constexpr size_t kWideSmemMax = 160 * 1024;
// Internal: the search needs its stacks in global memory.
constexpr int kNeedsSlab = -100;

template <typename T, int D, int M, int G>
int launch_wide_kdtree_as(const KnnLaunch& L, int height, cudaStream_t stream) {
  const int cap = height + 1;
  // the groups' stacks in shared memory: smaller blocks for tall trees of
  // long records
  int threads = kWideThreads;
  while (threads > 32 && wide_stack_bytes<T, D>(threads / G, cap) > kWideSmemMax) threads /= 2;
  const size_t smem = wide_stack_bytes<T, D>(threads / G, cap);
  if (smem > kWideSmemMax) return kNeedsSlab;
  cudaError_t e = cudaSuccess;
  if (smem > 48 * 1024)
    e = cudaFuncSetAttribute(k_knn_kdtree_wide<T, D, M, G>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem);
  if (e != cudaSuccess) return cuda_error(e, "wide kd-tree search shared memory");
  const int grid = ceil_div(L.nq, threads / G);
  k_knn_kdtree_wide<T, D, M, G><<<grid, threads, smem, stream>>>(L, cap);
  return kOk;
}

// Launches the group-per-query kd-tree search for L.k (or the batch's
// largest k) above kMaxK; `height` bounds the traversal stack. Returns
// kNeedsSlab when one warp's stacks do not fit in shared memory.
template <typename T, int D>
int launch_wide_kdtree(const KnnLaunch& L, int kMax, int height, cudaStream_t stream) {
  switch (wide_k(kMax)) {
#define NABO_WIDE(KK) \
  case KK:            \
    return launch_wide_kdtree_as<T, D, WideShape<KK>::M, WideShape<KK>::G>(L, height, stream);
    NABO_WIDE_LIST(NABO_WIDE)
#undef NABO_WIDE
  }
  return k_unsupported();
}

// Bytes of global memory one query's stack takes in a deep search (trees
// taller than the compiled stacks): `kMax` above kMaxK searches by groups.
template <typename T, int D>
int64_t deep_unit_bytes(int kMax, int height) {
  const int cap = height + 1;
  return kMax > kMaxK ? wide_group_slab_bytes<T, D>(cap) : (int64_t)deep_stack_bytes<T, D>(cap);
}

// Launches the deep search over L (L.slab, L.slabBytes and the cap or the
// device height set by the caller) with room for `units` concurrent
// queries.
template <typename T, int D>
int launch_deep(const KnnLaunch& L, int kMax, int64_t units, cudaStream_t stream) {
  if (units < 1) units = 1;
  if (kMax <= kMaxK) {
    const int grid = ceil_div(units, 128);
    switch (round_k(kMax)) {
#define NABO_DEEP(KK)                                 \
  case KK:                                            \
    launch_kdtree_deep<T, D, KK>(grid, stream, L);    \
    return kOk;
      NABO_K_LIST(NABO_DEEP)
#undef NABO_DEEP
    }
    return k_unsupported();
  }
  switch (wide_k(kMax)) {
#define NABO_WIDE(KK)                                                                                     \
  case KK: {                                                                                              \
    constexpr int G = WideShape<KK>::G;                                                                   \
    k_knn_kdtree_wide_deep<T, D, WideShape<KK>::M, G><<<ceil_div(units * G, 128), 128, 0, stream>>>(L);   \
    return kOk;                                                                                           \
  }
    NABO_WIDE_LIST(NABO_WIDE)
#undef NABO_WIDE
  }
  return k_unsupported();
}

template <typename T, int D>
int launch_wide_bruteforce(const KnnLaunch& L, cudaStream_t stream) {
  const int grid = ceil_div(L.nq, kWideBfWarps);
  switch (wide_k(L.k)) {
#define NABO_WIDE(KK)                                                                    \
  case KK:                                                                               \
    k_knn_bruteforce_wide<T, D, KK / 32><<<grid, 32 * kWideBfWarps, 0, stream>>>(L);     \
    return kOk;
    NABO_WIDE_LIST(NABO_WIDE)
#undef NABO_WIDE
  }
  return k_unsupported();
}

template <typename T, int D>
KnnLaunch make_launch(const DeviceCloud& c, const KnnArgs& a, const int32_t* order) {
  KnnLaunch L{};  // every field not set below is zero / null
  L.nodes = c.nodes;
  L.recs = c.recs;
  L.query = a.query;
  L.nq = a.nq;
  L.qStride = a.qStride;
  L.dim = c.dim;
  L.order = order;
  L.k = a.k;
  const T eps = (T)a.eps;
  const T one = T(1);
  const T e1 = one + eps;
  L.maxError2 = (double)(T)(e1 * e1);
  const T r = (T)a.maxRadius;
  L.maxRadius2 = (double)(T)(r * r);
  L.maxRadii = a.maxRadii;
  L.outIdx = a.indices;
  L.outD2 = a.dists2;
  L.touched = a.touched;
  L.found = a.found;
  L.n = c.n;
  L.allowSelf = (a.optionFlags & 1u) ? 1 : 0;
  L.stats = (a.touchStats && a.touched) ? 1 : 0;
  L.nqDevice = a.nqDevice;
  L.fallbackRadius = a.maxRadii ? a.fallbackRadius : -1.0;
  L.fallbacks = a.fallbacks;
  L.recs32 = c.recs32;
  L.coordMax = c.coordMax;
  L.bQueryOffset = nullptr;
  L.bNodeOffset = nullptr;
  L.bK = nullptr;
  L.bOutOffset = nullptr;
  L.bClouds = 0;
  L.slab = nullptr;
  L.slabBytes = 0;
  L.stackCap = 0;
  L.stackHeightDev = nullptr;
  L.tallGate = nullptr;
  L.tallGateLimit = 0;
  L.deepFail = nullptr;
  return L;
}

// The kd-tree search kernel(s) for one query order: one thread per query
// for k <= kMaxK (stack in local memory, 64 or 256 entries by the tree's
// height), a lane group per query above (stacks in shared memory), or, for
// trees too tall for those stacks, the deep kernels with the stacks in
// global memory: a.stackSlab when the caller gives one (a.stackSlabBytes),
// else scratch from the pool (at most kDeepSlabMax bytes; fewer queries then
// search at once).
constexpr int64_t kDeepSlabMax = int64_t(256) << 20;

template <typename T, int D>
int launch_search(const DeviceCloud& c, const KnnArgs& a, const int32_t* order, cudaStream_t stream) {
  const int K = round_k(a.k);
  if (K < 0 && a.k > kMaxWideK) return k_unsupported();
  KnnLaunch L = make_launch<T, D>(c, a, order);
  const int grid = ceil_div(a.nq, 128);
  const bool small = c.height <= kStackSmall;
  // Default: the reference visit order (it is also the faster one on the
  // measured workloads); the warp packet is opt-in for exact searches with
  // k <= kMaxK.
  const bool packet = a.traversal == 2 && K > 0;
  if (packet && (a.eps != 0.0 || L.stats))
    return set_error(kErrArgument, "the warp-packet traversal serves exact searches without TOUCH_STATISTICS only");
  if (packet && c.height > kStackLarge)
    return set_error(kErrUnsupported, "the warp-packet traversal serves kd-trees of at most 256 levels");
  if (a.evStart) cudaEventRecord(a.evStart, stream);
  int rc = kOk;
  bool deep = K > 0 && !packet && c.height > kStackLarge;
  if (K < 0) {
    rc = launch_wide_kdtree<T, D>(L, a.k, c.height, stream);
    if (rc == kNeedsSlab) {
      deep = true;
      rc = kOk;
    }
  } else if (!deep) {
#define NABO_LAUNCH(KK)                                                            \
  case KK:                                                                         \
    if (packet) {                                                                  \
      if (small)                                                                   \
        k_knn_kdtree_packet<T, D, KK, kStackSmall><<<grid, 128, 0, stream>>>(L);   \
      else                                                                         \
        k_knn_kdtree_packet<T, D, KK, kStackLarge><<<grid, 128, 0, stream>>>(L);   \
    } else {                                                                       \
      if (small)                                                                   \
        launch_kdtree<T, D, KK, kStackSmall>(grid, 128, stream, L);                \
      else                                                                         \
        launch_kdtree<T, D, KK, kStackLarge>(grid, 128, stream, L);                \
    }                                                                              \
    break;
    switch (K) { NABO_K_LIST(NABO_LAUNCH) }
#undef NABO_LAUNCH
  }
  void* owned = nullptr;
  if (rc == kOk && deep) {
    const int64_t unit = deep_unit_bytes<T, D>(a.k, c.height);
    int64_t bytes = a.stackSlab ? (int64_t)a.stackSlabBytes : std::min<int64_t>(kDeepSlabMax, unit * a.nq);
    if (bytes < unit) bytes = a.stackSlab ? 0 : unit;
    if (bytes < unit) {
      rc = set_error(kErrUnsupported, "kd-tree of height " + std::to_string(c.height) +
                                          ": one query's traversal stack does not fit the given scratch");
    } else {
      L.slab = a.stackSlab;
      if (!L.slab) {
        const cudaError_t e = scratch_alloc(&owned, (size_t)bytes, stream);
        if (e != cudaSuccess) rc = cuda_error(e, "deep search stacks");
        L.slab = owned;
      }
      if (rc == kOk) {
        L.slabBytes = bytes;
        L.stackCap = c.height + 1;
        rc = launch_deep<T, D>(L, a.k, std::min<int64_t>(a.nq, bytes / unit), stream);
      }
    }
  }
  if (a.evStop) cudaEventRecord(a.evStop, stream);
  const cudaError_t e = cudaGetLastError();
  if (owned) scratch_free(owned, stream);
  if (rc != kOk) return rc;
  if (e != cudaSuccess) return cuda_error(e, "kd-tree search launch");
  return kOk;
}

template <typename T, int D>
int knn_kdtree(const DeviceCloud& c, const KnnArgs& a, cudaStream_t stream) {
  if (a.nq == 0) return kOk;
  if (round_k(a.k) < 0 && a.k > kMaxWideK) return k_unsupported();
  int32_t* order = nullptr;
  if (a.sortQueries && worth_sorting(a.nq, a.k, c.dim)) {
    NABO_CUDA_TRY(scratch_alloc((void**)&order, (size_t)a.nq * sizeof(int32_t), stream));
    const int rc = knn_leaf_order<T, D>(c, a.query, a.nq, a.qStride, order, stream);
    if (rc != kOk) {
      scratch_free(order, stream);
      return rc;
    }
  }
  const int rc = launch_search<T, D>(c, a, order, stream);
  if (order) scratch_free(order, stream);
  return rc;
}

// Brute force for k <= kMaxK. A search with too few queries to give every
// SM kBfBlocksPerSm blocks splits the points into row chunks (block rows),
// each writing its k best per query to scratch, merged by k_bf_merge.
// (At 4 blocks per SM, 100 k x 100 k ran 16 warps per SM at 74 % issue.
// Rows chosen from the kernel's real occupancy instead, to fill whole waves
// (4 rows there instead of 2), measured slower, 3.50 -> 3.74 ms at k = 5 and
// 4.79 -> 5.78 ms at k = 10: each row's top-k lists start empty, and more
// of the points then meet a loose threshold.)
constexpr int kBfBlocksPerSm = 8;
template <typename T, int D, int K, int QT = BfShape<T, K>::QT, int J = BfShape<T, K>::J>
int launch_bruteforce(const KnnLaunch& L, cudaStream_t stream) {
  constexpr int64_t kTile = (int64_t)((24 * 1024) / sizeof(Rec<T, D>));
  const int qBlocks = ceil_div(L.nq, 128 * QT);
  int dev = 0, sms = 148;
  if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int64_t tiles = std::max<int64_t>(1, (L.n + kTile - 1) / kTile);
  int64_t rows = std::min<int64_t>({(kBfBlocksPerSm * (int64_t)sms + qBlocks - 1) / qBlocks, tiles / 4, 64});
  if (rows <= 1) {
    k_knn_bruteforce<T, D, K, QT, J><<<qBlocks, 128, 0, stream>>>(L, L.n, 0);
    return kOk;
  }
  const int64_t chunk = (tiles + rows - 1) / rows * kTile;
  rows = (L.n + chunk - 1) / chunk;
  const int64_t stride = L.nq * (int64_t)L.k;
  int32_t* pIdx = nullptr;
  T* pD2 = nullptr;
  NABO_CUDA_TRY(scratch_alloc((void**)&pIdx, (size_t)(rows * stride) * sizeof(int32_t), stream));
  cudaError_t e = scratch_alloc((void**)&pD2, (size_t)(rows * stride) * sizeof(T), stream);
  if (e != cudaSuccess) {
    scratch_free(pIdx, stream);
    return cuda_error(e, "brute-force partial results");
  }
  KnnLaunch P = L;
  P.outIdx = pIdx;
  P.outD2 = pD2;
  P.found = nullptr;
  k_knn_bruteforce<T, D, K, QT, J><<<dim3(qBlocks, (unsigned)rows), 128, 0, stream>>>(P, chunk, stride);
  k_bf_merge<T, K><<<ceil_div(L.nq, 128), 128, 0, stream>>>(pIdx, pD2, (int)rows, stride, L.nq, L.k, L.outIdx,
                                                           static_cast<T*>(L.outD2), L.found);
  scratch_free(pIdx, stream);
  scratch_free(pD2, stream);
  return kOk;
}

template <typename T, int D>
int knn_bruteforce(const DeviceCloud& c, const KnnArgs& a, cudaStream_t stream) {
  if (a.nq == 0) return kOk;
  const int K = round_k(a.k);
  if (K < 0 && a.k > kMaxWideK) return k_unsupported();
  const KnnLaunch L = make_launch<T, D>(c, a, nullptr);
  if (a.evStart) cudaEventRecord(a.evStart, stream);
  int rc = kOk;
  if (K < 0) rc = launch_wide_bruteforce<T, D>(L, stream);
#define NABO_LAUNCH(KK)                                 \
  case KK:                                              \
    rc = launch_bruteforce<T, D, KK>(L, stream);        \
    break;
  if (K > 0) switch (K) { NABO_K_LIST(NABO_LAUNCH) }
#undef NABO_LAUNCH
  if (a.evStop) cudaEventRecord(a.evStop, stream);
  if (rc != kOk) return rc;
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_error(e, "k_knn_bruteforce launch");
  return kOk;
}

// kd-tree search with a query order computed by the caller (`order` may be
// null); launches the search kernel only. It allocates nothing, except the
// traversal stacks of a tree taller than the compiled stacks when the
// caller gives no a.stackSlab.
template <typename T, int D>
int knn_kdtree_given_order(const DeviceCloud& c, const KnnArgs& a, const int32_t* order, cudaStream_t stream) {
  if (a.nq == 0) return kOk;
  return launch_search<T, D>(c, a, order, stream);
}

// The query order the kd-tree search uses (written to `order`, nq entries,
// device): a stable sort by a 30-bit Morton code over the cloud's bounding
// box for up to 3 dimensions, by the leaf each query descends to for more
// (where a Morton code over all dimensions gets too coarse). On lidar scans
// the Morton order runs the search kernel 1.34x faster than the leaf
// order with unordered ties: most queries there fall into a few large
// empty-space leaves, inside which only the Morton code keeps neighbours
// together.
template <typename T, int D>
int knn_leaf_order(const DeviceCloud& c, const void* query, int64_t nq, int64_t qStride, int32_t* order,
                   cudaStream_t stream) {
  if (nq == 0) return kOk;
  if (c.dim <= 3) return order_queries<T>(static_cast<const T*>(query), nq, qStride, c.dim, c.lo, c.hi, order, stream);
  uint32_t* cell = nullptr;
  NABO_CUDA_TRY(scratch_alloc((void**)&cell, (size_t)nq * sizeof(uint32_t), stream));
  k_leaf_cells<T, D><<<ceil_div(nq, 256), 256, 0, stream>>>(static_cast<const Node<T>*>(c.nodes),
                                                            static_cast<const T*>(query), nq, qStride, c.dim, cell,
                                                            nullptr, nullptr);
  int bits = 1;
  while ((int64_t(1) << bits) < c.nodeCount && bits < 31) ++bits;
  const int rc = sort_order_u32(cell, nq, bits, order, stream);
  scratch_free(cell, stream);
  return rc;
}

// Chunk-major Morton order (first by chunk, then along the curve) for a
// search split into consecutive query chunks, one launch each; clouds of up
// to 3 dimensions. With copyOut the queries are copied there as they are
// read (see order_queries).
template <typename T, int D>
int knn_chunk_order(const DeviceCloud& c, const void* query, int64_t nq, int64_t qStride, const QueryChunks& chunks,
                    int32_t* order, cudaStream_t stream, void* copyOut) {
  if (c.dim > 3) return set_error(kErrUnsupported, "chunked query order: more than 3 dimensions");
  return order_queries<T>(static_cast<const T*>(query), nq, qStride, c.dim, c.lo, c.hi, order, stream, &chunks,
                          static_cast<T*>(copyOut));
}

// Batched search over a forest: leaf order of all queries (each in its
// cloud's tree), then the reference-order kernel over that order. `order`,
// `hist` (nodeCap entries), `cell` and `rank` (nq each) are caller scratch.
// The leaves are numbered cloud by cloud, so the order is too: positions
// [qOffset[c0], qOffset[c1]) hold exactly the queries of clouds c0..c1-1,
// and search_batch over that range writes exactly their results.
template <typename T, int D>
int order_batch(const BatchArgs& b, cudaStream_t stream) {
  if (b.nq == 0) return kOk;
  // the forest's node count (nodeOffset[nClouds]) is known on the device
  // only; the histogram's cells past it stay unused
  const int64_t* nodesDev = b.nodeOffset + b.nClouds;
  const int zrc = zero_u32(b.hist, b.nodeCap, nodesDev, stream);
  if (zrc != kOk) return zrc;
  k_leaf_cells<T, D><<<ceil_div(b.nq, 256), 256, 0, stream>>>(static_cast<const Node<T>*>(b.nodes),
                                                              static_cast<const T*>(b.query), b.nq, b.qStride, b.dim,
                                                              b.cell, b.rank, b.hist, b.qOffset, b.nodeOffset,
                                                              b.nClouds);
  return order_by_cells(b.cell, b.rank, b.hist, b.nodeCap, b.nq, b.order, stream, nodesDev);
}

template <typename T, int D>
int search_batch(const BatchArgs& b, int64_t begin, int64_t end, cudaStream_t stream) {
  if (end <= begin) return kOk;
  int K = round_k(b.kMax);
  if (K < 0 && b.kMax > kMaxWideK) return k_unsupported();
  int rc = kOk;
  KnnLaunch L;
  std::memset(&L, 0, sizeof(L));
  L.nodes = b.nodes;
  L.recs = b.recs;
  L.query = b.query;
  L.nq = end - begin;
  L.qStride = b.qStride;
  L.dim = b.dim;
  L.order = b.order + begin;
  L.k = b.kMax;
  const T eps = (T)b.eps;
  const T e1 = T(1) + eps;
  L.maxError2 = (double)(T)(e1 * e1);
  const T r = (T)b.maxRadius;
  L.maxRadius2 = (double)(T)(r * r);
  L.outIdx = b.indices;
  L.outD2 = b.dists2;
  L.allowSelf = (b.optionFlags & 1u) ? 1 : 0;
  L.bQueryOffset = b.qOffset;
  L.bNodeOffset = b.nodeOffset;
  L.bK = b.kOf;
  L.bOutOffset = b.outOffset;
  L.bClouds = b.nClouds;
  L.recs32 = b.recs32;
  L.coordMax = b.coordMax;
  L.maxRadii = b.maxRadii;
  L.fallbackRadius = b.maxRadii ? b.maxRadius : -1.0;
  L.fallbacks = b.fallbacks;
  // The trees' heights are known only on the device: the kernels below keep
  // stacks of kStackLarge entries and return at once if the tallest tree
  // (read from the build's status) is taller; the deep kernel launched after
  // them then searches the range with stacks in b.slab sized by that tree,
  // and otherwise returns at once.
  L.tallGate = b.heightDev;
  L.tallGateLimit = kStackLarge;
  const int grid = ceil_div(L.nq, b.blockSize);
  if (K < 0) {  // some cloud wants more than kMaxK: the whole batch runs a lane group per query
    rc = launch_wide_kdtree<T, D>(L, b.kMax, kStackLarge, stream);
    if (rc != kOk) return rc == kNeedsSlab ? set_error(kErrInternal, "batched wide search stacks") : rc;
  } else if (b.lanesPerQuery == 8) {  // 8 lanes per query, the top-k spread over them
    rc = K <= 16 ? launch_wide_kdtree_as<T, D, 2, 8>(L, kStackLarge, stream)
                 : launch_wide_kdtree_as<T, D, 4, 8>(L, kStackLarge, stream);
    if (rc != kOk) return rc == kNeedsSlab ? set_error(kErrInternal, "batched group search stacks") : rc;
    K = 0;
  }
#define NABO_LAUNCH(KK)                                                                     \
  case KK:                                                                                  \
    launch_kdtree<T, D, KK, kStackLarge>(g, b.blockSize, stream, G);                        \
    break;
#define NABO_LAUNCH_ON(KK)                                                                  \
  case KK:                                                                                  \
    launch_kdtree<T, D, KK, kStackLarge>(g, b.blockSize, gs, G);                            \
    break;
  const BatchClassPlan* cp = b.classes;
  if (K > 0 && cp && cp->groups > 0 && b.hQOffset) {
    // one launch per group of clouds sharing a compiled top-k size, over the
    // group's clouds whose queries lie in [begin, end). The largest size
    // goes first on the caller's stream, the others side by side on two
    // more (forked from and joined back into it), so that their blocks fill
    // the SMs the register-heavy largest one leaves free and its tail.
    const int64_t* qo = b.hQOffset;
    const bool fork = cp->groups > 1 && b.aux[0] && b.aux[1] && b.evFork && b.evJoin[0] && b.evJoin[1];
    bool used[2] = {false, false};
    int next = 0;
    if (fork) NABO_CUDA_TRY(cudaEventRecord(b.evFork, stream));
    for (int gi = cp->groups - 1; gi >= 0; --gi) {
      const int32_t* rc0 = cp->runCloud.data();
      const int* r0p = std::lower_bound(rc0 + cp->runBegin[gi], rc0 + cp->runBegin[gi + 1], 0,
                                        [&](int32_t c, int) { return qo[c] < begin; });
      const int* r1p = std::lower_bound(r0p, rc0 + cp->runBegin[gi + 1], 0,
                                        [&](int32_t c, int) { return qo[c + 1] <= end; });
      const int r0 = (int)(r0p - rc0), r1 = (int)(r1p - rc0);
      if (r1 <= r0) continue;
      KnnLaunch G = L;
      G.order = b.order;
      G.runPrefix = cp->dRunPrefix;
      G.runCloud = cp->dRunCloud;
      G.runBegin = r0;
      G.runEnd = r1;
      G.nq = cp->runPrefix[(size_t)r1] - cp->runPrefix[(size_t)r0];
      G.k = cp->K[(size_t)gi];
      const int g = ceil_div(G.nq, b.blockSize);
      cudaStream_t gs = stream;
      if (fork && gi != cp->groups - 1) {
        const int a = next++ & 1;
        gs = b.aux[a];
        if (!used[a]) NABO_CUDA_TRY(cudaStreamWaitEvent(gs, b.evFork, 0));
        used[a] = true;
      }
      switch (round_k(cp->K[(size_t)gi])) { NABO_K_LIST(NABO_LAUNCH_ON) }
    }
    for (int a = 0; a < 2; ++a) {
      if (!used[a]) continue;
      NABO_CUDA_TRY(cudaEventRecord(b.evJoin[a], b.aux[a]));
      NABO_CUDA_TRY(cudaStreamWaitEvent(stream, b.evJoin[a], 0));
    }
  } else if (K > 0) {
    KnnLaunch G = L;
    const int g = grid;
    switch (K) { NABO_K_LIST(NABO_LAUNCH) }
  }
#undef NABO_LAUNCH
#undef NABO_LAUNCH_ON
  {
    KnnLaunch R = L;
    R.slab = b.slab;
    R.slabBytes = b.slabBytes;
    R.stackCap = 0;
    R.stackHeightDev = b.heightDev;
    R.deepFail = b.deepFail;
    // enough threads for every stack the slab holds once trees are taller
    // than kStackLarge
    const int64_t units = std::max<int64_t>(1, b.slabBytes / deep_unit_bytes<T, D>(b.kMax, kStackLarge + 1));
    rc = launch_deep<T, D>(R, b.kMax, std::min<int64_t>(units, L.nq), stream);
    if (rc != kOk) return rc;
  }
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_error(e, "batched search launch");
  return kOk;
}

template <typename T, int D>
int knn_batch(const BatchArgs& b, cudaStream_t stream) {
  if (b.nq == 0) return kOk;
  const int rc = order_batch<T, D>(b, stream);
  return rc != kOk ? rc : search_batch<T, D>(b, 0, b.nq, stream);
}

#define NABO_SEARCH_INSTANTIATE(T, D)                                              \
  template int knn_batch<T, D>(const BatchArgs&, cudaStream_t);                    \
  template int order_batch<T, D>(const BatchArgs&, cudaStream_t);                  \
  template int search_batch<T, D>(const BatchArgs&, int64_t, int64_t, cudaStream_t); \
  template int knn_leaf_order<T, D>(const DeviceCloud&, const void*, int64_t, int64_t, int32_t*, cudaStream_t); \
  template int knn_kdtree<T, D>(const DeviceCloud&, const KnnArgs&, cudaStream_t); \
  template int knn_bruteforce<T, D>(const DeviceCloud&, const KnnArgs&, cudaStream_t); \
  template int knn_kdtree_given_order<T, D>(const DeviceCloud&, const KnnArgs&, const int32_t*, cudaStream_t); \
  template int knn_chunk_order<T, D>(const DeviceCloud&, const void*, int64_t, int64_t, const QueryChunks&, int32_t*, \
                                     cudaStream_t, void*);

}  // namespace nabo_gb300
