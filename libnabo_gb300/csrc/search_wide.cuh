// search_wide.cuh -- kNN for k above 32: a group of G lanes per query.
//
// The reference's heaps have no cap on k (nabo/index_heap.h:51-165 grows an
// STL heap to k entries, nabo/index_heap.h:263-369 keeps a sorted vector of
// k). One thread's registers hold at most 32 (dist2, index) pairs, so for
// larger k a group of G lanes (8, 16 or 32; 32 / G queries per warp) serves
// one query: the top-k is spread over the group's registers, the traversal
// runs once per group (every lane of a group holds the same query state, so
// a group never diverges), a leaf's points are taken one per lane, and an
// insertion costs each lane a few compares and selects on its own slots
// plus one shuffle. Visit order, pruning tests, self-match rule, tie rule
// and TOUCH_STATISTICS are the one-thread kernels' (the reference's
// recurseKnn, nabo/kdtree_cpu.cpp:367-447), so results are identical to
// theirs and to the reference's for any k.
#pragma once

#include "search.cuh"

namespace nabo_gb300 {

// The lanes of the G-lane group holding `lane` (G divides 32).
template <int G>
__device__ __forceinline__ unsigned group_mask(int lane) {
  if constexpr (G == 32)
    return 0xffffffffu;
  else
    return ((1u << G) - 1u) << (lane & ~(G - 1));
}

// A group's top-k with K = G*M slots in ascending order; group lane g holds
// slots [g*M, g*M + M) in registers. The live entries are the last k slots,
// so the head (the k-th smallest pair) is always the group's last lane's
// last register; the K-k slots before them hold padding that orders below
// every pair. Inserting a pair below the head drops the head and moves every
// slot above the insertion point up by one: each lane compares and selects
// its own M slots and takes the slot below its first one from the previous
// lane. Called by all lanes of the group with the same arguments.
template <typename T, int M, int G>
struct GroupTopK;

// float: packed (dist2 bits << 32 | index) keys, as the one-thread TopK;
// an empty slot is (+inf, 0) and is written out as (-1, +inf); padding is 0.
template <int M, int G>
struct GroupTopK<float, M, G> {
  static constexpr int K = G * M;
  static constexpr uint64_t kEmpty = uint64_t(0x7f800000u) << 32;
  uint64_t a[M];
  uint64_t h;  // the head key, the same in every lane of the group
  __device__ __forceinline__ void init(int k, int g) {
#pragma unroll
    for (int r = 0; r < M; ++r) a[r] = g * M + r >= K - k ? kEmpty : 0ull;
    h = kEmpty;
  }
  __device__ __forceinline__ float head() const { return __uint_as_float((uint32_t)(h >> 32)); }
  // x < h
  __device__ __forceinline__ void insert_key(uint64_t x, int g, unsigned gm) {
    uint64_t prev = __shfl_up_sync(gm, a[M - 1], 1, G);
    if (g == 0) prev = 0ull;
    bool gt[M];
#pragma unroll
    for (int r = 0; r < M; ++r) gt[r] = a[r] > x;
#pragma unroll
    for (int r = M - 1; r >= 1; --r) a[r] = gt[r] ? (gt[r - 1] ? a[r - 1] : x) : a[r];
    a[0] = gt[0] ? (prev > x ? prev : x) : a[0];
    h = __shfl_sync(gm, a[M - 1], G - 1, G);
  }
  __device__ __forceinline__ int count(int k, int g, unsigned gm) const {
    int c = 0;
#pragma unroll
    for (int r = 0; r < M; ++r) c += (g * M + r >= K - k && (uint32_t)(a[r] >> 32) != 0x7f800000u) ? 1 : 0;
    return __reduce_add_sync(gm, c);
  }
  // The k entries in ascending order; returns how many are valid.
  __device__ __forceinline__ int store(int k, int g, unsigned gm, int32_t* __restrict__ oi,
                                       float* __restrict__ od) const {
#pragma unroll
    for (int r = 0; r < M; ++r) {
      const int s = g * M + r;
      if (s >= K - k) {
        const uint32_t db = (uint32_t)(a[r] >> 32);
        oi[s - (K - k)] = db == 0x7f800000u ? -1 : (int32_t)(uint32_t)a[r];
        od[s - (K - k)] = __uint_as_float(db);
      }
    }
    return count(k, g, gm);
  }
};

// double: (bit pattern of dist2, index) pairs compared as integers, as the
// one-thread TopK; an empty slot is (+inf, -1), padding (0, -1).
template <int M, int G>
struct GroupTopK<double, M, G> {
  static constexpr int K = G * M;
  unsigned long long d[M];
  int i[M];
  unsigned long long hd;
  int hi;
  static __device__ __forceinline__ bool greater(unsigned long long da, int ia, unsigned long long db, int ib) {
    return da > db || (da == db && ia > ib);
  }
  static __device__ __forceinline__ unsigned long long bits(double x) {
    return (unsigned long long)__double_as_longlong(x);
  }
  __device__ __forceinline__ void init(int k, int g) {
    const unsigned long long inf = bits(Ar<double>::inf());
#pragma unroll
    for (int r = 0; r < M; ++r) {
      d[r] = g * M + r >= K - k ? inf : 0ull;
      i[r] = -1;
    }
    hd = inf;
    hi = -1;
  }
  __device__ __forceinline__ double head() const { return __longlong_as_double((long long)hd); }
  __device__ __forceinline__ bool accepts(double dist, int idx) const { return greater(hd, hi, bits(dist), idx); }
  // accepts(dist, idx)
  __device__ __forceinline__ void insert(double dist, int idx, int g, unsigned gm) {
    const unsigned long long x = bits(dist);
    unsigned long long pd = __shfl_up_sync(gm, d[M - 1], 1, G);
    int pi = __shfl_up_sync(gm, i[M - 1], 1, G);
    if (g == 0) {
      pd = 0ull;
      pi = -1;
    }
    bool gt[M];
#pragma unroll
    for (int r = 0; r < M; ++r) gt[r] = greater(d[r], i[r], x, idx);
#pragma unroll
    for (int r = M - 1; r >= 1; --r) {
      d[r] = gt[r] ? (gt[r - 1] ? d[r - 1] : x) : d[r];
      i[r] = gt[r] ? (gt[r - 1] ? i[r - 1] : idx) : i[r];
    }
    const bool gp = greater(pd, pi, x, idx);
    d[0] = gt[0] ? (gp ? pd : x) : d[0];
    i[0] = gt[0] ? (gp ? pi : idx) : i[0];
    hd = __shfl_sync(gm, d[M - 1], G - 1, G);
    hi = __shfl_sync(gm, i[M - 1], G - 1, G);
  }
  __device__ __forceinline__ int count(int k, int g, unsigned gm) const {
    int c = 0;
#pragma unroll
    for (int r = 0; r < M; ++r) c += (g * M + r >= K - k && i[r] >= 0) ? 1 : 0;
    return __reduce_add_sync(gm, c);
  }
  __device__ __forceinline__ int store(int k, int g, unsigned gm, int32_t* __restrict__ oi,
                                       double* __restrict__ od) const {
#pragma unroll
    for (int r = 0; r < M; ++r) {
      const int s = g * M + r;
      if (s >= K - k) {
        oi[s - (K - k)] = i[r];
        od[s - (K - k)] = __longlong_as_double((long long)d[r]);
      }
    }
    return count(k, g, gm);
  }
};

// Offers the records [first, first + G) (those below avail), one per group
// lane, to the group's top-k: each lane tests its point against the head as
// it was when the batch started, and the candidates are inserted one by one
// in lane order, each re-tested against the current head. The k smallest
// pairs after the batch do not depend on that order. kShared: the records
// sit in shared memory (read with plain loads, not the read-only global
// path).
template <typename T, int D, int M, int G, bool kShared>
__device__ __forceinline__ void wide_offer(const Rec<T, D>* __restrict__ recs, int64_t first, int avail,
                                           const T (&q)[D], T maxRadius2, T minDist, GroupTopK<T, M, G>& heap,
                                           const LeafFilter<T, D>& flt, int g, unsigned gm) {
  const int shift = __ffs(gm) - 1;  // the group's first lane in the warp
  if constexpr (std::is_same<T, float>::value) {
    uint64_t key = ~0ull;
    bool ok = false;
    if (g < avail) {
      Rec<T, D> r;
      if constexpr (kShared)
        r = recs[first + g];
      else
        load_rec(recs, first + g, r);
      const float dist = dist2_seq(q, r);
      key = TopK<float, 1>::make(dist, r.p.idx);
      ok = dist <= maxRadius2 && key < heap.h && dist > minDist;
    }
    unsigned mask = (__ballot_sync(gm, ok) & gm) >> shift;
    while (mask) {
      const int src = __ffs(mask) - 1;
      mask &= mask - 1;
      const uint64_t x = __shfl_sync(gm, key, src, G);
      if (x < heap.h) heap.insert_key(x, g, gm);
    }
  } else {
    T dist = Ar<T>::inf();
    int idx = -1;
    bool ok = false;
    const float thr = flt.on() ? flt.threshold(heap.head(), maxRadius2) : 0.0f;
    if (g < avail && !(flt.on() && flt.rejects(first + g, thr))) {
      Rec<T, D> r;
      if constexpr (kShared)
        r = recs[first + g];
      else
        load_rec(recs, first + g, r);
      dist = dist2_seq(q, r);
      idx = r.p.idx;
      ok = dist <= maxRadius2 && heap.accepts(dist, idx) && dist > minDist;
    }
    unsigned mask = (__ballot_sync(gm, ok) & gm) >> shift;
    while (mask) {
      const int src = __ffs(mask) - 1;
      mask &= mask - 1;
      const T dv = __shfl_sync(gm, dist, src, G);
      const int iv = __shfl_sync(gm, idx, src, G);
      if (heap.accepts(dv, iv)) heap.insert(dv, iv, g, gm);
    }
  }
}

// Memory of one group's traversal stack: cap entries of rd, off[D] (T each)
// and the node (uint32). In shared memory a block lays out all groups' T
// parts followed by all groups' node parts; in a deep launch's global slab
// each group has its own region of this size (rounded up to 16 bytes).
template <typename T, int D>
inline size_t wide_stack_bytes(int groups, int cap) {
  return (size_t)groups * (size_t)cap * ((D + 1) * sizeof(T) + sizeof(uint32_t));
}
template <typename T, int D>
__host__ __device__ inline int64_t wide_group_slab_bytes(int cap) {
  return ((int64_t)cap * (int64_t)((D + 1) * sizeof(T) + sizeof(uint32_t)) + 15) & ~int64_t(15);
}

// One query (order position t) searched by the G-lane group: the
// reference's visit order with the stack at sRd / sOff / sNode (cap
// entries), written by the group's first lane and read by all its lanes;
// the caller guarantees cap > tree height.
template <typename T, int D, int M, int G>
__device__ __forceinline__ void wide_query(const KnnLaunch& a, int64_t t, T* sRd, T* sOff, uint32_t* sNode, int cap,
                                           int g, unsigned gm, uint32_t& touchedOut) {
  // the reference's self-match rule (nabo/kdtree_cpu.cpp:392-396)
  const T minDist = a.allowSelf ? T(-1) : Ar<T>::eps();
  const Node<T>* __restrict__ nodes = static_cast<const Node<T>*>(a.nodes);
  const Rec<T, D>* __restrict__ recs = static_cast<const Rec<T, D>*>(a.recs);
  const T* __restrict__ query = static_cast<const T*>(a.query);
  uint32_t touched = 0;
  const int64_t qi = a.order ? (int64_t)a.order[t] : t;
  int k = a.k;
  uint32_t root = 0;
  int64_t outBase = qi * (int64_t)a.k;
  if (a.bQueryOffset) {
    const int c = cloud_of(a.bQueryOffset, a.bClouds, qi);
    k = a.bK[c];
    root = (uint32_t)a.bNodeOffset[c];
    outBase = a.bOutOffset[c] + (qi - a.bQueryOffset[c]) * (int64_t)k;
  }
  T q[D];
#pragma unroll
  for (int d = 0; d < D; ++d) q[d] = d < a.dim ? query[qi * a.qStride + d] : T(0);
  T maxRadius2 = (T)a.maxRadius2;
  bool mayFall = false;
  if (a.maxRadii) {
    const T r = static_cast<const T*>(a.maxRadii)[qi];
    maxRadius2 = Ar<T>::mul(r, r);
    mayFall = a.fallbackRadius >= 0.0 && (double)r < a.fallbackRadius;
  }
  const T maxError2 = (T)a.maxError2;
  GroupTopK<T, M, G> heap;
  heap.init(k, g);
  LeafFilter<T, D> flt;
  flt.init(a.recs32, a.coordMax, q);
  T off[D];
  for (;;) {  // the search, and at most once more without the bound
#pragma unroll
    for (int d = 0; d < D; ++d) off[d] = T(0);
    int sp = 0;
    uint32_t node = root;
    T rd = T(0);
    for (;;) {
      __syncwarp(gm);  // the last pop's reads come before the next pushes
      Node<T> nd = load_node(nodes, node);
      while (!node_is_leaf(nd.meta)) {
        const int cd = (int)node_dim(nd.meta);
        const T newOff = Ar<T>::sub(pick(q, cd), nd.cut);
        const T oldOff = pick(off, cd);
        const T rdFar = Ar<T>::add(rd, Ar<T>::add(-Ar<T>::mul(oldOff, oldOff), Ar<T>::mul(newOff, newOff)));
        const uint32_t right = node_payload(nd.meta);
        const uint32_t nearN = newOff > T(0) ? right : node + 1;
        const uint32_t farN = newOff > T(0) ? node + 1 : right;
        const bool far = rdFar <= maxRadius2 && Ar<T>::mul(rdFar, maxError2) <= heap.head() && sp < cap;
        if (far) {
          if (g == 0) {
            sRd[sp] = rdFar;
#pragma unroll
            for (int d = 0; d < D; ++d) sOff[(size_t)sp * D + d] = d == cd ? newOff : off[d];
            sNode[sp] = farN;
          }
          ++sp;
        }
        node = nearN;
        nd = load_node(nodes, node);
      }
      const uint32_t cnt = node_payload(nd.meta);
      const uint32_t st = node_start(nd);
      for (uint32_t base = 0; base < cnt; base += G)
        wide_offer<T, D, M, G, false>(recs, (int64_t)st + base, (int)(cnt - base), q, maxRadius2, minDist, heap,
                                      flt, g, gm);
      touched += cnt;
      __syncwarp(gm);  // the first lane's pushes are visible to the group
      bool more = false;
      while (sp > 0) {
        --sp;
        const T e = sRd[sp];
        if (Ar<T>::mul(e, maxError2) <= heap.head()) {
          rd = e;
#pragma unroll
          for (int d = 0; d < D; ++d) off[d] = sOff[(size_t)sp * D + d];
          node = sNode[sp];
          more = true;
          break;
        }
      }
      if (!more) break;
    }
    if (!mayFall || heap.count(k, g, gm) == k) break;
    mayFall = false;
    maxRadius2 = (T)a.maxRadius2;
    heap.init(k, g);
    if (a.fallbacks && g == 0) atomicAdd(a.fallbacks, 1);
  }
  const int f = heap.store(k, g, gm, a.outIdx + outBase, static_cast<T*>(a.outD2) + outBase);
  if (a.found && g == 0) a.found[qi] = f;
  touchedOut += touched;
}

// Reference-order kd-tree search, one G-lane group per query (blockDim.x / G
// queries per block), stacks in shared memory; `cap` > the tree height
// bounds them (batches: returns at once when a.tallGate says a tree is
// taller, k_knn_kdtree_wide_deep searching instead).
template <typename T, int D, int M, int G>
__global__ void __launch_bounds__(128) k_knn_kdtree_wide(KnnLaunch a, int cap) {
  if (a.tallGate && *a.tallGate > a.tallGateLimit) return;  // uniform
  extern __shared__ __align__(16) unsigned char wideSmem[];
  const int lane = threadIdx.x & 31;
  const int g = lane & (G - 1);  // lane within the group
  const unsigned gm = group_mask<G>(lane);
  const int group = threadIdx.x / G;
  const int groups = blockDim.x / G;
  T* const sRd = reinterpret_cast<T*>(wideSmem) + (size_t)group * cap * (D + 1);
  T* const sOff = sRd + cap;
  uint32_t* const sNode = reinterpret_cast<uint32_t*>(reinterpret_cast<T*>(wideSmem) + (size_t)groups * cap * (D + 1)) +
                          (size_t)group * cap;
  const int64_t t = (int64_t)blockIdx.x * groups + group;
  uint32_t touched = 0;
  if (t < a.nq && (!a.nqDevice || t < (int64_t)*a.nqDevice))
    wide_query<T, D, M, G>(a, t, sRd, sOff, sNode, cap, g, gm, touched);
  if (a.stats && g == 0 && touched) atomicAdd(a.touched, (unsigned long long)touched);
}

// Trees of any height, k above 32: each group's stack in its own region of
// the global slab a.slab (cap = a.stackCap, or the height read from
// *a.stackHeightDev plus one); as many groups as the slab holds search, each
// taking every active-th query. A slab too small for one stack searches
// nothing and sets *a.deepFail to -1.
template <typename T, int D, int M, int G>
__global__ void __launch_bounds__(128) k_knn_kdtree_wide_deep(KnnLaunch a) {
  if (a.tallGate && *a.tallGate <= a.tallGateLimit) return;  // uniform
  const int lane = threadIdx.x & 31;
  const int g = lane & (G - 1);
  const unsigned gm = group_mask<G>(lane);
  const int64_t gid = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / G;
  const int64_t groupsAll = ((int64_t)gridDim.x * blockDim.x) / G;
  const int cap = a.stackCap > 0 ? a.stackCap : (a.stackHeightDev ? *a.stackHeightDev + 1 : 0);
  const int64_t per = wide_group_slab_bytes<T, D>(cap);
  int64_t active = cap > 0 ? a.slabBytes / per : 0;
  if (active > groupsAll) active = groupsAll;
  if (active <= 0 && a.nq > 0 && gid == 0 && g == 0 && a.deepFail) *a.deepFail = -1;
  uint32_t touched = 0;
  if (gid < active) {
    unsigned char* region = static_cast<unsigned char*>(a.slab) + gid * per;
    T* sRd = reinterpret_cast<T*>(region);
    T* sOff = sRd + cap;
    uint32_t* sNode = reinterpret_cast<uint32_t*>(sRd + (size_t)cap * (D + 1));
    for (int64_t t = gid; t < a.nq; t += active) {
      if (a.nqDevice && t >= (int64_t)*a.nqDevice) continue;
      wide_query<T, D, M, G>(a, t, sRd, sOff, sNode, cap, g, gm, touched);
    }
  }
  if (a.stats && g == 0 && touched) atomicAdd(a.touched, (unsigned long long)touched);
}

// Brute force (nabo/brute_force_cpu.cpp:63-103) for k above 32: one warp per
// query, blockDim.x / 32 queries per block sharing tiles of points staged in
// shared memory; each lane takes every 32nd point of a tile.
template <typename T, int D, int M>
__global__ void __launch_bounds__(256) k_knn_bruteforce_wide(KnnLaunch a) {
  const T minDist = a.allowSelf ? T(-1) : Ar<T>::eps();
  constexpr int kTile = (int)((24 * 1024) / sizeof(Rec<T, D>));
  __shared__ Rec<T, D> tile[kTile];
  const int lane = threadIdx.x & 31;
  const int warps = blockDim.x >> 5;
  const Rec<T, D>* __restrict__ recs = static_cast<const Rec<T, D>*>(a.recs);
  const T* __restrict__ query = static_cast<const T*>(a.query);
  const int64_t t = (int64_t)blockIdx.x * warps + (threadIdx.x >> 5);
  const bool active = t < a.nq;
  const int64_t qi = active ? (a.order ? (int64_t)a.order[t] : t) : 0;
  T q[D];
#pragma unroll
  for (int d = 0; d < D; ++d) q[d] = (active && d < a.dim) ? query[qi * a.qStride + d] : T(0);
  T maxRadius2 = (T)a.maxRadius2;
  if (a.maxRadii && active) {
    const T r = static_cast<const T*>(a.maxRadii)[qi];
    maxRadius2 = Ar<T>::mul(r, r);
  }
  GroupTopK<T, M, 32> heap;
  heap.init(a.k, lane);
  LeafFilter<T, D> flt;
  flt.init(nullptr, nullptr, q);
  for (int64_t base = 0; base < a.n; base += kTile) {
    const int m = (int)((a.n - base) < kTile ? (a.n - base) : kTile);
    __syncthreads();
    {
      const uint4* src = reinterpret_cast<const uint4*>(recs + base);
      uint4* dst = reinterpret_cast<uint4*>(tile);
      const int words = m * RecSize<T, D>::chunks;
      for (int w = threadIdx.x; w < words; w += blockDim.x) dst[w] = __ldg(src + w);
    }
    __syncthreads();
    if (active)
      for (int j = 0; j < m; j += 32)
        wide_offer<T, D, M, 32, true>(tile, j, m - j, q, maxRadius2, minDist, heap, flt, lane, 0xffffffffu);
  }
  if (active) {
    const int f = heap.store(a.k, lane, 0xffffffffu, a.outIdx + qi * a.k, static_cast<T*>(a.outD2) + qi * a.k);
    if (a.found && lane == 0) a.found[qi] = f;
  }
}

}  // namespace nabo_gb300
