// search.cuh -- kd-tree and brute-force kNN kernels (templates).
//
// One thread per query. The traversal is the reference's recurseKnn
// (nabo/kdtree_cpu.cpp:367-447) turned into a loop with an explicit stack:
// at an inner node the near child is entered at once and the far child is
// pushed with its incremental box distance
//     rd_far = rd + (-(old_off*old_off) + new_off*new_off)
// and the offset vector it must see; a popped far child is visited iff
//     rd_far <= maxRadius^2  and  rd_far * (1+eps)^2 <= head.
// The far child is pushed only if that test already holds, which changes no
// decision because head never grows. Every +,-,* is separately rounded
// (no FMA contraction) so distances are bit-identical to the CPU oracle.
//
// Top-k: K (dist2, index) entries in registers, kept in descending order so
// the head (largest) is slot 0; slots >= k hold a value below every entry so
// one instantiation serves every k <= K. Entries are ordered by (dist2,
// index): among equal distances the lower index is kept, which makes the
// result independent of visit order (the reference's
// IndexHeapBruteForceVector keeps the first visited, nabo/index_heap.h:
// 322-334). Insertion is branch-free: with g[j] = (slot j > new entry),
// which is true for a prefix of the slots, slot j takes slot j+1 while
// g[j+1], the new entry where the prefix ends, and keeps its value after.
#pragma once

#include <type_traits>

#include "common.cuh"

namespace nabo_gb300 {

// double: the distance's 64-bit pattern and the index in separate arrays.
// Distances are >= 0, where the pattern orders like the value, so the
// (dist2, index) order is decided by integer compares on the ALU, keeping
// the scarce FP64 pipe for distances. An empty slot is (+inf, -1): no finite
// distance compares above it, as the reference's strict `dist < head` with
// head = +inf; padding slots (>= k) hold (+0, -1), below every entry.
template <typename T, int K>
struct TopK {
  unsigned long long d[K];
  int i[K];
  static __device__ __forceinline__ bool greater(unsigned long long da, int ia, unsigned long long db, int ib) {
    return da > db || (da == db && ia > ib);
  }
  static __device__ __forceinline__ unsigned long long bits(T x) {
    return (unsigned long long)__double_as_longlong((double)x);
  }
  __device__ __forceinline__ void init(int k) {
#pragma unroll
    for (int j = 0; j < K; ++j) {
      d[j] = j < k ? bits(Ar<T>::inf()) : 0ull;
      i[j] = -1;
    }
  }
  __device__ __forceinline__ T head() const { return (T)__longlong_as_double((long long)d[0]); }
  __device__ __forceinline__ bool accepts(T dist, int idx) const { return greater(d[0], i[0], bits(dist), idx); }
  // Drops the head and inserts (dist, idx); requires accepts(dist, idx).
  __device__ __forceinline__ void insert(T dist, int idx) {
    const unsigned long long x = bits(dist);
    bool g[K];
#pragma unroll
    for (int j = 0; j < K; ++j) g[j] = greater(d[j], i[j], x, idx);
#pragma unroll
    for (int j = 0; j + 1 < K; ++j) {
      d[j] = g[j + 1] ? d[j + 1] : (g[j] ? x : d[j]);
      i[j] = g[j + 1] ? i[j + 1] : (g[j] ? idx : i[j]);
    }
    d[K - 1] = g[K - 1] ? x : d[K - 1];
    i[K - 1] = g[K - 1] ? idx : i[K - 1];
  }
  __device__ __forceinline__ int count(int k) const {
    int c = 0;
#pragma unroll
    for (int j = 0; j < K; ++j) c += (j < k && i[j] >= 0) ? 1 : 0;
    return c;
  }
  // Writes the k entries in ascending order; returns how many are valid.
  __device__ __forceinline__ int store(int k, int32_t* __restrict__ oi, T* __restrict__ od) const {
    int found = 0;
#pragma unroll
    for (int j = 0; j < K; ++j) {
      if (j < k) {
        oi[k - 1 - j] = i[j];
        od[k - 1 - j] = (T)__longlong_as_double((long long)d[j]);
        found += i[j] >= 0 ? 1 : 0;
      }
    }
    return found;
  }
};

// double lists of 16 or more entries in the kd-tree search: a binary
// max-heap of (dist2 bits, index) in shared memory, slot-major with one
// column per thread (blocks of at most kHeapThreads threads), the root kept
// in registers for the accept test. Held in registers, such a list (3
// registers an entry) spilled under the search kernel's register cap, and
// every insertion walked the spilled entries through local memory (8-D,
// k = 32: 2.2 G local loads a launch). Here an insertion sifts down at most
// log2(k) levels. The entries and their order are those of TopK: the k
// smallest (dist2, index) pairs, empty entries (+inf, -1), written out in
// ascending order.
constexpr int kHeapThreads = 128;
template <int K>
struct SmemTopK {
  unsigned long long* d;  // entry j of this thread's list at d[j * kHeapThreads]
  int* ix;
  int n;
  unsigned long long rootD;
  int rootI;
  static __device__ __forceinline__ bool greater(unsigned long long da, int ia, unsigned long long db, int ib) {
    return da > db || (da == db && ia > ib);
  }
  static __device__ __forceinline__ unsigned long long bits(double x) {
    return (unsigned long long)__double_as_longlong(x);
  }
  __device__ __forceinline__ void init(int k) {
    __shared__ unsigned long long sd[K * kHeapThreads];
    __shared__ int si[K * kHeapThreads];
    d = sd + threadIdx.x;
    ix = si + threadIdx.x;
    n = k < K ? k : K;
    rootD = bits(Ar<double>::inf());
    rootI = -1;
    for (int j = 0; j < n; ++j) {
      d[j * kHeapThreads] = rootD;
      ix[j * kHeapThreads] = -1;
    }
  }
  __device__ __forceinline__ double head() const { return __longlong_as_double((long long)rootD); }
  __device__ __forceinline__ bool accepts(double dist, int idx) const { return greater(rootD, rootI, bits(dist), idx); }
  // The root (the largest entry) drops out and (x, xi) sifts down from it
  // within the first m entries.
  __device__ __forceinline__ void sift(unsigned long long x, int xi, int m) {
    int j = 0;
    for (;;) {
      const int l = 2 * j + 1;
      if (l >= m) break;
      int c = l;
      unsigned long long cd = d[l * kHeapThreads];
      int ci = ix[l * kHeapThreads];
      if (l + 1 < m) {
        const unsigned long long rd = d[(l + 1) * kHeapThreads];
        const int ri = ix[(l + 1) * kHeapThreads];
        if (greater(rd, ri, cd, ci)) {
          c = l + 1;
          cd = rd;
          ci = ri;
        }
      }
      if (!greater(cd, ci, x, xi)) break;
      d[j * kHeapThreads] = cd;
      ix[j * kHeapThreads] = ci;
      j = c;
    }
    d[j * kHeapThreads] = x;
    ix[j * kHeapThreads] = xi;
  }
  // Drops the largest entry and inserts (dist, idx); requires accepts(dist, idx).
  __device__ __forceinline__ void insert(double dist, int idx) {
    sift(bits(dist), idx, n);
    rootD = d[0];
    rootI = ix[0];
  }
  __device__ __forceinline__ int count(int) const {
    int c = 0;
    for (int j = 0; j < n; ++j) c += ix[j * kHeapThreads] >= 0 ? 1 : 0;
    return c;
  }
  // Writes the entries in ascending order (the largest last), emptying the
  // heap; returns how many are valid.
  __device__ __forceinline__ int store(int, int32_t* __restrict__ oi, double* __restrict__ od) {
    int found = 0;
    for (int m = n; m > 0; --m) {
      const unsigned long long top = d[0];
      const int ti = ix[0];
      oi[m - 1] = ti;
      od[m - 1] = __longlong_as_double((long long)top);
      found += ti >= 0 ? 1 : 0;
      if (m > 1) sift(d[(m - 1) * kHeapThreads], ix[(m - 1) * kHeapThreads], m - 1);
    }
    return found;
  }
};

// The list the kd-tree search keeps: shared-memory heaps for double lists
// of 16 or more entries, registers otherwise. (Float lists stay in
// registers: the same heap over packed float keys was slower at every size
// measured -- lidar k = 10 kernel 0.990 -> 1.026 ms, batched k = 16 search
// 13.67 -> 14.60 ms, 8-D k = 32 search 92 -> 126 ms -- since the sorted
// register list's insertion is branch-free and a sift waits on dependent
// shared-memory loads; double lists spilled, float ones hardly.)
template <typename T, int K>
struct SearchHeap {
  using type = TopK<T, K>;
};
template <int K>
struct SearchHeap<double, K> {
  using type = std::conditional_t<(K >= 16), SmemTopK<K>, TopK<double, K>>;
};

// float: one 64-bit key per entry, (bit pattern of dist2) << 32 | index.
// Distances are >= 0, where the IEEE bit pattern orders like the value, so
// one unsigned comparison orders (dist2, index). An empty slot is
// (+inf, 0): no finite distance compares above it and no infinite one
// below, as the reference's strict `dist < head` with head = +inf
// (nabo/kdtree_cpu.cpp:392-396); it is written out as (-1, +inf). Padding
// slots (>= k) hold 0.
template <int K>
struct TopK<float, K> {
  uint64_t key[K];
  static __device__ __forceinline__ uint64_t make(float dist, int idx) {
    return (uint64_t(__float_as_uint(dist)) << 32) | (uint32_t)idx;
  }
  __device__ __forceinline__ void init(int k) {
#pragma unroll
    for (int j = 0; j < K; ++j) key[j] = j < k ? (uint64_t(0x7f800000u) << 32) : 0ull;
  }
  __device__ __forceinline__ float head() const { return __uint_as_float((uint32_t)(key[0] >> 32)); }
  __device__ __forceinline__ bool accepts(float dist, int idx) const { return make(dist, idx) < key[0]; }
  __device__ __forceinline__ void insert(float dist, int idx) { insert_key(make(dist, idx)); }
  // requires x < key[0]
  __device__ __forceinline__ void insert_key(uint64_t x) {
    bool g[K];
#pragma unroll
    for (int j = 0; j < K; ++j) g[j] = key[j] > x;
#pragma unroll
    for (int j = 0; j + 1 < K; ++j) key[j] = g[j + 1] ? key[j + 1] : (g[j] ? x : key[j]);
    key[K - 1] = g[K - 1] ? x : key[K - 1];
  }
  __device__ __forceinline__ int count(int k) const {
    int c = 0;
#pragma unroll
    for (int j = 0; j < K; ++j) c += (j < k && (uint32_t)(key[j] >> 32) != 0x7f800000u) ? 1 : 0;
    return c;
  }
  __device__ __forceinline__ uint32_t out_idx(int j) const {
    return (uint32_t)(key[j] >> 32) == 0x7f800000u ? 0xffffffffu : (uint32_t)key[j];
  }
  // Writes the k entries in ascending order (slot j goes to position
  // k-1-j); returns how many are valid. When both rows are 8-byte aligned,
  // positions (p, p+1) with p even go out as one 64-bit store per row.
  __device__ __forceinline__ int store(int k, int32_t* __restrict__ oi, float* __restrict__ od) const {
    int found = 0;
    const bool pairs = ((reinterpret_cast<uintptr_t>(oi) | reinterpret_cast<uintptr_t>(od)) & 7u) == 0;
#pragma unroll
    for (int j = 0; j < K; ++j) {
      if (j < k) {
        const int p = k - 1 - j;
        found += (uint32_t)(key[j] >> 32) == 0x7f800000u ? 0 : 1;
        if (!pairs) {
          oi[p] = (int32_t)out_idx(j);
          od[p] = __uint_as_float((uint32_t)(key[j] >> 32));
        } else if ((p & 1) == 0) {
          if (j >= 1) {  // slot j-1 is position p+1
            *reinterpret_cast<uint2*>(oi + p) = make_uint2(out_idx(j), out_idx(j - 1));
            *reinterpret_cast<uint2*>(od + p) = make_uint2((uint32_t)(key[j] >> 32), (uint32_t)(key[j - 1] >> 32));
          } else {
            oi[p] = (int32_t)out_idx(j);
            od[p] = __uint_as_float((uint32_t)(key[j] >> 32));
          }
        }
      }
    }
    return found;
  }
};

template <typename T, int D>
__device__ __forceinline__ T pick(const T (&v)[D], int c) {
  T r = v[0];
#pragma unroll
  for (int d = 1; d < D; ++d)
    if (c == d) r = v[d];
  return r;
}

template <typename T, int D>
__device__ __forceinline__ T dist2_seq(const T (&q)[D], const Rec<T, D>& r) {
  // (q0-p0)^2 first, then +(q1-p1)^2, ... (nabo/kdtree_cpu.cpp:383-391)
  T diff = Ar<T>::sub(q[0], r.p.c[0]);
  T dist = Ar<T>::mul(diff, diff);
#pragma unroll
  for (int d = 1; d < D; ++d) {
    diff = Ar<T>::sub(q[d], r.p.c[d]);
    dist = Ar<T>::add(dist, Ar<T>::mul(diff, diff));
  }
  return dist;
}

// Leaf cells for query ordering: each query's cell is the leaf it reaches
// by always taking its near side (new_off > 0 -> right, as the search
// does). Leaves are numbered in pre-order, so queries sorted by leaf are
// grouped at the scale of the data's own buckets. With `hist` set, also
// counts the queries per leaf and gives each its rank (for a counting
// sort).
template <typename T, int D>
__global__ void k_leaf_cells(const Node<T>* __restrict__ nodes, const T* __restrict__ query, int64_t nq,
                             int64_t qStride, int dim, uint32_t* cell, uint32_t* rank, uint32_t* hist,
                             const int64_t* __restrict__ bQueryOffset = nullptr,
                             const int64_t* __restrict__ bNodeOffset = nullptr, int bClouds = 0) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= nq) return;
  T q[D];
#pragma unroll
  for (int d = 0; d < D; ++d) q[d] = d < dim ? query[i * qStride + d] : T(0);
  uint32_t node = bQueryOffset ? (uint32_t)bNodeOffset[cloud_of(bQueryOffset, bClouds, i)] : 0u;
  for (;;) {
    const Node<T> nd = load_node(nodes, node);
    if (node_is_leaf(nd.meta)) break;
    const T newOff = Ar<T>::sub(pick(q, (int)node_dim(nd.meta)), nd.cut);
    node = newOff > T(0) ? node_payload(nd.meta) : node + 1;
  }
  cell[i] = node;
  if (hist) rank[i] = atomicAdd(hist + node, 1u);
}

struct KnnLaunch {
  const void* nodes;
  const void* recs;
  const void* query;
  int64_t nq;
  int64_t qStride;
  int dim;
  const int32_t* order;
  int k;
  double maxError2;
  double maxRadius2;
  const void* maxRadii;
  int32_t* outIdx;
  void* outD2;
  unsigned long long* touched;
  int32_t* found;
  int64_t n;  // points (brute force)
  int allowSelf;
  int stats;
  const int32_t* nqDevice;  // if set, only threads t < *nqDevice search (t < nq still bounds the grid)
  double fallbackRadius;    // >= 0: bounded searches that miss rerun with maxRadius2 (see KnnArgs)
  int32_t* fallbacks;
  const void* recs32;       // double clouds: float copies of recs for the leaf pre-filter, or null
  const float* coordMax;    // largest coordinate magnitude of the cloud (device float)
  // batches of clouds (all null for one cloud): queries of cloud c are
  // [bQueryOffset[c], bQueryOffset[c+1]), its tree starts at node
  // bNodeOffset[c], it wants bK[c] neighbours written from bOutOffset[c]
  const int64_t* bQueryOffset;
  const int64_t* bNodeOffset;
  const int32_t* bK;
  const int64_t* bOutOffset;
  int bClouds;
  // one group of a batch's queries (see BatchClassPlan): thread t searches
  // position runPrefix[runBegin] + t of the group's running query count;
  // null runPrefix: thread t searches leaf-order position t
  const int64_t* runPrefix;
  const int32_t* runCloud;
  int runBegin, runEnd;
  // Trees taller than the compiled stacks (the reference's recursion has no
  // depth limit, nabo/kdtree_cpu.cpp:367-447):
  //  - slab/slabBytes: traversal stacks in global memory for the deep
  //    kernels, `cap` entries per query (stackCap, or the tree height read
  //    from *stackHeightDev plus one);
  //  - tallGate (batches, whose tree heights only the device knows): the
  //    tallest tree's height. Kernels with stacks of tallGateLimit entries
  //    return at once when it is larger; the deep kernels return at once
  //    when it is not. Both are launched, and exactly one searches.
  //  - deepFail: set to -1 by a deep kernel whose slab holds no stack.
  void* slab;
  int64_t slabBytes;
  int stackCap;
  const int* stackHeightDev;
  const int* tallGate;
  int tallGateLimit;
  int32_t* deepFail;
};

// Leaf scan shared by the kernels: the bucket's records are read in chunks
// of 4 (independent loads in flight; the reference's buckets of at most 8
// hold 3.8 points on average on lidar scans, so wider chunks mostly compute
// empty slots), candidates that beat the current head are collected in a
// bit mask and inserted afterwards. The order of insertion inside a leaf
// does not change the heap after the leaf (the k smallest pairs of the
// union), so this matches the reference's point-by-point loop
// (nabo/kdtree_cpu.cpp:378-398); the warp pays for the largest number of
// insertions of any lane instead of for every point where some lane
// inserts.
// Float pre-filter of leaf points for double clouds (the GB300 runs FP64 at
// 1/64 of its FP32 rate, and the leaf distances are most of a double
// search's arithmetic). With q~ and p~ the float roundings of the query and
// point coordinates and e = (max|q~| + max|p~|) * 2^-22, every coordinate
// difference satisfies |q - p| >= |q~ - p~|_float - e (conversion and
// subtraction errors are at most 2.1 * 2^-24 * (|q| + |p|) each), so
//     LB = sum_d max(0, |q~_d - p~_d| - e)^2,  taken * (1 - 2^-17)
// is below the exact squared distance, float roundings of LB itself and the
// double sum's own rounding included. A point with LB above a float at or
// above min(head, maxRadius^2) cannot enter the heap, and only the others
// get the exact double distance: results are unchanged. Coordinates beyond
// the float range make e infinite, which rejects nothing.
template <typename T, int D>
struct LeafFilter {
  __device__ __forceinline__ void init(const void*, const float*, const T (&)[D]) {}
  __device__ __forceinline__ bool on() const { return false; }
  __device__ __forceinline__ float threshold(T, T) const { return 0.0f; }
  __device__ __forceinline__ bool rejects(int64_t, float) const { return false; }
};

template <int D>
struct LeafFilter<double, D> {
  const Rec<float, D>* recs32;
  float qf[D];
  float e;
  __device__ __forceinline__ void init(const void* r32, const float* coordMax, const double (&q)[D]) {
    recs32 = static_cast<const Rec<float, D>*>(r32);
    e = Ar<float>::inf();
    if (recs32) {
      float mq = 0.0f;
#pragma unroll
      for (int d = 0; d < D; ++d) {
        qf[d] = (float)q[d];
        mq = fmaxf(mq, fabsf(qf[d]));
      }
      e = (mq + *coordMax) * 0x1p-22f;
    }
  }
  __device__ __forceinline__ bool on() const { return recs32 != nullptr; }
  // a float at or above min(head, maxRadius2)
  __device__ __forceinline__ float threshold(double head, double maxRadius2) const {
    return __double2float_ru(fmin(head, maxRadius2));
  }
  __device__ __forceinline__ bool rejects(int64_t i, float thr) const {
    Rec<float, D> f;
    load_rec(recs32, i, f);
    float lb = 0.0f;
#pragma unroll
    for (int d = 0; d < D; ++d) {
      const float a = fmaxf(fabsf(qf[d] - f.p.c[d]) - e, 0.0f);
      lb += a * a;
    }
    return lb * (1.0f - 0x1p-17f) > thr;
  }
};

template <typename T, int D, int K, typename H>
__device__ __forceinline__ void scan_leaf(const Rec<T, D>* __restrict__ recs, uint32_t st, uint32_t cnt,
                                          const T (&q)[D], T maxRadius2, T minDist, bool want, H& heap,
                                          const LeafFilter<T, D>& flt) {
  constexpr int kChunk = 4;
  for (uint32_t base = 0; base < cnt; base += kChunk) {
    unsigned mask = 0;
    if constexpr (std::is_same<T, float>::value) {
      // float: candidates as packed (dist2 bits, index) keys, one 64-bit
      // compare against min(head, radius key) -- the radius key is the
      // largest key of distance maxRadius2, so d <= maxRadius2 && key <
      // head is key < that minimum (a NaN radius accepts nothing: 0) --
      // and one 64-bit select per insertion (4-9 % faster than separate
      // radius and head tests on lidar scans)
      const uint64_t radKey = maxRadius2 == maxRadius2 ? ((uint64_t(__float_as_uint(maxRadius2)) << 32) | 0xffffffffull) : 0ull;
      const uint64_t thrKey =
          (!want || radKey == 0ull) ? 0ull : (heap.key[0] <= radKey ? heap.key[0] : radKey + 1ull);
      uint64_t kj[kChunk];
#pragma unroll
      for (int j = 0; j < kChunk; ++j) {
        kj[j] = ~0ull;
        if (base + j < cnt) {
          Rec<T, D> r;
          load_rec(recs, (int64_t)st + base + j, r);
          const float d = dist2_seq(q, r);
          kj[j] = TopK<float, K>::make(d, r.p.idx);
          mask |= (kj[j] < thrKey && d > minDist) ? (1u << j) : 0u;
        }
      }
      while (mask) {
        const int j = __ffs(mask) - 1;
        mask &= mask - 1;
        uint64_t v = kj[0];
#pragma unroll
        for (int m = 1; m < kChunk; ++m)
          if (j == m) v = kj[m];
        if (v < heap.key[0]) heap.insert_key(v);
      }
    } else {
      T dj[kChunk];
      int ij[kChunk];
      const float thr = flt.on() ? flt.threshold(heap.head(), maxRadius2) : 0.0f;
#pragma unroll
      for (int j = 0; j < kChunk; ++j) {
        dj[j] = Ar<T>::inf();
        ij[j] = -1;
        if (base + j < cnt && !(flt.on() && flt.rejects((int64_t)st + base + j, thr))) {
          Rec<T, D> r;
          load_rec(recs, (int64_t)st + base + j, r);
          dj[j] = dist2_seq(q, r);
          ij[j] = r.p.idx;
          const bool ok = want && dj[j] <= maxRadius2 && heap.accepts(dj[j], ij[j]) && dj[j] > minDist;
          mask |= ok ? (1u << j) : 0u;
        }
      }
      while (mask) {
        const int j = __ffs(mask) - 1;
        mask &= mask - 1;
        T dv = dj[0];
        int iv = ij[0];
#pragma unroll
        for (int m = 1; m < kChunk; ++m) {
          if (j == m) {
            dv = dj[m];
            iv = ij[m];
          }
        }
        if (heap.accepts(dv, iv)) heap.insert(dv, iv);
      }
    }
  }
}

// Ascending bitonic sort of B (a power of 2) keys held in registers: every
// index is known at compile time, so a compare-exchange is one 64-bit
// compare and two selects.
template <int B>
__device__ __forceinline__ void sort_keys(uint64_t (&s)[B]) {
#pragma unroll
  for (int k2 = 2; k2 <= B; k2 <<= 1) {
#pragma unroll
    for (int j = k2 >> 1; j > 0; j >>= 1) {
#pragma unroll
      for (int i = 0; i < B; ++i) {
        const int l = i ^ j;
        if (l > i) {
          const uint64_t a = s[i], b = s[l];
          const bool sw = ((i & k2) == 0) ? (a > b) : (a < b);
          s[i] = sw ? b : a;
          s[l] = sw ? a : b;
        }
      }
    }
  }
}

// A query's first leaf into its still empty top-k (float, k == K): the
// first B points' keys -- those the leaf scan would not take (outside the
// radius, a forbidden self match, or !want) as the empty key -- sorted by a
// network and placed in the list as they are, then the rest of the leaf by
// the normal scan. The list ends as if the points had been inserted one at
// a time (it holds the K smallest keys, and the scan's order never matters
// to that), for a fraction of the work: about 6 B log2(B)^2 / 4 integer
// instructions against about 6 K per insertion.
template <int D, int K>
__device__ __forceinline__ void scan_first_leaf(const Rec<float, D>* __restrict__ recs, uint32_t st, uint32_t cnt,
                                                const float (&q)[D], float maxRadius2, float minDist, bool want,
                                                TopK<float, K>& heap, const LeafFilter<float, D>& flt) {
  constexpr int B = K <= 10 ? 8 : 16;
  constexpr uint64_t kEmpty = uint64_t(0x7f800000u) << 32;
  const uint64_t radKey = maxRadius2 == maxRadius2 ? ((uint64_t(__float_as_uint(maxRadius2)) << 32) | 0xffffffffull) : 0ull;
  const uint64_t thrKey = (!want || radKey == 0ull) ? 0ull : (kEmpty <= radKey ? kEmpty : radKey + 1ull);
  uint64_t sk[B];
#pragma unroll
  for (int j = 0; j < B; ++j) {
    sk[j] = kEmpty;
    if ((uint32_t)j < cnt) {
      Rec<float, D> r;
      load_rec(recs, (int64_t)st + j, r);
      const float d = dist2_seq(q, r);
      const uint64_t key = TopK<float, K>::make(d, r.p.idx);
      if (key < thrKey && d > minDist) sk[j] = key;
    }
  }
  sort_keys(sk);
#pragma unroll
  for (int j = 0; j < K; ++j) heap.key[j] = (K - 1 - j < B) ? sk[(K - 1 - j) < B ? (K - 1 - j) : 0] : kEmpty;
  if (cnt > (uint32_t)B) scan_leaf<float, D, K>(recs, st + B, cnt - B, q, maxRadius2, minDist, want, heap, flt);
}

// A pushed far child as 32-bit words [rd | off[0..D-1] | node] (a T is one
// word for float, two for double) in 16-byte chunks: a push is one 128-bit
// local store per chunk (a lone trailing word is stored alone), a pop reads
// the first chunk, which holds rd, and the rest only if the child is
// visited.
template <typename T, int D>
struct StackRec {
  static constexpr int kTW = (int)(sizeof(T) / 4);
  static constexpr int kWords = kTW * (D + 1) + 1;
  static constexpr int kChunks = (kWords + 3) / 4;
  static constexpr int kNode = kTW * (D + 1);
  uint4 v[kChunks];
};

__device__ __forceinline__ void put_t(uint32_t* w, int i, float x) { w[i] = __float_as_uint(x); }
__device__ __forceinline__ void put_t(uint32_t* w, int i, double x) {
  w[i] = (uint32_t)__double2loint(x);
  w[i + 1] = (uint32_t)__double2hiint(x);
}
template <typename T>
__device__ __forceinline__ T get_t(const uint32_t* w, int i);
template <>
__device__ __forceinline__ float get_t<float>(const uint32_t* w, int i) {
  return __uint_as_float(w[i]);
}
template <>
__device__ __forceinline__ double get_t<double>(const uint32_t* w, int i) {
  return __hiloint2double((int)w[i + 1], (int)w[i]);
}

template <typename T, int D>
__device__ __forceinline__ void stack_push(StackRec<T, D>& e, T rd, const T (&off)[D], int cd, T newOff,
                                           uint32_t node) {
  using R = StackRec<T, D>;
  uint32_t w[R::kChunks * 4];
#pragma unroll
  for (int i = 0; i < R::kChunks * 4; ++i) w[i] = 0u;
  put_t(w, 0, rd);
#pragma unroll
  for (int d = 0; d < D; ++d) put_t(w, R::kTW * (1 + d), d == cd ? newOff : off[d]);
  w[R::kNode] = node;
#pragma unroll
  for (int c = 0; c < R::kChunks; ++c) {
    if (c == R::kChunks - 1 && R::kWords % 4 == 1)
      e.v[c].x = w[4 * c];
    else
      e.v[c] = make_uint4(w[4 * c], w[4 * c + 1], w[4 * c + 2], w[4 * c + 3]);
  }
}

template <typename T, int D>
__device__ __forceinline__ T stack_rd(const StackRec<T, D>& e) {
  const uint4 c0 = e.v[0];
  const uint32_t w[4] = {c0.x, c0.y, c0.z, c0.w};
  return get_t<T>(w, 0);
}

template <typename T, int D>
__device__ __forceinline__ uint32_t stack_take(const StackRec<T, D>& e, T (&off)[D]) {
  using R = StackRec<T, D>;
  uint32_t w[R::kChunks * 4];
#pragma unroll
  for (int c = 0; c < R::kChunks; ++c) {
    if (c == R::kChunks - 1 && R::kWords % 4 == 1) {
      w[4 * c] = e.v[c].x;
      w[4 * c + 1] = w[4 * c + 2] = w[4 * c + 3] = 0u;
    } else {
      const uint4 v = e.v[c];
      w[4 * c] = v.x;
      w[4 * c + 1] = v.y;
      w[4 * c + 2] = v.z;
      w[4 * c + 3] = v.w;
    }
  }
#pragma unroll
  for (int d = 0; d < D; ++d) off[d] = get_t<T>(w, R::kTW * (1 + d));
  return w[R::kNode];
}

// Where a query's traversal stack lives: a local array of N entries (the
// compiled kernels), or entries of a global-memory slab shared by the threads
// of a deep launch, thread g's entry sp at slab[sp * stride + g] so that the
// pushes of a warp at one depth are coalesced.
template <typename T, int D, int N>
struct LocalStack {
  StackRec<T, D> s[N];
  __device__ __forceinline__ StackRec<T, D>& operator[](int sp) { return s[sp]; }
};
template <typename T, int D>
struct SlabStack {
  StackRec<T, D>* base;
  int64_t stride;
  __device__ __forceinline__ StackRec<T, D>& operator[](int sp) { return base[(int64_t)sp * stride]; }
};

// One query (order position t) in the reference's visit order, structured
// descend / leaf / pop so the lanes of a warp run each phase together: all
// lanes descend until every lane stands on a leaf, then all scan their
// leaves, then all pop. `cap` entries of `stk` are available; the caller
// guarantees cap >= tree height. Adds the points examined to `touchedOut`.
// EXACT (epsilon 0, so maxError2 = 1 and rd * maxError2 = rd exactly): the
// push test rd <= maxRadius2 && rd <= head is one compare against
// min(maxRadius2, head), refreshed after each leaf; decisions are the same.
template <typename T, int D, int K, bool EXACT, typename S>
__device__ __forceinline__ void knn_query(const KnnLaunch& a, int64_t t, S& stk, int cap, uint32_t& touchedOut) {
  // the reference's self-match rule (nabo/kdtree_cpu.cpp:392-396): without
  // ALLOW_SELF_MATCH a point at distance <= epsilon is skipped; one compare
  // against -1 (everything passes) or epsilon
  const T minDist = a.allowSelf ? T(-1) : Ar<T>::eps();
  const Node<T>* __restrict__ nodes = static_cast<const Node<T>*>(a.nodes);
  const Rec<T, D>* __restrict__ recs = static_cast<const Rec<T, D>*>(a.recs);
  const T* __restrict__ query = static_cast<const T*>(a.query);
  uint32_t touched = 0;  // a query touches at most the cloud's n < 2^31 points
  int64_t qi;
  int k = a.k;
  uint32_t root = 0;
  int64_t outBase;
  if (a.runPrefix) {
    const int64_t g = a.runPrefix[a.runBegin] + t;
    int lo = a.runBegin, hi = a.runEnd - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (a.runPrefix[mid] <= g)
        lo = mid;
      else
        hi = mid - 1;
    }
    const int c = a.runCloud[lo];
    qi = (int64_t)a.order[a.bQueryOffset[c] + (g - a.runPrefix[lo])];
    k = a.bK[c];
    root = (uint32_t)a.bNodeOffset[c];
    outBase = a.bOutOffset[c] + (qi - a.bQueryOffset[c]) * (int64_t)k;
  } else {
    qi = a.order ? (int64_t)a.order[t] : t;
    outBase = qi * (int64_t)a.k;
    if (a.bQueryOffset) {
      const int c = cloud_of(a.bQueryOffset, a.bClouds, qi);
      k = a.bK[c];
      root = (uint32_t)a.bNodeOffset[c];
      outBase = a.bOutOffset[c] + (qi - a.bQueryOffset[c]) * (int64_t)k;
    }
  }
  T q[D];
#pragma unroll
  for (int d = 0; d < D; ++d) q[d] = d < a.dim ? query[qi * a.qStride + d] : T(0);
  T maxRadius2 = (T)a.maxRadius2;
  // a bounded search (per-query radius) that misses may run once more
  // without its bound (the learned-radius form's fallback)
  bool mayFall = false;
  if (a.maxRadii) {
    const T r = static_cast<const T*>(a.maxRadii)[qi];
    maxRadius2 = Ar<T>::mul(r, r);
    mayFall = a.fallbackRadius >= 0.0 && (double)r < a.fallbackRadius;
  }
  const T maxError2 = (T)a.maxError2;
  typename SearchHeap<T, K>::type heap;
  heap.init(k);
  LeafFilter<T, D> flt;
  flt.init(a.recs32, a.coordMax, q);
  T off[D];
  for (;;) {  // the search, and at most once more without the bound
#pragma unroll
    for (int d = 0; d < D; ++d) off[d] = T(0);
    int sp = 0;
    uint32_t node = root;
    T rd = T(0);
    bool fresh = true;  // no leaf scanned yet: the top-k is empty
    for (;;) {
      // descend to a leaf, pushing far children
      // min(maxRadius2, head), where a NaN radius (which passes nothing) wins
      const T bound = EXACT ? (heap.head() < maxRadius2 ? heap.head() : maxRadius2) : T(0);
      Node<T> nd = load_node(nodes, node);
      while (!node_is_leaf(nd.meta)) {
        const int cd = (int)node_dim(nd.meta);
        const T newOff = Ar<T>::sub(pick(q, cd), nd.cut);
        const T oldOff = pick(off, cd);
        const T rdFar = Ar<T>::add(rd, Ar<T>::add(-Ar<T>::mul(oldOff, oldOff), Ar<T>::mul(newOff, newOff)));
        const uint32_t right = node_payload(nd.meta);
        const uint32_t nearN = newOff > T(0) ? right : node + 1;
        const uint32_t farN = newOff > T(0) ? node + 1 : right;
        const bool far = EXACT ? rdFar <= bound
                               : (rdFar <= maxRadius2 && Ar<T>::mul(rdFar, maxError2) <= heap.head());
        // sp <= tree height <= cap (checked by the caller); the test only
        // makes the bound explicit
        if (far && sp < cap) stack_push(stk[sp++], rdFar, off, cd, newOff, farN);
        node = nearN;
        nd = load_node(nodes, node);
      }
      // leaf
      const uint32_t cnt = node_payload(nd.meta);
      if constexpr (std::is_same<T, float>::value && K >= 8) {
        if (fresh && k == K)
          scan_first_leaf<D, K>(recs, node_start(nd), cnt, q, maxRadius2, minDist, true, heap, flt);
        else
          scan_leaf<T, D, K>(recs, node_start(nd), cnt, q, maxRadius2, minDist, true, heap, flt);
      } else {
        scan_leaf<T, D, K>(recs, node_start(nd), cnt, q, maxRadius2, minDist, true, heap, flt);
      }
      fresh = false;
      touched += cnt;
      // pop the next far child that can still hold a better neighbour
      bool more = false;
      while (sp > 0) {
        --sp;
        const T e = stack_rd(stk[sp]);
        if ((EXACT ? e : Ar<T>::mul(e, maxError2)) <= heap.head()) {
          rd = e;
          node = stack_take(stk[sp], off);
          more = true;
          break;
        }
      }
      if (!more) break;
    }
    if (!mayFall || heap.count(k) == k) break;
    mayFall = false;
    maxRadius2 = (T)a.maxRadius2;
    heap.init(k);
    if (a.fallbacks) atomicAdd(a.fallbacks, 1);
  }
  const int f = heap.store(k, a.outIdx + outBase, static_cast<T*>(a.outD2) + outBase);
  if (a.found) a.found[qi] = f;
  touchedOut += touched;
}

// The warp's TOUCH_STATISTICS counts summed into a.touched (every lane of
// the warp calls this).
__device__ __forceinline__ void add_touched(const KnnLaunch& a, uint32_t touched) {
  if (a.stats) {
    unsigned long long sum = touched;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
    if ((threadIdx.x & 31) == 0 && sum) atomicAdd(a.touched, sum);
  }
}

// One thread per query, stack of STACK entries in local memory.
template <typename T, int D, int K, int STACK, bool EXACT>
__device__ __forceinline__ void knn_kdtree_body(const KnnLaunch& a) {
  if (a.tallGate && *a.tallGate > a.tallGateLimit) return;  // the deep kernel searches (uniform)
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  uint32_t touched = 0;
  if (t < a.nq && (!a.nqDevice || t < (int64_t)*a.nqDevice)) {
    LocalStack<T, D, STACK> stk;
    knn_query<T, D, K, EXACT>(a, t, stk, STACK, touched);
  }
  add_touched(a, touched);
}

template <typename T, int D, int K, int STACK, bool EXACT>
__global__ void __launch_bounds__(128) k_knn_kdtree(KnnLaunch a) {
  knn_kdtree_body<T, D, K, STACK, EXACT>(a);
}

// Double searches with a long top-k hold ~100 registers of heap alone;
// limited to 128 registers a thread, 4 blocks share an SM, and the FP64 pipe
// gets the extra warps it needs to hide its latency (12 % faster on 8-D
// clouds, k = 32).
template <typename T, int D, int K, int STACK, bool EXACT>
__global__ void __launch_bounds__(128, 4) k_knn_kdtree_lean(KnnLaunch a) {
  knn_kdtree_body<T, D, K, STACK, EXACT>(a);
}

// Trees of any height: the stacks in a.slab, cap = a.stackCap entries per
// query (or the tree height read from *a.stackHeightDev, plus one, for
// batches whose heights the host does not know). As many threads as the
// slab holds stacks search (the others idle), each taking every active-th
// query. A slab too small for one stack searches nothing and sets
// *a.deepFail to -1.
template <typename T, int D, int K, bool EXACT>
__global__ void __launch_bounds__(128) k_knn_kdtree_deep(KnnLaunch a) {
  if (a.tallGate && *a.tallGate <= a.tallGateLimit) return;  // the local-stack kernel searches (uniform)
  const int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t threads = (int64_t)gridDim.x * blockDim.x;
  const int cap = a.stackCap > 0 ? a.stackCap : (a.stackHeightDev ? *a.stackHeightDev + 1 : 0);
  int64_t active = cap > 0 ? a.slabBytes / ((int64_t)sizeof(StackRec<T, D>) * cap) : 0;
  if (active > threads) active = threads;
  if (active <= 0 && a.nq > 0 && g == 0 && a.deepFail) *a.deepFail = -1;
  uint32_t touched = 0;
  if (g < active) {
    SlabStack<T, D> stk{static_cast<StackRec<T, D>*>(a.slab) + g, active};
    for (int64_t t = g; t < a.nq; t += active) {
      if (a.nqDevice && t >= (int64_t)*a.nqDevice) continue;
      knn_query<T, D, K, EXACT>(a, t, stk, cap, touched);
    }
  }
  add_touched(a, touched);
}

// Bytes of one query's stack in a deep launch's slab, for `cap` entries.
template <typename T, int D>
constexpr size_t deep_stack_bytes(int cap) {
  return sizeof(StackRec<T, D>) * (size_t)cap;
}

template <typename T, int D, int K, int STACK, bool EXACT>
void launch_kdtree_as(int grid, int block, cudaStream_t stream, const KnnLaunch& L) {
  if constexpr (sizeof(T) == 8 && K >= 16)
    k_knn_kdtree_lean<T, D, K, STACK, EXACT><<<grid, block, 0, stream>>>(L);
  else
    k_knn_kdtree<T, D, K, STACK, EXACT><<<grid, block, 0, stream>>>(L);
}

template <typename T, int D, int K, int STACK>
void launch_kdtree(int grid, int block, cudaStream_t stream, const KnnLaunch& L) {
  if (L.maxError2 == 1.0)
    launch_kdtree_as<T, D, K, STACK, true>(grid, block, stream, L);
  else
    launch_kdtree_as<T, D, K, STACK, false>(grid, block, stream, L);
}

template <typename T, int D, int K>
void launch_kdtree_deep(int grid, cudaStream_t stream, const KnnLaunch& L) {
  if (L.maxError2 == 1.0)
    k_knn_kdtree_deep<T, D, K, true><<<grid, 128, 0, stream>>>(L);
  else
    k_knn_kdtree_deep<T, D, K, false><<<grid, 128, 0, stream>>>(L);
}

// Warp-packet traversal for exact search (epsilon = 0).
//
// The 32 queries of a warp (neighbours along the Morton order) walk the
// tree together: one node sequence for the warp, chosen so that at each
// inner node the child that most lanes see as their near side comes first;
// every lane keeps its own offsets, box distance and top-k, and decides for
// itself whether a node can hold a better neighbour. A node is skipped only
// when no lane wants it, so every lane still examines every point that can
// enter its result. Leaf records are read with warp-uniform addresses
// (broadcast loads) and candidates are inserted after the whole leaf has
// been filtered, so the warp pays for the largest number of insertions of
// any one lane rather than for every point where some lane inserts.
//
// The box distance of a cell is the sequential sum over d of off[d]^2,
// rounded exactly as the point distance is. Rounding is monotone, so a
// point inside the cell is never closer than its cell's bound, and the
// pruning test rd <= head never drops an acceptable point: the result is
// the exact k smallest (dist2, index) pairs -- the brute-force answer.
template <typename T, int D>
__device__ __forceinline__ T box_dist2(const T (&off)[D]) {
  T rd = Ar<T>::mul(off[0], off[0]);
#pragma unroll
  for (int d = 1; d < D; ++d) rd = Ar<T>::add(rd, Ar<T>::mul(off[d], off[d]));
  return rd;
}

template <typename T, int D, int K, int STACK>
__global__ void __launch_bounds__(128) k_knn_kdtree_packet(KnnLaunch a) {
  constexpr unsigned kAll = 0xffffffffu;
  // the reference's self-match rule (nabo/kdtree_cpu.cpp:392-396): without
  // ALLOW_SELF_MATCH a point at distance <= epsilon is skipped; one compare
  // against -1 (everything passes) or epsilon
  const T minDist = a.allowSelf ? T(-1) : Ar<T>::eps();
  const Node<T>* __restrict__ nodes = static_cast<const Node<T>*>(a.nodes);
  const Rec<T, D>* __restrict__ recs = static_cast<const Rec<T, D>*>(a.recs);
  const T* __restrict__ query = static_cast<const T*>(a.query);
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
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
  if (!active) maxRadius2 = -Ar<T>::inf();  // wants nothing
  TopK<T, K> heap;
  heap.init(a.k);
  LeafFilter<T, D> flt;
  flt.init(nullptr, nullptr, q);
  T off[D];
#pragma unroll
  for (int d = 0; d < D; ++d) off[d] = T(0);
  uint32_t sNode[STACK];
  T sOff[STACK][D];
  int sp = 0;
  uint32_t node = 0;
  for (;;) {
    const T rd = box_dist2(off);
    const bool want = rd <= maxRadius2 && rd <= heap.head();
    if (__any_sync(kAll, want)) {
      const Node<T> nd = load_node(nodes, node);
      if (!node_is_leaf(nd.meta)) {
        const int cd = (int)node_dim(nd.meta);
        const T newOff = Ar<T>::sub(pick(q, cd), nd.cut);
        const bool nearRight = newOff > T(0);
        const int votesRight = __popc(__ballot_sync(kAll, want && nearRight));
        const int votes = __popc(__ballot_sync(kAll, want));
        const bool firstRight = 2 * votesRight > votes;
        const uint32_t right = node_payload(nd.meta);
        const uint32_t first = firstRight ? right : node + 1;
        const uint32_t second = firstRight ? node + 1 : right;
        // the second child is this lane's far side iff the first is its near side
        const bool secondFar = nearRight == firstRight;
        T offS[D];
#pragma unroll
        for (int d = 0; d < D; ++d) offS[d] = (d == cd && secondFar) ? newOff : off[d];
        const T rdS = box_dist2(offS);
        const bool wantS = want && rdS <= maxRadius2 && rdS <= heap.head();
        if (__any_sync(kAll, wantS) && sp < STACK) {
          sNode[sp] = second;
#pragma unroll
          for (int d = 0; d < D; ++d) sOff[sp][d] = offS[d];
          ++sp;
        }
#pragma unroll
        for (int d = 0; d < D; ++d)  // the first child is this lane's far side
          if (d == cd && !secondFar) off[d] = newOff;
        node = first;
        continue;
      }
      scan_leaf<T, D, K>(recs, node_start(nd), node_payload(nd.meta), q, maxRadius2, minDist, want, heap, flt);
    }
    if (sp == 0) break;
    --sp;
    node = sNode[sp];
#pragma unroll
    for (int d = 0; d < D; ++d) off[d] = sOff[sp][d];
  }
  if (active) {
    const int f = heap.store(a.k, a.outIdx + qi * a.k, static_cast<T*>(a.outD2) + qi * a.k);
    if (a.found) a.found[qi] = f;
  }
}

// Brute force (nabo/brute_force_cpu.cpp:63-103): every query against every
// point. The points are staged through shared memory in tiles of 24 KB; a
// thread owns QT queries (blockDim.x apart) and their top-k, so each record
// read from shared memory (a broadcast: every lane reads the same one) feeds
// QT distances. The distance is the reference's separately rounded
// sequential sum. Records are taken J at a time: the J x QT distances are
// computed, each query's smallest is compared with one float threshold,
// min(head, maxRadius^2) (NaN radius: NaN, which passes nothing), and only
// when some distance is at or below its threshold -- rare once the heaps
// are full -- do the group's points take the exact test, the reference's
// radius and self-match rules and the (dist2, index) order against the head
// (nabo/kdtree_cpu.cpp:392-396 with the lower index kept on ties). The
// result, the k smallest pairs, does not depend on the order points are
// offered in.
//
// With gridDim.y > 1 the points are split into chunks of `chunk` (a
// multiple of the tile): block row y offers points [y*chunk, (y+1)*chunk) and
// writes its k best to a.outIdx / a.outD2 + y*partStride, and
// k_bf_merge combines the rows (for searches with too few queries to give
// every SM several blocks).
template <typename T>
__device__ __forceinline__ T bf_threshold(T head, T maxRadius2) {
  return head < maxRadius2 ? head : maxRadius2;
}
__device__ __forceinline__ float fmin_t(float a, float b) { return fminf(a, b); }
__device__ __forceinline__ double fmin_t(double a, double b) { return fmin(a, b); }

// Float brute force filters each group of J points before the reference's
// distance: a = |p|^2 - 2 q.p, D fused multiply-adds per pair from |p|^2
// (computed once per point as the tile is staged, kept in the record's index
// slot, the index itself beside the tile) and -2q. With e the reference's
// distance (separately rounded squares, nabo/kdtree_cpu.cpp:383-391), a
// point it could accept has e <= thr, and then
//   a <= thr - |q|^2 + g (thr + 3 P + 2 |q|^2)
// (the dot product's rounding, bounded with 2|q||p| <= |q|^2 + |p|^2, plus
// e's own rounding and |q|^2's) with g = (D + 2) u / (1 - (D + 2) u),
// u = 2^-24, and P the tile's largest |p|^2; the test's bound
// thr - |q|^2 + 2^-17 (thr + 2 P + 2 |q|^2) exceeds that (g (thr + 3 P +
// 2 |q|^2)) over 4 times for D <= 16 and covers its own rounding, so it
// never drops a point that the exact pass would take. A group that passes
// is computed again exactly, as before.
template <int D>
struct BfFilter {
  float m2q[D];  // -2 q
  float qn;      // |q|^2
  float thrA;    // threshold on a
  __device__ __forceinline__ void init(const float (&q)[D]) {
    qn = 0.0f;
#pragma unroll
    for (int d = 0; d < D; ++d) {
      m2q[d] = -2.0f * q[d];
      qn = fmaf(q[d], q[d], qn);
    }
  }
  // A NaN threshold (an idle slot, or a NaN radius) passes nothing. Where
  // |p|^2, |q|^2 or the bound overflow, thrA is inf or NaN and the test
  // below (!(a > thrA)) passes every group to the exact pass.
  __device__ __forceinline__ void set(float thr, float pmax) {
    thrA = thr != thr ? -__int_as_float(0x7f800000) : (thr - qn) + 0x1p-17f * (thr + 2.0f * pmax + 2.0f * qn);
  }
  __device__ __forceinline__ float eval(const Rec<float, D>& r) const {
    float a = __int_as_float(r.p.idx);
#pragma unroll
    for (int d = 0; d < D; ++d) a = fmaf(m2q[d], r.p.c[d], a);
    return a;
  }
};

template <typename T, int D, int K, int QT, int J>
__global__ void __launch_bounds__(128) k_knn_bruteforce(KnnLaunch a, int64_t chunk, int64_t partStride) {
  constexpr bool kFilter = sizeof(T) == 4;
  const T minDist = a.allowSelf ? T(-1) : Ar<T>::eps();
  // a multiple of J, so that a group never reads past the tile
  constexpr int kTile = (int)((24 * 1024) / sizeof(Rec<T, D>)) / J * J;
  __shared__ Rec<T, D> tile[kTile];
  __shared__ int32_t tileIdx[kFilter ? kTile : 1];  // filter: the points' indices
  __shared__ float warpMax[4];                       // filter: largest |p|^2 per warp
  const Rec<T, D>* __restrict__ recs = static_cast<const Rec<T, D>*>(a.recs);
  const T* __restrict__ query = static_cast<const T*>(a.query);
  const int64_t base0 = (int64_t)blockIdx.x * blockDim.x * QT + threadIdx.x;
  T q[QT][D];
  T maxRadius2[QT];
  T thr[QT];
  int64_t qi[QT];
  bool active[QT];
  TopK<T, K> heap[QT];
  BfFilter<D> flt[kFilter ? QT : 1];
#pragma unroll
  for (int u = 0; u < QT; ++u) {
    const int64_t t = base0 + (int64_t)u * blockDim.x;
    active[u] = t < a.nq;
    qi[u] = active[u] ? (a.order ? (int64_t)a.order[t] : t) : 0;
#pragma unroll
    for (int d = 0; d < D; ++d) q[u][d] = (active[u] && d < a.dim) ? query[qi[u] * a.qStride + d] : T(0);
    maxRadius2[u] = (T)a.maxRadius2;
    if (a.maxRadii && active[u]) {
      const T r = static_cast<const T*>(a.maxRadii)[qi[u]];
      maxRadius2[u] = Ar<T>::mul(r, r);
    }
    // an idle slot wants nothing (a NaN threshold passes no point)
    if (!active[u]) maxRadius2[u] = __builtin_nan("");
    heap[u].init(a.k);
    thr[u] = bf_threshold(heap[u].head(), maxRadius2[u]);
    if constexpr (kFilter) flt[u].init(reinterpret_cast<const float(&)[D]>(q[u]));
  }
  const int64_t first = (int64_t)blockIdx.y * chunk;
  const int64_t last = first + chunk < a.n ? first + chunk : a.n;
  for (int64_t base = first; base < last; base += kTile) {
    const int m = (int)((last - base) < kTile ? (last - base) : kTile);
    __syncthreads();
    if constexpr (kFilter) {
      float pm = 0.0f;
      for (int j = threadIdx.x; j < m; j += blockDim.x) {
        Rec<T, D> r;
        load_rec(recs, base + j, r);
        float pn = 0.0f;
#pragma unroll
        for (int d = 0; d < D; ++d) pn = fmaf(r.p.c[d], r.p.c[d], pn);
        tileIdx[j] = r.p.idx;
        r.p.idx = __float_as_int(pn);
        tile[j] = r;
        pm = fmaxf(pm, pn);
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) pm = fmaxf(pm, __shfl_xor_sync(0xffffffffu, pm, o));
      if ((threadIdx.x & 31) == 0) warpMax[threadIdx.x >> 5] = pm;
    } else {
      const uint4* src = reinterpret_cast<const uint4*>(recs + base);
      uint4* dst = reinterpret_cast<uint4*>(tile);
      const int words = m * RecSize<T, D>::chunks;
      for (int w = threadIdx.x; w < words; w += blockDim.x) dst[w] = __ldg(src + w);
    }
    {
      // the last group's missing points: NaN coordinates (and |p|^2), whose
      // distance passes no threshold and lowers no minimum (a group's first
      // point is always a real one)
      const int padEnd = (m + J - 1) / J * J;
      for (int j = m + (int)threadIdx.x; j < padEnd; j += blockDim.x) {
        Rec<T, D> r;
#pragma unroll
        for (int d = 0; d < D; ++d) r.p.c[d] = __builtin_nan("");
        r.p.idx = kFilter ? __float_as_int(__builtin_nanf("")) : -1;
        tile[j] = r;
      }
    }
    __syncthreads();
    if constexpr (kFilter) {
      const float pmax = fmaxf(fmaxf(warpMax[0], warpMax[1]), fmaxf(warpMax[2], warpMax[3]));
#pragma unroll
      for (int u = 0; u < QT; ++u) flt[u].set((float)thr[u], pmax);
      for (int j0 = 0; j0 < m; j0 += J) {
        float amin[QT];
#pragma unroll
        for (int jj = 0; jj < J; ++jj) {
          const Rec<T, D> r = tile[j0 + jj];
#pragma unroll
          for (int u = 0; u < QT; ++u) {
            const float av = flt[u].eval(reinterpret_cast<const Rec<float, D>&>(r));
            amin[u] = jj == 0 ? av : fminf(amin[u], av);
          }
        }
        bool any = false;
#pragma unroll
        for (int u = 0; u < QT; ++u) any = any || !(amin[u] > flt[u].thrA);
        if (any) {  // rare once the heaps are full: the group exactly
#pragma unroll
          for (int jj = 0; jj < J; ++jj) {
            if (j0 + jj < m) {
              const Rec<T, D> r = tile[j0 + jj];
              const int idx = tileIdx[j0 + jj];
#pragma unroll
              for (int u = 0; u < QT; ++u) {
                const T d = dist2_seq(q[u], r);
                if (d <= thr[u] && d <= maxRadius2[u] && heap[u].accepts(d, idx) && d > minDist) {
                  heap[u].insert(d, idx);
                  thr[u] = bf_threshold(heap[u].head(), maxRadius2[u]);
                  flt[u].set((float)thr[u], pmax);
                }
              }
            }
          }
        }
      }
    } else {
      for (int j0 = 0; j0 < m; j0 += J) {
        // each query's smallest distance of the group (fmin ignores the NaN
        // padding; the group's first point is a real one)
        T dmin[QT];
#pragma unroll
        for (int jj = 0; jj < J; ++jj) {
          const Rec<T, D> r = tile[j0 + jj];
#pragma unroll
          for (int u = 0; u < QT; ++u) {
            const T d = dist2_seq(q[u], r);
            dmin[u] = jj == 0 ? d : fmin_t(dmin[u], d);
          }
        }
        bool any = false;
#pragma unroll
        for (int u = 0; u < QT; ++u) any = any || dmin[u] <= thr[u];
        if (any) {  // rare once the heaps are full: the group again, exactly
#pragma unroll
          for (int jj = 0; jj < J; ++jj) {
            if (j0 + jj < m) {
              const Rec<T, D> r = tile[j0 + jj];
#pragma unroll
              for (int u = 0; u < QT; ++u) {
                const T d = dist2_seq(q[u], r);
                if (d <= thr[u] && d <= maxRadius2[u] && heap[u].accepts(d, r.p.idx) && d > minDist) {
                  heap[u].insert(d, r.p.idx);
                  thr[u] = bf_threshold(heap[u].head(), maxRadius2[u]);
                }
              }
            }
          }
        }
      }
    }
  }
  const int64_t part = (int64_t)blockIdx.y * partStride;
#pragma unroll
  for (int u = 0; u < QT; ++u) {
    if (active[u]) {
      const int f = heap[u].store(a.k, a.outIdx + part + qi[u] * a.k, static_cast<T*>(a.outD2) + part + qi[u] * a.k);
      if (a.found) a.found[qi[u]] = f;
    }
  }
}

// The k best of `parts` partial results per query (each k entries, ascending,
// unfound slots index -1), written as the search's result.
template <typename T, int K>
__global__ void k_bf_merge(const int32_t* __restrict__ pIdx, const T* __restrict__ pD2, int parts, int64_t partStride,
                           int64_t nq, int k, int32_t* outIdx, T* outD2, int32_t* found) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= nq) return;
  TopK<T, K> heap;
  heap.init(k);
  for (int p = 0; p < parts; ++p) {
    const int64_t o = p * partStride + i * k;
    for (int j = 0; j < k; ++j) {
      const int32_t idx = pIdx[o + j];
      if (idx < 0) break;
      const T d = pD2[o + j];
      if (heap.accepts(d, idx)) heap.insert(d, idx);
    }
  }
  const int f = heap.store(k, outIdx + i * k, outD2 + i * k);
  if (found) found[i] = f;
}

// Shape of the brute force: QT queries per thread (more share each
// shared-memory read, fewer keep long top-k lists in registers) and J
// records per threshold test.
// Float, with the |p|^2 - 2 q.p filter, 100k x 100k 3-D points (kernel ms,
// k = 5 / k = 10): QT x J = 1 x 4 3.50 / 4.79, 1 x 8 3.51 / 5.06, 1 x 12
// 3.76 / 5.95, 2 x 4 3.92 / 6.63, 3 x 4 4.54 / 8.17, 1 x 16 4.59 / 6.58,
// 2 x 8 4.80 / 8.19, 4 x 4 5.89 / 10.97, 4 x 8 8.76 / 18.12.
// Before the filter (separately rounded distances for every pair, k = 5):
// 2 x 4 5.17, 2 x 8 5.72, 1 x 8 6.33, 4 x 4 6.83, 1 x 4 6.90, 4 x 8 7.88,
// 8 x 2 8.49; double, which keeps that kernel, uses 1 x 4.
template <typename T, int K>
struct BfShape {
  static constexpr int QT = 1;
  static constexpr int J = 4;
};

}  // namespace nabo_gb300
