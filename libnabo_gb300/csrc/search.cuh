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
// Top-k: K (dist2, index) pairs in registers, kept in descending order so
// the head (largest) is slot 0; slots >= k hold -inf so one instantiation
// serves every k <= K. Pairs are ordered by (dist2, index): among equal
// distances the lower index is kept, which makes the result independent of
// visit order (the reference's IndexHeapBruteForceVector keeps the first
// visited, nabo/index_heap.h:322-334).
#pragma once

#include "common.cuh"

namespace nabo_gb300 {

template <typename T>
__device__ __forceinline__ bool pair_greater(T da, int ia, T db, int ib) {
  return da > db || (da == db && ia > ib);
}

template <typename T, int K>
struct TopK {
  T d[K];
  int i[K];
  __device__ __forceinline__ void init(int k) {
#pragma unroll
    for (int j = 0; j < K; ++j) {
      d[j] = j < k ? Ar<T>::inf() : -Ar<T>::inf();
      i[j] = -1;
    }
  }
  __device__ __forceinline__ T head() const { return d[0]; }
  __device__ __forceinline__ bool accepts(T dist, int idx) const { return pair_greater(d[0], i[0], dist, idx); }
  // Drops the head and inserts (dist, idx); requires accepts(dist, idx).
  // Slot j takes its successor while that is still larger than the new
  // pair, then the new pair, then keeps its own value.
  __device__ __forceinline__ void insert(T dist, int idx) {
#pragma unroll
    for (int j = 0; j + 1 < K; ++j) {
      if (pair_greater(d[j + 1], i[j + 1], dist, idx)) {
        d[j] = d[j + 1];
        i[j] = i[j + 1];
      } else if (pair_greater(d[j], i[j], dist, idx)) {
        d[j] = dist;
        i[j] = idx;
      }
    }
    if (pair_greater(d[K - 1], i[K - 1], dist, idx)) {
      d[K - 1] = dist;
      i[K - 1] = idx;
    }
  }
  // Writes the k entries in ascending order; returns how many are valid.
  __device__ __forceinline__ int store(int k, int32_t* __restrict__ oi, T* __restrict__ od) const {
    int found = 0;
#pragma unroll
    for (int j = 0; j < K; ++j) {
      if (j < k) {
        oi[k - 1 - j] = i[j];
        od[k - 1 - j] = d[j];
        found += i[j] >= 0 ? 1 : 0;
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

// Query ordering for the kd-tree: each query's cell is the leaf it reaches
// by always taking its near side (new_off > 0 -> right, as the search
// does). Leaves are numbered in pre-order, so queries sorted by leaf are
// grouped at the scale of the data's own buckets.
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
  rank[i] = atomicAdd(hist + node, 1u);
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
  // batches of clouds (all null for one cloud): queries of cloud c are
  // [bQueryOffset[c], bQueryOffset[c+1]), its tree starts at node
  // bNodeOffset[c], it wants bK[c] neighbours written from bOutOffset[c]
  const int64_t* bQueryOffset;
  const int64_t* bNodeOffset;
  const int32_t* bK;
  const int64_t* bOutOffset;
  int bClouds;
};

// Leaf scan shared by the kernels: the bucket's records are read in chunks
// of 8 (independent loads in flight), candidates that beat the current head
// are collected in a bit mask and inserted afterwards. The order of
// insertion inside a leaf does not change the heap after the leaf (the k
// smallest pairs of the union), so this matches the reference's point-by-
// point loop (nabo/kdtree_cpu.cpp:378-398); the warp pays for the largest
// number of insertions of any lane instead of for every point where some
// lane inserts.
template <typename T, int D, int K>
__device__ __forceinline__ void scan_leaf(const Rec<T, D>* __restrict__ recs, uint32_t st, uint32_t cnt,
                                          const T (&q)[D], T maxRadius2, bool selfOk, bool want, TopK<T, K>& heap) {
  constexpr int kChunk = 8;
  for (uint32_t base = 0; base < cnt; base += kChunk) {
    T dj[kChunk];
    int ij[kChunk];
    unsigned mask = 0;
#pragma unroll
    for (int j = 0; j < kChunk; ++j) {
      dj[j] = Ar<T>::inf();
      ij[j] = -1;
      if (base + j < cnt) {
        Rec<T, D> r;
        load_rec(recs, (int64_t)st + base + j, r);
        dj[j] = dist2_seq(q, r);
        ij[j] = r.p.idx;
        const bool ok = want && dj[j] <= maxRadius2 && heap.accepts(dj[j], ij[j]) &&
                        (selfOk || dj[j] > Ar<T>::eps());
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

// Reference-order traversal, structured descend / leaf / pop so the lanes
// of a warp run each phase together: all lanes descend until every lane
// stands on a leaf, then all scan their leaves, then all pop.
template <typename T, int D, int K, int STACK>
__global__ void __launch_bounds__(128) k_knn_kdtree(KnnLaunch a) {
  const bool selfOk = a.allowSelf != 0;
  const Node<T>* __restrict__ nodes = static_cast<const Node<T>*>(a.nodes);
  const Rec<T, D>* __restrict__ recs = static_cast<const Rec<T, D>*>(a.recs);
  const T* __restrict__ query = static_cast<const T*>(a.query);
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  unsigned long long touched = 0;
  if (t < a.nq && (!a.nqDevice || t < (int64_t)*a.nqDevice)) {
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
    if (a.maxRadii) {
      const T r = static_cast<const T*>(a.maxRadii)[qi];
      maxRadius2 = Ar<T>::mul(r, r);
    }
    const T maxError2 = (T)a.maxError2;
    TopK<T, K> heap;
    heap.init(k);
    T off[D];
#pragma unroll
    for (int d = 0; d < D; ++d) off[d] = T(0);
    uint32_t sNode[STACK];
    T sRd[STACK];
    T sOff[STACK][D];
    int sp = 0;
    uint32_t node = root;
    T rd = T(0);
    for (;;) {
      // descend to a leaf, pushing far children
      Node<T> nd = load_node(nodes, node);
      while (!node_is_leaf(nd.meta)) {
        const int cd = (int)node_dim(nd.meta);
        const T newOff = Ar<T>::sub(pick(q, cd), nd.cut);
        const T oldOff = pick(off, cd);
        const T rdFar = Ar<T>::add(rd, Ar<T>::add(-Ar<T>::mul(oldOff, oldOff), Ar<T>::mul(newOff, newOff)));
        const uint32_t right = node_payload(nd.meta);
        const uint32_t nearN = newOff > T(0) ? right : node + 1;
        const uint32_t farN = newOff > T(0) ? node + 1 : right;
        // sp <= tree height <= STACK (checked on the host); the test only
        // makes the bound explicit
        if (rdFar <= maxRadius2 && Ar<T>::mul(rdFar, maxError2) <= heap.head() && sp < STACK) {
          sNode[sp] = farN;
          sRd[sp] = rdFar;
#pragma unroll
          for (int d = 0; d < D; ++d) sOff[sp][d] = d == cd ? newOff : off[d];
          ++sp;
        }
        node = nearN;
        nd = load_node(nodes, node);
      }
      // leaf
      const uint32_t cnt = node_payload(nd.meta);
      scan_leaf<T, D, K>(recs, node_start(nd), cnt, q, maxRadius2, selfOk, true, heap);
      touched += cnt;
      // pop the next far child that can still hold a better neighbour
      bool more = false;
      while (sp > 0) {
        --sp;
        const T e = sRd[sp];
        if (Ar<T>::mul(e, maxError2) <= heap.head()) {
          rd = e;
          node = sNode[sp];
#pragma unroll
          for (int d = 0; d < D; ++d) off[d] = sOff[sp][d];
          more = true;
          break;
        }
      }
      if (!more) break;
    }
    const int f = heap.store(k, a.outIdx + outBase, static_cast<T*>(a.outD2) + outBase);
    if (a.found) a.found[qi] = f;
  }
  if (a.stats) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) touched += __shfl_xor_sync(0xffffffffu, touched, o);
    if ((threadIdx.x & 31) == 0 && touched) atomicAdd(a.touched, touched);
  }
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
  const bool selfOk = a.allowSelf != 0;
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
      scan_leaf<T, D, K>(recs, node_start(nd), node_payload(nd.meta), q, maxRadius2, selfOk, want, heap);
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
// point, points staged through shared memory in tiles; each thread owns one
// query and its top-k. Points are offered in index order.
template <typename T, int D, int K>
__global__ void __launch_bounds__(128) k_knn_bruteforce(KnnLaunch a) {
  const bool selfOk = a.allowSelf != 0;
  constexpr int kTile = (int)((24 * 1024) / sizeof(Rec<T, D>));
  __shared__ Rec<T, D> tile[kTile];
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
  TopK<T, K> heap;
  heap.init(a.k);
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
    if (active) {
      for (int j = 0; j < m; ++j) {
        const Rec<T, D>& r = tile[j];
        const T dist = dist2_seq(q, r);
        if (dist <= maxRadius2 && heap.accepts(dist, r.p.idx) && (selfOk || dist > Ar<T>::eps()))
          heap.insert(dist, r.p.idx);
      }
    }
  }
  if (active) {
    const int f = heap.store(a.k, a.outIdx + qi * a.k, static_cast<T*>(a.outD2) + qi * a.k);
    if (a.found) a.found[qi] = f;
  }
}

}  // namespace nabo_gb300
