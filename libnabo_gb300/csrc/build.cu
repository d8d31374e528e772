// build.cu -- kd-tree construction on the device.
//
// Produces exactly the tree of the reference constructor
// KDTreeUnbalancedPtInLeavesImplicitBoundsStackOpt (nabo/kdtree_cpu.cpp:
// 109-272): sliding-midpoint split on the widest box dimension, cut clamped
// to the points' range, the two-pass in-place partition, the same leftCount
// rules, pre-order node numbering with the left child at n+1, and leaf
// buckets in the same point order. Points are stored in leaf order as
// 16-byte-aligned records, so a bucket is a contiguous run.
//
// Phases:
//   1. pack + bounds: records in cloud order, per-dimension min/max.
//   2. top levels (segments larger than kSmallMax points), level by level,
//      all segments of a level at once:
//        prepare  cut dimension from the segment's box
//        minmax   min/max of the cut coordinate over the segment
//        cut      clamp the box midpoint into [min, max]
//        count    #(< cut) and #(== cut)
//        pass 1/2 the reference's two Hoare-style passes: the i-th misplaced
//                 element from the left trades places with the i-th
//                 misplaced element from the right. Ranks come from a
//                 device-wide exclusive scan of the misplaced flags (block
//                 sums, their scan, then the block scans again writing each
//                 element straight to its pair slot), and the pairs in the
//                 two slot tables are swapped.
//        finalize leftCount, node, children
//   3. small segments: one thread each runs the reference's sequential
//      recursion (as an explicit stack in global scratch) on its points,
//      emitting a pre-order subtree into a private node range.
//   4. renumber: subtree sizes bottom-up, pre-order positions top-down,
//      then every node is written to its final slot.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <limits>
#include <vector>

#include "internal.cuh"

namespace nabo_gb300 {
namespace {

constexpr int kBlock = 256;
constexpr int kSmallMax = 256;
constexpr unsigned kFull = 0xffffffffu;

__device__ __forceinline__ int2 add2(int2 a, int2 b) { return make_int2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ uint32_t shfl_up(uint32_t v, int o) { return __shfl_up_sync(kFull, v, o); }
__device__ __forceinline__ unsigned long long shfl_up(unsigned long long v, int o) {
  return __shfl_up_sync(kFull, v, o);
}
__device__ __forceinline__ int2 shfl_up(int2 v, int o) {
  return make_int2(__shfl_up_sync(kFull, v.x, o), __shfl_up_sync(kFull, v.y, o));
}

struct MinOp {
  template <typename V>
  __device__ V operator()(V a, V b) const { return a < b ? a : b; }
};
struct MaxOp {
  template <typename V>
  __device__ V operator()(V a, V b) const { return a > b ? a : b; }
};
struct AddOp {
  __device__ int2 operator()(int2 a, int2 b) const { return add2(a, b); }
};

// Reduction over runs of equal segment id inside a warp (segments are
// contiguous position ranges, so equal ids form one run). Returns the run's
// reduction in the run's last lane (`tail`).
template <typename V, typename Op>
__device__ __forceinline__ V seg_warp_reduce(int s, V v, Op op, bool* tail) {
  const int lane = threadIdx.x & 31;
  const int prev = __shfl_up_sync(kFull, s, 1);
  const bool head = (lane == 0) || (prev != s);
  const unsigned heads = __ballot_sync(kFull, head);
  const unsigned upto = heads & (kFull >> (31 - lane));
  const int runStart = 31 - __clz(upto);
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const V y = shfl_up(v, o);
    if (lane - o >= runStart) v = op(v, y);
  }
  *tail = (lane == 31) || ((heads >> (lane + 1)) & 1u);
  return v;
}

__device__ __forceinline__ int2 warp_incl_scan(int2 v, int lane) {
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int2 y = shfl_up(v, o);
    if (lane >= o) v = add2(v, y);
  }
  return v;
}

// Exclusive scan over a block of kBlock threads.
__device__ __forceinline__ int2 block_excl_scan(int2 v, int2* total) {
  __shared__ int2 sw[kBlock / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int2 inc = warp_incl_scan(v, lane);
  if (lane == 31) sw[warp] = inc;
  __syncthreads();
  if (warp == 0) {
    int2 w = lane < kBlock / 32 ? sw[lane] : make_int2(0, 0);
    w = warp_incl_scan(w, lane);
    if (lane < kBlock / 32) sw[lane] = w;
  }
  __syncthreads();
  const int2 wpre = warp > 0 ? sw[warp - 1] : make_int2(0, 0);
  *total = sw[kBlock / 32 - 1];
  __syncthreads();
  return add2(wpre, make_int2(inc.x - v.x, inc.y - v.y));
}

template <typename T>
struct Box {
  T lo[kMaxDim];
  T hi[kMaxDim];
};

// ---------------------------------------------------------------------------
// Phase 1: packing and bounds.

template <typename T, int D>
__global__ void k_pack(const T* __restrict__ cloud, int64_t n, int64_t stride, int dim, Rec<T, D>* __restrict__ recs) {
  const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (p >= n) return;
  Rec<T, D> r;
#pragma unroll
  for (int c = 0; c < RecSize<T, D>::chunks; ++c) r.v[c] = make_uint4(0u, 0u, 0u, 0u);
#pragma unroll
  for (int d = 0; d < D; ++d) r.p.c[d] = d < dim ? cloud[p * stride + d] : T(0);
  r.p.idx = (int32_t)p;
  recs[p] = r;
}

template <typename K>
__device__ __forceinline__ K warp_min(K v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const K y = __shfl_xor_sync(kFull, v, o);
    v = y < v ? y : v;
  }
  return v;
}
template <typename K>
__device__ __forceinline__ K warp_max(K v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const K y = __shfl_xor_sync(kFull, v, o);
    v = y > v ? y : v;
  }
  return v;
}

template <typename T, int D>
__global__ void k_bounds(const Rec<T, D>* __restrict__ recs, int64_t n, int dim, typename KeyOf<T>::type* mnK,
                         typename KeyOf<T>::type* mxK, int* nonFinite) {
  using Key = typename KeyOf<T>::type;
  Key mn[D], mx[D];
  int bad = 0;
#pragma unroll
  for (int d = 0; d < D; ++d) {
    mn[d] = ordered_key(Ar<T>::inf());
    mx[d] = ordered_key(-Ar<T>::inf());
  }
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x) {
    Rec<T, D> r;
    load_rec(recs, p, r);
#pragma unroll
    for (int d = 0; d < D; ++d) {
      const Key k = ordered_key(r.p.c[d]);
      mn[d] = k < mn[d] ? k : mn[d];
      mx[d] = k > mx[d] ? k : mx[d];
      bad |= (d < dim && !isfinite(r.p.c[d])) ? 1 : 0;
    }
  }
  if (__any_sync(kFull, bad) && (threadIdx.x & 31) == 0) atomicOr(nonFinite, 1);
#pragma unroll
  for (int d = 0; d < D; ++d) {
    const Key a = warp_min(mn[d]);
    const Key b = warp_max(mx[d]);
    if ((threadIdx.x & 31) == 0 && d < dim) {
      atomicMin(mnK + d, a);
      atomicMax(mxK + d, b);
    }
  }
}

template <typename T>
__global__ void k_init_keys(typename KeyOf<T>::type* mnK, typename KeyOf<T>::type* mxK, int dim) {
  const int d = threadIdx.x;
  if (d < dim) {
    mnK[d] = ordered_key(Ar<T>::inf());
    mxK[d] = ordered_key(-Ar<T>::inf());
  }
}

template <typename T>
__global__ void k_decode_keys(const typename KeyOf<T>::type* mnK, const typename KeyOf<T>::type* mxK, int dim,
                              T* lo, T* hi) {
  const int d = threadIdx.x;
  if (d < dim) {
    lo[d] = ordered_val(mnK[d], T(0));
    hi[d] = ordered_val(mxK[d], T(0));
  }
}

// ---------------------------------------------------------------------------
// Phase 2: top levels.

template <typename T>
struct SegLevel {
  int* start;
  int* count;
  T* boxLo;  // [cap * kMaxDim]
  T* boxHi;
  int* cutDim;
  typename KeyOf<T>::type* mnK;
  typename KeyOf<T>::type* mxK;
  T* cut;
  int* mode;  // 0: midpoint inside range, 1: below min, 2: above max
  int* lt;
  int* eq;
  int* leftCount;
  int* newLeft;
  int* newRight;
};

template <typename T>
struct TopNodes {
  int* dim;
  T* cut;
  int* left;   // >= 0: top node id; < 0: ~small segment id
  int* right;
  int* size;
  int* pre;
};

// Level bookkeeping kept on the device, so a fixed number of levels can run
// without reading anything back (graph capture) and the host-driven loop
// reads only `nseg` after each level.
struct LevelState {
  int nseg;       // segments of the current level
  int levelBase;  // top-node id of the current level's first segment
  int level;      // current level
  int nLevels;    // levels finished
  int overflow;   // capacity exceeded
  int pad[3];
};

template <typename T>
struct SmallSegs {
  int* start;
  int* count;
  int* depth;
  T* boxLo;  // [cap * kMaxDim]
  T* boxHi;
  int* size;
  int* base;
};

template <typename T>
__global__ void k_root_segment(SegLevel<T> L, int n, Box<T> box, int dim) {
  L.start[0] = 0;
  L.count[0] = n;
  for (int d = 0; d < dim; ++d) {
    L.boxLo[d] = box.lo[d];
    L.boxHi[d] = box.hi[d];
  }
}

template <typename T>
__global__ void k_root_small(SmallSegs<T> S, int n, Box<T> box, int dim) {
  S.start[0] = 0;
  S.count[0] = n;
  S.depth[0] = 0;
  for (int d = 0; d < dim; ++d) {
    S.boxLo[d] = box.lo[d];
    S.boxHi[d] = box.hi[d];
  }
}

// argMax of the box extents (nabo/kdtree_cpu.cpp:76-90): first strict
// maximum, starting from 0, so all-zero extents give dimension 0.
template <typename T>
__device__ __forceinline__ int arg_max_extent(const T* lo, const T* hi, int dim) {
  T best = T(0);
  int bd = 0;
  for (int d = 0; d < dim; ++d) {
    const T e = Ar<T>::sub(hi[d], lo[d]);
    if (e > best) {
      best = e;
      bd = d;
    }
  }
  return bd;
}

template <typename T>
__global__ void k_prepare(SegLevel<T> L, const LevelState* st, int dim) {
  pdl_begin();
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= st->nseg) return;
  L.cutDim[s] = arg_max_extent(L.boxLo + (int64_t)s * kMaxDim, L.boxHi + (int64_t)s * kMaxDim, dim);
  L.mnK[s] = ordered_key(std::numeric_limits<T>::max());
  L.mxK[s] = ordered_key(std::numeric_limits<T>::lowest());
  L.lt[s] = 0;
  L.eq[s] = 0;
}

// Also keeps each position's coordinate along its segment's cut dimension in
// `val` for the rest of the level (4 or 8 bytes instead of a whole record;
// the swaps move it with the records). With `remap` (every level but the
// first) it first moves each position to the segment it fell into at the
// previous level `prev`: its left or right child segment, -1 once that is a
// small segment.
template <typename T, int D>
__global__ void k_minmax(const Rec<T, D>* __restrict__ recs, int* __restrict__ segOf, int n, SegLevel<T> L,
                         SegLevel<T> prev, int remap, const LevelState* st, T* __restrict__ val) {
  pdl_begin();
  using Key = typename KeyOf<T>::type;
  if (st->nseg == 0) return;
  for (int64_t tile = blockIdx.x; tile * kBlock < n; tile += gridDim.x) {
    const int64_t p = tile * kBlock + threadIdx.x;
    int s = -1;
    Key kmin = 0, kmax = 0;
    if (p < n) {
      s = segOf[p];
      if (remap && s >= 0) {
        s = (int)p - prev.start[s] < prev.leftCount[s] ? prev.newLeft[s] : prev.newRight[s];
        segOf[p] = s;
      }
      if (s >= 0) {
        const T v = recs[p].p.c[L.cutDim[s]];
        val[p] = v;
        kmin = kmax = ordered_key(v);
      }
    }
    bool tail;
    kmin = seg_warp_reduce(s, kmin, MinOp(), &tail);
    kmax = seg_warp_reduce(s, kmax, MaxOp(), &tail);
    if (tail && s >= 0) {
      atomicMin(L.mnK + s, kmin);
      atomicMax(L.mxK + s, kmax);
    }
  }
}

// Median-split trees (split rule 1): the cut is just above the median of the
// segment's coordinates along the cut dimension (sampled at kMedianSamples
// evenly spaced positions at the level-synchronous levels, where the
// segment's points are in no particular order; exact in k_small). Just above
// (the next representable value): points equal to the median go left and
// hardly any point lies on the cut, so the build's second partition pass,
// which only segments with points on their cut run, is skipped.
constexpr int kMedianSamples = 31;

__device__ __forceinline__ float next_up(float x) { return nextafterf(x, __builtin_huge_valf()); }
__device__ __forceinline__ double next_up(double x) { return nextafter(x, __builtin_huge_val()); }

template <typename T>
__device__ T sampled_median(const T* __restrict__ val, int start, int count) {
  T smp[kMedianSamples];
  for (int j = 0; j < kMedianSamples; ++j)
    smp[j] = val[start + (int)((int64_t)(2 * j + 1) * count / (2 * kMedianSamples))];
  for (int i = 1; i < kMedianSamples; ++i) {  // insertion sort
    const T x = smp[i];
    int j = i - 1;
    while (j >= 0 && x < smp[j]) {
      smp[j + 1] = smp[j];
      --j;
    }
    smp[j + 1] = x;
  }
  return smp[kMedianSamples / 2];
}

template <typename T>
__global__ void k_cut(SegLevel<T> L, const LevelState* st, const T* __restrict__ val, int splitRule) {
  pdl_begin();
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= st->nseg) return;
  const int cd = L.cutDim[s];
  const T mn = ordered_val(L.mnK[s], T(0));
  const T mx = ordered_val(L.mxK[s], T(0));
  // (max + min) / 2 as the reference writes it (nabo/kdtree_cpu.cpp:135);
  // halving is exact, so multiplying by 1/2 gives the same value. The
  // median rule takes a point's coordinate, which lies in [mn, mx].
  const T ideal = splitRule == 1
                      ? next_up(sampled_median(val, L.start[s], L.count[s]))
                      : Ar<T>::mul(Ar<T>::add(L.boxHi[(int64_t)s * kMaxDim + cd], L.boxLo[(int64_t)s * kMaxDim + cd]),
                                   T(0.5));
  T cut;
  int mode;
  if (ideal < mn) {
    cut = mn;
    mode = 1;
  } else if (ideal > mx) {
    cut = mx;
    mode = 2;
  } else {
    cut = ideal;
    mode = 0;
  }
  L.cut[s] = cut;
  L.mode[s] = mode;
}

template <typename T>
__global__ void k_count(const T* __restrict__ val, const int* __restrict__ segOf, int n, SegLevel<T> L,
                        const LevelState* st) {
  pdl_begin();
  if (st->nseg == 0) return;
  for (int64_t tile = blockIdx.x; tile * kBlock < n; tile += gridDim.x) {
    const int64_t p = tile * kBlock + threadIdx.x;
    int s = -1;
    int2 c = make_int2(0, 0);
    if (p < n) {
      s = segOf[p];
      if (s >= 0) {
        const T v = val[p];
        const T cut = L.cut[s];
        c = make_int2(v < cut ? 1 : 0, v == cut ? 1 : 0);
      }
    }
    bool tail;
    c = seg_warp_reduce(s, c, AddOp(), &tail);
    if (tail && s >= 0) {
      if (c.x) atomicAdd(L.lt + s, c.x);
      if (c.y) atomicAdd(L.eq + s, c.y);
    }
  }
}

// Misplaced flags of the reference's partition passes (nabo/kdtree_cpu.cpp
// :149-177). Pass 1 scans the whole segment for `< cut`: a left element
// that is not `< cut` inside the first L positions trades with a right
// element that is not `>= cut`. Pass 2 scans from br1 = L for `<= cut`.
// (A segment without points equal to its cut has nothing to move in pass 2:
// after pass 1 everything < cut is left of lt and everything else right.)
template <typename T>
__device__ __forceinline__ int2 misplaced(const T* __restrict__ val, const int* __restrict__ segOf, int n,
                                          const SegLevel<T>& L, int pass, int p, int* segOut) {
  int2 f = make_int2(0, 0);
  int s = -1;
  if (p < n) {
    s = segOf[p];
    if (s >= 0 && (pass == 1 || L.eq[s] != 0)) {
      const T v = val[p];
      const T cut = L.cut[s];
      const int loc = p - L.start[s];
      const int lt = L.lt[s];
      if (pass == 1) {
        f.x = (loc < lt && !(v < cut)) ? 1 : 0;
        f.y = (loc >= lt && !(v >= cut)) ? 1 : 0;
      } else {
        const int le = lt + L.eq[s];
        f.x = (loc >= lt && loc < le && !(v <= cut)) ? 1 : 0;
        f.y = (loc >= le && !(v > cut)) ? 1 : 0;
      }
    }
  }
  *segOut = s;
  return f;
}

// Block b owns tiles [b * tiles, (b + 1) * tiles) of kBlock positions and
// scans their misplaced flags in position order. Besides its total it
// records, for each segment, the block's running count at the segment's
// first position (exclusive) and last position (inclusive): with the block
// prefixes these give the segment's global range of ranks, so the pairing
// pass needs no per-position rank array.
template <typename T>
__global__ void k_flag_sums(const T* __restrict__ val, const int* __restrict__ segOf, int n, SegLevel<T> L,
                            int pass, int tiles, int2* blockSums, int2* segFirst, int2* segLast,
                            const LevelState* st) {
  pdl_begin();
  if (st->nseg == 0) return;
  int2 carry = make_int2(0, 0);
  for (int t = 0; t < tiles; ++t) {
    const int64_t p = ((int64_t)blockIdx.x * tiles + t) * kBlock + threadIdx.x;
    int s;
    const int2 f = misplaced(val, segOf, n, L, pass, p < n ? (int)p : n, &s);
    int2 total;
    const int2 ex = add2(block_excl_scan(f, &total), carry);
    if (s >= 0) {
      const int first = L.start[s];
      if (p == first) segFirst[s] = ex;
      if (p == first + L.count[s] - 1) segLast[s] = add2(ex, f);
    }
    carry = add2(carry, total);
  }
  if (threadIdx.x == 0) blockSums[blockIdx.x] = carry;
}

// Single block: exclusive scan of the per-block sums; the grand total goes
// to *total. Each thread scans a contiguous run serially and one block-wide
// scan joins the runs (a loop of block-wide scans over the sums would
// serialise on its barriers: 0.2 ms per call at 22 M points).
__global__ void k_scan_block_sums(int2* sums, int nb, int2* total, const LevelState* st) {
  pdl_begin();
  if (st->nseg == 0) {
    if (threadIdx.x == 0) *total = make_int2(0, 0);
    return;
  }
  const int per = (nb + kBlock - 1) / kBlock;
  const int b0 = threadIdx.x * per;
  const int b1 = min(b0 + per, nb);
  int2 run = make_int2(0, 0);
  for (int i = b0; i < b1; ++i) run = add2(run, sums[i]);
  int2 t;
  int2 carry = block_excl_scan(run, &t);
  for (int i = b0; i < b1; ++i) {
    const int2 v = sums[i];
    sums[i] = carry;
    carry = add2(carry, v);
  }
  if (threadIdx.x == 0) *total = t;
}

// The pairs of both passes: the i-th misplaced element from the left of a
// segment trades with its i-th misplaced element from the right. A left
// element's slot is its global rank among the left-misplaced; a right
// element of rank j among its segment's m goes to slot base + m - 1 - j,
// base being the segment's first global rank (so both tables list the
// segment's pairs in the same slots).
template <typename T>
__global__ void k_flag_pairs(const T* __restrict__ val, const int* __restrict__ segOf, int n, SegLevel<T> L,
                             int pass, int tiles, const int2* __restrict__ blockPrefix,
                             const int2* __restrict__ segFirst, const int2* __restrict__ segLast, int* pairA,
                             int* pairB, int cap, const LevelState* st) {
  pdl_begin();
  if (st->nseg == 0) return;
  const int perBlock = tiles * kBlock;
  int2 carry = blockPrefix[blockIdx.x];
  for (int t = 0; t < tiles; ++t) {
    const int64_t p = ((int64_t)blockIdx.x * tiles + t) * kBlock + threadIdx.x;
    int s;
    const int2 f = misplaced(val, segOf, n, L, pass, p < n ? (int)p : n, &s);
    int2 total;
    const int2 ex = add2(block_excl_scan(f, &total), carry);
    if (f.x && ex.x < cap) pairA[ex.x] = (int)p;
    if (f.y) {
      const int first = L.start[s];
      const int last = first + L.count[s] - 1;
      const int base = blockPrefix[first / perBlock].y + segFirst[s].y;
      const int end = blockPrefix[last / perBlock].y + segLast[s].y;  // base + m
      const int slot = base + end - 1 - ex.y;
      if (slot >= 0 && slot < cap) pairB[slot] = (int)p;
    }
    carry = add2(carry, total);
  }
}

// A pair outside [0, n) (a slot the pairing missed) is skipped and flagged
// in *err, which the build status reports.
template <typename T, int D>
__global__ void k_swap(Rec<T, D>* recs, T* val, const int* __restrict__ pairA, const int* __restrict__ pairB,
                       const int2* __restrict__ total, int cap, int n, int* err) {
  pdl_begin();
  const int m = min(cap, min(total->x, total->y));
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < m; t += gridDim.x * blockDim.x) {
    const int a = pairA[t], b = pairB[t];
    if ((unsigned)a >= (unsigned)n || (unsigned)b >= (unsigned)n) {
      atomicOr(err, 1);
      continue;
    }
    const Rec<T, D> ra = recs[a];
    recs[a] = recs[b];
    recs[b] = ra;
    const T va = val[a];
    val[a] = val[b];
    val[b] = va;
  }
}

// Writes the split of segment s of the current level (node levelBase + s):
// its node record and its two children, each either a segment of the next
// level (more than kSmallMax points) or a small segment, with the child
// boxes cut at `cut` along `cd` (nabo/kdtree_cpu.cpp:192-223). With
// `childDims` the children's cut dimensions are also recorded (the median
// split moves each point's next cut coordinate along with it).
template <typename T>
__device__ void emit_split(const SegLevel<T>& L, const SegLevel<T>& next, int s, int leftCount, int cd, T cut,
                           const TopNodes<T>& top, const SmallSegs<T>& small, int* counters, int dim, int segCap,
                           int smallCap, int node, int nextLevelBase, int level, bool childDims) {
  const int count = L.count[s];
  const int start = L.start[s];
  top.dim[node] = cd;
  top.cut[node] = cut;
  L.leftCount[s] = leftCount;
  const T* lo = L.boxLo + (int64_t)s * kMaxDim;
  const T* hi = L.boxHi + (int64_t)s * kMaxDim;
  for (int side = 0; side < 2; ++side) {
    const int cst = side == 0 ? start : start + leftCount;
    const int ccount = side == 0 ? leftCount : count - leftCount;
    int ref, newSeg = -1;
    T* dLo;
    T* dHi;
    if (ccount > kSmallMax) {
      const int id = atomicAdd(counters + 0, 1);
      if (id >= segCap) {
        atomicOr(counters + 3, 1);
        return;
      }
      next.start[id] = cst;
      next.count[id] = ccount;
      dLo = next.boxLo + (int64_t)id * kMaxDim;
      dHi = next.boxHi + (int64_t)id * kMaxDim;
      ref = nextLevelBase + id;
      newSeg = id;
    } else {
      const int sid = atomicAdd(counters + 1, 1);
      if (sid >= smallCap) {
        atomicOr(counters + 3, 1);
        return;
      }
      small.start[sid] = cst;
      small.count[sid] = ccount;
      small.depth[sid] = level + 1;
      dLo = small.boxLo + (int64_t)sid * kMaxDim;
      dHi = small.boxHi + (int64_t)sid * kMaxDim;
      ref = ~sid;
    }
    for (int d = 0; d < dim; ++d) {
      dLo[d] = lo[d];
      dHi[d] = hi[d];
    }
    if (side == 0) {
      dHi[cd] = cut;
      top.left[node] = ref;
      L.newLeft[s] = newSeg;
    } else {
      dLo[cd] = cut;
      top.right[node] = ref;
      L.newRight[s] = newSeg;
    }
    if (childDims && newSeg >= 0) next.cutDim[newSeg] = arg_max_extent(dLo, dHi, dim);
  }
}

// nabo/kdtree_cpu.cpp:180-223: leftCount rule, node, children.
template <typename T>
__global__ void k_finalize(SegLevel<T> L, SegLevel<T> next, const LevelState* st, TopNodes<T> top,
                           SmallSegs<T> small, int* counters, int dim, int segCap, int smallCap, int topCap) {
  pdl_begin();
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  const int nseg = st->nseg;
  if (s >= nseg) return;
  const int levelBase = st->levelBase;
  if (levelBase + s >= topCap) {
    atomicOr(counters + 3, 1);
    return;
  }
  const int count = L.count[s];
  const int br1 = L.lt[s];
  const int br2 = br1 + L.eq[s];
  const int mode = L.mode[s];
  int leftCount;
  if (mode == 1)
    leftCount = 1;
  else if (mode == 2)
    leftCount = count - 1;
  else if (br1 > count / 2)
    leftCount = br1;
  else if (br2 < count / 2)
    leftCount = br2;
  else
    leftCount = count / 2;
  // finite coordinates guarantee 1 <= leftCount < count; keep the split
  // productive whatever happens
  leftCount = leftCount < 1 ? 1 : (leftCount > count - 1 ? count - 1 : leftCount);
  emit_split(L, next, s, leftCount, L.cutDim[s], L.cut[s], top, small, counters, dim, segCap, smallCap,
             levelBase + s, levelBase + nseg, st->level, false);
}

// Closes a level: records its top-node range and makes the segments the
// level produced the current ones.
__global__ void k_advance(LevelState* st, int* counters, int* lvStart, int* lvCount, int maxLevels) {
  pdl_begin();
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  if (st->nseg > 0) {
    if (st->level < maxLevels) {
      lvStart[st->level] = st->levelBase;
      lvCount[st->level] = st->nseg;
      st->nLevels = st->level + 1;
    } else {
      st->overflow = 1;
    }
    st->levelBase += st->nseg;
    st->level += 1;
  }
  st->nseg = counters[0];
  counters[0] = 0;
}

// ---- median-split top levels (split rule 1): a stable partition by scatter
//
// The median-split tree is this library's own, so its top levels need not
// reproduce the reference's in-place swaps. Each level scans two flags per
// position of a large segment, coordinate <= m and coordinate < m (m the
// segment's sampled median), keeps one of them per segment and moves every
// record to its child's range, flagged records first, each side in position
// order, into the other of two record arrays. Records whose child is a
// small segment go straight to the final array that the small-segment phase
// reads. Segment ids and cut coordinates travel with the records, so a
// level reads each position's id and coordinate twice and its record once,
// and writes its record, next id and next coordinate once: 6 launches and
// about 56 bytes per position of a large segment per level, against 14
// launches for the reference's rule. The arrays in use alternate with the
// level's parity (LevelState::level), read on the device, so a fixed-level
// build needs no host decision.
constexpr int kItems = 4;               // consecutive positions per thread
constexpr int kTile = kBlock * kItems;  // positions per block and tile

template <typename T, int D>
struct MedianBufs {
  Rec<T, D>* rec[2];  // [n]
  int* seg[2];        // [nPad]: segment of the level, -1 outside large segments
  T* val[2];          // [nPad]: coordinate along the segment's cut dimension
  // selects rather than indexing, which would copy the struct to local memory
  __device__ Rec<T, D>* recs(int i) const { return i ? rec[1] : rec[0]; }
  __device__ int* segs(int i) const { return i ? seg[1] : seg[0]; }
  __device__ T* vals(int i) const { return i ? val[1] : val[0]; }
};

template <typename T>
__device__ __forceinline__ void load4(const T* __restrict__ p, T (&v)[kItems]) {
  if constexpr (sizeof(T) == 4) {
    const float4 x = *reinterpret_cast<const float4*>(p);
    v[0] = x.x;
    v[1] = x.y;
    v[2] = x.z;
    v[3] = x.w;
  } else {
    const double2 a = reinterpret_cast<const double2*>(p)[0];
    const double2 b = reinterpret_cast<const double2*>(p)[1];
    v[0] = a.x;
    v[1] = a.y;
    v[2] = b.x;
    v[3] = b.y;
  }
}

template <typename T, int D>
__device__ __forceinline__ T rec_coord(const Rec<T, D>& r, int cd) {
  T v = r.p.c[0];
#pragma unroll
  for (int d = 1; d < D; ++d) v = d == cd ? r.p.c[d] : v;
  return v;
}

// One tile's positions of a thread: segment ids, coordinates and the two
// flags (x: v <= m, y: v < m; m = L.cut[s] holds the median until the
// level's split is chosen).
template <typename T>
struct MedianItems {
  int s[kItems];
  T v[kItems];
};

template <typename T>
__device__ __forceinline__ void median_load(const int* __restrict__ seg, const T* __restrict__ val, int64_t p0,
                                            int64_t nPad, MedianItems<T>& it) {
  if (p0 < nPad) {
    const int4 s4 = *reinterpret_cast<const int4*>(seg + p0);
    it.s[0] = s4.x;
    it.s[1] = s4.y;
    it.s[2] = s4.z;
    it.s[3] = s4.w;
    load4(val + p0, it.v);
  } else {
#pragma unroll
    for (int i = 0; i < kItems; ++i) {
      it.s[i] = -1;
      it.v[i] = T(0);
    }
  }
}

template <typename T>
__device__ __forceinline__ int2 median_flag(const SegLevel<T>& L, int s, T v) {
  if (s < 0) return make_int2(0, 0);
  const T m = L.cut[s];
  return make_int2(v <= m ? 1 : 0, v < m ? 1 : 0);
}

template <typename T, int D>
__global__ void k_median_cut(SegLevel<T> L, const LevelState* st, MedianBufs<T, D> B) {
  pdl_begin();
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= st->nseg) return;
  L.cut[s] = sampled_median(B.vals(st->level & 1), L.start[s], L.count[s]);
}

// Block b scans tiles [b * tiles, (b + 1) * tiles) in position order and
// records, besides its totals, each segment's running flag counts at its
// first position (exclusive) and last position (inclusive), as k_flag_sums.
// The next tile's ids and coordinates are loaded before this tile's scan.
template <typename T, int D>
__global__ void k_median_sums(MedianBufs<T, D> B, int64_t nPad, SegLevel<T> L, int tiles, int2* blockSums,
                              int2* segFirst, int2* segLast, const LevelState* st) {
  pdl_begin();
  if (st->nseg == 0) return;
  const int par = st->level & 1;
  const int* seg = B.segs(par);
  const T* val = B.vals(par);
  const int64_t first = (int64_t)blockIdx.x * tiles * kTile + threadIdx.x * kItems;
  MedianItems<T> nxt;
  median_load(seg, val, first, nPad, nxt);
  int2 carry = make_int2(0, 0);
  for (int t = 0; t < tiles; ++t) {
    const MedianItems<T> it = nxt;
    const int64_t p0 = first + (int64_t)t * kTile;
    if (t + 1 < tiles) median_load(seg, val, p0 + kTile, nPad, nxt);
    int2 f[kItems];
    int2 sum = make_int2(0, 0);
#pragma unroll
    for (int i = 0; i < kItems; ++i) {
      f[i] = median_flag(L, it.s[i], it.v[i]);
      sum = add2(sum, f[i]);
    }
    int2 total;
    int2 ex = add2(block_excl_scan(sum, &total), carry);
#pragma unroll
    for (int i = 0; i < kItems; ++i) {
      const int s = it.s[i];
      if (s >= 0) {
        const int64_t p = p0 + i;
        const int st0 = L.start[s];
        if (p == st0) segFirst[s] = ex;
        if (p == st0 + L.count[s] - 1) segLast[s] = add2(ex, f[i]);
      }
      ex = add2(ex, f[i]);
    }
    carry = add2(carry, total);
  }
  if (threadIdx.x == 0) blockSums[blockIdx.x] = carry;
}

// Chooses each segment's split from its two flag totals and writes it:
//   some point above the median  -> cut just above it, left = v <= m
//   else some point below it     -> cut at it, left = v < m
//   else (all equal)             -> cut at it, first half left by position
// L.lt keeps the chosen flag's global rank at the segment's first position.
template <typename T>
__global__ void k_median_split(SegLevel<T> L, SegLevel<T> next, const LevelState* st, TopNodes<T> top,
                               SmallSegs<T> small, int* counters, int dim, int segCap, int smallCap, int topCap,
                               const int2* __restrict__ blockPrefix, const int2* __restrict__ segFirst,
                               const int2* __restrict__ segLast, int perBlock) {
  pdl_begin();
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  const int nseg = st->nseg;
  if (s >= nseg) return;
  const int levelBase = st->levelBase;
  if (levelBase + s >= topCap) {
    atomicOr(counters + 3, 1);
    return;
  }
  const int count = L.count[s];
  const int start = L.start[s];
  const int2 a = add2(blockPrefix[start / perBlock], segFirst[s]);
  const int2 b = add2(blockPrefix[(start + count - 1) / perBlock], segLast[s]);
  const int le = b.x - a.x, lt = b.y - a.y;
  const T m = L.cut[s];
  int mode, leftCount;
  T cut;
  if (le < count) {
    mode = 0;
    leftCount = le;
    cut = next_up(m);
    L.lt[s] = a.x;
  } else if (lt > 0) {
    mode = 1;
    leftCount = lt;
    cut = m;
    L.lt[s] = a.y;
  } else {
    mode = 2;
    leftCount = count / 2;
    cut = m;
  }
  leftCount = leftCount < 1 ? 1 : (leftCount > count - 1 ? count - 1 : leftCount);
  L.mode[s] = mode;
  emit_split(L, next, s, leftCount, L.cutDim[s], cut, top, small, counters, dim, segCap, smallCap, levelBase + s,
             levelBase + nseg, st->level, true);
}

// Moves every record of a large segment to its child's range: a record with
// r flagged records before it in its segment goes to start + r when flagged,
// to start + leftCount + (its offset - r) otherwise. Positions outside large
// segments only mark themselves outside in the next level's id array.
template <typename T, int D>
__global__ void k_median_scatter(MedianBufs<T, D> B, Rec<T, D>* __restrict__ finalRecs, int64_t nPad,
                                 SegLevel<T> L, SegLevel<T> next, int tiles, const int2* __restrict__ blockPrefix,
                                 const LevelState* st) {
  pdl_begin();
  if (st->nseg == 0) return;
  const int par = st->level & 1;
  const int* seg = B.segs(par);
  const T* val = B.vals(par);
  const Rec<T, D>* src = B.recs(par);
  Rec<T, D>* dst = B.recs(par ^ 1);
  int* segN = B.segs(par ^ 1);
  T* valN = B.vals(par ^ 1);
  const int64_t first = (int64_t)blockIdx.x * tiles * kTile + threadIdx.x * kItems;
  MedianItems<T> nxt;
  median_load(seg, val, first, nPad, nxt);
  int2 carry = blockPrefix[blockIdx.x];
  for (int t = 0; t < tiles; ++t) {
    const MedianItems<T> it = nxt;
    const int64_t p0 = first + (int64_t)t * kTile;
    if (t + 1 < tiles) median_load(seg, val, p0 + kTile, nPad, nxt);
    int2 f[kItems];
    int2 sum = make_int2(0, 0);
#pragma unroll
    for (int i = 0; i < kItems; ++i) {
      f[i] = median_flag(L, it.s[i], it.v[i]);
      sum = add2(sum, f[i]);
    }
    int2 total;
    int2 ex = add2(block_excl_scan(sum, &total), carry);
    carry = add2(carry, total);
    if (p0 >= nPad) continue;
#pragma unroll
    for (int i = 0; i < kItems; ++i) {
      const int s = it.s[i];
      const int64_t p = p0 + i;
      if (s < 0) {
        segN[p] = -1;
      } else {
        const int start = L.start[s];
        const int mode = L.mode[s];
        const int lc = L.leftCount[s];
        const int loc = (int)(p - start);
        int before;
        bool left;
        if (mode == 2) {
          before = loc < lc ? loc : lc;
          left = loc < lc;
        } else {
          before = (mode == 0 ? ex.x : ex.y) - L.lt[s];
          left = (mode == 0 ? f[i].x : f[i].y) != 0;
        }
        const int64_t dest = start + (left ? before : lc + (loc - before));
        const int child = left ? L.newLeft[s] : L.newRight[s];
        Rec<T, D> r;
        load_rec(src, p, r);
        if (child >= 0) {
          dst[dest] = r;
          segN[dest] = child;
          valN[dest] = rec_coord(r, next.cutDim[child]);
        } else {
          finalRecs[dest] = r;
          segN[dest] = -1;
        }
      }
      ex = add2(ex, f[i]);
    }
  }
}

// Staging a tile (record, destination, next id and coordinate per slot)
// within 47 KB of static shared memory: float records of up to 4
// dimensions.
template <typename T, int D>
constexpr bool median_staging_fits() {
  return (size_t)kTile * (sizeof(Rec<T, D>) + 2 * sizeof(int) + sizeof(T)) <= 47 * 1024;
}

// k_median_scatter with the tile's moves staged in shared memory: each
// record, with its destination and next id and coordinate, goes to a slot
// in destination order (the tile's flagged records first, each side in
// position order, so every run of one segment and side is contiguous in
// both), then the block writes the slots out, consecutive threads to
// consecutive destinations.
template <typename T, int D>
__global__ void k_median_scatter_staged(MedianBufs<T, D> B, Rec<T, D>* __restrict__ finalRecs, int64_t nPad,
                                        SegLevel<T> L, SegLevel<T> next, int tiles,
                                        const int2* __restrict__ blockPrefix, const LevelState* st) {
  // (instantiated only where the staging fits; see median_scatter)
  constexpr int kStage = median_staging_fits<T, D>() ? kTile : 1;
  __shared__ Rec<T, D> sRec[kStage];
  __shared__ int sDest[kStage];
  __shared__ int sChild[kStage];
  __shared__ T sVal[kStage];
  pdl_begin();
  if (st->nseg == 0) return;
  const int par = st->level & 1;
  const int* seg = B.segs(par);
  const T* val = B.vals(par);
  const Rec<T, D>* src = B.recs(par);
  Rec<T, D>* dst = B.recs(par ^ 1);
  int* segN = B.segs(par ^ 1);
  T* valN = B.vals(par ^ 1);
  const int64_t first = (int64_t)blockIdx.x * tiles * kTile + threadIdx.x * kItems;
  MedianItems<T> nxt;
  median_load(seg, val, first, nPad, nxt);
  int2 carry = blockPrefix[blockIdx.x];
  for (int t = 0; t < tiles; ++t) {
    const MedianItems<T> it = nxt;
    const int64_t p0 = first + (int64_t)t * kTile;
    if (t + 1 < tiles) median_load(seg, val, p0 + kTile, nPad, nxt);
    int2 f[kItems];
    int2 sum = make_int2(0, 0);
#pragma unroll
    for (int i = 0; i < kItems; ++i) {
      f[i] = median_flag(L, it.s[i], it.v[i]);
      sum = add2(sum, f[i]);
    }
    int2 total;
    int2 ex = add2(block_excl_scan(sum, &total), carry);
    carry = add2(carry, total);
    // destination of each held record and its side
    int dest[kItems];
    bool left[kItems];
    int2 side = make_int2(0, 0);  // (left, right) records this thread moves
#pragma unroll
    for (int i = 0; i < kItems; ++i) {
      const int s = it.s[i];
      dest[i] = -1;
      left[i] = false;
      if (s >= 0) {
        const int64_t p = p0 + i;
        const int start = L.start[s];
        const int mode = L.mode[s];
        const int lc = L.leftCount[s];
        const int loc = (int)(p - start);
        int before;
        if (mode == 2) {
          before = loc < lc ? loc : lc;
          left[i] = loc < lc;
        } else {
          before = (mode == 0 ? ex.x : ex.y) - L.lt[s];
          left[i] = (mode == 0 ? f[i].x : f[i].y) != 0;
        }
        dest[i] = start + (left[i] ? before : lc + (loc - before));
        side = add2(side, make_int2(left[i] ? 1 : 0, left[i] ? 0 : 1));
      } else if (p0 < nPad) {
        segN[p0 + i] = -1;
      }
      ex = add2(ex, f[i]);
    }
    int2 sideTotal;
    int2 slot = block_excl_scan(side, &sideTotal);
    slot.y += sideTotal.x;  // rights after all lefts
#pragma unroll
    for (int i = 0; i < kItems; ++i) {
      if (dest[i] < 0) continue;
      const int s = it.s[i];
      const int j = left[i] ? slot.x++ : slot.y++;
      const int child = left[i] ? L.newLeft[s] : L.newRight[s];
      Rec<T, D> r;
      load_rec(src, p0 + i, r);
      sRec[j] = r;
      sChild[j] = child;
      sDest[j] = dest[i];
      if (child >= 0) sVal[j] = rec_coord(r, next.cutDim[child]);
    }
    __syncthreads();
    const int moved = sideTotal.x + sideTotal.y;
    for (int j = threadIdx.x; j < moved; j += blockDim.x) {
      const int d = sDest[j];
      const int child = sChild[j];
      if (child >= 0) {
        dst[d] = sRec[j];
        segN[d] = child;
        valN[d] = sVal[j];
      } else {
        finalRecs[d] = sRec[j];
        segN[d] = -1;
      }
    }
    __syncthreads();
  }
}

// The scatter kernel for this record size.
template <typename T, int D>
constexpr auto median_scatter() {
  if constexpr (median_staging_fits<T, D>())
    return k_median_scatter_staged<T, D>;
  else
    return k_median_scatter<T, D>;
}

// A fixed-level build that ran out of levels leaves records of unfinished
// segments in the working arrays; they go to the final array, whose cloud
// ranges then hold every point (the one-leaf-per-cloud fallback reads them).
template <typename T, int D>
__global__ void k_median_flush(MedianBufs<T, D> B, Rec<T, D>* finalRecs, int64_t n, const LevelState* st) {
  if (st->nseg == 0) return;
  const int par = st->level & 1;
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x)
    if (B.segs(par)[p] >= 0) finalRecs[p] = B.recs(par)[p];
}

// ---- forest set-up: clouds are contiguous point ranges [off[c], off[c+1])

// Packs the clouds into records (index within the cloud) and reduces each
// cloud's per-dimension min/max (ordered keys) and a non-finite flag, in
// one pass. Block b takes the contiguous positions [b * chunk, (b + 1) *
// chunk) a tile of kBlock at a time, following the clouds with a cursor (a
// binary search once per thread); each lane keeps the running min/max of
// its current cloud, and the warp flushes them (reduced across the lanes
// of each cloud, one atomic per cloud and dimension) only when some lane's
// cloud changes, and at the end. With `smallRoots`, points of clouds whose
// root is already a small segment are also written there.
template <typename T, int D>
__global__ void k_pack_bounds(const T* __restrict__ cloud, int64_t n, int64_t stride, int dim,
                              const int64_t* __restrict__ off, int nClouds, int64_t chunk,
                              Rec<T, D>* __restrict__ recs, Rec<T, D>* __restrict__ smallRoots,
                              typename KeyOf<T>::type* mnK, typename KeyOf<T>::type* mxK, int* nonFinite) {
  using Key = typename KeyOf<T>::type;
  const int64_t begin = blockIdx.x * chunk;
  const int64_t end = begin + chunk < n ? begin + chunk : n;
  if (begin >= end) return;
  int c = cloud_of(off, nClouds, begin + threadIdx.x < end ? begin + threadIdx.x : begin);
  int cur = -1;  // cloud of the running min/max
  Key kmin[D], kmax[D];
#pragma unroll
  for (int d = 0; d < D; ++d) {
    kmin[d] = ~Key(0);
    kmax[d] = 0;
  }
  int bad = 0;
  auto flush = [&]() {
#pragma unroll
    for (int d = 0; d < D; ++d) {
      bool tail;
      const Key a = seg_warp_reduce(cur, kmin[d], MinOp(), &tail);
      const Key b = seg_warp_reduce(cur, kmax[d], MaxOp(), &tail);
      if (tail && cur >= 0 && d < dim) {
        atomicMin(mnK + (int64_t)cur * kMaxDim + d, a);
        atomicMax(mxK + (int64_t)cur * kMaxDim + d, b);
      }
      kmin[d] = ~Key(0);
      kmax[d] = 0;
    }
  };
  for (int64_t p0 = begin; p0 < end; p0 += kBlock) {
    const int64_t p = p0 + threadIdx.x;
    int cp = -1;
    Rec<T, D> r;
    if (p < end) {
      while (off[c + 1] <= p) ++c;
      cp = c;
#pragma unroll
      for (int q = 0; q < RecSize<T, D>::chunks; ++q) r.v[q] = make_uint4(0u, 0u, 0u, 0u);
#pragma unroll
      for (int d = 0; d < D; ++d) r.p.c[d] = d < dim ? cloud[p * stride + d] : T(0);
      r.p.idx = (int32_t)(p - off[c]);
      recs[p] = r;
      if (smallRoots && off[c + 1] - off[c] <= kSmallMax) smallRoots[p] = r;
    }
    if (__any_sync(kFull, cp != cur)) {
      flush();
      cur = cp;
    }
    if (cp >= 0) {
#pragma unroll
      for (int d = 0; d < D; ++d) {
        const Key k = ordered_key(r.p.c[d]);
        kmin[d] = k < kmin[d] ? k : kmin[d];
        kmax[d] = k > kmax[d] ? k : kmax[d];
        bad |= (d < dim && !isfinite(r.p.c[d])) ? 1 : 0;
      }
    }
  }
  flush();
  if (__any_sync(kFull, bad) && (threadIdx.x & 31) == 0) atomicOr(nonFinite, 1);
}

template <typename T>
__global__ void k_init_keys_forest(typename KeyOf<T>::type* mnK, typename KeyOf<T>::type* mxK, int nClouds) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nClouds * kMaxDim) return;
  mnK[i] = ordered_key(Ar<T>::inf());
  mxK[i] = ordered_key(-Ar<T>::inf());
}

// One root per cloud: a level-0 segment when it has more than kSmallMax
// points, else a small segment. Root box = (min, max(numeric_limits<T>::min(),
// max)), as the reference's constructor sets it (nabo/nabo.cpp:73-74,
// nabo/kdtree_cpu.cpp:256-267).
template <typename T>
__global__ void k_forest_roots(const int64_t* __restrict__ off, int nClouds, const typename KeyOf<T>::type* mnK,
                               const typename KeyOf<T>::type* mxK, int dim, SegLevel<T> L, SmallSegs<T> small,
                               LevelState* st, int* counters, int* rootRef, int* rootSeg, T* rootLo, T* rootHi) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nClouds) return;
  const int64_t start = off[c];
  const int count = (int)(off[c + 1] - start);
  T* lo;
  T* hi;
  if (count > kSmallMax) {
    const int id = atomicAdd(&st->nseg, 1);
    L.start[id] = (int)start;
    L.count[id] = count;
    lo = L.boxLo + (int64_t)id * kMaxDim;
    hi = L.boxHi + (int64_t)id * kMaxDim;
    rootRef[c] = id;  // level 0 starts at top-node id 0
    rootSeg[c] = id;
  } else {
    const int sid = atomicAdd(counters + 1, 1);
    small.start[sid] = (int)start;
    small.count[sid] = count;
    small.depth[sid] = 0;
    lo = small.boxLo + (int64_t)sid * kMaxDim;
    hi = small.boxHi + (int64_t)sid * kMaxDim;
    rootRef[c] = ~sid;
    rootSeg[c] = -1;
  }
  for (int d = 0; d < dim; ++d) {
    const T mn = ordered_val(mnK[(int64_t)c * kMaxDim + d], T(0));
    const T mx = ordered_val(mxK[(int64_t)c * kMaxDim + d], T(0));
    const T tiny = std::numeric_limits<T>::min();
    lo[d] = mn;
    hi[d] = mx > tiny ? mx : tiny;
    rootLo[(int64_t)c * kMaxDim + d] = lo[d];
    rootHi[(int64_t)c * kMaxDim + d] = hi[d];
  }
  // the root segment's cut dimension (the median split reads it before
  // any level kernel runs)
  if (count > kSmallMax) L.cutDim[rootSeg[c]] = arg_max_extent(lo, hi, dim);
}

// Each position's root segment (-1 for a small root, and for the median
// split's padding [n, nPad)), by contiguous block ranges with a cloud
// cursor as in k_pack_bounds. With `val` (the median split) also the
// position's coordinate along its root segment's cut dimension.
template <typename T, int D>
__global__ void k_init_segof(int* segOf, int64_t n, int64_t nPad, int64_t chunk, const int64_t* __restrict__ off,
                             int nClouds, const int* __restrict__ rootSeg, const Rec<T, D>* __restrict__ recs,
                             const int* __restrict__ cutDim, T* val) {
  const int64_t begin = blockIdx.x * chunk;
  const int64_t end = begin + chunk < nPad ? begin + chunk : nPad;
  if (begin >= end) return;
  int c = begin < n ? cloud_of(off, nClouds, begin + threadIdx.x < n ? begin + threadIdx.x : begin) : 0;
  for (int64_t p = begin + threadIdx.x; p < end; p += kBlock) {
    int s = -1;
    if (p < n) {
      while (off[c + 1] <= p) ++c;
      s = rootSeg[c];
      if (val && s >= 0) val[p] = recs[p].p.c[cutDim[s]];
    }
    segOf[p] = s;
  }
}

// ---------------------------------------------------------------------------
// Phase 3: one thread per small segment, the reference's recursion with an
// explicit stack held in global scratch at the segment's own position range.

template <typename T>
struct SmallStack {
  int* start;
  int* count;
  int* parent;
  int* depth;
  T* boxLo;  // [n * kMaxDim]
  T* boxHi;
};

// One of the reference's two partition passes (nabo/kdtree_cpu.cpp:149-177)
// over the node's points pts[0, count), by a warp. Scanning from both ends,
// the reference swaps the i-th element from the left that fails the test
// with the i-th element from the right that passes it, while the first
// stays left of the second. Those are exactly the failing elements inside
// [lo, mid) and the passing elements inside [mid, hi) (mid = lo + the
// number of passing elements of [lo, hi)), paired in order from the left
// and from the right: `less` is the test `v < cut` of pass 1 over
// [0, count) and `v <= cut` of pass 2 over [lt, count).
template <typename T, int D>
__device__ __forceinline__ void warp_partition_pass(Rec<T, D>* pts, int lo, int mid, int hi, int cd, T cut,
                                                    bool lessEq, int* posL, int* posR, int lane) {
  const unsigned below = (1u << lane) - 1u;
  int nl = 0, nr = 0;
  for (int c0 = lo; c0 < hi; c0 += 32) {
    const int i = c0 + lane;
    bool fl = false, fr = false;
    if (i < hi) {
      const T v = pts[i].p.c[cd];
      const bool pass = lessEq ? (v <= cut) : (v < cut);
      fl = i < mid && !pass;
      fr = i >= mid && pass;
    }
    const unsigned bl = __ballot_sync(0xffffffffu, fl);
    const unsigned br = __ballot_sync(0xffffffffu, fr);
    // at most half of the node's points are misplaced on either side
    const int jl = nl + __popc(bl & below), jr = nr + __popc(br & below);
    if (fl && jl < kSmallMax / 2) posL[jl] = i;
    if (fr && jr < kSmallMax / 2) posR[jr] = i;
    nl += __popc(bl);
    nr += __popc(br);
  }
  __syncwarp();
  int m = nl < nr ? nl : nr;  // equal for a consistent mid
  m = m < kSmallMax / 2 ? m : kSmallMax / 2;
  for (int j = lane; j < m; j += 32) {
    const int a = posL[j], b = posR[m - 1 - j];
    const Rec<T, D> t = pts[a];
    pts[a] = pts[b];
    pts[b] = t;
  }
  __syncwarp();
}

// Small segments (at most kSmallMax points), one warp each over a fixed
// grid: the segment's records are staged in shared memory and its subtree is
// built by the reference recursion (nabo/kdtree_cpu.cpp:110-225) in
// pre-order with an explicit stack (global scratch, written by lane 0). Each
// split's min/max, counts and partition passes run across the lanes; node
// records and bucket order come out as the reference's.
// Ascending bitonic sort of 32 R keys held R per lane (element lane + 32 r),
// across the warp: partners at distance below 32 are exchanged by shuffle,
// at 32 inside the lane.
template <int R, typename Key>
__device__ __forceinline__ void warp_sort_keys(Key (&e)[R], int lane) {
#pragma unroll
  for (int k2 = 2; k2 <= 32 * R; k2 <<= 1) {
#pragma unroll
    for (int j = k2 >> 1; j > 0; j >>= 1) {
      Key o[R];
#pragma unroll
      for (int r = 0; r < R; ++r) o[r] = j >= 32 ? e[r ^ (j >> 5)] : __shfl_xor_sync(0xffffffffu, e[r], j);
#pragma unroll
      for (int r = 0; r < R; ++r) {
        const int i = lane + 32 * r;
        const bool keepMin = ((i & j) == 0) == ((i & k2) == 0);
        e[r] = keepMin ? (o[r] < e[r] ? o[r] : e[r]) : (o[r] > e[r] ? o[r] : e[r]);
      }
    }
  }
}

// The lower median (rank count / 2) of the count values node[i].p.c[cd],
// computed by the warp over the values' order-preserving keys (padding
// sorts above every finite value's key, so it never holds the rank). Up to
// 64 values a bitonic sort across the warp (one or two keys per lane) and
// the key at the rank; above, a bitwise radix select, most significant bit
// first: each round counts the remaining candidates whose next bit is 0 (one
// compare per held value, summed across the warp) and keeps the half that
// holds the rank, 32 rounds for float and 64 for double.
template <typename T, int D>
__device__ T warp_median(const Rec<T, D>* node, int count, int cd, int lane) {
  using Key = typename KeyOf<T>::type;
  const int want0 = count / 2;
  if (count <= 32) {
    Key e[1] = {lane < count ? ordered_key(node[lane].p.c[cd]) : ~Key(0)};
    warp_sort_keys<1>(e, lane);
    return ordered_val(__shfl_sync(0xffffffffu, e[0], want0), T(0));
  }
  if (count <= 64) {
    Key e[2];
#pragma unroll
    for (int r = 0; r < 2; ++r) e[r] = lane + 32 * r < count ? ordered_key(node[lane + 32 * r].p.c[cd]) : ~Key(0);
    warp_sort_keys<2>(e, lane);
    const Key m = __shfl_sync(0xffffffffu, want0 >= 32 ? e[1] : e[0], want0 & 31);
    return ordered_val(m, T(0));
  }
  constexpr int kPer = kSmallMax / 32;
  constexpr int kBits = 8 * (int)sizeof(Key);
  Key k[kPer];
#pragma unroll
  for (int j = 0; j < kPer; ++j) {
    const int i = lane + 32 * j;
    // padding sorts above every finite value's key, so it never holds the rank
    k[j] = i < count ? ordered_key(node[i].p.c[cd]) : ~Key(0);
  }
  const int held = (count + 31) / 32;
  Key prefix = 0;
  int want = want0;
  for (int b = kBits - 1; b >= 0; --b) {
    const Key sel = prefix >> b;
    int c = 0;
#pragma unroll
    for (int j = 0; j < kPer; ++j) c += (j < held && (k[j] >> b) == sel) ? 1 : 0;
    c = __reduce_add_sync(0xffffffffu, c);
    if (want >= c) {
      want -= c;
      prefix |= Key(1) << b;
    }
  }
  return ordered_val(prefix, T(0));
}

template <typename T, int D>
__global__ void k_small(Rec<T, D>* recs, SmallSegs<T> small, const int* nSmall, Node<T>* scratch,
                        SmallStack<T> stk, int dim, unsigned bucketSize, int* counters, int splitRule,
                        int* nextSeg) {
  extern __shared__ __align__(16) unsigned char smallSmem[];
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  const int warps = blockDim.x >> 5;
  Rec<T, D>* pts = reinterpret_cast<Rec<T, D>*>(smallSmem) + (size_t)warp * kSmallMax;
  int* posL = reinterpret_cast<int*>(reinterpret_cast<Rec<T, D>*>(smallSmem) + (size_t)warps * kSmallMax) +
              (size_t)warp * kSmallMax;
  int* posR = posL + kSmallMax / 2;
  const int nS = *nSmall;
  int hmax = 0;
  // segments are taken one at a time from a counter (sizes differ up to 2x;
  // a fixed assignment left warps idle at the end)
  for (;;) {
    int sid = 0;
    if (lane == 0) sid = atomicAdd(nextSeg, 1);
    sid = __shfl_sync(0xffffffffu, sid, 0);
    if (sid >= nS) break;
    const int base = small.start[sid];
    const int segN = small.count[sid];
    for (int i = lane; i < segN; i += 32) pts[i] = recs[base + i];
    Node<T>* out = scratch + 2 * (int64_t)base;
    if (lane == 0) {
      stk.start[base] = 0;
      stk.count[base] = segN;
      stk.parent[base] = -1;
      stk.depth[base] = small.depth[sid];
      for (int d = 0; d < dim; ++d) {
        stk.boxLo[(int64_t)base * kMaxDim + d] = small.boxLo[(int64_t)sid * kMaxDim + d];
        stk.boxHi[(int64_t)base * kMaxDim + d] = small.boxHi[(int64_t)sid * kMaxDim + d];
      }
    }
    __syncwarp();
    int sp = 1;
    int emitted = 0;
    // the node's cell over the compiled dimensions (registers; entries past
    // `dim` stay 0 and never win the widest-extent test)
    T lo[D], hi[D];
    while (sp > 0) {
      --sp;
      const int e = base + sp;
      const int st = stk.start[e];  // local to the segment
      const int count = stk.count[e];
      const int parent = stk.parent[e];
      const int depth = stk.depth[e];
      const int local = emitted++;
      if (lane == 0 && parent >= 0) out[parent].meta = make_meta(node_dim(out[parent].meta), (uint32_t)local);
      if (count <= (int)bucketSize) {
        if (lane == 0) store_leaf(out + local, (uint32_t)count, (uint32_t)(base + st));
        hmax = depth > hmax ? depth : hmax;
        __syncwarp();
        continue;
      }
#pragma unroll
      for (int d = 0; d < D; ++d) {
        lo[d] = d < dim ? stk.boxLo[(int64_t)e * kMaxDim + d] : T(0);
        hi[d] = d < dim ? stk.boxHi[(int64_t)e * kMaxDim + d] : T(0);
      }
      // argMax of the extents as arg_max_extent (first strict maximum)
      int cd = 0;
      T lcd = lo[0], hcd = hi[0];
      {
        T best = T(0);
#pragma unroll
        for (int d = 0; d < D; ++d) {
          const T ext = Ar<T>::sub(hi[d], lo[d]);
          if (d < dim && ext > best) {
            best = ext;
            cd = d;
            lcd = lo[d];
            hcd = hi[d];
          }
        }
      }
      Rec<T, D>* node = pts + st;
      const T ideal = splitRule == 1 ? next_up(warp_median(node, count, cd, lane))
                                     : Ar<T>::mul(Ar<T>::add(hcd, lcd), T(0.5));
      T mn = std::numeric_limits<T>::max(), mx = std::numeric_limits<T>::lowest();
      for (int i = lane; i < count; i += 32) {
        const T v = node[i].p.c[cd];
        mn = (mn < v) ? mn : v;
        mx = (v < mx) ? mx : v;
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const T a = __shfl_xor_sync(0xffffffffu, mn, o);
        const T b = __shfl_xor_sync(0xffffffffu, mx, o);
        mn = (mn < a) ? mn : a;
        mx = (b < mx) ? mx : b;
      }
      T cut;
      if (ideal < mn)
        cut = mn;
      else if (ideal > mx)
        cut = mx;
      else
        cut = ideal;
      int lt = 0, eq = 0;
      for (int c0 = 0; c0 < count; c0 += 32) {
        const int i = c0 + lane;
        const T v = i < count ? node[i].p.c[cd] : T(0);
        lt += __popc(__ballot_sync(0xffffffffu, i < count && v < cut));
        eq += __popc(__ballot_sync(0xffffffffu, i < count && v == cut));
      }
      warp_partition_pass<T, D>(node, 0, lt, count, cd, cut, false, posL, posR, lane);
      if (eq > 0) warp_partition_pass<T, D>(node, lt, lt + eq, count, cd, cut, true, posL, posR, lane);
      const int br1 = lt, br2 = lt + eq;
      int leftCount;
      if (ideal < mn)
        leftCount = 1;
      else if (ideal > mx)
        leftCount = count - 1;
      else if (br1 > count / 2)
        leftCount = br1;
      else if (br2 < count / 2)
        leftCount = br2;
      else
        leftCount = count / 2;
      leftCount = leftCount < 1 ? 1 : (leftCount > count - 1 ? count - 1 : leftCount);
      if (sp + 2 > segN || local + 2 >= 2 * segN) {  // cannot happen for a valid split; never overrun
        if (lane == 0) atomicOr(counters + 3, 2);
        break;
      }
      if (lane == 0) {
        store_inner(out + local, (uint32_t)cd, 0u, cut);
        // push right (processed after the whole left subtree), then left
        int f = base + sp;
        stk.start[f] = st + leftCount;
        stk.count[f] = count - leftCount;
        stk.parent[f] = local;
        stk.depth[f] = depth + 1;
#pragma unroll
        for (int d = 0; d < D; ++d) {
          if (d < dim) {
            stk.boxLo[(int64_t)f * kMaxDim + d] = d == cd ? cut : lo[d];
            stk.boxHi[(int64_t)f * kMaxDim + d] = hi[d];
          }
        }
        f = base + sp + 1;
        stk.start[f] = st;
        stk.count[f] = leftCount;
        stk.parent[f] = -1;
        stk.depth[f] = depth + 1;
#pragma unroll
        for (int d = 0; d < D; ++d) {
          if (d < dim) {
            stk.boxLo[(int64_t)f * kMaxDim + d] = lo[d];
            stk.boxHi[(int64_t)f * kMaxDim + d] = d == cd ? cut : hi[d];
          }
        }
      }
      sp += 2;
      __syncwarp();
    }
    __syncwarp();
    for (int i = lane; i < segN; i += 32) recs[base + i] = pts[i];
    if (lane == 0) small.size[sid] = emitted;
    __syncwarp();
  }
  if (lane == 0) atomicMax(counters + 2, hmax);
}

template <typename T, int D>
inline int small_warps_per_block() {
  const size_t perWarp = (size_t)kSmallMax * (sizeof(Rec<T, D>) + sizeof(int));
  const size_t w = (48 * 1024) / perWarp;
  return (int)(w < 1 ? 1 : (w > 4 ? 4 : w));
}

// ---------------------------------------------------------------------------
// Phase 4: pre-order numbering (single block).

template <typename T>
__device__ __forceinline__ int subtree_size(const TopNodes<T>& top, const SmallSegs<T>& small, int ref) {
  return ref >= 0 ? top.size[ref] : small.size[~ref];
}

// Pre-order numbering of all trees (single block): subtree sizes bottom-up,
// each cloud's root at the running sum of the previous trees' sizes, then
// positions top-down.
//
// A build that did not finish (status[1]: levels left over after a fixed
// level count, or a capacity guard hit) has top nodes whose children were
// never split, so no numbering exists. Every cloud then gets one leaf
// holding all of its points instead: a well-formed forest that a search
// (or a captured graph's search) can still traverse, and which gives exact
// results for finite clouds.
template <typename T>
__global__ void k_renumber(TopNodes<T> top, SmallSegs<T> small, const int* lvStart, const int* lvCount,
                           const LevelState* st, const int* rootRef, const int64_t* __restrict__ off, int nClouds,
                           int* status, Node<T>* nodes, int64_t nodeCap, int64_t* nodeOffset) {
  __shared__ int64_t carry;
  if (status[1]) {
    for (int c = threadIdx.x; c <= nClouds; c += blockDim.x) {
      nodeOffset[c] = c;
      if (c < nClouds && c < nodeCap) store_leaf(nodes + c, (uint32_t)(off[c + 1] - off[c]), (uint32_t)off[c]);
    }
    if (threadIdx.x == 0) status[2] = 0;
    return;
  }
  const int nLevels = st->nLevels;
  for (int l = nLevels - 1; l >= 0; --l) {
    const int b = lvStart[l], c = lvCount[l];
    for (int i = threadIdx.x; i < c; i += blockDim.x) {
      const int t = b + i;
      top.size[t] = 1 + subtree_size(top, small, top.left[t]) + subtree_size(top, small, top.right[t]);
    }
    __syncthreads();
  }
  // tree offsets: exclusive scan of the root sizes, in cloud order
  if (threadIdx.x == 0) {
    carry = 0;
    for (int c = 0; c < nClouds; ++c) {
      const int ref = rootRef[c];
      nodeOffset[c] = carry;
      if (ref >= 0)
        top.pre[ref] = (int)carry;
      else
        small.base[~ref] = (int)carry;
      carry += subtree_size(top, small, ref);
    }
    nodeOffset[nClouds] = carry;
  }
  __syncthreads();
  for (int l = 0; l < nLevels; ++l) {
    const int b = lvStart[l], c = lvCount[l];
    for (int i = threadIdx.x; i < c; i += blockDim.x) {
      const int t = b + i;
      const int p = top.pre[t];
      const int lref = top.left[t], rref = top.right[t];
      const int lp = p + 1;
      const int rp = p + 1 + subtree_size(top, small, lref);
      if (lref >= 0)
        top.pre[lref] = lp;
      else
        small.base[~lref] = lp;
      if (rref >= 0)
        top.pre[rref] = rp;
      else
        small.base[~rref] = rp;
      if (p >= 0 && p < nodeCap)
        store_inner(nodes + p, (uint32_t)top.dim[t], (uint32_t)rp, top.cut[t]);
      else
        atomicOr(status + 1, 1);  // unreachable for a finished build
    }
    __syncthreads();
  }
}

template <typename T>
__global__ void k_copy_small(const Node<T>* scratch, SmallSegs<T> small, const int* nSmall, int* status,
                             Node<T>* nodes, int64_t nodeCap) {
  const int sid = blockIdx.x * blockDim.x + threadIdx.x;
  if (status[1] || sid >= *nSmall) return;
  const int base = small.base[sid];
  const Node<T>* src = scratch + 2 * (int64_t)small.start[sid];
  const int cnt = small.size[sid];
  if (base < 0 || base + (int64_t)cnt > nodeCap) {
    atomicOr(status + 1, 1);  // unreachable for a finished build
    return;
  }
  for (int i = 0; i < cnt; ++i) {
    Node<T> nd = src[i];
    if (!node_is_leaf(nd.meta)) nd.meta = make_meta(node_dim(nd.meta), (uint32_t)base + node_payload(nd.meta));
    nodes[base + i] = nd;
  }
}

// status[0] non-finite input (set by k_bounds_forest), [1] build did not
// finish (capacity exceeded or levels left over), [2] tallest tree's height,
// [3] top levels run. Runs before the numbering, which reads [1].
__global__ void k_forest_status(const LevelState* st, const int* counters, int* status) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  status[1] = (counters[3] || st->overflow || st->nseg > 0) ? 1 : 0;
  status[2] = counters[2];
  status[3] = st->nLevels;
}

// ---------------------------------------------------------------------------
// Host side.

// Stream-ordered scratch that is released when the owner goes out of scope.
struct Scratch {
  cudaStream_t stream;
  std::vector<void*> ptrs;
  explicit Scratch(cudaStream_t s) : stream(s) {}
  ~Scratch() {
    for (void* p : ptrs) scratch_free(p, stream);
  }
  template <typename V>
  cudaError_t get(V** out, int64_t count) {
    void* p = nullptr;
    const size_t bytes = (size_t)std::max<int64_t>(count, 1) * sizeof(V);
    cudaError_t e = scratch_alloc(&p, bytes, stream);
    if (e == cudaSuccess) ptrs.push_back(p);
    *out = static_cast<V*>(p);
    return e;
  }
};

template <typename T>
cudaError_t alloc_level(Scratch& sc, SegLevel<T>* L, int64_t cap) {
  cudaError_t e;
  if ((e = sc.get(&L->start, cap))) return e;
  if ((e = sc.get(&L->count, cap))) return e;
  if ((e = sc.get(&L->boxLo, cap * kMaxDim))) return e;
  if ((e = sc.get(&L->boxHi, cap * kMaxDim))) return e;
  if ((e = sc.get(&L->cutDim, cap))) return e;
  if ((e = sc.get(&L->mnK, cap))) return e;
  if ((e = sc.get(&L->mxK, cap))) return e;
  if ((e = sc.get(&L->cut, cap))) return e;
  if ((e = sc.get(&L->mode, cap))) return e;
  if ((e = sc.get(&L->lt, cap))) return e;
  if ((e = sc.get(&L->eq, cap))) return e;
  if ((e = sc.get(&L->leftCount, cap))) return e;
  if ((e = sc.get(&L->newLeft, cap))) return e;
  return sc.get(&L->newRight, cap);
}

template <typename T>
double host_key_to_double(typename KeyOf<T>::type k);
template <>
double host_key_to_double<float>(uint32_t k) {
  const uint32_t u = (k & 0x80000000u) ? (k & 0x7fffffffu) : ~k;
  float f;
  std::memcpy(&f, &u, 4);
  return (double)f;
}
template <>
double host_key_to_double<double>(unsigned long long k) {
  const unsigned long long u = (k & 0x8000000000000000ull) ? (k & 0x7fffffffffffffffull) : ~k;
  double f;
  std::memcpy(&f, &u, 8);
  return f;
}

// Per-dimension bounds; fails on NaN or infinite coordinates, for which
// the reference's split loop does not terminate (idealCutVal becomes NaN
// and leftCount 0, nabo/kdtree_cpu.cpp:180-190).
template <typename T, int D>
int compute_bounds(const Rec<T, D>* recs, int64_t n, int dim, cudaStream_t stream, Scratch& sc, double* lo,
                   double* hi) {
  using Key = typename KeyOf<T>::type;
  Key* keys;
  int* flag;
  NABO_CUDA_TRY(sc.get(&keys, 2 * kMaxDim));
  NABO_CUDA_TRY(sc.get(&flag, 1));
  NABO_CUDA_TRY(cudaMemsetAsync(flag, 0, sizeof(int), stream));
  k_init_keys<T><<<1, kMaxDim, 0, stream>>>(keys, keys + kMaxDim, dim);
  const int grid = (int)std::min<int64_t>(ceil_div(n, kBlock), 152 * 8);
  k_bounds<T, D><<<grid, kBlock, 0, stream>>>(recs, n, dim, keys, keys + kMaxDim, flag);
  NABO_CUDA_TRY(cudaGetLastError());
  Key h[2 * kMaxDim];
  int hflag = 0;
  NABO_CUDA_TRY(cudaMemcpyAsync(h, keys, sizeof(h), cudaMemcpyDeviceToHost, stream));
  NABO_CUDA_TRY(cudaMemcpyAsync(&hflag, flag, sizeof(int), cudaMemcpyDeviceToHost, stream));
  NABO_CUDA_TRY(cudaStreamSynchronize(stream));
  if (hflag) return set_error(kErrArgument, "Cloud has non-finite (NaN or infinite) coordinates");
  for (int d = 0; d < kMaxDim; ++d) {
    lo[d] = d < dim ? host_key_to_double<T>(h[d]) : 0.0;
    hi[d] = d < dim ? host_key_to_double<T>(h[kMaxDim + d]) : 0.0;
  }
  return kOk;
}

}  // namespace

template <typename T, int D>
int pack_cloud(const T* dCloud, int64_t n, int64_t stride, int dim, cudaStream_t stream, DeviceCloud* out) {
  Rec<T, D>* recs = nullptr;
  NABO_CUDA_TRY(cudaMalloc((void**)&recs, (size_t)n * sizeof(Rec<T, D>)));
  out->recs = recs;
  k_pack<T, D><<<ceil_div(n, kBlock), kBlock, 0, stream>>>(dCloud, n, stride, dim, recs);
  NABO_CUDA_TRY(cudaGetLastError());
  Scratch sc(stream);
  const int rc = compute_bounds<T, D>(recs, n, dim, stream, sc, out->lo, out->hi);
  if (rc != kOk) return rc;
  return kOk;
}

// Builds the trees of `nClouds` clouds stored back to back (cloud c =
// points [off[c], off[c+1]) of dCloud) into one record array and one node
// array: cloud c's tree is the pre-order range [nodeOffset[c],
// nodeOffset[c+1]), its points keep their index within the cloud.
// maxLevels < 0: the host runs levels until none is left (reads one int per
// level). maxLevels >= 0: exactly that many levels run with no host
// synchronisation at all, so the whole build can be captured in a CUDA
// graph; a tree needing more levels sets the overflow flag (f->status).
template <typename T, int D>
int build_forest(const T* dCloud, int64_t n, int64_t stride, int dim, unsigned bucketSize, const int64_t* dOff,
                 int nClouds, int maxLevels, cudaStream_t stream, ForestOut* f, int splitRule) {
  using Key = typename KeyOf<T>::type;
  const int N = (int)n;
  const bool hostDriven = maxLevels < 0;
  Scratch sc(stream);
  Rec<T, D>* recs = static_cast<Rec<T, D>*>(f->recs);
  // the median split works in two record arrays of its own (positions
  // padded to whole tiles) and leaves the final array to its scatter
  const bool median = splitRule == 1;
  const int64_t nPad = median ? (std::max<int64_t>(n, 1) + kTile - 1) / kTile * kTile : n;
  MedianBufs<T, D> mb = {};
  if (median) {
    for (int i = 0; i < 2; ++i) {
      NABO_CUDA_TRY(sc.get(&mb.rec[i], n));
      NABO_CUDA_TRY(sc.get(&mb.seg[i], nPad));
      NABO_CUDA_TRY(sc.get(&mb.val[i], nPad));
    }
  }
  Rec<T, D>* packed = median ? mb.rec[0] : recs;
  // per-position passes over contiguous block ranges: 8 blocks per SM
  int device = 0, sms = 0;
  NABO_CUDA_TRY(cudaGetDevice(&device));
  NABO_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
  const int rangeBlocks = std::max(1, std::min(ceil_div(std::max<int64_t>(n, 1), kBlock), 8 * std::max(sms, 1)));
  const int64_t rangeChunk = (int64_t)ceil_div(ceil_div(std::max<int64_t>(n, 1), rangeBlocks), kBlock) * kBlock;

  // records and per-cloud bounds in one pass
  Key* keys;
  NABO_CUDA_TRY(sc.get(&keys, 2 * (int64_t)nClouds * kMaxDim));
  NABO_CUDA_TRY(cudaMemsetAsync(f->status, 0, 4 * sizeof(int), stream));
  k_init_keys_forest<T><<<ceil_div(nClouds * kMaxDim, 256), 256, 0, stream>>>(keys, keys + nClouds * kMaxDim,
                                                                              nClouds);
  if (n > 0)
    k_pack_bounds<T, D><<<rangeBlocks, kBlock, 0, stream>>>(dCloud, n, stride, dim, dOff, nClouds, rangeChunk, packed,
                                                            median ? recs : nullptr, keys, keys + nClouds * kMaxDim,
                                                            f->status + 0);
  NABO_CUDA_TRY(cudaGetLastError());
  if (hostDriven) {
    int bad = 0;
    NABO_CUDA_TRY(cudaMemcpyAsync(&bad, f->status + 0, sizeof(int), cudaMemcpyDeviceToHost, stream));
    NABO_CUDA_TRY(cudaStreamSynchronize(stream));
    if (bad) return set_error(kErrArgument, "Cloud has non-finite (NaN or infinite) coordinates");
  }

  // working arrays
  int* segOf;
  int2* passTotal;
  int2* blockSums;
  int2* segFirst;
  int2* segLast;
  int* pairA;
  int* pairB;
  int* counters;
  int* lv;
  int* rootRef;
  int* rootSeg;
  LevelState* st;
  const int nb = ceil_div(n, kBlock);
  const int64_t pairCap = n + 1;
  const int64_t segCap = n / (kSmallMax + 1) + 2;
  const int64_t topCap = n + 1;
  const int64_t smallCap = n + nClouds + 1;
  // levels recorded for the numbering; a host-driven build grows the record
  // when a tree needs more (the split rule gives trees as tall as the cloud
  // is large on geometrically spaced coordinates)
  int lvCap = hostDriven ? 4096 : std::max(maxLevels, 1);
  T* val = nullptr;
  pairA = pairB = nullptr;
  if (median) {
    segOf = mb.seg[0];
  } else {
    NABO_CUDA_TRY(sc.get(&segOf, n));
    NABO_CUDA_TRY(sc.get(&val, n));
    NABO_CUDA_TRY(sc.get(&pairA, pairCap));
    NABO_CUDA_TRY(sc.get(&pairB, pairCap));
  }
  NABO_CUDA_TRY(sc.get(&passTotal, 1));
  NABO_CUDA_TRY(sc.get(&blockSums, nb));
  NABO_CUDA_TRY(sc.get(&segFirst, segCap));
  NABO_CUDA_TRY(sc.get(&segLast, segCap));
  NABO_CUDA_TRY(sc.get(&counters, 4));
  NABO_CUDA_TRY(sc.get(&lv, 2 * (int64_t)lvCap));
  NABO_CUDA_TRY(sc.get(&rootRef, nClouds));
  NABO_CUDA_TRY(sc.get(&rootSeg, nClouds));
  NABO_CUDA_TRY(sc.get(&st, 1));
  NABO_CUDA_TRY(cudaMemsetAsync(counters, 0, 4 * sizeof(int), stream));
  NABO_CUDA_TRY(cudaMemsetAsync(st, 0, sizeof(LevelState), stream));
  SegLevel<T> cur, nxt;
  NABO_CUDA_TRY(alloc_level(sc, &cur, segCap));
  NABO_CUDA_TRY(alloc_level(sc, &nxt, segCap));
  TopNodes<T> top;
  NABO_CUDA_TRY(sc.get(&top.dim, topCap));
  NABO_CUDA_TRY(sc.get(&top.cut, topCap));
  NABO_CUDA_TRY(sc.get(&top.left, topCap));
  NABO_CUDA_TRY(sc.get(&top.right, topCap));
  NABO_CUDA_TRY(sc.get(&top.size, topCap));
  NABO_CUDA_TRY(sc.get(&top.pre, topCap));
  SmallSegs<T> small;
  NABO_CUDA_TRY(sc.get(&small.start, smallCap));
  NABO_CUDA_TRY(sc.get(&small.count, smallCap));
  NABO_CUDA_TRY(sc.get(&small.depth, smallCap));
  NABO_CUDA_TRY(sc.get(&small.boxLo, smallCap * kMaxDim));
  NABO_CUDA_TRY(sc.get(&small.boxHi, smallCap * kMaxDim));
  NABO_CUDA_TRY(sc.get(&small.size, smallCap));
  NABO_CUDA_TRY(sc.get(&small.base, smallCap));

  k_forest_roots<T><<<ceil_div(nClouds, 128), 128, 0, stream>>>(
      dOff, nClouds, keys, keys + nClouds * kMaxDim, dim, cur, small, st, counters, rootRef, rootSeg,
      static_cast<T*>(f->rootLo), static_cast<T*>(f->rootHi));
  if (nPad > 0) {
    const int64_t segChunk = rangeChunk * ceil_div(nPad, rangeChunk * rangeBlocks);
    k_init_segof<T, D><<<ceil_div(nPad, segChunk), kBlock, 0, stream>>>(
        segOf, n, nPad, segChunk, dOff, nClouds, rootSeg, packed, cur.cutDim, median ? mb.val[0] : nullptr);
  }
  NABO_CUDA_TRY(cudaGetLastError());

  const int sg = ceil_div(segCap, 128);
  // per-position passes: a fixed grid of 8 blocks per SM looping over tiles
  // of kBlock positions; the two scan passes give each block a contiguous
  // run of `tiles` tiles
  const int grid = std::max(1, std::min(nb, 8 * std::max(sms, 1)));
  const int tiles = ceil_div(nb, grid);
  const int scanBlocks = ceil_div(nb, tiles);
  // median split: as many blocks as are resident at once, each scanning a
  // contiguous run of mTiles tiles of kTile positions
  const int mTilesTotal = (int)(nPad / kTile);
  int mOcc = 0;
  if (median)
    NABO_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&mOcc, median_scatter<T, D>(), kBlock, 0));
  const int mGrid = std::max(1, std::min(mTilesTotal, std::max(mOcc, 1) * std::max(sms, 1)));
  const int mTiles = ceil_div(mTilesTotal, mGrid);
  const int mBlocks = ceil_div(mTilesTotal, mTiles);
  for (int level = 0; hostDriven || level < maxLevels; ++level) {
    if (hostDriven) {
      int nseg = 0;
      NABO_CUDA_TRY(cudaMemcpyAsync(&nseg, &st->nseg, sizeof(int), cudaMemcpyDeviceToHost, stream));
      NABO_CUDA_TRY(cudaStreamSynchronize(stream));
      if (nseg == 0) break;
      if (level >= lvCap) {
        if (level >= N) return set_error(kErrInternal, "kd-tree build: more levels than points");
        const int grown = (int)std::min<int64_t>(2 * (int64_t)lvCap, (int64_t)N + 1);
        int* lv2 = nullptr;
        NABO_CUDA_TRY(sc.get(&lv2, 2 * (int64_t)grown));
        NABO_CUDA_TRY(cudaMemcpyAsync(lv2, lv, (size_t)lvCap * sizeof(int), cudaMemcpyDeviceToDevice, stream));
        NABO_CUDA_TRY(cudaMemcpyAsync(lv2 + grown, lv + lvCap, (size_t)lvCap * sizeof(int),
                                      cudaMemcpyDeviceToDevice, stream));
        lv = lv2;
        lvCap = grown;
      }
    }
    if (median) {
      NABO_CUDA_TRY(launch_pdl(k_median_cut<T, D>, sg, 128, 0, stream, cur, st, mb));
      NABO_CUDA_TRY(launch_pdl(k_median_sums<T, D>, mBlocks, kBlock, 0, stream, mb, nPad, cur, mTiles, blockSums,
                               segFirst, segLast, st));
      NABO_CUDA_TRY(launch_pdl(k_scan_block_sums, 1, kBlock, 0, stream, blockSums, mBlocks, passTotal, st));
      NABO_CUDA_TRY(launch_pdl(k_median_split<T>, sg, 128, 0, stream, cur, nxt, st, top, small, counters, dim,
                               (int)segCap, (int)smallCap, (int)topCap, (const int2*)blockSums,
                               (const int2*)segFirst, (const int2*)segLast, mTiles * kTile));
      NABO_CUDA_TRY(launch_pdl(median_scatter<T, D>(), mBlocks, kBlock, 0, stream, mb, recs, nPad, cur, nxt, mTiles,
                               (const int2*)blockSums, st));
      NABO_CUDA_TRY(launch_pdl(k_advance, 1, 1, 0, stream, st, counters, lv, lv + lvCap, lvCap));
      std::swap(cur, nxt);
      continue;
    }
    const int remap = level > 0 ? 1 : 0;
    NABO_CUDA_TRY(launch_pdl(k_prepare<T>, sg, 128, 0, stream, cur, st, dim));
    NABO_CUDA_TRY(launch_pdl(k_minmax<T, D>, grid, kBlock, 0, stream, recs, segOf, N, cur, nxt, remap, st, val));
    NABO_CUDA_TRY(launch_pdl(k_cut<T>, sg, 128, 0, stream, cur, st, (const T*)val, splitRule));
    NABO_CUDA_TRY(launch_pdl(k_count<T>, grid, kBlock, 0, stream, val, segOf, N, cur, st));
    for (int pass = 1; pass <= 2; ++pass) {
      NABO_CUDA_TRY(launch_pdl(k_flag_sums<T>, scanBlocks, kBlock, 0, stream, val, segOf, N, cur, pass, tiles,
                                 blockSums, segFirst, segLast, st));
      NABO_CUDA_TRY(launch_pdl(k_scan_block_sums, 1, kBlock, 0, stream, blockSums, scanBlocks, passTotal, st));
      NABO_CUDA_TRY(launch_pdl(k_flag_pairs<T>, scanBlocks, kBlock, 0, stream, val, segOf, N, cur, pass, tiles,
                                 blockSums, segFirst, segLast, pairA, pairB, (int)pairCap, st));
      NABO_CUDA_TRY(launch_pdl(k_swap<T, D>, grid, kBlock, 0, stream, recs, val, pairA, pairB, passTotal,
                                 (int)pairCap, N, counters + 3));
    }
    NABO_CUDA_TRY(launch_pdl(k_finalize<T>, sg, 128, 0, stream, cur, nxt, st, top, small, counters, dim,
                               (int)segCap, (int)smallCap, (int)topCap));
    NABO_CUDA_TRY(launch_pdl(k_advance, 1, 1, 0, stream, st, counters, lv, lv + lvCap, lvCap));
    std::swap(cur, nxt);
  }

  if (median) k_median_flush<T, D><<<grid, kBlock, 0, stream>>>(mb, recs, n, st);

  // small segments (their count is read on the device: grid for the most)
  Node<T>* scratchNodes;
  NABO_CUDA_TRY(sc.get(&scratchNodes, 2 * n));
  SmallStack<T> stk;
  NABO_CUDA_TRY(sc.get(&stk.start, n));
  NABO_CUDA_TRY(sc.get(&stk.count, n));
  NABO_CUDA_TRY(sc.get(&stk.parent, n));
  NABO_CUDA_TRY(sc.get(&stk.depth, n));
  NABO_CUDA_TRY(sc.get(&stk.boxLo, n * kMaxDim));
  NABO_CUDA_TRY(sc.get(&stk.boxHi, n * kMaxDim));
  int nSmallHost = (int)smallCap;
  if (hostDriven) {
    NABO_CUDA_TRY(cudaMemcpyAsync(&nSmallHost, counters + 1, sizeof(int), cudaMemcpyDeviceToHost, stream));
    NABO_CUDA_TRY(cudaStreamSynchronize(stream));
  }
  {
    const int wpb = small_warps_per_block<T, D>();
    const size_t smem = (size_t)wpb * kSmallMax * (sizeof(Rec<T, D>) + sizeof(int));
    // one wave of resident blocks, its warps taking segments from a counter
    int occ = 0;
    NABO_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_small<T, D>, 32 * wpb, smem));
    const int smallGrid =
        std::max(1, std::min(ceil_div(std::max(nSmallHost, 1), wpb), std::max(occ, 1) * std::max(sms, 1)));
    int* nextSeg;
    NABO_CUDA_TRY(sc.get(&nextSeg, 1));
    NABO_CUDA_TRY(cudaMemsetAsync(nextSeg, 0, sizeof(int), stream));
    k_small<T, D><<<smallGrid, 32 * wpb, smem, stream>>>(recs, small, counters + 1, scratchNodes, stk, dim,
                                                         bucketSize, counters, splitRule, nextSeg);
  }
  NABO_CUDA_TRY(cudaGetLastError());
  Node<T>* nodes = static_cast<Node<T>*>(f->nodes);
  k_forest_status<<<1, 1, 0, stream>>>(st, counters, f->status);
  k_renumber<T><<<1, 1024, 0, stream>>>(top, small, lv, lv + lvCap, st, rootRef, dOff, nClouds, f->status, nodes,
                                        f->nodeCap, f->nodeOffset);
  k_copy_small<T><<<ceil_div(nSmallHost, 128), 128, 0, stream>>>(scratchNodes, small, counters + 1, f->status,
                                                                 nodes, f->nodeCap);
  NABO_CUDA_TRY(cudaGetLastError());
  if (hostDriven) {
    int hs[4];
    NABO_CUDA_TRY(cudaMemcpyAsync(hs, f->status, 4 * sizeof(int), cudaMemcpyDeviceToHost, stream));
    NABO_CUDA_TRY(cudaStreamSynchronize(stream));
    if (hs[1]) return set_error(kErrInternal, "kd-tree build: capacity exceeded");
  }
  return kOk;
}

template <typename T, int D>
int build_kdtree(const T* dCloud, int64_t n, int64_t stride, int dim, unsigned bucketSize, cudaStream_t stream,
                 DeviceCloud* out, double* rootMin, double* rootMax, BuildStats* stats, int splitRule) {
  Scratch sc(stream);
  ForestOut f;
  Rec<T, D>* recs = nullptr;
  Node<T>* nodes = nullptr;
  NABO_CUDA_TRY(cudaMalloc((void**)&recs, (size_t)n * sizeof(Rec<T, D>)));
  out->recs = recs;  // owned by the caller from here on
  // Upper bound on the node count: every leaf holds at least one point.
  const int64_t nodeCap = 2 * n;
  NABO_CUDA_TRY(cudaMalloc((void**)&nodes, (size_t)nodeCap * sizeof(Node<T>)));
  out->nodes = nodes;
  int64_t* off;
  T* rootBox;
  NABO_CUDA_TRY(sc.get(&off, 2));
  NABO_CUDA_TRY(sc.get(&f.nodeOffset, 2));
  NABO_CUDA_TRY(sc.get(&f.status, 4));
  NABO_CUDA_TRY(sc.get(&rootBox, 2 * kMaxDim));
  const int64_t hoff[2] = {0, n};
  NABO_CUDA_TRY(cudaMemcpyAsync(off, hoff, sizeof(hoff), cudaMemcpyHostToDevice, stream));
  f.recs = recs;
  f.nodes = nodes;
  f.nodeCap = nodeCap;
  f.rootLo = rootBox;
  f.rootHi = rootBox + kMaxDim;
  const int rc = build_forest<T, D>(dCloud, n, stride, dim, bucketSize, off, 1, -1, stream, &f, splitRule);
  if (rc != kOk) return rc;
  int64_t hno[2];
  int hs[4];
  T hbox[2 * kMaxDim];
  NABO_CUDA_TRY(cudaMemcpyAsync(hno, f.nodeOffset, sizeof(hno), cudaMemcpyDeviceToHost, stream));
  NABO_CUDA_TRY(cudaMemcpyAsync(hs, f.status, sizeof(hs), cudaMemcpyDeviceToHost, stream));
  NABO_CUDA_TRY(cudaMemcpyAsync(hbox, rootBox, sizeof(hbox), cudaMemcpyDeviceToHost, stream));
  NABO_CUDA_TRY(cudaStreamSynchronize(stream));
  const int64_t total = hno[1];
  if (hs[1]) return set_error(kErrInternal, "kd-tree build: internal check failed (capacity or pairing)");
  if (total <= 0 || total > nodeCap) return set_error(kErrInternal, "kd-tree build: inconsistent node count");
  if (total - 1 > (int64_t)kMaxNodeIndex)
    return set_error(kErrUnsupported, "kd-tree build: the tree has more nodes than the device layout indexes");
  out->nodeCount = total;
  out->height = hs[2];
  for (int d = 0; d < kMaxDim; ++d) {
    rootMin[d] = d < dim ? (double)hbox[d] : 0.0;
    rootMax[d] = d < dim ? (double)hbox[kMaxDim + d] : 0.0;
    // true bounds for query ordering: the root box's max is the true max
    // unless the quirk lifted it to numeric_limits<T>::min()
    out->lo[d] = rootMin[d];
    out->hi[d] = rootMax[d];
  }
  if (stats) {
    stats->topLevels = hs[3];
    stats->topNodes = 0;
    stats->smallSegments = 0;
  }
  return kOk;
}

namespace {

// Float copies of double records (same order), for the search's float
// pre-filter of leaf points, and the largest coordinate magnitude over the
// searched dimensions (as float bits, atomicMax: non-negative floats order
// like their bit patterns). Coordinates beyond the float range become inf,
// which switches the pre-filter off.
template <int D>
__global__ void k_narrow(const Rec<double, D>* __restrict__ recs, int64_t n, int dim, Rec<float, D>* out,
                         unsigned* coordMaxBits) {
  const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  float m = 0.0f;
  if (p < n) {
    Rec<double, D> r;
    load_rec(recs, p, r);
    Rec<float, D> f;
#pragma unroll
    for (int c = 0; c < RecSize<float, D>::chunks; ++c) f.v[c] = make_uint4(0u, 0u, 0u, 0u);
#pragma unroll
    for (int d = 0; d < D; ++d) {
      f.p.c[d] = (float)r.p.c[d];
      if (d < dim) m = fmaxf(m, fabsf(f.p.c[d]));
    }
    f.p.idx = r.p.idx;
    out[p] = f;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(kFull, m, o));
  if ((threadIdx.x & 31) == 0 && m > 0.0f) atomicMax(coordMaxBits, __float_as_uint(m));
}

}  // namespace

template <int D>
int narrow_records(const void* recs, int64_t n, int dim, void* recs32, float* coordMax, cudaStream_t stream) {
  NABO_CUDA_TRY(cudaMemsetAsync(coordMax, 0, sizeof(float), stream));
  if (n > 0)
    k_narrow<D><<<ceil_div(n, kBlock), kBlock, 0, stream>>>(static_cast<const Rec<double, D>*>(recs), n, dim,
                                                            static_cast<Rec<float, D>*>(recs32),
                                                            reinterpret_cast<unsigned*>(coordMax));
  NABO_CUDA_TRY(cudaGetLastError());
  return kOk;
}
template int narrow_records<2>(const void*, int64_t, int, void*, float*, cudaStream_t);
template int narrow_records<3>(const void*, int64_t, int, void*, float*, cudaStream_t);
template int narrow_records<4>(const void*, int64_t, int, void*, float*, cudaStream_t);
template int narrow_records<8>(const void*, int64_t, int, void*, float*, cudaStream_t);
template int narrow_records<16>(const void*, int64_t, int, void*, float*, cudaStream_t);

#define NABO_BUILD_INSTANTIATE(T, D)                                                                          \
  template int build_kdtree<T, D>(const T*, int64_t, int64_t, int, unsigned, cudaStream_t, DeviceCloud*,      \
                                  double*, double*, BuildStats*, int);                                        \
  template int build_forest<T, D>(const T*, int64_t, int64_t, int, unsigned, const int64_t*, int, int,        \
                                  cudaStream_t, ForestOut*, int);                                             \
  template int pack_cloud<T, D>(const T*, int64_t, int64_t, int, cudaStream_t, DeviceCloud*);

NABO_BUILD_INSTANTIATE(float, 2)
NABO_BUILD_INSTANTIATE(float, 3)
NABO_BUILD_INSTANTIATE(float, 4)
NABO_BUILD_INSTANTIATE(float, 8)
NABO_BUILD_INSTANTIATE(float, 16)
NABO_BUILD_INSTANTIATE(double, 2)
NABO_BUILD_INSTANTIATE(double, 3)
NABO_BUILD_INSTANTIATE(double, 4)
NABO_BUILD_INSTANTIATE(double, 8)
NABO_BUILD_INSTANTIATE(double, 16)

}  // namespace nabo_gb300
