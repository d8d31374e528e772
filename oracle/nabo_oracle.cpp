// nabo_oracle.cpp -- TEST INFRASTRUCTURE ONLY.
//
// CPU restatement of libnabo 1.1.2's k-nearest-neighbour path, used by the
// tests and by bench.py's CPU-baseline leg as the checker. Nothing in the
// product (libnabo_gb300/) links, loads or calls this file.
//
// The reference itself cannot be compiled in this environment (its public
// header includes Eigen/Core and Eigen is not installed), so this file
// restates its algorithm in plain C++17 + OpenMP with raw column-major
// arrays. Every function cites the reference file:line it follows.
//
// Two search modes are provided:
//   MODE_REFERENCE  the reference's semantics exactly: strict `dist < head`
//                   acceptance, far-child visit iff `rd*(1+eps)^2 < head`,
//                   heaps IndexHeapBruteForceVector (linear) or IndexHeapSTL
//                   (std::push_heap/pop_heap/sort_heap), so ties at the k-th
//                   place are decided by visit order.
//   MODE_CANONICAL  identical traversal and arithmetic, but the heap is
//                   ordered by the pair (dist2, index) and the far-child test
//                   is `rd*(1+eps)^2 <= head` so that ties are always broken
//                   towards the lower point index, independent of visit
//                   order. This is the rule the CUDA kernels implement; the
//                   tests check that both modes agree wherever no exact
//                   distance tie exists.
//
// Floating point: compiled with -ffp-contract=off so that every +,-,* is
// rounded separately, as written in the reference's loops
// (nabo/kdtree_cpu.cpp:383-391, :415, :433). The squared distance is the
// sequential sum over d = 0..dim-1.

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <limits>
#include <string>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

thread_local std::string g_err;

enum { MODE_REFERENCE = 0, MODE_CANONICAL = 1 };
enum { HEAP_LINEAR = 0, HEAP_STL = 1 };
enum { ALLOW_SELF_MATCH = 1, SORT_RESULTS = 2 };
enum { TOUCH_STATISTICS = 1 };

// nabo/kdtree_cpu.cpp:60-70
uint32_t storageBitCount(uint32_t v) {
  for (uint32_t i = 0; i < 64; ++i) {
    if (v == 0) return i;
    v >>= 1;
  }
  return 64;
}

// nabo/index_heap.h:263-369 (IndexHeapBruteForceVector): sorted ascending
// array of k entries initialised to (-1, +inf); head is the last entry;
// insertion shifts entries while data[i-1].value > value.
template <typename T>
struct LinearHeap {
  std::vector<int> idx;
  std::vector<T> val;
  size_t km1;
  explicit LinearHeap(size_t k) : idx(k, -1), val(k, std::numeric_limits<T>::infinity()), km1(k - 1) {}
  void reset() {
    std::fill(idx.begin(), idx.end(), -1);
    std::fill(val.begin(), val.end(), std::numeric_limits<T>::infinity());
  }
  T headValue() const { return val[km1]; }
  bool accepts(int /*i*/, T d) const { return d < val[km1]; }
  void replaceHead(int index, T value) {
    size_t i;
    for (i = km1; i > 0; --i) {
      if (val[i - 1] > value) {
        val[i] = val[i - 1];
        idx[i] = idx[i - 1];
      } else {
        break;
      }
    }
    val[i] = value;
    idx[i] = index;
  }
  void sort() {}
  void getData(int* oi, T* od) const {
    for (size_t i = 0; i <= km1; ++i) {
      oi[i] = idx[i];
      od[i] = val[i];
    }
  }
};

// nabo/index_heap.h:51-165 (IndexHeapSTL): binary max-heap on value built
// with the standard heap algorithms; starts with one (-1, +inf) sentinel.
template <typename T>
struct STLHeap {
  struct Entry {
    int index;
    T value;
    Entry(int i, T v) : index(i), value(v) {}
    friend bool operator<(const Entry& a, const Entry& b) { return a.value < b.value; }
  };
  std::vector<Entry> data;
  size_t nb;
  explicit STLHeap(size_t k) : data(1, Entry(-1, std::numeric_limits<T>::infinity())), nb(k) { data.reserve(k); }
  void reset() {
    data.clear();
    data.push_back(Entry(-1, std::numeric_limits<T>::infinity()));
  }
  T headValue() const { return data.front().value; }
  bool accepts(int /*i*/, T d) const { return d < data.front().value; }
  void replaceHead(int index, T value) {
    if (data.size() == nb) {
      std::pop_heap(data.begin(), data.end());
      data.back() = Entry(index, value);
    } else {
      data.push_back(Entry(index, value));
    }
    std::push_heap(data.begin(), data.end());
  }
  void sort() { std::sort_heap(data.begin(), data.end()); }
  void getData(int* oi, T* od) const {
    size_t i = 0;
    for (; i < data.size(); ++i) {
      oi[i] = data[i].index;
      od[i] = data[i].value;
    }
    for (; i < nb; ++i) {
      oi[i] = -1;
      od[i] = std::numeric_limits<T>::infinity();
    }
  }
};

// Canonical heap: the LinearHeap layout, but entries are ordered by the
// pair (value, index), so an entry equal in value to the head replaces it
// when its index is lower. The result is the k smallest pairs, which does
// not depend on the order in which points are offered.
template <typename T>
struct CanonicalHeap {
  std::vector<int> idx;
  std::vector<T> val;
  size_t km1;
  explicit CanonicalHeap(size_t k) : idx(k, -1), val(k, std::numeric_limits<T>::infinity()), km1(k - 1) {}
  void reset() {
    std::fill(idx.begin(), idx.end(), -1);
    std::fill(val.begin(), val.end(), std::numeric_limits<T>::infinity());
  }
  static bool greater(T da, int ia, T db, int ib) { return da > db || (da == db && ia > ib); }
  T headValue() const { return val[km1]; }
  bool accepts(int i, T d) const { return greater(val[km1], idx[km1], d, i); }
  void replaceHead(int index, T value) {
    size_t i;
    for (i = km1; i > 0; --i) {
      if (greater(val[i - 1], idx[i - 1], value, index)) {
        val[i] = val[i - 1];
        idx[i] = idx[i - 1];
      } else {
        break;
      }
    }
    val[i] = value;
    idx[i] = index;
  }
  void sort() {}
  void getData(int* oi, T* od) const {
    for (size_t i = 0; i <= km1; ++i) {
      oi[i] = idx[i];
      od[i] = val[i];
    }
  }
};

template <typename T>
struct Tree {
  struct Node {
    int32_t cutDim;  // -1 for a leaf
    T cutVal;
    uint32_t right;        // pre-order index of the right child (inner)
    uint32_t bucketStart;  // leaf: first entry in `buckets`
    uint32_t bucketCount;  // leaf: number of entries
  };
  const T* cloud = nullptr;  // dim x n, column stride `stride`
  std::vector<T> cloudCopy;
  int64_t n = 0;
  int64_t stride = 0;
  int dim = 0;
  unsigned bucketSize = 8;
  std::vector<T> minBound, maxBound;
  std::vector<Node> nodes;
  std::vector<int32_t> buckets;
  uint32_t height = 0;  // max number of inner nodes on a root-to-leaf path

  T coeff(int d, int64_t i) const { return cloud[i * stride + d]; }

  // nabo/kdtree_cpu.cpp:93-107
  std::pair<T, T> getBounds(const int32_t* first, int count, int d) const {
    T minVal = std::numeric_limits<T>::max();
    T maxVal = std::numeric_limits<T>::lowest();
    for (int i = 0; i < count; ++i) {
      const T v = coeff(d, first[i]);
      minVal = std::min(v, minVal);
      maxVal = std::max(v, maxVal);
    }
    return std::make_pair(minVal, maxVal);
  }

  // nabo/kdtree_cpu.cpp:109-225
  uint32_t buildNodes(int32_t* first, int count, std::vector<T> minValues, std::vector<T> maxValues, uint32_t depth) {
    const uint32_t pos = (uint32_t)nodes.size();
    if (count <= (int)bucketSize) {
      Node nd;
      nd.cutDim = -1;
      nd.cutVal = 0;
      nd.right = 0;
      nd.bucketStart = (uint32_t)buckets.size();
      nd.bucketCount = (uint32_t)count;
      for (int i = 0; i < count; ++i) buckets.push_back(first[i]);
      nodes.push_back(nd);
      if (depth > height) height = depth;
      return pos;
    }
    // argMax of the box extents (nabo/kdtree_cpu.cpp:76-90, :134)
    int cutDim = 0;
    {
      T maxVal(0);
      for (int d = 0; d < dim; ++d) {
        const T ext = maxValues[d] - minValues[d];
        if (ext > maxVal) {
          maxVal = ext;
          cutDim = d;
        }
      }
    }
    const T idealCutVal = (maxValues[cutDim] + minValues[cutDim]) / 2;
    const std::pair<T, T> mm = getBounds(first, count, cutDim);
    T cutVal;
    if (idealCutVal < mm.first)
      cutVal = mm.first;
    else if (idealCutVal > mm.second)
      cutVal = mm.second;
    else
      cutVal = idealCutVal;

    // two-pass partition, nabo/kdtree_cpu.cpp:149-177
    int l = 0;
    int r = count - 1;
    for (;;) {
      while (l < count && coeff(cutDim, first[l]) < cutVal) ++l;
      while (r >= 0 && coeff(cutDim, first[r]) >= cutVal) --r;
      if (l > r) break;
      std::swap(first[l], first[r]);
      ++l;
      --r;
    }
    const int br1 = l;
    r = count - 1;
    for (;;) {
      while (l < count && coeff(cutDim, first[l]) <= cutVal) ++l;
      while (r >= br1 && coeff(cutDim, first[r]) > cutVal) --r;
      if (l > r) break;
      std::swap(first[l], first[r]);
      ++l;
      --r;
    }
    const int br2 = l;

    // nabo/kdtree_cpu.cpp:180-190
    int leftCount;
    if (idealCutVal < mm.first)
      leftCount = 1;
    else if (idealCutVal > mm.second)
      leftCount = count - 1;
    else if (br1 > count / 2)
      leftCount = br1;
    else if (br2 < count / 2)
      leftCount = br2;
    else
      leftCount = count / 2;

    std::vector<T> leftMax(maxValues);
    leftMax[cutDim] = cutVal;
    std::vector<T> rightMin(minValues);
    rightMin[cutDim] = cutVal;

    Node nd;
    nd.cutDim = cutDim;
    nd.cutVal = cutVal;
    nd.right = 0;
    nd.bucketStart = 0;
    nd.bucketCount = 0;
    nodes.push_back(nd);
    buildNodes(first, leftCount, minValues, leftMax, depth + 1);
    const uint32_t rightChild = buildNodes(first + leftCount, count - leftCount, rightMin, maxValues, depth + 1);
    nodes[pos].right = rightChild;
    return pos;
  }
};

template <typename T>
bool check_create(int rows, int64_t n, int dimIn, unsigned bucketSize, bool isTree, int* dimOut) {
  // nabo/nabo.cpp:137-138 (create), :69-80 (base ctor), nabo/kdtree_cpu.cpp:234-251
  if (dimIn <= 0) {
    g_err = "Your space must have at least one dimension";
    return false;
  }
  const int dim = std::min(dimIn, rows);
  if (n == 0) {
    g_err = "Cloud has no points";
    return false;
  }
  if (rows == 0) {
    g_err = "Cloud has 0 dimensions";
    return false;
  }
  if (isTree) {
    if (bucketSize < 2) {
      g_err = "Requested bucket size " + std::to_string(bucketSize) + ", but must be larger than 2";
      return false;
    }
    if (n > (int64_t)bucketSize) {
      const uint32_t dimBitCount = storageBitCount((uint32_t)dim);
      const uint64_t maxNodeCount = (0x1ULL << (32 - dimBitCount)) - 1;
      const uint64_t estimatedNodeCount = (uint64_t)n / (bucketSize / 2);
      if (estimatedNodeCount > maxNodeCount) {
        g_err = "Cloud has a risk to have more nodes (" + std::to_string(estimatedNodeCount) +
                ") than the kd-tree allows (" + std::to_string(maxNodeCount) +
                "). The kd-tree has " + std::to_string(dimBitCount) + " bits for dimensions and " +
                std::to_string(32 - dimBitCount) + " bits for node indices";
        return false;
      }
    }
  }
  *dimOut = dim;
  return true;
}

// nabo/kdtree_cpu.cpp:227-272 (constructor)
template <typename T>
Tree<T>* build_tree(const T* cloud, int rows, int64_t n, int64_t stride, int dimIn, unsigned bucketSize) {
  int dim = 0;
  if (!check_create<T>(rows, n, dimIn, bucketSize, true, &dim)) return nullptr;
  Tree<T>* t = new Tree<T>();
  t->cloudCopy.assign(cloud, cloud + (size_t)((n - 1) * stride + rows));
  t->cloud = t->cloudCopy.data();
  t->n = n;
  t->stride = stride;
  t->dim = dim;
  t->bucketSize = bucketSize;
  // base ctor bounds initialisation, nabo/nabo.cpp:73-74 (note: max bound
  // starts at numeric_limits<T>::min(), the smallest positive normal)
  t->minBound.assign(dim, std::numeric_limits<T>::max());
  t->maxBound.assign(dim, std::numeric_limits<T>::min());
  if (n <= (int64_t)bucketSize) {
    // single-bucket tree, nabo/kdtree_cpu.cpp:236-243 (bounds are not computed)
    typename Tree<T>::Node nd;
    nd.cutDim = -1;
    nd.cutVal = 0;
    nd.right = 0;
    nd.bucketStart = 0;
    nd.bucketCount = (uint32_t)n;
    for (int64_t i = 0; i < n; ++i) t->buckets.push_back((int32_t)i);
    t->nodes.push_back(nd);
    return t;
  }
  std::vector<int32_t> buildPoints((size_t)n);
  for (int64_t i = 0; i < n; ++i) {
    buildPoints[(size_t)i] = (int32_t)i;
    for (int d = 0; d < dim; ++d) {
      const T v = t->coeff(d, i);
      t->minBound[d] = std::min(t->minBound[d], v);
      t->maxBound[d] = std::max(t->maxBound[d], v);
    }
  }
  t->buildNodes(buildPoints.data(), (int)n, t->minBound, t->maxBound, 0);
  return t;
}

template <typename T, int MODE, typename Heap, bool SELF, bool STATS>
struct Searcher {
  const Tree<T>& t;
  const T* q;
  Heap& heap;
  std::vector<T>& off;
  T maxError2, maxRadius2;

  // nabo/kdtree_cpu.cpp:367-447 (recurseKnn)
  unsigned long recurse(uint32_t n, T rd) {
    const typename Tree<T>::Node& node = t.nodes[n];
    if (node.cutDim < 0) {
      const int32_t* b = &t.buckets[node.bucketStart];
      for (uint32_t i = 0; i < node.bucketCount; ++i) {
        const int32_t index = b[i];
        T dist(0);
        for (int d = 0; d < t.dim; ++d) {
          const T diff = q[d] - t.coeff(d, index);
          dist += diff * diff;
        }
        if ((dist <= maxRadius2) && heap.accepts(index, dist) &&
            (SELF || (dist > std::numeric_limits<T>::epsilon())))
          heap.replaceHead(index, dist);
      }
      return (unsigned long)node.bucketCount;
    }
    const int cd = node.cutDim;
    unsigned long visited = 0;
    T& offcd = off[cd];
    const T old_off = offcd;
    const T new_off = q[cd] - node.cutVal;
    const uint32_t left = n + 1, right = node.right;
    const uint32_t nearN = new_off > 0 ? right : left;
    const uint32_t farN = new_off > 0 ? left : right;
    visited += recurse(nearN, rd);
    rd += -old_off * old_off + new_off * new_off;
    const T lhs = rd * maxError2;
    const bool visitFar = (MODE == MODE_REFERENCE) ? (lhs < heap.headValue()) : (lhs <= heap.headValue());
    if ((rd <= maxRadius2) && visitFar) {
      offcd = new_off;
      visited += recurse(farN, rd);
      offcd = old_off;
    }
    return STATS ? visited : 0;
  }
};

// nabo/kdtree_cpu.cpp:274-365 (knn, both overloads, and onePointKnn)
template <typename T, int MODE, typename Heap>
unsigned long tree_knn_impl(const Tree<T>& t, const T* query, int64_t nq, int64_t qStride, int k, T epsilon,
                            unsigned flags, bool stats, T maxRadius, const T* maxRadii, int32_t* outIdx, T* outD2) {
  const bool allowSelf = flags & ALLOW_SELF_MATCH;
  const bool sortResults = flags & SORT_RESULTS;
  const T maxError2 = (1 + epsilon) * (1 + epsilon);
  unsigned long touched = 0;
#pragma omp parallel
  {
    Heap heap((size_t)k);
    std::vector<T> off((size_t)t.dim, 0);
#pragma omp for reduction(+ : touched) schedule(guided, 32)
    for (int64_t i = 0; i < nq; ++i) {
      const T r = maxRadii ? maxRadii[i] : maxRadius;
      const T maxRadius2 = r * r;
      std::fill(off.begin(), off.end(), T(0));
      heap.reset();
      const T* q = query + i * qStride;
      unsigned long c = 0;
      if (allowSelf) {
        if (stats) {
          Searcher<T, MODE, Heap, true, true> s{t, q, heap, off, maxError2, maxRadius2};
          c = s.recurse(0, 0);
        } else {
          Searcher<T, MODE, Heap, true, false> s{t, q, heap, off, maxError2, maxRadius2};
          s.recurse(0, 0);
        }
      } else {
        if (stats) {
          Searcher<T, MODE, Heap, false, true> s{t, q, heap, off, maxError2, maxRadius2};
          c = s.recurse(0, 0);
        } else {
          Searcher<T, MODE, Heap, false, false> s{t, q, heap, off, maxError2, maxRadius2};
          s.recurse(0, 0);
        }
      }
      if (sortResults) heap.sort();
      heap.getData(outIdx + i * k, outD2 + i * k);
      touched += c;
    }
  }
  return touched;
}

// nabo/nabo.cpp:102-131 (checkSizesKnn). Output matrices are always k x nq
// here, so only the cloud-size, query-dimension, radii and flag checks apply.
bool check_knn(int64_t cloudCols, int dim, int qRows, int k, unsigned flags, int64_t nRadii, int64_t nq) {
  const bool allowSelf = flags & ALLOW_SELF_MATCH;
  if (allowSelf) {
    if (k > cloudCols) {
      g_err = "Requesting more points (" + std::to_string(k) + ") than available in cloud (" +
              std::to_string(cloudCols) + ")";
      return false;
    }
  } else {
    if (k > cloudCols - 1) {
      g_err = "Requesting more points (" + std::to_string(k) + ") than available in cloud minus 1 (" +
              std::to_string(cloudCols - 1) + ") (as self match is forbidden)";
      return false;
    }
  }
  if (qRows < dim) {
    g_err = "Query has less dimensions (" + std::to_string(qRows) + ") than requested for cloud (" +
            std::to_string(dim) + ")";
    return false;
  }
  if (nRadii >= 0 && nRadii != nq) {
    g_err = "Maximum radii vector has not the same length (" + std::to_string(nRadii) +
            ") than query has columns (" + std::to_string(k) + ")";
    return false;
  }
  const unsigned maxFlags = ALLOW_SELF_MATCH | SORT_RESULTS;
  if (flags > maxFlags) {
    g_err = "OR-ed value of option flags (" + std::to_string(flags) + ") is larger than maximal valid value (" +
            std::to_string(maxFlags) + ")";
    return false;
  }
  return true;
}

template <typename T>
int tree_knn(const Tree<T>* t, const T* query, int qRows, int64_t nq, int64_t qStride, int k, T eps, unsigned flags,
             unsigned creationFlags, T maxRadius, const T* maxRadii, int mode, int heap, int32_t* outIdx, T* outD2,
             uint64_t* touched) {
  if (!check_knn(t->n, t->dim, qRows, k, flags, maxRadii ? nq : -1, nq)) return 1;
  if (k <= 0) {
    if (touched) *touched = 0;
    return 0;
  }
  const bool stats = creationFlags & TOUCH_STATISTICS;
  unsigned long c = 0;
  if (mode == MODE_CANONICAL)
    c = tree_knn_impl<T, MODE_CANONICAL, CanonicalHeap<T>>(*t, query, nq, qStride, k, eps, flags, stats, maxRadius,
                                                           maxRadii, outIdx, outD2);
  else if (heap == HEAP_STL)
    c = tree_knn_impl<T, MODE_REFERENCE, STLHeap<T>>(*t, query, nq, qStride, k, eps, flags, stats, maxRadius,
                                                     maxRadii, outIdx, outD2);
  else
    c = tree_knn_impl<T, MODE_REFERENCE, LinearHeap<T>>(*t, query, nq, qStride, k, eps, flags, stats, maxRadius,
                                                        maxRadii, outIdx, outD2);
  if (touched) *touched = stats ? c : 0;
  return 0;
}

// nabo/brute_force_cpu.cpp:63-103. The reference computes dist2 with Eigen's
// squaredNorm (nabo/nabo_private.h:64-68), whose summation order is Eigen's
// own; this restatement uses the sequential sum of the kd-tree leaf loop.
template <typename T, typename Heap>
void bf_impl(const T* cloud, int64_t n, int64_t stride, int dim, const T* query, int64_t nq, int64_t qStride, int k,
             unsigned flags, T maxRadius, const T* maxRadii, int32_t* outIdx, T* outD2) {
  const bool allowSelf = flags & ALLOW_SELF_MATCH;
  const bool sortResults = flags & SORT_RESULTS;
#pragma omp parallel
  {
    Heap heap((size_t)k);
#pragma omp for schedule(static)
    for (int64_t c = 0; c < nq; ++c) {
      const T r = maxRadii ? maxRadii[c] : maxRadius;
      const T maxRadius2 = r * r;
      const T* q = query + c * qStride;
      heap.reset();
      for (int64_t i = 0; i < n; ++i) {
        T dist(0);
        for (int d = 0; d < dim; ++d) {
          const T diff = cloud[i * stride + d] - q[d];
          dist += diff * diff;
        }
        if ((dist <= maxRadius2) && heap.accepts((int)i, dist) &&
            (allowSelf || (dist > std::numeric_limits<T>::epsilon())))
          heap.replaceHead((int)i, dist);
      }
      if (sortResults) heap.sort();
      heap.getData(outIdx + c * k, outD2 + c * k);
    }
  }
}

template <typename T>
int bf_knn(const T* cloud, int rows, int64_t n, int64_t stride, int dimIn, const T* query, int qRows, int64_t nq,
           int64_t qStride, int k, unsigned flags, unsigned creationFlags, T maxRadius, const T* maxRadii, int mode,
           int32_t* outIdx, T* outD2, uint64_t* touched) {
  int dim = 0;
  if (!check_create<T>(rows, n, dimIn, 0, false, &dim)) return 1;
  if (!check_knn(n, dim, qRows, k, flags, maxRadii ? nq : -1, nq)) return 1;
  if (k > 0) {
    if (mode == MODE_CANONICAL)
      bf_impl<T, CanonicalHeap<T>>(cloud, n, stride, dim, query, nq, qStride, k, flags, maxRadius, maxRadii, outIdx,
                                   outD2);
    else
      bf_impl<T, STLHeap<T>>(cloud, n, stride, dim, query, nq, qStride, k, flags, maxRadius, maxRadii, outIdx, outD2);
  }
  if (touched) *touched = (creationFlags & TOUCH_STATISTICS) ? (uint64_t)nq * (uint64_t)n : 0;
  return 0;
}

}  // namespace

extern "C" {

const char* oracle_last_error(void) { return g_err.c_str(); }

int oracle_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

void oracle_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}

#define ORACLE_DEFINE(SUF, T)                                                                                        \
  void* oracle_tree_build_##SUF(const T* cloud, int rows, int64_t n, int64_t stride, int dim, unsigned bucketSize) { \
    return build_tree<T>(cloud, rows, n, stride, dim, bucketSize);                                                   \
  }                                                                                                                  \
  void oracle_tree_free_##SUF(void* h) { delete static_cast<Tree<T>*>(h); }                                          \
  void oracle_tree_info_##SUF(void* h, int64_t* out) {                                                               \
    const Tree<T>* t = static_cast<Tree<T>*>(h);                                                                     \
    out[0] = (int64_t)t->nodes.size();                                                                               \
    out[1] = (int64_t)t->buckets.size();                                                                             \
    out[2] = t->dim;                                                                                                 \
    out[3] = t->height;                                                                                              \
  }                                                                                                                  \
  void oracle_tree_export_##SUF(void* h, int32_t* cutDim, T* cutVal, uint32_t* right, uint32_t* bStart,             \
                                uint32_t* bCount, int32_t* buckets, T* minB, T* maxB) {                              \
    const Tree<T>* t = static_cast<Tree<T>*>(h);                                                                     \
    for (size_t i = 0; i < t->nodes.size(); ++i) {                                                                   \
      cutDim[i] = t->nodes[i].cutDim;                                                                                \
      cutVal[i] = t->nodes[i].cutVal;                                                                                \
      right[i] = t->nodes[i].right;                                                                                  \
      bStart[i] = t->nodes[i].bucketStart;                                                                           \
      bCount[i] = t->nodes[i].bucketCount;                                                                           \
    }                                                                                                                \
    std::memcpy(buckets, t->buckets.data(), t->buckets.size() * sizeof(int32_t));                                    \
    for (int d = 0; d < t->dim; ++d) {                                                                               \
      minB[d] = t->minBound[d];                                                                                      \
      maxB[d] = t->maxBound[d];                                                                                      \
    }                                                                                                                \
  }                                                                                                                  \
  int oracle_tree_knn_##SUF(void* h, const T* q, int qRows, int64_t nq, int64_t qStride, int k, T eps,              \
                            unsigned flags, unsigned creationFlags, T maxRadius, const T* maxRadii, int mode,        \
                            int heap, int32_t* outIdx, T* outD2, uint64_t* touched) {                                \
    return tree_knn<T>(static_cast<Tree<T>*>(h), q, qRows, nq, qStride, k, eps, flags, creationFlags, maxRadius,     \
                       maxRadii, mode, heap, outIdx, outD2, touched);                                                \
  }                                                                                                                  \
  int oracle_bf_knn_##SUF(const T* cloud, int rows, int64_t n, int64_t stride, int dim, const T* q, int qRows,      \
                          int64_t nq, int64_t qStride, int k, unsigned flags, unsigned creationFlags, T maxRadius,   \
                          const T* maxRadii, int mode, int32_t* outIdx, T* outD2, uint64_t* touched) {               \
    return bf_knn<T>(cloud, rows, n, stride, dim, q, qRows, nq, qStride, k, flags, creationFlags, maxRadius,         \
                     maxRadii, mode, outIdx, outD2, touched);                                                        \
  }

ORACLE_DEFINE(f32, float)
ORACLE_DEFINE(f64, double)

}  // extern "C"
