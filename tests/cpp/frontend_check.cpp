// Exercises include/nabo_cuda.hpp the way a libnabo user would.
//   frontend_check errors                -- argument errors raised before any GPU work
//   frontend_check search <in> <out>     -- searches (float and double) and knn() size checks
// <in>: int32 n, nq, k, dim; float cloud[dim*n]; float query[dim*nq]; float radii[nq]
// <out>: per type (float, double): int32 idx[k*nq], T d2[k*nq] (plain), int32 idx, T d2 (radii),
//        uint64 touched
#include <cstdio>
#include <cstring>
#include <string>
#include <type_traits>
#include <vector>

#include "nabo_cuda.hpp"

template <typename S>
using M = nabo_cuda::DenseMatrix<S>;

// the reference's index type (nabo/nabo.h:267), so code that declares
// NNS::Index or stores it in int containers compiles unchanged
static_assert(std::is_same<nabo_cuda::NNSearchF::Index, int>::value, "Index must be int");
static_assert(std::is_same<nabo_cuda::NNSearchD::Index, int>::value, "Index must be int");

static int expect_error(const char* what, const std::string& needle, void (*fn)()) {
  try {
    fn();
  } catch (const nabo_cuda::runtime_error& e) {
    if (std::string(e.what()).find(needle) != std::string::npos) {
      std::printf("ok %s: %s\n", what, e.what());
      return 0;
    }
    std::printf("FAIL %s: wrong message: %s\n", what, e.what());
    return 1;
  } catch (const std::exception& e) {
    std::printf("FAIL %s: unexpected exception type: %s\n", what, e.what());
    return 1;
  }
  std::printf("FAIL %s: no exception\n", what);
  return 1;
}

static M<float> g_cloud(3, 50), g_empty(3, 0);

static int errors() {
  for (long i = 0; i < g_cloud.size(); ++i) g_cloud(i) = (float)(i % 7) * 0.1f;
  int bad = 0;
  bad += expect_error("dim 0", "Your space must have at least one dimension",
                      [] { delete nabo_cuda::NNSearchF::create(g_cloud, 0); });
  bad += expect_error("bucket size", "Requested bucket size 1, but must be larger than 2", [] {
    nabo_cuda::NNSearchF::Parameters p;
    p.bucketSize = 1;
    delete nabo_cuda::NNSearchF::create(g_cloud, 3, nabo_cuda::NNSearchF::KDTREE_CUDA, 0, p);
  });
  bad += expect_error("empty cloud", "Cloud has no points",
                      [] { delete nabo_cuda::NNSearchF::createKDTreeLinearHeap(g_empty); });
  bad += expect_error("cpu type", "only the CUDA search types",
                      [] { delete nabo_cuda::NNSearchF::create(g_cloud, 3, nabo_cuda::NNSearchF::KDTREE_TREE_HEAP); });
  return bad;
}

// Clouds held as the reference's other instantiations hold them
// (nabo/nabo.cpp:181-186): a matrix with 3 rows fixed at compile time
// (Matrix3X) and a non-owning view of a caller's column-major buffer
// (Map<const Matrix3X, Aligned>); queries and distances stay dynamic.
template <typename S>
class Fixed3X {
 public:
  using Scalar = S;
  explicit Fixed3X(long n) : n_(n), v_((size_t)(3 * n)) {}
  static constexpr long rows() { return 3; }
  long cols() const { return n_; }
  const S* data() const { return v_.data(); }
  S& operator()(long i) { return v_[(size_t)i]; }

 private:
  long n_;
  std::vector<S> v_;
};

template <typename S>
class ConstMap3X {
 public:
  using Scalar = S;
  ConstMap3X(const S* p, long n) : p_(p), n_(n) {}
  static constexpr long rows() { return 3; }
  long cols() const { return n_; }
  const S* data() const { return p_; }

 private:
  const S* p_;
  long n_;
};

// The same search through a fixed-row cloud and through a mapped cloud:
// results identical to the dense cloud's.
template <typename T>
static int other_cloud_types(const M<T>& cloud, const M<T>& query, const M<int>& idx, const M<T>& d2, int k) {
  using V = nabo_cuda::DenseVector<T>;
  using IV = nabo_cuda::DenseVector<int>;
  using NNSFixed = nabo_cuda::NearestNeighbourSearch<T, Fixed3X<T>, M<int>, V, IV, M<T>>;
  using NNSMap = nabo_cuda::NearestNeighbourSearch<T, ConstMap3X<T>, M<int>, V, IV, M<T>>;
  static_assert(std::is_same<typename NNSMap::Matrix, M<T>>::value, "queries and distances stay dynamic");
  int bad = 0;
  Fixed3X<T> fixed(cloud.cols());
  for (long i = 0; i < cloud.size(); ++i) fixed(i) = cloud(i);
  const ConstMap3X<T> mapped(cloud.data(), cloud.cols());
  M<int> i1(k, query.cols()), i2(k, query.cols());
  M<T> e1(k, query.cols()), e2(k, query.cols());
  NNSFixed* a = NNSFixed::createKDTreeLinearHeap(fixed);
  NNSMap* b = NNSMap::createKDTreeLinearHeap(mapped);
  a->knn(query, i1, e1, k, 0, NNSFixed::SORT_RESULTS, (T)1.0);
  b->knn(query, i2, e2, k, 0, NNSMap::SORT_RESULTS, (T)1.0);
  int diff1 = 0, diff2 = 0;
  for (long i = 0; i < idx.size(); ++i) {
    diff1 += (i1(i) != idx(i) || e1(i) != d2(i)) ? 1 : 0;
    diff2 += (i2(i) != idx(i) || e2(i) != d2(i)) ? 1 : 0;
  }
  std::printf("%s Matrix3X-like cloud: %d differences\n", diff1 ? "FAIL" : "ok", diff1);
  std::printf("%s Map<const Matrix3X>-like cloud: %d differences\n", diff2 ? "FAIL" : "ok", diff2);
  bad += (diff1 ? 1 : 0) + (diff2 ? 1 : 0);
  bad += (&b->cloud == &mapped) ? 0 : 1;  // held by reference, as the reference holds it
  delete a;
  delete b;
  return bad;
}

template <typename T>
static int search_type(const std::vector<float>& c, const std::vector<float>& q, const std::vector<float>& r, int n,
                       int nq, int k, int dim, FILE* out) {
  using NNS = nabo_cuda::NearestNeighbourSearch<T>;
  M<T> cloud(dim, n), query(dim, nq);
  nabo_cuda::DenseVector<T> radii(nq);
  for (long i = 0; i < cloud.size(); ++i) cloud(i) = (T)c[(size_t)i];
  for (long i = 0; i < query.size(); ++i) query(i) = (T)q[(size_t)i];
  for (long i = 0; i < nq; ++i) radii(i) = (T)r[(size_t)i];
  NNS* s = NNS::createKDTreeLinearHeap(cloud, dim, NNS::TOUCH_STATISTICS);
  M<int> idx(k, nq), idx2(k, nq);
  M<T> d2(k, nq), d22(k, nq);
  const unsigned long touched = s->knn(query, idx, d2, k, 0, NNS::SORT_RESULTS, (T)1.0);
  s->knn(query, idx2, d22, radii, k, 0, 0);
  int bad = dim == 3 ? other_cloud_types<T>(cloud, query, idx, d2, k) : 0;
  std::fwrite(idx.data(), 4, (size_t)idx.size(), out);
  std::fwrite(d2.data(), sizeof(T), (size_t)d2.size(), out);
  std::fwrite(idx2.data(), 4, (size_t)idx2.size(), out);
  std::fwrite(d22.data(), sizeof(T), (size_t)d22.size(), out);
  const uint64_t t64 = touched;
  std::fwrite(&t64, 8, 1, out);
  // the single-point overload (nabo/nabo.h:325) against the matrix call's columns
  {
    nabo_cuda::DenseVector<T> qv(dim + 1), dv;  // a longer vector: only the first dim entries count
    nabo_cuda::DenseVector<int> iv;
    int diff = 0;
    for (int j = 0; j < nq && j < 40; ++j) {
      for (int d = 0; d < dim; ++d) qv(d) = query(d, j);
      qv(dim) = (T)1e30;
      s->knn(qv, iv, dv, k, 0, 0, (T)1.0);
      if (iv.size() != k || dv.size() != k) ++diff;
      for (int r = 0; r < k && r < iv.size(); ++r) diff += (iv(r) != idx(r, j) || dv(r) != d2(r, j)) ? 1 : 0;
    }
    std::printf("%s single-vector knn: %d differences\n", diff ? "FAIL" : "ok", diff);
    bad += diff ? 1 : 0;
  }
  // knn() argument checks on a live object, in the reference's order
  auto must = [&](const char* what, const std::string& needle, auto fn) {
    try {
      fn();
      std::printf("FAIL %s: no exception\n", what);
      ++bad;
    } catch (const nabo_cuda::runtime_error& e) {
      const bool ok = std::string(e.what()).find(needle) != std::string::npos;
      std::printf("%s %s: %s\n", ok ? "ok" : "FAIL", what, e.what());
      bad += ok ? 0 : 1;
    }
  };
  M<int> wrongRows(k + 1, nq);
  M<T> wrongCols(k, nq + 1), fewDims(dim - 1, nq);
  nabo_cuda::DenseVector<T> shortRadii(nq - 1);
  must("k too large", "than available in cloud minus 1", [&] { s->knn(query, idx, d2, (long)n, 0, 0); });
  must("query dims", "Query has less dimensions", [&] { s->knn(fewDims, idx, d2, k); });
  must("index rows", "Index matrix has a different number of rows", [&] { s->knn(query, wrongRows, d2, k); });
  must("dist cols", "Distance matrix has a different number of columns", [&] { s->knn(query, idx, wrongCols, k); });
  must("radii", "Maximum radii vector has not the same length", [&] { s->knn(query, idx, d2, shortRadii, k); });
  must("flags", "OR-ed value of option flags (4)", [&] { s->knn(query, idx, d2, k, 0, 4); });
  std::printf("%s bounds %g..%g dim %ld\n", sizeof(T) == 4 ? "float" : "double", (double)s->minBound[0],
              (double)s->maxBound[0], (long)s->dim);
  delete s;
  return bad;
}

int main(int argc, char** argv) {
  if (argc >= 2 && std::strcmp(argv[1], "errors") == 0) return errors();
  if (argc < 4 || std::strcmp(argv[1], "search") != 0) {
    std::fprintf(stderr, "usage: frontend_check errors | search <in> <out>\n");
    return 2;
  }
  FILE* in = std::fopen(argv[2], "rb");
  if (!in) return 2;
  int hdr[4];
  if (std::fread(hdr, 4, 4, in) != 4) return 2;
  const int n = hdr[0], nq = hdr[1], k = hdr[2], dim = hdr[3];
  std::vector<float> c((size_t)dim * n), q((size_t)dim * nq), r((size_t)nq);
  if (std::fread(c.data(), 4, c.size(), in) != c.size() || std::fread(q.data(), 4, q.size(), in) != q.size() ||
      std::fread(r.data(), 4, r.size(), in) != r.size())
    return 2;
  std::fclose(in);
  FILE* out = std::fopen(argv[3], "wb");
  if (!out) return 2;
  int bad = 0;
  try {
    bad += search_type<float>(c, q, r, n, nq, k, dim, out);
    bad += search_type<double>(c, q, r, n, nq, k, dim, out);
  } catch (const std::exception& e) {
    std::printf("FAIL search: %s\n", e.what());
    bad += 1;
  }
  std::fclose(out);
  return bad;
}
