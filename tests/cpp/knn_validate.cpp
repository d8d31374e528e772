// The reference's CTest validation (tests/knnvalidate.cpp, run by
// tests/CMakeLists.txt:9-14 on tests/data/scan.*.txt) as a program written
// against include/nabo_cuda.hpp: loads a text cloud, makes the queries the
// reference's test helpers make, and checks that KDTREE_CUDA finds, rank by
// rank, points at the same squared distance (within epsilon of the scalar
// type) as BRUTE_FORCE_CUDA, in float and in double.
//
//   knn_validate DATA K DIM METHOD [MAX_RADIUS]
//       exit 0 on agreement; 1 usage, 2 bad data, 3 result shape, 4 a
//       neighbour differs (the reference's codes)
//   knn_validate --parse DATA
//       prints "dim D points N" for the loaded cloud (no GPU work)
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <limits>
#include <string>
#include <vector>

#include "nabo_cuda.hpp"

template <typename S>
using M = nabo_cuda::DenseMatrix<S>;

// A text cloud as tests/helpers.h:46-80 reads it: one point per line,
// values separated by any run of spaces, tabs, commas or semicolons, the
// first line's value count fixing the dimension; each value parsed as a
// double (atof) and stored as T. Returns false if the file cannot be read.
template <typename T>
static bool load_text(const char* path, M<T>* out) {
  std::ifstream in(path);
  if (!in) return false;
  std::vector<T> values;
  long dim = 0;
  bool first = true;
  std::string line;
  while (std::getline(in, line)) {
    long tokens = 0;
    size_t i = 0;
    while ((i = line.find_first_not_of(" \t,;", i)) != std::string::npos) {
      const size_t e = line.find_first_of(" \t,;", i);
      const std::string tok = line.substr(i, e == std::string::npos ? std::string::npos : e - i);
      values.push_back((T)std::atof(tok.c_str()));
      ++tokens;
      i = e;
    }
    if (first) dim = tokens;
    first = false;
  }
  if (dim <= 0) return false;
  const long n = (long)values.size() / dim;
  *out = M<T>(dim, n);
  for (long c = 0; c < n; ++c)
    for (long r = 0; r < dim; ++r) (*out)(r, c) = values[(size_t)(c * dim + r)];
  return true;
}

// The query matrix of tests/helpers.h:82-128. method < 0: 2 * n queries,
// query i is cloud point i mod n moved by +b (first n) or -b (last n) on
// every axis, b = sum of the bounds' extents / -method. method >= 0:
// `method` points drawn uniformly in the bounds with rand(). The bounds are
// those of search type 0, brute force (the true ones).
template <typename T>
static M<T> make_queries(const M<T>& d, const nabo_cuda::NearestNeighbourSearch<T>& bf, int method) {
  const long dim = d.rows(), n = d.cols();
  const long count = method == -1 ? 2 * n : (method < 0 ? 0 : method);
  M<T> q(dim, count);
  for (long i = 0; i < count; ++i) {
    if (method < 0) {
      T b = 0;
      for (long j = 0; j < dim; ++j) b += bf.maxBound[(size_t)j] - bf.minBound[(size_t)j];
      b /= (T)(-method);
      for (long j = 0; j < dim; ++j) q(j, i) = d(j, i % n) + (i < n ? b : -b);
    } else {
      for (long j = 0; j < dim; ++j) {
        const T lo = bf.minBound[(size_t)j], hi = bf.maxBound[(size_t)j];
        q(j, i) = lo + T(std::rand()) * (hi - lo) / T(RAND_MAX);
      }
    }
  }
  return q;
}

template <typename T>
static T dist2(const M<T>& d, long c, const M<T>& q, long i) {
  T s = 0;
  for (long j = 0; j < d.rows(); ++j) {
    const T v = d(j, c) - q(j, i);
    s += v * v;
  }
  return s;
}

template <typename T>
static int validate(const char* path, int K, int dim, int method, T maxRadius) {
  using NNS = nabo_cuda::NearestNeighbourSearch<T>;
  M<T> d;
  if (!load_text(path, &d)) {
    std::fprintf(stderr, "Cannot open file %s\n", path);
    return 2;
  }
  if (d.rows() != dim) {
    std::fprintf(stderr, "Provided data has %ld dimensions, but the requested dimensions were %d\n", d.rows(), dim);
    return 2;
  }
  if (K >= d.cols()) {
    std::fprintf(stderr, "Requested more nearest neighbour than points in the data set\n");
    return 2;
  }
  NNS* bf = NNS::create(d, d.rows(), NNS::BRUTE_FORCE_CUDA);
  NNS* kd = NNS::create(d, d.rows(), NNS::KDTREE_CUDA);
  const M<T> q = make_queries(d, *bf, method);
  M<int> ib(K, q.cols()), ik(K, q.cols());
  M<T> db(K, q.cols()), dk(K, q.cols());
  bf->knn(q, ib, db, K, 0, NNS::SORT_RESULTS, maxRadius);
  kd->knn(q, ik, dk, K, 0, NNS::SORT_RESULTS, maxRadius);
  int rc = 0;
  if (ib.rows() != K || ik.cols() != ib.cols()) rc = 3;
  long checked = 0;
  for (long i = 0; rc == 0 && i < q.cols(); ++i) {
    for (long r = 0; r < K; ++r) {
      if (db(r, i) == std::numeric_limits<T>::infinity()) continue;  // nothing within the radius
      const int kp = ik(r, i);
      if (kp < 0 || kp >= d.cols()) {
        std::fprintf(stderr, "query %ld, neighbour %ld of %d: invalid index %d\n", i, r, K, kp);
        rc = 4;
        break;
      }
      const T diff = std::fabs(dist2(d, ib(r, i), q, i) - dist2(d, kp, q, i));
      if (diff > std::numeric_limits<T>::epsilon()) {
        std::fprintf(stderr, "query %ld, neighbour %ld of %d: index %d (brute force) vs %d (kd-tree), dist2 diff %g\n",
                     i, r, K, ib(r, i), kp, (double)diff);
        rc = 4;
        break;
      }
      ++checked;
    }
  }
  std::printf("%s %s: %ld queries, %ld neighbours checked\n", rc ? "FAIL" : "ok", sizeof(T) == 4 ? "float" : "double",
              (long)q.cols(), checked);
  delete kd;
  delete bf;
  return rc;
}

int main(int argc, char* argv[]) {
  if (argc == 3 && std::string(argv[1]) == "--parse") {
    M<double> d;
    if (!load_text(argv[2], &d)) {
      std::fprintf(stderr, "Cannot open file %s\n", argv[2]);
      return 2;
    }
    std::printf("dim %ld points %ld\n", d.rows(), d.cols());
    for (long c = 0; c < d.cols() && c < 3; ++c) {
      for (long r = 0; r < d.rows(); ++r) std::printf("%s%.17g", r ? " " : "", d(r, c));
      std::printf("\n");
    }
    return 0;
  }
  if (argc < 5) {
    std::fprintf(stderr, "Usage %s DATA K DIM METHOD [MAX_RADIUS]\n", argv[0]);
    return 1;
  }
  const int K = std::atoi(argv[2]);
  const int dim = std::atoi(argv[3]);
  const int method = std::atoi(argv[4]);
  const double maxRadius = argc >= 6 ? std::atof(argv[5]) : std::numeric_limits<double>::infinity();
  try {
    int rc = validate<float>(argv[1], K, dim, method, (float)maxRadius);
    if (rc == 0) rc = validate<double>(argv[1], K, dim, method, maxRadius);
    return rc;
  } catch (const nabo_cuda::runtime_error& e) {
    std::fprintf(stderr, "error: %s\n", e.what());
    return 5;
  }
}
