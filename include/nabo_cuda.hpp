// nabo_cuda.hpp -- header-only C++ front end over the C ABI (nabo_gb300.h).
//
// The same shape as the reference's Nabo::NearestNeighbourSearch<T>
// (nabo/nabo.h:257-441): a factory returning an owning raw pointer, public
// members dim / creationOptionFlags / minBound / maxBound, and the two knn()
// overloads (scalar maxRadius, nabo/nabo.h:338; per-query maxRadii,
// nabo/nabo.h:351) with the reference's argument order, defaults, flag
// values, size checks and messages; errors are thrown as
// nabo_cuda::runtime_error, derived from std::runtime_error like
// Nabo::runtime_error (nabo/nabo.cpp:50-66).
//
// Matrices are column-major, one point per column, as the reference's Eigen
// matrices: any type with rows(), cols() and data() works (vectors also need
// resize()), so Eigen::MatrixXf / MatrixXi / VectorXf / VectorXi instantiate
// it directly; DenseMatrix and DenseVector below serve callers without Eigen. The cloud is copied to the GPU at creation; the
// object keeps a reference to the caller's cloud for the `cloud` member, as
// the reference does (nabo/nabo.h:273-274).
#pragma once

#include <cstdint>
#include <limits>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <vector>

#include "nabo_gb300.h"

namespace nabo_cuda {

struct runtime_error : std::runtime_error {
  explicit runtime_error(const std::string& what) : std::runtime_error(what) {}
};

// Column-major dense matrix for callers without Eigen.
template <typename S>
class DenseMatrix {
 public:
  using Scalar = S;
  DenseMatrix() = default;
  DenseMatrix(long rows, long cols) : rows_(rows), cols_(cols), v_((size_t)(rows * cols)) {}
  long rows() const { return rows_; }
  long cols() const { return cols_; }
  long size() const { return rows_ * cols_; }
  S* data() { return v_.data(); }
  const S* data() const { return v_.data(); }
  S& operator()(long r, long c) { return v_[(size_t)(c * rows_ + r)]; }
  const S& operator()(long r, long c) const { return v_[(size_t)(c * rows_ + r)]; }
  S& operator()(long i) { return v_[(size_t)i]; }
  const S& operator()(long i) const { return v_[(size_t)i]; }

 private:
  long rows_ = 0, cols_ = 0;
  std::vector<S> v_;
};

// Column vector for callers without Eigen (the reference's Vector and
// IndexVector, nabo/nabo.h:263-269).
template <typename S>
class DenseVector {
 public:
  using Scalar = S;
  DenseVector() = default;
  explicit DenseVector(long n) : v_((size_t)n) {}
  long rows() const { return (long)v_.size(); }
  long cols() const { return 1; }
  long size() const { return (long)v_.size(); }
  void resize(long n) { v_.resize((size_t)n); }
  S* data() { return v_.data(); }
  const S* data() const { return v_.data(); }
  S& operator()(long i) { return v_[(size_t)i]; }
  const S& operator()(long i) const { return v_[(size_t)i]; }

 private:
  std::vector<S> v_;
};

namespace detail {
template <typename T>
constexpr int dtype() {
  static_assert(std::is_same<T, float>::value || std::is_same<T, double>::value, "float or double");
  return std::is_same<T, float>::value ? NABO_CUDA_FLOAT32 : NABO_CUDA_FLOAT64;
}
inline void check(int rc) {
  if (rc != NABO_CUDA_OK) throw runtime_error(nabo_cuda_last_error());
}
}  // namespace detail

// CloudType is what the cloud is held as: an owning matrix, a fixed-row
// matrix (the reference's Matrix3X instantiation) or a non-owning mapped view
// (its Map<const Matrix3X, Aligned>, nabo/nabo.cpp:181-186); it needs rows(),
// cols() and a column-major data() with stride rows(). MatrixType is the
// matrix of queries and squared distances, dynamic in both dimensions as the
// reference's Matrix typedef (nabo/nabo.h:261); it defaults to CloudType for
// owning dynamic clouds.
template <typename T, typename CloudType = DenseMatrix<T>, typename IndexMatrixType = DenseMatrix<int>,
          typename VectorType = DenseVector<T>, typename IndexVectorType = DenseVector<int>,
          typename MatrixType = CloudType>
class NearestNeighbourSearch {
 public:
  using Matrix = MatrixType;
  using IndexMatrix = IndexMatrixType;
  using Vector = VectorType;
  using IndexVector = IndexVectorType;
  using Index = int;  // the reference's typedef int Index (nabo/nabo.h:267)

  // Values of the reference's enums (nabo/nabo.h:290-312), extended by the
  // two CUDA search types after BRUTE_FORCE_CL.
  enum SearchType {
    BRUTE_FORCE = 0,
    KDTREE_LINEAR_HEAP,
    KDTREE_TREE_HEAP,
    KDTREE_CL_PT_IN_NODES,
    KDTREE_CL_PT_IN_LEAVES,
    BRUTE_FORCE_CL,
    KDTREE_CUDA,
    BRUTE_FORCE_CUDA,
    SEARCH_TYPE_COUNT
  };
  enum CreationOptionFlags { TOUCH_STATISTICS = 1 };
  enum SearchOptionFlags { ALLOW_SELF_MATCH = 1, SORT_RESULTS = 2 };
  // the one Parameters key of the kd-tree (nabo/nabo.h:231-254, "bucketSize")
  struct Parameters {
    unsigned bucketSize = 8;
  };

  const CloudType& cloud;
  const Index dim;
  const unsigned creationOptionFlags;
  std::vector<T> minBound;
  std::vector<T> maxBound;

  // nabo/nabo.h:360: only the CUDA search types are served here.
  static NearestNeighbourSearch* create(const CloudType& cloud,
                                        Index dim = std::numeric_limits<Index>::max(),
                                        SearchType searchType = KDTREE_CUDA, unsigned creationOptionFlags = 0,
                                        const Parameters& parameters = Parameters()) {
    return new NearestNeighbourSearch(cloud, dim, searchType, creationOptionFlags, parameters);
  }
  // The kd-tree with a linear heap (nabo/nabo.h:377) on the GPU: the same
  // tree and, sorted, the same results.
  static NearestNeighbourSearch* createKDTreeLinearHeap(const CloudType& cloud,
                                                        Index dim = std::numeric_limits<Index>::max(),
                                                        unsigned creationOptionFlags = 0,
                                                        const Parameters& parameters = Parameters()) {
    return create(cloud, dim, KDTREE_CUDA, creationOptionFlags, parameters);
  }
  static NearestNeighbourSearch* createBruteForce(const CloudType& cloud,
                                                  Index dim = std::numeric_limits<Index>::max(),
                                                  unsigned creationOptionFlags = 0) {
    return create(cloud, dim, BRUTE_FORCE_CUDA, creationOptionFlags);
  }

  virtual ~NearestNeighbourSearch() { nabo_cuda_destroy(h_); }
  NearestNeighbourSearch(const NearestNeighbourSearch&) = delete;
  NearestNeighbourSearch& operator=(const NearestNeighbourSearch&) = delete;

  // nabo/nabo.h:338. indices and dists2 are k x query.cols(), pre-sized by
  // the caller; returns the touched count with TOUCH_STATISTICS, else 0.
  unsigned long knn(const Matrix& query, IndexMatrix& indices, Matrix& dists2, Index k = 1, T epsilon = 0,
                    unsigned optionFlags = 0,
                    T maxRadius = std::numeric_limits<T>::infinity()) const {
    return run(query, indices, dists2, nullptr, 0, k, epsilon, optionFlags, maxRadius);
  }
  // nabo/nabo.h:325 (nabo/nabo.cpp:82-100): one query point; the first dim
  // entries of `query` are used, indices and dists2 are resized to k.
  unsigned long knn(const Vector& query, IndexVector& indices, Vector& dists2, Index k = 1, T epsilon = 0,
                    unsigned optionFlags = 0, T maxRadius = std::numeric_limits<T>::infinity()) const {
    if ((Index)(query.rows() * query.cols()) < dim)
      throw runtime_error("Query has less dimensions (" + std::to_string((long)(query.rows() * query.cols())) +
                          ") than requested for cloud (" + std::to_string(dim) + ")");
    if (k < 0) throw runtime_error("k must be at least 1");
    indices.resize(k);
    dists2.resize(k);
    return run_raw(query.data(), (long)dim, 1, (long)dim, indices.data(), (long)k, 1, dists2.data(), (long)k, 1,
                   nullptr, 0, k, epsilon, optionFlags, maxRadius);
  }
  // nabo/nabo.h:351: one radius per query column.
  unsigned long knn(const Matrix& query, IndexMatrix& indices, Matrix& dists2, const Vector& maxRadii,
                    Index k = 1, T epsilon = 0, unsigned optionFlags = 0) const {
    return run(query, indices, dists2, maxRadii.data(), (long)(maxRadii.rows() * maxRadii.cols()), k, epsilon,
               optionFlags, std::numeric_limits<T>::infinity());
  }

 private:
  NearestNeighbourSearch(const CloudType& c, Index d, SearchType type, unsigned flags, const Parameters& p)
      : cloud(c), dim(d > (Index)c.rows() ? (Index)c.rows() : d), creationOptionFlags(flags) {
    nabo_cuda_params params;
    nabo_cuda_params_init(&params);
    params.bucketSize = p.bucketSize;
    detail::check(nabo_cuda_create(detail::dtype<T>(), c.data(), (int)c.rows(), (int64_t)c.cols(),
                                   (int64_t)c.rows(), (int)d, (int)type, flags, &params, &h_));
    minBound.resize((size_t)dim);
    maxBound.resize((size_t)dim);
    detail::check(nabo_cuda_get_bounds(h_, minBound.data(), maxBound.data()));
  }

  unsigned long run(const Matrix& query, IndexMatrix& indices, Matrix& dists2, const T* radii, long nRadii,
                    Index k, T epsilon, unsigned optionFlags, T maxRadius) const {
    return run_raw(query.data(), (long)query.rows(), (long)query.cols(), (long)query.rows(), indices.data(),
                   (long)indices.rows(), (long)indices.cols(), dists2.data(), (long)dists2.rows(),
                   (long)dists2.cols(), radii, nRadii, k, epsilon, optionFlags, maxRadius);
  }

  // the reference's checkSizesKnn (nabo/nabo.cpp:102-131), in its order and
  // with its messages (which print rows() in the column messages and k in
  // the radii message); the library repeats the checks it can make
  unsigned long run_raw(const T* qData, long qRows, long qCols, long qStride, int* iData, long iRows, long iCols,
                        T* dData, long dRows, long dCols, const T* radii, long nRadii, Index k, T epsilon,
                        unsigned optionFlags, T maxRadius) const {
    using std::to_string;
    const long n = (long)cloud.cols();
    if (optionFlags & ALLOW_SELF_MATCH) {
      if (k > n)
        throw runtime_error("Requesting more points (" + to_string(k) + ") than available in cloud (" +
                            to_string(n) + ")");
    } else if (k > n - 1) {
      throw runtime_error("Requesting more points (" + to_string(k) + ") than available in cloud minus 1 (" +
                          to_string(n - 1) + ") (as self match is forbidden)");
    }
    if ((Index)qRows < dim)
      throw runtime_error("Query has less dimensions (" + to_string(qRows) + ") than requested for cloud (" +
                          to_string(dim) + ")");
    if ((Index)iRows != k)
      throw runtime_error("Index matrix has a different number of rows (" + to_string(iRows) + ") than k (" +
                          to_string(k) + ")");
    if (iCols != qCols)
      throw runtime_error("Index matrix has a different number of columns (" + to_string(iRows) +
                          ") than query (" + to_string(qCols) + ")");
    if ((Index)dRows != k)
      throw runtime_error("Distance matrix has a different number of rows (" + to_string(dRows) + ") than k (" +
                          to_string(k) + ")");
    if (dCols != qCols)
      throw runtime_error("Distance matrix has a different number of columns (" + to_string(dRows) +
                          ") than query (" + to_string(qCols) + ")");
    if (radii && nRadii != qCols)
      throw runtime_error("Maximum radii vector has not the same length (" + to_string(nRadii) +
                          ") than query has columns (" + to_string(k) + ")");
    const unsigned maxFlags = ALLOW_SELF_MATCH | SORT_RESULTS;
    if (optionFlags > maxFlags)
      throw runtime_error("OR-ed value of option flags (" + to_string(optionFlags) +
                          ") is larger than maximal valid value (" + to_string(maxFlags) + ")");
    uint64_t touched = 0;
    detail::check(nabo_cuda_knn(h_, qData, (int)qRows, (int64_t)qCols, (int64_t)qStride, (int)k, (double)epsilon,
                                optionFlags, (double)maxRadius, radii, iData, dData, &touched));
    return (creationOptionFlags & TOUCH_STATISTICS) ? (unsigned long)touched : 0ul;
  }

  nabo_cuda_search* h_ = nullptr;
};

using NNSearchF = NearestNeighbourSearch<float>;
using NNSearchD = NearestNeighbourSearch<double>;

}  // namespace nabo_cuda
