// order.cu -- query ordering for warp coherence, and a device-wide scan.
//
// A query ordering is a counting sort by cell: every query gets a cell id
// and a rank inside its cell (an atomic increment of the cell's count), the
// counts are scanned into offsets and each query is placed at offset+rank.
// The kd-tree search uses the leaf each query descends to as its cell
// (k_leaf_cells in search.cuh), which groups queries at the scale of the
// data's own buckets. order_queries() offers a Morton (Z-order) cell over
// the bounding box for searches without a tree. The order inside a cell is
// whatever the atomics produce; results do not depend on it, only timing.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>

#include "internal.cuh"

namespace nabo_gb300 {
namespace {

constexpr int kB = 256;
constexpr int kMortonDims = 10;

__device__ __forceinline__ uint32_t block_excl_scan_u32(uint32_t v, uint32_t* total) {
  __shared__ uint32_t sw[kB / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) sw[warp] = x;
  __syncthreads();
  if (warp == 0) {
    uint32_t w = lane < kB / 32 ? sw[lane] : 0u;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += y;
    }
    if (lane < kB / 32) sw[lane] = w;
  }
  __syncthreads();
  const uint32_t wpre = warp > 0 ? sw[warp - 1] : 0u;
  *total = sw[kB / 32 - 1];
  __syncthreads();
  return wpre + x - v;
}

__global__ void k_block_sums(const uint32_t* __restrict__ data, int64_t n, uint32_t* sums) {
  const int64_t i = blockIdx.x * (int64_t)kB + threadIdx.x;
  const uint32_t v = i < n ? data[i] : 0u;
  uint32_t t;
  block_excl_scan_u32(v, &t);
  if (threadIdx.x == 0) sums[blockIdx.x] = t;
}

__global__ void k_scan_sums(uint32_t* sums, int nb, uint32_t* total) {
  uint32_t carry = 0;
  for (int base = 0; base < nb; base += kB) {
    const int i = base + threadIdx.x;
    const uint32_t v = i < nb ? sums[i] : 0u;
    uint32_t t;
    const uint32_t ex = block_excl_scan_u32(v, &t);
    if (i < nb) sums[i] = carry + ex;
    carry += t;
  }
  if (threadIdx.x == 0 && total) *total = carry;
}

__global__ void k_apply(uint32_t* data, int64_t n, const uint32_t* __restrict__ sums) {
  const int64_t i = blockIdx.x * (int64_t)kB + threadIdx.x;
  const uint32_t v = i < n ? data[i] : 0u;
  uint32_t t;
  const uint32_t ex = block_excl_scan_u32(v, &t);
  if (i < n) data[i] = ex + sums[blockIdx.x];
}

struct CellParams {
  float lo[kMortonDims];
  float scale[kMortonDims];
  int dims;
  int bits;
  int shift;
};

template <typename T>
__global__ void k_cells(const T* __restrict__ q, int64_t nq, int64_t qStride, CellParams p, uint32_t* cell,
                        uint32_t* rank, uint32_t* hist) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= nq) return;
  uint32_t c[kMortonDims];
  const float maxc = (float)((1u << p.bits) - 1u);
#pragma unroll
  for (int d = 0; d < kMortonDims; ++d) {
    if (d < p.dims) {
      float v = ((float)q[i * qStride + d] - p.lo[d]) * p.scale[d];
      v = fminf(fmaxf(v, 0.0f), maxc);
      c[d] = (uint32_t)v;
    } else {
      c[d] = 0;
    }
  }
  uint32_t key = 0;
  for (int b = p.bits - 1; b >= 0; --b)
    for (int d = 0; d < p.dims; ++d) key = (key << 1) | ((c[d] >> b) & 1u);
  const uint32_t cl = key >> p.shift;
  cell[i] = cl;
  rank[i] = atomicAdd(hist + cl, 1u);
}

__global__ void k_place(const uint32_t* __restrict__ cell, const uint32_t* __restrict__ rank,
                        const uint32_t* __restrict__ start, int64_t nq, int32_t* order) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= nq) return;
  order[start[cell[i]] + rank[i]] = (int32_t)i;
}

}  // namespace

int scan_exclusive_u32(uint32_t* data, int64_t n, uint32_t* dTotal, cudaStream_t stream) {
  const int nb = ceil_div(n, kB);
  uint32_t* sums = nullptr;
  NABO_CUDA_TRY(scratch_alloc((void**)&sums, (size_t)std::max(nb, 1) * sizeof(uint32_t), stream));
  k_block_sums<<<nb, kB, 0, stream>>>(data, n, sums);
  k_scan_sums<<<1, kB, 0, stream>>>(sums, nb, dTotal);
  k_apply<<<nb, kB, 0, stream>>>(data, n, sums);
  const cudaError_t e = cudaGetLastError();
  scratch_free(sums, stream);
  if (e != cudaSuccess) return cuda_error(e, "scan_exclusive_u32");
  return kOk;
}

int order_by_cells(const uint32_t* dCell, const uint32_t* dRank, uint32_t* dHist, int64_t bins, int64_t nq,
                   int32_t* dOrder, cudaStream_t stream) {
  const int rc = scan_exclusive_u32(dHist, bins, nullptr, stream);
  if (rc != kOk) return rc;
  k_place<<<ceil_div(nq, kB), kB, 0, stream>>>(dCell, dRank, dHist, nq, dOrder);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_error(e, "order_by_cells");
  return kOk;
}

template <typename T>
int order_queries(const T* dQuery, int64_t nq, int64_t qStride, int dim, const double* lo, const double* hi,
                  int32_t* dOrder, cudaStream_t stream) {
  CellParams p;
  p.dims = std::min(dim, kMortonDims);
  p.bits = 30 / p.dims;
  const int keyBits = p.bits * p.dims;
  int want = 1;
  while ((int64_t(1) << want) < nq && want < 30) ++want;
  const int B = std::max(1, std::min({keyBits, want + 1, 22}));
  p.shift = keyBits - B;
  for (int d = 0; d < kMortonDims; ++d) {
    if (d < p.dims) {
      const double ext = hi[d] - lo[d];
      p.lo[d] = (float)lo[d];
      p.scale[d] = (ext > 0.0 && std::isfinite(ext)) ? (float)(((1u << p.bits) - 1u) / ext) : 0.0f;
    } else {
      p.lo[d] = 0.0f;
      p.scale[d] = 0.0f;
    }
  }
  const int64_t bins = int64_t(1) << B;
  uint32_t *hist = nullptr, *cell = nullptr, *rank = nullptr;
  NABO_CUDA_TRY(scratch_alloc((void**)&hist, (size_t)bins * sizeof(uint32_t), stream));
  NABO_CUDA_TRY(scratch_alloc((void**)&cell, (size_t)nq * sizeof(uint32_t), stream));
  NABO_CUDA_TRY(scratch_alloc((void**)&rank, (size_t)nq * sizeof(uint32_t), stream));
  NABO_CUDA_TRY(cudaMemsetAsync(hist, 0, (size_t)bins * sizeof(uint32_t), stream));
  k_cells<T><<<ceil_div(nq, kB), kB, 0, stream>>>(dQuery, nq, qStride, p, cell, rank, hist);
  int rc = scan_exclusive_u32(hist, bins, nullptr, stream);
  if (rc == kOk) {
    k_place<<<ceil_div(nq, kB), kB, 0, stream>>>(cell, rank, hist, nq, dOrder);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) rc = cuda_error(e, "order_queries");
  }
  scratch_free(hist, stream);
  scratch_free(cell, stream);
  scratch_free(rank, stream);
  return rc;
}

template int order_queries<float>(const float*, int64_t, int64_t, int, const double*, const double*, int32_t*,
                                  cudaStream_t);
template int order_queries<double>(const double*, int64_t, int64_t, int, const double*, const double*, int32_t*,
                                   cudaStream_t);

}  // namespace nabo_gb300
