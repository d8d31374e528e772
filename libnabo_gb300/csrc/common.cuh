// common.cuh -- shared types and helpers for the GB300 kNN kernels.
//
// Layouts (all in HBM, built once per cloud):
//   Rec<T,D>   one point: D coordinates followed by its int32 index in the
//              user's cloud, padded to a multiple of 16 bytes so a point is
//              fetched with 128-bit loads (f32 D=3: 16 B = one uint4).
//              The kd-tree stores its points in leaf order, so a leaf bucket
//              is a contiguous run of records.
//   Node<T>    one kd-tree node, pre-order, left child implicit at n+1
//              (the reference's layout idea, nabo/nabo_private.h:138-153):
//                meta low 5 bits  = cut dimension (0..30) or 31 for a leaf
//                meta high 27 bits = right-child index (inner) or bucket
//                                    size (leaf)
//              f32: {meta, cut | bucketStart}            8 bytes
//              f64: {meta, bucketStart, cut}            16 bytes
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <limits>

namespace nabo_gb300 {

// Kernels launched by launch_pdl (programmatic dependent launch) start with
// this: wait for the previous kernel in the stream to complete and its
// memory to be visible (griddepcontrol.wait) before touching anything, then
// let the next kernel be scheduled. A dependent grid starts only once every
// block of this grid has passed this point, so its waiting blocks never hold
// room this grid still needs. Launched the ordinary way, both are no-ops.
__device__ __forceinline__ void pdl_begin() {
  asm volatile("griddepcontrol.wait;" ::: "memory");
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

constexpr int kMaxDim = 16;
constexpr uint32_t kLeafDim = 31u;
constexpr int kMetaShift = 5;
constexpr uint32_t kMaxNodeIndex = (1u << (32 - kMetaShift)) - 1u;

// Exactly rounded arithmetic that the compiler may not contract into FMA:
// the reference's loops round every +,-,* separately.
template <typename T>
struct Ar;
template <>
struct Ar<float> {
  static __device__ __forceinline__ float add(float a, float b) { return __fadd_rn(a, b); }
  static __device__ __forceinline__ float sub(float a, float b) { return __fsub_rn(a, b); }
  static __device__ __forceinline__ float mul(float a, float b) { return __fmul_rn(a, b); }
  static __host__ __device__ __forceinline__ float eps() { return 1.1920928955078125e-07f; }
  static __host__ __device__ __forceinline__ float inf() { return __builtin_huge_valf(); }
};
template <>
struct Ar<double> {
  static __device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
  static __device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }
  static __device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
  static __host__ __device__ __forceinline__ double eps() { return 2.220446049250313080847263336181640625e-16; }
  static __host__ __device__ __forceinline__ double inf() { return __builtin_huge_val(); }
};

// Point record.
template <typename T, int D>
struct RecSize {
  static constexpr int bytes = (int)(D * sizeof(T)) + 4;
  static constexpr int chunks = (bytes + 15) / 16;  // uint4 per record
  static constexpr int words = chunks * 4;          // 32-bit words per record
};

template <typename T, int D>
struct alignas(16) Rec {
  union {
    uint4 v[RecSize<T, D>::chunks];
    struct {
      T c[D];
      int32_t idx;
    } p;
  };
};

template <typename T, int D>
__device__ __forceinline__ void load_rec(const Rec<T, D>* __restrict__ base, int64_t i, Rec<T, D>& r) {
  const uint4* src = reinterpret_cast<const uint4*>(base + i);
#pragma unroll
  for (int c = 0; c < RecSize<T, D>::chunks; ++c) r.v[c] = __ldg(src + c);
}

// kd-tree node.
template <typename T>
struct Node;
template <>
struct alignas(8) Node<float> {
  uint32_t meta;
  union {
    float cut;
    uint32_t start;
  };
};
template <>
struct alignas(16) Node<double> {
  uint32_t meta;
  uint32_t start;
  double cut;
};

__host__ __device__ __forceinline__ bool node_is_leaf(uint32_t meta) { return (meta & 31u) == kLeafDim; }
__host__ __device__ __forceinline__ uint32_t node_dim(uint32_t meta) { return meta & 31u; }
__host__ __device__ __forceinline__ uint32_t node_payload(uint32_t meta) { return meta >> kMetaShift; }
__host__ __device__ __forceinline__ uint32_t make_meta(uint32_t dimOrLeaf, uint32_t payload) {
  return dimOrLeaf | (payload << kMetaShift);
}

template <typename T>
__device__ __forceinline__ void store_inner(Node<T>* n, uint32_t cd, uint32_t right, T cut);
template <>
__device__ __forceinline__ void store_inner<float>(Node<float>* n, uint32_t cd, uint32_t right, float cut) {
  Node<float> v;
  v.meta = make_meta(cd, right);
  v.cut = cut;
  *n = v;
}
template <>
__device__ __forceinline__ void store_inner<double>(Node<double>* n, uint32_t cd, uint32_t right, double cut) {
  Node<double> v;
  v.meta = make_meta(cd, right);
  v.start = 0;
  v.cut = cut;
  *n = v;
}
template <typename T>
__device__ __forceinline__ void store_leaf(Node<T>* n, uint32_t count, uint32_t start);
template <>
__device__ __forceinline__ void store_leaf<float>(Node<float>* n, uint32_t count, uint32_t start) {
  Node<float> v;
  v.meta = make_meta(kLeafDim, count);
  v.start = start;
  *n = v;
}
template <>
__device__ __forceinline__ void store_leaf<double>(Node<double>* n, uint32_t count, uint32_t start) {
  Node<double> v;
  v.meta = make_meta(kLeafDim, count);
  v.start = start;
  v.cut = 0.0;
  *n = v;
}
__device__ __forceinline__ uint32_t node_start(const Node<float>& n) { return n.start; }
__device__ __forceinline__ uint32_t node_start(const Node<double>& n) { return n.start; }

__device__ __forceinline__ Node<float> load_node(const Node<float>* __restrict__ nodes, uint32_t i) {
  const uint2 v = __ldg(reinterpret_cast<const uint2*>(nodes) + i);
  Node<float> n;
  n.meta = v.x;
  n.start = v.y;
  return n;
}
__device__ __forceinline__ Node<double> load_node(const Node<double>* __restrict__ nodes, uint32_t i) {
  const uint4 v = __ldg(reinterpret_cast<const uint4*>(nodes) + i);
  Node<double> n;
  n.meta = v.x;
  n.start = v.y;
  n.cut = __hiloint2double((int)v.w, (int)v.z);
  return n;
}

// Order-preserving map of a float to an unsigned key (for atomic min/max).
__device__ __forceinline__ uint32_t ordered_key(float f) {
  uint32_t u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float ordered_val(uint32_t k, float) {
  const uint32_t u = (k & 0x80000000u) ? (k & 0x7fffffffu) : ~k;
  return __uint_as_float(u);
}
__device__ __forceinline__ unsigned long long ordered_key(double f) {
  unsigned long long u = (unsigned long long)__double_as_longlong(f);
  return (u & 0x8000000000000000ull) ? ~u : (u | 0x8000000000000000ull);
}
__device__ __forceinline__ double ordered_val(unsigned long long k, double) {
  const unsigned long long u = (k & 0x8000000000000000ull) ? (k & 0x7fffffffffffffffull) : ~k;
  return __longlong_as_double((long long)u);
}
template <typename T>
struct KeyOf {
  using type = uint32_t;
};
template <>
struct KeyOf<double> {
  using type = unsigned long long;
};

inline int ceil_div(int64_t a, int64_t b) { return (int)((a + b - 1) / b); }

// Index c of the range [off[c], off[c+1]) holding p (off ascending, nClouds
// ranges); used for batches of clouds stored back to back.
__device__ __forceinline__ int cloud_of(const int64_t* __restrict__ off, int nClouds, int64_t p) {
  int lo = 0, hi = nClouds - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (off[mid] <= p)
      lo = mid;
    else
      hi = mid - 1;
  }
  return lo;
}

}  // namespace nabo_gb300
