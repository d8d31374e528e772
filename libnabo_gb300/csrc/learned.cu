// learned.cu -- learned per-query search radius for exact kNN.
//
// A small MLP predicts, for each query, the log of its k-th neighbour
// distance; the search then runs with a per-query radius of
// safety * exp(prediction) (the reference's per-query maxRadii overload,
// nabo/nabo.h:351, nabo/kdtree_cpu.cpp:306-336). A query that finds fewer
// than k points inside its radius is searched again without the learned
// bound, so every result equals the plain search's.
//
// Network: inputs padded to kF = 16, two hidden layers of kH = 64 SiLU
// units, one output. Weights are BF16, sums are FP32.
//   3-D clouds: inputs = 3 normalised coordinates + 8 voxel occupancies:
//               the log point count of the voxel holding the query at 8
//               octave scales h0 * 2^s, h0 half the median k-th distance of
//               the training queries. Each scale's counts sit in a hash
//               table (open addressing) holding only occupied voxels.
//   other dims: inputs = the normalised coordinates.
// Radius: safety * exp(mu + sigma * (output + margin)); `margin` is set
// after training so that about `targetMissRate` of the training queries
// would fall outside their radius (0 when that rate is met already).
// Training: targets are log(d_k) of training queries, computed by the exact
// GPU kd-tree search; MSE on the standardised target; Adam. The training
// kernel runs on the FP32 cores and rounds weights, inputs and the first
// hidden layer to BF16 exactly where the inference kernel does, so training
// fits the network that inference evaluates. Inference uses the tensor
// cores (mma.sync m16n8k16, BF16 in, FP32 accumulate), 16 queries per warp.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <random>
#include <string>
#include <vector>

#include "internal.cuh"
#include "nabo_gb300.h"

namespace nabo_gb300 {
namespace {

constexpr int kF = 16;
constexpr int kH = 64;
constexpr int kOffW1 = 0;                  // W1[kH][kF]
constexpr int kOffB1 = kOffW1 + kH * kF;   // b1[kH]
constexpr int kOffW2 = kOffB1 + kH;        // W2[kH][kH]
constexpr int kOffB2 = kOffW2 + kH * kH;   // b2[kH]
constexpr int kOffW3 = kOffB2 + kH;        // w3[kH]
constexpr int kOffB3 = kOffW3 + kH;        // b3
constexpr int kParams = kOffB3 + 1;        // 5313
constexpr int kScales = 8;

struct FeatureSpace {
  int dim;
  int nIn;
  float center[kMaxDim];
  float invHalf[kMaxDim];
  int useGrid;
  float lo[3];
  float invH0;                     // 1 / finest voxel size
  float invLogN;                   // 1 / log1p(points)
  unsigned long long* keys[kScales];  // hash tables: voxel key (0 = empty)
  uint32_t* counts[kScales];
  uint32_t mask[kScales];          // capacity - 1 (capacity a power of two)
};

// Voxel key of integer coordinates (21 bits each); 0 is reserved for empty.
__device__ __forceinline__ unsigned long long voxel_key(int x, int y, int z) {
  return ((((unsigned long long)x & 0x1FFFFFull) << 42) | (((unsigned long long)y & 0x1FFFFFull) << 21) |
          ((unsigned long long)z & 0x1FFFFFull)) + 1ull;
}
// 64-bit finaliser (splitmix64) for the slot.
__device__ __forceinline__ unsigned long long mix64(unsigned long long z) {
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}
constexpr int kVoxelCoordMax = (1 << 21) - 1;

__device__ __forceinline__ float bf16r(float x) { return __bfloat162float(__float2bfloat16_rn(x)); }
__device__ __forceinline__ float sigm(float z) { return 1.0f / (1.0f + __expf(-z)); }

// Inference SiLU: sigma(z) = (1 + tanh(z / 2)) / 2 with the hardware tanh
// approximation (PTX tanh.approx.f32, one special-function op; relative
// error about 2^-11, below the BF16 rounding the first layer's output gets).
__device__ __forceinline__ float silu_fast(float z) {
  float t;
  asm("tanh.approx.f32 %0, %1;" : "=f"(t) : "f"(0.5f * z));
  return z * fmaf(0.5f, t, 0.5f);
}

// Occupancies of scales [s0, s0 + n) for point p: the first probe of every
// scale is issued before any is inspected (independent loads in flight);
// collisions continue with the bounded linear probe.
template <int N>
__device__ __forceinline__ void voxel_counts(const FeatureSpace& fs, int s0, const float (&p)[3], float (&out)[N]) {
  unsigned long long key[N];
  uint32_t slot[N];
  bool inside[N];
#pragma unroll
  for (int j = 0; j < N; ++j) {
    const int s = s0 + j;
    const float inv = fs.invH0 * __int_as_float((127 - s) << 23);
    int c[3];
    inside[j] = true;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      const float v = floorf((p[d] - fs.lo[d]) * inv);
      inside[j] = inside[j] && (v >= 0.0f && v <= (float)kVoxelCoordMax);
      c[d] = inside[j] ? (int)v : 0;
    }
    key[j] = voxel_key(c[0], c[1], c[2]);
    slot[j] = (uint32_t)mix64(key[j]) & fs.mask[s];
  }
  unsigned long long k0[N];
#pragma unroll
  for (int j = 0; j < N; ++j) k0[j] = inside[j] ? __ldg(fs.keys[s0 + j] + slot[j]) : 0ull;
#pragma unroll
  for (int j = 0; j < N; ++j) {
    const int s = s0 + j;
    uint32_t cnt = 0u;
    if (inside[j] && k0[j] != 0ull) {
      if (k0[j] == key[j]) {
        cnt = __ldg(fs.counts[s] + slot[j]);
      } else {
        const uint32_t mask = fs.mask[s];
        uint32_t sl = (slot[j] + 1u) & mask;
        for (uint32_t probe = 1; probe <= mask; ++probe) {
          const unsigned long long kk = fs.keys[s][sl];
          if (kk == key[j]) {
            cnt = fs.counts[s][sl];
            break;
          }
          if (kk == 0ull) break;
          sl = (sl + 1u) & mask;
        }
      }
    }
    out[j] = log1pf((float)cnt) * fs.invLogN;
  }
}

template <typename T>
__device__ __forceinline__ void features(const T* __restrict__ q, const FeatureSpace& fs, float (&out)[kF]) {
#pragma unroll
  for (int f = 0; f < kF; ++f) out[f] = 0.0f;
  for (int d = 0; d < fs.dim && d < kF; ++d) out[d] = fminf(fmaxf(((float)q[d] - fs.center[d]) * fs.invHalf[d], -4.f), 4.f);
  if (fs.useGrid) {
    const float p[3] = {(float)q[0], (float)q[1], (float)q[2]};
    float occ[kScales];
    voxel_counts<kScales>(fs, 0, p, occ);
#pragma unroll
    for (int s = 0; s < kScales; ++s) out[3 + s] = occ[s];
  }
}

// ---------------------------------------------------------------------------
// voxel grid

// Inserts every point into the scale-s table (counts its voxel). A table
// holds at least twice as many slots as there are points, so an insert
// finds its key or a free slot; the bound only makes the loop finite.
template <typename T, int D>
__global__ void k_voxel_insert(const Rec<T, D>* __restrict__ recs, int64_t n, FeatureSpace fs, int s,
                               int* overflow) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const Rec<T, D> r = recs[i];
  const float inv = fs.invH0 * __int_as_float((127 - s) << 23);
  int c[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) c[d] = min(max((int)floorf(((float)r.p.c[d] - fs.lo[d]) * inv), 0), kVoxelCoordMax);
  const unsigned long long key = voxel_key(c[0], c[1], c[2]);
  const uint32_t mask = fs.mask[s];
  uint32_t slot = (uint32_t)mix64(key) & mask;
  for (uint32_t probe = 0; probe <= mask; ++probe) {
    const unsigned long long prev = atomicCAS(fs.keys[s] + slot, 0ull, key);
    if (prev == 0ull || prev == key) {
      atomicAdd(fs.counts[s] + slot, 1u);
      return;
    }
    slot = (slot + 1u) & mask;
  }
  atomicOr(overflow, 1);
}

// ---------------------------------------------------------------------------
// training data

template <typename T>
__global__ void k_features(const T* __restrict__ query, int64_t nq, int64_t qStride, FeatureSpace fs, float* X) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= nq) return;
  float f[kF];
  features(query + i * qStride, fs, f);
#pragma unroll
  for (int j = 0; j < kF; ++j) X[i * kF + j] = f[j];
}

// y = log(d_k) from the k-th squared distance; queries without k
// neighbours (d2 = inf) get a NaN target and are left out of training.
template <typename T>
__global__ void k_targets(const T* __restrict__ d2, int64_t nq, int k, double minD2, float* y) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= nq) return;
  const double v = (double)d2[i * k + (k - 1)];
  y[i] = isinf(v) ? __int_as_float(0x7fc00000) : (float)(0.5 * log(v > minD2 ? v : minD2));
}

// ---------------------------------------------------------------------------
// training step: gradient of the mean squared error over `count` samples
// (indices idx[0..count)), accumulated into grad[kParams]. One block of 256
// threads handles kSamplesPerBlock samples in tiles of 32.

constexpr int kTile = 32;
constexpr int kTrainThreads = 256;
constexpr int kSamplesPerBlock = 256;

struct TrainSmem {
  float W1[kH * kF];   // [j][f]
  float W2T[kH * kH];  // [i][j] = W2[j][i]
  float b1[kH], b2[kH], w3[kH];
  float b3;
  float x[kTile][kF];
  float z1[kTile][kH];
  float a1[kTile][kH];
  float z2[kTile][kH];
  float a2[kTile][kH];
  float dz2[kTile][kH];
  float y[kTile], yhat[kTile], dy[kTile];
  float gW1[kH * kF];
  float gb1[kH], gb2[kH], gw3[kH];
  float gb3;
  float loss;
};

__global__ void __launch_bounds__(kTrainThreads) k_mlp_grad(const float* __restrict__ X, const float* __restrict__ Y,
                                                            const int32_t* __restrict__ idx, int count,
                                                            const __nv_bfloat16* __restrict__ Wb, float* grad,
                                                            float* lossOut, float invBatch) {
  extern __shared__ float smemRaw[];
  TrainSmem& S = *reinterpret_cast<TrainSmem*>(smemRaw);
  const int tid = threadIdx.x;
  for (int i = tid; i < kH * kF; i += kTrainThreads) {
    S.W1[i] = __bfloat162float(Wb[kOffW1 + i]);
    S.gW1[i] = 0.0f;
  }
  for (int i = tid; i < kH * kH; i += kTrainThreads) {
    const int j = i / kH, c = i % kH;
    S.W2T[c * kH + j] = __bfloat162float(Wb[kOffW2 + i]);
  }
  for (int i = tid; i < kH; i += kTrainThreads) {
    S.b1[i] = __bfloat162float(Wb[kOffB1 + i]);
    S.b2[i] = __bfloat162float(Wb[kOffB2 + i]);
    S.w3[i] = __bfloat162float(Wb[kOffW3 + i]);
    S.gb1[i] = S.gb2[i] = S.gw3[i] = 0.0f;
  }
  if (tid == 0) {
    S.b3 = __bfloat162float(Wb[kOffB3]);
    S.gb3 = 0.0f;
    S.loss = 0.0f;
  }
  // W2 gradient: thread owns entries o = tid + 256 r, r < 16 (row j = o / 64, col i = o % 64)
  float gW2[(kH * kH) / kTrainThreads];
#pragma unroll
  for (int r = 0; r < (kH * kH) / kTrainThreads; ++r) gW2[r] = 0.0f;
  __syncthreads();

  const int first = blockIdx.x * kSamplesPerBlock;
  for (int t0 = first; t0 < min(first + kSamplesPerBlock, count); t0 += kTile) {
    const int m = min(kTile, count - t0);
    // inputs
    for (int i = tid; i < kTile * kF; i += kTrainThreads) {
      const int s = i / kF, f = i % kF;
      S.x[s][f] = s < m ? bf16r(X[(int64_t)idx[t0 + s] * kF + f]) : 0.0f;
    }
    if (tid < kTile) S.y[tid] = tid < m ? Y[idx[t0 + tid]] : 0.0f;
    __syncthreads();
    // layer 1
    for (int o = tid; o < kTile * kH; o += kTrainThreads) {
      const int s = o / kH, j = o % kH;
      float z = S.b1[j];
#pragma unroll
      for (int f = 0; f < kF; ++f) z += S.W1[j * kF + f] * S.x[s][f];
      S.z1[s][j] = z;
      S.a1[s][j] = bf16r(z * sigm(z));
    }
    __syncthreads();
    // layer 2
    for (int o = tid; o < kTile * kH; o += kTrainThreads) {
      const int s = o / kH, j = o % kH;
      float z = S.b2[j];
#pragma unroll 8
      for (int i = 0; i < kH; ++i) z += S.W2T[i * kH + j] * S.a1[s][i];
      S.z2[s][j] = z;
      S.a2[s][j] = z * sigm(z);
    }
    __syncthreads();
    // output and loss: one warp per 4 samples
    {
      const int warp = tid >> 5, lane = tid & 31;
      for (int s = warp; s < kTile; s += kTrainThreads / 32) {
        float acc = S.w3[lane] * S.a2[s][lane] + S.w3[lane + 32] * S.a2[s][lane + 32];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (lane == 0) {
          const float yh = acc + S.b3;
          const float e = s < m ? yh - S.y[s] : 0.0f;
          S.yhat[s] = yh;
          S.dy[s] = 2.0f * e * invBatch;
          atomicAdd(&S.loss, e * e);
        }
      }
    }
    __syncthreads();
    // output layer gradients and dz2
    if (tid < kH) {
      float g = 0.0f;
      for (int s = 0; s < m; ++s) g += S.dy[s] * S.a2[s][tid];
      S.gw3[tid] += g;
    }
    if (tid == kH) {
      float g = 0.0f;
      for (int s = 0; s < m; ++s) g += S.dy[s];
      S.gb3 += g;
    }
    for (int o = tid; o < kTile * kH; o += kTrainThreads) {
      const int s = o / kH, j = o % kH;
      const float z = S.z2[s][j];
      const float sg = sigm(z);
      S.dz2[s][j] = s < m ? S.dy[s] * S.w3[j] * sg * (1.0f + z * (1.0f - sg)) : 0.0f;
    }
    __syncthreads();
    // W2, b2 gradients
#pragma unroll
    for (int r = 0; r < (kH * kH) / kTrainThreads; ++r) {
      const int o = tid + kTrainThreads * r;
      const int j = o / kH, i = o % kH;
      float g = 0.0f;
      for (int s = 0; s < m; ++s) g += S.dz2[s][j] * S.a1[s][i];
      gW2[r] += g;
    }
    if (tid < kH) {
      float g = 0.0f;
      for (int s = 0; s < m; ++s) g += S.dz2[s][tid];
      S.gb2[tid] += g;
    }
    // back through layer 2 into dz1 (stored in z1; the rounding of a1 to
    // BF16 is passed straight through)
    for (int o = tid; o < kTile * kH; o += kTrainThreads) {
      const int s = o / kH, i = o % kH;
      float g = 0.0f;
#pragma unroll 8
      for (int j = 0; j < kH; ++j) g += S.W2T[i * kH + j] * S.dz2[s][j];
      const float z = S.z1[s][i];
      const float sg = sigm(z);
      S.a2[s][i] = g * sg * (1.0f + z * (1.0f - sg));  // reuse a2 as dz1
    }
    __syncthreads();
    // W1, b1 gradients
    for (int o = tid; o < kH * kF; o += kTrainThreads) {
      const int j = o / kF, f = o % kF;
      float g = 0.0f;
      for (int s = 0; s < m; ++s) g += S.a2[s][j] * S.x[s][f];
      S.gW1[o] += g;
    }
    if (tid < kH) {
      float g = 0.0f;
      for (int s = 0; s < m; ++s) g += S.a2[s][tid];
      S.gb1[tid] += g;
    }
    __syncthreads();
  }
  // flush
#pragma unroll
  for (int r = 0; r < (kH * kH) / kTrainThreads; ++r) atomicAdd(grad + kOffW2 + tid + kTrainThreads * r, gW2[r]);
  for (int i = tid; i < kH * kF; i += kTrainThreads) atomicAdd(grad + kOffW1 + i, S.gW1[i]);
  if (tid < kH) {
    atomicAdd(grad + kOffB1 + tid, S.gb1[tid]);
    atomicAdd(grad + kOffB2 + tid, S.gb2[tid]);
    atomicAdd(grad + kOffW3 + tid, S.gw3[tid]);
  }
  if (tid == 0) {
    atomicAdd(grad + kOffB3, S.gb3);
    if (lossOut) atomicAdd(lossOut, S.loss);
  }
}

__global__ void k_adam(float* p, float* m, float* v, float* g, __nv_bfloat16* pb, int n, float lr, float b1,
                       float b2, float c1, float c2, float eps) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float gi = g[i];
  const float mi = b1 * m[i] + (1.0f - b1) * gi;
  const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  const float pi = p[i] - lr * (mi * c1) / (sqrtf(vi * c2) + eps);
  p[i] = pi;
  pb[i] = __float2bfloat16_rn(pi);
  g[i] = 0.0f;
}

__global__ void k_to_bf16(const float* p, __nv_bfloat16* pb, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) pb[i] = __float2bfloat16_rn(p[i]);
}

// ---------------------------------------------------------------------------
// inference: 16 queries per warp on the tensor cores

__device__ __forceinline__ void mma16816(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

__device__ __forceinline__ uint32_t pack2(float lo, float hi) {
  const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<const uint32_t*>(&v);
}

struct RadiusOut {
  float mu, sigma, safety, margin;
  double maxRadius;
};

constexpr int kInferWarps = 8;

// The network's weights in shared memory.
struct InferSmem {
  __nv_bfloat16 W1[kH * kF];
  __nv_bfloat16 W2[kH * kH];
  float b1[kH], b2[kH], w3[kH];
  float b3;
  __nv_bfloat16 X[kInferWarps][16 * kF];
};

__device__ __forceinline__ void stage_weights(InferSmem& sm, const __nv_bfloat16* __restrict__ Wb) {
  const int tid = threadIdx.x;
  for (int i = tid; i < kH * kF; i += blockDim.x) sm.W1[i] = Wb[kOffW1 + i];
  for (int i = tid; i < kH * kH; i += blockDim.x) sm.W2[i] = Wb[kOffW2 + i];
  for (int i = tid; i < kH; i += blockDim.x) {
    sm.b1[i] = __bfloat162float(Wb[kOffB1 + i]);
    sm.b2[i] = __bfloat162float(Wb[kOffB2 + i]);
    sm.w3[i] = __bfloat162float(Wb[kOffW3 + i]);
  }
  if (tid == 0) sm.b3 = __bfloat162float(Wb[kOffB3]);
}

// The network on the warp's 16 feature rows (sm.X[warp], queries q0 ..
// q0 + 15) on the tensor cores; writes each query's radius (capped at
// ro.maxRadius) and, if rawOut, its standardised output.
template <typename T>
__device__ __forceinline__ void mlp_tile(const InferSmem& sm, int warp, int lane, int64_t q0, int64_t nq,
                                         const RadiusOut& ro, T* radii, float* rawOut) {
  const int g = lane >> 2, tig = lane & 3;
  const uint32_t* X32 = reinterpret_cast<const uint32_t*>(sm.X[warp]);  // row = 8 words
  uint32_t a[4];
  a[0] = X32[g * 8 + tig];
  a[1] = X32[(g + 8) * 8 + tig];
  a[2] = X32[g * 8 + 4 + tig];
  a[3] = X32[(g + 8) * 8 + 4 + tig];
  // layer 1: 8 n-tiles of 8 hidden units
  const uint32_t* W1w = reinterpret_cast<const uint32_t*>(sm.W1);  // row j = 8 words
  float z1[8][4];
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    z1[j][0] = z1[j][1] = z1[j][2] = z1[j][3] = 0.0f;
    const int n = 8 * j + g;
    mma16816(z1[j], a, W1w[n * 8 + tig], W1w[n * 8 + 4 + tig]);
  }
  // SiLU, BF16, repacked as the A operand of layer 2 (4 k-steps); fragment
  // order for m16n8k16 A: {row g k0-7, row g+8 k0-7, row g k8-15, row g+8
  // k8-15}
  uint32_t A2[4][4];
#pragma unroll
  for (int s = 0; s < 4; ++s) {
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int j = 2 * s + h;
      const int c = 8 * j + 2 * tig;
      float v[4];
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const float z = z1[j][e] + sm.b1[c + (e & 1)];
        v[e] = silu_fast(z);
      }
      A2[s][2 * h + 0] = pack2(v[0], v[1]);
      A2[s][2 * h + 1] = pack2(v[2], v[3]);
    }
  }
  // layer 2
  const uint32_t* W2w = reinterpret_cast<const uint32_t*>(sm.W2);  // row j = 32 words
  float z2[8][4];
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    z2[j][0] = z2[j][1] = z2[j][2] = z2[j][3] = 0.0f;
    const int n = 8 * j + g;
#pragma unroll
    for (int s = 0; s < 4; ++s) mma16816(z2[j], A2[s], W2w[n * 32 + 8 * s + tig], W2w[n * 32 + 8 * s + 4 + tig]);
  }
  // output layer: rows g and g+8
  float y0 = 0.0f, y1 = 0.0f;
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    const int c = 8 * j + 2 * tig;
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const float z = z2[j][e] + sm.b2[c + (e & 1)];
      const float act = silu_fast(z) * sm.w3[c + (e & 1)];
      if (e < 2)
        y0 += act;
      else
        y1 += act;
    }
  }
  y0 += __shfl_xor_sync(0xffffffffu, y0, 1);
  y0 += __shfl_xor_sync(0xffffffffu, y0, 2);
  y1 += __shfl_xor_sync(0xffffffffu, y1, 1);
  y1 += __shfl_xor_sync(0xffffffffu, y1, 2);
  if (tig == 0) {
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int64_t qi = q0 + g + 8 * h;
      if (qi < nq) {
        const float yn = (h == 0 ? y0 : y1) + sm.b3;
        if (rawOut) rawOut[qi] = yn;
        // single precision: the radius only steers the search, the
        // results are exact whatever it is
        const float r = ro.safety * expf(ro.mu + ro.sigma * (yn + ro.margin));
        radii[qi] = (double)r < ro.maxRadius ? (T)r : (T)ro.maxRadius;
      }
    }
  }
}

template <typename T>
__global__ void __launch_bounds__(kInferWarps * 32) k_mlp_radius(const T* __restrict__ query, int64_t nq,
                                                                 int64_t qStride, FeatureSpace fs,
                                                                 const __nv_bfloat16* __restrict__ Wb, RadiusOut ro,
                                                                 T* radii, float* rawOut) {
  __shared__ __align__(16) InferSmem sm;
  stage_weights(sm, Wb);
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t tiles = (nq + 15) / 16;
  for (int64_t tile = (int64_t)blockIdx.x * kInferWarps + warp; tile < tiles; tile += (int64_t)gridDim.x * kInferWarps) {
    const int64_t q0 = tile * 16;
    // features of the tile's 16 queries: lanes l and l + 16 share query l;
    // the first lane writes the coordinates and the finer half of the voxel
    // scales, the second the coarser half
    {
      const int row = lane & 15;
      const bool second = lane >= 16;
      const int64_t qi = q0 + row;
      __nv_bfloat16* xr = sm.X[warp] + row * kF;
      if (qi < nq) {
        const T* qp = query + qi * qStride;
        if (fs.useGrid) {
          const float p[3] = {(float)qp[0], (float)qp[1], (float)qp[2]};
          float occ[kScales / 2];
          voxel_counts<kScales / 2>(fs, second ? kScales / 2 : 0, p, occ);
#pragma unroll
          for (int j = 0; j < kScales / 2; ++j) xr[3 + (second ? kScales / 2 : 0) + j] = __float2bfloat16_rn(occ[j]);
          if (!second) {
#pragma unroll
            for (int d = 0; d < 3; ++d)
              xr[d] = __float2bfloat16_rn(fminf(fmaxf(((float)qp[d] - fs.center[d]) * fs.invHalf[d], -4.f), 4.f));
          } else {
#pragma unroll
            for (int j = 3 + kScales; j < kF; ++j) xr[j] = __float2bfloat16_rn(0.0f);
          }
        } else if (!second) {
          float f[kF];
          features(qp, fs, f);
#pragma unroll
          for (int j = 0; j < kF; ++j) xr[j] = __float2bfloat16_rn(f[j]);
        }
      } else if (!second) {
#pragma unroll
        for (int j = 0; j < kF; ++j) xr[j] = __float2bfloat16_rn(0.0f);
      }
    }
    __syncwarp();
    mlp_tile<T>(sm, warp, lane, q0, nq, ro, radii, rawOut);
    __syncwarp();
  }
}

// ---------------------------------------------------------------------------
// batched models: one network per (dimension, scalar type) for the clouds of
// batches, its 8 inputs taken from each query's own cloud and tree, so that
// one network serves clouds of every size and density

constexpr int kBatchInputs = 8;

template <typename T>
struct BatchFeat {
  const Node<T>* nodes;
  const void* recs;  // Rec<T, D>
  const int64_t* pointOff;
  const int64_t* nodeOffset;
  const T* rootLo;
  const T* rootHi;
  const int64_t* qOffset;
  const int32_t* kOf;
  int nClouds;
  int dim;
};

// Raw inputs of query qi: the query descends its cloud's tree to its home
// leaf (the near side at every node, as the search's first descent does);
// from that leaf's points the logs of the nearest, root-mean-square and
// farthest distances and of the point count; the log of the cloud's size
// and of its k; the leaf's depth; the mean log extent of the leaf's cell
// (the cloud's root box narrowed by the cuts on the way).
template <typename T, int D>
__device__ void batch_raw_features(const T* __restrict__ q, int64_t qi, const BatchFeat<T>& bf,
                                   float (&f)[kBatchInputs]) {
  const int c = cloud_of(bf.qOffset, bf.nClouds, qi);
  T qv[D];
  float lo[D], hi[D];
#pragma unroll
  for (int d = 0; d < D; ++d) {
    qv[d] = d < bf.dim ? q[d] : T(0);
    lo[d] = d < bf.dim ? (float)bf.rootLo[(int64_t)c * kMaxDim + d] : 0.0f;
    hi[d] = d < bf.dim ? (float)bf.rootHi[(int64_t)c * kMaxDim + d] : 0.0f;
  }
  uint32_t node = (uint32_t)bf.nodeOffset[c];
  int depth = 0;
  Node<T> nd = load_node(bf.nodes, node);
  while (!node_is_leaf(nd.meta)) {
    const int cd = (int)node_dim(nd.meta);
    T qc = qv[0];
#pragma unroll
    for (int d = 1; d < D; ++d)
      if (cd == d) qc = qv[d];
    const bool right = qc - nd.cut > T(0);
    const float cut = (float)nd.cut;
#pragma unroll
    for (int d = 0; d < D; ++d) {
      if (cd == d && right) lo[d] = cut;
      if (cd == d && !right) hi[d] = cut;
    }
    node = right ? node_payload(nd.meta) : node + 1;
    ++depth;
    nd = load_node(bf.nodes, node);
  }
  const uint32_t cnt = node_payload(nd.meta), start = node_start(nd);
  const Rec<T, D>* recs = static_cast<const Rec<T, D>*>(bf.recs);
  float mn = 3.0e38f, mx = 0.0f, sum = 0.0f;
  for (uint32_t j = 0; j < cnt; ++j) {
    Rec<T, D> r;
    load_rec(recs, (int64_t)start + j, r);
    float d2 = 0.0f;
#pragma unroll
    for (int d = 0; d < D; ++d) {
      const float v = (float)(qv[d] - r.p.c[d]);
      d2 += v * v;
    }
    mn = fminf(mn, d2);
    mx = fmaxf(mx, d2);
    sum += d2;
  }
  const float tiny = 1e-30f;
  const float n = (float)(cnt > 0 ? cnt : 1u);
  f[0] = 0.5f * logf(fmaxf(mn, tiny));
  f[1] = 0.5f * logf(fmaxf(sum / n, tiny));
  f[2] = 0.5f * logf(fmaxf(mx, tiny));
  f[3] = logf(n);
  f[4] = logf((float)(bf.pointOff[c + 1] - bf.pointOff[c]));
  f[5] = logf((float)bf.kOf[c]);
  f[6] = (float)depth;
  float le = 0.0f;
  for (int d = 0; d < bf.dim && d < D; ++d) le += logf(fmaxf(hi[d] - lo[d], tiny));
  f[7] = le / (float)(bf.dim > 0 ? bf.dim : 1);
}

// The network's inputs: raw inputs centred and scaled by the training set's
// statistics (fs.center, fs.invHalf), clamped to [-4, 4]; padding 0.
__device__ __forceinline__ float batch_input(const float (&f)[kBatchInputs], const FeatureSpace& fs, int j) {
  return j < kBatchInputs ? fminf(fmaxf((f[j] - fs.center[j]) * fs.invHalf[j], -4.f), 4.f) : 0.0f;
}

// Raw inputs (normalise = 0) or network inputs (1) of nq queries into X
// (nq x kF floats).
template <typename T, int D>
__global__ void k_batch_features(const T* __restrict__ query, int64_t nq, BatchFeat<T> bf, FeatureSpace fs,
                                 int normalise, float* X) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= nq) return;
  float f[kBatchInputs];
  batch_raw_features<T, D>(query + i * bf.dim, i, bf, f);
#pragma unroll
  for (int j = 0; j < kF; ++j) X[i * kF + j] = normalise ? batch_input(f, fs, j) : (j < kBatchInputs ? f[j] : 0.0f);
}

// Targets of batched training queries: log of the k-th distance of each
// query's own cloud's k (NaN when it has fewer neighbours).
template <typename T>
__global__ void k_batch_targets(const T* __restrict__ d2, int64_t nq, const int64_t* __restrict__ qOffset,
                                const int64_t* __restrict__ outOffset, const int32_t* __restrict__ kOf, int nClouds,
                                double minD2, float* y) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= nq) return;
  const int c = cloud_of(qOffset, nClouds, i);
  const int k = kOf[c];
  const T v = d2[outOffset[c] + (i - qOffset[c]) * k + (k - 1)];
  y[i] = isinf((double)v) ? __int_as_float(0x7fc00000) : (float)(0.5 * log(fmax((double)v, minD2)));
}

template <typename T, int D>
__global__ void __launch_bounds__(kInferWarps * 32) k_mlp_radius_batch(const T* __restrict__ query, int64_t nq,
                                                                       BatchFeat<T> bf, FeatureSpace fs,
                                                                       const __nv_bfloat16* __restrict__ Wb,
                                                                       RadiusOut ro, T* radii, float* rawOut) {
  __shared__ __align__(16) InferSmem sm;
  stage_weights(sm, Wb);
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t tiles = (nq + 15) / 16;
  for (int64_t tile = (int64_t)blockIdx.x * kInferWarps + warp; tile < tiles; tile += (int64_t)gridDim.x * kInferWarps) {
    const int64_t q0 = tile * 16;
    if (lane < 16) {
      const int64_t qi = q0 + lane;
      __nv_bfloat16* xr = sm.X[warp] + lane * kF;
      float f[kBatchInputs];
      if (qi < nq) {
        batch_raw_features<T, D>(query + qi * bf.dim, qi, bf, f);
      } else {
#pragma unroll
        for (int j = 0; j < kBatchInputs; ++j) f[j] = fs.center[j];
      }
#pragma unroll
      for (int j = 0; j < kF; ++j) xr[j] = __float2bfloat16_rn(batch_input(f, fs, j));
    }
    __syncwarp();
    mlp_tile<T>(sm, warp, lane, q0, nq, ro, radii, rawOut);
    __syncwarp();
  }
}

}  // namespace

// ---------------------------------------------------------------------------
// host side

struct RadiusModel {
  int dtype = 0;
  int dim = 0;
  int dpad = 0;
  int k = 1;
  const void* owner = nullptr;  // the search object the model was trained on
  FeatureSpace fs{};
  void* tables = nullptr;   // all scales' keys and counts
  float margin = 0.0f;      // calibration offset added to the standardised output
  double h0 = 0.0;          // finest voxel size (3-D features)
  float* params = nullptr;  // FP32 master
  float* adamM = nullptr;
  float* adamV = nullptr;
  float* grad = nullptr;
  __nv_bfloat16* pb = nullptr;
  float mu = 0.0f, sigma = 1.0f, safety = 1.2f;
  float trainLoss = 0.0f;
  int64_t trainSamples = 0;
  int kind = 0;  // 0: one cloud's model; 1: a batched model (inputs from the query's own cloud and tree)
};

namespace {

void free_model(RadiusModel* m) {
  if (m->tables) cudaFree(m->tables);
  if (m->params) cudaFree(m->params);
  if (m->adamM) cudaFree(m->adamM);
  if (m->adamV) cudaFree(m->adamV);
  if (m->grad) cudaFree(m->grad);
  if (m->pb) cudaFree(m->pb);
}

// Feature normalisation, and for 3-D clouds the voxel tables at the
// scales h0 * 2^s.
template <typename T, int D>
int build_grid(const DeviceCloud& c, RadiusModel* m, double h0, cudaStream_t st) {
  FeatureSpace& fs = m->fs;
  fs.dim = c.dim;
  for (int d = 0; d < kMaxDim; ++d) {
    const double lo = d < c.dim ? c.lo[d] : 0.0, hi = d < c.dim ? c.hi[d] : 0.0;
    fs.center[d] = (float)(0.5 * (lo + hi));
    const double half = 0.5 * (hi - lo);
    fs.invHalf[d] = half > 0.0 ? (float)(1.0 / half) : 0.0f;
  }
  fs.useGrid = (c.dim == 3) ? 1 : 0;
  fs.nIn = fs.useGrid ? 3 + kScales : std::min(c.dim, kF);
  if (!fs.useGrid) return kOk;
  if constexpr (D == 3) {
    double ext = 0.0;
    for (int d = 0; d < 3; ++d) ext = std::max(ext, c.hi[d] - c.lo[d]);
    if (!(ext > 0.0)) ext = 1.0;
    // the finest voxel: at least ext / 2^20 so voxel coordinates fit 21 bits
    h0 = std::max(h0, ext / (double)(1 << 20));
    m->h0 = h0;
    fs.invH0 = (float)(1.0 / h0);
    fs.invLogN = (float)(1.0 / std::log1p((double)c.n));
    for (int d = 0; d < 3; ++d) fs.lo[d] = (float)c.lo[d];
    size_t total = 0;
    uint32_t cap[kScales];
    for (int s = 0; s < kScales; ++s) {
      double cells = 1.0;
      for (int d = 0; d < 3; ++d) cells *= std::floor((c.hi[d] - c.lo[d]) / (h0 * std::ldexp(1.0, s))) + 1.0;
      const double need = 2.0 * std::min((double)c.n, cells);
      uint32_t cp = 64;
      while ((double)cp < need && cp < (1u << 30)) cp <<= 1;
      cap[s] = cp;
      fs.mask[s] = cp - 1;
      total += (size_t)cp * (sizeof(unsigned long long) + sizeof(uint32_t));
    }
    NABO_CUDA_TRY(cudaMalloc(&m->tables, total + sizeof(int)));
    NABO_CUDA_TRY(cudaMemsetAsync(m->tables, 0, total + sizeof(int), st));
    unsigned char* p = static_cast<unsigned char*>(m->tables);
    for (int s = 0; s < kScales; ++s) {
      fs.keys[s] = reinterpret_cast<unsigned long long*>(p);
      p += (size_t)cap[s] * sizeof(unsigned long long);
    }
    for (int s = 0; s < kScales; ++s) {
      fs.counts[s] = reinterpret_cast<uint32_t*>(p);
      p += (size_t)cap[s] * sizeof(uint32_t);
    }
    int* overflow = reinterpret_cast<int*>(p);
    for (int s = 0; s < kScales; ++s)
      k_voxel_insert<T, D><<<ceil_div(c.n, 256), 256, 0, st>>>(static_cast<const Rec<T, D>*>(c.recs), c.n, fs, s,
                                                               overflow);
    int hov = 0;
    NABO_CUDA_TRY(cudaGetLastError());
    NABO_CUDA_TRY(cudaMemcpyAsync(&hov, overflow, sizeof(int), cudaMemcpyDeviceToHost, st));
    NABO_CUDA_TRY(cudaStreamSynchronize(st));
    if (hov) return set_error(kErrInternal, "voxel table overflow");
    return kOk;
  } else {
    return set_error(kErrInternal, "voxel features need 3-D records");
  }
}

int launch_radius(const RadiusModel& m, const void* query, int64_t nq, int64_t qStride, double maxRadius, void* radii,
                  float* raw, cudaStream_t st) {
  if (nq == 0) return kOk;
  RadiusOut ro;
  ro.mu = m.mu;
  ro.sigma = m.sigma;
  ro.safety = m.safety;
  ro.margin = m.margin;
  ro.maxRadius = maxRadius;
  const int64_t tiles = (nq + 15) / 16;
  const int grid = (int)std::min<int64_t>(ceil_div(tiles, kInferWarps), 152 * 16);
  if (m.dtype == NABO_CUDA_FLOAT32)
    k_mlp_radius<float><<<grid, kInferWarps * 32, 0, st>>>(static_cast<const float*>(query), nq, qStride, m.fs, m.pb,
                                                             ro, static_cast<float*>(radii), raw);
  else
    k_mlp_radius<double><<<grid, kInferWarps * 32, 0, st>>>(static_cast<const double*>(query), nq, qStride, m.fs,
                                                              m.pb, ro, static_cast<double*>(radii), raw);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_error(e, "learned radius kernel");
  return kOk;
}

int launch_features(const RadiusModel& m, const void* query, int64_t nq, int64_t qStride, float* X, cudaStream_t st) {
  if (m.dtype == NABO_CUDA_FLOAT32)
    k_features<float><<<ceil_div(nq, 256), 256, 0, st>>>(static_cast<const float*>(query), nq, qStride, m.fs, X);
  else
    k_features<double><<<ceil_div(nq, 256), 256, 0, st>>>(static_cast<const double*>(query), nq, qStride, m.fs, X);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_error(e, "features kernel");
  return kOk;
}

size_t train_smem() { return sizeof(TrainSmem); }

int grad_step(const RadiusModel& m, const float* X, const float* Y, const int32_t* idx, int count, float* lossDev,
              cudaStream_t st) {
  NABO_CUDA_TRY(cudaFuncSetAttribute(k_mlp_grad, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)train_smem()));
  const int blocks = ceil_div(count, kSamplesPerBlock);
  k_mlp_grad<<<blocks, kTrainThreads, train_smem(), st>>>(X, Y, idx, count, m.pb, m.grad, lossDev,
                                                          1.0f / (float)count);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_error(e, "training kernel");
  return kOk;
}

// Initial weights: uniform(+-1/sqrt(fan_in)) from a seeded generator.
std::vector<float> init_params(uint64_t seed, int nIn) {
  std::mt19937_64 rng(seed);
  std::vector<float> p(kParams, 0.0f);
  auto fill = [&](int off, int count, double bound) {
    std::uniform_real_distribution<double> u(-bound, bound);
    for (int i = 0; i < count; ++i) p[off + i] = (float)u(rng);
  };
  fill(kOffW1, kH * kF, 1.0 / std::sqrt((double)std::max(nIn, 1)));
  for (int j = 0; j < kH; ++j)
    for (int f = nIn; f < kF; ++f) p[kOffW1 + j * kF + f] = 0.0f;
  fill(kOffW2, kH * kH, 1.0 / std::sqrt((double)kH));
  fill(kOffW3, kH, 1.0 / std::sqrt((double)kH));
  return p;
}

template <typename T>
int dispatch_grid(const DeviceCloud& c, RadiusModel* m, double h0, cudaStream_t st) {
  switch (c.dpad) {
    case 2: return build_grid<T, 2>(c, m, h0, st);
    case 3: return build_grid<T, 3>(c, m, h0, st);
    case 4: return build_grid<T, 4>(c, m, h0, st);
    case 8: return build_grid<T, 8>(c, m, h0, st);
    case 16: return build_grid<T, 16>(c, m, h0, st);
  }
  return set_error(kErrInternal, "bad dispatch");
}

int search_plain(const DeviceCloud& c, const KnnArgs& a, cudaStream_t st) {
#define NABO_L_CASE(TT, DD) \
  if (c.dpad == DD) return knn_kdtree<TT, DD>(c, a, st);
  if (c.dtype == NABO_CUDA_FLOAT32) {
    NABO_L_CASE(float, 2) NABO_L_CASE(float, 3) NABO_L_CASE(float, 4) NABO_L_CASE(float, 8) NABO_L_CASE(float, 16)
  } else {
    NABO_L_CASE(double, 2) NABO_L_CASE(double, 3) NABO_L_CASE(double, 4) NABO_L_CASE(double, 8)
    NABO_L_CASE(double, 16)
  }
#undef NABO_L_CASE
  return set_error(kErrInternal, "bad dispatch");
}

int leaf_order(const DeviceCloud& c, const void* query, int64_t nq, int64_t qStride, int32_t* order, cudaStream_t st) {
#define NABO_L_CASE(TT, DD) \
  if (c.dpad == DD) return knn_leaf_order<TT, DD>(c, query, nq, qStride, order, st);
  if (c.dtype == NABO_CUDA_FLOAT32) {
    NABO_L_CASE(float, 2) NABO_L_CASE(float, 3) NABO_L_CASE(float, 4) NABO_L_CASE(float, 8) NABO_L_CASE(float, 16)
  } else {
    NABO_L_CASE(double, 2) NABO_L_CASE(double, 3) NABO_L_CASE(double, 4) NABO_L_CASE(double, 8)
    NABO_L_CASE(double, 16)
  }
#undef NABO_L_CASE
  return set_error(kErrInternal, "bad dispatch");
}

int search_given(const DeviceCloud& c, const KnnArgs& a, const int32_t* order, cudaStream_t st) {
#define NABO_L_CASE(TT, DD) \
  if (c.dpad == DD) return knn_kdtree_given_order<TT, DD>(c, a, order, st);
  if (c.dtype == NABO_CUDA_FLOAT32) {
    NABO_L_CASE(float, 2) NABO_L_CASE(float, 3) NABO_L_CASE(float, 4) NABO_L_CASE(float, 8) NABO_L_CASE(float, 16)
  } else {
    NABO_L_CASE(double, 2) NABO_L_CASE(double, 3) NABO_L_CASE(double, 4) NABO_L_CASE(double, 8)
    NABO_L_CASE(double, 16)
  }
#undef NABO_L_CASE
  return set_error(kErrInternal, "bad dispatch");
}

}  // namespace

// Fits the parameters to standardised targets Y over the samples `valid`
// (features X): minibatches of tp.batch, Adam with a cosine learning-rate
// decay over tp.epochs; `order` (as many ints as samples) and `loss` (one
// float) are scratch. Leaves the last epoch's mean loss in m->trainLoss.
int fit_params(RadiusModel* m, const float* X, const float* Y, const std::vector<int32_t>& valid,
               const nabo_cuda_train_params& tp, int32_t* order, float* loss, cudaStream_t st) {
  const std::vector<float> p0 = init_params(tp.seed, m->fs.nIn);
  cudaError_t e = cudaMemcpyAsync(m->params, p0.data(), kParams * sizeof(float), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemsetAsync(m->adamM, 0, kParams * sizeof(float), st);
  if (e == cudaSuccess) e = cudaMemsetAsync(m->adamV, 0, kParams * sizeof(float), st);
  if (e == cudaSuccess) e = cudaMemsetAsync(m->grad, 0, kParams * sizeof(float), st);
  if (e != cudaSuccess) return cuda_error(e, "model init");
  k_to_bf16<<<ceil_div(kParams, 256), 256, 0, st>>>(m->params, m->pb, kParams);
  int rc = kOk;
  std::mt19937_64 rng(tp.seed ^ 0x9e3779b97f4a7c15ull);
  const int nValid = (int)valid.size();
  const int batch = std::max(32, std::min(tp.batch, nValid));
  const int stepsPerEpoch = std::max(1, nValid / batch);
  const int epochs = std::max(1, tp.epochs);
  const int total = epochs * stepsPerEpoch;
  std::vector<int32_t> perm(valid);
  int step = 0;
  float lastLoss = 0.0f;
  for (int ep = 0; ep < epochs && rc == kOk; ++ep) {
    std::shuffle(perm.begin(), perm.end(), rng);
    e = cudaMemcpyAsync(order, perm.data(), perm.size() * sizeof(int32_t), cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return cuda_error(e, "batch upload");
    const bool lastEpoch = ep + 1 == epochs;
    if (lastEpoch) cudaMemsetAsync(loss, 0, sizeof(float), st);
    for (int b = 0; b < stepsPerEpoch && rc == kOk; ++b, ++step) {
      rc = grad_step(*m, X, Y, order + (size_t)b * batch, batch, lastEpoch ? loss : nullptr, st);
      const double lr = tp.lr * 0.5 * (1.0 + std::cos(3.14159265358979323846 * step / total));
      const float b1 = 0.9f, b2 = 0.999f;
      const float c1 = (float)(1.0 / (1.0 - std::pow(b1, step + 1)));
      const float c2 = (float)(1.0 / (1.0 - std::pow(b2, step + 1)));
      k_adam<<<ceil_div(kParams, 256), 256, 0, st>>>(m->params, m->adamM, m->adamV, m->grad, m->pb, kParams,
                                                     (float)lr, b1, b2, c1, c2, 1e-8f);
    }
    if (lastEpoch && rc == kOk) {
      e = cudaMemcpyAsync(&lastLoss, loss, sizeof(float), cudaMemcpyDeviceToHost, st);
      if (e == cudaSuccess) e = cudaStreamSynchronize(st);
      if (e != cudaSuccess) rc = cuda_error(e, "training");
    }
  }
  m->trainLoss = lastLoss / (float)((size_t)stepsPerEpoch * batch);
  m->trainSamples = nValid;
  return rc;
}

// The margin: the residual quantile such that about tp.targetMissRate of the
// training samples would fall outside their radius. hy holds the
// standardised targets, raw (device, n) the network's outputs on them.
int calibrate_margin(RadiusModel* m, const std::vector<float>& hy, const std::vector<int32_t>& valid, const float* raw,
                     int64_t n, const nabo_cuda_train_params& tp, cudaStream_t st) {
  std::vector<float> hraw((size_t)n);
  cudaError_t e = cudaMemcpyAsync(hraw.data(), raw, (size_t)n * sizeof(float), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return cuda_error(e, "calibration");
  std::vector<float> res;
  res.reserve(valid.size());
  for (int32_t i : valid) res.push_back(hy[(size_t)i] - hraw[(size_t)i]);
  const size_t qi = std::min(res.size() - 1, (size_t)std::ceil((1.0 - tp.targetMissRate) * (double)res.size()));
  std::nth_element(res.begin(), res.begin() + qi, res.end());
  const double need = (double)res[qi] - std::log((double)m->safety) / (double)m->sigma;
  m->margin = (float)std::max(0.0, need);
  return kOk;
}

// Standardises the targets in hy (NaN: no k-th neighbour, left out): sets
// m->mu and m->sigma, returns the valid samples and the median d_k.
int standardise_targets(RadiusModel* m, std::vector<float>& hy, std::vector<int32_t>* valid, double* medianDk) {
  double sum = 0.0, sq = 0.0;
  std::vector<float> logs;
  for (size_t i = 0; i < hy.size(); ++i) {
    if (std::isnan(hy[i])) continue;
    valid->push_back((int32_t)i);
    logs.push_back(hy[i]);
    sum += hy[i];
    sq += (double)hy[i] * hy[i];
  }
  if (valid->size() < 16) return set_error(kErrArgument, "too few training queries have k neighbours within maxRadius");
  std::nth_element(logs.begin(), logs.begin() + logs.size() / 2, logs.end());
  *medianDk = std::exp((double)logs[logs.size() / 2]);
  const double mean = sum / valid->size();
  const double var = std::max(sq / valid->size() - mean * mean, 1e-12);
  m->mu = (float)mean;
  m->sigma = (float)std::sqrt(var);
  for (float& y : hy)
    if (!std::isnan(y)) y = (float)((y - mean) / m->sigma);
  return kOk;
}

// Trains a radius model for k-NN searches of `s` on `nTrain` training
// queries (device memory).
int radius_model_train(const nabo_cuda_search* s, const void* dTrain, int64_t nTrain, int64_t qStride, int k,
                       unsigned optionFlags, double maxRadius, const nabo_cuda_train_params& tp, RadiusModel** out,
                       cudaStream_t st) {
  const HandleView h = handle_view(s);
  const DeviceCloud& c = *h.cloud;
  RadiusModel* m = new RadiusModel();
  m->dtype = c.dtype;
  m->dim = c.dim;
  m->dpad = c.dpad;
  m->k = k;
  m->owner = s;
  m->safety = tp.safety;
  const size_t es = c.dtype == NABO_CUDA_FLOAT32 ? 4 : 8;
  int rc = kOk;
  auto fail = [&](int code) {
    cudaStreamSynchronize(st);
    free_model(m);
    delete m;
    return code;
  };
  cudaError_t e = cudaMalloc((void**)&m->params, kParams * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc((void**)&m->adamM, kParams * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc((void**)&m->adamV, kParams * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc((void**)&m->grad, kParams * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc((void**)&m->pb, kParams * sizeof(__nv_bfloat16));
  if (e != cudaSuccess) return fail(cuda_error(e, "model allocation"));

  // exact k-th distances of the training queries
  int32_t* idx = nullptr;
  void* d2 = nullptr;
  float *X = nullptr, *Y = nullptr, *loss = nullptr, *raw = nullptr;
  int32_t* order = nullptr;
  void* radii = nullptr;
  e = scratch_alloc((void**)&idx, (size_t)nTrain * k * sizeof(int32_t), st);
  if (e == cudaSuccess) e = scratch_alloc(&d2, (size_t)nTrain * k * es, st);
  if (e == cudaSuccess) e = scratch_alloc((void**)&X, (size_t)nTrain * kF * sizeof(float), st);
  if (e == cudaSuccess) e = scratch_alloc((void**)&Y, (size_t)nTrain * sizeof(float), st);
  if (e == cudaSuccess) e = scratch_alloc((void**)&loss, sizeof(float), st);
  if (e == cudaSuccess) e = scratch_alloc((void**)&order, (size_t)nTrain * sizeof(int32_t), st);
  if (e == cudaSuccess) e = scratch_alloc((void**)&raw, (size_t)nTrain * sizeof(float), st);
  if (e == cudaSuccess) e = scratch_alloc(&radii, (size_t)nTrain * es, st);
  if (e != cudaSuccess) rc = cuda_error(e, "training buffers");
  if (rc == kOk) {
    KnnArgs a;
    a.query = dTrain;
    a.nq = nTrain;
    a.qStride = qStride;
    a.k = k;
    a.optionFlags = optionFlags;
    a.maxRadius = maxRadius;
    a.indices = idx;
    a.dists2 = d2;
    a.traversal = h.traversal == 2 ? 1 : h.traversal;
    rc = search_plain(c, a, st);
  }
  std::vector<float> hy;
  if (rc == kOk) {
    double minD2 = 1e-30;
    if (m->dtype == NABO_CUDA_FLOAT32)
      k_targets<float><<<ceil_div(nTrain, 256), 256, 0, st>>>(static_cast<const float*>(d2), nTrain, k, minD2, Y);
    else
      k_targets<double><<<ceil_div(nTrain, 256), 256, 0, st>>>(static_cast<const double*>(d2), nTrain, k, minD2, Y);
    hy.resize((size_t)nTrain);
    e = cudaMemcpyAsync(hy.data(), Y, (size_t)nTrain * sizeof(float), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) rc = cuda_error(e, "training targets");
  }
  // standardise the targets; keep samples with a k-th neighbour
  std::vector<int32_t> valid;
  double medianDk = 0.0;
  if (rc == kOk) rc = standardise_targets(m, hy, &valid, &medianDk);
  if (rc == kOk) {
    e = cudaMemcpyAsync(Y, hy.data(), (size_t)nTrain * sizeof(float), cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) rc = cuda_error(e, "training targets upload");
  }
  // voxel tables (finest voxel = half the median k-th distance), features
  if (rc == kOk) {
    const double h0 = std::max(0.5 * medianDk, 1e-12);
    rc = c.dtype == NABO_CUDA_FLOAT32 ? dispatch_grid<float>(c, m, h0, st) : dispatch_grid<double>(c, m, h0, st);
  }
  if (rc == kOk) rc = launch_features(*m, dTrain, nTrain, qStride, X, st);
  // Adam with a cosine learning-rate decay
  if (rc == kOk) rc = fit_params(m, X, Y, valid, tp, order, loss, st);
  // margin: residual quantile so that ~targetMissRate of the training
  // queries would fall outside their radius
  m->margin = 0.0f;
  if (rc == kOk && tp.targetMissRate > 0.0f) rc = launch_radius(*m, dTrain, nTrain, qStride, 1e300, radii, raw, st);
  if (rc == kOk && tp.targetMissRate > 0.0f) rc = calibrate_margin(m, hy, valid, raw, nTrain, tp, st);
  if (idx) scratch_free(idx, st);
  if (d2) scratch_free(d2, st);
  if (X) scratch_free(X, st);
  if (Y) scratch_free(Y, st);
  if (loss) scratch_free(loss, st);
  if (order) scratch_free(order, st);
  if (raw) scratch_free(raw, st);
  if (radii) scratch_free(radii, st);
  if (rc != kOk) return fail(rc);
  e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return fail(cuda_error(e, "training"));
  *out = m;
  return kOk;
}

// ---------------------------------------------------------------------------
// batched models

template <typename T>
BatchFeat<T> batch_feat(const BatchView& v) {
  BatchFeat<T> bf;
  bf.nodes = static_cast<const Node<T>*>(v.nodes);
  bf.recs = v.recs;
  bf.pointOff = v.pointOff;
  bf.nodeOffset = v.nodeOffset;
  bf.rootLo = static_cast<const T*>(v.rootLo);
  bf.rootHi = static_cast<const T*>(v.rootHi);
  bf.qOffset = v.qOffset;
  bf.kOf = v.kOf;
  bf.nClouds = v.nClouds;
  bf.dim = v.dim;
  return bf;
}

// f(T(), integral_constant<int, D>()) for the batch's scalar type and
// compiled record dimension.
template <typename F>
int batch_dispatch(const BatchView& v, F&& f) {
  using std::integral_constant;
  if (v.dtype == NABO_CUDA_FLOAT32) {
    switch (v.dpad) {
      case 2: return f(float(), integral_constant<int, 2>());
      case 3: return f(float(), integral_constant<int, 3>());
      case 4: return f(float(), integral_constant<int, 4>());
      case 8: return f(float(), integral_constant<int, 8>());
      case 16: return f(float(), integral_constant<int, 16>());
    }
  } else {
    switch (v.dpad) {
      case 2: return f(double(), integral_constant<int, 2>());
      case 3: return f(double(), integral_constant<int, 3>());
      case 4: return f(double(), integral_constant<int, 4>());
      case 8: return f(double(), integral_constant<int, 8>());
      case 16: return f(double(), integral_constant<int, 16>());
    }
  }
  return set_error(kErrInternal, "bad dispatch");
}

int launch_radius_batch(const RadiusModel& m, const BatchView& v, const void* query, double maxRadius, void* radii,
                        float* raw, cudaStream_t st) {
  if (v.nq == 0) return kOk;
  RadiusOut ro;
  ro.mu = m.mu;
  ro.sigma = m.sigma;
  ro.safety = m.safety;
  ro.margin = m.margin;
  ro.maxRadius = maxRadius;
  const int64_t tiles = (v.nq + 15) / 16;
  const int grid = (int)std::min<int64_t>(ceil_div(tiles, kInferWarps), 152 * 16);
  const int rc = batch_dispatch(v, [&](auto t, auto d) {
    using T = decltype(t);
    k_mlp_radius_batch<T, decltype(d)::value><<<grid, kInferWarps * 32, 0, st>>>(
        static_cast<const T*>(query), v.nq, batch_feat<T>(v), m.fs, m.pb, ro, static_cast<T*>(radii), raw);
    return kOk;
  });
  if (rc != kOk) return rc;
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_error(e, "batched learned radius kernel");
  return kOk;
}

// Trains a batched model from the queries of the batch's current plan and
// their exact results (dists2 of a plain batched search of them).
int batch_radius_model_train(const BatchView& v, const void* query, const void* d2, const nabo_cuda_train_params& tp,
                             RadiusModel** out, cudaStream_t st) {
  RadiusModel* m = new RadiusModel();
  m->dtype = v.dtype;
  m->dim = v.dim;
  m->dpad = v.dpad;
  m->k = v.kMax;
  m->kind = 1;
  m->safety = tp.safety;
  const int64_t n = v.nq;
  const size_t es = v.dtype == NABO_CUDA_FLOAT32 ? 4 : 8;
  int rc = kOk;
  auto fail = [&](int code) {
    cudaStreamSynchronize(st);
    free_model(m);
    delete m;
    return code;
  };
  cudaError_t e = cudaMalloc((void**)&m->params, kParams * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc((void**)&m->adamM, kParams * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc((void**)&m->adamV, kParams * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc((void**)&m->grad, kParams * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc((void**)&m->pb, kParams * sizeof(__nv_bfloat16));
  if (e != cudaSuccess) return fail(cuda_error(e, "model allocation"));
  float *X = nullptr, *Y = nullptr, *loss = nullptr, *raw = nullptr;
  int32_t* order = nullptr;
  void* radii = nullptr;
  e = scratch_alloc((void**)&X, (size_t)n * kF * sizeof(float), st);
  if (e == cudaSuccess) e = scratch_alloc((void**)&Y, (size_t)n * sizeof(float), st);
  if (e == cudaSuccess) e = scratch_alloc((void**)&loss, sizeof(float), st);
  if (e == cudaSuccess) e = scratch_alloc((void**)&order, (size_t)n * sizeof(int32_t), st);
  if (e == cudaSuccess) e = scratch_alloc((void**)&raw, (size_t)n * sizeof(float), st);
  if (e == cudaSuccess) e = scratch_alloc(&radii, (size_t)n * es, st);
  if (e != cudaSuccess) rc = cuda_error(e, "training buffers");
  // targets (log d_k of each query's own k) and raw inputs
  if (rc == kOk) {
    rc = batch_dispatch(v, [&](auto t, auto d) {
      using T = decltype(t);
      k_batch_targets<T><<<ceil_div(n, 256), 256, 0, st>>>(static_cast<const T*>(d2), n, v.qOffset, v.outOffset,
                                                           v.kOf, v.nClouds, 1e-30, Y);
      k_batch_features<T, decltype(d)::value><<<ceil_div(n, 128), 128, 0, st>>>(
          static_cast<const T*>(query), n, batch_feat<T>(v), m->fs, 0, X);
      return kOk;
    });
  }
  std::vector<float> hy((size_t)n), hx;
  if (rc == kOk) {
    hx.resize((size_t)n * kF);
    e = cudaMemcpyAsync(hy.data(), Y, (size_t)n * sizeof(float), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(hx.data(), X, hx.size() * sizeof(float), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) rc = cuda_error(e, "training data");
  }
  std::vector<int32_t> valid;
  double medianDk = 0.0;
  if (rc == kOk) rc = standardise_targets(m, hy, &valid, &medianDk);
  // input normalisation from the training samples: centre = mean, scale so
  // that two standard deviations map to 1
  if (rc == kOk) {
    FeatureSpace& fs = m->fs;
    fs.dim = v.dim;
    fs.nIn = kBatchInputs;
    fs.useGrid = 0;
    for (int j = 0; j < kMaxDim; ++j) {
      fs.center[j] = 0.0f;
      fs.invHalf[j] = 0.0f;
    }
    for (int j = 0; j < kBatchInputs; ++j) {
      double sum = 0.0, sq = 0.0;
      for (int32_t i : valid) {
        const double x = hx[(size_t)i * kF + j];
        sum += x;
        sq += x * x;
      }
      const double mean = sum / valid.size();
      const double sd = std::sqrt(std::max(sq / valid.size() - mean * mean, 0.0));
      fs.center[j] = (float)mean;
      fs.invHalf[j] = sd > 1e-12 ? (float)(0.5 / sd) : 0.0f;
    }
    for (int64_t i = 0; i < n; ++i)
      for (int j = 0; j < kF; ++j) {
        float& x = hx[(size_t)i * kF + j];
        x = j < kBatchInputs ? std::min(4.0f, std::max(-4.0f, (x - fs.center[j]) * fs.invHalf[j])) : 0.0f;
      }
    e = cudaMemcpyAsync(X, hx.data(), hx.size() * sizeof(float), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(Y, hy.data(), (size_t)n * sizeof(float), cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) rc = cuda_error(e, "training data upload");
  }
  if (rc == kOk) rc = fit_params(m, X, Y, valid, tp, order, loss, st);
  m->margin = 0.0f;
  if (rc == kOk && tp.targetMissRate > 0.0f) rc = launch_radius_batch(*m, v, query, 1e300, radii, raw, st);
  if (rc == kOk && tp.targetMissRate > 0.0f) rc = calibrate_margin(m, hy, valid, raw, n, tp, st);
  for (void* p : {(void*)X, (void*)Y, (void*)loss, (void*)raw, (void*)order, radii})
    if (p) scratch_free(p, st);
  if (rc != kOk) return fail(rc);
  e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return fail(cuda_error(e, "training"));
  *out = m;
  return kOk;
}

void radius_model_free(RadiusModel* m) {
  if (!m) return;
  free_model(m);
  delete m;
}

int radius_model_predict(const RadiusModel& m, const void* query, int64_t nq, int64_t qStride, double maxRadius,
                         void* radii, float* raw, cudaStream_t st) {
  return launch_radius(m, query, nq, qStride, maxRadius, radii, raw, st);
}

// Bounded search with the learned radii; a query that finds fewer than k
// neighbours inside a radius below the caller's maxRadius searches again
// without the bound, in the same thread of the same launch (so the repeats
// spread over the whole grid instead of forming a small second launch).
int knn_learned(const nabo_cuda_search* s, const RadiusModel& m, const KnnArgs& base, int32_t* dFallbacks,
                cudaStream_t st) {
  const HandleView h = handle_view(s);
  const DeviceCloud& c = *h.cloud;
  if (base.nq == 0) return kOk;
  const size_t es = c.dtype == NABO_CUDA_FLOAT32 ? 4 : 8;
  void* radii = nullptr;
  int32_t *count = nullptr, *order = nullptr;
  const bool ordered = base.sortQueries && base.nq >= 4096;
  cudaError_t e = scratch_alloc(&radii, (size_t)base.nq * es, st);
  if (e == cudaSuccess) e = scratch_alloc((void**)&count, sizeof(int32_t), st);
  if (e == cudaSuccess && ordered) e = scratch_alloc((void**)&order, (size_t)base.nq * sizeof(int32_t), st);
  if (e == cudaSuccess) e = cudaMemsetAsync(count, 0, sizeof(int32_t), st);
  int rc = e == cudaSuccess ? kOk : cuda_error(e, "learned search buffers");
  if (rc == kOk) rc = launch_radius(m, base.query, base.nq, base.qStride, base.maxRadius, radii, nullptr, st);
  if (rc == kOk && ordered) rc = leaf_order(c, base.query, base.nq, base.qStride, order, st);
  if (rc == kOk) {
    KnnArgs a = base;
    a.maxRadii = radii;
    a.fallbackRadius = base.maxRadius;
    a.fallbacks = count;
    a.evStart = h.evStart;
    a.evStop = h.evStop;
    rc = search_given(c, a, order, st);
  }
  if (rc == kOk && dFallbacks) {
    e = cudaMemcpyAsync(dFallbacks, count, sizeof(int32_t), cudaMemcpyDeviceToDevice, st);
    if (e != cudaSuccess) rc = cuda_error(e, "fallback count");
  }
  if (radii) scratch_free(radii, st);
  if (count) scratch_free(count, st);
  if (order) scratch_free(order, st);
  return rc;
}

// Gradient of the training loss for given features/targets (for checks).
int radius_model_gradients(const RadiusModel& m, const float* dX, const float* dY, int64_t n, float* hGrad,
                           float* hLoss, cudaStream_t st) {
  int32_t* idx = nullptr;
  float* loss = nullptr;
  cudaError_t e = scratch_alloc((void**)&idx, (size_t)n * sizeof(int32_t), st);
  if (e == cudaSuccess) e = scratch_alloc((void**)&loss, sizeof(float), st);
  if (e != cudaSuccess) return cuda_error(e, "gradient buffers");
  std::vector<int32_t> seq((size_t)n);
  for (int64_t i = 0; i < n; ++i) seq[(size_t)i] = (int32_t)i;
  e = cudaMemcpyAsync(idx, seq.data(), (size_t)n * sizeof(int32_t), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemsetAsync(loss, 0, sizeof(float), st);
  if (e == cudaSuccess) e = cudaMemsetAsync(m.grad, 0, kParams * sizeof(float), st);
  int rc = e == cudaSuccess ? kOk : cuda_error(e, "gradient setup");
  if (rc == kOk) rc = grad_step(m, dX, dY, idx, (int)n, loss, st);
  if (rc == kOk) {
    e = cudaMemcpyAsync(hGrad, m.grad, kParams * sizeof(float), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(hLoss, loss, sizeof(float), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(m.grad, 0, kParams * sizeof(float), st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) rc = cuda_error(e, "gradient readback");
  }
  scratch_free(idx, st);
  scratch_free(loss, st);
  cudaStreamSynchronize(st);
  return rc;
}

int radius_model_features(const RadiusModel& m, const void* query, int64_t nq, int64_t qStride, float* dX,
                          cudaStream_t st) {
  return launch_features(m, query, nq, qStride, dX, st);
}

int radius_model_get(const RadiusModel& m, float* params, float* meta) {
  if (params) {
    const cudaError_t e = cudaMemcpy(params, m.params, kParams * sizeof(float), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_error(e, "model read");
  }
  if (meta) {
    meta[0] = m.mu;
    meta[1] = m.sigma;
    meta[2] = m.safety;
    meta[3] = (float)m.k;
    meta[4] = m.trainLoss;
    meta[5] = (float)m.trainSamples;
    meta[6] = (float)m.fs.nIn;
    meta[7] = m.margin;
    meta[8] = (float)m.h0;
    for (int i = 9; i < 16; ++i) meta[i] = 0.0f;
  }
  return kOk;
}

int radius_model_set(RadiusModel& m, const float* params, const float* meta) {
  if (meta && m.fs.useGrid && meta[8] > 0.0f && (float)m.h0 != meta[8]) {
    // rebuild the voxel tables at the saved scale
    const DeviceCloud& c = *handle_view(static_cast<const nabo_cuda_search*>(m.owner)).cloud;
    if (m.tables) cudaFree(m.tables);
    m.tables = nullptr;
    const int rc = c.dtype == NABO_CUDA_FLOAT32 ? dispatch_grid<float>(c, &m, meta[8], cudaStreamPerThread)
                                                : dispatch_grid<double>(c, &m, meta[8], cudaStreamPerThread);
    if (rc != kOk) return rc;
  }
  if (params) {
    cudaError_t e = cudaMemcpy(m.params, params, kParams * sizeof(float), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return cuda_error(e, "model write");
    k_to_bf16<<<ceil_div(kParams, 256), 256>>>(m.params, m.pb, kParams);
    e = cudaDeviceSynchronize();
    if (e != cudaSuccess) return cuda_error(e, "model write");
  }
  if (meta) {
    m.mu = meta[0];
    m.sigma = meta[1];
    m.safety = meta[2];
    m.margin = meta[7];
  }
  return kOk;
}

const void* radius_model_owner(const RadiusModel& m) { return m.owner; }
int radius_model_k(const RadiusModel& m) { return m.k; }

}  // namespace nabo_gb300

// ---------------------------------------------------------------------------
// C ABI

struct nabo_cuda_radius_model {
  nabo_gb300::RadiusModel* m;
  int device;
};

using namespace nabo_gb300;

namespace {
struct DevGuard {
  int prev = -1;
  explicit DevGuard(int dev) {
    if (cudaGetDevice(&prev) == cudaSuccess && prev != dev) cudaSetDevice(dev);
  }
  ~DevGuard() {
    int cur = -1;
    if (prev >= 0 && cudaGetDevice(&cur) == cudaSuccess && cur != prev) cudaSetDevice(prev);
  }
};
}  // namespace

extern "C" void nabo_cuda_train_params_init(nabo_cuda_train_params* p);

namespace {
const char* const kBatchModelOnly =
    "a batched radius model serves nabo_cuda_batch_knn_learned_device only (its inputs come from a batch's trees)";

// The caller's training parameters (defaults for NULL), checked.
int read_train_params(const nabo_cuda_train_params* params, nabo_cuda_train_params* tp) {
  nabo_cuda_train_params_init(tp);
  if (params) {
    tp->epochs = params->epochs;
    tp->batch = params->batch;
    tp->lr = params->lr;
    tp->safety = params->safety;
    tp->targetMissRate = params->targetMissRate;
    tp->seed = params->seed;
  }
  if (tp->epochs < 1 || tp->batch < 32 || !(tp->lr > 0.0f) || !(tp->safety >= 1.0f) ||
      !(tp->targetMissRate >= 0.0f && tp->targetMissRate < 1.0f))
    return set_error(kErrArgument,
                     "training parameters: epochs >= 1, batch >= 32, lr > 0, safety >= 1, 0 <= targetMissRate < 1");
  return kOk;
}
}  // namespace

extern "C" {

void nabo_cuda_train_params_init(nabo_cuda_train_params* p) {
  if (!p) return;
  std::memset(p, 0, sizeof(*p));
  p->struct_size = sizeof(nabo_cuda_train_params);
  p->epochs = 30;
  p->batch = 4096;
  p->lr = 3e-3f;
  p->safety = 1.2f;
  p->targetMissRate = 0.01f;
  p->seed = 1234;
}

int nabo_cuda_radius_model_train(const nabo_cuda_search* s, const void* trainQueries, int qRows, int64_t n,
                                 int64_t qStride, int k, unsigned optionFlags, double maxRadius,
                                 const nabo_cuda_train_params* params, nabo_cuda_radius_model** out) {
  if (!s || !out) return set_error(kErrArgument, "NULL search object or output pointer");
  *out = nullptr;
  const HandleView h = handle_view(s);
  if (h.searchType != NABO_SEARCH_KDTREE_CUDA)
    return set_error(kErrArgument, "a radius model is trained for a kd-tree search object");
  int rc = handle_check_knn(s, qRows, n, qStride, k, optionFlags, nullptr);
  if (rc != kOk) return rc;
  if (n < 16 || !trainQueries) return set_error(kErrArgument, "at least 16 training queries are needed");
  if (n > (int64_t)1 << 30) return set_error(kErrUnsupported, "too many training queries");
  nabo_cuda_train_params tp;
  rc = read_train_params(params, &tp);
  if (rc != kOk) return rc;
  DevGuard g(h.device);
  RadiusModel* m = nullptr;
  rc = radius_model_train(s, trainQueries, n, qStride, k, optionFlags, maxRadius, tp, &m, cudaStreamPerThread);
  if (rc != kOk) return rc;
  *out = new nabo_cuda_radius_model{m, h.device};
  return kOk;
}

int nabo_cuda_radius_model_destroy(nabo_cuda_radius_model* m) {
  if (!m) return kOk;
  DevGuard g(m->device);
  radius_model_free(m->m);
  delete m;
  return kOk;
}

int nabo_cuda_radius_model_predict_device(const nabo_cuda_radius_model* m, const void* query, int qRows, int64_t nq,
                                          int64_t qStride, double maxRadius, void* radii, float* raw, void* stream) {
  if (!m) return set_error(kErrArgument, "radius model is NULL");
  if (m->m->kind != 0) return set_error(kErrArgument, kBatchModelOnly);
  if (nq < 0 || qStride < qRows || qRows < m->m->dim) return set_error(kErrArgument, "bad query shape");
  if (nq == 0) return kOk;
  if (!query || !radii) return set_error(kErrArgument, "NULL query or radii buffer");
  DevGuard g(m->device);
  return radius_model_predict(*m->m, query, nq, qStride, maxRadius, radii, raw, static_cast<cudaStream_t>(stream));
}

int nabo_cuda_knn_learned_device(const nabo_cuda_search* s, const nabo_cuda_radius_model* m, const void* query,
                                 int qRows, int64_t nq, int64_t qStride, int k, double epsilon, unsigned optionFlags,
                                 double maxRadius, int32_t* indices, void* dists2, uint64_t* touched,
                                 int32_t* fallbacks, void* stream) {
  if (!s || !m) return set_error(kErrArgument, "NULL search object or radius model");
  if (radius_model_owner(*m->m) != s)
    return set_error(kErrArgument, "the radius model was trained for another search object");
  int rc = handle_check_knn(s, qRows, nq, qStride, k, optionFlags, nullptr);
  if (rc != kOk) return rc;
  if (nq == 0) return kOk;
  if (!query || !indices || !dists2) return set_error(kErrArgument, "NULL query or result buffer");
  const HandleView h = handle_view(s);
  DevGuard g(h.device);
  KnnArgs a;
  a.query = query;
  a.nq = nq;
  a.qStride = qStride;
  a.k = k;
  a.eps = epsilon;
  a.optionFlags = optionFlags;
  a.touchStats = (h.creationFlags & NABO_TOUCH_STATISTICS) != 0;
  a.touched = reinterpret_cast<unsigned long long*>(touched);
  a.maxRadius = maxRadius;
  a.indices = indices;
  a.dists2 = dists2;
  a.traversal = h.traversal == 2 ? 1 : h.traversal;
  return knn_learned(s, *m->m, a, fallbacks, static_cast<cudaStream_t>(stream));
}

int nabo_cuda_knn_learned(const nabo_cuda_search* s, const nabo_cuda_radius_model* m, const void* query, int qRows,
                          int64_t nq, int64_t qStride, int k, double epsilon, unsigned optionFlags, double maxRadius,
                          int32_t* indices, void* dists2, uint64_t* touched, int64_t* fallbacks) {
  if (!s || !m) return set_error(kErrArgument, "NULL search object or radius model");
  int rc = handle_check_knn(s, qRows, nq, qStride, k, optionFlags, nullptr);
  if (rc != kOk) return rc;
  if (touched) *touched = 0;
  if (fallbacks) *fallbacks = 0;
  if (nq == 0) return kOk;
  if (!query || !indices || !dists2) return set_error(kErrArgument, "NULL query or result buffer");
  const HandleView h = handle_view(s);
  DevGuard g(h.device);
  cudaStream_t st = cudaStreamPerThread;
  const size_t es = h.cloud->dtype == NABO_CUDA_FLOAT32 ? 4 : 8;
  const size_t qBytes = (size_t)((nq - 1) * qStride + qRows) * es;
  const size_t outN = (size_t)nq * (size_t)k;
  void *dq = nullptr, *dd = nullptr;
  int32_t *di = nullptr, *dfb = nullptr;
  unsigned long long* dt = nullptr;
  cudaError_t e = scratch_alloc(&dq, qBytes, st);
  if (e == cudaSuccess) e = scratch_alloc((void**)&di, outN * sizeof(int32_t), st);
  if (e == cudaSuccess) e = scratch_alloc(&dd, outN * es, st);
  if (e == cudaSuccess) e = scratch_alloc((void**)&dt, sizeof(unsigned long long), st);
  if (e == cudaSuccess) e = scratch_alloc((void**)&dfb, sizeof(int32_t), st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dq, query, qBytes, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemsetAsync(dt, 0, sizeof(unsigned long long), st);
  rc = e == cudaSuccess ? kOk : cuda_error(e, "learned knn setup");
  if (rc == kOk)
    rc = nabo_cuda_knn_learned_device(s, m, dq, qRows, nq, qStride, k, epsilon, optionFlags, maxRadius, di, dd,
                                      reinterpret_cast<uint64_t*>(dt), dfb, st);
  unsigned long long ht = 0;
  int32_t hfb = 0;
  if (rc == kOk) {
    e = cudaMemcpyAsync(indices, di, outN * sizeof(int32_t), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dists2, dd, outN * es, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&ht, dt, sizeof(ht), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&hfb, dfb, sizeof(hfb), cudaMemcpyDeviceToHost, st);
    if (e != cudaSuccess) rc = cuda_error(e, "learned knn results");
  }
  if (dq) scratch_free(dq, st);
  if (di) scratch_free(di, st);
  if (dd) scratch_free(dd, st);
  if (dt) scratch_free(dt, st);
  if (dfb) scratch_free(dfb, st);
  e = cudaStreamSynchronize(st);
  if (rc == kOk && e != cudaSuccess) rc = cuda_error(e, "learned knn");
  if (rc == kOk) {
    if (touched) *touched = (h.creationFlags & NABO_TOUCH_STATISTICS) ? ht : 0;
    if (fallbacks) *fallbacks = hfb;
  }
  return rc;
}

int nabo_cuda_radius_model_features_device(const nabo_cuda_radius_model* m, const void* query, int qRows, int64_t nq,
                                           int64_t qStride, float* features, void* stream) {
  if (!m) return set_error(kErrArgument, "radius model is NULL");
  if (m->m->kind != 0) return set_error(kErrArgument, kBatchModelOnly);
  if (nq < 0 || qStride < qRows || qRows < m->m->dim) return set_error(kErrArgument, "bad query shape");
  if (nq == 0) return kOk;
  DevGuard g(m->device);
  return radius_model_features(*m->m, query, nq, qStride, features, static_cast<cudaStream_t>(stream));
}

int nabo_cuda_radius_model_gradients(const nabo_cuda_radius_model* m, const float* features, const float* targets,
                                     int64_t n, float* grad, float* loss) {
  if (!m || !features || !targets || !grad || !loss) return set_error(kErrArgument, "NULL argument");
  if (n < 1 || n > (int64_t)1 << 28) return set_error(kErrArgument, "bad sample count");
  DevGuard g(m->device);
  return radius_model_gradients(*m->m, features, targets, n, grad, loss, cudaStreamPerThread);
}

int nabo_cuda_radius_model_get(const nabo_cuda_radius_model* m, float* params, float* meta) {
  if (!m) return set_error(kErrArgument, "radius model is NULL");
  DevGuard g(m->device);
  return radius_model_get(*m->m, params, meta);
}

int nabo_cuda_radius_model_set(nabo_cuda_radius_model* m, const float* params, const float* meta) {
  if (!m) return set_error(kErrArgument, "radius model is NULL");
  if (m->m->kind != 0) return set_error(kErrArgument, "a batched radius model keeps its trained input scaling; it is not set");
  DevGuard g(m->device);
  return radius_model_set(*m->m, params, meta);
}

int nabo_cuda_batch_radius_model_train(nabo_cuda_batch* b, const void* queries, const void* dists2,
                                       const nabo_cuda_train_params* params, nabo_cuda_radius_model** out) {
  if (!b || !out) return set_error(kErrArgument, "NULL batch or output pointer");
  *out = nullptr;
  BatchView v;
  int rc = batch_view(b, &v);
  if (rc != kOk) return rc;
  if (v.nq < 16 || !queries || !dists2) return set_error(kErrArgument, "at least 16 training queries are needed");
  if (v.nq > (int64_t)1 << 30) return set_error(kErrUnsupported, "too many training queries");
  nabo_cuda_train_params tp;
  rc = read_train_params(params, &tp);
  if (rc != kOk) return rc;
  DevGuard g(v.device);
  RadiusModel* m = nullptr;
  rc = batch_radius_model_train(v, queries, dists2, tp, &m, cudaStreamPerThread);
  if (rc != kOk) return rc;
  *out = new nabo_cuda_radius_model{m, v.device};
  return kOk;
}

int nabo_cuda_batch_knn_learned_device(nabo_cuda_batch* b, const nabo_cuda_radius_model* m, const void* queries,
                                       double epsilon, unsigned optionFlags, double maxRadius, int32_t* indices,
                                       void* dists2, int32_t* fallbacks, void* stream) {
  if (!b || !m) return set_error(kErrArgument, "NULL batch or radius model");
  BatchView v;
  int rc = batch_view(b, &v);
  if (rc != kOk) return rc;
  const RadiusModel& rm = *m->m;
  if (rm.kind != 1 || rm.dtype != v.dtype || rm.dim != v.dim)
    return set_error(kErrArgument, "the radius model was not trained for batches of this dimension and scalar type");
  if (v.nq == 0) return kOk;
  if (!queries || !indices || !dists2) return set_error(kErrArgument, "NULL query or result buffer");
  DevGuard g(v.device);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const size_t es = v.dtype == NABO_CUDA_FLOAT32 ? 4 : 8;
  void* radii = nullptr;
  int32_t* count = nullptr;
  cudaError_t e = scratch_alloc(&radii, (size_t)v.nq * es, st);
  if (e == cudaSuccess) e = scratch_alloc((void**)&count, sizeof(int32_t), st);
  if (e == cudaSuccess) e = cudaMemsetAsync(count, 0, sizeof(int32_t), st);
  rc = e == cudaSuccess ? kOk : cuda_error(e, "learned batch buffers");
  if (rc == kOk) rc = launch_radius_batch(rm, v, queries, maxRadius, radii, nullptr, st);
  if (rc == kOk)
    rc = nabo_cuda_batch_knn_radii_device(b, queries, radii, epsilon, optionFlags, maxRadius, indices, dists2, count,
                                          stream);
  if (rc == kOk && fallbacks) {
    e = cudaMemcpyAsync(fallbacks, count, sizeof(int32_t), cudaMemcpyDeviceToDevice, st);
    if (e != cudaSuccess) rc = cuda_error(e, "fallback count");
  }
  if (radii) scratch_free(radii, st);
  if (count) scratch_free(count, st);
  return rc;
}

int nabo_cuda_batch_radius_model_predict_device(nabo_cuda_batch* b, const nabo_cuda_radius_model* m,
                                                const void* queries, double maxRadius, void* radii, float* raw,
                                                void* stream) {
  if (!b || !m) return set_error(kErrArgument, "NULL batch or radius model");
  BatchView v;
  int rc = batch_view(b, &v);
  if (rc != kOk) return rc;
  const RadiusModel& rm = *m->m;
  if (rm.kind != 1 || rm.dtype != v.dtype || rm.dim != v.dim)
    return set_error(kErrArgument, "the radius model was not trained for batches of this dimension and scalar type");
  if (v.nq == 0) return kOk;
  if (!queries || !radii) return set_error(kErrArgument, "NULL query or radii buffer");
  DevGuard g(v.device);
  return launch_radius_batch(rm, v, queries, maxRadius, radii, raw, static_cast<cudaStream_t>(stream));
}

int nabo_cuda_batch_radius_model_features_device(nabo_cuda_batch* b, const nabo_cuda_radius_model* m,
                                                 const void* queries, float* features, void* stream) {
  if (!b || !m) return set_error(kErrArgument, "NULL batch or radius model");
  BatchView v;
  int rc = batch_view(b, &v);
  if (rc != kOk) return rc;
  const RadiusModel& rm = *m->m;
  if (rm.kind != 1 || rm.dtype != v.dtype || rm.dim != v.dim)
    return set_error(kErrArgument, "the radius model was not trained for batches of this dimension and scalar type");
  if (v.nq == 0) return kOk;
  if (!queries || !features) return set_error(kErrArgument, "NULL query or feature buffer");
  DevGuard g(v.device);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  rc = batch_dispatch(v, [&](auto t, auto d) {
    using T = decltype(t);
    k_batch_features<T, decltype(d)::value><<<ceil_div(v.nq, 128), 128, 0, st>>>(
        static_cast<const T*>(queries), v.nq, batch_feat<T>(v), rm.fs, 1, features);
    return kOk;
  });
  if (rc != kOk) return rc;
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? kOk : cuda_error(e, "batched features kernel");
}

}  // extern "C"
