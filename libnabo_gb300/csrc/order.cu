// order.cu -- query ordering for warp coherence, a stable radix sort and a
// device-wide scan.
//
// The kd-tree search runs one query per thread, so its warps stay coherent
// only if neighbouring threads get nearby queries. order_queries() sorts the
// queries by a 30-bit Morton (Z-order) code over the cloud's bounding box
// with a stable radix sort: ties (queries in one Morton cell) keep input
// order, which for scanned data keeps the points of one scan line together
// and makes the warps' result rows adjacent in memory. The kd-tree path for
// more than 3 dimensions sorts by the leaf each query descends to instead
// (same stable sort). order_by_cells() is the counting-sort placement the
// batched search uses (cells = leaves, ranks from atomics, then each
// cell's queries back in index order). Results never depend on the order,
// only timing does.
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cmath>

#include "internal.cuh"

namespace nabo_gb300 {
namespace {

constexpr int kB = 256;
constexpr int kMortonDims = 3;

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

// The scans cover the first m = min(n, *nDev) entries when nDev is given
// (a count only the device knows); blocks past m return at once.
__device__ __forceinline__ int64_t live_count(int64_t n, const int64_t* nDev) {
  return nDev ? min(n, *nDev) : n;
}

__global__ void k_block_sums(const uint32_t* __restrict__ data, int64_t n, uint32_t* sums, const int64_t* nDev) {
  n = live_count(n, nDev);
  if (blockIdx.x * (int64_t)kB >= n) return;
  const int64_t i = blockIdx.x * (int64_t)kB + threadIdx.x;
  const uint32_t v = i < n ? data[i] : 0u;
  uint32_t t;
  block_excl_scan_u32(v, &t);
  if (threadIdx.x == 0) sums[blockIdx.x] = t;
}

// Single block: each thread scans a contiguous run of the block sums
// serially, one block-wide scan of the runs' totals joins them.
__global__ void k_scan_sums(uint32_t* sums, int nb, uint32_t* total, const int64_t* nDev) {
  if (nDev) nb = (int)min((int64_t)nb, (live_count((int64_t)nb * kB, nDev) + kB - 1) / kB);
  const int per = (nb + kB - 1) / kB;
  const int b0 = threadIdx.x * per;
  const int b1 = min(b0 + per, nb);
  uint32_t run = 0;
  for (int i = b0; i < b1; ++i) run += sums[i];
  uint32_t t;
  uint32_t carry = block_excl_scan_u32(run, &t);
  for (int i = b0; i < b1; ++i) {
    const uint32_t v = sums[i];
    sums[i] = carry;
    carry += v;
  }
  if (threadIdx.x == 0 && total) *total = t;
}

__global__ void k_apply(uint32_t* data, int64_t n, const uint32_t* __restrict__ sums, const int64_t* nDev) {
  n = live_count(n, nDev);
  if (blockIdx.x * (int64_t)kB >= n) return;
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
  // nChunks > 1: element i's key carries its chunk number (the count of
  // chunkEnd entries <= i) above its dims*bits Morton bits
  int nChunks;
  int64_t chunkEnd[kMaxQueryChunks];
};

__device__ __forceinline__ uint32_t spread3_10(uint32_t x) {
  x &= 0x3ffu;
  x = (x | (x << 16)) & 0x030000ffu;
  x = (x | (x << 8)) & 0x0300f00fu;
  x = (x | (x << 4)) & 0x030c30c3u;
  x = (x | (x << 2)) & 0x09249249u;
  return x;
}

// bit b of x (x < 2^16) to bit 2b
__device__ __forceinline__ uint32_t spread2_16(uint32_t x) {
  x &= 0xffffu;
  x = (x | (x << 8)) & 0x00ff00ffu;
  x = (x | (x << 4)) & 0x0f0f0f0fu;
  x = (x | (x << 2)) & 0x33333333u;
  x = (x | (x << 1)) & 0x55555555u;
  return x;
}

// Morton code of up to 3 coordinates already loaded: bit b of dimension d
// lands at b * dims + (dims - 1 - d). order_queries() keeps dims <= 3 and
// bits <= 30 / dims (fewer when the chunk number takes the top of the key),
// so one of the spread forms below always applies.
template <typename T>
__device__ __forceinline__ uint32_t morton_key3(const T (&x)[3], const CellParams& p) {
  uint32_t c[3];
  const float maxc = (float)((1u << p.bits) - 1u);
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    float v = ((float)x[d] - p.lo[d]) * p.scale[d];
    v = fminf(fmaxf(v, 0.0f), maxc);  // NaN -> 0
    c[d] = d < p.dims ? (uint32_t)v : 0u;
  }
  if (p.dims == 3) return (spread3_10(c[0]) << 2) | (spread3_10(c[1]) << 1) | spread3_10(c[2]);
  if (p.dims == 2) return (spread2_16(c[0]) << 1) | spread2_16(c[1]);
  return c[0] & ((1u << p.bits) - 1u);  // maxc may round up to 2^bits in float
}

// ---- stable LSD radix sort of (key, value) pairs, 10-bit digits.
// A block of kTileWarps warps owns a tile of kTile consecutive elements,
// warp w the w-th run of kWarpRounds x 32 of them. Pass p: k_tile_hist
// counts the tile's digits into hist[tile][digit] (tile-major, so each
// block writes one contiguous row); k_tile_scan turns every digit's column
// into exclusive prefixes over the tiles and the digit totals;
// k_tile_scatter re-counts each warp's run into a warp-private histogram,
// offsets the warps of the tile one after another, and walks each run in
// element order, 32 at a time, ranking equal digits inside the 32 with
// __match_any_sync, so equal keys keep their order (stability, which LSD
// needs across passes).
constexpr int kRadixBits = 10;
constexpr int kRadix = 1 << kRadixBits;
constexpr int kTileWarps = 8;
constexpr int kTileThreads = 32 * kTileWarps;
constexpr int kWarpRounds = 8;
constexpr int kWarpSpan = 32 * kWarpRounds;
constexpr int kTile = kTileWarps * kWarpSpan;
constexpr int kDigitsPerThread = kRadix / kTileThreads;
static_assert(kRadix % kTileThreads == 0, "digits split evenly over the tile's threads");
static_assert(kTileThreads == kB, "block_excl_scan_u32 scans kB threads");

// Adds each distinct digit of the 32 live lanes once (equal digits are
// common: the keys are spatially sorted after the first pass).
__device__ __forceinline__ void count_digit(uint32_t* h, bool act, uint32_t d) {
  const unsigned live = __ballot_sync(0xffffffffu, act);
  if (act) {
    const unsigned peers = __match_any_sync(live, d);
    if ((threadIdx.x & 31) == __ffs(peers) - 1) atomicAdd(h + d, (uint32_t)__popc(peers));
  }
}

// Element u of the calling lane's run: all of a warp's loads are issued
// before any is used, so each warp keeps kWarpRounds requests in flight.
__device__ __forceinline__ int64_t run_index(int u) {
  return (int64_t)blockIdx.x * kTile + (threadIdx.x >> 5) * kWarpSpan + u * 32 + (threadIdx.x & 31);
}

// Writes the block's digit counts as the tile's row of hist.
__device__ __forceinline__ void store_tile_row(const uint32_t* h, uint32_t* hist) {
  __syncthreads();
  uint32_t* row = hist + (int64_t)blockIdx.x * kRadix;
  for (int d = threadIdx.x; d < kRadix; d += kTileThreads) row[d] = h[d];
}

__global__ void __launch_bounds__(kTileThreads) k_tile_hist(const uint32_t* __restrict__ key, int64_t n, int shift,
                                                            uint32_t* hist) {
  __shared__ uint32_t h[kRadix];
  for (int d = threadIdx.x; d < kRadix; d += kTileThreads) h[d] = 0u;
  __syncthreads();
  uint32_t kk[kWarpRounds];
#pragma unroll
  for (int u = 0; u < kWarpRounds; ++u) {
    const int64_t i = run_index(u);
    kk[u] = i < n ? key[i] : 0u;
  }
#pragma unroll
  for (int u = 0; u < kWarpRounds; ++u) count_digit(h, run_index(u) < n, (kk[u] >> shift) & (kRadix - 1));
  store_tile_row(h, hist);
}

// Morton keys of the queries, in the radix sort's tile layout, with the
// first pass's digit counts. With copyOut, the coordinates read (the first
// dims of each row) are also written there at the same offsets: q may then
// be page-locked host memory read over the host link, and the kernel is the
// queries' upload too.
template <typename T>
__global__ void __launch_bounds__(kTileThreads) k_morton_tiles(const T* __restrict__ q, int64_t n, int64_t qStride,
                                                               CellParams p, uint32_t* key, uint32_t* hist,
                                                               T* __restrict__ copyOut) {
  __shared__ uint32_t h[kRadix];
  for (int d = threadIdx.x; d < kRadix; d += kTileThreads) h[d] = 0u;
  __syncthreads();
  constexpr int kHalf = kWarpRounds > 8 ? kWarpRounds / 2 : kWarpRounds;  // coordinates in flight at once
#pragma unroll
  for (int r0 = 0; r0 < kWarpRounds; r0 += kHalf) {
    uint32_t kk[kHalf];
    T c[kHalf][3];
#pragma unroll
    for (int u = 0; u < kHalf; ++u) {
      const int64_t i = run_index(r0 + u);
#pragma unroll
      for (int d = 0; d < 3; ++d) c[u][d] = (i < n && d < p.dims) ? q[i * qStride + d] : T(0);
    }
    if (copyOut) {
#pragma unroll
      for (int u = 0; u < kHalf; ++u) {
        const int64_t i = run_index(r0 + u);
#pragma unroll
        for (int d = 0; d < 3; ++d)
          if (i < n && d < p.dims) copyOut[i * qStride + d] = c[u][d];
      }
    }
#pragma unroll
    for (int u = 0; u < kHalf; ++u) kk[u] = morton_key3(c[u], p);
#pragma unroll
    for (int u = 0; u < kHalf; ++u) {
      const int64_t i = run_index(r0 + u);
      if (p.nChunks > 1) {
        uint32_t cid = 0;
        for (int c = 0; c + 1 < p.nChunks; ++c) cid += i >= p.chunkEnd[c] ? 1u : 0u;
        kk[u] |= cid << (p.bits * p.dims);
      }
      if (i < n) key[i] = kk[u];
      count_digit(h, i < n, kk[u] & (kRadix - 1));
    }
  }
  store_tile_row(h, hist);
}

// Block b handles digits [32 b, 32 b + 32), one per lane; warp g of the
// block covers a contiguous range of tiles, so every load reads 32
// consecutive counts of one tile's row. Rewrites hist[tile][digit] in place
// as the count of the digit in the earlier tiles; the digit's total goes to
// total[digit].
constexpr int kScanGroups = 32;
__global__ void __launch_bounds__(32 * kScanGroups) k_tile_scan(uint32_t* hist, int64_t nTiles, uint32_t* total) {
  __shared__ uint32_t part[kScanGroups][32];
  const int lane = threadIdx.x & 31, g = threadIdx.x >> 5;
  const int d = blockIdx.x * 32 + lane;
  const int64_t per = (nTiles + kScanGroups - 1) / kScanGroups;
  const int64_t t0 = g * per;
  const int64_t t1 = t0 + per < nTiles ? t0 + per : nTiles;
  uint32_t run = 0;
  for (int64_t t = t0; t < t1; ++t) run += hist[t * kRadix + d];
  part[g][lane] = run;
  __syncthreads();
  uint32_t carry = 0;
  for (int h = 0; h < g; ++h) carry += part[h][lane];
  if (g == kScanGroups - 1) total[d] = carry + run;
  for (int64_t t = t0; t < t1; ++t) {
    const uint32_t v = hist[t * kRadix + d];
    hist[t * kRadix + d] = carry;
    carry += v;
  }
}

// offs = the scanned hist (hist[tile][digit] = the digit's count in the
// earlier tiles), total = the digit totals.
__global__ void __launch_bounds__(kTileThreads)
    k_tile_scatter(const uint32_t* __restrict__ keyIn, const uint32_t* __restrict__ valIn, int64_t n, int shift,
                   const uint32_t* __restrict__ offs, const uint32_t* __restrict__ total, uint32_t* keyOut,
                   uint32_t* valOut) {
  __shared__ uint32_t wh[kTileWarps][kRadix];  // counts, then first output slots, per warp and digit
  __shared__ uint32_t first[kRadix];           // the tile's first output slot per digit
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  uint32_t kk[kWarpRounds], vv[kWarpRounds];
#pragma unroll
  for (int u = 0; u < kWarpRounds; ++u) {
    const int64_t i = run_index(u);
    kk[u] = i < n ? keyIn[i] : 0u;
    vv[u] = i < n ? (valIn ? valIn[i] : (uint32_t)i) : 0u;
  }
  // the tile's first slot per digit: the totals of the smaller digits
  // (thread t holds digits [kDigitsPerThread t, kDigitsPerThread (t+1)))
  // plus the earlier tiles' counts of the digit
  {
    uint32_t tv[kDigitsPerThread];
    uint32_t run = 0;
#pragma unroll
    for (int j = 0; j < kDigitsPerThread; ++j) {
      tv[j] = total[threadIdx.x * kDigitsPerThread + j];
      run += tv[j];
    }
    uint32_t all;
    uint32_t carry = block_excl_scan_u32(run, &all);
    const uint32_t* row = offs + (int64_t)blockIdx.x * kRadix;
#pragma unroll
    for (int j = 0; j < kDigitsPerThread; ++j) {
      const int d = threadIdx.x * kDigitsPerThread + j;
      first[d] = carry + row[d];
      carry += tv[j];
    }
  }
  for (int d = lane; d < kRadix; d += 32) wh[warp][d] = 0u;
  __syncwarp();
  // each warp counts its own run; the equal-digit peers of every round are
  // kept for the ranking below
  unsigned peers[kWarpRounds];
#pragma unroll
  for (int u = 0; u < kWarpRounds; ++u) {
    const bool act = run_index(u) < n;
    const unsigned live = __ballot_sync(0xffffffffu, act);
    peers[u] = 0u;
    if (act) {
      const uint32_t d = (kk[u] >> shift) & (kRadix - 1);
      peers[u] = __match_any_sync(live, d);
      if (lane == __ffs(peers[u]) - 1) atomicAdd(&wh[warp][d], (uint32_t)__popc(peers[u]));
    }
  }
  __syncthreads();
  // warps of the tile one after another: warp w's first slot per digit
#pragma unroll
  for (int j = 0; j < kDigitsPerThread; ++j) {
    const int d = threadIdx.x * kDigitsPerThread + j;
    uint32_t run = first[d];
#pragma unroll
    for (int w = 0; w < kTileWarps; ++w) {
      const uint32_t c = wh[w][d];
      wh[w][d] = run;
      run += c;
    }
  }
  __syncthreads();
  const uint32_t below = (1u << lane) - 1u;
#pragma unroll
  for (int u = 0; u < kWarpRounds; ++u) {
    const bool act = peers[u] != 0u;  // an active lane is its own peer
    const uint32_t d = (kk[u] >> shift) & (kRadix - 1);
    const uint32_t pos = act ? wh[warp][d] + __popc(peers[u] & below) : 0u;
    __syncwarp();
    if (act && lane == 31 - __clz(peers[u])) wh[warp][d] += __popc(peers[u]);
    __syncwarp();
    if (act) {
      if (keyOut) keyOut[pos] = kk[u];
      valOut[pos] = vv[u];
    }
  }
}

__global__ void k_place(const uint32_t* __restrict__ cell, const uint32_t* __restrict__ rank,
                        const uint32_t* __restrict__ start, int64_t nq, int32_t* order) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= nq) return;
  order[start[cell[i]] + rank[i]] = (int32_t)i;
}

// Puts the queries of each cell back in index order (the atomic ranks of
// k_place are in arrival order): queries that are neighbours in the input
// (points of one scan line, say) then share warps in input order, so the
// warps' result rows lie side by side and their stores coalesce. Cells with
// more than kRunSort queries keep arrival order; the order only affects
// speed, never results.
// Runs of up to kRunRegs queries are loaded at once and sorted in registers
// by a network (independent loads instead of a chain of dependent ones);
// longer runs, up to kRunSort, by insertion in place.
constexpr int kRunSort = 64;
constexpr int kRunRegs = 16;
__global__ void k_sort_runs(const uint32_t* __restrict__ start, int64_t bins, int64_t nq, int32_t* order,
                            const int64_t* binsDev) {
  bins = live_count(bins, binsDev);
  const int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (b >= bins) return;
  const int64_t s = start[b];
  const int64_t e = b + 1 < bins ? (int64_t)start[b + 1] : nq;
  if (e - s < 2 || e - s > kRunSort) return;
  if (e - s <= kRunRegs) {
    const int len = (int)(e - s);
    int32_t v[kRunRegs];
#pragma unroll
    for (int j = 0; j < kRunRegs; ++j) v[j] = j < len ? order[s + j] : INT_MAX;
#pragma unroll
    for (int k2 = 2; k2 <= kRunRegs; k2 <<= 1) {
#pragma unroll
      for (int jj = k2 >> 1; jj > 0; jj >>= 1) {
#pragma unroll
        for (int i = 0; i < kRunRegs; ++i) {
          const int l = i ^ jj;
          if (l > i) {
            const int32_t lo = min(v[i], v[l]), hi = max(v[i], v[l]);
            const bool up = (i & k2) == 0;
            v[i] = up ? lo : hi;
            v[l] = up ? hi : lo;
          }
        }
      }
    }
#pragma unroll
    for (int j = 0; j < kRunRegs; ++j)
      if (j < len) order[s + j] = v[j];
    return;
  }
  for (int64_t i = s + 1; i < e; ++i) {
    const int32_t v = order[i];
    int64_t j = i - 1;
    while (j >= s && order[j] > v) {
      order[j + 1] = order[j];
      --j;
    }
    order[j + 1] = v;
  }
}

}  // namespace

__global__ void k_zero_u32(uint32_t* data, int64_t n, const int64_t* nDev) {
  n = live_count(n, nDev);
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    data[i] = 0u;
}

int scan_exclusive_u32(uint32_t* data, int64_t n, uint32_t* dTotal, cudaStream_t stream, const int64_t* nDev) {
  const int nb = ceil_div(n, kB);
  uint32_t* sums = nullptr;
  NABO_CUDA_TRY(scratch_alloc((void**)&sums, (size_t)std::max(nb, 1) * sizeof(uint32_t), stream));
  k_block_sums<<<nb, kB, 0, stream>>>(data, n, sums, nDev);
  k_scan_sums<<<1, kB, 0, stream>>>(sums, nb, dTotal, nDev);
  k_apply<<<nb, kB, 0, stream>>>(data, n, sums, nDev);
  const cudaError_t e = cudaGetLastError();
  scratch_free(sums, stream);
  if (e != cudaSuccess) return cuda_error(e, "scan_exclusive_u32");
  return kOk;
}

int zero_u32(uint32_t* data, int64_t n, const int64_t* nDev, cudaStream_t stream) {
  int device = 0, sms = 0;
  NABO_CUDA_TRY(cudaGetDevice(&device));
  NABO_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
  k_zero_u32<<<std::max(1, std::min(ceil_div(n, kB), 8 * std::max(sms, 1))), kB, 0, stream>>>(data, n, nDev);
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? kOk : cuda_error(e, "zero_u32");
}

int order_by_cells(const uint32_t* dCell, const uint32_t* dRank, uint32_t* dHist, int64_t bins, int64_t nq,
                   int32_t* dOrder, cudaStream_t stream, const int64_t* binsDev) {
  const int rc = scan_exclusive_u32(dHist, bins, nullptr, stream, binsDev);
  if (rc != kOk) return rc;
  k_place<<<ceil_div(nq, kB), kB, 0, stream>>>(dCell, dRank, dHist, nq, dOrder);
  k_sort_runs<<<ceil_div(bins, kB), kB, 0, stream>>>(dHist, bins, nq, dOrder, binsDev);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_error(e, "order_by_cells");
  return kOk;
}

namespace {

// One block per tile of kTile elements; the [tile][digit] counts take
// 4 kRadix / kTile bytes per element. (Tiles of 2048: 562 blocks for a
// million keys, twice the warps of 4096-element tiles to hide the ranking
// loop's shared-memory latency.) The sort's scratch is one allocation (a call makes one
// stream-ordered allocation and one free instead of six of each): the
// keys when the sort makes them, the counts, the digit totals, a second
// key array and two value arrays, each on a 256-byte boundary.
struct SortPlan {
  int64_t nTiles = 0;
  int blocks = 0;
  size_t offKeys = 0, offHist = 0, offTotals = 0, offK2 = 0, offV1 = 0, offV2 = 0, bytes = 0;
  SortPlan(int64_t n, bool ownKeys) {
    nTiles = ceil_div(n, (int64_t)kTile);
    blocks = (int)nTiles;
    const auto take = [this](size_t b) {
      const size_t at = bytes;
      bytes += (b + 255) & ~size_t(255);
      return at;
    };
    const size_t row = (size_t)n * sizeof(uint32_t);
    if (ownKeys) offKeys = take(row);
    offHist = take((size_t)nTiles * kRadix * sizeof(uint32_t));
    offTotals = take((size_t)kRadix * sizeof(uint32_t));
    offK2 = take(row);
    offV1 = take(row);
    offV2 = take(row);
  }
};

struct SortScratch {
  void* block = nullptr;
  uint32_t *keys = nullptr, *hist = nullptr, *totals = nullptr, *k2 = nullptr, *v1 = nullptr, *v2 = nullptr;
  cudaError_t alloc(const SortPlan& P, bool ownKeys, cudaStream_t stream) {
    const cudaError_t e = scratch_alloc(&block, P.bytes, stream);
    if (e != cudaSuccess) {
      block = nullptr;
      return e;
    }
    char* b = static_cast<char*>(block);
    const auto at = [b](size_t off) { return reinterpret_cast<uint32_t*>(b + off); };
    if (ownKeys) keys = at(P.offKeys);
    hist = at(P.offHist);
    totals = at(P.offTotals);
    k2 = at(P.offK2);
    v1 = at(P.offV1);
    v2 = at(P.offV2);
    return cudaSuccess;
  }
  void release(cudaStream_t stream) {
    if (block) scratch_free(block, stream);
    block = nullptr;
  }
};

// The radix passes over dKeys (clobbered). Pass 0 takes the values from
// dVals or, if null, the element indices; its digit counts are already in
// S.hist when `firstCounted`. The last pass writes the values to dOrder.
int radix_passes(uint32_t* dKeys, int64_t n, int bits, const uint32_t* dVals, int32_t* dOrder, const SortPlan& P,
                 const SortScratch& S, bool firstCounted, cudaStream_t stream) {
  const int passes = std::max(1, (bits + kRadixBits - 1) / kRadixBits);
  uint32_t* hist = S.hist;
  uint32_t* totals = S.totals;
  int rc = kOk;
  cudaError_t e = cudaSuccess;
  uint32_t* kin = dKeys;
  uint32_t* kout = S.k2;
  const uint32_t* vin = dVals;
  uint32_t* vbuf[2] = {S.v1, S.v2};
  for (int p = 0; p < passes && rc == kOk; ++p) {
    const int shift = p * kRadixBits;
    const bool last = p == passes - 1;
    if (p > 0 || !firstCounted) k_tile_hist<<<P.blocks, kTileThreads, 0, stream>>>(kin, n, shift, hist);
    k_tile_scan<<<kRadix / 32, 32 * kScanGroups, 0, stream>>>(hist, P.nTiles, totals);
    uint32_t* vout = last ? reinterpret_cast<uint32_t*>(dOrder) : vbuf[p & 1];
    k_tile_scatter<<<P.blocks, kTileThreads, 0, stream>>>(kin, vin, n, shift, hist, totals,
                                                           last ? nullptr : kout, vout);
    e = cudaGetLastError();
    if (e != cudaSuccess) rc = cuda_error(e, "radix sort");
    std::swap(kin, kout);
    vin = vout;
  }
  return rc;
}

}  // namespace

int sort_order_u32(uint32_t* dKeys, int64_t n, int bits, int32_t* dOrder, cudaStream_t stream, const uint32_t* dVals) {
  if (n <= 0) return kOk;
  if (n > (int64_t)INT32_MAX) return set_error(kErrUnsupported, "sort: too many elements");
  const SortPlan P(n, false);
  SortScratch S;
  NABO_CUDA_TRY(S.alloc(P, false, stream));
  const int rc = radix_passes(dKeys, n, bits, dVals, dOrder, P, S, false, stream);
  S.release(stream);
  return rc;
}

template <typename T>
int order_queries(const T* dQuery, int64_t nq, int64_t qStride, int dim, const double* lo, const double* hi,
                  int32_t* dOrder, cudaStream_t stream, const QueryChunks* chunks, T* copyOut) {
  if (nq <= 0) return kOk;
  if (nq > (int64_t)INT32_MAX) return set_error(kErrUnsupported, "sort: too many elements");
  if (dim < 1 || dim > kMortonDims) return set_error(kErrInternal, "Morton order: 1 to 3 dimensions");
  CellParams p;
  p.dims = dim;
  p.bits = 30 / p.dims;
  p.shift = 0;
  p.nChunks = chunks && chunks->n > 1 ? std::min(chunks->n, kMaxQueryChunks) : 0;
  for (int c = 0; c < kMaxQueryChunks; ++c) p.chunkEnd[c] = c < p.nChunks ? chunks->end[c] : nq;
  int chunkBits = 0;
  if (p.nChunks > 1) {
    while ((1 << chunkBits) < p.nChunks) ++chunkBits;
    // the chunk number above the Morton code, within 32 bits
    p.bits = std::min(p.bits, (32 - chunkBits) / p.dims);
  }
  if (p.bits < 1 || p.bits * p.dims + chunkBits > 32) return set_error(kErrInternal, "sort: too many query chunks");
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
  const SortPlan P(nq, true);
  SortScratch S;
  const cudaError_t e = S.alloc(P, true, stream);
  if (e != cudaSuccess) return cuda_error(e, "order scratch");
  k_morton_tiles<T><<<P.blocks, kTileThreads, 0, stream>>>(dQuery, nq, qStride, p, S.keys, S.hist, copyOut);
  const int rc = radix_passes(S.keys, nq, p.bits * p.dims + chunkBits, nullptr, dOrder, P, S, true, stream);
  S.release(stream);
  return rc;
}

QueryChunks shrinking_chunks(int64_t nq, int n) {
  QueryChunks q;
  q.n = std::max(1, std::min(n, kMaxQueryChunks));
  const int64_t total = (int64_t)q.n * (q.n + 1) / 2;
  int64_t w = 0;
  for (int c = 0; c < q.n; ++c) {
    w += q.n - c;
    q.end[c] = c + 1 == q.n ? nq : (int64_t)((double)nq * (double)w / (double)total);
  }
  return q;
}

template int order_queries<float>(const float*, int64_t, int64_t, int, const double*, const double*, int32_t*,
                                  cudaStream_t, const QueryChunks*, float*);
template int order_queries<double>(const double*, int64_t, int64_t, int, const double*, const double*, int32_t*,
                                   cudaStream_t, const QueryChunks*, double*);

}  // namespace nabo_gb300
