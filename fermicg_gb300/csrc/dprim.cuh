// Device primitives of the closed-sigma planner: an exclusive prefix sum and a stable
// least-significant-digit radix sort of (64-bit key, 32-bit value) pairs.
//
// Scan: tiles of 1024 values (256 threads x 4) are scanned in shared memory, the tile totals
// are scanned the same way (recursively), and added back.
//
// Radix sort: one pass per 8-bit digit, lowest digit first.  Per pass, every tile of 2048
// elements counts its digits (hist), the counts are laid out digit-major over tiles and
// scanned, and the tile scatters its elements to (digit offset of the tile + rank among the
// tile's elements of that digit).  The rank keeps the input order (steps of 256 consecutive
// elements; within a step, warps in order and lanes in order through __match_any_sync), so
// every pass is stable and the passes together sort by the whole key, ties in input order.
// A pass can take its digit from the key or from a per-element value computed from the
// 32-bit value (the planner's segment of a row), which sorts by a second key without
// storing it.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

namespace fcg {
namespace dprim {

constexpr int kScanThreads = 256;
constexpr int kScanItems = 4;
constexpr int kScanTile = kScanThreads * kScanItems;

// exclusive scan of each tile of a[0, n) in place; the tile's total to sums[tile] (when given)
template <typename T>
__global__ void __launch_bounds__(kScanThreads) scan_tiles_kernel(T* a, int64_t n, T* sums) {
  __shared__ T warp_tot[kScanThreads / 32];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int64_t base = int64_t(blockIdx.x) * kScanTile + int64_t(tid) * kScanItems;
  T v[kScanItems];
  T sum = 0;
#pragma unroll
  for (int i = 0; i < kScanItems; ++i) {
    v[i] = base + i < n ? a[base + i] : T(0);
    sum += v[i];
  }
  // inclusive scan of the thread sums within the warp
  T inc = sum;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const T o = __shfl_up_sync(0xffffffffu, inc, d);
    if (lane >= d) inc += o;
  }
  if (lane == 31) warp_tot[warp] = inc;
  __syncthreads();
  T before = 0, total = 0;
#pragma unroll
  for (int w = 0; w < kScanThreads / 32; ++w) {
    if (w < warp) before += warp_tot[w];
    total += warp_tot[w];
  }
  T run = before + inc - sum;
#pragma unroll
  for (int i = 0; i < kScanItems; ++i) {
    if (base + i < n) a[base + i] = run;
    run += v[i];
  }
  if (sums && tid == 0) sums[blockIdx.x] = total;
}

template <typename T>
__global__ void scan_add_kernel(T* a, int64_t n, const T* sums) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i < n) a[i] += sums[i / kScanTile];
}

// scratch values exclusive_scan needs for n values
inline int64_t scan_scratch(int64_t n) {
  int64_t s = 0;
  while (n > kScanTile) {
    n = (n + kScanTile - 1) / kScanTile;
    s += n;
  }
  return s;
}

// exclusive prefix sum of a[0, n) in place (scratch: scan_scratch(n) values)
template <typename T>
cudaError_t exclusive_scan(T* a, int64_t n, T* scratch, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  const int64_t tiles = (n + kScanTile - 1) / kScanTile;
  if (tiles == 1) {
    scan_tiles_kernel<T><<<1, kScanThreads, 0, s>>>(a, n, nullptr);
    return cudaGetLastError();
  }
  scan_tiles_kernel<T><<<unsigned(tiles), kScanThreads, 0, s>>>(a, n, scratch);
  cudaError_t e = exclusive_scan(scratch, tiles, scratch + tiles, s);
  if (e != cudaSuccess) return e;
  scan_add_kernel<T><<<unsigned((n + 255) / 256), 256, 0, s>>>(a, n, scratch);
  return cudaGetLastError();
}

// ---- radix sort ---------------------------------------------------------------------------
constexpr int kSortThreads = 256;
constexpr int kSortSteps = 8;
constexpr int kSortTile = kSortThreads * kSortSteps;  // elements per tile
constexpr int kRadix = 256;

// The digit of one pass: bits [shift, shift + 8) of the key (seg_n == 0), or of the segment
// seg_sector[v / seg_n] * seg_n + v % seg_n of the value v (seg_n > 0).
struct Digit {
  int shift;
  int seg_n;
  const int32_t* seg_sector;
  __device__ __forceinline__ unsigned operator()(uint64_t key, uint32_t v) const {
    if (seg_n > 0) {
      const uint64_t seg = uint64_t(__ldg(seg_sector + v / uint32_t(seg_n))) * uint64_t(seg_n) + v % uint32_t(seg_n);
      return unsigned(seg >> shift) & (kRadix - 1);
    }
    return unsigned(key >> shift) & (kRadix - 1);
  }
};

// digit counts of every tile, digit-major: cnt[d * n_tiles + tile]
__global__ void __launch_bounds__(kSortThreads) radix_hist_kernel(const uint64_t* __restrict__ keys,
                                                                  const uint32_t* __restrict__ vals, int64_t n,
                                                                  Digit dg, int32_t* __restrict__ cnt,
                                                                  int64_t n_tiles) {
  __shared__ int h[kRadix];
  const int tid = threadIdx.x;
  h[tid] = 0;
  __syncthreads();
  const int64_t base = int64_t(blockIdx.x) * kSortTile;
#pragma unroll
  for (int r = 0; r < kSortSteps; ++r) {
    const int64_t i = base + r * kSortThreads + tid;
    if (i < n) atomicAdd(&h[dg(keys[i], vals[i])], 1);
  }
  __syncthreads();
  cnt[int64_t(tid) * n_tiles + blockIdx.x] = h[tid];
}

// stable scatter of every tile to its scanned digit offsets
__global__ void __launch_bounds__(kSortThreads) radix_scatter_kernel(
    const uint64_t* __restrict__ kin, const uint32_t* __restrict__ vin, uint64_t* __restrict__ kout,
    uint32_t* __restrict__ vout, int64_t n, Digit dg, const int32_t* __restrict__ offs, int64_t n_tiles) {
  constexpr int kWarps = kSortThreads / 32;
  __shared__ int s_base[kRadix];
  __shared__ int s_run[kRadix];
  __shared__ int s_cnt[kWarps][kRadix];
  __shared__ int s_off[kWarps][kRadix];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  s_base[tid] = offs[int64_t(tid) * n_tiles + blockIdx.x];
  s_run[tid] = 0;
#pragma unroll
  for (int w = 0; w < kWarps; ++w) s_cnt[w][tid] = 0;
  __syncthreads();
  const unsigned lt = (1u << lane) - 1u;
  const int64_t base = int64_t(blockIdx.x) * kSortTile;
  for (int r = 0; r < kSortSteps; ++r) {
    const int64_t i = base + r * kSortThreads + tid;
    const bool valid = i < n;
    uint64_t k = 0;
    uint32_t v = 0;
    unsigned d = kRadix;  // past the last digit: an element beyond n (never counted or written)
    if (valid) {
      k = kin[i];
      v = vin[i];
      d = dg(k, v);
    }
    const unsigned peers = __match_any_sync(0xffffffffu, d);
    const int rank = __popc(peers & lt);
    if (valid && rank == 0) s_cnt[warp][d] = __popc(peers);
    __syncthreads();
    {  // thread tid: the offsets of digit tid for every warp of this step
      int acc = s_run[tid];
#pragma unroll
      for (int w = 0; w < kWarps; ++w) {
        const int c = s_cnt[w][tid];
        s_off[w][tid] = acc;
        acc += c;
        s_cnt[w][tid] = 0;
      }
      s_run[tid] = acc;
    }
    __syncthreads();
    if (valid) {
      const int pos = s_base[d] + s_off[warp][d] + rank;
      kout[pos] = k;
      vout[pos] = v;
    }
  }
}

inline int64_t sort_tiles(int64_t n) { return (n + kSortTile - 1) / kSortTile; }

// digit-count values (and their scan scratch) radix_sort needs for n elements
inline int64_t sort_scratch(int64_t n) {
  const int64_t c = kRadix * sort_tiles(n);
  return c + scan_scratch(c);
}

// Stable sort of (k[0], v[0]) by the given passes, ping-ponging with (k[1], v[1]); *which is
// the buffer holding the result.  n < 2^31.
inline cudaError_t radix_sort(uint64_t* k[2], uint32_t* v[2], int64_t n, const Digit* passes, int n_passes,
                              int32_t* scratch, int* which, cudaStream_t s) {
  *which = 0;
  if (n <= 1) return cudaSuccess;
  const int64_t tiles = sort_tiles(n);
  int32_t* cnt = scratch;
  int32_t* scan_tmp = scratch + kRadix * tiles;
  for (int p = 0; p < n_passes; ++p) {
    const int a = *which;
    radix_hist_kernel<<<unsigned(tiles), kSortThreads, 0, s>>>(k[a], v[a], n, passes[p], cnt, tiles);
    cudaError_t e = exclusive_scan<int32_t>(cnt, kRadix * tiles, scan_tmp, s);
    if (e != cudaSuccess) return e;
    radix_scatter_kernel<<<unsigned(tiles), kSortThreads, 0, s>>>(k[a], v[a], k[1 - a], v[1 - a], n, passes[p], cnt,
                                                                  tiles);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    *which = 1 - a;
  }
  return cudaSuccess;
}

}  // namespace dprim
}  // namespace fcg
