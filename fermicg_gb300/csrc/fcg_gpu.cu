// GB300 (sm_103a) TPSCI sigma build behind the C ABI of include/fcg_gpu.h.
//
// Device layout (one context, one stream):
//   op data      the TDM blocks of every cluster in one blob (float64 + float32 copy),
//                block (p, I, J) at off + p + nidx*(I + mb*J)
//   dressed ops  per term and per sector pair of its dressed cluster,
//                W[(rest), b, k] = sum_i ints[..i..] G[i, b, k]  (float64 + float32 copy);
//                1-body terms store their "H" block here
//   block index  dense int32 table (cluster, op, fb_a, fb_b, fk_a, fk_b) -> block id
//   state        local states int16 [n_cfg][N]
//   plan         work items (bra group x ket group x term-sector list), their triple
//                prefix sum, the grouping permutation pool and the term-sector records
//   vectors      coefficients / sigma row-major [n_cfg][R] in the compute precision
//
// Kernels:
//   dress_kernel         W blocks, once per problem (fcg_set_terms)
//   closed_sigma_kernel  one pass over the flattened (work item, bra, ket, term) triple
//                        space; each CTA takes a fixed chunk (exact load balance), each
//                        warp 32 consecutive triples; a matrix element is the W column of
//                        the dressed cluster contracted with the TDM columns of the other
//                        active clusters (contract_matrix_element, src/tpsci_inner.jl:10-216,
//                        re-associated); sigma is scattered with warp-segmented sums and
//                        one atomic per run of equal bra rows.
//   diag kernels         compute_diagonal (src/tpsci_outer.jl:694-757).
//   pack / unpack        column-major float64 <-> row-major compute precision.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <map>
#include <mutex>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/fcg_gpu.h"
#include "fcg_internal.h"

using namespace fcg;

#include "fcg_ctx.cuh"

// ---------------------------------------------------------------------------------------
// device code
namespace {

// ---- dressing ----------------------------------------------------------------------------
__global__ void dress_kernel(const DressJob* __restrict__ jobs, const double* __restrict__ op,
                             const double* __restrict__ ints, double* __restrict__ w) {
  const DressJob J = jobs[blockIdx.x];
  const int64_t n = int64_t(J.rest_len) * J.mb * J.mk;
  for (int64_t e = threadIdx.x; e < n; e += blockDim.x) {
    const int r = int(e % J.rest_len);
    const int64_t bk = e / J.rest_len;
    const int b = int(bk % J.mb);
    const int k = int(bk / J.mb);
    double acc;
    if (J.one_body) {
      acc = op[J.g_off + b + int64_t(J.mb) * k];
    } else {
      int64_t base = J.ints_off;
      int rr = r;
      for (int o = 0; o < J.nrem; ++o) {
        base += int64_t(rr % J.rem_dim[o]) * J.rem_stride[o];
        rr /= J.rem_dim[o];
      }
      const double* g = op + J.g_off + int64_t(J.nq) * (b + int64_t(J.mb) * k);
      acc = 0.0;
      for (int i = 0; i < J.nq; ++i) acc = fma(ints[base + int64_t(i) * J.stride_q], g[i], acc);
    }
    w[J.w_off + e] = acc;
  }
}

__global__ void to_float_kernel(const double* __restrict__ a, float* __restrict__ b, int64_t n) {
  int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  for (; i < n; i += int64_t(gridDim.x) * blockDim.x) b[i] = float(a[i]);
}

// One TDM block of the caller's blob placed at its aligned offset, with its float copy.
struct PlaceJob {
  int64_t src, dst, n;
};

__global__ void place_blocks_kernel(const PlaceJob* __restrict__ jobs, const double* __restrict__ raw,
                                    double* __restrict__ op64, float* __restrict__ op32) {
  const PlaceJob J = jobs[blockIdx.x];
  for (int64_t i = threadIdx.x; i < J.n; i += blockDim.x) {
    const double v = raw[J.src + i];
    op64[J.dst + i] = v;
    op32[J.dst + i] = float(v);
  }
}

// Column maxima over the bra index, used by the open-sigma screen:
// out[i + len*k] = max_b |in[i + len*(b + mb*k)]| for every block of a list.
struct MaxJob {
  int64_t in_off, out_off;
  int32_t len, mb, mk, pad;
};

__global__ void colmax_kernel(const MaxJob* __restrict__ jobs, const double* __restrict__ in,
                              double* __restrict__ out) {
  const MaxJob J = jobs[blockIdx.x];
  const int64_t n = int64_t(J.len) * J.mk;
  for (int64_t e = threadIdx.x; e < n; e += blockDim.x) {
    const int i = int(e % J.len);
    const int64_t k = e / J.len;
    double m = 0.0;
    for (int b = 0; b < J.mb; ++b) m = fmax(m, fabs(in[J.in_off + i + int64_t(J.len) * (b + int64_t(J.mb) * k)]));
    out[J.out_off + e] = m;
  }
}

// ---- closed sigma ------------------------------------------------------------------------
// ---- vector loads ---------------------------------------------------------------------------
// Vec4: 4 consecutive elements (16 bytes float, 32 bytes double); Chunk: 32 bytes (8 float
// or 4 double) in one 256-bit load.  Callers guarantee the alignment: device TDM and W
// blocks start on multiples of kAlign = 8 elements and the columns read this way have
// lengths that are multiples of the vector length.
template <typename T>
struct Vec4;
template <>
struct Vec4<float> {
  float v[4];
  __device__ __forceinline__ void load(const float* p) {
    const float4 q = __ldg(reinterpret_cast<const float4*>(p));
    v[0] = q.x, v[1] = q.y, v[2] = q.z, v[3] = q.w;
  }
};
template <>
struct Vec4<double> {
  double v[4];
  __device__ __forceinline__ void load(const double* p) {
    asm("ld.global.nc.v4.f64 {%0, %1, %2, %3}, [%4];" : "=d"(v[0]), "=d"(v[1]), "=d"(v[2]), "=d"(v[3]) : "l"(p));
  }
};

template <typename T>
struct Chunk;
template <>
struct Chunk<float> {
  static constexpr int n = 8;
  float v[8];
  __device__ __forceinline__ void load(const float* p) {
    asm("ld.global.nc.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
        : "=f"(v[0]), "=f"(v[1]), "=f"(v[2]), "=f"(v[3]), "=f"(v[4]), "=f"(v[5]), "=f"(v[6]), "=f"(v[7])
        : "l"(p));
  }
};
template <>
struct Chunk<double> {
  static constexpr int n = 4;
  double v[4];
  __device__ __forceinline__ void load(const double* p) {
    asm("ld.global.nc.v4.f64 {%0, %1, %2, %3}, [%4];" : "=d"(v[0]), "=d"(v[1]), "=d"(v[2]), "=d"(v[3]) : "l"(p));
  }
};

// one local state out of a 16-byte row of 8 int16 (no dynamic register indexing)
__device__ __forceinline__ int state_of(const uint4& r, int c) {
  const unsigned w = c < 4 ? (c < 2 ? r.x : r.y) : (c < 6 ? r.z : r.w);
  return int((w >> (16 * (c & 1))) & 0xFFFFu);
}

// <bra| term |ket> from a term-sector record: the dressed cluster's W column contracted
// with the other active clusters' TDM columns (contract_matrix_element re-associated).
// Columns whose length is a multiple of 4 are read with 16-byte loads (blocks are aligned
// on the device); the common n=4 shapes are fully unrolled.
template <typename T>
__device__ __forceinline__ T dressed_element(const TermSector& ts, const T* __restrict__ w,
                                             const T* __restrict__ op, const uint4& rb, const uint4& rk) {
  const T* wc = w + ts.w_off + int64_t(ts.rest_len) * (state_of(rb, ts.cw) + int64_t(ts.w_mb) * state_of(rk, ts.cw));
  if (ts.nrem == 0) return __ldg(wc);
  const int d0 = ts.g_dim[0];
  const T* g0 =
      op + ts.g_off[0] + int64_t(d0) * (state_of(rb, ts.cr[0]) + int64_t(ts.g_mb[0]) * state_of(rk, ts.cr[0]));
  T me = T(0);
  constexpr int C = Chunk<T>::n;
  if (ts.nrem == 1) {
    if (d0 % C == 0) {
      for (int i = 0; i < d0; i += C) {
        Chunk<T> a, g;
        a.load(wc + i);
        g.load(g0 + i);
#pragma unroll
        for (int q = 0; q < C; ++q) me = fma(a.v[q], g.v[q], me);
      }
    } else if ((d0 & 3) == 0) {
      for (int i = 0; i < d0; i += 4) {
        Vec4<T> a, g;
        a.load(wc + i);
        g.load(g0 + i);
#pragma unroll
        for (int q = 0; q < 4; ++q) me = fma(a.v[q], g.v[q], me);
      }
    } else {
      for (int i = 0; i < d0; ++i) me = fma(__ldg(wc + i), __ldg(g0 + i), me);
    }
  } else {
    const int d1 = ts.g_dim[1];
    const T* g1 =
        op + ts.g_off[1] + int64_t(d1) * (state_of(rb, ts.cr[1]) + int64_t(ts.g_mb[1]) * state_of(rk, ts.cr[1]));
    if (ts.nrem == 2) {
      if (d0 == 4 && d1 == 4) {
        Vec4<T> a0, a1;
        a0.load(g0);
        a1.load(g1);
#pragma unroll
        for (int c = 0; c < 16 / C; ++c) {
          Chunk<T> wv;
          wv.load(wc + C * c);
#pragma unroll
          for (int h = 0; h < C / 4; ++h) {
            T acc = wv.v[4 * h] * a0.v[0];
#pragma unroll
            for (int i = 1; i < 4; ++i) acc = fma(wv.v[4 * h + i], a0.v[i], acc);
            me = fma(acc, a1.v[c * (C / 4) + h], me);
          }
        }
      } else {
        for (int j = 0; j < d1; ++j) {
          const T* wj = wc + d0 * j;
          T acc = T(0);
          for (int i = 0; i < d0; ++i) acc = fma(__ldg(wj + i), __ldg(g0 + i), acc);
          me = fma(acc, __ldg(g1 + j), me);
        }
      }
    } else {
      const int d2 = ts.g_dim[2];
      const T* g2 =
          op + ts.g_off[2] + int64_t(d2) * (state_of(rb, ts.cr[2]) + int64_t(ts.g_mb[2]) * state_of(rk, ts.cr[2]));
      if (d0 == 4 && d1 == 4 && d2 == 4) {
        Vec4<T> a0, a1, a2;
        a0.load(g0);
        a1.load(g1);
        a2.load(g2);
#pragma unroll
        for (int l = 0; l < 4; ++l) {
          T accl = T(0);
#pragma unroll
          for (int c = 0; c < 16 / C; ++c) {
            Chunk<T> wv;
            wv.load(wc + 16 * l + C * c);
#pragma unroll
            for (int h = 0; h < C / 4; ++h) {
              T acc = wv.v[4 * h] * a0.v[0];
#pragma unroll
              for (int i = 1; i < 4; ++i) acc = fma(wv.v[4 * h + i], a0.v[i], acc);
              accl = fma(acc, a1.v[c * (C / 4) + h], accl);
            }
          }
          me = fma(accl, a2.v[l], me);
        }
      } else {
        for (int l = 0; l < d2; ++l) {
          T accl = T(0);
          for (int j = 0; j < d1; ++j) {
            const T* wj = wc + d0 * (j + d1 * l);
            T acc = T(0);
            for (int i = 0; i < d0; ++i) acc = fma(__ldg(wj + i), __ldg(g0 + i), acc);
            accl = fma(acc, __ldg(g1 + j), accl);
          }
          me = fma(accl, __ldg(g2 + l), me);
        }
      }
    }
  }
  return ts.sign < 0 ? -me : me;
}

constexpr int kSigmaThreads = 256;       // 8 warps per CTA
constexpr int kWarpsPerCta = kSigmaThreads / 32;
constexpr int kMaxR = 16;
constexpr int kTuneCandidates = 4;  // closed-sigma kernel candidates of the tuner

struct LaneParams {
  const LaneJob* jobs;       // 32 per warp task
  const int64_t* chunk_lo;   // n_chunks + 1: first warp task of each warp chunk
  const int64_t* chunk_val;  // n_chunks + 1: first stored value of each chunk
  int64_t n_chunks;
  const int32_t* perm;
  const TermSector* ts;
  const int16_t* cfg;  // [n_cfg][kCfgStride]
  int R;
};

// R coefficients of one row of a row-major [n][R] array (RR > 0: R == RR, known at compile
// time), with vector loads when exactly 2 or 4 roots; out[r] = 0 for r >= R
template <typename T, int RR, int RV>
__device__ __forceinline__ void load_row(const T* __restrict__ p, int R, T* out) {
  if (RR == 4 && sizeof(T) == 4) {
    const float4 q = __ldg(reinterpret_cast<const float4*>(p));
    out[0] = q.x, out[1] = q.y, out[2] = q.z, out[3] = q.w;
  } else if (RR == 4) {
    Vec4<double> q;
    q.load(reinterpret_cast<const double*>(p));
#pragma unroll
    for (int r = 0; r < 4; ++r) out[r] = T(q.v[r]);
  } else if (RR == 2 && sizeof(T) == 4) {
    const float2 q = __ldg(reinterpret_cast<const float2*>(p));
    out[0] = q.x, out[1] = q.y;
  } else if (RR == 2) {
    const double2 q = __ldg(reinterpret_cast<const double2*>(p));
    out[0] = T(q.x), out[1] = T(q.y);
  } else {
#pragma unroll
    for (int r = 0; r < RV; ++r) out[r] = r < R ? __ldg(p + r) : T(0);
  }
}

// sig[row] += acc for R roots: one vector reduction for exactly four float roots, else
// scalar atomics
template <typename T, int RR, int RV>
__device__ __forceinline__ void add_row(T* __restrict__ sig, int b, const T* acc, int R) {
  T* dst = sig + int64_t(b) * R;
  if (RR == 4 && sizeof(T) == 4) {
    asm volatile("red.global.add.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(dst), "f"(float(acc[0])), "f"(float(acc[1])),
                 "f"(float(acc[2])), "f"(float(acc[3]))
                 : "memory");
  } else {
#pragma unroll
    for (int r = 0; r < RV; ++r)
      if (r < R) atomicAdd(dst + r, acc[r]);
  }
}

// One warp chunk of the closed sigma: the chunk's warp tasks in order, lane i of a task
// running lane job 32 * task + i.  For each of its kets the lane sums the work item's terms
// (the lanes of a warp mostly share the term records: broadcast loads), multiplies by the
// ket's coefficients and keeps the bra row in registers; the row goes to sigma once per job.
// RR > 0: exactly RR roots; RR == 0: p.R roots, at most RMAX.
template <typename T, int RR, int RMAX = kMaxR>
__device__ __forceinline__ void closed_lane_warp(const LaneParams& p, const T* __restrict__ w,
                                                 const T* __restrict__ op, const T* __restrict__ cin,
                                                 T* __restrict__ sig, int64_t chunk) {
  constexpr int RV = RR > 0 ? RR : RMAX;
  const int R = RR > 0 ? RR : p.R;
  const int lane = threadIdx.x & 31;
  const int64_t t_lo = __ldg(p.chunk_lo + chunk), t_hi = __ldg(p.chunk_lo + chunk + 1);
  const uint4* cfg = reinterpret_cast<const uint4*>(p.cfg);
  for (int64_t wt = t_lo; wt < t_hi; ++wt) {
    const LaneJob j = p.jobs[wt * 32 + lane];
    if (j.len == 0) continue;
    const uint4 rb = __ldg(cfg + j.b);
    const TermSector* tsl = p.ts + j.ts_off;
    T acc[RV];
#pragma unroll
    for (int r = 0; r < RV; ++r) acc[r] = T(0);
    for (int kk = 0; kk < int(j.len); ++kk) {
      const int k = __ldg(p.perm + j.kp + kk);
      const uint4 rk = __ldg(cfg + k);
      T me = T(0);
      for (int t = 0; t < int(j.nt); ++t) me += dressed_element<T>(tsl[t], w, op, rb, rk);
      T c[RV];
      load_row<T, RR, RV>(cin + int64_t(k) * R, R, c);
#pragma unroll
      for (int r = 0; r < RV; ++r) acc[r] = fma(me, c[r], acc[r]);
    }
    add_row<T, RR, RV>(sig, j.b, acc, R);
  }
}

// MINB: resident CTAs per SM the register allocation is sized for (a tuning candidate)
template <typename T, int RR, int MINB>
__global__ void __launch_bounds__(kSigmaThreads, MINB)
    closed_sigma_lane_kernel(LaneParams p, const T* __restrict__ w, const T* __restrict__ op,
                             const T* __restrict__ cin, T* __restrict__ sig) {
  const int64_t chunk = int64_t(blockIdx.x) * kWarpsPerCta + (threadIdx.x >> 5);
  if (chunk >= p.n_chunks) return;
  closed_lane_warp<T, RR>(p, w, op, cin, sig, chunk);
}

// ---- stored Hamiltonian blocks -------------------------------------------------------------
// For every warp task the blocks hold 32 values per ket step, one per lane: the sum over the
// work item's terms of the dressed matrix element of the lane's (bra, ket) pair (added in term
// order in float64; 0 past the lane's kets), at chunk_val[chunk] + 32 * (longest job of each
// earlier task of the chunk, summed) + 32 * step + lane.  A sigma from the blocks reads each
// step's 32 values with one coalesced load instead of recomputing every term's contraction.
__device__ __forceinline__ int task_len(int len) { return __reduce_max_sync(0xffffffffu, unsigned(len)); }

__global__ void __launch_bounds__(kSigmaThreads) hcache_lane_build_kernel(LaneParams p, const double* __restrict__ w,
                                                                          const double* __restrict__ op,
                                                                          double* __restrict__ hc) {
  const int64_t chunk = int64_t(blockIdx.x) * kWarpsPerCta + (threadIdx.x >> 5);
  if (chunk >= p.n_chunks) return;
  const int lane = threadIdx.x & 31;
  const uint4* cfg = reinterpret_cast<const uint4*>(p.cfg);
  int64_t val = __ldg(p.chunk_val + chunk);
  const int64_t t_lo = __ldg(p.chunk_lo + chunk), t_hi = __ldg(p.chunk_lo + chunk + 1);
  for (int64_t wt = t_lo; wt < t_hi; ++wt) {
    const LaneJob j = p.jobs[wt * 32 + lane];
    const int steps = task_len(j.len);
    const uint4 rb = __ldg(cfg + j.b);
    for (int s = 0; s < steps; ++s) {
      double me = 0.0;
      if (s < int(j.len)) {
        const uint4 rk = __ldg(cfg + __ldg(p.perm + j.kp + s));
        for (int t = 0; t < int(j.nt); ++t) me += dressed_element<double>(p.ts[j.ts_off + t], w, op, rb, rk);
      }
      hc[val + 32 * s + lane] = me;
    }
    val += 32 * int64_t(steps);
  }
}

// sigma from the stored blocks: the chunk's warp tasks as in closed_lane_warp, one stored value
// per lane and ket in place of the term loop
template <typename T, int RR, int RMAX = kMaxR>
__device__ __forceinline__ void cached_lane_warp(const LaneParams& p, const T* __restrict__ hc,
                                                 const T* __restrict__ cin, T* __restrict__ sig, int64_t chunk) {
  constexpr int RV = RR > 0 ? RR : RMAX;
  const int R = RR > 0 ? RR : p.R;
  const int lane = threadIdx.x & 31;
  const int64_t t_lo = __ldg(p.chunk_lo + chunk), t_hi = __ldg(p.chunk_lo + chunk + 1);
  int64_t val = __ldg(p.chunk_val + chunk);
  for (int64_t wt = t_lo; wt < t_hi; ++wt) {
    const LaneJob j = p.jobs[wt * 32 + lane];
    const int steps = task_len(j.len);
    if (j.len > 0) {
      const T* hv = hc + val + lane;
      T acc[RV];
#pragma unroll
      for (int r = 0; r < RV; ++r) acc[r] = T(0);
      for (int s = 0; s < int(j.len); ++s) {
        const T v = __ldg(hv + 32 * s);
        T c[RV];
        load_row<T, RR, RV>(cin + int64_t(__ldg(p.perm + j.kp + s)) * R, R, c);
#pragma unroll
        for (int r = 0; r < RV; ++r) acc[r] = fma(v, c[r], acc[r]);
      }
      add_row<T, RR, RV>(sig, j.b, acc, R);
    }
    val += 32 * int64_t(steps);
  }
}

template <typename T, int RR>
__global__ void __launch_bounds__(kSigmaThreads) cached_sigma_lane_kernel(LaneParams p, const T* __restrict__ hc,
                                                                          const T* __restrict__ cin,
                                                                          T* __restrict__ sig) {
  const int64_t chunk = int64_t(blockIdx.x) * kWarpsPerCta + (threadIdx.x >> 5);
  if (chunk >= p.n_chunks) return;
  cached_lane_warp<T, RR>(p, hc, cin, sig, chunk);
}

// Many independent problems in one launch: problem q owns CTAs [cta0, cta0 + ceil(its chunks
// / 8)) of the grid; cta_problem maps every CTA to its problem.  Problems with stored
// Hamiltonian blocks (hc set) run in a second grid, numbered from cta0 there.
template <typename T>
struct GroupEntry {
  LaneParams p;
  const T* w;
  const T* op;
  const T* hc;       // stored Hamiltonian blocks, or null
  T* cin;            // row-major [n_cfg][R] working copy of C
  T* sig;            // row-major [n_cfg][R] sigma
  const double* src; // caller's column-major C
  double* dst;       // caller's column-major sigma
  int64_t cta0;
  int64_t n_cfg;
};

template <typename T, int RMAX>
__global__ void __launch_bounds__(kSigmaThreads, sizeof(T) == 4 ? 4 : 3)
    closed_sigma_grouped_kernel(const GroupEntry<T>* __restrict__ g, const int32_t* __restrict__ cta_problem) {
  const GroupEntry<T>& e = g[__ldg(cta_problem + blockIdx.x)];
  const LaneParams p = e.p;
  const int64_t chunk = (int64_t(blockIdx.x) - e.cta0) * kWarpsPerCta + (threadIdx.x >> 5);
  if (chunk >= p.n_chunks) return;
  closed_lane_warp<T, 0, RMAX>(p, e.w, e.op, e.cin, e.sig, chunk);
}

template <typename T, int RMAX>
__global__ void __launch_bounds__(kSigmaThreads)
    cached_sigma_grouped_kernel(const GroupEntry<T>* __restrict__ g, const int32_t* __restrict__ cta_problem) {
  const GroupEntry<T>& e = g[__ldg(cta_problem + blockIdx.x)];
  const LaneParams p = e.p;
  const int64_t chunk = (int64_t(blockIdx.x) - e.cta0) * kWarpsPerCta + (threadIdx.x >> 5);
  if (chunk >= p.n_chunks) return;
  cached_lane_warp<T, 0, RMAX>(p, e.hc, e.cin, e.sig, chunk);
}

// problem blockIdx.y: C to the row-major working copy, sigma zeroed
template <typename T>
__global__ void grouped_pack_kernel(const GroupEntry<T>* __restrict__ g) {
  const GroupEntry<T>& e = g[blockIdx.y];
  const int64_t n = e.n_cfg;
  const int R = e.p.R;
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n * R; i += int64_t(gridDim.x) * blockDim.x) {
    const int64_t row = i / R;
    const int r = int(i - row * R);
    e.cin[i] = T(e.src[row + n * r]);
    e.sig[i] = T(0);
  }
}

template <typename T>
__global__ void grouped_unpack_kernel(const GroupEntry<T>* __restrict__ g) {
  const GroupEntry<T>& e = g[blockIdx.y];
  const int64_t n = e.n_cfg;
  const int R = e.p.R;
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n * R; i += int64_t(gridDim.x) * blockDim.x) {
    const int64_t row = i % n;
    const int r = int(i / n);
    e.dst[i] = double(e.sig[row * R + r]);
  }
}

template <typename T>
__global__ void pack_in_kernel(const double* __restrict__ c, T* __restrict__ out, int64_t n, int R,
                               T* __restrict__ zero) {
  int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n * R) return;
  int64_t row = i / R;
  int r = int(i - row * R);
  out[i] = T(c[row + n * r]);
  if (zero) zero[i] = T(0);  // the sigma accumulator of the same shape, when given
}

template <typename T>
__global__ void unpack_out_kernel(const T* __restrict__ s, double* __restrict__ out, int64_t n, int R) {
  int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n * R) return;
  int64_t row = i % n;
  int r = int(i / n);
  out[i] = double(s[row * R + r]);
}

// ---- diagonal ------------------------------------------------------------------------------
struct DiagParams {
  const TermInfo* terms;
  const BlockInfo* blocks;
  const int32_t* blk_index;
  const int16_t* cfg;
  const int16_t* sec_fock;
  const int32_t* row_sector;
  int N;
  int nmax1;
};

__device__ __forceinline__ int block_of(const DiagParams& p, int c, int op, const int16_t* f) {
  return p.blk_index[dense_block_index(p.nmax1, c, op, f[2 * c], f[2 * c + 1], f[2 * c], f[2 * c + 1])];
}

// <cfg|term|cfg> in the order of _contract (src/tpsci_inner.jl:270-329)
__device__ double diag_element(const DiagParams& p, const TermInfo& tm, const double* __restrict__ op,
                               const double* __restrict__ ints, const int16_t* f, const int16_t* cf) {
  const double* g[4];
  int d[4];
  for (int o = 0; o < tm.nbody; ++o) {
    int c = tm.c[o];
    int bl = block_of(p, c, tm.op[o], f);
    if (bl < 0) return 0.0;
    BlockInfo bi = p.blocks[bl];
    g[o] = op + bi.off + int64_t(bi.nidx) * (cf[c] + int64_t(bi.mb) * cf[c]);
    d[o] = bi.nidx;
  }
  if (tm.nbody == 1) return g[0][0];
  const double* v = ints + tm.ints_off;
  double me = 0.0;
  if (tm.nbody == 2) {
    for (int j = 0; j < d[1]; ++j) {
      double acc = 0.0;
      for (int i = 0; i < d[0]; ++i) acc = fma(g[0][i], v[i + d[0] * j], acc);
      me = fma(acc, g[1][j], me);
    }
  } else if (tm.nbody == 3) {
    for (int kk = 0; kk < d[2]; ++kk) {
      double acck = 0.0;
      for (int j = 0; j < d[1]; ++j) {
        double acc = 0.0;
        const double* vj = v + d[0] * (j + d[1] * kk);
        for (int i = 0; i < d[0]; ++i) acc = fma(g[0][i], vj[i], acc);
        acck = fma(acc, g[1][j], acck);
      }
      me = fma(acck, g[2][kk], me);
    }
  } else {
    for (int l = 0; l < d[3]; ++l) {
      double accl = 0.0;
      for (int kk = 0; kk < d[2]; ++kk) {
        double acck = 0.0;
        for (int j = 0; j < d[1]; ++j) {
          double acc = 0.0;
          const double* vj = v + d[0] * (j + d[1] * (kk + d[2] * l));
          for (int i = 0; i < d[0]; ++i) acc = fma(g[0][i], vj[i], acc);
          acck = fma(acc, g[1][j], acck);
        }
        accl = fma(acck, g[2][kk], accl);
      }
      me = fma(accl, g[3][l], me);
    }
  }
  int s = 0;
  for (int o = 0; o < tm.nbody; ++o)
    if (tm.parity[o]) {
      int ne = 0;
      for (int ci = 0; ci < tm.c[o]; ++ci) ne += f[2 * ci] + f[2 * ci + 1];
      s ^= ne & 1;
    }
  return s ? -me : me;
}

__global__ void diag_terms_kernel(DiagParams p, const double* __restrict__ op, const double* __restrict__ ints,
                                  const int32_t* __restrict__ zero_terms, int n_zero, int64_t n,
                                  double* __restrict__ hd) {
  int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int16_t* f = p.sec_fock + int64_t(p.row_sector[i]) * 2 * p.N;
  double s = 0.0;
  for (int z = 0; z < n_zero; ++z) s += diag_element(p, p.terms[zero_terms[z]], op, ints, f, p.cfg + i * kCfgStride);
  hd[i] = s;
}

__global__ void diag_op_kernel(DiagParams p, const double* __restrict__ op, int opid, int64_t n,
                               double* __restrict__ hd, int* __restrict__ missing) {
  int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int16_t* f = p.sec_fock + int64_t(p.row_sector[i]) * 2 * p.N;
  double s = 0.0;
  for (int c = 0; c < p.N; ++c) {
    int bl = block_of(p, c, opid, f);
    if (bl < 0) {
      atomicExch(missing, 1);
      continue;
    }
    BlockInfo bi = p.blocks[bl];
    int st = p.cfg[i * kCfgStride + c];
    s += op[bi.off + st + int64_t(bi.mb) * st];
  }
  hd[i] = s;
}

}  // namespace

// ---------------------------------------------------------------------------------------
// host side

static LaneParams make_lane_params(fcg_ctx* ctx, int R) {
  LaneParams p{};
  p.jobs = ctx->d_jobs.p;
  p.chunk_lo = ctx->d_chunk_lo.p;
  p.chunk_val = ctx->d_chunk_val.p;
  p.n_chunks = ctx->n_chunks;
  p.perm = ctx->d_perm.p;
  p.ts = ctx->d_ts.p;
  p.cfg = ctx->d_cfg.p;
  p.R = R;
  return p;
}

// CTAs of a launch over n_chunks warp chunks
static int64_t lane_ctas(int64_t n_chunks) { return (n_chunks + kWarpsPerCta - 1) / kWarpsPerCta; }

static DiagParams make_diag_params(fcg_ctx* ctx) {
  DiagParams p{};
  p.terms = ctx->d_terms.p;
  p.blocks = ctx->d_blocks.p;
  p.blk_index = ctx->d_blk_index.p;
  p.cfg = ctx->d_cfg.p;
  p.sec_fock = ctx->d_sec_fock.p;
  p.row_sector = ctx->d_row_sector.p;
  p.N = ctx->N;
  p.nmax1 = ctx->nmax + 1;
  return p;
}

extern "C" {

int fcg_version(void) { return 2; }

int fcg_ctx_create(int device, fcg_ctx** out) {
  if (!out) return FCG_EINVAL;
  *out = nullptr;
  fcg_ctx* ctx = new fcg_ctx();
  ctx->device = device;
  cudaError_t e = cudaSetDevice(device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->own_stream, cudaStreamNonBlocking);
  ctx->stream = ctx->own_stream;
  if (e == cudaSuccess) e = cudaEventCreate(&ctx->ev0);
  if (e == cudaSuccess) e = cudaEventCreate(&ctx->ev1);
  if (e == cudaSuccess) e = cudaEventCreate(&ctx->ev2);
  if (e == cudaSuccess) e = cudaEventCreate(&ctx->ev3);
  if (e != cudaSuccess) {
    delete ctx;
    return FCG_ECUDA;
  }
  *out = ctx;
  return FCG_OK;
}

int fcg_ctx_destroy(fcg_ctx* ctx) {
  if (!ctx) return FCG_OK;
  cudaSetDevice(ctx->device);
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  if (ctx->ev0) cudaEventDestroy(ctx->ev0);
  if (ctx->ev1) cudaEventDestroy(ctx->ev1);
  if (ctx->ev2) cudaEventDestroy(ctx->ev2);
  if (ctx->ev3) cudaEventDestroy(ctx->ev3);
  if (ctx->ev_fork) cudaEventDestroy(ctx->ev_fork);
  if (ctx->ev_join) cudaEventDestroy(ctx->ev_join);
  if (ctx->aux_stream) cudaStreamDestroy(ctx->aux_stream);
  if (ctx->own_stream) cudaStreamDestroy(ctx->own_stream);
  delete ctx;
  return FCG_OK;
}

const char* fcg_last_error(const fcg_ctx* ctx) { return ctx ? ctx->err.c_str() : "null context"; }

int fcg_set_stream(fcg_ctx* ctx, void* stream) {
  if (!ctx) return FCG_EINVAL;
  FCG_CUDA(cudaSetDevice(ctx->device));
  FCG_CUDA(cudaStreamSynchronize(ctx->stream));
  ctx->stream = stream ? static_cast<cudaStream_t>(stream) : ctx->own_stream;
  return FCG_OK;
}

int fcg_set_ops(fcg_ctx* ctx, int n_clusters, const int32_t* cluster_norb, int64_t n_blocks,
                const int64_t* block_table, int64_t n_data, const double* data) {
  if (!ctx) return FCG_EINVAL;
  FCG_REQUIRE(n_clusters > 0 && n_clusters <= kMaxClusters, FCG_ELIMIT, "n_clusters must be in [1, 8]");
  FCG_REQUIRE(cluster_norb && block_table && (data || n_data == 0) && n_blocks >= 0, FCG_EINVAL, "null pointer");
  FCG_REQUIRE(n_blocks < (int64_t(1) << 31), FCG_ELIMIT, "at most 2^31 - 1 TDM blocks");
  FCG_CUDA(cudaSetDevice(ctx->device));
  ctx->N = n_clusters;
  ctx->norb.assign(cluster_norb, cluster_norb + n_clusters);
  ctx->nmax = 0;
  for (int n : ctx->norb) {
    FCG_REQUIRE(n > 0 && n <= 15, FCG_ELIMIT, "orbitals per cluster must be in [1, 15]");
    ctx->nmax = std::max(ctx->nmax, n);
  }
  ctx->opb.assign(block_table, block_table + n_blocks * kOpbCols);
  const int s = ctx->nmax + 1;
  ctx->h_blk_index.assign(size_t(n_clusters) * kNumOps * s * s * s * s, -1);
  ctx->h_blocks.assign(n_blocks, BlockInfo{});
  for (int64_t b = 0; b < n_blocks; ++b) {
    const int64_t* r = &ctx->opb[b * kOpbCols];
    FCG_REQUIRE(r[0] >= 0 && r[0] < n_clusters && r[1] >= 0 && r[1] < kNumOps, FCG_EINVAL,
                "block table: bad cluster or op id");
    for (int i = 2; i < 6; ++i)
      FCG_REQUIRE(r[i] >= 0 && r[i] <= ctx->norb[r[0]], FCG_EINVAL, "block table: bad Fock sector");
    FCG_REQUIRE(r[6] > 0 && r[7] > 0 && r[8] > 0 && r[6] <= 4096 && r[7] <= 256 && r[8] <= 256, FCG_ELIMIT,
                "block table: block dims out of range");
    FCG_REQUIRE(r[9] >= 0 && r[9] + r[6] * r[7] * r[8] <= n_data, FCG_EINVAL, "block table: data out of range");
    int64_t i = dense_block_index(s, int(r[0]), int(r[1]), int(r[2]), int(r[3]), int(r[4]), int(r[5]));
    ctx->h_blk_index[i] = int32_t(b);
  }
  // device copy: every block starts on a multiple of kAlign elements (32-byte vector loads
  // of TDM columns whose length is a multiple of 4)
  int64_t cursor = 0;
  for (int64_t b = 0; b < n_blocks; ++b) {
    const int64_t* r = &ctx->opb[b * kOpbCols];
    cursor = (cursor + kAlign - 1) / kAlign * kAlign;
    ctx->h_blocks[b] = BlockInfo{cursor, int32_t(r[6]), int32_t(r[7]), int32_t(r[8]), 0};
    cursor += r[6] * r[7] * r[8];
  }
  // the caller's blob goes up once; a kernel places every block at its aligned offset and
  // writes the float copy (the gaps between blocks are zero)
  {
    const size_t total = size_t(std::max<int64_t>(cursor, 1));
    FCG_CUDA(ctx->d_op64.alloc(total));
    FCG_CUDA(ctx->d_op32.alloc(total));
    FCG_CUDA(cudaMemsetAsync(ctx->d_op64.p, 0, sizeof(double) * total, ctx->stream));
    FCG_CUDA(cudaMemsetAsync(ctx->d_op32.p, 0, sizeof(float) * total, ctx->stream));
    if (n_blocks > 0) {
      std::vector<PlaceJob> pj(n_blocks);
      for (int64_t b = 0; b < n_blocks; ++b) {
        const int64_t* r = &ctx->opb[b * kOpbCols];
        pj[b] = PlaceJob{r[9], ctx->h_blocks[b].off, r[6] * r[7] * r[8]};
      }
      FCG_CUDA(ctx->d_op_raw.upload(data, size_t(n_data), ctx->stream));
      PlaceJob* d_pj = nullptr;
      FCG_CUDA(fcg_ctx::stage(ctx->scratch_b, pj.data(), pj.size(), ctx->stream, &d_pj));
      place_blocks_kernel<<<unsigned(n_blocks), 256, 0, ctx->stream>>>(d_pj, ctx->d_op_raw.p, ctx->d_op64.p,
                                                                        ctx->d_op32.p);
      FCG_CUDA(cudaGetLastError());
    }
  }
  FCG_CUDA(ctx->d_blocks.upload(ctx->h_blocks.data(), ctx->h_blocks.size(), ctx->stream));
  FCG_CUDA(ctx->d_blk_index.upload(ctx->h_blk_index.data(), ctx->h_blk_index.size(), ctx->stream));
  FCG_CUDA(ctx->d_norb.upload(ctx->norb.data(), ctx->norb.size(), ctx->stream));
  {
    std::vector<MaxJob> mj(n_blocks);
    ctx->gmax_off.assign(n_blocks, 0);
    int64_t tot = 0;
    for (int64_t b = 0; b < n_blocks; ++b) {
      const BlockInfo& B = ctx->h_blocks[b];
      mj[b] = MaxJob{B.off, tot, B.nidx, B.mb, B.mk, 0};
      ctx->gmax_off[b] = tot;
      tot += int64_t(B.nidx) * B.mk;
    }
    MaxJob* d_mj = nullptr;
    FCG_CUDA(fcg_ctx::stage(ctx->scratch_a, mj.data(), mj.size(), ctx->stream, &d_mj));
    FCG_CUDA(ctx->d_gmax.alloc(std::max<int64_t>(tot, 1)));
    if (n_blocks > 0) {
      colmax_kernel<<<unsigned(n_blocks), 128, 0, ctx->stream>>>(d_mj, ctx->d_op64.p, ctx->d_gmax.p);
      FCG_CUDA(cudaGetLastError());
    }
    FCG_CUDA(cudaStreamSynchronize(ctx->stream));
  }
  ctx->have_ops = true;
  ctx->have_terms = false;
  ctx->dj.ready = false;
  ctx->have_state = false;
  ctx->have_bst = false;
  ctx->drop_hcache();
  return FCG_OK;
}

}  // extern "C"

// The dressed operators W of every term (and their column maxima for the open-sigma
// screen) on the device, from the job list of fcg_set_terms; once per term set.
int ensure_dressed(fcg_ctx* ctx) {
  if (ctx->dressed) return FCG_OK;
  const std::vector<DressJob>& jobs = ctx->dress_jobs;
  const int64_t w_total = ctx->n_w;
  DressJob* d_jobs = nullptr;
  FCG_CUDA(fcg_ctx::stage(ctx->scratch_a, jobs.data(), jobs.size(), ctx->stream, &d_jobs));
  FCG_CUDA(ctx->d_w64.alloc(std::max<int64_t>(w_total, 1)));
  FCG_CUDA(ctx->d_w32.alloc(std::max<int64_t>(w_total, 1)));
  if (!jobs.empty()) {
    dress_kernel<<<unsigned(jobs.size()), 256, 0, ctx->stream>>>(d_jobs, ctx->d_op64.p, ctx->d_ints64.p,
                                                                 ctx->d_w64.p);
    FCG_CUDA(cudaGetLastError());
    to_float_kernel<<<1024, 256, 0, ctx->stream>>>(ctx->d_w64.p, ctx->d_w32.p, w_total);
    FCG_CUDA(cudaGetLastError());
  }
  FCG_CUDA(cudaStreamSynchronize(ctx->stream));  // the job list's staging buffer is reused by the next call
  ctx->wmax_built = false;
  ctx->dressed = true;
  return FCG_OK;
}

// Column maxima of the dressed operators for the open sigma's screen: Wmax[rest, k] per W
// block, indexed like w_index; built on the first open sigma after the dressing.
int ensure_wmax(fcg_ctx* ctx) {
  {
    const int rc = ensure_dressed(ctx);
    if (rc) return rc;
  }
  if (ctx->wmax_built) return FCG_OK;
  const std::vector<DressJob>& jobs = ctx->dress_jobs;
  std::vector<MaxJob> mj(jobs.size());
  ctx->wmax_index.assign(ctx->w_index.size(), -1);
  int64_t tot = 0;
  for (size_t j = 0; j < jobs.size(); ++j) {
    const DressJob& J = jobs[j];
    mj[j] = MaxJob{J.w_off, tot, J.rest_len, J.mb, J.mk, 0};
    tot += int64_t(J.rest_len) * J.mk;
  }
  for (size_t i = 0; i < ctx->w_index.size(); ++i) {
    if (ctx->w_index[i] < 0) continue;
    // jobs are in w_off order; find the job of this W block
    auto it = std::lower_bound(jobs.begin(), jobs.end(), ctx->w_index[i],
                               [](const DressJob& J, int64_t v) { return J.w_off < v; });
    ctx->wmax_index[i] = mj[it - jobs.begin()].out_off;
  }
  MaxJob* d_mj = nullptr;
  FCG_CUDA(fcg_ctx::stage(ctx->scratch_b, mj.data(), mj.size(), ctx->stream, &d_mj));
  FCG_CUDA(ctx->d_wmax.alloc(std::max<int64_t>(tot, 1)));
  if (!jobs.empty()) {
    colmax_kernel<<<unsigned(jobs.size()), 128, 0, ctx->stream>>>(d_mj, ctx->d_w64.p, ctx->d_wmax.p);
    FCG_CUDA(cudaGetLastError());
  }
  FCG_CUDA(cudaStreamSynchronize(ctx->stream));  // the job list's staging buffer is reused by the next call
  ctx->wmax_built = true;
  return FCG_OK;
}

extern "C" {

int fcg_set_terms(fcg_ctx* ctx, int n_terms, const int32_t* term_table, int64_t n_ints, const double* ints,
                  int n_transfers, const int16_t* transfers) {
  if (!ctx) return FCG_EINVAL;
  FCG_REQUIRE(ctx->have_ops, FCG_ESTATE, "fcg_set_ops must come first");
  FCG_REQUIRE(term_table && transfers && (ints || n_ints == 0) && n_terms >= 0 && n_transfers > 0, FCG_EINVAL,
              "bad term arguments");
  FCG_CUDA(cudaSetDevice(ctx->device));
  ctx->have_terms = false;
  ctx->have_state = false;
  ctx->have_bst = false;
  ctx->drop_hcache();
  ctx->n_terms = n_terms;
  ctx->trm.assign(term_table, term_table + int64_t(n_terms) * kTrmCols);
  ctx->n_trans = n_transfers;
  ctx->trans.assign(transfers, transfers + int64_t(n_transfers) * ctx->N * 2);
  ctx->terms.assign(n_terms, TermInfo{});
  for (int t = 0; t < n_terms; ++t) {
    const int32_t* r = &ctx->trm[int64_t(t) * kTrmCols];
    TermInfo& tm = ctx->terms[t];
    FCG_REQUIRE(r[0] >= 1 && r[0] <= 4, FCG_EINVAL, "term nbody must be in [1, 4]");
    FCG_REQUIRE(r[1] >= 0 && r[1] < n_transfers, FCG_EINVAL, "term transfer id out of range");
    tm.nbody = int8_t(r[0]);
    int64_t len = 1;
    for (int o = 0; o < 4; ++o) {
      tm.c[o] = int8_t(o < r[0] ? r[2 + o] : 0);
      tm.op[o] = int8_t(o < r[0] ? r[6 + o] : 0);
      tm.parity[o] = int8_t(o < r[0] ? r[18 + o] : 0);
      tm.dim[o] = int16_t(r[22 + o]);
      if (o < r[0]) {
        FCG_REQUIRE(r[2 + o] >= 0 && r[2 + o] < ctx->N, FCG_EINVAL, "term cluster out of range");
        FCG_REQUIRE(r[6 + o] >= 0 && r[6 + o] < kNumOps, FCG_EINVAL, "term op id out of range");
        FCG_REQUIRE(o == 0 || r[2 + o] > r[1 + o], FCG_EINVAL, "term clusters must increase");
        FCG_REQUIRE(r[22 + o] >= 1 && r[22 + o] <= 4096, FCG_EINVAL, "term dims out of range");
      }
      len *= r[22 + o];
    }
    tm.ints_off = int64_t(uint32_t(r[26])) | (int64_t(r[27]) << 32);
    if (r[0] > 1) FCG_REQUIRE(tm.ints_off >= 0 && tm.ints_off + len <= n_ints, FCG_EINVAL, "term ints out of range");
  }
  ctx->n_ints = n_ints;
  ctx->term_ints_norm.clear();  // computed when first needed (term_norms)
  std::vector<DressJob> jobs;
  int64_t w_total = 0;
  {
    std::string msg = build_dress(ctx->N, ctx->norb, ctx->nmax, ctx->trm, n_terms, ctx->h_blk_index, ctx->h_blocks,
                                  ctx->terms, ctx->dress, ctx->w_index, jobs, w_total);
    FCG_REQUIRE(msg.empty(), FCG_EINVAL, msg);
  }
  ctx->n_w = w_total;
  FCG_CUDA(ctx->d_terms.upload(ctx->terms.data(), ctx->terms.size(), ctx->stream));
  FCG_CUDA(ctx->d_ints64.upload(ints, n_ints, ctx->stream));
  FCG_CUDA(ctx->d_ints32.alloc(size_t(std::max<int64_t>(n_ints, 1))));
  if (n_ints > 0) {
    to_float_kernel<<<unsigned(std::min<int64_t>((n_ints + 255) / 256, 65535)), 256, 0, ctx->stream>>>(
        ctx->d_ints64.p, ctx->d_ints32.p, n_ints);
    FCG_CUDA(cudaGetLastError());
  }
  // the dressed operators themselves are built on the device by the first fcg_state_set
  // (only the closed and open sigmas use them; a BST-only context never needs them)
  ctx->dress_jobs.swap(jobs);
  ctx->dressed = false;
  ctx->dj.ready = false;
  FCG_CUDA(cudaStreamSynchronize(ctx->stream));
  ctx->have_terms = true;
  return FCG_OK;
}

}  // extern "C"

// Frobenius norm of every term's integrals (0 for 1-body terms), from the device copy of the
// integrals, on first use after fcg_set_terms.
int term_norms(fcg_ctx* ctx) {
  if (int64_t(ctx->term_ints_norm.size()) == ctx->n_terms) return FCG_OK;
  std::vector<double> ints(size_t(std::max<int64_t>(ctx->n_ints, 1)));
  if (ctx->n_ints > 0) {
    FCG_CUDA(cudaMemcpyAsync(ints.data(), ctx->d_ints64.p, sizeof(double) * size_t(ctx->n_ints),
                             cudaMemcpyDeviceToHost, ctx->stream));
    FCG_CUDA(cudaStreamSynchronize(ctx->stream));
  }
  std::vector<double> norm(size_t(ctx->n_terms), 0.0);
  for (int t = 0; t < ctx->n_terms; ++t) {
    const int32_t* r = &ctx->trm[int64_t(t) * kTrmCols];
    if (r[0] < 2) continue;
    int64_t len = 1;
    for (int o = 0; o < r[0]; ++o) len *= r[22 + o];
    double s2 = 0.0;
    const double* v = ints.data() + ctx->terms[t].ints_off;
    for (int64_t i = 0; i < len; ++i) s2 += v[i] * v[i];
    norm[size_t(t)] = std::sqrt(s2);
  }
  ctx->term_ints_norm.swap(norm);
  return FCG_OK;
}

ProblemInfo problem_info(fcg_ctx* ctx) {
  ProblemInfo pi;
  pi.N = ctx->N;
  pi.norb = ctx->norb;
  pi.nmax = ctx->nmax;
  pi.trm = &ctx->trm;
  pi.n_terms = ctx->n_terms;
  pi.trans = &ctx->trans;
  pi.n_trans = ctx->n_trans;
  pi.blk_index = &ctx->h_blk_index;
  pi.blocks = &ctx->h_blocks;
  pi.dress = &ctx->dress;
  pi.w_index = &ctx->w_index;
  return pi;
}

// The rows of a state and its Fock sectors (checked), on the device; the closed-sigma plan
// comes later (ensure_plan).
static int state_rows_impl(fcg_ctx* ctx, int64_t n_cfg, const int16_t* fock, const int16_t* cfg) {
  FCG_REQUIRE(ctx->have_ops && ctx->have_terms, FCG_ESTATE, "upload ops and terms first");
  FCG_REQUIRE(n_cfg > 0 && fock && cfg, FCG_EINVAL, "empty state");
  FCG_CUDA(cudaSetDevice(ctx->device));
  const auto t0 = std::chrono::steady_clock::now();
  ctx->have_state = false;
  ctx->have_plan = false;
  ctx->drop_hcache();
  if (ctx->plan_on_device) {
    const int rc = state_rows_device(ctx, n_cfg, fock, cfg);
    if (rc) return rc;
    ctx->h_fock.clear();  // the host planner fetches the rows from the device when it runs
    ctx->h_cfg.clear();
  } else {
    const ProblemInfo pi = problem_info(ctx);
    std::string msg = build_sectors(pi, n_cfg, fock, cfg, ctx->plan);
    FCG_REQUIRE(msg.empty(), FCG_EINVAL, msg);
    const Plan& P = ctx->plan;
    std::vector<int32_t> row_sector(n_cfg);
    for (size_t sct = 0; sct < P.sec_start.size(); ++sct)
      for (int64_t i = 0; i < P.sec_count[sct]; ++i) row_sector[P.sec_start[sct] + i] = int32_t(sct);
    ctx->h_fock.assign(fock, fock + n_cfg * 2 * ctx->N);
    ctx->h_cfg.assign(cfg, cfg + n_cfg * ctx->N);
    std::vector<int16_t> cfg8(size_t(n_cfg) * kCfgStride, 0);
    for (int64_t i = 0; i < n_cfg; ++i)
      for (int c = 0; c < ctx->N; ++c) cfg8[i * kCfgStride + c] = cfg[i * ctx->N + c];
    FCG_CUDA(ctx->d_cfg.upload(cfg8.data(), cfg8.size(), ctx->stream));
    FCG_CUDA(ctx->d_sec_fock.upload(P.sec_fock.data(), P.sec_fock.size(), ctx->stream));
    FCG_CUDA(ctx->d_row_sector.upload(row_sector.data(), row_sector.size(), ctx->stream));
    ctx->dj.table_ready = false;
  }
  const Plan& P = ctx->plan;
  ctx->n_cfg = n_cfg;
  FCG_CUDA(ctx->d_zero_terms.upload(P.zero_terms.data(), P.zero_terms.size(), ctx->stream));
  FCG_CUDA(cudaStreamSynchronize(ctx->stream));
  ctx->stats.n_cfg = n_cfg;
  ctx->stats.n_work_items = ctx->stats.n_triples = 0;  // until the plan is built
  ctx->stats.flops_reference = ctx->stats.flops_executed = 0;
  ctx->stats.n_sectors = int64_t(P.sec_start.size());
  ctx->stats.plan_seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  ctx->tuned[0] = ctx->tuned[1] = -1;  // a new shape: tune again (or find it in the shape cache)
  ctx->fine_built = false;
  ctx->have_state = true;
  return FCG_OK;
}

// The closed-sigma plan of the state (work items, lane jobs, warp chunks) and the dressed
// operators, built on first use.
int ensure_plan(fcg_ctx* ctx) {
  FCG_REQUIRE(ctx->have_state, FCG_ESTATE, "fcg_state_set must come first");
  if (ctx->have_plan) return FCG_OK;
  {
    const int rc = ensure_dressed(ctx);
    if (rc) return rc;
  }
  const auto t0 = std::chrono::steady_clock::now();
  if (ctx->plan_on_device) {
    const int rc = build_join_device(ctx);
    if (rc) return rc;
  } else {
    if (ctx->h_fock.empty()) {  // rows checked on the device: fetch them
      ctx->h_fock.resize(size_t(ctx->n_cfg) * 2 * ctx->N);
      ctx->h_cfg.resize(size_t(ctx->n_cfg) * ctx->N);
      FCG_CUDA(cudaMemcpyAsync(ctx->h_fock.data(), ctx->dj.d_fock_in.p, sizeof(int16_t) * ctx->h_fock.size(),
                               cudaMemcpyDeviceToHost, ctx->stream));
      FCG_CUDA(cudaMemcpyAsync(ctx->h_cfg.data(), ctx->dj.d_cfg_in.p, sizeof(int16_t) * ctx->h_cfg.size(),
                               cudaMemcpyDeviceToHost, ctx->stream));
      FCG_CUDA(cudaStreamSynchronize(ctx->stream));
    }
    const ProblemInfo pi = problem_info(ctx);
    std::string msg = build_join(pi, ctx->h_fock.data(), ctx->h_cfg.data(), ctx->plan);
    FCG_REQUIRE(msg.empty(), FCG_EINVAL, msg);
    const Plan& P = ctx->plan;
    FCG_CUDA(ctx->d_jobs.upload(P.jobs.data(), P.jobs.size(), ctx->stream));
    FCG_CUDA(ctx->d_chunk_lo.upload(P.chunk_lo.data(), P.chunk_lo.size(), ctx->stream));
    FCG_CUDA(ctx->d_chunk_val.upload(P.chunk_val.data(), P.chunk_val.size(), ctx->stream));
    FCG_CUDA(ctx->d_perm.upload(P.perm_pool.data(), P.perm_pool.size(), ctx->stream));
    FCG_CUDA(ctx->d_ts.upload(P.ts_pool.data(), P.ts_pool.size(), ctx->stream));
    FCG_CUDA(cudaStreamSynchronize(ctx->stream));
    ctx->n_chunks = int64_t(P.chunk_lo.size()) - 1;
    ctx->plan_jobs = int64_t(P.jobs.size());
    ctx->plan_wt = int64_t(P.wt_cost.size());
    ctx->plan_total_cost = 0;
    for (int32_t c : P.wt_cost) ctx->plan_total_cost += c;
    ctx->plan_items = int64_t(P.items.size());
    ctx->plan_ts = int64_t(P.ts_pool.size());
    ctx->plan_perm = int64_t(P.perm_pool.size());
  }
  FCG_REQUIRE(lane_ctas(ctx->n_chunks) < (int64_t(1) << 31), FCG_ELIMIT, "too many warp chunks for one launch");
  const Plan& P = ctx->plan;
  ctx->stats.n_work_items = ctx->plan_items;
  ctx->stats.n_triples = P.n_triples;
  ctx->stats.flops_reference = P.flops_ref;
  ctx->stats.flops_executed = P.flops_dressed;
  ctx->stats.dressed_elements = ctx->n_w;
  const double dt = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  ctx->stats.join_seconds = dt;
  ctx->stats.join_on_device = ctx->plan_on_device ? 1 : 0;
  ctx->stats.plan_seconds += dt;
  ctx->have_plan = true;
  return FCG_OK;
}

extern "C" {

int fcg_state_set(fcg_ctx* ctx, int64_t n_cfg, const int16_t* fock, const int16_t* cfg) {
  if (!ctx) return FCG_EINVAL;
  const int rc = state_rows_impl(ctx, n_cfg, fock, cfg);
  return rc ? rc : ensure_plan(ctx);
}

int fcg_state_rows(fcg_ctx* ctx, int64_t n_cfg, const int16_t* fock, const int16_t* cfg) {
  if (!ctx) return FCG_EINVAL;
  return state_rows_impl(ctx, n_cfg, fock, cfg);
}

int fcg_set_planner(fcg_ctx* ctx, int on_device) {
  if (!ctx) return FCG_EINVAL;
  FCG_REQUIRE(on_device == 0 || on_device == 1, FCG_EINVAL, "on_device must be 0 or 1");
  if (ctx->plan_on_device != (on_device == 1)) {
    ctx->plan_on_device = on_device == 1;
    ctx->have_plan = false;
    ctx->drop_hcache();
    ctx->fine_built = false;
  }
  return FCG_OK;
}

int fcg_plan_sizes(fcg_ctx* ctx, int64_t* sizes) {
  if (!ctx || !sizes) return FCG_EINVAL;
  const int rc = ensure_plan(ctx);
  if (rc) return rc;
  sizes[0] = ctx->plan_perm;
  sizes[1] = ctx->plan_ts;
  sizes[2] = ctx->plan_jobs;
  sizes[3] = ctx->n_chunks + 1;
  sizes[4] = ctx->plan_items;
  return FCG_OK;
}

int fcg_plan_copy(fcg_ctx* ctx, int which, void* dst, int64_t bytes) {
  if (!ctx || !dst) return FCG_EINVAL;
  const int rc = ensure_plan(ctx);
  if (rc) return rc;
  FCG_CUDA(cudaSetDevice(ctx->device));
  const void* src = nullptr;
  int64_t need = 0;
  switch (which) {
    case 0: src = ctx->d_perm.p; need = ctx->plan_perm * int64_t(sizeof(int32_t)); break;
    case 1: src = ctx->d_ts.p; need = ctx->plan_ts * int64_t(sizeof(TermSector)); break;
    case 2: src = ctx->d_jobs.p; need = ctx->plan_jobs * int64_t(sizeof(LaneJob)); break;
    case 3: src = ctx->d_chunk_lo.p; need = (ctx->n_chunks + 1) * int64_t(sizeof(int64_t)); break;
    case 4: src = ctx->d_chunk_val.p; need = (ctx->n_chunks + 1) * int64_t(sizeof(int64_t)); break;
    default: FCG_REQUIRE(false, FCG_EINVAL, "which must be 0..4");
  }
  FCG_REQUIRE(bytes == need, FCG_EINVAL, "bytes must be " + std::to_string(need));
  if (need > 0) FCG_CUDA(cudaMemcpyAsync(dst, src, size_t(need), cudaMemcpyDeviceToHost, ctx->stream));
  FCG_CUDA(cudaStreamSynchronize(ctx->stream));
  return FCG_OK;
}

int fcg_set_tuning(fcg_ctx* ctx, int mode) {
  if (!ctx) return FCG_EINVAL;
  FCG_REQUIRE(mode >= -1 && mode < kTuneCandidates, FCG_EINVAL, "tuning mode must be -1 (auto) or a candidate 0..3");
  ctx->tune_mode = mode;
  return FCG_OK;
}

int fcg_tuning(const fcg_ctx* ctx, int* chosen, float* candidate_ms) {
  if (!ctx || !chosen) return FCG_EINVAL;
  for (int prec = 0; prec < 2; ++prec) {
    chosen[prec] = ctx->tune_mode >= 0 ? ctx->tune_mode : ctx->tuned[prec];
    if (candidate_ms)
      for (int c = 0; c < kTuneCandidates; ++c) candidate_ms[prec * kTuneCandidates + c] = ctx->tune_ms[prec][c];
  }
  return FCG_OK;
}

}  // extern "C"

// ---- closed-sigma kernel tuning ---------------------------------------------------------
// Candidates per precision: the lane kernel compiled for two occupancy targets (float 4 or 3
// CTAs per SM, double 3 or 2) x two chunk granularities (about 4 or 16 waves of resident warps).
// Candidate c: occupancy variant c & 1, chunk table c >> 1.
template <typename T>
constexpr int tune_minb(int variant) {
  return sizeof(T) == 4 ? (variant ? 3 : 4) : (variant ? 2 : 3);
}

namespace {
std::mutex g_tune_mu;
std::map<std::string, int> g_tune_cache;  // shape key -> candidate, for this process

std::string tune_key(const fcg_ctx* ctx, int prec, int R) {
  const Plan& P = ctx->plan;
  return std::to_string(prec) + "/" + std::to_string(R) + "/" + std::to_string(ctx->N) + "/" +
         std::to_string(ctx->n_cfg) + "/" + std::to_string(ctx->n_terms) + "/" + std::to_string(P.n_triples) + "/" +
         std::to_string(ctx->plan_jobs) + "/" + std::to_string(ctx->device);
}
}  // namespace

// the finer chunk table of the tuning candidates (built on first use)
static int fine_chunks(fcg_ctx* ctx) {
  if (ctx->fine_built) return FCG_OK;
  if (ctx->plan_on_device) {
    int64_t nc = 0;
    const int rc = device_chunks(ctx, 4 * kTargetChunks, ctx->d_chunk_lo_fine, ctx->d_chunk_val_fine, &nc);
    if (rc) return rc;
    FCG_REQUIRE(lane_ctas(nc) < (int64_t(1) << 31), FCG_ELIMIT, "too many warp chunks for one launch");
    ctx->n_chunks_fine = nc;
    ctx->fine_built = true;
    return FCG_OK;
  }
  std::vector<int64_t> lo, val;
  make_chunks(ctx->plan, 4 * kTargetChunks, lo, val);
  FCG_REQUIRE(lane_ctas(int64_t(lo.size()) - 1) < (int64_t(1) << 31), FCG_ELIMIT, "too many warp chunks for one launch");
  FCG_CUDA(ctx->d_chunk_lo_fine.upload(lo.data(), lo.size(), ctx->stream));
  FCG_CUDA(ctx->d_chunk_val_fine.upload(val.data(), val.size(), ctx->stream));
  ctx->n_chunks_fine = int64_t(lo.size()) - 1;
  ctx->fine_built = true;
  return FCG_OK;
}

template <typename T, int MINB>
static void launch_lane(const LaneParams& p, int64_t grid, int R, const T* w, const T* op, const T* cin, T* sig,
                        cudaStream_t s) {
  switch (R) {
    case 1: closed_sigma_lane_kernel<T, 1, MINB><<<unsigned(grid), kSigmaThreads, 0, s>>>(p, w, op, cin, sig); break;
    case 2: closed_sigma_lane_kernel<T, 2, MINB><<<unsigned(grid), kSigmaThreads, 0, s>>>(p, w, op, cin, sig); break;
    case 4: closed_sigma_lane_kernel<T, 4, MINB><<<unsigned(grid), kSigmaThreads, 0, s>>>(p, w, op, cin, sig); break;
    default: closed_sigma_lane_kernel<T, 0, MINB><<<unsigned(grid), kSigmaThreads, 0, s>>>(p, w, op, cin, sig); break;
  }
}

// one direct closed sigma with candidate c
template <typename T>
static int launch_candidate(fcg_ctx* ctx, int c, int R, const T* w, const T* op, const T* cin, T* sig) {
  LaneParams p = make_lane_params(ctx, R);
  if (c >> 1) {
    const int rc = fine_chunks(ctx);
    if (rc) return rc;
    p.chunk_lo = ctx->d_chunk_lo_fine.p;
    p.chunk_val = ctx->d_chunk_val_fine.p;
    p.n_chunks = ctx->n_chunks_fine;
  }
  const int64_t grid = lane_ctas(p.n_chunks);
  if (grid == 0) return FCG_OK;
  if (c & 1)
    launch_lane<T, tune_minb<T>(1)>(p, grid, R, w, op, cin, sig, ctx->stream);
  else
    launch_lane<T, tune_minb<T>(0)>(p, grid, R, w, op, cin, sig, ctx->stream);
  FCG_CUDA(cudaGetLastError());
  return FCG_OK;
}

// Times every candidate once on this state (each run a complete sigma into sig), keeps the
// fastest for the context and for later states of the same shape in this process.
template <typename T>
static int tune_closed(fcg_ctx* ctx, int prec, int R, const T* w, const T* op, const T* cin, T* sig) {
  const auto t0 = std::chrono::steady_clock::now();
  const std::string key = tune_key(ctx, prec, R);
  {
    std::lock_guard<std::mutex> lock(g_tune_mu);
    auto it = g_tune_cache.find(key);
    if (it != g_tune_cache.end()) {
      ctx->tuned[prec] = it->second;
      ctx->stats.tune_cache_hits += 1;
      return FCG_OK;
    }
  }
  float best = 0.f;
  int best_c = 0;
  for (int c = 0; c < kTuneCandidates; ++c) {
    FCG_CUDA(cudaMemsetAsync(sig, 0, sizeof(T) * size_t(ctx->n_cfg) * R, ctx->stream));
    FCG_CUDA(cudaEventRecord(ctx->ev2, ctx->stream));
    const int rc = launch_candidate<T>(ctx, c, R, w, op, cin, sig);
    if (rc) return rc;
    FCG_CUDA(cudaEventRecord(ctx->ev3, ctx->stream));
    FCG_CUDA(cudaEventSynchronize(ctx->ev3));
    float ms = 0.f;
    FCG_CUDA(cudaEventElapsedTime(&ms, ctx->ev2, ctx->ev3));
    ctx->tune_ms[prec][c] = ms;
    if (c == 0 || ms < best) {
      best = ms;
      best_c = c;
    }
  }
  ctx->tuned[prec] = best_c;
  {
    std::lock_guard<std::mutex> lock(g_tune_mu);
    g_tune_cache[key] = best_c;
  }
  ctx->stats.tune_seconds += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  return FCG_OK;
}

template <typename T>
static int launch_closed(fcg_ctx* ctx, int R, const T* w, const T* op, const T* cin, T* sig, bool zero_sig = true,
                         bool timed = true) {
  const int prec = sizeof(T) == 4 ? 1 : 0;
  FCG_REQUIRE(ctx->have_plan, FCG_ESTATE, "the closed-sigma plan is missing (fcg_state_set builds it)");
  if (!ctx->have_hcache && ctx->tune_mode < 0 && ctx->tuned[prec] < 0 && timed) {
    const int rc = tune_closed<T>(ctx, prec, R, w, op, cin, sig);
    if (rc) return rc;
    zero_sig = true;  // the tuning runs left a sigma behind
  }
  const LaneParams p = make_lane_params(ctx, R);
  if (zero_sig) FCG_CUDA(cudaMemsetAsync(sig, 0, sizeof(T) * size_t(ctx->n_cfg) * R, ctx->stream));
  const int64_t grid = lane_ctas(p.n_chunks);
  int launches = 0;
  if (timed) FCG_CUDA(cudaEventRecord(ctx->ev0, ctx->stream));
  if (grid > 0 && ctx->have_hcache) {  // from the stored Hamiltonian blocks
    const T* hc = sizeof(T) == 4 ? reinterpret_cast<const T*>(ctx->d_hc32.p) : reinterpret_cast<const T*>(ctx->d_hc64.p);
    switch (R) {
      case 1: cached_sigma_lane_kernel<T, 1><<<unsigned(grid), kSigmaThreads, 0, ctx->stream>>>(p, hc, cin, sig); break;
      case 2: cached_sigma_lane_kernel<T, 2><<<unsigned(grid), kSigmaThreads, 0, ctx->stream>>>(p, hc, cin, sig); break;
      case 4: cached_sigma_lane_kernel<T, 4><<<unsigned(grid), kSigmaThreads, 0, ctx->stream>>>(p, hc, cin, sig); break;
      default: cached_sigma_lane_kernel<T, 0><<<unsigned(grid), kSigmaThreads, 0, ctx->stream>>>(p, hc, cin, sig); break;
    }
    FCG_CUDA(cudaGetLastError());
    launches = 1;
  } else if (grid > 0) {
    const int c = ctx->tune_mode >= 0 ? ctx->tune_mode : (ctx->tuned[prec] >= 0 ? ctx->tuned[prec] : 0);
    const int rc = launch_candidate<T>(ctx, c, R, w, op, cin, sig);
    if (rc) return rc;
    launches = 1;
  }
  if (timed) FCG_CUDA(cudaEventRecord(ctx->ev1, ctx->stream));
  ctx->stats.kernel_launches = launches;
  return FCG_OK;
}

static int sigma_device_impl(fcg_ctx* ctx, int R, const double* d_c, double* d_sigma, int precision,
                             bool wait = true) {
  FCG_REQUIRE(ctx->have_state, FCG_ESTATE, "fcg_state_set must come first");
  {
    const int rc = ensure_plan(ctx);
    if (rc) return rc;
  }
  FCG_REQUIRE(R >= 1 && R <= kMaxR, FCG_ELIMIT, "R must be in [1, 16]");
  FCG_REQUIRE(precision == FCG_FP64 || precision == FCG_FP32, FCG_EINVAL, "unknown precision");
  const int64_t n = ctx->n_cfg;
  const int64_t nR = n * R;
  const unsigned g = unsigned((nR + 255) / 256);
  ctx->stats.last_kernel_ms = 0.0;
  int rc;
  if (precision == FCG_FP64) {
    FCG_CUDA(ctx->d_c64.alloc(nR));
    FCG_CUDA(ctx->d_s64.alloc(nR));
    pack_in_kernel<double><<<g, 256, 0, ctx->stream>>>(d_c, ctx->d_c64.p, n, R, ctx->d_s64.p);
    rc = launch_closed<double>(ctx, R, ctx->d_w64.p, ctx->d_op64.p, ctx->d_c64.p, ctx->d_s64.p, false, wait);
    if (rc) return rc;
    unpack_out_kernel<double><<<g, 256, 0, ctx->stream>>>(ctx->d_s64.p, d_sigma, n, R);
  } else {
    FCG_CUDA(ctx->d_c32.alloc(nR));
    FCG_CUDA(ctx->d_s32.alloc(nR));
    pack_in_kernel<float><<<g, 256, 0, ctx->stream>>>(d_c, ctx->d_c32.p, n, R, ctx->d_s32.p);
    rc = launch_closed<float>(ctx, R, ctx->d_w32.p, ctx->d_op32.p, ctx->d_c32.p, ctx->d_s32.p, false, wait);
    if (rc) return rc;
    unpack_out_kernel<float><<<g, 256, 0, ctx->stream>>>(ctx->d_s32.p, d_sigma, n, R);
  }
  FCG_CUDA(cudaGetLastError());
  ctx->stats.kernel_launches += 2;
  if (!wait) return FCG_OK;  // untimed: no events were recorded
  FCG_CUDA(cudaStreamSynchronize(ctx->stream));
  float ms = 0.f;
  FCG_CUDA(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
  ctx->stats.last_kernel_ms = ms;
  return FCG_OK;
}

int sigma_closed_device_async(fcg_ctx* ctx, int R, const double* d_c, double* d_sigma, int precision) {
  return sigma_device_impl(ctx, R, d_c, d_sigma, precision, false);
}

extern "C" {

int fcg_sigma_closed_device(fcg_ctx* ctx, int R, const double* d_c, double* d_sigma, int precision) {
  if (!ctx) return FCG_EINVAL;
  FCG_REQUIRE(d_c && d_sigma, FCG_EINVAL, "null pointer");
  FCG_CUDA(cudaSetDevice(ctx->device));
  return sigma_device_impl(ctx, R, d_c, d_sigma, precision);
}

int fcg_cache_hamiltonian(fcg_ctx* ctx, double max_bytes, int64_t* bytes) {
  if (!ctx) return FCG_EINVAL;
  FCG_REQUIRE(ctx->have_state, FCG_ESTATE, "fcg_state_set must come first");
  FCG_CUDA(cudaSetDevice(ctx->device));
  if (max_bytes > 0) {
    const int rc = ensure_plan(ctx);
    if (rc) return rc;
  }
  const auto t0 = std::chrono::steady_clock::now();
  ctx->drop_hcache(!(max_bytes > 0));  // an explicit drop returns the memory
  ctx->stats.hcache_pairs = 0;
  ctx->stats.hcache_bytes = 0;
  ctx->stats.hcache_seconds = 0.0;
  if (bytes) *bytes = 0;
  if (!(max_bytes > 0)) return FCG_OK;  // 0: back to building every matrix element per sigma
  const Plan& P = ctx->plan;
  // one float64 and one float32 value per lane and task step (lanes without a pair hold 0)
  const int64_t pairs = P.task_values;
  const double need = double(pairs) * double(sizeof(double) + sizeof(float));
  if (bytes) *bytes = int64_t(need);
  FCG_REQUIRE(need <= max_bytes, FCG_ELIMIT,
              "stored Hamiltonian blocks need " + std::to_string(int64_t(need)) + " bytes, over max_bytes");
  FCG_CUDA(ctx->d_hc64.alloc(size_t(std::max<int64_t>(pairs, 1))));
  FCG_CUDA(ctx->d_hc32.alloc(size_t(std::max<int64_t>(pairs, 1))));
  if (pairs > 0) {
    const LaneParams p = make_lane_params(ctx, 1);
    hcache_lane_build_kernel<<<unsigned(lane_ctas(p.n_chunks)), kSigmaThreads, 0, ctx->stream>>>(
        p, ctx->d_w64.p, ctx->d_op64.p, ctx->d_hc64.p);
    FCG_CUDA(cudaGetLastError());
    to_float_kernel<<<unsigned(std::min<int64_t>((pairs + 255) / 256, 65535)), 256, 0, ctx->stream>>>(
        ctx->d_hc64.p, ctx->d_hc32.p, pairs);
    FCG_CUDA(cudaGetLastError());
  }
  FCG_CUDA(cudaStreamSynchronize(ctx->stream));
  ctx->hc_pairs = pairs;
  ctx->have_hcache = true;
  ctx->stats.hcache_pairs = pairs;
  ctx->stats.hcache_bytes = int64_t(need);
  ctx->stats.hcache_seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  return FCG_OK;
}

}  // extern "C"

// One grouped launch (plus one pack and one unpack launch) over the closed sigmas of several
// contexts on one device, on the first context's stream.
template <typename T>
static int grouped_impl(int n, fcg_ctx* const* ctxs, const int* R, const double* const* d_c,
                        double* const* d_sigma) {
  fcg_ctx* ctx = ctxs[0];
  std::vector<GroupEntry<T>> entries(n);
  std::vector<int32_t> cta_problem, cta_problem_hc;  // direct and stored-block grids
  int64_t cta = 0, cta_hc = 0, max_nr = 0;
  for (int q = 0; q < n; ++q) {
    fcg_ctx* c = ctxs[q];
    if (!c->have_plan) {
      const int rc = ensure_plan(c);
      if (rc) {
        ctx->err = c->err;
        return rc;
      }
    }
    const int64_t nr = c->n_cfg * R[q];
    GroupEntry<T>& e = entries[q];
    e.p = make_lane_params(c, R[q]);
    if (sizeof(T) == 4) {
      FCG_CUDA(c->d_c32.alloc(size_t(nr)));
      FCG_CUDA(c->d_s32.alloc(size_t(nr)));
      e.w = reinterpret_cast<const T*>(c->d_w32.p);
      e.op = reinterpret_cast<const T*>(c->d_op32.p);
      e.cin = reinterpret_cast<T*>(c->d_c32.p);
      e.sig = reinterpret_cast<T*>(c->d_s32.p);
    } else {
      FCG_CUDA(c->d_c64.alloc(size_t(nr)));
      FCG_CUDA(c->d_s64.alloc(size_t(nr)));
      e.w = reinterpret_cast<const T*>(c->d_w64.p);
      e.op = reinterpret_cast<const T*>(c->d_op64.p);
      e.cin = reinterpret_cast<T*>(c->d_c64.p);
      e.sig = reinterpret_cast<T*>(c->d_s64.p);
    }
    e.src = d_c[q];
    e.dst = d_sigma[q];
    e.n_cfg = c->n_cfg;
    e.hc = nullptr;
    const int64_t n_cta = lane_ctas(e.p.n_chunks);
    if (c->have_hcache) {
      e.hc = sizeof(T) == 4 ? reinterpret_cast<const T*>(c->d_hc32.p) : reinterpret_cast<const T*>(c->d_hc64.p);
      e.cta0 = cta_hc;
      FCG_REQUIRE(cta_hc + n_cta < (int64_t(1) << 31), FCG_ELIMIT, "too many CTAs for one grouped launch");
      cta_problem_hc.insert(cta_problem_hc.end(), size_t(n_cta), int32_t(q));
      cta_hc += n_cta;
    } else {
      e.cta0 = cta;
      FCG_REQUIRE(cta + n_cta < (int64_t(1) << 31), FCG_ELIMIT, "too many CTAs for one grouped launch");
      cta_problem.insert(cta_problem.end(), size_t(n_cta), int32_t(q));
      cta += n_cta;
    }
    max_nr = std::max(max_nr, nr);
  }
  FCG_CUDA(ctx->d_group.upload(reinterpret_cast<const unsigned char*>(entries.data()),
                               entries.size() * sizeof(GroupEntry<T>), ctx->stream));
  {
    std::vector<int32_t> both(cta_problem);
    both.insert(both.end(), cta_problem_hc.begin(), cta_problem_hc.end());
    FCG_CUDA(ctx->d_group_cta.upload(both.data(), both.size(), ctx->stream));
  }
  const GroupEntry<T>* dg = reinterpret_cast<const GroupEntry<T>*>(ctx->d_group.p);
  const dim3 pgrid = dim3(unsigned(std::min<int64_t>((max_nr + 255) / 256, 1024)), unsigned(n));
  grouped_pack_kernel<T><<<pgrid, 256, 0, ctx->stream>>>(dg);
  FCG_CUDA(cudaGetLastError());
  FCG_CUDA(cudaEventRecord(ctx->ev0, ctx->stream));
  if (cta > 0) {
    int rmax = 0;
    for (int q = 0; q < n; ++q) rmax = std::max(rmax, R[q]);
    if (rmax <= 4)
      closed_sigma_grouped_kernel<T, 4><<<unsigned(cta), kSigmaThreads, 0, ctx->stream>>>(dg, ctx->d_group_cta.p);
    else
      closed_sigma_grouped_kernel<T, kMaxR><<<unsigned(cta), kSigmaThreads, 0, ctx->stream>>>(dg, ctx->d_group_cta.p);
    FCG_CUDA(cudaGetLastError());
  }
  if (cta_hc > 0) {
    int rmax = 0;
    for (int q = 0; q < n; ++q) rmax = std::max(rmax, R[q]);
    const int32_t* tab = ctx->d_group_cta.p + cta;
    if (rmax <= 4)
      cached_sigma_grouped_kernel<T, 4><<<unsigned(cta_hc), kSigmaThreads, 0, ctx->stream>>>(dg, tab);
    else
      cached_sigma_grouped_kernel<T, kMaxR><<<unsigned(cta_hc), kSigmaThreads, 0, ctx->stream>>>(dg, tab);
    FCG_CUDA(cudaGetLastError());
  }
  FCG_CUDA(cudaEventRecord(ctx->ev1, ctx->stream));
  grouped_unpack_kernel<T><<<pgrid, 256, 0, ctx->stream>>>(dg);
  FCG_CUDA(cudaGetLastError());
  FCG_CUDA(cudaStreamSynchronize(ctx->stream));
  float ms = 0.f;
  FCG_CUDA(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
  ctx->stats.last_kernel_ms = ms;
  ctx->stats.kernel_launches = 2 + (cta > 0 ? 1 : 0) + (cta_hc > 0 ? 1 : 0);
  return FCG_OK;
}

extern "C" {

int fcg_sigma_closed_grouped(int n, fcg_ctx* const* ctxs, const int* R, const double* const* d_c,
                             double* const* d_sigma, int precision) {
  if (n < 1 || !ctxs || !ctxs[0]) return FCG_EINVAL;
  fcg_ctx* ctx = ctxs[0];
  FCG_REQUIRE(R && d_c && d_sigma, FCG_EINVAL, "null pointer");
  FCG_REQUIRE(n <= 65535, FCG_ELIMIT, "at most 65535 problems per grouped launch");
  FCG_REQUIRE(precision == FCG_FP64 || precision == FCG_FP32, FCG_EINVAL, "unknown precision");
  for (int q = 0; q < n; ++q) {
    FCG_REQUIRE(ctxs[q] && d_c[q] && d_sigma[q], FCG_EINVAL, "null context or buffer in the group");
    FCG_REQUIRE(ctxs[q]->device == ctx->device, FCG_EINVAL, "all contexts of a group must share a device");
    FCG_REQUIRE(ctxs[q]->have_state, FCG_ESTATE, "every context of the group needs fcg_state_set");
    FCG_REQUIRE(R[q] >= 1 && R[q] <= kMaxR, FCG_ELIMIT, "R must be in [1, 16]");
    for (int q2 = 0; q2 < q; ++q2)
      FCG_REQUIRE(ctxs[q2] != ctxs[q], FCG_EINVAL, "a context appears twice in the group");
  }
  FCG_CUDA(cudaSetDevice(ctx->device));
  return precision == FCG_FP64 ? grouped_impl<double>(n, ctxs, R, d_c, d_sigma)
                               : grouped_impl<float>(n, ctxs, R, d_c, d_sigma);
}

int fcg_sigma_closed(fcg_ctx* ctx, int R, const double* c, double* sigma, int precision) {
  if (!ctx) return FCG_EINVAL;
  FCG_REQUIRE(c && sigma, FCG_EINVAL, "null pointer");
  FCG_REQUIRE(ctx->have_state, FCG_ESTATE, "fcg_state_set must come first");
  FCG_REQUIRE(R >= 1 && R <= kMaxR, FCG_ELIMIT, "R must be in [1, 16]");
  FCG_CUDA(cudaSetDevice(ctx->device));
  const size_t nR = size_t(ctx->n_cfg) * R;
  FCG_CUDA(ctx->d_in64.alloc(nR));
  FCG_CUDA(ctx->d_out64.alloc(nR));
  FCG_CUDA(cudaMemcpyAsync(ctx->d_in64.p, c, nR * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
  int rc = sigma_device_impl(ctx, R, ctx->d_in64.p, ctx->d_out64.p, precision);
  if (rc) return rc;
  FCG_CUDA(cudaMemcpyAsync(sigma, ctx->d_out64.p, nR * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  FCG_CUDA(cudaStreamSynchronize(ctx->stream));
  return FCG_OK;
}

int fcg_expectation(fcg_ctx* ctx, int R, const double* c, double* e, int precision) {
  if (!ctx) return FCG_EINVAL;
  FCG_REQUIRE(c && e, FCG_EINVAL, "null pointer");
  FCG_REQUIRE(ctx->have_state, FCG_ESTATE, "fcg_state_set must come first");
  FCG_REQUIRE(R >= 1 && R <= kMaxR, FCG_ELIMIT, "R must be in [1, 16]");
  const int64_t n = ctx->n_cfg;
  std::vector<double> sig(size_t(n) * R);
  const int rc = fcg_sigma_closed(ctx, R, c, sig.data(), precision);
  if (rc) return rc;
  for (int r = 0; r < R; ++r) {
    double acc = 0.0;
    for (int64_t i = 0; i < n; ++i) acc += c[i + n * r] * sig[size_t(i) + size_t(n) * r];
    e[r] = acc;
  }
  return FCG_OK;
}

int fcg_build_full_h(fcg_ctx* ctx, double* H) {
  if (!ctx) return FCG_EINVAL;
  FCG_REQUIRE(H, FCG_EINVAL, "null pointer");
  FCG_REQUIRE(ctx->have_state, FCG_ESTATE, "fcg_state_set must come first");
  const int64_t n = ctx->n_cfg;
  FCG_REQUIRE(n <= 65536, FCG_ELIMIT, "fcg_build_full_h is for spaces of at most 65536 configurations");
  FCG_CUDA(cudaSetDevice(ctx->device));
  constexpr int kCols = 16;
  FCG_CUDA(ctx->d_in64.alloc(size_t(n) * kCols));
  FCG_CUDA(ctx->d_out64.alloc(size_t(n) * kCols));
  for (int64_t j0 = 0; j0 < n; j0 += kCols) {
    const int R = int(std::min<int64_t>(kCols, n - j0));
    // identity columns j0 .. j0+R-1 (column-major n x R)
    FCG_CUDA(cudaMemsetAsync(ctx->d_in64.p, 0, sizeof(double) * size_t(n) * R, ctx->stream));
    const double one = 1.0;
    for (int r = 0; r < R; ++r)
      FCG_CUDA(cudaMemcpyAsync(ctx->d_in64.p + (j0 + r) + n * r, &one, sizeof(double), cudaMemcpyHostToDevice,
                               ctx->stream));
    const int rc = sigma_device_impl(ctx, R, ctx->d_in64.p, ctx->d_out64.p, FCG_FP64);
    if (rc) return rc;
    FCG_CUDA(cudaMemcpyAsync(H + n * j0, ctx->d_out64.p, sizeof(double) * size_t(n) * R, cudaMemcpyDeviceToHost,
                             ctx->stream));
  }
  FCG_CUDA(cudaStreamSynchronize(ctx->stream));
  return FCG_OK;
}

int fcg_diagonal(fcg_ctx* ctx, int op_id, double* hd) {
  if (!ctx) return FCG_EINVAL;
  FCG_REQUIRE(ctx->have_state, FCG_ESTATE, "fcg_state_set must come first");
  FCG_REQUIRE(hd, FCG_EINVAL, "null pointer");
  FCG_REQUIRE(op_id < kNumOps, FCG_EINVAL, "op id out of range");
  FCG_CUDA(cudaSetDevice(ctx->device));
  const int64_t n = ctx->n_cfg;
  FCG_CUDA(ctx->d_hd.alloc(n));
  DiagParams p = make_diag_params(ctx);
  const unsigned g = unsigned((n + 127) / 128);
  if (op_id < 0) {
    diag_terms_kernel<<<g, 128, 0, ctx->stream>>>(p, ctx->d_op64.p, ctx->d_ints64.p, ctx->d_zero_terms.p,
                                                  int(ctx->plan.zero_terms.size()), n, ctx->d_hd.p);
    FCG_CUDA(cudaGetLastError());
  } else {
    DevBuf<int> missing;
    FCG_CUDA(missing.alloc(1));
    FCG_CUDA(cudaMemsetAsync(missing.p, 0, sizeof(int), ctx->stream));
    diag_op_kernel<<<g, 128, 0, ctx->stream>>>(p, ctx->d_op64.p, op_id, n, ctx->d_hd.p, missing.p);
    FCG_CUDA(cudaGetLastError());
    int miss = 0;
    FCG_CUDA(cudaMemcpyAsync(&miss, missing.p, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    FCG_CUDA(cudaStreamSynchronize(ctx->stream));
    FCG_REQUIRE(!miss, FCG_EINVAL, "a diagonal block of that op is missing for a sector of the state");
  }
  FCG_CUDA(cudaMemcpyAsync(hd, ctx->d_hd.p, n * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  FCG_CUDA(cudaStreamSynchronize(ctx->stream));
  return FCG_OK;
}

int fcg_get_stats(const fcg_ctx* ctx, fcg_stats* out) {
  if (!ctx || !out) return FCG_EINVAL;
  *out = ctx->stats;
  return FCG_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------------------
// Allocation-free closed sigma.
//
// The regular device entry point keeps its row-major working copies of C and sigma in
// context buffers that grow with cudaMalloc.  This variant takes them from a fixed
// file-scope device array instead, so the call itself allocates and frees nothing.
// The array is 2 x kNoAllocMaxElems float64 = 16 MiB and stays resident on every device
// that loads the library, until the process exits.  Every call on a device shares it:
// calls that overlap on the GPU (other streams, other contexts of the same device) race
// on it and must be serialised by the caller.
namespace {

constexpr int64_t kNoAllocMaxElems = int64_t(1) << 20;  // n_cfg * R of one call
constexpr int kNoAllocMaxDevices = 64;

static __device__ __align__(256) double g_noalloc_scratch[2 * kNoAllocMaxElems];

std::mutex g_noalloc_mu;
double* g_noalloc_ptr[kNoAllocMaxDevices] = {};

// Device address of the scratch array on the current device; resolved once per device
// (host code only sees a host-side stand-in under the array's name).
int noalloc_scratch(fcg_ctx* ctx, double** out) {
  FCG_REQUIRE(ctx->device >= 0 && ctx->device < kNoAllocMaxDevices, FCG_ELIMIT, "device ordinal too large");
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (!g_noalloc_ptr[ctx->device]) {
    void* p = nullptr;
    FCG_CUDA(cudaGetSymbolAddress(&p, g_noalloc_scratch));
    g_noalloc_ptr[ctx->device] = static_cast<double*>(p);
  }
  *out = g_noalloc_ptr[ctx->device];
  return FCG_OK;
}

}  // namespace

extern "C" int fcg_sigma_closed_noalloc(fcg_ctx* ctx, int R, const double* d_c, double* d_sigma, int precision) {
  if (!ctx) return FCG_EINVAL;
  FCG_REQUIRE(d_c && d_sigma, FCG_EINVAL, "null pointer");
  FCG_REQUIRE(ctx->have_state && ctx->have_plan, FCG_ESTATE,
              "fcg_state_set must come first (a state set by fcg_state_rows has no closed-sigma plan yet)");
  FCG_REQUIRE(R >= 1 && R <= kMaxR, FCG_ELIMIT, "R must be in [1, 16]");
  FCG_REQUIRE(precision == FCG_FP64 || precision == FCG_FP32, FCG_EINVAL, "unknown precision");
  FCG_REQUIRE(ctx->n_cfg * R <= kNoAllocMaxElems, FCG_ELIMIT,
              "fcg_sigma_closed_noalloc: n_cfg * R exceeds its fixed scratch of 1048576 elements");
  FCG_CUDA(cudaSetDevice(ctx->device));
  double* scratch = nullptr;
  int rc = noalloc_scratch(ctx, &scratch);
  if (rc) return rc;
  const int64_t n = ctx->n_cfg;
  const unsigned g = unsigned((n * R + 255) / 256);
  ctx->stats.last_kernel_ms = 0.0;
  if (precision == FCG_FP64) {
    double* cbuf = scratch;
    double* sbuf = scratch + kNoAllocMaxElems;
    pack_in_kernel<double><<<g, 256, 0, ctx->stream>>>(d_c, cbuf, n, R, nullptr);
    rc = launch_closed<double>(ctx, R, ctx->d_w64.p, ctx->d_op64.p, cbuf, sbuf);  // zeroes sbuf first
    if (rc) return rc;
    unpack_out_kernel<double><<<g, 256, 0, ctx->stream>>>(sbuf, d_sigma, n, R);
  } else {
    float* cbuf = reinterpret_cast<float*>(scratch);
    float* sbuf = reinterpret_cast<float*>(scratch + kNoAllocMaxElems);
    pack_in_kernel<float><<<g, 256, 0, ctx->stream>>>(d_c, cbuf, n, R, nullptr);
    rc = launch_closed<float>(ctx, R, ctx->d_w32.p, ctx->d_op32.p, cbuf, sbuf);
    if (rc) return rc;
    unpack_out_kernel<float><<<g, 256, 0, ctx->stream>>>(sbuf, d_sigma, n, R);
  }
  FCG_CUDA(cudaGetLastError());
  ctx->stats.kernel_launches += 2;
  FCG_CUDA(cudaStreamSynchronize(ctx->stream));
  float ms = 0.f;
  FCG_CUDA(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
  ctx->stats.last_kernel_ms = ms;
  return FCG_OK;
}

