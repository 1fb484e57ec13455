// Open (first-order interacting space) sigma on the GPU: open_matvec_thread
// (src/tpsci_matvec_thread.jl:11-885) behind fcg_sigma_open / fcg_sigma_open_fetch.
//
// For every ket row of the state and every term whose target sector passes the job
// filter (:26-56), every bra local-state tuple of the term's active clusters gets
//     x = sign * sum W[(rest), b_w, k_w] prod_c G_c[i_c, b_c, k_c]
// and contributes x * c_ket to sigma[bra config] when |x| > thresh / max_r |c_ket[r]|,
// the per-contribution test of _collect_significant_thread! (:830-885).
//
// Pipeline (one stream):
//   screen_kernel   one thread per (ket row, term) job: a rigorous max-norm bound
//                   sum_rest Wmax * prod Gmax skips jobs whose every contribution would
//                   fail the threshold (the role of upper_bound_thread, :897-1023; skipping
//                   changes no result), the survivors are compacted;
//   expand_jobs_kernel  persistent CTAs take the surviving (ket, term) jobs from a counter,
//                   stage the job's W block and TDM columns in shared memory, contract
//                   W with the first TDM once per job and evaluate every bra tuple from
//                   there (threshold per contribution, as the reference), then insert into
//                   an open-addressed table keyed by (bra sector, mixed-radix local-state
//                   index) with atomic accumulation of the R values;
//   compact_kernel  occupied slots -> (key, values).
// A table that overflows its probe limit sets a flag and the call is repeated with a
// table twice as large.
#include <cmath>
#include <cstring>
#include <unordered_map>
#include <unordered_set>

#include "fcg_ctx.cuh"

using namespace fcg;

namespace {

constexpr unsigned long long kEmpty = ~0ull;
constexpr int kMaxProbe = 1 << 16;
constexpr int kKeyIdxBits = 40;

// counters: [0] kept jobs, [1] elements of kept jobs, [2] table overflow, [3] output rows,
// [4] next job of the expand CTAs
struct OpenParams {
  const OpenTerm* ot;
  const OpenItem* items;
  const int64_t* prefix;  // job prefix over items
  int64_t n_items;
  int64_t n_jobs;
  const int16_t* cfg;
  const double* c;  // row-major [n_cfg][R]
  const int64_t* strides;  // [n_bra_sectors][N]
  int N;
  int R;
  double thresh;
};

__device__ __forceinline__ int64_t find_item(const int64_t* prefix, int64_t lo, int64_t hi, int64_t x) {
  while (lo < hi) {
    int64_t mid = (lo + hi + 1) >> 1;
    if (__ldg(prefix + mid) <= x)
      lo = mid;
    else
      hi = mid - 1;
  }
  return lo;
}

__device__ __forceinline__ double row_maxabs(const double* c, int R) {
  double m = 0.0;
  for (int r = 0; r < R; ++r) m = fmax(m, fabs(c[r]));
  return m;
}

// rigorous bound on max over bra tuples of |x| for one (ket, term) job
__device__ double job_bound(const OpenTerm& o, const double* __restrict__ wmax, const double* __restrict__ gmax,
                            const int16_t* ck) {
  const TermSector& ts = o.ts;
  const double* wm = wmax + o.wmax_off + int64_t(ts.rest_len) * ck[ts.cw];
  if (ts.nrem == 0) return wm[0];
  const double* g0 = gmax + o.gmax_off[0] + int64_t(ts.g_dim[0]) * ck[ts.cr[0]];
  const int d0 = ts.g_dim[0];
  double bnd = 0.0;
  if (ts.nrem == 1) {
    for (int i = 0; i < d0; ++i) bnd += wm[i] * g0[i];
    return bnd;
  }
  const double* g1 = gmax + o.gmax_off[1] + int64_t(ts.g_dim[1]) * ck[ts.cr[1]];
  const int d1 = ts.g_dim[1];
  if (ts.nrem == 2) {
    for (int j = 0; j < d1; ++j) {
      double a = 0.0;
      for (int i = 0; i < d0; ++i) a += wm[i + d0 * j] * g0[i];
      bnd += a * g1[j];
    }
    return bnd;
  }
  const double* g2 = gmax + o.gmax_off[2] + int64_t(ts.g_dim[2]) * ck[ts.cr[2]];
  const int d2 = ts.g_dim[2];
  for (int l = 0; l < d2; ++l) {
    double al = 0.0;
    for (int j = 0; j < d1; ++j) {
      double a = 0.0;
      for (int i = 0; i < d0; ++i) a += wm[i + d0 * (j + d1 * l)] * g0[i];
      al += a * g1[j];
    }
    bnd += al * g2[l];
  }
  return bnd;
}

__global__ void screen_kernel(OpenParams p, const double* __restrict__ wmax, const double* __restrict__ gmax,
                              int2* __restrict__ kept, unsigned long long* __restrict__ counters) {
  const int64_t j = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (j >= p.n_jobs) return;
  const int64_t it = find_item(p.prefix, 0, p.n_items - 1, j);
  const OpenItem I = p.items[it];
  const int64_t local = j - p.prefix[it];
  const int ti = int(local % I.nt);
  const int row = I.row0 + int(local / I.nt);
  const OpenTerm& o = p.ot[I.ot_off + ti];
  const double maxc = row_maxabs(p.c + int64_t(row) * p.R, p.R);
  if (!(maxc > 0.0)) return;
  const double bnd = job_bound(o, wmax, gmax, p.cfg + int64_t(row) * kCfgStride);
  // keep unless every |x| <= bnd < thresh / maxc (a 1e-9 margin covers the bound's rounding)
  if (!(bnd * (1.0 + 1e-9) > p.thresh / maxc)) return;
  const unsigned long long pos = atomicAdd(counters + 0, 1ull);
  kept[pos] = make_int2(row, I.ot_off + ti);
  atomicAdd(counters + 1, (unsigned long long)o.out_count);
}

__device__ __forceinline__ void table_add(unsigned long long* keys, double* vals, unsigned long long cap_mask,
                                          unsigned long long key, const double* add, int R,
                                          unsigned long long* overflow) {
  unsigned long long h = key * 0x9E3779B97F4A7C15ull;
  h ^= h >> 29;
  unsigned long long slot = h & cap_mask;
  for (int probe = 0; probe < kMaxProbe; ++probe) {
    unsigned long long cur = keys[slot];
    if (cur == kEmpty) {
      unsigned long long prev = atomicCAS(keys + slot, kEmpty, key);
      if (prev == kEmpty || prev == key) cur = key;
      else cur = prev;
    }
    if (cur == key) {
      for (int r = 0; r < R; ++r) atomicAdd(vals + slot * R + r, add[r]);
      return;
    }
    slot = (slot + 1) & cap_mask;
  }
  atomicExch(overflow, 1ull);
}

constexpr int kExpThreads = 256;
constexpr int kOpenMaxR = 16;  // roots of one open sigma at most (checked on the host)
constexpr int kExpSmemBytes = 96 * 1024;  // shared-memory budget of one expand CTA
// The float pre-filter keeps a contribution for the exact double evaluation unless
// |x32| + kFilterMargin * s32 <= thresh / max|c|, where s32 = sum of |products| of the same
// sum.  The float evaluation differs from the exact value by at most about
// (number of factors + summed terms) * 2^-24 * s (below 1e-5 s for every shape here), so
// the margin of 1e-4 s never drops a contribution the double evaluation would keep.
constexpr float kFilterMargin = 1e-4f;

// Shared-memory tiles of one job.  Doubles: the W block of the ket's dressed-cluster state
// for every bra state of that cluster [rest][mb0] and the TDM columns of the remaining
// clusters [d_r][mb_{r+1}] (for the exact evaluations).  Floats: the same tiles, and
// T1[pair + P*jl] = sum_i W[i + d0*jl, b0] G0[i, b1] with its absolute-value twin T1a
// (pair = b0 + mb0*b1, P = mb0*mb1, jl < rest/d0).
struct ExpandTiles {
  int w64, g64[3];           // offsets in doubles
  int w32, g32[3], t1, t1a;  // offsets in floats, after the doubles
  int bytes;
};

__host__ __device__ inline ExpandTiles expand_tiles(int nrem, int rest, const int16_t* g_dim, const int16_t* mb) {
  ExpandTiles t{};
  int d = 0;
  t.w64 = d;
  d += rest * mb[0];
  for (int r = 0; r < 3; ++r) {
    t.g64[r] = d;
    if (r < nrem) d += g_dim[r] * mb[r + 1];
  }
  d += d & 1;  // float part starts on an even double
  int f = 2 * d;
  t.w32 = f;
  f += rest * mb[0];
  for (int r = 0; r < 3; ++r) {
    t.g32[r] = f;
    if (r < nrem) f += g_dim[r] * mb[r + 1];
  }
  const int jlp = nrem >= 2 ? (rest / g_dim[0]) * mb[0] * mb[1] : 0;
  t.t1 = f;
  f += jlp;
  t.t1a = f;
  f += jlp;
  t.bytes = 4 * f;
  return t;
}

// The exact contribution of one bra tuple (columns already selected): the sums of the
// per-element formula, in its order, with its fused multiply-adds.
__device__ __forceinline__ double exact_x(int nrem, int d0, int d1, int d2, const double* wc, const double* g0,
                                          const double* g1, const double* g2) {
  if (nrem == 0) return wc[0];
  double x = 0.0;
  if (nrem == 1) {
    for (int i = 0; i < d0; ++i) x = fma(wc[i], g0[i], x);
  } else if (nrem == 2) {
    for (int jj = 0; jj < d1; ++jj) {
      double acc = 0.0;
      for (int i = 0; i < d0; ++i) acc = fma(wc[i + d0 * jj], g0[i], acc);
      x = fma(acc, g1[jj], x);
    }
  } else {
    for (int l = 0; l < d2; ++l) {
      double al = 0.0;
      for (int jj = 0; jj < d1; ++jj) {
        double acc = 0.0;
        for (int i = 0; i < d0; ++i) acc = fma(wc[i + d0 * (jj + d1 * l)], g0[i], acc);
        al = fma(acc, g1[jj], al);
      }
      x = fma(al, g2[l], x);
    }
  }
  return x;
}

// one contribution: threshold, bra key, accumulation of x * c_ket
__device__ __forceinline__ void expand_emit(const OpenParams& p, double x, double tc, const double* crow,
                                            unsigned long long keybase, int64_t idx, unsigned long long* keys,
                                            double* vals, unsigned long long cap_mask,
                                            unsigned long long* counters) {
  if (!(fabs(x) > tc)) return;
  double add[kOpenMaxR];
  for (int r = 0; r < p.R; ++r) add[r] = x * crow[r];
  table_add(keys, vals, cap_mask, keybase | (unsigned long long)idx, add, p.R, counters + 2);
}

// One (b0, b1, b2) unit of a four-cluster job: float sums over the third remaining cluster's
// index l < D2 for every b3, screened; survivors evaluated exactly.  D2 = 16 serves any
// d2 <= 16 with the run-time length `d2`.
template <int D2>
__device__ __forceinline__ void unit4(const OpenParams& p, const float* T1, const float* T1a, int P, int pr, int d1,
                                      const float* g1, const float* G2f, int mb3, float tcf, double tc,
                                      int d0, const double* wc, const double* g0d, const double* g1d,
                                      const double* G2d, const double* crow, unsigned long long keybase,
                                      int64_t idx3, int64_t sa3, unsigned long long* keys, double* vals,
                                      unsigned long long cap_mask, unsigned long long* counters, int d2 = D2) {
  float ul[D2], ua[D2];
#pragma unroll
  for (int l = 0; l < D2; ++l) {
    ul[l] = 0.f;
    ua[l] = 0.f;
    if (D2 != 16 || l < d2)
      for (int j = 0; j < d1; ++j) {
        ul[l] = fmaf(T1[pr + P * (j + d1 * l)], g1[j], ul[l]);
        ua[l] = fmaf(T1a[pr + P * (j + d1 * l)], fabsf(g1[j]), ua[l]);
      }
  }
  for (int b3 = 0; b3 < mb3; ++b3) {
    const float* g2 = G2f + d2 * b3;
    float x32 = 0.f, s32 = 0.f;
#pragma unroll
    for (int l = 0; l < D2; ++l)
      if (D2 != 16 || l < d2) {
        x32 = fmaf(ul[l], g2[l], x32);
        s32 = fmaf(ua[l], fabsf(g2[l]), s32);
      }
    if (fabsf(x32) + kFilterMargin * s32 > tcf) {
      const double x = exact_x(3, d0, d1, d2, wc, g0d, g1d, G2d + d2 * b3);
      expand_emit(p, x, tc, crow, keybase, idx3 + b3 * sa3, keys, vals, cap_mask, counters);
    }
  }
}

// Persistent CTAs take kept (ket, term) jobs from a counter.  Per job the W block and the
// TDM columns for all bra states are staged in shared memory (double and float copies) and,
// for three- and four-cluster terms, W is contracted with the first remaining cluster's
// TDM once in float (T1, with its absolute-value twin).  Every bra tuple is then screened
// in float (value and the sum of |products|); the tuples that can pass the threshold are
// evaluated exactly with the per-element double formula (exact_x) and thresholded as the
// reference does.  Jobs whose tiles exceed the shared-memory budget are evaluated per
// element, exactly, from global memory.
__global__ void __launch_bounds__(kExpThreads) expand_jobs_kernel(
    OpenParams p, const int2* __restrict__ kept, int64_t n_kept, const double* __restrict__ w,
    const double* __restrict__ op, unsigned long long* __restrict__ keys, double* __restrict__ vals,
    unsigned long long cap_mask, unsigned long long* __restrict__ counters, int smem_bytes) {
  extern __shared__ __align__(16) double xs[];
  float* xf = reinterpret_cast<float*>(xs);
  __shared__ unsigned long long s_job;
  __shared__ double s_cs[kOpenMaxR];
  for (;;) {
    if (threadIdx.x == 0) s_job = atomicAdd(counters + 4, 1ull);
    __syncthreads();
    const int64_t jn = int64_t(s_job);
    if (jn >= n_kept) break;  // uniform over the CTA
    const int2 job = kept[jn];
    const OpenTerm& o = p.ot[job.y];
    const TermSector& ts = o.ts;
    const int16_t* ck = p.cfg + int64_t(job.x) * kCfgStride;
    const double* c_ket = p.c + int64_t(job.x) * p.R;
    const double tc = p.thresh / row_maxabs(c_ket, p.R);
    const float tcf = float(tc * (1.0 - 1e-6));
    const int nrem = ts.nrem, rest = ts.rest_len;
    const int d0 = nrem >= 1 ? ts.g_dim[0] : 1, d1 = nrem >= 2 ? ts.g_dim[1] : 1, d2 = nrem >= 3 ? ts.g_dim[2] : 1;
    int mb[4] = {1, 1, 1, 1};
    int64_t sa[4] = {0, 0, 0, 0};
    // bra key of (b0, .., b3) = keybase | (base + sum_a b_a * st[c_a])
    const int64_t* st = p.strides + int64_t(o.bsec) * p.N;
    int64_t base = 0;
    for (int c = 0; c < p.N; ++c) base += int64_t(ck[c]) * st[c];
    for (int a = 0; a < o.n_act; ++a) {
      mb[a] = o.mb_act[a];
      sa[a] = st[o.c_act[a]];
      base -= int64_t(ck[o.c_act[a]]) * sa[a];
    }
    const unsigned long long keybase = (unsigned long long)(o.bsec) << kKeyIdxBits;
    const double sg = ts.sign < 0 ? -1.0 : 1.0;
    // the ket's coefficients times the term's sign (exact): a kept value x contributes
    // x * (sg * c) = (sg * x) * c to every root
    if (threadIdx.x < p.R) s_cs[threadIdx.x] = sg * c_ket[threadIdx.x];
    __syncthreads();
    const double* crow = s_cs;
    const double* wblk = w + ts.w_off + int64_t(rest) * ts.w_mb * ck[ts.cw];  // [rest][mb0] for the ket state
    const double* gblk[3] = {nullptr, nullptr, nullptr};
    for (int r = 0; r < nrem; ++r) gblk[r] = op + ts.g_off[r] + int64_t(ts.g_dim[r]) * ts.g_mb[r] * ck[ts.cr[r]];
    const ExpandTiles t = expand_tiles(nrem, rest, ts.g_dim, o.mb_act);
    if (t.bytes <= smem_bytes && d2 <= 16) {
      for (int i = threadIdx.x; i < rest * mb[0]; i += kExpThreads) {
        const double v = wblk[i];
        xs[t.w64 + i] = v;
        xf[t.w32 + i] = float(v);
      }
      for (int r = 0; r < nrem; ++r) {
        const int n = ts.g_dim[r] * mb[r + 1];
        for (int i = threadIdx.x; i < n; i += kExpThreads) {
          const double v = gblk[r][i];
          xs[t.g64[r] + i] = v;
          xf[t.g32[r] + i] = float(v);
        }
      }
      __syncthreads();
      const double* W = xs + t.w64;
      const float* Wf = xf + t.w32;
      const float* G0f = xf + t.g32[0];
      const int P = mb[0] * mb[1];
      if (nrem == 0) {
        for (int b0 = threadIdx.x; b0 < mb[0]; b0 += kExpThreads)
          expand_emit(p, W[b0], tc, crow, keybase, base + b0 * sa[0], keys, vals, cap_mask, counters);
      } else if (nrem == 1) {
        for (int pr = threadIdx.x; pr < P; pr += kExpThreads) {
          const int b1 = pr / mb[0], b0 = pr - b1 * mb[0];
          const float* wc = Wf + rest * b0;
          const float* g0 = G0f + d0 * b1;
          float x32 = 0.f, s32 = 0.f;
          for (int i = 0; i < d0; ++i) {
            x32 = fmaf(wc[i], g0[i], x32);
            s32 = fmaf(fabsf(wc[i]), fabsf(g0[i]), s32);
          }
          if (fabsf(x32) + kFilterMargin * s32 > tcf) {
            const double x = exact_x(1, d0, 1, 1, W + rest * b0, xs + t.g64[0] + d0 * b1, nullptr, nullptr);
            expand_emit(p, x, tc, crow, keybase, base + b0 * sa[0] + b1 * sa[1], keys, vals, cap_mask, counters);
          }
        }
      } else {
        const int JL = rest / d0;
        float* T1 = xf + t.t1;
        float* T1a = xf + t.t1a;
        for (int e = threadIdx.x; e < JL * P; e += kExpThreads) {
          const int jl = e / P, pr = e - jl * P;
          const int b1 = pr / mb[0], b0 = pr - b1 * mb[0];
          const float* wc = Wf + d0 * jl + rest * b0;
          const float* g0 = G0f + d0 * b1;
          float acc = 0.f, aa = 0.f;
          for (int i = 0; i < d0; ++i) {
            acc = fmaf(wc[i], g0[i], acc);
            aa = fmaf(fabsf(wc[i]), fabsf(g0[i]), aa);
          }
          T1[pr + P * jl] = acc;
          T1a[pr + P * jl] = aa;
        }
        __syncthreads();
        const float* G1f = xf + t.g32[1];
        const int units = P * mb[2];
        for (int u = threadIdx.x; u < units; u += kExpThreads) {
          const int b2 = u / P, pr = u - b2 * P;
          const int b1 = pr / mb[0], b0 = pr - b1 * mb[0];
          const int64_t idx3 = base + b0 * sa[0] + b1 * sa[1] + b2 * sa[2];
          const float* g1 = G1f + d1 * b2;
          const double* wc = W + rest * b0;
          const double* g0d = xs + t.g64[0] + d0 * b1;
          const double* g1d = xs + t.g64[1] + d1 * b2;
          if (nrem == 2) {
            float x32 = 0.f, s32 = 0.f;
            for (int j = 0; j < d1; ++j) {
              x32 = fmaf(T1[pr + P * j], g1[j], x32);
              s32 = fmaf(T1a[pr + P * j], fabsf(g1[j]), s32);
            }
            if (fabsf(x32) + kFilterMargin * s32 > tcf) {
              const double x = exact_x(2, d0, d1, 1, wc, g0d, g1d, nullptr);
              expand_emit(p, x, tc, crow, keybase, idx3, keys, vals, cap_mask, counters);
            }
          } else {
            switch (d2) {
              case 1: unit4<1>(p, T1, T1a, P, pr, d1, g1, xf + t.g32[2], mb[3], tcf, tc, d0, wc, g0d, g1d,
                               xs + t.g64[2], crow, keybase, idx3, sa[3], keys, vals, cap_mask, counters); break;
              case 2: unit4<2>(p, T1, T1a, P, pr, d1, g1, xf + t.g32[2], mb[3], tcf, tc, d0, wc, g0d, g1d,
                               xs + t.g64[2], crow, keybase, idx3, sa[3], keys, vals, cap_mask, counters); break;
              case 3: unit4<3>(p, T1, T1a, P, pr, d1, g1, xf + t.g32[2], mb[3], tcf, tc, d0, wc, g0d, g1d,
                               xs + t.g64[2], crow, keybase, idx3, sa[3], keys, vals, cap_mask, counters); break;
              case 4: unit4<4>(p, T1, T1a, P, pr, d1, g1, xf + t.g32[2], mb[3], tcf, tc, d0, wc, g0d, g1d,
                               xs + t.g64[2], crow, keybase, idx3, sa[3], keys, vals, cap_mask, counters); break;
              case 5: unit4<5>(p, T1, T1a, P, pr, d1, g1, xf + t.g32[2], mb[3], tcf, tc, d0, wc, g0d, g1d,
                               xs + t.g64[2], crow, keybase, idx3, sa[3], keys, vals, cap_mask, counters); break;
              case 6: unit4<6>(p, T1, T1a, P, pr, d1, g1, xf + t.g32[2], mb[3], tcf, tc, d0, wc, g0d, g1d,
                               xs + t.g64[2], crow, keybase, idx3, sa[3], keys, vals, cap_mask, counters); break;
              case 8: unit4<8>(p, T1, T1a, P, pr, d1, g1, xf + t.g32[2], mb[3], tcf, tc, d0, wc, g0d, g1d,
                               xs + t.g64[2], crow, keybase, idx3, sa[3], keys, vals, cap_mask, counters); break;
              default: unit4<16>(p, T1, T1a, P, pr, d1, g1, xf + t.g32[2], mb[3], tcf, tc, d0, wc, g0d, g1d,
                                 xs + t.g64[2], crow, keybase, idx3, sa[3], keys, vals, cap_mask, counters, d2); break;
            }
          }
        }
      }
    } else {
      // tiles too large: every element exactly, from global memory
      const int64_t n_el = o.out_count;
      for (int64_t e = threadIdx.x; e < n_el; e += kExpThreads) {
        int64_t loc = e;
        int b[4] = {0, 0, 0, 0};
        for (int a = 0; a < o.n_act; ++a) {
          b[a] = int(loc % mb[a]);
          loc /= mb[a];
        }
        const double xr = exact_x(nrem, d0, d1, d2, wblk + int64_t(rest) * b[0],
                                  nrem >= 1 ? gblk[0] + int64_t(d0) * b[1] : nullptr,
                                  nrem >= 2 ? gblk[1] + int64_t(d1) * b[2] : nullptr,
                                  nrem >= 3 ? gblk[2] + int64_t(d2) * b[3] : nullptr);
        const double x = xr;
        int64_t idx = base;
        for (int a = 0; a < o.n_act; ++a) idx += b[a] * sa[a];
        expand_emit(p, x, tc, crow, keybase, idx, keys, vals, cap_mask, counters);
      }
    }
    __syncthreads();  // tiles and s_job are rewritten for the next job
  }
}

__global__ void compact_kernel(const unsigned long long* __restrict__ keys, const double* __restrict__ vals,
                               unsigned long long cap, int R, unsigned long long* __restrict__ okeys,
                               double* __restrict__ ovals, unsigned long long* __restrict__ counters) {
  const unsigned long long s = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= cap) return;
  const unsigned long long k = keys[s];
  if (k == kEmpty) return;
  const unsigned long long pos = atomicAdd(counters + 3, 1ull);
  okeys[pos] = k;
  for (int r = 0; r < R; ++r) ovals[pos * R + r] = vals[s * R + r];
}

__global__ void pack_rows_kernel(const double* __restrict__ c, double* __restrict__ out, int64_t n, int R) {
  int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n * R) return;
  int64_t row = i / R;
  int r = int(i - row * R);
  out[i] = c[row + n * r];
}

inline bool fock_key(const int16_t* f, int N, uint64_t* key) {
  uint64_t k = 0;
  for (int i = 0; i < 2 * N; ++i) {
    if (f[i] < 0 || f[i] > 15) return false;
    k |= uint64_t(f[i]) << (4 * i);
  }
  *key = k;
  return true;
}

}  // namespace

#define FCG_CUDA(call)                                                               \
  do {                                                                               \
    cudaError_t e_ = (call);                                                         \
    if (e_ != cudaSuccess) {                                                         \
      ctx->err = std::string(#call) + ": " + cudaGetErrorString(e_);                 \
      return e_ == cudaErrorMemoryAllocation ? FCG_ENOMEM : FCG_ECUDA;               \
    }                                                                                \
  } while (0)

#define FCG_REQUIRE(cond, code, msg) \
  do {                               \
    if (!(cond)) {                   \
      ctx->err = (msg);              \
      return (code);                 \
    }                                \
  } while (0)

extern "C" {

int fcg_sigma_open(fcg_ctx* ctx, int R, const double* c, double thresh, int nbody, int64_t* n_out) {
  if (!ctx) return FCG_EINVAL;
  FCG_REQUIRE(ctx->have_state, FCG_ESTATE, "fcg_state_set must come first");
  FCG_REQUIRE(c && n_out, FCG_EINVAL, "null pointer");
  FCG_REQUIRE(R >= 1 && R <= kOpenMaxR, FCG_ELIMIT, "R must be in [1, 16]");
  FCG_REQUIRE(thresh >= 0.0, FCG_EINVAL, "thresh must be >= 0");
  FCG_CUDA(cudaSetDevice(ctx->device));
  {
    const int rc = ensure_wmax(ctx);
    if (rc) return rc;
  }
  *n_out = 0;
  const int N = ctx->N;
  const int nmax1 = ctx->nmax + 1;
  const Plan& P = ctx->plan;
  // ---- host plan: bra sectors and open term records per (ket sector, transfer) -------
  ProblemInfo pi;
  pi.N = N;
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
  std::vector<std::vector<int>> terms_of(ctx->n_trans);
  for (int t = 0; t < ctx->n_terms; ++t) terms_of[ctx->trm[int64_t(t) * kTrmCols + 1]].push_back(t);
  std::unordered_map<uint64_t, int32_t> bsec_of;
  ctx->open_bra_fock.clear();
  ctx->open_strides.clear();
  ctx->open_dims.clear();
  std::vector<OpenTerm> ots;
  std::vector<OpenItem> items;
  std::vector<int16_t> fb(2 * N);
  int64_t flops_ref = 0;
  std::unordered_set<int32_t> tdm_used;  // TDM blocks the jobs read
  for (size_t sk = 0; sk < P.sec_start.size(); ++sk) {
    const int16_t* fk = &P.sec_fock[sk * 2 * N];
    for (int tr = 0; tr < ctx->n_trans; ++tr) {
      if (terms_of[tr].empty()) continue;
      bool ok = true;
      for (int i = 0; i < 2 * N; ++i) {
        fb[i] = int16_t(fk[i] + ctx->trans[size_t(tr) * 2 * N + i]);
        if (fb[i] < 0 || fb[i] > ctx->norb[i / 2]) ok = false;
      }
      if (!ok) continue;
      // every cluster must have a local basis in its bra sector (:39-46)
      int64_t dims[kMaxClusters];
      for (int ci = 0; ci < N && ok; ++ci) {
        int bl = ctx->h_blk_index[dense_block_index(nmax1, ci, kOpH, fb[2 * ci], fb[2 * ci + 1], fb[2 * ci],
                                                    fb[2 * ci + 1])];
        if (bl < 0)
          ok = false;
        else
          dims[ci] = ctx->h_blocks[bl].mb;
      }
      if (!ok) continue;
      uint64_t key;
      fock_key(fb.data(), N, &key);
      int32_t bs;
      auto it = bsec_of.find(key);
      if (it == bsec_of.end()) {
        bs = int32_t(ctx->open_bra_fock.size() / (2 * N));
        FCG_REQUIRE(bs < (1 << 23), FCG_ELIMIT, "too many bra sectors for the open sigma key");
        bsec_of[key] = bs;
        ctx->open_bra_fock.insert(ctx->open_bra_fock.end(), fb.begin(), fb.end());
        int64_t stride = 1;
        for (int ci = 0; ci < N; ++ci) {
          ctx->open_strides.push_back(stride);
          ctx->open_dims.push_back(dims[ci]);
          stride *= dims[ci];
        }
        FCG_REQUIRE(stride < (int64_t(1) << kKeyIdxBits), FCG_ELIMIT, "bra sector product space exceeds 2^40");
      } else {
        bs = it->second;
      }
      const int32_t ot_off = int32_t(ots.size());
      for (int t : terms_of[tr]) {
        const int32_t* r = &ctx->trm[int64_t(t) * kTrmCols];
        if (r[0] > nbody) continue;
        OpenTerm o{};
        if (!make_term_sector(pi, t, fb.data(), fk, o.ts)) continue;
        const int pos = ctx->dress[t].pos < 0 ? 0 : ctx->dress[t].pos;
        const int cw = r[2 + pos];
        o.wmax_off = ctx->wmax_index[(int64_t(t) * nmax1 + fb[2 * cw]) * nmax1 + fb[2 * cw + 1]];
        o.bsec = bs;
        o.n_act = int8_t(1 + o.ts.nrem);
        o.c_act[0] = int8_t(cw);
        o.mb_act[0] = int16_t(o.ts.w_mb);
        int64_t cnt = o.ts.w_mb;
        for (int q = 0; q < o.ts.nrem; ++q) {
          const int cq = o.ts.cr[q];
          const int op = r[6 + ctx->dress[t].rem_pos[q]];
          const int bl = ctx->h_blk_index[dense_block_index(nmax1, cq, op, fb[2 * cq], fb[2 * cq + 1], fk[2 * cq],
                                                            fk[2 * cq + 1])];
          o.gmax_off[q] = ctx->gmax_off[bl];
          o.c_act[1 + q] = int8_t(cq);
          o.mb_act[1 + q] = int16_t(o.ts.g_mb[q]);
          cnt *= o.ts.g_mb[q];
        }
        FCG_REQUIRE(cnt < (int64_t(1) << 31), FCG_ELIMIT, "bra tuples of one term exceed 2^31");
        o.out_count = int32_t(cnt);
        // the reference's GEMM flops of this (ket, term) job (contract_matvec_thread,
        // src/tpsci_matvec_thread.jl:279-818, no prescreen): bra dims M and orbital index
        // lengths n in term order
        {
          const int nbd = r[0];
          int64_t M[4] = {1, 1, 1, 1}, nn[4] = {1, 1, 1, 1};
          for (int o2 = 0; o2 < nbd; ++o2) {
            const int cq = r[2 + o2];
            const int bl = ctx->h_blk_index[dense_block_index(nmax1, cq, r[6 + o2], fb[2 * cq], fb[2 * cq + 1],
                                                              fk[2 * cq], fk[2 * cq + 1])];
            M[o2] = ctx->h_blocks[bl].mb;
            nn[o2] = r[22 + o2];
            tdm_used.insert(bl);
          }
          int64_t f = 0;
          if (nbd == 2) f = nn[0] * nn[1] * M[0] + nn[1] * M[0] * M[1];
          if (nbd == 3) f = M[2] * (nn[0] * nn[1] * nn[2] + nn[0] * nn[1] * M[1] + nn[0] * M[0] * M[1]);
          if (nbd == 4)
            f = M[3] * (nn[0] * nn[1] * nn[2] * nn[3] +
                        M[2] * (nn[0] * nn[1] * nn[2] + nn[0] * nn[1] * M[1] + nn[0] * M[0] * M[1]));
          flops_ref += 2 * f * int64_t(P.sec_count[sk]);
        }
        ots.push_back(o);
      }
      const int32_t nt = int32_t(ots.size()) - ot_off;
      if (nt > 0) items.push_back(OpenItem{int32_t(P.sec_start[sk]), int32_t(P.sec_count[sk]), ot_off, nt});
    }
  }
  ctx->open_R = R;
  ctx->open_rows = 0;
  if (items.empty()) return FCG_OK;
  std::vector<int64_t> prefix(items.size() + 1, 0);
  for (size_t i = 0; i < items.size(); ++i) prefix[i + 1] = prefix[i] + int64_t(items[i].nrow) * items[i].nt;
  const int64_t n_jobs = prefix.back();
  // ---- device ---------------------------------------------------------------------------
  cudaStream_t s = ctx->stream;
  const int64_t n = ctx->n_cfg;
  FCG_CUDA(ctx->d_oterms.upload(ots.data(), ots.size(), s));
  FCG_CUDA(ctx->d_oitems.upload(items.data(), items.size(), s));
  FCG_CUDA(ctx->d_oprefix.upload(prefix.data(), prefix.size(), s));
  FCG_CUDA(ctx->d_ostrides.upload(ctx->open_strides.data(), ctx->open_strides.size(), s));
  FCG_CUDA(ctx->d_in64.alloc(size_t(n) * R));
  FCG_CUDA(ctx->d_c64.alloc(size_t(n) * R));
  FCG_CUDA(cudaMemcpyAsync(ctx->d_in64.p, c, sizeof(double) * n * R, cudaMemcpyHostToDevice, s));
  pack_rows_kernel<<<unsigned((n * R + 255) / 256), 256, 0, s>>>(ctx->d_in64.p, ctx->d_c64.p, n, R);
  FCG_CUDA(cudaGetLastError());
  FCG_CUDA(ctx->d_counters.alloc(5));
  FCG_CUDA(cudaMemsetAsync(ctx->d_counters.p, 0, 4 * sizeof(unsigned long long), s));
  FCG_CUDA(ctx->d_ojobs.alloc(size_t(n_jobs)));
  OpenParams p{};
  p.ot = ctx->d_oterms.p;
  p.items = ctx->d_oitems.p;
  p.prefix = ctx->d_oprefix.p;
  p.n_items = int64_t(items.size());
  p.n_jobs = n_jobs;
  p.cfg = ctx->d_cfg.p;
  p.c = ctx->d_c64.p;
  p.strides = ctx->d_ostrides.p;
  p.N = N;
  p.R = R;
  p.thresh = thresh;
  FCG_CUDA(cudaEventRecord(ctx->ev0, s));
  screen_kernel<<<unsigned((n_jobs + 255) / 256), 256, 0, s>>>(p, ctx->d_wmax.p, ctx->d_gmax.p, ctx->d_ojobs.p,
                                                              ctx->d_counters.p);
  FCG_CUDA(cudaGetLastError());
  unsigned long long cnt[4];
  FCG_CUDA(cudaMemcpyAsync(cnt, ctx->d_counters.p, sizeof(cnt), cudaMemcpyDeviceToHost, s));
  FCG_CUDA(cudaStreamSynchronize(s));
  const int64_t n_kept = int64_t(cnt[0]);
  const int64_t n_elem = int64_t(cnt[1]);
  int launches = 2;
  if (n_kept > 0) {
    // shared memory of the expand CTAs: the largest job tiles, up to the budget
    int smem_bytes = 0;
    for (const OpenTerm& o : ots)
      smem_bytes = std::max(smem_bytes, expand_tiles(o.ts.nrem, o.ts.rest_len, o.ts.g_dim, o.mb_act).bytes);
    smem_bytes = std::min(smem_bytes, kExpSmemBytes);
    const size_t smem = size_t(smem_bytes);
    FCG_CUDA(cudaFuncSetAttribute(expand_jobs_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kExpSmemBytes));
    int per_sm = 0, n_sm = 0;
    FCG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, expand_jobs_kernel, kExpThreads, smem));
    FCG_CUDA(cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, ctx->device));
    const int64_t grid = std::max<int64_t>(1, std::min<int64_t>(int64_t(std::max(per_sm, 1)) * n_sm, n_kept));
    // table: twice the contributions, power of two, at least 4096 slots; doubled on overflow
    unsigned long long cap = 4096;
    while (cap < 2ull * (unsigned long long)n_elem && cap < (1ull << 28)) cap <<= 1;
    for (int attempt = 0;; ++attempt) {
      FCG_CUDA(ctx->d_hkeys.alloc(cap));
      FCG_CUDA(ctx->d_hvals.alloc(cap * R));
      FCG_CUDA(cudaMemsetAsync(ctx->d_hkeys.p, 0xFF, cap * sizeof(unsigned long long), s));
      FCG_CUDA(cudaMemsetAsync(ctx->d_hvals.p, 0, cap * R * sizeof(double), s));
      FCG_CUDA(cudaMemsetAsync(ctx->d_counters.p + 2, 0, 3 * sizeof(unsigned long long), s));
      FCG_CUDA(cudaEventRecord(ctx->ev2, s));
      expand_jobs_kernel<<<unsigned(grid), kExpThreads, smem, s>>>(p, ctx->d_ojobs.p, n_kept, ctx->d_w64.p,
                                                                   ctx->d_op64.p, ctx->d_hkeys.p, ctx->d_hvals.p,
                                                                   cap - 1, ctx->d_counters.p, smem_bytes);
      FCG_CUDA(cudaGetLastError());
      FCG_CUDA(cudaEventRecord(ctx->ev3, s));
      FCG_CUDA(cudaMemcpyAsync(cnt, ctx->d_counters.p, sizeof(cnt), cudaMemcpyDeviceToHost, s));
      FCG_CUDA(cudaStreamSynchronize(s));
      launches += 2;
      if (cnt[2] == 0) break;
      FCG_REQUIRE(attempt < 3 && cap < (1ull << 31), FCG_ENOMEM, "open sigma hash table overflow");
      cap <<= 1;
    }
    FCG_CUDA(ctx->d_okeys.alloc(cap));
    FCG_CUDA(ctx->d_ovals.alloc(cap * R));
    compact_kernel<<<unsigned((cap + 255) / 256), 256, 0, s>>>(ctx->d_hkeys.p, ctx->d_hvals.p, cap, R,
                                                               ctx->d_okeys.p, ctx->d_ovals.p, ctx->d_counters.p);
    FCG_CUDA(cudaGetLastError());
    FCG_CUDA(cudaEventRecord(ctx->ev1, s));
    FCG_CUDA(cudaMemcpyAsync(cnt, ctx->d_counters.p, sizeof(cnt), cudaMemcpyDeviceToHost, s));
    FCG_CUDA(cudaStreamSynchronize(s));
    launches += 1;
    const int64_t n_rows = int64_t(cnt[3]);
    FCG_CUDA(ctx->open_keys.alloc(size_t(n_rows)));
    FCG_CUDA(ctx->open_vals.alloc(size_t(n_rows) * R));
    ctx->open_rows = n_rows;
    FCG_CUDA(cudaMemcpyAsync(ctx->open_keys.p, ctx->d_okeys.p, n_rows * sizeof(unsigned long long),
                             cudaMemcpyDeviceToHost, s));
    FCG_CUDA(cudaMemcpyAsync(ctx->open_vals.p, ctx->d_ovals.p, n_rows * R * sizeof(double),
                             cudaMemcpyDeviceToHost, s));
    FCG_CUDA(cudaStreamSynchronize(s));
    float ms = 0.f;
    FCG_CUDA(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
    ctx->stats.last_kernel_ms = ms;
    FCG_CUDA(cudaEventElapsedTime(&ms, ctx->ev2, ctx->ev3));
    ctx->stats.open_expand_ms = ms;
  }
  // compulsory bytes: the TDM blocks the jobs touch, C, and one key + row per output
  int64_t tdm_bytes = 0;
  for (int32_t bl : tdm_used) {
    const BlockInfo& B = ctx->h_blocks[bl];
    tdm_bytes += int64_t(B.nidx) * B.mb * B.mk * 8;
  }
  ctx->stats.open_flops_reference = flops_ref;
  ctx->stats.open_bytes = tdm_bytes + 8 * n * R + ctx->open_rows * (6 * int64_t(N) + 8 * int64_t(R));
  ctx->stats.kernel_launches = launches;
  ctx->stats.open_jobs = n_jobs;
  ctx->stats.open_jobs_kept = n_kept;
  ctx->stats.open_contractions = n_elem;
  *n_out = ctx->open_rows;
  return FCG_OK;
}

int fcg_sigma_open_fetch(fcg_ctx* ctx, int16_t* fock, int16_t* cfg, double* coeff) {
  if (!ctx) return FCG_EINVAL;
  FCG_REQUIRE(fock && cfg && coeff, FCG_EINVAL, "null pointer");
  const int N = ctx->N;
  const int R = ctx->open_R;
  const int64_t m = ctx->open_rows;
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < m; ++i) {
    const unsigned long long key = ctx->open_keys.p[i];
    const int64_t bs = int64_t(key >> kKeyIdxBits);
    int64_t idx = int64_t(key & ((1ull << kKeyIdxBits) - 1));
    std::memcpy(fock + i * 2 * N, &ctx->open_bra_fock[bs * 2 * N], sizeof(int16_t) * 2 * N);
    for (int c = 0; c < N; ++c) {
      const int64_t d = ctx->open_dims[bs * N + c];
      cfg[i * N + c] = int16_t(idx % d);
      idx /= d;
    }
    for (int r = 0; r < R; ++r) coeff[i + m * r] = ctx->open_vals.p[size_t(i) * R + r];
  }
  return FCG_OK;
}

}  // extern "C"
