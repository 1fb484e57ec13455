// Block-sparse Tucker (BST) sigma build on the GPU: cache_hamiltonian
// (src/tucker_inner.jl:90-159) and build_sigma! (src/tucker_inner.jl:165-245).
//
// fcg_bst_set plans, on the host, the (bra block, ket block, term) triples that pass
// check_term on TuckerConfigs and gathers them into groups (bra, ket, active clusters).
// On the device it then builds, once per BST structure,
//   gammas    g[p, kb, kk] = sum_{I,J} U_bra[I, kb] G[p, I, J] U_ket[J, kk] per (bra, ket, cluster, op)
//             (the first step of build_dense_H_term, src/tucker_build_dense_H_term.jl:5-175)
//   operators OP_group[kk, kb] = sum over the group's terms of sign * sum_p ints[p...] prod_a g_a
//             times the product of the rank-1 spectator overlaps (a scalar, as in
//             contract_dense_H_with_state, src/tucker_contract_dense_H_with_state.jl:93-105)
//   overlaps  S_c = U_bra,c^T U_ket,c for the other spectators.
// fcg_bst_sigma applies them: per group and root, the ket core's spectator modes go to the
// bra bases by mode products with S_c (transform_basis, src/hosvd.jl:634-670), then
// bra core[kb] += sum_kk OP[kk, kb_active] X[kk_active, kb_spectators]  (the op2^T * ket2 GEMM
// of contract_dense_H_with_state).
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstring>
#include <map>
#include <thread>
#include <unordered_map>
#include <vector>

#include "fcg_ctx.cuh"
#include "tcgen05.cuh"

using namespace fcg;

namespace {

constexpr int kBstThreads = 256;
constexpr int kOpThreads = 64;            // threads per group of the operator-cache build
constexpr int kGammaSmem = 6144;          // doubles of the per-p staging tile of the gamma kernel
constexpr int kSigmaSmemBytes = 96 * 1024;  // shared-memory workspace of a CTA-per-group sigma launch
// CTA-per-group launches by workspace size: a launch reserves its largest group's shared
// memory for every CTA, so groups are bucketed by the bytes they need (more resident CTAs for
// the small ones)
constexpr int kSmemBuckets = 4;
constexpr int kSmemBucket[kSmemBuckets] = {12 * 1024, 24 * 1024, 48 * 1024, kSigmaSmemBytes};
// shared memory of one warp of bst_sigma_bra_kernel (description + workspace); larger groups
// run one CTA per group.  Measured on the 32-orbital / 8-cluster vector with cores up to 12^4:
// float builds are fastest with 4 KB (9 % faster than 8 KB once the CTA-per-group launches
// were bucketed by workspace size), double builds with 2 KB.
constexpr int warp_smem_bytes(size_t elem) { return elem == 4 ? 4 * 1024 : 2 * 1024; }
constexpr int kWarpSmemMax = 8 * 1024;
constexpr int kAccBytes = 32 * 1024;        // shared-memory bra-core accumulator of bst_sigma_bra_kernel
constexpr int64_t kChunkWork = int64_t(1) << 16;  // multiply-adds per bst_sigma_bra_kernel CTA, about

// ---- operator cache ----------------------------------------------------------------------

// One CTA per gamma.  For each orbital multi-index p:  T[I, kk] = sum_J G[p, I, J] U_ket[J, kk]
// staged in shared memory, then g[p, kb, kk] = sum_I U_bra[I, kb] T[I, kk].  Tiles that do
// not fit the staging buffer use the direct double sum.
__global__ void __launch_bounds__(kBstThreads) bst_gamma_kernel(const BstGamma* __restrict__ gam,
                                                                const BstBlock* __restrict__ blocks,
                                                                const double* __restrict__ tdm,
                                                                const double* __restrict__ factors,
                                                                double* __restrict__ g) {
  __shared__ double tile[kGammaSmem];
  const BstGamma Q = gam[blockIdx.x];
  const BstBlock& B = blocks[Q.bra];
  const BstBlock& K = blocks[Q.ket];
  const int c = Q.c, np = Q.np, mb = Q.tdm_mb;
  const int rb = B.rank[c], rk = K.rank[c], Lb = B.len[c], Lk = K.len[c];
  const int sb = B.start[c], sk = K.start[c];
  const double* Ub = factors + B.factor_off[c];
  const double* Uk = factors + K.factor_off[c];
  const double* G = tdm + Q.tdm_off;
  double* out = g + Q.g_off;
  if (Lb * rk <= kGammaSmem) {
    for (int p = 0; p < np; ++p) {
      for (int e = threadIdx.x; e < Lb * rk; e += blockDim.x) {
        const int I = e % Lb, kk = e / Lb;
        const double* gcol = G + p + int64_t(np) * (sb + I);
        double s = 0.0;
        for (int J = 0; J < Lk; ++J) s = fma(gcol[int64_t(np) * mb * (sk + J)], Uk[J + int64_t(Lk) * kk], s);
        tile[e] = s;
      }
      __syncthreads();
      for (int e = threadIdx.x; e < rb * rk; e += blockDim.x) {
        const int kb = e % rb, kk = e / rb;
        double s = 0.0;
        for (int I = 0; I < Lb; ++I) s = fma(Ub[I + int64_t(Lb) * kb], tile[I + Lb * kk], s);
        out[p + int64_t(np) * e] = s;
      }
      __syncthreads();
    }
  } else {
    const int64_t n = int64_t(np) * rb * rk;
    for (int64_t e = threadIdx.x; e < n; e += blockDim.x) {
      const int p = int(e % np);
      const int kb = int((e / np) % rb);
      const int kk = int(e / (int64_t(np) * rb));
      double s = 0.0;
      for (int J = 0; J < Lk; ++J) {
        double inner = 0.0;
        for (int I = 0; I < Lb; ++I)
          inner = fma(Ub[I + int64_t(Lb) * kb], G[p + int64_t(np) * ((sb + I) + int64_t(mb) * (sk + J))], inner);
        s = fma(inner, Uk[J + int64_t(Lk) * kk], s);
      }
      out[e] = s;
    }
  }
}

// One CTA per group: the group operator, scaled by the product of the rank-1 spectator overlaps.
// Groups of two or more active clusters are built factored on the first active cluster: for
// each index tuple q' of the other clusters (their bra and ket ranks),
//   u[p0] = sum_{p1..} ints[p0, p1, ..] prod_{a>0} g_a[p_a, q'_a]
// once per term, then every element of the first cluster's (bra, ket) ranks is
// sum_p0 g_0[p0, kb0, kk0] u[p0] -- len(p1..) + rank^2 len(p0) multiply-adds per tuple in
// place of rank^2 len(p0..) (the successive contractions of build_dense_H_term,
// src/tucker_build_dense_H_term.jl:5-175).  A work item is one tuple and kOpChunk of the first
// cluster's elements; u lives in shared memory, one column per thread.
constexpr int kOpMaxD0 = 64;  // longest orbital multi-index of the first active cluster built factored
constexpr int kOpChunk = 16;  // operator elements per work item of the factored build

__global__ void __launch_bounds__(kOpThreads) bst_op_kernel(const BstGroup* __restrict__ groups,
                                                             const BstGroupTerm* __restrict__ gterms,
                                                             const BstBlock* __restrict__ blocks, int N,
                                                             const double* __restrict__ ints,
                                                             const double* __restrict__ g,
                                                             const double* __restrict__ factors,
                                                             double* __restrict__ opc) {
  __shared__ double scal;
  __shared__ double u_all[kOpMaxD0 * kOpThreads];
  const BstGroup& Gp = groups[blockIdx.x];
  const BstBlock& B = blocks[Gp.bra];
  const BstBlock& K = blocks[Gp.ket];
  if (threadIdx.x == 0) {
    double s = 1.0;
    for (int c = 0; c < N; ++c) {
      if ((Gp.act_mask >> c) & 1) continue;
      if (B.rank[c] != 1 || K.rank[c] != 1) continue;
      const double* ub = factors + B.factor_off[c];
      const double* uk = factors + K.factor_off[c];
      double d = 0.0;
      for (int x = 0; x < B.len[c]; ++x) d = fma(ub[x], uk[x], d);
      s *= d;
    }
    scal = s;
  }
  __syncthreads();
  int act[4], na = 0;
  for (int c = 0; c < N; ++c)
    if ((Gp.act_mask >> c) & 1) act[na++] = c;
  bool factored = na >= 2;
  for (int t = 0; t < Gp.nt && factored; ++t) {
    const BstGroupTerm& T = gterms[Gp.t_off + t];
    factored = T.ints_off >= 0 && T.nact == na && T.np[0] <= kOpMaxD0;
  }
  if (factored) {
    const int rb0 = B.rank[act[0]], rk0 = K.rank[act[0]];
    const int q0n = rb0 * rk0;
    const int krest = Gp.k / rk0, brest = Gp.m / rb0;
    const int nch = (q0n + kOpChunk - 1) / kOpChunk;
    const int64_t items = int64_t(krest) * brest * nch;
    double* u = u_all + threadIdx.x;  // u[p] at u[p * kOpThreads]
    for (int64_t item = threadIdx.x; item < items; item += blockDim.x) {
      const int64_t tq = item / nch;
      const int ch = int(item - tq * nch);
      const int kk_rest = int(tq % krest), kb_rest = int(tq / krest);
      int ik[4] = {0, 0, 0, 0}, ib[4] = {0, 0, 0, 0};
      {
        int x = kk_rest, y = kb_rest;
        for (int a = 1; a < na; ++a) {
          ik[a] = x % K.rank[act[a]];
          x /= K.rank[act[a]];
          ib[a] = y % B.rank[act[a]];
          y /= B.rank[act[a]];
        }
      }
      const int o0 = ch * kOpChunk;
      double acc[kOpChunk];
#pragma unroll
      for (int o = 0; o < kOpChunk; ++o) acc[o] = 0.0;
      for (int t = 0; t < Gp.nt; ++t) {
        const BstGroupTerm T = gterms[Gp.t_off + t];
        const double* v = ints + T.ints_off;
        const int d0 = T.np[0], d1 = T.np[1];
        const int d2 = T.nact > 2 ? T.np[2] : 1, d3 = T.nact > 3 ? T.np[3] : 1;
        const double* ga[4];
        for (int a = 1; a < T.nact; ++a)
          ga[a] = g + T.g_off[a] + int64_t(T.np[a]) * (ib[a] + int64_t(B.rank[act[a]]) * ik[a]);
        for (int p = 0; p < d0; ++p) u[p * kOpThreads] = 0.0;
        for (int l = 0; l < d3; ++l) {
          const double x3 = T.nact > 3 ? ga[3][l] : 1.0;
          for (int r = 0; r < d2; ++r) {
            const double x2 = (T.nact > 2 ? ga[2][r] : 1.0) * x3;
            for (int j = 0; j < d1; ++j) {
              const double x1 = ga[1][j] * x2;
              const double* vj = v + int64_t(d0) * (j + int64_t(d1) * (r + int64_t(d2) * l));
              for (int p = 0; p < d0; ++p) u[p * kOpThreads] = fma(vj[p], x1, u[p * kOpThreads]);
            }
          }
        }
        const double sg = double(T.sign);
        const double* g0 = g + T.g_off[0];
#pragma unroll
        for (int o = 0; o < kOpChunk; ++o) {
          const int q = o0 + o;
          if (q < q0n) {
            const double* g0q = g0 + int64_t(d0) * q;  // (ib0 + rb0 * ik0) = q
            double sacc = 0.0;
            for (int p = 0; p < d0; ++p) sacc = fma(g0q[p], u[p * kOpThreads], sacc);
            acc[o] = fma(sg, sacc, acc[o]);
          }
        }
      }
#pragma unroll
      for (int o = 0; o < kOpChunk; ++o) {
        const int q = o0 + o;
        if (q < q0n) {
          const int ib0 = q % rb0, ik0 = q / rb0;
          const int64_t kk = ik0 + int64_t(rk0) * kk_rest, kb = ib0 + int64_t(rb0) * kb_rest;
          opc[Gp.op_off + kk + int64_t(Gp.k) * kb] = scal * acc[o];
        }
      }
    }
    return;
  }
  const int64_t n = int64_t(Gp.m) * Gp.k;
  for (int64_t e = threadIdx.x; e < n; e += blockDim.x) {
    int64_t kk = e % Gp.k, kb = e / Gp.k;
    int ik[4], ib[4];
    for (int a = 0; a < na; ++a) {
      ik[a] = int(kk % K.rank[act[a]]);
      kk /= K.rank[act[a]];
      ib[a] = int(kb % B.rank[act[a]]);
      kb /= B.rank[act[a]];
    }
    double val = 0.0;
    for (int t = 0; t < Gp.nt; ++t) {
      const BstGroupTerm T = gterms[Gp.t_off + t];
      // the term's clusters are the group's active clusters, in increasing order
      const double* ga[4];
      for (int a = 0; a < T.nact; ++a)
        ga[a] = g + T.g_off[a] + int64_t(T.np[a]) * (ib[a] + int64_t(B.rank[act[a]]) * ik[a]);
      if (T.ints_off < 0) {
        val += double(T.sign) * ga[0][0];
        continue;
      }
      const double* v = ints + T.ints_off;
      const int d0 = T.np[0], d1 = T.np[1];
      const int d2 = T.nact > 2 ? T.np[2] : 1, d3 = T.nact > 3 ? T.np[3] : 1;
      double acc = 0.0;
      for (int l = 0; l < d3; ++l) {
        const double x3 = T.nact > 3 ? ga[3][l] : 1.0;
        for (int r = 0; r < d2; ++r) {
          const double x2 = (T.nact > 2 ? ga[2][r] : 1.0) * x3;
          for (int j = 0; j < d1; ++j) {
            const double x1 = ga[1][j] * x2;
            const double* vj = v + int64_t(d0) * (j + int64_t(d1) * (r + int64_t(d2) * l));
            double s = 0.0;
            for (int i = 0; i < d0; ++i) s = fma(ga[0][i], vj[i], s);
            acc = fma(s, x1, acc);
          }
        }
      }
      val = fma(double(T.sign), acc, val);
    }
    opc[Gp.op_off + e] = scal * val;
  }
}

// S_c = U_bra,c^T U_ket,c for each (group, spectator) with a non-scalar overlap.
struct BstOverlapJob {
  int64_t s_off;
  int32_t bra, ket, c, pad;
};

__global__ void bst_overlap_kernel(const BstOverlapJob* __restrict__ jobs, const BstBlock* __restrict__ blocks,
                                   const double* __restrict__ factors, double* __restrict__ S) {
  const BstOverlapJob J = jobs[blockIdx.x];
  const BstBlock& B = blocks[J.bra];
  const BstBlock& K = blocks[J.ket];
  const int c = J.c, rb = B.rank[c], rk = K.rank[c], L = B.len[c];
  const double* Ub = factors + B.factor_off[c];
  const double* Uk = factors + K.factor_off[c];
  for (int e = threadIdx.x; e < rb * rk; e += blockDim.x) {
    const int i = e % rb, j = e / rb;
    double s = 0.0;
    for (int x = 0; x < L; ++x) s = fma(Ub[x + int64_t(L) * i], Uk[x + int64_t(L) * j], s);
    S[J.s_off + e] = s;
  }
}

__global__ void bst_convert_kernel(const double* __restrict__ a, float* __restrict__ b, int64_t n) {
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
    b[i] = float(a[i]);
}

__global__ void bst_widen_kernel(const float* __restrict__ a, double* __restrict__ b, int64_t n) {
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
    b[i] = double(a[i]);
}

// One actives-first index table: block `block`'s positions for the active clusters `mask`,
// at perm[off, off + core_len).
struct BstPermTable {
  int64_t off;
  int32_t block, mask;
};

// One CTA per index table: perm[off + x] = core offset of position x of the block's
// actives-first layout for the active clusters `mask`, x = (mixed radix over the active
// clusters) + (their rank product) * (mixed radix over the other clusters), both in increasing
// cluster order; the core is column-major over the clusters (cluster 0 fastest).
__global__ void bst_perm_kernel(const BstPermTable* __restrict__ tables, const BstBlock* __restrict__ blocks, int N,
                                int32_t* __restrict__ perm) {
  const BstPermTable T = tables[blockIdx.x];
  const BstBlock& B = blocks[T.block];
  int rank[kMaxClusters];
  int ka_len = 1;
  for (int c = 0; c < N; ++c) {
    rank[c] = B.rank[c];
    if ((T.mask >> c) & 1) ka_len *= rank[c];
  }
  for (int e = threadIdx.x; e < B.core_len; e += blockDim.x) {
    int rem = e, ka = 0, kam = 1, sp = 0, spm = 1;
    for (int c = 0; c < N; ++c) {
      const int v = rem % rank[c];
      rem /= rank[c];
      if ((T.mask >> c) & 1) {
        ka += v * kam;
        kam *= rank[c];
      } else {
        sp += v * spm;
        spm *= rank[c];
      }
    }
    perm[T.off + ka + int64_t(ka_len) * sp] = e;
  }
}

// ---- sigma ---------------------------------------------------------------------------------

template <int TEAM>
__device__ __forceinline__ void team_sync() {
  if (TEAM == 32)
    __syncwarp();
  else
    __syncthreads();
}

// Copy a group description into shared memory (16-byte units) by a team.
template <int TEAM>
__device__ __forceinline__ void load_group(const BstGroup* __restrict__ src, BstGroup* dst, int tid) {
  const int4* s4 = reinterpret_cast<const int4*>(src);
  int4* d4 = reinterpret_cast<int4*>(dst);
  for (int i = tid; i < int(sizeof(BstGroup) / 16); i += TEAM) d4[i] = s4[i];
  team_sync<TEAM>();
}

// Prefetch [p, p + bytes) into L2 (or L1), one 128-byte line per request, by a team.
template <int TEAM, bool L1>
__device__ __forceinline__ void prefetch_range(const void* p, int64_t bytes, int tid) {
  const char* c = static_cast<const char*>(p);
  for (int64_t off = int64_t(tid) * 128; off < bytes; off += int64_t(TEAM) * 128) {
    if (L1)
      asm volatile("prefetch.global.L1 [%0];" ::"l"(c + off));
    else
      asm volatile("prefetch.global.L2 [%0];" ::"l"(c + off));
  }
}

// One group, all R roots, by a team of TEAM threads (a warp or the CTA); G is the group's
// description in shared memory, ws two buffers of `stride` elements per root.
// The ket core is gathered with the active clusters merged into one leading mode of length
// k (mixed radix in cluster order) followed by the spectator modes in cluster order, so that
//   X[kk + k*s]
// is the GEMM operand of contract_dense_H_with_state (actives permuted to the front).  The
// spectator modes then go to the bra bases (mode products with S_j = U_bra^T U_ket), and
// every (bra active column kb, spectator index s, root) is one dot product of length k of
// two contiguous vectors, OP[:, kb] and X[:, s], taken by a sub-warp of `lanes` threads
// (power of two, <= 32) and added to out[r * out_stride + bra core index].
// Steps 1-2 of a group (the GEMM operand X of every root), by a team; X of root r ends in
// ws[(2 r + cur) * stride], cur = ntr & 1 (one buffer swap per applied overlap), returned.
// ket ranks up to which a spectator mode product keeps a thread's input fibre in registers
constexpr int kModeRegs = 16;

template <typename T, int TEAM>
__device__ int bst_group_prepare(const BstGroup& G, int R, const T* __restrict__ S, const int32_t* __restrict__ perm,
                                 const T* __restrict__ cin, int64_t core_total, T* ws, int stride) {
  const int tid = TEAM == 32 ? int(threadIdx.x & 31) : int(threadIdx.x);
  const int k = G.k, nsp = G.nsp;
  // 1. gather the ket cores in X order (the ket's actives-first index table)
  {
    const int n = G.kcore;
    const int32_t* kp = perm + G.kperm_off;
    for (int r = 0; r < R; ++r) {
      const T* src = cin + int64_t(r) * core_total + G.k_off;
      T* dst = ws + int64_t(2 * r) * stride;
      for (int e = tid; e < n; e += TEAM) dst[e] = src[__ldg(kp + e)];
    }
  }
  team_sync<TEAM>();
  // 2. spectator modes to the bra bases
  int cur = 0;
  {
    int inner = k;
    for (int j = 0; j < nsp; ++j) {
      int outer = 1;
      for (int i = j + 1; i < nsp; ++i) outer *= G.s_kr[i];
      const int rb = G.s_br[j], rk = G.s_kr[j];
      if (G.s_off[j] < 0) {  // the identity: X keeps this mode as it is
        inner *= rb;
        continue;
      }
      const T* Sj = S + G.s_off[j];
      if (sizeof(T) == 4 && rk <= kModeRegs) {
        // one thread per (root, a, o): the rk inputs of its fibre in registers, all rb outputs
        // (float builds: the unrolled, predicated multiply-adds cost the FP64 pipe more than
        // the saved loads)
        const int n = inner * outer;
        for (int idx = tid; idx < R * n; idx += TEAM) {
          const int r = idx / n, e = idx - r * n;
          const int a = e % inner, o = e / inner;
          const T* src = ws + int64_t(2 * r + cur) * stride + a + int64_t(inner) * rk * o;
          T* dst = ws + int64_t(2 * r + (cur ^ 1)) * stride + a + int64_t(inner) * rb * o;
          T v[kModeRegs];
#pragma unroll
          for (int l = 0; l < kModeRegs; ++l) v[l] = l < rk ? src[int64_t(inner) * l] : T(0);
          for (int q = 0; q < rb; ++q) {
            T acc = T(0);
#pragma unroll
            for (int l = 0; l < kModeRegs; ++l)
              if (l < rk) acc = fma(__ldg(Sj + q + rb * l), v[l], acc);
            dst[int64_t(inner) * q] = acc;
          }
        }
      } else {
        const int n = inner * rb * outer;
        for (int idx = tid; idx < R * n; idx += TEAM) {
          const int r = idx / n, e = idx - r * n;
          const int a = e % inner, q = (e / inner) % rb, o = e / (inner * rb);
          const T* src = ws + int64_t(2 * r + cur) * stride + a + inner * rk * o;
          T acc = T(0);
          for (int l = 0; l < rk; ++l) acc = fma(Sj[q + rb * l], src[inner * l], acc);
          ws[int64_t(2 * r + (cur ^ 1)) * stride + e] = acc;
        }
      }
      team_sync<TEAM>();
      cur ^= 1;
      inner *= rb;
    }
  }
  return cur;
}

// 4 consecutive elements at a 16-byte aligned generic address (global or shared memory)
template <typename T>
__device__ __forceinline__ void load4(const T* p, T* v) {
  if constexpr (sizeof(T) == 4) {
    const float4 q = *reinterpret_cast<const float4*>(p);
    v[0] = q.x, v[1] = q.y, v[2] = q.z, v[3] = q.w;
  } else {
    const double2 a = *reinterpret_cast<const double2*>(p);
    const double2 b = *reinterpret_cast<const double2*>(p + 2);
    v[0] = a.x, v[1] = a.y, v[2] = b.x, v[3] = b.y;
  }
}

// Step 3 of a group in register tiles: each thread takes TM bra-active columns x TN
// spectator indices of one root, D[col, s] = OP[:, col] . X[:, s], so that one column load
// feeds TN (or TM) multiply-adds; columns of length k % 4 == 0 are read 4 elements at a time
// (operator and workspace columns then start on 16-byte boundaries).  Edge tiles repeat the
// last column and drop the extra results.
template <typename T, int TEAM, bool ATOMIC, int TM, int TN>
__device__ __forceinline__ void bst_tile_gemm(const T* __restrict__ opg, int k, int m, int ns, int R, const T* ws,
                                              int stride, int cur, const int32_t* __restrict__ bp, T* out,
                                              int64_t out_stride, int tid) {
  const int tm = (m + TM - 1) / TM, tn = (ns + TN - 1) / TN, tiles = tm * tn;
  const bool vec = (k & 3) == 0;
  for (int it = tid; it < tiles * R; it += TEAM) {
    const int r = it / tiles, t = it - r * tiles;
    const int c0 = (t % tm) * TM, s0 = (t / tm) * TN;
    const T* X = ws + int64_t(2 * r + cur) * stride;
    const T* a[TM];
    const T* b[TN];
#pragma unroll
    for (int i = 0; i < TM; ++i) a[i] = opg + int64_t(k) * min(c0 + i, m - 1);
#pragma unroll
    for (int j = 0; j < TN; ++j) b[j] = X + int64_t(k) * min(s0 + j, ns - 1);
    T acc[TM][TN];
#pragma unroll
    for (int i = 0; i < TM; ++i)
#pragma unroll
      for (int j = 0; j < TN; ++j) acc[i][j] = T(0);
    if (vec) {
      for (int kk = 0; kk < k; kk += 4) {
        T av[TM][4], bv[TN][4];
#pragma unroll
        for (int i = 0; i < TM; ++i) load4(a[i] + kk, av[i]);
#pragma unroll
        for (int j = 0; j < TN; ++j) load4(b[j] + kk, bv[j]);
#pragma unroll
        for (int q = 0; q < 4; ++q)
#pragma unroll
          for (int i = 0; i < TM; ++i)
#pragma unroll
            for (int j = 0; j < TN; ++j) acc[i][j] = fma(av[i][q], bv[j][q], acc[i][j]);
      }
    } else {
      for (int kk = 0; kk < k; ++kk) {
        T av[TM], bv[TN];
#pragma unroll
        for (int i = 0; i < TM; ++i) av[i] = a[i][kk];
#pragma unroll
        for (int j = 0; j < TN; ++j) bv[j] = b[j][kk];
#pragma unroll
        for (int i = 0; i < TM; ++i)
#pragma unroll
          for (int j = 0; j < TN; ++j) acc[i][j] = fma(av[i], bv[j], acc[i][j]);
      }
    }
    T* outr = out + int64_t(r) * out_stride;
#pragma unroll
    for (int i = 0; i < TM; ++i)
#pragma unroll
      for (int j = 0; j < TN; ++j) {
        const int col = c0 + i, sp = s0 + j;
        if (col < m && sp < ns) {
          T* dst = outr + __ldg(bp + col + m * sp);
          if (ATOMIC)
            atomicAdd(dst, acc[i][j]);
          else
            *dst += acc[i][j];
        }
      }
  }
}

template <typename T, int TEAM, bool ATOMIC>
__device__ void bst_group_apply(const BstGroup& G, int R, const T* __restrict__ op, const T* __restrict__ S,
                                const int32_t* __restrict__ perm, const T* __restrict__ cin, int64_t core_total,
                                T* ws, int stride, T* out, int64_t out_stride) {
  const int tid = TEAM == 32 ? int(threadIdx.x & 31) : int(threadIdx.x);
  const int k = G.k, m = G.m, nsp = G.nsp;
  prefetch_range<TEAM, true>(op + G.op_off, int64_t(m) * k * int64_t(sizeof(T)), tid);
  const int cur = bst_group_prepare<T, TEAM>(G, R, S, perm, cin, core_total, ws, stride);
  // 3. bra core[kb, s] += OP[:, kb] . X[:, s]; position col + m*s of the bra's actives-first
  // layout is bra core index bp[col + m*s]
  int ns = 1;
  for (int j = 0; j < nsp; ++j) ns *= G.s_br[j];
  const int mn = m * ns;
  const T* opg = op + G.op_off;
  const int32_t* bp = perm + G.bperm_off;
  if (mn * R >= 16 * TEAM) {
    bst_tile_gemm<T, TEAM, ATOMIC, 4, 4>(opg, k, m, ns, R, ws, stride, cur, bp, out, out_stride, tid);
    return;
  }
  if (mn * R >= 4 * TEAM) {
    bst_tile_gemm<T, TEAM, ATOMIC, 2, 2>(opg, k, m, ns, R, ws, stride, cur, bp, out, out_stride, tid);
    return;
  }
  if (k < 32) {
    // short columns: one thread per (kb, s) and root; items of one group never share an output
    for (int r = 0; r < R; ++r) {
      const T* Xr = ws + int64_t(2 * r + cur) * stride;
      T* outr = out + int64_t(r) * out_stride;
      for (int it = tid; it < mn; it += TEAM) {
        const int s = it / m, col = it - s * m;
        const T* o = opg + int64_t(k) * col;
        const T* X = Xr + int64_t(k) * s;
        T acc = T(0), acc2 = T(0);
        int kk = 0;
        for (; kk + 1 < k; kk += 2) {
          acc = fma(o[kk], X[kk], acc);
          acc2 = fma(o[kk + 1], X[kk + 1], acc2);
        }
        if (kk < k) acc = fma(o[kk], X[kk], acc);
        acc += acc2;
        T* dst = outr + __ldg(bp + it);
        if (ATOMIC)
          atomicAdd(dst, acc);
        else
          *dst += acc;
      }
    }
    return;
  }
  // long columns: a warp per (kb, s, root), lanes along the column (coalesced reads of OP)
  const int wid = tid >> 5, lane = tid & 31;
  constexpr int nw = TEAM >> 5;
  const int items = mn * R;
  for (int it = wid; it < items; it += nw) {
    const int r = it / mn, rem = it - r * mn;
    const int s = rem / m, col = rem - s * m;
    const T* o = opg + int64_t(k) * col;
    const T* X = ws + int64_t(2 * r + cur) * stride + int64_t(k) * s;
    T acc = T(0);
    for (int kk = lane; kk < k; kk += 32) acc = fma(o[kk], X[kk], acc);
    for (int w = 16; w > 0; w >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, w);
    if (lane == 0) {
      T* dst = out + int64_t(r) * out_stride + __ldg(bp + rem);
      if (ATOMIC)
        atomicAdd(dst, acc);
      else
        *dst += acc;
    }
  }
}

// Chunks of the groups of one bra block whose R cores fit shared memory: one CTA per
// chunk.  Its warps take the chunk's groups in turn (one group per warp, each warp with a
// slice of `slice` bytes: the group description, then its workspace) and add into
// shared-memory copies of the bra cores -- one private copy per warp when `priv` (plain
// adds), else one shared copy (shared-memory atomics) -- and the CTA adds the sum to sigma.
template <typename T>
__global__ void __launch_bounds__(kBstThreads) bst_sigma_bra_kernel(const int32_t* __restrict__ chunk_bra,
                                                                    const int64_t* __restrict__ chunk_ptr,
                                                                    const int32_t* __restrict__ glist,
                                                                    const BstGroup* __restrict__ groups,
                                                                    const BstBlock* __restrict__ blocks, int R,
                                                                    const T* __restrict__ op,
                                                                    const T* __restrict__ S,
                                                                    const int32_t* __restrict__ perm,
                                                                    const T* __restrict__ cin, T* __restrict__ cout,
                                                                    int64_t core_total, int slice, int priv) {
  extern __shared__ __align__(16) unsigned char bst_smem[];
  constexpr int kWarps = kBstThreads / 32;
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  BstGroup* G = reinterpret_cast<BstGroup*>(bst_smem + size_t(w) * slice);
  T* ws = reinterpret_cast<T*>(bst_smem + size_t(w) * slice + sizeof(BstGroup));
  T* acc = reinterpret_cast<T*>(bst_smem + size_t(kWarps) * slice);
  const BstBlock& B = blocks[chunk_bra[blockIdx.x]];
  const int n = B.core_len;
  const int copies = priv ? kWarps : 1;
  for (int i = threadIdx.x; i < copies * R * n; i += kBstThreads) acc[i] = T(0);
  __syncthreads();
  const int64_t j1 = chunk_ptr[blockIdx.x + 1];
  T* mine = acc + (priv ? size_t(w) * R * n : 0);
  for (int64_t j = chunk_ptr[blockIdx.x] + w; j < j1; j += kWarps) {
    if (j + kWarps < j1) {  // the operator of this warp's next group, to L2
      const BstGroup* nx = groups + glist[j + kWarps];
      prefetch_range<32, false>(op + nx->op_off, int64_t(nx->m) * nx->k * int64_t(sizeof(T)), lane);
    }
    load_group<32>(groups + glist[j], G, lane);
    if (priv)
      bst_group_apply<T, 32, false>(*G, R, op, S, perm, cin, core_total, ws, G->ws, mine, n);
    else
      bst_group_apply<T, 32, true>(*G, R, op, S, perm, cin, core_total, ws, G->ws, mine, n);
    __syncwarp();  // the next description overwrites this one
  }
  __syncthreads();
  for (int i = threadIdx.x; i < R * n; i += kBstThreads) {
    T v = T(0);
    for (int c = 0; c < copies; ++c) v += acc[size_t(c) * R * n + i];
    const int r = i / n, e = i - r * n;
    if (v != T(0)) atomicAdd(cout + int64_t(r) * core_total + B.core_off + e, v);
  }
}

// Medium groups: one CTA per group, description and workspace in shared memory.
template <typename T>
__global__ void __launch_bounds__(kBstThreads) bst_sigma_smem_kernel(const int32_t* __restrict__ list,
                                                                     const BstGroup* __restrict__ groups, int R,
                                                                     const T* __restrict__ op,
                                                                     const T* __restrict__ S,
                                                                     const int32_t* __restrict__ perm,
                                                                     const T* __restrict__ cin, T* __restrict__ cout,
                                                                     int64_t core_total) {
  extern __shared__ __align__(16) unsigned char bst_smem[];
  BstGroup* G = reinterpret_cast<BstGroup*>(bst_smem);
  T* ws = reinterpret_cast<T*>(bst_smem + sizeof(BstGroup));
  load_group<kBstThreads>(groups + list[blockIdx.x], G, threadIdx.x);
  bst_group_apply<T, kBstThreads, true>(*G, R, op, S, perm, cin, core_total, ws, G->ws, cout + G->b_off,
                                        core_total);
}

// Large groups: resident CTAs, each with its own global-memory workspace slice, taking the
// next group of the list (longest first) from a counter until it runs out.
template <typename T>
__global__ void __launch_bounds__(kBstThreads) bst_sigma_global_kernel(const int32_t* __restrict__ list, int n_list,
                                                                       const BstGroup* __restrict__ groups, int R,
                                                                       const T* __restrict__ op,
                                                                       const T* __restrict__ S,
                                                                       const int32_t* __restrict__ perm,
                                                                       const T* __restrict__ cin,
                                                                       T* __restrict__ cout, int64_t core_total,
                                                                       T* __restrict__ ws_all, int stride,
                                                                       unsigned* __restrict__ next) {
  __shared__ __align__(16) BstGroup G;
  __shared__ int s_i;
  T* ws = ws_all + int64_t(blockIdx.x) * 2 * R * stride;
  for (;;) {
    if (threadIdx.x == 0) s_i = int(atomicAdd(next, 1u));
    __syncthreads();
    const int i = s_i;
    if (i >= n_list) return;
    load_group<kBstThreads>(groups + list[i], &G, threadIdx.x);
    bst_group_apply<T, kBstThreads, true>(G, R, op, S, perm, cin, core_total, ws, stride, cout + G.b_off,
                                          core_total);
    __syncthreads();
  }
}


// ---- tensor-core path (float builds) -------------------------------------------------------
// Groups whose product bra[m x ns] += OP^T[m x k] X[k x ns] (per root) is GEMM-shaped run on
// the tcgen05 tensor cores: bst_tc_prep_kernel writes each group's operand X (steps 1-2 of
// bst_group_apply) to a global workspace, then bst_tc_gemm_kernel computes 128 x N tiles of
// D = A B^T with A[i][kk] = OP[kk + k i] and B[j][kk] = X_r[kk + k s] (j = s + ns r, the R
// roots side by side), in three TF32 products per K step (hi*hi + hi*lo + lo*hi, each
// operand split as x = hi + lo) accumulated in FP32 in tensor memory, and adds D into the bra
// cores through the bra's actives-first index table.
struct BstTcJob {
  int32_t tc;  // position in the tensor-core group list
  int32_t g;   // group
  int32_t m0;  // first bra-active row of the tile
  int32_t n0;  // first column (spectator index + ns * root) of the tile
};

constexpr int kTcThreads = 128;  // one warpgroup: thread i owns TMEM lane / tile row i
constexpr int kTcM = 128;        // tile rows (MMA M)
constexpr int kTcN = 256;        // tile columns at most (MMA N, a multiple of 16)
constexpr int kTcK = 16;         // K elements staged per round: two 8-element MMA steps
constexpr int kTcTmemCols = 256;
constexpr int kTcSmem = 2 * (2 * kTcM * kTcK * 4 + 2 * kTcN * kTcK * 4) + 64;  // two stages
constexpr long long kTcWaitCycles = 4000000000LL;  // about 2 s at 2 GHz: a stuck MMA becomes an error
// groups that go to the tensor cores: at least kTcMinM bra-active rows, kTcMinK ket-active
// columns and kTcMinN spectator columns over all roots
constexpr int kTcMinM = 64, kTcMinK = 16, kTcMinN = 32;

__global__ void __launch_bounds__(kBstThreads) bst_tc_prep_kernel(const int32_t* __restrict__ list,
                                                                  const int64_t* __restrict__ ws_off,
                                                                  const BstGroup* __restrict__ groups, int R,
                                                                  const float* __restrict__ S,
                                                                  const int32_t* __restrict__ perm,
                                                                  const float* __restrict__ cin, int64_t core_total,
                                                                  float* __restrict__ ws_all) {
  __shared__ __align__(16) BstGroup G;
  load_group<kBstThreads>(groups + list[blockIdx.x], &G, threadIdx.x);
  bst_group_prepare<float, kBstThreads>(G, R, S, perm, cin, core_total, ws_all + ws_off[blockIdx.x], G.ws);
}

// Two shared-memory stages: while the tensor cores multiply the tiles of one K step (16 K
// elements), the four warps stage the next step into the other stage, split into TF32 high
// and low parts (48 KB per stage: two CTAs per SM).  An mbarrier per stage,
// armed by tcgen05.commit, tells when a stage's MMAs are done and it may be overwritten.
__global__ void __launch_bounds__(kTcThreads, 2) bst_tc_gemm_kernel(const BstTcJob* __restrict__ jobs,
                                                                   const BstGroup* __restrict__ groups, int R,
                                                                   const float* __restrict__ op,
                                                                   const float* __restrict__ ws_all,
                                                                   const int64_t* __restrict__ ws_off,
                                                                   const int32_t* __restrict__ perm,
                                                                   float* __restrict__ cout, int64_t core_total,
                                                                   unsigned* __restrict__ err) {
  extern __shared__ __align__(1024) unsigned char tc_smem[];
  constexpr int kAB = kTcM * kTcK * 4;  // bytes of one A operand copy (hi or lo) of a stage
  constexpr int kBB = kTcN * kTcK * 4;  // bytes of one B operand copy
  constexpr int kStage = 2 * kAB + 2 * kBB;
  uint64_t* bar = reinterpret_cast<uint64_t*>(tc_smem + 2 * kStage);  // one per stage
  uint32_t* tslot = reinterpret_cast<uint32_t*>(bar + 2);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const BstTcJob J = jobs[blockIdx.x];
  const BstGroup& G = groups[J.g];
  const int m = G.m, k = G.k, ns = G.bcore / G.m, NT = ns * R;
  const int rows = min(kTcM, m - J.m0), cols = min(kTcN, NT - J.n0);
  const int nI = (cols + 15) & ~15;  // MMA N
  const int stride = G.ws, cur = G.ntr & 1;
  const float* A = op + G.op_off + int64_t(k) * J.m0;
  const float* X = ws_all + ws_off[J.tc];
  if (warp == 0) tc::tmem_alloc(tc::smem_u32(tslot), kTcTmemCols);
  if (tid == 0) {
    tc::mbar_init(tc::smem_u32(bar), 1);
    tc::mbar_init(tc::smem_u32(bar + 1), 1);
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t taddr = *tslot;
  const uint32_t idesc = tc::idesc_tf32(kTcM, nI);
  uint32_t phase[2] = {0u, 0u};
  bool ok = true;
  const int ntile = (k + kTcK - 1) / kTcK;
  for (int t = 0; t < ntile; ++t) {
    const int st = t & 1, k0 = t * kTcK;
    unsigned char* a_hi = tc_smem + st * kStage;
    unsigned char* a_lo = a_hi + kAB;
    unsigned char* b_hi = a_lo + kAB;
    unsigned char* b_lo = b_hi + kBB;
    if (t >= 2) {  // the MMAs of step t - 2 read this stage
      const bool done = tc::mbar_wait(tc::smem_u32(bar + st), phase[st], kTcWaitCycles);
      phase[st] ^= 1u;
      if (__syncthreads_or(!done)) {
        ok = false;
        break;
      }
    }
    // a warp instruction moves 8 rows x 4 K elements: lane = (row within the group of 8, element
    // within the group of 4), so that its shared-memory stores hit 32 different banks
    const int rl = lane >> 2, ql = lane & 3;
    // A: row groups warp, warp + 4, ...
    for (int rg = warp; rg < kTcM / 8; rg += 4) {
      const int r = 8 * rg + rl;
      const float* src = A + int64_t(k) * r + k0;
#pragma unroll
      for (int q4 = 0; q4 < kTcK / 4; ++q4) {
        const int q = 4 * q4 + ql;
        const float x = (r < rows && k0 + q < k) ? __ldg(src + q) : 0.f;
        float hi, lo;
        tc::split_tf32(x, hi, lo);
        const uint32_t o = uint32_t(q >> 3) * (kTcM * 32) + tc::kmajor_off(r, q & 7);
        *reinterpret_cast<float*>(a_hi + o) = hi;
        *reinterpret_cast<float*>(a_lo + o) = lo;
      }
    }
    // B: rows j = s + ns r (X_r[:, s]) of the tile's columns, in groups of 8
    for (int jg = warp; jg < nI / 8; jg += 4) {
      const int jj = 8 * jg + rl;
      const float* src = nullptr;
      if (jj < cols) {
        const int jp = J.n0 + jj;
        const int r = jp / ns, sidx = jp - r * ns;
        src = X + int64_t(2 * r + cur) * stride + int64_t(k) * sidx + k0;
      }
#pragma unroll
      for (int q4 = 0; q4 < kTcK / 4; ++q4) {
        const int q = 4 * q4 + ql;
        const float x = (src && k0 + q < k) ? __ldg(src + q) : 0.f;
        float hi, lo;
        tc::split_tf32(x, hi, lo);
        const uint32_t o = uint32_t(q >> 3) * (kTcN * 32) + tc::kmajor_off(jj, q & 7);
        *reinterpret_cast<float*>(b_hi + o) = hi;
        *reinterpret_cast<float*>(b_lo + o) = lo;
      }
    }
    tc::fence_proxy_async_smem();
    __syncthreads();
    if (tid == 0) {
      tc::fence_after_sync();
      const int steps = min(kTcK / 8, (k - k0 + 7) / 8);
      for (int q = 0; q < steps; ++q) {
        const uint64_t ah = tc::smem_desc(tc::smem_u32(a_hi + q * kTcM * 32));
        const uint64_t al = tc::smem_desc(tc::smem_u32(a_lo + q * kTcM * 32));
        const uint64_t bh = tc::smem_desc(tc::smem_u32(b_hi + q * kTcN * 32));
        const uint64_t bl = tc::smem_desc(tc::smem_u32(b_lo + q * kTcN * 32));
        tc::mma_tf32(taddr, ah, bh, idesc, (t > 0 || q > 0) ? 1u : 0u);
        tc::mma_tf32(taddr, ah, bl, idesc, 1u);
        tc::mma_tf32(taddr, al, bh, idesc, 1u);
      }
      tc::mma_commit(tc::smem_u32(bar + st));
    }
  }
  // the last one or two steps are still in flight
  if (ok) {
    for (int t = max(0, ntile - 2); t < ntile; ++t) {
      const int st = t & 1;
      const bool done = tc::mbar_wait(tc::smem_u32(bar + st), phase[st], kTcWaitCycles);
      phase[st] ^= 1u;
      if (__syncthreads_or(!done)) {
        ok = false;
        break;
      }
    }
  }
  tc::fence_after_sync();
  if (ok) {
    // epilogue: thread tid holds tile row tid; columns in runs of 16
    const int i = J.m0 + tid;
    const int32_t* bp = perm + G.bperm_off;
    float* outb = cout + G.b_off;
    for (int c0 = 0; c0 < nI; c0 += 16) {
      float v[16];
      tc::tmem_ld16(taddr + (uint32_t(32 * warp) << 16) + uint32_t(c0), v);
      if (tid < rows) {
#pragma unroll
        for (int q = 0; q < 16; ++q) {
          const int col = c0 + q;
          if (col < cols) {
            const int jp = J.n0 + col;
            const int r = jp / ns, sidx = jp - r * ns;
            atomicAdd(outb + int64_t(r) * core_total + __ldg(bp + i + m * sidx), v[q]);
          }
        }
      }
    }
  } else if (tid == 0) {
    atomicExch(err, 1u);  // the host reports it; the context stays usable
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(taddr, kTcTmemCols);
}

// ---- host planning ---------------------------------------------------------------------------

inline int64_t align_up(int64_t x) { return (x + kAlign - 1) / kAlign * kAlign; }

// compute_terms_state_sign (type_ClusteredTerm.jl:181-196) of term t on the ket sector fk (2N int16)
int term_state_sign(const int32_t* r, const int16_t* fk) {
  if (r[0] == 1) return 1;
  int odd = 0;
  for (int o = 0; o < r[0]; ++o)
    if (r[18 + o]) {
      int ne = 0;
      for (int ci = 0; ci < r[2 + o]; ++ci) ne += fk[2 * ci] + fk[2 * ci + 1];
      odd ^= ne & 1;
    }
  return odd ? -1 : 1;
}

struct BstPlan {
  std::vector<BstGamma> gammas;
  std::vector<BstGroupTerm> gterms;
  std::vector<BstGroup> groups;
  std::vector<BstOverlapJob> overlaps;
  std::vector<int32_t> triples;
  std::vector<BstPermTable> tables;  // actives-first index tables, filled on the device
  int64_t perm_total = 0;
  int64_t g_total = 0, op_total = 0, s_total = 0;
  int64_t flops_ref = 0, flops_exec = 0;
};

// The part of a BST plan that one range of bra blocks contributes, with offsets local to the
// part (g_off of its dressed TDMs, op_off of its operators, t_off of its group terms, s_off
// of its overlaps); plan_bst concatenates the parts in bra order and shifts the offsets.
// Everything in a part is keyed by its own bra blocks, so parts are built independently.
struct BstPart {
  std::vector<int32_t> triples;
  std::vector<BstGroup> groups;
  std::vector<std::vector<BstGroupTerm>> gt;   // terms per group
  std::vector<BstGroupTerm> gterms;            // the same, flattened by finish_part
  std::vector<BstGamma> gammas;
  std::vector<BstOverlapJob> overlaps;
  std::unordered_map<uint64_t, int64_t> gamma_at;    // (bra, ket, c, op) -> g offset
  std::unordered_map<uint64_t, int64_t> overlap_at;  // (bra, ket, c) -> S offset
  int64_t g_total = 0, op_total = 0, s_total = 0, flops_ref = 0, flops_exec = 0;
  std::string err;
};

// One (bra, ket, term) triple into its (bra, ket, active clusters) group, with the dressed
// TDMs it needs; grp maps (ket, mask) to the bra block's groups.
std::string add_triple(const fcg_ctx* ctx, const std::vector<BstBlock>& blk, BstPart& P, int64_t b, int32_t k, int t,
                       const int32_t* r, int mask, const int* tdm, int sign,
                       std::unordered_map<uint64_t, int32_t>& grp) {
  const int64_t nb = int64_t(blk.size());
  P.triples.insert(P.triples.end(), {int32_t(b), k, int32_t(t), int32_t(sign)});
  const uint64_t gk = (uint64_t(uint32_t(k)) << 8) | uint64_t(mask);
  auto gi = grp.find(gk);
  int32_t g;
  if (gi == grp.end()) {
    g = int32_t(P.groups.size());
    grp[gk] = g;
    BstGroup G{};
    G.bra = int32_t(b);
    G.ket = k;
    G.act_mask = mask;
    P.groups.push_back(G);
    P.gt.emplace_back();
  } else {
    g = gi->second;
  }
  BstGroupTerm T{};
  T.nact = r[0];
  T.sign = sign;
  T.ints_off = r[0] == 1 ? -1 : ctx->terms[t].ints_off;
  for (int o = 0; o < r[0]; ++o) {
    const int c = r[2 + o];
    const BlockInfo& BI = ctx->h_blocks[tdm[o]];
    if (r[0] > 1 && BI.nidx != r[22 + o]) return "BST: TDM multi-index length differs from the term's ints";
    const uint64_t key = ((uint64_t(b) * uint64_t(nb) + uint64_t(k)) * 8 + uint64_t(c)) * 32 + uint64_t(r[6 + o]);
    auto ga = P.gamma_at.find(key);
    if (ga == P.gamma_at.end()) {
      BstGamma Q{};
      Q.g_off = P.g_total;
      Q.tdm_off = BI.off;
      Q.bra = int32_t(b);
      Q.ket = k;
      Q.c = c;
      Q.np = BI.nidx;
      Q.tdm_mb = BI.mb;
      if (blk[b].start[c] + blk[b].len[c] > BI.mb || blk[k].start[c] + blk[k].len[c] > BI.mk)
        return "BST: a Tucker range exceeds the local basis of its Fock sector";
      P.gammas.push_back(Q);
      ga = P.gamma_at.emplace(key, P.g_total).first;
      P.g_total += align_up(int64_t(BI.nidx) * blk[b].rank[c] * blk[k].rank[c]);
    }
    T.g_off[o] = ga->second;
    T.np[o] = BI.nidx;
  }
  P.gt[g].push_back(T);
  return std::string();
}

// Group operators, spectator overlaps, workspace sizes and flop counts of a part (the
// index-table offsets are left to the merge: tables are shared between parts).
std::string finish_part(const std::vector<BstBlock>& blk, int N, BstPart& P) {
  const int64_t nb = int64_t(blk.size());
  size_t n_terms = 0;
  for (const auto& v : P.gt) n_terms += v.size();
  P.gterms.reserve(n_terms);
  for (size_t g = 0; g < P.groups.size(); ++g) {
    BstGroup& G = P.groups[g];
    const BstBlock& B = blk[G.bra];
    const BstBlock& K = blk[G.ket];
    int64_t m = 1, k = 1, n = 1;
    for (int c = 0; c < N; ++c) {
      if ((G.act_mask >> c) & 1) {
        m *= B.rank[c];
        k *= K.rank[c];
      } else {
        n *= B.rank[c];
      }
    }
    if (m * k > (int64_t(1) << 31)) return "BST: a cached operator exceeds 2^31 elements";
    G.m = int32_t(m);
    G.k = int32_t(k);
    G.op_off = P.op_total;
    P.op_total += align_up(m * k);
    G.t_off = int32_t(P.gterms.size());
    G.nt = int32_t(P.gt[g].size());
    P.gterms.insert(P.gterms.end(), P.gt[g].begin(), P.gt[g].end());
    // core strides and the index description of the rank > 1 clusters
    int64_t kst[kMaxClusters], bst[kMaxClusters];
    {
      int64_t a = 1, b2 = 1;
      for (int c = 0; c < N; ++c) {
        kst[c] = a;
        bst[c] = b2;
        a *= K.rank[c];
        b2 *= B.rank[c];
      }
    }
    G.k_off = K.core_off;
    G.b_off = B.core_off;
    G.kcore = K.core_len;
    G.bcore = B.core_len;
    G.na = 0;
    G.nsp = 0;
    for (int c = 0; c < N; ++c) {
      if (B.rank[c] == 1 && K.rank[c] == 1) continue;
      if ((G.act_mask >> c) & 1) {
        const int a = G.na++;
        G.a_kr[a] = K.rank[c];
        G.a_br[a] = B.rank[c];
        G.a_ks[a] = int32_t(kst[c]);
        G.a_bs[a] = int32_t(bst[c]);
      } else {
        const int j = G.nsp++;
        G.s_kr[j] = K.rank[c];
        G.s_br[j] = B.rank[c];
        G.s_ks[j] = int32_t(kst[c]);
        G.s_bs[j] = int32_t(bst[c]);
      }
    }
    int64_t size = K.core_len, ws = size, tf = 0;
    G.ntr = 0;
    for (int c = 0, j = 0; c < N; ++c) {
      if ((G.act_mask >> c) & 1) continue;
      if (B.rank[c] == 1 && K.rank[c] == 1) continue;
      if (G.bra == G.ket && ((B.ortho >> c) & 1)) {
        // U^T U of an orthonormal factor: the identity up to rounding, not applied
        G.s_off[j++] = -1;
        continue;
      }
      ++G.ntr;
      const uint64_t key = (uint64_t(G.bra) * uint64_t(nb) + uint64_t(G.ket)) * 8 + uint64_t(c);
      auto it = P.overlap_at.find(key);
      if (it == P.overlap_at.end()) {
        P.overlaps.push_back(BstOverlapJob{P.s_total, G.bra, G.ket, c, 0});
        it = P.overlap_at.emplace(key, P.s_total).first;
        P.s_total += align_up(int64_t(B.rank[c]) * K.rank[c]);
      }
      G.s_off[j++] = it->second;
      size = size / K.rank[c] * B.rank[c];
      tf += 2 * size * K.rank[c];
      ws = std::max(ws, size);
    }
    for (int j = G.nsp; j < kMaxClusters; ++j) G.s_off[j] = 0;
    if (ws > (int64_t(1) << 30)) return "BST: a core exceeds 2^30 elements";
    G.ws = int32_t(align_up(ws));
    const int64_t f = 2 * m * k * n + tf;
    P.flops_exec += f;
    P.flops_ref += f * G.nt;
  }
  P.gt.clear();
  P.gt.shrink_to_fit();
  return "";
}

// The triples of build_sigma! (every bra block against every ket block whose Fock sector
// differs by a TransferConfig of H, every term of that transfer with at most nbody clusters
// for which check_term holds on the TuckerConfigs: equal Fock sectors and equal ranges on
// the spectators), grouped by (bra, ket, active clusters).  Ranges of bra blocks are planned
// on host threads and concatenated in bra order, so the plan does not depend on the thread
// count.
std::string plan_bst(const fcg_ctx* ctx, int nbody, const std::vector<BstBlock>& blk, const int16_t* fock,
                     BstPlan& P, const int32_t* given = nullptr, int64_t n_given = 0, int64_t split = 0) {
  const int N = ctx->N;
  const int nmax1 = ctx->nmax + 1;
  const int64_t nb = int64_t(blk.size());
  std::vector<std::vector<int>> by_trans(ctx->n_trans);
  for (int t = 0; t < ctx->n_terms; ++t) {
    const int32_t* r = &ctx->trm[int64_t(t) * kTrmCols];
    if (r[0] <= nbody) by_trans[r[1]].push_back(t);
  }
  // ket lookup per active-cluster mask: hash of (fock, spectator ranges) -> blocks; the
  // candidates of a hash are compared in full before use
  auto mix = [](uint64_t h, uint64_t v) {
    h ^= v + 0x9e3779b97f4a7c15ULL + (h << 6) + (h >> 2);
    return h;
  };
  auto hash_of = [&](int64_t b, const int16_t* f, int mask) {
    uint64_t h = uint64_t(mask) * 0x100000001b3ULL;
    for (int c = 0; c < N; ++c) {
      h = mix(h, uint64_t(uint16_t(f[2 * c])) | (uint64_t(uint16_t(f[2 * c + 1])) << 16));
      if (!((mask >> c) & 1)) h = mix(h, uint64_t(uint32_t(blk[b].start[c])) | (uint64_t(uint32_t(blk[b].len[c])) << 32));
    }
    return h;
  };
  // ket sides: 0 = blocks [0, split), 1 = blocks [split, nb), 2 = all blocks (no split)
  auto in_side = [&](int64_t k, int side) { return side == 2 || ((k < split) == (side == 0)); };
  auto matches = [&](int64_t b, const int16_t* fk, int64_t k, int mask) {
    const int16_t* f = fock + 2 * N * k;
    for (int c = 0; c < N; ++c) {
      if (f[2 * c] != fk[2 * c] || f[2 * c + 1] != fk[2 * c + 1]) return false;
      if (!((mask >> c) & 1) && (blk[k].start[c] != blk[b].start[c] || blk[k].len[c] != blk[b].len[c])) return false;
    }
    return true;
  };
  std::vector<BstPart> parts;
  if (given) {
    // the caller's triples {bra, ket, term}, taken in bra order (the groups of one bra block
    // must be contiguous); each is checked as check_term would
    parts.resize(1);
    BstPart& part = parts[0];
    std::vector<int64_t> order(static_cast<size_t>(n_given));
    for (int64_t q = 0; q < n_given; ++q) order[size_t(q)] = q;
    std::stable_sort(order.begin(), order.end(), [&](int64_t x, int64_t y) { return given[3 * x] < given[3 * y]; });
    std::unordered_map<uint64_t, int32_t> grp;
    int64_t cur_bra = -1;
    for (int64_t q : order) {
      const int32_t* tq = given + 3 * q;
      const int64_t b = tq[0];
      const int32_t k = tq[1];
      const int t = tq[2];
      if (b < 0 || b >= nb || k < 0 || k >= nb || t < 0 || t >= ctx->n_terms) return "BST: a given triple is out of range";
      if (b != cur_bra) {
        grp.clear();
        cur_bra = b;
      }
      const int32_t* r = &ctx->trm[int64_t(t) * kTrmCols];
      if (r[0] > nbody) return "BST: a given triple's term has more than nbody clusters";
      const int16_t* fb = fock + 2 * N * b;
      const int16_t* fkk = fock + 2 * N * k;
      int mask = 0;
      for (int o = 0; o < r[0]; ++o) mask |= 1 << r[2 + o];
      for (int c = 0; c < N; ++c) {
        for (int s2 = 0; s2 < 2; ++s2)
          if (fb[2 * c + s2] - fkk[2 * c + s2] != ctx->trans[(int64_t(r[1]) * N + c) * 2 + s2])
            return "BST: a given triple's Fock sectors do not differ by its term's transfer";
        if (!((mask >> c) & 1) && (blk[b].start[c] != blk[k].start[c] || blk[b].len[c] != blk[k].len[c]))
          return "BST: a given triple fails check_term on the spectator ranges";
      }
      int tdm[4];
      for (int o = 0; o < r[0]; ++o) {
        const int c = r[2 + o];
        tdm[o] = ctx->h_blk_index[dense_block_index(nmax1, c, r[6 + o], fb[2 * c], fb[2 * c + 1], fkk[2 * c],
                                                    fkk[2 * c + 1])];
        if (tdm[o] < 0) return "BST: a given triple needs a TDM block that does not exist";
      }
      std::string msg = add_triple(ctx, blk, part, b, k, t, r, mask, tdm, term_state_sign(r, fkk), grp);
      if (!msg.empty()) return msg;
    }
    std::string msg = finish_part(blk, N, part);
    if (!msg.empty()) return msg;
  } else {
    // Fock sectors present (a transfer into any other sector has no ket), and the ket
    // lookups of every active-cluster mask the terms use, built before the threads read them
    std::unordered_map<uint64_t, int> sectors[3];
    for (int64_t k = 0; k < nb; ++k)
      for (int side = 0; side < 3; ++side)
        if (in_side(k, side)) sectors[side][hash_of(k, fock + 2 * N * k, (1 << N) - 1)] = 1;
    std::unordered_map<int, std::unordered_map<uint64_t, std::vector<int32_t>>> lookup;
    {
      std::vector<int> sides = split > 0 ? std::vector<int>{0, 1} : std::vector<int>{2};
      for (int t = 0; t < ctx->n_terms; ++t) {
        const int32_t* r = &ctx->trm[int64_t(t) * kTrmCols];
        if (r[0] > nbody) continue;
        int mask = 0;
        for (int o = 0; o < r[0]; ++o) mask |= 1 << r[2 + o];
        for (int side : sides) {
          const int key = mask * 4 + side;
          if (lookup.count(key)) continue;
          auto& m = lookup[key];
          for (int64_t k = 0; k < nb; ++k)
            if (in_side(k, side)) m[hash_of(k, fock + 2 * N * k, mask)].push_back(int32_t(k));
        }
      }
    }
    // the transfers with terms whose ket sector exists, once per distinct bra sector (and ket
    // side): blocks of one Fock sector share them
    std::unordered_map<uint64_t, int32_t> bra_sec;      // (fock, side) hash -> list
    std::vector<std::vector<int32_t>> sec_trans;         // list -> transfers
    std::vector<int64_t> sec_first;                      // list -> its first block
    std::vector<int> sec_side;                           // list -> ket side
    std::vector<int32_t> blk_list(size_t(nb), -1);
    for (int64_t b = 0; b < nb; ++b) {  // the list of every block (hash lookups only)
      const int16_t* fb = fock + 2 * N * b;
      const int kside = split > 0 ? (b < split ? 1 : 0) : 2;
      const uint64_t key = mix(hash_of(0, fb, (1 << N) - 1), uint64_t(kside));
      auto it = bra_sec.find(key);
      if (it != bra_sec.end()) {
        // equal hashes of different sectors would share a list: check the sector itself
        const int16_t* f0 = fock + 2 * N * sec_first[size_t(it->second)];
        if (std::equal(fb, fb + 2 * N, f0) && sec_side[size_t(it->second)] == kside) {
          blk_list[size_t(b)] = it->second;
          continue;
        }
      }
      const int32_t id = int32_t(sec_first.size());
      if (it == bra_sec.end()) bra_sec.emplace(key, id);
      sec_first.push_back(b);
      sec_side.push_back(kside);
      blk_list[size_t(b)] = id;
    }
    sec_trans.resize(sec_first.size());
    {  // the lists themselves on host threads
      std::atomic<size_t> next_list{0};
      auto list_worker = [&]() {
        std::vector<int16_t> fk(2 * N);
        for (size_t id = next_list.fetch_add(1); id < sec_first.size(); id = next_list.fetch_add(1)) {
          const int16_t* fb = fock + 2 * N * sec_first[id];
          std::vector<int32_t>& trs = sec_trans[id];
          for (int tr = 0; tr < ctx->n_trans; ++tr) {
            if (by_trans[tr].empty()) continue;
            bool ok = true;
            for (int c = 0; c < N && ok; ++c)
              for (int q = 0; q < 2; ++q) {
                const int v = fb[2 * c + q] - ctx->trans[(int64_t(tr) * N + c) * 2 + q];
                if (v < 0 || v > ctx->norb[c]) ok = false;
                fk[2 * c + q] = int16_t(v);
              }
            if (ok && sectors[sec_side[id]].count(hash_of(0, fk.data(), (1 << N) - 1))) trs.push_back(tr);
          }
        }
      };
      const int n_list_threads = int(std::max<size_t>(1, std::min<size_t>(
          {size_t(std::max(1u, std::thread::hardware_concurrency())), size_t(32), sec_first.size()})));
      std::vector<std::thread> lpool;
      for (int i = 1; i < n_list_threads; ++i) lpool.emplace_back(list_worker);
      list_worker();
      for (auto& th : lpool) th.join();
    }
    constexpr int64_t kBrasPerPart = 16;
    const int64_t n_parts = (nb + kBrasPerPart - 1) / kBrasPerPart;
    parts.resize(size_t(n_parts));
    std::atomic<int64_t> next{0};
    auto worker = [&]() {
      std::vector<int16_t> fk(2 * N);
      for (int64_t q = next.fetch_add(1); q < n_parts; q = next.fetch_add(1)) {
        BstPart& part = parts[size_t(q)];
        const int64_t b1 = std::min(nb, (q + 1) * kBrasPerPart);
        for (int64_t b = q * kBrasPerPart; b < b1 && part.err.empty(); ++b) {
          const int16_t* fb = fock + 2 * N * b;
          const int kside = split > 0 ? (b < split ? 1 : 0) : 2;  // the other state's blocks only
          std::unordered_map<uint64_t, int32_t> grp;              // (ket, mask) -> group
          for (const int32_t tr : sec_trans[size_t(blk_list[size_t(b)])]) {
            if (!part.err.empty()) break;
            for (int c = 0; c < N; ++c)
              for (int s = 0; s < 2; ++s)
                fk[2 * c + s] = int16_t(fb[2 * c + s] - ctx->trans[(int64_t(tr) * N + c) * 2 + s]);
            for (int t : by_trans[tr]) {
              const int32_t* r = &ctx->trm[int64_t(t) * kTrmCols];
              int mask = 0;
              for (int o = 0; o < r[0]; ++o) mask |= 1 << r[2 + o];
              // TDM blocks of the active clusters for this sector pair
              int tdm[4];
              bool have = true;
              for (int o = 0; o < r[0] && have; ++o) {
                const int c = r[2 + o];
                tdm[o] = ctx->h_blk_index[dense_block_index(nmax1, c, r[6 + o], fb[2 * c], fb[2 * c + 1], fk[2 * c],
                                                            fk[2 * c + 1])];
                have = tdm[o] >= 0;
              }
              if (!have) continue;
              const auto& m = lookup.at(mask * 4 + kside);
              auto it = m.find(hash_of(b, fk.data(), mask));
              if (it == m.end()) continue;
              const int sign = term_state_sign(r, fk.data());
              for (int32_t k : it->second) {
                if (!matches(b, fk.data(), k, mask)) continue;
                std::string msg = add_triple(ctx, blk, part, b, k, t, r, mask, tdm, sign, grp);
                if (!msg.empty()) {
                  part.err = msg;
                  break;
                }
              }
              if (!part.err.empty()) break;
            }
          }
        }
        if (part.err.empty()) part.err = finish_part(blk, N, part);
      }
    };
    const int n_threads = int(std::max<int64_t>(1, std::min<int64_t>(
        {int64_t(std::max(1u, std::thread::hardware_concurrency())), int64_t(32), n_parts})));
    std::vector<std::thread> pool;
    for (int i = 1; i < n_threads; ++i) pool.emplace_back(worker);
    worker();
    for (auto& th : pool) th.join();
    for (const BstPart& part : parts)
      if (!part.err.empty()) return part.err;
  }
  // concatenation in bra order; the index tables are shared: each (block, active mask) gets
  // its table where it is first used, as a serial walk over the groups would place it
  {
    size_t n_groups = 0, n_gterms = 0, n_triples = 0, n_gammas = 0, n_ov = 0;
    for (const BstPart& part : parts) {
      n_groups += part.groups.size();
      n_gterms += part.gterms.size();
      n_triples += part.triples.size();
      n_gammas += part.gammas.size();
      n_ov += part.overlaps.size();
    }
    P.groups.reserve(n_groups);
    P.gterms.reserve(n_gterms);
    P.triples.reserve(n_triples);
    P.gammas.reserve(n_gammas);
    P.overlaps.reserve(n_ov);
  }
  std::unordered_map<uint64_t, int64_t> perm_at;  // (block, active mask) -> index table offset
  for (BstPart& part : parts) {
    const int64_t g0 = P.g_total, op0 = P.op_total, s0 = P.s_total, t0 = int64_t(P.gterms.size());
    if (t0 + int64_t(part.gterms.size()) >= (int64_t(1) << 31)) return "BST: more than 2^31 group terms";
    for (BstGamma Q : part.gammas) {
      Q.g_off += g0;
      P.gammas.push_back(Q);
    }
    for (BstGroupTerm T : part.gterms) {
      for (int o = 0; o < T.nact; ++o) T.g_off[o] += g0;
      P.gterms.push_back(T);
    }
    for (BstOverlapJob J : part.overlaps) {
      J.s_off += s0;
      P.overlaps.push_back(J);
    }
    P.triples.insert(P.triples.end(), part.triples.begin(), part.triples.end());
    for (BstGroup G : part.groups) {
      G.op_off += op0;
      G.t_off += int32_t(t0);
      for (int j = 0; j < G.nsp; ++j)
        if (G.s_off[j] >= 0) G.s_off[j] += s0;
      for (int side = 0; side < 2; ++side) {
        const int32_t b = side == 0 ? G.ket : G.bra;
        const uint64_t key = uint64_t(b) * 256 + uint64_t(G.act_mask);
        auto it = perm_at.find(key);
        if (it == perm_at.end()) {
          it = perm_at.emplace(key, P.perm_total).first;
          P.tables.push_back(BstPermTable{P.perm_total, b, G.act_mask});
          P.perm_total += blk[b].core_len;
        }
        (side == 0 ? G.kperm_off : G.bperm_off) = it->second;
      }
      P.groups.push_back(G);
    }
    P.g_total += part.g_total;
    P.op_total += part.op_total;
    P.s_total += part.s_total;
    P.flops_exec += part.flops_exec;
    P.flops_ref += part.flops_ref;
    part = BstPart();  // free the part as it is consumed
  }
  return "";
}

// Every index the sigma kernels form from a group description, checked against the buffers
// it addresses (ket / bra cores, operator cache, overlaps, workspace).
std::string check_groups(const std::vector<BstGroup>& groups, const std::vector<BstBlock>& blk, int64_t core_total,
                         int64_t op_total, int64_t s_total, int64_t perm_total) {
  for (const BstGroup& G : groups) {
    if (G.bra < 0 || G.ket < 0 || size_t(G.bra) >= blk.size() || size_t(G.ket) >= blk.size()) return "BST check: block id";
    const BstBlock& B = blk[G.bra];
    const BstBlock& K = blk[G.ket];
    if (G.kcore != K.core_len || G.bcore != B.core_len || G.k_off != K.core_off || G.b_off != B.core_off)
      return "BST check: core extents";
    if (G.k_off + G.kcore > core_total || G.b_off + G.bcore > core_total) return "BST check: core offsets";
    if (G.na < 0 || G.na > 4 || G.nsp < 0 || G.nsp > kMaxClusters) return "BST check: mode counts";
    int64_t kprod = 1, bprod = 1, ka = 1, ba = 1, kmax = 0, bmax = 0;
    for (int a = 0; a < G.na; ++a) {
      if (G.a_kr[a] < 1 || G.a_br[a] < 1) return "BST check: active ranks";
      ka *= G.a_kr[a];
      ba *= G.a_br[a];
      kmax += int64_t(G.a_kr[a] - 1) * G.a_ks[a];
      bmax += int64_t(G.a_br[a] - 1) * G.a_bs[a];
    }
    kprod = ka;
    bprod = ba;
    int64_t size = G.kcore, ws_need = size;
    for (int j = 0; j < G.nsp; ++j) {
      if (G.s_kr[j] < 1 || G.s_br[j] < 1) return "BST check: spectator ranks";
      kprod *= G.s_kr[j];
      bprod *= G.s_br[j];
      kmax += int64_t(G.s_kr[j] - 1) * G.s_ks[j];
      bmax += int64_t(G.s_br[j] - 1) * G.s_bs[j];
      if (G.s_off[j] == -1) {
        if (G.s_br[j] != G.s_kr[j] || G.bra != G.ket) return "BST check: identity overlap";
      } else if (G.s_off[j] < 0 || G.s_off[j] + int64_t(G.s_br[j]) * G.s_kr[j] > s_total) {
        return "BST check: overlap extent";
      }
      size = size / G.s_kr[j] * G.s_br[j];
      ws_need = std::max(ws_need, size);
    }
    if (ka != G.k || ba != G.m) return "BST check: active products";
    if (kprod != G.kcore || bprod != G.bcore) return "BST check: mode products";
    if (kmax >= G.kcore || bmax >= G.bcore) return "BST check: core strides";
    if (int64_t(G.ws) < ws_need || int64_t(G.k) * (G.bcore / std::max(G.m, 1)) > G.ws) return "BST check: workspace";
    if (G.op_off < 0 || G.op_off + int64_t(G.m) * G.k > op_total) return "BST check: operator extent";
    if (G.kperm_off < 0 || G.kperm_off + G.kcore > perm_total || G.bperm_off < 0 || G.bperm_off + G.bcore > perm_total)
      return "BST check: index-table extent";
    if (int64_t(G.m) * (G.bcore / std::max(G.m, 1)) != G.bcore) return "BST check: bra layout";
  }
  return "";
}

// Groups by where they run.  Groups whose workspace fits a warp slice and whose bra block's
// R cores fit kAccBytes go to bst_sigma_bra_kernel, cut per bra block into chunks of about
// kChunkWork multiply-adds; the others run one CTA per group from shared memory, or from
// global memory.
// multiply-adds and element moves of one group's sigma step, about
int64_t group_work(const BstGroup& G, int R) {
  return int64_t(R) * (int64_t(G.m) * G.k * (G.bcore / std::max(G.m, 1)) + 2 * G.kcore + 64);
}

void bst_lists(fcg_ctx* ctx, int R, size_t elem) {
  ctx->bst_bra_ids.clear();
  ctx->bst_bra_ptr.assign(1, 0);
  ctx->bst_bra_glist.clear();
  ctx->bst_small.clear();
  ctx->bst_large.clear();
  ctx->bst_ws_large = 0;
  ctx->bst_bra_slice = 0;
  ctx->bst_bra_acc = 0;
  ctx->bst_tc.clear();
  ctx->bst_tc_ws_off.clear();
  ctx->bst_tc_jobs.clear();
  ctx->bst_tc_ws_total = 0;
  ctx->bst_tc_flops = 0;
  ctx->bst_tc_mma_flops = 0;
  const size_t ng = ctx->bst_groups.size();
  std::vector<int32_t> bucket[kSmemBuckets];
  std::vector<int64_t> chunk_work;  // per chunk of bst_sigma_bra_kernel
  size_t g = 0;
  while (g < ng) {
    const int32_t b = ctx->bst_groups[g].bra;
    size_t g1 = g;
    while (g1 < ng && ctx->bst_groups[g1].bra == b) ++g1;  // groups of one bra are contiguous
    const size_t acc = size_t(R) * ctx->bst_blocks[b].core_len * elem;
    const bool own = acc <= size_t(kAccBytes);
    int64_t work = 0;
    bool open = false;
    for (size_t q = g; q < g1; ++q) {
      const BstGroup& G = ctx->bst_groups[q];
      const size_t need = sizeof(BstGroup) + size_t(2) * R * G.ws * elem;
      const int64_t ns = G.bcore / std::max(G.m, 1);
      if (elem == 4 && ctx->bst_tc_on && G.m >= kTcMinM && G.k >= kTcMinK && ns * R >= kTcMinN) {
        // GEMM-shaped: tensor cores (its operand X in a global workspace of its own)
        const int32_t tc = int32_t(ctx->bst_tc.size());
        ctx->bst_tc.push_back(int32_t(q));
        ctx->bst_tc_ws_off.push_back(ctx->bst_tc_ws_total);
        ctx->bst_tc_ws_total += int64_t(2) * R * G.ws;
        for (int m0 = 0; m0 < G.m; m0 += kTcM)
          for (int64_t n0 = 0; n0 < ns * R; n0 += kTcN) {
            ctx->bst_tc_jobs.insert(ctx->bst_tc_jobs.end(), {tc, int32_t(q), m0, int32_t(n0)});
            const int64_t nI = (std::min<int64_t>(kTcN, ns * R - n0) + 15) / 16 * 16;
            ctx->bst_tc_mma_flops += 3 * 2 * int64_t(kTcM) * nI * ((G.k + 7) / 8 * 8);
          }
        ctx->bst_tc_flops += 2 * int64_t(G.m) * G.k * ns * R;
        continue;
      }
      if (own && need <= size_t(warp_smem_bytes(elem))) {
        if (!open || work > kChunkWork) {
          if (open) ctx->bst_bra_ptr.push_back(int64_t(ctx->bst_bra_glist.size()));
          ctx->bst_bra_ids.push_back(b);
          chunk_work.push_back(0);
          open = true;
          work = 0;
        }
        ctx->bst_bra_glist.push_back(int32_t(q));
        ctx->bst_bra_slice = std::max(ctx->bst_bra_slice, int((need + 15) / 16 * 16));
        work += group_work(G, R);
        chunk_work.back() += group_work(G, R);
      } else if (need <= size_t(kSigmaSmemBytes)) {
        int i = 0;
        while (need > size_t(kSmemBucket[i])) ++i;
        bucket[i].push_back(int32_t(q));
      } else {
        ctx->bst_large.push_back(int32_t(q));
        ctx->bst_ws_large = std::max(ctx->bst_ws_large, G.ws);
      }
    }
    if (open) {
      ctx->bst_bra_ptr.push_back(int64_t(ctx->bst_bra_glist.size()));
      ctx->bst_bra_acc = std::max(ctx->bst_bra_acc, int((acc + 15) / 16 * 16));
    }
    g = g1;
  }
  // chunks of the warp kernel longest first (CTAs start in launch order)
  {
    const size_t nc = ctx->bst_bra_ids.size();
    std::vector<size_t> order(nc);
    for (size_t i = 0; i < nc; ++i) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](size_t x, size_t y) { return chunk_work[x] > chunk_work[y]; });
    std::vector<int32_t> ids(nc), gl;
    std::vector<int64_t> ptr(1, 0);
    gl.reserve(ctx->bst_bra_glist.size());
    for (size_t i = 0; i < nc; ++i) {
      const size_t c = order[i];
      ids[i] = ctx->bst_bra_ids[c];
      gl.insert(gl.end(), ctx->bst_bra_glist.begin() + ctx->bst_bra_ptr[c],
                ctx->bst_bra_glist.begin() + ctx->bst_bra_ptr[c + 1]);
      ptr.push_back(int64_t(gl.size()));
    }
    ctx->bst_bra_ids.swap(ids);
    ctx->bst_bra_glist.swap(gl);
    ctx->bst_bra_ptr.swap(ptr);
  }
  // longest first: the global-workspace CTAs take the list in order
  std::stable_sort(ctx->bst_large.begin(), ctx->bst_large.end(), [&](int32_t x, int32_t y) {
    return group_work(ctx->bst_groups[x], R) > group_work(ctx->bst_groups[y], R);
  });
  ctx->bst_small_ptr.assign(1, 0);
  for (int i = 0; i < kSmemBuckets; ++i) {
    // CTAs start in launch order: longest first keeps the tail short
    std::stable_sort(bucket[i].begin(), bucket[i].end(), [&](int32_t x, int32_t y) {
      return group_work(ctx->bst_groups[x], R) > group_work(ctx->bst_groups[y], R);
    });
    ctx->bst_small.insert(ctx->bst_small.end(), bucket[i].begin(), bucket[i].end());
    ctx->bst_small_ptr.push_back(int64_t(ctx->bst_small.size()));
  }
}

template <typename T>
int bst_launch(fcg_ctx* ctx, int R, const T* op, const T* S, const T* cin, T* cout, DevBuf<T>& ws) {
  const size_t elem = sizeof(T);
  if (ctx->bst_list_R != R || ctx->bst_list_elem != elem) {
    bst_lists(ctx, R, elem);
    FCG_CUDA(ctx->d_bst_bra_ids.upload(ctx->bst_bra_ids.data(), ctx->bst_bra_ids.size(), ctx->stream));
    FCG_CUDA(ctx->d_bst_bra_ptr.upload(ctx->bst_bra_ptr.data(), ctx->bst_bra_ptr.size(), ctx->stream));
    FCG_CUDA(ctx->d_bst_bra_glist.upload(ctx->bst_bra_glist.data(), ctx->bst_bra_glist.size(), ctx->stream));
    FCG_CUDA(ctx->d_bst_small.upload(ctx->bst_small.data(), ctx->bst_small.size(), ctx->stream));
    FCG_CUDA(ctx->d_bst_large.upload(ctx->bst_large.data(), ctx->bst_large.size(), ctx->stream));
    FCG_CUDA(ctx->d_bst_tc.upload(ctx->bst_tc.data(), ctx->bst_tc.size(), ctx->stream));
    FCG_CUDA(ctx->d_bst_tc_ws_off.upload(ctx->bst_tc_ws_off.data(), ctx->bst_tc_ws_off.size(), ctx->stream));
    FCG_CUDA(ctx->d_bst_tc_jobs.upload(ctx->bst_tc_jobs.data(), ctx->bst_tc_jobs.size(), ctx->stream));
    FCG_CUDA(ctx->d_bst_tc_err.alloc(1));  // set by a tensor-core tile whose MMA wait timed out
    FCG_CUDA(cudaMemsetAsync(ctx->d_bst_tc_err.p, 0, sizeof(unsigned), ctx->stream));
    ctx->bst_list_R = R;
    ctx->bst_list_elem = elem;
  }
  const int64_t ct = ctx->bst_core_total;
  FCG_CUDA(cudaMemsetAsync(cout, 0, elem * size_t(ct) * R, ctx->stream));
  int launches = 1;
  // tensor-core groups (float builds) on the second stream, overlapping the CUDA-core
  // launches below: every kernel adds into the bra cores atomically
  bool forked = false;
  if constexpr (sizeof(T) == 4) {
    if (!ctx->bst_tc.empty()) {
      FCG_REQUIRE(ctx->bst_tc_jobs.size() / 4 < (size_t(1) << 31), FCG_ELIMIT, "too many tensor-core tiles");
      if (!ctx->aux_stream) {
        FCG_CUDA(cudaStreamCreateWithFlags(&ctx->aux_stream, cudaStreamNonBlocking));
        FCG_CUDA(cudaEventCreateWithFlags(&ctx->ev_fork, cudaEventDisableTiming));
        FCG_CUDA(cudaEventCreateWithFlags(&ctx->ev_join, cudaEventDisableTiming));
      }
      cudaStream_t aux = ctx->aux_stream;
      FCG_CUDA(ctx->d_bst_tc_ws.alloc(size_t(ctx->bst_tc_ws_total)));
      FCG_CUDA(cudaEventRecord(ctx->ev_fork, ctx->stream));
      FCG_CUDA(cudaStreamWaitEvent(aux, ctx->ev_fork, 0));
      forked = true;
      bst_tc_prep_kernel<<<unsigned(ctx->bst_tc.size()), kBstThreads, 0, aux>>>(
          ctx->d_bst_tc.p, ctx->d_bst_tc_ws_off.p, ctx->d_bst_groups.p, R, S, ctx->d_bst_perm.p, cin, ct,
          ctx->d_bst_tc_ws.p);
      FCG_CUDA(cudaGetLastError());
      FCG_CUDA(cudaFuncSetAttribute(bst_tc_gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kTcSmem));
      FCG_CUDA(cudaEventRecord(ctx->ev2, aux));
      bst_tc_gemm_kernel<<<unsigned(ctx->bst_tc_jobs.size() / 4), kTcThreads, kTcSmem, aux>>>(
          reinterpret_cast<const BstTcJob*>(ctx->d_bst_tc_jobs.p), ctx->d_bst_groups.p, R, op, ctx->d_bst_tc_ws.p,
          ctx->d_bst_tc_ws_off.p, ctx->d_bst_perm.p, cout, ct, ctx->d_bst_tc_err.p);
      FCG_CUDA(cudaGetLastError());
      FCG_CUDA(cudaEventRecord(ctx->ev3, aux));
      FCG_CUDA(cudaEventRecord(ctx->ev_join, aux));
      launches += 2;
    }
  }
  if (!ctx->bst_bra_ids.empty()) {
    constexpr int kWarps = kBstThreads / 32;
    const int priv = size_t(kWarps) * ctx->bst_bra_acc <= size_t(kAccBytes) ? 1 : 0;
    const size_t smem = size_t(kWarps) * ctx->bst_bra_slice + size_t(priv ? kWarps : 1) * ctx->bst_bra_acc;
    FCG_CUDA(cudaFuncSetAttribute(bst_sigma_bra_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  int(kWarps * kWarpSmemMax + kAccBytes)));
    bst_sigma_bra_kernel<T><<<unsigned(ctx->bst_bra_ids.size()), kBstThreads, smem, ctx->stream>>>(
        ctx->d_bst_bra_ids.p, ctx->d_bst_bra_ptr.p, ctx->d_bst_bra_glist.p, ctx->d_bst_groups.p, ctx->d_bst_blocks.p,
        R, op, S, ctx->d_bst_perm.p, cin, cout, ct, ctx->bst_bra_slice, priv);
    FCG_CUDA(cudaGetLastError());
    ++launches;
  }
  if (!ctx->bst_small.empty()) {
    FCG_CUDA(cudaFuncSetAttribute(bst_sigma_smem_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  int(kSigmaSmemBytes)));
    for (int i = 0; i < kSmemBuckets; ++i) {
      const int64_t a = ctx->bst_small_ptr[i], b = ctx->bst_small_ptr[i + 1];
      if (a == b) continue;
      int ws_max = 0;
      for (int64_t q = a; q < b; ++q) ws_max = std::max(ws_max, ctx->bst_groups[ctx->bst_small[q]].ws);
      const size_t smem = sizeof(BstGroup) + size_t(2) * R * ws_max * elem;
      bst_sigma_smem_kernel<T><<<unsigned(b - a), kBstThreads, smem, ctx->stream>>>(
          ctx->d_bst_small.p + a, ctx->d_bst_groups.p, R, op, S, ctx->d_bst_perm.p, cin, cout, ct);
      FCG_CUDA(cudaGetLastError());
      ++launches;
    }
  }
  if (!ctx->bst_large.empty()) {
    // as many CTAs as can be resident (each walks the list with the grid's stride)
    int per_sm = 1, n_sm = 152;
    FCG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, bst_sigma_global_kernel<T>, kBstThreads, 0));
    FCG_CUDA(cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, ctx->device));
    const int grid = int(std::min<size_t>(ctx->bst_large.size(), size_t(std::max(per_sm, 1)) * n_sm));
    const int64_t stride = ctx->bst_ws_large;
    FCG_CUDA(ws.alloc(size_t(grid) * 2 * R * stride));
    FCG_CUDA(ctx->d_bst_next.alloc(1));
    FCG_CUDA(cudaMemsetAsync(ctx->d_bst_next.p, 0, sizeof(unsigned), ctx->stream));
    bst_sigma_global_kernel<T><<<unsigned(grid), kBstThreads, 0, ctx->stream>>>(
        ctx->d_bst_large.p, int(ctx->bst_large.size()), ctx->d_bst_groups.p, R, op, S, ctx->d_bst_perm.p, cin, cout,
        ct, ws.p, int(stride), ctx->d_bst_next.p);
    FCG_CUDA(cudaGetLastError());
    ++launches;
  }
  if (forked) FCG_CUDA(cudaStreamWaitEvent(ctx->stream, ctx->ev_join, 0));
  ctx->stats.kernel_launches = launches;
  return FCG_OK;
}

}  // namespace

int bst_sigma_device_async(fcg_ctx* ctx, int R, const double* d_cores, double* d_sigma, int precision, bool timed) {
  FCG_REQUIRE(ctx->have_bst, FCG_ESTATE, "fcg_bst_set must come first");
  FCG_REQUIRE(R >= 1 && R <= 64, FCG_ELIMIT, "R must be in [1, 64]");
  FCG_REQUIRE(d_cores && d_sigma, FCG_EINVAL, "null pointer");
  FCG_REQUIRE(precision == FCG_FP64 || precision == FCG_FP32, FCG_EINVAL, "unknown precision");
  int64_t max_core = 0;
  for (const BstBlock& B : ctx->bst_blocks) max_core = std::max<int64_t>(max_core, B.core_len);
  FCG_REQUIRE(max_core * R < (int64_t(1) << 31), FCG_ELIMIT, "R times the largest core must stay below 2^31");
  const int64_t n = ctx->bst_core_total * R;
  ctx->stats.last_kernel_ms = 0.0;
  int rc;
  if (precision == FCG_FP64) {
    if (timed) FCG_CUDA(cudaEventRecord(ctx->ev0, ctx->stream));
    rc = bst_launch<double>(ctx, R, ctx->d_bst_op64.p, ctx->d_bst_s64.p, d_cores, d_sigma, ctx->d_bst_ws64);
    if (rc) return rc;
    if (timed) FCG_CUDA(cudaEventRecord(ctx->ev1, ctx->stream));
  } else {
    FCG_CUDA(ctx->d_bst_in32.alloc(size_t(n)));
    FCG_CUDA(ctx->d_bst_out32.alloc(size_t(n)));
    bst_convert_kernel<<<512, 256, 0, ctx->stream>>>(d_cores, ctx->d_bst_in32.p, n);
    FCG_CUDA(cudaGetLastError());
    if (timed) FCG_CUDA(cudaEventRecord(ctx->ev0, ctx->stream));
    rc = bst_launch<float>(ctx, R, ctx->d_bst_op32.p, ctx->d_bst_s32.p, ctx->d_bst_in32.p, ctx->d_bst_out32.p,
                           ctx->d_bst_ws32);
    if (rc) return rc;
    if (timed) FCG_CUDA(cudaEventRecord(ctx->ev1, ctx->stream));
    bst_widen_kernel<<<512, 256, 0, ctx->stream>>>(ctx->d_bst_out32.p, d_sigma, n);
    FCG_CUDA(cudaGetLastError());
    ctx->stats.kernel_launches += 2;
  }
  return FCG_OK;
}

int bst_tc_check(fcg_ctx* ctx) {
  if (ctx->bst_tc.empty()) return FCG_OK;
  unsigned err = 0;
  FCG_CUDA(cudaMemcpyAsync(&err, ctx->d_bst_tc_err.p, sizeof(unsigned), cudaMemcpyDeviceToHost, ctx->stream));
  FCG_CUDA(cudaStreamSynchronize(ctx->stream));
  if (err) {
    FCG_CUDA(cudaMemsetAsync(ctx->d_bst_tc_err.p, 0, sizeof(unsigned), ctx->stream));
    FCG_CUDA(cudaStreamSynchronize(ctx->stream));
  }
  FCG_REQUIRE(err == 0, FCG_ECUDA, "BST tensor-core tile: the MMA completion wait timed out");
  return FCG_OK;
}

int bst_set_impl(fcg_ctx* ctx, int nbody, int64_t n_blocks, const int16_t* fock, const int64_t* blocks,
                 const int64_t* factor_off, int64_t n_factors, const double* factors, const int32_t* triples,
                 int64_t n_triples, int64_t* core_total, int64_t split) {
  if (!ctx) return FCG_EINVAL;
  FCG_REQUIRE(ctx->have_ops && ctx->have_terms, FCG_ESTATE, "upload ops and terms first");
  FCG_REQUIRE(n_blocks > 0 && fock && blocks && factor_off && factors && core_total && n_factors > 0, FCG_EINVAL,
              "null pointer or empty BST vector");
  FCG_REQUIRE(nbody >= 1 && nbody <= 4, FCG_EINVAL, "nbody must be in [1, 4]");
  FCG_REQUIRE(n_blocks < (int64_t(1) << 24), FCG_ELIMIT, "at most 2^24 Tucker blocks");
  FCG_CUDA(cudaSetDevice(ctx->device));
  const auto t0 = std::chrono::steady_clock::now();
  ctx->have_bst = false;
  const int N = ctx->N;
  std::vector<BstBlock> blk(n_blocks);
  int64_t off = 0;
  for (int64_t b = 0; b < n_blocks; ++b) {
    BstBlock& B = blk[b];
    std::memset(&B, 0, sizeof(B));
    const int64_t* r = blocks + 3 * N * b;
    const int16_t* f = fock + 2 * N * b;
    int64_t len = 1;
    for (int c = 0; c < N; ++c) {
      FCG_REQUIRE(f[2 * c] >= 0 && f[2 * c] <= ctx->norb[c] && f[2 * c + 1] >= 0 && f[2 * c + 1] <= ctx->norb[c],
                  FCG_EINVAL, "BST: bad Fock sector");
      FCG_REQUIRE(r[c] >= 1 && r[2 * N + c] >= 1 && r[c] <= r[2 * N + c] && r[N + c] >= 0 && r[2 * N + c] <= 4096,
                  FCG_EINVAL, "BST: ranks must be in [1, range length] and ranges non-empty");
      FCG_REQUIRE(factor_off[N * b + c] >= 0 && factor_off[N * b + c] + r[c] * r[2 * N + c] <= n_factors, FCG_EINVAL,
                  "BST: factor out of range");
      B.rank[c] = int32_t(r[c]);
      B.start[c] = int32_t(r[N + c]);
      B.len[c] = int32_t(r[2 * N + c]);
      B.factor_off[c] = factor_off[N * b + c];
      len *= r[c];
      // orthonormal columns (U^T U = 1 to 1e-13): a block's overlap with itself is the identity
      {
        const double* U = factors + factor_off[N * b + c];
        const int64_t L = r[2 * N + c], rk = r[c];
        double dev = 0.0;
        for (int64_t x = 0; x < rk; ++x)
          for (int64_t y = 0; y <= x; ++y) {
            double d = 0.0;
            for (int64_t i = 0; i < L; ++i) d += U[i + L * x] * U[i + L * y];
            dev = std::max(dev, std::fabs(d - (x == y ? 1.0 : 0.0)));
          }
        if (dev < 1e-13) B.ortho |= 1 << c;
      }
    }
    FCG_REQUIRE(len < (int64_t(1) << 30), FCG_ELIMIT, "BST: a core exceeds 2^30 elements");
    B.core_off = off;
    B.core_len = int32_t(len);
    off += len;
  }
  BstPlan P;
  {
    std::string msg = plan_bst(ctx, nbody, blk, fock, P, triples, n_triples, split);
    FCG_REQUIRE(msg.empty(), FCG_EINVAL, msg);
  }
  const double plan_s = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  FCG_REQUIRE(P.groups.size() < (size_t(1) << 31), FCG_ELIMIT, "BST: too many groups");
  {
    std::string msg = check_groups(P.groups, blk, off, P.op_total, P.s_total, P.perm_total);
    FCG_REQUIRE(msg.empty(), FCG_EINVAL, msg);
  }
  // device structures and the operator cache
  FCG_CUDA(ctx->d_bst_factors.upload(factors, size_t(n_factors), ctx->stream));
  FCG_CUDA(ctx->d_bst_perm.alloc(size_t(std::max<int64_t>(P.perm_total, 1))));
  FCG_CUDA(ctx->d_bst_blocks.upload(blk.data(), blk.size(), ctx->stream));
  FCG_CUDA(ctx->d_bst_groups.upload(P.groups.data(), P.groups.size(), ctx->stream));
  FCG_REQUIRE(P.tables.size() < (size_t(1) << 31), FCG_ELIMIT, "BST: too many index tables");
  if (!P.tables.empty()) {
    DevBuf<BstPermTable> d_tab;
    FCG_CUDA(d_tab.upload(P.tables.data(), P.tables.size(), ctx->stream));
    bst_perm_kernel<<<unsigned(P.tables.size()), 256, 0, ctx->stream>>>(d_tab.p, ctx->d_bst_blocks.p, N,
                                                                      ctx->d_bst_perm.p);
    FCG_CUDA(cudaGetLastError());
    FCG_CUDA(cudaStreamSynchronize(ctx->stream));  // before d_tab goes
  }
  DevBuf<BstGamma> d_gam;
  DevBuf<BstGroupTerm> d_gt;
  DevBuf<BstOverlapJob> d_ov;
  DevBuf<double> d_g;
  FCG_CUDA(d_gam.upload(P.gammas.data(), P.gammas.size(), ctx->stream));
  FCG_CUDA(d_gt.upload(P.gterms.data(), P.gterms.size(), ctx->stream));
  FCG_CUDA(d_ov.upload(P.overlaps.data(), P.overlaps.size(), ctx->stream));
  FCG_CUDA(d_g.alloc(size_t(std::max<int64_t>(P.g_total, 1))));
  FCG_CUDA(ctx->d_bst_op64.alloc(size_t(std::max<int64_t>(P.op_total, 1))));
  FCG_CUDA(ctx->d_bst_op32.alloc(size_t(std::max<int64_t>(P.op_total, 1))));
  FCG_CUDA(ctx->d_bst_s64.alloc(size_t(std::max<int64_t>(P.s_total, 1))));
  FCG_CUDA(ctx->d_bst_s32.alloc(size_t(std::max<int64_t>(P.s_total, 1))));
  FCG_REQUIRE(P.gammas.size() < (size_t(1) << 31) && P.overlaps.size() < (size_t(1) << 31), FCG_ELIMIT,
              "BST: too many cache jobs");
  if (!P.gammas.empty()) {
    bst_gamma_kernel<<<unsigned(P.gammas.size()), kBstThreads, 0, ctx->stream>>>(
        d_gam.p, ctx->d_bst_blocks.p, ctx->d_op64.p, ctx->d_bst_factors.p, d_g.p);
    FCG_CUDA(cudaGetLastError());
  }
  if (!P.groups.empty()) {
    bst_op_kernel<<<unsigned(P.groups.size()), kOpThreads, 0, ctx->stream>>>(
        ctx->d_bst_groups.p, d_gt.p, ctx->d_bst_blocks.p, N, ctx->d_ints64.p, d_g.p, ctx->d_bst_factors.p,
        ctx->d_bst_op64.p);
    FCG_CUDA(cudaGetLastError());
    bst_convert_kernel<<<1024, 256, 0, ctx->stream>>>(ctx->d_bst_op64.p, ctx->d_bst_op32.p, P.op_total);
    FCG_CUDA(cudaGetLastError());
  }
  if (!P.overlaps.empty()) {
    bst_overlap_kernel<<<unsigned(P.overlaps.size()), 128, 0, ctx->stream>>>(d_ov.p, ctx->d_bst_blocks.p,
                                                                             ctx->d_bst_factors.p, ctx->d_bst_s64.p);
    FCG_CUDA(cudaGetLastError());
    bst_convert_kernel<<<256, 256, 0, ctx->stream>>>(ctx->d_bst_s64.p, ctx->d_bst_s32.p, P.s_total);
    FCG_CUDA(cudaGetLastError());
  }
  FCG_CUDA(cudaStreamSynchronize(ctx->stream));  // before the build-only buffers are freed
  ctx->bst_blocks = std::move(blk);
  ctx->bst_groups = std::move(P.groups);
  ctx->bst_triples = std::move(P.triples);
  ctx->bst_core_total = off;
  ctx->bst_list_R = 0;
  ctx->bst_list_elem = 0;
  *core_total = off;
  ctx->stats.bst_blocks = n_blocks;
  ctx->stats.bst_triples = int64_t(ctx->bst_triples.size() / 4);
  ctx->stats.bst_groups = int64_t(ctx->bst_groups.size());
  ctx->stats.bst_cache_elements = P.op_total;
  ctx->stats.bst_flops_reference = P.flops_ref;
  ctx->stats.bst_flops_executed = P.flops_exec;
  ctx->stats.bst_cache_seconds =
      std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  ctx->stats.bst_plan_seconds = plan_s;
  ctx->have_bst = true;
  return FCG_OK;
}

extern "C" {

int fcg_bst_set(fcg_ctx* ctx, int nbody, int64_t n_blocks, const int16_t* fock, const int64_t* blocks,
                const int64_t* factor_off, int64_t n_factors, const double* factors, int64_t* core_total) {
  return bst_set_impl(ctx, nbody, n_blocks, fock, blocks, factor_off, n_factors, factors, nullptr, 0, core_total, 0);
}

int fcg_bst_set_between(fcg_ctx* ctx, int nbody, int64_t n_first, int64_t n_blocks, const int16_t* fock,
                        const int64_t* blocks, const int64_t* factor_off, int64_t n_factors, const double* factors,
                        int64_t* core_total) {
  if (!ctx) return FCG_EINVAL;
  FCG_REQUIRE(n_first >= 1 && n_first < n_blocks, FCG_EINVAL, "n_first must split the blocks into two states");
  return bst_set_impl(ctx, nbody, n_blocks, fock, blocks, factor_off, n_factors, factors, nullptr, 0, core_total,
                      n_first);
}

int fcg_bst_sigma_device(fcg_ctx* ctx, int R, const double* d_cores, double* d_sigma, int precision) {
  if (!ctx) return FCG_EINVAL;
  FCG_CUDA(cudaSetDevice(ctx->device));
  int rc = bst_sigma_device_async(ctx, R, d_cores, d_sigma, precision, true);
  if (rc) return rc;
  FCG_CUDA(cudaStreamSynchronize(ctx->stream));
  float ms = 0.f;
  FCG_CUDA(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
  ctx->stats.last_kernel_ms = ms;
  ctx->stats.bst_tc_groups = 0;
  ctx->stats.bst_tc_ms = 0.0;
  if (precision == FCG_FP32 && !ctx->bst_tc.empty()) {
    if ((rc = bst_tc_check(ctx))) return rc;
    FCG_CUDA(cudaEventElapsedTime(&ms, ctx->ev2, ctx->ev3));
    ctx->stats.bst_tc_ms = ms;
    ctx->stats.bst_tc_groups = int64_t(ctx->bst_tc.size());
  }
  ctx->stats.bst_tc_flops = precision == FCG_FP32 ? ctx->bst_tc_flops : 0;
  ctx->stats.bst_tc_mma_flops = precision == FCG_FP32 ? ctx->bst_tc_mma_flops : 0;
  return FCG_OK;
}

int fcg_bst_tensor_cores(fcg_ctx* ctx, int enable) {
  if (!ctx) return FCG_EINVAL;
  ctx->bst_tc_on = enable != 0;
  ctx->bst_list_R = 0;  // the group lists are made again on the next sigma
  return FCG_OK;
}

int fcg_bst_sigma(fcg_ctx* ctx, int R, const double* cores, double* sigma, int precision) {
  if (!ctx) return FCG_EINVAL;
  FCG_REQUIRE(ctx->have_bst, FCG_ESTATE, "fcg_bst_set must come first");
  FCG_REQUIRE(R >= 1 && R <= 64, FCG_ELIMIT, "R must be in [1, 64]");
  FCG_REQUIRE(cores && sigma, FCG_EINVAL, "null pointer");
  FCG_CUDA(cudaSetDevice(ctx->device));
  const size_t n = size_t(ctx->bst_core_total) * R;
  FCG_CUDA(ctx->d_bst_in64.upload(cores, n, ctx->stream));
  FCG_CUDA(ctx->d_bst_out64.alloc(n));
  int rc = fcg_bst_sigma_device(ctx, R, ctx->d_bst_in64.p, ctx->d_bst_out64.p, precision);
  if (rc) return rc;
  FCG_CUDA(cudaMemcpyAsync(sigma, ctx->d_bst_out64.p, n * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  FCG_CUDA(cudaStreamSynchronize(ctx->stream));
  return FCG_OK;
}

int fcg_bst_triples(fcg_ctx* ctx, int32_t* out) {
  if (!ctx) return FCG_EINVAL;
  FCG_REQUIRE(ctx->have_bst, FCG_ESTATE, "fcg_bst_set must come first");
  FCG_REQUIRE(out || ctx->bst_triples.empty(), FCG_EINVAL, "null pointer");
  if (!ctx->bst_triples.empty()) std::memcpy(out, ctx->bst_triples.data(), ctx->bst_triples.size() * sizeof(int32_t));
  return FCG_OK;
}

}  // extern "C"
