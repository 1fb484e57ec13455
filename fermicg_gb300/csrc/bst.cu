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
#include <chrono>
#include <cmath>
#include <cstring>
#include <map>
#include <unordered_map>
#include <vector>

#include "fcg_ctx.cuh"

using namespace fcg;

namespace {

constexpr int kBstThreads = 256;
constexpr int kGammaSmem = 6144;          // doubles of the per-p staging tile of the gamma kernel
constexpr int kSigmaSmemBytes = 96 * 1024;  // shared-memory workspace of the sigma kernel

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
__global__ void __launch_bounds__(kBstThreads) bst_op_kernel(const BstGroup* __restrict__ groups,
                                                             const BstGroupTerm* __restrict__ gterms,
                                                             const BstBlock* __restrict__ blocks, int N,
                                                             const double* __restrict__ ints,
                                                             const double* __restrict__ g,
                                                             const double* __restrict__ factors,
                                                             double* __restrict__ opc) {
  __shared__ double scal;
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

// ---- sigma ---------------------------------------------------------------------------------

// One group, all R roots, by the CTA.  ws holds two buffers of `stride` elements per root.
template <typename T>
__device__ void bst_group_apply(const BstGroup& Gp, const BstBlock& B, const BstBlock& K, int N, int R,
                                const T* __restrict__ op, const T* __restrict__ S, const T* __restrict__ cin,
                                T* __restrict__ cout, int64_t core_total, T* ws, int stride) {
  int d[kMaxClusters];
  for (int c = 0; c < N; ++c) d[c] = K.rank[c];
  // 1. ket cores
  {
    const int n = K.core_len;
    for (int idx = threadIdx.x; idx < R * n; idx += blockDim.x) {
      const int r = idx / n, e = idx - r * n;
      ws[int64_t(2 * r) * stride + e] = cin[int64_t(r) * core_total + K.core_off + e];
    }
  }
  __syncthreads();
  // 2. spectator modes to the bra bases (mode products with S_c = U_bra^T U_ket)
  int cur = 0;
  for (int c = 0; c < N; ++c) {
    if (Gp.s_off[c] < 0) continue;
    int inner = 1, outer = 1;
    for (int c2 = 0; c2 < c; ++c2) inner *= d[c2];
    for (int c2 = c + 1; c2 < N; ++c2) outer *= d[c2];
    const int rb = B.rank[c], rk = d[c];
    const int n = inner * rb * outer;
    const T* Sc = S + Gp.s_off[c];
    for (int idx = threadIdx.x; idx < R * n; idx += blockDim.x) {
      const int r = idx / n, e = idx - r * n;
      const int a = e % inner, j = (e / inner) % rb, o = e / (inner * rb);
      const T* src = ws + int64_t(2 * r + cur) * stride + a + int64_t(inner) * rk * o;
      T s = T(0);
      for (int l = 0; l < rk; ++l) s = fma(Sc[j + rb * l], src[int64_t(inner) * l], s);
      ws[int64_t(2 * r + (cur ^ 1)) * stride + e] = s;
    }
    __syncthreads();
    cur ^= 1;
    d[c] = rb;
  }
  // 3. bra core += OP^T X over the active clusters
  int act[4], na = 0;
  int64_t sx[kMaxClusters];
  {
    int64_t s = 1;
    for (int c = 0; c < N; ++c) {
      sx[c] = s;
      s *= d[c];
      if ((Gp.act_mask >> c) & 1) act[na++] = c;
    }
  }
  int kr[4] = {1, 1, 1, 1};
  int64_t ks[4] = {0, 0, 0, 0};
  for (int a = 0; a < na; ++a) {
    kr[a] = K.rank[act[a]];
    ks[a] = sx[act[a]];
  }
  const int n = B.core_len;
  const T* opg = op + Gp.op_off;
  for (int idx = threadIdx.x; idx < R * n; idx += blockDim.x) {
    const int r = idx / n, e = idx - r * n;
    int rem = e;
    int64_t base = 0, kb = 0, kbm = 1;
    for (int c = 0; c < N; ++c) {
      const int v = rem % B.rank[c];
      rem /= B.rank[c];
      if ((Gp.act_mask >> c) & 1) {
        kb += v * kbm;
        kbm *= B.rank[c];
      } else {
        base += v * sx[c];
      }
    }
    const T* X = ws + int64_t(2 * r + cur) * stride + base;
    const T* o = opg + int64_t(Gp.k) * kb;
    T acc = T(0);
    for (int i3 = 0; i3 < kr[3]; ++i3)
      for (int i2 = 0; i2 < kr[2]; ++i2)
        for (int i1 = 0; i1 < kr[1]; ++i1) {
          const T* xp = X + i1 * ks[1] + i2 * ks[2] + i3 * ks[3];
          for (int i0 = 0; i0 < kr[0]; ++i0) acc = fma(o[i0], xp[i0 * ks[0]], acc);
          o += kr[0];
        }
    atomicAdd(cout + int64_t(r) * core_total + B.core_off + e, acc);
  }
}

// Groups whose two workspace buffers fit shared memory: one CTA per group.
template <typename T>
__global__ void __launch_bounds__(kBstThreads) bst_sigma_smem_kernel(const int32_t* __restrict__ list,
                                                                     const BstGroup* __restrict__ groups,
                                                                     const BstBlock* __restrict__ blocks, int N,
                                                                     int R, const T* __restrict__ op,
                                                                     const T* __restrict__ S,
                                                                     const T* __restrict__ cin, T* __restrict__ cout,
                                                                     int64_t core_total) {
  extern __shared__ __align__(16) unsigned char bst_smem[];
  T* ws = reinterpret_cast<T*>(bst_smem);
  const BstGroup Gp = groups[list[blockIdx.x]];
  bst_group_apply<T>(Gp, blocks[Gp.bra], blocks[Gp.ket], N, R, op, S, cin, cout, core_total, ws, Gp.ws);
}

// The other groups: a grid of CTAs, each with its own global-memory workspace slice,
// walking the list with a stride of the grid size.
template <typename T>
__global__ void __launch_bounds__(kBstThreads) bst_sigma_global_kernel(const int32_t* __restrict__ list, int n_list,
                                                                       const BstGroup* __restrict__ groups,
                                                                       const BstBlock* __restrict__ blocks, int N,
                                                                       int R, const T* __restrict__ op,
                                                                       const T* __restrict__ S,
                                                                       const T* __restrict__ cin,
                                                                       T* __restrict__ cout, int64_t core_total,
                                                                       T* __restrict__ ws_all, int stride) {
  T* ws = ws_all + int64_t(blockIdx.x) * 2 * R * stride;
  for (int i = blockIdx.x; i < n_list; i += gridDim.x) {
    const BstGroup Gp = groups[list[i]];
    bst_group_apply<T>(Gp, blocks[Gp.bra], blocks[Gp.ket], N, R, op, S, cin, cout, core_total, ws, stride);
    __syncthreads();
  }
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
  int64_t g_total = 0, op_total = 0, s_total = 0;
  int64_t flops_ref = 0, flops_exec = 0;
};

// The triples of build_sigma! (every bra block against every ket block whose Fock sector
// differs by a TransferConfig of H, every term of that transfer with at most nbody clusters
// for which check_term holds on the TuckerConfigs: equal Fock sectors and equal ranges on
// the spectators), grouped by (bra, ket, active clusters).
std::string plan_bst(const fcg_ctx* ctx, int nbody, const std::vector<BstBlock>& blk, const int16_t* fock,
                     BstPlan& P) {
  const int N = ctx->N;
  const int nmax1 = ctx->nmax + 1;
  const int64_t nb = int64_t(blk.size());
  std::vector<std::vector<int>> by_trans(ctx->n_trans);
  for (int t = 0; t < ctx->n_terms; ++t) {
    const int32_t* r = &ctx->trm[int64_t(t) * kTrmCols];
    if (r[0] <= nbody) by_trans[r[1]].push_back(t);
  }
  // ket lookup per active-cluster mask: (fock, spectator ranges) -> blocks
  std::map<int, std::map<std::vector<int32_t>, std::vector<int32_t>>> lookup;
  auto key_of = [&](int64_t b, const int16_t* f, int mask) {
    std::vector<int32_t> k(4 * N);
    for (int c = 0; c < N; ++c) {
      k[4 * c] = f[2 * c];
      k[4 * c + 1] = f[2 * c + 1];
      const bool a = (mask >> c) & 1;
      k[4 * c + 2] = a ? -1 : blk[b].start[c];
      k[4 * c + 3] = a ? -1 : blk[b].len[c];
    }
    return k;
  };
  auto kets_of = [&](int mask) -> std::map<std::vector<int32_t>, std::vector<int32_t>>& {
    auto it = lookup.find(mask);
    if (it != lookup.end()) return it->second;
    auto& m = lookup[mask];
    for (int64_t k = 0; k < nb; ++k) m[key_of(k, fock + 2 * N * k, mask)].push_back(int32_t(k));
    return m;
  };
  std::unordered_map<uint64_t, int64_t> gamma_at;   // (bra, ket, c, op) -> g offset
  std::unordered_map<uint64_t, int64_t> overlap_at; // (bra, ket, c) -> S offset
  std::vector<std::vector<BstGroupTerm>> gt;        // terms per group
  std::vector<int16_t> fk(2 * N);
  for (int64_t b = 0; b < nb; ++b) {
    const int16_t* fb = fock + 2 * N * b;
    std::map<std::pair<int32_t, int>, int32_t> grp;  // (ket, mask) -> group
    for (int tr = 0; tr < ctx->n_trans; ++tr) {
      if (by_trans[tr].empty()) continue;
      bool ok = true;
      for (int c = 0; c < N && ok; ++c)
        for (int s = 0; s < 2; ++s) {
          const int v = fb[2 * c + s] - ctx->trans[(int64_t(tr) * N + c) * 2 + s];
          if (v < 0 || v > ctx->norb[c]) ok = false;
          fk[2 * c + s] = int16_t(v);
        }
      if (!ok) continue;
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
        auto& m = kets_of(mask);
        auto it = m.find(key_of(b, fk.data(), mask));
        if (it == m.end()) continue;
        const int sign = term_state_sign(r, fk.data());
        for (int32_t k : it->second) {
          P.triples.insert(P.triples.end(), {int32_t(b), k, int32_t(t), int32_t(sign)});
          auto gi = grp.find({k, mask});
          int32_t g;
          if (gi == grp.end()) {
            g = int32_t(P.groups.size());
            grp[{k, mask}] = g;
            BstGroup G{};
            G.bra = int32_t(b);
            G.ket = k;
            G.act_mask = mask;
            P.groups.push_back(G);
            gt.emplace_back();
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
            auto ga = gamma_at.find(key);
            if (ga == gamma_at.end()) {
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
              ga = gamma_at.emplace(key, P.g_total).first;
              P.g_total += align_up(int64_t(BI.nidx) * blk[b].rank[c] * blk[k].rank[c]);
            }
            T.g_off[o] = ga->second;
            T.np[o] = BI.nidx;
          }
          gt[g].push_back(T);
        }
      }
    }
  }
  // group operators, spectator overlaps, workspace sizes and flop counts
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
    G.nt = int32_t(gt[g].size());
    P.gterms.insert(P.gterms.end(), gt[g].begin(), gt[g].end());
    int64_t size = K.core_len, ws = size, tf = 0;
    for (int c = 0; c < N; ++c) {
      G.s_off[c] = -1;
      if ((G.act_mask >> c) & 1) continue;
      if (B.rank[c] == 1 && K.rank[c] == 1) continue;
      const uint64_t key = (uint64_t(G.bra) * uint64_t(nb) + uint64_t(G.ket)) * 8 + uint64_t(c);
      auto it = overlap_at.find(key);
      if (it == overlap_at.end()) {
        P.overlaps.push_back(BstOverlapJob{P.s_total, G.bra, G.ket, c, 0});
        it = overlap_at.emplace(key, P.s_total).first;
        P.s_total += align_up(int64_t(B.rank[c]) * K.rank[c]);
      }
      G.s_off[c] = it->second;
      size = size / K.rank[c] * B.rank[c];
      tf += 2 * size * K.rank[c];
      ws = std::max(ws, size);
    }
    if (ws > (int64_t(1) << 30)) return "BST: a core exceeds 2^30 elements";
    G.ws = int32_t(align_up(ws));
    const int64_t f = 2 * m * k * n + tf;
    P.flops_exec += f;
    P.flops_ref += f * G.nt;
  }
  return "";
}

// Lists of groups that run from shared memory (two buffers per root fit) and from global memory.
void bst_lists(fcg_ctx* ctx, int R, size_t elem) {
  ctx->bst_small.clear();
  ctx->bst_large.clear();
  ctx->bst_ws_large = 0;
  for (size_t g = 0; g < ctx->bst_groups.size(); ++g) {
    const BstGroup& G = ctx->bst_groups[g];
    if (size_t(2) * R * G.ws * elem <= size_t(kSigmaSmemBytes)) {
      ctx->bst_small.push_back(int32_t(g));
    } else {
      ctx->bst_large.push_back(int32_t(g));
      ctx->bst_ws_large = std::max(ctx->bst_ws_large, G.ws);
    }
  }
}

template <typename T>
int bst_launch(fcg_ctx* ctx, int R, const T* op, const T* S, const T* cin, T* cout, DevBuf<T>& ws) {
  const size_t elem = sizeof(T);
  if (ctx->bst_list_R != R || ctx->bst_list_elem != elem) {
    bst_lists(ctx, R, elem);
    FCG_CUDA(ctx->d_bst_small.upload(ctx->bst_small.data(), ctx->bst_small.size(), ctx->stream));
    FCG_CUDA(ctx->d_bst_large.upload(ctx->bst_large.data(), ctx->bst_large.size(), ctx->stream));
    ctx->bst_list_R = R;
    ctx->bst_list_elem = elem;
  }
  const int N = ctx->N;
  const int64_t ct = ctx->bst_core_total;
  FCG_CUDA(cudaMemsetAsync(cout, 0, elem * size_t(ct) * R, ctx->stream));
  int launches = 1;
  if (!ctx->bst_small.empty()) {
    int ws_max = 0;
    for (int32_t g : ctx->bst_small) ws_max = std::max(ws_max, ctx->bst_groups[g].ws);
    const size_t smem = size_t(2) * R * ws_max * elem;
    FCG_CUDA(cudaFuncSetAttribute(bst_sigma_smem_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  int(kSigmaSmemBytes)));
    bst_sigma_smem_kernel<T><<<unsigned(ctx->bst_small.size()), kBstThreads, smem, ctx->stream>>>(
        ctx->d_bst_small.p, ctx->d_bst_groups.p, ctx->d_bst_blocks.p, N, R, op, S, cin, cout, ct);
    FCG_CUDA(cudaGetLastError());
    ++launches;
  }
  if (!ctx->bst_large.empty()) {
    const int grid = int(std::min<size_t>(ctx->bst_large.size(), 2 * 152));
    const int64_t stride = ctx->bst_ws_large;
    FCG_CUDA(ws.alloc(size_t(grid) * 2 * R * stride));
    bst_sigma_global_kernel<T><<<unsigned(grid), kBstThreads, 0, ctx->stream>>>(
        ctx->d_bst_large.p, int(ctx->bst_large.size()), ctx->d_bst_groups.p, ctx->d_bst_blocks.p, N, R, op, S, cin,
        cout, ct, ws.p, int(stride));
    FCG_CUDA(cudaGetLastError());
    ++launches;
  }
  ctx->stats.kernel_launches = launches;
  return FCG_OK;
}

}  // namespace

extern "C" {

int fcg_bst_set(fcg_ctx* ctx, int nbody, int64_t n_blocks, const int16_t* fock, const int64_t* blocks,
                const int64_t* factor_off, int64_t n_factors, const double* factors, int64_t* core_total) {
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
    }
    FCG_REQUIRE(len < (int64_t(1) << 30), FCG_ELIMIT, "BST: a core exceeds 2^30 elements");
    B.core_off = off;
    B.core_len = int32_t(len);
    off += len;
  }
  BstPlan P;
  {
    std::string msg = plan_bst(ctx, nbody, blk, fock, P);
    FCG_REQUIRE(msg.empty(), FCG_EINVAL, msg);
  }
  FCG_REQUIRE(P.groups.size() < (size_t(1) << 31), FCG_ELIMIT, "BST: too many groups");
  // device structures and the operator cache
  FCG_CUDA(ctx->d_bst_factors.upload(factors, size_t(n_factors), ctx->stream));
  FCG_CUDA(ctx->d_bst_blocks.upload(blk.data(), blk.size(), ctx->stream));
  FCG_CUDA(ctx->d_bst_groups.upload(P.groups.data(), P.groups.size(), ctx->stream));
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
    bst_op_kernel<<<unsigned(P.groups.size()), kBstThreads, 0, ctx->stream>>>(
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
  ctx->have_bst = true;
  return FCG_OK;
}

int fcg_bst_sigma_device(fcg_ctx* ctx, int R, const double* d_cores, double* d_sigma, int precision) {
  if (!ctx) return FCG_EINVAL;
  FCG_REQUIRE(ctx->have_bst, FCG_ESTATE, "fcg_bst_set must come first");
  FCG_REQUIRE(R >= 1 && R <= 64, FCG_ELIMIT, "R must be in [1, 64]");
  FCG_REQUIRE(d_cores && d_sigma, FCG_EINVAL, "null pointer");
  FCG_REQUIRE(precision == FCG_FP64 || precision == FCG_FP32, FCG_EINVAL, "unknown precision");
  FCG_CUDA(cudaSetDevice(ctx->device));
  const int64_t n = ctx->bst_core_total * R;
  ctx->stats.last_kernel_ms = 0.0;
  int rc;
  if (precision == FCG_FP64) {
    FCG_CUDA(cudaEventRecord(ctx->ev0, ctx->stream));
    rc = bst_launch<double>(ctx, R, ctx->d_bst_op64.p, ctx->d_bst_s64.p, d_cores, d_sigma, ctx->d_bst_ws64);
    if (rc) return rc;
    FCG_CUDA(cudaEventRecord(ctx->ev1, ctx->stream));
  } else {
    FCG_CUDA(ctx->d_bst_in32.alloc(size_t(n)));
    FCG_CUDA(ctx->d_bst_out32.alloc(size_t(n)));
    bst_convert_kernel<<<512, 256, 0, ctx->stream>>>(d_cores, ctx->d_bst_in32.p, n);
    FCG_CUDA(cudaGetLastError());
    FCG_CUDA(cudaEventRecord(ctx->ev0, ctx->stream));
    rc = bst_launch<float>(ctx, R, ctx->d_bst_op32.p, ctx->d_bst_s32.p, ctx->d_bst_in32.p, ctx->d_bst_out32.p,
                           ctx->d_bst_ws32);
    if (rc) return rc;
    FCG_CUDA(cudaEventRecord(ctx->ev1, ctx->stream));
    bst_widen_kernel<<<512, 256, 0, ctx->stream>>>(ctx->d_bst_out32.p, d_sigma, n);
    FCG_CUDA(cudaGetLastError());
    ctx->stats.kernel_launches += 2;
  }
  FCG_CUDA(cudaStreamSynchronize(ctx->stream));
  float ms = 0.f;
  FCG_CUDA(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
  ctx->stats.last_kernel_ms = ms;
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
