// CPU oracle for the TPSCI sigma build: TEST INFRASTRUCTURE ONLY.
//
// A plain FP64 restatement of FermiCG's sigma loops, used by the tests, by
// __graft_entry__.smoke() and by bench.py's CPU-baseline leg as the checker
// and as the timed CPU reference.  Nothing in the product links or calls it.
//
// It follows the reference's loop structure one-for-one:
//   closed sigma   tps_ci_matvec            src/tpsci_outer.jl:462-527
//                  check_term               src/type_ClusteredTerm.jl:92-176
//                  compute_terms_state_sign src/type_ClusteredTerm.jl:181-196
//                  contract_matrix_element  src/tpsci_inner.jl:10-216, _contract :270-329
//   diagonal       compute_diagonal         src/tpsci_outer.jl:694-715 (H terms)
//                  compute_diagonal!        src/tpsci_outer.jl:735-757 (op string)
//   open sigma     open_matvec_thread       src/tpsci_matvec_thread.jl:11-129 (job filter :26-56)
//                  _open_matvec_thread_job  :233-263
//                  contract_matvec_thread   1B :279-323, 2B :337-399, 3B :415-572, 4B :587-818
//                  _collect_significant_thread! :830-885
//                  (prescreen bounds upper_bound_thread / upper_bound2_thread :897-1284
//                   are pure skips of contributions below the threshold; this
//                   oracle runs with prescreen off, which keeps every result)
//
// Flat inputs are the layout documented in fermicg_gb300/pack.py.
// Coefficient matrices are column-major (n_cfg x R), as Julia passes them.

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <map>
#include <unordered_map>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

constexpr int OPB_COLS = 10;
constexpr int TRM_COLS = 28;

struct Problem {
  int N = 0;
  std::vector<int> norb;
  int nmax = 0;
  int n_ops = 0;
  // op blocks
  std::vector<int64_t> opb;  // n_blocks x OPB_COLS
  const double* opdata = nullptr;
  std::vector<int32_t> blk_index;  // dense (c, op, fba, fbb, fka, fkb) -> block id or -1
  // terms
  int n_terms = 0;
  std::vector<int32_t> trm;  // n_terms x TRM_COLS
  const double* ints = nullptr;
  int n_trans = 0;
  std::vector<int16_t> trans;  // n_trans x N x 2
  std::vector<std::vector<int>> terms_of_trans;

  int64_t bidx(int c, int op, int fba, int fbb, int fka, int fkb) const {
    int s = nmax + 1;
    if (fba < 0 || fbb < 0 || fka < 0 || fkb < 0 || fba > nmax || fbb > nmax || fka > nmax || fkb > nmax)
      return -1;
    return ((((int64_t(c) * n_ops + op) * s + fba) * s + fbb) * s + fka) * s + fkb;
  }
  int block(int c, int op, int fba, int fbb, int fka, int fkb) const {
    int64_t i = bidx(c, op, fba, fbb, fka, fkb);
    return i < 0 ? -1 : blk_index[i];
  }
};

struct State {
  int64_t n = 0;
  const int16_t* fock = nullptr;  // n x N x 2
  const int16_t* cfg = nullptr;   // n x N
  // sectors (contiguous rows)
  std::vector<int64_t> sec_start, sec_count;
  std::map<std::vector<int16_t>, int> sec_of;  // fock key -> sector id
};

std::vector<Problem*> g_probs;  // one per oracle_set_problem call (handle = index)

inline int32_t T(const Problem& P, int t, int col) { return P.trm[int64_t(t) * TRM_COLS + col]; }
inline int64_t TOff(const Problem& P, int t) {
  return int64_t(uint32_t(T(P, t, 26))) | (int64_t(T(P, t, 27)) << 32);
}

int state_sign(const Problem& P, int t, const int16_t* fk) {
  int s = 1;
  int nb = T(P, t, 0);
  for (int o = 0; o < nb; ++o) {
    if (T(P, t, 18 + o) == 1) {
      int c = T(P, t, 2 + o);
      int ne = 0;
      for (int ci = 0; ci < c; ++ci) ne += fk[2 * ci] + fk[2 * ci + 1];
      if (ne % 2) s = -s;
    }
  }
  return s;
}

bool check_term(const Problem& P, int t, const int16_t* fb, const int16_t* b, const int16_t* fk,
                const int16_t* k) {
  int nb = T(P, t, 0);
  for (int ci = 0; ci < P.N; ++ci) {
    bool active = false;
    for (int o = 0; o < nb; ++o) active |= (T(P, t, 2 + o) == ci);
    if (active) continue;
    if (fb[2 * ci] != fk[2 * ci] || fb[2 * ci + 1] != fk[2 * ci + 1]) return false;
    if (b[ci] != k[ci]) return false;
  }
  for (int o = 0; o < nb; ++o) {
    int c = T(P, t, 2 + o);
    if (fb[2 * c] != fk[2 * c] + T(P, t, 10 + o)) return false;
    if (fb[2 * c + 1] != fk[2 * c + 1] + T(P, t, 14 + o)) return false;
  }
  return true;
}

// contract_matrix_element: returns false when a TDM block is missing (the
// reference returns `nothing` there, tpsci_inner.jl:68-69).
bool matrix_element(const Problem& P, int t, const int16_t* fb, const int16_t* b, const int16_t* fk,
                    const int16_t* k, double* out) {
  int nb = T(P, t, 0);
  const double* g[4];
  int64_t nidx[4];
  for (int o = 0; o < nb; ++o) {
    int c = T(P, t, 2 + o);
    int op = T(P, t, 6 + o);
    int bl = P.block(c, op, fb[2 * c], fb[2 * c + 1], fk[2 * c], fk[2 * c + 1]);
    if (bl < 0) return false;
    const int64_t* r = &P.opb[int64_t(bl) * OPB_COLS];
    int64_t ni = r[6], mb = r[7];
    g[o] = P.opdata + r[9] + ni * (b[c] + mb * k[c]);
    nidx[o] = ni;
  }
  if (nb == 1) {  // 1B: plain lookup, no sign (tpsci_inner.jl:31)
    *out = g[0][0];
    return true;
  }
  const double* v = P.ints + TOff(P, t);
  double me = 0.0;
  if (nb == 2) {
    for (int64_t j = 0; j < nidx[1]; ++j) {
      double tmp = g[1][j];
      for (int64_t i = 0; i < nidx[0]; ++i) me += g[0][i] * v[i + nidx[0] * j] * tmp;
    }
  } else if (nb == 3) {
    for (int64_t kk = 0; kk < nidx[2]; ++kk)
      for (int64_t j = 0; j < nidx[1]; ++j) {
        double tmp = g[1][j] * g[2][kk];
        const double* vv = v + nidx[0] * (j + nidx[1] * kk);
        for (int64_t i = 0; i < nidx[0]; ++i) me += g[0][i] * vv[i] * tmp;
      }
  } else {
    for (int64_t l = 0; l < nidx[3]; ++l)
      for (int64_t kk = 0; kk < nidx[2]; ++kk) {
        double tmp2 = g[2][kk] * g[3][l];
        for (int64_t j = 0; j < nidx[1]; ++j) {
          double tmp = g[1][j] * tmp2;
          const double* vv = v + nidx[0] * (j + nidx[1] * (kk + nidx[2] * l));
          for (int64_t i = 0; i < nidx[0]; ++i) me += g[0][i] * vv[i] * tmp;
        }
      }
  }
  *out = state_sign(P, t, fk) * me;
  return true;
}

void build_sectors(const Problem& P, State& S) {
  S.sec_start.clear();
  S.sec_count.clear();
  S.sec_of.clear();
  std::vector<int16_t> key(2 * P.N);
  for (int64_t i = 0; i < S.n; ++i) {
    std::memcpy(key.data(), S.fock + i * 2 * P.N, sizeof(int16_t) * 2 * P.N);
    bool same = !S.sec_start.empty() &&
                std::memcmp(S.fock + S.sec_start.back() * 2 * P.N, key.data(), sizeof(int16_t) * 2 * P.N) == 0;
    if (same) {
      S.sec_count.back()++;
    } else {
      S.sec_of[key] = int(S.sec_start.size());
      S.sec_start.push_back(i);
      S.sec_count.push_back(1);
    }
  }
}

}  // namespace

extern "C" {

// returns a problem handle (>= 0) used by every other call
int oracle_set_problem(int n_clusters, const int32_t* cluster_norb, int n_ops, int64_t n_blocks,
                       const int64_t* opb, const double* opdata, int n_terms, const int32_t* trm,
                       const double* ints, int n_trans, const int16_t* trans) {
  g_probs.push_back(new Problem());
  Problem& P = *g_probs.back();
  P.N = n_clusters;
  P.norb.assign(cluster_norb, cluster_norb + n_clusters);
  P.nmax = *std::max_element(P.norb.begin(), P.norb.end());
  P.n_ops = n_ops;
  P.opb.assign(opb, opb + n_blocks * OPB_COLS);
  P.opdata = opdata;
  int s = P.nmax + 1;
  P.blk_index.assign(size_t(n_clusters) * n_ops * s * s * s * s, -1);
  for (int64_t b = 0; b < n_blocks; ++b) {
    const int64_t* r = &P.opb[b * OPB_COLS];
    P.blk_index[P.bidx(int(r[0]), int(r[1]), int(r[2]), int(r[3]), int(r[4]), int(r[5]))] = int32_t(b);
  }
  P.n_terms = n_terms;
  P.trm.assign(trm, trm + int64_t(n_terms) * TRM_COLS);
  P.ints = ints;
  P.n_trans = n_trans;
  P.trans.assign(trans, trans + int64_t(n_trans) * n_clusters * 2);
  P.terms_of_trans.assign(n_trans, {});
  for (int t = 0; t < n_terms; ++t) P.terms_of_trans[T(P, t, 1)].push_back(t);
  return int(g_probs.size()) - 1;
}

// tps_ci_matvec (tpsci_outer.jl:462-527): sigma = H c restricted to the configs of c.
// bra rows [row_begin, row_end) only (the full build is [0, n)); sigma rows outside are untouched.
int oracle_sigma_closed(int h, int64_t n_cfg, const int16_t* fock, const int16_t* cfg, int R, const double* c,
                        double* sigma, int64_t row_begin, int64_t row_end, int n_threads) {
  if (h < 0 || h >= int(g_probs.size())) return -1;
  const Problem& P = *g_probs[h];
  State S;
  S.n = n_cfg;
  S.fock = fock;
  S.cfg = cfg;
  build_sectors(P, S);
  const int N = P.N;
#ifdef _OPENMP
  if (n_threads > 0) omp_set_num_threads(n_threads);
#endif
#pragma omp parallel
  {
    std::vector<int16_t> fk(2 * N);
    std::vector<double> acc(R);
#pragma omp for schedule(dynamic, 16)
    for (int64_t ib = row_begin; ib < row_end; ++ib) {
      const int16_t* fb = fock + ib * 2 * N;
      const int16_t* b = cfg + ib * N;
      std::fill(acc.begin(), acc.end(), 0.0);
      for (int tr = 0; tr < P.n_trans; ++tr) {
        const int16_t* tv = &P.trans[int64_t(tr) * N * 2];
        for (int i = 0; i < 2 * N; ++i) fk[i] = int16_t(fb[i] - tv[i]);
        auto it = S.sec_of.find(fk);
        if (it == S.sec_of.end()) continue;
        int64_t ks = S.sec_start[it->second], kn = S.sec_count[it->second];
        for (int64_t ik = ks; ik < ks + kn; ++ik) {
          const int16_t* k = cfg + ik * N;
          for (int t : P.terms_of_trans[tr]) {
            if (!check_term(P, t, fb, b, fk.data(), k)) continue;
            double me;
            if (!matrix_element(P, t, fb, b, fk.data(), k, &me)) continue;
            for (int r = 0; r < R; ++r) acc[r] += me * c[ik + n_cfg * r];
          }
        }
      }
      for (int r = 0; r < R; ++r) sigma[ib + n_cfg * r] = acc[r];
    }
  }
  return 0;
}

// build_full_H (tpsci_outer.jl:10-150): dense H[bra, ket] (row-major n x n) over the configs.
int oracle_build_H(int h, int64_t n_cfg, const int16_t* fock, const int16_t* cfg, double* H) {
  if (h < 0 || h >= int(g_probs.size())) return -1;
  const Problem& P = *g_probs[h];
  State S;
  S.n = n_cfg;
  S.fock = fock;
  S.cfg = cfg;
  build_sectors(P, S);
  const int N = P.N;
#pragma omp parallel
  {
    std::vector<int16_t> fk(2 * N);
#pragma omp for schedule(dynamic, 16)
    for (int64_t ib = 0; ib < n_cfg; ++ib) {
      const int16_t* fb = fock + ib * 2 * N;
      const int16_t* b = cfg + ib * N;
      double* row = H + ib * n_cfg;
      for (int64_t j = 0; j < n_cfg; ++j) row[j] = 0.0;
      for (int tr = 0; tr < P.n_trans; ++tr) {
        const int16_t* tv = &P.trans[int64_t(tr) * N * 2];
        for (int i = 0; i < 2 * N; ++i) fk[i] = int16_t(fb[i] - tv[i]);
        auto it = S.sec_of.find(fk);
        if (it == S.sec_of.end()) continue;
        int64_t ks = S.sec_start[it->second], kn = S.sec_count[it->second];
        for (int64_t ik = ks; ik < ks + kn; ++ik) {
          const int16_t* k = cfg + ik * N;
          for (int t : P.terms_of_trans[tr]) {
            if (!check_term(P, t, fb, b, fk.data(), k)) continue;
            double me;
            if (!matrix_element(P, t, fb, b, fk.data(), k, &me)) continue;
            row[ik] += me;
          }
        }
      }
    }
  }
  return 0;
}

// compute_diagonal (tpsci_outer.jl:694-715): sum of zero-transfer terms with bra == ket.
int oracle_diagonal_H(int h, int64_t n_cfg, const int16_t* fock, const int16_t* cfg, double* hd) {
  if (h < 0 || h >= int(g_probs.size())) return -1;
  const Problem& P = *g_probs[h];
  const int N = P.N;
  int zero = -1;
  for (int tr = 0; tr < P.n_trans; ++tr) {
    bool z = true;
    for (int i = 0; i < 2 * N; ++i) z &= P.trans[int64_t(tr) * 2 * N + i] == 0;
    if (z) zero = tr;
  }
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n_cfg; ++i) {
    double s = 0.0;
    if (zero >= 0)
      for (int t : P.terms_of_trans[zero]) {
        double me;
        if (matrix_element(P, t, fock + i * 2 * N, cfg + i * N, fock + i * 2 * N, cfg + i * N, &me)) s += me;
      }
    hd[i] = s;
  }
  return 0;
}

// compute_diagonal! with an op string (tpsci_outer.jl:735-757): sum_c diag(op_c)[cfg_c].
int oracle_diagonal_op(int h, int64_t n_cfg, const int16_t* fock, const int16_t* cfg, int op, double* hd) {
  if (h < 0 || h >= int(g_probs.size())) return -1;
  const Problem& P = *g_probs[h];
  const int N = P.N;
  for (int64_t i = 0; i < n_cfg; ++i) {
    double s = 0.0;
    for (int c = 0; c < N; ++c) {
      int fa = fock[(i * N + c) * 2], fbb = fock[(i * N + c) * 2 + 1];
      int bl = P.block(c, op, fa, fbb, fa, fbb);
      if (bl < 0) return -2;
      const int64_t* r = &P.opb[int64_t(bl) * OPB_COLS];
      int st = cfg[i * N + c];
      s += P.opdata[r[9] + st + r[7] * st];
    }
    hd[i] = s;
  }
  return 0;
}

// ---------------------------------------------------------------------------
// open sigma (FOIS), tpsci_matvec_thread.jl:11-885 with prescreen off.
// Output: an unordered set of (fock, cfg) -> R coefficients, retrieved with
// oracle_open_fetch after oracle_sigma_open returns the row count.
namespace {
struct Key {
  std::vector<int16_t> v;  // fock (2N) then cfg (N)
  bool operator==(const Key& o) const { return v == o.v; }
};
struct KeyHash {
  size_t operator()(const Key& k) const {
    uint64_t h = 1469598103934665603ull;
    for (int16_t x : k.v) {
      h ^= uint16_t(x);
      h *= 1099511628211ull;
    }
    return size_t(h);
  }
};
using OutMap = std::unordered_map<Key, std::vector<double>, KeyHash>;
std::vector<Key> g_open_keys;
std::vector<double> g_open_vals;
int g_open_R = 0;

struct OpenCtx {
  const Problem* P;
  int R;
  double thresh;
  OutMap* out;
  std::vector<int16_t> fb;  // bra fock
  Key tmp;
};

inline void collect(OpenCtx& X, const int16_t* cfg_ket, const int16_t* fbra, int ca, int cb_, int nI, int nJ,
                    const double* x, int ldx, const double* coeff, int sign, bool one_index) {
  // _collect_significant_thread! (:830-885): keep |x| > thresh / max|c|
  const int N = X.P->N;
  double mx = 0.0;
  for (int r = 0; r < X.R; ++r) mx = std::max(mx, std::fabs(coeff[r]));
  double tc = X.thresh / mx;
  X.tmp.v.resize(3 * N);
  std::memcpy(X.tmp.v.data(), fbra, sizeof(int16_t) * 2 * N);
  std::memcpy(X.tmp.v.data() + 2 * N, cfg_ket, sizeof(int16_t) * N);
  for (int j = 0; j < nJ; ++j) {
    if (!one_index) X.tmp.v[2 * N + cb_] = int16_t(j);
    for (int i = 0; i < nI; ++i) {
      double v = x[i + ldx * j];
      bool keep = one_index ? (v > tc || v < -tc) : (std::fabs(v) > tc);
      if (!keep) continue;
      X.tmp.v[2 * N + ca] = int16_t(i);
      auto it = X.out->find(X.tmp);
      if (it == X.out->end()) it = X.out->emplace(X.tmp, std::vector<double>(X.R, 0.0)).first;
      for (int r = 0; r < X.R; ++r) it->second[r] += sign * v * coeff[r];
    }
  }
}

void open_contract(OpenCtx& X, int t, const int16_t* fbra, const int16_t* fket, const int16_t* kcfg,
                   const double* coeff, std::vector<double>& s1, std::vector<double>& s2,
                   std::vector<double>& s3, std::vector<double>& s4) {
  const Problem& P = *X.P;
  int nb = T(P, t, 0);
  int cl[4], bl[4];
  int64_t ni[4], mb[4], mk[4];
  const double* g[4];
  for (int o = 0; o < nb; ++o) {
    int c = T(P, t, 2 + o);
    cl[o] = c;
    bl[o] = P.block(c, T(P, t, 6 + o), fbra[2 * c], fbra[2 * c + 1], fket[2 * c], fket[2 * c + 1]);
    if (bl[o] < 0) return;  // haskey(...) || return
    const int64_t* r = &P.opb[int64_t(bl[o]) * OPB_COLS];
    ni[o] = r[6];
    mb[o] = r[7];
    mk[o] = r[8];
    // gamma[:, :, k] : (ni, mb) slab for the ket state
    g[o] = P.opdata + r[9] + ni[o] * mb[o] * kcfg[c];
  }
  int sign = state_sign(P, t, fket);
  if (nb == 1) {
    // x_i = s * H[i, k]
    s1.resize(mb[0]);
    for (int64_t i = 0; i < mb[0]; ++i) s1[i] = g[0][i] * sign;
    collect(X, kcfg, fbra, cl[0], -1, int(mb[0]), 1, s1.data(), int(mb[0]), coeff, 1, true);
    return;
  }
  const double* v = P.ints + TOff(P, t);
  if (nb == 2) {
    // scr1(q, I) = sum_p ints[p,q] G1[p,I];  X(I,J) = sum_q scr1(q,I) G2[q,J]
    int64_t np = ni[0], nq = ni[1];
    s1.assign(nq * mb[0], 0.0);
    for (int64_t I = 0; I < mb[0]; ++I)
      for (int64_t q = 0; q < nq; ++q) {
        double a = 0.0;
        for (int64_t p = 0; p < np; ++p) a += v[p + np * q] * g[0][p + np * I];
        s1[q + nq * I] = a;
      }
    s2.assign(mb[0] * mb[1], 0.0);
    for (int64_t J = 0; J < mb[1]; ++J)
      for (int64_t I = 0; I < mb[0]; ++I) {
        double a = 0.0;
        for (int64_t q = 0; q < nq; ++q) a += s1[q + nq * I] * g[1][q + nq * J];
        s2[I + mb[0] * J] = a;
      }
    collect(X, kcfg, fbra, cl[0], cl[1], int(mb[0]), int(mb[1]), s2.data(), int(mb[0]), coeff, sign, false);
    return;
  }
  std::vector<int16_t> kc(kcfg, kcfg + P.N);
  if (nb == 3) {
    int64_t np = ni[0], nq = ni[1], nr = ni[2];
    s1.resize(np * nq);
    s2.resize(np * mb[1]);
    s3.resize(mb[0] * mb[1]);
    for (int64_t K = 0; K < mb[2]; ++K) {
      const double* g3 = g[2] + nr * K;
      kc[cl[2]] = int16_t(K);
      for (int64_t pq = 0; pq < np * nq; ++pq) {
        double a = 0.0;
        for (int64_t r = 0; r < nr; ++r) a += v[pq + np * nq * r] * g3[r];
        s1[pq] = a;
      }
      for (int64_t J = 0; J < mb[1]; ++J)
        for (int64_t p = 0; p < np; ++p) {
          double a = 0.0;
          for (int64_t q = 0; q < nq; ++q) a += s1[p + np * q] * g[1][q + nq * J];
          s2[p + np * J] = a;
        }
      for (int64_t J = 0; J < mb[1]; ++J)
        for (int64_t I = 0; I < mb[0]; ++I) {
          double a = 0.0;
          for (int64_t p = 0; p < np; ++p) a += g[0][p + np * I] * s2[p + np * J];
          s3[I + mb[0] * J] = a;
        }
      collect(X, kc.data(), fbra, cl[0], cl[1], int(mb[0]), int(mb[1]), s3.data(), int(mb[0]), coeff, sign,
              false);
    }
    return;
  }
  // 4B
  int64_t np = ni[0], nq = ni[1], nr = ni[2], ns = ni[3];
  s1.resize(np * nq * nr);
  s2.resize(np * nq);
  s3.resize(np * mb[1]);
  s4.resize(mb[0] * mb[1]);
  for (int64_t L = 0; L < mb[3]; ++L) {
    const double* g4 = g[3] + ns * L;
    kc[cl[3]] = int16_t(L);
    for (int64_t pqr = 0; pqr < np * nq * nr; ++pqr) {
      double a = 0.0;
      for (int64_t s = 0; s < ns; ++s) a += v[pqr + np * nq * nr * s] * g4[s];
      s1[pqr] = a;
    }
    for (int64_t K = 0; K < mb[2]; ++K) {
      const double* g3 = g[2] + nr * K;
      kc[cl[2]] = int16_t(K);
      for (int64_t pq = 0; pq < np * nq; ++pq) {
        double a = 0.0;
        for (int64_t r = 0; r < nr; ++r) a += s1[pq + np * nq * r] * g3[r];
        s2[pq] = a;
      }
      for (int64_t J = 0; J < mb[1]; ++J)
        for (int64_t p = 0; p < np; ++p) {
          double a = 0.0;
          for (int64_t q = 0; q < nq; ++q) a += s2[p + np * q] * g[1][q + nq * J];
          s3[p + np * J] = a;
        }
      for (int64_t J = 0; J < mb[1]; ++J)
        for (int64_t I = 0; I < mb[0]; ++I) {
          double a = 0.0;
          for (int64_t p = 0; p < np; ++p) a += g[0][p + np * I] * s3[p + np * J];
          s4[I + mb[0] * J] = a;
        }
      collect(X, kc.data(), fbra, cl[0], cl[1], int(mb[0]), int(mb[1]), s4.data(), int(mb[0]), coeff, sign,
              false);
    }
  }
}
}  // namespace

// open_matvec_thread: returns the number of output configurations (or < 0 on error).
// ket rows [row_begin, row_end) only contribute (the full build is [0, n)).
int64_t oracle_sigma_open(int h, int64_t n_cfg, const int16_t* fock, const int16_t* cfg, int R, const double* c,
                          double thresh, int nbody, int64_t row_begin, int64_t row_end, int n_threads) {
  if (h < 0 || h >= int(g_probs.size())) return -1;
  const Problem& P = *g_probs[h];
  const int N = P.N;
  State S;
  S.n = n_cfg;
  S.fock = fock;
  S.cfg = cfg;
  build_sectors(P, S);
  // jobs: fock_bra -> list of (transfer, ket sector)   (:26-56)
  std::map<std::vector<int16_t>, std::vector<std::pair<int, int>>> jobs;
  for (size_t ks = 0; ks < S.sec_start.size(); ++ks) {
    const int16_t* fk = fock + S.sec_start[ks] * 2 * N;
    for (int tr = 0; tr < P.n_trans; ++tr) {
      std::vector<int16_t> fb(2 * N);
      bool ok = true;
      for (int i = 0; i < 2 * N; ++i) fb[i] = int16_t(fk[i] + P.trans[int64_t(tr) * 2 * N + i]);
      for (int ci = 0; ci < N && ok; ++ci) {
        if (fb[2 * ci] < 0 || fb[2 * ci + 1] < 0 || fb[2 * ci] > P.norb[ci] || fb[2 * ci + 1] > P.norb[ci])
          ok = false;
      }
      if (!ok) continue;
      for (int ci = 0; ci < N && ok; ++ci)
        if (P.block(ci, P.n_ops - 2, fb[2 * ci], fb[2 * ci + 1], fb[2 * ci], fb[2 * ci + 1]) < 0) ok = false;
      if (!ok) continue;
      jobs[fb].push_back({tr, int(ks)});
    }
  }
  std::vector<std::pair<std::vector<int16_t>, std::vector<std::pair<int, int>>>> jv(jobs.begin(), jobs.end());
#ifdef _OPENMP
  if (n_threads > 0) omp_set_num_threads(n_threads);
#endif
  int nthr = 1;
#ifdef _OPENMP
  nthr = omp_get_max_threads();
#endif
  std::vector<OutMap> outs(nthr);
#pragma omp parallel
  {
    int tid = 0;
#ifdef _OPENMP
    tid = omp_get_thread_num();
#endif
    OpenCtx X;
    X.P = &P;
    X.R = R;
    X.thresh = thresh;
    X.out = &outs[tid];
    std::vector<double> s1, s2, s3, s4, cf(R);
#pragma omp for schedule(dynamic, 1)
    for (int64_t j = 0; j < int64_t(jv.size()); ++j) {
      const std::vector<int16_t>& fb = jv[j].first;
      for (auto& job : jv[j].second) {
        int tr = job.first;
        int64_t ks = S.sec_start[job.second], kn = S.sec_count[job.second];
        const int16_t* fk = fock + ks * 2 * N;
        for (int t : P.terms_of_trans[tr]) {
          if (T(P, t, 0) > nbody) continue;
          for (int64_t ik = std::max(ks, row_begin); ik < std::min(ks + kn, row_end); ++ik) {
            for (int r = 0; r < R; ++r) cf[r] = c[ik + n_cfg * r];
            open_contract(X, t, fb.data(), fk, cfg + ik * N, cf.data(), s1, s2, s3, s4);
          }
        }
      }
    }
  }
  g_open_keys.clear();
  g_open_vals.clear();
  g_open_R = R;
  for (auto& m : outs)
    for (auto& kv : m) {
      g_open_keys.push_back(kv.first);
      g_open_vals.insert(g_open_vals.end(), kv.second.begin(), kv.second.end());
    }
  return int64_t(g_open_keys.size());
}

// rows of the last open sigma: fock (n x N x 2), cfg (n x N), coeff (n x R row-major)
int oracle_open_fetch(int h, int16_t* fock, int16_t* cfg, double* coeff) {
  if (h < 0 || h >= int(g_probs.size())) return -1;
  const int N = g_probs[h]->N;
  for (size_t i = 0; i < g_open_keys.size(); ++i) {
    std::memcpy(fock + i * 2 * N, g_open_keys[i].v.data(), sizeof(int16_t) * 2 * N);
    std::memcpy(cfg + i * N, g_open_keys[i].v.data() + 2 * N, sizeof(int16_t) * N);
  }
  std::memcpy(coeff, g_open_vals.data(), sizeof(double) * g_open_vals.size());
  return 0;
}

}  // extern "C"
