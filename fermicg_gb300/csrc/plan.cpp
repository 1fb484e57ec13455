// Host planner of the closed sigma (tps_ci_matvec, src/tpsci_outer.jl:462-527).
//
// The reference finds, for every bra, every ket of the sector fock_bra - trans
// and filters them with check_term (src/type_ClusteredTerm.jl:92-176): a ket
// couples through a term iff it equals the bra on every cluster the term does
// not touch.  Here that test is turned into a join: the rows of every
// (Fock sector, active-cluster set) are sorted by their spectator key (the
// local states on the untouched clusters), and for each (bra sector,
// transfer, active set) the bra and ket key lists are merge-joined.  Each
// matching key gives one work item = a dense block of (bra, ket, term)
// triples that all pass check_term.  The kernel walks the flattened triple
// space of all work items.
#include <algorithm>
#include <cstring>
#include <unordered_map>

#include "fcg_internal.h"
#ifdef _OPENMP
#include <omp.h>
#endif

namespace fcg {
namespace {

inline int32_t TT(const std::vector<int32_t>& trm, int t, int col) { return trm[size_t(t) * kTrmCols + col]; }

// Fock sector key: 4 bits per (n_alpha, n_beta) entry; valid for <= 15 electrons/spin/cluster.
inline bool fock_key(const int16_t* f, int N, uint64_t* key) {
  uint64_t k = 0;
  for (int i = 0; i < 2 * N; ++i) {
    if (f[i] < 0 || f[i] > 15) return false;
    k |= uint64_t(f[i]) << (4 * i);
  }
  *key = k;
  return true;
}

struct Group {
  uint64_t key;
  int32_t start;  // relative to the (sector, set) permutation
  int32_t count;
};

}  // namespace

std::string build_plan(int N, const std::vector<int>& norb, const std::vector<int32_t>& trm, int n_terms,
                       const std::vector<int16_t>& trans, int n_trans, int64_t n_cfg, const int16_t* fock,
                       const int16_t* cfg, Plan& P) {
  (void)norb;
  P = Plan();
  P.N = N;
  P.n_cfg = n_cfg;
  if (N > kMaxClusters) return "more than 8 clusters";
  if (n_cfg >= (int64_t(1) << 31)) return "too many configurations";
  // ---- sectors -------------------------------------------------------------
  std::unordered_map<uint64_t, int32_t> sec_of;
  for (int64_t i = 0; i < n_cfg; ++i) {
    const int16_t* f = fock + i * 2 * N;
    bool same = !P.sec_start.empty() &&
                std::memcmp(fock + P.sec_start.back() * 2 * N, f, sizeof(int16_t) * 2 * N) == 0;
    if (same) {
      P.sec_count.back()++;
      continue;
    }
    uint64_t k;
    if (!fock_key(f, N, &k)) return "Fock sector entry outside [0, 15]";
    if (sec_of.count(k)) return "rows of a Fock sector are not contiguous";
    sec_of[k] = int32_t(P.sec_start.size());
    P.sec_start.push_back(i);
    P.sec_count.push_back(1);
    P.sec_fock.insert(P.sec_fock.end(), f, f + 2 * N);
  }
  for (int64_t i = 0; i < n_cfg * N; ++i)
    if (cfg[i] < 0 || cfg[i] > 255) return "local state index outside [0, 255]";
  const int64_t n_sec = int64_t(P.sec_start.size());

  // ---- active sets and term lists per (transfer, set) ----------------------
  std::vector<uint32_t> masks;
  std::unordered_map<uint32_t, int> mask_id;
  struct TL {
    int s;
    int32_t off, n;
    int64_t flop;  // sum over the list of 2*len(ints)
  };
  std::vector<std::vector<TL>> tls(n_trans);
  {
    std::vector<std::vector<std::vector<int32_t>>> by(n_trans);
    for (int t = 0; t < n_terms; ++t) {
      int nb = TT(trm, t, 0);
      uint32_t m = 0;
      for (int o = 0; o < nb; ++o) m |= 1u << TT(trm, t, 2 + o);
      auto it = mask_id.find(m);
      int s;
      if (it == mask_id.end()) {
        s = int(masks.size());
        mask_id[m] = s;
        masks.push_back(m);
      } else {
        s = it->second;
      }
      int tr = TT(trm, t, 1);
      if (tr < 0 || tr >= n_trans) return "term transfer id out of range";
      if (int(by[tr].size()) <= s) by[tr].resize(s + 1);
      by[tr][s].push_back(t);
    }
    for (int tr = 0; tr < n_trans; ++tr)
      for (int s = 0; s < int(by[tr].size()); ++s) {
        if (by[tr][s].empty()) continue;
        TL tl{s, int32_t(P.term_pool.size()), int32_t(by[tr][s].size()), 0};
        for (int t : by[tr][s]) {
          P.term_pool.push_back(t);
          int nb = TT(trm, t, 0);
          int64_t len = 1;
          for (int o = 0; o < 4; ++o) len *= TT(trm, t, 22 + o);
          tl.flop += nb > 1 ? 2 * len : 0;
        }
        tls[tr].push_back(tl);
      }
    for (int tr = 0; tr < n_trans; ++tr) {
      bool zero = true;
      for (int i = 0; i < 2 * N; ++i) zero &= trans[size_t(tr) * 2 * N + i] == 0;
      if (zero)
        for (int t = 0; t < n_terms; ++t)
          if (TT(trm, t, 1) == tr) P.zero_terms.push_back(t);
    }
  }
  const int n_sets = int(masks.size());

  // ---- groups of every (sector, set) -----------------------------------------
  std::vector<int64_t> fs_perm_off(n_sec * n_sets + 1, 0);
  for (int64_t s = 0; s < n_sec; ++s)
    for (int k = 0; k < n_sets; ++k) fs_perm_off[s * n_sets + k + 1] = P.sec_count[s];
  for (int64_t i = 0; i < n_sec * n_sets; ++i) fs_perm_off[i + 1] += fs_perm_off[i];
  if (fs_perm_off.back() >= (int64_t(1) << 31)) return "grouping pool exceeds 2^31 rows";
  P.perm_pool.assign(fs_perm_off.back(), 0);
  std::vector<std::vector<Group>> groups(n_sec * n_sets);
#pragma omp parallel
  {
    std::vector<std::pair<uint64_t, int32_t>> kv;
#pragma omp for schedule(dynamic, 4)
    for (int64_t fs = 0; fs < n_sec * n_sets; ++fs) {
      int64_t s = fs / n_sets;
      uint32_t m = masks[fs % n_sets];
      int64_t st = P.sec_start[s], n = P.sec_count[s];
      kv.resize(n);
      for (int64_t i = 0; i < n; ++i) {
        const int16_t* c = cfg + (st + i) * N;
        uint64_t key = 0;
        for (int ci = 0; ci < N; ++ci)
          if (!((m >> ci) & 1)) key |= uint64_t(uint16_t(c[ci]) & 0xFF) << (8 * ci);
        kv[i] = {key, int32_t(st + i)};
      }
      std::sort(kv.begin(), kv.end());
      int32_t* perm = &P.perm_pool[fs_perm_off[fs]];
      auto& g = groups[fs];
      g.clear();
      for (int64_t i = 0; i < n; ++i) {
        perm[i] = kv[i].second;
        if (i == 0 || kv[i].first != kv[i - 1].first)
          g.push_back({kv[i].first, int32_t(i), 1});
        else
          g.back().count++;
      }
    }
  }

  // ---- work items: merge-join per (bra sector, transfer, set) --------------
  // items are collected per bra sector and concatenated in sector order, so the
  // plan (and the kernel's summation order) does not depend on thread timing
  std::vector<std::vector<WorkItem>> tItems(n_sec);
  std::vector<int64_t> tFlop(n_sec, 0);
#pragma omp parallel
  {
    std::vector<int16_t> fk(2 * N);
#pragma omp for schedule(dynamic, 1)
    for (int64_t sb = 0; sb < n_sec; ++sb) {
      const int16_t* fb = &P.sec_fock[sb * 2 * N];
      for (int tr = 0; tr < n_trans; ++tr) {
        if (tls[tr].empty()) continue;
        for (int i = 0; i < 2 * N; ++i) fk[i] = int16_t(fb[i] - trans[size_t(tr) * 2 * N + i]);
        uint64_t key;
        if (!fock_key(fk.data(), N, &key)) continue;
        auto it = sec_of.find(key);
        if (it == sec_of.end()) continue;
        int64_t sk = it->second;
        for (const TL& tl : tls[tr]) {
          const auto& gb = groups[sb * n_sets + tl.s];
          const auto& gk = groups[sk * n_sets + tl.s];
          int64_t pb = fs_perm_off[sb * n_sets + tl.s], pk = fs_perm_off[sk * n_sets + tl.s];
          size_t a = 0, b = 0;
          while (a < gb.size() && b < gk.size()) {
            if (gb[a].key < gk[b].key) {
              ++a;
            } else if (gk[b].key < gb[a].key) {
              ++b;
            } else {
              WorkItem w;
              w.bra_off = int32_t(pb + gb[a].start);
              w.ket_off = int32_t(pk + gk[b].start);
              w.nb = gb[a].count;
              w.nk = gk[b].count;
              w.tl_off = tl.off;
              w.nt = tl.n;
              w.sb = int32_t(sb);
              w.sk = int32_t(sk);
              tItems[sb].push_back(w);
              tFlop[sb] += int64_t(w.nb) * w.nk * tl.flop;
              ++a;
              ++b;
            }
          }
        }
      }
    }
  }
  size_t tot = 0;
  for (auto& v : tItems) tot += v.size();
  P.items.reserve(tot);
  for (auto& v : tItems) P.items.insert(P.items.end(), v.begin(), v.end());
  for (int64_t f : tFlop) P.flops_ref += f;
  P.prefix.assign(P.items.size() + 1, 0);
  for (size_t i = 0; i < P.items.size(); ++i)
    P.prefix[i + 1] = P.prefix[i] + int64_t(P.items[i].nb) * P.items[i].nk * P.items[i].nt;
  P.n_triples = P.prefix.back();
  return "";
}

}  // namespace fcg
