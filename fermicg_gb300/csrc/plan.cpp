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
// triples that all pass check_term.  Each bra row of a work item, with up to
// 32 of its kets, becomes one lane job of the sigma kernel; lane jobs are
// sorted so that a warp's 32 lanes do the same kind and amount of work.
#include <algorithm>
#include <array>
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

// A lane job while planning: its term shape (nbody) and planner cost ride along for the sort.
struct PJob {
  LaneJob j;
  int32_t cost;
  int32_t nbody;
};

}  // namespace

TermTables term_tables(const ProblemInfo& pi) {
  return TermTables{pi.trm->data(), pi.dress->data(), pi.w_index->data(), pi.blk_index->data(), pi.blocks->data(),
                    pi.nmax + 1};
}

bool make_term_sector(const ProblemInfo& pi, int t, const int16_t* fb, const int16_t* fk, TermSector& ts) {
  int64_t fma;
  return term_sector_of(term_tables(pi), t, fb, fk, ts, &fma);
}

std::string term_lists(const ProblemInfo& pi, TermLists& L) {
  const std::vector<int32_t>& trm = *pi.trm;
  L = TermLists();
  std::unordered_map<uint32_t, int> mask_id;
  // (transfer, set, term) of every term; sets numbered in order of first appearance
  std::vector<std::array<int32_t, 3>> key(size_t(pi.n_terms));
  for (int t = 0; t < pi.n_terms; ++t) {
    const int nb = TT(trm, t, 0);
    uint32_t m = 0;
    for (int o = 0; o < nb; ++o) m |= 1u << TT(trm, t, 2 + o);
    auto it = mask_id.find(m);
    int s;
    if (it == mask_id.end()) {
      s = int(L.masks.size());
      mask_id[m] = s;
      L.masks.push_back(m);
    } else {
      s = it->second;
    }
    const int tr = TT(trm, t, 1);
    if (tr < 0 || tr >= pi.n_trans) return "term transfer id out of range";
    key[size_t(t)] = {tr, s, t};
  }
  std::stable_sort(key.begin(), key.end(), [](const std::array<int32_t, 3>& x, const std::array<int32_t, 3>& y) {
    return x[0] != y[0] ? x[0] < y[0] : x[1] < y[1];
  });
  L.first_of_tr.assign(size_t(pi.n_trans) + 1, 0);
  L.off.push_back(0);
  size_t q = 0;
  for (int tr = 0; tr < pi.n_trans; ++tr) {
    L.first_of_tr[tr] = int32_t(L.tr.size());
    while (q < key.size() && key[q][0] == tr) {
      const int s = key[q][1];
      L.tr.push_back(tr);
      L.set.push_back(s);
      for (; q < key.size() && key[q][0] == tr && key[q][1] == s; ++q) L.terms.push_back(key[q][2]);
      L.off.push_back(int32_t(L.terms.size()));
    }
  }
  L.first_of_tr[pi.n_trans] = int32_t(L.tr.size());
  return "";
}

std::vector<int32_t> zero_transfer_terms(const ProblemInfo& pi) {
  // 1-body terms of the zero transfer (compute_diagonal, src/tpsci_outer.jl:694-715)
  std::vector<int32_t> out;
  for (int tr = 0; tr < pi.n_trans; ++tr) {
    bool zero = true;
    for (int i = 0; i < 2 * pi.N; ++i) zero &= (*pi.trans)[size_t(tr) * 2 * pi.N + i] == 0;
    if (zero)
      for (int t = 0; t < pi.n_terms; ++t)
        if (TT(*pi.trm, t, 1) == tr) out.push_back(t);
  }
  return out;
}

std::string build_sectors(const ProblemInfo& pi, int64_t n_cfg, const int16_t* fock, const int16_t* cfg, Plan& P) {
  const int N = pi.N;
  const std::vector<int32_t>& trm = *pi.trm;
  const int n_terms = pi.n_terms;
  const std::vector<int16_t>& trans = *pi.trans;
  const int n_trans = pi.n_trans;
  const int nmax1 = pi.nmax + 1;
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
  for (int64_t i = 0; i < n_cfg; ++i)
    for (int c = 0; c < N; ++c) {
      int fa = fock[(i * N + c) * 2], fbb = fock[(i * N + c) * 2 + 1];
      if (fa > pi.norb[c] || fbb > pi.norb[c]) return "Fock sector exceeds cluster size";
      int bl = (*pi.blk_index)[dense_block_index(nmax1, c, kOpH, fa, fbb, fa, fbb)];
      if (bl < 0) return "a row uses a Fock sector with no local basis";
      if (cfg[i * N + c] >= (*pi.blocks)[bl].mb) return "local state index beyond the sector's basis";
    }
  P.zero_terms = zero_transfer_terms(pi);
  return "";
}

std::string build_join(const ProblemInfo& pi, const int16_t* fock, const int16_t* cfg, Plan& P) {
  (void)fock;
  const int N = pi.N;
  const std::vector<int32_t>& trm = *pi.trm;
  const int n_terms = pi.n_terms;
  const std::vector<int16_t>& trans = *pi.trans;
  const int n_trans = pi.n_trans;
  const int64_t n_sec = int64_t(P.sec_start.size());
  std::unordered_map<uint64_t, int32_t> sec_of;
  for (int64_t sct = 0; sct < n_sec; ++sct) {
    uint64_t k;
    fock_key(&P.sec_fock[size_t(sct) * 2 * N], N, &k);
    sec_of[k] = int32_t(sct);
  }

  TermLists L;
  {
    const std::string m = term_lists(pi, L);
    if (!m.empty()) return m;
  }
  const std::vector<uint32_t>& masks = L.masks;
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
  // items and term-sector records are collected per bra sector and concatenated in
  // sector order, so the plan (and the kernel's summation order) does not depend on
  // thread timing
  std::vector<std::vector<WorkItem>> tItems(n_sec);
  std::vector<std::vector<TermSector>> tTS(n_sec);
  std::vector<std::vector<PJob>> tJobs(n_sec);
  std::vector<int64_t> tFlop(n_sec, 0), tFlopD(n_sec, 0);
  const TermTables tt = term_tables(pi);
#pragma omp parallel
  {
    std::vector<int16_t> fk(2 * N);
    std::vector<TermSector> tsl;
    std::vector<int64_t> tflop, tflopd;
#pragma omp for schedule(dynamic, 1)
    for (int64_t sb = 0; sb < n_sec; ++sb) {
      const int16_t* fb = &P.sec_fock[sb * 2 * N];
      for (int tr = 0; tr < n_trans; ++tr) {
        if (L.first_of_tr[tr] == L.first_of_tr[tr + 1]) continue;
        for (int i = 0; i < 2 * N; ++i) fk[i] = int16_t(fb[i] - trans[size_t(tr) * 2 * N + i]);
        uint64_t key;
        if (!fock_key(fk.data(), N, &key)) continue;
        auto it = sec_of.find(key);
        if (it == sec_of.end()) continue;
        int64_t sk = it->second;
        for (int j = L.first_of_tr[tr]; j < L.first_of_tr[tr + 1]; ++j) {
          // term-sector records of this (bra sector, ket sector, term list)
          tsl.clear();
          tflop.clear();
          tflopd.clear();
          for (int q = L.off[j]; q < L.off[j + 1]; ++q) {
            const int t = L.terms[q];
            TermSector ts;
            int64_t fma;
            if (!term_sector_of(tt, t, fb, fk.data(), ts, &fma)) continue;  // a missing TDM block contributes nothing
            tflop.push_back(term_ref_flops(trm.data(), t));
            tflopd.push_back(2 * fma);
            tsl.push_back(ts);
          }
          if (tsl.empty()) continue;
          int64_t flop = 0, flopd = 0;
          for (size_t i = 0; i < tsl.size(); ++i) {
            flop += tflop[i];
            flopd += tflopd[i];
          }
          const int32_t ts_off = int32_t(tTS[sb].size());  // relative; rebased at concatenation
          tTS[sb].insert(tTS[sb].end(), tsl.begin(), tsl.end());
          // one lane step (one ket): every term's multiply-adds, about 8 loads and index steps
          // per term, and the coefficient update
          const int64_t step_cost = flopd / 2 + 8 * int64_t(tsl.size()) + 4;
          const int nbody_tl = TT(trm, L.terms[L.off[j]], 0);
          const int set = L.set[j];
          const auto& gb = groups[sb * n_sets + set];
          const auto& gk = groups[sk * n_sets + set];
          int64_t pb = fs_perm_off[sb * n_sets + set], pk = fs_perm_off[sk * n_sets + set];
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
              w.ts_off = ts_off;
              w.nt = int32_t(tsl.size());
              tItems[sb].push_back(w);
              for (int bj = 0; bj < w.nb; ++bj)
                for (int k0 = 0; k0 < w.nk; k0 += kLaneKets) {
                  PJob pj;
                  pj.j.b = P.perm_pool[size_t(w.bra_off) + bj];
                  pj.j.kp = w.ket_off + k0;
                  pj.j.ts_off = w.ts_off;  // relative; rebased at concatenation
                  pj.j.len = uint16_t(std::min(kLaneKets, w.nk - k0));
                  pj.j.nt = uint16_t(w.nt);
                  pj.cost = int32_t(std::min<int64_t>(step_cost * pj.j.len, int64_t(1) << 30));
                  pj.nbody = nbody_tl;
                  tJobs[sb].push_back(pj);
                }
              tFlop[sb] += int64_t(w.nb) * w.nk * flop;
              tFlopD[sb] += int64_t(w.nb) * w.nk * flopd;
              ++a;
              ++b;
            }
          }
        }
      }
    }
  }
  size_t tot = 0, tots = 0;
  for (int64_t sb = 0; sb < n_sec; ++sb) {
    tot += tItems[sb].size();
    tots += tTS[sb].size();
  }
  if (tots >= (size_t(1) << 31)) return "term-sector pool exceeds 2^31 records";
  if (tot >= (size_t(1) << 31)) return "work items exceed 2^31";
  // concatenation in sector order, each sector's part copied by one thread
  std::vector<int64_t> item_off(n_sec + 1, 0), tsp_off(n_sec + 1, 0), job_off(n_sec + 1, 0);
  for (int64_t sb = 0; sb < n_sec; ++sb) {
    item_off[sb + 1] = item_off[sb] + int64_t(tItems[sb].size());
    tsp_off[sb + 1] = tsp_off[sb] + int64_t(tTS[sb].size());
    job_off[sb + 1] = job_off[sb] + int64_t(tJobs[sb].size());
    P.flops_ref += tFlop[sb];
    P.flops_dressed += tFlopD[sb];
  }
  P.items.resize(tot);
  P.ts_pool.resize(tots);
#pragma omp parallel for schedule(dynamic, 8)
  for (int64_t sb = 0; sb < n_sec; ++sb) {
    const int32_t base = int32_t(tsp_off[sb]);
    WorkItem* di = P.items.data() + item_off[sb];
    for (const WorkItem& w : tItems[sb]) {
      *di = w;
      di->ts_off += base;
      ++di;
    }
    std::copy(tTS[sb].begin(), tTS[sb].end(), P.ts_pool.begin() + tsp_off[sb]);
    for (PJob& q : tJobs[sb]) q.j.ts_off += base;
    std::vector<WorkItem>().swap(tItems[sb]);
    std::vector<TermSector>().swap(tTS[sb]);
  }
  // Lane jobs of windows of kSortWindow bra sectors sorted by term shape, then by decreasing
  // cost (ties in planning order: the rows of one work item stay together and share their kets), so that the
  // 32 lanes of a warp run the same code on about the same number of kets.  The last warp task
  // is padded with idle lanes (len 0).
  const int64_t n_jobs = job_off[n_sec];
  const int64_t n_wt = (n_jobs + 31) / 32;  // warp tasks
  P.jobs.resize(size_t(n_wt) * 32);
  for (int64_t i = n_jobs; i < n_wt * 32; ++i) P.jobs[size_t(i)] = LaneJob{0, 0, 0, 0, 0};
  std::vector<int32_t> job_cost(static_cast<size_t>(n_jobs));
  {
    constexpr int64_t kSortWindow = 8;
    const int64_t n_win = (n_sec + kSortWindow - 1) / kSortWindow;
#pragma omp parallel
    {
      std::vector<uint64_t> keys;  // (nbody, decreasing cost, position in the window): one sort key
      std::vector<const PJob*> src;
#pragma omp for schedule(dynamic, 1)
      for (int64_t wdx = 0; wdx < n_win; ++wdx) {
        const int64_t s0 = wdx * kSortWindow, s1 = std::min(n_sec, (wdx + 1) * kSortWindow);
        keys.clear();
        src.clear();
        for (int64_t sb = s0; sb < s1; ++sb)
          for (const PJob& q : tJobs[sb]) {
            const uint64_t c = uint64_t(std::min<int32_t>(q.cost, (1 << 26) - 1));
            keys.push_back((uint64_t(q.nbody) << 58) | (((uint64_t(1) << 26) - 1 - c) << 32) | uint64_t(src.size()));
            src.push_back(&q);
          }
        std::sort(keys.begin(), keys.end());
        const int64_t o = job_off[s0];
        for (size_t i = 0; i < keys.size(); ++i) {
          const PJob& q = *src[size_t(keys[i] & 0xFFFFFFFFu)];
          P.jobs[size_t(o) + i] = q.j;
          job_cost[size_t(o) + i] = q.cost;
        }
        for (int64_t sb = s0; sb < s1; ++sb) std::vector<PJob>().swap(tJobs[sb]);
      }
    }
  }
  P.wt_cost.assign(size_t(n_wt), 0);
  P.wt_len.assign(size_t(n_wt), 0);
#pragma omp parallel for schedule(static)
  for (int64_t w = 0; w < n_wt; ++w) {
    int32_t c = 0, l = 0;
    for (int64_t i = w * 32; i < std::min(n_jobs, w * 32 + 32); ++i) {
      c = std::max(c, job_cost[size_t(i)]);
      l = std::max<int32_t>(l, P.jobs[size_t(i)].len);
    }
    P.wt_cost[size_t(w)] = c;
    P.wt_len[size_t(w)] = l;
  }
  P.task_values = 0;
  for (int32_t l : P.wt_len) P.task_values += 32 * int64_t(l);
  make_chunks(P, kTargetChunks, P.chunk_lo, P.chunk_val);
  P.prefix.assign(P.items.size() + 1, 0);
  for (size_t i = 0; i < P.items.size(); ++i)
    P.prefix[i + 1] = P.prefix[i] + int64_t(P.items[i].nb) * P.items[i].nk * P.items[i].nt;
  P.n_triples = P.prefix.back();
  return "";
}

std::string build_plan(const ProblemInfo& pi, int64_t n_cfg, const int16_t* fock, const int16_t* cfg, Plan& P) {
  std::string m = build_sectors(pi, n_cfg, fock, cfg, P);
  return m.empty() ? build_join(pi, fock, cfg, P) : m;
}

void make_chunks(const Plan& P, int64_t target, std::vector<int64_t>& lo, std::vector<int64_t>& val) {
  // chunk c starts at the first warp task whose cost prefix reaches c times the chunk cost;
  // each chunk holds about 1 / target of the work, within [kMinChunkCost, kChunkCost]
  const int64_t n_wt = int64_t(P.wt_cost.size());
  int64_t total = 0;
  for (int32_t c : P.wt_cost) total += c;
  const int64_t chunk_cost =
      std::max<int64_t>(kMinChunkCost, std::min<int64_t>(kChunkCost, total / std::max<int64_t>(target, 1)));
  const int64_t n_chunks = (total + chunk_cost - 1) / chunk_cost;
  lo.assign(size_t(n_chunks) + 1, n_wt);
  val.assign(size_t(n_chunks) + 1, 0);
  int64_t cum = 0, vals = 0, c = 0;
  for (int64_t i = 0; i < n_wt; ++i) {
    while (c < n_chunks && cum >= c * chunk_cost) {
      lo[size_t(c)] = i;
      val[size_t(c)] = vals;
      ++c;
    }
    cum += P.wt_cost[size_t(i)];
    vals += 32 * int64_t(P.wt_len[size_t(i)]);
  }
  for (; c <= n_chunks; ++c) val[size_t(c)] = vals;
}

std::string build_dress(int N, const std::vector<int>& norb, int nmax, const std::vector<int32_t>& trm, int n_terms,
                        const std::vector<int32_t>& blk_index, const std::vector<BlockInfo>& blocks,
                        const std::vector<TermInfo>& terms, std::vector<TermDress>& dress,
                        std::vector<int64_t>& w_index, std::vector<DressJob>& jobs, int64_t& w_total) {
  (void)N;
  const int s = nmax + 1;
  dress.assign(n_terms, TermDress{});
  w_index.assign(size_t(n_terms) * s * s, -1);
  jobs.clear();
  w_total = 0;
  for (int t = 0; t < n_terms; ++t) {
    const int32_t* r = &trm[int64_t(t) * kTrmCols];
    TermDress& d = dress[t];
    const int nb = r[0];
    if (nb == 1) {
      d.pos = -1;
      d.rest_len = 1;
      d.nrem = 0;
    } else {
      // contract the ints with the cluster of the longest orbital multi-index
      d.pos = 0;
      for (int o = 1; o < nb; ++o)
        if (r[22 + o] > r[22 + d.pos]) d.pos = o;
      d.nrem = nb - 1;
      d.rest_len = 1;
      for (int o = 0, q = 0; o < nb; ++o) {
        if (o == d.pos) continue;
        d.rem_pos[q] = o;
        d.rem_dim[q] = r[22 + o];
        d.rest_len *= r[22 + o];
        ++q;
      }
      if (d.rest_len > 32767) return "dressed index too long";
    }
    const int pos = d.pos < 0 ? 0 : d.pos;
    const int cw = r[2 + pos], opw = r[6 + pos];
    int stride[4];
    stride[0] = 1;
    for (int o = 1; o < 4; ++o) stride[o] = stride[o - 1] * r[22 + o - 1];
    for (int fba = 0; fba <= norb[cw]; ++fba)
      for (int fbb = 0; fbb <= norb[cw]; ++fbb) {
        int fka = fba - r[10 + pos], fkb = fbb - r[14 + pos];
        if (fka < 0 || fkb < 0 || fka > norb[cw] || fkb > norb[cw]) continue;
        int bl = blk_index[dense_block_index(s, cw, opw, fba, fbb, fka, fkb)];
        if (bl < 0) continue;
        const BlockInfo& B = blocks[bl];
        if (nb > 1 && B.nidx != r[22 + pos]) return "term dims do not match the TDM block";
        w_total = (w_total + kAlign - 1) / kAlign * kAlign;  // vector-load alignment of W blocks
        DressJob J{};
        J.w_off = w_total;
        J.g_off = B.off;
        J.ints_off = terms[t].ints_off;
        J.rest_len = d.rest_len;
        J.mb = B.mb;
        J.mk = B.mk;
        J.nq = nb == 1 ? 1 : B.nidx;
        J.stride_q = stride[pos];
        J.nrem = d.nrem;
        for (int q = 0; q < d.nrem; ++q) {
          J.rem_dim[q] = d.rem_dim[q];
          J.rem_stride[q] = stride[d.rem_pos[q]];
        }
        J.one_body = nb == 1;
        jobs.push_back(J);
        w_index[(int64_t(t) * s + fba) * s + fbb] = w_total;
        w_total += int64_t(d.rest_len) * B.mb * B.mk;
      }
  }
  return "";
}

}  // namespace fcg
