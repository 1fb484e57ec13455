// The closed-sigma join on the device: build_join (plan.cpp) as kernels, in the same
// enumeration order, so that the permutation pool, the term-sector records, the lane jobs
// and the warp chunks are bit-identical to the host planner's.
//
// tps_ci_matvec (src/tpsci_outer.jl:462-527) finds, for every bra, the kets of the sector
// fock_bra - trans and filters them with check_term (src/type_ClusteredTerm.jl:92-176); its
// index keys are the FockConfig and ClusterConfig of src/type_FockConfig.jl:10,
// src/type_SparseIndex.jl:4-12 and src/Indexing.jl:5-25.  Here:
//  1. spectator keys: every (row, active-cluster set) gets the local states of the clusters
//     outside the set, packed with as many bits per cluster as the cluster's largest local
//     basis needs (the packing keeps the order of the host's 8-bit-per-cluster keys); a
//     stable radix sort by (segment = (sector, set), key) gives the permutation pool and the
//     groups (runs of one key) of every segment;
//  2. sector table: an open-addressed hash table of the sectors' Fock keys gives the ket
//     sector of every (bra sector, transfer);
//  3. term-sector records of every (bra sector, term list) pair whose ket sector exists, one
//     thread per pair, compacted in order;
//  4. join: every bra group of a pair looks its key up among the ket sector's groups (binary
//     search); each match is a work item;
//  5. lane jobs: each bra row of an item with up to 32 of its kets, then a stable radix sort
//     by (window of 8 bra sectors, term shape, decreasing cost): the host's window sort;
//  6. warp tasks (32 lane jobs), the prefix sums of their cost and stored values, and the
//     warp chunks.
// Four host waits read the sizes the next buffers need.
#include <algorithm>

#include "dprim.cuh"
#include "fcg_ctx.cuh"

namespace fcg {
namespace {

constexpr int kThreads = 256;
constexpr int kWindow = 8;  // bra sectors per lane-job sort window
constexpr uint8_t kActive = 255;  // spectator bit offset of a cluster inside the active set

// blocks of t threads covering n (at least one: kernels check their range)
inline unsigned grid_for(int64_t n, int t = kThreads) { return unsigned(std::max<int64_t>((n + t - 1) / t, 1)); }

__device__ __forceinline__ int64_t min64(int64_t a, int64_t b) { return a < b ? a : b; }

inline int bit_width(uint64_t x) {
  int b = 0;
  while (x) {
    ++b;
    x >>= 1;
  }
  return b;
}

__device__ __forceinline__ uint64_t sector_hash(uint64_t k) {
  k *= 0x9E3779B97F4A7C15ull;  // Fibonacci hashing
  return k ^ (k >> 29);
}

// bump allocation of one phase's buffers from a grow-only arena
struct Bump {
  unsigned char* base = nullptr;
  size_t off = 0;
  template <class T>
  T* take(int64_t n) {
    off = (off + 255) & ~size_t(255);
    T* p = reinterpret_cast<T*>(base + off);
    off += size_t(std::max<int64_t>(n, 1)) * sizeof(T);
    return p;
  }
};

template <class F>
cudaError_t carve(DevBuf<unsigned char>& arena, F f) {
  Bump dry;
  f(dry);
  const cudaError_t e = arena.alloc(dry.off);
  if (e != cudaSuccess) return e;
  Bump b{arena.p, 0};
  f(b);
  return cudaSuccess;
}

// ---- 1. spectator keys and groups ----------------------------------------------------------
__global__ void spectator_keys_kernel(int64_t n_cfg, int n_sets, int N, const int16_t* __restrict__ cfg,
                                      const int32_t* __restrict__ row_sector, const int64_t* __restrict__ sec_start,
                                      const int64_t* __restrict__ sec_count, const uint8_t* __restrict__ spec_off,
                                      uint64_t* __restrict__ keys, uint32_t* __restrict__ vals) {
  const int64_t idx = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (idx >= n_cfg * n_sets) return;
  const int64_t i = idx / n_sets;
  const int k = int(idx - i * n_sets);
  const int s = row_sector[i];
  const int64_t st = sec_start[s];
  // the host planner's layout: sector-major, then set, then the sector's rows
  const int64_t e = int64_t(n_sets) * st + int64_t(k) * sec_count[s] + (i - st);
  const uint8_t* so = spec_off + k * kMaxClusters;
  uint64_t key = 0;
  for (int c = 0; c < N; ++c)
    if (so[c] != kActive) key |= uint64_t(uint16_t(cfg[i * kCfgStride + c])) << so[c];
  keys[e] = key;
  vals[e] = uint32_t(idx);  // row * n_sets + set
}

__device__ __forceinline__ int64_t segment_of(uint32_t v, int n_sets, const int32_t* __restrict__ row_sector) {
  return int64_t(row_sector[v / uint32_t(n_sets)]) * n_sets + v % uint32_t(n_sets);
}

// group starts (flag, and a zero past the end for the scan) and the permutation pool
__global__ void group_flags_kernel(int64_t n_el, const uint64_t* __restrict__ keys, const uint32_t* __restrict__ vals,
                                   int n_sets, const int32_t* __restrict__ row_sector, int32_t* __restrict__ perm,
                                   int32_t* __restrict__ flag) {
  const int64_t x = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (x > n_el) return;
  if (x == n_el) {
    flag[x] = 0;
    return;
  }
  const uint32_t v = vals[x];
  bool start = x == 0;
  if (!start)
    start = keys[x] != keys[x - 1] || segment_of(v, n_sets, row_sector) != segment_of(vals[x - 1], n_sets, row_sector);
  flag[x] = start ? 1 : 0;
  perm[x] = int32_t(v / uint32_t(n_sets));
}

// groups: key, first position; the first group of every segment
__global__ void group_fill_kernel(int64_t n_el, const uint64_t* __restrict__ keys, const uint32_t* __restrict__ vals,
                                  int n_sets, const int32_t* __restrict__ row_sector, const int32_t* __restrict__ gid,
                                  uint64_t* __restrict__ g_key, int32_t* __restrict__ g_start,
                                  int64_t* __restrict__ seg_g) {
  const int64_t x = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (x >= n_el) return;
  const int32_t g = gid[x];
  if (gid[x + 1] == g) return;  // not a group start
  g_key[g] = keys[x];
  g_start[g] = int32_t(x);
  const int64_t seg = segment_of(vals[x], n_sets, row_sector);
  if (x == 0 || segment_of(vals[x - 1], n_sets, row_sector) != seg) seg_g[seg] = g;
}

__global__ void group_count_kernel(int64_t n_el, const int32_t* __restrict__ n_groups_at,
                                   const int32_t* __restrict__ g_start, int32_t* __restrict__ g_cnt,
                                   int64_t* __restrict__ seg_g, int64_t n_seg) {
  const int64_t g = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  const int32_t ng = *n_groups_at;
  if (g == 0) seg_g[n_seg] = ng;
  if (g >= ng) return;
  const int64_t end = g + 1 < ng ? g_start[g + 1] : n_el;
  g_cnt[g] = int32_t(end - g_start[g]);
}

// ---- rows of a state ------------------------------------------------------------------
// Checks of the rows, with the host planner's messages (build_sectors in plan.cpp) and its
// order: the first error by (check group, row, cluster), where group 0 is the sector scan
// (an entry outside [0, 15] at a sector's first row, a sector that comes back), group 1 the
// range of the local states, group 2 the per-cluster checks of each row.
enum RowError : int {
  kErrFockRange = 1,
  kErrSplitSector = 2,
  kErrStateRange = 3,
  kErrClusterSize = 4,
  kErrNoBasis = 5,
  kErrBeyondBasis = 6
};

__device__ __forceinline__ unsigned long long row_error(int group, int64_t row, int c, int code) {
  return (static_cast<unsigned long long>(group) << 60) | (static_cast<unsigned long long>(row) << 8) |
         (static_cast<unsigned long long>(c) << 4) | static_cast<unsigned long long>(code);
}

// per row: sector start flag (and a zero past the end for the scan), the checks, the
// device copy of its local states (padded to kCfgStride)
__global__ void rows_kernel(int64_t n, int N, const int16_t* __restrict__ fock, const int16_t* __restrict__ cfg,
                            const int32_t* __restrict__ norb, const int32_t* __restrict__ blk,
                            const BlockInfo* __restrict__ blocks, int nmax1, int16_t* __restrict__ cfg8,
                            int32_t* __restrict__ flag, unsigned long long* __restrict__ err) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i > n) return;
  if (i == n) {
    flag[n] = 0;
    return;
  }
  const int16_t* f = fock + i * 2 * N;
  const int16_t* r = cfg + i * N;
  bool start = i == 0;
  for (int k = 0; k < 2 * N && !start; ++k) start = f[k] != f[k - 2 * N];
  flag[i] = start ? 1 : 0;
  unsigned long long e = ~0ull;
  if (start)
    for (int k = 0; k < 2 * N; ++k)
      if (f[k] < 0 || f[k] > 15) {
        e = row_error(0, i, 0, kErrFockRange);
        break;
      }
  for (int c = 0; c < N; ++c)
    if (r[c] < 0 || r[c] > 255) {
      e = min(e, row_error(1, i, c, kErrStateRange));
      break;
    }
  for (int c = 0; c < N; ++c) {
    const int fa = f[2 * c], fb = f[2 * c + 1];
    if (fa > norb[c] || fb > norb[c]) {
      e = min(e, row_error(2, i, c, kErrClusterSize));
      break;
    }
    if (fa < 0 || fb < 0) continue;  // reported at the sector's first row (group 0)
    const int bl = blk[dense_block_index(nmax1, c, kOpH, fa, fb, fa, fb)];
    if (bl < 0) {
      e = min(e, row_error(2, i, c, kErrNoBasis));
      break;
    }
    if (r[c] >= blocks[bl].mb) {
      e = min(e, row_error(2, i, c, kErrBeyondBasis));
      break;
    }
  }
#pragma unroll
  for (int c = 0; c < kCfgStride; ++c) cfg8[i * kCfgStride + c] = c < N ? r[c] : int16_t(0);
  if (e != ~0ull) atomicMin(err, e);
}

// sector of every row; first row and Fock entries of every sector
__global__ void sectors_kernel(int64_t n, int N, const int16_t* __restrict__ fock, const int32_t* __restrict__ excl,
                               int32_t* __restrict__ row_sector, int64_t* __restrict__ sec_start,
                               int16_t* __restrict__ sec_fock) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int32_t s1 = excl[i + 1];
  row_sector[i] = s1 - 1;
  if (s1 == excl[i]) return;
  const int32_t sct = excl[i];
  sec_start[sct] = i;
  for (int k = 0; k < 2 * N; ++k) sec_fock[int64_t(sct) * 2 * N + k] = fock[i * 2 * N + k];
}

// ---- 2. sector table ------------------------------------------------------------------------
__device__ __forceinline__ bool dev_fock_key(const int16_t* f, int N, uint64_t* key) {
  uint64_t k = 0;
  for (int i = 0; i < 2 * N; ++i) {
    if (f[i] < 0 || f[i] > 15) return false;
    k |= uint64_t(f[i]) << (4 * i);
  }
  *key = k;
  return true;
}

__global__ void sector_insert_kernel(int64_t n_sec, int N, const int16_t* __restrict__ sec_fock,
                                     uint64_t* __restrict__ tkeys, int32_t* __restrict__ tvals, uint64_t mask) {
  const int64_t s = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (s >= n_sec) return;
  uint64_t key;
  if (!dev_fock_key(sec_fock + s * 2 * N, N, &key)) return;  // rows were checked: never taken
  uint64_t h = sector_hash(key) & mask;
  // the table holds at most half as many sectors as slots, so a free slot is always found
  for (uint64_t probe = 0; probe <= mask; ++probe) {
    if (atomicCAS(reinterpret_cast<int*>(tvals + h), -1, int(s)) == -1) {
      tkeys[h] = key;
      return;
    }
    h = (h + 1) & mask;
  }
}

// a sector whose Fock key an earlier sector already has: its rows are not contiguous
__global__ void sector_verify_kernel(int64_t n_sec, int N, const int16_t* __restrict__ sec_fock,
                                     const int64_t* __restrict__ sec_start, const uint64_t* __restrict__ tkeys,
                                     const int32_t* __restrict__ tvals, uint64_t mask,
                                     unsigned long long* __restrict__ err) {
  const int64_t s = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (s >= n_sec) return;
  uint64_t key;
  if (!dev_fock_key(sec_fock + s * 2 * N, N, &key)) return;  // an entry out of range: reported already
  uint64_t h = sector_hash(key) & mask;
  // every slot of this key lies on its probe sequence before the first free slot
  for (uint64_t probe = 0; probe <= mask; ++probe) {
    const int32_t v = tvals[h];
    if (v < 0) return;
    if (tkeys[h] == key && v < s) {
      atomicMin(err, row_error(0, sec_start[s], 0, kErrSplitSector));
      return;
    }
    h = (h + 1) & mask;
  }
}

// ket sector of every (bra sector, transfer) with term lists, -1 where it has no rows
__global__ void ket_sector_kernel(int64_t n_sec, int n_trans, int N, const int16_t* __restrict__ sec_fock,
                                  const int16_t* __restrict__ trans, const int32_t* __restrict__ first_of_tr,
                                  const uint64_t* __restrict__ tkeys, const int32_t* __restrict__ tvals, uint64_t mask,
                                  int32_t* __restrict__ sk_of) {
  const int64_t idx = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (idx >= n_sec * n_trans) return;
  const int64_t sb = idx / n_trans;
  const int tr = int(idx - sb * n_trans);
  int32_t out = -1;
  if (first_of_tr[tr] != first_of_tr[tr + 1]) {
    const int16_t* fb = sec_fock + sb * 2 * N;
    const int16_t* dt = trans + int64_t(tr) * 2 * N;
    uint64_t key = 0;
    bool ok = true;
    for (int i = 0; i < 2 * N; ++i) {
      const int v = fb[i] - dt[i];
      ok &= v >= 0 && v <= 15;
      key |= uint64_t(v & 15) << (4 * i);
    }
    if (ok) {
      uint64_t h = sector_hash(key) & mask;
      for (uint64_t probe = 0; probe <= mask; ++probe) {
        const int32_t s = tvals[h];
        if (s < 0) break;
        if (tkeys[h] == key) {
          out = s;
          break;
        }
        h = (h + 1) & mask;
      }
    }
  }
  sk_of[idx] = out;
}

// ---- 3. term-sector records per (bra sector, term list) -----------------------------------
struct PairParams {
  TermTables tt;
  const int16_t* sec_fock;
  const int32_t* sk_of;
  const int32_t* tl_tr;
  const int32_t* tl_set;
  const int32_t* tl_off;
  const int32_t* tl_terms;
  const int64_t* seg_g;
  int64_t n_pt;  // pairs: n_sec x n_tl
  int n_tl, n_trans, n_sets, N;
};

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) v += __shfl_xor_sync(0xffffffffu, v, d);
  return v;
}

// one thread per pair (a term list holds a few terms, and most pairs have no ket sector):
// the records that exist, their flop counts, and the bra groups to join
__global__ void pair_count_kernel(PairParams p, int64_t* __restrict__ pt_nt, int64_t* __restrict__ pt_ng,
                                  int64_t* __restrict__ pt_flop, int64_t* __restrict__ pt_flopd) {
  const int64_t w = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (w > p.n_pt) return;
  if (w == p.n_pt) {  // zeros past the end for the scans
    pt_nt[w] = pt_ng[w] = 0;
    return;
  }
  const int64_t sb = w / p.n_tl;
  const int j = int(w - sb * p.n_tl);
  const int32_t sk = p.sk_of[sb * p.n_trans + p.tl_tr[j]];
  int64_t nt = 0, flop = 0, flopd = 0;
  if (sk >= 0) {
    const int16_t* fb = p.sec_fock + sb * 2 * p.N;
    const int16_t* fk = p.sec_fock + int64_t(sk) * 2 * p.N;
    for (int q = p.tl_off[j]; q < p.tl_off[j + 1]; ++q) {
      const int t = p.tl_terms[q];
      TermSector ts;
      int64_t fma;
      if (term_sector_of(p.tt, t, fb, fk, ts, &fma)) {
        ++nt;
        flop += term_ref_flops(p.tt.trm, t);
        flopd += 2 * fma;
      }
    }
  }
  const int64_t seg = sb * p.n_sets + p.tl_set[j];
  pt_nt[w] = nt;
  pt_flop[w] = flop;
  pt_flopd[w] = flopd;
  pt_ng[w] = nt > 0 ? p.seg_g[seg + 1] - p.seg_g[seg] : 0;
}

// one thread per pair: its records, in term order, at its scanned offset
__global__ void pair_records_kernel(PairParams p, const int64_t* __restrict__ ts_off, TermSector* __restrict__ pool) {
  const int64_t w = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (w >= p.n_pt) return;
  int64_t o = ts_off[w];
  if (ts_off[w + 1] == o) return;
  const int64_t sb = w / p.n_tl;
  const int j = int(w - sb * p.n_tl);
  const int32_t sk = p.sk_of[sb * p.n_trans + p.tl_tr[j]];
  const int16_t* fb = p.sec_fock + sb * 2 * p.N;
  const int16_t* fk = p.sec_fock + int64_t(sk) * 2 * p.N;
  for (int q = p.tl_off[j]; q < p.tl_off[j + 1]; ++q) {
    TermSector ts;
    int64_t fma;
    if (term_sector_of(p.tt, p.tl_terms[q], fb, fk, ts, &fma)) pool[o++] = ts;
  }
}

// ---- 4. join ----------------------------------------------------------------------------
// the last index i in [0, n) with a[i] <= x (a non-decreasing, a[0] <= x)
template <typename T>
__device__ __forceinline__ int64_t last_le(const T* a, int64_t n, int64_t x) {
  int64_t lo = 0, hi = n - 1;
  while (lo < hi) {
    const int64_t mid = (lo + hi + 1) >> 1;
    if (int64_t(a[mid]) <= x)
      lo = mid;
    else
      hi = mid - 1;
  }
  return lo;
}

// every bra group of every pair: the ket group of the same spectator key, if any
__global__ void match_kernel(PairParams p, int64_t E, const int64_t* __restrict__ pt_e, const uint64_t* __restrict__ g_key,
                             int32_t* __restrict__ m_flag, int32_t* __restrict__ m_ket, int32_t* __restrict__ m_pair) {
  const int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (e > E) return;
  if (e == E) {
    m_flag[e] = 0;
    return;
  }
  const int64_t w = last_le(pt_e, p.n_pt + 1, e);
  const int64_t sb = w / p.n_tl;
  const int j = int(w - sb * p.n_tl);
  const int set = p.tl_set[j];
  const int32_t sk = p.sk_of[sb * p.n_trans + p.tl_tr[j]];
  const int64_t gb = p.seg_g[sb * p.n_sets + set] + (e - pt_e[w]);
  const uint64_t key = g_key[gb];
  int64_t lo = p.seg_g[int64_t(sk) * p.n_sets + set], hi = p.seg_g[int64_t(sk) * p.n_sets + set + 1];
  while (lo < hi) {  // first ket group with key >= the bra group's
    const int64_t mid = (lo + hi) >> 1;
    if (g_key[mid] < key)
      lo = mid + 1;
    else
      hi = mid;
  }
  const bool hit = lo < p.seg_g[int64_t(sk) * p.n_sets + set + 1] && g_key[lo] == key;
  m_flag[e] = hit ? 1 : 0;
  m_ket[e] = hit ? int32_t(lo) : -1;
  m_pair[e] = int32_t(w);
}

struct ItemOut {
  int32_t* bra;   // first position of the bra group in the permutation pool
  int32_t* ket;   // same, ket group
  int32_t* nk;    // kets
  int32_t* pair;  // (bra sector, term list) pair
  int64_t* jobs;  // lane jobs (E + 1 entries, zero past the last item)
};

// counters: 0 triples, 1 reference flops, 2 executed flops, 3 largest lane-job cost
__global__ void items_kernel(PairParams p, int64_t E, const int64_t* __restrict__ pt_e, const int64_t* __restrict__ pt_nt,
                             const int64_t* __restrict__ pt_flop, const int64_t* __restrict__ pt_flopd,
                             const int32_t* __restrict__ g_start, const int32_t* __restrict__ g_cnt,
                             const int32_t* __restrict__ item_of, const int32_t* __restrict__ m_ket,
                             const int32_t* __restrict__ m_pair, ItemOut out, unsigned long long* __restrict__ counters) {
  const int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  unsigned long long tri = 0, fl = 0, fld = 0, cmax = 0;
  if (e < E && item_of[e + 1] != item_of[e]) {
    const int32_t it = item_of[e];
    const int64_t w = m_pair[e];
    const int64_t sb = w / p.n_tl;
    const int j = int(w - sb * p.n_tl);
    const int64_t gb = p.seg_g[sb * p.n_sets + p.tl_set[j]] + (e - pt_e[w]);
    const int32_t gk = m_ket[e];
    const int64_t nb = g_cnt[gb], nk = g_cnt[gk];
    const int64_t nt = pt_nt[w + 1] - pt_nt[w];
    out.bra[it] = g_start[gb];
    out.ket[it] = g_start[gk];
    out.nk[it] = int32_t(nk);
    out.pair[it] = int32_t(w);
    out.jobs[it] = nb * ((nk + kLaneKets - 1) / kLaneKets);
    tri = (unsigned long long)(nb * nk * nt);
    fl = (unsigned long long)(nb * nk * pt_flop[w]);
    fld = (unsigned long long)(nb * nk * pt_flopd[w]);
    const int64_t step = pt_flopd[w] / 2 + 8 * nt + 4;
    cmax = (unsigned long long)min64(step * min64(kLaneKets, nk), int64_t(1) << 30);
  }
  tri = warp_sum(tri);
  fl = warp_sum(fl);
  fld = warp_sum(fld);
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) cmax = max(cmax, __shfl_xor_sync(0xffffffffu, cmax, d));
  if ((threadIdx.x & 31) == 0 && (tri | fl | fld | cmax)) {
    atomicAdd(counters + 0, tri);
    atomicAdd(counters + 1, fl);
    atomicAdd(counters + 2, fld);
    atomicMax(counters + 3, cmax);
  }
}

// the state's sector count, for the host
__global__ void rows_collect_kernel(const int32_t* __restrict__ n_sec_at, unsigned long long* __restrict__ counters) {
  counters[1] = (unsigned long long)*n_sec_at;
}

// the sizes the next phase needs, in one place for one copy
__global__ void collect_kernel(const int32_t* __restrict__ n_items_at, const int64_t* __restrict__ n_jobs_at,
                               unsigned long long* __restrict__ counters) {
  counters[4] = (unsigned long long)*n_items_at;
  counters[5] = (unsigned long long)*n_jobs_at;
}

// ---- 5. lane jobs -----------------------------------------------------------------------
struct JobParams {
  const int64_t* job_off;  // per item, scanned
  const int32_t* bra;
  const int32_t* ket;
  const int32_t* nk;
  const int32_t* pair;
  const int64_t* pt_ts;    // record offset of each pair (scanned)
  const int64_t* pt_flopd;
  const int32_t* tl_nbody;
  const int32_t* perm;
  int64_t n_items, n_jobs;
  int n_tl;
  int cost_bits;
};

__global__ void __launch_bounds__(kThreads) jobs_kernel(JobParams p, LaneJob* __restrict__ jobs,
                                                        int32_t* __restrict__ cost, uint64_t* __restrict__ keys,
                                                        uint32_t* __restrict__ vals) {
  __shared__ int64_t s_off[kThreads + 1];
  __shared__ int64_t s_lo, s_n;
  const int64_t first = int64_t(blockIdx.x) * kThreads;
  const int64_t last = min64(first + kThreads, p.n_jobs) - 1;
  if (threadIdx.x == 0) {
    const int64_t lo = last_le(p.job_off, p.n_items, first);
    s_lo = lo;
    s_n = last_le(p.job_off, p.n_items, last) - lo + 1;  // every item has a job: at most kThreads
  }
  __syncthreads();
  const int64_t lo = s_lo, n = s_n;
  for (int64_t t = threadIdx.x; t < n; t += kThreads) s_off[t] = p.job_off[lo + t];
  __syncthreads();
  const int64_t job = first + threadIdx.x;
  if (job > last) return;
  const int64_t loc = last_le(s_off, n, job);
  const int64_t it = lo + loc;
  const int64_t q = job - s_off[loc];
  const int nk = p.nk[it];
  const int nkc = (nk + kLaneKets - 1) / kLaneKets;
  const int64_t bj = q / nkc;
  const int k0 = int(q - bj * nkc) * kLaneKets;
  const int64_t w = p.pair[it];
  const int64_t sb = w / p.n_tl;
  const int j = int(w - sb * p.n_tl);
  const int64_t nt = (p.pt_ts[w + 1] - p.pt_ts[w]);
  LaneJob L;
  L.b = p.perm[p.bra[it] + bj];
  L.kp = p.ket[it] + k0;
  L.ts_off = int32_t(p.pt_ts[w]);
  L.len = uint16_t(min(kLaneKets, nk - k0));
  L.nt = uint16_t(nt);
  const int64_t step = p.pt_flopd[w] / 2 + 8 * nt + 4;
  const int32_t c = int32_t(min64(step * L.len, int64_t(1) << 30));
  const uint64_t cmask = (uint64_t(1) << p.cost_bits) - 1;
  const uint64_t cc = uint64_t(min(c, (1 << 26) - 1));
  jobs[job] = L;
  cost[job] = c;
  keys[job] = (uint64_t(sb / kWindow) << (p.cost_bits + 3)) | (uint64_t(p.tl_nbody[j]) << p.cost_bits) | (cmask - cc);
  vals[job] = uint32_t(job);
}

// sorted lane jobs (idle lanes past the last job) and their costs
__global__ void gather_jobs_kernel(int64_t n_jobs, int64_t n_slots, const uint32_t* __restrict__ order,
                                   const LaneJob* __restrict__ src, const int32_t* __restrict__ cost,
                                   LaneJob* __restrict__ dst, int32_t* __restrict__ cost_out) {
  const int64_t x = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (x >= n_slots) return;
  if (x < n_jobs) {
    const uint32_t o = order[x];
    dst[x] = src[o];
    cost_out[x] = cost[o];
  } else {
    dst[x] = LaneJob{0, 0, 0, 0, 0};
  }
}

// ---- 6. warp tasks and chunks -------------------------------------------------------------
__global__ void warp_tasks_kernel(int64_t n_jobs, int64_t n_wt, const LaneJob* __restrict__ jobs,
                                  const int32_t* __restrict__ cost, int64_t* __restrict__ wt_cum,
                                  int64_t* __restrict__ wt_vals) {
  const int64_t w = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (w > n_wt) return;
  int32_t c = 0, l = 0;
  if (w < n_wt)
    for (int64_t i = w * 32; i < min64(n_jobs, w * 32 + 32); ++i) {
      c = max(c, cost[i]);
      l = max(l, int32_t(jobs[i].len));
    }
  wt_cum[w] = c;
  wt_vals[w] = 32 * int64_t(l);
}

// chunk c starts at the first warp task whose exclusive cost prefix reaches c x chunk_cost
__global__ void chunks_kernel(int64_t n_wt, int64_t n_chunks, int64_t chunk_cost, const int64_t* __restrict__ wt_cum,
                              const int64_t* __restrict__ wt_vals, int64_t* __restrict__ lo_out,
                              int64_t* __restrict__ val_out) {
  const int64_t c = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (c > n_chunks) return;
  int64_t lo = n_wt;
  if (c < n_chunks) {
    const int64_t target = c * chunk_cost;
    int64_t a = 0, b = n_wt;
    while (a < b) {
      const int64_t mid = (a + b) >> 1;
      if (wt_cum[mid] < target)
        a = mid + 1;
      else
        b = mid;
    }
    lo = a;
  }
  lo_out[c] = lo;
  val_out[c] = wt_vals[lo];
}

}  // namespace
}  // namespace fcg

// Term tables of the term set on the device, and the spectator-key layout of its active sets
static int upload_term_tables(fcg_ctx* ctx) {
  if (ctx->dj.ready) return FCG_OK;
  const ProblemInfo pi = problem_info(ctx);
  auto& D = ctx->dj;
  const std::string msg = term_lists(pi, D.lists);
  FCG_REQUIRE(msg.empty(), FCG_EINVAL, msg);
  const TermLists& L = D.lists;
  const int N = ctx->N, nmax1 = ctx->nmax + 1;
  // bits per cluster: enough for the largest local basis of the cluster
  int bits[kMaxClusters] = {};
  for (int c = 0; c < N; ++c) {
    int mb = 1;
    for (int fa = 0; fa <= ctx->norb[c]; ++fa)
      for (int fb = 0; fb <= ctx->norb[c]; ++fb) {
        const int bl = ctx->h_blk_index[dense_block_index(nmax1, c, kOpH, fa, fb, fa, fb)];
        if (bl >= 0) mb = std::max(mb, ctx->h_blocks[bl].mb);
      }
    bits[c] = bit_width(uint64_t(mb - 1));
  }
  D.n_sets = int(L.masks.size());
  D.n_tl = int(L.tr.size());
  D.spec_bits = 0;
  std::vector<uint8_t> spec_off(size_t(std::max(D.n_sets, 1)) * kMaxClusters, kActive);
  for (int k = 0; k < D.n_sets; ++k) {
    int off = 0;
    for (int c = 0; c < N; ++c) {
      if ((L.masks[k] >> c) & 1) continue;
      spec_off[size_t(k) * kMaxClusters + c] = uint8_t(off);
      off += bits[c];
    }
    D.spec_bits = std::max(D.spec_bits, off);
  }
  FCG_REQUIRE(D.spec_bits <= 64, FCG_ELIMIT, "spectator keys exceed 64 bits");
  std::vector<int32_t> nbody(size_t(std::max(D.n_tl, 1)), 0);
  for (int j = 0; j < D.n_tl; ++j) nbody[j] = ctx->trm[size_t(L.terms[L.off[j]]) * kTrmCols];
  cudaStream_t s = ctx->stream;
  FCG_CUDA(D.d_trm.upload(ctx->trm.data(), ctx->trm.size(), s));
  FCG_CUDA(D.d_dress.upload(ctx->dress.data(), ctx->dress.size(), s));
  FCG_CUDA(D.d_w_index.upload(ctx->w_index.data(), ctx->w_index.size(), s));
  FCG_CUDA(D.d_trans.upload(ctx->trans.data(), ctx->trans.size(), s));
  FCG_CUDA(D.d_first_of_tr.upload(L.first_of_tr.data(), L.first_of_tr.size(), s));
  FCG_CUDA(D.d_tl_tr.upload(L.tr.data(), L.tr.size(), s));
  FCG_CUDA(D.d_tl_set.upload(L.set.data(), L.set.size(), s));
  FCG_CUDA(D.d_tl_off.upload(L.off.data(), L.off.size(), s));
  FCG_CUDA(D.d_tl_terms.upload(L.terms.data(), L.terms.size(), s));
  FCG_CUDA(D.d_tl_nbody.upload(nbody.data(), nbody.size(), s));
  FCG_CUDA(D.d_spec_off.upload(spec_off.data(), spec_off.size(), s));
  FCG_CUDA(D.d_cnt.alloc(8));
  FCG_CUDA(D.h_cnt.alloc(8));
  D.ready = true;
  return FCG_OK;
}

// host read of counters (one copy, one wait)
static int read_counters(fcg_ctx* ctx, int n) {
  FCG_CUDA(cudaMemcpyAsync(ctx->dj.h_cnt.p, ctx->dj.d_cnt.p, sizeof(unsigned long long) * n, cudaMemcpyDeviceToHost,
                           ctx->stream));
  FCG_CUDA(cudaStreamSynchronize(ctx->stream));
  return FCG_OK;
}

// the sector table of the state's sectors (Fock key -> sector), sized for n_sec sectors
static int build_sector_table(fcg_ctx* ctx, int64_t n_sec) {
  auto& D = ctx->dj;
  int64_t cap = 64;
  while (cap < 2 * n_sec) cap <<= 1;
  FCG_CUDA(D.d_tkeys.alloc(size_t(cap)));
  FCG_CUDA(D.d_tvals.alloc(size_t(cap)));
  FCG_CUDA(cudaMemsetAsync(D.d_tvals.p, 0xFF, sizeof(int32_t) * cap, ctx->stream));
  sector_insert_kernel<<<grid_for(n_sec), kThreads, 0, ctx->stream>>>(n_sec, ctx->N, ctx->d_sec_fock.p, D.d_tkeys.p,
                                                                      D.d_tvals.p, uint64_t(cap - 1));
  FCG_CUDA(cudaGetLastError());
  D.table_cap = cap;
  D.table_ready = true;
  return FCG_OK;
}

int state_rows_device(fcg_ctx* ctx, int64_t n_cfg, const int16_t* fock, const int16_t* cfg) {
  auto& D = ctx->dj;
  Plan& P = ctx->plan;
  const int N = ctx->N;
  P = Plan();
  P.N = N;
  P.n_cfg = n_cfg;
  D.table_ready = false;
  FCG_REQUIRE(N <= kMaxClusters, FCG_EINVAL, "more than 8 clusters");
  FCG_REQUIRE(n_cfg < (int64_t(1) << 31), FCG_EINVAL, "too many configurations");
  cudaStream_t s = ctx->stream;
  FCG_CUDA(D.d_cnt.alloc(8));
  FCG_CUDA(D.h_cnt.alloc(8));
  FCG_CUDA(D.d_fock_in.upload(fock, size_t(n_cfg) * 2 * N, s));
  FCG_CUDA(D.d_cfg_in.upload(cfg, size_t(n_cfg) * N, s));
  FCG_CUDA(ctx->d_cfg.alloc(size_t(n_cfg) * kCfgStride));
  FCG_CUDA(ctx->d_row_sector.alloc(size_t(n_cfg)));
  FCG_CUDA(ctx->d_sec_fock.alloc(size_t(n_cfg) * 2 * N));
  int32_t *flag, *tmp;
  int64_t* sec_start;
  FCG_CUDA(carve(D.arena_rows, [&](Bump& b) {
    flag = b.take<int32_t>(n_cfg + 1);
    tmp = b.take<int32_t>(dprim::scan_scratch(n_cfg + 1));
    sec_start = b.take<int64_t>(n_cfg);
  }));
  FCG_CUDA(cudaMemsetAsync(D.d_cnt.p, 0xFF, sizeof(unsigned long long), s));  // no error yet
  rows_kernel<<<grid_for(n_cfg + 1), kThreads, 0, s>>>(n_cfg, N, D.d_fock_in.p, D.d_cfg_in.p, ctx->d_norb.p,
                                                       ctx->d_blk_index.p, ctx->d_blocks.p, ctx->nmax + 1,
                                                       ctx->d_cfg.p, flag, D.d_cnt.p);
  FCG_CUDA(cudaGetLastError());
  FCG_CUDA(dprim::exclusive_scan<int32_t>(flag, n_cfg + 1, tmp, s));
  sectors_kernel<<<grid_for(n_cfg), kThreads, 0, s>>>(n_cfg, N, D.d_fock_in.p, flag, ctx->d_row_sector.p, sec_start,
                                                      ctx->d_sec_fock.p);
  FCG_CUDA(cudaGetLastError());
  rows_collect_kernel<<<1, 1, 0, s>>>(flag + n_cfg, D.d_cnt.p);
  FCG_CUDA(cudaGetLastError());
  {
    const int rc = read_counters(ctx, 2);
    if (rc) return rc;
  }
  const int64_t n_sec = int64_t(D.h_cnt.p[1]);
  {
    const int rc = build_sector_table(ctx, n_sec);
    if (rc) return rc;
  }
  sector_verify_kernel<<<grid_for(n_sec), kThreads, 0, s>>>(n_sec, N, ctx->d_sec_fock.p, sec_start, D.d_tkeys.p,
                                                            D.d_tvals.p, uint64_t(D.table_cap - 1), D.d_cnt.p);
  FCG_CUDA(cudaGetLastError());
  P.sec_start.resize(size_t(n_sec));
  P.sec_fock.resize(size_t(n_sec) * 2 * N);
  FCG_CUDA(cudaMemcpyAsync(P.sec_start.data(), sec_start, sizeof(int64_t) * n_sec, cudaMemcpyDeviceToHost, s));
  FCG_CUDA(cudaMemcpyAsync(P.sec_fock.data(), ctx->d_sec_fock.p, sizeof(int16_t) * n_sec * 2 * N,
                           cudaMemcpyDeviceToHost, s));
  {
    const int rc = read_counters(ctx, 1);
    if (rc) return rc;
  }
  const unsigned long long err = D.h_cnt.p[0];
  if (err != ~0ull) {
    D.table_ready = false;
    static const char* const kMsg[] = {"",
                                       "Fock sector entry outside [0, 15]",
                                       "rows of a Fock sector are not contiguous",
                                       "local state index outside [0, 255]",
                                       "Fock sector exceeds cluster size",
                                       "a row uses a Fock sector with no local basis",
                                       "local state index beyond the sector's basis"};
    const int code = int(err & 15);
    FCG_REQUIRE(false, FCG_EINVAL, code >= 1 && code <= 6 ? kMsg[code] : "bad rows");
  }
  P.sec_count.resize(size_t(n_sec));
  for (int64_t i = 0; i < n_sec; ++i) P.sec_count[i] = (i + 1 < n_sec ? P.sec_start[i + 1] : n_cfg) - P.sec_start[i];
  P.zero_terms = zero_transfer_terms(problem_info(ctx));
  return FCG_OK;
}

int device_chunks(fcg_ctx* ctx, int64_t target, DevBuf<int64_t>& lo, DevBuf<int64_t>& val, int64_t* n_chunks) {
  const int64_t total = ctx->plan_total_cost, n_wt = ctx->plan_wt;
  const int64_t chunk_cost =
      std::max<int64_t>(kMinChunkCost, std::min<int64_t>(kChunkCost, total / std::max<int64_t>(target, 1)));
  const int64_t nc = (total + chunk_cost - 1) / chunk_cost;
  FCG_CUDA(lo.alloc(size_t(nc + 1)));
  FCG_CUDA(val.alloc(size_t(nc + 1)));
  chunks_kernel<<<grid_for(nc + 1), kThreads, 0, ctx->stream>>>(n_wt, nc, chunk_cost, ctx->d_wt_cum.p,
                                                                 ctx->d_wt_vals.p, lo.p, val.p);
  FCG_CUDA(cudaGetLastError());
  *n_chunks = nc;
  return FCG_OK;
}

int build_join_device(fcg_ctx* ctx) {
  {
    const int rc = upload_term_tables(ctx);
    if (rc) return rc;
  }
  auto& D = ctx->dj;
  Plan& P = ctx->plan;
  cudaStream_t s = ctx->stream;
  const int N = ctx->N, n_sets = D.n_sets, n_tl = D.n_tl, n_trans = ctx->n_trans;
  const int64_t n_cfg = ctx->n_cfg, n_sec = int64_t(P.sec_start.size());
  const int64_t n_el = n_cfg * n_sets, n_seg = n_sec * n_sets, n_pt = n_sec * n_tl;
  FCG_REQUIRE(n_el < (int64_t(1) << 31), FCG_ELIMIT, "grouping pool exceeds 2^31 rows");
  FCG_REQUIRE(n_pt < (int64_t(1) << 31), FCG_ELIMIT, "too many (sector, term list) pairs");
  P.items.clear();
  P.jobs.clear();
  P.chunk_lo.clear();
  P.chunk_val.clear();
  P.wt_cost.clear();
  P.wt_len.clear();
  P.prefix.clear();
  P.ts_pool.clear();
  P.perm_pool.clear();
  P.n_triples = P.flops_ref = P.flops_dressed = P.task_values = 0;
  FCG_CUDA(D.d_sec_start.upload(P.sec_start.data(), P.sec_start.size(), s));
  FCG_CUDA(D.d_sec_count.upload(P.sec_count.data(), P.sec_count.size(), s));
  FCG_CUDA(cudaMemsetAsync(D.d_cnt.p, 0, 8 * sizeof(unsigned long long), s));

  // ---- 1. spectator keys, sort, groups --------------------------------------------------
  uint64_t* gk[2];
  uint32_t* gv[2];
  int32_t *flag, *sort_tmp, *g_start, *g_cnt;
  uint64_t* g_key;
  int64_t* seg_g;
  const int64_t tmp_n = std::max(dprim::sort_scratch(n_el), dprim::scan_scratch(n_el + 1));
  FCG_CUDA(carve(D.arena[0], [&](Bump& b) {
    gk[0] = b.take<uint64_t>(n_el);
    gk[1] = b.take<uint64_t>(n_el);
    gv[0] = b.take<uint32_t>(n_el);
    gv[1] = b.take<uint32_t>(n_el);
    flag = b.take<int32_t>(n_el + 1);
    sort_tmp = b.take<int32_t>(tmp_n);
    g_key = b.take<uint64_t>(n_el);
    g_start = b.take<int32_t>(n_el);
    g_cnt = b.take<int32_t>(n_el);
    seg_g = b.take<int64_t>(n_seg + 1);
  }));
  FCG_CUDA(ctx->d_perm.alloc(size_t(n_el)));
  spectator_keys_kernel<<<grid_for(n_el), kThreads, 0, s>>>(n_cfg, n_sets, N, ctx->d_cfg.p, ctx->d_row_sector.p,
                                                            D.d_sec_start.p, D.d_sec_count.p, D.d_spec_off.p, gk[0],
                                                            gv[0]);
  FCG_CUDA(cudaGetLastError());
  {
    dprim::Digit passes[16];
    int np = 0;
    for (int sh = 0; sh < D.spec_bits; sh += 8) passes[np++] = dprim::Digit{sh, 0, nullptr};
    const int seg_bits = bit_width(uint64_t(std::max<int64_t>(n_seg - 1, 0)));
    for (int sh = 0; sh < seg_bits; sh += 8) passes[np++] = dprim::Digit{sh, n_sets, ctx->d_row_sector.p};
    int which = 0;
    FCG_CUDA(dprim::radix_sort(gk, gv, n_el, passes, np, sort_tmp, &which, s));
    if (which) {
      std::swap(gk[0], gk[1]);
      std::swap(gv[0], gv[1]);
    }
  }
  group_flags_kernel<<<grid_for(n_el + 1), kThreads, 0, s>>>(n_el, gk[0], gv[0], n_sets, ctx->d_row_sector.p,
                                                             ctx->d_perm.p, flag);
  FCG_CUDA(cudaGetLastError());
  FCG_CUDA(dprim::exclusive_scan<int32_t>(flag, n_el + 1, sort_tmp, s));
  group_fill_kernel<<<grid_for(n_el), kThreads, 0, s>>>(n_el, gk[0], gv[0], n_sets, ctx->d_row_sector.p, flag, g_key,
                                                        g_start, seg_g);
  FCG_CUDA(cudaGetLastError());
  group_count_kernel<<<grid_for(n_el), kThreads, 0, s>>>(n_el, flag + n_el, g_start, g_cnt, seg_g, n_seg);
  FCG_CUDA(cudaGetLastError());

  // ---- 2. sector table (the state's rows built it, unless the host checked them) and ket
  // sectors --------------------------------------------------------------------------------
  if (!D.table_ready) {
    const int rc = build_sector_table(ctx, n_sec);
    if (rc) return rc;
  }
  int32_t* sk_of;
  int64_t *pt_nt, *pt_ng, *pt_flop, *pt_flopd, *pt_tmp;
  FCG_CUDA(carve(D.arena[1], [&](Bump& b) {
    sk_of = b.take<int32_t>(n_sec * n_trans);
    pt_nt = b.take<int64_t>(n_pt + 1);
    pt_ng = b.take<int64_t>(n_pt + 1);
    pt_flop = b.take<int64_t>(n_pt);
    pt_flopd = b.take<int64_t>(n_pt);
    pt_tmp = b.take<int64_t>(dprim::scan_scratch(n_pt + 1));
  }));
  ket_sector_kernel<<<grid_for(n_sec * n_trans), kThreads, 0, s>>>(n_sec, n_trans, N, ctx->d_sec_fock.p,
                                                                   D.d_trans.p, D.d_first_of_tr.p, D.d_tkeys.p,
                                                                   D.d_tvals.p, uint64_t(D.table_cap - 1), sk_of);
  FCG_CUDA(cudaGetLastError());

  // ---- 3. term-sector records ------------------------------------------------------------
  PairParams pp{};
  pp.tt = TermTables{D.d_trm.p, D.d_dress.p, D.d_w_index.p, ctx->d_blk_index.p, ctx->d_blocks.p, ctx->nmax + 1};
  pp.sec_fock = ctx->d_sec_fock.p;
  pp.sk_of = sk_of;
  pp.tl_tr = D.d_tl_tr.p;
  pp.tl_set = D.d_tl_set.p;
  pp.tl_off = D.d_tl_off.p;
  pp.tl_terms = D.d_tl_terms.p;
  pp.seg_g = seg_g;
  pp.n_pt = n_pt;
  pp.n_tl = n_tl;
  pp.n_trans = n_trans;
  pp.n_sets = n_sets;
  pp.N = N;
  pair_count_kernel<<<grid_for(n_pt + 1), kThreads, 0, s>>>(pp, pt_nt, pt_ng, pt_flop, pt_flopd);
  FCG_CUDA(cudaGetLastError());
  FCG_CUDA(dprim::exclusive_scan<int64_t>(pt_nt, n_pt + 1, pt_tmp, s));
  FCG_CUDA(dprim::exclusive_scan<int64_t>(pt_ng, n_pt + 1, pt_tmp, s));
  FCG_CUDA(cudaMemcpyAsync(D.d_cnt.p + 6, pt_nt + n_pt, sizeof(int64_t), cudaMemcpyDeviceToDevice, s));
  FCG_CUDA(cudaMemcpyAsync(D.d_cnt.p + 7, pt_ng + n_pt, sizeof(int64_t), cudaMemcpyDeviceToDevice, s));
  {
    const int rc = read_counters(ctx, 8);
    if (rc) return rc;
  }
  const int64_t n_ts = int64_t(D.h_cnt.p[6]), E = int64_t(D.h_cnt.p[7]);
  FCG_REQUIRE(n_ts < (int64_t(1) << 31), FCG_ELIMIT, "term-sector pool exceeds 2^31 records");
  FCG_REQUIRE(E < (int64_t(1) << 31), FCG_ELIMIT, "join exceeds 2^31 bra groups");
  FCG_CUDA(ctx->d_ts.alloc(size_t(n_ts)));
  if (n_ts > 0) {
    pair_records_kernel<<<grid_for(n_pt), kThreads, 0, s>>>(pp, pt_nt, ctx->d_ts.p);
    FCG_CUDA(cudaGetLastError());
  }

  // ---- 4. join -----------------------------------------------------------------------------
  int32_t *m_flag, *m_ket, *m_pair, *m_tmp;
  int64_t* j_tmp;
  ItemOut io{};
  FCG_CUDA(carve(D.arena[2], [&](Bump& b) {
    m_flag = b.take<int32_t>(E + 1);
    m_ket = b.take<int32_t>(E);
    m_pair = b.take<int32_t>(E);
    m_tmp = b.take<int32_t>(dprim::scan_scratch(E + 1));
    io.bra = b.take<int32_t>(E);
    io.ket = b.take<int32_t>(E);
    io.nk = b.take<int32_t>(E);
    io.pair = b.take<int32_t>(E);
    io.jobs = b.take<int64_t>(E + 1);
    j_tmp = b.take<int64_t>(dprim::scan_scratch(E + 1));
  }));
  match_kernel<<<grid_for(E + 1), kThreads, 0, s>>>(pp, E, pt_ng, g_key, m_flag, m_ket, m_pair);
  FCG_CUDA(cudaGetLastError());
  FCG_CUDA(dprim::exclusive_scan<int32_t>(m_flag, E + 1, m_tmp, s));
  FCG_CUDA(cudaMemsetAsync(io.jobs, 0, sizeof(int64_t) * (E + 1), s));
  if (E > 0) {
    items_kernel<<<grid_for(E), kThreads, 0, s>>>(pp, E, pt_ng, pt_nt, pt_flop, pt_flopd, g_start, g_cnt, m_flag,
                                                  m_ket, m_pair, io, D.d_cnt.p);
    FCG_CUDA(cudaGetLastError());
  }
  FCG_CUDA(dprim::exclusive_scan<int64_t>(io.jobs, E + 1, j_tmp, s));
  collect_kernel<<<1, 1, 0, s>>>(m_flag + E, io.jobs + E, D.d_cnt.p);
  FCG_CUDA(cudaGetLastError());
  {
    const int rc = read_counters(ctx, 6);
    if (rc) return rc;
  }
  const int64_t n_items = int64_t(D.h_cnt.p[4]), n_jobs = int64_t(D.h_cnt.p[5]);
  P.n_triples = int64_t(D.h_cnt.p[0]);
  P.flops_ref = int64_t(D.h_cnt.p[1]);
  P.flops_dressed = int64_t(D.h_cnt.p[2]);
  const int64_t cmax = std::min<int64_t>(int64_t(D.h_cnt.p[3]), (int64_t(1) << 26) - 1);
  FCG_REQUIRE(n_jobs < (int64_t(1) << 31) - 32, FCG_ELIMIT, "lane jobs exceed 2^31");

  // ---- 5. lane jobs, window sort -------------------------------------------------------
  const int64_t n_wt = (n_jobs + 31) / 32;
  LaneJob* jobs_tmp;
  int32_t *cost, *cost_s, *js_tmp;
  int64_t* wt_tmp;
  uint64_t* jk[2];
  uint32_t* jv[2];
  FCG_CUDA(carve(D.arena[3], [&](Bump& b) {
    jobs_tmp = b.take<LaneJob>(n_jobs);
    cost = b.take<int32_t>(n_jobs);
    cost_s = b.take<int32_t>(n_jobs);
    jk[0] = b.take<uint64_t>(n_jobs);
    jk[1] = b.take<uint64_t>(n_jobs);
    jv[0] = b.take<uint32_t>(n_jobs);
    jv[1] = b.take<uint32_t>(n_jobs);
    js_tmp = b.take<int32_t>(dprim::sort_scratch(n_jobs));
    wt_tmp = b.take<int64_t>(dprim::scan_scratch(n_wt + 1));
  }));
  FCG_CUDA(ctx->d_jobs.alloc(size_t(n_wt * 32)));
  FCG_CUDA(ctx->d_wt_cum.alloc(size_t(n_wt + 1)));
  FCG_CUDA(ctx->d_wt_vals.alloc(size_t(n_wt + 1)));
  if (n_jobs > 0) {
    JobParams jp{};
    jp.job_off = io.jobs;
    jp.bra = io.bra;
    jp.ket = io.ket;
    jp.nk = io.nk;
    jp.pair = io.pair;
    jp.pt_ts = pt_nt;
    jp.pt_flopd = pt_flopd;
    jp.tl_nbody = D.d_tl_nbody.p;
    jp.perm = ctx->d_perm.p;
    jp.n_items = n_items;
    jp.n_jobs = n_jobs;
    jp.n_tl = n_tl;
    jp.cost_bits = bit_width(uint64_t(cmax));
    jobs_kernel<<<grid_for(n_jobs), kThreads, 0, s>>>(jp, jobs_tmp, cost, jk[0], jv[0]);
    FCG_CUDA(cudaGetLastError());
    dprim::Digit passes[16];
    int np = 0;
    const int bits = jp.cost_bits + 3 + bit_width(uint64_t(std::max<int64_t>(n_sec - 1, 0) / kWindow));
    for (int sh = 0; sh < bits; sh += 8) passes[np++] = dprim::Digit{sh, 0, nullptr};
    int which = 0;
    FCG_CUDA(dprim::radix_sort(jk, jv, n_jobs, passes, np, js_tmp, &which, s));
    gather_jobs_kernel<<<grid_for(n_wt * 32), kThreads, 0, s>>>(n_jobs, n_wt * 32, jv[which], jobs_tmp, cost,
                                                                ctx->d_jobs.p, cost_s);
    FCG_CUDA(cudaGetLastError());
  }

  // ---- 6. warp tasks, chunks ------------------------------------------------------------------
  warp_tasks_kernel<<<grid_for(n_wt + 1), kThreads, 0, s>>>(n_jobs, n_wt, ctx->d_jobs.p, cost_s, ctx->d_wt_cum.p,
                                                            ctx->d_wt_vals.p);
  FCG_CUDA(cudaGetLastError());
  FCG_CUDA(dprim::exclusive_scan<int64_t>(ctx->d_wt_cum.p, n_wt + 1, wt_tmp, s));
  FCG_CUDA(dprim::exclusive_scan<int64_t>(ctx->d_wt_vals.p, n_wt + 1, wt_tmp, s));
  FCG_CUDA(cudaMemcpyAsync(D.d_cnt.p + 0, ctx->d_wt_cum.p + n_wt, sizeof(int64_t), cudaMemcpyDeviceToDevice, s));
  FCG_CUDA(cudaMemcpyAsync(D.d_cnt.p + 1, ctx->d_wt_vals.p + n_wt, sizeof(int64_t), cudaMemcpyDeviceToDevice, s));
  {
    const int rc = read_counters(ctx, 2);
    if (rc) return rc;
  }
  ctx->plan_total_cost = int64_t(D.h_cnt.p[0]);
  P.task_values = int64_t(D.h_cnt.p[1]);
  ctx->plan_wt = n_wt;
  ctx->plan_jobs = n_wt * 32;
  ctx->plan_items = n_items;
  ctx->plan_ts = n_ts;
  ctx->plan_perm = n_el;
  {
    const int rc = device_chunks(ctx, kTargetChunks, ctx->d_chunk_lo, ctx->d_chunk_val, &ctx->n_chunks);
    if (rc) return rc;
  }
  FCG_CUDA(cudaStreamSynchronize(s));
  return FCG_OK;
}
