// Internal types shared by the host planner (plan.cpp) and the CUDA side (fcg_gpu.cu).
#pragma once
#include <cstdint>
#include <string>
#include <vector>

#ifdef __CUDACC__
#define FCG_HD __host__ __device__
#else
#define FCG_HD
#endif

namespace fcg {

constexpr int kMaxClusters = 8;
constexpr int kOpbCols = 10;
constexpr int kTrmCols = 28;
constexpr int kNumOps = 24;  // 22 op strings + "H" + "Hcmf"
constexpr int kOpH = 22;
constexpr int kOpHcmf = 23;
constexpr int kCfgStride = 8;  // device rows of local states are padded to 8 int16 (16 bytes)
constexpr int kAlign = 8;      // device TDM / W blocks start on multiples of 8 elements (32-byte loads)

// One TDM block on the device.
struct BlockInfo {
  int64_t off;   // element offset into the op data blob
  int32_t nidx;  // orbital multi-index length
  int32_t mb;    // bra local states
  int32_t mk;    // ket local states
  int32_t pad;
};

// Compact device copy of one ClusteredTerm's metadata.
struct TermInfo {
  int64_t ints_off;
  int16_t dim[4];
  int8_t nbody;
  int8_t c[4];
  int8_t op[4];
  int8_t parity[4];
  int8_t pad[3];
};

// How a term is "dressed": its integrals are contracted once per problem with the TDM
// of one active cluster (the one with the longest orbital multi-index), giving
//   W[(rest), b, k] = sum_i ints[.. i ..] G_dressed[i, b, k]
// for every (bra, ket) local-state pair of every sector pair of that cluster.  The
// remaining clusters' TDM columns are contracted per matrix element.
struct TermDress {
  int pos;            // dressed position in the term (0..nbody-1); -1 for 1-body terms
  int rest_len;       // product of the other dims
  int nrem;           // nbody - 1
  int rem_pos[3];     // the other positions, in order
  int rem_dim[3];
};

// Per (sector pair, term): everything one matrix element needs besides the local states.
struct TermSector {
  int64_t w_off;      // W block base in the dressed array (1-body: the H block)
  int64_t g_off[3];   // TDM block base of the remaining clusters
  int32_t w_mb;       // bra states of the dressed cluster's block
  int32_t g_mb[3];    // bra states of the remaining clusters' blocks
  int16_t rest_len;   // W column length
  int16_t g_dim[3];   // orbital multi-index length of the remaining clusters
  int8_t cw;          // dressed cluster
  int8_t cr[3];       // remaining clusters
  int8_t nrem;        // number of remaining clusters (0..3)
  int8_t sign;        // compute_terms_state_sign for the ket sector (+1 / -1)
  int8_t pad[10];
};
static_assert(sizeof(TermSector) == 72, "TermSector layout");

// Open (FOIS) sigma: one term acting from one ket sector into one bra sector
// (open_matvec_thread, src/tpsci_matvec_thread.jl:11-263).
struct OpenTerm {
  TermSector ts;        // dressed W / remaining TDM columns, ket-sector sign
  int64_t wmax_off;     // Wmax[rest, k] at wmax_off + rest + rest_len*k
  int64_t gmax_off[3];  // Gmax[i, k] of the remaining clusters at off + i + g_dim*k
  int32_t bsec;         // bra sector id
  int32_t out_count;    // product of the bra dims of the active clusters
  int16_t mb_act[4];    // bra dims of the active clusters, order [dressed, remaining...]
  int8_t c_act[4];      // cluster ids in the same order
  int8_t n_act;
  int8_t pad[3];
};
static_assert(sizeof(OpenTerm) == 128, "OpenTerm layout");

// Open sigma work item: every (ket row in [row0, row0+nrow), term in [ot_off, ot_off+nt)) job.
struct OpenItem {
  int32_t row0, nrow, ot_off, nt;
};

// A closed-sigma work item: every (bra in group, ket in group, term in list) triple.
struct WorkItem {
  int32_t bra_off;  // offset of the bra group in the permutation pool
  int32_t ket_off;  // offset of the ket group in the permutation pool
  int32_t nb;       // bra group size
  int32_t nk;       // ket group size
  int32_t ts_off;   // offset of the term list in the TermSector pool
  int32_t nt;       // number of terms
};

// A closed-sigma lane job: one bra row of a work item against up to kLaneKets of the item's
// kets.  Warps run 32 consecutive lane jobs, one per lane; a lane sums the item's terms for
// each of its (bra, ket) pairs, multiplies by the ket's coefficients and adds its row to
// sigma once.  The planner orders lane jobs so that the lanes of a warp have the same term
// shape and about the same work.
struct LaneJob {
  int32_t b;       // bra row
  int32_t kp;      // offset of the first ket in the permutation pool
  int32_t ts_off;  // the item's term-sector records
  uint16_t len;    // kets (0: an idle lane)
  uint16_t nt;     // terms
};
static_assert(sizeof(LaneJob) == 16, "LaneJob layout");
constexpr int kLaneKets = 32;

// One W block to compute (fcg_set_terms): term t dressed with TDM block g of its dressed cluster.
struct DressJob {
  int64_t w_off;
  int64_t g_off;
  int64_t ints_off;
  int32_t rest_len, mb, mk, nq;  // nq: dressed orbital multi-index length
  int32_t stride_q;              // ints stride of the dressed index
  int32_t nrem;
  int32_t rem_dim[3];
  int32_t rem_stride[3];
  int32_t one_body;  // 1: copy the H block
  int32_t pad;
};

// ---- block-sparse Tucker (BST) vectors ---------------------------------------------------

// One Tucker block (fock sector, TuckerConfig) of a BST vector on the device.
struct BstBlock {
  int64_t core_off;                    // core of root r at cores[r * core_total + core_off], column-major
  int64_t factor_off[kMaxClusters];    // factor of cluster c: (len[c] x rank[c]) column-major
  int32_t rank[kMaxClusters];
  int32_t start[kMaxClusters];         // first local state of the range (0-based)
  int32_t len[kMaxClusters];           // range length
  int32_t core_len;
  int32_t ortho;                       // bit c: the factor of cluster c has orthonormal columns
};

// Dressed TDM of one active cluster between a bra and a ket block:
//   g[p, kb, kk] = sum_{I,J} U_bra[I, kb] G[p, start_bra + I, start_ket + J] U_ket[J, kk]
struct BstGamma {
  int64_t g_off;
  int64_t tdm_off;   // TDM block in the device op blob
  int32_t bra, ket, c;
  int32_t np;        // orbital multi-index length of the TDM
  int32_t tdm_mb;    // bra dimension of the TDM block
  int32_t pad;
};

// One term's share of a group operator.
struct BstGroupTerm {
  int64_t g_off[4];  // dressed TDMs of the active clusters, in term order
  int64_t ints_off;  // -1: 1-body term (coefficient 1)
  int32_t np[4];
  int32_t nact;
  int32_t sign;      // compute_terms_state_sign on the ket sector (1 for 1-body terms)
};

// All terms that couple one bra block to one ket block through the same active clusters:
//   OP[kk + k*kb] = (prod of scalar spectator overlaps) * sum_t sign_t sum_p ints_t[p] prod_a g_{t,a}[p_a, kb_a, kk_a]
// (kk / kb: mixed-radix over the active clusters in increasing cluster order, ket / bra ranks),
// with the index description the sigma kernels use: only clusters of rank > 1 on the bra or
// the ket side appear (a rank-1 cluster has a single index value on both sides).
struct BstGroup {
  int64_t op_off;
  int64_t k_off, b_off;          // ket / bra core offsets
  int64_t s_off[kMaxClusters];   // overlap U_bra^T U_ket (rank_bra x rank_ket) of spectator mode j; -1:
                                 // the identity (bra and ket share an orthonormal factor), not applied
  int32_t bra, ket;
  int32_t m, k;                  // products of the active bra / ket ranks
  int32_t act_mask;
  int32_t t_off, nt;             // terms in the group-term pool
  int32_t ws;                    // largest intermediate tensor of the sigma step (elements per root)
  int32_t kcore, bcore;          // ket / bra core lengths
  int32_t na, nsp;               // active clusters / spectator modes with rank > 1 on either side
  int32_t a_kr[4], a_br[4];      // their ket / bra ranks
  int32_t a_ks[4], a_bs[4];      // their strides in the ket / bra core
  int32_t s_kr[kMaxClusters], s_br[kMaxClusters];
  int32_t s_ks[kMaxClusters], s_bs[kMaxClusters];
  int32_t ntr;                   // spectator modes with an overlap to apply (the others: U^T U = 1)
  int32_t pad;
  // index tables (core offset of every position of the actives-first layout) of the ket and
  // the bra block for this group's active clusters
  int64_t kperm_off, bperm_off;
};
static_assert(sizeof(BstGroup) % 16 == 0, "BstGroup is copied to shared memory in 16-byte units");

// Problem description the planner needs (host copies).
struct ProblemInfo {
  int N = 0;
  std::vector<int> norb;
  int nmax = 0;
  const std::vector<int32_t>* trm = nullptr;
  int n_terms = 0;
  const std::vector<int16_t>* trans = nullptr;
  int n_trans = 0;
  const std::vector<int32_t>* blk_index = nullptr;  // dense (c, op, fba, fbb, fka, fkb) -> block
  const std::vector<BlockInfo>* blocks = nullptr;
  const std::vector<TermDress>* dress = nullptr;
  const std::vector<int64_t>* w_index = nullptr;    // [term][fb_a][fb_b] of the dressed cluster -> W offset
};

// Host-side plan of the closed sigma for one state.
struct Plan {
  int N = 0;
  int64_t n_cfg = 0;
  std::vector<int64_t> sec_start, sec_count;
  std::vector<int16_t> sec_fock;  // n_sec x N x 2
  std::vector<int32_t> perm_pool;
  std::vector<TermSector> ts_pool;
  std::vector<WorkItem> items;
  std::vector<int64_t> prefix;  // n_items + 1
  int64_t n_triples = 0;
  int64_t flops_ref = 0;        // sum over triples of 2*len(ints) (the reference's count)
  int64_t flops_dressed = 0;    // multiply-adds actually done per sigma (x2), excluding the R update
  std::vector<int32_t> zero_terms;
  // lane jobs (32 per warp task, the last warp task padded with idle lanes) and the warp
  // chunks: chunk c runs warp tasks [chunk_lo[c], chunk_lo[c+1]) (about kChunkCost of work);
  // chunk_val[c] is the first stored value of the chunk (32 per ket step of each warp task)
  std::vector<LaneJob> jobs;
  std::vector<int64_t> chunk_lo;
  std::vector<int64_t> chunk_val;
  int64_t task_values = 0;      // 32 x the longest lane job of every warp task, summed
  std::vector<int32_t> wt_cost;  // planner cost of every warp task (its most expensive lane)
  std::vector<int32_t> wt_len;   // longest lane job of every warp task
};

// Warp chunks of about `target` chunks over the plan's warp tasks (chunk c runs warp tasks
// [lo[c], lo[c+1]); val[c] is its first stored value).
void make_chunks(const Plan& P, int64_t target, std::vector<int64_t>& lo, std::vector<int64_t>& val);

// work of one warp chunk of the closed sigma, in the planner's cost units (about one unit
// per multiply-add or load of a lane's ket step): the total cut into about kTargetChunks
// chunks (four waves of 32 resident warps on each of 152 SMs), each within
// [kMinChunkCost, kChunkCost]
constexpr int64_t kChunkCost = int64_t(1) << 13;
constexpr int64_t kMinChunkCost = 256;
constexpr int64_t kTargetChunks = 4 * 152 * 32;


FCG_HD inline int64_t dense_block_index(int nmax1, int c, int op, int fba, int fbb, int fka, int fkb) {
  return ((((int64_t(c) * kNumOps + op) * nmax1 + fba) * nmax1 + fbb) * nmax1 + fka) * nmax1 + fkb;
}

// The term tables a term-sector record is made from, as plain arrays (host vectors or their
// device copies): term rows (kTrmCols each), dressing, W offsets [term][fb_a][fb_b] of the
// dressed cluster, the dense TDM block index and the blocks.
struct TermTables {
  const int32_t* trm;
  const TermDress* dress;
  const int64_t* w_index;
  const int32_t* blk;
  const BlockInfo* blocks;
  int nmax1;
};

// The term-sector record of term t between bra sector fb and ket sector fk (N x 2 each) and
// its multiply-add count per (bra, ket) pair (fma); false when a TDM block the term needs does
// not exist there.  The host and the device planner both make their records here.
FCG_HD inline bool term_sector_of(const TermTables& tt, int t, const int16_t* fb, const int16_t* fk,
                                  TermSector& ts, int64_t* fma) {
  const int32_t* r = tt.trm + int64_t(t) * kTrmCols;
  const TermDress& d = tt.dress[t];
  const int nmax1 = tt.nmax1;
  const int nbody = r[0];
  ts = TermSector{};
  const int pos = d.pos < 0 ? 0 : d.pos;
  const int cw = r[2 + pos], opw = r[6 + pos];
  const int bw = tt.blk[dense_block_index(nmax1, cw, opw, fb[2 * cw], fb[2 * cw + 1], fk[2 * cw], fk[2 * cw + 1])];
  const int64_t woff = tt.w_index[(int64_t(t) * nmax1 + fb[2 * cw]) * nmax1 + fb[2 * cw + 1]];
  if (bw < 0 || woff < 0) return false;
  ts.w_off = woff;
  ts.w_mb = tt.blocks[bw].mb;
  ts.cw = int8_t(cw);
  ts.rest_len = int16_t(nbody == 1 ? 1 : d.rest_len);
  ts.nrem = int8_t(nbody == 1 ? 0 : d.nrem);
  for (int q = 0; q < ts.nrem; ++q) {
    const int o = d.rem_pos[q];
    const int c = r[2 + o], op = r[6 + o];
    const int bl = tt.blk[dense_block_index(nmax1, c, op, fb[2 * c], fb[2 * c + 1], fk[2 * c], fk[2 * c + 1])];
    if (bl < 0) return false;
    ts.g_off[q] = tt.blocks[bl].off;
    ts.g_mb[q] = tt.blocks[bl].mb;
    ts.g_dim[q] = int16_t(tt.blocks[bl].nidx);
    ts.cr[q] = int8_t(c);
  }
  // compute_terms_state_sign (type_ClusteredTerm.jl:181-196) on the ket sector
  int sgn = 0;
  for (int o = 0; o < nbody; ++o)
    if (r[18 + o]) {
      int ne = 0;
      for (int ci = 0; ci < r[2 + o]; ++ci) ne += fk[2 * ci] + fk[2 * ci + 1];
      sgn ^= ne & 1;
    }
  ts.sign = int8_t(nbody == 1 ? 1 : (sgn ? -1 : 1));
  int64_t f = 0;
  if (ts.nrem == 1) f = ts.rest_len;
  if (ts.nrem == 2) f = ts.rest_len + ts.g_dim[1];
  if (ts.nrem == 3) f = ts.rest_len + int64_t(ts.g_dim[1]) * ts.g_dim[2] + ts.g_dim[2];
  *fma = f;
  return true;
}

// the reference's flop count of one (bra, ket) pair of term t: 2 x len(ints) for terms of two
// or more bodies
FCG_HD inline int64_t term_ref_flops(const int32_t* trm, int t) {
  const int32_t* r = trm + int64_t(t) * kTrmCols;
  if (r[0] <= 1) return 0;
  int64_t len = 1;
  for (int o = 0; o < 4; ++o) len *= r[22 + o];
  return 2 * len;
}

// The plan of one state in two parts: build_sectors checks the rows and finds the Fock sectors
// (enough for the diagonal and the open sigma); build_join adds the closed-sigma work items,
// lane jobs and warp chunks.  build_plan does both.
std::string build_sectors(const ProblemInfo& pi, int64_t n_cfg, const int16_t* fock, const int16_t* cfg, Plan& plan);
std::string build_join(const ProblemInfo& pi, const int16_t* fock, const int16_t* cfg, Plan& plan);
std::string build_plan(const ProblemInfo& pi, int64_t n_cfg, const int16_t* fock, const int16_t* cfg, Plan& plan);

// The term-sector record of term t between bra sector fb and ket sector fk (N x 2 each);
// false when a TDM block the term needs does not exist there.
bool make_term_sector(const ProblemInfo& pi, int t, const int16_t* fb, const int16_t* fk, TermSector& ts);
TermTables term_tables(const ProblemInfo& pi);

// the terms of the zero transfer (the diagonal's terms), in term order
std::vector<int32_t> zero_transfer_terms(const ProblemInfo& pi);

// Active-cluster sets of the terms and the term lists of every (transfer, set), in the order
// the closed-sigma join visits them: transfers ascending, then sets in order of first
// appearance among the terms, each list's terms ascending.
struct TermLists {
  std::vector<uint32_t> masks;       // active clusters of each set (bit c: cluster c)
  std::vector<int32_t> tr, set;      // transfer and set of every list
  std::vector<int32_t> off;          // list j holds terms[off[j], off[j+1])
  std::vector<int32_t> terms;
  std::vector<int32_t> first_of_tr;  // lists of transfer tr: [first_of_tr[tr], first_of_tr[tr+1])
};
std::string term_lists(const ProblemInfo& pi, TermLists& lists);

// Dressing plan of every term (which cluster is dressed, the W block of each of its
// TDM blocks); fills dress, w_index ([term][fb_a][fb_b] -> W offset or -1), jobs, w_total.
std::string build_dress(int N, const std::vector<int>& norb, int nmax, const std::vector<int32_t>& trm, int n_terms,
                        const std::vector<int32_t>& blk_index, const std::vector<BlockInfo>& blocks,
                        const std::vector<TermInfo>& terms, std::vector<TermDress>& dress,
                        std::vector<int64_t>& w_index, std::vector<DressJob>& jobs, int64_t& w_total);

}  // namespace fcg
