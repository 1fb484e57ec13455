// Internal types shared by the host planner (plan.cpp) and the CUDA side (fcg_gpu.cu).
#pragma once
#include <cstdint>
#include <string>
#include <vector>

namespace fcg {

constexpr int kMaxClusters = 8;
constexpr int kOpbCols = 10;
constexpr int kTrmCols = 28;
constexpr int kNumOps = 24;  // 22 op strings + "H" + "Hcmf"
constexpr int kOpH = 22;
constexpr int kOpHcmf = 23;

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

// A closed-sigma work item: every (bra in group, ket in group, term in list) triple.
struct WorkItem {
  int32_t bra_off;  // offset of the bra group in the permutation pool
  int32_t ket_off;  // offset of the ket group in the permutation pool
  int32_t nb;       // bra group size
  int32_t nk;       // ket group size
  int32_t tl_off;   // offset of the term list in the term pool
  int32_t nt;       // number of terms
  int32_t sb;       // bra sector id
  int32_t sk;       // ket sector id
};

// Host-side plan of the closed sigma for one state.
struct Plan {
  int N = 0;
  int64_t n_cfg = 0;
  // sectors (contiguous runs of rows)
  std::vector<int64_t> sec_start, sec_count;
  std::vector<int16_t> sec_fock;  // n_sec x N x 2
  // grouping pool: rows of every (sector, active set) sorted by spectator key
  std::vector<int32_t> perm_pool;
  // term lists per (transfer, active set)
  std::vector<int32_t> term_pool;
  // work items and the triple prefix sum
  std::vector<WorkItem> items;
  std::vector<int64_t> prefix;  // n_items + 1
  int64_t n_triples = 0;
  int64_t flops_ref = 0;
  // zero-transfer term list (diagonal)
  std::vector<int32_t> zero_terms;
};

// Builds the plan; returns an empty string on success or an error message.
std::string build_plan(int N, const std::vector<int>& norb, const std::vector<int32_t>& trm, int n_terms,
                       const std::vector<int16_t>& trans, int n_trans, int64_t n_cfg, const int16_t* fock,
                       const int16_t* cfg, Plan& plan);

}  // namespace fcg
