// Context object and helpers shared by the CUDA translation units.
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <string>
#include <vector>

#include "../../include/fcg_gpu.h"
#include "fcg_internal.h"

namespace fcg {

template <typename T>
struct DevBuf {
  T* p = nullptr;
  size_t n = 0;
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  ~DevBuf() { release(); }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
  cudaError_t alloc(size_t count) {
    if (count <= n && p) return cudaSuccess;
    release();
    size_t bytes = std::max<size_t>(count, 1) * sizeof(T);
    cudaError_t e = cudaMalloc(&p, bytes);
    if (e != cudaSuccess) {
      p = nullptr;
      return e;
    }
    n = count;
    return cudaSuccess;
  }
  cudaError_t upload(const T* h, size_t count, cudaStream_t s) {
    cudaError_t e = alloc(count);
    if (e != cudaSuccess) return e;
    if (count == 0) return cudaSuccess;
    return cudaMemcpyAsync(p, h, count * sizeof(T), cudaMemcpyHostToDevice, s);
  }
};

// Grow-only page-locked host buffer (fast device-to-host copies of large results).
template <typename T>
struct PinnedBuf {
  T* p = nullptr;
  size_t n = 0;
  PinnedBuf() = default;
  PinnedBuf(const PinnedBuf&) = delete;
  PinnedBuf& operator=(const PinnedBuf&) = delete;
  ~PinnedBuf() {
    if (p) cudaFreeHost(p);
  }
  cudaError_t alloc(size_t count) {
    if (count <= n && p) return cudaSuccess;
    if (p) cudaFreeHost(p);
    p = nullptr;
    n = 0;
    cudaError_t e = cudaMallocHost(reinterpret_cast<void**>(&p), std::max<size_t>(count, 1) * sizeof(T));
    if (e != cudaSuccess) {
      p = nullptr;
      return e;
    }
    n = count;
    return cudaSuccess;
  }
};

}  // namespace fcg

using namespace fcg;

struct fcg_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;      // stream every call runs on
  cudaStream_t own_stream = nullptr;  // the context's own stream
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  cudaEvent_t ev2 = nullptr, ev3 = nullptr;  // around one kernel inside a timed sequence
  // a second stream for work that overlaps the context stream's (created on first use),
  // and the events that fork it from and join it back to that stream
  cudaStream_t aux_stream = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  std::string err;
  // problem
  int N = 0;
  std::vector<int> norb;
  int nmax = 0;
  bool have_ops = false, have_terms = false, have_state = false;
  bool have_plan = false;             // the closed-sigma plan of the state (built on first use)
  std::vector<int16_t> h_fock, h_cfg;  // the state's rows, for that plan
  std::vector<int64_t> opb;
  std::vector<BlockInfo> h_blocks;
  std::vector<int32_t> h_blk_index;
  DevBuf<double> d_op64;
  DevBuf<float> d_op32;
  DevBuf<double> d_op_raw;  // the caller's TDM blob as given (fcg_set_ops), placed into d_op64 / d_op32
  DevBuf<BlockInfo> d_blocks;
  DevBuf<int32_t> d_blk_index;
  DevBuf<int32_t> d_norb;
  int n_terms = 0;
  std::vector<int32_t> trm;
  std::vector<TermInfo> terms;
  std::vector<double> term_ints_norm;  // Frobenius norm of each term's integrals (0 for 1-body terms; term_norms)
  int64_t n_ints = 0;
  std::vector<TermDress> dress;
  std::vector<int64_t> w_index;
  int64_t n_w = 0;
  DevBuf<TermInfo> d_terms;
  DevBuf<double> d_ints64;
  DevBuf<float> d_ints32;
  DevBuf<double> d_w64;
  DevBuf<float> d_w32;
  std::vector<DressJob> dress_jobs;  // W blocks to build (fcg_set_terms), built by the first fcg_state_set
  bool dressed = false;
  bool wmax_built = false;  // column maxima of the dressed operators (open-sigma screen)
  int n_trans = 0;
  std::vector<int16_t> trans;
  // state + plan
  int64_t n_cfg = 0;
  Plan plan;
  DevBuf<int16_t> d_cfg;
  DevBuf<int16_t> d_sec_fock;
  DevBuf<int32_t> d_row_sector;
  DevBuf<LaneJob> d_jobs;           // closed-sigma lane jobs, 32 per warp task
  DevBuf<int64_t> d_chunk_lo;       // first warp task of each warp chunk
  DevBuf<int64_t> d_chunk_val;      // first stored value of each warp chunk
  // sizes of the plan on the device (either planner): warp chunks of the chunk table, lane
  // jobs (with the idle lanes of the last warp task), warp tasks, their summed cost, work
  // items, term-sector records, permutation-pool entries
  int64_t n_chunks = 0, plan_jobs = 0, plan_wt = 0, plan_total_cost = 0, plan_items = 0, plan_ts = 0,
          plan_perm = 0;
  bool plan_on_device = true;           // the join runs on the device (dplan.cu), else plan.cpp
  DevBuf<int64_t> d_wt_cum, d_wt_vals;  // exclusive prefix of warp-task cost / stored values (device planner)
  // device planner: the term set's tables on the device (uploaded at the first plan after
  // fcg_set_ops / fcg_set_terms), the state's sector offsets, counters, grow-only arenas
  struct {
    bool ready = false;
    TermLists lists;
    int n_sets = 0, n_tl = 0, spec_bits = 0;
    DevBuf<int32_t> d_trm;
    DevBuf<TermDress> d_dress;
    DevBuf<int64_t> d_w_index;
    DevBuf<int16_t> d_trans;
    DevBuf<int32_t> d_first_of_tr, d_tl_tr, d_tl_set, d_tl_off, d_tl_terms, d_tl_nbody;
    DevBuf<uint8_t> d_spec_off;
    DevBuf<int64_t> d_sec_start, d_sec_count;
    DevBuf<unsigned long long> d_cnt;
    PinnedBuf<unsigned long long> h_cnt;
    DevBuf<unsigned char> arena[4], arena_rows;
    // the state's rows as given (kept for the host planner) and its sector table: open
    // addressing, Fock key -> sector (slots: key, sector or -1), built with the rows
    DevBuf<int16_t> d_fock_in, d_cfg_in;
    DevBuf<uint64_t> d_tkeys;
    DevBuf<int32_t> d_tvals;
    int64_t table_cap = 0;
    bool table_ready = false;
  } dj;
  // closed-sigma kernel tuning: candidate per precision (0 fp64, 1 fp32; -1 not yet tuned),
  // forced candidate (-1: auto), the finer chunk table of candidates 2-3, candidate timings
  int tuned[2] = {-1, -1};
  int tune_mode = -1;
  bool fine_built = false;
  DevBuf<int64_t> d_chunk_lo_fine, d_chunk_val_fine;
  int64_t n_chunks_fine = 0;
  float tune_ms[2][4] = {};
  DevBuf<int32_t> d_perm;
  DevBuf<TermSector> d_ts;
  DevBuf<unsigned char> d_group;    // entries of the last grouped closed sigma led by this context
  DevBuf<int32_t> d_group_cta;      // problem of every CTA of that launch
  DevBuf<int32_t> d_zero_terms;
  // stored Hamiltonian blocks of the state (fcg_cache_hamiltonian): per work item and
  // (bra, ket) pair, the sum over the item's terms of the matrix element
  bool have_hcache = false;
  int64_t hc_pairs = 0;
  DevBuf<double> d_hc64;
  DevBuf<float> d_hc32;
  // release = false keeps the buffers for the next state's blocks (grow-only; a cudaFree
  // would wait for every stream of the device)
  void drop_hcache(bool release = false) {
    have_hcache = false;
    hc_pairs = 0;
    if (!release) return;
    d_hc64.release();
    d_hc32.release();
  }
  // job lists of the set-up calls (fcg_set_ops, fcg_set_terms, fcg_cache_hamiltonian), grow-only
  DevBuf<unsigned char> scratch_a, scratch_b;
  template <class T>
  static cudaError_t stage(DevBuf<unsigned char>& buf, const T* h, size_t count, cudaStream_t s, T** d) {
    const cudaError_t e = buf.upload(reinterpret_cast<const unsigned char*>(h), count * sizeof(T), s);
    *d = reinterpret_cast<T*>(buf.p);
    return e;
  }
  // Davidson working buffers of this context, grow-only and reused by its later solves
  DevBuf<double> dav_V, dav_AV, dav_X, dav_tmp, dav_hd, dav_part, dav_rn, dav_out, dav_up;
  DevBuf<unsigned> dav_counters;
  PinnedBuf<double> dav_h_out, dav_h_up;
  // vectors
  DevBuf<double> d_in64, d_out64;  // column-major staging for host calls
  DevBuf<double> d_c64, d_s64;     // row-major fp64
  DevBuf<float> d_c32, d_s32;      // row-major fp32
  DevBuf<double> d_hd;
  // screening maxima: Gmax[i, k] = max_b |G[i, b, k]| per TDM block, Wmax likewise per W block
  std::vector<int64_t> gmax_off;   // per block
  std::vector<int64_t> wmax_index; // parallel to w_index
  DevBuf<double> d_gmax;
  DevBuf<double> d_wmax;
  // open sigma (FOIS) working set and last result
  DevBuf<OpenTerm> d_oterms;
  DevBuf<OpenItem> d_oitems;
  DevBuf<int64_t> d_oprefix;
  DevBuf<int64_t> d_ostrides;     // [n_bra_sectors][N]
  DevBuf<int2> d_ojobs;           // kept (row, open term) pairs
  DevBuf<int64_t> d_ojob_prefix;
  DevBuf<unsigned long long> d_hkeys;
  DevBuf<double> d_hvals;
  DevBuf<unsigned long long> d_okeys;
  DevBuf<double> d_ovals;
  DevBuf<unsigned long long> d_counters;
  DevBuf<unsigned char> d_scan_tmp;
  std::vector<int16_t> open_bra_fock;   // [n_bra_sectors][N][2]
  std::vector<int64_t> open_strides;    // [n_bra_sectors][N]
  std::vector<int64_t> open_dims;       // [n_bra_sectors][N]
  PinnedBuf<unsigned long long> open_keys;  // keys of the last open sigma, open_rows of them
  PinnedBuf<double> open_vals;              // [open_rows][R] row-major
  int64_t open_rows = 0;
  int open_R = 0;
  // block-sparse Tucker vector structure and its operator cache (bst.cu)
  bool have_bst = false;
  int64_t bst_core_total = 0;
  std::vector<BstBlock> bst_blocks;
  std::vector<BstGroup> bst_groups;
  std::vector<int32_t> bst_triples;     // [n][4] = {bra, ket, term, sign}
  std::vector<int32_t> bst_small, bst_large;  // groups run one CTA per group from shared / global memory
  std::vector<int64_t> bst_small_ptr;         // bst_small in buckets of workspace size: [ptr[i], ptr[i+1])
  int32_t bst_ws_large = 0;
  std::vector<int32_t> bst_bra_ids, bst_bra_glist;  // bra block of each chunk, and the chunks' groups
  std::vector<int64_t> bst_bra_ptr;                 // chunk c holds bst_bra_glist[ptr[c], ptr[c+1])
  int bst_bra_slice = 0, bst_bra_acc = 0;           // shared-memory bytes per warp slice / accumulator
  int bst_list_R = 0;          // R and element size the lists were made for
  size_t bst_list_elem = 0;
  DevBuf<BstBlock> d_bst_blocks;
  DevBuf<BstGroup> d_bst_groups;
  DevBuf<int32_t> d_bst_small, d_bst_large, d_bst_bra_ids, d_bst_bra_glist;
  DevBuf<unsigned> d_bst_next;  // work counter of the global-workspace sigma launch
  DevBuf<int64_t> d_bst_bra_ptr;
  DevBuf<double> d_bst_factors;
  DevBuf<int32_t> d_bst_perm;      // actives-first index tables per (block, active clusters)
  DevBuf<double> d_bst_op64, d_bst_s64;
  DevBuf<float> d_bst_op32, d_bst_s32;
  DevBuf<double> d_bst_in64, d_bst_out64, d_bst_ws64;
  DevBuf<float> d_bst_in32, d_bst_out32, d_bst_ws32;
  // tensor-core groups of the float sigma: group ids, their X workspace offsets, the 128 x N
  // tile jobs {tc index, group, m0, n0}, algorithmic and executed MMA flops per sigma
  bool bst_tc_on = true;
  std::vector<int32_t> bst_tc;
  std::vector<int64_t> bst_tc_ws_off;
  std::vector<int32_t> bst_tc_jobs;
  int64_t bst_tc_ws_total = 0, bst_tc_flops = 0, bst_tc_mma_flops = 0;
  DevBuf<int32_t> d_bst_tc, d_bst_tc_jobs;
  DevBuf<int64_t> d_bst_tc_ws_off;
  DevBuf<float> d_bst_tc_ws;
  DevBuf<unsigned> d_bst_tc_err;
  // the last compressed first-order space (bst_fois.cu), in the fcg_bst_set layout
  struct {
    int R = 0;
    int64_t n_blocks = 0, core_total = 0;
    std::vector<int16_t> fock;
    std::vector<int64_t> blocks, factor_off;
    std::vector<double> factors, cores;
  } fois;
  fcg_stats stats{};
};

// closed sigma on device vectors (column-major n_cfg x R) queued on ctx->stream, without the
// host wait of fcg_sigma_closed_device; for drivers that keep working on the same stream
// (fcg_gpu.cu)
int sigma_closed_device_async(fcg_ctx* ctx, int R, const double* d_c, double* d_sigma, int precision);

// The dressed operators of the term set, and the closed-sigma plan of the state, built on
// first use (fcg_gpu.cu)
int ensure_dressed(fcg_ctx* ctx);
int ensure_wmax(fcg_ctx* ctx);  // the open sigma's column maxima of the dressed operators
int ensure_plan(fcg_ctx* ctx);
ProblemInfo problem_info(fcg_ctx* ctx);
int term_norms(fcg_ctx* ctx);

// The closed-sigma join of the state on the device (dplan.cu): fills d_perm, d_ts, d_jobs,
// d_chunk_lo / d_chunk_val, d_wt_cum / d_wt_vals and the plan sizes; and a chunk table of
// about `target` warp chunks over its warp tasks.
int build_join_device(fcg_ctx* ctx);

// The rows of a state checked, their sectors found and the sector table built on the device
// (dplan.cu); same results and messages as build_sectors.
int state_rows_device(fcg_ctx* ctx, int64_t n_cfg, const int16_t* fock, const int16_t* cfg);
int device_chunks(fcg_ctx* ctx, int64_t target, DevBuf<int64_t>& lo, DevBuf<int64_t>& val, int64_t* n_chunks);

// BST sigma on device vectors [R][core_total] queued on ctx->stream without the host wait
// (timed: CUDA events around the kernels), and the check of the tensor-core error flag (one
// host wait) (bst.cu)
int bst_sigma_device_async(fcg_ctx* ctx, int R, const double* d_cores, double* d_sigma, int precision, bool timed);
int bst_tc_check(fcg_ctx* ctx);

// fcg_bst_set with an optional caller-given triple list {bra, ket, term} (n_triples of them)
// in place of the check_term enumeration, or (split > 0) with only the triples that couple a
// block of [0, split) with a block of [split, n_blocks) (bst.cu)
int bst_set_impl(fcg_ctx* ctx, int nbody, int64_t n_blocks, const int16_t* fock, const int64_t* blocks,
                 const int64_t* factor_off, int64_t n_factors, const double* factors, const int32_t* triples,
                 int64_t n_triples, int64_t* core_total, int64_t split = 0);

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

