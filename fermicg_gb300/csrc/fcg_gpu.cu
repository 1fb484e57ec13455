// GB300 (sm_103a) TPSCI sigma build behind the C ABI of include/fcg_gpu.h.
//
// Device layout (one context, one stream):
//   op data      the TDM blocks of every cluster in one blob, float64 and a float32 copy,
//                block (p, I, J) at off + p + nidx*(I + mb*J)
//   block index  dense int32 table (cluster, op, fb_a, fb_b, fk_a, fk_b) -> block id
//   terms        TermInfo per ClusteredTerm, integrals in a float64 blob (+ float32 copy)
//   state        local states int16 [n_cfg][N]; sector fock int16 [n_sec][N][2]
//   plan         work items (bra group x ket group x term list), their triple prefix sum,
//                the grouping permutation pool and the term pool (plan.cpp)
//   vectors      coefficients / sigma row-major [n_cfg][R] in the compute precision
//
// Kernels:
//   closed_sigma_kernel  one pass over the flattened (work item, bra, ket, term)
//                        triple space; each CTA takes a fixed chunk (load balance is
//                        exact), contracts term integrals with the TDM columns
//                        (contract_matrix_element, src/tpsci_inner.jl:10-216) and
//                        scatters sigma with warp-segmented sums + one atomic per run.
//   diag_kernels         compute_diagonal (src/tpsci_outer.jl:694-757).
//   pack / unpack        column-major float64 <-> row-major compute precision.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/fcg_gpu.h"
#include "fcg_internal.h"

using namespace fcg;

namespace {

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

}  // namespace

struct fcg_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;       // stream every call runs on
  cudaStream_t own_stream = nullptr;   // the context's own stream
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  std::string err;
  // problem
  int N = 0;
  std::vector<int> norb;
  int nmax = 0;
  bool have_ops = false, have_terms = false, have_state = false;
  std::vector<int64_t> opb;
  DevBuf<double> d_op64;
  DevBuf<float> d_op32;
  DevBuf<BlockInfo> d_blocks;
  DevBuf<int32_t> d_blk_index;
  int n_terms = 0;
  std::vector<int32_t> trm;
  std::vector<TermInfo> terms;
  DevBuf<TermInfo> d_terms;
  DevBuf<double> d_ints64;
  DevBuf<float> d_ints32;
  int n_trans = 0;
  std::vector<int16_t> trans;
  // state + plan
  int64_t n_cfg = 0;
  Plan plan;
  DevBuf<int16_t> d_cfg;
  DevBuf<int16_t> d_sec_fock;
  DevBuf<int32_t> d_row_sector;
  DevBuf<WorkItem> d_items;
  DevBuf<int64_t> d_prefix;
  DevBuf<int32_t> d_perm;
  DevBuf<int32_t> d_term_pool;
  DevBuf<int32_t> d_zero_terms;
  // vectors
  DevBuf<double> d_in64, d_out64;  // column-major staging for host calls
  DevBuf<double> d_c64, d_s64;     // row-major fp64
  DevBuf<float> d_c32, d_s32;      // row-major fp32
  DevBuf<double> d_hd;
  fcg_stats stats{};
};

#define FCG_CUDA(call)                                                                       \
  do {                                                                                       \
    cudaError_t e_ = (call);                                                                 \
    if (e_ != cudaSuccess) {                                                                 \
      ctx->err = std::string(#call) + ": " + cudaGetErrorString(e_);                         \
      return e_ == cudaErrorMemoryAllocation ? FCG_ENOMEM : FCG_ECUDA;                       \
    }                                                                                        \
  } while (0)

#define FCG_REQUIRE(cond, code, msg) \
  do {                               \
    if (!(cond)) {                   \
      ctx->err = (msg);              \
      return (code);                 \
    }                                \
  } while (0)

// ---------------------------------------------------------------------------------------
// device code
namespace {

struct SigmaParams {
  const WorkItem* items;
  const int64_t* prefix;
  int64_t n_items;
  int64_t n_triples;
  const int32_t* perm;
  const int32_t* term_pool;
  const TermInfo* terms;
  const BlockInfo* blocks;
  const int32_t* blk_index;
  const int16_t* cfg;       // [n_cfg][N]
  const int16_t* sec_fock;  // [n_sec][N][2]
  int N;
  int nmax1;  // nmax + 1
  int R;
};

__device__ __forceinline__ int block_of(const SigmaParams& p, int c, int op, const int16_t* fb,
                                        const int16_t* fk) {
  int s = p.nmax1;
  int64_t i = ((((int64_t(c) * kNumOps + op) * s + fb[2 * c]) * s + fb[2 * c + 1]) * s + fk[2 * c]) * s +
              fk[2 * c + 1];
  return p.blk_index[i];
}

// compute_terms_state_sign (src/type_ClusteredTerm.jl:181-196) from the ket sector
__device__ __forceinline__ int term_sign(const TermInfo& tm, const int16_t* fk) {
  int s = 0;
  for (int o = 0; o < tm.nbody; ++o) {
    if (tm.parity[o]) {
      int ne = 0;
      for (int ci = 0; ci < tm.c[o]; ++ci) ne += fk[2 * ci] + fk[2 * ci + 1];
      s ^= ne & 1;
    }
  }
  return s ? -1 : 1;
}

// One matrix element <bra|term|ket>: ints contracted with one TDM column per active
// cluster, in the order of _contract (src/tpsci_inner.jl:270-329).
template <typename T>
__device__ T matrix_element(const SigmaParams& p, const TermInfo& tm, const T* __restrict__ op,
                            const T* __restrict__ ints, const int16_t* fb, const int16_t* fk, int b, int k) {
  const T* g[4];
  int d[4];
  for (int o = 0; o < tm.nbody; ++o) {
    int c = tm.c[o];
    int bl = block_of(p, c, tm.op[o], fb, fk);
    if (bl < 0) return T(0);
    BlockInfo bi = p.blocks[bl];
    int sb = p.cfg[int64_t(b) * p.N + c];
    int sk = p.cfg[int64_t(k) * p.N + c];
    g[o] = op + bi.off + int64_t(bi.nidx) * (sb + int64_t(bi.mb) * sk);
    d[o] = bi.nidx;
  }
  if (tm.nbody == 1) return g[0][0];
  const T* v = ints + tm.ints_off;
  T me = T(0);
  if (tm.nbody == 2) {
    for (int j = 0; j < d[1]; ++j) {
      T acc = T(0);
      const T* vj = v + d[0] * j;
      for (int i = 0; i < d[0]; ++i) acc = fma(g[0][i], __ldg(vj + i), acc);
      me = fma(acc, g[1][j], me);
    }
  } else if (tm.nbody == 3) {
    for (int kk = 0; kk < d[2]; ++kk) {
      T acck = T(0);
      for (int j = 0; j < d[1]; ++j) {
        T acc = T(0);
        const T* vj = v + d[0] * (j + d[1] * kk);
        for (int i = 0; i < d[0]; ++i) acc = fma(g[0][i], __ldg(vj + i), acc);
        acck = fma(acc, g[1][j], acck);
      }
      me = fma(acck, g[2][kk], me);
    }
  } else {
    for (int l = 0; l < d[3]; ++l) {
      T accl = T(0);
      for (int kk = 0; kk < d[2]; ++kk) {
        T acck = T(0);
        for (int j = 0; j < d[1]; ++j) {
          T acc = T(0);
          const T* vj = v + d[0] * (j + d[1] * (kk + d[2] * l));
          for (int i = 0; i < d[0]; ++i) acc = fma(g[0][i], __ldg(vj + i), acc);
          acck = fma(acc, g[1][j], acck);
        }
        accl = fma(acck, g[2][kk], accl);
      }
      me = fma(accl, g[3][l], me);
    }
  }
  return term_sign(tm, fk) * me;
}

constexpr int kSigmaThreads = 256;
constexpr int kSigmaIters = 8;
constexpr int64_t kSigmaChunk = int64_t(kSigmaThreads) * kSigmaIters;
constexpr int kMaxR = 16;

// largest w in [lo, hi] with prefix[w] <= x
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

template <typename T, int RR>
__global__ void __launch_bounds__(kSigmaThreads) closed_sigma_kernel(SigmaParams p, const T* __restrict__ op,
                                                                      const T* __restrict__ ints,
                                                                      const T* __restrict__ cin,
                                                                      T* __restrict__ sig) {
  const int64_t s0 = int64_t(blockIdx.x) * kSigmaChunk;
  const int64_t e0 = (s0 + kSigmaChunk < p.n_triples) ? s0 + kSigmaChunk : p.n_triples;
  __shared__ int64_t w_lo, w_hi;
  if (threadIdx.x == 0) {
    w_lo = find_item(p.prefix, 0, p.n_items - 1, s0);
    w_hi = find_item(p.prefix, w_lo, p.n_items - 1, e0 - 1);
  }
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int R = RR > 0 ? RR : p.R;
  int64_t w = w_lo;
  for (int it = 0; it < kSigmaIters; ++it) {
    const int64_t idx = s0 + int64_t(it) * kSigmaThreads + threadIdx.x;
    int key = -1;
    T val[RR > 0 ? RR : kMaxR];
#pragma unroll
    for (int r = 0; r < (RR > 0 ? RR : kMaxR); ++r) val[r] = T(0);
    if (idx < e0) {
      w = find_item(p.prefix, w, w_hi, idx);
      const WorkItem wi = p.items[w];
      const int64_t local = idx - p.prefix[w];
      // triple order inside an item: term fastest, then ket, then bra
      const int ti = int(local % wi.nt);
      const int64_t rest = local / wi.nt;
      const int kj = int(rest % wi.nk);
      const int bj = int(rest / wi.nk);
      const int b = p.perm[wi.bra_off + bj];
      const int k = p.perm[wi.ket_off + kj];
      const TermInfo tm = p.terms[p.term_pool[wi.tl_off + ti]];
      const int16_t* fb = p.sec_fock + int64_t(wi.sb) * 2 * p.N;
      const int16_t* fk = p.sec_fock + int64_t(wi.sk) * 2 * p.N;
      const T me = matrix_element<T>(p, tm, op, ints, fb, fk, b, k);
      key = b;
      const T* ck = cin + int64_t(k) * R;
#pragma unroll
      for (int r = 0; r < (RR > 0 ? RR : kMaxR); ++r)
        if (r < R) val[r] = me * ck[r];
    }
    // segmented suffix sums over runs of equal bra rows, then one atomic per run.
    // The same bra can come back later in the warp (a new work item), so a lane
    // only sums up to the next run head, never across another run.
    const int prev = __shfl_up_sync(0xffffffffu, key, 1);
    const bool head = (lane == 0) || (prev != key);
    const unsigned heads = __ballot_sync(0xffffffffu, head);
    const unsigned after = heads & ~((2u << lane) - 1u);
    const int seg_end = after ? (__ffs(int(after)) - 1) : 32;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
      const bool take = (lane + off < seg_end);
#pragma unroll
      for (int r = 0; r < (RR > 0 ? RR : kMaxR); ++r) {
        if (r < R) {
          T vo = __shfl_down_sync(0xffffffffu, val[r], off);
          if (take) val[r] += vo;
        }
      }
    }
    if (head && key >= 0) {
#pragma unroll
      for (int r = 0; r < (RR > 0 ? RR : kMaxR); ++r)
        if (r < R) atomicAdd(sig + int64_t(key) * R + r, val[r]);
    }
  }
}

template <typename T>
__global__ void pack_in_kernel(const double* __restrict__ c, T* __restrict__ out, int64_t n, int R) {
  int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n * R) return;
  int64_t row = i / R;
  int r = int(i - row * R);
  out[i] = T(c[row + n * r]);
}

template <typename T>
__global__ void unpack_out_kernel(const T* __restrict__ s, double* __restrict__ out, int64_t n, int R) {
  int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n * R) return;
  int64_t row = i % n;
  int r = int(i / n);
  out[i] = double(s[row * R + r]);
}

__global__ void diag_terms_kernel(SigmaParams p, const double* __restrict__ op, const double* __restrict__ ints,
                                  const int32_t* __restrict__ zero_terms, int n_zero,
                                  const int32_t* __restrict__ row_sector, int64_t n, double* __restrict__ hd) {
  int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int16_t* f = p.sec_fock + int64_t(row_sector[i]) * 2 * p.N;
  double s = 0.0;
  for (int z = 0; z < n_zero; ++z) {
    const TermInfo tm = p.terms[zero_terms[z]];
    s += matrix_element<double>(p, tm, op, ints, f, f, int(i), int(i));
  }
  hd[i] = s;
}

__global__ void diag_op_kernel(SigmaParams p, const double* __restrict__ op, int opid,
                               const int32_t* __restrict__ row_sector, int64_t n, double* __restrict__ hd,
                               int* __restrict__ missing) {
  int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int16_t* f = p.sec_fock + int64_t(row_sector[i]) * 2 * p.N;
  double s = 0.0;
  for (int c = 0; c < p.N; ++c) {
    int bl = block_of(p, c, opid, f, f);
    if (bl < 0) {
      atomicExch(missing, 1);
      continue;
    }
    BlockInfo bi = p.blocks[bl];
    int st = p.cfg[i * p.N + c];
    s += op[bi.off + st + int64_t(bi.mb) * st];
  }
  hd[i] = s;
}

}  // namespace

// ---------------------------------------------------------------------------------------
// host side

static SigmaParams make_params(fcg_ctx* ctx, int R) {
  SigmaParams p{};
  p.items = ctx->d_items.p;
  p.prefix = ctx->d_prefix.p;
  p.n_items = int64_t(ctx->plan.items.size());
  p.n_triples = ctx->plan.n_triples;
  p.perm = ctx->d_perm.p;
  p.term_pool = ctx->d_term_pool.p;
  p.terms = ctx->d_terms.p;
  p.blocks = ctx->d_blocks.p;
  p.blk_index = ctx->d_blk_index.p;
  p.cfg = ctx->d_cfg.p;
  p.sec_fock = ctx->d_sec_fock.p;
  p.N = ctx->N;
  p.nmax1 = ctx->nmax + 1;
  p.R = R;
  return p;
}

extern "C" {

int fcg_version(void) { return 1; }

int fcg_ctx_create(int device, fcg_ctx** out) {
  if (!out) return FCG_EINVAL;
  *out = nullptr;
  fcg_ctx* ctx = new fcg_ctx();
  ctx->device = device;
  cudaError_t e = cudaSetDevice(device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->own_stream, cudaStreamNonBlocking);
  ctx->stream = ctx->own_stream;
  if (e == cudaSuccess) e = cudaEventCreate(&ctx->ev0);
  if (e == cudaSuccess) e = cudaEventCreate(&ctx->ev1);
  if (e != cudaSuccess) {
    delete ctx;
    return FCG_ECUDA;
  }
  *out = ctx;
  return FCG_OK;
}

int fcg_ctx_destroy(fcg_ctx* ctx) {
  if (!ctx) return FCG_OK;
  cudaSetDevice(ctx->device);
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  if (ctx->ev0) cudaEventDestroy(ctx->ev0);
  if (ctx->ev1) cudaEventDestroy(ctx->ev1);
  if (ctx->own_stream) cudaStreamDestroy(ctx->own_stream);
  delete ctx;
  return FCG_OK;
}

const char* fcg_last_error(const fcg_ctx* ctx) { return ctx ? ctx->err.c_str() : "null context"; }

int fcg_set_stream(fcg_ctx* ctx, void* stream) {
  if (!ctx) return FCG_EINVAL;
  FCG_CUDA(cudaSetDevice(ctx->device));
  FCG_CUDA(cudaStreamSynchronize(ctx->stream));
  ctx->stream = stream ? static_cast<cudaStream_t>(stream) : ctx->own_stream;
  return FCG_OK;
}

int fcg_set_ops(fcg_ctx* ctx, int n_clusters, const int32_t* cluster_norb, int64_t n_blocks,
                const int64_t* block_table, int64_t n_data, const double* data) {
  if (!ctx) return FCG_EINVAL;
  FCG_REQUIRE(n_clusters > 0 && n_clusters <= kMaxClusters, FCG_ELIMIT, "n_clusters must be in [1, 8]");
  FCG_REQUIRE(cluster_norb && block_table && (data || n_data == 0), FCG_EINVAL, "null pointer");
  FCG_CUDA(cudaSetDevice(ctx->device));
  ctx->N = n_clusters;
  ctx->norb.assign(cluster_norb, cluster_norb + n_clusters);
  ctx->nmax = 0;
  for (int n : ctx->norb) {
    FCG_REQUIRE(n > 0 && n <= 15, FCG_ELIMIT, "orbitals per cluster must be in [1, 15]");
    ctx->nmax = std::max(ctx->nmax, n);
  }
  ctx->opb.assign(block_table, block_table + n_blocks * kOpbCols);
  const int s = ctx->nmax + 1;
  std::vector<int32_t> index(size_t(n_clusters) * kNumOps * s * s * s * s, -1);
  std::vector<BlockInfo> blocks(n_blocks);
  for (int64_t b = 0; b < n_blocks; ++b) {
    const int64_t* r = &ctx->opb[b * kOpbCols];
    FCG_REQUIRE(r[0] >= 0 && r[0] < n_clusters && r[1] >= 0 && r[1] < kNumOps, FCG_EINVAL,
                "block table: bad cluster or op id");
    for (int i = 2; i < 6; ++i)
      FCG_REQUIRE(r[i] >= 0 && r[i] <= ctx->norb[r[0]], FCG_EINVAL, "block table: bad Fock sector");
    FCG_REQUIRE(r[6] > 0 && r[7] > 0 && r[8] > 0 && r[7] <= 256 && r[8] <= 256, FCG_ELIMIT,
                "block table: block dims must be in [1, 256]");
    FCG_REQUIRE(r[9] >= 0 && r[9] + r[6] * r[7] * r[8] <= n_data, FCG_EINVAL, "block table: data out of range");
    int64_t i = ((((r[0] * kNumOps + r[1]) * s + r[2]) * s + r[3]) * s + r[4]) * s + r[5];
    index[i] = int32_t(b);
    blocks[b] = BlockInfo{r[9], int32_t(r[6]), int32_t(r[7]), int32_t(r[8]), 0};
  }
  std::vector<float> d32(data, data + n_data);
  FCG_CUDA(ctx->d_op64.upload(data, n_data, ctx->stream));
  FCG_CUDA(ctx->d_op32.upload(d32.data(), n_data, ctx->stream));
  FCG_CUDA(ctx->d_blocks.upload(blocks.data(), blocks.size(), ctx->stream));
  FCG_CUDA(ctx->d_blk_index.upload(index.data(), index.size(), ctx->stream));
  FCG_CUDA(cudaStreamSynchronize(ctx->stream));
  ctx->have_ops = true;
  ctx->have_state = false;
  return FCG_OK;
}

int fcg_set_terms(fcg_ctx* ctx, int n_terms, const int32_t* term_table, int64_t n_ints, const double* ints,
                  int n_transfers, const int16_t* transfers) {
  if (!ctx) return FCG_EINVAL;
  FCG_REQUIRE(ctx->have_ops, FCG_ESTATE, "fcg_set_ops must come first");
  FCG_REQUIRE(term_table && transfers && (ints || n_ints == 0) && n_terms >= 0 && n_transfers > 0, FCG_EINVAL,
              "bad term arguments");
  FCG_CUDA(cudaSetDevice(ctx->device));
  ctx->n_terms = n_terms;
  ctx->trm.assign(term_table, term_table + int64_t(n_terms) * kTrmCols);
  ctx->n_trans = n_transfers;
  ctx->trans.assign(transfers, transfers + int64_t(n_transfers) * ctx->N * 2);
  ctx->terms.assign(n_terms, TermInfo{});
  for (int t = 0; t < n_terms; ++t) {
    const int32_t* r = &ctx->trm[int64_t(t) * kTrmCols];
    TermInfo& tm = ctx->terms[t];
    FCG_REQUIRE(r[0] >= 1 && r[0] <= 4, FCG_EINVAL, "term nbody must be in [1, 4]");
    FCG_REQUIRE(r[1] >= 0 && r[1] < n_transfers, FCG_EINVAL, "term transfer id out of range");
    tm.nbody = int8_t(r[0]);
    int64_t len = 1;
    for (int o = 0; o < 4; ++o) {
      tm.c[o] = int8_t(o < r[0] ? r[2 + o] : 0);
      tm.op[o] = int8_t(o < r[0] ? r[6 + o] : 0);
      tm.parity[o] = int8_t(o < r[0] ? r[18 + o] : 0);
      tm.dim[o] = int16_t(r[22 + o]);
      if (o < r[0]) {
        FCG_REQUIRE(r[2 + o] >= 0 && r[2 + o] < ctx->N, FCG_EINVAL, "term cluster out of range");
        FCG_REQUIRE(r[6 + o] >= 0 && r[6 + o] < kNumOps, FCG_EINVAL, "term op id out of range");
        FCG_REQUIRE(o == 0 || r[2 + o] > r[1 + o], FCG_EINVAL, "term clusters must increase");
      }
      len *= r[22 + o];
    }
    tm.ints_off = int64_t(uint32_t(r[26])) | (int64_t(r[27]) << 32);
    if (r[0] > 1) FCG_REQUIRE(tm.ints_off >= 0 && tm.ints_off + len <= n_ints, FCG_EINVAL, "term ints out of range");
  }
  std::vector<float> i32(ints, ints + n_ints);
  FCG_CUDA(ctx->d_terms.upload(ctx->terms.data(), ctx->terms.size(), ctx->stream));
  FCG_CUDA(ctx->d_ints64.upload(ints, n_ints, ctx->stream));
  FCG_CUDA(ctx->d_ints32.upload(i32.data(), n_ints, ctx->stream));
  FCG_CUDA(cudaStreamSynchronize(ctx->stream));
  ctx->have_terms = true;
  ctx->have_state = false;
  return FCG_OK;
}

int fcg_state_set(fcg_ctx* ctx, int64_t n_cfg, const int16_t* fock, const int16_t* cfg) {
  if (!ctx) return FCG_EINVAL;
  FCG_REQUIRE(ctx->have_ops && ctx->have_terms, FCG_ESTATE, "upload ops and terms first");
  FCG_REQUIRE(n_cfg > 0 && fock && cfg, FCG_EINVAL, "empty state");
  FCG_CUDA(cudaSetDevice(ctx->device));
  auto t0 = std::chrono::steady_clock::now();
  std::string msg = build_plan(ctx->N, ctx->norb, ctx->trm, ctx->n_terms, ctx->trans, ctx->n_trans, n_cfg, fock,
                               cfg, ctx->plan);
  FCG_REQUIRE(msg.empty(), FCG_EINVAL, msg);
  for (int64_t i = 0; i < n_cfg; ++i)
    for (int c = 0; c < ctx->N; ++c) {
      int16_t fa = fock[(i * ctx->N + c) * 2], fbb = fock[(i * ctx->N + c) * 2 + 1];
      FCG_REQUIRE(fa <= ctx->norb[c] && fbb <= ctx->norb[c], FCG_EINVAL, "Fock sector exceeds cluster size");
    }
  const Plan& P = ctx->plan;
  std::vector<int32_t> row_sector(n_cfg);
  for (size_t s = 0; s < P.sec_start.size(); ++s)
    for (int64_t i = 0; i < P.sec_count[s]; ++i) row_sector[P.sec_start[s] + i] = int32_t(s);
  ctx->n_cfg = n_cfg;
  FCG_CUDA(ctx->d_cfg.upload(cfg, size_t(n_cfg) * ctx->N, ctx->stream));
  FCG_CUDA(ctx->d_sec_fock.upload(P.sec_fock.data(), P.sec_fock.size(), ctx->stream));
  FCG_CUDA(ctx->d_row_sector.upload(row_sector.data(), row_sector.size(), ctx->stream));
  FCG_CUDA(ctx->d_items.upload(P.items.data(), P.items.size(), ctx->stream));
  FCG_CUDA(ctx->d_prefix.upload(P.prefix.data(), P.prefix.size(), ctx->stream));
  FCG_CUDA(ctx->d_perm.upload(P.perm_pool.data(), P.perm_pool.size(), ctx->stream));
  FCG_CUDA(ctx->d_term_pool.upload(P.term_pool.data(), P.term_pool.size(), ctx->stream));
  FCG_CUDA(ctx->d_zero_terms.upload(P.zero_terms.data(), P.zero_terms.size(), ctx->stream));
  FCG_CUDA(cudaStreamSynchronize(ctx->stream));
  auto t1 = std::chrono::steady_clock::now();
  ctx->stats.n_cfg = n_cfg;
  ctx->stats.n_sectors = int64_t(P.sec_start.size());
  ctx->stats.n_work_items = int64_t(P.items.size());
  ctx->stats.n_triples = P.n_triples;
  ctx->stats.flops_reference = P.flops_ref;
  ctx->stats.plan_seconds = std::chrono::duration<double>(t1 - t0).count();
  ctx->have_state = true;
  return FCG_OK;
}

}  // extern "C"

template <typename T>
static int launch_closed(fcg_ctx* ctx, int R, const T* op, const T* ints, const T* cin, T* sig) {
  SigmaParams p = make_params(ctx, R);
  FCG_CUDA(cudaMemsetAsync(sig, 0, sizeof(T) * size_t(ctx->n_cfg) * R, ctx->stream));
  int launches = 0;
  if (p.n_triples > 0) {
    int64_t grid = (p.n_triples + kSigmaChunk - 1) / kSigmaChunk;
    FCG_REQUIRE(grid < (int64_t(1) << 31), FCG_ELIMIT, "too many triples for one launch");
    FCG_CUDA(cudaEventRecord(ctx->ev0, ctx->stream));
    switch (R) {
      case 1: closed_sigma_kernel<T, 1><<<unsigned(grid), kSigmaThreads, 0, ctx->stream>>>(p, op, ints, cin, sig); break;
      case 2: closed_sigma_kernel<T, 2><<<unsigned(grid), kSigmaThreads, 0, ctx->stream>>>(p, op, ints, cin, sig); break;
      case 4: closed_sigma_kernel<T, 4><<<unsigned(grid), kSigmaThreads, 0, ctx->stream>>>(p, op, ints, cin, sig); break;
      default: closed_sigma_kernel<T, 0><<<unsigned(grid), kSigmaThreads, 0, ctx->stream>>>(p, op, ints, cin, sig); break;
    }
    FCG_CUDA(cudaGetLastError());
    FCG_CUDA(cudaEventRecord(ctx->ev1, ctx->stream));
    launches = 1;
  }
  ctx->stats.kernel_launches = launches;
  return FCG_OK;
}

static int sigma_device_impl(fcg_ctx* ctx, int R, const double* d_c, double* d_sigma, int precision) {
  FCG_REQUIRE(ctx->have_state, FCG_ESTATE, "fcg_state_set must come first");
  FCG_REQUIRE(R >= 1 && R <= kMaxR, FCG_ELIMIT, "R must be in [1, 16]");
  FCG_REQUIRE(precision == FCG_FP64 || precision == FCG_FP32, FCG_EINVAL, "unknown precision");
  const int64_t n = ctx->n_cfg;
  const int64_t nR = n * R;
  const unsigned g = unsigned((nR + 255) / 256);
  ctx->stats.last_kernel_ms = 0.0;
  int rc;
  if (precision == FCG_FP64) {
    FCG_CUDA(ctx->d_c64.alloc(nR));
    FCG_CUDA(ctx->d_s64.alloc(nR));
    pack_in_kernel<double><<<g, 256, 0, ctx->stream>>>(d_c, ctx->d_c64.p, n, R);
    rc = launch_closed<double>(ctx, R, ctx->d_op64.p, ctx->d_ints64.p, ctx->d_c64.p, ctx->d_s64.p);
    if (rc) return rc;
    unpack_out_kernel<double><<<g, 256, 0, ctx->stream>>>(ctx->d_s64.p, d_sigma, n, R);
  } else {
    FCG_CUDA(ctx->d_c32.alloc(nR));
    FCG_CUDA(ctx->d_s32.alloc(nR));
    pack_in_kernel<float><<<g, 256, 0, ctx->stream>>>(d_c, ctx->d_c32.p, n, R);
    rc = launch_closed<float>(ctx, R, ctx->d_op32.p, ctx->d_ints32.p, ctx->d_c32.p, ctx->d_s32.p);
    if (rc) return rc;
    unpack_out_kernel<float><<<g, 256, 0, ctx->stream>>>(ctx->d_s32.p, d_sigma, n, R);
  }
  FCG_CUDA(cudaGetLastError());
  ctx->stats.kernel_launches += 2;
  FCG_CUDA(cudaStreamSynchronize(ctx->stream));
  if (ctx->plan.n_triples > 0) {
    float ms = 0.f;
    FCG_CUDA(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
    ctx->stats.last_kernel_ms = ms;
  }
  return FCG_OK;
}

extern "C" {

int fcg_sigma_closed_device(fcg_ctx* ctx, int R, const double* d_c, double* d_sigma, int precision) {
  if (!ctx) return FCG_EINVAL;
  FCG_REQUIRE(d_c && d_sigma, FCG_EINVAL, "null pointer");
  FCG_CUDA(cudaSetDevice(ctx->device));
  return sigma_device_impl(ctx, R, d_c, d_sigma, precision);
}

int fcg_sigma_closed(fcg_ctx* ctx, int R, const double* c, double* sigma, int precision) {
  if (!ctx) return FCG_EINVAL;
  FCG_REQUIRE(c && sigma, FCG_EINVAL, "null pointer");
  FCG_REQUIRE(ctx->have_state, FCG_ESTATE, "fcg_state_set must come first");
  FCG_REQUIRE(R >= 1 && R <= kMaxR, FCG_ELIMIT, "R must be in [1, 16]");
  FCG_CUDA(cudaSetDevice(ctx->device));
  const size_t nR = size_t(ctx->n_cfg) * R;
  FCG_CUDA(ctx->d_in64.alloc(nR));
  FCG_CUDA(ctx->d_out64.alloc(nR));
  FCG_CUDA(cudaMemcpyAsync(ctx->d_in64.p, c, nR * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
  int rc = sigma_device_impl(ctx, R, ctx->d_in64.p, ctx->d_out64.p, precision);
  if (rc) return rc;
  FCG_CUDA(cudaMemcpyAsync(sigma, ctx->d_out64.p, nR * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  FCG_CUDA(cudaStreamSynchronize(ctx->stream));
  return FCG_OK;
}

int fcg_diagonal(fcg_ctx* ctx, int op_id, double* hd) {
  if (!ctx) return FCG_EINVAL;
  FCG_REQUIRE(ctx->have_state, FCG_ESTATE, "fcg_state_set must come first");
  FCG_REQUIRE(hd, FCG_EINVAL, "null pointer");
  FCG_REQUIRE(op_id < kNumOps, FCG_EINVAL, "op id out of range");
  FCG_CUDA(cudaSetDevice(ctx->device));
  const int64_t n = ctx->n_cfg;
  FCG_CUDA(ctx->d_hd.alloc(n));
  SigmaParams p = make_params(ctx, 1);
  const unsigned g = unsigned((n + 127) / 128);
  if (op_id < 0) {
    diag_terms_kernel<<<g, 128, 0, ctx->stream>>>(p, ctx->d_op64.p, ctx->d_ints64.p, ctx->d_zero_terms.p,
                                                  int(ctx->plan.zero_terms.size()), ctx->d_row_sector.p, n,
                                                  ctx->d_hd.p);
    FCG_CUDA(cudaGetLastError());
  } else {
    DevBuf<int> missing;
    FCG_CUDA(missing.alloc(1));
    FCG_CUDA(cudaMemsetAsync(missing.p, 0, sizeof(int), ctx->stream));
    diag_op_kernel<<<g, 128, 0, ctx->stream>>>(p, ctx->d_op64.p, op_id, ctx->d_row_sector.p, n, ctx->d_hd.p,
                                               missing.p);
    FCG_CUDA(cudaGetLastError());
    int miss = 0;
    FCG_CUDA(cudaMemcpyAsync(&miss, missing.p, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    FCG_CUDA(cudaStreamSynchronize(ctx->stream));
    FCG_REQUIRE(!miss, FCG_EINVAL, "a diagonal block of that op is missing for a sector of the state");
  }
  FCG_CUDA(cudaMemcpyAsync(hd, ctx->d_hd.p, n * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  FCG_CUDA(cudaStreamSynchronize(ctx->stream));
  return FCG_OK;
}

int fcg_get_stats(const fcg_ctx* ctx, fcg_stats* out) {
  if (!ctx || !out) return FCG_EINVAL;
  *out = ctx->stats;
  return FCG_OK;
}

}  // extern "C"
