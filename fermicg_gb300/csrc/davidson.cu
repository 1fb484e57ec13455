// Block Davidson eigensolver on the device, driving the closed sigma build.
//
// Replaces the BlockDavidson.jl solve behind tps_ci_davidson (src/tpsci_outer.jl:364-454):
// Davidson(Hmap; v0, max_iter, max_ss_vecs, nroots=R, tol, lindep_thresh) with
// eigs(davidson; Adiag = compute_diagonal(...)).  BlockDavidson.jl itself is not in
// the reference tree; this is a standard block Davidson written from its call sites.
//
// Everything of size n stays on the GPU in float64: the subspace V and H V (column-major,
// one column per vector), the Ritz vectors X = V Y, the residuals r = (HV) Y - X theta and
// the preconditioned corrections t = r / (theta - H_dd), written straight behind V.  The
// host keeps the projected matrix V^T H V (extended by one block of columns per
// iteration) and solves the small problems: the Rayleigh-Ritz eigenproblem and the Cholesky
// factors of the new directions' Gram matrices (small_dense.h).
//
// One iteration waits for the device at most three times: for the new columns of V^T H V,
// for the residual norms together with [V T]^T T, and for the Gram matrix after the first
// projection of T.  The projections (classical Gram-Schmidt, twice) are fused with the
// unit scaling and the Cholesky QR of the new block into one kernel each; a second Cholesky
// QR pass runs only when the block's Gram matrix is ill-conditioned.  All partial sums are
// reduced in a fixed order, so a solve gives the same bits whatever runs beside it.
//
// Restarts keep the current and the previous Ritz vectors (GD+k, "locally optimal"
// restart; Stathopoulos & Saad, "Restarting techniques for the (Jacobi-)Davidson symmetric
// eigenvalue methods", ETNA 7, 1998): the kept basis V Q and H V Q are formed on the
// device from an orthonormal Q of the two coefficient blocks, the projected matrix as
// Q^T (V^T H V) Q on the host, so a restart costs no sigma build.
//
// Precision: FCG_FP64 runs every sigma in float64.  FCG_FP32 ("mixed") runs the sigma
// builds in float32 until the residual norms reach max(tol, 1e-5), then restarts from
// the Ritz vectors with float64 sigma builds (the refinement) until tol.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <functional>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

#include "fcg_ctx.cuh"
#include "small_dense.h"

using namespace fcg;

namespace {

constexpr int kDavThreads = 256;
constexpr int kGramWarps = 8;
constexpr int kMaxB = 16;         // columns of the right-hand block of a Gram product (<= R)
constexpr int kMaxRowBlocks = 128;  // row blocks of a Gram product (partial sums per output)
constexpr int kGramRows = 64;       // rows per row block while the block count allows

// One problem's share of a Davidson device operation.  Each kernel body below runs one
// descriptor's block `blk` of `blocks`; a direct launch runs one descriptor (passed by value),
// a grouped launch runs many (descriptors in device memory, ordered by `first`: CTA c works
// for the descriptor whose [first, first + blocks) holds c), so that one launch serves every
// problem of a lockstep round.
struct GramDesc {  // out[i + a*j] = sum_r A[r + n*i] * B[r + n*j], i < a, j < b
  const double* A;
  const double* B;
  double* part;
  double* out;
  unsigned* counters;
  int64_t n, rows_per_block;
  int a, b, row_blocks, first, blocks;
};
struct RitzDesc {  // Ritz vectors, residuals and corrections of R roots
  const double* V;
  const double* AV;
  const double* Y;
  const double* theta;
  const double* hd;
  double* X;
  double* T;
  double* rn_part;
  double* rn_out;
  unsigned* counter;
  int64_t ld, n;
  int nv, R, precond, first, blocks;
};
struct CombineDesc {  // T = V[:, nv : nv + kt] <- T M - V[:, :nv] P
  double* V;
  const double* M;
  const double* P;
  int64_t ld, n;
  int nv, kt, mo, first, blocks;
};
struct UpdateDesc {  // C[:, j] = sum_i A[:, i] Y[i + a*j], j < b
  const double* A;
  const double* Y;
  double* C;
  int64_t lda, ldc, n;
  int a, b, first, blocks;
};
constexpr int kMoveCols = 32;
struct MoveDesc {  // dst[j][0 : n) = src[j][0 : n), j < cols
  const double* src[kMoveCols];
  double* dst[kMoveCols];
  int64_t n;
  int cols, first, blocks;
};

// index of the descriptor that CTA c works for (descriptors ordered by `first`)
template <class D>
__device__ __forceinline__ int find_desc(const D* ds, int nd, int c) {
  int lo = 0, hi = nd - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (ds[mid].first <= c) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// Gram product, block `blk` = row block + row_blocks * column group.  A lane owns one column
// of A, each warp a contiguous slice of the block's rows.  Each block writes its partial sums
// to part[row block][i + a*j]; the last block of a column group to finish (counted in
// counters[group], which it resets) adds the group's partials in row-block order, so the
// result does not depend on the order in which blocks run.  The kernels of this file are
// compiled for block widths BM = 1, 2, 4, 8, 16 and launched with the smallest that fits:
// unrolled loops over unused columns would still issue their FP64 instructions.
template <int BM>
__device__ __forceinline__ void gram_body(const GramDesc& d, int blk) {
  __shared__ double red[kGramWarps][BM][32];
  __shared__ unsigned ticket;
  const int rb = blk % d.row_blocks, group = blk / d.row_blocks;
  const int a = d.a, b = d.b;
  const int64_t n = d.n;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int i = group * 32 + lane;
  const int64_t r0 = int64_t(rb) * d.rows_per_block;
  const int64_t r1 = r0 + d.rows_per_block < n ? r0 + d.rows_per_block : n;
  const int64_t slice = (d.rows_per_block + kGramWarps - 1) / kGramWarps;
  const int64_t s0 = r0 + warp * slice;
  const int64_t s1 = s0 + slice < r1 ? s0 + slice : r1;
  double acc[BM];
#pragma unroll
  for (int j = 0; j < BM; ++j) acc[j] = 0.0;
  if (i < a) {
    const double* Ai = d.A + n * i;
    int64_t r = s0;
    for (; r + 8 <= s1; r += 8) {  // eight rows per step: independent loads in flight
      double x[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) x[u] = Ai[r + u];
#pragma unroll
      for (int j = 0; j < BM; ++j)
        if (j < b) {
          const double* Bj = d.B + n * j + r;
#pragma unroll
          for (int u = 0; u < 8; ++u) acc[j] = fma(x[u], Bj[u], acc[j]);
        }
    }
    for (; r < s1; ++r) {
      const double x = Ai[r];
#pragma unroll
      for (int j = 0; j < BM; ++j)
        if (j < b) acc[j] = fma(x, d.B[r + n * j], acc[j]);
    }
  }
#pragma unroll
  for (int j = 0; j < BM; ++j)
    if (j < b) red[warp][j][lane] = acc[j];
  __syncthreads();
  const int64_t P = int64_t(a) * b;
  for (int t = threadIdx.x; t < b * 32; t += blockDim.x) {
    const int j = t >> 5, l = t & 31;
    const int col = group * 32 + l;
    double s = 0.0;
    for (int w = 0; w < kGramWarps; ++w) s += red[w][j][l];
    if (col < a) d.part[int64_t(rb) * P + col + int64_t(a) * j] = s;
  }
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) ticket = atomicAdd(d.counters + group, 1u);
  __syncthreads();
  if (ticket != unsigned(d.row_blocks) - 1u) return;
  for (int t = threadIdx.x; t < b * 32; t += blockDim.x) {
    const int j = t >> 5, l = t & 31;
    const int col = group * 32 + l;
    if (col >= a) continue;
    const int64_t p = col + int64_t(a) * j;
    double s = 0.0;
    for (int k = 0; k < d.row_blocks; ++k) s += __ldcg(d.part + int64_t(k) * P + p);
    d.out[p] = s;
  }
  if (threadIdx.x == 0) d.counters[group] = 0u;
}

// Ritz vectors and corrections for R roots: per row r,
//   x_j = sum_i V[r, i] Y[i, j],  hx_j = sum_i AV[r, i] Y[i, j],  res_j = hx_j - theta_j x_j,
//   X[r, j] = x_j,  T[r, j] = res_j / (theta_j - hd[r])  (res_j when !precond; the denominator
//   is kept at least 1e-6 away from zero), and rn_out[j] = sum_r res_j^2 (per-block partial
//   sums in rn_part, added in block order by the last block to finish).
// Y (nv x R, column-major) and theta are staged in shared memory.
template <int BM>
__device__ __forceinline__ void ritz_body(const RitzDesc& d, int blk) {
  extern __shared__ double sm[];
  __shared__ double red[kDavThreads / 32][BM];
  __shared__ unsigned ticket;
  const int nv = d.nv, R = d.R;
  const int64_t n = d.n, ld = d.ld;
  double* sY = sm;             // nv * R
  double* sth = sm + nv * R;   // R
  for (int t = threadIdx.x; t < nv * R; t += blockDim.x) sY[t] = d.Y[t];
  for (int t = threadIdx.x; t < R; t += blockDim.x) sth[t] = d.theta[t];
  __syncthreads();
  const int64_t r = int64_t(blk) * blockDim.x + threadIdx.x;
  double x[BM], hx[BM];
#pragma unroll
  for (int j = 0; j < BM; ++j) x[j] = hx[j] = 0.0;
  if (r < n) {
    for (int i0 = 0; i0 < nv; i0 += 8) {  // eight columns' loads in flight before their use
      double v[8], av[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const bool in = i0 + u < nv;
        v[u] = in ? d.V[r + ld * (i0 + u)] : 0.0;
        av[u] = in ? d.AV[r + ld * (i0 + u)] : 0.0;
      }
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        if (i0 + u >= nv) break;
        const double* y = sY + i0 + u;
#pragma unroll
        for (int j = 0; j < BM; ++j)
          if (j < R) {
            x[j] = fma(v[u], y[nv * j], x[j]);
            hx[j] = fma(av[u], y[nv * j], hx[j]);
          }
      }
    }
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int j = 0; j < BM; ++j) {
    if (j >= R) break;
    double res = 0.0;
    if (r < n) {
      res = hx[j] - sth[j] * x[j];
      double den = d.precond ? sth[j] - d.hd[r] : 1.0;
      if (fabs(den) < 1e-6) den = den < 0 ? -1e-6 : 1e-6;
      d.X[r + n * j] = x[j];
      d.T[r + ld * j] = res / den;
    }
    double s = res * res;
    for (int off = 16; off > 0; off >>= 1) s += __shfl_down_sync(0xffffffffu, s, off);
    if (lane == 0) red[warp][j] = s;
  }
  __syncthreads();
  if (threadIdx.x < R) {
    double s = 0.0;
    for (int w = 0; w < int(blockDim.x >> 5); ++w) s += red[w][threadIdx.x];
    d.rn_part[int64_t(blk) * R + threadIdx.x] = s;
  }
  // the last block to finish adds the blocks' partial sums in block order
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) ticket = atomicAdd(d.counter, 1u);
  __syncthreads();
  if (ticket != unsigned(d.blocks) - 1u) return;
  if (threadIdx.x < R) {
    double s = 0.0;
    for (int k = 0; k < d.blocks; ++k) s += __ldcg(d.rn_part + int64_t(k) * R + threadIdx.x);
    d.rn_out[threadIdx.x] = s;
  }
  if (threadIdx.x == 0) *d.counter = 0u;
}

// In place on the new block T = V[:, nv : nv + kt] (leading dimension ld):
//   T[:, j] <- sum_{i < kt} T[:, i] M[i + kt*j] - sum_{i < nv} V[:, i] P[i + nv*j],  j < mo.
// A thread owns a row: it reads the row's T entries before writing any (kt, mo <= BM).
// M (kt x mo) and P (nv x mo) are staged in shared memory; P may be null (no projection).
template <int BM>
__device__ __forceinline__ void combine_body(const CombineDesc& d, int blk) {
  extern __shared__ double sm[];
  const int nv = d.nv, kt = d.kt, mo = d.mo;
  const int64_t ld = d.ld;
  double* sM = sm;            // kt * mo
  double* sP = sm + kt * mo;  // nv * mo
  for (int t = threadIdx.x; t < kt * mo; t += blockDim.x) sM[t] = d.M[t];
  if (d.P)
    for (int t = threadIdx.x; t < nv * mo; t += blockDim.x) sP[t] = d.P[t];
  __syncthreads();
  const int64_t r = int64_t(blk) * blockDim.x + threadIdx.x;
  if (r >= d.n) return;
  double* T = d.V + ld * nv;
  double t_in[BM], out[BM];
#pragma unroll
  for (int i = 0; i < BM; ++i) t_in[i] = i < kt ? T[r + ld * i] : 0.0;
#pragma unroll
  for (int j = 0; j < BM; ++j) {
    double s = 0.0;
    if (j < mo) {
#pragma unroll
      for (int i = 0; i < BM; ++i)
        if (i < kt) s = fma(t_in[i], sM[i + kt * j], s);
    }
    out[j] = s;
  }
  if (d.P) {
    for (int i0 = 0; i0 < nv; i0 += 8) {  // eight columns' loads in flight before their use
      double v[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) v[u] = i0 + u < nv ? d.V[r + ld * (i0 + u)] : 0.0;
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        if (i0 + u >= nv) break;
        const double* pp = sP + i0 + u;
#pragma unroll
        for (int j = 0; j < BM; ++j)
          if (j < mo) out[j] = fma(-v[u], pp[nv * j], out[j]);
      }
    }
  }
#pragma unroll
  for (int j = 0; j < BM; ++j)
    if (j < mo) T[r + ld * j] = out[j];
}

// C[:, j] = sum_i A[:, i] * Y[i + a*j] for j < b (C and A must not overlap)
__device__ __forceinline__ void update_body(const UpdateDesc& d, int blk) {
  const int64_t r = int64_t(blk) * blockDim.x + threadIdx.x;
  if (r >= d.n) return;
  for (int j = 0; j < d.b; ++j) {
    double s = 0.0;
    for (int i = 0; i < d.a; ++i) s = fma(d.A[r + d.lda * i], d.Y[i + int64_t(d.a) * j], s);
    d.C[r + d.ldc * j] = s;
  }
}

// dst[j][r] = src[j][r]: a thread owns a row and reads all its sources before it writes a
// destination, so a destination column may be another move's source
__device__ __forceinline__ void move_body(const MoveDesc& d, int blk) {
  const int64_t r = int64_t(blk) * blockDim.x + threadIdx.x;
  if (r >= d.n) return;
  double v[kMoveCols];
#pragma unroll
  for (int j = 0; j < kMoveCols; ++j)
    if (j < d.cols) v[j] = d.src[j][r];
#pragma unroll
  for (int j = 0; j < kMoveCols; ++j)
    if (j < d.cols) d.dst[j][r] = v[j];
}

template <int BM>
__global__ void __launch_bounds__(kDavThreads) gram_kernel(GramDesc d) { gram_body<BM>(d, int(blockIdx.x)); }
template <int BM>
__global__ void __launch_bounds__(kDavThreads) ritz_residual_kernel(RitzDesc d) { ritz_body<BM>(d, int(blockIdx.x)); }
template <int BM>
__global__ void __launch_bounds__(kDavThreads) combine_kernel(CombineDesc d) { combine_body<BM>(d, int(blockIdx.x)); }
__global__ void __launch_bounds__(kDavThreads) update_kernel(UpdateDesc d) { update_body(d, int(blockIdx.x)); }

// grouped launches: one CTA per block of every descriptor
#define FCG_GROUP_KERNEL(NAME, DESC, BODY)                                              \
  template <int BM>                                                                     \
  __global__ void __launch_bounds__(kDavThreads) NAME(const DESC* __restrict__ ds, int nd) { \
    const int q = find_desc(ds, nd, int(blockIdx.x));                                   \
    const DESC d = ds[q];                                                               \
    BODY<BM>(d, int(blockIdx.x) - d.first);                                             \
  }
FCG_GROUP_KERNEL(gram_group_kernel, GramDesc, gram_body)
FCG_GROUP_KERNEL(ritz_group_kernel, RitzDesc, ritz_body)
FCG_GROUP_KERNEL(combine_group_kernel, CombineDesc, combine_body)
#undef FCG_GROUP_KERNEL
__global__ void __launch_bounds__(kDavThreads) update_group_kernel(const UpdateDesc* __restrict__ ds, int nd) {
  const int q = find_desc(ds, nd, int(blockIdx.x));
  const UpdateDesc d = ds[q];
  update_body(d, int(blockIdx.x) - d.first);
}
__global__ void __launch_bounds__(kDavThreads) move_group_kernel(const MoveDesc* __restrict__ ds, int nd) {
  const int q = find_desc(ds, nd, int(blockIdx.x));
  const int first = ds[q].first;
  move_body(ds[q], int(blockIdx.x) - first);
}

// the smallest compiled block width (1, 2, 4, 8, 16) that holds w columns
inline int width_class(int w) { return w <= 1 ? 1 : w <= 2 ? 2 : w <= 4 ? 4 : w <= 8 ? 8 : 16; }

#define FCG_WIDTH_SWITCH(w, KERNEL, GRID, BLOCK, SMEM, STREAM, ...)                \
  switch (width_class(w)) {                                                        \
    case 1: KERNEL<1><<<GRID, BLOCK, SMEM, STREAM>>>(__VA_ARGS__); break;          \
    case 2: KERNEL<2><<<GRID, BLOCK, SMEM, STREAM>>>(__VA_ARGS__); break;          \
    case 4: KERNEL<4><<<GRID, BLOCK, SMEM, STREAM>>>(__VA_ARGS__); break;          \
    case 8: KERNEL<8><<<GRID, BLOCK, SMEM, STREAM>>>(__VA_ARGS__); break;          \
    default: KERNEL<16><<<GRID, BLOCK, SMEM, STREAM>>>(__VA_ARGS__); break;        \
  }

}  // namespace

extern "C" int fcg_diagonal(fcg_ctx* ctx, int op_id, double* hd);

namespace {

// Device work of one problem recorded during a lockstep round, for the round's grouped launches.
enum class OpKind : int { kGram, kRitz, kCombine, kUpdate, kMove };
struct RecOp {
  OpKind kind;
  int width;    // block-width class of the kernel (0 for the width-free kernels)
  size_t smem;  // dynamic shared memory bytes
  union {
    GramDesc g;
    RitzDesc r;
    CombineDesc c;
    UpdateDesc u;
    MoveDesc m;
  };
};
constexpr int kMaxRoundOps = 16;  // device operations one problem records between two waits

// Page-locked staging of a lockstep round with its device mirror: the problems' uploads and
// the round's descriptors are reserved at [0, used) from any host thread, and one copy moves
// them to the device before the round's launches.
struct RoundArena {
  PinnedBuf<unsigned char> h;
  DevBuf<unsigned char> d;
  std::atomic<size_t> used{0};
  static constexpr size_t npos = ~size_t(0);
  size_t cap() const { return std::min(h.n, d.n); }
  size_t reserve(size_t bytes) {
    bytes = (bytes + 15) & ~size_t(15);
    const size_t off = used.fetch_add(bytes);
    return off + bytes <= cap() ? off : npos;
  }
};

struct DavidsonWork {
  fcg_ctx* ctx = nullptr;
  int64_t n = 0;
  int R = 0, kmax = 0, kcap = 0;  // kcap = kmax + R columns of V and AV
  int row_blocks = 1;             // Gram products: row blocks, rows per block
  int64_t rows_per_block = 1;
  int res_blocks = 1;             // residual kernel blocks
  // views of the context's grow-only buffers (fcg_ctx::dav_*), sized by init
  template <class T>
  struct Span {
    T* p = nullptr;
    size_t n = 0;
  };
  Span<double> V, AV, X, tmp, hd, part, rn_part, d_out, d_up;
  Span<unsigned> counters;  // last-block tickets: [0, ngroups) Gram column groups, [ngroups] residual
  int ngroups = 1;
  Span<double> h_out, h_up;
  size_t up_used = 0, up_sent = 0;
  size_t up_cap = 0, out_cap = 0;  // doubles staged between two waits; fetched values
  double* hout = nullptr;          // the fetched values (h_out, or hout_vec in grouped mode)
  std::vector<double> hout_vec;
  // Grouped mode (arena set): device work is recorded in `ops` and launched with the other
  // problems' work of the round; uploads go to the round's arena; the round copies
  // d_out[0 : fetch_count) to hout, and fin_count doubles from fin_src to fin_dst.
  RoundArena* arena = nullptr;
  std::vector<RecOp> ops;
  size_t fetch_count = 0;
  const double* fin_src = nullptr;
  double* fin_dst = nullptr;
  size_t fin_count = 0;

  bool grouped() const { return arena != nullptr; }
  int record(const RecOp& op) {
    fcg_ctx* ctx = this->ctx;
    FCG_REQUIRE(ops.size() < size_t(kMaxRoundOps), FCG_ELIMIT, "Davidson: too many device operations in a round");
    ops.push_back(op);
    return FCG_OK;
  }

  // Stage `count` doubles for the device and return where they will be once flush() (or the
  // round's copy) has moved them.  The area is reused only after the next wait.
  int upload(const double* src, size_t count, const double** dptr) {
    fcg_ctx* ctx = this->ctx;
    if (grouped()) {
      const size_t off = arena->reserve(count * sizeof(double));
      FCG_REQUIRE(off != RoundArena::npos, FCG_ELIMIT, "Davidson: round staging area exhausted");
      if (count) std::memcpy(arena->h.p + off, src, count * sizeof(double));
      *dptr = reinterpret_cast<const double*>(arena->d.p + off);
      return FCG_OK;
    }
    const size_t off = (up_used + 3) & ~size_t(3);
    FCG_REQUIRE(off + count <= h_up.n, FCG_ELIMIT, "Davidson: staging area exhausted");
    if (count) std::memcpy(h_up.p + off, src, count * sizeof(double));
    up_used = off + count;
    *dptr = d_up.p + off;
    return FCG_OK;
  }
  // one host-to-device copy of everything staged since the last flush
  int flush() {
    fcg_ctx* ctx = this->ctx;
    if (grouped()) return FCG_OK;
    if (up_used > up_sent)
      FCG_CUDA(cudaMemcpyAsync(d_up.p + up_sent, h_up.p + up_sent, (up_used - up_sent) * sizeof(double),
                               cudaMemcpyHostToDevice, ctx->stream));
    up_sent = up_used;
    return FCG_OK;
  }
  // out[0 : a*b) = A^T B on the device (A: a columns, B: b columns, leading dimension n)
  int gram(const double* A, int a, const double* B, int b, double* out) {
    fcg_ctx* ctx = this->ctx;
    FCG_REQUIRE(a >= 1 && a <= kcap && b >= 1 && b <= R, FCG_ELIMIT, "Davidson: Gram block out of range");
    RecOp op;
    op.kind = OpKind::kGram;
    op.width = width_class(b);
    op.smem = 0;
    GramDesc& d = op.g;
    d = GramDesc{A, B, part.p, out, counters.p, n, rows_per_block, a, b, row_blocks, 0, row_blocks * ((a + 31) / 32)};
    if (grouped()) return record(op);
    FCG_WIDTH_SWITCH(b, gram_kernel, unsigned(d.blocks), kDavThreads, 0, ctx->stream, d)
    FCG_CUDA(cudaGetLastError());
    return FCG_OK;
  }
  // Ritz vectors X, corrections T = V[:, nv : nv + R] and squared residual norms d_out[0 : R)
  int ritz(int nv, const double* dY, const double* dth, int precond) {
    fcg_ctx* ctx = this->ctx;
    RecOp op;
    op.kind = OpKind::kRitz;
    op.width = width_class(R);
    op.smem = sizeof(double) * (size_t(nv) * R + R);
    RitzDesc& d = op.r;
    d = RitzDesc{V.p, AV.p, dY, dth, hd.p, X.p, V.p + n * nv, rn_part.p, d_out.p, counters.p + ngroups,
                 n, n, nv, R, precond, 0, res_blocks};
    if (grouped()) return record(op);
    FCG_WIDTH_SWITCH(R, ritz_residual_kernel, unsigned(d.blocks), kDavThreads, op.smem, ctx->stream, d)
    FCG_CUDA(cudaGetLastError());
    return FCG_OK;
  }
  // C[:, :b] = A[:, :a] Y (Y on the device, a x b)
  int update(const double* A, int a, const double* dY, int b, double* C) {
    fcg_ctx* ctx = this->ctx;
    RecOp op;
    op.kind = OpKind::kUpdate;
    op.width = 0;
    op.smem = 0;
    UpdateDesc& d = op.u;
    d = UpdateDesc{A, dY, C, n, n, n, a, b, 0, int((n + kDavThreads - 1) / kDavThreads)};
    if (grouped()) return record(op);
    update_kernel<<<unsigned(d.blocks), kDavThreads, 0, ctx->stream>>>(d);
    FCG_CUDA(cudaGetLastError());
    return FCG_OK;
  }
  // columns dst[j] = src[j] (n doubles each), j < cols.  Direct mode copies the columns in
  // order, grouped mode row by row with a row's sources read before its destinations are
  // written; both agree when a destination is at most an earlier column's source.
  int move(int cols, const double* const* src, double* const* dst) {
    fcg_ctx* ctx = this->ctx;
    FCG_REQUIRE(cols >= 0 && cols <= kMoveCols, FCG_ELIMIT, "Davidson: too many columns in one move");
    if (cols == 0) return FCG_OK;
    if (grouped()) {
      RecOp op;
      op.kind = OpKind::kMove;
      op.width = 0;
      op.smem = 0;
      MoveDesc& d = op.m;
      for (int j = 0; j < cols; ++j) {
        d.src[j] = src[j];
        d.dst[j] = dst[j];
      }
      d.n = n;
      d.cols = cols;
      d.first = 0;
      d.blocks = int((n + kDavThreads - 1) / kDavThreads);
      return record(op);
    }
    for (int j = 0; j < cols; ++j)
      FCG_CUDA(cudaMemcpyAsync(dst[j], src[j], sizeof(double) * n, cudaMemcpyDeviceToDevice, ctx->stream));
    return FCG_OK;
  }
  // the contiguous columns dst[:, :cols] = src[:, :cols] (leading dimension n, no overlap)
  int copy_block(double* dst, const double* src, int cols) {
    fcg_ctx* ctx = this->ctx;
    if (!grouped()) {
      FCG_CUDA(cudaMemcpyAsync(dst, src, sizeof(double) * n * cols, cudaMemcpyDeviceToDevice, ctx->stream));
      return FCG_OK;
    }
    const double* s[kMoveCols];
    double* t[kMoveCols];
    for (int c0 = 0; c0 < cols; c0 += kMoveCols) {
      const int m = std::min(kMoveCols, cols - c0);
      for (int j = 0; j < m; ++j) {
        s[j] = src + n * (c0 + j);
        t[j] = dst + n * (c0 + j);
      }
      const int rc = move(m, s, t);
      if (rc) return rc;
    }
    return FCG_OK;
  }
  // queue hout[0 : count) = d_out[0 : count); the values are there after the next wait for
  // the stream, after which after_wait() frees the staging area
  int enqueue_fetch(size_t count) {
    fcg_ctx* ctx = this->ctx;
    FCG_REQUIRE(count <= out_cap, FCG_ELIMIT, "Davidson: fetch larger than its buffer");
    if (grouped()) {
      fetch_count = count;
      return FCG_OK;
    }
    FCG_CUDA(cudaMemcpyAsync(h_out.p, d_out.p, count * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    return FCG_OK;
  }
  // queue dst[0 : count) = src[0 : count) to the host (the final vectors)
  int fetch_final(double* dst, const double* src, size_t count) {
    fcg_ctx* ctx = this->ctx;
    if (grouped()) {
      fin_dst = dst;
      fin_src = src;
      fin_count = count;
      return FCG_OK;
    }
    FCG_CUDA(cudaMemcpyAsync(dst, src, sizeof(double) * count, cudaMemcpyDeviceToHost, ctx->stream));
    return FCG_OK;
  }
  void after_wait() { up_used = up_sent = 0; }
  // T = V[:, nv : nv + kt] <- T M - V[:, :nv] P  (M: kt x mo, P: nv x mo or null)
  int combine(int nv, int kt, const std::vector<double>& M, const std::vector<double>* P, int mo) {
    fcg_ctx* ctx = this->ctx;
    FCG_REQUIRE(kt >= 1 && kt <= kMaxB && mo >= 1 && mo <= kMaxB, FCG_ELIMIT, "Davidson: block out of range");
    const double *dM = nullptr, *dP = nullptr;
    int rc;
    if ((rc = upload(M.data(), size_t(kt) * mo, &dM))) return rc;
    const bool proj = P && nv > 0;
    if (proj && (rc = upload(P->data(), size_t(nv) * mo, &dP))) return rc;
    if ((rc = flush())) return rc;
    RecOp op;
    op.kind = OpKind::kCombine;
    op.width = width_class(std::max(kt, mo));
    op.smem = sizeof(double) * (size_t(kt) * mo + (proj ? size_t(nv) * mo : 0));
    CombineDesc& d = op.c;
    d = CombineDesc{V.p, dM, dP, n, n, nv, kt, mo, 0, int((n + kDavThreads - 1) / kDavThreads)};
    if (grouped()) return record(op);
    FCG_WIDTH_SWITCH(std::max(kt, mo), combine_kernel, unsigned(d.blocks), kDavThreads, op.smem, ctx->stream, d)
    FCG_CUDA(cudaGetLastError());
    return FCG_OK;
  }
  // Resumable orthonormalisation of the new directions V[:, nv : nv + nt] (see ortho_start):
  // each call either finishes (*wait = false; the kept count in o_kept) or has queued a Gram
  // product and its fetch (*wait = true) and continues in ortho_resume after the wait.
  int ortho_start(int nv, int nt, std::vector<double> G0, double drop, bool* wait);
  int ortho_resume(bool* wait);
  int ortho_solve(std::vector<double> G2, int k1, bool* wait);
  int o_state = 0;  // 0 idle, 1 waiting for the Gram matrix after the first projection, 2 for the second QR
  int o_nv = 0, o_nt = 0, o_k1 = 0, o_good = 0, o_kept = 0;
  double o_drop = 0.0;
  std::vector<double> o_S2;
};

// Orthonormalise the new directions T = V[:, nv : nv + nt] against V[:, :nv] and among
// themselves, given G0 = [V T]^T T ((nv + nt) x nt, column-major).  Every direction is first
// scaled to unit norm and projected out of V (classical Gram-Schmidt, twice); a direction is
// dropped when less than `drop` of it survives (it lies in the subspace already, up to
// rounding).  The survivors are orthonormalised by Cholesky QR (stopping at the first
// dependent column), twice when their Gram matrix has a condition number above 1e4.  The
// kept directions end up in V[:, nv : nv + o_kept].  The work pauses (*wait) where it needs a
// Gram matrix from the device: after the first projection, and before the second QR.
int DavidsonWork::ortho_start(int nv, int nt, std::vector<double> G0, double drop, bool* wait) {
  *wait = false;
  o_state = 0;
  o_kept = 0;
  o_nv = nv;
  o_nt = nt;
  o_drop = drop;
  const int ld0 = nv + nt;
  int rc;
  // 1. unit scaling (and the first projection)
  std::vector<int> keep;
  for (int j = 0; j < nt; ++j) {
    const double g = G0[nv + j + size_t(ld0) * j];
    if (std::isfinite(g) && g > 1e-300) keep.push_back(j);
  }
  const int k1 = int(keep.size());
  o_k1 = k1;
  if (k1 == 0) return FCG_OK;
  std::vector<double> M1(size_t(nt) * k1, 0.0), dsc(k1);
  for (int q = 0; q < k1; ++q) {
    dsc[q] = 1.0 / std::sqrt(G0[nv + keep[q] + size_t(ld0) * keep[q]]);
    M1[keep[q] + size_t(nt) * q] = dsc[q];
  }
  if (nv == 0) {
    if ((rc = combine(0, nt, M1, nullptr, k1))) return rc;
    std::vector<double> G2(size_t(k1) * k1);
    for (int q = 0; q < k1; ++q)
      for (int p = 0; p < k1; ++p) G2[p + size_t(k1) * q] = dsc[p] * dsc[q] * G0[keep[p] + size_t(ld0) * keep[q]];
    o_S2.clear();
    return ortho_solve(std::move(G2), k1, wait);
  }
  std::vector<double> P1(size_t(nv) * k1);
  for (int q = 0; q < k1; ++q)
    for (int i = 0; i < nv; ++i) P1[i + size_t(nv) * q] = G0[i + size_t(ld0) * keep[q]] * dsc[q];
  if ((rc = combine(nv, nt, M1, &P1, k1))) return rc;
  // 2. second projection, from the Gram matrix of the projected block
  if ((rc = gram(V.p, nv + k1, V.p + n * nv, k1, d_out.p))) return rc;
  if ((rc = enqueue_fetch(size_t(nv + k1) * k1))) return rc;
  o_state = 1;
  *wait = true;
  return FCG_OK;
}

int DavidsonWork::ortho_resume(bool* wait) {
  *wait = false;
  const int nv = o_nv;
  if (o_state == 1) {
    o_state = 0;
    const int k1 = o_k1, ld1 = nv + k1;
    const double* G1 = hout;
    o_S2.assign(size_t(nv) * k1, 0.0);
    for (int q = 0; q < k1; ++q)
      for (int i = 0; i < nv; ++i) o_S2[i + size_t(nv) * q] = G1[i + size_t(ld1) * q];
    // Gram matrix after the second projection: T1^T T1 - S2^T S2 (V orthonormal)
    std::vector<double> G2(size_t(k1) * k1);
    for (int q = 0; q < k1; ++q)
      for (int p = 0; p < k1; ++p) {
        double s = G1[nv + p + size_t(ld1) * q];
        for (int i = 0; i < nv; ++i) s -= o_S2[i + size_t(nv) * p] * o_S2[i + size_t(nv) * q];
        G2[p + size_t(k1) * q] = s;
      }
    for (int q = 0; q < k1; ++q)
      for (int p = 0; p < q; ++p) {
        const double a = 0.5 * (G2[p + size_t(k1) * q] + G2[q + size_t(k1) * p]);
        G2[p + size_t(k1) * q] = G2[q + size_t(k1) * p] = a;
      }
    return ortho_solve(std::move(G2), k1, wait);
  }
  if (o_state == 2) {  // the second Cholesky QR (and projection)
    o_state = 0;
    const int good = o_good, ld3 = nv + good;
    const double* G3 = hout;
    std::vector<double> S3(size_t(nv) * good), G3t(size_t(good) * good);
    for (int q = 0; q < good; ++q)
      for (int i = 0; i < nv; ++i) S3[i + size_t(nv) * q] = G3[i + size_t(ld3) * q];
    for (int q = 0; q < good; ++q)
      for (int p = 0; p < good; ++p) {
        double s = 0.5 * (G3[nv + p + size_t(ld3) * q] + G3[nv + q + size_t(ld3) * p]);
        for (int i = 0; i < nv; ++i) s -= S3[i + size_t(nv) * p] * S3[i + size_t(nv) * q];
        G3t[p + size_t(good) * q] = s;
      }
    std::vector<double> Ri3;
    const int good3 = fcg_small::chol_inverse(good, G3t.data(), good, o_drop, Ri3);
    if (good3 == 0) {
      o_kept = 0;
      return FCG_OK;
    }
    std::vector<double> M3(size_t(good) * good3, 0.0);
    for (int c = 0; c < good3; ++c)
      for (int i = 0; i < good3; ++i) M3[i + size_t(good) * c] = Ri3[i + size_t(good3) * c];
    std::vector<double> P3;
    if (nv > 0) {
      P3.assign(size_t(nv) * good3, 0.0);
      for (int c = 0; c < good3; ++c)
        for (int p = 0; p < good3; ++p) {
          const double m = M3[p + size_t(good) * c];
          for (int i = 0; i < nv; ++i) P3[i + size_t(nv) * c] += S3[i + size_t(nv) * p] * m;
        }
    }
    const int rc = combine(nv, good, M3, nv > 0 ? &P3 : nullptr, good3);
    if (rc) return rc;
    o_kept = good3;
  }
  return FCG_OK;
}

// 3. survivors, Cholesky QR fused with the second projection; then the second QR when the
// block's Gram matrix is ill-conditioned (it needs one more Gram matrix: *wait)
int DavidsonWork::ortho_solve(std::vector<double> G2, int k1, bool* wait) {
  *wait = false;
  const int nv = o_nv;
  const double drop = o_drop;
  int rc;
  std::vector<int> keep2;
  for (int p = 0; p < k1; ++p) {
    const double g = G2[p + size_t(k1) * p];
    if (std::isfinite(g) && g >= drop * drop) keep2.push_back(p);
  }
  const int k2 = int(keep2.size());
  if (k2 == 0) return FCG_OK;
  std::vector<double> G2k(size_t(k2) * k2);
  for (int q = 0; q < k2; ++q)
    for (int p = 0; p < k2; ++p) G2k[p + size_t(k2) * q] = G2[keep2[p] + size_t(k1) * keep2[q]];
  std::vector<double> Ri;
  const int good = fcg_small::chol_inverse(k2, G2k.data(), k2, drop, Ri);
  if (good == 0) return FCG_OK;
  std::vector<double> M2(size_t(k1) * good, 0.0);
  for (int c = 0; c < good; ++c)
    for (int q = 0; q < good; ++q) M2[keep2[q] + size_t(k1) * c] = Ri[q + size_t(good) * c];
  if (nv == 0) {
    if ((rc = combine(0, k1, M2, nullptr, good))) return rc;
  } else {
    std::vector<double> P2(size_t(nv) * good, 0.0);
    for (int c = 0; c < good; ++c)
      for (int p = 0; p < k1; ++p) {
        const double m = M2[p + size_t(k1) * c];
        if (m == 0.0) continue;
        for (int i = 0; i < nv; ++i) P2[i + size_t(nv) * c] += o_S2[i + size_t(nv) * p] * m;
      }
    if ((rc = combine(nv, k1, M2, &P2, good))) return rc;
  }
  o_kept = good;
  if (fcg_small::spd_condition(good, G2k.data(), k2) > 1e4) {
    o_good = good;
    if ((rc = gram(V.p, nv + good, V.p + n * nv, good, d_out.p))) return rc;
    if ((rc = enqueue_fetch(size_t(nv + good) * good))) return rc;
    o_state = 2;
    *wait = true;
  }
  return FCG_OK;
}


// One problem's block Davidson as a resumable state machine: step() runs until the problem
// needs the device (WAIT: work and a fetch are queued on its stream), needs the sigma of its
// new block (SIGMA: columns [sig_col, sig_col + sig_m) of V into the same columns of AV, in
// precision sig_prec), or is done.  A driver waits for the stream and runs the sigma builds,
// for one problem (fcg_davidson) or for many at once (fcg_davidson_grouped).
enum class Act { kWait, kSigma, kDone };

struct DavidsonRun {
  DavidsonWork W;
  fcg_ctx* ctx = nullptr;
  bool bst = false;  // the operator is the BST sigma of the context's fcg_bst_set structure
  int R = 0, max_iter = 0, precond = 0, prec = 0;
  double tol = 0, drop = 0, switch_tol = 0;
  // float32 phase: best largest residual so far and the iterations since it last fell by 10%
  double best32 = 0;
  int stall32 = 0;
  bool gdk = false;
  const double* v0 = nullptr;
  double *energies = nullptr, *vectors = nullptr, *residuals = nullptr;
  int* iters = nullptr;
  // iteration state
  enum St { kInit, kInitG0, kInitOrtho, kInitDone, kAfterInitSigma, kIter, kRRWait, kResWait, kOrtho, kOrthoDone,
            kAfterSigma, kSwG0, kSwOrtho, kSwDone, kAfterSwSigma, kFinish, kFinished };
  St st = kInit;
  int nv = 0, newlo = 0, m = 0, it = 0;
  int64_t sigma_calls = 0;
  std::vector<double> Hs, A, w, Y, th, rn, Yprev;
  int yprev_rows = 0;
  int sig_col = 0, sig_m = 0, sig_prec = 0;

  // grouped: the solve runs in a lockstep round executor, which provides W.arena before the
  // first step (no staging buffers of its own are allocated)
  // bst_op: solve with the BST sigma (ci_solve, src/tucker_outer.jl:68-215) over the cores of
  // the last fcg_bst_set, preconditioned by bst_hd (core_total values) when given
  int init(fcg_ctx* c, int R_, const double* v0_, int max_iter_, int max_ss_vecs, double tol_, double lindep,
           int precision, int precond_, double* e, double* vecs, double* res, int* its, bool grouped = false,
           bool bst_op = false, const double* bst_hd = nullptr) {
    ctx = c;
    bst = bst_op;
    if (bst) precond_ = bst_hd != nullptr;
    R = R_;
    v0 = v0_;
    max_iter = max_iter_;
    tol = tol_;
    precond = precond_;
    prec = precision;
    energies = e;
    vectors = vecs;
    residuals = res;
    iters = its;
    if (bst) {
      FCG_REQUIRE(ctx->have_bst, FCG_ESTATE, "fcg_bst_set must come first");
    } else {
      FCG_REQUIRE(ctx->have_state, FCG_ESTATE, "fcg_state_set must come first");
      const int rc = ensure_plan(ctx);
      if (rc) return rc;
    }
    const int64_t n = bst ? ctx->bst_core_total : ctx->n_cfg;
    FCG_REQUIRE(v0 && energies && vectors && residuals && iters, FCG_EINVAL, "null pointer");
    FCG_REQUIRE(R >= 1 && R <= kMaxB && R <= n, FCG_ELIMIT, "R must be in [1, min(16, vector length)]");
    FCG_REQUIRE(max_ss_vecs >= 2 && max_iter >= 1 && tol > 0, FCG_EINVAL, "bad Davidson settings");
    FCG_REQUIRE(precision == FCG_FP64 || precision == FCG_FP32, FCG_EINVAL, "unknown precision");
    W.ctx = ctx;
    W.n = n;
    W.R = R;
    W.kmax = int(std::min<int64_t>(int64_t(max_ss_vecs) * R, n));
    W.kmax = std::max(W.kmax, std::min<int>(2 * R, int(n)));
    W.kcap = W.kmax + R;
    const int kmax = W.kmax, kcap = W.kcap;
    // shared memory of the residual and combine kernels: (kcap x R) + R doubles at most
    const size_t smem_max = sizeof(double) * (size_t(kcap) * R + size_t(R) * R + R);
    FCG_REQUIRE(smem_max <= 200 * 1024, FCG_ELIMIT, "max_ss_vecs * R too large for the subspace kernels");
    if (smem_max > 48 * 1024) {
      const int sm = int(smem_max);
      const auto attr = cudaFuncAttributeMaxDynamicSharedMemorySize;
      FCG_CUDA(cudaFuncSetAttribute(ritz_residual_kernel<1>, attr, sm));
      FCG_CUDA(cudaFuncSetAttribute(ritz_residual_kernel<2>, attr, sm));
      FCG_CUDA(cudaFuncSetAttribute(ritz_residual_kernel<4>, attr, sm));
      FCG_CUDA(cudaFuncSetAttribute(ritz_residual_kernel<8>, attr, sm));
      FCG_CUDA(cudaFuncSetAttribute(ritz_residual_kernel<16>, attr, sm));
      FCG_CUDA(cudaFuncSetAttribute(combine_kernel<1>, attr, sm));
      FCG_CUDA(cudaFuncSetAttribute(combine_kernel<2>, attr, sm));
      FCG_CUDA(cudaFuncSetAttribute(combine_kernel<4>, attr, sm));
      FCG_CUDA(cudaFuncSetAttribute(combine_kernel<8>, attr, sm));
      FCG_CUDA(cudaFuncSetAttribute(combine_kernel<16>, attr, sm));
      FCG_CUDA(cudaFuncSetAttribute(ritz_group_kernel<1>, attr, sm));
      FCG_CUDA(cudaFuncSetAttribute(ritz_group_kernel<2>, attr, sm));
      FCG_CUDA(cudaFuncSetAttribute(ritz_group_kernel<4>, attr, sm));
      FCG_CUDA(cudaFuncSetAttribute(ritz_group_kernel<8>, attr, sm));
      FCG_CUDA(cudaFuncSetAttribute(ritz_group_kernel<16>, attr, sm));
      FCG_CUDA(cudaFuncSetAttribute(combine_group_kernel<1>, attr, sm));
      FCG_CUDA(cudaFuncSetAttribute(combine_group_kernel<2>, attr, sm));
      FCG_CUDA(cudaFuncSetAttribute(combine_group_kernel<4>, attr, sm));
      FCG_CUDA(cudaFuncSetAttribute(combine_group_kernel<8>, attr, sm));
      FCG_CUDA(cudaFuncSetAttribute(combine_group_kernel<16>, attr, sm));
    }
    W.row_blocks = int(std::max<int64_t>(1, std::min<int64_t>(kMaxRowBlocks, (n + kGramRows - 1) / kGramRows)));
    W.rows_per_block = (n + W.row_blocks - 1) / W.row_blocks;
    W.res_blocks = int((n + kDavThreads - 1) / kDavThreads);
    // the context's buffers grow to this solve's sizes and stay for its later solves
    auto take = [](auto& buf, auto& span, size_t count) {
      const cudaError_t e = buf.alloc(count);
      span.p = buf.p;
      span.n = count;
      return e;
    };
    FCG_CUDA(take(ctx->dav_V, W.V, size_t(n) * kcap));
    FCG_CUDA(take(ctx->dav_AV, W.AV, size_t(n) * kcap));
    FCG_CUDA(take(ctx->dav_X, W.X, size_t(n) * R));
    FCG_CUDA(take(ctx->dav_tmp, W.tmp, size_t(n) * std::min(kmax, 2 * R)));
    FCG_CUDA(take(ctx->dav_hd, W.hd, size_t(n)));
    FCG_CUDA(take(ctx->dav_part, W.part, size_t(W.row_blocks) * kcap * R));
    FCG_CUDA(take(ctx->dav_rn, W.rn_part, size_t(W.res_blocks) * R));
    W.ngroups = (kcap + 31) / 32;
    FCG_CUDA(take(ctx->dav_counters, W.counters, size_t(W.ngroups) + 1));
    FCG_CUDA(cudaMemsetAsync(W.counters.p, 0, sizeof(unsigned) * (W.ngroups + 1), ctx->stream));
    W.out_cap = size_t(R) + size_t(kcap) * R + 16;
    W.up_cap = size_t(4) * (size_t(kcap) * 2 * R + size_t(R) * R + 64);
    FCG_CUDA(take(ctx->dav_out, W.d_out, W.out_cap));
    if (grouped) {
      W.hout_vec.assign(W.out_cap, 0.0);
      W.hout = W.hout_vec.data();
    } else {
      FCG_CUDA(take(ctx->dav_h_out, W.h_out, W.out_cap));
      FCG_CUDA(take(ctx->dav_up, W.d_up, W.up_cap));
      FCG_CUDA(take(ctx->dav_h_up, W.h_up, W.up_cap));
      W.hout = W.h_out.p;
    }
    if (precond && bst) {
      FCG_CUDA(cudaMemcpyAsync(W.hd.p, bst_hd, sizeof(double) * n, cudaMemcpyHostToDevice, ctx->stream));
      FCG_CUDA(cudaStreamSynchronize(ctx->stream));  // bst_hd belongs to the caller
    } else if (precond) {
      std::vector<double> hd(n);
      int rc = fcg_diagonal(ctx, -1, hd.data());  // leaves the diagonal in ctx->d_hd as well
      if (rc) return rc;
      FCG_CUDA(cudaMemcpyAsync(W.hd.p, ctx->d_hd.p, sizeof(double) * n, cudaMemcpyDeviceToDevice, ctx->stream));
    }
    // a new direction must keep at least this fraction of its norm after projection
    drop = std::max(lindep, 1e-8);
    switch_tol = std::max(tol, 1e-5);
    // GD+k restarts keep 2R vectors when the subspace has room for them and a new block
    gdk = kmax >= 3 * R;
    Hs.assign(size_t(kcap) * kcap, 0.0);
    th.assign(R, 0.0);
    rn.assign(R, 0.0);
    FCG_CUDA(cudaMemcpyAsync(W.V.p, v0, sizeof(double) * n * R, cudaMemcpyHostToDevice, ctx->stream));
    st = kInit;
    return FCG_OK;
  }

  // request the sigma of columns [col, col + cols) in precision p
  Act sigma(int col, int cols, int p, St next) {
    sig_col = col;
    sig_m = cols;
    sig_prec = p;
    st = next;
    return Act::kSigma;
  }

  int step(Act* act);
  int new_directions(bool* wait);
};

int DavidsonRun::step(Act* act) {
  const int64_t n = W.n;
  const int kcap = W.kcap;
  int rc;
  bool wait = false;
  for (;;) {
    switch (st) {
      case kInit:  // the initial block on its own
        if ((rc = W.gram(W.V.p, R, W.V.p, R, W.d_out.p))) return rc;
        if ((rc = W.enqueue_fetch(size_t(R) * R))) return rc;
        st = kInitG0;
        *act = Act::kWait;
        return FCG_OK;
      case kInitG0: {
        std::vector<double> G0(W.hout, W.hout + size_t(R) * R);
        if ((rc = W.ortho_start(0, R, std::move(G0), drop, &wait))) return rc;
        st = wait ? kInitOrtho : kInitDone;
        if (wait) {
          *act = Act::kWait;
          return FCG_OK;
        }
        break;
      }
      case kInitOrtho:
        if ((rc = W.ortho_resume(&wait))) return rc;
        if (wait) {
          *act = Act::kWait;
          return FCG_OK;
        }
        st = kInitDone;
        break;
      case kInitDone: {
        m = W.o_kept;
        if (m != R) {
          double nrm_min = 1e300, nrm_max = 0.0;
          int nonfinite = 0;
          for (int j = 0; j < R; ++j) {
            double s2 = 0.0;
            for (int64_t i = 0; i < n; ++i) {
              const double x = v0[i + n * j];
              if (!std::isfinite(x)) ++nonfinite;
              s2 += x * x;
            }
            nrm_min = std::min(nrm_min, s2);
            nrm_max = std::max(nrm_max, s2);
          }
          ctx->err = "initial vectors are linearly dependent (kept " + std::to_string(m) + " of " +
                     std::to_string(R) + ", n " + std::to_string(n) + ", squared norms " + std::to_string(nrm_min) +
                     ".." + std::to_string(nrm_max) + ", non-finite entries " + std::to_string(nonfinite) + ")";
          return FCG_EINVAL;
        }
        *act = sigma(0, R, prec, kAfterInitSigma);
        return FCG_OK;
      }
      case kAfterInitSigma:
        nv = R;
        newlo = 0;
        it = 0;
        sigma_calls = 1;
        st = kIter;
        break;
      case kIter: {  // Rayleigh-Ritz: the new columns of V^T H V
        if (++it > max_iter) {
          st = kFinish;
          break;
        }
        const int nb = nv - newlo;
        if ((rc = W.gram(W.V.p, nv, W.AV.p + n * newlo, nb, W.d_out.p))) return rc;
        if ((rc = W.enqueue_fetch(size_t(nv) * nb))) return rc;
        st = kRRWait;
        *act = Act::kWait;
        return FCG_OK;
      }
      case kRRWait: {  // the projected eigenproblem; Ritz vectors, residuals, corrections, [V T]^T T
        const int nb = nv - newlo;
        const double* C = W.hout;
        for (int c = 0; c < nb; ++c) {
          const int col = newlo + c;
          for (int i = 0; i < nv; ++i) {
            double h = C[i + size_t(nv) * c];
            if (i >= newlo) h = 0.5 * (h + C[col + size_t(nv) * (i - newlo)]);
            if (!std::isfinite(h)) {
              ctx->err = "Davidson: non-finite subspace matrix at iteration " + std::to_string(it) + " (subspace " +
                         std::to_string(nv) + ")";
              return FCG_ECUDA;
            }
            Hs[i + size_t(kcap) * col] = Hs[col + size_t(kcap) * i] = h;
          }
        }
        A.resize(size_t(nv) * nv);
        for (int j = 0; j < nv; ++j)
          for (int i = 0; i < nv; ++i) A[i + size_t(nv) * j] = Hs[i + size_t(kcap) * j];
        if (fcg_small::symeig(nv, A.data(), w, Y, R)) {
          ctx->err = "Davidson: subspace eigensolver did not converge at iteration " + std::to_string(it);
          return FCG_ECUDA;
        }
        for (int j = 0; j < R; ++j) th[j] = w[j];
        const double *dY = nullptr, *dth = nullptr;
        if ((rc = W.upload(Y.data(), size_t(nv) * R, &dY))) return rc;
        if ((rc = W.upload(th.data(), size_t(R), &dth))) return rc;
        if ((rc = W.flush())) return rc;
        if ((rc = W.ritz(nv, dY, dth, precond))) return rc;
        if ((rc = W.gram(W.V.p, nv + R, W.V.p + n * nv, R, W.d_out.p + R))) return rc;
        if ((rc = W.enqueue_fetch(size_t(R) + size_t(nv + R) * R))) return rc;
        st = kResWait;
        *act = Act::kWait;
        return FCG_OK;
      }
      case kResWait: {
        double rmax = 0.0;
        for (int j = 0; j < R; ++j) {
          rn[j] = std::sqrt(W.hout[j]);
          rmax = std::max(rmax, rn[j]);
          if (!std::isfinite(rn[j]) || !std::isfinite(th[j])) {
            ctx->err = "Davidson: non-finite residual or Ritz value at iteration " + std::to_string(it);
            return FCG_ECUDA;
          }
        }
        if (rmax < tol && prec == FCG_FP64) {
          st = kFinish;
          break;
        }
        bool to_fp64 = false;
        if (prec == FCG_FP32) {
          // The float32 sigma leaves a residual floor from its rounding of |H| |x| (measured
          // 3-5e-7 * |theta| on 50-65 Eh problems); the solve moves to float64 below the larger
          // of switch_tol and 5e-7 * |theta|, or once the residual has stopped falling
          // (5 iterations without a 10% gain while below 1e-3).
          double tmax = 0.0;
          for (int j = 0; j < R; ++j) tmax = std::max(tmax, std::fabs(th[j]));
          if (best32 == 0.0 || rmax < 0.9 * best32) {
            best32 = rmax;
            stall32 = 0;
          } else {
            ++stall32;
          }
          to_fp64 = rmax < std::max(switch_tol, 5e-7 * tmax) || (stall32 >= 5 && rmax < 1e-3);
        }
        if (to_fp64) {
          // refinement: restart from the Ritz vectors with float64 sigma builds
          prec = FCG_FP64;
          if ((rc = W.copy_block(W.V.p, W.X.p, R))) return rc;
          if ((rc = W.gram(W.V.p, R, W.V.p, R, W.d_out.p))) return rc;
          if ((rc = W.enqueue_fetch(size_t(R) * R))) return rc;
          st = kSwG0;
          *act = Act::kWait;
          return FCG_OK;
        }
        if ((rc = new_directions(&wait))) return rc;
        st = wait ? kOrtho : kOrthoDone;
        if (wait) {
          *act = Act::kWait;
          return FCG_OK;
        }
        break;
      }
      case kOrtho:
        if ((rc = W.ortho_resume(&wait))) return rc;
        if (wait) {
          *act = Act::kWait;
          return FCG_OK;
        }
        st = kOrthoDone;
        break;
      case kOrthoDone:
        m = W.o_kept;
        if (m == 0) {  // the subspace cannot grow: converged as far as lindep allows
          st = kFinish;
          break;
        }
        *act = sigma(nv, m, prec, kAfterSigma);
        return FCG_OK;
      case kAfterSigma:
        ++sigma_calls;
        newlo = nv;
        nv += m;
        st = kIter;
        break;
      case kSwG0: {
        std::vector<double> G0(W.hout, W.hout + size_t(R) * R);
        if ((rc = W.ortho_start(0, R, std::move(G0), drop, &wait))) return rc;
        st = wait ? kSwOrtho : kSwDone;
        if (wait) {
          *act = Act::kWait;
          return FCG_OK;
        }
        break;
      }
      case kSwOrtho:
        if ((rc = W.ortho_resume(&wait))) return rc;
        if (wait) {
          *act = Act::kWait;
          return FCG_OK;
        }
        st = kSwDone;
        break;
      case kSwDone:
        m = W.o_kept;
        if (m < R) {  // Ritz vectors numerically dependent: keep the float32 result
          st = kFinish;
          break;
        }
        *act = sigma(0, m, prec, kAfterSwSigma);
        return FCG_OK;
      case kAfterSwSigma:
        ++sigma_calls;
        nv = m;
        newlo = 0;
        yprev_rows = 0;
        st = kIter;
        break;
      case kFinish:
        for (int j = 0; j < R; ++j) {
          energies[j] = th[j];
          residuals[j] = rn[j];
        }
        if ((rc = W.fetch_final(vectors, W.X.p, size_t(n) * R))) return rc;
        *iters = std::min(it, max_iter);
        ctx->stats.davidson_sigma_calls = sigma_calls;
        st = kFinished;
        *act = Act::kWait;  // the vectors are the caller's once the stream has been waited for
        return FCG_OK;
      case kFinished:
        *act = Act::kDone;
        return FCG_OK;
    }
  }
}

// New directions: corrections of the roots not yet converged (all roots in float32), with a
// restart on span{Y, Yprev} when the subspace is full (Q orthonormal, V <- V Q, AV <- AV Q,
// Hs <- Q^T Hs Q), then the orthonormalisation of the corrections against V (may wait).
int DavidsonRun::new_directions(bool* wait) {
  const int64_t n = W.n;
  const int kcap = W.kcap, kmax = W.kmax;
  int rc;
  std::vector<int> sel;
  for (int j = 0; j < R; ++j)
    if (rn[j] >= tol || prec == FCG_FP32) sel.push_back(j);
  const int nt = int(sel.size());
  const int ldg = nv + R;
  const double* Gall = W.hout + R;  // [V T]^T T, (nv + R) x R
  std::vector<double> S(size_t(nv) * nt), Gtt(size_t(nt) * nt);
  for (int q = 0; q < nt; ++q) {
    for (int i = 0; i < nv; ++i) S[i + size_t(nv) * q] = Gall[i + size_t(ldg) * sel[q]];
    for (int p = 0; p < nt; ++p) Gtt[p + size_t(nt) * q] = Gall[nv + sel[p] + size_t(ldg) * sel[q]];
  }
  const int nv_old = nv;
  if (nv + nt > kmax) {
    const int zc = R + ((gdk && yprev_rows > 0) ? R : 0);
    std::vector<double> Q;
    int q = 0;
    for (int c = 0; c < zc; ++c) {
      std::vector<double> z(nv, 0.0);
      if (c < R)
        for (int i = 0; i < nv; ++i) z[i] = Y[i + size_t(nv) * c];
      else
        for (int i = 0; i < yprev_rows; ++i) z[i] = Yprev[i + size_t(yprev_rows) * (c - R)];
      double n0 = 0.0;
      for (double x : z) n0 += x * x;
      n0 = std::sqrt(n0);
      for (int pass = 0; pass < 2; ++pass)
        for (int k = 0; k < q; ++k) {
          double d = 0.0;
          for (int i = 0; i < nv; ++i) d += Q[i + size_t(nv) * k] * z[i];
          for (int i = 0; i < nv; ++i) z[i] -= d * Q[i + size_t(nv) * k];
        }
      double nz = 0.0;
      for (double x : z) nz += x * x;
      nz = std::sqrt(nz);
      if (!(nz > 1e-8 * n0)) continue;
      for (double& x : z) x /= nz;
      Q.insert(Q.end(), z.begin(), z.end());
      ++q;
    }
    const double* dQ = nullptr;
    if ((rc = W.upload(Q.data(), size_t(nv) * q, &dQ))) return rc;
    if ((rc = W.flush())) return rc;
    if ((rc = W.update(W.V.p, nv, dQ, q, W.tmp.p))) return rc;
    if ((rc = W.copy_block(W.V.p, W.tmp.p, q))) return rc;
    if ((rc = W.update(W.AV.p, nv, dQ, q, W.tmp.p))) return rc;
    if ((rc = W.copy_block(W.AV.p, W.tmp.p, q))) return rc;
    std::vector<double> HQ(size_t(nv) * q, 0.0), Hn(size_t(q) * q, 0.0), Sn(size_t(q) * nt, 0.0),
        Yp(size_t(q) * R, 0.0);
    for (int c = 0; c < q; ++c)
      for (int k = 0; k < nv; ++k) {
        const double qk = Q[k + size_t(nv) * c];
        for (int i = 0; i < nv; ++i) HQ[i + size_t(nv) * c] += Hs[i + size_t(kcap) * k] * qk;
      }
    for (int c = 0; c < q; ++c)
      for (int r2 = 0; r2 < q; ++r2) {
        double s = 0.0;
        for (int i = 0; i < nv; ++i) s += Q[i + size_t(nv) * r2] * HQ[i + size_t(nv) * c];
        Hn[r2 + size_t(q) * c] = s;
      }
    for (int c = 0; c < q; ++c)
      for (int r2 = 0; r2 < c; ++r2) {
        const double a = 0.5 * (Hn[r2 + size_t(q) * c] + Hn[c + size_t(q) * r2]);
        Hn[r2 + size_t(q) * c] = Hn[c + size_t(q) * r2] = a;
      }
    for (int c = 0; c < nt; ++c)
      for (int r2 = 0; r2 < q; ++r2) {
        double s = 0.0;
        for (int i = 0; i < nv; ++i) s += Q[i + size_t(nv) * r2] * S[i + size_t(nv) * c];
        Sn[r2 + size_t(q) * c] = s;
      }
    for (int c = 0; c < R; ++c)
      for (int r2 = 0; r2 < q; ++r2) {
        double s = 0.0;
        for (int i = 0; i < nv; ++i) s += Q[i + size_t(nv) * r2] * Y[i + size_t(nv) * c];
        Yp[r2 + size_t(q) * c] = s;
      }
    for (int c = 0; c < q; ++c)
      for (int r2 = 0; r2 < q; ++r2) Hs[r2 + size_t(kcap) * c] = Hn[r2 + size_t(q) * c];
    S.swap(Sn);
    Yprev.swap(Yp);
    yprev_rows = q;
    nv = q;
  } else {
    Yprev = Y;
    yprev_rows = nv;
  }
  // the selected corrections move to V[:, nv : nv + nt] (never onto a later source column)
  {
    const double* srcs[kMaxB];
    double* dsts[kMaxB];
    int moves = 0;
    for (int q = 0; q < nt; ++q) {
      const int src = nv_old + sel[q], dst = nv + q;
      if (src == dst) continue;
      srcs[moves] = W.V.p + n * src;
      dsts[moves] = W.V.p + n * dst;
      ++moves;
    }
    if ((rc = W.move(moves, srcs, dsts))) return rc;
  }
  std::vector<double> G0(size_t(nv + nt) * nt);
  for (int c = 0; c < nt; ++c) {
    for (int i = 0; i < nv; ++i) G0[i + size_t(nv + nt) * c] = S[i + size_t(nv) * c];
    for (int p = 0; p < nt; ++p) G0[nv + p + size_t(nv + nt) * c] = Gtt[p + size_t(nt) * c];
  }
  return W.ortho_start(nv, nt, std::move(G0), drop, wait);
}

}  // namespace

extern "C" int fcg_sigma_closed_grouped(int n, fcg_ctx* const* ctxs, const int* R, const double* const* d_c,
                                        double* const* d_sigma, int precision);

namespace {

// One problem alone on its context's stream: waits and asynchronous sigma builds as it asks.
int run_solo(DavidsonRun& r) {
  fcg_ctx* ctx = r.ctx;
  for (;;) {
    Act a = Act::kDone;
    const int rc = r.step(&a);
    if (rc) return rc;
    if (a == Act::kDone) return FCG_OK;
    if (a == Act::kWait) {
      FCG_CUDA(cudaStreamSynchronize(ctx->stream));
      r.W.after_wait();
    } else {
      const int64_t n = r.W.n;
      const int rs = r.bst ? bst_sigma_device_async(ctx, r.sig_m, r.W.V.p + n * r.sig_col, r.W.AV.p + n * r.sig_col,
                                                    r.sig_prec, false)
                           : sigma_closed_device_async(ctx, r.sig_m, r.W.V.p + n * r.sig_col,
                                                       r.W.AV.p + n * r.sig_col, r.sig_prec);
      if (rs) return rs;
    }
  }
}

// Host threads that run fn(i), i < count, together with the calling thread.
class StepPool {
 public:
  explicit StepPool(int helpers) {
    for (int i = 0; i < helpers; ++i) th_.emplace_back([this] { work(); });
  }
  ~StepPool() {
    {
      std::lock_guard<std::mutex> lk(mu_);
      quit_ = true;
    }
    cv_.notify_all();
    for (auto& t : th_) t.join();
  }
  void run(int count, const std::function<void(int)>& fn) {
    if (th_.empty() || count < 4) {
      for (int i = 0; i < count; ++i) fn(i);
      return;
    }
    {
      std::lock_guard<std::mutex> lk(mu_);
      fn_ = &fn;
      count_ = count;
      next_.store(0);
      pending_ = int(th_.size());
      ++gen_;
    }
    cv_.notify_all();
    drain();
    std::unique_lock<std::mutex> lk(mu_);
    done_.wait(lk, [&] { return pending_ == 0; });
    fn_ = nullptr;
  }

 private:
  void drain() {
    for (int i = next_.fetch_add(1); i < count_; i = next_.fetch_add(1)) (*fn_)(i);
  }
  void work() {
    int seen = 0;
    for (;;) {
      {
        std::unique_lock<std::mutex> lk(mu_);
        cv_.wait(lk, [&] { return quit_ || gen_ != seen; });
        if (quit_) return;
        seen = gen_;
      }
      drain();
      std::lock_guard<std::mutex> lk(mu_);
      if (--pending_ == 0) done_.notify_all();
    }
  }
  std::vector<std::thread> th_;
  std::mutex mu_;
  std::condition_variable cv_, done_;
  const std::function<void(int)>* fn_ = nullptr;
  int count_ = 0, pending_ = 0, gen_ = 0;
  std::atomic<int> next_{0};
  bool quit_ = false;
};

// fetched values of one problem to the round's output area
struct GatherDesc {
  const double* src;
  double* dst;
  int64_t n;
  int first, blocks;
};
__global__ void __launch_bounds__(kDavThreads) gather_group_kernel(const GatherDesc* __restrict__ ds, int nd) {
  const int q = find_desc(ds, nd, int(blockIdx.x));
  const GatherDesc d = ds[q];
  const int64_t r = int64_t(int(blockIdx.x) - d.first) * blockDim.x + threadIdx.x;
  if (r < d.n) d.dst[r] = d.src[r];
}

#define FCG_LS_CUDA(call)                                                  \
  do {                                                                     \
    cudaError_t e_ = (call);                                               \
    if (e_ != cudaSuccess) {                                               \
      err = std::string(#call) + ": " + cudaGetErrorString(e_);            \
      return e_ == cudaErrorMemoryAllocation ? FCG_ENOMEM : FCG_ECUDA;     \
    }                                                                      \
  } while (0)

// Independent Davidson solves advanced together on one stream.  A round steps every ready
// problem until it needs the device (the host work of different problems on the step pool's
// threads), then runs the device work all of them recorded: one copy of the round's uploads
// and descriptors to the device; the operations level by level (each problem's i-th
// operation in level i, one grouped launch per kernel and block width in a level, so every
// problem's operations keep their order); the fetched values gathered into one area and
// copied to the host at once; the sigma builds asked for, as one grouped launch per
// precision; and one wait for the stream.  The problems' contexts must use this stream.
class Lockstep {
 public:
  enum State { kReady, kWaiting, kSigma, kDone, kFailed };
  struct Entry {
    DavidsonRun* run;
    int state;
    int rc;
  };
  std::vector<Entry> entries;
  std::string err;  // what made round() fail
  int64_t rounds = 0, launches = 0;
  double step_s = 0, issue_s = 0, wait_s = 0;  // host stepping, issuing, sigma builds and waits

  Lockstep(cudaStream_t s, int helpers) : stream_(s), pool_(helpers) {}

  // A problem joins between rounds (its init ran with grouped = true); nothing may be in
  // flight on the stream from an earlier round, as the staging areas may move.
  int add(DavidsonRun* r) {
    need_in_ += in_bytes(*r);
    need_out_ += out_doubles(*r);
    if (need_in_ > arena_.cap()) {
      const size_t cap = need_in_ + need_in_ / 2 + (size_t(64) << 10);
      FCG_LS_CUDA(arena_.h.alloc(cap));
      FCG_LS_CUDA(arena_.d.alloc(cap));
    }
    if (need_out_ > out_h_.n || need_out_ > out_d_.n) {
      const size_t cap = need_out_ + need_out_ / 2 + 1024;
      FCG_LS_CUDA(out_h_.alloc(cap));
      FCG_LS_CUDA(out_d_.alloc(cap));
    }
    r->W.arena = &arena_;
    entries.push_back({r, kReady, FCG_OK});
    return FCG_OK;
  }
  void erase(size_t i) {
    need_in_ -= in_bytes(*entries[i].run);
    need_out_ -= out_doubles(*entries[i].run);
    entries.erase(entries.begin() + i);
  }
  bool running() const {
    for (const Entry& e : entries)
      if (e.state == kReady) return true;
    return false;
  }
  int round();

 private:
  enum LaunchKind { kLGram, kLRitz, kLCombine, kLUpdate, kLMove, kLGather };
  struct Launch {
    int kind, width;
    size_t smem, off;
    int nd, blocks;
  };
  static size_t in_bytes(const DavidsonRun& r) {
    return r.W.up_cap * sizeof(double) + 16 * 16 + size_t(kMaxRoundOps) * (sizeof(MoveDesc) + 16) +
           sizeof(GatherDesc) + 16;
  }
  static size_t out_doubles(const DavidsonRun& r) { return r.W.out_cap + 2; }
  static int width_index(int w) { return w <= 0 ? 0 : w == 1 ? 1 : w == 2 ? 2 : w == 4 ? 3 : w == 8 ? 4 : 5; }

  // descriptors of one launch into the arena, numbered by their first block
  template <class D, class Get>
  int put(int kind, int width, size_t smem, size_t count, Get get) {
    const size_t off = arena_.reserve(count * sizeof(D));
    if (off == RoundArena::npos) {
      err = "Davidson rounds: staging area exhausted";
      return FCG_ELIMIT;
    }
    D* h = reinterpret_cast<D*>(arena_.h.p + off);
    int first = 0;
    for (size_t k = 0; k < count; ++k) {
      D d = get(k);
      d.first = first;
      first += d.blocks;
      h[k] = d;
    }
    launches_.push_back({kind, width, smem, off, int(count), first});
    return FCG_OK;
  }
  int launch(const Launch& L) {
    const unsigned g = unsigned(L.blocks);
    const unsigned char* p = arena_.d.p + L.off;
    switch (L.kind) {
      case kLGram:
        FCG_WIDTH_SWITCH(L.width, gram_group_kernel, g, kDavThreads, 0, stream_,
                         reinterpret_cast<const GramDesc*>(p), L.nd)
        break;
      case kLRitz:
        FCG_WIDTH_SWITCH(L.width, ritz_group_kernel, g, kDavThreads, L.smem, stream_,
                         reinterpret_cast<const RitzDesc*>(p), L.nd)
        break;
      case kLCombine:
        FCG_WIDTH_SWITCH(L.width, combine_group_kernel, g, kDavThreads, L.smem, stream_,
                         reinterpret_cast<const CombineDesc*>(p), L.nd)
        break;
      case kLUpdate:
        update_group_kernel<<<g, kDavThreads, 0, stream_>>>(reinterpret_cast<const UpdateDesc*>(p), L.nd);
        break;
      case kLMove:
        move_group_kernel<<<g, kDavThreads, 0, stream_>>>(reinterpret_cast<const MoveDesc*>(p), L.nd);
        break;
      default:
        gather_group_kernel<<<g, kDavThreads, 0, stream_>>>(reinterpret_cast<const GatherDesc*>(p), L.nd);
        break;
    }
    FCG_LS_CUDA(cudaGetLastError());
    ++launches;
    return FCG_OK;
  }

  cudaStream_t stream_;
  StepPool pool_;
  RoundArena arena_;
  DevBuf<double> out_d_;
  PinnedBuf<double> out_h_;
  size_t need_in_ = 0, need_out_ = 0;
  std::vector<Launch> launches_;
};

int Lockstep::round() {
  std::vector<int> ready;
  for (int i = 0; i < int(entries.size()); ++i)
    if (entries[i].state == kReady) ready.push_back(i);
  if (ready.empty()) return FCG_OK;
  ++rounds;
  using clock = std::chrono::steady_clock;
  const auto t0 = clock::now();
  arena_.used.store(0);
  pool_.run(int(ready.size()), [&](int k) {
    Entry& e = entries[ready[k]];
    DavidsonWork& W = e.run->W;
    W.ops.clear();
    W.fetch_count = W.fin_count = 0;
    Act a = Act::kDone;
    const int rc = e.run->step(&a);
    if (rc) {  // nothing of a failed step runs
      e.state = kFailed;
      e.rc = rc;
      W.ops.clear();
      W.fetch_count = W.fin_count = 0;
      return;
    }
    e.state = a == Act::kWait ? kWaiting : a == Act::kSigma ? kSigma : kDone;
  });
  const auto t1 = clock::now();
  step_s += std::chrono::duration<double>(t1 - t0).count();
  // the recorded operations, level by level
  launches_.clear();
  size_t levels = 0;
  for (int i : ready) levels = std::max(levels, entries[i].run->W.ops.size());
  static constexpr int kWidths[6] = {0, 1, 2, 4, 8, 16};
  std::vector<const RecOp*> bucket[5][6];
  int rc;
  for (size_t lev = 0; lev < levels; ++lev) {
    for (auto& row : bucket)
      for (auto& b : row) b.clear();
    for (int i : ready) {
      const std::vector<RecOp>& ops = entries[i].run->W.ops;
      if (lev < ops.size()) bucket[int(ops[lev].kind)][width_index(ops[lev].width)].push_back(&ops[lev]);
    }
    for (int kd = 0; kd < 5; ++kd)
      for (int wi = 0; wi < 6; ++wi) {
        const std::vector<const RecOp*>& b = bucket[kd][wi];
        if (b.empty()) continue;
        size_t smem = 0;
        for (const RecOp* op : b) smem = std::max(smem, op->smem);
        const int w = kWidths[wi];
        switch (OpKind(kd)) {
          case OpKind::kGram:
            rc = put<GramDesc>(kLGram, w, smem, b.size(), [&](size_t k) { return b[k]->g; });
            break;
          case OpKind::kRitz:
            rc = put<RitzDesc>(kLRitz, w, smem, b.size(), [&](size_t k) { return b[k]->r; });
            break;
          case OpKind::kCombine:
            rc = put<CombineDesc>(kLCombine, w, smem, b.size(), [&](size_t k) { return b[k]->c; });
            break;
          case OpKind::kUpdate:
            rc = put<UpdateDesc>(kLUpdate, w, smem, b.size(), [&](size_t k) { return b[k]->u; });
            break;
          default:
            rc = put<MoveDesc>(kLMove, w, smem, b.size(), [&](size_t k) { return b[k]->m; });
            break;
        }
        if (rc) return rc;
      }
  }
  // the fetched values of every problem into one area
  std::vector<std::pair<int, size_t>> fetched;  // entry, offset in the output area
  size_t out_used = 0;
  for (int i : ready) {
    const DavidsonWork& W = entries[i].run->W;
    if (!W.fetch_count) continue;
    fetched.push_back({i, out_used});
    out_used += (W.fetch_count + 1) & ~size_t(1);
  }
  if (out_used > out_d_.n) {
    err = "Davidson rounds: output area exhausted";
    return FCG_ELIMIT;
  }
  if (!fetched.empty()) {
    rc = put<GatherDesc>(kLGather, 0, 0, fetched.size(), [&](size_t k) {
      const DavidsonWork& W = entries[fetched[k].first].run->W;
      return GatherDesc{W.d_out.p, out_d_.p + fetched[k].second, int64_t(W.fetch_count), 0,
                        int((W.fetch_count + kDavThreads - 1) / kDavThreads)};
    });
    if (rc) return rc;
  }
  const size_t staged = std::min(arena_.used.load(), arena_.cap());
  if (staged) FCG_LS_CUDA(cudaMemcpyAsync(arena_.d.p, arena_.h.p, staged, cudaMemcpyHostToDevice, stream_));
  for (const Launch& L : launches_)
    if ((rc = launch(L))) return rc;
  if (out_used)
    FCG_LS_CUDA(cudaMemcpyAsync(out_h_.p, out_d_.p, out_used * sizeof(double), cudaMemcpyDeviceToHost, stream_));
  for (int i : ready) {
    const DavidsonWork& W = entries[i].run->W;
    if (W.fin_count)
      FCG_LS_CUDA(cudaMemcpyAsync(W.fin_dst, W.fin_src, W.fin_count * sizeof(double), cudaMemcpyDeviceToHost,
                                  stream_));
  }
  const auto t2 = clock::now();
  issue_s += std::chrono::duration<double>(t2 - t1).count();
  // the sigma builds, one grouped launch per precision
  for (int p : {FCG_FP32, FCG_FP64}) {
    std::vector<fcg_ctx*> cs;
    std::vector<int> Rs;
    std::vector<const double*> dc;
    std::vector<double*> ds;
    for (int i : ready) {
      const DavidsonRun& r = *entries[i].run;
      if (entries[i].state != kSigma || r.sig_prec != p) continue;
      const int64_t n = r.W.n;
      if (r.bst) {  // BST sigma: a launch sequence of its own on the lane's stream
        if ((rc = bst_sigma_device_async(r.ctx, r.sig_m, r.W.V.p + n * r.sig_col, r.W.AV.p + n * r.sig_col, p,
                                         false))) {
          err = r.ctx->err;
          return rc;
        }
        launches += 3;
        continue;
      }
      cs.push_back(r.ctx);
      Rs.push_back(r.sig_m);
      dc.push_back(r.W.V.p + n * r.sig_col);
      ds.push_back(r.W.AV.p + n * r.sig_col);
    }
    if (cs.empty()) continue;
    rc = cs.size() == 1 ? sigma_closed_device_async(cs[0], Rs[0], dc[0], ds[0], p)
                        : fcg_sigma_closed_grouped(int(cs.size()), cs.data(), Rs.data(), dc.data(), ds.data(), p);
    if (rc) {
      err = cs[0]->err;
      return rc;
    }
    launches += 3;
  }
  FCG_LS_CUDA(cudaStreamSynchronize(stream_));
  wait_s += std::chrono::duration<double>(clock::now() - t2).count();
  for (const auto& f : fetched) {
    DavidsonWork& W = entries[f.first].run->W;
    std::memcpy(W.hout, out_h_.p + f.second, W.fetch_count * sizeof(double));
  }
  for (int i : ready) {
    Entry& e = entries[i];
    if (e.state == kWaiting || e.state == kSigma) {
      e.run->W.after_wait();
      e.state = kReady;
    }
  }
  return FCG_OK;
}

// host threads that help a lockstep executor step its problems
int step_helpers(int share) {
  const int hw = int(std::max(1u, std::thread::hardware_concurrency()));
  return std::max(0, std::min(15, hw / std::max(share, 1) - 1));
}

}  // namespace

extern "C" int fcg_davidson(fcg_ctx* ctx, int R, const double* v0, int max_iter, int max_ss_vecs, double tol,
                            double lindep, int precision, int precond, double* energies, double* vectors,
                            double* residuals, int* iters) {
  if (!ctx) return FCG_EINVAL;
  FCG_CUDA(cudaSetDevice(ctx->device));
  DavidsonRun run;
  const int rc = run.init(ctx, R, v0, max_iter, max_ss_vecs, tol, lindep, precision, precond, energies, vectors,
                          residuals, iters);
  if (rc) return rc;
  return run_solo(run);
}

extern "C" int fcg_bst_davidson(fcg_ctx* ctx, int R, const double* v0, const double* hdiag, int max_iter,
                                int max_ss_vecs, double tol, double lindep, int precision, double* energies,
                                double* vectors, double* residuals, int* iters) {
  if (!ctx) return FCG_EINVAL;
  FCG_CUDA(cudaSetDevice(ctx->device));
  DavidsonRun run;
  int rc = run.init(ctx, R, v0, max_iter, max_ss_vecs, tol, lindep, precision, 0, energies, vectors, residuals, iters,
                    false, true, hdiag);
  if (rc) return rc;
  rc = run_solo(run);
  if (rc) return rc;
  return precision == FCG_FP32 ? bst_tc_check(ctx) : FCG_OK;
}

extern "C" int fcg_davidson_grouped(int n, fcg_ctx* const* ctxs, const int* R, const double* const* v0, int max_iter,
                                    int max_ss_vecs, double tol, double lindep, int precision, int precond,
                                    double* const* energies, double* const* vectors, double* const* residuals,
                                    int* iters) {
  if (n < 1 || !ctxs || !ctxs[0]) return FCG_EINVAL;
  fcg_ctx* ctx = ctxs[0];
  FCG_REQUIRE(R && v0 && energies && vectors && residuals && iters, FCG_EINVAL, "null pointer");
  FCG_REQUIRE(n <= 65535, FCG_ELIMIT, "at most 65535 problems per group");
  for (int q = 0; q < n; ++q) {
    FCG_REQUIRE(ctxs[q], FCG_EINVAL, "null context in the group");
    FCG_REQUIRE(ctxs[q]->device == ctx->device, FCG_EINVAL, "all contexts of a group must share a device");
    for (int q2 = 0; q2 < q; ++q2) FCG_REQUIRE(ctxs[q2] != ctxs[q], FCG_EINVAL, "a context appears twice in the group");
  }
  FCG_CUDA(cudaSetDevice(ctx->device));
  if (n == 1)
    return fcg_davidson(ctx, R[0], v0[0], max_iter, max_ss_vecs, tol, lindep, precision, precond, energies[0],
                        vectors[0], residuals[0], &iters[0]);
  // Lanes: interleaved subsets of the problems, each solved in lockstep on its first
  // problem's stream by a host thread of its own, so that one lane's host work overlaps the
  // others' device work (one lane below 64 problems).
  const int lanes = std::max(1, std::min(4, n / 32));
  struct LaneOut {
    int rc = FCG_OK;
    int64_t bad = -1;  // failing problem, -1 for a failure of the lane's stream
    std::string err;
    int64_t rounds = 0, launches = 0;
    double setup = 0, step = 0, issue = 0, wait = 0;
  };
  std::vector<LaneOut> out(static_cast<size_t>(lanes));
  std::vector<cudaStream_t> saved(n);
  for (int q = 0; q < n; ++q) saved[q] = ctxs[q]->stream;
  auto run_lane = [&](int l) {
    LaneOut& o = out[size_t(l)];
    cudaSetDevice(ctx->device);
    std::vector<int> mem;
    for (int q = l; q < n; q += lanes) mem.push_back(q);
    const cudaStream_t stream = saved[mem[0]];
    for (int q : mem) ctxs[q]->stream = stream;  // the lane's work on its first problem's stream
    {
      std::vector<std::unique_ptr<DavidsonRun>> runs;
      Lockstep L(stream, step_helpers(lanes));
      const auto t0 = std::chrono::steady_clock::now();
      for (size_t i = 0; i < mem.size() && o.rc == FCG_OK; ++i) {
        const int q = mem[i];
        runs.emplace_back(new DavidsonRun());
        o.rc = runs[i]->init(ctxs[q], R[q], v0[q], max_iter, max_ss_vecs, tol, lindep, precision, precond,
                             energies[q], vectors[q], residuals[q], &iters[q], true);
        if (o.rc) {
          o.bad = q;
          o.err = ctxs[q]->err;
        } else if ((o.rc = L.add(runs[i].get()))) {
          o.bad = q;
          o.err = L.err;
        }
      }
      o.setup = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
      while (o.rc == FCG_OK && L.running()) {
        if ((o.rc = L.round())) {
          o.bad = -1;
          o.err = L.err;
          break;
        }
        for (size_t i = 0; i < L.entries.size(); ++i)
          if (L.entries[i].state == Lockstep::kFailed) {
            o.rc = L.entries[i].rc;
            o.bad = mem[i];
            o.err = ctxs[mem[i]]->err;
            break;
          }
      }
      cudaStreamSynchronize(stream);  // nothing of the lane in flight when its runs go
      o.rounds = L.rounds;
      o.launches = L.launches;
      o.step = L.step_s;
      o.issue = L.issue_s;
      o.wait = L.wait_s;
    }
    for (int q : mem) ctxs[q]->stream = saved[q];
  };
  {
    std::vector<std::thread> pool;
    for (int l = 1; l < lanes; ++l) pool.emplace_back(run_lane, l);
    run_lane(0);
    for (auto& t : pool) t.join();
  }
  // the failure of the lowest problem (a stream failure first), named as one group would
  int rc = FCG_OK;
  int64_t first = n;
  for (const LaneOut& o : out)
    if (o.rc != FCG_OK && o.bad < first) {
      rc = o.rc;
      first = o.bad;
      ctx->err = o.bad >= 0 ? o.err + " (problem " + std::to_string(o.bad) + ")" : o.err;
    }
  ctx->stats.group_rounds = 0;
  ctx->stats.group_launches = 0;
  ctx->stats.group_setup_seconds = ctx->stats.group_step_seconds = 0.0;
  ctx->stats.group_issue_seconds = ctx->stats.group_wait_seconds = 0.0;
  for (const LaneOut& o : out) {  // lanes run side by side: the longest of each
    ctx->stats.group_rounds = std::max(ctx->stats.group_rounds, o.rounds);
    ctx->stats.group_launches += o.launches;
    ctx->stats.group_setup_seconds = std::max(ctx->stats.group_setup_seconds, o.setup);
    ctx->stats.group_step_seconds = std::max(ctx->stats.group_step_seconds, o.step);
    ctx->stats.group_issue_seconds = std::max(ctx->stats.group_issue_seconds, o.issue);
    ctx->stats.group_wait_seconds = std::max(ctx->stats.group_wait_seconds, o.wait);
  }
  return rc;
}

// ---- serving: continuous batching of Davidson solves ---------------------------------------
//
// A server owns scheduler threads (lanes), each with a stream of its own.  Callers prepare a
// context per request (fcg_set_ops, fcg_set_terms, fcg_state_set -- in their own threads) and
// submit it with a guess; a lane admits requests while slots and the memory budget allow, and
// runs its admitted solves in lockstep rounds as fcg_davidson_grouped does: every round
// advances each solve to its next need of the device, then serves all of them with grouped
// launches and one wait for the stream.  Solves that finish leave after the round, queued
// requests join at the next, so a request's work overlaps with whatever is in flight.  A
// solve's result is the same as fcg_davidson's on its own (the grouped sigma adds each
// problem's sums in another order).

struct fcg_server {
  int device = 0;
  int max_active = 1;  // admitted solves over all lanes
  int lanes = 1;       // scheduler threads, each with its own stream and lockstep group
  double budget = 0;
  std::vector<cudaStream_t> streams;  // one per lane
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  bool stop = false;
  std::vector<std::thread> workers;
  struct Ticket {
    int64_t id = 0;
    fcg_ctx* ctx = nullptr;
    int R = 0, max_iter = 0, max_ss_vecs = 0, precision = 0, precond = 0;
    double tol = 0, lindep = 0;
    bool bst = false;            // a BST solve (fcg_submit_bst)
    std::vector<double> bst_hd;  // its preconditioner diagonal, or empty
    std::vector<double> v0, energies, vectors, residuals;
    int iters = 0;
    int state = 0;  // 0 queued, 1 running, 2 done, 3 failed
    int rc = 0;
    std::string err;
    double footprint = 0;
  };
  std::map<int64_t, std::shared_ptr<Ticket>> tickets;
  std::deque<std::shared_ptr<Ticket>> queue;
  int64_t next_id = 1;
  double in_use = 0;
  int running = 0;  // admitted solves over all lanes

  void lane_loop(int lane);
};

namespace {

struct Slot {
  std::shared_ptr<fcg_server::Ticket> t;
  std::unique_ptr<DavidsonRun> run;
  cudaStream_t saved = nullptr;
};

}  // namespace

// One lane: admits queued requests while it runs fewer than its share of max_active, the
// server runs fewer than max_active and the memory budget allows (a request larger than the
// budget runs when nothing else does), and advances its admitted solves in lockstep rounds on
// its own stream.  Lanes overlap one another's kernels and host work.
void fcg_server::lane_loop(int lane) {
  cudaSetDevice(device);
  cudaStream_t stream = streams[lane];
  const int share = (max_active + lanes - 1) / lanes;
  Lockstep L(stream, step_helpers(lanes));
  std::vector<Slot> active;  // active[i] runs as L.entries[i]
  auto finish = [&](Slot& sl, int rc) {  // under the lock
    sl.t->ctx->stream = sl.saved;
    sl.t->rc = rc;
    sl.t->state = rc == FCG_OK ? 2 : 3;
    if (rc != FCG_OK) sl.t->err = sl.t->ctx->err;
    in_use -= sl.t->footprint;
    --running;
    cv_done.notify_all();
    cv_work.notify_all();  // memory and a slot are free for the other lanes
  };
  for (;;) {
    {
      std::unique_lock<std::mutex> lk(mu);
      while (!queue.empty() && int(active.size()) < share && running < max_active &&
             (running == 0 || in_use + queue.front()->footprint <= budget)) {
        auto t = queue.front();
        queue.pop_front();
        Slot sl;
        sl.t = t;
        sl.saved = t->ctx->stream;
        t->ctx->stream = stream;
        t->state = 1;
        in_use += t->footprint;
        ++running;
        sl.run.reset(new DavidsonRun());
        lk.unlock();
        int rc = sl.run->init(t->ctx, t->R, t->v0.data(), t->max_iter, t->max_ss_vecs, t->tol, t->lindep,
                              t->precision, t->precond, t->energies.data(), t->vectors.data(),
                              t->residuals.data(), &t->iters, true, t->bst,
                              t->bst_hd.empty() ? nullptr : t->bst_hd.data());
        if (rc == FCG_OK && (rc = L.add(sl.run.get()))) t->ctx->err = L.err;
        lk.lock();
        if (rc) {
          cudaStreamSynchronize(stream);
          finish(sl, rc);
        } else {
          active.push_back(std::move(sl));
        }
      }
      if (active.empty()) {
        if (stop && queue.empty()) return;
        cv_work.wait_for(lk, std::chrono::milliseconds(20));
        continue;
      }
    }
    const int rc_round = L.round();
    if (rc_round) cudaStreamSynchronize(stream);
    // retire finished and failed solves
    std::unique_lock<std::mutex> lk(mu);
    for (size_t i = active.size(); i-- > 0;) {
      const Lockstep::Entry& e = L.entries[i];
      if (e.state != Lockstep::kDone && e.state != Lockstep::kFailed && rc_round == FCG_OK) continue;
      Slot& sl = active[i];
      if (e.state == Lockstep::kDone) {
        // a float BST solve: its tensor-core tiles must all have completed
        const int rc_tc = sl.t->bst && sl.t->precision == FCG_FP32 ? bst_tc_check(sl.t->ctx) : FCG_OK;
        finish(sl, rc_tc);
      } else if (e.state == Lockstep::kFailed) {
        finish(sl, e.rc);
      } else {
        sl.t->ctx->err = "serving: the lane's stream failed: " + L.err;
        finish(sl, rc_round);
      }
      L.erase(i);
      active.erase(active.begin() + i);
    }
  }
}

extern "C" {

int fcg_server_create(int device, int max_active, int lanes, double memory_budget, fcg_server** out) {
  if (!out || max_active < 1 || lanes < 1 || lanes > 64 || !(memory_budget > 0)) return FCG_EINVAL;
  *out = nullptr;
  if (cudaSetDevice(device) != cudaSuccess) return FCG_ECUDA;
  std::unique_ptr<fcg_server> s(new fcg_server());
  s->device = device;
  s->max_active = max_active;
  s->lanes = std::min(lanes, max_active);
  s->budget = memory_budget;
  for (int l = 0; l < s->lanes; ++l) {
    cudaStream_t st = nullptr;
    if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) {
      for (cudaStream_t x : s->streams) cudaStreamDestroy(x);
      return FCG_ECUDA;
    }
    s->streams.push_back(st);
  }
  fcg_server* raw = s.get();
  for (int l = 0; l < s->lanes; ++l) s->workers.emplace_back([raw, l] { raw->lane_loop(l); });
  *out = s.release();
  return FCG_OK;
}

int fcg_server_destroy(fcg_server* s) {
  if (!s) return FCG_EINVAL;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
    for (auto& t : s->queue) {  // never admitted: failed, their contexts untouched
      t->state = 3;
      t->rc = FCG_ESTATE;
      t->err = "serving: the server was destroyed before the request ran";
    }
    s->queue.clear();
    s->cv_done.notify_all();
  }
  s->cv_work.notify_all();
  for (auto& w : s->workers) w.join();  // the admitted solves finish first (each is bounded by its max_iter)
  for (cudaStream_t x : s->streams) cudaStreamDestroy(x);
  delete s;
  return FCG_OK;
}

static int submit_impl(fcg_server* s, fcg_ctx* ctx, int R, const double* v0, int max_iter, int max_ss_vecs,
                       double tol, double lindep, int precision, int precond, int64_t* ticket, bool bst,
                       const double* bst_hd) {
  if (!s || !ctx || !v0 || !ticket || R < 1 || R > kMaxB) return FCG_EINVAL;
  if (bst ? (!ctx->have_bst || ctx->bst_core_total < R) : (!ctx->have_state || ctx->n_cfg < R)) return FCG_ESTATE;
  if (ctx->device != s->device) return FCG_EINVAL;
  auto t = std::make_shared<fcg_server::Ticket>();
  const int64_t n = bst ? ctx->bst_core_total : ctx->n_cfg;
  t->bst = bst;
  if (bst && bst_hd) t->bst_hd.assign(bst_hd, bst_hd + n);
  t->ctx = ctx;
  t->R = R;
  t->max_iter = max_iter;
  t->max_ss_vecs = max_ss_vecs;
  t->tol = tol;
  t->lindep = lindep;
  t->precision = precision;
  t->precond = precond;
  t->v0.assign(v0, v0 + n * R);
  t->energies.assign(R, 0.0);
  t->residuals.assign(R, 0.0);
  t->vectors.assign(size_t(n) * R, 0.0);
  // device memory the solve holds: V and H V (max_ss_vecs R + R columns), X, the restart
  // scratch, the Gram partial sums and the float64 / float32 sigma copies
  const double kcap = double(std::min<int64_t>(int64_t(std::max(max_ss_vecs, 2)) * R, n) + R);
  t->footprint = 8.0 * double(n) * (2.0 * kcap + 6.0 * R) + 8.0 * 128.0 * kcap * R;
  std::lock_guard<std::mutex> lk(s->mu);
  for (auto& kv : s->tickets)
    if (kv.second->ctx == ctx && kv.second->state < 2) return FCG_EINVAL;  // the context is busy
  t->id = s->next_id++;
  s->tickets[t->id] = t;
  s->queue.push_back(t);
  *ticket = t->id;
  s->cv_work.notify_all();
  return FCG_OK;
}

int fcg_submit(fcg_server* s, fcg_ctx* ctx, int R, const double* v0, int max_iter, int max_ss_vecs, double tol,
               double lindep, int precision, int precond, int64_t* ticket) {
  return submit_impl(s, ctx, R, v0, max_iter, max_ss_vecs, tol, lindep, precision, precond, ticket, false, nullptr);
}

int fcg_submit_bst(fcg_server* s, fcg_ctx* ctx, int R, const double* v0, const double* hdiag, int max_iter,
                   int max_ss_vecs, double tol, double lindep, int precision, int64_t* ticket) {
  return submit_impl(s, ctx, R, v0, max_iter, max_ss_vecs, tol, lindep, precision, 0, ticket, true, hdiag);
}

int fcg_poll(fcg_server* s, int64_t ticket, int* state) {
  if (!s || !state) return FCG_EINVAL;
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->tickets.find(ticket);
  if (it == s->tickets.end()) return FCG_EINVAL;
  *state = it->second->state;
  return FCG_OK;
}

int fcg_wait(fcg_server* s, int64_t ticket, int timeout_ms, double* energies, double* vectors, double* residuals,
             int* iters) {
  if (!s) return FCG_EINVAL;
  std::unique_lock<std::mutex> lk(s->mu);
  auto it = s->tickets.find(ticket);
  if (it == s->tickets.end()) return FCG_EINVAL;
  std::shared_ptr<fcg_server::Ticket> t = it->second;
  const bool ended = s->cv_done.wait_for(lk, std::chrono::milliseconds(std::max(timeout_ms, 0)),
                                         [&] { return t->state >= 2; });
  if (!ended) return FCG_ETIMEDOUT;
  if (t->state == 3) {
    t->ctx->err = t->err;
    const int rc = t->rc ? t->rc : FCG_ECUDA;
    s->tickets.erase(it);
    return rc;
  }
  if (energies) std::copy(t->energies.begin(), t->energies.end(), energies);
  if (residuals) std::copy(t->residuals.begin(), t->residuals.end(), residuals);
  if (vectors) std::copy(t->vectors.begin(), t->vectors.end(), vectors);
  if (iters) *iters = t->iters;
  s->tickets.erase(it);
  return FCG_OK;
}

}  // extern "C"
