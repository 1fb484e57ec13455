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
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
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

// out[i + a*j] = sum_r A[r + lda*i] * B[r + ldb*j] for i < a, j < b <= BM.  The kernels of
// this file are compiled for block widths BM = 1, 2, 4, 8, 16 and launched with the smallest
// that fits: unrolled loops over unused columns would still issue their FP64 instructions.
// Grid: x = row blocks, y = groups of 32 columns of A; a lane owns one column of A, each warp
// a contiguous slice of the block's rows.  Each block writes its partial sums to
// part[blk][i + a*j]; the last block of a column group to finish (counted in
// counters[blockIdx.y], which it resets) adds the group's partials in row-block order, so
// the result does not depend on the order in which blocks run.
template <int BM>
__global__ void __launch_bounds__(kDavThreads) gram_kernel(const double* __restrict__ A, int64_t lda, int a,
                                                           const double* __restrict__ B, int64_t ldb, int b, int64_t n,
                                                           int64_t rows_per_block, double* __restrict__ part,
                                                           double* __restrict__ out, unsigned* __restrict__ counters) {
  __shared__ double red[kGramWarps][BM][32];
  __shared__ unsigned ticket;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int i = blockIdx.y * 32 + lane;
  const int64_t r0 = int64_t(blockIdx.x) * rows_per_block;
  const int64_t r1 = r0 + rows_per_block < n ? r0 + rows_per_block : n;
  const int64_t slice = (rows_per_block + kGramWarps - 1) / kGramWarps;
  const int64_t s0 = r0 + warp * slice;
  const int64_t s1 = s0 + slice < r1 ? s0 + slice : r1;
  double acc[BM];
#pragma unroll
  for (int j = 0; j < BM; ++j) acc[j] = 0.0;
  if (i < a) {
    const double* Ai = A + lda * i;
    int64_t r = s0;
    for (; r + 8 <= s1; r += 8) {  // eight rows per step: independent loads in flight
      double x[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) x[u] = Ai[r + u];
#pragma unroll
      for (int j = 0; j < BM; ++j)
        if (j < b) {
          const double* Bj = B + ldb * j + r;
#pragma unroll
          for (int u = 0; u < 8; ++u) acc[j] = fma(x[u], Bj[u], acc[j]);
        }
    }
    for (; r < s1; ++r) {
      const double x = Ai[r];
#pragma unroll
      for (int j = 0; j < BM; ++j)
        if (j < b) acc[j] = fma(x, B[r + ldb * j], acc[j]);
    }
  }
#pragma unroll
  for (int j = 0; j < BM; ++j)
    if (j < b) red[warp][j][lane] = acc[j];
  __syncthreads();
  const int64_t P = int64_t(a) * b;
  for (int t = threadIdx.x; t < b * 32; t += blockDim.x) {
    const int j = t >> 5, l = t & 31;
    const int col = blockIdx.y * 32 + l;
    double s = 0.0;
    for (int w = 0; w < kGramWarps; ++w) s += red[w][j][l];
    if (col < a) part[int64_t(blockIdx.x) * P + col + int64_t(a) * j] = s;
  }
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) ticket = atomicAdd(counters + blockIdx.y, 1u);
  __syncthreads();
  if (ticket != gridDim.x - 1) return;
  for (int t = threadIdx.x; t < b * 32; t += blockDim.x) {
    const int j = t >> 5, l = t & 31;
    const int col = blockIdx.y * 32 + l;
    if (col >= a) continue;
    const int64_t p = col + int64_t(a) * j;
    double s = 0.0;
    for (unsigned k = 0; k < gridDim.x; ++k) s += __ldcg(part + int64_t(k) * P + p);
    out[p] = s;
  }
  if (threadIdx.x == 0) counters[blockIdx.y] = 0u;
}

// C[:, j] = sum_i A[:, i] * Y[i + a*j] for j < b (C and A must not overlap)
__global__ void update_kernel(const double* __restrict__ A, int64_t lda, int a, const double* __restrict__ Y, int b,
                              double* __restrict__ C, int64_t ldc, int64_t n) {
  const int64_t r = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (r >= n) return;
  for (int j = 0; j < b; ++j) {
    double s = 0.0;
    for (int i = 0; i < a; ++i) s = fma(A[r + lda * i], Y[i + int64_t(a) * j], s);
    C[r + ldc * j] = s;
  }
}

// Ritz vectors and corrections for R roots: per row r,
//   x_j = sum_i V[r, i] Y[i, j],  hx_j = sum_i AV[r, i] Y[i, j],  res_j = hx_j - theta_j x_j,
//   X[r, j] = x_j,  T[r, j] = res_j / (theta_j - hd[r])  (res_j when !precond; the denominator
//   is kept at least 1e-6 away from zero), and rn_out[j] = sum_r res_j^2 (per-block partial
//   sums in rn_part, added in block order by the last block to finish).
// Y (nv x R, column-major) and theta are staged in shared memory.
template <int BM>
__global__ void __launch_bounds__(kDavThreads) ritz_residual_kernel(const double* __restrict__ V,
                                                                    const double* __restrict__ AV, int64_t ld, int nv,
                                                                    const double* __restrict__ Y,
                                                                    const double* __restrict__ theta,
                                                                    const double* __restrict__ hd, int R, int64_t n,
                                                                    double* __restrict__ X, double* __restrict__ T,
                                                                    int precond, double* __restrict__ rn_part,
                                                                    double* __restrict__ rn_out,
                                                                    unsigned* __restrict__ counter) {
  extern __shared__ double sm[];
  double* sY = sm;              // nv * R
  double* sth = sm + nv * R;    // R
  __shared__ double red[kDavThreads / 32][BM];
  for (int t = threadIdx.x; t < nv * R; t += blockDim.x) sY[t] = Y[t];
  for (int t = threadIdx.x; t < R; t += blockDim.x) sth[t] = theta[t];
  __syncthreads();
  const int64_t r = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  double x[BM], hx[BM];
#pragma unroll
  for (int j = 0; j < BM; ++j) x[j] = hx[j] = 0.0;
  if (r < n) {
    for (int i0 = 0; i0 < nv; i0 += 8) {  // eight columns' loads in flight before their use
      double v[8], av[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const bool in = i0 + u < nv;
        v[u] = in ? V[r + ld * (i0 + u)] : 0.0;
        av[u] = in ? AV[r + ld * (i0 + u)] : 0.0;
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
      double d = precond ? sth[j] - hd[r] : 1.0;
      if (fabs(d) < 1e-6) d = d < 0 ? -1e-6 : 1e-6;
      X[r + n * j] = x[j];
      T[r + ld * j] = res / d;
    }
    double s = res * res;
    for (int off = 16; off > 0; off >>= 1) s += __shfl_down_sync(0xffffffffu, s, off);
    if (lane == 0) red[warp][j] = s;
  }
  __syncthreads();
  if (threadIdx.x < R) {
    double s = 0.0;
    for (int w = 0; w < int(blockDim.x >> 5); ++w) s += red[w][threadIdx.x];
    rn_part[int64_t(blockIdx.x) * R + threadIdx.x] = s;
  }
  // the last block to finish adds the blocks' partial sums in block order
  __shared__ unsigned ticket;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) ticket = atomicAdd(counter, 1u);
  __syncthreads();
  if (ticket != gridDim.x - 1) return;
  if (threadIdx.x < R) {
    double s = 0.0;
    for (unsigned k = 0; k < gridDim.x; ++k) s += __ldcg(rn_part + int64_t(k) * R + threadIdx.x);
    rn_out[threadIdx.x] = s;
  }
  if (threadIdx.x == 0) *counter = 0u;
}

// In place on the new block T = V[:, nv : nv + kt] (leading dimension ld):
//   T[:, j] <- sum_{i < kt} T[:, i] M[i + kt*j] - sum_{i < nv} V[:, i] P[i + nv*j],  j < mo.
// A thread owns a row: it reads the row's T entries before writing any (kt, mo <= BM).
// M (kt x mo) and P (nv x mo) are staged in shared memory; P may be null (no projection).
template <int BM>
__global__ void __launch_bounds__(kDavThreads) combine_kernel(double* __restrict__ V, int64_t ld, int nv, int kt,
                                                              const double* __restrict__ M,
                                                              const double* __restrict__ P, int mo, int64_t n) {
  extern __shared__ double sm[];
  double* sM = sm;            // kt * mo
  double* sP = sm + kt * mo;  // nv * mo
  for (int t = threadIdx.x; t < kt * mo; t += blockDim.x) sM[t] = M[t];
  if (P)
    for (int t = threadIdx.x; t < nv * mo; t += blockDim.x) sP[t] = P[t];
  __syncthreads();
  const int64_t r = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (r >= n) return;
  double* T = V + ld * nv;
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
  if (P) {
    for (int i0 = 0; i0 < nv; i0 += 8) {  // eight columns' loads in flight before their use
      double v[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) v[u] = i0 + u < nv ? V[r + ld * (i0 + u)] : 0.0;
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

// the smallest compiled block width (1, 2, 4, 8, 16) that holds w columns
inline int width_class(int w) { return w <= 1 ? 1 : w <= 2 ? 2 : w <= 4 ? 4 : w <= 8 ? 8 : 16; }

#define FCG_WIDTH_SWITCH(w, KERNEL, LAUNCH, ...)       \
  switch (width_class(w)) {                            \
    case 1: KERNEL<1><<<LAUNCH>>>(__VA_ARGS__); break; \
    case 2: KERNEL<2><<<LAUNCH>>>(__VA_ARGS__); break; \
    case 4: KERNEL<4><<<LAUNCH>>>(__VA_ARGS__); break; \
    case 8: KERNEL<8><<<LAUNCH>>>(__VA_ARGS__); break; \
    default: KERNEL<16><<<LAUNCH>>>(__VA_ARGS__); break; \
  }

}  // namespace

extern "C" int fcg_diagonal(fcg_ctx* ctx, int op_id, double* hd);

namespace {

struct DavidsonWork {
  fcg_ctx* ctx = nullptr;
  int64_t n = 0;
  int R = 0, kmax = 0, kcap = 0;  // kcap = kmax + R columns of V and AV
  int row_blocks = 1;             // Gram products: row blocks, rows per block
  int64_t rows_per_block = 1;
  int res_blocks = 1;             // residual kernel blocks
  DevBuf<double> V, AV, X, tmp, hd, part, rn_part, d_out, d_up;
  DevBuf<unsigned> counters;  // last-block tickets: [0, ngroups) Gram column groups, [ngroups] residual
  int ngroups = 1;
  PinnedBuf<double> h_out, h_up;
  size_t up_used = 0, up_sent = 0;

  // Stage `count` doubles in the pinned upload area and return where they will be on the
  // device once flush() has queued the copy.  The area is reused only after the next fetch().
  int upload(const double* src, size_t count, const double** dptr) {
    fcg_ctx* ctx = this->ctx;
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
    const dim3 grid(unsigned(row_blocks), unsigned((a + 31) / 32));
#define FCG_GRAM_LAUNCH grid, kDavThreads, 0, ctx->stream
    FCG_WIDTH_SWITCH(b, gram_kernel, FCG_GRAM_LAUNCH, A, n, a, B, n, b, n, rows_per_block, part.p, out, counters.p)
#undef FCG_GRAM_LAUNCH
    FCG_CUDA(cudaGetLastError());
    return FCG_OK;
  }
  // queue h_out[0 : count) = d_out[0 : count); the values are there after the next wait for
  // the stream, after which after_wait() frees the staging area
  int enqueue_fetch(size_t count) {
    fcg_ctx* ctx = this->ctx;
    FCG_CUDA(cudaMemcpyAsync(h_out.p, d_out.p, count * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
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
    const size_t smem = sizeof(double) * (size_t(kt) * mo + (proj ? size_t(nv) * mo : 0));
    const unsigned blocks = unsigned((n + kDavThreads - 1) / kDavThreads);
#define FCG_COMBINE_LAUNCH blocks, kDavThreads, smem, ctx->stream
    FCG_WIDTH_SWITCH(std::max(kt, mo), combine_kernel, FCG_COMBINE_LAUNCH, V.p, n, nv, kt, dM, dP, mo, n)
#undef FCG_COMBINE_LAUNCH
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
    const double* G1 = h_out.p;
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
    const double* G3 = h_out.p;
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

  int init(fcg_ctx* c, int R_, const double* v0_, int max_iter_, int max_ss_vecs, double tol_, double lindep,
           int precision, int precond_, double* e, double* vecs, double* res, int* its) {
    ctx = c;
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
    FCG_REQUIRE(ctx->have_state, FCG_ESTATE, "fcg_state_set must come first");
    FCG_REQUIRE(v0 && energies && vectors && residuals && iters, FCG_EINVAL, "null pointer");
    FCG_REQUIRE(R >= 1 && R <= kMaxB && R <= ctx->n_cfg, FCG_ELIMIT, "R must be in [1, min(16, n_cfg)]");
    FCG_REQUIRE(max_ss_vecs >= 2 && max_iter >= 1 && tol > 0, FCG_EINVAL, "bad Davidson settings");
    FCG_REQUIRE(precision == FCG_FP64 || precision == FCG_FP32, FCG_EINVAL, "unknown precision");
    const int64_t n = ctx->n_cfg;
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
    }
    W.row_blocks = int(std::max<int64_t>(1, std::min<int64_t>(kMaxRowBlocks, (n + kGramRows - 1) / kGramRows)));
    W.rows_per_block = (n + W.row_blocks - 1) / W.row_blocks;
    W.res_blocks = int((n + kDavThreads - 1) / kDavThreads);
    FCG_CUDA(W.V.alloc(size_t(n) * kcap));
    FCG_CUDA(W.AV.alloc(size_t(n) * kcap));
    FCG_CUDA(W.X.alloc(size_t(n) * R));
    FCG_CUDA(W.tmp.alloc(size_t(n) * std::min(kmax, 2 * R)));
    FCG_CUDA(W.hd.alloc(n));
    FCG_CUDA(W.part.alloc(size_t(W.row_blocks) * kcap * R));
    FCG_CUDA(W.rn_part.alloc(size_t(W.res_blocks) * R));
    W.ngroups = (kcap + 31) / 32;
    FCG_CUDA(W.counters.alloc(size_t(W.ngroups) + 1));
    FCG_CUDA(cudaMemsetAsync(W.counters.p, 0, sizeof(unsigned) * (W.ngroups + 1), ctx->stream));
    const size_t out_cap = size_t(R) + size_t(kcap) * R + 16;
    const size_t up_cap = size_t(4) * (size_t(kcap) * 2 * R + size_t(R) * R + 64);
    FCG_CUDA(W.d_out.alloc(out_cap));
    FCG_CUDA(W.h_out.alloc(out_cap));
    FCG_CUDA(W.d_up.alloc(up_cap));
    FCG_CUDA(W.h_up.alloc(up_cap));
    if (precond) {
      std::vector<double> hd(n);
      int rc = fcg_diagonal(ctx, -1, hd.data());
      if (rc) return rc;
      FCG_CUDA(cudaMemcpyAsync(W.hd.p, hd.data(), sizeof(double) * n, cudaMemcpyHostToDevice, ctx->stream));
      FCG_CUDA(cudaStreamSynchronize(ctx->stream));  // hd is a local vector
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
        std::vector<double> G0(W.h_out.p, W.h_out.p + size_t(R) * R);
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
        const double* C = W.h_out.p;
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
        const size_t ritz_smem = sizeof(double) * (size_t(nv) * R + R);
#define FCG_RITZ_LAUNCH unsigned(W.res_blocks), kDavThreads, ritz_smem, ctx->stream
        FCG_WIDTH_SWITCH(R, ritz_residual_kernel, FCG_RITZ_LAUNCH, W.V.p, W.AV.p, n, nv, dY, dth, W.hd.p, R, n, W.X.p,
                         W.V.p + n * nv, precond, W.rn_part.p, W.d_out.p, W.counters.p + W.ngroups)
#undef FCG_RITZ_LAUNCH
        FCG_CUDA(cudaGetLastError());
        if ((rc = W.gram(W.V.p, nv + R, W.V.p + n * nv, R, W.d_out.p + R))) return rc;
        if ((rc = W.enqueue_fetch(size_t(R) + size_t(nv + R) * R))) return rc;
        st = kResWait;
        *act = Act::kWait;
        return FCG_OK;
      }
      case kResWait: {
        double rmax = 0.0;
        for (int j = 0; j < R; ++j) {
          rn[j] = std::sqrt(W.h_out.p[j]);
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
          FCG_CUDA(cudaMemcpyAsync(W.V.p, W.X.p, sizeof(double) * n * R, cudaMemcpyDeviceToDevice, ctx->stream));
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
        std::vector<double> G0(W.h_out.p, W.h_out.p + size_t(R) * R);
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
        FCG_CUDA(cudaMemcpyAsync(vectors, W.X.p, sizeof(double) * n * R, cudaMemcpyDeviceToHost, ctx->stream));
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
  const double* Gall = W.h_out.p + R;  // [V T]^T T, (nv + R) x R
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
    const unsigned g = unsigned((n + 255) / 256);
    update_kernel<<<g, 256, 0, ctx->stream>>>(W.V.p, n, nv, dQ, q, W.tmp.p, n, n);
    FCG_CUDA(cudaGetLastError());
    FCG_CUDA(cudaMemcpyAsync(W.V.p, W.tmp.p, sizeof(double) * n * q, cudaMemcpyDeviceToDevice, ctx->stream));
    update_kernel<<<g, 256, 0, ctx->stream>>>(W.AV.p, n, nv, dQ, q, W.tmp.p, n, n);
    FCG_CUDA(cudaGetLastError());
    FCG_CUDA(cudaMemcpyAsync(W.AV.p, W.tmp.p, sizeof(double) * n * q, cudaMemcpyDeviceToDevice, ctx->stream));
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
  for (int q = 0; q < nt; ++q) {
    const int src = nv_old + sel[q], dst = nv + q;
    if (src != dst)
      FCG_CUDA(cudaMemcpyAsync(W.V.p + n * dst, W.V.p + n * src, sizeof(double) * n, cudaMemcpyDeviceToDevice,
                               ctx->stream));
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

// Drive the problems to completion on the leader's stream: every round runs each ready
// problem until it needs the device; then either one wait for the stream serves all problems
// that queued work, or -- when every unfinished problem asks for its sigma -- the sigma builds
// run (one asynchronous launch for a single problem, one grouped launch per precision for
// several), and the round repeats.
int run_lockstep(std::vector<std::unique_ptr<DavidsonRun>>& runs, fcg_ctx* leader) {
  fcg_ctx* ctx = leader;
  enum { kReady, kWaiting, kSigma, kDone };
  const int P = int(runs.size());
  std::vector<int> state(P, kReady);
  int active = P;
  while (active > 0) {
    for (int q = 0; q < P; ++q) {
      if (state[q] != kReady) continue;
      Act a = Act::kDone;
      const int rc = runs[q]->step(&a);
      if (rc) {
        if (runs[q]->ctx != leader) leader->err = runs[q]->ctx->err + " (problem " + std::to_string(q) + ")";
        return rc;
      }
      state[q] = a == Act::kWait ? kWaiting : a == Act::kSigma ? kSigma : kDone;
      if (a == Act::kDone) --active;
    }
    bool waiting = false;
    for (int q = 0; q < P; ++q) waiting = waiting || state[q] == kWaiting;
    if (waiting) {
      FCG_CUDA(cudaStreamSynchronize(ctx->stream));
      for (int q = 0; q < P; ++q)
        if (state[q] == kWaiting) {
          runs[q]->W.after_wait();
          state[q] = kReady;
        }
      continue;
    }
    if (P == 1) {
      if (state[0] == kSigma) {
        DavidsonRun& r = *runs[0];
        const int64_t n = r.W.n;
        const int rc = sigma_closed_device_async(r.ctx, r.sig_m, r.W.V.p + n * r.sig_col, r.W.AV.p + n * r.sig_col,
                                                 r.sig_prec);
        if (rc) return rc;
        state[0] = kReady;
      }
      continue;
    }
    for (int p : {FCG_FP32, FCG_FP64}) {
      std::vector<fcg_ctx*> cs;
      std::vector<int> Rs, who;
      std::vector<const double*> dc;
      std::vector<double*> ds;
      for (int q = 0; q < P; ++q) {
        DavidsonRun& r = *runs[q];
        if (state[q] != kSigma || r.sig_prec != p) continue;
        const int64_t n = r.W.n;
        cs.push_back(r.ctx);
        Rs.push_back(r.sig_m);
        dc.push_back(r.W.V.p + n * r.sig_col);
        ds.push_back(r.W.AV.p + n * r.sig_col);
        who.push_back(q);
      }
      if (cs.empty()) continue;
      const int rc = fcg_sigma_closed_grouped(int(cs.size()), cs.data(), Rs.data(), dc.data(), ds.data(), p);
      if (rc) {
        if (cs[0] != leader) leader->err = cs[0]->err;
        return rc;
      }
      for (int q : who) {
        runs[q]->W.after_wait();
        state[q] = kReady;
      }
    }
  }
  return FCG_OK;
}

}  // namespace

extern "C" int fcg_davidson(fcg_ctx* ctx, int R, const double* v0, int max_iter, int max_ss_vecs, double tol,
                            double lindep, int precision, int precond, double* energies, double* vectors,
                            double* residuals, int* iters) {
  if (!ctx) return FCG_EINVAL;
  FCG_CUDA(cudaSetDevice(ctx->device));
  std::vector<std::unique_ptr<DavidsonRun>> runs;
  runs.emplace_back(new DavidsonRun());
  const int rc = runs[0]->init(ctx, R, v0, max_iter, max_ss_vecs, tol, lindep, precision, precond, energies, vectors,
                               residuals, iters);
  if (rc) return rc;
  return run_lockstep(runs, ctx);
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
  // every problem's work goes to the leader's stream while the group is solved
  std::vector<cudaStream_t> saved(n);
  for (int q = 0; q < n; ++q) {
    saved[q] = ctxs[q]->stream;
    ctxs[q]->stream = ctx->stream;
  }
  std::vector<std::unique_ptr<DavidsonRun>> runs;
  int rc = FCG_OK;
  for (int q = 0; q < n && rc == FCG_OK; ++q) {
    runs.emplace_back(new DavidsonRun());
    rc = runs[q]->init(ctxs[q], R[q], v0[q], max_iter, max_ss_vecs, tol, lindep, precision, precond, energies[q],
                       vectors[q], residuals[q], &iters[q]);
    if (rc && q > 0) ctx->err = ctxs[q]->err + " (problem " + std::to_string(q) + ")";
  }
  if (rc == FCG_OK) rc = run_lockstep(runs, ctx);
  cudaStreamSynchronize(ctx->stream);  // nothing of the group in flight when the streams change back
  for (int q = 0; q < n; ++q) ctxs[q]->stream = saved[q];
  return rc;
}

// ---- serving: continuous batching of Davidson solves ---------------------------------------
//
// A server owns one stream and a scheduler thread.  Callers prepare a context per request
// (fcg_set_ops, fcg_set_terms, fcg_state_set -- in their own threads) and submit it with a
// guess; the scheduler admits requests while slots and the memory budget allow, and runs all
// admitted solves in lockstep rounds as fcg_davidson_grouped does: every round advances each
// solve to its next need of the device, then serves all of them with one wait for the stream
// or one grouped sigma launch per precision.  Solves that finish leave after the round,
// queued requests join at the next, so a request's work overlaps with whatever is in flight.
// A solve's result is the same as fcg_davidson's on its own (the grouped sigma adds each
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
  int state = 0;  // 0 ready, 1 waiting, 2 sigma, 3 failed, 4 done
  int rc = 0;
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
  std::vector<Slot> active;
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
        const int rc = sl.run->init(t->ctx, t->R, t->v0.data(), t->max_iter, t->max_ss_vecs, t->tol, t->lindep,
                                    t->precision, t->precond, t->energies.data(), t->vectors.data(),
                                    t->residuals.data(), &t->iters);
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
    // one round over the admitted solves
    for (size_t q = 0; q < active.size(); ++q) {
      Slot& sl = active[q];
      while (sl.state == 0) {
        Act a = Act::kDone;
        const int rc = sl.run->step(&a);
        if (rc) {
          sl.rc = rc;
          sl.state = 3;
          break;
        }
        sl.state = a == Act::kWait ? 1 : a == Act::kSigma ? 2 : 4;
      }
    }
    bool waiting = false;
    for (auto& sl : active) waiting = waiting || sl.state == 1;
    int rc_round = FCG_OK;
    if (waiting) {
      rc_round = cudaStreamSynchronize(stream) == cudaSuccess ? FCG_OK : FCG_ECUDA;
      for (auto& sl : active)
        if (sl.state == 1) {
          sl.run->W.after_wait();
          sl.state = 0;
        }
    } else {
      for (int p : {FCG_FP32, FCG_FP64}) {
        std::vector<fcg_ctx*> cs;
        std::vector<int> Rs;
        std::vector<const double*> dc;
        std::vector<double*> ds;
        std::vector<Slot*> who;
        for (auto& sl : active) {
          DavidsonRun& r = *sl.run;
          if (sl.state != 2 || r.sig_prec != p) continue;
          const int64_t n = r.W.n;
          cs.push_back(r.ctx);
          Rs.push_back(r.sig_m);
          dc.push_back(r.W.V.p + n * r.sig_col);
          ds.push_back(r.W.AV.p + n * r.sig_col);
          who.push_back(&sl);
        }
        if (cs.empty()) continue;
        const int rc = fcg_sigma_closed_grouped(int(cs.size()), cs.data(), Rs.data(), dc.data(), ds.data(), p);
        for (Slot* sl : who) {
          if (rc) {
            sl->state = 3;
            sl->rc = rc;
            sl->t->ctx->err = cs[0]->err;
          } else {
            sl->run->W.after_wait();
            sl->state = 0;
          }
        }
      }
    }
    // retire finished and failed solves
    std::unique_lock<std::mutex> lk(mu);
    std::vector<Slot> keep;
    for (size_t q = 0; q < active.size(); ++q) {
      Slot& sl = active[q];
      if (sl.state == 4) {
        finish(sl, FCG_OK);
      } else if (sl.state == 3 || rc_round != FCG_OK) {
        cudaStreamSynchronize(stream);
        if (sl.state != 3) sl.t->ctx->err = "serving: the shared stream failed";
        finish(sl, sl.state == 3 ? sl.rc : rc_round);
      } else {
        keep.push_back(std::move(sl));
      }
    }
    active.swap(keep);
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

int fcg_submit(fcg_server* s, fcg_ctx* ctx, int R, const double* v0, int max_iter, int max_ss_vecs, double tol,
               double lindep, int precision, int precond, int64_t* ticket) {
  if (!s || !ctx || !v0 || !ticket || R < 1 || R > kMaxB) return FCG_EINVAL;
  if (!ctx->have_state || ctx->n_cfg < R) return FCG_ESTATE;
  if (ctx->device != s->device) return FCG_EINVAL;
  auto t = std::make_shared<fcg_server::Ticket>();
  const int64_t n = ctx->n_cfg;
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
