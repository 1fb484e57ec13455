// Block Davidson eigensolver on the device, driving the closed sigma build.
//
// Replaces the BlockDavidson.jl solve behind tps_ci_davidson (src/tpsci_outer.jl:364-454):
// Davidson(Hmap; v0, max_iter, max_ss_vecs, nroots=R, tol, lindep_thresh) with
// eigs(davidson; Adiag = compute_diagonal(...)).  BlockDavidson.jl itself is not in
// the reference tree; this is a standard block Davidson written from its call sites.
//
// Everything of size n stays on the GPU in float64: the subspace V and H V (column-major,
// one column per vector), Gram matrices V^T W, Ritz vectors X = V Y and H X = (HV) Y,
// residuals r = HX - X theta, the diagonal preconditioner t = r / (theta - H_dd), and
// classical Gram-Schmidt applied twice.  Only the k x k Rayleigh-Ritz problem (k <=
// max_ss_vecs * R) goes to the host (cyclic Jacobi).
//
// Precision: FCG_FP64 runs every sigma in float64.  FCG_FP32 ("mixed") runs the sigma
// builds in float32 until the residual norms reach max(tol, 1e-5), then restarts from
// the Ritz vectors with float64 sigma builds (the refinement) until tol.
#include <cmath>

#include "fcg_ctx.cuh"

using namespace fcg;

namespace {

// out[i + a*j] = sum_rows A[row + lda*i] * B[row + ldb*j]  (out zeroed by the caller)
__global__ void gram_kernel(const double* __restrict__ A, int64_t lda, int a, const double* __restrict__ B,
                            int64_t ldb, int b, int64_t n, double* __restrict__ out) {
  extern __shared__ double red[];
  const int64_t rows_per = (n + gridDim.x - 1) / gridDim.x;
  const int64_t r0 = int64_t(blockIdx.x) * rows_per;
  const int64_t r1 = (r0 + rows_per < n) ? r0 + rows_per : n;
  for (int p = 0; p < a * b; ++p) {
    const int i = p % a, j = p / a;
    double s = 0.0;
    for (int64_t r = r0 + threadIdx.x; r < r1; r += blockDim.x) s = fma(A[r + lda * i], B[r + ldb * j], s);
    // block reduction
    for (int off = 16; off > 0; off >>= 1) s += __shfl_down_sync(0xffffffffu, s, off);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
      double t = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
      for (int off = 16; off > 0; off >>= 1) t += __shfl_down_sync(0xffffffffu, t, off);
      if (threadIdx.x == 0) atomicAdd(out + p, t);
    }
    __syncthreads();
  }
}

// C[:, j] (+)= sum_i A[:, i] * Y[i + a*j]   (ldc columns); beta = 0 overwrites, 1 accumulates, -1 subtracts
__global__ void update_kernel(const double* __restrict__ A, int64_t lda, int a, const double* __restrict__ Y, int b,
                              double* __restrict__ C, int64_t ldc, int64_t n, int mode) {
  const int64_t r = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (r >= n) return;
  for (int j = 0; j < b; ++j) {
    double s = 0.0;
    for (int i = 0; i < a; ++i) s = fma(A[r + lda * i], Y[i + a * j], s);
    double* c = C + r + ldc * j;
    if (mode == 0)
      *c = s;
    else if (mode == 1)
      *c += s;
    else
      *c -= s;
  }
}

// residual r_j = HX_j - theta_j X_j, its squared norm, and the preconditioned
// correction t_j = r_j / (theta_j - Hd) (denominator kept away from zero)
__global__ void residual_kernel(const double* __restrict__ X, const double* __restrict__ HX,
                                const double* __restrict__ theta, const double* __restrict__ hd, int R, int64_t n,
                                double* __restrict__ T, double* __restrict__ rnorm2, int precond) {
  const int64_t r = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  for (int j = 0; j < R; ++j) {
    double res = 0.0;
    if (r < n) {
      res = HX[r + n * j] - theta[j] * X[r + n * j];
      double d = precond ? theta[j] - hd[r] : 1.0;
      if (fabs(d) < 1e-6) d = d < 0 ? -1e-6 : 1e-6;
      T[r + n * j] = res / d;
    }
    double s = res * res;
    for (int off = 16; off > 0; off >>= 1) s += __shfl_down_sync(0xffffffffu, s, off);
    if ((threadIdx.x & 31) == 0) atomicAdd(rnorm2 + j, s);
  }
}

__global__ void scale_cols_kernel(double* __restrict__ A, int64_t lda, const double* __restrict__ L, int b,
                                  int64_t n, double* __restrict__ tmp) {
  // A[:, 0..b) <- A[:, 0..b) * L  (L upper-triangular b x b, column-major); tmp: n x b scratch
  const int64_t r = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (r >= n) return;
  for (int j = 0; j < b; ++j) {
    double s = 0.0;
    for (int i = 0; i <= j; ++i) s = fma(A[r + lda * i], L[i + b * j], s);
    tmp[r + n * j] = s;
  }
  for (int j = 0; j < b; ++j) A[r + lda * j] = tmp[r + n * j];
}

// cyclic Jacobi eigen-decomposition of a symmetric k x k matrix (column-major, in place);
// eigenvalues ascending in w, eigenvectors in the columns of Vv
void jacobi_eigh(int k, std::vector<double>& A, std::vector<double>& w, std::vector<double>& Vv) {
  Vv.assign(size_t(k) * k, 0.0);
  for (int i = 0; i < k; ++i) Vv[i + k * i] = 1.0;
  for (int sweep = 0; sweep < 100; ++sweep) {
    double off = 0.0, tot = 0.0;
    for (int j = 0; j < k; ++j)
      for (int i = 0; i < k; ++i) {
        tot += A[i + k * j] * A[i + k * j];
        if (i != j) off += A[i + k * j] * A[i + k * j];
      }
    if (off <= 1e-30 * std::max(tot, 1e-300)) break;
    for (int p = 0; p < k - 1; ++p)
      for (int q = p + 1; q < k; ++q) {
        const double apq = A[p + k * q];
        if (std::fabs(apq) < 1e-300) continue;
        const double app = A[p + k * p], aqq = A[q + k * q];
        const double tau = (aqq - app) / (2.0 * apq);
        const double t = (tau >= 0 ? 1.0 : -1.0) / (std::fabs(tau) + std::sqrt(1.0 + tau * tau));
        const double c = 1.0 / std::sqrt(1.0 + t * t), s = t * c;
        for (int r = 0; r < k; ++r) {  // columns p, q
          const double arp = A[r + k * p], arq = A[r + k * q];
          A[r + k * p] = c * arp - s * arq;
          A[r + k * q] = s * arp + c * arq;
        }
        for (int r = 0; r < k; ++r) {  // rows p, q
          const double apr = A[p + k * r], aqr = A[q + k * r];
          A[p + k * r] = c * apr - s * aqr;
          A[q + k * r] = s * apr + c * aqr;
        }
        for (int r = 0; r < k; ++r) {
          const double vrp = Vv[r + k * p], vrq = Vv[r + k * q];
          Vv[r + k * p] = c * vrp - s * vrq;
          Vv[r + k * q] = s * vrp + c * vrq;
        }
      }
  }
  std::vector<int> idx(k);
  for (int i = 0; i < k; ++i) idx[i] = i;
  std::sort(idx.begin(), idx.end(), [&](int a, int b) { return A[a + k * a] < A[b + k * b]; });
  std::vector<double> Vs(size_t(k) * k);
  w.assign(k, 0.0);
  for (int j = 0; j < k; ++j) {
    w[j] = A[idx[j] + k * idx[j]];
    for (int i = 0; i < k; ++i) Vs[i + k * j] = Vv[i + k * idx[j]];
  }
  Vv.swap(Vs);
}

}  // namespace

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

namespace {

struct DavidsonWork {
  fcg_ctx* ctx;
  int64_t n;
  int kmax;
  DevBuf<double> V, AV, X, HX, T, tmp, small, theta, hd, rn;
  int gram_grid;

  int gram(const double* A, int a, const double* B, int b, std::vector<double>& out) {
    fcg_ctx* ctx = this->ctx;
    FCG_CUDA(cudaMemsetAsync(small.p, 0, sizeof(double) * a * b, ctx->stream));
    gram_kernel<<<gram_grid, 256, 8 * sizeof(double), ctx->stream>>>(A, n, a, B, n, b, n, small.p);
    FCG_CUDA(cudaGetLastError());
    out.resize(size_t(a) * b);
    FCG_CUDA(cudaMemcpyAsync(out.data(), small.p, sizeof(double) * a * b, cudaMemcpyDeviceToHost, ctx->stream));
    FCG_CUDA(cudaStreamSynchronize(ctx->stream));
    return FCG_OK;
  }
  // C (+/-)= A * Y with Y a host a x b matrix
  int update(const double* A, int a, const std::vector<double>& Y, int b, double* C, int mode) {
    fcg_ctx* ctx = this->ctx;
    FCG_CUDA(cudaMemcpyAsync(small.p, Y.data(), sizeof(double) * a * b, cudaMemcpyHostToDevice, ctx->stream));
    update_kernel<<<unsigned((n + 255) / 256), 256, 0, ctx->stream>>>(A, n, a, small.p, b, C, n, n, mode);
    FCG_CUDA(cudaGetLastError());
    // no wait: a pageable host-to-device copy has staged Y when it returns, and every later
    // use of C runs behind this kernel on the same stream
    return FCG_OK;
  }
};

// Orthonormalise columns [0, b) of T against V[:, 0..nv) and among themselves; the kept
// columns are packed to the front and their count returned in *kept.  Every column is
// first scaled to unit norm, then projected out of V (classical Gram-Schmidt, twice); a
// direction is dropped when less than `drop` of it survives the projection (it lies in
// the subspace already, up to rounding).  The survivors are orthonormalised by Cholesky
// QR, twice.
int orthonormalize_block(DavidsonWork& W, double* Tp, int b, const double* Vp, int nv, double drop, int* kept) {
  fcg_ctx* ctx = W.ctx;
  std::vector<double> S;
  int rc;
  auto scale_to_unit = [&](int m, std::vector<int>& keep, double floor2) -> int {
    if ((rc = W.gram(Tp, m, Tp, m, S))) return rc;
    keep.clear();
    std::vector<double> D(size_t(m) * m, 0.0);
    for (int j = 0; j < m; ++j) {
      const double n2 = S[j + m * j];
      if (std::isfinite(n2) && n2 > floor2) {
        D[j + m * j] = 1.0 / std::sqrt(n2);
        keep.push_back(j);
      }
    }
    FCG_CUDA(cudaMemcpyAsync(W.small.p, D.data(), sizeof(double) * m * m, cudaMemcpyHostToDevice, ctx->stream));
    scale_cols_kernel<<<unsigned((W.n + 255) / 256), 256, 0, ctx->stream>>>(Tp, W.n, W.small.p, m, W.n, W.tmp.p);
    FCG_CUDA(cudaGetLastError());
    return FCG_OK;
  };
  auto pack = [&](const std::vector<int>& keep) -> int {
    for (size_t q = 0; q < keep.size(); ++q)
      if (int(q) != keep[q])
        FCG_CUDA(cudaMemcpyAsync(Tp + W.n * q, Tp + W.n * keep[q], sizeof(double) * W.n, cudaMemcpyDeviceToDevice,
                                 ctx->stream));
    return FCG_OK;
  };
  std::vector<int> keep;
  if ((rc = scale_to_unit(b, keep, 1e-300))) return rc;
  if ((rc = pack(keep))) return rc;
  int m = int(keep.size());
  if (m > 0 && nv > 0) {
    for (int pass = 0; pass < 2; ++pass) {
      if ((rc = W.gram(Vp, nv, Tp, m, S))) return rc;
      if ((rc = W.update(Vp, nv, S, m, Tp, 2))) return rc;
    }
    // what survived the projection, relative to the unit input
    if ((rc = scale_to_unit(m, keep, drop * drop))) return rc;
    if ((rc = pack(keep))) return rc;
    m = int(keep.size());
  }
  for (int it = 0; it < 2 && m > 0; ++it) {
    if ((rc = W.gram(Tp, m, Tp, m, S))) return rc;
    // Cholesky S = R^T R, stopping at the first column that is dependent on the previous ones
    std::vector<double> Lc(size_t(m) * m, 0.0);
    int good = 0;
    for (int j = 0; j < m; ++j) {
      double d = S[j + m * j];
      for (int p = 0; p < j; ++p) d -= Lc[p + m * j] * Lc[p + m * j];
      if (!(d > drop * drop * S[j + m * j])) break;
      Lc[j + m * j] = std::sqrt(d);
      for (int q = j + 1; q < m; ++q) {
        double v = S[j + m * q];
        for (int p = 0; p < j; ++p) v -= Lc[p + m * j] * Lc[p + m * q];
        Lc[j + m * q] = v / Lc[j + m * j];
      }
      ++good;
    }
    m = good;
    if (m == 0) break;
    std::vector<double> Ri(size_t(m) * m, 0.0);  // inverse of the leading m x m block of R
    for (int j = 0; j < m; ++j) {
      Ri[j + m * j] = 1.0 / Lc[j + m * j];
      for (int i = j - 1; i >= 0; --i) {
        double s2 = 0.0;
        for (int p = i + 1; p <= j; ++p) s2 += Lc[i + m * p] * Ri[p + m * j];
        Ri[i + m * j] = -s2 / Lc[i + m * i];
      }
    }
    FCG_CUDA(cudaMemcpyAsync(W.small.p, Ri.data(), sizeof(double) * m * m, cudaMemcpyHostToDevice, ctx->stream));
    scale_cols_kernel<<<unsigned((W.n + 255) / 256), 256, 0, ctx->stream>>>(Tp, W.n, W.small.p, m, W.n, W.tmp.p);
    FCG_CUDA(cudaGetLastError());
    if (nv > 0) {  // restore orthogonality to V lost in the rescaling
      if ((rc = W.gram(Vp, nv, Tp, m, S))) return rc;
      if ((rc = W.update(Vp, nv, S, m, Tp, 2))) return rc;
    }
  }
  *kept = m;
  return FCG_OK;
}

}  // namespace

extern "C" int fcg_sigma_closed_device(fcg_ctx* ctx, int R, const double* d_c, double* d_sigma, int precision);
extern "C" int fcg_diagonal(fcg_ctx* ctx, int op_id, double* hd);

extern "C" int fcg_davidson(fcg_ctx* ctx, int R, const double* v0, int max_iter, int max_ss_vecs, double tol,
                            double lindep, int precision, int precond, double* energies, double* vectors,
                            double* residuals, int* iters) {
  if (!ctx) return FCG_EINVAL;
  FCG_REQUIRE(ctx->have_state, FCG_ESTATE, "fcg_state_set must come first");
  FCG_REQUIRE(v0 && energies && vectors && residuals && iters, FCG_EINVAL, "null pointer");
  FCG_REQUIRE(R >= 1 && R <= 16 && R <= ctx->n_cfg, FCG_ELIMIT, "R must be in [1, min(16, n_cfg)]");
  FCG_REQUIRE(max_ss_vecs >= 2 && max_iter >= 1 && tol > 0, FCG_EINVAL, "bad Davidson settings");
  FCG_REQUIRE(precision == FCG_FP64 || precision == FCG_FP32, FCG_EINVAL, "unknown precision");
  FCG_CUDA(cudaSetDevice(ctx->device));
  const int64_t n = ctx->n_cfg;
  DavidsonWork W;
  W.ctx = ctx;
  W.n = n;
  W.kmax = int(std::min<int64_t>(int64_t(max_ss_vecs) * R, n));
  W.kmax = std::max(W.kmax, std::min<int>(2 * R, int(n)));
  const int kmax = W.kmax;
  W.gram_grid = int(std::min<int64_t>(304, (n + 255) / 256));
  // room for a full subspace plus one block of new directions (restart keeps nv <= kmax)
  FCG_CUDA(W.V.alloc(size_t(n) * (kmax + R)));
  FCG_CUDA(W.AV.alloc(size_t(n) * (kmax + R)));
  FCG_CUDA(W.X.alloc(size_t(n) * R));
  FCG_CUDA(W.HX.alloc(size_t(n) * R));
  FCG_CUDA(W.T.alloc(size_t(n) * R));
  FCG_CUDA(W.tmp.alloc(size_t(n) * std::max(R, kmax)));
  FCG_CUDA(W.small.alloc(size_t(kmax) * kmax + 16));
  FCG_CUDA(W.theta.alloc(16));
  FCG_CUDA(W.rn.alloc(16));
  FCG_CUDA(W.hd.alloc(n));
  if (precond) {
    std::vector<double> hd(n);
    int rc = fcg_diagonal(ctx, -1, hd.data());
    if (rc) return rc;
    FCG_CUDA(cudaMemcpyAsync(W.hd.p, hd.data(), sizeof(double) * n, cudaMemcpyHostToDevice, ctx->stream));
  }
  int prec = precision;  // current sigma precision
  // a new direction must keep at least this fraction of its norm after projection
  const double drop = std::max(lindep, 1e-8);
  const double switch_tol = std::max(tol, 1e-5);
  // initial block
  FCG_CUDA(cudaMemcpyAsync(W.V.p, v0, sizeof(double) * n * R, cudaMemcpyHostToDevice, ctx->stream));
  int nv = 0, m = 0, rc;
  if ((rc = orthonormalize_block(W, W.V.p, R, nullptr, 0, drop, &m))) return rc;
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
    ctx->err = "initial vectors are linearly dependent (kept " + std::to_string(m) + " of " + std::to_string(R) +
               ", n " + std::to_string(n) + ", squared norms " + std::to_string(nrm_min) + ".." +
               std::to_string(nrm_max) + ", non-finite entries " + std::to_string(nonfinite) + ")";
    return FCG_EINVAL;
  }
  if ((rc = fcg_sigma_closed_device(ctx, R, W.V.p, W.AV.p, prec))) return rc;
  nv = R;
  std::vector<double> Hs, w, Y, th(R), rn(R);
  int it = 0;
  int64_t sigma_calls = 1;
  bool converged = false;
  for (it = 1; it <= max_iter; ++it) {
    // Rayleigh-Ritz
    if ((rc = W.gram(W.V.p, nv, W.AV.p, nv, Hs))) return rc;
    for (int j = 0; j < nv; ++j)
      for (int i = 0; i < j; ++i) {
        double a = 0.5 * (Hs[i + nv * j] + Hs[j + nv * i]);
        Hs[i + nv * j] = Hs[j + nv * i] = a;
      }
    for (double x : Hs)
      if (!std::isfinite(x)) {
        ctx->err = "Davidson: non-finite subspace matrix at iteration " + std::to_string(it) + " (subspace " +
                   std::to_string(nv) + ")";
        return FCG_ECUDA;
      }
    jacobi_eigh(nv, Hs, w, Y);
    Y.resize(size_t(nv) * R);
    for (int j = 0; j < R; ++j) th[j] = w[j];
    if ((rc = W.update(W.V.p, nv, Y, R, W.X.p, 0))) return rc;
    if ((rc = W.update(W.AV.p, nv, Y, R, W.HX.p, 0))) return rc;
    FCG_CUDA(cudaMemcpyAsync(W.theta.p, th.data(), sizeof(double) * R, cudaMemcpyHostToDevice, ctx->stream));
    FCG_CUDA(cudaMemsetAsync(W.rn.p, 0, sizeof(double) * R, ctx->stream));
    residual_kernel<<<unsigned((n + 255) / 256), 256, 0, ctx->stream>>>(W.X.p, W.HX.p, W.theta.p, W.hd.p, R, n,
                                                                        W.T.p, W.rn.p, precond);
    FCG_CUDA(cudaGetLastError());
    FCG_CUDA(cudaMemcpyAsync(rn.data(), W.rn.p, sizeof(double) * R, cudaMemcpyDeviceToHost, ctx->stream));
    FCG_CUDA(cudaStreamSynchronize(ctx->stream));
    double rmax = 0.0;
    for (int j = 0; j < R; ++j) {
      rn[j] = std::sqrt(rn[j]);
      rmax = std::max(rmax, rn[j]);
      if (!std::isfinite(rn[j]) || !std::isfinite(th[j])) {
        ctx->err = "Davidson: non-finite residual or Ritz value at iteration " + std::to_string(it);
        return FCG_ECUDA;
      }
    }
    const bool switching = (prec == FCG_FP32) && rmax < switch_tol;
    if (rmax < tol && prec == FCG_FP64) {
      converged = true;
      break;
    }
    if (switching || nv + R > kmax) {
      // restart from the Ritz vectors (and, when switching precision, rebuild H X in float64)
      FCG_CUDA(cudaMemcpyAsync(W.V.p, W.X.p, sizeof(double) * n * R, cudaMemcpyDeviceToDevice, ctx->stream));
      if (switching) {
        prec = FCG_FP64;
        if ((rc = orthonormalize_block(W, W.V.p, R, nullptr, 0, drop, &m))) return rc;
        if ((rc = fcg_sigma_closed_device(ctx, R, W.V.p, W.AV.p, prec))) return rc;
        ++sigma_calls;
        nv = R;
        continue;
      }
      FCG_CUDA(cudaMemcpyAsync(W.AV.p, W.HX.p, sizeof(double) * n * R, cudaMemcpyDeviceToDevice, ctx->stream));
      nv = R;
    }
    // new directions: preconditioned residuals of the roots not yet converged,
    // orthonormalised against the subspace
    int nt = 0;
    for (int j = 0; j < R; ++j)
      if (rn[j] >= tol || prec == FCG_FP32) {
        FCG_CUDA(cudaMemcpyAsync(W.V.p + n * (nv + nt), W.T.p + n * j, sizeof(double) * n,
                                 cudaMemcpyDeviceToDevice, ctx->stream));
        ++nt;
      }
    if ((rc = orthonormalize_block(W, W.V.p + n * nv, nt, W.V.p, nv, drop, &m))) return rc;
    if (m == 0) {  // the subspace cannot grow: converged as far as lindep allows
      converged = rmax < tol;
      break;
    }
    if ((rc = fcg_sigma_closed_device(ctx, m, W.V.p + n * nv, W.AV.p + n * nv, prec))) return rc;
    ++sigma_calls;
    nv += m;
  }
  for (int j = 0; j < R; ++j) {
    energies[j] = th[j];
    residuals[j] = rn[j];
  }
  FCG_CUDA(cudaMemcpyAsync(vectors, W.X.p, sizeof(double) * n * R, cudaMemcpyDeviceToHost, ctx->stream));
  FCG_CUDA(cudaStreamSynchronize(ctx->stream));
  *iters = std::min(it, max_iter);
  ctx->stats.davidson_sigma_calls = sigma_calls;
  (void)converged;
  return FCG_OK;
}
