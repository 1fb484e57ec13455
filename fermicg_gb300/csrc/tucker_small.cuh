// Small dense tensor algebra for Tucker tensors, written once for the host and the device:
// the mode Gram matrices and mode products of a column-major core, and Jacobi eigensolvers
// for symmetric matrices up to kTuckMaxDim -- serial versions, and cooperative versions in
// which the threads of one CTA share one small problem.  These carry the compressions of the block-sparse Tucker first-order
// space: HOSVD truncation (tucker_decompose, src/hosvd.jl:450-545), the left singular
// vectors of stacked factors (nonorth_add, src/hosvd.jl:83-156) and of the pre-contracted
// local operators of 3- and 4-body terms (src/tucker_form_sigma_block_expand.jl:325-390).
#pragma once

#include <cmath>
#include <cstdint>

#ifdef __CUDACC__
#define FCG_HD __host__ __device__
#else
#define FCG_HD
#endif

namespace fcg_tucker {

constexpr int kTuckMaxModes = 8;
constexpr int kTuckMaxDim = 64;

// elements of a column-major tensor of the given dims
FCG_HD inline int64_t tensor_len(const int32_t* dims, int n) {
  int64_t s = 1;
  for (int i = 0; i < n; ++i) s *= dims[i];
  return s;
}

// G[i + d*j] (+)= sum over all other indices of A[.., i, ..] * A[.., j, ..] for mode m
// (A column-major with dims[0] fastest; d = dims[m]).  accumulate = 0 overwrites G.
FCG_HD inline void mode_gram(const double* A, const int32_t* dims, int n, int m, double* G, int accumulate) {
  const int d = dims[m];
  int64_t inner = 1, outer = 1;
  for (int i = 0; i < m; ++i) inner *= dims[i];
  for (int i = m + 1; i < n; ++i) outer *= dims[i];
  if (!accumulate)
    for (int k = 0; k < d * d; ++k) G[k] = 0.0;
  for (int j = 0; j < d; ++j)
    for (int i = 0; i <= j; ++i) {
      double s = 0.0;
      for (int64_t o = 0; o < outer; ++o) {
        const double* a = A + o * inner * d;
        for (int64_t q = 0; q < inner; ++q) s += a[q + inner * i] * a[q + inner * j];
      }
      G[i + d * j] += s;
      if (i != j) G[j + d * i] += s;
    }
}

// B = A x_m M^T: B[.., k, ..] = sum_i M[i + ld*k] A[.., i, ..] for k < knew (M is dims[m] x knew
// with leading dimension ld).  B has dims[m] replaced by knew; A and B must not overlap.
FCG_HD inline void mode_product_t(const double* A, const int32_t* dims, int n, int m, const double* M, int ld,
                                  int knew, double* B) {
  const int d = dims[m];
  int64_t inner = 1, outer = 1;
  for (int i = 0; i < m; ++i) inner *= dims[i];
  for (int i = m + 1; i < n; ++i) outer *= dims[i];
  for (int64_t o = 0; o < outer; ++o) {
    const double* a = A + o * inner * d;
    double* b = B + o * inner * knew;
    for (int k = 0; k < knew; ++k)
      for (int64_t q = 0; q < inner; ++q) {
        double s = 0.0;
        for (int i = 0; i < d; ++i) s += M[i + int64_t(ld) * k] * a[q + inner * i];
        b[q + inner * k] = s;
      }
  }
}

// Eigen-decomposition of the symmetric n x n matrix A (column-major, overwritten) by cyclic
// Jacobi rotations; eigenvalues to w and eigenvectors to the columns of V (n x n), both in
// descending order of eigenvalue.  n <= kTuckMaxDim.
FCG_HD inline void jacobi_eigh_desc(int n, double* A, double* w, double* V) {
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < n; ++i) V[i + n * j] = (i == j) ? 1.0 : 0.0;
  for (int sweep = 0; sweep < 60; ++sweep) {
    double off = 0.0, tot = 0.0;
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i) {
        const double a = A[i + n * j];
        tot += a * a;
        if (i != j) off += a * a;
      }
    if (!(off > 1e-26 * tot)) break;
    for (int p = 0; p < n - 1; ++p)
      for (int q = p + 1; q < n; ++q) {
        const double apq = A[p + n * q];
        if (fabs(apq) < 1e-300) continue;
        const double app = A[p + n * p], aqq = A[q + n * q];
        const double tau = (aqq - app) / (2.0 * apq);
        const double t = (tau >= 0 ? 1.0 : -1.0) / (fabs(tau) + sqrt(1.0 + tau * tau));
        const double c = 1.0 / sqrt(1.0 + t * t), s = t * c;
        for (int r = 0; r < n; ++r) {
          const double arp = A[r + n * p], arq = A[r + n * q];
          A[r + n * p] = c * arp - s * arq;
          A[r + n * q] = s * arp + c * arq;
        }
        for (int r = 0; r < n; ++r) {
          const double apr = A[p + n * r], aqr = A[q + n * r];
          A[p + n * r] = c * apr - s * aqr;
          A[q + n * r] = s * apr + c * aqr;
        }
        for (int r = 0; r < n; ++r) {
          const double vrp = V[r + n * p], vrq = V[r + n * q];
          V[r + n * p] = c * vrp - s * vrq;
          V[r + n * q] = s * vrp + c * vrq;
        }
      }
  }
  for (int i = 0; i < n; ++i) w[i] = A[i + n * i];
  // selection sort, descending (n is small); columns of V follow
  for (int i = 0; i < n; ++i) {
    int best = i;
    for (int j = i + 1; j < n; ++j)
      if (w[j] > w[best]) best = j;
    if (best != i) {
      const double tw = w[i];
      w[i] = w[best];
      w[best] = tw;
      for (int r = 0; r < n; ++r) {
        const double tv = V[r + n * i];
        V[r + n * i] = V[r + n * best];
        V[r + n * best] = tv;
      }
    }
  }
}

// C (m x k) = A (m x r) B (r x k), all column-major with leading dimensions m, r, m
FCG_HD inline void matmul(const double* A, const double* B, int m, int r, int k, double* C) {
  for (int j = 0; j < k; ++j)
    for (int i = 0; i < m; ++i) {
      double s = 0.0;
      for (int t = 0; t < r; ++t) s += A[i + int64_t(m) * t] * B[t + int64_t(r) * j];
      C[i + int64_t(m) * j] = s;
    }
}

// ---- cooperative versions: every thread of a CTA calls them with its index tid and the thread
// count nt; each ends with a barrier.  On the host (nt = 1) they run serially.
#if defined(__CUDA_ARCH__)
#define FCG_SYNC() __syncthreads()
#else
#define FCG_SYNC() ((void)0)
#endif

// G (d x d, d = dims[m]) (+)= the mode-m Gram matrix of A; pairs (i <= j) spread over threads
FCG_HD inline void coop_mode_gram(const double* A, const int32_t* dims, int n, int m, double* G, int accumulate,
                                  int tid, int nt) {
  const int d = dims[m];
  int64_t inner = 1, outer = 1;
  for (int i = 0; i < m; ++i) inner *= dims[i];
  for (int i = m + 1; i < n; ++i) outer *= dims[i];
  const int npairs = d * (d + 1) / 2;
  for (int p = tid; p < npairs; p += nt) {
    int j = int((sqrt(8.0 * p + 1.0) - 1.0) * 0.5);
    while (j * (j + 1) / 2 > p) --j;
    while ((j + 1) * (j + 2) / 2 <= p) ++j;
    const int i = p - j * (j + 1) / 2;
    double s = 0.0;
    for (int64_t o = 0; o < outer; ++o) {
      const double* a = A + o * inner * d;
      for (int64_t q = 0; q < inner; ++q) s += a[q + inner * i] * a[q + inner * j];
    }
    if (accumulate) {
      G[i + d * j] += s;
      if (i != j) G[j + d * i] += s;
    } else {
      G[i + d * j] = s;
      G[j + d * i] = s;
    }
  }
  FCG_SYNC();
}

// B = A x_m M^T (see mode_product_t), output elements spread over threads
FCG_HD inline void coop_mode_product_t(const double* A, const int32_t* dims, int n, int m, const double* M, int ld,
                                       int knew, double* B, int tid, int nt) {
  const int d = dims[m];
  int64_t inner = 1, outer = 1;
  for (int i = 0; i < m; ++i) inner *= dims[i];
  for (int i = m + 1; i < n; ++i) outer *= dims[i];
  const int64_t total = outer * knew * inner;
  for (int64_t e = tid; e < total; e += nt) {
    const int64_t q = e % inner;
    const int64_t k = (e / inner) % knew;
    const int64_t o = e / (inner * knew);
    const double* a = A + o * inner * d + q;
    double s = 0.0;
    for (int i = 0; i < d; ++i) s += M[i + int64_t(ld) * k] * a[inner * i];
    B[o * inner * knew + q + inner * k] = s;
  }
  FCG_SYNC();
}

// the pair of round r, slot k of a round-robin over np1 players (np1 even): player 0 stays,
// the others rotate; p < q on return
FCG_HD inline int rr_player(int np1, int r, int slot) { return slot == 0 ? 0 : ((slot - 1 + r) % (np1 - 1)) + 1; }

FCG_HD inline void rr_pair(int np1, int r, int k, int* p, int* q) {
  int a = rr_player(np1, r, k), b = rr_player(np1, r, np1 - 1 - k);
  if (a > b) {
    const int t = a;
    a = b;
    b = t;
  }
  *p = a;
  *q = b;
}

// Eigen-decomposition of the symmetric n x n matrix A (column-major, overwritten) by parallel
// two-sided Jacobi: each round rotates n/2 disjoint index pairs (round-robin order, all
// rotations of a round computed from the matrix at its start).  On return w holds the
// eigenvalues and perm their order (perm[0] the largest); the eigenvector of w[perm[j]] is
// column perm[j] of V.  Scratch: cs (n + 1 doubles), red (2 doubles).
FCG_HD inline void coop_jacobi_eigh(int n, double* A, double* w, double* V, int* perm, double* cs, double* red, int tid,
                                    int nt) {
  for (int e = tid; e < n * n; e += nt) V[e] = (e % n == e / n) ? 1.0 : 0.0;
  const int np1 = n + (n & 1), npairs = np1 / 2;
  FCG_SYNC();
  for (int sweep = 0; sweep < 60 && n > 1; ++sweep) {
    if (tid == 0) {
      double off = 0.0, tot = 0.0;
      for (int j = 0; j < n; ++j)
        for (int i = 0; i < n; ++i) {
          const double a = A[i + n * j];
          tot += a * a;
          if (i != j) off += a * a;
        }
      red[0] = (off > 1e-26 * tot) ? 1.0 : 0.0;
    }
    FCG_SYNC();
    const bool go = red[0] != 0.0;
    FCG_SYNC();
    if (!go) break;
    for (int r = 0; r < np1 - 1; ++r) {
      for (int k = tid; k < npairs; k += nt) {
        int p, q;
        rr_pair(np1, r, k, &p, &q);
        double c = 1.0, s = 0.0;
        if (q < n) {
          const double apq = A[p + n * q];
          if (fabs(apq) >= 1e-300) {
            const double app = A[p + n * p], aqq = A[q + n * q];
            const double tau = (aqq - app) / (2.0 * apq);
            const double t = (tau >= 0 ? 1.0 : -1.0) / (fabs(tau) + sqrt(1.0 + tau * tau));
            c = 1.0 / sqrt(1.0 + t * t);
            s = t * c;
          }
        }
        cs[2 * k] = c;
        cs[2 * k + 1] = s;
      }
      FCG_SYNC();
      for (int e = tid; e < npairs * n; e += nt) {  // columns p, q of A and V
        const int k = e / n, row = e % n;
        int p, q;
        rr_pair(np1, r, k, &p, &q);
        if (q >= n) continue;
        const double c = cs[2 * k], s = cs[2 * k + 1];
        const double arp = A[row + n * p], arq = A[row + n * q];
        A[row + n * p] = c * arp - s * arq;
        A[row + n * q] = s * arp + c * arq;
        const double vrp = V[row + n * p], vrq = V[row + n * q];
        V[row + n * p] = c * vrp - s * vrq;
        V[row + n * q] = s * vrp + c * vrq;
      }
      FCG_SYNC();
      for (int e = tid; e < npairs * n; e += nt) {  // rows p, q of A
        const int k = e / n, col = e % n;
        int p, q;
        rr_pair(np1, r, k, &p, &q);
        if (q >= n) continue;
        const double c = cs[2 * k], s = cs[2 * k + 1];
        const double apr = A[p + n * col], aqr = A[q + n * col];
        A[p + n * col] = c * apr - s * aqr;
        A[q + n * col] = s * apr + c * aqr;
      }
      FCG_SYNC();
    }
  }
  if (tid == 0) {
    for (int i = 0; i < n; ++i) {
      w[i] = A[i + n * i];
      perm[i] = i;
    }
    for (int i = 0; i < n; ++i) {  // selection sort of perm by decreasing eigenvalue
      int best = i;
      for (int j = i + 1; j < n; ++j)
        if (w[perm[j]] > w[perm[best]]) best = j;
      const int tp = perm[i];
      perm[i] = perm[best];
      perm[best] = tp;
    }
  }
  FCG_SYNC();
}

}  // namespace fcg_tucker
