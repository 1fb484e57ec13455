// Small dense linear algebra on the host for the Davidson driver: the Rayleigh-Ritz
// eigenproblem of the projected matrix (k <= a few hundred) and the Cholesky factors of the
// Gram matrices of new subspace directions (m <= 16).  Column-major storage throughout.
//
// symeig: Householder reduction to tridiagonal form followed by the implicit QL iteration
// with Wilkinson-type shifts (Bowdler, Martin, Reinsch & Wilkinson, "The QR and QL
// algorithms for symmetric matrices", Numer. Math. 11 (1968); Golub & Van Loan, Matrix
// Computations, sections 8.3.1-8.3.3).  Only the wanted (lowest) eigenvectors are formed,
// by replaying the recorded QL rotations and Householder reflections on unit vectors.
#pragma once

#include <algorithm>
#include <cmath>
#include <limits>
#include <numeric>
#include <vector>

namespace fcg_small {

// Eigen-decomposition of the symmetric k x k matrix A (column-major, leading dimension k;
// only the lower triangle is read, A is overwritten).  On return w holds all k eigenvalues
// in ascending order and the columns of Z (k x nvec) the orthonormal eigenvectors of the
// nvec lowest ones (nvec < 0: all k).  The QL rotations are recorded and replayed on unit
// vectors, so the eigenvectors cost O(k^2) each instead of an O(k^3) accumulation of the
// full eigenvector matrix.  Returns 0 on success, 1 when the QL iteration did not converge
// (non-finite input).
inline int symeig(int k, double* A, std::vector<double>& w, std::vector<double>& Z, int nvec = -1) {
  if (nvec < 0 || nvec > k) nvec = k;
  w.assign(size_t(k), 0.0);
  Z.assign(size_t(k) * nvec, 0.0);
  if (k <= 0) return 0;
  auto a = [&](int i, int j) -> double& { return A[i + size_t(k) * j]; };
  for (int j = 0; j < k; ++j)
    for (int i = 0; i < j; ++i) a(i, j) = a(j, i);  // full symmetric storage
  std::vector<double> v(k), p(k), e(k, 0.0);
  std::vector<double> hv(size_t(k) * k, 0.0), hbeta(k, 0.0);  // Householder vectors and factors
  // 1. Householder: for column j, reflect A[j+1:k, j] onto a multiple of the first unit vector
  //    with H_j = I - beta v v^T acting on rows and columns j+1..k-1; A = Q T Q^T with
  //    Q = H_0 H_1 ... H_{k-3}.
  for (int j = 0; j + 2 < k; ++j) {
    const int len = k - j - 1;
    double tail = 0.0;  // squared norm below the subdiagonal entry
    for (int i = j + 2; i < k; ++i) tail += a(i, j) * a(i, j);
    if (tail == 0.0) continue;  // already tridiagonal in this column
    const double x0 = a(j + 1, j);
    const double alpha = std::sqrt(x0 * x0 + tail);
    const double s = x0 >= 0.0 ? 1.0 : -1.0;
    v[0] = x0 + s * alpha;
    for (int i = 1; i < len; ++i) v[i] = a(j + 1 + i, j);
    const double beta = 2.0 / (v[0] * v[0] + tail);
    // p = beta * A22 v
    for (int i = 0; i < len; ++i) p[i] = 0.0;
    for (int c = 0; c < len; ++c) {
      const double vc = v[c];
      const double* col = &a(j + 1, j + 1 + c);
      for (int i = 0; i < len; ++i) p[i] += col[i] * vc;
    }
    double ptv = 0.0;
    for (int i = 0; i < len; ++i) {
      p[i] *= beta;
      ptv += p[i] * v[i];
    }
    // w = p - (beta / 2)(p^T v) v  (stored in p); A22 -= v w^T + w v^T
    const double kf = 0.5 * beta * ptv;
    for (int i = 0; i < len; ++i) p[i] -= kf * v[i];
    for (int c = 0; c < len; ++c) {
      double* col = &a(j + 1, j + 1 + c);
      const double vc = v[c], wc = p[c];
      for (int i = 0; i < len; ++i) col[i] -= v[i] * wc + p[i] * vc;
    }
    a(j + 1, j) = a(j, j + 1) = -s * alpha;
    for (int i = j + 2; i < k; ++i) a(i, j) = a(j, i) = 0.0;
    std::copy(v.begin(), v.begin() + len, &hv[size_t(k) * j + j + 1]);
    hbeta[j] = beta;
  }
  for (int i = 0; i < k; ++i) w[i] = a(i, i);
  for (int i = 0; i + 1 < k; ++i) e[i] = a(i + 1, i);  // e[i] couples i and i+1; e[k-1] = 0
  // 2. implicit QL on the tridiagonal (w, e); each plane rotation G of columns (i, i+1) is
  //    recorded: the eigenvector matrix of T is G_1 G_2 ... G_last.
  struct Rot {
    int i;
    double c, s;
  };
  std::vector<Rot> rots;
  rots.reserve(size_t(2) * k * k);
  const double eps = std::numeric_limits<double>::epsilon();
  for (int l = 0; l < k; ++l) {
    int iter = 0;
    for (;;) {
      int m = l;
      for (; m + 1 < k; ++m) {
        const double dd = std::fabs(w[m]) + std::fabs(w[m + 1]);
        if (std::fabs(e[m]) <= eps * dd) break;
      }
      if (m == l) break;
      if (++iter > 60) return 1;
      // shift from the leading 2 x 2 block at l
      double g = (w[l + 1] - w[l]) / (2.0 * e[l]);
      double r = std::hypot(g, 1.0);
      g = w[m] - w[l] + e[l] / (g + (g >= 0.0 ? r : -r));
      double s = 1.0, c = 1.0, pp = 0.0;
      bool deflated = false;
      for (int i = m - 1; i >= l; --i) {
        const double f = s * e[i];
        const double b = c * e[i];
        r = std::hypot(f, g);
        e[i + 1] = r;
        if (r == 0.0) {  // underflow: split the matrix here
          w[i + 1] -= pp;
          e[m] = 0.0;
          deflated = true;
          break;
        }
        s = f / r;
        c = g / r;
        g = w[i + 1] - pp;
        r = (w[i] - g) * s + 2.0 * c * b;
        pp = s * r;
        w[i + 1] = g + pp;
        g = c * r - b;
        rots.push_back({i, c, s});
      }
      if (deflated) continue;
      w[l] -= pp;
      e[l] = g;
      e[m] = 0.0;
    }
  }
  for (int i = 0; i < k; ++i)
    if (!std::isfinite(w[i])) return 1;
  // 3. ascending order; eigenvector of sorted position j = Q G_1 ... G_last e_idx[j]
  std::vector<int> idx(k);
  std::iota(idx.begin(), idx.end(), 0);
  std::stable_sort(idx.begin(), idx.end(), [&](int x, int y) { return w[x] < w[y]; });
  std::vector<double> ws(k);
  for (int j = 0; j < k; ++j) ws[j] = w[idx[j]];
  for (int j = 0; j < nvec; ++j) {
    double* u = &Z[size_t(k) * j];
    u[idx[j]] = 1.0;
    for (size_t t = rots.size(); t-- > 0;) {  // G_last first
      const Rot& g = rots[t];
      const double ui = u[g.i], ui1 = u[g.i + 1];
      u[g.i] = g.c * ui + g.s * ui1;
      u[g.i + 1] = g.c * ui1 - g.s * ui;
    }
    for (int h = k - 3; h >= 0; --h) {  // H_{k-3} first
      if (hbeta[h] == 0.0) continue;
      const double* vh = &hv[size_t(k) * h];
      double d = 0.0;
      for (int i = h + 1; i < k; ++i) d += vh[i] * u[i];
      d *= hbeta[h];
      for (int i = h + 1; i < k; ++i) u[i] -= d * vh[i];
    }
  }
  w.swap(ws);
  return 0;
}

// Cholesky G = R^T R of the leading columns of the symmetric m x m matrix G (column-major,
// leading dimension ldg), stopping at the first column j whose pivot falls to
// drop^2 * G[j, j] or below (it depends linearly on the columns before it).  Returns the
// number of columns factored, `good`, and writes R^{-1} (good x good, upper triangular,
// column-major) to Ri.
inline int chol_inverse(int m, const double* G, int ldg, double drop, std::vector<double>& Ri) {
  std::vector<double> Rf(size_t(m) * m, 0.0);
  auto g = [&](int i, int j) { return G[i + size_t(ldg) * j]; };
  auto rf = [&](int i, int j) -> double& { return Rf[i + size_t(m) * j]; };
  int good = 0;
  for (int j = 0; j < m; ++j) {
    double d = g(j, j);
    for (int p = 0; p < j; ++p) d -= rf(p, j) * rf(p, j);
    if (!(d > drop * drop * g(j, j))) break;
    rf(j, j) = std::sqrt(d);
    for (int q = j + 1; q < m; ++q) {
      double v = g(j, q);
      for (int p = 0; p < j; ++p) v -= rf(p, j) * rf(p, q);
      rf(j, q) = v / rf(j, j);
    }
    ++good;
  }
  Ri.assign(size_t(good) * good, 0.0);
  auto ri = [&](int i, int j) -> double& { return Ri[i + size_t(good) * j]; };
  for (int j = 0; j < good; ++j) {
    ri(j, j) = 1.0 / rf(j, j);
    for (int i = j - 1; i >= 0; --i) {
      double s2 = 0.0;
      for (int p = i + 1; p <= j; ++p) s2 += rf(i, p) * ri(p, j);
      ri(i, j) = -s2 / rf(i, i);
    }
  }
  return good;
}

// Condition number lambda_max / lambda_min of a small symmetric positive definite matrix
// (m x m, column-major, leading dimension ldg); infinity when it is not positive definite.
inline double spd_condition(int m, const double* G, int ldg) {
  if (m <= 0) return 1.0;
  std::vector<double> A(size_t(m) * m), w, Z;
  for (int j = 0; j < m; ++j)
    for (int i = 0; i < m; ++i) A[i + size_t(m) * j] = G[i + size_t(ldg) * j];
  if (symeig(m, A.data(), w, Z, 0)) return std::numeric_limits<double>::infinity();
  if (!(w[0] > 0.0)) return std::numeric_limits<double>::infinity();
  return w[m - 1] / w[0];
}

}  // namespace fcg_small
