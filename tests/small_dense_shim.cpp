// C entry points over fermicg_gb300/csrc/small_dense.h so that the host-side linear algebra
// of the Davidson driver can be checked against numpy on a machine without a GPU.
#include "../fermicg_gb300/csrc/small_dense.h"

#include <cstring>

extern "C" int sd_symeig(int k, double* A, double* w, double* Z, int nvec) {
  std::vector<double> wv, Zv;
  const int rc = fcg_small::symeig(k, A, wv, Zv, nvec);
  if (k > 0) {
    std::memcpy(w, wv.data(), sizeof(double) * k);
    std::memcpy(Z, Zv.data(), sizeof(double) * Zv.size());
  }
  return rc;
}

extern "C" int sd_chol_inverse(int m, const double* G, int ldg, double drop, double* Ri) {
  std::vector<double> R;
  const int good = fcg_small::chol_inverse(m, G, ldg, drop, R);
  if (good > 0) std::memcpy(Ri, R.data(), sizeof(double) * size_t(good) * good);
  return good;
}

extern "C" double sd_spd_condition(int m, const double* G, int ldg) { return fcg_small::spd_condition(m, G, ldg); }

#include "../fermicg_gb300/csrc/tucker_small.cuh"

extern "C" void sd_coop_jacobi(int n, double* A, double* w, double* V, int* perm) {
  std::vector<double> cs(size_t(n) + 2), red(4);
  fcg_tucker::coop_jacobi_eigh(n, A, w, V, perm, cs.data(), red.data(), 0, 1);
}

extern "C" void sd_coop_mode_gram(const double* A, const int32_t* dims, int n, int m, double* G) {
  fcg_tucker::coop_mode_gram(A, dims, n, m, G, 0, 0, 1);
}

extern "C" void sd_coop_mode_product_t(const double* A, const int32_t* dims, int n, int m, const double* M, int ld,
                                       int knew, double* B) {
  fcg_tucker::coop_mode_product_t(A, dims, n, m, M, ld, knew, B, 0, 1);
}
