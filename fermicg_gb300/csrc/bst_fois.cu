// The compressed first-order interacting space of a block-sparse Tucker state on the GPU:
// build_compressed_1st_order_state (src/tucker_outer.jl:717-910).
//
// For every target Fock sector, every term of H (at most nbody clusters) and every block of
// the state, the term is applied to the block into each TuckerConfig reachable on the active
// clusters (their P or Q range in the target sector; spectators keep the block's ranges):
// form_sigma_block_expand (src/tucker_form_sigma_block_expand.jl:7-722).  Each such
// contribution is compressed by HOSVD, the contributions to one target TuckerConfig are added
// (nonorth_add, src/hosvd.jl:83-156) and compressed again, and the whole space is compressed
// until its length stops falling (compress_iteratively, src/type_BSTstate.jl:283-296).
//
// Device work:
//   fois_precontract_kernel   the local operators of 3- and 4-body terms are truncated by SVD
//                             on their bra index (precontract = true in the reference): one
//                             thread per (contribution, active cluster), from the Gram matrix
//                             of g[I, (p, l)] = sum_J G[p, I, J] U_ket[J, l]
//   the BST sigma machinery   every contribution is a bra block of its own (identity bra
//                             factors on the active clusters of 1- and 2-body terms, the
//                             truncated factors for 3- and 4-body terms, the ket's factors on
//                             the spectators) with exactly one (bra, ket, term) triple; one
//                             operator-cache build and one sigma launch give all their cores
//   tucker_compress_kernel    HOSVD truncation, one thread per Tucker tensor
//   tucker_add_kernel         nonorth_add of the contributions to one target block, one
//                             thread per block
// The host plans the contributions in the reference's loop order and reads back only ranks.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <unordered_map>
#include <vector>

#include "fcg_ctx.cuh"
#include "tucker_small.cuh"

using namespace fcg;
using namespace fcg_tucker;

namespace {

constexpr int kCtaThreads = 128;  // threads of the CTA that works on one small problem

// One Tucker tensor of a batch: the core of root r starts at core_off + r * stride (stride is
// the batch's), column-major with dims rank[0..N); factor m is (dim[m] x rank[m]) column-major.
struct TuckDesc {
  int64_t core_off;
  int64_t fac_off[kTuckMaxModes];
  int32_t dim[kTuckMaxModes];
  int32_t rank[kTuckMaxModes];
  int64_t work_off;  // scratch of the thread that handles this tensor
};

// Truncated SVD of one active cluster's local operator of a 3- or 4-body contribution.
struct PrecJob {
  int64_t tdm_off;   // TDM block (np x mb x mk, column-major) in the op blob
  int64_t kfac_off;  // ket factor (ket_len x L) in the factor blob
  int64_t out_off;   // output factor, capacity bra_len x bra_len
  int64_t work_off;  // scratch: g (bra_len x np L), Gram, eigenvectors, eigenvalues
  int32_t np, mb, bra_start, bra_len, ket_start, ket_len, L, pad;
  double scale1;     // max(1, max_r |ket core_r|) * |ints|
};

// Shared memory of one CTA working on one small problem: the d x d matrix and eigenvectors,
// eigenvalues, rotation pairs, two flags, a reduction row and the eigenvalue order.
struct CtaSmem {
  double *A, *V, *w, *cs, *red, *row;
  int* perm;
};

__device__ inline CtaSmem carve(double* sm, int dmax) {
  CtaSmem S;
  S.A = sm;
  S.V = S.A + dmax * dmax;
  S.w = S.V + dmax * dmax;
  S.cs = S.w + dmax;
  S.red = S.cs + dmax + 2;
  S.row = S.red + 4;
  S.perm = reinterpret_cast<int*>(S.row + kCtaThreads);
  return S;
}

size_t cta_smem_bytes(int dmax) {
  return sizeof(double) * (2 * size_t(dmax) * dmax + 2 * size_t(dmax) + 6 + kCtaThreads) + sizeof(int) * size_t(dmax);
}

// One CTA per job: g[I, (p, l)] = sum_J G[p, start_b + I, start_k + J] U_ket[J, l] in the job's
// scratch, its Gram matrix over I, the eigenvectors with sqrt|eigenvalue| * scale1 > prescreen
// (the left singular vectors of the reference's SVD, largest first) to out.
__global__ void __launch_bounds__(kCtaThreads) fois_precontract_kernel(int n, const PrecJob* __restrict__ jobs,
                                                                      const double* __restrict__ tdm,
                                                                      const double* __restrict__ fac, double prescreen,
                                                                      double* __restrict__ out,
                                                                      int32_t* __restrict__ nkeep,
                                                                      double* __restrict__ work, int64_t work_total,
                                                                      int dmax, int* __restrict__ err) {
  extern __shared__ double sm[];
  const int i = blockIdx.x;
  if (i >= n) return;
  const int tid = threadIdx.x, nt = blockDim.x;
  const CtaSmem S = carve(sm, dmax);
  const PrecJob J = jobs[i];
  const int bl = J.bra_len;
  const int64_t PL = int64_t(J.np) * J.L;
  if (bl > dmax || J.work_off < 0 || J.work_off + int64_t(bl) * PL > work_total) {  // extents the host sized
    if (tid == 0) atomicExch(err, 1);
    return;
  }
  double* D = work + J.work_off;
  const double* Gm = tdm + J.tdm_off;
  const double* U = fac + J.kfac_off;
  for (int64_t e = tid; e < int64_t(bl) * PL; e += nt) {
    const int I = int(e % bl);
    const int64_t pl = e / bl;
    const int p = int(pl % J.np), l = int(pl / J.np);
    double s = 0.0;
    for (int q = 0; q < J.ket_len; ++q)
      s += Gm[p + int64_t(J.np) * ((J.bra_start + I) + int64_t(J.mb) * (J.ket_start + q))] *
           U[q + int64_t(J.ket_len) * l];
    D[e] = s;
  }
  __syncthreads();
  for (int pp = tid; pp < bl * (bl + 1) / 2; pp += nt) {
    int b = int((sqrt(8.0 * pp + 1.0) - 1.0) * 0.5);
    while (b * (b + 1) / 2 > pp) --b;
    while ((b + 1) * (b + 2) / 2 <= pp) ++b;
    const int a = pp - b * (b + 1) / 2;
    double s = 0.0;
    for (int64_t e = 0; e < PL; ++e) s += D[a + bl * e] * D[b + bl * e];
    S.A[a + bl * b] = s;
    S.A[b + bl * a] = s;
  }
  __syncthreads();
  coop_jacobi_eigh(bl, S.A, S.w, S.V, S.perm, S.cs, S.red, tid, nt);
  if (tid == 0) {
    int k = 0;
    for (int a = 0; a < bl; ++a)
      if (sqrt(fabs(S.w[a])) * J.scale1 > prescreen) ++k;
    S.red[1] = k;
    nkeep[i] = k;
  }
  __syncthreads();
  const int k = int(S.red[1]);
  for (int e = tid; e < bl * k; e += nt) {
    const int a = e % bl, j = e / bl;
    out[J.out_off + e] = S.V[a + bl * S.perm[j]];
  }
}

// HOSVD truncation (tucker_decompose + compress, src/hosvd.jl:337-545), one CTA per tensor: per
// mode the eigenvectors of the summed Gram matrix of the R cores with sqrt|eigenvalue| > thresh;
// the cores projected onto them, the factors multiplied by them.  out_rank[t][m] receives the
// new ranks (a 0 anywhere: the tensor vanished).  Global scratch per tensor: the kept vectors
// of every mode (sum rank_m^2) and two core buffers of the input core length.
__global__ void __launch_bounds__(kCtaThreads) tucker_compress_kernel(
    int n, int N, int R, double thresh, const TuckDesc* __restrict__ in, int64_t in_stride,
    const double* __restrict__ in_core, const double* __restrict__ in_fac, const int32_t* __restrict__ in_rank,
    const TuckDesc* __restrict__ out, int64_t out_stride, double* __restrict__ out_core, double* __restrict__ out_fac,
    int32_t* __restrict__ out_rank, double* __restrict__ work, int64_t work_total, int dmax, int* __restrict__ err) {
  extern __shared__ double sm[];
  const int t = blockIdx.x;
  if (t >= n) return;
  const int tid = threadIdx.x, nt = blockDim.x;
  const CtaSmem S = carve(sm, dmax);
  const TuckDesc A = in[t];
  const TuckDesc O = out[t];
  int32_t dims[kTuckMaxModes], k[kTuckMaxModes];
  for (int m = 0; m < N; ++m) dims[m] = in_rank ? in_rank[int64_t(t) * N + m] : A.rank[m];
  const int64_t len = tensor_len(dims, N);
  if (len == 0) {
    if (tid == 0)
      for (int m = 0; m < N; ++m) out_rank[int64_t(t) * N + m] = 0;
    return;
  }
  double* W = work + A.work_off;
  int64_t wo[kTuckMaxModes];
  int64_t acc = 0;
  int dm = 0;
  for (int m = 0; m < N; ++m) {
    wo[m] = acc;
    acc += int64_t(dims[m]) * dims[m];
    dm = max(dm, int(dims[m]));
  }
  if (dm > dmax || A.work_off < 0 || A.work_off + acc + 2 * len > work_total) {  // extents the host sized
    if (tid == 0) atomicExch(err, 1);
    return;
  }
  double* buf0 = W + acc;
  double* buf1 = buf0 + len;
  bool empty = false;
  for (int m = 0; m < N; ++m) {
    const int d = dims[m];
    for (int r = 0; r < R; ++r) coop_mode_gram(in_core + A.core_off + r * in_stride, dims, N, m, S.A, r > 0, tid, nt);
    coop_jacobi_eigh(d, S.A, S.w, S.V, S.perm, S.cs, S.red, tid, nt);
    if (tid == 0) {
      int nk = 0;
      for (int a = 0; a < d; ++a)
        if (sqrt(fabs(S.w[a])) > thresh) ++nk;
      S.red[1] = nk;
    }
    __syncthreads();
    const int nk = int(S.red[1]);
    for (int e = tid; e < d * nk; e += nt) {
      const int a = e % d, j = e / d;
      W[wo[m] + e] = S.V[a + d * S.perm[j]];
    }
    __syncthreads();
    k[m] = nk;
    if (nk == 0) empty = true;
  }
  if (tid == 0)
    for (int m = 0; m < N; ++m) out_rank[int64_t(t) * N + m] = k[m];
  if (empty) return;
  const int64_t nlen = tensor_len(k, N);
  for (int r = 0; r < R; ++r) {
    int32_t cur[kTuckMaxModes];
    for (int m = 0; m < N; ++m) cur[m] = dims[m];
    const double* src = in_core + A.core_off + r * in_stride;
    double* dst = buf0;
    for (int m = 0; m < N; ++m) {
      coop_mode_product_t(src, cur, N, m, W + wo[m], dims[m], k[m], dst, tid, nt);
      cur[m] = k[m];
      src = dst;
      dst = (dst == buf0) ? buf1 : buf0;
    }
    double* o = out_core + O.core_off + r * out_stride;
    for (int64_t e = tid; e < nlen; e += nt) o[e] = src[e];
    __syncthreads();
  }
  for (int m = 0; m < N; ++m) {
    const int rows = A.dim[m], d = dims[m];
    const double* F = in_fac + A.fac_off[m];
    for (int e = tid; e < rows * k[m]; e += nt) {
      const int i = e % rows, j = e / rows;
      double s = 0.0;
      for (int q = 0; q < d; ++q) s += F[i + int64_t(rows) * q] * W[wo[m] + q + int64_t(d) * j];
      out_fac[O.fac_off[m] + e] = s;
    }
  }
}

// nonorth_add (src/hosvd.jl:83-156) of the tensors members[ptr[g] .. ptr[g+1]) that are not
// empty, one CTA per target block: taken by decreasing norm; per mode the left singular vectors
// of the stacked factors with singular value > thresh (from the eigen-decomposition of their
// Gram matrix, ignoring eigenvalues at rounding level); the sum of the members' cores
// transformed into those bases.  A single member is copied.  Global scratch per block
// (host-sized): member order and norms, one transform and two core buffers.
__global__ void __launch_bounds__(kCtaThreads) tucker_add_kernel(
    int ng, int N, int R, double thresh, const int64_t* __restrict__ ptr, const int32_t* __restrict__ members,
    const TuckDesc* __restrict__ in, int64_t in_stride, const double* __restrict__ in_core,
    const double* __restrict__ in_fac, const int32_t* __restrict__ in_rank, const TuckDesc* __restrict__ out,
    int64_t out_stride, double* __restrict__ out_core, double* __restrict__ out_fac, int32_t* __restrict__ out_rank,
    double* __restrict__ work, const int64_t* __restrict__ work_off, const int64_t* __restrict__ buf_len,
    int64_t work_total, int dmax, int* __restrict__ err) {
  extern __shared__ double sm[];
  const int g = blockIdx.x;
  if (g >= ng) return;
  const int tid = threadIdx.x, nt = blockDim.x;
  const CtaSmem S = carve(sm, dmax);
  const TuckDesc O = out[g];
  const int64_t nmem = ptr[g + 1] - ptr[g];
  {
    int dm = 0;
    for (int m = 0; m < N; ++m) dm = max(dm, int(O.dim[m]));
    if (dm > dmax || work_off[g] < 0 || work_off[g] + 2 * nmem + int64_t(dmax) * dmax + 2 * buf_len[g] > work_total) {
      if (tid == 0) atomicExch(err, 1);  // extents the host sized
      return;
    }
  }
  double* ord = work + work_off[g];  // member ids (exact in a double) in the order of addition
  double* nrm = ord + nmem;
  if (tid == 0) {
    int nv = 0;
    for (int64_t q = ptr[g]; q < ptr[g + 1]; ++q) {
      const int32_t t = members[q];
      int64_t l = 1;
      for (int m = 0; m < N; ++m) l *= in_rank[int64_t(t) * N + m];
      if (l > 0) ord[nv++] = double(t);
    }
    S.red[1] = nv;
  }
  __syncthreads();
  const int nval = int(S.red[1]);
  if (nval == 0) {
    if (tid == 0)
      for (int m = 0; m < N; ++m) out_rank[int64_t(g) * N + m] = 0;
    return;
  }
  for (int a = 0; a < nval; ++a) {  // norms over all roots
    const int32_t t = int32_t(ord[a]);
    int32_t dims[kTuckMaxModes];
    for (int m = 0; m < N; ++m) dims[m] = in_rank[int64_t(t) * N + m];
    const int64_t l = tensor_len(dims, N);
    double s = 0.0;
    for (int r = 0; r < R; ++r) {
      const double* c = in_core + in[t].core_off + r * in_stride;
      for (int64_t e = tid; e < l; e += nt) s += c[e] * c[e];
    }
    S.row[tid] = s;
    __syncthreads();
    if (tid == 0) {
      double tot = 0.0;
      for (int q = 0; q < nt; ++q) tot += S.row[q];
      nrm[a] = sqrt(tot);
    }
    __syncthreads();
  }
  if (tid == 0)  // stable insertion sort by decreasing norm
    for (int a = 1; a < nval; ++a) {
      const double kn = nrm[a], kt = ord[a];
      int b = a - 1;
      while (b >= 0 && nrm[b] < kn) {
        nrm[b + 1] = nrm[b];
        ord[b + 1] = ord[b];
        --b;
      }
      nrm[b + 1] = kn;
      ord[b + 1] = kt;
    }
  __syncthreads();
  if (nval == 1) {
    const int32_t t0 = int32_t(ord[0]);
    int32_t dims[kTuckMaxModes];
    for (int m = 0; m < N; ++m) dims[m] = in_rank[int64_t(t0) * N + m];
    const int64_t l = tensor_len(dims, N);
    for (int r = 0; r < R; ++r)
      for (int64_t e = tid; e < l; e += nt)
        out_core[O.core_off + r * out_stride + e] = in_core[in[t0].core_off + r * in_stride + e];
    for (int m = 0; m < N; ++m) {
      const int64_t fl = int64_t(in[t0].dim[m]) * dims[m];
      for (int64_t e = tid; e < fl; e += nt) out_fac[O.fac_off[m] + e] = in_fac[in[t0].fac_off[m] + e];
    }
    if (tid == 0)
      for (int m = 0; m < N; ++m) out_rank[int64_t(g) * N + m] = dims[m];
    return;
  }
  double* M = nrm + nmem;  // transform (r x k), at most dmax x dmax
  double* buf0 = M + dmax * dmax;
  double* buf1 = buf0 + buf_len[g];
  int32_t k[kTuckMaxModes];
  bool empty = false;
  for (int m = 0; m < N; ++m) {
    const int d = O.dim[m];
    for (int pp = tid; pp < d * (d + 1) / 2; pp += nt) {
      int j = int((sqrt(8.0 * pp + 1.0) - 1.0) * 0.5);
      while (j * (j + 1) / 2 > pp) --j;
      while ((j + 1) * (j + 2) / 2 <= pp) ++j;
      const int i = pp - j * (j + 1) / 2;
      double s = 0.0;
      for (int a = 0; a < nval; ++a) {
        const int32_t t = int32_t(ord[a]);
        const int rt = in_rank[int64_t(t) * N + m];
        const double* F = in_fac + in[t].fac_off[m];
        for (int c = 0; c < rt; ++c) s += F[i + int64_t(d) * c] * F[j + int64_t(d) * c];
      }
      S.A[i + d * j] = s;
      S.A[j + d * i] = s;
    }
    __syncthreads();
    coop_jacobi_eigh(d, S.A, S.w, S.V, S.perm, S.cs, S.red, tid, nt);
    if (tid == 0) {
      const double floor2 = fmax(thresh * thresh, 64.0 * 2.220446049250313e-16 * fmax(S.w[S.perm[0]], 0.0));
      int nk = 0;
      for (int a = 0; a < d; ++a)
        if (S.w[a] > floor2) ++nk;
      S.red[1] = min(nk, int(O.rank[m]));  // the host's capacity (never binding)
    }
    __syncthreads();
    const int nk = int(S.red[1]);
    for (int e = tid; e < d * nk; e += nt) {
      const int a = e % d, j = e / d;
      out_fac[O.fac_off[m] + e] = S.V[a + d * S.perm[j]];
    }
    __syncthreads();
    k[m] = nk;
    if (nk == 0) empty = true;
  }
  if (tid == 0)
    for (int m = 0; m < N; ++m) out_rank[int64_t(g) * N + m] = k[m];
  if (empty) return;
  const int64_t nlen = tensor_len(k, N);
  for (int r = 0; r < R; ++r)
    for (int64_t e = tid; e < nlen; e += nt) out_core[O.core_off + r * out_stride + e] = 0.0;
  __syncthreads();
  for (int a = 0; a < nval; ++a) {
    const int32_t t = int32_t(ord[a]);
    const TuckDesc& Ad = in[t];
    int32_t dims[kTuckMaxModes];
    for (int m = 0; m < N; ++m) dims[m] = in_rank[int64_t(t) * N + m];
    for (int r = 0; r < R; ++r) {
      int32_t cur[kTuckMaxModes];
      for (int m = 0; m < N; ++m) cur[m] = dims[m];
      const double* src = in_core + Ad.core_off + r * in_stride;
      double* dst = buf0;
      for (int m = 0; m < N; ++m) {
        // M[c + rt * j] = sum_i F_t[i, c] Unew[i, j]  (the transform Unew^T F_t, transposed)
        const int d = O.dim[m], rt = dims[m];
        const double* F = in_fac + Ad.fac_off[m];
        const double* Un = out_fac + O.fac_off[m];
        for (int e = tid; e < rt * k[m]; e += nt) {
          const int c = e % rt, j = e / rt;
          double s = 0.0;
          for (int i = 0; i < d; ++i) s += F[i + int64_t(d) * c] * Un[i + int64_t(d) * j];
          M[e] = s;
        }
        __syncthreads();
        coop_mode_product_t(src, cur, N, m, M, rt, k[m], dst, tid, nt);
        cur[m] = k[m];
        src = dst;
        dst = (dst == buf0) ? buf1 : buf0;
      }
      double* o = out_core + O.core_off + r * out_stride;
      for (int64_t e = tid; e < nlen; e += nt) o[e] += src[e];
      __syncthreads();
    }
  }
}

}  // namespace

namespace {

// A Tucker batch on the device: descriptors, cores [R][stride] and factors.
struct TuckBatch {
  std::vector<TuckDesc> desc;  // capacities (ranks) per tensor
  int64_t stride = 0;          // core elements per root
  int64_t n_fac = 0;
  DevBuf<TuckDesc> d_desc;
  DevBuf<double> core, fac;
  DevBuf<int32_t> rank;        // actual ranks, [n][N]
};

// capacities of `b` as a compact layout: core offsets and factor offsets from ranks and dims
void lay_out(TuckBatch& b, int N) {
  int64_t co = 0, fo = 0;
  for (TuckDesc& d : b.desc) {
    d.core_off = co;
    int64_t l = 1;
    for (int m = 0; m < N; ++m) {
      d.fac_off[m] = fo;
      fo += int64_t(d.dim[m]) * d.rank[m];
      l *= d.rank[m];
    }
    co += l;
  }
  b.stride = std::max<int64_t>(co, 1);
  b.n_fac = std::max<int64_t>(fo, 1);
}

// scratch of tucker_compress_kernel for a tensor of capacity ranks rk
int64_t compress_work(const TuckDesc& d, int N) {
  int64_t sq = 0, len = 1;
  for (int m = 0; m < N; ++m) {
    sq += int64_t(d.rank[m]) * d.rank[m];
    len *= d.rank[m];
  }
  return sq + 2 * len;
}

// dynamic shared memory of a CTA-per-problem launch with matrices up to dmax x dmax
template <typename K>
int cta_smem(K kernel, int dmax, size_t* bytes) {
  *bytes = cta_smem_bytes(std::max(dmax, 1));
  if (*bytes > 48 * 1024)
    return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(*bytes)) == cudaSuccess ? 0
                                                                                                                  : 1;
  return 0;
}

int run_compress(fcg_ctx* ctx, int N, int R, double thresh, TuckBatch& in, const int32_t* d_in_rank, TuckBatch& out,
                 DevBuf<double>& work, int* d_err) {
  const int n = int(in.desc.size());
  out.desc = in.desc;
  lay_out(out, N);
  int64_t wo = 0;
  int dmax = 1;
  for (size_t t = 0; t < in.desc.size(); ++t) {
    in.desc[t].work_off = wo;
    wo += compress_work(in.desc[t], N);
    for (int m = 0; m < N; ++m) dmax = std::max(dmax, int(in.desc[t].rank[m]));
  }
  size_t smem = 0;
  FCG_REQUIRE(!cta_smem(tucker_compress_kernel, dmax, &smem), FCG_ECUDA, "FOIS: shared memory attribute");
  FCG_CUDA(in.d_desc.upload(in.desc.data(), in.desc.size(), ctx->stream));
  FCG_CUDA(out.d_desc.upload(out.desc.data(), out.desc.size(), ctx->stream));
  FCG_CUDA(out.core.alloc(size_t(out.stride) * R));
  FCG_CUDA(out.fac.alloc(size_t(out.n_fac)));
  FCG_CUDA(out.rank.alloc(size_t(std::max(n, 1)) * N));
  FCG_CUDA(work.alloc(size_t(std::max<int64_t>(wo, 1))));
  if (n > 0) {
    tucker_compress_kernel<<<unsigned(n), kCtaThreads, smem, ctx->stream>>>(
        n, N, R, thresh, in.d_desc.p, in.stride, in.core.p, in.fac.p, d_in_rank, out.d_desc.p, out.stride,
        out.core.p, out.fac.p, out.rank.p, work.p, int64_t(work.n), dmax, d_err);
    FCG_CUDA(cudaGetLastError());
  }
  return FCG_OK;
}

std::string fock_key(const int16_t* f, int N) { return std::string(reinterpret_cast<const char*>(f), 4 * N); }

}  // namespace

extern "C" {

int fcg_bst_fois(fcg_ctx* ctx, int R, int nbody, double thresh, int compress_twice, int64_t n_blocks,
                 const int16_t* fock, const int64_t* blocks, const int64_t* factor_off, int64_t n_factors,
                 const double* factors, const double* cores, const int32_t* spaces, int64_t* out_n_blocks,
                 int64_t* out_core_total, int64_t* out_n_factors) {
  if (!ctx) return FCG_EINVAL;
  FCG_REQUIRE(ctx->have_ops && ctx->have_terms, FCG_ESTATE, "upload ops and terms first");
  FCG_REQUIRE(fock && blocks && factor_off && factors && cores && spaces && out_n_blocks && out_core_total &&
                  out_n_factors && n_blocks > 0 && n_factors > 0,
              FCG_EINVAL, "null pointer or empty BST state");
  FCG_REQUIRE(R >= 1 && R <= 64, FCG_ELIMIT, "R must be in [1, 64]");
  FCG_REQUIRE(nbody >= 1 && nbody <= 4, FCG_EINVAL, "nbody must be in [1, 4]");
  FCG_REQUIRE(thresh > 0, FCG_EINVAL, "thresh must be positive");
  const int N = ctx->N;
  FCG_REQUIRE(N <= kTuckMaxModes, FCG_ELIMIT, "at most 8 clusters");
  FCG_CUDA(cudaSetDevice(ctx->device));
  const auto t0 = std::chrono::steady_clock::now();
  {
    const int rc = term_norms(ctx);
    if (rc) return rc;
  }
  const int nmax1 = ctx->nmax + 1;
  // the state's blocks: validation, core offsets, and their grouping by Fock sector
  std::vector<int64_t> coff(n_blocks), clen(n_blocks);
  int64_t ctot = 0;
  for (int64_t b = 0; b < n_blocks; ++b) {
    int64_t l = 1;
    for (int c = 0; c < N; ++c) {
      const int64_t rk = blocks[3 * N * b + c], st = blocks[3 * N * b + N + c], ln = blocks[3 * N * b + 2 * N + c];
      FCG_REQUIRE(rk >= 1 && rk <= ln && st >= 0 && ln <= kTuckMaxDim, FCG_EINVAL,
                  "FOIS: ranks must be in [1, range length] and ranges at most 64 states");
      FCG_REQUIRE(factor_off[N * b + c] >= 0 && factor_off[N * b + c] + rk * ln <= n_factors, FCG_EINVAL,
                  "FOIS: factor out of range");
      const int fa = fock[2 * N * b + 2 * c], fbv = fock[2 * N * b + 2 * c + 1];
      FCG_REQUIRE(fa >= 0 && fa <= ctx->norb[c] && fbv >= 0 && fbv <= ctx->norb[c], FCG_EINVAL, "FOIS: bad Fock sector");
      l *= rk;
    }
    coff[b] = ctot;
    clen[b] = l;
    ctot += l;
  }
  std::vector<double> cnorm(n_blocks, 0.0);  // max over roots of the core norm
  for (int64_t b = 0; b < n_blocks; ++b)
    for (int r = 0; r < R; ++r) {
      double s = 0.0;
      for (int64_t e = 0; e < clen[b]; ++e) s += cores[r * ctot + coff[b] + e] * cores[r * ctot + coff[b] + e];
      cnorm[b] = std::max(cnorm[b], std::sqrt(s));
    }
  std::vector<std::vector<int64_t>> fgroups;
  std::vector<const int16_t*> fgroup_fock;
  {
    std::unordered_map<std::string, size_t> at;
    for (int64_t b = 0; b < n_blocks; ++b) {
      const std::string key = fock_key(fock + 2 * N * b, N);
      auto it = at.find(key);
      if (it == at.end()) {
        it = at.emplace(key, fgroups.size()).first;
        fgroups.emplace_back();
        fgroup_fock.push_back(fock + 2 * N * b);
      }
      fgroups[it->second].push_back(b);
    }
  }
  std::vector<std::vector<int>> by_trans(ctx->n_trans);
  for (int t = 0; t < ctx->n_terms; ++t) {
    const int32_t* r = &ctx->trm[int64_t(t) * kTrmCols];
    by_trans[r[1]].push_back(t);
  }
  // jobs: target Fock sector -> (transfer, state sector group), in order of discovery
  struct Job {
    std::vector<int16_t> fock;
    std::vector<std::pair<int, size_t>> parts;
  };
  std::vector<Job> jobs;
  {
    std::unordered_map<std::string, size_t> at;
    std::vector<int16_t> fs(2 * N);
    for (size_t gi = 0; gi < fgroups.size(); ++gi) {
      const int16_t* fk = fgroup_fock[gi];
      for (int tr = 0; tr < ctx->n_trans; ++tr) {
        bool ok = true;
        for (int c = 0; c < N && ok; ++c)
          for (int s = 0; s < 2; ++s) {
            const int v = fk[2 * c + s] + ctx->trans[(int64_t(tr) * N + c) * 2 + s];
            if (v < 0 || v > ctx->norb[c]) ok = false;
            fs[2 * c + s] = int16_t(v);
          }
        for (int c = 0; c < N && ok; ++c)
          ok = ctx->h_blk_index[dense_block_index(nmax1, c, kOpH, fs[2 * c], fs[2 * c + 1], fs[2 * c], fs[2 * c + 1])] >=
               0;
        if (!ok) continue;
        const std::string key = fock_key(fs.data(), N);
        auto it = at.find(key);
        if (it == at.end()) {
          it = at.emplace(key, jobs.size()).first;
          jobs.push_back(Job{fs, {}});
        }
        jobs[it->second].parts.emplace_back(tr, gi);
      }
    }
  }
  // contributions (term, ket block, target TuckerConfig) in the reference's loop order, and
  // the target blocks they add into
  struct Item {
    int32_t term, ket, group;
    int32_t start[kMaxClusters], len[kMaxClusters];
  };
  std::vector<Item> items;
  std::vector<std::vector<int16_t>> gfock;
  std::vector<std::vector<int32_t>> granges;  // [start[N], len[N]]
  auto space = [&](int c, int na, int nb_, int which, int* st, int* ln) {
    const int32_t* sp = spaces + ((int64_t(c) * nmax1 + na) * nmax1 + nb_) * 4;
    *st = sp[2 * which];
    *ln = sp[2 * which + 1];
    return *ln > 0;
  };
  for (const Job& J : jobs) {
    std::unordered_map<std::string, int32_t> gat;  // target TuckerConfig -> group
    const int16_t* fs = J.fock.data();
    for (const auto& part : J.parts) {
      const int tr = part.first;
      const std::vector<int64_t>& kets = fgroups[part.second];
      for (int t : by_trans[tr]) {
        const int32_t* r = &ctx->trm[int64_t(t) * kTrmCols];
        if (r[0] > nbody) continue;
        const int na = r[0];
        // every active cluster's TDM block for this sector pair must exist
        const int16_t* fk0 = fock + 2 * N * kets[0];
        bool have = true;
        for (int o = 0; o < na && have; ++o) {
          const int c = r[2 + o];
          have = ctx->h_blk_index[dense_block_index(nmax1, c, r[6 + o], fs[2 * c], fs[2 * c + 1], fk0[2 * c],
                                                    fk0[2 * c + 1])] >= 0;
        }
        if (!have) continue;
        int opt_st[4][2], opt_ln[4][2], nopt[4];
        for (int o = 0; o < na; ++o) {
          const int c = r[2 + o];
          nopt[o] = 0;
          for (int which = 0; which < 2; ++which) {
            int st, ln;
            if (space(c, fs[2 * c], fs[2 * c + 1], which, &st, &ln)) {
              opt_st[o][nopt[o]] = st;
              opt_ln[o][nopt[o]] = ln;
              ++nopt[o];
            }
          }
        }
        for (int64_t k : kets) {
          int idx[4] = {0, 0, 0, 0};
          bool done = false;
          for (int o = 0; o < na; ++o)
            if (nopt[o] == 0) done = true;
          while (!done) {
            Item it{};
            it.term = t;
            it.ket = int32_t(k);
            for (int c = 0; c < N; ++c) {
              it.start[c] = int32_t(blocks[3 * N * k + N + c]);
              it.len[c] = int32_t(blocks[3 * N * k + 2 * N + c]);
            }
            for (int o = 0; o < na; ++o) {
              it.start[r[2 + o]] = opt_st[o][idx[o]];
              it.len[r[2 + o]] = opt_ln[o][idx[o]];
            }
            bool fits = true;
            for (int c = 0; c < N; ++c) fits = fits && it.len[c] <= kTuckMaxDim;
            FCG_REQUIRE(fits, FCG_ELIMIT, "FOIS: a target range exceeds 64 local states");
            std::vector<int32_t> rg(2 * N);
            for (int c = 0; c < N; ++c) {
              rg[c] = it.start[c];
              rg[N + c] = it.len[c];
            }
            const std::string key(reinterpret_cast<const char*>(rg.data()), rg.size() * sizeof(int32_t));
            auto gi = gat.find(key);
            if (gi == gat.end()) {
              gi = gat.emplace(key, int32_t(gfock.size())).first;
              gfock.push_back(J.fock);
              granges.push_back(rg);
            }
            it.group = gi->second;
            items.push_back(it);
            // next product of the active clusters' options (first cluster fastest, as
            // Iterators.product runs)
            int o = 0;
            while (o < na) {
              if (++idx[o] < nopt[o]) break;
              idx[o] = 0;
              ++o;
            }
            if (o == na) done = true;
          }
        }
      }
    }
  }
  const int64_t n_items = int64_t(items.size());
  FCG_REQUIRE(n_items < (int64_t(1) << 24), FCG_ELIMIT, "FOIS: more than 2^24 contributions");
  // every kernel checks the scratch extents it was given and raises this flag instead of
  // touching memory outside them
  DevBuf<int> d_err;
  FCG_CUDA(d_err.alloc(1));
  FCG_CUDA(cudaMemsetAsync(d_err.p, 0, sizeof(int), ctx->stream));
  auto check_err = [&]() -> int {
    int e = 0;
    FCG_CUDA(cudaMemcpyAsync(&e, d_err.p, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    FCG_CUDA(cudaStreamSynchronize(ctx->stream));
    FCG_REQUIRE(e == 0, FCG_ECUDA, "FOIS: a kernel found its scratch smaller than it needs");
    return FCG_OK;
  };
  // 1. the truncated bra factors of 3- and 4-body contributions
  std::vector<int32_t> item_nk(size_t(n_items) * 4, 0);  // per active cluster: kept vectors
  std::vector<int64_t> prec_of(size_t(n_items), -1);     // first job of the item
  std::vector<PrecJob> pj;
  int64_t pout = 0, pwork = 0;
  for (int64_t i = 0; i < n_items; ++i) {
    const Item& it = items[size_t(i)];
    const int32_t* r = &ctx->trm[int64_t(it.term) * kTrmCols];
    if (r[0] < 3) continue;
    prec_of[size_t(i)] = int64_t(pj.size());
    const int16_t* fs = gfock[size_t(it.group)].data();
    const int16_t* fk = fock + 2 * N * it.ket;
    const double scale1 = std::max(1.0, cnorm[it.ket]) * ctx->term_ints_norm[size_t(it.term)];
    for (int o = 0; o < r[0]; ++o) {
      const int c = r[2 + o];
      const int bi = ctx->h_blk_index[dense_block_index(nmax1, c, r[6 + o], fs[2 * c], fs[2 * c + 1], fk[2 * c],
                                                        fk[2 * c + 1])];
      const BlockInfo& BI = ctx->h_blocks[size_t(bi)];
      PrecJob J{};
      J.tdm_off = BI.off;
      J.kfac_off = factor_off[N * it.ket + c];
      J.np = BI.nidx;
      J.mb = BI.mb;
      J.bra_start = it.start[c];
      J.bra_len = it.len[c];
      J.ket_start = int32_t(blocks[3 * N * it.ket + N + c]);
      J.ket_len = int32_t(blocks[3 * N * it.ket + 2 * N + c]);
      J.L = int32_t(blocks[3 * N * it.ket + c]);
      J.scale1 = scale1;
      FCG_REQUIRE(J.bra_start + J.bra_len <= BI.mb && J.ket_start + J.ket_len <= BI.mk, FCG_EINVAL,
                  "FOIS: a Tucker range exceeds the local basis of its Fock sector");
      J.out_off = pout;
      pout += int64_t(J.bra_len) * J.bra_len;
      J.work_off = pwork;
      pwork += int64_t(J.bra_len) * J.np * J.L;
      pj.push_back(J);
    }
  }
  std::vector<double> pfac;
  if (!pj.empty()) {
    DevBuf<PrecJob> d_pj;
    DevBuf<double> d_pfac, d_pwork, d_kfac;
    DevBuf<int32_t> d_nk;
    FCG_CUDA(d_pj.upload(pj.data(), pj.size(), ctx->stream));
    FCG_CUDA(d_kfac.upload(factors, size_t(n_factors), ctx->stream));
    FCG_CUDA(d_pfac.alloc(size_t(std::max<int64_t>(pout, 1))));
    FCG_CUDA(d_pwork.alloc(size_t(std::max<int64_t>(pwork, 1))));
    FCG_CUDA(d_nk.alloc(pj.size()));
    const int n = int(pj.size());
    int dmax = 1;
    for (const PrecJob& J : pj) dmax = std::max(dmax, J.bra_len);
    size_t smem = 0;
    FCG_REQUIRE(!cta_smem(fois_precontract_kernel, dmax, &smem), FCG_ECUDA, "FOIS: shared memory attribute");
    fois_precontract_kernel<<<unsigned(n), kCtaThreads, smem, ctx->stream>>>(
        n, d_pj.p, ctx->d_op64.p, d_kfac.p, thresh, d_pfac.p, d_nk.p, d_pwork.p, int64_t(d_pwork.n), dmax, d_err.p);
    FCG_CUDA(cudaGetLastError());
    std::vector<int32_t> nk(pj.size());
    pfac.resize(size_t(std::max<int64_t>(pout, 1)));
    FCG_CUDA(cudaMemcpyAsync(nk.data(), d_nk.p, sizeof(int32_t) * nk.size(), cudaMemcpyDeviceToHost, ctx->stream));
    FCG_CUDA(cudaMemcpyAsync(pfac.data(), d_pfac.p, sizeof(double) * pfac.size(), cudaMemcpyDeviceToHost,
                             ctx->stream));
    FCG_CUDA(cudaStreamSynchronize(ctx->stream));
    {
      const int rc = check_err();
      if (rc) return rc;
    }
    for (int64_t i = 0; i < n_items; ++i) {
      if (prec_of[size_t(i)] < 0) continue;
      const int32_t* r = &ctx->trm[int64_t(items[size_t(i)].term) * kTrmCols];
      for (int o = 0; o < r[0]; ++o) item_nk[size_t(i) * 4 + o] = nk[size_t(prec_of[size_t(i)] + o)];
    }
  }
  // 2. the expansion structure: the state's blocks, then one block per surviving contribution
  std::vector<int16_t> sfock(fock, fock + 2 * N * n_blocks);
  std::vector<int64_t> sblk(blocks, blocks + 3 * N * n_blocks);
  std::vector<int64_t> sfoff(factor_off, factor_off + N * n_blocks);
  std::vector<double> sfac(factors, factors + n_factors);
  std::vector<int32_t> triples;
  std::vector<int64_t> kept;  // item of each contribution block
  for (int64_t i = 0; i < n_items; ++i) {
    const Item& it = items[size_t(i)];
    const int32_t* r = &ctx->trm[int64_t(it.term) * kTrmCols];
    bool ok = true;
    for (int o = 0; o < r[0] && r[0] >= 3; ++o) ok = ok && item_nk[size_t(i) * 4 + o] > 0;
    if (!ok) continue;  // an empty factor: the contribution has length 0
    const int16_t* fs = gfock[size_t(it.group)].data();
    sfock.insert(sfock.end(), fs, fs + 2 * N);
    std::vector<int64_t> row(3 * N), fo(N);
    for (int c = 0; c < N; ++c) {
      row[c] = blocks[3 * N * it.ket + c];
      row[N + c] = it.start[c];
      row[2 * N + c] = it.len[c];
      fo[c] = factor_off[N * it.ket + c];
    }
    for (int o = 0; o < r[0]; ++o) {
      const int c = r[2 + o];
      const int L = it.len[c];
      fo[c] = int64_t(sfac.size());
      if (r[0] < 3) {
        row[c] = L;
        for (int j = 0; j < L; ++j)
          for (int a = 0; a < L; ++a) sfac.push_back(a == j ? 1.0 : 0.0);
      } else {
        const int nk = item_nk[size_t(i) * 4 + o];
        row[c] = nk;
        const PrecJob& J = pj[size_t(prec_of[size_t(i)] + o)];
        sfac.insert(sfac.end(), pfac.begin() + J.out_off, pfac.begin() + J.out_off + int64_t(L) * nk);
      }
    }
    sblk.insert(sblk.end(), row.begin(), row.end());
    sfoff.insert(sfoff.end(), fo.begin(), fo.end());
    triples.insert(triples.end(), {int32_t(n_blocks + int64_t(kept.size())), it.ket, it.term});
    kept.push_back(i);
  }
  const int64_t n_kept = int64_t(kept.size());
  ctx->fois = {};
  ctx->fois.R = R;
  if (n_kept == 0) {
    *out_n_blocks = 0;
    *out_core_total = 0;
    *out_n_factors = 0;
    return FCG_OK;
  }
  const int64_t n_struct = n_blocks + n_kept;
  int64_t core_total = 0;
  {
    const int rc = bst_set_impl(ctx, nbody, n_struct, sfock.data(), sblk.data(), sfoff.data(),
                                int64_t(sfac.size()), sfac.data(), triples.data(), n_kept, &core_total);
    if (rc) return rc;
  }
  // 3. every contribution's core: one BST sigma of the state's cores
  TuckBatch T0;
  FCG_CUDA(T0.core.alloc(size_t(core_total) * R));
  {
    std::vector<double> cin(size_t(core_total) * R, 0.0);
    for (int64_t b = 0; b < n_blocks; ++b)
      for (int r = 0; r < R; ++r)
        std::memcpy(&cin[size_t(r * core_total + ctx->bst_blocks[size_t(b)].core_off)], &cores[r * ctot + coff[b]],
                    sizeof(double) * size_t(clen[b]));
    DevBuf<double> d_in;
    FCG_CUDA(d_in.upload(cin.data(), cin.size(), ctx->stream));
    const int rc = fcg_bst_sigma_device(ctx, R, d_in.p, T0.core.p, FCG_FP64);
    if (rc) return rc;
  }
  T0.stride = core_total;
  T0.desc.resize(size_t(n_kept));
  for (int64_t q = 0; q < n_kept; ++q) {
    const BstBlock& B = ctx->bst_blocks[size_t(n_blocks + q)];
    TuckDesc& d = T0.desc[size_t(q)];
    d = TuckDesc{};
    d.core_off = B.core_off;
    for (int c = 0; c < N; ++c) {
      d.fac_off[c] = B.factor_off[c];
      d.dim[c] = B.len[c];
      d.rank[c] = B.rank[c];
    }
  }
  // T0's factors are the structure's factor blob on the device
  const double* d_sfac = ctx->d_bst_factors.p;
  // 4. compress every contribution
  TuckBatch T1;
  DevBuf<double> work;
  {
    TuckBatch& in = T0;
    in.fac.p = const_cast<double*>(d_sfac);  // borrowed, released below before T0 goes out of scope
    int rc = run_compress(ctx, N, R, thresh, in, nullptr, T1, work, d_err.p);
    in.fac.p = nullptr;
    if (rc) return rc;
  }
  // 5. nonorth_add of the contributions to each target block
  const int64_t ng = int64_t(gfock.size());
  std::vector<int64_t> gptr(size_t(ng) + 1, 0);
  std::vector<int32_t> gmem(static_cast<size_t>(n_kept));
  {
    std::vector<int64_t> cnt(size_t(ng), 0);
    for (int64_t q = 0; q < n_kept; ++q) ++cnt[size_t(items[size_t(kept[size_t(q)])].group)];
    for (int64_t g = 0; g < ng; ++g) gptr[size_t(g) + 1] = gptr[size_t(g)] + cnt[size_t(g)];
    std::vector<int64_t> pos(gptr.begin(), gptr.end() - 1);
    for (int64_t q = 0; q < n_kept; ++q) gmem[size_t(pos[size_t(items[size_t(kept[size_t(q)])].group)]++)] = int32_t(q);
  }
  TuckBatch T2;
  T2.desc.resize(static_cast<size_t>(ng));
  std::vector<int64_t> gwork(static_cast<size_t>(ng)), gbuf(static_cast<size_t>(ng)), gnm(static_cast<size_t>(ng));
  int64_t wtot = 0, gdmax = 1;
  for (int64_t g = 0; g < ng; ++g) {
    TuckDesc& d = T2.desc[size_t(g)];
    d = TuckDesc{};
    int64_t buf = 1, dmax = 1;
    for (int c = 0; c < N; ++c) {
      const int dim = granges[size_t(g)][size_t(N + c)];
      int64_t sum = 0, rmax = 0;
      for (int64_t q = gptr[size_t(g)]; q < gptr[size_t(g) + 1]; ++q) {
        sum += T0.desc[size_t(gmem[size_t(q)])].rank[c];
        rmax = std::max<int64_t>(rmax, T0.desc[size_t(gmem[size_t(q)])].rank[c]);
      }
      d.dim[c] = dim;
      d.rank[c] = int32_t(std::max<int64_t>(1, std::min<int64_t>(dim, sum)));
      buf *= std::max<int64_t>(d.rank[c], std::max<int64_t>(rmax, 1));
      dmax = std::max<int64_t>(dmax, dim);
    }
    gbuf[size_t(g)] = buf;
    gnm[size_t(g)] = gptr[size_t(g) + 1] - gptr[size_t(g)];
    gdmax = std::max<int64_t>(gdmax, dmax);
  }
  // the kernel places each block's transform (gdmax x gdmax, the launch's largest dimension)
  // between the member lists and the core buffers
  for (int64_t g = 0; g < ng; ++g) {
    gwork[size_t(g)] = wtot;
    wtot += 2 * gnm[size_t(g)] + gdmax * gdmax + 2 * gbuf[size_t(g)];
  }
  lay_out(T2, N);
  FCG_CUDA(T2.d_desc.upload(T2.desc.data(), T2.desc.size(), ctx->stream));
  FCG_CUDA(T2.core.alloc(size_t(T2.stride) * R));
  FCG_CUDA(T2.fac.alloc(size_t(T2.n_fac)));
  FCG_CUDA(T2.rank.alloc(size_t(std::max<int64_t>(ng, 1)) * N));
  {
    DevBuf<int64_t> d_gptr, d_gwork, d_gbuf;
    DevBuf<int32_t> d_gmem;
    DevBuf<double> d_work;
    FCG_CUDA(d_gptr.upload(gptr.data(), gptr.size(), ctx->stream));
    FCG_CUDA(d_gmem.upload(gmem.data(), gmem.size(), ctx->stream));
    FCG_CUDA(d_gwork.upload(gwork.data(), gwork.size(), ctx->stream));
    FCG_CUDA(d_gbuf.upload(gbuf.data(), gbuf.size(), ctx->stream));
    FCG_CUDA(d_work.alloc(size_t(std::max<int64_t>(wtot, 1))));
    size_t smem = 0;
    FCG_REQUIRE(!cta_smem(tucker_add_kernel, int(gdmax), &smem), FCG_ECUDA, "FOIS: shared memory attribute");
    tucker_add_kernel<<<unsigned(ng), kCtaThreads, smem, ctx->stream>>>(
        int(ng), N, R, 1e-10, d_gptr.p, d_gmem.p, T1.d_desc.p, T1.stride, T1.core.p, T1.fac.p, T1.rank.p,
        T2.d_desc.p, T2.stride, T2.core.p, T2.fac.p, T2.rank.p, d_work.p, d_gwork.p, d_gbuf.p, int64_t(d_work.n),
        int(gdmax), d_err.p);
    FCG_CUDA(cudaGetLastError());
    const int rc = check_err();  // waits for the launch before its buffers are freed
    if (rc) return rc;
  }
  // 6. compress each target block (compress_twice), then the whole space until its length
  //    stops falling (compress_iteratively: at least one pass)
  TuckBatch A, B;
  TuckBatch* cur = &T2;
  if (compress_twice) {
    const int rc = run_compress(ctx, N, R, thresh, T2, T2.rank.p, A, work, d_err.p);
    if (rc) return rc;
    cur = &A;
  }
  std::vector<int32_t> rk(size_t(ng) * N);
  auto length_of = [&](TuckBatch* b) -> int64_t {
    if (cudaMemcpyAsync(rk.data(), b->rank.p, sizeof(int32_t) * rk.size(), cudaMemcpyDeviceToHost, ctx->stream) !=
            cudaSuccess ||
        cudaStreamSynchronize(ctx->stream) != cudaSuccess)
      return -1;
    int64_t tot = 0;
    for (int64_t g = 0; g < ng; ++g) {
      int64_t l = 1;
      for (int c = 0; c < N; ++c) l *= rk[size_t(g * N + c)];
      tot += l;
    }
    return tot;
  };
  int64_t len0 = length_of(cur);
  FCG_REQUIRE(len0 >= 0, FCG_ECUDA, "FOIS: rank read-back failed");
  for (int pass = 0; pass < 20; ++pass) {
    TuckBatch* next = (cur == &A) ? &B : &A;
    const int rc = run_compress(ctx, N, R, thresh, *cur, cur->rank.p, *next, work, d_err.p);
    if (rc) return rc;
    const int64_t len1 = length_of(next);
    FCG_REQUIRE(len1 >= 0, FCG_ECUDA, "FOIS: rank read-back failed");
    cur = next;
    if (!(len1 < len0)) break;
    len0 = len1;
  }
  {
    const int rc = check_err();
    if (rc) return rc;
  }
  // 7. the result in the fcg_bst_set layout, empty blocks dropped
  std::vector<double> hcore(size_t(cur->stride) * R), hfac(size_t(cur->n_fac));
  FCG_CUDA(cudaMemcpyAsync(hcore.data(), cur->core.p, sizeof(double) * hcore.size(), cudaMemcpyDeviceToHost,
                           ctx->stream));
  FCG_CUDA(cudaMemcpyAsync(hfac.data(), cur->fac.p, sizeof(double) * hfac.size(), cudaMemcpyDeviceToHost, ctx->stream));
  FCG_CUDA(cudaStreamSynchronize(ctx->stream));
  auto& F = ctx->fois;
  std::vector<std::vector<double>> rc_cores(static_cast<size_t>(R));
  for (int64_t g = 0; g < ng; ++g) {
    int64_t l = 1;
    for (int c = 0; c < N; ++c) l *= rk[size_t(g * N + c)];
    if (l == 0) continue;
    const TuckDesc& d = cur->desc[size_t(g)];
    F.fock.insert(F.fock.end(), gfock[size_t(g)].begin(), gfock[size_t(g)].end());
    for (int c = 0; c < N; ++c) F.blocks.push_back(rk[size_t(g * N + c)]);
    for (int c = 0; c < N; ++c) F.blocks.push_back(granges[size_t(g)][size_t(c)]);
    for (int c = 0; c < N; ++c) F.blocks.push_back(granges[size_t(g)][size_t(N + c)]);
    for (int c = 0; c < N; ++c) {
      F.factor_off.push_back(int64_t(F.factors.size()));
      const int64_t fl = int64_t(d.dim[c]) * rk[size_t(g * N + c)];
      F.factors.insert(F.factors.end(), hfac.begin() + d.fac_off[c], hfac.begin() + d.fac_off[c] + fl);
    }
    for (int r = 0; r < R; ++r)
      rc_cores[size_t(r)].insert(rc_cores[size_t(r)].end(), hcore.begin() + r * cur->stride + d.core_off,
                                 hcore.begin() + r * cur->stride + d.core_off + l);
    F.core_total += l;
    ++F.n_blocks;
  }
  for (int r = 0; r < R; ++r) F.cores.insert(F.cores.end(), rc_cores[size_t(r)].begin(), rc_cores[size_t(r)].end());
  *out_n_blocks = F.n_blocks;
  *out_core_total = F.core_total;
  *out_n_factors = int64_t(F.factors.size());
  ctx->stats.bst_fois_items = n_items;
  ctx->stats.bst_fois_seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  return FCG_OK;
}

int fcg_bst_fois_get(fcg_ctx* ctx, int16_t* fock, int64_t* blocks, int64_t* factor_off, double* factors,
                     double* cores) {
  if (!ctx) return FCG_EINVAL;
  const auto& F = ctx->fois;
  if (F.n_blocks == 0) return FCG_OK;
  FCG_REQUIRE(fock && blocks && factor_off && factors && cores, FCG_EINVAL, "null pointer");
  std::memcpy(fock, F.fock.data(), sizeof(int16_t) * F.fock.size());
  std::memcpy(blocks, F.blocks.data(), sizeof(int64_t) * F.blocks.size());
  std::memcpy(factor_off, F.factor_off.data(), sizeof(int64_t) * F.factor_off.size());
  std::memcpy(factors, F.factors.data(), sizeof(double) * F.factors.size());
  std::memcpy(cores, F.cores.data(), sizeof(double) * F.cores.size());
  return FCG_OK;
}

}  // extern "C"
