/*
 * fcg_gpu.h -- C ABI of the GB300 TPSCI sigma build (libfcg_gpu.so).
 *
 * The library replaces the hot path of FermiCG's tensor-product-state CI:
 * the sigma build sigma = H c over a ClusteredOperator, for TPSCIstate vectors.
 * Every entry point takes plain pointers and sizes, returns an int status
 * (FCG_OK = 0, negative on error; fcg_last_error() gives the message) and
 * never throws.  A context owns one GPU stream and all device memory; it is
 * not thread-safe (one context per host thread, or serialise calls).
 *
 * Layouts (all integers little-endian, all indices 0-based):
 *   op block table  int64 [n_blocks][10] = {cluster, op_id, fb_a, fb_b, fk_a, fk_b,
 *                   n_idx, m_bra, m_ket, offset}; block element (p, I, J) is
 *                   data[offset + p + n_idx*(I + m_bra*J)]  (Julia column-major
 *                   (orbital-multi-index, I, J) of build_local_quantities.jl:176-188).
 *                   op ids: 0..21 = A a B b AA aa BB bb Aa Bb Ab Ba AB ab AAa Aaa BBb Bbb
 *                   ABa Aba ABb Bba, 22 = "H", 23 = "Hcmf".
 *   term table      int32 [n_terms][28] = {nbody, transfer_id, cluster[4], op[4],
 *                   delta_a[4], delta_b[4], parity[4], dim[4], ints_off_lo, ints_off_hi};
 *                   a term's integrals are ints[off ...] flattened column-major.
 *   transfers       int16 [n_transfers][n_clusters][2]  (TransferConfig).
 *   state           fock int16 [n_cfg][n_clusters][2], cfg int16 [n_cfg][n_clusters]
 *                   (ClusterConfig minus one); rows of one Fock sector contiguous,
 *                   in TPSCIstate (get_vector) order.
 *   coefficients    float64 column-major [R][n_cfg] (Julia Matrix{Float64}(n_cfg, R)).
 * Limits: n_clusters <= 8, local states per sector <= 256, orbitals per cluster <= 15.
 */
#ifndef FCG_GPU_H
#define FCG_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FCG_OK 0
#define FCG_EINVAL -1
#define FCG_ECUDA -2
#define FCG_ENOMEM -3
#define FCG_ESTATE -4
#define FCG_ETIMEDOUT -5
#define FCG_ELIMIT -6

#define FCG_FP64 0  /* all arithmetic in float64 */
#define FCG_FP32 1  /* contractions in float32 with float32 accumulation ("mixed") */

typedef struct fcg_ctx fcg_ctx;

typedef struct fcg_stats {
  int64_t n_cfg;
  int64_t n_sectors;
  int64_t n_work_items;     /* (bra group, ket group, term list) blocks of the closed sigma */
  int64_t n_triples;        /* (bra, ket, term) contractions of one closed sigma */
  int64_t flops_reference;  /* sum over triples of 2*len(ints) (the reference's count) */
  int64_t flops_executed;   /* 2 x multiply-adds the dressed contraction does per sigma (R update excluded) */
  int64_t dressed_elements; /* elements of the dressed operators W (one copy per precision) */
  double plan_seconds;      /* host time of the last fcg_state_set */
  double last_kernel_ms;    /* device time of the last sigma kernel(s) (CUDA events) */
  int64_t kernel_launches;  /* kernels launched by the last sigma call */
  int64_t open_jobs;        /* (ket, term) pairs of the last open sigma */
  int64_t open_jobs_kept;   /* of those, the ones the screen kept */
  int64_t open_contractions;/* (ket, term, bra tuple) elements evaluated */
  int64_t davidson_sigma_calls; /* sigma builds of the last fcg_davidson */
  int64_t bst_blocks;       /* Tucker blocks of the last fcg_bst_set */
  int64_t bst_triples;      /* (bra block, ket block, term) triples passing check_term */
  int64_t bst_groups;       /* (bra block, ket block, active clusters) groups = cached operators */
  int64_t bst_cache_elements; /* elements of the cached group operators */
  int64_t bst_flops_reference; /* per root: sum over triples of 2*m*k*n + spectator transforms (reference count) */
  int64_t bst_flops_executed;  /* per root: the same sums over groups (what one fcg_bst_sigma root does) */
  double bst_cache_seconds; /* wall time of the last fcg_bst_set (planning + operator cache) */
  double bst_plan_seconds;  /* of which host planning (triples, groups, cache layout) */
  int64_t bst_fois_items;   /* (term, ket block, target TuckerConfig) contributions of the last fcg_bst_fois */
  double bst_fois_seconds;  /* wall time of the last fcg_bst_fois */
  int64_t group_rounds;     /* lockstep rounds of the last fcg_davidson_grouped (first context; longest lane) */
  int64_t group_launches;   /* kernels those rounds launched, all lanes (grouped sigma: 3) */
  double group_setup_seconds; /* its problems' set-up: buffers, diagonals, guesses */
  double group_step_seconds;  /* host work of the rounds (problems stepped in parallel) */
  double group_issue_seconds; /* descriptors, copies and launches of the rounds */
  double group_wait_seconds;  /* sigma builds and waits for the stream */
  int64_t hcache_pairs;     /* (work item, bra, ket) pairs of the stored Hamiltonian blocks */
  int64_t hcache_bytes;     /* device bytes they take (float64 and float32 copies, index) */
  double hcache_seconds;    /* wall time of the last fcg_cache_hamiltonian */
  double open_expand_ms;    /* device time of the expansion kernel of the last open sigma (CUDA events) */
  int64_t open_flops_reference; /* the reference's GEMM flops of the last open sigma's jobs (no prescreen) */
  int64_t open_bytes;       /* its compulsory bytes: TDM blocks touched, C, output rows */
  double tune_seconds;      /* host time spent timing closed-sigma kernel candidates */
  int64_t tune_cache_hits;  /* tunings answered from the process's shape cache */
  int64_t bst_tc_groups;    /* groups of the last float BST sigma that ran on the tensor cores */
  int64_t bst_tc_flops;     /* their algorithmic flops (2 m k n per root) */
  int64_t bst_tc_mma_flops; /* flops the MMAs executed (3 TF32 products, tiles padded) */
  double bst_tc_ms;         /* device time of the tensor-core GEMM kernel (CUDA events) */
  double join_seconds;      /* wall time of the last closed-sigma join (part of plan_seconds) */
  int64_t join_on_device;   /* 1: that join ran on the device (the default), 0: on the host */
} fcg_stats;

int fcg_version(void);

/* Create a context on CUDA device `device` (replaces nothing: setup). */
int fcg_ctx_create(int device, fcg_ctx** out);
int fcg_ctx_destroy(fcg_ctx* ctx);
const char* fcg_last_error(const fcg_ctx* ctx);

/* Run all later calls of this context on `stream` (a cudaStream_t of the
 * context's device, owned by the caller); NULL returns to the context's own
 * stream.  Calls still synchronise before returning. */
int fcg_set_stream(fcg_ctx* ctx, void* stream);

/* ClusterOps upload: Vector{ClusterOps} of compute_cluster_ops
 * (src/build_local_quantities.jl:40-191, type src/type_ClusterOps.jl:1). */
int fcg_set_ops(fcg_ctx* ctx, int n_clusters, const int32_t* cluster_norb, int64_t n_blocks,
                const int64_t* block_table, int64_t n_data, const double* data);

/* ClusteredOperator upload: the Dict{TransferConfig, Vector{ClusteredTerm}} of
 * extract_ClusteredTerms (src/type_ClusteredOperator.jl:5, 53-636). */
int fcg_set_terms(fcg_ctx* ctx, int n_terms, const int32_t* term_table, int64_t n_ints,
                  const double* ints, int n_transfers, const int16_t* transfers);

/* TPSCIstate structure (src/type_TPSCIstate.jl:11-14): uploads the rows and
 * builds the device index used by every sigma call on this state. */
int fcg_state_set(fcg_ctx* ctx, int64_t n_cfg, const int16_t* fock, const int16_t* cfg);

/* The rows of a TPSCIstate and its Fock sectors only (no closed-sigma plan yet): enough for
 * fcg_diagonal and fcg_sigma_open, as compute_diagonal (src/tpsci_outer.jl:694-787) and
 * open_matvec_thread need.  A later closed sigma, cache or Davidson call on the state builds
 * the plan first; fcg_sigma_closed_noalloc needs fcg_state_set (it allocates nothing). */
int fcg_state_rows(fcg_ctx* ctx, int64_t n_cfg, const int16_t* fock, const int16_t* cfg);

/* tps_ci_matvec (src/tpsci_outer.jl:462-527): sigma = H c within the state's
 * configurations.  Host buffers, column-major n_cfg x R; copies in and out
 * inside the call.  precision: FCG_FP64 or FCG_FP32. */
int fcg_sigma_closed(fcg_ctx* ctx, int R, const double* c, double* sigma, int precision);

/* Same, on device buffers (column-major n_cfg x R float64) already resident
 * on the context's device; runs on the context stream and synchronises. */
int fcg_sigma_closed_device(fcg_ctx* ctx, int R, const double* d_c, double* d_sigma, int precision);

/* compute_expectation_value_parallel (src/tpsci_outer.jl:601-687): e[r] = c_r^T H c_r for
 * the state's configurations (c: host, column-major n_cfg x R; not normalised, as in the
 * reference). */
int fcg_expectation(fcg_ctx* ctx, int R, const double* c, double* e, int precision);

/* build_full_H_parallel (src/tpsci_outer.jl:59-150) with the same state on both sides:
 * the dense n_cfg x n_cfg H (host, column-major), built from closed sigmas of identity
 * blocks in float64; n_cfg <= 65536. */
int fcg_build_full_h(fcg_ctx* ctx, double* H);

/* compute_diagonal (src/tpsci_outer.jl:694-715) when op_id < 0 (all zero-transfer
 * terms, bra == ket), else compute_diagonal! with that op string
 * (src/tpsci_outer.jl:735-757, e.g. op_id 23 = "Hcmf").  hd: host, n_cfg. */
int fcg_diagonal(fcg_ctx* ctx, int op_id, double* hd);

/* open_matvec_thread (src/tpsci_matvec_thread.jl:11-129): sigma over the first-order
 * interacting space of the state's configurations, keeping each (ket, term, bra)
 * contribution x with |x| > thresh / max_r |c_ket[r]| (_collect_significant_thread!,
 * :830-885), terms of at most `nbody` clusters.  c: host, column-major n_cfg x R.
 * Returns the number of output configurations in *n_out; fetch them with
 * fcg_sigma_open_fetch.  Output order is unspecified (as in the reference). */
int fcg_sigma_open(fcg_ctx* ctx, int R, const double* c, double thresh, int nbody, int64_t* n_out);

/* Rows of the last fcg_sigma_open: fock int16 [n_out][N][2], cfg int16 [n_out][N],
 * coeff float64 column-major n_out x R. */
int fcg_sigma_open_fetch(fcg_ctx* ctx, int16_t* fock, int16_t* cfg, double* coeff);

/* The Davidson solve of tps_ci_davidson (src/tpsci_outer.jl:364-454; BlockDavidson
 * Davidson(Hmap; v0, max_iter, max_ss_vecs, nroots=R, tol, lindep_thresh) + eigs with
 * Adiag = compute_diagonal): lowest R eigenpairs of H within the state's configurations.
 * v0, vectors: host column-major n_cfg x R; energies, residuals: R; tol is the residual
 * norm.  precision FCG_FP64, or FCG_FP32 = float32 sigma builds until the largest residual
 * is below max(tol, 1e-5, 5e-7 * max|theta|) (the float32 sigma's residual floor) or has
 * not fallen by 10% in 5 iterations while below 1e-3, then float64 sigma builds to tol.  precond: 1 = diagonal
 * preconditioner.  Subspace holds at most max_ss_vecs * R vectors. */
int fcg_davidson(fcg_ctx* ctx, int R, const double* v0, int max_iter, int max_ss_vecs, double tol, double lindep,
                 int precision, int precond, double* energies, double* vectors, double* residuals, int* iters);

/* The Davidson solve of the BST ci_solve (src/tucker_outer.jl:68-215, BlockDavidson with the
 * build_sigma! matvec of :101-112) on the device: R lowest eigenpairs of H over the cores of
 * the last fcg_bst_set (vector length core_total, [R][core_total] for v0 and vectors, like
 * fcg_bst_sigma).  hdiag (core_total values, or NULL) is the preconditioner diagonal (the
 * reference's precond option passes its Hcmf diagonal); NULL runs unpreconditioned (the
 * reference's precond = false).  Settings, precision and results as fcg_davidson; FCG_FP32
 * builds every sigma but the final refinements in float32, its GEMM-shaped groups on the
 * tensor cores. */
int fcg_bst_davidson(fcg_ctx* ctx, int R, const double* v0, const double* hdiag, int max_iter, int max_ss_vecs,
                     double tol, double lindep, int precision, double* energies, double* vectors,
                     double* residuals, int* iters);

/* The Davidson solves of n independent problems (one context each, state set) in lockstep:
 * every problem runs fcg_davidson's algorithm on its lane's stream (below).  In each round
 * every problem advances to its next need of the device (host work on a thread pool); then
 * all their Gram products, Ritz/residual passes, orthonormalisation and restart updates run
 * as one launch per kernel and block width and step, the fetched values come back in one
 * copy, the sigma builds of their new blocks run as one grouped launch
 * (fcg_sigma_closed_grouped) per precision, and the round ends with one wait.  From 64
 * problems on, the problems are dealt round-robin to up to 4 lanes, each a lockstep group on
 * its first problem's stream with a host thread of its own, so that lanes overlap one
 * another's host and device work.  The reference solves independent
 * problems one after another (tps_ci_davidson, src/tpsci_outer.jl:364-454, per problem).
 * Per problem q: R[q] roots, v0[q] / vectors[q] host column-major n_cfg_q x R[q],
 * energies[q], residuals[q], iters[q]; the settings are shared.  All contexts on one device
 * and distinct; errors name the problem. */
int fcg_davidson_grouped(int n, fcg_ctx* const* ctxs, const int* R, const double* const* v0, int max_iter,
                         int max_ss_vecs, double tol, double lindep, int precision, int precond,
                         double* const* energies, double* const* vectors, double* const* residuals, int* iters);

/* ---- serving: continuous batching of Davidson solves ---------------------------------
 * A server owns `lanes` scheduler threads on `device`, each with a stream of its own (lanes
 * is clipped to max_active).  The caller prepares one context per request (fcg_set_ops,
 * fcg_set_terms, fcg_state_set, in any thread) and submits it with a guess; a lane admits
 * requests while it runs fewer than ceil(max_active / lanes), the server fewer than
 * max_active, and their device memory (Davidson subspace and sigma copies) fits
 * memory_budget bytes (a larger request runs when nothing else does).  Each lane runs its
 * solves in lockstep rounds as fcg_davidson_grouped does: finished solves leave and queued
 * ones join between rounds, so their sigma builds are grouped per iteration, while the lanes
 * overlap one another's kernels and host work.  A
 * submitted context belongs to the server until its ticket is waited for.  fcg_poll: state
 * 0 queued, 1 running, 2 done, 3 failed.  fcg_wait returns FCG_ETIMEDOUT after timeout_ms
 * (0: just look) and never blocks longer; on success it copies the results (energies R,
 * vectors column-major n_cfg x R, residuals R, iterations; any may be null) and retires the
 * ticket; a failed solve returns its error code with the message in fcg_last_error(ctx).
 * A finished ticket holds its result vectors on the host until it is waited for: a caller
 * that polls or abandons requests retires each one with fcg_wait (null outputs drop the
 * results), or the results stay until fcg_server_destroy.
 * fcg_server_destroy fails the queued requests, lets the running ones finish (each is
 * bounded by its max_iter) and must come after the last wait.  The reference has no
 * serving loop: each request is the tps_ci_davidson solve of fcg_davidson. */
typedef struct fcg_server fcg_server;
int fcg_server_create(int device, int max_active, int lanes, double memory_budget, fcg_server** out);
int fcg_server_destroy(fcg_server* s);
int fcg_submit(fcg_server* s, fcg_ctx* ctx, int R, const double* v0, int max_iter, int max_ss_vecs, double tol,
               double lindep, int precision, int precond, int64_t* ticket);
/* A BST solve (fcg_bst_davidson's arguments) as a request: the context's fcg_bst_set
 * structure is the problem; the results come back through fcg_wait (vectors core_total x R). */
int fcg_submit_bst(fcg_server* s, fcg_ctx* ctx, int R, const double* v0, const double* hdiag, int max_iter,
                   int max_ss_vecs, double tol, double lindep, int precision, int64_t* ticket);
int fcg_poll(fcg_server* s, int64_t ticket, int* state);
int fcg_wait(fcg_server* s, int64_t ticket, int timeout_ms, double* energies, double* vectors, double* residuals,
             int* iters);

/* Stored Hamiltonian blocks of the state: the TPSCI analogue of cache_hamiltonian
 * (src/tucker_inner.jl:90-159, which stores dense operator blocks for the BST sigma).  For
 * every work item of the closed sigma (a bra group, a ket group and the terms coupling them,
 * the job structure of tps_ci_matvec, src/tpsci_outer.jl:462-527) the matrix element
 * <bra|H|ket> of each of its (bra, ket) pairs, summed over the item's terms in float64, is
 * computed once and kept on the device (float64 and float32 copies).  Every later closed
 * sigma of this state -- fcg_sigma_closed*, fcg_davidson, fcg_davidson_grouped,
 * fcg_sigma_closed_grouped, fcg_build_full_h, fcg_expectation -- then reads those values
 * instead of contracting every (bra, ket, term) triple again.  Float64 results equal the
 * direct build up to the order of the additions; float32 results are closer to float64
 * than the direct float32 build (the term sums are rounded once).  The blocks take 12 bytes
 * per pair: *bytes returns the need; FCG_ELIMIT (nothing stored) when it exceeds max_bytes.
 * max_bytes <= 0 drops them and frees their memory.  fcg_set_ops, fcg_set_terms and
 * fcg_state_set drop them too but keep the memory for the context's next stored blocks.
 * The Davidson working buffers of a context likewise stay allocated for its next solve
 * (a freed buffer would make the call wait for every stream of the device). */
int fcg_cache_hamiltonian(fcg_ctx* ctx, double max_bytes, int64_t* bytes);

int fcg_get_stats(const fcg_ctx* ctx, fcg_stats* out);

/* The closed sigma (tps_ci_matvec, src/tpsci_outer.jl:462-527) of n independent problems in
 * one grouped launch: problem q lives in ctxs[q] (ops, terms and state set), with R[q] roots
 * and device buffers d_c[q] / d_sigma[q] (column-major n_cfg_q x R[q] float64).  The
 * reference runs independent problems one after another; here every problem's triples are
 * CTAs of one grid (plus one pack and one unpack launch), on ctxs[0]'s stream.  All
 * contexts must be on one device and distinct; the call synchronises.  Timing and launch
 * counts go to ctxs[0]'s stats. */
int fcg_sigma_closed_grouped(int n, fcg_ctx* const* ctxs, const int* R, const double* const* d_c,
                             double* const* d_sigma, int precision);

/* ---- block-sparse Tucker (BST) vectors ----------------------------------------------
 * A BSTstate (src/type_BSTstate.jl:13-18) is flattened to blocks, one per (FockConfig,
 * TuckerConfig) in iteration order:
 *   fock     int16 [n_blocks][N][2]
 *   blocks   int64 [n_blocks][3N] = {rank[N], range_start[N] (0-based), range_len[N]}
 *            (the TuckerConfig UnitRanges and the Tucker ranks)
 *   factor_off int64 [n_blocks][N]: offset in `factors` of each (range_len x rank) factor,
 *            column-major (Tucker.factors)
 *   cores    float64 [R][core_total]: each block's core (rank_1 x ... x rank_N, column-major,
 *            cluster 0 fastest) at the block's core offset; blocks are concatenated in order,
 *            so block b starts at sum_{b' < b} prod(rank of b').
 * fcg_bst_set plans the (bra block, ket block, term) triples of build_sigma!
 * (src/tucker_inner.jl:165-245: check_term on TuckerConfigs, terms of at most `nbody`
 * clusters) and builds every dense term operator in the Tucker bases once, as
 * cache_hamiltonian does (src/tucker_inner.jl:90-159, build_dense_H_term
 * src/tucker_build_dense_H_term.jl:5-175).  Terms that couple the same two blocks
 * through the same active clusters share one cached operator (their sign-weighted sum).
 * The operators, terms and op blocks of this context must be set.  *core_total receives
 * the core length of one root. */
int fcg_bst_set(fcg_ctx* ctx, int nbody, int64_t n_blocks, const int16_t* fock, const int64_t* blocks,
                const int64_t* factor_off, int64_t n_factors, const double* factors, int64_t* core_total);

/* build_sigma! with the cache (src/tucker_inner.jl:165-245, form_sigma_block! :253-304,
 * contract_dense_H_with_state src/tucker_contract_dense_H_with_state.jl:4-330):
 * sigma = H * cores over the blocks of the last fcg_bst_set (sigma is overwritten; the
 * reference adds into a zeroed sigma).  Host buffers [R][core_total].  precision:
 * FCG_FP64, or FCG_FP32 (float32 operators, cores and accumulation).  In FCG_FP32 the
 * groups whose op2^T * ket2 product is GEMM-shaped (at least 64 bra-active rows, 16
 * ket-active columns and 32 spectator columns over all roots) run on the tcgen05 tensor
 * cores: three TF32 products per operand pair (each operand split into a TF32 high part
 * and a TF32 remainder) accumulated in FP32, about FP32 accuracy. */
int fcg_bst_sigma(fcg_ctx* ctx, int R, const double* cores, double* sigma, int precision);

/* Same on device buffers [R][core_total] float64 of the context's device. */
int fcg_bst_sigma_device(fcg_ctx* ctx, int R, const double* d_cores, double* d_sigma, int precision);

/* FCG_FP32 BST sigma: GEMM-shaped groups on the tensor cores (enable = 1, the default) or
 * every group on the CUDA cores (0).  No counterpart in the reference (its GEMMs are BLAS
 * calls); fcg_stats reports the groups, flops and kernel time of the tensor-core part. */
int fcg_bst_tensor_cores(fcg_ctx* ctx, int enable);

/* fcg_bst_set for build_sigma! between two different BST states (src/tucker_inner.jl:165-245
 * with sigma_vector and ci_vector distinct): blocks [0, n_first) are one state, blocks
 * [n_first, n_blocks) the other, and only the triples that couple a block of one state with a
 * block of the other are planned (both directions), so one fcg_bst_sigma gives <A|H|B> and
 * <B|H|A> without the couplings inside either state. */
int fcg_bst_set_between(fcg_ctx* ctx, int nbody, int64_t n_first, int64_t n_blocks, const int16_t* fock,
                        const int64_t* blocks, const int64_t* factor_off, int64_t n_factors, const double* factors,
                        int64_t* core_total);

/* The triples of the last fcg_bst_set: int32 [bst_triples][4] = {bra block, ket block,
 * term index (term-table row), state sign}. */
int fcg_bst_triples(fcg_ctx* ctx, int32_t* out);

/* The compressed first-order interacting space of a BST state: build_compressed_1st_order_state
 * (src/tucker_outer.jl:717-910) with form_sigma_block_expand (src/tucker_form_sigma_block_expand.jl
 * :7-722; 3- and 4-body local operators truncated by SVD, precontract = true), the HOSVD
 * compressions (compress, src/hosvd.jl:337-349) and nonorth_add (src/hosvd.jl:83-156), and a
 * final compress_iteratively (src/type_BSTstate.jl:283-296).  The state is given in the
 * fcg_bst_set layout with R roots of cores [R][core_total]; `spaces` holds each cluster's P and Q
 * ranges per local Fock sector, int32 [N][nmax+1][nmax+1][4] = {p_start, p_len, q_start, q_len}
 * (0-based, length 0: absent), as BSTstate.p_spaces / q_spaces.  thresh is the reference's
 * `thresh` (HOSVD threshold and prescreen), compress_twice its flag.  The result stays in the
 * context; its sizes go to *out_n_blocks, *out_core_total (per root) and *out_n_factors, and
 * fcg_bst_fois_get copies it out.  The context's BST structure (fcg_bst_set) is replaced by the
 * expansion's. */
int fcg_bst_fois(fcg_ctx* ctx, int R, int nbody, double thresh, int compress_twice, int64_t n_blocks,
                 const int16_t* fock, const int64_t* blocks, const int64_t* factor_off, int64_t n_factors,
                 const double* factors, const double* cores, const int32_t* spaces, int64_t* out_n_blocks,
                 int64_t* out_core_total, int64_t* out_n_factors);

/* The last fcg_bst_fois result in the fcg_bst_set layout: fock [n][N][2], blocks [n][3N]
 * {rank, start, len}, factor_off [n][N], factors [n_factors], cores [R][core_total]. */
int fcg_bst_fois_get(fcg_ctx* ctx, int16_t* fock, int64_t* blocks, int64_t* factor_off, double* factors,
                     double* cores);

/* Closed-sigma kernel tuning (no counterpart in the reference: its matvec has no kernel
 * variants).  The library has four candidates per precision (two occupancy targets x two
 * chunk granularities of the lane kernel).  With mode -1 (the default) the first timed sigma
 * of each precision on a state runs every candidate once, keeps the fastest for the context
 * and remembers it for later states of the same shape (configurations, terms, triples) in
 * this process; 0..3 forces a candidate.  fcg_state_set clears the choice.  fcg_tuning
 * reports the candidate in use per precision (chosen[0] double, chosen[1] float; -1: not
 * tuned yet) and, when candidate_ms is given (8 floats), the timings of the last tuning. */
int fcg_set_tuning(fcg_ctx* ctx, int mode);

/* Where the closed-sigma join of the next plan runs (no counterpart in the reference: its
 * check_term filter runs per (bra, ket, term) in tps_ci_matvec, src/tpsci_outer.jl:462-527).
 * on_device = 1 (the default): spectator-key radix sorts, a sector hash table and the joins
 * in device kernels; 0: the host planner (C++/OpenMP), kept as its reference.  Both give
 * bit-identical plans.  The state's plan is rebuilt on its next use. */
int fcg_set_planner(fcg_ctx* ctx, int on_device);

/* The state's closed-sigma plan, for tests and inspection (builds it when needed).
 * fcg_plan_sizes: sizes[0] permutation-pool entries (int32), [1] term-sector records
 * (72 bytes), [2] lane jobs (16 bytes, idle lanes included), [3] warp-chunk table entries
 * (int64, chunks + 1), [4] work items.  fcg_plan_copy copies array `which` (0..3 as above;
 * 4: the chunk table's first stored values, int64) to host memory of `bytes` bytes. */
int fcg_plan_sizes(fcg_ctx* ctx, int64_t* sizes);
int fcg_plan_copy(fcg_ctx* ctx, int which, void* dst, int64_t bytes);
int fcg_tuning(const fcg_ctx* ctx, int* chosen, float* candidate_ms);

/* Allocation-free variant of fcg_sigma_closed_device (no counterpart in the reference).
 * For callers that cannot call cudaMalloc/cudaFree during a solve: applications whose
 * device memory is owned by their own pool allocator or held to a fixed budget, and
 * loops driving several streams that cannot afford the device-wide synchronisation
 * cudaFree implies.  Same arguments and results as fcg_sigma_closed_device; the working
 * copies of C and sigma live in a fixed 16 MiB device array built into the library
 * (placed on a device when the library's device code is first used there, and held until
 * exit), so n_cfg * R must not exceed 1048576 (FCG_ELIMIT otherwise).  The state,
 * operators and terms must already be set.  The first call on a device looks up the
 * array's device address (cudaGetSymbolAddress) and keeps it for the life of the process:
 * that first call should come before any stream capture, and the device's primary context
 * must not be reset (cudaDeviceReset) while the library is in use.  Like the other sigma
 * calls it waits for its stream before returning.  All calls on one device share the
 * array: calls that overlap on the GPU race and must be serialised by the caller. */
int fcg_sigma_closed_noalloc(fcg_ctx* ctx, int R, const double* d_c, double* d_sigma, int precision);

#ifdef __cplusplus
}
#endif
#endif /* FCG_GPU_H */
