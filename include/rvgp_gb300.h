/*
 * librvgp_gb300 — C ABI of the GB300 (sm_103a) RVGP numerical core.
 *
 * Conventions for every entry point:
 *  - pointers are device pointers unless stated; the caller owns all memory;
 *  - `stream` is a cudaStream_t passed as void*; work is stream-ordered and
 *    asynchronous unless a function says it synchronises;
 *  - functions that need scratch take (workspace, ws_bytes) and have a
 *    matching *_workspace() size query;
 *  - return 0 on success, > 0 for numerical information (documented per
 *    function), < 0 for bad arguments (-1), launch failures (-2), short
 *    workspace (-3) or unsupported sizes (-4); rvgp_last_error() gives the
 *    message of the last failure on the calling host thread.
 *
 * Reference paths below are inside the agosztolai/RVGP checkout.
 */
#ifndef RVGP_GB300_H
#define RVGP_GB300_H
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

const char* rvgp_last_error(void);
int rvgp_abi_version(void);
/* Kernels launched by this library since it was loaded (all host threads). */
long long rvgp_launch_count(void);

/* ---- graph ------------------------------------------------------------ */

/* Exact kNN, FP64 distances, ties to the lower index, self excluded.
 * Replaces sklearn.neighbors.kneighbors_graph(X, k, mode='connectivity',
 * include_self=False) at RVGP/geometry.py:103-110.  X: (n, D) f64 row-major;
 * idx: (n, k) int32, each row ascending by (distance, index). */
size_t rvgp_knn_workspace(int n, int D, int k);
int rvgp_knn(const double* X, int n, int D, int k, int* idx, void* workspace, size_t ws_bytes, void* stream);
/* rvgp_knn without any device allocation, for callers that cannot allocate
 * device memory when they search (a device-memory budget fixed at start-up,
 * a host framework that owns the memory pool, no allocation latency allowed).
 * No counterpart in the reference.  Scratch is a 32 MiB buffer compiled into
 * the library (held by every GPU that loads it until exit); problems needing
 * more (rvgp_knn_workspace(n, D, k) > 32 MiB) are rejected with an error.
 * The first call on a device caches the buffer's address and should come
 * before any stream capture.  Calls share the buffer: calls that overlap on
 * the GPU race and must be serialised by the caller. */
int rvgp_knn_noalloc(const double* X, int n, int D, int k, int* idx, void* stream);
/* Rows the last rvgp_knn on this workspace settled by the exact fallback scan
 * (synchronises the stream; diagnostics only). */
int rvgp_knn_fallback_rows(int n, int D, int k, void* workspace, void* stream);

/* Symmetrised CSR of kNN + I with sorted columns and unit weights.  Replaces
 * A += I; nx.from_scipy_sparse_array(A) (RVGP/geometry.py:111-112) and the
 * max(A, Aᵀ) symmetrisation of RVGP/lib/ptu_dijkstra.pyx:84-103.
 * indptr: n+1; indices: capacity n*(2k+1); e_out, maxdeg_out: one device int
 * each (stored entries; largest degree without the self-loop). */
size_t rvgp_graph_workspace(int n, int k);
int rvgp_graph_build(const int* knn, int n, int k, int* indptr, int* indices, int* e_out, int* maxdeg_out,
                     void* workspace, size_t ws_bytes, void* stream);

/* Values of L = D - A on that pattern (deg on the diagonal, -1 elsewhere).
 * Replaces nx.laplacian_matrix(G) at RVGP/geometry.py:55-63. */
int rvgp_laplacian_values(const int* indptr, const int* indices, int n, double* vals, void* stream);

/* ---- gauges and connections ------------------------------------------- */

/* Geodesic-neighbourhood local PCA.  Replaces
 * ptu_dijkstra.tangent_frames(X, G, d, K) (RVGP/lib/ptu_dijkstra.pyx:33-125,
 * kernel pyx:300-437).  tangents: (n, D, d_out); sigma: (n, min(D, K+1));
 * nbh_out (optional): (n, K+1) scan order.  status: 3 device ints, left
 * >= n when fine, else [0] = first point whose component has fewer than K+1
 * nodes, [2] = first point whose heap pool overflowed. */
size_t rvgp_gauges_workspace(int n, int D, int K, int maxdeg);
int rvgp_gauges(const double* X, int n, int D, const int* indptr, const int* indices, int K, int maxdeg, int d_out,
                double* tangents, double* sigma, int* nbh_out, int* status, void* workspace, size_t ws_bytes,
                void* stream);

/* Per-edge transports R_ij = polar(T_iᵀ T_j) in CSR order and the block
 * connection Laplacian values (deg R_ii diagonal, -R_ij off-diagonal).
 * Replaces ptu_dijkstra.connections(tangents, G, d) (pyx:128-199, kernel
 * pyx:221-293) and compute_connection_laplacian (RVGP/geometry.py:14-52).
 * T: (n, D, ld) f64 (first d columns used); R, lc64: (E, d, d) f64; lc32:
 * (E, d, d) f32; any output may be null. */
int rvgp_connections(const double* T, int n, int D, int ld, int d, const int* indptr, const int* indices, double* R,
                     double* lc64, float* lc32, void* stream);

/* ---- sparse products -------------------------------------------------- */

/* Y = alpha*(A X) + beta*X + gamma*Z, A block-CSR with DB x DB blocks
 * (DB in 1..4), X/Y/Z (n*DB) x b row-major, leading dimension ld.  b and ld
 * multiples of 4 (f32) or 2 (f64); 16-byte aligned.  The products scipy's
 * eigsh performs inside compute_spectrum (RVGP/geometry.py:73). */
int rvgp_bspmm_f32(int n, int DB, const int* indptr, const int* indices, const float* vals, const float* X, float* Y,
                   const float* Z, int b, int ld, float alpha, float beta, float gamma, void* stream);
int rvgp_bspmm_f64(int n, int DB, const int* indptr, const int* indices, const double* vals, const double* X,
                   double* Y, const double* Z, int b, int ld, double alpha, double beta, double gamma, void* stream);

/* Planned forms of the same product for a matrix used many times (the
 * eigensolver's filter, RVGP/geometry.py:73): a plan built once per matrix
 * holds, per group of 4 consecutive block rows, the merged list of their
 * columns (each shared neighbour's rows are gathered once for the group),
 * and per tile of 32 block rows the distinct columns its entries reference
 * (a shared-memory staged form).  The launch tuner picks among these and the
 * plain variants.  nnz = indptr[n].  Same bits as rvgp_bspmm_*; a null plan
 * runs rvgp_bspmm_*.  On request (RVGP_SPMM_PLAN=1) rvgp_eigsh builds one
 * itself when its workspace has rvgp_spmm_plan_bytes + 256 bytes beyond
 * rvgp_eigsh_workspace; on GB300 both planned forms measure slower than the
 * chunked plain variant at the eigensolver's shapes. */
size_t rvgp_spmm_plan_bytes(int n, int DB, long long nnz);
int rvgp_spmm_plan_build(int n, int DB, const int* indptr, const int* indices, long long nnz, void* plan,
                         size_t plan_bytes, void* stream);
int rvgp_bspmm_planned_f32(const void* plan, size_t plan_bytes, int n, int DB, long long nnz, const int* indptr,
                           const int* indices, const float* vals, const float* X, float* Y, const float* Z, int b,
                           int ld, float alpha, float beta, float gamma, void* stream);
int rvgp_bspmm_planned_f64(const void* plan, size_t plan_bytes, int n, int DB, long long nnz, const int* indptr,
                           const int* indices, const double* vals, const double* X, double* Y, const double* Z, int b,
                           int ld, double alpha, double beta, double gamma, void* stream);

/* Eigendecomposition of a symmetric FP32 matrix (the Rayleigh-Ritz step of the
 * eigensolver; ARPACK's inside scipy's eigsh, RVGP/geometry.py:73): H (p x p,
 * read only) -> w ascending, V (p x p) eigenvectors by column, after at most
 * max_sweeps Jacobi sweeps, stopping at off(H) <= tol ||H||_F; *sweeps_used
 * (host, may be null).  method 0: block Jacobi (32-wide block pairs, two grid
 * barriers per round) for p >= 64, else scalar; 1: scalar parallel Jacobi;
 * 2: block.  Synchronises. */
size_t rvgp_symeig_f32_workspace(int p);
int rvgp_symeig_f32(const float* H, int p, float* w, float* V, int max_sweeps, double tol, int* sweeps_used,
                    int method, void* workspace, size_t ws_bytes, void* stream);

/* ---- eigensolver ------------------------------------------------------ */

/* m smallest eigenpairs of a symmetric PSD block-CSR matrix by Chebyshev-
 * filtered subspace iteration.  Replaces compute_spectrum (ARPACK eigsh,
 * which="SM") at RVGP/geometry.py:66-80 for L and Lc.  mode 0: all FP64;
 * mode 1: FP32 SpMM / tall products (FP64-reduced Grams), FP64 p x p
 * Cholesky and Rayleigh-Ritz, then FP64 refinement.  p: block size
 * (m < p <= n*DB, multiple of 4).  tol / tol32: residual tolerances relative to
 * the Gershgorin bound.  evals ascending (m); evecs N x m (ld_evecs) times
 * `scale` (the reference scales by sqrt(N)).  stats: 16 host ints (iterations,
 * SpMMs, Jacobi sweeps, converged, refinement iterations, Cholesky rescues,
 * 1 when the FP32 Grams and block products ran on the tensor cores (mode 1,
 * p <= 256; RVGP_TENSOR_CORES=0 in the environment selects the CUDA-core
 * kernels), 1 when the shared-memory tiled SpMM ran, then microseconds spent
 * in filter / orthonormalisation / Rayleigh-Ritz tall products / Jacobi,
 * then the number of vectors the FP32 stage locked).  When tol >= tol32
 * (mode 1) no FP64 iteration runs.
 * Returns 0, or the number of unconverged pairs.  Synchronises the stream. */
size_t rvgp_eigsh_workspace(int n, int DB, int m, int p, int mode);
int rvgp_eigsh(const int* indptr, const int* indices, const double* vals64, const float* vals32, int n, int DB, int m,
               int p, int mode, double tol, double tol32, int max_iter, unsigned long long seed, double* evals,
               double* evecs, int ld_evecs, double scale, int* stats, void* workspace, size_t ws_bytes, void* stream);
/* The same solve on a renumbered matrix (rvgp_permute_csr): block row r is the
 * caller's block row perm[r].  The start block is the caller-order one,
 * permuted, and evecs come back in the caller's row order, so the result is
 * rvgp_eigsh's on the original matrix up to summation order. */
int rvgp_eigsh_ordered(const int* indptr, const int* indices, const double* vals64, const float* vals32, int n,
                       int DB, int m, int p, int mode, double tol, double tol32, int max_iter, unsigned long long seed,
                       const int* perm, double* evals, double* evecs, int ld_evecs, double scale, int* stats,
                       void* workspace, size_t ws_bytes, void* stream);

/* ---- tensor-core tall products ----------------------------------------- */

/* Launch-variant autotuner of this library (no counterpart in the reference):
 * kernels with several equivalent launch forms (the block SpMM: row per warp,
 * column-chunked with 2 or 4 neighbours per iteration, all giving the same
 * bits) time them once per shape class and keep the fastest in an on-disk
 * cache ($RVGP_AUTOTUNE_CACHE, else ~/.cache/rvgp_gb300/autotune.txt).
 * cache_path: the file in use; lookup: the cached variant of a key, or -1. */
const char* rvgp_autotune_cache_path(void);
int rvgp_autotune_lookup(const char* key);
/* The eigensolver's FP32 tall products on the tcgen05 tensor cores with
 * split-TF32 operands (x = tf32(x) + remainder; three TF32 products per
 * term, FP32-level accuracy), p, q, K <= 2048 (outputs wider than 256
 * columns run as 256-column blocks of TMEM accumulators).  No reference counterpart: they
 * are the block operations inside the subspace iteration that replaces ARPACK
 * (RVGP/geometry.py:66-80).  Synchronous; a timed-out pipeline wait returns
 * RVGP_ELAUNCH.
 * gram: C (p x q, FP64, ldc) = Aᵀ B, A: N x p (lda), B: N x q (ldb).
 * gemm: C (N x q, ldc) = A (N x K, lda % 4 == 0, 16-byte aligned) Bm (K x q, ldb). */
size_t rvgp_tc_gram_workspace(long long N, int p, int q);
int rvgp_tc_gram_f32(const float* A, int lda, const float* B, int ldb, long long N, int p, int q, double* C, int ldc,
                     void* workspace, size_t ws_bytes, void* stream);
size_t rvgp_tc_gemm_workspace(int K, int q);
int rvgp_tc_gemm_f32(const float* A, int lda, long long N, int K, const float* Bm, int ldb, int q, float* C, int ldc,
                     void* workspace, size_t ws_bytes, void* stream);

/* ---- locality renumbering for the sparse products ---------------------- */

/* perm (n, device): new position -> point, along a Morton curve of the three
 * coordinates of largest extent (10 bits each over the bounding box; ties in
 * point order); rank its inverse.  No reference counterpart: the sparse
 * products of the eigensolves (RVGP/geometry.py:66-80) run on matrices
 * renumbered by it.  Synchronises the stream once. */
size_t rvgp_locality_order_workspace(int n, int D);
int rvgp_locality_order(const double* X, int n, int D, int* perm, int* rank, void* workspace, size_t ws_bytes,
                        void* stream);
/* Block-CSR renumbered by perm/rank: new row r = old row perm[r], columns
 * c -> rank[c], entries of a row in their original order.  vals32 and
 * out_vals32 may be null. */
size_t rvgp_permute_csr_workspace(int n);
int rvgp_permute_csr(int n, int DB, const int* indptr, const int* indices, const double* vals64, const float* vals32,
                     const int* perm, const int* rank, int* out_indptr, int* out_indices, double* out_vals64,
                     float* out_vals32, void* workspace, size_t ws_bytes, void* stream);
/* dst[(i*DB+q), :m] = src[(rank[i]*DB+q), :m]: renumbered rows back to point order. */
int rvgp_unpermute_rows(const double* src, int lds, const int* rank, int n, int DB, int m, double* dst, int ldd,
                        void* stream);

/* ---- spectral kernel and GP ------------------------------------------- */

/* S_l = sigma_f * n_rows * s_l / sum(s), s_l = (λ_l + 2ν/κ²)^(-ν) (typ 0,
 * Matérn) or exp(-λ_l κ²/2) (typ 1, SE), and dS (3 x m) = dS/d(ν, κ, σ_f).
 * theta (device) = [nu, kappa, sigma_f, noise].  tmp3m: 3m doubles scratch.
 * Replaces ManifoldKernel.eval_S (RVGP/kernels.py:41-53). */
int rvgp_spectral_S(const double* evals, int m, const double* theta, double n_rows, int typ, double* S, double* dS,
                    double* tmp3m, void* stream);
/* evecs_Lc[(i*D+a), j] = sum_q T[i,a,q] U[(i*d+q), j]: RVGP/dataclass.py:57-59. */
int rvgp_lift(const double* T, int n, int D, int ld, int d, const double* U, int m, double* out, void* stream);
/* GP rows (point, coordinate) of the selected points, as RVGP/main.py:31,47-50
 * builds them: Phi[(t*D+a), :] = src[(idx[t]*D+a), :], y[(t*D+a)] = vec[idx[t]*D+a]. */
int rvgp_gather_rows(const double* src, int m, int D, const int* idx, int nt, const double* vec, double* Phi,
                     float* Phi32, double* y, void* stream);
/* C = PhiᵀPhi, b = Phiᵀy, yy = yᵀy (mode 1: C from FP32 Phi32, FP64-reduced). */
size_t rvgp_gp_prepare_workspace(long long N, int m);
int rvgp_gp_prepare(const double* Phi, const float* Phi32, const double* y, long long N, int m, int mode, double* C,
                    double* b, double* yy, void* workspace, size_t ws_bytes, void* stream);
/* Log marginal likelihood of GPflow GPR (RVGP/main.py:55-95; training_loss =
 * -LML) with Φ S Φᵀ + σ² I, through the exact rank-m (Woodbury) algebra, and
 * its gradient w.r.t. [nu, kappa, sigma_f, noise].  out (device, 5 doubles);
 * state (device, rvgp_gp_state_size(m) doubles) feeds rvgp_gp_predict.  No
 * host synchronisation. */
size_t rvgp_gp_lml_workspace(int m);
size_t rvgp_gp_state_size(int m);
int rvgp_gp_lml(const double* C, const double* b, const double* yy, long long N, int m, const double* evals,
                double n_rows, int typ, const double* theta, double* out, double* state, void* workspace,
                size_t ws_bytes, void* stream);
/* Hyperparameter learning on the device: `steps` Adam steps on the
 * softplus-unconstrained parameters minimising -LML (the optimisation of
 * RVGP/main.py:77,87-95 with Adam in place of L-BFGS-B), no host
 * synchronisation.  theta0 (device, 4); lower, mask (host, 4 each); theta_out
 * (device, 4); hist (device, steps, optional): LML before each step; out/state
 * as rvgp_gp_lml at theta_out. */
int rvgp_gp_fit_adam(const double* C, const double* b, const double* yy, long long N, int m, const double* evals,
                     double n_rows, int typ, const double* theta0, const double* lower, const int* mask, int steps,
                     double lr, double beta1, double beta2, double eps, double* theta_out, double* hist, double* out,
                     double* state, void* workspace, size_t ws_bytes, void* stream);
/* Mixed-precision form of rvgp_gp_fit_adam (the same Adam steps on the same
 * likelihood, RVGP/main.py:55-95 with GPflow's GPR): the m x m algebra of every
 * step runs in FP32 (Jacobi-scaled capacitance matrix, blocked Cholesky and
 * triangular inverse in one SM's shared memory), all steps in one launch of
 * one CTA; S(θ) and the gradient assembly stay FP64, and out / state are FP64
 * at theta_out.  *status (host): 0 = done, 1 = an FP32 pivot was not positive
 * (nothing written; run rvgp_gp_fit_adam instead).  Requires
 * m <= rvgp_gp_fit_mixed_max_m().  Synchronises the stream. */
int rvgp_gp_fit_mixed_max_m(void);
size_t rvgp_gp_fit_mixed_workspace(int m);
int rvgp_gp_fit_adam_mixed(const double* C, const double* b, const double* yy, long long N, int m,
                           const double* evals, double n_rows, int typ, const double* theta0, const double* lower,
                           const int* mask, int steps, double lr, double beta1, double beta2, double eps,
                           double* theta_out, double* hist, double* out, double* state, int* status, void* workspace,
                           size_t ws_bytes, void* stream);
/* The same in two calls: _launch enqueues the fit without waiting (the host
 * may queue other work, e.g. on another stream, while the one-CTA fit runs);
 * _finish, on the same stream and workspace, waits and sets *status as above. */
int rvgp_gp_fit_adam_mixed_launch(const double* C, const double* b, const double* yy, long long N, int m,
                                  const double* evals, double n_rows, int typ, const double* theta0,
                                  const double* lower, const int* mask, int steps, double lr, double beta1,
                                  double beta2, double eps, double* theta_out, double* hist, void* workspace,
                                  size_t ws_bytes, void* stream);
int rvgp_gp_fit_adam_mixed_finish(const double* C, const double* b, const double* yy, long long N, int m,
                                  const double* evals, double n_rows, int typ, const double* theta_out, double* out,
                                  double* state, int* status, void* workspace, size_t ws_bytes, void* stream);
/* The same C, b, yy for the lifted rows of the training points idx without
 * forming them (the rows built at RVGP/main.py:31,47-50 from
 * evecs_Lc = T_i U_i, RVGP/dataclass.py:57-59): with L_i the Cholesky factor
 * of T_iᵀT_i, the d rows L_iᵀU_i and targets L_i⁻¹T_iᵀy_i give ΦᵀΦ and Φᵀy
 * exactly (d rows per point instead of D); yy sums the full D-vectors.
 * T: n x D x ld gauges (first d <= 8 columns used), U: n*d x m local
 * eigenvectors, vec: n x D vectors. */
size_t rvgp_gp_prepare_local_workspace(int nt, int d, int m, int mode);
int rvgp_gp_prepare_local(const double* T, int n, int D, int ld, int d, const double* U, int m, const int* idx,
                          int nt, const double* vec, int mode, double* C, double* b, double* yy, void* workspace,
                          size_t ws_bytes, void* stream);
/* predict_f(full_cov=False) mean and variance (nt x D each, the reshape of
 * RVGP/main.py:114-116) at the test points idx from the lifted rows' local
 * factors: Q = U_te (r ∘ L_A⁻ᵀ), then per point its d x d Gram of Q rows and
 * the gauge's quadratic forms (d rows per point instead of D). */
size_t rvgp_gp_predict_local_workspace(int nt, int d, int m, int mode);
int rvgp_gp_predict_local(const double* T, int n, int D, int ld, int d, const double* U, int m, const int* idx,
                          int nt, int mode, const double* state, double* mean, double* var, void* workspace,
                          size_t ws_bytes, void* stream);
/* R independent mixed-form Adam fits of one problem from R starts (theta0,
 * device R x 4), each the optimisation of RVGP/main.py:87-95 from its own
 * initial parameters, then the FP64 LML of every fit at its final parameters
 * and the best fit: the multi-start hyperparameter search of a batch of fields
 * (no counterpart in the reference, which fits once from its defaults).
 * lower / mask on the device; theta_out (R x 4), hist (R x steps, optional),
 * lml (R; -inf for a stopped fit), status (R), outs (R x 5 scratch: LML and
 * gradient per fit), best (1 int), theta_best (4).  No host synchronisation. */
size_t rvgp_gp_fit_restarts_workspace(int m, int R);
int rvgp_gp_fit_restarts(const double* C, const double* b, const double* yy, long long N, int m, const double* evals,
                         double n_rows, int typ, const double* theta0, const double* lower, const int* mask, int R,
                         int steps, double lr, double beta1, double beta2, double eps, double* theta_out,
                         double* hist, double* lml, int* status, double* outs, int* best, double* theta_best,
                         void* workspace, size_t ws_bytes, void* stream);
/* predict_f(full_cov=False) mean and variance at Nte rows (RVGP/main.py:102-116). */
size_t rvgp_gp_predict_workspace(long long Nte, int m, int mode);
int rvgp_gp_predict(const double* Phi_star, const float* Phi_star32, long long Nte, int m, int mode,
                    const double* state, double* mean, double* var, void* workspace, size_t ws_bytes, void* stream);
/* Posterior means (Nte x B) and LMLs (B, optional) of B fields Y (N x B)
 * observed at the rows Phi (N x m), from the state and theta of an
 * rvgp_gp_lml evaluation on the same rows: the per-time-sample fits of a field
 * sequence (examples/eeg_example/eeg_utils.py:26-35) for every field at once. */
size_t rvgp_gp_posterior_batch_workspace(int m, int B);
int rvgp_gp_posterior_batch(const double* Phi, long long N, int m, const double* Y, int B, const double* theta,
                            const double* state, const double* Phi_star, long long Nte, double* mean, double* lml,
                            void* workspace, size_t ws_bytes, void* stream);
/* K = (X S) X2ᵀ and diag((X S) Xᵀ): ManifoldKernel.K / K_diag (RVGP/kernels.py:55-67). */
int rvgp_kernel_matrix(const double* X, long long N1, const double* X2, long long N2, int m, const double* S,
                       double* K, void* stream);
int rvgp_kernel_diag(const double* X, long long N, int m, const double* S, double* out, void* stream);

/* Sparse GP with M inducing inputs Z (M x m, M <= 3072): the collapsed bound
 * of GPflow 2.6.5 SGPR (RVGP/main.py:59-67,119-137, manifold_SGPR; jitter on
 * Kuu) from C = ΦᵀΦ, b = Φᵀy, yᵀy.  out (device, 5) = [F, ∂F/∂nu, ∂F/∂kappa,
 * ∂F/∂sigma_f, ∂F/∂noise], F NaN when a Cholesky factorisation failed (info,
 * device, 2 ints: Kuu, B).  dZ (device, M x m, optional) = ∂F/∂Z; state
 * (device, rvgp_sgpr_state_size(m), optional) feeds rvgp_sgpr_predict.  No
 * host synchronisation. */
size_t rvgp_sgpr_workspace(int M, int m);
size_t rvgp_sgpr_state_size(int m);
int rvgp_sgpr_elbo(const double* C, const double* b, const double* yy, long long N, int m, const double* Z, int M,
                   const double* evals, double n_rows, const double* theta, int typ, double jitter, double* out,
                   double* dZ, double* state, int* info, void* workspace, size_t ws_bytes, void* stream);
/* Divergence and curl estimates of B fields V (B x n x 3) at the points P
 * (n x 3) from their k nearest neighbours nbr (n x k, the point excluded)
 * (examples/eeg_example/eeg_utils.py:46-80): div (B x n), curl (B x n x 3).
 * ref_first = 1 differences every unit vector against point 0's, as the
 * reference does; 0 against the point's own. */
size_t rvgp_vectorfield_features_workspace(int n, int B, int k);
int rvgp_vectorfield_features(const double* P, int n, const double* V, int B, const int* nbr, int k, int ref_first,
                              double* div, double* curl, void* workspace, size_t ws_bytes, void* stream);

/* Dense GP with GPflow's RBF kernel on N <= 3072 rows X (N x m) of the scalar
 * eigenbasis and D <= 16 output columns Y (kernel='rbf', RVGP/main.py:33-37,
 * 55-58): theta (device, 3) = [variance, lengthscale, noise].  out (device,
 * 4) = [LML, ∂/∂variance, ∂/∂lengthscale, ∂/∂noise], LML NaN when the
 * Cholesky factorisation failed (info, device).  state (device,
 * rvgp_rbf_state_size(N, D)) feeds rvgp_rbf_predict: mean (Nte x D) and
 * variance (Nte).  rvgp_rbf_matrix: the kernel matrix (N1 x N2). */
size_t rvgp_rbf_workspace(long long N, int D);
size_t rvgp_rbf_state_size(long long N, int D);
int rvgp_rbf_matrix(const double* X1, long long N1, const double* X2, long long N2, int m, const double* theta,
                    double* K, void* stream);
int rvgp_rbf_lml(const double* X, long long N, int m, const double* Y, int D, const double* theta, double* out,
                 double* state, int* info, void* workspace, size_t ws_bytes, void* stream);
size_t rvgp_rbf_predict_workspace(long long Nte, long long N);
int rvgp_rbf_predict(const double* Xs, long long Nte, const double* X, long long N, int m, int D,
                     const double* theta, const double* state, double* mean, double* var, void* workspace,
                     size_t ws_bytes, void* stream);
/* SGPR.predict_f(full_cov=False) mean and variance at Nte spectral rows. */
size_t rvgp_sgpr_predict_workspace(long long Nte, int m);
int rvgp_sgpr_predict(const double* Phi_star, long long Nte, int m, const double* state, double* mean, double* var,
                      void* workspace, size_t ws_bytes, void* stream);

/* ---- fields and diffusion --------------------------------------------- */

/* manifold_dimension (RVGP/geometry.py:83-97): var_exp (c), dim (device int,
 * -1 when no column reaches frac). */
int rvgp_manifold_dimension(const double* sigma, int n, int c, double frac, double* var_exp, int* dim, void* stream);
/* mode 0: T Tᵀ v (project_to_manifold, RVGP/geometry.py:165-168); 1: Tᵀ v;
 * 2: T c (express_in_local_frame, RVGP/geometry.py:171-175). */
int rvgp_frame_map(const double* T, int n, int D, int ld, int d, const double* v, int mode, double* out, void* stream);
int rvgp_normalise_rows(double* v, int n, int D, void* stream);
/* exp(-tA) X without forming the exponential (scipy.linalg.expm(-t A) @ x at
 * RVGP/smoothing.py:13-15); A block-CSR with spectrum in [shift, bound]
 * (shift = a lower bound, e.g. λ_min, for accuracy at large t), b <= 4. */
size_t rvgp_expm_action_workspace(int n, int DB, int b);
int rvgp_expm_action(const int* indptr, const int* indices, const double* vals, int n, int DB, const double* X, int b,
                     double t, double bound, double shift, double* Y, void* workspace, size_t ws_bytes, void* stream);
/* vector_diffusion(x, t, Lc, L, method="matrix_exp", normalise=True)
 * (RVGP/smoothing.py:37-63) on the local-frame field x_loc (n, d); shift_Lc
 * a lower bound of Lc's spectrum. */
size_t rvgp_vector_diffusion_workspace(int n, int d);
int rvgp_vector_diffusion(const int* indptr, const int* indices, const double* L_vals, const double* Lc_vals, int n,
                          int d, const double* x_loc, double t, double bound_L, double bound_Lc, double shift_Lc,
                          double* out, void* workspace, size_t ws_bytes, void* stream);
/* Y = Φ diag(exp(-tλ)) Φᵀ X with orthonormal Φ (the spectral branch of
 * RVGP/smoothing.py:17-32). */
size_t rvgp_spectral_diffusion_workspace(long long N, int m, int b);
int rvgp_spectral_diffusion(const double* Phi, long long N, int m, const double* lam, const double* X, int b, double t,
                            double* Y, void* workspace, size_t ws_bytes, void* stream);

/* ---- sampling --------------------------------------------------------- */

/* Greedy furthest-point sampling, exact FP64 distances, first-index argmax
 * (furthest_point_sampling, RVGP/geometry.py:126-162).  perm (N_max ints),
 * lambdas (N_max doubles).  diam (device, optional): stop when
 * lambda/diam < spacing; count (device int) = points taken, -1 when all N_max. */
size_t rvgp_fps_workspace(int n);
int rvgp_fps(const double* X, int n, int D, int N_max, int start, const double* diam, double spacing, int* perm,
             double* lambdas, int* count, void* workspace, size_t ws_bytes, void* stream);
/* Largest pairwise exact distance (D.max() at RVGP/geometry.py:143). */
/* The same furthest-point sampling in one cooperative launch (D <= 8): a
 * bounded grid barrier per selection, the new distances screened in FP32
 * with a certified error bound and computed exactly in FP64 only where the
 * running minimum can change, so perm / lambdas equal rvgp_fps's
 * (RVGP/geometry.py:126-162).  exact_evals (device, optional): exact
 * distances evaluated.  Synchronises the stream (barrier status). */
size_t rvgp_fps_persistent_workspace(int n);
int rvgp_fps_persistent(const double* X, int n, int D, int N_max, int start, const double* diam, double spacing,
                        int* perm, double* lambdas, int* count, long long* exact_evals, void* workspace,
                        size_t ws_bytes, void* stream);

/* The same selections by spatial pruning (D <= 8, n <= rvgp_fps_spatial_max_n(D)):
 * points renumbered along a Morton curve into blocks of 32 and superblocks of
 * 1024 with FP64 bounding boxes and running maxima; each selection updates
 * only the blocks whose box comes closer to the new point than their maximum,
 * in one CTA (no grid-wide barrier).  Same arguments and results as
 * rvgp_fps_persistent (RVGP/geometry.py:126-162). */
int rvgp_fps_spatial_max_n(int D);
size_t rvgp_fps_spatial_workspace(int n, int D);
int rvgp_fps_spatial(const double* X, int n, int D, int N_max, int start, const double* diam, double spacing,
                     int* perm, double* lambdas, int* count, long long* exact_evals, void* workspace, size_t ws_bytes,
                     void* stream);
size_t rvgp_diameter_workspace(int n);
int rvgp_diameter(const double* X, int n, int D, double* out, void* workspace, size_t ws_bytes, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* RVGP_GB300_H */
