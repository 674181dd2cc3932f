/* C ABI of libtfx_gb300.so: Tensor Fox's damped Gauss-Newton CPD path on GB300.
 *
 * Every pointer argument is a device pointer owned by the caller unless stated
 * otherwise; every function enqueues work on `stream` (a cudaStream_t, NULL for
 * the legacy stream) and returns a tfx_status.  No function throws; on failure
 * tfx_last_error() returns a message for the calling thread.  Tensors are dense
 * C-order arrays; factor matrices use the reference's flat layout
 * concat_l vec_F(W_l) unless a function says "row-major".  dtype is TFX_F32 or
 * TFX_F64.  Scratch buffers are caller-owned; *_scratch_bytes() give their size.
 *
 * Reference interfaces (Tensor Fox 1.2.1, modules/TensorFox/) replaced here are
 * named beside each entry point.
 */
#ifndef TFX_GB300_H
#define TFX_GB300_H

#include <stddef.h>

#include "tfx_gb300_types.h"

#ifdef __cplusplus
extern "C" {
#endif

/* ---- library ------------------------------------------------------------ */
/* Host memory staging (no reference counterpart: the reference's rank/stats
 * sweeps hand one tensor at a time to cpd): copies n host buffers src[i] of
 * bytes[i] bytes to dst + dst_off[i] (dst: host memory, e.g. pinned), split
 * over `threads` host threads.  Used to send a batch of tensors to the device
 * in one copy. */
int tfx_host_gather(const void* const* src, const long long* bytes, const long long* dst_off, int n, void* dst,
                    int threads);
const char* tfx_last_error(void);
long long tfx_launch_count(void); /* kernels enqueued by this library so far */
int tfx_version(void);
/* The bounded-wait error path of the tensor-core kernels, exercised on its own
 * (no reference counterpart): one warp waits with `limit` polls (1..2^26) on an
 * mbarrier that nothing arrives on, so the wait runs out and *status (device
 * int) receives TFX_STATUS_ERR_TIMEOUT; nothing is left in flight. */
int tfx_wait_probe(unsigned int limit, int* status, void* stream);

/* ---- damped Gauss-Newton ------------------------------------------------
 * GaussNewton.py:29 dGN(T, factors, R, options) -> (best_factors, step_sizes,
 * errors, improv, gradients, stop), for a batch of independent problems: one
 * thread-block cluster of `cluster` CTAs (1..16) per problem runs every
 * iteration on the device (GaussNewton.py:254-398, 472-517, 713-795).
 * h_probs: host array; d_probs: device buffer of nprob descriptors. */
size_t tfx_dgn_workspace_bytes(int dtype, int L, const int* dims, int R);
int tfx_dgn_solve(int dtype, const tfx_dgn_problem* h_probs, tfx_dgn_problem* d_probs, int nprob,
                  const tfx_dgn_options* options, int cluster, void* stream);
/* The solver's per-iteration products at one point, without iterating, by the
 * same device code as tfx_dgn_solve on a cluster of `cluster` CTAs:
 * grad = GaussNewton.py:401-427 compute_grad (g_l = W_l P1_l - T_(l) KR_l,
 * flat layout) and jtjv = J^T J v (GaussNewton.py:551-581 matvec, the product
 * inside every CG iteration), after the Gramians and preconditioner set-up of
 * GaussNewton.py:520-548, 584-627 with damping `damp`.  h_prob->x holds the
 * point (flat factors); tensor, work (tfx_dgn_workspace_bytes) and result are
 * used, result[2] receives the status of the bounded waits.  Either product
 * may be skipped by passing NULL (v and jtjv together). */
int tfx_jtj_matvec(int dtype, const tfx_dgn_problem* h_prob, tfx_dgn_problem* d_prob, const tfx_dgn_options* options,
                   int cluster, double damp, const void* v, void* jtjv, void* grad, void* stream);
/* The dogleg trials that follow a rejected step (GaussNewton.py:713-795
 * compute_dogleg_steps / dogleg / update_delta), by the solver's own device
 * code: from the point x (h_prob->x), the rejected step y, the gradient grad
 * and J^T J grad as the CG hands them over, and the rejected step's relative
 * error; options->symm / factors_norm apply as in the solve.  Outputs: the
 * best point, step and (unbalanced, transformed) factors in the flat layout,
 * and the best error (device double). */
int tfx_dgn_dogleg(int dtype, const tfx_dgn_problem* h_prob, tfx_dgn_problem* d_prob, const tfx_dgn_options* options,
                   int cluster, double damp, double error, const void* y, const void* grad, const void* jtj,
                   void* best_x, void* best_y, void* best_W, double* best_error, void* stream);

/* ---- alternating least squares ---------------------------------------------
 * Alternating_Least_Squares.py:18 als(T, factors, R, options) -> (factors,
 * step_sizes, errors, improv, gradients, stop), any order 2..12, rank <= 96.
 * x: the start point (flat layout), overwritten with the LAST iterate (which
 * the reference returns); best: the best iterate; stats: [4*maxiter] errors,
 * step sizes, improvements, gradients; result: [4] stop code, iterations,
 * status, pseudo-inverse fallbacks; info: [5] |T|, best error, 0, sum|T|, 0.
 * options: maxiter, tol, tol_step, tol_improv, tol_grad, symm, factors_norm.
 * fix_mode: -1, or the mode whose factor stays as given (bicpd of the tensor-
 * train path, TensorFox.py:658-817; Alternating_Least_Squares.py:64-71, 236-264).
 * The whole solve is one CUDA-graph launch on `stream` (a while-node repeats
 * one iteration until the stop tests fire); work: tfx_als_workspace_bytes()
 * bytes, 256-byte aligned. */
size_t tfx_als_workspace_bytes(int dtype, int L, const int* dims, int R);
int tfx_als_solve(int dtype, const void* T, int L, const int* dims, int R, void* x, void* best, double* stats,
                  int* result, double* info, const tfx_dgn_options* options, int fix_mode, void* work,
                  size_t work_bytes, void* stream);

/* One ALS iteration in place on x (flat layout), no error and no stop tests:
 * the 'als' inner method of dGN (GaussNewton.py:275-278 ->
 * Alternating_Least_Squares.py:204-264).  work: tfx_als_workspace_bytes(). */
int tfx_als_sweep(int dtype, const void* T, int L, const int* dims, int R, void* x, int fix_mode, void* work,
                  size_t work_bytes, void* stream);

/* ---- dGN inner methods outside the engine ('direct', and the update after
 * every inner step), one host-driven iteration at a time
 * (GaussNewton.py:254-312 compute_step).
 * tfx_dgn_direct_step: GaussNewton.py:630-653 direct(): y (FP64, n = R*sum(dims))
 * solves (H + damp diag(Gamma)) y = grad, H the reference's Gauss-Newton matrix
 * (GaussNewton.py:656-701, its truncated off-diagonal blocks included), grad
 * (FP64, flat layout) = -compute_grad at the factors W; LU with partial
 * pivoting, y = 0 when a pivot is zero.  n <= 24576.  work:
 * tfx_dgn_direct_workspace_bytes() (about 8 n^2 bytes), 256-byte aligned.
 * tfx_dgn_step_update: GaussNewton.py:284-297: x += y (from_W = 0) or x = W
 * (from_W = 1, after tfx_als_sweep); W = x2cpd(x) balanced (Conversion.py:
 * 21-49, 361-387) and transformed (Conversion.py:412-444); the fix_mode factor
 * copied back from Wfix.  aliased = 1: the factor list holds one array L times
 * (after a symmetrising transform), whose in-place semantics are reproduced.
 * out[4] (device): ||x_new - x||^2, ||x||^2, (x_new - x).(grad + damp (x_new - x))
 * and max|grad| (the last two NaN when grad is NULL). */
size_t tfx_dgn_direct_workspace_bytes(int dtype, int L, const int* dims, int R);
int tfx_dgn_direct_step(int dtype, const void* T, int L, const int* dims, int R, const void* W, double damp,
                        double* y, double* grad, void* work, size_t work_bytes, void* stream);
int tfx_dgn_step_update(int dtype, int L, const int* dims, int R, void* x, void* W, const double* y,
                        const double* grad, double damp, int from_W, int symm, double factors_norm, int aliased,
                        int fix_mode, const void* Wfix, double* out, void* stream);

/* ---- batches of small problems (the rank/stats sweeps, TensorFox.py:820-1039,
 * run cpd on many small tensors): one CTA per problem.
 * tfx_batch_mlsvd: Compression.py:141-156 (mlsvd 'seq') per problem, modes <= 64;
 * n_components <= 0 means min(R, d_l).  tfx_batch_decompress: U_l W_l
 * (TensorFox.py:573-574); wcore_dev/wfull_dev: device arrays of per-problem flat
 * factor pointers.  tfx_batch_residual: out2[2p] = ||T_p - [[W_p]]||^2,
 * out2[2p+1] = ||T_p||^2 (Auxiliar.py:131-151). */
int tfx_batch_mlsvd(int dtype, const tfx_batch_problem* h_probs, tfx_batch_problem* d_probs, int nprob,
                    double tol_mlsvd, int n_components, void* stream);
int tfx_batch_decompress(int dtype, const tfx_batch_problem* d_probs, int nprob, const void* const* wcore_dev,
                         void* const* wfull_dev, void* stream);
int tfx_batch_residual(int dtype, const tfx_batch_problem* d_probs, int nprob, void* const* wfull_dev, double* out2,
                       void* stream);
/* Auxiliar.py:93-115 sort_dims for a whole batch on the device: problem p's
 * tensor (h_probs[p].tensor, dims = the sorted dims) is filled from src_dev[p],
 * the caller's C-order tensor; perm_dev[p*L + l] is the caller's axis that
 * becomes sorted mode l. */
int tfx_batch_permute(int dtype, const tfx_batch_problem* h_probs, tfx_batch_problem* d_probs, int nprob,
                      const void* const* src_dev, const int* perm_dev, void* stream);

/* ---- compression (MLSVD) --------------------------------------------------
 * Compression.py:192-237 compute_svd / 400-518 randomized_svd: the unfolding's
 * Gram S_(l) S_(l)^T (D x D) of a C-order tensor viewed as (P, D, Q). */
size_t tfx_mode_gram_scratch_bytes(int dtype, long long P, int D, long long Q);
int tfx_mode_gram(int dtype, const void* S, long long P, int D, long long Q, void* G, void* scratch,
                  size_t scratch_bytes, void* stream);
/* Strided batched C = alpha*A*B + beta*C (mode products of Compression.py:153-156
 * and MultilinearAlgebra.py:72-105, TensorFox.py:573-574 U_l W_l).
 * strides = {sAb, sAm, sAk, sBb, sBk, sBn, sCb, sCm, sCn} (elements). */
int tfx_gemm(int dtype, const void* A, const void* B, void* C, long long M, long long N, long long K, long long batch,
             const long long* strides, double alpha, double beta, void* stream);
/* Mode-l product with a truncated factor, out[p] (n x Q) = Ut (n x D) S[p] (D x Q)
 * for S of shape (P, D, Q) and Ut (n x D), all row-major (Compression.py:153-156,
 * the multilin_mult of MultilinearAlgebra.py:72-105 with U_l^T).  FP32 with
 * D, Q multiples of 4 runs a dedicated register-tiled kernel; other shapes use
 * tfx_gemm. */
int tfx_ttm(int dtype, const void* S, long long P, int D, long long Q, const void* Ut, int n, void* out,
            void* stream);
/* The same product on the tensor cores for precision 'mixed' (3xTF32: both
 * operands split hi + lo, FP32 accumulation; the truncation of
 * Compression.py:152-156 / 170-173): FP32 S (P, D, Q) and Ut (n x D), both 16-byte aligned, out
 * (P, n, Q); D % 32 == 0, n <= 64, Q >= 128, Q % 4 == 0 (tfx_ttm_tc_supported), else
 * TFX_STATUS_ERR_UNSUPPORTED.  err: device int, non-zero when a bounded wait
 * ran out. */
int tfx_ttm_tc_supported(long long P, int D, long long Q, int n);
int tfx_ttm_tc(const float* S, long long P, int D, long long Q, const float* Ut, int n, float* out, int* err,
               void* stream);
/* The same Gram on the 5th-generation tensor cores: TMA-fed SWIZZLE_128B tiles,
 * tcgen05.mma kind::tf32 into TMEM, FP32 accumulation, split-K partials summed
 * in compensated FP32.  FP32 input only; Q >= 32 and Q % 4 == 0; S 16-byte aligned.  *err
 * (device int) receives a non-zero code if a bounded wait expired. */
size_t tfx_mode_gram_tc_scratch_bytes(long long P, int D, long long Q);
int tfx_mode_gram_tc(const float* S, long long P, int D, long long Q, float* G, void* scratch, size_t scratch_bytes,
                     int* err, void* stream);
/* Allocation-free variant of tfx_mode_gram, for callers that cannot allocate
 * device memory when they call (their host's memory pool owns the device, the
 * call sits on a latency-critical path, or allocation is forbidden after
 * start-up).  No counterpart in the reference.  The split-K scratch comes from a
 * 32 MiB array built into the library (held by every GPU that loads it until
 * exit; tfx_mode_gram_noalloc_capacity_bytes() returns its size), so
 * D*D*element size must not exceed 32 MiB (D <= 2896 in float32, 2048 in
 * float64); larger D is refused with TFX_STATUS_ERR_ARG.  The first call on a
 * device looks the array's address up and should come before any stream
 * capture; the address is cached with the device's context, and a call after
 * that context changed (cudaDeviceReset) looks it up again.  Calls share the
 * array: calls that overlap on the GPU race. */
size_t tfx_mode_gram_noalloc_capacity_bytes(void);
int tfx_mode_gram_noalloc(int dtype, const void* S, long long P, int D, long long Q, void* G, void* stream);
/* Orthonormal basis of the k columns of Y (D x k column-major), in place
 * (scipy qr in Compression.py:392). */
int tfx_orthonormalize(int dtype, void* Y, int D, int k, void* stream);
/* Eigen-decomposition of a symmetric n x n matrix: eigenvalues descending,
 * eigenvectors as rows of V (scipy svd of Compression.py:501). */
size_t tfx_sym_eig_smem_bytes(int dtype, int n);
int tfx_sym_eig(int dtype, const void* A, int n, void* evals, void* V, int max_sweeps, int* sweeps, void* stream);
/* svd_flip (Compression.py:521-564): the largest |entry| of every column of
 * U (D x n column-major) becomes positive. */
int tfx_flip_signs(int dtype, void* U, int D, int n, void* stream);

/* ---- full-tensor residual ------------------------------------------------
 * Critical.py:14-22 fastnorm(T1, cpd2unfold1(factors))^2 (Conversion.py:117-141),
 * fused: *out = ||T - [[W]]||^2 (double). */
size_t tfx_cp_residual_scratch_bytes(void);
int tfx_cp_residual(int dtype, const void* T, int L, const int* dims, int R, const void* W, double* out, void* scratch,
                    void* stream);
/* norm(T)^2 and sum|T| (TensorFox.py:503, GaussNewton.py:113) into out2[0..1]. */
int tfx_tensor_norms(int dtype, const void* T, long long N, double* out2, void* scratch, void* stream);

/* ---- differentiable CP layer (forward / backward kernels) -------------------
 * tfx_mttkrp: T_(l) (W_{L-1} o ... o W_{l+1} o W_{l-1} o ... o W_0), the product
 * in GaussNewton.py:411-423, out (d_l x R column-major).  tfx_cp_full: the dense
 * tensor of a CPD (Conversion.py:52-79 cpd2tens).  tfx_cp_wp1: W_l P1_l for every
 * mode, P1_l = o_{m != l} W_m^T W_m (GaussNewton.py:520-548, :424), flat layout. */
size_t tfx_mttkrp_scratch_bytes(int dtype, int L, const int* dims, int R, int mode);
int tfx_mttkrp(int dtype, const void* T, int L, const int* dims, int R, const void* W, int mode, void* out, void* scratch,
               size_t scratch_bytes, void* stream);
int tfx_cp_full(int dtype, int L, const int* dims, int R, const void* W, void* out, void* stream);
/* The same product T_(l) KR_l of an FP32 tensor on the 5th-generation tensor
 * cores (GaussNewton.py:401-427 compute_grad's contraction, 411-423): the
 * tensor viewed as (P, d_l, Q) is the A operand, TMA-loaded straight from the
 * C-order array; the B operand (the factor products) is formed in shared
 * memory; tcgen05.mma kind::tf32 with every operand split hi + lo (3xTF32:
 * FP32 accuracy), FP32 accumulation in TMEM, split-K partials summed in
 * compensated FP32.  W: HOST array of L device pointers to the factors
 * (column r of W_m at W[m] + r dims[m]).  Needs R <= 64, mode < L - 1 (for the
 * last mode pass a copy of the tensor with that mode moved first), the product
 * of the later dims a multiple of 4, T 16-byte aligned.  out: d_mode x R,
 * row-major (col_major = 0) or column-major.  *err (device int) is set if a
 * bounded wait ran out.  scratch: tfx_mttkrp_tc_scratch_bytes(). */
size_t tfx_mttkrp_tc_scratch_bytes(int L, const int* dims, int R, int mode);
int tfx_mttkrp_tc(const float* T, int L, const int* dims, int R, const float* const* W, int mode, float* out,
                  int col_major, void* scratch, size_t scratch_bytes, int* err, void* stream);
size_t tfx_cp_wp1_scratch_bytes(int L, int R);
int tfx_cp_wp1(int dtype, int L, const int* dims, int R, const void* W, void* out, void* scratch, void* stream);
/* Backward of the fit loss ||T - [[W]]||^2 in one call: grad (flat layout) =
 * 2 (W_l P1_l - T_(l) KR_l) for every mode, twice the gradient g of
 * GaussNewton.py:401-427 (compute_grad). */
size_t tfx_cp_fit_grad_scratch_bytes(int dtype, int L, const int* dims, int R);
int tfx_cp_fit_grad(int dtype, const void* T, int L, const int* dims, int R, const void* W, void* grad, void* scratch,
                    size_t scratch_bytes, void* stream);

/* ---- sparse (COO) ----------------------------------------------------------
 * TensorFox.py:476-481: int64 (nnz x L) coordinates -> int32 L x nnz; *err = 1
 * when a coordinate is out of range. */
int tfx_coo_encode(const long long* idx64, long long nnz, int L, const int* dims, int* idx32, int* err, void* stream);
/* Conversion.py:255-302 sparse_unfold: entries grouped by their mode-`mode`
 * index (rowptr[d+1], permuted copies).  counts_scratch: 2*d ints. */
int tfx_coo_sort_mode(int dtype, const int* idx32, const void* vals, long long nnz, int L, const int* dims, int mode,
                      int* counts_scratch, long long* rowptr, int* sidx, void* svals, void* stream);
/* COO MTTKRP T_(l) (KR of the other factors) -> out (d_mode x R row-major);
 * Wrow_dev: device array of L pointers to row-major (d_m x R) factors.  The
 * reference forms this product only through dense unfoldings
 * (GaussNewton.py:401-427 on sparse2dense, Conversion.py:144-164). */
int tfx_coo_mttkrp(int dtype, const int* sidx, const void* svals, long long nnz, const long long* rowptr, int L,
                   const int* dims, int R, int mode, const void* const* Wrow_dev, void* out, void* stream);
/* The same COO MTTKRP from BF16 factor rows with per-column scaling (FP32
 * values and sums): tfx_factors_bf16 writes row-major BF16 copies of the flat
 * FP32 factors, column r of mode m divided by scale[m*R + r], a power of two
 * near the column's largest magnitude; tfx_coo_mttkrp_bf16 gathers them
 * (Wbf_dev: device array of L pointers) and multiplies the result by the other
 * modes' scales; out (d_mode x R row-major, FP32).  R in {8, 16, 32, 64}.  No
 * reference counterpart (the reference computes in FP64). */
int tfx_factors_bf16(int L, const int* dims, int R, const float* W, void* Wbf, float* scale, void* stream);
int tfx_coo_mttkrp_bf16(const int* sidx, const float* svals, long long nnz, const long long* rowptr, int L,
                        const int* dims, int R, int mode, const void* const* Wbf_dev, const float* scale, float* out,
                        void* stream);
/* Critical.py:25-53 sparse_fastnorm^2: *out = sum over stored entries of
 * (value - model)^2. */
size_t tfx_sparse_residual_scratch_bytes(void);
int tfx_sparse_residual(int dtype, const int* idx32, const void* vals, long long nnz, int L, const int* dims, int R,
                        const void* const* Wrow_dev, double* out, void* scratch, void* stream);
/* Compression.py:211-215 with 240-258 (dot_product_mkl(Tl, Tl.T)): dense
 * T_(l) T_(l)^T from COO; entries of one fibre are matched by comparing their
 * coordinates, so any dimensions are exact; nnz < 2^31 (TFX_STATUS_ERR_ARG
 * otherwise); *err = 2 if the fibre hash table overflows. */
size_t tfx_coo_gram_scratch_bytes(long long nnz, int d);
int tfx_coo_gram(int dtype, const int* idx32, const void* vals, long long nnz, const void* svals_sorted,
                 const long long* rowptr, int L, const int* dims, int mode, void* G, void* scratch, size_t scratch_bytes,
                 int* err, void* stream);
/* MultilinearAlgebra.py:145-190 sparse_multilin_mult (Critical.py:2703-2720):
 * dense core S (n_0 x ... x n_{L-1}) = T x_1 U_1^T ... ; U_dev: device array of
 * L pointers to row-major (d_l x n_l) matrices. */
/* ---- dGN driven by MTTKRPs (the direct COO solver; no reference
 * counterpart: the reference compresses a COO tensor before dGN).  The
 * reference's objective with absent entries as zeros:
 * ||T - [[W]]||^2 = ||T||^2 - 2 <W_0, T_(0) KR_0> + sum prod_l G_l.
 * tfx_coo_dgn_cg: one dGN iteration's inner solve (GaussNewton.py:315-398):
 * Gramians, P1/P2 (:520-548), regularisation and preconditioner (:584-627),
 * y = M (CG solution), grad = T_(l) KR_l - W_l P1_l (the CG's grad, -g of
 * :401-427) and J^T J grad, all FP64 flat vectors, from the factors W (flat)
 * and the L MTTKRPs Mrm (row-major d_l x R blocks at the flat offsets); ONE
 * cooperative launch (one CTA per SM) whose CTAs meet at bounded grid
 * barriers; out[0] = J^T J products, out[1] = the last residual norm^2,
 * out[2] = 3 if a barrier ran out.  work: 256-byte aligned,
 * tfx_coo_dgn_cg_workspace_bytes().  Order and rank within the kernel's shared
 * memory (3 L R^2 + L^2 R^2 elements <= 200 KB).
 * tfx_coo_model_error: out[0] = ||T - [[W]]||^2 from ||T||^2, W and the mode-0
 * MTTKRP (row-major), out[1] = <W_0, M_0>, out[2] = ||[[W]]||^2.
 * tfx_factors_to_rows: the flat factors as row-major d_l x R blocks.
 * tfx_dogleg_dots: out3 = {a.b, c.d, e.f}; tfx_dogleg_trial: one trial of
 * GaussNewton.py:713-795: y <- ca y + cb grad (rounded to the working type),
 * x = x_old + y, W = x, out2 = {(x - x_old).(grad + damp (x - x_old)),
 * |x - x_old|^2}; tfx_step_sums: out4 = {(x - x_old).(grad + damp (x -
 * x_old)), |x - x_old|^2, |x_old|^2, max|grad|}; tfx_step_revert: x_out =
 * x - y.  scratch: tfx_dogleg_scratch_bytes().
 * tfx_step_update_wide: the step update of GaussNewton.py:284-297 without
 * symmetric transform, fixed norm or fixed factor, over the whole grid: x +=
 * y (rounded to the working type), W = x with balanced columns
 * (Conversion.py:361-387), out4 = {|x - x_old|^2, |x_old|^2, (x - x_old).(grad +
 * damp (x - x_old)), max|grad| (NaN if any entry is)} -- the out4 of
 * tfx_dgn_step_update for the same call.  R <= 64; scratch:
 * tfx_step_update_wide_scratch_bytes(). */
size_t tfx_coo_dgn_cg_workspace_bytes(int dtype, int L, const int* dims, int R);
int tfx_coo_dgn_cg(int dtype, int L, const int* dims, int R, const void* W, const void* Mrm, double damp, int budget,
                   double cg_tol, double* y, double* grad, double* jtj, double* out, void* work, size_t work_bytes,
                   void* stream);
size_t tfx_coo_model_error_scratch_bytes(int L, int R);
int tfx_coo_model_error(int dtype, int L, const int* dims, int R, const void* W, const void* M0rm, double tnorm2,
                        double* out, void* scratch, size_t scratch_bytes, void* stream);
int tfx_factors_to_rows(int dtype, int L, const int* dims, int R, const void* W, void* Wrm, void* stream);
size_t tfx_dogleg_scratch_bytes(void);
int tfx_dogleg_dots(long long n, const double* a, const double* b, const double* c, const double* d, const double* e,
                    const double* f, double* out3, void* scratch, void* stream);
int tfx_dogleg_trial(int dtype, long long n, const void* x_old, double* y, const double* grad, double ca, double cb,
                     double damp, void* x, void* W, double* out2, void* scratch, void* stream);
int tfx_step_sums(int dtype, long long n, const void* x, const void* x_old, const double* grad, double damp,
                  double* out4, void* scratch, void* stream);
int tfx_step_revert(int dtype, long long n, const void* x, const double* y, void* x_out, void* stream);
size_t tfx_step_update_wide_scratch_bytes(int L, const int* dims, int R);
int tfx_step_update_wide(int dtype, int L, const int* dims, int R, void* x, void* W, const double* y,
                         const double* grad, double damp, double* out4, void* scratch, size_t scratch_bytes,
                         void* stream);

size_t tfx_sparse_ttmc_scratch_bytes(int dtype, long long nnz, int L, const int* n);
int tfx_sparse_ttmc(int dtype, const int* idx32, const void* vals, long long nnz, int L, const int* dims, const int* n,
                    const void* const* U_dev, void* S, void* scratch, size_t scratch_bytes, void* stream);

#ifdef __cplusplus
}
#endif
#endif
