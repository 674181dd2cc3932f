/* Plain-C descriptor types shared by the C ABI (tfx_gb300.h) and the kernels. */
#ifndef TFX_GB300_TYPES_H
#define TFX_GB300_TYPES_H

#ifdef __cplusplus
extern "C" {
#endif

#define TFX_MAX_ORDER 12

/* Status codes returned by every entry point. */
enum tfx_status {
  TFX_STATUS_OK = 0,
  TFX_STATUS_ERR_ARG = 1,        /* invalid argument (shape, rank, pointer) */
  TFX_STATUS_ERR_NUMERIC = 2,    /* non-finite value met where the reference would stop */
  TFX_STATUS_ERR_TIMEOUT = 3,    /* a bounded device wait ran out */
  TFX_STATUS_ERR_CUDA = 4,       /* CUDA runtime error (message via tfx_last_error) */
  TFX_STATUS_ERR_UNSUPPORTED = 5 /* configuration outside the supported set */
};

/* Element type of tensors and factors. */
enum tfx_dtype { TFX_F32 = 0, TFX_F64 = 1 };

/* One dense damped Gauss-Newton problem (GaussNewton.py:29 dGN(T, factors, R, options)).
 * All pointers are device pointers owned by the caller.
 *   tensor : C-order array of prod(dims) elements
 *   x      : flat start point, concat_l vec_F(W_l), R*sum(dims) elements (read)
 *   best   : best factors found, same layout (written)
 *   work   : scratch of tfx_dgn_workspace_bytes() bytes
 *   budgets: [maxiter] CG iteration caps (GaussNewton.py:267 or cg_maxiter)
 *   damp_sched: [maxiter] damping schedule when options.init_damp is a list, else NULL
 *   stats  : [4*maxiter] errors, step_sizes, improv, gradients (written)
 *   result : [4] stop code, iterations run, status, dogleg fallbacks (written)
 *   info   : [5] |T|, best error, final damping, mean|T|, J^T J v products run (written)
 *   prof   : optional [24] SM clock cycles per phase (gramians, gradient, CG,
 *            update, residual, dogleg, control, total), per CG step part
 *            (publish+barrier, staging, A_k, Y_l, z_l, two reductions, update)
 *            and per third-order gradient part (setup, chunk issue, chunk wait,
 *            Y and M2, barrier, M0 and M1, finish, team barrier), or NULL */
typedef struct tfx_dgn_problem {
  int L;
  int R;
  int dims[TFX_MAX_ORDER];
  const void* tensor;
  const void* x;
  void* best;
  void* work;
  const int* budgets;
  const double* damp_sched;
  double* stats;
  int* result;
  double* info;
  long long* prof;
} tfx_dgn_problem;

/* One small dense problem of a batched compression (every dimension <= 64).
 *   tensor     : C-order input (modes already in decreasing size)
 *   work       : scratch of work_elems >= 2*prod(dims) elements
 *   Ut         : output, per mode the (n_l x d_l) row-major U_l^T, concatenated
 *   core       : output core, prod(n_l) elements
 *   core_dims  : output n_l per mode (L ints)
 *   sigma      : output singular values, min(R, d_l) slots per mode */
typedef struct tfx_batch_problem {
  int L;
  int R;
  int dims[TFX_MAX_ORDER];
  const void* tensor;
  void* work;
  long long work_elems;
  void* Ut;
  void* core;
  int* core_dims;
  double* sigma;
} tfx_batch_problem;

/* Solver options (Auxiliar.py:258-283 defaults; TensorFox.py:84-213 meaning). */
typedef struct tfx_dgn_options {
  int maxiter;
  double tol;
  double tol_step;
  double tol_improv;
  double tol_grad;
  double tol_jump;
  double cg_tol;
  double init_damp;
  int use_damp_sched; /* 1: damp_sched holds init_damp as a list */
  int symm;           /* options.symm */
  double factors_norm; /* options.factors_norm (0 = off) */
  int tile;           /* engine register tile of the small contractions: 1, 2 or 4
                         (16*tile rows and columns per CTA tile); 0 = chosen from
                         the largest dimension or rank of the batch */
  int aliased;        /* 1: the start's factor list holds one array L times (a
                         symmetric start, Initialization.py:83); the reference's
                         in-place x2cpd / transform then act on that one array */
  int fixed;          /* 1 + the mode whose factor is put back after every step
                         (bicpd, third order, GaussNewton.py:92-99, 293-297);
                         0 = none */
} tfx_dgn_options;

#ifdef __cplusplus
}
#endif
#endif
