// C ABI of the dGN engine: workspace sizing, validation and dispatch.
#include "dgn_engine.cuh"

using namespace tfx;

extern "C" size_t tfx_dgn_workspace_bytes(int dtype, int L, const int* dims, int R) {
  if (L < 2 || L > TFX_MAX_ORDER || R < 1 || dims == nullptr) return 0;
  int s = 0;
  for (int l = 0; l < L; ++l) s += dims[l];
  return ws_layout(L, R, R * s, dtype == TFX_F64 ? 8 : 4).total;
}

// Validates a set of problems and picks the engine's register tile and
// shared-memory plan for them (shared by the solve and the units entry point).
static int dgn_plan(int dtype, const tfx_dgn_problem* h_probs, int nprob, const tfx_dgn_options* op, int cluster,
                    int* TS_out, SmemPlan* sp_out) {
  if (h_probs == nullptr || op == nullptr || nprob < 1) return tfx_set_error(TFX_STATUS_ERR_ARG, "null argument");
  if (cluster < 1 || cluster > 16) return tfx_set_error(TFX_STATUS_ERR_ARG, "cluster must be in 1..16");
  if (op->maxiter < 1) return tfx_set_error(TFX_STATUS_ERR_ARG, "maxiter must be >= 1");
  if (dtype != TFX_F32 && dtype != TFX_F64) return tfx_set_error(TFX_STATUS_ERR_ARG, "dtype");
  int maxL = 0, maxR = 0, maxd = 0, maxdim_or_R = 0;
  for (int p = 0; p < nprob; ++p) {
    const tfx_dgn_problem& q = h_probs[p];
    if (q.L < 2 || q.L > TFX_MAX_ORDER || q.R < 1) return tfx_set_error(TFX_STATUS_ERR_ARG, "bad order or rank");
    if (q.R < cluster) return tfx_set_error(TFX_STATUS_ERR_ARG, "rank smaller than cluster size");
    long long n = 1;
    for (int l = 0; l < q.L; ++l) {
      if (q.dims[l] < 1) return tfx_set_error(TFX_STATUS_ERR_ARG, "bad dimension");
      n *= q.dims[l];
      maxd = q.dims[l] > maxd ? q.dims[l] : maxd;
    }
    if (n > (1LL << 40)) return tfx_set_error(TFX_STATUS_ERR_ARG, "tensor too large");
    if (op->fixed < 0 || op->fixed > q.L) return tfx_set_error(TFX_STATUS_ERR_ARG, "fixed mode out of range");
    if (op->fixed > 0 && (op->symm || op->aliased))
      return tfx_set_error(TFX_STATUS_ERR_UNSUPPORTED, "a fixed factor with symm");
    if (op->symm || op->aliased) {
      for (int l = 1; l < q.L; ++l)
        if (q.dims[l] != q.dims[0]) return tfx_set_error(TFX_STATUS_ERR_ARG, "symm (or one factor array for every mode) needs equal dims");
    }
    maxL = q.L > maxL ? q.L : maxL;
    maxR = q.R > maxR ? q.R : maxR;
  }
  maxdim_or_R = maxd > maxR ? maxd : maxR;
  if (op->tile != 0 && op->tile != 1 && op->tile != 2 && op->tile != 4)
    return tfx_set_error(TFX_STATUS_ERR_ARG, "tile must be 0, 1, 2 or 4");
  const int TS = op->tile ? op->tile : (maxdim_or_R <= 16 ? 1 : (maxdim_or_R <= 32 ? 2 : 4));
  const int maxncol = (maxR + cluster - 1) / cluster;
  const size_t es = dtype == TFX_F64 ? 8 : 4;
  if (op->maxiter > 4096) return tfx_set_error(TFX_STATUS_ERR_UNSUPPORTED, "maxiter above 4096");
  int maxnx = 0, maxsumd = 0;
  for (int p = 0; p < nprob; ++p) {
    int sd = 0;
    for (int l = 0; l < h_probs[p].L; ++l) sd += h_probs[p].dims[l];
    maxnx = sd * h_probs[p].R > maxnx ? sd * h_probs[p].R : maxnx;
    maxsumd = sd > maxsumd ? sd : maxsumd;
  }
  // stage the CG operands in shared memory when they fit, else read them from L2
  SmemPlan sp = smem_plan(TS, es, maxL, maxR, maxd, maxncol, op->maxiter, maxnx, maxsumd, 1);
  if (sp.total > 200 * 1024) sp = smem_plan(TS, es, maxL, maxR, maxd, maxncol, op->maxiter, maxnx, maxsumd, 0);
  if (sp.total > 220 * 1024) return tfx_set_error(TFX_STATUS_ERR_UNSUPPORTED, "problem too large for the engine's shared memory; use a larger cluster");
  *TS_out = TS;
  *sp_out = sp;
  return TFX_STATUS_OK;
}

extern "C" int tfx_dgn_solve(int dtype, const tfx_dgn_problem* h_probs, tfx_dgn_problem* d_probs, int nprob,
                             const tfx_dgn_options* op, int cluster, void* stream) {
  if (h_probs == nullptr || d_probs == nullptr || op == nullptr || nprob < 1)
    return tfx_set_error(TFX_STATUS_ERR_ARG, "null argument");
  for (int p = 0; p < nprob; ++p) {
    const tfx_dgn_problem& q = h_probs[p];
    if (!q.tensor || !q.x || !q.best || !q.work || !q.budgets || !q.stats || !q.result || !q.info)
      return tfx_set_error(TFX_STATUS_ERR_ARG, "null device pointer in problem");
    if (op->use_damp_sched && !q.damp_sched) return tfx_set_error(TFX_STATUS_ERR_ARG, "missing damp schedule");
  }
  int TS = 0;
  SmemPlan sp;
  if (int s = dgn_plan(dtype, h_probs, nprob, op, cluster, &TS, &sp)) return s;
  cudaStream_t st = (cudaStream_t)stream;
  cudaError_t e = cudaMemcpyAsync(d_probs, h_probs, sizeof(tfx_dgn_problem) * nprob, cudaMemcpyHostToDevice, st);
  if (e != cudaSuccess) return tfx_set_cuda_error(e, "descriptor copy");
  if (dtype == TFX_F32) return launch_dgn_f32(TS, d_probs, nprob, op, cluster, sp, st);
  return launch_dgn_f64(TS, d_probs, nprob, op, cluster, sp, st);
}

extern "C" int tfx_jtj_matvec(int dtype, const tfx_dgn_problem* h_prob, tfx_dgn_problem* d_prob,
                              const tfx_dgn_options* op, int cluster, double damp, const void* v, void* jtjv,
                              void* grad, void* stream) {
  if (h_prob == nullptr || d_prob == nullptr || op == nullptr) return tfx_set_error(TFX_STATUS_ERR_ARG, "null argument");
  if (!h_prob->tensor || !h_prob->x || !h_prob->work || !h_prob->result)
    return tfx_set_error(TFX_STATUS_ERR_ARG, "null device pointer in problem");
  if ((v == nullptr) != (jtjv == nullptr)) return tfx_set_error(TFX_STATUS_ERR_ARG, "v and jtjv go together");
  if (op->aliased || op->fixed) return tfx_set_error(TFX_STATUS_ERR_ARG, "aliased/fixed factors are solve options");
  int TS = 0;
  SmemPlan sp;
  if (int s = dgn_plan(dtype, h_prob, 1, op, cluster, &TS, &sp)) return s;
  cudaStream_t st = (cudaStream_t)stream;
  cudaError_t e = cudaMemcpyAsync(d_prob, h_prob, sizeof(tfx_dgn_problem), cudaMemcpyHostToDevice, st);
  if (e != cudaSuccess) return tfx_set_cuda_error(e, "descriptor copy");
  UnitsArgs ua = {};
  ua.mode = 0;
  ua.damp = damp;
  ua.v = v;
  ua.jtjv = jtjv;
  ua.grad = grad;
  if (dtype == TFX_F32) return launch_units_f32(TS, d_prob, op, cluster, sp, ua, st);
  return launch_units_f64(TS, d_prob, op, cluster, sp, ua, st);
}

extern "C" int tfx_dgn_dogleg(int dtype, const tfx_dgn_problem* h_prob, tfx_dgn_problem* d_prob,
                              const tfx_dgn_options* op, int cluster, double damp, double error, const void* y,
                              const void* grad, const void* jtj, void* best_x, void* best_y, void* best_W,
                              double* best_error, void* stream) {
  if (h_prob == nullptr || d_prob == nullptr || op == nullptr) return tfx_set_error(TFX_STATUS_ERR_ARG, "null argument");
  if (!h_prob->tensor || !h_prob->x || !h_prob->work || !h_prob->result || !y || !grad || !jtj || !best_x ||
      !best_y || !best_W || !best_error)
    return tfx_set_error(TFX_STATUS_ERR_ARG, "null device pointer");
  if (op->aliased || op->fixed) return tfx_set_error(TFX_STATUS_ERR_ARG, "aliased/fixed factors are solve options");
  int TS = 0;
  SmemPlan sp;
  if (int s = dgn_plan(dtype, h_prob, 1, op, cluster, &TS, &sp)) return s;
  cudaStream_t st = (cudaStream_t)stream;
  cudaError_t e = cudaMemcpyAsync(d_prob, h_prob, sizeof(tfx_dgn_problem), cudaMemcpyHostToDevice, st);
  if (e != cudaSuccess) return tfx_set_cuda_error(e, "descriptor copy");
  UnitsArgs ua = {};
  ua.mode = 1;
  ua.damp = damp;
  ua.error = error;
  ua.grad = (void*)grad;
  ua.y = y;
  ua.jtj = jtj;
  ua.best_x = best_x;
  ua.best_y = best_y;
  ua.best_W = best_W;
  ua.best_error = best_error;
  if (dtype == TFX_F32) return launch_units_f32(TS, d_prob, op, cluster, sp, ua, st);
  return launch_units_f64(TS, d_prob, op, cluster, sp, ua, st);
}
