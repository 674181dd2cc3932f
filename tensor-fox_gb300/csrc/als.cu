// Alternating least squares CPD on the device (Tensor Fox v1.2.1
// Alternating_Least_Squares.py:18-201 als, :204-235 als_iteration).
//
// One ALS iteration updates the factors mode after mode with the freshly
// updated ones (Gauss-Seidel order), W_l = T_(l) pinv(KR_l^T), then applies
// `transform` (Conversion.py:412-444), measures the relative error and runs the
// reference's stop tests.  With H_l = KR_l^T KR_l = o_{m != l} G_m (G_m = W_m^T W_m),
// pinv(KR_l^T) = KR_l H_l^+ whenever KR_l has full column rank, so
//   W_l = MTTKRP_l H_l^+,
// and the only contraction with the tensor is the MTTKRP (tfx_mttkrp).  H_l^+
// comes from the symmetric sweep operator (Gauss-Jordan elimination on an SPD
// matrix, in shared memory; FP32 on the FP32 path, FP64 otherwise or when the
// FP32 pivots degrade); when an FP64 pivot falls below 1e-12 of its diagonal
// (H_l numerically singular) the solve switches to a Jacobi eigen-decomposition
// and inverts the eigenvalues above 1e-13 of the largest (a pseudo-inverse).
//
// The whole solve is ONE graph launch: a CUDA graph whose while-node repeats
// the body (per mode: MTTKRP, inverse, apply + partial Gramians, Gramian sum;
// then step size and transform, residual, control) until the control kernel
// clears the loop condition with cudaGraphSetConditional.  No host round trip
// per iteration; the loop always ends after maxiter iterations at the latest.
//
// Precision: factors, the MTTKRP and H_l^+ in the working type (H_l^+ from an
// FP64 sweep whenever the FP32 one loses its pivots); Gramians, H_l, the step
// size, the residual and every control scalar in FP64.
#include <math.h>
#include <stdint.h>

#include <algorithm>

#include "tfx_capi_internal.h"
#include "tfx_common.cuh"
#include "tfx_gb300.h"
#include "linalg.cuh"

namespace tfx {
namespace als {

constexpr int NT = 256;        // threads of the single-CTA kernels
constexpr int RMAX = 96;       // largest rank: two padded R x R FP64 matrices in shared memory
constexpr int ROWS = 8;        // factor rows per CTA in the apply / Gramian kernels

// Device state of one solve (first 256 bytes of the workspace).
struct State {
  int it;          // iterations completed
  int stop;        // stop code (5 until a test fires)
  int fallbacks;   // pseudo-inverse fallbacks taken (H_l numerically singular)
  int pad;
  double error;    // relative error of the last iteration (1 before the first)
  double best_error;
  double step2;    // ||x - x_old||^2 of the current iteration
  double res2;     // ||T - [[W]]||^2 of the current iteration
  double tn[2];    // ||T||^2, sum |T|
};

struct Layout {
  size_t state, G, Hinv, M, gpart, xo, xfix, mtt, res, total;
  size_t mtt_bytes;
};

__host__ inline size_t up256(size_t v) { return (v + 255) & ~(size_t)255; }

static Layout layout(int dtype, int L, const int* dims, int R) {
  const size_t es = dtype == TFX_F64 ? 8 : 4;
  int maxd = 0;
  long long nx = 0;
  size_t mtt = 0;
  for (int l = 0; l < L; ++l) {
    maxd = std::max(maxd, dims[l]);
    nx += (long long)dims[l] * R;
    mtt = std::max(mtt, tfx_mttkrp_scratch_bytes(dtype, L, dims, R, l));
  }
  const size_t nblk = (size_t)(maxd + ROWS - 1) / ROWS;
  Layout y;
  size_t o = 0;
  y.state = o;  o += 256;
  y.G = o;      o += up256((size_t)L * R * R * 8);
  y.Hinv = o;   o += up256((size_t)R * R * es);
  y.M = o;      o += up256((size_t)maxd * R * es);
  y.gpart = o;  o += up256(nblk * R * R * 8);
  y.xo = o;     o += up256((size_t)nx * es);
  y.xfix = o;   o += up256((size_t)nx * es);
  y.mtt = o;    o += up256(mtt);
  y.mtt_bytes = mtt;
  y.res = o;    o += up256(tfx_cp_residual_scratch_bytes());
  y.total = o;
  return y;
}

// ---------------------------------------------------------------------------
// Partial Gramians of a block of ROWS rows of W (d x R, column-major):
// gpart[blk][a][b] = sum_{i in block} W[i][a] W[i][b].  FP32 products are
// chained over the block (8 terms) and stored in FP64; FP64 inputs stay FP64.
// ---------------------------------------------------------------------------
template <class T>
__device__ __forceinline__ void block_gram(const T* sW, int nr, int R, double* out) {
  const int n = R * (R + 1) / 2;
  for (int e = threadIdx.x; e < n; e += blockDim.x) {
    // e -> (a, b), a <= b, row-major upper triangle
    int a = 0, rem = e;
    while (rem >= R - a) {
      rem -= R - a;
      ++a;
    }
    const int b = a + rem;
    T acc = T(0);
    for (int i = 0; i < nr; ++i) acc = fma(sW[i * R + a], sW[i * R + b], acc);
    out[(size_t)a * R + b] = (double)acc;
    out[(size_t)b * R + a] = (double)acc;
  }
}

template <class T>
__global__ void __launch_bounds__(NT) k_als_gram_part(const T* __restrict__ W, int d, int R, double* __restrict__ gpart) {
  extern __shared__ __align__(16) char smem[];
  T* sW = (T*)smem;  // ROWS x R, row-major
  const int r0 = blockIdx.x * ROWS;
  const int nr = min(ROWS, d - r0);
  for (int e = threadIdx.x; e < nr * R; e += blockDim.x) {
    const int i = e % nr, a = e / nr;
    sW[i * R + a] = W[(size_t)a * d + r0 + i];
  }
  __syncthreads();
  block_gram<T>(sW, nr, R, gpart + (size_t)blockIdx.x * R * R);
}

// G = sum over blocks of the partials, in block order (deterministic)
__global__ void k_als_gram_sum(const double* __restrict__ gpart, int nblk, int R, double* __restrict__ G) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= R * R) return;
  double s = 0.0;
  for (int b = 0; b < nblk; ++b) s += gpart[(size_t)b * R * R + e];
  G[e] = s;
}

// ---------------------------------------------------------------------------
// Sweep operator on A (R x R inside an m x m row-major buffer): after sweeping
// pivot k, A[k][k] = -1/p, A[i][k] = A[k][i] = A[i][k]/p and
// A[i][j] -= A[i][k] A[k][j] / p; after all pivots A = -H^{-1}.  Returns false
// (uniformly across the CTA) when a pivot is not above thr times H's own
// diagonal entry piv[k].
// ---------------------------------------------------------------------------
template <class C>
__device__ bool sweep_inverse(C* A, int m, int R, const double* piv, C* cs, volatile int* fail, double thr) {
  const int tid = threadIdx.x, RR = R * R;
  if (tid == 0) *fail = 0;
  __syncthreads();
  for (int k = 0; k < R; ++k) {
    const C p = A[k * m + k];
    if (!((double)p > thr * piv[k])) {
      if (tid == 0) *fail = 1;
      break;
    }
    for (int i = tid; i < R; i += NT) cs[i] = A[i * m + k];
    __syncthreads();
    const C ip = C(1) / p;
    for (int e = tid; e < RR; e += NT) {
      const int i = e / R, j = e - i * R;
      const C aik = cs[i], akj = cs[j];
      C v;
      if (i == k && j == k) v = -ip;
      else if (i == k) v = akj * ip;
      else if (j == k) v = aik * ip;
      else v = A[i * m + j] - aik * akj * ip;
      A[i * m + j] = v;
    }
    __syncthreads();
  }
  __syncthreads();
  return *fail == 0;
}

// ---------------------------------------------------------------------------
// H_l^+ for H_l = o_{m != l} G_m (one CTA), written as Hinv (R x R) in the
// working type.  FP32 path: the sweep runs in FP32 (the factor update it feeds
// is FP32; an update off by a relative e moves the ALS objective by O(e^2)),
// with a pivot floor of 1e-4 of the diagonal; FP64 path, or when that floor is
// crossed: the sweep in FP64 with a floor of 1e-12.  Below that H is singular
// to working accuracy and the pseudo-inverse comes from a Jacobi
// eigen-decomposition (eigenvalues above 1e-13 of the largest inverted).
// ---------------------------------------------------------------------------
template <class T>
__global__ void __launch_bounds__(NT) k_als_inv(const double* __restrict__ G, int L, int l, int R, T* __restrict__ Hinv,
                                                State* st) {
  extern __shared__ __align__(16) char smem[];
  const int m = (R + 1) & ~1;
  double* A = (double*)smem;          // m x m
  double* V = A + (size_t)m * m;      // m x m (FP32 sweep, then eigenvectors in the fallback)
  double* cs = V + (size_t)m * m;     // m values
  int* pr = (int*)(cs + m);           // m + 2 ints
  double* red = (double*)(pr + m + 2);  // 4 doubles
  double* piv = red + 4;              // H's diagonal
  const int tid = threadIdx.x;
  const int RR = R * R;
  volatile int* fail = (volatile int*)(red + 2);
  auto h_entry = [&](int a, int b) {
    double p = 1.0;
    for (int k = 0; k < L; ++k)
      if (k != l) p *= G[(size_t)k * RR + a * R + b];
    return p;
  };
  for (int e = tid; e < m * m; e += NT) {
    const int a = e / m, b = e - a * m;
    A[e] = (a < R && b < R) ? h_entry(a, b) : (a == b ? 1.0 : 0.0);
  }
  __syncthreads();
  for (int k = tid; k < R; k += NT) piv[k] = A[k * m + k];
  __syncthreads();
  if (sizeof(T) == 4) {
    float* A32 = (float*)V;
    for (int e = tid; e < m * m; e += NT) A32[e] = (float)A[e];
    __syncthreads();
    if (sweep_inverse<float>(A32, m, R, piv, (float*)cs, fail, 1e-4)) {
      for (int e = tid; e < RR; e += NT) {
        const int i = e / R, j = e - i * R;
        Hinv[e] = (T)(-A32[i * m + j]);
      }
      return;
    }
  }
  if (sweep_inverse<double>(A, m, R, piv, cs, fail, 1e-12)) {
    for (int e = tid; e < RR; e += NT) {
      const int i = e / R, j = e - i * R;
      Hinv[e] = (T)(-A[i * m + j]);
    }
    return;
  }
  // pseudo-inverse from the eigen-decomposition of H (H singular to working
  // accuracy)
  for (int e = tid; e < m * m; e += NT) {
    const int a = e / m, b = e - a * m;
    A[e] = (a < R && b < R) ? h_entry(a, b) : 0.0;
    V[e] = (a == b) ? 1.0 : 0.0;
  }
  __syncthreads();
  cta_jacobi<double>(A, V, cs, pr, red, m, 60);
  if (tid == 0) {
    double lmax = 0.0;
    for (int i = 0; i < R; ++i) lmax = fmax(lmax, A[i * m + i]);
    red[3] = lmax;
    atomicAdd(&st->fallbacks, 1);
  }
  __syncthreads();
  const double cut = 1e-13 * red[3];
  for (int e = tid; e < RR; e += NT) {
    const int a = e / R, b = e - a * R;
    double s = 0.0;
    for (int i = 0; i < R; ++i) {
      const double lam = A[i * m + i];
      if (lam > cut) s += V[i * m + a] * V[i * m + b] / lam;
    }
    Hinv[e] = (T)s;
  }
}

// ---------------------------------------------------------------------------
// W_l rows of this block = M rows (d x R column-major) times Hinv, written
// into the flat factor vector; then the block's partial Gramian.
// ---------------------------------------------------------------------------
template <class T>
__global__ void __launch_bounds__(NT) k_als_apply(const T* __restrict__ M, const T* __restrict__ Hinv, int d, int R,
                                                  T* __restrict__ W, double* __restrict__ gpart) {
  extern __shared__ __align__(16) char smem[];
  T* sH = (T*)smem;               // R x R
  T* sM = sH + (size_t)R * R;     // ROWS x R
  T* sW = sM + (size_t)ROWS * R;  // ROWS x R
  const int r0 = blockIdx.x * ROWS;
  const int nr = min(ROWS, d - r0);
  for (int e = threadIdx.x; e < R * R; e += blockDim.x) sH[e] = Hinv[e];
  for (int e = threadIdx.x; e < nr * R; e += blockDim.x) {
    const int i = e % nr, a = e / nr;
    sM[i * R + a] = M[(size_t)a * d + r0 + i];
  }
  __syncthreads();
  for (int e = threadIdx.x; e < nr * R; e += blockDim.x) {
    const int i = e % nr, b = e / nr;
    T acc = T(0);
    for (int a = 0; a < R; ++a) acc = fma(sM[i * R + a], sH[a * R + b], acc);
    sW[i * R + b] = acc;
    W[(size_t)b * d + r0 + i] = acc;
  }
  __syncthreads();
  block_gram<T>(sW, nr, R, gpart + (size_t)blockIdx.x * R * R);
}

// ---------------------------------------------------------------------------
// Step size ||x - x_old||^2 (x = the factors before `transform`, as in the
// reference), x_old <- x, then `transform` (symmetrisation / fixed norm).
// ---------------------------------------------------------------------------
struct Dims {
  int L, R;
  int d[TFX_MAX_ORDER];
  int off[TFX_MAX_ORDER];
  long long nx;
};

template <class T>
__global__ void __launch_bounds__(NT) k_als_post(T* __restrict__ x, T* __restrict__ xo, Dims sh, int symm,
                                                 double factors_norm, int fix, const T* __restrict__ xfix,
                                                 State* st) {
  __shared__ double red[NT / 32];
  __shared__ double nrm[TFX_MAX_ORDER];
  const int tid = threadIdx.x;
  double s = 0.0;
  for (long long e = tid; e < sh.nx; e += NT) {
    const double dv = (double)x[e] - (double)xo[e];
    s = fma(dv, dv, s);
    xo[e] = x[e];
  }
  s = warp_sum(s);
  if ((tid & 31) == 0) red[tid >> 5] = s;
  __syncthreads();
  if (tid == 0) {
    double t = 0.0;
    for (int w = 0; w < NT / 32; ++w) t += red[w];
    st->step2 = t;
  }
  __syncthreads();
  if (symm) {
    // factors[0] = (((W0 + W1) + W2) + ...) / L, every factor = factors[0]
    const int n = sh.d[0] * sh.R;
    for (int e = tid; e < n; e += NT) {
      T acc = x[e];
      for (int l = 1; l < sh.L; ++l) acc = acc + x[sh.off[l] + e];
      acc = acc / (T)sh.L;
      for (int l = 0; l < sh.L; ++l) x[sh.off[l] + e] = acc;
    }
    __syncthreads();
  }
  if (factors_norm > 0.0) {
    for (int l = 0; l < sh.L; ++l) {
      double q = 0.0;
      const int n = sh.d[l] * sh.R;
      for (int e = tid; e < n; e += NT) {
        const double v = (double)x[sh.off[l] + e];
        q = fma(v, v, q);
      }
      q = warp_sum(q);
      if ((tid & 31) == 0) red[tid >> 5] = q;
      __syncthreads();
      if (tid == 0) {
        double t = 0.0;
        for (int w = 0; w < NT / 32; ++w) t += red[w];
        nrm[l] = sqrt(t);
      }
      __syncthreads();
    }
    for (int l = 0; l < sh.L; ++l) {
      const T sc = (T)(factors_norm * (1.0 / nrm[l]));
      const int n = sh.d[l] * sh.R;
      for (int e = tid; e < n; e += NT) x[sh.off[l] + e] = sc * x[sh.off[l] + e];
    }
  }
  if (fix >= 0 && (symm || factors_norm > 0.0)) {
    // the fixed factor is restored after the transform
    // (Alternating_Least_Squares.py:116-121)
    __syncthreads();
    const int n = sh.d[fix] * sh.R;
    for (int e = tid; e < n; e += NT) x[sh.off[fix] + e] = xfix[sh.off[fix] + e];
  }
}

// ---------------------------------------------------------------------------
// Error, statistics, best iterate, stop tests (Alternating_Least_Squares.py:
// 119-190) and the loop condition of the graph's while-node.
// stats: [0,m) errors, [m,2m) step sizes, [2m,3m) improvements, [3m,4m) gradients.
// ---------------------------------------------------------------------------
template <class T>
__global__ void __launch_bounds__(NT) k_als_control(const T* __restrict__ x, T* __restrict__ best, long long nx,
                                                    tfx_dgn_options op, double* __restrict__ stats,
                                                    int* __restrict__ result, double* __restrict__ info, State* st,
                                                    cudaGraphConditionalHandle cond) {
  __shared__ int s_improved;
  const int tid = threadIdx.x;
  const int m = op.maxiter;
  if (tid == 0) {
    const int it = st->it;
    const double Tsize = sqrt(st->tn[0]);
    const double error = sqrt(fmax(st->res2, 0.0)) / Tsize;
    const double old_error = st->error;
    const double step = sqrt(st->step2);
    s_improved = error < st->best_error;
    if (s_improved) st->best_error = error;
    stats[it] = error;
    stats[m + it] = step;
    stats[3 * m + it] = fabs(old_error - error) / step;
    stats[2 * m + it] = it == 0 ? error : fabs(stats[it - 1] - error);
    int stop = -1;
    if (it > 1) {
      const int cnst = 1 + m / 10;
      if (stats[it] < op.tol) stop = 0;
      else if (stats[m + it] < op.tol_step) stop = 1;
      else if (stats[2 * m + it] < op.tol_improv) stop = 2;
      else if (stats[3 * m + it] < op.tol_grad) stop = 3;
      else {
        if (it > 2 * cnst && it % cnst == 0) {
          double m1 = 0.0, m2 = 0.0, m3 = 0.0;
          for (int k = it - 2 * cnst; k < it - cnst; ++k) m1 += stats[k];
          for (int k = it - cnst; k < it; ++k) m2 += stats[k];
          for (int k = it - cnst; k < it; ++k) m3 += stats[2 * m + k];
          m1 /= cnst;
          m2 /= cnst;
          m3 /= cnst;
          if (m1 - m2 <= op.tol_improv) stop = 4;
          else if (m3 < 1e-3 * m2) stop = 7;
        }
        if (stop < 0 && error > fmax(1.0, Tsize * Tsize) / (1e-16 + op.tol)) stop = 6;
      }
    }
    st->error = error;
    st->it = it + 1;
    const bool finished = stop >= 0 || it + 1 >= m;
    if (stop >= 0) st->stop = stop;
    if (finished) {
      result[0] = st->stop;
      result[1] = it + 1;
      result[2] = TFX_STATUS_OK;
      result[3] = st->fallbacks;
      info[0] = Tsize;
      info[1] = st->best_error;
      info[2] = 0.0;
      info[3] = st->tn[1];
      info[4] = 0.0;
    }
    cudaGraphSetConditional(cond, finished ? 0u : 1u);
  }
  __syncthreads();
  if (s_improved)
    for (long long e = tid; e < nx; e += NT) best[e] = x[e];
}

template <class T>
__global__ void k_als_init(const T* __restrict__ x, T* __restrict__ xo, T* __restrict__ best, long long nx, State* st) {
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e < nx) {
    xo[e] = x[e];
    best[e] = x[e];
  }
  if (e == 0) {
    st->it = 0;
    st->stop = 5;
    st->fallbacks = 0;
    st->error = 1.0;
    st->best_error = INFINITY;
    st->step2 = 0.0;
    st->res2 = 0.0;
  }
}

static size_t inv_smem(int R) {
  const int m = (R + 1) & ~1;
  return (size_t)2 * m * m * 8 + (size_t)m * 8 + (size_t)(m + 2) * 4 + 8 + 4 * 8 + (size_t)R * 8 + 16;
}

static int check(const char* w) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return tfx_set_cuda_error(e, w);
  tfx_count_launch(1);
  return TFX_STATUS_OK;
}

// Kernels of the Gramian of every mode (partials + sum).
template <class T>
static int grams_all(const T* x, const Dims& sh, const Layout& y, char* w, cudaStream_t s) {
  double* G = (double*)(w + y.G);
  double* gp = (double*)(w + y.gpart);
  const int R = sh.R;
  for (int l = 0; l < sh.L; ++l) {
    const int nb = (sh.d[l] + ROWS - 1) / ROWS;
    k_als_gram_part<T><<<nb, NT, (size_t)ROWS * R * sizeof(T), s>>>(x + sh.off[l], sh.d[l], R, gp);
    if (int r = check("als gram")) return r;
    k_als_gram_sum<<<(R * R + 255) / 256, 256, 0, s>>>(gp, nb, R, G + (size_t)l * R * R);
    if (int r = check("als gram sum")) return r;
  }
  return TFX_STATUS_OK;
}

// The mode-by-mode factor updates of one ALS iteration (Alternating_Least_Squares.py:
// 204-264); G must hold every mode's Gramian on entry and holds them on exit.
template <class T>
static int sweep(int dtype, const T* Tt, const int* dims, T* x, const Dims& sh, int fix, const Layout& y, char* w,
                 cudaStream_t s) {
  const int L = sh.L, R = sh.R;
  State* st = (State*)(w + y.state);
  double* G = (double*)(w + y.G);
  T* Hinv = (T*)(w + y.Hinv);
  T* M = (T*)(w + y.M);
  double* gp = (double*)(w + y.gpart);
  for (int l = 0; l < L; ++l) {
    if (l == fix) continue;  // bicpd: this factor stays as given
    int r = tfx_mttkrp(dtype, Tt, L, dims, R, x, l, M, w + y.mtt, y.mtt_bytes, s);
    if (r) return r;
    k_als_inv<T><<<1, NT, inv_smem(R), s>>>(G, L, l, R, Hinv, st);
    if ((r = check("als inverse"))) return r;
    const int nb = (sh.d[l] + ROWS - 1) / ROWS;
    const size_t smb = ((size_t)R * R + 2 * (size_t)ROWS * R) * sizeof(T);
    k_als_apply<T><<<nb, NT, smb, s>>>(M, Hinv, sh.d[l], R, x + sh.off[l], gp);
    if ((r = check("als apply"))) return r;
    k_als_gram_sum<<<(R * R + 255) / 256, 256, 0, s>>>(gp, nb, R, G + (size_t)l * R * R);
    if ((r = check("als gram sum"))) return r;
  }
  return TFX_STATUS_OK;
}

// One iteration's launches (the body of the graph's while-node).
template <class T>
static int body(int dtype, const T* Tt, const int* dims, T* x, T* best, const Dims& sh, const tfx_dgn_options& op,
                int fix, double* stats, int* result, double* info, const Layout& y, char* w,
                cudaGraphConditionalHandle cond, cudaStream_t s) {
  State* st = (State*)(w + y.state);
  if (int r = sweep<T>(dtype, Tt, dims, x, sh, fix, y, w, s)) return r;
  k_als_post<T><<<1, NT, 0, s>>>(x, (T*)(w + y.xo), sh, op.symm, op.factors_norm, fix, (const T*)(w + y.xfix), st);
  if (int r = check("als post")) return r;
  if (op.symm || op.factors_norm > 0.0)
    if (int r = grams_all<T>(x, sh, y, w, s)) return r;
  if (int r = tfx_cp_residual(dtype, Tt, sh.L, dims, sh.R, x, &st->res2, w + y.res, s)) return r;
  k_als_control<T><<<1, NT, 0, s>>>(x, best, sh.nx, op, stats, result, info, st, cond);
  return check("als control");
}

static Dims dims_of(int L, const int* dims, int R, long long* N) {
  Dims sh;
  sh.L = L;
  sh.R = R;
  long long n = 1, acc = 0;
  for (int l = 0; l < L; ++l) {
    sh.d[l] = dims[l];
    sh.off[l] = (int)acc;
    acc += (long long)dims[l] * R;
    n *= dims[l];
  }
  sh.nx = acc;
  *N = n;
  return sh;
}

template <class T>
static int set_attributes(int R) {
  cudaError_t e = cudaFuncSetAttribute(k_als_inv<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)inv_smem(R));
  if (e != cudaSuccess) return tfx_set_cuda_error(e, "als inverse attribute");
  const size_t asm_ = ((size_t)R * R + 2 * (size_t)ROWS * R) * sizeof(T);
  e = cudaFuncSetAttribute(k_als_apply<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)asm_);
  if (e != cudaSuccess) return tfx_set_cuda_error(e, "als apply attribute");
  return TFX_STATUS_OK;
}

// One ALS iteration in place, without the error and the stop tests (the
// 'als' inner method of dGN, GaussNewton.py:275-278).
template <class T>
static int sweep_once(int dtype, const T* Tt, int L, const int* dims, int R, T* x, int fix, char* w, const Layout& y,
                      cudaStream_t s) {
  long long N;
  const Dims sh = dims_of(L, dims, R, &N);
  if (int r = set_attributes<T>(R)) return r;
  cudaError_t e = cudaMemsetAsync(w + y.state, 0, sizeof(State), s);
  if (e != cudaSuccess) return tfx_set_cuda_error(e, "als sweep state");
  if (int r = grams_all<T>(x, sh, y, w, s)) return r;
  return sweep<T>(dtype, Tt, dims, x, sh, fix, y, w, s);
}

template <class T>
static int solve(int dtype, const T* Tt, int L, const int* dims, int R, T* x, T* best, double* stats, int* result,
                 double* info, const tfx_dgn_options& op, int fix, char* w, const Layout& y, cudaStream_t s) {
  long long N;
  const Dims sh = dims_of(L, dims, R, &N);
  State* st = (State*)(w + y.state);
  if (int r = set_attributes<T>(R)) return r;
  cudaError_t e = cudaSuccess;
  // set-up on the caller's stream: state, x_old, best, |T|, Gramians
  k_als_init<T><<<(int)((sh.nx + 255) / 256), 256, 0, s>>>(x, (T*)(w + y.xo), best, sh.nx, st);
  if (int r = check("als init")) return r;
  if (fix >= 0) {
    cudaError_t ce = cudaMemcpyAsync(w + y.xfix, x, (size_t)sh.nx * sizeof(T), cudaMemcpyDeviceToDevice, s);
    if (ce != cudaSuccess) return tfx_set_cuda_error(ce, "als fixed factor copy");
  }
  if (int r = tfx_tensor_norms(dtype, Tt, N, st->tn, w + y.res, s)) return r;
  if (int r = grams_all<T>(x, sh, y, w, s)) return r;

  // graph: one while-node whose body is one iteration
  cudaGraph_t g = nullptr;
  cudaGraphExec_t ge = nullptr;
  cudaStream_t cs = nullptr;
  int status = TFX_STATUS_OK;
  bool capturing = false;
  do {
    if ((e = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking)) != cudaSuccess) break;
    if ((e = cudaGraphCreate(&g, 0)) != cudaSuccess) break;
    cudaGraphConditionalHandle cond;
    if ((e = cudaGraphConditionalHandleCreate(&cond, g, 1, cudaGraphCondAssignDefault)) != cudaSuccess) break;
    cudaGraphNodeParams np = {};
    np.type = cudaGraphNodeTypeConditional;
    np.conditional.handle = cond;
    np.conditional.type = cudaGraphCondTypeWhile;
    np.conditional.size = 1;
    cudaGraphNode_t node;
    if ((e = cudaGraphAddNode(&node, g, nullptr, nullptr, 0, &np)) != cudaSuccess) break;
    cudaGraph_t bodyg = np.conditional.phGraph_out[0];
    if ((e = cudaStreamBeginCaptureToGraph(cs, bodyg, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed)) !=
        cudaSuccess)
      break;
    capturing = true;
    status = body<T>(dtype, Tt, dims, x, best, sh, op, fix, stats, result, info, y, w, cond, cs);
    cudaGraph_t captured = nullptr;
    e = cudaStreamEndCapture(cs, &captured);
    capturing = false;
    if (status != TFX_STATUS_OK || e != cudaSuccess) break;
    if ((e = cudaGraphInstantiate(&ge, g, 0)) != cudaSuccess) break;
    if ((e = cudaGraphLaunch(ge, s)) != cudaSuccess) break;
    tfx_count_launch(1);
  } while (0);
  if (capturing) {
    cudaGraph_t junk = nullptr;
    cudaStreamEndCapture(cs, &junk);
  }
  if (ge) cudaGraphExecDestroy(ge);  // freed after the launch completes
  if (g) cudaGraphDestroy(g);
  if (cs) cudaStreamDestroy(cs);
  if (status != TFX_STATUS_OK) return status;
  if (e != cudaSuccess) return tfx_set_cuda_error(e, "als graph");
  return TFX_STATUS_OK;
}

}  // namespace als
}  // namespace tfx

using namespace tfx;

extern "C" size_t tfx_als_workspace_bytes(int dtype, int L, const int* dims, int R) {
  if (L < 2 || L > TFX_MAX_ORDER || !dims || R < 1) return 0;
  return als::layout(dtype, L, dims, R).total;
}

extern "C" int tfx_als_solve(int dtype, const void* T, int L, const int* dims, int R, void* x, void* best,
                             double* stats, int* result, double* info, const tfx_dgn_options* options, int fix_mode,
                             void* work, size_t work_bytes, void* stream) {
  if (!T || !dims || !x || !best || !stats || !result || !info || !options || !work)
    return tfx_set_error(TFX_STATUS_ERR_ARG, "als: null argument");
  if (dtype != TFX_F32 && dtype != TFX_F64) return tfx_set_error(TFX_STATUS_ERR_ARG, "als: dtype");
  if (L < 2 || L > TFX_MAX_ORDER || R < 1 || options->maxiter < 1)
    return tfx_set_error(TFX_STATUS_ERR_ARG, "als: order, rank or maxiter out of range");
  for (int l = 0; l < L; ++l)
    if (dims[l] < 1) return tfx_set_error(TFX_STATUS_ERR_ARG, "als: dimension < 1");
  if (R > als::RMAX) return tfx_set_error(TFX_STATUS_ERR_UNSUPPORTED, "als: rank above 96");
  if (fix_mode < -1 || fix_mode >= L) return tfx_set_error(TFX_STATUS_ERR_ARG, "als: fix_mode out of range");
  if (options->symm)
    for (int l = 1; l < L; ++l)
      if (dims[l] != dims[0]) return tfx_set_error(TFX_STATUS_ERR_ARG, "als: symm needs equal dimensions");
  if (((uintptr_t)work & 255) != 0) return tfx_set_error(TFX_STATUS_ERR_ARG, "als: workspace not 256-byte aligned");
  const als::Layout y = als::layout(dtype, L, dims, R);
  if (work_bytes < y.total) return tfx_set_error(TFX_STATUS_ERR_ARG, "als: workspace too small");
  cudaStream_t s = (cudaStream_t)stream;
  if (dtype == TFX_F32)
    return als::solve<float>(dtype, (const float*)T, L, dims, R, (float*)x, (float*)best, stats, result, info,
                             *options, fix_mode, (char*)work, y, s);
  return als::solve<double>(dtype, (const double*)T, L, dims, R, (double*)x, (double*)best, stats, result, info,
                            *options, fix_mode, (char*)work, y, s);
}

extern "C" int tfx_als_sweep(int dtype, const void* T, int L, const int* dims, int R, void* x, int fix_mode,
                             void* work, size_t work_bytes, void* stream) {
  if (!T || !dims || !x || !work) return tfx_set_error(TFX_STATUS_ERR_ARG, "als sweep: null argument");
  if (dtype != TFX_F32 && dtype != TFX_F64) return tfx_set_error(TFX_STATUS_ERR_ARG, "als sweep: dtype");
  if (L < 2 || L > TFX_MAX_ORDER || R < 1) return tfx_set_error(TFX_STATUS_ERR_ARG, "als sweep: order or rank");
  for (int l = 0; l < L; ++l)
    if (dims[l] < 1) return tfx_set_error(TFX_STATUS_ERR_ARG, "als sweep: dimension < 1");
  if (R > als::RMAX) return tfx_set_error(TFX_STATUS_ERR_UNSUPPORTED, "als sweep: rank above 96");
  if (fix_mode < -1 || fix_mode >= L) return tfx_set_error(TFX_STATUS_ERR_ARG, "als sweep: fix_mode out of range");
  if (((uintptr_t)work & 255) != 0)
    return tfx_set_error(TFX_STATUS_ERR_ARG, "als sweep: workspace not 256-byte aligned");
  const als::Layout y = als::layout(dtype, L, dims, R);
  if (work_bytes < y.total) return tfx_set_error(TFX_STATUS_ERR_ARG, "als sweep: workspace too small");
  cudaStream_t s = (cudaStream_t)stream;
  if (dtype == TFX_F32)
    return als::sweep_once<float>(dtype, (const float*)T, L, dims, R, (float*)x, fix_mode, (char*)work, y, s);
  return als::sweep_once<double>(dtype, (const double*)T, L, dims, R, (double*)x, fix_mode, (char*)work, y, s);
}
