// The inner methods of dGN that run outside the persistent engine (Tensor Fox
// v1.2.1 GaussNewton.py:254-312 compute_step), one host-driven iteration at a
// time:
//
//  * tfx_dgn_direct_step -- the 'direct' inner method (GaussNewton.py:630-653):
//    the Gauss-Newton matrix H of GaussNewton.py:656-701 is formed explicitly
//    (n x n FP64, n = R * sum(dims)), damped on the diagonal, and the step
//    y = (H + damp diag(Gamma))^{-1} grad comes from an LU factorisation with
//    partial pivoting.  The reference row-scales the system by M^2 and solves
//    it by QR; both give the same y up to rounding.  H is the reference's
//    matrix, not exactly J^T J: its off-diagonal blocks (l, m), l > m, are
//    filled through a helper that loops over the block's row count in both
//    indices (MultilinearAlgebra.py:276-289 hadamard), so only the leading
//    R d_l columns of each such block are set and the rest stay zero.  That
//    matrix need not be positive definite, hence LU rather than Cholesky.
//  * tfx_dgn_step_update -- what follows every inner step (GaussNewton.py:
//    284-297): x += y (or x = the swept factors), x2cpd with column balancing
//    (Conversion.py:21-49, 361-387), transform (Conversion.py:412-444), the
//    fixed factor of bicpd restored, and the scalars of the gain ratio, the
//    step size and the gradient norm.
//
// The 'als' inner method's sweep is tfx_als_sweep (als.cu).  No kernel here
// waits on another: every dependency is a kernel boundary on one stream.
#include <math.h>
#include <stdint.h>

#include <algorithm>

#include "tfx_capi_internal.h"
#include "tfx_common.cuh"
#include "tfx_gb300.h"

namespace tfx {
namespace stepped {

constexpr int NB = 32;            // LU panel width and triangular-solve block
constexpr int PANEL_THREADS = 1024;
constexpr long long NMAX = 24576; // largest system: the permuted right-hand side sits in shared memory

struct Shape {
  int L, R;
  int d[TFX_MAX_ORDER];
  long long off[TFX_MAX_ORDER + 1];  // block offsets of the flat point
  long long n;
};

static Shape shape_of(int L, const int* dims, int R) {
  Shape sh;
  sh.L = L;
  sh.R = R;
  long long acc = 0;
  for (int l = 0; l < L; ++l) {
    sh.d[l] = dims[l];
    sh.off[l] = acc;
    acc += (long long)dims[l] * R;
  }
  for (int l = L; l <= TFX_MAX_ORDER; ++l) sh.off[l] = acc;
  for (int l = L; l < TFX_MAX_ORDER; ++l) sh.d[l] = 0;
  sh.n = acc;
  return sh;
}

__host__ inline size_t up256(size_t v) { return (v + 255) & ~(size_t)255; }

struct Layout {
  size_t G, P1, P2, gamma, flag, piv, b, z, M, mtt, H, total;
  size_t mtt_bytes;
};

static Layout layout(int dtype, int L, const int* dims, int R) {
  const size_t es = dtype == TFX_F64 ? 8 : 4;
  const Shape sh = shape_of(L, dims, R);
  const size_t n = (size_t)sh.n, RR = (size_t)R * R;
  int maxd = 0;
  size_t mtt = 0;
  for (int l = 0; l < L; ++l) {
    maxd = std::max(maxd, dims[l]);
    mtt = std::max(mtt, tfx_mttkrp_scratch_bytes(dtype, L, dims, R, l));
  }
  Layout y;
  size_t o = 0;
  y.G = o;     o += up256((size_t)L * RR * 8);
  y.P1 = o;    o += up256((size_t)L * RR * 8);
  y.P2 = o;    o += up256((size_t)L * L * RR * 8);
  y.gamma = o; o += up256((size_t)L * R * 8);
  y.flag = o;  o += 256;
  y.piv = o;   o += up256(n * 4);
  y.b = o;     o += up256(n * 8);
  y.z = o;     o += up256(n * 8);
  y.M = o;     o += up256((size_t)maxd * R * es);
  y.mtt = o;   o += up256(mtt);
  y.mtt_bytes = mtt;
  y.H = o;     o += up256(n * n * 8);
  y.total = o;
  return y;
}

// ---------------------------------------------------------------------------
// G_l = W_l^T W_l in FP64 (GaussNewton.py:520-548); grid (ceil(R^2/256), L).
// ---------------------------------------------------------------------------
template <class T>
__global__ void k_grams(const T* __restrict__ W, Shape sh, double* __restrict__ G) {
  const int l = blockIdx.y, R = sh.R, d = sh.d[l];
  const T* Wl = W + sh.off[l];
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < R * R; e += gridDim.x * blockDim.x) {
    const int a = e / R, b = e - a * R;
    double s = 0.0;
    for (int i = 0; i < d; ++i) s = fma((double)Wl[(size_t)a * d + i], (double)Wl[(size_t)b * d + i], s);
    G[(size_t)l * R * R + e] = s;
  }
}

// P1[l] = o_{m != l} G_m, P2[l][m] = o_{k not in {l, m}} G_k, and the
// regularisation gamma[l][r] = max|P1[L-1]| sqrt|P1[l]_{rr}| (GaussNewton.py:
// 584-607: the maximum of the LAST mode's P1, as the reference computes it).
// One CTA.
__global__ void k_direct_prep(const double* __restrict__ G, int L, int R, double* __restrict__ P1,
                              double* __restrict__ P2, double* __restrict__ gamma) {
  __shared__ double red[32];
  const int tid = threadIdx.x, RR = R * R;
  for (int e = tid; e < L * L * RR; e += blockDim.x) {
    const int l = e / (L * RR), rem = e - l * L * RR, m = rem / RR, ab = rem - m * RR;
    double p = 1.0;
    for (int k = 0; k < L; ++k)
      if (k != l && k != m) p *= G[(size_t)k * RR + ab];
    P2[e] = p;
  }
  for (int e = tid; e < L * RR; e += blockDim.x) {
    const int l = e / RR, ab = e - l * RR;
    double p = 1.0;
    for (int k = 0; k < L; ++k)
      if (k != l) p *= G[(size_t)k * RR + ab];
    P1[e] = p;
  }
  __syncthreads();
  double mx = 0.0;
  for (int e = tid; e < RR; e += blockDim.x) mx = fmax(mx, fabs(P1[(size_t)(L - 1) * RR + e]));
  mx = warp_max(mx);
  if ((tid & 31) == 0) red[tid >> 5] = mx;
  __syncthreads();
  if (tid == 0) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t = fmax(t, red[w]);
    red[0] = t;
  }
  __syncthreads();
  const double s = red[0];
  for (int e = tid; e < L * R; e += blockDim.x) {
    const int l = e / R, r = e - l * R;
    gamma[e] = s * sqrt(fabs(P1[(size_t)l * RR + (size_t)r * R + r]));
  }
}

// grad block l (vec_F) = MTTKRP_l - W_l P1[l]  (the negated compute_grad,
// GaussNewton.py:401-427 and :645).
template <class T>
__global__ void k_direct_grad(const T* __restrict__ M, const T* __restrict__ W, int d, int R,
                              const double* __restrict__ P1l, double* __restrict__ g) {
  const long long n = (long long)d * R;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
    const int r = (int)(e / d), i = (int)(e - (long long)r * d);
    double acc = 0.0;
    for (int s = 0; s < R; ++s) acc = fma((double)W[(size_t)s * d + i], P1l[(size_t)s * R + r], acc);
    g[e] = (double)M[e] - acc;
  }
}

__device__ __forceinline__ void decode(const Shape& sh, long long p, int& l, int& r, int& i) {
  l = 0;
  while (l + 1 < sh.L && p >= sh.off[l + 1]) ++l;
  const long long loc = p - sh.off[l];
  r = (int)(loc / sh.d[l]);
  i = (int)(loc - (long long)r * sh.d[l]);
}

// H + damp diag(Gamma), row-major n x n.  Block (l, l): kron(P1[l], I);
// block (l, m), l > m: entry ((l, r, i), (m, s, j)) = P2[l][m][r][s] W_l[i, s] W_m[j, r]
// where the column inside the block is below R d_l, else 0; block (m, l) is its
// transpose.  Block 32 x 8 threads, each thread 4 rows of one column.
template <class T>
__global__ void k_direct_hessian(const T* __restrict__ W, Shape sh, const double* __restrict__ P1,
                                 const double* __restrict__ P2, const double* __restrict__ gamma, double damp,
                                 double* __restrict__ H) {
  const long long n = sh.n;
  const long long q = (long long)blockIdx.x * 32 + threadIdx.x;
  if (q >= n) return;
  const int R = sh.R, RR = R * R, L = sh.L;
  int m, s, j;
  decode(sh, q, m, s, j);
  for (int k = 0; k < 4; ++k) {
    const long long p = (long long)blockIdx.y * 32 + threadIdx.y + 8 * k;
    if (p >= n) break;
    int l, r, i;
    decode(sh, p, l, r, i);
    double v = 0.0;
    if (l == m) {
      if (i == j) v = P1[(size_t)l * RR + (size_t)r * R + s];
      if (p == q) v += damp * gamma[(size_t)l * R + r];
    } else {
      const bool keep = l > m ? (q - sh.off[m]) < (long long)R * sh.d[l] : (p - sh.off[l]) < (long long)R * sh.d[m];
      if (keep)
        v = P2[((size_t)l * L + m) * RR + (size_t)r * R + s] * (double)W[sh.off[l] + (size_t)s * sh.d[l] + i] *
            (double)W[sh.off[m] + (size_t)r * sh.d[m] + j];
    }
    H[p * n + q] = v;
  }
}

// ---------------------------------------------------------------------------
// LU with partial pivoting, right-looking, panels of NB columns.
// ---------------------------------------------------------------------------

// Panel k0 .. k0 + kb - 1 over rows k0 .. n - 1 (one CTA): per column the
// first row of largest |value| is the pivot (LAPACK's choice), the pivot row
// is swapped inside the panel, the column below is divided by the pivot and
// the panel's later columns get the rank-one update.  A zero pivot marks the
// matrix singular (flag) and leaves the column as it is.  Each thread owns
// rows; a row's panel segment is read in two chunks of 16 independent loads
// (the pivot row comes from shared memory), so a row costs two memory round
// trips per column rather than one per updated entry.
constexpr int PCH = 16;  // panel entries per register chunk
__global__ void __launch_bounds__(PANEL_THREADS) k_lu_panel(double* __restrict__ H, long long n, int k0, int kb,
                                                            int* __restrict__ piv, int* __restrict__ flag) {
  __shared__ double sv[PANEL_THREADS / 32];
  __shared__ long long si[PANEL_THREADS / 32];
  __shared__ long long s_p;
  __shared__ double sp[NB];  // the pivot row's panel segment
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  for (int j = 0; j < kb; ++j) {
    const long long c = k0 + j;
    double best = -1.0;
    long long bi = c;
#pragma unroll 4
    for (long long i = c + tid; i < n; i += PANEL_THREADS) {
      const double v = fabs(H[i * n + c]);
      if (v > best) {
        best = v;
        bi = i;
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const double ov = __shfl_xor_sync(0xffffffffu, best, o);
      const long long oi = __shfl_xor_sync(0xffffffffu, bi, o);
      if (ov > best || (ov == best && oi < bi)) {
        best = ov;
        bi = oi;
      }
    }
    if (lane == 0) {
      sv[wid] = best;
      si[wid] = bi;
    }
    __syncthreads();
    if (tid == 0) {
      double bv = sv[0];
      long long bb = si[0];
      for (int w = 1; w < PANEL_THREADS / 32; ++w)
        if (sv[w] > bv || (sv[w] == bv && si[w] < bb)) {
          bv = sv[w];
          bb = si[w];
        }
      s_p = bb;
      piv[c] = (int)bb;
    }
    __syncthreads();
    const long long pr = s_p;
    if (pr != c)
      for (int t = tid; t < kb; t += PANEL_THREADS) {
        const double a = H[c * n + k0 + t];
        H[c * n + k0 + t] = H[pr * n + k0 + t];
        H[pr * n + k0 + t] = a;
      }
    __syncthreads();
    if (tid < kb) sp[tid] = H[c * n + k0 + tid];
    __syncthreads();
    const double pv = sp[j];
    if (pv == 0.0) {
      if (tid == 0) *flag = 1;
      __syncthreads();
      continue;
    }
    for (long long i = c + 1 + tid; i < n; i += PANEL_THREADS) {
      double* row = H + i * n + k0;
      const double lic = row[j] / pv;
      for (int t0 = 0; t0 < kb; t0 += PCH) {
        if (t0 + PCH <= j + 1) continue;  // chunk entirely at or left of column j
        double v[PCH];
#pragma unroll
        for (int u = 0; u < PCH; ++u) {
          const int t = t0 + u;
          v[u] = (t > j && t < kb) ? row[t] : 0.0;
        }
#pragma unroll
        for (int u = 0; u < PCH; ++u) {
          const int t = t0 + u;
          if (t > j && t < kb) row[t] = v[u] - lic * sp[t];
        }
      }
      row[j] = lic;
    }
    __syncthreads();
  }
}

// The panel's row swaps applied, in order, to every column outside the panel.
__global__ void k_lu_swap(double* __restrict__ H, long long n, int k0, int kb, const int* __restrict__ piv) {
  const long long col = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (col >= n || (col >= k0 && col < k0 + kb)) return;
  for (int j = 0; j < kb; ++j) {
    const long long c = k0 + j, pr = piv[c];
    if (pr != c) {
      const double a = H[c * n + col];
      H[c * n + col] = H[pr * n + col];
      H[pr * n + col] = a;
    }
  }
}

// U12 = L11^{-1} A12 (L11 unit lower, kb x kb): one column per thread.
__global__ void k_lu_trsm(double* __restrict__ H, long long n, int k0, int kb) {
  __shared__ double sL[NB][NB + 1];
  for (int e = threadIdx.x; e < kb * kb; e += blockDim.x) {
    const int r = e / kb, t = e - r * kb;
    sL[r][t] = H[(k0 + r) * n + k0 + t];
  }
  __syncthreads();
  const long long col = (long long)k0 + kb + (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (col >= n) return;
  double a[NB];
#pragma unroll
  for (int r = 0; r < NB; ++r) a[r] = r < kb ? H[(k0 + r) * n + col] : 0.0;
#pragma unroll
  for (int r = 1; r < NB; ++r) {
    double v = a[r];
#pragma unroll
    for (int t = 0; t < r; ++t) v -= sL[r][t] * a[t];
    a[r] = v;
  }
#pragma unroll
  for (int r = 0; r < NB; ++r)
    if (r < kb) H[(k0 + r) * n + col] = a[r];
}

// A22 -= L21 U12 on 64 x 64 tiles; 256 threads, a 4 x 4 block of outputs each
// (rows ty + 16 a, columns tx + 16 b).
__global__ void __launch_bounds__(256) k_lu_gemm(double* __restrict__ H, long long n, int k0, int kb) {
  __shared__ double sA[64][NB + 1];
  __shared__ double sB[NB][64 + 1];
  const long long base = (long long)k0 + kb;
  const long long r0 = base + (long long)blockIdx.y * 64, c0 = base + (long long)blockIdx.x * 64;
  const int tid = threadIdx.x;
  for (int e = tid; e < 64 * NB; e += 256) {
    const int r = e / NB, t = e - r * NB;
    const long long row = r0 + r;
    sA[r][t] = (row < n && t < kb) ? H[row * n + k0 + t] : 0.0;
  }
  for (int e = tid; e < NB * 64; e += 256) {
    const int t = e / 64, c = e - t * 64;
    const long long col = c0 + c;
    sB[t][c] = (col < n && t < kb) ? H[(k0 + t) * n + col] : 0.0;
  }
  __syncthreads();
  const int tx = tid & 15, ty = tid >> 4;
  double acc[4][4];
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b) acc[a][b] = 0.0;
  for (int t = 0; t < kb; ++t) {
    double av[4], bv[4];
#pragma unroll
    for (int a = 0; a < 4; ++a) av[a] = sA[ty + 16 * a][t];
#pragma unroll
    for (int b = 0; b < 4; ++b) bv[b] = sB[t][tx + 16 * b];
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
      for (int b = 0; b < 4; ++b) acc[a][b] = fma(av[a], bv[b], acc[a][b]);
  }
#pragma unroll
  for (int a = 0; a < 4; ++a) {
    const long long row = r0 + ty + 16 * a;
    if (row >= n) continue;
#pragma unroll
    for (int b = 0; b < 4; ++b) {
      const long long col = c0 + tx + 16 * b;
      if (col < n) H[row * n + col] -= acc[a][b];
    }
  }
}

// b = P grad: the pivots' swaps applied in order (one CTA, b staged in shared memory).
__global__ void k_permute_rhs(const double* __restrict__ grad, const int* __restrict__ piv, long long n,
                              double* __restrict__ b) {
  extern __shared__ double sb[];
  for (long long e = threadIdx.x; e < n; e += blockDim.x) sb[e] = grad[e];
  __syncthreads();
  if (threadIdx.x == 0)
    for (long long c = 0; c < n; ++c) {
      const long long p = piv[c];
      if (p != c) {
        const double a = sb[c];
        sb[c] = sb[p];
        sb[p] = a;
      }
    }
  __syncthreads();
  for (long long e = threadIdx.x; e < n; e += blockDim.x) b[e] = sb[e];
}

// Forward substitution, block k0: every CTA solves the unit-lower diagonal
// block for z[k0 .. k0+kb) from b (CTA 0 stores it), then updates the rows
// below it that it owns: b[i] -= L[i, k0:k0+kb] z.
__global__ void k_fwd_block(const double* __restrict__ H, long long n, int k0, int kb, double* __restrict__ b,
                            double* __restrict__ z) {
  __shared__ double sz[NB];
  if (threadIdx.x == 0) {
    for (int r = 0; r < kb; ++r) {
      double v = b[k0 + r];
      for (int t = 0; t < r; ++t) v -= H[(k0 + r) * n + k0 + t] * sz[t];
      sz[r] = v;
    }
  }
  __syncthreads();
  if (blockIdx.x == 0 && threadIdx.x < kb) z[k0 + threadIdx.x] = sz[threadIdx.x];
  const long long i = (long long)k0 + kb + (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double v = b[i];
  for (int t = 0; t < kb; ++t) v -= H[i * n + k0 + t] * sz[t];
  b[i] = v;
}

// Backward substitution, block k0 (blocks taken last to first): every CTA
// solves the upper diagonal block for y[k0 .. k0+kb) from z (CTA 0 stores it),
// then updates the rows above it that it owns: z[i] -= U[i, k0:k0+kb] y.
__global__ void k_bwd_block(const double* __restrict__ H, long long n, int k0, int kb, double* __restrict__ z,
                            double* __restrict__ y) {
  __shared__ double sy[NB];
  if (threadIdx.x == 0) {
    for (int r = kb - 1; r >= 0; --r) {
      double v = z[k0 + r];
      for (int t = r + 1; t < kb; ++t) v -= H[(k0 + r) * n + k0 + t] * sy[t];
      sy[r] = v / H[(k0 + r) * n + k0 + r];
    }
  }
  __syncthreads();
  if (blockIdx.x == 0 && threadIdx.x < kb) y[k0 + threadIdx.x] = sy[threadIdx.x];
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= k0) return;
  double v = z[i];
  for (int t = 0; t < kb; ++t) v -= H[i * n + k0 + t] * sy[t];
  z[i] = v;
}

// A singular matrix gives y = 0 (the reference's LinAlgError branch, GaussNewton.py:648-651).
__global__ void k_zero_if_flag(double* __restrict__ y, long long n, const int* __restrict__ flag) {
  if (*flag == 0) return;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x)
    y[e] = 0.0;
}

// ---------------------------------------------------------------------------
// The update after an inner step (one CTA).  Phase 1: x_new = W (from_W) or
// x + y; out[0] = ||x_new - x||^2, out[1] = ||x||^2, out[2] = (x_new - x) .
// (grad + damp (x_new - x)) and out[3] = max|grad| (NaN without a gradient,
// as the 'als' step's [nan] gradient gives).  Phase 2: the factors W from
// x_new -- column balancing, transform, fixed factor.
//
// ``aliased``: the reference's factor list holds ONE array L times (after a
// symmetrising transform, Conversion.py:432-437, or a symmetric start).  Then
// x2cpd writes every block into that array, so it ends holding the LAST
// block; balancing multiplies it once per mode; and the in-place sum of
// transform doubles it L - 1 times before the division by L.
// ---------------------------------------------------------------------------
template <class T>
__global__ void __launch_bounds__(1024) k_step_update(T* __restrict__ x, T* __restrict__ W, const double* __restrict__ y,
                                                      const double* __restrict__ grad, double damp, int from_W,
                                                      Shape sh, int symm, double factors_norm, int aliased, int fix,
                                                      const T* __restrict__ Wfix, double* __restrict__ out) {
  extern __shared__ double sm[];  // L * R column norms, then L * R balancing factors
  __shared__ double red[4][32];
  __shared__ double fnorm[TFX_MAX_ORDER];
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5, nw = blockDim.x >> 5;
  const int L = sh.L, R = sh.R;
  const long long n = sh.n;
  double s0 = 0.0, s1 = 0.0, s2 = 0.0, gi = 0.0;
  bool gnan = false;
  for (long long e = tid; e < n; e += blockDim.x) {
    const double xo = (double)x[e];
    const T xn = from_W ? W[e] : (T)(xo + y[e]);
    const double dv = (double)xn - xo;
    s0 = fma(xo, xo, s0);
    s1 = fma(dv, dv, s1);
    if (grad) {
      const double g = grad[e];
      s2 = fma(dv, g + damp * dv, s2);
      if (g != g) gnan = true;
      gi = fmax(gi, fabs(g));
    }
    x[e] = xn;
  }
  s0 = warp_sum(s0);
  s1 = warp_sum(s1);
  s2 = warp_sum(s2);
  gi = warp_max(gi);
  const int anynan = __any_sync(0xffffffffu, gnan);
  if (lane == 0) {
    red[0][wid] = s0;
    red[1][wid] = s1;
    red[2][wid] = s2;
    red[3][wid] = anynan ? NAN : gi;
  }
  __syncthreads();
  if (tid == 0) {
    double a = 0.0, b = 0.0, c = 0.0, m = 0.0;
    bool mn = false;
    for (int w = 0; w < nw; ++w) {
      a += red[0][w];
      b += red[1][w];
      c += red[2][w];
      if (red[3][w] != red[3][w]) mn = true;
      m = fmax(m, red[3][w]);
    }
    out[0] = b;
    out[1] = a;
    out[2] = grad ? c : NAN;
    out[3] = grad ? (mn ? NAN : m) : NAN;
  }
  __syncthreads();

  // column norms of x_new (per mode, or of the last block when aliased)
  double* nrm = sm;
  double* fac = sm + L * R;
  for (int p = wid; p < L * R; p += nw) {
    const int l = aliased ? L - 1 : p / R, r = p % R;
    const int d = sh.d[l];
    const T* col = x + sh.off[l] + (size_t)r * d;
    double s = 0.0;
    for (int i = lane; i < d; i += 32) s = fma((double)col[i], (double)col[i], s);
    s = warp_sum(s);
    if (lane == 0) nrm[p] = sqrt(s);
  }
  __syncthreads();
  for (int r = tid; r < R; r += blockDim.x) {
    double prod = 1.0;
    for (int l = 0; l < L; ++l) prod *= nrm[l * R + r];
    if (prod != 0.0) {
      const double num = pow(prod, 1.0 / (double)L);
      for (int l = 0; l < L; ++l) fac[l * R + r] = num / nrm[l * R + r];
    } else {
      for (int l = 0; l < L; ++l) fac[l * R + r] = 1.0;
    }
  }
  __syncthreads();
  if (aliased) {
    // one array: the last block, scaled once per mode, then (symm) doubled L-1 times and divided by L
    const int d = sh.d[L - 1];
    for (long long e = tid; e < (long long)d * R; e += blockDim.x) {
      const int r = (int)(e / d);
      double v = (double)x[sh.off[L - 1] + e];
      for (int l = 0; l < L; ++l) v = (double)(T)(v * fac[l * R + r]);
      if (symm) {
        for (int l = 1; l < L; ++l) v = (double)(T)(v + v);
        v = v / (double)L;
      }
      for (int l = 0; l < L; ++l) W[sh.off[l] + e] = (T)v;
    }
  } else {
    for (long long e = tid; e < n; e += blockDim.x) {
      int l = 0;
      while (l + 1 < L && e >= sh.off[l + 1]) ++l;
      const int r = (int)((e - sh.off[l]) / sh.d[l]);
      W[e] = (T)(fac[l * R + r] * (double)x[e]);
    }
    if (symm) {
      __syncthreads();
      const int d = sh.d[0];
      for (long long e = tid; e < (long long)d * R; e += blockDim.x) {
        T s = W[e];
        for (int l = 1; l < L; ++l) s = s + W[sh.off[l] + e];
        s = s / (T)L;
        for (int l = 0; l < L; ++l) W[sh.off[l] + e] = s;
      }
    }
  }
  __syncthreads();
  if (factors_norm > 0.0) {
    for (int l = 0; l < L; ++l) {
      const long long nl = (long long)sh.d[l] * R;
      double q = 0.0;
      for (long long e = tid; e < nl; e += blockDim.x) {
        const double v = (double)W[sh.off[l] + e];
        q = fma(v, v, q);
      }
      q = warp_sum(q);
      if (lane == 0) red[0][wid] = q;
      __syncthreads();
      if (tid == 0) {
        double t = 0.0;
        for (int w = 0; w < nw; ++w) t += red[0][w];
        fnorm[l] = sqrt(t);
      }
      __syncthreads();
    }
    for (long long e = tid; e < n; e += blockDim.x) {
      int l = 0;
      while (l + 1 < L && e >= sh.off[l + 1]) ++l;
      W[e] = (T)(factors_norm * (1.0 / fnorm[l]) * (double)W[e]);
    }
    __syncthreads();
  }
  if (fix >= 0) {
    const long long nl = (long long)sh.d[fix] * R;
    for (long long e = tid; e < nl; e += blockDim.x) W[sh.off[fix] + e] = Wfix[sh.off[fix] + e];
  }
}

static int check(const char* w) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return tfx_set_cuda_error(e, w);
  tfx_count_launch(1);
  return TFX_STATUS_OK;
}

template <class T>
static int direct_step(int dtype, const T* Tt, int L, const int* dims, int R, const T* W, double damp, double* y,
                       double* grad, char* w, const Layout& ly, cudaStream_t s) {
  const Shape sh = shape_of(L, dims, R);
  const long long n = sh.n;
  const int RR = R * R;
  double* G = (double*)(w + ly.G);
  double* P1 = (double*)(w + ly.P1);
  double* P2 = (double*)(w + ly.P2);
  double* gamma = (double*)(w + ly.gamma);
  int* flag = (int*)(w + ly.flag);
  int* piv = (int*)(w + ly.piv);
  double* b = (double*)(w + ly.b);
  double* z = (double*)(w + ly.z);
  T* M = (T*)(w + ly.M);
  double* H = (double*)(w + ly.H);

  k_grams<T><<<dim3((RR + 255) / 256, L), 256, 0, s>>>(W, sh, G);
  if (int r = check("direct grams")) return r;
  k_direct_prep<<<1, 256, 0, s>>>(G, L, R, P1, P2, gamma);
  if (int r = check("direct prep")) return r;
  cudaError_t ce = cudaMemsetAsync(flag, 0, sizeof(int), s);
  if (ce != cudaSuccess) return tfx_set_cuda_error(ce, "direct flag");
  for (int l = 0; l < L; ++l) {
    if (int r = tfx_mttkrp(dtype, Tt, L, dims, R, W, l, M, w + ly.mtt, ly.mtt_bytes, s)) return r;
    const long long nl = (long long)dims[l] * R;
    const int nb = (int)std::min<long long>((nl + 255) / 256, 4096);
    k_direct_grad<T><<<nb, 256, 0, s>>>(M, W + sh.off[l], dims[l], R, P1 + (size_t)l * RR, grad + sh.off[l]);
    if (int r = check("direct gradient")) return r;
  }
  const int tiles = (int)((n + 31) / 32);
  k_direct_hessian<T><<<dim3(tiles, tiles), dim3(32, 8), 0, s>>>(W, sh, P1, P2, gamma, damp, H);
  if (int r = check("direct hessian")) return r;
  for (long long k0 = 0; k0 < n; k0 += NB) {
    const int kb = (int)std::min<long long>(NB, n - k0);
    k_lu_panel<<<1, PANEL_THREADS, 0, s>>>(H, n, (int)k0, kb, piv, flag);
    if (int r = check("lu panel")) return r;
    k_lu_swap<<<(int)((n + 255) / 256), 256, 0, s>>>(H, n, (int)k0, kb, piv);
    if (int r = check("lu swap")) return r;
    const long long rest = n - k0 - kb;
    if (rest > 0) {
      k_lu_trsm<<<(int)((rest + 127) / 128), 128, 0, s>>>(H, n, (int)k0, kb);
      if (int r = check("lu trsm")) return r;
      const int t = (int)((rest + 63) / 64);
      k_lu_gemm<<<dim3(t, t), 256, 0, s>>>(H, n, (int)k0, kb);
      if (int r = check("lu update")) return r;
    }
  }
  k_permute_rhs<<<1, 1024, (size_t)n * 8, s>>>(grad, piv, n, b);
  if (int r = check("rhs permutation")) return r;
  for (long long k0 = 0; k0 < n; k0 += NB) {
    const int kb = (int)std::min<long long>(NB, n - k0);
    const long long rest = n - k0 - kb;
    const int nb = (int)std::max<long long>(1, (rest + 255) / 256);
    k_fwd_block<<<nb, 256, 0, s>>>(H, n, (int)k0, kb, b, z);
    if (int r = check("forward substitution")) return r;
  }
  const long long last = ((n - 1) / NB) * NB;
  for (long long k0 = last; k0 >= 0; k0 -= NB) {
    const int kb = (int)std::min<long long>(NB, n - k0);
    const int nb = (int)std::max<long long>(1, (k0 + 255) / 256);
    k_bwd_block<<<nb, 256, 0, s>>>(H, n, (int)k0, kb, z, y);
    if (int r = check("backward substitution")) return r;
  }
  k_zero_if_flag<<<(int)std::min<long long>((n + 255) / 256, 1024), 256, 0, s>>>(y, n, flag);
  return check("singular step");
}

}  // namespace stepped
}  // namespace tfx

using namespace tfx;

static int validate(const char* who, int dtype, int L, const int* dims, int R) {
  if (dtype != TFX_F32 && dtype != TFX_F64) return tfx_set_error(TFX_STATUS_ERR_ARG, who);
  if (L < 2 || L > TFX_MAX_ORDER || !dims || R < 1) return tfx_set_error(TFX_STATUS_ERR_ARG, who);
  for (int l = 0; l < L; ++l)
    if (dims[l] < 1) return tfx_set_error(TFX_STATUS_ERR_ARG, who);
  return TFX_STATUS_OK;
}

extern "C" size_t tfx_dgn_direct_workspace_bytes(int dtype, int L, const int* dims, int R) {
  if (validate("direct workspace", dtype, L, dims, R)) return 0;
  return stepped::layout(dtype, L, dims, R).total;
}

extern "C" int tfx_dgn_direct_step(int dtype, const void* T, int L, const int* dims, int R, const void* W, double damp,
                                   double* y, double* grad, void* work, size_t work_bytes, void* stream) {
  if (!T || !W || !y || !grad || !work) return tfx_set_error(TFX_STATUS_ERR_ARG, "direct step: null argument");
  if (int r = validate("direct step: dtype, order, rank or dimension out of range", dtype, L, dims, R)) return r;
  long long n = 0;
  for (int l = 0; l < L; ++l) n += (long long)dims[l] * R;
  if (n > stepped::NMAX)
    return tfx_set_error(TFX_STATUS_ERR_UNSUPPORTED, "direct step: R * sum(dims) above 24576");
  if (((uintptr_t)work & 255) != 0)
    return tfx_set_error(TFX_STATUS_ERR_ARG, "direct step: workspace not 256-byte aligned");
  const stepped::Layout ly = stepped::layout(dtype, L, dims, R);
  if (work_bytes < ly.total) return tfx_set_error(TFX_STATUS_ERR_ARG, "direct step: workspace too small");
  cudaError_t e = cudaFuncSetAttribute(stepped::k_permute_rhs, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)(n * 8));
  if (e != cudaSuccess) return tfx_set_cuda_error(e, "direct step attribute");
  cudaStream_t s = (cudaStream_t)stream;
  if (dtype == TFX_F32)
    return stepped::direct_step<float>(dtype, (const float*)T, L, dims, R, (const float*)W, damp, y, grad,
                                       (char*)work, ly, s);
  return stepped::direct_step<double>(dtype, (const double*)T, L, dims, R, (const double*)W, damp, y, grad,
                                      (char*)work, ly, s);
}

extern "C" int tfx_dgn_step_update(int dtype, int L, const int* dims, int R, void* x, void* W, const double* y,
                                   const double* grad, double damp, int from_W, int symm, double factors_norm,
                                   int aliased, int fix_mode, const void* Wfix, double* out, void* stream) {
  if (!x || !W || !out || (!from_W && !y)) return tfx_set_error(TFX_STATUS_ERR_ARG, "step update: null argument");
  if (int r = validate("step update: dtype, order, rank or dimension out of range", dtype, L, dims, R)) return r;
  if (fix_mode < -1 || fix_mode >= L || (fix_mode >= 0 && !Wfix))
    return tfx_set_error(TFX_STATUS_ERR_ARG, "step update: fix_mode out of range or no fixed factor");
  if (symm || aliased)
    for (int l = 1; l < L; ++l)
      if (dims[l] != dims[0]) return tfx_set_error(TFX_STATUS_ERR_ARG, "step update: symm needs equal dimensions");
  const stepped::Shape sh = stepped::shape_of(L, dims, R);
  const size_t smem = (size_t)2 * L * R * 8;
  if (smem > 200 * 1024) return tfx_set_error(TFX_STATUS_ERR_UNSUPPORTED, "step update: L * R too large");
  cudaStream_t s = (cudaStream_t)stream;
  cudaError_t e;
  if (dtype == TFX_F32) {
    e = cudaFuncSetAttribute(stepped::k_step_update<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return tfx_set_cuda_error(e, "step update attribute");
    stepped::k_step_update<float><<<1, 1024, smem, s>>>((float*)x, (float*)W, y, grad, damp, from_W, sh, symm,
                                                        factors_norm, aliased, fix_mode, (const float*)Wfix, out);
  } else {
    e = cudaFuncSetAttribute(stepped::k_step_update<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return tfx_set_cuda_error(e, "step update attribute");
    stepped::k_step_update<double><<<1, 1024, smem, s>>>((double*)x, (double*)W, y, grad, damp, from_W, sh, symm,
                                                         factors_norm, aliased, fix_mode, (const double*)Wfix, out);
  }
  return stepped::check("step update");
}
