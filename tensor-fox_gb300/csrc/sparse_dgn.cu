// Damped Gauss-Newton directly on a COO tensor, without compression.
//
// The reference always compresses a sparse tensor first (its MLSVD of the
// dense T_(l) T_(l)^T, Compression.py:123-137) and runs dGN on the dense core.
// This path runs the same dGN iteration (GaussNewton.py:29-251, 315-398) on
// the factors of the full COO tensor, with the reference's objective: absent
// entries are zeros of the data (TensorFox.py:476-481), so
//   ||T - [[W]]||^2 = ||T||^2 - 2 <W_0, T_(0) KR_0> + sum_{a,b} prod_l G_l[a,b]
// and the gradient is W_l P1_l - T_(l) KR_l with T_(l) KR_l the COO MTTKRP.
// Only the MTTKRPs touch the entries; J^T J v needs the factors' Gramians only.
//
//   tfx_coo_dgn_cg        Gramians, regularisation, preconditioner, gradient,
//                         J^T J grad and the preconditioned CG of one dGN
//                         iteration, as ONE cooperative launch (the CTAs meet
//                         at bounded grid barriers of this file)
//   tfx_coo_model_error   ||T - [[W]]||^2 from the mode-0 MTTKRP and Gramians
//   tfx_factors_to_rows   flat (column-major per mode) factors -> row-major
//                         copies for the COO gathers
//   tfx_dogleg_dots       the dot products of one dogleg trial decision
//   tfx_dogleg_trial      y <- a y + b grad, x <- x_old + y, the factors, and
//                         the step's gain-ratio sums
//
// Flat layout: block l holds W_l column-major (column r contiguous), offset
// R * sum_{m<l} d_m, as everywhere in this library.  Rows of all modes are
// split into contiguous ranges, one per CTA; every vector entry is read and
// written only by the CTA owning its row, so only Gramians, the R x R
// products A_k and the scalars cross CTAs.
#include <math.h>

#include <algorithm>

#include "tfx_capi_internal.h"
#include "tfx_common.cuh"

namespace tfx {

struct CooDgnShape {
  int L, R, nb;              // order, rank, CTAs of the launch
  int dims[TFX_MAX_ORDER];
  int rowoff[TFX_MAX_ORDER + 1];   // sum_{m<l} d_m
  long long off[TFX_MAX_ORDER + 1];  // R * rowoff[l]
  long long nx;              // R * sum(dims)
};

// ---------------------------------------------------------------------------
// Bounded grid barrier (sense by generation).  Thread 0 of each CTA arrives
// on a global counter; the last arriver resets it and advances the
// generation; the others poll the generation with a limit.  A barrier that
// runs out sets *err, and every later barrier returns at once, so the launch
// always ends (with an error status the host reads).
// ---------------------------------------------------------------------------
#define COO_BAR_LIMIT (1u << 22)

__device__ __forceinline__ unsigned ld_acquire(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ void grid_barrier(unsigned* bar, int nb, int* err) {
  __syncthreads();
  if (threadIdx.x == 0) {
    if (*(volatile int*)err == 0) {
      unsigned* count = bar;
      unsigned* gen = bar + 1;
      const unsigned g = ld_acquire(gen);
      __threadfence();
      if (atomicAdd(count, 1u) == (unsigned)nb - 1) {
        atomicExch(count, 0u);
        __threadfence();
        atomicAdd(gen, 1u);
      } else {
        unsigned it = 0;
        while (ld_acquire(gen) == g) {
          if (++it > COO_BAR_LIMIT) {
            atomicExch(err, 3);
            break;
          }
          __nanosleep(100);
        }
      }
      __threadfence();
    }
  }
  __syncthreads();
}

// Sum over the CTAs of NV per-CTA values (double), the same fixed order in
// every CTA; `part` holds nb x NV slots per buffer, two buffers alternate.
template <int NV>
__device__ __forceinline__ void grid_sum(double (&v)[NV], double* part, int& flip, unsigned* bar, int nb, int* err,
                                         double* sred) {
  // v: this CTA's totals (valid in thread 0)
  if (threadIdx.x == 0)
#pragma unroll
    for (int j = 0; j < NV; ++j) part[(size_t)flip * nb * NV + (size_t)blockIdx.x * NV + j] = v[j];
  grid_barrier(bar, nb, err);
  if (threadIdx.x < NV) {
    double s = 0.0;
    const double* p = part + (size_t)flip * nb * NV + threadIdx.x;
    for (int q = 0; q < nb; ++q) s += __ldcg(p + (size_t)q * NV);
    sred[threadIdx.x] = s;
  }
  __syncthreads();
#pragma unroll
  for (int j = 0; j < NV; ++j) v[j] = sred[j];
  flip ^= 1;
  __syncthreads();
}

// CTA-wide sum of one accumulator per thread into thread 0 (double)
template <class T>
__device__ __forceinline__ double cta_sum(Acc<T> a, double* swarp) {
  a.warp_reduce();
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) swarp[wid] = a.value();
  __syncthreads();
  double s = 0.0;
  if (threadIdx.x == 0)
    for (int w = 0; w < TFX_THREADS / 32; ++w) s += swarp[w];
  __syncthreads();
  return s;
}

// Workspace of tfx_coo_dgn_cg (bytes from the 256-aligned base)
struct CooCgWs {
  size_t bar, err, G, part, partA, A, r, P, Q, z, y, g, total;
};

__host__ __device__ inline size_t al256c(size_t v) { return (v + 255) & ~(size_t)255; }

__host__ __device__ inline CooCgWs coo_cg_ws(int L, int R, long long nx, int nb, size_t es) {
  CooCgWs w;
  size_t o = 0;
  const size_t LRR = (size_t)L * R * R;
  w.bar = o; o += 256;
  w.err = o; o += 256;
  w.G = o; o += al256c(LRR * 8);
  w.part = o; o += al256c((size_t)2 * nb * 4 * 8);
  w.partA = o; o += al256c((size_t)nb * LRR * 8);
  w.A = o; o += al256c(LRR * 8);
  w.r = o; o += al256c((size_t)nx * es);
  w.P = o; o += al256c((size_t)nx * es);
  w.Q = o; o += al256c((size_t)nx * es);
  w.z = o; o += al256c((size_t)nx * es);
  w.y = o; o += al256c((size_t)nx * es);
  w.g = o; o += al256c((size_t)nx * es);
  w.total = o;
  return w;
}

// shared memory of the CG kernel (elements of T unless noted)
__host__ __device__ inline size_t coo_cg_smem(int L, int R, size_t es) {
  const size_t LRR = (size_t)L * R * R;
  return LRR * es /*P1*/ + (size_t)L * LRR * es /*P2*/ + 2 * LRR * es /*A, Y*/ + 2 * (size_t)L * R * es /*M, DG*/ +
         64 * 8 /*scalars*/ + 64;
}

template <class T>
struct CooCgArgs {
  const T* W;        // flat factors
  const T* Mrm;      // L MTTKRPs at W, row-major (d_l x R) blocks at off[l]
  double damp;
  int budget;
  double cg_tol;
  double* y_out;     // M y (flat, double)
  double* grad_out;  // -g = T_(l) KR_l - W_l P1_l (flat, double)
  double* jtj_out;   // J^T J grad (flat, double)
  double* out;       // [0] CG products + 1, [1] final residual norm^2, [2] status
  char* ws;
};

template <class T>
__global__ void __launch_bounds__(TFX_THREADS, 1) k_coo_dgn_cg(CooDgnShape sh, CooCgArgs<T> a) {
  extern __shared__ __align__(16) char smraw[];
  const int L = sh.L, R = sh.R, nb = sh.nb, tid = threadIdx.x;
  const int RR = R * R, LRR = L * RR;
  const long long nx = sh.nx;
  const CooCgWs w = coo_cg_ws(L, R, nx, nb, sizeof(T));
  unsigned* bar = (unsigned*)(a.ws + w.bar);
  int* err = (int*)(a.ws + w.err);
  double* G = (double*)(a.ws + w.G);
  double* part = (double*)(a.ws + w.part);
  double* partA = (double*)(a.ws + w.partA);
  double* Ag = (double*)(a.ws + w.A);
  T* r = (T*)(a.ws + w.r);
  T* P = (T*)(a.ws + w.P);
  T* Q = (T*)(a.ws + w.Q);
  T* z = (T*)(a.ws + w.z);
  T* yv = (T*)(a.ws + w.y);
  T* gv = (T*)(a.ws + w.g);
  T* sP1 = (T*)smraw;
  T* sP2 = sP1 + LRR;
  T* sA = sP2 + (size_t)L * LRR;
  T* sY = sA + LRR;
  T* sM = sY + LRR;
  T* sDG = sM + L * R;
  double* sred = (double*)(sDG + L * R);  // 64 doubles
  sred = (double*)(((uintptr_t)sred + 15) & ~(uintptr_t)15);
  int flip = 0;
  // this CTA's rows of the concatenated row space
  const int SR = sh.rowoff[L];
  const int r0 = (int)((long long)SR * blockIdx.x / nb), r1 = (int)((long long)SR * (blockIdx.x + 1) / nb);
  auto mode_of = [&](int row) {
    int l = 0;
    while (row >= sh.rowoff[l + 1]) ++l;
    return l;
  };
  // loop over the CTA's own vector entries: (flat index, mode, column)
  auto for_rows = [&](auto f) {
    for (int rr = r0 + tid; rr < r1; rr += TFX_THREADS) {
      const int l = mode_of(rr), i = rr - sh.rowoff[l], dl = sh.dims[l];
      f(rr, l, i, dl);
    }
  };
  // ---- R x R products over the CTA's rows, summed over the grid ------------
  // out[k][p][q] = sum_i X_k[i, p] Y_k[i, q] for all modes (p, q < R)
  auto grid_rr = [&](const T* X, const T* Y, double* out, bool sym) {
    for (int e = tid; e < LRR; e += TFX_THREADS) {
      const int k = e / RR, pq = e - k * RR, p = pq / R, q = pq - p * R;
      double v = 0.0;
      if (!sym || p <= q) {
        const int lo = max(r0, sh.rowoff[k]), hi = min(r1, sh.rowoff[k + 1]);
        const int dk = sh.dims[k];
        const T* xp = X + sh.off[k] + (long long)p * dk - sh.rowoff[k];
        const T* yp = Y + sh.off[k] + (long long)q * dk - sh.rowoff[k];
        Acc<T> acc;
        for (int rr = lo; rr < hi; ++rr) acc.fma_(xp[rr], yp[rr]);
        v = acc.value();
      }
      partA[(size_t)blockIdx.x * LRR + e] = v;
    }
    grid_barrier(bar, nb, err);
    for (int e = blockIdx.x * TFX_THREADS + tid; e < LRR; e += nb * TFX_THREADS) {
      const int k = e / RR, pq = e - k * RR, p = pq / R, q = pq - p * R;
      const int src = (sym && p > q) ? k * RR + q * R + p : e;
      double s = 0.0;
      for (int c = 0; c < nb; ++c) s += __ldcg(partA + (size_t)c * LRR + src);
      out[e] = s;
    }
    grid_barrier(bar, nb, err);
  };
  // ---- J^T J v on the own rows (GaussNewton.py:551-581) --------------------
  auto matvec = [&](const T* v, T* zout) {
    grid_rr(v, a.W, Ag, false);  // A_k = V_k^T W_k
    for (int e = tid; e < LRR; e += TFX_THREADS) sA[e] = (T)__ldcg(Ag + e);
    __syncthreads();
    for (int e = tid; e < LRR; e += TFX_THREADS) {
      const int l = e / RR, pq = e - l * RR;
      T s = T(0);
      for (int k = 0; k < L; ++k)
        if (k != l) s += sP2[((size_t)(l * L + k)) * RR + pq] * sA[k * RR + pq];
      sY[e] = s;
    }
    __syncthreads();
    // z_l = V_l P1_l + W_l Y_l
    for_rows([&](int rr, int l, int i, int dl) {
      const long long base = sh.off[l] + i;
      const T* P1l = sP1 + l * RR;
      const T* Yl = sY + l * RR;
      for (int c = 0; c < R; ++c) {
        T s = T(0);
        for (int p = 0; p < R; ++p) {
          s = fma(v[base + (long long)p * dl], P1l[p * R + c], s);
          s = fma(a.W[base + (long long)p * dl], Yl[p * R + c], s);
        }
        zout[base + (long long)c * dl] = s;
      }
    });
  };

  // ---- Gramians (FP64 sums of float-float partials), P1, P2 ----------------
  grid_rr(a.W, a.W, G, true);
  for (int e = tid; e < LRR; e += TFX_THREADS) {
    const int l = e / RR, pq = e - l * RR;
    // P1 with the reference's product order (GaussNewton.py:520-548)
    const int k = (l == 0) ? 1 : (l < L - 1 ? l - 1 : 0);
    double p2 = 1.0;
    for (int m = 0; m < L; ++m)
      if (m != l && m != k) p2 *= __ldcg(G + m * RR + pq);
    sP1[e] = (T)(p2 * __ldcg(G + k * RR + pq));
    for (int kk = 0; kk < L; ++kk) {
      double q2 = 1.0;
      for (int m = 0; m < L; ++m)
        if (m != l && m != kk) q2 *= __ldcg(G + m * RR + pq);
      sP2[((size_t)(l * L + kk)) * RR + pq] = (T)q2;
    }
  }
  // regularisation (GaussNewton.py:584-607): gamma[l, c] = max|P1[L-1]| sqrt|P1[l][c, c]|
  {
    double mx = 0.0;
    for (int pq = tid; pq < RR; pq += TFX_THREADS) {
      double p1 = 1.0;
      // P1[L-1] = P2[L-1][0] o G_0
      for (int m = 0; m < L; ++m)
        if (m != L - 1 && m != 0) p1 *= __ldcg(G + m * RR + pq);
      p1 *= __ldcg(G + pq);
      mx = fmax(mx, fabs(p1));
    }
    mx = warp_max(mx);
    if ((tid & 31) == 0) sred[32 + (tid >> 5)] = mx;
    __syncthreads();
    if (tid == 0) {
      double m2 = sred[32];
      for (int ww = 1; ww < TFX_THREADS / 32; ++ww) m2 = fmax(m2, sred[32 + ww]);
      sred[40] = m2;
    }
    __syncthreads();
    const double tmp = sred[40];
    for (int e = tid; e < L * R; e += TFX_THREADS) {
      const int l = e / R, c = e - l * R;
      const int k = (l == 0) ? 1 : (l < L - 1 ? l - 1 : 0);
      double p1 = __ldcg(G + k * RR + c * R + c);
      for (int m = 0; m < L; ++m)
        if (m != l && m != k) p1 *= __ldcg(G + m * RR + c * R + c);
      const double gma = tmp * sqrt(fabs(p1));
      sM[e] = (T)(1.0 / sqrt(gma * gma + a.damp * a.damp * (gma * gma)));
      sDG[e] = (T)(a.damp * gma);
    }
    __syncthreads();
  }
  // ---- gradient: -g_l = T_(l) KR_l - W_l P1_l ------------------------------
  for_rows([&](int rr, int l, int i, int dl) {
    const long long base = sh.off[l] + i;
    const T* mrow = a.Mrm + sh.off[l] + (long long)i * R;
    for (int c = 0; c < R; ++c) {
      T wp = T(0);
      for (int p = 0; p < R; ++p) wp = fma(a.W[base + (long long)p * dl], sP1[l * RR + p * R + c], wp);
      const T gv_ = mrow[c] - wp;
      gv[base + (long long)c * dl] = gv_;
      a.grad_out[base + (long long)c * dl] = (double)gv_;
    }
  });
  __syncthreads();
  // J^T J grad (kept for the dogleg)
  matvec(gv, z);
  Acc<T> rn_acc;
  for_rows([&](int rr, int l, int i, int dl) {
    const long long base = sh.off[l] + i;
    for (int c = 0; c < R; ++c) {
      const long long e = base + (long long)c * dl;
      a.jtj_out[e] = (double)z[e];
      const T rv = sM[l * R + c] * gv[e];
      r[e] = rv;
      P[e] = rv;
      yv[e] = T(0);
      rn_acc.fma_(rv, rv);
    }
  });
  double s1[1] = {cta_sum(rn_acc, sred)};
  grid_sum<1>(s1, part, flip, bar, nb, err, sred);
  double rn = s1[0];
  if (rn == 0.0) rn = 1e-6;
  int maxit = a.budget;
  double tol = a.cg_tol;
  if (nx > 100)
    maxit = (int)min((long long)maxit, nx);
  else
    tol = 0.0;
  int itn = 0;
  for (itn = 0; itn < maxit; ++itn) {
    for_rows([&](int rr, int l, int i, int dl) {
      const long long base = sh.off[l] + i;
      for (int c = 0; c < R; ++c) Q[base + (long long)c * dl] = sM[l * R + c] * P[base + (long long)c * dl];
    });
    __syncthreads();
    matvec(Q, z);
    // z = M (z + damp Gamma Q); denominator P.z
    Acc<T> den_acc;
    for_rows([&](int rr, int l, int i, int dl) {
      const long long base = sh.off[l] + i;
      for (int c = 0; c < R; ++c) {
        const long long e = base + (long long)c * dl;
        const T zz = sM[l * R + c] * (z[e] + sDG[l * R + c] * Q[e]);
        z[e] = zz;
        den_acc.fma_(P[e], zz);
      }
    });
    double s2[1] = {cta_sum(den_acc, sred)};
    grid_sum<1>(s2, part, flip, bar, nb, err, sred);
    double den = s2[0];
    if (den == 0.0) den = 1e-6;
    const T alpha = (T)(rn / den);
    // y += alpha P; r -= alpha z; on the first iteration P is the residual
    // array itself (the reference's P = residual_cg aliasing), so it moves too
    Acc<T> rn2_acc;
    const bool alias = itn == 0;
    for_rows([&](int rr, int l, int i, int dl) {
      const long long base = sh.off[l] + i;
      for (int c = 0; c < R; ++c) {
        const long long e = base + (long long)c * dl;
        yv[e] += alpha * P[e];
        const T rv = r[e] - alpha * z[e];
        r[e] = rv;
        if (alias) P[e] = rv;
        rn2_acc.fma_(rv, rv);
      }
    });
    double s3[1] = {cta_sum(rn2_acc, sred)};
    grid_sum<1>(s3, part, flip, bar, nb, err, sred);
    const double rn_new = s3[0];
    const T beta = (T)(rn_new / rn);
    rn = rn_new;
    for_rows([&](int rr, int l, int i, int dl) {
      const long long base = sh.off[l] + i;
      for (int c = 0; c < R; ++c) {
        const long long e = base + (long long)c * dl;
        P[e] = r[e] + beta * P[e];
      }
    });
    __syncthreads();
    if (rn <= tol) break;
  }
  for_rows([&](int rr, int l, int i, int dl) {
    const long long base = sh.off[l] + i;
    for (int c = 0; c < R; ++c) {
      const long long e = base + (long long)c * dl;
      a.y_out[e] = (double)(sM[l * R + c] * yv[e]);
    }
  });
  if (blockIdx.x == 0 && tid == 0) {
    a.out[0] = (double)(min(itn, maxit - 1) + 1 + 1);  // CG products, J^T J grad included
    a.out[1] = rn;
  }
}

// ---------------------------------------------------------------------------
// ||T - [[W]]||^2 = ||T||^2 - 2 <W_0, M_0> + sum_{a,b} prod_l G_l[a,b]
// ---------------------------------------------------------------------------
template <class T>
__global__ void __launch_bounds__(TFX_THREADS) k_coo_err_partials(CooDgnShape sh, const T* __restrict__ W,
                                                                   const T* __restrict__ M0rm,
                                                                   double* __restrict__ part) {
  __shared__ double swarp[TFX_THREADS / 32];
  const int L = sh.L, R = sh.R, RR = R * R, LRR = L * RR, nb = gridDim.x, tid = threadIdx.x;
  const int SR = sh.rowoff[L];
  const int r0 = (int)((long long)SR * blockIdx.x / nb), r1 = (int)((long long)SR * (blockIdx.x + 1) / nb);
  for (int e = tid; e < LRR; e += TFX_THREADS) {
    const int k = e / RR, pq = e - k * RR, p = pq / R, q = pq - p * R;
    const int lo = max(r0, sh.rowoff[k]), hi = min(r1, sh.rowoff[k + 1]);
    const int dk = sh.dims[k];
    const T* xp = W + sh.off[k] + (long long)p * dk - sh.rowoff[k];
    const T* yp = W + sh.off[k] + (long long)q * dk - sh.rowoff[k];
    Acc<T> acc;
    for (int rr = lo; rr < hi; ++rr) acc.fma_(xp[rr], yp[rr]);
    part[(size_t)blockIdx.x * (LRR + 1) + e] = acc.value();
  }
  // <W_0, M_0> over the CTA's rows of mode 0
  Acc<T> ip;
  const int d0 = sh.dims[0];
  for (int rr = r0 + tid; rr < min(r1, d0); rr += TFX_THREADS)
    for (int c = 0; c < R; ++c) ip.fma_(W[(long long)c * d0 + rr], M0rm[(long long)rr * R + c]);
  ip.warp_reduce();
  if ((tid & 31) == 0) swarp[tid >> 5] = ip.value();
  __syncthreads();
  if (tid == 0) {
    double s = 0.0;
    for (int wq = 0; wq < TFX_THREADS / 32; ++wq) s += swarp[wq];
    part[(size_t)blockIdx.x * (LRR + 1) + LRR] = s;
  }
}

// the CTAs' partials summed per entry: one warp per (Gram entry | <W_0, M_0>),
// lanes stride the CTAs, so the order is fixed
__global__ void __launch_bounds__(256) k_coo_err_gsum(int nb, int ne, const double* __restrict__ part,
                                                      double* __restrict__ G) {
  const int lane = threadIdx.x & 31;
  const int e = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (e >= ne) return;
  double s = 0.0;
  for (int c = lane; c < nb; c += 32) s += part[(size_t)c * ne + e];
  s = warp_sum(s);
  if (lane == 0) G[e] = s;
}

__global__ void __launch_bounds__(TFX_THREADS) k_coo_err_final(CooDgnShape sh, const double* __restrict__ G,
                                                                double tnorm2, double* __restrict__ out) {
  __shared__ double swarp[TFX_THREADS / 32];
  const int L = sh.L, R = sh.R, RR = R * R, LRR = L * RR, tid = threadIdx.x;
  double model2 = 0.0;
  for (int pq = tid; pq < RR; pq += TFX_THREADS) {
    double prod = 1.0;
    for (int l = 0; l < L; ++l) prod *= G[l * RR + pq];
    model2 += prod;
  }
  model2 = warp_sum(model2);
  if ((tid & 31) == 0) swarp[tid >> 5] = model2;
  __syncthreads();
  if (tid == 0) {
    double m2 = 0.0;
    for (int w = 0; w < TFX_THREADS / 32; ++w) m2 += swarp[w];
    const double ip = G[LRR];
    out[0] = tnorm2 - 2.0 * ip + m2;
    out[1] = ip;
    out[2] = m2;
  }
}

// flat (column-major per mode) -> row-major (d_l x R) copies, same offsets
template <class T>
__global__ void k_flat_to_rows(CooDgnShape sh, const T* __restrict__ W, T* __restrict__ Wrm) {
  const long long nx = sh.nx;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < nx; e += (long long)gridDim.x * blockDim.x) {
    int l = 0;
    while (e >= sh.off[l + 1]) ++l;
    const long long loc = e - sh.off[l];
    const int dl = sh.dims[l];
    const long long i = loc / sh.R, c = loc - i * sh.R;
    Wrm[e] = W[sh.off[l] + c * dl + i];
  }
}

// dogleg: out = {a.b, c.d, e.f} over n entries (double inputs), per-block partials
__global__ void __launch_bounds__(TFX_THREADS) k_dots3(long long n, const double* a, const double* b, const double* c,
                                                        const double* d, const double* e, const double* f,
                                                        double* part) {
  __shared__ double sw[3][TFX_THREADS / 32];
  double s[3] = {0.0, 0.0, 0.0};
  for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
    s[0] = fma(a[k], b[k], s[0]);
    s[1] = fma(c[k], d[k], s[1]);
    s[2] = fma(e[k], f[k], s[2]);
  }
  for (int j = 0; j < 3; ++j) {
    const double v = warp_sum(s[j]);
    if ((threadIdx.x & 31) == 0) sw[j][threadIdx.x >> 5] = v;
  }
  __syncthreads();
  if (threadIdx.x < 3) {
    double t = 0.0;
    for (int w = 0; w < TFX_THREADS / 32; ++w) t += sw[threadIdx.x][w];
    part[(size_t)blockIdx.x * 3 + threadIdx.x] = t;
  }
}

__global__ void k_sum_parts(const double* part, int nb, int nv, double* out) {
  if (threadIdx.x < nv) {
    double s = 0.0;
    for (int c = 0; c < nb; ++c) s += part[(size_t)c * nv + threadIdx.x];
    out[threadIdx.x] = s;
  }
}

// dogleg trial: y <- ca y + cb grad; x <- x_old + y; W <- x (no balancing);
// partials of (x - x_old).(grad + damp (x - x_old)) and |x - x_old|^2
template <class T>
__global__ void __launch_bounds__(TFX_THREADS) k_dogleg_trial(long long n, const T* __restrict__ x_old,
                                                               double* __restrict__ y, const double* __restrict__ grad,
                                                               double ca, double cb, double damp, T* __restrict__ x,
                                                               T* __restrict__ W, double* __restrict__ part) {
  __shared__ double sw[2][TFX_THREADS / 32];
  double s[2] = {0.0, 0.0};
  for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
    const T yn = (T)(ca * y[k] + cb * grad[k]);
    y[k] = (double)yn;
    const T xo = x_old[k];
    const T xv = xo + yn;
    x[k] = xv;
    W[k] = xv;
    const double dx = (double)xv - (double)xo;
    s[0] += dx * (grad[k] + damp * dx);
    s[1] += dx * dx;
  }
  for (int j = 0; j < 2; ++j) {
    const double v = warp_sum(s[j]);
    if ((threadIdx.x & 31) == 0) sw[j][threadIdx.x >> 5] = v;
  }
  __syncthreads();
  if (threadIdx.x < 2) {
    double t = 0.0;
    for (int w = 0; w < TFX_THREADS / 32; ++w) t += sw[threadIdx.x][w];
    part[(size_t)blockIdx.x * 2 + threadIdx.x] = t;
  }
}

// the scalars of an accepted step (GaussNewton.py:472-487, 199-211):
// partials of (x - x_old).(grad + damp (x - x_old)), |x - x_old|^2, |x_old|^2, max|grad|
template <class T>
__global__ void __launch_bounds__(TFX_THREADS) k_step_sums(long long n, const T* __restrict__ x,
                                                            const T* __restrict__ x_old,
                                                            const double* __restrict__ grad, double damp,
                                                            double* __restrict__ part) {
  __shared__ double sw[4][TFX_THREADS / 32];
  double s[4] = {0.0, 0.0, 0.0, 0.0};
  for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
    const double dx = (double)x[k] - (double)x_old[k];
    s[0] += dx * (grad[k] + damp * dx);
    s[1] += dx * dx;
    s[2] += (double)x_old[k] * (double)x_old[k];
    s[3] = fmax(s[3], fabs(grad[k]));
  }
  for (int j = 0; j < 4; ++j) {
    const double v = j == 3 ? warp_max(s[j]) : warp_sum(s[j]);
    if ((threadIdx.x & 31) == 0) sw[j][threadIdx.x >> 5] = v;
  }
  __syncthreads();
  if (threadIdx.x < 4) {
    double t = 0.0;
    for (int w = 0; w < TFX_THREADS / 32; ++w)
      t = threadIdx.x == 3 ? fmax(t, sw[3][w]) : t + sw[threadIdx.x][w];
    part[(size_t)blockIdx.x * 4 + threadIdx.x] = t;
  }
}

__global__ void k_sum_parts4(const double* part, int nb, double* out) {
  if (threadIdx.x < 4) {
    double s = 0.0;
    for (int c = 0; c < nb; ++c) {
      const double v = part[(size_t)c * 4 + threadIdx.x];
      s = threadIdx.x == 3 ? fmax(s, v) : s + v;
    }
    out[threadIdx.x] = s;
  }
}

// x_out = x - y (the reference's revert of a rejected step, in floating point)
template <class T>
__global__ void k_revert(long long n, const T* __restrict__ x, const double* __restrict__ y, T* __restrict__ x_out) {
  for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x)
    x_out[k] = x[k] - (T)y[k];
}

// ---------------------------------------------------------------------------
// The step update of GaussNewton.py:284-297 for large factor vectors (no
// symmetric transform, no fixed norm, no fixed factor): x += y, the step's
// scalars, column balancing (Conversion.py:361-387) -- over the whole grid.
// Work item = (column, segment of up to STEP_SEG rows), one warp each; the
// column sums are kept per item, the step's scalars per CTA, and both are
// summed in a fixed order, so the result does not vary between runs.
// ---------------------------------------------------------------------------
#define STEP_SEG 256
#define STEP_THREADS 256

struct StepShape {
  int L, R, nseg_total;
  int dims[TFX_MAX_ORDER];
  long long off[TFX_MAX_ORDER + 1];
  int segs[TFX_MAX_ORDER];        // segments per column of mode l
  int item0[TFX_MAX_ORDER + 1];   // first item of mode l
};

// colp[item] = column norm^2 of x_new over the item's rows; blk[4 b ..] =
// the CTA's {|x_old|^2, |dx|^2, dx.(g + damp dx), max|g| (NaN if any g is)}
template <class T>
__global__ void __launch_bounds__(STEP_THREADS) k_step_wide1(StepShape sh, T* __restrict__ x,
                                                             const double* __restrict__ y,
                                                             const double* __restrict__ grad, double damp,
                                                             double* __restrict__ colp, double* __restrict__ blk) {
  __shared__ double sw[STEP_THREADS / 32][4];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int warps = (gridDim.x * blockDim.x) >> 5;
  double s0 = 0.0, s1 = 0.0, s2 = 0.0, gi = 0.0;
  bool gnan = false;
  for (int item = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; item < sh.nseg_total; item += warps) {
    int l = 0;
    while (item >= sh.item0[l + 1]) ++l;
    const int loc = item - sh.item0[l];
    const int r = loc / sh.segs[l], sg = loc - r * sh.segs[l];
    const int d = sh.dims[l];
    const long long base = sh.off[l] + (long long)r * d;
    const int i0 = sg * STEP_SEG, i1 = min(d, i0 + STEP_SEG);
    double cn = 0.0;
#pragma unroll 4
    for (int i = i0 + lane; i < i1; i += 32) {
      const long long e = base + i;
      const double xo = (double)x[e];
      const T xn = (T)(xo + y[e]);
      const double dv = (double)xn - xo;
      const double g = grad[e];
      s0 = fma(xo, xo, s0);
      s1 = fma(dv, dv, s1);
      s2 = fma(dv, g + damp * dv, s2);
      if (g != g) gnan = true;
      gi = fmax(gi, fabs(g));
      cn = fma((double)xn, (double)xn, cn);
      x[e] = xn;
    }
    cn = warp_sum(cn);
    if (lane == 0) colp[item] = cn;
  }
  s0 = warp_sum(s0);
  s1 = warp_sum(s1);
  s2 = warp_sum(s2);
  gi = warp_max(gi);
  const int anynan = __any_sync(0xffffffffu, gnan);
  if (lane == 0) {
    sw[wid][0] = s0;
    sw[wid][1] = s1;
    sw[wid][2] = s2;
    sw[wid][3] = anynan ? NAN : gi;
  }
  __syncthreads();
  if (threadIdx.x < 4) {
    const int k = threadIdx.x;
    double v = 0.0;
    bool vn = false;
    for (int w = 0; w < STEP_THREADS / 32; ++w) {
      const double q = sw[w][k];
      if (k < 3) {
        v += q;
      } else {
        if (q != q) vn = true;
        v = fmax(v, q);
      }
    }
    blk[(size_t)blockIdx.x * 4 + k] = (k == 3 && vn) ? NAN : v;
  }
}

// column balancing factors (the reference's equalize: (prod_l n_l)^(1/L) / n_l,
// 1 when a column vanishes) and the step's scalars out4 = {|dx|^2, |x_old|^2,
// dx.(g + damp dx), max|g|}
__global__ void __launch_bounds__(STEP_THREADS) k_step_wide2(StepShape sh, int nblk, const double* __restrict__ colp,
                                                             const double* __restrict__ blk,
                                                             double* __restrict__ fac, double* __restrict__ out) {
  __shared__ double nrm[TFX_MAX_ORDER * 64];
  __shared__ double sw[STEP_THREADS / 32][4];
  const int L = sh.L, R = sh.R, tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  for (int c = wid; c < L * R; c += STEP_THREADS / 32) {
    const int l = c / R, r = c - l * R;
    const int it0 = sh.item0[l] + r * sh.segs[l];
    double v = 0.0;
    for (int q = lane; q < sh.segs[l]; q += 32) v += colp[it0 + q];
    v = warp_sum(v);
    if (lane == 0) nrm[c] = sqrt(v);
  }
  double a = 0.0, b = 0.0, c = 0.0, m = 0.0;
  bool mn = false;
  for (int q = tid; q < nblk; q += STEP_THREADS) {
    const double* o = blk + (size_t)q * 4;
    a += o[0];
    b += o[1];
    c += o[2];
    if (o[3] != o[3]) mn = true;
    m = fmax(m, o[3]);
  }
  a = warp_sum(a);
  b = warp_sum(b);
  c = warp_sum(c);
  m = warp_max(m);
  const int anynan = __any_sync(0xffffffffu, mn);
  if (lane == 0) {
    sw[wid][0] = a;
    sw[wid][1] = b;
    sw[wid][2] = c;
    sw[wid][3] = anynan ? NAN : m;
  }
  __syncthreads();
  for (int r = tid; r < R; r += STEP_THREADS) {
    double prod = 1.0;
    for (int l = 0; l < L; ++l) prod *= nrm[l * R + r];
    if (prod != 0.0) {
      const double num = pow(prod, 1.0 / (double)L);
      for (int l = 0; l < L; ++l) fac[l * R + r] = num / nrm[l * R + r];
    } else {
      for (int l = 0; l < L; ++l) fac[l * R + r] = 1.0;
    }
  }
  if (tid == 0) {
    double t0 = 0.0, t1 = 0.0, t2 = 0.0, t3 = 0.0;
    bool tn = false;
    for (int w = 0; w < STEP_THREADS / 32; ++w) {
      t0 += sw[w][0];
      t1 += sw[w][1];
      t2 += sw[w][2];
      if (sw[w][3] != sw[w][3]) tn = true;
      t3 = fmax(t3, sw[w][3]);
    }
    out[0] = t1;
    out[1] = t0;
    out[2] = t2;
    out[3] = tn ? NAN : t3;
  }
}

template <class T>
__global__ void k_step_wide3(StepShape sh, const T* __restrict__ x, const double* __restrict__ fac,
                             T* __restrict__ W) {
  const long long n = sh.off[sh.L];
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
    int l = 0;
    while (e >= sh.off[l + 1]) ++l;
    const int r = (int)((e - sh.off[l]) / sh.dims[l]);
    W[e] = (T)(fac[l * sh.R + r] * (double)x[e]);
  }
}

static int launched(const char* where) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return tfx_set_cuda_error(e, where);
  tfx_count_launch(1);
  return TFX_STATUS_OK;
}

static int sm_total() {
  int dev = 0, sms = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  return sms < 1 ? 1 : sms;
}

__global__ void k_copy_status(const int* err, double* out) {
  if (threadIdx.x == 0) *out = (double)*err;
}

static int fill_coo_shape(CooDgnShape& sh, int L, const int* dims, int R) {
  if (L < 2 || L > TFX_MAX_ORDER || R < 1 || !dims) return 1;
  sh.L = L;
  sh.R = R;
  sh.rowoff[0] = 0;
  sh.off[0] = 0;
  long long s = 0;
  for (int l = 0; l < L; ++l) {
    if (dims[l] < 1) return 1;
    sh.dims[l] = dims[l];
    s += dims[l];
    if (s > 0x7fffffffLL) return 1;
    sh.rowoff[l + 1] = (int)s;
    sh.off[l + 1] = (long long)R * s;
  }
  sh.nx = (long long)R * s;
  return 0;
}

// one CTA per SM (every CTA resident: the launch is cooperative)
static int coo_cg_blocks(const void* kfn, size_t smem) {
  int per = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kfn, TFX_THREADS, smem);
  return per >= 1 ? sm_total() : 0;
}

}  // namespace tfx

using namespace tfx;

extern "C" size_t tfx_coo_dgn_cg_workspace_bytes(int dtype, int L, const int* dims, int R) {
  CooDgnShape sh;
  if (fill_coo_shape(sh, L, dims, R)) return 0;
  return coo_cg_ws(L, R, sh.nx, sm_total(), dtype == TFX_F64 ? 8 : 4).total + 256;
}

extern "C" int tfx_coo_dgn_cg(int dtype, int L, const int* dims, int R, const void* W, const void* Mrm, double damp,
                              int budget, double cg_tol, double* y, double* grad, double* jtj, double* out,
                              void* work, size_t work_bytes, void* stream) {
  CooDgnShape sh;
  if (fill_coo_shape(sh, L, dims, R) || !W || !Mrm || !y || !grad || !jtj || !out || !work || budget < 0)
    return tfx_set_error(TFX_STATUS_ERR_ARG, "coo_dgn_cg args");
  if (((uintptr_t)work & 255) != 0) return tfx_set_error(TFX_STATUS_ERR_ARG, "coo_dgn_cg: work must be 256-byte aligned");
  const size_t es = dtype == TFX_F64 ? 8 : 4;
  const size_t smem = coo_cg_smem(L, R, es);
  if (smem > 200 * 1024)
    return tfx_set_error(TFX_STATUS_ERR_UNSUPPORTED,
                         "coo_dgn_cg: order and rank too large for the kernel's shared memory (L^2 R^2 terms)");
  const void* kfn = dtype == TFX_F64 ? (const void*)k_coo_dgn_cg<double> : (const void*)k_coo_dgn_cg<float>;
  cudaError_t e = cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return tfx_set_cuda_error(e, "coo_dgn_cg smem");
  const int nb = coo_cg_blocks(kfn, smem);
  if (nb < 1) return tfx_set_error(TFX_STATUS_ERR_UNSUPPORTED, "coo_dgn_cg: no resident CTA");
  sh.nb = nb;
  const CooCgWs w = coo_cg_ws(L, R, sh.nx, nb, es);
  if (work_bytes < w.total) return tfx_set_error(TFX_STATUS_ERR_ARG, "coo_dgn_cg: work too small");
  cudaStream_t st = (cudaStream_t)stream;
  e = cudaMemsetAsync(work, 0, 512, st);  // barrier counter, generation, error flag
  if (e != cudaSuccess) return tfx_set_cuda_error(e, "coo_dgn_cg memset");
  if (dtype == TFX_F64) {
    CooCgArgs<double> a = {(const double*)W, (const double*)Mrm, damp, budget, cg_tol, y, grad, jtj, out, (char*)work};
    void* args[] = {&sh, &a};
    e = cudaLaunchCooperativeKernel((const void*)k_coo_dgn_cg<double>, dim3(nb), dim3(TFX_THREADS), args, smem, st);
  } else {
    CooCgArgs<float> a = {(const float*)W, (const float*)Mrm, damp, budget, cg_tol, y, grad, jtj, out, (char*)work};
    void* args[] = {&sh, &a};
    e = cudaLaunchCooperativeKernel((const void*)k_coo_dgn_cg<float>, dim3(nb), dim3(TFX_THREADS), args, smem, st);
  }
  if (e != cudaSuccess) return tfx_set_cuda_error(e, "coo_dgn_cg launch");
  tfx_count_launch(1);
  // status: the barrier error flag (0, or 3 when a grid barrier ran out)
  k_copy_status<<<1, 32, 0, st>>>((const int*)((char*)work + w.err), out + 2);
  return launched("coo_dgn_cg status");
}

extern "C" size_t tfx_coo_model_error_scratch_bytes(int L, int R) {
  return ((size_t)sm_total() + 1) * ((size_t)L * R * R + 1) * 8 + 256;
}

extern "C" int tfx_coo_model_error(int dtype, int L, const int* dims, int R, const void* W, const void* M0rm,
                                   double tnorm2, double* out, void* scratch, size_t scratch_bytes, void* stream) {
  CooDgnShape sh;
  if (fill_coo_shape(sh, L, dims, R) || !W || !M0rm || !out || !scratch)
    return tfx_set_error(TFX_STATUS_ERR_ARG, "coo_model_error args");
  const int nb = std::max(1, std::min(sm_total(), (sh.rowoff[L] + TFX_THREADS - 1) / TFX_THREADS));
  const int ne = L * R * R + 1;
  const size_t need = ((size_t)nb + 1) * ne * 8;
  if (scratch_bytes < need) return tfx_set_error(TFX_STATUS_ERR_ARG, "coo_model_error scratch");
  sh.nb = nb;
  cudaStream_t st = (cudaStream_t)stream;
  if (dtype == TFX_F64)
    k_coo_err_partials<double><<<nb, TFX_THREADS, 0, st>>>(sh, (const double*)W, (const double*)M0rm, (double*)scratch);
  else
    k_coo_err_partials<float><<<nb, TFX_THREADS, 0, st>>>(sh, (const float*)W, (const float*)M0rm, (double*)scratch);
  if (int s = launched("coo_err_partials")) return s;
  double* G = (double*)scratch + (size_t)nb * ne;
  k_coo_err_gsum<<<(ne * 32 + 255) / 256, 256, 0, st>>>(nb, ne, (const double*)scratch, G);
  if (int s = launched("coo_err_gsum")) return s;
  k_coo_err_final<<<1, TFX_THREADS, 0, st>>>(sh, G, tnorm2, out);
  return launched("coo_err_final");
}

extern "C" int tfx_factors_to_rows(int dtype, int L, const int* dims, int R, const void* W, void* Wrm, void* stream) {
  CooDgnShape sh;
  if (fill_coo_shape(sh, L, dims, R) || !W || !Wrm) return tfx_set_error(TFX_STATUS_ERR_ARG, "factors_to_rows args");
  cudaStream_t st = (cudaStream_t)stream;
  const int blocks = (int)std::max<long long>(1, std::min<long long>((sh.nx + 255) / 256, 8LL * sm_total()));
  if (dtype == TFX_F64)
    k_flat_to_rows<double><<<blocks, 256, 0, st>>>(sh, (const double*)W, (double*)Wrm);
  else
    k_flat_to_rows<float><<<blocks, 256, 0, st>>>(sh, (const float*)W, (float*)Wrm);
  return launched("flat_to_rows");
}

extern "C" size_t tfx_dogleg_scratch_bytes(void) { return (size_t)1024 * 4 * 8 + 256; }

extern "C" int tfx_dogleg_dots(long long n, const double* a, const double* b, const double* c, const double* d,
                               const double* e, const double* f, double* out3, void* scratch, void* stream) {
  if (n < 0 || !a || !b || !c || !d || !e || !f || !out3 || !scratch)
    return tfx_set_error(TFX_STATUS_ERR_ARG, "dogleg_dots args");
  cudaStream_t st = (cudaStream_t)stream;
  const int blocks = (int)std::max<long long>(1, std::min<long long>((n + 255) / 256, 1024));
  k_dots3<<<blocks, TFX_THREADS, 0, st>>>(n, a, b, c, d, e, f, (double*)scratch);
  if (int s = launched("dots3")) return s;
  k_sum_parts<<<1, 32, 0, st>>>((const double*)scratch, blocks, 3, out3);
  return launched("sum_parts");
}

extern "C" int tfx_dogleg_trial(int dtype, long long n, const void* x_old, double* y, const double* grad, double ca,
                                double cb, double damp, void* x, void* W, double* out2, void* scratch, void* stream) {
  if (n < 0 || !x_old || !y || !grad || !x || !W || !out2 || !scratch)
    return tfx_set_error(TFX_STATUS_ERR_ARG, "dogleg_trial args");
  cudaStream_t st = (cudaStream_t)stream;
  const int blocks = (int)std::max<long long>(1, std::min<long long>((n + 255) / 256, 1024));
  if (dtype == TFX_F64)
    k_dogleg_trial<double><<<blocks, TFX_THREADS, 0, st>>>(n, (const double*)x_old, y, grad, ca, cb, damp, (double*)x,
                                                           (double*)W, (double*)scratch);
  else
    k_dogleg_trial<float><<<blocks, TFX_THREADS, 0, st>>>(n, (const float*)x_old, y, grad, ca, cb, damp, (float*)x,
                                                          (float*)W, (double*)scratch);
  if (int s = launched("dogleg_trial")) return s;
  k_sum_parts<<<1, 32, 0, st>>>((const double*)scratch, blocks, 2, out2);
  return launched("sum_parts");
}

extern "C" int tfx_step_sums(int dtype, long long n, const void* x, const void* x_old, const double* grad, double damp,
                             double* out4, void* scratch, void* stream) {
  if (n < 0 || !x || !x_old || !grad || !out4 || !scratch) return tfx_set_error(TFX_STATUS_ERR_ARG, "step_sums args");
  cudaStream_t st = (cudaStream_t)stream;
  const int blocks = (int)std::max<long long>(1, std::min<long long>((n + 255) / 256, 1024));
  if (dtype == TFX_F64)
    k_step_sums<double><<<blocks, TFX_THREADS, 0, st>>>(n, (const double*)x, (const double*)x_old, grad, damp,
                                                        (double*)scratch);
  else
    k_step_sums<float><<<blocks, TFX_THREADS, 0, st>>>(n, (const float*)x, (const float*)x_old, grad, damp,
                                                       (double*)scratch);
  if (int s = launched("step_sums")) return s;
  k_sum_parts4<<<1, 32, 0, st>>>((const double*)scratch, blocks, out4);
  return launched("sum_parts4");
}

extern "C" int tfx_step_revert(int dtype, long long n, const void* x, const double* y, void* x_out, void* stream) {
  if (n < 0 || !x || !y || !x_out) return tfx_set_error(TFX_STATUS_ERR_ARG, "step_revert args");
  cudaStream_t st = (cudaStream_t)stream;
  const int blocks = (int)std::max<long long>(1, std::min<long long>((n + 255) / 256, 1024));
  if (dtype == TFX_F64)
    k_revert<double><<<blocks, 256, 0, st>>>(n, (const double*)x, y, (double*)x_out);
  else
    k_revert<float><<<blocks, 256, 0, st>>>(n, (const float*)x, y, (float*)x_out);
  return launched("step_revert");
}

static int fill_step_shape(StepShape& sh, int L, const int* dims, int R) {
  if (L < 2 || L > TFX_MAX_ORDER || R < 1 || R > 64 || !dims) return 1;
  sh.L = L;
  sh.R = R;
  sh.off[0] = 0;
  sh.item0[0] = 0;
  for (int l = 0; l < L; ++l) {
    if (dims[l] < 1) return 1;
    sh.dims[l] = dims[l];
    sh.off[l + 1] = sh.off[l] + (long long)R * dims[l];
    sh.segs[l] = (dims[l] + STEP_SEG - 1) / STEP_SEG;
    sh.item0[l + 1] = sh.item0[l] + R * sh.segs[l];
  }
  sh.nseg_total = sh.item0[L];
  return 0;
}

static int step_blocks(const StepShape& sh) {
  return std::max(1, std::min((sh.nseg_total * 32 + STEP_THREADS - 1) / STEP_THREADS, 16 * sm_total()));
}

extern "C" size_t tfx_step_update_wide_scratch_bytes(int L, const int* dims, int R) {
  StepShape sh;
  if (fill_step_shape(sh, L, dims, R)) return 0;
  return ((size_t)sh.nseg_total + (size_t)step_blocks(sh) * 4 + (size_t)L * R) * 8 + 256;
}

extern "C" int tfx_step_update_wide(int dtype, int L, const int* dims, int R, void* x, void* W, const double* y,
                                    const double* grad, double damp, double* out4, void* scratch,
                                    size_t scratch_bytes, void* stream) {
  StepShape sh;
  if (fill_step_shape(sh, L, dims, R) || !x || !W || !y || !grad || !out4 || !scratch)
    return tfx_set_error(TFX_STATUS_ERR_ARG, "step_update_wide args (R <= 64)");
  if (scratch_bytes < tfx_step_update_wide_scratch_bytes(L, dims, R))
    return tfx_set_error(TFX_STATUS_ERR_ARG, "step_update_wide scratch");
  const int b1 = step_blocks(sh);
  double* colp = (double*)scratch;
  double* blk = colp + sh.nseg_total;
  double* fac = blk + (size_t)b1 * 4;
  cudaStream_t st = (cudaStream_t)stream;
  const long long n = sh.off[L];
  const int b3 = (int)std::max<long long>(1, std::min<long long>((n + 255) / 256, 8LL * sm_total()));
  if (dtype == TFX_F64)
    k_step_wide1<double><<<b1, STEP_THREADS, 0, st>>>(sh, (double*)x, y, grad, damp, colp, blk);
  else
    k_step_wide1<float><<<b1, STEP_THREADS, 0, st>>>(sh, (float*)x, y, grad, damp, colp, blk);
  if (int s = launched("step_wide1")) return s;
  k_step_wide2<<<1, STEP_THREADS, 0, st>>>(sh, b1, colp, blk, fac, out4);
  if (int s = launched("step_wide2")) return s;
  if (dtype == TFX_F64)
    k_step_wide3<double><<<b3, 256, 0, st>>>(sh, (const double*)x, fac, (double*)W);
  else
    k_step_wide3<float><<<b3, 256, 0, st>>>(sh, (const float*)x, fac, (float*)W);
  return launched("step_wide3");
}
