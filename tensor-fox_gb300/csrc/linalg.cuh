// CTA-level dense linear algebra shared by the single-problem and batched kernels.
#pragma once
#include "tfx_common.cuh"

namespace tfx {

// Symmetric eigensolver on one CTA: cyclic Jacobi with the round-robin
// (tournament) ordering, m/2 disjoint rotations per round applied in parallel.
// A (m x m, m even, row-major, symmetric, zero-padded beyond n) and Vs (m x m,
// column p at Vs[p*m]) live in shared memory; cs holds m values, pr m+2 ints,
// red 2*(TFX_THREADS/32) doubles.  On return the diagonal of A holds the
// eigenvalues and the columns of Vs the eigenvectors (unsorted).
template <class T>
__device__ int cta_jacobi(T* A, T* Vs, T* cs, int* pr, double* red, int m, int max_sweeps) {
  const int tid = threadIdx.x;
  const double eps = sizeof(T) == 8 ? 1e-14 : 2e-6;
  int sweep = 0;
  for (sweep = 0; sweep < max_sweeps; ++sweep) {
    double off = 0.0, tot = 0.0;
    for (int e = tid; e < m * m; e += blockDim.x) {
      const double v = (double)A[e];
      tot += v * v;
      if (e / m != e % m) off += v * v;
    }
    off = warp_sum(off);
    tot = warp_sum(tot);
    if ((tid & 31) == 0) {
      red[2 * (tid >> 5)] = off;
      red[2 * (tid >> 5) + 1] = tot;
    }
    __syncthreads();
    double so = 0.0, st = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
      so += red[2 * w];
      st += red[2 * w + 1];
    }
    __syncthreads();
    if (so <= eps * eps * st || st == 0.0) break;
    for (int round = 0; round < m - 1; ++round) {
      for (int kk = tid; kk < m / 2; kk += blockDim.x) {
        const int a = (kk == 0) ? m - 1 : (kk + round) % (m - 1);
        const int b = (m - 1 - kk + round) % (m - 1);
        const int p = a < b ? a : b, q = a < b ? b : a;
        pr[2 * kk] = p;
        pr[2 * kk + 1] = q;
        // rotation in the working precision (FP64 division and square root
        // are slow on GB300; the FP64 path keeps them in FP64)
        const T apq = A[p * m + q];
        T c = T(1), s = T(0);
        if (apq != T(0)) {
          const T tau = (A[q * m + q] - A[p * m + p]) / (T(2) * apq);
          const T at = fabs(tau);
          // for huge |tau| use t ~ 1/(2 tau) to avoid overflow of tau*tau
          const T t = (at > T(1e18)) ? T(1) / (T(2) * tau)
                                      : (tau >= T(0) ? T(1) : T(-1)) / (at + sqrt(T(1) + tau * tau));
          c = T(1) / sqrt(T(1) + t * t);
          s = t * c;
        }
        cs[kk] = c;
        cs[m / 2 + kk] = s;
      }
      __syncthreads();
      for (int e = tid; e < (m / 2) * m; e += blockDim.x) {
        const int kk = e / m, i = e - kk * m;
        const int p = pr[2 * kk], q = pr[2 * kk + 1];
        const T c = cs[kk], s = cs[m / 2 + kk];
        const T aip = A[i * m + p], aiq = A[i * m + q];
        A[i * m + p] = c * aip - s * aiq;
        A[i * m + q] = s * aip + c * aiq;
        const T vip = Vs[p * m + i], viq = Vs[q * m + i];
        Vs[p * m + i] = c * vip - s * viq;
        Vs[q * m + i] = s * vip + c * viq;
      }
      __syncthreads();
      for (int e = tid; e < (m / 2) * m; e += blockDim.x) {
        const int kk = e / m, j = e - kk * m;
        const int p = pr[2 * kk], q = pr[2 * kk + 1];
        const T c = cs[kk], s = cs[m / 2 + kk];
        const T apj = A[p * m + j], aqj = A[q * m + j];
        A[p * m + j] = c * apj - s * aqj;
        A[q * m + j] = s * apj + c * aqj;
      }
      __syncthreads();
    }
  }
  return sweep;
}

// rank of eigenvalue i in descending order (ties by index)
template <class T>
__device__ __forceinline__ int eig_rank(const T* A, int m, int n, int i) {
  const T li = A[i * m + i];
  int rank = 0;
  for (int j = 0; j < n; ++j) {
    const T lj = A[j * m + j];
    if (lj > li || (lj == li && j < i)) ++rank;
  }
  return rank;
}

}  // namespace tfx
