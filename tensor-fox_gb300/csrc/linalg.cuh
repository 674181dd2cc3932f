// CTA-level dense linear algebra shared by the single-problem and batched kernels.
#pragma once
#include "tfx_common.cuh"

namespace tfx {

// Symmetric eigensolver on one CTA: cyclic Jacobi with the round-robin
// (tournament) ordering, m/2 disjoint rotations per round.  A (m x m, m even,
// row-major, symmetric, zero-padded beyond n) and Vs (m x m, column p at
// Vs[p*m]) live in shared memory; cs holds m values, pr m+2 ints, red at least
// two doubles (used as three int flags).  On return the diagonal of A holds the
// eigenvalues and the columns of Vs the eigenvectors (unsorted).
//
// A pair (p, q) is rotated while |a_pq| > tol * sqrt(|a_pp a_qq|) (the
// relative threshold of Demmel and Veselic, "Jacobi's method is more accurate
// than QR", 1992), and the rotated a_pq is set to zero exactly, so the sweeps
// end once a whole sweep rotates nothing; max_sweeps is only a safety cap.
// One round updates every 2 x 2 block (rows of pair P, columns of pair Q) in
// a single pass, R_P^T A_PQ R_Q, written to both triangles so A stays exactly
// symmetric.  blockDim.x must be a multiple of 32.
template <class T>
__device__ int cta_jacobi(T* A, T* Vs, T* cs, int* pr, double* red, int m, int max_sweeps,
                          unsigned* blk = nullptr, T* cs2 = nullptr, int* pr2 = nullptr) {
  const int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, wid = tid >> 5, nw = nt >> 5;
  const int h = m / 2;
  const T tol = sizeof(T) == 8 ? T(4.5e-16) : T(2.4e-7);
  // flag[s % 3]: a rotation happened in sweep s.  The flag cleared at the
  // start of sweep s was last read at the end of sweep s - 2, with the
  // barriers of sweep s - 1 in between.
  volatile int* flag = (volatile int*)red;
  if (tid == 0) flag[0] = 0;
  // optional list of the h(h+1)/2 upper-triangle blocks (kp << 16 | kq), so
  // that every thread takes at most a few blocks without index arithmetic
  const int nblk = h * (h + 1) / 2;
  if (blk)
    for (int kp = wid; kp < h; kp += nw)
      for (int kq = kp + lane; kq < h; kq += 32) blk[kp * h - kp * (kp - 1) / 2 + (kq - kp)] = (kp << 16) | kq;
  // the rotations of one round: pair kk = (p, q) and its (c, s), by threads
  // t0, t0 + step, ...; a rotation sets flag[fl]
  auto params = [&](int round, T* csx, int* prx, int fl, int t0, int step) {
    for (int kk = t0; kk < h; kk += step) {
      // round-robin pairs; both sums stay below 2(m-1), so one subtraction
      // replaces the modulo
      int a = kk + round, b = m - 1 - kk + round;
      if (a >= m - 1) a -= m - 1;
      if (b >= m - 1) b -= m - 1;
      if (kk == 0) a = m - 1;
      const int p = a < b ? a : b, q = a < b ? b : a;
      prx[2 * kk] = p;
      prx[2 * kk + 1] = q;
      // rotation in the working precision (FP64 division and square root
      // are slow on GB300; the FP64 path keeps them in FP64).  This chain
      // runs on one warp while the block waits, so the FP32 path uses the
      // approximate reciprocal / reciprocal square root: an angle off by an
      // ulp still gives an orthogonal rotation (c = 1/sqrt(1+t^2), s = t c)
      // and the next sweep corrects the residue.
      const T apq = A[p * m + q], app = A[p * m + p], aqq = A[q * m + q];
      T c = T(1), s = T(0);
      if (apq != T(0) && fabs(apq) * fabs(apq) > tol * tol * fabs(app * aqq)) {
        T t;
        if (sizeof(T) == 8) {
          const T tau = (aqq - app) / (T(2) * apq);
          const T at = fabs(tau);
          // for huge |tau| use t ~ 1/(2 tau) to avoid overflow of tau*tau
          t = (at > T(1e150)) ? T(1) / (T(2) * tau) : (tau >= T(0) ? T(1) : T(-1)) / (at + sqrt(T(1) + tau * tau));
          c = T(1) / sqrt(T(1) + t * t);
        } else {
          const float tau = __fdividef((float)(aqq - app), 2.f * (float)apq);
          const float at = fabsf(tau);
          const float s2 = fmaf(tau, tau, 1.f);
          const float tt = (at > 1e18f) ? __fdividef(0.5f, tau) : copysignf(__fdividef(1.f, at + s2 * rsqrtf(s2)), tau);
          t = (T)tt;
          c = (T)rsqrtf(fmaf(tt, tt, 1.f));
        }
        s = t * c;
        flag[fl] = 1;
      }
      csx[kk] = c;
      csx[h + kk] = s;
    }
  };
  // R_P^T A_PQ R_Q for one upper-triangle block, mirrored below
  auto rotate_block = [&](const T* csx, const int* prx, int kp, int kq) {
    const int p = prx[2 * kp], q = prx[2 * kp + 1], r = prx[2 * kq], u = prx[2 * kq + 1];
    const T cp = csx[kp], sp = csx[h + kp], cr = csx[kq], sr = csx[h + kq];
    if (sp == T(0) && sr == T(0)) return;
    // columns (r, u) rotated first, then rows (p, q)
    const T apr = A[p * m + r], apu = A[p * m + u], aqr = A[q * m + r], aqu = A[q * m + u];
    const T xpr = cr * apr - sr * apu, xpu = sr * apr + cr * apu;
    const T xqr = cr * aqr - sr * aqu, xqu = sr * aqr + cr * aqu;
    T ypr = cp * xpr - sp * xqr, yqr = sp * xpr + cp * xqr;
    T ypu = cp * xpu - sp * xqu, yqu = sp * xpu + cp * xqu;
    if (kp == kq) {
      // diagonal block: the rotation annihilates a_pq exactly
      ypu = T(0);
      yqr = T(0);
    }
    A[p * m + r] = ypr;
    A[p * m + u] = ypu;
    A[q * m + r] = yqr;
    A[q * m + u] = yqu;
    if (kp != kq) {
      A[r * m + p] = ypr;
      A[u * m + p] = ypu;
      A[r * m + q] = yqr;
      A[u * m + q] = yqu;
    }
  };
  auto blocks = [&](const T* csx, const int* prx) {
    if (blk) {
      for (int e = tid; e < nblk; e += nt) rotate_block(csx, prx, (int)(blk[e] >> 16), (int)(blk[e] & 0xffffu));
    } else {
      // warp w takes block rows kp = w, w + nw, ...; its lanes the columns
      for (int kp = wid; kp < h; kp += nw)
        for (int kq = kp + lane; kq < h; kq += 32) rotate_block(csx, prx, kp, kq);
    }
  };
  // V's columns of every rotated pair, warps w0, w0 + nws, ...
  auto vupd = [&](const T* csx, const int* prx, int w0, int nws) {
    for (int kk = wid - w0; kk < h; kk += nws) {
      const T s = csx[h + kk];
      if (s == T(0)) continue;
      const int p = prx[2 * kk], q = prx[2 * kk + 1];
      const T c = csx[kk];
      T* vp = Vs + p * m;
      T* vq = Vs + q * m;
      for (int i = lane; i < m; i += 32) {
        const T vip = vp[i], viq = vq[i];
        vp[i] = c * vip - s * viq;
        vq[i] = s * vip + c * viq;
      }
    }
  };
  // true when some pair still exceeds the rotation threshold (the test of
  // params): a sweep after which none does would rotate nothing, so the loop
  // stops without running it (same result, one sweep fewer)
  auto pending = [&]() -> bool {
    bool mine = false;
    for (int p = wid; p < m; p += nw)
      for (int q = p + 1 + lane; q < m; q += 32) {
        const T apq = A[p * m + q], app = A[p * m + p], aqq = A[q * m + q];
        if (apq != T(0) && fabs(apq) * fabs(apq) > tol * tol * fabs(app * aqq)) mine = true;
      }
    return __syncthreads_or(mine) != 0;
  };
  __syncthreads();
  int sweep = 0;
  if (cs2 && pr2 && nw >= 2) {
    // two parameter slots: while warp 0 computes the next round's rotations
    // (from the matrix this round's blocks left), warps 1.. apply this
    // round's rotations to V, so V's update leaves the critical path.  The
    // same operations in the same order per element as the one-slot form.
    T* CS[2] = {cs, cs2};
    int* PR[2] = {pr, pr2};
    if (wid == 0) params(0, CS[0], PR[0], 0, lane, 32);
    __syncthreads();
    int g = 0;
    for (sweep = 0; sweep < max_sweeps; ++sweep) {
      if (tid == 0) flag[(sweep + 1) % 3] = 0;
      for (int round = 0; round < m - 1; ++round, ++g) {
        const int sl = g & 1;
        blocks(CS[sl], PR[sl]);
        __syncthreads();
        if (wid == 0) {
          const bool last = round + 1 == m - 1;
          params(last ? 0 : round + 1, CS[sl ^ 1], PR[sl ^ 1], (last ? sweep + 1 : sweep) % 3, lane, 32);
        } else {
          vupd(CS[sl], PR[sl], 1, nw - 1);
        }
        __syncthreads();
      }
      if (!pending()) {
        ++sweep;
        break;
      }
      const int rotated = flag[sweep % 3];
      if (!rotated) break;
    }
  } else {
    for (sweep = 0; sweep < max_sweeps; ++sweep) {
      if (tid == 0) flag[(sweep + 1) % 3] = 0;
      for (int round = 0; round < m - 1; ++round) {
        params(round, cs, pr, sweep % 3, tid, nt);
        __syncthreads();
        blocks(cs, pr);
        vupd(cs, pr, 0, nw);
        __syncthreads();
      }
      if (!pending()) {
        ++sweep;
        break;
      }
      const int rotated = flag[sweep % 3];
      if (!rotated) break;
    }
  }
  __syncthreads();
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
