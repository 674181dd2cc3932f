#pragma once
// Cluster-persistent damped Gauss-Newton CPD engine (device code, included by
// dgn_engine_f32.cu and dgn_engine_f64.cu).
//
// One thread-block cluster (1..16 CTAs) solves one dense CPD problem from start
// to finish: Gramians and Hadamard products, the MTTKRP gradient, the
// regularised preconditioned CG inner solve, the step update with column
// balancing, the residual norm, the dogleg fallback, the gain-ratio damping
// update and every stop test all run on the device, with no host round trip.
// A batch of problems is one launch (one cluster per problem).
//
// Algorithm: Tensor Fox v1.2.1 GaussNewton.py:29-251 (dGN), :254-312
// (compute_step), :315-398 (cg / cg_iterations), :401-427 (compute_grad),
// :520-581 (gramians / matvec), :584-627 (regularization / precond),
// :472-517 (gain ratio, damping, trust radius), :713-795 (dogleg);
// Conversion.py:21-49,361-387,412-444 (x2cpd / equalize / transform),
// Conversion.py:117-141 with Critical.py:14-22 (model unfolding and its
// distance to the tensor).
//
// Work split inside a team:
//   * Gramian entries, residual tiles and MTTKRP contraction ranges are split
//     across CTAs; MTTKRP partials are summed through distributed shared memory.
//   * Every n_x-vector of the CG (x, y, r, P, z, gradient) is split by factor
//     COLUMN: CTA c owns columns [c0, c1) of every mode.  With that split the
//     J^T J v product, the preconditioner, column balancing and the
//     best-iterate copy are all local; only the search direction Q is shared
//     (written to global memory, read back after a cluster barrier) and the
//     CG scalars are reduced deterministically.
#include "tfx_common.cuh"
#include "../../include/tfx_gb300_types.h"

#include <math.h>
#include <type_traits>
#include <stdio.h>

namespace tfx {

__host__ __device__ inline size_t al256(size_t v) { return (v + 255) & ~(size_t)255; }

// Per-problem workspace layout (offsets in bytes from problem.work).
struct WsLayout {
  size_t xc, xn, W, grad, jtj, y, r, P, Q, z, bx, by, bW, P1, P2, G, total;
};

__host__ __device__ inline WsLayout ws_layout(int L, int R, int nx, size_t es) {
  WsLayout w;
  size_t o = 0;
  size_t v = al256((size_t)nx * es);
  w.xc = o; o += v;
  w.xn = o; o += v;
  w.W = o; o += v;
  w.grad = o; o += v;
  w.jtj = o; o += v;
  w.y = o; o += v;
  w.r = o; o += v;
  w.P = o; o += v;
  w.Q = o; o += v;
  w.z = o; o += v;
  w.bx = o; o += v;
  w.by = o; o += v;
  w.bW = o; o += v;
  w.P1 = o; o += al256((size_t)L * R * R * es);
  w.P2 = o; o += al256((size_t)L * L * R * R * es);
  w.G = o; o += al256((size_t)L * R * R * sizeof(double));
  w.total = o;
  return w;
}

// Shared-memory layout of the third-order gradient (elements of the working
// type): three unpadded slab stages of d1*d2 values, the transposed own
// columns of the factors and M0 | M1 | M2 ((d0 + d1 + d2p) x 4 each), two
// buffers of per-warp M0 partials, per-warp M2 partials; then the stage
// barriers.  d2p: d2 rounded up to a multiple of four.
__host__ __device__ inline size_t g3_stage(int d1, int d2) { return ((size_t)d1 * d2 + 4 + 3) & ~(size_t)3; }
__host__ __device__ inline size_t g3_floats(int d0, int d1, int d2) {
  const size_t d2p = ((size_t)d2 + 3) & ~(size_t)3;
  return 3 * g3_stage(d1, d2) + 2 * (d0 + d1 + d2p) * 4 + 2 * (TFX_THREADS / 32) * 4 +
         (TFX_THREADS / 32) * d2p * 4 + 2 * (TFX_THREADS / 32) * 64;
}
// offset (elements) of the slab-split gradient's M0 warp partials inside it
__host__ __device__ inline size_t g3_p0x(int d0, int d1, int d2) {
  return g3_floats(d0, d1, d2) - 2 * (TFX_THREADS / 32) * 64;
}

struct SmemPlan {
  size_t sA, sB, sPart, sAk, sY, sM, sDG, sGam, sNorm, sBase, sIdx, rs4, rs12, misc, hist, rs1, rs1b, sScale, wsl, sG3, sE3;
  size_t sQf, sWf, sP1o, sP2o, sVec;  // staged operands of the CG (valid when stage != 0)
  int stage;
  size_t total;
};

__host__ __device__ inline size_t al16(size_t v) { return (v + 15) & ~(size_t)15; }

__host__ __device__ inline SmemPlan smem_plan(int TS, size_t es, int maxL, int maxR, int maxd, int maxncol,
                                               int maxiter, int maxnx, int maxsumd, int stage) {
  SmemPlan p;
  const int BM = 16 * TS, BN = 16 * TS;
  size_t o = 0;
  p.sA = o; o += al16((size_t)TFX_BK * (BM + 1) * es);
  p.sB = o; o += al16((size_t)TFX_BK * (BN + 1) * es);
  p.sPart = o; o += al16((size_t)maxd * maxR * es);
  p.sAk = o; o += al16((size_t)maxL * maxR * maxncol * es);
  p.sY = o; o += al16((size_t)maxL * maxR * ((maxncol + 3) & ~3) * es);
  p.sM = o; o += al16((size_t)maxL * maxncol * es);
  p.sDG = o; o += al16((size_t)maxL * maxncol * es);
  p.sGam = o; o += al16((size_t)maxL * maxncol * sizeof(double));
  p.sNorm = o; o += al16((size_t)maxL * maxncol * sizeof(double));
  const int NB = TFX_BK > BN ? TFX_BK : BN;
  p.sBase = o; o += al16((size_t)NB * sizeof(long long));
  p.sIdx = o; o += al16((size_t)NB * maxL * sizeof(int));
  p.rs4 = o; o += al16(sizeof(RedScratch<4>));
  p.rs12 = o; o += al16(sizeof(RedScratch<TFX_MAX_ORDER>));
  p.misc = o; o += 64 + 16 * TFX_MAX_ORDER * 8;
  p.hist = o; o += al16((size_t)2 * maxiter * sizeof(double));
  p.rs1 = o; o += al16(sizeof(RedScratch<1>));
  p.rs1b = o; o += al16(sizeof(RedScratch<1>));
  p.sScale = o; o += al16((size_t)maxL * maxncol * es);
  p.wsl = o; o += al16(sizeof(PushSlots<3>));
  // third-order gradient scratch (every mode up to 64): three slab stages,
  // transposed own factor columns, M0 | M1 | M2, partial sums, stage barriers
  p.sG3 = 0;
  p.sE3 = 0;
  if (maxL == 3 && maxd <= 64) {
    p.sG3 = o;
    o += al16(g3_floats(maxd, maxd, maxd) * es + 64);
    // residual scratch: W1 and W2 with rows padded to four (R x d padded)
    p.sE3 = o;
    o += al16((size_t)maxR * 2 * (((size_t)maxd + 3) & ~(size_t)3) * es);
  }
  p.stage = stage;
  p.sQf = p.sWf = p.sP1o = p.sP2o = p.sVec = o;
  if (stage) {
    p.sQf = o; o += al16((size_t)maxnx * es);
    p.sWf = o; o += al16((size_t)maxnx * es);
    p.sP1o = o; o += al16((size_t)maxL * maxR * ((maxncol + 3) & ~3) * es);
    p.sP2o = o; o += al16((size_t)maxL * maxL * maxR * maxncol * es);
    // the CTA's own slices of r, P, y, z and the expanded M, damp*Gamma
    const size_t own = (size_t)maxncol * (size_t)maxsumd;
    p.sVec = o; o += al16(6 * own * es);
  }
  p.total = o;
  return p;
}

__device__ __forceinline__ char* dyn_smem() {
  extern __shared__ __align__(16) char tfx_dsm[];
  return tfx_dsm;
}

// ---------------------------------------------------------------------------
// CG inner solve of one team, written with register-resident scalars and
// shared-memory pointers derived from the dynamic shared-memory symbol, so
// that its hot loops use direct shared-memory accesses.
//
// J^T J v for the owned columns (GaussNewton.py:371-377, 551-581):
//   A_k = D_k^T W_k,  Y_l = sum_{k != l} P2[l][k] o A_k,  z_l = W_l Y_l + D_l P1_l
// Preconditioned CG (GaussNewton.py:315-398), reference quirks included: the
// first new direction is (1+beta) r because P aliases the residual array.
// STAGED: the full input vector, the factors and the owned P1/P2 columns sit in
// shared memory; otherwise they are read from global memory (L2).
// ---------------------------------------------------------------------------
struct CgOffsets {
  size_t d, sQf, sWf, sP1o, sP2o, sAk, sY, sM, sDG, rs4, rs1, sVec, wsl;
};

// Copy n elements written by other CTAs of the team from global memory into
// shared memory.  ld.global.cg reads at L2 (coherent across SMs) and lets the
// loads of one thread overlap instead of queueing behind its shared stores.
template <class T>
__device__ __forceinline__ void stage_copy(T* sdst, const T* gsrc, int n) {
  constexpr int V = 16 / sizeof(T);
  using V4 = typename std::conditional<sizeof(T) == 4, float4, double2>::type;
  const int nv = n / V;
  const V4* src = reinterpret_cast<const V4*>(gsrc);
  V4* dst = reinterpret_cast<V4*>(sdst);
  int e = threadIdx.x;
  for (; e + 3 * TFX_THREADS < nv; e += 4 * TFX_THREADS) {
    const V4 a = __ldcg(src + e), b = __ldcg(src + e + TFX_THREADS);
    const V4 c = __ldcg(src + e + 2 * TFX_THREADS), d4 = __ldcg(src + e + 3 * TFX_THREADS);
    dst[e] = a;
    dst[e + TFX_THREADS] = b;
    dst[e + 2 * TFX_THREADS] = c;
    dst[e + 3 * TFX_THREADS] = d4;
  }
  for (; e < nv; e += TFX_THREADS) dst[e] = __ldcg(src + e);
  for (int t = nv * V + threadIdx.x; t < n; t += TFX_THREADS) sdst[t] = __ldcg(gsrc + t);
}

// Two rows (dv0, dv1) of D_k against CN owned columns of W_k (column u at
// wv + u dk): out[j][u] = sum_i dv_j[i] wv[u dk + i] as two chains, even and
// odd i, added at the end.  V2: pairs of i as one 8- or 16-byte read (dk and
// the offsets even).
template <class T, int CN, bool V2>
__device__ __forceinline__ void ak_tile(const int dk, const T* dv0, const T* dv1, const T* wv, T (&out)[2][4]) {
  using T2 = typename std::conditional<sizeof(T) == 4, float2, double2>::type;
  T ev[2][CN], od[2][CN];
#pragma unroll
  for (int u = 0; u < CN; ++u) ev[0][u] = ev[1][u] = od[0][u] = od[1][u] = T(0);
  int i = 0;
  if (V2) {
#pragma unroll 2
    for (; i < dk; i += 2) {
      const T2 x0 = *reinterpret_cast<const T2*>(dv0 + i);
      const T2 x1 = *reinterpret_cast<const T2*>(dv1 + i);
#pragma unroll
      for (int u = 0; u < CN; ++u) {
        const T2 w = *reinterpret_cast<const T2*>(wv + u * dk + i);
        ev[0][u] = fma((T)x0.x, (T)w.x, ev[0][u]);
        od[0][u] = fma((T)x0.y, (T)w.y, od[0][u]);
        ev[1][u] = fma((T)x1.x, (T)w.x, ev[1][u]);
        od[1][u] = fma((T)x1.y, (T)w.y, od[1][u]);
      }
    }
  } else {
#pragma unroll 2
    for (; i + 1 < dk; i += 2) {
      const T x00 = dv0[i], x01 = dv0[i + 1], x10 = dv1[i], x11 = dv1[i + 1];
#pragma unroll
      for (int u = 0; u < CN; ++u) {
        const T w0 = wv[u * dk + i], w1 = wv[u * dk + i + 1];
        ev[0][u] = fma(x00, w0, ev[0][u]);
        od[0][u] = fma(x01, w1, od[0][u]);
        ev[1][u] = fma(x10, w0, ev[1][u]);
        od[1][u] = fma(x11, w1, od[1][u]);
      }
    }
    if (i < dk) {
#pragma unroll
      for (int u = 0; u < CN; ++u) {
        ev[0][u] = fma(dv0[i], wv[u * dk + i], ev[0][u]);
        ev[1][u] = fma(dv1[i], wv[u * dk + i], ev[1][u]);
      }
    }
  }
#pragma unroll
  for (int u = 0; u < CN; ++u) {
    out[0][u] = ev[0][u] + od[0][u];
    out[1][u] = ev[1][u] + od[1][u];
  }
}

// z rows of CN owned columns (the scalar-load path of the matvec's last pass):
// a1[u] += W_l[i, r] Y_l[r, u], a2[u] += D_l[i, r] P1_l[r, u], r ascending
template <class T, int CN>
__device__ __forceinline__ void z_cols(const int R, const int dl, const T* wrow, const T* drow, const T* yc,
                                       const int ys, const T* p1c, const int p1s, T (&a1)[4], T (&a2)[4]) {
#pragma unroll 4
  for (int r = 0; r < R; ++r) {
    const T w = wrow[r * dl], dd = drow[r * dl];
#pragma unroll
    for (int u = 0; u < CN; ++u) {
      a1[u] = fma(w, yc[r * ys + u], a1[u]);
      a2[u] = fma(dd, p1c[r * p1s + u], a2[u]);
    }
  }
}

template <class T, bool STAGED>
__device__ __forceinline__ void cg_matvec(const int L, const int R, const int nx, const int ncol, const int c0,
                                          const CgOffsets so, const T* Dglob, T* zout, const T* Wg, const T* P1g,
                                          const T* P2g, T* zloc = nullptr, long long* cprof = nullptr,
                                          bool prestaged = false) {
  // timers accumulate in registers of thread 0 (cprof points at its private array)
  long long tc = cprof ? clock64() : 0;
  auto ctick = [&](int ph) {
    if (cprof) {
      const long long now = clock64();
      cprof[ph] += now - tc;
      tc = now;
    }
  };
  char* sm = dyn_smem();
  const int* d = (const int*)(sm + so.d);
  const int* off = d + TFX_MAX_ORDER;
  T* sAk = (T*)(sm + so.sAk);
  T* sY = (T*)(sm + so.sY);
  const int tid = threadIdx.x;
  const T* Din;
  const T* Wr;
  if (STAGED) {
    // prestaged: the team already pushed the full input into sQf
    T* sQf = (T*)(sm + so.sQf);
    if (!prestaged) {
      stage_copy(sQf, Dglob, nx);
      __syncthreads();
    }
    ctick(1);
    Din = sQf;
    Wr = (const T*)(sm + so.sWf);
  } else {
    Din = Dglob;
    Wr = Wg;
  }
  const T* sP1o = (const T*)(sm + so.sP1o);
  const T* sP2o = (const T*)(sm + so.sP2o);
  const int RN = R * ncol;
  // A_k = D_k^T W_k on the owned columns: a thread takes rows a and a + RP of
  // D_k and up to four owned columns, so that every loaded value feeds two or
  // more multiply-adds (the pass is bound by shared-memory wavefronts); each
  // dot keeps its two interleaved chains (even and odd i), as one output per
  // thread would.
  {
    const int RP = (R + 1) >> 1, ncg4 = (ncol + 3) >> 2;
    for (int e = tid; e < L * ncg4 * RP; e += TFX_THREADS) {
      const int k = e / (ncg4 * RP), rem = e - k * ncg4 * RP, cg = rem / RP, ap = rem - cg * RP;
      const int a0 = ap, a1 = ap + RP < R ? ap + RP : ap;
      const int dk = d[k], cb = cg * 4, cn = min(4, ncol - cb);
      const T* dv0 = Din + off[k] + a0 * dk;
      const T* dv1 = Din + off[k] + a1 * dk;
      const T* wv = Wr + off[k] + (c0 + cb) * dk;
      const bool v2 = ((dk | off[k]) & 1) == 0 &&
                      (((unsigned long long)Din | (unsigned long long)Wr) & (2 * sizeof(T) - 1)) == 0;
      T out[2][4];
      switch (cn) {
        case 1: v2 ? ak_tile<T, 1, true>(dk, dv0, dv1, wv, out) : ak_tile<T, 1, false>(dk, dv0, dv1, wv, out); break;
        case 2: v2 ? ak_tile<T, 2, true>(dk, dv0, dv1, wv, out) : ak_tile<T, 2, false>(dk, dv0, dv1, wv, out); break;
        case 3: v2 ? ak_tile<T, 3, true>(dk, dv0, dv1, wv, out) : ak_tile<T, 3, false>(dk, dv0, dv1, wv, out); break;
        default: v2 ? ak_tile<T, 4, true>(dk, dv0, dv1, wv, out) : ak_tile<T, 4, false>(dk, dv0, dv1, wv, out); break;
      }
      T* o0 = sAk + (size_t)k * RN + a0 * ncol + cb;
      T* o1 = sAk + (size_t)k * RN + a1 * ncol + cb;
#pragma unroll
      for (int u = 0; u < 4; ++u)
        if (u < cn) {
          o0[u] = out[0][u];
          if (a1 != a0) o1[u] = out[1][u];
        }
    }
  }
  __syncthreads();
  ctick(2);
  // Y_l (rows of stride ncp, the owned column count rounded up to four, so
  // that the last pass reads four columns at once), one output per thread
  const int ncp = (ncol + 3) & ~3;
  for (int e = tid; e < L * RN; e += TFX_THREADS) {
    const int l = e / RN, q = e - l * RN, a = q / ncol, c = q - a * ncol;
    T acc = T(0);
    for (int k = 0; k < L; ++k) {
      if (k == l) continue;
      const T p2 = STAGED ? sP2o[((size_t)(l * L + k) * R + a) * ncol + c]
                          : P2g[((size_t)(l * L + k) * R + a) * R + c0 + c];
      acc += p2 * sAk[(size_t)k * RN + q];
    }
    sY[((size_t)l * R + a) * ncp + c] = acc;
  }
  __syncthreads();
  ctick(3);
  // z_l = W_l Y_l + D_l P1_l over all owned outputs of all modes at once;
  // a thread takes one row i of one mode and four owned columns
  const int sumd = nx / R;
  const int ncg = (ncol + 3) >> 2;
  for (int e = tid; e < ncg * sumd; e += TFX_THREADS) {
    const int cgi = e / sumd;
    int l = 0, i = e - cgi * sumd;
    while (i >= d[l]) {
      i -= d[l];
      ++l;
    }
    const int cb = cgi * 4, cn = min(4, ncol - cb);
    const int dl = d[l], ol = off[l];
    const T* wrow = Wr + ol + i;
    const T* drow = Din + ol + i;
    const T* yc = sY + (size_t)l * R * ncp + cb;
    const T* p1c = STAGED ? sP1o + (size_t)l * R * ncp + cb : P1g + (size_t)l * R * R + c0 + cb;
    const int p1s = STAGED ? ncp : R;
    T a1[4] = {T(0), T(0), T(0), T(0)}, a2[4] = {T(0), T(0), T(0), T(0)};
    if (sizeof(T) == 4 && STAGED) {
      // four owned columns as one 16-byte read of Y and of P1 per r (a
      // partial last group computes the padding columns and drops them)
#pragma unroll 4
      for (int r = 0; r < R; ++r) {
        const T w = wrow[r * dl], dd = drow[r * dl];
        const float4 y4 = *reinterpret_cast<const float4*>(yc + r * ncp);
        const float4 p4 = *reinterpret_cast<const float4*>(p1c + r * p1s);
        a1[0] = fma(w, (T)y4.x, a1[0]);
        a1[1] = fma(w, (T)y4.y, a1[1]);
        a1[2] = fma(w, (T)y4.z, a1[2]);
        a1[3] = fma(w, (T)y4.w, a1[3]);
        a2[0] = fma(dd, (T)p4.x, a2[0]);
        a2[1] = fma(dd, (T)p4.y, a2[1]);
        a2[2] = fma(dd, (T)p4.z, a2[2]);
        a2[3] = fma(dd, (T)p4.w, a2[3]);
      }
    } else {
      switch (cn) {
        case 1: z_cols<T, 1>(R, dl, wrow, drow, yc, ncp, p1c, p1s, a1, a2); break;
        case 2: z_cols<T, 2>(R, dl, wrow, drow, yc, ncp, p1c, p1s, a1, a2); break;
        case 3: z_cols<T, 3>(R, dl, wrow, drow, yc, ncp, p1c, p1s, a1, a2); break;
        default: z_cols<T, 4>(R, dl, wrow, drow, yc, ncp, p1c, p1s, a1, a2); break;
      }
    }
#pragma unroll
    for (int u = 0; u < 4; ++u)
      if (u < cn) {
        if (zloc)
          zloc[ncol * (ol / R) + (cb + u) * dl + i] = a1[u] + a2[u];
        else
          zout[ol + (c0 + cb + u) * dl + i] = a1[u] + a2[u];
      }
  }
  __syncthreads();
  ctick(4);
}

template <class T, bool STAGED>
__device__ __forceinline__ int cg_team(const Team tm, const int L, const int R, const int nx, const int ncol,
                                       const int c0, const CgOffsets so, T* grad, T* jtj, T* y, T* r, T* P, T* Q,
                                       T* z, const T* Wg, const T* P1g, const T* P2g, const int budget,
                                       const double cg_tol, double& rn_out, int& flipw, long long* cprof_g) {
  long long lprof[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  long long* cprof = cprof_g ? lprof : nullptr;
  long long tc = cprof ? clock64() : 0;
  auto ctick = [&](int ph) {
    if (cprof) {
      const long long now = clock64();
      cprof[ph] += now - tc;
      tc = now;
    }
  };
  char* sm = dyn_smem();
  const int* d = (const int*)(sm + so.d);
  const int* off = d + TFX_MAX_ORDER;
  const T* sM = (const T*)(sm + so.sM);
  const T* sDG = (const T*)(sm + so.sDG);
  PushSlots<1>* ps1 = (PushSlots<1>*)(sm + so.wsl);
  PushSlots<3>* ps3 = (PushSlots<3>*)(sm + so.wsl);
  T* sQf = (T*)(sm + so.sQf);
  const int tid = threadIdx.x;
  // own slice: element (l, c, i) lives at local index ncol*(off[l]/R) + c*d[l] + i
  const int own = ncol * (nx / R);
  T *vr, *vP, *vy, *vz, *vM, *vDG;
  if (STAGED) {
    vr = (T*)(sm + so.sVec);
    vP = vr + own;
    vy = vP + own;
    vz = vy + own;
    vM = vz + own;
    vDG = vM + own;
  }
  cg_matvec<T, STAGED>(L, R, nx, ncol, c0, so, grad, jtj, Wg, P1g, P2g);
  // the CG scalars live in the working precision: on the FP32 path every
  // thread would otherwise run FP64 divisions, which GB300 executes slowly
  Acc<T> v[1], tot[1];
  for (int l = 0; l < L; ++l) {
    const int dl = d[l], base = off[l] + c0 * dl, n = ncol * dl, lb = ncol * (off[l] / R);
    for (int e = tid; e < n; e += TFX_THREADS) {
      const int c = e / dl, g = base + e;
      const T m = sM[l * ncol + c];
      const T rr = m * __ldcg(grad + g);
      if (STAGED) {
        vM[lb + e] = m;
        vDG[lb + e] = sDG[l * ncol + c];
        vr[lb + e] = rr;
        vP[lb + e] = rr;
        vy[lb + e] = T(0);
      } else {
        r[g] = rr;
        P[g] = rr;
        y[g] = T(0);
      }
      v[0].fma_(rr, rr);
    }
  }
  team_sum_push<1>(tm, v, tot, ps1, flipw);
  Acc<T> rnA = tot[0];
  T rn = acc_val(rnA);
  if (rn == T(0)) {
    rn = T(1e-6);
    rnA = Acc<T>();
    rnA.add(rn);
  }
  int maxit = budget;
  T tol = (T)cg_tol;
  if (nx > 100) {
    maxit = min(maxit, nx);
  } else {
    tol = T(0);
  }
  int itn = 0;
  bool broke = false;
  for (itn = 0; itn < maxit; ++itn) {
    // Q = M P on the owned slice.  Staged: pushed straight into every team
    // member's shared-memory copy of the full vector (their previous reads of
    // it ended before the last team barrier); otherwise published through
    // global memory.  (Measured alternatives: publishing through global
    // memory and copying the full vector back from L2, by threads or by one
    // multicast bulk copy, take as long as the push.)
    for (int l = 0; l < L; ++l) {
      const int dl = d[l], base = off[l] + c0 * dl, n = ncol * dl, lb = ncol * (off[l] / R);
      for (int e = tid; e < n; e += TFX_THREADS) {
        if (STAGED) {
          const T q = vM[lb + e] * vP[lb + e];
          for (int rr = 0; rr < tm.size; ++rr) tm.peer(sQf, rr)[base + e] = q;
        } else {
          const int c = e / dl;
          Q[base + e] = sM[l * ncol + c] * P[base + e];
        }
      }
    }
    ctick(1);
    tm.sync();
    ctick(0);
    cg_matvec<T, STAGED>(L, R, nx, ncol, c0, so, Q, z, Wg, P1g, P2g, STAGED ? vz : nullptr, cprof, STAGED);
    if (cprof) tc = clock64();
    // FP32: one reduction gives P.z, r.z and z.z, and |r - alpha z|^2 follows
    // as rn - 2 alpha r.z + alpha^2 z.z in float-float; FP64 keeps the
    // reference's separate reduction of the updated residual
    constexpr bool MERGED = sizeof(T) == 4;
    Acc<T> w[3];
    const T* Qs = STAGED ? (const T*)sQf : Q;
    for (int l = 0; l < L; ++l) {
      const int dl = d[l], base = off[l] + c0 * dl, n = ncol * dl, lb = ncol * (off[l] / R);
      for (int e = tid; e < n; e += TFX_THREADS) {
        if (STAGED) {
          const T zz = vM[lb + e] * (vz[lb + e] + vDG[lb + e] * Qs[base + e]);
          vz[lb + e] = zz;
          w[0].fma_(vP[lb + e], zz);
          if (MERGED) {
            w[1].fma_(vr[lb + e], zz);
            w[2].fma_(zz, zz);
          }
        } else {
          const int c = e / dl, g = base + e;
          const T zz = sM[l * ncol + c] * (z[g] + sDG[l * ncol + c] * Q[g]);
          z[g] = zz;
          w[0].fma_(P[g], zz);
          if (MERGED) {
            w[1].fma_(r[g], zz);
            w[2].fma_(zz, zz);
          }
        }
      }
    }
    Acc<T> t3[3];
    if (MERGED) {
      team_sum_push<3>(tm, w, t3, ps3, flipw);
    } else {
      Acc<T> w1[1] = {w[0]};
      team_sum_push<1>(tm, w1, tot, ps1, flipw);
      t3[0] = tot[0];
    }
    ctick(5);
    T den = acc_val(t3[0]);
    if (den == T(0)) den = T(1e-6);
    const T ta = rn / den;
    Acc<T> u[1];
    if (STAGED) {
      for (int e = tid; e < own; e += TFX_THREADS) {
        vy[e] += ta * vP[e];
        const T rr = vr[e] - ta * vz[e];
        vr[e] = rr;
        u[0].fma_(rr, rr);
      }
    } else {
      for (int l = 0; l < L; ++l) {
        const int dl = d[l], base = off[l] + c0 * dl, n = ncol * dl;
        for (int e = tid; e < n; e += TFX_THREADS) {
          const int g = base + e;
          y[g] += ta * P[g];
          const T rr = r[g] - ta * z[g];
          r[g] = rr;
          u[0].fma_(rr, rr);
        }
      }
    }
    Acc<T> rnN;
    bool exact = !MERGED;
    if (MERGED) {
      // rn_new = rn - 2 alpha (r.z) + alpha^2 (z.z), exact products
      rnN = rnA;
      const T m2a = T(-2) * ta;
      rnN.fma_(m2a, t3[1].hi_or_v());
      rnN.fma_(m2a, t3[1].lo_or_0());
      const T a2 = ta * ta, a2e = fma(ta, ta, -a2);
      rnN.fma_(a2, t3[2].hi_or_v());
      rnN.fma_(a2e, t3[2].hi_or_v());
      rnN.fma_(a2, t3[2].lo_or_0());
      // deep cancellation: the stored residual's own rounding dominates, so
      // its norm is reduced directly (the same decision in every thread)
      if (!(acc_val(rnN) > T(1e-4) * rn)) exact = true;
    }
    if (exact) {
      team_sum_push<1>(tm, u, tot, ps1, flipw);
      rnN = tot[0];
    }
    ctick(6);
    const T rn_new = acc_val(rnN);
    const T tb = rn_new / rn;
    rn = rn_new;
    rnA = rnN;
    if (STAGED) {
      for (int e = tid; e < own; e += TFX_THREADS) vP[e] = (itn == 0) ? vr[e] + tb * vr[e] : vr[e] + tb * vP[e];
    } else {
      for (int l = 0; l < L; ++l) {
        const int dl = d[l], base = off[l] + c0 * dl, n = ncol * dl;
        for (int e = tid; e < n; e += TFX_THREADS) {
          const int g = base + e;
          P[g] = (itn == 0) ? r[g] + tb * r[g] : r[g] + tb * P[g];
        }
      }
    }
    ctick(7);
    if (rn <= tol) {
      broke = true;
      break;
    }
  }
  if (STAGED) {
    // the step leaves the team's shared memory for the update phase
    __syncthreads();
    for (int l = 0; l < L; ++l) {
      const int dl = d[l], base = off[l] + c0 * dl, n = ncol * dl, lb = ncol * (off[l] / R);
      for (int e = tid; e < n; e += TFX_THREADS) y[base + e] = vy[lb + e];
    }
  }
  // the next reader of sQf (the next matvec's staging) runs after a team barrier
  __syncthreads();
  if (cprof_g)
    for (int k = 0; k < 8; ++k) cprof_g[k] += lprof[k];
  rn_out = (double)rn;
  return broke ? itn + 1 : maxit;
}

// four consecutive 16-byte aligned values from shared memory as vector reads
__device__ __forceinline__ void lds4(const float* p, float (&v)[4]) {
  const float4 a = *reinterpret_cast<const float4*>(p);
  v[0] = a.x;
  v[1] = a.y;
  v[2] = a.z;
  v[3] = a.w;
}
__device__ __forceinline__ void lds4(const double* p, double (&v)[4]) {
  const double2 a = *reinterpret_cast<const double2*>(p), b = *reinterpret_cast<const double2*>(p + 2);
  v[0] = a.x;
  v[1] = a.y;
  v[2] = b.x;
  v[3] = b.y;
}

template <class T, int TS>
struct Engine {
  using TL = Tile<TS, TS>;
  Team tm;
  int tid;
  int L, R, nx, ncol, c0, c1, maxd;
  // problem shape, kept in shared memory (dynamically indexed in hot loops)
  int* d;
  int* off;
  long long* st;
  long long N;
  const T* Tt;
  T *xc, *xn, *W, *grad, *jtj, *y, *r, *P, *Q, *z, *bx, *by, *bW, *P1, *P2;
  double* G;
  T *sA, *sB, *sPart, *sAk, *sY, *sM, *sDG;
  double *sGam, *sNorm, *sMisc;
  long long* sBase;
  int* sIdx;
  RedScratch<4>* rs4;
  RedScratch<TFX_MAX_ORDER>* rs12;
  int flip4, flip12, flip1, flip1b, flipw;
  RedScratch<1>* rs1b;
  T* sScale;
  double damp, Tsize;
  tfx_dgn_options op;
  // The reference's factor list holds ONE array L times (after a symmetrising
  // transform, or a symmetric start); see to_factors.
  bool aliased;
  // staged operands: full search direction and factors, owned P1/P2 columns
  int stage;
  T *sQf, *sWf, *sP1o, *sP2o;
  T* sG3;       // third-order gradient scratch, or nullptr
  size_t g3off; // its offset in dynamic shared memory
  unsigned g3base;  // slabs streamed so far: slab n uses stage n % 3, phase (n / 3) & 1
  size_t e3off;     // third-order residual scratch offset
  int g3err;      // a slab wait ran out
  const T* Wr;  // factors to read: shared-memory copy when staged

  __device__ __forceinline__ T& P1at(int l, int a, int c) {
    return stage ? sP1o[((size_t)l * R + a) * ((ncol + 3) & ~3) + c] : P1[((size_t)l * R + a) * R + c0 + c];
  }
  __device__ __forceinline__ T& P2at(int l, int k, int a, int c) {
    return stage ? sP2o[((size_t)(l * L + k) * R + a) * ncol + c] : P2[((size_t)(l * L + k) * R + a) * R + c0 + c];
  }

  // copy the (complete, synchronised) global factors into shared memory
  __device__ void stage_W() {
    if (stage) {
      stage_copy(sWf, W, nx);
      __syncthreads();
      Wr = sWf;
    } else {
      Wr = W;
    }
  }

  // -------------------------------------------------------------------------
  // generic small contraction: out(m, n) = sum_k A(m, k) B(k, n)
  // -------------------------------------------------------------------------
  template <class FA, class FB, class FE>
  __device__ void gemm(int M, int Nn, int K, FA fa, FB fb, FE fe) {
    const int tx = tid & 15, ty = tid >> 4;
    for (int m0 = 0; m0 < M; m0 += TL::BM) {
      for (int n0 = 0; n0 < Nn; n0 += TL::BN) {
        T acc[TS][TS];
        tile_zero<T, TS, TS>(acc);
        for (int k0 = 0; k0 < K; k0 += TFX_BK) {
          const int kc = min(TFX_BK, K - k0);
          for (int e = tid; e < TFX_BK * TL::BM; e += TFX_THREADS) {
            const int kk = e / TL::BM, mm = e - kk * TL::BM;
            sA[kk * TL::LDA + mm] = (kk < kc && m0 + mm < M) ? fa(m0 + mm, k0 + kk) : T(0);
          }
          for (int e = tid; e < TFX_BK * TL::BN; e += TFX_THREADS) {
            const int kk = e / TL::BN, nn = e - kk * TL::BN;
            sB[kk * TL::LDB + nn] = (kk < kc && n0 + nn < Nn) ? fb(k0 + kk, n0 + nn) : T(0);
          }
          __syncthreads();
          tile_fma<T, TS, TS>(sA, sB, acc, kc);
          __syncthreads();
        }
#pragma unroll
        for (int u = 0; u < TS; ++u)
#pragma unroll
          for (int v = 0; v < TS; ++v) {
            const int m = m0 + ty + 16 * u, n = n0 + tx + 16 * v;
            if (m < M && n < Nn) fe(m, n, acc[u][v]);
          }
      }
    }
  }

  // loop over the elements this CTA owns (columns [c0, c1) of every mode)
  template <class F>
  __device__ __forceinline__ void for_own(F f) {
    for (int l = 0; l < L; ++l) {
      const int n = ncol * d[l];
      const int base = off[l] + c0 * d[l];
      for (int e = tid; e < n; e += TFX_THREADS) {
        const int c = e / d[l];
        f(base + e, l, c);
      }
    }
  }

  // -------------------------------------------------------------------------
  __device__ void tensor_norms(double& tsize, double& meanabs) {
    double v[4] = {0.0, 0.0, 0.0, 0.0};
    for (long long e = (long long)tm.rank * TFX_THREADS + tid; e < N; e += (long long)tm.size * TFX_THREADS) {
      const double t = (double)Tt[e];
      v[0] += t * t;
      v[1] += fabs(t);
    }
    team_sum<4>(tm, v, rs4, flip4);
    tsize = sqrt(v[0]);
    meanabs = v[1] / (double)N;
  }

  // GaussNewton.py:520-548 and :584-627.  G in FP64 (FP32 products summed in
  // FP64 every 16 terms when T is float); P1/P2 rounded to T for the matvec.
  __device__ void gramians_and_precond() {
    const int RR = R * R;
    for (int u = tm.rank * TFX_THREADS + tid; u < L * RR; u += tm.size * TFX_THREADS) {
      const int l = u / RR, q = u - l * RR, a = q / R, b = q - a * R;
      if (a > b) continue;
      const T* pa = Wr + off[l] + a * d[l];
      const T* pb = Wr + off[l] + b * d[l];
      double acc = 0.0;
      for (int i0 = 0; i0 < d[l]; i0 += 16) {
        T p = T(0);
        const int ie = min(d[l], i0 + 16);
        for (int i = i0; i < ie; ++i) p = fma(pa[i], pb[i], p);
        acc += (double)p;
      }
      G[(size_t)l * RR + a * R + b] = acc;
      G[(size_t)l * RR + b * R + a] = acc;
    }
    tm.sync();
    // P2[l][k] = prod_{m not in {l,k}} G_m (ascending m), own columns only
    for (int e = tid; e < L * L * R * ncol; e += TFX_THREADS) {
      const int lk = e / (R * ncol), q = e - lk * (R * ncol), a = q / ncol, c = q - a * ncol;
      const int l = lk / L, k = lk - l * L;
      if (l == k) continue;
      const int b = c0 + c;
      double p = 1.0;
      for (int m = 0; m < L; ++m)
        if (m != l && m != k) p *= G[(size_t)m * RR + a * R + b];
      P2at(l, k, a, c) = (T)p;
    }
    // P1 with the reference's product order
    for (int e = tid; e < L * R * ncol; e += TFX_THREADS) {
      const int l = e / (R * ncol), q = e - l * (R * ncol), a = q / ncol, c = q - a * ncol;
      const int b = c0 + c;
      P1at(l, a, c) = (T)p1_value(l, a, b);
    }
    // tmp = max |P1[L-1]| over the whole matrix (every CTA computes it)
    double mx = 0.0;
    for (int q = tid; q < RR; q += TFX_THREADS) mx = fmax(mx, fabs(p1_value(L - 1, q / R, q % R)));
    mx = warp_max(mx);
    if ((tid & 31) == 0) rs4->warp[tid >> 5][0] = mx;
    __syncthreads();
    if (tid == 0) {
      double m2 = rs4->warp[0][0];
      for (int w = 1; w < TFX_THREADS / 32; ++w) m2 = fmax(m2, rs4->warp[w][0]);
      sMisc[0] = m2;
    }
    __syncthreads();
    const double tmp = sMisc[0];
    for (int e = tid; e < L * ncol; e += TFX_THREADS) {
      const int l = e / ncol, c = e - l * ncol, b = c0 + c;
      const double g = tmp * sqrt(fabs(p1_value(l, b, b)));
      sGam[e] = g;
      const double m = 1.0 / sqrt(g * g + damp * damp * (g * g));
      sM[e] = (T)m;
      sDG[e] = (T)(damp * g);
    }
    __syncthreads();
  }

  __device__ __forceinline__ double p2_value(int l, int k, int a, int b) const {
    const int RR = R * R;
    double p = 1.0;
    for (int m = 0; m < L; ++m)
      if (m != l && m != k) p *= G[(size_t)m * RR + a * R + b];
    return p;
  }
  __device__ __forceinline__ double p1_value(int l, int a, int b) const {
    const int RR = R * R;
    int k;
    if (l == 0) k = 1;
    else if (l < L - 1) k = l - 1;
    else k = 0;
    return p2_value(l, k, a, b) * G[(size_t)k * RR + a * R + b];
  }

  // -------------------------------------------------------------------------
  // Third-order gradient for the owned columns without team communication.
  // The tensor streams through a ring of three shared-memory stages, one slab
  // T[i, :, :] (contiguous, d1*d2 values) per bulk copy (cp.async.bulk,
  // completion on an mbarrier).  Per group of four owned columns c and slab i,
  // eight threads per row j (rows j and j + 32) take k-groups q and q + 8 and form
  //   Y[j, c]   = sum_k T[i, j, k] W2[k, c]           (W2 rows in registers)
  //   M2[k, c] += T[i, j, k] W0[i, c] W1[j, c]         (registers, summed at the end)
  //   M1[j, c] += Y[j, c] W0[i, c],  M0[i, c] = sum_j Y[j, c] W1[j, c]
  // (the dimension tree of MTTKRP), and grad_l = M_l - W_l P1_l, the negative
  // of GaussNewton.py:401-427.  Every sum has a fixed order: deterministic.
  // Needs every mode <= 64, d1*d2 % 4 == 0 and a 16-byte aligned tensor.
  // -------------------------------------------------------------------------
  template <bool STAGED>
  __device__ __noinline__ void gradient_l3() {
    long long gt = gprof ? clock64() : 0;
    auto gtick = [&](int ph) {
      if (gprof) {
        const long long now = clock64();
        gprof[ph] += now - gt;
        gt = now;
      }
    };
    constexpr int NW = TFX_THREADS / 32;
    const int d0 = d[0], d1 = d[1], d2 = d[2];
    const int d2p = (d2 + 3) & ~3;
    const int nkg = d2p >> 2;  // <= 16
    char* smb = dyn_smem();
    const T* Wl = STAGED ? (const T*)(smb + cgo.sWf) : W;
    const T* P1l = STAGED ? (const T*)(smb + cgo.sP1o) : P1;
    const int p1s = STAGED ? ((ncol + 3) & ~3) : R;  // P1 column stride
    const int p1c = STAGED ? 0 : c0;    // P1 column offset
    const int SL = (int)g3_stage(d1, d2);
    T* sT = (T*)(smb + g3off);                 // 3 stages
    T* sF = sT + 3 * SL;                       // (d0 + d1 + d2p) x 4, own columns transposed
    T* sMM = sF + (d0 + d1 + d2p) * 4;         // M0 | M1 | M2
    T* sP0 = sMM + (d0 + d1 + d2p) * 4;        // [2][NW][4] M0 warp partials
    T* sR2 = sP0 + 2 * NW * 4;                 // [NW][d2p][4] M2 warp partials
    unsigned long long* mbar = (unsigned long long*)(smb + g3off + g3_floats(d0, d1, d2) * sizeof(T));
    const T* sA4 = sF;
    const T* sB4 = sF + d0 * 4;
    const T* sC4 = sF + (d0 + d1) * 4;
    T* sM0 = sMM;
    T* sM1 = sMM + d0 * 4;
    T* sM2 = sMM + (d0 + d1) * 4;
    const int lane = tid & 31, wid = tid >> 5;
    const int rs = tid >> 3, q8 = tid & 7;  // rows rs and rs + 32; k-groups q8 and q8 + 8
    const unsigned bytes = (unsigned)((size_t)d1 * d2 * sizeof(T));
    auto issue = [&](int i) {
      if (tid == 0) {
        const int b = (int)((g3base + i) % 3);
        const unsigned mb = (unsigned)__cvta_generic_to_shared(mbar + b);
        const unsigned dst = (unsigned)__cvta_generic_to_shared(sT + b * SL);
        // the stage's previous contents were read by the generic proxy
        asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(mb), "r"(bytes) : "memory");
        asm volatile(
            "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(dst),
            "l"(Tt + (long long)i * d1 * d2), "r"(bytes), "r"(mb)
            : "memory");
      }
    };
    // bounded wait for slab i; a wait that runs out flags the solve
    auto wait_slab = [&](int i) {
      const unsigned n = g3base + i;
      const unsigned mb = (unsigned)__cvta_generic_to_shared(mbar + n % 3);
      const unsigned par = (n / 3) & 1;
      unsigned ok = 0;
      for (int it = 0; it < (1 << 24) && !ok; ++it)
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(ok)
            : "r"(mb), "r"(par)
            : "memory");
      if (!ok) g3err = 1;
    };
    for (int cb = 0; cb < ncol; cb += 4) {
      const int cn = min(4, ncol - cb);
      for (int e = tid; e < (d0 + d1 + d2p) * 4; e += TFX_THREADS) {
        const int c = e & 3;
        int l = 0, i = e >> 2;
        if (i >= d0) {
          i -= d0;
          l = 1;
          if (i >= d1) {
            i -= d1;
            l = 2;
          }
        }
        sF[e] = (c < cn && i < d[l]) ? Wl[off[l] + (c0 + cb + c) * d[l] + i] : T(0);
        sMM[e] = T(0);
      }
      __syncthreads();  // sF ready; the previous group is done with every stage
      issue(0);
      if (d0 > 1) issue(1);
      // own k-groups q8 and q8 + 8 and their rows of W2
      T creg[2][4][4], acc2[2][4][4];
#pragma unroll
      for (int s2 = 0; s2 < 2; ++s2) {
        const int kg = q8 + 8 * s2;
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          T cc[4] = {T(0), T(0), T(0), T(0)};
          if (kg < nkg) lds4(sC4 + (4 * kg + u) * 4, cc);
#pragma unroll
          for (int c = 0; c < 4; ++c) {
            creg[s2][u][c] = cc[c];
            acc2[s2][u][c] = T(0);
          }
        }
      }
      T bj[2][4], m1[2][4];
#pragma unroll
      for (int h = 0; h < 2; ++h) {
#pragma unroll
        for (int c = 0; c < 4; ++c) {
          bj[h][c] = T(0);
          m1[h][c] = T(0);
        }
        if (rs + 32 * h < d1) lds4(sB4 + (rs + 32 * h) * 4, bj[h]);
      }
      gtick(0);
      for (int i = 0; i < d0; ++i) {
        wait_slab(i);
        __syncthreads();  // every warp is past slab i-1: its stage may be refilled
        gtick(1);
        if (i + 2 < d0) issue(i + 2);
        if (wid == NW - 1 && lane < 4 && i > 0) {  // M0 of slab i-1 from its warp partials
          T sacc = T(0);
          for (int w = 0; w < NW; ++w) sacc += sP0[((i - 1) & 1) * NW * 4 + w * 4 + lane];
          sM0[(i - 1) * 4 + lane] = sacc;
        }
        gtick(2);
        T ai[4];
        lds4(sA4 + i * 4, ai);
        T p0[4] = {T(0), T(0), T(0), T(0)};
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          const int row = rs + 32 * h;
          T y[4] = {T(0), T(0), T(0), T(0)};
          if (row < d1) {
            const T* tr = sT + ((g3base + i) % 3) * SL + row * d2;
            T kr[4];
#pragma unroll
            for (int c = 0; c < 4; ++c) kr[c] = ai[c] * bj[h][c];
#pragma unroll
            for (int s2 = 0; s2 < 2; ++s2) {
              const int kg = q8 + 8 * s2;
              if (kg < nkg) {
                T tv[4];
#pragma unroll
                for (int u = 0; u < 4; ++u) tv[u] = (4 * kg + u < d2) ? tr[4 * kg + u] : T(0);
#pragma unroll
                for (int u = 0; u < 4; ++u)
#pragma unroll
                  for (int c = 0; c < 4; ++c) {
                    y[c] = fma(tv[u], creg[s2][u][c], y[c]);
                    acc2[s2][u][c] = fma(tv[u], kr[c], acc2[s2][u][c]);
                  }
              }
            }
          }
#pragma unroll
          for (int c = 0; c < 4; ++c) {
            y[c] += __shfl_xor_sync(0xffffffffu, y[c], 1);
            y[c] += __shfl_xor_sync(0xffffffffu, y[c], 2);
            y[c] += __shfl_xor_sync(0xffffffffu, y[c], 4);
            m1[h][c] = fma(y[c], ai[c], m1[h][c]);
            if (q8 == 0) p0[c] = fma(y[c], bj[h][c], p0[c]);
          }
        }
#pragma unroll
        for (int c = 0; c < 4; ++c) {
          p0[c] += __shfl_xor_sync(0xffffffffu, p0[c], 8);
          p0[c] += __shfl_xor_sync(0xffffffffu, p0[c], 16);
        }
        if (lane == 0)
#pragma unroll
          for (int c = 0; c < 4; ++c) sP0[(i & 1) * NW * 4 + wid * 4 + c] = p0[c];
        gtick(3);
      }
      __syncthreads();
      if (wid == NW - 1 && lane < 4) {
        T sacc = T(0);
        for (int w = 0; w < NW; ++w) sacc += sP0[((d0 - 1) & 1) * NW * 4 + w * 4 + lane];
        sM0[(d0 - 1) * 4 + lane] = sacc;
      }
      if (q8 == 0)
#pragma unroll
        for (int h = 0; h < 2; ++h)
          if (rs + 32 * h < d1)
#pragma unroll
            for (int c = 0; c < 4; ++c) sM1[(rs + 32 * h) * 4 + c] = m1[h][c];
      // M2: the rows of a warp (lanes with the same q8), then the warps
#pragma unroll
      for (int s2 = 0; s2 < 2; ++s2)
#pragma unroll
        for (int u = 0; u < 4; ++u)
#pragma unroll
          for (int c = 0; c < 4; ++c) {
            T v = acc2[s2][u][c];
            v += __shfl_xor_sync(0xffffffffu, v, 8);
            v += __shfl_xor_sync(0xffffffffu, v, 16);
            const int kg = q8 + 8 * s2;
            if (lane < 8 && kg < nkg) sR2[(wid * d2p + 4 * kg + u) * 4 + c] = v;
          }
      __syncthreads();
      for (int e = tid; e < nkg * 16; e += TFX_THREADS) {
        T v = T(0);
        for (int w = 0; w < NW; ++w) v += sR2[w * d2p * 4 + e];
        sM2[e] = v;
      }
      __syncthreads();
      gtick(4);
      const int sd = d0 + d1 + d2;
      for (int e = tid; e < sd * cn; e += TFX_THREADS) {
        const int c = e / sd;
        int l = 0, i = e - c * sd;
        const T* Ml = sM0;
        if (i >= d0) {
          i -= d0;
          l = 1;
          Ml = sM1;
          if (i >= d1) {
            i -= d1;
            l = 2;
            Ml = sM2;
          }
        }
        const int dl = d[l];
        T wp = T(0);
        const T* p1 = P1l + (size_t)l * R * p1s + p1c + cb + c;
        for (int s2 = 0; s2 < R; ++s2) wp = fma(Wl[off[l] + s2 * dl + i], p1[s2 * p1s], wp);
        grad[off[l] + (c0 + cb + c) * dl + i] = Ml[i * 4 + c] - wp;
      }
      __syncthreads();  // sF and the M slots are rewritten by the next group
      g3base += d0;
      gtick(5);
    }
    // the CG reads every column of the gradient
    tm.sync();
    gtick(7);
  }

  // -------------------------------------------------------------------------
  // Third-order gradient with the SLABS split across the team (every mode <=
  // 64, R <= 64, and the partials below fit in the three slab stages).  CTA q
  // streams its own slabs T[i, :, :], i in [d0 q / n, d0 (q + 1) / n), and forms
  // for every column at once (64 x 64 register tiles, 4 x 4 outputs a thread):
  //   Y = T[i] W2                      M0[i, :] = sum_j Y[j, :] o W1[j, :]
  //   M1 += Y o (1 W0[i, :])           M2 += (T[i]^T W1) o (1 W0[i, :])
  // (the MTTKRP dimension tree, two small products per slab).  M0's rows go to
  // a global scratch vector, the M1 and M2 partials to the CTA's (then idle)
  // slab stages; after a team barrier the CTA owning column c sums the peers'
  // partials of that column through distributed shared memory in rank order
  // and writes grad_l = M_l - W_l P1_l (the negative of GaussNewton.py:401-427).
  // Deterministic: every sum has a fixed order.
  // -------------------------------------------------------------------------
  __device__ bool l3_slab_split_ok() const {
    const int SL = (int)g3_stage(d[1], d[2]);
    return R <= 64 && (d[1] + d[2]) * 64 <= 3 * SL;
  }

  template <bool STAGED>
  __device__ __noinline__ void gradient_l3s() {
    long long gt = gprof ? clock64() : 0;
    auto gtick = [&](int ph) {
      if (gprof) {
        const long long now = clock64();
        gprof[ph] += now - gt;
        gt = now;
      }
    };
    constexpr int NW = TFX_THREADS / 32;
    const int d0 = d[0], d1 = d[1], d2 = d[2];
    char* smb = dyn_smem();
    const T* Wl = STAGED ? (const T*)(smb + cgo.sWf) : W;
    const T* P1l = STAGED ? (const T*)(smb + cgo.sP1o) : P1;
    const int p1s = STAGED ? ((ncol + 3) & ~3) : R;  // P1 column stride
    const int p1c = STAGED ? 0 : c0;    // P1 column offset
    const int SL = (int)g3_stage(d1, d2);
    T* sT = (T*)(smb + g3off);  // 3 stages, then the M1 | M2 partials (64 columns a row)
    T* sM1p = sT;
    T* sM2p = sT + d1 * 64;
    T* sP0x = sT + g3_p0x(d0, d1, d2);  // [2][NW][64] M0 warp partials
    unsigned long long* mbar = (unsigned long long*)(smb + g3off + g3_floats(d0, d1, d2) * sizeof(T));
    const T* W0 = Wl + off[0];
    const T* W1 = Wl + off[1];
    const T* W2 = Wl + off[2];
    T* M0g = z + off[0];  // M0 rows, column-major like the factors (z is free outside the CG)
    const int lane = tid & 31, wid = tid >> 5;
    const int tx = tid & 15, ty = tid >> 4;
    const int i0 = (int)((long long)d0 * tm.rank / tm.size);
    const int ns = (int)((long long)d0 * (tm.rank + 1) / tm.size) - i0;
    const unsigned bytes = (unsigned)((size_t)d1 * d2 * sizeof(T));
    auto issue = [&](int t) {
      if (tid == 0) {
        const int b = (int)((g3base + t) % 3);
        const unsigned mb = (unsigned)__cvta_generic_to_shared(mbar + b);
        const unsigned dst = (unsigned)__cvta_generic_to_shared(sT + b * SL);
        // the stage's previous contents were read (or written) by the generic proxy
        asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(mb), "r"(bytes) : "memory");
        asm volatile(
            "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(dst),
            "l"(Tt + (long long)(i0 + t) * d1 * d2), "r"(bytes), "r"(mb)
            : "memory");
      }
    };
    auto wait_slab = [&](int t) {
      const unsigned n = g3base + t;
      const unsigned mb = (unsigned)__cvta_generic_to_shared(mbar + n % 3);
      const unsigned par = (n / 3) & 1;
      if (!mbar_wait_bounded(mb, par, 1u << 24)) g3err = 1;
    };
    // M0 row of slab t from the warp partials of buffer (t & 1), by 64 threads
    auto m0_row = [&](int t) {
      if (tid < 64 && tid < R) {
        const T* pp = sP0x + (t & 1) * NW * 64 + tid;
        T sacc = pp[0];
#pragma unroll
        for (int w = 1; w < NW; ++w) sacc += pp[w * 64];
        M0g[tid * d0 + i0 + t] = sacc;
      }
    };
    __syncthreads();  // every stage is free (the previous phase ended with barriers)
    if (ns > 0) issue(0);
    if (ns > 1) issue(1);
    T m1a[4][4], m2a[4][4];
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
      for (int v = 0; v < 4; ++v) {
        m1a[u][v] = T(0);
        m2a[u][v] = T(0);
      }
    gtick(0);
    for (int t = 0; t < ns; ++t) {
      wait_slab(t);
      __syncthreads();  // every warp is past slab t-1: its stage may be refilled
      gtick(1);
      if (t + 2 < ns) issue(t + 2);
      if (t > 0) m0_row(t - 1);
      gtick(2);
      const T* tr = sT + ((g3base + t) % 3) * SL;
      const int i = i0 + t;
      T w0[4];
#pragma unroll
      for (int v = 0; v < 4; ++v) {
        const int r = tx + 16 * v;
        w0[v] = r < R ? W0[r * d0 + i] : T(0);
      }
      // Y = T[i] W2 (rows j = ty + 16u, columns r = tx + 16v)
      T y[4][4];
#pragma unroll
      for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int v = 0; v < 4; ++v) y[u][v] = T(0);
#pragma unroll 2
      for (int k = 0; k < d2; ++k) {
        T a[4], b[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) a[u] = (ty + 16 * u < d1) ? tr[(ty + 16 * u) * d2 + k] : T(0);
#pragma unroll
        for (int v = 0; v < 4; ++v) b[v] = (tx + 16 * v < R) ? W2[(tx + 16 * v) * d2 + k] : T(0);
#pragma unroll
        for (int u = 0; u < 4; ++u)
#pragma unroll
          for (int v = 0; v < 4; ++v) y[u][v] = fma(a[u], b[v], y[u][v]);
      }
      // M1 partial and this slab's M0 partial (over the thread's rows)
      T p[4] = {T(0), T(0), T(0), T(0)};
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int j = ty + 16 * u;
#pragma unroll
        for (int v = 0; v < 4; ++v) {
          const int r = tx + 16 * v;
          m1a[u][v] = fma(y[u][v], w0[v], m1a[u][v]);
          if (j < d1 && r < R) p[v] = fma(y[u][v], W1[r * d1 + j], p[v]);
        }
      }
#pragma unroll
      for (int v = 0; v < 4; ++v) p[v] += __shfl_xor_sync(0xffffffffu, p[v], 16);
      if (lane < 16)
#pragma unroll
        for (int v = 0; v < 4; ++v) sP0x[(t & 1) * NW * 64 + wid * 64 + tx + 16 * v] = p[v];
      // M2 partial: (T[i]^T W1)[k, r] W0[i, r] (rows k = ty + 16u)
#pragma unroll
      for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int v = 0; v < 4; ++v) y[u][v] = T(0);
#pragma unroll 2
      for (int j = 0; j < d1; ++j) {
        T a[4], b[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) a[u] = (ty + 16 * u < d2) ? tr[j * d2 + ty + 16 * u] : T(0);
#pragma unroll
        for (int v = 0; v < 4; ++v) b[v] = (tx + 16 * v < R) ? W1[(tx + 16 * v) * d1 + j] : T(0);
#pragma unroll
        for (int u = 0; u < 4; ++u)
#pragma unroll
          for (int v = 0; v < 4; ++v) y[u][v] = fma(a[u], b[v], y[u][v]);
      }
#pragma unroll
      for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int v = 0; v < 4; ++v) m2a[u][v] = fma(y[u][v], w0[v], m2a[u][v]);
      gtick(3);
    }
    __syncthreads();  // every slab consumed; the stages are idle (every copy was waited for)
    if (ns > 0) m0_row(ns - 1);
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
      for (int v = 0; v < 4; ++v) {
        const int r = tx + 16 * v, row = ty + 16 * u;
        if (r < R) {
          if (row < d1) sM1p[row * 64 + r] = m1a[u][v];
          if (row < d2) sM2p[row * 64 + r] = m2a[u][v];
        }
      }
    g3base += ns;
    tm.sync();  // partials and M0 rows visible to the team
    gtick(4);
    const int sd = d0 + d1 + d2;
    for (int e = tid; e < sd * ncol; e += TFX_THREADS) {
      const int c = e / sd;
      int l = 0, i = e - c * sd;
      if (i >= d0) {
        i -= d0;
        l = 1;
        if (i >= d1) {
          i -= d1;
          l = 2;
        }
      }
      const int col = c0 + c;
      T m;
      if (l == 0) {
        m = __ldcg(M0g + col * d0 + i);
      } else {
        const T* part = (l == 1 ? sM1p : sM2p) + i * 64 + col;
        T pv[TFX_MAX_TEAM];
#pragma unroll
        for (int q = 0; q < TFX_MAX_TEAM; ++q) pv[q] = q < tm.size ? *tm.peer(part, q) : T(0);
        m = pv[0];
#pragma unroll
        for (int q = 1; q < TFX_MAX_TEAM; ++q)
          if (q < tm.size) m += pv[q];
      }
      const int dl = d[l];
      T wp = T(0);
      const T* p1 = P1l + (size_t)l * R * p1s + p1c + c;
      for (int s2 = 0; s2 < R; ++s2) wp = fma(Wl[off[l] + s2 * dl + i], p1[s2 * p1s], wp);
      grad[off[l] + col * dl + i] = m - wp;
    }
    gtick(5);
    // the peers are done reading this CTA's partials; the CG reads every column
    tm.sync();
    gtick(7);
  }

  // the gradient by the fastest form that applies
  __device__ void gradient_any() {
    if (sG3 && l3_slab_split_ok()) {
      if (stage)
        gradient_l3s<true>();
      else
        gradient_l3s<false>();
    } else if (sG3) {
      if (stage)
        gradient_l3<true>();
      else
        gradient_l3<false>();
    } else {
      gradient();
    }
  }

  // -------------------------------------------------------------------------
  // Gradient (GaussNewton.py:401-427): grad_l = T_(l) KR_l - W_l P1_l, the
  // negative of the reference's g.  Split-K over the team, partial d_l x R
  // tiles summed through distributed shared memory by the CTA owning the column.
  // -------------------------------------------------------------------------
  __device__ void gradient() {
    const int tx = tid & 15, ty = tid >> 4;
    for (int l = 0; l < L; ++l) {
      const long long Kl = N / d[l];
      const long long kb = Kl * tm.rank / tm.size, ke = Kl * (tm.rank + 1) / tm.size;
      for (int m0 = 0; m0 < d[l]; m0 += TL::BM) {
        for (int n0 = 0; n0 < R; n0 += TL::BN) {
          T acc[TS][TS];
          tile_zero<T, TS, TS>(acc);
          for (long long k0 = kb; k0 < ke; k0 += TFX_BK) {
            const int kc = (int)min((long long)TFX_BK, ke - k0);
            if (tid < kc) {
              long long k = k0 + tid, base = 0;
              for (int m = L - 1; m >= 0; --m) {
                if (m == l) continue;
                const long long im = k % d[m];
                k /= d[m];
                base += im * st[m];
                sIdx[tid * L + m] = (int)im;
              }
              sBase[tid] = base;
            }
            __syncthreads();
            // all of this thread's tensor loads are issued before any shared
            // store (read-only path: the tensor is constant during the solve)
            constexpr int NPT = (TFX_BK * TL::BM + TFX_THREADS - 1) / TFX_THREADS;
            T av[NPT];
            const long long stl = st[l];
            const int dl = d[l];
#pragma unroll
            for (int j = 0; j < NPT; ++j) {
              const int e = tid + j * TFX_THREADS;
              int kk, mm;
              if (l == L - 1) {
                kk = e / TL::BM;
                mm = e - kk * TL::BM;
              } else {
                mm = e / TFX_BK;
                kk = e - mm * TFX_BK;
              }
              av[j] = (e < TFX_BK * TL::BM && kk < kc && m0 + mm < dl) ? __ldg(Tt + sBase[kk] + (long long)(m0 + mm) * stl)
                                                                     : T(0);
            }
#pragma unroll
            for (int j = 0; j < NPT; ++j) {
              const int e = tid + j * TFX_THREADS;
              if (e < TFX_BK * TL::BM) {
                int kk, mm;
                if (l == L - 1) {
                  kk = e / TL::BM;
                  mm = e - kk * TL::BM;
                } else {
                  mm = e / TFX_BK;
                  kk = e - mm * TFX_BK;
                }
                sA[kk * TL::LDA + mm] = av[j];
              }
            }
            for (int e = tid; e < TFX_BK * TL::BN; e += TFX_THREADS) {
              const int kk = e / TL::BN, nn = e - kk * TL::BN;
              T v = T(0);
              if (kk < kc && n0 + nn < R) {
                v = T(1);
                for (int m = L - 1; m >= 0; --m)
                  if (m != l) v *= Wr[off[m] + (n0 + nn) * d[m] + sIdx[kk * L + m]];
              }
              sB[kk * TL::LDB + nn] = v;
            }
            __syncthreads();
            tile_fma<T, TS, TS>(sA, sB, acc, kc);
            __syncthreads();
          }
#pragma unroll
          for (int u = 0; u < TS; ++u)
#pragma unroll
            for (int v = 0; v < TS; ++v) {
              const int m = m0 + ty + 16 * u, n = n0 + tx + 16 * v;
              if (m < d[l] && n < R) sPart[m * R + n] = acc[u][v];
            }
        }
      }
      tm.sync();
      // reduce own columns and subtract W_l P1_l
      for (int e = tid; e < d[l] * ncol; e += TFX_THREADS) {
        const int c = e / d[l], i = e - c * d[l], b = c0 + c;
        // issue every peer's load before summing (independent remote loads)
        T pv[TFX_MAX_TEAM];
#pragma unroll
        for (int rr = 0; rr < TFX_MAX_TEAM; ++rr) pv[rr] = rr < tm.size ? tm.peer(sPart, rr)[i * R + b] : T(0);
        T mk = T(0);
#pragma unroll
        for (int rr = 0; rr < TFX_MAX_TEAM; ++rr)
          if (rr < tm.size) mk += pv[rr];
        T wp = T(0);
        for (int s = 0; s < R; ++s) wp = fma(Wr[off[l] + s * d[l] + i], P1at(l, s, c), wp);
        grad[off[l] + b * d[l] + i] = mk - wp;
      }
      tm.sync();
    }
  }

  // CG inner solve (see cg_team above)
  CgOffsets cgo;
  long long* cprof;  // optional CG sub-phase timers (rank 0, thread 0)
  long long* gprof;  // optional third-order gradient sub-phase timers
  __device__ int cg(int budget, double& rn_out) {
    if (stage)
      return cg_team<T, true>(tm, L, R, nx, ncol, c0, cgo, grad, jtj, y, r, P, Q, z, W, P1, P2, budget, op.cg_tol,
                              rn_out, flipw, cprof);
    return cg_team<T, false>(tm, L, R, nx, ncol, c0, cgo, grad, jtj, y, r, P, Q, z, W, P1, P2, budget, op.cg_tol,
                             rn_out, flipw, cprof);
  }

  // Column balancing of x into the factor buffer (Conversion.py:361-387),
  // then transform (Conversion.py:412-444).  Owned columns only, except the
  // factors_norm rescaling which needs a team-wide norm per mode.
  __device__ void to_factors(const T* src, T* dst, bool eq) {
    if (aliased) {
      // The reference's x2cpd writes every block of x into the one shared
      // array, which ends holding the LAST block; balancing then scales it once
      // per mode (all its column norms are equal), and transform's in-place sum
      // adds the array to itself L - 1 times before dividing by L
      // (Conversion.py:21-49, 361-387, 432-437).
      const int dl = d[L - 1];
      if (eq) {
        const int lane = tid & 31, wid = tid >> 5;
        for (int c = wid; c < ncol; c += TFX_THREADS / 32) {
          const T* col = src + off[L - 1] + (c0 + c) * dl;
          Acc<T> s;
          for (int i = lane; i < dl; i += 32) s.fma_(col[i], col[i]);
          s.warp_reduce();
          if (lane == 0) {
            const double nr = sqrt(s.value());
            double prod = 1.0;
            for (int m = 0; m < L; ++m) prod *= nr;
            sScale[c] = prod != 0.0 ? (T)(pow(prod, 1.0 / (double)L) / nr) : T(1);
          }
        }
        __syncthreads();
      }
      for_own([&](int e, int l, int c) {
        const int i = e - off[l] - (c0 + c) * d[l];
        T v = src[off[L - 1] + (c0 + c) * dl + i];
        if (eq)
          for (int m = 0; m < L; ++m) v = sScale[c] * v;
        if (op.symm) {
          for (int m = 1; m < L; ++m) v = v + v;
          v = v / (T)L;
        }
        dst[e] = v;
      });
      __syncthreads();
    } else if (eq) {
      const int lane = tid & 31, wid = tid >> 5;
      for (int p = wid; p < L * ncol; p += TFX_THREADS / 32) {
        const int l = p / ncol, c = p - l * ncol;
        const T* col = src + off[l] + (c0 + c) * d[l];
        Acc<T> s;
        for (int i = lane; i < d[l]; i += 32) s.fma_(col[i], col[i]);
        s.warp_reduce();
        if (lane == 0) sNorm[p] = sqrt(s.value());
      }
      __syncthreads();
      // one balancing factor per (mode, column): (prod_m n_m)^(1/L) / n_l
      for (int c = tid; c < ncol; c += TFX_THREADS) {
        double prod = 1.0;
        for (int m = 0; m < L; ++m) prod *= sNorm[m * ncol + c];
        if (prod != 0.0) {
          const double num = pow(prod, 1.0 / (double)L);
          for (int m = 0; m < L; ++m) sScale[m * ncol + c] = (T)(num / sNorm[m * ncol + c]);
        } else {
          for (int m = 0; m < L; ++m) sScale[m * ncol + c] = T(1);
        }
      }
      __syncthreads();
      for_own([&](int e, int l, int c) { dst[e] = sScale[l * ncol + c] * src[e]; });
    } else {
      for_own([&](int e, int l, int c) { dst[e] = src[e]; });
    }
    __syncthreads();
    if (op.symm && !aliased) {
      // all dims equal: W_0 = mean_l W_l, then every mode copies W_0
      const int dd = d[0];
      for (int e = tid; e < ncol * dd; e += TFX_THREADS) {
        const int c = e / dd, i = e - c * dd;
        T s = dst[off[0] + (c0 + c) * dd + i];
        for (int l = 1; l < L; ++l) s += dst[off[l] + (c0 + c) * dd + i];
        s = s / (T)L;
        for (int l = 0; l < L; ++l) dst[off[l] + (c0 + c) * dd + i] = s;
      }
      __syncthreads();
    }
    if (op.factors_norm > 0.0) {
      double v[TFX_MAX_ORDER];
#pragma unroll
      for (int l = 0; l < TFX_MAX_ORDER; ++l) v[l] = 0.0;
      for_own([&](int e, int l, int c) {
        const double t = (double)dst[e];
        for (int m = 0; m < TFX_MAX_ORDER; ++m)
          if (m == l) v[m] += t * t;
      });
      team_sum<TFX_MAX_ORDER>(tm, v, rs12, flip12);
      for_own([&](int e, int l, int c) {
        double nl = 0.0;
        for (int m = 0; m < TFX_MAX_ORDER; ++m)
          if (m == l) nl = v[m];
        dst[e] = (T)(op.factors_norm * (1.0 / sqrt(nl)) * (double)dst[e]);
      });
      __syncthreads();
    }
    // symmetrising leaves one array; the fixed-norm rescaling gives each mode its own
    aliased = (op.symm || aliased) && !(op.factors_norm > 0.0);
  }

  // ||T - [[W]]|| / ||T|| (Conversion.py:117-141 + Critical.py:14-22), fused:
  // the model tile is built in registers and never stored.
  // -------------------------------------------------------------------------
  // Third-order relative error |T - [[W]]| / |T| (Auxiliar.py:131-158 via
  // GaussNewton.py:197): the team splits the slabs T[i, :, :], which stream
  // through the gradient's stage ring; a thread forms a 4 x 4 block of
  //   X[j, k] = sum_r W0[i, r] W1[j, r] W2[k, r]
  // from W1 and W2 staged with rows padded to four, and sums (T - X)^2 in
  // float-float.  Same conditions as the third-order gradient.
  // -------------------------------------------------------------------------
  __device__ double rel_error_l3(const T* Wf) {
    const int d0 = d[0], d1 = d[1], d2 = d[2];
    const int d1p = (d1 + 3) & ~3, d2p = (d2 + 3) & ~3;
    char* smb = dyn_smem();
    T* sBt = (T*)(smb + e3off);  // R x d1p
    T* sCt = sBt + R * d1p;      // R x d2p
    const int SL = (int)g3_stage(d1, d2);
    T* sT = (T*)(smb + g3off);
    unsigned long long* mbar = (unsigned long long*)(smb + g3off + g3_floats(d0, d1, d2) * sizeof(T));
    for (int e = tid; e < R * d1p; e += TFX_THREADS) {
      const int r = e / d1p, j = e - r * d1p;
      sBt[e] = j < d1 ? Wf[off[1] + r * d1 + j] : T(0);
    }
    for (int e = tid; e < R * d2p; e += TFX_THREADS) {
      const int r = e / d2p, k = e - r * d2p;
      sCt[e] = k < d2 ? Wf[off[2] + r * d2 + k] : T(0);
    }
    const int first = tm.rank, step = tm.size;
    const int nmy = first < d0 ? (d0 - 1 - first) / step + 1 : 0;
    const unsigned bytes = (unsigned)((size_t)d1 * d2 * sizeof(T));
    auto issue = [&](int t) {
      if (tid == 0) {
        const int b = (int)((g3base + t) % 3);
        const unsigned mb = (unsigned)__cvta_generic_to_shared(mbar + b);
        const unsigned dst = (unsigned)__cvta_generic_to_shared(sT + b * SL);
        asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(mb), "r"(bytes) : "memory");
        asm volatile(
            "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(dst),
            "l"(Tt + (long long)(first + t * step) * d1 * d2), "r"(bytes), "r"(mb)
            : "memory");
      }
    };
    __syncthreads();  // staged W1, W2; every stage is free (the gradient ended with barriers)
    if (nmy > 0) issue(0);
    if (nmy > 1) issue(1);
    const int nk4 = d2p >> 2, nj4 = d1p >> 2;
    const int j4 = tid / nk4, k4 = tid - j4 * nk4;
    const bool active = tid < nj4 * nk4;  // <= 16 x 16
    Acc<T> acc;
    for (int t = 0; t < nmy; ++t) {
      const unsigned n = g3base + t;
      {
        const unsigned mb = (unsigned)__cvta_generic_to_shared(mbar + n % 3);
        const unsigned par = (n / 3) & 1;
        unsigned ok = 0;
        for (int it = 0; it < (1 << 24) && !ok; ++it)
          asm volatile(
              "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
              : "=r"(ok)
              : "r"(mb), "r"(par)
              : "memory");
        if (!ok) g3err = 1;
      }
      __syncthreads();  // every warp is past slab t-1: its stage may be refilled
      if (t + 2 < nmy) issue(t + 2);
      if (active) {
        const int i = first + t * step;
        T x[4][4];
#pragma unroll
        for (int u = 0; u < 4; ++u)
#pragma unroll
          for (int v = 0; v < 4; ++v) x[u][v] = T(0);
        const T* a = Wf + off[0] + i;
#pragma unroll 2
        for (int r = 0; r < R; ++r) {
          const T ai = a[r * d0];
          T b[4], c[4];
          lds4(sBt + r * d1p + 4 * j4, b);
          lds4(sCt + r * d2p + 4 * k4, c);
#pragma unroll
          for (int u = 0; u < 4; ++u) {
            const T bu = ai * b[u];
#pragma unroll
            for (int v = 0; v < 4; ++v) x[u][v] = fma(bu, c[v], x[u][v]);
          }
        }
        const T* slab = sT + (n % 3) * SL;
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const int j = 4 * j4 + u;
#pragma unroll
          for (int v = 0; v < 4; ++v) {
            const int k = 4 * k4 + v;
            if (j < d1 && k < d2) {
              const T df = slab[j * d2 + k] - x[u][v];
              acc.fma_(df, df);
            }
          }
        }
      }
    }
    g3base += nmy;
    Acc<T> v1[1] = {acc}, tot[1];
    team_sum_push<1>(tm, v1, tot, (PushSlots<1>*)(smb + cgo.wsl), flipw);
    // one thread forms the double result (FP64 is slow on GB300), the CTA reads it
    double* res = (double*)(smb + e3off);
    __syncthreads();  // the staged factors are no longer read
    if (tid == 0) *res = sqrt(acc_val_d(tot[0])) / Tsize;
    __syncthreads();
    const double out = *res;
    __syncthreads();  // the slot is scratch again
    return out;
  }

  __device__ double rel_error(const T* Wf) {
    const int tx = tid & 15, ty = tid >> 4;
    const long long Q0 = N / d[0];
    const int tm_ = (d[0] + TL::BM - 1) / TL::BM;
    const long long tn_ = (Q0 + TL::BN - 1) / TL::BN;
    const long long ntiles = (long long)tm_ * tn_;
    double part = 0.0;
    for (long long t = tm.rank; t < ntiles; t += tm.size) {
      const int m0 = (int)(t % tm_) * TL::BM;
      const long long q0 = (t / tm_) * TL::BN;
      if (tid < TL::BN) {
        long long q = q0 + tid;
        if (q < Q0) {
          for (int m = L - 1; m >= 1; --m) {
            sIdx[tid * L + m] = (int)(q % d[m]);
            q /= d[m];
          }
        }
      }
      __syncthreads();
      T acc[TS][TS];
      tile_zero<T, TS, TS>(acc);
      for (int k0 = 0; k0 < R; k0 += TFX_BK) {
        const int kc = min(TFX_BK, R - k0);
        for (int e = tid; e < TFX_BK * TL::BM; e += TFX_THREADS) {
          const int kk = e / TL::BM, mm = e - kk * TL::BM;
          sA[kk * TL::LDA + mm] = (kk < kc && m0 + mm < d[0]) ? Wf[off[0] + (k0 + kk) * d[0] + m0 + mm] : T(0);
        }
        for (int e = tid; e < TFX_BK * TL::BN; e += TFX_THREADS) {
          const int kk = e / TL::BN, nn = e - kk * TL::BN;
          T v = T(0);
          if (kk < kc && q0 + nn < Q0) {
            v = T(1);
            for (int m = L - 1; m >= 1; --m) v *= Wf[off[m] + (k0 + kk) * d[m] + sIdx[nn * L + m]];
          }
          sB[kk * TL::LDB + nn] = v;
        }
        __syncthreads();
        tile_fma<T, TS, TS>(sA, sB, acc, kc);
        __syncthreads();
      }
      T ps = T(0);
#pragma unroll
      for (int u = 0; u < TS; ++u)
#pragma unroll
        for (int v = 0; v < TS; ++v) {
          const int m = m0 + ty + 16 * u;
          const long long q = q0 + tx + 16 * v;
          if (m < d[0] && q < Q0) {
            const T df = __ldg(Tt + (long long)m * Q0 + q) - acc[u][v];
            ps = fma(df, df, ps);
          }
        }
      part += (double)ps;
    }
    double v4[4] = {part, 0.0, 0.0, 0.0};
    team_sum<4>(tm, v4, rs4, flip4);
    return sqrt(v4[0]) / Tsize;
  }

  // -------------------------------------------------------------------------
  // Dogleg fallback (GaussNewton.py:713-795).  On entry xn holds x_old + y and
  // W the rejected (balanced) factors; on exit xn/y/W hold the best trial.
  // -------------------------------------------------------------------------
  __device__ double dogleg(double error) {
    // x = x - y  (the reference reverts in floating point)
    for_own([&](int e, int l, int c) {
      const T xv = xn[e] - y[e];
      xn[e] = xv;
      bx[e] = xv;
      by[e] = y[e];
      bW[e] = W[e];
    });
    double g2[4] = {0.0, 0.0, 0.0, 0.0};
    for_own([&](int e, int l, int c) {
      g2[0] += (double)grad[e] * (double)grad[e];
      g2[1] += (double)grad[e] * (double)jtj[e];
    });
    team_sum<4>(tm, g2, rs4, flip4);
    const double gnorm = sqrt(g2[0]);
    const double alpha = (gnorm * gnorm) / g2[1];
    double best_error = error, gain = 1.0, delta = 1.0;
    int count = 0;
    while (gain > 0.0) {
      const double old_error = error;
      // dogleg(y, grad, JT_J_grad, delta)
      double c[4] = {0.0, 0.0, 0.0, 0.0};
      for_own([&](int e, int l, int cc) {
        const double ysd = alpha * (double)grad[e];
        const double dy = (double)y[e] - ysd;
        c[0] += dy * ysd;
        c[1] += dy * dy;
        c[2] += (double)y[e] * (double)y[e];
      });
      team_sum<4>(tm, c, rs4, flip4);
      const double c1 = fabs(alpha) * gnorm;
      const double c2 = c[0], c3 = c[1];
      const double c4 = delta * delta - c1 * c1;
      const double mm = c2 * c2 + c3 * c4;
      int mode;
      double coef = 0.0;
      if (sqrt(c[2]) < delta) {
        mode = 0;
      } else if (c1 >= delta) {
        mode = 1;
        coef = delta / c1;
      } else if (mm < 0.0) {
        mode = 0;
      } else {
        const double c5 = sqrt(mm);
        coef = (c2 <= 0.0) ? (-c2 + c5) / c3 : c4 / (c2 + c5);
        mode = 2;
      }
      // y <- y_dl; x <- x + y; W <- x (no balancing)
      double s[4] = {0.0, 0.0, 0.0, 0.0};
      for_own([&](int e, int l, int cc) {
        double yn;
        if (mode == 0) {
          yn = (double)y[e];
        } else if (mode == 1) {
          yn = coef * (alpha * (double)grad[e]);
        } else {
          const double ysd = alpha * (double)grad[e];
          yn = ysd + coef * ((double)y[e] - ysd);
        }
        const T ty_ = (T)yn;
        y[e] = ty_;
        const T xo = xn[e];
        const T xv = xo + ty_;
        xn[e] = xv;
        const double dx = (double)xv - (double)xo;
        s[0] += dx * ((double)grad[e] + damp * dx);
        s[1] += dx * dx;
      });
      __syncthreads();
      to_factors(xn, W, false);
      tm.sync();
      stage_W();
      team_sum<4>(tm, s, rs4, flip4);
      error = sG3 ? rel_error_l3(Wr) : rel_error(Wr);
      const double num = (Tsize * Tsize) * (old_error * old_error - error * error);
      if (s[0] != 0.0) {
        gain = num / s[0];
      } else if (num != 0.0) {
        gain = (num > 0.0 ? 1.0 : -1.0) * INFINITY;
      } else {
        gain = -INFINITY;
      }
      if (error < old_error) {
        for_own([&](int e, int l, int cc) {
          bx[e] = xn[e];
          by[e] = y[e];
          bW[e] = W[e];
        });
        best_error = error;
      }
      const double step = sqrt(s[1]);
      if (gain > 0.75) {
        delta = fmax(delta, 2.0 * step);
      } else {
        const double sg = 0.25 / (1.0 + exp(-14.0 * (gain - 0.75))) + 0.75;
        delta = fmin(sg * delta, delta);
      }
      ++count;
      if (count > 10) break;
    }
    __syncthreads();
    for_own([&](int e, int l, int cc) {
      xn[e] = bx[e];
      y[e] = by[e];
      W[e] = bW[e];
    });
    __syncthreads();
    tm.sync();
    stage_W();
    return best_error;
  }
};

// Binds an engine to one problem: shape tables, workspace and shared-memory
// pointers, the third-order slab barriers.  Used by the solve and by the
// standalone gradient / J^T J v entry point.
template <class T, int TS>
__device__ __forceinline__ void engine_setup(Engine<T, TS>& E, const tfx_dgn_problem& pb, const tfx_dgn_options& op,
                                             Team tm, char* smem, const SmemPlan& sp) {
  E.d = (int*)(smem + sp.misc + 64);
  E.off = E.d + TFX_MAX_ORDER;
  E.st = (long long*)(smem + sp.misc + 64 + 4 * TFX_MAX_ORDER * 8);
  E.tm = tm;
  E.tid = threadIdx.x;
  E.op = op;
  E.L = pb.L;
  E.R = pb.R;
  int sumd = 0;
  E.N = 1;
  E.maxd = 0;
  for (int l = 0; l < E.L; ++l) {
    if (threadIdx.x == 0) {
      E.d[l] = pb.dims[l];
      E.off[l] = E.R * sumd;
    }
    sumd += pb.dims[l];
    E.N *= pb.dims[l];
    E.maxd = max(E.maxd, pb.dims[l]);
  }
  if (threadIdx.x == 0) {
    E.off[E.L] = E.R * sumd;
    long long s = 1;
    for (int l = E.L - 1; l >= 0; --l) {
      E.st[l] = s;
      s *= pb.dims[l];
    }
  }
  E.nx = E.R * sumd;
  __syncthreads();
  E.c0 = (int)((long long)E.R * tm.rank / tm.size);
  E.c1 = (int)((long long)E.R * (tm.rank + 1) / tm.size);
  E.ncol = E.c1 - E.c0;
  E.Tt = (const T*)pb.tensor;
  const WsLayout w = ws_layout(E.L, E.R, E.nx, sizeof(T));
  char* base = (char*)pb.work;
  E.xc = (T*)(base + w.xc);
  E.xn = (T*)(base + w.xn);
  E.W = (T*)(base + w.W);
  E.grad = (T*)(base + w.grad);
  E.jtj = (T*)(base + w.jtj);
  E.y = (T*)(base + w.y);
  E.r = (T*)(base + w.r);
  E.P = (T*)(base + w.P);
  E.Q = (T*)(base + w.Q);
  E.z = (T*)(base + w.z);
  E.bx = (T*)(base + w.bx);
  E.by = (T*)(base + w.by);
  E.bW = (T*)(base + w.bW);
  E.P1 = (T*)(base + w.P1);
  E.P2 = (T*)(base + w.P2);
  E.G = (double*)(base + w.G);
  E.sA = (T*)(smem + sp.sA);
  E.sB = (T*)(smem + sp.sB);
  E.sPart = (T*)(smem + sp.sPart);
  E.sAk = (T*)(smem + sp.sAk);
  E.sY = (T*)(smem + sp.sY);
  E.sM = (T*)(smem + sp.sM);
  E.sDG = (T*)(smem + sp.sDG);
  E.sGam = (double*)(smem + sp.sGam);
  E.sNorm = (double*)(smem + sp.sNorm);
  E.sBase = (long long*)(smem + sp.sBase);
  E.sIdx = (int*)(smem + sp.sIdx);
  E.rs4 = (RedScratch<4>*)(smem + sp.rs4);
  E.rs12 = (RedScratch<TFX_MAX_ORDER>*)(smem + sp.rs12);
  E.sMisc = (double*)(smem + sp.misc);
  E.stage = sp.stage;
  E.sQf = (T*)(smem + sp.sQf);
  E.sWf = (T*)(smem + sp.sWf);
  E.sP1o = (T*)(smem + sp.sP1o);
  E.sP2o = (T*)(smem + sp.sP2o);
  E.Wr = E.W;
  E.cgo.d = sp.misc + 64;
  E.cgo.sQf = sp.sQf;
  E.cgo.sWf = sp.sWf;
  E.cgo.sP1o = sp.sP1o;
  E.cgo.sP2o = sp.sP2o;
  E.cgo.sAk = sp.sAk;
  E.cgo.sY = sp.sY;
  E.cgo.sM = sp.sM;
  E.cgo.sDG = sp.sDG;
  E.cgo.rs4 = sp.rs4;
  E.cgo.rs1 = sp.rs1;
  E.cgo.sVec = sp.sVec;
  E.cgo.wsl = sp.wsl;
  E.rs1b = (RedScratch<1>*)(smem + sp.rs1b);
  E.sScale = (T*)(smem + sp.sScale);
  E.aliased = op.aliased != 0;
  // third-order gradient path: every mode <= 64 (the plan), 16-byte slabs
  E.sG3 = (sp.sG3 && pb.L == 3 && ((size_t)pb.dims[1] * pb.dims[2]) % 4 == 0 &&
           (((unsigned long long)pb.tensor) & 15) == 0)
              ? (T*)(smem + sp.sG3)
              : nullptr;
  E.g3off = sp.sG3;
  E.e3off = sp.sE3;
  E.g3base = 0;
  E.g3err = 0;
  if (E.sG3 && threadIdx.x == 0) {
    unsigned long long* mb =
        (unsigned long long*)(smem + sp.sG3 + g3_floats(pb.dims[0], pb.dims[1], pb.dims[2]) * sizeof(T));
    for (int b = 0; b < 3; ++b)
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"((unsigned)__cvta_generic_to_shared(mb + b)));
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  __syncthreads();
  E.flip1 = 0;
  E.flip1b = 0;
  E.flip4 = 0;
  E.flip12 = 0;
  E.flipw = 0;
}

template <class T, int TS>
__device__ void solve_problem(const tfx_dgn_problem& pb, const tfx_dgn_options& op, Team tm, char* smem,
                              const SmemPlan& sp) {
  Engine<T, TS> E;
  engine_setup<T, TS>(E, pb, op, tm, smem, sp);

  // error / improvement history: every CTA keeps its own copy in shared
  // memory so that the stop tests never depend on another SM's writes
  double* hErr = (double*)(smem + sp.hist);
  double* hImp = hErr + op.maxiter;
  const T* x0 = (const T*)pb.x;
  T* best = (T*)pb.best;
  const int maxiter = op.maxiter;
  double* errors = pb.stats;
  double* step_sizes = pb.stats + maxiter;
  double* improv = pb.stats + 2 * maxiter;
  double* gradients = pb.stats + 3 * maxiter;

  // initial state: x (mutable copy), W = factors as given, best = factors
  E.for_own([&](int e, int l, int c) {
    const T v = x0[e];
    E.xc[e] = v;
    E.W[e] = v;
    best[e] = v;
  });
  double meanabs;
  E.tensor_norms(E.Tsize, meanabs);
  const double Tsize = E.Tsize;
  E.damp = op.use_damp_sched ? pb.damp_sched[0] : op.init_damp * meanabs;
  double tol = op.tol, tol_step = op.tol_step, tol_improv = op.tol_improv, tol_grad = op.tol_grad;
  if ((long long)E.nx <= 100) {
    tol = tol_step = tol_improv = tol_grad = 0.0;
  }
  const int cnst = 1 + maxiter / 10;
  double error = 1.0, best_error = INFINITY;
  int stop = 5, it = 0, n_dogleg = 0;
  long long matvecs = 0;
  E.tm.sync();
  E.stage_W();

  // optional phase timers (rank 0, thread 0): SM clock cycles per phase
  long long* prof = (E.tm.rank == 0 && threadIdx.x == 0) ? pb.prof : nullptr;
  E.cprof = prof ? prof + 8 : nullptr;
  E.gprof = prof ? prof + 16 : nullptr;
  long long tclk = clock64(), t_start = tclk;
  auto tick = [&](int ph) {
    if (prof) {
      const long long now = clock64();
      prof[ph] += now - tclk;
      tclk = now;
    }
  };
  for (it = 0; it < maxiter; ++it) {
    const double old_error = error;
    tick(6);
    E.gramians_and_precond();
    tick(0);
    E.gradient_any();
    tick(1);
    double rn;
    const int itn = E.cg(pb.budgets[it], rn);
    matvecs += itn + 1;  // CG products plus J^T J grad
    tick(2);
    // y <- M y ; xn <- x + y ; W <- balanced(xn)
    E.for_own([&](int e, int l, int c) {
      const T yy = E.sM[l * E.ncol + c] * E.y[e];
      E.y[e] = yy;
      E.xn[e] = E.xc[e] + yy;
    });
    __syncthreads();
    E.to_factors(E.xn, E.W, true);
    if (op.fixed > 0 && E.L == 3) {
      // bicpd: the fixed factor is put back after every step (GaussNewton.py:
      // 293-297); the dogleg trials do not (GaussNewton.py:737-742)
      const int fm = op.fixed - 1;
      E.for_own([&](int e, int l, int c) {
        if (l == fm) E.W[e] = x0[e];
      });
      __syncthreads();
    }
    E.tm.sync();
    E.stage_W();
    tick(3);
    error = E.sG3 ? E.rel_error_l3(E.Wr) : E.rel_error(E.Wr);
    tick(4);
    if (it > 3 && error > op.tol_jump * old_error) {
      error = E.dogleg(error);
      ++n_dogleg;
    }
    tick(5);
    // gain ratio, step size, gradient norm (x_new - x_old with the final x)
    Acc<T> va[4];
    MaxAcc<T> ga[1];
    double v[4], gm[1];
    const T dmp = (T)E.damp;
    E.for_own([&](int e, int l, int c) {
      const T dx = E.xn[e] - E.xc[e];
      va[0].fma_(dx, E.grad[e] + dmp * dx);
      va[1].fma_(dx, dx);
      va[2].fma_(E.xc[e], E.xc[e]);
      ga[0].v = fmax(ga[0].v, fabs(E.grad[e]));
    });
    team_sum_acc<4, T>(E.tm, va, v, E.rs4, E.flip4);
    team_reduce_acc<1, true>(E.tm, ga, gm, E.rs1b, E.flip1b);
    const double num = (Tsize * Tsize) * (old_error * old_error - error * error);
    double gain;
    if (v[0] != 0.0) {
      gain = num / v[0];
    } else if (num != 0.0) {
      gain = (num > 0.0 ? 1.0 : -1.0) * INFINITY;
    } else {
      gain = -INFINITY;
    }
    if (op.use_damp_sched) {
      E.damp = pb.damp_sched[it];
    } else if (gain < 0.25) {
      E.damp = 3.0 * E.damp;
    } else if (gain > 0.75) {
      E.damp = E.damp / 3.0;
    }
    if (error < best_error) {
      best_error = error;
      E.for_own([&](int e, int l, int c) { best[e] = E.W[e]; });
    }
    const double ssz = sqrt(v[1]) / sqrt(v[2]);
    const double imp = (it == 0) ? error : fabs(error - old_error);
    __syncthreads();
    if (threadIdx.x == 0) {
      hErr[it] = error;
      hImp[it] = imp;
      if (E.tm.rank == 0) {
        errors[it] = error;
        step_sizes[it] = ssz;
        improv[it] = imp;
        gradients[it] = gm[0];
      }
    }
    __syncthreads();
    // swap x buffers: xc <- xn
    {
      T* t = E.xc;
      E.xc = E.xn;
      E.xn = t;
    }
    E.tm.sync();
    if (it > 1) {
      if (error < tol) { stop = 0; break; }
      if (ssz < tol_step) { stop = 1; break; }
      if (imp < tol_improv) { stop = 2; break; }
      if (gm[0] < tol_grad) { stop = 3; break; }
      if (it > 2 * cnst && it % cnst == 0) {
        double m1 = 0.0, m2 = 0.0, m3 = 0.0;
        for (int j = it - 2 * cnst; j < it - cnst; ++j) m1 += hErr[j];
        for (int j = it - cnst; j < it; ++j) m2 += hErr[j];
        for (int j = it - cnst; j < it; ++j) m3 += hImp[j];
        m1 /= cnst;
        m2 /= cnst;
        m3 /= cnst;
        if (m1 - m2 <= tol_improv) { stop = 4; break; }
        if (m3 < 1e-3 * m2) { stop = 7; break; }
      }
      if (error > fmax(1.0, Tsize * Tsize) / (1e-16 + tol)) { stop = 6; break; }
    }
  }
  const int iters = (it < maxiter) ? it + 1 : maxiter;
  tick(6);
  if (prof) prof[7] += clock64() - t_start;
  if (E.tm.rank == 0 && threadIdx.x == 0) pb.result[2] = TFX_OK;
  E.tm.sync();
  // any CTA whose bounded slab wait ran out marks the solve (after rank 0's write)
  if (threadIdx.x == 0 && E.g3err) atomicMax(&pb.result[2], 3);
  if (E.tm.rank == 0 && threadIdx.x == 0) {
    pb.result[0] = stop;
    pb.result[1] = iters;
    pb.result[3] = n_dogleg;
    pb.info[0] = Tsize;
    pb.info[1] = best_error;
    pb.info[2] = E.damp;
    pb.info[3] = meanabs;
    pb.info[4] = (double)matvecs;
  }
}

template <class T, int TS>
__global__ void __launch_bounds__(TFX_THREADS, 1)
    dgn_kernel(const tfx_dgn_problem* __restrict__ probs, int nprob, tfx_dgn_options op, int cluster, SmemPlan sp) {
  extern __shared__ __align__(16) char smem[];
  Team tm = make_team(cluster);
  const int pid = blockIdx.x / cluster;
  if (pid >= nprob) return;
  tfx_dgn_problem pb = probs[pid];
  solve_problem<T, TS>(pb, op, tm, smem, sp);
}

// The same engine for batches of small problems, one CTA each: compiled for
// TFX_DENSE_CTAS resident CTAs per SM (fewer registers per thread), so that
// more problems run at once when their shared-memory plans fit.
#ifndef TFX_DENSE_CTAS
#define TFX_DENSE_CTAS 2
#endif
template <class T, int TS>
__global__ void __launch_bounds__(TFX_THREADS, TFX_DENSE_CTAS)
    dgn_kernel_dense(const tfx_dgn_problem* __restrict__ probs, int nprob, tfx_dgn_options op, SmemPlan sp) {
  extern __shared__ __align__(16) char smem[];
  Team tm = make_team(1);
  const int pid = blockIdx.x;
  if (pid >= nprob) return;
  tfx_dgn_problem pb = probs[pid];
  solve_problem<T, TS>(pb, op, tm, smem, sp);
}

// Arguments of the standalone evaluations (tfx_jtj_matvec, tfx_dgn_dogleg).
struct UnitsArgs {
  int mode;            // 0: gradient and/or J^T J v; 1: dogleg trials
  double damp;
  double error;        // dogleg: the rejected step's relative error
  const void* v;       // J^T J v input (flat), or null
  void* jtjv;          // J^T J v output, or null
  void* grad;          // gradient output (mode 0, or null) / dogleg gradient input (mode 1)
  const void* y;       // dogleg: the rejected step
  const void* jtj;     // dogleg: J^T J grad
  void* best_x;        // dogleg outputs: best point, step, factors and error
  void* best_y;
  void* best_W;
  double* best_error;
};

// One evaluation of the solver's own device code at a given point, without
// iterating.  Mode 0: the MTTKRP gradient g (GaussNewton.py:401-427
// compute_grad, the reference's sign) and J^T J v for a caller's vector v
// through the CG's product (GaussNewton.py:551-581), after the same Gramians
// and preconditioner set-up (GaussNewton.py:520-548, 584-627) as every dGN
// iteration; either output may be skipped (null).  Mode 1: the dogleg trials
// that follow a rejected step (GaussNewton.py:713-795) from the point x, the
// step y, the gradient and J^T J grad.
template <class T, int TS>
__global__ void __launch_bounds__(TFX_THREADS, 1)
    dgn_units_kernel(const tfx_dgn_problem* __restrict__ probs, tfx_dgn_options op, int cluster, SmemPlan sp,
                     UnitsArgs ua) {
  extern __shared__ __align__(16) char smem[];
  Team tm = make_team(cluster);
  tfx_dgn_problem pb = probs[0];
  Engine<T, TS> E;
  engine_setup<T, TS>(E, pb, op, tm, smem, sp);
  E.cprof = nullptr;
  E.gprof = nullptr;
  const T* x0 = (const T*)pb.x;
  E.damp = ua.damp;
  if (ua.mode == 0) {
    E.for_own([&](int e, int l, int c) { E.W[e] = x0[e]; });
    E.tm.sync();
    E.stage_W();
    E.gramians_and_precond();
    if (ua.grad) {
      T* gout = (T*)ua.grad;
      E.gradient_any();
      // the engine keeps M_l - W_l P1_l; the reference's g is its negative
      E.for_own([&](int e, int l, int c) { gout[e] = -E.grad[e]; });
    }
    E.tm.sync();
    if (ua.v && ua.jtjv) {
      if (E.stage)
        cg_matvec<T, true>(E.L, E.R, E.nx, E.ncol, E.c0, E.cgo, (const T*)ua.v, (T*)ua.jtjv, E.W, E.P1, E.P2);
      else
        cg_matvec<T, false>(E.L, E.R, E.nx, E.ncol, E.c0, E.cgo, (const T*)ua.v, (T*)ua.jtjv, E.W, E.P1, E.P2);
    }
  } else {
    double meanabs;
    E.tensor_norms(E.Tsize, meanabs);
    const T* yin = (const T*)ua.y;
    const T* gin = (const T*)ua.grad;
    const T* jin = (const T*)ua.jtj;
    // the state after a rejected step: xn = x + y, W = the rejected factors
    // (zero here: only read back when no trial improves)
    E.for_own([&](int e, int l, int c) {
      E.xn[e] = x0[e] + yin[e];
      E.y[e] = yin[e];
      E.grad[e] = gin[e];
      E.jtj[e] = jin[e];
      E.W[e] = T(0);
    });
    E.tm.sync();
    E.stage_W();
    const double err = E.dogleg(ua.error);
    T* bx = (T*)ua.best_x;
    T* by = (T*)ua.best_y;
    T* bw = (T*)ua.best_W;
    E.for_own([&](int e, int l, int c) {
      bx[e] = E.xn[e];
      by[e] = E.y[e];
      bw[e] = E.W[e];
    });
    if (E.tm.rank == 0 && threadIdx.x == 0) *ua.best_error = err;
  }
  if (E.tm.rank == 0 && threadIdx.x == 0) pb.result[2] = TFX_OK;
  E.tm.sync();
  if (threadIdx.x == 0 && E.g3err) atomicMax(&pb.result[2], 3);
}

}  // namespace tfx


// ============================================================================
// launch helper shared by the two instantiation units
// ============================================================================
#include "tfx_capi_internal.h"

namespace tfx {

template <class T, int TS>
static int launch_dgn(const tfx_dgn_problem* d_probs, int nprob, const tfx_dgn_options* op, int cluster,
                      const SmemPlan& sp, cudaStream_t st) {
  if (cluster == 1 && TS <= 2 && nprob > 1 && TFX_DENSE_CTAS * (sp.total + 1024) <= 227 * 1024) {
    // many small problems: several CTAs per SM
    auto kd = dgn_kernel_dense<T, TS>;
    cudaError_t e = cudaFuncSetAttribute(kd, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sp.total);
    if (e != cudaSuccess) return tfx_set_cuda_error(e, "dgn smem attribute");
    kd<<<nprob, TFX_THREADS, sp.total, st>>>(d_probs, nprob, *op, sp);
    e = cudaGetLastError();
    if (e != cudaSuccess) return tfx_set_cuda_error(e, "dgn launch");
    tfx_count_launch(1);
    return TFX_STATUS_OK;
  }
  auto kfn = dgn_kernel<T, TS>;
  cudaError_t e = cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sp.total);
  if (e != cudaSuccess) return tfx_set_cuda_error(e, "dgn smem attribute");
  if (cluster > 8) {
    // clusters of 9..16 CTAs are beyond the portable size
    e = cudaFuncSetAttribute(kfn, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    if (e != cudaSuccess) return tfx_set_cuda_error(e, "dgn cluster attribute");
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)(nprob * cluster));
  cfg.blockDim = dim3(TFX_THREADS);
  cfg.dynamicSmemBytes = sp.total;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = (unsigned)cluster;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  if (cluster > 1) {
    int ncl = 0;
    e = cudaOccupancyMaxActiveClusters(&ncl, kfn, &cfg);
    if (e != cudaSuccess) return tfx_set_cuda_error(e, "dgn cluster occupancy");
    if (ncl < 1) return tfx_set_error(TFX_STATUS_ERR_UNSUPPORTED, "cluster size cannot be scheduled");
  }
  e = cudaLaunchKernelEx(&cfg, kfn, d_probs, nprob, *op, cluster, sp);
  if (e != cudaSuccess) return tfx_set_cuda_error(e, "dgn launch");
  tfx_count_launch(1);
  return TFX_STATUS_OK;
}

template <class T, int TS>
static int launch_units(const tfx_dgn_problem* d_prob, const tfx_dgn_options* op, int cluster, const SmemPlan& sp,
                        const UnitsArgs& ua, cudaStream_t st) {
  auto kfn = dgn_units_kernel<T, TS>;
  cudaError_t e = cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sp.total);
  if (e != cudaSuccess) return tfx_set_cuda_error(e, "dgn units smem attribute");
  if (cluster > 8) {
    e = cudaFuncSetAttribute(kfn, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    if (e != cudaSuccess) return tfx_set_cuda_error(e, "dgn units cluster attribute");
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)cluster);
  cfg.blockDim = dim3(TFX_THREADS);
  cfg.dynamicSmemBytes = sp.total;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = (unsigned)cluster;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  if (cluster > 1) {
    int ncl = 0;
    e = cudaOccupancyMaxActiveClusters(&ncl, kfn, &cfg);
    if (e != cudaSuccess) return tfx_set_cuda_error(e, "dgn units cluster occupancy");
    if (ncl < 1) return tfx_set_error(TFX_STATUS_ERR_UNSUPPORTED, "cluster size cannot be scheduled");
  }
  e = cudaLaunchKernelEx(&cfg, kfn, d_prob, *op, cluster, sp, ua);
  if (e != cudaSuccess) return tfx_set_cuda_error(e, "dgn units launch");
  tfx_count_launch(1);
  return TFX_STATUS_OK;
}

int launch_dgn_f32(int TS, const tfx_dgn_problem* d_probs, int nprob, const tfx_dgn_options* op, int cluster,
                   const SmemPlan& sp, cudaStream_t st);
int launch_units_f32(int TS, const tfx_dgn_problem* d_prob, const tfx_dgn_options* op, int cluster, const SmemPlan& sp,
                     const UnitsArgs& ua, cudaStream_t st);
int launch_units_f64(int TS, const tfx_dgn_problem* d_prob, const tfx_dgn_options* op, int cluster, const SmemPlan& sp,
                     const UnitsArgs& ua, cudaStream_t st);
int launch_dgn_f64(int TS, const tfx_dgn_problem* d_probs, int nprob, const tfx_dgn_options* op, int cluster,
                   const SmemPlan& sp, cudaStream_t st);

}  // namespace tfx
