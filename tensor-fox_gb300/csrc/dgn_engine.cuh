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

struct SmemPlan {
  size_t sA, sB, sPart, sAk, sY, sM, sDG, sGam, sNorm, sBase, sIdx, rs4, rs12, misc, hist, rs1, rs1b, sScale;
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
  p.sY = o; o += al16((size_t)maxL * maxR * maxncol * es);
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
  p.stage = stage;
  p.sQf = p.sWf = p.sP1o = p.sP2o = p.sVec = o;
  if (stage) {
    p.sQf = o; o += al16((size_t)maxnx * es);
    p.sWf = o; o += al16((size_t)maxnx * es);
    p.sP1o = o; o += al16((size_t)maxL * maxR * maxncol * es);
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
  size_t d, sQf, sWf, sP1o, sP2o, sAk, sY, sM, sDG, rs4, rs1, sVec;
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

template <class T, bool STAGED>
__device__ __forceinline__ void cg_matvec(const int L, const int R, const int nx, const int ncol, const int c0,
                                          const CgOffsets so, const T* Dglob, T* zout, const T* Wg, const T* P1g,
                                          const T* P2g, T* zloc = nullptr, long long* cprof = nullptr) {
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
    T* sQf = (T*)(sm + so.sQf);
    stage_copy(sQf, Dglob, nx);
    __syncthreads();
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
  for (int e = tid; e < L * RN; e += TFX_THREADS) {
    const int k = e / RN, q = e - k * RN, a = q / ncol, c = q - a * ncol;
    const int dk = d[k];
    const T* dv = Din + off[k] + a * dk;
    const T* wv = Wr + off[k] + (c0 + c) * dk;
    T acc = T(0);
#pragma unroll 4
    for (int i = 0; i < dk; ++i) acc = fma(dv[i], wv[i], acc);
    sAk[e] = acc;
  }
  __syncthreads();
  ctick(2);
  for (int e = tid; e < L * RN; e += TFX_THREADS) {
    const int l = e / RN, q = e - l * RN, a = q / ncol, c = q - a * ncol;
    T acc = T(0);
    for (int k = 0; k < L; ++k) {
      if (k == l) continue;
      const T p2 = STAGED ? sP2o[((size_t)(l * L + k) * R + a) * ncol + c]
                          : P2g[((size_t)(l * L + k) * R + a) * R + c0 + c];
      acc += p2 * sAk[(size_t)k * RN + q];
    }
    sY[e] = acc;
  }
  __syncthreads();
  ctick(3);
  // z_l = W_l Y_l + D_l P1_l over all owned outputs of all modes at once
  const int ownn = ncol * (nx / R);
  for (int e = tid; e < ownn; e += TFX_THREADS) {
    int l = 0, rem = e;
    while (rem >= ncol * d[l]) {
      rem -= ncol * d[l];
      ++l;
    }
    const int dl = d[l], ol = off[l];
    const int c = rem / dl, i = rem - c * dl;
    const T* wrow = Wr + ol + i;
    const T* drow = Din + ol + i;
    const T* yc = sY + (size_t)l * RN + c;
    const T* p1c = STAGED ? sP1o + (size_t)l * R * ncol + c : P1g + (size_t)l * R * R + c0 + c;
    const int p1s = STAGED ? ncol : R;
    T a1 = T(0), a2 = T(0);
#pragma unroll 4
    for (int r = 0; r < R; ++r) {
      a1 = fma(wrow[r * dl], yc[r * ncol], a1);
      a2 = fma(drow[r * dl], p1c[r * p1s], a2);
    }
    if (zloc)
      zloc[e] = a1 + a2;
    else
      zout[ol + (c0 + c) * dl + i] = a1 + a2;
  }
  __syncthreads();
  ctick(4);
}

template <class T, bool STAGED>
__device__ __forceinline__ int cg_team(const Team tm, const int L, const int R, const int nx, const int ncol,
                                       const int c0, const CgOffsets so, T* grad, T* jtj, T* y, T* r, T* P, T* Q,
                                       T* z, const T* Wg, const T* P1g, const T* P2g, const int budget,
                                       const double cg_tol, double& rn_out, int& flip4, long long* cprof_g) {
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
  RedScratch<1>* rs1 = (RedScratch<1>*)(sm + so.rs1);
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
  Acc<T> v[1];
  double red[1];
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
  team_sum_acc<1, T>(tm, v, red, rs1, flip4);
  double rn = red[0];
  if (rn == 0.0) rn = 1e-6;
  int maxit = budget;
  double tol = cg_tol;
  if (nx > 100) {
    maxit = min(maxit, nx);
  } else {
    tol = 0.0;
  }
  int itn = 0;
  bool broke = false;
  for (itn = 0; itn < maxit; ++itn) {
    // Q = M P (owned part, published through global memory)
    for (int l = 0; l < L; ++l) {
      const int dl = d[l], base = off[l] + c0 * dl, n = ncol * dl, lb = ncol * (off[l] / R);
      for (int e = tid; e < n; e += TFX_THREADS) {
        if (STAGED) {
          Q[base + e] = vM[lb + e] * vP[lb + e];
        } else {
          const int c = e / dl;
          Q[base + e] = sM[l * ncol + c] * P[base + e];
        }
      }
    }
    tm.sync();
    ctick(0);
    cg_matvec<T, STAGED>(L, R, nx, ncol, c0, so, Q, z, Wg, P1g, P2g, STAGED ? vz : nullptr, cprof);
    if (cprof) tc = clock64();
    Acc<T> w[1];
    const T* Qs = STAGED ? (const T*)(sm + so.sQf) : Q;  // full Q, staged by the matvec
    for (int l = 0; l < L; ++l) {
      const int dl = d[l], base = off[l] + c0 * dl, n = ncol * dl, lb = ncol * (off[l] / R);
      for (int e = tid; e < n; e += TFX_THREADS) {
        if (STAGED) {
          const T zz = vM[lb + e] * (vz[lb + e] + vDG[lb + e] * Qs[base + e]);
          vz[lb + e] = zz;
          w[0].fma_(vP[lb + e], zz);
        } else {
          const int c = e / dl, g = base + e;
          const T zz = sM[l * ncol + c] * (z[g] + sDG[l * ncol + c] * Q[g]);
          z[g] = zz;
          w[0].fma_(P[g], zz);
        }
      }
    }
    team_sum_acc<1, T>(tm, w, red, rs1, flip4);
    ctick(5);
    double den = red[0];
    if (den == 0.0) den = 1e-6;
    const double alpha = rn / den;
    const T ta = (T)alpha;
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
    team_sum_acc<1, T>(tm, u, red, rs1, flip4);
    ctick(6);
    const double rn_new = red[0];
    const double beta = rn_new / rn;
    rn = rn_new;
    const T tb = (T)beta;
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
  __syncthreads();
  if (cprof_g)
    for (int k = 0; k < 8; ++k) cprof_g[k] += lprof[k];
  rn_out = rn;
  return broke ? itn + 1 : maxit;
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
  int flip4, flip12, flip1, flip1b;
  RedScratch<1>* rs1b;
  T* sScale;
  double damp, Tsize;
  tfx_dgn_options op;
  // staged operands: full search direction and factors, owned P1/P2 columns
  int stage;
  T *sQf, *sWf, *sP1o, *sP2o;
  const T* Wr;  // factors to read: shared-memory copy when staged

  __device__ __forceinline__ T& P1at(int l, int a, int c) {
    return stage ? sP1o[((size_t)l * R + a) * ncol + c] : P1[((size_t)l * R + a) * R + c0 + c];
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
  __device__ int cg(int budget, double& rn_out) {
    if (stage)
      return cg_team<T, true>(tm, L, R, nx, ncol, c0, cgo, grad, jtj, y, r, P, Q, z, W, P1, P2, budget, op.cg_tol,
                              rn_out, flip1, cprof);
    return cg_team<T, false>(tm, L, R, nx, ncol, c0, cgo, grad, jtj, y, r, P, Q, z, W, P1, P2, budget, op.cg_tol,
                             rn_out, flip1, cprof);
  }

  // Column balancing of x into the factor buffer (Conversion.py:361-387),
  // then transform (Conversion.py:412-444).  Owned columns only, except the
  // factors_norm rescaling which needs a team-wide norm per mode.
  __device__ void to_factors(const T* src, T* dst, bool eq) {
    if (eq) {
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
    if (op.symm) {
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
  }

  // ||T - [[W]]|| / ||T|| (Conversion.py:117-141 + Critical.py:14-22), fused:
  // the model tile is built in registers and never stored.
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
      error = rel_error(Wr);
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

template <class T, int TS>
__device__ void solve_problem(const tfx_dgn_problem& pb, const tfx_dgn_options& op, Team tm, char* smem,
                              const SmemPlan& sp) {
  Engine<T, TS> E;
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
  E.rs1b = (RedScratch<1>*)(smem + sp.rs1b);
  E.sScale = (T*)(smem + sp.sScale);
  E.flip1 = 0;
  E.flip1b = 0;
  E.flip4 = 0;
  E.flip12 = 0;

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
    E.gradient();
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
    E.tm.sync();
    E.stage_W();
    tick(3);
    error = E.rel_error(E.Wr);
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
  E.tm.sync();
  if (E.tm.rank == 0 && threadIdx.x == 0) {
    pb.result[0] = stop;
    pb.result[1] = iters;
    pb.result[2] = TFX_OK;
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

}  // namespace tfx


// ============================================================================
// launch helper shared by the two instantiation units
// ============================================================================
#include "tfx_capi_internal.h"

namespace tfx {

template <class T, int TS>
static int launch_dgn(const tfx_dgn_problem* d_probs, int nprob, const tfx_dgn_options* op, int cluster,
                      const SmemPlan& sp, cudaStream_t st) {
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

int launch_dgn_f32(int TS, const tfx_dgn_problem* d_probs, int nprob, const tfx_dgn_options* op, int cluster,
                   const SmemPlan& sp, cudaStream_t st);
int launch_dgn_f64(int TS, const tfx_dgn_problem* d_probs, int nprob, const tfx_dgn_options* op, int cluster,
                   const SmemPlan& sp, cudaStream_t st);

}  // namespace tfx
