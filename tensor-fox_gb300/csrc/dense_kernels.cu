// Grid-level dense kernels of the compression (MLSVD) and full-tensor stages.
//
//   tfx_mode_gram      S_(l) S_(l)^T of a C-order tensor viewed as (P, D, Q)
//                      (Compression.py:192-237: the Gram route replaces the
//                      randomized SVD's streaming passes over the unfolding)
//   tfx_gemm           strided batched C = alpha A B + beta C (TTM, subspace
//                      products, decompression U_l W_l; TensorFox.py:573-574)
//   tfx_orthonormalize CGS2 on the columns of a tall matrix (one CTA)
//   tfx_sym_eig        cyclic parallel Jacobi eigensolver (one CTA)
//   tfx_cp_residual    ||T - [[W]]||^2 fused (Conversion.py:117-141 +
//                      Critical.py:14-22) -- the model tile is never stored
//   tfx_tensor_norms   sum t^2 and sum |t| (TensorFox.py:503, GaussNewton.py:113)
//   tfx_flip_signs     largest |entry| of every column made positive
//                      (Compression.py:521-564)
#include <math.h>

#include <algorithm>

#include "tfx_capi_internal.h"
#include "tfx_common.cuh"
#include "linalg.cuh"

namespace tfx {

// ---------------------------------------------------------------------------
// mode Gram: partial[s][i][j] = sum_{k in split s} A(i,k) A(j,k),
// A(i, k) = S[p*D*Q + i*Q + q] with k = p*Q + q; upper tile pairs only.
// ---------------------------------------------------------------------------
template <class T, int TS>
__global__ void __launch_bounds__(TFX_THREADS) k_mode_gram(const T* __restrict__ S, long long P, int D, long long Q,
                                                           int ksplit, T* __restrict__ part) {
  using TL = Tile<TS, TS>;
  __shared__ T sA[TFX_BK * TL::LDA];
  __shared__ T sB[TFX_BK * TL::LDB];
  const int nt = (D + TL::BM - 1) / TL::BM;
  // tile pair index -> (bi, bj), bi <= bj
  int t = blockIdx.x, bi = 0;
  while (t >= nt - bi) {
    t -= nt - bi;
    ++bi;
  }
  const int bj = bi + t;
  const int i0 = bi * TL::BM, j0 = bj * TL::BN;
  const long long K = P * Q;
  const long long kb = K * blockIdx.y / ksplit, ke = K * (blockIdx.y + 1) / ksplit;
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  T acc[TS][TS];
  tile_zero<T, TS, TS>(acc);
  const bool kfast = Q > 1;
  for (long long k0 = kb; k0 < ke; k0 += TFX_BK) {
    const int kc = (int)min((long long)TFX_BK, ke - k0);
    for (int e = tid; e < TFX_BK * TL::BM; e += TFX_THREADS) {
      int kk, mm;
      if (kfast) {
        mm = e / TFX_BK;
        kk = e - mm * TFX_BK;
      } else {
        kk = e / TL::BM;
        mm = e - kk * TL::BM;
      }
      T va = T(0), vb = T(0);
      if (kk < kc) {
        const long long k = k0 + kk, p = k / Q, q = k - p * Q;
        const long long base = p * (long long)D * Q + q;
        if (i0 + mm < D) va = S[base + (long long)(i0 + mm) * Q];
        if (j0 + mm < D) vb = S[base + (long long)(j0 + mm) * Q];
      }
      sA[kk * TL::LDA + mm] = va;
      sB[kk * TL::LDB + mm] = vb;
    }
    __syncthreads();
    tile_fma<T, TS, TS>(sA, sB, acc, kc);
    __syncthreads();
  }
  T* out = part + (size_t)blockIdx.y * D * D;
#pragma unroll
  for (int u = 0; u < TS; ++u)
#pragma unroll
    for (int v = 0; v < TS; ++v) {
      const int i = i0 + ty + 16 * u, j = j0 + tx + 16 * v;
      if (i < D && j < D) out[(size_t)i * D + j] = acc[u][v];
    }
}

template <class T, int BMt>
__global__ void k_gram_reduce(const T* __restrict__ part, int D, int ksplit, T* __restrict__ G) {
  const long long n = (long long)D * D;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(e / D), j = (int)(e - (long long)i * D);
    const long long src = (i / BMt <= j / BMt) ? e : (long long)j * D + i;
    double s = 0.0;
    for (int k = 0; k < ksplit; ++k) s += (double)part[(size_t)k * n + src];
    G[e] = (T)s;
  }
}

// ---------------------------------------------------------------------------
// strided batched GEMM: C[b](m,n) = alpha * sum_k A[b](m,k) B[b](k,n) + beta C
// ---------------------------------------------------------------------------
struct GemmArgs {
  long long M, N, K, batch;
  long long sAb, sAm, sAk, sBb, sBk, sBn, sCb, sCm, sCn;
  double alpha, beta;
};

template <class T, int TS>
__global__ void __launch_bounds__(TFX_THREADS) k_gemm(const T* __restrict__ A, const T* __restrict__ B, T* C,
                                                      GemmArgs g) {
  using TL = Tile<TS, TS>;
  __shared__ T sA[TFX_BK * TL::LDA];
  __shared__ T sB[TFX_BK * TL::LDB];
  const long long tilesM = (g.M + TL::BM - 1) / TL::BM;
  const long long m0 = (blockIdx.x % tilesM) * TL::BM;
  const long long n0 = (blockIdx.x / tilesM) * TL::BN;
  for (long long b = blockIdx.y; b < g.batch; b += gridDim.y) {
    const T* Ab = A + b * g.sAb;
    const T* Bb = B + b * g.sBb;
    T* Cb = C + b * g.sCb;
    const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
    T acc[TS][TS];
    tile_zero<T, TS, TS>(acc);
    const bool a_mfast = g.sAm == 1, b_nfast = g.sBn == 1;
    for (long long k0 = 0; k0 < g.K; k0 += TFX_BK) {
      const int kc = (int)min((long long)TFX_BK, g.K - k0);
      for (int e = tid; e < TFX_BK * TL::BM; e += TFX_THREADS) {
        int kk, mm;
        if (a_mfast) {
          kk = e / TL::BM;
          mm = e - kk * TL::BM;
        } else {
          mm = e / TFX_BK;
          kk = e - mm * TFX_BK;
        }
        sA[kk * TL::LDA + mm] = (kk < kc && m0 + mm < g.M) ? Ab[(m0 + mm) * g.sAm + (k0 + kk) * g.sAk] : T(0);
      }
      for (int e = tid; e < TFX_BK * TL::BN; e += TFX_THREADS) {
        int kk, nn;
        if (b_nfast) {
          kk = e / TL::BN;
          nn = e - kk * TL::BN;
        } else {
          nn = e / TFX_BK;
          kk = e - nn * TFX_BK;
        }
        sB[kk * TL::LDB + nn] = (kk < kc && n0 + nn < g.N) ? Bb[(k0 + kk) * g.sBk + (n0 + nn) * g.sBn] : T(0);
      }
      __syncthreads();
      tile_fma<T, TS, TS>(sA, sB, acc, kc);
      __syncthreads();
    }
#pragma unroll
    for (int u = 0; u < TS; ++u)
#pragma unroll
      for (int v = 0; v < TS; ++v) {
        const long long m = m0 + ty + 16 * u, n = n0 + tx + 16 * v;
        if (m < g.M && n < g.N) {
          T* c = Cb + m * g.sCm + n * g.sCn;
          const T r = (T)(g.alpha * (double)acc[u][v]);
          *c = (g.beta == 0.0) ? r : (T)((double)r + g.beta * (double)*c);
        }
      }
  }
}

// ---------------------------------------------------------------------------
// Mode product for FP32 with a short left factor: out[p] (n x Q) = Ut (n x D)
// times S[p] (D x Q), all row-major.  One warp owns 8 rows of the output tile
// and each lane 8 x TN outputs; per 4 k steps a lane reads 8 broadcast float4
// of Ut and TN float4 of S for 32*TN FMAs.  The (BK x BN) slab of S and the
// (BM x BK) slab of Ut are double-buffered in shared memory and filled with
// cp.async (16-byte copies, zero-filled past the edges), so the next slab
// streams in while the current one is multiplied.  The block has
// 32 * ceil(rows/8) threads (at most 8 warps): a 50-row factor wastes 6 rows
// instead of 14.  Needs D % 4 == 0, Q % 4 == 0 and 16-byte aligned pointers.
// ---------------------------------------------------------------------------
constexpr int TTM_BK = 16;

__device__ __forceinline__ void cp_async16(void* sdst, const void* gsrc, int src_bytes) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(sdst);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(sa), "l"(gsrc), "r"(src_bytes) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

template <int TN>
__global__ void __launch_bounds__(256, 2) k_ttm_f32(const float* __restrict__ Ut, const float* __restrict__ S,
                                                    float* __restrict__ out, int n, int D, long long Q, long long P) {
  constexpr int BN = 32 * TN;
  constexpr int AKS = TTM_BK + 4;  // padded row stride of the Ut slab
  __shared__ __align__(16) float sA[2][64][AKS];
  __shared__ __align__(16) float sB[2][TTM_BK][BN];
  const int nw = blockDim.x >> 5, nt = blockDim.x;
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  const int BM = 8 * nw;
  const int m0 = blockIdx.z * BM;
  const long long q0 = (long long)blockIdx.x * BN;
  const int nk = (D + TTM_BK - 1) / TTM_BK;
  for (long long p = blockIdx.y; p < P; p += gridDim.y) {
    const float* Sp = S + p * (long long)D * Q;
    auto issue = [&](int t, int b) {
      const int k0 = t * TTM_BK;
      for (int e = tid; e < BM * (TTM_BK / 4); e += nt) {
        const int m = e >> 2, k4 = (e & 3) * 4;
        const bool ok = m0 + m < n && k0 + k4 < D;
        cp_async16(&sA[b][m][k4], ok ? (const void*)(Ut + (long long)(m0 + m) * D + k0 + k4) : (const void*)Ut,
                   ok ? 16 : 0);
      }
      for (int e = tid; e < TTM_BK * (BN / 4); e += nt) {
        const int kk = e / (BN / 4), c4 = (e - kk * (BN / 4)) * 4;
        const bool ok = k0 + kk < D && q0 + c4 < Q;
        cp_async16(&sB[b][kk][c4], ok ? (const void*)(Sp + (long long)(k0 + kk) * Q + q0 + c4) : (const void*)Sp,
                   ok ? 16 : 0);
      }
      cp_async_commit();
    };
    float acc[8][TN];
#pragma unroll
    for (int i = 0; i < 8; ++i)
#pragma unroll
      for (int j = 0; j < TN; ++j) acc[i][j] = 0.f;
    __syncthreads();  // the previous p's readers are done with both buffers
    issue(0, 0);
    for (int t = 0; t < nk; ++t) {
      const int b = t & 1;
      if (t + 1 < nk) {
        issue(t + 1, b ^ 1);
        cp_async_wait<1>();
      } else {
        cp_async_wait<0>();
      }
      __syncthreads();
#pragma unroll
      for (int k4 = 0; k4 < TTM_BK; k4 += 4) {
        float4 a[8];
#pragma unroll
        for (int i = 0; i < 8; ++i) a[i] = *(const float4*)&sA[b][wid * 8 + i][k4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          float bv[TN];
#pragma unroll
          for (int j4 = 0; j4 < TN / 4; ++j4) {
            const float4 v = *(const float4*)&sB[b][k4 + u][j4 * 128 + lane * 4];
            bv[4 * j4 + 0] = v.x;
            bv[4 * j4 + 1] = v.y;
            bv[4 * j4 + 2] = v.z;
            bv[4 * j4 + 3] = v.w;
          }
#pragma unroll
          for (int i = 0; i < 8; ++i) {
            const float ai = u == 0 ? a[i].x : u == 1 ? a[i].y : u == 2 ? a[i].z : a[i].w;
#pragma unroll
            for (int j = 0; j < TN; ++j) acc[i][j] = fmaf(ai, bv[j], acc[i][j]);
          }
        }
      }
      __syncthreads();  // slab b is free for the copy issued next iteration
    }
    float* op = out + p * (long long)n * Q;
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const int m = m0 + wid * 8 + i;
      if (m >= n) continue;
#pragma unroll
      for (int j4 = 0; j4 < TN / 4; ++j4) {
        const long long q = q0 + j4 * 128 + lane * 4;
        if (q < Q)
          *(float4*)(op + (long long)m * Q + q) =
              make_float4(acc[i][4 * j4], acc[i][4 * j4 + 1], acc[i][4 * j4 + 2], acc[i][4 * j4 + 3]);
      }
    }
  }
}

// ---------------------------------------------------------------------------
// CGS2 orthonormalisation of the k columns of Y (D x k, column-major), in place.
// ---------------------------------------------------------------------------
// Shared-memory variant: the whole D x k block lives in shared memory, so each
// of the 4k dependent phases costs a barrier instead of an L2 round trip.
template <class T>
__global__ void __launch_bounds__(TFX_THREADS) k_orth_smem(T* Y, int D, int k) {
  extern __shared__ __align__(16) char smem_o[];
  T* Ys = (T*)smem_o;                          // k columns of length D
  T* coef = Ys + (size_t)D * k;                // k coefficients
  size_t roff = ((size_t)D * k + ((k + 1) & ~1) + 2) * sizeof(T);
  roff = (roff + 15) & ~(size_t)15;
  double* red = (double*)(smem_o + roff);
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  for (int e = tid; e < D * k; e += TFX_THREADS) Ys[e] = Y[e];
  __syncthreads();
  for (int j = 0; j < k; ++j) {
    T* yj = Ys + (size_t)j * D;
    for (int pass = 0; pass < 2; ++pass) {
      for (int i = wid; i < j; i += TFX_THREADS / 32) {
        const T* yi = Ys + (size_t)i * D;
        T s = T(0);
        for (int r = lane; r < D; r += 32) s = fma(yi[r], yj[r], s);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (lane == 0) coef[i] = s;
      }
      __syncthreads();
      for (int r = tid; r < D; r += TFX_THREADS) {
        T v = yj[r];
        for (int i = 0; i < j; ++i) v = fma(-coef[i], Ys[(size_t)i * D + r], v);
        yj[r] = v;
      }
      __syncthreads();
    }
    double sq = 0.0;
    for (int r = tid; r < D; r += TFX_THREADS) sq += (double)yj[r] * (double)yj[r];
    sq = warp_sum(sq);
    if (lane == 0) red[wid] = sq;
    __syncthreads();
    double nrm = 0.0;
    for (int w = 0; w < TFX_THREADS / 32; ++w) nrm += red[w];
    const T inv = (T)(nrm > 0.0 ? 1.0 / sqrt(nrm) : 0.0);
    for (int r = tid; r < D; r += TFX_THREADS) yj[r] = yj[r] * inv;
    __syncthreads();
  }
  for (int e = tid; e < D * k; e += TFX_THREADS) Y[e] = Ys[e];
}

// Blocked CGS2 (BCGS2): panels of ORTH_B columns are projected against the
// finished columns twice with two matrix products (coefficients C = Q^T P,
// then P -= Q C), and orthonormalised inside the panel by column CGS2 with
// thread-private rows.  The serial chain is k / ORTH_B panel steps instead of
// k column steps, and each finished column is read once per panel instead of
// once per later column.  Y (D x k, column-major) is staged in shared memory
// with a column stride ldy = D rounded up to 1 mod 32 elements, so that lanes
// reading the same row of 32 different columns hit 32 different banks.
constexpr int ORTH_NT = 256, ORTH_NW = ORTH_NT / 32, ORTH_B = 8;

__host__ __device__ inline int orth_ldy(int D) { return D + ((33 - (D & 31)) & 31); }

__host__ __device__ inline size_t orth_align16(size_t b) { return (b + 15) & ~(size_t)15; }

template <class T>
__device__ __forceinline__ void load_row8(const T* p, T (&v)[ORTH_B]) {
#pragma unroll
  for (int c = 0; c < ORTH_B; ++c) v[c] = p[c];
}
template <>
__device__ __forceinline__ void load_row8<float>(const float* p, float (&v)[ORTH_B]) {
  const float4 a = *(const float4*)p, b = *(const float4*)(p + 4);
  v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w;
  v[4] = b.x; v[5] = b.y; v[6] = b.z; v[7] = b.w;
}
template <>
__device__ __forceinline__ void load_row8<double>(const double* p, double (&v)[ORTH_B]) {
#pragma unroll
  for (int c = 0; c < ORTH_B; c += 2) {
    const double2 a = *(const double2*)(p + c);
    v[c] = a.x;
    v[c + 1] = a.y;
  }
}

template <class T>
static __host__ __device__ size_t orth_bcgs_offsets(int D, int k, size_t* oP, size_t* oPart, size_t* oC,
                                                    size_t* oRed) {
  size_t o = orth_align16((size_t)k * orth_ldy(D) * sizeof(T));
  *oP = o;
  o = orth_align16(o + (size_t)D * ORTH_B * sizeof(T));
  *oPart = o;
  o = orth_align16(o + (size_t)ORTH_NW * 32 * ORTH_B * sizeof(T));
  *oC = o;
  o = orth_align16(o + (size_t)k * ORTH_B * sizeof(T));
  *oRed = o;
  return o;
}

// Column CGS2 of the (D x cb) panel by one warp with the panel in registers:
// lane l holds rows l, l + 32, ... (RPL of them).  Every loop is unrolled
// over compile-time column indices, so the dots, shuffles and updates of a
// column are independent instructions rather than a chain of shared-memory
// round trips.
template <class T, int RPL>
__device__ __forceinline__ void panel_cgs2_warp(T* Pb, int D, int cb) {
  const int lane = threadIdx.x & 31;
  T v[RPL][ORTH_B];
#pragma unroll
  for (int t = 0; t < RPL; ++t) {
    const int r = lane + 32 * t;
    if (r < D) {
      load_row8<T>(Pb + (size_t)r * ORTH_B, v[t]);
    } else {
#pragma unroll
      for (int c = 0; c < ORTH_B; ++c) v[t][c] = T(0);
    }
  }
#pragma unroll
  for (int c = 0; c < ORTH_B; ++c) {
    if (c < cb) {
#pragma unroll
      for (int pass = 0; pass < 2; ++pass) {
        if (c > 0) {
          T d[ORTH_B];
#pragma unroll
          for (int c2 = 0; c2 < c; ++c2) {
            d[c2] = T(0);
#pragma unroll
            for (int t = 0; t < RPL; ++t) d[c2] = fma(v[t][c2], v[t][c], d[c2]);
          }
#pragma unroll
          for (int o = 16; o > 0; o >>= 1)
#pragma unroll
            for (int c2 = 0; c2 < c; ++c2) d[c2] += __shfl_xor_sync(0xffffffffu, d[c2], o);
#pragma unroll
          for (int t = 0; t < RPL; ++t)
#pragma unroll
            for (int c2 = 0; c2 < c; ++c2) v[t][c] = fma(-d[c2], v[t][c2], v[t][c]);
        }
      }
      T nq = T(0);
#pragma unroll
      for (int t = 0; t < RPL; ++t) nq = fma(v[t][c], v[t][c], nq);
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) nq += __shfl_xor_sync(0xffffffffu, nq, o);
      const T inv = nq > T(0) ? T(1) / sqrt(nq) : T(0);
#pragma unroll
      for (int t = 0; t < RPL; ++t) v[t][c] *= inv;
    }
  }
#pragma unroll
  for (int t = 0; t < RPL; ++t) {
    const int r = lane + 32 * t;
    if (r < D)
#pragma unroll
      for (int c = 0; c < ORTH_B; ++c) Pb[(size_t)r * ORTH_B + c] = v[t][c];
  }
}

// The same panel CGS2 on the first NWP warps: lane l of warp w holds rows
// (w RPW + t) 32 + l, t < RPW (D <= 32 NWP RPW), so every dot product is a
// warp sum plus a fixed-order sum of the NWP warp partials through shared
// memory (part: 2 x NWP x ORTH_B values, used alternately), one named barrier
// of the NWP warps per reduction.  Four warps take a quarter of the one-warp
// form's multiply-adds per column.
template <class T, int RPW, int NWP>
__device__ __forceinline__ void panel_cgs2_warps(T* Pb, int D, int cb, T* part) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  T v[RPW][ORTH_B];
#pragma unroll
  for (int t = 0; t < RPW; ++t) {
    const int r = (w * RPW + t) * 32 + lane;
    if (r < D) {
      load_row8<T>(Pb + (size_t)r * ORTH_B, v[t]);
    } else {
#pragma unroll
      for (int c = 0; c < ORTH_B; ++c) v[t][c] = T(0);
    }
  }
  int buf = 0;
  // d[0..n) summed over the NWP warps, identical in every lane of every warp
  auto allsum = [&](T (&d)[ORTH_B], int n) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
#pragma unroll
      for (int c2 = 0; c2 < ORTH_B; ++c2)
        if (c2 < n) d[c2] += __shfl_xor_sync(0xffffffffu, d[c2], o);
    T* pb = part + buf * NWP * ORTH_B;
    if (lane == 0)
#pragma unroll
      for (int c2 = 0; c2 < ORTH_B; ++c2)
        if (c2 < n) pb[w * ORTH_B + c2] = d[c2];
    asm volatile("bar.sync 1, %0;" ::"r"(NWP * 32) : "memory");
#pragma unroll
    for (int c2 = 0; c2 < ORTH_B; ++c2)
      if (c2 < n) {
        T x = pb[c2];
#pragma unroll
        for (int q = 1; q < NWP; ++q) x += pb[q * ORTH_B + c2];
        d[c2] = x;
      }
    buf ^= 1;
  };
#pragma unroll
  for (int c = 0; c < ORTH_B; ++c) {
    if (c < cb) {
#pragma unroll
      for (int pass = 0; pass < 2; ++pass) {
        if (c > 0) {
          T d[ORTH_B];
#pragma unroll
          for (int c2 = 0; c2 < ORTH_B; ++c2) {
            d[c2] = T(0);
            if (c2 < c)
#pragma unroll
              for (int t = 0; t < RPW; ++t) d[c2] = fma(v[t][c2], v[t][c], d[c2]);
          }
          allsum(d, c);
#pragma unroll
          for (int t = 0; t < RPW; ++t)
#pragma unroll
            for (int c2 = 0; c2 < ORTH_B; ++c2)
              if (c2 < c) v[t][c] = fma(-d[c2], v[t][c2], v[t][c]);
        }
      }
      T nq[ORTH_B];
      nq[0] = T(0);
#pragma unroll
      for (int t = 0; t < RPW; ++t) nq[0] = fma(v[t][c], v[t][c], nq[0]);
      allsum(nq, 1);
      const T inv = nq[0] > T(0) ? T(1) / sqrt(nq[0]) : T(0);
#pragma unroll
      for (int t = 0; t < RPW; ++t) v[t][c] *= inv;
    }
  }
#pragma unroll
  for (int t = 0; t < RPW; ++t) {
    const int r = (w * RPW + t) * 32 + lane;
    if (r < D)
#pragma unroll
      for (int c = 0; c < ORTH_B; ++c) Pb[(size_t)r * ORTH_B + c] = v[t][c];
  }
}

template <class T, int RPL>
__global__ void __launch_bounds__(ORTH_NT) k_orth_bcgs(T* Y, int D, int k) {
  extern __shared__ __align__(16) char smem_b[];
  size_t oP, oPart, oC, oRed;
  orth_bcgs_offsets<T>(D, k, &oP, &oPart, &oC, &oRed);
  const int ldy = orth_ldy(D);
  T* Ys = (T*)smem_b;               // column j at Ys[j * ldy]
  T* Pb = (T*)(smem_b + oP);        // panel, row r at Pb[r * ORTH_B]
  T* part = (T*)(smem_b + oPart);   // partial coefficients [slice][i][c]
  T* C = (T*)(smem_b + oC);         // coefficients [i][c]
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  for (int e = tid; e < D * k; e += ORTH_NT) {
    const int j = e / D, r = e - j * D;
    Ys[(size_t)j * ldy + r] = Y[e];
  }
  for (int j0 = 0; j0 < k; j0 += ORTH_B) {
    const int cb = min(ORTH_B, k - j0);
    __syncthreads();
    for (int e = tid; e < D * ORTH_B; e += ORTH_NT) {
      const int r = e / ORTH_B, c = e - r * ORTH_B;
      Pb[e] = c < cb ? Ys[(size_t)(j0 + c) * ldy + r] : T(0);
    }
    __syncthreads();
    if (j0 > 0) {
      const int g = (j0 + 31) >> 5;        // groups of 32 finished columns
      const int S = ORTH_NW / g;           // row slices
      const int rows = (D + S - 1) / S;
      for (int pass = 0; pass < 2; ++pass) {
        // C = Q^T P: warp (grp, slice) forms 32 columns x ORTH_B partial dots
        const int grp = wid % g, slice = wid / g;
        const int i = grp * 32 + lane;
        if (slice < S && i < j0) {
          T acc[ORTH_B];
#pragma unroll
          for (int c = 0; c < ORTH_B; ++c) acc[c] = T(0);
          const int r0 = slice * rows, r1 = min(D, r0 + rows);
          const T* yi = Ys + (size_t)i * ldy;
#pragma unroll 4
          for (int r = r0; r < r1; ++r) {
            const T y = yi[r];
            T pv[ORTH_B];
            load_row8<T>(Pb + (size_t)r * ORTH_B, pv);
#pragma unroll
            for (int c = 0; c < ORTH_B; ++c) acc[c] = fma(y, pv[c], acc[c]);
          }
#pragma unroll
          for (int c = 0; c < ORTH_B; ++c) part[((size_t)slice * g * 32 + i) * ORTH_B + c] = acc[c];
        }
        __syncthreads();
        for (int e = tid; e < j0 * ORTH_B; e += ORTH_NT) {
          const int ii = e / ORTH_B, c = e - ii * ORTH_B;
          T x = T(0);
          for (int sl = 0; sl < S; ++sl) x += part[((size_t)sl * g * 32 + ii) * ORTH_B + c];
          C[e] = x;
        }
        __syncthreads();
        // P -= Q C, one row per thread
        for (int r = tid; r < D; r += ORTH_NT) {
          T v[ORTH_B];
          load_row8<T>(Pb + (size_t)r * ORTH_B, v);
#pragma unroll 4
          for (int ii = 0; ii < j0; ++ii) {
            const T y = Ys[(size_t)ii * ldy + r];
            T cc[ORTH_B];
            load_row8<T>(C + (size_t)ii * ORTH_B, cc);
#pragma unroll
            for (int c = 0; c < ORTH_B; ++c) v[c] = fma(-y, cc[c], v[c]);
          }
#pragma unroll
          for (int c = 0; c < ORTH_B; ++c) Pb[(size_t)r * ORTH_B + c] = v[c];
        }
        __syncthreads();
      }
    }
    // column CGS2 inside the panel by the first four warps (RPL >= 4, the
    // panel in registers, D <= 32 * RPL; reductions at a named barrier of
    // those warps) or by warp 0 alone (its sums are warp shuffles)
    if (RPL >= 4) {
      if (wid < 4) panel_cgs2_warps<T, (RPL >= 4 ? RPL / 4 : 1), 4>(Pb, D, cb, part);
    } else if (RPL > 0) {
      if (wid == 0) panel_cgs2_warp<T, (RPL > 0 ? RPL : 1)>(Pb, D, cb);
    } else if (wid == 0) {
      for (int c = 0; c < cb; ++c) {
        for (int pass = 0; pass < 2 && c > 0; ++pass) {
          T d[ORTH_B];
#pragma unroll
          for (int c2 = 0; c2 < ORTH_B; ++c2) d[c2] = T(0);
          for (int r = lane; r < D; r += 32) {
            T v[ORTH_B];
            load_row8<T>(Pb + (size_t)r * ORTH_B, v);
            const T vc = Pb[(size_t)r * ORTH_B + c];
#pragma unroll
            for (int c2 = 0; c2 < ORTH_B; ++c2)
              if (c2 < c) d[c2] = fma(v[c2], vc, d[c2]);
          }
#pragma unroll
          for (int c2 = 0; c2 < ORTH_B; ++c2)
            if (c2 < c)
#pragma unroll
              for (int o = 16; o > 0; o >>= 1) d[c2] += __shfl_xor_sync(0xffffffffu, d[c2], o);
          for (int r = lane; r < D; r += 32) {
            T v[ORTH_B];
            load_row8<T>(Pb + (size_t)r * ORTH_B, v);
            T x = Pb[(size_t)r * ORTH_B + c];
#pragma unroll
            for (int c2 = 0; c2 < ORTH_B; ++c2)
              if (c2 < c) x = fma(-d[c2], v[c2], x);
            Pb[(size_t)r * ORTH_B + c] = x;
          }
          __syncwarp();
        }
        T nq = T(0);
        for (int r = lane; r < D; r += 32) {
          const T x = Pb[(size_t)r * ORTH_B + c];
          nq = fma(x, x, nq);
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) nq += __shfl_xor_sync(0xffffffffu, nq, o);
        const T inv = nq > T(0) ? T(1) / sqrt(nq) : T(0);
        for (int r = lane; r < D; r += 32) Pb[(size_t)r * ORTH_B + c] *= inv;
        __syncwarp();
      }
    }
    __syncthreads();
    // finished panel back into Ys (fenced by the next barrier)
    for (int e = tid; e < D * cb; e += ORTH_NT) {
      const int c = e / D, r = e - c * D;
      Ys[(size_t)(j0 + c) * ldy + r] = Pb[(size_t)r * ORTH_B + c];
    }
  }
  __syncthreads();
  for (int e = tid; e < D * k; e += ORTH_NT) {
    const int j = e / D, r = e - j * D;
    Y[e] = Ys[(size_t)j * ldy + r];
  }
}

static size_t orth_smem_bytes(int D, int k, size_t es) {
  return (size_t)D * k * es + (size_t)(((k + 1) & ~1) + 2) * es + 16 + (TFX_THREADS / 32) * sizeof(double) + 16;
}

template <class T>
__global__ void __launch_bounds__(TFX_THREADS) k_orth(T* Y, int D, int k) {
  // arithmetic in the working precision T: GB300's FP64 rate is a small
  // fraction of its FP32 rate, and the second CGS pass restores orthogonality
  __shared__ T coef[1024];
  __shared__ double red[TFX_THREADS / 32];
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  for (int j = 0; j < k; ++j) {
    T* yj = Y + (size_t)j * D;
    for (int pass = 0; pass < 2; ++pass) {
      for (int i = wid; i < j; i += TFX_THREADS / 32) {
        const T* yi = Y + (size_t)i * D;
        T s = T(0);
        for (int r = lane; r < D; r += 32) s = fma(yi[r], yj[r], s);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (lane == 0) coef[i] = s;
      }
      __syncthreads();
      for (int r = tid; r < D; r += TFX_THREADS) {
        T v = yj[r];
        for (int i = 0; i < j; ++i) v = fma(-coef[i], Y[(size_t)i * D + r], v);
        yj[r] = v;
      }
      __syncthreads();
    }
    double s = 0.0;
    for (int r = tid; r < D; r += TFX_THREADS) s += (double)yj[r] * (double)yj[r];
    s = warp_sum(s);
    if (lane == 0) red[wid] = s;
    __syncthreads();
    double nrm = 0.0;
    for (int w = 0; w < TFX_THREADS / 32; ++w) nrm += red[w];
    nrm = sqrt(nrm);
    const T inv = (T)(nrm > 0.0 ? 1.0 / nrm : 0.0);
    for (int r = tid; r < D; r += TFX_THREADS) yj[r] = yj[r] * inv;
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// Symmetric eigensolver: cyclic Jacobi with the round-robin (tournament)
// ordering, n/2 disjoint rotations per round applied in parallel.  Input A
// (n x n, symmetric, row-major), output eigenvalues in descending order and
// the matching eigenvectors as columns of V (n x n, column-major).
// ---------------------------------------------------------------------------
template <class T>
__global__ void __launch_bounds__(512) k_jacobi(const T* __restrict__ Ain, int n, T* __restrict__ evals,
                                                        T* __restrict__ V, int max_sweeps, int* __restrict__ sweeps_out) {
  extern __shared__ __align__(16) char smem[];
  const int m = (n + 1) & ~1;  // even size (a zero row/column pads odd n)
  T* A = (T*)smem;             // m x m
  T* Vs = A + (size_t)m * m;   // m x m, column p at Vs[p*m]
  T* cs = Vs + (size_t)m * m;  // c[m/2], s[m/2]
  int* pr = (int*)(cs + m);    // pairs
  double* red = (double*)(pr + m + 2);
  unsigned* blk = (unsigned*)(red + 2);  // (m/2)(m/2+1)/2 block indices
  const int hb = m / 2;
  // the second parameter slot of the pipelined sweep: c, s then the pairs
  T* cs2 = (T*)(((uintptr_t)(blk + hb * (hb + 1) / 2) + 15) & ~(uintptr_t)15);
  int* pr2 = (int*)(cs2 + m);
  const int tid = threadIdx.x;
  for (int e = tid; e < m * m; e += blockDim.x) {
    const int i = e / m, j = e - i * m;
    // symmetrised on load: Rayleigh-Ritz matrices arrive symmetric only up to rounding
    A[e] = (i < n && j < n) ? (T)(0.5 * ((double)Ain[i * n + j] + (double)Ain[j * n + i])) : T(0);
    Vs[e] = (i == j) ? T(1) : T(0);
  }
  __syncthreads();
  const int sweep = cta_jacobi<T>(A, Vs, cs, pr, red, m, max_sweeps, blk, cs2, pr2);
  // sort eigenvalues (descending) with their vectors
  for (int i = tid; i < n; i += blockDim.x) {
    const int rank = eig_rank<T>(A, m, n, i);
    evals[rank] = A[i * m + i];
    for (int r = 0; r < n; ++r) V[(size_t)rank * n + r] = Vs[i * m + r];
  }
  if (tid == 0 && sweeps_out) *sweeps_out = sweep;
}

// ---------------------------------------------------------------------------
// Column signs: the entry of largest magnitude (first one on ties) of every
// column of U (D x n, column-major) becomes positive.
// ---------------------------------------------------------------------------
template <class T>
__global__ void k_flip_signs(T* U, int D, int n) {
  const int lane = threadIdx.x & 31;
  const int col = blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5);
  if (col >= n) return;
  T* u = U + (size_t)col * D;
  double best = -1.0;
  int bi = 0;
  for (int r = lane; r < D; r += 32) {
    const double a = fabs((double)u[r]);
    if (a > best) {
      best = a;
      bi = r;
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    const double ob = __shfl_xor_sync(0xffffffffu, best, o);
    const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
    if (ob > best || (ob == best && oi < bi)) {
      best = ob;
      bi = oi;
    }
  }
  const bool neg = u[bi] < T(0);
  if (neg)
    for (int r = lane; r < D; r += 32) u[r] = -u[r];
}

// ---------------------------------------------------------------------------
// ||T - [[W]]||^2, T C-order (d0, Q0) with Q0 = prod_{l>0} d_l; W in the flat
// column-major factor layout.  Partial sums per block, then one fixed-order sum.
// ---------------------------------------------------------------------------
struct CpShape {
  int L, R;
  int d[TFX_MAX_ORDER];
  int off[TFX_MAX_ORDER];
};

template <class T, int TS>
__global__ void __launch_bounds__(TFX_THREADS) k_cp_residual(const T* __restrict__ Tt, const T* __restrict__ W,
                                                             CpShape sh, double* __restrict__ partial) {
  using TL = Tile<TS, TS>;
  __shared__ T sA[TFX_BK * TL::LDA];
  __shared__ T sB[TFX_BK * TL::LDB];
  __shared__ int sIdx[TL::BN * TFX_MAX_ORDER];
  __shared__ double red[TFX_THREADS / 32];
  const int L = sh.L, R = sh.R, d0 = sh.d[0];
  long long Q0 = 1;
  for (int l = 1; l < L; ++l) Q0 *= sh.d[l];
  const int tm_ = (d0 + TL::BM - 1) / TL::BM;
  const long long ntiles = (long long)tm_ * ((Q0 + TL::BN - 1) / TL::BN);
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  double part = 0.0;
  for (long long t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const int m0 = (int)(t % tm_) * TL::BM;
    const long long q0 = (t / tm_) * TL::BN;
    if (tid < TL::BN) {
      long long q = q0 + tid;
      if (q < Q0)
        for (int l = L - 1; l >= 1; --l) {
          sIdx[tid * TFX_MAX_ORDER + l] = (int)(q % sh.d[l]);
          q /= sh.d[l];
        }
    }
    __syncthreads();
    T acc[TS][TS];
    tile_zero<T, TS, TS>(acc);
    for (int k0 = 0; k0 < R; k0 += TFX_BK) {
      const int kc = min(TFX_BK, R - k0);
      for (int e = tid; e < TFX_BK * TL::BM; e += TFX_THREADS) {
        const int kk = e / TL::BM, mm = e - kk * TL::BM;
        sA[kk * TL::LDA + mm] = (kk < kc && m0 + mm < d0) ? W[sh.off[0] + (k0 + kk) * d0 + m0 + mm] : T(0);
      }
      for (int e = tid; e < TFX_BK * TL::BN; e += TFX_THREADS) {
        const int kk = e / TL::BN, nn = e - kk * TL::BN;
        T v = T(0);
        if (kk < kc && q0 + nn < Q0) {
          v = T(1);
          for (int l = L - 1; l >= 1; --l) v *= W[sh.off[l] + (k0 + kk) * sh.d[l] + sIdx[nn * TFX_MAX_ORDER + l]];
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
        if (m < d0 && q < Q0) {
          const T df = Tt[(long long)m * Q0 + q] - acc[u][v];
          ps = fma(df, df, ps);
        }
      }
    part += (double)ps;
  }
  part = warp_sum(part);
  if ((tid & 31) == 0) red[tid >> 5] = part;
  __syncthreads();
  if (tid == 0) {
    double s = 0.0;
    for (int w = 0; w < TFX_THREADS / 32; ++w) s += red[w];
    partial[blockIdx.x] = s;
  }
}

template <class T>
__global__ void k_tensor_norms(const T* __restrict__ Tt, long long N, double* __restrict__ partial) {
  __shared__ double red[2][TFX_THREADS / 32];
  // compensated accumulation in the working precision (FP64 per element would
  // run at GB300's FP64 rate)
  // 16-byte loads, four of them in flight per thread (independent
  // accumulators), so the read runs at HBM speed rather than at one
  // outstanding scalar load per thread
  Acc<T> a2, a1, b2, b1;
  constexpr int V = 16 / sizeof(T);  // elements per 16-byte vector
  const bool vec = (((uintptr_t)Tt) & 15) == 0;
  const long long nv = vec ? N / V : 0;
  const long long stride = (long long)gridDim.x * TFX_THREADS;
  long long e = (long long)blockIdx.x * TFX_THREADS + threadIdx.x;
  if constexpr (sizeof(T) == 4) {
    const float4* p = (const float4*)Tt;
    for (; e + stride < nv; e += 2 * stride) {
      const float4 u = __ldg(p + e), w = __ldg(p + e + stride);
      a2.fma_((T)u.x, (T)u.x); a1.add(fabs((T)u.x)); b2.fma_((T)w.x, (T)w.x); b1.add(fabs((T)w.x));
      a2.fma_((T)u.y, (T)u.y); a1.add(fabs((T)u.y)); b2.fma_((T)w.y, (T)w.y); b1.add(fabs((T)w.y));
      a2.fma_((T)u.z, (T)u.z); a1.add(fabs((T)u.z)); b2.fma_((T)w.z, (T)w.z); b1.add(fabs((T)w.z));
      a2.fma_((T)u.w, (T)u.w); a1.add(fabs((T)u.w)); b2.fma_((T)w.w, (T)w.w); b1.add(fabs((T)w.w));
    }
    for (; e < nv; e += stride) {
      const float4 u = __ldg(p + e);
      a2.fma_((T)u.x, (T)u.x); a1.add(fabs((T)u.x));
      a2.fma_((T)u.y, (T)u.y); a1.add(fabs((T)u.y));
      a2.fma_((T)u.z, (T)u.z); a1.add(fabs((T)u.z));
      a2.fma_((T)u.w, (T)u.w); a1.add(fabs((T)u.w));
    }
  } else {
    const double2* p = (const double2*)Tt;
    for (; e + stride < nv; e += 2 * stride) {
      const double2 u = __ldg(p + e), w = __ldg(p + e + stride);
      a2.fma_((T)u.x, (T)u.x); a1.add(fabs((T)u.x)); b2.fma_((T)w.x, (T)w.x); b1.add(fabs((T)w.x));
      a2.fma_((T)u.y, (T)u.y); a1.add(fabs((T)u.y)); b2.fma_((T)w.y, (T)w.y); b1.add(fabs((T)w.y));
    }
    for (; e < nv; e += stride) {
      const double2 u = __ldg(p + e);
      a2.fma_((T)u.x, (T)u.x); a1.add(fabs((T)u.x));
      a2.fma_((T)u.y, (T)u.y); a1.add(fabs((T)u.y));
    }
  }
  // the scalar tail (and the whole tensor when it is not 16-byte aligned)
  for (long long t = nv * V + (long long)blockIdx.x * TFX_THREADS + threadIdx.x; t < N; t += stride) {
    const T v = __ldg(Tt + t);
    a2.fma_(v, v);
    a1.add(fabs(v));
  }
  a2.add(b2.hi_or_v());
  a2.add(b2.lo_or_0());
  a1.add(b1.hi_or_v());
  a1.add(b1.lo_or_0());
  a2.warp_reduce();
  a1.warp_reduce();
  if ((threadIdx.x & 31) == 0) {
    red[0][threadIdx.x >> 5] = a2.value();
    red[1][threadIdx.x >> 5] = a1.value();
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0.0, b = 0.0;
    for (int w = 0; w < TFX_THREADS / 32; ++w) {
      a += red[0][w];
      b += red[1][w];
    }
    partial[2 * blockIdx.x] = a;
    partial[2 * blockIdx.x + 1] = b;
  }
}

// fixed-order sum of `n` partials with stride `stride` into out[0..stride)
__global__ void k_sum_partials(const double* __restrict__ partial, int n, int stride, double* __restrict__ out) {
  if (threadIdx.x < stride) {
    double s = 0.0;
    for (int i = 0; i < n; ++i) s += partial[(size_t)i * stride + threadIdx.x];
    out[threadIdx.x] = s;
  }
}

}  // namespace tfx

// ============================================================================
// C ABI
// ============================================================================
using namespace tfx;

static int g_num_sms = 0;
static int num_sms() {
  if (g_num_sms == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&g_num_sms, cudaDevAttrMultiProcessorCount, dev);
    if (g_num_sms <= 0) g_num_sms = 1;
  }
  return g_num_sms;
}

static int check_launch(const char* where) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return tfx_set_cuda_error(e, where);
  tfx_count_launch(1);
  return TFX_STATUS_OK;
}

extern "C" size_t tfx_mode_gram_scratch_bytes(int dtype, long long P, int D, long long Q) {
  const int BM = 64;
  const int nt = (D + BM - 1) / BM;
  const long long tiles = (long long)nt * (nt + 1) / 2;
  const long long K = P * Q;
  long long ks = (4LL * num_sms() + tiles - 1) / tiles;
  const long long kmax = (K + 255) / 256;
  if (ks > kmax) ks = kmax;
  if (ks < 1) ks = 1;
  if (ks > 64) ks = 64;
  return (size_t)ks * D * D * (dtype == TFX_F64 ? 8 : 4);
}

extern "C" int tfx_mode_gram(int dtype, const void* S, long long P, int D, long long Q, void* G, void* scratch,
                             size_t scratch_bytes, void* stream) {
  if (!S || !G || !scratch || P < 1 || D < 1 || Q < 1) return tfx_set_error(TFX_STATUS_ERR_ARG, "mode_gram args");
  const size_t es = dtype == TFX_F64 ? 8 : 4;
  const int BM = 64;
  const int nt = (D + BM - 1) / BM;
  const long long tiles = (long long)nt * (nt + 1) / 2;
  int ks = (int)(scratch_bytes / ((size_t)D * D * es));
  const size_t want = tfx_mode_gram_scratch_bytes(dtype, P, D, Q) / ((size_t)D * D * es);
  if ((size_t)ks > want) ks = (int)want;
  if (ks < 1) return tfx_set_error(TFX_STATUS_ERR_ARG, "mode_gram scratch too small");
  cudaStream_t st = (cudaStream_t)stream;
  dim3 grid((unsigned)tiles, (unsigned)ks);
  const long long n = (long long)D * D;
  const int rb = (int)std::min<long long>((n + 255) / 256, 4LL * num_sms());
  if (dtype == TFX_F32) {
    k_mode_gram<float, 4><<<grid, TFX_THREADS, 0, st>>>((const float*)S, P, D, Q, ks, (float*)scratch);
    int s = check_launch("mode_gram");
    if (s) return s;
    k_gram_reduce<float, 64><<<rb, 256, 0, st>>>((const float*)scratch, D, ks, (float*)G);
  } else {
    k_mode_gram<double, 4><<<grid, TFX_THREADS, 0, st>>>((const double*)S, P, D, Q, ks, (double*)scratch);
    int s = check_launch("mode_gram");
    if (s) return s;
    k_gram_reduce<double, 64><<<rb, 256, 0, st>>>((const double*)scratch, D, ks, (double*)G);
  }
  return check_launch("gram_reduce");
}

// ---------------------------------------------------------------------------
// C = alpha A B + beta C for a short left factor (M <= 64 rows) and a long K:
// the eigen-step's products (60 x 512 by 512 x 512, 60 x 512 by 512 x 60).  A
// CTA owns SK_NB columns of C and every row; its 256 threads are 64 rows x 4
// quarters of each K chunk, each accumulating SK_NB outputs, and the four
// quarter sums are added in a fixed order at the end.  One output per thread
// over all of K (the general kernel's smallest tile) leaves a 512-long
// dependent chain per thread.
// ---------------------------------------------------------------------------
#define SK_NB 16
#define SK_KC 128

template <class T>
__global__ void __launch_bounds__(256) k_gemm_skinny(const T* __restrict__ A, const T* __restrict__ B, T* C,
                                                     GemmArgs g) {
  extern __shared__ __align__(16) char sk_smem[];
  T* As = (T*)sk_smem;                         // [64][SK_KC + 1]
  T* Bs = As + 64 * (SK_KC + 1);               // [SK_KC][SK_NB]
  T* red = Bs + SK_KC * SK_NB;                 // [4][64][SK_NB]
  const int tid = threadIdx.x, row = tid & 63, kq = tid >> 6;
  const long long n0 = (long long)blockIdx.x * SK_NB;
  const int M = (int)g.M;
  T acc[SK_NB];
#pragma unroll
  for (int j = 0; j < SK_NB; ++j) acc[j] = T(0);
  for (long long k0 = 0; k0 < g.K; k0 += SK_KC) {
    const int kc = (int)(g.K - k0 < SK_KC ? g.K - k0 : SK_KC);
    // the chunk's operands: every load of a thread issued before any store
    // (one L2 round trip a chunk instead of one per element)
    constexpr int NA = 64 * SK_KC / 256, NB = SK_KC * SK_NB / 256;
    T ra[NA], rb[NB];
#pragma unroll
    for (int u = 0; u < NA; ++u) {
      const int e = tid + 256 * u, m = e / SK_KC, k = e - m * SK_KC;
      ra[u] = (m < M && k < kc) ? A[m * g.sAm + (k0 + k) * g.sAk] : T(0);
    }
#pragma unroll
    for (int u = 0; u < NB; ++u) {
      const int e = tid + 256 * u, k = e / SK_NB, j = e - k * SK_NB;
      rb[u] = (k < kc && n0 + j < g.N) ? B[(k0 + k) * g.sBk + (n0 + j) * g.sBn] : T(0);
    }
    __syncthreads();  // the previous chunk is consumed
#pragma unroll
    for (int u = 0; u < NA; ++u) {
      const int e = tid + 256 * u, m = e / SK_KC, k = e - m * SK_KC;
      As[m * (SK_KC + 1) + k] = ra[u];
    }
#pragma unroll
    for (int u = 0; u < NB; ++u) Bs[tid + 256 * u] = rb[u];
    __syncthreads();
    const T* ar = As + row * (SK_KC + 1) + kq * (SK_KC / 4);
    const T* br = Bs + kq * (SK_KC / 4) * SK_NB;
    // B's row as 16-byte reads (broadcast across the warp): 4 (FP32) or 8
    // (FP64) loads per k instead of 16
    using V = typename std::conditional<sizeof(T) == 4, float4, double2>::type;
    constexpr int PV = 16 / sizeof(T);
#pragma unroll 4
    for (int kk = 0; kk < SK_KC / 4; ++kk) {
      const T a = ar[kk];
      const V* bv = reinterpret_cast<const V*>(br + kk * SK_NB);
#pragma unroll
      for (int j4 = 0; j4 < SK_NB / PV; ++j4) {
        const V b = bv[j4];
        const T* bb = reinterpret_cast<const T*>(&b);
#pragma unroll
        for (int u = 0; u < PV; ++u) acc[j4 * PV + u] = fma(a, bb[u], acc[j4 * PV + u]);
      }
    }
  }
#pragma unroll
  for (int j = 0; j < SK_NB; ++j) red[(kq * 64 + row) * SK_NB + j] = acc[j];
  __syncthreads();
  for (int e = tid; e < 64 * SK_NB; e += 256) {
    const int m = e / SK_NB, j = e - m * SK_NB;
    if (m >= M || n0 + j >= g.N) continue;
    const T v = ((red[m * SK_NB + j] + red[(64 + m) * SK_NB + j]) + red[(128 + m) * SK_NB + j]) +
                red[(192 + m) * SK_NB + j];
    T* c = C + m * g.sCm + (n0 + j) * g.sCn;
    *c = g.beta != 0.0 ? (T)(g.alpha * (double)v + g.beta * (double)*c) : (T)(g.alpha * (double)v);
  }
}

static size_t skinny_smem(size_t es) {
  return (size_t)(64 * (SK_KC + 1) + SK_KC * SK_NB + 4 * 64 * SK_NB) * es;
}

extern "C" int tfx_gemm(int dtype, const void* A, const void* B, void* C, long long M, long long N, long long K,
                        long long batch, const long long* strides /* sAb sAm sAk sBb sBk sBn sCb sCm sCn */,
                        double alpha, double beta, void* stream) {
  if (!A || !B || !C || !strides || M < 1 || N < 1 || K < 0 || batch < 1)
    return tfx_set_error(TFX_STATUS_ERR_ARG, "gemm args");
  GemmArgs g;
  g.M = M;
  g.N = N;
  g.K = K;
  g.batch = batch;
  g.sAb = strides[0];
  g.sAm = strides[1];
  g.sAk = strides[2];
  g.sBb = strides[3];
  g.sBk = strides[4];
  g.sBn = strides[5];
  g.sCb = strides[6];
  g.sCm = strides[7];
  g.sCn = strides[8];
  g.alpha = alpha;
  g.beta = beta;
  cudaStream_t st = (cudaStream_t)stream;
  if (batch == 1 && M <= 64 && K >= 32 && N <= 65535LL * SK_NB) {
    const size_t sm = skinny_smem(dtype == TFX_F32 ? 4 : 8);
    const unsigned grid = (unsigned)((N + SK_NB - 1) / SK_NB);
    cudaError_t e;
    if (dtype == TFX_F32) {
      e = cudaFuncSetAttribute(k_gemm_skinny<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
      if (e != cudaSuccess) return tfx_set_cuda_error(e, "gemm_skinny smem");
      k_gemm_skinny<float><<<grid, 256, sm, st>>>((const float*)A, (const float*)B, (float*)C, g);
    } else {
      e = cudaFuncSetAttribute(k_gemm_skinny<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
      if (e != cudaSuccess) return tfx_set_cuda_error(e, "gemm_skinny smem");
      k_gemm_skinny<double><<<grid, 256, sm, st>>>((const double*)A, (const double*)B, (double*)C, g);
    }
    return check_launch("gemm_skinny");
  }
  // smaller tiles when the output is too small to fill the GPU with 64x64 tiles
  int ts = 4;
  const long long by = std::min<long long>(batch, 65535);
  while (ts > 1) {
    const long long b = 16LL * ts;
    if (((M + b - 1) / b) * ((N + b - 1) / b) * by >= 2LL * num_sms()) break;
    ts >>= 1;
  }
  const long long bs = 16LL * ts;
  const long long tiles = ((M + bs - 1) / bs) * ((N + bs - 1) / bs);
  if (tiles > 0x7fffffffLL) return tfx_set_error(TFX_STATUS_ERR_ARG, "gemm too large");
  dim3 grid((unsigned)tiles, (unsigned)by);
  if (dtype == TFX_F32) {
    if (ts == 4) k_gemm<float, 4><<<grid, TFX_THREADS, 0, st>>>((const float*)A, (const float*)B, (float*)C, g);
    else if (ts == 2) k_gemm<float, 2><<<grid, TFX_THREADS, 0, st>>>((const float*)A, (const float*)B, (float*)C, g);
    else k_gemm<float, 1><<<grid, TFX_THREADS, 0, st>>>((const float*)A, (const float*)B, (float*)C, g);
  } else {
    if (ts == 4) k_gemm<double, 4><<<grid, TFX_THREADS, 0, st>>>((const double*)A, (const double*)B, (double*)C, g);
    else if (ts == 2) k_gemm<double, 2><<<grid, TFX_THREADS, 0, st>>>((const double*)A, (const double*)B, (double*)C, g);
    else k_gemm<double, 1><<<grid, TFX_THREADS, 0, st>>>((const double*)A, (const double*)B, (double*)C, g);
  }
  return check_launch("gemm");
}

extern "C" int tfx_ttm(int dtype, const void* S, long long P, int D, long long Q, const void* Ut, int n, void* out,
                       void* stream) {
  if (!S || !Ut || !out || P < 1 || D < 1 || Q < 1 || n < 1) return tfx_set_error(TFX_STATUS_ERR_ARG, "ttm args");
  cudaStream_t st = (cudaStream_t)stream;
  const bool vec = dtype == TFX_F32 && D % 4 == 0 && Q % 4 == 0 && ((uintptr_t)S & 15) == 0 &&
                   ((uintptr_t)Ut & 15) == 0 && ((uintptr_t)out & 15) == 0;
  if (vec && Q >= 128) {
    const int rows = n < 64 ? n : 64;
    const int nw = (rows + 7) / 8;
    const int mt = (n + 8 * nw - 1) / (8 * nw);
    // wide tiles when there are enough of them to fill the GPU twice over
    const bool wide = ((Q + 255) / 256) * P * mt >= 2LL * num_sms();
    const long long tq = wide ? (Q + 255) / 256 : (Q + 127) / 128;
    if (tq > 2147483647LL) return tfx_set_error(TFX_STATUS_ERR_UNSUPPORTED, "ttm too wide");
    dim3 grid((unsigned)tq, (unsigned)(P < 65535 ? P : 65535), (unsigned)mt);
    if (wide)
      k_ttm_f32<8><<<grid, 32 * nw, 0, st>>>((const float*)Ut, (const float*)S, (float*)out, n, D, Q, P);
    else
      k_ttm_f32<4><<<grid, 32 * nw, 0, st>>>((const float*)Ut, (const float*)S, (float*)out, n, D, Q, P);
    return check_launch("ttm");
  }
  // general shapes: strided batched GEMM, batched over p (Q >= 16) or over q
  long long sd[9];
  if (Q >= 16) {
    const long long t[9] = {0, D, 1, (long long)D * Q, Q, 1, (long long)n * Q, Q, 1};
    for (int i = 0; i < 9; ++i) sd[i] = t[i];
    return tfx_gemm(dtype, Ut, S, out, n, Q, D, P, sd, 1.0, 0.0, stream);
  }
  const long long t[9] = {1, (long long)D * Q, Q, 0, 1, D, 1, (long long)n * Q, Q};
  for (int i = 0; i < 9; ++i) sd[i] = t[i];
  return tfx_gemm(dtype, S, Ut, out, P, n, D, Q, sd, 1.0, 0.0, stream);
}

template <class T, int RPL>
static cudaError_t launch_orth(T* Y, int D, int k, size_t smb, cudaStream_t st) {
  cudaError_t e = cudaFuncSetAttribute(k_orth_bcgs<T, RPL>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smb);
  if (e != cudaSuccess) return e;
  k_orth_bcgs<T, RPL><<<1, ORTH_NT, smb, st>>>(Y, D, k);
  return cudaSuccess;
}

extern "C" int tfx_orthonormalize(int dtype, void* Y, int D, int k, void* stream) {
  if (!Y || D < 1 || k < 1 || k > 1024) return tfx_set_error(TFX_STATUS_ERR_ARG, "orthonormalize args");
  cudaStream_t st = (cudaStream_t)stream;
  const size_t es = dtype == TFX_F64 ? 8 : 4;
  size_t oP, oPart, oC, oRed;
  const size_t smb = dtype == TFX_F32 ? orth_bcgs_offsets<float>(D, k, &oP, &oPart, &oC, &oRed)
                                      : orth_bcgs_offsets<double>(D, k, &oP, &oPart, &oC, &oRed);
  if (smb <= 220 * 1024 && k <= 32 * ORTH_NW) {
    cudaError_t e = cudaSuccess;
    if (dtype == TFX_F32) {
      if (D <= 128) e = launch_orth<float, 4>((float*)Y, D, k, smb, st);
      else if (D <= 256) e = launch_orth<float, 8>((float*)Y, D, k, smb, st);
      else if (D <= 512) e = launch_orth<float, 16>((float*)Y, D, k, smb, st);
      else e = launch_orth<float, 0>((float*)Y, D, k, smb, st);
    } else {
      if (D <= 128) e = launch_orth<double, 4>((double*)Y, D, k, smb, st);
      else if (D <= 256) e = launch_orth<double, 8>((double*)Y, D, k, smb, st);
      else e = launch_orth<double, 0>((double*)Y, D, k, smb, st);
    }
    if (e != cudaSuccess) return tfx_set_cuda_error(e, "orth attr");
    return check_launch("orthonormalize");
  }
  const size_t sm = orth_smem_bytes(D, k, es);
  if (sm <= 200 * 1024) {
    cudaError_t e;
    if (dtype == TFX_F32) {
      e = cudaFuncSetAttribute(k_orth_smem<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
      if (e != cudaSuccess) return tfx_set_cuda_error(e, "orth attr");
      k_orth_smem<float><<<1, TFX_THREADS, sm, st>>>((float*)Y, D, k);
    } else {
      e = cudaFuncSetAttribute(k_orth_smem<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
      if (e != cudaSuccess) return tfx_set_cuda_error(e, "orth attr");
      k_orth_smem<double><<<1, TFX_THREADS, sm, st>>>((double*)Y, D, k);
    }
    return check_launch("orthonormalize");
  }
  if (dtype == TFX_F32)
    k_orth<float><<<1, TFX_THREADS, 0, st>>>((float*)Y, D, k);
  else
    k_orth<double><<<1, TFX_THREADS, 0, st>>>((double*)Y, D, k);
  return check_launch("orthonormalize");
}

extern "C" size_t tfx_sym_eig_smem_bytes(int dtype, int n) {
  const int m = (n + 1) & ~1;
  const size_t es = dtype == TFX_F64 ? 8 : 4;
  size_t b = 2 * (size_t)m * m * es + (size_t)m * es + (size_t)(m + 2) * sizeof(int);
  b = (b + 15) & ~(size_t)15;
  const size_t h = (size_t)m / 2;
  return b + 2 * (TFX_THREADS / 32) * sizeof(double) + h * (h + 1) / 2 * sizeof(unsigned) + 16 + (size_t)m * es +
         (size_t)(m + 2) * sizeof(int);
}

extern "C" int tfx_sym_eig(int dtype, const void* A, int n, void* evals, void* V, int max_sweeps, int* sweeps,
                           void* stream) {
  if (!A || !evals || !V || n < 1) return tfx_set_error(TFX_STATUS_ERR_ARG, "sym_eig args");
  const size_t sm = tfx_sym_eig_smem_bytes(dtype, n);
  if (sm > 220 * 1024) return tfx_set_error(TFX_STATUS_ERR_UNSUPPORTED, "sym_eig matrix too large");
  cudaStream_t st = (cudaStream_t)stream;
  cudaError_t e;
  if (dtype == TFX_F32) {
    e = cudaFuncSetAttribute(k_jacobi<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return tfx_set_cuda_error(e, "sym_eig attr");
    k_jacobi<float><<<1, 512, sm, st>>>((const float*)A, n, (float*)evals, (float*)V, max_sweeps, sweeps);
  } else {
    e = cudaFuncSetAttribute(k_jacobi<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return tfx_set_cuda_error(e, "sym_eig attr");
    k_jacobi<double><<<1, 512, sm, st>>>((const double*)A, n, (double*)evals, (double*)V, max_sweeps, sweeps);
  }
  return check_launch("sym_eig");
}

extern "C" int tfx_flip_signs(int dtype, void* U, int D, int n, void* stream) {
  if (!U || D < 1 || n < 1) return tfx_set_error(TFX_STATUS_ERR_ARG, "flip_signs args");
  cudaStream_t st = (cudaStream_t)stream;
  const int blocks = (n + 7) / 8;
  if (dtype == TFX_F32)
    k_flip_signs<float><<<blocks, 256, 0, st>>>((float*)U, D, n);
  else
    k_flip_signs<double><<<blocks, 256, 0, st>>>((double*)U, D, n);
  return check_launch("flip_signs");
}

extern "C" size_t tfx_cp_residual_scratch_bytes(void) { return (size_t)8 * (8 * 1024 + 8); }

namespace tfx {
__global__ void k_nan_if_flag(const int* err, double* out) {
  if (*err) *out = nan("");
}
}  // namespace tfx
int tfx_cp_residual_tc_launch(const float* T, const int* dims, int R, const float* W, double* partial,
                              int max_partials, int* err, int* nblocks, cudaStream_t st);

// ---------------------------------------------------------------------------
// FP32 ||T - [[W]]||^2 as a register-tiled GEMM with the Khatri-Rao operand
// generated on the fly.  A block owns 256 columns q of the other modes: it
// forms their Khatri-Rao rows once (R x 256, shared memory, R <= 64), then
// walks every row tile of mode 0: the model tile (8 rows per warp, 8 x 8
// outputs per lane as in k_ttm_f32) = W_0 (rows x R) KR^T (R x 256), and the
// epilogue subtracts the streamed tensor tile and accumulates squares in
// float-float.  Block partials are summed in FP64 by k_sum_partials.
// ---------------------------------------------------------------------------
constexpr int RES_BN = 256, RES_RMAX = 64;

__global__ void __launch_bounds__(256, 2) k_cp_residual_f32(const float* __restrict__ Tt, const float* __restrict__ W,
                                                            CpShape sh, long long Q0, double* __restrict__ partial) {
  constexpr int TN = 8, BN = RES_BN, AKS = RES_RMAX + 4;
  extern __shared__ __align__(16) float res_sm[];
  float* sKR = res_sm;                      // [RES_RMAX][BN]
  float* sA = sKR + RES_RMAX * BN;          // [64][AKS]
  __shared__ int sIdx[BN][TFX_MAX_ORDER];
  __shared__ double red[8];
  __shared__ int sD[TFX_MAX_ORDER], sOff[TFX_MAX_ORDER];  // shape, indexed at run time
  const int nw = blockDim.x >> 5, nt = blockDim.x;
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
#pragma unroll
  for (int l = 0; l < TFX_MAX_ORDER; ++l)
    if (tid == l) {
      sD[l] = sh.d[l];
      sOff[l] = sh.off[l];
    }
  const int L = sh.L, R = sh.R, d0 = sh.d[0];
  const int Rp = (R + 3) & ~3;
  const int BM = 8 * nw;
  const long long qt = (Q0 + BN - 1) / BN;
  Acc<float> acc2;
  for (long long t = blockIdx.x; t < qt; t += gridDim.x) {
    const long long q0 = t * BN;
    __syncthreads();  // shape copied; the previous tile's readers are done
    for (int c = tid; c < BN; c += nt) {
      long long q = q0 + c;
      if (q >= Q0) q = Q0 - 1;  // padding columns repeat a valid one; their terms are skipped
      for (int l = L - 1; l >= 1; --l) {
        sIdx[c][l] = (int)(q % sD[l]);
        q /= sD[l];
      }
    }
    __syncthreads();
    for (int e = tid; e < Rp * BN; e += nt) {
      const int r = e / BN, c = e - r * BN;
      float v = 0.f;
      if (r < R) {
        v = 1.f;
        for (int l = 1; l < L; ++l) v *= __ldg(W + sOff[l] + (size_t)r * sD[l] + sIdx[c][l]);
      }
      sKR[r * BN + c] = v;
    }
    for (int m0 = 0; m0 < d0; m0 += BM) {
      __syncthreads();  // KR rows ready / the previous row tile's W_0 slab consumed
      for (int e = tid; e < BM * Rp; e += nt) {
        const int m = e / Rp, r = e - m * Rp;
        sA[m * AKS + r] = (m0 + m < d0 && r < R) ? __ldg(W + (size_t)r * d0 + m0 + m) : 0.f;
      }
      __syncthreads();
      float acc[8][TN];
#pragma unroll
      for (int i = 0; i < 8; ++i)
#pragma unroll
        for (int j = 0; j < TN; ++j) acc[i][j] = 0.f;
      for (int k4 = 0; k4 < Rp; k4 += 4) {
        float4 a[8];
#pragma unroll
        for (int i = 0; i < 8; ++i) a[i] = *(const float4*)&sA[(wid * 8 + i) * AKS + k4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          float bv[TN];
#pragma unroll
          for (int j4 = 0; j4 < TN / 4; ++j4) {
            const float4 v = *(const float4*)&sKR[(k4 + u) * BN + j4 * 128 + lane * 4];
            bv[4 * j4 + 0] = v.x;
            bv[4 * j4 + 1] = v.y;
            bv[4 * j4 + 2] = v.z;
            bv[4 * j4 + 3] = v.w;
          }
#pragma unroll
          for (int i = 0; i < 8; ++i) {
            const float ai = u == 0 ? a[i].x : u == 1 ? a[i].y : u == 2 ? a[i].z : a[i].w;
#pragma unroll
            for (int j = 0; j < TN; ++j) acc[i][j] = fmaf(ai, bv[j], acc[i][j]);
          }
        }
      }
      // epilogue: the tensor tile (4 consecutive q per read when aligned)
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        const int m = m0 + wid * 8 + i;
        if (m >= d0) continue;
#pragma unroll
        for (int j4 = 0; j4 < TN / 4; ++j4) {
          const long long q = q0 + j4 * 128 + lane * 4;
          const float* tp = Tt + (long long)m * Q0 + q;
          if (q + 3 < Q0 && ((((unsigned long long)tp) & 15) == 0)) {
            const float4 tv = __ldcs(reinterpret_cast<const float4*>(tp));
            const float e0 = tv.x - acc[i][4 * j4], e1 = tv.y - acc[i][4 * j4 + 1];
            const float e2 = tv.z - acc[i][4 * j4 + 2], e3 = tv.w - acc[i][4 * j4 + 3];
            acc2.fma_(e0, e0);
            acc2.fma_(e1, e1);
            acc2.fma_(e2, e2);
            acc2.fma_(e3, e3);
          } else {
#pragma unroll
            for (int u = 0; u < 4; ++u)
              if (q + u < Q0) {
                const float df = __ldcs(tp + u) - acc[i][4 * j4 + u];
                acc2.fma_(df, df);
              }
          }
        }
      }
    }
  }
  acc2.warp_reduce();
  if (lane == 0) red[wid] = acc2.value();
  __syncthreads();
  if (tid == 0) {
    double sum = 0.0;
    for (int w = 0; w < nw; ++w) sum += red[w];
    partial[blockIdx.x] = sum;
  }
}

extern "C" int tfx_cp_residual(int dtype, const void* T, int L, const int* dims, int R, const void* W, double* out,
                               void* scratch, void* stream) {
  if (!T || !dims || !W || !out || !scratch || L < 2 || L > TFX_MAX_ORDER || R < 1)
    return tfx_set_error(TFX_STATUS_ERR_ARG, "cp_residual args");
  CpShape sh;
  sh.L = L;
  sh.R = R;
  int s = 0;
  long long Q0 = 1;
  for (int l = 0; l < L; ++l) {
    sh.d[l] = dims[l];
    sh.off[l] = R * s;
    s += dims[l];
    if (l) Q0 *= dims[l];
  }
  cudaStream_t st = (cudaStream_t)stream;
  double* partial = (double*)scratch;
  if (dtype == TFX_F32 && L == 3 && R <= 64) {
    // tensor-core path (residual_tc.cu); its bounded-wait flag sits in the
    // scratch's last slot and turns the result into NaN if a wait ran out
    int* err = (int*)((char*)scratch + tfx_cp_residual_scratch_bytes() - sizeof(double));
    cudaError_t ce = cudaMemsetAsync(err, 0, sizeof(int), st);
    if (ce != cudaSuccess) return tfx_set_cuda_error(ce, "cp_residual flag");
    int nb = 0;
    const int r = tfx_cp_residual_tc_launch((const float*)T, dims, R, (const float*)W, partial, 8 * 1024, err, &nb, st);
    if (r == TFX_STATUS_OK) {
      k_sum_partials<<<1, 32, 0, st>>>(partial, nb, 1, out);
      int c = check_launch("sum_partials");
      if (c) return c;
      k_nan_if_flag<<<1, 1, 0, st>>>(err, out);
      return check_launch("cp_residual flag");
    }
    if (r != TFX_STATUS_ERR_UNSUPPORTED) return r;
  }
  if (dtype == TFX_F32 && Q0 >= RES_BN && R <= RES_RMAX) {
    const int rows = dims[0] < 64 ? dims[0] : 64;
    const int nw = (rows + 7) / 8;
    const long long tiles = (Q0 + RES_BN - 1) / RES_BN;
    const int blocks = (int)std::max<long long>(1, std::min<long long>(tiles, 2LL * num_sms()));
    const size_t smb = ((size_t)RES_RMAX * RES_BN + 64 * (RES_RMAX + 4)) * sizeof(float);
    cudaError_t e = cudaFuncSetAttribute(k_cp_residual_f32, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smb);
    if (e != cudaSuccess) return tfx_set_cuda_error(e, "cp_residual attr");
    k_cp_residual_f32<<<blocks, 32 * nw, smb, st>>>((const float*)T, (const float*)W, sh, Q0, partial);
    int r = check_launch("cp_residual");
    if (r) return r;
    k_sum_partials<<<1, 32, 0, st>>>(partial, blocks, 1, out);
    return check_launch("sum_partials");
  }
  const long long tiles = ((dims[0] + 63) / 64) * ((Q0 + 63) / 64);
  const int blocks = (int)std::max<long long>(1, std::min<long long>(tiles, 8LL * num_sms()));
  if (dtype == TFX_F32)
    k_cp_residual<float, 4><<<blocks, TFX_THREADS, 0, st>>>((const float*)T, (const float*)W, sh, partial);
  else
    k_cp_residual<double, 4><<<blocks, TFX_THREADS, 0, st>>>((const double*)T, (const double*)W, sh, partial);
  int r = check_launch("cp_residual");
  if (r) return r;
  k_sum_partials<<<1, 32, 0, st>>>(partial, blocks, 1, out);
  return check_launch("sum_partials");
}

extern "C" int tfx_tensor_norms(int dtype, const void* T, long long N, double* out2, void* scratch, void* stream) {
  if (!T || !out2 || !scratch || N < 1) return tfx_set_error(TFX_STATUS_ERR_ARG, "tensor_norms args");
  const int blocks = (int)std::max<long long>(1, std::min<long long>((N + 255) / 256, 4LL * num_sms()));
  cudaStream_t st = (cudaStream_t)stream;
  double* partial = (double*)scratch;
  if (dtype == TFX_F32)
    k_tensor_norms<float><<<blocks, TFX_THREADS, 0, st>>>((const float*)T, N, partial);
  else
    k_tensor_norms<double><<<blocks, TFX_THREADS, 0, st>>>((const double*)T, N, partial);
  int r = check_launch("tensor_norms");
  if (r) return r;
  k_sum_partials<<<1, 32, 0, st>>>(partial, blocks, 2, out2);
  return check_launch("sum_partials");
}

// ============================================================================
// Allocation-free mode Gram.
//
// Some callers cannot allocate device memory when they call us: a host that
// lets another framework own all device memory through its own pool (a
// cudaMalloc from us would fail or fragment that pool), code on a
// latency-critical path that cannot afford cudaMalloc's implicit
// synchronisation, or services that forbid any allocation after start-up.
// For them tfx_mode_gram_noalloc takes its split-K scratch from a fixed array
// compiled into this library instead of from a caller buffer.
//
// * The array has TFX_NOALLOC_SCRATCH_BYTES (32 MiB).  Every GPU that loads the
//   library holds it until the process exits.
// * The first call on each device looks up the array's device address with
//   cudaGetSymbolAddress while that device is current (the symbol's host-side
//   name is not a device address).  That first call on a device should come
//   before any stream capture.  The address is cached per device together with
//   the device's current context; when that context changes (after
//   cudaDeviceReset, or a new primary context on the ordinal) the next call
//   looks the address up again instead of reusing the destroyed context's.
// * Every call shares the one array: calls that overlap on the GPU (other
//   streams, other host threads) race on it.  The kernels overwrite every
//   scratch entry they later read, so nothing needs clearing between calls.
// ============================================================================
#include <mutex>

#define TFX_NOALLOC_SCRATCH_BYTES (32u << 20)
#define TFX_NOALLOC_MAX_DEVICES 64

static __device__ __align__(256) unsigned char g_noalloc_gram_scratch[TFX_NOALLOC_SCRATCH_BYTES];

static std::mutex g_noalloc_mu;
static void* g_noalloc_addr[TFX_NOALLOC_MAX_DEVICES] = {nullptr};
static void* g_noalloc_ctx[TFX_NOALLOC_MAX_DEVICES] = {nullptr};

// the driver's current context (cuCtxGetCurrent), resolved through the runtime
// so that only the CUDA runtime is linked
typedef int (*CtxGetCurrentFn)(void**);
static CtxGetCurrentFn ctx_get_current_fn() {
  static CtxGetCurrentFn fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (CtxGetCurrentFn)p;
  });
  return fn;
}

static int noalloc_scratch_address(void** out) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return tfx_set_cuda_error(e, "mode_gram_noalloc: current device");
  if (dev < 0 || dev >= TFX_NOALLOC_MAX_DEVICES)
    return tfx_set_error(TFX_STATUS_ERR_UNSUPPORTED, "mode_gram_noalloc: device ordinal above 63");
  CtxGetCurrentFn get = ctx_get_current_fn();
  if (!get) return tfx_set_error(TFX_STATUS_ERR_CUDA, "mode_gram_noalloc: cuCtxGetCurrent unavailable");
  void* ctx = nullptr;
  if (get(&ctx) != 0) ctx = nullptr;  // null before the runtime has bound this device's context
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (g_noalloc_addr[dev] == nullptr || ctx == nullptr || g_noalloc_ctx[dev] != ctx) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_gram_scratch);  // binds the primary context if needed
    if (e != cudaSuccess || p == nullptr)
      return tfx_set_cuda_error(e == cudaSuccess ? cudaErrorInvalidSymbol : e, "mode_gram_noalloc: scratch address");
    if (get(&ctx) != 0) ctx = nullptr;  // a null context is never matched, so the lookup repeats
    g_noalloc_addr[dev] = p;
    g_noalloc_ctx[dev] = ctx;
  }
  *out = g_noalloc_addr[dev];
  return TFX_STATUS_OK;
}

extern "C" size_t tfx_mode_gram_noalloc_capacity_bytes(void) { return TFX_NOALLOC_SCRATCH_BYTES; }

extern "C" int tfx_mode_gram_noalloc(int dtype, const void* S, long long P, int D, long long Q, void* G, void* stream) {
  if (!S || !G || P < 1 || D < 1 || Q < 1) return tfx_set_error(TFX_STATUS_ERR_ARG, "mode_gram_noalloc args");
  if (dtype != TFX_F32 && dtype != TFX_F64) return tfx_set_error(TFX_STATUS_ERR_ARG, "mode_gram_noalloc dtype");
  const size_t es = dtype == TFX_F64 ? 8 : 4;
  // one D x D partial must fit: D <= 2896 in float32, D <= 2048 in float64
  if ((size_t)D * (size_t)D * es > (size_t)TFX_NOALLOC_SCRATCH_BYTES)
    return tfx_set_error(TFX_STATUS_ERR_ARG,
                         "mode_gram_noalloc: D*D*element size exceeds the 32 MiB built-in scratch "
                         "(D <= 2896 for float32, D <= 2048 for float64); use tfx_mode_gram with a caller buffer");
  void* scratch = nullptr;
  const int s = noalloc_scratch_address(&scratch);
  if (s) return s;
  return tfx_mode_gram(dtype, S, P, D, Q, G, scratch, TFX_NOALLOC_SCRATCH_BYTES, stream);
}
