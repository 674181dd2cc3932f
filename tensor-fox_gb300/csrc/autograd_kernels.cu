// Kernels of the differentiable CP layer (forward: reconstruction / fit loss;
// backward: MTTKRP).
//
//   tfx_mttkrp     M_l = T_(l) (W_{L-1} o ... o W_{l+1} o W_{l-1} o ... o W_0), any
//                  order, grid-level split-K (GaussNewton.py:401-427 compute_grad's
//                  product); the Khatri-Rao rows are generated in shared memory
//                  from the factors, never stored
//   tfx_cp_full    the dense tensor [[W_0, ..., W_{L-1}]] (Conversion.py:52-79 cpd2tens)
//   tfx_cp_wp1     W_l P1_l with P1_l = o_{m != l} W_m^T W_m for every mode
//                  (GaussNewton.py:520-548, :424)
// Factors use the flat column-major layout; outputs of tfx_mttkrp and tfx_cp_wp1
// are (d_l x R) column-major.
#include <math.h>

#include <algorithm>

#include "tfx_capi_internal.h"
#include "tfx_common.cuh"

namespace tfx {

struct CpDims {
  int L, R;
  int d[TFX_MAX_ORDER];
  int off[TFX_MAX_ORDER];
};

template <class T, int TS>
__global__ void __launch_bounds__(TFX_THREADS) k_mttkrp(const T* __restrict__ Tt, const T* __restrict__ W, CpDims sh,
                                                        int l, int ksplit, T* __restrict__ part) {
  using TL = Tile<TS, TS>;
  __shared__ T sA[TFX_BK * TL::LDA];
  __shared__ T sB[TFX_BK * TL::LDB];
  __shared__ long long sBase[TFX_BK];
  __shared__ int sIdx[TFX_BK * TFX_MAX_ORDER];
  const int L = sh.L, R = sh.R, D = sh.d[l];
  long long P = 1, Q = 1;
  for (int m = 0; m < l; ++m) P *= sh.d[m];
  for (int m = l + 1; m < L; ++m) Q *= sh.d[m];
  const int tilesM = (D + TL::BM - 1) / TL::BM;
  const int m0 = (blockIdx.x % tilesM) * TL::BM;
  const int n0 = (blockIdx.x / tilesM) * TL::BN;
  const long long K = P * Q;
  const long long kb = K * blockIdx.y / ksplit, ke = K * (blockIdx.y + 1) / ksplit;
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  T acc[TS][TS];
  tile_zero<T, TS, TS>(acc);
  for (long long k0 = kb; k0 < ke; k0 += TFX_BK) {
    const int kc = (int)min((long long)TFX_BK, ke - k0);
    if (tid < kc) {
      // k = p*Q + q; p and q decompose into the indices of the other modes
      long long k = k0 + tid, q = k % Q, p = k / Q, base = 0, stride = 1;
      for (int m = L - 1; m > l; --m) {
        const long long im = q % sh.d[m];
        q /= sh.d[m];
        sIdx[tid * TFX_MAX_ORDER + m] = (int)im;
        base += im * stride;
        stride *= sh.d[m];
      }
      stride *= D;
      for (int m = l - 1; m >= 0; --m) {
        const long long im = p % sh.d[m];
        p /= sh.d[m];
        sIdx[tid * TFX_MAX_ORDER + m] = (int)im;
        base += im * stride;
        stride *= sh.d[m];
      }
      sBase[tid] = base;
    }
    __syncthreads();
    for (int e = tid; e < TFX_BK * TL::BM; e += TFX_THREADS) {
      int kk, mm;
      if (Q > 1) {
        mm = e / TFX_BK;
        kk = e - mm * TFX_BK;
      } else {
        kk = e / TL::BM;
        mm = e - kk * TL::BM;
      }
      sA[kk * TL::LDA + mm] = (kk < kc && m0 + mm < D) ? __ldg(Tt + sBase[kk] + (long long)(m0 + mm) * Q) : T(0);
    }
    for (int e = tid; e < TFX_BK * TL::BN; e += TFX_THREADS) {
      const int kk = e / TL::BN, nn = e - kk * TL::BN;
      T v = T(0);
      if (kk < kc && n0 + nn < R) {
        v = T(1);
        for (int m = L - 1; m >= 0; --m)
          if (m != l) v *= W[sh.off[m] + (n0 + nn) * sh.d[m] + sIdx[kk * TFX_MAX_ORDER + m]];
      }
      sB[kk * TL::LDB + nn] = v;
    }
    __syncthreads();
    tile_fma<T, TS, TS>(sA, sB, acc, kc);
    __syncthreads();
  }
  T* out = part + (size_t)blockIdx.y * D * R;
#pragma unroll
  for (int u = 0; u < TS; ++u)
#pragma unroll
    for (int v = 0; v < TS; ++v) {
      const int i = m0 + ty + 16 * u, r = n0 + tx + 16 * v;
      if (i < D && r < R) out[(size_t)r * D + i] = acc[u][v];
    }
}

// ---------------------------------------------------------------------------
// Short-mode MTTKRP (d_l <= DM, R <= 256): the generic tile kernel would run a
// 64-row tile for a handful of rows.  Here one CTA takes a contiguous chunk of
// the contraction index k (the multi-index of the other modes, k = p*Q + q),
// stages TFX_THREADS of them at a time (indices and the d_l tensor values
// T[p, :, q], loaded coalesced across k), and its threads, split into
// k-groups x R, accumulate acc[i] += T[p, i, q] * KR[k, r] with the Khatri-Rao
// value formed once per (k, r) from a row-major copy of the factors (reads
// coalesced across r).  Per-CTA partials (d_l x R column-major) are summed in
// k order by k_sum_parts.
// ---------------------------------------------------------------------------
template <class T, int DM>
__global__ void __launch_bounds__(TFX_THREADS) k_mttkrp_short(const T* __restrict__ Tt, const T* __restrict__ Wrm,
                                                              CpDims sh, int l, int ksplit, T* __restrict__ part) {
  constexpr int KC = TFX_THREADS;
  __shared__ T sT[KC * DM];
  __shared__ int sIdx[KC * TFX_MAX_ORDER];
  const int L = sh.L, R = sh.R, D = sh.d[l];
  long long P = 1, Q = 1;
  for (int m = 0; m < l; ++m) P *= sh.d[m];
  for (int m = l + 1; m < L; ++m) Q *= sh.d[m];
  const long long K = P * Q;
  const long long kb = K * blockIdx.x / ksplit, ke = K * (blockIdx.x + 1) / ksplit;
  const int tid = threadIdx.x;
  const int G = TFX_THREADS / R;  // k-groups (R <= TFX_THREADS)
  const int g = tid / R, r = tid - g * R;
  const bool act = g < G;
  T acc[DM];
#pragma unroll
  for (int i = 0; i < DM; ++i) acc[i] = T(0);
  for (long long k0 = kb; k0 < ke; k0 += KC) {
    const int kc = (int)min((long long)KC, ke - k0);
    if (tid < kc) {
      long long k = k0 + tid, q = k % Q, p = k / Q, base = 0, stride = 1;
      for (int m = L - 1; m > l; --m) {
        const long long im = q % sh.d[m];
        q /= sh.d[m];
        sIdx[tid * TFX_MAX_ORDER + m] = (int)im;
        base += im * stride;
        stride *= sh.d[m];
      }
      stride *= D;
      for (int m = l - 1; m >= 0; --m) {
        const long long im = p % sh.d[m];
        p /= sh.d[m];
        sIdx[tid * TFX_MAX_ORDER + m] = (int)im;
        base += im * stride;
        stride *= sh.d[m];
      }
#pragma unroll
      for (int i = 0; i < DM; ++i)
        if (i < D) sT[tid * DM + i] = __ldg(Tt + base + (long long)i * Q);
    }
    __syncthreads();
    if (act)
      for (int kk = g; kk < kc; kk += G) {
        T kr = T(1);
        for (int m = L - 1; m >= 0; --m)
          if (m != l) kr *= Wrm[sh.off[m] + sIdx[kk * TFX_MAX_ORDER + m] * R + r];
#pragma unroll
        for (int i = 0; i < DM; ++i) acc[i] = fma(sT[kk * DM + i], kr, acc[i]);
      }
    __syncthreads();
  }
  // sum the k-groups through shared memory (sT is free now)
  if (act)
#pragma unroll
    for (int i = 0; i < DM; ++i) sT[(g * R + r) * DM + i] = acc[i];
  __syncthreads();
  T* out = part + (size_t)blockIdx.x * D * R;
  for (int e = tid; e < D * R; e += TFX_THREADS) {
    const int rr = e / D, i = e - rr * D;
    T s = T(0);
    for (int gg = 0; gg < G; ++gg) s += sT[(gg * R + rr) * DM + i];
    out[(size_t)rr * D + i] = s;
  }
}

// row-major copy of the flat column-major factors: Wrm[off_m + i*R + r] = W_m[i, r]
template <class T>
__global__ void k_factors_rowmajor(const T* __restrict__ W, CpDims sh, long long nx, T* __restrict__ Wrm) {
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nx) return;
  int m = 0;
  while (m + 1 < sh.L && e >= sh.off[m + 1]) ++m;
  const long long w = e - sh.off[m];
  const int d = sh.d[m];
  const long long r = w / d, i = w - r * d;
  Wrm[sh.off[m] + i * sh.R + r] = W[e];
}

template <class T>
__global__ void k_sum_parts(const T* __restrict__ part, long long n, int ks, T* __restrict__ out) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    Acc<T> s;
    for (int k = 0; k < ks; ++k) s.add(part[(size_t)k * n + i]);
    out[i] = (T)s.value();
  }
}

template <class T, int TS>
__global__ void __launch_bounds__(TFX_THREADS) k_cp_full(const T* __restrict__ W, CpDims sh, T* __restrict__ out) {
  using TL = Tile<TS, TS>;
  __shared__ T sA[TFX_BK * TL::LDA];
  __shared__ T sB[TFX_BK * TL::LDB];
  __shared__ int sIdx[TL::BN * TFX_MAX_ORDER];
  const int L = sh.L, R = sh.R, d0 = sh.d[0];
  long long Q0 = 1;
  for (int l = 1; l < L; ++l) Q0 *= sh.d[l];
  const int tm_ = (d0 + TL::BM - 1) / TL::BM;
  const long long ntiles = (long long)tm_ * ((Q0 + TL::BN - 1) / TL::BN);
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
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
#pragma unroll
    for (int u = 0; u < TS; ++u)
#pragma unroll
      for (int v = 0; v < TS; ++v) {
        const int m = m0 + ty + 16 * u;
        const long long q = q0 + tx + 16 * v;
        if (m < d0 && q < Q0) out[(long long)m * Q0 + q] = acc[u][v];
      }
  }
}

// Gramians of every mode, G_m = W_m^T W_m (FP64, compensated sums of the
// working-type products): grid L * ceil(R*R / 256), one entry per thread.
template <class T>
__global__ void __launch_bounds__(TFX_THREADS) k_cp_grams(const T* __restrict__ W, CpDims sh,
                                                          double* __restrict__ gram) {
  const int R = sh.R, RR = R * R;
  const int per = (RR + TFX_THREADS - 1) / TFX_THREADS;
  const int m = blockIdx.x / per;
  const int e = (blockIdx.x - m * per) * TFX_THREADS + threadIdx.x;
  if (e >= RR) return;
  const int a = e / R, b = e - a * R;
  if (a > b) return;
  const int d = sh.d[m];
  const T* wa = W + sh.off[m] + a * d;
  const T* wb = W + sh.off[m] + b * d;
  Acc<T> s;
  for (int i = 0; i < d; ++i) s.fma_(wa[i], wb[i]);
  const double v = s.value();
  gram[(size_t)m * RR + a * R + b] = v;
  gram[(size_t)m * RR + b * R + a] = v;
}

// out_l = scale (W_l P1_l - M_l), P1_l = o_{m != l} G_m (ascending m, FP64,
// rounded to the working type in shared memory); M == nullptr means M_l = 0.
// Grid (L, ceil(max d / 32)), 32 rows per CTA.
template <class T>
__global__ void __launch_bounds__(TFX_THREADS) k_cp_wp1(const T* __restrict__ W, CpDims sh,
                                                        const double* __restrict__ gram, const T* __restrict__ M,
                                                        T scale, T* __restrict__ out) {
  extern __shared__ __align__(16) char smem[];
  T* sP = (T*)smem;
  const int l = blockIdx.x, L = sh.L, R = sh.R, RR = R * R, tid = threadIdx.x;
  const int dl = sh.d[l], r0 = blockIdx.y * 32;
  if (r0 >= dl) return;
  for (int e = tid; e < RR; e += TFX_THREADS) {
    double p = 1.0;
    for (int m = 0; m < L; ++m)
      if (m != l) p *= gram[(size_t)m * RR + e];
    sP[e] = (T)p;
  }
  __syncthreads();
  const int nr = min(32, dl - r0);
  for (int e = tid; e < 32 * R; e += TFX_THREADS) {
    const int ii = e & 31, r = e >> 5;
    if (ii >= nr) continue;
    const int i = r0 + ii;
    Acc<T> s;
    for (int q = 0; q < R; ++q) s.fma_(W[sh.off[l] + q * dl + i], sP[q * R + r]);
    const size_t o = (size_t)sh.off[l] + (size_t)r * dl + i;
    if (M) s.add(-M[o]);
    out[o] = scale * (T)s.value();
  }
}

}  // namespace tfx

using namespace tfx;

static int nsm() {
  static int n = 0;
  if (!n) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    if (n < 1) n = 1;
  }
  return n;
}

static int cpdims(CpDims& sh, int L, const int* dims, int R) {
  if (L < 2 || L > TFX_MAX_ORDER || !dims || R < 1) return 1;
  sh.L = L;
  sh.R = R;
  int s = 0;
  for (int l = 0; l < L; ++l) {
    if (dims[l] < 1) return 1;
    sh.d[l] = dims[l];
    sh.off[l] = R * s;
    s += dims[l];
  }
  return 0;
}

static int done(const char* w) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return tfx_set_cuda_error(e, w);
  tfx_count_launch(1);
  return TFX_STATUS_OK;
}

static int mttkrp_splits(long long K, int D, int R, int dtype) {
  const long long tiles = (long long)((D + 63) / 64) * ((R + 63) / 64);
  long long ks = (4LL * nsm() + tiles - 1) / tiles;
  // FP64 runs at a small fraction of the FP32 rate on GB300: spread small
  // contractions over more SMs
  ks = std::min<long long>(ks, std::max<long long>(1, K / (dtype == TFX_F64 ? 32 : 128)));
  return (int)std::max<long long>(1, std::min<long long>(ks, 128));
}

// short modes: d_l <= 16 and R <= TFX_THREADS
static bool mttkrp_short(int D, int R) { return D <= 16 && R <= TFX_THREADS; }
static int mttkrp_short_splits(long long K) {
  return (int)std::max<long long>(1, std::min<long long>(4LL * nsm(), K / 1024));
}
static size_t al256(size_t v) { return (v + 255) & ~(size_t)255; }

extern "C" size_t tfx_mttkrp_scratch_bytes(int dtype, int L, const int* dims, int R, int mode) {
  if (L < 2 || L > TFX_MAX_ORDER || !dims || mode < 0 || mode >= L) return 0;
  long long K = 1, S = 0;
  for (int m = 0; m < L; ++m) {
    if (m != mode) K *= dims[m];
    S += dims[m];
  }
  const size_t es = dtype == TFX_F64 ? 8 : 4;
  if (mttkrp_short(dims[mode], R))  // partials, then the row-major factors
    return al256((size_t)mttkrp_short_splits(K) * dims[mode] * R * es) + (size_t)S * R * es;
  return (size_t)mttkrp_splits(K, dims[mode], R, dtype) * dims[mode] * R * es;
}

extern "C" int tfx_mttkrp(int dtype, const void* T, int L, const int* dims, int R, const void* W, int mode, void* out,
                          void* scratch, size_t scratch_bytes, void* stream) {
  CpDims sh;
  if (cpdims(sh, L, dims, R) || !T || !W || !out || !scratch || mode < 0 || mode >= L)
    return tfx_set_error(TFX_STATUS_ERR_ARG, "mttkrp args");
  long long K = 1;
  for (int m = 0; m < L; ++m)
    if (m != mode) K *= dims[m];
  const size_t es = dtype == TFX_F64 ? 8 : 4;
  const int D = dims[mode];
  cudaStream_t st0 = (cudaStream_t)stream;
  if (mttkrp_short(D, R)) {
    const int ks = mttkrp_short_splits(K);
    long long nx = 0;
    for (int m = 0; m < L; ++m) nx += (long long)dims[m] * R;
    const size_t pb = al256((size_t)ks * D * R * es);
    if (scratch_bytes < pb + (size_t)nx * es) return tfx_set_error(TFX_STATUS_ERR_ARG, "mttkrp scratch too small");
    void* Wrm = (char*)scratch + pb;
    const long long n = (long long)D * R;
    const int rb = (int)std::max<long long>(1, std::min<long long>((n + 255) / 256, 4LL * nsm()));
    const int xb = (int)((nx + 255) / 256);
    if (dtype == TFX_F32) {
      k_factors_rowmajor<float><<<xb, 256, 0, st0>>>((const float*)W, sh, nx, (float*)Wrm);
      if (int s = done("mttkrp rowmajor")) return s;
      if (D <= 4)
        k_mttkrp_short<float, 4><<<ks, TFX_THREADS, 0, st0>>>((const float*)T, (const float*)Wrm, sh, mode, ks,
                                                              (float*)scratch);
      else
        k_mttkrp_short<float, 16><<<ks, TFX_THREADS, 0, st0>>>((const float*)T, (const float*)Wrm, sh, mode, ks,
                                                               (float*)scratch);
      if (int s = done("mttkrp short")) return s;
      k_sum_parts<float><<<rb, 256, 0, st0>>>((const float*)scratch, n, ks, (float*)out);
    } else {
      k_factors_rowmajor<double><<<xb, 256, 0, st0>>>((const double*)W, sh, nx, (double*)Wrm);
      if (int s = done("mttkrp rowmajor")) return s;
      if (D <= 4)
        k_mttkrp_short<double, 4><<<ks, TFX_THREADS, 0, st0>>>((const double*)T, (const double*)Wrm, sh, mode, ks,
                                                               (double*)scratch);
      else
        k_mttkrp_short<double, 16><<<ks, TFX_THREADS, 0, st0>>>((const double*)T, (const double*)Wrm, sh, mode,
                                                                ks, (double*)scratch);
      if (int s = done("mttkrp short")) return s;
      k_sum_parts<double><<<rb, 256, 0, st0>>>((const double*)scratch, n, ks, (double*)out);
    }
    return done("mttkrp_sum");
  }
  int ks = mttkrp_splits(K, D, R, dtype);
  ks = (int)std::min<size_t>((size_t)ks, scratch_bytes / ((size_t)D * R * es));
  if (ks < 1) return tfx_set_error(TFX_STATUS_ERR_ARG, "mttkrp scratch too small");
  cudaStream_t st = (cudaStream_t)stream;
  const int tiles = ((D + 63) / 64) * ((R + 63) / 64);
  dim3 grid(tiles, ks);
  const long long n = (long long)D * R;
  const int rb = (int)std::max<long long>(1, std::min<long long>((n + 255) / 256, 4LL * nsm()));
  if (dtype == TFX_F32) {
    k_mttkrp<float, 4><<<grid, TFX_THREADS, 0, st>>>((const float*)T, (const float*)W, sh, mode, ks, (float*)scratch);
    if (int s = done("mttkrp")) return s;
    k_sum_parts<float><<<rb, 256, 0, st>>>((const float*)scratch, n, ks, (float*)out);
  } else {
    k_mttkrp<double, 4><<<grid, TFX_THREADS, 0, st>>>((const double*)T, (const double*)W, sh, mode, ks,
                                                      (double*)scratch);
    if (int s = done("mttkrp")) return s;
    k_sum_parts<double><<<rb, 256, 0, st>>>((const double*)scratch, n, ks, (double*)out);
  }
  return done("mttkrp_sum");
}

extern "C" int tfx_cp_full(int dtype, int L, const int* dims, int R, const void* W, void* out, void* stream) {
  CpDims sh;
  if (cpdims(sh, L, dims, R) || !W || !out) return tfx_set_error(TFX_STATUS_ERR_ARG, "cp_full args");
  long long Q0 = 1;
  for (int l = 1; l < L; ++l) Q0 *= dims[l];
  const long long tiles = ((dims[0] + 63) / 64) * ((Q0 + 63) / 64);
  const int blocks = (int)std::max<long long>(1, std::min<long long>(tiles, 8LL * nsm()));
  cudaStream_t st = (cudaStream_t)stream;
  if (dtype == TFX_F32)
    k_cp_full<float, 4><<<blocks, TFX_THREADS, 0, st>>>((const float*)W, sh, (float*)out);
  else
    k_cp_full<double, 4><<<blocks, TFX_THREADS, 0, st>>>((const double*)W, sh, (double*)out);
  return done("cp_full");
}

extern "C" size_t tfx_cp_wp1_scratch_bytes(int L, int R) { return (size_t)L * R * R * 8; }

extern "C" int tfx_cp_wp1(int dtype, int L, const int* dims, int R, const void* W, void* out, void* scratch,
                          void* stream) {
  CpDims sh;
  if (cpdims(sh, L, dims, R) || !W || !out || !scratch) return tfx_set_error(TFX_STATUS_ERR_ARG, "cp_wp1 args");
  cudaStream_t st = (cudaStream_t)stream;
  int maxd = 0;
  for (int l = 0; l < L; ++l) maxd = std::max(maxd, dims[l]);
  const int gb = L * ((R * R + TFX_THREADS - 1) / TFX_THREADS);
  const dim3 grid(L, (maxd + 31) / 32);
  const size_t es = dtype == TFX_F64 ? 8 : 4;
  const size_t smb = (size_t)R * R * es;
  if (smb > 200 * 1024) return tfx_set_error(TFX_STATUS_ERR_UNSUPPORTED, "cp_wp1: rank too large");
  cudaError_t e = dtype == TFX_F32
                      ? cudaFuncSetAttribute(k_cp_wp1<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smb)
                      : cudaFuncSetAttribute(k_cp_wp1<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smb);
  if (e != cudaSuccess) return tfx_set_cuda_error(e, "cp_wp1 attribute");
  if (dtype == TFX_F32) {
    k_cp_grams<float><<<gb, TFX_THREADS, 0, st>>>((const float*)W, sh, (double*)scratch);
    if (int r = done("cp_grams")) return r;
    k_cp_wp1<float><<<grid, TFX_THREADS, smb, st>>>((const float*)W, sh, (const double*)scratch, nullptr, 1.f,
                                                    (float*)out);
  } else {
    k_cp_grams<double><<<gb, TFX_THREADS, 0, st>>>((const double*)W, sh, (double*)scratch);
    if (int r = done("cp_grams")) return r;
    k_cp_wp1<double><<<grid, TFX_THREADS, smb, st>>>((const double*)W, sh, (const double*)scratch, nullptr, 1.0,
                                                     (double*)out);
  }
  return done("cp_wp1");
}

// grad_l = 2 (W_l P1_l - T_(l) KR_l) for every mode: the gradient of
// ||T - [[W]]||^2 (twice GaussNewton.py:401-427's g), flat layout.  Scratch:
// the Gramians, the MTTKRPs and the MTTKRP split-K partials.
struct FitGradLayout {
  size_t gram, M, mtt, mtt_bytes, total;
};
static FitGradLayout fit_grad_layout(int dtype, int L, const int* dims, int R) {
  const size_t es = dtype == TFX_F64 ? 8 : 4;
  long long nx = 0;
  size_t mtt = 0;
  for (int l = 0; l < L; ++l) {
    nx += (long long)dims[l] * R;
    mtt = std::max(mtt, tfx_mttkrp_scratch_bytes(dtype, L, dims, R, l));
  }
  FitGradLayout y;
  y.gram = 0;
  y.M = al256((size_t)L * R * R * 8);
  y.mtt = y.M + al256((size_t)nx * es);
  y.mtt_bytes = mtt;
  y.total = y.mtt + al256(mtt);
  return y;
}

extern "C" size_t tfx_cp_fit_grad_scratch_bytes(int dtype, int L, const int* dims, int R) {
  CpDims sh;
  if (cpdims(sh, L, dims, R)) return 0;
  return fit_grad_layout(dtype, L, dims, R).total;
}

extern "C" int tfx_cp_fit_grad(int dtype, const void* T, int L, const int* dims, int R, const void* W, void* grad,
                               void* scratch, size_t scratch_bytes, void* stream) {
  CpDims sh;
  if (cpdims(sh, L, dims, R) || !T || !W || !grad || !scratch) return tfx_set_error(TFX_STATUS_ERR_ARG, "cp_fit_grad args");
  const FitGradLayout y = fit_grad_layout(dtype, L, dims, R);
  if (scratch_bytes < y.total) return tfx_set_error(TFX_STATUS_ERR_ARG, "cp_fit_grad scratch too small");
  cudaStream_t st = (cudaStream_t)stream;
  const size_t es = dtype == TFX_F64 ? 8 : 4;
  char* sc = (char*)scratch;
  int maxd = 0;
  for (int l = 0; l < L; ++l) maxd = std::max(maxd, dims[l]);
  const size_t smb = (size_t)R * R * es;
  if (smb > 200 * 1024) return tfx_set_error(TFX_STATUS_ERR_UNSUPPORTED, "cp_fit_grad: rank too large");
  cudaError_t e = dtype == TFX_F32
                      ? cudaFuncSetAttribute(k_cp_wp1<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smb)
                      : cudaFuncSetAttribute(k_cp_wp1<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smb);
  if (e != cudaSuccess) return tfx_set_cuda_error(e, "cp_fit_grad attribute");
  const int gb = L * ((R * R + TFX_THREADS - 1) / TFX_THREADS);
  if (dtype == TFX_F32)
    k_cp_grams<float><<<gb, TFX_THREADS, 0, st>>>((const float*)W, sh, (double*)(sc + y.gram));
  else
    k_cp_grams<double><<<gb, TFX_THREADS, 0, st>>>((const double*)W, sh, (double*)(sc + y.gram));
  if (int r = done("cp_grams")) return r;
  for (int l = 0; l < L; ++l) {
    void* Ml = sc + y.M + (size_t)sh.off[l] * es;
    if (int r = tfx_mttkrp(dtype, T, L, dims, R, W, l, Ml, sc + y.mtt, y.mtt_bytes, stream)) return r;
  }
  const dim3 grid(L, (maxd + 31) / 32);
  if (dtype == TFX_F32)
    k_cp_wp1<float><<<grid, TFX_THREADS, smb, st>>>((const float*)W, sh, (const double*)(sc + y.gram),
                                                    (const float*)(sc + y.M), 2.f, (float*)grad);
  else
    k_cp_wp1<double><<<grid, TFX_THREADS, smb, st>>>((const double*)W, sh, (const double*)(sc + y.gram),
                                                     (const double*)(sc + y.M), 2.0, (double*)grad);
  return done("cp_fit_grad");
}
