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

// one CTA per mode l: P1_l = o_{m != l} W_m^T W_m (FP64), out_l = W_l P1_l
template <class T>
__global__ void __launch_bounds__(TFX_THREADS) k_cp_wp1(const T* __restrict__ W, CpDims sh, double* __restrict__ gram,
                                                        T* __restrict__ out) {
  const int l = blockIdx.x, L = sh.L, R = sh.R, tid = threadIdx.x;
  double* P1 = gram + (size_t)l * R * R;  // per-CTA scratch (R x R)
  for (int e = tid; e < R * R; e += TFX_THREADS) {
    const int a = e / R, b = e - a * R;
    double p = 1.0;
    for (int m = 0; m < L; ++m) {
      if (m == l) continue;
      const T* wa = W + sh.off[m] + a * sh.d[m];
      const T* wb = W + sh.off[m] + b * sh.d[m];
      Acc<T> s;
      for (int i = 0; i < sh.d[m]; ++i) s.fma_(wa[i], wb[i]);
      p *= s.value();
    }
    P1[e] = p;
  }
  __syncthreads();
  const int dl = sh.d[l];
  for (int e = tid; e < dl * R; e += TFX_THREADS) {
    const int r = e / dl, i = e - r * dl;
    Acc<T> s;
    for (int q = 0; q < R; ++q) s.fma_(W[sh.off[l] + q * dl + i], (T)P1[q * R + r]);
    out[sh.off[l] + r * dl + i] = (T)s.value();
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

static int mttkrp_splits(long long K, int D, int R) {
  const long long tiles = (long long)((D + 63) / 64) * ((R + 63) / 64);
  long long ks = (4LL * nsm() + tiles - 1) / tiles;
  ks = std::min<long long>(ks, std::max<long long>(1, K / 512));
  return (int)std::max<long long>(1, std::min<long long>(ks, 128));
}

extern "C" size_t tfx_mttkrp_scratch_bytes(int dtype, int L, const int* dims, int R, int mode) {
  if (L < 2 || L > TFX_MAX_ORDER || !dims || mode < 0 || mode >= L) return 0;
  long long K = 1;
  for (int m = 0; m < L; ++m)
    if (m != mode) K *= dims[m];
  return (size_t)mttkrp_splits(K, dims[mode], R) * dims[mode] * R * (dtype == TFX_F64 ? 8 : 4);
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
  int ks = mttkrp_splits(K, D, R);
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
  if (dtype == TFX_F32)
    k_cp_wp1<float><<<L, TFX_THREADS, 0, st>>>((const float*)W, sh, (double*)scratch, (float*)out);
  else
    k_cp_wp1<double><<<L, TFX_THREADS, 0, st>>>((const double*)W, sh, (double*)scratch, (double*)out);
  return done("cp_wp1");
}
