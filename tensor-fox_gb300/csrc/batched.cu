// Batched kernels for many small dense CPDs (the workload of Tensor Fox's rank
// and statistics sweeps, TensorFox.py:820-1039, which call cpd in a loop).
//
//   tfx_batch_mlsvd      one CTA per problem runs the whole sequentially
//                        truncated MLSVD (Compression.py:141-156): per mode the
//                        Gram of the current core, a Jacobi eigensolver in
//                        shared memory (modes up to 64), svd_flip signs,
//                        clean_compression truncation and the mode product.
//   tfx_batch_decompress factors_l = U_l W_l per problem (TensorFox.py:573-574)
//   tfx_batch_residual   ||T - [[W]]||^2 and ||T||^2 per problem (Auxiliar.py:131-151)
//   tfx_batch_permute    per problem, the caller's tensor with its modes put in
//                        decreasing size (Auxiliar.py:93-115 sort_dims) on the device
//
// Problems are described by tfx_batch_problem (include/tfx_gb300_types.h).
#include <math.h>

#include <algorithm>

#include "../../include/tfx_gb300_types.h"
#include "linalg.cuh"
#include "tfx_capi_internal.h"
#include "tfx_common.cuh"

namespace tfx {

#define TFX_BATCH_MAXD 64

template <class T>
struct BatchSmem {
  T A[TFX_BATCH_MAXD * TFX_BATCH_MAXD];
  T V[TFX_BATCH_MAXD * TFX_BATCH_MAXD];
  T cs[TFX_BATCH_MAXD];
  int pr[TFX_BATCH_MAXD + 2];
  double red[2 * TFX_THREADS / 32];
  T Ut[TFX_BATCH_MAXD * TFX_BATCH_MAXD];
  T sA[TFX_BK * (TFX_BATCH_MAXD + 1)];
  double sig[TFX_BATCH_MAXD];
  int order[TFX_BATCH_MAXD];
  int misc[4];
};

template <class T>
__global__ void __launch_bounds__(TFX_THREADS) k_batch_mlsvd(const tfx_batch_problem* __restrict__ probs, int nprob,
                                                             double tol_mlsvd, int n_components) {
  extern __shared__ __align__(16) char smem_raw[];
  BatchSmem<T>& S = *reinterpret_cast<BatchSmem<T>*>(smem_raw);
  const int pid = blockIdx.x;
  if (pid >= nprob) return;
  const tfx_batch_problem pb = probs[pid];
  const int L = pb.L, R = pb.R, tid = threadIdx.x;
  int cur[TFX_MAX_ORDER];
  for (int l = 0; l < L; ++l) cur[l] = pb.dims[l];
  const T* src = (const T*)pb.tensor;
  T* bufs[2] = {(T*)pb.work, (T*)pb.work + pb.work_elems / 2};
  int ut_off = 0, sig_off = 0;
  using TL = Tile<4, 4>;
  for (int l = 0; l < L; ++l) {
    long long P = 1, Q = 1;
    for (int m = 0; m < l; ++m) P *= cur[m];
    for (int m = l + 1; m < L; ++m) Q *= cur[m];
    const int D = cur[l];
    const int mm = (D + 1) & ~1;
    // Gram G = S_(l) S_(l)^T into A (D <= 64: one 64 x 64 tile, split over K)
    {
      const int tx = tid & 15, ty = tid >> 4;
      T acc[4][4];
      tile_zero<T, 4, 4>(acc);
      const long long K = P * Q;
      for (long long k0 = 0; k0 < K; k0 += TFX_BK) {
        const int kc = (int)min((long long)TFX_BK, K - k0);
        for (int e = tid; e < TFX_BK * TL::BM; e += TFX_THREADS) {
          int kk, i;
          if (Q > 1) {
            i = e / TFX_BK;
            kk = e - i * TFX_BK;
          } else {
            kk = e / TL::BM;
            i = e - kk * TL::BM;
          }
          T v = T(0);
          if (kk < kc && i < D) {
            const long long k = k0 + kk, p = k / Q, q = k - p * Q;
            v = src[p * D * Q + (long long)i * Q + q];
          }
          S.sA[kk * TL::LDA + i] = v;
        }
        __syncthreads();
        tile_fma<T, 4, 4>(S.sA, S.sA, acc, kc);
        __syncthreads();
      }
      for (int e = tid; e < mm * mm; e += TFX_THREADS) {
        S.A[e] = T(0);
        S.V[e] = (e / mm == e % mm) ? T(1) : T(0);
      }
      __syncthreads();
#pragma unroll
      for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int v = 0; v < 4; ++v) {
          const int i = ty + 16 * u, j = tx + 16 * v;
          if (i < D && j < D) S.A[i * mm + j] = acc[u][v];
        }
      __syncthreads();
    }
    cta_jacobi<T>(S.A, S.V, S.cs, S.pr, S.red, mm, 40);
    int n = n_components > 0 ? n_components : min(R, pb.dims[l]);
    if (n > D) n = D;
    // order by descending eigenvalue
    for (int i = tid; i < D; i += TFX_THREADS) {
      const int rank = eig_rank<T>(S.A, mm, D, i);
      S.order[rank] = i;
    }
    __syncthreads();
    if (tid < n) {
      const double lam = (double)S.A[S.order[tid] * mm + S.order[tid]];
      S.sig[tid] = sqrt(lam > 0.0 ? lam : 0.0);
    }
    __syncthreads();
    // clean_compression (Compression.py:261-301)
    if (tid == 0) {
      double tot = 0.0;
      for (int i = 0; i < n; ++i) tot += S.sig[i] * S.sig[i];
      int dim = n;
      const double eps = tol_mlsvd / L;
      for (int i = 1; i < n; ++i) {
        double tail = 0.0;
        for (int j = i; j < n; ++j) tail += S.sig[j] * S.sig[j];
        if (tail / tot < eps) {
          dim = i;
          break;
        }
      }
      S.misc[0] = dim;
    }
    __syncthreads();
    const int dim = S.misc[0];
    // U^T rows with svd_flip signs (largest |entry| positive, first on ties)
    for (int j = tid >> 5; j < dim; j += TFX_THREADS / 32) {
      const int lane = tid & 31;
      const T* col = S.V + S.order[j] * mm;
      T best = T(-1);
      int bi = 0;
      for (int i = lane; i < D; i += 32) {
        const T a = fabs(col[i]);
        if (a > best) {
          best = a;
          bi = i;
        }
      }
      for (int o = 16; o > 0; o >>= 1) {
        const T ob = __shfl_xor_sync(0xffffffffu, best, o);
        const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
        if (ob > best || (ob == best && oi < bi)) {
          best = ob;
          bi = oi;
        }
      }
      const T sgn = col[bi] < T(0) ? T(-1) : T(1);
      for (int i = lane; i < D; i += 32) S.Ut[j * D + i] = sgn * col[i];
    }
    __syncthreads();
    T* ut_out = (T*)pb.Ut + ut_off;
    for (int e = tid; e < dim * D; e += TFX_THREADS) ut_out[e] = S.Ut[e];
    for (int j = tid; j < dim; j += TFX_THREADS) pb.sigma[sig_off + j] = S.sig[j];
    if (tid == 0) pb.core_dims[l] = dim;
    ut_off += dim * D;
    sig_off += n;
    // mode product: dst[p, j, q] = sum_i Ut[j, i] src[p, i, q]
    T* dst = (l == L - 1) ? (T*)pb.core : bufs[l & 1];
    for (long long pq = tid; pq < P * Q; pq += TFX_THREADS) {
      const long long p = pq / Q, q = pq - p * Q;
      const T* s = src + p * D * Q + q;
      T* o = dst + p * dim * Q + q;
      for (int j0 = 0; j0 < dim; j0 += 16) {  // 16 outputs in registers at a time
        T a[16];
#pragma unroll
        for (int j = 0; j < 16; ++j) a[j] = T(0);
        for (int i = 0; i < D; ++i) {
          const T v = s[(long long)i * Q];
#pragma unroll
          for (int j = 0; j < 16; ++j)
            if (j0 + j < dim) a[j] = fma(S.Ut[(j0 + j) * D + i], v, a[j]);
        }
#pragma unroll
        for (int j = 0; j < 16; ++j)
          if (j0 + j < dim) o[(long long)(j0 + j) * Q] = a[j];
      }
    }
    cur[l] = dim;
    src = dst;
    __syncthreads();
  }
}

// factors_l (d_l x R, column-major, flat layout) = U_l (d_l x n_l) Wc_l (n_l x R)
template <class T>
__global__ void k_batch_decompress(const tfx_batch_problem* __restrict__ probs, int nprob, const T* const* wcore,
                                   T* const* wfull) {
  const int pid = blockIdx.x;
  if (pid >= nprob) return;
  const tfx_batch_problem pb = probs[pid];
  const T* Ut = (const T*)pb.Ut;
  const T* Wc = wcore[pid];
  T* Wf = wfull[pid];
  int ut_off = 0, wc_off = 0, wf_off = 0;
  for (int l = 0; l < pb.L; ++l) {
    const int d = pb.dims[l], n = pb.core_dims[l];
    for (int e = threadIdx.x; e < d * pb.R; e += blockDim.x) {
      const int r = e / d, i = e - r * d;
      T acc = T(0);
      for (int j = 0; j < n; ++j) acc = fma(Ut[ut_off + j * d + i], Wc[wc_off + r * n + j], acc);
      Wf[wf_off + r * d + i] = acc;
    }
    ut_off += n * d;
    wc_off += n * pb.R;
    wf_off += d * pb.R;
  }
}

template <class T>
__global__ void __launch_bounds__(TFX_THREADS) k_batch_residual(const tfx_batch_problem* __restrict__ probs, int nprob,
                                                                T* const* wfull, double* __restrict__ out) {
  __shared__ double red[2][TFX_THREADS / 32];
  const int pid = blockIdx.x;
  if (pid >= nprob) return;
  const tfx_batch_problem pb = probs[pid];
  const T* Tt = (const T*)pb.tensor;
  const T* W = wfull[pid];
  int off[TFX_MAX_ORDER];
  long long N = 1;
  int s = 0;
  for (int l = 0; l < pb.L; ++l) {
    off[l] = s;
    s += pb.dims[l] * pb.R;
    N *= pb.dims[l];
  }
  Acc<T> res, nt;
  for (long long e = threadIdx.x; e < N; e += TFX_THREADS) {
    long long rem = e;
    int idx[TFX_MAX_ORDER];
    for (int l = pb.L - 1; l >= 0; --l) {
      idx[l] = (int)(rem % pb.dims[l]);
      rem /= pb.dims[l];
    }
    T model = T(0);
    for (int r = 0; r < pb.R; ++r) {
      T p = W[off[0] + r * pb.dims[0] + idx[0]];
      for (int l = 1; l < pb.L; ++l) p *= W[off[l] + r * pb.dims[l] + idx[l]];
      model += p;
    }
    const T t = Tt[e];
    const T df = t - model;
    res.fma_(df, df);
    nt.fma_(t, t);
  }
  res.warp_reduce();
  nt.warp_reduce();
  if ((threadIdx.x & 31) == 0) {
    red[0][threadIdx.x >> 5] = res.value();
    red[1][threadIdx.x >> 5] = nt.value();
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0.0, b = 0.0;
    for (int w = 0; w < TFX_THREADS / 32; ++w) {
      a += red[0][w];
      b += red[1][w];
    }
    out[2 * pid] = a;
    out[2 * pid + 1] = b;
  }
}

}  // namespace tfx

using namespace tfx;

static int batch_check(const tfx_batch_problem* h, int nprob) {
  if (!h || nprob < 1) return tfx_set_error(TFX_STATUS_ERR_ARG, "batch: no problems");
  for (int p = 0; p < nprob; ++p) {
    if (h[p].L < 2 || h[p].L > TFX_MAX_ORDER || h[p].R < 1) return tfx_set_error(TFX_STATUS_ERR_ARG, "batch: order/rank");
    long long N = 1;
    for (int l = 0; l < h[p].L; ++l) {
      if (h[p].dims[l] < 1 || h[p].dims[l] > TFX_BATCH_MAXD)
        return tfx_set_error(TFX_STATUS_ERR_ARG, "batch: every dimension must be in 1..64");
      N *= h[p].dims[l];
    }
    if (h[p].work_elems < 2 * N) return tfx_set_error(TFX_STATUS_ERR_ARG, "batch: work buffer too small");
    if (!h[p].tensor || !h[p].work || !h[p].Ut || !h[p].core || !h[p].core_dims || !h[p].sigma)
      return tfx_set_error(TFX_STATUS_ERR_ARG, "batch: null pointer");
  }
  return TFX_STATUS_OK;
}

extern "C" int tfx_batch_mlsvd(int dtype, const tfx_batch_problem* h_probs, tfx_batch_problem* d_probs, int nprob,
                               double tol_mlsvd, int n_components, void* stream) {
  if (int s = batch_check(h_probs, nprob)) return s;
  cudaStream_t st = (cudaStream_t)stream;
  cudaError_t e = cudaMemcpyAsync(d_probs, h_probs, sizeof(tfx_batch_problem) * nprob, cudaMemcpyHostToDevice, st);
  if (e != cudaSuccess) return tfx_set_cuda_error(e, "batch descriptors");
  if (dtype == TFX_F32) {
    const size_t sm = sizeof(BatchSmem<float>);
    e = cudaFuncSetAttribute(k_batch_mlsvd<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return tfx_set_cuda_error(e, "batch smem");
    k_batch_mlsvd<float><<<nprob, TFX_THREADS, sm, st>>>(d_probs, nprob, tol_mlsvd, n_components);
  } else {
    const size_t sm = sizeof(BatchSmem<double>);
    e = cudaFuncSetAttribute(k_batch_mlsvd<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return tfx_set_cuda_error(e, "batch smem");
    k_batch_mlsvd<double><<<nprob, TFX_THREADS, sm, st>>>(d_probs, nprob, tol_mlsvd, n_components);
  }
  e = cudaGetLastError();
  if (e != cudaSuccess) return tfx_set_cuda_error(e, "batch_mlsvd");
  tfx_count_launch(1);
  return TFX_STATUS_OK;
}

// One CTA per problem: dst (the problem's tensor, C-order over the sorted dims)
// gathers from src[p] (C-order over the caller's dims); perm[p*L + l] is the
// caller's axis that became sorted mode l.  Writes are coalesced; the strided
// reads stay within one small tensor (L2-resident).
template <class T>
__global__ void __launch_bounds__(256) k_batch_permute(const tfx_batch_problem* __restrict__ probs, int nprob,
                                                       const T* const* __restrict__ src, const int* __restrict__ perm) {
  const int p = blockIdx.x;
  if (p >= nprob) return;
  const tfx_batch_problem& q = probs[p];
  const int L = q.L;
  long long sstride[TFX_MAX_ORDER];   // caller's stride of sorted mode l
  long long ostr[TFX_MAX_ORDER];      // caller's C-order strides
  int odim[TFX_MAX_ORDER];
  for (int l = 0; l < L; ++l) {
    const int a = perm[p * L + l];
    if (a < 0 || a >= L) return;  // not a permutation of 0..L-1: leave the problem untouched
    odim[a] = q.dims[l];
  }
  long long s = 1;
  for (int a = L - 1; a >= 0; --a) {
    ostr[a] = s;
    s *= odim[a];
  }
  long long N = 1;
  for (int l = 0; l < L; ++l) {
    sstride[l] = ostr[perm[p * L + l]];
    N *= q.dims[l];
  }
  const T* in = src[p];
  T* out = (T*)q.tensor;
  for (long long e = threadIdx.x; e < N; e += blockDim.x) {
    long long r = e, off = 0;
    for (int l = L - 1; l >= 0; --l) {
      const long long i = r % q.dims[l];
      r /= q.dims[l];
      off += i * sstride[l];
    }
    out[e] = in[off];
  }
}

extern "C" int tfx_batch_permute(int dtype, const tfx_batch_problem* h_probs, tfx_batch_problem* d_probs, int nprob,
                                 const void* const* src_dev, const int* perm_dev, void* stream) {
  if (int s = batch_check(h_probs, nprob)) return s;
  if (!d_probs || !src_dev || !perm_dev) return tfx_set_error(TFX_STATUS_ERR_ARG, "batch_permute");
  cudaStream_t st = (cudaStream_t)stream;
  cudaError_t e = cudaMemcpyAsync(d_probs, h_probs, sizeof(tfx_batch_problem) * nprob, cudaMemcpyHostToDevice, st);
  if (e != cudaSuccess) return tfx_set_cuda_error(e, "batch descriptors");
  if (dtype == TFX_F32)
    k_batch_permute<float><<<nprob, 256, 0, st>>>(d_probs, nprob, (const float* const*)src_dev, perm_dev);
  else
    k_batch_permute<double><<<nprob, 256, 0, st>>>(d_probs, nprob, (const double* const*)src_dev, perm_dev);
  e = cudaGetLastError();
  if (e != cudaSuccess) return tfx_set_cuda_error(e, "batch_permute");
  tfx_count_launch(1);
  return TFX_STATUS_OK;
}

extern "C" int tfx_batch_decompress(int dtype, const tfx_batch_problem* d_probs, int nprob, const void* const* wcore_dev,
                                    void* const* wfull_dev, void* stream) {
  if (!d_probs || nprob < 1 || !wcore_dev || !wfull_dev) return tfx_set_error(TFX_STATUS_ERR_ARG, "batch_decompress");
  cudaStream_t st = (cudaStream_t)stream;
  if (dtype == TFX_F32)
    k_batch_decompress<float><<<nprob, 256, 0, st>>>(d_probs, nprob, (const float* const*)wcore_dev,
                                                     (float* const*)wfull_dev);
  else
    k_batch_decompress<double><<<nprob, 256, 0, st>>>(d_probs, nprob, (const double* const*)wcore_dev,
                                                      (double* const*)wfull_dev);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return tfx_set_cuda_error(e, "batch_decompress");
  tfx_count_launch(1);
  return TFX_STATUS_OK;
}

extern "C" int tfx_batch_residual(int dtype, const tfx_batch_problem* d_probs, int nprob, void* const* wfull_dev,
                                  double* out2, void* stream) {
  if (!d_probs || nprob < 1 || !wfull_dev || !out2) return tfx_set_error(TFX_STATUS_ERR_ARG, "batch_residual");
  cudaStream_t st = (cudaStream_t)stream;
  if (dtype == TFX_F32)
    k_batch_residual<float><<<nprob, TFX_THREADS, 0, st>>>(d_probs, nprob, (float* const*)wfull_dev, out2);
  else
    k_batch_residual<double><<<nprob, TFX_THREADS, 0, st>>>(d_probs, nprob, (double* const*)wfull_dev, out2);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return tfx_set_cuda_error(e, "batch_residual");
  tfx_count_launch(1);
  return TFX_STATUS_OK;
}
