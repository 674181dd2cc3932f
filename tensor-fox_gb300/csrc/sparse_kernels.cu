// Sparse (COO) kernels of the dGN path.
//
//   tfx_coo_encode       int64 (nnz x L) coordinates -> int32 structure-of-arrays,
//                        bounds-checked (TensorFox.py:476-481 casts; the GPU keeps
//                        4-byte indices: nnz*(4L+4) bytes per pass in FP32)
//   tfx_coo_sort_mode    counting sort of the entries by their mode-l index
//                        (row pointers + physically permuted copy), the device
//                        counterpart of the CSR unfolding of Conversion.py:255-302
//   tfx_coo_mttkrp       M[i,:] = sum over the row's entries of v * prod_{m!=l} W_m[i_m,:]
//                        one warp per row, lanes reduce with shuffles (no atomics)
//   tfx_sparse_residual  sum over stored entries of (v - model)^2 (Critical.py:25-53)
//   tfx_coo_gram         dense T_(l) T_(l)^T from COO (Compression.py:211-215,
//                        MultilinearAlgebra.py:524-575): diagonal from the rows,
//                        off-diagonal from entries sharing a fibre (hash grouping)
//   tfx_sparse_ttmc      dense core S = T x_1 U_1^T ... x_L U_L^T from COO
//                        (MultilinearAlgebra.py:145-190, Critical.py:2703-2720)
//
// Factor matrices are read ROW-major here (d_l x R, a row of R values contiguous)
// so that the gather of one factor row per entry touches R*4 contiguous bytes.
#include <math.h>

#include <cuda_bf16.h>

#include <algorithm>

#include "tfx_capi_internal.h"
#include "tfx_common.cuh"

namespace tfx {

struct CooShape {
  int L, R;
  int dims[TFX_MAX_ORDER];
};

// ---------------------------------------------------------------------------
__global__ void k_coo_encode(const long long* __restrict__ idx64, long long nnz, int L, CooShape sh,
                             int* __restrict__ idx32, int* __restrict__ err) {
  for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < nnz; k += (long long)gridDim.x * blockDim.x) {
    for (int l = 0; l < L; ++l) {
      const long long v = idx64[k * L + l];
      if (v < 0 || v >= sh.dims[l]) {
        atomicExch(err, 1);
        idx32[(size_t)l * nnz + k] = 0;
      } else {
        idx32[(size_t)l * nnz + k] = (int)v;
      }
    }
  }
}

// counting sort by the mode-l index -------------------------------------------
__global__ void k_count_rows(const int* __restrict__ rows, long long nnz, int* __restrict__ counts) {
  for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < nnz; k += (long long)gridDim.x * blockDim.x)
    atomicAdd(counts + rows[k], 1);
}

// exclusive scan of n counts into rowptr[0..n] with one CTA (chunked)
__global__ void k_scan_counts(const int* __restrict__ counts, int n, long long* __restrict__ rowptr) {
  __shared__ long long part[TFX_THREADS];
  __shared__ long long carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int base = 0; base < n; base += TFX_THREADS * 8) {
    // each thread sums 8 consecutive counts
    long long loc[8];
    long long s = 0;
    for (int j = 0; j < 8; ++j) {
      const int i = base + threadIdx.x * 8 + j;
      loc[j] = i < n ? counts[i] : 0;
      s += loc[j];
    }
    part[threadIdx.x] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
      long long run = carry;
      for (int t = 0; t < TFX_THREADS; ++t) {
        const long long v = part[t];
        part[t] = run;
        run += v;
      }
      carry = run;
    }
    __syncthreads();
    long long run = part[threadIdx.x];
    for (int j = 0; j < 8; ++j) {
      const int i = base + threadIdx.x * 8 + j;
      if (i < n) rowptr[i] = run;
      run += loc[j];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) rowptr[n] = carry;
}

template <class T>
__global__ void k_scatter_rows(const int* __restrict__ idx32, const T* __restrict__ vals, long long nnz, int L, int mode,
                               const long long* __restrict__ rowptr, int* __restrict__ cursor,
                               int* __restrict__ sidx, T* __restrict__ svals) {
  const int* rows = idx32 + (size_t)mode * nnz;
  for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < nnz; k += (long long)gridDim.x * blockDim.x) {
    const int row = rows[k];
    const long long pos = rowptr[row] + atomicAdd(cursor + row, 1);
    svals[pos] = vals[k];
    for (int l = 0; l < L; ++l) sidx[(size_t)l * nnz + pos] = idx32[(size_t)l * nnz + k];
  }
}

// ---------------------------------------------------------------------------
// COO MTTKRP on a row-sorted copy.  One warp per row; each lane keeps RB
// partial sums (float-float on the FP32 path, so the result does not depend
// on the order in which the counting sort placed the row's entries).
// ---------------------------------------------------------------------------
template <class T, int RB>
__global__ void __launch_bounds__(256) k_coo_mttkrp(const int* __restrict__ sidx, const T* __restrict__ svals,
                                                    long long nnz, const long long* __restrict__ rowptr, CooShape sh,
                                                    int mode, const T* const* __restrict__ Wrow, T* __restrict__ out,
                                                    int r0) {
  const int lane = threadIdx.x & 31;
  const int warps = (gridDim.x * blockDim.x) >> 5;
  const int d = sh.dims[mode];
  const int R = sh.R;
  for (int row = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; row < d; row += warps) {
    const long long b = rowptr[row], e = rowptr[row + 1];
    Acc<T> acc[RB];
    for (long long k = b + lane; k < e; k += 32) {
      T p[RB];
      const T v = svals[k];
#pragma unroll
      for (int j = 0; j < RB; ++j) p[j] = v;
      for (int m = 0; m < sh.L; ++m) {
        if (m == mode) continue;
        const T* w = Wrow[m] + (size_t)sidx[(size_t)m * nnz + k] * R + r0;
#pragma unroll
        for (int j = 0; j < RB; ++j)
          if (r0 + j < R) p[j] *= w[j];
      }
#pragma unroll
      for (int j = 0; j < RB; ++j) acc[j].add(p[j]);
    }
#pragma unroll
    for (int j = 0; j < RB; ++j) {
      acc[j].warp_reduce();
      if (lane == j && r0 + j < R) out[(size_t)row * R + r0 + j] = (T)acc[j].value();
    }
  }
}

// four consecutive factor values: one 16-byte read when the row is aligned
__device__ __forceinline__ float4 ld4(const float* p, bool aligned) {
  if (aligned) return __ldg(reinterpret_cast<const float4*>(p));
  return make_float4(__ldg(p), __ldg(p + 1), __ldg(p + 2), __ldg(p + 3));
}

// FP32 COO MTTKRP with R % 4 == 0: four lanes per entry, lane q holding components r0 + 4q .. r0 + 4q + 3, so each factor
// row of an entry is gathered as four 16-byte reads by four lanes (one 64-byte
// row per entry and mode) instead of sixteen scalar reads by one lane; eight
// entries of the row are in flight per warp.  Lanes with the same q combine
// their float-float partial sums with shuffles at the end of the row.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256, 4) k_coo_mttkrp_f4(const int* __restrict__ sidx, const float* __restrict__ svals,
                                                       long long nnz, const long long* __restrict__ rowptr, CooShape sh,
                                                       int mode, const float* const* __restrict__ Wrow,
                                                       float* __restrict__ out, int r0) {
  const int lane = threadIdx.x & 31, q = lane & 3, slot = lane >> 2;
  const int warps = (gridDim.x * blockDim.x) >> 5;
  const int d = sh.dims[mode];
  const int R = sh.R;
  const int rq = r0 + 4 * q;
  const bool on = rq < R;
  bool al = true;  // rows are 16-byte aligned when every factor base is (R % 4 == 0)
  for (int m = 0; m < sh.L; ++m) al = al && ((unsigned long long)Wrow[m] & 15ull) == 0;
  for (int row = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; row < d; row += warps) {
    const long long b = rowptr[row], e = rowptr[row + 1];
    Acc<float> acc[4];
    // four entries of the slot per pass (k, k + 8, k + 16, k + 24): per mode
    // their four coordinates are loaded together, then their four factor
    // rows, so a pass waits for two round trips per mode instead of eight;
    // the sums keep the slot's entry order
    constexpr int UNR = 4;
    for (long long k = b + slot; k < e; k += 8 * UNR) {
      float pv[UNR][4];
#pragma unroll
      for (int u = 0; u < UNR; ++u) {
        const long long kk = k + 8 * u;
        const float v = kk < e ? svals[kk] : 0.f;
        pv[u][0] = pv[u][1] = pv[u][2] = pv[u][3] = v;
      }
      if (on && sh.L == 3) {
        // third order: both other modes' coordinates, then both modes' rows,
        // in flight together (two round trips a pass instead of four); the
        // products keep the mode order of the general loop
        const int ma = mode == 0 ? 1 : 0, mb = mode == 2 ? 1 : 2;
        const int* ia = sidx + (size_t)ma * nnz;
        const int* ib = sidx + (size_t)mb * nnz;
        int xa[UNR], xb[UNR];
#pragma unroll
        for (int u = 0; u < UNR; ++u) {
          const bool in = k + 8 * u < e;
          xa[u] = in ? ia[k + 8 * u] : 0;
          xb[u] = in ? ib[k + 8 * u] : 0;
        }
        const float* wa = Wrow[ma] + rq;
        const float* wb = Wrow[mb] + rq;
        float4 ya[UNR], yb[UNR];
#pragma unroll
        for (int u = 0; u < UNR; ++u) {
          ya[u] = ld4(wa + (size_t)xa[u] * R, al);
          yb[u] = ld4(wb + (size_t)xb[u] * R, al);
        }
#pragma unroll
        for (int u = 0; u < UNR; ++u) {
          pv[u][0] = pv[u][0] * ya[u].x * yb[u].x;
          pv[u][1] = pv[u][1] * ya[u].y * yb[u].y;
          pv[u][2] = pv[u][2] * ya[u].z * yb[u].z;
          pv[u][3] = pv[u][3] * ya[u].w * yb[u].w;
        }
      } else if (on) {
        for (int m = 0; m < sh.L; ++m) {
          if (m == mode) continue;
          const int* im = sidx + (size_t)m * nnz;
          int ix[UNR];
#pragma unroll
          for (int u = 0; u < UNR; ++u) ix[u] = (k + 8 * u < e) ? im[k + 8 * u] : 0;
          const float* wm = Wrow[m] + rq;
          float4 w[UNR];
#pragma unroll
          for (int u = 0; u < UNR; ++u) w[u] = ld4(wm + (size_t)ix[u] * R, al);
#pragma unroll
          for (int u = 0; u < UNR; ++u) {
            pv[u][0] *= w[u].x;
            pv[u][1] *= w[u].y;
            pv[u][2] *= w[u].z;
            pv[u][3] *= w[u].w;
          }
        }
      }
#pragma unroll
      for (int u = 0; u < UNR; ++u) {
        if (k + 8 * u < e) {
          acc[0].add(pv[u][0]);
          acc[1].add(pv[u][1]);
          acc[2].add(pv[u][2]);
          acc[3].add(pv[u][3]);
        }
      }
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) {
#pragma unroll
      for (int o = 4; o < 32; o <<= 1) {
        const float oh = __shfl_xor_sync(0xffffffffu, acc[u].hi, o);
        const float ol = __shfl_xor_sync(0xffffffffu, acc[u].lo, o);
        acc[u].add2(oh, ol);
      }
    }
    if (slot == 0 && on) {
      const float4 r4 = make_float4(acc[0].hi + acc[0].lo, acc[1].hi + acc[1].lo, acc[2].hi + acc[2].lo,
                                    acc[3].hi + acc[3].lo);
      *reinterpret_cast<float4*>(out + (size_t)row * R + rq) = r4;
    }
  }
}

// BF16 COO MTTKRP with per-column scaling (R in {8, 16, 32, 64}): the
// factors are gathered as BF16 rows (half the bytes of FP32), each column r of
// mode m stored as W_m[:, r] / s_{m,r} with s_{m,r} a power of two near the
// column's largest magnitude; products and sums in FP32 (float-float), the
// result scaled back by prod_{m != mode} s_{m,r}.  A lane holds eight columns
// (one 16-byte read per factor row), R / 8 lanes per entry, 256 / R entries
// in flight per warp.  Rows of the output as in the FP32 kernel.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256, 4) k_coo_mttkrp_bf16(const int* __restrict__ sidx, const float* __restrict__ svals,
                                                         long long nnz, const long long* __restrict__ rowptr,
                                                         CooShape sh, int mode,
                                                         const __nv_bfloat16* const* __restrict__ Wbf,
                                                         const float* __restrict__ scale, float* __restrict__ out) {
  const int R = sh.R;
  const int lpe = R >> 3;              // lanes per entry (1, 2, 4 or 8)
  const int lane = threadIdx.x & 31, q = lane % lpe, slot = lane / lpe, nslot = 32 / lpe;
  const int warps = (gridDim.x * blockDim.x) >> 5;
  const int d = sh.dims[mode];
  const int c0 = 8 * q;                // this lane's eight columns
  for (int row = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; row < d; row += warps) {
    const long long b = rowptr[row], e = rowptr[row + 1];
    Acc<float> acc[8];
    // two entries of the slot per pass, their coordinates and rows loaded
    // together; the sums keep the slot's entry order
    for (long long k = b + slot; k < e; k += 2 * nslot) {
      float p[2][8];
#pragma unroll
      for (int u = 0; u < 2; ++u) {
        const long long kk = k + (long long)u * nslot;
        const float v = kk < e ? svals[kk] : 0.f;
#pragma unroll
        for (int j = 0; j < 8; ++j) p[u][j] = v;
      }
      for (int m = 0; m < sh.L; ++m) {
        if (m == mode) continue;
        const int* im = sidx + (size_t)m * nnz;
        int ix[2];
#pragma unroll
        for (int u = 0; u < 2; ++u) ix[u] = (k + (long long)u * nslot < e) ? im[k + (long long)u * nslot] : 0;
        uint4 raw[2];
#pragma unroll
        for (int u = 0; u < 2; ++u)
          raw[u] = __ldg(reinterpret_cast<const uint4*>(Wbf[m] + (size_t)ix[u] * R + c0));
#pragma unroll
        for (int u = 0; u < 2; ++u) {
          const uint32_t w4[4] = {raw[u].x, raw[u].y, raw[u].z, raw[u].w};
#pragma unroll
          for (int j = 0; j < 4; ++j) {
            p[u][2 * j] *= __uint_as_float(w4[j] << 16);
            p[u][2 * j + 1] *= __uint_as_float(w4[j] & 0xffff0000u);
          }
        }
      }
#pragma unroll
      for (int u = 0; u < 2; ++u)
        if (k + (long long)u * nslot < e)
#pragma unroll
          for (int j = 0; j < 8; ++j) acc[j].add(p[u][j]);
    }
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      for (int o = lpe; o < 32; o <<= 1) {
        const float oh = __shfl_xor_sync(0xffffffffu, acc[j].hi, o);
        const float ol = __shfl_xor_sync(0xffffffffu, acc[j].lo, o);
        acc[j].add2(oh, ol);
      }
    }
    if (slot == 0) {
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        float sc = 1.f;
        for (int m = 0; m < sh.L; ++m)
          if (m != mode) sc *= scale[m * R + c0 + j];
        out[(size_t)row * R + c0 + j] = (acc[j].hi + acc[j].lo) * sc;
      }
    }
  }
}

// per-column power-of-two scales and the BF16 row-major copies of the flat
// (column-major) factors: one CTA per column (mode l, column r)
__global__ void __launch_bounds__(256) k_factors_bf16(CooShape sh, const float* __restrict__ W,
                                                      __nv_bfloat16* __restrict__ Wbf, float* __restrict__ scale) {
  __shared__ float smax[8];
  const int L = sh.L, R = sh.R;
  const int col = blockIdx.x;  // l * R + r
  const int l = col / R, r = col - l * R;
  long long off = 0;
  for (int m = 0; m < l; ++m) off += (long long)sh.dims[m] * R;
  const int d = sh.dims[l];
  const float* w = W + off + (long long)r * d;
  float mx = 0.f;
  for (int i = threadIdx.x; i < d; i += blockDim.x) mx = fmaxf(mx, fabsf(w[i]));
  for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  if ((threadIdx.x & 31) == 0) smax[threadIdx.x >> 5] = mx;
  __syncthreads();
  if (threadIdx.x < 32) {
    float v = threadIdx.x < 8 ? smax[threadIdx.x] : 0.f;
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    if (threadIdx.x == 0) smax[0] = v;
  }
  __syncthreads();
  // a power of two: dividing by it is exact, so the scaling adds no rounding
  const float sc = smax[0] > 0.f ? exp2f(ceilf(log2f(smax[0]))) : 1.f;
  if (threadIdx.x == 0) scale[l * R + r] = sc;
  const float inv = 1.f / sc;
  for (int i = threadIdx.x; i < d; i += blockDim.x) Wbf[off + (long long)i * R + r] = __float2bfloat16_rn(w[i] * inv);
  (void)L;
}

// FP32 residual with R % 4 == 0: 16-byte gathers of the factor rows (when
// aligned), the model summed in a fixed order.
__global__ void __launch_bounds__(256) k_sparse_residual_f4(const int* __restrict__ idx32, const float* __restrict__ vals,
                                                            long long nnz, CooShape sh,
                                                            const float* const* __restrict__ Wrow,
                                                            double* __restrict__ partial) {
  __shared__ double red[8];
  Acc<float> acc;
  const int R = sh.R, L = sh.L;
  bool al = true;
  for (int l = 0; l < L; ++l) al = al && ((unsigned long long)Wrow[l] & 15ull) == 0;
  const long long S = (long long)gridDim.x * blockDim.x;
  if (L == 3) {
    // third order: two entries a pass, their coordinates and then all six
    // factor rows in flight together (the general loop indexes its row
    // pointers at run time and waits on each mode in turn); products, sums
    // and the order of the squared differences are those of the general loop
    const float* W0 = Wrow[0];
    const float* W1 = Wrow[1];
    const float* W2 = Wrow[2];
    for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < nnz; k += 2 * S) {
      const long long k2 = k + S;
      const bool two = k2 < nnz;
      const int a0 = idx32[k], b0 = idx32[nnz + k], c0 = idx32[2 * nnz + k];
      const int a1 = two ? idx32[k2] : 0, b1 = two ? idx32[nnz + k2] : 0, c1 = two ? idx32[2 * nnz + k2] : 0;
      const float v0 = vals[k], v1 = two ? vals[k2] : 0.f;
      const float* x0 = W0 + (size_t)a0 * R;
      const float* y0 = W1 + (size_t)b0 * R;
      const float* z0 = W2 + (size_t)c0 * R;
      const float* x1 = W0 + (size_t)a1 * R;
      const float* y1 = W1 + (size_t)b1 * R;
      const float* z1 = W2 + (size_t)c1 * R;
      float m0 = 0.f, m1 = 0.f;
#pragma unroll 4
      for (int r = 0; r < R; r += 4) {
        float4 p = ld4(x0 + r, al), q = ld4(x1 + r, al);
        const float4 u0 = ld4(y0 + r, al), u1 = ld4(y1 + r, al);
        const float4 t0 = ld4(z0 + r, al), t1 = ld4(z1 + r, al);
        p.x *= u0.x; p.y *= u0.y; p.z *= u0.z; p.w *= u0.w;
        p.x *= t0.x; p.y *= t0.y; p.z *= t0.z; p.w *= t0.w;
        q.x *= u1.x; q.y *= u1.y; q.z *= u1.z; q.w *= u1.w;
        q.x *= t1.x; q.y *= t1.y; q.z *= t1.z; q.w *= t1.w;
        m0 += (p.x + p.y) + (p.z + p.w);
        m1 += (q.x + q.y) + (q.z + q.w);
      }
      const float d0 = v0 - m0;
      acc.fma_(d0, d0);
      if (two) {
        const float d1 = v1 - m1;
        acc.fma_(d1, d1);
      }
    }
  } else
  for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < nnz; k += S) {
    const float* w[TFX_MAX_ORDER];
    for (int l = 0; l < L; ++l) w[l] = Wrow[l] + (size_t)idx32[(size_t)l * nnz + k] * R;
    float model = 0.f;
    for (int r = 0; r < R; r += 4) {
      float4 p = ld4(w[0] + r, al);
      for (int l = 1; l < L; ++l) {
        const float4 x = ld4(w[l] + r, al);
        p.x *= x.x;
        p.y *= x.y;
        p.z *= x.z;
        p.w *= x.w;
      }
      model += (p.x + p.y) + (p.z + p.w);
    }
    const float df = vals[k] - model;
    acc.fma_(df, df);
  }
  acc.warp_reduce();
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc.value();
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += red[w];
    partial[blockIdx.x] = s;
  }
}

// ---------------------------------------------------------------------------
// nnz-only residual: partial sums of (v - sum_r prod_l W_l[i_l, r])^2 per block
// ---------------------------------------------------------------------------
template <class T>
__global__ void __launch_bounds__(256) k_sparse_residual(const int* __restrict__ idx32, const T* __restrict__ vals,
                                                         long long nnz, CooShape sh, const T* const* __restrict__ Wrow,
                                                         double* __restrict__ partial) {
  __shared__ double red[8];
  Acc<T> acc;
  const int R = sh.R;
  for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < nnz; k += (long long)gridDim.x * blockDim.x) {
    const T* w[TFX_MAX_ORDER];
    for (int l = 0; l < sh.L; ++l) w[l] = Wrow[l] + (size_t)idx32[(size_t)l * nnz + k] * R;
    T model = T(0);
    for (int r = 0; r < R; ++r) {
      T p = w[0][r];
      for (int l = 1; l < sh.L; ++l) p *= w[l][r];
      model += p;
    }
    const T df = vals[k] - model;
    acc.fma_(df, df);
  }
  acc.warp_reduce();
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc.value();
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += red[w];
    partial[blockIdx.x] = s;
  }
}

// ---------------------------------------------------------------------------
// COO Gram.  Diagonal: sum of v^2 per row of the row-sorted copy.  Entries of
// one fibre (same indices in every mode but l) are grouped in a hash table with
// bounded linear probing.  A slot holds the id of the first entry that claimed
// it (the fibre's representative); an entry joins a slot only when its
// coordinates equal the representative's in every mode but l, so two fibres
// never merge, whatever the dimensions (no mixed-radix key that could wrap).
// Each pair of distinct rows in a fibre adds v*v' to G[i,i'] and G[i',i].
// ---------------------------------------------------------------------------
__device__ __forceinline__ unsigned long long mix64(unsigned long long x) {
  x ^= x >> 33;
  x *= 0xff51afd7ed558ccdULL;
  x ^= x >> 33;
  x *= 0xc4ceb9fe1a85ec53ULL;
  x ^= x >> 33;
  return x;
}

// hash of the coordinates of entry k in every mode but `mode` (a hash only:
// equal hashes are resolved by comparing coordinates)
__device__ __forceinline__ unsigned long long fibre_hash(const int* __restrict__ idx32, long long nnz, long long k,
                                                         int L, int mode) {
  unsigned long long h = 0x9e3779b97f4a7c15ULL;
  for (int m = 0; m < L; ++m) {
    if (m == mode) continue;
    h = mix64(h ^ (unsigned long long)(unsigned int)idx32[(size_t)m * nnz + k]);
  }
  return h;
}

__device__ __forceinline__ bool same_fibre(const int* __restrict__ idx32, long long nnz, long long a, long long b,
                                           int L, int mode) {
  for (int m = 0; m < L; ++m) {
    if (m == mode) continue;
    if (idx32[(size_t)m * nnz + a] != idx32[(size_t)m * nnz + b]) return false;
  }
  return true;
}

#define TFX_EMPTY_SLOT 0xffffffffffffffffULL
#define TFX_MAX_PROBES 4096

// insert every entry into its fibre's slot; heads form per-slot lists
__global__ void k_fibre_insert(const int* __restrict__ idx32, long long nnz, int L, int mode,
                               unsigned long long* __restrict__ rep, long long nslots, int* __restrict__ head,
                               int* __restrict__ next, int* __restrict__ err) {
  for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < nnz; k += (long long)gridDim.x * blockDim.x) {
    long long s = (long long)(fibre_hash(idx32, nnz, k, L, mode) % (unsigned long long)nslots);
    int probes = 0;
    while (true) {
      const unsigned long long prev = atomicCAS(rep + s, TFX_EMPTY_SLOT, (unsigned long long)k);
      if (prev == TFX_EMPTY_SLOT || same_fibre(idx32, nnz, (long long)prev, k, L, mode)) break;
      if (++probes >= TFX_MAX_PROBES) {
        atomicExch(err, 2);
        s = -1;
        break;
      }
      s = (s + 1 == nslots) ? 0 : s + 1;
    }
    if (s >= 0) next[k] = atomicExch(head + s, (int)k);
  }
}

template <class T>
__global__ void k_fibre_pairs(const int* __restrict__ idx32, const T* __restrict__ vals, long long nnz, int mode,
                              long long nslots, const int* __restrict__ head, const int* __restrict__ next, int d,
                              double* __restrict__ G) {
  const int* rows = idx32 + (size_t)mode * nnz;
  for (long long s = (long long)blockIdx.x * blockDim.x + threadIdx.x; s < nslots; s += (long long)gridDim.x * blockDim.x) {
    const int h = head[s];
    if (h < 0 || next[h] < 0) continue;  // empty or single-entry fibre
    for (int a = h; a >= 0; a = next[a]) {
      for (int b = next[a]; b >= 0; b = next[b]) {
        const int ia = rows[a], ib = rows[b];
        const double p = (double)vals[a] * (double)vals[b];
        atomicAdd(G + (size_t)ia * d + ib, p);
        atomicAdd(G + (size_t)ib * d + ia, p);
      }
    }
  }
}

template <class T>
__global__ void k_gram_diag(const T* __restrict__ svals, const long long* __restrict__ rowptr, int d,
                            double* __restrict__ G) {
  const int lane = threadIdx.x & 31;
  const int warps = (gridDim.x * blockDim.x) >> 5;
  for (int row = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; row < d; row += warps) {
    Acc<T> acc;
    for (long long k = rowptr[row] + lane; k < rowptr[row + 1]; k += 32) acc.fma_(svals[k], svals[k]);
    acc.warp_reduce();
    if (lane == 0) G[(size_t)row * d + row] += acc.value();
  }
}

template <class T>
__global__ void k_double_to(const double* __restrict__ a, long long n, T* __restrict__ b) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    b[i] = (T)a[i];
}

// ---------------------------------------------------------------------------
// Sparse TTMc: S[a, q] = sum_k v_k U_0[i_0k, a] prod_{m>=1} U_m[i_mk, q_m], with
// q the C-order index over the output modes 1..L-1.  Split-K over entries;
// each CTA accumulates a (16*TS x 16*TS) tile of S_(0), partials summed after.
// U_m are (d_m x n_m) row-major.
// ---------------------------------------------------------------------------
struct TtmcShape {
  int L;
  int dims[TFX_MAX_ORDER];
  int n[TFX_MAX_ORDER];
};

template <class T, int TS>
__global__ void __launch_bounds__(TFX_THREADS) k_sparse_ttmc(const int* __restrict__ idx32, const T* __restrict__ vals,
                                                             long long nnz, TtmcShape sh, const T* const* __restrict__ U,
                                                             int ksplit, T* __restrict__ part) {
  using TL = Tile<TS, TS>;
  __shared__ T sA[TFX_BK * TL::LDA];
  __shared__ T sB[TFX_BK * TL::LDB];
  __shared__ int qidx[TL::BN * TFX_MAX_ORDER];
  const int n0 = sh.n[0];
  long long Q = 1;
  for (int m = 1; m < sh.L; ++m) Q *= sh.n[m];
  const int tilesM = (n0 + TL::BM - 1) / TL::BM;
  const int a0 = (blockIdx.x % tilesM) * TL::BM;
  const long long q0 = (long long)(blockIdx.x / tilesM) * TL::BN;
  const long long kb = nnz * blockIdx.y / ksplit, ke = nnz * (blockIdx.y + 1) / ksplit;
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  if (tid < TL::BN) {
    long long q = q0 + tid;
    for (int m = sh.L - 1; m >= 1; --m) {
      qidx[tid * TFX_MAX_ORDER + m] = (int)(q % sh.n[m]);
      q /= sh.n[m];
    }
  }
  __syncthreads();
  T acc[TS][TS];
  tile_zero<T, TS, TS>(acc);
  for (long long k0 = kb; k0 < ke; k0 += TFX_BK) {
    const int kc = (int)min((long long)TFX_BK, ke - k0);
    for (int e = tid; e < TFX_BK * TL::BM; e += TFX_THREADS) {
      const int kk = e / TL::BM, mm = e - kk * TL::BM;
      T v = T(0);
      if (kk < kc && a0 + mm < n0) {
        const long long k = k0 + kk;
        v = vals[k] * U[0][(size_t)idx32[k] * n0 + a0 + mm];
      }
      sA[kk * TL::LDA + mm] = v;
    }
    for (int e = tid; e < TFX_BK * TL::BN; e += TFX_THREADS) {
      const int kk = e / TL::BN, nn = e - kk * TL::BN;
      T v = T(0);
      if (kk < kc && q0 + nn < Q) {
        const long long k = k0 + kk;
        v = T(1);
        for (int m = 1; m < sh.L; ++m)
          v *= U[m][(size_t)idx32[(size_t)m * nnz + k] * sh.n[m] + qidx[nn * TFX_MAX_ORDER + m]];
      }
      sB[kk * TL::LDB + nn] = v;
    }
    __syncthreads();
    tile_fma<T, TS, TS>(sA, sB, acc, kc);
    __syncthreads();
  }
  T* out = part + (size_t)blockIdx.y * n0 * Q;
#pragma unroll
  for (int u = 0; u < TS; ++u)
#pragma unroll
    for (int v = 0; v < TS; ++v) {
      const int a = a0 + ty + 16 * u;
      const long long q = q0 + tx + 16 * v;
      if (a < n0 && q < Q) out[(size_t)a * Q + q] = acc[u][v];
    }
}

__global__ void k_sum_partials_sp(const double* __restrict__ partial, int n, double* __restrict__ out) {
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int i = 0; i < n; ++i) s += partial[i];
    out[0] = s;
  }
}

template <class T>
__global__ void k_sum_split(const T* __restrict__ part, long long n, int ks, T* __restrict__ out) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int k = 0; k < ks; ++k) s += (double)part[(size_t)k * n + i];
    out[i] = (T)s;
  }
}

}  // namespace tfx

// ============================================================================
// C ABI
// ============================================================================
using namespace tfx;

static int sms() {
  static int n = 0;
  if (!n) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    if (n < 1) n = 1;
  }
  return n;
}

static int launched(const char* where) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return tfx_set_cuda_error(e, where);
  tfx_count_launch(1);
  return TFX_STATUS_OK;
}

static int grid_for(long long n, int per_block = 256) {
  return (int)std::max<long long>(1, std::min<long long>((n + per_block - 1) / per_block, 8LL * sms()));
}

static int fill_shape(CooShape& sh, int L, const int* dims, int R) {
  if (L < 2 || L > TFX_MAX_ORDER || !dims || R < 1) return 1;
  sh.L = L;
  sh.R = R;
  for (int l = 0; l < L; ++l) {
    if (dims[l] < 1) return 1;
    sh.dims[l] = dims[l];
  }
  return 0;
}

extern "C" int tfx_coo_encode(const long long* idx64, long long nnz, int L, const int* dims, int* idx32, int* err,
                              void* stream) {
  CooShape sh;
  if (fill_shape(sh, L, dims, 1) || !idx64 || !idx32 || !err || nnz < 0)
    return tfx_set_error(TFX_STATUS_ERR_ARG, "coo_encode args");
  if (nnz == 0) return TFX_STATUS_OK;
  k_coo_encode<<<grid_for(nnz), 256, 0, (cudaStream_t)stream>>>(idx64, nnz, L, sh, idx32, err);
  return launched("coo_encode");
}

extern "C" int tfx_coo_sort_mode(int dtype, const int* idx32, const void* vals, long long nnz, int L, const int* dims,
                                 int mode, int* counts_scratch, long long* rowptr, int* sidx, void* svals,
                                 void* stream) {
  CooShape sh;
  if (fill_shape(sh, L, dims, 1) || mode < 0 || mode >= L || !idx32 || !vals || !counts_scratch || !rowptr || !sidx ||
      !svals)
    return tfx_set_error(TFX_STATUS_ERR_ARG, "coo_sort_mode args");
  cudaStream_t st = (cudaStream_t)stream;
  const int d = dims[mode];
  cudaError_t e = cudaMemsetAsync(counts_scratch, 0, sizeof(int) * (size_t)d * 2, st);
  if (e != cudaSuccess) return tfx_set_cuda_error(e, "coo_sort memset");
  if (nnz > 0) {
    k_count_rows<<<grid_for(nnz), 256, 0, st>>>(idx32 + (size_t)mode * nnz, nnz, counts_scratch);
    if (int s = launched("count_rows")) return s;
  }
  k_scan_counts<<<1, TFX_THREADS, 0, st>>>(counts_scratch, d, rowptr);
  if (int s = launched("scan_counts")) return s;
  if (nnz > 0) {
    if (dtype == TFX_F32)
      k_scatter_rows<float><<<grid_for(nnz), 256, 0, st>>>(idx32, (const float*)vals, nnz, L, mode, rowptr,
                                                           counts_scratch + d, sidx, (float*)svals);
    else
      k_scatter_rows<double><<<grid_for(nnz), 256, 0, st>>>(idx32, (const double*)vals, nnz, L, mode, rowptr,
                                                            counts_scratch + d, sidx, (double*)svals);
    return launched("scatter_rows");
  }
  return TFX_STATUS_OK;
}

extern "C" int tfx_coo_mttkrp(int dtype, const int* sidx, const void* svals, long long nnz, const long long* rowptr,
                              int L, const int* dims, int R, int mode, const void* const* Wrow_dev, void* out,
                              void* stream) {
  CooShape sh;
  if (fill_shape(sh, L, dims, R) || mode < 0 || mode >= L || !sidx || !svals || !rowptr || !Wrow_dev || !out)
    return tfx_set_error(TFX_STATUS_ERR_ARG, "coo_mttkrp args");
  cudaStream_t st = (cudaStream_t)stream;
  const int d = dims[mode];
  const int blocks = (int)std::max<long long>(1, std::min<long long>(((long long)d * 32 + 255) / 256, 16LL * sms()));
  for (int r0 = 0; r0 < R; r0 += 16) {
    if (dtype == TFX_F32 && R % 4 == 0 && ((unsigned long long)out & 15) == 0)
      k_coo_mttkrp_f4<<<blocks, 256, 0, st>>>(sidx, (const float*)svals, nnz, rowptr, sh, mode,
                                              (const float* const*)Wrow_dev, (float*)out, r0);
    else if (dtype == TFX_F32)
      k_coo_mttkrp<float, 16><<<blocks, 256, 0, st>>>(sidx, (const float*)svals, nnz, rowptr, sh, mode,
                                                      (const float* const*)Wrow_dev, (float*)out, r0);
    else
      k_coo_mttkrp<double, 16><<<blocks, 256, 0, st>>>(sidx, (const double*)svals, nnz, rowptr, sh, mode,
                                                       (const double* const*)Wrow_dev, (double*)out, r0);
    if (int s = launched("coo_mttkrp")) return s;
  }
  return TFX_STATUS_OK;
}

extern "C" size_t tfx_sparse_residual_scratch_bytes(void) { return (size_t)8 * (16 * 1024 + 8); }

extern "C" int tfx_sparse_residual(int dtype, const int* idx32, const void* vals, long long nnz, int L, const int* dims,
                                   int R, const void* const* Wrow_dev, double* out, void* scratch, void* stream) {
  CooShape sh;
  if (fill_shape(sh, L, dims, R) || !idx32 || !vals || !Wrow_dev || !out || !scratch)
    return tfx_set_error(TFX_STATUS_ERR_ARG, "sparse_residual args");
  cudaStream_t st = (cudaStream_t)stream;
  const int blocks = (int)std::max<long long>(1, std::min<long long>((nnz + 255) / 256, 8LL * sms()));
  double* partial = (double*)scratch;
  if (dtype == TFX_F32 && R % 4 == 0)
    k_sparse_residual_f4<<<blocks, 256, 0, st>>>(idx32, (const float*)vals, nnz, sh, (const float* const*)Wrow_dev,
                                                 partial);
  else if (dtype == TFX_F32)
    k_sparse_residual<float><<<blocks, 256, 0, st>>>(idx32, (const float*)vals, nnz, sh, (const float* const*)Wrow_dev,
                                                     partial);
  else
    k_sparse_residual<double><<<blocks, 256, 0, st>>>(idx32, (const double*)vals, nnz, sh,
                                                      (const double* const*)Wrow_dev, partial);
  if (int s = launched("sparse_residual")) return s;
  k_sum_partials_sp<<<1, 32, 0, st>>>(partial, blocks, out);
  return launched("sum_partials");
}

extern "C" size_t tfx_coo_gram_scratch_bytes(long long nnz, int d) {
  const long long nslots = 2 * std::max<long long>(nnz, 1) + 1;
  return (size_t)nslots * 8 + (size_t)nslots * 4 + (size_t)std::max<long long>(nnz, 1) * 4 + (size_t)d * d * 8 + 64;
}

extern "C" int tfx_coo_gram(int dtype, const int* idx32, const void* vals, long long nnz, const void* svals_sorted,
                            const long long* rowptr, int L, const int* dims, int mode, void* G, void* scratch,
                            size_t scratch_bytes, int* err, void* stream) {
  CooShape sh;
  if (fill_shape(sh, L, dims, 1) || mode < 0 || mode >= L || !idx32 || !vals || !svals_sorted || !rowptr || !G ||
      !scratch || !err)
    return tfx_set_error(TFX_STATUS_ERR_ARG, "coo_gram args");
  // the per-entry fibre lists hold 32-bit entry ids
  if (nnz < 0 || nnz >= (1LL << 31))
    return tfx_set_error(TFX_STATUS_ERR_ARG, "coo_gram: the number of stored entries must be below 2^31");
  const int d = dims[mode];
  const long long nslots = 2 * std::max<long long>(nnz, 1) + 1;
  if (scratch_bytes < tfx_coo_gram_scratch_bytes(nnz, d)) return tfx_set_error(TFX_STATUS_ERR_ARG, "coo_gram scratch");
  char* p = (char*)scratch;
  unsigned long long* rep = (unsigned long long*)p;
  p += (size_t)nslots * 8;
  int* head = (int*)p;
  p += (size_t)nslots * 4;
  int* next = (int*)p;
  p += (size_t)std::max<long long>(nnz, 1) * 4;
  p = (char*)(((uintptr_t)p + 15) & ~(uintptr_t)15);
  double* Gd = (double*)p;
  cudaStream_t st = (cudaStream_t)stream;
  cudaError_t e = cudaMemsetAsync(rep, 0xff, (size_t)nslots * 8, st);
  if (e == cudaSuccess) e = cudaMemsetAsync(head, 0xff, (size_t)nslots * 4, st);
  if (e == cudaSuccess) e = cudaMemsetAsync(Gd, 0, (size_t)d * d * 8, st);
  if (e != cudaSuccess) return tfx_set_cuda_error(e, "coo_gram memset");
  if (nnz > 0) {
    k_fibre_insert<<<grid_for(nnz), 256, 0, st>>>(idx32, nnz, L, mode, rep, nslots, head, next, err);
    if (int s = launched("fibre_insert")) return s;
    if (dtype == TFX_F32)
      k_fibre_pairs<float><<<grid_for(nslots), 256, 0, st>>>(idx32, (const float*)vals, nnz, mode, nslots, head, next,
                                                             d, Gd);
    else
      k_fibre_pairs<double><<<grid_for(nslots), 256, 0, st>>>(idx32, (const double*)vals, nnz, mode, nslots, head,
                                                              next, d, Gd);
    if (int s = launched("fibre_pairs")) return s;
  }
  const int blocks = (int)std::max<long long>(1, std::min<long long>(((long long)d * 32 + 255) / 256, 8LL * sms()));
  if (dtype == TFX_F32) {
    k_gram_diag<float><<<blocks, 256, 0, st>>>((const float*)svals_sorted, rowptr, d, Gd);
    if (int s = launched("gram_diag")) return s;
    k_double_to<float><<<grid_for((long long)d * d), 256, 0, st>>>(Gd, (long long)d * d, (float*)G);
  } else {
    k_gram_diag<double><<<blocks, 256, 0, st>>>((const double*)svals_sorted, rowptr, d, Gd);
    if (int s = launched("gram_diag")) return s;
    k_double_to<double><<<grid_for((long long)d * d), 256, 0, st>>>(Gd, (long long)d * d, (double*)G);
  }
  return launched("gram_convert");
}

extern "C" size_t tfx_sparse_ttmc_scratch_bytes(int dtype, long long nnz, int L, const int* n) {
  long long Q = 1;
  for (int l = 1; l < L; ++l) Q *= n[l];
  const long long tiles = ((n[0] + 63) / 64) * ((Q + 63) / 64);
  long long ks = std::max<long long>(1, std::min<long long>((4LL * sms() + tiles - 1) / tiles, (nnz + 1023) / 1024));
  ks = std::min<long long>(ks, 64);
  return (size_t)ks * n[0] * Q * (dtype == TFX_F64 ? 8 : 4);
}

extern "C" int tfx_sparse_ttmc(int dtype, const int* idx32, const void* vals, long long nnz, int L, const int* dims,
                               const int* n, const void* const* U_dev, void* S, void* scratch, size_t scratch_bytes,
                               void* stream) {
  if (L < 2 || L > TFX_MAX_ORDER || !idx32 || !vals || !dims || !n || !U_dev || !S || !scratch)
    return tfx_set_error(TFX_STATUS_ERR_ARG, "sparse_ttmc args");
  TtmcShape sh;
  sh.L = L;
  long long Q = 1;
  for (int l = 0; l < L; ++l) {
    sh.dims[l] = dims[l];
    sh.n[l] = n[l];
    if (l) Q *= n[l];
  }
  const size_t es = dtype == TFX_F64 ? 8 : 4;
  const size_t per = (size_t)n[0] * Q * es;
  int ks = (int)std::min<size_t>(scratch_bytes / per, tfx_sparse_ttmc_scratch_bytes(dtype, nnz, L, n) / per);
  if (ks < 1) return tfx_set_error(TFX_STATUS_ERR_ARG, "sparse_ttmc scratch");
  cudaStream_t st = (cudaStream_t)stream;
  const long long tiles = ((n[0] + 63) / 64) * ((Q + 63) / 64);
  dim3 grid((unsigned)tiles, (unsigned)ks);
  if (dtype == TFX_F32)
    k_sparse_ttmc<float, 4><<<grid, TFX_THREADS, 0, st>>>(idx32, (const float*)vals, nnz, sh,
                                                          (const float* const*)U_dev, ks, (float*)scratch);
  else
    k_sparse_ttmc<double, 4><<<grid, TFX_THREADS, 0, st>>>(idx32, (const double*)vals, nnz, sh,
                                                           (const double* const*)U_dev, ks, (double*)scratch);
  if (int s = launched("sparse_ttmc")) return s;
  const long long tot = (long long)n[0] * Q;
  if (dtype == TFX_F32)
    k_sum_split<float><<<grid_for(tot), 256, 0, st>>>((const float*)scratch, tot, ks, (float*)S);
  else
    k_sum_split<double><<<grid_for(tot), 256, 0, st>>>((const double*)scratch, tot, ks, (double*)S);
  return launched("ttmc_sum");
}

extern "C" int tfx_factors_bf16(int L, const int* dims, int R, const float* W, void* Wbf, float* scale, void* stream) {
  CooShape sh;
  if (fill_shape(sh, L, dims, R) || !W || !Wbf || !scale) return tfx_set_error(TFX_STATUS_ERR_ARG, "factors_bf16 args");
  k_factors_bf16<<<L * R, 256, 0, (cudaStream_t)stream>>>(sh, W, (__nv_bfloat16*)Wbf, scale);
  return launched("factors_bf16");
}

extern "C" int tfx_coo_mttkrp_bf16(const int* sidx, const float* svals, long long nnz, const long long* rowptr, int L,
                                   const int* dims, int R, int mode, const void* const* Wbf_dev, const float* scale,
                                   float* out, void* stream) {
  CooShape sh;
  if (fill_shape(sh, L, dims, R) || mode < 0 || mode >= L || !sidx || !svals || !rowptr || !Wbf_dev || !scale || !out)
    return tfx_set_error(TFX_STATUS_ERR_ARG, "coo_mttkrp_bf16 args");
  if (R != 8 && R != 16 && R != 32 && R != 64)
    return tfx_set_error(TFX_STATUS_ERR_UNSUPPORTED, "coo_mttkrp_bf16: R must be 8, 16, 32 or 64");
  const int d = dims[mode];
  const int blocks = (int)std::max<long long>(1, std::min<long long>(((long long)d * 32 + 255) / 256, 16LL * sms()));
  k_coo_mttkrp_bf16<<<blocks, 256, 0, (cudaStream_t)stream>>>(sidx, svals, nnz, rowptr, sh, mode,
                                                               (const __nv_bfloat16* const*)Wbf_dev, scale, out);
  return launched("coo_mttkrp_bf16");
}
