// ||T - [[W0, W1, W2]]||^2 of a third-order FP32 tensor on the 5th-generation
// tensor cores (Critical.py:14-22 fastnorm of Conversion.py:117-141's model).
//
// The model unfolding is M = W0 KR^T with KR[q, r] = W1[j, r] W2[k, r],
// q = j*d2 + k.  A persistent CTA takes 256-column blocks of the unfolding:
// it forms the block's Khatri-Rao rows once in shared memory (K-major,
// SWIZZLE_128B layout, rank padded to 64), then for every 128-row block of
// mode 0 stages W0's rows the same way, issues the products with
// tcgen05.mma kind::tf32 (M = 128, N = 256, K = 8) into a TMEM accumulator, and
// its eight warps read the 128 x 256 model tile back (tcgen05.ld), subtract the
// tensor tile streamed from global memory and accumulate squares in
// float-float.  Operands are split hi + lo (x = tf32(x) + (x - tf32(x))) and
// the product is Ahi Bhi + Ahi Blo + Alo Bhi, so the model carries FP32
// accuracy, not TF32's.  Used for R <= 64, d1*d2 % 4 == 0, 16-byte aligned T.
// Every wait is bounded; a wait that runs out sets *err and the CTA skips the
// rest of its work.
#include <math.h>
#include <stdint.h>

#include <algorithm>

#include "tfx_capi_internal.h"
#include "tfx_common.cuh"

namespace tfx {
namespace rtc {

constexpr int BM = 128, BN = 256, KP = 64, NT = 256, BU = 8;
constexpr uint32_t SPIN = 1u << 26;

__device__ __forceinline__ uint32_t su32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// K-major SWIZZLE_128B: row r of an atom (32 fp32 of K) is 128 bytes, 8-row
// groups 1024 bytes apart, 16-byte chunk c stored at c ^ (r % 8)
__device__ __forceinline__ uint32_t sw_off(int r, int k) {
  return (uint32_t)(r * 128 + ((((k >> 2) ^ (r & 7)) & 7) << 4) + ((k & 3) << 2));
}

// entry e of an operand tile (rows x KP ranks) -> (row n, rank k): lane bits
// 0-2 are the row within 8, bits 3-4 the rank within 4, then rank groups of
// four, then row groups of eight (KP % 4 == 0)
__device__ __forceinline__ void tile_nk(int e, int& n, int& k) {
  const int blk = e >> 5;
  const int kb = blk % (KP / 4), nb = blk / (KP / 4);
  n = nb * 8 + (e & 7);
  k = kb * 4 + ((e >> 3) & 3);
}

__device__ __forceinline__ uint64_t desc(const void* tile) {
  const uint64_t a = su32(tile);
  uint64_t d = 0;
  d |= (a >> 4) & 0x3FFFull;
  d |= (uint64_t)1 << 16;
  d |= (uint64_t)(1024 >> 4) << 32;
  d |= (uint64_t)1 << 46;
  d |= (uint64_t)2 << 61;
  return d;
}

// D = F32, A = B = TF32, K-major, M = 128, N = 256
__host__ __device__ constexpr uint32_t idesc() {
  return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(BN >> 3) << 17) | ((uint32_t)(BM >> 4) << 24);
}

__device__ __forceinline__ void mma(uint32_t tmem, uint64_t a, uint64_t b, uint32_t acc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem),
      "l"(a), "l"(b), "r"(idesc()), "r"(acc)
      : "memory");
}

__device__ __forceinline__ bool wait_bar(uint64_t* bar, uint32_t parity) {
  return mbar_wait_bounded(su32(bar), parity, SPIN);
}

__device__ __forceinline__ float tf32_hi(float x) {
  uint32_t u;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(u) : "f"(x));
  return __uint_as_float(u);
}

struct Smem {
  alignas(1024) unsigned char ahi[2][BM * 128];
  alignas(1024) unsigned char alo[2][BM * 128];
  alignas(1024) unsigned char bhi[2][BN * 128];
  alignas(1024) unsigned char blo[2][BN * 128];
  alignas(8) uint64_t done;
  uint32_t tmem;
  int abort;
  double red[NT / 32][2];
};

struct Shape {
  int d0, d1, d2, R;
  long long Q0;
  const float* W0;
  const float* W1;
  const float* W2;
};

__global__ void __launch_bounds__(NT, 1) k_residual_tc(const float* __restrict__ T, Shape sh, double* __restrict__ part,
                                                       int* err) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  Smem& S = *reinterpret_cast<Smem*>((((uintptr_t)smem_raw) + 1023) & ~(uintptr_t)1023);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int d0 = sh.d0, d2 = sh.d2, R = sh.R;
  const long long Q0 = sh.Q0;
  const int ncb = (int)((Q0 + BN - 1) / BN), nib = (d0 + BM - 1) / BM;
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(su32(&S.done)));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    S.abort = 0;
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 256;" ::"r"(su32(&S.tmem))
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = S.tmem;
  Acc<float> acc[4];  // independent chains: the float-float update is a long dependent sequence
  uint32_t phase = 0;
  for (int cb = blockIdx.x; cb < ncb; cb += gridDim.x) {
    const long long q0 = (long long)cb * BN;
    // Khatri-Rao rows of the column block: hi and lo parts.  Sixteen entries
    // a pass, their factor loads issued together (the loads come from L2);
    // a warp covers 8 columns x 4 ranks, so that its loads of W2 are four
    // 32-byte runs and its swizzled stores hit 32 distinct banks.
    constexpr int BB = 2 * BU;  // sixteen entries a pass (the column block's operand is the larger one)
    for (int e0 = tid; e0 < BN * KP; e0 += NT * BB) {
      float f1[BB], f2[BB];
#pragma unroll
      for (int u = 0; u < BB; ++u) {
        const int e = e0 + u * NT;
        int n, k;
        tile_nk(e, n, k);
        const long long q = q0 + n;
        f1[u] = 0.f;
        f2[u] = 0.f;
        if (e < BN * KP && k < R && q < Q0) {
          // Q0 < 2^31 (checked on the host): 32-bit division
          const unsigned qq = (unsigned)q;
          const unsigned j = qq / (unsigned)d2, kk = qq - j * (unsigned)d2;
          f1[u] = __ldg(sh.W1 + (size_t)k * sh.d1 + j);
          f2[u] = __ldg(sh.W2 + (size_t)k * d2 + kk);
        }
      }
#pragma unroll
      for (int u = 0; u < BB; ++u) {
        const int e = e0 + u * NT;
        if (e < BN * KP) {
          int n, k;
          tile_nk(e, n, k);
          const float v = f1[u] * f2[u];
          const float h = tf32_hi(v);
          const uint32_t o = sw_off(n, k & 31);
          *(float*)(S.bhi[k >> 5] + o) = h;
          *(float*)(S.blo[k >> 5] + o) = v - h;
        }
      }
    }
    for (int ib = 0; ib < nib; ++ib) {
      const int i0 = ib * BM;
      // W0's rows of the block, eight entries a pass with their loads issued
      // together (the shared-memory stores go through a generic pointer, so
      // the compiler would not move later loads above them)
      for (int e0 = tid; e0 < BM * KP; e0 += NT * BU) {
        float f[BU];
#pragma unroll
        for (int u = 0; u < BU; ++u) {
          const int e = e0 + u * NT;
          int m, k;
          tile_nk(e, m, k);
          const int i = i0 + m;
          f[u] = (e < BM * KP && k < R && i < d0) ? __ldg(sh.W0 + (size_t)k * d0 + i) : 0.f;
        }
#pragma unroll
        for (int u = 0; u < BU; ++u) {
          const int e = e0 + u * NT;
          if (e < BM * KP) {
            int m, k;
            tile_nk(e, m, k);
            const float h = tf32_hi(f[u]);
            const uint32_t o = sw_off(m, k & 31);
            *(float*)(S.ahi[k >> 5] + o) = h;
            *(float*)(S.alo[k >> 5] + o) = f[u] - h;
          }
        }
      }
      // the thread's 128 tensor values of this tile (row 32 (warp % 4) + lane,
      // columns (warp / 4) 128 ..), loaded after W0's rows (issued first, the
      // 32 16-byte loads a thread would hold the operand loads back) and
      // before the products, so the tile is in flight while they run
      const int erow = 32 * (warp & 3) + lane;
      const int ei = i0 + erow;
      const int ech = (warp >> 2) * (BN / 2);
      const long long eqb = q0 + ech;
      const bool efull = ei < d0 && eqb + BN / 2 <= Q0;
      float4 tv[BN / 8];
      if (efull) {
        const float4* t4 = reinterpret_cast<const float4*>(T + (size_t)ei * Q0 + eqb);
#pragma unroll
        for (int u = 0; u < BN / 8; ++u) tv[u] = __ldcs(t4 + u);
      }
      // generic-proxy writes -> visible to the tensor core's async proxy
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      __syncthreads();
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      if (*(volatile int*)&S.abort) break;
      if (tid == 0) {
        uint32_t first = 1;
        for (int pass = 0; pass < 3; ++pass) {
          // hi*hi, hi*lo, lo*hi
          for (int s = 0; s < KP / 8; ++s) {
            const int atom = s >> 2, kk = s & 3;
            const unsigned char* a = (pass == 2) ? S.alo[atom] : S.ahi[atom];
            const unsigned char* b = (pass == 1) ? S.blo[atom] : S.bhi[atom];
            mma(tmem, desc(a) + (uint64_t)(kk * 2), desc(b) + (uint64_t)(kk * 2), first ? 0u : 1u);
            first = 0;
          }
        }
        asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                         su32(&S.done))
                     : "memory");
      }
      __syncwarp();
      if (!wait_bar(&S.done, phase & 1)) {
        if (lane == 0) {
          atomicExch(err, 1);
          S.abort = 1;
        }
      }
      ++phase;
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      if (!*(volatile int*)&S.abort) {
        // warp w: TMEM lanes 32*(w % 4) .. +31 (rows), columns half w / 4
#pragma unroll
        for (int cc = 0; cc < BN / 2; cc += 32) {
          uint32_t v[32];
          const uint32_t taddr = tmem + ((uint32_t)(32 * (warp & 3)) << 16) + (uint32_t)(ech + cc);
          asm volatile(
              "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
              "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
              : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
                "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]),
                "=r"(v[15]), "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]),
                "=r"(v[22]), "=r"(v[23]), "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]),
                "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
              : "r"(taddr));
          asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
          const long long qb = eqb + cc;
          if (efull) {
#pragma unroll
            for (int u = 0; u < 8; ++u) {
              const float4 t = tv[cc / 4 + u];
              float df;
              df = t.x - __uint_as_float(v[4 * u + 0]); acc[0].fma_(df, df);
              df = t.y - __uint_as_float(v[4 * u + 1]); acc[1].fma_(df, df);
              df = t.z - __uint_as_float(v[4 * u + 2]); acc[2].fma_(df, df);
              df = t.w - __uint_as_float(v[4 * u + 3]); acc[3].fma_(df, df);
            }
          } else if (ei < d0) {
            const float* trow = T + (size_t)ei * Q0 + qb;
            for (int u = 0; u < 32; ++u)
              if (qb + u < Q0) {
                const float df = trow[u] - __uint_as_float(v[u]);
                acc[u & 3].fma_(df, df);
              }
          }
        }
      }
      // every warp is done with TMEM and with this row block's operands
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      __syncthreads();
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    }
    if (*(volatile int*)&S.abort) break;
  }
  // CTA total (double), one partial per CTA
  double hv = 0.0;
  for (int a = 0; a < 4; ++a) hv += (double)acc[a].hi + (double)acc[a].lo;
  hv = warp_sum(hv);
  if (lane == 0) S.red[warp][0] = hv;
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (tid == 0) {
    double t = 0.0;
    for (int w = 0; w < NT / 32; ++w) t += S.red[w][0];
    part[blockIdx.x] = t;
  }
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 256;" ::"r"(tmem) : "memory");
}

}  // namespace rtc
}  // namespace tfx

using namespace tfx;

// Called by tfx_cp_residual for FP32 third-order tensors; returns
// TFX_STATUS_ERR_UNSUPPORTED when the shape is outside the kernel's range so the
// caller uses its SIMT kernel.  out = sum of the per-CTA partials (k_sum_partials
// is launched by the caller on `partial`); *nblocks receives the partial count.
int tfx_cp_residual_tc_launch(const float* T, const int* dims, int R, const float* W, double* partial,
                              int max_partials, int* err, int* nblocks, cudaStream_t st) {
  const long long Q0 = (long long)dims[1] * dims[2];
  // the tensor-core path pays for forming its operands once per 128 x 256 tile:
  // it wins on large tensors only (measured: 1.3-1.4x on 512^3 at rank 50)
  if (R > rtc::KP || (Q0 % 4) != 0 || Q0 >= (1LL << 31) || (((uintptr_t)T) & 15) != 0 || !err ||
      (long long)dims[0] * Q0 < (1LL << 22))
    return TFX_STATUS_ERR_UNSUPPORTED;
  static int nsm = 0;
  if (!nsm) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    if (nsm < 1) nsm = 1;
  }
  rtc::Shape sh;
  sh.d0 = dims[0];
  sh.d1 = dims[1];
  sh.d2 = dims[2];
  sh.R = R;
  sh.Q0 = Q0;
  sh.W0 = W;
  sh.W1 = W + (size_t)R * dims[0];
  sh.W2 = W + (size_t)R * (dims[0] + dims[1]);
  const int ncb = (int)((Q0 + rtc::BN - 1) / rtc::BN);
  const int grid = std::max(1, std::min(std::min(ncb, nsm), max_partials));
  const size_t sm = sizeof(rtc::Smem) + 1024;
  cudaError_t e = cudaFuncSetAttribute(rtc::k_residual_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  if (e != cudaSuccess) return tfx_set_cuda_error(e, "residual_tc smem");
  rtc::k_residual_tc<<<grid, rtc::NT, sm, st>>>(T, sh, partial, err);
  e = cudaGetLastError();
  if (e != cudaSuccess) return tfx_set_cuda_error(e, "residual_tc launch");
  tfx_count_launch(1);
  *nblocks = grid;
  return TFX_STATUS_OK;
}
