// Mode product with U^T on the 5th-generation tensor cores, 3xTF32 with FP32
// accumulation (precision 'mixed'):
//
//   out[p, j, q] = sum_d U[d, j] T[p, d, q]
//
// the MLSVD's truncation step (Compression.py:152-156, where the sequential
// method forms U_l^T S_(l) as Sigma V^T, and :170-173 with
// MultilinearAlgebra.py:72-105 multilin_mult for the classic one).  The
// contraction index d is the strided one in memory (T[p, d, q] has q
// contiguous), so the tensor is the A operand with M = q and K = d after a
// transposition in shared memory; U^T (n x D, n <= 64) is the B operand.
// Both are split x = x_hi + x_lo (x_hi: 13 low mantissa bits cleared, exact
// in TF32) and the product is A_hi B_hi + A_hi B_lo + A_lo B_hi, so the core
// keeps FP32 accuracy (a single TF32 pass moved the headline CPD's final
// error by 1%).
//
// A persistent CTA takes 128-wide q tiles.  Per tile the D axis runs in chunks
// of 32:
//   * warp 0 (producer) brings each chunk's 32 x 128 tensor tile and the
//     chunk's 64 x 32 block of U^T (K-major SWIZZLE_128B) by TMA into a
//     four-stage ring (a stage is refilled once the converters read it);
//   * warps 2-9 (converters) each take 32 rows q and half the d range of the
//     tile and write them, split hi / lo, into the A operands (128 x 32, K-major
//     SWIZZLE_128B: four d values as one 16-byte store, conflict-free), and
//     split the U^T block in place of layout, into a two-stage ring;
//   * warp 1 issues tcgen05.mma kind::tf32 (M = 128, N = 64, K = 8), three
//     per K step, into one TMEM accumulator and commits each operand stage
//     back to the converters;
//   * after a tile's last chunk the converters read the accumulator
//     (tcgen05.ld) and store out[p, j, q0 + row] for j < n.
// Every wait is bounded; a wait that runs out sets *err, the CTA stops, waits
// (bounded) for its copies and products in flight and frees TMEM.
#include <cuda.h>
#include <math.h>
#include <stdint.h>

#include <algorithm>

#include "tfx_capi_internal.h"
#include "tfx_common.cuh"

namespace tfx {
namespace ttc {

constexpr int BQ = 128, BD = 32, NJ = 64, NCW = 8, NT = 64 + 32 * NCW, TST = 4, AST = 2, DMAX = 8192;
constexpr uint32_t SPIN = 1u << 26;
constexpr uint32_t TTILE = BD * BQ * 4;      // one tensor tile, bytes
constexpr uint32_t BCHUNK = NJ * BD * 4;     // one chunk of U^T, bytes

__device__ __forceinline__ uint32_t su32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(su32(bar)), "r"(count));
}

__device__ __forceinline__ void expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(su32(bar)), "r"(bytes) : "memory");
}

__device__ __forceinline__ void arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(su32(bar)) : "memory");
}

__device__ __forceinline__ bool wait_bar(uint64_t* bar, uint32_t parity) {
  return mbar_wait_bounded(su32(bar), parity, SPIN);
}

__device__ __forceinline__ void tma_2d(void* dst, const CUtensorMap* map, uint64_t* bar, int x, int y) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
          su32(dst)),
      "l"(map), "r"(x), "r"(y), "r"(su32(bar))
      : "memory");
}

__device__ __forceinline__ void tma_3d(void* dst, const CUtensorMap* map, uint64_t* bar, int x, int y, int z) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(
          su32(dst)),
      "l"(map), "r"(x), "r"(y), "r"(z), "r"(su32(bar))
      : "memory");
}

// K-major SWIZZLE_128B operand: row r (32 fp32 of K) is 128 bytes, 8-row
// groups 1024 bytes apart, 16-byte chunk c stored at c ^ (r % 8)
__device__ __forceinline__ uint64_t desc(const void* tile) {
  const uint64_t a = su32(tile);
  uint64_t d = 0;
  d |= (a >> 4) & 0x3FFFull;          // start address
  d |= (uint64_t)1 << 16;             // leading byte offset (unused for swizzled K-major)
  d |= (uint64_t)(1024 >> 4) << 32;   // stride byte offset: 8-row groups
  d |= (uint64_t)1 << 46;             // descriptor version
  d |= (uint64_t)2 << 61;             // SWIZZLE_128B
  return d;
}

// D = F32, A = B = TF32, both K-major, M = 128, N = 64
__host__ __device__ constexpr uint32_t idesc() {
  return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(NJ >> 3) << 17) | ((uint32_t)(BQ >> 4) << 24);
}

__device__ __forceinline__ void mma(uint32_t tmem, uint64_t a, uint64_t b, uint32_t acc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem),
      "l"(a), "l"(b), "r"(idesc()), "r"(acc)
      : "memory");
}

__device__ __forceinline__ void commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(su32(bar))
               : "memory");
}

__device__ __forceinline__ float hi13(float x) { return __uint_as_float(__float_as_uint(x) & 0xFFFFE000u); }

struct Smem {
  alignas(1024) unsigned char t[TST][TTILE];           // tensor tiles [32 d][128 q]
  alignas(1024) unsigned char u[TST][BCHUNK];          // U^T blocks, 64 rows j x 32 d (swizzled)
  alignas(1024) unsigned char ahi[AST][BQ * 128];      // transposed tiles: 128 rows q x 32 d
  alignas(1024) unsigned char alo[AST][BQ * 128];
  alignas(1024) unsigned char bhi[AST][BCHUNK];
  alignas(1024) unsigned char blo[AST][BCHUNK];
  alignas(8) uint64_t tfull[TST];
  alignas(8) uint64_t tfree[TST];
  alignas(8) uint64_t afull[AST];
  alignas(8) uint64_t afree[AST];
  alignas(8) uint64_t accfull;
  alignas(8) uint64_t accfree;
  uint32_t tmem;
  int abort;
  int tissued;    // chunks whose tensor copies the producer issued
  int tconsumed;  // chunks the converters took from the ring
  int missued;    // chunks whose products were issued
};

struct Shape {
  int D, n, dchunks;
  long long P, Q;
  int qtiles;
};

__global__ void __launch_bounds__(NT, 1)
    k_ttm_tc(const __grid_constant__ CUtensorMap tmap, const __grid_constant__ CUtensorMap umap, Shape sh,
             float* __restrict__ out, int* err) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  Smem& S = *reinterpret_cast<Smem*>((((uintptr_t)smem_raw) + 1023) & ~(uintptr_t)1023);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int DC = sh.dchunks;
  const long long ntiles = sh.P * sh.qtiles;
  // this CTA's tiles: blockIdx.x, blockIdx.x + gridDim.x, ...
  const int mytiles = ntiles > blockIdx.x ? (int)((ntiles - 1 - blockIdx.x) / gridDim.x + 1) : 0;
  const int nchunk = mytiles * DC;
  if (tid == 0) {
    for (int s = 0; s < TST; ++s) {
      mbar_init(&S.tfull[s], 1);
      mbar_init(&S.tfree[s], NCW);
    }
    for (int s = 0; s < AST; ++s) {
      mbar_init(&S.afull[s], NCW);
      mbar_init(&S.afree[s], 1);
    }
    mbar_init(&S.accfull, 1);
    mbar_init(&S.accfree, NCW);
    S.abort = 0;
    S.tissued = 0;
    S.tconsumed = 0;
    S.missued = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 64;" ::"r"(su32(&S.tmem)) : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = S.tmem;
  auto tile_of = [&](int local, long long& p, long long& q0) {
    const long long t = blockIdx.x + (long long)local * gridDim.x;
    p = t / sh.qtiles;
    q0 = (t - p * sh.qtiles) * BQ;
  };
  if (warp == 0) {
    // producer: every chunk's tensor tile and U^T block
    if (lane == 0 && nchunk > 0) {
      for (int g = 0; g < nchunk; ++g) {
        const int s = g % TST;
        if (g >= TST && !wait_bar(&S.tfree[s], (uint32_t)(g / TST - 1) & 1u)) {
          atomicExch(err, 4);
          S.abort = 1;
        }
        if (*(volatile int*)&S.abort) break;
        long long p, q0;
        tile_of(g / DC, p, q0);
        const int c = g - (g / DC) * DC;
        expect_tx(&S.tfull[s], TTILE + BCHUNK);
        tma_3d(S.t[s], &tmap, &S.tfull[s], (int)q0, c * BD, (int)p);
        tma_2d(S.u[s], &umap, &S.tfull[s], c * BD, 0);
        S.tissued = g + 1;
      }
    }
  } else if (warp == 1) {
    // MMA issuer
    if (lane == 0 && nchunk > 0) {
      for (int g = 0; g < nchunk && !*(volatile int*)&S.abort; ++g) {
        const int as = g % AST, c = g % DC, tl = g / DC;
        if (!wait_bar(&S.afull[as], (uint32_t)(g / AST) & 1u)) {
          atomicExch(err, 6);
          S.abort = 1;
          break;
        }
        if (c == 0 && tl > 0 && !wait_bar(&S.accfree, (uint32_t)(tl - 1) & 1u)) {
          atomicExch(err, 7);
          S.abort = 1;
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const uint64_t ah = desc(S.ahi[as]), al = desc(S.alo[as]);
        const uint64_t bh = desc(S.bhi[as]), bl = desc(S.blo[as]);
#pragma unroll
        for (int pass = 0; pass < 3; ++pass) {
          // hi*hi, hi*lo, lo*hi
          const uint64_t da = pass == 2 ? al : ah, db = pass == 1 ? bl : bh;
#pragma unroll
          for (int kk = 0; kk < BD / 8; ++kk)
            mma(tmem, da + (uint64_t)(kk * 2), db + (uint64_t)(kk * 2), (c > 0 || pass > 0 || kk > 0) ? 1u : 0u);
        }
        commit(&S.afree[as]);
        if (c == DC - 1) commit(&S.accfull);
        S.missued = g + 1;
      }
    }
  } else {
    // converters (warps 2-9): transpose, then the epilogue of each finished tile
    const int cw = warp - 2;
    const int qr = (cw & 3) * 32 + lane;        // the row this thread transposes
    const int dh = cw >> 2;                     // its half of the chunk's d range
    const int erow = 32 * (warp & 3) + lane;    // the accumulator lane it reads
    for (int g = 0; g < nchunk; ++g) {
      const int s = g % TST, as = g % AST, c = g % DC, tl = g / DC;
      if (!wait_bar(&S.tfull[s], (uint32_t)(g / TST) & 1u)) {
        if (lane == 0) {
          atomicExch(err, 1);
          S.abort = 1;
        }
      }
      if (g >= AST && !wait_bar(&S.afree[as], (uint32_t)(g / AST - 1) & 1u)) {
        if (lane == 0) {
          atomicExch(err, 2);
          S.abort = 1;
        }
      }
      if (*(volatile int*)&S.abort) break;
      if (warp == 2 && lane == 0) S.tconsumed = g + 1;
      {
        const float* tt = reinterpret_cast<const float*>(S.t[s]);
        const uint32_t ro = (uint32_t)qr * 128;
#pragma unroll
        for (int d4 = dh * (BD / 8); d4 < (dh + 1) * (BD / 8); ++d4) {
          float4 v, h, lo;
          v.x = tt[(4 * d4 + 0) * BQ + qr];
          v.y = tt[(4 * d4 + 1) * BQ + qr];
          v.z = tt[(4 * d4 + 2) * BQ + qr];
          v.w = tt[(4 * d4 + 3) * BQ + qr];
          h.x = hi13(v.x); lo.x = v.x - h.x;
          h.y = hi13(v.y); lo.y = v.y - h.y;
          h.z = hi13(v.z); lo.z = v.z - h.z;
          h.w = hi13(v.w); lo.w = v.w - h.w;
          const uint32_t o = ro + ((((uint32_t)d4 ^ (uint32_t)(qr & 7)) & 7u) << 4);
          *reinterpret_cast<float4*>(S.ahi[as] + o) = h;
          *reinterpret_cast<float4*>(S.alo[as] + o) = lo;
        }
        // U^T block: element-wise, the layout stays (the MMA reads hi and lo
        // with the same descriptor form)
        const float4* u4 = reinterpret_cast<const float4*>(S.u[s]);
        float4* bh4 = reinterpret_cast<float4*>(S.bhi[as]);
        float4* bl4 = reinterpret_cast<float4*>(S.blo[as]);
        for (int e = cw * 32 + lane; e < (int)(BCHUNK / 16); e += 32 * NCW) {
          const float4 v = u4[e];
          float4 h, lo;
          h.x = hi13(v.x); lo.x = v.x - h.x;
          h.y = hi13(v.y); lo.y = v.y - h.y;
          h.z = hi13(v.z); lo.z = v.z - h.z;
          h.w = hi13(v.w); lo.w = v.w - h.w;
          bh4[e] = h;
          bl4[e] = lo;
        }
      }
      // generic-proxy writes -> visible to the tensor core's async proxy; the
      // tensor stage goes back to the producer, the operand to the MMA warp
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      __syncwarp();
      if (lane == 0) {
        arrive(&S.tfree[s]);
        arrive(&S.afull[as]);
      }
      if (c == DC - 1) {
        // the tile's accumulator: rows q0 + erow, columns j
        if (!wait_bar(&S.accfull, (uint32_t)tl & 1u)) {
          if (lane == 0) {
            atomicExch(err, 3);
            S.abort = 1;
          }
        }
        if (*(volatile int*)&S.abort) break;
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        long long p, q0;
        tile_of(tl, p, q0);
        const long long q = q0 + erow;
        float* orow = out + (size_t)p * sh.n * sh.Q + q;
#pragma unroll 1
        for (int cc = dh * 32; cc < (dh + 1) * 32; cc += 32) {
          uint32_t v[32];
          const uint32_t taddr = tmem + ((uint32_t)(32 * (warp & 3)) << 16) + (uint32_t)cc;
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
          if (q < sh.Q)
#pragma unroll
            for (int j = 0; j < 32; ++j)
              if (cc + j < sh.n) orow[(size_t)(cc + j) * sh.Q] = __uint_as_float(v[j]);
        }
        // every read of the accumulator is done before the next tile's products
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        __syncwarp();
        if (lane == 0) arrive(&S.accfree);
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  // after an abort: every issued copy lands and every issued product finishes
  // (bounded waits) before the CTA frees TMEM and exits
  if (tid == 0 && *(volatile int*)&S.abort) {
    const int issued = S.tissued, consumed = S.tconsumed, mi = S.missued;
    for (int g = consumed; g < issued; ++g) wait_bar(&S.tfull[g % TST], (uint32_t)(g / TST) & 1u);
    if (mi > 0) wait_bar(&S.afree[(mi - 1) % AST], (uint32_t)((mi - 1) / AST) & 1u);
  }
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 64;" ::"r"(tmem) : "memory");
}

typedef CUresult (*EncodeFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                             const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                             CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static EncodeFn encode_fn() {
  static EncodeFn fn = nullptr;
  if (!fn) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (EncodeFn)p;
  }
  return fn;
}

static int sms() {
  int dev = 0, n = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
  return n < 1 ? 1 : n;
}

}  // namespace ttc
}  // namespace tfx

using namespace tfx;

extern "C" int tfx_ttm_tc_supported(long long P, int D, long long Q, int n) {
  return P >= 1 && P <= 0x7fffffffLL && D >= ttc::BD && D <= ttc::DMAX && D % ttc::BD == 0 && n >= 1 &&
         n <= ttc::NJ && Q >= ttc::BQ && Q % 4 == 0 && Q <= 0x7fffffffLL;
}

// S: (P, D, Q) C-order FP32, 16-byte aligned; Ut: n x D row-major (U^T),
// 16-byte aligned; out: (P, n, Q).  err: device int, set non-zero when a
// bounded wait ran out (the caller raises on it).
extern "C" int tfx_ttm_tc(const float* S, long long P, int D, long long Q, const float* Ut, int n, float* out,
                          int* err, void* stream) {
  if (!S || !Ut || !out || !err) return tfx_set_error(TFX_STATUS_ERR_ARG, "ttm_tc args");
  if (!tfx_ttm_tc_supported(P, D, Q, n))
    return tfx_set_error(TFX_STATUS_ERR_UNSUPPORTED, "ttm_tc: D % 32 == 0, n <= 64, Q >= 128, Q % 4 == 0");
  if (((uintptr_t)S & 15) != 0 || ((uintptr_t)Ut & 15) != 0)
    return tfx_set_error(TFX_STATUS_ERR_ARG, "ttm_tc needs 16-byte aligned operands");
  ttc::EncodeFn enc = ttc::encode_fn();
  if (!enc) return tfx_set_error(TFX_STATUS_ERR_UNSUPPORTED, "cuTensorMapEncodeTiled unavailable");
  CUtensorMap tmap, umap;
  {
    const cuuint64_t gdim[3] = {(cuuint64_t)Q, (cuuint64_t)D, (cuuint64_t)P};
    const cuuint64_t gstride[2] = {(cuuint64_t)Q * 4, (cuuint64_t)Q * D * 4};
    const cuuint32_t box[3] = {ttc::BQ, ttc::BD, 1};
    const cuuint32_t estr[3] = {1, 1, 1};
    CUresult r = enc(&tmap, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, (void*)S, gdim, gstride, box, estr,
                     CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                     CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return tfx_set_error(TFX_STATUS_ERR_ARG, "ttm_tc tensor map encoding failed");
  }
  {
    const cuuint64_t gdim[2] = {(cuuint64_t)D, (cuuint64_t)n};
    const cuuint64_t gstride[1] = {(cuuint64_t)D * 4};
    const cuuint32_t box[2] = {ttc::BD, ttc::NJ};
    const cuuint32_t estr[2] = {1, 1};
    CUresult r = enc(&umap, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, (void*)Ut, gdim, gstride, box, estr,
                     CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                     CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return tfx_set_error(TFX_STATUS_ERR_ARG, "ttm_tc U map encoding failed");
  }
  ttc::Shape sh;
  sh.D = D;
  sh.n = n;
  sh.dchunks = D / ttc::BD;
  sh.P = P;
  sh.Q = Q;
  sh.qtiles = (int)((Q + ttc::BQ - 1) / ttc::BQ);
  const long long ntiles = P * sh.qtiles;
  const int grid = (int)std::max<long long>(1, std::min<long long>(ntiles, ttc::sms()));
  cudaStream_t st = (cudaStream_t)stream;
  const size_t sm = sizeof(ttc::Smem) + 1024;
  cudaError_t e = cudaFuncSetAttribute(ttc::k_ttm_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  if (e != cudaSuccess) return tfx_set_cuda_error(e, "ttm_tc smem");
  ttc::k_ttm_tc<<<grid, ttc::NT, sm, st>>>(tmap, umap, sh, out, err);
  e = cudaGetLastError();
  if (e != cudaSuccess) return tfx_set_cuda_error(e, "ttm_tc launch");
  tfx_count_launch(1);
  return TFX_STATUS_OK;
}
