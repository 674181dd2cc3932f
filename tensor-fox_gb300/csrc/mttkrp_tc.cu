// MTTKRP of a dense FP32 tensor on the 5th-generation tensor cores, fed by TMA.
//
//   M[d, r] = sum_p sum_q T[p, d, q] * before_p[r] * after_q[r]
//
// with the tensor viewed as (P, D, Q) for mode l (P = prod of the earlier
// dims, D = d_l, Q = prod of the later dims), before_p[r] = prod_{m<l}
// W_m[i_m(p), r] and after_q[r] = prod_{m>l} W_m[i_m(q), r]: the product
// T_(l) KR_l of GaussNewton.py:411-423 (the gradient's contraction,
// GaussNewton.py:401-427).  Summing over p inside the accumulator turns every
// mode but the last into one GEMM whose A operand is the tensor itself, rows d
// contiguous in q (K-major), so TMA loads it straight from the C-order tensor.
// The last mode has no contiguous K and is served by a copy of the tensor with
// that mode moved to the front (its mode 0).
//
// A CTA owns 256 rows of M (two 128-row tiles, two TMEM accumulators of 64
// columns) and a contiguous range of (p, 32-wide q chunk) pairs (split-K):
//   * warp 0 (producer) brings the two 128 x 32 tensor tiles of a chunk by TMA
//     (3-D map over (q, d, p), SWIZZLE_128B) into a two-stage ring, a stage
//     being refilled as soon as the products that read it have completed;
//   * warps 2-17 form the chunk's B operand (64 x 32, K-major, SWIZZLE_128B)
//     from the factor rows as soon as the stage's previous products are done
//     (while the tensor tiles are still in flight), then split every tile
//     value x into x_hi = x with its 13 low mantissa bits cleared (exact in
//     TF32) and x_lo = x - x_hi, B the same way, and arrive on the stage's
//     "formed" mbarrier;
//   * warp 1 issues tcgen05.mma kind::tf32 (M = 128, N = 64, K = 8):
//     A_hi B_hi + A_hi B_lo + A_lo B_hi per tile, FP32 accumulation in TMEM,
//     so the product keeps FP32 accuracy (3xTF32), and commits to the stage's
//     mbarrier, while the converters work on the next chunk.
// The accumulators are written as per-CTA partials and summed in a fixed
// order (compensated FP32) by a second kernel.  Every wait is bounded; a wait
// that runs out sets *err, the CTA drains its copies (bounded) and frees TMEM.
#include <cuda.h>
#include <math.h>
#include <stdint.h>

#include <algorithm>

#include "tfx_capi_internal.h"
#include "tfx_common.cuh"

namespace tfx {
namespace mtc {

constexpr int BM = 128, BK = 32, NR = 64, NTILE = 2, NT = 576, STAGES = 2;
constexpr uint32_t SPIN = 1u << 26;
constexpr uint32_t TILE_BYTES = BM * BK * 4;

__device__ __forceinline__ uint32_t su32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(su32(bar)), "r"(count));
}

__device__ __forceinline__ void expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(su32(bar)), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool wait_bar(uint64_t* bar, uint32_t parity) {
  return mbar_wait_bounded(su32(bar), parity, SPIN);
}

__device__ __forceinline__ void tma_3d(void* dst, const CUtensorMap* map, uint64_t* bar, int x, int y, int z) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(
          su32(dst)),
      "l"(map), "r"(x), "r"(y), "r"(z), "r"(su32(bar))
      : "memory");
}

// K-major SWIZZLE_128B: row r of an atom (32 fp32 of K) is 128 bytes, 8-row
// groups 1024 bytes apart, 16-byte chunk c stored at c ^ (r % 8)
__device__ __forceinline__ uint32_t sw_off(int r, int k) {
  return (uint32_t)(r * 128 + ((((k >> 2) ^ (r & 7)) & 7) << 4) + ((k & 3) << 2));
}

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
  return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(NR >> 3) << 17) | ((uint32_t)(BM >> 4) << 24);
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
  alignas(1024) unsigned char a[STAGES][NTILE][BM * 128];
  alignas(1024) unsigned char alo[STAGES][NTILE][BM * 128];
  alignas(1024) unsigned char bhi[STAGES][NR * 128];
  alignas(1024) unsigned char blo[STAGES][NR * 128];
  alignas(8) uint64_t full[STAGES];
  alignas(8) uint64_t done[STAGES];
  alignas(8) uint64_t conv[STAGES];
  uint32_t tmem;
  int abort;
  int issued;    // chunks whose copies the producer issued
  int consumed;  // chunks whose products were issued
};

// The factors in the kernel's mode order: mode m of the (possibly permuted)
// tensor has dims[m] rows, column r of W_m at W[m] + r * dims[m].
struct Shape {
  int L, R, mode, D;
  long long P, Q;
  int dims[TFX_MAX_ORDER];
  const float* W[TFX_MAX_ORDER];
};

__global__ void __launch_bounds__(NT, 1)
    k_mttkrp_tc(const __grid_constant__ CUtensorMap tmap, Shape sh, int qchunks, int ksplit, float* __restrict__ part,
                int* err) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  Smem& S = *reinterpret_cast<Smem*>((((uintptr_t)smem_raw) + 1023) & ~(uintptr_t)1023);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int group = blockIdx.x / ksplit, split = blockIdx.x - group * ksplit;
  const int row0 = group * (NTILE * BM);
  const long long nchunk = sh.P * qchunks;
  const long long cbeg = nchunk * split / ksplit, cend = nchunk * (split + 1) / ksplit;
  const int n = (int)(cend - cbeg);
  const int R = sh.R, l = sh.mode;
  if (tid == 0) {
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(&S.full[s], 1);
      mbar_init(&S.done[s], 1);
      mbar_init(&S.conv[s], NT / 32 - 2);
    }
    S.abort = 0;
    S.issued = 0;
    S.consumed = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 128;" ::"r"(su32(&S.tmem))
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = S.tmem;
  auto issue = [&](int c) {  // the producer: TMA of chunk cbeg + c into stage c % 2
    const long long cc = cbeg + c;
    const int p = (int)(cc / qchunks);
    const int q0 = (int)(cc - (long long)p * qchunks) * BK;
    const int s = c & 1;
    expect_tx(&S.full[s], NTILE * TILE_BYTES);
    for (int t = 0; t < NTILE; ++t) tma_3d(S.a[s][t], &tmap, &S.full[s], q0, row0 + t * BM, p);
  };
  constexpr int NCW = NT / 32 - 2;  // converter warps (2..17: 6 -> 16 took a mode from 0.34 to 0.27 ms)
  if (warp == 0) {
    // producer: chunk c goes into stage c % 2 once the products of chunk c - 2
    // (the stage's last reader) have completed
    if (lane == 0) {
      for (int c = 0; c < n; ++c) {
        const int s = c & 1;
        if (c >= 2 && !wait_bar(&S.done[s], (uint32_t)((c - 2) >> 1) & 1u)) {
          atomicExch(err, 4);
          S.abort = 1;
        }
        if (*(volatile int*)&S.abort) break;
        issue(c);
        S.issued = c + 1;
      }
    }
  } else if (warp == 1) {
    // MMA issuer: the products of chunk c once its operands are formed
    if (lane == 0) {
      for (int c = 0; c < n; ++c) {
        const int s = c & 1;
        if (!wait_bar(&S.conv[s], (uint32_t)(c >> 1) & 1u)) {
          atomicExch(err, 5);
          S.abort = 1;
        }
        if (*(volatile int*)&S.abort) break;
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        for (int t = 0; t < NTILE; ++t) {
          const uint64_t ah = desc(S.a[s][t]), al = desc(S.alo[s][t]);
          const uint64_t bh = desc(S.bhi[s]), bl = desc(S.blo[s]);
          for (int pass = 0; pass < 3; ++pass) {
            const uint64_t da = pass == 2 ? al : ah;
            const uint64_t db = pass == 1 ? bl : bh;
#pragma unroll
            for (int kk = 0; kk < BK / 8; ++kk)
              mma(tmem + (uint32_t)(t * NR), da + (uint64_t)(kk * 2), db + (uint64_t)(kk * 2),
                  (c > 0 || pass > 0 || kk > 0) ? 1u : 0u);
          }
        }
        commit(&S.done[s]);
        S.consumed = c + 1;
      }
      // every product has finished before TMEM is read
      if (n > 0 && !*(volatile int*)&S.abort) {
        const int c = n - 1;
        if (!wait_bar(&S.done[c & 1], (uint32_t)(c >> 1) & 1u)) {
          atomicExch(err, 3);
          S.abort = 1;
        }
      }
    }
  } else {
    // converters (warps 2..17): form B, split the tiles, hand the stage over.
    // B does not depend on the tensor tile: it is formed as soon as the
    // stage's previous products (chunk c - 2) have completed, while the
    // chunk's TMA copy is still in flight.
    const int ct = tid - 64;
    for (int c = 0; c < n; ++c) {
      const int s = c & 1;
      if (c >= 2 && !wait_bar(&S.done[s], (uint32_t)((c - 2) >> 1) & 1u)) {
        if (lane == 0) {
          atomicExch(err, 6);
          S.abort = 1;
        }
      }
      if (*(volatile int*)&S.abort) break;
      // B: 64 x 32, B[r][q] = before_p[r] * after_{q0+q}[r].  A thread takes
      // one q (its lane) and the ranks r = (warp - 2) + NCW u; the indices of p
      // and q are decomposed once per chunk (32-bit: P, Q < 2^31) into
      // registers (loops unrolled over the modes), then one factor load per
      // other mode and rank.
      {
        const long long cc = cbeg + c;
        const unsigned p = (unsigned)(cc / qchunks);
        const unsigned q = (unsigned)(cc - (long long)p * qchunks) * BK + (unsigned)lane;
        const bool qok = q < (unsigned)sh.Q;
        int idx[TFX_MAX_ORDER];
        unsigned rb = p, ra = qok ? q : 0u;
#pragma unroll
        for (int m = TFX_MAX_ORDER - 1; m >= 0; --m) {
          idx[m] = 0;
          if (m < sh.L && m != l) {
            const unsigned dm = (unsigned)sh.dims[m];
            unsigned& rem = (m < l) ? rb : ra;
            const unsigned qm = rem / dm;
            idx[m] = (int)(rem - qm * dm);
            rem = qm;
          }
        }
        // every factor load of a mode is issued before any is used: one L2
        // round trip per mode instead of one per rank
        constexpr int NU = (NR + NCW - 1) / NCW;
        float v[NU];
#pragma unroll
        for (int u = 0; u < NU; ++u) {
          const int r = warp - 2 + NCW * u;
          v[u] = (r < R && qok) ? 1.f : 0.f;
        }
#pragma unroll
        for (int m = 0; m < TFX_MAX_ORDER; ++m) {
          if (m < sh.L && m != l) {
            const float* wm = sh.W[m] + idx[m];
            const long long dm = sh.dims[m];
            float w[NU];
#pragma unroll
            for (int u = 0; u < NU; ++u) {
              const int r = warp - 2 + NCW * u;
              w[u] = (r < R && qok) ? __ldg(wm + (long long)r * dm) : 0.f;
            }
#pragma unroll
            for (int u = 0; u < NU; ++u) v[u] *= w[u];
          }
        }
#pragma unroll
        for (int u = 0; u < NU; ++u) {
          const int r = warp - 2 + NCW * u;
          if (r < NR) {
            const float h = hi13(v[u]);
            const uint32_t o = sw_off(r, lane);
            *(float*)(S.bhi[s] + o) = h;
            *(float*)(S.blo[s] + o) = v[u] - h;
          }
        }
      }
      if (!wait_bar(&S.full[s], (uint32_t)(c >> 1) & 1u)) {
        if (lane == 0) {
          atomicExch(err, 1);
          S.abort = 1;
        }
      }
      if (*(volatile int*)&S.abort) break;
      // A: hi in place, lo beside it (element-wise: the layout is the same)
      {
        float4* a4 = reinterpret_cast<float4*>(&S.a[s][0][0]);
        float4* l4 = reinterpret_cast<float4*>(&S.alo[s][0][0]);
        for (int e = ct; e < NTILE * BM * BK / 4; e += NCW * 32) {
          const float4 v = a4[e];
          float4 h, lo;
          h.x = hi13(v.x); lo.x = v.x - h.x;
          h.y = hi13(v.y); lo.y = v.y - h.y;
          h.z = hi13(v.z); lo.z = v.z - h.z;
          h.w = hi13(v.w); lo.w = v.w - h.w;
          a4[e] = h;
          l4[e] = lo;
        }
      }
      // generic-proxy writes -> visible to the tensor core's async proxy; one
      // arrival per converter warp
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      __syncwarp();
      if (lane == 0) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(su32(&S.conv[s])) : "memory");
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  // after an abort: every copy issued lands and every product committed
  // finishes (bounded waits) before the CTA frees TMEM and exits
  if (tid == 0 && *(volatile int*)&S.abort) {
    const int issued = S.issued, consumed = S.consumed;
    for (int c = consumed; c < issued; ++c) wait_bar(&S.full[c & 1], (uint32_t)(c >> 1) & 1u);
    if (consumed > 0) wait_bar(&S.done[(consumed - 1) & 1], (uint32_t)((consumed - 1) >> 1) & 1u);
  }
  __syncthreads();
  const bool ok = !*(volatile int*)&S.abort;
  // epilogue: warp w < 8 reads TMEM lanes 32 (w % 4) .. + 31 of tile w / 4
  if (warp < 4 * NTILE) {
    const int t = warp >> 2;
    const int row = row0 + t * BM + 32 * (warp & 3) + lane;
    float* out = part + (size_t)split * sh.D * R;
#pragma unroll 1
    for (int cc = 0; cc < NR; cc += 32) {
      uint32_t v[32];
      if (ok && n > 0) {
        const uint32_t taddr = tmem + ((uint32_t)(32 * (warp & 3)) << 16) + (uint32_t)(t * NR + cc);
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
      } else {
#pragma unroll
        for (int j = 0; j < 32; ++j) v[j] = 0u;
      }
      if (row < sh.D)
        for (int j = 0; j < 32; ++j)
          if (cc + j < R) out[(size_t)row * R + cc + j] = __uint_as_float(v[j]);
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 128;" ::"r"(tmem) : "memory");
}

// M = sum over the split-K partials, fixed order, compensated FP32; written
// row-major (D x R) or, with col_major, as column-major (column r contiguous)
__global__ void k_mttkrp_tc_reduce(const float* __restrict__ part, int D, int R, int ksplit, int col_major,
                                   float* __restrict__ out) {
  const long long n = (long long)D * R;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
    Acc<float> s;
    for (int k = 0; k < ksplit; ++k) s.add(__ldcs(part + (size_t)k * n + e));
    const long long d = e / R, r = e - d * R;
    out[col_major ? r * D + d : e] = s.hi + s.lo;
  }
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

// split-K count: about one wave of CTAs over the row groups
static int ksplit_for(int groups, long long nchunk) {
  long long k = (sms() + groups - 1) / groups;
  k = std::max<long long>(1, std::min<long long>(k, nchunk));
  return (int)k;
}

}  // namespace mtc
}  // namespace tfx

using namespace tfx;

extern "C" size_t tfx_mttkrp_tc_scratch_bytes(int L, const int* dims, int R, int mode) {
  if (L < 3 || L > TFX_MAX_ORDER || !dims || mode < 0 || mode >= L) return 0;
  const long long D = dims[mode];
  long long P = 1, Q = 1;
  for (int m = 0; m < mode; ++m) P *= dims[m];
  for (int m = mode + 1; m < L; ++m) Q *= dims[m];
  const int groups = (int)((D + mtc::NTILE * mtc::BM - 1) / (mtc::NTILE * mtc::BM));
  const int ks = mtc::ksplit_for(groups, P * ((Q + mtc::BK - 1) / mtc::BK));
  return (size_t)ks * D * R * 4 + 256;
}

// T: C-order FP32 tensor of dims (L modes), 16-byte aligned, prod of the dims
// after `mode` a multiple of 4; W: HOST array of L device pointers to the
// factors (column r of W_m at W[m] + r * dims[m]); out: d_mode x R row-major, or column-major with
// col_major = 1.  mode < L - 1 (the last mode has no contiguous K: pass a copy
// of the tensor with that mode first).
extern "C" int tfx_mttkrp_tc(const float* T, int L, const int* dims, int R, const float* const* W, int mode,
                             float* out, int col_major, void* scratch, size_t scratch_bytes, int* err, void* stream) {
  if (!T || !dims || !W || !out || !scratch || !err || L < 2 || L > TFX_MAX_ORDER || mode < 0 || mode >= L - 1 ||
      R < 1 || R > mtc::NR)
    return tfx_set_error(TFX_STATUS_ERR_ARG, "mttkrp_tc args (R <= 64, mode < L - 1)");
  long long P = 1, Q = 1;
  for (int m = 0; m < L; ++m)
    if (dims[m] < 1) return tfx_set_error(TFX_STATUS_ERR_ARG, "mttkrp_tc dims");
  for (int m = 0; m < mode; ++m) P *= dims[m];
  for (int m = mode + 1; m < L; ++m) Q *= dims[m];
  const int D = dims[mode];
  if ((Q % 4) != 0 || ((uintptr_t)T & 15) != 0)
    return tfx_set_error(TFX_STATUS_ERR_ARG, "mttkrp_tc needs the later dims' product % 4 == 0 and a 16-byte aligned tensor");
  if (P > 0x7fffffffLL || Q > 0x7fffffffLL) return tfx_set_error(TFX_STATUS_ERR_ARG, "mttkrp_tc extent");
  mtc::EncodeFn enc = mtc::encode_fn();
  if (!enc) return tfx_set_error(TFX_STATUS_ERR_UNSUPPORTED, "cuTensorMapEncodeTiled unavailable");
  const int qchunks = (int)((Q + mtc::BK - 1) / mtc::BK);
  const int groups = (D + mtc::NTILE * mtc::BM - 1) / (mtc::NTILE * mtc::BM);
  const int ks = mtc::ksplit_for(groups, P * qchunks);
  if (scratch_bytes < (size_t)ks * D * R * 4) return tfx_set_error(TFX_STATUS_ERR_ARG, "mttkrp_tc scratch too small");
  mtc::Shape sh;
  sh.L = L;
  sh.R = R;
  sh.mode = mode;
  sh.D = D;
  sh.P = P;
  sh.Q = Q;
  for (int m = 0; m < L; ++m) {
    if (!W[m]) return tfx_set_error(TFX_STATUS_ERR_ARG, "mttkrp_tc factor pointer");
    sh.dims[m] = dims[m];
    sh.W[m] = W[m];
  }
  cudaError_t e;
  CUtensorMap map;
  const cuuint64_t gdim[3] = {(cuuint64_t)Q, (cuuint64_t)D, (cuuint64_t)P};
  const cuuint64_t gstride[2] = {(cuuint64_t)Q * 4, (cuuint64_t)Q * D * 4};
  const cuuint32_t box[3] = {mtc::BK, mtc::BM, 1};
  const cuuint32_t estr[3] = {1, 1, 1};
  CUresult r = enc(&map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, (void*)T, gdim, gstride, box, estr,
                   CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                   CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return tfx_set_error(TFX_STATUS_ERR_ARG, "tensor map encoding failed");
  cudaStream_t st = (cudaStream_t)stream;
  const size_t sm = sizeof(mtc::Smem) + 1024;
  e = cudaFuncSetAttribute(mtc::k_mttkrp_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  if (e != cudaSuccess) return tfx_set_cuda_error(e, "mttkrp_tc smem");
  mtc::k_mttkrp_tc<<<groups * ks, mtc::NT, sm, st>>>(map, sh, qchunks, ks, (float*)scratch, err);
  e = cudaGetLastError();
  if (e != cudaSuccess) return tfx_set_cuda_error(e, "mttkrp_tc launch");
  tfx_count_launch(1);
  const long long n = (long long)D * R;
  const int rb = (int)std::max<long long>(1, std::min<long long>((n + 255) / 256, 4LL * mtc::sms()));
  mtc::k_mttkrp_tc_reduce<<<rb, 256, 0, st>>>((const float*)scratch, D, R, ks, col_major, out);
  e = cudaGetLastError();
  if (e != cudaSuccess) return tfx_set_cuda_error(e, "mttkrp_tc reduce");
  tfx_count_launch(1);
  return TFX_STATUS_OK;
}
