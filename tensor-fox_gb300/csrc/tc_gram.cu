// Mode Gram S_(l) S_(l)^T on the 5th-generation tensor cores (tcgen05, TF32).
//
// The unfolding is read straight from the C-order tensor through a 3-D TMA
// tensor map over (q, i, p) -- the tensor viewed as (P, D, Q) with q contiguous
// -- so both MMA operands are K-major SWIZZLE_128B tiles of 128 rows x 32 fp32.
// One CTA computes a 128 x 128 block (bi, bj), bi <= bj, of the Gram over a
// slice of the contraction index k = (p, q); the FP32 accumulator lives in
// TMEM.  Warp 0 issues TMA loads into a ring of shared-memory stages, warp 1
// issues tcgen05.mma (kind::tf32, M = N = 128, K = 8, four per stage), and all
// four warps read the accumulator back with tcgen05.ld for the epilogue.
// Split-K partials are summed in float-float (compensated FP32).
//
// Replaces the streaming passes of the randomized SVD (Compression.py:337-518)
// for dense modes with Q a multiple of 4 (TMA row pitch) and Q >= 32.
//
// Every mbarrier wait is bounded: on timeout the kernel records an error code,
// skips its epilogue, waits (bounded) for copies it issued and frees its TMEM.
#include <cuda.h>
#include <math.h>

#include <algorithm>

#include "tfx_capi_internal.h"
#include "tfx_common.cuh"

namespace tfx {

#define TCG_STAGES 5
#define TCG_BM 128
#define TCG_BK 32  // fp32 elements per 128-byte swizzled row
#define TCG_TILE_BYTES (TCG_BM * TCG_BK * 4)
#define TCG_SPIN_LIMIT (1u << 26)

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

// bounded wait for phase `parity`; returns false on timeout
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
  return mbar_wait_bounded(smem_u32(bar), parity, TCG_SPIN_LIMIT);
}

__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, uint64_t* bar, int x, int y, int z) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(
          smem_u32(dst)),
      "l"(map), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
      : "memory");
}

// shared-memory matrix descriptor: K-major, SWIZZLE_128B, 8-row groups 1024 B apart
__device__ __forceinline__ uint64_t sw128_desc(const void* tile) {
  const uint64_t addr = smem_u32(tile);
  uint64_t d = 0;
  d |= (addr >> 4) & 0x3FFFull;          // start address
  d |= (uint64_t)1 << 16;                // leading byte offset (unused for swizzled K-major)
  d |= (uint64_t)(1024 >> 4) << 32;      // stride byte offset
  d |= (uint64_t)1 << 46;                // descriptor version
  d |= (uint64_t)2 << 61;                // SWIZZLE_128B
  return d;
}

// instruction descriptor: D = F32, A = B = TF32, both K-major, M = 128, N = 128
__host__ __device__ constexpr uint32_t tf32_idesc() {
  return (1u << 4) | (2u << 7) | (2u << 10) | ((128u >> 3) << 17) | ((128u >> 4) << 24);
}

__device__ __forceinline__ void mma_tf32(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem_d),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

struct TcGramSmem {
  alignas(1024) unsigned char a[TCG_STAGES][TCG_TILE_BYTES];
  alignas(1024) unsigned char b[TCG_STAGES][TCG_TILE_BYTES];
  alignas(8) uint64_t full[TCG_STAGES];
  alignas(8) uint64_t empty[TCG_STAGES];
  alignas(8) uint64_t done;
  uint32_t tmem_base;
  int abort;
};

__global__ void __launch_bounds__(128, 1)
    k_gram_tc(const __grid_constant__ CUtensorMap tmap, int D, long long P, int qchunks, int ksplit, float* part,
              int* err) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  // align the carve-out to 1024 bytes (SWIZZLE_128B atoms)
  TcGramSmem& S = *reinterpret_cast<TcGramSmem*>((((uintptr_t)smem_raw) + 1023) & ~(uintptr_t)1023);
  const int nt = (D + TCG_BM - 1) / TCG_BM;
  int t = blockIdx.x, bi = 0;
  while (t >= nt - bi) {
    t -= nt - bi;
    ++bi;
  }
  const int bj = bi + t;
  const bool diag = bi == bj;
  const long long nchunk = P * qchunks;
  const long long c0 = nchunk * blockIdx.y / ksplit, c1 = nchunk * (blockIdx.y + 1) / ksplit;
  const int nit = (int)(c1 - c0);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

  if (threadIdx.x == 0) {
    for (int s = 0; s < TCG_STAGES; ++s) {
      mbar_init(&S.full[s], 1);
      mbar_init(&S.empty[s], 1);
    }
    mbar_init(&S.done, 1);
    S.abort = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 128;" ::"r"(smem_u32(&S.tmem_base))
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = S.tmem_base;
  const uint32_t tx = diag ? TCG_TILE_BYTES : 2 * TCG_TILE_BYTES;

  if (warp == 0 && lane == 0) {
    // producer: TMA loads into the ring
    int issued = 0;
    for (int it = 0; it < nit; ++it) {
      const int s = it % TCG_STAGES;
      if (it >= TCG_STAGES) {
        if (!mbar_wait(&S.empty[s], ((it / TCG_STAGES) - 1) & 1)) {
          atomicExch(err, 1);
          S.abort = 1;
          break;
        }
      }
      if (*(volatile int*)&S.abort) break;
      const long long c = c0 + it;
      const int p = (int)(c / qchunks);
      const int q = (int)(c - (long long)p * qchunks) * TCG_BK;
      mbar_expect_tx(&S.full[s], tx);
      tma_load_3d(S.a[s], &tmap, &S.full[s], q, bi * TCG_BM, p);
      if (!diag) tma_load_3d(S.b[s], &tmap, &S.full[s], q, bj * TCG_BM, p);
      ++issued;
    }
    // on abort: wait (bounded) for the copies already issued to land
    if (*(volatile int*)&S.abort) {
      for (int it = (issued > TCG_STAGES ? issued - TCG_STAGES : 0); it < issued; ++it)
        mbar_wait(&S.full[it % TCG_STAGES], (it / TCG_STAGES) & 1);
    }
  } else if (warp == 1 && lane == 0) {
    // MMA issuer
    constexpr uint32_t idesc = tf32_idesc();
    for (int it = 0; it < nit; ++it) {
      const int s = it % TCG_STAGES;
      if (!mbar_wait(&S.full[s], (it / TCG_STAGES) & 1)) {
        atomicExch(err, 2);
        S.abort = 1;
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint64_t da = sw128_desc(S.a[s]);
      const uint64_t db = sw128_desc(diag ? S.a[s] : S.b[s]);
#pragma unroll
      for (int kk = 0; kk < TCG_BK / 8; ++kk) {
        // advance 8 tf32 (32 bytes) along K inside the swizzle atom
        mma_tf32(tmem, da + (uint64_t)(kk * 2), db + (uint64_t)(kk * 2), idesc, (it > 0 || kk > 0) ? 1u : 0u);
      }
      mma_commit(&S.empty[s]);
    }
    mma_commit(&S.done);
  }
  __syncwarp();
  // epilogue: one thread waits for the accumulator, the outcome is shared so
  // that the warp-collective TMEM loads below run uniformly
  if (threadIdx.x == 0) {
    if (!mbar_wait(&S.done, 0)) {
      atomicExch(err, 3);
      S.abort = 1;
    }
  }
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const bool ok_all = !*(volatile int*)&S.abort;
  if (ok_all && nit > 0) {
    float* out = part + (size_t)blockIdx.y * D * D;
    const int row = bi * TCG_BM + warp * 32 + lane;
#pragma unroll 1
    for (int cc = 0; cc < TCG_BM; cc += 32) {
      uint32_t v[32];
      const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)cc;
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
          "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
          : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
            "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15]),
            "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]),
            "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
          : "r"(taddr));
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
      if (row < D) {
        const int col0 = bj * TCG_BM + cc;
        float* o = out + (size_t)row * D + col0;
        for (int j = 0; j < 32; ++j)
          if (col0 + j < D) o[j] = __uint_as_float(v[j]);
      }
    }
  } else if (ok_all && nit == 0) {
    // empty contraction slice: the partial block is zero
    float* out = part + (size_t)blockIdx.y * D * D;
    for (int e = threadIdx.x; e < TCG_BM * TCG_BM; e += blockDim.x) {
      const int r = bi * TCG_BM + e / TCG_BM, c = bj * TCG_BM + e % TCG_BM;
      if (r < D && c < D) out[(size_t)r * D + c] = 0.f;
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 128;" ::"r"(tmem) : "memory");
  }
}

// ---------------------------------------------------------------------------
// Two-by-two variant: one CTA computes a 256 x 256 super-block (I, J), I <= J,
// i.e. the four 128 x 128 blocks of row tiles {2I, 2I+1} x column tiles
// {2J, 2J+1} (three on the diagonal), with four accumulators filling the
// SM's 512 TMEM columns.  A stage holds four tiles (two when I == J) for 16
// (12) MMAs, so every byte brought from L2 feeds twice the MMAs of the
// single-block kernel.  Same split-K partial layout (upper blocks only).
// ---------------------------------------------------------------------------
#define TC2_STAGES 3

struct TcGram2Smem {
  alignas(1024) unsigned char t[TC2_STAGES][4][TCG_TILE_BYTES];  // row tiles 2I, 2I+1, 2J, 2J+1
  alignas(8) uint64_t full[TC2_STAGES];
  alignas(8) uint64_t empty[TC2_STAGES];
  alignas(8) uint64_t done;
  uint32_t tmem_base;
  int abort;
};

__global__ void __launch_bounds__(128, 1)
    k_gram_tc2(const __grid_constant__ CUtensorMap tmap, int D, long long P, int qchunks, int ks_d, int ks_o,
               float* part, int* err) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  TcGram2Smem& S = *reinterpret_cast<TcGram2Smem*>((((uintptr_t)smem_raw) + 1023) & ~(uintptr_t)1023);
  const int nt = (D + TCG_BM - 1) / TCG_BM;
  const int ns = (nt + 1) / 2;
  // CTAs [0, ns*ks_d): diagonal super-blocks (I, I), ks_d splits each; then the
  // off-diagonal ones (I < J), ks_o splits each -- split counts in proportion to
  // the blocks computed (3 vs 4), so every CTA carries about the same work
  int I, J, split, ksplit;
  if ((int)blockIdx.x < ns * ks_d) {
    I = J = blockIdx.x / ks_d;
    split = blockIdx.x - I * ks_d;
    ksplit = ks_d;
  } else {
    const int v = blockIdx.x - ns * ks_d;
    int t = v / ks_o;
    split = v - t * ks_o;
    ksplit = ks_o;
    I = 0;
    while (t >= ns - 1 - I) {
      t -= ns - 1 - I;
      ++I;
    }
    J = I + 1 + t;
  }
  const bool diag = I == J;
  // accumulator p: (A slot, B slot, block row tile, block column tile)
  const int npair = diag ? 3 : 4;
  const int pa[4] = {0, 0, diag ? 1 : 1, 1};
  const int pb[4] = {diag ? 0 : 2, diag ? 1 : 3, diag ? 1 : 2, 3};
  // chunks split, split + ksplit, ...: every CTA sweeps the whole contraction
  // range at the same pace, so the diagonal and off-diagonal super-blocks that
  // share row tiles read each chunk at about the same time and the second
  // reader finds it in L2 (contiguous ranges of different lengths per class
  // read the shared tiles far apart and fetch them from DRAM twice)
  const long long nchunk = P * qchunks;
  const int nit = split < nchunk ? (int)((nchunk - split + ksplit - 1) / ksplit) : 0;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

  if (threadIdx.x == 0) {
    for (int s2 = 0; s2 < TC2_STAGES; ++s2) {
      mbar_init(&S.full[s2], 1);
      mbar_init(&S.empty[s2], 1);
    }
    mbar_init(&S.done, 1);
    S.abort = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 512;" ::"r"(smem_u32(&S.tmem_base))
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = S.tmem_base;
  const int nload = diag ? 2 : 4;
  const uint32_t tx = (uint32_t)nload * TCG_TILE_BYTES;

  if (warp == 0 && lane == 0) {
    int issued = 0;
    for (int it = 0; it < nit; ++it) {
      const int s2 = it % TC2_STAGES;
      if (it >= TC2_STAGES) {
        if (!mbar_wait(&S.empty[s2], ((it / TC2_STAGES) - 1) & 1)) {
          atomicExch(err, 1);
          S.abort = 1;
          break;
        }
      }
      if (*(volatile int*)&S.abort) break;
      const long long c = split + (long long)it * ksplit;
      const int p = (int)(c / qchunks);
      const int q = (int)(c - (long long)p * qchunks) * TCG_BK;
      mbar_expect_tx(&S.full[s2], tx);
      tma_load_3d(S.t[s2][0], &tmap, &S.full[s2], q, (2 * I) * TCG_BM, p);
      tma_load_3d(S.t[s2][1], &tmap, &S.full[s2], q, (2 * I + 1) * TCG_BM, p);
      if (!diag) {
        tma_load_3d(S.t[s2][2], &tmap, &S.full[s2], q, (2 * J) * TCG_BM, p);
        tma_load_3d(S.t[s2][3], &tmap, &S.full[s2], q, (2 * J + 1) * TCG_BM, p);
      }
      ++issued;
    }
    if (*(volatile int*)&S.abort) {
      for (int it = (issued > TC2_STAGES ? issued - TC2_STAGES : 0); it < issued; ++it)
        mbar_wait(&S.full[it % TC2_STAGES], (it / TC2_STAGES) & 1);
    }
  } else if (warp == 1 && lane == 0) {
    constexpr uint32_t idesc = tf32_idesc();
    for (int it = 0; it < nit; ++it) {
      const int s2 = it % TC2_STAGES;
      if (!mbar_wait(&S.full[s2], (it / TC2_STAGES) & 1)) {
        atomicExch(err, 2);
        S.abort = 1;
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      for (int pp = 0; pp < npair; ++pp) {
        const uint64_t da = sw128_desc(S.t[s2][pa[pp]]);
        const uint64_t db = sw128_desc(S.t[s2][pb[pp]]);
#pragma unroll
        for (int kk = 0; kk < TCG_BK / 8; ++kk)
          mma_tf32(tmem + (uint32_t)(pp * TCG_BM), da + (uint64_t)(kk * 2), db + (uint64_t)(kk * 2), idesc,
                   (it > 0 || kk > 0) ? 1u : 0u);
      }
      mma_commit(&S.empty[s2]);
    }
    mma_commit(&S.done);
  }
  __syncwarp();
  if (threadIdx.x == 0) {
    if (!mbar_wait(&S.done, 0)) {
      atomicExch(err, 3);
      S.abort = 1;
    }
  }
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const bool ok_all = !*(volatile int*)&S.abort;
  float* out = part + (size_t)split * D * D;
  for (int pp = 0; pp < npair; ++pp) {
    const int bi = (pa[pp] == 0 ? 2 * I : 2 * I + 1);
    const int bj = (pb[pp] == 0 ? 2 * I : pb[pp] == 1 ? 2 * I + 1 : pb[pp] == 2 ? 2 * J : 2 * J + 1);
    if (ok_all && nit > 0) {
      const int row = bi * TCG_BM + warp * 32 + lane;
#pragma unroll 1
      for (int cc = 0; cc < TCG_BM; cc += 32) {
        uint32_t v[32];
        const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(pp * TCG_BM + cc);
        asm volatile(
            "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
            "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
            : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
              "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15]),
              "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]),
              "=r"(v[23]), "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]),
              "=r"(v[30]), "=r"(v[31])
            : "r"(taddr));
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
        if (row < D) {
          const int col0 = bj * TCG_BM + cc;
          float* o = out + (size_t)row * D + col0;
          for (int j = 0; j < 32; ++j)
            if (col0 + j < D) o[j] = __uint_as_float(v[j]);
        }
      }
    } else if (ok_all && nit == 0) {
      for (int e = threadIdx.x; e < TCG_BM * TCG_BM; e += blockDim.x) {
        const int r = bi * TCG_BM + e / TCG_BM, c = bj * TCG_BM + e % TCG_BM;
        if (r < D && c < D) out[(size_t)r * D + c] = 0.f;
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 512;" ::"r"(tmem) : "memory");
  }
}

// G from the split-K partials of the upper blocks.  ks_d partials for blocks of
// the diagonal 256 x 256 super-blocks, ks_o for the others (super2 == 0: one
// count, ks_d, for every block).
__global__ void k_gram_tc_reduce(const float* __restrict__ part, int D, int ks_d, int ks_o, int super2,
                                 float* __restrict__ G) {
  const long long n = (long long)D * D;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(e / D), j = (int)(e - (long long)i * D);
    const long long src = (i / TCG_BM <= j / TCG_BM) ? e : (long long)j * D + i;
    const int ksplit = (!super2 || (i / (2 * TCG_BM)) == (j / (2 * TCG_BM))) ? ks_d : ks_o;
    // compensated FP32 sum of the partials, in split order (FP64 adds are slow on GB300)
    Acc<float> s;
    for (int k = 0; k < ksplit; ++k) s.add(__ldcs(part + (size_t)k * n + src));
    G[e] = s.hi + s.lo;
  }
}

// The bounded-wait error path on its own: one warp waits, with `limit` polls,
// on phase 0 of a freshly initialised mbarrier that nothing arrives on (no
// copy or MMA is in flight), so the wait always runs out; the kernel then
// records TFX_STATUS_ERR_TIMEOUT and returns like the tensor-core kernels do.
__global__ void k_wait_probe(uint32_t limit, int* status) {
  __shared__ __align__(8) uint64_t bar;
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  const bool landed = mbar_wait_bounded(smem_u32(&bar), 0, limit);
  if (threadIdx.x == 0) *status = landed ? TFX_STATUS_OK : TFX_STATUS_ERR_TIMEOUT;
}

}  // namespace tfx

using namespace tfx;

typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static EncodeTiledFn encode_fn() {
  static EncodeTiledFn fn = nullptr;
  if (!fn) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (EncodeTiledFn)p;
  }
  return fn;
}

static int sm_count() {
  static int n = 0;
  if (!n) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    if (n < 1) n = 1;
  }
  return n;
}

// the 2 x 2 super-block kernel serves Grams with at least two row tiles
static bool tc_use2(int D) { return (D + TCG_BM - 1) / TCG_BM >= 2; }

// Split-K counts.  Every kernel keeps one CTA per SM, so the grid is sized to
// fit one wave: the single-block kernel splits each of its blocks evenly; the
// 2 x 2 kernel gives diagonal super-blocks (3 blocks computed) and
// off-diagonal ones (4 blocks) split counts in the ratio 3 : 4.
struct TcSplits {
  int ks_d, ks_o;
};
static TcSplits tc_splits(long long P, int D, long long Q) {
  const int nt = (D + TCG_BM - 1) / TCG_BM;
  const long long chunks = P * ((Q + TCG_BK - 1) / TCG_BK);
  const long long cap = std::max<long long>(1, std::min<long long>(64, chunks / 8));
  const int sms = sm_count();
  TcSplits r;
  if (!tc_use2(D)) {
    const long long tiles = (long long)nt * (nt + 1) / 2;
    const long long ks = std::max<long long>(1, std::min<long long>(cap, sms / tiles));
    r.ks_d = r.ks_o = (int)ks;
    return r;
  }
  const int ns = (nt + 1) / 2;
  const long long noff = (long long)ns * (ns - 1) / 2;
  const double x = (double)sms / (3.0 * ns + 4.0 * noff);
  long long kd = std::max<long long>(1, (long long)(3.0 * x));
  long long ko = std::max<long long>(1, (long long)(4.0 * x));
  if (noff == 0) kd = std::max<long long>(1, sms / ns);
  r.ks_d = (int)std::min<long long>(cap, kd);
  r.ks_o = (int)std::min<long long>(cap, ko);
  return r;
}

extern "C" size_t tfx_mode_gram_tc_scratch_bytes(long long P, int D, long long Q) {
  const TcSplits k = tc_splits(P, D, Q);
  return (size_t)std::max(k.ks_d, k.ks_o) * D * D * 4 + 16;
}

extern "C" int tfx_mode_gram_tc(const float* S, long long P, int D, long long Q, float* G, void* scratch,
                                size_t scratch_bytes, int* err, void* stream) {
  if (!S || !G || !scratch || !err || P < 1 || D < 1 || Q < TCG_BK)
    return tfx_set_error(TFX_STATUS_ERR_ARG, "mode_gram_tc args");
  if ((Q % 4) != 0 || ((uintptr_t)S & 15) != 0)
    return tfx_set_error(TFX_STATUS_ERR_ARG, "mode_gram_tc needs Q % 4 == 0 and a 16-byte aligned tensor");
  if (P > 0x7fffffffLL || Q > 0x7fffffffLL) return tfx_set_error(TFX_STATUS_ERR_ARG, "mode_gram_tc extent");
  EncodeTiledFn enc = encode_fn();
  if (!enc) return tfx_set_error(TFX_STATUS_ERR_UNSUPPORTED, "cuTensorMapEncodeTiled unavailable");
  TcSplits kk = tc_splits(P, D, Q);
  const size_t per = (size_t)D * D * 4;
  if (scratch_bytes < per) return tfx_set_error(TFX_STATUS_ERR_ARG, "mode_gram_tc scratch too small");
  kk.ks_d = (int)std::min<size_t>((size_t)kk.ks_d, scratch_bytes / per);
  kk.ks_o = (int)std::min<size_t>((size_t)kk.ks_o, scratch_bytes / per);
  CUtensorMap map;
  const cuuint64_t gdim[3] = {(cuuint64_t)Q, (cuuint64_t)D, (cuuint64_t)P};
  const cuuint64_t gstride[2] = {(cuuint64_t)Q * 4, (cuuint64_t)Q * D * 4};
  const cuuint32_t box[3] = {TCG_BK, TCG_BM, 1};
  const cuuint32_t estr[3] = {1, 1, 1};
  CUresult r = enc(&map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, (void*)S, gdim, gstride, box, estr,
                   CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                   CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return tfx_set_error(TFX_STATUS_ERR_ARG, "tensor map encoding failed");
  const int nt = (D + TCG_BM - 1) / TCG_BM;
  const int qchunks = (int)((Q + TCG_BK - 1) / TCG_BK);
  cudaStream_t st = (cudaStream_t)stream;
  cudaError_t e;
  if (tc_use2(D)) {
    const int ns = (nt + 1) / 2;
    const int ncta = ns * kk.ks_d + (ns * (ns - 1) / 2) * kk.ks_o;
    const size_t sm = sizeof(TcGram2Smem) + 1024;
    e = cudaFuncSetAttribute(k_gram_tc2, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return tfx_set_cuda_error(e, "mode_gram_tc smem");
    k_gram_tc2<<<ncta, 128, sm, st>>>(map, D, P, qchunks, kk.ks_d, kk.ks_o, (float*)scratch, err);
  } else {
    const int tiles = nt * (nt + 1) / 2;
    const size_t sm = sizeof(TcGramSmem) + 1024;
    e = cudaFuncSetAttribute(k_gram_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return tfx_set_cuda_error(e, "mode_gram_tc smem");
    k_gram_tc<<<dim3(tiles, kk.ks_d), 128, sm, st>>>(map, D, P, qchunks, kk.ks_d, (float*)scratch, err);
  }
  e = cudaGetLastError();
  if (e != cudaSuccess) return tfx_set_cuda_error(e, "mode_gram_tc launch");
  tfx_count_launch(1);
  const long long n = (long long)D * D;
  const int rb = (int)std::max<long long>(1, std::min<long long>((n + 255) / 256, 4LL * sm_count()));
  k_gram_tc_reduce<<<rb, 256, 0, st>>>((const float*)scratch, D, kk.ks_d, kk.ks_o, tc_use2(D) ? 1 : 0, G);
  e = cudaGetLastError();
  if (e != cudaSuccess) return tfx_set_cuda_error(e, "mode_gram_tc reduce");
  tfx_count_launch(1);
  return TFX_STATUS_OK;
}

extern "C" int tfx_wait_probe(unsigned int limit, int* status, void* stream) {
  if (!status || limit == 0 || limit > (1u << 26)) return tfx_set_error(TFX_STATUS_ERR_ARG, "wait_probe args");
  k_wait_probe<<<1, 32, 0, (cudaStream_t)stream>>>(limit, status);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return tfx_set_cuda_error(e, "wait_probe launch");
  tfx_count_launch(1);
  return TFX_STATUS_OK;
}
