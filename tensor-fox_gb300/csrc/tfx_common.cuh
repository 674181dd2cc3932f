// Shared device helpers for the Tensor Fox GB300 kernels.
//
// * Team: the CTAs that cooperate on one CPD problem.  A team is a thread-block
//   cluster (1..16 CTAs on distinct SMs) whose CTAs exchange partial results
//   through distributed shared memory and meet at cluster barriers.  With one
//   CTA the same code runs with __syncthreads only.
// * Deterministic reductions: every partial sum is combined in a fixed order
//   (warp shuffle tree, then warps in index order, then CTAs in rank order), so
//   every CTA of a team obtains bit-identical scalars and takes the same
//   control-flow decisions without a broadcast.
// * A 16x16-thread register-tiled microkernel used by all small contractions.
#pragma once
#include <cooperative_groups.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace cgx = cooperative_groups;

#define TFX_MAX_ORDER 12
#define TFX_THREADS 256

struct Team {
  int rank;
  int size;
  __device__ __forceinline__ void sync() const {
    if (size > 1) {
      cgx::this_cluster().sync();
    } else {
      __syncthreads();
    }
  }
  template <class P>
  __device__ __forceinline__ P* peer(P* p, int r) const {
    if (size > 1) return cgx::this_cluster().map_shared_rank(p, r);
    return p;
  }
};

__device__ __forceinline__ Team make_team(int cluster_size) {
  Team t;
  if (cluster_size > 1) {
    t.rank = (int)cgx::this_cluster().block_rank();
  } else {
    t.rank = 0;
  }
  t.size = cluster_size;
  return t;
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ double warp_max(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

// Reduction scratch living in shared memory: per-warp partials and a
// double-buffered per-CTA slot read by the peers of the team.
template <int NV>
struct RedScratch {
  double warp[TFX_THREADS / 32][NV];
  double part[2][NV];
};

// Sums NV per-thread values over the whole team; every thread of every CTA
// returns the same totals.  `flip` alternates the slot buffer so that only one
// team barrier is needed per call.
template <int NV>
__device__ __forceinline__ void team_sum(const Team& tm, double (&v)[NV], RedScratch<NV>* rs, int& flip) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int j = 0; j < NV; ++j) {
    double s = warp_sum(v[j]);
    if (lane == 0) rs->warp[wid][j] = s;
  }
  __syncthreads();
  if (threadIdx.x < NV) {
    double s = 0.0;
    for (int w = 0; w < TFX_THREADS / 32; ++w) s += rs->warp[w][threadIdx.x];
    rs->part[flip][threadIdx.x] = s;
  }
  tm.sync();
#pragma unroll
  for (int j = 0; j < NV; ++j) {
    double s = 0.0;
    for (int r = 0; r < tm.size; ++r) s += tm.peer(&rs->part[flip][0], r)[j];
    v[j] = s;
  }
  flip ^= 1;
  __syncthreads();  // warp slots may be rewritten by the next call
}

template <int NV>
__device__ __forceinline__ void team_max(const Team& tm, double (&v)[NV], RedScratch<NV>* rs, int& flip) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int j = 0; j < NV; ++j) {
    double s = warp_max(v[j]);
    if (lane == 0) rs->warp[wid][j] = s;
  }
  __syncthreads();
  if (threadIdx.x < NV) {
    double s = rs->warp[0][threadIdx.x];
    for (int w = 1; w < TFX_THREADS / 32; ++w) s = fmax(s, rs->warp[w][threadIdx.x]);
    rs->part[flip][threadIdx.x] = s;
  }
  tm.sync();
#pragma unroll
  for (int j = 0; j < NV; ++j) {
    double s = tm.peer(&rs->part[flip][0], 0)[j];
    for (int r = 1; r < tm.size; ++r) s = fmax(s, tm.peer(&rs->part[flip][0], r)[j]);
    v[j] = s;
  }
  flip ^= 1;
  __syncthreads();
}

// ---------------------------------------------------------------------------
// Register-tiled microkernel: 256 threads as a 16x16 grid, each owning a TMxTN
// block of a (16*TM) x (16*TN) output tile.  A chunk is staged k-major in shared
// memory: sA[k][m] (ld = BM+1) and sB[k][n] (ld = BN+1).
// ---------------------------------------------------------------------------
#define TFX_BK 16

template <int TM, int TN>
struct Tile {
  static constexpr int BM = 16 * TM;
  static constexpr int BN = 16 * TN;
  static constexpr int LDA = BM + 1;
  static constexpr int LDB = BN + 1;
};

template <class T, int TM, int TN>
__device__ __forceinline__ void tile_fma(const T* __restrict__ sA, const T* __restrict__ sB, T (&acc)[TM][TN],
                                         int kc) {
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  for (int k = 0; k < kc; ++k) {
    T a[TM], b[TN];
#pragma unroll
    for (int u = 0; u < TM; ++u) a[u] = sA[k * Tile<TM, TN>::LDA + ty + 16 * u];
#pragma unroll
    for (int v = 0; v < TN; ++v) b[v] = sB[k * Tile<TM, TN>::LDB + tx + 16 * v];
#pragma unroll
    for (int u = 0; u < TM; ++u)
#pragma unroll
      for (int v = 0; v < TN; ++v) acc[u][v] = fma(a[u], b[v], acc[u][v]);
  }
}

template <class T, int TM, int TN>
__device__ __forceinline__ void tile_zero(T (&acc)[TM][TN]) {
#pragma unroll
  for (int u = 0; u < TM; ++u)
#pragma unroll
    for (int v = 0; v < TN; ++v) acc[u][v] = T(0);
}

// Status codes shared with the C ABI.
#define TFX_OK 0
#define TFX_ERR_ARG 1
#define TFX_ERR_NUMERIC 2
#define TFX_ERR_TIMEOUT 3
#define TFX_ERR_CUDA 4
#define TFX_ERR_UNSUPPORTED 5
