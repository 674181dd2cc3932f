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

// ---------------------------------------------------------------------------
// Accumulators.  GB300 executes FP64 at a small fraction of its FP32 rate, so
// the FP32 path accumulates sums in float-float form (an unevaluated pair
// hi + lo with |lo| <= ulp(hi)/2, combined with Knuth's TwoSum and exact FMA
// products: about 48 significant bits).  The FP64 path accumulates in double.
// ---------------------------------------------------------------------------
template <class T>
struct Acc;

template <>
struct Acc<float> {
  float hi, lo;
  __device__ __forceinline__ Acc() : hi(0.f), lo(0.f) {}
  __device__ __forceinline__ void add2(float bh, float bl) {
    const float s = hi + bh;
    const float bb = s - hi;
    float err = (hi - (s - bb)) + (bh - bb);
    err += lo + bl;
    hi = s + err;
    lo = err - (hi - s);
  }
  __device__ __forceinline__ void add(float x) { add2(x, 0.f); }
  __device__ __forceinline__ void fma_(float x, float y) {
    const float p = x * y;
    add2(p, fmaf(x, y, -p));
  }
  __device__ __forceinline__ double value() const { return (double)hi + (double)lo; }
  __device__ __forceinline__ void warp_reduce() {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const float oh = __shfl_xor_sync(0xffffffffu, hi, o);
      const float ol = __shfl_xor_sync(0xffffffffu, lo, o);
      add2(oh, ol);
    }
  }
};

template <>
struct Acc<double> {
  double v;
  __device__ __forceinline__ Acc() : v(0.0) {}
  __device__ __forceinline__ void add(double x) { v += x; }
  __device__ __forceinline__ void fma_(double x, double y) { v = fma(x, y, v); }
  __device__ __forceinline__ double value() const { return v; }
  __device__ __forceinline__ void warp_reduce() { v = warp_sum(v); }
};

// Reduction scratch living in shared memory: per-warp partials, a
// double-buffered per-CTA slot read by the peers of the team, and the team's
// totals broadcast to the CTA.
#define TFX_MAX_TEAM 16
template <int NV>
struct RedScratch {
  double warp[TFX_THREADS / 32][NV];
  double part[2][NV];
  double tot[NV];
};

// Team-wide sum (or max) of NV per-thread values; every thread of every CTA
// returns the same totals.  Warps reduce first, then one thread per value
// combines the warps, the CTAs' partials are read from distributed shared
// memory by one thread per value and summed in rank order.  `flip`
// alternates the slot buffer so that one team barrier per call suffices.
template <int NV, bool MAX, class A>
__device__ __forceinline__ void team_reduce_acc(const Team& tm, A (&v)[NV], double (&out)[NV], RedScratch<NV>* rs,
                                                int& flip) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int j = 0; j < NV; ++j) {
    v[j].warp_reduce();
    if (lane == 0) rs->warp[wid][j] = v[j].value();
  }
  __syncthreads();
  if (threadIdx.x < NV) {
    double s = rs->warp[0][threadIdx.x];
    for (int w = 1; w < TFX_THREADS / 32; ++w) s = MAX ? fmax(s, rs->warp[w][threadIdx.x]) : s + rs->warp[w][threadIdx.x];
    rs->part[flip][threadIdx.x] = s;
  }
  tm.sync();
  if (threadIdx.x < NV) {
    const int j = threadIdx.x;
    double pv[TFX_MAX_TEAM];
#pragma unroll
    for (int r = 0; r < TFX_MAX_TEAM; ++r) pv[r] = r < tm.size ? tm.peer(&rs->part[flip][0], r)[j] : 0.0;
    double s = pv[0];
#pragma unroll
    for (int r = 1; r < TFX_MAX_TEAM; ++r)
      if (r < tm.size) s = MAX ? fmax(s, pv[r]) : s + pv[r];
    rs->tot[j] = s;
  }
  __syncthreads();
#pragma unroll
  for (int j = 0; j < NV; ++j) out[j] = rs->tot[j];
  flip ^= 1;
  __syncthreads();  // tot and warp slots may be rewritten by the next call
}

struct DAcc {  // plain double accumulator used by the double-valued wrappers
  double v;
  __device__ __forceinline__ void warp_reduce() { v = warp_sum(v); }
  __device__ __forceinline__ double value() const { return v; }
};
struct DMax {
  double v;
  __device__ __forceinline__ void warp_reduce() { v = warp_max(v); }
  __device__ __forceinline__ double value() const { return v; }
};
template <class T>
struct MaxAcc {  // running maximum in the working precision
  T v;
  __device__ __forceinline__ MaxAcc() : v(T(0)) {}
  __device__ __forceinline__ void warp_reduce() {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  }
  __device__ __forceinline__ double value() const { return (double)v; }
};

template <int NV, bool MAX>
__device__ __forceinline__ void team_reduce(const Team& tm, double (&v)[NV], RedScratch<NV>* rs, int& flip) {
  if (MAX) {
    DMax a[NV];
#pragma unroll
    for (int j = 0; j < NV; ++j) a[j].v = v[j];
    team_reduce_acc<NV, true>(tm, a, v, rs, flip);
  } else {
    DAcc a[NV];
#pragma unroll
    for (int j = 0; j < NV; ++j) a[j].v = v[j];
    team_reduce_acc<NV, false>(tm, a, v, rs, flip);
  }
}

template <int NV, class T>
__device__ __forceinline__ void team_sum_acc(const Team& tm, Acc<T> (&v)[NV], double (&out)[NV], RedScratch<NV>* rs,
                                             int& flip) {
  team_reduce_acc<NV, false>(tm, v, out, rs, flip);
}

template <int NV>
__device__ __forceinline__ void team_sum(const Team& tm, double (&v)[NV], RedScratch<NV>* rs, int& flip) {
  team_reduce<NV, false>(tm, v, rs, flip);
}

template <int NV>
__device__ __forceinline__ void team_max(const Team& tm, double (&v)[NV], RedScratch<NV>* rs, int& flip) {
  team_reduce<NV, true>(tm, v, rs, flip);
}

// ---------------------------------------------------------------------------
// Register-tiled microkernel: 256 threads as a 16x16 grid, each owning a TMxTN
// block of a (16*TM) x (16*TN) output tile.  A chunk is staged k-major in shared
// memory: sA[k][m] (ld = BM+1) and sB[k][n] (ld = BN+1).
// ---------------------------------------------------------------------------
#define TFX_BK 32

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
