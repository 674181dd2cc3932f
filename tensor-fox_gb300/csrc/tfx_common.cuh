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
  __device__ __forceinline__ float hi_or_v() const { return hi; }
  __device__ __forceinline__ float lo_or_0() const { return lo; }
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
  __device__ __forceinline__ double hi_or_v() const { return v; }
  __device__ __forceinline__ double lo_or_0() const { return 0.0; }
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

// One-barrier team sum for the CG loop.  Every warp publishes its reduced
// partial (a float-float pair, or a double on the FP64 path) in its own
// double-buffered shared-memory slot; after one team barrier every warp of
// every CTA reads all team_size x 8 partials, local and remote, and combines
// them with shuffles.  No CTA-level barrier and no FP64 arithmetic on the FP32
// path; every thread returns the totals as accumulators.  Two calls in a row
// may reuse a slot buffer only after the barrier of the call in between,
// which the alternating `flip` guarantees.
template <int NV>
struct WarpSlots {
  double raw[2][TFX_THREADS / 32][NV];
};

template <int NV>
__device__ __forceinline__ void team_sum_fast(const Team& tm, Acc<float> (&v)[NV], Acc<float> (&out)[NV],
                                              WarpSlots<NV>* ws, int& flip) {
  constexpr int NW = TFX_THREADS / 32;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int j = 0; j < NV; ++j) v[j].warp_reduce();
  float2* mine = reinterpret_cast<float2*>(&ws->raw[flip][0][0]);
  if (lane == 0)
#pragma unroll
    for (int j = 0; j < NV; ++j) mine[wid * NV + j] = make_float2(v[j].hi, v[j].lo);
  tm.sync();
  const int np = tm.size * NW;
  float2 p[(TFX_MAX_TEAM * NW + 31) / 32][NV];
#pragma unroll
  for (int u = 0; u < (TFX_MAX_TEAM * NW + 31) / 32; ++u) {
    const int q = lane + 32 * u;
    if (q < np) {
      const float2* src = tm.peer(mine, q / NW) + (q % NW) * NV;
#pragma unroll
      for (int j = 0; j < NV; ++j) p[u][j] = src[j];
    } else {
#pragma unroll
      for (int j = 0; j < NV; ++j) p[u][j] = make_float2(0.f, 0.f);
    }
  }
#pragma unroll
  for (int j = 0; j < NV; ++j) {
    Acc<float> a;
#pragma unroll
    for (int u = 0; u < (TFX_MAX_TEAM * NW + 31) / 32; ++u) a.add2(p[u][j].x, p[u][j].y);
    a.warp_reduce();
    out[j] = a;
  }
  flip ^= 1;
}

template <int NV>
__device__ __forceinline__ void team_sum_fast(const Team& tm, Acc<double> (&v)[NV], Acc<double> (&out)[NV],
                                              WarpSlots<NV>* ws, int& flip) {
  constexpr int NW = TFX_THREADS / 32;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int j = 0; j < NV; ++j) v[j].warp_reduce();
  double* mine = &ws->raw[flip][0][0];
  if (lane == 0)
#pragma unroll
    for (int j = 0; j < NV; ++j) mine[wid * NV + j] = v[j].v;
  tm.sync();
  const int np = tm.size * NW;
  double p[(TFX_MAX_TEAM * NW + 31) / 32][NV];
#pragma unroll
  for (int u = 0; u < (TFX_MAX_TEAM * NW + 31) / 32; ++u) {
    const int q = lane + 32 * u;
    if (q < np) {
      const double* src = tm.peer(mine, q / NW) + (q % NW) * NV;
#pragma unroll
      for (int j = 0; j < NV; ++j) p[u][j] = src[j];
    } else {
#pragma unroll
      for (int j = 0; j < NV; ++j) p[u][j] = 0.0;
    }
  }
#pragma unroll
  for (int j = 0; j < NV; ++j) {
    Acc<double> a;
#pragma unroll
    for (int u = 0; u < (TFX_MAX_TEAM * NW + 31) / 32; ++u) a.add(p[u][j]);
    a.warp_reduce();
    out[j] = a;
  }
  flip ^= 1;
}

// Push-based team sum: the CTA reduces its warps' partials first (one CTA
// barrier), then one lane per team member stores the CTA's partial into that
// member's shared memory; after one team barrier every warp combines the
// team_size partials sitting in its own shared memory with shuffles.  Remote
// traffic is team_size stores per CTA and nothing remote is on the path after
// the barrier.  Slots alternate with `flip` (see team_sum_fast).
template <int NV>
struct PushSlots {
  double team[2][TFX_MAX_TEAM][NV];
  double warp[TFX_THREADS / 32][NV];
};

template <int NV>
__device__ __forceinline__ void team_sum_push(const Team& tm, Acc<float> (&v)[NV], Acc<float> (&out)[NV],
                                              PushSlots<NV>* ps, int& flip) {
  constexpr int NW = TFX_THREADS / 32;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  float2* wslot = reinterpret_cast<float2*>(&ps->warp[0][0]);
  float2* tslot = reinterpret_cast<float2*>(&ps->team[flip][0][0]);
#pragma unroll
  for (int j = 0; j < NV; ++j) v[j].warp_reduce();
  if (lane == 0)
#pragma unroll
    for (int j = 0; j < NV; ++j) wslot[wid * NV + j] = make_float2(v[j].hi, v[j].lo);
  __syncthreads();
  if (wid == 0) {
#pragma unroll
    for (int j = 0; j < NV; ++j) {
      Acc<float> a;
      if (lane < NW) {
        const float2 q = wslot[lane * NV + j];
        a.hi = q.x;
        a.lo = q.y;
      }
#pragma unroll
      for (int o = 1; o < NW; o <<= 1) {
        const float oh = __shfl_xor_sync(0xffffffffu, a.hi, o);
        const float ol = __shfl_xor_sync(0xffffffffu, a.lo, o);
        a.add2(oh, ol);
      }
      // lanes 0..NW-1 hold the CTA total; every storing lane takes lane 0's
      a.hi = __shfl_sync(0xffffffffu, a.hi, 0);
      a.lo = __shfl_sync(0xffffffffu, a.lo, 0);
      if (lane < tm.size) tm.peer(tslot, lane)[tm.rank * NV + j] = make_float2(a.hi, a.lo);
    }
  }
  tm.sync();
#pragma unroll
  for (int j = 0; j < NV; ++j) {
    Acc<float> a;
    if (lane < tm.size) {
      const float2 q = tslot[lane * NV + j];
      a.hi = q.x;
      a.lo = q.y;
    }
#pragma unroll
    for (int o = 1; o < TFX_MAX_TEAM; o <<= 1) {
      const float oh = __shfl_xor_sync(0xffffffffu, a.hi, o);
      const float ol = __shfl_xor_sync(0xffffffffu, a.lo, o);
      a.add2(oh, ol);
    }
    a.hi = __shfl_sync(0xffffffffu, a.hi, 0);
    a.lo = __shfl_sync(0xffffffffu, a.lo, 0);
    out[j] = a;
  }
  flip ^= 1;
}

template <int NV>
__device__ __forceinline__ void team_sum_push(const Team& tm, Acc<double> (&v)[NV], Acc<double> (&out)[NV],
                                              PushSlots<NV>* ps, int& flip) {
  constexpr int NW = TFX_THREADS / 32;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  double* wslot = &ps->warp[0][0];
  double* tslot = &ps->team[flip][0][0];
#pragma unroll
  for (int j = 0; j < NV; ++j) v[j].warp_reduce();
  if (lane == 0)
#pragma unroll
    for (int j = 0; j < NV; ++j) wslot[wid * NV + j] = v[j].v;
  __syncthreads();
  if (wid == 0) {
#pragma unroll
    for (int j = 0; j < NV; ++j) {
      double a = lane < NW ? wslot[lane * NV + j] : 0.0;
#pragma unroll
      for (int o = 1; o < NW; o <<= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
      a = __shfl_sync(0xffffffffu, a, 0);
      if (lane < tm.size) tm.peer(tslot, lane)[tm.rank * NV + j] = a;
    }
  }
  tm.sync();
#pragma unroll
  for (int j = 0; j < NV; ++j) {
    double a = lane < tm.size ? tslot[lane * NV + j] : 0.0;
#pragma unroll
    for (int o = 1; o < TFX_MAX_TEAM; o <<= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
    out[j].v = __shfl_sync(0xffffffffu, a, 0);
  }
  flip ^= 1;
}

// the accumulator's value in the working precision
__device__ __forceinline__ float acc_val(const Acc<float>& a) { return a.hi + a.lo; }
__device__ __forceinline__ double acc_val(const Acc<double>& a) { return a.v; }
// the accumulator's value in double
__device__ __forceinline__ double acc_val_d(const Acc<float>& a) { return (double)a.hi + (double)a.lo; }
__device__ __forceinline__ double acc_val_d(const Acc<double>& a) { return a.v; }

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
// Bounded wait on phase `parity` of a shared-memory mbarrier (its 32-bit
// shared address): at most `limit` polls with mbarrier.try_wait.parity.
// Returns false when the wait ran out; the caller then records an error status
// instead of spinning on (the tensor-core kernels' copy and MMA waits use it).
__device__ __forceinline__ bool mbar_wait_bounded(uint32_t bar_addr, uint32_t parity, uint32_t limit) {
  for (uint32_t it = 0; it < limit; ++it) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(bar_addr), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

#define TFX_OK 0
#define TFX_ERR_ARG 1
#define TFX_ERR_NUMERIC 2
#define TFX_ERR_TIMEOUT 3
#define TFX_ERR_CUDA 4
#define TFX_ERR_UNSUPPORTED 5
