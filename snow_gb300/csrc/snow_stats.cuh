// Commit of the bulk-statistics partial sums: a warp shuffle reduction, one
// pass over the block's warps in shared memory, one record per block, and a
// fixed-order sum of the records by the grid's last block (no contended
// atomics, and the totals do not depend on block scheduling).
#pragma once

#include "snow_internal.h"

namespace snow {

struct StatsPartial {
  double acc[9];  // mass, momentum x3, kinetic energy, mass-weighted position x3, sum J_p
  float bmin[3], bmax[3];
  unsigned long long bad;
};

__device__ __forceinline__ int stats_order_key(float f) {
  const int i = __float_as_int(f);
  return i >= 0 ? i : i ^ 0x7fffffff;
}

__device__ __forceinline__ void stats_init(StatsPartial& t) {
#pragma unroll
  for (int k = 0; k < 9; k++) t.acc[k] = 0.0;
#pragma unroll
  for (int k = 0; k < 3; k++) {
    t.bmin[k] = 3.4e38f;
    t.bmax[k] = -3.4e38f;
  }
  t.bad = 0;
}

constexpr int kStatsThreads = 256;  // the block size of every statistics kernel

// Bounds and the non-finite count of the calling warp, combined with
// shuffles (FP32 min/max, integer sums: cheap), in lane 0.
__device__ __forceinline__ void stats_warp_bounds(StatsPartial& t) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
    for (int k = 0; k < 3; k++) {
      t.bmin[k] = fminf(t.bmin[k], __shfl_down_sync(0xffffffffu, t.bmin[k], o));
      t.bmax[k] = fmaxf(t.bmax[k], __shfl_down_sync(0xffffffffu, t.bmax[k], o));
    }
    t.bad += __shfl_down_sync(0xffffffffu, t.bad, o);
  }
}

// FP64 sum over 32 lanes (the result in lane 0).
__device__ __forceinline__ double stats_warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

// Every thread of the block (kStatsThreads of them) calls this once with
// its partials; gridDim.x is at most kStatsMaxBlocks. The nine FP64 sums
// are transposed through shared memory: warp w sums fields w, w + 8 over
// the block's threads (8 values per lane, then 5 shuffle steps), so each
// field costs 31 + 32 * 7 additions instead of every lane reducing all nine
// fields (FP64 arithmetic is slow on this part). Each block stores its sums
// in slot->part; the last block to do so adds the records up the same way,
// in block order, publishes the totals to `host` and re-arms the slot. The
// order of every addition is fixed, so the totals do not depend on block
// scheduling.
__device__ __forceinline__ void stats_commit(StatsPartial& t, StatsSlot* slot, StatsAccum* host) {
  __shared__ double sacc[9][kStatsThreads];
  __shared__ double bsum[9];
  __shared__ float wmin[kStatsThreads / 32][3], wmax[kStatsThreads / 32][3];
  __shared__ unsigned long long wbad[kStatsThreads / 32];
  __shared__ bool last;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  constexpr int nwarps = kStatsThreads / 32;
#pragma unroll
  for (int k = 0; k < 9; k++) sacc[k][tid] = t.acc[k];
  stats_warp_bounds(t);
  if (lane == 0) {
#pragma unroll
    for (int k = 0; k < 3; k++) {
      wmin[warp][k] = t.bmin[k];
      wmax[warp][k] = t.bmax[k];
    }
    wbad[warp] = t.bad;
  }
  __syncthreads();
  for (int k = warp; k < 9; k += nwarps) {
    double v = 0.0;
#pragma unroll
    for (int i = 0; i < kStatsThreads / 32; i++) v += sacc[k][lane + 32 * i];
    v = stats_warp_sum(v);
    if (lane == 0) bsum[k] = v;
  }
  __syncthreads();
  if (tid == 0) {
    StatsBlockSum& mine = slot->part[blockIdx.x];
    for (int k = 0; k < 9; k++) mine.acc[k] = bsum[k];
    for (int k = 0; k < 3; k++) {
      float lo = wmin[0][k], hi = wmax[0][k];
      for (int w = 1; w < nwarps; w++) {
        lo = fminf(lo, wmin[w][k]);
        hi = fmaxf(hi, wmax[w][k]);
      }
      mine.bmin[k] = lo;
      mine.bmax[k] = hi;
    }
    unsigned long long bad = 0;
    for (int w = 0; w < nwarps; w++) bad += wbad[w];
    mine.bad = bad;
    __threadfence();
    last = atomicAdd(&slot->done, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!last) return;
  // the last block: warp w sums fields w, w + 8 over the records (lane l
  // takes records l, l + 32, ...; L2 reads: other blocks wrote them before
  // their fence), every thread the bounds of records tid, tid + 256, ...
  __threadfence();
  const int nb = (int)gridDim.x;
  for (int k = warp; k < 9; k += nwarps) {
    double v = 0.0;
    for (int q = lane; q < nb; q += 32) v += __ldcg(&slot->part[q].acc[k]);
    v = stats_warp_sum(v);
    if (lane == 0) bsum[k] = v;
  }
  StatsPartial b;
  stats_init(b);
  for (int q = tid; q < nb; q += kStatsThreads) {
    const StatsBlockSum* p = &slot->part[q];
    for (int k = 0; k < 3; k++) {
      b.bmin[k] = fminf(b.bmin[k], __ldcg(&p->bmin[k]));
      b.bmax[k] = fmaxf(b.bmax[k], __ldcg(&p->bmax[k]));
    }
    b.bad += __ldcg(&p->bad);
  }
  stats_warp_bounds(b);
  __syncthreads();  // wmin / wmax / wbad are reused
  if (lane == 0) {
#pragma unroll
    for (int k = 0; k < 3; k++) {
      wmin[warp][k] = b.bmin[k];
      wmax[warp][k] = b.bmax[k];
    }
    wbad[warp] = b.bad;
  }
  __syncthreads();
  if (tid == 0) {
    StatsAccum r;
    r.mass = bsum[0];
    for (int k = 0; k < 3; k++) {
      float lo = wmin[0][k], hi = wmax[0][k];
      for (int w = 1; w < nwarps; w++) {
        lo = fminf(lo, wmin[w][k]);
        hi = fmaxf(hi, wmax[w][k]);
      }
      r.mom[k] = bsum[1 + k];
      r.com[k] = bsum[5 + k];
      r.bmin_key[k] = stats_order_key(lo);
      r.bmax_key[k] = stats_order_key(hi);
    }
    r.ke = bsum[4];
    r.jp = bsum[8];
    unsigned long long bad = 0;
    for (int w = 0; w < nwarps; w++) bad += wbad[w];
    r.nonfinite = bad;
    *host = r;  // visible to the host once it has waited for the kernel
    slot->done = 0u;
  }
}

}  // namespace snow
