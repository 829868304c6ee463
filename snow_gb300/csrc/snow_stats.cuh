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

// Every thread of the block calls this once with its partials; blockDim.x is a
// multiple of 32 and at most 1024, gridDim.x at most kStatsMaxBlocks. Each
// block stores its sums in slot->part; the last block to do so adds them up
// in block order, publishes the totals to `host` and re-arms the slot.
__device__ __forceinline__ void stats_commit(StatsPartial& t, StatsSlot* slot, StatsAccum* host) {
  __shared__ StatsPartial warp_sums[32];
  __shared__ bool last;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
    for (int k = 0; k < 9; k++) t.acc[k] += __shfl_down_sync(0xffffffffu, t.acc[k], o);
#pragma unroll
    for (int k = 0; k < 3; k++) {
      t.bmin[k] = fminf(t.bmin[k], __shfl_down_sync(0xffffffffu, t.bmin[k], o));
      t.bmax[k] = fmaxf(t.bmax[k], __shfl_down_sync(0xffffffffu, t.bmax[k], o));
    }
    t.bad += __shfl_down_sync(0xffffffffu, t.bad, o);
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  if (lane == 0) warp_sums[warp] = t;
  __syncthreads();
  if (threadIdx.x == 0) {
    StatsPartial b = warp_sums[0];
    for (int w = 1; w < nwarps; w++) {
      for (int k = 0; k < 9; k++) b.acc[k] += warp_sums[w].acc[k];
      for (int k = 0; k < 3; k++) {
        b.bmin[k] = fminf(b.bmin[k], warp_sums[w].bmin[k]);
        b.bmax[k] = fmaxf(b.bmax[k], warp_sums[w].bmax[k]);
      }
      b.bad += warp_sums[w].bad;
    }
    StatsBlockSum& mine = slot->part[blockIdx.x];
    for (int k = 0; k < 9; k++) mine.acc[k] = b.acc[k];
    for (int k = 0; k < 3; k++) {
      mine.bmin[k] = b.bmin[k];
      mine.bmax[k] = b.bmax[k];
    }
    mine.bad = b.bad;
    __threadfence();
    last = atomicAdd(&slot->done, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!last) return;
  // the last block: thread i sums blocks i, i + blockDim.x, ... then the
  // block's warps and threads combine in a fixed order
  __threadfence();
  StatsPartial s;
  stats_init(s);
  for (int q = threadIdx.x; q < (int)gridDim.x; q += blockDim.x) {
    // L2 reads (the records were written by other blocks before their fence)
    const StatsBlockSum* p = &slot->part[q];
    for (int k = 0; k < 9; k++) s.acc[k] += __ldcg(&p->acc[k]);
    for (int k = 0; k < 3; k++) {
      s.bmin[k] = fminf(s.bmin[k], __ldcg(&p->bmin[k]));
      s.bmax[k] = fmaxf(s.bmax[k], __ldcg(&p->bmax[k]));
    }
    s.bad += __ldcg(&p->bad);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
    for (int k = 0; k < 9; k++) s.acc[k] += __shfl_down_sync(0xffffffffu, s.acc[k], o);
#pragma unroll
    for (int k = 0; k < 3; k++) {
      s.bmin[k] = fminf(s.bmin[k], __shfl_down_sync(0xffffffffu, s.bmin[k], o));
      s.bmax[k] = fmaxf(s.bmax[k], __shfl_down_sync(0xffffffffu, s.bmax[k], o));
    }
    s.bad += __shfl_down_sync(0xffffffffu, s.bad, o);
  }
  __syncthreads();  // warp_sums is reused
  if (lane == 0) warp_sums[warp] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    StatsPartial b = warp_sums[0];
    for (int w = 1; w < nwarps; w++) {
      for (int k = 0; k < 9; k++) b.acc[k] += warp_sums[w].acc[k];
      for (int k = 0; k < 3; k++) {
        b.bmin[k] = fminf(b.bmin[k], warp_sums[w].bmin[k]);
        b.bmax[k] = fmaxf(b.bmax[k], warp_sums[w].bmax[k]);
      }
      b.bad += warp_sums[w].bad;
    }
    StatsAccum r;
    r.mass = b.acc[0];
    for (int k = 0; k < 3; k++) {
      r.mom[k] = b.acc[1 + k];
      r.com[k] = b.acc[5 + k];
      r.bmin_key[k] = stats_order_key(b.bmin[k]);
      r.bmax_key[k] = stats_order_key(b.bmax[k]);
    }
    r.ke = b.acc[4];
    r.jp = b.acc[8];
    r.nonfinite = b.bad;
    *host = r;  // visible to the host once it has waited for the kernel
    slot->done = 0u;
  }
}

}  // namespace snow
