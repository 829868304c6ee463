// Block-level commit of the bulk-statistics partial sums: a warp shuffle
// reduction, then one pass over the block's warps in shared memory, then one
// set of global atomics per block (not per warp: the 10 double sums are a
// handful of addresses that every block hits).
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

// Every thread of the block calls this once with its partials; blockDim.x is a
// multiple of 32 and at most 1024.
__device__ __forceinline__ void stats_commit(StatsPartial& t, StatsAccum* out) {
  __shared__ StatsPartial warp_sums[32];
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
    atomicAdd(&out->mass, b.acc[0]);
    for (int k = 0; k < 3; k++) atomicAdd(&out->mom[k], b.acc[1 + k]);
    atomicAdd(&out->ke, b.acc[4]);
    for (int k = 0; k < 3; k++) atomicAdd(&out->com[k], b.acc[5 + k]);
    atomicAdd(&out->jp, b.acc[8]);
    if (b.bad) atomicAdd(&out->nonfinite, b.bad);
    for (int k = 0; k < 3; k++) {
      atomicMin(&out->bmin_key[k], stats_order_key(b.bmin[k]));
      atomicMax(&out->bmax_key[k], stats_order_key(b.bmax[k]));
    }
  }
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

}  // namespace snow
