// SNOW_MODE_FAST kernels for sm_103a: the explicit snow-MPM step of the
// reference (shader/compute/mpm/*.glsl) in FP32 without fixed-point
// quantisation, on a blocked grid.
//
// Grid layout in HBM. The grid is cut into 4x4x4-node blocks.
//   acc      dense, one 3584-byte record per block: the P2G sums (m, p, f)
//            as fixed-point integers (seven int64 words per node,
//            word-major), so that they do not depend on the order they are
//            added in. All zero between steps: the grid update clears what
//            it consumes.
//   blk_flag blocks that received P2G sums (set by the P2G tile flush).
//   compact  turns the flags into the active-block list and gives each
//            active block a slot in the output pool.
//   gout     the pool: per slot the grid update's output v* and
//            d = v* - alpha p/m, one 6-float record per node (1536 bytes).
//
// Kernels of one step (every scene of a batch in one launch each):
//   compact      flags -> slots, active list             (thread per block)
//   grid         per active block: v* = p/m + dt (f/m + g), colliders, d
//   g2p2g        per work item (<= 256 particles binned to one home block):
//                bulk-copy (TMA) the 27 pool blocks around the home block
//                into shared memory, gather v* and d (G2P), update F_E with
//                the SVD clamp, J_p, velocity, colliders, position (particle
//                advance), then scatter the updated particles (P2G of the
//                next step) into a 9^3-node shared tile, cell by cell, and
//                add the tile to acc. A CTA takes a contiguous range of
//                items; consecutive items of one home block (a run) share
//                the staged grid blocks and the tile, which is added to acc
//                once per run.
// Separate P2G and G2P kernels serve the first step after set-up and the
// per-kernel dispatch entry point.
#include "snow_internal.h"
#include "snow_math.cuh"
#include "snow_stats.cuh"
#include "snow_tma.cuh"
#include "fast_item.cuh"

namespace snow {
namespace {

// ===========================================================================
__device__ __forceinline__ void form_prefixes(const SceneDev* __restrict__ scenes, int nscenes, int* items,
                                              int* active) {
  int ai = 0, aa = 0;
  for (int s = 0; s < nscenes; s++) {
    items[s] = ai;
    active[s] = aa;
    ai += *(volatile int*)&scenes[s].counters[CNT_ITEMS];
    aa += min(*(volatile int*)&scenes[s].counters[CNT_ACTIVE], scenes[s].pool_cap);
  }
  items[nscenes] = ai;
  active[nscenes] = aa;
}

__global__ void k_prefix(const SceneDev* __restrict__ scenes, int nscenes, int* items, int* active) {
  if (threadIdx.x == 0 && blockIdx.x == 0) form_prefixes(scenes, nscenes, items, active);
}

// One CTA per scene: the step's counters reset, colliders advanced.
__global__ void k_begin_step(const SceneDev* __restrict__ scenes, int nscenes, int rigid) {
  const int s = blockIdx.x;
  if (s >= nscenes) return;
  const SceneDev& S = scenes[s];
  if (threadIdx.x == 0) {
    S.counters[CNT_ACTIVE] = 0;
    S.counters[CNT_OVERFLOW] = 0;
    S.counters[CNT_BINNED] = 0;
    // the magnitudes of the particles the pending P2G scattered become the
    // ones this step's P2G chooses its fixed-point scales from
    FixState& f = *S.fix;
    f.m_prev = f.m_cur;
    f.v_prev = f.v_cur;
    f.a_prev = f.a_cur;
    f.m_cur = f.v_cur = f.a_cur = 0u;
  }
  if (rigid)  // rigidAdvance.glsl:14-18
    for (int i = threadIdx.x; i < S.ncoll; i += blockDim.x)
      for (int k = 0; k < 3; k++) S.coll[i].pos[k] = S.coll[i].pos[k] + S.dt * S.coll[i].vel[k];
  if (S.crs) {  // the semi-implicit solve's scalars start from zero each step
    int* c = reinterpret_cast<int*>(S.crs);
    for (int i = threadIdx.x; i < (int)(offsetof(CrScalars, skipping) / sizeof(int)); i += blockDim.x) c[i] = 0;
    if (threadIdx.x == 0) {  // a step within kCrSkipSteps of a start below kCrSkipFactor * tol skips the solve
      CrScalars& cs = *S.crs;
      cs.skipping = cs.skip_left > 0 ? 1 : 0;
      if (cs.skip_left > 0) cs.skip_left--;
    }
  }
}

__global__ void k_gather_counters(const SceneDev* __restrict__ scenes, int nscenes, int* out) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nscenes * kCounterStride; i += gridDim.x * blockDim.x)
    out[i] = scenes[i / kCounterStride].counters[i % kCounterStride];
  __threadfence_system();
}

// Flags -> active-block list and pool slots (one thread per block); the CTA
// that finishes last forms the item and active-block prefixes.
__global__ void k_compact(const SceneDev* __restrict__ scenes, const int* __restrict__ block_prefix, int nscenes,
                          long long total, int* items_prefix, int* active_prefix) {
  for (long long u = blockIdx.x * (long long)blockDim.x + threadIdx.x; u < total;
       u += (long long)gridDim.x * blockDim.x) {
    const int s = find_scene(block_prefix, nscenes, u);
    const SceneDev& S = scenes[s];
    const int b = (int)(u - block_prefix[s]);
    int slot = -1;
    if (S.blk_flag[b]) {
      S.blk_flag[b] = 0;
      slot = atomicAdd(&S.counters[CNT_ACTIVE], 1);
      if (slot >= S.pool_cap) {
        atomicAdd(&S.counters[CNT_OVERFLOW], 1);
        slot = -1;
      } else {
        S.active[slot] = b;
      }
    }
    S.blk_slot[b] = slot;
  }
  __shared__ bool last;
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    last = atomicAdd(&scenes[0].counters[CNT_DONE], 1) == (int)gridDim.x - 1;
  }
  __syncthreads();
  if (last && threadIdx.x == 0) {
    __threadfence();
    form_prefixes(scenes, nscenes, items_prefix, active_prefix);
    scenes[0].counters[CNT_DONE] = 0;
  }
}

// Largest mass, |v|, force-term bound and initial volume of the particles a
// P2G of the stored state scatters (with_stress: A from an SVD of F_E, as
// that P2G computes it), into FixState's *_prev and *_cur (zeroed before).
__global__ void __launch_bounds__(256) k_fix_measure(const SceneDev* __restrict__ sd, int with_stress) {
  const SceneDev& S = *sd;
  float mm = 0.0f, vm = 0.0f, am = 0.0f, v0 = 0.0f;
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < S.n; p += gridDim.x * blockDim.x) {
    const float4 xm = S.xm[p];
    if (!(fabsf(xm.w) <= 100.0f)) continue;  // not scattered (p2gTransfer.glsl:64-66)
    const float4 vv = S.vv[p];
    mm = fmaxf(mm, fabsf(xm.w));
    vm = fmaxf(vm, sqrtf(vv.x * vv.x + vv.y * vv.y + vv.z * vv.z));
    v0 = fmaxf(v0, vv.w);
    if (with_stress) am = fmaxf(am, p2g_particle(S, p, xm, false).a);
  }
  const unsigned bm = __reduce_max_sync(0xffffffffu, __float_as_uint(mm));
  const unsigned bv = __reduce_max_sync(0xffffffffu, __float_as_uint(vm));
  const unsigned ba = __reduce_max_sync(0xffffffffu, __float_as_uint(am));
  const unsigned b0 = __reduce_max_sync(0xffffffffu, __float_as_uint(v0));
  if ((threadIdx.x & 31) == 0) {
    FixState& f = *S.fix;
    atomicMax(&f.m_prev, bm);
    atomicMax(&f.m_cur, bm);
    atomicMax(&f.v_prev, bv);
    atomicMax(&f.v_cur, bv);
    atomicMax(&f.a_prev, ba);
    atomicMax(&f.a_cur, ba);
    atomicMax(&f.v0max, b0);
  }
}

// P2G of the stored particle state (p2gTransfer.glsl:44-151, or
// gMassCompute.glsl:33-84 when MASS_ONLY), at the scales k_fix_measure's
// magnitudes give; the CTA that takes a scene's first item records them for
// the grid update.
template <bool MASS_ONLY>
__global__ void __launch_bounds__(kItemMax, 2) k_p2g(const SceneDev* __restrict__ scenes,
                                                  const int* __restrict__ item_prefix, int nscenes) {
  extern __shared__ float4 smem_raw[];
  ItemShared& sh = *reinterpret_cast<ItemShared*>(smem_raw);
  tile_init(sh);
  constexpr int KIND = MASS_ONLY ? kP2gMass : kP2gFull;
  const int total = item_prefix[nscenes];
  for (int u = blockIdx.x; u < total; u += gridDim.x) {
    const int s = find_scene(item_prefix, nscenes, u);
    const SceneDev& S = scenes[s];
    const int4 it = S.items[u - item_prefix[s]];
    const FixScale sc = measured_scales(S);
    if (u == item_prefix[s] && threadIdx.x == 0) {
      S.fix->scale[0] = sc.m;
      S.fix->scale[1] = sc.p;
      S.fix->scale[2] = sc.f;
    }
    tile_zero(sh, P2gFields<KIND>::nf);
    int bx, by, bz;
    home_coords(S, it.x, bx, by, bz);
    const int i = threadIdx.x;
    bool have = false;
    P2GParticle q;
    q.force = false;
    q.a = 0.0f;
    AxisW w;
    int base[3] = {0, 0, 0};
    if (i < min(it.z, kItemMax)) {
      const int p = it.y + i;
      const float4 xm = S.xm[p];
      if (fabsf(xm.w) <= 100.0f) {  // p2gTransfer.glsl:64-66
        float pg[3];
        grid_coords(S, xm, pg, base);
        all_weights(pg, base, w);
        q = p2g_particle(S, p, xm, MASS_ONLY);
        have = true;
      }
    }
    p2g_tile_accumulate<KIND>(sh, S, bx, by, bz, have, q, w, base, sc);
    p2g_tile_flush<KIND>(sh, S, bx, by, bz);
    __syncthreads();
  }
}

// gForceCompute.glsl:57-103 for one node of active block b (pool slot
// `slot`) from its seven fixed-point sums w.
__device__ __forceinline__ void grid_node(const SceneDev& S, int slot, int b, int node,
                                          const unsigned long long (&w)[kAccWords]) {
  // the fixed-point sums back to floats (the scales are powers of two)
  const FixState& fx = *S.fix;
  const float ism = 1.0f / fx.scale[0], isp = 1.0f / fx.scale[1], isf = 1.0f / fx.scale[2];
  const long long mq = (long long)w[0];
  const float v[kAccFields] = {(float)mq * ism,
                               (float)(long long)w[1] * isp,
                               (float)(long long)w[2] * isp,
                               (float)(long long)w[3] * isp,
                               (float)(long long)w[4] * isf,
                               (float)(long long)w[5] * isf,
                               (float)(long long)w[6] * isf};
  float2* out = reinterpret_cast<float2*>(S.gout + (size_t)slot * kOutBlockFloats + kOutFields * node);
  const float mi = v[0];
  float vs[3] = {0.0f, 0.0f, 0.0f}, d[3] = {0.0f, 0.0f, 0.0f};
  if (mq > 0) {
    const float inv = 1.0f / mi;
    const float vold[3] = {v[1] * inv, v[2] * inv, v[3] * inv};
#pragma unroll
    for (int k = 0; k < 3; k++) vs[k] = vold[k] + S.dt * (v[4 + k] * inv + S.grav[k]);
    const int bx = b % S.bdim[0], by = (b / S.bdim[0]) % S.bdim[1], bz = b / (S.bdim[0] * S.bdim[1]);
    const int gi = 4 * bx + (node & 3), gj = 4 * by + ((node >> 2) & 3), gk = 4 * bz + (node >> 4);
    // node position as Grid::initSSBO forms it: x_off + h * (float)i
    const float xi[3] = {__fadd_rn(S.gpos[0], __fmul_rn(S.h, (float)gi)),
                         __fadd_rn(S.gpos[1], __fmul_rn(S.h, (float)gj)),
                         __fadd_rn(S.gpos[2], __fmul_rn(S.h, (float)gk))};
    collide(S.coll, S.ncoll, xi, vs);
#pragma unroll
    for (int k = 0; k < 3; k++) d[k] = vs[k] - S.alpha * vold[k];
  }
  out[0] = make_float2(vs[0], vs[1]);
  out[1] = make_float2(vs[2], d[0]);
  out[2] = make_float2(d[1], d[2]);
  if (S.crs && !S.crs->skipping) {  // semi-implicit: the solve starts from x = v* and applies K to v* first
    const size_t i = (size_t)slot * kBlockNodes + node;
    S.crv[i] = make_float4(vs[0], vs[1], vs[2], mi > 0.0f ? mi : 0.0f);
    float* u = S.cru + (size_t)slot * kImpBlockFloats + 3 * node;
    u[0] = vs[0];
    u[1] = vs[1];
    u[2] = vs[2];
  }
}

// The grid update on the active blocks, one 64-thread group per block (a
// warp lies inside one group, so inside one scene). Each group's blocks are
// staged by TMA: a block's fixed-point record is one contiguous 3,584-byte
// bulk copy into the group's shared buffer, and the group's next block is
// copied while it converts, updates and writes the current one. The P2G
// sums are consumed (zeroed) here. clear_only: the sums are zeroed and
// nothing is staged or written (scene set-up).
constexpr int kGridGroups = 4;  // 64-thread groups per CTA
__global__ void __launch_bounds__(kGridGroups * kBlockNodes) k_grid(const SceneDev* __restrict__ scenes,
                                                                    const int* __restrict__ active_prefix,
                                                                    int nscenes, int clear_only) {
  __shared__ __align__(128) unsigned long long buf[kGridGroups][kAccBlockWords];
  __shared__ uint64_t bar[kGridGroups];
  __shared__ int gabort[kGridGroups];
  const int g = threadIdx.x / kBlockNodes, node = threadIdx.x % kBlockNodes;
  const long long total = active_prefix[nscenes];
  const long long stride = (long long)gridDim.x * kGridGroups;
  long long u = (long long)blockIdx.x * kGridGroups + g;
  if (clear_only) {
    for (; u < total; u += stride) {
      const int s = find_scene(active_prefix, nscenes, u);
      const SceneDev& S = scenes[s];
      unsigned long long* acc = S.acc + (size_t)S.active[(int)(u - active_prefix[s])] * kAccBlockWords + node;
#pragma unroll
      for (int k = 0; k < kAccWords; k++) acc[k * kBlockNodes] = 0ull;
    }
    return;
  }
  constexpr uint32_t kBytes = kAccBlockWords * sizeof(unsigned long long);
  static_assert(kBytes % 16 == 0, "bulk copies move multiples of 16 bytes");
  if (node == 0) {
    mbar_init(&bar[g], 1);
    gabort[g] = 0;
  }
  __syncthreads();
  // the block of work unit uu: its scene, pool slot and block id
  auto locate = [&](long long uu, int& s, int& slot, int& b) {
    s = find_scene(active_prefix, nscenes, uu);
    slot = (int)(uu - active_prefix[s]);
    b = scenes[s].active[slot];
  };
  auto issue = [&](long long uu) {  // by the group's thread 0
    int s, slot, b;
    locate(uu, s, slot, b);
    const SceneDev& S = scenes[s];
    mbar_arrive_expect_tx(&bar[g], kBytes + S.tx_unsent);
    fence_proxy_async_smem();
    bulk_g2s(buf[g], S.acc + (size_t)b * kAccBlockWords, kBytes, &bar[g]);
  };
  if (u < total && node == 0) issue(u);
  uint32_t phase = 0;
  for (; u < total; u += stride) {
    int s, slot, b;
    locate(u, s, slot, b);
    const SceneDev& S = scenes[s];
    unsigned long long w[kAccWords];
    const bool landed = mbar_wait(&bar[g], phase, S.wait_ns);
    if (landed) {
#pragma unroll
      for (int k = 0; k < kAccWords; k++) w[k] = buf[g][k * kBlockNodes + node];
    } else {
      gabort[g] = 1 + (int)phase;
    }
    asm volatile("bar.sync %0, %1;" ::"r"(g + 1), "r"(kBlockNodes) : "memory");  // the group has read its buffer
    if (gabort[g]) {
      // the copy did not land in time: counted, one more bounded wait for it
      // (the CTA must not exit while it may still land), and the group stops
      if (node == 0) {
        atomicAdd(&S.counters[CNT_TIMEOUT], 1);
        mbar_wait(&bar[g], (uint32_t)(gabort[g] - 1), S.wait_ns);
      }
      return;
    }
    phase ^= 1u;
    if (node == 0 && u + stride < total) issue(u + stride);
    unsigned long long* acc = S.acc + (size_t)b * kAccBlockWords + node;
#pragma unroll
    for (int k = 0; k < kAccWords; k++) acc[k * kBlockNodes] = 0ull;
    grid_node(S, slot, b, node, w);
  }
}

// pVolumeCompute.glsl:32-83: rho0 = sum_i m_i w_ip / h^3 from the grid mass,
// stored as V0 = m / rho0 (0 when rho0 <= 0, which disables the force as
// p2gTransfer.glsl:126 does).
__global__ void __launch_bounds__(256) k_volume(const SceneDev* __restrict__ sd) {
  const SceneDev& S = *sd;
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < S.n; p += gridDim.x * blockDim.x) {
    const float4 xm = S.xm[p];
    float pg[3];
    int base[3];
    grid_coords(S, xm, pg, base);
    AxisW w;
    all_weights(pg, base, w);
    float rho = 0.0f;
    for (int c = 0; c < 4; c++)
      for (int b = 0; b < 4; b++)
        for (int a = 0; a < 4; a++) {
          const int g0 = base[0] - 1 + a, g1 = base[1] - 1 + b, g2 = base[2] - 1 + c;
          if (!node_in_grid(S, g0, g1, g2)) continue;
          const int blk = block_id(S, g0 >> 2, g1 >> 2, g2 >> 2);
          const long long mq = (long long)S.acc[(size_t)blk * kAccBlockWords + (g0 & 3) + 4 * (g1 & 3) + 16 * (g2 & 3)];
          const float mi = (float)mq / S.fix->scale[0];
          rho += mi * (sel4(a, w.wx[0], w.wx[1], w.wx[2], w.wx[3]) * sel4(b, w.wy[0], w.wy[1], w.wy[2], w.wy[3]) *
                       sel4(c, w.wz[0], w.wz[1], w.wz[2], w.wz[3]));
        }
    rho = rho / (S.h * S.h * S.h);
    float4 vv = S.vv[p];
    vv.w = rho > 0.0f ? xm.w / rho : 0.0f;
    S.vv[p] = vv;
  }
}

// g2pTransfer.glsl:53-143 fused with particleAdvance.glsl:75-217 (no P2G).
__global__ void __launch_bounds__(kItemMax) k_g2p_advance(const SceneDev* __restrict__ scenes,
                                                          const int* __restrict__ item_prefix, int nscenes) {
  extern __shared__ float4 smem_raw[];
  ItemShared& sh = *reinterpret_cast<ItemShared*>(smem_raw);
  tile_init(sh);
  const int total = item_prefix[nscenes];
  uint32_t phase = 0;
  for (int u = blockIdx.x; u < total; u += gridDim.x) {
    const int s = find_scene(item_prefix, nscenes, u);
    const SceneDev& S = scenes[s];
    const int4 it = S.items[u - item_prefix[s]];
    int bx, by, bz;
    home_coords(S, it.x, bx, by, bz);
    if (threadIdx.x < 32) stage_issue(sh, S, tile_slot(S, it, threadIdx.x));
    load_colliders(sh, S);
    stage_wait(sh, S, phase);
    __syncthreads();
    if (sh.abort) {
      stage_abort(sh, S);
      return;
    }
    for (int i = threadIdx.x; i < it.z; i += blockDim.x) {
      const int p = it.y + i;
      const PState ps = load_state(S, p, false);  // per-kernel dispatches: binned in place
      float pg[3];
      int base[3];
      grid_coords(S, ps.xm, pg, base);
      AxisW w;
      all_weights(pg, base, w);
      float dv[3], L[3][3];
      g2p_gather(sh, S, bx, by, bz, base, w, dv, L);
      Advanced adv;
      advance_particle(S, p, ps, load_def(S, p, false), dv, L, sh, adv);
    }
    __syncthreads();
  }
}

// One explicit step per particle: G2P + particle advance of this step and
// P2G of the next, in one pass over the item's particles. The P2G stress uses
// the rotation R = W V^T of the advance's SVD: F_E' = W S' V^T with S'
// diagonal up to the Jacobi residual, whose polar rotation is W V^T.
// A CTA takes a contiguous range of work items. Consecutive items of one
// home block form a run: they share
// the staged pool blocks (copied once, by bulk copies issued while the
// previous run's last item sums its P2G) and the P2G tile (added to acc
// once, at the run's end). The P2G sums are fixed
// point at the scales step_scales gives; the CTA that takes a scene's first
// item records them for the next grid update, and every CTA records the
// magnitudes of its particles for the next step's scales. BINNED: a step that
// re-binned some scene; such a scene's particles are read from its binned
// copies (CNT_BINNED) and, like every scene's, written to its streams.
template <bool BINNED>
__global__ void __launch_bounds__(kItemMax, 2) k_g2p2g(const SceneDev* __restrict__ scenes,
                                                       const int* __restrict__ item_prefix, int nscenes) {
  extern __shared__ float4 smem_raw[];
  ItemShared& sh = *reinterpret_cast<ItemShared*>(smem_raw);
  tile_init(sh);
  const int total = item_prefix[nscenes];
  const int chunk = (total + (int)gridDim.x - 1) / (int)gridDim.x;
  const int u0 = min(total, (int)blockIdx.x * chunk), u1 = min(total, u0 + chunk);
  if (u0 >= u1) return;
  // The last warp, which holds the fewest particles of an item (items are
  // filled from thread 0), looks up the next item and its pool slots.
  const int lane = threadIdx.x & 31;
  const bool lastw = (threadIdx.x >> 5) == (blockDim.x >> 5) - 1;
  if (lastw) {
    const int s0 = find_scene(item_prefix, nscenes, u0);
    const int4 it0 = scenes[s0].items[u0 - item_prefix[s0]];
    stage_issue(sh, scenes[s0], tile_slot(scenes[s0], it0, lane));
    if (lane == 0) {
      sh.item_q[0] = it0;
      sh.scene_q[0] = s0;
      sh.coll_scene = -1;
      sh.next_same = 0;
    }
  }
  uint32_t phase = 0;
  int par = 0;
  bool run_start = true;  // uniform across the CTA
  for (int u = u0; u < u1; u++, par ^= 1) {
    __syncthreads();  // this item's queue entry is written; the last flush is done
    const int s = sh.scene_q[par];
    const SceneDev& S = scenes[s];
    if (s != sh.coll_scene) {  // uniform across the CTA
      if (threadIdx.x == 0) {
        sh.fscale = step_scales(S);
        sh.seen[0] = sh.seen[1] = sh.seen[2] = 0u;
        sh.pushed[0] = sh.pushed[1] = sh.pushed[2] = 0u;
      }
      load_colliders(sh, S);  // its closing barrier publishes fscale as well
      if (threadIdx.x == 0) {
        sh.coll_scene = s;
        if (u == item_prefix[s]) {
          S.fix->scale[0] = sh.fscale.m;
          S.fix->scale[1] = sh.fscale.p;
          S.fix->scale[2] = sh.fscale.f;
        }
      }
    }
    if (run_start) {
      tile_zero(sh, kAccFields);
      if (threadIdx.x == 0) sh.run_bound = 0.0f;
    }
    const int4 it = sh.item_q[par];
    const int un = u + 1;
    // the next item's descriptor and pool slots: loaded now, so that the
    // loads' latency overlaps this item's G2P instead of delaying the last
    // warp, and put in shared memory before this item's P2G
    int sn = 0, slot = -1;
    int4 itn = make_int4(0, 0, 0, 0);
    bool same = false;
    if (lastw && un < u1) {
      sn = find_scene(item_prefix, nscenes, un);
      itn = scenes[sn].items[un - item_prefix[sn]];
      same = sn == s && itn.x == it.x;
      if (!same) slot = tile_slot(scenes[sn], itn, lane);
    }
    int bx, by, bz;
    home_coords(S, it.x, bx, by, bz);
    const int i = threadIdx.x;
    const bool mine = i < min(it.z, kItemMax);
    const int p = it.y + i;
    PState ps;
    const bool binned = BINNED && particles_binned(S);
    if (mine) ps = load_state(S, p, binned);
    const bool landed = run_start ? stage_wait(sh, S, phase) : true;
    bool have = false;
    P2GParticle q;
    q.force = false;
    q.a = 0.0f;
    AxisW wn;
    int nbase[3] = {0, 0, 0};
    float rec_v = 0.0f;
    if (mine && landed) {
      float pg[3];
      int base[3];
      grid_coords(S, ps.xm, pg, base);
      AxisW w;
      all_weights(pg, base, w);
      float dv[3], L[3][3];
      g2p_gather(sh, S, bx, by, bz, base, w, dv, L);
      const PDef def = load_def(S, p, binned);
      Advanced adv;
      advance_particle(S, p, ps, def, dv, L, sh, adv);
      // P2G quantities of the advanced particle
      q.m = adv.xm.w;
      if (fabsf(q.m) <= 100.0f) {  // p2gTransfer.glsl:64-66
        have = true;
        q.mv[0] = q.m * adv.vv.x;
        q.mv[1] = q.m * adv.vv.y;
        q.mv[2] = q.m * adv.vv.z;
        rec_v = sqrtf(adv.vv.x * adv.vv.x + adv.vv.y * adv.vv.y + adv.vv.z * adv.vv.z);
        if (adv.vv.w > 0.0f) p2g_stress(S, adv.fe, adv.R, adv.jp, adv.vv.w, q);
        float npg[3];
        grid_coords(S, adv.xm, npg, nbase);
        all_weights(npg, nbase, wn);
      }
    }
    {  // the magnitudes the next step's scales are chosen from (per warp, then per CTA)
      const unsigned bm = __reduce_max_sync(0xffffffffu, have ? __float_as_uint(fabsf(q.m)) : 0u);
      const unsigned bv = __reduce_max_sync(0xffffffffu, __float_as_uint(rec_v));
      const unsigned ba = __reduce_max_sync(0xffffffffu, __float_as_uint(q.a));
      if (lane == 0) {
        atomicMax(&sh.seen[0], bm);
        atomicMax(&sh.seen[1], bv);
        atomicMax(&sh.seen[2], ba);
      }
    }
    // the next item's queue entry: every thread read this one's at the loop
    // top, and the accumulation's barriers publish it before the flush
    // decision below
    if (lastw) {  // kept in shared memory, not registers, across the accumulation
      sh.next_slot[lane] = slot;
      if (lane == 0) {
        sh.item_q[par ^ 1] = itn;
        sh.scene_q[par ^ 1] = sn;
        sh.next_same = same ? 1 : 0;
        sh.next_issue = un < u1 && !same ? 1 : 0;
      }
    }
    if (!p2g_tile_accumulate<kP2gFull, true>(sh, S, bx, by, bz, have, q, wn, nbase, sh.fscale)) {
      stage_abort(sh, S);  // a copy wait ran out: this item's particles keep their state, the CTA stops
      return;
    }
    if (lastw && sh.next_issue)  // uniform in the warp
      stage_issue(sh, scenes[sh.scene_q[par ^ 1]], lane < 27 ? sh.next_slot[lane] : -1);
    if (threadIdx.x == 0) {  // only maxima above what this CTA already recorded go to HBM
      unsigned* cur[3] = {&S.fix->m_cur, &S.fix->v_cur, &S.fix->a_cur};
#pragma unroll
      for (int k = 0; k < 3; k++)
        if (sh.seen[k] > sh.pushed[k]) {
          atomicMax(cur[k], sh.seen[k]);
          sh.pushed[k] = sh.seen[k];
        }
    }
    const bool cont = sh.next_same != 0;  // uniform across the CTA
    if (!cont) p2g_tile_flush<kP2gFull>(sh, S, bx, by, bz);
    run_start = !cont;
  }
}

// Bulk statistics: per-thread sums in FP32 over a dozen particles, then FP64
// across threads (FP64 arithmetic is slow on this part: the per-particle work
// stays in FP32).
__global__ void __launch_bounds__(kStatsThreads) k_stats(const SceneDev* __restrict__ sd, int n, StatsSlot* slot,
                                               StatsAccum* host) {
  const SceneDev& S = *sd;
  float acc[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  StatsPartial t;
  stats_init(t);
  // four particles per thread and pass, their loads issued together
  constexpr int U = 4;
  const int stride = gridDim.x * blockDim.x;
  for (int p0 = blockIdx.x * blockDim.x + threadIdx.x; p0 < n; p0 += U * stride) {
    float4 xm[U], vv[U];
    float jp[U];
#pragma unroll
    for (int u = 0; u < U; u++) {
      const int p = p0 + u * stride;
      if (p < n) {
        xm[u] = S.xm[p];
        vv[u] = S.vv[p];
        jp[u] = S.fc[p].y;
      }
    }
#pragma unroll
    for (int u = 0; u < U; u++) {
      if (p0 + u * stride >= n) break;
      const float m = xm[u].w;
      const bool ok = isfinite(xm[u].x) && isfinite(xm[u].y) && isfinite(xm[u].z) && isfinite(vv[u].x) &&
                      isfinite(vv[u].y) && isfinite(vv[u].z) && isfinite(jp[u]);
      if (!ok) {
        t.bad++;
        continue;
      }
      acc[0] += m;
      acc[1] += m * vv[u].x;
      acc[2] += m * vv[u].y;
      acc[3] += m * vv[u].z;
      acc[4] += 0.5f * m * (vv[u].x * vv[u].x + vv[u].y * vv[u].y + vv[u].z * vv[u].z);
      acc[5] += m * xm[u].x;
      acc[6] += m * xm[u].y;
      acc[7] += m * xm[u].z;
      acc[8] += jp[u];
      t.bmin[0] = fminf(t.bmin[0], xm[u].x); t.bmin[1] = fminf(t.bmin[1], xm[u].y); t.bmin[2] = fminf(t.bmin[2], xm[u].z);
      t.bmax[0] = fmaxf(t.bmax[0], xm[u].x); t.bmax[1] = fmaxf(t.bmax[1], xm[u].y); t.bmax[2] = fmaxf(t.bmax[2], xm[u].z);
    }
  }
#pragma unroll
  for (int k = 0; k < 9; k++) t.acc[k] = acc[k];
  stats_commit(t, slot, host);
}

// Upload: the caller's arrays (x, v: N x 3; m: N; FE, FP: N x 9 row-major or
// null for identity), copied to the device as they are, packed into the
// particle streams. J_p = det F_P in double without contraction, as the
// host formerly computed it.
__global__ void __launch_bounds__(256) k_pack(const float* __restrict__ x, const float* __restrict__ v,
                                              const float* __restrict__ m, const float* __restrict__ FE,
                                              const float* __restrict__ FP, size_t n, float4* xm, float4* vv,
                                              float4* fa, float4* fb, float2* fc, uint32_t* pid, float4* vq) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    xm[i] = make_float4(x[3 * i], x[3 * i + 1], x[3 * i + 2], m[i]);
    vv[i] = make_float4(v[3 * i], v[3 * i + 1], v[3 * i + 2], 0.0f);
    float F[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
    if (FE)
#pragma unroll
      for (int k = 0; k < 9; k++) F[k] = FE[9 * i + k];
    fa[i] = make_float4(F[0], F[3], F[6], F[1]);
    fb[i] = make_float4(F[4], F[7], F[2], F[5]);
    float jp = 1.0f;
    if (FP) {
      const float* f = FP + 9 * i;
      const double a = f[0], b = f[1], c = f[2], d = f[3], e = f[4], g = f[5], h = f[6], ii = f[7], j = f[8];
      const double t0 = __dsub_rn(__dmul_rn(e, j), __dmul_rn(g, ii));
      const double t1 = __dsub_rn(__dmul_rn(d, j), __dmul_rn(g, h));
      const double t2 = __dsub_rn(__dmul_rn(d, ii), __dmul_rn(e, h));
      jp = (float)__dadd_rn(__dsub_rn(__dmul_rn(a, t0), __dmul_rn(b, t1)), __dmul_rn(c, t2));
    }
    fc[i] = make_float2(F[8], jp);
    pid[i] = (uint32_t)i;
    vq[i] = make_float4(1.0f, 0.0f, 0.0f, 0.0f);  // no previous SVD: identity frame
  }
}

// Download: the particle streams back to the caller's layout and order
// (slot i holds upload index pid[i]); any output may be null.
__global__ void __launch_bounds__(256) k_unpack(const SceneDev* __restrict__ sd, size_t n, float* x, float* v,
                                                float* FE, float* Jp, float* volume) {
  const SceneDev& S = *sd;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const size_t j = S.pid[i];
    if (j >= n) continue;  // cannot happen: pid is a permutation
    const float4 xm = S.xm[i], vv = S.vv[i];
    if (x) {
      x[3 * j] = xm.x;
      x[3 * j + 1] = xm.y;
      x[3 * j + 2] = xm.z;
    }
    if (v) {
      v[3 * j] = vv.x;
      v[3 * j + 1] = vv.y;
      v[3 * j + 2] = vv.z;
    }
    const float2 c = S.fc[i];
    if (FE) {
      // fa = (m00, m01, m02, m10), fb = (m11, m12, m20, m21), fc = (m22, Jp); m[c][r]
      const float4 a = S.fa[i], b = S.fb[i];
      const float mcr[9] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w, c.x};
#pragma unroll
      for (int r = 0; r < 3; r++)
#pragma unroll
        for (int q = 0; q < 3; q++) FE[9 * j + 3 * r + q] = mcr[3 * q + r];
    }
    if (Jp) Jp[j] = c.y;
    if (volume) volume[j] = vv.w;
  }
}

// Dense copies of the P2G sums (acc) and of v* (pool) of the active blocks.
__global__ void k_download_grid(const SceneDev* __restrict__ sd, float* mass, float* mom, float* force, float* vstar) {
  const SceneDev& S = *sd;
  const int count = min(S.counters[CNT_ACTIVE], S.pool_cap);
  for (long long u = blockIdx.x * (long long)blockDim.x + threadIdx.x; u < (long long)count * kBlockNodes;
       u += (long long)gridDim.x * blockDim.x) {
    const int slot = (int)(u / kBlockNodes), node = (int)(u % kBlockNodes);
    const int b = S.active[slot];
    const int bx = b % S.bdim[0], by = (b / S.bdim[0]) % S.bdim[1], bz = b / (S.bdim[0] * S.bdim[1]);
    const int gi = 4 * bx + (node & 3), gj = 4 * by + ((node >> 2) & 3), gk = 4 * bz + (node >> 4);
    if (gi >= S.dim[0] || gj >= S.dim[1] || gk >= S.dim[2]) continue;
    const long long g = gi + (long long)S.dim[0] * (gj + (long long)S.dim[1] * gk);
    const float* out = S.gout + (size_t)slot * kOutBlockFloats + kOutFields * node;
    if (vstar)
      for (int k = 0; k < 3; k++) vstar[3 * g + k] = out[k];
  }
  // acc is dense: every block, every node
  for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x;
       g < (long long)S.dim[0] * S.dim[1] * S.dim[2]; g += (long long)gridDim.x * blockDim.x) {
    const int gi = (int)(g % S.dim[0]), gj = (int)((g / S.dim[0]) % S.dim[1]),
              gk = (int)(g / ((long long)S.dim[0] * S.dim[1]));
    const int blk = block_id(S, gi >> 2, gj >> 2, gk >> 2);
    const unsigned long long* acc = S.acc + (size_t)blk * kAccBlockWords + (gi & 3) + 4 * (gj & 3) + 16 * (gk & 3);
    const FixState& fx = *S.fix;
    if (mass) mass[g] = (float)(long long)acc[0] / fx.scale[0];
    for (int k = 0; k < 3; k++) {
      if (mom) mom[3 * g + k] = (float)(long long)acc[(1 + k) * kBlockNodes] / fx.scale[1];
      if (force) force[3 * g + k] = (float)(long long)acc[(4 + k) * kBlockNodes] / fx.scale[2];
    }
  }
}

template <class K>
void smem_opt_in(K kernel, int bytes) {
  cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
}

// Shared-memory opt-in of the work-item kernels, once per device (the
// attribute belongs to the function in each device's context).
int item_smem() {
  static bool configured[kMaxDevices] = {};
  const int bytes = (int)sizeof(ItemShared);
  const int dev = current_device();
  if (!configured[dev]) {
    smem_opt_in(k_p2g<true>, bytes);
    smem_opt_in(k_p2g<false>, bytes);
    smem_opt_in(k_g2p_advance, bytes);
    smem_opt_in(k_g2p2g<false>, bytes);
    smem_opt_in(k_g2p2g<true>, bytes);
    configured[dev] = true;
  }
  return bytes;
}

}  // namespace

int current_device() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) dev = 0;
  return dev;
}

// SM count of the current device (cached per device: launch grids are sized
// for the GPU the launch goes to).
int num_sms() {
  static int n[kMaxDevices] = {};
  const int dev = current_device();
  if (n[dev] == 0) {
    int v = 0;
    cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
    n[dev] = v > 0 ? v : 1;
  }
  return n[dev];
}


void fast_prefix(const SceneDev* scenes, int nscenes, int* items_prefix, int* active_prefix, cudaStream_t st) {
  k_prefix<<<1, 32, 0, st>>>(scenes, nscenes, items_prefix, active_prefix);
}

void fast_begin_step(const SceneDev* scenes, int nscenes, bool rigid, cudaStream_t st) {
  if (nscenes > 0) k_begin_step<<<nscenes, 32, 0, st>>>(scenes, nscenes, rigid ? 1 : 0);
}

void fast_gather_counters(const SceneDev* scenes, int nscenes, int* out, cudaStream_t st) {
  const int n = nscenes * kCounterStride;
  k_gather_counters<<<(n + 255) / 256, 256, 0, st>>>(scenes, nscenes, out);
}

void fast_compact(const SceneDev* scenes, const int* block_prefix, int nscenes, long long total_blocks,
                  int* items_prefix, int* active_prefix, cudaStream_t st) {
  long long g = (total_blocks + 255) / 256;
  g = g > (long long)num_sms() * 16 ? (long long)num_sms() * 16 : (g < 1 ? 1 : g);
  k_compact<<<(int)g, 256, 0, st>>>(scenes, block_prefix, nscenes, total_blocks, items_prefix, active_prefix);
}

void fast_p2g(const SceneDev* scenes, const SceneDev& sd_host, const int* item_prefix, int nscenes, int grid_ctas,
              bool mass_only, cudaStream_t st) {
  const int smem = item_smem();
  // the magnitudes of the particles, from which k_p2g chooses its scales
  cudaMemsetAsync(&sd_host.fix->m_prev, 0, offsetof(FixState, wide) - offsetof(FixState, m_prev), st);
  if (sd_host.n > 0) {
    int g = (sd_host.n + 255) / 256;
    if (g > num_sms() * 8) g = num_sms() * 8;
    k_fix_measure<<<g, 256, 0, st>>>(scenes, mass_only ? 0 : 1);
  }
  if (mass_only)
    k_p2g<true><<<grid_ctas, kItemMax, smem, st>>>(scenes, item_prefix, nscenes);
  else
    k_p2g<false><<<grid_ctas, kItemMax, smem, st>>>(scenes, item_prefix, nscenes);
}

void fast_grid(const SceneDev* scenes, const int* active_prefix, int nscenes, int grid_ctas, bool clear_only,
               cudaStream_t st) {
  k_grid<<<grid_ctas, kGridGroups * kBlockNodes, 0, st>>>(scenes, active_prefix, nscenes, clear_only ? 1 : 0);
}

void fast_volume(const SceneDev* sd_dev, int n, cudaStream_t st) {
  if (n <= 0) return;
  int g = (n + 255) / 256;
  if (g > num_sms() * 8) g = num_sms() * 8;
  k_volume<<<g, 256, 0, st>>>(sd_dev);
}

void fast_g2p_advance(const SceneDev* scenes, const int* item_prefix, int nscenes, int grid_ctas, cudaStream_t st) {
  k_g2p_advance<<<grid_ctas, kItemMax, item_smem(), st>>>(scenes, item_prefix, nscenes);
}

void fast_g2p2g(const SceneDev* scenes, const int* item_prefix, int nscenes, int grid_ctas, bool binned,
                cudaStream_t st) {
  if (binned)
    k_g2p2g<true><<<grid_ctas, kItemMax, item_smem(), st>>>(scenes, item_prefix, nscenes);
  else
    k_g2p2g<false><<<grid_ctas, kItemMax, item_smem(), st>>>(scenes, item_prefix, nscenes);
}

void fast_stats(const SceneDev* sd_dev, int n, StatsSlot* slot, StatsAccum* host, cudaStream_t st) {
  int g = (n + kStatsThreads - 1) / kStatsThreads;  // at least one block: it publishes the empty sums
  if (g > num_sms()) g = num_sms();  // one block per SM: measured fastest (fixed costs dominate)
  if (g > kStatsMaxBlocks) g = kStatsMaxBlocks;
  if (g < 1) g = 1;
  k_stats<<<g, kStatsThreads, 0, st>>>(sd_dev, n < 0 ? 0 : n, slot, host);
}


void fast_pack(const float* x, const float* v, const float* m, const float* FE, const float* FP, size_t n,
               const SceneDev& sd, cudaStream_t st) {
  if (n == 0) return;
  size_t g = (n + 255) / 256;
  if (g > (size_t)num_sms() * 8) g = (size_t)num_sms() * 8;
  k_pack<<<(int)g, 256, 0, st>>>(x, v, m, FE, FP, n, sd.xm, sd.vv, sd.fa, sd.fb, sd.fc, sd.pid, sd.vq);
}

void fast_unpack(const SceneDev* sd_dev, size_t n, float* x, float* v, float* FE, float* Jp, float* volume,
                 cudaStream_t st) {
  if (n == 0) return;
  size_t g = (n + 255) / 256;
  if (g > (size_t)num_sms() * 8) g = (size_t)num_sms() * 8;
  k_unpack<<<(int)g, 256, 0, st>>>(sd_dev, n, x, v, FE, Jp, volume);
}

void fast_download_grid(const SceneDev* sd_dev, float* mass, float* mom, float* force, float* vstar,
                        cudaStream_t st) {
  k_download_grid<<<num_sms() * 8, 256, 0, st>>>(sd_dev, mass, mom, force, vstar);
}

}  // namespace snow
