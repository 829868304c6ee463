// SNOW_MODE_FAST kernels for sm_103a: the explicit snow-MPM step of the
// reference (shader/compute/mpm/*.glsl) in FP32 without fixed-point
// quantisation, on a sparse blocked grid.
//
// Grid layout in HBM: the grid is cut into 4x4x4-node blocks. Each step the
// blocks touched by some particle's 4x4x4 stencil get a slot in a pool; the
// slot holds the block's P2G sums (acc: 7 fields x 64 nodes, field-major) and
// the grid update's output (gout: v* and d = v* - alpha p/m, 6 x 64).
// blk_slot maps block id -> slot for the current step; blk_flag collects the
// blocks the next step will touch (written by the particle update).
//
// Kernels of one step (all scenes of a batch in one launch each):
//   compact      flags -> slots, active list            (one thread per block)
//   p2g          per work item (<= 256 particles binned to one home block):
//                scatter into a 9x9x9-node shared-memory tile with shared
//                atomics, then flush the tile's non-empty nodes to the pool
//                with global atomics
//   grid         per active block: v* = p/m + dt (f/m + g), colliders, d
//   g2p_advance  per particle: gather v*, d; PIC/FLIP, velocity gradient,
//                F_E update with the SVD clamp, J_p, colliders, advection;
//                marks the blocks of the new stencil for the next step
// Work spaces of a batch are concatenated; prefix arrays map a unit to
// (scene, local unit).
#include "snow_internal.h"
#include "snow_math.cuh"

namespace snow {
namespace {

constexpr int kTile = 9;                     // tile nodes per axis: [4b-2, 4b+6]
constexpr int kTile3 = kTile * kTile * kTile;

__device__ __forceinline__ int find_scene(const int* __restrict__ prefix, int nscenes, long long u) {
  int lo = 0, hi = nscenes;
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if ((long long)prefix[mid] <= u)
      lo = mid;
    else
      hi = mid;
  }
  return lo;
}

__device__ __forceinline__ float sel4(int i, float a0, float a1, float a2, float a3) {
  return i == 0 ? a0 : (i == 1 ? a1 : (i == 2 ? a2 : a3));
}

// Axis weights of the 4 stencil nodes base-1 .. base+2 (cubic.include.glsl):
// w[a] = N(d_a), g[a] = N'(-d_a) with d_a = node - x/h, as the shaders
// evaluate weighting(d) and weightingGradient(-d).
__device__ __forceinline__ void axis_weights(float pg, int base, float w[4], float g[4]) {
#pragma unroll
  for (int a = 0; a < 4; a++) {
    const float d = (float)(base + a - 1) - pg;
    w[a] = bspline(d);
    g[a] = bspline_d(-d);
  }
}

__device__ __forceinline__ void load_fe(const SceneDev& S, int p, M3& F, float& jp) {
  const float4 a = S.fa[p];
  const float4 b = S.fb[p];
  const float2 c = S.fc[p];
  F.m[0][0] = a.x; F.m[0][1] = a.y; F.m[0][2] = a.z;
  F.m[1][0] = a.w; F.m[1][1] = b.x; F.m[1][2] = b.y;
  F.m[2][0] = b.z; F.m[2][1] = b.w; F.m[2][2] = c.x;
  jp = c.y;
}
__device__ __forceinline__ void store_fe(const SceneDev& S, int p, const M3& F, float jp) {
  S.fa[p] = make_float4(F.m[0][0], F.m[0][1], F.m[0][2], F.m[1][0]);
  S.fb[p] = make_float4(F.m[1][1], F.m[1][2], F.m[2][0], F.m[2][1]);
  S.fc[p] = make_float2(F.m[2][2], jp);
}

__device__ __forceinline__ int block_id(const SceneDev& S, int bx, int by, int bz) {
  return (bz * S.bdim[1] + by) * S.bdim[0] + bx;
}

// Flags every grid block that holds a node of the stencil of a particle at
// grid coordinates pg (nodes outside the grid are not part of any block).
__device__ __forceinline__ void mark_stencil(const SceneDev& S, const float pg[3]) {
  int lo[3], hi[3];
#pragma unroll
  for (int k = 0; k < 3; k++) {
    const int base = (int)pg[k];
    lo[k] = max(base - 1, 0);
    hi[k] = min(base + 2, S.dim[k] - 1);
    if (lo[k] > hi[k]) return;
    lo[k] >>= 2;
    hi[k] >>= 2;
  }
  for (int bz = lo[2]; bz <= hi[2]; bz++)
    for (int by = lo[1]; by <= hi[1]; by++)
      for (int bx = lo[0]; bx <= hi[0]; bx++) S.blk_flag[block_id(S, bx, by, bz)] = 1;
}

// Collider projection of gForceCompute.glsl:72-93 / particleAdvance.glsl:182-204.
__device__ __forceinline__ void collide(const SceneDev& S, const float x[3], float v[3]) {
  for (int i = 0; i < S.ncoll; i++) {
    const snow_collider c = S.coll[i];
    float n[3] = {c.normal[0], c.normal[1], c.normal[2]};
    bool hit = false;
    if (c.type == 0) {
      hit = (x[0] - c.pos[0]) * c.normal[0] + (x[1] - c.pos[1]) * c.normal[1] + (x[2] - c.pos[2]) * c.normal[2] <=
            0.0f;
    } else if (c.type == 1) {
      const float d[3] = {x[0] - c.pos[0], x[1] - c.pos[1], x[2] - c.pos[2]};
      const float len = sqrtf(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
      n[0] = d[0] / len;
      n[1] = d[1] / len;
      n[2] = d[2] / len;
      hit = len < c.radius;
    }
    if (!hit) continue;
    const float vrel[3] = {v[0] - c.vel[0], v[1] - c.vel[1], v[2] - c.vel[2]};
    const float vn = vrel[0] * n[0] + vrel[1] * n[1] + vrel[2] * n[2];
    if (vn < 0.0f) {
      const float vt[3] = {vrel[0] - n[0] * vn, vrel[1] - n[1] * vn, vrel[2] - n[2] * vn};
      const float muvn = c.friction * vn;
      const float lvt = sqrtf(vt[0] * vt[0] + vt[1] * vt[1] + vt[2] * vt[2]);
      if (lvt <= -muvn) {
        v[0] = c.vel[0];
        v[1] = c.vel[1];
        v[2] = c.vel[2];
      } else {
        const float s = muvn / lvt;
#pragma unroll
        for (int k = 0; k < 3; k++) v[k] = vt[k] + s * vt[k] + c.vel[k];
      }
    }
  }
}

// ---------------------------------------------------------------------------
__global__ void k_prefix(const SceneDev* __restrict__ scenes, int nscenes, int counter, int* prefix) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    int acc = 0;
    for (int s = 0; s < nscenes; s++) {
      prefix[s] = acc;
      int c = scenes[s].counters[counter];
      if (counter == CNT_ACTIVE) c = min(c, scenes[s].pool_cap);
      acc += c;
    }
    prefix[nscenes] = acc;
  }
}

__global__ void k_compact(const SceneDev* __restrict__ scenes, const int* __restrict__ block_prefix, int nscenes,
                          long long total) {
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
}

// Marks the stencil blocks of every particle (first step after init).
__global__ void k_mark(const SceneDev* __restrict__ scenes, const int* __restrict__ chunk_prefix, int nscenes,
                       long long total_chunks) {
  for (long long u = blockIdx.x; u < total_chunks; u += gridDim.x) {
    const int s = find_scene(chunk_prefix, nscenes, u);
    const SceneDev& S = scenes[s];
    const int p = (int)(u - chunk_prefix[s]) * blockDim.x + threadIdx.x;
    if (p >= S.n) continue;
    const float4 xm = S.xm[p];
    const float pg[3] = {(xm.x - S.gpos[0]) / S.h, (xm.y - S.gpos[1]) / S.h, (xm.z - S.gpos[2]) / S.h};
    mark_stencil(S, pg);
  }
}

// Per-particle P2G quantities: mass, momentum and A = -V0 * stress where
// stress = 2 mu(Jp) (FE - R) FE^T + lambda(Jp) (JE - 1) JE I, R the polar
// rotation of FE (p2gTransfer.glsl:109-141).
struct P2GParticle {
  float m, mv[3];
  float A[3][3];  // A[r][c]
  bool force;
};

__device__ __forceinline__ P2GParticle p2g_particle(const SceneDev& S, int p, float4 xm, bool mass_only) {
  P2GParticle q;
  q.m = xm.w;
  q.force = false;
  if (mass_only) return q;
  const float4 vv = S.vv[p];
  q.mv[0] = q.m * vv.x;
  q.mv[1] = q.m * vv.y;
  q.mv[2] = q.m * vv.z;
  const float vol = vv.w;
  if (vol > 0.0f) {
    M3 F;
    float jp;
    load_fe(S, p, F, jp);
    M3 W, Sg, V;
    svd3<false>(F, W, Sg, V);
    const M3 R = m3_mul_bt(W, V);
    const float je = m3_det(F);
    const float e = expf(S.hardening * (1.0f - jp));
    const float mu = S.young / (2.0f * (1.0f + S.poisson)) * e;
    const float lam = S.young * S.poisson / ((1.0f + S.poisson) * (1.0f - 2.0f * S.poisson)) * e;
    M3 D;
#pragma unroll
    for (int c = 0; c < 3; c++)
#pragma unroll
      for (int r = 0; r < 3; r++) D.m[c][r] = F.m[c][r] - R.m[c][r];
    const M3 P = m3_mul_bt(D, F);  // (FE - R) FE^T
    const float s2 = lam * (je - 1.0f) * je;
#pragma unroll
    for (int r = 0; r < 3; r++)
#pragma unroll
      for (int c = 0; c < 3; c++) q.A[r][c] = -vol * (2.0f * mu * P.m[c][r] + (r == c ? s2 : 0.0f));
    q.force = true;
  }
  return q;
}

// Scatter of one particle's 64 stencil nodes. ACC(field, ax, by, cz, value)
// receives node (a, b, c) of the stencil. The (b, c) rows are visited in a
// lane-rotated order so lanes holding particles of the same cell hit
// different nodes in the same instruction.
template <bool MASS_ONLY, class Acc>
__device__ __forceinline__ void scatter_particle(const P2GParticle& q, const float wx[4], const float gx[4],
                                                 const float wy[4], const float gy[4], const float wz[4],
                                                 const float gz[4], int lane, Acc acc) {
  const int rb = (lane >> 2) & 3, rc = lane & 3;
#pragma unroll
  for (int cc = 0; cc < 4; cc++) {
    const int c = (cc + rc) & 3;
    const float wzc = sel4(c, wz[0], wz[1], wz[2], wz[3]);
    const float gzc = sel4(c, gz[0], gz[1], gz[2], gz[3]);
#pragma unroll
    for (int bb = 0; bb < 4; bb++) {
      const int b = (bb + rb) & 3;
      const float wyb = sel4(b, wy[0], wy[1], wy[2], wy[3]);
      const float gyb = sel4(b, gy[0], gy[1], gy[2], gy[3]);
      const float t1 = wyb * wzc;  // wy wz
      const float mw = q.m * t1;
      if (MASS_ONLY) {
#pragma unroll
        for (int a = 0; a < 4; a++) acc(0, a, b, c, wx[a] * mw);
        continue;
      }
      const float t2 = gyb * wzc;  // gy wz
      const float t3 = wyb * gzc;  // wy gz
      float pv[3], kk[3], hh[3];
#pragma unroll
      for (int r = 0; r < 3; r++) {
        pv[r] = q.mv[r] * t1;
        kk[r] = q.A[r][0] * t1;
        hh[r] = q.A[r][1] * t2 + q.A[r][2] * t3;
      }
      if (!q.force) {
#pragma unroll
        for (int r = 0; r < 3; r++) kk[r] = hh[r] = 0.0f;
      }
#pragma unroll
      for (int a = 0; a < 4; a++) {
        acc(0, a, b, c, wx[a] * mw);
#pragma unroll
        for (int r = 0; r < 3; r++) acc(1 + r, a, b, c, wx[a] * pv[r]);
#pragma unroll
        for (int r = 0; r < 3; r++) acc(4 + r, a, b, c, gx[a] * kk[r] + wx[a] * hh[r]);
      }
    }
  }
}

// P2G work item: up to kItemMax particles binned to one home block b. The
// tile covers nodes [4b-2, 4b+6] per axis, so a particle whose base cell
// lies in [4b-1, 4b+4] (its home block plus one cell of drift each way)
// scatters into it; such a base cell has tile-local coordinates
// lc = base - (4b-2) - 1 in [0, 5]^3 (216 cells).
constexpr int kItemMax = 256;
constexpr int kCellsPerAxis = kTile - 3;  // 6
constexpr int kCells = kCellsPerAxis * kCellsPerAxis * kCellsPerAxis;
constexpr int kPd = 10;  // float4 per particle in shared memory

struct P2GShared {
  float tile[kAccFields * kTile3];
  // per particle: [m, mv] [A00 A01 A02 A10] [A11 A12 A20 A21] [A22 - - -]
  //               [wx0..3] [gx0..3] [wy0..3] [gy0..3] [wz0..3] [gz0..3]
  float4 pd[kItemMax][kPd];
  short plist[kItemMax];
  short cells[kCells];
  int cstart[kCells + 1];
  int ccount[kCells];
  int slots[27];
  int ncells;
};

// P2G (p2gTransfer.glsl:44-151, or gMassCompute.glsl:33-84 when MASS_ONLY),
// cell-centric: each particle's stress and axis weights are computed once
// and parked in shared memory; the CTA buckets its particles by current
// cell; then each half-warp owns one cell's 4x4x4 stencil (lane = one x-row
// of 4 nodes, (b, c) = (lane & 3, lane >> 2)), sums the cell's particles in
// registers and adds the row to the shared tile. The tile's non-empty nodes
// are then added to the block pool with global atomics.
template <bool MASS_ONLY>
__global__ void __launch_bounds__(256) k_p2g(const SceneDev* __restrict__ scenes, const int* __restrict__ item_prefix,
                                             int nscenes) {
  extern __shared__ float4 smem_raw[];
  P2GShared& sh = *reinterpret_cast<P2GShared*>(smem_raw);
  constexpr int nf = MASS_ONLY ? 1 : kAccFields;
  const int total = item_prefix[nscenes];
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  for (int u = blockIdx.x; u < total; u += gridDim.x) {
    const int s = find_scene(item_prefix, nscenes, u);
    const SceneDev& S = scenes[s];
    const int4 it = S.items[u - item_prefix[s]];
    const int blk = it.x, start = it.y, cnt = min(it.z, kItemMax);
    const int bx = blk % S.bdim[0], by = (blk / S.bdim[0]) % S.bdim[1], bz = blk / (S.bdim[0] * S.bdim[1]);
    const int ox = 4 * bx - 2, oy = 4 * by - 2, oz = 4 * bz - 2;
    for (int i = threadIdx.x; i < nf * kTile3; i += blockDim.x) sh.tile[i] = 0.0f;
    for (int i = threadIdx.x; i < kCells; i += blockDim.x) sh.ccount[i] = 0;
    if (threadIdx.x < 27) {
      const int k = threadIdx.x;
      const int cx = bx - 1 + k % 3, cy = by - 1 + (k / 3) % 3, cz = bz - 1 + k / 9;
      sh.slots[k] = (cx >= 0 && cy >= 0 && cz >= 0 && cx < S.bdim[0] && cy < S.bdim[1] && cz < S.bdim[2])
                        ? S.blk_slot[block_id(S, cx, cy, cz)]
                        : -1;
    }
    __syncthreads();
    // ---- phase 1: one thread per particle -------------------------------
    int my_cell = -1, my_rank = 0;
    const int i = threadIdx.x;
    if (i < cnt) {
      const int p = start + i;
      const float4 xm = S.xm[p];
      if (MASS_ONLY || fabsf(xm.w) <= 100.0f) {  // p2gTransfer.glsl:64-66
        const float pg[3] = {(xm.x - S.gpos[0]) / S.h, (xm.y - S.gpos[1]) / S.h, (xm.z - S.gpos[2]) / S.h};
        const int base[3] = {(int)pg[0], (int)pg[1], (int)pg[2]};
        float wx[4], gx[4], wy[4], gy[4], wz[4], gz[4];
        axis_weights(pg[0], base[0], wx, gx);
        axis_weights(pg[1], base[1], wy, gy);
        axis_weights(pg[2], base[2], wz, gz);
        const P2GParticle q = p2g_particle(S, p, xm, MASS_ONLY);
        const int lx = base[0] - 1 - ox, ly = base[1] - 1 - oy, lz = base[2] - 1 - oz;
        if (lx >= 0 && ly >= 0 && lz >= 0 && lx < kCellsPerAxis && ly < kCellsPerAxis && lz < kCellsPerAxis) {
          my_cell = lx + kCellsPerAxis * ly + kCellsPerAxis * kCellsPerAxis * lz;
          my_rank = atomicAdd(&sh.ccount[my_cell], 1);
          float4* d = sh.pd[i];
          if (MASS_ONLY) {
            d[0] = make_float4(q.m, 0.0f, 0.0f, 0.0f);
          } else {
            const bool f = q.force;
            d[0] = make_float4(q.m, q.mv[0], q.mv[1], q.mv[2]);
            d[1] = f ? make_float4(q.A[0][0], q.A[0][1], q.A[0][2], q.A[1][0]) : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            d[2] = f ? make_float4(q.A[1][1], q.A[1][2], q.A[2][0], q.A[2][1]) : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            d[3] = make_float4(f ? q.A[2][2] : 0.0f, 0.0f, 0.0f, 0.0f);
          }
          d[4] = make_float4(wx[0], wx[1], wx[2], wx[3]);
          d[5] = make_float4(gx[0], gx[1], gx[2], gx[3]);
          d[6] = make_float4(wy[0], wy[1], wy[2], wy[3]);
          d[7] = make_float4(gy[0], gy[1], gy[2], gy[3]);
          d[8] = make_float4(wz[0], wz[1], wz[2], wz[3]);
          d[9] = make_float4(gz[0], gz[1], gz[2], gz[3]);
        } else {
          // The particle drifted out of its home block's tile since the last
          // binning: scatter it straight into the pool.
          atomicAdd(&S.counters[CNT_FALLBACK], 1);
          scatter_particle<MASS_ONLY>(q, wx, gx, wy, gy, wz, gz, lane, [&](int fld, int a, int b, int c, float v) {
            const int g0 = base[0] - 1 + a, g1 = base[1] - 1 + b, g2 = base[2] - 1 + c;
            if (g0 < 0 || g1 < 0 || g2 < 0 || g0 >= S.dim[0] || g1 >= S.dim[1] || g2 >= S.dim[2]) return;
            const int sl = S.blk_slot[block_id(S, g0 >> 2, g1 >> 2, g2 >> 2)];
            if (sl < 0) return;
            atomicAdd(&S.acc[(size_t)sl * kAccBlockFloats + fld * kBlockNodes + (g0 & 3) + 4 * (g1 & 3) + 16 * (g2 & 3)],
                      v);
          });
        }
      }
    }
    __syncthreads();
    // ---- bucket offsets and the list of occupied cells (warp 0) -----------
    if (warp == 0) {
      constexpr int per = (kCells + 31) / 32;  // 7 cells per lane
      int cntv[per];
      int sum = 0, occ = 0;
#pragma unroll
      for (int j = 0; j < per; j++) {
        const int ci = lane * per + j;
        cntv[j] = ci < kCells ? sh.ccount[ci] : 0;
        sum += cntv[j];
        occ += cntv[j] > 0;
      }
      int isum = sum, iocc = occ;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int a = __shfl_up_sync(0xffffffffu, isum, o);
        const int b = __shfl_up_sync(0xffffffffu, iocc, o);
        if (lane >= o) {
          isum += a;
          iocc += b;
        }
      }
      int run = isum - sum, rocc = iocc - occ;
#pragma unroll
      for (int j = 0; j < per; j++) {
        const int ci = lane * per + j;
        if (ci < kCells) {
          sh.cstart[ci] = run;
          if (cntv[j] > 0) sh.cells[rocc++] = (short)ci;
          run += cntv[j];
        }
      }
      if (lane == 31) {
        sh.cstart[kCells] = isum;
        sh.ncells = iocc;
      }
    }
    __syncthreads();
    if (my_cell >= 0) sh.plist[sh.cstart[my_cell] + my_rank] = (short)i;
    __syncthreads();
    // ---- phase 2: one half-warp per occupied cell ---------------------------
    {
      const int hw = threadIdx.x >> 4, l16 = threadIdx.x & 15;
      const int b = l16 & 3, c = l16 >> 2;
      const int nhw = blockDim.x >> 4;
      for (int k = hw; k < sh.ncells; k += nhw) {
        const int ci = sh.cells[k];
        const int j0 = sh.cstart[ci], j1 = sh.cstart[ci + 1];
        float acc[4][kAccFields];
#pragma unroll
        for (int a = 0; a < 4; a++)
#pragma unroll
          for (int f = 0; f < kAccFields; f++) acc[a][f] = 0.0f;
        for (int j = j0; j < j1; j++) {
          const float4* d = sh.pd[sh.plist[j]];
          const float* df = reinterpret_cast<const float*>(d);
          const float4 w4 = d[4];
          const float wxa[4] = {w4.x, w4.y, w4.z, w4.w};
          const float wyb = df[6 * 4 + b], wzc = df[8 * 4 + c];
          const float t1 = wyb * wzc;
          const float4 d0 = d[0];
          const float mw = d0.x * t1;
          if (MASS_ONLY) {
#pragma unroll
            for (int a = 0; a < 4; a++) acc[a][0] += wxa[a] * mw;
            continue;
          }
          const float4 g4 = d[5];
          const float gxa[4] = {g4.x, g4.y, g4.z, g4.w};
          const float gyb = df[7 * 4 + b], gzc = df[9 * 4 + c];
          const float t2 = gyb * wzc, t3 = wyb * gzc;
          const float4 a1 = d[1], a2 = d[2], a3 = d[3];
          // A rows: r0 = (a1.x a1.y a1.z), r1 = (a1.w a2.x a2.y), r2 = (a2.z a2.w a3.x)
          const float pv[3] = {d0.y * t1, d0.z * t1, d0.w * t1};
          const float kk[3] = {a1.x * t1, a1.w * t1, a2.z * t1};
          const float hh[3] = {a1.y * t2 + a1.z * t3, a2.x * t2 + a2.y * t3, a2.w * t2 + a3.x * t3};
#pragma unroll
          for (int a = 0; a < 4; a++) {
            acc[a][0] += wxa[a] * mw;
#pragma unroll
            for (int r = 0; r < 3; r++) {
              acc[a][1 + r] += wxa[a] * pv[r];
              acc[a][4 + r] += gxa[a] * kk[r] + wxa[a] * hh[r];
            }
          }
        }
        const int lx = ci % kCellsPerAxis, ly = (ci / kCellsPerAxis) % kCellsPerAxis,
                  lz = ci / (kCellsPerAxis * kCellsPerAxis);
        const int t0 = lx + kTile * (ly + b) + kTile * kTile * (lz + c);
#pragma unroll
        for (int a = 0; a < 4; a++)
#pragma unroll
          for (int f = 0; f < nf; f++) atomicAdd(&sh.tile[f * kTile3 + t0 + a], acc[a][f]);
      }
    }
    __syncthreads();
    // ---- flush the tile's non-empty nodes to the pool -----------------------
    for (int t = threadIdx.x; t < kTile3; t += blockDim.x) {
      const float m = sh.tile[t];
      if (m == 0.0f) continue;
      const int tx = t % kTile, ty = (t / kTile) % kTile, tz = t / (kTile * kTile);
      const int g0 = ox + tx, g1 = oy + ty, g2 = oz + tz;
      if (g0 < 0 || g1 < 0 || g2 < 0 || g0 >= S.dim[0] || g1 >= S.dim[1] || g2 >= S.dim[2]) continue;
      const int k = ((g0 >> 2) - bx + 1) + 3 * ((g1 >> 2) - by + 1) + 9 * ((g2 >> 2) - bz + 1);
      const int sl = sh.slots[k];
      if (sl < 0) continue;
      float* dst = S.acc + (size_t)sl * kAccBlockFloats + (g0 & 3) + 4 * (g1 & 3) + 16 * (g2 & 3);
#pragma unroll
      for (int f = 0; f < nf; f++) atomicAdd(dst + f * kBlockNodes, sh.tile[f * kTile3 + t]);
    }
    __syncthreads();
  }
}

// gForceCompute.glsl:57-103 on the active blocks. One 64-thread group per
// block; the P2G sums are consumed (zeroed) here, so the pool is all zero
// again before the next P2G.
__global__ void __launch_bounds__(256) k_grid(const SceneDev* __restrict__ scenes, const int* __restrict__ active_prefix,
                                              int nscenes, int clear_only) {
  const int groups = blockDim.x / kBlockNodes;
  const int node = threadIdx.x % kBlockNodes;
  const long long total = active_prefix[nscenes];
  for (long long u = (long long)blockIdx.x * groups + threadIdx.x / kBlockNodes; u < total;
       u += (long long)gridDim.x * groups) {
    const int s = find_scene(active_prefix, nscenes, u);
    const SceneDev& S = scenes[s];
    const int slot = (int)(u - active_prefix[s]);
    float* acc = S.acc + (size_t)slot * kAccBlockFloats + node;
    float v[kAccFields];
#pragma unroll
    for (int f = 0; f < kAccFields; f++) {
      v[f] = acc[f * kBlockNodes];
      acc[f * kBlockNodes] = 0.0f;
    }
    if (clear_only) continue;
    float* out = S.gout + (size_t)slot * kOutBlockFloats + node;
    const float mi = v[0];
    float vs[3] = {0.0f, 0.0f, 0.0f}, d[3] = {0.0f, 0.0f, 0.0f};
    if (mi > 0.0f) {
      const float inv = 1.0f / mi;
      const float vold[3] = {v[1] * inv, v[2] * inv, v[3] * inv};
#pragma unroll
      for (int k = 0; k < 3; k++) vs[k] = vold[k] + S.dt * (v[4 + k] * inv + S.grav[k]);
      const int b = S.active[slot];
      const int bx = b % S.bdim[0], by = (b / S.bdim[0]) % S.bdim[1], bz = b / (S.bdim[0] * S.bdim[1]);
      const int gi = 4 * bx + (node & 3), gj = 4 * by + ((node >> 2) & 3), gk = 4 * bz + (node >> 4);
      // node position as Grid::initSSBO forms it: x_off + h * (float)i
      const float xi[3] = {__fadd_rn(S.gpos[0], __fmul_rn(S.h, (float)gi)),
                           __fadd_rn(S.gpos[1], __fmul_rn(S.h, (float)gj)),
                           __fadd_rn(S.gpos[2], __fmul_rn(S.h, (float)gk))};
      collide(S, xi, vs);
#pragma unroll
      for (int k = 0; k < 3; k++) d[k] = vs[k] - S.alpha * vold[k];
    }
#pragma unroll
    for (int k = 0; k < 3; k++) {
      out[k * kBlockNodes] = vs[k];
      out[(3 + k) * kBlockNodes] = d[k];
    }
  }
}

// pVolumeCompute.glsl:32-83 on the pool: rho0 = sum_i m_i w_ip / h^3,
// stored as V0 = m / rho0 (0 when rho0 <= 0, which disables the force as
// p2gTransfer.glsl:126 does).
__global__ void __launch_bounds__(256) k_volume(const SceneDev* __restrict__ scenes, const int* __restrict__ chunk_prefix,
                                                int nscenes, long long total_chunks) {
  for (long long u = blockIdx.x; u < total_chunks; u += gridDim.x) {
    const int s = find_scene(chunk_prefix, nscenes, u);
    const SceneDev& S = scenes[s];
    const int p = (int)(u - chunk_prefix[s]) * blockDim.x + threadIdx.x;
    if (p >= S.n) continue;
    const float4 xm = S.xm[p];
    const float pg[3] = {(xm.x - S.gpos[0]) / S.h, (xm.y - S.gpos[1]) / S.h, (xm.z - S.gpos[2]) / S.h};
    const int base[3] = {(int)pg[0], (int)pg[1], (int)pg[2]};
    float wx[4], gx[4], wy[4], gy[4], wz[4], gz[4];
    axis_weights(pg[0], base[0], wx, gx);
    axis_weights(pg[1], base[1], wy, gy);
    axis_weights(pg[2], base[2], wz, gz);
    float rho = 0.0f;
    for (int c = 0; c < 4; c++)
      for (int b = 0; b < 4; b++)
        for (int a = 0; a < 4; a++) {
          const int g0 = base[0] - 1 + a, g1 = base[1] - 1 + b, g2 = base[2] - 1 + c;
          if (g0 < 0 || g1 < 0 || g2 < 0 || g0 >= S.dim[0] || g1 >= S.dim[1] || g2 >= S.dim[2]) continue;
          const int sl = S.blk_slot[block_id(S, g0 >> 2, g1 >> 2, g2 >> 2)];
          if (sl < 0) continue;
          const float mi = S.acc[(size_t)sl * kAccBlockFloats + (g0 & 3) + 4 * (g1 & 3) + 16 * (g2 & 3)];
          rho += mi * (wx[a] * wy[b] * wz[c]);
        }
    rho = rho / (S.h * S.h * S.h);
    float4 vv = S.vv[p];
    vv.w = rho > 0.0f ? xm.w / rho : 0.0f;
    S.vv[p] = vv;
  }
}

// g2pTransfer.glsl:53-143 fused with particleAdvance.glsl:75-217.
__global__ void __launch_bounds__(128) k_g2p_advance(const SceneDev* __restrict__ scenes,
                                                     const int* __restrict__ chunk_prefix, int nscenes,
                                                     long long total_chunks) {
  for (long long u = blockIdx.x; u < total_chunks; u += gridDim.x) {
    const int s = find_scene(chunk_prefix, nscenes, u);
    const SceneDev& S = scenes[s];
    const int p = (int)(u - chunk_prefix[s]) * blockDim.x + threadIdx.x;
    if (p >= S.n) continue;
    float4 xm = S.xm[p];
    float4 vv = S.vv[p];
    const float pg[3] = {(xm.x - S.gpos[0]) / S.h, (xm.y - S.gpos[1]) / S.h, (xm.z - S.gpos[2]) / S.h};
    const int base[3] = {(int)pg[0], (int)pg[1], (int)pg[2]};
    float wx[4], gx[4], wy[4], gy[4], wz[4], gz[4];
    axis_weights(pg[0], base[0], wx, gx);
    axis_weights(pg[1], base[1], wy, gy);
    axis_weights(pg[2], base[2], wz, gz);
    // slots of the (up to) 2 x 2 x 2 blocks under the stencil
    const int b0[3] = {(base[0] - 1) >> 2, (base[1] - 1) >> 2, (base[2] - 1) >> 2};
    int sl[2][2][2];
#pragma unroll
    for (int k = 0; k < 2; k++)
#pragma unroll
      for (int j = 0; j < 2; j++)
#pragma unroll
        for (int i = 0; i < 2; i++) {
          const int cx = b0[0] + i, cy = b0[1] + j, cz = b0[2] + k;
          sl[k][j][i] = (cx >= 0 && cy >= 0 && cz >= 0 && cx < S.bdim[0] && cy < S.bdim[1] && cz < S.bdim[2])
                            ? __ldg(&S.blk_slot[block_id(S, cx, cy, cz)])
                            : -1;
        }
    int xsel[4], lx[4];
    bool xin[4];
#pragma unroll
    for (int a = 0; a < 4; a++) {
      const int g = base[0] - 1 + a;
      xin[a] = g >= 0 && g < S.dim[0];
      xsel[a] = (g >> 2) != b0[0];
      lx[a] = g & 3;
    }
    float dv[3] = {0.0f, 0.0f, 0.0f};
    float L[3][3] = {{0.0f, 0.0f, 0.0f}, {0.0f, 0.0f, 0.0f}, {0.0f, 0.0f, 0.0f}};  // L[r][c]
#pragma unroll
    for (int c = 0; c < 4; c++) {
      const int gk = base[2] - 1 + c;
      if (gk < 0 || gk >= S.dim[2]) continue;
      const int zs = (gk >> 2) != b0[2];
#pragma unroll
      for (int b = 0; b < 4; b++) {
        const int gj = base[1] - 1 + b;
        if (gj < 0 || gj >= S.dim[1]) continue;
        const int ys = (gj >> 2) != b0[1];
        const int s0 = zs ? (ys ? sl[1][1][0] : sl[1][0][0]) : (ys ? sl[0][1][0] : sl[0][0][0]);
        const int s1 = zs ? (ys ? sl[1][1][1] : sl[1][0][1]) : (ys ? sl[0][1][1] : sl[0][0][1]);
        const int lyz = 4 * (gj & 3) + 16 * (gk & 3);
        float S1[3] = {0.0f, 0.0f, 0.0f}, S2[3] = {0.0f, 0.0f, 0.0f}, D[3] = {0.0f, 0.0f, 0.0f};
#pragma unroll
        for (int a = 0; a < 4; a++) {
          const int slot = xsel[a] ? s1 : s0;
          if (!xin[a] || slot < 0) continue;
          const float* o = S.gout + (size_t)slot * kOutBlockFloats + lyz + lx[a];
#pragma unroll
          for (int r = 0; r < 3; r++) {
            const float vs = __ldg(o + r * kBlockNodes);
            const float dd = __ldg(o + (3 + r) * kBlockNodes);
            S1[r] += wx[a] * vs;
            S2[r] += gx[a] * vs;
            D[r] += wx[a] * dd;
          }
        }
        const float t1 = wy[b] * wz[c], t2 = gy[b] * wz[c], t3 = wy[b] * gz[c];
#pragma unroll
        for (int r = 0; r < 3; r++) {
          dv[r] += t1 * D[r];
          L[r][0] += t1 * S2[r];
          L[r][1] += t2 * S1[r];
          L[r][2] += t3 * S1[r];
        }
      }
    }
    // ---- particle update (particleAdvance.glsl:87-210) ----
    M3 FE;
    float jp;
    load_fe(S, p, FE, jp);
    M3 step;
#pragma unroll
    for (int c = 0; c < 3; c++)
#pragma unroll
      for (int r = 0; r < 3; r++) step.m[c][r] = (c == r ? 1.0f : 0.0f) + S.dt * L[r][c];
    const M3 fe_trial = m3_mul(step, FE);
    M3 W, Sg, V;
    svd3<false>(fe_trial, W, Sg, V);
    float ratio = 1.0f;
#pragma unroll
    for (int i = 0; i < 3; i++) {
      const float sv = Sg.m[i][i];
      const float cl = fminf(fmaxf(sv, S.crit_lo), S.crit_hi);
      ratio *= sv / cl;
      Sg.m[i][i] = cl;
    }
    const M3 fe_new = m3_mul_bt(m3_mul(W, Sg), V);
    // det F_P' = det F_P * det(FE_trial) / det(FE'): the shader's
    // F_P' = V S^-1 W^T (I + dt L) FE FP (particleAdvance.glsl:132) has this
    // determinant; only det F_P is ever read (p2gTransfer.glsl:119).
    jp *= ratio;
    float v[3] = {S.alpha * vv.x + dv[0], S.alpha * vv.y + dv[1], S.alpha * vv.z + dv[2]};
    const float xold[3] = {xm.x, xm.y, xm.z};
    collide(S, xold, v);
    xm.x += S.dt * v[0];
    xm.y += S.dt * v[1];
    xm.z += S.dt * v[2];
    vv.x = v[0];
    vv.y = v[1];
    vv.z = v[2];
    S.xm[p] = xm;
    S.vv[p] = vv;
    store_fe(S, p, fe_new, jp);
    bool finite = isfinite(xm.x) && isfinite(xm.y) && isfinite(xm.z) && isfinite(v[0]) && isfinite(v[1]) &&
                  isfinite(v[2]) && isfinite(jp);
#pragma unroll
    for (int c = 0; c < 3; c++)
#pragma unroll
      for (int r = 0; r < 3; r++) finite = finite && isfinite(fe_new.m[c][r]);
    if (!finite) atomicAdd(&S.counters[CNT_NONFINITE], 1);
    const float pgn[3] = {(xm.x - S.gpos[0]) / S.h, (xm.y - S.gpos[1]) / S.h, (xm.z - S.gpos[2]) / S.h};
    mark_stencil(S, pgn);
  }
}

__global__ void k_begin_step(const SceneDev* __restrict__ scenes, int nscenes) {
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < nscenes; s += gridDim.x * blockDim.x) {
    scenes[s].counters[CNT_ACTIVE] = 0;
    scenes[s].counters[CNT_OVERFLOW] = 0;
  }
}

__global__ void k_count_flags(const SceneDev* __restrict__ sd, int nblocks) {
  int c = 0;
  for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < nblocks; b += gridDim.x * blockDim.x)
    c += sd->blk_flag[b] != 0;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(0xffffffffu, c, o);
  if ((threadIdx.x & 31) == 0 && c) atomicAdd(&sd->counters[CNT_ACTIVE], c);
}

__global__ void k_rigid(const SceneDev* __restrict__ scenes, int nscenes) {  // rigidAdvance.glsl:14-18
  const int s = blockIdx.x;
  if (s >= nscenes) return;
  const SceneDev& S = scenes[s];
  for (int i = threadIdx.x; i < S.ncoll; i += blockDim.x)
    for (int k = 0; k < 3; k++) S.coll[i].pos[k] = S.coll[i].pos[k] + S.dt * S.coll[i].vel[k];
}

// Monotone map float -> int: a < b  <=>  key(a) < key(b) (finite values).
__device__ __forceinline__ int float_order_key(float f) {
  const int i = __float_as_int(f);
  return i >= 0 ? i : i ^ 0x7fffffff;
}

// Bulk statistics (double accumulation).
__global__ void __launch_bounds__(256) k_stats(const SceneDev* __restrict__ sd, int n, StatsAccum* out) {
  const SceneDev& S = *sd;
  double acc[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
  float bmin[3] = {3.4e38f, 3.4e38f, 3.4e38f}, bmax[3] = {-3.4e38f, -3.4e38f, -3.4e38f};
  unsigned long long bad = 0;
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
    const float4 xm = S.xm[p];
    const float4 vv = S.vv[p];
    const float jp = S.fc[p].y;
    const double m = xm.w;
    const bool ok = isfinite(xm.x) && isfinite(xm.y) && isfinite(xm.z) && isfinite(vv.x) && isfinite(vv.y) &&
                    isfinite(vv.z) && isfinite(jp);
    if (!ok) {
      bad++;
      continue;
    }
    acc[0] += m;
    acc[1] += m * vv.x;
    acc[2] += m * vv.y;
    acc[3] += m * vv.z;
    acc[4] += 0.5 * m * ((double)vv.x * vv.x + (double)vv.y * vv.y + (double)vv.z * vv.z);
    acc[5] += m * xm.x;
    acc[6] += m * xm.y;
    acc[7] += m * xm.z;
    acc[8] += jp;
    bmin[0] = fminf(bmin[0], xm.x); bmin[1] = fminf(bmin[1], xm.y); bmin[2] = fminf(bmin[2], xm.z);
    bmax[0] = fmaxf(bmax[0], xm.x); bmax[1] = fmaxf(bmax[1], xm.y); bmax[2] = fmaxf(bmax[2], xm.z);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
    for (int k = 0; k < 9; k++) acc[k] += __shfl_down_sync(0xffffffffu, acc[k], o);
#pragma unroll
    for (int k = 0; k < 3; k++) {
      bmin[k] = fminf(bmin[k], __shfl_down_sync(0xffffffffu, bmin[k], o));
      bmax[k] = fmaxf(bmax[k], __shfl_down_sync(0xffffffffu, bmax[k], o));
    }
    bad += __shfl_down_sync(0xffffffffu, bad, o);
  }
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(&out->mass, acc[0]);
    atomicAdd(&out->mom[0], acc[1]);
    atomicAdd(&out->mom[1], acc[2]);
    atomicAdd(&out->mom[2], acc[3]);
    atomicAdd(&out->ke, acc[4]);
    atomicAdd(&out->com[0], acc[5]);
    atomicAdd(&out->com[1], acc[6]);
    atomicAdd(&out->com[2], acc[7]);
    atomicAdd(&out->jp, acc[8]);
    atomicAdd(&out->nonfinite, bad);
    // min / max of floats through an order-preserving int key
    for (int k = 0; k < 3; k++) {
      atomicMin(&out->bmin_key[k], float_order_key(bmin[k]));
      atomicMax(&out->bmax_key[k], float_order_key(bmax[k]));
    }
  }
}

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
    const float* acc = S.acc + (size_t)slot * kAccBlockFloats + node;
    const float* out = S.gout + (size_t)slot * kOutBlockFloats + node;
    if (mass) mass[g] = acc[0];
    for (int k = 0; k < 3; k++) {
      if (mom) mom[3 * g + k] = acc[(1 + k) * kBlockNodes];
      if (force) force[3 * g + k] = acc[(4 + k) * kBlockNodes];
      if (vstar) vstar[3 * g + k] = out[k * kBlockNodes];
    }
  }
}

}  // namespace

int num_sms() {
  static int n = 0;
  if (n == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    if (n <= 0) n = 1;
  }
  return n;
}

void fast_prefix(const SceneDev* scenes, int nscenes, int counter, int* prefix, cudaStream_t st) {
  k_prefix<<<1, 32, 0, st>>>(scenes, nscenes, counter, prefix);
}

void fast_compact(const SceneDev* scenes, const int* block_prefix, int nscenes, long long total_blocks,
                  cudaStream_t st) {
  if (total_blocks <= 0) return;
  long long g = (total_blocks + 255) / 256;
  g = g > (long long)num_sms() * 16 ? (long long)num_sms() * 16 : g;
  k_compact<<<(int)g, 256, 0, st>>>(scenes, block_prefix, nscenes, total_blocks);
}

void fast_mark(const SceneDev* scenes, const int* chunk_prefix, int nscenes, long long total_chunks,
               cudaStream_t st) {
  if (total_chunks <= 0) return;
  const long long g = total_chunks > (long long)num_sms() * 16 ? (long long)num_sms() * 16 : total_chunks;
  k_mark<<<(int)g, 128, 0, st>>>(scenes, chunk_prefix, nscenes, total_chunks);
}

void fast_p2g(const SceneDev* scenes, const int* item_prefix, int nscenes, int grid_ctas, bool mass_only,
              int threads, cudaStream_t st) {
  static bool configured = false;
  const int smem = (int)sizeof(P2GShared);
  if (!configured) {
    cudaFuncSetAttribute(k_p2g<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    cudaFuncSetAttribute(k_p2g<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    configured = true;
  }
  (void)threads;  // the item layout needs exactly kItemMax threads
  if (mass_only)
    k_p2g<true><<<grid_ctas, kItemMax, smem, st>>>(scenes, item_prefix, nscenes);
  else
    k_p2g<false><<<grid_ctas, kItemMax, smem, st>>>(scenes, item_prefix, nscenes);
}

void fast_grid(const SceneDev* scenes, const int* active_prefix, int nscenes, int grid_ctas, bool clear_only,
               cudaStream_t st) {
  k_grid<<<grid_ctas, 256, 0, st>>>(scenes, active_prefix, nscenes, clear_only ? 1 : 0);
}

void fast_volume(const SceneDev* scenes, const int* chunk_prefix, int nscenes, long long total_chunks,
                 cudaStream_t st) {
  if (total_chunks <= 0) return;
  const long long g = total_chunks > (long long)num_sms() * 16 ? (long long)num_sms() * 16 : total_chunks;
  k_volume<<<(int)g, 128, 0, st>>>(scenes, chunk_prefix, nscenes, total_chunks);
}

void fast_g2p_advance(const SceneDev* scenes, const int* chunk_prefix, int nscenes, long long total_chunks,
                      int threads, cudaStream_t st) {
  if (total_chunks <= 0) return;
  const long long g = total_chunks > (long long)num_sms() * 32 ? (long long)num_sms() * 32 : total_chunks;
  k_g2p_advance<<<(int)g, threads, 0, st>>>(scenes, chunk_prefix, nscenes, total_chunks);
}

void fast_rigid(const SceneDev* scenes, int nscenes, const snow_collider*, cudaStream_t st) {
  if (nscenes > 0) k_rigid<<<nscenes, 32, 0, st>>>(scenes, nscenes);
}

void fast_begin_step(const SceneDev* scenes, int nscenes, cudaStream_t st) {
  if (nscenes > 0) k_begin_step<<<(nscenes + 127) / 128, 128, 0, st>>>(scenes, nscenes);
}

void fast_count_flags(const SceneDev* sd_dev, int nblocks, cudaStream_t st) {
  int g = (nblocks + 255) / 256;
  if (g > num_sms() * 8) g = num_sms() * 8;
  if (g < 1) g = 1;
  k_count_flags<<<g, 256, 0, st>>>(sd_dev, nblocks);
}

void fast_stats(const SceneDev* sd_dev, int n, StatsAccum* out_dev, cudaStream_t st) {
  if (n <= 0) return;
  int g = (n + 255) / 256;
  if (g > num_sms() * 8) g = num_sms() * 8;
  k_stats<<<g, 256, 0, st>>>(sd_dev, n, out_dev);
}

void fast_download_grid(const SceneDev* sd_dev, long long G, float* mass, float* mom, float* force, float* vstar,
                        cudaStream_t st) {
  (void)G;
  k_download_grid<<<num_sms() * 8, 256, 0, st>>>(sd_dev, mass, mom, force, vstar);
}

}  // namespace snow
