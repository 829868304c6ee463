// Semi-implicit velocity update of the FAST path for sm_103a.
//
// The reference declares SemiImplicitTimeUpdate but leaves it empty
// (src/snow/simulation/timeUpdate/semiimplicittimeupdate.cpp:3-5). This is
// the scheme of Stomakhin et al. 2013 (sec. 4, eq. 9): after the grid update
// has formed v* (colliders applied), solve
//     (M + beta dt^2 K) v = M v*,   K u = sum_p V0_p dP(F_p; G_p F_p) F_p^T grad w_ip,
//     G_p = sum_j u_j (grad w_jp)^T,
// apply the colliders to v, and hand v to G2P in place of v* (d = v - alpha
// p/m follows). The solve runs conjugate residuals on the mass-scaled form
//     (I + c M^-1/2 K M^-1/2) y = M^1/2 v*,   v = M^-1/2 y,   c = beta dt^2,
// from y = M^1/2 v*: the scaling by the lumped masses keeps the nodes at the
// material's edge, whose masses are tiny, from stalling the iteration, and
// the residual is measured in the kinetic-energy norm |M^1/2 v*|. P is the first
// Piola-Kirchhoff stress of the shaders' fixed-corotated energy
// (p2gTransfer.glsl:109-141 forms P F^T), with F = F_E, mu(J_p), lambda(J_p)
// held at the step's start; the weight gradients are the explicit force's
// (grid units), so K is the derivative of the force the explicit step
// applies.
//
// Layout in HBM, per active pool slot (the grid update's slots):
//   crv  three float4 planes of pool_cap x 64 nodes: (v, m), (p, 0), (A p, 0)
//        with p and A p in the scaled variables
//   cru  pool_cap x 192 floats: u = M^-1/2 r, the vector K is applied to,
//        3 floats per node, so that a work item bulk-copies (TMA) its 27
//        blocks like the G2P gather does
//   acc  the dense P2G sums, zero between steps: K u accumulates in its
//        force slots and is cleared by the pass that consumes it
//   crs  per scene: |M^1/2 v*|^2 and per iteration (r, A r), |A p|^2, |r|^2 in FP64
// Kernels of one iteration k: K u over the work items (k_hess), then three
// passes over the active nodes: (r, A r); the directions p, A p and |A p|^2;
// v, r and |r|^2; then k_cr_cond advances k (a device counter) and decides
// whether iteration k runs. Inside a captured step graph the iterations are
// the body of a conditional WHILE node that k_cr_cond sets, so the loop ends
// on the device as soon as every scene has converged; without a graph the
// host launches max_iters iterations and the finished ones return at once.
#include "fast_item.cuh"

namespace snow {
namespace {

// Iteration k (k >= 1) of scene S runs while iteration k - 1 left a residual
// above the tolerance; iteration 0 is the K v* pass of every implicit scene
// that does not skip this step's solve (CrScalars::skipping).
__device__ __forceinline__ bool cr_running(const SceneDev& S, int k) {
  if (!S.crs) return false;
  const CrScalars& c = *S.crs;
  if (c.skipping) return false;
  if (k == 0) return true;
  if (k > S.imp_maxit) return false;
  const double tol = (double)S.imp_tol;
  return c.rr[k - 1] > tol * tol * c.bb;
}

// Whether any scene of the launch runs iteration k (a launch of an iteration
// that every scene has finished returns at once).
__device__ __forceinline__ bool any_running(const SceneDev* __restrict__ scenes, int nscenes, int k) {
  for (int s = 0; s < nscenes; s++)
    if (cr_running(scenes[s], k)) return true;
  return false;
}

// G = sum_j u_j (grad w_j)^T over the particle's stencil, contracted along x
// first for each (y, z) row; node(a, b, c, u) fills u at stencil node
// (a, b, c) (zero for a node that contributes nothing).
template <class Node>
__device__ __forceinline__ void hess_sums(const AxisW& w, Node node, float Gm[3][3]) {
#pragma unroll
  for (int r = 0; r < 3; r++) Gm[r][0] = Gm[r][1] = Gm[r][2] = 0.0f;
#pragma unroll
  for (int c = 0; c < 4; c++) {
#pragma unroll
    for (int b = 0; b < 4; b++) {
      float S1[3] = {0.0f, 0.0f, 0.0f}, S2[3] = {0.0f, 0.0f, 0.0f};
#pragma unroll
      for (int a = 0; a < 4; a++) {
        float u[3];
        node(a, b, c, u);
#pragma unroll
        for (int r = 0; r < 3; r++) {
          S1[r] += w.wx[a] * u[r];
          S2[r] += w.gx[a] * u[r];
        }
      }
      const float t1 = w.wy[b] * w.wz[c], t2 = w.gy[b] * w.wz[c], t3 = w.wy[b] * w.gz[c];
#pragma unroll
      for (int r = 0; r < 3; r++) {
        Gm[r][0] += t1 * S2[r];
        Gm[r][1] += t2 * S1[r];
        Gm[r][2] += t3 * S1[r];
      }
    }
  }
}

// The gather of u (3 floats per node) from the staged tile when the stencil
// lies in it (decided once per particle), else from cru.
__device__ __forceinline__ void hess_gather(const ItemShared& sh, const SceneDev& S, int bx, int by, int bz,
                                            const int base[3], const AxisW& w, float Gm[3][3]) {
  const int tx = base[0] - 1 - (4 * bx - 2), ty = base[1] - 1 - (4 * by - 2), tz = base[2] - 1 - (4 * bz - 2);
  if (tx >= 0 && ty >= 0 && tz >= 0 && tx <= kTile - 4 && ty <= kTile - 4 && tz <= kTile - 4) {
    // tile node t (0..8) lies in tile block floor((t + 2) / 4) at local (t + 2) & 3
    int X[4], Y[4], Z[4];
#pragma unroll
    for (int a = 0; a < 4; a++) {
      const int t = tx + a, q = ty + a, r = tz + a;
      X[a] = ((t + 2) >> 2) * kOutBlockFloats + 3 * ((t + 2) & 3);
      Y[a] = ((q + 2) >> 2) * 3 * kOutBlockFloats + 3 * 4 * ((q + 2) & 3);
      Z[a] = ((r + 2) >> 2) * 9 * kOutBlockFloats + 3 * 16 * ((r + 2) & 3);
    }
    const float* st = &sh.stage[0][0];
    hess_sums(w,
              [&](int a, int b, int c, float u[3]) {
                const float* o = st + X[a] + Y[b] + Z[c];
                u[0] = o[0];
                u[1] = o[1];
                u[2] = o[2];
              },
              Gm);
  } else {
    hess_sums(w,
              [&](int a, int b, int c, float u[3]) {
                const int g0 = base[0] - 1 + a, g1 = base[1] - 1 + b, g2 = base[2] - 1 + c;
                u[0] = u[1] = u[2] = 0.0f;
                if (!node_in_grid(S, g0, g1, g2)) return;
                const int sl = __ldg(&S.blk_slot[block_id(S, g0 >> 2, g1 >> 2, g2 >> 2)]);
                if (sl < 0) return;
                const float* o = S.cru + (size_t)sl * kImpBlockFloats + 3 * ((g0 & 3) + 4 * (g1 & 3) + 16 * (g2 & 3));
                u[0] = __ldg(o);
                u[1] = __ldg(o + 1);
                u[2] = __ldg(o + 2);
              },
              Gm);
  }
}

__device__ __forceinline__ void cross3(const float a[3], const float b[3], float o[3]) {
  o[0] = a[1] * b[2] - a[2] * b[1];
  o[1] = a[2] * b[0] - a[0] * b[2];
  o[2] = a[0] * b[1] - a[1] * b[0];
}

// q.A = V0 dP(F; G F) F^T for particle p (false: the particle carries no
// stress force, p2gTransfer.glsl:126). dP = 2 mu (dF - dR) + lambda dJ C +
// lambda (J - 1) dC with C = J F^-T the cofactor matrix; with F^T F = V
// diag(s^2) V^T (warm-started Jacobi from the particle's stored frame),
// W = F V diag(1/s) and G' = W^T dF V, the rotation's differential is
// dR = W X V^T, X skew with X_ij = (G'_ij - G'_ji) / (s_i + s_j).
__device__ __forceinline__ bool hess_particle(const SceneDev& S, int p, bool binned, const float Gm[3][3],
                                              P2GParticle& q) {
  const float vol = (binned ? S.bvv : S.vv)[p].w;
  if (!(vol > 0.0f)) return false;
  M3 F;
  float jp;
  load_fe(S, p, F, jp, binned);
  const float4 f4 = (binned ? S.bvq : S.vq)[p];
  float qv[4] = {f4.x, f4.y, f4.z, f4.w};
  M3 V;
  float lam[3];
  eigen_warm(F, qv, V, lam);
  const M3 B = m3_mul(F, V);  // W diag(s)
  float sig[3];
  M3 W;
#pragma unroll
  for (int c = 0; c < 3; c++) {
    const float inv = rsqrt_nr(fmaxf(lam[c], 1e-30f));
    sig[c] = lam[c] * inv;
#pragma unroll
    for (int r = 0; r < 3; r++) W.m[c][r] = B.m[c][r] * inv;
  }
  M3 dF;  // G F
#pragma unroll
  for (int c = 0; c < 3; c++)
#pragma unroll
    for (int r = 0; r < 3; r++) dF.m[c][r] = Gm[r][0] * F.m[c][0] + Gm[r][1] * F.m[c][1] + Gm[r][2] * F.m[c][2];
  const M3 Gw = m3_mul_at(W, m3_mul(dF, V));  // W^T dF V; Gw.m[c][r] is row r, column c
  // singular values of a deformation gradient are O(1): the fast divide's
  // 2 ulp are far inside the solve's tolerance
  const float x01 = __fdividef(Gw.m[1][0] - Gw.m[0][1], sig[0] + sig[1]);
  const float x02 = __fdividef(Gw.m[2][0] - Gw.m[0][2], sig[0] + sig[2]);
  const float x12 = __fdividef(Gw.m[2][1] - Gw.m[1][2], sig[1] + sig[2]);
  M3 X;
  X.m[0][0] = 0.0f; X.m[1][0] = x01;  X.m[2][0] = x02;
  X.m[0][1] = -x01; X.m[1][1] = 0.0f; X.m[2][1] = x12;
  X.m[0][2] = -x02; X.m[1][2] = -x12; X.m[2][2] = 0.0f;
  const M3 dR = m3_mul_bt(m3_mul(W, X), V);
  // cofactor C (columns f1 x f2, f2 x f0, f0 x f1) and its differential
  M3 C, dC;
  cross3(F.m[1], F.m[2], C.m[0]);
  cross3(F.m[2], F.m[0], C.m[1]);
  cross3(F.m[0], F.m[1], C.m[2]);
  float dJ = 0.0f;
#pragma unroll
  for (int c = 0; c < 3; c++)
#pragma unroll
    for (int r = 0; r < 3; r++) dJ += C.m[c][r] * dF.m[c][r];
#pragma unroll
  for (int c = 0; c < 3; c++) {
    const int c1 = (c + 1) % 3, c2 = (c + 2) % 3;
    float t0[3], t1[3];
    cross3(dF.m[c1], F.m[c2], t0);
    cross3(F.m[c1], dF.m[c2], t1);
#pragma unroll
    for (int r = 0; r < 3; r++) dC.m[c][r] = t0[r] + t1[r];
  }
  const float J = m3_det(F);
  const float e = expf(S.hardening * (1.0f - jp));
  const float mu2 = 2.0f * S.mu0 * e, la = S.lambda0 * e;
  const float la_dj = la * dJ, la_j1 = la * (J - 1.0f);
  M3 dP;
#pragma unroll
  for (int c = 0; c < 3; c++)
#pragma unroll
    for (int r = 0; r < 3; r++)
      dP.m[c][r] = mu2 * (dF.m[c][r] - dR.m[c][r]) + la_dj * C.m[c][r] + la_j1 * dC.m[c][r];
  const M3 A = m3_mul_bt(dP, F);
#pragma unroll
  for (int r = 0; r < 3; r++)
#pragma unroll
    for (int c = 0; c < 3; c++) q.A[r][c] = vol * A.m[c][r];
  q.force = true;
  return true;
}

// The first item u' >= u of this CTA's round-robin share (u' = u mod the
// grid) whose scene runs iteration k (total when none is left); s gets its
// scene. The items of a finished scene are stepped over in one jump.
__device__ __forceinline__ int next_running(const SceneDev* __restrict__ scenes, const int* __restrict__ item_prefix,
                                            int nscenes, int k, int u, int total, int& s) {
  const int g = gridDim.x;
  while (u < total) {
    s = find_scene(item_prefix, nscenes, u);
    if (cr_running(scenes[s], k)) return u;
    u += (item_prefix[s + 1] - u + g - 1) / g * g;
  }
  s = 0;
  return total;
}

// K u for the items of every scene whose iteration k runs, into acc's force
// slots (iteration 0: u = v*). Persistent over the items like the fused
// explicit kernel: the bulk copies of the CTA's next item are issued by the
// last warp while the current item's per-cell sums are flushed.
__global__ void __launch_bounds__(kItemMax, 2) k_hess(const SceneDev* __restrict__ scenes,
                                                      const int* __restrict__ item_prefix, int nscenes,
                                                      const int* __restrict__ iter) {
  const int k = iter ? *iter : 0;  // iteration 0: K v*
  if (!any_running(scenes, nscenes, k)) return;
  extern __shared__ float4 smem_raw[];
  ItemShared& sh = *reinterpret_cast<ItemShared*>(smem_raw);
  tile_init(sh);
  const int total = item_prefix[nscenes];
  const int lane = threadIdx.x & 31;
  const bool lastw = (threadIdx.x >> 5) == (blockDim.x >> 5) - 1;
  int s = 0;
  int u = next_running(scenes, item_prefix, nscenes, k, blockIdx.x, total, s);
  if (u >= total) return;  // uniform across the CTA
  int4 it = scenes[s].items[u - item_prefix[s]];
  if (lastw) stage_issue(sh, scenes[s].cru, kImpBlockFloats, tile_slot(scenes[s], it, lane), scenes[s].tx_unsent);
  uint32_t phase = 0;
  while (u < total) {
    __syncthreads();  // zero-filled stage blocks are visible; the last flush is done
    tile_zero(sh, 3);
    const SceneDev& S = scenes[s];
    // the next item and (last warp) its pool slots, loaded ahead of use
    int sn = 0;
    const int un = next_running(scenes, item_prefix, nscenes, k, u + gridDim.x, total, sn);
    int4 itn = make_int4(0, 0, 0, 0);
    int slot = -1;
    if (un < total) {
      itn = scenes[sn].items[un - item_prefix[sn]];
      if (lastw) slot = tile_slot(scenes[sn], itn, lane);
    }
    int bx, by, bz;
    home_coords(S, it.x, bx, by, bz);
    const int i = threadIdx.x;
    const bool mine = i < min(it.z, kItemMax);
    float4 xm = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    const bool binned = particles_binned(S);  // the solve runs before the step's fused kernel
    if (mine) xm = (binned ? S.bxm : S.xm)[it.y + i];
    const bool landed = stage_wait(sh, S, phase);
    bool have = false;
    P2GParticle q;
    q.force = false;
    q.a = 0.0f;
    AxisW w;
    int base[3] = {0, 0, 0};
    if (mine && landed && fabsf(xm.w) <= 100.0f) {  // p2gTransfer.glsl:64-66
      float pg[3];
      grid_coords(S, xm, pg, base);
      all_weights(pg, base, w);
      float Gm[3][3];
      hess_gather(sh, S, bx, by, bz, base, w, Gm);
      have = hess_particle(S, it.y + i, binned, Gm, q);
    }
    if (!p2g_tile_accumulate<kP2gForce>(sh, S, bx, by, bz, have, q, w, base, FixScale{1.0f, 1.0f, 1.0f})) {
      stage_abort(sh, S);  // a copy wait ran out: the CTA stops
      return;
    }
    if (lastw && un < total)
      stage_issue(sh, scenes[sn].cru, kImpBlockFloats, lane < 27 ? slot : -1, scenes[sn].tx_unsent);
    p2g_tile_flush<kP2gForce>(sh, S, bx, by, bz);
    u = un;
    s = sn;
    it = itn;
  }
}

// Per-warp FP64 sum added to *dst. All 32 lanes call it together.
__device__ __forceinline__ void warp_sum_add(double* dst, double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0 && v != 0.0) atomicAdd(dst, v);
}

// Runs body(S, slot, node) -> (d0, d1) over the active nodes of the scenes for
// which run(S) holds (one 64-thread group per active block) and adds the two
// per-scene sums to the doubles that target(S) names. A warp lies inside one
// group, so its scene changes only between blocks and the sums flush per warp.
template <class Run, class Body, class Target>
__device__ __forceinline__ void for_active_nodes(const SceneDev* __restrict__ scenes,
                                                 const int* __restrict__ active_prefix, int nscenes, Run run,
                                                 Body body, Target target) {
  bool any = false;
  for (int s = 0; s < nscenes && !any; s++) any = run(scenes[s]);
  if (!any) return;
  const int groups = blockDim.x / kBlockNodes;
  const int node = threadIdx.x % kBlockNodes;
  const long long total = active_prefix[nscenes];
  int cur = -1;
  double s0 = 0.0, s1 = 0.0;
  for (long long u = (long long)blockIdx.x * groups + threadIdx.x / kBlockNodes; u < total;
       u += (long long)gridDim.x * groups) {
    const int s = find_scene(active_prefix, nscenes, u);
    const SceneDev& S = scenes[s];
    if (!run(S)) continue;
    if (s != cur) {
      if (cur >= 0) {
        double *d0, *d1;
        target(scenes[cur], d0, d1);
        warp_sum_add(d0, s0);
        if (d1) warp_sum_add(d1, s1);
      }
      cur = s;
      s0 = s1 = 0.0;
    }
    const int slot = (int)(u - active_prefix[s]);
    double a = 0.0, b = 0.0;
    body(S, slot, node, a, b);
    s0 += a;
    s1 += b;
  }
  if (cur >= 0) {
    double *d0, *d1;
    target(scenes[cur], d0, d1);
    warp_sum_add(d0, s0);
    if (d1) warp_sum_add(d1, s1);
  }
}

// K u of block `slot` at `node`: floats in the low 4 bytes of acc's force
// words (cleared, as whole words, when `take`).
__device__ __forceinline__ void take_ku(const SceneDev& S, int slot, int node, bool take, float ku[3]) {
  unsigned long long* acc = S.acc + (size_t)S.active[slot] * kAccBlockWords + 4 * kBlockNodes + node;
#pragma unroll
  for (int k = 0; k < 3; k++) {
    ku[k] = *reinterpret_cast<const float*>(acc + k * kBlockNodes);
    if (take) acc[k * kBlockNodes] = 0ull;
  }
}

__device__ __forceinline__ float dot3f(const float a[3], const float b[3]) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }

// M^1/2 and M^-1/2 at a node (both 0 without mass).
__device__ __forceinline__ void mass_scales(float m, float& sq, float& isq) {
  isq = m > 0.0f ? rsqrt_nr(m) : 0.0f;
  sq = m * isq;
}

// r_0 = M^1/2 v* - (I + c M^-1/2 K M^-1/2) M^1/2 v* = -c M^-1/2 K v*
// (c = beta dt^2), u = M^-1/2 r_0; |M^1/2 v*|^2 and |r_0|^2.
__global__ void __launch_bounds__(256) k_cr_begin(const SceneDev* __restrict__ scenes,
                                                  const int* __restrict__ active_prefix, int nscenes) {
  for_active_nodes(
      scenes, active_prefix, nscenes, [](const SceneDev& S) { return cr_running(S, 0); },
      [](const SceneDev& S, int slot, int node, double& bb, double& rr) {
        const size_t i = (size_t)slot * kBlockNodes + node;
        float ku[3];
        take_ku(S, slot, node, true, ku);
        const float4 vm = S.crv[i];
        float sq, isq;
        mass_scales(vm.w, sq, isq);
        const float ci = -S.imp_beta * S.dt * S.dt * isq;
        const float r[3] = {ci * ku[0], ci * ku[1], ci * ku[2]};
        float* u = S.cru + (size_t)slot * kImpBlockFloats + 3 * node;
        u[0] = isq * r[0];
        u[1] = isq * r[1];
        u[2] = isq * r[2];
        const float b[3] = {sq * vm.x, sq * vm.y, sq * vm.z};
        bb = (double)dot3f(b, b);
        rr = (double)dot3f(r, r);
      },
      [](const SceneDev& S, double*& d0, double*& d1) {
        d0 = &S.crs->bb;
        d1 = &S.crs->rr[0];
      });
}

// The residual r = M^1/2 u at one node and A r = r + c M^-1/2 K u (zero
// where the node has no mass).
__device__ __forceinline__ void residual_and_ar(const SceneDev& S, int slot, int node, bool take, float r[3],
                                                float ar[3]) {
  float ku[3];
  take_ku(S, slot, node, take, ku);
  float sq, isq;
  mass_scales(S.crv[(size_t)slot * kBlockNodes + node].w, sq, isq);
  const float ci = S.imp_beta * S.dt * S.dt * isq;
  const float* u = S.cru + (size_t)slot * kImpBlockFloats + 3 * node;
#pragma unroll
  for (int k = 0; k < 3; k++) {
    r[k] = sq * u[k];
    ar[k] = r[k] + ci * ku[k];
  }
}

// Iteration k: (r_{k-1}, A r_{k-1}).
__global__ void __launch_bounds__(256) k_cr_rar(const SceneDev* __restrict__ scenes,
                                                const int* __restrict__ active_prefix, int nscenes,
                                                const int* __restrict__ iter) {
  const int k = *iter;
  for_active_nodes(
      scenes, active_prefix, nscenes, [k](const SceneDev& S) { return cr_running(S, k); },
      [](const SceneDev& S, int slot, int node, double& rar, double&) {
        float r[3], ar[3];
        residual_and_ar(S, slot, node, false, r, ar);
        rar = (double)dot3f(r, ar);
      },
      [k](const SceneDev& S, double*& d0, double*& d1) {
        d0 = &S.crs->rAr[k];
        d1 = nullptr;
      });
}

// Iteration k: beta = rAr[k] / rAr[k-1]; p = r + beta p, A p = A r + beta A p
// (k = 1: p = r, A p = A r); |A p|^2. K r is consumed here.
__global__ void __launch_bounds__(256) k_cr_dir(const SceneDev* __restrict__ scenes,
                                                const int* __restrict__ active_prefix, int nscenes,
                                                const int* __restrict__ iter) {
  const int k = *iter;
  for_active_nodes(
      scenes, active_prefix, nscenes, [k](const SceneDev& S) { return cr_running(S, k); },
      [k](const SceneDev& S, int slot, int node, double& apap, double&) {
        const size_t i = (size_t)slot * kBlockNodes + node;
        const size_t plane = (size_t)S.pool_cap * kBlockNodes;
        float r[3], ar[3];
        residual_and_ar(S, slot, node, true, r, ar);
        const CrScalars& c = *S.crs;
        float beta = 0.0f;
        if (k > 1 && c.rAr[k - 1] != 0.0) beta = (float)(c.rAr[k] / c.rAr[k - 1]);
        float p[3] = {r[0], r[1], r[2]}, ap[3] = {ar[0], ar[1], ar[2]};
        if (k > 1) {
          const float4 p0 = S.crv[plane + i], a0 = S.crv[2 * plane + i];
          p[0] += beta * p0.x;
          p[1] += beta * p0.y;
          p[2] += beta * p0.z;
          ap[0] += beta * a0.x;
          ap[1] += beta * a0.y;
          ap[2] += beta * a0.z;
        }
        S.crv[plane + i] = make_float4(p[0], p[1], p[2], 0.0f);
        S.crv[2 * plane + i] = make_float4(ap[0], ap[1], ap[2], 0.0f);
        apap = (double)dot3f(ap, ap);
      },
      [k](const SceneDev& S, double*& d0, double*& d1) {
        d0 = &S.crs->ApAp[k];
        d1 = nullptr;
      });
}

// Iteration k: alpha = rAr[k] / ApAp[k]; y += alpha p (v += alpha M^-1/2 p),
// r -= alpha A p (u = M^-1/2 r); |r|^2.
__global__ void __launch_bounds__(256) k_cr_update(const SceneDev* __restrict__ scenes,
                                                   const int* __restrict__ active_prefix, int nscenes,
                                                   const int* __restrict__ iter) {
  const int k = *iter;
  for_active_nodes(
      scenes, active_prefix, nscenes, [k](const SceneDev& S) { return cr_running(S, k); },
      [k](const SceneDev& S, int slot, int node, double& rr, double&) {
        const size_t i = (size_t)slot * kBlockNodes + node;
        const size_t plane = (size_t)S.pool_cap * kBlockNodes;
        const CrScalars& c = *S.crs;
        const float alpha = c.ApAp[k] > 0.0 ? (float)(c.rAr[k] / c.ApAp[k]) : 0.0f;
        float4 vm = S.crv[i];
        float sq, isq;
        mass_scales(vm.w, sq, isq);
        const float4 p = S.crv[plane + i], ap = S.crv[2 * plane + i];
        const float ai = alpha * isq;
        vm.x += ai * p.x;
        vm.y += ai * p.y;
        vm.z += ai * p.z;
        S.crv[i] = vm;
        float* u = S.cru + (size_t)slot * kImpBlockFloats + 3 * node;
        const float r[3] = {sq * u[0] - alpha * ap.x, sq * u[1] - alpha * ap.y, sq * u[2] - alpha * ap.z};
        u[0] = isq * r[0];
        u[1] = isq * r[1];
        u[2] = isq * r[2];
        if (slot == 0 && node == 0) S.crs->iters = k;
        rr = (double)dot3f(r, r);
      },
      [k](const SceneDev& S, double*& d0, double*& d1) {
        d0 = &S.crs->rr[k];
        d1 = nullptr;
      });
}

// The colliders on the solved v (gForceCompute.glsl:72-93 at the node), then
// gout's (v*, d) becomes (v, d + v - v*) so that d = v - alpha p/m. A scene
// that skips this step's solve keeps v = v*, already in gout.
__global__ void __launch_bounds__(256) k_cr_end(const SceneDev* __restrict__ scenes,
                                                const int* __restrict__ active_prefix, int nscenes) {
  for_active_nodes(
      scenes, active_prefix, nscenes, [](const SceneDev& S) { return S.crs != nullptr && !S.crs->skipping; },
      [](const SceneDev& S, int slot, int node, double&, double&) {
        const float4 xm = S.crv[(size_t)slot * kBlockNodes + node];
        if (xm.w > 0.0f) {
          const int b = S.active[slot];
          const int bx = b % S.bdim[0], by = (b / S.bdim[0]) % S.bdim[1], bz = b / (S.bdim[0] * S.bdim[1]);
          const int gi = 4 * bx + (node & 3), gj = 4 * by + ((node >> 2) & 3), gk = 4 * bz + (node >> 4);
          const float xi[3] = {__fadd_rn(S.gpos[0], __fmul_rn(S.h, (float)gi)),
                               __fadd_rn(S.gpos[1], __fmul_rn(S.h, (float)gj)),
                               __fadd_rn(S.gpos[2], __fmul_rn(S.h, (float)gk))};
          float v[3] = {xm.x, xm.y, xm.z};
          collide(S.coll, S.ncoll, xi, v);
          float* o = S.gout + (size_t)slot * kOutBlockFloats + kOutFields * node;
          const float vs[3] = {o[0], o[1], o[2]};
#pragma unroll
          for (int k = 0; k < 3; k++) {
            o[3 + k] += v[k] - vs[k];
            o[k] = v[k];
          }
        }
      },
      [](const SceneDev& S, double*& d0, double*& d1) {
        d0 = &S.crs->bb;  // nothing is added (both sums are zero)
        d1 = nullptr;
      });
}

// Advances the iteration counter (first: to 1) and, inside a graph, sets the
// WHILE node's condition: whether any scene runs the new iteration. The
// first call also starts skipped steps for each scene whose initial
// residual is below kCrSkipFactor * its tolerance (CrScalars).
__global__ void k_cr_cond(const SceneDev* __restrict__ scenes, int nscenes, int* iter, int first,
                          cudaGraphConditionalHandle cond, int use_cond) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const int k = first ? 1 : *iter + 1;
  *iter = k;
  if (first)
    for (int s = 0; s < nscenes; s++) {
      const SceneDev& S = scenes[s];
      if (!S.crs || S.crs->skipping) continue;
      double t = kCrSkipFactor * (double)S.imp_tol;
      if (S.crs->rr[0] <= t * t * S.crs->bb) {
        int skip = kCrSkipSteps;
        for (int d = 0; d < kCrSkipDoublings; d++) {
          t *= 0.1;
          if (S.crs->rr[0] > t * t * S.crs->bb) break;
          skip *= 2;
        }
        S.crs->skip_left = skip;
      }
    }
  if (use_cond) cudaGraphSetConditional(cond, any_running(scenes, nscenes, k) ? 1u : 0u);
}

int hess_smem() {
  static bool configured[kMaxDevices] = {};
  const int bytes = (int)sizeof(ItemShared);
  const int dev = current_device();
  if (!configured[dev]) {
    cudaFuncSetAttribute(k_hess, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    configured[dev] = true;
  }
  return bytes;
}

}  // namespace

void fast_implicit_setup() { hess_smem(); }

namespace {
// The gate of a captured solve: taken when any scene solves in this step
// (a scene within its skipped steps leaves v = v* in place).
__global__ void k_cr_gate(const SceneDev* __restrict__ scenes, int nscenes, cudaGraphConditionalHandle gate) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  bool any = false;
  for (int s = 0; s < nscenes && !any; s++) any = scenes[s].crs && !scenes[s].crs->skipping;
  cudaGraphSetConditional(gate, any ? 1u : 0u);
}

void solve_body(const SceneDev* scenes, const int* item_prefix, const int* active_prefix, int nscenes,
                int max_iters, int item_ctas, int grid_ctas, int* d_iter, cudaStream_t body, cudaStream_t st) {
  const int smem = hess_smem();
  auto iteration = [&](cudaStream_t s) {
    k_hess<<<item_ctas, kItemMax, smem, s>>>(scenes, item_prefix, nscenes, d_iter);
    k_cr_rar<<<grid_ctas, 256, 0, s>>>(scenes, active_prefix, nscenes, d_iter);
    k_cr_dir<<<grid_ctas, 256, 0, s>>>(scenes, active_prefix, nscenes, d_iter);
    k_cr_update<<<grid_ctas, 256, 0, s>>>(scenes, active_prefix, nscenes, d_iter);
  };
  k_hess<<<item_ctas, kItemMax, smem, st>>>(scenes, item_prefix, nscenes, nullptr);
  k_cr_begin<<<grid_ctas, 256, 0, st>>>(scenes, active_prefix, nscenes);
  cudaGraphConditionalHandle cond;
  if (capture_handle(st, &cond)) {
    // a conditional WHILE node in the graph being captured (its body is
    // captured from the second stream); errors invalidate the capture and
    // surface at its end
    k_cr_cond<<<1, 32, 0, st>>>(scenes, nscenes, d_iter, 1, cond, 1);
    capture_conditional(st, cond, cudaGraphCondTypeWhile, body, [&](cudaStream_t b) {
      iteration(b);
      k_cr_cond<<<1, 32, 0, b>>>(scenes, nscenes, d_iter, 0, cond, 1);
    });
  } else {
    k_cr_cond<<<1, 32, 0, st>>>(scenes, nscenes, d_iter, 1, cudaGraphConditionalHandle(), 0);
    for (int k = 1; k <= max_iters && k <= kCrMaxIters; k++) {
      iteration(st);
      k_cr_cond<<<1, 32, 0, st>>>(scenes, nscenes, d_iter, 0, cudaGraphConditionalHandle(), 0);
    }
  }
  k_cr_end<<<grid_ctas, 256, 0, st>>>(scenes, active_prefix, nscenes);
}
}  // namespace

void fast_implicit_solve(const SceneDev* scenes, const int* item_prefix, const int* active_prefix, int nscenes,
                         int max_iters, int item_ctas, int grid_ctas, int* d_iter, cudaStream_t body,
                         cudaStream_t gate, cudaStream_t st) {
  cudaGraphConditionalHandle taken;
  if (capture_handle(st, &taken)) {
    k_cr_gate<<<1, 32, 0, st>>>(scenes, nscenes, taken);
    // a failure invalidates the capture, which then fails at its end
    capture_conditional(st, taken, cudaGraphCondTypeIf, gate, [&](cudaStream_t g) {
      solve_body(scenes, item_prefix, active_prefix, nscenes, max_iters, item_ctas, grid_ctas, d_iter, body, g);
    });
    return;
  }
  solve_body(scenes, item_prefix, active_prefix, nscenes, max_iters, item_ctas, grid_ctas, d_iter, body, st);
}

}  // namespace snow
