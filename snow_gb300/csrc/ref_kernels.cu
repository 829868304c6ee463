// SNOW_MODE_REFERENCE kernels: the arithmetic of the reference's compute
// shaders (shader/compute/mpm/*.glsl) on their own std140 buffers, written
// for sm_103a. This translation unit is compiled with -fmad=false so every
// multiply and add rounds separately, as in the shaders; the remaining
// differences to the shaders' results come from expf (CUDA's, within 2 ulp)
// and from atomics being integer (order-independent).
//
// Differences in structure, not in results:
//   * one thread per particle walks the 64 neighbours (the reference launches
//     one invocation per particle x neighbour, (N/1024+1, 64, 1));
//   * the polar decomposition of F_E is computed once per particle instead
//     of once per neighbour (p2gTransfer.glsl:109-110 recomputes it 64x);
//   * every grid kernel is bounds-checked (gReset.glsl and gForceCompute.glsl
//     have no bounds check and run past the grid's end).
#include "snow_internal.h"
#include "snow_math.cuh"
#include "snow_stats.cuh"

namespace snow {
namespace {

constexpr int kThreads = 256;

__device__ __forceinline__ M3 load_mat4(const float4* m) {
  M3 a;
#pragma unroll
  for (int c = 0; c < 3; c++) {
    const float4 col = m[c];
    a.m[c][0] = col.x;
    a.m[c][1] = col.y;
    a.m[c][2] = col.z;
  }
  return a;
}
// mat4(mat3): identity outside the upper-left block.
__device__ __forceinline__ void store_mat4(float4* m, const M3& a) {
#pragma unroll
  for (int c = 0; c < 3; c++) m[c] = make_float4(a.m[c][0], a.m[c][1], a.m[c][2], 0.0f);
  m[3] = make_float4(0.0f, 0.0f, 0.0f, 1.0f);
}

__device__ __forceinline__ void neighbour(int y, int o[3]) {  // neighborIndex.include.glsl:6-12
  const int t = y % 16;
  o[0] = t % 4 - 1;
  o[1] = t / 4 - 1;
  o[2] = y / 16 - 1;
}

// Collider projection, gForceCompute.glsl:72-93 / particleAdvance.glsl:182-204.
__device__ void collide(const snow_collider* coll, int ncoll, const float x[3], float v[3]) {
  for (int i = 0; i < ncoll; i++) {
    const snow_collider c = coll[i];
    float n[3] = {c.normal[0], c.normal[1], c.normal[2]};
    bool hit = false;
    const unsigned t = (unsigned)c.type;
    if (t == 0u) {
      hit = (x[0] - c.pos[0]) * c.normal[0] + (x[1] - c.pos[1]) * c.normal[1] + (x[2] - c.pos[2]) * c.normal[2] <=
            0.0f;
    } else if (t == 1u) {
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
      float vrelt[3] = {vt[0], vt[1], vt[2]};
      if (lvt <= -muvn) {
        vrelt[0] = vrelt[1] = vrelt[2] = 0.0f;
      } else {
#pragma unroll
        for (int k = 0; k < 3; k++) vrelt[k] = vrelt[k] + (muvn * vt[k]) / lvt;
      }
#pragma unroll
      for (int k = 0; k < 3; k++) v[k] = vrelt[k] + c.vel[k];
    }
  }
}

__global__ void k_rigid(snow_collider* coll, int ncoll, float dt) {  // rigidAdvance.glsl:14-18
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < ncoll)
    for (int k = 0; k < 3; k++) coll[i].pos[k] = coll[i].pos[k] + dt * coll[i].vel[k];
}

// p2gTransfer.glsl:44-151; with MASS_ONLY, gMassCompute.glsl:33-84.
template <bool MASS_ONLY>
__global__ void __launch_bounds__(kThreads) k_p2g(RefArgs a) {
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < a.n; p += gridDim.x * blockDim.x) {
    const float4 xm = a.pxm[p];
    const float mp = xm.w;
    if (!MASS_ONLY && fabsf(mp) > 100.0f) continue;
    const int4 pvi = a.pv[p];
    const float vp[3] = {(float)pvi.x * 1e-8f, (float)pvi.y * 1e-8f, (float)pvi.z * 1e-8f};
    const float pp0 = (float)pvi.w * 1e-6f;
    const float pg[3] = {(xm.x - a.gpos[0]) / a.h, (xm.y - a.gpos[1]) / a.h, (xm.z - a.gpos[2]) / a.h};
    const int base[3] = {(int)pg[0], (int)pg[1], (int)pg[2]};
    M3 stress;
    float vol_scale = 0.0f;
    if (!MASS_ONLY) {
      const M3 FE = load_mat4(a.pfe + 4 * (size_t)p);
      const M3 FP = load_mat4(a.pfp + 4 * (size_t)p);
      M3 W, S, V;
      svd3<true>(FE, W, S, V);
      M3 R = m3_mul(W, m3_transpose(V));
#pragma unroll
      for (int c = 0; c < 3; c++)
#pragma unroll
        for (int r = 0; r < 3; r++) R.m[c][r] = quantize(R.m[c][r], 1e9f);
      const float jpp = m3_det(FP);
      const float jep = m3_det(FE);
      const float s1 = 2.0f * lame_mu(a.young, a.poisson, a.hardening, jpp);
      M3 t;
#pragma unroll
      for (int c = 0; c < 3; c++)
#pragma unroll
        for (int r = 0; r < 3; r++) t.m[c][r] = s1 * (FE.m[c][r] - R.m[c][r]);
      const M3 A = m3_mul(t, m3_transpose(FE));
      const float s2 = lame_lambda(a.young, a.poisson, a.hardening, jpp) * (jep - 1.0f) * jep;
#pragma unroll
      for (int c = 0; c < 3; c++)
#pragma unroll
        for (int r = 0; r < 3; r++) stress.m[c][r] = A.m[c][r] + s2 * (c == r ? 1.0f : 0.0f);
      vol_scale = -(mp / pp0);
    }
    for (int y = 0; y < 64; y++) {
      int o[3];
      neighbour(y, o);
      const int g[3] = {base[0] + o[0], base[1] + o[1], base[2] + o[2]};
      if (!(g[0] >= 0 && g[1] >= 0 && g[2] >= 0 && g[0] < a.dim[0] && g[1] < a.dim[1] && g[2] < a.dim[2]))
        continue;
      const float d[3] = {(float)g[0] - pg[0], (float)g[1] - pg[1], (float)g[2] - pg[2]};
      const float w = bspline(d[0]) * bspline(d[1]) * bspline(d[2]);
      const long long gI = (long long)g[0] + (long long)g[1] * a.dim[0] + (long long)g[2] * a.dim[1] * a.dim[0];
      atomicAdd(&a.gv[gI].w, (int)(mp * w * 1e8f));
      if (MASS_ONLY) continue;
      atomicAdd(&a.gv[gI].x, (int)(vp[0] * mp * w * 1e8f));
      atomicAdd(&a.gv[gI].y, (int)(vp[1] * mp * w * 1e8f));
      atomicAdd(&a.gv[gI].z, (int)(vp[2] * mp * w * 1e8f));
      if (pp0 > 0.0f) {
        const float nd[3] = {-d[0], -d[1], -d[2]};
        const float wg[3] = {bspline_d(nd[0]) * bspline(nd[1]) * bspline(nd[2]),
                             bspline(nd[0]) * bspline_d(nd[1]) * bspline(nd[2]),
                             bspline(nd[0]) * bspline(nd[1]) * bspline_d(nd[2])};
        float f[3];
#pragma unroll
        for (int r = 0; r < 3; r++)
          f[r] = vol_scale *
                 (stress.m[0][r] * wg[0] + stress.m[1][r] * wg[1] + stress.m[2][r] * wg[2]);
        atomicAdd(&a.gf[gI].x, (int)(f[0] * 1e6f));
        atomicAdd(&a.gf[gI].y, (int)(f[1] * 1e6f));
        atomicAdd(&a.gf[gI].z, (int)(f[2] * 1e6f));
      }
    }
  }
}

// pVolumeCompute.glsl:32-83: the density sum runs in a register (the shader
// sums the same truncated terms with atomicAdd into pv.w).
__global__ void __launch_bounds__(kThreads) k_volume(RefArgs a) {
  const float cell = a.h * a.h * a.h;
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < a.n; p += gridDim.x * blockDim.x) {
    const float4 xm = a.pxm[p];
    const float pg[3] = {(xm.x - a.gpos[0]) / a.h, (xm.y - a.gpos[1]) / a.h, (xm.z - a.gpos[2]) / a.h};
    const int base[3] = {(int)pg[0], (int)pg[1], (int)pg[2]};
    unsigned acc = (unsigned)a.pv[p].w;
    for (int y = 0; y < 64; y++) {
      int o[3];
      neighbour(y, o);
      const int g[3] = {base[0] + o[0], base[1] + o[1], base[2] + o[2]};
      if (!(g[0] >= 0 && g[1] >= 0 && g[2] >= 0 && g[0] < a.dim[0] && g[1] < a.dim[1] && g[2] < a.dim[2]))
        continue;
      const float d[3] = {(float)g[0] - pg[0], (float)g[1] - pg[1], (float)g[2] - pg[2]};
      const float w = bspline(d[0]) * bspline(d[1]) * bspline(d[2]);
      const long long gI = (long long)g[0] + (long long)g[1] * a.dim[0] + (long long)g[2] * a.dim[1] * a.dim[0];
      const float mi = (float)a.gv[gI].w * 1e-8f;
      acc += (unsigned)(int)(mi * w / cell * 1e6f);
    }
    a.pv[p].w = (int)acc;
  }
}

// gForceCompute.glsl:57-103
__global__ void __launch_bounds__(kThreads) k_grid(RefArgs a, float dt) {
  for (long long gI = blockIdx.x * (long long)blockDim.x + threadIdx.x; gI < a.G;
       gI += (long long)gridDim.x * blockDim.x) {
    const int4 gv = a.gv[gI];
    const float mi = (float)gv.w * 1e-8f;
    if (!(mi > 0.0f)) {
      a.gvn[gI] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
      continue;
    }
    const int4 gf = a.gf[gI];
    const float vi[3] = {(float)gv.x * 1e-8f, (float)gv.y * 1e-8f, (float)gv.z * 1e-8f};
    const float fi[3] = {(float)gf.x * 1e-6f, (float)gf.y * 1e-6f, (float)gf.z * 1e-6f};
    float vin[3];
#pragma unroll
    for (int k = 0; k < 3; k++) vin[k] = vi[k] / mi + dt * (fi[k] / mi + a.grav[k]);
    // Grid::initSSBO node position x_off + h * (float)i (grid.cpp:96-107)
    const int i = (int)(gI % a.dim[0]);
    const int j = (int)((gI / a.dim[0]) % a.dim[1]);
    const int k = (int)(gI / ((long long)a.dim[0] * a.dim[1]));
    const float xi[3] = {a.gpos[0] + a.h * (float)i, a.gpos[1] + a.h * (float)j, a.gpos[2] + a.h * (float)k};
    collide(a.coll, a.ncoll, xi, vin);
    a.gvn[gI] = make_float4(vin[0], vin[1], vin[2], 0.0f);
  }
}

// g2pTransfer.glsl:53-143: per-particle sums of truncated contributions.
__global__ void __launch_bounds__(kThreads) k_g2p(RefArgs a) {
  const float alpha = a.alpha;
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < a.n; p += gridDim.x * blockDim.x) {
    const float4 xm = a.pxm[p];
    const float pg[3] = {(xm.x - a.gpos[0]) / a.h, (xm.y - a.gpos[1]) / a.h, (xm.z - a.gpos[2]) / a.h};
    const int base[3] = {(int)pg[0], (int)pg[1], (int)pg[2]};
    unsigned av[3] = {0u, 0u, 0u};
    unsigned ad[3][3] = {{0u, 0u, 0u}, {0u, 0u, 0u}, {0u, 0u, 0u}};
    for (int y = 0; y < 64; y++) {
      int o[3];
      neighbour(y, o);
      const int g[3] = {base[0] + o[0], base[1] + o[1], base[2] + o[2]};
      if (!(g[0] >= 0 && g[1] >= 0 && g[2] >= 0 && g[0] < a.dim[0] && g[1] < a.dim[1] && g[2] < a.dim[2]))
        continue;
      const float d[3] = {(float)g[0] - pg[0], (float)g[1] - pg[1], (float)g[2] - pg[2]};
      const float w = bspline(d[0]) * bspline(d[1]) * bspline(d[2]);
      const float nd[3] = {-d[0], -d[1], -d[2]};
      const float gw[3] = {bspline_d(nd[0]) * bspline(nd[1]) * bspline(nd[2]),
                           bspline(nd[0]) * bspline_d(nd[1]) * bspline(nd[2]),
                           bspline(nd[0]) * bspline(nd[1]) * bspline_d(nd[2])};
      const long long gI = (long long)g[0] + (long long)g[1] * a.dim[0] + (long long)g[2] * a.dim[1] * a.dim[0];
      const float4 vn4 = a.gvn[gI];
      const int4 gv = a.gv[gI];
      const float vin[3] = {vn4.x, vn4.y, vn4.z};
      const float vi[3] = {(float)gv.x * 1e-8f, (float)gv.y * 1e-8f, (float)gv.z * 1e-8f};
      const float mi = (float)gv.w * 1e-8f;
      if (mi > 0.0f) {
#pragma unroll
        for (int k = 0; k < 3; k++) {
          const float vpn = (1.0f - alpha) * vin[k] * w + alpha * (vin[k] - vi[k] / mi) * w;
          av[k] += (unsigned)(int)(vpn * 1e8f);
        }
#pragma unroll
        for (int c = 0; c < 3; c++)
#pragma unroll
          for (int r = 0; r < 3; r++) ad[c][r] += (unsigned)(int)(vin[r] * gw[c] * 1e8f);
      }
    }
    a.pvn[p] = make_int4((int)av[0], (int)av[1], (int)av[2], a.pvn[p].w);
    a.pd0[p] = make_int4((int)ad[0][0], (int)ad[0][1], (int)ad[0][2], a.pd0[p].w);
    a.pd1[p] = make_int4((int)ad[1][0], (int)ad[1][1], (int)ad[1][2], a.pd1[p].w);
    a.pd2[p] = make_int4((int)ad[2][0], (int)ad[2][1], (int)ad[2][2], a.pd2[p].w);
  }
}

// particleAdvance.glsl:75-217
__global__ void __launch_bounds__(kThreads) k_advance(RefArgs a, float dt) {
  const float lo = 1.0f - a.crit_c, hi = 1.0f + a.crit_s;
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < a.n; p += gridDim.x * blockDim.x) {
    const M3 FE = load_mat4(a.pfe + 4 * (size_t)p);
    const M3 FP = load_mat4(a.pfp + 4 * (size_t)p);
    const int4 d0 = a.pd0[p], d1 = a.pd1[p], d2 = a.pd2[p];
    M3 dvp;
    dvp.m[0][0] = (float)d0.x * 1e-8f; dvp.m[0][1] = (float)d0.y * 1e-8f; dvp.m[0][2] = (float)d0.z * 1e-8f;
    dvp.m[1][0] = (float)d1.x * 1e-8f; dvp.m[1][1] = (float)d1.y * 1e-8f; dvp.m[1][2] = (float)d1.z * 1e-8f;
    dvp.m[2][0] = (float)d2.x * 1e-8f; dvp.m[2][1] = (float)d2.y * 1e-8f; dvp.m[2][2] = (float)d2.z * 1e-8f;
    M3 step;
#pragma unroll
    for (int c = 0; c < 3; c++)
#pragma unroll
      for (int r = 0; r < 3; r++) step.m[c][r] = (c == r ? 1.0f : 0.0f) + dt * dvp.m[c][r];
    M3 fe = m3_mul(step, FE);
    const M3 fall = m3_mul(step, m3_mul(FE, FP));
    M3 W, S, V;
    svd3<true>(fe, W, S, V);
#pragma unroll
    for (int i = 0; i < 3; i++) S.m[i][i] = (S.m[i][i] < lo) ? lo : (S.m[i][i] > hi) ? hi : S.m[i][i];
    fe = m3_mul(m3_mul(W, S), m3_transpose(V));
#pragma unroll
    for (int c = 0; c < 3; c++)
#pragma unroll
      for (int r = 0; r < 3; r++) fe.m[c][r] = quantize(fe.m[c][r], 1e9f);
    M3 sinv = m3_diag(0.0f);
#pragma unroll
    for (int i = 0; i < 3; i++) sinv.m[i][i] = 1.0f / S.m[i][i];
    M3 fp = m3_mul(m3_mul(m3_mul(V, sinv), m3_transpose(W)), fall);
#pragma unroll
    for (int c = 0; c < 3; c++)
#pragma unroll
      for (int r = 0; r < 3; r++) fp.m[c][r] = quantize(fp.m[c][r], 1e9f);
    store_mat4(a.pfe + 4 * (size_t)p, fe);
    store_mat4(a.pfp + 4 * (size_t)p, fp);
    const int4 pn = a.pvn[p];
    const int4 pv = a.pv[p];
    float v[3] = {(float)pv.x * 1e-8f * a.alpha + (float)pn.x * 1e-8f, (float)pv.y * 1e-8f * a.alpha + (float)pn.y * 1e-8f,
                  (float)pv.z * 1e-8f * a.alpha + (float)pn.z * 1e-8f};
    float4 xm = a.pxm[p];
    const float x[3] = {xm.x, xm.y, xm.z};
    collide(a.coll, a.ncoll, x, v);
    a.pv[p] = make_int4((int)(v[0] * 1e8f), (int)(v[1] * 1e8f), (int)(v[2] * 1e8f), pv.w);
    xm.x = xm.x + dt * v[0];
    xm.y = xm.y + dt * v[1];
    xm.z = xm.z + dt * v[2];
    a.pxm[p] = xm;
    a.pvn[p] = make_int4(0, 0, 0, pn.w);
    a.pd0[p] = make_int4(0, 0, 0, d0.w);
    a.pd1[p] = make_int4(0, 0, 0, d1.w);
    a.pd2[p] = make_int4(0, 0, 0, d2.w);
  }
}

static_assert(kThreads == kStatsThreads, "the statistics commit assumes this block size");
__global__ void __launch_bounds__(kThreads) k_stats(RefArgs a, StatsSlot* slot, StatsAccum* host) {
  StatsPartial t;
  stats_init(t);
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < a.n; p += gridDim.x * blockDim.x) {
    const float4 xm = a.pxm[p];
    const int4 pv = a.pv[p];
    const double v[3] = {pv.x * 1e-8, pv.y * 1e-8, pv.z * 1e-8};
    const float jp = m3_det(load_mat4(a.pfp + 4 * (size_t)p));
    if (!(isfinite(xm.x) && isfinite(xm.y) && isfinite(xm.z) && isfinite(jp))) {
      t.bad++;
      continue;
    }
    const double m = xm.w;
    t.acc[0] += m;
    t.acc[1] += m * v[0];
    t.acc[2] += m * v[1];
    t.acc[3] += m * v[2];
    t.acc[4] += 0.5 * m * (v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    t.acc[5] += m * xm.x;
    t.acc[6] += m * xm.y;
    t.acc[7] += m * xm.z;
    t.acc[8] += jp;
    t.bmin[0] = fminf(t.bmin[0], xm.x); t.bmin[1] = fminf(t.bmin[1], xm.y); t.bmin[2] = fminf(t.bmin[2], xm.z);
    t.bmax[0] = fmaxf(t.bmax[0], xm.x); t.bmax[1] = fmaxf(t.bmax[1], xm.y); t.bmax[2] = fmaxf(t.bmax[2], xm.z);
  }
  stats_commit(t, slot, host);
}

int grid_for(long long n) {
  const long long b = (n + kThreads - 1) / kThreads;
  const long long cap = (long long)num_sms() * 8;
  return (int)(b < 1 ? 1 : (b > cap ? cap : b));
}

}  // namespace

void ref_rigid(snow_collider* coll, int ncoll, float dt, cudaStream_t st) {
  if (ncoll > 0) k_rigid<<<(ncoll + 63) / 64, 64, 0, st>>>(coll, ncoll, dt);
}
void ref_reset(const RefArgs& a, cudaStream_t st) {  // gReset.glsl:11-16
  cudaMemsetAsync(a.gv, 0, sizeof(int4) * a.G, st);
  cudaMemsetAsync(a.gf, 0, sizeof(int4) * a.G, st);
}
void ref_p2g(const RefArgs& a, bool mass_only, cudaStream_t st) {
  if (a.n <= 0) return;
  if (mass_only)
    k_p2g<true><<<grid_for(a.n), kThreads, 0, st>>>(a);
  else
    k_p2g<false><<<grid_for(a.n), kThreads, 0, st>>>(a);
}
void ref_volume(const RefArgs& a, cudaStream_t st) {
  if (a.n > 0) k_volume<<<grid_for(a.n), kThreads, 0, st>>>(a);
}
void ref_grid(const RefArgs& a, float dt, cudaStream_t st) { k_grid<<<grid_for(a.G), kThreads, 0, st>>>(a, dt); }
void ref_g2p(const RefArgs& a, cudaStream_t st) {
  if (a.n > 0) k_g2p<<<grid_for(a.n), kThreads, 0, st>>>(a);
}
void ref_stats(const RefArgs& a, StatsSlot* slot, StatsAccum* host, cudaStream_t st) {
  // at least one block (it publishes empty sums), at most one partial per slot entry
  const int g = a.n > 0 ? grid_for(a.n) : 1;
  k_stats<<<g < kStatsMaxBlocks ? g : kStatsMaxBlocks, kThreads, 0, st>>>(a, slot, host);
}
void ref_advance(const RefArgs& a, float dt, cudaStream_t st) {
  if (a.n > 0) k_advance<<<grid_for(a.n), kThreads, 0, st>>>(a, dt);
}

}  // namespace snow
