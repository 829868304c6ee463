// Device helpers of the FAST path shared by its kernel files
// (fast_kernels.cu: the explicit step; implicit.cu: the semi-implicit
// velocity solve): B-spline weights, colliders, the P2G quantities of a
// particle, the shared memory of a work item with its bulk copies (TMA) of
// pool blocks, the G2P gather, the particle advance and the P2G tile pass.
#pragma once
#include "snow_internal.h"
#include "snow_math.cuh"
#include "snow_tma.cuh"

namespace snow {
namespace {

constexpr int kTile = 9;  // tile nodes per axis: [4b-2, 4b+6]
constexpr int kTile3 = kTile * kTile * kTile;
// A work item holds up to kItemMax particles binned to one home block b. A
// particle whose base cell lies in [4b-1, 4b+4] (the home block plus one
// cell of drift each way) has its whole stencil inside the tile; its base
// cell has tile-local coordinates lc = base - (4b-2) - 1 in [0, 5]^3.
constexpr int kItemMax = 256;
// What a P2G tile pass accumulates: the grid mass alone (gMassCompute.glsl),
// mass, momentum and stress force (p2gTransfer.glsl), or only a force-like
// 3-vector per node (the semi-implicit solve's K u, into the force slots).
enum P2gKind { kP2gMass = 0, kP2gFull = 1, kP2gForce = 2 };
template <int KIND> struct P2gFields {
  static constexpr int nf = KIND == kP2gMass ? 1 : (KIND == kP2gFull ? kAccFields : 3);
  static constexpr int acc_first = KIND == kP2gForce ? 4 : 0;  // first acc field written
};
constexpr int kCellsPerAxis = kTile - 3;  // 6
constexpr int kCells = kCellsPerAxis * kCellsPerAxis * kCellsPerAxis;
constexpr int kPd = 11;  // float4 per particle of P2G data in shared memory: 10 used, the 11th pads
                         // the stride to 44 words so the 8 threads of a 16-byte store phase hit 8
                         // distinct groups of 4 banks
constexpr int kShColliders = 16;  // colliders cached in shared memory

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
__device__ __forceinline__ void axis_weights_general(float pg, int base, float w[4], float g[4]) {
#pragma unroll
  for (int a = 0; a < 4; a++) {
    const float d = (float)(base + a - 1) - pg;
    w[a] = bspline(d);
    g[a] = bspline_d(-d);
  }
}

// The same weights without branches for pg >= 0, where base = floor(pg) and
// f = pg - base is in [0, 1): the stencil distances are |d| = 1+f, f, 1-f,
// 2-f, each on a known piece of the spline. With u = 1 - f:
//   w = (u^3/6, f^3/2 - f^2 + 2/3, u^3/2 - u^2 + 2/3, f^3/6)
//   g = (-u^2/2, 3f^2/2 - 2f, -3u^2/2 + 2u, f^2/2)
// Particles below the grid origin (pg < 0, truncated toward zero) take the
// general path.
__device__ __forceinline__ void axis_weights(float pg, int base, float w[4], float g[4]) {
  if (pg < 0.0f) {
    axis_weights_general(pg, base, w, g);
    return;
  }
  const float f = pg - (float)base;
  const float u = 1.0f - f;
  const float f2 = f * f, u2 = u * u;
  const float f3 = f2 * f, u3 = u2 * u;
  w[0] = u3 * (1.0f / 6.0f);
  w[1] = 0.5f * f3 - f2 + 2.0f / 3.0f;
  w[2] = 0.5f * u3 - u2 + 2.0f / 3.0f;
  w[3] = f3 * (1.0f / 6.0f);
  g[0] = -0.5f * u2;
  g[1] = 1.5f * f2 - 2.0f * f;
  g[2] = -1.5f * u2 + 2.0f * u;
  g[3] = 0.5f * f2;
}

struct AxisW {
  float wx[4], gx[4], wy[4], gy[4], wz[4], gz[4];
};

// Grid coordinates (x - gGridPos) / h. Multiplying by 1/h can move a value
// by an ulp against the shaders' division; at a cell boundary that only
// swaps which stencil end carries the (zero) weight, so the sums agree.
__device__ __forceinline__ void grid_coords(const SceneDev& S, float4 xm, float pg[3], int base[3]) {
  pg[0] = (xm.x - S.gpos[0]) * S.inv_h;
  pg[1] = (xm.y - S.gpos[1]) * S.inv_h;
  pg[2] = (xm.z - S.gpos[2]) * S.inv_h;
#pragma unroll
  for (int k = 0; k < 3; k++) base[k] = (int)pg[k];  // ivec3(): truncation toward zero
}

__device__ __forceinline__ void all_weights(const float pg[3], const int base[3], AxisW& w) {
  axis_weights(pg[0], base[0], w.wx, w.gx);
  axis_weights(pg[1], base[1], w.wy, w.gy);
  axis_weights(pg[2], base[2], w.wz, w.gz);
}

// Whether this step's binning left the particles in the binned copies.
__device__ __forceinline__ bool particles_binned(const SceneDev& S) { return S.counters[CNT_BINNED] != 0; }

__device__ __forceinline__ void load_fe(const SceneDev& S, int p, M3& F, float& jp, bool binned = false) {
  const float4 a = (binned ? S.bfa : S.fa)[p];
  const float4 b = (binned ? S.bfb : S.fb)[p];
  const float2 c = (binned ? S.bfc : S.fc)[p];
  F.m[0][0] = a.x; F.m[0][1] = a.y; F.m[0][2] = a.z;
  F.m[1][0] = a.w; F.m[1][1] = b.x; F.m[1][2] = b.y;
  F.m[2][0] = b.z; F.m[2][1] = b.w; F.m[2][2] = c.x;
  jp = c.y;
}
__device__ __forceinline__ void store_fe(const SceneDev& S, int p, const M3& F, float jp) {
  __stcs(&S.fa[p], make_float4(F.m[0][0], F.m[0][1], F.m[0][2], F.m[1][0]));
  __stcs(&S.fb[p], make_float4(F.m[1][1], F.m[1][2], F.m[2][0], F.m[2][1]));
  __stcs(&S.fc[p], make_float2(F.m[2][2], jp));
}

__device__ __forceinline__ int block_id(const SceneDev& S, int bx, int by, int bz) {
  return (bz * S.bdim[1] + by) * S.bdim[0] + bx;
}

__device__ __forceinline__ bool node_in_grid(const SceneDev& S, int g0, int g1, int g2) {
  return g0 >= 0 && g1 >= 0 && g2 >= 0 && g0 < S.dim[0] && g1 < S.dim[1] && g2 < S.dim[2];
}

// Collider projection of gForceCompute.glsl:72-93 / particleAdvance.glsl:182-204
// for one collider that the point x hits: the velocity relative to the
// collider loses its normal inward part, with Coulomb friction.
__device__ __forceinline__ void collide_hit(const snow_collider& c, const float x[3], float v[3]) {
  float n[3] = {c.normal[0], c.normal[1], c.normal[2]};
  if (c.type == 1) {
    const float d[3] = {x[0] - c.pos[0], x[1] - c.pos[1], x[2] - c.pos[2]};
    const float len = sqrtf(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
    n[0] = d[0] / len;
    n[1] = d[1] / len;
    n[2] = d[2] / len;
  }
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

// All colliders in order (half-plane: dot(x - c, n) <= 0; sphere: |x - c| < r).
// A record is three 16-byte words, (pos, type), (vel, radius), (normal,
// friction): the test reads the first and the one it needs, the projection
// the whole record, only for a hit.
__device__ __forceinline__ void collide(const snow_collider* coll, int ncoll, const float x[3], float v[3]) {
  static_assert(sizeof(snow_collider) == 48, "three 16-byte words per collider");
  for (int i = 0; i < ncoll; i++) {
    const float4* c4 = reinterpret_cast<const float4*>(coll + i);
    const float4 a = c4[0];
    const int type = __float_as_int(a.w);
    bool hit = false;
    if (type == 0) {
      const float4 nf = c4[2];
      hit = (x[0] - a.x) * nf.x + (x[1] - a.y) * nf.y + (x[2] - a.z) * nf.z <= 0.0f;
    } else if (type == 1) {
      const float r = c4[1].w;
      const float d[3] = {x[0] - a.x, x[1] - a.y, x[2] - a.z};
      hit = sqrtf(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]) < r;
    }
    if (hit) collide_hit(coll[i], x, v);
  }
}

// The same with the hit tests on a packed form of the colliders (half-plane:
// (n, n . c), tested as n . x <= n . c; sphere: (c, r^2), tested as
// |x - c|^2 < r^2): one 16-byte shared load per collider, the full record
// only for the rare hit.
__device__ __forceinline__ void collide_packed(const snow_collider* coll, const float4* hitf, const int* type,
                                               int ncoll, const float x[3], float v[3]) {
  for (int i = 0; i < ncoll; i++) {
    const float4 h = hitf[i];
    const int t = type[i];
    bool hit = false;
    if (t == 0) {
      hit = fmaf(h.z, x[2], fmaf(h.y, x[1], h.x * x[0])) <= h.w;
    } else if (t == 1) {
      const float d0 = x[0] - h.x, d1 = x[1] - h.y, d2 = x[2] - h.z;
      hit = fmaf(d2, d2, fmaf(d1, d1, d0 * d0)) < h.w;
    }
    if (hit) collide_hit(coll[i], x, v);
  }
}

// ---- fixed-point P2G sums ------------------------------------------------------
// Every contribution of a particle to a grid node (mass m w, momentum m v w,
// force A grad w) is rounded to an integer at a per-scene power-of-two scale
// (s_m, s_p, s_f), and integers are summed: in registers and in the shared
// tile as int32 (modulo 2^32; each particle adds a bound of its largest
// contribution to its item, and a tile is added to acc before the bounds of
// the particles it holds could reach 2^31, so its sums never wrap), into
// acc as int64. Integer sums do not depend on the
// order in which they are formed, so the grid a particle state produces does
// not depend on how particles are grouped into work items, on the binning
// schedule, on CTA scheduling or on the other scenes of a batch. The rounding
// of one contribution is the same on every path that forms it: the tile path
// and the per-node scatter of a particle outside its work item's tile both
// compute it with the same pinned (_rn) operations.
//
// A contribution y (|y| < 2^22 after scaling) is rounded by one FMA against
// kMagic = 1.5 * 2^23: fma(w, x, kMagic) lies in [2^23, 2^24), where floats
// are spaced by 1, so its bits minus kMagicBits are round(w x). A force
// contribution g_x kk + w_x hh is rounded as round(g_x kk + round(w_x hh));
// with a = max over rows r of |A_r0| + |A_r1| + |A_r2|, both terms and their
// sum are at most a (2/3)^3 s_f. The mass scale puts the largest
// contribution near 2^21; the momentum and force scales put bounds that
// already carry a growth margin (1.25 max|v| + margins, twice the largest
// stress term) into [2^21, 2^22), the fast range's limit. A particle whose
// contributions reach the limit (it outgrew the magnitudes the scales were
// chosen from) is scattered with int64 contributions rounded in double
// precision ("wide"), which depends only on the particle itself, so it is
// as deterministic.
constexpr float kMagic = 12582912.0f;  // 1.5 * 2^23
constexpr int kMagicBits = 0x4B400000;
constexpr float kWmax = 0.2962963f;       // (2/3)^3 >= any weight or weight-gradient product
constexpr float kFastLimit = 4190208.0f;       // 2^22 (1 - 2^-11): bound of a fast-path contribution
constexpr float kTileSumBound = 2126008832.0f;  // 0.99 * 2^31: bound of a tile's sums of contribution bounds

// The largest power of two s with x s <= 2^bits (1 for x <= 0 or not finite).
__device__ __forceinline__ float pow2_scale(float x, int bits) {
  if (!(x > 0.0f) || !isfinite(x)) return 1.0f;
  int e;
  frexpf(x, &e);  // x = f 2^e, f in [0.5, 1): x 2^(bits - e) in [2^(bits-1), 2^bits)
  return ldexpf(1.0f, max(-126, min(127, bits - e)));
}

struct FixScale {
  float m, p, f;
};

__device__ __forceinline__ float bits_float(uint32_t b) { return __uint_as_float(b); }

// Scales of a P2G that follows a grid update in the same step (the fused
// kernel): from the magnitudes of the particles the previous P2G scattered
// (FixState::*_prev). The momentum scale allows particle speeds up to
// 1.25 max|v_p| + 2 max|v_collider| + 2 |g| dt (a collider projection adds
// at most twice the collider's speed; the last term keeps the scale finite
// for a scene at rest, which gravity moves by |g| dt a step).
// It is taken from particle speeds alone: v* = p/m + dt (f/m + g) of a node
// that holds a sliver of mass can exceed every particle's speed by orders of
// magnitude, while the G2P weights such a node by as small a sliver. The
// force scale allows twice the previous largest stress term (the floor
// 1e-9 E0 V0max keeps it finite for a scene without stress). A particle
// beyond either takes the wide path.
__device__ __forceinline__ FixScale step_scales(const SceneDev& S) {
  const FixState& f = *S.fix;
  const float mmax = bits_float(f.m_prev);
  float vcoll = 0.0f;
  for (int i = 0; i < S.ncoll; i++) {
    const float* cv = S.coll[i].vel;
    vcoll = fmaxf(vcoll, sqrtf(cv[0] * cv[0] + cv[1] * cv[1] + cv[2] * cv[2]));
  }
  const float g = sqrtf(S.grav[0] * S.grav[0] + S.grav[1] * S.grav[1] + S.grav[2] * S.grav[2]);
  const float vb = 1.25f * bits_float(f.v_prev) + 2.0f * vcoll + 2.0f * g * S.dt;
  const float afloor = 1e-9f * S.young * bits_float(f.v0max);
  FixScale sc;
  sc.m = pow2_scale(mmax * kWmax, 21);
  sc.p = pow2_scale(mmax * vb * kWmax, 22);
  sc.f = pow2_scale(fmaxf(2.0f * bits_float(f.a_prev), afloor) * kWmax, 22);
  return sc;
}

// Scales of a P2G of the stored state (set-up, per-kernel dispatches): from
// the exact magnitudes a pass over the particles just measured (k_fix_measure).
__device__ __forceinline__ FixScale measured_scales(const SceneDev& S) {
  const FixState& f = *S.fix;
  const float mmax = bits_float(f.m_prev);
  const float afloor = 1e-9f * S.young * bits_float(f.v0max);
  FixScale sc;
  sc.m = pow2_scale(mmax * kWmax, 21);
  sc.p = pow2_scale(mmax * bits_float(f.v_prev) * kWmax, 22);
  sc.f = pow2_scale(fmaxf(bits_float(f.a_prev), afloor) * kWmax, 22);
  return sc;
}

// Adds one node's integer sums v[0..6] (m, p, f; mass_only: v[0]) into acc
// (two's complement adds: a sum of int64 values, whatever the order).
__device__ __forceinline__ void acc_add(const SceneDev& S, int blk, int node, const long long v[7], bool mass_only) {
  unsigned long long* a = S.acc + (size_t)blk * kAccBlockWords + node;
  const int nw = mass_only ? 1 : kAccWords;
  for (int f = 0; f < nw; f++)
    if (v[f]) atomicAdd(a + f * kBlockNodes, (unsigned long long)v[f]);
}

// ---- P2G quantities of one particle -----------------------------------------
// mass, momentum and A = -V0 * stress, stress = 2 mu(Jp) (FE - R) FE^T +
// lambda(Jp) (JE - 1) JE I with R the polar rotation of FE
// (p2gTransfer.glsl:109-141); V0 = m / rho0. `a` = max over rows r of
// |A_r0| + |A_r1| + |A_r2| bounds a force contribution and both its terms
// (in units of the weight products' bound (2/3)^3).
struct P2GParticle {
  float m, mv[3];
  float A[3][3];  // A[r][c]
  float a;
  bool force;
};

__device__ __forceinline__ void p2g_stress(const SceneDev& S, const M3& F, const M3& R, float jp, float vol,
                                           P2GParticle& q) {
  const float je = m3_det(F);
  const float e = expf(S.hardening * (1.0f - jp));
  const float mu = S.mu0 * e;
  const float lam = S.lambda0 * e;
  M3 D;
#pragma unroll
  for (int c = 0; c < 3; c++)
#pragma unroll
    for (int r = 0; r < 3; r++) D.m[c][r] = F.m[c][r] - R.m[c][r];
  const M3 P = m3_mul_bt(D, F);  // (FE - R) FE^T
  const float s2 = lam * (je - 1.0f) * je;
  float a = 0.0f;
#pragma unroll
  for (int r = 0; r < 3; r++) {
#pragma unroll
    for (int c = 0; c < 3; c++) q.A[r][c] = -vol * (2.0f * mu * P.m[c][r] + (r == c ? s2 : 0.0f));
    a = fmaxf(a, fabsf(q.A[r][0]) + fabsf(q.A[r][1]) + fabsf(q.A[r][2]));
  }
  q.a = a;
  q.force = true;
}

// From the stored state: R by an SVD of F_E.
__device__ __forceinline__ P2GParticle p2g_particle(const SceneDev& S, int p, float4 xm, bool mass_only) {
  P2GParticle q;
  q.m = xm.w;
  q.force = false;
  q.a = 0.0f;
  q.mv[0] = q.mv[1] = q.mv[2] = 0.0f;
  if (mass_only) return q;
  const float4 vv = S.vv[p];
  q.mv[0] = q.m * vv.x;
  q.mv[1] = q.m * vv.y;
  q.mv[2] = q.m * vv.z;
  if (vv.w > 0.0f) {
    M3 F;
    float jp;
    load_fe(S, p, F, jp);
    M3 W, Sg, V;
    svd3<false>(F, W, Sg, V);
    p2g_stress(S, F, m3_mul_bt(W, V), jp, vv.w, q);
  }
  return q;
}

// The largest magnitude any of the particle's scaled contributions (and
// contribution terms) can take at scales sc (KIND kP2gMass: the mass alone);
// not finite for a non-finite particle.
template <int KIND>
__device__ __forceinline__ float fix_bound(const P2GParticle& q, const FixScale& sc) {
  float b = fabsf(q.m) * sc.m;
  if (KIND == kP2gFull) {
    const float mv = fmaxf(fabsf(q.mv[0]), fmaxf(fabsf(q.mv[1]), fabsf(q.mv[2])));
    b = fmaxf(b, mv * sc.p);
    if (q.force) b = fmaxf(b, q.a * sc.f);
  }
  return b * kWmax;
}

// The per-lane factors of one particle's contributions in stencil row
// (b, c), the same operations on every path: t1 = wy wz, t2 = gy wz,
// t3 = wy gz; mw = m_s t1, pv = mv_s t1, kk = A_s[r][0] t1,
// hh = A_s[r][1] t2 + A_s[r][2] t3 (scaled quantities, _s).
struct RowFactors {
  float mw, pv[3], kk[3], hh[3];
};
__device__ __forceinline__ void row_factors(float ms, const float mvs[3], const float As[3][3], float wyb, float gyb,
                                            float wzc, float gzc, bool mass_only, RowFactors& f) {
  const float t1 = __fmul_rn(wyb, wzc);
  f.mw = __fmul_rn(ms, t1);
  if (mass_only) return;
  const float t2 = __fmul_rn(gyb, wzc), t3 = __fmul_rn(wyb, gzc);
#pragma unroll
  for (int r = 0; r < 3; r++) {
    f.pv[r] = __fmul_rn(mvs[r], t1);
    f.kk[r] = __fmul_rn(As[r][0], t1);
    f.hh[r] = __fmaf_rn(As[r][1], t2, __fmul_rn(As[r][2], t3));
  }
}
// Rounded contributions (as magic-offset bits) at node x-weights (wxa, gxa).
__device__ __forceinline__ int fix_mass(float wxa, const RowFactors& f) {
  return __float_as_int(__fmaf_rn(wxa, f.mw, kMagic));
}
__device__ __forceinline__ int fix_mom(float wxa, const RowFactors& f, int r) {
  return __float_as_int(__fmaf_rn(wxa, f.pv[r], kMagic));
}
__device__ __forceinline__ int fix_force(float wxa, float gxa, const RowFactors& f, int r) {
  return __float_as_int(__fmaf_rn(gxa, f.kk[r], __fmaf_rn(wxa, f.hh[r], kMagic)));
}

// Scatter of one particle's 64 stencil nodes straight into acc (global
// atomics), for a particle outside its work item's tile. FAST: the particle
// fits the fast path's range and its contributions are rounded exactly as
// the tile path rounds them; otherwise (wide) each contribution is rounded in
// double precision to int64. ms, mvs, As: the scaled quantities.
template <int KIND, bool FAST>
__device__ __forceinline__ void scatter_fix(const SceneDev& S, float ms, const float mvs[3], const float As[3][3],
                                            const AxisW& w, const int base[3]) {
  constexpr bool mo = KIND == kP2gMass;
  for (int c = 0; c < 4; c++)
    for (int b = 0; b < 4; b++) {
      const int g1 = base[1] - 1 + b, g2 = base[2] - 1 + c;
      if (g1 < 0 || g2 < 0 || g1 >= S.dim[1] || g2 >= S.dim[2]) continue;
      RowFactors f;
      row_factors(ms, mvs, As, sel4(b, w.wy[0], w.wy[1], w.wy[2], w.wy[3]), sel4(b, w.gy[0], w.gy[1], w.gy[2], w.gy[3]),
                  sel4(c, w.wz[0], w.wz[1], w.wz[2], w.wz[3]), sel4(c, w.gz[0], w.gz[1], w.gz[2], w.gz[3]), mo, f);
      for (int a = 0; a < 4; a++) {
        const int g0 = base[0] - 1 + a;
        if (g0 < 0 || g0 >= S.dim[0]) continue;
        const float wxa = sel4(a, w.wx[0], w.wx[1], w.wx[2], w.wx[3]);
        const float gxa = sel4(a, w.gx[0], w.gx[1], w.gx[2], w.gx[3]);
        long long v[7] = {0, 0, 0, 0, 0, 0, 0};
        if (FAST) {
          v[0] = fix_mass(wxa, f) - kMagicBits;
          if (!mo)
#pragma unroll
            for (int r = 0; r < 3; r++) {
              v[1 + r] = fix_mom(wxa, f, r) - kMagicBits;
              v[4 + r] = fix_force(wxa, gxa, f, r) - kMagicBits;
            }
        } else {
          auto wide = [](double x) { return isfinite(x) && fabs(x) < 4.0e18 ? __double2ll_rn(x) : 0ll; };
          v[0] = wide((double)wxa * (double)f.mw);
          if (!mo)
#pragma unroll
            for (int r = 0; r < 3; r++) {
              v[1 + r] = wide((double)wxa * (double)f.pv[r]);
              const double h = (double)wide((double)wxa * (double)f.hh[r]);
              v[4 + r] = wide(fma((double)gxa, (double)f.kk[r], h));
            }
        }
        if (!(v[0] | v[1] | v[2] | v[3] | v[4] | v[5] | v[6])) continue;
        const int blk = block_id(S, g0 >> 2, g1 >> 2, g2 >> 2);
        acc_add(S, blk, (g0 & 3) + 4 * (g1 & 3) + 16 * (g2 & 3), v, mo);
        S.blk_flag[blk] = 1;
      }
    }
}

// The semi-implicit solve's K u scatter for a particle outside its tile:
// float sums into the low 4 bytes of acc's force words (free between the
// grid update and the next P2G; the solve's node passes read and clear them).
__device__ __forceinline__ void scatter_force(const SceneDev& S, const P2GParticle& q, const AxisW& w, const int base[3]) {
  if (!q.force) return;
  for (int c = 0; c < 4; c++)
    for (int b = 0; b < 4; b++)
      for (int a = 0; a < 4; a++) {
        const int g0 = base[0] - 1 + a, g1 = base[1] - 1 + b, g2 = base[2] - 1 + c;
        if (!node_in_grid(S, g0, g1, g2)) continue;
        const float wxa = sel4(a, w.wx[0], w.wx[1], w.wx[2], w.wx[3]);
        const float gxa = sel4(a, w.gx[0], w.gx[1], w.gx[2], w.gx[3]);
        const float wyb = sel4(b, w.wy[0], w.wy[1], w.wy[2], w.wy[3]);
        const float gyb = sel4(b, w.gy[0], w.gy[1], w.gy[2], w.gy[3]);
        const float wzc = sel4(c, w.wz[0], w.wz[1], w.wz[2], w.wz[3]);
        const float gzc = sel4(c, w.gz[0], w.gz[1], w.gz[2], w.gz[3]);
        const float gw[3] = {gxa * wyb * wzc, wxa * gyb * wzc, wxa * wyb * gzc};
        const int blk = block_id(S, g0 >> 2, g1 >> 2, g2 >> 2);
        if (__ldg(&S.blk_slot[blk]) < 0) continue;  // only active blocks' words are read and cleared by the solve
        float* dst = reinterpret_cast<float*>(S.acc + (size_t)blk * kAccBlockWords + 4 * kBlockNodes +
                                              (g0 & 3) + 4 * (g1 & 3) + 16 * (g2 & 3));
#pragma unroll
        for (int r = 0; r < 3; r++)
          atomicAdd(dst + 2 * r * kBlockNodes, q.A[r][0] * gw[0] + q.A[r][1] * gw[1] + q.A[r][2] * gw[2]);
      }
}

// ---- shared memory of one work item --------------------------------------
struct ItemShared {
  float stage[27][kOutBlockFloats];  // G2P: the pool blocks around the home block
  float4 pd[kItemMax][kPd];          // P2G: per-particle data, in tile-cell order
  union {
    int tilei[kAccFields * kTile3];  // P2G sums of the tile's nodes (fixed point: mass, momentum, force) ...
    float tile[kAccFields * kTile3]; // ... or float (the semi-implicit solve's K u)
  };
  int cstart[kCells + 1];            // first pd slot of each tile cell
  int ccount[kCells];                // particles per tile cell (zero between items)
  int wsum[kItemMax / 32];
  int wocc[kItemMax / 32];
  short cells[kCells];               // occupied tile cells
  int ncells;
  int4 item_q[2];                    // this and the next work item of the CTA
  int scene_q[2];                    // ... and their scenes
  int coll_scene;                    // scene whose colliders sit in coll
  FixScale fscale;                   // fixed-point scales of coll_scene's P2G in this launch
  unsigned seen[3];                  // largest mass, |v|, force-term bound of coll_scene's particles (bits) ...
  unsigned pushed[3];                // ... and the part of them already recorded in FixState
  int next_same;                     // the CTA's next work item continues this item's home-block run
  int next_issue;                    // ... or starts a run whose pool blocks the last warp copies
  int next_slot[32];                 // the pool slots of those blocks (lane k: tile block k)
  float run_bound;                   // sum of the contribution bounds of the particles in the tile's sums
  float item_bound;                  // ... and of this item's particles headed for the tile
  int abort;                         // 1 + parity of a copy wait that ran out, else 0
  uint64_t bar;
  snow_collider coll[kShColliders];
  float4 chit[kShColliders];         // packed hit tests of the colliders
  int ctype[kShColliders];
};

// Tile block k (0..26) around home block (bx, by, bz), or -1 outside the grid.
__device__ __forceinline__ int tile_block(const SceneDev& S, int bx, int by, int bz, int k) {
  const int cx = bx - 1 + k % 3, cy = by - 1 + (k / 3) % 3, cz = bz - 1 + k / 9;
  const bool in = cx >= 0 && cy >= 0 && cz >= 0 && cx < S.bdim[0] && cy < S.bdim[1] && cz < S.bdim[2];
  return in ? block_id(S, cx, cy, cz) : -1;
}

__device__ __forceinline__ void home_coords(const SceneDev& S, int blk, int& bx, int& by, int& bz) {
  bx = blk % S.bdim[0];
  by = (blk / S.bdim[0]) % S.bdim[1];
  bz = blk / (S.bdim[0] * S.bdim[1]);
}

// Pool slot of tile block k of item `it`; -1: no block.
__device__ __forceinline__ int tile_slot(const SceneDev& S, int4 it, int k) {
  if (k >= 27) return -1;
  int bx, by, bz;
  home_coords(S, it.x, bx, by, bz);
  const int b = tile_block(S, bx, by, bz, k);
  return b < 0 ? -1 : __ldg(&S.blk_slot[b]);
}

// One full warp issues the bulk copies (TMA) of the tile's pool blocks into
// `stage` (lane k < 27 copies block k, `block_floats` floats from pool slot
// `slot` of `pool`; block_floats <= 384 and a multiple of 4) and zero-fills
// the blocks without a slot; completion lands on sh.bar, which expects
// `unsent` bytes more than are copied (0 except in tests of the timeout
// path). The caller guarantees nobody reads `stage` until the barrier's
// phase completes and that all earlier reads of `stage` are done.
__device__ __forceinline__ void stage_issue(ItemShared& sh, const float* pool, int block_floats, int slot,
                                            uint32_t unsent) {
  const int k = threadIdx.x & 31;
  const bool mine = k < 27 && slot >= 0;
  const uint32_t bytes = (uint32_t)(block_floats * sizeof(float));
  const uint32_t valid = __ballot_sync(0xffffffffu, mine);
  if (k == 0) mbar_arrive_expect_tx(&sh.bar, __popc(valid) * bytes + unsent);
  __syncwarp();
  if (mine) {
    fence_proxy_async_smem();
    bulk_g2s(sh.stage[k], pool + (size_t)slot * block_floats, bytes, &sh.bar);
  }
  uint32_t missing = __ballot_sync(0xffffffffu, k < 27 && slot < 0);
  while (missing) {
    const int m = __ffs(missing) - 1;
    missing &= missing - 1;
    float4* dst = reinterpret_cast<float4*>(sh.stage[m]);
    for (int i = k; i < block_floats / 4; i += 32) dst[i] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  }
}
// ... of the grid update's output (v*, d).
__device__ __forceinline__ void stage_issue(ItemShared& sh, const SceneDev& S, int slot) {
  stage_issue(sh, S.gout, kOutBlockFloats, slot, S.tx_unsent);
}

// Every thread waits for the stage copies of the current phase, at most
// S.wait_ns. Returns false if the wait ran out; the thread then records the
// phase in sh.abort (1 + parity), and the CTA stops at its next barrier that
// checks it (stage_abort) without reading the stage.
__device__ __forceinline__ bool stage_wait(ItemShared& sh, const SceneDev& S, uint32_t& phase) {
  if (!mbar_wait(&sh.bar, phase, S.wait_ns)) {
    sh.abort = 1 + (int)phase;
    return false;
  }
  phase ^= 1u;
  return true;
}

// The end of a CTA whose copy wait ran out (every thread calls it, after a
// barrier that made sh.abort visible): the timeout is counted once (the host
// returns SNOW_ETIMEDOUT) and thread 0 gives the copies still in flight one
// more bounded wait, so the CTA does not exit while bulk copies into its
// shared memory may still land. Issues no copies.
__device__ __forceinline__ void stage_abort(ItemShared& sh, const SceneDev& S) {
  if (threadIdx.x == 0) {
    atomicAdd(&S.counters[CNT_TIMEOUT], 1);
    mbar_wait(&sh.bar, (uint32_t)(sh.abort - 1), S.wait_ns);
  }
}

// Colliders of scene S into shared memory (when they fit). Ends with
// __syncthreads.
__device__ __forceinline__ void load_colliders(ItemShared& sh, const SceneDev& S) {
  if (S.ncoll <= kShColliders && threadIdx.x < S.ncoll) {
    const snow_collider c = S.coll[threadIdx.x];
    sh.coll[threadIdx.x] = c;
    sh.ctype[threadIdx.x] = c.type;
    float4 h = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    if (c.type == 0)
      h = make_float4(c.normal[0], c.normal[1], c.normal[2],
                      fmaf(c.normal[2], c.pos[2], fmaf(c.normal[1], c.pos[1], c.normal[0] * c.pos[0])));
    else if (c.type == 1)
      h = make_float4(c.pos[0], c.pos[1], c.pos[2], c.radius * c.radius);
    sh.chit[threadIdx.x] = h;
  }
  __syncthreads();
}

// Zeroes the first nf fields of the P2G tile (at the start of each item,
// after the previous item's flush has read it).
__device__ __forceinline__ void tile_zero(ItemShared& sh, int nf) {
  static_assert(offsetof(ItemShared, tile) % 16 == 0, "tile must be 16-byte aligned");
  float4* t4 = reinterpret_cast<float4*>(sh.tile);
  const int n4 = nf * kTile3 / 4;
  for (int i = threadIdx.x; i < n4; i += blockDim.x) t4[i] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  for (int i = 4 * n4 + threadIdx.x; i < nf * kTile3; i += blockDim.x) sh.tile[i] = 0.0f;
}

// Kernel start: cell counts, flags and the bulk-copy barrier. Ends with
// __syncthreads.
__device__ __forceinline__ void tile_init(ItemShared& sh) {
  for (int i = threadIdx.x; i < kCells; i += blockDim.x) sh.ccount[i] = 0;
  if (threadIdx.x == 0) {
    mbar_init(&sh.bar, 1);
    sh.abort = 0;
    sh.run_bound = sh.item_bound = 0.0f;
  }
  __syncthreads();
}

// G2P sums of one particle: dv = sum_i w_ip d_i (PIC/FLIP increment,
// g2pTransfer.glsl:99-104) and L = sum_i v*_i (grad w_ip)^T (velocity
// gradient, :121-129), contracted along x first for each (y, z) row.
// node(a, b, c, v6) fills the 6 values (v*, d) of stencil node (a, b, c) or
// returns false for a node that contributes nothing.
template <class Node>
__device__ __forceinline__ void g2p_sums(const AxisW& w, Node node, float dv[3], float L[3][3]) {
#pragma unroll
  for (int r = 0; r < 3; r++) {
    dv[r] = 0.0f;
    L[r][0] = L[r][1] = L[r][2] = 0.0f;
  }
#pragma unroll
  for (int c = 0; c < 4; c++) {
#pragma unroll
    for (int b = 0; b < 4; b++) {
      float S1[3] = {0.0f, 0.0f, 0.0f}, S2[3] = {0.0f, 0.0f, 0.0f}, D[3] = {0.0f, 0.0f, 0.0f};
#pragma unroll
      for (int a = 0; a < 4; a++) {
        float v6[6];
        if (!node(a, b, c, v6)) continue;
#pragma unroll
        for (int r = 0; r < 3; r++) {
          S1[r] += w.wx[a] * v6[r];
          S2[r] += w.gx[a] * v6[r];
          D[r] += w.wx[a] * v6[3 + r];
        }
      }
      const float t1 = w.wy[b] * w.wz[c], t2 = w.gy[b] * w.wz[c], t3 = w.wy[b] * w.gz[c];
#pragma unroll
      for (int r = 0; r < 3; r++) {
        dv[r] += t1 * D[r];
        L[r][0] += t1 * S2[r];
        L[r][1] += t2 * S1[r];
        L[r][2] += t3 * S1[r];
      }
    }
  }
}

// Gather for particle at base cell `base` of the item at home block
// (bx, by, bz): from the staged tile when the stencil lies in it, else from
// the pool in global memory. Pool nodes are 6-float records (v*, d).
__device__ __forceinline__ void g2p_gather(const ItemShared& sh, const SceneDev& S, int bx, int by, int bz,
                                           const int base[3], const AxisW& w, float dv[3], float L[3][3]) {
  const int tx = base[0] - 1 - (4 * bx - 2), ty = base[1] - 1 - (4 * by - 2), tz = base[2] - 1 - (4 * bz - 2);
  if (tx >= 0 && ty >= 0 && tz >= 0 && tx <= kTile - 4 && ty <= kTile - 4 && tz <= kTile - 4) {
    // tile node t (0..8) lies in tile block floor((t + 2) / 4) at local (t + 2) & 3
    int X[4], Y[4], Z[4];
#pragma unroll
    for (int a = 0; a < 4; a++) {
      const int t = tx + a, q = ty + a, r = tz + a;
      X[a] = ((t + 2) >> 2) * kOutBlockFloats + kOutFields * ((t + 2) & 3);
      Y[a] = ((q + 2) >> 2) * 3 * kOutBlockFloats + kOutFields * 4 * ((q + 2) & 3);
      Z[a] = ((r + 2) >> 2) * 9 * kOutBlockFloats + kOutFields * 16 * ((r + 2) & 3);
    }
    const float* st = &sh.stage[0][0];
    g2p_sums(w,
             [&](int a, int b, int c, float v6[6]) {
               const float2* o = reinterpret_cast<const float2*>(st + X[a] + Y[b] + Z[c]);
               const float2 p0 = o[0], p1 = o[1], p2 = o[2];
               v6[0] = p0.x; v6[1] = p0.y; v6[2] = p1.x;
               v6[3] = p1.y; v6[4] = p2.x; v6[5] = p2.y;
               return true;
             },
             dv, L);
  } else {
    g2p_sums(w,
             [&](int a, int b, int c, float v6[6]) {
               const int g0 = base[0] - 1 + a, g1 = base[1] - 1 + b, g2 = base[2] - 1 + c;
               if (!node_in_grid(S, g0, g1, g2)) return false;
               const int sl = __ldg(&S.blk_slot[block_id(S, g0 >> 2, g1 >> 2, g2 >> 2)]);
               if (sl < 0) return false;
               const float* o = S.gout + (size_t)sl * kOutBlockFloats +
                                kOutFields * ((g0 & 3) + 4 * (g1 & 3) + 16 * (g2 & 3));
#pragma unroll
               for (int f = 0; f < 6; f++) v6[f] = __ldg(o + f);
               return true;
             },
             dv, L);
  }
}

// Position and velocity of one particle, loaded ahead of the gather.
struct PState {
  float4 xm, vv;
};

__device__ __forceinline__ PState load_state(const SceneDev& S, int p, bool binned) {
  PState t;
  t.xm = __ldcs((binned ? S.bxm : S.xm) + p);
  t.vv = __ldcs((binned ? S.bvv : S.vv) + p);
  return t;
}

// particleAdvance.glsl:87-210 for particle p given its G2P sums; stores the
// new state and returns it with the rotation R = W V^T of the SVD.
struct Advanced {
  float4 xm, vv;
  M3 fe, R;
  float jp;
};

// F_E, J_p and the previous SVD frame of one particle.
struct PDef {
  float4 fa, fb, vq;
  float2 fc;
};

__device__ __forceinline__ PDef load_def(const SceneDev& S, int p, bool binned) {
  PDef d;
  d.fa = __ldcs((binned ? S.bfa : S.fa) + p);
  d.fb = __ldcs((binned ? S.bfb : S.fb) + p);
  d.vq = __ldcs((binned ? S.bvq : S.vq) + p);
  d.fc = __ldcs((binned ? S.bfc : S.fc) + p);
  return d;
}

__device__ __forceinline__ void advance_particle(const SceneDev& S, int p, const PState& ps, const PDef& def,
                                                 const float dv[3], const float L[3][3], const ItemShared& sh,
                                                 Advanced& out) {
  M3 FE;
  FE.m[0][0] = def.fa.x; FE.m[0][1] = def.fa.y; FE.m[0][2] = def.fa.z;
  FE.m[1][0] = def.fa.w; FE.m[1][1] = def.fb.x; FE.m[1][2] = def.fb.y;
  FE.m[2][0] = def.fb.z; FE.m[2][1] = def.fb.w; FE.m[2][2] = def.fc.x;
  const float jp = def.fc.y;
  float4 xm = ps.xm, vv = ps.vv;
  M3 step;
#pragma unroll
  for (int c = 0; c < 3; c++)
#pragma unroll
    for (int r = 0; r < 3; r++) step.m[c][r] = (c == r ? 1.0f : 0.0f) + S.dt * L[r][c];
  const M3 fe_trial = m3_mul(step, FE);
  M3 V;
  float lam[3];
  float q[4] = {def.vq.x, def.vq.y, def.vq.z, def.vq.w};
  eigen_warm(fe_trial, q, V, lam);
  __stcs(&S.vq[p], make_float4(q[0], q[1], q[2], q[3]));
  // With FE_trial = W S V^T and B = FE_trial V = W S (columns of norm
  // sigma_i), the clamped F_E' = W clamp(S) V^T = B diag(clamp(sigma)/sigma) V^T
  // and the polar rotation R = W V^T = B diag(1/sigma) V^T: the sort and QR
  // of the shader's SVD (which only serve to find W) are not needed here.
  const M3 B = m3_mul(fe_trial, V);
  M3 Br, Bc;
  float ratio = 1.0f;
  bool clamped = false;
#pragma unroll
  for (int c = 0; c < 3; c++) {
    const float inv = rsqrt_nr(fmaxf(lam[c], 1e-30f));
    const float sig = lam[c] * inv;
    const float cl = fminf(fmaxf(sig, S.crit_lo), S.crit_hi);
    clamped = clamped || cl != sig;
    ratio *= __fdividef(sig, cl);
    const float sc = cl * inv;
#pragma unroll
    for (int r = 0; r < 3; r++) {
      Br.m[c][r] = B.m[c][r] * inv;
      Bc.m[c][r] = B.m[c][r] * sc;
    }
  }
  out.R = m3_mul_bt(Br, V);
  // no singular value clamped: F_E' = FE_trial exactly, J_p unchanged
  out.fe = clamped ? m3_mul_bt(Bc, V) : fe_trial;
  // det F_P' = det F_P * det(FE_trial) / det(FE'): the shader's
  // F_P' = V S^-1 W^T (I + dt L) FE FP (particleAdvance.glsl:132) has this
  // determinant; only det F_P is ever read (p2gTransfer.glsl:119).
  out.jp = clamped ? jp * ratio : jp;
  float v[3] = {S.alpha * vv.x + dv[0], S.alpha * vv.y + dv[1], S.alpha * vv.z + dv[2]};
  const float xold[3] = {xm.x, xm.y, xm.z};
  if (S.ncoll <= kShColliders)
    collide_packed(sh.coll, sh.chit, sh.ctype, S.ncoll, xold, v);
  else
    collide(S.coll, S.ncoll, xold, v);
  xm.x += S.dt * v[0];
  xm.y += S.dt * v[1];
  xm.z += S.dt * v[2];
  vv.x = v[0];
  vv.y = v[1];
  vv.z = v[2];
  __stcs(&S.xm[p], xm);
  __stcs(&S.vv[p], vv);
  store_fe(S, p, out.fe, out.jp);
  out.xm = xm;
  out.vv = vv;
  bool finite = isfinite(xm.x) && isfinite(xm.y) && isfinite(xm.z) && isfinite(v[0]) && isfinite(v[1]) &&
                isfinite(v[2]) && isfinite(out.jp);
#pragma unroll
  for (int c = 0; c < 3; c++)
#pragma unroll
    for (int r = 0; r < 3; r++) finite = finite && isfinite(out.fe.m[c][r]);
  if (!finite) atomicAdd(&S.counters[CNT_NONFINITE], 1);
}

// Adds the particles of one tile cell (list slots j0..j1) to this lane's
// x-row (b, c) of the cell's 4x4x4 stencil: acc[a] holds node x = lx + a.
// The semi-implicit solve's K u (float sums of A grad w).
__device__ __forceinline__ void cell_sums_force(const ItemShared& sh, int j0, int j1, int b, int c,
                                                float (&acc)[4][kAccFields]) {
  for (int j = j0; j < j1; j++) {
    const float4* d = sh.pd[j];
    const float* df = reinterpret_cast<const float*>(d);
    const float4 w4 = d[4], g4 = d[5];
    const float wxa[4] = {w4.x, w4.y, w4.z, w4.w};
    const float gxa[4] = {g4.x, g4.y, g4.z, g4.w};
    const float wyb = df[6 * 4 + b], wzc = df[8 * 4 + c];
    const float gyb = df[7 * 4 + b], gzc = df[9 * 4 + c];
    const float t1 = wyb * wzc, t2 = gyb * wzc, t3 = wyb * gzc;
    const float4 a1 = d[1], a2 = d[2];
    const float a22 = df[3 * 4];
    // A rows: r0 = (a1.x a1.y a1.z), r1 = (a1.w a2.x a2.y), r2 = (a2.z a2.w a22)
    const float kk[3] = {a1.x * t1, a1.w * t1, a2.z * t1};
    const float hh[3] = {a1.y * t2 + a1.z * t3, a2.x * t2 + a2.y * t3, a2.w * t2 + a22 * t3};
#pragma unroll
    for (int a = 0; a < 4; a++)
#pragma unroll
      for (int r = 0; r < 3; r++) acc[a][r] += gxa[a] * kk[r] + wxa[a] * hh[r];
  }
}

// The same for the fixed-point sums (mass alone, or mass, momentum and force):
// each contribution is rounded by the magic-offset FMA (fix_mass, fix_mom,
// fix_force) and its bits are added to the unsigned accumulators, so every
// accumulator gains kMagicBits per particle; np counts the particles summed.
template <int KIND>
__device__ __forceinline__ void cell_sums_fix(const ItemShared& sh, int j0, int j1, int b, int c,
                                              unsigned (&acc)[4][kAccFields], int& np) {
  constexpr bool mo = KIND == kP2gMass;
  for (int j = j0; j < j1; j++, np++) {
    const float4* d = sh.pd[j];
    const float* df = reinterpret_cast<const float*>(d);
    const float4 w4 = d[4];
    const float wxa[4] = {w4.x, w4.y, w4.z, w4.w};
    const float4 d0 = d[0];
    const float mvs[3] = {d0.y, d0.z, d0.w};
    float As[3][3] = {{0.0f, 0.0f, 0.0f}, {0.0f, 0.0f, 0.0f}, {0.0f, 0.0f, 0.0f}};
    float gyb = 0.0f, gzc = 0.0f;
    float gxa[4] = {0.0f, 0.0f, 0.0f, 0.0f};
    if (!mo) {
      const float4 a1 = d[1], a2 = d[2], g4 = d[5];
      As[0][0] = a1.x; As[0][1] = a1.y; As[0][2] = a1.z;
      As[1][0] = a1.w; As[1][1] = a2.x; As[1][2] = a2.y;
      As[2][0] = a2.z; As[2][1] = a2.w; As[2][2] = df[3 * 4];
      gyb = df[7 * 4 + b];
      gzc = df[9 * 4 + c];
      gxa[0] = g4.x; gxa[1] = g4.y; gxa[2] = g4.z; gxa[3] = g4.w;
    }
    RowFactors f;
    row_factors(d0.x, mvs, As, df[6 * 4 + b], gyb, df[8 * 4 + c], gzc, mo, f);
#pragma unroll
    for (int a = 0; a < 4; a++) {
      acc[a][0] += (unsigned)fix_mass(wxa[a], f);
      if (mo) continue;
#pragma unroll
      for (int r = 0; r < 3; r++) {
        acc[a][1 + r] += (unsigned)fix_mom(wxa[a], f, r);
        acc[a][4 + r] += (unsigned)fix_force(wxa[a], gxa[a], f, r);
      }
    }
  }
}

// Adds the 4 nodes of this lane's row (tile nodes t0 .. t0 + 3) to the
// shared tile and clears them (float sums).
template <int NF>
__device__ __forceinline__ void row_flush(ItemShared& sh, int t0, float (&acc)[4][kAccFields]) {
#pragma unroll
  for (int a = 0; a < 4; a++) {
#pragma unroll
    for (int f = 0; f < NF; f++) {
      atomicAdd(&sh.tile[f * kTile3 + t0 + a], acc[a][f]);
      acc[a][f] = 0.0f;
    }
  }
}
// ... fixed-point sums: `base` = np kMagicBits, the offset every accumulator
// carries (a cleared accumulator restarts at it).
template <int NF>
__device__ __forceinline__ void row_flush_fix(ItemShared& sh, int t0, unsigned (&acc)[4][kAccFields], unsigned base) {
#pragma unroll
  for (int a = 0; a < 4; a++) {
#pragma unroll
    for (int f = 0; f < NF; f++) {
      atomicAdd(&sh.tilei[f * kTile3 + t0 + a], (int)(acc[a][f] - base));
      acc[a][f] = base;
    }
  }
}

__device__ __forceinline__ int cell_row_node(int ci, int b, int c) {
  const int lx = ci % kCellsPerAxis, ly = (ci / kCellsPerAxis) % kCellsPerAxis, lz = ci / (kCellsPerAxis * kCellsPerAxis);
  return lx + kTile * (ly + b) + kTile * kTile * (lz + c);
}

// P2G of the item's particles into the shared tile (every thread of the CTA
// calls it; thread i holds particle i of the item when `have`):
//   1. each particle inside the tile whose contributions fit the fast
//      path's range counts itself in its base cell; the others scatter
//      straight to acc (scatter_fix; K u: scatter_force);
//   2. a scan of the cell counts gives each cell its first slot and lists the
//      occupied cells; each particle stores its (scaled) mass, momentum, A
//      and axis weights at its slot, so the particles lie in tile-cell order;
//   3. each half-warp owns one occupied cell at a time: lane l sums the
//      x-row (b, c) = (l & 3, l >> 2) of the cell's stencil over the cell's
//      particles in registers and adds the row to the shared tile.
// The tile keeps accumulating until p2g_tile_flush adds it to acc, so the
// items of one home block can share it. Returns false (at its first barrier,
// before any write beyond the cell counts and the straight scatters) when a
// copy wait of the CTA ran out (sh.abort): the caller then stops the CTA.
// RUN: the tile may already hold earlier items' sums (sh.run_bound bounds
// them); when this item's particles could take a sum past kTileSumBound, the
// tile is first added to acc and cleared. Ends with a barrier.
template <int KIND>
__device__ __forceinline__ void p2g_tile_flush(ItemShared& sh, const SceneDev& S, int bx, int by, int bz);
template <int KIND, bool RUN = false>
__device__ __forceinline__ bool p2g_tile_accumulate(ItemShared& sh, const SceneDev& S, int bx, int by, int bz,
                                                    bool have, const P2GParticle& q, const AxisW& w,
                                                    const int base[3], const FixScale& sc) {
  constexpr int nf = P2gFields<KIND>::nf;
  constexpr bool fix = KIND != kP2gForce;
  const int ox = 4 * bx - 2, oy = 4 * by - 2, oz = 4 * bz - 2;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int my_cell = -1, my_rank = 0;
  float tile_bound = 0.0f;  // the particle's contribution bound, if it goes to the tile
  // the particle's quantities as the tile stores them (fixed point: scaled)
  float ms = 0.0f, mvs[3] = {0.0f, 0.0f, 0.0f}, As[3][3];
#pragma unroll
  for (int r = 0; r < 3; r++)
#pragma unroll
    for (int c = 0; c < 3; c++) As[r][c] = fix ? (q.force ? q.A[r][c] * sc.f : 0.0f) : q.A[r][c];
  if (fix) {
    ms = q.m * sc.m;
#pragma unroll
    for (int r = 0; r < 3; r++) mvs[r] = q.mv[r] * sc.p;
  }
  if (have) {
    const float bound = fix ? fix_bound<KIND>(q, sc) : 0.0f;
    const bool fast = !fix || bound < kFastLimit;  // false for a non-finite particle as well
    const int lx = base[0] - 1 - ox, ly = base[1] - 1 - oy, lz = base[2] - 1 - oz;
    const bool inside = lx >= 0 && ly >= 0 && lz >= 0 && lx < kCellsPerAxis && ly < kCellsPerAxis && lz < kCellsPerAxis;
    if (inside && fast) {
      my_cell = lx + kCellsPerAxis * ly + kCellsPerAxis * kCellsPerAxis * lz;
      my_rank = atomicAdd(&sh.ccount[my_cell], 1);
      tile_bound = bound;
    } else {
      // the particle drifted out of its home block's tile since the last
      // binning, or outgrew the fast path's range
      if (!inside) atomicAdd(&S.counters[CNT_FALLBACK], 1);
      if (!fix)
        scatter_force(S, q, w, base);
      else if (fast)
        scatter_fix<KIND, true>(S, ms, mvs, As, w, base);
      else {
        atomicAdd(&S.fix->wide, 1u);
        scatter_fix<KIND, false>(S, ms, mvs, As, w, base);
      }
    }
  }
  if (RUN) {  // per warp: its tile particles times their largest bound (no lower than their sum)
    const uint32_t in = __ballot_sync(0xffffffffu, my_cell >= 0);
    const float bmax = __uint_as_float(__reduce_max_sync(0xffffffffu, __float_as_uint(tile_bound)));
    if (lane == 0 && in) atomicAdd(&sh.item_bound, (float)__popc(in) * bmax);
  }
  __syncthreads();  // counts done
  if (sh.abort) return false;  // a copy wait ran out
  if (RUN && sh.run_bound + sh.item_bound > kTileSumBound) {  // uniform across the CTA
    // this item's sums could wrap the tile's int32 sums: the earlier items'
    // go to acc first (integer sums: the split changes no bit of the result)
    p2g_tile_flush<KIND>(sh, S, bx, by, bz);
    __syncthreads();
    if (threadIdx.x == 0) sh.run_bound = 0.0f;
    tile_zero(sh, nf);
  }
  // exclusive scan of the cell counts and list of the occupied cells, one
  // cell per thread
  const int t = threadIdx.x;
  const int cnt = t < kCells ? sh.ccount[t] : 0;
  int incl = cnt;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int v = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += v;
  }
  const uint32_t occ = __ballot_sync(0xffffffffu, cnt > 0);
  if (lane == 31) {
    sh.wsum[warp] = incl;
    sh.wocc[warp] = __popc(occ);
  }
  __syncthreads();
  int off = 0, ooff = 0;
  for (int k = 0; k < warp; k++) {
    off += sh.wsum[k];
    ooff += sh.wocc[k];
  }
  if (t < kCells) {
    sh.cstart[t] = off + incl - cnt;
    sh.ccount[t] = 0;
    if (cnt > 0) sh.cells[ooff + __popc(occ & ((1u << lane) - 1u))] = (short)t;
  }
  if (t == kCells - 1) sh.cstart[kCells] = off + incl;
  if (t == blockDim.x - 1) sh.ncells = ooff + __popc(occ);
  if (RUN && t == 0) {  // every thread has read both bounds (two barriers ago)
    sh.run_bound += sh.item_bound;
    sh.item_bound = 0.0f;
  }
  __syncthreads();
  if (my_cell >= 0) {
    // the particle's P2G data, stored in tile-cell order
    float4* d = sh.pd[sh.cstart[my_cell] + my_rank];
    const bool f = KIND != kP2gMass && q.force;
    if (KIND == kP2gMass)
      d[0] = make_float4(ms, 0.0f, 0.0f, 0.0f);
    else if (KIND == kP2gFull)
      d[0] = make_float4(ms, mvs[0], mvs[1], mvs[2]);
    d[1] = f ? make_float4(As[0][0], As[0][1], As[0][2], As[1][0]) : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    d[2] = f ? make_float4(As[1][1], As[1][2], As[2][0], As[2][1]) : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    d[3] = make_float4(f ? As[2][2] : 0.0f, __int_as_float(my_cell), 0.0f, 0.0f);
    d[4] = make_float4(w.wx[0], w.wx[1], w.wx[2], w.wx[3]);
    d[5] = make_float4(w.gx[0], w.gx[1], w.gx[2], w.gx[3]);
    d[6] = make_float4(w.wy[0], w.wy[1], w.wy[2], w.wy[3]);
    d[7] = make_float4(w.gy[0], w.gy[1], w.gy[2], w.gy[3]);
    d[8] = make_float4(w.wz[0], w.wz[1], w.wz[2], w.wz[3]);
    d[9] = make_float4(w.gz[0], w.gz[1], w.gz[2], w.gz[3]);
  }
  __syncthreads();
  {
    // half-warp h takes a contiguous slice of the occupied-cell list (the
    // two halves of a warp get neighbouring slices, whose particle counts
    // are alike). Cells of a slice often follow each other along x: the
    // row's sums then slide one node instead of being flushed, so only the
    // node that leaves the window goes to the shared tile.
    constexpr int NF = nf;
    const int hw = threadIdx.x >> 4, l16 = threadIdx.x & 15;
    const int b = l16 & 3, c = l16 >> 2;
    const int nhw = blockDim.x >> 4;
    const int ncells = sh.ncells;
    const int k0 = (ncells * hw) / nhw, k1 = (ncells * (hw + 1)) / nhw;
    int cur = -1;
    if (fix) {
      unsigned acc[4][kAccFields];
#pragma unroll
      for (int a = 0; a < 4; a++)
#pragma unroll
        for (int f = 0; f < kAccFields; f++) acc[a][f] = 0u;
      int np = 0;
      for (int k = k0; k < k1; k++) {
        const int ci = sh.cells[k];
        if (cur >= 0) {
          const unsigned base_bits = (unsigned)np * (unsigned)kMagicBits;
          if (ci == cur + 1 && ci % kCellsPerAxis != 0) {
            // only node 0 leaves the window: flush it, slide the rest
#pragma unroll
            for (int f = 0; f < NF; f++) {
              atomicAdd(&sh.tilei[f * kTile3 + cell_row_node(cur, b, c)], (int)(acc[0][f] - base_bits));
              acc[0][f] = acc[1][f];
              acc[1][f] = acc[2][f];
              acc[2][f] = acc[3][f];
              acc[3][f] = base_bits;
            }
          } else {
            row_flush_fix<NF>(sh, cell_row_node(cur, b, c), acc, base_bits);
          }
        }
        cell_sums_fix<KIND>(sh, sh.cstart[ci], sh.cstart[ci + 1], b, c, acc, np);
        cur = ci;
      }
      if (cur >= 0) row_flush_fix<NF>(sh, cell_row_node(cur, b, c), acc, (unsigned)np * (unsigned)kMagicBits);
    } else {
      float acc[4][kAccFields];
#pragma unroll
      for (int a = 0; a < 4; a++)
#pragma unroll
        for (int f = 0; f < kAccFields; f++) acc[a][f] = 0.0f;
      for (int k = k0; k < k1; k++) {
        const int ci = sh.cells[k];
        if (cur >= 0) {
          if (ci == cur + 1 && ci % kCellsPerAxis != 0) {
#pragma unroll
            for (int f = 0; f < NF; f++) {
              atomicAdd(&sh.tile[f * kTile3 + cell_row_node(cur, b, c)], acc[0][f]);
              acc[0][f] = acc[1][f];
              acc[1][f] = acc[2][f];
              acc[2][f] = acc[3][f];
              acc[3][f] = 0.0f;
            }
          } else {
            row_flush<NF>(sh, cell_row_node(cur, b, c), acc);
          }
        }
        cell_sums_force(sh, sh.cstart[ci], sh.cstart[ci + 1], b, c, acc);
        cur = ci;
      }
      if (cur >= 0) row_flush<NF>(sh, cell_row_node(cur, b, c), acc);
    }
  }
  __syncthreads();
  return true;
}

// Adds the tile's non-zero nodes that lie in the grid to acc and flags
// their blocks (fixed point: each node's non-zero sums into its int64
// words; K u: three float adds into the force words of blocks active in
// this step). One tile node per thread, x fastest, so consecutive threads
// add to consecutive words. Every thread of the CTA calls it after
// p2g_tile_accumulate's closing barrier; the caller separates it from the
// next use of the tile with a barrier.
template <int KIND>
__device__ __forceinline__ void p2g_tile_flush(ItemShared& sh, const SceneDev& S, int bx, int by, int bz) {
  constexpr int nf = P2gFields<KIND>::nf;
  const int ox = 4 * bx - 2, oy = 4 * by - 2, oz = 4 * bz - 2;
  for (int t = threadIdx.x; t < kTile3; t += blockDim.x) {
    const int x = t % kTile, y = (t / kTile) % kTile, z = t / (kTile * kTile);
    const int g0 = ox + x, g1 = oy + y, g2 = oz + z;
    if (g0 < 0 || g1 < 0 || g2 < 0 || g0 >= S.dim[0] || g1 >= S.dim[1] || g2 >= S.dim[2]) continue;
    int v[nf];
    int any = 0;
#pragma unroll
    for (int f = 0; f < nf; f++) {
      v[f] = sh.tilei[f * kTile3 + t];  // float K u: its bits (zero for 0.0f)
      any |= v[f];
    }
    if (!any) continue;
    const int blk = block_id(S, g0 >> 2, g1 >> 2, g2 >> 2);
    unsigned long long* a = S.acc + (size_t)blk * kAccBlockWords + (g0 & 3) + 4 * (g1 & 3) + 16 * (g2 & 3);
    if (KIND == kP2gForce) {
      // K u goes only to blocks active in this step: the solve's node passes
      // read and clear the words of those alone (a block whose fixed-point
      // sums all rounded to zero is not active, although its K u may not be)
      if (__ldg(&S.blk_slot[blk]) < 0) continue;
      float* fw = reinterpret_cast<float*>(a + 4 * kBlockNodes);
#pragma unroll
      for (int f = 0; f < 3; f++) atomicAdd(fw + 2 * f * kBlockNodes, __int_as_float(v[f]));
      continue;
    }
#pragma unroll
    for (int f = 0; f < nf; f++)
      if (v[f]) atomicAdd(a + f * kBlockNodes, (unsigned long long)(long long)v[f]);
    S.blk_flag[blk] = 1;
  }
}
}  // namespace
}  // namespace snow
