// ORACLE / TEST INFRASTRUCTURE ONLY. The product never links, loads or calls
// this file: tests/, __graft_entry__.smoke() and bench.py's CPU baseline use
// it to check results and to time the CPU.
//
// A CPU restatement of the snow reference's explicit MPM step (the GLSL
// compute shaders under shader/compute/), written independently of them and
// templated on
//   Real  : float or double arithmetic;
//   FIXED : true  -> the shaders' int32 fixed-point storage and accumulation
//                    (mass/momentum x1e8, force x1e6, velocity x1e8, density
//                    x1e6, each contribution truncated toward zero);
//           false -> plain Real sums, no quantisation.
// Two more switches follow the shaders' own rounding steps:
//   vround : V rounded to 1e-5 inside the SVD   (SVD.include.glsl:354-358)
//   qround : R, F_E, F_P rounded to 1e-9         (p2gTransfer.glsl:112-116,
//                                                 particleAdvance.glsl:120-140)
// Modes exported:
//   ORACLE_FAITHFUL32 : float, FIXED, vround, qround. Follows the shaders
//                       operation by operation; it agrees to the bit with the
//                       reference's shaders compiled as C++ (oracle/_ref).
//   ORACLE_EXACT64    : double, no fixed point, rounding switchable. The
//                       FP64 oracle for the FP32 GPU path's error budget.
//   ORACLE_EXACT32    : float, no fixed point (diagnostics).
//
// Parity is pinned by tests/golden/*.npz, produced by the reference's own
// shader code run through oracle/_ref (tests/golden/make_golden.py).
//
// Each routine names the reference file:line it restates. Implementation-
// defined GLSL built-ins (round, inversesqrt, determinant, normalize) come from
// glsl_builtins.hpp, the same definitions the compiled reference uses.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <numeric>
#include <vector>

#include "glsl_builtins.hpp"

namespace {

using glslb::g_exp;
using glslb::g_inversesqrt;
using glslb::g_max;
using glslb::g_round;

// ---- small column-major 3-vector / 3x3 types (m[c][r]) -----------------
template <class R>
struct V3 {
  R v[3];
  R& operator[](int i) { return v[i]; }
  const R& operator[](int i) const { return v[i]; }
};
template <class R>
struct M3 {
  V3<R> c[3];
  V3<R>& operator[](int i) { return c[i]; }
  const V3<R>& operator[](int i) const { return c[i]; }
};

template <class R> inline V3<R> v3(R a, R b, R c) { return V3<R>{{a, b, c}}; }
template <class R> inline V3<R> vadd(const V3<R>& a, const V3<R>& b) { return v3<R>(a[0] + b[0], a[1] + b[1], a[2] + b[2]); }
template <class R> inline V3<R> vsub(const V3<R>& a, const V3<R>& b) { return v3<R>(a[0] - b[0], a[1] - b[1], a[2] - b[2]); }
template <class R> inline V3<R> vneg(const V3<R>& a) { return v3<R>(-a[0], -a[1], -a[2]); }
template <class R> inline V3<R> smul(R s, const V3<R>& a) { return v3<R>(s * a[0], s * a[1], s * a[2]); }
template <class R> inline V3<R> muls(const V3<R>& a, R s) { return v3<R>(a[0] * s, a[1] * s, a[2] * s); }
template <class R> inline V3<R> divs(const V3<R>& a, R s) { return v3<R>(a[0] / s, a[1] / s, a[2] / s); }
template <class R> inline R dot3(const V3<R>& a, const V3<R>& b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
template <class R> inline R len3(const V3<R>& a) { return std::sqrt(dot3(a, a)); }

template <class R> inline M3<R> mdiag(R s) {
  M3<R> m;
  for (int c = 0; c < 3; c++)
    for (int r = 0; r < 3; r++) m[c][r] = (c == r) ? s : R(0);
  return m;
}
template <class R> inline M3<R> mcols(const V3<R>& a, const V3<R>& b, const V3<R>& c) {
  M3<R> m;
  m[0] = a; m[1] = b; m[2] = c;
  return m;
}
template <class R> inline M3<R> madd(const M3<R>& a, const M3<R>& b) {
  M3<R> m;
  for (int c = 0; c < 3; c++) m[c] = vadd(a[c], b[c]);
  return m;
}
template <class R> inline M3<R> msub(const M3<R>& a, const M3<R>& b) {
  M3<R> m;
  for (int c = 0; c < 3; c++) m[c] = vsub(a[c], b[c]);
  return m;
}
template <class R> inline M3<R> msmul(R s, const M3<R>& a) {
  M3<R> m;
  for (int c = 0; c < 3; c++) m[c] = smul(s, a[c]);
  return m;
}
// (A*B)[c][r] = sum_k A[k][r] * B[c][k], k = 0, 1, 2 in order.
template <class R> inline M3<R> mmul(const M3<R>& a, const M3<R>& b) {
  M3<R> m;
  for (int c = 0; c < 3; c++)
    for (int r = 0; r < 3; r++) m[c][r] = a[0][r] * b[c][0] + a[1][r] * b[c][1] + a[2][r] * b[c][2];
  return m;
}
template <class R> inline V3<R> mvmul(const M3<R>& a, const V3<R>& v) {
  V3<R> o;
  for (int r = 0; r < 3; r++) o[r] = a[0][r] * v[0] + a[1][r] * v[1] + a[2][r] * v[2];
  return o;
}
template <class R> inline M3<R> mtrans(const M3<R>& a) {
  M3<R> m;
  for (int c = 0; c < 3; c++)
    for (int r = 0; r < 3; r++) m[c][r] = a[r][c];
  return m;
}
template <class R> inline R mdet(const M3<R>& m) { return glslb::det3_cm<M3<R>, R>(m); }

template <class R> inline R rnd_q(R x, R scale) { return g_round(scale * x) / scale; }

// ---- cubic B-spline, cubic.include.glsl:7-40 ----------------------------
template <class R> inline R bspline(R x) {
  const R ax = std::fabs(x);
  if (ax < R(1)) return R(0.5) * ax * ax * ax - x * x + R(2) / R(3);
  if (ax < R(2)) return -R(1) / R(6) * ax * ax * ax + x * x - R(2) * ax + R(4) / R(3);
  return R(0);
}
template <class R> inline R bspline_d(R x) {
  const R ax = std::fabs(x);
  if (ax < R(1)) return R(1.5) * x * ax - R(2) * x;
  if (ax < R(2)) return -R(1) / R(2) * ax * x + R(2) * x - R(2) * x / ax;
  return R(0);
}
template <class R> inline R weight3(const V3<R>& d) { return bspline(d[0]) * bspline(d[1]) * bspline(d[2]); }
template <class R> inline V3<R> weight3_grad(const V3<R>& d) {
  return v3<R>(bspline_d(d[0]) * bspline(d[1]) * bspline(d[2]),
               bspline(d[0]) * bspline_d(d[1]) * bspline(d[2]),
               bspline(d[0]) * bspline(d[1]) * bspline_d(d[2]));
}

// ---- 3x3 SVD: quaternion Jacobi on A^T A, sort, Givens QR ---------------
// Restates SVD.include.glsl (McAdams et al. 2011, "Computing the singular
// value decomposition of 3x3 matrices with minimal branching"): constants
// :20-23, Jacobi step :71-128, 4 sweeps :130-162, sort :191-228, QR :231-332,
// computeSVD :334-371, computePD :374-385.
template <class R> struct SvdConst {
  static R gamma() { return R(5.828427124); }
  static R cstar() { return R(0.923879532); }
  static R sstar() { return R(0.3826834323); }
  static R eps() { return R(1e-6); }
};

template <class R> inline M3<R> quat_to_mat(const R q[4]) {
  const R qxx = q[1] * q[1], qyy = q[2] * q[2], qzz = q[3] * q[3];
  const R qxz = q[1] * q[3], qxy = q[1] * q[2], qyz = q[2] * q[3];
  const R qwx = q[0] * q[1], qwy = q[0] * q[2], qwz = q[0] * q[3];
  M3<R> m;
  m[0][0] = R(1) - R(2) * (qyy + qzz);
  m[0][1] = R(2) * (qxy + qwz);
  m[0][2] = R(2) * (qxz - qwy);
  m[1][0] = R(2) * (qxy - qwz);
  m[1][1] = R(1) - R(2) * (qxx + qzz);
  m[1][2] = R(2) * (qyz + qwx);
  m[2][0] = R(2) * (qxz + qwy);
  m[2][1] = R(2) * (qyz - qwx);
  m[2][2] = R(1) - R(2) * (qxx + qyy);
  return m;
}

// One approximate Givens conjugation eliminating S(0,1); the matrix comes back
// cyclically relabelled so the next call works on the next pair.
template <class R> inline void jacobi_step(int x, int y, int z, M3<R>& S, R q[4]) {
  R ch = R(2) * (S[0][0] - S[1][1]);
  R ch2 = ch * ch;
  R sh = S[0][1];
  R sh2 = sh * sh;
  const bool exact = SvdConst<R>::gamma() * sh2 < ch2;
  if (exact) {
    const R w = g_inversesqrt(ch2 + sh2);
    ch = w * ch;
    sh = w * sh;
  } else {
    ch = SvdConst<R>::cstar();
    sh = SvdConst<R>::sstar();
  }
  ch2 = ch * ch;
  sh2 = sh * sh;
  const R scale = R(1) / (ch2 + sh2);
  const R a = (ch2 - sh2) * scale;
  const R b = (R(2) * sh * ch) * scale;
  const R a2 = a * a, b2 = b * b, ab = a * b;
  const R s0 = a2 * S[0][0] + R(2) * ab * S[1][0] + b2 * S[1][1];
  const R s2 = a * S[2][0] + b * S[2][1];
  const R s3 = (a2 - b2) * S[1][0] + ab * (S[1][1] - S[0][0]);
  const R s4 = b2 * S[0][0] - R(2) * ab * S[1][0] + a2 * S[1][1];
  const R s5 = a * S[1][2] - b * S[0][2];
  const R s8 = S[2][2];
  S[0] = v3<R>(s4, s5, s3);
  S[1] = v3<R>(s5, s8, s2);
  S[2] = v3<R>(s3, s2, s0);
  const R t[3] = {sh * q[1], sh * q[2], sh * q[3]};
  sh *= q[0];
  for (int i = 0; i < 4; i++) q[i] *= ch;
  q[z + 1] += sh;
  q[0] -= t[z];
  q[x + 1] += t[y];
  q[y + 1] -= t[x];
}

template <class R> inline void jacobi_eigen(M3<R>& S, R q[4]) {
  q[0] = R(1); q[1] = R(0); q[2] = R(0); q[3] = R(0);
  for (int sweep = 0; sweep < 4; sweep++) {
    jacobi_step<R>(0, 1, 2, S, q);
    jacobi_step<R>(1, 2, 0, S, q);
    jacobi_step<R>(2, 0, 1, S, q);
  }
}

template <class R> inline void cond_swap(bool c, R& x, R& y) {
  const R t = x;
  x = c ? y : x;
  y = c ? t : y;
}
template <class R> inline void cond_neg_swap(bool c, V3<R>& x, V3<R>& y) {
  const V3<R> t = vneg(x);
  x = c ? y : x;
  y = c ? t : y;
}

template <class R> inline void sort_singular(M3<R>& B, M3<R>& V) {
  V3<R> b1 = B[0], b2 = B[1], b3 = B[2];
  V3<R> v1 = V[0], v2 = V[1], v3c = V[2];
  R rho1 = dot3(b1, b1), rho2 = dot3(b2, b2), rho3 = dot3(b3, b3);
  bool c = rho1 < rho2;
  cond_neg_swap(c, b1, b2);
  cond_neg_swap(c, v1, v2);
  cond_swap(c, rho1, rho2);
  c = rho1 < rho3;
  cond_neg_swap(c, b1, b3);
  cond_neg_swap(c, v1, v3c);
  cond_swap(c, rho1, rho3);
  c = rho2 < rho3;
  cond_neg_swap(c, b2, b3);
  cond_neg_swap(c, v2, v3c);
  B = mcols(b1, b2, b3);
  V = mcols(v1, v2, v3c);
}

template <class R> inline void givens_quat(R a1, R a2, R& ch, R& sh) {
  const R rho = std::sqrt(a1 * a1 + a2 * a2);
  sh = rho > SvdConst<R>::eps() ? a2 : R(0);
  ch = std::fabs(a1) + g_max(rho, SvdConst<R>::eps());
  cond_swap(a1 < R(0), sh, ch);
  const R w = g_inversesqrt(ch * ch + sh * sh);
  ch *= w;
  sh *= w;
}

template <class R> inline void qr_givens(const M3<R>& B, M3<R>& Q, M3<R>& Rm) {
  Rm = B;
  R ch, sh, s0, s1;
  R q[4];
  M3<R> U;
  // eliminate (1,0)
  givens_quat(Rm[0][0], Rm[0][1], ch, sh);
  s0 = R(1) - R(2) * sh * sh;
  s1 = R(2) * sh * ch;
  U[0] = v3<R>(s0, s1, R(0));
  U[1] = v3<R>(-s1, s0, R(0));
  U[2] = v3<R>(R(0), R(0), R(1));
  Rm = mmul(mtrans(U), Rm);
  q[0] = R(1); q[1] = R(0); q[2] = R(0); q[3] = R(0);
  {
    const R q0 = ch * q[0] - sh * q[3], q1 = ch * q[1] + sh * q[2];
    const R q2 = ch * q[2] - sh * q[1], q3 = sh * q[0] + ch * q[3];
    q[0] = q0; q[1] = q1; q[2] = q2; q[3] = q3;
  }
  // eliminate (2,0)
  givens_quat(Rm[0][0], Rm[0][2], ch, sh);
  s0 = R(1) - R(2) * sh * sh;
  s1 = R(2) * sh * ch;
  U[0] = v3<R>(s0, R(0), s1);
  U[1] = v3<R>(R(0), R(1), R(0));
  U[2] = v3<R>(-s1, R(0), s0);
  Rm = mmul(mtrans(U), Rm);
  {
    const R q0 = ch * q[0] + sh * q[2], q1 = ch * q[1] + sh * q[3];
    const R q2 = ch * q[2] - sh * q[0], q3 = ch * q[3] - sh * q[1];
    q[0] = q0; q[1] = q1; q[2] = q2; q[3] = q3;
  }
  // eliminate (2,1)
  givens_quat(Rm[1][1], Rm[1][2], ch, sh);
  s0 = R(1) - R(2) * sh * sh;
  s1 = R(2) * sh * ch;
  U[0] = v3<R>(R(1), R(0), R(0));
  U[1] = v3<R>(R(0), s0, s1);
  U[2] = v3<R>(R(0), -s1, s0);
  Rm = mmul(mtrans(U), Rm);
  {
    const R q0 = ch * q[0] - sh * q[1], q1 = sh * q[0] + ch * q[1];
    const R q2 = ch * q[2] + sh * q[3], q3 = ch * q[3] - sh * q[2];
    q[0] = q0; q[1] = q1; q[2] = q2; q[3] = q3;
  }
  Q = quat_to_mat(q);
}

template <class R> inline void svd3(const M3<R>& A, M3<R>& W, M3<R>& S, M3<R>& V, bool vround) {
  M3<R> ata = mmul(mtrans(A), A);
  R q[4];
  jacobi_eigen(ata, q);
  V = quat_to_mat(q);
  if (vround)
    for (int c = 0; c < 3; c++)
      for (int r = 0; r < 3; r++) V[c][r] = rnd_q(V[c][r], R(1e5));
  M3<R> B = mmul(A, V);
  sort_singular(B, V);
  qr_givens(B, W, S);
}

// ---- scene description (mirrors snow_mpm.h's parameters) ----------------
struct OracleDesc {
  double grid_pos[3];
  int grid_dim[3];
  double grid_spacing;
  double young, poisson, hardening, crit_compression, crit_stretch;
  double alpha;
  double gravity[3];
  int n_colliders;
  const double* collider_pos;       // n x 3
  const int* collider_type;         // n
  const double* collider_vel;       // n x 3
  const double* collider_radius;    // n
  const double* collider_normal;    // n x 3
  const double* collider_friction;  // n
  int vround;
  int qround;
  int threads;
};

struct OracleBase {
  virtual ~OracleBase() {}
  virtual void upload(const double* x, const double* v, const double* m, const double* FE, const double* FP,
                      size_t n) = 0;
  virtual void upload_std140(const float* pxm, const int* pv, const float* pFE, const float* pFP, size_t n) = 0;
  virtual void phase(int which, double dt) = 0;
  virtual void download(double* x, double* v, double* m, double* FE, double* FP, double* rho) const = 0;
  virtual void download_std140(float* pxm, int* pv, float* pFE, float* pFP) const = 0;
  virtual void download_grid(double* mass, double* mom, double* force, double* vstar) const = 0;
  virtual void download_grid_fixed(int* gv, int* gf) const = 0;
  virtual void download_accumulators(double* vpic, double* dv) const = 0;
  virtual void download_colliders(double* pos) const = 0;
  virtual void set_density(const double* rho) = 0;
  // semi-implicit velocity update (EXACT modes only)
  virtual void set_implicit(double beta, double tol, int max_iters) = 0;
  virtual void hessian(const double* u, double* out) const = 0;
  virtual void force_at(const double* u, double eps, double* out) const = 0;
  virtual void solver_report(double* out) const = 0;
  // Per particle, the magnitude scale of its FLIP velocity update from the
  // current grid (after the grid phase, before G2P): alpha |v_p| +
  // sum_i w_ip (|v*_i| + alpha |p_i / m_i|) over stencil nodes with mass.
  // The update v' = alpha v_p + sum_i w_ip (v*_i - alpha p_i / m_i) sums
  // terms of these sizes, so a float result is resolved only to ~1e-7 of it.
  virtual void flip_scale(double* out) const = 0;
};

enum {
  PH_RIGID = 0, PH_RESET = 1, PH_P2G = 2, PH_GRID = 3, PH_G2P = 4, PH_ADVANCE = 5, PH_GMASS = 6, PH_PVOLUME = 7,
  PH_IMPLICIT = 8,
};

template <class T> inline void atomic_add(T& dst, T v, bool par) {
  if (par) {
#pragma omp atomic
    dst += v;
  } else {
    dst += v;
  }
}
// int32 wrap-around add, like GLSL atomicAdd.
inline void atomic_add_i(int& dst, int v, bool par) {
  if (par)
    __atomic_fetch_add(&dst, v, __ATOMIC_RELAXED);
  else
    dst = (int)((unsigned)dst + (unsigned)v);
}

template <class R, bool FIXED>
struct Oracle : OracleBase {
  // parameters
  R pos[3];
  int dim[3];
  R h, young, poisson, hardening, crit_c, crit_s, alpha;
  R grav[3];
  bool vround, qround;
  int threads;
  size_t G = 0;
  // colliders: cx = (pos, type), cv = (vel, radius), cn = (normal, friction)
  std::vector<V3<R>> cpos, cvel, cnor;
  std::vector<R> crad, cfric;
  std::vector<int> ctype;
  // particles
  size_t N = 0;
  std::vector<V3<R>> x;
  std::vector<R> m;
  std::vector<V3<R>> v;     // !FIXED
  std::vector<R> rho;       // !FIXED
  std::vector<int> vi;      // FIXED: N x 3, velocity * 1e8
  std::vector<int> rhoi;    // FIXED: density * 1e6
  std::vector<M3<R>> FE, FP;
  // G2P accumulators (per particle)
  std::vector<V3<R>> acc_v;     // !FIXED
  std::vector<M3<R>> acc_dv;    // !FIXED: columns pdvp0..2
  std::vector<int> acc_vi;      // FIXED: N x 3
  std::vector<int> acc_dvi;     // FIXED: N x 9 (column c, row r at 3c + r)
  // grid
  std::vector<R> gm;            // !FIXED
  std::vector<V3<R>> gp, gf;    // !FIXED
  std::vector<int> gi;          // FIXED: G x 7 (px, py, pz, m, fx, fy, fz)
  std::vector<V3<R>> gvn;

  bool par() const { return threads > 1; }

  explicit Oracle(const OracleDesc* d) {
    for (int i = 0; i < 3; i++) {
      pos[i] = R(d->grid_pos[i]);
      dim[i] = d->grid_dim[i];
      grav[i] = R(d->gravity[i]);
    }
    h = R(d->grid_spacing);
    young = R(d->young);
    poisson = R(d->poisson);
    hardening = R(d->hardening);
    crit_c = R(d->crit_compression);
    crit_s = R(d->crit_stretch);
    alpha = R(d->alpha);
    vround = d->vround != 0;
    qround = d->qround != 0;
    threads = d->threads > 0 ? d->threads : 1;
    G = (size_t)dim[0] * dim[1] * dim[2];
    for (int c = 0; c < d->n_colliders; c++) {
      cpos.push_back(v3<R>(R(d->collider_pos[3 * c]), R(d->collider_pos[3 * c + 1]), R(d->collider_pos[3 * c + 2])));
      cvel.push_back(v3<R>(R(d->collider_vel[3 * c]), R(d->collider_vel[3 * c + 1]), R(d->collider_vel[3 * c + 2])));
      cnor.push_back(v3<R>(R(d->collider_normal[3 * c]), R(d->collider_normal[3 * c + 1]),
                           R(d->collider_normal[3 * c + 2])));
      crad.push_back(R(d->collider_radius[c]));
      cfric.push_back(R(d->collider_friction[c]));
      ctype.push_back(d->collider_type[c]);
    }
    if (FIXED) {
      gi.assign(G * 7, 0);
    } else {
      gm.assign(G, R(0));
      gp.assign(G, v3<R>(0, 0, 0));
      gf.assign(G, v3<R>(0, 0, 0));
    }
    gvn.assign(G, v3<R>(0, 0, 0));
  }

  void alloc(size_t n) {
    N = n;
    x.assign(n, v3<R>(0, 0, 0));
    m.assign(n, R(0));
    FE.assign(n, mdiag<R>(1));
    FP.assign(n, mdiag<R>(1));
    if (FIXED) {
      vi.assign(3 * n, 0);
      rhoi.assign(n, 0);
      acc_vi.assign(3 * n, 0);
      acc_dvi.assign(9 * n, 0);
    } else {
      v.assign(n, v3<R>(0, 0, 0));
      rho.assign(n, R(0));
      acc_v.assign(n, v3<R>(0, 0, 0));
      acc_dv.assign(n, mdiag<R>(0));
    }
  }

  // Row-major N x 9 input (F[r][c] at 9p + 3r + c).
  static M3<R> from_rowmajor(const double* f) {
    M3<R> mm;
    for (int r = 0; r < 3; r++)
      for (int c = 0; c < 3; c++) mm[c][r] = R(f[3 * r + c]);
    return mm;
  }

  void upload(const double* xx, const double* vv, const double* mm, const double* fe, const double* fp,
              size_t n) override {
    alloc(n);
    for (size_t p = 0; p < n; p++) {
      x[p] = v3<R>(R(xx[3 * p]), R(xx[3 * p + 1]), R(xx[3 * p + 2]));
      m[p] = R(mm[p]);
      if (FIXED) {
        // Particle(..., Vector3i v) stores v * 1e8 as int (particle.hpp:4-36).
        for (int k = 0; k < 3; k++) vi[3 * p + k] = (int)(float)(vv[3 * p + k] * 1e8);
      } else {
        v[p] = v3<R>(R(vv[3 * p]), R(vv[3 * p + 1]), R(vv[3 * p + 2]));
      }
      if (fe) FE[p] = from_rowmajor(fe + 9 * p);
      if (fp) FP[p] = from_rowmajor(fp + 9 * p);
    }
  }

  // The reference's std140 buffers: pxm N x vec4, pv N x ivec4, pFE/pFP N x mat4.
  void upload_std140(const float* pxm, const int* pv, const float* pFE, const float* pFP, size_t n) override {
    alloc(n);
    for (size_t p = 0; p < n; p++) {
      x[p] = v3<R>(R(pxm[4 * p]), R(pxm[4 * p + 1]), R(pxm[4 * p + 2]));
      m[p] = R(pxm[4 * p + 3]);
      if (FIXED) {
        for (int k = 0; k < 3; k++) vi[3 * p + k] = pv[4 * p + k];
        rhoi[p] = pv[4 * p + 3];
      } else {
        v[p] = v3<R>(R(float(pv[4 * p]) * 1e-8f), R(float(pv[4 * p + 1]) * 1e-8f), R(float(pv[4 * p + 2]) * 1e-8f));
        rho[p] = R(float(pv[4 * p + 3]) * 1e-6f);
      }
      for (int c = 0; c < 3; c++)
        for (int r = 0; r < 3; r++) {
          FE[p][c][r] = R(pFE[16 * p + 4 * c + r]);
          FP[p][c][r] = R(pFP[16 * p + 4 * c + r]);
        }
    }
  }

  // ---- per-particle helpers -------------------------------------------
  V3<R> particle_in_grid(size_t p) const {
    return v3<R>((x[p][0] - pos[0]) / h, (x[p][1] - pos[1]) / h, (x[p][2] - pos[2]) / h);
  }
  // Neighbour 0..63 -> offset (-1..2)^3, x fastest (neighborIndex.include.glsl:6-12).
  static void neighbour_offset(int y, int o[3]) {
    const int t = y % 16;
    o[0] = t % 4 - 1;
    o[1] = t / 4 - 1;
    o[2] = y / 16 - 1;
  }
  bool in_grid(const int g[3]) const {
    return g[0] >= 0 && g[1] >= 0 && g[2] >= 0 && g[0] < dim[0] && g[1] < dim[1] && g[2] < dim[2];
  }
  // gridIndex.include.glsl:7-9
  size_t node_index(const int g[3]) const {
    return (size_t)(g[0] + g[1] * dim[0] + g[2] * dim[1] * dim[0]);
  }
  V3<R> vel(size_t p) const {
    if (FIXED)
      return v3<R>(R(float(vi[3 * p])) * R(1e-8f), R(float(vi[3 * p + 1])) * R(1e-8f), R(float(vi[3 * p + 2])) * R(1e-8f));
    return v[p];
  }
  R density(size_t p) const { return FIXED ? R(float(rhoi[p])) * R(1e-6f) : rho[p]; }
  R node_mass(size_t g) const { return FIXED ? R(float(gi[7 * g + 3])) * R(1e-8f) : gm[g]; }
  V3<R> node_mom(size_t g) const {
    if (FIXED)
      return v3<R>(R(float(gi[7 * g])) * R(1e-8f), R(float(gi[7 * g + 1])) * R(1e-8f), R(float(gi[7 * g + 2])) * R(1e-8f));
    return gp[g];
  }
  V3<R> node_force(size_t g) const {
    if (FIXED)
      return v3<R>(R(float(gi[7 * g + 4])) * R(1e-6f), R(float(gi[7 * g + 5])) * R(1e-6f), R(float(gi[7 * g + 6])) * R(1e-6f));
    return gf[g];
  }
  // Grid::initSSBO node position x_off + h * (float)i (grid.cpp:96-107).
  V3<R> node_pos(size_t g) const {
    const int i = (int)(g % dim[0]);
    const int j = (int)((g / dim[0]) % dim[1]);
    const int k = (int)(g / ((size_t)dim[0] * dim[1]));
    return v3<R>(pos[0] + h * R(i), pos[1] + h * R(j), pos[2] + h * R(k));
  }

  // lame.include.glsl:11-27
  R mu(R jp) const { return young / (R(2) * (R(1) + poisson)) * g_exp(hardening * (R(1) - jp)); }
  R lambda(R jp) const {
    return young * poisson / ((R(1) + poisson) * (R(1) - R(2) * poisson)) * g_exp(hardening * (R(1) - jp));
  }

  // Collider projection shared by the grid update (gForceCompute.glsl:72-93)
  // and the particle update (particleAdvance.glsl:182-204).
  V3<R> collide(const V3<R>& xq, V3<R> vin) const {
    for (size_t i = 0; i < ctype.size(); i++) {
      V3<R> n = cnor[i];
      bool hit = false;
      const unsigned t = (unsigned)(float)ctype[i];
      if (t == 0u) {
        hit = dot3(vsub(xq, cpos[i]), cnor[i]) <= R(0);
      } else if (t == 1u) {
        const V3<R> d = vsub(xq, cpos[i]);
        n = divs(d, len3(d));
        hit = len3(vsub(xq, cpos[i])) < crad[i];
      }
      if (!hit) continue;
      const V3<R> vco = cvel[i];
      const V3<R> vrel = vsub(vin, vco);
      const R vn = dot3(vrel, n);
      if (vn < R(0)) {
        const V3<R> vt = vsub(vrel, muls(n, vn));
        const R muvn = cfric[i] * vn;
        V3<R> vrelt = vt;
        const R lvt = len3(vt);
        if (lvt <= -muvn)
          vrelt = v3<R>(0, 0, 0);
        else
          vrelt = vadd(vrelt, divs(smul(muvn, vt), lvt));
        vin = vadd(vrelt, vco);
      }
    }
    return vin;
  }

  // ---- kernels ---------------------------------------------------------
  // rigidAdvance.glsl:14-18
  void rigid_advance(R dt) {
    for (size_t i = 0; i < cpos.size(); i++) cpos[i] = vadd(cpos[i], smul(dt, cvel[i]));
  }

  // gReset.glsl:11-16
  void reset() {
    if (FIXED) {
      std::fill(gi.begin(), gi.end(), 0);
    } else {
      std::fill(gm.begin(), gm.end(), R(0));
      std::fill(gp.begin(), gp.end(), v3<R>(0, 0, 0));
      std::fill(gf.begin(), gf.end(), v3<R>(0, 0, 0));
    }
  }

  // gMassCompute.glsl:33-84 (mass only) and p2gTransfer.glsl:44-151.
  void p2g(bool mass_only) {
    const bool pp = par();
#pragma omp parallel for schedule(dynamic, 256) num_threads(threads) if (pp)
    for (long long pl = 0; pl < (long long)N; pl++) {
      const size_t p = (size_t)pl;
      const R mp = m[p];
      if (!mass_only && std::fabs(mp) > R(100)) continue;
      const V3<R> vp = vel(p);
      const R pp0 = density(p);
      const V3<R> pg = particle_in_grid(p);
      const int base[3] = {(int)pg[0], (int)pg[1], (int)pg[2]};
      // Stress part, the same for all 64 neighbours: the shader recomputes it
      // in each of its 64 invocations (p2gTransfer.glsl:109-146).
      M3<R> stress;
      R vol_scale = R(0);
      const bool has_force = !mass_only && pp0 > R(0);
      if (!mass_only) {
        M3<R> W, S, V;
        svd3(FE[p], W, S, V, vround);
        M3<R> Rp = mmul(W, mtrans(V));
        if (qround)
          for (int c = 0; c < 3; c++)
            for (int r = 0; r < 3; r++) Rp[c][r] = rnd_q(Rp[c][r], R(1e9));
        const R jpp = mdet(FP[p]);
        const R jep = mdet(FE[p]);
        const M3<R> a = mmul(msmul(R(2) * mu(jpp), msub(FE[p], Rp)), mtrans(FE[p]));
        const M3<R> b = msmul(lambda(jpp) * (jep - R(1)) * jep, mdiag<R>(1));
        stress = madd(a, b);
        vol_scale = -(mp / pp0);
      }
      for (int y = 0; y < 64; y++) {
        int o[3];
        neighbour_offset(y, o);
        const int g[3] = {base[0] + o[0], base[1] + o[1], base[2] + o[2]};
        if (!in_grid(g)) continue;
        const V3<R> d = v3<R>(R(g[0]) - pg[0], R(g[1]) - pg[1], R(g[2]) - pg[2]);
        const R w = weight3(d);
        const size_t gI = node_index(g);
        if (FIXED) {
          atomic_add_i(gi[7 * gI + 3], (int)(mp * w * R(1e8f)), pp);
        } else {
          atomic_add(gm[gI], mp * w, pp);
        }
        if (mass_only) continue;
        const V3<R> mv = muls(muls(vp, mp), w);
        if (FIXED) {
          for (int k = 0; k < 3; k++) atomic_add_i(gi[7 * gI + k], (int)(mv[k] * R(1e8f)), pp);
        } else {
          for (int k = 0; k < 3; k++) atomic_add(gp[gI][k], mv[k], pp);
        }
        if (!has_force) continue;
        const V3<R> wg = weight3_grad(vneg(d));
        const V3<R> f = smul(vol_scale, mvmul(stress, wg));
        if (FIXED) {
          for (int k = 0; k < 3; k++) atomic_add_i(gi[7 * gI + 4 + k], (int)(f[k] * R(1e6f)), pp);
        } else {
          for (int k = 0; k < 3; k++) atomic_add(gf[gI][k], f[k], pp);
        }
      }
    }
  }

  // pVolumeCompute.glsl:32-83
  void p_volume() {
    const R cell = h * h * h;
#pragma omp parallel for schedule(dynamic, 256) num_threads(threads) if (par())
    for (long long pl = 0; pl < (long long)N; pl++) {
      const size_t p = (size_t)pl;
      const V3<R> pg = particle_in_grid(p);
      const int base[3] = {(int)pg[0], (int)pg[1], (int)pg[2]};
      for (int y = 0; y < 64; y++) {
        int o[3];
        neighbour_offset(y, o);
        const int g[3] = {base[0] + o[0], base[1] + o[1], base[2] + o[2]};
        if (!in_grid(g)) continue;
        const V3<R> d = v3<R>(R(g[0]) - pg[0], R(g[1]) - pg[1], R(g[2]) - pg[2]);
        const R w = weight3(d);
        const R mi = node_mass(node_index(g));
        if (FIXED)
          rhoi[p] = (int)((unsigned)rhoi[p] + (unsigned)(int)(mi * w / cell * R(1e6f)));
        else
          rho[p] += mi * w / cell;
      }
    }
  }

  // gForceCompute.glsl:57-103
  void grid_update(R dt) {
#pragma omp parallel for schedule(static) num_threads(threads) if (par())
    for (long long gl = 0; gl < (long long)G; gl++) {
      const size_t g = (size_t)gl;
      const R mi = node_mass(g);
      if (!(mi > R(0))) {
        gvn[g] = v3<R>(0, 0, 0);
        continue;
      }
      const V3<R> vi_ = node_mom(g);
      const V3<R> fi = node_force(g);
      V3<R> vin = vadd(divs(vi_, mi), smul(dt, vadd(divs(fi, mi), v3<R>(grav[0], grav[1], grav[2]))));
      vin = collide(node_pos(g), vin);
      gvn[g] = vin;
    }
  }

  // g2pTransfer.glsl:53-143: PIC/FLIP increment and velocity gradient,
  // accumulated per particle.
  void g2p() {
#pragma omp parallel for schedule(dynamic, 256) num_threads(threads) if (par())
    for (long long pl = 0; pl < (long long)N; pl++) {
      const size_t p = (size_t)pl;
      const V3<R> pg = particle_in_grid(p);
      const int base[3] = {(int)pg[0], (int)pg[1], (int)pg[2]};
      for (int y = 0; y < 64; y++) {
        int o[3];
        neighbour_offset(y, o);
        const int g[3] = {base[0] + o[0], base[1] + o[1], base[2] + o[2]};
        if (!in_grid(g)) continue;
        const V3<R> d = v3<R>(R(g[0]) - pg[0], R(g[1]) - pg[1], R(g[2]) - pg[2]);
        const R w = weight3(d);
        const V3<R> gw = weight3_grad(vneg(d));
        const size_t gI = node_index(g);
        const V3<R> vin = gvn[gI];
        const V3<R> vi_ = node_mom(gI);
        const R mi = node_mass(gI);
        if (!(mi > R(0))) continue;
        const V3<R> pic = muls(smul(R(1) - alpha, vin), w);
        const V3<R> flip = muls(smul(alpha, vsub(vin, divs(vi_, mi))), w);
        const V3<R> vpn = vadd(pic, flip);
        if (FIXED) {
          for (int k = 0; k < 3; k++) acc_vi[3 * p + k] += (int)(vpn[k] * R(1e8f));
          for (int c = 0; c < 3; c++)
            for (int r = 0; r < 3; r++) acc_dvi[9 * p + 3 * c + r] += (int)(vin[r] * gw[c] * R(1e8f));
        } else {
          acc_v[p] = vadd(acc_v[p], vpn);
          for (int c = 0; c < 3; c++)
            for (int r = 0; r < 3; r++) acc_dv[p][c][r] += vin[r] * gw[c];
        }
      }
    }
  }

  // particleAdvance.glsl:75-217
  void advance(R dt) {
    const R lo = R(1) - crit_c, hi = R(1) + crit_s;
#pragma omp parallel for schedule(dynamic, 256) num_threads(threads) if (par())
    for (long long pl = 0; pl < (long long)N; pl++) {
      const size_t p = (size_t)pl;
      M3<R> dvp;
      if (FIXED) {
        for (int c = 0; c < 3; c++)
          for (int r = 0; r < 3; r++) dvp[c][r] = R(float(acc_dvi[9 * p + 3 * c + r])) * R(1e-8f);
      } else {
        dvp = acc_dv[p];
      }
      const M3<R> step = madd(mdiag<R>(1), msmul(dt, dvp));
      M3<R> fe = mmul(step, FE[p]);
      const M3<R> fall = mmul(step, mmul(FE[p], FP[p]));
      M3<R> W, S, V;
      svd3(fe, W, S, V, vround);
      for (int i = 0; i < 3; i++) S[i][i] = (S[i][i] < lo) ? lo : (S[i][i] > hi) ? hi : S[i][i];
      fe = mmul(mmul(W, S), mtrans(V));
      if (qround)
        for (int c = 0; c < 3; c++)
          for (int r = 0; r < 3; r++) fe[c][r] = rnd_q(fe[c][r], R(1e9));
      M3<R> sinv = mdiag<R>(0);
      for (int i = 0; i < 3; i++) sinv[i][i] = R(1) / S[i][i];
      M3<R> fp = mmul(mmul(mmul(V, sinv), mtrans(W)), fall);
      if (qround)
        for (int c = 0; c < 3; c++)
          for (int r = 0; r < 3; r++) fp[c][r] = rnd_q(fp[c][r], R(1e9));
      FE[p] = fe;
      FP[p] = fp;
      V3<R> vpn;
      if (FIXED)
        vpn = v3<R>(R(float(acc_vi[3 * p])) * R(1e-8f), R(float(acc_vi[3 * p + 1])) * R(1e-8f),
                    R(float(acc_vi[3 * p + 2])) * R(1e-8f));
      else
        vpn = acc_v[p];
      V3<R> vpn1 = vadd(muls(vel(p), alpha), vpn);
      vpn1 = collide(x[p], vpn1);
      if (FIXED)
        for (int k = 0; k < 3; k++) vi[3 * p + k] = (int)(vpn1[k] * R(1e8f));
      else
        v[p] = vpn1;
      x[p] = vadd(x[p], smul(dt, vpn1));
      if (FIXED) {
        for (int k = 0; k < 3; k++) acc_vi[3 * p + k] = 0;
        for (int k = 0; k < 9; k++) acc_dvi[9 * p + k] = 0;
      } else {
        acc_v[p] = v3<R>(0, 0, 0);
        acc_dv[p] = mdiag<R>(0);
      }
    }
  }

  // ---- semi-implicit velocity update ------------------------------------
  // The reference ships SemiImplicitTimeUpdate as an empty stub
  // (src/snow/simulation/timeUpdate/semiimplicittimeupdate.cpp:3-5). This
  // restates the scheme of Stomakhin et al. 2013 (sec. 4, eq. 9, and the
  // force differential below it) on top of the explicit step: after the grid
  // update has formed v* (with colliders), solve
  //     (M + beta dt^2 K) v = M v*
  // by conjugate residuals, K u = sum_p V0_p dP(F_p; G_p F_p) F_p^T grad w_ip,
  // G_p = sum_j u_j (grad w_jp)^T, then apply the colliders to v again. The
  // weight gradients are the explicit force's own (grid units, as
  // p2gTransfer.glsl:121-146 uses them), so K is the derivative of the force
  // the explicit step applies. Only the EXACT modes (no fixed point) solve.
  R imp_beta = R(0), imp_tol = R(1e-6);
  int imp_maxit = 0;
  int imp_iters = 0;
  double imp_res = 0.0, imp_res0 = 0.0;

  void set_implicit(double beta, double tol, int max_iters) override {
    imp_beta = R(beta);
    imp_tol = R(tol);
    imp_maxit = max_iters;
  }
  void solver_report(double* out) const override {
    out[0] = imp_iters;
    out[1] = imp_res;
    out[2] = imp_res0;
  }

  // Calls fn(node, w, grad w) for each in-grid stencil node of particle p
  // (the neighbour order and distances of p2gTransfer.glsl:83-91,121-122).
  template <class Fn> void stencil(size_t p, Fn fn) const {
    const V3<R> pg = particle_in_grid(p);
    const int base[3] = {(int)pg[0], (int)pg[1], (int)pg[2]};
    for (int y = 0; y < 64; y++) {
      int o[3];
      neighbour_offset(y, o);
      const int g[3] = {base[0] + o[0], base[1] + o[1], base[2] + o[2]};
      if (!in_grid(g)) continue;
      const V3<R> d = v3<R>(R(g[0]) - pg[0], R(g[1]) - pg[1], R(g[2]) - pg[2]);
      fn(node_index(g), weight3(d), weight3_grad(vneg(d)));
    }
  }
  // The particles that carry a stress force (p2gTransfer.glsl:64-66,126).
  bool has_force(size_t p) const { return !(std::fabs(m[p]) > R(100)) && density(p) > R(0); }

  // Cofactor matrix J F^-T: columns f1 x f2, f2 x f0, f0 x f1.
  static V3<R> cross3(const V3<R>& a, const V3<R>& b) {
    return v3<R>(a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]);
  }
  static M3<R> cofactor(const M3<R>& F) {
    M3<R> C;
    C[0] = cross3(F[1], F[2]);
    C[1] = cross3(F[2], F[0]);
    C[2] = cross3(F[0], F[1]);
    return C;
  }
  // First Piola-Kirchhoff stress of the fixed-corotated energy,
  // P = 2 mu (F - R) + lambda (J - 1) J F^-T; P F^T is the shader's stress.
  // R is the polar rotation to working precision (Newton's iteration
  // R <- (R + R^-T) / 2, which converges quadratically for det F > 0), so
  // that finite differences of the force resolve the differential below
  // rather than the approximate SVD's residual.
  static M3<R> polar_rotation(const M3<R>& F) {
    M3<R> Rp = F;
    for (int it = 0; it < 60; it++) {
      const M3<R> inv_t = msmul(R(1) / mdet(Rp), cofactor(Rp));
      const M3<R> next = msmul(R(0.5), madd(Rp, inv_t));
      R delta = R(0);
      for (int c = 0; c < 3; c++)
        for (int r = 0; r < 3; r++) delta = std::max(delta, std::fabs(next[c][r] - Rp[c][r]));
      Rp = next;
      if (delta <= R(4) * std::numeric_limits<R>::epsilon()) break;
    }
    return Rp;
  }
  M3<R> piola(const M3<R>& F, R mu_, R lam_) const {
    const M3<R> Rp = polar_rotation(F);
    return madd(msmul(R(2) * mu_, msub(F, Rp)), msmul(lam_ * (mdet(F) - R(1)), cofactor(F)));
  }
  // dP(F; dF). The rotation's differential: with F = W S V^T and
  // G = W^T dF V, dR = W X V^T, X skew with X_ij = (G_ij - G_ji)/(s_i + s_j)
  // (from R^T dF - dF^T R = X' S + S X' in the frame of V).
  M3<R> stress_differential(const M3<R>& F, R mu_, R lam_, const M3<R>& dF) const {
    M3<R> W, S, V;
    svd3(F, W, S, V, vround);
    const M3<R> Gm = mmul(mmul(mtrans(W), dF), V);
    M3<R> X = mdiag<R>(0);
    for (int i = 0; i < 3; i++)
      for (int j = i + 1; j < 3; j++) {
        const R xij = (Gm[j][i] - Gm[i][j]) / (S[i][i] + S[j][j]);  // row i, column j
        X[j][i] = xij;
        X[i][j] = -xij;
      }
    const M3<R> dR = mmul(mmul(W, X), mtrans(V));
    const M3<R> C = cofactor(F);
    R dJ = R(0);
    for (int c = 0; c < 3; c++)
      for (int r = 0; r < 3; r++) dJ += C[c][r] * dF[c][r];
    M3<R> dC;
    dC[0] = vadd(cross3(dF[1], F[2]), cross3(F[1], dF[2]));
    dC[1] = vadd(cross3(dF[2], F[0]), cross3(F[2], dF[0]));
    dC[2] = vadd(cross3(dF[0], F[1]), cross3(F[0], dF[1]));
    return madd(msmul(R(2) * mu_, msub(dF, dR)),
                madd(msmul(lam_ * dJ, C), msmul(lam_ * (mdet(F) - R(1)), dC)));
  }
  // G_p = sum_j u_j (grad w_jp)^T.
  M3<R> particle_gradient(size_t p, const std::vector<V3<R>>& u) const {
    M3<R> Gm = mdiag<R>(0);
    stencil(p, [&](size_t gI, R, const V3<R>& gw) {
      for (int c = 0; c < 3; c++)
        for (int r = 0; r < 3; r++) Gm[c][r] += u[gI][r] * gw[c];
    });
    return Gm;
  }
  // out = K u on the dense grid.
  void hessian_action(const std::vector<V3<R>>& u, std::vector<V3<R>>& out) const {
    out.assign(G, v3<R>(0, 0, 0));
    const bool pp = par();
#pragma omp parallel for schedule(dynamic, 256) num_threads(threads) if (pp)
    for (long long pl = 0; pl < (long long)N; pl++) {
      const size_t p = (size_t)pl;
      if (!has_force(p)) continue;
      const R jpp = mdet(FP[p]);
      const M3<R> dF = mmul(particle_gradient(p, u), FE[p]);
      const M3<R> dP = stress_differential(FE[p], mu(jpp), lambda(jpp), dF);
      const M3<R> A = msmul(m[p] / density(p), mmul(dP, mtrans(FE[p])));
      stencil(p, [&](size_t gI, R, const V3<R>& gw) {
        const V3<R> f = mvmul(A, gw);
        for (int k = 0; k < 3; k++) atomic_add(out[gI][k], f[k], pp);
      });
    }
  }
  // The grid force at the deformed positions x_i + eps u_i:
  // f_i = -sum_p V0 P((I + eps G_p) F_p) F_p^T grad w_ip (finite-difference
  // checks of K: K u = -(f(eps) - f(-eps)) / (2 eps) + O(eps^2)).
  void force_at_grid(const std::vector<V3<R>>& u, R eps, std::vector<V3<R>>& out) const {
    out.assign(G, v3<R>(0, 0, 0));
    const bool pp = par();
#pragma omp parallel for schedule(dynamic, 256) num_threads(threads) if (pp)
    for (long long pl = 0; pl < (long long)N; pl++) {
      const size_t p = (size_t)pl;
      if (!has_force(p)) continue;
      const R jpp = mdet(FP[p]);
      const M3<R> Fh = mmul(madd(mdiag<R>(1), msmul(eps, particle_gradient(p, u))), FE[p]);
      const M3<R> A = msmul(-(m[p] / density(p)), mmul(piola(Fh, mu(jpp), lambda(jpp)), mtrans(FE[p])));
      stencil(p, [&](size_t gI, R, const V3<R>& gw) {
        const V3<R> f = mvmul(A, gw);
        for (int k = 0; k < 3; k++) atomic_add(out[gI][k], f[k], pp);
      });
    }
  }
  static std::vector<V3<R>> grid_from(const double* a, size_t n) {
    std::vector<V3<R>> u(n);
    for (size_t g = 0; g < n; g++) u[g] = v3<R>(R(a[3 * g]), R(a[3 * g + 1]), R(a[3 * g + 2]));
    return u;
  }
  static void grid_to(const std::vector<V3<R>>& u, double* a) {
    for (size_t g = 0; g < u.size(); g++)
      for (int k = 0; k < 3; k++) a[3 * g + k] = double(u[g][k]);
  }
  void hessian(const double* u, double* out) const override {
    std::vector<V3<R>> r;
    hessian_action(grid_from(u, G), r);
    grid_to(r, out);
  }
  void force_at(const double* u, double eps, double* out) const override {
    std::vector<V3<R>> r;
    force_at_grid(grid_from(u, G), R(eps), r);
    grid_to(r, out);
  }

  // Conjugate residuals on the mass-scaled system
  //     (I + c M^-1/2 K M^-1/2) y = M^1/2 v*,   v = M^-1/2 y,   c = beta dt^2,
  // (the same solution as (M + c K) v = M v*; the scaling by the lumped
  // masses keeps the nodes at the material's edge, whose masses are tiny,
  // from stalling the iteration), from y = M^1/2 v*. Stops when
  // |r| <= tol |M^1/2 v*| (the residual in the kinetic-energy norm) or after
  // imp_maxit iterations. Nodes without mass keep v = 0.
  void implicit_solve(R dt) {
    imp_iters = 0;
    imp_res = imp_res0 = 0.0;
    if (FIXED || !(imp_beta > R(0))) return;
    const R c = imp_beta * dt * dt;
    std::vector<R> sq(G, R(0)), isq(G, R(0));
    for (size_t g = 0; g < G; g++)
      if (node_mass(g) > R(0)) {
        sq[g] = std::sqrt(node_mass(g));
        isq[g] = R(1) / sq[g];
      }
    auto dotg = [&](const std::vector<V3<R>>& a, const std::vector<V3<R>>& b) {
      R t = R(0);
      for (size_t g = 0; g < G; g++) t += dot3(a[g], b[g]);
      return t;
    };
    std::vector<V3<R>> u(G), ku;
    // out = y + c M^-1/2 K M^-1/2 y on the nodes with mass
    auto apply = [&](const std::vector<V3<R>>& y, std::vector<V3<R>>& out) {
      for (size_t g = 0; g < G; g++) u[g] = smul(isq[g], y[g]);
      hessian_action(u, ku);
      out.resize(G);
      for (size_t g = 0; g < G; g++) out[g] = sq[g] > R(0) ? vadd(y[g], smul(c * isq[g], ku[g])) : v3<R>(0, 0, 0);
    };
    std::vector<V3<R>> y(G), b(G), r(G), p, Ar, Ap;
    for (size_t g = 0; g < G; g++) b[g] = y[g] = smul(sq[g], gvn[g]);
    const R bb = dotg(b, b);
    apply(y, Ar);
    for (size_t g = 0; g < G; g++) r[g] = vsub(b[g], Ar[g]);
    R rr = dotg(r, r);
    imp_res0 = bb > R(0) ? double(std::sqrt(rr / bb)) : 0.0;
    const R tol2 = imp_tol * imp_tol * bb;
    if (rr > tol2) {
      apply(r, Ar);
      p = r;
      Ap = Ar;
      R rAr = dotg(r, Ar);
      for (int k = 1; k <= imp_maxit; k++) {
        const R ApAp = dotg(Ap, Ap);
        const R alpha_k = ApAp > R(0) ? rAr / ApAp : R(0);
        for (size_t g = 0; g < G; g++) {
          y[g] = vadd(y[g], smul(alpha_k, p[g]));
          r[g] = vsub(r[g], smul(alpha_k, Ap[g]));
        }
        rr = dotg(r, r);
        imp_iters = k;
        if (rr <= tol2 || k == imp_maxit) break;
        apply(r, Ar);
        const R rAr_new = dotg(r, Ar);
        const R beta_k = rAr != R(0) ? rAr_new / rAr : R(0);
        rAr = rAr_new;
        for (size_t g = 0; g < G; g++) {
          p[g] = vadd(r[g], smul(beta_k, p[g]));
          Ap[g] = vadd(Ar[g], smul(beta_k, Ap[g]));
        }
      }
    }
    imp_res = bb > R(0) ? double(std::sqrt(rr / bb)) : 0.0;
    for (size_t g = 0; g < G; g++)
      gvn[g] = sq[g] > R(0) ? collide(node_pos(g), smul(isq[g], y[g])) : v3<R>(0, 0, 0);
  }

  void flip_scale(double* out) const override {
#pragma omp parallel for schedule(dynamic, 256) num_threads(threads) if (par())
    for (long long pl = 0; pl < (long long)N; pl++) {
      const size_t p = (size_t)pl;
      const V3<R> pg = particle_in_grid(p);
      const int base[3] = {(int)pg[0], (int)pg[1], (int)pg[2]};
      const V3<R> vp = vel(p);
      double sc = double(alpha) * std::sqrt(double(vp[0] * vp[0] + vp[1] * vp[1] + vp[2] * vp[2]));
      for (int y = 0; y < 64; y++) {
        int o[3];
        neighbour_offset(y, o);
        const int g[3] = {base[0] + o[0], base[1] + o[1], base[2] + o[2]};
        if (!in_grid(g)) continue;
        const size_t gI = node_index(g);
        const R mi = node_mass(gI);
        if (!(mi > R(0))) continue;
        const V3<R> d = v3<R>(R(g[0]) - pg[0], R(g[1]) - pg[1], R(g[2]) - pg[2]);
        const double w = double(weight3(d));
        const V3<R> vs = gvn[gI];
        const V3<R> vo = divs(node_mom(gI), mi);
        const double a = std::sqrt(double(vs[0] * vs[0] + vs[1] * vs[1] + vs[2] * vs[2]));
        const double b = std::sqrt(double(vo[0] * vo[0] + vo[1] * vo[1] + vo[2] * vo[2]));
        sc += w * (a + double(alpha) * b);
      }
      out[p] = sc;
    }
  }

  void phase(int which, double dt_d) override {
    const R dt = R(float(dt_d));
    switch (which) {
      case PH_RIGID: rigid_advance(dt); break;
      case PH_RESET: reset(); break;
      case PH_P2G: p2g(false); break;
      case PH_GRID: grid_update(dt); break;
      case PH_G2P: g2p(); break;
      case PH_ADVANCE: advance(dt); break;
      case PH_GMASS: p2g(true); break;
      case PH_PVOLUME: p_volume(); break;
      case PH_IMPLICIT: implicit_solve(dt); break;
      default: break;
    }
  }

  void download(double* xx, double* vv, double* mm, double* fe, double* fp, double* rh) const override {
    for (size_t p = 0; p < N; p++) {
      const V3<R> vp = vel(p);
      for (int k = 0; k < 3; k++) {
        if (xx) xx[3 * p + k] = double(x[p][k]);
        if (vv) vv[3 * p + k] = double(vp[k]);
      }
      if (mm) mm[p] = double(m[p]);
      if (rh) rh[p] = double(density(p));
      for (int r = 0; r < 3; r++)
        for (int c = 0; c < 3; c++) {
          if (fe) fe[9 * p + 3 * r + c] = double(FE[p][c][r]);
          if (fp) fp[9 * p + 3 * r + c] = double(FP[p][c][r]);
        }
    }
  }

  void download_std140(float* pxm, int* pv, float* pFE, float* pFP) const override {
    for (size_t p = 0; p < N; p++) {
      if (pxm) {
        for (int k = 0; k < 3; k++) pxm[4 * p + k] = float(x[p][k]);
        pxm[4 * p + 3] = float(m[p]);
      }
      if (pv) {
        if (FIXED) {
          for (int k = 0; k < 3; k++) pv[4 * p + k] = vi[3 * p + k];
          pv[4 * p + 3] = rhoi[p];
        } else {
          for (int k = 0; k < 3; k++) pv[4 * p + k] = (int)(float(v[p][k]) * 1e8f);
          pv[4 * p + 3] = (int)(float(rho[p]) * 1e6f);
        }
      }
      for (int c = 0; c < 4; c++)
        for (int r = 0; r < 4; r++) {
          const bool in3 = c < 3 && r < 3;
          // mat4(mat3): identity outside the 3x3 block.
          if (pFE) pFE[16 * p + 4 * c + r] = in3 ? float(FE[p][c][r]) : (c == r ? 1.0f : 0.0f);
          if (pFP) pFP[16 * p + 4 * c + r] = in3 ? float(FP[p][c][r]) : (c == r ? 1.0f : 0.0f);
        }
    }
  }

  void download_grid(double* mass, double* mom, double* force, double* vstar) const override {
    for (size_t g = 0; g < G; g++) {
      if (mass) mass[g] = double(node_mass(g));
      const V3<R> pm = node_mom(g), fo = node_force(g);
      for (int k = 0; k < 3; k++) {
        if (mom) mom[3 * g + k] = double(pm[k]);
        if (force) force[3 * g + k] = double(fo[k]);
        if (vstar) vstar[3 * g + k] = double(gvn[g][k]);
      }
    }
  }

  // FIXED only: gv (px, py, pz, m) and gf (fx, fy, fz, 0) as G x 4 ints.
  void download_grid_fixed(int* gv, int* gfo) const override {
    if (!FIXED) return;
    for (size_t g = 0; g < G; g++) {
      if (gv)
        for (int k = 0; k < 4; k++) gv[4 * g + k] = gi[7 * g + k];
      if (gfo) {
        for (int k = 0; k < 3; k++) gfo[4 * g + k] = gi[7 * g + 4 + k];
        gfo[4 * g + 3] = 0;
      }
    }
  }

  void download_accumulators(double* vpic, double* dv) const override {
    for (size_t p = 0; p < N; p++) {
      for (int k = 0; k < 3; k++)
        if (vpic) vpic[3 * p + k] = FIXED ? double(acc_vi[3 * p + k]) * 1e-8 : double(acc_v[p][k]);
      if (dv)
        for (int r = 0; r < 3; r++)
          for (int c = 0; c < 3; c++)
            dv[9 * p + 3 * r + c] = FIXED ? double(acc_dvi[9 * p + 3 * c + r]) * 1e-8 : double(acc_dv[p][c][r]);
    }
  }

  void set_density(const double* rh) override {
    for (size_t p = 0; p < N; p++) {
      if (FIXED)
        rhoi[p] = (int)(float(rh[p]) * 1e6f);
      else
        rho[p] = R(rh[p]);
    }
  }

  void download_colliders(double* out) const override {
    for (size_t i = 0; i < cpos.size(); i++)
      for (int k = 0; k < 3; k++) out[3 * i + k] = double(cpos[i][k]);
  }
};

}  // namespace

extern "C" {

enum { ORACLE_FAITHFUL32 = 0, ORACLE_EXACT64 = 1, ORACLE_EXACT32 = 2, ORACLE_FAITHFUL64 = 3 };

void* oracle_create(const OracleDesc* d, int mode) {
  switch (mode) {
    case ORACLE_FAITHFUL32: return static_cast<OracleBase*>(new Oracle<float, true>(d));
    case ORACLE_EXACT64: return static_cast<OracleBase*>(new Oracle<double, false>(d));
    case ORACLE_EXACT32: return static_cast<OracleBase*>(new Oracle<float, false>(d));
    case ORACLE_FAITHFUL64: return static_cast<OracleBase*>(new Oracle<double, true>(d));
    default: return nullptr;
  }
}
void oracle_destroy(void* h) { delete static_cast<OracleBase*>(h); }
void oracle_upload(void* h, const double* x, const double* v, const double* m, const double* FE, const double* FP,
                   size_t n) {
  static_cast<OracleBase*>(h)->upload(x, v, m, FE, FP, n);
}
void oracle_upload_std140(void* h, const float* pxm, const int* pv, const float* pFE, const float* pFP, size_t n) {
  static_cast<OracleBase*>(h)->upload_std140(pxm, pv, pFE, pFP, n);
}
void oracle_phase(void* h, int which, double dt) { static_cast<OracleBase*>(h)->phase(which, dt); }
// ExplicitTimeUpdate::init (explicittimeupdate.cpp:29-33)
void oracle_init(void* h) {
  OracleBase* o = static_cast<OracleBase*>(h);
  o->phase(PH_RESET, 0.0);
  o->phase(PH_GMASS, 0.0);
  o->phase(PH_PVOLUME, 0.0);
}
// ExplicitTimeUpdate::update (explicittimeupdate.cpp:36-63)
void oracle_step(void* h, double dt, int n_steps) {
  OracleBase* o = static_cast<OracleBase*>(h);
  for (int s = 0; s < n_steps; s++) {
    o->phase(PH_RIGID, dt);
    o->phase(PH_RESET, dt);
    o->phase(PH_P2G, dt);
    o->phase(PH_GRID, dt);
    o->phase(PH_IMPLICIT, dt);  // no-op unless a semi-implicit update was set
    o->phase(PH_G2P, dt);
    o->phase(PH_ADVANCE, dt);
  }
}
void oracle_download(void* h, double* x, double* v, double* m, double* FE, double* FP, double* rho) {
  static_cast<OracleBase*>(h)->download(x, v, m, FE, FP, rho);
}
void oracle_download_std140(void* h, float* pxm, int* pv, float* pFE, float* pFP) {
  static_cast<OracleBase*>(h)->download_std140(pxm, pv, pFE, pFP);
}
void oracle_download_grid(void* h, double* mass, double* mom, double* force, double* vstar) {
  static_cast<OracleBase*>(h)->download_grid(mass, mom, force, vstar);
}
void oracle_download_grid_fixed(void* h, int* gv, int* gf) {
  static_cast<OracleBase*>(h)->download_grid_fixed(gv, gf);
}
void oracle_download_accumulators(void* h, double* vpic, double* dv) {
  static_cast<OracleBase*>(h)->download_accumulators(vpic, dv);
}
void oracle_set_density(void* h, const double* rho) { static_cast<OracleBase*>(h)->set_density(rho); }
void oracle_download_colliders(void* h, double* pos) { static_cast<OracleBase*>(h)->download_colliders(pos); }
// Semi-implicit velocity update: beta = 0 keeps the explicit step.
void oracle_set_implicit(void* h, double beta, double tol, int max_iters) {
  static_cast<OracleBase*>(h)->set_implicit(beta, tol, max_iters);
}
// K u on the dense grid (G x 3) for the current particle state.
void oracle_hessian(void* h, const double* u, double* out) { static_cast<OracleBase*>(h)->hessian(u, out); }
// The grid force with every particle's F_E deformed by eps u (G x 3).
void oracle_force_at(void* h, const double* u, double eps, double* out) {
  static_cast<OracleBase*>(h)->force_at(u, eps, out);
}
// (iterations, final relative residual, initial relative residual) of the
// last solve.
void oracle_solver_report(void* h, double* out) { static_cast<OracleBase*>(h)->solver_report(out); }
void oracle_flip_scale(void* h, double* out) { static_cast<OracleBase*>(h)->flip_scale(out); }

// 3x3 SVD of row-major matrices (KAT / property tests): A = W S V^T.
void oracle_svd(const double* a, double* w, double* s, double* vmat, int n, int fp64, int vround) {
  for (int i = 0; i < n; i++) {
    if (fp64) {
      M3<double> A, W, S, V;
      for (int r = 0; r < 3; r++)
        for (int c = 0; c < 3; c++) A[c][r] = a[9 * i + 3 * r + c];
      svd3(A, W, S, V, vround != 0);
      for (int r = 0; r < 3; r++)
        for (int c = 0; c < 3; c++) {
          w[9 * i + 3 * r + c] = W[c][r];
          s[9 * i + 3 * r + c] = S[c][r];
          vmat[9 * i + 3 * r + c] = V[c][r];
        }
    } else {
      M3<float> A, W, S, V;
      for (int r = 0; r < 3; r++)
        for (int c = 0; c < 3; c++) A[c][r] = float(a[9 * i + 3 * r + c]);
      svd3(A, W, S, V, vround != 0);
      for (int r = 0; r < 3; r++)
        for (int c = 0; c < 3; c++) {
          w[9 * i + 3 * r + c] = W[c][r];
          s[9 * i + 3 * r + c] = S[c][r];
          vmat[9 * i + 3 * r + c] = V[c][r];
        }
    }
  }
}

// Lame parameters (lame.include.glsl:11-27) in FP32, for the comment KATs.
void oracle_lame(float young, float poisson, float hardening, float jp, float* mu, float* lambda) {
  *mu = young / (2.0f * (1.0f + poisson)) * g_exp(hardening * (1.0f - jp));
  *lambda = young * poisson / ((1.0f + poisson) * (1.0f - 2.0f * poisson)) * g_exp(hardening * (1.0f - jp));
}

// Cell keys and the particle -> cell binning (stable sort by key), the CPU
// side of the bit-exact check of the GPU binning. The cell is the shaders'
// ivec3((x - gGridPos) / gridSpacing) in FP32 (p2gTransfer.glsl:76-81),
// clamped into the grid. Two keys are produced:
//   linear_key = i + j*X + k*X*Y                   (gridIndex.include.glsl:7-9)
//   block_key  = block(i>>2, j>>2, k>>2) * 64 + (i&3) + 4*(j&3) + 16*(k&3),
//                blocks numbered x fastest over ceil(X/4) x ceil(Y/4) x ceil(Z/4).
// perm lists particle indices in stable order of block_key.
void oracle_cell_keys(const float* x, size_t n, const float* grid_pos, const int* dim, float h,
                      uint32_t* linear_key, uint32_t* block_key, uint32_t* perm) {
  const uint32_t BX = (uint32_t)(dim[0] + 3) / 4, BY = (uint32_t)(dim[1] + 3) / 4;
  for (size_t p = 0; p < n; p++) {
    int c[3];
    for (int k = 0; k < 3; k++) {
      int v = (int)((x[3 * p + k] - grid_pos[k]) / h);
      v = v < 0 ? 0 : (v > dim[k] - 1 ? dim[k] - 1 : v);
      c[k] = v;
    }
    if (linear_key) linear_key[p] = (uint32_t)(c[0] + c[1] * dim[0] + c[2] * dim[1] * dim[0]);
    const uint32_t b = ((uint32_t)(c[2] >> 2) * BY + (uint32_t)(c[1] >> 2)) * BX + (uint32_t)(c[0] >> 2);
    block_key[p] = b * 64u + (uint32_t)(c[0] & 3) + 4u * (uint32_t)(c[1] & 3) + 16u * (uint32_t)(c[2] & 3);
  }
  if (perm) {
    std::vector<uint32_t> idx(n);
    std::iota(idx.begin(), idx.end(), 0u);
    std::stable_sort(idx.begin(), idx.end(), [&](uint32_t a, uint32_t b) { return block_key[a] < block_key[b]; });
    std::memcpy(perm, idx.data(), sizeof(uint32_t) * n);
  }
}

}  // extern "C"
