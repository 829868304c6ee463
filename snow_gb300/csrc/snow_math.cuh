// Device math shared by the snow MPM kernels: column-major 3x3 algebra, the
// cubic B-spline of shader/compute/interpolation/cubic.include.glsl:7-40,
// the Lame parameters of shader/compute/lame/lame.include.glsl:11-27 and the
// quaternion-Jacobi 3x3 SVD of shader/compute/svd/SVD.include.glsl (McAdams
// et al. 2011, "Computing the singular value decomposition of 3x3 matrices
// with minimal branching and elementary floating point operations").
//
// Every routine is templated on FAITHFUL:
//   true  -> the shaders' operation order, the 1e-5 rounding of V inside the
//            SVD and 1/sqrt(x) for inversesqrt; the reference-mode kernels
//            are compiled without FMA contraction so each operation rounds
//            as in the shaders;
//   false -> the same algorithm for the FP32 fast path: rsqrtf, FMA, no
//            rounding of V.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace snow {

struct M3 {
  float m[3][3];  // m[c][r]: column c, row r (GLSL mat3 layout)
};

__device__ __forceinline__ M3 m3_diag(float s) {
  M3 a;
#pragma unroll
  for (int c = 0; c < 3; c++)
#pragma unroll
    for (int r = 0; r < 3; r++) a.m[c][r] = (c == r) ? s : 0.0f;
  return a;
}

// (A*B)[c][r] = A[0][r]*B[c][0] + A[1][r]*B[c][1] + A[2][r]*B[c][2]
__device__ __forceinline__ M3 m3_mul(const M3& a, const M3& b) {
  M3 o;
#pragma unroll
  for (int c = 0; c < 3; c++)
#pragma unroll
    for (int r = 0; r < 3; r++) o.m[c][r] = a.m[0][r] * b.m[c][0] + a.m[1][r] * b.m[c][1] + a.m[2][r] * b.m[c][2];
  return o;
}
// A * B^T
__device__ __forceinline__ M3 m3_mul_bt(const M3& a, const M3& b) {
  M3 o;
#pragma unroll
  for (int c = 0; c < 3; c++)
#pragma unroll
    for (int r = 0; r < 3; r++) o.m[c][r] = a.m[0][r] * b.m[0][c] + a.m[1][r] * b.m[1][c] + a.m[2][r] * b.m[2][c];
  return o;
}
// A^T * B
__device__ __forceinline__ M3 m3_mul_at(const M3& a, const M3& b) {
  M3 o;
#pragma unroll
  for (int c = 0; c < 3; c++)
#pragma unroll
    for (int r = 0; r < 3; r++) o.m[c][r] = a.m[r][0] * b.m[c][0] + a.m[r][1] * b.m[c][1] + a.m[r][2] * b.m[c][2];
  return o;
}
__device__ __forceinline__ M3 m3_transpose(const M3& a) {
  M3 o;
#pragma unroll
  for (int c = 0; c < 3; c++)
#pragma unroll
    for (int r = 0; r < 3; r++) o.m[c][r] = a.m[r][c];
  return o;
}
// GLSL determinant, cofactor expansion along the first row (m[c][r]).
__device__ __forceinline__ float m3_det(const M3& a) {
  const float (*m)[3] = a.m;
  return m[0][0] * (m[1][1] * m[2][2] - m[2][1] * m[1][2]) - m[1][0] * (m[0][1] * m[2][2] - m[2][1] * m[0][2]) +
         m[2][0] * (m[0][1] * m[1][2] - m[1][1] * m[0][2]);
}

template <bool FAITHFUL>
__device__ __forceinline__ float inv_sqrt(float x) {
  if (FAITHFUL) return 1.0f / sqrtf(x);
  return rsqrtf(x);
}

// 1/sqrt(x) to FP32 rounding: the hardware estimate refined by one
// Newton-Raphson step y <- y (3 - x y^2) / 2.
__device__ __forceinline__ float rsqrt_nr(float x) {
  const float y = rsqrtf(x);
  return y * (1.5f - 0.5f * x * y * y);
}

// Rescales a quaternion to unit length. The FAST path applies it before a
// quaternion becomes a matrix: the shaders' rotations are exact only when the
// accumulated quaternion stays unit, and with approximate 1/sqrt its length
// drifts by ~1e-7 per Givens step, which would leave V and W non-orthogonal.
__device__ __forceinline__ void quat_normalize(float q[4]) {
  const float s = rsqrt_nr(q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3]);
#pragma unroll
  for (int i = 0; i < 4; i++) q[i] *= s;
}

// round(s*x)/s with round = ties-to-even (the oracle pins GLSL round that way)
__device__ __forceinline__ float quantize(float x, float s) { return rintf(s * x) / s; }

// ---- cubic B-spline, cubic.include.glsl:7-40 ------------------------------
__device__ __forceinline__ float bspline(float x) {
  const float ax = fabsf(x);
  if (ax < 1.0f) return 0.5f * ax * ax * ax - x * x + 2.0f / 3.0f;
  if (ax < 2.0f) return -1.0f / 6.0f * ax * ax * ax + x * x - 2.0f * ax + 4.0f / 3.0f;
  return 0.0f;
}
__device__ __forceinline__ float bspline_d(float x) {
  const float ax = fabsf(x);
  if (ax < 1.0f) return 1.5f * x * ax - 2.0f * x;
  if (ax < 2.0f) return -1.0f / 2.0f * ax * x + 2.0f * x - 2.0f * x / ax;
  return 0.0f;
}

// ---- SVD.include.glsl --------------------------------------------------------
#define SNOW_SVD_GAMMA 5.828427124f
#define SNOW_SVD_CSTAR 0.923879532f
#define SNOW_SVD_SSTAR 0.3826834323f
#define SNOW_SVD_EPS 1e-6f

__device__ __forceinline__ M3 quat_to_m3(const float q[4]) {
  const float qxx = q[1] * q[1], qyy = q[2] * q[2], qzz = q[3] * q[3];
  const float qxz = q[1] * q[3], qxy = q[1] * q[2], qyz = q[2] * q[3];
  const float qwx = q[0] * q[1], qwy = q[0] * q[2], qwz = q[0] * q[3];
  M3 m;
  m.m[0][0] = 1.0f - 2.0f * (qyy + qzz);
  m.m[0][1] = 2.0f * (qxy + qwz);
  m.m[0][2] = 2.0f * (qxz - qwy);
  m.m[1][0] = 2.0f * (qxy - qwz);
  m.m[1][1] = 1.0f - 2.0f * (qxx + qzz);
  m.m[1][2] = 2.0f * (qyz + qwx);
  m.m[2][0] = 2.0f * (qxz + qwy);
  m.m[2][1] = 2.0f * (qyz - qwx);
  m.m[2][2] = 1.0f - 2.0f * (qxx + qyy);
  return m;
}

// One approximate Givens conjugation (SVD.include.glsl:71-128). The
// symmetric matrix is relabelled cyclically so that each call works on the
// (0,1) pair; (X, Y, Z) names the original axes for the quaternion update.
template <bool FAITHFUL, int X, int Y, int Z>
__device__ __forceinline__ void jacobi_step(M3& S, float q[4]) {
  float ch = 2.0f * (S.m[0][0] - S.m[1][1]);
  float ch2 = ch * ch;
  float sh = S.m[0][1];
  float sh2 = sh * sh;
  const bool exact = SNOW_SVD_GAMMA * sh2 < ch2;
  const float w = inv_sqrt<FAITHFUL>(ch2 + sh2);
  ch = exact ? w * ch : SNOW_SVD_CSTAR;
  sh = exact ? w * sh : SNOW_SVD_SSTAR;
  ch2 = ch * ch;
  sh2 = sh * sh;
  const float scale = FAITHFUL ? 1.0f / (ch2 + sh2) : __fdividef(1.0f, ch2 + sh2);
  const float a = (ch2 - sh2) * scale;
  const float b = (2.0f * sh * ch) * scale;
  const float a2 = a * a, b2 = b * b, ab = a * b;
  const float s0 = a2 * S.m[0][0] + 2.0f * ab * S.m[1][0] + b2 * S.m[1][1];
  const float s2 = a * S.m[2][0] + b * S.m[2][1];
  const float s3 = (a2 - b2) * S.m[1][0] + ab * (S.m[1][1] - S.m[0][0]);
  const float s4 = b2 * S.m[0][0] - 2.0f * ab * S.m[1][0] + a2 * S.m[1][1];
  const float s5 = a * S.m[1][2] - b * S.m[0][2];
  const float s8 = S.m[2][2];
  S.m[0][0] = s4; S.m[0][1] = s5; S.m[0][2] = s3;
  S.m[1][0] = s5; S.m[1][1] = s8; S.m[1][2] = s2;
  S.m[2][0] = s3; S.m[2][1] = s2; S.m[2][2] = s0;
  const float t[3] = {sh * q[1], sh * q[2], sh * q[3]};
  sh *= q[0];
#pragma unroll
  for (int i = 0; i < 4; i++) q[i] *= ch;
  q[Z + 1] += sh;
  q[0] -= t[Z];
  q[X + 1] += t[Y];
  q[Y + 1] -= t[X];
}

template <bool FAITHFUL>
__device__ __forceinline__ void jacobi_eigen(M3& S, float q[4]) {
  q[0] = 1.0f; q[1] = 0.0f; q[2] = 0.0f; q[3] = 0.0f;
#pragma unroll
  for (int sweep = 0; sweep < 4; sweep++) {
    jacobi_step<FAITHFUL, 0, 1, 2>(S, q);
    jacobi_step<FAITHFUL, 1, 2, 0>(S, q);
    jacobi_step<FAITHFUL, 2, 0, 1>(S, q);
  }
}

__device__ __forceinline__ void cond_neg_swap_cols(bool c, M3& B, int i, int j) {
#pragma unroll
  for (int r = 0; r < 3; r++) {
    const float bi = B.m[i][r], bj = B.m[j][r];
    B.m[i][r] = c ? bj : bi;
    B.m[j][r] = c ? -bi : bj;
  }
}

// SVD.include.glsl:191-228: order columns of B = A V by decreasing norm,
// swapping with a sign flip so V stays a rotation.
__device__ __forceinline__ void sort_singular(M3& B, M3& V) {
  float rho1 = B.m[0][0] * B.m[0][0] + B.m[0][1] * B.m[0][1] + B.m[0][2] * B.m[0][2];
  float rho2 = B.m[1][0] * B.m[1][0] + B.m[1][1] * B.m[1][1] + B.m[1][2] * B.m[1][2];
  float rho3 = B.m[2][0] * B.m[2][0] + B.m[2][1] * B.m[2][1] + B.m[2][2] * B.m[2][2];
  bool c = rho1 < rho2;
  cond_neg_swap_cols(c, B, 0, 1);
  cond_neg_swap_cols(c, V, 0, 1);
  {
    const float t = rho1;
    rho1 = c ? rho2 : rho1;
    rho2 = c ? t : rho2;
  }
  c = rho1 < rho3;
  cond_neg_swap_cols(c, B, 0, 2);
  cond_neg_swap_cols(c, V, 0, 2);
  {
    const float t = rho1;
    rho1 = c ? rho3 : rho1;
    rho3 = c ? t : rho3;
  }
  c = rho2 < rho3;
  cond_neg_swap_cols(c, B, 1, 2);
  cond_neg_swap_cols(c, V, 1, 2);
}

template <bool FAITHFUL>
__device__ __forceinline__ void givens_quat(float a1, float a2, float& ch, float& sh) {
  const float rho = sqrtf(a1 * a1 + a2 * a2);
  sh = rho > SNOW_SVD_EPS ? a2 : 0.0f;
  ch = fabsf(a1) + (rho < SNOW_SVD_EPS ? SNOW_SVD_EPS : rho);
  const bool b = a1 < 0.0f;
  const float t = sh;
  sh = b ? ch : sh;
  ch = b ? t : ch;
  const float w = inv_sqrt<FAITHFUL>(ch * ch + sh * sh);
  ch *= w;
  sh *= w;
}

// Left-multiplies R by the transpose of a Givens rotation acting on rows
// (i, j): the U^T * R of SVD.include.glsl:273, :296, :316.
__device__ __forceinline__ void givens_apply_t(M3& R, int i, int j, float s0, float s1) {
#pragma unroll
  for (int c = 0; c < 3; c++) {
    const float ri = R.m[c][i], rj = R.m[c][j];
    R.m[c][i] = s0 * ri + s1 * rj;
    R.m[c][j] = -s1 * ri + s0 * rj;
  }
}

// SVD.include.glsl:253-332: QR of B by three Givens rotations; Q is rebuilt
// from the accumulated quaternion.
template <bool FAITHFUL>
__device__ __forceinline__ void qr_givens(const M3& B, M3& Q, M3& R) {
  R = B;
  float ch, sh, s0, s1, q[4];
  givens_quat<FAITHFUL>(R.m[0][0], R.m[0][1], ch, sh);
  s0 = 1.0f - 2.0f * sh * sh;
  s1 = 2.0f * sh * ch;
  if (FAITHFUL) {
    M3 U;
    U.m[0][0] = s0; U.m[0][1] = s1; U.m[0][2] = 0.0f;
    U.m[1][0] = -s1; U.m[1][1] = s0; U.m[1][2] = 0.0f;
    U.m[2][0] = 0.0f; U.m[2][1] = 0.0f; U.m[2][2] = 1.0f;
    R = m3_mul(m3_transpose(U), R);
  } else {
    givens_apply_t(R, 0, 1, s0, s1);
  }
  q[0] = ch; q[1] = 0.0f; q[2] = 0.0f; q[3] = sh;
  if (FAITHFUL) {  // the shader's general update from the identity quaternion
    q[0] = ch * 1.0f - sh * 0.0f;
    q[1] = ch * 0.0f + sh * 0.0f;
    q[2] = ch * 0.0f - sh * 0.0f;
    q[3] = sh * 1.0f + ch * 0.0f;
  }
  givens_quat<FAITHFUL>(R.m[0][0], R.m[0][2], ch, sh);
  s0 = 1.0f - 2.0f * sh * sh;
  s1 = 2.0f * sh * ch;
  if (FAITHFUL) {
    M3 U;
    U.m[0][0] = s0; U.m[0][1] = 0.0f; U.m[0][2] = s1;
    U.m[1][0] = 0.0f; U.m[1][1] = 1.0f; U.m[1][2] = 0.0f;
    U.m[2][0] = -s1; U.m[2][1] = 0.0f; U.m[2][2] = s0;
    R = m3_mul(m3_transpose(U), R);
  } else {
    givens_apply_t(R, 0, 2, s0, s1);
  }
  {
    const float q0 = ch * q[0] + sh * q[2], q1 = ch * q[1] + sh * q[3];
    const float q2 = ch * q[2] - sh * q[0], q3 = ch * q[3] - sh * q[1];
    q[0] = q0; q[1] = q1; q[2] = q2; q[3] = q3;
  }
  givens_quat<FAITHFUL>(R.m[1][1], R.m[1][2], ch, sh);
  s0 = 1.0f - 2.0f * sh * sh;
  s1 = 2.0f * sh * ch;
  if (FAITHFUL) {
    M3 U;
    U.m[0][0] = 1.0f; U.m[0][1] = 0.0f; U.m[0][2] = 0.0f;
    U.m[1][0] = 0.0f; U.m[1][1] = s0; U.m[1][2] = s1;
    U.m[2][0] = 0.0f; U.m[2][1] = -s1; U.m[2][2] = s0;
    R = m3_mul(m3_transpose(U), R);
  } else {
    givens_apply_t(R, 1, 2, s0, s1);
  }
  {
    const float q0 = ch * q[0] - sh * q[1], q1 = sh * q[0] + ch * q[1];
    const float q2 = ch * q[2] + sh * q[3], q3 = ch * q[3] - sh * q[2];
    q[0] = q0; q[1] = q1; q[2] = q2; q[3] = q3;
  }
  if (!FAITHFUL) quat_normalize(q);
  Q = quat_to_m3(q);
}

// A = W S V^T (SVD.include.glsl:334-371). S is the upper-triangular QR
// factor of A V; its diagonal holds the singular values.
template <bool FAITHFUL>
__device__ __forceinline__ void svd3(const M3& A, M3& W, M3& S, M3& V) {
  M3 ata = m3_mul_at(A, A);  // A^T A, the shader's transpose(A) * A
  float q[4];
  jacobi_eigen<FAITHFUL>(ata, q);
  if (!FAITHFUL) quat_normalize(q);
  V = quat_to_m3(q);
  if (FAITHFUL) {
#pragma unroll
    for (int c = 0; c < 3; c++)
#pragma unroll
      for (int r = 0; r < 3; r++) V.m[c][r] = quantize(V.m[c][r], 1e5f);
  }
  M3 B = m3_mul(A, V);
  sort_singular(B, V);
  qr_givens<FAITHFUL>(B, W, S);
}

// FAST path only: the Jacobi eigen-solve of A^T A started from the frame q
// of the particle's previous step (in: that frame, out: the new one). F_E
// changes little per step, so Q^T A^T A Q is nearly diagonal and one or two
// sweeps reach the convergence the four cold sweeps give; sweeps stop once
// the off-diagonal part is below 1e-6 of the diagonal (at most 4). Returns V
// (the eigenvectors, unsorted) and lam, the eigenvalues sigma_i^2 in V's
// column order.
__device__ __forceinline__ void eigen_warm(const M3& A, float q[4], M3& V, float lam[3]) {
  const M3 ata = m3_mul_at(A, A);
  quat_normalize(q);
  const M3 Q = quat_to_m3(q);
  const M3 t = m3_mul(m3_mul_at(Q, ata), Q);  // Q^T A^T A Q
  M3 sym;
#pragma unroll
  for (int c = 0; c < 3; c++)
#pragma unroll
    for (int r = 0; r < 3; r++) sym.m[c][r] = r <= c ? t.m[c][r] : t.m[r][c];
#pragma unroll 1
  for (int sweep = 0; sweep < 4; sweep++) {
    const float off = sym.m[1][0] * sym.m[1][0] + sym.m[2][0] * sym.m[2][0] + sym.m[2][1] * sym.m[2][1];
    const float dia = sym.m[0][0] * sym.m[0][0] + sym.m[1][1] * sym.m[1][1] + sym.m[2][2] * sym.m[2][2];
    if (off <= 1e-12f * dia) break;
    jacobi_step<false, 0, 1, 2>(sym, q);
    jacobi_step<false, 1, 2, 0>(sym, q);
    jacobi_step<false, 2, 0, 1>(sym, q);
  }
  quat_normalize(q);
  V = quat_to_m3(q);
  lam[0] = sym.m[0][0];
  lam[1] = sym.m[1][1];
  lam[2] = sym.m[2][2];
}

// ---- lame.include.glsl:11-27 -------------------------------------------------
__device__ __forceinline__ float lame_mu(float young, float poisson, float hardening, float jp) {
  return young / (2.0f * (1.0f + poisson)) * expf(hardening * (1.0f - jp));
}
__device__ __forceinline__ float lame_lambda(float young, float poisson, float hardening, float jp) {
  return young * poisson / ((1.0f + poisson) * (1.0f - 2.0f * poisson)) * expf(hardening * (1.0f - jp));
}

}  // namespace snow
