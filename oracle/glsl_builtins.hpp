// ORACLE / TEST INFRASTRUCTURE ONLY. Nothing in the product links this file.
//
// The GLSL built-ins whose results the GLSL 4.40 specification leaves to the
// implementation, pinned to one definition. Both CPU paths of the oracle use
// these same definitions:
//   * glsl_compat.hpp (the reference's compute shaders compiled as C++), and
//   * snow_oracle.cpp (this project's restatement of those shaders),
// so that the two agree to the bit in FP32 and the choice is made once.
//
// Choices (GLSL 4.40 spec sections 8.3, 8.5, 8.6):
//   round(x)        -> round half to even (nearbyint under the default
//                      rounding mode); GLSL allows either direction on ties.
//   inversesqrt(x)  -> 1 / sqrt(x), both correctly rounded.
//   normalize(v)    -> v / length(v), length(v) = sqrt(dot(v, v)).
//   dot(a, b)       -> a.x*b.x + a.y*b.y + a.z*b.z, left to right.
//   determinant(M)  -> cofactor expansion along the first row (see det3).
//   max(x, y)       -> (x < y) ? y : x.
//   mat*mat, mat*vec-> sum over k = 0, 1, 2 in that order.
#pragma once
#include <cmath>

namespace glslb {

inline float  g_round(float x)  { return std::nearbyint(x); }
inline double g_round(double x) { return std::nearbyint(x); }

inline float  g_inversesqrt(float x)  { return 1.0f / std::sqrt(x); }
inline double g_inversesqrt(double x) { return 1.0 / std::sqrt(x); }

inline float  g_exp(float x)  { return std::exp(x); }
inline double g_exp(double x) { return std::exp(x); }

template <class R> inline R g_max(R x, R y) { return (x < y) ? y : x; }

// Determinant of a 3x3 matrix given as m[c][r] (GLSL column-major indexing):
//   m00*(m11*m22 - m21*m12) - m10*(m01*m22 - m21*m02) + m20*(m01*m12 - m11*m02)
template <class M, class R>
inline R det3_cm(const M& m) {
  return m[0][0] * (m[1][1] * m[2][2] - m[2][1] * m[1][2]) -
         m[1][0] * (m[0][1] * m[2][2] - m[2][1] * m[0][2]) +
         m[2][0] * (m[0][1] * m[1][2] - m[1][1] * m[0][2]);
}

}  // namespace glslb
