// ORACLE / TEST INFRASTRUCTURE ONLY. Nothing in the product links this file.
//
// A small GLSL 4.40 compute-shader environment for C++ (g++, GNU dialect):
// the vector / matrix types, swizzles, constructors and built-ins that the
// snow reference's compute shaders use (shader/compute/**.glsl), with GLSL
// semantics. oracle/ref_translate.py rewrites each shader's declarations
// (uniforms, SSBO blocks, inout parameters, float literals) and compiles the
// shader body unchanged against this header, so the reference's own kernel
// code runs on the host cores, one invocation at a time.
//
// GLSL semantics kept:
//   * mat3/mat4 are column-major: m[c] is column c, m[c][r] row r.
//   * constructors: mat3(s) = s*I, mat4(mat3) fills the rest with identity,
//     mat3(mat4) takes the upper-left 3x3, vecN(ivecN) converts each
//     component, ivecN(vecN) truncates toward zero, vec3(ivec4) drops w.
//   * an int scalar accepts the .x swizzle (gGridDim[0].x).
//   * atomicAdd on an int SSBO member wraps in two's complement and is a
//     real atomic, so a dispatch may run its invocations on several threads.
// Implementation-defined built-ins are pinned in glsl_builtins.hpp.
#pragma once
#include <cmath>
#include <cstdint>

#include "glsl_builtins.hpp"

namespace glslc {

typedef unsigned int uint;

struct ivec3;
struct ivec4;
struct vec4;

// Reference to one int component, usable as an int and through GLSL's
// scalar swizzle ".x" (the shaders write gGridDim[0].x).
struct IComp {
  int& x;
  operator int() const { return x; }
};

struct vec3 {
  float x, y, z;
  vec3() = default;
  vec3(float a, float b, float c) : x(a), y(b), z(c) {}
  explicit vec3(float s) : x(s), y(s), z(s) {}
  explicit vec3(const ivec3& v);
  explicit vec3(const ivec4& v);
  explicit vec3(const vec4& v);
  float& operator[](int i) { return (&x)[i]; }
  float operator[](int i) const { return (&x)[i]; }
  vec3& operator+=(const vec3& o) { x += o.x; y += o.y; z += o.z; return *this; }
  vec3& operator-=(const vec3& o) { x -= o.x; y -= o.y; z -= o.z; return *this; }
  vec3& operator*=(float s) { x *= s; y *= s; z *= s; return *this; }
};

struct ivec3 {
  int x, y, z;
  ivec3() = default;
  ivec3(int a, int b, int c) : x(a), y(b), z(c) {}
  explicit ivec3(const vec3& v) : x(int(v.x)), y(int(v.y)), z(int(v.z)) {}
  IComp operator[](int i) { return IComp{(&x)[i]}; }
  int operator[](int i) const { return (&x)[i]; }
};

struct uvec3 {
  uint x, y, z;
};

struct vec4 {
  union {
    struct { float x, y, z, w; };
    vec3 xyz;
    float c_[4];
  };
  vec4() = default;
  vec4(float a, float b, float c, float d) { x = a; y = b; z = c; w = d; }
  vec4(const vec3& v, float d) { x = v.x; y = v.y; z = v.z; w = d; }
  explicit vec4(float s) { x = y = z = w = s; }
  vec4(const ivec4& v);  // implicit int -> float conversion, as in GLSL
  float& operator[](int i) { return c_[i]; }
  float operator[](int i) const { return c_[i]; }
  vec4& operator*=(float s) { x *= s; y *= s; z *= s; w *= s; return *this; }
};

struct ivec4 {
  union {
    struct { int x, y, z, w; };
    ivec3 xyz;
    int c_[4];
  };
  ivec4() = default;
  ivec4(int a, int b, int c, int d) { x = a; y = b; z = c; w = d; }
  int& operator[](int i) { return c_[i]; }
  int operator[](int i) const { return c_[i]; }
};

inline vec3::vec3(const ivec3& v) : x(float(v.x)), y(float(v.y)), z(float(v.z)) {}
inline vec3::vec3(const ivec4& v) : x(float(v.x)), y(float(v.y)), z(float(v.z)) {}
inline vec3::vec3(const vec4& v) : x(v.x), y(v.y), z(v.z) {}
inline vec4::vec4(const ivec4& v) { x = float(v.x); y = float(v.y); z = float(v.z); w = float(v.w); }

inline ivec3 operator+(const ivec3& a, const ivec3& b) { return ivec3(a.x + b.x, a.y + b.y, a.z + b.z); }

inline vec3 operator+(const vec3& a, const vec3& b) { return vec3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline vec3 operator-(const vec3& a, const vec3& b) { return vec3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline vec3 operator-(const vec3& a) { return vec3(-a.x, -a.y, -a.z); }
inline vec3 operator*(const vec3& a, const vec3& b) { return vec3(a.x * b.x, a.y * b.y, a.z * b.z); }
inline vec3 operator*(const vec3& a, float s) { return vec3(a.x * s, a.y * s, a.z * s); }
inline vec3 operator*(float s, const vec3& a) { return vec3(s * a.x, s * a.y, s * a.z); }
inline vec3 operator/(const vec3& a, float s) { return vec3(a.x / s, a.y / s, a.z / s); }

struct mat3 {
  vec3 c[3];
  mat3() = default;
  explicit mat3(float s) {
    c[0] = vec3(s, 0.0f, 0.0f);
    c[1] = vec3(0.0f, s, 0.0f);
    c[2] = vec3(0.0f, 0.0f, s);
  }
  mat3(float a0, float a1, float a2, float b0, float b1, float b2, float c0, float c1, float c2) {
    c[0] = vec3(a0, a1, a2);
    c[1] = vec3(b0, b1, b2);
    c[2] = vec3(c0, c1, c2);
  }
  mat3(const vec3& a, const vec3& b, const vec3& d) { c[0] = a; c[1] = b; c[2] = d; }
  explicit mat3(const struct mat4& m);
  vec3& operator[](int i) { return c[i]; }
  const vec3& operator[](int i) const { return c[i]; }
};

struct mat4 {
  vec4 c[4];
  mat4() = default;
  explicit mat4(const mat3& m) {
    for (int i = 0; i < 3; i++) c[i] = vec4(m.c[i], 0.0f);
    c[3] = vec4(0.0f, 0.0f, 0.0f, 1.0f);
  }
  vec4& operator[](int i) { return c[i]; }
  const vec4& operator[](int i) const { return c[i]; }
};

inline mat3::mat3(const mat4& m) {
  for (int i = 0; i < 3; i++) c[i] = vec3(m.c[i].x, m.c[i].y, m.c[i].z);
}

inline mat3 operator+(const mat3& a, const mat3& b) {
  mat3 r;
  for (int i = 0; i < 3; i++) r.c[i] = a.c[i] + b.c[i];
  return r;
}
inline mat3 operator-(const mat3& a, const mat3& b) {
  mat3 r;
  for (int i = 0; i < 3; i++) r.c[i] = a.c[i] - b.c[i];
  return r;
}
inline mat3 operator*(float s, const mat3& a) {
  mat3 r;
  for (int i = 0; i < 3; i++) r.c[i] = s * a.c[i];
  return r;
}
inline mat3 operator*(const mat3& a, float s) {
  mat3 r;
  for (int i = 0; i < 3; i++) r.c[i] = a.c[i] * s;
  return r;
}
// (A*B)[c][r] = A[0][r]*B[c][0] + A[1][r]*B[c][1] + A[2][r]*B[c][2]
inline mat3 operator*(const mat3& a, const mat3& b) {
  mat3 r;
  for (int cc = 0; cc < 3; cc++)
    for (int rr = 0; rr < 3; rr++)
      r.c[cc][rr] = a.c[0][rr] * b.c[cc][0] + a.c[1][rr] * b.c[cc][1] + a.c[2][rr] * b.c[cc][2];
  return r;
}
inline vec3 operator*(const mat3& a, const vec3& v) {
  vec3 r;
  for (int rr = 0; rr < 3; rr++) r[rr] = a.c[0][rr] * v.x + a.c[1][rr] * v.y + a.c[2][rr] * v.z;
  return r;
}

// ---- built-in functions -------------------------------------------------
inline float abs(float x) { return std::fabs(x); }
inline int abs(int x) { return x < 0 ? -x : x; }
inline float exp(float x) { return glslb::g_exp(x); }
inline float sqrt(float x) { return std::sqrt(x); }
inline float inversesqrt(float x) { return glslb::g_inversesqrt(x); }
inline float round(float x) { return glslb::g_round(x); }
inline float max(float x, float y) { return glslb::g_max(x, y); }
inline float dot(const vec3& a, const vec3& b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline float length(const vec3& a) { return std::sqrt(dot(a, a)); }
inline vec3 normalize(const vec3& a) { return a / length(a); }
inline mat3 transpose(const mat3& m) {
  mat3 r;
  for (int cc = 0; cc < 3; cc++)
    for (int rr = 0; rr < 3; rr++) r.c[cc][rr] = m.c[rr][cc];
  return r;
}
inline float determinant(const mat3& m) { return glslb::det3_cm<mat3, float>(m); }

// GLSL atomicAdd on an int buffer member: atomic, two's-complement wrap.
inline int atomicAdd(int& mem, int data) { return __atomic_fetch_add(&mem, data, __ATOMIC_RELAXED); }

}  // namespace glslc

// Buffer bindings and uniform values handed to a translated shader's
// dispatch entry point (see ref_translate.py and ref_driver.cpp).
struct RefBindings {
  void* ptr[32];  // indexed by the shader's SSBO binding point
};
struct RefUniforms {
  float gGridPos[3];
  int gGridDim[3];
  float gridSpacing;
  float young, poisson, hardening;
  float critComp, critStretch;
  float dt;
  unsigned indexSize;
  unsigned gNumColliders;
};
