// Minimal vector-math shim standing in for the missing LiteMath library, written
// for compiling the reference's hot-path translation units in place (oracle
// pinning only; see oracle/build_ref.py).  Conventions match the oracle's
// restatement: float4x4 is row-major m(row, col), matrix * vector sums columns
// left to right, normalize(u) = u / length(u), sign(x) = x < 0 ? -1 : 1.
#pragma once
#include <cmath>
#include <cstdint>
#include <cstring>
#include <algorithm>

#undef M_PI
#undef M_TWOPI
namespace LiteMath {
typedef unsigned int uint;
constexpr float M_PI = 3.14159265358979323846f;
constexpr float M_TWOPI = 6.28318530717958647692f;
constexpr float DEG_TO_RAD = M_PI / 180.0f;
constexpr float INF_POSITIVE = +1e38f;
constexpr float INF_NEGATIVE = -1e38f;

using std::min;
using std::max;
using std::abs;
using std::sqrt;
using std::floor;

static inline float clamp(float u, float a, float b) { return std::min(std::max(a, u), b); }
static inline int clamp(int u, int a, int b) { return std::min(std::max(a, u), b); }
static inline uint clamp(uint u, uint a, uint b) { return std::min(std::max(a, u), b); }
static inline float sign(float a) { return a < 0.0f ? -1.0f : 1.0f; }
static inline float fract(float x) { return x - std::floor(x); }
static inline float lerp(float a, float b, float t) { return a + t * (b - a); }
static inline float mix(float a, float b, float t) { return a + t * (b - a); }
static inline float step(float edge, float x) { return x < edge ? 0.0f : 1.0f; }
static inline float smoothstep(float e0, float e1, float x) {
  float t = clamp((x - e0) / (e1 - e0), 0.0f, 1.0f);
  return t * t * (3.0f - 2.0f * t);
}
static inline float rnd(float, float) { return 0.0f; }

#define LM_VEC_OPS(V, T, N)                                                                              \
  static inline V operator+(V a, V b) { V r; for (int i = 0; i < N; i++) r[i] = a[i] + b[i]; return r; } \
  static inline V operator-(V a, V b) { V r; for (int i = 0; i < N; i++) r[i] = a[i] - b[i]; return r; } \
  static inline V operator*(V a, V b) { V r; for (int i = 0; i < N; i++) r[i] = a[i] * b[i]; return r; } \
  static inline V operator/(V a, V b) { V r; for (int i = 0; i < N; i++) r[i] = a[i] / b[i]; return r; } \
  static inline V operator+(V a, T b) { V r; for (int i = 0; i < N; i++) r[i] = a[i] + b; return r; }    \
  static inline V operator-(V a, T b) { V r; for (int i = 0; i < N; i++) r[i] = a[i] - b; return r; }    \
  static inline V operator*(V a, T b) { V r; for (int i = 0; i < N; i++) r[i] = a[i] * b; return r; }    \
  static inline V operator/(V a, T b) { V r; for (int i = 0; i < N; i++) r[i] = a[i] / b; return r; }    \
  static inline V operator+(T a, V b) { V r; for (int i = 0; i < N; i++) r[i] = a + b[i]; return r; }    \
  static inline V operator-(T a, V b) { V r; for (int i = 0; i < N; i++) r[i] = a - b[i]; return r; }    \
  static inline V operator*(T a, V b) { V r; for (int i = 0; i < N; i++) r[i] = a * b[i]; return r; }    \
  static inline V operator/(T a, V b) { V r; for (int i = 0; i < N; i++) r[i] = a / b[i]; return r; }    \
  static inline V &operator+=(V &a, V b) { for (int i = 0; i < N; i++) a[i] += b[i]; return a; }        \
  static inline V &operator-=(V &a, V b) { for (int i = 0; i < N; i++) a[i] -= b[i]; return a; }        \
  static inline V &operator*=(V &a, V b) { for (int i = 0; i < N; i++) a[i] *= b[i]; return a; }        \
  static inline V &operator/=(V &a, V b) { for (int i = 0; i < N; i++) a[i] /= b[i]; return a; }        \
  static inline V &operator+=(V &a, T b) { for (int i = 0; i < N; i++) a[i] += b; return a; }           \
  static inline V &operator-=(V &a, T b) { for (int i = 0; i < N; i++) a[i] -= b; return a; }           \
  static inline V &operator*=(V &a, T b) { for (int i = 0; i < N; i++) a[i] *= b; return a; }           \
  static inline V &operator/=(V &a, T b) { for (int i = 0; i < N; i++) a[i] /= b; return a; }           \
  static inline V min(V a, V b) { V r; for (int i = 0; i < N; i++) r[i] = std::min(a[i], b[i]); return r; } \
  static inline V max(V a, V b) { V r; for (int i = 0; i < N; i++) r[i] = std::max(a[i], b[i]); return r; } \
  static inline V clamp(V u, T a, T b) { V r; for (int i = 0; i < N; i++) r[i] = clamp(u[i], a, b); return r; } \
  static inline V clamp(V u, V a, V b) { V r; for (int i = 0; i < N; i++) r[i] = clamp(u[i], a[i], b[i]); return r; } \
  static inline bool operator==(V a, V b) { for (int i = 0; i < N; i++) if (!(a[i] == b[i])) return false; return true; } \
  static inline bool operator!=(V a, V b) { return !(a == b); }

template <typename T, int N> struct VecBase {};

struct float3;
struct float4;
struct int2 { int x, y; int2() : x(0), y(0) {} int2(int a, int b) : x(a), y(b) {} explicit int2(int a) : x(a), y(a) {}
  int &operator[](int i) { return (&x)[i]; } int operator[](int i) const { return (&x)[i]; } };
struct int3 { int x, y, z; int3() : x(0), y(0), z(0) {} int3(int a, int b, int c) : x(a), y(b), z(c) {} explicit int3(int a) : x(a), y(a), z(a) {}
  explicit int3(const float3 &f);
  int &operator[](int i) { return (&x)[i]; } int operator[](int i) const { return (&x)[i]; } };
struct int4 { int x, y, z, w; int4() : x(0), y(0), z(0), w(0) {} int4(int a, int b, int c, int d) : x(a), y(b), z(c), w(d) {} explicit int4(int a) : x(a), y(a), z(a), w(a) {}
  int &operator[](int i) { return (&x)[i]; } int operator[](int i) const { return (&x)[i]; } };
struct uint2 { uint x, y; uint2() : x(0), y(0) {} uint2(uint a, uint b) : x(a), y(b) {} explicit uint2(uint a) : x(a), y(a) {}
  uint &operator[](int i) { return (&x)[i]; } uint operator[](int i) const { return (&x)[i]; } };
struct uint3 { uint x, y, z; uint3() : x(0), y(0), z(0) {} uint3(uint a, uint b, uint c) : x(a), y(b), z(c) {} explicit uint3(uint a) : x(a), y(a), z(a) {}
  explicit uint3(const float3 &f);
  uint &operator[](int i) { return (&x)[i]; } uint operator[](int i) const { return (&x)[i]; } };
struct uint4 { uint x, y, z, w; uint4() : x(0), y(0), z(0), w(0) {} uint4(uint a, uint b, uint c, uint d) : x(a), y(b), z(c), w(d) {} explicit uint4(uint a) : x(a), y(a), z(a), w(a) {}
  explicit uint4(const float4 &f);
  uint &operator[](int i) { return (&x)[i]; } uint operator[](int i) const { return (&x)[i]; } };

struct float2 {
  float x, y;
  float2() : x(0), y(0) {}
  float2(float a, float b) : x(a), y(b) {}
  explicit float2(float a) : x(a), y(a) {}
  float &operator[](int i) { return (&x)[i]; }
  float operator[](int i) const { return (&x)[i]; }
};
struct float3 {
  float x, y, z;
  float3() : x(0), y(0), z(0) {}
  float3(float a, float b, float c) : x(a), y(b), z(c) {}
  explicit float3(float a) : x(a), y(a), z(a) {}
  explicit float3(int3 v) : x(float(v.x)), y(float(v.y)), z(float(v.z)) {}
  explicit float3(uint3 v) : x(float(v.x)), y(float(v.y)), z(float(v.z)) {}
  float &operator[](int i) { return (&x)[i]; }
  float operator[](int i) const { return (&x)[i]; }
};
struct float4 {
  float x, y, z, w;
  float4() : x(0), y(0), z(0), w(0) {}
  float4(float a, float b, float c, float d) : x(a), y(b), z(c), w(d) {}
  explicit float4(float a) : x(a), y(a), z(a), w(a) {}
  float &operator[](int i) { return (&x)[i]; }
  float operator[](int i) const { return (&x)[i]; }
};
// float -> integer vector conversions (truncation)
inline int3::int3(const float3 &f) : x(int(f.x)), y(int(f.y)), z(int(f.z)) {}
inline uint3::uint3(const float3 &f) : x(uint(f.x)), y(uint(f.y)), z(uint(f.z)) {}
inline uint4::uint4(const float4 &f) : x(uint(f.x)), y(uint(f.y)), z(uint(f.z)), w(uint(f.w)) {}
LM_VEC_OPS(float2, float, 2)
LM_VEC_OPS(float3, float, 3)
LM_VEC_OPS(float4, float, 4)
LM_VEC_OPS(int2, int, 2)
LM_VEC_OPS(int3, int, 3)
LM_VEC_OPS(int4, int, 4)
LM_VEC_OPS(uint2, uint, 2)
LM_VEC_OPS(uint3, uint, 3)
LM_VEC_OPS(uint4, uint, 4)

static inline float2 operator-(float2 a) { return float2(-a.x, -a.y); }
static inline float3 operator-(float3 a) { return float3(-a.x, -a.y, -a.z); }
static inline float4 operator-(float4 a) { return float4(-a.x, -a.y, -a.z, -a.w); }

static inline float dot(float2 a, float2 b) { return a.x * b.x + a.y * b.y; }
static inline float dot(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline float dot(float4 a, float4 b) { return a.x * b.x + a.y * b.y + a.z * b.z + a.w * b.w; }
static inline float3 cross(float3 a, float3 b) { return float3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
static inline float length(float2 a) { return std::sqrt(dot(a, a)); }
static inline float length(float3 a) { return std::sqrt(dot(a, a)); }
static inline float length(float4 a) { return std::sqrt(dot(a, a)); }
static inline float2 normalize(float2 a) { return a / length(a); }
static inline float3 normalize(float3 a) { return a / length(a); }
static inline float4 normalize(float4 a) { return a / length(a); }
static inline float2 abs(float2 a) { return float2(std::abs(a.x), std::abs(a.y)); }
static inline float3 abs(float3 a) { return float3(std::abs(a.x), std::abs(a.y), std::abs(a.z)); }
static inline float4 abs(float4 a) { return float4(std::abs(a.x), std::abs(a.y), std::abs(a.z), std::abs(a.w)); }
static inline float2 floor(float2 a) { return float2(std::floor(a.x), std::floor(a.y)); }
static inline float3 floor(float3 a) { return float3(std::floor(a.x), std::floor(a.y), std::floor(a.z)); }
static inline float4 floor(float4 a) { return float4(std::floor(a.x), std::floor(a.y), std::floor(a.z), std::floor(a.w)); }
static inline float3 sign(float3 a) { return float3(sign(a.x), sign(a.y), sign(a.z)); }
static inline float4 sign(float4 a) { return float4(sign(a.x), sign(a.y), sign(a.z), sign(a.w)); }
static inline float3 lerp(float3 a, float3 b, float t) { return a + t * (b - a); }
static inline float4 lerp(float4 a, float4 b, float t) { return a + t * (b - a); }
static inline float3 mix(float3 a, float3 b, float t) { return a + t * (b - a); }
static inline float3 fract(float3 a) { return float3(fract(a.x), fract(a.y), fract(a.z)); }
static inline float3 sqrt(float3 a) { return float3(std::sqrt(a.x), std::sqrt(a.y), std::sqrt(a.z)); }
static inline float3 to_float3(float4 a) { return float3(a.x, a.y, a.z); }
static inline float4 to_float4(float3 a, float w) { return float4(a.x, a.y, a.z, w); }
static inline float3 make_float3(float a, float b, float c) { return float3(a, b, c); }
static inline float4 make_float4(float a, float b, float c, float d) { return float4(a, b, c, d); }
static inline float2 make_float2(float a, float b) { return float2(a, b); }
static inline float3 to_float3(int3 a) { return float3(float(a.x), float(a.y), float(a.z)); }
static inline float3 to_float3(uint3 a) { return float3(float(a.x), float(a.y), float(a.z)); }
static inline float hmin(float3 a) { return std::min(a.x, std::min(a.y, a.z)); }
static inline float hmax(float3 a) { return std::max(a.x, std::max(a.y, a.z)); }
static inline bool all_of(bool b) { return b; }

struct float3x3 {
  float3 row[3];
  float3x3() { row[0] = float3(1, 0, 0); row[1] = float3(0, 1, 0); row[2] = float3(0, 0, 1); }
  float &operator()(int r, int c) { return row[r][c]; }
  float operator()(int r, int c) const { return row[r][c]; }
};
static inline float3 operator*(const float3x3 &m, float3 v) { return float3(dot(m.row[0], v), dot(m.row[1], v), dot(m.row[2], v)); }
static inline float3x3 make_float3x3(float3 r0, float3 r1, float3 r2) {
  float3x3 m; m.row[0] = r0; m.row[1] = r1; m.row[2] = r2; return m;
}
static inline float3x3 make_float3x3_by_columns(float3 c0, float3 c1, float3 c2) {
  float3x3 m;
  m.row[0] = float3(c0.x, c1.x, c2.x); m.row[1] = float3(c0.y, c1.y, c2.y); m.row[2] = float3(c0.z, c1.z, c2.z);
  return m;
}

struct float4x4 {
  float m[16];   // row-major
  float4x4() { std::memset(m, 0, sizeof(m)); m[0] = m[5] = m[10] = m[15] = 1.0f; }
  explicit float4x4(const float *a) { std::memcpy(m, a, sizeof(m)); }
  float &operator()(int r, int c) { return m[r * 4 + c]; }
  float operator()(int r, int c) const { return m[r * 4 + c]; }
  float4 get_row(int r) const { return float4(m[r * 4], m[r * 4 + 1], m[r * 4 + 2], m[r * 4 + 3]); }
  float4 get_col(int c) const { return float4(m[c], m[4 + c], m[8 + c], m[12 + c]); }
  void set_row(int r, float4 v) { for (int i = 0; i < 4; i++) m[r * 4 + i] = v[i]; }
  void set_col(int c, float4 v) { for (int i = 0; i < 4; i++) m[i * 4 + c] = v[i]; }
};
static inline float4 operator*(const float4x4 &a, float4 v) {
  float4 r;
  for (int i = 0; i < 4; i++) r[i] = a(i, 0) * v.x + a(i, 1) * v.y + a(i, 2) * v.z + a(i, 3) * v.w;
  return r;
}
static inline float4x4 operator*(const float4x4 &a, const float4x4 &b) {
  float4x4 r;
  for (int i = 0; i < 4; i++)
    for (int j = 0; j < 4; j++) r(i, j) = a(i, 0) * b(0, j) + a(i, 1) * b(1, j) + a(i, 2) * b(2, j) + a(i, 3) * b(3, j);
  return r;
}
static inline float4x4 transpose(const float4x4 &a) {
  float4x4 r;
  for (int i = 0; i < 4; i++) for (int j = 0; j < 4; j++) r(i, j) = a(j, i);
  return r;
}
static inline float4x4 inverse4x4(const float4x4 &a) {
  double t[4][8];
  for (int i = 0; i < 4; i++) for (int j = 0; j < 8; j++) t[i][j] = j < 4 ? double(a(i, j)) : (j - 4 == i ? 1.0 : 0.0);
  for (int c = 0; c < 4; c++) {
    int p = c;
    for (int r = c + 1; r < 4; r++) if (std::fabs(t[r][c]) > std::fabs(t[p][c])) p = r;
    if (p != c) for (int j = 0; j < 8; j++) std::swap(t[c][j], t[p][j]);
    const double inv = 1.0 / t[c][c];
    for (int j = 0; j < 8; j++) t[c][j] *= inv;
    for (int r = 0; r < 4; r++) if (r != c) { const double f = t[r][c]; for (int j = 0; j < 8; j++) t[r][j] -= f * t[c][j]; }
  }
  float4x4 r;
  for (int i = 0; i < 4; i++) for (int j = 0; j < 4; j++) r(i, j) = float(t[i][j + 4]);
  return r;
}
// perspectiveMatrix / lookAt with the conventions the engine's camera helpers use
// (row-major, right-handed view looking down -z, OpenGL depth range)
static inline float4x4 perspectiveMatrix(float fovy, float aspect, float zNear, float zFar) {
  float4x4 r;
  std::memset(r.m, 0, sizeof(r.m));
  const float ymax = zNear * std::tan(fovy * 3.14159265358979323846f / 180.0f * 0.5f);
  const float xmax = ymax * aspect;
  const float left = -xmax, right = xmax, bottom = -ymax, top = ymax;
  r(0, 0) = 2.0f * zNear / (right - left);
  r(0, 2) = (right + left) / (right - left);
  r(1, 1) = 2.0f * zNear / (top - bottom);
  r(1, 2) = (top + bottom) / (top - bottom);
  r(2, 2) = (-zFar - zNear) / (zFar - zNear);
  r(2, 3) = (-2.0f * zNear * zFar) / (zFar - zNear);
  r(3, 2) = -1.0f;
  return r;
}
static inline float4x4 lookAt(float3 eye, float3 center, float3 up) {
  float3 z = eye - center;
  z = z / std::sqrt(dot(z, z));
  float3 x = cross(up, z);
  x = x / std::sqrt(dot(x, x));
  const float3 y = cross(z, x);
  float4x4 r;
  r(0, 0) = x.x; r(0, 1) = x.y; r(0, 2) = x.z; r(0, 3) = -(x.x * eye.x + x.y * eye.y + x.z * eye.z);
  r(1, 0) = y.x; r(1, 1) = y.y; r(1, 2) = y.z; r(1, 3) = -(y.x * eye.x + y.y * eye.y + y.z * eye.z);
  r(2, 0) = z.x; r(2, 1) = z.y; r(2, 2) = z.z; r(2, 3) = -(z.x * eye.x + z.y * eye.y + z.z * eye.z);
  r(3, 0) = 0; r(3, 1) = 0; r(3, 2) = 0; r(3, 3) = 1;
  return r;
}
static inline float4x4 translate4x4(float3 t) { float4x4 r; r(0, 3) = t.x; r(1, 3) = t.y; r(2, 3) = t.z; return r; }
static inline float4x4 scale4x4(float3 s) { float4x4 r; r(0, 0) = s.x; r(1, 1) = s.y; r(2, 2) = s.z; return r; }

struct Box4f {
  float4 boxMin, boxMax;
  Box4f() : boxMin(float4(+1e30f)), boxMax(float4(-1e30f)) {}
  Box4f(float4 a, float4 b) : boxMin(a), boxMax(b) {}
  void include(float4 p) { boxMin = min(boxMin, p); boxMax = max(boxMax, p); }
  void include(const Box4f &b) { boxMin = min(boxMin, b.boxMin); boxMax = max(boxMax, b.boxMax); }
  float4 center() const { return 0.5f * (boxMin + boxMax); }
};
}  // namespace LiteMath
