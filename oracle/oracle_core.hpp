// ORACLE — test infrastructure only.
//
// CPU restatement of baby_shark's implicit-modelling path (crate baby_shark
// v0.3.12, Rust).  This code is the parity checker for the CUDA product in
// baby_shark_gb300/; the product never links, loads or calls it.  Only the
// test-suite, the smoke check and the CPU-baseline leg of the benchmark do.
//
// Floating point follows the reference operation by operation: every dot
// product is accumulated left to right ((x*x + y*y) + z*z), 3x3 Frobenius
// products column-major, and the file is compiled with -ffp-contract=off so
// that no multiply-add is fused (Rust never fuses).  nalgebra 0.34 / glm 0.20
// are not vendored in the reference tree; the accumulation orders above are
// the ones their published small-vector code paths use and are an assumption
// of this restatement.
#pragma once

#include <array>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <functional>
#include <map>
#include <memory>
#include <vector>

namespace orc {

// ---------------------------------------------------------------- vectors --
struct V3 {
  float x, y, z;
  float& operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
  float operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};
inline V3 v3(float x, float y, float z) { return V3{x, y, z}; }
inline V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 operator*(V3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
inline V3 operator*(float s, V3 a) { return {s * a.x, s * a.y, s * a.z}; }
inline V3 operator/(V3 a, float s) { return {a.x / s, a.y / s, a.z / s}; }
inline V3& operator+=(V3& a, V3 b) { a = a + b; return a; }
// nalgebra Vector3::dot: (x1*x2 + y1*y2) + z1*z2
inline float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline float norm_sq(V3 a) { return dot(a, a); }
inline float norm(V3 a) { return std::sqrt(norm_sq(a)); }
inline V3 cross(V3 a, V3 b) {
  return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
inline V3 vmin(V3 a, V3 b) { return {a.x < b.x ? a.x : b.x, a.y < b.y ? a.y : b.y, a.z < b.z ? a.z : b.z}; }
inline V3 vmax(V3 a, V3 b) { return {a.x > b.x ? a.x : b.x, a.y > b.y ? a.y : b.y, a.z > b.z ? a.z : b.z}; }

// 3x3 column-major matrix, m[col][row]
struct M3 {
  float m[3][3];
};
inline M3 m3_zero() { M3 r; std::memset(&r, 0, sizeof r); return r; }
inline M3 outer(V3 u, V3 v) {  // u * v^T
  M3 r;
  for (int j = 0; j < 3; ++j)
    for (int i = 0; i < 3; ++i) r.m[j][i] = u[i] * v[j];
  return r;
}
inline M3 operator+(const M3& a, const M3& b) {
  M3 r;
  for (int j = 0; j < 3; ++j)
    for (int i = 0; i < 3; ++i) r.m[j][i] = a.m[j][i] + b.m[j][i];
  return r;
}
inline M3 operator-(const M3& a, const M3& b) {
  M3 r;
  for (int j = 0; j < 3; ++j)
    for (int i = 0; i < 3; ++i) r.m[j][i] = a.m[j][i] - b.m[j][i];
  return r;
}
// Frobenius product accumulated column-major (nalgebra Matrix::dot).
inline float mdot(const M3& a, const M3& b) {
  float r = 0.0f;
  for (int j = 0; j < 3; ++j)
    for (int i = 0; i < 3; ++i) r += a.m[j][i] * b.m[j][i];
  return r;
}

struct I3 {
  int64_t x, y, z;
  int64_t& operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
  int64_t operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
  bool operator==(const I3& o) const { return x == o.x && y == o.y && z == o.z; }
  bool operator!=(const I3& o) const { return !(*this == o); }
  bool operator<(const I3& o) const {
    if (x != o.x) return x < o.x;
    if (y != o.y) return y < o.y;
    return z < o.z;
  }
};
inline I3 i3(int64_t x, int64_t y, int64_t z) { return I3{x, y, z}; }
inline I3 operator+(I3 a, I3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }

// -------------------------------------------------------------- triangles --
struct Tri {
  V3 a, b, c;
};

// triangle3.rs:117-124
inline float tri_max_side(const Tri& t) {
  float ab = norm_sq(t.b - t.a);
  float ac = norm_sq(t.c - t.a);
  float bc = norm_sq(t.c - t.b);
  float m = std::fmax(std::fmax(ab, ac), bc);
  return std::sqrt(m);
}
// triangle3.rs:307-315 (glm min2/max2)
inline void tri_bbox(const Tri& t, V3& mn, V3& mx) {
  mn = vmin(t.c, vmin(t.a, t.b));
  mx = vmax(t.c, vmax(t.a, t.b));
}

// triangle3.rs:317-382  (Ericson, Real-Time Collision Detection 5.1.5)
inline V3 closest_point(const Tri& t, V3 p) {
  V3 ab = t.b - t.a, ac = t.c - t.a, ap = p - t.a;
  float d1 = dot(ab, ap), d2 = dot(ac, ap);
  if (d1 <= 0.0f && d2 <= 0.0f) return t.a;
  V3 bp = p - t.b;
  float d3 = dot(ab, bp), d4 = dot(ac, bp);
  if (d3 >= 0.0f && d4 <= d3) return t.b;
  float vc = d1 * d4 - d3 * d2;
  if (vc <= 0.0f && d1 >= 0.0f && d3 <= 0.0f) {
    float v = d1 / (d1 - d3);
    return t.a + ab * v;
  }
  V3 cp = p - t.c;
  float d5 = dot(ab, cp), d6 = dot(ac, cp);
  if (d6 >= 0.0f && d5 <= d6) return t.c;
  float vb = d5 * d2 - d1 * d6;
  if (vb <= 0.0f && d2 >= 0.0f && d6 <= 0.0f) {
    float w = d2 / (d2 - d6);
    return t.a + ac * w;
  }
  float va = d3 * d6 - d5 * d4;
  if (va <= 0.0f && (d4 - d3) >= 0.0f && (d5 - d6) >= 0.0f) {
    float w = (d4 - d3) / ((d4 - d3) + (d5 - d6));
    return t.b + (t.c - t.b) * w;
  }
  float denom = 1.0f / (va + vb + vc);
  float v = vb * denom;
  float w = vc * denom;
  return t.a + ab * v + ac * w;
}

// ----------------------------------------------------------------- bitset --
// Index semantics of data_structures/bitset.rs (find_first_on = lowest index).
template <int N>
struct Bits {
  static constexpr int W = (N + 63) / 64;
  uint64_t w[W];
  Bits() { off_all(); }
  bool at(int i) const { return (w[i >> 6] >> (i & 63)) & 1u; }
  void on(int i) { w[i >> 6] |= (uint64_t(1) << (i & 63)); }
  void off(int i) { w[i >> 6] &= ~(uint64_t(1) << (i & 63)); }
  void set(int i, bool v) { v ? on(i) : off(i); }
  void on_all() { for (int k = 0; k < W; ++k) w[k] = ~uint64_t(0); }
  void off_all() { for (int k = 0; k < W; ++k) w[k] = 0; }
  uint64_t used(int k) const {
    int rem = N - k * 64;
    return rem >= 64 ? ~uint64_t(0) : ((uint64_t(1) << rem) - 1);
  }
  bool is_empty() const {
    for (int k = 0; k < W; ++k)
      if (w[k] & used(k)) return false;
    return true;
  }
  bool is_full() const {
    for (int k = 0; k < W; ++k)
      if ((w[k] & used(k)) != used(k)) return false;
    return true;
  }
  int find_first_on() const {
    for (int k = 0; k < W; ++k) {
      uint64_t v = w[k] & used(k);
      if (v) return k * 64 + __builtin_ctzll(v);
    }
    return -1;
  }
  void operator|=(const Bits& o) { for (int k = 0; k < W; ++k) w[k] |= o.w[k]; }
};

// ------------------------------------------------------------ sign values --
// value/f32.rs:7-31
enum class Sign { Pos, Neg };
inline Sign sign_of(float v) { return std::signbit(v) ? Sign::Neg : Sign::Pos; }
inline void set_sign(float& v, Sign s) {
  float num = (s == Sign::Pos) ? std::copysign(v, 1.0f) : std::copysign(v, -1.0f);
  v = std::copysign(v, num);
}
constexpr float FAR = 3.40282347e+38f;  // f32::MAX

}  // namespace orc
