// glsl.h — the GLSL 4.50 types and built-in functions that the reference's
// compute shaders use, so that their source compiles as C++.
//
// TEST INFRASTRUCTURE ONLY: it lets the oracle be checked against the
// reference's own shader code run on the CPU (oracle/ref_shaders/).  The
// product never includes it.
//
// Two arithmetic precisions share one set of types:
//   glsl::f32 — the shaders' float arithmetic, one rounding per operation
//               (built with -ffp-contract=off);
//   glsl::f64 — the same source with float promoted to double.
// Built-ins follow the GLSL 4.50 specification, section 8 (length = sqrt of
// the dot product, normalize = v / length(v), smoothstep's Hermite formula,
// distance = length(p0 - p1)).  Texture lookups follow the GL 4.5 core
// specification, section 8.14: GL_LINEAR with GL_CLAMP_TO_EDGE, texel
// centres at (i + 1/2) / size, weights in full precision (hardware filter
// units quantise them; that difference is outside this check).
#pragma once

#include <math.h>
#include <stdint.h>

#include <utility>

namespace glsl {

// ---------------------------------------------------------- swizzles ----
// A swizzle is a union member over the vector's storage: reading converts to
// the vector type V it names, assigning writes the named components.
template <class V, class S, int N, int... I>
struct Swz {
  S e[N];
  operator V() const { return V(e[I]...); }
  Swz& operator=(const V& v) {
    assign(v, std::make_integer_sequence<int, (int)sizeof...(I)>());
    return *this;
  }
  // a.xyz = b.xyz writes the named components only
  Swz& operator=(const Swz& o) { return *this = V(o); }
  Swz& operator+=(const V& v) { return *this = V(*this) + v; }
  Swz& operator-=(const V& v) { return *this = V(*this) - v; }
  Swz& operator*=(S s) { return *this = V(*this) * s; }
  Swz& operator+=(S s) {
    V v = V(*this);
    v += s;
    return *this = v;
  }

 private:
  template <int... K>
  void assign(const V& v, std::integer_sequence<int, K...>) {
    const S t[] = {v[K]...};
    ((e[I] = t[K]), ...);
  }
};

template <class S> struct tvec2;
template <class S> struct tvec3;
template <class S> struct tvec4;

#define GLSL_VEC_COMMON(T, N)                                                      \
  S& operator[](int k) { return e[k]; }                                            \
  const S& operator[](int k) const { return e[k]; }                                \
  T& operator+=(const T& o) { for (int k = 0; k < N; ++k) e[k] = e[k] + o.e[k]; return *this; } \
  T& operator-=(const T& o) { for (int k = 0; k < N; ++k) e[k] = e[k] - o.e[k]; return *this; } \
  T& operator*=(const T& o) { for (int k = 0; k < N; ++k) e[k] = e[k] * o.e[k]; return *this; } \
  T& operator/=(const T& o) { for (int k = 0; k < N; ++k) e[k] = e[k] / o.e[k]; return *this; } \
  T& operator*=(S s) { for (int k = 0; k < N; ++k) e[k] = e[k] * s; return *this; }            \
  T& operator+=(S s) { for (int k = 0; k < N; ++k) e[k] = e[k] + s; return *this; }            \
  T& operator-=(S s) { for (int k = 0; k < N; ++k) e[k] = e[k] - s; return *this; }            \
  T& operator/=(S s) { for (int k = 0; k < N; ++k) e[k] = e[k] / s; return *this; }            \
  friend T operator+(const T& a, const T& b) { T r; for (int k = 0; k < N; ++k) r.e[k] = a.e[k] + b.e[k]; return r; } \
  friend T operator-(const T& a, const T& b) { T r; for (int k = 0; k < N; ++k) r.e[k] = a.e[k] - b.e[k]; return r; } \
  friend T operator*(const T& a, const T& b) { T r; for (int k = 0; k < N; ++k) r.e[k] = a.e[k] * b.e[k]; return r; } \
  friend T operator/(const T& a, const T& b) { T r; for (int k = 0; k < N; ++k) r.e[k] = a.e[k] / b.e[k]; return r; } \
  friend T operator*(const T& a, S s) { T r; for (int k = 0; k < N; ++k) r.e[k] = a.e[k] * s; return r; }             \
  friend T operator*(S s, const T& a) { T r; for (int k = 0; k < N; ++k) r.e[k] = s * a.e[k]; return r; }             \
  friend T operator/(const T& a, S s) { T r; for (int k = 0; k < N; ++k) r.e[k] = a.e[k] / s; return r; }             \
  friend T operator+(const T& a, S s) { T r; for (int k = 0; k < N; ++k) r.e[k] = a.e[k] + s; return r; }             \
  friend T operator-(const T& a, S s) { T r; for (int k = 0; k < N; ++k) r.e[k] = a.e[k] - s; return r; }             \
  friend T operator+(S s, const T& a) { T r; for (int k = 0; k < N; ++k) r.e[k] = s + a.e[k]; return r; }             \
  friend T operator-(S s, const T& a) { T r; for (int k = 0; k < N; ++k) r.e[k] = s - a.e[k]; return r; }             \
  friend T operator-(const T& a) { T r; for (int k = 0; k < N; ++k) r.e[k] = -a.e[k]; return r; }

template <class S>
struct tvec2 {
  union {
    struct { S x, y; };
    struct { S r, g; };
    S e[2];
  };
  tvec2() { e[0] = e[1] = S(0); }
  explicit tvec2(S s) { e[0] = e[1] = s; }
  tvec2(S a, S b) { e[0] = a; e[1] = b; }
  tvec2(const tvec2& o) { e[0] = o.e[0]; e[1] = o.e[1]; }
  explicit tvec2(const tvec4<S>& v);  // the first two components
  tvec2& operator=(const tvec2& o) { e[0] = o.e[0]; e[1] = o.e[1]; return *this; }
  GLSL_VEC_COMMON(tvec2, 2)
};

template <class S>
struct tvec3 {
  union {
    struct { S x, y, z; };
    struct { S r, g, b; };
    S e[3];
    Swz<tvec2<S>, S, 3, 0, 2> xz;
    Swz<tvec2<S>, S, 3, 0, 1> xy;
  };
  tvec3() { e[0] = e[1] = e[2] = S(0); }
  explicit tvec3(S s) { e[0] = e[1] = e[2] = s; }
  tvec3(S a, S b, S c) { e[0] = a; e[1] = b; e[2] = c; }
  tvec3(const tvec3& o) { for (int k = 0; k < 3; ++k) e[k] = o.e[k]; }
  explicit tvec3(const tvec4<S>& v);  // the first three components
  tvec3& operator=(const tvec3& o) { for (int k = 0; k < 3; ++k) e[k] = o.e[k]; return *this; }
  GLSL_VEC_COMMON(tvec3, 3)
};

template <class S>
struct tvec4 {
  union {
    struct { S x, y, z, w; };
    struct { S r, g, b, a; };
    S e[4];
    Swz<tvec3<S>, S, 4, 0, 1, 2> xyz;
    Swz<tvec3<S>, S, 4, 0, 1, 2> rgb;
    Swz<tvec2<S>, S, 4, 0, 2> xz;
    Swz<tvec2<S>, S, 4, 0, 1> xy;
  };
  tvec4() { e[0] = e[1] = e[2] = e[3] = S(0); }
  tvec4(const tvec3<S>& v, S d) { e[0] = v.e[0]; e[1] = v.e[1]; e[2] = v.e[2]; e[3] = d; }
  explicit tvec4(S s) { e[0] = e[1] = e[2] = e[3] = s; }
  tvec4(S a, S b, S c, S d) { e[0] = a; e[1] = b; e[2] = c; e[3] = d; }
  tvec4(const tvec2<S>& v, S c, S d) { e[0] = v.e[0]; e[1] = v.e[1]; e[2] = c; e[3] = d; }
  tvec4(const tvec4& o) { for (int k = 0; k < 4; ++k) e[k] = o.e[k]; }
  tvec4& operator=(const tvec4& o) { for (int k = 0; k < 4; ++k) e[k] = o.e[k]; return *this; }
  GLSL_VEC_COMMON(tvec4, 4)
};

#undef GLSL_VEC_COMMON

template <class S>
tvec2<S>::tvec2(const tvec4<S>& v) { e[0] = v.e[0]; e[1] = v.e[1]; }
template <class S>
tvec3<S>::tvec3(const tvec4<S>& v) { e[0] = v.e[0]; e[1] = v.e[1]; e[2] = v.e[2]; }

// Column-major 4x4: m[c * 4 + r] is column c, row r (GLSL's layout).
template <class S>
struct tmat4 {
  S m[16];
  tmat4() { for (int k = 0; k < 16; ++k) m[k] = S(0); }
  friend tvec4<S> operator*(const tmat4& a, const tvec4<S>& v) {
    tvec4<S> r;
    for (int row = 0; row < 4; ++row)
      r.e[row] = a.m[row] * v.e[0] + a.m[4 + row] * v.e[1] + a.m[8 + row] * v.e[2] + a.m[12 + row] * v.e[3];
    return r;
  }
  friend tmat4 operator*(const tmat4& a, const tmat4& b) {
    tmat4 r;
    for (int c = 0; c < 4; ++c)
      for (int row = 0; row < 4; ++row) {
        S acc = S(0);
        for (int k = 0; k < 4; ++k) acc = acc + a.m[k * 4 + row] * b.m[c * 4 + k];
        r.m[c * 4 + row] = acc;
      }
    return r;
  }
};

// inverse (GLSL 4.50, 8.6): the adjugate over the determinant, by cofactor
// expansion.
template <class S>
tmat4<S> inverse_of(const tmat4<S>& a) {
  const S* m = a.m;
  S inv[16];
  inv[0] = m[5] * m[10] * m[15] - m[5] * m[11] * m[14] - m[9] * m[6] * m[15] + m[9] * m[7] * m[14] +
           m[13] * m[6] * m[11] - m[13] * m[7] * m[10];
  inv[4] = -m[4] * m[10] * m[15] + m[4] * m[11] * m[14] + m[8] * m[6] * m[15] - m[8] * m[7] * m[14] -
           m[12] * m[6] * m[11] + m[12] * m[7] * m[10];
  inv[8] = m[4] * m[9] * m[15] - m[4] * m[11] * m[13] - m[8] * m[5] * m[15] + m[8] * m[7] * m[13] +
           m[12] * m[5] * m[11] - m[12] * m[7] * m[9];
  inv[12] = -m[4] * m[9] * m[14] + m[4] * m[10] * m[13] + m[8] * m[5] * m[14] - m[8] * m[6] * m[13] -
            m[12] * m[5] * m[10] + m[12] * m[6] * m[9];
  inv[1] = -m[1] * m[10] * m[15] + m[1] * m[11] * m[14] + m[9] * m[2] * m[15] - m[9] * m[3] * m[14] -
           m[13] * m[2] * m[11] + m[13] * m[3] * m[10];
  inv[5] = m[0] * m[10] * m[15] - m[0] * m[11] * m[14] - m[8] * m[2] * m[15] + m[8] * m[3] * m[14] +
           m[12] * m[2] * m[11] - m[12] * m[3] * m[10];
  inv[9] = -m[0] * m[9] * m[15] + m[0] * m[11] * m[13] + m[8] * m[1] * m[15] - m[8] * m[3] * m[13] -
           m[12] * m[1] * m[11] + m[12] * m[3] * m[9];
  inv[13] = m[0] * m[9] * m[14] - m[0] * m[10] * m[13] - m[8] * m[1] * m[14] + m[8] * m[2] * m[13] +
            m[12] * m[1] * m[10] - m[12] * m[2] * m[9];
  inv[2] = m[1] * m[6] * m[15] - m[1] * m[7] * m[14] - m[5] * m[2] * m[15] + m[5] * m[3] * m[14] +
           m[13] * m[2] * m[7] - m[13] * m[3] * m[6];
  inv[6] = -m[0] * m[6] * m[15] + m[0] * m[7] * m[14] + m[4] * m[2] * m[15] - m[4] * m[3] * m[14] -
           m[12] * m[2] * m[7] + m[12] * m[3] * m[6];
  inv[10] = m[0] * m[5] * m[15] - m[0] * m[7] * m[13] - m[4] * m[1] * m[15] + m[4] * m[3] * m[13] +
            m[12] * m[1] * m[7] - m[12] * m[3] * m[5];
  inv[14] = -m[0] * m[5] * m[14] + m[0] * m[6] * m[13] + m[4] * m[1] * m[14] - m[4] * m[2] * m[13] -
            m[12] * m[1] * m[6] + m[12] * m[2] * m[5];
  inv[3] = -m[1] * m[6] * m[11] + m[1] * m[7] * m[10] + m[5] * m[2] * m[11] - m[5] * m[3] * m[10] -
           m[9] * m[2] * m[7] + m[9] * m[3] * m[6];
  inv[7] = m[0] * m[6] * m[11] - m[0] * m[7] * m[10] - m[4] * m[2] * m[11] + m[4] * m[3] * m[10] +
           m[8] * m[2] * m[7] - m[8] * m[3] * m[6];
  inv[11] = -m[0] * m[5] * m[11] + m[0] * m[7] * m[9] + m[4] * m[1] * m[11] - m[4] * m[3] * m[9] -
            m[8] * m[1] * m[7] + m[8] * m[3] * m[5];
  inv[15] = m[0] * m[5] * m[10] - m[0] * m[6] * m[9] - m[4] * m[1] * m[10] + m[4] * m[2] * m[9] +
            m[8] * m[1] * m[6] - m[8] * m[2] * m[5];
  const S det = m[0] * inv[0] + m[1] * inv[4] + m[2] * inv[8] + m[3] * inv[12];
  tmat4<S> r;
  for (int k = 0; k < 16; ++k) r.m[k] = inv[k] / det;
  return r;
}

struct bvec2 {
  bool x, y;
};

struct uvec2 {
  unsigned x, y;
  uvec2() : x(0), y(0) {}
  uvec2(unsigned a, unsigned b) : x(a), y(b) {}
  unsigned operator[](int k) const { return k == 0 ? x : y; }
};

struct uvec3 {
  union {
    struct { unsigned x, y, z; };
    unsigned e[3];
    Swz<uvec2, unsigned, 3, 0, 1> xy;
  };
  uvec3() { e[0] = e[1] = e[2] = 0u; }
  uvec3(unsigned a, unsigned b, unsigned c) { e[0] = a; e[1] = b; e[2] = c; }
  uvec3(const uvec3& o) { for (int k = 0; k < 3; ++k) e[k] = o.e[k]; }
  uvec3& operator=(const uvec3& o) { for (int k = 0; k < 3; ++k) e[k] = o.e[k]; return *this; }
};

// ivec2 converts implicitly to the float vectors, as GLSL converts int
// arguments of the float built-ins (distance(ivec2, ivec2)).
struct ivec2 {
  union {
    struct { int x, y; };
    int e[2];
    Swz<ivec2, int, 2, 0, 1> xy;
  };
  ivec2() { e[0] = e[1] = 0; }
  explicit ivec2(int s) { e[0] = e[1] = s; }
  ivec2(int a, int b) { e[0] = a; e[1] = b; }
  explicit ivec2(const uvec2& u) { e[0] = (int)u.x; e[1] = (int)u.y; }
  explicit ivec2(const tvec2<float>& v) { e[0] = (int)v.e[0]; e[1] = (int)v.e[1]; }
  explicit ivec2(const tvec2<double>& v) { e[0] = (int)v.e[0]; e[1] = (int)v.e[1]; }
  explicit ivec2(const tvec4<float>& v) { e[0] = (int)v.e[0]; e[1] = (int)v.e[1]; }
  explicit ivec2(const tvec4<double>& v) { e[0] = (int)v.e[0]; e[1] = (int)v.e[1]; }
  ivec2(const ivec2& o) { e[0] = o.e[0]; e[1] = o.e[1]; }
  ivec2& operator=(const ivec2& o) { e[0] = o.e[0]; e[1] = o.e[1]; return *this; }
  int& operator[](int k) { return e[k]; }
  int operator[](int k) const { return e[k]; }
  operator tvec2<float>() const { return tvec2<float>((float)e[0], (float)e[1]); }
  operator tvec2<double>() const { return tvec2<double>((double)e[0], (double)e[1]); }
  friend ivec2 operator+(const ivec2& a, const ivec2& b) { return ivec2(a.e[0] + b.e[0], a.e[1] + b.e[1]); }
  friend ivec2 operator-(const ivec2& a, const ivec2& b) { return ivec2(a.e[0] - b.e[0], a.e[1] - b.e[1]); }
  friend ivec2 operator*(const ivec2& a, const ivec2& b) { return ivec2(a.e[0] * b.e[0], a.e[1] * b.e[1]); }
  // GLSL == on vectors: every component equal
  friend bool operator==(const ivec2& a, const ivec2& b) { return a.e[0] == b.e[0] && a.e[1] == b.e[1]; }
  // float * ivec2: the int vector converts to a float vector first
  friend tvec2<float> operator*(float s, const ivec2& a) { return tvec2<float>(s * (float)a.e[0], s * (float)a.e[1]); }
  friend tvec2<double> operator*(double s, const ivec2& a) {
    return tvec2<double>(s * (double)a.e[0], s * (double)a.e[1]);
  }
};

struct ivec3 {
  union {
    struct { int x, y, z; };
    int e[3];
  };
  ivec3() { e[0] = e[1] = e[2] = 0; }
  explicit ivec3(int s) { e[0] = e[1] = e[2] = s; }
  ivec3(int a, int b, int c) { e[0] = a; e[1] = b; e[2] = c; }
  explicit ivec3(const tvec3<float>& v) { for (int k = 0; k < 3; ++k) e[k] = (int)v.e[k]; }
  explicit ivec3(const tvec3<double>& v) { for (int k = 0; k < 3; ++k) e[k] = (int)v.e[k]; }
  ivec3(const ivec3& o) { for (int k = 0; k < 3; ++k) e[k] = o.e[k]; }
  ivec3& operator=(const ivec3& o) { for (int k = 0; k < 3; ++k) e[k] = o.e[k]; return *this; }
  int& operator[](int k) { return e[k]; }
  int operator[](int k) const { return e[k]; }
  friend ivec3 operator+(const ivec3& a, const ivec3& b) { return ivec3(a.x + b.x, a.y + b.y, a.z + b.z); }
  friend ivec3 operator-(const ivec3& a, const ivec3& b) { return ivec3(a.x - b.x, a.y - b.y, a.z - b.z); }
  friend ivec3 operator*(const ivec3& a, const ivec3& b) { return ivec3(a.x * b.x, a.y * b.y, a.z * b.z); }
  friend bool operator==(const ivec3& a, const ivec3& b) { return a.x == b.x && a.y == b.y && a.z == b.z; }
};

inline ivec3 max(const ivec3& a, const ivec3& b) {
  return ivec3(b.x > a.x ? b.x : a.x, b.y > a.y ? b.y : a.y, b.z > a.z ? b.z : a.z);
}

struct ivec4 {
  union {
    struct { int x, y, z, w; };
    int e[4];
    Swz<ivec3, int, 4, 0, 1, 2> xyz;
  };
  ivec4() { e[0] = e[1] = e[2] = e[3] = 0; }
  explicit ivec4(int s) { e[0] = e[1] = e[2] = e[3] = s; }
  ivec4(int a, int b, int c, int d) { e[0] = a; e[1] = b; e[2] = c; e[3] = d; }
  ivec4(const ivec4& o) { for (int k = 0; k < 4; ++k) e[k] = o.e[k]; }
  ivec4& operator=(const ivec4& o) { for (int k = 0; k < 4; ++k) e[k] = o.e[k]; return *this; }
  int& operator[](int k) { return e[k]; }
  int operator[](int k) const { return e[k]; }
};

inline ivec3 clamp(const ivec3& v, const ivec3& lo, const ivec3& hi) {
  ivec3 r;
  for (int k = 0; k < 3; ++k) r.e[k] = v.e[k] < lo.e[k] ? lo.e[k] : (v.e[k] > hi.e[k] ? hi.e[k] : v.e[k]);
  return r;
}

// atomicAdd on a buffer element: the invocations of a dispatch run one after
// another, so the returned old values come in invocation order.
inline int atomicAdd(int& mem, int v) {
  const int old = mem;
  mem = old + v;
  return old;
}
// float atomics (GL_NV_shader_atomic_float), and their double-build form
inline float atomicAdd(float& mem, float v) {
  const float old = mem;
  mem = old + v;
  return old;
}
inline double atomicAdd(double& mem, double v) {
  const double old = mem;
  mem = old + v;
  return old;
}

inline ivec2 clamp(const ivec2& v, const ivec2& lo, const ivec2& hi) {
  ivec2 r;
  for (int k = 0; k < 2; ++k) r.e[k] = v.e[k] < lo.e[k] ? lo.e[k] : (v.e[k] > hi.e[k] ? hi.e[k] : v.e[k]);
  return r;
}
inline ivec2 max(const ivec2& a, const ivec2& b) { return ivec2(b.x > a.x ? b.x : a.x, b.y > a.y ? b.y : a.y); }
inline bvec2 greaterThanEqual(const ivec2& a, const ivec2& b) { return bvec2{a.x >= b.x, a.y >= b.y}; }
inline bool any(const bvec2& b) { return b.x || b.y; }
inline bool all(const bvec2& b) { return b.x && b.y; }

// ---------------------------------------------------- textures, images ----
// A bound texture: w x h texels of `comps` floats (1: the red channel only,
// green, blue and alpha read 0, 1 reads 1 for alpha as GL does for a
// one-channel format; 4: RGBA).
struct sampler2D {
  const float* texels = nullptr;
  int w = 0, h = 0, comps = 1;
  float at(int x, int y, int c) const {
    if (c < comps) return texels[((size_t)y * w + x) * comps + c];
    return c == 3 ? 1.0f : 0.0f;
  }
};

inline ivec2 textureSize(const sampler2D& s, int) { return ivec2(s.w, s.h); }

// A bound 1D texture: w texels of `comps` floats.
struct sampler1D {
  const float* texels = nullptr;
  int w = 0, comps = 4;
  float at(int x, int c) const {
    if (c < comps) return texels[(size_t)x * comps + c];
    return c == 3 ? 1.0f : 0.0f;
  }
};

inline int textureSize(const sampler1D& s, int) { return s.w; }

// A bound cube map: 6 faces (+x, -x, +y, -y, +z, -z) of size x size RGBA8
// texels, read as c / 255.
struct samplerCube {
  const uint8_t* faces = nullptr;
  int size = 0;
  float at(int face, int x, int y, int c) const {
    return faces[(((size_t)face * size + y) * size + x) * 4 + c] / 255.0f;
  }
};

// A bound image1D, rgba32f: w texels of 4 scalars, float or double.
struct image1D {
  void* data = nullptr;
  int w = 0;
  bool is_double = false;
};

inline int imageSize(const image1D& im) { return im.w; }

// A bound image2D, rgba32f: w x h texels of 4 scalars, float or double.
struct image2D {
  void* data = nullptr;
  int w = 0, h = 0;
  bool is_double = false;
};

inline ivec2 imageSize(const image2D& im) { return ivec2(im.w, im.h); }

namespace detail {

template <class S>
tvec4<S> filter_linear(const sampler2D& t, S s, S u) {
  // GL 4.5 core, 8.14.2: u' = s * w - 1/2, i0 = floor(u'), alpha = frac(u'),
  // each index clamped to [0, w - 1] (GL_CLAMP_TO_EDGE)
  const S us = s * (S)t.w - (S)0.5, vs = u * (S)t.h - (S)0.5;
  const S fi = floor(us), fj = floor(vs);
  const S a = us - fi, b = vs - fj;
  auto cl = [](long v, int n) { return (int)(v < 0 ? 0 : (v > n - 1 ? n - 1 : v)); };
  const long i0 = (long)fi, j0 = (long)fj;
  const int x0 = cl(i0, t.w), x1 = cl(i0 + 1, t.w), y0 = cl(j0, t.h), y1 = cl(j0 + 1, t.h);
  tvec4<S> r;
  for (int c = 0; c < 4; ++c) {
    const S t00 = t.at(x0, y0, c), t10 = t.at(x1, y0, c), t01 = t.at(x0, y1, c), t11 = t.at(x1, y1, c);
    r.e[c] = ((S)1 - a) * ((S)1 - b) * t00 + a * ((S)1 - b) * t10 + ((S)1 - a) * b * t01 + a * b * t11;
  }
  return r;
}

template <class S>
tvec4<S> filter_linear_1d(const sampler1D& t, S s) {
  const S us = s * (S)t.w - (S)0.5;
  const S fi = floor(us);
  const S a = us - fi;
  auto cl = [](long v, int n) { return (int)(v < 0 ? 0 : (v > n - 1 ? n - 1 : v)); };
  const long i0 = (long)fi;
  const int x0 = cl(i0, t.w), x1 = cl(i0 + 1, t.w);
  tvec4<S> r;
  for (int c = 0; c < 4; ++c) r.e[c] = ((S)1 - a) * (S)t.at(x0, c) + a * (S)t.at(x1, c);
  return r;
}

// GL 4.5 core, 8.13: the face of the major axis, (s, t) = ((sc / |ma|) + 1) / 2,
// ((tc / |ma|) + 1) / 2 from table 8.19, then GL_LINEAR with the coordinates
// clamped within the face (GL_TEXTURE_CUBE_MAP_SEAMLESS off).
template <class S>
tvec4<S> filter_cube(const samplerCube& t, S rx, S ry, S rz) {
  tvec4<S> r;
  if (!t.faces) return r;
  const S ax = rx < 0 ? -rx : rx, ay = ry < 0 ? -ry : ry, az = rz < 0 ? -rz : rz;
  int face;
  S sc, tc, ma;
  if (ax >= ay && ax >= az) {
    face = rx >= 0 ? 0 : 1, sc = rx >= 0 ? -rz : rz, tc = -ry, ma = ax;
  } else if (ay >= az) {
    face = ry >= 0 ? 2 : 3, sc = rx, tc = ry >= 0 ? rz : -rz, ma = ay;
  } else {
    face = rz >= 0 ? 4 : 5, sc = rz >= 0 ? rx : -rx, tc = -ry, ma = az;
  }
  if (ma == 0) return r;
  const S s = (S)0.5 * (sc / ma + (S)1), tt = (S)0.5 * (tc / ma + (S)1);
  const S u = s * (S)t.size - (S)0.5, v = tt * (S)t.size - (S)0.5;
  const S u0 = floor(u), v0 = floor(v), a = u - u0, b = v - v0;
  auto cl = [&](long i) { return (int)(i < 0 ? 0 : (i > t.size - 1 ? t.size - 1 : i)); };
  const int x0 = cl((long)u0), x1 = cl((long)u0 + 1), y0 = cl((long)v0), y1 = cl((long)v0 + 1);
  for (int c = 0; c < 4; ++c)
    r.e[c] = ((S)1 - a) * ((S)1 - b) * (S)t.at(face, x0, y0, c) + a * ((S)1 - b) * (S)t.at(face, x1, y0, c) +
             ((S)1 - a) * b * (S)t.at(face, x0, y1, c) + a * b * (S)t.at(face, x1, y1, c);
  return r;
}

template <class S>
tvec4<S> image_load_1d(const image1D& im, int x) {
  tvec4<S> r;
  if (x < 0 || x >= im.w) return r;
  for (int c = 0; c < 4; ++c)
    r.e[c] = im.is_double ? (S) static_cast<const double*>(im.data)[4 * (size_t)x + c]
                          : (S) static_cast<const float*>(im.data)[4 * (size_t)x + c];
  return r;
}

template <class S>
void image_store_1d(const image1D& im, int x, const tvec4<S>& v) {
  if (x < 0 || x >= im.w) return;
  for (int c = 0; c < 4; ++c) {
    if (im.is_double)
      static_cast<double*>(im.data)[4 * (size_t)x + c] = (double)v.e[c];
    else
      static_cast<float*>(im.data)[4 * (size_t)x + c] = (float)v.e[c];
  }
}

template <class S>
tvec4<S> image_load(const image2D& im, const ivec2& p) {
  tvec4<S> r;  // out of range: zero (GLSL 4.50, 8.12)
  if (p.x < 0 || p.y < 0 || p.x >= im.w || p.y >= im.h) return r;
  const size_t o = ((size_t)p.y * im.w + p.x) * 4;
  for (int c = 0; c < 4; ++c)
    r.e[c] = im.is_double ? (S) static_cast<const double*>(im.data)[o + c] : (S) static_cast<const float*>(im.data)[o + c];
  return r;
}

template <class S>
void image_store(const image2D& im, const ivec2& p, const tvec4<S>& v) {
  if (p.x < 0 || p.y < 0 || p.x >= im.w || p.y >= im.h) return;  // ignored out of range
  const size_t o = ((size_t)p.y * im.w + p.x) * 4;
  for (int c = 0; c < 4; ++c) {
    if (im.is_double)
      static_cast<double*>(im.data)[o + c] = (double)v.e[c];
    else
      static_cast<float*>(im.data)[o + c] = (float)v.e[c];
  }
}

}  // namespace detail

// ------------------------------------------------ per-precision built-ins ----
#define GLSL_BUILTINS(S, NS)                                                                  \
  namespace NS {                                                                              \
  using scalar = S;                                                                           \
  using vec2 = tvec2<S>;                                                                      \
  using vec3 = tvec3<S>;                                                                      \
  using vec4 = tvec4<S>;                                                                      \
  using mat4 = tmat4<S>;                                                                      \
  inline S pow(S a, S b) { return ::pow(a, b); }                                              \
  inline S sqrt(S a) { return ::sqrt(a); }                                                    \
  inline S abs(S a) { return ::fabs(a); }                                                     \
  inline S max(S a, S b) { return b > a ? b : a; } /* GLSL: y if x < y, else x */             \
  inline S min(S a, S b) { return b < a ? b : a; }                                            \
  inline S clamp(S x, S lo, S hi) { return min(max(x, lo), hi); }                             \
  inline S floor(S a) { return ::floor(a); }                                                  \
  inline S exp(S a) { return ::exp(a); }                                                      \
  inline S sin(S a) { return ::sin(a); }                                                      \
  inline S cos(S a) { return ::cos(a); }                                                      \
  inline S acos(S a) { return ::acos(a); }                                                    \
  inline S fract(S a) { return a - floor(a); }                                                \
  inline S mix(S x, S y, S a) { return x * ((S)1 - a) + y * a; }                              \
  inline S sign(S a) { return a > (S)0 ? (S)1 : (a < (S)0 ? (S)-1 : (S)0); }                  \
  inline vec2 max(const vec2& a, const vec2& b) { return vec2(max(a.x, b.x), max(a.y, b.y)); } \
  inline vec2 min(const vec2& a, const vec2& b) { return vec2(min(a.x, b.x), min(a.y, b.y)); } \
  inline bvec2 greaterThan(const vec2& a, const vec2& b) { return bvec2{a.x > b.x, a.y > b.y}; } \
  inline bvec2 lessThan(const vec2& a, const vec2& b) { return bvec2{a.x < b.x, a.y < b.y}; }   \
  inline vec4 texture(const sampler1D& t, S s) { return detail::filter_linear_1d<S>(t, s); }  \
  inline vec4 texelFetch(const sampler1D& t, int x, int) {                                    \
    vec4 r;                                                                                   \
    if (x < 0 || x >= t.w) return r;                                                          \
    for (int c = 0; c < 4; ++c) r.e[c] = (S)t.at(x, c);                                       \
    return r;                                                                                 \
  }                                                                                           \
  inline vec4 imageLoad(const image1D& im, int x) { return detail::image_load_1d<S>(im, x); } \
  inline void imageStore(const image1D& im, int x, const vec4& v) { detail::image_store_1d<S>(im, x, v); } \
  inline vec3 floor(const vec3& v) { return vec3(floor(v.x), floor(v.y), floor(v.z)); }       \
  inline vec2 floor(const vec2& v) { return vec2(floor(v.x), floor(v.y)); }                    \
  inline vec4 max(const vec4& a, const vec4& b) {                                             \
    return vec4(max(a.x, b.x), max(a.y, b.y), max(a.z, b.z), max(a.w, b.w));                  \
  }                                                                                           \
  inline vec4 min(const vec4& a, const vec4& b) {                                             \
    return vec4(min(a.x, b.x), min(a.y, b.y), min(a.z, b.z), min(a.w, b.w));                  \
  }                                                                                           \
  inline S smoothstep(S e0, S e1, S x) {                                                      \
    const S t = clamp((x - e0) / (e1 - e0), (S)0, (S)1);                                      \
    return t * t * ((S)3 - (S)2 * t);                                                         \
  }                                                                                           \
  inline S dot(const vec2& a, const vec2& b) { return a.x * b.x + a.y * b.y; }                \
  inline S dot(const vec3& a, const vec3& b) { return a.x * b.x + a.y * b.y + a.z * b.z; }    \
  inline S length(const vec2& v) { return sqrt(dot(v, v)); }                                  \
  inline S length(const vec3& v) { return sqrt(dot(v, v)); }                                  \
  inline S distance(const vec2& a, const vec2& b) { return length(a - b); }                   \
  inline vec3 normalize(const vec3& v) { return v / length(v); }                              \
  inline vec2 normalize(const vec2& v) { return v / length(v); }                              \
  inline vec3 reflect(const vec3& i, const vec3& n) { return i - (S)2 * dot(n, i) * n; }      \
  inline vec3 refract(const vec3& i, const vec3& n, S eta) {                                  \
    const S d = dot(n, i), k = (S)1 - eta * eta * ((S)1 - d * d);                             \
    if (k < (S)0) return vec3((S)0);                                                          \
    return eta * i - (eta * d + sqrt(k)) * n;                                                 \
  }                                                                                           \
  inline vec4 mix(const vec4& x, const vec4& y, S a) { return x * ((S)1 - a) + y * a; }       \
  inline vec4 texture(const samplerCube& t, const vec3& r) { return detail::filter_cube<S>(t, r.x, r.y, r.z); } \
  inline mat4 inverse(const mat4& m) { return inverse_of(m); }                                \
  inline vec3 cross(const vec3& a, const vec3& b) {                                           \
    return vec3(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y);         \
  }                                                                                           \
  inline vec4 texture(const sampler2D& t, const vec2& uv) { return detail::filter_linear<S>(t, uv.x, uv.y); } \
  inline vec4 texelFetch(const sampler2D& t, const ivec2& p, int) {                           \
    vec4 r;                                                                                   \
    if (p.x < 0 || p.y < 0 || p.x >= t.w || p.y >= t.h) return r;                             \
    for (int c = 0; c < 4; ++c) r.e[c] = (S)t.at(p.x, p.y, c);                                \
    return r;                                                                                 \
  }                                                                                           \
  inline vec4 imageLoad(const image2D& im, const ivec2& p) { return detail::image_load<S>(im, p); } \
  inline void imageStore(const image2D& im, const ivec2& p, const vec4& v) { detail::image_store<S>(im, p, v); } \
  }

GLSL_BUILTINS(float, f32)
GLSL_BUILTINS(double, f64)
#undef GLSL_BUILTINS

}  // namespace glsl

// Opens a shader's namespace body: its types and built-ins at precision NS
// (f32 or f64), found by ordinary lookup ahead of the C library's names, and
// the invocation id that the dispatch loop sets.  Before the shader's text
// the dispatch unit defines GLSL_CONST(name, init): `(init)` for the float
// build, the float build's folded constant for the double build.
#define GLSL_PRELUDE(NS)                                                                  \
  using glsl::bvec2;                                                                      \
  using glsl::ivec2;                                                                      \
  using glsl::ivec3;                                                                      \
  using glsl::ivec4;                                                                      \
  using glsl::atomicAdd;                                                                  \
  using glsl::NS::floor;                                                                  \
  using glsl::uvec3;                                                                      \
  using glsl::sampler2D;                                                                  \
  using glsl::image2D;                                                                    \
  using glsl::NS::vec2;                                                                   \
  using glsl::NS::vec3;                                                                   \
  using glsl::NS::vec4;                                                                   \
  using glsl::NS::mat4;                                                                   \
  using glsl::NS::pow;                                                                    \
  using glsl::NS::sqrt;                                                                   \
  using glsl::NS::abs;                                                                    \
  using glsl::NS::max;                                                                    \
  using glsl::NS::min;                                                                    \
  using glsl::NS::clamp;                                                                  \
  using glsl::clamp;                                                                      \
  using glsl::NS::smoothstep;                                                             \
  using glsl::NS::dot;                                                                    \
  using glsl::NS::length;                                                                 \
  using glsl::NS::distance;                                                               \
  using glsl::NS::normalize;                                                              \
  using glsl::NS::cross;                                                                  \
  using glsl::NS::texture;                                                                \
  using glsl::NS::texelFetch;                                                             \
  using glsl::NS::imageLoad;                                                              \
  using glsl::NS::imageStore;                                                             \
  using glsl::textureSize;                                                                \
  using glsl::imageSize;                                                                  \
  using glsl::greaterThanEqual;                                                           \
  using glsl::any;                                                                        \
  using glsl::all;                                                                        \
  using glsl::max;                                                                        \
  using glsl::sampler1D;                                                                  \
  using glsl::image1D;                                                                    \
  using glsl::NS::exp;                                                                    \
  using glsl::NS::sin;                                                                    \
  using glsl::NS::cos;                                                                    \
  using glsl::NS::acos;                                                                   \
  using glsl::NS::fract;                                                                  \
  using glsl::NS::mix;                                                                    \
  using glsl::NS::reflect;                                                                \
  using glsl::NS::refract;                                                                \
  using glsl::NS::inverse;                                                                \
  using glsl::samplerCube;                                                                \
  using glsl::NS::sign;                                                                   \
  using glsl::NS::greaterThan;                                                            \
  using glsl::NS::lessThan;                                                               \
  typedef unsigned int uint;                                                              \
  typedef glsl::NS::scalar glsl_cfloat;                                                   \
  thread_local uvec3 gl_GlobalInvocationID;
