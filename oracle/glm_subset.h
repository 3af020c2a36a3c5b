// glm_subset.h -- test infrastructure for the erosion oracle, not product code.
//
// The reference (SimpleHydrology, source/*.h) is written against glm, which is
// not installed here. This header supplies the small part of glm's surface that
// the erosion headers use (vec2, ivec2, vec3, vec4, and the free functions length,
// normalize, dot, cross), written from glm's documented semantics:
//   * component-wise arithmetic, each component rounded to its own type;
//   * dot(a, b)      = sum of the component products, summed left to right;
//   * length(v)      = sqrt(dot(v, v));
//   * normalize(v)   = v * inversesqrt(dot(v, v)), inversesqrt(x) = 1 / sqrt(x);
//   * cross(x, y)    = (x.y*y.z - y.y*x.z, x.z*y.x - y.z*x.x, x.x*y.y - y.x*x.y);
//   * conversions between float and int vectors are implicit and per component
//     (float -> int truncates toward zero, as static_cast does).
// glm itself is an unvendored third-party dependency of the reference with no
// pinned version; its agreement with this header is asserted, not tested.
#pragma once

#include <cmath>

namespace glm {

template <typename T> struct tvec2;
template <typename T> struct tvec3;

template <typename T> struct tvec2 {
  T x, y;
  constexpr tvec2() : x(0), y(0) {}
  constexpr explicit tvec2(T s) : x(s), y(s) {}
  template <typename A, typename B>
  constexpr tvec2(A a, B b) : x(static_cast<T>(a)), y(static_cast<T>(b)) {}
  template <typename U>
  constexpr tvec2(const tvec2<U>& o) : x(static_cast<T>(o.x)), y(static_cast<T>(o.y)) {}

  tvec2& operator+=(const tvec2& o) { x = x + o.x; y = y + o.y; return *this; }
  tvec2& operator-=(const tvec2& o) { x = x - o.x; y = y - o.y; return *this; }
  tvec2& operator*=(T s) { x = x * s; y = y * s; return *this; }
  tvec2& operator/=(T s) { x = x / s; y = y / s; return *this; }
  tvec2& operator/=(const tvec2& o) { x = x / o.x; y = y / o.y; return *this; }
};

template <typename T> struct tvec3 {
  T x, y, z;
  constexpr tvec3() : x(0), y(0), z(0) {}
  constexpr explicit tvec3(T s) : x(s), y(s), z(s) {}
  template <typename A, typename B, typename C>
  constexpr tvec3(A a, B b, C c)
      : x(static_cast<T>(a)), y(static_cast<T>(b)), z(static_cast<T>(c)) {}

  tvec3& operator+=(const tvec3& o) { x = x + o.x; y = y + o.y; z = z + o.z; return *this; }
};

template <typename T> inline tvec2<T> operator+(tvec2<T> a, tvec2<T> b) { return tvec2<T>(a.x + b.x, a.y + b.y); }
template <typename T> inline tvec2<T> operator-(tvec2<T> a, tvec2<T> b) { return tvec2<T>(a.x - b.x, a.y - b.y); }
template <typename T> inline tvec2<T> operator*(tvec2<T> a, tvec2<T> b) { return tvec2<T>(a.x * b.x, a.y * b.y); }
template <typename T> inline tvec2<T> operator/(tvec2<T> a, tvec2<T> b) { return tvec2<T>(a.x / b.x, a.y / b.y); }
template <typename T> inline tvec2<T> operator*(tvec2<T> a, T s) { return tvec2<T>(a.x * s, a.y * s); }
template <typename T> inline tvec2<T> operator*(T s, tvec2<T> a) { return tvec2<T>(s * a.x, s * a.y); }
template <typename T> inline tvec2<T> operator/(tvec2<T> a, T s) { return tvec2<T>(a.x / s, a.y / s); }
template <typename T> inline tvec2<T> operator-(tvec2<T> a) { return tvec2<T>(-a.x, -a.y); }

template <typename T> inline tvec3<T> operator+(tvec3<T> a, tvec3<T> b) { return tvec3<T>(a.x + b.x, a.y + b.y, a.z + b.z); }
template <typename T> inline tvec3<T> operator-(tvec3<T> a, tvec3<T> b) { return tvec3<T>(a.x - b.x, a.y - b.y, a.z - b.z); }
template <typename T> inline tvec3<T> operator*(tvec3<T> a, tvec3<T> b) { return tvec3<T>(a.x * b.x, a.y * b.y, a.z * b.z); }
template <typename T> inline tvec3<T> operator*(tvec3<T> a, T s) { return tvec3<T>(a.x * s, a.y * s, a.z * s); }
template <typename T> inline tvec3<T> operator*(T s, tvec3<T> a) { return tvec3<T>(s * a.x, s * a.y, s * a.z); }
template <typename T> inline tvec3<T> operator/(tvec3<T> a, T s) { return tvec3<T>(a.x / s, a.y / s, a.z / s); }

// int * vec and vec / int appear with the reference's integer constants
// (quad::lodsize); glm promotes through the vector's value type.
inline tvec2<int> operator*(int s, tvec2<int> a) { return tvec2<int>(s * a.x, s * a.y); }
inline tvec2<int> operator/(tvec2<int> a, int s) { return tvec2<int>(a.x / s, a.y / s); }
inline tvec2<float> operator*(int s, tvec2<float> a) { return static_cast<float>(s) * a; }

template <typename T> inline T dot(tvec2<T> a, tvec2<T> b) {
  tvec2<T> t = a * b;
  return t.x + t.y;
}
template <typename T> inline T dot(tvec3<T> a, tvec3<T> b) {
  tvec3<T> t = a * b;
  return t.x + t.y + t.z;
}
template <typename T> inline T length(tvec2<T> v) { return std::sqrt(dot(v, v)); }
template <typename T> inline T length(tvec3<T> v) { return std::sqrt(dot(v, v)); }
template <typename T> inline T inversesqrt(T x) { return static_cast<T>(1) / std::sqrt(x); }
template <typename T> inline tvec2<T> normalize(tvec2<T> v) { return v * inversesqrt(dot(v, v)); }
template <typename T> inline tvec3<T> normalize(tvec3<T> v) { return v * inversesqrt(dot(v, v)); }
template <typename T> inline tvec3<T> cross(tvec3<T> x, tvec3<T> y) {
  return tvec3<T>(x.y * y.z - y.y * x.z, x.z * y.x - y.z * x.x, x.x * y.y - y.x * x.y);
}

// vec4 as the front end builds its texels: from four scalars, or from a vec3
// and a scalar, each converted to the component type
template <typename T> struct tvec4 {
  T x, y, z, w;
  template <typename A, typename B, typename C, typename D>
  constexpr tvec4(A a, B b, C c, D d)
      : x(static_cast<T>(a)), y(static_cast<T>(b)), z(static_cast<T>(c)), w(static_cast<T>(d)) {}
  template <typename S>
  constexpr tvec4(tvec3<T> v, S s) : x(v.x), y(v.y), z(v.z), w(static_cast<T>(s)) {}
};

typedef tvec2<float> vec2;
typedef tvec2<int> ivec2;
typedef tvec3<float> vec3;
typedef tvec4<float> vec4;

}  // namespace glm
