/* Stand-in for the dependency's small fixed-size vector type. */
#pragma once
#include <cmath>
template <int N> struct Vec {
  float v[N];
  Vec() { for (int i = 0; i < N; ++i) v[i] = 0; }
  Vec(float a, float b, float c) { v[0] = a; v[1] = b; v[2] = c; }
  Vec(float a, float b, float c, float d) { v[0] = a; v[1] = b; v[2] = c; v[3] = d; }
  float& operator[](int i) { return v[i]; }
  const float& operator[](int i) const { return v[i]; }
  Vec operator-(const Vec& o) const { Vec r; for (int i = 0; i < N; ++i) r.v[i] = v[i] - o.v[i]; return r; }
  Vec operator+(const Vec& o) const { Vec r; for (int i = 0; i < N; ++i) r.v[i] = v[i] + o.v[i]; return r; }
  Vec& operator+=(const Vec& o) { for (int i = 0; i < N; ++i) v[i] += o.v[i]; return *this; }
  Vec operator/(float s) const { Vec r; for (int i = 0; i < N; ++i) r.v[i] = v[i] / s; return r; }
  Vec operator*(float s) const { Vec r; for (int i = 0; i < N; ++i) r.v[i] = v[i] * s; return r; }
};
/* dot product: left-to-right sum of products */
template <int N> float operator^(const Vec<N>& a, const Vec<N>& b) {
  float s = a[0] * b[0];
  for (int i = 1; i < N; ++i) s += a[i] * b[i];
  return s;
}
inline Vec<3> operator%(const Vec<3>& a, const Vec<3>& b) {
  return Vec<3>(a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]);
}
template <int N> Vec<N> operator*(float s, const Vec<N>& a) { return a * s; }
template <int N> float len(const Vec<N>& a) { return std::sqrt(a ^ a); }
typedef Vec<3> vec3;
typedef Vec<4> vec4;
typedef Vec<3> point;
#define DOT ^
#define CROSS %
