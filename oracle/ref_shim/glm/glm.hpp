// Stand-in for <glm/glm.hpp> (test infrastructure: the reference-pin builds
// only).  GLM is a third-party dependency of the reference that this image
// does not have.  This header provides the GLM types and functions the
// reference's host geometry (tool.cpp, geometric_primitives.cpp) and its
// device code (actions_gpu.cu, leap_frog.cu, grid.cu, FEM_thermal_gpu.cu,
// tool_FEM.cu) use, written from
// GLM's documented semantics:
//   - vectors with component-wise +, -, *, / and scalar forms;
//   - column-major matrices built column by column (m[c][r] is column c, row
//     r); the scalar constructor puts the scalar on the diagonal;
//   - matrix + - matrix and scalar * matrix component-wise; matrix * matrix
//     the linear-algebra product, column c of the result being
//     a[0] * b[c][0] + a[1] * b[c][1] (+ a[2] * b[c][2]);
//   - transpose; the inverse of a 2x2 as its adjugate over its determinant;
//     row vector * matrix is the vector's dot product with each column;
//   - == / != of vectors component-wise;
//   - dot(a, b) = (a * b).x + (a * b).y; length(v) = sqrt(dot(v, v));
//     distance(a, b) = length(b - a); normalize(v) = v * inversesqrt(dot(v, v))
//     with inversesqrt(x) = 1 / sqrt(x);
//   - determinant of a 3x3 by cofactor expansion along the first column.
// Under nvcc every function is __host__ __device__.
// kernels.cuh and plasticity.cuh (the other pinned headers) use none of it.
#pragma once

// the standard headers GLM's own glm.hpp brings in
#include <cassert>
#include <cfloat>
#include <climits>
#include <cmath>
#include <limits>

#if defined(__CUDACC__)
#define GLMS_HD __host__ __device__
#else
#define GLMS_HD
#endif

namespace glm {

template <class T>
struct tvec2 {
    T x, y;
    GLMS_HD tvec2() : x(0), y(0) {}
    GLMS_HD tvec2(T a, T b) : x(a), y(b) {}
    GLMS_HD explicit tvec2(T s) : x(s), y(s) {}
    GLMS_HD T &operator[](int i) { return i ? y : x; }
    GLMS_HD const T &operator[](int i) const { return i ? y : x; }
    GLMS_HD tvec2 &operator+=(const tvec2 &o) { x += o.x; y += o.y; return *this; }
    GLMS_HD tvec2 &operator-=(const tvec2 &o) { x -= o.x; y -= o.y; return *this; }
    GLMS_HD tvec2 &operator*=(T s) { x *= s; y *= s; return *this; }
    GLMS_HD tvec2 &operator/=(T s) { x /= s; y /= s; return *this; }
};

template <class T> GLMS_HD tvec2<T> operator+(const tvec2<T> &a, const tvec2<T> &b) { return tvec2<T>(a.x + b.x, a.y + b.y); }
template <class T> GLMS_HD tvec2<T> operator-(const tvec2<T> &a, const tvec2<T> &b) { return tvec2<T>(a.x - b.x, a.y - b.y); }
template <class T> GLMS_HD tvec2<T> operator-(const tvec2<T> &a) { return tvec2<T>(-a.x, -a.y); }
template <class T> GLMS_HD tvec2<T> operator*(const tvec2<T> &a, const tvec2<T> &b) { return tvec2<T>(a.x * b.x, a.y * b.y); }
template <class T> GLMS_HD tvec2<T> operator/(const tvec2<T> &a, const tvec2<T> &b) { return tvec2<T>(a.x / b.x, a.y / b.y); }
template <class T> GLMS_HD tvec2<T> operator*(const tvec2<T> &a, T s) { return tvec2<T>(a.x * s, a.y * s); }
template <class T> GLMS_HD tvec2<T> operator*(T s, const tvec2<T> &a) { return tvec2<T>(s * a.x, s * a.y); }
template <class T> GLMS_HD tvec2<T> operator/(const tvec2<T> &a, T s) { return tvec2<T>(a.x / s, a.y / s); }
template <class T> GLMS_HD tvec2<T> operator+(const tvec2<T> &a, T s) { return tvec2<T>(a.x + s, a.y + s); }
template <class T> GLMS_HD tvec2<T> operator-(const tvec2<T> &a, T s) { return tvec2<T>(a.x - s, a.y - s); }

template <class T>
struct tvec3 {
    T x, y, z;
    GLMS_HD tvec3() : x(0), y(0), z(0) {}
    GLMS_HD tvec3(T a, T b, T c) : x(a), y(b), z(c) {}
    GLMS_HD T &operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
    GLMS_HD const T &operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};

template <class T> GLMS_HD tvec3<T> operator+(const tvec3<T> &a, const tvec3<T> &b) { return tvec3<T>(a.x + b.x, a.y + b.y, a.z + b.z); }
template <class T> GLMS_HD tvec3<T> operator-(const tvec3<T> &a, const tvec3<T> &b) { return tvec3<T>(a.x - b.x, a.y - b.y, a.z - b.z); }
template <class T> GLMS_HD tvec3<T> operator*(const tvec3<T> &a, T s) { return tvec3<T>(a.x * s, a.y * s, a.z * s); }
template <class T> GLMS_HD tvec3<T> operator*(T s, const tvec3<T> &a) { return tvec3<T>(s * a.x, s * a.y, s * a.z); }

template <class T>
struct tmat2x2 {
    tvec2<T> c[2];
    GLMS_HD tmat2x2() : c{tvec2<T>(1, 0), tvec2<T>(0, 1)} {}
    GLMS_HD explicit tmat2x2(T s) : c{tvec2<T>(s, 0), tvec2<T>(0, s)} {}
    GLMS_HD tmat2x2(T x0, T y0, T x1, T y1) : c{tvec2<T>(x0, y0), tvec2<T>(x1, y1)} {}
    GLMS_HD tvec2<T> &operator[](int i) { return c[i]; }
    GLMS_HD const tvec2<T> &operator[](int i) const { return c[i]; }
};

template <class T>
struct tmat3x3 {
    tvec3<T> c[3];
    GLMS_HD tmat3x3() : c{tvec3<T>(1, 0, 0), tvec3<T>(0, 1, 0), tvec3<T>(0, 0, 1)} {}
    GLMS_HD explicit tmat3x3(T s) : c{tvec3<T>(s, 0, 0), tvec3<T>(0, s, 0), tvec3<T>(0, 0, s)} {}
    GLMS_HD tmat3x3(T x0, T y0, T z0, T x1, T y1, T z1, T x2, T y2, T z2)
        : c{tvec3<T>(x0, y0, z0), tvec3<T>(x1, y1, z1), tvec3<T>(x2, y2, z2)} {}
    GLMS_HD tvec3<T> &operator[](int i) { return c[i]; }
    GLMS_HD const tvec3<T> &operator[](int i) const { return c[i]; }
};

// 3 columns of 2 rows
template <class T>
struct tmat3x2 {
    tvec2<T> c[3];
    GLMS_HD tmat3x2() : c{tvec2<T>(1, 0), tvec2<T>(0, 1), tvec2<T>(0, 0)} {}
    GLMS_HD explicit tmat3x2(T s) : c{tvec2<T>(s, 0), tvec2<T>(0, s), tvec2<T>(0, 0)} {}
    GLMS_HD tmat3x2(T x0, T y0, T x1, T y1, T x2, T y2) : c{tvec2<T>(x0, y0), tvec2<T>(x1, y1), tvec2<T>(x2, y2)} {}
    GLMS_HD tvec2<T> &operator[](int i) { return c[i]; }
    GLMS_HD const tvec2<T> &operator[](int i) const { return c[i]; }
};

// 2 columns of 3 rows
template <class T>
struct tmat2x3 {
    tvec3<T> c[2];
    GLMS_HD tmat2x3() : c{tvec3<T>(1, 0, 0), tvec3<T>(0, 1, 0)} {}
    GLMS_HD explicit tmat2x3(T s) : c{tvec3<T>(s, 0, 0), tvec3<T>(0, s, 0)} {}
    GLMS_HD tmat2x3(T x0, T y0, T z0, T x1, T y1, T z1) : c{tvec3<T>(x0, y0, z0), tvec3<T>(x1, y1, z1)} {}
    GLMS_HD tvec3<T> &operator[](int i) { return c[i]; }
    GLMS_HD const tvec3<T> &operator[](int i) const { return c[i]; }
};

template <class T> GLMS_HD bool operator==(const tvec2<T> &a, const tvec2<T> &b) { return a.x == b.x && a.y == b.y; }
template <class T> GLMS_HD bool operator!=(const tvec2<T> &a, const tvec2<T> &b) { return !(a == b); }
template <class T> GLMS_HD bool operator==(const tvec3<T> &a, const tvec3<T> &b) {
    return a.x == b.x && a.y == b.y && a.z == b.z;
}
template <class T> GLMS_HD bool operator!=(const tvec3<T> &a, const tvec3<T> &b) { return !(a == b); }

// transposes
template <class T> GLMS_HD tmat2x2<T> transpose(const tmat2x2<T> &m) {
    return tmat2x2<T>(m[0][0], m[1][0], m[0][1], m[1][1]);
}
template <class T> GLMS_HD tmat3x2<T> transpose(const tmat2x3<T> &m) {
    return tmat3x2<T>(m[0][0], m[1][0], m[0][1], m[1][1], m[0][2], m[1][2]);
}
template <class T> GLMS_HD tmat2x3<T> transpose(const tmat3x2<T> &m) {
    return tmat2x3<T>(m[0][0], m[1][0], m[2][0], m[0][1], m[1][1], m[2][1]);
}

// inverse of a 2x2: the adjugate over the determinant
template <class T> GLMS_HD tmat2x2<T> inverse(const tmat2x2<T> &m) {
    const T one_over_det = static_cast<T>(1) / (m[0][0] * m[1][1] - m[1][0] * m[0][1]);
    return tmat2x2<T>(m[1][1] * one_over_det, -m[0][1] * one_over_det, -m[1][0] * one_over_det,
                      m[0][0] * one_over_det);
}

// products: column c of a * b is the sum over k of a's column k times b[c][k]
template <class T> GLMS_HD tmat3x2<T> operator*(const tmat2x2<T> &a, const tmat3x2<T> &b) {
    tmat3x2<T> r;
    for (int c = 0; c < 3; c++) r[c] = a[0] * b[c][0] + a[1] * b[c][1];
    return r;
}
template <class T> GLMS_HD tmat3x3<T> operator*(const tmat2x3<T> &a, const tmat3x2<T> &b) {
    tmat3x3<T> r;
    for (int c = 0; c < 3; c++) r[c] = a[0] * b[c][0] + a[1] * b[c][1];
    return r;
}
template <class T> GLMS_HD tmat2x3<T> operator*(T s, const tmat2x3<T> &m) {
    tmat2x3<T> r;
    for (int i = 0; i < 2; i++) r[i] = s * m[i];
    return r;
}

template <class T> GLMS_HD T dot(const tvec2<T> &a, const tvec2<T> &b) {
    tvec2<T> t = a * b;
    return t.x + t.y;
}
template <class T> GLMS_HD T length(const tvec2<T> &v) { return sqrt(dot(v, v)); }
template <class T> GLMS_HD T distance(const tvec2<T> &a, const tvec2<T> &b) { return length(b - a); }
template <class T> GLMS_HD T inversesqrt(T x) { return static_cast<T>(1) / sqrt(x); }
template <class T> GLMS_HD tvec2<T> normalize(const tvec2<T> &v) { return v * inversesqrt(dot(v, v)); }

// row vector times column-major matrix
template <class T> GLMS_HD tvec2<T> operator*(const tvec2<T> &v, const tmat2x2<T> &m) {
    return tvec2<T>(v.x * m[0][0] + v.y * m[0][1], v.x * m[1][0] + v.y * m[1][1]);
}

template <class T> GLMS_HD tmat3x3<T> operator+(const tmat3x3<T> &a, const tmat3x3<T> &b) {
    tmat3x3<T> r;
    for (int i = 0; i < 3; i++) r[i] = a[i] + b[i];
    return r;
}
template <class T> GLMS_HD tmat3x3<T> operator-(const tmat3x3<T> &a, const tmat3x3<T> &b) {
    tmat3x3<T> r;
    for (int i = 0; i < 3; i++) r[i] = a[i] - b[i];
    return r;
}
template <class T> GLMS_HD tmat3x3<T> operator*(T s, const tmat3x3<T> &m) {
    tmat3x3<T> r;
    for (int i = 0; i < 3; i++) r[i] = s * m[i];
    return r;
}
template <class T> GLMS_HD tmat3x3<T> operator*(const tmat3x3<T> &m, T s) {
    tmat3x3<T> r;
    for (int i = 0; i < 3; i++) r[i] = m[i] * s;
    return r;
}
template <class T> GLMS_HD tmat3x3<T> operator*(const tmat3x3<T> &a, const tmat3x3<T> &b) {
    tmat3x3<T> r;
    for (int c = 0; c < 3; c++) r[c] = a[0] * b[c][0] + a[1] * b[c][1] + a[2] * b[c][2];
    return r;
}
template <class T> GLMS_HD tmat3x3<T> &operator+=(tmat3x3<T> &a, const tmat3x3<T> &b) {
    for (int i = 0; i < 3; i++) a[i] = a[i] + b[i];
    return a;
}
template <class T> GLMS_HD tmat3x3<T> transpose(const tmat3x3<T> &m) {
    return tmat3x3<T>(m[0][0], m[1][0], m[2][0], m[0][1], m[1][1], m[2][1], m[0][2], m[1][2], m[2][2]);
}

template <class T> GLMS_HD T determinant(const tmat3x3<T> &m) {
    return m[0][0] * (m[1][1] * m[2][2] - m[2][1] * m[1][2]) - m[1][0] * (m[0][1] * m[2][2] - m[2][1] * m[0][2]) +
           m[2][0] * (m[0][1] * m[1][2] - m[1][1] * m[0][2]);
}

typedef tvec2<double> dvec2;
typedef tvec2<float> vec2;
typedef tvec3<double> dvec3;
typedef tvec3<float> vec3;
typedef tmat2x2<double> dmat2x2;
typedef tmat2x2<float> mat2x2;
typedef tmat3x3<double> dmat3x3;
typedef tmat3x3<float> mat3x3;
typedef tmat3x2<double> dmat3x2;
typedef tmat3x2<float> mat3x2;
typedef tmat2x3<double> dmat2x3;
typedef tmat2x3<float> mat2x3;

}  // namespace glm
