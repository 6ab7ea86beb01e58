// The part of glm (OpenGL Mathematics, the reference's vector library, absent from the
// reference tree: an unfetched git submodule) that the reference's kernels and their
// structs use when they are compiled for the CPU: the neighbour search
// (ParticleSearchKernels.cu) and the step (DFSPHKernels.cu with the kernel table, the
// volume-map interpolation and the bounding box). Written here from glm's documented
// semantics:
//   * vec3 / ivec3 / uvec3 / dvec3 with component-wise arithmetic, implicit conversions
//     by static_cast of each component, operator[] over x, y, z, equality; default
//     construction to zero;
//   * dot(a, b) = (a.x b.x + a.y b.y) + a.z b.z, length2 = dot(v, v), length = sqrt(dot),
//     normalize(v) = v * (1 / sqrt(dot(v, v))), cross, component-wise min / max
//     (min(a, b) = b < a ? b : a, max(a, b) = a < b ? b : a), compAdd = x + y + z;
//   * mat3x3 stored as three columns (m[c] is column c, m[c][r] its row r); mat * vec
//     sums the columns weighted by the components in column order; outerProduct(c, r)
//     has column j = c * r[j]; identity; inverse by the adjugate over the determinant;
//     default construction to zero (the reference writes glm::mat3x3() for an empty sum);
//   * vec2 / vec4 / dvec2 / dvec4 / mat4 as types only (the reference declares host
//     functions that take them).
// Test infrastructure only: the last ulp of inverse and normalize can differ from glm's
// own code.
#ifndef VFD_REF_SEARCH_GLM_SUBSET_H
#define VFD_REF_SEARCH_GLM_SUBSET_H

#include <cmath>

namespace glm {

template <class T>
struct tvec3 {
    T x, y, z;
    tvec3() : x(0), y(0), z(0) {}
    explicit tvec3(T s) : x(s), y(s), z(s) {}
    tvec3(T a, T b, T c) : x(a), y(b), z(c) {}
    template <class U>
    tvec3(const tvec3<U>& o) : x(static_cast<T>(o.x)), y(static_cast<T>(o.y)), z(static_cast<T>(o.z)) {}
    T& operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
    const T& operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
    tvec3& operator+=(const tvec3& o) { x += o.x; y += o.y; z += o.z; return *this; }
    tvec3& operator-=(const tvec3& o) { x -= o.x; y -= o.y; z -= o.z; return *this; }
    tvec3& operator*=(T s) { x *= s; y *= s; z *= s; return *this; }
    tvec3& operator/=(T s) { x /= s; y /= s; z /= s; return *this; }
    tvec3& operator*=(const tvec3& o) { x *= o.x; y *= o.y; z *= o.z; return *this; }
    tvec3& operator/=(const tvec3& o) { x /= o.x; y /= o.y; z /= o.z; return *this; }
};
template <class T> tvec3<T> operator+(const tvec3<T>& a, const tvec3<T>& b) { return tvec3<T>(a.x + b.x, a.y + b.y, a.z + b.z); }
template <class T> tvec3<T> operator-(const tvec3<T>& a, const tvec3<T>& b) { return tvec3<T>(a.x - b.x, a.y - b.y, a.z - b.z); }
template <class T> tvec3<T> operator-(const tvec3<T>& a) { return tvec3<T>(-a.x, -a.y, -a.z); }
template <class T> tvec3<T> operator*(const tvec3<T>& a, const tvec3<T>& b) { return tvec3<T>(a.x * b.x, a.y * b.y, a.z * b.z); }
template <class T> tvec3<T> operator/(const tvec3<T>& a, const tvec3<T>& b) { return tvec3<T>(a.x / b.x, a.y / b.y, a.z / b.z); }
template <class T> tvec3<T> operator*(const tvec3<T>& a, T s) { return tvec3<T>(a.x * s, a.y * s, a.z * s); }
template <class T> tvec3<T> operator*(T s, const tvec3<T>& a) { return tvec3<T>(s * a.x, s * a.y, s * a.z); }
template <class T> tvec3<T> operator/(const tvec3<T>& a, T s) { return tvec3<T>(a.x / s, a.y / s, a.z / s); }
template <class T> tvec3<T> operator/(T s, const tvec3<T>& a) { return tvec3<T>(s / a.x, s / a.y, s / a.z); }
template <class T> bool operator==(const tvec3<T>& a, const tvec3<T>& b) { return a.x == b.x && a.y == b.y && a.z == b.z; }
template <class T> bool operator!=(const tvec3<T>& a, const tvec3<T>& b) { return !(a == b); }
template <class T> tvec3<T> operator+(const tvec3<T>& a, T s) { return tvec3<T>(a.x + s, a.y + s, a.z + s); }
template <class T> tvec3<T> operator-(const tvec3<T>& a, T s) { return tvec3<T>(a.x - s, a.y - s, a.z - s); }

using vec3 = tvec3<float>;
using ivec3 = tvec3<int>;
using uvec3 = tvec3<unsigned int>;
using dvec3 = tvec3<double>;
// two- and four-component vectors as types only (the reference declares host functions on them)
template <class T> struct tvec2 { T x, y; };
template <class T> struct tvec4 { T x, y, z, w; };
using vec2 = tvec2<float>;
using vec4 = tvec4<float>;
using dvec2 = tvec2<double>;
using dvec4 = tvec4<double>;

template <class T> T dot(const tvec3<T>& a, const tvec3<T>& b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
template <class T> T length2(const tvec3<T>& v) { return dot(v, v); }
template <class T> T length(const tvec3<T>& v) { return std::sqrt(dot(v, v)); }
template <class T> tvec3<T> normalize(const tvec3<T>& v) { return v * (static_cast<T>(1) / std::sqrt(dot(v, v))); }
template <class T> tvec3<T> cross(const tvec3<T>& a, const tvec3<T>& b) {
    return tvec3<T>(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y);
}
template <class T> T compAdd(const tvec3<T>& v) { return (v.x + v.y) + v.z; }
template <class T> T min(T a, T b) { return b < a ? b : a; }
template <class T> T max(T a, T b) { return a < b ? b : a; }
template <class T> tvec3<T> min(const tvec3<T>& a, const tvec3<T>& b) { return tvec3<T>(min(a.x, b.x), min(a.y, b.y), min(a.z, b.z)); }
template <class T> tvec3<T> max(const tvec3<T>& a, const tvec3<T>& b) { return tvec3<T>(max(a.x, b.x), max(a.y, b.y), max(a.z, b.z)); }

struct mat3x3 {
    vec3 c[3];
    mat3x3() {}
    explicit mat3x3(float s) { c[0] = vec3(s, 0.f, 0.f); c[1] = vec3(0.f, s, 0.f); c[2] = vec3(0.f, 0.f, s); }
    vec3& operator[](int i) { return c[i]; }
    const vec3& operator[](int i) const { return c[i]; }
    mat3x3& operator+=(const mat3x3& o) { c[0] += o.c[0]; c[1] += o.c[1]; c[2] += o.c[2]; return *this; }
    mat3x3& operator-=(const mat3x3& o) { c[0] -= o.c[0]; c[1] -= o.c[1]; c[2] -= o.c[2]; return *this; }
};
using mat3 = mat3x3;
inline mat3x3 operator+(const mat3x3& a, const mat3x3& b) { mat3x3 r = a; r += b; return r; }
inline mat3x3 operator-(const mat3x3& a, const mat3x3& b) { mat3x3 r = a; r -= b; return r; }
inline mat3x3 operator*(float s, const mat3x3& m) { mat3x3 r; for (int i = 0; i < 3; i++) r.c[i] = s * m.c[i]; return r; }
inline mat3x3 operator*(const mat3x3& m, float s) { mat3x3 r; for (int i = 0; i < 3; i++) r.c[i] = m.c[i] * s; return r; }
inline vec3 operator*(const mat3x3& m, const vec3& v) {
    return vec3((m.c[0].x * v.x + m.c[1].x * v.y) + m.c[2].x * v.z, (m.c[0].y * v.x + m.c[1].y * v.y) + m.c[2].y * v.z,
                (m.c[0].z * v.x + m.c[1].z * v.y) + m.c[2].z * v.z);
}
inline mat3x3 operator*(const mat3x3& a, const mat3x3& b) { mat3x3 r; for (int i = 0; i < 3; i++) r.c[i] = a * b.c[i]; return r; }
inline mat3x3 outerProduct(const vec3& col, const vec3& row) {
    mat3x3 r;
    for (int j = 0; j < 3; j++) r.c[j] = col * row[j];
    return r;
}
template <class M> M identity() { return M(1.0f); }
// Inverse: the transposed cofactor matrix divided by the determinant (expanded along the
// first column).
inline mat3x3 inverse(const mat3x3& m) {
    auto e = [&](int col, int row) { return m.c[col][row]; };
    const float c00 = e(1, 1) * e(2, 2) - e(2, 1) * e(1, 2);
    const float c01 = e(0, 1) * e(2, 2) - e(2, 1) * e(0, 2);
    const float c02 = e(0, 1) * e(1, 2) - e(1, 1) * e(0, 2);
    const float inv = 1.0f / (e(0, 0) * c00 - e(1, 0) * c01 + e(2, 0) * c02);
    mat3x3 r;
    r.c[0] = vec3(c00 * inv, -c01 * inv, c02 * inv);
    r.c[1] = vec3(-(e(1, 0) * e(2, 2) - e(2, 0) * e(1, 2)) * inv, (e(0, 0) * e(2, 2) - e(2, 0) * e(0, 2)) * inv,
                  -(e(0, 0) * e(1, 2) - e(1, 0) * e(0, 2)) * inv);
    r.c[2] = vec3((e(1, 0) * e(2, 1) - e(2, 0) * e(1, 1)) * inv, -(e(0, 0) * e(2, 1) - e(2, 0) * e(0, 1)) * inv,
                  (e(0, 0) * e(1, 1) - e(1, 0) * e(0, 1)) * inv);
    return r;
}

struct mat4 {
    float v[16];
};

}  // namespace glm

#endif
