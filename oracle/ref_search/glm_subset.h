// The part of glm (OpenGL Mathematics, the reference's vector library, absent from the
// reference tree: an unfetched git submodule) that the reference's neighbour-search
// kernels and their structs use: vec3 / ivec3 / uvec3 with component-wise arithmetic
// and the explicit conversions between them, written here from glm's documented
// semantics (component-wise operators, conversions by static_cast of each component).
// Test infrastructure only.
#ifndef VFD_REF_SEARCH_GLM_SUBSET_H
#define VFD_REF_SEARCH_GLM_SUBSET_H

namespace glm {

template <class T>
struct tvec3 {
    T x, y, z;
    tvec3() : x(0), y(0), z(0) {}
    explicit tvec3(T s) : x(s), y(s), z(s) {}
    tvec3(T a, T b, T c) : x(a), y(b), z(c) {}
    template <class U>
    explicit tvec3(const tvec3<U>& o) : x(static_cast<T>(o.x)), y(static_cast<T>(o.y)), z(static_cast<T>(o.z)) {}
    tvec3& operator+=(const tvec3& o) { x += o.x; y += o.y; z += o.z; return *this; }
    tvec3& operator-=(const tvec3& o) { x -= o.x; y -= o.y; z -= o.z; return *this; }
};
template <class T> tvec3<T> operator+(const tvec3<T>& a, const tvec3<T>& b) { return tvec3<T>(a.x + b.x, a.y + b.y, a.z + b.z); }
template <class T> tvec3<T> operator-(const tvec3<T>& a, const tvec3<T>& b) { return tvec3<T>(a.x - b.x, a.y - b.y, a.z - b.z); }
template <class T> tvec3<T> operator*(const tvec3<T>& a, const tvec3<T>& b) { return tvec3<T>(a.x * b.x, a.y * b.y, a.z * b.z); }
template <class T> tvec3<T> operator*(const tvec3<T>& a, T s) { return tvec3<T>(a.x * s, a.y * s, a.z * s); }

using vec3 = tvec3<float>;
using ivec3 = tvec3<int>;
using uvec3 = tvec3<unsigned int>;

}  // namespace glm

#endif
