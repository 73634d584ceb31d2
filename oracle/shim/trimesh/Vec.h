// Minimal fixed-size vector type providing only the subset of the trimesh2
// Vec<N,T> interface that the reference's thinning, cell-complex, geometry,
// space-conversion and surfacing sources call.  Written from those call
// sites; it is test infrastructure for the oracle build and is never linked
// into the GPU library.
#pragma once
#include <algorithm>
#include <cmath>
#include <cstddef>
#include <ostream>

namespace trimesh {

template <std::size_t D, class T = float>
class Vec {
    T v[D];

public:
    typedef T value_type;
    typedef T* iterator;
    typedef const T* const_iterator;

    Vec() { for (std::size_t i = 0; i < D; ++i) v[i] = T(0); }
    explicit Vec(T x) { for (std::size_t i = 0; i < D; ++i) v[i] = x; }
    Vec(T x, T y) { static_assert(D == 2, "arity"); v[0] = x; v[1] = y; }
    Vec(T x, T y, T z) { static_assert(D == 3, "arity"); v[0] = x; v[1] = y; v[2] = z; }
    Vec(T x, T y, T z, T w) { static_assert(D == 4, "arity"); v[0] = x; v[1] = y; v[2] = z; v[3] = w; }
    template <class S> explicit Vec(const S* p) { for (std::size_t i = 0; i < D; ++i) v[i] = T(p[i]); }
    template <class S> explicit Vec(const Vec<D, S>& o) { for (std::size_t i = 0; i < D; ++i) v[i] = T(o[i]); }

    // a scalar assigned to a vector sets every component (octree.cpp assigns
    // an int to its ivec3 sizes)
    Vec& operator=(T x) { for (std::size_t i = 0; i < D; ++i) v[i] = x; return *this; }

    T& operator[](std::size_t i) { return v[i]; }
    const T& operator[](std::size_t i) const { return v[i]; }
    T* data() { return v; }
    const T* data() const { return v; }
    iterator begin() { return v; }
    iterator end() { return v + D; }
    const_iterator begin() const { return v; }
    const_iterator end() const { return v + D; }
    static constexpr std::size_t size() { return D; }

    Vec& operator+=(const Vec& o) { for (std::size_t i = 0; i < D; ++i) v[i] += o.v[i]; return *this; }
    Vec& operator-=(const Vec& o) { for (std::size_t i = 0; i < D; ++i) v[i] -= o.v[i]; return *this; }
    Vec& operator*=(T s) { for (std::size_t i = 0; i < D; ++i) v[i] *= s; return *this; }
    Vec& operator/=(T s) { for (std::size_t i = 0; i < D; ++i) v[i] /= s; return *this; }

    T dot(const Vec& o) const { T s = T(0); for (std::size_t i = 0; i < D; ++i) s += v[i] * o.v[i]; return s; }
    T max() const { T m = v[0]; for (std::size_t i = 1; i < D; ++i) m = std::max(m, v[i]); return m; }
    T min() const { T m = v[0]; for (std::size_t i = 1; i < D; ++i) m = std::min(m, v[i]); return m; }
};

template <std::size_t D, class T> inline Vec<D, T> operator+(Vec<D, T> a, const Vec<D, T>& b) { return a += b; }
template <std::size_t D, class T> inline Vec<D, T> operator-(Vec<D, T> a, const Vec<D, T>& b) { return a -= b; }
template <std::size_t D, class T> inline Vec<D, T> operator-(Vec<D, T> a) { for (auto& x : a) x = -x; return a; }
template <std::size_t D, class T> inline Vec<D, T> operator*(Vec<D, T> a, T s) { return a *= s; }
template <std::size_t D, class T> inline Vec<D, T> operator*(T s, Vec<D, T> a) { return a *= s; }
template <std::size_t D, class T> inline Vec<D, T> operator/(Vec<D, T> a, T s) { return a /= s; }
template <std::size_t D, class T> inline bool operator==(const Vec<D, T>& a, const Vec<D, T>& b) {
    for (std::size_t i = 0; i < D; ++i) if (a[i] != b[i]) return false;
    return true;
}
template <std::size_t D, class T> inline bool operator!=(const Vec<D, T>& a, const Vec<D, T>& b) { return !(a == b); }
template <std::size_t D, class T> inline bool operator<(const Vec<D, T>& a, const Vec<D, T>& b) {
    for (std::size_t i = 0; i < D; ++i) {
        if (a[i] < b[i]) return true;
        if (b[i] < a[i]) return false;
    }
    return false;
}

template <class T> inline T sqr(const T& x) { return x * x; }
// Squared length accumulated component by component in T, then sqrt in T.
template <std::size_t D, class T> inline T len2(const Vec<D, T>& a) { T s = T(0); for (std::size_t i = 0; i < D; ++i) s += sqr(a[i]); return s; }
template <std::size_t D, class T> inline T len(const Vec<D, T>& a) { return std::sqrt(len2(a)); }
template <std::size_t D, class T> inline T dist2(const Vec<D, T>& a, const Vec<D, T>& b) {
    T s = T(0); for (std::size_t i = 0; i < D; ++i) s += sqr(a[i] - b[i]); return s;
}
template <std::size_t D, class T> inline T dist(const Vec<D, T>& a, const Vec<D, T>& b) { return std::sqrt(dist2(a, b)); }
template <std::size_t D, class T> inline Vec<D, T>& normalize(Vec<D, T>& a) {
    T l = len(a);
    if (l > T(0)) a *= T(1) / l;
    return a;
}
template <std::size_t D, class T, class S> inline Vec<D, T> mix(const Vec<D, T>& a, const Vec<D, T>& b, S t) {
    Vec<D, T> r;
    for (std::size_t i = 0; i < D; ++i) r[i] = a[i] + (b[i] - a[i]) * T(t);
    return r;
}
template <class T> inline Vec<3, T> cross(const Vec<3, T>& a, const Vec<3, T>& b) {
    return Vec<3, T>(a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]);
}

template <std::size_t D, class T> inline std::ostream& operator<<(std::ostream& os, const Vec<D, T>& a) {
    os << "(";
    for (std::size_t i = 0; i < D; ++i) os << (i ? ", " : "") << a[i];
    return os << ")";
}

typedef Vec<3, float> vec;
typedef Vec<3, float> point;
typedef Vec<2, float> vec2;
typedef Vec<3, float> vec3;
typedef Vec<4, float> vec4;
typedef Vec<2, int> ivec2;
typedef Vec<3, int> ivec3;
typedef Vec<4, int> ivec4;

}  // namespace trimesh
