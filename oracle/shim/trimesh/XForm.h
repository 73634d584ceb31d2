// 4x4 affine transform subset (identity, scale, translate, product, apply to
// a point, inverse, element access, printing) used by the reference sources
// compiled for the oracle.  Column major, as the reference's callers only
// ever use the identity (the .sog octree reader, which sets translations, is
// compiled but not driven).  Test infrastructure only.
#pragma once
#include <ostream>
#include "Vec.h"

namespace trimesh {

template <class T = double>
class XForm {
public:
    T m[16];
    XForm() { *this = identity(); }
    static XForm identity() {
        XForm x(0);
        x.m[0] = x.m[5] = x.m[10] = x.m[15] = T(1);
        return x;
    }
    static XForm scale(T s) { XForm x = identity(); x.m[0] = x.m[5] = x.m[10] = s; return x; }
    static XForm trans(T a, T b, T c) { XForm x = identity(); x.m[12] = a; x.m[13] = b; x.m[14] = c; return x; }
    template <class S> static XForm trans(const Vec<3, S>& v) { return trans(T(v[0]), T(v[1]), T(v[2])); }
    XForm operator*(const XForm& o) const {
        XForm r(0);
        for (int i = 0; i < 4; ++i)
            for (int j = 0; j < 4; ++j) {
                T s = T(0);
                for (int k = 0; k < 4; ++k) s += m[i + 4 * k] * o.m[k + 4 * j];
                r.m[i + 4 * j] = s;
            }
        return r;
    }
    static constexpr int size() { return 16; }
    T& operator[](int i) { return m[i]; }
    const T& operator[](int i) const { return m[i]; }
    template <class S> Vec<3, S> operator*(const Vec<3, S>& p) const {
        if (m[0] == T(1) && m[5] == T(1) && m[10] == T(1) && m[1] == T(0) && m[2] == T(0) && m[4] == T(0) &&
            m[6] == T(0) && m[8] == T(0) && m[9] == T(0) && m[12] == T(0) && m[13] == T(0) && m[14] == T(0))
            return p;  // identity: return the point bit-for-bit
        Vec<3, S> r;
        for (int i = 0; i < 3; ++i)
            r[i] = S(m[i] * p[0] + m[i + 4] * p[1] + m[i + 8] * p[2] + m[i + 12]);
        return r;
    }

private:
    explicit XForm(int) { for (int i = 0; i < 16; ++i) m[i] = T(0); }
};

// Inverse by Gauss-Jordan elimination with partial pivoting.
template <class T>
inline XForm<T> inv(const XForm<T>& x) {
    double a[4][8];
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j) {
            a[i][j] = x.m[i + 4 * j];
            a[i][j + 4] = i == j ? 1.0 : 0.0;
        }
    for (int c = 0; c < 4; ++c) {
        int p = c;
        for (int r = c + 1; r < 4; ++r)
            if (std::abs(a[r][c]) > std::abs(a[p][c])) p = r;
        for (int j = 0; j < 8; ++j) std::swap(a[c][j], a[p][j]);
        const double d = a[c][c];
        for (int j = 0; j < 8; ++j) a[c][j] /= d;
        for (int r = 0; r < 4; ++r)
            if (r != c) {
                const double f = a[r][c];
                for (int j = 0; j < 8; ++j) a[r][j] -= f * a[c][j];
            }
    }
    XForm<T> y;
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j) y.m[i + 4 * j] = T(a[i][j + 4]);
    return y;
}

template <class T>
inline std::ostream& operator<<(std::ostream& os, const XForm<T>& x) {
    for (int i = 0; i < 16; ++i) os << x.m[i] << (i == 15 ? "" : " ");
    return os;
}

typedef XForm<double> xform;  // trimesh2's xform holds doubles

}  // namespace trimesh
