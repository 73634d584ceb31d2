// 4x4 affine transform subset (identity, scale, translate, product, apply to
// a point) used by the reference sources compiled for the oracle.  Column
// major, as the reference's callers only ever use the identity.  Test
// infrastructure only.
#pragma once
#include "Vec.h"

namespace trimesh {

template <class T = float>
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

typedef XForm<float> xform;

}  // namespace trimesh
