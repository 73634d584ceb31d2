// Axis-aligned box subset used by the reference sources compiled for the
// oracle (accumulate points, size, centre, radius, clear).  Test
// infrastructure only.
#pragma once
#include "Vec.h"
#include <limits>

namespace trimesh {

template <std::size_t D, class T = float>
class Box {
public:
    Vec<D, T> min, max;
    bool valid;

    Box() { clear(); }
    void clear() {
        valid = false;
        for (std::size_t i = 0; i < D; ++i) {
            min[i] = std::numeric_limits<T>::max();
            max[i] = std::numeric_limits<T>::lowest();
        }
    }
    Box& operator+=(const Vec<D, T>& p) {
        for (std::size_t i = 0; i < D; ++i) {
            if (p[i] < min[i]) min[i] = p[i];
            if (p[i] > max[i]) max[i] = p[i];
        }
        valid = true;
        return *this;
    }
    Vec<D, T> center() const { Vec<D, T> c; for (std::size_t i = 0; i < D; ++i) c[i] = (min[i] + max[i]) / T(2); return c; }
    Vec<D, T> size() const { Vec<D, T> s; for (std::size_t i = 0; i < D; ++i) s[i] = max[i] - min[i]; return s; }
    T radius() const { return valid ? T(0.5) * len(size()) : T(0); }
};

typedef Box<3, float> box;
typedef Box<3, float> box3;

}  // namespace trimesh
