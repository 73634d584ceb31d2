// Dense volume stand-in: a non-owning view over an X*Y*Z uint8 occupancy
// array stored x-major (z fastest), answering getDataAt with the stored value.
// Test infrastructure only.
#pragma once
#include <cstdint>

class Volume {
    const std::uint8_t* d_;
    int sx_, sy_, sz_;

public:
    Volume(const std::uint8_t* d, int sx, int sy, int sz) : d_(d), sx_(sx), sy_(sy), sz_(sz) {}
    int getSizeX() const { return sx_; }
    int getSizeY() const { return sy_; }
    int getSizeZ() const { return sz_; }
    double getDataAt(int x, int y, int z) const {
        return double(d_[(static_cast<long long>(x) * sy_ + y) * sz_ + z]);
    }
};
