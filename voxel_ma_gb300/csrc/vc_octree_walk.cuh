// One subtree of a .sof / .sog node stream, walked in pre-order (the order
// of the reference's read_sof_file / read_sog_file, src/octree.cpp:259-498): internal nodes (type
// 0) have eight children, x outermost and z innermost; an empty node (type 1)
// sets every cell of its cube to 0xff (sign byte 1) or 0x00 (any other
// sign); a leaf (type 2, one cell) sets its corner byte.  The same code runs
// on the host and in the decode kernel (one thread per subtree).
#pragma once

#include <cstdint>

#ifdef __CUDACC__
#define VC_HD __host__ __device__
#else
#define VC_HD
#endif

namespace vc {

// A node in 8 bytes: x, y, z (15 bits each), log2 of its edge length (4 bits)
// and a corner byte.
VC_HD inline uint64_t oct_pack(int x, int y, int z, int lg, uint8_t v) {
    return (uint64_t)x | ((uint64_t)y << 15) | ((uint64_t)z << 30) | ((uint64_t)lg << 45) | ((uint64_t)v << 49);
}
VC_HD inline int oct_x(uint64_t p) { return (int)(p & 0x7fff); }
VC_HD inline int oct_y(uint64_t p) { return (int)((p >> 15) & 0x7fff); }
VC_HD inline int oct_z(uint64_t p) { return (int)((p >> 30) & 0x7fff); }
VC_HD inline int oct_lg(uint64_t p) { return (int)((p >> 45) & 15); }
VC_HD inline uint8_t oct_v(uint64_t p) { return (uint8_t)(p >> 49); }

// Subtrees the walker takes have edge length <= 16 (lg <= 4): a terminal
// node is at most 16^3 cells, written row by row.
constexpr int kOctSubLg = 4;

// Cube of edge 1 << lg at (x, y, z) set to v.  x, y, z are multiples of the
// edge and R is a multiple of it, so every row starts on an edge-aligned byte.
VC_HD inline void oct_fill(uint8_t* cell, int R, int x, int y, int z, int lg, uint8_t v) {
    const int len = 1 << lg;
    const uint64_t v8 = 0x0101010101010101ull * v;
    for (int a = 0; a < len; ++a)
        for (int b = 0; b < len; ++b) {
            uint8_t* row = cell + ((int64_t)(x + a) * R + (y + b)) * R + z;
            switch (lg) {
                case 0: *row = v; break;
                case 1: *reinterpret_cast<uint16_t*>(row) = (uint16_t)v8; break;
                case 2: *reinterpret_cast<uint32_t*>(row) = (uint32_t)v8; break;
                case 3: *reinterpret_cast<uint64_t*>(row) = v8; break;
                default:
                    reinterpret_cast<uint64_t*>(row)[0] = v8;
                    reinterpret_cast<uint64_t*>(row)[1] = v8;
                    break;
            }
        }
}

// Walk the subtree whose first token is at byte pos and whose root is the
// packed node root (corner byte unused).  LEAF_EXTRA: bytes after a leaf's
// corner byte (0 in .sof; 12 in .sog, the three floats of its feature point,
// src/octree.cpp:403-410).  FILL: write the cells and count
// the mixed leaves (corner byte neither 0x00 nor 0xff) into *nmixed.
// !FILL: write the mixed leaves, packed, to out[0 .. *nmixed).  Returns 0, or
// 1 for a stream that is not a valid subtree (a read past nbytes, an unknown
// type, an internal node of one cell, a leaf or empty node too large for the
// walker).
template <bool FILL, int LEAF_EXTRA = 0>
VC_HD inline int oct_walk(const uint8_t* b, int64_t nbytes, int64_t pos, uint64_t root, uint8_t* cell, int R,
                          uint64_t* out, int64_t* nmixed) {
    struct Frame {
        int x, y, z, lg, child;
    };
    Frame st[kOctSubLg + 1];
    int sp = 0;
    int64_t n = 0;
    int x = oct_x(root), y = oct_y(root), z = oct_z(root), lg = oct_lg(root);
    if (lg > kOctSubLg) return 1;
    for (;;) {
        // visit node (x, y, z, lg)
        if (pos >= nbytes) return 1;
        const uint8_t type = b[pos++];
        if (type == 0) {
            if (lg == 0) return 1;
            st[sp++] = Frame{x, y, z, lg, 0};
        } else if (type == 1 || type == 2) {
            if (pos >= nbytes) return 1;
            const uint8_t raw = b[pos++];
            uint8_t v;
            if (type == 2) {
                if (lg != 0) return 1;
                if (LEAF_EXTRA) {
                    if (nbytes - pos < LEAF_EXTRA) return 1;
                    pos += LEAF_EXTRA;
                }
                v = raw;
                if (v != 0x00 && v != 0xff) {
                    if (!FILL) out[n] = oct_pack(x, y, z, 0, 0);
                    ++n;
                }
            } else {
                v = raw == 1 ? 0xff : 0x00;
            }
            if (FILL) oct_fill(cell, R, x, y, z, lg, v);
        } else {
            return 1;
        }
        // next node: the next child of the innermost unfinished frame
        while (sp > 0 && st[sp - 1].child == 8) --sp;
        if (sp == 0) break;
        Frame& f = st[sp - 1];
        const int h = 1 << (f.lg - 1), ch = f.child++;
        x = f.x + (ch >> 2) * h;
        y = f.y + ((ch >> 1) & 1) * h;
        z = f.z + (ch & 1) * h;
        lg = f.lg - 1;
    }
    if (FILL) *nmixed = n;
    return 0;
}

}  // namespace vc
