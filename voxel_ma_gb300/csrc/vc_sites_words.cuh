// Word-parallel boundary-corner site rule, written once for the device
// kernels (vc_sites.cu) and for a host check against the oracle
// (tests/cpp/sites_words_check.cpp).
//
// The reference sweeps voxels i -> j -> k and, for each face neighbour
// (-x,+x,-y,+y,-z,+z) whose occupancy differs, appends the four shared
// corners it has not seen before (src/surfacing.cpp:223-321).  A corner is
// therefore first met at the earliest voxel, in sweep order, of the 2x2x2
// block around it that is inside the box and differs from one of its three
// block neighbours.  Here 32 consecutive voxels of a z-row are one 32-bit
// word (bit t = voxel 32w + t), so that rule is evaluated for all of them at
// once with bitwise operations on the 27 z-shifted words of the voxel
// neighbourhood: for corner c, D[q] marks the block voxels q (in-box, and
// different from a block neighbour) and the corner is new at the voxel iff
// the voxel's own block position is the lowest marked one.
#pragma once

#include <cstdint>

#ifndef __CUDACC__
#define VC_HD
#else
#define VC_HD __host__ __device__
#endif

namespace vc {

// Corner c of a voxel as the lattice offset {0,1}^3 from the voxel's lowest
// corner, in the reference's corner numbering (surfacing.h:74-96).
VC_HD inline int sw_corner_off(int c, int axis) {
    // rows: {1,0,0},{1,1,0},{0,0,0},{0,1,0},{1,0,1},{1,1,1},{0,0,1},{0,1,1}
    const uint32_t x = 0x33u, y = 0xAAu, z = 0xF0u;  // bit c of each axis
    return (int)((((axis == 0) ? x : (axis == 1) ? y : z) >> c) & 1u);
}
// The four corners shared with face neighbour dd (-x,+x,-y,+y,-z,+z), in
// visiting order (surfacing.h:182-190), packed 4 bits per slot.
VC_HD inline int sw_shared(int dd, int s) {
    const uint32_t tab[6] = {0x6732u, 0x4510u, 0x0264u, 0x5731u, 0x1320u, 0x4675u};
    return (int)((tab[dd] >> (4 * s)) & 0xFu);
}

struct SiteWords {
    uint32_t S[27];   // occupancy of voxel k + (dx,dy,dz) at bit t, index (dx+1)*9+(dy+1)*3+(dz+1)
    uint32_t nw[8];   // bit t: corner c of voxel 32w+t is a new site there
    uint32_t valid;   // bit t: voxel 32w+t exists
};

// word(ii, jj, ww) returns the packed occupancy word ww of row (ii, jj)
// (0 outside the volume; bits past the row's end are 0).
template <class Word>
VC_HD inline void site_words(Word word, int i, int j, int w, int X, int Y, int Z, SiteWords& r) {
    const int k0 = 32 * w;
    const int nz = Z - k0;  // voxels of this word that exist (>= 1)
    r.valid = nz >= 32 ? 0xFFFFFFFFu : ((1u << nz) - 1u);
    // z in-box masks of the shifted words: k-1 >= 0 and k+1 <= Z-1
    const uint32_t zlo = w == 0 ? 0xFFFFFFFEu : 0xFFFFFFFFu;
    const uint32_t zhi = (nz - 1) >= 32 ? 0xFFFFFFFFu : (((nz - 1) <= 0) ? 0u : ((1u << (nz - 1)) - 1u));
    uint32_t M[27];
    for (int dx = -1; dx <= 1; ++dx)
        for (int dy = -1; dy <= 1; ++dy) {
            const int ii = i + dx, jj = j + dy;
            const bool rin = ii >= 0 && ii < X && jj >= 0 && jj < Y;
            uint32_t wm = 0, w0 = 0, wp = 0;
            if (rin) {
                wm = w > 0 ? word(ii, jj, w - 1) : 0u;
                w0 = word(ii, jj, w);
                wp = nz > 32 ? word(ii, jj, w + 1) : 0u;
            }
            const int b = (dx + 1) * 9 + (dy + 1) * 3;
            r.S[b + 0] = (w0 << 1) | (wm >> 31);
            r.S[b + 1] = w0;
            r.S[b + 2] = (w0 >> 1) | (wp << 31);
            const uint32_t rm = rin ? 0xFFFFFFFFu : 0u;
            M[b + 0] = rm & zlo;
            M[b + 1] = rm;
            M[b + 2] = rm & zhi;
        }
    for (int c = 0; c < 8; ++c) {
        const int ox = sw_corner_off(c, 0), oy = sw_corner_off(c, 1), oz = sw_corner_off(c, 2);
        uint32_t P[8], Mq[8];
        for (int q = 0; q < 8; ++q) {
            const int n = (ox + (q >> 2)) * 9 + (oy + ((q >> 1) & 1)) * 3 + (oz + (q & 1));
            P[q] = r.S[n];
            Mq[q] = M[n];
        }
        const int own = ((1 - ox) << 2) | ((1 - oy) << 1) | (1 - oz);
        uint32_t lower = 0, mine = 0;
        for (int q = 0; q < 8; ++q) {
            const uint32_t D = Mq[q] & ((P[q] ^ P[q ^ 4]) | (P[q] ^ P[q ^ 2]) | (P[q] ^ P[q ^ 1]));
            if (q < own) lower |= D;
            if (q == own) mine = D;
        }
        r.nw[c] = mine & ~lower & r.valid;
    }
}

VC_HD inline int site_word_count(const SiteWords& r) {
    int n = 0;
    for (int c = 0; c < 8; ++c) {
#ifdef __CUDA_ARCH__
        n += __popc(r.nw[c]);
#else
        n += __builtin_popcount(r.nw[c]);
#endif
    }
    return n;
}

// The sites of the word's voxels, in the reference's order, numbered from
// `first`: emit(index, a, b, c) with (a, b, c) the corner's lattice point.
template <class Emit>
VC_HD inline void site_word_emit(const SiteWords& r, int i, int j, int w, int64_t first, Emit emit) {
    uint32_t any = 0;
    for (int c = 0; c < 8; ++c) any |= r.nw[c];
    int64_t o = first;
    while (any) {
#ifdef __CUDA_ARCH__
        const int t = __ffs(any) - 1;
#else
        const int t = __builtin_ctz(any);
#endif
        any &= any - 1u;
        const uint32_t bit = 1u << t;
        const uint32_t cur = r.S[13] & bit;
        // face neighbours in sweep order: -x, +x, -y, +y, -z, +z
        const int nbi[6] = {4, 22, 10, 16, 12, 14};
        uint32_t done = 0;
        for (int dd = 0; dd < 6; ++dd) {
            if ((r.S[nbi[dd]] & bit) == cur) continue;
            for (int s = 0; s < 4; ++s) {
                const int c = sw_shared(dd, s);
                if (!(r.nw[c] & bit) || (done & (1u << c))) continue;
                done |= 1u << c;
                emit(o++, i + sw_corner_off(c, 0), j + sw_corner_off(c, 1), 32 * w + t + sw_corner_off(c, 2));
            }
        }
    }
}

}  // namespace vc
