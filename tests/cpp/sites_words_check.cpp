// Host run of the word-parallel site rule (voxel_ma_gb300/csrc/
// vc_sites_words.cuh, the same source the device kernels run): reads a
// uint8 volume (X, Y, Z, then X*Y*Z bytes) and writes the sites in order as
// int32 lattice points (a, b, c), so the caller can compare them with the
// oracle.  Usage: sites_words_check in.bin out.bin
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "../../voxel_ma_gb300/csrc/vc_sites_words.cuh"

int main(int argc, char** argv) {
    if (argc < 3) return 2;
    FILE* f = std::fopen(argv[1], "rb");
    if (!f) return 2;
    int32_t d[3];
    if (std::fread(d, 4, 3, f) != 3) return 2;
    const int X = d[0], Y = d[1], Z = d[2];
    std::vector<uint8_t> occ((size_t)X * Y * Z);
    if (std::fread(occ.data(), 1, occ.size(), f) != occ.size()) return 2;
    std::fclose(f);
    const int Wz = (Z + 31) / 32;
    std::vector<uint32_t> bits((size_t)X * Y * Wz, 0u);
    for (int i = 0; i < X; ++i)
        for (int j = 0; j < Y; ++j)
            for (int k = 0; k < Z; ++k)
                if (occ[((size_t)i * Y + j) * Z + k] > 0) bits[((size_t)i * Y + j) * Wz + k / 32] |= 1u << (k % 32);
    auto word = [&](int ii, int jj, int ww) { return bits[((size_t)ii * Y + jj) * Wz + ww]; };
    std::vector<int64_t> first((size_t)X * Y * Wz + 1, 0);
    vc::SiteWords r;
    for (int i = 0; i < X; ++i)
        for (int j = 0; j < Y; ++j)
            for (int w = 0; w < Wz; ++w) {
                const size_t id = ((size_t)i * Y + j) * Wz + w;
                vc::site_words(word, i, j, w, X, Y, Z, r);
                first[id + 1] = first[id] + vc::site_word_count(r);
            }
    const int64_t n = first.back();
    std::vector<int32_t> out((size_t)n * 3, -1);
    for (int i = 0; i < X; ++i)
        for (int j = 0; j < Y; ++j)
            for (int w = 0; w < Wz; ++w) {
                const size_t id = ((size_t)i * Y + j) * Wz + w;
                vc::site_words(word, i, j, w, X, Y, Z, r);
                vc::site_word_emit(r, i, j, w, first[id], [&](int64_t o, int a, int b, int c) {
                    out[3 * o] = a;
                    out[3 * o + 1] = b;
                    out[3 * o + 2] = c;
                });
            }
    f = std::fopen(argv[2], "wb");
    if (!f) return 2;
    std::fwrite(&n, 8, 1, f);
    std::fwrite(out.data(), 4, out.size(), f);
    std::fclose(f);
    return 0;
}
