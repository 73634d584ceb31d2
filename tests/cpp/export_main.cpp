// Host-only driver of the C++ output-format adapters: reads a complex from a
// binary file (nv ne nt, then float vts, float radii, int edges, int tris)
// and writes it with vcgpu::writeToPLY / vcgpu::writeToDotma to <prefix>.ply
// and <prefix>.ma; and writes a dense volume's octree with
// vcgpu::writeOctreeFile to <prefix>.sof / <prefix>.sog.
#include <cstdio>
#include <fstream>
#include <vector>

#include "voxelcore_gb300.hpp"

struct P3 {
    float v[3];
    float operator[](int k) const { return v[k]; }
};
struct I2 {
    int v[2];
    int operator[](int k) const { return v[k]; }
};
struct I3 {
    int v[3];
    int operator[](int k) const { return v[k]; }
};

int main(int argc, char** argv) {
    if (argc != 3) {
        std::fprintf(stderr, "usage: export_main complex.bin prefix\n");
        return 2;
    }
    std::ifstream f(argv[1], std::ios::binary);
    int64_t n[3];
    f.read(reinterpret_cast<char*>(n), sizeof n);
    std::vector<P3> vts((size_t)n[0]);
    std::vector<float> radii((size_t)n[0]);
    std::vector<I2> edges((size_t)n[1]);
    std::vector<I3> tris((size_t)n[2]);
    f.read(reinterpret_cast<char*>(vts.data()), (std::streamsize)(vts.size() * sizeof(P3)));
    f.read(reinterpret_cast<char*>(radii.data()), (std::streamsize)(radii.size() * sizeof(float)));
    f.read(reinterpret_cast<char*>(edges.data()), (std::streamsize)(edges.size() * sizeof(I2)));
    f.read(reinterpret_cast<char*>(tris.data()), (std::streamsize)(tris.size() * sizeof(I3)));
    const std::string prefix = argv[2];
    if (vcgpu::writeToPLY((prefix + ".ply").c_str(), vts, edges, tris) != vcgpu::ExportErrCode::SUCCESS) return 1;
    if (vcgpu::writeToDotma(prefix + ".ma", vts, edges, tris, radii) != vcgpu::ExportErrCode::SUCCESS) return 1;
    // a small dense volume: a 9 x 7 x 5 box with a hole
    std::vector<uint8_t> occ(9 * 7 * 5, 1);
    occ[(4 * 7 + 3) * 5 + 2] = 0;
    const vcgpu::DenseVolume vol{occ.data(), 9, 7, 5};
    if (!vcgpu::writeOctreeFile(vol, prefix + ".sof") || !vcgpu::writeOctreeFile(vol, prefix + ".sog")) return 1;
    return 0;
}
