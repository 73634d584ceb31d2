// Drives the GPU path through the C++ adapters exactly the way
// exportInsideVoroMesh drives the reference (highlevelalgo.cpp:739-838):
// extractInsideWithMeasure -> cellcomplex -> CellComplexThinning::setup /
// assignElementValues / preprocess / prune(thresh, thresh) / remainingCC.
// Reads an occupancy volume (X Y Z then X*Y*Z bytes) and writes the surviving
// flags and the remaining complex sizes to stdout for the parity test.
#include <array>
#include <cstdio>
#include <fstream>
#include <iostream>
#include <vector>

#include "voxelcore_gb300.hpp"

int main(int argc, char** argv) {
    if (argc < 3) {
        std::cerr << "usage: adapter_main volume.bin t\n";
        return 2;
    }
    std::ifstream in(argv[1], std::ios::binary);
    int dims[3];
    in.read(reinterpret_cast<char*>(dims), sizeof(dims));
    std::vector<uint8_t> occ((size_t)dims[0] * dims[1] * dims[2]);
    in.read(reinterpret_cast<char*>(occ.data()), (std::streamsize)occ.size());
    const double t = std::atof(argv[2]);
    try {
        vcgpu::Context ctx(0);
        vcgpu::DenseVolume vol{occ.data(), dims[0], dims[1], dims[2]};
        std::vector<std::array<float, 3>> sites;
        vcgpu::Surfacer surf(ctx);
        if (surf.extractBoundaryVts(vol, sites) != vcgpu::SurfacerErrCode::SUCCESS) return 1;
        std::vector<std::array<float, 3>> vts;
        std::vector<std::array<int, 2>> edges;
        std::vector<std::array<int, 3>> tris;
        std::vector<int> from_fi;
        std::vector<float> vm, em, fm;
        const float inside = vcgpu::extractInsideWithMeasure(ctx, vol, vts, edges, tris, from_fi, vm, em, fm);
        std::vector<float> radii;
        vcgpu::getRadii(ctx, vts, radii);
        vcgpu::Context ctx2(0);
        vcgpu::cellcomplex cc(ctx2, vts, edges, tris);
        vcgpu::CellComplexThinning ccthin;
        ccthin.setup(&cc);
        ccthin.assignElementValues(vm, em, fm);
        ccthin.preprocess();
        const float thresh = (float)((double)inside * t);
        ccthin.prune(thresh, thresh, false);
        std::vector<int> rv, re, rf;
        ccthin.getRemainedVts(rv);
        ccthin.getRemainedEdges(re);
        ccthin.getRemainedFaces(rf);
        std::vector<std::array<float, 3>> ov;
        std::vector<std::array<int, 2>> oe;
        std::vector<std::array<int, 3>> ot;
        ccthin.remainingCC(ov, oe, ot);
        std::printf("sites %zu\nthresh %.9g\ncomplex %zu %zu %zu\n", sites.size(), thresh, vts.size(), cc.numEdges(),
                    tris.size());
        std::printf("remaining %zu %zu %zu\n", ov.size(), oe.size(), ot.size());
        std::printf("keep_v");
        for (int i : rv) std::printf(" %d", i);
        std::printf("\nkeep_e");
        for (int i : re) std::printf(" %d", i);
        std::printf("\nkeep_f");
        for (int i : rf) std::printf(" %d", i);
        std::printf("\nradius");
        for (float r : radii) std::printf(" %.9g", r);
        std::printf("\n");
    } catch (const vcgpu::Error& e) {
        std::cerr << e.what() << "\n";
        return 1;
    }
    return 0;
}
