// A caller written against the reference's classes, exactly as
// exportInsideVoroMesh (src/highlevelalgo.cpp:739-838) and nClosedComponents
// (:993-1020) call them -- no GPU context appears anywhere: the adapters of
// voxelcore_gb300.hpp create their own.  Only the namespace differs.
//
// Reads an occupancy volume (X Y Z then X*Y*Z bytes) behind a
// Volume3DScalar-like class, and prints the sites, the threshold, the
// surviving cells, the remaining complex (both remainingCC forms, with
// from_fi) and the closed components for the parity test.
#include <array>
#include <cstdio>
#include <fstream>
#include <iostream>
#include <memory>
#include <vector>

#include "voxelcore_gb300.hpp"

using namespace vcgpu;
using point = std::array<float, 3>;
using ivec2 = std::array<int, 2>;
using uTriFace = std::array<int, 3>;

// the reference's abstract volume: getDataAt + sizes (include/Volume3DScalar.h)
class Volume3DScalar {
public:
    virtual ~Volume3DScalar() = default;
    virtual double getDataAt(int x, int y, int z) const = 0;
    int getSizeX() const { return n_[0]; }
    int getSizeY() const { return n_[1]; }
    int getSizeZ() const { return n_[2]; }

protected:
    int n_[3] = {0, 0, 0};
};
class BytesVolume : public Volume3DScalar {
public:
    BytesVolume(std::vector<uint8_t> v, int X, int Y, int Z) : v_(std::move(v)) {
        n_[0] = X;
        n_[1] = Y;
        n_[2] = Z;
    }
    double getDataAt(int x, int y, int z) const override {
        if (x < 0 || y < 0 || z < 0 || x >= n_[0] || y >= n_[1] || z >= n_[2]) return 0.0;
        return v_[((size_t)x * n_[1] + y) * n_[2] + z];
    }

private:
    std::vector<uint8_t> v_;
};

static int fail(const char* what) {
    std::cerr << "failed: " << what << "\n";
    return 1;
}

int main(int argc, char** argv) {
    if (argc < 3) {
        std::cerr << "usage: dropin_main volume.bin t [same-volume.mrc]\n";
        return 2;
    }
    std::ifstream in(argv[1], std::ios::binary);
    int dims[3];
    in.read(reinterpret_cast<char*>(dims), sizeof(dims));
    std::vector<uint8_t> bytes((size_t)dims[0] * dims[1] * dims[2]);
    in.read(reinterpret_cast<char*>(bytes.data()), (std::streamsize)bytes.size());
    const double t = std::atof(argv[2]);
    std::shared_ptr<Volume3DScalar> vol = std::make_shared<BytesVolume>(bytes, dims[0], dims[1], dims[2]);
    try {
        // sites (Surfacer::extractBoundaryVts)
        Surfacer surf;
        std::vector<point> sites;
        if (surf.extractBoundaryVts(vol, sites) != SurfacerErrCode::SUCCESS) return fail("extractBoundaryVts");
        std::shared_ptr<Volume3DScalar> empty;
        std::vector<point> none_sites;
        if (surf.extractBoundaryVts(empty, none_sites) != SurfacerErrCode::EMPTY_VOL) return fail("EMPTY_VOL");
        // the inside part with measures (VoroInfo::extractInsideWithMeasure)
        VoroInfo voro(vol);
        std::vector<point> vts;
        std::vector<ivec2> edges;
        std::vector<uTriFace> tri_faces;
        std::vector<int> from_fi;
        std::vector<float> vts_msure, edges_msure, all_tri_msure;
        voro.extractInsideWithMeasure(MeasureForMA::LAMBDA, vts, edges, tri_faces, from_fi, vts_msure, edges_msure,
                                      all_tri_msure);
        const std::vector<float>& radii = voro.getRadii();
        // thinning (CellComplexThinning on a cellcomplex)
        CellComplexThinning ccthin;
        cellcomplex cc(vts, edges, tri_faces);
        ccthin.setup(&cc);
        ccthin.assignElementValues(vts_msure, edges_msure, all_tri_msure);
        ccthin.preprocess();
        const float thresh = voro.getInsidePartSize() * t;
        ccthin.prune(thresh, thresh, false);
        std::vector<point> rv;
        std::vector<ivec2> re;
        std::vector<uTriFace> rt;
        std::vector<int> rfrom;
        ccthin.remainingCC(rv, re, rt, &rfrom);
        cellcomplex rem = ccthin.remainingCC();
        std::vector<int> kv, ke, kf;
        ccthin.getRemainedVts(kv);
        ccthin.getRemainedEdges(ke);
        ccthin.getRemainedFaces(kf);
        // the closed pockets of the full complex (nClosedComponents)
        const int closed = nClosedComponents(cc);
        std::printf("sites %zu\nthresh %.9g\ncomplex %zu %zu %zu\n", sites.size(), thresh, vts.size(),
                    cc.numEdges(), tri_faces.size());
        std::printf("remaining %zu %zu %zu\n", rv.size(), re.size(), rt.size());
        std::printf("remaining_cc %zu %zu %zu\n", rem.numVts(), rem.numEdges(), rem.numFaces());
        std::printf("closed %d\n", closed);
        std::printf("radii %zu\n", radii.size());
        if (argc > 3) {
            // the same volume as a file, through readVolume (importers.h)
            std::shared_ptr<GpuVolume> fv;
            if (readVolume(argv[3], fv) != ImportErrCode::SUCCESS) return fail("readVolume");
            std::vector<point> fsites;
            if (surf.extractBoundaryVts(fv, fsites) != SurfacerErrCode::SUCCESS) return fail("extractBoundaryVts(file)");
            VoroInfo fvoro(fv);
            std::printf("file_sites %zu\nfile_complex %lld %lld %lld\n", fsites.size(), (long long)fvoro.sizes().nv,
                        (long long)fvoro.sizes().ne, (long long)fvoro.sizes().nt);
            std::shared_ptr<GpuVolume> none;
            if (readVolume("no_such_file.mrc", none) != ImportErrCode::NOOPENINPUT) return fail("NOOPENINPUT");
        }
        std::printf("keep_f");
        for (int i : kf) std::printf(" %d", i);
        std::printf("\nfrom_fi");
        for (int i : rfrom) std::printf(" %d", i);
        std::printf("\nrem_tris");
        for (const auto& f : rt) std::printf(" %d %d %d", f[0], f[1], f[2]);
        std::printf("\nrem_edges");
        for (const auto& e : re) std::printf(" %d %d", e[0], e[1]);
        std::printf("\n");
    } catch (const Error& e) {
        std::cerr << "vcgpu::Error: " << e.what() << "\n";
        return 1;
    }
    return 0;
}
