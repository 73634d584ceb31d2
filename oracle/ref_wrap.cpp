// C entry points over the reference's own C++ sources (ccthin.cpp,
// cellcomplex.cpp, geomalgo.cpp, octree.cpp, spaceinfo.cpp, surfacing.cpp), compiled
// unmodified against the API shim in oracle/shim.  TEST INFRASTRUCTURE: only
// tests/ and the golden-fixture script load the resulting library
// (oracle/_ref/libvcref.so); the product never does.
//
// Pinned entry points of the reference that these wrappers drive:
//   Surfacer::extractBoundaryVts            src/surfacing.cpp:223-321
//   cellcomplex::cellcomplex / finalize     src/cellcomplex.cpp:13-26, 364-491
//   CellComplexThinning::prune              src/ccthin.cpp:201-424
//   CellComplexThinning::remainingCC        src/ccthin.cpp:467-512
//   util::computeEulerChar                  src/geomalgo.cpp:181-214
//   CellComplexThinning::remainingCC()      src/ccthin.cpp:426-464
//   OctreeVolume (build, .sof write/read)   src/octree.cpp:50-63, 259-357, 499-560, 864-930
//   OctreeVolume::getDataAt                 src/octree.cpp:233-256
//   Surfacer::extractBoundaryVts (octree)   src/surfacing.cpp:286-301, 666-685
//   cellcomplex::compute_conn_cmpnts        src/cellcomplex.cpp:73-147
#include <voxelcore/ccthin.h>
#include <voxelcore/cellcomplex.h>
#include <voxelcore/densevolume.h>
#include <voxelcore/geomalgo.h>
#include <voxelcore/octree.h>
#include <voxelcore/spaceinfo.h>
#include <voxelcore/surfacing.h>

#include <cstdint>
#include <cstring>
#include <iostream>
#include <memory>
#include <sstream>
#include <vector>

namespace {
// The reference prints progress to std::cout; keep the test output quiet.
struct QuietCout {
    std::streambuf* old;
    std::ostringstream sink;
    QuietCout() : old(std::cout.rdbuf(sink.rdbuf())) {}
    ~QuietCout() { std::cout.rdbuf(old); }
};

struct RefComplex {
    cellcomplex cc;
    CellComplexThinning thin;
    std::vector<point> rem_vts;
    std::vector<ivec2> rem_edges;
    std::vector<uTriFace> rem_tris;
    bool pruned = false;
};
}  // namespace

extern "C" {

// Boundary-corner sites of an X*Y*Z occupancy volume (x-major, z fastest),
// in the reference's first-encounter order.  Returns the number of sites;
// writes up to `cap` xyz triples into `out_xyz`.
long long vcref_extract_sites(const std::uint8_t* occ, int X, int Y, int Z, float* out_xyz, long long cap) {
    QuietCout q;
    auto vol = std::make_shared<Volume>(occ, X, Y, Z);
    std::shared_ptr<Volume3DScalar> dv = std::make_shared<DenseVolume>(vol);
    Surfacer surf;
    std::vector<point> sites;
    if (surf.extractBoundaryVts(dv, sites) != SurfacerErrCode::SUCCESS) return -1;
    long long n = static_cast<long long>(sites.size());
    for (long long i = 0; i < n && i < cap; ++i) {
        out_xyz[3 * i + 0] = sites[i][0];
        out_xyz[3 * i + 1] = sites[i][1];
        out_xyz[3 * i + 2] = sites[i][2];
    }
    return n;
}

// The reference's octree of an X*Y*Z occupancy volume written as a .sof
// file (OctreeVolume(const Volume3DScalar*) then writeToFile).  0 on success.
int vcref_sof_write(const std::uint8_t* occ, int X, int Y, int Z, const char* path) {
    QuietCout q;
    auto vol = std::make_shared<Volume>(occ, X, Y, Z);
    DenseVolume dv(vol);
    OctreeVolume oct(&dv);
    return oct.writeToFile(path) ? 0 : -1;
}

// The reference's reading of a .sof file: the occupancy of every voxel of
// its (R+1)^3 grid (SpaceConverter::get_occupancy_at_vox on the octree,
// x-major, z fastest).  Returns R+1; `out` may be null to get the size.
int vcref_sof_occupancy(const char* path, std::uint8_t* out) {
    QuietCout q;
    OctreeVolume oct(path);
    const int n = oct.getSizeX();
    if (out)
        for (int x = 0; x < n; ++x)
            for (int y = 0; y < n; ++y)
                for (int z = 0; z < n; ++z)
                    out[((long long)x * n + y) * n + z] =
                        (std::uint8_t)SpaceConverter::get_occupancy_at_vox(ivec3(x, y, z), &oct);
    return n;
}

// Surfacer::extractBoundaryVts on the octree read from a .sof file (its
// octree branch: the centres of the leaves with mixed corners, in tree
// order).  Returns the number of sites; writes up to `cap` xyz triples.
long long vcref_sof_sites(const char* path, float* out_xyz, long long cap) {
    QuietCout q;
    std::shared_ptr<Volume3DScalar> oct = std::make_shared<OctreeVolume>(path);
    Surfacer surf;
    std::vector<point> sites;
    if (surf.extractBoundaryVts(oct, sites) != SurfacerErrCode::SUCCESS) return -1;
    long long n = static_cast<long long>(sites.size());
    for (long long i = 0; i < n && i < cap; ++i)
        for (int k = 0; k < 3; ++k) out_xyz[3 * i + k] = sites[i][k];
    return n;
}

// Build and finalize a reference cellcomplex from (V float3, E int2, T int3).
void* vcref_cc_create(int nv, const float* vts, int ne, const int* edges, int nt, const int* tris) {
    QuietCout q;
    std::vector<point> V(nv);
    std::vector<ivec2> E(ne);
    std::vector<uTriFace> T(nt);
    for (int i = 0; i < nv; ++i) V[i] = point(vts[3 * i], vts[3 * i + 1], vts[3 * i + 2]);
    for (int i = 0; i < ne; ++i) E[i] = ivec2(edges[2 * i], edges[2 * i + 1]);
    for (int i = 0; i < nt; ++i)
        T[i] = uTriFace((unsigned)tris[3 * i], (unsigned)tris[3 * i + 1], (unsigned)tris[3 * i + 2]);
    auto* h = new RefComplex();
    h->cc = cellcomplex(V, E, T, true);
    h->thin.setup(&h->cc);
    return h;
}

void vcref_cc_destroy(void* h) { delete static_cast<RefComplex*>(h); }

int vcref_cc_num_edges(void* h) { return (int)static_cast<RefComplex*>(h)->cc.numEdges(); }

// Finalized edge list (E' x 2) and per-face edge ids (F x 3, triangles only).
void vcref_cc_get_edges(void* h, int* out) {
    auto& cc = static_cast<RefComplex*>(h)->cc;
    for (size_t i = 0; i < cc.numEdges(); ++i) {
        out[2 * i] = cc.getEdge(i)[0];
        out[2 * i + 1] = cc.getEdge(i)[1];
    }
}
void vcref_cc_get_face_edges(void* h, int* out) {
    auto& cc = static_cast<RefComplex*>(h)->cc;
    std::vector<int> fe;
    for (size_t f = 0; f < cc.numFaces(); ++f) {
        cc.getFaceERep((int)f, fe);
        for (int k = 0; k < 3; ++k) out[3 * f + k] = fe[k];
    }
}
// Adjacency lists as CSR: V->E (offsets nV+1, ids) and E->F (offsets nE+1, ids).
long long vcref_cc_adj_size(void* h, int which) {
    auto& cc = static_cast<RefComplex*>(h)->cc;
    long long s = 0;
    if (which == 0)
        for (size_t v = 0; v < cc.numVts(); ++v) s += cc.cntNbEdgesofVert((unsigned)v);
    else
        for (size_t e = 0; e < cc.numEdges(); ++e) s += cc.cntNbFacesofEdge((unsigned)e);
    return s;
}
void vcref_cc_get_adj(void* h, int which, int* offs, int* ids) {
    auto& cc = static_cast<RefComplex*>(h)->cc;
    size_t n = which == 0 ? cc.numVts() : cc.numEdges();
    int o = 0;
    for (size_t i = 0; i < n; ++i) {
        offs[i] = o;
        int c = which == 0 ? cc.cntNbEdgesofVert((unsigned)i) : cc.cntNbFacesofEdge((unsigned)i);
        for (int k = 0; k < c; ++k)
            ids[o++] = which == 0 ? cc.nbEdgeofVert((unsigned)i, k) : cc.nbFaceofEdge((unsigned)i, k);
    }
    offs[n] = o;
}

// Run the reference thinning (assignElementValues, preprocess, prune) and
// report the surviving-cell flags: keep_v[v] = vertex not removed,
// keep_e[e] = edge not removed AND referenced by no remaining face (the
// reference's getRemainedEdges), keep_f[f] = face not removed,
// removed_e[e] = the edge removal tag.
int vcref_thin(void* hv, const float* vm, const float* em, const float* fm, float f_t, float l_t,
               std::uint8_t* keep_v, std::uint8_t* keep_e, std::uint8_t* keep_f, std::uint8_t* removed_e) {
    QuietCout q;
    auto* h = static_cast<RefComplex*>(hv);
    auto& cc = h->cc;
    std::vector<float> V(vm, vm + cc.numVts()), E(em, em + cc.numEdges()), F(fm, fm + cc.numFaces());
    h->thin.assignElementValues(V, E, F);
    h->thin.preprocess();
    h->thin.prune(f_t, l_t, false);
    h->pruned = true;
    std::vector<int> ids;
    std::memset(keep_v, 0, cc.numVts());
    std::memset(keep_e, 0, cc.numEdges());
    std::memset(keep_f, 0, cc.numFaces());
    h->thin.getRemainedVts(ids);
    for (int i : ids) keep_v[i] = 1;
    h->thin.getRemainedEdges(ids);
    for (int i : ids) keep_e[i] = 1;
    h->thin.getRemainedFaces(ids);
    for (int i : ids) keep_f[i] = 1;
    const auto& re = h->thin.getEdgeRemovedTags();
    for (size_t i = 0; i < re.size(); ++i) removed_e[i] = re[i] ? 1 : 0;
    return 0;
}

// remainingCC(vts, edges, tris) after vcref_thin; sizes first, then copy.
void vcref_remaining_sizes(void* hv, int* nv, int* ne, int* nt) {
    QuietCout q;
    auto* h = static_cast<RefComplex*>(hv);
    h->thin.remainingCC(h->rem_vts, h->rem_edges, h->rem_tris, nullptr);
    *nv = (int)h->rem_vts.size();
    *ne = (int)h->rem_edges.size();
    *nt = (int)h->rem_tris.size();
}
void vcref_remaining_get(void* hv, float* vts, int* edges, int* tris) {
    auto* h = static_cast<RefComplex*>(hv);
    for (size_t i = 0; i < h->rem_vts.size(); ++i)
        for (int k = 0; k < 3; ++k) vts[3 * i + k] = h->rem_vts[i][k];
    for (size_t i = 0; i < h->rem_edges.size(); ++i)
        for (int k = 0; k < 2; ++k) edges[2 * i + k] = h->rem_edges[i][k];
    for (size_t i = 0; i < h->rem_tris.size(); ++i)
        for (int k = 0; k < 3; ++k) tris[3 * i + k] = (int)h->rem_tris[i][k];
}

// The steps of nClosedComponents (src/highlevelalgo.cpp:993-1020, a file
// not built here) with the reference's own classes: a fresh thinning with
// every measure 0 pruned at thresholds 1, its remaining complex, and that
// complex's face-connected components (0 when it has no face).
int vcref_closed_components(int nv, const float* vts, int ne, const int* edges, int nt, const int* tris) {
    QuietCout q;
    void* hv = vcref_cc_create(nv, vts, ne, edges, nt, tris);
    auto* h = static_cast<RefComplex*>(hv);
    std::vector<float> V(h->cc.numVts(), 0.0f), E(h->cc.numEdges(), 0.0f), F(h->cc.numFaces(), 0.0f);
    h->thin.assignElementValues(V, E, F);
    h->thin.preprocess();
    h->thin.prune(1.0f, 1.0f, false);
    cellcomplex rest = h->thin.remainingCC();
    const int n = rest.numFaces() == 0 ? 0 : rest.compute_conn_cmpnts();
    vcref_cc_destroy(hv);
    return n;
}

// util::computeEulerChar(vts, edges, tris): out = {V, E, F, C, euler}.
void vcref_euler(int nv, const float* vts, int ne, const int* edges, int nt, const int* tris, int* out) {
    QuietCout q;
    std::vector<point> V(nv);
    std::vector<ivec2> E(ne);
    std::vector<uTriFace> T(nt);
    for (int i = 0; i < nv; ++i) V[i] = point(vts[3 * i], vts[3 * i + 1], vts[3 * i + 2]);
    for (int i = 0; i < ne; ++i) E[i] = ivec2(edges[2 * i], edges[2 * i + 1]);
    for (int i = 0; i < nt; ++i)
        T[i] = uTriFace((unsigned)tris[3 * i], (unsigned)tris[3 * i + 1], (unsigned)tris[3 * i + 2]);
    eulerchar ec;
    util::computeEulerChar(V, E, T, ec);
    out[0] = ec.V; out[1] = ec.E; out[2] = ec.F; out[3] = ec.C; out[4] = ec.euler;
}

// util::simpleTriangulate of one polygon: writes (n-2) triangles.
int vcref_simple_triangulate(int n, const int* poly, int* out_tris) {
    std::vector<int> p(poly, poly + n);
    std::vector<uTriFace> t;
    util::simpleTriangulate(p, t);
    for (size_t i = 0; i < t.size(); ++i)
        for (int k = 0; k < 3; ++k) out_tris[3 * i + k] = (int)t[i][k];
    return (int)t.size();
}

}  // extern "C"
