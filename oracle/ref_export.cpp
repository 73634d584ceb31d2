// Reference-side output formats for the parity tests.  TEST INFRASTRUCTURE:
// only tests/ load the library this is part of (oracle/_ref/libvcref.so).
//
//   writeToDotma          src/exporters.cpp:244-287, the reference's own
//                         function: the Makefile cuts it out of exporters.cpp
//                         into _ref/dotma.inc (the file's other writers need
//                         the absent trimesh2, ply, tetgen and isosurface
//                         libraries, so the whole file does not compile here).
//   .ma edge assembly     src/highlevelalgo.cpp:925-937, on the reference's own
//                         ivec2, ivec2Hash (include/commondefs.h:30-43) and
//                         util::makeEdgesFromTri (include/geomalgo.h:85-91).
#include <voxelcore/commondefs.h>
#include <voxelcore/geomalgo.h>

#include <cstdint>
#include <fstream>
#include <limits>
#include <string>
#include <unordered_set>
#include <vector>

namespace voxelvoro {
// include/exporters.h:15-23 (that header includes an absent library)
enum class ExportErrCode { FAILURE, SUCCESS, INPUT_NOT_OPEN, OUTPUT_NOT_OPEN, INPUT_NOT_SUPPORTED, OUTPUT_NOT_SUPPORTED };
using std::ofstream;
using std::string;
using std::vector;
#include "_ref/dotma.inc"
}  // namespace voxelvoro

extern "C" int vcref_write_dotma(const char* path, const float* vts, const float* radii, long long nv,
                                 const int32_t* edges, long long ne, const int32_t* tris, long long nt) {
    std::vector<point> v;
    std::vector<ivec2> e;
    std::vector<uTriFace> t;
    for (long long k = 0; k < nv; ++k) v.push_back(point(vts[3 * k], vts[3 * k + 1], vts[3 * k + 2]));
    for (long long k = 0; k < ne; ++k) e.push_back(ivec2(edges[2 * k], edges[2 * k + 1]));
    for (long long k = 0; k < nt; ++k) t.push_back(uTriFace(tris[3 * k], tris[3 * k + 1], tris[3 * k + 2]));
    std::vector<float> r(radii, radii + nv);
    return voxelvoro::writeToDotma(std::string(path), v, e, t, r) == voxelvoro::ExportErrCode::SUCCESS ? 0 : 1;
}

extern "C" long long vcref_dotma_edges(const int32_t* edges, long long ne, const int32_t* tris, long long nt,
                                       int32_t* out) {
    std::vector<ivec2> all;
    for (long long k = 0; k < ne; ++k) all.push_back(ivec2(edges[2 * k], edges[2 * k + 1]));
    std::unordered_set<ivec2, ivec2Hash> unique_edges;
    ivec2 es_f[3];
    for (long long k = 0; k < nt; ++k) {
        const uTriFace f(tris[3 * k], tris[3 * k + 1], tris[3 * k + 2]);
        util::makeEdgesFromTri(f, es_f);
        unique_edges.insert(es_f[0]);
        unique_edges.insert(es_f[1]);
        unique_edges.insert(es_f[2]);
    }
    all.insert(all.end(), unique_edges.begin(), unique_edges.end());
    if (out)
        for (size_t k = 0; k < all.size(); ++k) {
            out[2 * k] = all[k][0];
            out[2 * k + 1] = all[k][1];
        }
    return (long long)all.size();
}
