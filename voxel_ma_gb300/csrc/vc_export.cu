// Output formats of the remaining complex: the files the reference's pipeline
// writes after thinning at one threshold (src/highlevelalgo.cpp:855-955).
//
//   .ply  writeToPLY (src/exporters.cpp:341-476) through ply::PLYWriter::write
//         (src/plyall.cpp:98-171): an ASCII PLY file with the elements vertex
//         (x, y, z), edge (vertex1, vertex2) and face (vertex_indices); the
//         measure and site properties the caller prepares are never described
//         to the writer, so they are not in the file.  The text is that of the
//         ply library's ASCII writer (Greg Turk's ply.c, 1998 revision): the
//         header lines, then one line per element, each value followed by a
//         space ("%g" for floats, "%d" / "%u" for integers).
//   .r    writeRadiiToFile with the remaining vertex ids
//         (src/exporters.cpp:478-552): the count, then "x y z r" per vertex.
//   .ma   writeToDotma (src/exporters.cpp:244-287) with the caller's edge
//         list (src/highlevelalgo.cpp:911-945): "nv ne nf", "v x y z r",
//         "e a b", "f a b c"; the edges are the remaining edges followed by
//         the edges of the remaining triangles, in the order the caller's
//         unordered_set<ivec2, ivec2Hash> holds them (a fresh set, as on the
//         first threshold of a run).
//
// Floats are written as std::ostream writes them by default (the "%g" rule,
// 6 significant digits).  The volumes have the identity voxel-to-model
// matrix, so a radius is written as len((r, 0, 0)) = sqrt(r * r) in float.
#include "vc_internal.cuh"

#include <charconv>
#include <cmath>
#include <cstdio>
#include <string>
#include <unordered_set>

namespace vc {
namespace {

struct Text {
    std::string s;
    void g(double v) {  // "%g": 6 significant digits, shortest of %e / %f
        char buf[32];
        const auto r = std::to_chars(buf, buf + sizeof buf, v, std::chars_format::general, 6);
        s.append(buf, r.ptr);
    }
    void i(int64_t v) {
        char buf[24];
        const auto r = std::to_chars(buf, buf + sizeof buf, v);
        s.append(buf, r.ptr);
    }
    void c(char ch) { s.push_back(ch); }
    void str(const char* t) { s.append(t); }
};

int write_file(const char* path, const std::string& s) {
    FILE* f = std::fopen(path, "wb");
    if (!f) return VC_ERR_ARG;
    const size_t n = std::fwrite(s.data(), 1, s.size(), f);
    const int rc = std::fclose(f);
    return (n == s.size() && rc == 0) ? VC_OK : VC_ERR_ARG;
}

// ivec2Hash (include/commondefs.h:30-43): h = h * 31 + std::hash<int>(x),
// over the two ids; std::hash<int> is the value itself
struct EdgeHash {
    size_t operator()(uint64_t e) const {
        size_t h = 0;
        h = (h << 5) - h + (size_t)(int64_t)(int32_t)(uint32_t)(e >> 32);
        h = (h << 5) - h + (size_t)(int64_t)(int32_t)(uint32_t)e;
        return h;
    }
};
inline uint64_t edge_key(int a, int b) {  // util::makeEdge: (min, max)
    if (a > b) std::swap(a, b);
    return ((uint64_t)(uint32_t)a << 32) | (uint32_t)b;
}

}  // namespace

int format_ply(const float* vts, int64_t nv, const int32_t* edges, int64_t ne, const int32_t* tris, int64_t nt,
               std::string& out) {
    Text t;
    t.s.reserve((size_t)(nv * 30 + ne * 16 + nt * 24 + 256));
    t.str("ply\nformat ascii 1.0\ncomment Generated by VoxelCore\nelement vertex ");
    t.i(nv);
    t.str("\nproperty float32 x\nproperty float32 y\nproperty float32 z\nelement edge ");
    t.i(ne);
    t.str("\nproperty int32 vertex1\nproperty int32 vertex2\nelement face ");
    t.i(nt);
    t.str("\nproperty list uint8 int32 vertex_indices\nend_header\n");
    for (int64_t k = 0; k < nv; ++k) {
        for (int d = 0; d < 3; ++d) {
            t.g(vts[3 * k + d]);
            t.c(' ');
        }
        t.c('\n');
    }
    for (int64_t k = 0; k < ne; ++k) {
        t.i(edges[2 * k]);
        t.c(' ');
        t.i(edges[2 * k + 1]);
        t.str(" \n");
    }
    for (int64_t k = 0; k < nt; ++k) {
        t.str("3 ");
        for (int d = 0; d < 3; ++d) {
            t.i(tris[3 * k + d]);
            t.c(' ');
        }
        t.c('\n');
    }
    out.swap(t.s);
    return VC_OK;
}

int format_radii(const float* vts, const float* radii, int64_t n, std::string& out) {
    Text t;
    t.s.reserve((size_t)(n * 40 + 32));
    t.i(n);
    t.c('\n');
    for (int64_t k = 0; k < n; ++k) {
        const float r = radii[k];
        for (int d = 0; d < 3; ++d) {
            t.g(vts[3 * k + d]);
            t.c(' ');
        }
        t.g(std::sqrt(r * r));
        t.c('\n');
    }
    out.swap(t.s);
    return VC_OK;
}

int format_dotma(const float* vts, const float* radii, int64_t nv, const int32_t* edges, int64_t ne,
                 const int32_t* tris, int64_t nt, std::string& out) {
    Text t;
    t.s.reserve((size_t)(nv * 40 + ne * 16 + nt * 24 + 64));
    t.i(nv);
    t.c(' ');
    t.i(ne);
    t.c(' ');
    t.i(nt);
    t.c('\n');
    for (int64_t k = 0; k < nv; ++k) {
        t.str("v ");
        for (int d = 0; d < 3; ++d) {
            t.g(vts[3 * k + d]);
            t.c(' ');
        }
        t.g(radii[k]);
        t.c('\n');
    }
    for (int64_t k = 0; k < ne; ++k) {
        t.str("e ");
        t.i(edges[2 * k]);
        t.c(' ');
        t.i(edges[2 * k + 1]);
        t.c('\n');
    }
    for (int64_t k = 0; k < nt; ++k) {
        t.str("f ");
        t.i((uint32_t)tris[3 * k]);
        t.c(' ');
        t.i((uint32_t)tris[3 * k + 1]);
        t.c(' ');
        t.i((uint32_t)tris[3 * k + 2]);
        t.c('\n');
    }
    out.swap(t.s);
    return VC_OK;
}

// the caller's .ma edge list: remaining edges, then the triangles' edges in
// the iteration order of a fresh unordered_set filled triangle by triangle
void dotma_edges(const int32_t* edges, int64_t ne, const int32_t* tris, int64_t nt, std::vector<int32_t>& out) {
    out.assign(edges, edges + 2 * ne);
    std::unordered_set<uint64_t, EdgeHash> unique;
    for (int64_t k = 0; k < nt; ++k)
        for (int d = 0; d < 3; ++d) unique.insert(edge_key(tris[3 * k + d], tris[3 * k + (d + 1) % 3]));
    for (const uint64_t e : unique) {
        out.push_back((int32_t)(e >> 32));
        out.push_back((int32_t)(uint32_t)e);
    }
}

}  // namespace vc

extern "C" int vc_write_ply(const char* path, const float* vts, int64_t nv, const int32_t* edges, int64_t ne,
                            const int32_t* tris, int64_t nt) {
    if (!path || nv < 0 || ne < 0 || nt < 0 || (nv && !vts) || (ne && !edges) || (nt && !tris)) return VC_ERR_ARG;
    std::string s;
    VC_TRY(vc::format_ply(vts, nv, edges, ne, tris, nt, s));
    return vc::write_file(path, s);
}

extern "C" int vc_write_radii(const char* path, const float* vts, const float* radii, int64_t n) {
    if (!path || n < 0 || (n && (!vts || !radii))) return VC_ERR_ARG;
    std::string s;
    VC_TRY(vc::format_radii(vts, radii, n, s));
    return vc::write_file(path, s);
}

extern "C" int vc_write_dotma(const char* path, const float* vts, const float* radii, int64_t nv,
                              const int32_t* edges, int64_t ne, const int32_t* tris, int64_t nt) {
    if (!path || nv < 0 || ne < 0 || nt < 0 || (nv && (!vts || !radii)) || (ne && !edges) || (nt && !tris))
        return VC_ERR_ARG;
    std::string s;
    VC_TRY(vc::format_dotma(vts, radii, nv, edges, ne, tris, nt, s));
    return vc::write_file(path, s);
}

extern "C" int vc_dotma_edges(const int32_t* edges, int64_t ne, const int32_t* tris, int64_t nt, int32_t* out,
                              int64_t cap, int64_t* n_out) {
    if (!n_out || ne < 0 || nt < 0 || (ne && !edges) || (nt && !tris)) return VC_ERR_ARG;
    std::vector<int32_t> e;
    vc::dotma_edges(edges, ne, tris, nt, e);
    *n_out = (int64_t)e.size() / 2;
    if (out) {
        if (cap < *n_out) return VC_ERR_ARG;
        std::copy(e.begin(), e.end(), out);
    }
    return VC_OK;
}

extern "C" int vc_write_remaining(vc_ctx* c, const char* prefix, int what) {
    if (!c || !prefix || (what & ~(VC_WRITE_PLY | VC_WRITE_RADII | VC_WRITE_MA)) != 0) return VC_ERR_ARG;
    if (!c->rem_valid) return VC_ERR_STATE;
    const vc_rem_sizes rs = c->rem;
    std::vector<float> vts((size_t)(3 * rs.nv));
    std::vector<int32_t> edges((size_t)(2 * rs.ne)), tris((size_t)(3 * rs.nt));
    VC_TRY(vc_get_remaining(c, vts.data(), edges.data(), tris.data(), VC_MEM_HOST));
    const std::string base(prefix);
    if (what & VC_WRITE_PLY)
        VC_TRY(vc_write_ply((base + ".ply").c_str(), vts.data(), rs.nv, edges.data(), rs.ne, tris.data(), rs.nt));
    if (what & (VC_WRITE_RADII | VC_WRITE_MA)) {
        // radii of the remaining vertices: the kept vertices of the lattice
        // complex in id order (getRemainedVts, src/ccthin.cpp:127-146)
        if (!c->vd_valid || c->cc_batched || c->nv != c->vd.nv) return VC_ERR_STATE;
        const int64_t nv = c->vd.nv;
        std::vector<float> all((size_t)nv), radii;
        std::vector<uint8_t> keep((size_t)nv);
        VC_TRY(vc_vertex_radii(c, all.data(), VC_MEM_HOST));
        VC_TRY(vc_get_thin_flags(c, keep.data(), nullptr, nullptr, nullptr, VC_MEM_HOST));
        radii.reserve((size_t)rs.nv);
        for (int64_t v = 0; v < nv; ++v)
            if (keep[v]) radii.push_back(all[v]);
        if ((int64_t)radii.size() != rs.nv) return VC_ERR_STATE;
        if (what & VC_WRITE_RADII)
            VC_TRY(vc_write_radii((base + ".r").c_str(), vts.data(), radii.data(), rs.nv));
        if (what & VC_WRITE_MA) {
            for (float& r : radii) r = std::sqrt(r * r);  // the caller's len(xform * (r, 0, 0))
            std::vector<int32_t> ma_edges;
            vc::dotma_edges(edges.data(), rs.ne, tris.data(), rs.nt, ma_edges);
            VC_TRY(vc_write_dotma((base + ".ma").c_str(), vts.data(), radii.data(), rs.nv, ma_edges.data(),
                                  (int64_t)ma_edges.size() / 2, tris.data(), rs.nt));
        }
    }
    return VC_OK;
}
