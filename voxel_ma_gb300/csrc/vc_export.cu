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
// 6 significant digits).  vc_write_remaining writes vertices and radii in
// model space: the volume's voxel-to-model matrix (the identity, or a .sog
// file's) applied as trimesh's xform * point, a radius r as
// len(M (r, 0, 0) - M (0, 0, 0)) in float; vc_write_radii takes model-space
// values and writes len((r, 0, 0)) = r.
#include "vc_internal.cuh"

#include <charconv>
#include <cmath>
#include <cstdio>
#include <string>
#include <thread>
#include <unordered_set>
#if defined(__GLIBCXX__)
#include <bits/hashtable_policy.h>  // std::__detail::_Prime_rehash_policy, the set's growth rule
#endif

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

int worker_threads(size_t n, size_t per_thread) {
    const size_t hw = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    return (int)std::max<size_t>(1, std::min(hw, n / per_thread + 1));
}
template <class F>
void parallel_for(int nth, F&& f) {
    if (nth <= 1) {
        f(0);
        return;
    }
    std::vector<std::thread> th;
    for (int t = 0; t < nth; ++t) th.emplace_back([&f, t] { f(t); });
    for (auto& x : th) x.join();
}

using Parts = std::vector<std::string>;

int write_file(const char* path, const Parts& parts) {
    FILE* f = std::fopen(path, "wb");
    if (!f) return VC_ERR_ARG;
    bool ok = true;
    for (const std::string& s : parts) ok = ok && std::fwrite(s.data(), 1, s.size(), f) == s.size();
    const int rc = std::fclose(f);
    return (ok && rc == 0) ? VC_OK : VC_ERR_ARG;
}

// lines [0, n) formatted by line(Text&, k), in chunks on worker threads,
// appended to parts in order
template <class F>
void lines(Parts& parts, int64_t n, size_t bytes_per_line, F&& line) {
    const int nth = worker_threads((size_t)n, 1 << 15);
    const size_t first = parts.size();
    parts.resize(first + nth);
    parallel_for(nth, [&](int t) {
        const int64_t k0 = n * t / nth, k1 = n * (t + 1) / nth;
        Text x;
        x.s.reserve((size_t)(k1 - k0) * bytes_per_line + 64);
        for (int64_t k = k0; k < k1; ++k) line(x, k);
        parts[first + t].swap(x.s);
    });
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

// trimesh's xform * point (SpaceConverter::fromVoxToModel, src/spaceinfo.cpp):
// each coordinate one double expression, times 1 / h, rounded to float
inline void xf_point(const double* m, const float* p, float* q) {
    float h = (float)(m[3] * p[0] + m[7] * p[1] + m[11] * p[2] + m[15]);
    h = 1.0f / h;
    for (int i = 0; i < 3; ++i) q[i] = (float)((m[i] * p[0] + m[i + 4] * p[1] + m[i + 8] * p[2] + m[i + 12]) * h);
}

}  // namespace

void format_ply(const float* vts, int64_t nv, const int32_t* edges, int64_t ne, const int32_t* tris, int64_t nt,
                Parts& out) {
    Text h;
    h.str("ply\nformat ascii 1.0\ncomment Generated by VoxelCore\nelement vertex ");
    h.i(nv);
    h.str("\nproperty float32 x\nproperty float32 y\nproperty float32 z\nelement edge ");
    h.i(ne);
    h.str("\nproperty int32 vertex1\nproperty int32 vertex2\nelement face ");
    h.i(nt);
    h.str("\nproperty list uint8 int32 vertex_indices\nend_header\n");
    out.push_back(std::move(h.s));
    lines(out, nv, 32, [&](Text& t, int64_t k) {
        for (int d = 0; d < 3; ++d) {
            t.g(vts[3 * k + d]);
            t.c(' ');
        }
        t.c('\n');
    });
    lines(out, ne, 18, [&](Text& t, int64_t k) {
        t.i(edges[2 * k]);
        t.c(' ');
        t.i(edges[2 * k + 1]);
        t.str(" \n");
    });
    lines(out, nt, 28, [&](Text& t, int64_t k) {
        t.str("3 ");
        for (int d = 0; d < 3; ++d) {
            t.i(tris[3 * k + d]);
            t.c(' ');
        }
        t.c('\n');
    });
}

void format_radii(const float* vts, const float* radii, int64_t n, Parts& out) {
    Text h;
    h.i(n);
    h.c('\n');
    out.push_back(std::move(h.s));
    lines(out, n, 40, [&](Text& t, int64_t k) {
        const float r = radii[k];
        for (int d = 0; d < 3; ++d) {
            t.g(vts[3 * k + d]);
            t.c(' ');
        }
        t.g(std::sqrt(r * r));
        t.c('\n');
    });
}

void format_dotma(const float* vts, const float* radii, int64_t nv, const int32_t* edges, int64_t ne,
                  const int32_t* tris, int64_t nt, Parts& out) {
    Text h;
    h.i(nv);
    h.c(' ');
    h.i(ne);
    h.c(' ');
    h.i(nt);
    h.c('\n');
    out.push_back(std::move(h.s));
    lines(out, nv, 42, [&](Text& t, int64_t k) {
        t.str("v ");
        for (int d = 0; d < 3; ++d) {
            t.g(vts[3 * k + d]);
            t.c(' ');
        }
        t.g(radii[k]);
        t.c('\n');
    });
    lines(out, ne, 18, [&](Text& t, int64_t k) {
        t.str("e ");
        t.i(edges[2 * k]);
        t.c(' ');
        t.i(edges[2 * k + 1]);
        t.c('\n');
    });
    lines(out, nt, 28, [&](Text& t, int64_t k) {
        t.str("f ");
        for (int d = 0; d < 3; ++d) {
            t.i((uint32_t)tris[3 * k + d]);
            t.c(d < 2 ? ' ' : '\n');
        }
    });
}

// Keys in first-insertion order.  Each thread owns a hash shard of the keys
// and marks their first occurrences; a sequential pass keeps the marked ones.
std::vector<uint64_t> first_occurrences(const std::vector<uint64_t>& ins) {
    const size_t n = ins.size();
    const int nth = worker_threads(n, 1 << 16);
    std::vector<uint8_t> first(n, 0);
    parallel_for(nth, [&](int t) {
        size_t cap = 16;
        while (cap < 2 * (n / nth) + 16) cap <<= 1;
        std::vector<uint64_t> tab(cap, ~0ull);
        for (size_t i = 0; i < n; ++i) {
            const uint64_t k = ins[i], m = k * 0x9E3779B97F4A7C15ull;
            if ((int)((m >> 59) % (uint64_t)nth) != t) continue;
            size_t h = (m >> 7) & (cap - 1);
            while (tab[h] != ~0ull && tab[h] != k) h = (h + 1) & (cap - 1);
            if (tab[h] == ~0ull) {
                tab[h] = k;
                first[i] = 1;
            }
        }
    });
    std::vector<uint64_t> u;
    u.reserve(n);
    for (size_t i = 0; i < n; ++i)
        if (first[i]) u.push_back(ins[i]);
    return u;
}

#if defined(__GLIBCXX__)
// The iteration order of a std::unordered_set<key, EdgeHash> (libstdc++)
// after inserting ins in order, replayed on arrays: every node goes to the
// front of its bucket; a bucket that was empty goes to the front of the
// list; a rehash (when the set's own _Prime_rehash_policy asks for one,
// starting from one bucket) walks the list in order and re-inserts each node
// the same way.  Equal to the set's order by construction; faster because no
// node is allocated and the bucket heads are prefetched.
std::vector<uint64_t> unordered_set_order(const std::vector<uint64_t>& ins) {
    const std::vector<uint64_t> uniq = first_occurrences(ins);
    const size_t n = uniq.size();
    EdgeHash H;
    std::vector<size_t> code(n);
    for (size_t i = 0; i < n; ++i) code[i] = H(uniq[i]);
    std::__detail::_Prime_rehash_policy pol;
    size_t nb = 1;
    std::vector<int32_t> head(1, -1), nxt(n, -1);
    std::vector<uint32_t> order;  // buckets in the order they became non-empty (the list is its reverse)
    auto rehash = [&](size_t nbn) {
        std::vector<int32_t> nh(nbn, -1);
        std::vector<uint32_t> nord;
        nord.reserve(std::min(nbn, n));
        for (size_t oi = order.size(); oi-- > 0;) {
            if (oi >= 16) __builtin_prefetch(&head[order[oi - 16]]);
            for (int32_t p = head[order[oi]]; p >= 0;) {
                const int32_t q = nxt[p];
                const size_t b = code[p] % nbn;
                if (nh[b] < 0) nord.push_back((uint32_t)b);
                nxt[p] = nh[b];
                nh[b] = p;
                p = q;
            }
        }
        head.swap(nh);
        order.swap(nord);
        nb = nbn;
    };
    for (size_t i = 0; i < n; ++i) {
        if (i + 24 < n) __builtin_prefetch(&head[code[i + 24] % nb]);
        const auto r = pol._M_need_rehash(nb, i, 1);
        if (r.first) rehash(r.second);
        const size_t b = code[i] % nb;
        if (head[b] < 0) order.push_back((uint32_t)b);
        nxt[i] = head[b];
        head[b] = (int32_t)i;
    }
    std::vector<uint64_t> out;
    out.reserve(n);
    for (size_t oi = order.size(); oi-- > 0;)
        for (int32_t p = head[order[oi]]; p >= 0; p = nxt[p]) out.push_back(uniq[p]);
    return out;
}
#else
// Other standard libraries: a real std::unordered_set filled in the same
// order, iterated in its own order (the reference's order is libstdc++'s).
std::vector<uint64_t> unordered_set_order(const std::vector<uint64_t>& ins) {
    std::unordered_set<uint64_t, EdgeHash> set;
    for (const uint64_t k : ins) set.insert(k);
    return std::vector<uint64_t>(set.begin(), set.end());
}
#endif

// the caller's .ma edge list: remaining edges, then the triangles' edges in
// the iteration order of a fresh unordered_set filled triangle by triangle
void dotma_edges(const int32_t* edges, int64_t ne, const int32_t* tris, int64_t nt, std::vector<int32_t>& out) {
    out.assign(edges, edges + 2 * ne);
    std::vector<uint64_t> ins((size_t)(3 * nt));
    for (int64_t k = 0; k < nt; ++k)
        for (int d = 0; d < 3; ++d) ins[3 * k + d] = edge_key(tris[3 * k + d], tris[3 * k + (d + 1) % 3]);
    for (const uint64_t e : unordered_set_order(ins)) {
        out.push_back((int32_t)(e >> 32));
        out.push_back((int32_t)(uint32_t)e);
    }
}

}  // namespace vc

extern "C" int vc_write_ply(const char* path, const float* vts, int64_t nv, const int32_t* edges, int64_t ne,
                            const int32_t* tris, int64_t nt) {
    if (!path || nv < 0 || ne < 0 || nt < 0 || (nv && !vts) || (ne && !edges) || (nt && !tris)) return VC_ERR_ARG;
    vc::Parts parts;
    vc::format_ply(vts, nv, edges, ne, tris, nt, parts);
    return vc::write_file(path, parts);
}

extern "C" int vc_write_radii(const char* path, const float* vts, const float* radii, int64_t n) {
    if (!path || n < 0 || (n && (!vts || !radii))) return VC_ERR_ARG;
    vc::Parts parts;
    vc::format_radii(vts, radii, n, parts);
    return vc::write_file(path, parts);
}

extern "C" int vc_write_dotma(const char* path, const float* vts, const float* radii, int64_t nv,
                              const int32_t* edges, int64_t ne, const int32_t* tris, int64_t nt) {
    if (!path || nv < 0 || ne < 0 || nt < 0 || (nv && (!vts || !radii)) || (ne && !edges) || (nt && !tris))
        return VC_ERR_ARG;
    vc::Parts parts;
    vc::format_dotma(vts, radii, nv, edges, ne, tris, nt, parts);
    return vc::write_file(path, parts);
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
    // the written vertices are in model space (vts_trans, src/highlevelalgo.cpp:750-760)
    const double* M = c->vox_to_model;
    for (int64_t k = 0; k < rs.nv; ++k) {
        const float p[3] = {vts[3 * k], vts[3 * k + 1], vts[3 * k + 2]};
        vc::xf_point(M, p, &vts[3 * k]);
    }
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
        // r in model space: len(xform * (r, 0, 0) - xform * (0, 0, 0)) in float
        // (src/exporters.cpp:520-530, src/highlevelalgo.cpp:914-922)
        const float zero[3] = {0, 0, 0};
        float o[3];
        vc::xf_point(M, zero, o);
        for (int64_t v = 0; v < nv; ++v)
            if (keep[v]) {
                const float p[3] = {all[v], 0, 0};
                float q[3];
                vc::xf_point(M, p, q);
                const float d[3] = {q[0] - o[0], q[1] - o[1], q[2] - o[2]};
                radii.push_back(std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]));
            }
        if ((int64_t)radii.size() != rs.nv) return VC_ERR_STATE;
        // vc_write_radii writes len((r, 0, 0)) = r for these non-negative r
        if (what & VC_WRITE_RADII)
            VC_TRY(vc_write_radii((base + ".r").c_str(), vts.data(), radii.data(), rs.nv));
        if (what & VC_WRITE_MA) {
            std::vector<int32_t> ma_edges;
            vc::dotma_edges(edges.data(), rs.ne, tris.data(), rs.nt, ma_edges);
            VC_TRY(vc_write_dotma((base + ".ma").c_str(), vts.data(), radii.data(), rs.nv, ma_edges.data(),
                                  (int64_t)ma_edges.size() / 2, tris.data(), rs.nt));
        }
    }
    return VC_OK;
}
