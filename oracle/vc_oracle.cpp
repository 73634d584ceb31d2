// CPU restatement of the Voxel Cores hot path ("oracle").  TEST
// INFRASTRUCTURE: see vc_oracle.h for who may load it and for the shared
// conventions.  Every function restates the reference behaviour cited beside
// it; the GPU library never links this file.
#include "vc_oracle.h"

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstring>
#include <deque>
#include <functional>
#include <queue>
#include <thread>
#include <unordered_map>
#include <unordered_set>
#include <vector>

namespace {

// ---------------------------------------------------------------------------
// Site extraction tables (surfacing.h:121-136, 170-198).
// Corner c of a voxel, as the lattice offset (dx,dy,dz) in {0,1}^3 of that
// corner from the voxel's lowest corner: the reference numbers corners
// 0:(+x,-y,-z) 1:(+x,+y,-z) 2:(-x,-y,-z) 3:(-x,+y,-z)
// 4:(+x,-y,+z) 5:(+x,+y,+z) 6:(-x,-y,+z) 7:(-x,+y,+z).
const int kCornerOff[8][3] = {{1, 0, 0}, {1, 1, 0}, {0, 0, 0}, {0, 1, 0},
                              {1, 0, 1}, {1, 1, 1}, {0, 0, 1}, {0, 1, 1}};
// Face-neighbour directions in sweep order -x,+x,-y,+y,-z,+z.
const int kNbOff[6][3] = {{-1, 0, 0}, {1, 0, 0}, {0, -1, 0}, {0, 1, 0}, {0, 0, -1}, {0, 0, 1}};
// The four corners shared with each face neighbour, in visiting order.
const int kShared[6][4] = {{2, 3, 7, 6}, {0, 1, 5, 4}, {4, 6, 2, 0}, {1, 3, 7, 5}, {0, 2, 3, 1}, {5, 7, 6, 4}};

inline int occ_at(const uint8_t* occ, int X, int Y, int Z, int i, int j, int k) {
    if (i < 0 || j < 0 || k < 0 || i >= X || j >= Y || k >= Z) return 0;
    return occ[((int64_t)i * Y + j) * Z + k] > 0 ? 1 : 0;
}

// ---------------------------------------------------------------------------
// Feature transform helpers.
// Packed candidate: (value << 32) | id, so that integer order is the
// lexicographic (value, id) order.  value = partial squared distance.
const int64_t kInf = INT64_MAX;
inline int64_t pack(int64_t g, int32_t id) { return (g << 32) | (uint32_t)id; }
inline int64_t pk_g(int64_t p) { return p >> 32; }
inline int32_t pk_id(int64_t p) { return (int32_t)(uint32_t)(p & 0xffffffffLL); }

inline int64_t floordiv(int64_t n, int64_t d) {  // d > 0
    int64_t q = n / d;
    if ((n % d) != 0 && n < 0) --q;
    return q;
}
// Smallest integer x at which candidate r (position qr) beats candidate p
// (position qp < qr) in the lexicographic (value, id) order.
inline int64_t cross_threshold(int64_t qp, int64_t gp, int32_t idp, int64_t qr, int64_t gr, int32_t idr) {
    int64_t den = 2 * (qr - qp);
    int64_t num = qr * qr - qp * qp + gr - gp;
    int64_t fl = floordiv(num, den);
    if (fl * den == num && idr < idp) return fl;
    return fl + 1;
}
// One lower-envelope pass over a line of length L: in[x] are packed
// candidates (kInf = none); out[x] = packed (x-q)^2 + g of the winner.
void envelope_line(int L, const int64_t* in, int64_t* out, int* vq, int64_t* vz) {
    int k = 0;
    for (int q = 0; q < L; ++q) {
        int64_t c = in[q];
        if (c == kInf) continue;
        int64_t g = pk_g(c);
        int32_t id = pk_id(c);
        int64_t T = 0;
        while (k > 0) {
            int64_t t = vq[k - 1];
            int64_t pc = in[t];
            T = cross_threshold(t, pk_g(pc), pk_id(pc), q, g, id);
            if (T <= vz[k - 1]) {
                --k;
                continue;
            }
            break;
        }
        if (k == 0) {
            vq[0] = q;
            vz[0] = 0;
            k = 1;
        } else if (T < L) {
            vq[k] = q;
            vz[k] = T;
            ++k;
        }
    }
    if (k == 0) {
        for (int x = 0; x < L; ++x) out[x] = kInf;
        return;
    }
    int w = 0;
    for (int x = 0; x < L; ++x) {
        while (w + 1 < k && vz[w + 1] <= x) ++w;
        int64_t c = in[vq[w]];
        int64_t d = (int64_t)x - vq[w];
        out[x] = pack(pk_g(c) + d * d, pk_id(c));
    }
}

template <class F>
void parallel_for(int64_t n, int nthreads, F f) {
    if (nthreads <= 1 || n < 2) {
        f(0, n);
        return;
    }
    std::vector<std::thread> ts;
    int64_t chunk = (n + nthreads - 1) / nthreads;
    for (int t = 0; t < nthreads; ++t) {
        int64_t b = t * chunk, e = std::min(n, b + chunk);
        if (b >= e) break;
        ts.emplace_back([=] { f(b, e); });
    }
    for (auto& t : ts) t.join();
}

inline float lambda_of(const float* sxyz, int32_t s0, int32_t s1) {
    // MeasureForMA::lambdaForFace = trimesh::dist (measureforMA_imp.h:1-4):
    // squared differences accumulated in float, then a float square root.
    float d = 0.0f;
    for (int k = 0; k < 3; ++k) {
        float t = sxyz[3 * (int64_t)s0 + k] - sxyz[3 * (int64_t)s1 + k];
        d += t * t;
    }
    return std::sqrt(d);
}

struct VD {
    std::vector<float> vts, vm, em, fm, radius;
    std::vector<int32_t> edges, tris, tri_face, face_sites;
    long long nface = 0;
    float inside_size = 0.0f;
};

inline uint64_t ekey(int32_t a, int32_t b) { return ((uint64_t)(uint32_t)a << 32) | (uint32_t)b; }
inline void make_edge(int32_t u, int32_t v, int32_t& a, int32_t& b) {
    // util::makeEdge (geomalgo.h:79-82): smaller index first.
    if (u > v) { a = v; b = u; } else { a = u; b = v; }
}

// Finalized complex in CSR form.
struct Fin {
    std::vector<int32_t> edges;      // 2*E
    std::vector<int32_t> tri_edges;  // 3*T
    std::vector<int32_t> ve_off, ve_ids, ef_off, ef_ids;
};

// Edge key -> first edge id, open addressing with linear probing (keys are
// ordered vertex pairs, so all-ones never occurs and marks an empty slot).
// Same mapping as the reference's unordered_map, far less memory at 10^8 keys.
struct EdgeIndex {
    std::vector<uint64_t> keys;
    std::vector<int32_t> vals;
    size_t mask = 0, count = 0;
    static constexpr uint64_t kEmpty = ~0ULL;
    static uint64_t mix(uint64_t z) {
        z ^= z >> 31;
        z *= 0x7fb5d329728ea185ULL;
        z ^= z >> 27;
        z *= 0x81dadef4bc2dd44dULL;
        return z ^ (z >> 33);
    }
    explicit EdgeIndex(size_t expect) { rehash(std::max<size_t>(64, expect * 2)); }
    void rehash(size_t want) {
        size_t cap = 64;
        while (cap < want) cap <<= 1;
        std::vector<uint64_t> ok;
        std::vector<int32_t> ov;
        ok.swap(keys);
        ov.swap(vals);
        keys.assign(cap, kEmpty);
        vals.assign(cap, 0);
        mask = cap - 1;
        for (size_t i = 0; i < ok.size(); ++i)
            if (ok[i] != kEmpty) place(ok[i], ov[i]);
    }
    void place(uint64_t k, int32_t v) {
        size_t s = mix(k) & mask;
        while (keys[s] != kEmpty) s = (s + 1) & mask;
        keys[s] = k;
        vals[s] = v;
    }
    // the id stored for k, or -1 after storing v for it
    int32_t find_or_insert(uint64_t k, int32_t v) {
        size_t s = mix(k) & mask;
        while (keys[s] != kEmpty) {
            if (keys[s] == k) return vals[s];
            s = (s + 1) & mask;
        }
        keys[s] = k;
        vals[s] = v;
        if (++count * 2 > mask + 1) rehash((mask + 1) * 2);
        return -1;
    }
};

void finalize(long long nv, long long ne, const int32_t* edges, long long nt, const int32_t* tris, Fin& F,
              bool adjacency = true) {
    // cellcomplex::finalize (cellcomplex.cpp:364-491).  Edge keys are ORDERED
    // pairs: given edges keep first-occurrence order, then face sides (made
    // with makeEdge) that are new are appended in face order.
    EdgeIndex idx((size_t)ne);
    F.edges.clear();
    for (long long i = 0; i < ne; ++i) {
        uint64_t k = ekey(edges[2 * i], edges[2 * i + 1]);
        if (idx.find_or_insert(k, (int32_t)(F.edges.size() / 2)) < 0) {
            F.edges.push_back(edges[2 * i]);
            F.edges.push_back(edges[2 * i + 1]);
        }
    }
    F.tri_edges.resize((size_t)(3 * nt));
    for (long long f = 0; f < nt; ++f) {
        for (int s = 0; s < 3; ++s) {
            int32_t a, b;
            make_edge(tris[3 * f + s], tris[3 * f + (s + 1) % 3], a, b);
            int32_t id = idx.find_or_insert(ekey(a, b), (int32_t)(F.edges.size() / 2));
            if (id < 0) {
                id = (int32_t)(F.edges.size() / 2);
                F.edges.push_back(a);
                F.edges.push_back(b);
            }
            F.tri_edges[3 * f + s] = id;
        }
    }
    { EdgeIndex drop(0); std::swap(idx, drop); }
    if (!adjacency) return;
    long long E = (long long)F.edges.size() / 2;
    // V->E: every edge id is appended to both endpoints, in id order.
    F.ve_off.assign((size_t)nv + 1, 0);
    for (long long e = 0; e < E; ++e) {
        F.ve_off[F.edges[2 * e] + 1]++;
        F.ve_off[F.edges[2 * e + 1] + 1]++;
    }
    for (long long v = 0; v < nv; ++v) F.ve_off[v + 1] += F.ve_off[v];
    F.ve_ids.resize((size_t)F.ve_off[nv]);
    {
        std::vector<int32_t> cur(F.ve_off.begin(), F.ve_off.end() - 1);
        for (long long e = 0; e < E; ++e) {
            F.ve_ids[cur[F.edges[2 * e]]++] = (int32_t)e;
            F.ve_ids[cur[F.edges[2 * e + 1]]++] = (int32_t)e;
        }
    }
    // E->F: every face id is appended to each of its sides, in face order.
    F.ef_off.assign((size_t)E + 1, 0);
    for (long long i = 0; i < 3 * nt; ++i) F.ef_off[F.tri_edges[i] + 1]++;
    for (long long e = 0; e < E; ++e) F.ef_off[e + 1] += F.ef_off[e];
    F.ef_ids.resize((size_t)F.ef_off[E]);
    {
        std::vector<int32_t> cur(F.ef_off.begin(), F.ef_off.end() - 1);
        for (long long f = 0; f < nt; ++f)
            for (int s = 0; s < 3; ++s) F.ef_ids[cur[F.tri_edges[3 * f + s]]++] = (int32_t)f;
    }
}

}  // namespace

extern "C" {

long long vco_extract_sites(const uint8_t* occ, int X, int Y, int Z, float* xyz, int64_t* lattice_idx,
                            long long cap) {
    // Surfacer::extractBoundaryVts (surfacing.cpp:223-321): sweep every voxel
    // i -> j -> k; for each face neighbour with a different occupancy, add the
    // four shared corners not seen before.  A dense seen-array stands in for
    // the reference's hash map; the order of first encounters is the same.
    const int64_t NB = Y + 1, NC = Z + 1;
    std::vector<uint8_t> seen((size_t)((int64_t)(X + 1) * NB * NC), 0);
    long long n = 0;
    for (int i = 0; i < X; ++i)
        for (int j = 0; j < Y; ++j)
            for (int k = 0; k < Z; ++k) {
                int cur = occ_at(occ, X, Y, Z, i, j, k);
                for (int o = 0; o < 6; ++o) {
                    int nb = occ_at(occ, X, Y, Z, i + kNbOff[o][0], j + kNbOff[o][1], k + kNbOff[o][2]);
                    if (nb == cur) continue;
                    for (int ii = 0; ii < 4; ++ii) {
                        const int* co = kCornerOff[kShared[o][ii]];
                        int a = i + co[0], b = j + co[1], c = k + co[2];
                        int64_t p = ((int64_t)a * NB + b) * NC + c;
                        if (seen[p]) continue;
                        seen[p] = 1;
                        if (n < cap) {
                            if (xyz) {
                                xyz[3 * n + 0] = (float)a - 0.5f;
                                xyz[3 * n + 1] = (float)b - 0.5f;
                                xyz[3 * n + 2] = (float)c - 0.5f;
                            }
                            if (lattice_idx) lattice_idx[n] = p;
                        }
                        ++n;
                    }
                }
            }
    return n;
}

void vco_ft_bruteforce(int X, int Y, int Z, long long nsites, const int64_t* sl, int32_t* d2, int32_t* id) {
    const int64_t NA = X + 1, NB = Y + 1, NC = Z + 1;
    std::vector<int32_t> sa(nsites), sb(nsites), sc(nsites);
    for (long long s = 0; s < nsites; ++s) {
        sa[s] = (int32_t)(sl[s] / (NB * NC));
        sb[s] = (int32_t)((sl[s] / NC) % NB);
        sc[s] = (int32_t)(sl[s] % NC);
    }
    for (int64_t a = 0; a < NA; ++a)
        for (int64_t b = 0; b < NB; ++b)
            for (int64_t c = 0; c < NC; ++c) {
                int64_t best = INT64_MAX;
                int32_t bi = -1;
                for (long long s = 0; s < nsites; ++s) {
                    int64_t da = a - sa[s], db = b - sb[s], dc = c - sc[s];
                    int64_t dd = da * da + db * db + dc * dc;
                    if (dd < best) { best = dd; bi = (int32_t)s; }  // strict: lowest index wins ties
                }
                int64_t p = (a * NB + b) * NC + c;
                d2[p] = bi < 0 ? INT32_MAX : (int32_t)best;
                id[p] = bi;
            }
}

void vco_ft(int X, int Y, int Z, long long nsites, const int64_t* sl, int32_t* d2, int32_t* id, int nthreads) {
    // No reference counterpart (the reference has no feature transform); the
    // relation it restates is "nearest boundary-corner site, lowest index on
    // ties" over the corner lattice.
    const int64_t NA = X + 1, NB = Y + 1, NC = Z + 1, N = NA * NB * NC;
    std::vector<int64_t> g((size_t)N, kInf), h((size_t)N);
    for (long long s = 0; s < nsites; ++s) g[sl[s]] = pack(0, (int32_t)s);
    // Pass 1 (along c): nearest site in each row, by a forward and a backward scan.
    parallel_for(NA * NB, nthreads, [&](int64_t r0, int64_t r1) {
        for (int64_t r = r0; r < r1; ++r) {
            int64_t* row = &g[r * NC];
            int64_t* out = &h[r * NC];
            int64_t last = -1;
            int32_t lastid = -1;
            for (int64_t c = 0; c < NC; ++c) {
                if (row[c] != kInf) { last = c; lastid = pk_id(row[c]); }
                out[c] = last < 0 ? kInf : pack((c - last) * (c - last), lastid);
            }
            last = -1;
            for (int64_t c = NC - 1; c >= 0; --c) {
                if (row[c] != kInf) { last = c; lastid = pk_id(row[c]); }
                if (last >= 0) out[c] = std::min(out[c], pack((last - c) * (last - c), lastid));
            }
        }
    });
    // Pass 2 (along b) and pass 3 (along a): lower envelopes.
    auto pass = [&](const std::vector<int64_t>& in, std::vector<int64_t>& out, int64_t L, int64_t stride,
                    int64_t nlines, auto line_base) {
        parallel_for(nlines, nthreads, [&](int64_t l0, int64_t l1) {
            std::vector<int64_t> bin(L), bout(L), vz(L);
            std::vector<int> vq(L);
            for (int64_t l = l0; l < l1; ++l) {
                int64_t base = line_base(l);
                for (int64_t x = 0; x < L; ++x) bin[x] = in[base + x * stride];
                envelope_line((int)L, bin.data(), bout.data(), vq.data(), vz.data());
                for (int64_t x = 0; x < L; ++x) out[base + x * stride] = bout[x];
            }
        });
    };
    pass(h, g, NB, NC, NA * NC, [&](int64_t l) { return (l / NC) * NB * NC + (l % NC); });
    pass(g, h, NA, NB * NC, NB * NC, [&](int64_t l) { return l; });
    for (int64_t p = 0; p < N; ++p) {
        if (h[p] == kInf) {
            d2[p] = INT32_MAX;
            id[p] = -1;
        } else {
            d2[p] = (int32_t)pk_g(h[p]);
            id[p] = pk_id(h[p]);
        }
    }
}

void* vco_lattice_vd(const uint8_t* occ, int X, int Y, int Z, const int32_t* ft_id, const float* sxyz) {
    // Lattice Voronoi complex: the dual square of every corner-lattice edge
    // whose two endpoints have different nearest sites is a Voronoi face
    // piece; its vertices are the centres of the four voxels around the edge.
    // The inside part, measures, triangulation and compaction follow
    // VoroInfo::extractInsideWithMeasure (voroinfo.cpp:624-729) with the
    // validity rules of voroinfo_imp.h:5-48 and the lambda measures of
    // voroinfo.cpp:1432-1574.
    auto* R = new VD();
    const int64_t NB = Y + 1, NC = Z + 1;
    const int64_t NV = (int64_t)X * Y * Z;
    auto vox = [&](int64_t i, int64_t j, int64_t k) { return (i * Y + j) * Z + k; };
    auto inside = [&](int64_t i, int64_t j, int64_t k) { return occ_at(occ, X, Y, Z, (int)i, (int)j, (int)k) == 1; };
    auto lid = [&](int64_t a, int64_t b, int64_t c) { return (a * NB + b) * NC + c; };
    auto cand = [&](int64_t a, int64_t b, int64_t c, int d) -> bool {
        // lattice edge from (a,b,c) along axis d differs in label?
        int64_t e[3] = {a, b, c};
        e[d] += 1;
        if (a < 0 || b < 0 || c < 0 || e[0] > X || e[1] > Y || e[2] > Z) return false;
        int32_t i0 = ft_id[lid(a, b, c)], i1 = ft_id[lid(e[0], e[1], e[2])];
        return i0 >= 0 && i1 >= 0 && i0 != i1;
    };
    // Quad vertex (s,t) of the dual square of lattice edge (p, d): voxel
    // coordinate p_d along d, p_u-1+s along u=(d+1)%3, p_w-1+t along w=(d+2)%3.
    const int qs[4] = {0, 1, 1, 0}, qt[4] = {0, 0, 1, 1};
    auto quad_voxel = [&](const int64_t p[3], int d, int q, int64_t out[3]) {
        int u = (d + 1) % 3, w = (d + 2) % 3;
        out[d] = p[d];
        out[u] = p[u] - 1 + qs[q];
        out[w] = p[w] - 1 + qt[q];
    };
    // 1) valid vertices: inside voxels that are a corner of some candidate face.
    std::vector<int32_t> vid((size_t)NV, -1);
    std::vector<uint8_t> vtx((size_t)NV, 0);
    for (int64_t a = 0; a <= X; ++a)
        for (int64_t b = 0; b <= Y; ++b)
            for (int64_t c = 0; c <= Z; ++c)
                for (int d = 0; d < 3; ++d) {
                    if (!cand(a, b, c, d)) continue;
                    int64_t p[3] = {a, b, c}, v[3];
                    for (int q = 0; q < 4; ++q) {
                        quad_voxel(p, d, q, v);
                        if (inside(v[0], v[1], v[2])) vtx[vox(v[0], v[1], v[2])] = 1;
                    }
                }
    float bmin[3] = {INFINITY, INFINITY, INFINITY}, bmax[3] = {-INFINITY, -INFINITY, -INFINITY};
    int32_t nvv = 0;
    for (int64_t i = 0; i < X; ++i)
        for (int64_t j = 0; j < Y; ++j)
            for (int64_t k = 0; k < Z; ++k) {
                if (!vtx[vox(i, j, k)]) continue;
                vid[vox(i, j, k)] = nvv++;
                float pc[3] = {(float)i, (float)j, (float)k};
                for (int m = 0; m < 3; ++m) {
                    R->vts.push_back(pc[m]);
                    bmin[m] = std::min(bmin[m], pc[m]);
                    bmax[m] = std::max(bmax[m], pc[m]);
                }
            }
    R->inside_size = nvv ? std::max(bmax[0] - bmin[0], std::max(bmax[1] - bmin[1], bmax[2] - bmin[2])) : 0.0f;
    // 2) valid faces in (lattice point, axis) order with their lambda.
    std::vector<int64_t> face_p;
    std::vector<int8_t> face_d;
    std::vector<float> face_l;
    for (int64_t a = 0; a <= X; ++a)
        for (int64_t b = 0; b <= Y; ++b)
            for (int64_t c = 0; c <= Z; ++c)
                for (int d = 0; d < 3; ++d) {
                    if (!cand(a, b, c, d)) continue;
                    int64_t p[3] = {a, b, c}, v[3];
                    bool ok = true;
                    for (int q = 0; q < 4 && ok; ++q) {
                        quad_voxel(p, d, q, v);
                        ok = inside(v[0], v[1], v[2]);
                    }
                    if (!ok) continue;
                    int64_t e[3] = {a, b, c};
                    e[d] += 1;
                    int32_t s0 = ft_id[lid(a, b, c)], s1 = ft_id[lid(e[0], e[1], e[2])];
                    face_p.push_back(lid(a, b, c));
                    face_d.push_back((int8_t)d);
                    face_l.push_back(lambda_of(sxyz, s0, s1));
                    R->face_sites.push_back(s0);
                    R->face_sites.push_back(s1);
                }
    R->nface = (long long)face_p.size();
    // 3) vertex measure: max lambda over valid faces having the vertex.
    R->vm.assign((size_t)nvv, 0.0f);
    auto decode = [&](int64_t lp, int64_t p[3]) {
        p[0] = lp / (NB * NC);
        p[1] = (lp / NC) % NB;
        p[2] = lp % NC;
    };
    for (size_t f = 0; f < face_p.size(); ++f) {
        int64_t p[3], v[3];
        decode(face_p[f], p);
        for (int q = 0; q < 4; ++q) {
            quad_voxel(p, face_d[f], q, v);
            float& m = R->vm[vid[vox(v[0], v[1], v[2])]];
            m = std::max(m, face_l[f]);
        }
    }
    // 3b) radius per vertex, VoroInfo::computeInfoRelatedtoSites
    // (voroinfo.cpp:286-325): for every Voronoi face in face order (here all
    // candidate faces, valid or not, in (lattice point, axis) order), each
    // vertex of the face gets r = dist(first site of the face, vertex); the
    // last face to touch a vertex wins (voroinfo.cpp:316).  The first site of
    // face (p, d) is the label of its lower end p.
    R->radius.assign((size_t)nvv, 0.0f);
    for (int64_t a = 0; a <= X; ++a)
        for (int64_t b = 0; b <= Y; ++b)
            for (int64_t c = 0; c <= Z; ++c)
                for (int d = 0; d < 3; ++d) {
                    if (!cand(a, b, c, d)) continue;
                    const int32_t s0 = ft_id[lid(a, b, c)];
                    int64_t p[3] = {a, b, c}, v[3];
                    for (int q = 0; q < 4; ++q) {
                        quad_voxel(p, d, q, v);
                        if (!inside(v[0], v[1], v[2])) continue;
                        const int32_t vi = vid[vox(v[0], v[1], v[2])];
                        float r = 0.0f;  // trimesh::dist(site_p, v_p), float accumulation
                        for (int k = 0; k < 3; ++k) {
                            float t = (float)v[k] - sxyz[3 * (int64_t)s0 + k];
                            r += t * t;
                        }
                        R->radius[(size_t)vi] = std::sqrt(r);
                    }
                }
    // 4) valid edges (both ends inside, side of some candidate face) in
    // (voxel, axis) order; measure = max lambda over incident valid faces.
    // The dual edge (v, v+e_d) is a side of the dual squares of the four
    // lattice edges bounding the plaquette shared by the two voxels: lattice
    // edges along u and w through corners (v+e_d) + {0,1}e_u + {0,1}e_w.
    for (int64_t i = 0; i < X; ++i)
        for (int64_t j = 0; j < Y; ++j)
            for (int64_t k = 0; k < Z; ++k) {
                if (vid[vox(i, j, k)] < 0) continue;
                for (int d = 0; d < 3; ++d) {
                    int64_t w2[3] = {i, j, k};
                    w2[d] += 1;
                    if (w2[d] >= (d == 0 ? X : d == 1 ? Y : Z)) continue;
                    if (vid[vox(w2[0], w2[1], w2[2])] < 0) continue;
                    int u = (d + 1) % 3, w = (d + 2) % 3;
                    bool any = false;
                    float m = 0.0f;
                    // corners of the plaquette: lattice coords c = v + e_d + s e_u + t e_w
                    for (int s = 0; s < 2; ++s)
                        for (int t = 0; t < 2; ++t) {
                            int64_t c[3] = {i, j, k};
                            c[d] += 1;
                            c[u] += s;
                            c[w] += t;
                            // lattice edge along u from c (only from t side corners with s==0)
                            if (s == 0) {
                                if (cand(c[0], c[1], c[2], u)) {
                                    any = true;
                                    // face valid?  its 4 voxels along (w, d) around it
                                    int64_t pv[3], vv[3];
                                    pv[0] = c[0]; pv[1] = c[1]; pv[2] = c[2];
                                    bool ok = true;
                                    for (int q = 0; q < 4 && ok; ++q) {
                                        quad_voxel(pv, u, q, vv);
                                        ok = inside(vv[0], vv[1], vv[2]);
                                    }
                                    if (ok) {
                                        int64_t e2[3] = {c[0], c[1], c[2]};
                                        e2[u] += 1;
                                        m = std::max(m, lambda_of(sxyz, ft_id[lid(c[0], c[1], c[2])],
                                                                  ft_id[lid(e2[0], e2[1], e2[2])]));
                                    }
                                }
                            }
                            if (t == 0) {
                                if (cand(c[0], c[1], c[2], w)) {
                                    any = true;
                                    int64_t pv[3] = {c[0], c[1], c[2]}, vv[3];
                                    bool ok = true;
                                    for (int q = 0; q < 4 && ok; ++q) {
                                        quad_voxel(pv, w, q, vv);
                                        ok = inside(vv[0], vv[1], vv[2]);
                                    }
                                    if (ok) {
                                        int64_t e2[3] = {c[0], c[1], c[2]};
                                        e2[w] += 1;
                                        m = std::max(m, lambda_of(sxyz, ft_id[lid(c[0], c[1], c[2])],
                                                                  ft_id[lid(e2[0], e2[1], e2[2])]));
                                    }
                                }
                            }
                        }
                    if (!any) continue;
                    R->edges.push_back(vid[vox(i, j, k)]);
                    R->edges.push_back(vid[vox(w2[0], w2[1], w2[2])]);
                    R->em.push_back(m);
                }
            }
    // 5) triangulate each valid face (util::simpleTriangulate, geomalgo.cpp:13-34):
    // quad [q0,q1,q2,q3] -> (q3,q0,q1), (q3,q1,q2); the new diagonal (q1,q3)
    // is appended to the edge list with the face measure (voroinfo.cpp:688-710).
    for (size_t f = 0; f < face_p.size(); ++f) {
        int64_t p[3], v[3];
        decode(face_p[f], p);
        int32_t q[4];
        for (int m = 0; m < 4; ++m) {
            quad_voxel(p, face_d[f], m, v);
            q[m] = vid[vox(v[0], v[1], v[2])];
        }
        const int32_t t0[3] = {q[3], q[0], q[1]}, t1[3] = {q[3], q[1], q[2]};
        for (int m = 0; m < 3; ++m) R->tris.push_back(t0[m]);
        for (int m = 0; m < 3; ++m) R->tris.push_back(t1[m]);
        R->fm.push_back(face_l[f]);
        R->fm.push_back(face_l[f]);
        R->tri_face.push_back((int32_t)f);
        R->tri_face.push_back((int32_t)f);
        int32_t a, b;
        make_edge(q[1], q[3], a, b);
        R->edges.push_back(a);
        R->edges.push_back(b);
        R->em.push_back(face_l[f]);
    }
    return R;
}

void vco_lattice_vd_counts(const uint8_t* occ, int X, int Y, int Z, const int32_t* ft_id, long long* sizes,
                           float* inside_size) {
    // The sizes vco_lattice_vd gives -- vertices, edges (axis edges, then one
    // diagonal per face), triangles, faces -- and the inside size, counted by
    // the same validity rules without building the complex: for volumes whose
    // complex does not fit in host memory (the 1024^3 random field).
    const int64_t NB = Y + 1, NC = Z + 1;
    const int64_t NV = (int64_t)X * Y * Z;
    auto vox = [&](int64_t i, int64_t j, int64_t k) { return (i * Y + j) * Z + k; };
    auto inside = [&](int64_t i, int64_t j, int64_t k) { return occ_at(occ, X, Y, Z, (int)i, (int)j, (int)k) == 1; };
    auto lid = [&](int64_t a, int64_t b, int64_t c) { return (a * NB + b) * NC + c; };
    auto cand = [&](int64_t a, int64_t b, int64_t c, int d) -> bool {
        int64_t e[3] = {a, b, c};
        e[d] += 1;
        if (a < 0 || b < 0 || c < 0 || e[0] > X || e[1] > Y || e[2] > Z) return false;
        const int32_t i0 = ft_id[lid(a, b, c)], i1 = ft_id[lid(e[0], e[1], e[2])];
        return i0 >= 0 && i1 >= 0 && i0 != i1;
    };
    const int qs[4] = {0, 1, 1, 0}, qt[4] = {0, 0, 1, 1};
    // vertices: inside voxels at a corner of a candidate face; faces: the
    // candidates whose four voxels are all inside
    std::vector<uint8_t> vtx((size_t)NV, 0);
    long long nface = 0;
    for (int64_t a = 0; a <= X; ++a)
        for (int64_t b = 0; b <= Y; ++b)
            for (int64_t c = 0; c <= Z; ++c)
                for (int d = 0; d < 3; ++d) {
                    if (!cand(a, b, c, d)) continue;
                    const int u = (d + 1) % 3, w = (d + 2) % 3;
                    const int64_t p[3] = {a, b, c};
                    bool all = true;
                    for (int q = 0; q < 4; ++q) {
                        int64_t v[3];
                        v[d] = p[d];
                        v[u] = p[u] - 1 + qs[q];
                        v[w] = p[w] - 1 + qt[q];
                        if (inside(v[0], v[1], v[2])) vtx[(size_t)vox(v[0], v[1], v[2])] = 1;
                        else all = false;
                    }
                    if (all) ++nface;
                }
    long long nv = 0;
    int64_t lo[3] = {INT64_MAX, INT64_MAX, INT64_MAX}, hi[3] = {-1, -1, -1};
    for (int64_t i = 0; i < X; ++i)
        for (int64_t j = 0; j < Y; ++j)
            for (int64_t k = 0; k < Z; ++k) {
                if (!vtx[(size_t)vox(i, j, k)]) continue;
                ++nv;
                const int64_t pc[3] = {i, j, k};
                for (int m = 0; m < 3; ++m) {
                    lo[m] = std::min(lo[m], pc[m]);
                    hi[m] = std::max(hi[m], pc[m]);
                }
            }
    // axis edges: both voxels vertices and a candidate lattice edge among the
    // four bounding the plaquette the two voxels share
    long long naxis = 0;
    const int64_t dims[3] = {X, Y, Z};
    for (int64_t i = 0; i < X; ++i)
        for (int64_t j = 0; j < Y; ++j)
            for (int64_t k = 0; k < Z; ++k) {
                if (!vtx[(size_t)vox(i, j, k)]) continue;
                for (int d = 0; d < 3; ++d) {
                    int64_t n2[3] = {i, j, k};
                    n2[d] += 1;
                    if (n2[d] >= dims[d] || !vtx[(size_t)vox(n2[0], n2[1], n2[2])]) continue;
                    const int u = (d + 1) % 3, w = (d + 2) % 3;
                    int64_t c0[3] = {i, j, k};
                    c0[d] += 1;
                    int64_t cu[3] = {c0[0], c0[1], c0[2]}, cw[3] = {c0[0], c0[1], c0[2]};
                    cw[w] += 1;  // corner + e_w: lattice edge along u
                    cu[u] += 1;  // corner + e_u: lattice edge along w
                    if (cand(c0[0], c0[1], c0[2], u) || cand(cw[0], cw[1], cw[2], u) || cand(c0[0], c0[1], c0[2], w) ||
                        cand(cu[0], cu[1], cu[2], w))
                        ++naxis;
                }
            }
    sizes[0] = nv;
    sizes[1] = naxis + nface;
    sizes[2] = 2 * nface;
    sizes[3] = nface;
    *inside_size = nv ? (float)std::max(hi[0] - lo[0], std::max(hi[1] - lo[1], hi[2] - lo[2])) : 0.0f;
}

void vco_vd_sizes(void* h, long long* nv, long long* ne, long long* nt, long long* nface, float* inside_size) {
    auto* R = static_cast<VD*>(h);
    *nv = (long long)R->vts.size() / 3;
    *ne = (long long)R->edges.size() / 2;
    *nt = (long long)R->tris.size() / 3;
    *nface = R->nface;
    *inside_size = R->inside_size;
}

void vco_vd_get(void* h, float* vts, int32_t* edges, int32_t* tris, float* vm, float* em, float* fm,
                int32_t* tri_face, int32_t* face_sites) {
    auto* R = static_cast<VD*>(h);
    auto cp = [](auto* dst, const auto& v) {
        if (dst && !v.empty()) std::memcpy(dst, v.data(), v.size() * sizeof(v[0]));
    };
    cp(vts, R->vts);
    cp(edges, R->edges);
    cp(tris, R->tris);
    cp(vm, R->vm);
    cp(em, R->em);
    cp(fm, R->fm);
    cp(tri_face, R->tri_face);
    cp(face_sites, R->face_sites);
}

void vco_vd_radius(void* h, float* radius) {
    auto* R = static_cast<VD*>(h);
    if (radius && !R->radius.empty()) std::memcpy(radius, R->radius.data(), R->radius.size() * sizeof(float));
}

void vco_vd_free(void* h) { delete static_cast<VD*>(h); }

long long vco_finalize(long long nv, long long ne, const int32_t* edges, long long nt, const int32_t* tris,
                       int32_t* edges_out, int32_t* tri_edges, int32_t* ve_off, int32_t* ve_ids, int32_t* ef_off,
                       int32_t* ef_ids) {
    Fin F;
    finalize(nv, ne, edges, nt, tris, F, ve_off || ve_ids || ef_off || ef_ids);
    auto cp = [](int32_t* dst, const std::vector<int32_t>& v) {
        if (dst && !v.empty()) std::memcpy(dst, v.data(), v.size() * sizeof(int32_t));
    };
    cp(edges_out, F.edges);
    cp(tri_edges, F.tri_edges);
    cp(ve_off, F.ve_off);
    cp(ve_ids, F.ve_ids);
    cp(ef_off, F.ef_off);
    cp(ef_ids, F.ef_ids);
    return (long long)F.edges.size() / 2;
}

int vco_thin(long long nv, long long ne, const int32_t* edges, long long nt, const int32_t* tris, const float* em,
             const float* fm, float f_t, float l_t, uint8_t* keep_v, uint8_t* keep_e, uint8_t* keep_f,
             uint8_t* removed_e, long long* stats) {
    Fin F;
    finalize(nv, ne, edges, nt, tris, F);
    const long long E = (long long)F.edges.size() / 2;
    std::vector<uint8_t> rm_v((size_t)nv, 0), rm_e((size_t)E, 0), rm_f((size_t)nt, 0);
    std::vector<int32_t> ref_v((size_t)nv), ref_e((size_t)E);
    for (long long v = 0; v < nv; ++v) ref_v[v] = F.ve_off[v + 1] - F.ve_off[v];
    for (long long e = 0; e < E; ++e) ref_e[e] = F.ef_off[e + 1] - F.ef_off[e];
    // Queue item: type 1 = face-edge pair (idx0 face, idx1 edge), type 0 =
    // edge-vertex pair (idx0 edge, idx1 vertex) (ccthin.h:22-54).
    struct Item {
        int8_t type;
        int32_t i0, i1;
        int32_t gen;
    };
    std::deque<Item> q;
    long long pushes = 0, done = 0, skipped = 0;
    int32_t max_gen = -1;
    auto below_e = [&](int32_t e) { return em[e] < l_t; };  // ccthin.cpp:514-518
    auto below_f = [&](int32_t f) { return fm[f] < f_t; };  // ccthin.cpp:520-527 (no face is ever marked)
    // Seed: face-edge pairs in edge order, then edge-vertex pairs in vertex
    // order (ccthin.cpp:248-270).
    for (long long e = 0; e < E; ++e)
        if (ref_e[e] == 1) {
            int32_t f = F.ef_ids[F.ef_off[e]];
            if (below_f(f)) { q.push_back({1, f, (int32_t)e, 0}); ++pushes; }
        }
    for (long long v = 0; v < nv; ++v)
        if (ref_v[v] == 1) {
            int32_t e = F.ve_ids[F.ve_off[v]];
            if (below_e(e)) { q.push_back({0, e, (int32_t)v, 0}); ++pushes; }
        }
    // FIFO collapse (ccthin.cpp:529-771).
    while (!q.empty()) {
        Item it = q.front();
        q.pop_front();
        max_gen = std::max(max_gen, it.gen);
        bool gone = it.type == 1 ? rm_f[it.i0] : rm_e[it.i0];
        if (gone) { ++skipped; continue; }
        if (!((it.type == 1 && ref_e[it.i1] == 1) || (it.type == 0 && ref_v[it.i1] == 1))) return -1;
        ++done;
        if (it.type == 0) {
            rm_e[it.i0] = 1;
            rm_v[it.i1] = 1;
            int32_t a = F.edges[2 * it.i0], b = F.edges[2 * it.i0 + 1];
            ref_v[a]--;
            ref_v[b]--;
            int32_t other = a != it.i1 ? a : b;
            if (ref_v[other] == 1) {
                for (int32_t k = F.ve_off[other]; k < F.ve_off[other + 1]; ++k) {
                    int32_t ne2 = F.ve_ids[k];
                    if (!rm_e[ne2]) {
                        if (below_e(ne2)) { q.push_back({0, ne2, other, it.gen + 1}); ++pushes; }
                        break;
                    }
                }
            }
        } else {
            rm_f[it.i0] = 1;
            rm_e[it.i1] = 1;
            ref_e[it.i1]--;
            for (int s = 0; s < 3; ++s) {
                int32_t e = F.tri_edges[3 * it.i0 + s];
                if (rm_e[e]) continue;
                ref_e[e]--;
                if (ref_e[e] == 1) {
                    for (int32_t k = F.ef_off[e]; k < F.ef_off[e + 1]; ++k) {
                        int32_t nf = F.ef_ids[k];
                        if (!rm_f[nf]) {
                            if (below_f(nf)) { q.push_back({1, nf, e, it.gen + 1}); ++pushes; }
                            break;
                        }
                    }
                }
            }
            for (int s = 0; s < 2; ++s) {
                int32_t v = F.edges[2 * it.i1 + s];
                ref_v[v]--;
                if (ref_v[v] == 1) {
                    for (int32_t k = F.ve_off[v]; k < F.ve_off[v + 1]; ++k) {
                        int32_t ne2 = F.ve_ids[k];
                        if (!rm_e[ne2]) {
                            if (below_e(ne2)) { q.push_back({0, ne2, v, it.gen + 1}); ++pushes; }
                            break;
                        }
                    }
                }
            }
        }
    }
    for (long long v = 0; v < nv; ++v) keep_v[v] = rm_v[v] ? 0 : 1;
    for (long long e = 0; e < E; ++e) {
        keep_e[e] = (!rm_e[e] && ref_e[e] == 0) ? 1 : 0;  // getRemainedEdges (ccthin.cpp:156-166)
        if (removed_e) removed_e[e] = rm_e[e];
    }
    for (long long f = 0; f < nt; ++f) keep_f[f] = rm_f[f] ? 0 : 1;
    if (stats) {
        stats[0] = pushes;
        stats[1] = done;
        stats[2] = skipped;
        stats[3] = max_gen + 1;
    }
    return 0;
}

void vco_remaining(long long nv, const float* vts, long long ne_fin, const int32_t* edges_fin, long long nt,
                   const int32_t* tris, const uint8_t* keep_v, const uint8_t* keep_e, const uint8_t* keep_f,
                   long long* nv_out, long long* ne_out, long long* nt_out, float* vts_out, int32_t* edges_out,
                   int32_t* tris_out) {
    // remainingCC (ccthin.cpp:467-512): surviving edges in id order; every
    // surviving triangle re-triangulated by simpleTriangulate, which turns
    // (a,b,c) into (c,a,b); surviving vertices in id order; then
    // util::compactify renames vertex ids (geomalgo.cpp:215-235).
    std::vector<int32_t> newid((size_t)nv, 0);
    long long cv = 0, ce = 0, ct = 0;
    for (long long v = 0; v < nv; ++v)
        if (keep_v[v]) {
            if (vts_out)
                for (int k = 0; k < 3; ++k) vts_out[3 * cv + k] = vts[3 * v + k];
            newid[v] = (int32_t)cv++;
        }
    for (long long e = 0; e < ne_fin; ++e)
        if (keep_e[e]) {
            if (edges_out) {
                edges_out[2 * ce] = newid[edges_fin[2 * e]];
                edges_out[2 * ce + 1] = newid[edges_fin[2 * e + 1]];
            }
            ++ce;
        }
    for (long long f = 0; f < nt; ++f)
        if (keep_f[f]) {
            if (tris_out) {
                tris_out[3 * ct + 0] = newid[tris[3 * f + 2]];
                tris_out[3 * ct + 1] = newid[tris[3 * f + 0]];
                tris_out[3 * ct + 2] = newid[tris[3 * f + 1]];
            }
            ++ct;
        }
    *nv_out = cv;
    *ne_out = ce;
    *nt_out = ct;
}

void vco_euler(long long nv, long long ne, const int32_t* edges, long long nt, const int32_t* tris, long long* out) {
    // util::computeEulerChar(vts, edges, tris) (geomalgo.cpp:181-214): the
    // given edges (as ordered pairs) together with the triangles' sides (made
    // with makeEdge), vertex count = all given vertices, components by BFS.
    std::unordered_set<uint64_t> ue;
    ue.reserve((size_t)(ne + 3 * nt) * 2 + 16);
    for (long long e = 0; e < ne; ++e) ue.insert(ekey(edges[2 * e], edges[2 * e + 1]));
    for (long long f = 0; f < nt; ++f)
        for (int s = 0; s < 3; ++s) {
            int32_t a, b;
            make_edge(tris[3 * f + s], tris[3 * f + (s + 1) % 3], a, b);
            ue.insert(ekey(a, b));
        }
    // union-find for the component count (same count as the reference's BFS)
    std::vector<int64_t> par((size_t)nv);
    for (long long v = 0; v < nv; ++v) par[v] = v;
    auto find = [&](int64_t x) {
        while (par[x] != x) { par[x] = par[par[x]]; x = par[x]; }
        return x;
    };
    for (uint64_t k : ue) {
        int64_t a = (int64_t)(k >> 32), b = (int64_t)(k & 0xffffffffULL);
        a = find(a);
        b = find(b);
        if (a != b) par[a] = b;
    }
    long long C = 0;
    for (long long v = 0; v < nv; ++v)
        if (find(v) == v) ++C;
    out[0] = nv;
    out[1] = (long long)ue.size();
    out[2] = nt;
    out[3] = C;
    out[4] = nv - (long long)ue.size() + nt;
}

}  // extern "C"

long long vco_closed_components(long long nv, long long ne, const int32_t* edges, long long nt, const int32_t* tris) {
    Fin F;
    finalize(nv, ne, edges, nt, tris, F);
    const long long E = (long long)F.edges.size() / 2;
    // every measure 0, thresholds 1: every pair passes the filter
    std::vector<float> em((size_t)E, 0.0f), fm((size_t)nt, 0.0f);
    std::vector<uint8_t> kv((size_t)nv), ke((size_t)E), kf((size_t)nt), re((size_t)E);
    if (vco_thin(nv, ne, edges, nt, tris, em.data(), fm.data(), 1.0f, 1.0f, kv.data(), ke.data(), kf.data(),
                 re.data(), nullptr) != 0)
        return -1;
    // breadth-first over the remaining faces, through their sides
    std::vector<uint8_t> seen_f((size_t)nt, 0), seen_e((size_t)E, 0);
    std::vector<int32_t> stack;
    long long ncc = 0;
    for (long long f0 = 0; f0 < nt; ++f0) {
        if (!kf[f0] || seen_f[f0]) continue;
        ++ncc;
        seen_f[f0] = 1;
        stack.assign(1, (int32_t)f0);
        while (!stack.empty()) {
            const int32_t f = stack.back();
            stack.pop_back();
            for (int s = 0; s < 3; ++s) {
                const int32_t e = F.tri_edges[3 * f + s];
                if (seen_e[e]) continue;
                seen_e[e] = 1;
                for (int32_t k = F.ef_off[e]; k < F.ef_off[e + 1]; ++k) {
                    const int32_t g = F.ef_ids[k];
                    if (kf[g] && !seen_f[g]) {
                        seen_f[g] = 1;
                        stack.push_back(g);
                    }
                }
            }
        }
    }
    return ncc;
}

// start: the byte of R (0 in .sof, 128 in .sog); leaf_extra: bytes after a
// leaf's corner byte (0 in .sof, 12 in .sog: its feature point, read and
// dropped by read_sog_file, octree.cpp:403-410)
static int octree_decode(const uint8_t* b, long long nbytes, long long start, int leaf_extra, int* size_out,
                         uint8_t* occ, float* sites, long long* nsites) {
    if (nbytes < start + 4) return -1;
    int32_t R = 0;
    std::memcpy(&R, b + start, 4);
    if (R < 1 || (R & (R - 1)) != 0 || R > 16384) return -1;
    const long long S = (long long)R + 1;
    std::vector<uint8_t> cell;
    if (occ) cell.assign((size_t)R * R * R, 0);
    long long pos = start + 4, ns = 0;
    bool ok = true;
    std::function<void(int, int, int, int)> node = [&](int x, int y, int z, int len) {
        if (!ok || pos >= nbytes) {
            ok = false;
            return;
        }
        const uint8_t type = b[pos++];
        if (type == 2) {  // leaf: one cell
            if (len != 1 || pos >= nbytes) {
                ok = false;
                return;
            }
            const uint8_t v = b[pos++];
            if (nbytes - pos < leaf_extra) {
                ok = false;
                return;
            }
            pos += leaf_extra;
            if (occ) cell[((size_t)x * R + y) * R + z] = v;
            if (v != 0x00 && v != 0xFF) {
                if (sites) {
                    sites[3 * ns + 0] = (float)x + 0.5f;
                    sites[3 * ns + 1] = (float)y + 0.5f;
                    sites[3 * ns + 2] = (float)z + 0.5f;
                }
                ++ns;
            }
        } else if (type == 1) {  // empty: one sign for the whole cube
            if (pos >= nbytes) {
                ok = false;
                return;
            }
            const uint8_t v = b[pos++] == 1 ? 0xFF : 0x00;
            if (occ)
                for (int i = 0; i < len; ++i)
                    for (int j = 0; j < len; ++j)
                        for (int k = 0; k < len; ++k) cell[((size_t)(x + i) * R + (y + j)) * R + (z + k)] = v;
        } else if (type == 0) {  // internal: eight children
            if (len < 2) {
                ok = false;
                return;
            }
            const int h = len / 2;
            for (int i = 0; i < 2; ++i)
                for (int j = 0; j < 2; ++j)
                    for (int k = 0; k < 2; ++k) node(x + i * h, y + j * h, z + k * h, h);
        } else {
            ok = false;
        }
    };
    node(0, 0, 0, R);
    if (!ok) return -1;
    *size_out = (int)S;
    *nsites = ns;
    if (occ)
        for (long long x = 0; x < S; ++x)
            for (long long y = 0; y < S; ++y)
                for (long long z = 0; z < S; ++z) {
                    const int off = (x == R ? 4 : 0) | (y == R ? 2 : 0) | (z == R ? 1 : 0);
                    const long long cx = x == R ? R - 1 : x, cy = y == R ? R - 1 : y, cz = z == R ? R - 1 : z;
                    const uint8_t v = cell[((size_t)cx * R + cy) * R + cz];
                    occ[(x * S + y) * S + z] = ((v >> off) & 1) == 0 ? 1 : 0;
                }
    return 0;
}

int vco_sof_decode(const uint8_t* b, long long nbytes, int* size_out, uint8_t* occ, float* sites,
                   long long* nsites) {
    return octree_decode(b, nbytes, 0, 0, size_out, occ, sites, nsites);
}

// read_sog_file (octree.cpp:351-498): the 128-byte header (title "SOG.Format
// 1.0" and its terminator, lower-left corner, bounding-box length), then R
// and the nodes; a stream without the title is rejected
int vco_sog_decode(const uint8_t* b, long long nbytes, int* size_out, uint8_t* occ, float* sites,
                   long long* nsites) {
    if (nbytes < 128 || std::memcmp(b, "SOG.Format 1.0", 15) != 0) return -1;
    return octree_decode(b, nbytes, 128, 12, size_out, occ, sites, nsites);
}

// ---------------------------------------------------------------------------
// Output formats: the files written for the remaining complex after thinning
// (highlevelalgo.cpp:855-955).  Written with the same stream facilities the
// reference uses (std::ofstream with its default formatting, or stdio for the
// ply library), one value at a time.

#include <fstream>

// writeToDotma (exporters.cpp:244-287)
extern "C" int vco_write_dotma(const char* path, const float* vts, const float* radii, long long nv,
                               const int32_t* edges, long long ne, const int32_t* tris, long long nt) {
    std::ofstream f(path);
    if (!f.is_open()) return 1;
    f << (unsigned long)nv << " " << (unsigned long)ne << " " << (unsigned long)nt << std::endl;
    for (long long k = 0; k < nv; ++k)
        f << "v " << vts[3 * k] << " " << vts[3 * k + 1] << " " << vts[3 * k + 2] << " " << radii[k] << std::endl;
    for (long long k = 0; k < ne; ++k) f << "e " << edges[2 * k] << " " << edges[2 * k + 1] << std::endl;
    for (long long k = 0; k < nt; ++k)
        f << "f " << (unsigned)tris[3 * k] << " " << (unsigned)tris[3 * k + 1] << " " << (unsigned)tris[3 * k + 2]
          << std::endl;
    return f.good() ? 0 : 1;
}

// writeRadiiToFile (exporters.cpp:478-552), the branch with the remaining
// vertex ids, identity voxel-to-model matrix: r = len((r, 0, 0))
extern "C" int vco_write_radii(const char* path, const float* vts, const float* radii, long long n) {
    std::ofstream f(path);
    if (!f.is_open()) return 1;
    f << (unsigned long)n << std::endl;
    for (long long k = 0; k < n; ++k) {
        float r = radii[k];
        r = std::sqrt(r * r + 0.0f * 0.0f + 0.0f * 0.0f);
        f << vts[3 * k] << " " << vts[3 * k + 1] << " " << vts[3 * k + 2] << " " << r << std::endl;
    }
    return f.good() ? 0 : 1;
}

// ply::PLYWriter::write (plyall.cpp:98-171) through the ply library's ASCII
// writer (Greg Turk's ply.c, 1998 revision: the reference's 3rdparty/ply
// submodule, not vendored): header_complete_ply, then put_element_ply per
// element -- write_ascii_item prints "%g " for floats, "%d " for ints, "%u "
// for the uchar list count, and each element ends with "\n".
extern "C" int vco_write_ply(const char* path, const float* vts, long long nv, const int32_t* edges, long long ne,
                             const int32_t* tris, long long nt) {
    FILE* f = std::fopen(path, "w");
    if (!f) return 1;
    std::fprintf(f, "ply\nformat ascii 1.0\ncomment Generated by VoxelCore\n");
    std::fprintf(f, "element vertex %lld\n", nv);
    for (const char* p : {"x", "y", "z"}) std::fprintf(f, "property float32 %s\n", p);
    std::fprintf(f, "element edge %lld\n", ne);
    for (const char* p : {"vertex1", "vertex2"}) std::fprintf(f, "property int32 %s\n", p);
    std::fprintf(f, "element face %lld\n", nt);
    std::fprintf(f, "property list uint8 int32 vertex_indices\n");
    std::fprintf(f, "end_header\n");
    for (long long k = 0; k < nv; ++k) {
        for (int d = 0; d < 3; ++d) std::fprintf(f, "%g ", (double)vts[3 * k + d]);
        std::fprintf(f, "\n");
    }
    for (long long k = 0; k < ne; ++k) {
        for (int d = 0; d < 2; ++d) std::fprintf(f, "%d ", edges[2 * k + d]);
        std::fprintf(f, "\n");
    }
    for (long long k = 0; k < nt; ++k) {
        std::fprintf(f, "%u ", 3u);
        for (int d = 0; d < 3; ++d) std::fprintf(f, "%d ", tris[3 * k + d]);
        std::fprintf(f, "\n");
    }
    return std::fclose(f) == 0 ? 0 : 1;
}

// The .ma edge list (highlevelalgo.cpp:911-945): the remaining edges, then
// each remaining triangle's edges (util::makeEdgesFromTri: (t0,t1), (t1,t2),
// (t2,t0), each as (min, max)) through an unordered_set with ivec2Hash
// (commondefs.h:30-43), appended in the set's iteration order.  Returns the
// number of edges; out (2 ints per edge) may be null.
namespace {
struct OEdge {
    int a, b;
    bool operator==(const OEdge& o) const { return a == o.a && b == o.b; }
};
struct OEdgeHash {
    size_t operator()(const OEdge& e) const {
        size_t h = 0;
        h = ((h << 5) - h) + std::hash<int>()(e.a);
        h = ((h << 5) - h) + std::hash<int>()(e.b);
        return h;
    }
};
}  // namespace

extern "C" long long vco_dotma_edges(const int32_t* edges, long long ne, const int32_t* tris, long long nt,
                                     int32_t* out) {
    std::vector<OEdge> all;
    for (long long k = 0; k < ne; ++k) all.push_back(OEdge{edges[2 * k], edges[2 * k + 1]});
    std::unordered_set<OEdge, OEdgeHash> unique;
    for (long long k = 0; k < nt; ++k)
        for (int d = 0; d < 3; ++d) {
            const int i = tris[3 * k + d], j = tris[3 * k + (d + 1) % 3];
            unique.insert(i > j ? OEdge{j, i} : OEdge{i, j});
        }
    all.insert(all.end(), unique.begin(), unique.end());
    if (out)
        for (size_t k = 0; k < all.size(); ++k) {
            out[2 * k] = all[k].a;
            out[2 * k + 1] = all[k].b;
        }
    return (long long)all.size();
}
