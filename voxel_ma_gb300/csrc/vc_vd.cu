// Lattice Voronoi complex of the sites, inside part, with lambda measures.
//
// The feature transform labels every corner-lattice point with its nearest
// site.  Wherever the two ends of a lattice edge carry different labels, the
// Voronoi boundary between those two sites crosses the edge; the dual square
// of that edge (its four surrounding voxel centres) is taken as a piece of
// the Voronoi face between the two sites.  From this complex the kernels
// below produce exactly what VoroInfo::extractInsideWithMeasure
// (src/voroinfo.cpp:624-729) produces for a Voronoi diagram:
//   * vertices: voxel centres that are corners of some Voronoi face and lie
//     in an inside voxel (tagVert, voroinfo.cpp:447-454: round to the nearest
//     voxel and test occupancy), in voxel order;
//   * edges: sides of Voronoi faces with both ends valid
//     (voroinfo_imp.h:22-25), in (lower voxel, axis) order, then the new
//     triangulation diagonals in face order (voroinfo.cpp:688-710);
//   * faces: Voronoi faces with all four vertices valid (voroinfo_imp.h:
//     35-41), in (lattice point, axis) order, each split by
//     util::simpleTriangulate into (q3,q0,q1), (q3,q1,q2) (geomalgo.cpp:13-34);
//   * measures: face lambda = distance between its two sites
//     (measureforMA_imp.h:1-4), edge lambda = max over incident valid faces
//     (0 if none), vertex lambda = max over valid faces through the vertex,
//     diagonal edges and both triangles take the face's lambda
//     (voroinfo.cpp:1432-1574).
// Since every triangle side is in the edge list, cellcomplex::finalize
// (cellcomplex.cpp:364-491) adds no edge and the complex is finalized by
// building its adjacency lists.
#include "vc_internal.cuh"

namespace vc {

namespace {

struct Grid {
    const uint8_t* occ;
    const int32_t* lab;
    int X, Y, Z;
    int64_t NB, NC;
    __device__ __forceinline__ bool inside(int i, int j, int k) const {
        if (i < 0 || j < 0 || k < 0 || i >= X || j >= Y || k >= Z) return false;
        return occ[((int64_t)i * Y + j) * Z + k] > 0;
    }
    __device__ __forceinline__ int64_t lid(int a, int b, int c) const { return ((int64_t)a * NB + b) * NC + c; }
    __device__ __forceinline__ int32_t label(int a, int b, int c) const { return lab[lid(a, b, c)]; }
};

// The grid of volume bv of the batch: its voxels and its lattice labels
// (labels are batch-wide site indices, so they index the batch's site list).
__device__ __forceinline__ Grid grid_of(const VolTab& T, int bv, const uint8_t* occ, const int32_t* lab) {
    const int4 d = T.dim(bv);
    return Grid{occ + T.start(kVox, bv), lab + T.start(kLat, bv), d.x, d.y, d.z, (int64_t)d.y + 1, (int64_t)d.z + 1};
}


// Lattice coordinates of point p (the lattice has fewer than 2^32 points).
__device__ __forceinline__ void decode32(int64_t p, int64_t NB, int64_t NC, int& a, int& b, int& c) {
    const uint32_t q = (uint32_t)p, nc = (uint32_t)NC, nb = (uint32_t)NB;
    const uint32_t r = q / nc;
    c = (int)(q - r * nc);
    a = (int)(r / nb);
    b = (int)(r - (uint32_t)a * nb);
}

// quad vertex m of the dual square of lattice edge (a,b,c)+axis d
__device__ __forceinline__ void quad_voxel(int a, int b, int c, int d, int m, int& i, int& j, int& k) {
    const int s = (m == 1 || m == 2) ? 1 : 0;
    const int t = (m >= 2) ? 1 : 0;
    int p[3] = {a, b, c};
    const int u = (d + 1) % 3, w = (d + 2) % 3;
    int v[3];
    v[d] = p[d];
    v[u] = p[u] - 1 + s;
    v[w] = p[w] - 1 + t;
    i = v[0];
    j = v[1];
    k = v[2];
}

__device__ __forceinline__ float lambda_of(const float* __restrict__ sxyz, int32_t s0, int32_t s1) {
    const float dx = sxyz[3 * (int64_t)s0 + 0] - sxyz[3 * (int64_t)s1 + 0];
    const float dy = sxyz[3 * (int64_t)s0 + 1] - sxyz[3 * (int64_t)s1 + 1];
    const float dz = sxyz[3 * (int64_t)s0 + 2] - sxyz[3 * (int64_t)s1 + 2];
    float s = 0.0f;
    s = __fadd_rn(s, __fmul_rn(dx, dx));
    s = __fadd_rn(s, __fmul_rn(dy, dy));
    s = __fadd_rn(s, __fmul_rn(dz, dz));
    return __fsqrt_rn(s);
}

// Face validity of lattice edge (a,b,c)+d: labels differ and the 4 voxels are inside.
__device__ __forceinline__ bool face_valid(const Grid& g, int a, int b, int c, int d) {
    int e[3] = {a, b, c};
    e[d] += 1;
    if (e[0] > g.X || e[1] > g.Y || e[2] > g.Z) return false;
    const int32_t l0 = g.label(a, b, c), l1 = g.label(e[0], e[1], e[2]);
    if (l0 < 0 || l1 < 0 || l0 == l1) return false;
#pragma unroll
    for (int m = 0; m < 4; ++m) {
        int i, j, k;
        quad_voxel(a, b, c, d, m, i, j, k);
        if (!g.inside(i, j, k)) return false;
    }
    return true;
}

// flags: bits 0-2 valid face along axis d; bit 3 vertex; bits 4-6 valid edge
// along d.  lam[3p+d]: lambda of the valid face (p, d), computed once here.
// One block per lattice row along z (volume bv, a, b) of the batch.
__global__ void vd_flags_kernel(const uint8_t* __restrict__ occ, const int32_t* __restrict__ lab, VolTab T,
                                const float* __restrict__ sxyz, uint8_t* __restrict__ flags_all,
                                float* __restrict__ lam_all) {
    const int64_t nrows = T.total(kLRow);
    for (int64_t grow = blockIdx.x; grow < nrows; grow += gridDim.x) {
        const int bv = T.find(kLRow, grow);
        const Grid g = grid_of(T, bv, occ, lab);
        const int64_t lat0 = T.start(kLat, bv);
        uint8_t* flags = flags_all + lat0;
        float* lam = lam_all + 3 * lat0;
        const int64_t row = grow - T.start(kLRow, bv);
        const int a = (int)(row / g.NB), b = (int)(row - (int64_t)a * g.NB);
        for (int c = threadIdx.x; c < (int)g.NC; c += blockDim.x) {
            const int64_t p = row * g.NC + c;
            uint32_t f = 0;
            float l3[3] = {0.0f, 0.0f, 0.0f};
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                if (face_valid(g, a, b, c, d)) {
                    f |= 1u << d;
                    int e[3] = {a, b, c};
                    e[d] += 1;
                    l3[d] = lambda_of(sxyz, g.lab[p], g.label(e[0], e[1], e[2]));
                }
            }
            if (a < g.X && b < g.Y && c < g.Z && g.inside(a, b, c)) {
                int32_t L[8];
#pragma unroll
                for (int q = 0; q < 8; ++q) L[q] = g.label(a + ((q >> 2) & 1), b + ((q >> 1) & 1), c + (q & 1));
                bool alleq = true;
#pragma unroll
                for (int q = 1; q < 8; ++q) alleq &= (L[q] == L[0]);
                if (!alleq) {
                    f |= 8u;
#pragma unroll
                    for (int d = 0; d < 3; ++d) {
                        const int ni = a + (d == 0), nj = b + (d == 1), nk = c + (d == 2);
                        if (!g.inside(ni, nj, nk)) continue;
                        const int bit = 1 << (2 - d);  // corner offset bit of axis d: x->4, y->2, z->1
                        int32_t ref = -2;
                        bool eq = true;
#pragma unroll
                        for (int q = 0; q < 8; ++q) {
                            if (!(q & bit)) continue;
                            if (ref == -2) ref = L[q];
                            else eq &= (L[q] == ref);
                        }
                        if (!eq) f |= 16u << d;
                    }
                }
            }
            flags[p] = (uint8_t)f;
            lam[3 * p + 0] = l3[0];
            lam[3 * p + 1] = l3[1];
            lam[3 * p + 2] = l3[2];
        }
    }
}

__device__ __forceinline__ int32_t rank_below(uint32_t bits, int d) { return __popc(bits & ((1u << d) - 1u)); }

// Valid faces incident to the axis edge (voxel (a,b,c), axis d): the lattice
// edges of the plaquette shared by the voxel and its +d neighbour.  For each,
// the lattice point, its axis and which of the face's two triangles carries
// the edge (0: (q3,q0,q1), 1: (q3,q1,q2)).
struct Inc {
    int64_t lp;
    int axis;
    int tri;
};
__device__ __forceinline__ int plaquette_faces(const Grid& g, const uint8_t* __restrict__ flags, int a, int b, int c,
                                               int d, Inc out[4]) {
    const int u = (d + 1) % 3, w = (d + 2) % 3;
    const int v[3] = {a, b, c};
    int nb[3] = {a, b, c};
    nb[d] += 1;
    int k = 0;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        // j < 2: lattice edge along u from nb + j e_w; j >= 2: along w from nb + (j-2) e_u
        int cc[3] = {nb[0], nb[1], nb[2]};
        const int ax = j < 2 ? u : w;
        if (j < 2) cc[w] += j;
        else cc[u] += j - 2;
        const int64_t lp = g.lid(cc[0], cc[1], cc[2]);
        if (!(flags[lp] & (1u << ax))) continue;
        // position (s,t) of the edge's lower voxel in the face's quad
        const int u2 = (ax + 1) % 3, w2 = (ax + 2) % 3;
        const int s = v[u2] - (cc[u2] - 1), t = v[w2] - (cc[w2] - 1);
        const int tri = d == u2 ? (t == 0 ? 0 : 1) : (s == 0 ? 0 : 1);
        out[k++] = Inc{lp, ax, tri};
    }
    return k;
}

// Per lattice point: 1 if vertex; edges; faces; E->F entries of its axis
// edges; V->E entries of its vertex.
__global__ void vd_counts_kernel(const uint8_t* __restrict__ occ, const int32_t* __restrict__ lab, VolTab T,
                                 const uint8_t* __restrict__ flags_all, int32_t* __restrict__ cv_all,
                                 int32_t* __restrict__ ce_all, int32_t* __restrict__ cf_all,
                                 int32_t* __restrict__ cef_all, int32_t* __restrict__ cve_all) {
    const int64_t nrows = T.total(kLRow);
    for (int64_t grow = blockIdx.x; grow < nrows; grow += gridDim.x) {
        const int bv = T.find(kLRow, grow);
        const Grid g = grid_of(T, bv, occ, lab);
        const int64_t lat0 = T.start(kLat, bv);
        const uint8_t* flags = flags_all + lat0;
        int32_t *cv = cv_all + lat0, *ce = ce_all + lat0, *cf = cf_all + lat0, *cef = cef_all + lat0,
                *cve = cve_all + lat0;
        const int64_t row = grow - T.start(kLRow, bv);
        const int a = (int)(row / g.NB), b = (int)(row - (int64_t)a * g.NB);
        for (int c = threadIdx.x; c < (int)g.NC; c += blockDim.x) {
            const int64_t p = row * g.NC + c;
            const uint32_t fl = flags[p];
            int nef = 0, nve = 0;
            if (fl & 0x70u) {
                Inc inc[4];
#pragma unroll
                for (int d = 0; d < 3; ++d)
                    if (fl & (16u << d)) nef += plaquette_faces(g, flags, a, b, c, d, inc);
            }
            if (fl & 8u) {
                const int v[3] = {a, b, c};
#pragma unroll
                for (int d = 0; d < 3; ++d) {
                    if (v[d] > 0) {
                        int q[3] = {a, b, c};
                        q[d] -= 1;
                        if (flags[g.lid(q[0], q[1], q[2])] & (16u << d)) ++nve;
                    }
                    if (fl & (16u << d)) ++nve;
                    const int u = (d + 1) % 3, w = (d + 2) % 3;
                    int p1[3] = {a, b, c}, p3[3] = {a, b, c};
                    p1[w] += 1;  // the vertex is q1 of face (p1, d)
                    p3[u] += 1;  // the vertex is q3 of face (p3, d)
                    if (flags[g.lid(p1[0], p1[1], p1[2])] & (1u << d)) ++nve;
                    if (flags[g.lid(p3[0], p3[1], p3[2])] & (1u << d)) ++nve;
                }
            }
            cv[p] = (fl >> 3) & 1u;
            ce[p] = __popc((fl >> 4) & 7u);
            cf[p] = __popc(fl & 7u);
            cef[p] = nef;
            cve[p] = nve;
        }
    }
}

struct Offs {
    const int32_t* voff;
    const int32_t* eoff;
    const int32_t* foff;
    const int32_t* efoff;
    const int32_t* veoff;
    // the same scans seen from a volume whose lattice starts at lat0
    __device__ __forceinline__ Offs at(int64_t lat0) const {
        return Offs{voff + lat0, eoff + lat0, foff + lat0, efoff + lat0, veoff + lat0};
    }
};

// Batch-wide cell ids are volume-major (vertices; axis edges then diagonals;
// triangles).  The scans count axis edges and faces over the whole batch, so
// in volume bv an axis edge of scan rank e has id e + (faces before bv), the
// diagonal of face f has id (axis edges up to and including bv) + f, an axis
// edge's E->F list starts at its scan offset + 2 (faces before bv) and a
// diagonal's at (axis E->F entries up to and including bv) + 2 f.
struct Shift {
    int64_t fb;    // faces before the volume
    int64_t eb1;   // axis edges of volumes <= bv
    int64_t efb1;  // axis-edge E->F entries of volumes <= bv
    int64_t site;  // first site of the volume
};
__device__ __forceinline__ Shift shift_of(const Bases& B, int bv) {
    return Shift{B.b[kBFace][bv], B.b[kBAxis][bv + 1], B.b[kBEfAxis][bv + 1], B.b[kBSite][bv]};
}

__device__ __forceinline__ int32_t edge_id(const uint8_t* flags, const Offs& o, int64_t lp, int d) {
    return o.eoff[lp] + rank_below((flags[lp] >> 4) & 7u, d);
}
__device__ __forceinline__ int32_t face_id(const uint8_t* flags, const Offs& o, int64_t lp, int d) {
    return o.foff[lp] + rank_below(flags[lp] & 7u, d);
}

template <int N>
__device__ __forceinline__ void sort_small(int32_t* x, int k) {
    for (int i = 1; i < k; ++i) {
        const int32_t v = x[i];
        int j = i - 1;
        while (j >= 0 && x[j] > v) {
            x[j + 1] = x[j];
            --j;
        }
        x[j + 1] = v;
    }
}

// After the scans: the lattice position of every vertex, axis edge and face
// (p, or p*4 + axis), so that the emit kernels run one thread per cell with
// coalesced writes; also each vertex's V->E and each axis edge's E->F offset.
// Positions are batch-wide lattice indices; epos is indexed by axis-edge
// scan rank, ef_off by edge id.
__global__ void vd_positions_kernel(const uint8_t* __restrict__ occ, const int32_t* __restrict__ lab, VolTab T,
                                    Bases B, const uint8_t* __restrict__ flags_all, Offs oall,
                                    int64_t* __restrict__ vpos, int64_t* __restrict__ epos,
                                    int64_t* __restrict__ fpos, int32_t* __restrict__ ve_off,
                                    int32_t* __restrict__ ef_off) {
    const int64_t nrows = T.total(kLRow);
    for (int64_t grow = blockIdx.x; grow < nrows; grow += gridDim.x) {
        const int bv = T.find(kLRow, grow);
        const Grid g = grid_of(T, bv, occ, lab);
        const int64_t lat0 = T.start(kLat, bv);
        const uint8_t* flags = flags_all + lat0;
        const Offs o = oall.at(lat0);
        const int64_t fb = B.b[kBFace][bv];
        const int64_t row = grow - T.start(kLRow, bv);
        const int a = (int)(row / g.NB), b = (int)(row - (int64_t)a * g.NB);
        for (int c = threadIdx.x; c < (int)g.NC; c += blockDim.x) {
            const int64_t p = row * g.NC + c;
            const uint32_t fl = flags[p];
            if (fl & 8u) {
                const int32_t v = o.voff[p];
                vpos[v] = lat0 + p;
                ve_off[v] = o.veoff[p];
            }
            if (fl & 0x70u) {
                int32_t e = o.eoff[p];
                int64_t efo = o.efoff[p] + 2 * fb;
                Inc inc[4];
#pragma unroll
                for (int d = 0; d < 3; ++d) {
                    if (!(fl & (16u << d))) continue;
                    epos[e] = (lat0 + p) * 4 + d;
                    ef_off[e + fb] = (int32_t)efo;
                    efo += plaquette_faces(g, flags, a, b, c, d, inc);
                    ++e;
                }
            }
            if (fl & 7u) {
                int32_t f = o.foff[p];
#pragma unroll
                for (int d = 0; d < 3; ++d)
                    if (fl & (1u << d)) fpos[f++] = (lat0 + p) * 4 + d;
            }
        }
    }
}

__global__ void vd_vertices_kernel(const uint8_t* __restrict__ occ, const int32_t* __restrict__ lab, VolTab T,
                                   Bases B, const uint8_t* __restrict__ flags_all, Offs oall,
                                   const float* __restrict__ lam_all, const int64_t* __restrict__ vpos, int32_t nv,
                                   float* __restrict__ vts, float* __restrict__ vm, const int32_t* __restrict__ ve_off,
                                   int32_t* __restrict__ ve_ids, VertRec* __restrict__ V) {
    for (int32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < nv; v += gridDim.x * blockDim.x) {
        {
            const int64_t gp = vpos[v];
            const int bv = T.find(kLat, gp);
            const Grid g = grid_of(T, bv, occ, lab);
            const int64_t lat0 = T.start(kLat, bv);
            const uint8_t* flags = flags_all + lat0;
            const float* lam = lam_all + 3 * lat0;
            const Offs o = oall.at(lat0);
            const Shift sh = shift_of(B, bv);
            int32_t* bbox = B.bbox + 6 * bv;
            const int64_t p = gp - lat0;
            int a, b, c;
            decode32(p, g.NB, g.NC, a, b, c);
            const uint32_t fl = flags[p];
            vts[3 * (int64_t)v + 0] = (float)a;
            vts[3 * (int64_t)v + 1] = (float)b;
            vts[3 * (int64_t)v + 2] = (float)c;
            // vertex lambda: max over the valid faces of the voxel's 12 cube edges
            float m = 0.0f;
#pragma unroll
            for (int d = 0; d < 3; ++d)
#pragma unroll
                for (int s = 0; s < 2; ++s)
#pragma unroll
                    for (int t = 0; t < 2; ++t) {
                        int q[3] = {a, b, c};
                        q[(d + 1) % 3] += s;
                        q[(d + 2) % 3] += t;
                        const int64_t lp = g.lid(q[0], q[1], q[2]);
                        if (flags[lp] & (1u << d)) m = fmaxf(m, lam[3 * lp + d]);
                    }
            vm[v] = m;
            // V->E list in edge-id order: axis edges (their lower voxels precede
            // this one in lattice order, then this voxel's own), then diagonals
            const int32_t off = ve_off[v];
            int k = 0;
            const int vv[3] = {a, b, c};
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                if (vv[d] == 0) continue;
                int q[3] = {a, b, c};
                q[d] -= 1;
                const int64_t lq = g.lid(q[0], q[1], q[2]);
                if (flags[lq] & (16u << d)) ve_ids[off + k++] = edge_id(flags, o, lq, d) + (int32_t)sh.fb;
            }
#pragma unroll
            for (int d = 0; d < 3; ++d)
                if (fl & (16u << d)) ve_ids[off + k++] = edge_id(flags, o, p, d) + (int32_t)sh.fb;
            int32_t dg[6];
            int nd = 0;
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                const int u = (d + 1) % 3, w = (d + 2) % 3;
                int p1[3] = {a, b, c}, p3[3] = {a, b, c};
                p1[w] += 1;
                p3[u] += 1;
                const int64_t l1 = g.lid(p1[0], p1[1], p1[2]), l3 = g.lid(p3[0], p3[1], p3[2]);
                if (flags[l1] & (1u << d)) dg[nd++] = face_id(flags, o, l1, d);
                if (flags[l3] & (1u << d)) dg[nd++] = face_id(flags, o, l3, d);
            }
            sort_small<6>(dg, nd);
            for (int i = 0; i < nd; ++i) ve_ids[off + k++] = (int32_t)sh.eb1 + dg[i];
            if (V) {
                unsigned long long idsum = 0;
                for (int q = 0; q < k; ++q) idsum += (unsigned)ve_ids[off + q];
                VertRec r;
                r.rs = rs_make((unsigned)k, 0, idsum);
                r.trig = 0;
                r.rm = kAlive;
                r.pad0 = r.pad1 = r.pad2 = 0;
                V[v] = r;
            }
            // the volume's bounding box: lanes of the same volume reduce in
            // the warp first, so each warp issues one set of atomics per volume
            const unsigned grp = __match_any_sync(__activemask(), bv);
            const int mn0 = __reduce_min_sync(grp, a), mn1 = __reduce_min_sync(grp, b),
                      mn2 = __reduce_min_sync(grp, c);
            const int mx0 = __reduce_max_sync(grp, a), mx1 = __reduce_max_sync(grp, b),
                      mx2 = __reduce_max_sync(grp, c);
            if ((int)(threadIdx.x & 31) == __ffs(grp) - 1) {
                atomicMin(&bbox[0], mn0);
                atomicMin(&bbox[1], mn1);
                atomicMin(&bbox[2], mn2);
                atomicMax(&bbox[3], mx0);
                atomicMax(&bbox[4], mx1);
                atomicMax(&bbox[5], mx2);
            }
        }
    }
}

// Thinning filter folded into the records (batched runs): with `thr` set,
// a record's measure becomes -1 when it is below its volume's threshold and
// +1 otherwise, and the thinning then runs with threshold 0.
__device__ __forceinline__ float rec_measure(float m, const float* thr, int bv) {
    if (!thr) return m;
    return m < thr[bv] ? -1.0f : 1.0f;
}

__global__ void vd_edges_kernel(const uint8_t* __restrict__ occ, const int32_t* __restrict__ lab, VolTab T, Bases B,
                                const uint8_t* __restrict__ flags_all, Offs oall, const float* __restrict__ lam_all,
                                const int64_t* __restrict__ epos, int32_t ne_axis, int2* __restrict__ edges,
                                float* __restrict__ em, const int32_t* __restrict__ ef_off, int32_t* __restrict__ ef_ids,
                                EdgeRec* __restrict__ E, const float* __restrict__ thr) {
    for (int32_t ea = blockIdx.x * blockDim.x + threadIdx.x; ea < ne_axis; ea += gridDim.x * blockDim.x) {
        const int64_t q = epos[ea];
        const int64_t gp = q >> 2;
        const int d = (int)(q & 3);
        const int bv = T.find(kLat, gp);
        const Grid g = grid_of(T, bv, occ, lab);
        const int64_t lat0 = T.start(kLat, bv);
        const uint8_t* flags = flags_all + lat0;
        const float* lam = lam_all + 3 * lat0;
        const Offs o = oall.at(lat0);
        const int32_t e = ea + (int32_t)B.b[kBFace][bv];
        const int64_t p = gp - lat0;
        int a, b, c;
        decode32(p, g.NB, g.NC, a, b, c);
        int nb[3] = {a, b, c};
        nb[d] += 1;
        const int32_t v0 = o.voff[p], v1 = o.voff[g.lid(nb[0], nb[1], nb[2])];
        Inc inc[4];
        const int k = plaquette_faces(g, flags, a, b, c, d, inc);
        float m = 0.0f;
        int32_t tl[4];
        unsigned npass = 0;  // incident triangles that pass the thinning filter
        const float tb = thr ? thr[bv] : 0.0f;
        for (int j = 0; j < k; ++j) {
            const float lj = lam[3 * inc[j].lp + inc[j].axis];
            m = fmaxf(m, lj);
            npass += lj < tb ? 1u : 0u;
            tl[j] = 2 * face_id(flags, o, inc[j].lp, inc[j].axis) + inc[j].tri;
        }
        sort_small<4>(tl, k);
        const int32_t efo = ef_off[e];
        for (int j = 0; j < k; ++j) ef_ids[efo + j] = tl[j];
        edges[e] = make_int2(v0, v1);
        em[e] = m;
        if (thr) {
            unsigned long long idsum = 0;
            for (int j = 0; j < k; ++j) idsum += (unsigned)tl[j];
            EdgeRec r;
            r.v0 = v0;
            r.v1 = v1;
            r.rs = rs_make((unsigned)k, npass, idsum);
            r.trig = 0;
            r.em = rec_measure(m, thr, bv);
            r.rm = kAlive;
            E[e] = r;
        }
    }
}

// tri_face and face_sites are per volume: the face's index within its
// volume and the volume's own site indices.
__global__ void vd_faces_kernel(const uint8_t* __restrict__ occ, const int32_t* __restrict__ lab, VolTab T, Bases B,
                                const uint8_t* __restrict__ flags_all, Offs oall, const float* __restrict__ lam_all,
                                const int64_t* __restrict__ fpos, int32_t nface, int2* __restrict__ edges,
                                float* __restrict__ em, int32_t* __restrict__ ef_off, int32_t* __restrict__ ef_ids,
                                int32_t* __restrict__ tris, int32_t* __restrict__ tri_edges, float* __restrict__ fm,
                                int32_t* __restrict__ tri_face, int2* __restrict__ face_sites,
                                FaceRec* __restrict__ F, EdgeRec* __restrict__ E, const float* __restrict__ thr) {
    for (int32_t f = blockIdx.x * blockDim.x + threadIdx.x; f < nface; f += gridDim.x * blockDim.x) {
        const int64_t qq = fpos[f];
        const int64_t gp = qq >> 2;
        const int d = (int)(qq & 3);
        const int bv = T.find(kLat, gp);
        const Grid g = grid_of(T, bv, occ, lab);
        const int64_t lat0 = T.start(kLat, bv);
        const uint8_t* flags = flags_all + lat0;
        const float* lam = lam_all + 3 * lat0;
        const Offs o = oall.at(lat0);
        const Shift sh = shift_of(B, bv);
        const int32_t fbs = (int32_t)sh.fb;
        const int64_t p = gp - lat0;
        int a, b, c;
        decode32(p, g.NB, g.NC, a, b, c);
        {
            {
                const int u = (d + 1) % 3, w = (d + 2) % 3;
                int e1[3] = {a, b, c};
                e1[d] += 1;
                const int32_t s0 = g.lab[p], s1 = g.label(e1[0], e1[1], e1[2]);
                const float lm = lam[3 * p + d];
                int64_t ql[4];
                int32_t q[4];
#pragma unroll
                for (int m = 0; m < 4; ++m) {
                    int i, j, k;
                    quad_voxel(a, b, c, d, m, i, j, k);
                    ql[m] = g.lid(i, j, k);
                    q[m] = o.voff[ql[m]];
                }
                const int32_t diag = (int32_t)sh.eb1 + f;
                const int32_t e01 = edge_id(flags, o, ql[0], u) + fbs;
                const int32_t e12 = edge_id(flags, o, ql[1], w) + fbs;
                const int32_t e32 = edge_id(flags, o, ql[3], u) + fbs;
                const int32_t e03 = edge_id(flags, o, ql[0], w) + fbs;
                const int64_t t0 = 2 * (int64_t)f, t1 = t0 + 1;
                tris[3 * t0 + 0] = q[3];
                tris[3 * t0 + 1] = q[0];
                tris[3 * t0 + 2] = q[1];
                tris[3 * t1 + 0] = q[3];
                tris[3 * t1 + 1] = q[1];
                tris[3 * t1 + 2] = q[2];
                // sides in traceFace order: (t0,t1), (t1,t2), (t2,t0)
                tri_edges[3 * t0 + 0] = e03;
                tri_edges[3 * t0 + 1] = e01;
                tri_edges[3 * t0 + 2] = diag;
                tri_edges[3 * t1 + 0] = diag;
                tri_edges[3 * t1 + 1] = e12;
                tri_edges[3 * t1 + 2] = e32;
                fm[t0] = lm;
                fm[t1] = lm;
                tri_face[t0] = f - fbs;
                tri_face[t1] = f - fbs;
                face_sites[f] = make_int2(s0 - (int32_t)sh.site, s1 - (int32_t)sh.site);
                if (thr) {
                const float lr = rec_measure(lm, thr, bv);
                FaceRec fr;
                fr.fm = lr;
                fr.rm = kAlive;
                fr.pad0 = fr.pad1 = fr.pad2 = 0;
                fr.e0 = e03;
                fr.e1 = e01;
                fr.e2 = diag;
                F[t0] = fr;
                fr.e0 = diag;
                fr.e1 = e12;
                fr.e2 = e32;
                F[t1] = fr;
                }
                // the diagonal: new edge of this face, incident to both triangles
                const int32_t dv0 = min(q[1], q[3]), dv1 = max(q[1], q[3]);
                const int32_t efo = (int32_t)sh.efb1 + 2 * f;
                edges[diag] = make_int2(dv0, dv1);
                em[diag] = lm;
                ef_off[diag] = efo;
                ef_ids[efo] = (int32_t)t0;
                ef_ids[efo + 1] = (int32_t)t1;
                if (thr) {
                    EdgeRec er;
                    er.v0 = dv0;
                    er.v1 = dv1;
                    er.rs = rs_make(2, lm < thr[bv] ? 2u : 0u, (unsigned long long)t0 + (unsigned long long)t1);
                    er.trig = 0;
                    er.em = rec_measure(lm, thr, bv);
                    er.rm = kAlive;
                    E[diag] = er;
                }
            }
        }
    }
}

__global__ void vd_tail_kernel(int32_t* ve_off, int32_t nv, int32_t nve, int32_t* ef_off, int32_t ne, int32_t nef) {
    if (threadIdx.x == 0) {
        ve_off[nv] = nve;
        ef_off[ne] = nef;
    }
}

__global__ void init_bbox_kernel(int32_t* bbox, int nvol) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < 6 * nvol; i += gridDim.x * blockDim.x)
        bbox[i] = (i % 6) < 3 ? INT32_MAX : INT32_MIN;
}

// Inside-part size of every volume, VoroInfo::getInsidePartSize
// (voroinfo.cpp:496): trimesh::box::size().max() of the float vertex
// coordinates (0 without vertices); with t >= 0 also the thinning threshold
// float(size * t) of exportInsideVoroMesh (highlevelalgo.cpp:836), the float
// times double product rounded to float.
__global__ void inside_size_kernel(Bases B, int nvol, double t) {
    for (int bv = blockIdx.x * blockDim.x + threadIdx.x; bv < nvol; bv += gridDim.x * blockDim.x) {
        const int32_t* bb = B.bbox + 6 * bv;
        float isz = 0.0f;
        if (B.b[kBVert][bv + 1] > B.b[kBVert][bv]) {
            const float sx = (float)bb[3] - (float)bb[0], sy = (float)bb[4] - (float)bb[1],
                        sz = (float)bb[5] - (float)bb[2];
            isz = fmaxf(sx, fmaxf(sy, sz));
        }
        B.inside[bv] = isz;
        if (t >= 0.0) B.thr[bv] = (float)__dmul_rn((double)isz, t);
    }
}

inline int cell_grid(vc_ctx* c, int64_t n) {
    return (int)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, (int64_t)c->num_sms * 16));
}

// Radius per vertex, VoroInfo::computeInfoRelatedtoSites
// (voroinfo.cpp:286-325): every Voronoi face, in face order, writes
// r = dist(first site of the face, vertex) into each of its vertices, so a
// vertex keeps the value of the LAST face that has it (voroinfo.cpp:316).
// The Voronoi faces through voxel v are the candidate edges among the 12
// edges of v's cube; in (lattice point, axis) order the last one is found by
// scanning the cube corners q = 7..0 (corner order is lattice order) and the
// axes 2..0.  The first site of face (p, d) is the label of p.  The distance
// is accumulated in float in trimesh's order and rounded by one correctly
// rounded square root (exact for boxes up to 2^11 per side).
__global__ void vd_radius_kernel(const uint8_t* __restrict__ occ, const int32_t* __restrict__ lab, VolTab T,
                                 const float* __restrict__ sxyz, const int64_t* __restrict__ vpos, int32_t nv,
                                 float* __restrict__ radius) {
    for (int32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < nv; v += gridDim.x * blockDim.x) {
        const int64_t gp = vpos[v];
        const int bv = T.find(kLat, gp);
        const Grid g = grid_of(T, bv, occ, lab);
        int a, b, c;
        decode32(gp - T.start(kLat, bv), g.NB, g.NC, a, b, c);
        int32_t L[8];
#pragma unroll
        for (int q = 0; q < 8; ++q) L[q] = g.label(a + ((q >> 2) & 1), b + ((q >> 1) & 1), c + (q & 1));
        int32_t s = L[0];
        bool found = false;
#pragma unroll
        for (int q = 7; q >= 0; --q)
#pragma unroll
            for (int d = 2; d >= 0; --d) {
                const int bit = 4 >> d;
                if (found || (q & bit)) continue;
                if (L[q] != L[q | bit]) {
                    s = L[q];
                    found = true;
                }
            }
        const float dx = (float)a - sxyz[3 * (int64_t)s + 0];
        const float dy = (float)b - sxyz[3 * (int64_t)s + 1];
        const float dz = (float)c - sxyz[3 * (int64_t)s + 2];
        float r = 0.0f;
        r = __fadd_rn(r, __fmul_rn(dx, dx));
        r = __fadd_rn(r, __fmul_rn(dy, dy));
        r = __fadd_rn(r, __fmul_rn(dz, dz));
        radius[v] = __fsqrt_rn(r);
    }
}

inline int row_grid(vc_ctx* c, int64_t rows) {
    return (int)std::max<int64_t>(1, std::min<int64_t>(rows, (int64_t)c->num_sms * 32));
}


}  // namespace

// t_thr >= 0: also compute every volume's thinning threshold float(size *
// t_thr) and fold it into the thinning records (see rec_measure).
int run_lattice_vd(vc_ctx* c, vc_vd_sizes* sizes, double t_thr) {
    if (!c->ft_valid) return VC_ERR_STATE;
    const int nvol = c->nvol;
    for (int b = 0; b < nvol; ++b)
        if (space_size(kLat, c->h_dims[3 * b], c->h_dims[3 * b + 1], c->h_dims[3 * b + 2]) >= ((int64_t)1 << 32))
            return VC_ERR_ARG;
    const int64_t N = c->h_off[kLat][nvol];
    const int64_t nrows = c->h_off[kLRow][nvol];
    Region stage(c, "stage_vd");
    VC_TRY(ensure_n<uint8_t>(c, c->vd_flags, N));
    VC_TRY(ensure_n<float>(c, c->vd_lam, 3 * N));
    VC_TRY(ensure_n<int32_t>(c, c->vd_voff, N));
    VC_TRY(ensure_n<int32_t>(c, c->vd_eoff, N));
    VC_TRY(ensure_n<int32_t>(c, c->vd_foff, N));
    VC_TRY(ensure_n<int32_t>(c, c->vd_efoff, N));
    VC_TRY(ensure_n<int32_t>(c, c->vd_veoff, N));
    VC_TRY(ensure_n<int64_t>(c, c->scratch2, 8));
    const uint8_t* occ = ptr<uint8_t>(c->occ);
    const int32_t* lab = ptr<int32_t>(c->ft_id);
    uint8_t* flags = ptr<uint8_t>(c->vd_flags);
    float* lam = ptr<float>(c->vd_lam);
    int32_t* cnt[5] = {ptr<int32_t>(c->vd_voff), ptr<int32_t>(c->vd_eoff), ptr<int32_t>(c->vd_foff),
                       ptr<int32_t>(c->vd_efoff), ptr<int32_t>(c->vd_veoff)};
    const float* sxyz = ptr<float>(c->site_xyz);
    {
        Region r(c, "vd_flags");
        vd_flags_kernel<<<row_grid(c, nrows), 128, 0, c->stream>>>(occ, lab, c->tab, sxyz, flags, lam);
        launched(c);
        vd_counts_kernel<<<row_grid(c, nrows), 128, 0, c->stream>>>(occ, lab, c->tab, flags, cnt[0], cnt[1], cnt[2],
                                                                     cnt[3], cnt[4]);
        launched(c);
        VC_CUDA(c, cudaGetLastError());
    }
    int64_t* tot = ptr<int64_t>(c->scratch2);
    {
        Region r(c, "vd_scan");
        const int base_of[5] = {kBVert, kBAxis, kBFace, kBEfAxis, kBVe};
        for (int k = 0; k < 5; ++k) {
            VC_TRY(scan_exclusive_i32(c, cnt[k], cnt[k], N, tot + k));
            VC_TRY(fill_bases(c, base_of[k], kLat, cnt[k], tot + k));
        }
    }
    int64_t h[5];
    VC_CUDA(c, cudaMemcpyAsync(h, tot, 5 * sizeof(int64_t), cudaMemcpyDeviceToHost, c->stream));
    VC_TRY(sync_check(c));
    const int64_t nv = h[0], ne_axis = h[1], nface = h[2], nef_axis = h[3], nve = h[4];
    const int64_t ne = ne_axis + nface, nt = 2 * nface;
    if (ne >= INT32_MAX || 3 * nt >= INT32_MAX || nv >= INT32_MAX || nve >= INT32_MAX) return VC_ERR_ARG;
    if (nef_axis != 4 * nface || nve != 2 * ne) {
        c->last_error = "lattice complex incidence counts are inconsistent";
        return VC_ERR_INVARIANT;
    }
    // the complex becomes the context's finalized cell complex
    c->cc_valid = c->cc_finalized = c->meas_valid = c->thin_valid = c->rem_valid = false;
    c->records_fresh = false;
    VC_TRY(ensure_n<float>(c, c->vts, 3 * nv));
    VC_TRY(ensure_n<int2>(c, c->edges, ne));
    VC_TRY(ensure_n<int32_t>(c, c->tris, 3 * nt));
    VC_TRY(ensure_n<int32_t>(c, c->tri_edges, 3 * nt));
    VC_TRY(ensure_n<float>(c, c->vm, nv));
    VC_TRY(ensure_n<float>(c, c->em, ne));
    VC_TRY(ensure_n<float>(c, c->fm, nt));
    VC_TRY(ensure_n<int32_t>(c, c->vd_tri_face, nt));
    VC_TRY(ensure_n<int2>(c, c->vd_face_sites, nface));
    VC_TRY(ensure_n<int32_t>(c, c->ve_off, nv + 1));
    VC_TRY(ensure_n<int32_t>(c, c->ve_ids, 2 * ne));
    VC_TRY(ensure_n<int32_t>(c, c->ef_off, ne + 1));
    VC_TRY(ensure_n<int32_t>(c, c->ef_ids, 3 * nt));
    VC_TRY(ensure_n<FaceRec>(c, c->face_rec, nt));
    VC_TRY(ensure_n<EdgeRec>(c, c->edge_rec, ne));
    VC_TRY(ensure_n<VertRec>(c, c->vert_rec, nv));
    VC_TRY(ensure_n<int64_t>(c, c->vd_vpos, nv));
    VC_TRY(ensure_n<int64_t>(c, c->vd_epos, ne_axis));
    VC_TRY(ensure_n<int64_t>(c, c->vd_fpos, nface));
    init_bbox_kernel<<<(6 * nvol + 255) / 256, 256, 0, c->stream>>>(c->bases.bbox, nvol);
    launched(c);
    Offs o{cnt[0], cnt[1], cnt[2], cnt[3], cnt[4]};
    const float* thr = t_thr >= 0.0 ? c->bases.thr : nullptr;
    {
        Region r(c, "vd_emit");
        {
            Region k(c, "vd_positions");
            vd_positions_kernel<<<row_grid(c, nrows), 128, 0, c->stream>>>(
                occ, lab, c->tab, c->bases, flags, o, ptr<int64_t>(c->vd_vpos), ptr<int64_t>(c->vd_epos),
                ptr<int64_t>(c->vd_fpos), ptr<int32_t>(c->ve_off), ptr<int32_t>(c->ef_off));
            launched(c);
        }
        {
            Region k(c, "vd_vertices");
            vd_vertices_kernel<<<cell_grid(c, nv), 256, 0, c->stream>>>(
                occ, lab, c->tab, c->bases, flags, o, lam, ptr<int64_t>(c->vd_vpos), (int32_t)nv, ptr<float>(c->vts),
                ptr<float>(c->vm), ptr<int32_t>(c->ve_off), ptr<int32_t>(c->ve_ids),
                thr ? ptr<VertRec>(c->vert_rec) : nullptr);
            launched(c);
            inside_size_kernel<<<(nvol + 255) / 256, 256, 0, c->stream>>>(c->bases, nvol, t_thr);
            launched(c);
        }
        {
            Region k(c, "vd_edges");
            vd_edges_kernel<<<cell_grid(c, ne_axis), 256, 0, c->stream>>>(
                occ, lab, c->tab, c->bases, flags, o, lam, ptr<int64_t>(c->vd_epos), (int32_t)ne_axis,
                ptr<int2>(c->edges), ptr<float>(c->em), ptr<int32_t>(c->ef_off), ptr<int32_t>(c->ef_ids),
                ptr<EdgeRec>(c->edge_rec), thr);
            launched(c);
        }
        {
            Region k(c, "vd_faces");
            vd_faces_kernel<<<cell_grid(c, nface), 256, 0, c->stream>>>(
                occ, lab, c->tab, c->bases, flags, o, lam, ptr<int64_t>(c->vd_fpos), (int32_t)nface,
                ptr<int2>(c->edges), ptr<float>(c->em), ptr<int32_t>(c->ef_off), ptr<int32_t>(c->ef_ids),
                ptr<int32_t>(c->tris), ptr<int32_t>(c->tri_edges), ptr<float>(c->fm), ptr<int32_t>(c->vd_tri_face),
                ptr<int2>(c->vd_face_sites), ptr<FaceRec>(c->face_rec), ptr<EdgeRec>(c->edge_rec), thr);
            launched(c);
        }
        vd_tail_kernel<<<1, 32, 0, c->stream>>>(ptr<int32_t>(c->ve_off), (int32_t)nv, (int32_t)nve,
                                                ptr<int32_t>(c->ef_off), (int32_t)ne, (int32_t)(3 * nt));
        launched(c);
        VC_CUDA(c, cudaGetLastError());
    }
    c->vol_inside.resize((size_t)nvol);
    VC_CUDA(c, cudaMemcpyAsync(c->vol_inside.data(), c->bases.inside, (size_t)nvol * sizeof(float),
                               cudaMemcpyDeviceToHost, c->stream));
    VC_TRY(sync_check(c));
    c->nv = nv;
    c->ne_in = ne;
    c->ne = ne;
    c->nt = nt;
    c->vd = vc_vd_sizes{nv, ne, nt, nface, c->vol_inside[0]};
    c->vd_valid = true;
    c->cc_valid = true;
    c->cc_finalized = true;
    c->meas_valid = true;
    // records are written only with the thresholds folded in (their filter
    // counts need the thresholds); otherwise the thinning builds them
    c->records_fresh = t_thr >= 0.0;
    c->records_thr_folded = t_thr >= 0.0;
    c->cc_batched = nvol > 1;
    if (sizes) *sizes = c->vd;
    return VC_OK;
}

int run_vertex_radii(vc_ctx* c) {
    if (!c->vd_valid || !c->ft_valid) return VC_ERR_STATE;
    const int64_t nv = c->vd.nv;
    VC_TRY(ensure_n<float>(c, c->vd_radius, nv));
    if (nv == 0) return VC_OK;
    Region r(c, "vd_radius");
    vd_radius_kernel<<<cell_grid(c, nv), 256, 0, c->stream>>>(ptr<uint8_t>(c->occ), ptr<int32_t>(c->ft_id), c->tab,
                                                              ptr<float>(c->site_xyz), ptr<int64_t>(c->vd_vpos),
                                                              (int32_t)nv, ptr<float>(c->vd_radius));
    launched(c);
    VC_CUDA(c, cudaGetLastError());
    return VC_OK;
}

}  // namespace vc
