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
//
// Layout: one pass over the lattice writes, per 32-point segment of a
// lattice row, seven bit planes (vertex, valid axis edge per axis, valid
// face per axis) and the three cell counts; after one scan of the segment
// counts any cell's id is an O(1) population count.  The emission kernels
// run one thread per lattice point (a warp per segment, so writes of
// consecutive ids are coalesced) and write what the thinning and the
// remaining complex read: vertex coordinates, edges, triangles and the
// thinning records.  The measures, triangle faces, face sites, triangle
// sides and adjacency lists are written on demand (ensure_vd_aux), when a
// getter or a thinning with explicit thresholds asks for them.
#include "vc_internal.cuh"

#include <algorithm>
#include <cstring>

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


// ---------------------------------------------------------------------------
// Cell bit planes.  Each lattice row along z is cut into 32-point segments;
// per segment seven 32-bit planes say, for every point, whether its voxel is
// a vertex (v), whether its axis edge along d is a valid edge (e0..e2) and
// whether its lattice edge along d carries a valid face (f0..f2).  After one
// scan of the per-segment counts, a cell's id is its segment's first id plus
// a population count of the planes below it, so every kernel finds any
// neighbour's id in O(1) from 48 bytes (planes + three first ids) instead of
// per-point offset arrays.
struct __align__(32) SegPlanes {
    uint32_t v, e0, e1, e2, f0, f1, f2, pad;
};

__device__ __forceinline__ uint32_t plane_e(const SegPlanes& s, int d) { return d == 0 ? s.e0 : (d == 1 ? s.e1 : s.e2); }
__device__ __forceinline__ uint32_t plane_f(const SegPlanes& s, int d) { return d == 0 ? s.f0 : (d == 1 ? s.f1 : s.f2); }

// The segments of volume bv: point (a, b, c) is bit c & 31 of segment
// seg0 + (a * NB + b) * nsr + (c >> 5).  vb / eb / fb hold the batch-wide id
// of the segment's first vertex / axis edge (scan rank) / face.
struct Segs {
    const SegPlanes* planes;
    const int32_t* vb;
    const int32_t* eb;
    const int32_t* fb;
    int64_t seg0, NB;
    int nsr;
    __device__ __forceinline__ int64_t at(int a, int b, int c) const {
        return seg0 + ((int64_t)a * NB + b) * nsr + (c >> 5);
    }
};
__device__ __forceinline__ Segs segs_of(const VolTab& T, int bv, const SegPlanes* planes, const int32_t* vb,
                                        const int32_t* eb, const int32_t* fb) {
    const int4 d = T.dim(bv);
    return Segs{planes, vb, eb, fb, T.start(kLSeg, bv), (int64_t)d.y + 1, (d.z + 32) / 32};
}
__device__ __forceinline__ SegPlanes load_planes(const SegPlanes* p) {
    const uint4 x = __ldg(reinterpret_cast<const uint4*>(p));
    const uint4 y = __ldg(reinterpret_cast<const uint4*>(p) + 1);
    return SegPlanes{x.x, x.y, x.z, x.w, y.x, y.y, y.z, y.w};
}
__device__ __forceinline__ uint32_t below(int c) { return (1u << (c & 31)) - 1u; }
__device__ __forceinline__ bool bit(uint32_t w, int c) { return (w >> (c & 31)) & 1u; }

// batch-wide vertex id of the voxel at (a, b, c) (which must be a vertex)
__device__ __forceinline__ int32_t vid_at(const Segs& S, int a, int b, int c) {
    const int64_t s = S.at(a, b, c);
    return __ldg(S.vb + s) + __popc(__ldg(&S.planes[s].v) & below(c));
}
// scan rank (batch-wide, axis edges only) of the axis edge (a, b, c) + d
__device__ __forceinline__ int32_t erank_at(const Segs& S, int a, int b, int c, int d) {
    const int64_t s = S.at(a, b, c);
    const SegPlanes P = load_planes(S.planes + s);
    const uint32_t m = below(c);
    int32_t r = __ldg(S.eb + s) + __popc(P.e0 & m) + __popc(P.e1 & m) + __popc(P.e2 & m);
    if (d >= 1) r += bit(P.e0, c);
    if (d >= 2) r += bit(P.e1, c);
    return r;
}
// batch-wide face id of the lattice edge (a, b, c) + d
__device__ __forceinline__ int32_t fid_at(const Segs& S, int a, int b, int c, int d) {
    const int64_t s = S.at(a, b, c);
    const SegPlanes P = load_planes(S.planes + s);
    const uint32_t m = below(c);
    int32_t r = __ldg(S.fb + s) + __popc(P.f0 & m) + __popc(P.f1 & m) + __popc(P.f2 & m);
    if (d >= 1) r += bit(P.f0, c);
    if (d >= 2) r += bit(P.f1, c);
    return r;
}
__device__ __forceinline__ bool ebit_at(const Segs& S, int a, int b, int c, int d) {
    return bit(plane_e(load_planes(S.planes + S.at(a, b, c)), d), c);
}
__device__ __forceinline__ bool fbit_at(const Segs& S, int a, int b, int c, int d) {
    return bit(plane_f(load_planes(S.planes + S.at(a, b, c)), d), c);
}

// Segment loop of the emission kernels: each block takes kSegChunk
// consecutive segments at a time and its warps walk them in order, so the
// neighbouring segments a warp reads stay in the block's L1 (rows of every
// length pack into chunks, which keeps small volumes of a batch busy).
constexpr int kSegChunk = 64;
#define SEG_LOOP(gs, nseg)                                                                                \
    for (int64_t seg_base_ = (int64_t)blockIdx.x * kSegChunk; seg_base_ < (nseg);                          \
         seg_base_ += (int64_t)gridDim.x * kSegChunk)                                                        \
        for (int64_t gs = seg_base_ + (threadIdx.x >> 5), seg_end_ = min((int64_t)(nseg), seg_base_ + kSegChunk); \
             gs < seg_end_; gs += blockDim.x >> 5)

// Batch-wide cell ids are volume-major (vertices; axis edges then
// diagonals; triangles).  The scans count axis edges and faces over the
// whole batch, so in volume bv an axis edge of scan rank e has id
// e + (faces before bv) and the diagonal of face f has id (axis edges up to
// and including bv) + f.
struct Shift {
    int64_t fb;    // faces before the volume
    int64_t eb1;   // axis edges of volumes <= bv
    int64_t site;  // first site of the volume
};
__device__ __forceinline__ Shift shift_of(const Bases& B, int bv) {
    return Shift{B.b[kBFace][bv], B.b[kBAxis][bv + 1], B.b[kBSite][bv]};
}

// Thinning filter folded into the records: with `thr` set, a record's
// measure becomes -1 when it is below its volume's threshold and +1
// otherwise, and the thinning then runs with threshold 0.
__device__ __forceinline__ float rec_measure(float m, const float* thr, int bv) {
    if (!thr) return m;
    return m < thr[bv] ? -1.0f : 1.0f;
}

// Per lattice point: whether its voxel is a vertex (inside, not all 8
// corner labels equal -- tagVert plus "corner of some Voronoi face"),
// whether each axis edge is valid (both voxels inside, the shared square's
// 4 labels not all equal) and whether each lattice edge carries a valid
// face (labels differ and the 4 voxels around it inside).  One warp per
// 32-point segment of a lattice row, lane = point: the occupancy tests run
// for the whole segment at once on the packed voxel words (bit t of a row's
// word = voxel c0 + t; shifted copies give c0 + t - 1 and c0 + t + 1), the
// label tests run per lane (the c + 1 labels come from the next lane) and
// ballots turn them into bit planes.  Also the volumes' vertex bounding
// boxes (VoroInfo::getInsidePartSize reads them).
__global__ void __launch_bounds__(128) vd_segments_kernel(const uint32_t* __restrict__ obits,
                                                          const int32_t* __restrict__ lab, VolTab T,
                                                          SegPlanes* __restrict__ planes, int32_t* __restrict__ cv,
                                                          int32_t* __restrict__ ce, int32_t* __restrict__ cf,
                                                          int32_t* __restrict__ bbox_all) {
    const int lane = threadIdx.x & 31;
    int cur_bv = -1;
    // warp-uniform bounding box of the current volume's vertices
    int mn0 = INT32_MAX, mn1 = INT32_MAX, mn2 = INT32_MAX, mx0 = INT32_MIN, mx1 = INT32_MIN, mx2 = INT32_MIN;
    auto flush = [&]() {
        if (lane == 0 && cur_bv >= 0 && mn0 != INT32_MAX) {
            int32_t* bb = bbox_all + 6 * cur_bv;
            atomicMin(&bb[0], mn0);
            atomicMin(&bb[1], mn1);
            atomicMin(&bb[2], mn2);
            atomicMax(&bb[3], mx0);
            atomicMax(&bb[4], mx1);
            atomicMax(&bb[5], mx2);
        }
        mn0 = mn1 = mn2 = INT32_MAX;
        mx0 = mx1 = mx2 = INT32_MIN;
    };
    const int64_t nseg = T.total(kLSeg);
    VolTab::Cache vcache;
    SEG_LOOP(gs, nseg) {
        const int bv = T.find_cached(kLSeg, gs, vcache);
        if (bv != cur_bv) {
            flush();
            cur_bv = bv;
        }
        const int4 dm = T.dim(bv);
        const int X = dm.x, Y = dm.y, Z = dm.z;
        const int64_t NB = Y + 1, NC = Z + 1;
        const int nsr = (Z + 32) / 32;
        const int64_t ls = gs - T.start(kLSeg, bv);
        const int64_t row = ls / nsr;
        const int c0 = (int)(ls - row * nsr) * 32;
        const int a = (int)(row / NB), b = (int)(row - (int64_t)a * NB);
        // occupancy words of the voxel rows around the segment
        const int sw = c0 >> 5, Wz = (Z + 31) >> 5;
        const uint32_t* ob = obits + T.start(kVWord, bv);
        auto word = [&](int i, int j, int w) -> uint32_t {
            return (i >= 0 && i < X && j >= 0 && j < Y && w >= 0 && w < Wz) ? __ldg(ob + ((int64_t)i * Y + j) * Wz + w)
                                                                           : 0u;
        };
        // bit t: voxel (i, j, c0 + t - 1) / (i, j, c0 + t) / (i, j, c0 + t + 1) inside
        struct Rw {
            uint32_t m1, z0, p1;
        };
        auto rw = [&](int i, int j) {
            const uint32_t prv = word(i, j, sw - 1), cur = word(i, j, sw), nxt = word(i, j, sw + 1);
            return Rw{(cur << 1) | (prv >> 31), cur, (cur >> 1) | (nxt << 31)};
        };
        const Rw Rmm = rw(a - 1, b - 1), Rm0 = rw(a - 1, b), R0m = rw(a, b - 1), R00 = rw(a, b), Rp0 = rw(a + 1, b),
                 R0p = rw(a, b + 1);
        const uint32_t qx = R0m.m1 & R0m.z0 & R00.m1 & R00.z0;  // voxels (a, b-1..b, c-1..c)
        const uint32_t qy = Rm0.m1 & Rm0.z0 & R00.m1 & R00.z0;  // voxels (a-1..a, b, c-1..c)
        const uint32_t qz = Rmm.z0 & Rm0.z0 & R0m.z0 & R00.z0;  // voxels (a-1..a, b-1..b, c)
        // labels of the voxel's 8 corners (a + qx, b + qy, c + qz), -1 outside the lattice
        const int c = c0 + lane;
        const bool valid = c < NC;
        const int32_t* lb = lab + T.start(kLat, bv);
        auto lat = [&](int i, int j, int k) -> int32_t {
            return (i <= X && j <= Y && k <= Z) ? __ldg(lb + ((int64_t)i * NB + j) * NC + k) : -1;
        };
        int32_t L[8];
        L[0] = valid ? lat(a, b, c) : -1;
        L[2] = valid ? lat(a, b + 1, c) : -1;
        L[4] = valid ? lat(a + 1, b, c) : -1;
        L[6] = valid ? lat(a + 1, b + 1, c) : -1;
#pragma unroll
        for (int q = 0; q < 8; q += 2) {
            L[q + 1] = __shfl_down_sync(0xffffffffu, L[q], 1);
            if (lane == 31) L[q + 1] = valid ? lat(a + (q >> 2), b + ((q >> 1) & 1), c + 1) : -1;
        }
        bool alleq = true;
#pragma unroll
        for (int q = 1; q < 8; ++q) alleq &= (L[q] == L[0]);
        auto differ = [](int32_t x, int32_t y) { return x >= 0 && y >= 0 && x != y; };
        auto square_differs = [&](int bitd) {
            int32_t ref = -2;
            bool eq = true;
#pragma unroll
            for (int q = 0; q < 8; ++q) {
                if (!(q & bitd)) continue;
                if (ref == -2) ref = L[q];
                else eq &= (L[q] == ref);
            }
            return !eq;
        };
        SegPlanes P;
        P.f0 = qx & __ballot_sync(0xffffffffu, valid && differ(L[0], L[4]));
        P.f1 = qy & __ballot_sync(0xffffffffu, valid && differ(L[0], L[2]));
        P.f2 = qz & __ballot_sync(0xffffffffu, valid && differ(L[0], L[1]));
        P.v = R00.z0 & __ballot_sync(0xffffffffu, valid && !alleq);
        P.e0 = P.v & Rp0.z0 & __ballot_sync(0xffffffffu, square_differs(4));
        P.e1 = P.v & R0p.z0 & __ballot_sync(0xffffffffu, square_differs(2));
        P.e2 = P.v & R00.p1 & __ballot_sync(0xffffffffu, square_differs(1));
        P.pad = 0;
        if (P.v) {
            mn0 = min(mn0, a);
            mn1 = min(mn1, b);
            mn2 = min(mn2, c0 + __ffs(P.v) - 1);
            mx0 = max(mx0, a);
            mx1 = max(mx1, b);
            mx2 = max(mx2, c0 + 31 - __clz(P.v));
        }
        if (lane == 0) {
            reinterpret_cast<uint4*>(planes + gs)[0] = make_uint4(P.v, P.e0, P.e1, P.e2);
            reinterpret_cast<uint4*>(planes + gs)[1] = make_uint4(P.f0, P.f1, P.f2, 0u);
            cv[gs] = __popc(P.v);
            ce[gs] = __popc(P.e0) + __popc(P.e1) + __popc(P.e2);
            cf[gs] = __popc(P.f0) + __popc(P.f1) + __popc(P.f2);
        }
    }
    flush();
}

// One block per lattice row of the batch, one thread per point (c = a
// multiple of 32 plus the lane, so a warp is one segment): the row's
// vertices (vts and, with records, their thinning records: incident edges
// counted and summed).  Incident edges: the axis edges into the voxel from
// -x, -y, -z, its own axis edges, then the diagonals of the faces (p1, d)
// and (p3, d) that have it as q1 / q3.
__global__ void __launch_bounds__(128) vd_vertices_kernel(VolTab T, Bases B, const SegPlanes* __restrict__ planes,
                                                          const int32_t* __restrict__ vb, const int32_t* __restrict__ eb,
                                                          const int32_t* __restrict__ fbs, float* __restrict__ vts,
                                                          uint32_t* __restrict__ vlat, VertRec* __restrict__ V,
                                                          const EdgeRec* __restrict__ E, int32_t* __restrict__ g0,
                                                          int64_t ne) {
    const int lane = threadIdx.x & 31;
    const int64_t nseg = T.total(kLSeg);
    VolTab::Cache vcache;
    SEG_LOOP(gs, nseg) {
        const int bv = T.find_cached(kLSeg, gs, vcache);
        const Segs S = segs_of(T, bv, planes, vb, eb, fbs);
        const Shift sh = shift_of(B, bv);
        const int nsr_ = (T.dim(bv).z + 32) / 32;
        const int64_t ls_ = gs - T.start(kLSeg, bv);
        const int64_t row = ls_ / nsr_;
        const int c0 = (int)(ls_ - row * nsr_) * 32;
        const int a = (int)(row / S.NB), b = (int)(row - (int64_t)a * S.NB);
        {
            const int c = c0 + lane;
            const int64_t s = S.at(a, b, c);
            const SegPlanes P = load_planes(planes + s);
            if (!bit(P.v, c)) continue;
            const int32_t v = __ldg(vb + s) + __popc(P.v & below(c));
            if (vts) {
                vts[3 * (int64_t)v + 0] = (float)a;
                vts[3 * (int64_t)v + 1] = (float)b;
                vts[3 * (int64_t)v + 2] = (float)c;
            }
            if (vlat) vlat[v] = (uint32_t)((((int64_t)a * S.NB + b) * (T.dim(bv).z + 1)) + c);  // within its volume
            if (!V) continue;
            unsigned k = 0;
            unsigned long long idsum = 0;
            const int p[3] = {a, b, c};
            // each neighbour segment is read once (its edge or face planes)
            auto add_edge = [&](int x, int y, int z, int d) {  // axis edge (x,y,z)+d, if valid
                const int64_t sq = S.at(x, y, z);
                const uint4 pe = __ldg(reinterpret_cast<const uint4*>(planes + sq));  // v e0 e1 e2
                const uint32_t pd = d == 0 ? pe.y : (d == 1 ? pe.z : pe.w);
                if (!bit(pd, z)) return;
                const uint32_t mk = below(z);
                int32_t r = __ldg(eb + sq) + __popc(pe.y & mk) + __popc(pe.z & mk) + __popc(pe.w & mk);
                if (d >= 1) r += bit(pe.y, z);
                if (d >= 2) r += bit(pe.z, z);
                ++k;
                idsum += (unsigned)(r + (int32_t)sh.fb);
            };
            auto add_diag = [&](int x, int y, int z, int d) {  // diagonal of face (x,y,z)+d, if valid
                const int64_t sq = S.at(x, y, z);
                const uint4 pf = __ldg(reinterpret_cast<const uint4*>(planes + sq) + 1);  // f0 f1 f2 -
                const uint32_t pd = d == 0 ? pf.x : (d == 1 ? pf.y : pf.z);
                if (!bit(pd, z)) return;
                const uint32_t mk = below(z);
                int32_t r = __ldg(fbs + sq) + __popc(pf.x & mk) + __popc(pf.y & mk) + __popc(pf.z & mk);
                if (d >= 1) r += bit(pf.x, z);
                if (d >= 2) r += bit(pf.y, z);
                ++k;
                idsum += (unsigned)((int32_t)sh.eb1 + r);
            };
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                if (p[d] == 0) continue;
                int q[3] = {a, b, c};
                q[d] -= 1;
                add_edge(q[0], q[1], q[2], d);
            }
            {
                const uint32_t mk = below(c);
                int32_t r = __ldg(eb + s) + __popc(P.e0 & mk) + __popc(P.e1 & mk) + __popc(P.e2 & mk);
#pragma unroll
                for (int d = 0; d < 3; ++d)
                    if (bit(plane_e(P, d), c)) {
                        ++k;
                        idsum += (unsigned)(r++ + (int32_t)sh.fb);
                    }
            }
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                const int u = (d + 1) % 3, w = (d + 2) % 3;
                int p1[3] = {a, b, c}, p3[3] = {a, b, c};
                p1[w] += 1;  // the vertex is q1 of face (p1, d)
                p3[u] += 1;  // the vertex is q3 of face (p3, d)
                add_diag(p1[0], p1[1], p1[2], d);
                add_diag(p3[0], p3[1], p3[2], d);
            }
            VertRec r;
            r.rs = rs_make(k, 0, idsum);
            r.trig = 0;
            r.rm = kAlive;
            V[v] = r;
            // generation 0: an EV pair when the one edge passes the filter
            // (its record, written before, holds the folded measure)
            g0[ne + v] = (k == 1 && E[idsum].em < 0.0f) ? (int32_t)idsum : -1;
        }
    }
}

// The faces of the axis edge (a,b,c)+d: the valid faces of the plaquette
// shared by voxel (a,b,c) and its +d neighbour, i.e. the lattice edges along
// u from nb and nb + e_w and along w from nb and nb + e_u, nb = (a,b,c) +
// e_d (u = d+1, w = d+2 mod 3).  For each, fn(face id, triangle) is called
// with the triangle of the face that carries the edge (0: (q3,q0,q1),
// 1: (q3,q1,q2)).  Three segment loads.
template <int D, class Fn>
__device__ __forceinline__ void for_plaquette(const Segs& S, int a, int b, int c, Fn fn) {
    constexpr int U = (D + 1) % 3, W = (D + 2) % 3;
    int nb[3] = {a, b, c};
    nb[D] += 1;
    const int v[3] = {a, b, c};
#pragma unroll
    for (int g = 0; g < 3; ++g) {  // g = 0: nb (axes u and w); 1: nb + e_w (axis u); 2: nb + e_u (axis w)
        int cc[3] = {nb[0], nb[1], nb[2]};
        if (g == 1) cc[W] += 1;
        if (g == 2) cc[U] += 1;
        const int64_t sg = S.at(cc[0], cc[1], cc[2]);
        const SegPlanes P = load_planes(S.planes + sg);
        const int z = cc[2];
        const uint32_t m = below(z);
        const int32_t f0 = __ldg(S.fb + sg) + __popc(P.f0 & m) + __popc(P.f1 & m) + __popc(P.f2 & m);
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            if (g == 1 && h == 1) continue;
            if (g == 2 && h == 0) continue;
            const int ax = h == 0 ? U : W;
            if (!bit(plane_f(P, ax), z)) continue;
            const int32_t fid = f0 + (ax >= 1 ? (int)bit(P.f0, z) : 0) + (ax >= 2 ? (int)bit(P.f1, z) : 0);
            // position (s,t) of the edge's lower voxel in the face's quad
            const int u2 = (ax + 1) % 3, w2 = (ax + 2) % 3;
            const int s = v[u2] - (cc[u2] - 1), t = v[w2] - (cc[w2] - 1);
            const int tri = D == u2 ? (t == 0 ? 0 : 1) : (s == 0 ? 0 : 1);
            fn(fid, tri);
        }
    }
}

template <class Fn>
__device__ __forceinline__ void for_plaquette_d(int d, const Segs& S, int a, int b, int c, Fn fn) {
    if (d == 0) for_plaquette<0>(S, a, b, c, fn);
    else if (d == 1) for_plaquette<1>(S, a, b, c, fn);
    else for_plaquette<2>(S, a, b, c, fn);
}

// The row's axis edges: endpoints and, with records, thinning records
// (incident triangles counted, summed and tested against the threshold;
// measure = max lambda of the incident faces, voroinfo.cpp:1490-1538).
// Face lambdas come from lamf (one per face, written by vd_faces_kernel).
__global__ void __launch_bounds__(128, 8) vd_edges_kernel(VolTab T, Bases B, const SegPlanes* __restrict__ planes,
                                                       const int32_t* __restrict__ vb, const int32_t* __restrict__ eb,
                                                       const int32_t* __restrict__ fbs, const float* __restrict__ lamf,
                                                       int2* __restrict__ edges, EdgeRec* __restrict__ E,
                                                       int32_t* __restrict__ g0, const float* __restrict__ thr) {
    const int lane = threadIdx.x & 31;
    const int64_t nseg = T.total(kLSeg);
    VolTab::Cache vcache;
    SEG_LOOP(gs, nseg) {
        const int bv = T.find_cached(kLSeg, gs, vcache);
        const Segs S = segs_of(T, bv, planes, vb, eb, fbs);
        const Shift sh = shift_of(B, bv);
        const int nsr_ = (T.dim(bv).z + 32) / 32;
        const int64_t ls_ = gs - T.start(kLSeg, bv);
        const int64_t row = ls_ / nsr_;
        const int c0 = (int)(ls_ - row * nsr_) * 32;
        const int a = (int)(row / S.NB), b = (int)(row - (int64_t)a * S.NB);
        const float tb = thr ? thr[bv] : 0.0f;
        {
            const int c = c0 + lane;
            const int64_t s = S.at(a, b, c);
            const SegPlanes P = load_planes(planes + s);
            const uint32_t m = below(c);
            if (!bit(P.e0 | P.e1 | P.e2, c)) continue;
            int32_t e = __ldg(eb + s) + __popc(P.e0 & m) + __popc(P.e1 & m) + __popc(P.e2 & m) + (int32_t)sh.fb;
            const int32_t v0 = __ldg(vb + s) + __popc(P.v & m);
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                if (!bit(plane_e(P, d), c)) continue;
                int nb[3] = {a, b, c};
                nb[d] += 1;
                const int32_t v1 = vid_at(S, nb[0], nb[1], nb[2]);
                if (edges) edges[e] = make_int2(v0, v1);
                if (E) {
                    float mx = 0.0f;
                    unsigned k = 0, npass = 0;
                    unsigned long long idsum = 0;
                    for_plaquette_d(d, S, a, b, c, [&](int32_t fid, int tri) {
                        const float lj = __ldg(lamf + fid);
                        mx = fmaxf(mx, lj);
                        npass += lj < tb ? 1u : 0u;
                        idsum += (unsigned)(2 * fid + tri);
                        ++k;
                    });
                    EdgeRec r;
                    r.v0 = v0;
                    r.v1 = v1;
                    r.rs = rs_make(k, npass, idsum);
                    r.trig = 0;
                    r.em = rec_measure(mx, thr, bv);
                    r.rm = kAlive;
                    r.pad = 0;
                    E[e] = r;
                    // generation 0: an FE pair when the one face passes the filter
                    g0[e] = (k == 1 && npass == 1) ? (int32_t)idsum : -1;
                }
                ++e;
            }
        }
    }
}

// The row's faces: two triangles each (util::simpleTriangulate of the quad
// (q0,q1,q2,q3): (q3,q0,q1), (q3,q1,q2)), the diagonal edge (q1,q3) and,
// with records, the thinning records of both triangles and the diagonal.
__global__ void __launch_bounds__(128, 8) vd_faces_kernel(VolTab T, Bases B, const SegPlanes* __restrict__ planes,
                                                       const int32_t* __restrict__ vb, const int32_t* __restrict__ eb,
                                                       const int32_t* __restrict__ fbs, const int32_t* __restrict__ lab,
                                                       const float* __restrict__ sxyz, float* __restrict__ lamf,
                                                       int32_t* __restrict__ tris, int2* __restrict__ edges,
                                                       FaceRec* __restrict__ F, EdgeRec* __restrict__ E,
                                                       int32_t* __restrict__ g0, const float* __restrict__ thr) {
    const int lane = threadIdx.x & 31;
    const int64_t nseg = T.total(kLSeg);
    VolTab::Cache vcache;
    SEG_LOOP(gs, nseg) {
        const int bv = T.find_cached(kLSeg, gs, vcache);
        const Segs S = segs_of(T, bv, planes, vb, eb, fbs);
        const Shift sh = shift_of(B, bv);
        const int32_t* lb = lab + T.start(kLat, bv);
        const int64_t NC = T.dim(bv).z + 1;
        const int nsr_ = (T.dim(bv).z + 32) / 32;
        const int64_t ls_ = gs - T.start(kLSeg, bv);
        const int64_t row = ls_ / nsr_;
        const int c0 = (int)(ls_ - row * nsr_) * 32;
        const int a = (int)(row / S.NB), b = (int)(row - (int64_t)a * S.NB);
        const int32_t fbv = (int32_t)sh.fb;
        {
            const int c = c0 + lane;
            const int64_t s = S.at(a, b, c);
            const SegPlanes P = load_planes(planes + s);
            if (!bit(P.f0 | P.f1 | P.f2, c)) continue;
            const uint32_t m = below(c);
            int32_t f = __ldg(fbs + s) + __popc(P.f0 & m) + __popc(P.f1 & m) + __popc(P.f2 & m);
            const int64_t p = row * NC + c;
            const int32_t l0 = __ldg(lb + p);
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                if (!bit(plane_f(P, d), c)) continue;
                const int u = (d + 1) % 3, w = (d + 2) % 3;
                // the quad's voxels: vertex ids and (q0, q1, q3) their axis-edge
                // ranks, one 16-byte plane load (v, e0, e1, e2) per voxel
                int32_t q[4], er[4];
                uint4 pl[4];
                int qz[4];
#pragma unroll
                for (int mm = 0; mm < 4; ++mm) {
                    int x, y, z;
                    quad_voxel(a, b, c, d, mm, x, y, z);
                    const int64_t sm = S.at(x, y, z);
                    pl[mm] = __ldg(reinterpret_cast<const uint4*>(S.planes + sm));
                    qz[mm] = z;
                    const uint32_t mk = below(z);
                    q[mm] = __ldg(S.vb + sm) + __popc(pl[mm].x & mk);
                    er[mm] = mm == 2 ? 0 : __ldg(S.eb + sm) + __popc(pl[mm].y & mk) + __popc(pl[mm].z & mk) +
                                           __popc(pl[mm].w & mk);
                }
                // rank of voxel mm's axis edge along dd
                auto erank = [&](int mm, int dd) {
                    return er[mm] + (dd >= 1 ? (int)bit(pl[mm].y, qz[mm]) : 0) +
                           (dd >= 2 ? (int)bit(pl[mm].z, qz[mm]) : 0);
                };
                const int32_t diag = (int32_t)sh.eb1 + f;
                const int64_t t0 = 2 * (int64_t)f, t1 = t0 + 1;
                if (tris) {
                    tris[3 * t0 + 0] = q[3];
                    tris[3 * t0 + 1] = q[0];
                    tris[3 * t0 + 2] = q[1];
                    tris[3 * t1 + 0] = q[3];
                    tris[3 * t1 + 1] = q[1];
                    tris[3 * t1 + 2] = q[2];
                }
                const int32_t dv0 = min(q[1], q[3]), dv1 = max(q[1], q[3]);
                if (edges) edges[diag] = make_int2(dv0, dv1);
                // lambda of the face: distance of its two sites (measureforMA_imp.h:1-4)
                const int64_t p1 = p + (d == 0 ? S.NB * NC : (d == 1 ? NC : 1));
                const float lm = lambda_of(sxyz, l0, __ldg(lb + p1));
                lamf[f] = lm;
                if (F) {
                    // sides in traceFace order: (t0,t1), (t1,t2), (t2,t0)
                    const int32_t e01 = erank(0, u) + fbv;
                    const int32_t e12 = erank(1, w) + fbv;
                    const int32_t e32 = erank(3, u) + fbv;
                    const int32_t e03 = erank(0, w) + fbv;
                    const float lr = rec_measure(lm, thr, bv);
                    const int32_t pass = lr < 0.0f ? kFacePass : 0;
                    // both triangles' records: one 32-byte sector
                    FaceRec fr;
                    fr.rm = kAlive;
                    fr.e0 = e03;
                    fr.e1 = e01;
                    fr.e2 = diag | pass;
                    F[t0] = fr;
                    fr.e0 = diag;
                    fr.e1 = e12;
                    fr.e2 = e32 | pass;
                    F[t1] = fr;
                    EdgeRec er;
                    er.v0 = dv0;
                    er.v1 = dv1;
                    er.rs = rs_make(2, lm < thr[bv] ? 2u : 0u, (unsigned long long)t0 + (unsigned long long)t1);
                    er.trig = 0;
                    er.em = lr;
                    er.rm = kAlive;
                    er.pad = 0;
                    E[diag] = er;
                    g0[diag] = -1;  // two triangles: no FE pair
                }
                ++f;
            }
        }
    }
}

// The complex's arrays that only its getters read (vc_get_vd,
// vc_get_finalized) or that a thinning with explicit thresholds rebuilds
// its records from: vertex measure (max lambda over the valid faces of the
// voxel's 12 cube edges), edge measures, triangle measures, each triangle's
// face, each face's two sites and the triangles' sides.  Written on demand.
__global__ void __launch_bounds__(128) vd_aux_kernel(VolTab T, Bases B, const SegPlanes* __restrict__ planes,
                                                     const int32_t* __restrict__ vb, const int32_t* __restrict__ eb,
                                                     const int32_t* __restrict__ fbs, const int32_t* __restrict__ lab,
                                                     const float* __restrict__ lamf, float* __restrict__ vm,
                                                     float* __restrict__ em, float* __restrict__ fm,
                                                     int32_t* __restrict__ tri_face, int2* __restrict__ face_sites,
                                                     int32_t* __restrict__ tri_edges) {
    const int lane = threadIdx.x & 31;
    const int64_t nseg = T.total(kLSeg);
    VolTab::Cache vcache;
    SEG_LOOP(gs, nseg) {
        const int bv = T.find_cached(kLSeg, gs, vcache);
        const Segs S = segs_of(T, bv, planes, vb, eb, fbs);
        const Shift sh = shift_of(B, bv);
        const int64_t lat0 = T.start(kLat, bv);
        const int32_t* lb = lab + lat0;
        const int64_t NC = T.dim(bv).z + 1;
        const int nsr_ = (T.dim(bv).z + 32) / 32;
        const int64_t ls_ = gs - T.start(kLSeg, bv);
        const int64_t row = ls_ / nsr_;
        const int c0 = (int)(ls_ - row * nsr_) * 32;
        const int a = (int)(row / S.NB), b = (int)(row - (int64_t)a * S.NB);
        const int32_t fbv = (int32_t)sh.fb;
        auto lid = [&](int x, int y, int z) { return ((int64_t)x * S.NB + y) * NC + z; };
        {
            const int c = c0 + lane;
            const int64_t s = S.at(a, b, c);
            const SegPlanes P = load_planes(planes + s);
            const uint32_t m = below(c);
            const int64_t p = row * NC + c;
            if (bit(P.v, c)) {
                const int32_t v = __ldg(vb + s) + __popc(P.v & m);
                float mv = 0.0f;
#pragma unroll
                for (int d = 0; d < 3; ++d)
#pragma unroll
                    for (int s2 = 0; s2 < 2; ++s2)
#pragma unroll
                        for (int t2 = 0; t2 < 2; ++t2) {
                            int q[3] = {a, b, c};
                            q[(d + 1) % 3] += s2;
                            q[(d + 2) % 3] += t2;
                            if (fbit_at(S, q[0], q[1], q[2], d))
                                mv = fmaxf(mv, __ldg(lamf + fid_at(S, q[0], q[1], q[2], d)));
                        }
                vm[v] = mv;
            }
            if (bit(P.e0 | P.e1 | P.e2, c)) {
                int32_t e = __ldg(eb + s) + __popc(P.e0 & m) + __popc(P.e1 & m) + __popc(P.e2 & m) + fbv;
#pragma unroll
                for (int d = 0; d < 3; ++d) {
                    if (!bit(plane_e(P, d), c)) continue;
                    float mx = 0.0f;
                    for_plaquette_d(d, S, a, b, c, [&](int32_t fid, int) { mx = fmaxf(mx, __ldg(lamf + fid)); });
                    em[e++] = mx;
                }
            }
            if (bit(P.f0 | P.f1 | P.f2, c)) {
                int32_t f = __ldg(fbs + s) + __popc(P.f0 & m) + __popc(P.f1 & m) + __popc(P.f2 & m);
#pragma unroll
                for (int d = 0; d < 3; ++d) {
                    if (!bit(plane_f(P, d), c)) continue;
                    const int u = (d + 1) % 3, w = (d + 2) % 3;
                    int qv[4][3];
#pragma unroll
                    for (int mm = 0; mm < 4; ++mm) quad_voxel(a, b, c, d, mm, qv[mm][0], qv[mm][1], qv[mm][2]);
                    const int32_t diag = (int32_t)sh.eb1 + f;
                    const int32_t e01 = erank_at(S, qv[0][0], qv[0][1], qv[0][2], u) + fbv;
                    const int32_t e12 = erank_at(S, qv[1][0], qv[1][1], qv[1][2], w) + fbv;
                    const int32_t e32 = erank_at(S, qv[3][0], qv[3][1], qv[3][2], u) + fbv;
                    const int32_t e03 = erank_at(S, qv[0][0], qv[0][1], qv[0][2], w) + fbv;
                    const int64_t t0 = 2 * (int64_t)f, t1 = t0 + 1;
                    tri_edges[3 * t0 + 0] = e03;
                    tri_edges[3 * t0 + 1] = e01;
                    tri_edges[3 * t0 + 2] = diag;
                    tri_edges[3 * t1 + 0] = diag;
                    tri_edges[3 * t1 + 1] = e12;
                    tri_edges[3 * t1 + 2] = e32;
                    const float lm = __ldg(lamf + f);
                    fm[t0] = lm;
                    fm[t1] = lm;
                    tri_face[t0] = f - fbv;
                    tri_face[t1] = f - fbv;
                    em[diag] = lm;
                    int e1[3] = {a, b, c};
                    e1[d] += 1;
                    face_sites[f] = make_int2(lb[p] - (int32_t)sh.site, lb[lid(e1[0], e1[1], e1[2])] - (int32_t)sh.site);
                    ++f;
                }
            }
        }
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

// FP64 cross-check of the face measures (the report of an FP32 path with
// FP64 rescue): every face's lambda recomputed in double from its two
// sites; out[0] = the largest relative difference to the float lambda the
// path uses (as the bits of a non-negative double, so atomicMax orders
// them), out[1] = how many faces' threshold test (lambda < the volume's
// thinning threshold) comes out differently in double (thr null: not
// counted).  The path keeps the reference's float semantics either way.
__global__ void lambda_fp64_kernel(const int2* __restrict__ face_sites, const float* __restrict__ sxyz, Bases B,
                                   int nvol, const float* __restrict__ lamf, const float* __restrict__ thr,
                                   int64_t nface, unsigned long long* out) {
    double worst = 0.0;
    unsigned long long flips = 0;
    for (int64_t f = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; f < nface; f += (int64_t)gridDim.x * blockDim.x) {
        const int bv = nvol > 1 ? find_base(B.b[kBFace], nvol, f) : 0;
        const int64_t sb = B.b[kBSite][bv];
        const int2 st = face_sites[f];
        const int64_t s0 = sb + st.x, s1 = sb + st.y;
        const double dx = (double)sxyz[3 * s0] - (double)sxyz[3 * s1];
        const double dy = (double)sxyz[3 * s0 + 1] - (double)sxyz[3 * s1 + 1];
        const double dz = (double)sxyz[3 * s0 + 2] - (double)sxyz[3 * s1 + 2];
        const double l64 = sqrt(dx * dx + dy * dy + dz * dz);
        const float l32 = lamf[f];
        if (l64 > 0.0) worst = fmax(worst, fabs((double)l32 - l64) / l64);
        if (thr && ((double)l32 < (double)thr[bv]) != (l64 < (double)thr[bv])) ++flips;
    }
    const unsigned long long wb = (unsigned long long)__double_as_longlong(worst);
    atomicMax(out, wb);
    if (flips) atomicAdd(out + 1, flips);
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
                                 const float* __restrict__ sxyz, const float* __restrict__ vts, Bases B, int32_t nv,
                                 float* __restrict__ radius) {
    for (int32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < nv; v += gridDim.x * blockDim.x) {
        // the vertex's volume: the last one whose first vertex is <= v
        int bv = 0;
        if (T.nvol > 1) {
            int lo = 0, hi = T.nvol - 1;
            while (lo < hi) {
                const int mid = (lo + hi + 1) >> 1;
                if (B.b[kBVert][mid] <= v) lo = mid;
                else hi = mid - 1;
            }
            bv = lo;
        }
        const Grid g = grid_of(T, bv, occ, lab);
        const int a = (int)vts[3 * (int64_t)v + 0], b = (int)vts[3 * (int64_t)v + 1], c = (int)vts[3 * (int64_t)v + 2];
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

// 128-thread blocks, kSegChunk segments per block at a time (grid-stride)
inline int seg_grid(vc_ctx* c, int64_t nseg) {
    return (int)std::max<int64_t>(1, std::min<int64_t>((nseg + kSegChunk - 1) / kSegChunk, (int64_t)c->num_sms * 16));
}

}  // namespace

int build_adjacency(vc_ctx* c);

// t_thr >= 0: also compute every volume's thinning threshold float(size *
// t_thr) and write the thinning records with it folded in (see
// rec_measure); otherwise the thinning builds its records when it runs.
int run_lattice_vd(vc_ctx* c, vc_vd_sizes* sizes, double t_thr) {
    if (!c->ft_valid) return VC_ERR_STATE;
    const int nvol = c->nvol;
    for (int b = 0; b < nvol; ++b)
        if (space_size(kLat, c->h_dims[3 * b], c->h_dims[3 * b + 1], c->h_dims[3 * b + 2]) >= ((int64_t)1 << 32))
            return VC_ERR_ARG;
    const int64_t N = c->h_off[kLat][nvol];
    const int64_t nseg = c->h_off[kLSeg][nvol];
    Region stage(c, "stage_vd");
    VC_TRY(ensure_n<SegPlanes>(c, c->vd_seg, nseg));
    VC_TRY(ensure_n<int32_t>(c, c->vd_voff, nseg));
    VC_TRY(ensure_n<int32_t>(c, c->vd_eoff, nseg));
    VC_TRY(ensure_n<int32_t>(c, c->vd_foff, nseg));
    VC_TRY(ensure_n<int64_t>(c, c->scratch2, 8));
    SegPlanes* planes = ptr<SegPlanes>(c->vd_seg);
    int32_t* vb = ptr<int32_t>(c->vd_voff);
    int32_t* eb = ptr<int32_t>(c->vd_eoff);
    int32_t* fb = ptr<int32_t>(c->vd_foff);
    init_bbox_kernel<<<(6 * nvol + 255) / 256, 256, 0, c->stream>>>(c->bases.bbox, nvol);
    launched(c);
    {
        Region r(c, "vd_flags");
        // the packed occupancy words of the site extraction (same volumes)
        vd_segments_kernel<<<seg_grid(c, nseg), 128, 0, c->stream>>>(ptr<uint32_t>(c->site_bits),
                                                                       ptr<int32_t>(c->ft_id), c->tab, planes, vb, eb,
                                                                       fb, c->bases.bbox);
        launched(c);
        VC_CUDA(c, cudaGetLastError());
    }
    int64_t* tot = ptr<int64_t>(c->scratch2);
    {
        Region r(c, "vd_scan");
        int32_t* cnt[3] = {vb, eb, fb};
        const int base_of[3] = {kBVert, kBAxis, kBFace};
        for (int k = 0; k < 3; ++k) {
            VC_TRY(scan_exclusive_i32(c, cnt[k], cnt[k], nseg, tot + k));
            VC_TRY(fill_bases(c, base_of[k], kLSeg, cnt[k], tot + k));
        }
        inside_size_kernel<<<(nvol + 255) / 256, 256, 0, c->stream>>>(c->bases, nvol, t_thr);
        launched(c);
    }
    int64_t h[3];
    VC_CUDA(c, cudaMemcpyAsync(h, tot, 3 * sizeof(int64_t), cudaMemcpyDeviceToHost, c->stream));
    VC_TRY(sync_check(c));
    const int64_t nv = h[0], ne_axis = h[1], nface = h[2];
    const int64_t ne = ne_axis + nface, nt = 2 * nface;
    if (ne >= INT32_MAX || 3 * nt >= INT32_MAX || nv >= INT32_MAX) return VC_ERR_ARG;
    // the complex becomes the context's finalized cell complex
    c->cc_valid = c->cc_finalized = c->meas_valid = c->thin_valid = c->rem_valid = false;
    c->records_fresh = false;
    c->vd_aux_meas = c->vd_aux_topo = false;
    const bool folded = t_thr >= 0.0;
    // The path that thins at once (records with the thresholds folded in)
    // writes no vertex, edge or triangle arrays: the thinning and the
    // remaining complex read the records, and the arrays are written on
    // demand for the getters (ensure_vd_geometry).
    const bool geom = !folded;
    c->vd_geom = false;
    if (geom) {
        VC_TRY(ensure_n<float>(c, c->vts, 3 * nv));
        VC_TRY(ensure_n<int2>(c, c->edges, ne));
        VC_TRY(ensure_n<int32_t>(c, c->tris, 3 * nt));
    } else {
        VC_TRY(ensure_n<uint32_t>(c, c->vd_vlat, nv));  // each vertex's lattice point, for the remaining complex
    }
    VC_TRY(ensure_n<float>(c, c->vd_lam, nface));  // lambda per face
    if (folded) {
        VC_TRY(ensure_n<FaceRec>(c, c->face_rec, nt));
        VC_TRY(ensure_n<EdgeRec>(c, c->edge_rec, ne));
        VC_TRY(ensure_n<VertRec>(c, c->vert_rec, nv));
        VC_TRY(ensure_n<int32_t>(c, c->thin_g0, nv + ne));
    }
    const float* thr = folded ? c->bases.thr : nullptr;
    {
        Region r(c, "vd_emit");
        int32_t* g0 = folded ? ptr<int32_t>(c->thin_g0) : nullptr;
        {
            Region k(c, "vd_faces");
            vd_faces_kernel<<<seg_grid(c, nseg), 128, 0, c->stream>>>(
                c->tab, c->bases, planes, vb, eb, fb, ptr<int32_t>(c->ft_id), ptr<float>(c->site_xyz),
                ptr<float>(c->vd_lam), geom ? ptr<int32_t>(c->tris) : nullptr, geom ? ptr<int2>(c->edges) : nullptr,
                folded ? ptr<FaceRec>(c->face_rec) : nullptr, folded ? ptr<EdgeRec>(c->edge_rec) : nullptr, g0, thr);
            launched(c);
        }
        {
            Region k(c, "vd_edges");
            vd_edges_kernel<<<seg_grid(c, nseg), 128, 0, c->stream>>>(
                c->tab, c->bases, planes, vb, eb, fb, ptr<float>(c->vd_lam), geom ? ptr<int2>(c->edges) : nullptr,
                folded ? ptr<EdgeRec>(c->edge_rec) : nullptr, g0, thr);
            launched(c);
        }
        {
            Region k(c, "vd_vertices");
            vd_vertices_kernel<<<seg_grid(c, nseg), 128, 0, c->stream>>>(
                c->tab, c->bases, planes, vb, eb, fb, geom ? ptr<float>(c->vts) : nullptr,
                geom ? nullptr : ptr<uint32_t>(c->vd_vlat), folded ? ptr<VertRec>(c->vert_rec) : nullptr,
                folded ? ptr<EdgeRec>(c->edge_rec) : nullptr, g0, ne);
            launched(c);
        }
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
    c->vd_geom = geom;
    c->cc_valid = true;
    c->cc_finalized = true;
    c->meas_valid = true;  // written on demand (ensure_vd_aux)
    c->records_fresh = folded;
    c->records_thr_folded = folded;
    c->vd_thr_valid = folded;
    c->cc_batched = nvol > 1;
    if (sizes) *sizes = c->vd;
    return VC_OK;
}

// The lattice complex's vertex, edge and triangle arrays when the fast path
// did not write them: the emission kernels run again, writing only those.
int ensure_vd_geometry(vc_ctx* c) {
    if (!c->vd_valid || c->vd_geom) return VC_OK;
    const int64_t nv = c->vd.nv, ne = c->vd.ne, nt = c->vd.nt;
    const int64_t nseg = c->h_off[kLSeg][c->nvol];
    VC_TRY(ensure_n<float>(c, c->vts, 3 * nv));
    VC_TRY(ensure_n<int2>(c, c->edges, ne));
    VC_TRY(ensure_n<int32_t>(c, c->tris, 3 * nt));
    const SegPlanes* planes = ptr<SegPlanes>(c->vd_seg);
    const int32_t *vb = ptr<int32_t>(c->vd_voff), *eb = ptr<int32_t>(c->vd_eoff), *fb = ptr<int32_t>(c->vd_foff);
    Region r(c, "vd_geometry");
    vd_faces_kernel<<<seg_grid(c, nseg), 128, 0, c->stream>>>(
        c->tab, c->bases, planes, vb, eb, fb, ptr<int32_t>(c->ft_id), ptr<float>(c->site_xyz), ptr<float>(c->vd_lam),
        ptr<int32_t>(c->tris), ptr<int2>(c->edges), nullptr, nullptr, nullptr, nullptr);
    vd_edges_kernel<<<seg_grid(c, nseg), 128, 0, c->stream>>>(c->tab, c->bases, planes, vb, eb, fb,
                                                               ptr<float>(c->vd_lam), ptr<int2>(c->edges), nullptr,
                                                               nullptr, nullptr);
    vd_vertices_kernel<<<seg_grid(c, nseg), 128, 0, c->stream>>>(c->tab, c->bases, planes, vb, eb, fb,
                                                                  ptr<float>(c->vts), nullptr, nullptr, nullptr,
                                                                  nullptr, ne);
    launched(c, 3);
    VC_CUDA(c, cudaGetLastError());
    c->vd_geom = true;
    return VC_OK;
}

namespace {

// Lattice point (a, b, c) of vertex v, from the lattice index the vertex
// kernel recorded (within the vertex's volume).
__device__ __forceinline__ void lattice_vertex(const VolTab& T, const Bases& B, int nvol,
                                               const uint32_t* __restrict__ vlat, int32_t v, float* o) {
    const int bv = nvol > 1 ? find_base(B.b[kBVert], nvol, v) : 0;
    const int4 d = T.dim(bv);
    const uint32_t p = __ldg(vlat + v);
    const uint32_t NC = (uint32_t)d.z + 1u, NB = (uint32_t)d.y + 1u;
    const uint32_t ab = p / NC;
    o[0] = (float)(ab / NB);
    o[1] = (float)(ab % NB);
    o[2] = (float)(p % NC);
}

// remainingCC of the lattice complex from the thinning records: a kept
// vertex's coordinates from its lattice point, a kept edge's ends from its record,
// a kept triangle's corners from the records of its first two sides (sides
// (a,b), (b,c), (c,a) in face order: b is the vertex the first two share).
__global__ void vd_rem_write_kernel(int32_t nv, int32_t ne, int32_t nt, Kept K, VolTab T, int nvol,
                                    const uint32_t* __restrict__ vlat, const EdgeRec* __restrict__ E,
                                    const FaceRec* __restrict__ F,
                                    float* __restrict__ ovts, int2* __restrict__ oedges, int32_t* __restrict__ otris,
                                    Bases B, int nmap) {
    const int lane = threadIdx.x & 31;
    const uint32_t lowm = (1u << lane) - 1u;
    const int64_t nwv = ((int64_t)nv + 31) / 32, nwe = ((int64_t)ne + 31) / 32, nwf = ((int64_t)nt + 31) / 32;
    const int64_t nw = nwv + nwe + nwf;
    const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
    for (int64_t w = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); w < nw; w += warps) {
        if (w < nwv) {
            const uint32_t word = __ldg(K.bv + w);
            if (!((word >> lane) & 1u)) continue;
            const int64_t o = __ldg(K.pv + w) + __popc(word & lowm);
            lattice_vertex(T, B, nvol, vlat, (int32_t)(w * 32 + lane), ovts + 3 * o);
        } else if (w < nwv + nwe) {
            const int64_t we = w - nwv;
            const uint32_t word = __ldg(K.be + we);
            if (!((word >> lane) & 1u)) continue;
            const int4 er = __ldg(reinterpret_cast<const int4*>(E + we * 32 + lane));  // v0 v1 rm em
            const int32_t sh = nmap > 1 ? (int32_t)B.b[kBRemV][find_base(B.b[kBVert], nmap, er.x)] : 0;
            oedges[__ldg(K.pe + we) + __popc(word & lowm)] =
                make_int2(kept_rank(K.bv, K.pv, er.x) - sh, kept_rank(K.bv, K.pv, er.y) - sh);
        } else {
            const int64_t wf = w - nwv - nwe;
            const uint32_t word = __ldg(K.bf + wf);
            if (!((word >> lane) & 1u)) continue;
            const int64_t f = wf * 32 + lane;
            const int64_t o = __ldg(K.pf + wf) + __popc(word & lowm);
            const int4 fr = __ldg(reinterpret_cast<const int4*>(F + f));  // e0 e1 e2|pass rm
            const int2 s0 = *reinterpret_cast<const int2*>(E + fr.x);
            const int2 s1 = *reinterpret_cast<const int2*>(E + fr.y);
            const int32_t vb_ = (s0.x == s1.x || s0.x == s1.y) ? s0.x : s0.y;
            const int32_t va = s0.x == vb_ ? s0.y : s0.x;
            const int32_t vc = s1.x == vb_ ? s1.y : s1.x;
            const int32_t sh = nmap > 1 ? (int32_t)B.b[kBRemV][find_base(B.b[kBVert], nmap, va)] : 0;
            // simpleTriangulate turns (a, b, c) into (c, a, b)
            otris[3 * o + 0] = kept_rank(K.bv, K.pv, vc) - sh;
            otris[3 * o + 1] = kept_rank(K.bv, K.pv, va) - sh;
            otris[3 * o + 2] = kept_rank(K.bv, K.pv, vb_) - sh;
        }
    }
}

}  // namespace

int lattice_rem_write(vc_ctx* c, const Kept& K, int nmap) {
    const int64_t nv = c->nv, ne = c->ne, nt = c->nt;
    const int64_t nw = (nv + 31) / 32 + (ne + 31) / 32 + (nt + 31) / 32;
    vd_rem_write_kernel<<<cell_grid(c, 32 * nw), 256, 0, c->stream>>>(
        (int32_t)nv, (int32_t)ne, (int32_t)nt, K, c->tab, c->nvol, ptr<uint32_t>(c->vd_vlat),
        ptr<EdgeRec>(c->edge_rec), ptr<FaceRec>(c->face_rec), ptr<float>(c->rem_vts),
        ptr<int2>(c->rem_edges), ptr<int32_t>(c->rem_tris), c->bases, nmap);
    launched(c);
    VC_CUDA(c, cudaGetLastError());
    return VC_OK;
}

// Write the lattice complex's on-demand arrays: with meas, vm / em / fm /
// tri_face / face_sites; with topo, tri_edges and the V->E / E->F lists
// (cellcomplex::finalize's adjacency, built from edges and tri_edges).
// Nothing to do for a complex that did not come from the lattice.
int ensure_vd_aux(vc_ctx* c, bool meas, bool topo) {
    if (!c->vd_valid) return VC_OK;
    const bool need_meas = meas && !c->vd_aux_meas;
    const bool need_topo = topo && !c->vd_aux_topo;
    if (!need_meas && !need_topo) return VC_OK;
    if (need_topo) VC_TRY(ensure_vd_geometry(c));  // the adjacency is built from the edges
    const int64_t nv = c->nv, ne = c->ne, nt = c->nt, nface = c->vd.nface;
    // the kernel writes both groups; a group already written (possibly by
    // vc_set_measures) goes to scratch copies so it is not overwritten
    VC_TRY(ensure_n<float>(c, c->vm, nv));
    VC_TRY(ensure_n<float>(c, c->em, ne));
    VC_TRY(ensure_n<float>(c, c->fm, nt));
    VC_TRY(ensure_n<int32_t>(c, c->vd_tri_face, nt));
    VC_TRY(ensure_n<int2>(c, c->vd_face_sites, nface));
    VC_TRY(ensure_n<int32_t>(c, c->tri_edges, 3 * nt));
    float *vm = ptr<float>(c->vm), *em = ptr<float>(c->em), *fm = ptr<float>(c->fm);
    int32_t* te = ptr<int32_t>(c->tri_edges);
    if (!need_meas) {
        VC_TRY(ensure_n<uint8_t>(c, c->ft_tmp, (nv + ne + nt) * (int64_t)sizeof(float)));
        vm = ptr<float>(c->ft_tmp);
        em = vm + nv;
        fm = em + ne;
    }
    if (!need_topo) {
        VC_TRY(ensure_n<int32_t>(c, c->scratch, 3 * nt));
        te = ptr<int32_t>(c->scratch);
    }
    {
        Region r(c, "vd_aux");
        vd_aux_kernel<<<seg_grid(c, c->h_off[kLSeg][c->nvol]), 128, 0, c->stream>>>(
            c->tab, c->bases, ptr<SegPlanes>(c->vd_seg), ptr<int32_t>(c->vd_voff), ptr<int32_t>(c->vd_eoff),
            ptr<int32_t>(c->vd_foff), ptr<int32_t>(c->ft_id), ptr<float>(c->vd_lam), vm, em, fm,
            ptr<int32_t>(c->vd_tri_face), ptr<int2>(c->vd_face_sites), te);
        launched(c);
        VC_CUDA(c, cudaGetLastError());
    }
    if (need_meas) c->vd_aux_meas = true;
    if (need_topo) {
        VC_TRY(build_adjacency(c));
        c->vd_aux_topo = true;
    }
    return VC_OK;
}

int run_lambda_check(vc_ctx* c, double* max_rel_err, int64_t* flips) {
    if (!c->vd_valid) return VC_ERR_STATE;
    VC_TRY(ensure_vd_aux(c, true, false));  // the faces' sites
    VC_TRY(ensure_n<int64_t>(c, c->scratch2, 4));
    unsigned long long* out = reinterpret_cast<unsigned long long*>(ptr<int64_t>(c->scratch2));
    VC_CUDA(c, cudaMemsetAsync(out, 0, 2 * sizeof(unsigned long long), c->stream));
    const int64_t nface = c->vd.nface;
    if (nface > 0) {
        lambda_fp64_kernel<<<cell_grid(c, nface), 256, 0, c->stream>>>(
            ptr<int2>(c->vd_face_sites), ptr<float>(c->site_xyz), c->bases, c->nvol, ptr<float>(c->vd_lam),
            c->vd_thr_valid ? c->bases.thr : nullptr, nface, out);
        launched(c);
        VC_CUDA(c, cudaGetLastError());
    }
    unsigned long long h[2] = {0, 0};
    VC_CUDA(c, cudaMemcpyAsync(h, out, sizeof(h), cudaMemcpyDeviceToHost, c->stream));
    VC_TRY(sync_check(c));
    double w;
    std::memcpy(&w, &h[0], sizeof(w));
    *max_rel_err = w;
    *flips = c->vd_thr_valid ? (int64_t)h[1] : -1;
    return VC_OK;
}

int run_vertex_radii(vc_ctx* c) {
    if (!c->vd_valid || !c->ft_valid) return VC_ERR_STATE;
    VC_TRY(ensure_vd_geometry(c));
    const int64_t nv = c->vd.nv;
    VC_TRY(ensure_n<float>(c, c->vd_radius, nv));
    if (nv == 0) return VC_OK;
    Region r(c, "vd_radius");
    vd_radius_kernel<<<cell_grid(c, nv), 256, 0, c->stream>>>(ptr<uint8_t>(c->occ), ptr<int32_t>(c->ft_id), c->tab,
                                                              ptr<float>(c->site_xyz), ptr<float>(c->vts), c->bases,
                                                              (int32_t)nv, ptr<float>(c->vd_radius));
    launched(c);
    VC_CUDA(c, cudaGetLastError());
    return VC_OK;
}

}  // namespace vc
