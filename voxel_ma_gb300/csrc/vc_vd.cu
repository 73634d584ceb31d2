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
// (faces, then vertices with axis edges) walk lattice rows, a warp per row
// and one lane per face or per point of a segment (so writes of consecutive
// ids are coalesced), and write what the thinning and the remaining complex
// read: the thinning records and each vertex's lattice point, or, on
// demand, vertex coordinates, edges and triangles.  The measures, triangle
// faces, face sites, triangle sides and adjacency lists are written on
// demand (ensure_vd_aux), when a getter or a thinning with explicit
// thresholds asks for them.
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
__device__ __forceinline__ bool fbit_at(const Segs& S, int a, int b, int c, int d) {
    return bit(plane_f(load_planes(S.planes + S.at(a, b, c)), d), c);
}

// Segment loop of the getter-only kernel: each block takes kSegChunk
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

// Row loop of the row-walking kernels: each block takes kRowChunk
// consecutive lattice rows at a time and its warps take every fourth one, so
// the neighbouring rows that warps of a block read at once stay in its L1.
constexpr int kRowChunk = 16;
#define ROW_LOOP(gr, nrow)                                                                                 \
    for (int64_t row_base_ = (int64_t)blockIdx.x * kRowChunk; row_base_ < (nrow);                          \
         row_base_ += (int64_t)gridDim.x * kRowChunk)                                                        \
        for (int64_t gr = row_base_ + (threadIdx.x >> 5), row_end_ = min((int64_t)(nrow), row_base_ + kRowChunk); \
             gr < row_end_; gr += blockDim.x >> 5)

// Per lattice point: whether its voxel is a vertex (inside, not all 8
// corner labels equal -- tagVert plus "corner of some Voronoi face"),
// whether each axis edge is valid (both voxels inside, the shared square's
// 4 labels not all equal) and whether each lattice edge carries a valid
// face (labels differ and the 4 voxels around it inside).  One warp per
// lattice row, walking its 32-point segments in order, lane = point: the
// occupancy tests run for the whole segment at once on the packed voxel
// words (bit t of a row's word = voxel c0 + t; shifted copies give
// c0 + t - 1 and c0 + t + 1).  Lanes 0-5 each own one of the six voxel rows
// around the lattice row and carry its words; shuffles hand the combined
// words to the warp.  The label tests run per lane on four label rows (the
// c + 1 labels come from the next lane, and for lane 31 from the next
// segment's labels); labels and words are requested two segments ahead of
// the one computed.  Ballots turn the tests into bit planes.  Also the
// volumes' vertex bounding boxes (VoroInfo::getInsidePartSize reads them).
__global__ void __launch_bounds__(128, 6) vd_segments_kernel(const uint32_t* __restrict__ obits,
                                                             const int32_t* __restrict__ lab, VolTab T,
                                                             SegPlanes* __restrict__ planes, int32_t* __restrict__ cv,
                                                             int32_t* __restrict__ ce, int32_t* __restrict__ cf,
                                                             int32_t* __restrict__ bbox_all) {
    const unsigned full = 0xffffffffu;
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
    // voxel row owned by lanes 0-5: (a-1,b-1), (a-1,b), (a,b-1), (a,b), (a+1,b), (a,b+1)
    const int di = (lane == 0 || lane == 1) ? -1 : (lane == 4 ? 1 : 0);
    const int dj = (lane == 0 || lane == 2) ? -1 : (lane == 5 ? 1 : 0);
    const int64_t nrow = T.total(kLRow);
    VolTab::Cache vcache;
    ROW_LOOP(gr, nrow) {
        const int bv = T.find_cached(kLRow, gr, vcache);
        if (bv != cur_bv) {
            flush();
            cur_bv = bv;
        }
        const int4 dm = T.dim(bv);
        const int X = dm.x, Y = dm.y, Z = dm.z;
        const int NB = Y + 1, NC = Z + 1;
        const int nsr = (Z + 32) / 32, Wz = (Z + 31) >> 5;
        const int lr = (int)(gr - T.start(kLRow, bv));
        const int a = lr / NB, b = lr - a * NB;
        const int64_t seg_row = T.start(kLSeg, bv) + (int64_t)lr * nsr;
        // this lane's voxel row (lanes 0-5), or none
        const int ri = a + di, rj = b + dj;
        const bool rok = lane < 6 && ri >= 0 && ri < X && rj >= 0 && rj < Y;
        const uint32_t* rp = obits + T.start(kVWord, bv) + (rok ? ((int64_t)ri * Y + rj) * Wz : 0);
        auto wload = [&](int w) -> uint32_t { return (rok && w < Wz) ? __ldg(rp + w) : 0u; };
        // label rows (a,b), (a,b+1), (a+1,b), (a+1,b+1): corners 0, 2, 4, 6 of the voxel
        const int32_t* l0 = lab + T.start(kLat, bv) + ((int64_t)a * NB + b) * NC;
        const bool ok2 = b + 1 <= Y, ok4 = a + 1 <= X, ok6 = ok2 && ok4;
        const int32_t* l2 = l0 + (ok2 ? NC : 0);
        const int32_t* l4 = l0 + (ok4 ? (int64_t)NB * NC : 0);
        const int32_t* l6 = l0 + (ok6 ? (int64_t)NB * NC + NC : 0);
        // labels (corners 0, 2, 4, 6 at the lane's point) and voxel words of
        // segments k (L*, wcur), k + 1 (M*, w1) and k + 2 (N*, w2)
        int32_t L0, L2, L4, L6, M0, M2, M4, M6, N0, N2, N4, N6;
        auto lrow = [&](int cc, int32_t& x0, int32_t& x2, int32_t& x4, int32_t& x6) {
            const bool v = cc < NC;
            x0 = v ? __ldg(l0 + cc) : -1;
            x2 = (v && ok2) ? __ldg(l2 + cc) : -1;
            x4 = (v && ok4) ? __ldg(l4 + cc) : -1;
            x6 = (v && ok6) ? __ldg(l6 + cc) : -1;
        };
        lrow(lane, L0, L2, L4, L6);
        lrow(32 + lane, M0, M2, M4, M6);
        uint32_t wprv = 0u, wcur = wload(0), w1 = wload(1);
        int zlo = -1, zhi = -1;  // first and last vertex point of the row
        for (int k = 0; k < nsr; ++k) {
            const int c0 = k * 32, c = c0 + lane;
            lrow(c + 64, N0, N2, N4, N6);
            const uint32_t w2 = wload(k + 2);
            const bool valid = c < NC;
            // bit t: voxel c0 + t - 1 / c0 + t / c0 + t + 1 inside, for this lane's voxel row
            const uint32_t z0 = wcur;
            const uint32_t m1 = (wcur << 1) | (wprv >> 31);
            const uint32_t p1 = (wcur >> 1) | (w1 << 31);
            const uint32_t g = m1 & z0;  // voxels c - 1 and c
            const uint32_t g0m = __shfl_sync(full, g, 2), gm0 = __shfl_sync(full, g, 1), g00 = __shfl_sync(full, g, 3);
            const uint32_t zmm = __shfl_sync(full, z0, 0), zm0 = __shfl_sync(full, z0, 1);
            const uint32_t z0m = __shfl_sync(full, z0, 2), z00 = __shfl_sync(full, z0, 3);
            const uint32_t zp0 = __shfl_sync(full, z0, 4), z0p = __shfl_sync(full, z0, 5);
            const uint32_t p00 = __shfl_sync(full, p1, 3);
            const uint32_t qx = g0m & g00;              // voxels (a, b-1..b, c-1..c)
            const uint32_t qy = gm0 & g00;              // voxels (a-1..a, b, c-1..c)
            const uint32_t qz = zmm & zm0 & z0m & z00;  // voxels (a-1..a, b-1..b, c)
            // labels of the voxel's 8 corners (a + qx, b + qy, c + qz), -1 outside the lattice
            int32_t L[8];
            L[0] = L0;
            L[2] = L2;
            L[4] = L4;
            L[6] = L6;
            {
                const int32_t nx0 = __shfl_sync(full, M0, 0), nx2 = __shfl_sync(full, M2, 0);
                const int32_t nx4 = __shfl_sync(full, M4, 0), nx6 = __shfl_sync(full, M6, 0);
                L[1] = __shfl_down_sync(full, L0, 1);
                L[3] = __shfl_down_sync(full, L2, 1);
                L[5] = __shfl_down_sync(full, L4, 1);
                L[7] = __shfl_down_sync(full, L6, 1);
                if (lane == 31) {
                    L[1] = nx0;
                    L[3] = nx2;
                    L[5] = nx4;
                    L[7] = nx6;
                }
            }
            bool alleq = true;
#pragma unroll
            for (int q = 1; q < 8; ++q) alleq &= (L[q] == L[0]);
            auto differ = [](int32_t x, int32_t y) { return x >= 0 && y >= 0 && x != y; };
            // the 4 labels of the corners with bit bitd set not all equal
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
            const uint32_t f0 = qx & __ballot_sync(full, valid && differ(L[0], L[4]));
            const uint32_t f1 = qy & __ballot_sync(full, valid && differ(L[0], L[2]));
            const uint32_t f2 = qz & __ballot_sync(full, valid && differ(L[0], L[1]));
            const uint32_t v = z00 & __ballot_sync(full, valid && !alleq);
            const uint32_t e0 = v & zp0 & __ballot_sync(full, square_differs(4));
            const uint32_t e1 = v & z0p & __ballot_sync(full, square_differs(2));
            const uint32_t e2 = v & p00 & __ballot_sync(full, square_differs(1));
            if (v) {
                if (zlo < 0) zlo = c0 + __ffs(v) - 1;
                zhi = c0 + 31 - __clz(v);
            }
            if (lane == 0) {
                const int64_t gs = seg_row + k;
                reinterpret_cast<uint4*>(planes + gs)[0] = make_uint4(v, e0, e1, e2);
                reinterpret_cast<uint4*>(planes + gs)[1] = make_uint4(f0, f1, f2, 0u);
                cv[gs] = __popc(v);
                ce[gs] = __popc(e0) + __popc(e1) + __popc(e2);
                cf[gs] = __popc(f0) + __popc(f1) + __popc(f2);
            }
            // advance the pipeline by one segment
            L0 = M0;
            L2 = M2;
            L4 = M4;
            L6 = M6;
            M0 = N0;
            M2 = N2;
            M4 = N4;
            M6 = N6;
            wprv = wcur;
            wcur = w1;
            w1 = w2;
        }
        if (zlo >= 0) {
            mn0 = min(mn0, a);
            mn1 = min(mn1, b);
            mn2 = min(mn2, zlo);
            mx0 = max(mx0, a);
            mx1 = max(mx1, b);
            mx2 = max(mx2, zhi);
        }
    }
    flush();
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

// The cells of one segment that up to three of its planes name, in (point,
// plane) order -- the order of their ids: slot r (r < the returned count)
// gets point << 2 | plane of the r-th cell.  Lane = point; the warp's slot
// array holds 96 entries.
__device__ __forceinline__ int compact_cells(uint32_t p0, uint32_t p1, uint32_t p2, int lane,
                                             uint8_t* __restrict__ slots) {
    const uint32_t m = below(lane);
    int r = __popc(p0 & m) + __popc(p1 & m) + __popc(p2 & m);
    if (bit(p0, lane)) slots[r++] = (uint8_t)(lane << 2);
    if (bit(p1, lane)) slots[r++] = (uint8_t)(lane << 2 | 1);
    if (bit(p2, lane)) slots[r] = (uint8_t)(lane << 2 | 2);
    __syncwarp();
    return __popc(p0) + __popc(p1) + __popc(p2);
}

// The emission kernels walk lattice rows (one warp per row, its segments in
// order).  Per segment, the planes and first ids of the neighbouring rows
// that the segment's cells refer to are loaded once by the whole warp (one
// address per load), then the segment's cells are handed out one per lane in
// id order (compact_cells), so every lane works and consecutive ids are
// written by consecutive lanes.  A neighbour's id is then a population count
// of those words: at point c of a row, the vertex / axis edges / faces before
// c are first id + popcount(planes & below(c)); a neighbour at c - 1 (which
// the rules make a vertex, or an edge or face whose bit is tested) is the last
// one before c, and one at c + 1 the first one after c.  Bits at c - 1 and
// c + 1 come from plane words shifted by one point, whose end bit is read
// from the previous / next segment only when lane 0 / lane 31 needs it.
struct RowPlanes {  // one row's segment: planes and first ids
    uint32_t v, e0, e1, e2, f0, f1, f2;
    int32_t vb, eb, fb;
};
__device__ __forceinline__ RowPlanes row_planes(const SegPlanes* __restrict__ planes, const int32_t* __restrict__ vb,
                                                const int32_t* __restrict__ eb, const int32_t* __restrict__ fbs,
                                                int64_t s, bool want_ve, bool want_f) {
    RowPlanes R{};
    if (s < 0) return R;
    if (want_ve) {
        const uint4 x = __ldg(reinterpret_cast<const uint4*>(planes + s));
        R.v = x.x;
        R.e0 = x.y;
        R.e1 = x.z;
        R.e2 = x.w;
        R.vb = __ldg(vb + s);
        R.eb = __ldg(eb + s);
    }
    if (want_f) {
        const uint4 y = __ldg(reinterpret_cast<const uint4*>(planes + s) + 1);
        R.f0 = y.x;
        R.f1 = y.y;
        R.f2 = y.z;
        R.fb = __ldg(fbs + s);
    }
    return R;
}
__device__ __forceinline__ int32_t pc3(uint32_t a, uint32_t b, uint32_t c, uint32_t m) {
    return __popc(a & m) + __popc(b & m) + __popc(c & m);
}
__device__ __forceinline__ int32_t bt(uint32_t w, int t) { return (int32_t)((w >> t) & 1u); }
// the face (if any) of row R's lattice edge at point t (t = lane index of c)
// along axis ax, at c (nx = false) or at c + 1 (nx = true, with the row's
// face planes shifted down one point in S0..S2); -1 when none
__device__ __forceinline__ int32_t face_at(const RowPlanes& R, uint32_t S0, uint32_t S1, uint32_t S2, int t, bool nx,
                                           int ax) {
    const uint32_t m = below(t);
    if (!nx) {
        const uint32_t w = ax == 0 ? R.f0 : (ax == 1 ? R.f1 : R.f2);
        if (!bt(w, t)) return -1;
        return R.fb + pc3(R.f0, R.f1, R.f2, m) + (ax >= 1 ? bt(R.f0, t) : 0) + (ax >= 2 ? bt(R.f1, t) : 0);
    }
    const uint32_t w = ax == 0 ? S0 : (ax == 1 ? S1 : S2);
    if (!bt(w, t)) return -1;
    // faces before c + 1: those before c and those at c
    const uint32_t mi = m | (1u << t);
    return R.fb + pc3(R.f0, R.f1, R.f2, mi) + (ax >= 1 ? bt(S0, t) : 0) + (ax >= 2 ? bt(S1, t) : 0);
}

// Vertices and axis edges of a row, one lane per point.  Vertices: vts or, in
// the thinning path, each vertex's lattice point, and with records their
// thinning records: incident edges counted and summed -- the axis edges into
// the voxel from -x, -y, -z, its own axis edges, and the diagonals of the
// faces (p1, d) and (p3, d) that have it as q1 / q3 (p1 = p + e_w, p3 = p +
// e_u).  Axis edges: endpoints and, with records, thinning records
// (incident triangles counted, summed and tested against the threshold;
// measure = max lambda of the incident faces, voroinfo.cpp:1490-1538, folded
// to -1 below the threshold and +1 otherwise).  With the threshold folded in,
// only whether each face's lambda is below it matters: the faces kernel
// writes that per segment as three bit planes (fpass), read here beside the
// face planes.  The faces of the plaquettes of the point's three axis edges
// (the lattice edges along u from nb and nb + e_w and along w from nb and
// nb + e_u, nb = the point + e_d, u = d+1, w = d+2 mod 3) are nine lattice
// edges, looked up once:
//   d = 0: (a+1,b,c)+y, (a+1,b,c)+z [triangle 1]; (a+1,b,c+1)+y, (a+1,b+1,c)+z [0]
//   d = 1: (a,b+1,c)+z, (a,b+1,c)+x [1]; (a+1,b+1,c)+z, (a,b+1,c+1)+x [0]
//   d = 2: (a,b,c+1)+x, (a,b,c+1)+y [1]; (a,b+1,c+1)+x, (a+1,b,c+1)+y [0]
// (the triangle of each face that carries the edge: 1 for the two faces at
// nb); the vertex's six diagonals are the faces of (a,b,c+1)+x, (a,b+1,c)+x,
// (a+1,b,c)+y, (a,b,c+1)+y, (a,b+1,c)+z and (a+1,b,c)+z among them, and the
// plaquettes of the edges into the voxel take three more: the lattice edges
// from the point itself.  Six blocks per SM (80 registers, a few spilled)
// measured 3.80 ms at 512^3 against 3.85 ms with five (92 registers).
__global__ void __launch_bounds__(128, 6) vd_vertices_edges_kernel(VolTab T, Bases B, const SegPlanes* __restrict__ planes,
                                                       const int32_t* __restrict__ vb, const int32_t* __restrict__ eb,
                                                       const int32_t* __restrict__ fbs, const uint4* __restrict__ fpass,
                                                       int2* __restrict__ edges, EdgeRecs E,
                                                       float* __restrict__ vts, uint32_t* __restrict__ vlat,
                                                       VertRec* __restrict__ V, int32_t* __restrict__ g0, int64_t ne,
                                                       const float* __restrict__ thr) {
    const int lane = threadIdx.x & 31;
    const bool rec = E.h != nullptr;  // records (E and V) or the complex's arrays
    const int64_t nrow = T.total(kLRow);
    VolTab::Cache vcache;
    ROW_LOOP(gr, nrow) {
        const int bv = T.find_cached(kLRow, gr, vcache);
        const int4 dm = T.dim(bv);
        const int NB = dm.y + 1, NC = dm.z + 1, nsr = (dm.z + 32) / 32;
        const int lr = (int)(gr - T.start(kLRow, bv));
        const int a = lr / NB, b = lr - a * NB;
        if (a >= dm.x || b >= dm.y) continue;  // no voxel in this row
        const Shift sh = shift_of(B, bv);
        const int32_t fbv = (int32_t)sh.fb, eb1 = (int32_t)sh.eb1;
        const float tb = thr ? thr[bv] : 0.0f;
        // rows (a,b), (a+1,b), (a,b+1), (a+1,b+1) (inside the lattice), (a-1,b), (a,b-1)
        const int64_t s0 = T.start(kLSeg, bv) + (int64_t)lr * nsr;
        const int64_t sp0 = s0 + (int64_t)NB * nsr, s0p = s0 + nsr, spp = sp0 + nsr;
        const int64_t sm0 = a >= 1 ? s0 - (int64_t)NB * nsr : -1, s0m = b >= 1 ? s0 - nsr : -1;
        const uint32_t lat_row = (uint32_t)((int64_t)lr * NC);
        // the vertex and edge planes of the row's segments, one segment ahead
        uint4 pv_next = __ldg(reinterpret_cast<const uint4*>(planes + s0));
        for (int k = 0; k < nsr; ++k) {
            const uint4 pv = pv_next;
            if (k + 1 < nsr) pv_next = __ldg(reinterpret_cast<const uint4*>(planes + s0 + k + 1));
            if (pv.x == 0u) continue;  // no vertex, so no axis edge
            // every load of the segment goes out before any is used
            const RowPlanes R0 = row_planes(planes, vb, eb, fbs, s0 + k, true, rec);
            const RowPlanes Rp0 = row_planes(planes, vb, eb, fbs, sp0 + k, true, rec);
            const RowPlanes R0p = row_planes(planes, vb, eb, fbs, s0p + k, true, rec);
            const RowPlanes Rpp = row_planes(planes, vb, eb, fbs, rec ? spp + k : -1, false, true);
            const RowPlanes Rm0 = row_planes(planes, vb, eb, fbs, (rec && sm0 >= 0) ? sm0 + k : -1, true, false);
            const RowPlanes R0m = row_planes(planes, vb, eb, fbs, (rec && s0m >= 0) ? s0m + k : -1, true, false);
            // face planes at c + 1: lane 31 reads the next segment's first bits;
            // the z edge of voxel c - 1: lane 0 reads the previous segment's last bit
            uint4 n0 = make_uint4(0u, 0u, 0u, 0u), np0 = n0, n0p = n0;
            if (rec && k + 1 < nsr && (pv.x >> 31)) {
                n0 = __ldg(reinterpret_cast<const uint4*>(planes + s0 + k + 1) + 1);
                np0 = __ldg(reinterpret_cast<const uint4*>(planes + sp0 + k + 1) + 1);
                n0p = __ldg(reinterpret_cast<const uint4*>(planes + s0p + k + 1) + 1);
            }
            uint32_t pe2 = 0u;
            if (rec && k > 0 && (pv.x & 1u)) pe2 = __ldg(&planes[s0 + k - 1].e2);
            // the faces' filter planes of the same rows (and segments)
            uint4 q0 = make_uint4(0u, 0u, 0u, 0u), qp0 = q0, q0p = q0, qpp = q0, m0 = q0, mp0 = q0, m0p = q0;
            if (rec) {
                q0 = __ldg(fpass + s0 + k);
                qp0 = __ldg(fpass + sp0 + k);
                q0p = __ldg(fpass + s0p + k);
                qpp = __ldg(fpass + spp + k);
                if (k + 1 < nsr && (pv.x >> 31)) {
                    m0 = __ldg(fpass + s0 + k + 1);
                    mp0 = __ldg(fpass + sp0 + k + 1);
                    m0p = __ldg(fpass + s0p + k + 1);
                }
            }
            const int t = lane;
            if (!bt(pv.x, t)) continue;
            const uint32_t m = below(t);
            const int c = 32 * k + t;
            const int32_t v0 = R0.vb + __popc(R0.v & m);
            if (vts) {
                vts[3 * (int64_t)v0 + 0] = (float)a;
                vts[3 * (int64_t)v0 + 1] = (float)b;
                vts[3 * (int64_t)v0 + 2] = (float)c;
            }
            if (vlat) vlat[v0] = lat_row + (uint32_t)c;  // within its volume
            const int32_t e_own = R0.eb + pc3(R0.e0, R0.e1, R0.e2, m) + fbv;
            const bool h0 = bt(R0.e0, t), h1 = bt(R0.e1, t), h2 = bt(R0.e2, t);
            // the +d neighbours: (a+1,b,c), (a,b+1,c), (a,b,c+1) (the vertex after v0 in its row)
            const int32_t v1[3] = {Rp0.vb + __popc(Rp0.v & m), R0p.vb + __popc(R0p.v & m), v0 + 1};
            if (!rec) {
                int32_t e = e_own;
                if (edges) {
                    if (h0) edges[e++] = make_int2(v0, v1[0]);
                    if (h1) edges[e++] = make_int2(v0, v1[1]);
                    if (h2) edges[e] = make_int2(v0, v1[2]);
                }
                continue;
            }
            const uint32_t S00 = (R0.f0 >> 1) | (n0.x << 31), S01 = (R0.f1 >> 1) | (n0.y << 31);
            const uint32_t Sp00 = (Rp0.f0 >> 1) | (np0.x << 31), Sp01 = (Rp0.f1 >> 1) | (np0.y << 31);
            const uint32_t S0p0 = (R0p.f0 >> 1) | (n0p.x << 31);
            // the nine faces (-1: none)
            int32_t fid[9];
            fid[0] = face_at(Rp0, 0u, 0u, 0u, t, false, 1);                             // (a+1,b,c)+y
            fid[1] = face_at(Rp0, 0u, 0u, 0u, t, false, 2);                             // (a+1,b,c)+z
            fid[2] = (h0 || h2) ? face_at(Rp0, Sp00, Sp01, 0u, t, true, 1) : -1;        // (a+1,b,c+1)+y
            fid[3] = (h0 || h1) ? face_at(Rpp, 0u, 0u, 0u, t, false, 2) : -1;           // (a+1,b+1,c)+z
            fid[4] = face_at(R0p, 0u, 0u, 0u, t, false, 2);                             // (a,b+1,c)+z
            fid[5] = face_at(R0p, 0u, 0u, 0u, t, false, 0);                             // (a,b+1,c)+x
            fid[6] = (h1 || h2) ? face_at(R0p, S0p0, 0u, 0u, t, true, 0) : -1;          // (a,b+1,c+1)+x
            fid[7] = face_at(R0, S00, S01, 0u, t, true, 0);                             // (a,b,c+1)+x
            fid[8] = face_at(R0, S00, S01, 0u, t, true, 1);                             // (a,b,c+1)+y
            // the faces of the lattice edges from the point itself: with the
            // nine above they carry the plaquettes of the three axis edges
            // into the voxel (from -x, -y, -z)
            const bool hx = bt(Rm0.e0, t), hy = bt(R0m.e1, t), hz = bt((R0.e2 << 1) | (pe2 >> 31), t);
            const int32_t fx = (hy || hz) ? face_at(R0, 0u, 0u, 0u, t, false, 0) : -1;
            const int32_t fy = (hx || hz) ? face_at(R0, 0u, 0u, 0u, t, false, 1) : -1;
            const int32_t fz = (hx || hy) ? face_at(R0, 0u, 0u, 0u, t, false, 2) : -1;
            // whether each of these faces passes the filter (read where the face exists)
            auto at_c = [&](const uint4& q, int ax) { return bt(ax == 0 ? q.x : (ax == 1 ? q.y : q.z), t) != 0; };
            auto at_c1 = [&](const uint4& q, const uint4& qn, int ax) {  // at c + 1
                const uint32_t w = ax == 0 ? q.x : q.y, wn = ax == 0 ? qn.x : qn.y;
                return bt((w >> 1) | (wn << 31), t) != 0;
            };
            bool pj[9];
            pj[0] = at_c(qp0, 1);
            pj[1] = at_c(qp0, 2);
            pj[2] = at_c1(qp0, mp0, 1);
            pj[3] = at_c(qpp, 2);
            pj[4] = at_c(q0p, 2);
            pj[5] = at_c(q0p, 0);
            pj[6] = at_c1(q0p, m0p, 0);
            pj[7] = at_c1(q0, m0, 0);
            pj[8] = at_c1(q0, m0, 1);
            const bool px = at_c(q0, 0), py = at_c(q0, 1), pz = at_c(q0, 2);
            // an edge passes when its largest face lambda (0 without faces) is
            // below the threshold: every face passes, and 0 < threshold
            const bool zero_passes = 0.0f < tb;
            // the axis edges' records
            constexpr int kSlot[3][4] = {{0, 1, 2, 3}, {4, 5, 3, 6}, {7, 8, 6, 2}};
            bool epass[3] = {false, false, false};
            {
                int32_t e = e_own;
#pragma unroll
                for (int d = 0; d < 3; ++d) {
                    if (!(d == 0 ? h0 : (d == 1 ? h1 : h2))) continue;
                    unsigned kk = 0, npass = 0;
                    unsigned long long idsum = 0;
#pragma unroll
                    for (int i = 0; i < 4; ++i) {
                        const int s = kSlot[d][i];
                        if (fid[s] >= 0) {
                            npass += pj[s] ? 1u : 0u;
                            idsum += (unsigned)(2 * fid[s] + (i < 2 ? 1 : 0));
                            ++kk;
                        }
                    }
                    if (edges) edges[e] = make_int2(v0, v1[d]);
                    // the measure folded to -1 below the threshold, +1 otherwise
                    epass[d] = npass == kk && zero_passes;
                    E.h[e] = EdgeHead{v0, v1[d], kAlive, epass[d] ? -1.0f : 1.0f};
                    E.n[e] = EdgeCnt{rs_make(kk, npass, idsum), 0ull};
                    // generation 0: an FE pair when the one face passes the filter
                    g0[e] = (kk == 1 && npass == 1) ? (int32_t)idsum : -1;
                    ++e;
                }
            }
            // the vertex record: its incident edges counted, and 2 e + (e
            // passes the filter) summed over them
            {
                unsigned kk = 0;
                unsigned long long idsum = 0;
                auto add = [&](int32_t e, bool pass) {
                    ++kk;
                    idsum += 2u * (unsigned)e + (pass ? 1u : 0u);
                };
                // every existing face of the four passes (and 0 < threshold)
                auto passes4 = [&](int32_t f1, bool p1, int32_t f2, bool p2, int32_t f3, bool p3, int32_t f4, bool p4) {
                    return (f1 < 0 || p1) && (f2 < 0 || p2) && (f3 < 0 || p3) && (f4 < 0 || p4) && zero_passes;
                };
                if (hx)  // (a-1,b,c)+x: faces (a,b,c)+y, +z, (a,b,c+1)+y, (a,b+1,c)+z
                    add(Rm0.eb + pc3(Rm0.e0, Rm0.e1, Rm0.e2, m) + fbv,
                        passes4(fy, py, fz, pz, fid[8], pj[8], fid[4], pj[4]));
                if (hy)  // (a,b-1,c)+y: faces (a,b,c)+z, +x, (a+1,b,c)+z, (a,b,c+1)+x
                    add(R0m.eb + pc3(R0m.e0, R0m.e1, R0m.e2, m) + bt(R0m.e0, t) + fbv,
                        passes4(fz, pz, fx, px, fid[1], pj[1], fid[7], pj[7]));
                if (hz)  // (a,b,c-1)+z: the last axis edge before c; faces
                    add(e_own - 1, passes4(fx, px, fy, py, fid[5], pj[5], fid[0], pj[0]));  // (a,b,c)+x, +y, (a,b+1,c)+x, (a+1,b,c)+y
                {
                    int32_t e = e_own;
                    if (h0) add(e++, epass[0]);
                    if (h1) add(e++, epass[1]);
                    if (h2) add(e, epass[2]);
                }
                const int dg[6] = {7, 5, 0, 8, 4, 1};  // the diagonals' faces (a diagonal's measure is its face's)
#pragma unroll
                for (int i = 0; i < 6; ++i)
                    if (fid[dg[i]] >= 0) add(eb1 + fid[dg[i]], pj[dg[i]]);
                VertRec vr;
                vr.rs = rs_make(kk, 0, idsum);
                vr.trig = 0;
                V[v0] = vr;
                // generation 0: an EV pair when the one edge passes the filter
                g0[ne + v0] = (kk == 1 && (idsum & 1u)) ? (int32_t)(idsum >> 1) : -1;
            }
        }
    }
}

// Faces: two triangles each (util::simpleTriangulate of the quad
// (q0,q1,q2,q3): (q3,q0,q1), (q3,q1,q2)), the diagonal edge (q1,q3), the
// face's lambda and, with records, the thinning records of both triangles
// and the diagonal.  The quad of lattice edge (a,b,c)+d lies in rows R0
// (a,b), R0m (a,b-1), Rm0 (a-1,b), Rmm (a-1,b-1) at points c - 1 and c:
//   d = 0: q0 (a,b-1,c-1) q1 (a,b,c-1) q2 (a,b,c) q3 (a,b-1,c)
//   d = 1: q0 (a-1,b,c-1) q1 (a-1,b,c) q2 (a,b,c) q3 (a,b,c-1)
//   d = 2: q0 (a-1,b-1,c) q1 (a,b-1,c) q2 (a,b,c) q3 (a-1,b,c)
// All four are vertices (inside, and the face's labels differ), so the one
// at c - 1 is the last vertex before c in its row; its axis edge along dd is
// (axis edges before c) minus its edges along the axes >= dd.
__global__ void __launch_bounds__(128, 6) vd_faces_kernel(VolTab T, Bases B, const SegPlanes* __restrict__ planes,
                                                       const int32_t* __restrict__ vb, const int32_t* __restrict__ eb,
                                                       const int32_t* __restrict__ fbs, const int32_t* __restrict__ lab,
                                                       const float* __restrict__ sxyz, float* __restrict__ lamf,
                                                       int32_t* __restrict__ tris, int2* __restrict__ edges,
                                                       FaceRec* __restrict__ F, EdgeRecs E,
                                                       int32_t* __restrict__ g0, const float* __restrict__ thr,
                                                       uint4* __restrict__ fpass) {
    __shared__ uint8_t s_slots[4][96];
    const int lane = threadIdx.x & 31;
    uint8_t* slots = s_slots[threadIdx.x >> 5];
    const int64_t nrow = T.total(kLRow);
    VolTab::Cache vcache;
    ROW_LOOP(gr, nrow) {
        const int bv = T.find_cached(kLRow, gr, vcache);
        const int4 dm = T.dim(bv);
        const int NB = dm.y + 1, NC = dm.z + 1, nsr = (dm.z + 32) / 32;
        const int lr = (int)(gr - T.start(kLRow, bv));
        const int a = lr / NB, b = lr - a * NB;
        if (a >= dm.x || b >= dm.y) continue;  // no face in this row
        const Shift sh = shift_of(B, bv);
        const int32_t fbv = (int32_t)sh.fb, eb1 = (int32_t)sh.eb1;
        const float tb = thr ? thr[bv] : 0.0f;
        const int64_t s0 = T.start(kLSeg, bv) + (int64_t)lr * nsr;
        const int64_t s0m = b >= 1 ? s0 - nsr : -1;
        const int64_t sm0 = a >= 1 ? s0 - (int64_t)NB * nsr : -1;
        const int64_t smm = (a >= 1 && b >= 1) ? sm0 - nsr : -1;
        const int32_t* lrow = lab + T.start(kLat, bv) + (int64_t)lr * NC;
        // the face planes (f0 f1 f2 -) of the row's segments, one segment ahead
        uint4 fo_next = __ldg(reinterpret_cast<const uint4*>(planes + s0) + 1);
        for (int k = 0; k < nsr; ++k) {
            const uint4 fo = fo_next;
            if (k + 1 < nsr) fo_next = __ldg(reinterpret_cast<const uint4*>(planes + s0 + k + 1) + 1);
            if ((fo.x | fo.y | fo.z) == 0u) continue;
            // the labels at the lane's point c and at c + e_x, c + e_y, c + e_z
            // (rows a + 1 and b + 1 exist: a < X, b < Y), loaded with the planes
            const int cl = 32 * k + lane;
            const int32_t l_c = cl < NC ? __ldg(lrow + cl) : -1;
            const int32_t l_x = cl < NC ? __ldg(lrow + (int64_t)NB * NC + cl) : -1;
            const int32_t l_y = cl < NC ? __ldg(lrow + NC + cl) : -1;
            const int32_t l_z = cl + 1 < NC ? __ldg(lrow + cl + 1) : -1;
            const int n = compact_cells(fo.x, fo.y, fo.z, lane, slots);
            const int32_t f_first = __ldg(fbs + s0 + k);
            const RowPlanes R0 = row_planes(planes, vb, eb, fbs, s0 + k, true, false);
            const RowPlanes R0m = row_planes(planes, vb, eb, fbs, s0m < 0 ? -1 : s0m + k, true, false);
            const RowPlanes Rm0 = row_planes(planes, vb, eb, fbs, sm0 < 0 ? -1 : sm0 + k, true, false);
            const RowPlanes Rmm = row_planes(planes, vb, eb, fbs, (smm < 0 || fo.z == 0u) ? -1 : smm + k, true, false);
            // edge planes shifted up one point (bit t = point c - 1): lane 0
            // reads the previous segment's last bits (faces along x and y
            // only reach back to c - 1)
            uint4 p0 = make_uint4(0u, 0u, 0u, 0u), p0m = p0, pm0 = p0;
            if (k > 0 && ((fo.x | fo.y) & 1u)) {
                p0 = __ldg(reinterpret_cast<const uint4*>(planes + s0 + k - 1));
                if (s0m >= 0) p0m = __ldg(reinterpret_cast<const uint4*>(planes + s0m + k - 1));
                if (sm0 >= 0) pm0 = __ldg(reinterpret_cast<const uint4*>(planes + sm0 + k - 1));
            }
            // per point (lane = point): vertices and axis edges before the
            // point in each row, and the edge bits the quads read, for the
            // face lanes to fetch by shuffle
            const uint32_t ml = below(lane);
            const int32_t pv0 = R0.vb + __popc(R0.v & ml), pv0m = R0m.vb + __popc(R0m.v & ml);
            const int32_t pvm0 = Rm0.vb + __popc(Rm0.v & ml), pvmm = Rmm.vb + __popc(Rmm.v & ml);
            const int32_t px0 = R0.eb + pc3(R0.e0, R0.e1, R0.e2, ml) + fbv;
            const int32_t px0m = R0m.eb + pc3(R0m.e0, R0m.e1, R0m.e2, ml) + fbv;
            const int32_t pxm0 = Rm0.eb + pc3(Rm0.e0, Rm0.e1, Rm0.e2, ml) + fbv;
            const int32_t pxmm = Rmm.eb + pc3(Rmm.e0, Rmm.e1, Rmm.e2, ml) + fbv;
            // bits at the point's c - 1 (edge planes shifted up one point) and at c
            const int32_t pbits = bt((R0.e2 << 1) | (p0.w >> 31), lane) |                  // 0: (a,b,c-1)+z
                                  bt((R0m.e1 << 1) | (p0m.z >> 31), lane) << 1 |           // 1: (a,b-1,c-1)+y
                                  bt((R0m.e2 << 1) | (p0m.w >> 31), lane) << 2 |           // 2: (a,b-1,c-1)+z
                                  bt(R0m.e0, lane) << 3 |                                  // 3: (a,b-1,c)+x
                                  bt((Rm0.e0 << 1) | (pm0.y >> 31), lane) << 4 |           // 4: (a-1,b,c-1)+x
                                  bt((Rm0.e1 << 1) | (pm0.z >> 31), lane) << 5 |           // 5: (a-1,b,c-1)+y
                                  bt((Rm0.e2 << 1) | (pm0.w >> 31), lane) << 6 |           // 6: (a-1,b,c-1)+z
                                  bt(Rmm.e0, lane) << 7;                                   // 7: (a-1,b-1,c)+x
            uint32_t fp0 = 0u, fp1 = 0u, fp2 = 0u;  // this lane's faces that pass, by axis
            for (int r0 = 0; r0 < n; r0 += 32) {
                // every lane takes part in the shuffles; lanes past the last
                // face skip the rest
                const int r = r0 + lane;
                const int sl = r < n ? slots[r] : 0;
                const int t = sl >> 2, d = sl & 3;
                const unsigned full = 0xffffffffu;
                const int32_t s_c = __shfl_sync(full, l_c, t);
                const int32_t s_x = __shfl_sync(full, l_x, t);
                const int32_t s_y = __shfl_sync(full, l_y, t);
                const int32_t s_z = __shfl_sync(full, l_z, t);
                const int32_t v0 = __shfl_sync(full, pv0, t), v0m = __shfl_sync(full, pv0m, t);
                const int32_t vm0 = __shfl_sync(full, pvm0, t), vmm = __shfl_sync(full, pvmm, t);
                const int32_t x0 = __shfl_sync(full, px0, t), x0m = __shfl_sync(full, px0m, t);
                const int32_t xm0 = __shfl_sync(full, pxm0, t), xmm = __shfl_sync(full, pxmm, t);
                const int32_t bits = __shfl_sync(full, pbits, t);
                if (r >= n) continue;
                auto bb = [&](int i) { return (bits >> i) & 1; };
                int32_t q0, q1, q2, q3, e01, e12, e32, e03;
                if (d == 0) {
                    q0 = v0m - 1;
                    q1 = v0 - 1;
                    q2 = v0;
                    q3 = v0m;
                    e01 = x0m - bb(2) - bb(1);  // q0 along y
                    e12 = x0 - bb(0);           // q1 along z
                    e32 = x0m + bb(3);          // q3 along y
                    e03 = x0m - bb(2);          // q0 along z
                } else if (d == 1) {
                    q0 = vm0 - 1;
                    q1 = vm0;
                    q2 = v0;
                    q3 = v0 - 1;
                    e01 = xm0 - bb(6);                  // q0 along z
                    e12 = xm0;                          // q1 along x
                    e32 = x0 - bb(0);                   // q3 along z
                    e03 = xm0 - bb(4) - bb(5) - bb(6);  // q0 along x
                } else {
                    q0 = vmm;
                    q1 = v0m;
                    q2 = v0;
                    q3 = vm0;
                    e01 = xmm;           // q0 along x
                    e12 = x0m + bb(3);   // q1 along y
                    e32 = xm0;           // q3 along x
                    e03 = xmm + bb(7);   // q0 along y
                }
                const int32_t f = f_first + r;
                const int32_t diag = eb1 + f;
                const int64_t t0 = 2 * (int64_t)f, t1 = t0 + 1;
                if (tris) {
                    tris[3 * t0 + 0] = q3;
                    tris[3 * t0 + 1] = q0;
                    tris[3 * t0 + 2] = q1;
                    tris[3 * t1 + 0] = q3;
                    tris[3 * t1 + 1] = q1;
                    tris[3 * t1 + 2] = q2;
                }
                const int32_t dv0 = min(q1, q3), dv1 = max(q1, q3);
                if (edges) edges[diag] = make_int2(dv0, dv1);
                // lambda of the face: distance of its two sites (measureforMA_imp.h:1-4)
                const float lm = lambda_of(sxyz, s_c, d == 0 ? s_x : (d == 1 ? s_y : s_z));
                lamf[f] = lm;
                if (F) {
                    const float lr_ = rec_measure(lm, thr, bv);
                    const int32_t pass = lr_ < 0.0f ? kFacePass : 0;
                    // sides in traceFace order: (t0,t1), (t1,t2), (t2,t0)
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
                    E.h[diag] = EdgeHead{dv0, dv1, kAlive, lr_};
                    E.n[diag] = EdgeCnt{rs_make(2, lm < tb ? 2u : 0u, (unsigned long long)t0 + (unsigned long long)t1), 0ull};
                    g0[diag] = -1;  // two triangles: no FE pair
                    if (pass) {
                        if (d == 0) fp0 |= 1u << t;
                        else if (d == 1) fp1 |= 1u << t;
                        else fp2 |= 1u << t;
                    }
                }
            }
            if (fpass) {
                // the segment's filter planes: bit t of word d = the face of
                // lattice edge (c0 + t) + d passes (its lambda below the threshold)
                const uint32_t w0 = __reduce_or_sync(0xffffffffu, fp0), w1 = __reduce_or_sync(0xffffffffu, fp1),
                               w2 = __reduce_or_sync(0xffffffffu, fp2);
                if (lane == 0) fpass[s0 + k] = make_uint4(w0, w1, w2, 0u);
            }
            __syncwarp();
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

// up to 64 blocks of 256 threads per SM (16 measured 0.025 ms slower on the remaining complex's write at 512^3)
inline int cell_grid(vc_ctx* c, int64_t n) {
    return (int)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, (int64_t)c->num_sms * 64));
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

// 128-thread blocks, one chunk of kRowChunk lattice rows per block (the loop is grid-stride past 2^20 blocks):
// capping the grid at 16 or 32 blocks per SM left a tail (faces and vertex/edge kernels 0.73 / 0.29 ms longer at
// 512^3)
inline int row_grid(vc_ctx* c, int64_t nrow) {
    (void)c;
    return (int)std::max<int64_t>(1, std::min<int64_t>((nrow + kRowChunk - 1) / kRowChunk, (int64_t)1 << 20));
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
        vd_segments_kernel<<<row_grid(c, c->h_off[kLRow][nvol]), 128, 0, c->stream>>>(ptr<uint32_t>(c->site_bits),
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
    // cell ids are 31-bit (the records tag them with bit 31); the adjacency
    // lists the getters and the generic thinning use have 32-bit offsets and
    // check their own sizes (build_adjacency)
    if (ne >= INT32_MAX || nt >= INT32_MAX || nv >= INT32_MAX) return VC_ERR_ARG;
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
    EdgeRecs ER;  // none unless folded
    uint4* fpass = nullptr;
    if (folded) {
        VC_TRY(ensure_n<uint4>(c, c->vd_fpass, nseg));  // the faces' filter bits per segment
        fpass = ptr<uint4>(c->vd_fpass);
        VC_TRY(ensure_n<FaceRec>(c, c->face_rec, nt));
        VC_TRY(ensure_edge_recs(c, c->edge_rec, ne, &ER));
        VC_TRY(ensure_n<VertRec>(c, c->vert_rec, nv));
        VC_TRY(ensure_n<int32_t>(c, c->thin_g0, nv + ne));
    }
    const float* thr = folded ? c->bases.thr : nullptr;
    {
        Region r(c, "vd_emit");
        int32_t* g0 = folded ? ptr<int32_t>(c->thin_g0) : nullptr;
        {
            Region k(c, "vd_faces");
            vd_faces_kernel<<<row_grid(c, c->h_off[kLRow][c->nvol]), 128, 0, c->stream>>>(
                c->tab, c->bases, planes, vb, eb, fb, ptr<int32_t>(c->ft_id), ptr<float>(c->site_xyz),
                ptr<float>(c->vd_lam), geom ? ptr<int32_t>(c->tris) : nullptr, geom ? ptr<int2>(c->edges) : nullptr,
                folded ? ptr<FaceRec>(c->face_rec) : nullptr, ER, g0, thr, fpass);
            launched(c);
        }
        {
            Region k(c, "vd_vertices_edges");
            vd_vertices_edges_kernel<<<row_grid(c, c->h_off[kLRow][c->nvol]), 128, 0, c->stream>>>(
                c->tab, c->bases, planes, vb, eb, fb, fpass, geom ? ptr<int2>(c->edges) : nullptr, ER,
                geom ? ptr<float>(c->vts) : nullptr,
                geom ? nullptr : ptr<uint32_t>(c->vd_vlat), folded ? ptr<VertRec>(c->vert_rec) : nullptr, g0, ne,
                thr);
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
    VC_TRY(ensure_n<float>(c, c->vts, 3 * nv));
    VC_TRY(ensure_n<int2>(c, c->edges, ne));
    VC_TRY(ensure_n<int32_t>(c, c->tris, 3 * nt));
    const SegPlanes* planes = ptr<SegPlanes>(c->vd_seg);
    const int32_t *vb = ptr<int32_t>(c->vd_voff), *eb = ptr<int32_t>(c->vd_eoff), *fb = ptr<int32_t>(c->vd_foff);
    Region r(c, "vd_geometry");
    vd_faces_kernel<<<row_grid(c, c->h_off[kLRow][c->nvol]), 128, 0, c->stream>>>(
        c->tab, c->bases, planes, vb, eb, fb, ptr<int32_t>(c->ft_id), ptr<float>(c->site_xyz), ptr<float>(c->vd_lam),
        ptr<int32_t>(c->tris), ptr<int2>(c->edges), nullptr, EdgeRecs{}, nullptr, nullptr, nullptr);
    vd_vertices_edges_kernel<<<row_grid(c, c->h_off[kLRow][c->nvol]), 128, 0, c->stream>>>(
        c->tab, c->bases, planes, vb, eb, fb, nullptr, ptr<int2>(c->edges), EdgeRecs{}, ptr<float>(c->vts),
        nullptr, nullptr, nullptr, ne, nullptr);
    launched(c, 2);
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
// One warp per 32 consecutive survivor words (vertices, then edges, then
// triangles, in one index space of words): the kept cells of those words are
// handed out one per lane in index order, and lane r finds its cell's word by
// a binary search over the warp's running counts and its bit by one over the
// word's population counts, so every lane works on a kept cell.
__device__ __forceinline__ int select_bit(uint32_t w, int k) {  // position of the k-th set bit (k < popc(w))
    int p = 0;
#pragma unroll
    for (int s = 16; s >= 1; s >>= 1) {
        const int c = __popc(w & ((1u << (p + s)) - 1u));  // set bits below p + s
        if (c <= k) p += s;
    }
    return p;
}
__global__ void __launch_bounds__(256) vd_rem_write_kernel(int32_t nv, int32_t ne, int32_t nt, Kept K, VolTab T,
                                                           int nvol, const uint32_t* __restrict__ vlat,
                                                           const EdgeHead* __restrict__ E, const FaceRec* __restrict__ F,
                                                           float* __restrict__ ovts, int2* __restrict__ oedges,
                                                           int32_t* __restrict__ otris, Bases B, int nmap) {
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const int64_t nwv = ((int64_t)nv + 31) / 32, nwe = ((int64_t)ne + 31) / 32, nwf = ((int64_t)nt + 31) / 32;
    const int64_t nw = nwv + nwe + nwf;
    const int64_t nchunk = (nw + 31) / 32;
    const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
    for (int64_t ch = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); ch < nchunk; ch += warps) {
        // this lane's word and the kept cells before it in the chunk
        const int64_t w = ch * 32 + lane;
        uint32_t word = 0u;
        if (w < nwv) word = __ldg(K.bv + w);
        else if (w < nwv + nwe) word = __ldg(K.be + (w - nwv));
        else if (w < nw) word = __ldg(K.bf + (w - nwv - nwe));
        const int cnt = __popc(word);
        int incl = cnt;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(full, incl, o);
            if (lane >= o) incl += y;
        }
        const int total = __shfl_sync(full, incl, 31);
        for (int base = 0; base < total; base += 32) {
            const int r = base + lane;
            // the lane L whose word holds kept cell r: the number of lanes with incl <= r
            int L = 0;
#pragma unroll
            for (int s = 16; s >= 1; s >>= 1) {
                const int y = __shfl_sync(full, incl, L + s - 1);
                if (y <= r) L += s;
            }
            const uint32_t wordL = __shfl_sync(full, word, L & 31);
            const int exclL = __shfl_sync(full, incl, L & 31) - __shfl_sync(full, cnt, L & 31);
            if (r >= total) continue;
            const int k = r - exclL;  // kept cells of word L before this one
            const int bitp = select_bit(wordL, k);
            const int64_t wl = ch * 32 + L;
            if (wl < nwv) {
                const int64_t o = __ldg(K.pv + wl) + k;
                lattice_vertex(T, B, nvol, vlat, (int32_t)(wl * 32 + bitp), ovts + 3 * o);
            } else if (wl < nwv + nwe) {
                const int64_t we = wl - nwv;
                const int4 er = __ldg(reinterpret_cast<const int4*>(E + we * 32 + bitp));  // v0 v1 rm em
                const int32_t sh = nmap > 1 ? (int32_t)B.b[kBRemV][find_base(B.b[kBVert], nmap, er.x)] : 0;
                oedges[__ldg(K.pe + we) + k] =
                    make_int2(kept_rank(K.bv, K.pv, er.x) - sh, kept_rank(K.bv, K.pv, er.y) - sh);
            } else {
                const int64_t wf = wl - nwv - nwe;
                const int64_t f = wf * 32 + bitp;
                const int64_t o = __ldg(K.pf + wf) + k;
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
}

}  // namespace

int lattice_rem_write(vc_ctx* c, const Kept& K, int nmap) {
    const int64_t nv = c->nv, ne = c->ne, nt = c->nt;
    const int64_t nw = (nv + 31) / 32 + (ne + 31) / 32 + (nt + 31) / 32;
    vd_rem_write_kernel<<<cell_grid(c, nw), 256, 0, c->stream>>>(
        (int32_t)nv, (int32_t)ne, (int32_t)nt, K, c->tab, c->nvol, ptr<uint32_t>(c->vd_vlat),
        ptr<EdgeHead>(c->edge_rec), ptr<FaceRec>(c->face_rec), ptr<float>(c->rem_vts),
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
    if (need_topo && (2 * c->ne >= INT32_MAX || 3 * c->nt >= INT32_MAX)) return VC_ERR_ARG;  // (build_adjacency)
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
