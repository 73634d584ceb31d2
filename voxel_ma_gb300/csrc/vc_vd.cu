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

int build_adjacency(vc_ctx* c);

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

__device__ __forceinline__ void decode(int64_t p, int64_t NB, int64_t NC, int& a, int& b, int& c) {
    c = (int)(p % NC);
    b = (int)((p / NC) % NB);
    a = (int)(p / (NB * NC));
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

// flags: bits 0-2 valid face along axis d; bit 3 vertex; bits 4-6 valid edge along d.
__global__ void vd_flags_kernel(Grid g, uint8_t* __restrict__ flags, int32_t* __restrict__ vcnt,
                                int32_t* __restrict__ ecnt, int32_t* __restrict__ fcnt, int64_t n) {
    for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x) {
        int a, b, c;
        decode(p, g.NB, g.NC, a, b, c);
        uint32_t f = 0;
#pragma unroll
        for (int d = 0; d < 3; ++d)
            if (face_valid(g, a, b, c, d)) f |= 1u << d;
        if (a < g.X && b < g.Y && c < g.Z && g.inside(a, b, c)) {
            int32_t L[8];
#pragma unroll
            for (int q = 0; q < 8; ++q) L[q] = g.label(a + ((q >> 2) & 1), b + ((q >> 1) & 1), c + (q & 1));
            bool alleq = true;
#pragma unroll
            for (int q = 1; q < 8; ++q) alleq &= (L[q] == L[0]);
            if (!alleq) {
                f |= 8u;
                // plaquette of axis d: corners with offset 1 along d
#pragma unroll
                for (int d = 0; d < 3; ++d) {
                    int ni = a + (d == 0), nj = b + (d == 1), nk = c + (d == 2);
                    if (!g.inside(ni, nj, nk)) continue;
                    const int bit = 1 << (2 - d);  // q bit of axis d: x->4, y->2, z->1
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
        vcnt[p] = (f >> 3) & 1;
        ecnt[p] = __popc((f >> 4) & 7u);
        fcnt[p] = __popc(f & 7u);
    }
}

__device__ __forceinline__ int32_t edge_id(const uint8_t* flags, const int32_t* eoff, int64_t lp, int axis) {
    const uint32_t f = flags[lp];
    return eoff[lp] + __popc((f >> 4) & ((1u << axis) - 1u));
}

__global__ void vd_vertices_kernel(Grid g, const uint8_t* __restrict__ flags, const int32_t* __restrict__ voff,
                                   const float* __restrict__ sxyz, float* __restrict__ vts, float* __restrict__ vm,
                                   int32_t* __restrict__ bbox, int64_t n) {
    for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x) {
        if (!(flags[p] & 8u)) continue;
        int a, b, c;
        decode(p, g.NB, g.NC, a, b, c);
        const int32_t v = voff[p];
        vts[3 * (int64_t)v + 0] = (float)a;
        vts[3 * (int64_t)v + 1] = (float)b;
        vts[3 * (int64_t)v + 2] = (float)c;
        // the 12 cube edges of voxel (a,b,c): along d, starting at the cube
        // corners whose d-offset is 0
        float m = 0.0f;
#pragma unroll
        for (int d = 0; d < 3; ++d)
#pragma unroll
            for (int s = 0; s < 2; ++s)
#pragma unroll
                for (int t = 0; t < 2; ++t) {
                    int o[3];
                    o[d] = 0;
                    o[(d + 1) % 3] = s;
                    o[(d + 2) % 3] = t;
                    const int64_t lp = g.lid(a + o[0], b + o[1], c + o[2]);
                    if (!(flags[lp] & (1u << d))) continue;
                    int e[3] = {a + o[0], b + o[1], c + o[2]};
                    e[d] += 1;
                    m = fmaxf(m, lambda_of(sxyz, g.lab[lp], g.label(e[0], e[1], e[2])));
                }
        vm[v] = m;
        atomicMin(&bbox[0], a);
        atomicMin(&bbox[1], b);
        atomicMin(&bbox[2], c);
        atomicMax(&bbox[3], a);
        atomicMax(&bbox[4], b);
        atomicMax(&bbox[5], c);
    }
}

__global__ void vd_edges_kernel(Grid g, const uint8_t* __restrict__ flags, const int32_t* __restrict__ voff,
                                const int32_t* __restrict__ eoff, const float* __restrict__ sxyz,
                                int2* __restrict__ edges, float* __restrict__ em, int64_t n) {
    for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t f = flags[p];
        if (!(f & 0x70u)) continue;
        int a, b, c;
        decode(p, g.NB, g.NC, a, b, c);
        int32_t e = eoff[p];
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            if (!(f & (16u << d))) continue;
            const int u = (d + 1) % 3, w = (d + 2) % 3;
            int nb[3] = {a, b, c};
            nb[d] += 1;
            const int32_t v0 = voff[p], v1 = voff[g.lid(nb[0], nb[1], nb[2])];
            // plaquette corners: (v + e_d) + s e_u + t e_w; its lattice edges run
            // along u from the t corners with s = 0 and along w from the s corners with t = 0
            float m = 0.0f;
#pragma unroll
            for (int t = 0; t < 2; ++t) {
                int cc[3] = {nb[0], nb[1], nb[2]};
                cc[w] += t;
                const int64_t lp = g.lid(cc[0], cc[1], cc[2]);
                if (flags[lp] & (1u << u)) {
                    int ee[3] = {cc[0], cc[1], cc[2]};
                    ee[u] += 1;
                    m = fmaxf(m, lambda_of(sxyz, g.lab[lp], g.label(ee[0], ee[1], ee[2])));
                }
            }
#pragma unroll
            for (int s = 0; s < 2; ++s) {
                int cc[3] = {nb[0], nb[1], nb[2]};
                cc[u] += s;
                const int64_t lp = g.lid(cc[0], cc[1], cc[2]);
                if (flags[lp] & (1u << w)) {
                    int ee[3] = {cc[0], cc[1], cc[2]};
                    ee[w] += 1;
                    m = fmaxf(m, lambda_of(sxyz, g.lab[lp], g.label(ee[0], ee[1], ee[2])));
                }
            }
            edges[e] = make_int2(v0, v1);
            em[e] = m;
            ++e;
        }
    }
}

__global__ void vd_faces_kernel(Grid g, const uint8_t* __restrict__ flags, const int32_t* __restrict__ voff,
                                const int32_t* __restrict__ eoff, const int32_t* __restrict__ foff,
                                const float* __restrict__ sxyz, int32_t ne_axis, int2* __restrict__ edges,
                                float* __restrict__ em, int32_t* __restrict__ tris, int32_t* __restrict__ tri_edges,
                                float* __restrict__ fm, int32_t* __restrict__ tri_face,
                                int2* __restrict__ face_sites, int64_t n) {
    for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t fl = flags[p];
        if (!(fl & 7u)) continue;
        int a, b, c;
        decode(p, g.NB, g.NC, a, b, c);
        int32_t f = foff[p];
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            if (!(fl & (1u << d))) continue;
            const int u = (d + 1) % 3, w = (d + 2) % 3;
            int e1[3] = {a, b, c};
            e1[d] += 1;
            const int32_t s0 = g.lab[p], s1 = g.label(e1[0], e1[1], e1[2]);
            const float lam = lambda_of(sxyz, s0, s1);
            int64_t ql[4];
            int32_t q[4];
#pragma unroll
            for (int m = 0; m < 4; ++m) {
                int i, j, k;
                quad_voxel(a, b, c, d, m, i, j, k);
                ql[m] = g.lid(i, j, k);
                q[m] = voff[ql[m]];
            }
            const int32_t diag = ne_axis + f;
            const int32_t e01 = edge_id(flags, eoff, ql[0], u);
            const int32_t e12 = edge_id(flags, eoff, ql[1], w);
            const int32_t e32 = edge_id(flags, eoff, ql[3], u);
            const int32_t e03 = edge_id(flags, eoff, ql[0], w);
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
            fm[t0] = lam;
            fm[t1] = lam;
            tri_face[t0] = f;
            tri_face[t1] = f;
            face_sites[f] = make_int2(s0, s1);
            edges[diag] = make_int2(min(q[1], q[3]), max(q[1], q[3]));
            em[diag] = lam;
            ++f;
        }
    }
}

__global__ void init_bbox_kernel(int32_t* bbox) {
    if (threadIdx.x < 3) bbox[threadIdx.x] = INT32_MAX;
    else if (threadIdx.x < 6) bbox[threadIdx.x] = INT32_MIN;
}

inline int grid_for(vc_ctx* c, int64_t n, int threads) {
    int64_t b = (n + threads - 1) / threads;
    return (int)std::max<int64_t>(1, std::min<int64_t>(b, (int64_t)c->num_sms * 16));
}

}  // namespace

int run_lattice_vd(vc_ctx* c, vc_vd_sizes* sizes) {
    if (!c->ft_valid) return VC_ERR_STATE;
    const int64_t NB = c->Y + 1, NC = c->Z + 1;
    const int64_t N = (int64_t)(c->X + 1) * NB * NC;
    VC_TRY(ensure_n<uint8_t>(c, c->vd_flags, N));
    VC_TRY(ensure_n<int32_t>(c, c->vd_voff, N));
    VC_TRY(ensure_n<int32_t>(c, c->vd_eoff, N));
    VC_TRY(ensure_n<int32_t>(c, c->vd_foff, N));
    VC_TRY(ensure_n<int64_t>(c, c->scratch2, 4));
    VC_TRY(ensure_n<int32_t>(c, c->vd_bbox, 8));
    Region stage(c, "stage_vd");
    Grid g{ptr<uint8_t>(c->occ), ptr<int32_t>(c->ft_id), c->X, c->Y, c->Z, NB, NC};
    uint8_t* flags = ptr<uint8_t>(c->vd_flags);
    int32_t* voff = ptr<int32_t>(c->vd_voff);
    int32_t* eoff = ptr<int32_t>(c->vd_eoff);
    int32_t* foff = ptr<int32_t>(c->vd_foff);
    {
    Region r(c, "vd_flags");
    vd_flags_kernel<<<grid_for(c, N, 256), 256, 0, c->stream>>>(g, flags, voff, eoff, foff, N);
    launched(c);
    }
    VC_CUDA(c, cudaGetLastError());
    int64_t* tot = ptr<int64_t>(c->scratch2);
    VC_TRY(scan_exclusive_i32(c, voff, voff, N, tot + 0));
    VC_TRY(scan_exclusive_i32(c, eoff, eoff, N, tot + 1));
    VC_TRY(scan_exclusive_i32(c, foff, foff, N, tot + 2));
    int64_t h[3];
    VC_CUDA(c, cudaMemcpyAsync(h, tot, 3 * sizeof(int64_t), cudaMemcpyDeviceToHost, c->stream));
    VC_TRY(sync_check(c));
    const int64_t nv = h[0], ne_axis = h[1], nface = h[2];
    const int64_t ne = ne_axis + nface, nt = 2 * nface;
    if (ne >= INT32_MAX || nt >= INT32_MAX || nv >= INT32_MAX) return VC_ERR_ARG;
    // the complex becomes the context's finalized cell complex
    c->cc_valid = c->cc_finalized = c->meas_valid = c->thin_valid = c->rem_valid = false;
    VC_TRY(ensure_n<float>(c, c->vts, 3 * nv));
    VC_TRY(ensure_n<int2>(c, c->edges, ne));
    VC_TRY(ensure_n<int32_t>(c, c->tris, 3 * nt));
    VC_TRY(ensure_n<int32_t>(c, c->tri_edges, 3 * nt));
    VC_TRY(ensure_n<float>(c, c->vm, nv));
    VC_TRY(ensure_n<float>(c, c->em, ne));
    VC_TRY(ensure_n<float>(c, c->fm, nt));
    VC_TRY(ensure_n<int32_t>(c, c->vd_tri_face, nt));
    VC_TRY(ensure_n<int2>(c, c->vd_face_sites, nface));
    int32_t* bbox = ptr<int32_t>(c->vd_bbox);
    init_bbox_kernel<<<1, 32, 0, c->stream>>>(bbox);
    launched(c);
    const float* sxyz = ptr<float>(c->site_xyz);
    {
    Region r(c, "vd_emit");
    vd_vertices_kernel<<<grid_for(c, N, 256), 256, 0, c->stream>>>(g, flags, voff, sxyz, ptr<float>(c->vts),
                                                                    ptr<float>(c->vm), bbox, N);
    launched(c);
    vd_edges_kernel<<<grid_for(c, N, 256), 256, 0, c->stream>>>(g, flags, voff, eoff, sxyz, ptr<int2>(c->edges),
                                                                 ptr<float>(c->em), N);
    launched(c);
    vd_faces_kernel<<<grid_for(c, N, 256), 256, 0, c->stream>>>(
        g, flags, voff, eoff, foff, sxyz, (int32_t)ne_axis, ptr<int2>(c->edges), ptr<float>(c->em),
        ptr<int32_t>(c->tris), ptr<int32_t>(c->tri_edges), ptr<float>(c->fm), ptr<int32_t>(c->vd_tri_face),
        ptr<int2>(c->vd_face_sites), N);
    launched(c);
    }
    VC_CUDA(c, cudaGetLastError());
    int32_t hb[6];
    VC_CUDA(c, cudaMemcpyAsync(hb, bbox, 6 * sizeof(int32_t), cudaMemcpyDeviceToHost, c->stream));
    VC_TRY(sync_check(c));
    float isz = 0.0f;
    if (nv > 0) {
        // trimesh::box::size().max() over float vertex coordinates
        const float sx = (float)hb[3] - (float)hb[0], sy = (float)hb[4] - (float)hb[1],
                    sz = (float)hb[5] - (float)hb[2];
        isz = std::max(sx, std::max(sy, sz));
    }
    c->nv = nv;
    c->ne_in = ne;
    c->ne = ne;
    c->nt = nt;
    c->vd = vc_vd_sizes{nv, ne, nt, nface, isz};
    c->vd_valid = true;
    c->cc_valid = true;
    VC_TRY(build_adjacency(c));
    c->cc_finalized = true;
    c->meas_valid = true;
    if (sizes) *sizes = c->vd;
    return VC_OK;
}

}  // namespace vc
