// CPU restatement of the Voxel Cores hot path ("oracle").
//
// TEST INFRASTRUCTURE.  Only tests/, __graft_entry__.smoke() and the
// cpu_baseline / reference legs of bench.py may load liboracle.so, and only as
// the checker or as the timed CPU baseline -- never as part of the product
// path.  Each function cites the reference file:line whose behaviour it
// restates; the restatement itself is checked against the reference's own
// sources compiled in oracle/_ref (see tests/test_oracle_vs_reference.py).
//
// Conventions shared with the GPU library:
//   * occupancy volume: uint8 X*Y*Z, x-major (z fastest); inside <=> value > 0;
//     voxels outside the box count as outside (spaceinfo.h:122-129).
//   * corner lattice: (X+1)*(Y+1)*(Z+1) points, point (a,b,c) sits at voxel
//     coordinates (a-0.5, b-0.5, c-0.5); linear index (a*(Y+1)+b)*(Z+1)+c.
//   * sites: boundary voxel corners in the reference's first-encounter order.
//   * feature transform: for every lattice point, d2 = squared distance (voxel
//     units, exact integer) to the nearest site and id = index of that site;
//     ties go to the lowest site index.
#pragma once
#include <cstdint>

#ifdef __cplusplus
extern "C" {
#endif

// Boundary-corner sites (surfacing.cpp:223-321).  Returns the site count;
// writes up to `cap` entries of xyz (float voxel coordinates) and of the
// site's corner-lattice linear index (either pointer may be null).
long long vco_extract_sites(const uint8_t* occ, int X, int Y, int Z, float* xyz, int64_t* lattice_idx,
                            long long cap);

// Exact feature transform by brute force over all sites (small cases only).
void vco_ft_bruteforce(int X, int Y, int Z, long long nsites, const int64_t* site_lattice_idx, int32_t* d2,
                       int32_t* id);

// Exact feature transform by three separable lower-envelope passes with
// integer crossing thresholds that carry the lowest-index tie-break.
void vco_ft(int X, int Y, int Z, long long nsites, const int64_t* site_lattice_idx, int32_t* d2, int32_t* id,
            int nthreads);

// Inside part of the lattice Voronoi complex with lambda measures, laid out
// as VoroInfo::extractInsideWithMeasure lays out its outputs
// (voroinfo.cpp:624-729).  Returns an opaque handle.
void* vco_lattice_vd(const uint8_t* occ, int X, int Y, int Z, const int32_t* ft_id, const float* site_xyz);
void vco_vd_sizes(void* h, long long* nv, long long* ne, long long* nt, long long* nface, float* inside_size);
// The sizes vco_lattice_vd would give, {nv, ne, nt, nface}, and its inside
// size, counted without building the complex (same validity rules).
void vco_lattice_vd_counts(const uint8_t* occ, int X, int Y, int Z, const int32_t* ft_id, long long* sizes,
                           float* inside_size);
// vts: nv*3 float; edges: ne*2 int; tris: nt*3 int; vm/em/fm: measures (fm per
// triangle); tri_face: polygon face index per triangle; face_sites: nface*2.
void vco_vd_get(void* h, float* vts, int32_t* edges, int32_t* tris, float* vm, float* em, float* fm,
                int32_t* tri_face, int32_t* face_sites);
// Radius per vertex (nv floats), VoroInfo::computeInfoRelatedtoSites
// (voroinfo.cpp:286-325): distance from the vertex to the first site of the
// last Voronoi face, in face order, that has the vertex.
void vco_vd_radius(void* h, float* radius);
void vco_vd_free(void* h);

// cellcomplex(vts, edges, tris).finalize() (cellcomplex.cpp:13-26, 364-491):
// returns the finalized edge count; with non-null outputs also writes the
// finalized edge list (ne_out*2), per-triangle edge ids (nt*3), V->E CSR
// (ve_off nv+1, ve_ids 2*ne_out) and E->F CSR (ef_off ne_out+1, ef_ids 3*nt).
long long vco_finalize(long long nv, long long ne, const int32_t* edges, long long nt, const int32_t* tris,
                       int32_t* edges_out, int32_t* tri_edges, int32_t* ve_off, int32_t* ve_ids, int32_t* ef_off,
                       int32_t* ef_ids);

// CellComplexThinning::prune(f_t, l_t) on the finalized complex
// (ccthin.cpp:201-424, 514-771).  em has one entry per FINALIZED edge, fm one
// per triangle.  Outputs (per finalized cell): keep_v = vertex not removed,
// keep_e = edge not removed and unreferenced (getRemainedEdges), keep_f = face
// not removed, removed_e = edge removal tag.  Returns 0, or -1 when the
// reference would have hit its exit(1) invariant check (ccthin.cpp:570-584).
// stats (may be null): [0] queue pushes, [1] pops processed, [2] pops skipped,
// [3] FIFO generations.
int vco_thin(long long nv, long long ne, const int32_t* edges, long long nt, const int32_t* tris, const float* em,
             const float* fm, float f_t, float l_t, uint8_t* keep_v, uint8_t* keep_e, uint8_t* keep_f,
             uint8_t* removed_e, long long* stats);

// remainingCC (ccthin.cpp:467-512) from the finalized complex and the
// survivor flags: compacted vertices (float3), edges and triangles.  Two-call:
// pass null outputs to get the sizes.
void vco_remaining(long long nv, const float* vts, long long ne_fin, const int32_t* edges_fin, long long nt,
                   const int32_t* tris, const uint8_t* keep_v, const uint8_t* keep_e, const uint8_t* keep_f,
                   long long* nv_out, long long* ne_out, long long* nt_out, float* vts_out, int32_t* edges_out,
                   int32_t* tris_out);

// util::computeEulerChar(vts, edges, tris) (geomalgo.cpp:181-214):
// out = {V, E, F, C, euler}.
void vco_euler(long long nv, long long ne, const int32_t* edges, long long nt, const int32_t* tris, long long* out);

// nClosedComponents(cc) (highlevelalgo.cpp:993-1020): the thinning with every
// measure 0 and both thresholds 1 (every pair passes), then the number of
// face-connected components of the remaining faces (cellcomplex::
// compute_conn_cmpnts, cellcomplex.cpp:73-147: faces joined through shared
// edges), 0 when no face remains; -1 on the invariant case of vco_thin.
long long vco_closed_components(long long nv, long long ne, const int32_t* edges, long long nt, const int32_t* tris);

// A .sof octree file (OctreeVolume::read_sof_file, octree.cpp:259-357): an
// int32 resolution R (a power of two), then the nodes in pre-order, each a
// type byte -- 0 internal (eight children, x outermost, z innermost), 1
// empty (a sign byte: 1 outside, else inside, for every cell below), 2 leaf
// (one cell; bit 4x+2y+z = corner (x,y,z) outside).  Decoded as the
// reference reads it: the occupancy of the (R+1)^3 voxels (getDataAt,
// octree.cpp:233-256: the voxel's own cell, its lowest corner, or for a
// coordinate R the last cell's far corner; get_occupancy_at_vox) and the
// sites of its octree branch of Surfacer::extractBoundaryVts
// (surfacing.cpp:286-301, 666-685: the centre (x+.5,y+.5,z+.5) of every
// leaf whose corners differ, in pre-order).  Two-call: with occ and sites
// null only *size_out = R+1 and *nsites are set.  Returns 0, or -1 when the
// stream is malformed.
int vco_sof_decode(const uint8_t* bytes, long long nbytes, int* size_out, uint8_t* occ, float* sites,
                   long long* nsites);
/* The same for a .sog file (octree.cpp:351-498): 128-byte header, R, nodes
 * with 12 bytes after each leaf's corner byte. */
int vco_sog_decode(const uint8_t* bytes, long long nbytes, int* size_out, uint8_t* occ, float* sites,
                   long long* nsites);

/* Output formats of the remaining complex (see vc_oracle.cpp). */
int vco_write_dotma(const char* path, const float* vts, const float* radii, long long nv, const int32_t* edges,
                    long long ne, const int32_t* tris, long long nt);
int vco_write_radii(const char* path, const float* vts, const float* radii, long long n);
int vco_write_ply(const char* path, const float* vts, long long nv, const int32_t* edges, long long ne,
                  const int32_t* tris, long long nt);
long long vco_dotma_edges(const int32_t* edges, long long ne, const int32_t* tris, long long nt, int32_t* out);

#ifdef __cplusplus
}
#endif
