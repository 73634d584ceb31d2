/*
 * voxelcore_gb300.h -- C ABI of the GB300 (sm_103a) Voxel Cores hot path.
 *
 * One context = one CUDA stream on one device.  Every entry point returns an
 * int status (VC_OK or a VC_ERR_* code); nothing exits the process and no
 * exception crosses the ABI.  Array arguments are plain pointers; `mem` says
 * whether a pointer is host memory (VC_MEM_HOST) or device memory on the
 * context's device (VC_MEM_DEVICE).  The context owns every intermediate
 * buffer; getters copy out and, for host destinations, synchronize.
 *
 * Each group of entry points replaces one reference interface; the citations
 * are into the reference project (danielyan86129/voxel_ma).
 */
#ifndef VOXELCORE_GB300_H
#define VOXELCORE_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define VC_OK 0
#define VC_ERR_ARG 1       /* bad argument, size or degenerate input            */
#define VC_ERR_OOM 2       /* device allocation failed                           */
#define VC_ERR_TIMEOUT 3   /* a bounded device-side wait gave up                 */
#define VC_ERR_INVARIANT 4 /* the reference's exit(1) check (ccthin.cpp:570-584) */
#define VC_ERR_CUDA 5      /* CUDA runtime error (see vc_ctx_last_error)         */
#define VC_ERR_STATE 6     /* entry point called before its inputs exist         */

#define VC_MEM_HOST 0
#define VC_MEM_DEVICE 1

typedef struct vc_ctx vc_ctx;

/* ---- context ----------------------------------------------------------- */
int vc_version(void);
const char* vc_status_string(int status);
/* Create a context on `device`, with its own non-blocking stream. */
int vc_ctx_create(vc_ctx** ctx, int device);
int vc_ctx_destroy(vc_ctx* ctx);
/* The context's cudaStream_t (as void*), for event timing by the caller. */
void* vc_ctx_stream(vc_ctx* ctx);
int vc_ctx_sync(vc_ctx* ctx);
const char* vc_ctx_last_error(vc_ctx* ctx);
/* Bytes of device memory currently held by the context's buffers. */
int64_t vc_ctx_device_bytes(vc_ctx* ctx);
/* Number of kernels the library has launched on this context. */
int64_t vc_ctx_launch_count(vc_ctx* ctx);
/* CUDA-event timing of the library's named regions on the context stream
 * (off by default).  get_timings writes up to `cap` entries: region names
 * (each `name_len` bytes, NUL-terminated), accumulated ms and counts; *n is
 * the number of regions recorded.                                          */
int vc_ctx_set_timing(vc_ctx* ctx, int enable);
int vc_ctx_reset_timings(vc_ctx* ctx);
int vc_ctx_get_timings(vc_ctx* ctx, char* names, int name_len, double* ms, int64_t* counts, int cap, int* n);

/* ---- volume and boundary sites -----------------------------------------
 * Replaces Surfacer::extractBoundaryVts(const shared_ptr<Volume3DScalar>&,
 * vector<point>&) (include/surfacing.h:57-58, src/surfacing.cpp:223-321).
 * occ: X*Y*Z bytes, x-major (z fastest), inside <=> value > 0; voxels outside
 * the box count as outside (include/spaceinfo.h:122-129).  Sites come out in
 * the reference's first-encounter order as float xyz voxel coordinates.   */
int vc_set_volume(vc_ctx* ctx, const uint8_t* occ, int X, int Y, int Z, int mem);
/* An octree volume from the bytes of a .sof file (OctreeVolume::
 * read_sof_file, src/octree.cpp:259-357): decoded on the GPU into the
 * (R+1)^3 occupancy the reference's OctreeVolume::getDataAt gives
 * (src/octree.cpp:233-256), and *size = R+1.  vc_extract_sites then follows
 * the reference's octree rule (Surfacer::extractBoundaryVts,
 * src/surfacing.cpp:286-301, 666-685): the centres of the leaves whose
 * corners differ, in the file's order.  VC_ERR_ARG for a malformed stream,
 * a resolution that is not a power of two, or a leaf above the cell level. */
int vc_set_volume_sof(vc_ctx* ctx, const void* bytes, int64_t nbytes, int* size);
/* The same from a .sog file (OctreeVolume::read_sog_file,
 * src/octree.cpp:351-498): a 128-byte header opening with "SOG.Format 1.0"
 * (VC_ERR_ARG otherwise), the lower-left corner and bounding-box length as
 * floats, then R and the nodes, each leaf followed by its feature point
 * (three floats, skipped).  The volume's voxel-to-model matrix becomes
 * trans(lower-left) * scale(length / R), as the reference sets it.         */
int vc_set_volume_sog(vc_ctx* ctx, const void* bytes, int64_t nbytes, int* size);
/* A density map from the bytes of an .mrc file: the reference's readMRC
 * (src/importers.cpp:45-60: Tao Ju's MRC reader wrapped as a DenseVolume,
 * inside <=> value > 0).  Tao's reader is not in the reference tree, so this
 * follows the public MRC2014 layout: a 1024-byte header (column / row /
 * section counts, mode 0 int8, 1 int16, 2 float32, 6 uint16 or 12 float16,
 * the axis of columns / rows / sections, the extended-header length, the
 * machine stamp for the byte order) and the values, columns fastest.  The
 * map becomes the context's volume, dims = its X, Y, Z.  VC_ERR_ARG for an
 * unknown mode, a bad size or a truncated file.                            */
int vc_set_volume_mrc(vc_ctx* ctx, const void* bytes, int64_t nbytes, int* dims);
/* The X, Y, Z of an .mrc file's map (header only; no context).            */
int vc_mrc_dims(const void* bytes, int64_t nbytes, int* dims);
/* The installed volume's voxel-to-model matrix (16 doubles, column-major as
 * trimesh::xform): the identity except for .sog volumes.                   */
int vc_get_vox_to_model(vc_ctx* ctx, double* m);
/* The installed occupancy (all volumes of a batch, one after another).     */
int vc_get_volume(vc_ctx* ctx, uint8_t* occ, int mem);
/* The .sof stream of an X*Y*Z host occupancy volume (x-major, z fastest) as
 * the reference writes it (OctreeVolume(const Volume3DScalar*) and
 * write_sof_file, src/octree.cpp:50-63, 499-560, 864-930).  Host code, no
 * context.  *nbytes = the stream's length; with out non-null and cap at
 * least that, the stream is copied to out.                                 */
int vc_encode_sof(const uint8_t* occ, int X, int Y, int Z, uint8_t* out, int64_t cap, int64_t* nbytes);
/* The .sog stream of the same octree (write_sog_file, src/octree.cpp:569-668):
 * header (title, lower-left 0, length R; the header bytes the reference
 * leaves uninitialised are zero), R, the nodes with each leaf's cell centre. */
int vc_encode_sog(const uint8_t* occ, int X, int Y, int Z, uint8_t* out, int64_t cap, int64_t* nbytes);
/* Sites of the installed volume; a second call for the same volume returns
 * the count of the sites already on the device without recomputing them.  */
int vc_extract_sites(vc_ctx* ctx, int64_t* n_sites);
int vc_get_sites(vc_ctx* ctx, float* xyz, int mem);

/* ---- exact feature transform -------------------------------------------
 * No reference function: the reference keeps the nearest-boundary-point
 * relation only implicitly, as the two sites of each Voronoi face
 * (src/voroinfo.cpp:185-231).  On the (X+1)(Y+1)(Z+1) corner lattice (point
 * (a,b,c) at voxel coordinates (a-.5,b-.5,c-.5)) d2 = exact squared distance
 * to the nearest site, id = that site's index; ties -> lowest index.       */
int vc_feature_transform(vc_ctx* ctx);
int vc_get_ft(vc_ctx* ctx, int32_t* d2, int32_t* id, int mem);

/* ---- lattice Voronoi complex, inside part, with lambda measures ---------
 * Replaces VoroInfo::extractInsideWithMeasure(MeasureForMA::LAMBDA, vts,
 * edges, tris, from_fi, vts_msure, edges_msure, faces_msure)
 * (include/voroinfo.h:127-131, src/voroinfo.cpp:624-729) for the Voronoi
 * complex read off the feature transform; lambda as in
 * MeasureForMA::lambdaForFace (include/measureforMA_imp.h:1-4) and
 * src/voroinfo.cpp:1432-1574.  The resulting complex is also installed as
 * the context's (already finalized) cell complex.                         */
typedef struct {
    int64_t nv, ne, nt, nface;
    float inside_size; /* VoroInfo::getInsidePartSize (voroinfo.cpp:496)   */
} vc_vd_sizes;
int vc_lattice_vd(vc_ctx* ctx, vc_vd_sizes* sizes);
int vc_get_vd(vc_ctx* ctx, float* vts, int32_t* edges, int32_t* tris, int32_t* tri_face, float* vm, float* em,
              float* fm, int32_t* face_sites, int mem);

/* Radius per vertex of the lattice complex (nv floats, vc_get_vd's vertex
 * order).  Replaces VoroInfo::computeInfoRelatedtoSites
 * (src/voroinfo.cpp:286-325) + VoroInfo::getRadii (include/voroinfo.h):
 * r = dist(vertex, first site of the last Voronoi face, in face order, that
 * has the vertex); the values writeRadiiToFile (src/exporters.cpp:478-552)
 * writes for the valid vertices.  Needs vc_lattice_vd.                    */
int vc_vertex_radii(vc_ctx* ctx, float* radius, int mem);

/* ---- cell complex in ----------------------------------------------------
 * Replaces cellcomplex(const vector<point>&, const vector<ivec2>&,
 * const vector<uTriFace>&, bool finalize = true) + cellcomplex::finalize()
 * (include/cellcomplex.h:33-34, 106; src/cellcomplex.cpp:13-26, 364-491):
 * edge ids keep the given order, new face sides are appended in face order,
 * V->E lists are in edge-id order and E->F lists in face-id order.
 * Triangles with a repeated vertex and loop edges are rejected (VC_ERR_ARG). */
int vc_set_complex(vc_ctx* ctx, int64_t nv, const float* vts, int64_t ne, const int32_t* edges, int64_t nt,
                   const int32_t* tris, int mem);
int vc_finalize(vc_ctx* ctx, int64_t* ne_final);
int vc_get_finalized(vc_ctx* ctx, int32_t* edges, int32_t* tri_edges, int32_t* ve_off, int32_t* ve_ids,
                     int32_t* ef_off, int32_t* ef_ids, int mem);

/* ---- measures -----------------------------------------------------------
 * Replaces CellComplexThinning::assignElementValues (src/ccthin.cpp:178-189):
 * vm per vertex, em per FINALIZED edge, fm per triangle.                   */
int vc_set_measures(vc_ctx* ctx, const float* vm, const float* em, const float* fm, int mem);

/* ---- thinning -----------------------------------------------------------
 * Replaces CellComplexThinning::prune(float f_t, float l_t, bool)
 * (src/ccthin.cpp:201-424, 514-771): the same surviving set as the
 * reference's FIFO queue, replayed generation by generation on the GPU.   */
typedef struct {
    int64_t pushes, processed, skipped, generations;
} vc_thin_stats;
int vc_thin(vc_ctx* ctx, float f_t, float l_t, vc_thin_stats* stats);
/* keep_v: !removed; keep_e: !removed && no remaining face
 * (getRemainedEdges, ccthin.cpp:156-166); keep_f: !removed;
 * removed_e: getEdgeRemovedTags (ccthin.cpp:117-120).  Any may be NULL.    */
int vc_get_thin_flags(vc_ctx* ctx, uint8_t* keep_v, uint8_t* keep_e, uint8_t* keep_f, uint8_t* removed_e, int mem);

/* ---- remaining complex --------------------------------------------------
 * Replaces CellComplexThinning::remainingCC(vector<point>&, vector<ivec2>&,
 * vector<uTriFace>&, vector<int>*) (src/ccthin.cpp:467-512), including the
 * re-triangulation (a,b,c)->(c,a,b) and util::compactify.                 */
typedef struct {
    int64_t nv, ne, nt;
} vc_rem_sizes;
int vc_remaining(vc_ctx* ctx, vc_rem_sizes* sizes);
int vc_get_remaining(vc_ctx* ctx, float* vts, int32_t* edges, int32_t* tris, int mem);

/* ---- output formats -----------------------------------------------------
 * The files the reference writes for the remaining complex after thinning at
 * one threshold (src/highlevelalgo.cpp:855-955), byte for byte:
 *   vc_write_ply    replaces writeToPLY (src/exporters.cpp:341-476) and
 *                   ply::PLYWriter::write (src/plyall.cpp:98-171): ASCII PLY,
 *                   vertex x y z, edge vertex1 vertex2, face vertex_indices.
 *   vc_write_radii  replaces writeRadiiToFile (src/exporters.cpp:478-552)
 *                   with the remaining vertex ids and the identity
 *                   voxel-to-model matrix: "n", then "x y z r" per vertex.
 *   vc_write_dotma  replaces writeToDotma (src/exporters.cpp:244-287).
 * Host arrays; VC_ERR_ARG when the file cannot be written.
 * vc_write_remaining writes <prefix>.ply / .r / .ma (VC_WRITE_* bits) from
 * the context's remaining complex (vc_remaining); the radii need the lattice
 * complex of one volume (vc_lattice_vd), else VC_ERR_STATE.  The .ma edge
 * list is the caller's (src/highlevelalgo.cpp:911-945): the remaining
 * edges, then the remaining triangles' edges in the order of its
 * unordered_set<ivec2, ivec2Hash>.                                          */
#define VC_WRITE_PLY 1
#define VC_WRITE_RADII 2
#define VC_WRITE_MA 4
int vc_write_ply(const char* path, const float* vts, int64_t nv, const int32_t* edges, int64_t ne,
                 const int32_t* tris, int64_t nt);
int vc_write_radii(const char* path, const float* vts, const float* radii, int64_t n);
int vc_write_dotma(const char* path, const float* vts, const float* radii, int64_t nv, const int32_t* edges,
                   int64_t ne, const int32_t* tris, int64_t nt);
int vc_write_remaining(vc_ctx* ctx, const char* prefix, int what);
/* The .ma edge list vc_write_remaining writes, for given remaining edges and
 * triangles (ne_out pairs; out may be NULL to size it, cap in pairs).       */
int vc_dotma_edges(const int32_t* edges, int64_t ne, const int32_t* tris, int64_t nt, int32_t* out, int64_t cap,
                   int64_t* ne_out);

/* ---- topology of the remaining complex ----------------------------------
 * util::computeEulerChar(vts, edges, tris, eulerchar&)
 * (src/geomalgo.cpp:181-214) on the remainingCC output.                    */
typedef struct {
    int64_t V, E, F, C, euler;
} vc_euler_info;
int vc_euler_remaining(vc_ctx* ctx, vc_euler_info* out);

/* nClosedComponents(cc) (src/highlevelalgo.cpp:993-1020) on the installed
 * finalized complex (vc_finalize, or the lattice complex after
 * vc_lattice_vd): the thinning with every measure 0 and both thresholds 1 --
 * every pair passes, so only closed pockets survive -- then the number of
 * face-connected components of the remaining faces (cellcomplex::
 * compute_conn_cmpnts, src/cellcomplex.cpp:73-147), 0 when no face remains.
 * Installed measures are neither read nor changed; the thinning flags and
 * statistics of the context are this thinning's afterwards.                 */
int vc_closed_components(vc_ctx* ctx, int64_t* n_closed);

/* ---- the plain single-volume path ---------------------------------------
 * Sites, feature transform, lattice Voronoi complex with measures,
 * thinning at thresh = float(inside_size * t) (highlevelalgo.cpp:825-837)
 * and the remaining complex, in one call (exportInsideVoroMesh's .ply
 * branch without file output, highlevelalgo.cpp:731-961).                 */
typedef struct {
    int64_t n_sites;
    vc_vd_sizes vd;
    float thresh;
    vc_thin_stats thin;
    vc_rem_sizes rem;
} vc_plain_result;
int vc_run_plain(vc_ctx* ctx, const uint8_t* occ, int X, int Y, int Z, int mem, double t, vc_plain_result* out);

/* ---- batched path --------------------------------------------------------
 * Many volumes through one pass of the pipeline: every stage is one set of
 * launches over all volumes of the batch (per-volume tables on the device)
 * and the thinning replays the FIFO of all their complexes at once.  The
 * reference processes one volume per exportInsideVoroMesh call
 * (src/highlevelalgo.cpp:731-961); each volume's results here are those of
 * vc_run_plain on that volume alone (its own site order, threshold
 * float(inside_size_b * t) and surviving set): the volumes' complexes share
 * no cell, and the FIFO order restricted to one complex is the order of
 * that complex alone.
 *
 * vc_batch_set_volumes: dims = 3 ints (X, Y, Z) per volume, each in
 * [1, 32766]; occ = the volumes' voxels one after another (each x-major, z
 * fastest), host or device per `mem`.                                      */
typedef struct {
    int64_t n_sites;
    vc_vd_sizes vd;        /* the volume's lattice complex and inside-part size */
    float thresh;          /* float(inside_size * t) */
    vc_rem_sizes rem;      /* its remaining complex */
    vc_euler_info euler;   /* of its remaining complex (with_euler != 0) */
    int64_t site_off;                   /* first site in vc_get_sites */
    int64_t v_off, e_off, t_off;        /* first cell in the batch complex (vc_get_vd, vc_get_thin_flags) */
    int64_t rem_v_off, rem_e_off, rem_t_off;  /* first cell in vc_get_remaining (ids local to the volume) */
} vc_batch_volume;
int vc_batch_set_volumes(vc_ctx* ctx, int nvol, const int32_t* dims, const uint8_t* occ, int mem);
/* Runs sites -> feature transform -> lattice complex with lambda -> thinning
 * -> remaining complex (-> Euler characteristic and components) for every
 * volume; out (host) receives nvol entries, stats (optional) the totals of
 * the batch's thinning.                                                    */
int vc_batch_run(vc_ctx* ctx, double t, int with_euler, vc_thin_stats* stats, vc_batch_volume* out);

/* ---- request loop (continuous batching) ---------------------------------
 * The reference serves one volume per process run (src/voroUtility.cpp
 * main -> exportInsideVoroMesh, src/highlevelalgo.cpp:731-961).  A server
 * queues volumes as they are submitted and `workers` threads, each with its
 * own context and stream, serve them: a worker that becomes free takes the
 * oldest pending requests that fit as one batch (vc_batch_run), so requests
 * that arrive while other batches are on the GPU join the next batch, and
 * the workers' batches overlap on the device.  Memory admission: a request's
 * footprint is estimated as bytes_per_voxel (default 640) x voxels; a batch
 * must fit mem_cap_bytes / workers, a request that cannot is refused at
 * submission (VC_ERR_ARG), and a worker whose context holds more than its
 * share after a batch frees its buffers.  Each result equals the plain
 * single-volume result for that volume.  Submission copies the volume
 * (host memory); results stay until vc_server_release.                     */
typedef struct vc_server vc_server;
typedef struct {
    int status;        /* VC_OK, or the status of the batch the request ran in */
    int batch_size;    /* requests in that batch */
    int64_t n_sites;
    vc_vd_sizes vd;
    float thresh;
    vc_rem_sizes rem;
    vc_euler_info euler;
    double queue_ms;   /* submission -> start of its batch */
    double run_ms;     /* start of its batch -> results on the host */
    double latency_ms; /* submission -> results on the host */
} vc_request_result;
typedef struct {
    int64_t submitted, completed, failed, refused, batches, pending, device_bytes;
} vc_server_stats;
int vc_server_create(vc_server** server, int device, int workers, int64_t mem_cap_bytes, int max_batch);
/* The same server over several GPUs: workers_per_device workers on each of
 * devices[0..ndev), each device with its own memory cap; a free worker on
 * any device takes the next batch, so whole volumes go to whichever GPU is
 * free (a volume is never split across GPUs; the reference thins one volume
 * per process).  vc_server_create(dev, w, cap, b) is this with one device. */
int vc_server_create_devices(vc_server** server, const int* devices, int ndev, int workers_per_device,
                             int64_t mem_cap_per_device, int max_batch);
/* Whole volumes to nparts parts (GPUs or ranks) by voxels, largest first to
 * the part with the fewest voxels so far (lowest part on ties); part_of[i]
 * receives volume i's part.  Host code, no context.  Each part runs its
 * share as one batch; the union of the parts' results equals the result of
 * the whole set, volume by volume.                                         */
int vc_partition_volumes(int n, const int64_t* voxels, int nparts, int32_t* part_of);
int vc_server_set_bytes_per_voxel(vc_server* server, double bytes_per_voxel);
int vc_server_submit(vc_server* server, const uint8_t* occ, int X, int Y, int Z, double t, int64_t* request_id);
/* Blocks until the request is served (timeout_s < 0: no limit; a host-side
 * wait that returns VC_ERR_TIMEOUT when the limit passes).                 */
int vc_server_wait(vc_server* server, int64_t request_id, double timeout_s, vc_request_result* out);
/* The request's remaining complex (sizes in its vc_request_result.rem).    */
int vc_server_get_remaining(vc_server* server, int64_t request_id, float* vts, int32_t* edges, int32_t* tris);
int vc_server_release(vc_server* server, int64_t request_id);
int vc_server_get_stats(vc_server* server, vc_server_stats* out);
int vc_server_destroy(vc_server* server);
/* Failure injection: the next batch a worker takes runs with
 * vc_debug_fail_alloc_after(k) on its context, so its requests fail with
 * VC_ERR_OOM; later batches run normally.                                  */
int vc_server_debug_fail_alloc_after(vc_server* server, int64_t k);
/* The batching rule the workers apply, on a list of requests in arrival
 * order: consecutive requests share a batch while they have the same t, the
 * batch holds fewer than max_batch requests and bytes_per_voxel x voxels
 * summed over it stays within share_bytes; batch_of[i] receives request i's
 * batch number, or -1 when the request alone exceeds the share.  Host only. */
int vc_plan_batches(int n, const int64_t* voxels, const double* t, int64_t share_bytes, double bytes_per_voxel,
                    int max_batch, int32_t* batch_of);

/* ---- site extraction without device allocation ---------------------------
 * No counterpart in the reference.  For callers that cannot call cudaMalloc
 * (a host framework or allocator that owns the device heap, or a plugin that
 * must not grow the process's device footprint): the same sites as
 * vc_extract_sites + vc_get_sites, computed with no context and no
 * allocation.  The scratch is a fixed array inside the library that every
 * GPU loading the library holds until the process exits; volumes are
 * limited to 4,194,304 voxels (X*Y*Z), larger ones return VC_ERR_ARG.
 * occ: device pointer to X*Y*Z bytes; xyz: device pointer with room for
 * `capacity` sites (3 floats each); *n_sites (host) receives the site count
 * -- when it exceeds `capacity` the call returns VC_ERR_ARG and writes no
 * site.  stream: a cudaStream_t (NULL = the legacy default stream); the
 * call synchronizes it.  The first call on a device looks up the scratch
 * addresses, so make it before capturing a stream on that device.  All
 * calls share the scratch: calls that overlap on the GPU (other streams or
 * host threads) race and must be serialized by the caller.                */
int vc_extract_sites_noalloc(const uint8_t* occ, int X, int Y, int Z, float* xyz, int64_t capacity, int64_t* n_sites,
                             void* stream);

/* FP64 cross-check of the lattice complex's face measures: every face's
 * lambda is recomputed in double from its two sites.  *max_rel_err = the
 * largest |lambda_float - lambda_double| / lambda_double; *flips = how many
 * faces' threshold test (lambda < the volume's threshold) differs in double
 * (-1 when the complex was built without thresholds, vc_lattice_vd).  The
 * path keeps the reference's float semantics (trimesh::dist in float,
 * measureforMA_imp.h:1-4); lambda is the correctly rounded square root of
 * an exact integer, so no FP64 rescue is needed and this is a report.     */
int vc_lambda_fp64_check(vc_ctx* ctx, double* max_rel_err, int64_t* flips);

/* ---- autotuner -----------------------------------------------------------
 * Chooses, for the volume or batch installed in the context (vc_set_volume
 * or vc_batch_set_volumes), the launch shapes of the two kernels whose best
 * shape depends on the input: the feature transform's envelope passes (how
 * many stack entries of each line stay in shared memory: 4, 8 or 16; then
 * the envelope or the window method, see vc_set_ft_method) and
 * the thinning kernel (threads per block and blocks per SM: 512 x 2,
 * 512 x 2 with two items per thread, 512 x 4, 256 x 8, 1024 x 1).  Each candidate runs on the installed input
 * and is timed with CUDA events on the context's stream (after one untimed
 * run); the fastest stays in the context for every later run of it.  Results
 * never depend on these shapes.  t is the thinning's threshold factor, as
 * in vc_run_plain.  The reference has no counterpart (it is single-threaded
 * C++).                                                                    */
typedef struct {
    int ft_ring;                /* chosen (envelope kernel) */
    int thin_threads;           /* chosen */
    int thin_blocks_per_sm;     /* chosen */
    float ft_ms[3];             /* both envelope passes, ring 4 / 8 / 16 */
    int thin_items;             /* chosen: items per thread in the thinning's first phase */
    float thin_ms[5];           /* thinning kernel, 512x2 / 512x2 with 2 items / 512x4 / 256x8 / 1024x1 */
    int ft_method;              /* chosen: VC_FT_ENVELOPE or VC_FT_WINDOW */
    float ft_window_ms;         /* both passes with the window kernel (envelope ring: the best of ft_ms) */
} vc_tune_result;
int vc_autotune(vc_ctx* ctx, double t, vc_tune_result* out);

/* Method of the feature transform's y and x passes (results are identical):
 * VC_FT_ENVELOPE: lower envelope of the parabolas, one thread per line; its
 *   cost per point does not depend on the distances.
 * VC_FT_WINDOW: a window kernel first -- each point scans outward from
 *   itself until no farther candidate can win or tie, over tiles of 32 lines
 *   staged in shared memory -- which is faster on dense inputs (distances of
 *   a few voxels, e.g. random fields); tiles whose scans run long are left to
 *   the envelope kernel.  Only below 2048 points per axis (otherwise the
 *   envelope runs).
 * VC_FT_AUTO (the default): the window method when the volume or batch has
 *   at least one site per 10 lattice points, else the envelope.
 * vc_autotune times the envelope and the window method on the installed
 * input and keeps the faster.                                              */
#define VC_FT_ENVELOPE 0
#define VC_FT_WINDOW 1
#define VC_FT_AUTO 2
int vc_set_ft_method(vc_ctx* ctx, int method);

/* ---- diagnostics ---------------------------------------------------------
 * Per-generation trace of the thinning kernel: with cap > 0 the next vc_thin
 * records, for up to `cap` generations, {items, t_phaseA, t_phaseB, t_phaseC}
 * (GPU global timer, ns).  blocks_per_sm overrides the persistent grid's
 * blocks per SM (0 = default).                                             */
int vc_debug_thin_trace(vc_ctx* ctx, int cap, int blocks_per_sm);
int vc_debug_get_thin_trace(vc_ctx* ctx, int64_t* out, int cap, int* ngen);
/* Launch shape of the thinning kernel: threads per block (256, 512 or 1024;
 * 0 = library default), blocks per SM (0 = library default) and items per
 * thread in its first phase (1 or 2, 512 x 2 only; 0 = 1).  Results do not
 * depend on it.                                                            */
int vc_debug_thin_shape(vc_ctx* ctx, int threads, int blocks_per_sm, int items);
/* Rate at which this GPU serves random touches of 32-byte records in an
 * array of `bytes` (allocated for the call; rounded down to a power-of-two
 * number of records), the access pattern of the thinning kernel's records:
 * op 0 one 8-byte load per record, 1 two 16-byte loads, 2 one 64-bit
 * atomicAdd whose result is used, 3 an atomicMax and an atomicAdd.  Touches
 * per second, best of three launches of 201 M touches.                     */
int vc_debug_random_rate(vc_ctx* ctx, int op, int64_t bytes, double* touches_per_s);
/* With wide != 0 the feature transform's envelope passes use 64-bit
 * arithmetic even when every lattice axis is below 2048 (where 32-bit
 * arithmetic is exact and is the default); results are identical.         */
int vc_debug_ft_wide(vc_ctx* ctx, int wide);

/* ---- failure injection (host side; no kernel is made to fault) -----------
 * Every device wait of the library is bounded: the thinning kernel's grid
 * barriers give up after `polls` polls (about 64 ns each) and the call
 * returns VC_ERR_TIMEOUT with the context still usable.  polls = 0 restores
 * the default (2^26).                                                      */
int vc_debug_set_spin_limit(vc_ctx* ctx, unsigned long long polls);
/* The next k device allocations of the context succeed and the one after
 * fails, as cudaMallocAsync failing would (VC_ERR_OOM); k < 0 switches it
 * off.  The context stays usable after the failure.                       */
int vc_debug_fail_alloc_after(vc_ctx* ctx, int64_t k);
/* The thinning queue: `capacity` > 0 caps the items one generation may hold
 * (0 = library default: V + E + 1, or the room the device has left when that
 * does not fit), and the queue positions start at `first_position` instead
 * of 0 (positions are unsigned 32-bit; VC_ERR_ARG when first_position + V +
 * E + 1 passes 2^32 - 1).  Results do not depend on either while the largest
 * generation fits; a generation larger than the capacity ends vc_thin with
 * VC_ERR_OOM and the context stays usable.                                */
int vc_debug_thin_queue(vc_ctx* ctx, int64_t capacity, uint32_t first_position);
/* A broken reference count: the next thinnings raise (delta = +1) or lower
 * (-1) vertex `vertex`'s count of incident edges by one after its record is
 * built (delta = 0 switches it off).  An edge-vertex pair popped for that
 * vertex then fails the check the reference makes before removing a pair
 * (src/ccthin.cpp:570-584, which exits the process); here vc_thin returns
 * VC_ERR_INVARIANT.                                                        */
int vc_debug_ref_bias(vc_ctx* ctx, int64_t vertex, int delta);

#ifdef __cplusplus
}
#endif
#endif /* VOXELCORE_GB300_H */
