// Internal definitions shared by the sm_103a kernels of the Voxel Cores hot
// path: the context, its device buffers, error plumbing, block/device scans
// and a bounded grid barrier for cooperative (persistent) kernels.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/voxelcore_gb300.h"

namespace vc {

// ---------------------------------------------------------------------------
// Device-side error word: kernels never trap; they record the first error
// code here and return.  The host reads it back at the next sync point.
enum DeviceError : int {
    kDevOk = 0,
    kDevTimeout = VC_ERR_TIMEOUT,
    kDevInvariant = VC_ERR_INVARIANT,
    kDevArg = VC_ERR_ARG,
};

__device__ __forceinline__ void set_error(int* err, int code) { atomicCAS(err, 0, code); }
inline void set_identity(double* m) {  // 4x4, column-major
    for (int i = 0; i < 16; ++i) m[i] = (i % 5 == 0) ? 1.0 : 0.0;
}

// ---------------------------------------------------------------------------
// A growable device buffer owned by the context (stream-ordered allocation).
struct DevBuf {
    void* p = nullptr;
    size_t cap = 0;
};

template <class T>
T* ptr(const DevBuf& b) {
    return static_cast<T*>(b.p);
}

// Per-cell records of the thinning kernel: static data and thinning state of
// one cell in one DRAM sector (its accesses are random).  Random accesses
// cost per request, not per byte, so each phase of the thinning finds what it
// needs about a cell in one aligned 16-byte piece: a face record is one piece,
// a vertex record is one piece, and an edge record is two: its head (what an
// item removing the edge reads) and its count (what a decrement and the child
// step touch), kept in two arrays, so that the sector a random touch brings
// in holds the same piece of the neighbouring edge (ids follow the lattice).
// Removal state of a face or an edge: the queue position of the item that
// removed it (kAlive while it is present).  Positions are unsigned 32-bit:
// a thinning pushes at most one item per vertex and edge, so they stay
// below V + E < 2^32 - 1.
constexpr uint32_t kAlive = 0xFFFFFFFFu;
// An edge's faces (a vertex's edges) still present, as one 64-bit word: their
// count in bits 0-15, how many of them pass the thinning filter (measure
// below threshold) in bits 16-31, and the sum of their ids (mod 2^32) in
// bits 32-63.  Removing incident cell x subtracts (x << 32) + (pass << 16) +
// 1 in one atomic; when the count is 1 the sum is the id of the one cell
// left and the pass field says whether it passes the filter.  Vertex words
// sum 2 e + p over their edges e instead of e (p = 1 when edge e passes the
// filter, its measure below the edge threshold): when the count is 1 the sum
// is the one edge left, shifted up one bit, with its filter in bit 0; their
// pass field is 1 (kVertGone) once the vertex is removed.
constexpr int kRefBits = 16;
constexpr unsigned long long kRefMask = (1ull << kRefBits) - 1ull;  // largest incidence count
constexpr unsigned long long kVertGone = 1ull << kRefBits;          // vertex word: the vertex was removed
__host__ __device__ __forceinline__ unsigned long long rs_make(unsigned long long count, unsigned long long pass,
                                                               unsigned long long id_sum) {
    return (id_sum << 32) | ((pass & kRefMask) << 16) | count;
}
__host__ __device__ __forceinline__ unsigned long long rs_drop(int32_t id, unsigned pass) {
    return ~(((unsigned long long)(uint32_t)id << 32) + ((unsigned long long)pass << 16) + 1ull) + 1ull;
}
__host__ __device__ __forceinline__ int32_t rs_count(unsigned long long w) { return (int32_t)(w & kRefMask); }
__host__ __device__ __forceinline__ int32_t rs_pass(unsigned long long w) { return (int32_t)((w >> 16) & kRefMask); }
__host__ __device__ __forceinline__ int32_t rs_last(unsigned long long w) { return (int32_t)(uint32_t)(w >> 32); }
// trig: the last decrement of a generation, as (queue position << 1 | bit)
// in 64 bits, bit = which of the decrementing item's cells of that kind this
// is: for an edge, the first or second of the face's other sides (child slot
// 0 or 1); for a vertex, the first or second end of the removed edge (child
// slot 2 or 3).
constexpr int32_t kFacePass = (int32_t)0x80000000u;  // FaceRec::e2 bit: the face passes the filter
struct __align__(16) FaceRec {
    int32_t e0, e1;  // edge ids of the sides, in face order
    int32_t e2;      // third side; bit 31 (kFacePass): measure below the face threshold
    uint32_t rm;
};
struct __align__(16) EdgeHead {  // ends, removal position, measure
    int32_t v0, v1;
    uint32_t rm;
    float em;
};
struct __align__(16) EdgeCnt {  // faces still present (count | pass | id sum), last decrement
    unsigned long long rs;
    unsigned long long trig;
};
// The edge records of a complex of ne edges: ne heads, then ne counts, in
// one buffer of 32 bytes per edge.
struct EdgeRecs {
    EdgeHead* h = nullptr;
    EdgeCnt* n = nullptr;
};
struct __align__(16) VertRec {
    unsigned long long rs;    // edges still present: count | kVertGone once removed | id sum
    unsigned long long trig;  // last decrement: position << 1 | end bit
};
static_assert(sizeof(FaceRec) == 16 && sizeof(EdgeHead) == 16 && sizeof(EdgeCnt) == 16 && sizeof(VertRec) == 16,
              "record size");

// ---------------------------------------------------------------------------
// Volume table.  Every stage runs over a batch of volumes stored one after
// another (volume-major) in each per-voxel, per-lattice-point, per-site and
// per-cell array; one volume is a batch of one.  For each index space a
// kernel walks (voxels, lattice points, voxel rows along z, lattice rows
// along z, lattice lines along y and along x) the table holds the start of
// every volume and, at index nvol, the total.  With one volume nothing is
// read from memory: the starts follow from the dims held in the table.
enum Space : int { kVox = 0, kLat, kVRow, kLRow, kYLine, kXLine, kVWord, kLSeg, kNumSpaces };

__host__ __device__ __forceinline__ int64_t space_size(int s, int X, int Y, int Z) {
    const int64_t x = X, y = Y, z = Z;
    switch (s) {
        case kVox: return x * y * z;
        case kLat: return (x + 1) * (y + 1) * (z + 1);
        case kVRow: return x * y;
        case kLRow: return (x + 1) * (y + 1);
        case kYLine: return (x + 1) * (z + 1);
        case kXLine: return (y + 1) * (z + 1);
        case kVWord: return x * y * ((z + 31) / 32);  // 32-voxel words of the voxel rows
        default: return (x + 1) * (y + 1) * ((z + 32) / 32);  // kLSeg: 32-point segments of the lattice rows
    }
}

struct VolTab {
    int nvol = 0;
    int4 d0{};                      // dims of volume 0 (the only one when nvol == 1)
    const int4* dims = nullptr;     // nvol entries (x, y, z, 0)
    const int64_t* off[kNumSpaces] = {};  // nvol + 1 starts per space

    __device__ __forceinline__ int4 dim(int b) const { return nvol == 1 ? d0 : dims[b]; }
    __device__ __forceinline__ int64_t start(int s, int b) const {
        if (nvol == 1) return b == 0 ? 0 : space_size(s, d0.x, d0.y, d0.z);
        return off[s][b];
    }
    __device__ __forceinline__ int64_t total(int s) const { return start(s, nvol); }
    // find() with a per-thread cache of the last volume and its range: a
    // thread walking nearby indices searches only when it leaves the range
    struct Cache {
        int bv = -1;
        int64_t lo = 0, hi = 0;
    };
    __device__ __forceinline__ int find_cached(int s, int64_t x, Cache& c) const {
        if (x >= c.lo && x < c.hi) return c.bv;
        c.bv = find(s, x);
        c.lo = start(s, c.bv);
        c.hi = start(s, c.bv + 1);
        return c.bv;
    }
    // the volume whose range of space s holds index x
    __device__ __forceinline__ int find(int s, int64_t x) const {
        if (nvol == 1) return 0;
        const int64_t* o = off[s];
        int lo = 0, hi = nvol - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (__ldg(o + mid) <= x) lo = mid;
            else hi = mid - 1;
        }
        return lo;
    }
};

// Per-volume bases of the outputs, filled on the device after the scans
// (nvol + 1 entries each, the last one the total): first site, vertex, axis
// edge, face, axis-edge E->F entry and V->E entry of every volume, and its
// first vertex, edge and triangle of the remaining complex.  The cell
// ids of volume b are volume-major: its vertices, then its axis edges
// followed by its triangulation diagonals, then its triangles, all after
// those of volumes < b.
enum Base : int { kBSite = 0, kBVert, kBAxis, kBFace, kBEfAxis, kBVe, kBRemV, kBRemE, kBRemT, kNumBases };
struct Bases {
    int64_t* b[kNumBases] = {};
    int32_t* bbox = nullptr;  // 6 per volume: min xyz, max xyz of the vertices
    float* inside = nullptr;  // per volume: inside-part size
    float* thr = nullptr;     // per volume: thinning threshold (batched runs)
};

}  // namespace vc

// The opaque context.  Members are grouped by pipeline stage.
struct vc_ctx {
    int device = 0;
    int num_sms = 0;
    cudaStream_t stream = nullptr;
    std::string last_error;
    int64_t bytes_held = 0;

    vc::DevBuf err;      // int device error word + control words
    vc::DevBuf scratch;  // scan tile sums and small temporaries
    vc::DevBuf scratch2;

    // volumes: one (X, Y, Z) or a batch described by the table
    int X = 0, Y = 0, Z = 0;
    int nvol = 0;
    std::vector<int32_t> h_dims;                      // 3 per volume
    std::vector<int64_t> h_off[vc::kNumSpaces];       // nvol + 1 per space
    vc::VolTab tab;
    vc::DevBuf tab_buf;  // device copy of the table's arrays (batches only)
    std::vector<uint8_t> h_tab_stage;
    vc::Bases bases;
    vc::DevBuf bases_buf;
    vc::DevBuf occ;  // uint8, all voxels of all volumes
    // an octree (.sof) volume: its mixed leaves give the sites (vc_set_volume_sof)
    bool sites_from_octree = false;
    double vox_to_model[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};  // column-major, of the volume
    int64_t oct_n_sites = 0;            // mixed leaves of the installed octree
    vc::DevBuf oct_leaves;              // those leaves (packed x, y, z) in stream order
    vc::DevBuf oct_stream, oct_cells, oct_nodes;  // decode scratch: the stream; corner byte per cell; node lists
    // sites
    int64_t n_sites = -1;
    vc::DevBuf site_xyz;    // float3 per site
    vc::DevBuf site_count;  // int32 per-word new-corner counts, then offsets
    vc::DevBuf site_bits;   // uint32 per 32-voxel word of a z-row: packed occupancy
    vc::DevBuf site_id_lat; // int32 per lattice point: site id or -1
    // feature transform
    bool ft_valid = false;
    vc::DevBuf ft_d2, ft_id;  // int32 per lattice point
    vc::DevBuf ft_tmp;        // int64 per lattice point (separable pass scratch)
    // lattice Voronoi complex
    bool vd_valid = false;
    vc_vd_sizes vd{};
    vc::DevBuf vd_seg;                     // per 32-point lattice segment: 7 cell bit planes (32 bytes)
    vc::DevBuf vd_voff, vd_eoff, vd_foff;  // int32 per segment: cell counts, then first cell ids
    vc::DevBuf vd_tri_face, vd_face_sites, vd_lam;
    bool vd_aux_meas = false;  // vm, em, fm, tri_face, face_sites of the lattice complex written
    bool vd_aux_topo = false;  // tri_edges and the V->E / E->F lists of the lattice complex written
    bool vd_geom = false;      // vts / edges / tris of the lattice complex written (on demand after the timed path)
    bool vd_thr_valid = false; // bases.thr holds the volumes' thinning thresholds of this complex
    vc::DevBuf vd_radius;             // float per vertex of the lattice complex
    vc::DevBuf vd_vlat;               // uint32 per vertex: its lattice point within its volume (timed path)
    vc::DevBuf vd_fpass;              // uint4 per segment: faces whose lambda is below the threshold (timed path)
    std::vector<float> vol_inside;  // inside-part size per volume
    bool cc_batched = false;        // the complex is the lattice complex of a batch of > 1 volumes
    // cell complex (finalized, CSR)
    bool cc_valid = false;
    bool cc_finalized = false;
    int64_t nv = 0, ne_in = 0, ne = 0, nt = 0;
    vc::DevBuf vts;        // float3 [nv]
    vc::DevBuf edges_in;   // int2 [ne_in]
    vc::DevBuf edges;      // int2 [ne] finalized
    vc::DevBuf tris;       // int3 [nt]
    vc::DevBuf tri_edges;  // int3 [nt]
    vc::DevBuf ve_off, ve_ids, ef_off, ef_ids;
    vc::DevBuf hash_keys, hash_pos, hash_id, side_slot;  // finalize hash table
    // measures
    bool meas_valid = false;
    vc::DevBuf vm, em, fm;
    // thinning state
    bool thin_valid = false;
    vc_thin_stats thin_stats{};
    vc::DevBuf face_rec, edge_rec, vert_rec;  // per-cell thinning records (16, 32, 16 bytes)
    // generation 0 of the thinning queue, written with the records: per edge
    // the face of its FE pair, then per vertex the edge of its EV pair, -1
    // where the cell starts no pair (ne + nv int32)
    vc::DevBuf thin_g0;
    bool records_fresh = false;               // records already hold this complex in reset state
    bool records_thr_folded = false;          // ... with the per-volume thresholds folded in (threshold 0)
    vc::DevBuf q0, q1, child, cells, blk_cnt, thr;
    vc::DevBuf keep_v, keep_e, keep_f, removed_e;  // uint8 survivor flags of the last thinning
    // the same survivor flags as 32-bit words, vertices | edges | faces, and
    // per word its count of survivors (then, scanned, the survivors before it)
    vc::DevBuf keep_bits, keep_wv, keep_we, keep_wf;
    vc::DevBuf trace;           // optional per-generation trace of the thinning kernel
    int trace_cap = 0, trace_gens = 0;
    int thin_blocks_per_sm = 0;  // 0 = library default
    int thin_threads = 0;        // threads per block of the thinning kernel (0 = library default)
    int thin_items = 1;          // items per thread and piece in the thinning's phase A (1 or 2)
    bool ft_force_wide = false;  // feature transform: 64-bit arithmetic at every size
    int ft_ring = 16;            // feature transform: envelope stack entries in shared memory per line
    vc::DevBuf ft_far;           // feature transform: tiles the window kernel left to the envelope kernel
    int ft_method = 2;           // feature transform: VC_FT_ENVELOPE, VC_FT_WINDOW or VC_FT_AUTO (default)
    std::mutex* thin_lock = nullptr;  // shared by contexts whose thinning kernels must not overlap
    // failure injection (host side; the kernels only see ordinary inputs)
    unsigned long long spin_limit = 1ull << 26;  // polls before a grid barrier gives up (VC_ERR_TIMEOUT)
    int64_t thin_qcap = 0;          // > 0: the thinning queue's capacity (items per generation)
    uint32_t thin_pos0 = 0;         // queue position of the thinning's first item
    int64_t fail_alloc_after = -1;  // >= 0: that many more device allocations succeed, the next fails
    int64_t ref_bias_vertex = -1;   // >= 0: this vertex's thinning count is raised by ref_bias after
    int ref_bias = 0;               //   its record is built (a broken reference count)
    // remaining complex
    bool rem_valid = false;
    vc_rem_sizes rem{};
    vc::DevBuf rem_vts, rem_edges, rem_tris;
    vc::DevBuf uf_parent, euler_tmp;
    std::vector<int64_t> h_rem_bases;         // batches: remaining V / E / T starts, nvol + 1 each
    std::vector<vc_euler_info> vol_euler;     // per volume, from the last vc_euler_remaining

    // instrumentation: kernels launched, and optional CUDA-event timing of
    // named regions on the context stream (resolved at the next sync)
    int64_t launches = 0;
    bool timing = false;
    struct PendingTimer {
        std::string name;
        cudaEvent_t a, b;
    };
    std::vector<PendingTimer> pending;
    std::vector<cudaEvent_t> event_pool;
    std::map<std::string, std::pair<double, int64_t>> timers;  // name -> (ms, count)
};

namespace vc {

// Record a CUDA error into the context and map it to a status.
int cuda_fail(vc_ctx* c, cudaError_t e, const char* what);
#define VC_CUDA(ctx, call)                                   \
    do {                                                     \
        cudaError_t _e = (call);                             \
        if (_e != cudaSuccess) return vc::cuda_fail((ctx), _e, #call); \
    } while (0)
#define VC_TRY(expr)                 \
    do {                             \
        int _s = (expr);             \
        if (_s != VC_OK) return _s;  \
    } while (0)

int ensure_ctx(vc_ctx* c, DevBuf& b, size_t bytes);
template <class T>
inline int ensure_n(vc_ctx* c, DevBuf& b, int64_t n) {
    return ensure_ctx(c, b, (size_t)(n > 0 ? n : 1) * sizeof(T));
}
// The context's edge records for ne edges (heads, then counts), allocated.
inline int ensure_edge_recs(vc_ctx* c, DevBuf& b, int64_t ne, EdgeRecs* out) {
    VC_TRY(ensure_n<EdgeHead>(c, b, 2 * ne));
    out->h = ptr<EdgeHead>(b);
    out->n = reinterpret_cast<EdgeCnt*>(out->h + ne);
    return VC_OK;
}
// Synchronize the stream and fold the device error word into a status.
int sync_check(vc_ctx* c);
// Copy n bytes between a context buffer and a caller pointer.
int copy_out(vc_ctx* c, void* dst, const void* src, size_t bytes, int mem);
int copy_in(vc_ctx* c, void* dst, const void* src, size_t bytes, int mem);
int* dev_err(vc_ctx* c);
// Describe the context's volumes (dims: 3 ints per volume) and size the
// per-volume base arrays.
int set_volume_table(vc_ctx* c, int nvol, const int32_t* dims);
// The lattice complex's vertex / edge / triangle arrays, written on demand.
int ensure_vd_geometry(vc_ctx* c);
// The entry of a base array (nvol + 1 ascending starts) whose range holds x.
// Rank of cell x among the kept cells of its kind: the kept cells are bit
// words (bit x & 31 of word x >> 5) and base[w] is the number kept before
// word w (an exclusive scan of the words' population counts).
// Survivors of a thinning as bit words (vertices | edges | faces) with
// scanned per-word counts: a survivor's output position is its kept_rank.
struct Kept {
    const uint32_t* bv;  // vertex words
    const uint32_t* be;  // edge words
    const uint32_t* bf;  // face words
    const int32_t* pv;
    const int32_t* pe;
    const int32_t* pf;
};
__device__ __forceinline__ int32_t kept_rank(const uint32_t* __restrict__ bits, const int32_t* __restrict__ base,
                                             int64_t x) {
    const int64_t w = x >> 5;
    return __ldg(base + w) + __popc(__ldg(bits + w) & ((1u << (x & 31)) - 1u));
}

__device__ __forceinline__ int find_base(const int64_t* base, int nvol, int64_t x) {
    if (nvol <= 1) return 0;
    int lo = 0, hi = nvol - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (__ldg(base + mid) <= x) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}
// Fill one base array from an exclusive scan over a space: entry b = the scan
// at volume b's start, entry nvol = the total (device, from total_dev).
int fill_bases(vc_ctx* c, int base, int space, const int32_t* scan, const int64_t* total_dev);
// Count kernel launches issued by the library on this context.
inline void launched(vc_ctx* c, int n = 1) { c->launches += n; }
// Resolve finished timing events into c->timers (called after a sync).
void resolve_timers(vc_ctx* c);
// RAII timing of a named region on the context stream (no-op when disabled).
struct Region {
    vc_ctx* c;
    const char* name;
    cudaEvent_t a = nullptr;
    Region(vc_ctx* ctx, const char* n);
    ~Region();
};
// Exclusive scan helpers (device-wide), results and optional total on device.
// out may alias in.  total_dev may be null.
int scan_exclusive_i32(vc_ctx* c, const int32_t* in, int32_t* out, int64_t n, int64_t* total_dev);
int scan_exclusive_i64(vc_ctx* c, const int64_t* in, int64_t* out, int64_t n, int64_t* total_dev);
// Read one int64 from device memory (synchronizes).
int read_i64(vc_ctx* c, const int64_t* src, int64_t* out);

// ---------------------------------------------------------------------------
// Warp / block scans (inclusive), blockDim.x a multiple of 32, <= 1024.
template <class T>
__device__ __forceinline__ T warp_inclusive_sum(T v) {
    const unsigned lane = threadIdx.x & 31u;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        T n = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= (unsigned)o) v += n;
    }
    return v;
}

// Block-wide exclusive sum; returns the exclusive prefix of `v` and writes
// the block total to *total.  blockDim.x must be a multiple of 32; `smem`
// must hold 33 Ts.  All threads of the block call it.
template <class T>
__device__ __forceinline__ T block_exclusive_sum(T v, T* smem, T* total) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    T inc = warp_inclusive_sum(v);
    if (lane == 31) smem[wid] = inc;
    __syncthreads();
    if (wid == 0) {
        T s = lane < nw ? smem[lane] : T(0);
        T si = warp_inclusive_sum(s);
        if (lane < nw) smem[lane] = si - s;
        if (lane == 31) smem[32] = si;
    }
    __syncthreads();
    T res = smem[wid] + inc - v;
    *total = smem[32];
    __syncthreads();
    return res;
}

// ---------------------------------------------------------------------------
// Bounded grid barrier for cooperative launches.  `bar` points to two
// unsigned words {arrived, generation}.  Every block calls it with all its
// threads.  A block that waits longer than `limit` polls records
// VC_ERR_TIMEOUT in *err and proceeds.  Returns, the same for every thread of
// the block, whether *err was set when the block left (thread 0 reads it once
// and shares it), so callers leave their loop together: no block waits
// forever, and no thread of a block goes on while another leaves.
__device__ __forceinline__ bool grid_barrier(unsigned* bar, int* err, unsigned long long limit) {
    __shared__ int s_stop;
    __syncthreads();
    if (threadIdx.x == 0) {
        volatile unsigned* vgen = bar + 1;
        unsigned my_gen = *vgen;
        __threadfence();
        unsigned arrived = atomicAdd(bar, 1u);
        if (arrived == gridDim.x - 1) {
            atomicExch(bar, 0u);
            __threadfence();
            atomicAdd(bar + 1, 1u);
        } else {
            unsigned long long spins = 0;
            while (*vgen == my_gen) {
                if (++spins > limit) {
                    set_error(err, VC_ERR_TIMEOUT);
                    break;
                }
                __nanosleep(64);
            }
        }
        __threadfence();
        s_stop = *((volatile int*)err) != 0;
    }
    __syncthreads();
    return s_stop != 0;
}

__device__ __forceinline__ int ld_cg(const int* p) { return __ldcg(p); }

inline int div_up(int64_t a, int64_t b) { return (int)((a + b - 1) / b); }

}  // namespace vc
