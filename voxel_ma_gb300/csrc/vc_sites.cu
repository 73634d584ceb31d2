// Boundary-corner site extraction on the GPU (replaces
// Surfacer::extractBoundaryVts, src/surfacing.cpp:223-321).
//
// The reference sweeps voxels i -> j -> k and, for each face neighbour
// (-x,+x,-y,+y,-z,+z) whose occupancy differs, appends the four shared
// corners it has not seen before.  A corner is therefore first met at the
// earliest voxel (in sweep order) of the 2x2x2 block around it that is inside
// the box and has a differing block neighbour; inside that voxel its rank is
// the first (direction, corner slot) that names it.  Each thread decides this
// per voxel from the voxel's 3x3x3 neighbourhood, so the site list comes out
// in the reference's order after one exclusive scan of per-voxel counts.
//
// The main path evaluates the rule for 32 voxels of a z-row at once
// (vc_sites_words.cuh): the occupancy is packed to one bit per voxel (a
// 512^3 volume becomes 16 MB, resident in L2), one thread per word counts
// the word's new corners, a scan of the word counts numbers the sites, and
// one thread per word writes them.  The per-voxel kernels below the word
// kernels serve the allocation-free entry point.
#include "vc_internal.cuh"
#include "vc_scan.cuh"
#include "vc_sites_words.cuh"

#include <mutex>

namespace vc {
namespace {

// Corner c of a voxel as the lattice offset {0,1}^3 from the voxel's lowest
// corner, in the reference's corner numbering (surfacing.h:74-96).
__device__ constexpr int8_t kCornerOff[8][3] = {{1, 0, 0}, {1, 1, 0}, {0, 0, 0}, {0, 1, 0},
                                        {1, 0, 1}, {1, 1, 1}, {0, 0, 1}, {0, 1, 1}};
// Face-neighbour offsets in sweep order (surfacing.h:170-179).
__constant__ int8_t kNbOff[6][3] = {{-1, 0, 0}, {1, 0, 0}, {0, -1, 0}, {0, 1, 0}, {0, 0, -1}, {0, 0, 1}};
// The four corners shared with each face neighbour, in visiting order
// (surfacing.h:182-190).
__constant__ int8_t kShared[6][4] = {{2, 3, 7, 6}, {0, 1, 5, 4}, {4, 6, 2, 0},
                                     {1, 3, 7, 5}, {0, 2, 3, 1}, {5, 7, 6, 4}};

struct Vol {
    const uint8_t* occ;
    int X, Y, Z;
    __device__ __forceinline__ int at(int i, int j, int k) const {
        if (i < 0 || j < 0 || k < 0 || i >= X || j >= Y || k >= Z) return 0;
        return occ[((int64_t)i * Y + j) * Z + k] > 0 ? 1 : 0;
    }
};

// 27-bit neighbourhood: bit (dx+1)*9 + (dy+1)*3 + (dz+1) = occupancy of
// voxel (i+dx, j+dy, k+dz); out-of-box voxels read 0.
__device__ __forceinline__ uint32_t load_nbhd(const Vol& v, int i, int j, int k) {
    uint32_t m = 0;
#pragma unroll
    for (int dx = -1; dx <= 1; ++dx)
#pragma unroll
        for (int dy = -1; dy <= 1; ++dy)
#pragma unroll
            for (int dz = -1; dz <= 1; ++dz)
                m |= (uint32_t)v.at(i + dx, j + dy, k + dz) << ((dx + 1) * 9 + (dy + 1) * 3 + (dz + 1));
    return m;
}
__device__ __forceinline__ int nb_bit(uint32_t m, int dx, int dy, int dz) {
    return (m >> ((dx + 1) * 9 + (dy + 1) * 3 + (dz + 1))) & 1;
}

// 27-bit in-box mask of the same neighbourhood.
__device__ __forceinline__ uint32_t inbox_nbhd(const Vol& v, int i, int j, int k) {
    const uint32_t xm = (i > 0 ? 1u : 0u) | 2u | (i < v.X - 1 ? 4u : 0u);
    const uint32_t ym = (j > 0 ? 1u : 0u) | 2u | (j < v.Y - 1 ? 4u : 0u);
    const uint32_t zm = (k > 0 ? 1u : 0u) | 2u | (k < v.Z - 1 ? 4u : 0u);
    uint32_t m = 0;
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int b = 0; b < 3; ++b)
            if (((xm >> a) & 1u) && ((ym >> b) & 1u)) m |= zm << (a * 9 + b * 3);
    return m;
}

// The 2x2x2 block of voxels around corner c of the voxel, as 8 bits:
// bit q = qx<<2 | qy<<1 | qz is the voxel at offset (ox-1+qx, oy-1+qy,
// oz-1+qz), i.e. neighbourhood bit (ox+qx)*9 + (oy+qy)*3 + (oz+qz).
__device__ __forceinline__ uint32_t block_bits(uint32_t m27, int ox, int oy, int oz) {
    const uint32_t t = m27 >> (ox * 9 + oy * 3 + oz);
    return (t & 3u) | ((t >> 1) & 0xCu) | ((t >> 5) & 0x30u) | ((t >> 6) & 0xC0u);
}

// Mask of the corners of voxel (i,j,k) that are first encountered there.
// Within a corner's block, the sweep meets first the in-box voxel of lowest
// (qx,qy,qz) that differs from one of its three block neighbours; the corner
// is new at (i,j,k) iff that voxel is (i,j,k) itself.
__device__ __forceinline__ uint32_t new_corner_mask(uint32_t nb, uint32_t inb) {
    uint32_t res = 0;
#pragma unroll
    for (int c = 0; c < 8; ++c) {
        const int ox = kCornerOff[c][0], oy = kCornerOff[c][1], oz = kCornerOff[c][2];
        const uint32_t P = block_bits(nb, ox, oy, oz);
        const uint32_t M = block_bits(inb, ox, oy, oz);
        const uint32_t sx = ((P >> 4) & 0x0Fu) | ((P << 4) & 0xF0u);
        const uint32_t sy = ((P >> 2) & 0x33u) | ((P << 2) & 0xCCu);
        const uint32_t sz = ((P >> 1) & 0x55u) | ((P << 1) & 0xAAu);
        const uint32_t D = ((P ^ sx) | (P ^ sy) | (P ^ sz)) & M;
        const int own = ((1 - ox) << 2) | ((1 - oy) << 1) | (1 - oz);
        if (D && (__ffs(D) - 1) == own) res |= 1u << c;
    }
    return res;
}

// One block per voxel row (volume b, x, y) of the batch, threads along z.
__global__ void sites_count_kernel(const uint8_t* __restrict__ occ, VolTab T, int32_t* __restrict__ cnt) {
    const int64_t nrows = T.total(kVRow);
    for (int64_t row = blockIdx.x; row < nrows; row += gridDim.x) {
        const int bv = T.find(kVRow, row);
        const int4 d = T.dim(bv);
        const Vol v{occ + T.start(kVox, bv), d.x, d.y, d.z};
        const int64_t r = row - T.start(kVRow, bv);
        const int i = (int)(r / v.Y), j = (int)(r - (int64_t)i * v.Y);
        int32_t* out = cnt + T.start(kVox, bv) + r * v.Z;
        for (int k = threadIdx.x; k < v.Z; k += blockDim.x) {
            const uint32_t nb = load_nbhd(v, i, j, k);
            out[k] = __popc(new_corner_mask(nb, inbox_nbhd(v, i, j, k)));
        }
    }
}

// Sites are written at their batch-wide index; volume b's sites are the
// contiguous range starting at its first site, in the reference's order.
// site_id_lat (optional) receives the batch-wide index at each site's
// lattice point.
__global__ void sites_emit_kernel(const uint8_t* __restrict__ occ, VolTab T, const int32_t* __restrict__ off,
                                  float* __restrict__ xyz, int32_t* __restrict__ site_id_lat) {
    const int64_t nrows = T.total(kVRow);
    for (int64_t row = blockIdx.x; row < nrows; row += gridDim.x) {
        const int bv = T.find(kVRow, row);
        const int4 d = T.dim(bv);
        const Vol v{occ + T.start(kVox, bv), d.x, d.y, d.z};
        const int64_t NB = v.Y + 1, NC = v.Z + 1;
        const int64_t r = row - T.start(kVRow, bv);
        const int i = (int)(r / v.Y), j = (int)(r - (int64_t)i * v.Y);
        const int32_t* offr = off + T.start(kVox, bv) + r * v.Z;
        int32_t* lat = site_id_lat ? site_id_lat + T.start(kLat, bv) : nullptr;
        for (int k = threadIdx.x; k < v.Z; k += blockDim.x) {
            const uint32_t nb = load_nbhd(v, i, j, k);
            const uint32_t mask = new_corner_mask(nb, inbox_nbhd(v, i, j, k));
            if (!mask) continue;
            int32_t o = offr[k];
            const int cur = nb_bit(nb, 0, 0, 0);
            uint32_t done = 0;
            for (int dd = 0; dd < 6; ++dd) {
                if (nb_bit(nb, kNbOff[dd][0], kNbOff[dd][1], kNbOff[dd][2]) == cur) continue;
                for (int s = 0; s < 4; ++s) {
                    const int c = kShared[dd][s];
                    if (!(mask & (1u << c)) || (done & (1u << c))) continue;
                    done |= 1u << c;
                    const int a = i + kCornerOff[c][0], b = j + kCornerOff[c][1], cc = k + kCornerOff[c][2];
                    xyz[3 * (int64_t)o + 0] = (float)a - 0.5f;
                    xyz[3 * (int64_t)o + 1] = (float)b - 0.5f;
                    xyz[3 * (int64_t)o + 2] = (float)cc - 0.5f;
                    if (lat) lat[((int64_t)a * NB + b) * NC + cc] = o;
                    ++o;
                }
            }
        }
    }
}

// Pack the occupancy: one warp per voxel row (volume b, x, y), one ballot
// per 32 voxels; bits past the row's end are 0.
__global__ void sites_pack_kernel(const uint8_t* __restrict__ occ, VolTab T, uint32_t* __restrict__ bits) {
    const int lane = threadIdx.x & 31;
    const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
    const int64_t nrows = T.total(kVRow);
    for (int64_t row = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); row < nrows; row += warps) {
        const int bv = T.find(kVRow, row);
        const int Z = T.dim(bv).z;
        const int Wz = (Z + 31) / 32;
        const int64_t r = row - T.start(kVRow, bv);
        const uint8_t* src = occ + T.start(kVox, bv) + r * Z;
        uint32_t* dst = bits + T.start(kVWord, bv) + r * Wz;
        for (int w = 0; w < Wz; ++w) {
            const int k = 32 * w + lane;
            const bool in = k < Z && __ldcs(src + k) > 0;
            const uint32_t word = __ballot_sync(0xffffffffu, in);
            if (lane == 0) dst[w] = word;
        }
    }
}

struct WordPos {
    int bv, i, j, w;
    int4 d;
};
__device__ __forceinline__ WordPos word_pos(const VolTab& T, int64_t gw) {
    WordPos p;
    p.bv = T.find(kVWord, gw);
    p.d = T.dim(p.bv);
    const uint32_t Wz = (uint32_t)((p.d.z + 31) / 32);
    const uint64_t lw = (uint64_t)(gw - T.start(kVWord, p.bv));
    const uint64_t row = lw / Wz;
    p.w = (int)(lw - row * Wz);
    p.i = (int)(row / (uint64_t)p.d.y);
    p.j = (int)(row - (uint64_t)p.i * p.d.y);
    return p;
}

// One thread per word: its count of new corners.
__global__ void __launch_bounds__(256) sites_wcount_kernel(const uint32_t* __restrict__ bits, VolTab T,
                                                           int32_t* __restrict__ cnt) {
    const int64_t n = T.total(kVWord);
    for (int64_t gw = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; gw < n; gw += (int64_t)gridDim.x * blockDim.x) {
        const WordPos p = word_pos(T, gw);
        const uint32_t Wz = (uint32_t)((p.d.z + 31) / 32);
        const uint32_t* vb = bits + T.start(kVWord, p.bv);
        auto word = [&](int ii, int jj, int ww) { return __ldg(vb + ((int64_t)ii * p.d.y + jj) * Wz + ww); };
        SiteWords r;
        site_words(word, p.i, p.j, p.w, p.d.x, p.d.y, p.d.z, r);
        cnt[gw] = site_word_count(r);
    }
}

// One thread per word: its sites at their batch-wide indices (volume b's
// sites are the contiguous range starting at its first site, in the
// reference's order) and each site's index at its lattice point.
__global__ void __launch_bounds__(256) sites_wemit_kernel(const uint32_t* __restrict__ bits, VolTab T,
                                                          const int32_t* __restrict__ off, float* __restrict__ xyz,
                                                          int32_t* __restrict__ site_id_lat) {
    const int64_t n = T.total(kVWord);
    for (int64_t gw = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; gw < n; gw += (int64_t)gridDim.x * blockDim.x) {
        const WordPos p = word_pos(T, gw);
        const uint32_t Wz = (uint32_t)((p.d.z + 31) / 32);
        const uint32_t* vb = bits + T.start(kVWord, p.bv);
        auto word = [&](int ii, int jj, int ww) { return __ldg(vb + ((int64_t)ii * p.d.y + jj) * Wz + ww); };
        SiteWords r;
        site_words(word, p.i, p.j, p.w, p.d.x, p.d.y, p.d.z, r);
        const int64_t NB = p.d.y + 1, NC = p.d.z + 1;
        int32_t* lat = site_id_lat + T.start(kLat, p.bv);
        site_word_emit(r, p.i, p.j, p.w, (int64_t)off[gw], [&](int64_t o, int a, int b, int c) {
            xyz[3 * o + 0] = (float)a - 0.5f;
            xyz[3 * o + 1] = (float)b - 0.5f;
            xyz[3 * o + 2] = (float)c - 0.5f;
            lat[((int64_t)a * NB + b) * NC + c] = (int32_t)o;
        });
    }
}

inline int row_grid(int num_sms, int64_t rows) {
    return (int)std::max<int64_t>(1, std::min<int64_t>(rows, (int64_t)num_sms * 32));
}


}  // namespace

int octree_sites(vc_ctx* c, uint32_t* bits, int32_t* cnt, int64_t nwords, int64_t* total, int64_t* n_out);

int run_sites(vc_ctx* c, int64_t* n_sites) {
    if (!c->occ.p || c->nvol <= 0) return VC_ERR_STATE;
    const int64_t nlat = c->h_off[kLat][c->nvol];
    const int64_t nrows = c->h_off[kVRow][c->nvol];
    const int64_t nwords = c->h_off[kVWord][c->nvol];
    VC_TRY(ensure_n<uint32_t>(c, c->site_bits, nwords));
    VC_TRY(ensure_n<int32_t>(c, c->site_count, nwords));
    VC_TRY(ensure_n<int32_t>(c, c->site_id_lat, nlat));
    VC_TRY(ensure_n<int64_t>(c, c->scratch2, 4));
    Region stage(c, "stage_sites");
    uint32_t* bits = ptr<uint32_t>(c->site_bits);
    int32_t* cnt = ptr<int32_t>(c->site_count);
    // as many blocks as fit (the emission at 512^3: 0.72 -> 0.56 ms against 8 per SM)
    const int wgrid = (int)std::max<int64_t>(1, std::min<int64_t>((nwords + 255) / 256, (int64_t)c->num_sms * 32));
    {
        Region r(c, "sites_count");
        sites_pack_kernel<<<(int)std::max<int64_t>(1, std::min<int64_t>((nrows + 7) / 8, (int64_t)c->num_sms * 16)),
                            256, 0, c->stream>>>(ptr<uint8_t>(c->occ), c->tab, bits);
        launched(c);
        sites_wcount_kernel<<<wgrid, 256, 0, c->stream>>>(bits, c->tab, cnt);
        launched(c);
        VC_CUDA(c, cudaGetLastError());
    }
    int64_t* total = ptr<int64_t>(c->scratch2);
    if (c->sites_from_octree) {
        // an octree volume: the sites are its mixed leaves (Surfacer's octree rule)
        int64_t n = 0;
        VC_TRY(octree_sites(c, bits, cnt, nwords, total, &n));
        c->n_sites = n;
        if (n_sites) *n_sites = n;
        return VC_OK;
    }
    VC_TRY(scan_exclusive_i32(c, cnt, cnt, nwords, total));
    VC_TRY(fill_bases(c, kBSite, kVWord, cnt, total));
    int64_t n = 0;
    VC_TRY(read_i64(c, total, &n));
    if (n > INT32_MAX) return VC_ERR_ARG;
    VC_TRY(ensure_n<float>(c, c->site_xyz, 3 * n));
    {
        Region r(c, "sites_emit");
        VC_CUDA(c, cudaMemsetAsync(c->site_id_lat.p, 0xff, (size_t)nlat * sizeof(int32_t), c->stream));
        sites_wemit_kernel<<<wgrid, 256, 0, c->stream>>>(bits, c->tab, cnt, ptr<float>(c->site_xyz),
                                                        ptr<int32_t>(c->site_id_lat));
        launched(c);
        VC_CUDA(c, cudaGetLastError());
    }
    c->n_sites = n;
    if (n_sites) *n_sites = n;
    return VC_OK;
}


// ---------------------------------------------------------------------------
// Site extraction for callers that cannot allocate device memory.
//
// Code that runs where cudaMalloc is unavailable or unwanted -- inside a
// memory-capped allocator that owns the whole device heap, a host framework
// that forbids allocation on its hot path, or a plugin that must not change
// the process's memory footprint after start-up -- still needs scratch for the
// per-voxel counts and the scan.  This variant takes that scratch from a
// fixed-size array in this file instead of allocating: every GPU that loads
// the library holds it (16 MiB of counts plus the scan's tile sums) until the
// process exits.  Volumes are limited to kNoAllocMaxVoxels voxels.
namespace {

constexpr int64_t kNoAllocMaxVoxels = (int64_t)1 << 22;  // 4,194,304 voxels, e.g. 128 x 128 x 256
constexpr int64_t kNoAllocTiles = kNoAllocMaxVoxels / kScanTile + 1;

// Device-side scratch.  In host code these names are host-side stand-ins,
// not device addresses: the host takes their addresses with
// cudaGetSymbolAddress (once per device) and passes those to the kernels.
static __device__ __align__(256) int32_t g_noalloc_counts[kNoAllocMaxVoxels];
static __device__ __align__(256) int64_t g_noalloc_tiles[kNoAllocTiles + 1];  // last entry: the total

struct NoAllocScratch {
    int32_t* counts = nullptr;
    int64_t* tiles = nullptr;
    int64_t* total = nullptr;
    int num_sms = 0;
    bool ready = false;
};
constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mu;
NoAllocScratch g_noalloc[kMaxDevices];

// Device addresses of the scratch arrays for the current device; the first
// call on a device looks them up (so that first call must not be made while
// a stream is being captured).
int noalloc_scratch(NoAllocScratch* out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
        cudaGetLastError();
        return VC_ERR_CUDA;
    }
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    NoAllocScratch& s = g_noalloc[dev];
    if (!s.ready) {
        void* counts = nullptr;
        void* tiles = nullptr;
        if (cudaGetSymbolAddress(&counts, g_noalloc_counts) != cudaSuccess ||
            cudaGetSymbolAddress(&tiles, g_noalloc_tiles) != cudaSuccess ||
            cudaDeviceGetAttribute(&s.num_sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
            cudaGetLastError();
            return VC_ERR_CUDA;
        }
        s.counts = static_cast<int32_t*>(counts);
        s.tiles = static_cast<int64_t*>(tiles);
        s.total = s.tiles + kNoAllocTiles;
        s.ready = true;
    }
    *out = s;
    return VC_OK;
}

}  // namespace
}  // namespace vc

extern "C" int vc_extract_sites_noalloc(const uint8_t* occ, int X, int Y, int Z, float* xyz, int64_t capacity,
                                        int64_t* n_sites, void* stream) {
    using namespace vc;
    if (!occ || !n_sites || X <= 0 || Y <= 0 || Z <= 0 || capacity < 0) return VC_ERR_ARG;
    const int64_t nvox = (int64_t)X * Y * Z;
    if (nvox > kNoAllocMaxVoxels) return VC_ERR_ARG;  // beyond the static scratch
    NoAllocScratch s;
    VC_TRY(noalloc_scratch(&s));
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    // a one-volume table lives entirely in the kernel arguments
    VolTab one;
    one.nvol = 1;
    one.d0 = make_int4(X, Y, Z, 0);
    // every scratch word read below is written first in this call: counts by
    // the count kernel, tile sums and the total by the scan.  Each launch's own
    // status is checked (cudaLaunchKernelEx returns it), so a launch that
    // fails leaves *n_sites untouched and no stale total is read; an error the
    // calling thread had pending before this call is neither read nor cleared.
    const int64_t tiles = (nvox + kScanTile - 1) / kScanTile;
    const unsigned row_blocks = row_grid(s.num_sms, (int64_t)X * Y);
    auto cfg = [st](unsigned grid, unsigned block) {
        cudaLaunchConfig_t c = {};
        c.gridDim = dim3(grid);
        c.blockDim = dim3(block);
        c.stream = st;
        return c;
    };
    auto failed = [](cudaError_t e) {
        if (e == cudaSuccess) return false;
        cudaGetLastError();  // this call's own launch error: do not leave it to the caller
        return true;
    };
    cudaLaunchConfig_t c_rows = cfg(row_blocks, 128), c_tiles = cfg((unsigned)tiles, kScanThreads),
                       c_one = cfg(1, 1024);
    if (failed(cudaLaunchKernelEx(&c_rows, sites_count_kernel, occ, one, s.counts)) ||
        failed(cudaLaunchKernelEx(&c_tiles, scan_tile_sums<int32_t>, (const int32_t*)s.counts, nvox, s.tiles)) ||
        failed(cudaLaunchKernelEx(&c_one, scan_sums_single, s.tiles, tiles, s.total)) ||
        failed(cudaLaunchKernelEx(&c_tiles, scan_apply<int32_t>, (const int32_t*)s.counts, s.counts, nvox,
                                  (const int64_t*)s.tiles)))
        return VC_ERR_CUDA;
    int64_t n = 0;
    if (failed(cudaMemcpyAsync(&n, s.total, sizeof(int64_t), cudaMemcpyDeviceToHost, st)) ||
        failed(cudaStreamSynchronize(st)))
        return VC_ERR_CUDA;
    *n_sites = n;
    if (n > capacity) return VC_ERR_ARG;  // *n_sites tells the caller how much room is needed
    if (n > 0) {
        if (!xyz) return VC_ERR_ARG;
        if (failed(cudaLaunchKernelEx(&c_rows, sites_emit_kernel, occ, one, (const int32_t*)s.counts, xyz,
                                      (int32_t*)nullptr)))
            return VC_ERR_CUDA;
    }
    if (failed(cudaStreamSynchronize(st))) return VC_ERR_CUDA;
    return VC_OK;
}
