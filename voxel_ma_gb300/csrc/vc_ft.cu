// Exact feature transform of the boundary-corner sites on the corner lattice.
//
// The reference has no distance transform: its nearest-boundary relation is
// the pair of Voronoi sites of each face (src/voroinfo.cpp:185-231).  This
// file computes, for every corner-lattice point, the exact squared distance
// d2 (voxel units) to the nearest site and that site's index, breaking ties
// toward the lowest index.  Three separable passes carry the packed pair
// (partial d2 << 32 | id), whose integer order is the lexicographic
// (distance, index) order, so every pass keeps exactly the lexicographic
// minimum:
//   pass 1 (along z, contiguous rows): nearest site in the row, one warp per
//          row: the row's site ids are staged in shared memory, then a
//          forward max-scan and a backward min-scan of site positions;
//   pass 2 (along y) and pass 3 (along x): the minimum over q of the
//          packed ((x - q)^2 + g(q), id(q)) at every point x of a line.
//          Window kernel first: tiles of 32 consecutive lines are staged
//          in shared memory 64 points at a time, and each point scans
//          outward from itself until r^2 exceeds its best distance (a
//          candidate r away is worth at least r^2, so none further can win
//          or tie); a tile with a point whose scan would pass 64 is left
//          to the envelope kernel: lower
//          envelope of the parabolas (x - q)^2 + g(q), one thread per line,
//          with integer crossing thresholds that include the index
//          tie-break (the smallest x at which the later parabola wins is
//          computed exactly), so the envelope is the lexicographic minimum
//          at every integer x.  Both give that minimum exactly, so a line's
//          result does not depend on which kernel wrote it.
//
// Memory behaviour: pass 1 stages each row in shared memory and writes it
// with streaming stores.  In the window kernel a warp's lanes are the tile's
// 32 lines at one point, so every global load and store is one contiguous
// warp access and the shared-memory scans are free of bank conflicts.  In
// the envelope kernel consecutive lanes own consecutive lines, so the
// candidate loads of a step are one contiguous warp access, issued a chunk
// ahead of their use; each point is written as soon as it is final, so the
// live stack of a line stays a few entries deep and sits in shared memory
// (vc_ft_line.cuh).
#include "vc_internal.cuh"
#include "vc_ft_line.cuh"

namespace vc {
namespace {

constexpr int64_t kInf = kFtInf;
constexpr int kEnvThreads = 256;
constexpr int kPrefetch = 8;

__device__ __forceinline__ int64_t pack(int64_t g, int32_t id) { return ft_pack(g, id); }

// Pass 1: one warp per lattice row along z (volume b, a, b'), NC = Z_b + 1
// points; `ncmax` is the longest row of the batch.  Per warp the shared
// memory holds the row's site ids and the forward scan (2 * ncmax int32).
__global__ void __launch_bounds__(256) ft_rows_kernel(const int32_t* __restrict__ site_id, int64_t* __restrict__ out,
                                                      VolTab T, int ncmax) {
    extern __shared__ int32_t rows_sm[];
    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    int32_t* ids = rows_sm + (int64_t)wib * 2 * ncmax;
    int32_t* left = ids + ncmax;
    const int64_t warps_total = (int64_t)gridDim.x * (blockDim.x >> 5);
    const int64_t nrows = T.total(kLRow);
    for (int64_t row = (int64_t)blockIdx.x * (blockDim.x >> 5) + wib; row < nrows; row += warps_total) {
        const int bv = T.find(kLRow, row);
        const int NC = T.dim(bv).z + 1;
        const int64_t rbase = T.start(kLat, bv) + (row - T.start(kLRow, bv)) * NC;
        const int32_t* in = site_id + rbase;
        // stage the row (independent loads, all in flight together)
#pragma unroll 4
        for (int c = lane; c < NC; c += 32) ids[c] = __ldcs(in + c);
        __syncwarp();
        // forward: position of the latest site at or before c (-1: none)
        int carry = -1;
        for (int c0 = 0; c0 < NC; c0 += 32) {
            const int c = c0 + lane;
            int v = (c < NC && ids[c] >= 0) ? c : -1;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int n = __shfl_up_sync(0xffffffffu, v, o);
                if (lane >= o) v = max(v, n);
            }
            v = max(v, carry);
            if (c < NC) left[c] = v;
            carry = __shfl_sync(0xffffffffu, v, 31);
        }
        __syncwarp();
        // backward: position of the earliest site at or after c; the nearer
        // of the two (lower index on a tie) is the row's nearest site
        int rcarry = INT32_MAX;
        const int nchunks = (NC + 31) / 32;
        for (int ch = nchunks - 1; ch >= 0; --ch) {
            const int c = ch * 32 + lane;
            int v = (c < NC && ids[c] >= 0) ? c : INT32_MAX;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int n = __shfl_down_sync(0xffffffffu, v, o);
                if (lane + o < 32) v = min(v, n);
            }
            v = min(v, rcarry);
            rcarry = __shfl_sync(0xffffffffu, v, 0);
            if (c < NC) {
                int64_t best = kInf;
                const int l = left[c];
                if (l >= 0) {
                    const int64_t d = c - l;
                    best = pack(d * d, ids[l]);
                }
                if (v != INT32_MAX) {
                    const int64_t d = v - c;
                    best = min(best, pack(d * d, ids[v]));
                }
                __stcs(out + rbase + c, best);
            }
        }
        __syncwarp();
    }
}

// Geometry of lattice line gl of pass PASS: its length, first point and stride.
template <int PASS>
__device__ __forceinline__ void line_geom(const VolTab& T, int64_t gl, int& L, int64_t& base, int64_t& stride) {
    constexpr int kSpace = PASS == 2 ? kYLine : kXLine;
    const int bv = T.find(kSpace, gl);
    const int4 dm = T.dim(bv);
    const int64_t NB = dm.y + 1, NC = dm.z + 1;
    const int64_t l = gl - T.start(kSpace, bv);
    L = PASS == 2 ? (int)NB : dm.x + 1;
    stride = PASS == 2 ? NC : NB * NC;
    base = T.start(kLat, bv) + (PASS == 2 ? (l / NC) * NB * NC + (l % NC) : l);
}

// Passes 2 and 3, window kernel (every axis below 2048).  A tile is
// kWinLines consecutive lines (consecutive addresses within a volume); its
// points are staged kWinChunk at a time in a ring of four chunks per line,
// so that while chunk k is computed, chunks k - 1 and k + 1 (every candidate
// within kWinChunk of it) are in shared memory.  Positions outside the line
// hold kWinNone, a packed value above every distance that stays exact when a
// squared offset is added, so the scans need no bounds checks.  Warp w
// computes points w, w + kWinWarps, ... of chunk k, lane j for line j: every global
// access of a warp is contiguous and every shared-memory access is free of
// bank conflicts.  The first kWinNear offsets on both sides are evaluated for
// every point; a point whose best is still (kWinNear + 1)^2 or more goes to its warp's
// queue, and the queue is scanned further outward 32 points at a time (one
// point per lane), so the long scans of a few points do not hold up the
// other lanes.  A tile is left to the envelope kernel (all its lines, which
// keeps that kernel's loads coalesced) as soon as one of its points needs an
// offset beyond kWinFar.  The envelope kernel's cost per point is about
// constant while a scan grows with the distance, so on sparse inputs (large
// distances) the envelope method is the faster one; vc_autotune times both.
constexpr int kWinLines = 32;
constexpr int kWinChunk = 64;
constexpr int kWinRing = 4 * kWinChunk;   // power of two: ring index = position & (kWinRing - 1)
constexpr int kWinPitch = kWinRing + 1;   // odd pitch: line j's column starts at bank 2j
constexpr int kWinThreads = 512;  // 16 warps (8 and 32 measured slower at 512^3)
constexpr int64_t kWinNone = ((int64_t)1 << 62) | 0xffffffffLL;  // distance 2^30, index -1
constexpr int kWinWarps = kWinThreads / 32;
constexpr int kWinQueue = 64;  // continuing points queued per warp
// offsets evaluated for every point, per pass: y 7, x 5 (the x pass's
// distances are smaller; measured at 512^3 against 6 and 6: y 1.343 -> 1.330
// ms, x 1.164 -> 1.161 ms; 4 for x or 5 for y were slower)
template <int PASS>
__host__ __device__ constexpr int win_near() {
    return PASS == 2 ? 7 : 5;
}
constexpr int kWinFar = 64;    // largest offset scanned (the ring holds +-kWinChunk)
// VC_FT_AUTO takes the window method when there is at least one site per
// kWinDensity lattice points: random fields at level 0 have 0.14-0.16 sites
// per point, meshes and sphere or box unions at these sizes 0.004-0.07.
constexpr double kWinDensity = 10.0;
constexpr size_t kWinSmem = (size_t)kWinLines * kWinPitch * sizeof(int64_t) +
                            (size_t)kWinWarps * kWinQueue * (sizeof(int64_t) + sizeof(int32_t));

template <int PASS>
__global__ void __launch_bounds__(kWinThreads) ft_window_kernel(const int64_t* __restrict__ in,
                                                                int64_t* __restrict__ out, int32_t* __restrict__ d2o,
                                                                int32_t* __restrict__ ido, VolTab T,
                                                                int32_t* __restrict__ far_tiles,
                                                                int* __restrict__ nfar) {
    constexpr bool FINAL = PASS == 3;
    constexpr int kWinNear = win_near<PASS>();
    constexpr int kSpace = PASS == 2 ? kYLine : kXLine;
    constexpr int kRows = kWinThreads / kWinLines;  // points of a chunk per warp row
    constexpr int kMask = kWinRing - 1;
    extern __shared__ int64_t win_sm[];  // [kWinLines][kWinPitch], then the warps' queues
    __shared__ int64_t s_base[kWinLines], s_stride[kWinLines];
    __shared__ int s_len[kWinLines], s_lmax, s_far;
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
    int64_t* qbest = win_sm + kWinLines * kWinPitch + w * kWinQueue;                           // [kWinQueue]
    int32_t* qpt = reinterpret_cast<int32_t*>(win_sm + kWinLines * kWinPitch + kWinWarps * kWinQueue) +
                   w * kWinQueue;                                                              // q << 5 | line
    const int64_t nlines = T.total(kSpace);
    const int64_t ntiles = (nlines + kWinLines - 1) / kWinLines;
    // the result of the point at lattice index o
    auto emit_at = [&](int64_t o, int64_t best) {
        const bool none = (best >> 32) >= ((int64_t)1 << 30);
        if (FINAL) {
            __stcs(d2o + o, none ? INT32_MAX : (int32_t)ft_g(best));
            __stcs(ido + o, none ? -1 : ft_id(best));
        } else {
            __stcs(out + o, none ? kFtInf : best);
        }
    };
    // continue a queued point from offset kWinNear + 1 on (one per lane, n lanes)
    auto drain = [&](int n) {
        if (lane < n) {
            const int32_t m = qpt[lane];
            const int j = m & 31, q = m >> 5;
            const int64_t* svj = win_sm + j * kWinPitch;
            const int qm = q & kMask;
            int64_t best = qbest[lane];
            bool far = false;
            for (int r = kWinNear + 1;; ++r) {
                const int64_t r2 = (int64_t)r * r;
                if (r2 > (best >> 32)) break;  // a candidate r away is worth at least r^2
                if (r > kWinFar) {
                    far = true;
                    break;
                }
                // both candidates r away get the same r^2: one add for the pair
                best = min(best, min(svj[(qm - r) & kMask], svj[(qm + r) & kMask]) + (r2 << 32));
            }
            if (far) s_far = 1;
            else emit_at(s_base[j] + (int64_t)q * s_stride[j], best);
        }
        __syncwarp();
    };
    for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        __syncthreads();  // every thread is done with the previous tile's flags
        if (t == 0) {
            s_lmax = 0;
            s_far = 0;
        }
        if (t < kWinLines) {
            const int64_t gl = tile * kWinLines + t;
            int L = 0;
            int64_t base = 0, stride = 0;
            if (gl < nlines) line_geom<PASS>(T, gl, L, base, stride);
            s_len[t] = L;
            s_base[t] = base;
            s_stride[t] = stride;
        }
        __syncthreads();
        if (t < kWinLines) atomicMax(&s_lmax, s_len[t]);
        __syncthreads();
        const int nch = (s_lmax + kWinChunk - 1) / kWinChunk;
        // this lane's line
        const int L = s_len[lane];
        const int64_t base = s_base[lane], stride = s_stride[lane];
        int64_t* sv = win_sm + lane * kWinPitch;
        // chunk k is loaded into registers (fetch) while chunk k - 2 is
        // computed, and stored into its ring slot (put) after that
        const int64_t rstep = (int64_t)kRows * stride;  // lattice step between a warp's points
        int64_t pre[kWinChunk / kRows];
        auto fetch = [&](int k) {
            const int p0 = k * kWinChunk + w;
            const int64_t* src = in + base + (int64_t)p0 * stride;
#pragma unroll
            for (int i = 0; i < kWinChunk / kRows; ++i, src += rstep) {
                const int p = p0 + i * kRows;
                pre[i] = (p >= 0 && p < L) ? __ldcs(src) : kFtInf;
            }
        };
        auto put = [&](int k) {
#pragma unroll
            for (int i = 0; i < kWinChunk / kRows; ++i) {
                const int p = k * kWinChunk + w + i * kRows;
                sv[p & kMask] = pre[i] == kFtInf ? kWinNone : pre[i];
            }
        };
        fetch(-1);  // the positions before the line: nothing
        put(-1);
        fetch(0);
        put(0);
        fetch(1);
        put(1);
        bool give_up = false;
        for (int k = 0; k < nch; ++k) {
            fetch(k + 2);  // in flight while chunk k is computed
            __syncthreads();
            int qn = 0;  // queued points of this warp (warp-uniform)
            int64_t o = base + (int64_t)(k * kWinChunk + w) * stride;
#pragma unroll 1
            for (int i = 0; i < kWinChunk / kRows; ++i, o += rstep) {
                const int q = k * kWinChunk + w + i * kRows;  // the same for the whole warp
                const bool active = q < L;
                const int qm = q & kMask;
                int64_t best;
                if (qm >= kWinNear && qm <= kMask - kWinNear) {  // no wrap around the ring
                    const int64_t* c = sv + qm;
                    best = c[0];
#pragma unroll
                    for (int r = 1; r <= kWinNear; ++r) best = min(best, min(c[-r], c[r]) + ((int64_t)(r * r) << 32));
                } else {
                    best = sv[qm];
#pragma unroll
                    for (int r = 1; r <= kWinNear; ++r)
                        best = min(best, min(sv[(qm - r) & kMask], sv[(qm + r) & kMask]) + ((int64_t)(r * r) << 32));
                }
                const bool cont = active && (best >> 32) >= (kWinNear + 1) * (kWinNear + 1);
                if (active && !cont) emit_at(o, best);
                const unsigned mk = __ballot_sync(0xffffffffu, cont);
                if (cont) {
                    const int pos = qn + __popc(mk & ((1u << lane) - 1u));
                    qbest[pos] = best;
                    qpt[pos] = (q << 5) | lane;
                }
                qn += __popc(mk);
                __syncwarp();
                if (qn >= 32) {
                    drain(32);
                    // move the rest to the front
                    int64_t b2 = 0;
                    int32_t m2 = 0;
                    if (lane < qn - 32) {
                        b2 = qbest[32 + lane];
                        m2 = qpt[32 + lane];
                    }
                    __syncwarp();
                    if (lane < qn - 32) {
                        qbest[lane] = b2;
                        qpt[lane] = m2;
                    }
                    qn -= 32;
                    __syncwarp();
                }
            }
            drain(qn);
            __syncthreads();
            // the same decision in every thread (flags read after the barrier)
            give_up = s_far != 0;
            if (give_up) break;
            put(k + 2);  // the slot of chunk k - 2
        }
        // the envelope kernel does the whole tile
        if (give_up && t == 0) far_tiles[atomicAdd(nfar, 1)] = (int32_t)tile;
    }
}

// Passes 2 and 3: lower envelope along the lattice lines of every volume:
// PASS 2 along y (local line (a, c), L = Y+1 points, stride Z+1), PASS 3
// along x (local line (b, c), L = X+1 points, stride (Y+1)(Z+1)), one
// thread per line (ft_envelope_line).  Consecutive lines of a volume are
// consecutive addresses, so the candidate loads of a step are one coalesced
// warp access.  The ring of each line is a column of shared memory (slot j
// of thread t at j * blockDim + t: no bank conflicts); spilled entry k of
// local line l of volume b goes to gmeta / gval at lattice start of b +
// k * (lines of b) + l.
template <int PASS, int RING, class I>
__global__ void __launch_bounds__(kEnvThreads) ft_envelope_kernel(const int64_t* __restrict__ in,
                                                                  int64_t* __restrict__ out, int32_t* __restrict__ d2o,
                                                                  int32_t* __restrict__ ido,
                                                                  int32_t* __restrict__ gmeta,
                                                                  int64_t* __restrict__ gval, VolTab T,
                                                                  const int32_t* __restrict__ list,
                                                                  const int* __restrict__ list_len) {
    constexpr bool FINAL = PASS == 3;
    constexpr int kSpace = PASS == 2 ? kYLine : kXLine;
    extern __shared__ int64_t env_sm[];
    int64_t* s_val = env_sm;                                                    // [RING][kEnvThreads]
    int32_t* s_meta = reinterpret_cast<int32_t*>(env_sm + RING * kEnvThreads);  // [RING][kEnvThreads]
    const int t = threadIdx.x;
    // every line, or the lines of the tiles of a list (those the window
    // kernel left: kWinLines consecutive lines each)
    const int64_t all = T.total(kSpace);
    const int64_t nlines = list ? (int64_t)*list_len * kWinLines : all;
    for (int64_t li = (int64_t)blockIdx.x * blockDim.x + t; li < nlines; li += (int64_t)gridDim.x * blockDim.x) {
        const int64_t gl = list ? (int64_t)list[li / kWinLines] * kWinLines + li % kWinLines : li;
        if (gl >= all) continue;
        const int bv = T.find(kSpace, gl);
        const int4 dm = T.dim(bv);
        const int64_t NB = dm.y + 1, NC = dm.z + 1;
        const int64_t lat0 = T.start(kLat, bv);
        const int64_t l = gl - T.start(kSpace, bv);
        const int L = PASS == 2 ? (int)NB : dm.x + 1;
        const int64_t stride = PASS == 2 ? NC : NB * NC;
        const int64_t nl = PASS == 2 ? (int64_t)(dm.x + 1) * NC : NB * NC;
        const int64_t base = lat0 + (PASS == 2 ? (l / NC) * NB * NC + (l % NC) : l);
        const int64_t* src = in + base;
        auto load = [&](int q) -> int64_t { return __ldcs(src + (int64_t)q * stride); };
        auto emit = [&](int x, int64_t v) {
            const int64_t o = base + (int64_t)x * stride;
            if (FINAL) {
                __stcs(d2o + o, (int32_t)ft_g(v));
                __stcs(ido + o, ft_id(v));
            } else {
                __stcs(out + o, v);
            }
        };
        ft_envelope_line<I, RING, kPrefetch>(L, load, emit, s_meta + t, s_val + t, kEnvThreads, gmeta + lat0 + l,
                                          gval + lat0 + l, nl);
    }
}

template <int RING>
constexpr size_t env_smem() {
    return (size_t)RING * kEnvThreads * (sizeof(int64_t) + sizeof(int32_t));
}

template <int PASS, class I, int RING>
int launch_envelope_t(vc_ctx* c, const int64_t* in, int64_t* out, int32_t* d2o, int32_t* ido, int32_t* gmeta,
                      int64_t* gval, int64_t nlines, const int32_t* list, const int* list_len) {
    auto kern = ft_envelope_kernel<PASS, RING, I>;
    constexpr size_t smem = env_smem<RING>();
    VC_CUDA(c, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int per_sm = 0;
    VC_CUDA(c, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kEnvThreads, smem));
    per_sm = std::max(per_sm, 1);
    const int blocks = (int)std::max<int64_t>(
        1, std::min<int64_t>((nlines + kEnvThreads - 1) / kEnvThreads, (int64_t)c->num_sms * per_sm));
    kern<<<blocks, kEnvThreads, smem, c->stream>>>(in, out, d2o, ido, gmeta, gval, c->tab, list, list_len);
    launched(c);
    VC_CUDA(c, cudaGetLastError());
    return VC_OK;
}

// int32 arithmetic when every lattice axis of the batch is below 2048; the
// ring (stack entries kept in shared memory per line) is the context's
// tuned size (4, 8 or 16; 16 by default)
template <int PASS>
int launch_envelope(vc_ctx* c, bool small, const int64_t* in, int64_t* out, int32_t* d2o, int32_t* ido,
                    int32_t* gmeta, int64_t* gval, int64_t nlines, const int32_t* list = nullptr,
                    const int* list_len = nullptr) {
    if (!small) return launch_envelope_t<PASS, int64_t, 8>(c, in, out, d2o, ido, gmeta, gval, nlines, list, list_len);
    if (c->ft_ring == 4)
        return launch_envelope_t<PASS, int32_t, 4>(c, in, out, d2o, ido, gmeta, gval, nlines, list, list_len);
    if (c->ft_ring == 8)
        return launch_envelope_t<PASS, int32_t, 8>(c, in, out, d2o, ido, gmeta, gval, nlines, list, list_len);
    return launch_envelope_t<PASS, int32_t, 16>(c, in, out, d2o, ido, gmeta, gval, nlines, list, list_len);
}

// A pass with 32-bit arithmetic: the window kernel over every tile, then the
// envelope kernel over the tiles it left (their count stays on the device;
// the envelope launch walks the list up to it).
template <int PASS>
int launch_window(vc_ctx* c, const int64_t* in, int64_t* out, int32_t* d2o, int32_t* ido, int32_t* gmeta,
                  int64_t* gval, int64_t nlines, int32_t* hard, int* nhard) {
    auto kern = ft_window_kernel<PASS>;
    VC_CUDA(c, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kWinSmem));
    int per_sm = 0;
    VC_CUDA(c, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kWinThreads, kWinSmem));
    per_sm = std::max(per_sm, 1);
    const int64_t ntiles = (nlines + kWinLines - 1) / kWinLines;
    const int blocks = (int)std::max<int64_t>(1, std::min<int64_t>(ntiles, (int64_t)c->num_sms * per_sm));
    {
        Region r(c, PASS == 2 ? "ft_window_y" : "ft_window_x");
        kern<<<blocks, kWinThreads, kWinSmem, c->stream>>>(in, out, d2o, ido, c->tab, hard, nhard);
        launched(c);
        VC_CUDA(c, cudaGetLastError());
    }
    Region r(c, PASS == 2 ? "ft_far_y" : "ft_far_x");
    return launch_envelope<PASS>(c, true, in, out, d2o, ido, gmeta, gval, nlines, hard, nhard);
}

}  // namespace

int run_ft(vc_ctx* c) {
    if (c->n_sites < 0) return VC_ERR_STATE;
    const int nvol = c->nvol;
    int ncmax = 0, nmax = 0;
    for (int b = 0; b < nvol; ++b) {
        const int64_t NA = c->h_dims[3 * b] + 1, NB = c->h_dims[3 * b + 1] + 1, NC = c->h_dims[3 * b + 2] + 1;
        if (NA > 32767 || NB > 32767 || NC > 32767) return VC_ERR_ARG;
        ncmax = std::max<int>(ncmax, (int)NC);
        nmax = std::max<int>(nmax, (int)std::max(NA, std::max(NB, NC)));
    }
    const bool small = nmax <= 2048 && !c->ft_force_wide;
    const int64_t N = c->h_off[kLat][nvol];
    // the window method where the sites are dense (then the distances are a
    // few voxels): at least one site per kWinDensity lattice points
    const bool dense = (double)c->n_sites * kWinDensity >= (double)N;
    const bool win = small && (c->ft_method == VC_FT_WINDOW || (c->ft_method == VC_FT_AUTO && dense));
    VC_TRY(ensure_n<int32_t>(c, c->ft_d2, N));
    VC_TRY(ensure_n<int32_t>(c, c->ft_id, N));
    VC_TRY(ensure_n<int64_t>(c, c->ft_tmp, 3 * N));
    // tiles the window kernel leaves: [0], [1] counts of passes 2 and 3, then the list
    const int64_t nlmax = std::max(c->h_off[kYLine][nvol], c->h_off[kXLine][nvol]);
    if (win) {
        VC_TRY(ensure_n<int32_t>(c, c->ft_far, (nlmax + kWinLines - 1) / kWinLines + 2));
        VC_CUDA(c, cudaMemsetAsync(c->ft_far.p, 0, 2 * sizeof(int32_t), c->stream));
    }
    int32_t* far_cnt = win ? ptr<int32_t>(c->ft_far) : nullptr;
    int32_t* far_list = win ? far_cnt + 2 : nullptr;
    Region stage(c, "stage_ft");
    int64_t* A = ptr<int64_t>(c->ft_tmp);
    int64_t* B = A + N;
    int64_t* C = B + N;
    {
        const int warps_per_block = 8;
        const size_t smem = (size_t)warps_per_block * 2 * ncmax * sizeof(int32_t);
        if (smem > 200 * 1024) return VC_ERR_ARG;
        if (smem > 48 * 1024)
            VC_CUDA(c, cudaFuncSetAttribute(ft_rows_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        const int64_t nrows = c->h_off[kLRow][nvol];
        int blocks = (int)std::min<int64_t>((nrows + warps_per_block - 1) / warps_per_block,
                                            (int64_t)c->num_sms * 16);  // as many as fit (0.54 -> 0.46 ms against 8 per SM)
        Region r(c, "ft_rows");
        ft_rows_kernel<<<blocks, warps_per_block * 32, smem, c->stream>>>(ptr<int32_t>(c->site_id_lat), A, c->tab,
                                                                          ncmax);
        launched(c);
        VC_CUDA(c, cudaGetLastError());
    }
    {
        // pass 2 along y: stack spills go to C (values) and to the d2
        // output (positions), which pass 3 writes last
        Region r(c, "ft_envelope_y");
        if (win)
            VC_TRY(launch_window<2>(c, A, B, nullptr, nullptr, ptr<int32_t>(c->ft_d2), C, c->h_off[kYLine][nvol],
                                    far_list, far_cnt + 0));
        else
            VC_TRY(launch_envelope<2>(c, small, A, B, nullptr, nullptr, ptr<int32_t>(c->ft_d2), C,
                                      c->h_off[kYLine][nvol]));
    }
    {
        // pass 3 along x: spills go to the pass-1 buffer A (values) and to C
        // (positions), both dead by now
        Region r(c, "ft_envelope_x");
        if (win)
            VC_TRY(launch_window<3>(c, B, nullptr, ptr<int32_t>(c->ft_d2), ptr<int32_t>(c->ft_id),
                                    reinterpret_cast<int32_t*>(C), A, c->h_off[kXLine][nvol], far_list, far_cnt + 1));
        else
            VC_TRY(launch_envelope<3>(c, small, B, nullptr, ptr<int32_t>(c->ft_d2), ptr<int32_t>(c->ft_id),
                                      reinterpret_cast<int32_t*>(C), A, c->h_off[kXLine][nvol]));
    }
    c->ft_valid = true;
    return VC_OK;
}

}  // namespace vc

extern "C" int vc_set_ft_method(vc_ctx* c, int method) {
    if (!c || (method != VC_FT_ENVELOPE && method != VC_FT_WINDOW && method != VC_FT_AUTO)) return VC_ERR_ARG;
    c->ft_method = method;
    return VC_OK;
}

extern "C" int vc_debug_ft_wide(vc_ctx* c, int wide) {
    if (!c) return VC_ERR_ARG;
    c->ft_force_wide = wide != 0;
    return VC_OK;
}
