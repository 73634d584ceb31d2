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
//          row, by a forward max-scan and a backward min-scan over the row;
//   pass 2 (along y) and pass 3 (along x): lower envelope of the parabolas
//          (x - q)^2 + g(q), one thread per line, with integer crossing
//          thresholds that include the index tie-break (the smallest x at
//          which the later parabola wins is computed exactly), so the
//          envelope is the lexicographic minimum at every integer x.
#include "vc_internal.cuh"

namespace vc {
namespace {

constexpr int64_t kInf = INT64_MAX;

__device__ __forceinline__ int64_t pack(int64_t g, int32_t id) { return (g << 32) | (uint32_t)id; }
__device__ __forceinline__ int64_t pk_g(int64_t p) { return p >> 32; }
__device__ __forceinline__ int32_t pk_id(int64_t p) { return (int32_t)(uint32_t)(p & 0xffffffffLL); }

// floor(n / d) for d > 0
__device__ __forceinline__ int64_t floordiv(int64_t n, int64_t d) {
    int64_t q = n / d;
    if ((n % d) != 0 && n < 0) --q;
    return q;
}
// Smallest integer x at which candidate r (position qr, value gr, index ir)
// beats candidate p (position qp < qr) in the (value, index) order.
__device__ __forceinline__ int64_t cross_threshold(int64_t qp, int64_t gp, int32_t ip, int64_t qr, int64_t gr,
                                                   int32_t ir) {
    const int64_t den = 2 * (qr - qp);
    const int64_t num = qr * qr - qp * qp + gr - gp;
    const int64_t fl = floordiv(num, den);
    if (fl * den == num && ir < ip) return fl;
    return fl + 1;
}

// Pass 1: one warp per lattice row along z (volume b, a, b'), NC = Z_b + 1
// points; `ncmax` is the longest row of the batch (shared memory per warp).
__global__ void __launch_bounds__(256) ft_rows_kernel(const int32_t* __restrict__ site_id, int64_t* __restrict__ out,
                                                      VolTab T, int ncmax) {
    extern __shared__ int64_t left_sm[];  // per warp: ncmax entries
    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    int64_t* left = left_sm + (int64_t)wib * ncmax;
    const int64_t warps_total = (int64_t)gridDim.x * (blockDim.x >> 5);
    const int64_t nrows = T.total(kLRow);
    for (int64_t row = (int64_t)blockIdx.x * (blockDim.x >> 5) + wib; row < nrows; row += warps_total) {
        const int bv = T.find(kLRow, row);
        const int NC = T.dim(bv).z + 1;
        const int64_t rbase = T.start(kLat, bv) + (row - T.start(kLRow, bv)) * NC;
        const int32_t* in = site_id + rbase;
        // forward: latest site at or before c, packed (pos << 32 | id); -1 = none
        int64_t carry = -1;
        for (int c0 = 0; c0 < NC; c0 += 32) {
            const int c = c0 + lane;
            int32_t s = c < NC ? in[c] : -1;
            int64_t v = s >= 0 ? (((int64_t)c << 32) | (uint32_t)s) : -1;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                int64_t n = __shfl_up_sync(0xffffffffu, v, o);
                if (lane >= o) v = max(v, n);
            }
            v = max(v, carry);
            if (c < NC) left[c] = v;
            carry = __shfl_sync(0xffffffffu, v, 31);
        }
        __syncwarp();
        // backward: earliest site at or after c; combine with the left one
        int64_t rcarry = kInf;
        const int nchunks = (NC + 31) / 32;
        for (int ch = nchunks - 1; ch >= 0; --ch) {
            const int c = ch * 32 + lane;
            int32_t s = c < NC ? in[c] : -1;
            int64_t v = s >= 0 ? (((int64_t)c << 32) | (uint32_t)s) : kInf;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                int64_t n = __shfl_down_sync(0xffffffffu, v, o);
                if (lane + o < 32) v = min(v, n);
            }
            v = min(v, rcarry);
            rcarry = __shfl_sync(0xffffffffu, v, 0);
            if (c < NC) {
                int64_t best = kInf;
                int64_t l = left[c];
                if (l >= 0) {
                    int64_t d = c - (l >> 32);
                    best = pack(d * d, (int32_t)(uint32_t)(l & 0xffffffffLL));
                }
                if (v != kInf) {
                    int64_t d = (v >> 32) - c;
                    best = min(best, pack(d * d, (int32_t)(uint32_t)(v & 0xffffffffLL)));
                }
                out[rbase + c] = best;
            }
        }
        __syncwarp();
    }
}

// Passes 2 and 3: lower envelope along the lattice lines of every volume:
// PASS 2 along y (local line (a, c), L = Y+1 points, stride Z+1), PASS 3
// along x (local line (b, c), L = X+1 points, stride (Y+1)(Z+1)).
// Consecutive lines of a volume are consecutive addresses, so each step is a
// coalesced access across the warp.  The envelope stack (position | start
// threshold << 16, both < 2^15) of local line l of volume b lives in `stack`
// at lattice start of b + l * L + k.
template <int PASS>
__global__ void __launch_bounds__(256) ft_envelope_kernel(const int64_t* __restrict__ in, int64_t* __restrict__ out,
                                                          int32_t* __restrict__ d2o, int32_t* __restrict__ ido,
                                                          int32_t* __restrict__ stack, VolTab T) {
    constexpr bool FINAL = PASS == 3;
    constexpr int kSpace = PASS == 2 ? kYLine : kXLine;
    const int64_t nlines = T.total(kSpace);
    for (int64_t gl = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; gl < nlines;
         gl += (int64_t)gridDim.x * blockDim.x) {
        const int bv = T.find(kSpace, gl);
        const int4 dm = T.dim(bv);
        const int64_t NB = dm.y + 1, NC = dm.z + 1;
        const int64_t lat0 = T.start(kLat, bv);
        const int64_t l = gl - T.start(kSpace, bv);
        const int L = PASS == 2 ? (int)NB : dm.x + 1;
        const int64_t stride = PASS == 2 ? NC : NB * NC;
        const int64_t base = lat0 + (PASS == 2 ? (l / NC) * NB * NC + (l % NC) : l);
        int32_t* st = stack + lat0 + l * L;
        int k = 0;
        // cached top of stack
        int64_t tq = 0, tg = 0, tz = 0;
        int32_t tid = 0;
        for (int q = 0; q < L; ++q) {
            const int64_t cv = __ldg(in + base + (int64_t)q * stride);
            if (cv == kInf) continue;
            const int64_t g = pk_g(cv);
            const int32_t id = pk_id(cv);
            int64_t T = 0;
            while (k > 0) {
                T = cross_threshold(tq, tg, tid, q, g, id);
                if (T <= tz) {
                    --k;
                    if (k > 0) {
                        const int32_t e = st[k - 1];
                        tq = e & 0xffff;
                        tz = (e >> 16) & 0xffff;
                        const int64_t pv = __ldg(in + base + tq * stride);
                        tg = pk_g(pv);
                        tid = pk_id(pv);
                    }
                    continue;
                }
                break;
            }
            if (k == 0) {
                st[0] = q;
                tq = q; tz = 0; tg = g; tid = id;
                k = 1;
            } else if (T < L) {
                st[k] = q | ((int32_t)T << 16);
                tq = q; tz = T; tg = g; tid = id;
                ++k;
            }
        }
        if (k == 0) {
            for (int x = 0; x < L; ++x) {
                const int64_t o = base + (int64_t)x * stride;
                if (FINAL) {
                    d2o[o] = INT32_MAX;
                    ido[o] = -1;
                } else {
                    out[o] = kInf;
                }
            }
            continue;
        }
        int w = 0;
        int32_t e = st[0];
        int64_t wq = e & 0xffff;
        int64_t wv = __ldg(in + base + wq * stride);
        int32_t nz = k > 1 ? ((st[1] >> 16) & 0xffff) : INT32_MAX;
        for (int x = 0; x < L; ++x) {
            while (w + 1 < k && nz <= x) {
                ++w;
                e = st[w];
                wq = e & 0xffff;
                wv = __ldg(in + base + wq * stride);
                nz = w + 1 < k ? ((st[w + 1] >> 16) & 0xffff) : INT32_MAX;
            }
            const int64_t d = (int64_t)x - wq;
            const int64_t g = pk_g(wv) + d * d;
            const int64_t o = base + (int64_t)x * stride;
            if (FINAL) {
                d2o[o] = (int32_t)g;
                ido[o] = pk_id(wv);
            } else {
                out[o] = pack(g, pk_id(wv));
            }
        }
    }
}

}  // namespace

int run_ft(vc_ctx* c) {
    if (c->n_sites < 0) return VC_ERR_STATE;
    const int nvol = c->nvol;
    int ncmax = 0;
    for (int b = 0; b < nvol; ++b) {
        const int64_t NA = c->h_dims[3 * b] + 1, NB = c->h_dims[3 * b + 1] + 1, NC = c->h_dims[3 * b + 2] + 1;
        if (NA > 32767 || NB > 32767 || NC > 32767) return VC_ERR_ARG;
        ncmax = std::max<int>(ncmax, (int)NC);
    }
    const int64_t N = c->h_off[kLat][nvol];
    VC_TRY(ensure_n<int32_t>(c, c->ft_d2, N));
    VC_TRY(ensure_n<int32_t>(c, c->ft_id, N));
    VC_TRY(ensure_n<int64_t>(c, c->ft_tmp, 2 * N));
    Region stage(c, "stage_ft");
    int64_t* A = ptr<int64_t>(c->ft_tmp);
    int64_t* B = A + N;
    {
        const int warps_per_block = 8;
        const size_t smem = (size_t)warps_per_block * ncmax * sizeof(int64_t);
        if (smem > 200 * 1024) return VC_ERR_ARG;
        if (smem > 48 * 1024)
            VC_CUDA(c, cudaFuncSetAttribute(ft_rows_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        const int64_t nrows = c->h_off[kLRow][nvol];
        int blocks = (int)std::min<int64_t>((nrows + warps_per_block - 1) / warps_per_block,
                                            (int64_t)c->num_sms * 8);
        Region r(c, "ft_rows");
        ft_rows_kernel<<<blocks, warps_per_block * 32, smem, c->stream>>>(ptr<int32_t>(c->site_id_lat), A, c->tab,
                                                                          ncmax);
        launched(c);
        VC_CUDA(c, cudaGetLastError());
    }
    {
        // pass 2 along y; its envelope stacks (one int32 per lattice point)
        // live in the d2 output, which pass 3 writes last
        const int64_t nlines = c->h_off[kYLine][nvol];
        int blocks = (int)std::min<int64_t>((nlines + 255) / 256, (int64_t)c->num_sms * 8);
        Region r(c, "ft_envelope_y");
        ft_envelope_kernel<2><<<blocks, 256, 0, c->stream>>>(A, B, nullptr, nullptr, ptr<int32_t>(c->ft_d2), c->tab);
        launched(c);
        VC_CUDA(c, cudaGetLastError());
    }
    {
        // pass 3 along x; its stacks take the pass-1 buffer, dead by now
        const int64_t nlines = c->h_off[kXLine][nvol];
        int blocks = (int)std::min<int64_t>((nlines + 255) / 256, (int64_t)c->num_sms * 8);
        Region r(c, "ft_envelope_x");
        ft_envelope_kernel<3><<<blocks, 256, 0, c->stream>>>(B, nullptr, ptr<int32_t>(c->ft_d2), ptr<int32_t>(c->ft_id),
                                                             reinterpret_cast<int32_t*>(A), c->tab);
        launched(c);
        VC_CUDA(c, cudaGetLastError());
    }
    c->ft_valid = true;
    return VC_OK;
}

}  // namespace vc
