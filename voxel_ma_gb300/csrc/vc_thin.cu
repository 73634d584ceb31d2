// FIFO-exact simple-pair thinning on the GPU (replaces
// CellComplexThinning::prune, src/ccthin.cpp:201-424 and 514-771).
//
// The reference pops a FIFO queue of simple pairs: face-edge (FE) pairs and
// edge-vertex (EV) pairs.  Its queue is generation-major: generation 0 is
// every FE pair in edge order followed by every EV pair in vertex order
// (ccthin.cpp:248-270); generation g+1 is the children pushed while popping
// generation g, ordered by (parent position, push order inside the parent).
// This kernel replays one generation at a time and reproduces the sequential
// result exactly, because within a generation:
//   * an item is skipped iff its first cell (the face of an FE pair, the edge
//     of an EV pair) was removed earlier; a cell is removed only by the first
//     item naming it (an atomicMin "claim" on its queue position);
//   * reference counts only fall, so a count reaches 1 at exactly one
//     decrement; if the count ends the generation at 1 after falling in it,
//     that happened at the LAST decrement, i.e. at the largest position that
//     decremented it (atomicMax), and the unique remaining face/edge at that
//     moment is the unique one left at the end of the generation;
//   * if the count fell through 1 to 0 inside the generation, the child the
//     reference pushed is skipped when popped (its cell is gone), so it can
//     be dropped;
//   * children are written in (parent position, slot) order with one
//     exclusive scan, slots being the face's other sides in face order, then
//     the removed edge's two ends (ccthin.cpp:659-767), or the other end of
//     an EV pair's edge (ccthin.cpp:610-636).
// One persistent cooperative kernel runs all generations with three bounded
// grid barriers per generation; the claims of generation g+1 are made while
// generation g writes it.  Removal state is kept as the queue position of the
// removing item (INT32_MAX = alive), so every check is position-exact.
#include "vc_internal.cuh"

namespace vc {
namespace {

constexpr int kThreads = 256;
constexpr int32_t kAlive = INT32_MAX;
constexpr unsigned kFE = 0x80000000u;

struct ThinArgs {
    const int2* edges;
    const int32_t* tri_edges;
    const int32_t* ve_off;
    const int32_t* ve_ids;
    const int32_t* ef_off;
    const int32_t* ef_ids;
    const float* em;
    const float* fm;
    const float* thr;  // [0] f_t, [1] l_t
    int32_t* rm_f;
    int32_t* rm_e;
    int32_t* rm_v;
    int32_t* ref_e;
    int32_t* ref_v;
    int32_t* trig_e;
    int32_t* trig_v;
    int2* qa;
    int2* qb;
    int2* child;
    uint8_t* child_cnt;
    int64_t* blk_cnt;
    unsigned* bar;
    int* err;
    int64_t* ctl;  // [0] gen-0 size; out: [1] pushes, [2] processed, [3] skipped, [4] generations
    unsigned long long spin_limit;
};

__device__ __forceinline__ int2 make_fe(int32_t f, int32_t e) { return make_int2((int32_t)((unsigned)f | kFE), e); }
__device__ __forceinline__ int2 make_ev(int32_t e, int32_t v) { return make_int2(e, v); }
__device__ __forceinline__ bool is_fe(int2 it) { return ((unsigned)it.x & kFE) != 0; }
__device__ __forceinline__ int32_t idx0(int2 it) { return (int32_t)((unsigned)it.x & ~kFE); }

__device__ __forceinline__ int2 ld_item(const int2* p) {
    return __ldcg(p);
}

__global__ void thin_init_kernel(const int32_t* __restrict__ ve_off, const int32_t* __restrict__ ef_off, int32_t nv,
                                 int32_t ne, int32_t nt, int32_t* rm_f, int32_t* rm_e, int32_t* rm_v, int32_t* ref_e,
                                 int32_t* ref_v, int32_t* trig_e, int32_t* trig_v) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    const int64_t n = (int64_t)nv + ne + nt;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        if (i < ne) {
            ref_e[i] = ef_off[i + 1] - ef_off[i];
            rm_e[i] = kAlive;
            trig_e[i] = -1;
        } else if (i < (int64_t)ne + nv) {
            const int64_t v = i - ne;
            ref_v[v] = ve_off[v + 1] - ve_off[v];
            rm_v[v] = kAlive;
            trig_v[v] = -1;
        } else {
            rm_f[i - ne - nv] = kAlive;
        }
    }
}

// Generation 0: FE pairs of edges with one face (edge order), then EV pairs
// of vertices with one edge (vertex order), filtered by the thresholds.
__global__ void gen0_flags_kernel(ThinArgs A, int32_t nv, int32_t ne, int32_t* __restrict__ flag) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    const float f_t = A.thr[0], l_t = A.thr[1];
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < (int64_t)ne + nv; i += stride) {
        int32_t ok = 0;
        if (i < ne) {
            if (A.ref_e[i] == 1) ok = A.fm[A.ef_ids[A.ef_off[i]]] < f_t;
        } else {
            const int64_t v = i - ne;
            if (A.ref_v[v] == 1) ok = A.em[A.ve_ids[A.ve_off[v]]] < l_t;
        }
        flag[i] = ok;
    }
}

__global__ void gen0_write_kernel(ThinArgs A, int32_t nv, int32_t ne, const int32_t* __restrict__ flag,
                                  const int32_t* __restrict__ pos) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < (int64_t)ne + nv; i += stride) {
        if (!flag[i]) continue;
        const int32_t p = pos[i];
        if (i < ne) {
            const int32_t f = A.ef_ids[A.ef_off[i]];
            A.qa[p] = make_fe(f, (int32_t)i);
            atomicMin(&A.rm_f[f], p);
        } else {
            const int32_t v = (int32_t)(i - ne);
            const int32_t e = A.ve_ids[A.ve_off[v]];
            A.qa[p] = make_ev(e, v);
            atomicMin(&A.rm_e[e], p);
        }
    }
}

// Unique remaining face of edge e (the first with no removal position).
__device__ __forceinline__ int32_t live_face(const ThinArgs& A, int32_t e) {
    const int32_t b = A.ef_off[e], t = A.ef_off[e + 1];
    for (int32_t k = b; k < t; ++k) {
        const int32_t f = A.ef_ids[k];
        if (__ldcg(A.rm_f + f) == kAlive) return f;
    }
    return -1;
}
__device__ __forceinline__ int32_t live_edge(const ThinArgs& A, int32_t v) {
    const int32_t b = A.ve_off[v], t = A.ve_off[v + 1];
    for (int32_t k = b; k < t; ++k) {
        const int32_t e = A.ve_ids[k];
        if (__ldcg(A.rm_e + e) == kAlive) return e;
    }
    return -1;
}

__global__ void __launch_bounds__(kThreads) thin_generations_kernel(ThinArgs A) {
    __shared__ int64_t sm[33];
    __shared__ int64_t s_red[2];
    const int G = gridDim.x, b = blockIdx.x;
    const float f_t = A.thr[0], l_t = A.thr[1];
    int64_t n = A.ctl[0];
    int64_t base = 0, pushes = n;
    int gen = 0;
    int64_t my_processed = 0, my_skipped = 0;
    while (n > 0) {
        const int2* cur = (gen & 1) ? A.qb : A.qa;
        int2* nxt = (gen & 1) ? A.qa : A.qb;
        const int64_t chunk = (n + G - 1) / G;
        const int64_t i0 = min(n, (int64_t)b * chunk), i1 = min(n, i0 + chunk);
        // ---- phase A: apply the removals of the items that won their claim
        for (int64_t i = i0 + threadIdx.x; i < i1; i += blockDim.x) {
            const int2 it = ld_item(cur + i);
            const int32_t p = (int32_t)(base + i);
            if (is_fe(it)) {
                const int32_t f = idx0(it), e = it.y;
                if (__ldcg(A.rm_f + f) != p) {
                    ++my_skipped;
                    continue;
                }
                if (__ldcg(A.ref_e + e) != 1) {
                    set_error(A.err, VC_ERR_INVARIANT);
                    continue;
                }
                ++my_processed;
                atomicMin(&A.rm_e[e], p);
                A.ref_e[e] = 0;
#pragma unroll
                for (int s = 0; s < 3; ++s) {
                    const int32_t e2 = A.tri_edges[3 * (int64_t)f + s];
                    if (e2 == e || __ldcg(A.rm_e + e2) < p) continue;
                    atomicSub(&A.ref_e[e2], 1);
                    atomicMax(&A.trig_e[e2], p);
                }
                const int2 ev = A.edges[e];
                atomicSub(&A.ref_v[ev.x], 1);
                atomicMax(&A.trig_v[ev.x], p);
                atomicSub(&A.ref_v[ev.y], 1);
                atomicMax(&A.trig_v[ev.y], p);
            } else {
                const int32_t e = it.x, v = it.y;
                if (__ldcg(A.rm_e + e) != p) {
                    ++my_skipped;
                    continue;
                }
                if (__ldcg(A.ref_v + v) != 1) {
                    set_error(A.err, VC_ERR_INVARIANT);
                    continue;
                }
                ++my_processed;
                A.rm_v[v] = p;
                const int2 ev = A.edges[e];
                atomicSub(&A.ref_v[ev.x], 1);
                atomicMax(&A.trig_v[ev.x], p);
                atomicSub(&A.ref_v[ev.y], 1);
                atomicMax(&A.trig_v[ev.y], p);
            }
        }
        grid_barrier(A.bar, A.err, A.spin_limit);
        if (*((volatile int*)A.err)) break;
        // ---- phase B: find each processed item's children (in slot order)
        int64_t local = 0;
        for (int64_t i = i0 + threadIdx.x; i < i1; i += blockDim.x) {
            const int2 it = ld_item(cur + i);
            const int32_t p = (int32_t)(base + i);
            int cnt = 0;
            int2* out = A.child + 4 * i;
            if (is_fe(it)) {
                const int32_t f = idx0(it), e = it.y;
                if (__ldcg(A.rm_f + f) == p) {
#pragma unroll
                    for (int s = 0; s < 3; ++s) {
                        const int32_t e2 = A.tri_edges[3 * (int64_t)f + s];
                        if (e2 == e) continue;
                        if (__ldcg(A.trig_e + e2) == p && __ldcg(A.ref_e + e2) == 1) {
                            const int32_t f2 = live_face(A, e2);
                            if (f2 < 0) {
                                set_error(A.err, VC_ERR_INVARIANT);
                            } else if (A.fm[f2] < f_t) {
                                out[cnt++] = make_fe(f2, e2);
                            }
                        }
                    }
                    const int2 ev = A.edges[e];
#pragma unroll
                    for (int s = 0; s < 2; ++s) {
                        const int32_t u = s == 0 ? ev.x : ev.y;
                        if (__ldcg(A.trig_v + u) == p && __ldcg(A.ref_v + u) == 1) {
                            const int32_t e3 = live_edge(A, u);
                            if (e3 < 0) {
                                set_error(A.err, VC_ERR_INVARIANT);
                            } else if (A.em[e3] < l_t) {
                                out[cnt++] = make_ev(e3, u);
                            }
                        }
                    }
                }
            } else {
                const int32_t e = it.x, v = it.y;
                if (__ldcg(A.rm_e + e) == p) {
                    const int2 ev = A.edges[e];
                    const int32_t u = ev.x != v ? ev.x : ev.y;
                    if (__ldcg(A.trig_v + u) == p && __ldcg(A.ref_v + u) == 1) {
                        const int32_t e3 = live_edge(A, u);
                        if (e3 < 0) {
                            set_error(A.err, VC_ERR_INVARIANT);
                        } else if (A.em[e3] < l_t) {
                            out[cnt++] = make_ev(e3, u);
                        }
                    }
                }
            }
            A.child_cnt[i] = (uint8_t)cnt;
            local += cnt;
        }
        {
            int64_t tot;
            block_exclusive_sum<int64_t>(local, sm, &tot);
            if (threadIdx.x == 0) A.blk_cnt[b] = tot;
        }
        grid_barrier(A.bar, A.err, A.spin_limit);
        if (*((volatile int*)A.err)) break;
        // ---- phase C: block prefix, write generation g+1 and make its claims
        {
            int64_t before = 0, all = 0;
            for (int k = threadIdx.x; k < G; k += blockDim.x) {
                const int64_t v = __ldcg(A.blk_cnt + k);
                all += v;
                if (k < b) before += v;
            }
            int64_t t1, t2;
            block_exclusive_sum<int64_t>(before, sm, &t1);
            block_exclusive_sum<int64_t>(all, sm, &t2);
            if (threadIdx.x == 0) {
                s_red[0] = t1;
                s_red[1] = t2;
            }
            __syncthreads();
        }
        const int64_t prefix = s_red[0], total = s_red[1];
        const int64_t nbase = base + n;
        int64_t running = prefix;
        for (int64_t r = i0; r < i1; r += blockDim.x) {
            const int64_t i = r + threadIdx.x;
            const int cnt = i < i1 ? (int)A.child_cnt[i] : 0;
            int64_t tot;
            const int64_t ex = block_exclusive_sum<int64_t>((int64_t)cnt, sm, &tot);
            for (int k = 0; k < cnt; ++k) {
                const int2 ch = A.child[4 * i + k];
                const int64_t slot = running + ex + k;
                nxt[slot] = ch;
                const int32_t q = (int32_t)(nbase + slot);
                if (is_fe(ch)) atomicMin(&A.rm_f[idx0(ch)], q);
                else atomicMin(&A.rm_e[ch.x], q);
            }
            running += tot;
        }
        __syncthreads();
        base = nbase;
        n = total;
        pushes += total;
        ++gen;
        grid_barrier(A.bar, A.err, A.spin_limit);
        if (*((volatile int*)A.err)) break;
    }
    atomicAdd((unsigned long long*)&A.ctl[2], (unsigned long long)my_processed);
    atomicAdd((unsigned long long*)&A.ctl[3], (unsigned long long)my_skipped);
    if (b == 0 && threadIdx.x == 0) {
        A.ctl[1] = pushes;
        A.ctl[4] = gen;
    }
}

__global__ void set_thr_kernel(float* thr, float f_t, float l_t) {
    thr[0] = f_t;
    thr[1] = l_t;
}

__global__ void thin_flags_kernel(const int32_t* __restrict__ rm_v, const int32_t* __restrict__ rm_e,
                                  const int32_t* __restrict__ ref_e, const int32_t* __restrict__ rm_f, int32_t nv,
                                  int32_t ne, int32_t nt, uint8_t* kv, uint8_t* ke, uint8_t* kf, uint8_t* re) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < (int64_t)nv + ne + nt; i += stride) {
        if (i < nv) {
            if (kv) kv[i] = rm_v[i] == kAlive;
        } else if (i < (int64_t)nv + ne) {
            const int64_t e = i - nv;
            if (ke) ke[e] = rm_e[e] == kAlive && ref_e[e] == 0;
            if (re) re[e] = rm_e[e] != kAlive;
        } else {
            const int64_t f = i - nv - ne;
            if (kf) kf[f] = rm_f[f] == kAlive;
        }
    }
}

inline int grid_for(vc_ctx* c, int64_t n, int threads) {
    int64_t b = (n + threads - 1) / threads;
    return (int)std::max<int64_t>(1, std::min<int64_t>(b, (int64_t)c->num_sms * 16));
}

}  // namespace

int run_thin_with_device_thr(vc_ctx* c, vc_thin_stats* stats);

int run_thin(vc_ctx* c, float f_t, float l_t, vc_thin_stats* stats) {
    if (!c->cc_finalized || !c->meas_valid) return VC_ERR_STATE;
    VC_TRY(ensure_n<float>(c, c->thr, 2));
    set_thr_kernel<<<1, 1, 0, c->stream>>>(ptr<float>(c->thr), f_t, l_t);
    launched(c);
    VC_CUDA(c, cudaGetLastError());
    return run_thin_with_device_thr(c, stats);
}

// Thinning with thresholds already in c->thr (device), e.g. computed from the
// complex's inside size on the device.
int run_thin_with_device_thr(vc_ctx* c, vc_thin_stats* stats) {
    if (!c->cc_finalized || !c->meas_valid) return VC_ERR_STATE;
    const int64_t nv = c->nv, ne = c->ne, nt = c->nt;
    if (nv + ne >= INT32_MAX) return VC_ERR_ARG;
    const int64_t qcap = nv + ne + 1;
    Region stage(c, "stage_thin");
    VC_TRY(ensure_n<int32_t>(c, c->rm_f, nt));
    VC_TRY(ensure_n<int32_t>(c, c->rm_e, ne));
    VC_TRY(ensure_n<int32_t>(c, c->rm_v, nv));
    VC_TRY(ensure_n<int32_t>(c, c->ref_e, ne));
    VC_TRY(ensure_n<int32_t>(c, c->ref_v, nv));
    VC_TRY(ensure_n<int32_t>(c, c->trig_e, ne));
    VC_TRY(ensure_n<int32_t>(c, c->trig_v, nv));
    VC_TRY(ensure_n<int2>(c, c->q0, qcap));
    VC_TRY(ensure_n<int2>(c, c->q1, qcap));
    VC_TRY(ensure_n<int2>(c, c->child, 4 * qcap));
    VC_TRY(ensure_n<uint8_t>(c, c->child_cnt, qcap));
    VC_TRY(ensure_n<int32_t>(c, c->scratch2, 2 * (nv + ne) + 2));
    VC_TRY(ensure_n<int64_t>(c, c->euler_tmp, 16));
    ThinArgs A{};
    A.edges = ptr<int2>(c->edges);
    A.tri_edges = ptr<int32_t>(c->tri_edges);
    A.ve_off = ptr<int32_t>(c->ve_off);
    A.ve_ids = ptr<int32_t>(c->ve_ids);
    A.ef_off = ptr<int32_t>(c->ef_off);
    A.ef_ids = ptr<int32_t>(c->ef_ids);
    A.em = ptr<float>(c->em);
    A.fm = ptr<float>(c->fm);
    A.thr = ptr<float>(c->thr);
    A.rm_f = ptr<int32_t>(c->rm_f);
    A.rm_e = ptr<int32_t>(c->rm_e);
    A.rm_v = ptr<int32_t>(c->rm_v);
    A.ref_e = ptr<int32_t>(c->ref_e);
    A.ref_v = ptr<int32_t>(c->ref_v);
    A.trig_e = ptr<int32_t>(c->trig_e);
    A.trig_v = ptr<int32_t>(c->trig_v);
    A.qa = ptr<int2>(c->q0);
    A.qb = ptr<int2>(c->q1);
    A.child = ptr<int2>(c->child);
    A.child_cnt = ptr<uint8_t>(c->child_cnt);
    A.err = dev_err(c);
    int64_t* ctl = ptr<int64_t>(c->euler_tmp);
    A.ctl = ctl;
    A.bar = reinterpret_cast<unsigned*>(ctl + 8);
    A.spin_limit = 1ull << 26;
    thin_init_kernel<<<grid_for(c, nv + ne + nt, 256), 256, 0, c->stream>>>(
        A.ve_off, A.ef_off, (int32_t)nv, (int32_t)ne, (int32_t)nt, A.rm_f, A.rm_e, A.rm_v, A.ref_e, A.ref_v,
        A.trig_e, A.trig_v);
    launched(c);
    int32_t* flag = ptr<int32_t>(c->scratch2);
    int32_t* pos = flag + (nv + ne + 1);
    gen0_flags_kernel<<<grid_for(c, nv + ne, 256), 256, 0, c->stream>>>(A, (int32_t)nv, (int32_t)ne, flag);
    launched(c);
    VC_CUDA(c, cudaMemsetAsync(ctl, 0, 16 * sizeof(int64_t), c->stream));
    VC_TRY(scan_exclusive_i32(c, flag, pos, nv + ne, ctl + 0));
    gen0_write_kernel<<<grid_for(c, nv + ne, 256), 256, 0, c->stream>>>(A, (int32_t)nv, (int32_t)ne, flag, pos);
    launched(c);
    VC_CUDA(c, cudaGetLastError());
    // persistent cooperative launch: every block resident
    int per_sm = 0;
    VC_CUDA(c, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, thin_generations_kernel, kThreads, 0));
    if (per_sm <= 0) return VC_ERR_CUDA;
    int G = c->num_sms * std::min(per_sm, 4);
    VC_TRY(ensure_n<int64_t>(c, c->blk_cnt, G));
    A.blk_cnt = ptr<int64_t>(c->blk_cnt);
    void* args[] = {&A};
    {
        Region r(c, "thin_generations");
        VC_CUDA(c, cudaLaunchCooperativeKernel((void*)thin_generations_kernel, dim3(G), dim3(kThreads), args, 0,
                                               c->stream));
        launched(c);
    }
    int64_t h[5];
    VC_CUDA(c, cudaMemcpyAsync(h, ctl, 5 * sizeof(int64_t), cudaMemcpyDeviceToHost, c->stream));
    int s = sync_check(c);
    if (s != VC_OK) return s;
    c->thin_stats = vc_thin_stats{h[1], h[2], h[3], h[4]};
    c->thin_valid = true;
    c->rem_valid = false;
    if (stats) *stats = c->thin_stats;
    return VC_OK;
}

int get_thin_flags(vc_ctx* c, uint8_t* kv, uint8_t* ke, uint8_t* kf, uint8_t* re, int mem) {
    if (!c->thin_valid) return VC_ERR_STATE;
    const int64_t nv = c->nv, ne = c->ne, nt = c->nt;
    VC_TRY(ensure_n<uint8_t>(c, c->scratch, nv + 2 * ne + nt + 16));
    uint8_t* d = ptr<uint8_t>(c->scratch);
    uint8_t *dkv = d, *dke = d + nv, *dre = d + nv + ne, *dkf = d + nv + 2 * ne;
    thin_flags_kernel<<<grid_for(c, nv + ne + nt, 256), 256, 0, c->stream>>>(
        ptr<int32_t>(c->rm_v), ptr<int32_t>(c->rm_e), ptr<int32_t>(c->ref_e), ptr<int32_t>(c->rm_f), (int32_t)nv,
        (int32_t)ne, (int32_t)nt, dkv, dke, dkf, dre);
    launched(c);
    VC_CUDA(c, cudaGetLastError());
    VC_TRY(copy_out(c, kv, dkv, nv, mem));
    VC_TRY(copy_out(c, ke, dke, ne, mem));
    VC_TRY(copy_out(c, kf, dkf, nt, mem));
    VC_TRY(copy_out(c, re, dre, ne, mem));
    return sync_check(c);
}

}  // namespace vc
