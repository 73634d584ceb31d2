// Context lifetime, device buffers, copies, error plumbing and device-wide
// exclusive scans for the Voxel Cores GB300 library.
#include "vc_internal.cuh"
#include "vc_scan.cuh"

#include <nvtx3/nvToolsExt.h>

#include <algorithm>
#include <cstring>

namespace vc {

int cuda_fail(vc_ctx* c, cudaError_t e, const char* what) {
    if (c) {
        c->last_error = std::string(what) + ": " + cudaGetErrorString(e);
    }
    cudaGetLastError();  // clear sticky-free errors so the context stays usable
    return e == cudaErrorMemoryAllocation ? VC_ERR_OOM : VC_ERR_CUDA;
}

int ensure_ctx(vc_ctx* c, DevBuf& b, size_t bytes) {
    if (b.cap >= bytes && b.p) return VC_OK;
    if (b.p) {
        VC_CUDA(c, cudaFreeAsync(b.p, c->stream));
        c->bytes_held -= (int64_t)b.cap;
        b.p = nullptr;
        b.cap = 0;
    }
    size_t want = std::max<size_t>(bytes, 256);
    if (c->fail_alloc_after >= 0 && c->fail_alloc_after-- == 0) {
        c->last_error = "cudaMallocAsync: allocation failure injected (vc_debug_fail_alloc_after)";
        return VC_ERR_OOM;
    }
    cudaError_t e = cudaMallocAsync(&b.p, want, c->stream);
    if (e != cudaSuccess) {
        b.p = nullptr;
        return cuda_fail(c, e, "cudaMallocAsync");
    }
    b.cap = want;
    c->bytes_held += (int64_t)want;
    return VC_OK;
}

int* dev_err(vc_ctx* c) { return ptr<int>(c->err); }

static cudaEvent_t take_event(vc_ctx* c) {
    if (!c->event_pool.empty()) {
        cudaEvent_t e = c->event_pool.back();
        c->event_pool.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    if (cudaEventCreate(&e) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return e;
}

// Every named region is also an NVTX range (header-only NVTX 3: near-free
// when no profiler is attached), so Nsight timelines show the library's
// stages beside the CUDA-event timings.
Region::Region(vc_ctx* ctx, const char* n) : c(ctx), name(n) {
    nvtxRangePushA(n);
    if (!c->timing) return;
    a = take_event(c);
    if (a) cudaEventRecord(a, c->stream);
}

Region::~Region() {
    nvtxRangePop();
    if (!c->timing || !a) return;
    cudaEvent_t b = take_event(c);
    if (!b) {
        c->event_pool.push_back(a);
        return;
    }
    cudaEventRecord(b, c->stream);
    c->pending.push_back({name, a, b});
}

void resolve_timers(vc_ctx* c) {
    for (auto& p : c->pending) {
        float ms = 0.0f;
        if (cudaEventElapsedTime(&ms, p.a, p.b) == cudaSuccess) {
            auto& t = c->timers[p.name];
            t.first += ms;
            t.second += 1;
        } else {
            cudaGetLastError();
        }
        c->event_pool.push_back(p.a);
        c->event_pool.push_back(p.b);
    }
    c->pending.clear();
}

int sync_check(vc_ctx* c) {
    VC_CUDA(c, cudaStreamSynchronize(c->stream));
    VC_CUDA(c, cudaGetLastError());
    if (!c->pending.empty()) resolve_timers(c);
    int h = 0;
    VC_CUDA(c, cudaMemcpy(&h, c->err.p, sizeof(int), cudaMemcpyDeviceToHost));
    if (h != 0) {
        int zero = 0;
        VC_CUDA(c, cudaMemcpy(c->err.p, &zero, sizeof(int), cudaMemcpyHostToDevice));
        c->last_error = std::string("device-side error: ") + vc_status_string(h);
        return h;
    }
    return VC_OK;
}

int copy_out(vc_ctx* c, void* dst, const void* src, size_t bytes, int mem) {
    if (!dst || bytes == 0) return VC_OK;
    if (mem == VC_MEM_DEVICE) {
        VC_CUDA(c, cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToDevice, c->stream));
        return VC_OK;
    }
    VC_CUDA(c, cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, c->stream));
    return sync_check(c);
}

int copy_in(vc_ctx* c, void* dst, const void* src, size_t bytes, int mem) {
    if (bytes == 0) return VC_OK;
    if (!src) return VC_ERR_ARG;
    VC_CUDA(c, cudaMemcpyAsync(dst, src, bytes, mem == VC_MEM_DEVICE ? cudaMemcpyDeviceToDevice
                                                                     : cudaMemcpyHostToDevice,
                               c->stream));
    return VC_OK;
}

int set_volume_table(vc_ctx* c, int nvol, const int32_t* dims) {
    if (nvol <= 0 || !dims) return VC_ERR_ARG;
    c->nvol = nvol;
    c->h_dims.assign(dims, dims + 3 * (size_t)nvol);
    for (int s = 0; s < kNumSpaces; ++s) {
        auto& o = c->h_off[s];
        o.assign((size_t)nvol + 1, 0);
        for (int b = 0; b < nvol; ++b) o[b + 1] = o[b] + space_size(s, dims[3 * b], dims[3 * b + 1], dims[3 * b + 2]);
    }
    VolTab t;
    t.nvol = nvol;
    t.d0 = make_int4(dims[0], dims[1], dims[2], 0);
    if (nvol > 1) {
        // device copy: int4 dims[nvol], then the starts of every space
        const size_t n4 = (size_t)nvol, n8 = (size_t)nvol + 1;
        const size_t bytes = n4 * sizeof(int4) + kNumSpaces * n8 * sizeof(int64_t);
        c->h_tab_stage.resize(bytes);
        auto* d4 = reinterpret_cast<int4*>(c->h_tab_stage.data());
        for (int b = 0; b < nvol; ++b) d4[b] = make_int4(dims[3 * b], dims[3 * b + 1], dims[3 * b + 2], 0);
        auto* o8 = reinterpret_cast<int64_t*>(c->h_tab_stage.data() + n4 * sizeof(int4));
        for (int s = 0; s < kNumSpaces; ++s)
            for (size_t b = 0; b < n8; ++b) o8[s * n8 + b] = c->h_off[s][b];
        VC_TRY(ensure_n<uint8_t>(c, c->tab_buf, (int64_t)bytes));
        VC_CUDA(c, cudaMemcpyAsync(c->tab_buf.p, c->h_tab_stage.data(), bytes, cudaMemcpyHostToDevice, c->stream));
        VC_CUDA(c, cudaStreamSynchronize(c->stream));
        t.dims = ptr<int4>(c->tab_buf);
        const int64_t* d8 = reinterpret_cast<const int64_t*>(ptr<uint8_t>(c->tab_buf) + n4 * sizeof(int4));
        for (int s = 0; s < kNumSpaces; ++s) t.off[s] = d8 + s * n8;
    }
    c->tab = t;
    // per-volume bases: kNumBases int64 arrays, bbox, inside size, threshold
    const size_t n8 = (size_t)nvol + 1;
    const size_t bytes = kNumBases * n8 * sizeof(int64_t) + 6 * (size_t)nvol * sizeof(int32_t) +
                         2 * (size_t)nvol * sizeof(float);
    VC_TRY(ensure_n<uint8_t>(c, c->bases_buf, (int64_t)bytes));
    uint8_t* p = ptr<uint8_t>(c->bases_buf);
    for (int k = 0; k < kNumBases; ++k) c->bases.b[k] = reinterpret_cast<int64_t*>(p) + k * n8;
    p += kNumBases * n8 * sizeof(int64_t);
    c->bases.bbox = reinterpret_cast<int32_t*>(p);
    p += 6 * (size_t)nvol * sizeof(int32_t);
    c->bases.inside = reinterpret_cast<float*>(p);
    c->bases.thr = c->bases.inside + nvol;
    return VC_OK;
}

namespace {
__global__ void fill_bases_kernel(VolTab T, int space, const int32_t* __restrict__ scan, const int64_t* total,
                                  int64_t* __restrict__ out) {
    for (int b = blockIdx.x * blockDim.x + threadIdx.x; b <= T.nvol; b += gridDim.x * blockDim.x)
        out[b] = b < T.nvol ? (int64_t)scan[T.start(space, b)] : *total;
}
}  // namespace

int fill_bases(vc_ctx* c, int base, int space, const int32_t* scan, const int64_t* total_dev) {
    const int n = c->nvol + 1;
    fill_bases_kernel<<<(n + 255) / 256, 256, 0, c->stream>>>(c->tab, space, scan, total_dev, c->bases.b[base]);
    launched(c);
    VC_CUDA(c, cudaGetLastError());
    return VC_OK;
}

int read_i64(vc_ctx* c, const int64_t* src, int64_t* out) {
    VC_CUDA(c, cudaMemcpyAsync(out, src, sizeof(int64_t), cudaMemcpyDeviceToHost, c->stream));
    return sync_check(c);
}

template <class T>
static int scan_impl(vc_ctx* c, const T* in, T* out, int64_t n, int64_t* total_dev) {
    if (n <= 0) {
        if (total_dev) VC_CUDA(c, cudaMemsetAsync(total_dev, 0, sizeof(int64_t), c->stream));
        return VC_OK;
    }
    int64_t tiles = (n + kScanTile - 1) / kScanTile;
    VC_TRY(ensure_n<int64_t>(c, c->scratch, tiles + 1));
    int64_t* sums = ptr<int64_t>(c->scratch);
    scan_tile_sums<T><<<(unsigned)tiles, kScanThreads, 0, c->stream>>>(in, n, sums);
    scan_sums_single<<<1, 1024, 0, c->stream>>>(sums, tiles, total_dev);
    scan_apply<T><<<(unsigned)tiles, kScanThreads, 0, c->stream>>>(in, out, n, sums);
    launched(c, 3);
    VC_CUDA(c, cudaGetLastError());
    return VC_OK;
}

int scan_exclusive_i32(vc_ctx* c, const int32_t* in, int32_t* out, int64_t n, int64_t* total_dev) {
    return scan_impl<int32_t>(c, in, out, n, total_dev);
}
int scan_exclusive_i64(vc_ctx* c, const int64_t* in, int64_t* out, int64_t n, int64_t* total_dev) {
    return scan_impl<int64_t>(c, in, out, n, total_dev);
}

// Every device buffer of a context except its error word.
std::vector<DevBuf*> ctx_buffers(vc_ctx* c) {
    return {&c->scratch, &c->scratch2, &c->occ, &c->oct_cells, &c->oct_nodes, &c->oct_stream, &c->oct_leaves, &c->site_xyz, &c->site_count, &c->site_bits, &c->site_id_lat, &c->ft_d2,
            &c->ft_id, &c->ft_tmp, &c->ft_far, &c->vd_seg, &c->vd_voff, &c->vd_eoff, &c->vd_foff, &c->vd_tri_face,
            &c->vd_face_sites, &c->vd_lam, &c->vd_radius, &c->vd_vlat, &c->vd_fpass, &c->tab_buf, &c->bases_buf, &c->vts, &c->edges_in, &c->edges, &c->tris,
            &c->tri_edges, &c->ve_off, &c->ve_ids, &c->ef_off, &c->ef_ids, &c->hash_keys, &c->hash_pos,
            &c->hash_id, &c->side_slot, &c->vm, &c->em, &c->fm, &c->face_rec, &c->edge_rec, &c->vert_rec, &c->thin_g0, &c->q0,
            &c->q1, &c->child, &c->cells, &c->blk_cnt, &c->keep_v, &c->keep_e,
            &c->keep_f, &c->removed_e, &c->keep_bits, &c->keep_wv, &c->keep_we, &c->keep_wf, &c->trace, &c->thr,
            &c->rem_vts, &c->rem_edges, &c->rem_tris, &c->uf_parent, &c->euler_tmp};
}

// Free every buffer of the context (it keeps its stream and error word);
// all results are gone and the next call starts from vc_set_volume,
// vc_batch_set_volumes or vc_set_complex.
int ctx_release_buffers(vc_ctx* c) {
    VC_CUDA(c, cudaSetDevice(c->device));
    VC_CUDA(c, cudaStreamSynchronize(c->stream));
    for (DevBuf* b : ctx_buffers(c)) {
        if (b->p) {
            cudaFreeAsync(b->p, c->stream);
            c->bytes_held -= (int64_t)b->cap;
        }
        b->p = nullptr;
        b->cap = 0;
    }
    c->n_sites = -1;
    c->ft_valid = c->vd_valid = c->cc_valid = c->cc_finalized = c->meas_valid = c->thin_valid = c->rem_valid = false;
    c->records_fresh = c->records_thr_folded = c->cc_batched = false;
    c->vd_geom = c->vd_aux_meas = c->vd_aux_topo = false;
    c->nvol = 0;
    c->tab = VolTab{};
    c->bases = Bases{};
    VC_CUDA(c, cudaStreamSynchronize(c->stream));
    return VC_OK;
}

}  // namespace vc

// ---------------------------------------------------------------------------
// Context entry points.
extern "C" {

int vc_version(void) { return 100; }

const char* vc_status_string(int s) {
    switch (s) {
        case VC_OK: return "ok";
        case VC_ERR_ARG: return "invalid argument";
        case VC_ERR_OOM: return "out of device memory";
        case VC_ERR_TIMEOUT: return "device-side wait timed out";
        case VC_ERR_INVARIANT: return "thinning invariant violated (reference exit(1) case)";
        case VC_ERR_CUDA: return "CUDA error";
        case VC_ERR_STATE: return "inputs for this call are missing";
        default: return "unknown status";
    }
}

int vc_ctx_create(vc_ctx** out, int device) {
    if (!out) return VC_ERR_ARG;
    *out = nullptr;
    vc_ctx* c = new vc_ctx();
    c->device = device;
    cudaError_t e = cudaSetDevice(device);
    if (e != cudaSuccess) {
        delete c;
        cudaGetLastError();
        return VC_ERR_CUDA;
    }
    e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        delete c;
        cudaGetLastError();
        return VC_ERR_CUDA;
    }
    cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, device);
    // The context's buffers live in the device's default stream-ordered pool
    // and are reused across calls; keep freed pool memory mapped instead of
    // returning it to the driver at every synchronization.
    {
        cudaMemPool_t pool;
        if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
            uint64_t keep = UINT64_MAX;
            cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
        }
        cudaGetLastError();
    }
    int s = vc::ensure_n<int64_t>(c, c->err, 16);
    if (s == VC_OK) {
        e = cudaMemsetAsync(c->err.p, 0, 16 * sizeof(int64_t), c->stream);
        if (e != cudaSuccess) s = vc::cuda_fail(c, e, "memset");
    }
    if (s == VC_OK) s = vc::sync_check(c);
    if (s != VC_OK) {
        vc_ctx_destroy(c);
        return s;
    }
    *out = c;
    return VC_OK;
}

static void free_buf(vc_ctx* c, vc::DevBuf& b) {
    if (b.p) cudaFreeAsync(b.p, c->stream);
    b.p = nullptr;
    b.cap = 0;
}

int vc_ctx_destroy(vc_ctx* c) {
    if (!c) return VC_OK;
    cudaSetDevice(c->device);
    for (auto* b : vc::ctx_buffers(c)) free_buf(c, *b);
    free_buf(c, c->err);
    if (c->stream) cudaStreamSynchronize(c->stream);
    for (auto& p : c->pending) {
        cudaEventDestroy(p.a);
        cudaEventDestroy(p.b);
    }
    for (auto e : c->event_pool) cudaEventDestroy(e);
    if (c->stream) {
        cudaStreamSynchronize(c->stream);
        cudaStreamDestroy(c->stream);
    }
    cudaGetLastError();
    delete c;
    return VC_OK;
}

void* vc_ctx_stream(vc_ctx* c) { return c ? (void*)c->stream : nullptr; }

int vc_ctx_sync(vc_ctx* c) {
    if (!c) return VC_ERR_ARG;
    return vc::sync_check(c);
}

const char* vc_ctx_last_error(vc_ctx* c) { return c ? c->last_error.c_str() : "no context"; }

int64_t vc_ctx_device_bytes(vc_ctx* c) { return c ? c->bytes_held : 0; }

int64_t vc_ctx_launch_count(vc_ctx* c) { return c ? c->launches : 0; }

int vc_ctx_set_timing(vc_ctx* c, int enable) {
    if (!c) return VC_ERR_ARG;
    int s = vc::sync_check(c);
    c->timing = enable != 0;
    return s;
}

int vc_ctx_reset_timings(vc_ctx* c) {
    if (!c) return VC_ERR_ARG;
    int s = vc::sync_check(c);
    c->timers.clear();
    return s;
}

int vc_ctx_get_timings(vc_ctx* c, char* names, int name_len, double* ms, int64_t* counts, int cap, int* n) {
    if (!c || !n || name_len <= 1) return VC_ERR_ARG;
    int s = vc::sync_check(c);
    int k = 0;
    for (auto& kv : c->timers) {
        if (k < cap) {
            if (names) {
                std::strncpy(names + (size_t)k * name_len, kv.first.c_str(), (size_t)name_len - 1);
                names[(size_t)k * name_len + name_len - 1] = 0;
            }
            if (ms) ms[k] = kv.second.first;
            if (counts) counts[k] = kv.second.second;
        }
        ++k;
    }
    *n = k;
    return s;
}

}  // extern "C"
