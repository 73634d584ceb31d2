// Request loop: continuous batching of volumes on one GPU.
//
// The reference answers one volume per process run (voroUtility main ->
// exportInsideVoroMesh, src/highlevelalgo.cpp:731-961).  Here requests are
// queued as they arrive and served by a few worker threads, each owning a
// context (its own CUDA stream and device buffers).  A worker that becomes
// free takes the oldest pending requests that fit its share of the memory
// cap as one batch (vc_batch_run), so requests arriving while other batches
// are on the GPU join the next batch as soon as a slot and memory free up,
// and the workers' batches overlap on the device.  Every result equals the
// plain single-volume result (the batched path guarantees it per volume).
//
// Memory admission: a request's footprint is estimated as bytes_per_voxel x
// voxels; a batch's estimate must fit the worker's share (cap / workers),
// and a worker whose context holds more than its share after a batch
// releases its buffers.  Requests that cannot fit a share are refused at
// submission.
#include "vc_internal.cuh"

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <thread>
#include <unordered_map>

namespace vc {
int ctx_release_buffers(vc_ctx* c);
}

namespace {

double now_s() {
    using namespace std::chrono;
    return duration<double>(steady_clock::now().time_since_epoch()).count();
}

struct Request {
    int64_t id = 0;
    int X = 0, Y = 0, Z = 0;
    double t = 0.0;
    int64_t est = 0;
    std::vector<uint8_t> occ;
    double t_submit = 0, t_start = 0, t_done = 0;
    bool done = false;
    vc_request_result res{};
    std::vector<float> vts;
    std::vector<int32_t> edges, tris;
};

}  // namespace

struct vc_server {
    std::vector<int> devices;  // worker w runs on devices[w % devices.size()]
    int nworkers = 1;
    int64_t cap = 0, share = 0;  // cap per device; share = a worker's part of its device's cap
    int max_batch = 1;
    double bytes_per_voxel = 640.0;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::vector<std::unique_ptr<std::mutex>> thin_locks;  // one per device
    std::deque<Request*> pending;
    std::unordered_map<int64_t, std::unique_ptr<Request>> reqs;
    int64_t next_id = 1;
    bool stop = false;
    std::vector<vc_ctx*> ctxs;
    std::vector<std::thread> threads;
    vc_server_stats stats{};
    int64_t fail_alloc_after = -1;  // failure injection for the next batch taken (-1: off)
};

extern "C" int vc_plan_batches(int n, const int64_t* voxels, const double* t, int64_t share_bytes,
                               double bytes_per_voxel, int max_batch, int32_t* batch_of) {
    // Consecutive requests (in arrival order) form one batch while they have
    // the same t, the batch holds fewer than max_batch requests and its
    // footprint estimate stays within the share.  A request alone above the
    // share gets batch -1 (refused).
    if (n < 0 || (n > 0 && (!voxels || !t || !batch_of)) || share_bytes <= 0 || bytes_per_voxel <= 0 ||
        max_batch <= 0)
        return VC_ERR_ARG;
    int32_t b = -1;
    int count = 0;
    double sum = 0.0, tb = 0.0;
    for (int i = 0; i < n; ++i) {
        const double e = bytes_per_voxel * (double)voxels[i];
        if (voxels[i] <= 0 || e > (double)share_bytes) {
            batch_of[i] = -1;
            continue;
        }
        if (b < 0 || count >= max_batch || t[i] != tb || sum + e > (double)share_bytes) {
            ++b;
            count = 0;
            sum = 0.0;
            tb = t[i];
        }
        batch_of[i] = b;
        ++count;
        sum += e;
    }
    return VC_OK;
}

namespace {

// Page-locked host staging that grows on demand (host <-> device copies at
// full link speed, asynchronous on the worker's stream).
struct Pinned {
    void* p = nullptr;
    size_t cap = 0;
    void* get(size_t bytes) {
        if (bytes <= cap) return p;
        if (p) cudaFreeHost(p);
        p = nullptr;
        cap = 0;
        if (cudaMallocHost(&p, bytes) != cudaSuccess) {
            cudaGetLastError();
            p = nullptr;
            return nullptr;
        }
        cap = bytes;
        return p;
    }
    ~Pinned() {
        if (p) cudaFreeHost(p);
    }
};

struct Staging {
    Pinned occ, vts, edges, tris;
};

// One batch on one worker context; fills every request's result.
void serve_batch(vc_server* s, vc_ctx* c, std::vector<Request*>& batch, Staging& stage) {
    const int n = (int)batch.size();
    std::vector<int32_t> dims(3 * (size_t)n);
    size_t total = 0;
    for (int i = 0; i < n; ++i) {
        dims[3 * i] = batch[i]->X;
        dims[3 * i + 1] = batch[i]->Y;
        dims[3 * i + 2] = batch[i]->Z;
        total += batch[i]->occ.size();
    }
    auto* occ = static_cast<uint8_t*>(stage.occ.get(total));
    std::vector<vc_batch_volume> out((size_t)n);
    int st = occ ? VC_OK : VC_ERR_OOM;
    if (st == VC_OK) {
        size_t off = 0;
        for (Request* r : batch) {
            std::memcpy(occ + off, r->occ.data(), r->occ.size());
            off += r->occ.size();
        }
        st = vc_batch_set_volumes(c, n, dims.data(), occ, VC_MEM_HOST);
    }
    if (st == VC_OK) st = vc_batch_run(c, batch[0]->t, 1, nullptr, out.data());
    float* vts = nullptr;
    int32_t *edges = nullptr, *tris = nullptr;
    if (st == VC_OK) {
        int64_t nv = 0, ne = 0, nt = 0;
        for (const auto& o : out) {
            nv += o.rem.nv;
            ne += o.rem.ne;
            nt += o.rem.nt;
        }
        vts = static_cast<float*>(stage.vts.get(12 * (size_t)nv + 4));
        edges = static_cast<int32_t*>(stage.edges.get(8 * (size_t)ne + 4));
        tris = static_cast<int32_t*>(stage.tris.get(12 * (size_t)nt + 4));
        st = (vts && edges && tris) ? vc_get_remaining(c, vts, edges, tris, VC_MEM_HOST) : VC_ERR_OOM;
    }
    const double t_done = now_s();
    {
        std::lock_guard<std::mutex> lk(s->mu);
        for (int i = 0; i < n; ++i) {
            Request* r = batch[i];
            vc_request_result& q = r->res;
            q.status = st;
            q.batch_size = n;
            if (st == VC_OK) {
                const vc_batch_volume& o = out[i];
                q.n_sites = o.n_sites;
                q.vd = o.vd;
                q.thresh = o.thresh;
                q.rem = o.rem;
                q.euler = o.euler;
                r->vts.assign(vts + 3 * o.rem_v_off, vts + 3 * (o.rem_v_off + o.rem.nv));
                r->edges.assign(edges + 2 * o.rem_e_off, edges + 2 * (o.rem_e_off + o.rem.ne));
                r->tris.assign(tris + 3 * o.rem_t_off, tris + 3 * (o.rem_t_off + o.rem.nt));
            }
            r->t_done = t_done;
            q.queue_ms = (r->t_start - r->t_submit) * 1e3;
            q.run_ms = (t_done - r->t_start) * 1e3;
            q.latency_ms = (t_done - r->t_submit) * 1e3;
            r->done = true;
            std::vector<uint8_t>().swap(r->occ);
        }
        s->stats.batches += 1;
        s->stats.completed += n;
        if (st != VC_OK) s->stats.failed += n;
    }
    s->cv_done.notify_all();
}

void worker_main(vc_server* s, int w) {
    vc_ctx* c = s->ctxs[w];
    cudaSetDevice(c->device);
    Staging stage;
    for (;;) {
        std::vector<Request*> batch;
        {
            std::unique_lock<std::mutex> lk(s->mu);
            s->cv_work.wait(lk, [&] { return s->stop || !s->pending.empty(); });
            if (s->stop && s->pending.empty()) return;
            // the oldest pending requests that form one batch (vc_plan_batches)
            int64_t sum = 0;
            const double t0 = s->pending.front()->t;
            while (!s->pending.empty() && (int)batch.size() < s->max_batch) {
                Request* r = s->pending.front();
                if (r->t != t0 || (!batch.empty() && sum + r->est > s->share)) break;
                batch.push_back(r);
                sum += r->est;
                s->pending.pop_front();
            }
            const double ts = now_s();
            for (Request* r : batch) r->t_start = ts;
            if (!s->pending.empty()) s->cv_work.notify_one();
            if (s->fail_alloc_after >= 0) {  // armed for this batch only
                c->fail_alloc_after = s->fail_alloc_after;
                s->fail_alloc_after = -1;
            }
        }
        try {
            serve_batch(s, c, batch, stage);
        } catch (...) {  // host allocation failure: the batch fails, the worker goes on
            std::lock_guard<std::mutex> lk(s->mu);
            for (Request* r : batch) {
                r->res.status = VC_ERR_OOM;
                r->done = true;
            }
            s->stats.failed += (int64_t)batch.size();
            s->cv_done.notify_all();
        }
        c->fail_alloc_after = -1;
        if (vc_ctx_device_bytes(c) > s->share) vc::ctx_release_buffers(c);
    }
}

}  // namespace

extern "C" {

int vc_server_create_devices(vc_server** out, const int* devices, int ndev, int workers_per_device,
                             int64_t mem_cap_per_device, int max_batch) {
    if (!out || !devices || ndev <= 0 || ndev > 64 || workers_per_device <= 0 || workers_per_device > 16 ||
        mem_cap_per_device <= 0 || max_batch <= 0)
        return VC_ERR_ARG;
    *out = nullptr;
    auto s = std::make_unique<vc_server>();
    s->devices.assign(devices, devices + ndev);
    s->nworkers = ndev * workers_per_device;
    s->cap = mem_cap_per_device;
    s->share = mem_cap_per_device / workers_per_device;
    s->max_batch = max_batch;
    for (int d = 0; d < ndev; ++d) s->thin_locks.push_back(std::make_unique<std::mutex>());
    for (int w = 0; w < s->nworkers; ++w) {
        vc_ctx* c = nullptr;
        const int st = vc_ctx_create(&c, devices[w % ndev]);
        if (st != VC_OK) {
            for (vc_ctx* x : s->ctxs) vc_ctx_destroy(x);
            return st;
        }
        // the persistent thinning kernels of one device's workers each take
        // the whole GPU, one at a time; their other stages overlap freely
        c->thin_lock = s->thin_locks[w % ndev].get();
        s->ctxs.push_back(c);
    }
    vc_server* raw = s.release();
    for (int w = 0; w < raw->nworkers; ++w) raw->threads.emplace_back(worker_main, raw, w);
    *out = raw;
    return VC_OK;
}

int vc_server_create(vc_server** out, int device, int workers, int64_t mem_cap_bytes, int max_batch) {
    return vc_server_create_devices(out, &device, 1, workers, mem_cap_bytes, max_batch);
}

int vc_partition_volumes(int n, const int64_t* voxels, int nparts, int32_t* part_of) {
    // Whole volumes to parts (devices or ranks), largest first, each to the
    // part with the fewest voxels so far (the lowest part on ties).  Volumes
    // are independent, so every part runs its share as one batch and the
    // union of the parts' results is the result of the whole set.
    if (n < 0 || nparts <= 0 || (n > 0 && (!voxels || !part_of))) return VC_ERR_ARG;
    std::vector<int> order((size_t)n);
    for (int i = 0; i < n; ++i) {
        if (voxels[i] < 0) return VC_ERR_ARG;
        order[(size_t)i] = i;
    }
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return voxels[a] > voxels[b]; });
    std::vector<int64_t> load((size_t)nparts, 0);
    for (const int i : order) {
        int best = 0;
        for (int p = 1; p < nparts; ++p)
            if (load[(size_t)p] < load[(size_t)best]) best = p;
        part_of[i] = best;
        load[(size_t)best] += voxels[i];
    }
    return VC_OK;
}

int vc_server_set_bytes_per_voxel(vc_server* s, double bytes_per_voxel) {
    if (!s || !(bytes_per_voxel > 0)) return VC_ERR_ARG;
    std::lock_guard<std::mutex> lk(s->mu);
    s->bytes_per_voxel = bytes_per_voxel;
    return VC_OK;
}

int vc_server_submit(vc_server* s, const uint8_t* occ, int X, int Y, int Z, double t, int64_t* id) {
    if (!s || !occ || !id || X <= 0 || Y <= 0 || Z <= 0 || X > 32766 || Y > 32766 || Z > 32766) return VC_ERR_ARG;
    const int64_t nvox = (int64_t)X * Y * Z;
    auto r = std::make_unique<Request>();
    r->X = X;
    r->Y = Y;
    r->Z = Z;
    r->t = t;
    r->occ.assign(occ, occ + nvox);
    std::lock_guard<std::mutex> lk(s->mu);
    r->est = (int64_t)(s->bytes_per_voxel * (double)nvox);
    if (r->est > s->share) {
        s->stats.refused += 1;
        return VC_ERR_ARG;  // cannot fit one worker's share of the memory cap
    }
    r->id = s->next_id++;
    r->t_submit = now_s();
    *id = r->id;
    s->pending.push_back(r.get());
    s->reqs.emplace(r->id, std::move(r));
    s->stats.submitted += 1;
    s->cv_work.notify_one();
    return VC_OK;
}

int vc_server_wait(vc_server* s, int64_t id, double timeout_s, vc_request_result* out) {
    if (!s || !out) return VC_ERR_ARG;
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->reqs.find(id);
    if (it == s->reqs.end()) return VC_ERR_ARG;
    Request* r = it->second.get();
    const auto pred = [&] { return r->done; };
    if (timeout_s < 0) s->cv_done.wait(lk, pred);
    else if (!s->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), pred)) return VC_ERR_TIMEOUT;
    *out = r->res;
    return VC_OK;
}

int vc_server_get_remaining(vc_server* s, int64_t id, float* vts, int32_t* edges, int32_t* tris) {
    if (!s) return VC_ERR_ARG;
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->reqs.find(id);
    if (it == s->reqs.end()) return VC_ERR_ARG;
    Request* r = it->second.get();
    if (!r->done) return VC_ERR_STATE;
    if (r->res.status != VC_OK) return r->res.status;
    if (vts && !r->vts.empty()) std::memcpy(vts, r->vts.data(), r->vts.size() * sizeof(float));
    if (edges && !r->edges.empty()) std::memcpy(edges, r->edges.data(), r->edges.size() * sizeof(int32_t));
    if (tris && !r->tris.empty()) std::memcpy(tris, r->tris.data(), r->tris.size() * sizeof(int32_t));
    return VC_OK;
}

int vc_server_release(vc_server* s, int64_t id) {
    if (!s) return VC_ERR_ARG;
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->reqs.find(id);
    if (it == s->reqs.end()) return VC_ERR_ARG;
    if (!it->second->done) return VC_ERR_STATE;
    s->reqs.erase(it);
    return VC_OK;
}

int vc_server_get_stats(vc_server* s, vc_server_stats* out) {
    if (!s || !out) return VC_ERR_ARG;
    std::lock_guard<std::mutex> lk(s->mu);
    *out = s->stats;
    out->pending = (int64_t)s->pending.size();
    out->device_bytes = 0;
    for (vc_ctx* c : s->ctxs) out->device_bytes += vc_ctx_device_bytes(c);
    return VC_OK;
}

int vc_server_debug_fail_alloc_after(vc_server* s, int64_t k) {
    if (!s) return VC_ERR_ARG;
    std::lock_guard<std::mutex> lk(s->mu);
    s->fail_alloc_after = k < 0 ? -1 : k;
    return VC_OK;
}

int vc_server_destroy(vc_server* s) {
    if (!s) return VC_OK;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
    }
    s->cv_work.notify_all();
    for (auto& th : s->threads) th.join();
    for (vc_ctx* c : s->ctxs) vc_ctx_destroy(c);
    delete s;
    return VC_OK;
}

}  // extern "C"
