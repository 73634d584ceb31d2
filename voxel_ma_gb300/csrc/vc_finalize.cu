// cellcomplex construction and finalize() on the GPU
// (src/cellcomplex.cpp:13-26, 364-491).
//
// Edge ids: the given edges keep their order (a repeated ordered pair keeps
// its first index), then every face side (made with util::makeEdge,
// smaller id first) that is not yet an edge is appended in face order.  The
// reference does this with a hash map; here all keys (given edges first,
// then 3 sides per face) go into a device hash table that keeps, per key, the
// smallest position at which the key occurs.  A position is a "first
// occurrence" iff it holds that minimum, and an exclusive scan over the
// first-occurrence flags in position order yields exactly the reference's
// edge ids.
// Adjacency: V->E lists hold edge ids in increasing order (each edge appended
// to both ends in id order); E->F lists hold face ids in increasing order.
// They are filled with atomics and then each short list is sorted.
#include "vc_internal.cuh"

namespace vc {
namespace {

constexpr unsigned long long kEmpty = ~0ull;

__device__ __forceinline__ unsigned long long key_of(int32_t a, int32_t b) {
    return ((unsigned long long)(uint32_t)a << 32) | (uint32_t)b;
}
__device__ __forceinline__ unsigned long long hash64(unsigned long long k) {
    k ^= k >> 33;
    k *= 0xff51afd7ed558ccdull;
    k ^= k >> 33;
    k *= 0xc4ceb9fe1a85ec53ull;
    k ^= k >> 33;
    return k;
}

// Validate the input complex: ids in range, no loop edge, no triangle with a
// repeated vertex.
__global__ void validate_kernel(const int2* __restrict__ edges, int64_t ne, const int32_t* __restrict__ tris,
                                int64_t nt, int64_t nv, int* err) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < ne + nt; i += stride) {
        if (i < ne) {
            int2 e = edges[i];
            if (e.x < 0 || e.y < 0 || e.x >= nv || e.y >= nv || e.x == e.y) set_error(err, VC_ERR_ARG);
        } else {
            const int64_t f = i - ne;
            int32_t a = tris[3 * f], b = tris[3 * f + 1], c = tris[3 * f + 2];
            if (a < 0 || b < 0 || c < 0 || a >= nv || b >= nv || c >= nv || a == b || b == c || a == c)
                set_error(err, VC_ERR_ARG);
        }
    }
}

__device__ __forceinline__ unsigned long long key_at(const int2* edges, int64_t ne, const int32_t* tris, int64_t pos) {
    if (pos < ne) {
        int2 e = edges[pos];
        return key_of(e.x, e.y);
    }
    const int64_t j = pos - ne, f = j / 3;
    const int s = (int)(j % 3);
    const int32_t u = tris[3 * f + s], v = tris[3 * f + (s + 1) % 3];
    return u < v ? key_of(u, v) : key_of(v, u);
}

__global__ void hash_insert_kernel(const int2* __restrict__ edges, int64_t ne, const int32_t* __restrict__ tris,
                                   int64_t nt, unsigned long long* __restrict__ keys, int64_t* __restrict__ minpos,
                                   int64_t* __restrict__ slot_of, unsigned long long mask, int* err) {
    const int64_t n = ne + 3 * nt;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t pos = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; pos < n; pos += stride) {
        const unsigned long long k = key_at(edges, ne, tris, pos);
        unsigned long long h = hash64(k) & mask;
        bool done = false;
        for (unsigned long long probe = 0; probe <= mask; ++probe) {
            unsigned long long prev = atomicCAS(&keys[h], kEmpty, k);
            if (prev == kEmpty || prev == k) {
                atomicMin((unsigned long long*)&minpos[h], (unsigned long long)pos);
                slot_of[pos] = (int64_t)h;
                done = true;
                break;
            }
            h = (h + 1) & mask;
        }
        if (!done) set_error(err, VC_ERR_OOM);
    }
}

__global__ void first_flags_kernel(const int64_t* __restrict__ slot_of, const int64_t* __restrict__ minpos,
                                   int32_t* __restrict__ first, int64_t n) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t pos = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; pos < n; pos += stride)
        first[pos] = minpos[slot_of[pos]] == pos ? 1 : 0;
}

__global__ void assign_ids_kernel(const int2* __restrict__ edges, int64_t ne, const int32_t* __restrict__ tris,
                                  const int64_t* __restrict__ slot_of, const int64_t* __restrict__ minpos,
                                  const int32_t* __restrict__ rank, int32_t* __restrict__ slot_id,
                                  int2* __restrict__ edges_out, int64_t n) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t pos = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; pos < n; pos += stride) {
        const int64_t s = slot_of[pos];
        if (minpos[s] != pos) continue;
        const int32_t id = rank[pos];
        slot_id[s] = id;
        const unsigned long long k = key_at(edges, ne, tris, pos);
        edges_out[id] = make_int2((int32_t)(k >> 32), (int32_t)(k & 0xffffffffull));
    }
}

__global__ void side_ids_kernel(const int64_t* __restrict__ slot_of, const int32_t* __restrict__ slot_id,
                                int32_t* __restrict__ tri_edges, int64_t ne, int64_t nsides) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < nsides; j += stride)
        tri_edges[j] = slot_id[slot_of[ne + j]];
}

// ---- adjacency --------------------------------------------------------------
__global__ void ve_count_kernel(const int2* __restrict__ edges, int64_t ne, int32_t* __restrict__ cnt) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < ne; e += stride) {
        int2 v = edges[e];
        atomicAdd(&cnt[v.x], 1);
        atomicAdd(&cnt[v.y], 1);
    }
}
__global__ void ve_fill_kernel(const int2* __restrict__ edges, int64_t ne, int32_t* __restrict__ cur,
                               int32_t* __restrict__ ids) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < ne; e += stride) {
        int2 v = edges[e];
        ids[atomicAdd(&cur[v.x], 1)] = (int32_t)e;
        ids[atomicAdd(&cur[v.y], 1)] = (int32_t)e;
    }
}
__global__ void ef_count_kernel(const int32_t* __restrict__ tri_edges, int64_t nsides, int32_t* __restrict__ cnt) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < nsides; j += stride)
        atomicAdd(&cnt[tri_edges[j]], 1);
}
__global__ void ef_fill_kernel(const int32_t* __restrict__ tri_edges, int64_t nsides, int32_t* __restrict__ cur,
                               int32_t* __restrict__ ids) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < nsides; j += stride)
        ids[atomicAdd(&cur[tri_edges[j]], 1)] = (int32_t)(j / 3);
}
// Sort every list ids[off[i] .. off[i+1]) ascending (lists are short).
__global__ void sort_segments_kernel(const int32_t* __restrict__ off, int32_t* __restrict__ ids, int64_t n) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const int32_t b = off[i], e = off[i + 1];
        for (int32_t x = b + 1; x < e; ++x) {
            const int32_t v = ids[x];
            int32_t y = x - 1;
            while (y >= b && ids[y] > v) {
                ids[y + 1] = ids[y];
                --y;
            }
            ids[y + 1] = v;
        }
    }
}

inline int grid_for(vc_ctx* c, int64_t n, int threads) {
    int64_t b = (n + threads - 1) / threads;
    return (int)std::max<int64_t>(1, std::min<int64_t>(b, (int64_t)c->num_sms * 16));
}

}  // namespace

// Build V->E and E->F lists of the context's finalized edges / tri_edges.
int build_adjacency(vc_ctx* c) {
    const int64_t nv = c->nv, ne = c->ne, nt = c->nt;
    if (2 * ne >= INT32_MAX || 3 * nt >= INT32_MAX) return VC_ERR_ARG;  // 32-bit list offsets
    Region stage(c, "adjacency");
    VC_TRY(ensure_n<int32_t>(c, c->ve_off, nv + 1));
    VC_TRY(ensure_n<int32_t>(c, c->ve_ids, 2 * ne));
    VC_TRY(ensure_n<int32_t>(c, c->ef_off, ne + 1));
    VC_TRY(ensure_n<int32_t>(c, c->ef_ids, 3 * nt));
    VC_TRY(ensure_n<int32_t>(c, c->hash_id, std::max(nv, ne) + 1));  // cursor scratch
    int32_t* cur = ptr<int32_t>(c->hash_id);
    const int2* edges = ptr<int2>(c->edges);
    const int32_t* te = ptr<int32_t>(c->tri_edges);
    // V->E
    int32_t* ve_off = ptr<int32_t>(c->ve_off);
    VC_CUDA(c, cudaMemsetAsync(ve_off, 0, (nv + 1) * sizeof(int32_t), c->stream));
    if (ne > 0) {
        ve_count_kernel<<<grid_for(c, ne, 256), 256, 0, c->stream>>>(edges, ne, ve_off);
        launched(c);
    }
    VC_TRY(scan_exclusive_i32(c, ve_off, ve_off, nv + 1, nullptr));
    VC_CUDA(c, cudaMemcpyAsync(cur, ve_off, (nv + 1) * sizeof(int32_t), cudaMemcpyDeviceToDevice, c->stream));
    if (ne > 0) {
        ve_fill_kernel<<<grid_for(c, ne, 256), 256, 0, c->stream>>>(edges, ne, cur, ptr<int32_t>(c->ve_ids));
        launched(c);
    }
    if (nv > 0) {
        sort_segments_kernel<<<grid_for(c, nv, 256), 256, 0, c->stream>>>(ve_off, ptr<int32_t>(c->ve_ids), nv);
        launched(c);
    }
    // E->F
    int32_t* ef_off = ptr<int32_t>(c->ef_off);
    VC_CUDA(c, cudaMemsetAsync(ef_off, 0, (ne + 1) * sizeof(int32_t), c->stream));
    if (nt > 0) {
        ef_count_kernel<<<grid_for(c, 3 * nt, 256), 256, 0, c->stream>>>(te, 3 * nt, ef_off);
        launched(c);
    }
    VC_TRY(scan_exclusive_i32(c, ef_off, ef_off, ne + 1, nullptr));
    VC_CUDA(c, cudaMemcpyAsync(cur, ef_off, (ne + 1) * sizeof(int32_t), cudaMemcpyDeviceToDevice, c->stream));
    if (nt > 0) {
        ef_fill_kernel<<<grid_for(c, 3 * nt, 256), 256, 0, c->stream>>>(te, 3 * nt, cur, ptr<int32_t>(c->ef_ids));
        launched(c);
    }
    if (ne > 0) {
        sort_segments_kernel<<<grid_for(c, ne, 256), 256, 0, c->stream>>>(ef_off, ptr<int32_t>(c->ef_ids), ne);
        launched(c);
    }
    VC_CUDA(c, cudaGetLastError());
    return VC_OK;
}

int run_finalize(vc_ctx* c, int64_t* ne_final) {
    if (!c->cc_valid) return VC_ERR_STATE;
    if (c->cc_finalized) {
        if (ne_final) *ne_final = c->ne;
        return VC_OK;
    }
    const int64_t ne = c->ne_in, nt = c->nt, nv = c->nv;
    const int64_t n = ne + 3 * nt;
    validate_kernel<<<grid_for(c, ne + nt, 256), 256, 0, c->stream>>>(ptr<int2>(c->edges_in), ne,
                                                                       ptr<int32_t>(c->tris), nt, nv, dev_err(c));
    launched(c);
    VC_TRY(sync_check(c));
    unsigned long long cap = 1024;
    while (cap < (unsigned long long)(2 * n)) cap <<= 1;
    VC_TRY(ensure_n<unsigned long long>(c, c->hash_keys, (int64_t)cap));
    VC_TRY(ensure_n<int64_t>(c, c->hash_pos, (int64_t)cap));
    VC_TRY(ensure_n<int32_t>(c, c->hash_id, (int64_t)cap));
    VC_TRY(ensure_n<int64_t>(c, c->side_slot, n));
    VC_TRY(ensure_n<int32_t>(c, c->scratch2, n + 2));  // first-occurrence flags -> ranks
    VC_TRY(ensure_n<int64_t>(c, c->euler_tmp, 2));
    auto* keys = ptr<unsigned long long>(c->hash_keys);
    auto* minpos = ptr<int64_t>(c->hash_pos);
    VC_CUDA(c, cudaMemsetAsync(keys, 0xff, cap * sizeof(unsigned long long), c->stream));
    VC_CUDA(c, cudaMemsetAsync(minpos, 0x7f, cap * sizeof(int64_t), c->stream));
    int64_t* slot_of = ptr<int64_t>(c->side_slot);
    if (n > 0) {
        hash_insert_kernel<<<grid_for(c, n, 256), 256, 0, c->stream>>>(ptr<int2>(c->edges_in), ne,
                                                                        ptr<int32_t>(c->tris), nt, keys, minpos,
                                                                        slot_of, cap - 1, dev_err(c));
        launched(c);
    }
    int32_t* rank = ptr<int32_t>(c->scratch2);
    if (n > 0) {
        first_flags_kernel<<<grid_for(c, n, 256), 256, 0, c->stream>>>(slot_of, minpos, rank, n);
        launched(c);
    }
    int64_t* total = ptr<int64_t>(c->euler_tmp);
    VC_TRY(scan_exclusive_i32(c, rank, rank, n, total));
    int64_t ne_out = 0;
    VC_TRY(read_i64(c, total, &ne_out));
    if (ne_out >= INT32_MAX) return VC_ERR_ARG;
    VC_TRY(ensure_n<int2>(c, c->edges, ne_out));
    VC_TRY(ensure_n<int32_t>(c, c->tri_edges, 3 * nt));
    int32_t* slot_id = ptr<int32_t>(c->hash_id);
    if (n > 0) {
        assign_ids_kernel<<<grid_for(c, n, 256), 256, 0, c->stream>>>(ptr<int2>(c->edges_in), ne,
                                                                       ptr<int32_t>(c->tris), slot_of, minpos, rank,
                                                                       slot_id, ptr<int2>(c->edges), n);
        launched(c);
    }
    if (nt > 0) {
        side_ids_kernel<<<grid_for(c, 3 * nt, 256), 256, 0, c->stream>>>(slot_of, slot_id,
                                                                          ptr<int32_t>(c->tri_edges), ne, 3 * nt);
        launched(c);
    }
    VC_CUDA(c, cudaGetLastError());
    c->ne = ne_out;
    VC_TRY(build_adjacency(c));
    VC_TRY(sync_check(c));
    c->cc_finalized = true;
    if (ne_final) *ne_final = ne_out;
    return VC_OK;
}

}  // namespace vc
