// Remaining complex after thinning (replaces CellComplexThinning::remainingCC,
// src/ccthin.cpp:467-512) and its Euler characteristic / component count
// (util::computeEulerChar(vts, edges, tris), src/geomalgo.cpp:181-214).
//
// remainingCC keeps, in id order, the vertices not removed, the edges not
// removed and referenced by no remaining face, and the faces not removed;
// each surviving triangle (a,b,c) goes through util::simpleTriangulate, which
// returns (c,a,b); util::compactify then renames vertex ids in the order the
// vertices were kept.  computeEulerChar counts the given edges together with
// the triangles' sides as a set (every one of them is a finalized edge of the
// thinned complex, so the set is the set of their edge ids), all given
// vertices, and the connected components of that edge set.
#include "vc_internal.cuh"

namespace vc {
namespace {


// Per-volume starts of the remaining complex (batches): the survivors before
// each volume's first vertex, edge and triangle.
__global__ void rem_bases_kernel(Bases B, int nvol, int32_t nv, int32_t ne, int32_t nt, Kept K,
                                 const int64_t* __restrict__ tot) {
    for (int b = blockIdx.x * blockDim.x + threadIdx.x; b <= nvol; b += gridDim.x * blockDim.x) {
        const int64_t v0 = B.b[kBVert][b], e0 = B.b[kBAxis][b] + B.b[kBFace][b], t0 = 2 * B.b[kBFace][b];
        B.b[kBRemV][b] = v0 < nv ? kept_rank(K.bv, K.pv, v0) : tot[0];
        B.b[kBRemE][b] = e0 < ne ? kept_rank(K.be, K.pe, e0) : tot[1];
        B.b[kBRemT][b] = t0 < nt ? kept_rank(K.bf, K.pf, t0) : tot[2];
    }
}

// One warp per 32 cells of a kind: the survivors at their kept ranks.  In a
// batch (nmap > 1) vertex ids are made local to each volume's remaining
// complex.
__global__ void rem_write_kernel(int32_t nv, int32_t ne, int32_t nt, Kept K, const float* __restrict__ vts,
                                 const int2* __restrict__ edges, const int32_t* __restrict__ tris,
                                 float* __restrict__ ovts, int2* __restrict__ oedges, int32_t* __restrict__ otris,
                                 Bases B, int nmap) {
    const int lane = threadIdx.x & 31;
    const uint32_t lowm = (1u << lane) - 1u;
    const int64_t nwv = ((int64_t)nv + 31) / 32, nwe = ((int64_t)ne + 31) / 32, nwf = ((int64_t)nt + 31) / 32;
    const int64_t nw = nwv + nwe + nwf;
    const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
    for (int64_t w = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); w < nw; w += warps) {
        if (w < nwv) {
            const uint32_t word = __ldg(K.bv + w);
            if (!((word >> lane) & 1u)) continue;
            const int64_t i = w * 32 + lane;
            const int64_t o = __ldg(K.pv + w) + __popc(word & lowm);
            ovts[3 * o + 0] = vts[3 * i + 0];
            ovts[3 * o + 1] = vts[3 * i + 1];
            ovts[3 * o + 2] = vts[3 * i + 2];
        } else if (w < nwv + nwe) {
            const int64_t we = w - nwv;
            const uint32_t word = __ldg(K.be + we);
            if (!((word >> lane) & 1u)) continue;
            const int64_t e = we * 32 + lane;
            const int2 ev = edges[e];
            const int32_t sh = nmap > 1 ? (int32_t)B.b[kBRemV][find_base(B.b[kBVert], nmap, ev.x)] : 0;
            oedges[__ldg(K.pe + we) + __popc(word & lowm)] =
                make_int2(kept_rank(K.bv, K.pv, ev.x) - sh, kept_rank(K.bv, K.pv, ev.y) - sh);
        } else {
            const int64_t wf = w - nwv - nwe;
            const uint32_t word = __ldg(K.bf + wf);
            if (!((word >> lane) & 1u)) continue;
            const int64_t f = wf * 32 + lane;
            const int64_t o = __ldg(K.pf + wf) + __popc(word & lowm);
            const int32_t t0 = tris[3 * f], t1 = tris[3 * f + 1], t2 = tris[3 * f + 2];
            const int32_t sh = nmap > 1 ? (int32_t)B.b[kBRemV][find_base(B.b[kBVert], nmap, t0)] : 0;
            otris[3 * o + 0] = kept_rank(K.bv, K.pv, t2) - sh;
            otris[3 * o + 1] = kept_rank(K.bv, K.pv, t0) - sh;
            otris[3 * o + 2] = kept_rank(K.bv, K.pv, t1) - sh;
        }
    }
}

// Euler: mark every finalized edge that is a remaining edge or a side of a
// remaining face (the sides are read from the thinning's face records).
__global__ void euler_mark_kernel(const uint8_t* __restrict__ ke, const uint8_t* __restrict__ kf,
                                  const FaceRec* __restrict__ F, int32_t ne, int32_t nt, int32_t* __restrict__ mark) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < (int64_t)ne + nt; i += stride) {
        if (i < ne) {
            if (ke[i]) mark[i] = 1;
        } else {
            const int64_t f = i - ne;
            if (!kf[f]) continue;
            const int4 sides = __ldg(reinterpret_cast<const int4*>(F + f));
            mark[sides.x] = 1;
            mark[sides.y] = 1;
            mark[sides.z & ~kFacePass] = 1;
        }
    }
}

__device__ __forceinline__ int32_t uf_find(int32_t* parent, int32_t x) {
    int32_t p = __ldcg(parent + x);
    while (p != x) {
        const int32_t gp = __ldcg(parent + p);
        if (gp != p) parent[x] = gp;  // path halving (benign race)
        x = p;
        p = gp;
    }
    return x;
}

// Join the sets of a and b (the smaller root becomes the root); false when
// the bounded retries ran out.
__device__ __forceinline__ bool uf_join(int32_t* parent, int32_t a, int32_t b) {
    for (int it = 0; it < (1 << 20); ++it) {
        a = uf_find(parent, a);
        b = uf_find(parent, b);
        if (a == b) return true;
        if (a > b) {
            const int32_t t = a;
            a = b;
            b = t;
        }
        if (atomicCAS(&parent[b], b, a) == b) return true;
    }
    return false;
}

__global__ void uf_init_kernel(int32_t* parent, int32_t n) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) parent[i] = (int32_t)i;
}

__global__ void uf_union_kernel(const int32_t* __restrict__ mark, const EdgeHead* __restrict__ E, Kept K, int32_t ne,
                                int32_t* parent, int* err) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < ne; e += stride) {
        if (!mark[e]) continue;
        const int2 ev = *reinterpret_cast<const int2*>(E + e);  // the record's ends v0, v1
        if (!uf_join(parent, kept_rank(K.bv, K.pv, ev.x), kept_rank(K.bv, K.pv, ev.y))) set_error(err, VC_ERR_TIMEOUT);
    }
}

// Components: roots of the union-find forest, per volume in a batch
// (remaining vertex -> volume through the remaining-complex vertex starts).
__global__ void uf_roots_kernel(int32_t* parent, int32_t n, unsigned long long* roots, Bases B, int nmap) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    unsigned long long local = 0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        if (uf_find(parent, (int32_t)i) != i) continue;
        if (nmap > 1) atomicAdd(roots + find_base(B.b[kBRemV], nmap, i), 1ull);
        else ++local;
    }
    if (local) atomicAdd(roots, local);
}

// Marked edges, per volume in a batch (edge -> volume through its vertex).
__global__ void count_kernel(const int32_t* __restrict__ mark, const EdgeHead* __restrict__ E, int64_t n,
                             unsigned long long* cnt, Bases B, int nmap) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    unsigned long long local = 0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        if (mark[i] == 0) continue;
        if (nmap > 1) atomicAdd(cnt + find_base(B.b[kBVert], nmap, E[i].v0), 1ull);
        else ++local;
    }
    if (local) atomicAdd(cnt, local);
}

// Closed components: the remaining faces joined through their sides (node f
// for face f, node nt + e for edge e), then one count per set holding a face.
__global__ void cc_join_kernel(const uint8_t* __restrict__ kf, const FaceRec* __restrict__ F, int32_t nt,
                               int32_t* parent, int* err) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t f = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; f < nt; f += stride) {
        if (!kf[f]) continue;
        const int4 r = __ldg(reinterpret_cast<const int4*>(F + f));  // e0 e1 e2|pass rm
        const int32_t side[3] = {r.x, r.y, r.z & ~kFacePass};
#pragma unroll
        for (int k = 0; k < 3; ++k)
            if (!uf_join(parent, (int32_t)f, nt + side[k])) set_error(err, VC_ERR_TIMEOUT);
    }
}

__global__ void cc_count_kernel(const uint8_t* __restrict__ kf, int32_t* parent, int32_t nt, int32_t* seen,
                                unsigned long long* count) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    unsigned long long local = 0;
    for (int64_t f = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; f < nt; f += stride) {
        if (!kf[f]) continue;
        if (atomicExch(seen + uf_find(parent, (int32_t)f), 1) == 0) ++local;
    }
    if (local) atomicAdd(count, local);
}

inline int grid_for(vc_ctx* c, int64_t n, int threads) {
    int64_t b = (n + threads - 1) / threads;
    return (int)std::max<int64_t>(1, std::min<int64_t>(b, (int64_t)c->num_sms * 16));
}

}  // namespace

Kept kept_of(vc_ctx* c) {
    const int64_t nwv = (c->nv + 31) / 32, nwe = (c->ne + 31) / 32;
    const uint32_t* bits = ptr<uint32_t>(c->keep_bits);
    return Kept{bits, bits + nwv, bits + nwv + nwe, ptr<int32_t>(c->keep_wv), ptr<int32_t>(c->keep_we),
                ptr<int32_t>(c->keep_wf)};
}

int lattice_rem_write(vc_ctx* c, const Kept& K, int nmap);

int run_remaining(vc_ctx* c, vc_rem_sizes* sizes) {
    if (!c->thin_valid) return VC_ERR_STATE;
    if (c->rem_valid) {  // this thinning's remaining complex is built already (the word scans below are in place)
        if (sizes) *sizes = c->rem;
        return VC_OK;
    }
    const int64_t nv = c->nv, ne = c->ne, nt = c->nt;
    const int64_t nwv = (nv + 31) / 32, nwe = (ne + 31) / 32, nwf = (nt + 31) / 32;
    VC_TRY(ensure_n<int64_t>(c, c->scratch2, 4));
    Region stage(c, "stage_remaining");
    // the thinning left the survivors as bit words with per-word counts
    int64_t* tot = ptr<int64_t>(c->scratch2);
    VC_TRY(scan_exclusive_i32(c, ptr<int32_t>(c->keep_wv), ptr<int32_t>(c->keep_wv), nwv, tot + 0));
    VC_TRY(scan_exclusive_i32(c, ptr<int32_t>(c->keep_we), ptr<int32_t>(c->keep_we), nwe, tot + 1));
    VC_TRY(scan_exclusive_i32(c, ptr<int32_t>(c->keep_wf), ptr<int32_t>(c->keep_wf), nwf, tot + 2));
    const Kept K = kept_of(c);
    const int nmap = c->cc_batched ? c->nvol : 1;
    if (nmap > 1) {
        rem_bases_kernel<<<(nmap + 256) / 256, 256, 0, c->stream>>>(c->bases, nmap, (int32_t)nv, (int32_t)ne,
                                                                    (int32_t)nt, K, tot);
        launched(c);
        c->h_rem_bases.resize(3 * ((size_t)nmap + 1));
        for (int k = 0; k < 3; ++k)
            VC_CUDA(c, cudaMemcpyAsync(c->h_rem_bases.data() + k * ((size_t)nmap + 1), c->bases.b[kBRemV + k],
                                       ((size_t)nmap + 1) * sizeof(int64_t), cudaMemcpyDeviceToHost, c->stream));
    }
    int64_t h[3] = {0, 0, 0};
    VC_CUDA(c, cudaMemcpyAsync(h, tot, 3 * sizeof(int64_t), cudaMemcpyDeviceToHost, c->stream));
    VC_TRY(sync_check(c));
    VC_TRY(ensure_n<float>(c, c->rem_vts, 3 * h[0]));
    VC_TRY(ensure_n<int2>(c, c->rem_edges, h[1]));
    VC_TRY(ensure_n<int32_t>(c, c->rem_tris, 3 * h[2]));
    if (c->vd_valid && !c->vd_geom) {
        // the lattice complex of the timed path keeps no vertex, edge or
        // triangle arrays: the survivors come from the thinning records
        VC_TRY(lattice_rem_write(c, K, nmap));
    } else {
        rem_write_kernel<<<grid_for(c, 32 * (nwv + nwe + nwf), 256), 256, 0, c->stream>>>(
            (int32_t)nv, (int32_t)ne, (int32_t)nt, K, ptr<float>(c->vts), ptr<int2>(c->edges), ptr<int32_t>(c->tris),
            ptr<float>(c->rem_vts), ptr<int2>(c->rem_edges), ptr<int32_t>(c->rem_tris), c->bases, nmap);
        launched(c);
    }
    VC_CUDA(c, cudaGetLastError());
    c->rem = vc_rem_sizes{h[0], h[1], h[2]};
    c->rem_valid = true;
    if (sizes) *sizes = c->rem;
    return VC_OK;
}

int run_thin_all_pass(vc_ctx* c, vc_thin_stats* stats);

// nClosedComponents (highlevelalgo.cpp:993-1020): the thinning with every
// pair passing, then the face-connected components of the remaining faces
// (cellcomplex::compute_conn_cmpnts, cellcomplex.cpp:73-147).  The thinning
// flags of the context are this thinning's afterwards.
int run_closed_components(vc_ctx* c, int64_t* n) {
    if (c->nt + c->ne >= INT32_MAX) return VC_ERR_ARG;
    VC_TRY(run_thin_all_pass(c, nullptr));
    const int64_t ne = c->ne, nt = c->nt, nodes = nt + ne;
    *n = 0;
    if (nt == 0) return VC_OK;
    VC_TRY(ensure_n<int32_t>(c, c->uf_parent, nodes + 1));
    VC_TRY(ensure_n<int32_t>(c, c->scratch, nodes + 1));
    VC_TRY(ensure_n<int64_t>(c, c->scratch2, 2));
    int32_t* parent = ptr<int32_t>(c->uf_parent);
    int32_t* seen = ptr<int32_t>(c->scratch);
    auto* cnt = reinterpret_cast<unsigned long long*>(ptr<int64_t>(c->scratch2));
    VC_CUDA(c, cudaMemsetAsync(seen, 0, (size_t)nodes * sizeof(int32_t), c->stream));
    VC_CUDA(c, cudaMemsetAsync(cnt, 0, sizeof(unsigned long long), c->stream));
    uf_init_kernel<<<grid_for(c, nodes, 256), 256, 0, c->stream>>>(parent, (int32_t)nodes);
    cc_join_kernel<<<grid_for(c, nt, 256), 256, 0, c->stream>>>(ptr<uint8_t>(c->keep_f), ptr<FaceRec>(c->face_rec),
                                                                 (int32_t)nt, parent, dev_err(c));
    cc_count_kernel<<<grid_for(c, nt, 256), 256, 0, c->stream>>>(ptr<uint8_t>(c->keep_f), parent, (int32_t)nt, seen,
                                                                  cnt);
    launched(c, 3);
    VC_CUDA(c, cudaGetLastError());
    unsigned long long h = 0;
    VC_CUDA(c, cudaMemcpyAsync(&h, cnt, sizeof(h), cudaMemcpyDeviceToHost, c->stream));
    VC_TRY(sync_check(c));
    *n = (int64_t)h;
    return VC_OK;
}

int run_euler_remaining(vc_ctx* c, vc_euler_info* out) {
    if (!c->rem_valid) return VC_ERR_STATE;
    const int64_t ne = c->ne, nt = c->nt, nvr = c->rem.nv;
    VC_TRY(ensure_n<int32_t>(c, c->uf_parent, std::max<int64_t>(nvr, ne) + 1));
    VC_TRY(ensure_n<int32_t>(c, c->scratch, ne + 1));
    const int nmap = c->cc_batched ? c->nvol : 1;
    VC_TRY(ensure_n<int64_t>(c, c->scratch2, 2 * (int64_t)nmap + 2));
    int32_t* mark = ptr<int32_t>(c->scratch);
    // [0, nmap): marked edges per volume; [nmap, 2 nmap): components per volume
    auto* cnt = reinterpret_cast<unsigned long long*>(ptr<int64_t>(c->scratch2));
    VC_CUDA(c, cudaMemsetAsync(mark, 0, (ne + 1) * sizeof(int32_t), c->stream));
    VC_CUDA(c, cudaMemsetAsync(cnt, 0, 2 * (size_t)nmap * sizeof(unsigned long long), c->stream));
    euler_mark_kernel<<<grid_for(c, ne + nt, 256), 256, 0, c->stream>>>(
        ptr<uint8_t>(c->keep_e), ptr<uint8_t>(c->keep_f), ptr<FaceRec>(c->face_rec), (int32_t)ne, (int32_t)nt,
        mark);
    launched(c);
    // edge ends from the thinning records (the lattice complex of the timed
    // path keeps no edge array)
    count_kernel<<<grid_for(c, ne, 256), 256, 0, c->stream>>>(mark, ptr<EdgeHead>(c->edge_rec), ne, cnt, c->bases,
                                                              nmap);
    launched(c);
    int32_t* parent = ptr<int32_t>(c->uf_parent);
    if (nvr > 0) {
        uf_init_kernel<<<grid_for(c, nvr, 256), 256, 0, c->stream>>>(parent, (int32_t)nvr);
        launched(c);
        uf_union_kernel<<<grid_for(c, ne, 256), 256, 0, c->stream>>>(mark, ptr<EdgeHead>(c->edge_rec), kept_of(c),
                                                                      (int32_t)ne, parent, dev_err(c));
        launched(c);
        uf_roots_kernel<<<grid_for(c, nvr, 256), 256, 0, c->stream>>>(parent, (int32_t)nvr, cnt + nmap, c->bases,
                                                                       nmap);
        launched(c);
    }
    VC_CUDA(c, cudaGetLastError());
    std::vector<unsigned long long> h(2 * (size_t)nmap);
    VC_CUDA(c, cudaMemcpyAsync(h.data(), cnt, h.size() * sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                               c->stream));
    VC_TRY(sync_check(c));
    c->vol_euler.assign((size_t)nmap, vc_euler_info{});
    vc_euler_info all{};
    for (int b = 0; b < nmap; ++b) {
        vc_euler_info& e = c->vol_euler[b];
        if (nmap > 1) {
            const size_t n1 = (size_t)nmap + 1;
            e.V = c->h_rem_bases[b + 1] - c->h_rem_bases[b];
            e.F = c->h_rem_bases[2 * n1 + b + 1] - c->h_rem_bases[2 * n1 + b];
        } else {
            e.V = nvr;
            e.F = c->rem.nt;
        }
        e.E = (int64_t)h[b];
        e.C = (int64_t)h[nmap + b];
        e.euler = e.V - e.E + e.F;
        all.V += e.V;
        all.E += e.E;
        all.F += e.F;
        all.C += e.C;
    }
    all.euler = all.V - all.E + all.F;
    *out = all;
    return VC_OK;
}

}  // namespace vc
