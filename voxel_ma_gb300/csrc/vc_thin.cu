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
// grid barriers per generation:
//   A (per item)  claims are checked, removals applied, counts decremented;
//                 the decrement that takes a count from 2 to 1 lists its cell
//                 with its own position, decrements that leave 2 or more
//                 raise the cell's last-decrement position (items are handed
//                 out to blocks in blockDim-item pieces from a shared cursor,
//                 so the blocks stay balanced);
//   B (per listed cell)  a cell still at 1 gives its child to the item at
//                 its last-decrement position, in the cell's slot;
//   C (per item)  children are written in order as generation g+1 and that
//                 generation's claims are made.
// Removal state is the queue position of the removing item (unsigned
// 32-bit, kAlive = 2^32 - 1 while present), so every check is
// position-exact.
//
// Memory layout: the accesses are random and cost per request, so every
// cell's static data and thinning state share one record, and each phase
// reads what it needs about a cell with one 16-byte load:
//   face   {e0, e1, e2 | pass bit, rm}                  16 B
//   edge   {v0, v1, rm, em} {rs, trig}                  32 B
//   vertex {rs (with a removed bit), trig}              16 B
// Phase A reads a face record and an edge's head (FE) or a vertex record and
// an edge's head (EV); the decrements and phase B touch an edge's count or a
// vertex record.
// rs packs the count of incident faces (edges) still present, how many of
// them pass the filter, and the sum of their ids: one atomic removes an
// incident cell, and when the count is 1 the sum names the remaining cell
// and (for an edge) the pass count says whether its child is pushed, so no
// incidence list and no face record is read while thinning.  trig packs the
// position of the last decrement with the slot of the cell in that item, so
// the child's slot needs no per-item record of the decremented cells.
#include "vc_internal.cuh"
#include "vc_scan.cuh"

namespace vc {
namespace {

constexpr int kThreads = 256;
constexpr unsigned kFE = 0x80000000u;
constexpr int32_t kEdgeBit = (int32_t)0x80000000u;

struct ThinArgs {
    FaceRec* F;
    EdgeHead* EH;  // edge records: heads and counts
    EdgeCnt* EN;
    VertRec* V;
    const float* thr;  // [0] f_t, [1] l_t
    int2* qa;
    int2* qb;
    int2* child;           // per item: up to 4 children, by slot ({-1, -1}: none)
    int2* cells;           // cells whose count reached 1 in this generation (kEdgeBit: edge), each with
                           // the trig of the decrement that took it to 1
    int* counters;         // [2][4] by generation parity: list length, phase-A work cursor
    int64_t* blk_cnt;      // [2][G][warps per block] children per phase-C warp range, by generation parity
    unsigned* bar;
    int* err;
    int64_t* ctl;  // [0] gen-0 size; out: [1] pushes, [2] processed, [3] skipped, [4] generations
    unsigned long long spin_limit;
    int64_t* trace;  // optional: per generation {items, t_A, t_B, t_C} (global timer, ns)
    int trace_cap;
    int64_t qcap;   // items one generation may hold (qa, qb; 4 child slots and 4 list entries per item)
    uint32_t pos0;  // queue position of the first item of generation 0
};

__device__ __forceinline__ int64_t global_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return (int64_t)t;
}

__device__ __forceinline__ int2 make_fe(int32_t f, int32_t e) { return make_int2((int32_t)((unsigned)f | kFE), e); }
__device__ __forceinline__ int2 make_ev(int32_t e, int32_t v) { return make_int2(e, v); }
__device__ __forceinline__ bool is_fe(int2 it) { return ((unsigned)it.x & kFE) != 0; }

// Queue items, cell lists and child slots are written in one phase and read
// in the next (the list by phase B, the slots by phase C, the next
// generation's items by phase A); vertex records (16 bytes per vertex, the
// smallest record array) take two decrements per face-edge pair besides
// their own pairs and phase B.  Their accesses (cached at L2 only, as every
// access of the generation kernel to data another block wrote is) carry an
// evict-last L2 policy, so that they stay in L2 while the random touches of
// edge and face records, which mostly miss anyway, take the rest.  Measured
// at 512^3 on one box: default policy 44.0 ms, the streams evict-last 43.0 ms
// (half of their lines 43.2 ms, evict-first 45.2 ms); on another box the
// vertex records as well 39.9 against 40.3 ms, the edge counts as well 0.06
// ms less again, the face records as well 0.3 ms more.
__device__ __forceinline__ unsigned long long keep_policy() {
    unsigned long long p;
    asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(p));
    return p;
}
__device__ __forceinline__ int2 ld_stream(const int2* a, unsigned long long pol) {
    int2 v;
    asm volatile("ld.global.cg.L2::cache_hint.v2.s32 {%0, %1}, [%2], %3;" : "=r"(v.x), "=r"(v.y) : "l"(a), "l"(pol));
    return v;
}
__device__ __forceinline__ int4 ld_stream4(const int4* a, unsigned long long pol) {
    int4 v;
    asm volatile("ld.global.cg.L2::cache_hint.v4.s32 {%0, %1, %2, %3}, [%4], %5;"
                 : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w)
                 : "l"(a), "l"(pol));
    return v;
}
__device__ __forceinline__ void st_stream(int2* a, int2 v, unsigned long long pol) {
    asm volatile("st.global.cg.L2::cache_hint.v2.s32 [%0], {%1, %2}, %3;" ::"l"(a), "r"(v.x), "r"(v.y), "l"(pol)
                 : "memory");
}
__device__ __forceinline__ unsigned long long atom_add_keep(unsigned long long* a, unsigned long long v,
                                                            unsigned long long pol) {
    unsigned long long old;
    asm volatile("atom.global.add.L2::cache_hint.u64 %0, [%1], %2, %3;" : "=l"(old) : "l"(a), "l"(v), "l"(pol) : "memory");
    return old;
}
__device__ __forceinline__ void red_max_keep(unsigned long long* a, unsigned long long v, unsigned long long pol) {
    asm volatile("red.global.max.L2::cache_hint.u64 [%0], %1, %2;" ::"l"(a), "l"(v), "l"(pol) : "memory");
}
__device__ __forceinline__ void red_or_keep(unsigned long long* a, unsigned long long v, unsigned long long pol) {
    asm volatile("red.global.or.L2::cache_hint.b64 [%0], %1, %2;" ::"l"(a), "l"(v), "l"(pol) : "memory");
}
__device__ __forceinline__ void st_stream4(int4* a, int4 v, unsigned long long pol) {
    asm volatile("st.global.cg.L2::cache_hint.v4.s32 [%0], {%1, %2, %3, %4}, %5;" ::"l"(a), "r"(v.x), "r"(v.y),
                 "r"(v.z), "r"(v.w), "l"(pol)
                 : "memory");
}
__device__ __forceinline__ int32_t idx0(int2 it) { return (int32_t)((unsigned)it.x & ~kFE); }

// Build the records from the finalized complex (CSR), the measures and the
// thresholds thr = {f_t, l_t}, and reset the thinning state; with all_pass
// every cell passes the filter and no measure is read (measures 0 under
// thresholds 1, as nClosedComponents thins).  A cell with 2^16 or more
// incident cells cannot be represented (VC_ERR_ARG).
__global__ void build_records_kernel(const int2* __restrict__ edges, const int32_t* __restrict__ tri_edges,
                                     const int32_t* __restrict__ ve_off, const int32_t* __restrict__ ve_ids,
                                     const int32_t* __restrict__ ef_off, const int32_t* __restrict__ ef_ids,
                                     const float* __restrict__ em, const float* __restrict__ fm,
                                     const float* __restrict__ thr, int all_pass, int32_t nv, int32_t ne, int32_t nt,
                                     FaceRec* F,
                                     EdgeRecs E, VertRec* V, int32_t* __restrict__ g0, int* err) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    const int64_t n = (int64_t)nv + ne + nt;
    const float f_t = thr[0], l_t = thr[1];
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        if (i < nt) {
            FaceRec r;
            r.e0 = tri_edges[3 * i];
            r.e1 = tri_edges[3 * i + 1];
            r.e2 = tri_edges[3 * i + 2] | ((all_pass || fm[i] < f_t) ? kFacePass : 0);
            r.rm = kAlive;
            F[i] = r;
        } else if (i < (int64_t)nt + ne) {
            const int64_t e = i - nt;
            const int32_t o0 = ef_off[e], o1 = ef_off[e + 1];
            unsigned long long idsum = 0, pass = 0;
            for (int32_t k = o0; k < o1; ++k) {
                const int32_t f = ef_ids[k];
                idsum += (unsigned)f;
                pass += (all_pass || fm[f] < f_t) ? 1u : 0u;
            }
            if ((unsigned long long)(o1 - o0) > kRefMask) set_error(err, VC_ERR_ARG);
            const int2 ev = edges[e];
            E.h[e] = EdgeHead{ev.x, ev.y, kAlive, all_pass ? 0.0f : em[e]};
            E.n[e] = EdgeCnt{rs_make((unsigned)(o1 - o0), pass, idsum), 0ull};
            g0[e] = (o1 - o0 == 1 && pass == 1) ? (int32_t)idsum : -1;
        } else {
            const int64_t v = i - nt - ne;
            const int32_t o0 = ve_off[v], o1 = ve_off[v + 1];
            unsigned long long idsum = 0;  // 2 e + (e passes the filter): the measure the edge record holds, below l_t
            for (int32_t k = o0; k < o1; ++k) {
                const int32_t e = ve_ids[k];
                idsum += 2u * (unsigned)e + ((all_pass ? 0.0f : em[e]) < l_t ? 1u : 0u);
            }
            if ((unsigned long long)(o1 - o0) > kRefMask) set_error(err, VC_ERR_ARG);
            VertRec r;
            r.rs = rs_make((unsigned)(o1 - o0), 0, idsum);
            r.trig = 0;
            V[v] = r;
            g0[(int64_t)ne + v] = (o1 - o0 == 1 && (idsum & 1u)) ? (int32_t)(idsum >> 1) : -1;
        }
    }
}

// Generation 0: FE pairs of edges with one face (edge order), then EV pairs
// of vertices with one edge (vertex order), filtered by the thresholds: the
// entries of g0 that are not -1, compacted in order (tile counts, one scan
// of the tile counts, then each tile writes its items and their claims).
constexpr int kG0Items = 8;
constexpr int64_t kG0Tile = (int64_t)kThreads * kG0Items;

// Generation-0 code i (edges first, then vertices) names an item when it is
// >= 0.
__global__ void __launch_bounds__(kThreads) gen0_count_kernel(const int32_t* __restrict__ g0, int64_t n,
                                                              int64_t* __restrict__ sums) {
    __shared__ int64_t sm[33];
    const int64_t i0 = (int64_t)blockIdx.x * kG0Tile + (int64_t)threadIdx.x * kG0Items;
    int64_t acc = 0;
    if (i0 + kG0Items <= n) {
        const int4 a = __ldcs(reinterpret_cast<const int4*>(g0 + i0));
        const int4 b = __ldcs(reinterpret_cast<const int4*>(g0 + i0) + 1);
        acc = (a.x >= 0) + (a.y >= 0) + (a.z >= 0) + (a.w >= 0) + (b.x >= 0) + (b.y >= 0) + (b.z >= 0) + (b.w >= 0);
    } else {
        for (int r = 0; r < kG0Items; ++r)
            if (i0 + r < n) acc += __ldcs(g0 + i0 + r) >= 0 ? 1 : 0;
    }
    int64_t tot;
    block_exclusive_sum<int64_t>(acc, sm, &tot);
    if (threadIdx.x == 0) sums[blockIdx.x] = tot;
}

// Each thread takes kG0Items consecutive codes of the tile (the tile's items
// then come out in code order with one block scan) and writes their items
// with the queue's evict-last policy (generation 0 reads them next); an item
// beyond the queue's capacity is not written (VC_ERR_OOM).
__global__ void __launch_bounds__(kThreads) gen0_write_kernel(ThinArgs A, int32_t ne, const int32_t* __restrict__ g0,
                                                              int64_t n, const int64_t* __restrict__ sums) {
    static_assert(kG0Items == 8, "two 16-byte loads per thread");
    __shared__ int64_t sm[33];
    const unsigned long long keep_pol = keep_policy();
    const int64_t i0 = (int64_t)blockIdx.x * kG0Tile + (int64_t)threadIdx.x * kG0Items;
    int32_t x[kG0Items];
    if (i0 + kG0Items <= n) {
        const int4 a = __ldcs(reinterpret_cast<const int4*>(g0 + i0));
        const int4 b = __ldcs(reinterpret_cast<const int4*>(g0 + i0) + 1);
        x[0] = a.x, x[1] = a.y, x[2] = a.z, x[3] = a.w, x[4] = b.x, x[5] = b.y, x[6] = b.z, x[7] = b.w;
    } else {
#pragma unroll
        for (int r = 0; r < kG0Items; ++r) x[r] = i0 + r < n ? __ldcs(g0 + i0 + r) : -1;
    }
    int cnt = 0;
#pragma unroll
    for (int r = 0; r < kG0Items; ++r) cnt += x[r] >= 0 ? 1 : 0;
    int64_t tot;
    int64_t p = sums[blockIdx.x] + block_exclusive_sum<int64_t>(cnt, sm, &tot);
#pragma unroll
    for (int r = 0; r < kG0Items; ++r) {
        if (x[r] < 0) continue;
        const int64_t i = i0 + r, li = p++;
        if (li >= A.qcap) {
            set_error(A.err, VC_ERR_OOM);
            continue;
        }
        const uint32_t q = A.pos0 + (uint32_t)li;
        if (i < ne) {
            st_stream(A.qa + li, make_fe(x[r], (int32_t)i), keep_pol);
            atomicMin(&A.F[x[r]].rm, q);
        } else {
            st_stream(A.qa + li, make_ev(x[r], (int32_t)(i - ne)), keep_pol);
            atomicMin(&A.EH[x[r]].rm, q);
        }
    }
}

// Warp-aggregated append of {cell, trig} for a cell whose count fell from 2
// to 1 to the block's shared-memory list of the current piece (all lanes call).
__device__ __forceinline__ void append_pair(int2* region, int* s_count, bool want, int2 pair) {
    const unsigned m = __ballot_sync(0xffffffffu, want);
    if (!m) return;
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(m) - 1;
    int basei = 0;
    if (lane == leader) basei = atomicAdd(s_count, __popc(m));
    basei = __shfl_sync(0xffffffffu, basei, leader);
    if (want) region[basei + __popc(m & ((1u << lane) - 1u))] = pair;
}

// The last decrement of a cell that ends a generation at count 1 is the
// largest position among its decrements in it.  The decrement that takes the
// count from 2 to 1 carries its own trig in the cell's list entry; only
// decrements that leave a count of 2 or more (which may be followed by others
// in the same generation) raise the record's trig with an atomicMax, and
// decrements to 0 need none.  Phase B takes the larger of the two (a trig
// left by an earlier generation holds an earlier position).  Measured at
// 512^3: 46.3 ms against 46.9 ms with every decrement raising the trig (same
// box, same build otherwise).
template <int THREADS, int MINB, int ITEMS>
__global__ void __launch_bounds__(THREADS, MINB) thin_generations_kernel(ThinArgs A) {
    __shared__ int64_t sm[33];
    __shared__ int64_t s_red[2], s_wpre[32];
    __shared__ int s_ncell, s_start, s_gbase;
    __shared__ int2 s_cells[4 * THREADS * ITEMS];
    const int G = gridDim.x, b = blockIdx.x;
    const float l_t = A.thr[1];
    int64_t n = A.ctl[0];
    int64_t base = A.pos0, pushes = n;
    if (n > A.qcap) n = 0;  // generation 0 did not fit the queue (VC_ERR_OOM is set)
    int gen = 0;
    int64_t my_processed = 0, my_skipped = 0;
    int64_t slots_ready = 0;  // child slots [0, 4 slots_ready) hold {-1, -1} or this generation's children
    const int lane = threadIdx.x & 31;
    const unsigned long long keep_pol = keep_policy();
    while (n > 0) {
        const int par = gen & 1;
        const int2* cur = par ? A.qb : A.qa;
        int2* nxt = par ? A.qa : A.qb;
        // phase C: block b writes the children of items [b chunk, (b + 1) chunk),
        // its warp w those of a wchunk-item range of that; the children of each
        // warp range are counted (blk) by the phase that places them
        const int W = blockDim.x >> 5;
        int64_t* blk = A.blk_cnt + (int64_t)par * G * W;
        const int64_t chunk = (n + G - 1) / G;
        const int64_t wchunk = (chunk + W - 1) / W;
        auto range_of = [&](int64_t i) {
            const int64_t bi = i / chunk;
            return bi * W + (i - bi * chunk) / wchunk;
        };
        int* ctr = A.counters + 4 * par;  // [0] list length, [1] phase-A cursor
        // trigs are absolute positions (64-bit); per item and in the cell
        // list they are kept relative to the generation's first position
        const unsigned long long tb2 = (unsigned long long)base << 1;
        const int64_t i0 = min(n, (int64_t)b * chunk), i1 = min(n, i0 + chunk);
        const bool tr = A.trace && b == 0 && threadIdx.x == 0 && gen < A.trace_cap;
        if (tr) {
            A.trace[4 * gen + 0] = n;
            A.trace[4 * gen + 1] = global_ns();
        }
        // the child slots of items beyond any earlier generation start empty
        // (phase B of this generation writes them after the barrier below)
        if (n > slots_ready) {
            const int64_t lo4 = 4 * slots_ready, hi4 = 4 * n;
            for (int64_t k = lo4 + (int64_t)b * blockDim.x + threadIdx.x; k < hi4; k += (int64_t)G * blockDim.x)
                st_stream(A.child + k, make_int2(-1, -1), keep_pol);
            slots_ready = n;
        }
        // ---- phase A: apply the removals of the items that won their claim
        // items are taken in blockDim-item pieces from a shared cursor, so
        // that blocks finishing early take more (the per-item cost varies);
        // the next piece is claimed while the current one is processed
        if (threadIdx.x == 0) {
            s_start = atomicAdd(ctr + 1, (int)blockDim.x * ITEMS);
            s_ncell = 0;
        }
        for (;;) {
            __syncthreads();
            const int64_t r0 = s_start;
            if (r0 >= n) break;
            int next_start = 0;
            if (threadIdx.x == 0) next_start = atomicAdd(ctr + 1, (int)blockDim.x * ITEMS);
            // each thread takes ITEMS items of the piece; their loads are issued
            // together (items, then all their records) before any is used
            int2 it[ITEMS];
            bool has[ITEMS];
#pragma unroll
            for (int k = 0; k < ITEMS; ++k) {
                const int64_t i = r0 + threadIdx.x + (int64_t)k * blockDim.x;
                has[k] = i < n;
                it[k] = has[k] ? ld_stream(cur + i, keep_pol) : make_int2(0, 0);
            }
            // FE item: face record (ra) and the edge's head (ea); EV item:
            // vertex record (ra) and the edge's head (ea)
            int4 ra[ITEMS], ea[ITEMS];
#pragma unroll
            for (int k = 0; k < ITEMS; ++k) {
                ra[k] = ea[k] = make_int4(0, 0, 0, 0);
                if (!has[k]) continue;
                const bool fe = is_fe(it[k]);
                const int32_t e = fe ? it[k].y : it[k].x;
                ra[k] = fe ? __ldcg(reinterpret_cast<const int4*>(A.F + idx0(it[k])))
                           : ld_stream4(reinterpret_cast<const int4*>(A.V + it[k].y), keep_pol);
                ea[k] = __ldcg(reinterpret_cast<const int4*>(A.EH + e));
            }
            int32_t one[4 * ITEMS];  // cells whose count fell to 1 here
            int32_t dec[4 * ITEMS];  // cells decremented here (kEdgeBit: edge) and this item's trig there
            uint32_t dtg[4 * ITEMS];  // (relative), recorded once the decrements have come back (measured faster)
#pragma unroll
            for (int q = 0; q < 4 * ITEMS; ++q) one[q] = dec[q] = -1;
            // a decrement that took the count to 1 or 0 raises no trig
            auto keep_dec = [&](int q, int old_count) {
                if (old_count <= 2) dec[q] = -1;
            };
#pragma unroll
            for (int k = 0; k < ITEMS; ++k) {
                if (!has[k]) continue;
                const int64_t li = r0 + threadIdx.x + (int64_t)k * blockDim.x;  // index in the generation
                const uint32_t p = (uint32_t)(base + li);                        // queue position
                const uint32_t lt = (uint32_t)li << 1;                           // relative trig, bit 0
                if (is_fe(it[k])) {
                    // the edge of an FE item has exactly one face, the item's:
                    // its count fell to 1 once, and only removing that face
                    // lowers it further
                    const int32_t f = idx0(it[k]), e = it[k].y;
                    const uint32_t frm = (uint32_t)ra[k].w;  // FaceRec: e0 e1 e2|pass rm
                    if (frm != p) {
                        ++my_skipped;
                    } else {
                        ++my_processed;
                        // the face's other two sides, in face order (the sides of a
                        // live face other than e are never removed)
                        const int32_t s0 = ra[k].x, s1 = ra[k].y, s2 = ra[k].z & ~kFacePass;
                        const unsigned fpass = ra[k].z < 0 ? 1u : 0u;
                        const int32_t sa = s0 == e ? s1 : s0;
                        const int32_t sb = (s0 == e || s1 == e) ? s2 : s1;
                        const int32_t v0 = ea[k].x, v1 = ea[k].y;  // EdgeHead: v0 v1 rm em
                        // the edge is named by no other item of this generation
                        A.EH[e].rm = p;
                        // the edge's filter: its measure below the edge threshold
                        const unsigned epass = __int_as_float(ea[k].w) < l_t ? 1u : 0u;
                        const unsigned long long df = rs_drop(f, fpass), de = rs_drop((int32_t)(2u * (unsigned)e + epass), 0u);
                        const int oa = rs_count(atomicAdd(&A.EN[sa].rs, df));
                        const int ob = rs_count(atomicAdd(&A.EN[sb].rs, df));
                        const int o0 = rs_count(atom_add_keep(&A.V[v0].rs, de, keep_pol));
                        const int o1 = rs_count(atom_add_keep(&A.V[v1].rs, de, keep_pol));
                        dec[4 * k + 0] = sa | kEdgeBit;
                        dec[4 * k + 1] = sb | kEdgeBit;
                        dec[4 * k + 2] = v0;
                        dec[4 * k + 3] = v1;
                        dtg[4 * k + 0] = dtg[4 * k + 2] = lt;
                        dtg[4 * k + 1] = dtg[4 * k + 3] = lt | 1u;
                        if (oa == 2) one[4 * k + 0] = sa | kEdgeBit;
                        if (ob == 2) one[4 * k + 1] = sb | kEdgeBit;
                        if (o0 == 2) one[4 * k + 2] = v0;
                        if (o1 == 2) one[4 * k + 3] = v1;
                        keep_dec(4 * k + 0, oa);
                        keep_dec(4 * k + 1, ob);
                        keep_dec(4 * k + 2, o0);
                        keep_dec(4 * k + 3, o1);
                    }
                } else {
                    const int32_t e = it[k].x, v = it[k].y;
                    const uint32_t erm = (uint32_t)ea[k].z;  // EdgeHead: v0 v1 rm em
                    const int32_t vref =
                        rs_count(((unsigned long long)(uint32_t)ra[k].y << 32) | (uint32_t)ra[k].x);  // VertRec: rs trig rm
                    if (erm != p) {
                        ++my_skipped;
                    } else if (vref != 1) {
                        set_error(A.err, VC_ERR_INVARIANT);
                    } else {
                        ++my_processed;
                        // v's one edge is e: no later decrement meets v's word
                        red_or_keep(&A.V[v].rs, kVertGone, keep_pol);
                        const int32_t v0 = ea[k].x, v1 = ea[k].y;
                        const int32_t u = v0 != v ? v0 : v1;
                        const unsigned epass = __int_as_float(ea[k].w) < l_t ? 1u : 0u;
                        const int ou =
                            rs_count(atom_add_keep(&A.V[u].rs, rs_drop((int32_t)(2u * (unsigned)e + epass), 0u), keep_pol));
                        if (ou == 2) one[4 * k + 2] = u;
                        dec[4 * k + 2] = u;
                        dtg[4 * k + 2] = lt;
                        keep_dec(4 * k + 2, ou);
                    }
                }
            }
#pragma unroll
            for (int q = 0; q < 4 * ITEMS; ++q)
                append_pair(s_cells, &s_ncell, one[q] != -1, make_int2(one[q], (int32_t)dtg[q]));
#pragma unroll
            for (int q = 0; q < 4 * ITEMS; ++q) {
                if (dec[q] == -1) continue;
                if (dec[q] & kEdgeBit) atomicMax(&A.EN[dec[q] & ~kEdgeBit].trig, tb2 + dtg[q]);
                else red_max_keep(&A.V[dec[q]].trig, tb2 + dtg[q], keep_pol);
            }
            __syncthreads();
            if (threadIdx.x == 0) s_gbase = s_ncell ? atomicAdd(ctr + 0, s_ncell) : 0;
            __syncthreads();
            for (int k = threadIdx.x; k < s_ncell; k += blockDim.x) st_stream(A.cells + s_gbase + k, s_cells[k], keep_pol);
            __syncthreads();
            if (threadIdx.x == 0) {
                s_start = next_start;
                s_ncell = 0;
            }
        }
        if (grid_barrier(A.bar, A.err, A.spin_limit)) break;
        // ---- phase B: a listed cell still at 1 gives its child to the item
        // that decremented it last (its trig position), in the cell's slot
        if (tr) A.trace[4 * gen + 2] = global_ns();
        {
            // contiguous share of the list: cells listed by neighbouring items
            // stay together, as do the records they touch
            const int64_t m = __ldcg(ctr + 0);
            const int64_t mchunk = (m + G - 1) / G;
            const int64_t j1 = min(m, ((int64_t)b + 1) * mchunk);
            for (int64_t jb = (int64_t)b * mchunk; jb < j1; jb += blockDim.x) {
                const int64_t j = jb + threadIdx.x;
                bool want = false;
                int64_t i = 0;
                int slot = 0;
                int2 ch = make_int2(-1, -1);
                if (j < j1) {
                    const int2 ent = ld_stream(A.cells + j, keep_pol);
                    const int32_t code = ent.x;
                    const unsigned long long ltg = tb2 + (uint32_t)ent.y;  // the trig of the decrement to 1
                    unsigned long long tg = 0;
                    if (code & kEdgeBit) {
                        const int32_t e2 = code & ~kEdgeBit;
                        const int4 eb = __ldcg(reinterpret_cast<const int4*>(A.EN + e2));  // rs trig
                        const unsigned long long rs = ((unsigned long long)(uint32_t)eb.y << 32) | (uint32_t)eb.x;
                        want = rs_count(rs) == 1 && rs_pass(rs) == 1;
                        tg = max(((unsigned long long)(uint32_t)eb.w << 32) | (uint32_t)eb.z, ltg);
                        slot = (int)(tg & 1u);
                        ch = make_fe(rs_last(rs), e2);
                    } else {
                        const int32_t u = code;
                        const int4 va = ld_stream4(reinterpret_cast<const int4*>(A.V + u), keep_pol);  // rs trig
                        const unsigned long long rs = ((unsigned long long)(uint32_t)va.y << 32) | (uint32_t)va.x;
                        const uint32_t code = (uint32_t)rs_last(rs);  // 2 e + filter of the one edge left
                        const int32_t e3 = (int32_t)(code >> 1);
                        want = rs_count(rs) == 1 && (code & 1u);
                        tg = max(((unsigned long long)(uint32_t)va.w << 32) | (uint32_t)va.z, ltg);
                        slot = 2 + (int)(tg & 1u);
                        ch = make_ev(e3, u);
                    }
                    i = (int64_t)(tg >> 1) - base;
                    if (want && (i < 0 || i >= n)) {
                        set_error(A.err, VC_ERR_INVARIANT);
                        want = false;
                    }
                }
                if (want) st_stream(A.child + 4 * i + slot, ch, keep_pol);
                // children per phase-C warp range, one atomic per warp and range
                const int64_t bi = want ? range_of(i) : -1;
                const unsigned grp = __match_any_sync(0xffffffffu, bi);
                if (want && lane == __ffs(grp) - 1)
                    atomicAdd((unsigned long long*)(blk + bi), (unsigned long long)__popc(grp));
            }
        }
        if (grid_barrier(A.bar, A.err, A.spin_limit)) break;
        // ---- phase C: prefixes, write generation g+1 and make its claims;
        // each warp writes its range on its own (no block-wide step per item)
        if (tr) A.trace[4 * gen + 3] = global_ns();
        {
            int64_t before = 0, all = 0;
            const int64_t nr = (int64_t)G * W, mine = (int64_t)b * W;
            for (int64_t k = threadIdx.x; k < nr; k += blockDim.x) {
                const int64_t v = __ldcg(blk + k);
                all += v;
                if (k < mine) before += v;
            }
            int64_t t1, t2;
            block_exclusive_sum<int64_t>(before, sm, &t1);
            block_exclusive_sum<int64_t>(all, sm, &t2);
            if (threadIdx.x < 32) {
                // the earlier warp ranges of this block
                const int64_t v = threadIdx.x < W ? __ldcg(blk + mine + threadIdx.x) : 0;
                const int64_t inc = warp_inclusive_sum(v);
                if (threadIdx.x < W) s_wpre[threadIdx.x] = inc - v;
            }
            if (threadIdx.x == 0) {
                s_red[0] = t1;
                s_red[1] = t2;
            }
            __syncthreads();
        }
        const int64_t total = s_red[1];
        const int64_t nbase = base + n;
        if (total > A.qcap) {  // every block sees the same total and leaves here
            if (b == 0 && threadIdx.x == 0) set_error(A.err, VC_ERR_OOM);
            break;
        }
        const int wid = threadIdx.x >> 5;
        int64_t running = s_red[0] + s_wpre[wid];
        const int64_t w0 = min(i1, i0 + (int64_t)wid * wchunk), w1 = min(i1, w0 + wchunk);
        for (int64_t r0 = w0; r0 < w1; r0 += 32) {
            const int64_t i = r0 + lane;
            int2 cs[4] = {make_int2(-1, -1), make_int2(-1, -1), make_int2(-1, -1), make_int2(-1, -1)};
            unsigned msk = 0;
            if (i < w1) {
                int4* sp = reinterpret_cast<int4*>(A.child + 4 * i);
                const int4 s01 = ld_stream4(sp, keep_pol), s23 = ld_stream4(sp + 1, keep_pol);
                cs[0] = make_int2(s01.x, s01.y);
                cs[1] = make_int2(s01.z, s01.w);
                cs[2] = make_int2(s23.x, s23.y);
                cs[3] = make_int2(s23.z, s23.w);
#pragma unroll
                for (int sl = 0; sl < 4; ++sl) msk |= cs[sl].y >= 0 ? (1u << sl) : 0u;
                // empty the slots for the next generation
                if (msk & 3u) st_stream4(sp, make_int4(-1, -1, -1, -1), keep_pol);
                if (msk & 12u) st_stream4(sp + 1, make_int4(-1, -1, -1, -1), keep_pol);
            }
            const int cnt = __popc(msk);
            const int inc = warp_inclusive_sum(cnt);
            const int64_t ex = inc - cnt, tot = __shfl_sync(0xffffffffu, inc, 31);
            int k = 0;
#pragma unroll
            for (int sl = 0; sl < 4; ++sl) {
                if (!(msk & (1u << sl))) continue;
                const int2 ch = cs[sl];
                const int64_t slot = running + ex + k;
                ++k;
                st_stream(nxt + slot, ch, keep_pol);
                const uint32_t q = (uint32_t)(nbase + slot);
                if (is_fe(ch)) atomicMin(&A.F[idx0(ch)].rm, q);
                else atomicMin(&A.EH[ch.x].rm, q);
            }
            running += tot;
        }
        // counters of the next generation start at zero
        if (threadIdx.x < W) A.blk_cnt[(int64_t)(par ^ 1) * G * W + (int64_t)b * W + threadIdx.x] = 0;
        if (threadIdx.x == 0) {
            if (b == 0) {
                int* nc = A.counters + 4 * (par ^ 1);
                nc[0] = nc[1] = nc[2] = 0;
            }
        }
        __syncthreads();
        base = nbase;
        n = total;
        pushes += total;
        ++gen;
        if (grid_barrier(A.bar, A.err, A.spin_limit)) break;
    }
    atomicAdd((unsigned long long*)&A.ctl[2], (unsigned long long)my_processed);
    atomicAdd((unsigned long long*)&A.ctl[3], (unsigned long long)my_skipped);
    if (b == 0 && threadIdx.x == 0) {
        A.ctl[1] = pushes;
        A.ctl[4] = gen;
    }
}

__global__ void bias_vertex_kernel(VertRec* V, int64_t v, int delta) {
    // the count is the low field of rs; a count of 0 is not lowered (the
    // borrow would reach the removed bit)
    if (delta < 0 && rs_count(V[v].rs) == 0) return;
    V[v].rs += (unsigned long long)(long long)delta;
}

__global__ void set_thr_kernel(float* thr, float f_t, float l_t) {
    thr[0] = f_t;
    thr[1] = l_t;
}

// Survivor flags from the records: keep_v = vertex not removed; keep_e =
// edge not removed and referenced by no remaining face (getRemainedEdges);
// keep_f = face not removed; removed_e = edge removal tag.  One warp per 32
// cells of a kind (vertices, then edges, then faces): the same flags also go
// out as one bit word per warp with its population count, for the remaining
// complex's compaction.
__global__ void export_flags_kernel(const FaceRec* __restrict__ F, const EdgeHead* __restrict__ EH,
                                    const EdgeCnt* __restrict__ EN,
                                    const VertRec* __restrict__ V, int32_t nv, int32_t ne, int32_t nt, uint8_t* kv,
                                    uint8_t* ke, uint8_t* kf, uint8_t* re, uint32_t* __restrict__ bits,
                                    int32_t* __restrict__ wv, int32_t* __restrict__ we, int32_t* __restrict__ wf) {
    const int lane = threadIdx.x & 31;
    const int64_t nwv = ((int64_t)nv + 31) / 32, nwe = ((int64_t)ne + 31) / 32, nwf = ((int64_t)nt + 31) / 32;
    const int64_t nw = nwv + nwe + nwf;
    const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
    for (int64_t w = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); w < nw; w += warps) {
        bool keep = false;
        if (w < nwv) {
            const int64_t i = w * 32 + lane;
            if (i < nv) {
                keep = !(__ldcs(&V[i].rs) & kVertGone);
                kv[i] = keep;
            }
        } else if (w < nwv + nwe) {
            const int64_t e = (w - nwv) * 32 + lane;
            if (e < ne) {
                const int4 ea = __ldcs(reinterpret_cast<const int4*>(EH + e));  // v0 v1 rm em
                const int4 eb = __ldcs(reinterpret_cast<const int4*>(EN + e));  // rs trig
                const uint32_t rm = (uint32_t)ea.z;
                const int32_t ref = rs_count(((unsigned long long)(uint32_t)eb.y << 32) | (uint32_t)eb.x);
                keep = rm == kAlive && ref == 0;
                ke[e] = keep;
                re[e] = rm != kAlive;
            }
        } else {
            const int64_t f = (w - nwv - nwe) * 32 + lane;
            if (f < nt) {
                keep = __ldcs(&F[f].rm) == kAlive;
                kf[f] = keep;
            }
        }
        const uint32_t word = __ballot_sync(0xffffffffu, keep);
        if (lane == 0) {
            bits[w] = word;
            if (w < nwv) wv[w] = __popc(word);
            else if (w < nwv + nwe) we[w - nwv] = __popc(word);
            else wf[w - nwv - nwe] = __popc(word);
        }
    }
}

inline int grid_for(vc_ctx* c, int64_t n, int threads) {
    int64_t b = (n + threads - 1) / threads;
    return (int)std::max<int64_t>(1, std::min<int64_t>(b, (int64_t)c->num_sms * 16));
}

// Bytes of queue per item of capacity: two item arrays (generations g and
// g + 1), four child slots and four cell-list entries.
constexpr int64_t kQueueBytes = 2 * (int64_t)sizeof(int2) + 4 * (int64_t)sizeof(int2) + 4 * (int64_t)sizeof(int2);
// A generation's cell list (four entries per item) has a 32-bit length.
constexpr int64_t kMaxQueue = ((int64_t)1 << 29) - 1;
// Device memory left for the queue at most: free memory, free memory of the
// default stream-ordered pool (the context's buffers live there) and what
// the queue buffers hold already, less a reserve for the rest of the call.
int64_t queue_room(vc_ctx* c) {
    size_t fr = 0, tot = 0;
    if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    int64_t room = (int64_t)fr;
    cudaMemPool_t pool;
    uint64_t reserved = 0, used = 0;
    if (cudaDeviceGetDefaultMemPool(&pool, c->device) != cudaSuccess ||
        cudaMemPoolGetAttribute(pool, cudaMemPoolAttrReservedMemCurrent, &reserved) != cudaSuccess ||
        cudaMemPoolGetAttribute(pool, cudaMemPoolAttrUsedMemCurrent, &used) != cudaSuccess) {
        cudaGetLastError();
        reserved = used = 0;
    }
    if (reserved > used) room += (int64_t)(reserved - used);
    room += (int64_t)(c->q0.cap + c->q1.cap + c->child.cap + c->cells.cap);
    return room - ((int64_t)2 << 30);
}

}  // namespace

int run_thin_with_device_thr(vc_ctx* c, vc_thin_stats* stats, bool all_pass = false);
int ensure_vd_aux(vc_ctx* c, bool meas, bool topo);

int run_thin(vc_ctx* c, float f_t, float l_t, vc_thin_stats* stats) {
    if (!c->cc_finalized || !c->meas_valid) return VC_ERR_STATE;
    if (c->records_thr_folded) {
        // records hold filter signs, not measures: rebuild them from em / fm
        c->records_fresh = false;
        c->records_thr_folded = false;
    }
    VC_TRY(ensure_n<float>(c, c->thr, 2));
    set_thr_kernel<<<1, 1, 0, c->stream>>>(ptr<float>(c->thr), f_t, l_t);
    launched(c);
    VC_CUDA(c, cudaGetLastError());
    return run_thin_with_device_thr(c, stats);
}

// Thinning of a batch whose per-volume thresholds were folded into the
// records by the lattice emission: the filter is then "record < 0".
int run_thin_folded(vc_ctx* c, vc_thin_stats* stats) {
    if (!c->records_thr_folded || !c->records_fresh) return VC_ERR_STATE;
    VC_TRY(ensure_n<float>(c, c->thr, 2));
    set_thr_kernel<<<1, 1, 0, c->stream>>>(ptr<float>(c->thr), 0.0f, 0.0f);
    launched(c);
    VC_CUDA(c, cudaGetLastError());
    c->records_thr_folded = false;
    return run_thin_with_device_thr(c, stats);
}

// Thinning in which every pair passes the filter, whatever the measures:
// the reference's nClosedComponents sets every measure to 0 and thins at
// thresholds 1 (highlevelalgo.cpp:993-1020).
int run_thin_all_pass(vc_ctx* c, vc_thin_stats* stats) {
    if (!c->cc_finalized) return VC_ERR_STATE;
    VC_TRY(ensure_n<float>(c, c->thr, 2));
    set_thr_kernel<<<1, 1, 0, c->stream>>>(ptr<float>(c->thr), 1.0f, 1.0f);
    launched(c);
    VC_CUDA(c, cudaGetLastError());
    c->records_fresh = false;  // the records are rebuilt with every cell passing
    c->records_thr_folded = false;
    return run_thin_with_device_thr(c, stats, true);
}

// Thinning with thresholds already in c->thr (device).
int run_thin_with_device_thr(vc_ctx* c, vc_thin_stats* stats, bool all_pass) {
    if (!c->cc_finalized || (!all_pass && !c->meas_valid)) return VC_ERR_STATE;
    const int64_t nv = c->nv, ne = c->ne, nt = c->nt;
    // ids are 31-bit (items and lists tag them with bit 31); queue positions
    // are 32-bit: a thinning pushes at most one item per vertex and edge
    if (nv >= INT32_MAX || ne >= INT32_MAX || nt >= INT32_MAX) return VC_ERR_ARG;
    if ((int64_t)c->thin_pos0 + nv + ne + 1 >= (int64_t)kAlive) return VC_ERR_ARG;
    Region stage(c, "stage_thin");
    if (!c->records_fresh) {
        // the records are built from the measures, sides and lists
        VC_TRY(ensure_vd_aux(c, !all_pass, true));
        VC_TRY(ensure_n<FaceRec>(c, c->face_rec, nt));
        VC_TRY(ensure_n<VertRec>(c, c->vert_rec, nv));
        VC_TRY(ensure_n<int32_t>(c, c->thin_g0, nv + ne));
    }
    EdgeRecs ER;
    VC_TRY(ensure_edge_recs(c, c->edge_rec, ne, &ER));  // (written by the lattice complex when fresh)
    VC_TRY(ensure_n<int64_t>(c, c->euler_tmp, 16));
    VC_TRY(ensure_n<uint8_t>(c, c->keep_v, nv));
    VC_TRY(ensure_n<uint8_t>(c, c->keep_e, ne));
    VC_TRY(ensure_n<uint8_t>(c, c->keep_f, nt));
    VC_TRY(ensure_n<uint8_t>(c, c->removed_e, ne));
    const int64_t nwv = (nv + 31) / 32, nwe = (ne + 31) / 32, nwf = (nt + 31) / 32;
    VC_TRY(ensure_n<uint32_t>(c, c->keep_bits, nwv + nwe + nwf + 1));
    VC_TRY(ensure_n<int32_t>(c, c->keep_wv, nwv + 1));
    VC_TRY(ensure_n<int32_t>(c, c->keep_we, nwe + 1));
    VC_TRY(ensure_n<int32_t>(c, c->keep_wf, nwf + 1));
    // Queue capacity: one generation holds at most one item per vertex and
    // edge, so V + E + 1 items always suffice.  When that does not fit (the
    // 1024^3 random field: 2.6e9 items, 209 GB, while its largest generation
    // is a small fraction of it), the queue takes at most 2^29 items and half
    // of the room the device has left, the other half staying for the stages
    // after the thinning; a generation beyond the capacity ends the thinning
    // with VC_ERR_OOM.
    int64_t qcap = std::min<int64_t>(nv + ne + 1, kMaxQueue);
    if (c->thin_qcap > 0) {
        qcap = std::min(qcap, c->thin_qcap);
    } else if (qcap * kQueueBytes > (int64_t)(c->q0.cap + c->q1.cap + c->child.cap + c->cells.cap)) {
        qcap = std::max<int64_t>(1, std::min(qcap, queue_room(c) / 2 / kQueueBytes));
    }
    VC_TRY(ensure_n<int2>(c, c->q0, qcap));
    VC_TRY(ensure_n<int2>(c, c->q1, qcap));
    VC_TRY(ensure_n<int2>(c, c->child, 4 * qcap));
    VC_TRY(ensure_n<int2>(c, c->cells, 4 * qcap));
    ThinArgs A{};
    A.qcap = qcap;
    A.pos0 = c->thin_pos0;
    A.F = ptr<FaceRec>(c->face_rec);
    A.EH = ER.h;
    A.EN = ER.n;
    A.V = ptr<VertRec>(c->vert_rec);
    A.thr = ptr<float>(c->thr);
    A.qa = ptr<int2>(c->q0);
    A.qb = ptr<int2>(c->q1);
    A.child = ptr<int2>(c->child);
    A.cells = ptr<int2>(c->cells);
    A.err = dev_err(c);
    int64_t* ctl = ptr<int64_t>(c->euler_tmp);
    A.ctl = ctl;
    A.bar = reinterpret_cast<unsigned*>(ctl + 8);

    A.spin_limit = c->spin_limit;
    if (c->trace_cap > 0) {
        VC_TRY(ensure_n<int64_t>(c, c->trace, 4 * (int64_t)c->trace_cap));
        VC_CUDA(c, cudaMemsetAsync(c->trace.p, 0, 4 * sizeof(int64_t) * c->trace_cap, c->stream));
        A.trace = ptr<int64_t>(c->trace);
        A.trace_cap = c->trace_cap;
    }
    {
        Region r(c, "thin_setup");
        if (c->records_fresh) {
            c->records_fresh = false;  // the next thinning of this complex rebuilds them
        } else {
            build_records_kernel<<<grid_for(c, nv + ne + nt, 256), 256, 0, c->stream>>>(
                ptr<int2>(c->edges), ptr<int32_t>(c->tri_edges), ptr<int32_t>(c->ve_off), ptr<int32_t>(c->ve_ids),
                ptr<int32_t>(c->ef_off), ptr<int32_t>(c->ef_ids), ptr<float>(c->em), ptr<float>(c->fm), A.thr,
                all_pass ? 1 : 0, (int32_t)nv, (int32_t)ne, (int32_t)nt, A.F, ER, A.V, ptr<int32_t>(c->thin_g0),
                dev_err(c));
            launched(c);
        }
        if (c->ref_bias_vertex >= 0 && c->ref_bias_vertex < nv) {
            // a broken reference count, as the reference's logic check meets it
            bias_vertex_kernel<<<1, 1, 0, c->stream>>>(A.V, c->ref_bias_vertex, c->ref_bias);
            launched(c);
        }
        VC_CUDA(c, cudaMemsetAsync(ctl, 0, 16 * sizeof(int64_t), c->stream));
        const int64_t ng = nv + ne;
        const int64_t tiles = (ng + kG0Tile - 1) / kG0Tile;
        if (tiles > 0) {
            VC_TRY(ensure_n<int64_t>(c, c->scratch, tiles + 1));
            int64_t* sums = ptr<int64_t>(c->scratch);
            const int32_t* g0 = ptr<int32_t>(c->thin_g0);
            gen0_count_kernel<<<(unsigned)tiles, kThreads, 0, c->stream>>>(g0, ng, sums);
            scan_sums_single<<<1, 1024, 0, c->stream>>>(sums, tiles, ctl + 0);
            gen0_write_kernel<<<(unsigned)tiles, kThreads, 0, c->stream>>>(A, (int32_t)ne, g0, ng, sums);
            launched(c, 3);
        }
        VC_CUDA(c, cudaGetLastError());
    }
    // persistent cooperative launch: every block resident
    // launch shapes (threads per block x blocks per SM, items per thread and
    // piece): 512 x 2 (default), 512 x 2 with 2 items, 512 x 4, 256 x 8,
    // 1024 x 1
    const int threads = c->thin_threads == 256 ? 256 : (c->thin_threads == 1024 ? 1024 : 512);
    void* kern = threads == 256    ? (void*)thin_generations_kernel<256, 8, 1>
                 : threads == 1024 ? (void*)thin_generations_kernel<1024, 1, 1>
                 : (c->thin_blocks_per_sm >= 3)
                     ? (void*)thin_generations_kernel<512, 4, 1>
                     : (c->thin_items == 2 ? (void*)thin_generations_kernel<512, 2, 2>
                                           : (void*)thin_generations_kernel<512, 2, 1>);
    int per_sm = 0;
    VC_CUDA(c, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, threads, 0));
    if (per_sm <= 0) return VC_ERR_CUDA;
    const int G = c->num_sms * std::min(per_sm, c->thin_blocks_per_sm > 0 ? c->thin_blocks_per_sm : 2048 / threads);
    const int64_t nrange = 2 * (int64_t)G * (threads / 32);  // phase-C warp ranges, both parities
    VC_TRY(ensure_n<int64_t>(c, c->blk_cnt, nrange + 8));
    VC_CUDA(c, cudaMemsetAsync(c->blk_cnt.p, 0, (nrange + 8) * sizeof(int64_t), c->stream));
    A.blk_cnt = ptr<int64_t>(c->blk_cnt);
    A.counters = reinterpret_cast<int*>(A.blk_cnt + nrange);
    void* args[] = {&A};
    {
        // Contexts that share a thinning lock (the request loop's workers)
        // run their persistent kernels one at a time, each on the whole GPU;
        // the lock is held from the launch until the kernel has finished.
        std::unique_lock<std::mutex> lk;
        if (c->thin_lock) {
            VC_CUDA(c, cudaStreamSynchronize(c->stream));
            lk = std::unique_lock<std::mutex>(*c->thin_lock);
        }
        Region r(c, "thin_generations");
        VC_CUDA(c, cudaLaunchCooperativeKernel(kern, dim3(G), dim3(threads), args, 0, c->stream));
        launched(c);
        if (c->thin_lock) VC_CUDA(c, cudaStreamSynchronize(c->stream));
    }
    {
        export_flags_kernel<<<grid_for(c, 32 * (nwv + nwe + nwf), 256), 256, 0, c->stream>>>(
            A.F, A.EH, A.EN, A.V, (int32_t)nv, (int32_t)ne, (int32_t)nt, ptr<uint8_t>(c->keep_v), ptr<uint8_t>(c->keep_e),
            ptr<uint8_t>(c->keep_f), ptr<uint8_t>(c->removed_e), ptr<uint32_t>(c->keep_bits), ptr<int32_t>(c->keep_wv),
            ptr<int32_t>(c->keep_we), ptr<int32_t>(c->keep_wf));
        launched(c);
    }
    int64_t h[5];
    VC_CUDA(c, cudaMemcpyAsync(h, ctl, 5 * sizeof(int64_t), cudaMemcpyDeviceToHost, c->stream));
    int s = sync_check(c);
    if (s != VC_OK) return s;
    c->thin_stats = vc_thin_stats{h[1], h[2], h[3], h[4]};
    c->trace_gens = (int)std::min<int64_t>(h[4], c->trace_cap);
    c->thin_valid = true;
    c->rem_valid = false;
    if (stats) *stats = c->thin_stats;
    return VC_OK;
}

int get_thin_flags(vc_ctx* c, uint8_t* kv, uint8_t* ke, uint8_t* kf, uint8_t* re, int mem) {
    if (!c->thin_valid) return VC_ERR_STATE;
    VC_TRY(copy_out(c, kv, c->keep_v.p, c->nv, mem));
    VC_TRY(copy_out(c, ke, c->keep_e.p, c->ne, mem));
    VC_TRY(copy_out(c, kf, c->keep_f.p, c->nt, mem));
    VC_TRY(copy_out(c, re, c->removed_e.p, c->ne, mem));
    return sync_check(c);
}

}  // namespace vc

extern "C" {

int vc_debug_thin_trace(vc_ctx* c, int cap, int blocks_per_sm) {
    if (!c) return VC_ERR_ARG;
    c->trace_cap = cap > 0 ? cap : 0;
    c->thin_blocks_per_sm = blocks_per_sm;
    return VC_OK;
}

int vc_debug_thin_shape(vc_ctx* c, int threads, int blocks_per_sm, int items) {
    if (!c || (threads != 0 && threads != 256 && threads != 512 && threads != 1024) || blocks_per_sm < 0 ||
        (items != 0 && items != 1 && items != 2))
        return VC_ERR_ARG;
    c->thin_threads = threads;
    c->thin_blocks_per_sm = blocks_per_sm;
    c->thin_items = items == 2 ? 2 : 1;
    return VC_OK;
}

int vc_debug_set_spin_limit(vc_ctx* c, unsigned long long polls) {
    if (!c) return VC_ERR_ARG;
    c->spin_limit = polls ? polls : (1ull << 26);
    return VC_OK;
}

int vc_debug_fail_alloc_after(vc_ctx* c, int64_t k) {
    if (!c) return VC_ERR_ARG;
    c->fail_alloc_after = k < 0 ? -1 : k;
    return VC_OK;
}

int vc_debug_thin_queue(vc_ctx* c, int64_t capacity, uint32_t first_position) {
    if (!c || capacity < 0) return VC_ERR_ARG;
    c->thin_qcap = capacity;
    c->thin_pos0 = first_position;
    return VC_OK;
}

int vc_debug_ref_bias(vc_ctx* c, int64_t vertex, int delta) {
    if (!c || delta < -1 || delta > 1) return VC_ERR_ARG;
    c->ref_bias_vertex = delta ? vertex : -1;
    c->ref_bias = delta;
    return VC_OK;
}

int vc_debug_get_thin_trace(vc_ctx* c, int64_t* out, int cap, int* ngen) {
    if (!c || !ngen) return VC_ERR_ARG;
    *ngen = c->trace_gens;
    if (!out || c->trace_gens == 0) return VC_OK;
    const int n = std::min(cap, c->trace_gens);
    return vc::copy_out(c, out, c->trace.p, 4 * sizeof(int64_t) * n, VC_MEM_HOST);
}

}  // extern "C"
