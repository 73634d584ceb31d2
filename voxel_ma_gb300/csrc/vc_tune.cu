// Autotuner: per-input choice of the launch shapes that depend on the input
// (declared in include/voxelcore_gb300.h, vc_autotune).  Each candidate runs
// on the installed volume or batch and is timed with CUDA events on the
// context's stream; the fastest stays in the context.
#include "vc_internal.cuh"

namespace vc {
int run_sites(vc_ctx* c, int64_t* n_sites);
int run_ft(vc_ctx* c);
int run_lattice_vd(vc_ctx* c, vc_vd_sizes* sizes, double t_thr);
int run_thin_folded(vc_ctx* c, vc_thin_stats* stats);

namespace {

// Milliseconds of fn() on the context's stream (the stream is drained first).
template <class Fn>
int time_on_stream(vc_ctx* c, Fn fn, float* ms) {
    cudaEvent_t a = nullptr, b = nullptr;
    VC_CUDA(c, cudaEventCreate(&a));
    if (cudaEventCreate(&b) != cudaSuccess) {
        cudaEventDestroy(a);
        return cuda_fail(c, cudaGetLastError(), "cudaEventCreate");
    }
    int st = VC_OK;
    if (cudaStreamSynchronize(c->stream) != cudaSuccess || cudaEventRecord(a, c->stream) != cudaSuccess) {
        st = cuda_fail(c, cudaGetLastError(), "timing");
    } else {
        st = fn();
        if (st == VC_OK) {
            if (cudaEventRecord(b, c->stream) != cudaSuccess || cudaEventSynchronize(b) != cudaSuccess ||
                cudaEventElapsedTime(ms, a, b) != cudaSuccess)
                st = cuda_fail(c, cudaGetLastError(), "timing");
        }
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    return st;
}

}  // namespace
}  // namespace vc

using namespace vc;

extern "C" int vc_autotune(vc_ctx* c, double t, vc_tune_result* out) {
    if (!c || !out || t < 0.0) return VC_ERR_ARG;
    if (cudaSetDevice(c->device) != cudaSuccess) return cuda_fail(c, cudaGetLastError(), "cudaSetDevice");
    if (!c->occ.p || c->nvol <= 0) return VC_ERR_STATE;
    *out = vc_tune_result{};
    VC_TRY(run_sites(c, nullptr));
    // feature transform: ring size of the envelope kernel
    c->ft_method = VC_FT_ENVELOPE;
    const int rings[3] = {4, 8, 16};
    int best_ring = 8;
    float best = 1e30f;
    for (int k = 0; k < 3; ++k) {
        c->ft_ring = rings[k];
        VC_TRY(run_ft(c));  // untimed: first launch of this shape
        float ms = 0.0f;
        VC_TRY(time_on_stream(c, [&] { return run_ft(c); }, &ms));
        out->ft_ms[k] = ms;
        if (ms < best) {
            best = ms;
            best_ring = rings[k];
        }
    }
    c->ft_ring = best_ring;
    // then the window method (its far tiles use the chosen ring)
    {
        c->ft_method = VC_FT_WINDOW;
        VC_TRY(run_ft(c));  // untimed
        float ms = 0.0f;
        VC_TRY(time_on_stream(c, [&] { return run_ft(c); }, &ms));
        out->ft_window_ms = ms;
        c->ft_method = ms < best ? VC_FT_WINDOW : VC_FT_ENVELOPE;
    }
    out->ft_method = c->ft_method;
    VC_TRY(run_ft(c));
    // thinning: threads per block and blocks per SM; every trial thins a
    // fresh copy of the same records (the lattice complex is rebuilt)
    const int shapes[5][3] = {{512, 2, 1}, {512, 2, 2}, {512, 4, 1}, {256, 8, 1}, {1024, 1, 1}};
    int best_shape = 0;
    best = 1e30f;
    for (int k = 0; k < 5; ++k) {
        c->thin_threads = shapes[k][0];
        c->thin_blocks_per_sm = shapes[k][1];
        c->thin_items = shapes[k][2];
        float ms = 0.0f;
        for (int rep = 0; rep < 2; ++rep) {  // the first run is untimed
            VC_TRY(run_lattice_vd(c, nullptr, t));
            VC_TRY(time_on_stream(c, [&] { return run_thin_folded(c, nullptr); }, &ms));
        }
        out->thin_ms[k] = ms;
        if (ms < best) {
            best = ms;
            best_shape = k;
        }
    }
    c->thin_threads = shapes[best_shape][0];
    c->thin_blocks_per_sm = shapes[best_shape][1];
    c->thin_items = shapes[best_shape][2];
    out->ft_ring = c->ft_ring;
    out->thin_threads = c->thin_threads;
    out->thin_blocks_per_sm = c->thin_blocks_per_sm;
    out->thin_items = c->thin_items;
    return sync_check(c);
}

// ---------------------------------------------------------------------------
// Random-access probe (declared in include/voxelcore_gb300.h,
// vc_debug_random_rate): how fast this GPU serves touches of random 32-byte
// records, the access pattern of the thinning kernel's records.  Each thread
// step touches six records whose indices come from an integer hash of the
// step; the kinds of touch are those the thinning makes.
namespace vc {
namespace {

__device__ __forceinline__ uint32_t probe_mix(uint32_t x) {
    x ^= x >> 16;
    x *= 0x21f0aaadu;
    x ^= x >> 15;
    x *= 0x735a2d97u;
    x ^= x >> 15;
    return x;
}

template <int OP>
__global__ void __launch_bounds__(256) random_probe_kernel(unsigned long long* rec, uint32_t mask, uint32_t steps,
                                                           uint32_t seed, unsigned long long* sink) {
    unsigned long long acc = 0;
    for (uint32_t s = blockIdx.x * blockDim.x + threadIdx.x; s < steps; s += gridDim.x * blockDim.x) {
        uint32_t r[6];
#pragma unroll
        for (int j = 0; j < 6; ++j) r[j] = probe_mix(s * 6u + (uint32_t)j + seed) & mask;
#pragma unroll
        for (int j = 0; j < 6; ++j) {
            unsigned long long* p = rec + 4ull * r[j];
            if (OP == 0) {
                acc += __ldcg(p);
            } else if (OP == 1) {
                const int4 a = __ldcg(reinterpret_cast<const int4*>(p)), b = __ldcg(reinterpret_cast<const int4*>(p) + 1);
                acc += (unsigned)(a.x + b.w);
            } else if (OP == 2) {
                acc += atomicAdd(p, 1ull);
            } else {
                acc += atomicMax(reinterpret_cast<unsigned*>(p + 1), s);
                acc += atomicAdd(p, 1ull);
            }
        }
    }
    if (acc == 0x5eedull) *sink = acc;  // keeps the loads
}

}  // namespace
}  // namespace vc

extern "C" int vc_debug_random_rate(vc_ctx* c, int op, int64_t bytes, double* touches_per_s) {
    if (!c || !touches_per_s || op < 0 || op > 3 || bytes < (int64_t)32 << 10) return VC_ERR_ARG;
    if (cudaSetDevice(c->device) != cudaSuccess) return cuda_fail(c, cudaGetLastError(), "cudaSetDevice");
    int64_t nrec = 1;
    while (nrec * 2 * 32 <= bytes && nrec < ((int64_t)1 << 31)) nrec *= 2;
    void* buf = nullptr;
    VC_CUDA(c, cudaMallocAsync(&buf, (size_t)nrec * 32 + 64, c->stream));
    int st = VC_OK;
    auto* rec = static_cast<unsigned long long*>(buf);
    auto* sink = reinterpret_cast<unsigned long long*>(static_cast<char*>(buf) + nrec * 32);
    const uint32_t steps = 32u << 20, mask = (uint32_t)(nrec - 1);
    const int grid = c->num_sms * 8;
    float best = 1e30f;
    if (cudaMemsetAsync(buf, 0, (size_t)nrec * 32 + 64, c->stream) != cudaSuccess)
        st = cuda_fail(c, cudaGetLastError(), "cudaMemsetAsync");
    for (int rep = 0; rep < 4 && st == VC_OK; ++rep) {
        float ms = 0.0f;
        st = time_on_stream(c, [&] {
            const uint32_t seed = 7919u * (uint32_t)rep;
            if (op == 0) random_probe_kernel<0><<<grid, 256, 0, c->stream>>>(rec, mask, steps, seed, sink);
            else if (op == 1) random_probe_kernel<1><<<grid, 256, 0, c->stream>>>(rec, mask, steps, seed, sink);
            else if (op == 2) random_probe_kernel<2><<<grid, 256, 0, c->stream>>>(rec, mask, steps, seed, sink);
            else random_probe_kernel<3><<<grid, 256, 0, c->stream>>>(rec, mask, steps, seed, sink);
            launched(c);
            return cudaGetLastError() == cudaSuccess ? VC_OK : VC_ERR_CUDA;
        }, &ms);
        if (rep > 0 && ms < best) best = ms;  // the first launch is untimed
    }
    cudaFreeAsync(buf, c->stream);
    if (st != VC_OK) return st;
    *touches_per_s = 6.0 * steps / (best * 1e-3);
    return sync_check(c);
}
