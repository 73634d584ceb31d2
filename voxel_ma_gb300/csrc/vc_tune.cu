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
    c->ft_window = false;
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
        c->ft_window = true;
        VC_TRY(run_ft(c));  // untimed
        float ms = 0.0f;
        VC_TRY(time_on_stream(c, [&] { return run_ft(c); }, &ms));
        out->ft_window_ms = ms;
        c->ft_window = ms < best;
    }
    out->ft_method = c->ft_window ? VC_FT_WINDOW : VC_FT_ENVELOPE;
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
