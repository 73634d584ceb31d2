// Device-wide exclusive scan kernels: reduce tiles, scan the tile sums in
// one block, then rescan each tile with its offset.  Tiles are kScanItems rows
// of kScanThreads consecutive elements, so every global access is coalesced.
// Internal linkage: every translation unit that launches them gets its own
// copy.
#pragma once
#include "vc_internal.cuh"

namespace vc {
namespace {
constexpr int kScanThreads = 256;
constexpr int kScanItems = 8;
constexpr int64_t kScanTile = (int64_t)kScanThreads * kScanItems;

template <class T>
__global__ void __launch_bounds__(kScanThreads) scan_tile_sums(const T* __restrict__ in, int64_t n, int64_t* sums) {
    __shared__ int64_t sm[33];
    int64_t base = (int64_t)blockIdx.x * kScanTile;
    int64_t acc = 0;
#pragma unroll
    for (int r = 0; r < kScanItems; ++r) {
        int64_t i = base + (int64_t)r * kScanThreads + threadIdx.x;
        if (i < n) acc += (int64_t)in[i];
    }
    int64_t tot;
    block_exclusive_sum<int64_t>(acc, sm, &tot);
    if (threadIdx.x == 0) sums[blockIdx.x] = tot;
}

__global__ void __launch_bounds__(1024) scan_sums_single(int64_t* sums, int64_t n, int64_t* total) {
    __shared__ int64_t sm[33];
    int64_t carry = 0;
    for (int64_t b = 0; b < n; b += blockDim.x) {
        int64_t i = b + threadIdx.x;
        int64_t v = i < n ? sums[i] : 0;
        int64_t tot;
        int64_t ex = block_exclusive_sum<int64_t>(v, sm, &tot);
        if (i < n) sums[i] = carry + ex;
        carry += tot;
    }
    if (threadIdx.x == 0 && total) *total = carry;
}

template <class T>
__global__ void __launch_bounds__(kScanThreads) scan_apply(const T* in, T* out, int64_t n, const int64_t* sums) {
    __shared__ int64_t sm[33];
    int64_t base = (int64_t)blockIdx.x * kScanTile;
    int64_t carry = sums[blockIdx.x];
    for (int r = 0; r < kScanItems; ++r) {
        int64_t i = base + (int64_t)r * kScanThreads + threadIdx.x;
        int64_t v = i < n ? (int64_t)in[i] : 0;
        int64_t tot;
        int64_t ex = block_exclusive_sum<int64_t>(v, sm, &tot);
        if (i < n) out[i] = (T)(carry + ex);
        carry += tot;
    }
}


}  // namespace
}  // namespace vc
