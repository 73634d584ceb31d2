// MRC density maps as input volumes (the reference's readMRC,
// src/importers.cpp:45-60, which goes through Tao Ju's MRC reader -- absent
// from the reference tree -- and wraps the map as a DenseVolume whose
// getDataAt > 0 is inside, include/spaceinfo.h:122-135).
//
// Written from the public MRC header layout (MRC2014; the CCP4 / IMOD
// format): a 1024-byte header of 4-byte words -- word 0..2 the column, row
// and section counts, word 3 the mode (0 int8, 1 int16, 2 float32, 6 uint16,
// 12 float16), words 16..18 which axis (1 = x, 2 = y, 3 = z) columns, rows
// and sections run along, word 23 the bytes of extended header that follow
// the 1024, bytes 212..213 the machine stamp (0x44 0x44 or 0x44 0x41 little
// endian, 0x11 0x11 big endian) -- then the values, columns fastest.  A map
// whose axis words are not a permutation of 1..3 is read as columns = x,
// rows = y, sections = z.
//
// The header is read on the host; the values go to the device as they are
// and one kernel writes the occupancy (value > 0) in the library's layout
// (x-major, z fastest), through a shared-memory tile when the file's fastest
// axis is not z, so both the loads and the stores are coalesced.
#include "vc_internal.cuh"

#include <cstring>

namespace vc {
namespace {

constexpr int kMrcHeader = 1024;
constexpr int kTile = 32;
struct Half16 {  // mode 12: IEEE half, read as its bits
    uint16_t bits;
};

template <class T>
__device__ __forceinline__ bool positive(const uint8_t* p, bool swap);

__device__ __forceinline__ uint16_t ld16(const uint8_t* p, bool swap) {
    const uint16_t v = (uint16_t)p[0] | ((uint16_t)p[1] << 8);
    return swap ? (uint16_t)((v >> 8) | (v << 8)) : v;
}
__device__ __forceinline__ uint32_t ld32(const uint8_t* p, bool swap) {
    const uint32_t v = (uint32_t)p[0] | ((uint32_t)p[1] << 8) | ((uint32_t)p[2] << 16) | ((uint32_t)p[3] << 24);
    return swap ? __byte_perm(v, 0, 0x0123) : v;
}
// value > 0 for each mode (NaN is not > 0)
template <>
__device__ __forceinline__ bool positive<int8_t>(const uint8_t* p, bool) {
    return (int8_t)p[0] > 0;
}
template <>
__device__ __forceinline__ bool positive<int16_t>(const uint8_t* p, bool swap) {
    return (int16_t)ld16(p, swap) > 0;
}
template <>
__device__ __forceinline__ bool positive<uint16_t>(const uint8_t* p, bool swap) {
    return ld16(p, swap) > 0;
}
template <>
__device__ __forceinline__ bool positive<float>(const uint8_t* p, bool swap) {
    return __uint_as_float(ld32(p, swap)) > 0.0f;
}
template <>
__device__ __forceinline__ bool positive<Half16>(const uint8_t* p, bool swap) {
    // a half is > 0 iff its sign bit is clear and it is neither zero nor NaN
    const uint16_t h = ld16(p, swap);
    return !(h & 0x8000u) && h != 0 && (h & 0x7fffu) <= 0x7c00u;
}

struct MrcMap {
    int n[3];     // columns, rows, sections
    int axis[3];  // volume axis (0 = x, 1 = y, 2 = z) of columns, rows, sections
    int dim[3];   // volume sizes X, Y, Z
};

// Coordinates of volume axis a -> position along it; the file index of
// voxel (x, y, z) is (s * rows + r) * cols + c.
__device__ __forceinline__ int64_t file_index(const MrcMap& m, const int v[3]) {
    return ((int64_t)v[m.axis[2]] * m.n[1] + v[m.axis[1]]) * m.n[0] + v[m.axis[0]];
}

// Columns run along z: file and volume are both z-fastest along that axis;
// one thread per voxel, consecutive threads on consecutive z.
template <class T>
__global__ void mrc_direct_kernel(const uint8_t* __restrict__ raw, MrcMap m, bool swap, uint8_t* __restrict__ occ) {
    const int64_t n = (int64_t)m.dim[0] * m.dim[1] * m.dim[2];
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int v[3] = {(int)(i / ((int64_t)m.dim[1] * m.dim[2])), (int)((i / m.dim[2]) % m.dim[1]),
                          (int)(i % m.dim[2])};
        occ[i] = positive<T>(raw + file_index(m, v) * (int64_t)sizeof(T), swap) ? 1 : 0;
    }
}

// Columns run along axis A != z: a 32 x 32 tile of the (A, z) plane at one
// position of the third axis B goes through shared memory; loads walk A
// (the file's fastest), stores walk z (the volume's fastest).
template <class T>
__global__ void __launch_bounds__(kTile * 8) mrc_tile_kernel(const uint8_t* __restrict__ raw, MrcMap m, bool swap,
                                                             int A, int B, uint8_t* __restrict__ occ) {
    __shared__ uint8_t tile[kTile][kTile + 1];
    const int tilesA = (m.dim[A] + kTile - 1) / kTile, tilesZ = (m.dim[2] + kTile - 1) / kTile;
    const int64_t ntiles = (int64_t)tilesA * tilesZ * m.dim[B];
    for (int64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const int b = (int)(t / ((int64_t)tilesA * tilesZ));
        const int rem = (int)(t - (int64_t)b * tilesA * tilesZ);
        const int a0 = (rem / tilesZ) * kTile, z0 = (rem % tilesZ) * kTile;
        for (int r = threadIdx.y; r < kTile; r += blockDim.y) {
            const int a = a0 + threadIdx.x, z = z0 + r;
            uint8_t bit = 0;
            if (a < m.dim[A] && z < m.dim[2]) {
                int v[3];
                v[A] = a;
                v[B] = b;
                v[2] = z;
                bit = positive<T>(raw + file_index(m, v) * (int64_t)sizeof(T), swap) ? 1 : 0;
            }
            tile[r][threadIdx.x] = bit;
        }
        __syncthreads();
        for (int r = threadIdx.y; r < kTile; r += blockDim.y) {
            const int a = a0 + r, z = z0 + threadIdx.x;
            if (a < m.dim[A] && z < m.dim[2]) {
                int v[3];
                v[A] = a;
                v[B] = b;
                v[2] = z;
                occ[((int64_t)v[0] * m.dim[1] + v[1]) * m.dim[2] + v[2]] = tile[threadIdx.x][r];
            }
        }
        __syncthreads();
    }
}

int32_t word(const uint8_t* h, int i, bool swap) {
    uint32_t v;
    std::memcpy(&v, h + 4 * i, 4);
    if (swap) v = (v >> 24) | ((v >> 8) & 0xff00u) | ((v << 8) & 0xff0000u) | (v << 24);
    return (int32_t)v;
}

int elem_size(int mode) {
    switch (mode) {
        case 0: return 1;
        case 1: case 6: case 12: return 2;
        case 2: return 4;
        default: return 0;
    }
}

template <class T>
void launch(vc_ctx* c, const uint8_t* raw, const MrcMap& m, bool swap, uint8_t* occ) {
    const int64_t n = (int64_t)m.dim[0] * m.dim[1] * m.dim[2];
    const int64_t cap = (int64_t)c->num_sms * 16;
    if (m.axis[0] == 2) {
        mrc_direct_kernel<T><<<(int)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, cap)), 256, 0,
                               c->stream>>>(raw, m, swap, occ);
    } else {
        const int A = m.axis[0], B = 3 - A - 2;  // the axes other than z: A (columns) and B
        const int64_t tiles = (int64_t)((m.dim[A] + kTile - 1) / kTile) * ((m.dim[2] + kTile - 1) / kTile) * m.dim[B];
        mrc_tile_kernel<T><<<(int)std::max<int64_t>(1, std::min<int64_t>(tiles, cap)), dim3(kTile, 8), 0,
                             c->stream>>>(raw, m, swap, A, B, occ);
    }
    launched(c);
}

}  // namespace

// Parse and validate the header; fills the map, the mode, the byte order
// and the offset of the values.
int mrc_header(const uint8_t* b, int64_t nbytes, MrcMap* m, int* mode, bool* swap, int64_t* data_off) {
    if (nbytes < kMrcHeader) return VC_ERR_ARG;
    const uint8_t s0 = b[212], s1 = b[213];
    bool big = s0 == 0x11 && s1 == 0x11;
    if (!(s0 == 0x44 && (s1 == 0x44 || s1 == 0x41)) && !big) {
        // no stamp (older files): the byte order whose mode word is valid
        const int32_t le = word(b, 3, false);
        big = elem_size(le) == 0 && elem_size(word(b, 3, true)) != 0;
    }
    const int32_t n0 = word(b, 0, big), n1 = word(b, 1, big), n2 = word(b, 2, big), md = word(b, 3, big);
    const int32_t nsym = word(b, 23, big);
    if (n0 <= 0 || n1 <= 0 || n2 <= 0 || n0 > 32766 || n1 > 32766 || n2 > 32766 || elem_size(md) == 0 || nsym < 0)
        return VC_ERR_ARG;
    int ax[3] = {word(b, 16, big) - 1, word(b, 17, big) - 1, word(b, 18, big) - 1};
    const bool perm = ax[0] >= 0 && ax[0] < 3 && ax[1] >= 0 && ax[1] < 3 && ax[2] >= 0 && ax[2] < 3 &&
                      ax[0] != ax[1] && ax[1] != ax[2] && ax[0] != ax[2];
    if (!perm) ax[0] = 0, ax[1] = 1, ax[2] = 2;
    const int64_t n = (int64_t)n0 * n1 * n2;
    const int64_t off = (int64_t)kMrcHeader + nsym;
    if (nbytes < off || (nbytes - off) / elem_size(md) < n) return VC_ERR_ARG;  // truncated
    m->n[0] = n0;
    m->n[1] = n1;
    m->n[2] = n2;
    for (int k = 0; k < 3; ++k) {
        m->axis[k] = ax[k];
        m->dim[ax[k]] = m->n[k];
    }
    if ((int64_t)(m->dim[0] + 1) * (m->dim[1] + 1) * (m->dim[2] + 1) >= ((int64_t)1 << 33)) return VC_ERR_ARG;
    *mode = md;
    *swap = big;
    *data_off = off;
    return VC_OK;
}

int install_mrc(vc_ctx* c, const uint8_t* bytes, int64_t nbytes, int* dims) {
    MrcMap m{};
    int mode = 0;
    bool swap = false;
    int64_t off = 0;
    VC_TRY(mrc_header(bytes, nbytes, &m, &mode, &swap, &off));
    const int64_t nvox = (int64_t)m.dim[0] * m.dim[1] * m.dim[2];
    const int64_t raw_bytes = nvox * elem_size(mode);
    // results of the previous volume are stale from here on
    c->n_sites = -1;
    c->ft_valid = c->vd_valid = false;
    VC_TRY(ensure_n<uint8_t>(c, c->oct_stream, raw_bytes));
    VC_TRY(ensure_n<uint8_t>(c, c->occ, nvox));
    VC_CUDA(c, cudaMemcpyAsync(c->oct_stream.p, bytes + off, (size_t)raw_bytes, cudaMemcpyHostToDevice, c->stream));
    {
        Region r(c, "mrc_decode");
        const uint8_t* raw = ptr<uint8_t>(c->oct_stream);
        uint8_t* occ = ptr<uint8_t>(c->occ);
        switch (mode) {
            case 0: launch<int8_t>(c, raw, m, swap, occ); break;
            case 1: launch<int16_t>(c, raw, m, swap, occ); break;
            case 2: launch<float>(c, raw, m, swap, occ); break;
            case 6: launch<uint16_t>(c, raw, m, swap, occ); break;
            default: launch<Half16>(c, raw, m, swap, occ); break;
        }
        VC_CUDA(c, cudaGetLastError());
    }
    VC_TRY(set_volume_table(c, 1, m.dim));
    c->X = m.dim[0];
    c->Y = m.dim[1];
    c->Z = m.dim[2];
    c->sites_from_octree = false;
    c->oct_n_sites = 0;
    set_identity(c->vox_to_model);
    for (int k = 0; k < 3; ++k) dims[k] = m.dim[k];
    return sync_check(c);  // the caller's bytes may go once this returns
}

}  // namespace vc

extern "C" int vc_set_volume_mrc(vc_ctx* c, const void* bytes, int64_t nbytes, int* dims) {
    if (!c || !bytes || nbytes < 0 || !dims) return VC_ERR_ARG;
    if (cudaSetDevice(c->device) != cudaSuccess) return vc::cuda_fail(c, cudaGetLastError(), "cudaSetDevice");
    return vc::install_mrc(c, static_cast<const uint8_t*>(bytes), nbytes, dims);
}

extern "C" int vc_mrc_dims(const void* bytes, int64_t nbytes, int* dims) {
    if (!bytes || nbytes < 0 || !dims) return VC_ERR_ARG;
    vc::MrcMap m{};
    int mode = 0;
    bool swap = false;
    int64_t off = 0;
    const int s = vc::mrc_header(static_cast<const uint8_t*>(bytes), nbytes, &m, &mode, &swap, &off);
    if (s != VC_OK) return s;
    for (int k = 0; k < 3; ++k) dims[k] = m.dim[k];
    return VC_OK;
}
