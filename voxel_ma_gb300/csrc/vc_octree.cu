// Octree volume input: the .sof files of the reference's OctreeVolume
// (read_sof_file, src/octree.cpp:259-357), decoded on the GPU into the dense
// occupancy the rest of the path reads, and the reference's octree rule for
// the sites (Surfacer::extractBoundaryVts on an OctreeVolume,
// src/surfacing.cpp:286-301, 666-685).
//
// The stream is an int32 resolution R (a power of two), then the nodes in
// pre-order: a type byte -- 0 internal (eight children, x outermost, z
// innermost), 1 empty (a sign byte: 1 outside, anything else inside, for
// every cell of the cube), 2 leaf (one cell; bit 4x + 2y + z = corner
// (x, y, z) outside).  The host walks the nodes larger than 16^3 and skips
// over each subtree of edge <= 16 (one pass over the type bytes, which only
// counts open children), recording its root and first byte.  The stream goes
// to the device once; one thread per subtree walks it (vc_octree_walk.cuh),
// writing every cell's corner byte and counting its mixed leaves, and after
// a prefix over the counts a second walk writes the mixed leaves -- the
// sites, in stream order (the order of the reference's tree walk).  Larger
// empty nodes are one block each.  Every voxel of the (R + 1)^3 grid then
// reads its cell as OctreeVolume::getDataAt does (src/octree.cpp:233-256):
// its own cell's lowest corner, or, at a coordinate R, the last cell's far
// corner.
//
// .sog files (read_sog_file, src/octree.cpp:351-498) hold the same node
// stream after a 128-byte header (title, lower-left corner, bounding-box
// length), with R after the header and twelve more bytes after each leaf's
// corner byte (its feature point, skipped); they also set the volume's
// voxel-to-model matrix, which the exporters apply.
#include "vc_internal.cuh"
#include "vc_octree_walk.cuh"

#include <cstring>
#include <new>
#include <thread>

namespace vc {
namespace {

// .sog: a 128-byte header opening with the title "SOG.Format 1.0" and its
// terminator (15 bytes), then the lower-left corner and the bounding-box
// length as floats (src/octree.cpp:353-379, 569-605)
constexpr int64_t kSogHeader = 128;
constexpr int kSogTitle = 15;

__global__ void oct_large_kernel(const uint64_t* __restrict__ nodes, int64_t n, uint8_t* __restrict__ cell, int R) {
    for (int64_t i = blockIdx.x; i < n; i += gridDim.x) {
        const uint64_t nd = __ldg(nodes + i);
        const int len = 1 << oct_lg(nd), x = oct_x(nd), y = oct_y(nd), z = oct_z(nd);
        const uint8_t v = oct_v(nd);
        const int64_t cells = (int64_t)len * len * len;
        for (int64_t k = threadIdx.x; k < cells; k += blockDim.x) {
            const int cz = (int)(k % len);
            const int64_t ab = k / len;
            const int b = (int)(ab % len), a = (int)(ab / len);
            cell[((int64_t)(x + a) * R + (y + b)) * R + z + cz] = v;
        }
    }
}

// one thread per subtree; FILL: cells + mixed-leaf counts, else the leaves
template <bool FILL, int LEAF_EXTRA>
__global__ void oct_walk_kernel(const uint8_t* __restrict__ b, int64_t nbytes, const uint64_t* __restrict__ sub_node,
                                const int64_t* __restrict__ sub_pos, int64_t nsub, uint8_t* __restrict__ cell, int R,
                                int32_t* __restrict__ cnt, const int64_t* __restrict__ base,
                                uint64_t* __restrict__ leaves, int* err) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nsub) return;
    int64_t n = 0;
    if (oct_walk<FILL, LEAF_EXTRA>(b, nbytes, sub_pos[i], sub_node[i], cell, R, FILL ? nullptr : leaves + base[i], &n) != 0) {
        set_error(err, VC_ERR_ARG);
        return;
    }
    if (FILL) cnt[i] = (int32_t)n;  // a subtree holds at most 16^3 leaves
}

// voxel (x, y, z) of the (R + 1)^3 grid: inside iff its corner bit is 0
__global__ void oct_voxels_kernel(const uint8_t* __restrict__ cell, int R, uint8_t* __restrict__ occ) {
    const int64_t S = (int64_t)R + 1, n = S * S * S;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const int z = (int)(i % S);
        const int64_t xy = i / S;
        const int y = (int)(xy % S), x = (int)(xy / S);
        const int off = (x == R ? 4 : 0) | (y == R ? 2 : 0) | (z == R ? 1 : 0);
        const int cx = min(x, R - 1), cy = min(y, R - 1), cz = min(z, R - 1);
        const uint8_t v = __ldg(cell + ((int64_t)cx * R + cy) * R + cz);
        occ[i] = ((v >> off) & 1) == 0 ? 1 : 0;
    }
}

// the octree sites: centre of mixed leaf (x, y, z) = lattice point (x+1, y+1, z+1)
__global__ void oct_sites_kernel(const uint64_t* __restrict__ leaves, int64_t n, int S, float* __restrict__ xyz,
                                 int32_t* __restrict__ site_id_lat) {
    const int64_t L = (int64_t)S + 1;  // lattice points per axis
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const uint64_t p = __ldg(leaves + i);
        const int x = oct_x(p), y = oct_y(p), z = oct_z(p);
        xyz[3 * i + 0] = (float)x + 0.5f;
        xyz[3 * i + 1] = (float)y + 0.5f;
        xyz[3 * i + 2] = (float)z + 0.5f;
        site_id_lat[((int64_t)(x + 1) * L + (y + 1)) * L + (z + 1)] = (int32_t)i;
    }
}

inline int grid_of(vc_ctx* c, int64_t n, int threads) {
    return (int)std::max<int64_t>(1, std::min<int64_t>((n + threads - 1) / threads, (int64_t)c->num_sms * 16));
}

// Walk the nodes of edge > 16: the subtrees of edge <= 16 (root, first
// byte), in stream order, and the empty nodes above them.
// Skip one subtree: each node is one token, an internal one opens eight
// more.  The loop is one dependent chain (the type byte decides where the
// next one is), so the stride is kept to a compare and an add; LEAF_EXTRA is
// a constant.  Returns the byte after the subtree, or -1.
template <int LEAF_EXTRA>
int64_t skip_subtree(const uint8_t* b, int64_t nbytes, int64_t pos) {
    int64_t open = 1;
    while (open > 0) {
        if (pos >= nbytes) return -1;
        const uint8_t t = b[pos];
        if (t > 2) return -1;
        pos += LEAF_EXTRA ? (t == 0 ? 1 : t == 1 ? 2 : 2 + LEAF_EXTRA) : 1 + (t != 0);
        open += t == 0 ? 7 : -1;
    }
    return pos > nbytes ? -1 : pos;
}

// The resolution is the int32 at byte `start` (0 in .sof, after the 128-byte
// header in .sog); a leaf has leaf_extra bytes after its corner byte.
int split_sof(const uint8_t* b, int64_t nbytes, int64_t start, int leaf_extra, int& R,
              std::vector<uint64_t>& sub_node, std::vector<int64_t>& sub_pos, std::vector<uint64_t>& large) {
    if (nbytes < start + 4) return VC_ERR_ARG;
    int32_t r = 0;
    std::memcpy(&r, b + start, 4);
    if (r < 1 || (r & (r - 1)) != 0 || r > 16384) return VC_ERR_ARG;
    R = r;
    int lgR = 0;
    while ((1 << lgR) < R) ++lgR;
    struct Frame {
        int x, y, z, lg, child;
    };
    std::vector<Frame> stack;
    int64_t pos = start + 4;
    auto visit = [&](int x, int y, int z, int lg) -> int {
        if (lg <= kOctSubLg) {
            sub_node.push_back(oct_pack(x, y, z, lg, 0));
            sub_pos.push_back(pos);
            pos = leaf_extra ? skip_subtree<12>(b, nbytes, pos) : skip_subtree<0>(b, nbytes, pos);
            return pos < 0 ? VC_ERR_ARG : VC_OK;
        }
        if (pos >= nbytes) return VC_ERR_ARG;
        const uint8_t type = b[pos++];
        if (type == 0) {
            stack.push_back(Frame{x, y, z, lg, 0});
            return VC_OK;
        }
        if (type != 1 || pos >= nbytes) return VC_ERR_ARG;  // a leaf is one cell
        large.push_back(oct_pack(x, y, z, lg, b[pos++] == 1 ? 0xff : 0x00));
        return VC_OK;
    };
    VC_TRY(visit(0, 0, 0, lgR));
    while (!stack.empty()) {
        Frame& f = stack.back();
        if (f.child == 8) {
            stack.pop_back();
            continue;
        }
        const int h = 1 << (f.lg - 1), ch = f.child++;
        const Frame cur = f;  // visit() may grow the stack
        VC_TRY(visit(cur.x + (ch >> 2) * h, cur.y + ((ch >> 1) & 1) * h, cur.z + (ch & 1) * h, cur.lg - 1));
    }
    return VC_OK;
}

}  // namespace

int install_octree(vc_ctx* c, const uint8_t* bytes, int64_t nbytes, bool sog, int* size_out) {
    int R = 0;
    std::vector<uint64_t> sub_node, large;
    std::vector<int64_t> sub_pos;
    const int64_t start = sog ? kSogHeader : 0;
    // the stream goes to the device on a second host thread while this one
    // splits it; the thread is joined before anything else enters the stream
    VC_TRY(ensure_n<uint8_t>(c, c->oct_stream, nbytes));
    cudaError_t copy_err = cudaSuccess;
    std::thread copier([&] {
        copy_err = cudaSetDevice(c->device);
        if (copy_err == cudaSuccess)
            copy_err = cudaMemcpyAsync(c->oct_stream.p, bytes, (size_t)nbytes, cudaMemcpyHostToDevice, c->stream);
    });
    // the node lists grow with the stream's contents: running out of host
    // memory must neither escape the C ABI nor leave the copier joinable
    int split_rc = VC_OK;
    try {
        split_rc = split_sof(bytes, nbytes, start, sog ? 12 : 0, R, sub_node, sub_pos, large);
    } catch (const std::bad_alloc&) {
        split_rc = VC_ERR_OOM;
    }
    copier.join();
    VC_CUDA(c, copy_err);
    VC_TRY(split_rc);
    const int S = R + 1;
    if ((int64_t)(S + 1) * (S + 1) * (S + 1) >= ((int64_t)1 << 33) || S > 32766) return VC_ERR_ARG;
    const int64_t ncell = (int64_t)R * R * R, nvox = (int64_t)S * S * S;
    const int64_t nsub = (int64_t)sub_node.size(), nlarge = (int64_t)large.size();
    // node lists: sub roots | sub first bytes | leaf bases | large nodes | counts (int32)
    VC_TRY(ensure_n<uint8_t>(c, c->oct_cells, ncell));
    VC_TRY(ensure_n<uint64_t>(c, c->oct_nodes, 3 * nsub + nlarge + (nsub + 1) / 2 + 1));
    uint8_t* db = ptr<uint8_t>(c->oct_stream);
    uint8_t* cell = ptr<uint8_t>(c->oct_cells);
    uint64_t* d_node = ptr<uint64_t>(c->oct_nodes);
    int64_t* d_pos = reinterpret_cast<int64_t*>(d_node + nsub);
    int64_t* d_base = d_pos + nsub;
    uint64_t* d_large = reinterpret_cast<uint64_t*>(d_base + nsub);
    int32_t* d_cnt = reinterpret_cast<int32_t*>(d_large + nlarge);
    if (nsub) {
        VC_CUDA(c, cudaMemcpyAsync(d_node, sub_node.data(), nsub * sizeof(uint64_t), cudaMemcpyHostToDevice,
                                   c->stream));
        VC_CUDA(c, cudaMemcpyAsync(d_pos, sub_pos.data(), nsub * sizeof(int64_t), cudaMemcpyHostToDevice, c->stream));
    }
    if (nlarge)
        VC_CUDA(c, cudaMemcpyAsync(d_large, large.data(), nlarge * sizeof(uint64_t), cudaMemcpyHostToDevice,
                                   c->stream));
    std::vector<int32_t> cnt((size_t)nsub);
    {
        Region r(c, "octree_decode");
        if (nlarge) {
            oct_large_kernel<<<(int)std::min<int64_t>(nlarge, (int64_t)c->num_sms * 8), 256, 0, c->stream>>>(
                d_large, nlarge, cell, R);
            launched(c);
        }
        if (nsub) {  // none when the whole cube is one empty node
            auto walk = sog ? oct_walk_kernel<true, 12> : oct_walk_kernel<true, 0>;
            walk<<<(int)((nsub + 127) / 128), 128, 0, c->stream>>>(db, nbytes, d_node, d_pos, nsub, cell, R, d_cnt,
                                                                   nullptr, nullptr, dev_err(c));
            launched(c);
            VC_CUDA(c, cudaGetLastError());
            VC_CUDA(c, cudaMemcpyAsync(cnt.data(), d_cnt, nsub * sizeof(int32_t), cudaMemcpyDeviceToHost, c->stream));
        }
    }
    VC_TRY(sync_check(c));  // a malformed subtree stops here, before the installed volume changes
    std::vector<int64_t> base((size_t)nsub);
    int64_t nleaf = 0;
    for (int64_t i = 0; i < nsub; ++i) {
        base[i] = nleaf;
        nleaf += cnt[i];
    }
    VC_TRY(ensure_n<uint64_t>(c, c->oct_leaves, nleaf + 1));
    VC_TRY(ensure_n<uint8_t>(c, c->occ, nvox));
    {
        Region r(c, "octree_decode");
        if (nleaf) {
            VC_CUDA(c, cudaMemcpyAsync(d_base, base.data(), nsub * sizeof(int64_t), cudaMemcpyHostToDevice,
                                       c->stream));
            auto walk = sog ? oct_walk_kernel<false, 12> : oct_walk_kernel<false, 0>;
            walk<<<(int)((nsub + 127) / 128), 128, 0, c->stream>>>(db, nbytes, d_node, d_pos, nsub, cell, R, nullptr,
                                                                   d_base, ptr<uint64_t>(c->oct_leaves), dev_err(c));
            launched(c);
        }
        oct_voxels_kernel<<<grid_of(c, nvox, 256), 256, 0, c->stream>>>(cell, R, ptr<uint8_t>(c->occ));
        launched(c);
        VC_CUDA(c, cudaGetLastError());
    }
    const int32_t dims[3] = {S, S, S};
    VC_TRY(set_volume_table(c, 1, dims));
    c->X = c->Y = c->Z = S;
    c->n_sites = -1;
    c->ft_valid = c->vd_valid = false;
    c->oct_n_sites = nleaf;
    c->sites_from_octree = true;
    set_identity(c->vox_to_model);
    if (sog) {
        // read_sof's header: lower-left corner and bounding-box length (floats
        // after the title); vox-to-mesh = trans(lower-left) * scale(len / R)
        float ll[3], len;
        std::memcpy(ll, bytes + kSogTitle, 12);
        std::memcpy(&len, bytes + kSogTitle + 12, 4);
        const double sc = (double)len / (double)R;
        c->vox_to_model[0] = c->vox_to_model[5] = c->vox_to_model[10] = sc;
        c->vox_to_model[12] = ll[0];
        c->vox_to_model[13] = ll[1];
        c->vox_to_model[14] = ll[2];
    }
    if (size_out) *size_out = S;
    return sync_check(c);  // the host lists go out of scope
}

// The octree rule for the sites (run_sites calls it for an octree volume):
// the centres of the mixed leaves, in stream order; the packed occupancy
// words are written as for a dense volume.
int octree_sites(vc_ctx* c, uint32_t* bits, int32_t* cnt, int64_t nwords, int64_t* total, int64_t* n_out) {
    const int64_t n = c->oct_n_sites;
    const int64_t nlat = c->h_off[kLat][c->nvol];
    VC_TRY(ensure_n<float>(c, c->site_xyz, 3 * n + 3));
    // per-volume site bases: one volume, n sites
    VC_CUDA(c, cudaMemsetAsync(cnt, 0, (size_t)std::max<int64_t>(nwords, 1) * sizeof(int32_t), c->stream));
    VC_CUDA(c, cudaMemcpyAsync(total, &n, sizeof(int64_t), cudaMemcpyHostToDevice, c->stream));
    VC_TRY(fill_bases(c, kBSite, kVWord, cnt, total));
    VC_CUDA(c, cudaMemsetAsync(c->site_id_lat.p, 0xff, (size_t)nlat * sizeof(int32_t), c->stream));
    if (n > 0) {
        oct_sites_kernel<<<grid_of(c, n, 256), 256, 0, c->stream>>>(ptr<uint64_t>(c->oct_leaves), n, c->X,
                                                                     ptr<float>(c->site_xyz),
                                                                     ptr<int32_t>(c->site_id_lat));
        launched(c);
    }
    VC_CUDA(c, cudaGetLastError());
    (void)bits;
    *n_out = n;
    return sync_check(c);  // n is read from host memory by the copy above
}

}  // namespace vc

extern "C" int vc_set_volume_sof(vc_ctx* c, const void* bytes, int64_t nbytes, int* size) {
    if (!c || !bytes || nbytes < 0) return VC_ERR_ARG;
    if (cudaSetDevice(c->device) != cudaSuccess) return vc::cuda_fail(c, cudaGetLastError(), "cudaSetDevice");
    return vc::install_octree(c, static_cast<const uint8_t*>(bytes), nbytes, false, size);
}

extern "C" int vc_set_volume_sog(vc_ctx* c, const void* bytes, int64_t nbytes, int* size) {
    if (!c || !bytes || nbytes < 0) return VC_ERR_ARG;
    if (nbytes < vc::kSogHeader || std::memcmp(bytes, "SOG.Format 1.0", vc::kSogTitle) != 0) return VC_ERR_ARG;
    if (cudaSetDevice(c->device) != cudaSuccess) return vc::cuda_fail(c, cudaGetLastError(), "cudaSetDevice");
    return vc::install_octree(c, static_cast<const uint8_t*>(bytes), nbytes, true, size);
}

extern "C" int vc_get_vox_to_model(vc_ctx* c, double* m) {
    if (!c || !m) return VC_ERR_ARG;
    std::memcpy(m, c->vox_to_model, sizeof c->vox_to_model);
    return VC_OK;
}

// ---------------------------------------------------------------------------
// Writing: the .sof stream of a dense occupancy volume as the reference
// writes it (OctreeVolume(const Volume3DScalar*), src/octree.cpp:50-63 and
// build, :864-930; write_sof_file, :499-560).  R is the smallest power of two
// >= max(X, Y, Z) - 1 (util::log2Int); a cube that does not touch the volume
// (closed boxes, util::intersect) is an empty node with sign 1; a cell is a
// leaf whose bit 4i + 2j + k is set when voxel (x+i, y+j, z+k) is outside;
// eight children that are all uniform with one sign merge into an empty
// node.  Built bottom-up (one byte of state per node and level), then
// written in pre-order.
namespace vc {
namespace {

// node state: bit 7 uniform, bit 0 its sign; bits 1-2 the type to write
// (0 internal, 1 empty, 2 leaf); leaves keep their corner byte separately
constexpr uint8_t kUni = 0x80;

inline int log2_int(int n) {  // util::log2Int: ceil(log2(n)), 0 for n <= 1
    int hib = 0;
    if (n) {
        int m = n, r = 1;
        while (m >>= 1) ++r;
        hib = r - 1;
    }
    return hib + ((1 << hib) < n ? 1 : 0);
}

}  // namespace

// sog: write_sog_file's layout (src/octree.cpp:569-668): the 128-byte header
// (title, lower-left 0, length R; the reference leaves the rest of the header
// uninitialised, here it is zero), R, then the nodes with each leaf's feature
// point, its cell centre, as three floats.
int encode_sof(const uint8_t* occ, int X, int Y, int Z, bool sog, std::vector<uint8_t>& out) {
    const int mx = std::max(X, std::max(Y, Z));
    const int R = 1 << log2_int(mx - 1);
    auto inside = [&](int x, int y, int z) -> bool {
        return x >= 0 && y >= 0 && z >= 0 && x < X && y < Y && z < Z && occ[((int64_t)x * Y + y) * Z + z] > 0;
    };
    auto touches = [&](int x, int y, int z, int l) {  // closed boxes [p, p+l] and [0, size]
        return !(x > X || y > Y || z > Z);  // p >= 0 and 0 <= p + l always
    };
    // levels: level k holds (R >> k)^3 nodes
    int nlev = 0;
    while ((1 << nlev) <= R) ++nlev;  // len 1 .. R
    std::vector<std::vector<uint8_t>> st(nlev);
    std::vector<uint8_t> leafv((size_t)R * R * R);
    // level 0: cells
    st[0].assign((size_t)R * R * R, 0);
    {
        const int nth = (int)std::max(1u, std::min(32u, std::thread::hardware_concurrency()));
        std::vector<std::thread> th;
        for (int t = 0; t < nth; ++t)
            th.emplace_back([&, t] {
                for (int x = t; x < R; x += nth)
                    for (int y = 0; y < R; ++y)
                        for (int z = 0; z < R; ++z) {
                            const size_t i = ((size_t)x * R + y) * R + z;
                            if (!touches(x, y, z, 1)) {
                                st[0][i] = kUni | 1 | (1 << 1);  // empty, sign 1
                                continue;
                            }
                            uint8_t b = 0;
                            for (int a = 0; a < 2; ++a)
                                for (int c = 0; c < 2; ++c)
                                    for (int d = 0; d < 2; ++d)
                                        if (!inside(x + a, y + c, z + d)) b |= (uint8_t)(1 << (4 * a + 2 * c + d));
                            leafv[i] = b;
                            st[0][i] = (uint8_t)((b == 0x00 || b == 0xff ? kUni : 0) | (b & 1) | (2 << 1));  // leaf
                        }
            });
        for (auto& t : th) t.join();
    }
    for (int k = 1; k < nlev; ++k) {
        const int n = R >> k, l = 1 << k, nc = n * 2;
        st[k].assign((size_t)n * n * n, 0);
        for (int x = 0; x < n; ++x)
            for (int y = 0; y < n; ++y)
                for (int z = 0; z < n; ++z) {
                    uint8_t& s = st[k][((size_t)x * n + y) * n + z];
                    if (!touches(x * l, y * l, z * l, l)) {
                        s = kUni | 1 | (1 << 1);
                        continue;
                    }
                    bool uni = true;
                    int sign = -1;
                    for (int a = 0; a < 2 && uni; ++a)
                        for (int c = 0; c < 2 && uni; ++c)
                            for (int d = 0; d < 2 && uni; ++d) {
                                const uint8_t cs = st[k - 1][((size_t)(2 * x + a) * nc + (2 * y + c)) * nc + 2 * z + d];
                                if (!(cs & kUni) || (sign >= 0 && (cs & 1) != sign)) uni = false;
                                else sign = cs & 1;
                            }
                    s = uni ? (uint8_t)(kUni | sign | (1 << 1)) : (uint8_t)0;  // merged empty, or internal
                }
    }
    // pre-order
    out.clear();
    const int32_t r32 = R;
    if (sog) {
        out.assign((size_t)kSogHeader, 0);
        std::memcpy(out.data(), "SOG.Format 1.0", kSogTitle);
        const float len = (float)R;
        std::memcpy(out.data() + kSogTitle + 12, &len, 4);
    }
    const size_t at = out.size();
    out.resize(at + 4);
    std::memcpy(out.data() + at, &r32, 4);
    struct F {
        int k, x, y, z, child;
    };
    std::vector<F> stack;
    auto emit = [&](int k, int x, int y, int z) {
        const int n = R >> k;
        const uint8_t s = st[k][((size_t)x * n + y) * n + z];
        const int type = (s >> 1) & 3;
        if (type == 0) {
            out.push_back(0);
            stack.push_back(F{k, x, y, z, 0});
        } else if (type == 1) {
            out.push_back(1);
            out.push_back((uint8_t)(s & 1));
        } else {
            out.push_back(2);
            out.push_back(leafv[((size_t)x * R + y) * R + z]);
            if (sog) {
                const float feat[3] = {(float)(x + 0.5), (float)(y + 0.5), (float)(z + 0.5)};
                const size_t q = out.size();
                out.resize(q + 12);
                std::memcpy(out.data() + q, feat, 12);
            }
        }
    };
    emit(nlev - 1, 0, 0, 0);
    while (!stack.empty()) {
        F& f = stack.back();
        if (f.child == 8) {
            stack.pop_back();
            continue;
        }
        const int a = f.child >> 2, c = (f.child >> 1) & 1, d = f.child & 1;
        ++f.child;
        const F cur = f;
        emit(cur.k - 1, 2 * cur.x + a, 2 * cur.y + c, 2 * cur.z + d);
    }
    return VC_OK;
}

}  // namespace vc

static int encode_octree(const uint8_t* occ, int X, int Y, int Z, bool sog, uint8_t* out, int64_t cap,
                         int64_t* nbytes) {
    if (!occ || !nbytes || X <= 0 || Y <= 0 || Z <= 0 || std::max(X, std::max(Y, Z)) > 16385) return VC_ERR_ARG;
    std::vector<uint8_t> buf;
    VC_TRY(vc::encode_sof(occ, X, Y, Z, sog, buf));
    *nbytes = (int64_t)buf.size();
    if (out) {
        if (cap < (int64_t)buf.size()) return VC_ERR_ARG;
        std::memcpy(out, buf.data(), buf.size());
    }
    return VC_OK;
}

extern "C" int vc_encode_sof(const uint8_t* occ, int X, int Y, int Z, uint8_t* out, int64_t cap, int64_t* nbytes) {
    return encode_octree(occ, X, Y, Z, false, out, cap, nbytes);
}

extern "C" int vc_encode_sog(const uint8_t* occ, int X, int Y, int Z, uint8_t* out, int64_t cap, int64_t* nbytes) {
    return encode_octree(occ, X, Y, Z, true, out, cap, nbytes);
}
