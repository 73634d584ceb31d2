// voxelcore_gb300.hpp -- C++ host adapters over the C ABI (voxelcore_gb300.h)
// that keep the reference's class surfaces, so that code written against the
// reference (danielyan86129/voxel_ma) switches to the GPU path by including
// this header and naming the vcgpu namespace; the call sites stay as they are:
//
//   reference                                   GPU adapter
//   Surfacer().extractBoundaryVts(vol, vts)     vcgpu::Surfacer, same call, any volume
//     -> SurfacerErrCode (include/surfacing.h:   type with getSizeX/Y/Z and getDataAt,
//     17-27, 57-58)                              or a vcgpu::OctreeVolume
//   VoroInfo::extractInsideWithMeasure(         vcgpu::VoroInfo (the lattice Voronoi
//     MeasureForMA::LAMBDA, vts, edges, tris,    complex of a volume, which stands in
//     from_fi, vm, em, fm), getInsidePartSize,   for the TetGen diagram the reference
//     getRadii, getSitesOfFace                   loads)
//     (include/voroinfo.h:84-131)
//   cellcomplex(vts, edges, tris, finalize)     vcgpu::cellcomplex (owns a GPU context)
//     (include/cellcomplex.h:33-34)
//   CellComplexThinning::{setup,                vcgpu::CellComplexThinning
//     assignElementValues, preprocess, prune,
//     getRemainedVts/Edges/Faces,
//     getEdgeRemovedTags, getFaceRemovedTags,
//     remainingCC() and remainingCC(vts, edges,
//     tris, from_fi)} (include/ccthin.h:57-113)
//   nClosedComponents (highlevelalgo.cpp:993)   vcgpu::nClosedComponents
//   OctreeVolume(filename) (.sof / .sog,        vcgpu::OctreeVolume
//     octree.cpp:22-47), writeToFile (:66-83)
//   readVolume / readMRC / readOctree           vcgpu::readVolume / readMRC / readOctree
//     -> ImportErrCode (importers.h:10-36)       (vcgpu::MRCVolume, vcgpu::OctreeVolume)
//   writeToPLY, writeToDotma                    vcgpu::writeToPLY, vcgpu::writeToDotma
//     (exporters.cpp:244-287, 341-476)
//
// Objects the reference constructs without arguments get a GPU context of
// their own (cellcomplex, VoroInfo, OctreeVolume) or share one per device
// (Surfacer); the device is $VC_GB300_DEVICE, else 0.  Every adapter also
// takes an explicit vcgpu::Context to place the work.  Point types are any
// type with operator[] over 3 floats (trimesh::point), edges any type with
// operator[] over 2 ints (trimesh::ivec2), triangles any type with
// operator[] over 3 ints (uTriFace).  Where the reference returns an error
// code (SurfacerErrCode, ExportErrCode) so does the adapter; elsewhere
// errors are vcgpu::Error exceptions carrying the VC_ERR_* status (the
// reference exits the process on its invariant check, ccthin.cpp:570-584;
// here the caller decides).  Header-only; link against libvoxelcore_gb300.so.
#pragma once

#include <array>
#include <cctype>
#include <cstdint>
#include <cstdlib>
#include <fstream>
#include <iterator>
#include <map>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <vector>

#include "voxelcore_gb300.h"

namespace vcgpu {

class Error : public std::runtime_error {
public:
    Error(int status, const std::string& what) : std::runtime_error(what), status(status) {}
    int status;
};

inline void check(vc_ctx* c, int s, const char* where) {
    if (s != VC_OK) {
        std::string msg = std::string(where) + ": " + vc_status_string(s);
        if (c) msg += std::string(" (") + vc_ctx_last_error(c) + ")";
        throw Error(s, msg);
    }
}

// One GPU context (one CUDA stream on one device).
class Context {
public:
    explicit Context(int device = 0) : device_(device) {
        check(nullptr, vc_ctx_create(&c_, device), "vc_ctx_create");
    }
    ~Context() { vc_ctx_destroy(c_); }
    Context(const Context&) = delete;
    Context& operator=(const Context&) = delete;
    vc_ctx* get() const { return c_; }
    int device() const { return device_; }

private:
    vc_ctx* c_ = nullptr;
    int device_ = 0;
};
using ContextPtr = std::shared_ptr<Context>;

// The device of adapters built without a context: $VC_GB300_DEVICE, else 0.
inline int defaultDevice() {
    const char* s = std::getenv("VC_GB300_DEVICE");
    return s ? std::atoi(s) : 0;
}

// One context per device shared by the adapters that hold no complex of
// their own (Surfacer).  Kept until the process exits (never destroyed, so
// no CUDA call runs during static destruction).
inline ContextPtr sharedContext(int device = defaultDevice()) {
    static std::mutex mu;
    static auto* ctxs = new std::map<int, ContextPtr>();
    std::lock_guard<std::mutex> lk(mu);
    ContextPtr& p = (*ctxs)[device];
    if (!p) p = std::make_shared<Context>(device);
    return p;
}

// A caller's context, not owned.
inline ContextPtr borrow(Context& c) { return ContextPtr(&c, [](Context*) {}); }

// A dense occupancy volume: X*Y*Z bytes, x-major (z fastest), inside <=> > 0.
struct DenseVolume {
    const uint8_t* data;
    int X, Y, Z;
};

namespace detail {
template <int N, class T, class V>
std::vector<T> flatten(const std::vector<V>& v) {
    std::vector<T> out(v.size() * N);
    for (size_t i = 0; i < v.size(); ++i)
        for (int k = 0; k < N; ++k) out[N * i + k] = (T)v[i][k];
    return out;
}
template <int N, class V, class T>
void unflatten(const std::vector<T>& in, std::vector<V>& out) {
    out.resize(in.size() / N);
    for (size_t i = 0; i < out.size(); ++i)
        for (int k = 0; k < N; ++k) out[i][k] = in[N * i + k];
}
inline bool ends_with(const std::string& s, const char* ext) {
    const std::string e(ext);
    return s.size() >= e.size() && s.compare(s.size() - e.size(), e.size(), e) == 0;
}
// The occupancy of any volume type with the reference's Volume3DScalar
// interface (getSizeX/Y/Z, getDataAt(x, y, z) > 0 inside; spaceinfo.h:122-135).
template <class V>
std::vector<uint8_t> sample_occupancy(const V& vol) {
    const int X = vol.getSizeX(), Y = vol.getSizeY(), Z = vol.getSizeZ();
    std::vector<uint8_t> occ((size_t)X * Y * Z);
    for (int x = 0; x < X; ++x)
        for (int y = 0; y < Y; ++y)
            for (int z = 0; z < Z; ++z) occ[((size_t)x * Y + y) * Z + z] = vol.getDataAt(x, y, z) > 0 ? 1 : 0;
    return occ;
}
}  // namespace detail

// ---- volumes read from files ----------------------------------------------
// A volume decoded on the GPU into a context of its own: an octree (.sof /
// .sog) or an MRC map.  getSizeX/Y/Z and getDataAt read it as the
// reference's Volume3DScalar does (the occupancy is read back once, on first
// use); the Surfacer and VoroInfo adapters use it where it lies.
class GpuVolume {
public:
    virtual ~GpuVolume() = default;
    int getSizeX() const { return dims_[0]; }
    int getSizeY() const { return dims_[1]; }
    int getSizeZ() const { return dims_[2]; }
    double getDataAt(int x, int y, int z) const {
        if (x < 0 || y < 0 || z < 0 || x >= dims_[0] || y >= dims_[1] || z >= dims_[2]) return 0.0;
        if (occ_.empty()) {
            occ_.resize((size_t)dims_[0] * dims_[1] * dims_[2]);
            check(ctx_->get(), vc_get_volume(ctx_->get(), occ_.data(), VC_MEM_HOST), "vc_get_volume");
        }
        return occ_[((size_t)x * dims_[1] + y) * dims_[2] + z];
    }
    Context& context() const { return *ctx_; }

protected:
    explicit GpuVolume(ContextPtr ctx) : ctx_(std::move(ctx)) {}
    static std::vector<char> read_file(const std::string& filename) {
        std::ifstream f(filename, std::ios::binary);
        if (!f) throw Error(VC_ERR_ARG, "cannot open " + filename);
        return std::vector<char>((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
    }
    ContextPtr ctx_;
    int dims_[3] = {0, 0, 0};
    mutable std::vector<uint8_t> occ_;
};

// OctreeVolume(const char* filename) (octree.cpp:22-47): a .sof or .sog file,
// chosen by its extension ((R+1)^3 voxels, the octree site rule, and for
// .sog its voxel-to-model matrix).
class OctreeVolume : public GpuVolume {
public:
    explicit OctreeVolume(const std::string& filename)
        : OctreeVolume(std::make_shared<Context>(defaultDevice()), filename) {}
    OctreeVolume(Context& ctx, const std::string& filename) : OctreeVolume(borrow(ctx), filename) {}
    int getMaxRes() const { return dims_[0] - 1; }  // R
    int size() const { return dims_[0]; }           // voxels per axis, R + 1

private:
    OctreeVolume(ContextPtr ctx, const std::string& filename) : GpuVolume(std::move(ctx)) {
        const bool sog = detail::ends_with(filename, ".sog"), sof = detail::ends_with(filename, ".sof");
        if (!sog && !sof) throw Error(VC_ERR_ARG, "not a .sof or .sog file: " + filename);
        const std::vector<char> bytes = read_file(filename);
        vc_ctx* c = ctx_->get();
        int n = 0;
        check(c, (sog ? vc_set_volume_sog : vc_set_volume_sof)(c, bytes.data(), (int64_t)bytes.size(), &n),
              sog ? "vc_set_volume_sog" : "vc_set_volume_sof");
        dims_[0] = dims_[1] = dims_[2] = n;
    }
};

// An .mrc density map (readMRC, importers.cpp:45-60), inside <=> value > 0.
class MRCVolume : public GpuVolume {
public:
    explicit MRCVolume(const std::string& filename) : MRCVolume(std::make_shared<Context>(defaultDevice()), filename) {}
    MRCVolume(Context& ctx, const std::string& filename) : MRCVolume(borrow(ctx), filename) {}

private:
    MRCVolume(ContextPtr ctx, const std::string& filename) : GpuVolume(std::move(ctx)) {
        const std::vector<char> bytes = read_file(filename);
        check(ctx_->get(), vc_set_volume_mrc(ctx_->get(), bytes.data(), (int64_t)bytes.size(), dims_),
              "vc_set_volume_mrc");
    }
};

// readVolume / readMRC / readOctree (importers.h:22-36), by extension.
enum class ImportErrCode { FAILURE, SUCCESS, NOOPENINPUT, INVALID_VOL_FILE, INVALID_FORMAT };

namespace detail {
template <class Make>
ImportErrCode read_into(const char* file, std::shared_ptr<GpuVolume>& vol, Make make) {
    if (!std::ifstream(file, std::ios::binary)) return ImportErrCode::NOOPENINPUT;
    try {
        vol = make();
    } catch (const Error&) {
        vol.reset();
        return ImportErrCode::INVALID_FORMAT;
    }
    return ImportErrCode::SUCCESS;
}
}  // namespace detail
inline ImportErrCode readMRC(const char* file, std::shared_ptr<GpuVolume>& vol) {
    return detail::read_into(file, vol, [&] { return std::make_shared<MRCVolume>(file); });
}
inline ImportErrCode readOctree(const char* file, std::shared_ptr<GpuVolume>& vol) {
    return detail::read_into(file, vol, [&] { return std::make_shared<OctreeVolume>(file); });
}
inline ImportErrCode readVolume(const char* file, std::shared_ptr<GpuVolume>& vol) {
    std::string f(file);
    for (auto& ch : f) ch = (char)std::tolower((unsigned char)ch);
    if (detail::ends_with(f, ".mrc")) return readMRC(file, vol);
    if (detail::ends_with(f, ".sof") || detail::ends_with(f, ".sog")) return readOctree(file, vol);
    return ImportErrCode::INVALID_VOL_FILE;
}

// ---- boundary sites --------------------------------------------------------
enum class SurfacerErrCode { FAILURE, SUCCESS, EMPTY_VOL, INVALID_VOL_TYPE };  // include/surfacing.h:17-27

class Surfacer {
public:
    Surfacer() : ctx_(sharedContext()) {}
    explicit Surfacer(Context& ctx) : ctx_(borrow(ctx)) {}
    Context& context() const { return *ctx_; }

    // Surfacer::extractBoundaryVts(const shared_ptr<Volume3DScalar>&,
    // vector<point>&): boundary voxel corners in the reference's
    // first-encounter order, for any volume type with the Volume3DScalar
    // interface.  The occupancy is sampled on the host (one getDataAt per
    // voxel) and the sites are computed on the GPU.
    template <class V, class P, std::enable_if_t<!std::is_base_of<GpuVolume, V>::value, int> = 0>
    SurfacerErrCode extractBoundaryVts(const std::shared_ptr<V>& vol, std::vector<P>& vts) {
        if (!vol || vol->getSizeX() <= 0 || vol->getSizeY() <= 0 || vol->getSizeZ() <= 0)
            return SurfacerErrCode::EMPTY_VOL;
        const std::vector<uint8_t> occ = detail::sample_occupancy(*vol);
        return extract(ctx_->get(), &occ, vol->getSizeX(), vol->getSizeY(), vol->getSizeZ(), vts);
    }
    // A volume read from a file lies on its own context already: an MRC map
    // by the dense rule, an octree by the reference's octree rule
    // (surfacing.cpp:286-301, 666-685).
    template <class V, class P, std::enable_if_t<std::is_base_of<GpuVolume, V>::value, int> = 0>
    SurfacerErrCode extractBoundaryVts(const std::shared_ptr<V>& vol, std::vector<P>& vts) {
        if (!vol || vol->getSizeX() <= 0) return SurfacerErrCode::EMPTY_VOL;
        return extract(vol->context().get(), nullptr, 0, 0, 0, vts);
    }
    template <class P>
    SurfacerErrCode extractBoundaryVts(const DenseVolume& vol, std::vector<P>& vts) {
        if (!vol.data || vol.X <= 0 || vol.Y <= 0 || vol.Z <= 0) return SurfacerErrCode::EMPTY_VOL;
        return extract_raw(ctx_->get(), vol.data, vol.X, vol.Y, vol.Z, vts);
    }

private:
    template <class P>
    static SurfacerErrCode extract(vc_ctx* c, const std::vector<uint8_t>* occ, int X, int Y, int Z,
                                   std::vector<P>& vts) {
        return extract_raw(c, occ ? occ->data() : nullptr, X, Y, Z, vts);
    }
    template <class P>
    static SurfacerErrCode extract_raw(vc_ctx* c, const uint8_t* occ, int X, int Y, int Z, std::vector<P>& vts) {
        if (occ && vc_set_volume(c, occ, X, Y, Z, VC_MEM_HOST) != VC_OK) return SurfacerErrCode::FAILURE;
        int64_t n = 0;
        if (vc_extract_sites(c, &n) != VC_OK) return SurfacerErrCode::FAILURE;
        std::vector<float> xyz((size_t)n * 3);
        if (n > 0 && vc_get_sites(c, xyz.data(), VC_MEM_HOST) != VC_OK) return SurfacerErrCode::FAILURE;
        detail::unflatten<3>(xyz, vts);
        return SurfacerErrCode::SUCCESS;
    }
    ContextPtr ctx_;
};

// ---- the Voronoi complex with measures -------------------------------------
namespace MeasureForMA {
enum meassuretype { LAMBDA };  // include/measureforMA.h: the measure the thinning uses
}

namespace detail {
// The lattice Voronoi complex of the volume (and sites) installed in `c`.
inline vc_vd_sizes lattice_vd(vc_ctx* c) {
    int64_t n = 0;
    check(c, vc_extract_sites(c, &n), "vc_extract_sites");  // no work if the sites are there already
    check(c, vc_feature_transform(c), "vc_feature_transform");
    vc_vd_sizes s{};
    check(c, vc_lattice_vd(c, &s), "vc_lattice_vd");
    return s;
}
template <class P, class E, class T>
void read_vd(vc_ctx* c, const vc_vd_sizes& s, std::vector<P>& vts, std::vector<E>& edges, std::vector<T>& tris,
             std::vector<int>& from_fi, std::vector<float>& vts_msure, std::vector<float>& edges_msure,
             std::vector<float>& faces_msure) {
    std::vector<float> v((size_t)s.nv * 3);
    std::vector<int32_t> e((size_t)s.ne * 2), t((size_t)s.nt * 3), tf((size_t)s.nt);
    vts_msure.resize((size_t)s.nv);
    edges_msure.resize((size_t)s.ne);
    faces_msure.resize((size_t)s.nt);
    check(c, vc_get_vd(c, v.data(), e.data(), t.data(), tf.data(), vts_msure.data(), edges_msure.data(),
                       faces_msure.data(), nullptr, VC_MEM_HOST),
          "vc_get_vd");
    unflatten<3>(v, vts);
    unflatten<2>(e, edges);
    unflatten<3>(t, tris);
    from_fi.assign(tf.begin(), tf.end());
}
}  // namespace detail

// VoroInfo for the lattice Voronoi complex of a volume.  The reference loads
// a TetGen diagram (loadFromTetgenFiles, voroinfo.cpp:113-251); here the
// diagram is read off the exact feature transform of the volume's boundary
// sites.  Built from a volume (its own context), or from the volume and
// sites a Surfacer already installed in a given context (nothing is uploaded
// or extracted again).
class VoroInfo {
public:
    template <class V, std::enable_if_t<!std::is_base_of<GpuVolume, V>::value, int> = 0>
    explicit VoroInfo(const std::shared_ptr<V>& vol) : ctx_(std::make_shared<Context>(defaultDevice())) {
        const std::vector<uint8_t> occ = detail::sample_occupancy(*vol);
        check(ctx_->get(), vc_set_volume(ctx_->get(), occ.data(), vol->getSizeX(), vol->getSizeY(), vol->getSizeZ(),
                                         VC_MEM_HOST),
              "vc_set_volume");
        sizes_ = detail::lattice_vd(ctx_->get());
    }
    // a volume read from a file: on its own context, kept alive with it
    template <class V, std::enable_if_t<std::is_base_of<GpuVolume, V>::value, int> = 0>
    explicit VoroInfo(const std::shared_ptr<V>& vol) : ctx_(borrow(vol->context())), keep_(vol) {
        sizes_ = detail::lattice_vd(ctx_->get());
    }
    explicit VoroInfo(Context& ctx) : ctx_(borrow(ctx)) { sizes_ = detail::lattice_vd(ctx_->get()); }

    // extractInsideWithMeasure(MeasureForMA::LAMBDA, vts, edges, tris,
    // from_fi, vts_msure, edges_msure, faces_msure) (voroinfo.cpp:624-729)
    template <class P, class E, class T>
    void extractInsideWithMeasure(MeasureForMA::meassuretype, std::vector<P>& vts, std::vector<E>& edges,
                                  std::vector<T>& tris, std::vector<int>& from_fi, std::vector<float>& vts_msure,
                                  std::vector<float>& edges_msure, std::vector<float>& faces_msure) const {
        detail::read_vd(ctx_->get(), sizes_, vts, edges, tris, from_fi, vts_msure, edges_msure, faces_msure);
    }
    float getInsidePartSize() const { return sizes_.inside_size; }  // voroinfo.cpp:496
    // radius per vertex of the inside part (voroinfo.cpp:286-325)
    const std::vector<float>& getRadii() const {
        if (radii_.empty() && sizes_.nv > 0) {
            radii_.resize((size_t)sizes_.nv);
            check(ctx_->get(), vc_vertex_radii(ctx_->get(), radii_.data(), VC_MEM_HOST), "vc_vertex_radii");
        }
        return radii_;
    }
    // the two sites of Voronoi face fi (the from_fi ids of the inside triangles)
    std::array<int, 2> getSitesOfFace(int fi) const {
        if (face_sites_.empty() && sizes_.nface > 0) {
            face_sites_.resize(2 * (size_t)sizes_.nface);
            check(ctx_->get(),
                  vc_get_vd(ctx_->get(), nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr,
                            face_sites_.data(), VC_MEM_HOST),
                  "vc_get_vd");
        }
        return {face_sites_[2 * (size_t)fi], face_sites_[2 * (size_t)fi + 1]};
    }
    const vc_vd_sizes& sizes() const { return sizes_; }
    Context& context() const { return *ctx_; }

private:
    ContextPtr ctx_;
    std::shared_ptr<GpuVolume> keep_;
    vc_vd_sizes sizes_{};
    mutable std::vector<float> radii_;
    mutable std::vector<int32_t> face_sites_;
};

// The same as free functions on a caller's context.  With a volume: install
// it and compute everything; without one: use the volume and sites the
// context holds (e.g. after Surfacer(ctx).extractBoundaryVts on it).
// Returns the inside-part size used for the thinning threshold.
template <class P, class E, class T>
float extractInsideWithMeasure(Context& ctx, const DenseVolume& vol, std::vector<P>& vts, std::vector<E>& edges,
                               std::vector<T>& tris, std::vector<int>& from_fi, std::vector<float>& vts_msure,
                               std::vector<float>& edges_msure, std::vector<float>& faces_msure) {
    vc_ctx* c = ctx.get();
    check(c, vc_set_volume(c, vol.data, vol.X, vol.Y, vol.Z, VC_MEM_HOST), "vc_set_volume");
    const vc_vd_sizes s = detail::lattice_vd(c);
    detail::read_vd(c, s, vts, edges, tris, from_fi, vts_msure, edges_msure, faces_msure);
    return s.inside_size;
}
template <class P, class E, class T>
float extractInsideWithMeasure(Context& ctx, std::vector<P>& vts, std::vector<E>& edges, std::vector<T>& tris,
                               std::vector<int>& from_fi, std::vector<float>& vts_msure,
                               std::vector<float>& edges_msure, std::vector<float>& faces_msure) {
    const vc_vd_sizes s = detail::lattice_vd(ctx.get());
    detail::read_vd(ctx.get(), s, vts, edges, tris, from_fi, vts_msure, edges_msure, faces_msure);
    return s.inside_size;
}

// VoroInfo::getRadii after computeInfoRelatedtoSites (voroinfo.cpp:286-325),
// for the vertices extractInsideWithMeasure returned on this context.
template <class P>
void getRadii(Context& ctx, const std::vector<P>& vts, std::vector<float>& radii) {
    radii.resize(vts.size());
    check(ctx.get(), vc_vertex_radii(ctx.get(), radii.data(), VC_MEM_HOST), "vc_vertex_radii");
}

// ---- cell complex and thinning ---------------------------------------------
// cellcomplex(vts, edges, tris, finalize=true): the complex lives on the GPU,
// in a context of its own (or the caller's).  Copies share that context.
class cellcomplex {
public:
    template <class P, class E, class T>
    cellcomplex(const std::vector<P>& vts, const std::vector<E>& edges, const std::vector<T>& tris,
                bool perform_finalize = true)
        : cellcomplex(std::make_shared<Context>(defaultDevice()), vts, edges, tris, perform_finalize) {}
    template <class P, class E, class T>
    cellcomplex(Context& ctx, const std::vector<P>& vts, const std::vector<E>& edges, const std::vector<T>& tris,
                bool perform_finalize = true)
        : cellcomplex(borrow(ctx), vts, edges, tris, perform_finalize) {}
    template <class P, class E, class T>
    cellcomplex(ContextPtr ctx, const std::vector<P>& vts, const std::vector<E>& edges, const std::vector<T>& tris,
                bool perform_finalize = true)
        : ctx_(std::move(ctx)) {
        vts_ = detail::flatten<3, float>(vts);
        const auto e = detail::flatten<2, int32_t>(edges);
        const auto t = detail::flatten<3, int32_t>(tris);
        check(ctx_->get(),
              vc_set_complex(ctx_->get(), (int64_t)vts.size(), vts_.data(), (int64_t)edges.size(), e.data(),
                             (int64_t)tris.size(), t.data(), VC_MEM_HOST),
              "vc_set_complex");
        nv_ = (int64_t)vts.size();
        nt_ = (int64_t)tris.size();
        if (perform_finalize) finalize();
    }
    void finalize() { check(ctx_->get(), vc_finalize(ctx_->get(), &ne_), "vc_finalize"); }
    size_t numVts() const { return (size_t)nv_; }
    size_t numEdges() const { return (size_t)ne_; }
    size_t numFaces() const { return (size_t)nt_; }
    std::array<float, 3> getVert(int i) const { return {vts_[3 * (size_t)i], vts_[3 * (size_t)i + 1], vts_[3 * (size_t)i + 2]}; }
    // the finalized edge i (finalize may append face sides to the given edges)
    std::array<int, 2> getEdge(int i) const {
        fetch();
        return {fin_edges_[2 * (size_t)i], fin_edges_[2 * (size_t)i + 1]};
    }
    // the finalized edge ids of triangle fi's sides, in face order
    std::array<int, 3> getFaceERep(int fi) const {
        fetch();
        return {tri_edges_[3 * (size_t)fi], tri_edges_[3 * (size_t)fi + 1], tri_edges_[3 * (size_t)fi + 2]};
    }
    Context& context() const { return *ctx_; }
    const std::vector<float>& vertexCoords() const { return vts_; }

private:
    void fetch() const {
        if (!fin_edges_.empty() || ne_ == 0) return;
        std::vector<int32_t> e(2 * (size_t)ne_), t(3 * (size_t)nt_), vo((size_t)nv_ + 1), vi(2 * (size_t)ne_),
            eo((size_t)ne_ + 1), ei(3 * (size_t)nt_);
        check(ctx_->get(),
              vc_get_finalized(ctx_->get(), e.data(), t.data(), vo.data(), vi.data(), eo.data(), ei.data(),
                               VC_MEM_HOST),
              "vc_get_finalized");
        fin_edges_.swap(e);
        tri_edges_.swap(t);
    }
    ContextPtr ctx_;
    std::vector<float> vts_;
    int64_t nv_ = 0, ne_ = 0, nt_ = 0;
    mutable std::vector<int32_t> fin_edges_, tri_edges_;
};

class CellComplexThinning {
public:
    void setup(cellcomplex* cc) { cc_ = cc; }
    void reset() { cc_ = nullptr; }
    // em is indexed by FINALIZED edge id (finalize may append face sides).
    void assignElementValues(const std::vector<float>& vm, const std::vector<float>& em,
                             const std::vector<float>& fm) {
        vc_ctx* c = cc_->context().get();
        check(c, vc_set_measures(c, vm.empty() ? nullptr : vm.data(), em.data(), fm.data(), VC_MEM_HOST),
              "vc_set_measures");
    }
    void preprocess() {}
    void prune(float f_t, float l_t, bool /*remove_small_components: unused by the reference*/) {
        vc_ctx* c = cc_->context().get();
        check(c, vc_thin(c, f_t, l_t, &stats_), "vc_thin");
        kv_.resize(cc_->numVts());
        ke_.resize(cc_->numEdges());
        kf_.resize(cc_->numFaces());
        re_.resize(cc_->numEdges());
        check(c, vc_get_thin_flags(c, kv_.data(), ke_.data(), kf_.data(), re_.data(), VC_MEM_HOST),
              "vc_get_thin_flags");
    }
    void getRemainedVts(std::vector<int>& ids) const { collect(kv_, ids); }
    void getRemainedEdges(std::vector<int>& ids) const { collect(ke_, ids); }
    void getRemainedFaces(std::vector<int>& ids) const { collect(kf_, ids); }
    std::vector<bool> getEdgeRemovedTags() const { return std::vector<bool>(re_.begin(), re_.end()); }
    std::vector<bool> getFaceRemovedTags() const {
        std::vector<bool> r(kf_.size());
        for (size_t i = 0; i < kf_.size(); ++i) r[i] = !kf_[i];
        return r;
    }
    // remainingCC(vts, edges, tris, from_fi) (ccthin.cpp:467-512): the
    // remaining complex, compacted; from_fi (optional) receives, per
    // remaining triangle, the id of the face it came from.
    template <class P, class E, class T>
    void remainingCC(std::vector<P>& vts, std::vector<E>& edges, std::vector<T>& tris,
                     std::vector<int>* from_fi = nullptr) const {
        vc_ctx* c = cc_->context().get();
        vc_rem_sizes s{};
        check(c, vc_remaining(c, &s), "vc_remaining");
        std::vector<float> v((size_t)s.nv * 3);
        std::vector<int32_t> e((size_t)s.ne * 2), t((size_t)s.nt * 3);
        check(c, vc_get_remaining(c, v.data(), e.data(), t.data(), VC_MEM_HOST), "vc_get_remaining");
        detail::unflatten<3>(v, vts);
        detail::unflatten<2>(e, edges);
        detail::unflatten<3>(t, tris);
        if (from_fi) getRemainedFaces(*from_fi);  // one triangle per remaining triangle face
    }
    // remainingCC() (ccthin.cpp:438-465): the remaining complex as a new,
    // finalized cell complex (in a context of its own).
    cellcomplex remainingCC() const {
        std::vector<std::array<float, 3>> v;
        std::vector<std::array<int, 2>> e;
        std::vector<std::array<int, 3>> t;
        remainingCC(v, e, t);
        return cellcomplex(v, e, t);
    }
    const vc_thin_stats& stats() const { return stats_; }

private:
    static void collect(const std::vector<uint8_t>& f, std::vector<int>& ids) {
        ids.clear();
        for (size_t i = 0; i < f.size(); ++i)
            if (f[i]) ids.push_back((int)i);
    }
    cellcomplex* cc_ = nullptr;
    vc_thin_stats stats_{};
    std::vector<uint8_t> kv_, ke_, kf_, re_;
};

// nClosedComponents(cc) (highlevelalgo.cpp:993-1020): the closed pockets an
// all-pass thinning of the complex leaves, as face-connected components.
inline int nClosedComponents(const cellcomplex& cc) {
    int64_t n = 0;
    check(cc.context().get(), vc_closed_components(cc.context().get(), &n), "vc_closed_components");
    return (int)n;
}

// OctreeVolume(const Volume3DScalar*) + writeToFile(filename): the octree of
// a dense volume written as .sof or .sog (by extension).  Host code.
inline bool writeOctreeFile(const DenseVolume& vol, const std::string& filename) {
    const bool sog = detail::ends_with(filename, ".sog");
    auto enc = sog ? vc_encode_sog : vc_encode_sof;
    int64_t n = 0;
    check(nullptr, enc(vol.data, vol.X, vol.Y, vol.Z, nullptr, 0, &n), "vc_encode_sof");
    std::vector<uint8_t> buf((size_t)n);
    check(nullptr, enc(vol.data, vol.X, vol.Y, vol.Z, buf.data(), n, &n), "vc_encode_sof");
    std::ofstream f(filename, std::ios::binary);
    f.write(reinterpret_cast<const char*>(buf.data()), (std::streamsize)buf.size());
    return (bool)f;
}

// ---- output formats (exporters.h) -----------------------------------------
enum class ExportErrCode { FAILURE, SUCCESS, INPUT_NOT_OPEN, OUTPUT_NOT_OPEN, INPUT_NOT_SUPPORTED, OUTPUT_NOT_SUPPORTED };

// writeToPLY(filename, vts, edges, tris, ...) (exporters.cpp:341-476): the
// file holds the vertices, edges and triangles (the measure and site
// arguments of the reference never reach its file).
template <class P, class E, class T>
ExportErrCode writeToPLY(const char* filename, const std::vector<P>& vts, const std::vector<E>& edges,
                         const std::vector<T>& tris) {
    const auto v = detail::flatten<3, float>(vts);
    const auto e = detail::flatten<2, int32_t>(edges);
    const auto t = detail::flatten<3, int32_t>(tris);
    return vc_write_ply(filename, v.data(), (int64_t)vts.size(), e.data(), (int64_t)edges.size(), t.data(),
                        (int64_t)tris.size()) == VC_OK
               ? ExportErrCode::SUCCESS
               : ExportErrCode::FAILURE;
}

// writeToDotma(filename, vts, edges, tri_faces, radii) (exporters.cpp:244-287)
template <class P, class E, class T>
ExportErrCode writeToDotma(const std::string& filename, const std::vector<P>& vts, const std::vector<E>& edges,
                           const std::vector<T>& tris, const std::vector<float>& radii) {
    if (radii.size() != vts.size()) return ExportErrCode::FAILURE;
    const auto v = detail::flatten<3, float>(vts);
    const auto e = detail::flatten<2, int32_t>(edges);
    const auto t = detail::flatten<3, int32_t>(tris);
    return vc_write_dotma(filename.c_str(), v.data(), radii.data(), (int64_t)vts.size(), e.data(),
                          (int64_t)edges.size(), t.data(), (int64_t)tris.size()) == VC_OK
               ? ExportErrCode::SUCCESS
               : ExportErrCode::FAILURE;
}

}  // namespace vcgpu
