// voxelcore_gb300.hpp -- C++ host adapters over the C ABI (voxelcore_gb300.h)
// that keep the reference's class surfaces, so that code written against the
// reference (danielyan86129/voxel_ma) switches to the GPU path by changing a
// namespace:
//
//   reference                                   GPU adapter
//   Surfacer::extractBoundaryVts(vol, vts)      vcgpu::Surfacer::extractBoundaryVts
//     (include/surfacing.h:57-58)
//   cellcomplex(vts, edges, tris, finalize)     vcgpu::cellcomplex
//     (include/cellcomplex.h:33-34)
//   CellComplexThinning::{setup,                vcgpu::CellComplexThinning
//     assignElementValues, preprocess, prune,
//     getRemainedVts/Edges/Faces,
//     getEdgeRemovedTags, getFaceRemovedTags,
//     remainingCC}  (include/ccthin.h:57-113)
//   VoroInfo::extractInsideWithMeasure          vcgpu::extractInsideWithMeasure
//     (include/voroinfo.h:127-131), for the lattice Voronoi complex
//   VoroInfo::getRadii (voroinfo.cpp:286-325)   vcgpu::getRadii
//   nClosedComponents (highlevelalgo.cpp:993)   vcgpu::nClosedComponents
//   OctreeVolume(filename) (.sof / .sog,        vcgpu::OctreeVolume
//     octree.cpp:22-47), writeToFile (:66-83)
//   writeToPLY, writeToDotma                    vcgpu::writeToPLY, vcgpu::writeToDotma
//     (exporters.cpp:244-287, 341-476)
//
// Point types are any type with operator[] over 3 floats (trimesh::point),
// edges any type with operator[] over 2 ints (trimesh::ivec2), triangles any
// type with operator[] over 3 ints (uTriFace).  Errors are reported as
// vcgpu::Error exceptions carrying the VC_ERR_* status (the reference exits
// the process on its invariant check, ccthin.cpp:570-584; here the caller
// decides).  Header-only; link against libvoxelcore_gb300.so.
#pragma once

#include <cstdint>
#include <fstream>
#include <iterator>
#include <stdexcept>
#include <string>
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
    explicit Context(int device = 0) { check(nullptr, vc_ctx_create(&c_, device), "vc_ctx_create"); }
    ~Context() { vc_ctx_destroy(c_); }
    Context(const Context&) = delete;
    Context& operator=(const Context&) = delete;
    vc_ctx* get() const { return c_; }

private:
    vc_ctx* c_ = nullptr;
};

// A dense occupancy volume: X*Y*Z bytes, x-major (z fastest), inside <=> > 0.
struct DenseVolume {
    const uint8_t* data;
    int X, Y, Z;
};

class Surfacer {
public:
    explicit Surfacer(Context& ctx) : ctx_(ctx) {}
    // Surfacer::extractBoundaryVts: boundary voxel corners in the reference's
    // first-encounter order.  Returns true on success (the reference returns
    // SurfacerErrCode::SUCCESS).
    template <class P>
    bool extractBoundaryVts(const DenseVolume& vol, std::vector<P>& vts) {
        vc_ctx* c = ctx_.get();
        check(c, vc_set_volume(c, vol.data, vol.X, vol.Y, vol.Z, VC_MEM_HOST), "vc_set_volume");
        int64_t n = 0;
        check(c, vc_extract_sites(c, &n), "vc_extract_sites");
        std::vector<float> xyz((size_t)n * 3);
        check(c, vc_get_sites(c, xyz.data(), VC_MEM_HOST), "vc_get_sites");
        vts.resize((size_t)n);
        for (int64_t i = 0; i < n; ++i)
            for (int k = 0; k < 3; ++k) vts[(size_t)i][k] = xyz[(size_t)(3 * i + k)];
        return true;
    }

private:
    Context& ctx_;
};

// VoroInfo::extractInsideWithMeasure for the lattice Voronoi complex of a
// volume: vts, edges, tris, from_fi and the vertex / edge / triangle lambda
// measures, plus the inside-part size used for the thinning threshold.
template <class P, class E, class T>
float extractInsideWithMeasure(Context& ctx, const DenseVolume& vol, std::vector<P>& vts, std::vector<E>& edges,
                               std::vector<T>& tris, std::vector<int>& from_fi, std::vector<float>& vts_msure,
                               std::vector<float>& edges_msure, std::vector<float>& faces_msure) {
    vc_ctx* c = ctx.get();
    check(c, vc_set_volume(c, vol.data, vol.X, vol.Y, vol.Z, VC_MEM_HOST), "vc_set_volume");
    int64_t n = 0;
    check(c, vc_extract_sites(c, &n), "vc_extract_sites");
    check(c, vc_feature_transform(c), "vc_feature_transform");
    vc_vd_sizes s{};
    check(c, vc_lattice_vd(c, &s), "vc_lattice_vd");
    std::vector<float> v((size_t)s.nv * 3);
    std::vector<int32_t> e((size_t)s.ne * 2), t((size_t)s.nt * 3), tf((size_t)s.nt);
    vts_msure.resize((size_t)s.nv);
    edges_msure.resize((size_t)s.ne);
    faces_msure.resize((size_t)s.nt);
    check(c, vc_get_vd(c, v.data(), e.data(), t.data(), tf.data(), vts_msure.data(), edges_msure.data(),
                       faces_msure.data(), nullptr, VC_MEM_HOST),
          "vc_get_vd");
    vts.resize((size_t)s.nv);
    for (size_t i = 0; i < vts.size(); ++i)
        for (int k = 0; k < 3; ++k) vts[i][k] = v[3 * i + k];
    edges.resize((size_t)s.ne);
    for (size_t i = 0; i < edges.size(); ++i)
        for (int k = 0; k < 2; ++k) edges[i][k] = e[2 * i + k];
    tris.resize((size_t)s.nt);
    for (size_t i = 0; i < tris.size(); ++i)
        for (int k = 0; k < 3; ++k) tris[i][k] = t[3 * i + k];
    from_fi.assign(tf.begin(), tf.end());
    return s.inside_size;
}

// VoroInfo::getRadii after computeInfoRelatedtoSites (voroinfo.cpp:286-325),
// for the vertices extractInsideWithMeasure returned (the valid vertices
// writeRadiiToFile writes, exporters.cpp:478-552).
// `vts` is the vertex list extractInsideWithMeasure filled.
template <class P>
void getRadii(Context& ctx, const std::vector<P>& vts, std::vector<float>& radii) {
    radii.resize(vts.size());
    check(ctx.get(), vc_vertex_radii(ctx.get(), radii.data(), VC_MEM_HOST), "vc_vertex_radii");
}

// cellcomplex(vts, edges, tris, finalize=true): the complex lives on the GPU.
class cellcomplex {
public:
    template <class P, class E, class T>
    cellcomplex(Context& ctx, const std::vector<P>& vts, const std::vector<E>& edges, const std::vector<T>& tris,
                bool perform_finalize = true)
        : ctx_(ctx) {
        std::vector<float> v(vts.size() * 3);
        for (size_t i = 0; i < vts.size(); ++i)
            for (int k = 0; k < 3; ++k) v[3 * i + k] = (float)vts[i][k];
        std::vector<int32_t> e(edges.size() * 2), t(tris.size() * 3);
        for (size_t i = 0; i < edges.size(); ++i)
            for (int k = 0; k < 2; ++k) e[2 * i + k] = (int32_t)edges[i][k];
        for (size_t i = 0; i < tris.size(); ++i)
            for (int k = 0; k < 3; ++k) t[3 * i + k] = (int32_t)tris[i][k];
        vts_ = v;
        check(ctx_.get(),
              vc_set_complex(ctx_.get(), (int64_t)vts.size(), v.data(), (int64_t)edges.size(), e.data(),
                             (int64_t)tris.size(), t.data(), VC_MEM_HOST),
              "vc_set_complex");
        nv_ = (int64_t)vts.size();
        nt_ = (int64_t)tris.size();
        if (perform_finalize) finalize();
    }
    void finalize() { check(ctx_.get(), vc_finalize(ctx_.get(), &ne_), "vc_finalize"); }
    size_t numVts() const { return (size_t)nv_; }
    size_t numEdges() const { return (size_t)ne_; }
    size_t numFaces() const { return (size_t)nt_; }
    Context& context() const { return ctx_; }
    const std::vector<float>& vertexCoords() const { return vts_; }

private:
    Context& ctx_;
    std::vector<float> vts_;
    int64_t nv_ = 0, ne_ = 0, nt_ = 0;
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
    template <class P, class E, class T>
    void remainingCC(std::vector<P>& vts, std::vector<E>& edges, std::vector<T>& tris) const {
        vc_ctx* c = cc_->context().get();
        vc_rem_sizes s{};
        check(c, vc_remaining(c, &s), "vc_remaining");
        std::vector<float> v((size_t)s.nv * 3);
        std::vector<int32_t> e((size_t)s.ne * 2), t((size_t)s.nt * 3);
        check(c, vc_get_remaining(c, v.data(), e.data(), t.data(), VC_MEM_HOST), "vc_get_remaining");
        vts.resize((size_t)s.nv);
        for (size_t i = 0; i < vts.size(); ++i)
            for (int k = 0; k < 3; ++k) vts[i][k] = v[3 * i + k];
        edges.resize((size_t)s.ne);
        for (size_t i = 0; i < edges.size(); ++i)
            for (int k = 0; k < 2; ++k) edges[i][k] = e[2 * i + k];
        tris.resize((size_t)s.nt);
        for (size_t i = 0; i < tris.size(); ++i)
            for (int k = 0; k < 3; ++k) tris[i][k] = t[3 * i + k];
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

// ---- octree volumes -------------------------------------------------------
// OctreeVolume(const char* filename) (octree.cpp:22-47): a .sof or .sog file,
// chosen by its extension, installed as the context's volume ((R+1)^3 voxels,
// the octree site rule, and for .sog its voxel-to-model matrix).
class OctreeVolume {
public:
    OctreeVolume(Context& ctx, const std::string& filename) : ctx_(ctx) {
        std::ifstream f(filename, std::ios::binary);
        if (!f) throw Error(VC_ERR_ARG, "cannot open " + filename);
        const std::vector<char> bytes((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
        const bool sog = filename.size() >= 4 && filename.compare(filename.size() - 4, 4, ".sog") == 0;
        const bool sof = filename.size() >= 4 && filename.compare(filename.size() - 4, 4, ".sof") == 0;
        if (!sog && !sof) throw Error(VC_ERR_ARG, "not a .sof or .sog file: " + filename);
        vc_ctx* c = ctx.get();
        check(c, (sog ? vc_set_volume_sog : vc_set_volume_sof)(c, bytes.data(), (int64_t)bytes.size(), &size_),
              sog ? "vc_set_volume_sog" : "vc_set_volume_sof");
    }
    int getMaxRes() const { return size_ - 1; }  // R
    int size() const { return size_; }           // voxels per axis, R + 1

private:
    Context& ctx_;
    int size_ = 0;
};

// OctreeVolume(const Volume3DScalar*) + writeToFile(filename): the octree of
// a dense volume written as .sof or .sog (by extension).  Host code.
inline bool writeOctreeFile(const DenseVolume& vol, const std::string& filename) {
    const bool sog = filename.size() >= 4 && filename.compare(filename.size() - 4, 4, ".sog") == 0;
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

namespace detail {
template <int N, class T, class V>
std::vector<T> flatten(const std::vector<V>& v) {
    std::vector<T> out(v.size() * N);
    for (size_t i = 0; i < v.size(); ++i)
        for (int k = 0; k < N; ++k) out[N * i + k] = (T)v[i][k];
    return out;
}
}  // namespace detail

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
