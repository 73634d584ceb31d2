// extern "C" entry points of libvoxelcore_gb300.so (declared in
// include/voxelcore_gb300.h).  Argument checks, device selection, buffer
// staging and the plain single-volume pipeline live here; the kernels live
// in the per-stage files.
#include "vc_internal.cuh"

namespace vc {
int run_sites(vc_ctx* c, int64_t* n_sites);
int run_ft(vc_ctx* c);
int run_lattice_vd(vc_ctx* c, vc_vd_sizes* sizes, double t_thr);
int ensure_vd_aux(vc_ctx* c, bool meas, bool topo);
int run_lambda_check(vc_ctx* c, double* max_rel_err, int64_t* flips);
int run_vertex_radii(vc_ctx* c);
int run_finalize(vc_ctx* c, int64_t* ne_final);
int build_adjacency(vc_ctx* c);
int run_thin(vc_ctx* c, float f_t, float l_t, vc_thin_stats* stats);
int run_thin_folded(vc_ctx* c, vc_thin_stats* stats);
int get_thin_flags(vc_ctx* c, uint8_t* kv, uint8_t* ke, uint8_t* kf, uint8_t* re, int mem);
int run_remaining(vc_ctx* c, vc_rem_sizes* sizes);
int run_euler_remaining(vc_ctx* c, vc_euler_info* out);
int run_closed_components(vc_ctx* c, int64_t* n);
}  // namespace vc

using namespace vc;

namespace {
int enter(vc_ctx* c) {
    if (!c) return VC_ERR_ARG;
    cudaError_t e = cudaSetDevice(c->device);
    if (e != cudaSuccess) return cuda_fail(c, e, "cudaSetDevice");
    return VC_OK;
}
bool good_mem(int mem) { return mem == VC_MEM_HOST || mem == VC_MEM_DEVICE; }
}  // namespace

extern "C" {

int vc_set_volume(vc_ctx* c, const uint8_t* occ, int X, int Y, int Z, int mem) {
    VC_TRY(enter(c));
    if (X <= 0 || Y <= 0 || Z <= 0 || !occ || !good_mem(mem)) return VC_ERR_ARG;
    if ((int64_t)(X + 1) * (Y + 1) * (Z + 1) >= ((int64_t)1 << 33) || X > 32766 || Y > 32766 || Z > 32766)
        return VC_ERR_ARG;
    const int64_t n = (int64_t)X * Y * Z;
    // results of the previous volume are stale from here on, even if an
    // allocation below fails
    c->n_sites = -1;
    c->ft_valid = c->vd_valid = false;
    VC_TRY(ensure_n<uint8_t>(c, c->occ, n));
    VC_TRY(copy_in(c, c->occ.p, occ, (size_t)n, mem));
    const int32_t dims[3] = {X, Y, Z};
    VC_TRY(set_volume_table(c, 1, dims));
    c->X = X;
    c->Y = Y;
    c->Z = Z;
    c->n_sites = -1;
    c->ft_valid = c->vd_valid = false;
    c->sites_from_octree = false;
    c->oct_n_sites = 0;
    set_identity(c->vox_to_model);
    return VC_OK;
}

int vc_get_volume(vc_ctx* c, uint8_t* occ, int mem) {
    VC_TRY(enter(c));
    if (!occ || !good_mem(mem)) return VC_ERR_ARG;
    if (!c->occ.p || c->nvol <= 0) return VC_ERR_STATE;
    VC_TRY(copy_out(c, occ, c->occ.p, (size_t)c->h_off[kVox][c->nvol], mem));
    return sync_check(c);
}

int vc_extract_sites(vc_ctx* c, int64_t* n_sites) {
    VC_TRY(enter(c));
    if (c->n_sites >= 0) {  // the installed volume's sites are already on the device
        if (n_sites) *n_sites = c->n_sites;
        return VC_OK;
    }
    VC_TRY(run_sites(c, n_sites));
    return sync_check(c);
}

int vc_get_sites(vc_ctx* c, float* xyz, int mem) {
    VC_TRY(enter(c));
    if (c->n_sites < 0) return VC_ERR_STATE;
    if (!good_mem(mem)) return VC_ERR_ARG;
    VC_TRY(copy_out(c, xyz, c->site_xyz.p, (size_t)c->n_sites * 3 * sizeof(float), mem));
    return sync_check(c);
}

int vc_feature_transform(vc_ctx* c) {
    VC_TRY(enter(c));
    VC_TRY(run_ft(c));
    return sync_check(c);
}

int vc_get_ft(vc_ctx* c, int32_t* d2, int32_t* id, int mem) {
    VC_TRY(enter(c));
    if (!c->ft_valid) return VC_ERR_STATE;
    if (!good_mem(mem)) return VC_ERR_ARG;
    const size_t n = (size_t)c->h_off[kLat][c->nvol];  // all lattice points of the batch
    VC_TRY(copy_out(c, d2, c->ft_d2.p, n * sizeof(int32_t), mem));
    VC_TRY(copy_out(c, id, c->ft_id.p, n * sizeof(int32_t), mem));
    return sync_check(c);
}

int vc_lattice_vd(vc_ctx* c, vc_vd_sizes* sizes) {
    VC_TRY(enter(c));
    VC_TRY(run_lattice_vd(c, sizes, -1.0));
    return sync_check(c);
}

int vc_get_vd(vc_ctx* c, float* vts, int32_t* edges, int32_t* tris, int32_t* tri_face, float* vm, float* em,
              float* fm, int32_t* face_sites, int mem) {
    VC_TRY(enter(c));
    if (!c->vd_valid) return VC_ERR_STATE;
    if (!good_mem(mem)) return VC_ERR_ARG;
    VC_TRY(ensure_vd_aux(c, true, false));
    if (vts || edges || tris) VC_TRY(ensure_vd_geometry(c));
    const vc_vd_sizes& s = c->vd;
    VC_TRY(copy_out(c, vts, c->vts.p, (size_t)s.nv * 3 * sizeof(float), mem));
    VC_TRY(copy_out(c, edges, c->edges.p, (size_t)s.ne * 2 * sizeof(int32_t), mem));
    VC_TRY(copy_out(c, tris, c->tris.p, (size_t)s.nt * 3 * sizeof(int32_t), mem));
    VC_TRY(copy_out(c, tri_face, c->vd_tri_face.p, (size_t)s.nt * sizeof(int32_t), mem));
    VC_TRY(copy_out(c, vm, c->vm.p, (size_t)s.nv * sizeof(float), mem));
    VC_TRY(copy_out(c, em, c->em.p, (size_t)s.ne * sizeof(float), mem));
    VC_TRY(copy_out(c, fm, c->fm.p, (size_t)s.nt * sizeof(float), mem));
    VC_TRY(copy_out(c, face_sites, c->vd_face_sites.p, (size_t)s.nface * 2 * sizeof(int32_t), mem));
    return sync_check(c);
}

int vc_lambda_fp64_check(vc_ctx* c, double* max_rel_err, int64_t* flips) {
    VC_TRY(enter(c));
    if (!max_rel_err || !flips) return VC_ERR_ARG;
    return run_lambda_check(c, max_rel_err, flips);
}

int vc_vertex_radii(vc_ctx* c, float* radius, int mem) {
    VC_TRY(enter(c));
    if (!good_mem(mem)) return VC_ERR_ARG;
    VC_TRY(run_vertex_radii(c));
    VC_TRY(copy_out(c, radius, c->vd_radius.p, (size_t)c->vd.nv * sizeof(float), mem));
    return sync_check(c);
}

int vc_set_complex(vc_ctx* c, int64_t nv, const float* vts, int64_t ne, const int32_t* edges, int64_t nt,
                   const int32_t* tris, int mem) {
    VC_TRY(enter(c));
    if (nv < 0 || ne < 0 || nt < 0 || !good_mem(mem)) return VC_ERR_ARG;
    if (nv >= INT32_MAX || ne + 3 * nt >= INT32_MAX) return VC_ERR_ARG;
    if ((nv && !vts) || (ne && !edges) || (nt && !tris)) return VC_ERR_ARG;
    VC_TRY(ensure_n<float>(c, c->vts, 3 * nv));
    VC_TRY(ensure_n<int2>(c, c->edges_in, ne));
    VC_TRY(ensure_n<int32_t>(c, c->tris, 3 * nt));
    VC_TRY(copy_in(c, c->vts.p, vts, (size_t)nv * 3 * sizeof(float), mem));
    VC_TRY(copy_in(c, c->edges_in.p, edges, (size_t)ne * 2 * sizeof(int32_t), mem));
    VC_TRY(copy_in(c, c->tris.p, tris, (size_t)nt * 3 * sizeof(int32_t), mem));
    c->nv = nv;
    c->ne_in = ne;
    c->ne = 0;
    c->nt = nt;
    c->cc_valid = true;
    c->cc_finalized = c->meas_valid = c->thin_valid = c->rem_valid = false;
    c->records_fresh = false;
    c->cc_batched = false;
    c->vd_valid = false;  // the complex no longer comes from the lattice VD
    return VC_OK;
}

int vc_finalize(vc_ctx* c, int64_t* ne_final) {
    VC_TRY(enter(c));
    VC_TRY(run_finalize(c, ne_final));
    return sync_check(c);
}

int vc_get_finalized(vc_ctx* c, int32_t* edges, int32_t* tri_edges, int32_t* ve_off, int32_t* ve_ids,
                     int32_t* ef_off, int32_t* ef_ids, int mem) {
    VC_TRY(enter(c));
    if (!c->cc_finalized) return VC_ERR_STATE;
    if (!good_mem(mem)) return VC_ERR_ARG;
    VC_TRY(ensure_vd_aux(c, false, true));  // (writes the lattice complex's edges too)
    VC_TRY(copy_out(c, edges, c->edges.p, (size_t)c->ne * 2 * sizeof(int32_t), mem));
    VC_TRY(copy_out(c, tri_edges, c->tri_edges.p, (size_t)c->nt * 3 * sizeof(int32_t), mem));
    VC_TRY(copy_out(c, ve_off, c->ve_off.p, (size_t)(c->nv + 1) * sizeof(int32_t), mem));
    VC_TRY(copy_out(c, ve_ids, c->ve_ids.p, (size_t)c->ne * 2 * sizeof(int32_t), mem));
    VC_TRY(copy_out(c, ef_off, c->ef_off.p, (size_t)(c->ne + 1) * sizeof(int32_t), mem));
    VC_TRY(copy_out(c, ef_ids, c->ef_ids.p, (size_t)c->nt * 3 * sizeof(int32_t), mem));
    return sync_check(c);
}

int vc_set_measures(vc_ctx* c, const float* vm, const float* em, const float* fm, int mem) {
    VC_TRY(enter(c));
    if (!c->cc_finalized) return VC_ERR_STATE;
    if (!good_mem(mem) || (c->ne && !em) || (c->nt && !fm)) return VC_ERR_ARG;
    VC_TRY(ensure_n<float>(c, c->vm, c->nv));
    VC_TRY(ensure_n<float>(c, c->em, c->ne));
    VC_TRY(ensure_n<float>(c, c->fm, c->nt));
    // a lattice complex's own measures are written first, so that a missing
    // vm keeps the lattice's values
    if (!vm) VC_TRY(ensure_vd_aux(c, true, false));
    if (vm) VC_TRY(copy_in(c, c->vm.p, vm, (size_t)c->nv * sizeof(float), mem));
    VC_TRY(copy_in(c, c->em.p, em, (size_t)c->ne * sizeof(float), mem));
    VC_TRY(copy_in(c, c->fm.p, fm, (size_t)c->nt * sizeof(float), mem));
    c->vd_aux_meas = true;  // the caller's measures: never overwritten by the lattice's
    c->meas_valid = true;
    c->records_fresh = false;
    c->thin_valid = c->rem_valid = false;
    return VC_OK;
}

int vc_thin(vc_ctx* c, float f_t, float l_t, vc_thin_stats* stats) {
    VC_TRY(enter(c));
    VC_TRY(run_thin(c, f_t, l_t, stats));
    return VC_OK;
}

int vc_get_thin_flags(vc_ctx* c, uint8_t* keep_v, uint8_t* keep_e, uint8_t* keep_f, uint8_t* removed_e, int mem) {
    VC_TRY(enter(c));
    if (!good_mem(mem)) return VC_ERR_ARG;
    return get_thin_flags(c, keep_v, keep_e, keep_f, removed_e, mem);
}

int vc_remaining(vc_ctx* c, vc_rem_sizes* sizes) {
    VC_TRY(enter(c));
    VC_TRY(run_remaining(c, sizes));
    return sync_check(c);
}

int vc_get_remaining(vc_ctx* c, float* vts, int32_t* edges, int32_t* tris, int mem) {
    VC_TRY(enter(c));
    if (!c->rem_valid) return VC_ERR_STATE;
    if (!good_mem(mem)) return VC_ERR_ARG;
    VC_TRY(copy_out(c, vts, c->rem_vts.p, (size_t)c->rem.nv * 3 * sizeof(float), mem));
    VC_TRY(copy_out(c, edges, c->rem_edges.p, (size_t)c->rem.ne * 2 * sizeof(int32_t), mem));
    VC_TRY(copy_out(c, tris, c->rem_tris.p, (size_t)c->rem.nt * 3 * sizeof(int32_t), mem));
    return sync_check(c);
}

int vc_euler_remaining(vc_ctx* c, vc_euler_info* out) {
    VC_TRY(enter(c));
    if (!out) return VC_ERR_ARG;
    return run_euler_remaining(c, out);
}

int vc_closed_components(vc_ctx* c, int64_t* n) {
    VC_TRY(enter(c));
    if (!n) return VC_ERR_ARG;
    return run_closed_components(c, n);
}

int vc_run_plain(vc_ctx* c, const uint8_t* occ, int X, int Y, int Z, int mem, double t, vc_plain_result* out) {
    VC_TRY(enter(c));
    if (!out) return VC_ERR_ARG;
    VC_TRY(vc_set_volume(c, occ, X, Y, Z, mem));
    VC_TRY(run_sites(c, &out->n_sites));
    VC_TRY(run_ft(c));
    // the threshold (highlevelalgo.cpp:836: float thresh = getInsidePartSize()
    // * t, float * double -> float) is computed on the device and folded into
    // the thinning records as they are written
    VC_TRY(run_lattice_vd(c, &out->vd, t));
    out->thresh = (float)((double)out->vd.inside_size * t);
    VC_TRY(run_thin_folded(c, &out->thin));
    VC_TRY(run_remaining(c, &out->rem));
    return sync_check(c);
}

int vc_batch_set_volumes(vc_ctx* c, int nvol, const int32_t* dims, const uint8_t* occ, int mem) {
    VC_TRY(enter(c));
    if (nvol <= 0 || !dims || !occ || !good_mem(mem)) return VC_ERR_ARG;
    int64_t nvox = 0;
    for (int b = 0; b < nvol; ++b) {
        const int X = dims[3 * b], Y = dims[3 * b + 1], Z = dims[3 * b + 2];
        if (X <= 0 || Y <= 0 || Z <= 0 || X > 32766 || Y > 32766 || Z > 32766) return VC_ERR_ARG;
        if (space_size(kLat, X, Y, Z) >= ((int64_t)1 << 32)) return VC_ERR_ARG;
        nvox += (int64_t)X * Y * Z;
    }
    c->n_sites = -1;
    c->ft_valid = c->vd_valid = false;
    VC_TRY(ensure_n<uint8_t>(c, c->occ, nvox));
    VC_TRY(copy_in(c, c->occ.p, occ, (size_t)nvox, mem));
    VC_TRY(set_volume_table(c, nvol, dims));
    c->X = dims[0];
    c->Y = dims[1];
    c->Z = dims[2];
    c->n_sites = -1;
    c->ft_valid = c->vd_valid = false;
    c->sites_from_octree = false;
    c->oct_n_sites = 0;
    set_identity(c->vox_to_model);
    return VC_OK;
}

int vc_batch_run(vc_ctx* c, double t, int with_euler, vc_thin_stats* stats, vc_batch_volume* out) {
    VC_TRY(enter(c));
    if (!out || c->nvol <= 0) return c->nvol <= 0 ? VC_ERR_STATE : VC_ERR_ARG;
    const int nvol = c->nvol;
    int64_t n_sites = 0;
    vc_vd_sizes vd{};
    vc_thin_stats th{};
    vc_rem_sizes rem{};
    VC_TRY(run_sites(c, &n_sites));
    VC_TRY(run_ft(c));
    VC_TRY(run_lattice_vd(c, &vd, t));
    VC_TRY(run_thin_folded(c, &th));
    VC_TRY(run_remaining(c, &rem));
    vc_euler_info eu{};
    if (with_euler) VC_TRY(run_euler_remaining(c, &eu));
    // per-volume bookkeeping: the base tables
    const size_t n1 = (size_t)nvol + 1;
    std::vector<int64_t> hb((size_t)kNumBases * n1);
    std::vector<float> hthr((size_t)nvol);
    VC_CUDA(c, cudaMemcpyAsync(hb.data(), c->bases.b[0], hb.size() * sizeof(int64_t), cudaMemcpyDeviceToHost,
                               c->stream));
    VC_CUDA(c, cudaMemcpyAsync(hthr.data(), c->bases.thr, hthr.size() * sizeof(float), cudaMemcpyDeviceToHost,
                               c->stream));
    VC_TRY(sync_check(c));
    auto B = [&](int k, int b) { return hb[(size_t)k * n1 + b]; };
    for (int b = 0; b < nvol; ++b) {
        vc_batch_volume& o = out[b];
        o = vc_batch_volume{};
        o.n_sites = B(kBSite, b + 1) - B(kBSite, b);
        const int64_t nf = B(kBFace, b + 1) - B(kBFace, b);
        o.vd.nv = B(kBVert, b + 1) - B(kBVert, b);
        o.vd.ne = B(kBAxis, b + 1) - B(kBAxis, b) + nf;
        o.vd.nt = 2 * nf;
        o.vd.nface = nf;
        o.vd.inside_size = c->vol_inside[b];
        o.thresh = hthr[b];
        o.site_off = B(kBSite, b);
        o.v_off = B(kBVert, b);
        o.e_off = B(kBAxis, b) + B(kBFace, b);
        o.t_off = 2 * B(kBFace, b);
        if (nvol > 1) {
            const auto& r = c->h_rem_bases;
            o.rem = vc_rem_sizes{r[b + 1] - r[b], r[n1 + b + 1] - r[n1 + b], r[2 * n1 + b + 1] - r[2 * n1 + b]};
            o.rem_v_off = r[b];
            o.rem_e_off = r[n1 + b];
            o.rem_t_off = r[2 * n1 + b];
        } else {
            o.rem = rem;
        }
        if (with_euler) o.euler = c->vol_euler[b];
    }
    if (stats) *stats = th;
    return VC_OK;
}

}  // extern "C"
