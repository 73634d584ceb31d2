"""Python host layer over the C ABI, mirroring the reference's C++ surfaces.

``Context`` wraps one ``vc_ctx`` (one CUDA stream on one device).  Arrays may
be numpy arrays (host) or torch CUDA tensors (device); outputs come back as
numpy arrays unless ``device=True`` is asked for, in which case they are
torch tensors on the context's device.

The classes ``Surfacer``, ``cellcomplex``, ``CellComplexThinning`` and the
function ``extract_inside_with_measure`` keep the reference's names, argument
meaning and call order (include/surfacing.h:57-58, include/cellcomplex.h:33,
include/ccthin.h:57-113, include/voroinfo.h:127-131) so that code written
against the reference reads the same.
"""
from __future__ import annotations

import ctypes
import os
from typing import Optional

import numpy as np

from . import _lib as L


def _is_torch(x) -> bool:
    return type(x).__module__.startswith("torch")


def _ptr_mem(x):
    """(pointer, mem flag) of a numpy array or a torch tensor."""
    if x is None:
        return None, L.VC_MEM_HOST
    if _is_torch(x):
        if not x.is_contiguous():
            raise ValueError("tensor must be contiguous")
        return ctypes.c_void_p(x.data_ptr()), (L.VC_MEM_DEVICE if x.is_cuda else L.VC_MEM_HOST)
    if not x.flags["C_CONTIGUOUS"]:
        raise ValueError("array must be C-contiguous")
    return x.ctypes.data_as(ctypes.c_void_p), L.VC_MEM_HOST


class Context:
    """One GPU context of the hot path (vc_ctx)."""

    def __init__(self, device: int = 0):
        self.lib = L.load()
        self.device = device
        h = ctypes.c_void_p()
        st = self.lib.vc_ctx_create(ctypes.byref(h), device)
        if st != L.VC_OK:
            raise L.VoxelCoreError(st, "vc_ctx_create")
        self.h = h
        self.shape = None

    # -- plumbing ---------------------------------------------------------
    def close(self):
        if getattr(self, "h", None):
            self.lib.vc_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def check(self, st: int, where: str):
        if st != L.VC_OK:
            detail = self.lib.vc_ctx_last_error(self.h)
            raise L.VoxelCoreError(st, where, detail.decode() if detail else "")

    @property
    def stream_ptr(self) -> int:
        return int(self.lib.vc_ctx_stream(self.h) or 0)

    def torch_stream(self):
        import torch
        return torch.cuda.ExternalStream(self.stream_ptr, device=torch.device("cuda", self.device))

    def sync(self):
        self.check(self.lib.vc_ctx_sync(self.h), "vc_ctx_sync")

    def device_bytes(self) -> int:
        return int(self.lib.vc_ctx_device_bytes(self.h))

    def launch_count(self) -> int:
        return int(self.lib.vc_ctx_launch_count(self.h))

    def set_timing(self, on: bool):
        self.check(self.lib.vc_ctx_set_timing(self.h, 1 if on else 0), "vc_ctx_set_timing")

    def reset_timings(self):
        self.check(self.lib.vc_ctx_reset_timings(self.h), "vc_ctx_reset_timings")

    def timings(self) -> dict:
        """{region: (total ms, count)} of the CUDA-event-timed library regions."""
        cap, nl = 64, 48
        names = ctypes.create_string_buffer(cap * nl)
        ms = (ctypes.c_double * cap)()
        cnt = (ctypes.c_int64 * cap)()
        n = ctypes.c_int()
        self.check(self.lib.vc_ctx_get_timings(self.h, names, nl, ms, cnt, cap, ctypes.byref(n)), "vc_ctx_get_timings")
        out = {}
        for i in range(min(n.value, cap)):
            nm = names.raw[i * nl:(i + 1) * nl].split(b"\0", 1)[0].decode()
            out[nm] = (float(ms[i]), int(cnt[i]))
        return out

    def debug_thin_trace(self, cap: int = 4096, blocks_per_sm: int = 0):
        self.check(self.lib.vc_debug_thin_trace(self.h, cap, blocks_per_sm), "vc_debug_thin_trace")

    def lambda_fp64_check(self) -> dict:
        """Face measures of the current lattice complex against an FP64
        recomputation: the largest relative error and the threshold flips."""
        e = ctypes.c_double()
        n = ctypes.c_int64()
        self.check(self.lib.vc_lambda_fp64_check(self.h, ctypes.byref(e), ctypes.byref(n)), "vc_lambda_fp64_check")
        return dict(max_rel_err=e.value, flips=n.value)

    def autotune(self, t: float = 0.04) -> dict:
        """Time the input-dependent launch shapes on the installed volume or
        batch and keep the fastest (vc_autotune); returns the choice and the
        measured milliseconds per candidate."""
        r = L.TuneResult()
        self.check(self.lib.vc_autotune(self.h, ctypes.c_double(t), ctypes.byref(r)), "vc_autotune")
        return dict(ft_ring=r.ft_ring, thin_threads=r.thin_threads, thin_blocks_per_sm=r.thin_blocks_per_sm,
                    thin_items=r.thin_items, ft_method="window" if r.ft_method == 1 else "envelope",
                    ft_ms={k: round(float(v), 4) for k, v in zip((4, 8, 16), r.ft_ms)},
                    ft_window_ms=round(float(r.ft_window_ms), 4),
                    thin_ms={k: round(float(v), 4)
                             for k, v in zip(("512x2", "512x2x2", "512x4", "256x8", "1024x1"), r.thin_ms)})

    def debug_thin_shape(self, threads: int = 0, blocks_per_sm: int = 0, items: int = 0):
        """Launch shape of the thinning kernel (identical results)."""
        self.check(self.lib.vc_debug_thin_shape(self.h, threads, blocks_per_sm, items), "vc_debug_thin_shape")

    def closed_components(self) -> int:
        """nClosedComponents of the installed finalized complex
        (vc_closed_components): the closed pockets left by an all-pass thinning."""
        n = ctypes.c_int64()
        self.check(self.lib.vc_closed_components(self.h, ctypes.byref(n)), "vc_closed_components")
        return n.value

    def set_ft_method(self, method: str = "auto"):
        """Method of the feature transform's y and x passes: "envelope",
        "window" or "auto" (vc_set_ft_method; identical results)."""
        m = {"envelope": 0, "window": 1, "auto": 2}[method]
        self.check(self.lib.vc_set_ft_method(self.h, m), "vc_set_ft_method")

    def debug_random_rate(self, op: int, nbytes: int) -> float:
        """Random 32-byte record touches per second in an nbytes array
        (vc_debug_random_rate; op 0 load, 1 two 16-byte loads, 2 atomicAdd,
        3 atomicMax + atomicAdd)."""
        out = ctypes.c_double()
        self.check(self.lib.vc_debug_random_rate(self.h, op, nbytes, ctypes.byref(out)), "vc_debug_random_rate")
        return out.value

    def debug_set_spin_limit(self, polls: int = 0):
        """Polls before a grid barrier of the thinning gives up (0 = default)."""
        self.check(self.lib.vc_debug_set_spin_limit(self.h, polls), "vc_debug_set_spin_limit")

    def debug_fail_alloc_after(self, k: int = -1):
        """The next k device allocations succeed, the one after fails (k < 0: off)."""
        self.check(self.lib.vc_debug_fail_alloc_after(self.h, k), "vc_debug_fail_alloc_after")

    def debug_ref_bias(self, vertex: int = -1, delta: int = 0):
        """Raise (+1) or lower (-1) one vertex's thinning count after its record is built (0: off)."""
        self.check(self.lib.vc_debug_ref_bias(self.h, vertex, delta), "vc_debug_ref_bias")

    def debug_thin_queue(self, capacity: int = 0, first_position: int = 0):
        """Cap the thinning queue at `capacity` items per generation (0 = default) and start its positions at
        `first_position`; results are the same while the largest generation fits, else vc_thin fails (OOM)."""
        self.check(self.lib.vc_debug_thin_queue(self.h, capacity, first_position), "vc_debug_thin_queue")

    def debug_ft_wide(self, wide: bool = True):
        """Force 64-bit arithmetic in the feature transform (identical results)."""
        self.check(self.lib.vc_debug_ft_wide(self.h, 1 if wide else 0), "vc_debug_ft_wide")

    def thin_trace(self):
        n = ctypes.c_int()
        self.check(self.lib.vc_debug_get_thin_trace(self.h, None, 0, ctypes.byref(n)), "vc_debug_get_thin_trace")
        out = np.zeros((max(n.value, 1), 4), np.int64)
        self.check(self.lib.vc_debug_get_thin_trace(self.h, out.ctypes.data_as(ctypes.c_void_p), n.value,
                                                     ctypes.byref(n)), "vc_debug_get_thin_trace")
        return out[: n.value]

    def _out(self, shape, dtype, device: bool):
        if device:
            import torch
            tdt = {np.float32: torch.float32, np.int32: torch.int32, np.uint8: torch.uint8}[dtype]
            return torch.empty(shape, dtype=tdt, device=torch.device("cuda", self.device))
        return np.empty(shape, dtype=dtype)

    # -- volume / sites / FT ----------------------------------------------
    def set_volume(self, occ):
        X, Y, Z = (int(s) for s in occ.shape)
        p, mem = _ptr_mem(occ)
        self.check(self.lib.vc_set_volume(self.h, p, X, Y, Z, mem), "vc_set_volume")
        self.shape = (X, Y, Z)

    def set_volume_sof(self, data: bytes) -> int:
        """Install an octree volume from the bytes of a .sof file
        (vc_set_volume_sof); returns its voxels per axis (R + 1)."""
        buf = np.frombuffer(data, dtype=np.uint8)
        size = ctypes.c_int()
        self.check(self.lib.vc_set_volume_sof(self.h, buf.ctypes.data_as(ctypes.c_void_p), len(buf),
                                              ctypes.byref(size)), "vc_set_volume_sof")
        n = int(size.value)
        self.shape = (n, n, n)
        return n

    def set_volume_sog(self, data: bytes) -> int:
        """Install an octree volume from the bytes of a .sog file
        (vc_set_volume_sog); returns its voxels per axis (R + 1)."""
        buf = np.frombuffer(data, dtype=np.uint8)
        size = ctypes.c_int()
        self.check(self.lib.vc_set_volume_sog(self.h, buf.ctypes.data_as(ctypes.c_void_p), len(buf),
                                              ctypes.byref(size)), "vc_set_volume_sog")
        n = int(size.value)
        self.shape = (n, n, n)
        return n

    def set_volume_mrc(self, data: bytes):
        """Install the map of an .mrc file (vc_set_volume_mrc); returns (X, Y, Z)."""
        buf = np.frombuffer(data, dtype=np.uint8)
        dims = np.zeros(3, np.int32)
        self.check(self.lib.vc_set_volume_mrc(self.h, buf.ctypes.data_as(ctypes.c_void_p), len(buf),
                                              dims.ctypes.data_as(ctypes.c_void_p)), "vc_set_volume_mrc")
        self.shape = tuple(int(x) for x in dims)
        return self.shape

    def vox_to_model(self) -> np.ndarray:
        """The installed volume's voxel-to-model matrix, 4x4 (vc_get_vox_to_model)."""
        m = np.zeros(16, np.float64)
        self.check(self.lib.vc_get_vox_to_model(self.h, m.ctypes.data_as(ctypes.c_void_p)), "vc_get_vox_to_model")
        return m.reshape(4, 4).T  # column-major storage

    def volume(self, device: bool = False):
        """The installed occupancy (vc_get_volume)."""
        out = self._out(self.shape, np.uint8, device)
        p, mem = _ptr_mem(out)
        self.check(self.lib.vc_get_volume(self.h, p, mem), "vc_get_volume")
        return out

    def extract_sites(self) -> int:
        n = ctypes.c_int64()
        self.check(self.lib.vc_extract_sites(self.h, ctypes.byref(n)), "vc_extract_sites")
        self.n_sites = int(n.value)
        return self.n_sites

    def sites(self, device: bool = False):
        out = self._out((self.n_sites, 3), np.float32, device)
        p, mem = _ptr_mem(out)
        self.check(self.lib.vc_get_sites(self.h, p, mem), "vc_get_sites")
        return out

    def feature_transform(self):
        self.check(self.lib.vc_feature_transform(self.h), "vc_feature_transform")

    def ft(self, device: bool = False):
        X, Y, Z = self.shape
        shp = (X + 1, Y + 1, Z + 1)
        d2, ids = self._out(shp, np.int32, device), self._out(shp, np.int32, device)
        (p1, mem), (p2, _) = _ptr_mem(d2), _ptr_mem(ids)
        self.check(self.lib.vc_get_ft(self.h, p1, p2, mem), "vc_get_ft")
        return d2, ids

    # -- lattice Voronoi complex ------------------------------------------
    def lattice_vd(self) -> dict:
        s = L.VdSizes()
        self.check(self.lib.vc_lattice_vd(self.h, ctypes.byref(s)), "vc_lattice_vd")
        self.vd_sizes = dict(nv=s.nv, ne=s.ne, nt=s.nt, nface=s.nface, inside_size=s.inside_size)
        self.use_vd_as_complex()  # vc_lattice_vd installs it as the context's cell complex
        return self.vd_sizes

    def vd(self, device: bool = False) -> dict:
        s = self.vd_sizes
        o = dict(vts=self._out((s["nv"], 3), np.float32, device), edges=self._out((s["ne"], 2), np.int32, device),
                 tris=self._out((s["nt"], 3), np.int32, device), tri_face=self._out((s["nt"],), np.int32, device),
                 vm=self._out((s["nv"],), np.float32, device), em=self._out((s["ne"],), np.float32, device),
                 fm=self._out((s["nt"],), np.float32, device),
                 face_sites=self._out((s["nface"], 2), np.int32, device))
        keys = ("vts", "edges", "tris", "tri_face", "vm", "em", "fm", "face_sites")
        ptrs = [_ptr_mem(o[k])[0] for k in keys]
        mem = L.VC_MEM_DEVICE if device else L.VC_MEM_HOST
        self.check(self.lib.vc_get_vd(self.h, *ptrs, mem), "vc_get_vd")
        o["inside_size"] = s["inside_size"]
        return o

    def vertex_radii(self, device: bool = False):
        """VoroInfo::getRadii for the lattice complex's vertices (voroinfo.cpp:286-325)."""
        r = self._out((self.vd_sizes["nv"],), np.float32, device)
        p, mem = _ptr_mem(r)
        self.check(self.lib.vc_vertex_radii(self.h, p, mem), "vc_vertex_radii")
        return r

    # -- cell complex -----------------------------------------------------
    def set_complex(self, vts, edges, tris):
        vts = vts.reshape(-1, 3) if vts is not None else None
        nv, ne, nt = int(vts.shape[0]), int(edges.reshape(-1, 2).shape[0]), int(tris.reshape(-1, 3).shape[0])
        (pv, mem), (pe, _), (pt, _) = _ptr_mem(vts), _ptr_mem(edges), _ptr_mem(tris)
        self.check(self.lib.vc_set_complex(self.h, nv, pv, ne, pe, nt, pt, mem), "vc_set_complex")
        self.nv, self.nt = nv, nt

    def finalize(self) -> int:
        n = ctypes.c_int64()
        self.check(self.lib.vc_finalize(self.h, ctypes.byref(n)), "vc_finalize")
        self.ne = int(n.value)
        return self.ne

    def finalized(self) -> dict:
        nv, ne, nt = self.nv, self.ne, self.nt
        o = dict(edges=np.empty((ne, 2), np.int32), tri_edges=np.empty((nt, 3), np.int32),
                 ve_off=np.empty(nv + 1, np.int32), ve_ids=np.empty(2 * ne, np.int32),
                 ef_off=np.empty(ne + 1, np.int32), ef_ids=np.empty(3 * nt, np.int32))
        ptrs = [_ptr_mem(o[k])[0] for k in ("edges", "tri_edges", "ve_off", "ve_ids", "ef_off", "ef_ids")]
        self.check(self.lib.vc_get_finalized(self.h, *ptrs, L.VC_MEM_HOST), "vc_get_finalized")
        return o

    def use_vd_as_complex(self):
        s = self.vd_sizes
        self.nv, self.ne, self.nt = s["nv"], s["ne"], s["nt"]

    def set_measures(self, vm, em, fm):
        (p1, mem), (p2, _), (p3, _) = _ptr_mem(vm), _ptr_mem(em), _ptr_mem(fm)
        self.check(self.lib.vc_set_measures(self.h, p1, p2, p3, mem), "vc_set_measures")

    def thin(self, f_t: float, l_t: float) -> dict:
        st = L.ThinStats()
        self.check(self.lib.vc_thin(self.h, ctypes.c_float(f_t), ctypes.c_float(l_t), ctypes.byref(st)), "vc_thin")
        return dict(pushes=st.pushes, processed=st.processed, skipped=st.skipped, generations=st.generations)

    def thin_flags(self, device: bool = False) -> dict:
        o = dict(keep_v=self._out((self.nv,), np.uint8, device), keep_e=self._out((self.ne,), np.uint8, device),
                 keep_f=self._out((self.nt,), np.uint8, device), removed_e=self._out((self.ne,), np.uint8, device))
        ptrs = [_ptr_mem(o[k])[0] for k in ("keep_v", "keep_e", "keep_f", "removed_e")]
        mem = L.VC_MEM_DEVICE if device else L.VC_MEM_HOST
        self.check(self.lib.vc_get_thin_flags(self.h, *ptrs, mem), "vc_get_thin_flags")
        return o

    def remaining(self) -> dict:
        s = L.RemSizes()
        self.check(self.lib.vc_remaining(self.h, ctypes.byref(s)), "vc_remaining")
        self.rem_sizes = dict(nv=s.nv, ne=s.ne, nt=s.nt)
        return self.rem_sizes

    def remaining_arrays(self, device: bool = False):
        s = self.rem_sizes
        v = self._out((s["nv"], 3), np.float32, device)
        e = self._out((s["ne"], 2), np.int32, device)
        t = self._out((s["nt"], 3), np.int32, device)
        mem = L.VC_MEM_DEVICE if device else L.VC_MEM_HOST
        self.check(self.lib.vc_get_remaining(self.h, _ptr_mem(v)[0], _ptr_mem(e)[0], _ptr_mem(t)[0], mem),
                   "vc_get_remaining")
        return v, e, t

    def remaining_arrays_into(self, vts, edges, tris):
        """Copy the remaining complex into caller buffers (numpy, pinned host or CUDA tensors)."""
        (pv, mem), (pe, _), (pt, _) = _ptr_mem(vts), _ptr_mem(edges), _ptr_mem(tris)
        self.check(self.lib.vc_get_remaining(self.h, pv, pe, pt, mem), "vc_get_remaining")

    def write_remaining(self, prefix: str, ply: bool = True, radii: bool = True, ma: bool = True) -> None:
        """Write <prefix>.ply / .r / .ma for the remaining complex (vc_write_remaining)."""
        what = (L.VC_WRITE_PLY if ply else 0) | (L.VC_WRITE_RADII if radii else 0) | (L.VC_WRITE_MA if ma else 0)
        self.check(self.lib.vc_write_remaining(self.h, os.fsencode(prefix), what), "vc_write_remaining")

    def euler_remaining(self) -> dict:
        s = L.EulerInfo()
        self.check(self.lib.vc_euler_remaining(self.h, ctypes.byref(s)), "vc_euler_remaining")
        return dict(V=s.V, E=s.E, F=s.F, C=s.C, euler=s.euler)

    def run_plain(self, occ, t: float = 0.04) -> dict:
        X, Y, Z = (int(s) for s in occ.shape)
        p, mem = _ptr_mem(occ)
        r = L.PlainResult()
        self.check(self.lib.vc_run_plain(self.h, p, X, Y, Z, mem, ctypes.c_double(t), ctypes.byref(r)),
                   "vc_run_plain")
        self.shape = (X, Y, Z)
        self.n_sites = r.n_sites
        self.vd_sizes = dict(nv=r.vd.nv, ne=r.vd.ne, nt=r.vd.nt, nface=r.vd.nface, inside_size=r.vd.inside_size)
        self.use_vd_as_complex()
        self.rem_sizes = dict(nv=r.rem.nv, ne=r.rem.ne, nt=r.rem.nt)
        return dict(n_sites=r.n_sites, vd=dict(self.vd_sizes), thresh=r.thresh,
                    thin=dict(pushes=r.thin.pushes, processed=r.thin.processed, skipped=r.thin.skipped,
                              generations=r.thin.generations),
                    rem=dict(self.rem_sizes))

    # -- batched path ------------------------------------------------------
    def batch_set_volumes(self, vols=None, *, occ=None, dims=None):
        """Install a batch: a list of volumes, or their voxels concatenated
        (1-D, host array or CUDA tensor) with dims (nvol x 3)."""
        if vols is not None:
            dims = np.array([tuple(int(x) for x in v.shape) for v in vols], np.int32)
            if _is_torch(vols[0]):
                import torch
                occ = torch.cat([v.contiguous().reshape(-1) for v in vols])
            else:
                occ = np.concatenate([np.ascontiguousarray(v, dtype=np.uint8).reshape(-1) for v in vols])
        dims = np.ascontiguousarray(np.asarray(dims, np.int32).reshape(-1, 3))
        p, mem = _ptr_mem(occ)
        self.check(self.lib.vc_batch_set_volumes(self.h, len(dims), dims.ctypes.data_as(ctypes.c_void_p), p, mem),
                   "vc_batch_set_volumes")
        self.batch_dims = dims
        self.shape = tuple(int(x) for x in dims[0])

    def batch_run(self, t: float = 0.04, euler: bool = True) -> list:
        """vc_batch_run: per-volume results (sizes, threshold, Euler and the
        volume's offsets into the batch-wide outputs)."""
        n = len(self.batch_dims)
        out = (L.BatchVolume * n)()
        st = L.ThinStats()
        self.check(self.lib.vc_batch_run(self.h, ctypes.c_double(t), int(euler), ctypes.byref(st), out),
                   "vc_batch_run")
        res = []
        for o in out:
            res.append(dict(
                n_sites=o.n_sites, thresh=o.thresh,
                vd=dict(nv=o.vd.nv, ne=o.vd.ne, nt=o.vd.nt, nface=o.vd.nface, inside_size=o.vd.inside_size),
                rem=dict(nv=o.rem.nv, ne=o.rem.ne, nt=o.rem.nt),
                euler=dict(V=o.euler.V, E=o.euler.E, F=o.euler.F, C=o.euler.C, euler=o.euler.euler),
                site_off=o.site_off, v_off=o.v_off, e_off=o.e_off, t_off=o.t_off,
                rem_v_off=o.rem_v_off, rem_e_off=o.rem_e_off, rem_t_off=o.rem_t_off))
        self.batch_stats = dict(pushes=st.pushes, processed=st.processed, skipped=st.skipped,
                                generations=st.generations)
        self.n_sites = sum(r["n_sites"] for r in res)
        self.vd_sizes = dict(nv=sum(r["vd"]["nv"] for r in res), ne=sum(r["vd"]["ne"] for r in res),
                             nt=sum(r["vd"]["nt"] for r in res), nface=sum(r["vd"]["nface"] for r in res),
                             inside_size=res[0]["vd"]["inside_size"])
        self.use_vd_as_complex()
        self.rem_sizes = dict(nv=sum(r["rem"]["nv"] for r in res), ne=sum(r["rem"]["ne"] for r in res),
                              nt=sum(r["rem"]["nt"] for r in res))
        return res

    def batch_split(self, res: list, device: bool = False) -> list:
        """Per-volume (sites, keep flags, remaining arrays) of the last batch_run."""
        sites = self.sites()
        fl = self.thin_flags()
        rv, re_, rt = self.remaining_arrays(device)
        out = []
        for r in res:
            v0, e0, t0 = r["v_off"], r["e_off"], r["t_off"]
            a, b, c = r["rem_v_off"], r["rem_e_off"], r["rem_t_off"]
            out.append(dict(
                sites=sites[r["site_off"]:r["site_off"] + r["n_sites"]],
                keep_v=fl["keep_v"][v0:v0 + r["vd"]["nv"]], keep_e=fl["keep_e"][e0:e0 + r["vd"]["ne"]],
                keep_f=fl["keep_f"][t0:t0 + r["vd"]["nt"]], removed_e=fl["removed_e"][e0:e0 + r["vd"]["ne"]],
                rem_vts=rv[a:a + r["rem"]["nv"]], rem_edges=re_[b:b + r["rem"]["ne"]],
                rem_tris=rt[c:c + r["rem"]["nt"]]))
        return out


class Server:
    """The request loop (vc_server_*): submit host volumes, wait for results."""

    def __init__(self, device=0, workers: int = 2, mem_cap_bytes: int = 120 << 30, max_batch: int = 64,
                 bytes_per_voxel: Optional[float] = None):
        """device: one GPU, or a list of GPUs (workers and mem_cap_bytes are then per GPU)."""
        self.lib = L.load()
        h = ctypes.c_void_p()
        devs = np.array(device if isinstance(device, (list, tuple)) else [device], np.int32)
        st = self.lib.vc_server_create_devices(ctypes.byref(h), devs.ctypes.data_as(ctypes.c_void_p), len(devs),
                                               workers, mem_cap_bytes, max_batch)
        if st != L.VC_OK:
            raise L.VoxelCoreError(st, "vc_server_create_devices", "")
        self.h = h
        if bytes_per_voxel is not None:
            self._check(self.lib.vc_server_set_bytes_per_voxel(self.h, float(bytes_per_voxel)),
                        "vc_server_set_bytes_per_voxel")

    def _check(self, st, where):
        if st != L.VC_OK:
            raise L.VoxelCoreError(st, where, "")

    def submit(self, occ, t: float = 0.04) -> int:
        occ = np.ascontiguousarray(occ, dtype=np.uint8)
        X, Y, Z = (int(x) for x in occ.shape)
        rid = ctypes.c_int64()
        self._check(self.lib.vc_server_submit(self.h, occ.ctypes.data_as(ctypes.c_void_p), X, Y, Z,
                                              ctypes.c_double(t), ctypes.byref(rid)), "vc_server_submit")
        return int(rid.value)

    def wait(self, rid: int, timeout_s: float = -1.0) -> dict:
        r = L.RequestResult()
        self._check(self.lib.vc_server_wait(self.h, rid, ctypes.c_double(timeout_s), ctypes.byref(r)),
                    "vc_server_wait")
        return dict(status=r.status, batch_size=r.batch_size, n_sites=r.n_sites, thresh=r.thresh,
                    vd=dict(nv=r.vd.nv, ne=r.vd.ne, nt=r.vd.nt, nface=r.vd.nface, inside_size=r.vd.inside_size),
                    rem=dict(nv=r.rem.nv, ne=r.rem.ne, nt=r.rem.nt),
                    euler=dict(V=r.euler.V, E=r.euler.E, F=r.euler.F, C=r.euler.C, euler=r.euler.euler),
                    queue_ms=r.queue_ms, run_ms=r.run_ms, latency_ms=r.latency_ms)

    def remaining(self, rid: int, res: dict):
        n = res["rem"]
        v = np.empty((n["nv"], 3), np.float32)
        e = np.empty((n["ne"], 2), np.int32)
        t = np.empty((n["nt"], 3), np.int32)
        self._check(self.lib.vc_server_get_remaining(self.h, rid, v.ctypes.data_as(ctypes.c_void_p),
                                                     e.ctypes.data_as(ctypes.c_void_p),
                                                     t.ctypes.data_as(ctypes.c_void_p)), "vc_server_get_remaining")
        return v, e, t

    def release(self, rid: int):
        self._check(self.lib.vc_server_release(self.h, rid), "vc_server_release")

    def debug_fail_alloc_after(self, k: int):
        """The next batch a worker takes fails its (k+1)-th device allocation."""
        self._check(self.lib.vc_server_debug_fail_alloc_after(self.h, k), "vc_server_debug_fail_alloc_after")

    def stats(self) -> dict:
        s = L.ServerStats()
        self._check(self.lib.vc_server_get_stats(self.h, ctypes.byref(s)), "vc_server_get_stats")
        return {k: getattr(s, k) for k, _ in L.ServerStats._fields_}

    def close(self):
        if getattr(self, "h", None):
            self.lib.vc_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def encode_sof(occ) -> bytes:
    """The .sof octree stream of a dense occupancy volume (host numpy array),
    as the reference's OctreeVolume writes it (vc_encode_sof)."""
    return _encode_octree(occ, "vc_encode_sof")


def encode_sog(occ) -> bytes:
    """The .sog octree stream of a dense occupancy volume (vc_encode_sog)."""
    return _encode_octree(occ, "vc_encode_sog")


def _encode_octree(occ, name: str) -> bytes:
    lib = L.load()
    occ = np.ascontiguousarray(occ, dtype=np.uint8)
    X, Y, Z = (int(s) for s in occ.shape)
    p = occ.ctypes.data_as(ctypes.c_void_p)
    n = ctypes.c_int64()
    st = getattr(lib, name)(p, X, Y, Z, None, 0, ctypes.byref(n))
    if st != L.VC_OK:
        raise L.VoxelCoreError(st, name)
    out = np.zeros(n.value, np.uint8)
    st = getattr(lib, name)(p, X, Y, Z, out.ctypes.data_as(ctypes.c_void_p), n.value, ctypes.byref(n))
    if st != L.VC_OK:
        raise L.VoxelCoreError(st, name)
    return out.tobytes()


def _call(name, *args):
    st = getattr(L.load(), name)(*args)
    if st != L.VC_OK:
        raise L.VoxelCoreError(st, name)


def _arr(a, dtype, cols):
    a = np.ascontiguousarray(np.asarray(a, dtype).reshape(-1, cols) if cols else np.asarray(a, dtype).ravel())
    return a, a.ctypes.data_as(ctypes.c_void_p)


def write_ply(path: str, vts, edges, tris) -> None:
    """writeToPLY: ASCII PLY of a complex (vc_write_ply)."""
    v, pv = _arr(vts, np.float32, 3)
    e, pe = _arr(edges, np.int32, 2)
    t, pt = _arr(tris, np.int32, 3)
    _call("vc_write_ply", os.fsencode(path), pv, len(v), pe, len(e), pt, len(t))


def write_radii(path: str, vts, radii) -> None:
    """writeRadiiToFile: "n", then "x y z r" per vertex (vc_write_radii)."""
    v, pv = _arr(vts, np.float32, 3)
    r, pr = _arr(radii, np.float32, 0)
    if len(r) != len(v):
        raise ValueError("one radius per vertex")
    _call("vc_write_radii", os.fsencode(path), pv, pr, len(v))


def write_dotma(path: str, vts, radii, edges, tris) -> None:
    """writeToDotma: the .ma medial-axis file (vc_write_dotma)."""
    v, pv = _arr(vts, np.float32, 3)
    r, pr = _arr(radii, np.float32, 0)
    e, pe = _arr(edges, np.int32, 2)
    t, pt = _arr(tris, np.int32, 3)
    if len(r) != len(v):
        raise ValueError("one radius per vertex")
    _call("vc_write_dotma", os.fsencode(path), pv, pr, len(v), pe, len(e), pt, len(t))


def dotma_edges(edges, tris) -> np.ndarray:
    """The .ma edge list for remaining edges and triangles (vc_dotma_edges)."""
    e, pe = _arr(edges, np.int32, 2)
    t, pt = _arr(tris, np.int32, 3)
    n = ctypes.c_int64()
    _call("vc_dotma_edges", pe, len(e), pt, len(t), None, 0, ctypes.byref(n))
    out = np.zeros((n.value, 2), np.int32)
    _call("vc_dotma_edges", pe, len(e), pt, len(t), out.ctypes.data_as(ctypes.c_void_p), n.value, ctypes.byref(n))
    return out


def partition_volumes(voxels, nparts: int) -> np.ndarray:
    """Part (GPU or rank) of each volume: vc_partition_volumes."""
    v = np.ascontiguousarray(voxels, dtype=np.int64)
    out = np.zeros(len(v), np.int32)
    _call("vc_partition_volumes", len(v), v.ctypes.data_as(ctypes.c_void_p), nparts,
          out.ctypes.data_as(ctypes.c_void_p))
    return out


def plan_batches(voxels, t, share_bytes: int, bytes_per_voxel: float = 640.0, max_batch: int = 64) -> np.ndarray:
    """vc_plan_batches: the batch number each request (in arrival order) gets."""
    lib = L.load()
    v = np.ascontiguousarray(voxels, np.int64)
    tt = np.ascontiguousarray(np.broadcast_to(np.asarray(t, np.float64), v.shape))
    out = np.empty(len(v), np.int32)
    st = lib.vc_plan_batches(len(v), v.ctypes.data_as(ctypes.c_void_p), tt.ctypes.data_as(ctypes.c_void_p),
                             int(share_bytes), float(bytes_per_voxel), int(max_batch),
                             out.ctypes.data_as(ctypes.c_void_p))
    if st != L.VC_OK:
        raise L.VoxelCoreError(st, "vc_plan_batches", "")
    return out


# ---------------------------------------------------------------------------
# Reference-shaped surfaces

class Surfacer:
    """Surfacer::extractBoundaryVts (include/surfacing.h:57-58) on the GPU."""

    def __init__(self, ctx: Optional[Context] = None):
        self.ctx = ctx or Context()

    def extractBoundaryVts(self, vol, vts: Optional[list] = None):
        self.ctx.set_volume(vol)
        self.ctx.extract_sites()
        pts = self.ctx.sites()
        if vts is not None:
            vts.clear()
            vts.extend(pts)
        return pts


def extract_inside_with_measure(ctx: Context, occ) -> dict:
    """VoroInfo::extractInsideWithMeasure(LAMBDA, ...) for the lattice Voronoi complex of ``occ``.

    Returns vts, edges, tris, from_fi (polygon face per triangle), vts_msure,
    edges_msure, faces_msure, face_sites and inside_size.
    """
    ctx.set_volume(occ)
    ctx.extract_sites()
    ctx.feature_transform()
    ctx.lattice_vd()
    o = ctx.vd()
    return dict(vts=o["vts"], edges=o["edges"], tris=o["tris"], from_fi=o["tri_face"], vts_msure=o["vm"],
                edges_msure=o["em"], faces_msure=o["fm"], face_sites=o["face_sites"], inside_size=o["inside_size"])


class cellcomplex:  # noqa: N801 - reference name
    """cellcomplex(vts, edges, tris, finalize=True) backed by a GPU context."""

    def __init__(self, vts, edges, tris, perform_finalize: bool = True, ctx: Optional[Context] = None):
        self.ctx = ctx or Context()
        self.ctx.set_complex(np.ascontiguousarray(vts, np.float32).reshape(-1, 3),
                             np.ascontiguousarray(edges, np.int32).reshape(-1, 2),
                             np.ascontiguousarray(tris, np.int32).reshape(-1, 3))
        self.vts = np.ascontiguousarray(vts, np.float32).reshape(-1, 3)
        self._fin = None
        if perform_finalize:
            self.finalize()

    def finalize(self):
        self.ctx.finalize()
        self._fin = None

    def _f(self):
        if self._fin is None:
            self._fin = self.ctx.finalized()
        return self._fin

    def numVts(self):
        return self.ctx.nv

    def numEdges(self):
        return self.ctx.ne

    def numFaces(self):
        return self.ctx.nt

    def getEdge(self, i):
        return tuple(self._f()["edges"][i])

    def getFaceERep(self, fi):
        return list(self._f()["tri_edges"][fi])

    def nbEdgesofVert(self, v):
        f = self._f()
        return list(f["ve_ids"][f["ve_off"][v]:f["ve_off"][v + 1]])

    def nbFacesofEdge(self, e):
        f = self._f()
        return list(f["ef_ids"][f["ef_off"][e]:f["ef_off"][e + 1]])

    def refCntPerVert(self):
        return np.diff(self._f()["ve_off"])

    def refCntPerEdge(self):
        return np.diff(self._f()["ef_off"])


class CellComplexThinning:
    """CellComplexThinning (include/ccthin.h:57-113) with prune() on the GPU."""

    def __init__(self):
        self.cc: Optional[cellcomplex] = None
        self._flags = None

    def setup(self, cc: cellcomplex):
        self.cc = cc

    def reset(self):
        self.cc = None
        self._flags = None

    def assignElementValues(self, vert_measures, edge_measures, face_measures):
        self.cc.ctx.set_measures(np.ascontiguousarray(vert_measures, np.float32),
                                 np.ascontiguousarray(edge_measures, np.float32),
                                 np.ascontiguousarray(face_measures, np.float32))

    def preprocess(self):
        self._flags = None

    def prune(self, f_t: float, l_t: float, remove_small_components: bool = False):
        self.stats = self.cc.ctx.thin(f_t, l_t)
        self._flags = self.cc.ctx.thin_flags()
        return self.stats

    def getEdgeRemovedTags(self):
        return self._flags["removed_e"].astype(bool)

    def getFaceRemovedTags(self):
        return ~self._flags["keep_f"].astype(bool)

    def getRemainedVts(self):
        return np.nonzero(self._flags["keep_v"])[0].astype(np.int32)

    def getRemainedEdges(self):
        return np.nonzero(self._flags["keep_e"])[0].astype(np.int32)

    def getRemainedFaces(self):
        return np.nonzero(self._flags["keep_f"])[0].astype(np.int32)

    def remainingCC(self):
        self.cc.ctx.remaining()
        return self.cc.ctx.remaining_arrays()
