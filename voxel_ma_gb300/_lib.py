"""ctypes binding of libvoxelcore_gb300.so (the C ABI in include/voxelcore_gb300.h).

The library is the only compute path: when it is missing or cannot be loaded
on a machine with a GPU, every call raises -- there is no CPU fallback.
"""
from __future__ import annotations

import ctypes
import os
import threading

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libvoxelcore_gb300.so")

VC_OK, VC_ERR_ARG, VC_ERR_OOM, VC_ERR_TIMEOUT, VC_ERR_INVARIANT, VC_ERR_CUDA, VC_ERR_STATE = range(7)
VC_MEM_HOST, VC_MEM_DEVICE = 0, 1
VC_WRITE_PLY, VC_WRITE_RADII, VC_WRITE_MA = 1, 2, 4

c_i64 = ctypes.c_int64
c_vp = ctypes.c_void_p
c_int = ctypes.c_int
c_float = ctypes.c_float


class VdSizes(ctypes.Structure):
    _fields_ = [("nv", c_i64), ("ne", c_i64), ("nt", c_i64), ("nface", c_i64), ("inside_size", c_float)]


class ThinStats(ctypes.Structure):
    _fields_ = [("pushes", c_i64), ("processed", c_i64), ("skipped", c_i64), ("generations", c_i64)]


class RemSizes(ctypes.Structure):
    _fields_ = [("nv", c_i64), ("ne", c_i64), ("nt", c_i64)]


class EulerInfo(ctypes.Structure):
    _fields_ = [("V", c_i64), ("E", c_i64), ("F", c_i64), ("C", c_i64), ("euler", c_i64)]


class PlainResult(ctypes.Structure):
    _fields_ = [("n_sites", c_i64), ("vd", VdSizes), ("thresh", c_float), ("thin", ThinStats), ("rem", RemSizes)]


class BatchVolume(ctypes.Structure):
    _fields_ = [("n_sites", c_i64), ("vd", VdSizes), ("thresh", c_float), ("rem", RemSizes), ("euler", EulerInfo),
                ("site_off", c_i64), ("v_off", c_i64), ("e_off", c_i64), ("t_off", c_i64),
                ("rem_v_off", c_i64), ("rem_e_off", c_i64), ("rem_t_off", c_i64)]


class RequestResult(ctypes.Structure):
    _fields_ = [("status", c_int), ("batch_size", c_int), ("n_sites", c_i64), ("vd", VdSizes), ("thresh", c_float),
                ("rem", RemSizes), ("euler", EulerInfo), ("queue_ms", ctypes.c_double), ("run_ms", ctypes.c_double),
                ("latency_ms", ctypes.c_double)]


class ServerStats(ctypes.Structure):
    _fields_ = [("submitted", c_i64), ("completed", c_i64), ("failed", c_i64), ("refused", c_i64),
                ("batches", c_i64), ("pending", c_i64), ("device_bytes", c_i64)]


class TuneResult(ctypes.Structure):
    _fields_ = [("ft_ring", c_int), ("thin_threads", c_int), ("thin_blocks_per_sm", c_int),
                ("ft_ms", c_float * 3), ("thin_items", c_int), ("thin_ms", c_float * 5),
                ("ft_method", c_int), ("ft_window_ms", c_float)]


# name -> (restype, argtypes)
SIGNATURES = {
    "vc_version": (c_int, []),
    "vc_status_string": (ctypes.c_char_p, [c_int]),
    "vc_ctx_create": (c_int, [ctypes.POINTER(c_vp), c_int]),
    "vc_ctx_destroy": (c_int, [c_vp]),
    "vc_ctx_stream": (c_vp, [c_vp]),
    "vc_ctx_sync": (c_int, [c_vp]),
    "vc_ctx_last_error": (ctypes.c_char_p, [c_vp]),
    "vc_ctx_device_bytes": (c_i64, [c_vp]),
    "vc_ctx_launch_count": (c_i64, [c_vp]),
    "vc_ctx_set_timing": (c_int, [c_vp, c_int]),
    "vc_ctx_reset_timings": (c_int, [c_vp]),
    "vc_ctx_get_timings": (c_int, [c_vp, ctypes.c_char_p, c_int, ctypes.POINTER(ctypes.c_double),
                                   ctypes.POINTER(c_i64), c_int, ctypes.POINTER(c_int)]),
    "vc_set_volume": (c_int, [c_vp, c_vp, c_int, c_int, c_int, c_int]),
    "vc_extract_sites": (c_int, [c_vp, ctypes.POINTER(c_i64)]),
    "vc_get_sites": (c_int, [c_vp, c_vp, c_int]),
    "vc_feature_transform": (c_int, [c_vp]),
    "vc_get_ft": (c_int, [c_vp, c_vp, c_vp, c_int]),
    "vc_lattice_vd": (c_int, [c_vp, ctypes.POINTER(VdSizes)]),
    "vc_get_vd": (c_int, [c_vp] + [c_vp] * 8 + [c_int]),
    "vc_vertex_radii": (c_int, [c_vp, c_vp, c_int]),
    "vc_batch_set_volumes": (c_int, [c_vp, c_int, c_vp, c_vp, c_int]),
    "vc_batch_run": (c_int, [c_vp, ctypes.c_double, c_int, ctypes.POINTER(ThinStats), c_vp]),
    "vc_server_create": (c_int, [ctypes.POINTER(c_vp), c_int, c_int, c_i64, c_int]),
    "vc_server_set_bytes_per_voxel": (c_int, [c_vp, ctypes.c_double]),
    "vc_server_submit": (c_int, [c_vp, c_vp, c_int, c_int, c_int, ctypes.c_double, ctypes.POINTER(c_i64)]),
    "vc_server_wait": (c_int, [c_vp, c_i64, ctypes.c_double, ctypes.POINTER(RequestResult)]),
    "vc_server_get_remaining": (c_int, [c_vp, c_i64, c_vp, c_vp, c_vp]),
    "vc_server_release": (c_int, [c_vp, c_i64]),
    "vc_server_get_stats": (c_int, [c_vp, ctypes.POINTER(ServerStats)]),
    "vc_server_destroy": (c_int, [c_vp]),
    "vc_server_create_devices": (c_int, [c_vp, c_vp, c_int, c_int, c_i64, c_int]),
    "vc_partition_volumes": (c_int, [c_int, c_vp, c_int, c_vp]),
    "vc_server_debug_fail_alloc_after": (c_int, [c_vp, c_i64]),
    "vc_plan_batches": (c_int, [c_int, c_vp, c_vp, c_i64, ctypes.c_double, c_int, c_vp]),
    "vc_set_complex": (c_int, [c_vp, c_i64, c_vp, c_i64, c_vp, c_i64, c_vp, c_int]),
    "vc_finalize": (c_int, [c_vp, ctypes.POINTER(c_i64)]),
    "vc_get_finalized": (c_int, [c_vp] + [c_vp] * 6 + [c_int]),
    "vc_set_measures": (c_int, [c_vp, c_vp, c_vp, c_vp, c_int]),
    "vc_thin": (c_int, [c_vp, c_float, c_float, ctypes.POINTER(ThinStats)]),
    "vc_get_thin_flags": (c_int, [c_vp, c_vp, c_vp, c_vp, c_vp, c_int]),
    "vc_remaining": (c_int, [c_vp, ctypes.POINTER(RemSizes)]),
    "vc_get_remaining": (c_int, [c_vp, c_vp, c_vp, c_vp, c_int]),
    "vc_euler_remaining": (c_int, [c_vp, ctypes.POINTER(EulerInfo)]),
    "vc_extract_sites_noalloc": (c_int, [c_vp, c_int, c_int, c_int, c_vp, c_i64, ctypes.POINTER(c_i64), c_vp]),
    "vc_debug_thin_trace": (c_int, [c_vp, c_int, c_int]),
    "vc_debug_get_thin_trace": (c_int, [c_vp, c_vp, c_int, ctypes.POINTER(c_int)]),
    "vc_debug_ft_wide": (c_int, [c_vp, c_int]),
    "vc_set_ft_method": (c_int, [c_vp, c_int]),
    "vc_closed_components": (c_int, [c_vp, ctypes.POINTER(c_i64)]),
    "vc_set_volume_sof": (c_int, [c_vp, c_vp, c_i64, ctypes.POINTER(c_int)]),
    "vc_get_volume": (c_int, [c_vp, c_vp, c_int]),
    "vc_encode_sof": (c_int, [c_vp, c_int, c_int, c_int, c_vp, c_i64, ctypes.POINTER(c_i64)]),
    "vc_encode_sog": (c_int, [c_vp, c_int, c_int, c_int, c_vp, c_i64, ctypes.POINTER(c_i64)]),
    "vc_set_volume_sog": (c_int, [c_vp, c_vp, c_i64, ctypes.POINTER(c_int)]),
    "vc_set_volume_mrc": (c_int, [c_vp, c_vp, c_i64, c_vp]),
    "vc_mrc_dims": (c_int, [c_vp, c_i64, c_vp]),
    "vc_get_vox_to_model": (c_int, [c_vp, c_vp]),
    "vc_write_ply": (c_int, [ctypes.c_char_p, c_vp, c_i64, c_vp, c_i64, c_vp, c_i64]),
    "vc_write_radii": (c_int, [ctypes.c_char_p, c_vp, c_vp, c_i64]),
    "vc_write_dotma": (c_int, [ctypes.c_char_p, c_vp, c_vp, c_i64, c_vp, c_i64, c_vp, c_i64]),
    "vc_dotma_edges": (c_int, [c_vp, c_i64, c_vp, c_i64, c_vp, c_i64, ctypes.POINTER(c_i64)]),
    "vc_write_remaining": (c_int, [c_vp, ctypes.c_char_p, c_int]),
    "vc_debug_random_rate": (c_int, [c_vp, c_int, c_i64, ctypes.POINTER(ctypes.c_double)]),
    "vc_debug_thin_shape": (c_int, [c_vp, c_int, c_int, c_int]),
    "vc_debug_set_spin_limit": (c_int, [c_vp, ctypes.c_ulonglong]),
    "vc_debug_fail_alloc_after": (c_int, [c_vp, c_i64]),
    "vc_debug_ref_bias": (c_int, [c_vp, c_i64, c_int]),
    "vc_debug_thin_queue": (c_int, [c_vp, c_i64, ctypes.c_uint32]),
    "vc_autotune": (c_int, [c_vp, ctypes.c_double, ctypes.POINTER(TuneResult)]),
    "vc_lambda_fp64_check": (c_int, [c_vp, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(c_i64)]),
    "vc_run_plain": (c_int, [c_vp, c_vp, c_int, c_int, c_int, c_int, ctypes.c_double, ctypes.POINTER(PlainResult)]),
}

_lib = None
_lock = threading.Lock()


class VoxelCoreError(RuntimeError):
    def __init__(self, status: int, where: str, detail: str = ""):
        self.status = status
        super().__init__(f"{where}: status {status} ({STATUS_NAMES.get(status, '?')}) {detail}".strip())


STATUS_NAMES = {VC_OK: "ok", VC_ERR_ARG: "VC_ERR_ARG", VC_ERR_OOM: "VC_ERR_OOM", VC_ERR_TIMEOUT: "VC_ERR_TIMEOUT",
                VC_ERR_INVARIANT: "VC_ERR_INVARIANT", VC_ERR_CUDA: "VC_ERR_CUDA", VC_ERR_STATE: "VC_ERR_STATE"}


def load(build_if_missing: bool = True):
    """Load (building first if needed) libvoxelcore_gb300.so and bind every entry point."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if build_if_missing:
            from . import build as _build
            _build.build()
        if not os.path.exists(LIB_PATH):
            raise FileNotFoundError(f"{LIB_PATH} is missing; run voxel_ma_gb300.build.build()")
        lib = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
        return lib
