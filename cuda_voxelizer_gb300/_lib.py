"""ctypes binding of libcvx.so (include/cvx.h).  Importing this module loads the native library and
raises ImportError if it has not been built: there is no fallback path."""
from __future__ import annotations

import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libcvx.so")

if not os.path.exists(LIB_PATH):
    raise ImportError(f"{LIB_PATH} is missing; build it with `python cuda_voxelizer_gb300/build.py` "
                      "(or __graft_entry__.build())")

lib = ctypes.CDLL(LIB_PATH)

c_status = ctypes.c_int
vp = ctypes.c_void_p
u32 = ctypes.c_uint32
u64 = ctypes.c_uint64


class CvxVoxinfo(ctypes.Structure):
    """cvx_voxinfo == the reference voxinfo (src/util.h:50-69), 64 bytes."""

    _fields_ = [("bbox_min", ctypes.c_float * 3), ("bbox_max", ctypes.c_float * 3),
                ("gridsize", ctypes.c_uint32 * 3), ("_pad0", ctypes.c_uint32),
                ("n_triangles", ctypes.c_uint64), ("unit", ctypes.c_float * 3), ("_pad1", ctypes.c_uint32)]


class CvxJob(ctypes.Structure):
    _fields_ = [("info", CvxVoxinfo), ("d_triangles", vp), ("d_table", vp), ("morton", ctypes.c_int32),
                ("solid", ctypes.c_int32)]


class CvxHostJob(ctypes.Structure):
    _fields_ = [("info", CvxVoxinfo), ("h_triangles", vp), ("d_triangles", vp), ("d_table", vp), ("h_table", vp),
                ("morton", ctypes.c_int32), ("solid", ctypes.c_int32)]


class CvxServerConfig(ctypes.Structure):
    _fields_ = [("memory_budget_bytes", u64), ("max_batch", u32), ("max_inflight", u32)]


class CvxServerRequest(ctypes.Structure):
    _fields_ = [("info", CvxVoxinfo), ("h_triangles", vp), ("d_triangles", vp), ("h_table", vp),
                ("morton", ctypes.c_int32), ("solid", ctypes.c_int32)]


class CvxServerStats(ctypes.Structure):
    _fields_ = [("completed", u64), ("pending", u64), ("batches", u64), ("mean_batch", ctypes.c_double),
                ("memory_used", u64), ("memory_budget", u64), ("memory_peak", u64), ("p50_ms", ctypes.c_double),
                ("p99_ms", ctypes.c_double), ("max_ms", ctypes.c_double), ("meshes_per_s", ctypes.c_double),
                ("queue_p99_ms", ctypes.c_double), ("replay_late_p99_ms", ctypes.c_double),
                ("replay_late_max_ms", ctypes.c_double), ("service_p50_ms", ctypes.c_double),
                ("service_p99_ms", ctypes.c_double), ("issue_p50_us", ctypes.c_double)]


class CvxTuning(ctypes.Structure):
    _fields_ = [("small_vox", ctypes.c_uint32), ("small_cols", ctypes.c_uint32), ("brick_pairs", ctypes.c_uint32)]


assert ctypes.sizeof(CvxVoxinfo) == 64

# Every symbol of include/cvx.h with its signature.
SIGNATURES = {
    "cvx_status_string": (ctypes.c_char_p, [c_status]),
    "cvx_last_error_message": (ctypes.c_char_p, []),
    "cvx_version": (ctypes.c_int, []),
    "cvx_voxinfo_init": (c_status, [ctypes.POINTER(CvxVoxinfo), vp, vp, vp, u64]),
    "cvx_bbox_cube": (c_status, [vp, vp, vp, vp]),
    "cvx_mesh_bbox": (c_status, [vp, u64, vp, vp]),
    "cvx_table_words": (u64, [ctypes.POINTER(CvxVoxinfo)]),
    "cvx_voxelize": (c_status, [ctypes.POINTER(CvxVoxinfo), vp, vp, ctypes.c_int, vp]),
    "cvx_voxelize_solid": (c_status, [ctypes.POINTER(CvxVoxinfo), vp, vp, ctypes.c_int, vp]),
    "cvx_workspace_size": (u64, [ctypes.POINTER(CvxVoxinfo), ctypes.c_int]),
    "cvx_voxelize_ws": (c_status, [ctypes.POINTER(CvxVoxinfo), vp, vp, ctypes.c_int, ctypes.c_int, vp, u64, vp]),
    "cvx_voxelize_solid_noalloc": (c_status, [ctypes.POINTER(CvxVoxinfo), vp, vp, ctypes.c_int, vp]),
    "cvx_device_status": (c_status, [vp]),
    "cvx_stream_release": (c_status, [vp]),
    "cvx_voxelize_batch": (c_status, [ctypes.POINTER(CvxJob), u32, vp]),
    "cvx_plan_create": (c_status, [ctypes.POINTER(CvxJob), u32, u32, ctypes.POINTER(vp)]),
    "cvx_plan_create_host": (c_status, [ctypes.POINTER(CvxHostJob), u32, u32, ctypes.POINTER(vp)]),
    "cvx_plan_launch": (c_status, [vp, vp]),
    "cvx_plan_kernel_nodes": (c_status, [vp, ctypes.POINTER(u32)]),
    "cvx_plan_destroy": (c_status, [vp]),
    "cvx_server_create": (c_status, [ctypes.POINTER(CvxServerConfig), ctypes.POINTER(vp)]),
    "cvx_server_submit": (c_status, [vp, ctypes.POINTER(CvxServerRequest), ctypes.POINTER(u64)]),
    "cvx_server_wait": (c_status, [vp, u64, ctypes.c_double, ctypes.POINTER(ctypes.c_double)]),
    "cvx_server_table": (c_status, [vp, u64, ctypes.POINTER(vp)]),
    "cvx_server_release": (c_status, [vp, u64]),
    "cvx_server_stats_get": (c_status, [vp, ctypes.POINTER(CvxServerStats)]),
    "cvx_server_replay": (c_status, [vp, ctypes.POINTER(CvxServerRequest), u32, ctypes.POINTER(ctypes.c_double),
                                     ctypes.POINTER(ctypes.c_double)]),
    "cvx_server_destroy": (c_status, [vp]),
    "cvx_mesh_bbox_device": (c_status, [vp, u64, vp, vp, vp]),
    "cvx_voxinfo_from_device": (c_status, [vp, u64, vp, ctypes.POINTER(CvxVoxinfo), vp]),
    "cvx_gather_soup": (c_status, [vp, u64, vp, u64, vp, vp, vp]),
    "cvx_transcode": (c_status, [vp, vp, u32, ctypes.c_int, vp]),
    "cvx_encode_binvox": (c_status, [ctypes.POINTER(CvxVoxinfo), vp, vp, u64, ctypes.POINTER(u64), vp]),
    "cvx_encode_voxel_list": (c_status, [ctypes.POINTER(CvxVoxinfo), vp, vp, u64, ctypes.POINTER(u64), vp]),
    "cvx_get_tuning": (c_status, [ctypes.c_int, ctypes.POINTER(CvxTuning)]),
    "cvx_set_tuning": (c_status, [ctypes.c_int, ctypes.POINTER(CvxTuning)]),
    "cvx_profile_enable": (c_status, [ctypes.c_int]),
    "cvx_profile_collect": (ctypes.c_int, [ctypes.POINTER(ctypes.c_char_p), ctypes.POINTER(ctypes.c_float), ctypes.c_int]),
}

for _name, (_res, _args) in SIGNATURES.items():
    _f = getattr(lib, _name)
    _f.restype = _res
    _f.argtypes = _args

STATUS = {0: "CVX_OK", 1: "CVX_ERR_INVALID_VALUE", 2: "CVX_ERR_UNSUPPORTED", 3: "CVX_ERR_OUT_OF_MEMORY",
          4: "CVX_ERR_CUDA", 5: "CVX_ERR_DEVICE_CHECK", 6: "CVX_ERR_CAPTURING"}


class CvxError(RuntimeError):
    def __init__(self, status: int, where: str):
        self.status = status
        msg = lib.cvx_last_error_message().decode(errors="replace")
        super().__init__(f"{where}: {STATUS.get(status, status)}: {msg}")


def check(status: int, where: str) -> None:
    if status != 0:
        raise CvxError(status, where)


def diag_lib():
    """libcvx_diag.so (include/cvx_diag.h): the atomicOr-rate measurement behind the roofline.  Not
    part of the voxelization library; loaded on demand by measurement code."""
    global _diag
    try:
        return _diag
    except NameError:
        pass
    d = ctypes.CDLL(os.path.join(_HERE, "_lib", "libcvx_diag.so"))
    d.cvx_microbench_atomic_or.restype = ctypes.c_double
    d.cvx_microbench_atomic_or.argtypes = [vp, u64, ctypes.c_int, u32, u32]
    _diag = d
    return d
