"""Python mirror of the reference's voxelization interface, on top of the C ABI.

Names and argument meaning follow the reference: ``voxelize(info, triangle_data, vtable,
morton_code)`` and ``voxelize_solid(...)`` (src/voxelize.cu:192, src/voxelize_solid.cu:147), a
``voxinfo`` with bbox / gridsize / n_triangles / unit (src/util.h:50-69), ``createMeshBBCube``
(src/util.h:80-110).  Device buffers are torch CUDA tensors or raw device pointers (int); PyTorch
is only used for device memory and streams.  Errors raise :class:`CvxError` (the reference exits the
process instead).
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass
from typing import Sequence

import numpy as np

from ._lib import (CvxError, CvxHostJob, CvxJob, CvxServerConfig, CvxServerRequest, CvxServerStats, CvxTuning, CvxVoxinfo,
                   check, lib)

__all__ = ["VoxInfo", "voxelize", "voxelize_solid", "voxelize_ws", "workspace_size", "create_mesh_bbox_cube",
           "mesh_bbox", "make_voxinfo", "table_words", "Job", "voxelize_batch", "Plan", "HostJob", "HostPlan",
           "device_status", "get_tuning", "set_tuning", "CvxError", "stream_release", "voxelize_host",
           "profile_enable", "profile_collect", "Server", "mesh_bbox_device", "voxinfo_from_device", "gather_soup",
           "transcode", "encode_binvox", "binvox_header", "encode_voxel_list"]


VoxInfo = CvxVoxinfo


def _vec3(a) -> ctypes.Array:
    a = np.asarray(a, dtype=np.float32).reshape(3)
    return (ctypes.c_float * 3)(*[float(x) for x in a])


def make_info(bbox_min, bbox_max, gridsize, n_triangles: int) -> VoxInfo:
    """voxinfo constructor (src/util.h:56-61): unit = (max - min) / float(gridsize)."""
    if np.isscalar(gridsize):
        gridsize = (gridsize, gridsize, gridsize)
    g = (ctypes.c_uint32 * 3)(*[int(x) for x in gridsize])
    info = VoxInfo()
    check(lib.cvx_voxinfo_init(ctypes.byref(info), _vec3(bbox_min), _vec3(bbox_max), g, int(n_triangles)),
          "cvx_voxinfo_init")
    return info


def create_mesh_bbox_cube(bbox_min, bbox_max):
    """createMeshBBCube (src/util.h:80-110) on float32 bounds."""
    lo = (ctypes.c_float * 3)()
    hi = (ctypes.c_float * 3)()
    check(lib.cvx_bbox_cube(_vec3(bbox_min), _vec3(bbox_max), lo, hi), "cvx_bbox_cube")
    return np.array(lo[:], dtype=np.float32), np.array(hi[:], dtype=np.float32)


def mesh_bbox(triangles: np.ndarray):
    t = np.ascontiguousarray(triangles, dtype=np.float32).reshape(-1, 9)
    lo = (ctypes.c_float * 3)()
    hi = (ctypes.c_float * 3)()
    check(lib.cvx_mesh_bbox(t.ctypes.data, t.shape[0], lo, hi), "cvx_mesh_bbox")
    return np.array(lo[:], dtype=np.float32), np.array(hi[:], dtype=np.float32)


def make_voxinfo(triangles: np.ndarray, gridsize) -> VoxInfo:
    """What the reference's main() does (src/main.cpp:179-186): vertex bbox, padded to a cube,
    then the voxinfo for a gridsize^3 grid."""
    t = np.ascontiguousarray(triangles, dtype=np.float32).reshape(-1, 9)
    lo, hi = mesh_bbox(t)
    clo, chi = create_mesh_bbox_cube(lo, hi)
    return make_info(clo, chi, gridsize, t.shape[0])


def table_words(info: VoxInfo) -> int:
    return int(lib.cvx_table_words(ctypes.byref(info)))


def _ptr(x) -> int:
    if x is None:
        return 0
    if isinstance(x, int):
        return x
    if hasattr(x, "data_ptr"):
        if not x.is_cuda:
            raise ValueError("device buffers must be CUDA tensors (or raw device pointers)")
        if not x.is_contiguous():
            raise ValueError("device buffers must be contiguous")
        return int(x.data_ptr())
    raise TypeError(f"cannot take a device pointer of {type(x)}")


def _stream(stream) -> int:
    if stream is None:
        import torch
        return int(torch.cuda.current_stream().cuda_stream)
    if isinstance(stream, int):
        return stream
    return int(stream.cuda_stream)


def _check_sizes(info: VoxInfo, triangle_data, vtable) -> None:
    if hasattr(triangle_data, "numel") and triangle_data.numel() < 9 * info.n_triangles:
        raise ValueError(f"triangle_data holds {triangle_data.numel()} floats, need {9 * info.n_triangles}")
    if hasattr(vtable, "numel") and vtable.numel() * vtable.element_size() < 4 * table_words(info):
        raise ValueError(f"vtable holds {vtable.numel() * vtable.element_size()} bytes, "
                         f"need {4 * table_words(info)}")


def voxelize(info: VoxInfo, triangle_data, vtable, morton_code: bool = False, stream=None) -> None:
    """Surface voxelization into ``vtable`` (ORs bits in; zero it first), asynchronous on ``stream``
    (default: torch's current stream)."""
    _check_sizes(info, triangle_data, vtable)
    check(lib.cvx_voxelize(ctypes.byref(info), _ptr(triangle_data), _ptr(vtable), int(bool(morton_code)),
                           _stream(stream)), "cvx_voxelize")


def voxelize_solid(info: VoxInfo, triangle_data, vtable, morton_code: bool = False, stream=None) -> None:
    """Solid voxelization into ``vtable`` (XORs bits in; zero it first)."""
    _check_sizes(info, triangle_data, vtable)
    check(lib.cvx_voxelize_solid(ctypes.byref(info), _ptr(triangle_data), _ptr(vtable), int(bool(morton_code)),
                                 _stream(stream)), "cvx_voxelize_solid")


def stream_release(stream=None) -> None:
    """cvx_stream_release: synchronize ``stream`` and free the scratch the library keeps for it
    (call before destroying a stream used with the library)."""
    check(lib.cvx_stream_release(_stream(stream)), "cvx_stream_release")


def workspace_size(info: VoxInfo, solid: bool) -> int:
    return int(lib.cvx_workspace_size(ctypes.byref(info), int(bool(solid))))


def voxelize_ws(info: VoxInfo, triangle_data, vtable, workspace, morton_code=False, solid=False, stream=None):
    """Voxelize with caller-owned scratch (a CUDA tensor of at least workspace_size() bytes)."""
    _check_sizes(info, triangle_data, vtable)
    nbytes = workspace.numel() * workspace.element_size() if hasattr(workspace, "numel") else 1 << 62
    check(lib.cvx_voxelize_ws(ctypes.byref(info), _ptr(triangle_data), _ptr(vtable), int(bool(morton_code)),
                              int(bool(solid)), _ptr(workspace), int(nbytes), _stream(stream)), "cvx_voxelize_ws")


def device_status(stream=None) -> None:
    check(lib.cvx_device_status(_stream(stream)), "cvx_device_status")


@dataclass
class Job:
    """One mesh of a batch: its voxinfo, device triangles and table, and mode."""

    info: VoxInfo
    triangles: object
    table: object
    morton: bool = False
    solid: bool = False


def _jobs_array(jobs: Sequence[Job]):
    arr = (CvxJob * max(1, len(jobs)))()
    for i, j in enumerate(jobs):
        _check_sizes(j.info, j.triangles, j.table)
        arr[i].info = j.info
        arr[i].d_triangles = _ptr(j.triangles)
        arr[i].d_table = _ptr(j.table)
        arr[i].morton = int(bool(j.morton))
        arr[i].solid = int(bool(j.solid))
    return arr


def voxelize_batch(jobs: Sequence[Job], stream=None) -> None:
    """All jobs in one launch sequence; bit-identical to one voxelize / voxelize_solid per job."""
    arr = _jobs_array(jobs)
    check(lib.cvx_voxelize_batch(arr, len(jobs), _stream(stream)), "cvx_voxelize_batch")


def _apply_tuning() -> None:
    """The device's cached autotuner choice (cuda_voxelizer_gb300.autotune), applied once per device
    and process before the first plan or server is built; without a cache the defaults stay."""
    import torch
    from . import autotune
    autotune.apply_cached_once(torch.cuda.current_device())


class Plan:
    """A batch captured once into a CUDA graph and replayed with one launch."""

    CLEAR_TABLES = 1

    def __init__(self, jobs: Sequence[Job], clear_tables: bool = True):
        _apply_tuning()
        self._jobs = list(jobs)  # keep buffers alive
        arr = _jobs_array(self._jobs)
        h = ctypes.c_void_p()
        check(lib.cvx_plan_create(arr, len(self._jobs), self.CLEAR_TABLES if clear_tables else 0, ctypes.byref(h)),
              "cvx_plan_create")
        self._h = h

    def launch(self, stream=None) -> None:
        check(lib.cvx_plan_launch(self._h, _stream(stream)), "cvx_plan_launch")

    def kernel_nodes(self) -> int:
        """Kernel launches one launch() makes (the graph's kernel nodes)."""
        n = ctypes.c_uint32()
        check(lib.cvx_plan_kernel_nodes(self._h, ctypes.byref(n)), "cvx_plan_kernel_nodes")
        return int(n.value)

    def close(self) -> None:
        if getattr(self, "_h", None):
            lib.cvx_plan_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


@dataclass
class HostJob:
    """One mesh of a host-buffer plan: host triangles in, host table out, with the device buffers
    the plan copies through.  Host buffers must be page-locked (``tensor.pin_memory()``)."""

    info: VoxInfo
    h_triangles: object
    d_triangles: object
    h_table: object
    d_table: object
    morton: bool = False
    solid: bool = False


class HostPlan:
    """cvx_plan_create_host: the whole round trip -- tables zeroed, triangles up in ``n_chunks``
    pieces (0: the library's default), surface jobs voxelizing each piece as it lands, solid jobs
    after the last, each table copied down as soon as it is complete -- as one CUDA graph launch.
    Plans share no device state: two plans over their own device buffers and host tables, launched
    on two streams in turn, overlap one round trip's upload with the other's read-back."""

    def __init__(self, jobs: Sequence[HostJob], n_chunks: int = 0):
        self._jobs = list(jobs)  # keep buffers alive
        arr = (CvxHostJob * max(1, len(self._jobs)))()
        for i, j in enumerate(self._jobs):
            _check_sizes(j.info, j.d_triangles, j.d_table)
            if j.info.n_triangles and _host_nbytes(j.h_triangles) < 36 * j.info.n_triangles:
                raise ValueError(f"job {i}: h_triangles holds fewer than {9 * j.info.n_triangles} floats")
            if _host_nbytes(j.h_table) < 4 * table_words(j.info):
                raise ValueError(f"job {i}: h_table holds fewer than {4 * table_words(j.info)} bytes")
            arr[i].info = j.info
            arr[i].h_triangles = _host_ptr(j.h_triangles, False) if j.info.n_triangles else 0
            arr[i].d_triangles = _ptr(j.d_triangles)
            arr[i].d_table = _ptr(j.d_table)
            arr[i].h_table = _host_ptr(j.h_table, True)
            arr[i].morton = int(bool(j.morton))
            arr[i].solid = int(bool(j.solid))
        h = ctypes.c_void_p()
        check(lib.cvx_plan_create_host(arr, len(self._jobs), int(n_chunks), ctypes.byref(h)), "cvx_plan_create_host")
        self._h = h

    def launch(self, stream=None) -> None:
        check(lib.cvx_plan_launch(self._h, _stream(stream)), "cvx_plan_launch")

    def kernel_nodes(self) -> int:
        """Kernel launches one launch() makes (the graph's kernel nodes)."""
        n = ctypes.c_uint32()
        check(lib.cvx_plan_kernel_nodes(self._h, ctypes.byref(n)), "cvx_plan_kernel_nodes")
        return int(n.value)

    def close(self) -> None:
        if getattr(self, "_h", None):
            lib.cvx_plan_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class HostPipeline:
    """Round trips back to back: ``len(slots)`` host plans, each over its own device buffers and
    host tables (``slots[i]`` is slot i's list of HostJob), launched on their own streams in turn,
    so that one round trip's upload and kernels run while the previous one's tables are still
    going down.  ``submit()`` launches the next slot and returns its index; that slot's host tables
    are complete once ``wait(slot)`` returns.  A slot's next launch rewrites its host tables, so
    read them before the rotation comes back to it (after ``len(slots)`` more submits)."""

    def __init__(self, slots: Sequence[Sequence[HostJob]], n_chunks: int = 0):
        import torch
        if not slots:
            raise ValueError("a pipeline needs at least one slot")
        # slots run at the same time: no buffer may belong to two of them (jobs of one slot may
        # share an upload, as in a single host plan)
        owner = {}
        for i, s in enumerate(slots):
            for j in s:
                for ptr in (_host_ptr(j.h_table, True), _ptr(j.d_table), _ptr(j.d_triangles)):
                    if ptr and owner.setdefault(ptr, i) != i:
                        raise ValueError(f"slots {owner[ptr]} and {i} share a buffer: every slot needs its own")
        self._plans = [HostPlan(s, n_chunks) for s in slots]
        self._streams = [torch.cuda.Stream() for _ in slots]
        self._done = [torch.cuda.Event() for _ in slots]
        self._next = 0

    @property
    def slots(self) -> int:
        return len(self._plans)

    def begin(self, stream=None) -> None:
        """Every slot's next launch follows the work queued so far on `stream` (default: current)."""
        import torch
        s = stream if stream is not None else torch.cuda.current_stream()
        for st in self._streams:
            st.wait_stream(s)

    def submit(self) -> int:
        i = self._next
        self._plans[i].launch(self._streams[i])
        self._done[i].record(self._streams[i])
        self._next = (i + 1) % len(self._plans)
        return i

    def wait(self, slot: int) -> None:
        self._done[slot].synchronize()

    def end(self, stream=None) -> None:
        """Work queued on `stream` (default: current) after this call follows every submitted round trip."""
        import torch
        s = stream if stream is not None else torch.cuda.current_stream()
        for st in self._streams:
            s.wait_stream(st)

    def kernel_nodes(self) -> int:
        """Kernel launches of one submit."""
        return self._plans[0].kernel_nodes()

    def close(self) -> None:
        for p in getattr(self, "_plans", []):
            p.close()


def profile_enable(on: bool = True) -> None:
    """Record per-kernel CUDA events for the calls of this thread (see profile_collect)."""
    check(lib.cvx_profile_enable(int(bool(on))), "cvx_profile_enable")


def profile_collect(max_entries: int = 4096) -> list:
    """[(kernel name, ms), ...] of the calls made since the last collect, in launch order."""
    names = (ctypes.c_char_p * max_entries)()
    ms = (ctypes.c_float * max_entries)()
    n = lib.cvx_profile_collect(names, ms, max_entries)
    return [(names[i].decode(), float(ms[i])) for i in range(n)]


def get_tuning(device: int = 0) -> dict:
    t = CvxTuning()
    check(lib.cvx_get_tuning(device, ctypes.byref(t)), "cvx_get_tuning")
    return {"small_vox": t.small_vox, "small_cols": t.small_cols, "brick_pairs": t.brick_pairs}


def set_tuning(device: int = 0, small_vox: int | None = None, small_cols: int | None = None,
               brick_pairs: int | None = None) -> None:
    cur = get_tuning(device)
    t = CvxTuning(small_vox if small_vox is not None else cur["small_vox"],
                  small_cols if small_cols is not None else cur["small_cols"],
                  brick_pairs if brick_pairs is not None else cur["brick_pairs"])
    check(lib.cvx_set_tuning(device, ctypes.byref(t)), "cvx_set_tuning")


def voxelize_host(info: VoxInfo, triangles: np.ndarray, morton: bool = False, solid: bool = False) -> np.ndarray:
    """Host arrays in, host table out: copies the soup to the device, voxelizes into a zeroed table
    and copies it back (what the reference's main() does around voxelize, src/main.cpp:205-222)."""
    import torch
    t = torch.from_numpy(np.ascontiguousarray(triangles, dtype=np.float32).reshape(-1)).cuda()
    table = torch.zeros(table_words(info), dtype=torch.int32, device="cuda")
    (voxelize_solid if solid else voxelize)(info, t, table, morton)
    return table.cpu().numpy().view(np.uint32)


def _host_ptr(x, writable: bool) -> int:
    """Address of a contiguous host buffer (numpy array or CPU tensor; pinned memory lets the
    server's copies overlap with other batches)."""
    if hasattr(x, "data_ptr"):
        if x.is_cuda:
            raise ValueError("expected a host buffer, got a CUDA tensor")
        if not x.is_contiguous():
            raise ValueError("host buffers must be contiguous")
        return int(x.data_ptr())
    if not isinstance(x, np.ndarray) or not x.flags.c_contiguous or (writable and not x.flags.writeable):
        raise ValueError("host buffers must be C-contiguous numpy arrays (writable for the table) or CPU tensors")
    return int(x.ctypes.data)


def _host_nbytes(x) -> int:
    return x.numel() * x.element_size() if hasattr(x, "numel") else x.nbytes


class Server:
    """Voxelization server (cvx_server_*): requests are admitted by the device memory they need out
    of a fixed budget and batched continuously on ``max_inflight`` streams.  Each request reads its
    triangles from a host buffer and writes its table to a host buffer; both must stay alive until
    the request has been waited for."""

    def __init__(self, memory_budget_bytes: int = 40 << 30, max_batch: int = 256, max_inflight: int = 4):
        _apply_tuning()
        cfg = CvxServerConfig(int(memory_budget_bytes), int(max_batch), int(max_inflight))
        h = ctypes.c_void_p()
        check(lib.cvx_server_create(ctypes.byref(cfg), ctypes.byref(h)), "cvx_server_create")
        self._h = h
        self._keep = {}

    @staticmethod
    def request(info: VoxInfo, triangles, table, morton_code: bool = False, solid: bool = False) -> CvxServerRequest:
        """``triangles``: a host buffer (copied in) or a CUDA tensor (read in place on the device).
        ``table``: a host buffer the result is copied to, or None to keep the table resident on
        the device (see :meth:`table` and :meth:`release`)."""
        if hasattr(triangles, "is_cuda") and triangles.is_cuda:
            _check_sizes(info, triangles, None)
            h_t, d_t = None, _ptr(triangles)
        else:
            if _host_nbytes(triangles) < 36 * info.n_triangles:
                raise ValueError("triangle buffer smaller than 9 floats per triangle")
            h_t, d_t = _host_ptr(triangles, False), None
        if table is not None and _host_nbytes(table) < 4 * table_words(info):
            raise ValueError(f"table buffer smaller than {4 * table_words(info)} bytes")
        h_tab = _host_ptr(table, True) if table is not None else None
        return CvxServerRequest(info, h_t, d_t, h_tab, int(bool(morton_code)), int(bool(solid)))

    def submit(self, info: VoxInfo, triangles, table=None, morton_code: bool = False, solid: bool = False) -> int:
        req = self.request(info, triangles, table, morton_code, solid)
        rid = ctypes.c_uint64()
        check(lib.cvx_server_submit(self._h, ctypes.byref(req), ctypes.byref(rid)), "cvx_server_submit")
        self._keep[rid.value] = (triangles, table)
        return rid.value

    def table(self, rid: int) -> int:
        """Device address of a completed request's resident table (valid until release)."""
        p = ctypes.c_void_p()
        check(lib.cvx_server_table(self._h, int(rid), ctypes.byref(p)), "cvx_server_table")
        return int(p.value or 0)

    def release(self, rid: int) -> None:
        """Frees a completed request's resident table."""
        check(lib.cvx_server_release(self._h, int(rid)), "cvx_server_release")
        self._keep.pop(int(rid), None)

    def wait(self, rid: int, timeout_ms: float = -1.0) -> float:
        """Waits for request ``rid``; returns its latency in ms (submission to table written)."""
        lat = ctypes.c_double()
        st = lib.cvx_server_wait(self._h, int(rid), float(timeout_ms), ctypes.byref(lat))
        if not (st == 1 and b"timed out" in lib.cvx_last_error_message()):
            self._keep.pop(int(rid), None)
        check(st, "cvx_server_wait")
        return lat.value

    def stats(self) -> dict:
        s = CvxServerStats()
        check(lib.cvx_server_stats_get(self._h, ctypes.byref(s)), "cvx_server_stats_get")
        return {k: getattr(s, k) for k, _ in CvxServerStats._fields_}

    def replay(self, pool: Sequence[CvxServerRequest], index, arrival_s) -> np.ndarray:
        """Open-loop load: request i is ``pool[index[i]]``, submitted at ``arrival_s[i]`` seconds
        (ascending) after the call starts.  Returns per-request latency in ms, counted from the
        scheduled arrival.  The pool's buffers must stay alive during the call."""
        index = np.asarray(index, dtype=np.int64)
        arrival = np.ascontiguousarray(arrival_s, dtype=np.float64)
        if index.shape != arrival.shape:
            raise ValueError("index and arrival_s differ in length")
        size = ctypes.sizeof(CvxServerRequest)
        pool_arr = (CvxServerRequest * len(pool))(*pool)
        rows = np.frombuffer(pool_arr, dtype=np.uint8).reshape(len(pool), size)
        reqs = np.ascontiguousarray(rows[index])
        lat = np.zeros(len(index), dtype=np.float64)
        dp = ctypes.POINTER(ctypes.c_double)
        check(lib.cvx_server_replay(self._h, reqs.ctypes.data_as(ctypes.POINTER(CvxServerRequest)), len(index),
                                    arrival.ctypes.data_as(dp), lat.ctypes.data_as(dp)), "cvx_server_replay")
        return lat

    def close(self) -> None:
        if getattr(self, "_h", None):
            lib.cvx_server_destroy(self._h)
            self._h = None
            self._keep.clear()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---- mesh ingest, layouts and output encoders on the GPU ------------------------------------------

def mesh_bbox_device(triangles, stream=None):
    """Vertex bounding box of a device triangle soup (CUDA tensor); host float32 arrays."""
    n = triangles.numel() // 9
    lo = (ctypes.c_float * 3)()
    hi = (ctypes.c_float * 3)()
    check(lib.cvx_mesh_bbox_device(_ptr(triangles), n, lo, hi, _stream(stream)), "cvx_mesh_bbox_device")
    return np.array(lo[:], dtype=np.float32), np.array(hi[:], dtype=np.float32)


def voxinfo_from_device(triangles, gridsize, stream=None) -> VoxInfo:
    """main()'s setup (bbox, createMeshBBCube, voxinfo) for a device triangle soup."""
    if np.isscalar(gridsize):
        gridsize = (gridsize, gridsize, gridsize)
    g = (ctypes.c_uint32 * 3)(*[int(x) for x in gridsize])
    info = VoxInfo()
    check(lib.cvx_voxinfo_from_device(_ptr(triangles), triangles.numel() // 9, g, ctypes.byref(info),
                                      _stream(stream)), "cvx_voxinfo_from_device")
    return info


def gather_soup(vertices, faces, stream=None):
    """Indexed mesh (CUDA float32 vertices (V, 3), int32/uint32 faces (F, 3)) -> (soup (F*9,),
    number of faces with an index out of range).  Synchronizes to read the count."""
    import torch
    f = faces.reshape(-1, 3)
    soup = torch.empty(f.shape[0] * 9, dtype=torch.float32, device=vertices.device)
    bad = torch.zeros(1, dtype=torch.int64, device=vertices.device)
    check(lib.cvx_gather_soup(_ptr(vertices), vertices.numel() // 3, _ptr(f), f.shape[0], _ptr(soup), _ptr(bad),
                              _stream(stream)), "cvx_gather_soup")
    return soup, int(bad.item())


def transcode(table, gridsize: int, to_morton: bool, stream=None):
    """Morton <-> linear copy of a g^3 table (CUDA tensor); returns a new tensor."""
    import torch
    out = torch.empty_like(table)
    check(lib.cvx_transcode(_ptr(table), _ptr(out), int(gridsize), int(bool(to_morton)), _stream(stream)),
          "cvx_transcode")
    return out


def encode_binvox(info: VoxInfo, table, stream=None) -> bytes:
    """binvox run-length payload of a linear-order device table (the bytes after the header)."""
    import torch
    n = ctypes.c_uint64()
    check(lib.cvx_encode_binvox(ctypes.byref(info), _ptr(table), None, 0, ctypes.byref(n), _stream(stream)),
          "cvx_encode_binvox")
    out = torch.empty(max(1, n.value), dtype=torch.uint8, device=table.device)
    check(lib.cvx_encode_binvox(ctypes.byref(info), _ptr(table), _ptr(out), n.value, ctypes.byref(n),
                                _stream(stream)), "cvx_encode_binvox")
    return out[:n.value].cpu().numpy().tobytes()


def binvox_header(info: VoxInfo) -> bytes:
    """The ASCII header write_binvox puts before the payload (src/util_io.cpp:209-215), with the
    stream's default float formatting (6 significant digits)."""
    lo = [np.float32(v) for v in info.bbox_min]
    hi = [np.float32(v) for v in info.bbox_max]
    ext = [np.float32(hi[i] - lo[i]) for i in range(3)]
    scale = max(max(ext[0], ext[1]), ext[2])
    g = list(info.gridsize)
    return (f"#binvox 1\ndim {g[0]} {g[1]} {g[2]}\n"
            f"translate {'%g' % float(lo[0])} {'%g' % float(lo[1])} {'%g' % float(lo[2])}\n"
            f"scale {'%g' % float(scale)}\ndata\n").encode()


def encode_voxel_list(info: VoxInfo, table, stream=None):
    """The (x, gz - z, y) int32 triples write_vox hands to its MagicaVoxel writer, in its order."""
    import torch
    n = ctypes.c_uint64()
    check(lib.cvx_encode_voxel_list(ctypes.byref(info), _ptr(table), None, 0, ctypes.byref(n), _stream(stream)),
          "cvx_encode_voxel_list")
    out = torch.empty((max(1, n.value), 3), dtype=torch.int32, device=table.device)
    check(lib.cvx_encode_voxel_list(ctypes.byref(info), _ptr(table), _ptr(out), n.value, ctypes.byref(n),
                                    _stream(stream)), "cvx_encode_voxel_list")
    return out[:n.value]
