"""CPU tests of the C ABI: the library loads, exports every function declared in include/*.h, the
voxinfo layout is the reference's, and argument validation answers without touching a GPU."""
import ctypes
import os
import re

import numpy as np
import pytest

from cuda_voxelizer_gb300 import _lib
from cuda_voxelizer_gb300 import api as cv

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for h in ("cvx.h",):
        src = open(os.path.join(ROOT, "include", h)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b(cvx_\w+)\s*\(", src, flags=re.M):
            names.add(m.group(1))
    return sorted(names)


def test_header_declares_functions():
    names = declared_functions()
    assert "cvx_voxelize" in names and "cvx_voxelize_solid" in names and len(names) >= 15


@pytest.mark.parametrize("name", declared_functions())
def test_every_declared_function_is_exported(name):
    assert hasattr(_lib.lib, name)
    assert name in _lib.SIGNATURES, f"{name} has no ctypes signature"


def test_diagnostics_library_is_separate():
    # the atomicOr-rate measurement (include/cvx_diag.h) lives in libcvx_diag.so, not in the ABI library
    assert not hasattr(_lib.lib, "cvx_microbench_atomic_or")
    assert hasattr(_lib.diag_lib(), "cvx_microbench_atomic_or")


def test_dropin_cxx_symbols_exported():
    # void voxelize(const voxinfo&, float*, unsigned int*, bool) and voxelize_solid(...), C++ linkage
    for sym in ("_Z8voxelizeRK7voxinfoPfPjb", "_Z14voxelize_solidRK7voxinfoPfPjb"):
        assert hasattr(_lib.lib, sym)


def test_voxinfo_layout_matches_reference():
    V = _lib.CvxVoxinfo
    assert ctypes.sizeof(V) == 64
    assert V.bbox_min.offset == 0 and V.bbox_max.offset == 12
    assert V.gridsize.offset == 24 and V.n_triangles.offset == 40 and V.unit.offset == 48


def test_version_and_status_strings():
    assert _lib.lib.cvx_version() >= 1000
    assert _lib.lib.cvx_status_string(0) == b"CVX_OK"
    assert _lib.lib.cvx_status_string(2) == b"CVX_ERR_UNSUPPORTED"


def _info(g=64, n=1):
    return cv.make_info((0, 0, 0), (1, 1, 1), g, n)


def test_validation_rejects_null_and_zero_grid():
    info = _info()
    assert _lib.lib.cvx_voxelize(None, 1, 1, 0, None) == 1
    assert _lib.lib.cvx_voxelize(ctypes.byref(info), None, 1, 0, None) == 1
    assert _lib.lib.cvx_voxelize(ctypes.byref(info), 1, None, 0, None) == 1
    bad = _info()
    bad.gridsize[1] = 0
    assert _lib.lib.cvx_voxelize_solid(ctypes.byref(bad), 1, 1, 0, None) == 1
    assert b"gridsize" in _lib.lib.cvx_last_error_message()


def test_morton_needs_cubic_power_of_two():
    for g in ((100, 100, 100), (64, 64, 32)):
        info = cv.make_info((0, 0, 0), (1, 1, 1), g, 1)
        assert _lib.lib.cvx_voxelize(ctypes.byref(info), 1, 1, 1, None) == 2
        assert _lib.lib.cvx_voxelize_solid(ctypes.byref(info), 1, 1, 1, None) == 2


def test_noalloc_applies_the_per_axis_limit():
    """cvx_voxelize_solid_noalloc refuses an axis above 2^22 like cvx_voxelize_solid, although a
    2^23 x 2 x 1 grid fits its fixed scratch; the checks run before any CUDA call."""
    info = _info()
    info.gridsize[0], info.gridsize[1], info.gridsize[2] = 1 << 23, 2, 1
    assert _lib.lib.cvx_voxelize_solid_noalloc(ctypes.byref(info), 1, 1, 0, None) == 2
    assert b"above 2^22" in _lib.lib.cvx_last_error_message()
    assert _lib.lib.cvx_voxelize_solid_noalloc(None, 1, 1, 0, None) == 1
    m = cv.make_info((0, 0, 0), (1, 1, 1), (100, 100, 100), 1)
    assert _lib.lib.cvx_voxelize_solid_noalloc(ctypes.byref(m), 1, 1, 1, None) == 2


def test_empty_mesh_is_a_no_op():
    info = _info(n=0)
    assert _lib.lib.cvx_voxelize(ctypes.byref(info), None, 1, 0, None) == 0


def test_workspace_size():
    info = _info(64, 1000)
    s = _lib.lib.cvx_workspace_size(ctypes.byref(info), 0)
    d = _lib.lib.cvx_workspace_size(ctypes.byref(info), 1)
    assert s >= 1000 * 32 and d >= s + 64 ** 3 // 8


def test_ws_rejects_small_or_misaligned_workspace():
    info = _info(64, 10)
    need = _lib.lib.cvx_workspace_size(ctypes.byref(info), 0)
    assert _lib.lib.cvx_voxelize_ws(ctypes.byref(info), 1, 1, 0, 0, 256, need - 1, None) == 1
    assert _lib.lib.cvx_voxelize_ws(ctypes.byref(info), 1, 1, 0, 0, 257, need, None) == 1


def test_mesh_bbox_host():
    t = np.array([[0, 1, 2, 3, -4, 5, 6, 7, 8]], dtype=np.float32)
    lo, hi = cv.mesh_bbox(t)
    assert list(lo) == [0, -4, 2] and list(hi) == [6, 7, 8]
    with pytest.raises(cv.CvxError):
        cv.mesh_bbox(np.zeros((0, 9), np.float32))


def test_server_config_validation_answers_without_a_gpu():
    h = ctypes.c_void_p()
    for budget, batch, inflight in ((0, 8, 2), (64 << 20, 0, 2), (64 << 20, 65537, 2), (64 << 20, 8, 0),
                                    (64 << 20, 8, 65)):
        cfg = _lib.CvxServerConfig(budget, batch, inflight)
        assert _lib.lib.cvx_server_create(ctypes.byref(cfg), ctypes.byref(h)) == 1
    assert b"budget" in _lib.lib.cvx_last_error_message()
    assert _lib.lib.cvx_server_submit(None, None, None) == 1
    assert _lib.lib.cvx_server_destroy(None) == 0


def test_server_request_struct_layout():
    R = _lib.CvxServerRequest
    assert ctypes.sizeof(R) == 64 + 8 + 8 + 8 + 4 + 4
    assert R.h_triangles.offset == 64 and R.d_triangles.offset == 72 and R.h_table.offset == 80
    assert R.solid.offset == 92


def test_host_job_struct_layout():
    J = _lib.CvxHostJob
    assert ctypes.sizeof(J) == 104  # static_assert in the library
    assert (J.h_triangles.offset, J.d_triangles.offset, J.d_table.offset, J.h_table.offset) == (64, 72, 80, 88)
    assert J.morton.offset == 96 and J.solid.offset == 100


def test_host_plan_validation_answers_without_a_gpu():
    info = _info()
    info.n_triangles = 10
    h = ctypes.c_void_p()
    job = _lib.CvxHostJob()
    job.info = info
    job.h_triangles, job.d_triangles, job.d_table, job.h_table = 16, 32, 48, 64
    assert _lib.lib.cvx_plan_create_host(ctypes.byref(job), 1, 0, None) == 1  # out is null
    assert _lib.lib.cvx_plan_create_host(None, 1, 0, ctypes.byref(h)) == 1  # jobs is null
    assert _lib.lib.cvx_plan_create_host(ctypes.byref(job), 1, 65, ctypes.byref(h)) == 1
    assert b"n_chunks" in _lib.lib.cvx_last_error_message()
    for field in ("h_table", "h_triangles", "d_table", "d_triangles"):
        bad = _lib.CvxHostJob.from_buffer_copy(bytes(job))
        setattr(bad, field, None)
        assert _lib.lib.cvx_plan_create_host(ctypes.byref(bad), 1, 0, ctypes.byref(h)) == 1
        assert not h.value
    job.morton = 1
    job.info.gridsize[1] = 32  # Morton order needs a cubic power-of-two grid
    assert _lib.lib.cvx_plan_create_host(ctypes.byref(job), 1, 0, ctypes.byref(h)) != 0


def test_server_stats_struct_layout():
    S = _lib.CvxServerStats
    assert ctypes.sizeof(S) == 136  # static_assert in the library
    assert S.meshes_per_s.offset == 80 and S.queue_p99_ms.offset == 88 and S.issue_p50_us.offset == 128


def test_host_pipeline_refuses_slots_sharing_a_buffer():
    """Slots of a HostPipeline run at the same time, so no device buffer or host table may belong
    to two of them; the check runs before any plan is built (no GPU call)."""
    info = _info()
    h1, h2 = np.zeros(16, np.uint32), np.zeros(16, np.uint32)
    tri = np.zeros(9, np.float32)
    a = [cv.HostJob(info, tri, 4096, h1, 8192)]
    for b in ([cv.HostJob(info, tri, 12288, h1, 16384)],   # the same host table
              [cv.HostJob(info, tri, 12288, h2, 8192)],    # the same device table
              [cv.HostJob(info, tri, 4096, h2, 16384)]):   # the same device triangles
        with pytest.raises(ValueError, match="share a buffer"):
            cv.HostPipeline([a, b])
    with pytest.raises(ValueError):
        cv.HostPipeline([])
