"""GB300-native voxelization engine: a drop-in for the voxelize / voxelize_solid path of
Forceflow/cuda_voxelizer, implemented as hand-written sm_103a CUDA behind a C ABI (include/cvx.h).

The native library ``_lib/libcvx.so`` is required; importing this package without it raises
ImportError.
"""
from .api import (CvxError, HostJob, HostPipeline, HostPlan, Job, Plan, Server, VoxInfo, binvox_header, create_mesh_bbox_cube,
                  device_status, encode_binvox, encode_voxel_list, gather_soup, get_tuning, make_info, make_voxinfo,
                  mesh_bbox, mesh_bbox_device, profile_collect, profile_enable, set_tuning, stream_release,
                  table_words, transcode, voxelize, voxelize_batch, voxelize_host, voxelize_solid, voxelize_ws,
                  voxinfo_from_device, workspace_size)

__all__ = ["CvxError", "HostJob", "HostPipeline", "HostPlan", "Job", "Plan", "Server", "VoxInfo", "binvox_header",
           "create_mesh_bbox_cube", "device_status", "encode_binvox", "encode_voxel_list", "gather_soup",
           "get_tuning", "make_info", "make_voxinfo", "mesh_bbox", "mesh_bbox_device", "profile_collect",
           "profile_enable", "set_tuning", "stream_release", "table_words", "transcode", "voxelize",
           "voxelize_batch", "voxelize_host", "voxelize_solid", "voxelize_ws", "voxinfo_from_device",
           "workspace_size"]
