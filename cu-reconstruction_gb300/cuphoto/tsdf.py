"""Python mirror of the reference's TSDF volume interface.

Same names and argument meaning as the reference's C++ API:

  TSDFVolumeConfig              modules/include/cuda/tsdf_volume.cuh:17-29
  TSDFVolume(cfg)               tsdf_volume.cu:194-212
  TSDFVolume.integrate(color, depth, camera_pose) -> bool
                                tsdf_volume.cu:257-290
  TSDFVolume accessors          tsdf_volume.cuh:57-92
  generate_triangular_surface(volume, vertices, triangles)
                                marching_cubes.cu:191-237

Errors follow the reference: ``integrate`` logs and returns False for a
missing or empty depth/colour image; CUDA failures raise.  Everything runs on
the engine's CUDA kernels through the C ABI; torch provides device memory and
streams only.
"""
import ctypes as C
import os
import sys
from dataclasses import dataclass, field

import numpy as np

from . import _lib as L

_TORCH = None


def _torch():
    global _TORCH
    if _TORCH is None:
        import torch
        _TORCH = torch
    return _TORCH


@dataclass
class TSDFVolumeConfig:
    """Fields of cuphoto::TSDFVolumeConfig (tsdf_volume.cuh:17-29) plus the
    engine's options (mode, arith, truncation, max_depth, min_z, memory)."""
    voxel_grid_size: tuple = (256, 256, 256)
    physical_size: tuple = (2.56, 2.56, 2.56)
    global_offset: tuple = (0.0, 0.0, 0.0)
    max_weight: float = 128.0
    focal_x: float = 525.0
    focal_y: float = 525.0
    cx: float = 319.5
    cy: float = 239.5
    camera_width: int = 640
    camera_height: int = 480
    max_cell_size: float = 0.0
    mode: str = "compat"          # "compat" (reference arithmetic and quirks) or "fixed"
    arith: str = "reference"      # compat only: "reference" (fast-math division) or "ieee"
    truncation: float = 0.0       # <= 0: 1.1 * |voxel size|
    max_depth: float = 0.0        # <= 0: 24 m
    min_z: float = 0.0
    memory: str = "device"        # "device" or "managed"

    def to_c(self):
        c = L.VolumeCfg()
        for i in range(3):
            c.voxel_grid_size[i] = int(self.voxel_grid_size[i])
            c.physical_size[i] = float(self.physical_size[i])
            c.global_offset[i] = float(self.global_offset[i])
        c.max_weight = float(self.max_weight)
        c.focal_x, c.focal_y = float(self.focal_x), float(self.focal_y)
        c.cx, c.cy = float(self.cx), float(self.cy)
        c.camera_width, c.camera_height = int(self.camera_width), int(self.camera_height)
        c.max_cell_size = float(self.max_cell_size)
        c.mode = {"compat": L.MODE_COMPAT, "fixed": L.MODE_FIXED}[self.mode]
        c.arith = {"reference": L.ARITH_REFERENCE, "ieee": L.ARITH_IEEE}[self.arith]
        c.truncation = float(self.truncation)
        c.max_depth = float(self.max_depth)
        c.min_z = float(self.min_z)
        c.memory = {"device": L.MEMORY_DEVICE, "managed": L.MEMORY_MANAGED}[self.memory]
        return c

    @classmethod
    def from_c(cls, c):
        return cls(voxel_grid_size=tuple(int(x) for x in c.voxel_grid_size),
                   physical_size=tuple(float(x) for x in c.physical_size),
                   global_offset=tuple(float(x) for x in c.global_offset), max_weight=float(c.max_weight),
                   focal_x=float(c.focal_x), focal_y=float(c.focal_y), cx=float(c.cx), cy=float(c.cy),
                   camera_width=int(c.camera_width), camera_height=int(c.camera_height),
                   max_cell_size=float(c.max_cell_size),
                   mode={L.MODE_COMPAT: "compat", L.MODE_FIXED: "fixed"}[c.mode],
                   arith={L.ARITH_REFERENCE: "reference", L.ARITH_IEEE: "ieee"}[c.arith],
                   truncation=float(c.truncation), max_depth=float(c.max_depth), min_z=float(c.min_z),
                   memory={L.MEMORY_DEVICE: "device", L.MEMORY_MANAGED: "managed"}[c.memory])


class _DeviceArray:
    """Zero-copy wrapper of a device pointer for torch.as_tensor."""

    def __init__(self, ptr, shape, typestr, owner):
        self.__cuda_array_interface__ = {"shape": tuple(shape), "typestr": typestr, "data": (int(ptr), False),
                                         "version": 3, "strides": None}
        self._owner = owner


def _stream_handle(stream):
    torch = _torch()
    if stream is None:
        stream = torch.cuda.current_stream()
    return C.c_void_p(stream.cuda_stream)


def _log_error(msg):
    sys.stderr.write("[gbt] " + msg + "\n")


def make_frame(depth, pose, depth_scale=0.001):
    """A gbt_frame for a CUDA depth tensor (H, W) of float32 metres or uint16."""
    torch = _torch()
    L.device_image(depth, "depth", (torch.float32, torch.uint16, torch.int16))
    f = L.Frame()
    f.depth = depth.data_ptr()
    f.height, f.width = int(depth.shape[0]), int(depth.shape[1])
    f.pitch_bytes = int(depth.stride(0) * depth.element_size())
    f.format = L.DEPTH_F32_M if depth.dtype == torch.float32 else L.DEPTH_U16
    f.depth_scale = float(depth_scale)
    for k in range(7):
        f.pose[k] = float(pose[k])
    return f


class TSDFVolume:
    """cuphoto::TSDFVolume on the engine (tsdf_volume.cuh:31-105)."""

    def __init__(self, cfg: TSDFVolumeConfig, stream=None, _handle=None):
        self.cfg = cfg
        self._lib = L.lib()
        self._h = C.c_void_p()
        if _handle is not None:
            self._h = _handle
        else:
            L.check(self._lib.gbt_volume_create(C.byref(cfg.to_c()), _stream_handle(stream), C.byref(self._h)))
        self._info = L.VolumeInfo()
        L.check(self._lib.gbt_volume_get_info(self._h, C.byref(self._info)))

    # -- checkpoint and resume (gbt_volume_save / gbt_volume_load) -------------
    def save(self, path, stream=None):
        """Writes the configuration and the distance and weight grids to `path`
        (waits for `stream`)."""
        L.check(self._lib.gbt_volume_save(self._h, os.fsencode(path), _stream_handle(stream)))

    @classmethod
    def load(cls, path, stream=None):
        """A volume created from a file written by save(); integrating more
        frames into it continues the saved volume exactly."""
        lib = L.lib()
        h = C.c_void_p()
        L.check(lib.gbt_volume_load(os.fsencode(path), _stream_handle(stream), C.byref(h)))
        c = L.VolumeCfg()
        L.check(lib.gbt_volume_get_cfg(h, C.byref(c)))
        return cls(TSDFVolumeConfig.from_c(c), _handle=h)

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            self._lib.gbt_volume_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    # -- reference accessors -------------------------------------------------
    def voxel_grid_size(self):
        return tuple(self._info.voxel_grid_size)

    def global_offset(self):
        return tuple(self._info.global_offset)

    def scale_voxel_size(self):
        return tuple(self._info.voxel_size)

    def voxel_phys_size(self):
        return tuple(self._info.physical_size)

    @property
    def truncation(self):
        return self._info.truncation

    def _view(self, ptr):
        torch = _torch()
        nx, ny, nz = self.voxel_grid_size()
        return torch.as_tensor(_DeviceArray(ptr, (nz, ny, nx), "<f4", self), device="cuda")

    def voxel_distances_data(self):
        """Distance grid as a (z, y, x) float32 CUDA tensor sharing the volume's memory."""
        return self._view(self._info.tsdf)

    def voxel_weights_data(self):
        return self._view(self._info.weights)

    def transformation_voxels_data(self, stream=None):
        """Packed 28-byte {float3 centre, float4 quaternion} records, materialised on first use."""
        torch = _torch()
        p = C.c_void_p()
        L.check(self._lib.gbt_volume_transformation_voxels(self._h, _stream_handle(stream), C.byref(p)))
        n = self._info.num_voxels
        return torch.as_tensor(_DeviceArray(p.value, (n, 7), "<f4", self), device="cuda")

    def reset(self, stream=None):
        L.check(self._lib.gbt_volume_reset(self._h, _stream_handle(stream)))

    def check(self, stream=None):
        """Synchronises and raises GbtError (GBT_ERR_TIMEOUT) if a kernel gave up
        a bounded wait while working on this volume (its contents are then
        undefined until reset); the mark is cleared."""
        L.check(self._lib.gbt_volume_check(self._h, _stream_handle(stream)))

    # -- integrate -----------------------------------------------------------
    def integrate(self, color, depth, camera_pose, depth_scale=0.001, stream=None):
        """TSDFVolume::integrate(color, depth, pose) (tsdf_volume.cu:257-290).

        color is checked (non-empty) but not read, as in the reference.
        camera_pose = (qw, qx, qy, qz, tx, ty, tz), world to camera.
        Returns False (after logging) when an image is missing or empty.
        Unlike the reference the call does not synchronise the device."""
        if depth is None or color is None:
            _log_error("TSDFVolume::integrate() -- depth or color map is null pointer")
            return False
        if depth.numel() == 0 or color.numel() == 0:
            _log_error("TSDFVolume::integrate() -- depth width/height parameters are zero")
            return False
        f = make_frame(depth, camera_pose, depth_scale)
        st = self._lib.gbt_integrate(self._h, C.byref(f), 1, _stream_handle(stream))
        if st == L.GBT_ERR_INVALID_ARG:
            _log_error("TSDFVolume::integrate() -- " + self._lib.gbt_last_error().decode())
            return False
        L.check(st)
        return True

    def integrate_frames(self, depths, poses, depth_scale=0.001, brick=0, ctas_per_sm=0, stream=None):
        """Integrates up to 32 frames in one pass over the volume (frames applied in order).
        brick: the tile shape of gbt_integrate_tuned (0..7), or 8 for bricks
        streamed into shared memory by the Tensor Memory Accelerator (passes
        of up to 16 frames, x extent a multiple of 4); results are the same."""
        n = len(depths)
        arr = (L.Frame * n)()
        for i in range(n):
            arr[i] = make_frame(depths[i], poses[i], depth_scale)
        L.check(self._lib.gbt_integrate_tuned(self._h, arr, n, int(brick), int(ctas_per_sm), _stream_handle(stream)))

    def integrate_sequence(self, depths, poses, frames_per_pass=16, depth_scale=0.001, stream=None, **kw):
        """Integrates any number of frames, frames_per_pass at a time."""
        for s in range(0, len(depths), frames_per_pass):
            self.integrate_frames(depths[s:s + frames_per_pass], poses[s:s + frames_per_pass],
                                  depth_scale=depth_scale, stream=stream, **kw)


def extract_mesh_indexed(volume, normals=True, index_base=0, stream=None):
    """Fixed-mode mesh with shared vertices (gbt_extract_mesh_indexed):
    (verts (V, 3) f32, normals (V, 3) f32 or None, tris (T, 3) i32) CUDA
    tensors; the triangles are extract_mesh_device's, in the same order."""
    torch = _torch()
    lib = L.lib()
    s = _stream_handle(stream)
    nv, nt = C.c_int64(), C.c_int64()
    L.check(lib.gbt_extract_mesh_indexed(volume.handle, None, None, None, 0, 0, index_base, C.byref(nv), C.byref(nt), s))
    V = torch.empty((max(nv.value, 1), 3), dtype=torch.float32, device="cuda")
    N = torch.empty((max(nv.value, 1), 3), dtype=torch.float32, device="cuda") if normals else None
    T = torch.empty((max(nt.value, 1), 3), dtype=torch.int32, device="cuda")
    L.check(lib.gbt_extract_mesh_indexed(volume.handle, C.c_void_p(V.data_ptr()),
                                         C.c_void_p(N.data_ptr()) if normals else None, C.c_void_p(T.data_ptr()),
                                         nv.value, nt.value, index_base, C.byref(nv), C.byref(nt), s))
    return V[:nv.value], (N[:nv.value] if normals else None), T[:nt.value]


def extract_mesh_device(volume, capacity=None, index_base=0, stream=None):
    """Runs the engine's marching cubes; returns (verts (T,3,3) f32, tris (T,3) i32) CUDA tensors."""
    torch = _torch()
    lib = L.lib()
    s = _stream_handle(stream)
    n = C.c_int64()
    if capacity is None:
        L.check(lib.gbt_extract_mesh(volume.handle, None, None, 0, index_base, C.byref(n), s))
        capacity = n.value
    verts = torch.empty((max(capacity, 1), 3, 3), dtype=torch.float32, device="cuda")
    tris = torch.empty((max(capacity, 1), 3), dtype=torch.int32, device="cuda")
    st = lib.gbt_extract_mesh(volume.handle, C.c_void_p(verts.data_ptr()), C.c_void_p(tris.data_ptr()),
                              int(capacity), int(index_base), C.byref(n), s)
    if st == L.GBT_ERR_CAPACITY:
        return extract_mesh_device(volume, n.value, index_base, stream)
    L.check(st)
    return verts[:n.value], tris[:n.value]


def generate_triangular_surface(volume, vertices=None, triangles=None, stream=None):
    """generate_triangular_surface (marching_cubes.cu:191-237).

    Appends to `vertices` (list of (x, y, z)) / `triangles` (list of (i, j, k))
    when given, with triangle indices offset by the vertices already present,
    as the reference's std::vector outputs do.  Returns numpy arrays
    (vertices (3T, 3) float32, triangles (T, 3) int32) of this call's output."""
    base = len(vertices) if vertices is not None else 0
    v, t = extract_mesh_device(volume, index_base=base, stream=stream)
    v = v.reshape(-1, 3).cpu().numpy()
    t = t.cpu().numpy()
    if vertices is not None:
        vertices.extend(map(tuple, v))
    if triangles is not None:
        triangles.extend(map(tuple, t))
    return v, t
