"""cudaPointCloud (cuda_point_cloud.cuh:13-103, cuda_point_cloud.cu) on the engine.

A cloud keeps its points in a CUDA uint8 tensor of shape (capacity, 33), the
reference's packed Vertex layout (float pos[3], float normal[4], uint8
color[3], uint16 classID), and a count.  The per-point work runs in the
engine's kernels through the C ABI (gbt_points_*): back-projection, rigid
transform, and the z-buffer projection that the reference runs as a host
loop.  Methods keep the reference's names, argument meaning and bool + log
error behaviour, including its quirks:

* camera_matrix is read as m[0], m[4], m[6], m[7] (fx, fy, cx, cy) when
  back-projecting and as m[0], m[4], m[2], m[5] when projecting
  (cuda_point_cloud.cu:44-47 vs :248-251);
* extract_points writes frame frame_idx at points [frame_idx*W*H, ...) and
  counts all W*H of them, leaving the slots of pixels without depth as they
  were (zero in a fresh cloud);
* filter_depth keeps the points whose z is outside (min, max)
  (cuda_point_cloud.cu:409-435).
"""
import ctypes as C
import sys

import numpy as np

from . import _lib as L
from .tsdf import _stream_handle, _torch

POINT_DTYPE = np.dtype([("pos", "<f4", 3), ("normal", "<f4", 4), ("color", "u1", 3), ("class_id", "<u2")])
assert POINT_DTYPE.itemsize == L.POINT_BYTES
FLT_MIN = float(np.finfo(np.float32).tiny)
FLT_MAX = float(np.finfo(np.float32).max)


def _log(msg):
    sys.stderr.write("[cuphoto] " + msg + "\n")


def _k9(m):
    a = (C.c_double * 9)(*[float(x) for x in m])
    return a


def _pose7(p):
    return (C.c_double * 7)(*[float(x) for x in p])


class PointCloud:
    """cuphoto::cudaPointCloud."""

    def __init__(self, camera_mat, total_number_pts):
        torch = _torch()
        self.camera_matrix = [float(x) for x in camera_mat]
        if len(self.camera_matrix) != 9:
            raise ValueError("camera matrix needs 9 values")
        self.total_num_pts = int(total_number_pts)
        self.num_pts = 0
        self.has_rgb = False
        self.device_pts = torch.zeros((max(self.total_num_pts, 0), L.POINT_BYTES), dtype=torch.uint8, device="cuda")

    @staticmethod
    def create(camera_mat, total_number_pts):
        return PointCloud(camera_mat, total_number_pts)

    @staticmethod
    def merge(pc1, pc2):
        pc = PointCloud(pc1.camera_matrix, pc1.num_pts + pc2.num_pts)
        pc.device_pts[:pc1.num_pts] = pc1.device_pts[:pc1.num_pts]
        pc.device_pts[pc1.num_pts:] = pc2.device_pts[:pc2.num_pts]
        pc.set_total_number_pts()
        return pc

    # -- accessors --------------------------------------------------------------
    def get_total_num_points(self):
        return self.total_num_pts

    def get_num_points(self):
        return self.num_pts

    def get_size(self):
        return self.num_pts * L.POINT_BYTES

    def get_points(self):
        """(num_points, 33) uint8 CUDA tensor of the packed vertices."""
        return self.device_pts[:self.num_pts]

    def get_camera_parameters(self):
        return list(self.camera_matrix)

    def set_total_number_pts(self):
        self.num_pts = self.total_num_pts

    def to_numpy(self):
        """The points as a structured array (fields pos, normal, color, class_id)."""
        return self.get_points().cpu().numpy().reshape(-1).view(POINT_DTYPE)

    # -- kernels ----------------------------------------------------------------
    def extract_points(self, depth, colors, transform, frame_idx, depth_scale=0.001, stream=None):
        """cudaPointCloud::extract_points (cuda_point_cloud.cu:179-226): depth (H, W)
        float32 metres or uint16; colors (H, W, 3) uint8 or None; transform
        {qw,qx,qy,qz,tx,ty,tz}."""
        torch = _torch()
        if depth is None:
            _log("cudaPointCloud::extract_points() -- depth map is null pointer")
            return False
        if depth.numel() == 0:
            _log("cudaPointCloud::extract_points() -- depth width/height parameters are zero")
            return False
        L.device_image(depth, "depth", (torch.float32, torch.uint16, torch.int16))
        H, W = int(depth.shape[0]), int(depth.shape[1])
        fmt = L.DEPTH_U16 if depth.dtype in (torch.uint16, torch.int16) else L.DEPTH_F32_M
        cptr, cpitch = None, 0
        if colors is not None:
            L.device_image(colors, "colors", (torch.uint8,), channels=3)
            if tuple(colors.shape[:2]) != (H, W):
                raise ValueError("colors are %dx%d, depth %dx%d" % (colors.shape[1], colors.shape[0], W, H))
            self.has_rgb = True
            cptr, cpitch = C.c_void_p(colors.data_ptr()), int(colors.stride(0) * colors.element_size())
        start = int(frame_idx) * W * H
        st = L.lib().gbt_points_extract(C.byref(_k9(self.camera_matrix)), C.c_void_p(depth.data_ptr()),
                                        int(depth.stride(0) * depth.element_size()), fmt, float(depth_scale), cptr,
                                        cpitch, W, H, C.byref(_pose7(transform)), start,
                                        C.c_void_p(self.device_pts.data_ptr()), self.total_num_pts,
                                        _stream_handle(stream))
        if st != L.GBT_OK:
            _log("cudaPointCloud::extract_points() -- " + L.lib().gbt_last_error().decode())
            return False
        self.num_pts += W * H
        return True

    def _project(self, color, depth, camera_pose, stream):
        torch = _torch()
        L.device_image(depth, "depth", (torch.float32,))
        H, W = int(depth.shape[0]), int(depth.shape[1])
        scratch = torch.empty(H * W, dtype=torch.int64, device="cuda")
        cptr, cpitch = None, 0
        if color is not None:
            L.device_image(color, "color", (torch.uint8,), channels=3)
            if tuple(color.shape[:2]) != (H, W):
                raise ValueError("color is %dx%d, depth %dx%d" % (color.shape[1], color.shape[0], W, H))
            cptr, cpitch = C.c_void_p(color.data_ptr()), int(color.stride(0) * color.element_size())
        n = self.num_pts
        st = L.lib().gbt_points_project(C.c_void_p(self.device_pts.data_ptr()) if n else None, n,
                                        C.byref(_k9(self.camera_matrix)), C.byref(_pose7(camera_pose)),
                                        C.c_void_p(depth.data_ptr()), int(depth.stride(0) * 4), cptr, cpitch, W, H,
                                        C.c_void_p(scratch.data_ptr()), _stream_handle(stream))
        if st != L.GBT_OK:
            _log("cudaPointCloud::project_to_depth() -- " + L.lib().gbt_last_error().decode())
            return False
        return True

    def project_to_depth(self, depth, camera_pose, stream=None):
        """cudaPointCloud::project_to_depth (cuda_point_cloud.cu:229-288): depth (H, W) float32."""
        if depth is None:
            _log("cudaPointCloud::project_to_depth() -- depth map is null pointer")
            return False
        if depth.numel() == 0:
            _log("cudaPointCloud::project_to_depth() -- depth width/height parameters are zero")
            return False
        return self._project(None, depth, camera_pose, stream)

    def project_to_color_depth(self, color, depth, camera_pose, stream=None):
        """cudaPointCloud::project_to_color_depth (cuda_point_cloud.cu:292-353):
        color (H, W, 3) uint8, depth (H, W) float32."""
        if depth is None or color is None:
            _log("cudaPointCloud::project_to_depth() -- depth or color map is null pointer")
            return False
        if depth.numel() == 0:
            _log("cudaPointCloud::project_to_depth() -- depth width/height parameters are zero")
            return False
        return self._project(color, depth, camera_pose, stream)

    def transform(self, T, stream=None):
        """cudaPointCloud::transform (cuda_point_cloud.cu:356-385)."""
        if self.num_pts == 0:
            _log("cudaPointCloud::transform() -- the number of points is 0")
            return False
        st = L.lib().gbt_points_transform(C.c_void_p(self.device_pts.data_ptr()), self.num_pts,
                                          C.byref(_pose7(T)), _stream_handle(stream))
        if st != L.GBT_OK:
            _log("cudaPointCloud::transform() -- " + L.lib().gbt_last_error().decode())
            return False
        return True

    # -- host-side edits ------------------------------------------------------------
    def add_vertex(self, pos, color, idx, normal=(0.0, 0.0, 0.0, 0.0)):
        """cudaPointCloud::add_vertex (cuda_point_cloud.cu:389-407)."""
        torch = _torch()
        if idx >= self.total_num_pts:
            _log("cudaPointCloud::add_vertex() -- index out of range")
            return False
        rec = np.zeros(1, POINT_DTYPE)
        rec["pos"] = pos
        rec["normal"] = normal
        rec["color"] = color
        self.device_pts[idx] = torch.from_numpy(rec.view(np.uint8).copy()).cuda()
        return True

    def filter_depth(self, depth_threshold_min=FLT_MIN, depth_threshold_max=FLT_MAX):
        """cudaPointCloud::filter_depth (cuda_point_cloud.cu:409-435): keeps the
        points with z <= min or z >= max, as the reference does."""
        pts = self.get_points()
        z = pts[:, 8:12].contiguous().view(_torch().float32).reshape(-1)
        keep = (z <= np.float32(depth_threshold_min)) | (z >= np.float32(depth_threshold_max))
        kept = pts[keep].clone()
        self.device_pts = kept
        self.num_pts = int(kept.shape[0])

    def add_point_cloud(self, other):
        """cudaPointCloud::add_point_cloud (cuda_point_cloud.cu:438-456)."""
        torch = _torch()
        self.device_pts = torch.cat([self.get_points(), other.get_points()]).contiguous()
        self.num_pts = int(self.device_pts.shape[0])
        self.total_num_pts = self.num_pts
        return True

    def clear(self):
        self.device_pts[:self.num_pts].zero_()
        self.num_pts = 0

    def free(self):
        self.device_pts = _torch().zeros((0, L.POINT_BYTES), dtype=_torch().uint8, device="cuda")
        self.num_pts = 0

    def save_ply(self, filepath):
        """cudaPointCloud::save_ply (cuda_point_cloud.cu:459-495): ASCII, y and z
        negated, colour as 0..255 integers."""
        if not filepath:
            _log("cudaPointCloud::save_ply() -- empty file path for store point cloud")
            return False
        if self.num_pts <= 0:
            _log("cudaPointCloud::save_ply() -- can't store, point cloud is empty")
            return False
        v = self.to_numpy()
        with open(filepath, "w") as f:
            f.write("ply\nformat ascii 1.0\nelement vertex %d\nproperty float x\nproperty float y\n"
                    "property float z\nproperty uchar red\nproperty uchar green\nproperty uchar blue\n"
                    "end_header\n" % self.num_pts)
            for p, c in zip(v["pos"], v["color"]):
                f.write("%g %g %g %d %d %d\n" % (p[0], p[1] * np.float32(-1), p[2] * np.float32(-1), c[0], c[1], c[2]))
        return True
