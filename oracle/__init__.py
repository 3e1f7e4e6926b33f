"""Python access to the CPU oracle and to the reference's own kernels.

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py as the checker.  The engine never imports it.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "_build", "liboracle.so")
HARNESS_SO = os.path.join(HERE, "_build", "libref_harness.so")
REF_CUBIN = os.path.join(HERE, "_ref", "ref_tsdf.cubin")
REF_NAMES = os.path.join(HERE, "_ref", "ref_kernels.txt")


class OracleCfg(C.Structure):
    _fields_ = [
        ("grid", C.c_int32 * 3),
        ("phys", C.c_float * 3),
        ("offset", C.c_float * 3),
        ("fx", C.c_float), ("fy", C.c_float), ("cx", C.c_float), ("cy", C.c_float),
        ("max_weight", C.c_float),
        ("truncation", C.c_float),
        ("max_depth", C.c_float),
        ("min_z", C.c_float),
    ]


_so = None


def ensure_built():
    """Builds the oracle (and the reference kernels where possible) if stale."""
    import importlib
    return importlib.import_module(__name__ + ".build").build_all()


def lib():
    global _so
    if _so is None:
        if not os.path.exists(ORACLE_SO):
            ensure_built()
        so = C.CDLL(ORACLE_SO)
        f, d, i32, i64, vp = C.c_float, C.c_double, C.c_int32, C.c_int64, C.c_void_p
        P = C.POINTER
        so.oracle_derive.argtypes = [P(OracleCfg), vp, vp]
        so.oracle_volume_init.argtypes = [P(OracleCfg), vp, vp]
        so.oracle_integrate_compat.argtypes = [P(OracleCfg), vp, vp, vp, i64, i32, i32, vp, i32]
        so.oracle_compat_ambiguous.argtypes = [P(OracleCfg), vp, i32, i32, f, vp, i32]
        so.oracle_integrate_fixed.argtypes = [P(OracleCfg), vp, vp, vp, i64, i32, i32, i32, f, vp, i32]
        so.oracle_mc_compat.argtypes = [P(OracleCfg), vp, vp, vp, i64, i64, i32]
        so.oracle_mc_compat.restype = i64
        so.oracle_mc_fixed.argtypes = [P(OracleCfg), vp, vp, vp, vp, i64, i64, i32]
        so.oracle_mc_fixed.restype = i64
        _so = so
    return _so


def cfg_from(tc):
    """OracleCfg from a cuphoto.TSDFVolumeConfig (or any object with its fields)."""
    c = OracleCfg()
    for i in range(3):
        c.grid[i] = int(tc.voxel_grid_size[i])
        c.phys[i] = float(tc.physical_size[i])
        c.offset[i] = float(tc.global_offset[i])
    c.fx, c.fy, c.cx, c.cy = float(tc.focal_x), float(tc.focal_y), float(tc.cx), float(tc.cy)
    c.max_weight = float(tc.max_weight)
    c.truncation = float(getattr(tc, "truncation", 0.0))
    c.max_depth = float(getattr(tc, "max_depth", 0.0))
    c.min_z = float(getattr(tc, "min_z", 0.0))
    return c


def _p(a):
    return C.c_void_p(a.ctypes.data)


def derive(cfg):
    vs = np.zeros(3, np.float32)
    tr = np.zeros(1, np.float32)
    lib().oracle_derive(C.byref(cfg), _p(vs), _p(tr))
    return vs, float(tr[0])


def init_volume(cfg):
    n = cfg.grid[0] * cfg.grid[1] * cfg.grid[2]
    D = np.empty(n, np.float32)
    W = np.empty(n, np.float32)
    lib().oracle_volume_init(C.byref(cfg), _p(D), _p(W))
    shape = (cfg.grid[2], cfg.grid[1], cfg.grid[0])
    return D.reshape(shape), W.reshape(shape)


def _pose(pose):
    return np.ascontiguousarray(pose, np.float64)


def integrate_compat(cfg, D, W, depth_m, pose, threads=0):
    depth_m = np.ascontiguousarray(depth_m, np.float32)
    p = _pose(pose)
    lib().oracle_integrate_compat(C.byref(cfg), _p(D), _p(W), _p(depth_m), depth_m.strides[0],
                                  depth_m.shape[1], depth_m.shape[0], _p(p), threads)


def compat_ambiguous(cfg, pose, width, height, ulps=8.0, flags=None, threads=0):
    n = cfg.grid[0] * cfg.grid[1] * cfg.grid[2]
    if flags is None:
        flags = np.zeros((cfg.grid[2], cfg.grid[1], cfg.grid[0]), np.uint8)
    p = _pose(pose)
    lib().oracle_compat_ambiguous(C.byref(cfg), _p(p), width, height, float(ulps), _p(flags), threads)
    return flags


def integrate_fixed(cfg, D, W, depth, pose, depth_scale=0.001, threads=0):
    depth = np.ascontiguousarray(depth)
    fmt = 1 if depth.dtype in (np.uint16, np.int16) else 0
    if fmt == 0:
        depth = depth.astype(np.float32, copy=False)
    p = _pose(pose)
    lib().oracle_integrate_fixed(C.byref(cfg), _p(D), _p(W), _p(depth), depth.strides[0], depth.shape[1],
                                 depth.shape[0], fmt, float(depth_scale), _p(p), threads)


def mc_compat(cfg, D, index_base=0, threads=0):
    n = lib().oracle_mc_compat(C.byref(cfg), _p(D), None, None, 0, index_base, threads)
    V = np.empty((max(n, 1), 3, 3), np.float32)
    T = np.empty((max(n, 1), 3), np.int32)
    lib().oracle_mc_compat(C.byref(cfg), _p(D), _p(V), _p(T), n, index_base, threads)
    return V[:n], T[:n]


def mc_fixed(cfg, D, W, index_base=0, threads=0):
    n = lib().oracle_mc_fixed(C.byref(cfg), _p(D), _p(W), None, None, 0, index_base, threads)
    V = np.empty((max(n, 1), 3, 3), np.float32)
    T = np.empty((max(n, 1), 3), np.int32)
    lib().oracle_mc_fixed(C.byref(cfg), _p(D), _p(W), _p(V), _p(T), n, index_base, threads)
    return V[:n], T[:n]


# ---------------------------------------------------------------------------
# Differentiable integrate

class OracleDiffCfg(C.Structure):
    _fields_ = [
        ("grid", C.c_uint32 * 3),
        ("vs", C.c_float * 3),
        ("off", C.c_float * 3),
        ("fx", C.c_float), ("fy", C.c_float), ("cx", C.c_float), ("cy", C.c_float),
        ("trunc", C.c_float), ("max_weight", C.c_float), ("max_depth", C.c_float), ("min_z", C.c_float),
        ("width", C.c_int32), ("height", C.c_int32),
        ("dtype", C.c_int32),
    ]


def diff_cfg(grid, vs, off, K, trunc, max_weight, max_depth, min_z, width, height, dtype):
    c = OracleDiffCfg()
    for i in range(3):
        c.grid[i], c.vs[i], c.off[i] = int(grid[i]), float(vs[i]), float(off[i])
    c.fx, c.fy, c.cx, c.cy = (float(k) for k in K)
    c.trunc, c.max_weight, c.max_depth, c.min_z = float(trunc), float(max_weight), float(max_depth), float(min_z)
    c.width, c.height, c.dtype = int(width), int(height), int(dtype)
    return c


def _diff_lib():
    so = lib()
    if not getattr(so, "_diff_ready", False):
        vp = C.c_void_p
        so.oracle_diff_forward.argtypes = [C.POINTER(OracleDiffCfg), vp, vp, vp, vp, C.c_int32, vp, vp, C.c_int32]
        so.oracle_diff_backward.argtypes = [C.POINTER(OracleDiffCfg), vp, vp, vp, vp, vp, C.c_int32, vp, vp, vp, vp,
                                            vp, vp]
        so._diff_ready = True
    return so


def diff_forward(cfg, D, W, depth, rot, trans, threads=0):
    """In place on D, W (float32 or float64 per cfg.dtype); returns the signature."""
    sig = np.zeros(D.size, np.uint32)
    depth = np.ascontiguousarray(depth)
    rot = np.ascontiguousarray(rot)
    trans = np.ascontiguousarray(trans)
    _diff_lib().oracle_diff_forward(C.byref(cfg), _p(D), _p(W), _p(sig), _p(depth), len(depth), _p(rot), _p(trans),
                                    threads)
    return sig.reshape(D.shape)


def diff_backward(cfg, grad_D, grad_W, D0, W0, depth, rot, trans):
    """float64 reverse mode: (grad_depth [F,H,W], grad_pose [F,12], grad_D0, grad_W0)."""
    f64 = lambda a: np.ascontiguousarray(a, np.float64)
    depth = f64(depth)
    gdep = np.zeros(depth.shape, np.float64)
    gpose = np.zeros((len(depth), 12), np.float64)
    gD0 = np.zeros(np.shape(D0), np.float64)
    gW0 = np.zeros(np.shape(D0), np.float64)
    gW = None if grad_W is None else f64(grad_W)
    _diff_lib().oracle_diff_backward(C.byref(cfg), _p(f64(grad_D)), None if gW is None else _p(gW), _p(f64(D0)),
                                     _p(f64(W0)), _p(depth), len(depth), _p(f64(rot)), _p(f64(trans)), _p(gdep),
                                     _p(gpose), _p(gD0), _p(gW0))
    return gdep, gpose, gD0, gW0


# ---------------------------------------------------------------------------
# Point clouds (cuda_point_cloud.cu).  A cloud is an (n, 33) uint8 array of
# the reference's packed vertices; POINT_DTYPE views it field by field.
POINT_DTYPE = np.dtype([("pos", "<f4", 3), ("normal", "<f4", 4), ("color", "u1", 3), ("class_id", "<u2")])
assert POINT_DTYPE.itemsize == 33


def _points_lib():
    so = lib()
    if not getattr(so, "_points_ready", False):
        vp = C.c_void_p
        so.oracle_points_extract.argtypes = [vp, vp, vp, C.c_int32, C.c_int32, vp, C.c_int64, vp]
        so.oracle_points_transform.argtypes = [vp, C.c_int64, vp]
        so.oracle_points_project.argtypes = [vp, C.c_int64, vp, vp, C.c_int32, C.c_int32, vp, vp]
        so.oracle_filter_if.argtypes = [vp, C.c_int64, C.c_float, C.c_float]
        so._points_ready = True
    return so


def points_extract(K9, depth, rgb, pose, points, start=0):
    """In place on points ((n, 33) uint8): the pixels with depth > 0."""
    depth = np.ascontiguousarray(depth, np.float32)
    H, W = depth.shape
    K9 = np.ascontiguousarray(K9, np.float64)
    pose = np.ascontiguousarray(pose, np.float64)
    rgb = None if rgb is None else np.ascontiguousarray(rgb, np.uint8)
    assert points.dtype == np.uint8 and points.flags.c_contiguous and points.size >= (start + W * H) * 33
    _points_lib().oracle_points_extract(_p(K9), _p(depth), None if rgb is None else _p(rgb), W, H, _p(pose),
                                        start, _p(points))
    return points


def points_transform(points, pose):
    pose = np.ascontiguousarray(pose, np.float64)
    _points_lib().oracle_points_transform(_p(points), points.size // 33, _p(pose))
    return points


def points_project(points, K9, pose, W, H, color=True):
    """(depth (H, W) float32, rgb (H, W, 3) uint8 or None)."""
    K9 = np.ascontiguousarray(K9, np.float64)
    pose = np.ascontiguousarray(pose, np.float64)
    depth = np.empty((H, W), np.float32)
    rgb = np.empty((H, W, 3), np.uint8) if color else None
    _points_lib().oracle_points_project(_p(points), points.size // 33, _p(K9), _p(pose), W, H, _p(depth),
                                        None if rgb is None else _p(rgb))
    return depth, rgb


def filter_if(img, filter_value, set_value):
    img = np.ascontiguousarray(img, np.float32).copy()
    _points_lib().oracle_filter_if(_p(img), img.size, filter_value, set_value)
    return img


# ---------------------------------------------------------------------------
class RefHarness:
    """The reference's own kernels (compiled from its sources) driven with its
    host-side logic.  Needs a GPU and oracle/_ref/ref_tsdf.cubin."""

    _so = None

    @classmethod
    def available(cls):
        return os.path.exists(REF_CUBIN) and os.path.exists(REF_NAMES) and os.path.exists(HARNESS_SO)

    @classmethod
    def lib(cls):
        if cls._so is None:
            so = C.CDLL(HARNESS_SO)
            vp, i32, i64, f = C.c_void_p, C.c_int32, C.c_int64, C.c_float
            so.ref_last_error.restype = C.c_char_p
            so.ref_load.argtypes = [C.c_char_p, C.c_char_p]
            so.ref_volume_create.argtypes = [vp, vp, vp, f, f, f, f, f, C.POINTER(vp)]
            so.ref_volume_destroy.argtypes = [vp]
            so.ref_truncation.argtypes = [vp]
            so.ref_truncation.restype = f
            so.ref_integrate.argtypes = [vp, vp, C.c_size_t, i32, i32, vp, C.POINTER(f)]
            so.ref_read_volume.argtypes = [vp, vp, vp]
            so.ref_write_distances.argtypes = [vp, vp]
            so.ref_extract.argtypes = [vp, vp, vp, i64, C.POINTER(f)]
            so.ref_extract.restype = i64
            so.ref_points_extract.argtypes = [vp, vp, C.c_size_t, i32, i32, vp, C.c_size_t, vp, i64, vp]
            so.ref_points_transform.argtypes = [vp, C.c_uint32, vp]
            so.ref_filter_if.argtypes = [vp, C.c_size_t, i32, i32, f, f]
            if so.ref_load(REF_CUBIN.encode(), REF_NAMES.encode()) != 0:
                raise RuntimeError("reference kernels: " + so.ref_last_error().decode())
            cls._so = so
        return cls._so

    def __init__(self, tc):
        so = self.lib()
        self.grid = np.array(tc.voxel_grid_size, np.uint32)
        phys = np.array(tc.physical_size, np.float32)
        off = np.array(tc.global_offset, np.float32)
        self.h = C.c_void_p()
        if so.ref_volume_create(_p(self.grid), _p(phys), _p(off), float(tc.max_weight), float(tc.focal_x),
                                float(tc.focal_y), float(tc.cx), float(tc.cy), C.byref(self.h)) != 0:
            raise RuntimeError("reference volume: " + so.ref_last_error().decode())

    def close(self):
        if self.h and self.h.value:
            self.lib().ref_volume_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def truncation(self):
        return self.lib().ref_truncation(self.h)

    # -- the reference's point-cloud kernels (device pointers in and out) -----
    @classmethod
    def points_extract(cls, K9, depth_ptr, pitch, width, height, color_ptr, color_pitch, pose, start, points_ptr):
        K9 = np.ascontiguousarray(K9, np.float64)
        p = np.ascontiguousarray(pose, np.float64)
        if cls.lib().ref_points_extract(_p(K9), C.c_void_p(depth_ptr), pitch, width, height,
                                        C.c_void_p(color_ptr) if color_ptr else None, color_pitch, _p(p), start,
                                        C.c_void_p(points_ptr)) != 0:
            raise RuntimeError(cls.lib().ref_last_error().decode())

    @classmethod
    def points_transform(cls, points_ptr, n, pose):
        p = np.ascontiguousarray(pose, np.float64)
        if cls.lib().ref_points_transform(C.c_void_p(points_ptr), n, _p(p)) != 0:
            raise RuntimeError(cls.lib().ref_last_error().decode())

    @classmethod
    def filter_if(cls, img_ptr, pitch, width, height, filter_value, set_value):
        if cls.lib().ref_filter_if(C.c_void_p(img_ptr), pitch, width, height, filter_value, set_value) != 0:
            raise RuntimeError(cls.lib().ref_last_error().decode())

    def integrate(self, depth_ptr, pitch, width, height, pose):
        """depth_ptr: device float32 metres.  Returns the kernel time in ms."""
        p = _pose(pose)
        ms = C.c_float()
        if self.lib().ref_integrate(self.h, C.c_void_p(depth_ptr), pitch, width, height, _p(p), C.byref(ms)) != 0:
            raise RuntimeError(self.lib().ref_last_error().decode())
        return ms.value

    def read(self):
        n = int(np.prod(self.grid.astype(np.int64)))
        D = np.empty(n, np.float32)
        W = np.empty(n, np.float32)
        if self.lib().ref_read_volume(self.h, _p(D), _p(W)) != 0:
            raise RuntimeError(self.lib().ref_last_error().decode())
        shape = (int(self.grid[2]), int(self.grid[1]), int(self.grid[0]))
        return D.reshape(shape), W.reshape(shape)

    def write_distances(self, D):
        D = np.ascontiguousarray(D, np.float32)
        if self.lib().ref_write_distances(self.h, _p(D)) != 0:
            raise RuntimeError(self.lib().ref_last_error().decode())

    def extract(self, cap=None):
        so = self.lib()
        ms = C.c_float()
        if cap is None:
            cap = 0
        V = np.empty((max(cap, 1), 3, 3), np.float32)
        T = np.empty((max(cap, 1), 3), np.int32)
        n = so.ref_extract(self.h, _p(V), _p(T), cap, C.byref(ms))
        if n < 0:
            raise RuntimeError(so.ref_last_error().decode())
        if n > cap:
            return self.extract(int(n))
        return V[:n], T[:n], ms.value
