"""ctypes view of the engine's C ABI (include/gbt_tsdf.h).

The shared library is built in-tree by ``cu-reconstruction_gb300/build.py``
(``__graft_entry__.build()`` runs it).  There is no fallback: if the library
is missing, :func:`lib` raises.
"""
import ctypes as C
import os
import threading

PKG_ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_PATH = os.path.join(PKG_ROOT, "_build", "libgbt_tsdf.so")

GBT_OK = 0
GBT_ERR_INVALID_ARG = 1
GBT_ERR_CUDA = 2
GBT_ERR_ALLOC = 3
GBT_ERR_CAPACITY = 4
GBT_ERR_TIMEOUT = 5
GBT_ERR_IO = 6
VOLUME_FILE_MAGIC = b"GBTVOL\x00\x01"
VOLUME_FILE_HEADER_BYTES = 256

MODE_COMPAT = 0
MODE_FIXED = 1
ARITH_REFERENCE = 0
ARITH_IEEE = 1
DEPTH_F32_M = 0
DEPTH_U16 = 1
MEMORY_DEVICE = 0
MEMORY_MANAGED = 1
MAX_FRAMES_PER_PASS = 32
INJECT_NONE = 0
INJECT_ALLOC = 1
INJECT_LAUNCH_ERROR = 2
INJECT_HOLD_COPY = 3
BRICK_STREAMED = 8


class VolumeCfg(C.Structure):
    _fields_ = [
        ("voxel_grid_size", C.c_uint32 * 3),
        ("physical_size", C.c_float * 3),
        ("global_offset", C.c_float * 3),
        ("max_weight", C.c_float),
        ("focal_x", C.c_float), ("focal_y", C.c_float), ("cx", C.c_float), ("cy", C.c_float),
        ("camera_width", C.c_uint32), ("camera_height", C.c_uint32),
        ("max_cell_size", C.c_float),
        ("mode", C.c_int32),
        ("arith", C.c_int32),
        ("truncation", C.c_float),
        ("max_depth", C.c_float),
        ("min_z", C.c_float),
        ("memory", C.c_int32),
    ]


class VolumeInfo(C.Structure):
    _fields_ = [
        ("voxel_grid_size", C.c_uint32 * 3),
        ("voxel_size", C.c_float * 3),
        ("truncation", C.c_float),
        ("global_offset", C.c_float * 3),
        ("physical_size", C.c_float * 3),
        ("num_voxels", C.c_int64),
        ("tsdf", C.c_void_p),
        ("weights", C.c_void_p),
        ("mode", C.c_int32),
        ("arith", C.c_int32),
    ]


class Frame(C.Structure):
    _fields_ = [
        ("depth", C.c_void_p),
        ("pitch_bytes", C.c_size_t),
        ("width", C.c_int32), ("height", C.c_int32),
        ("format", C.c_int32),
        ("depth_scale", C.c_float),
        ("pose", C.c_double * 7),
    ]


# gbt_frame as a numpy record, for filling many frame descriptors at once
FRAME_DTYPE = None


def frame_dtype():
    global FRAME_DTYPE
    if FRAME_DTYPE is None:
        import numpy as np
        FRAME_DTYPE = np.dtype({"names": ["depth", "pitch_bytes", "width", "height", "format", "depth_scale", "pose"],
                                "formats": ["<u8", "<u8", "<i4", "<i4", "<i4", "<f4", ("<f8", 7)],
                                "offsets": [Frame.depth.offset, Frame.pitch_bytes.offset, Frame.width.offset,
                                            Frame.height.offset, Frame.format.offset, Frame.depth_scale.offset,
                                            Frame.pose.offset],
                                "itemsize": C.sizeof(Frame)})
    return FRAME_DTYPE


class DiffCfg(C.Structure):
    _fields_ = [
        ("voxel_grid_size", C.c_uint32 * 3),
        ("voxel_size", C.c_float * 3),
        ("global_offset", C.c_float * 3),
        ("focal_x", C.c_float), ("focal_y", C.c_float), ("cx", C.c_float), ("cy", C.c_float),
        ("truncation", C.c_float), ("max_weight", C.c_float), ("max_depth", C.c_float), ("min_z", C.c_float),
        ("width", C.c_int32), ("height", C.c_int32),
        ("dtype", C.c_int32),
    ]


class BatchItem(C.Structure):
    _fields_ = [("volume", C.c_void_p), ("first_frame", C.c_int32), ("nframes", C.c_int32)]


MAX_FRAMES_PER_SCENE_PASS = 128
DIFF_CHUNK_FRAMES = 8
POINT_BYTES = 33   # gbt_point, the reference's packed cudaPointCloud::Vertex

# (name, restype, argtypes) of every exported entry point, in header order.
SIGNATURES = [
    ("gbt_volume_create", C.c_int, [C.POINTER(VolumeCfg), C.c_void_p, C.POINTER(C.c_void_p)]),
    ("gbt_volume_destroy", C.c_int, [C.c_void_p]),
    ("gbt_volume_reset", C.c_int, [C.c_void_p, C.c_void_p]),
    ("gbt_volume_check", C.c_int, [C.c_void_p, C.c_void_p]),
    ("gbt_volume_save", C.c_int, [C.c_void_p, C.c_char_p, C.c_void_p]),
    ("gbt_volume_load", C.c_int, [C.c_char_p, C.c_void_p, C.POINTER(C.c_void_p)]),
    ("gbt_volume_get_cfg", C.c_int, [C.c_void_p, C.POINTER(VolumeCfg)]),
    ("gbt_volume_get_info", C.c_int, [C.c_void_p, C.POINTER(VolumeInfo)]),
    ("gbt_volume_transformation_voxels", C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(C.c_void_p)]),
    ("gbt_integrate", C.c_int, [C.c_void_p, C.POINTER(Frame), C.c_int32, C.c_void_p]),
    ("gbt_integrate_tuned", C.c_int, [C.c_void_p, C.POINTER(Frame), C.c_int32, C.c_int32, C.c_int32, C.c_void_p]),
    ("gbt_batch_create", C.c_int, [C.c_int32, C.c_int32, C.POINTER(C.c_void_p)]),
    ("gbt_batch_destroy", C.c_int, [C.c_void_p]),
    ("gbt_integrate_batch", C.c_int, [C.c_void_p, C.POINTER(BatchItem), C.c_int32, C.POINTER(Frame), C.c_int32,
                                      C.c_int32, C.c_int32, C.c_int32, C.c_void_p]),
    ("gbt_diff_forward", C.c_int, [C.POINTER(DiffCfg), C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                   C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p]),
    ("gbt_diff_backward", C.c_int, [C.POINTER(DiffCfg), C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                    C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                    C.c_void_p, C.c_void_p, C.c_void_p]),
    ("gbt_extract_mesh", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_int64,
                                   C.POINTER(C.c_int64), C.c_void_p]),
    ("gbt_extract_mesh_async", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_int64,
                                         C.c_void_p, C.c_void_p]),
    ("gbt_extract_mesh_indexed", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_int64,
                                           C.c_int64, C.POINTER(C.c_int64), C.POINTER(C.c_int64), C.c_void_p]),
    ("gbt_extract_mesh_noalloc", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_int64,
                                           C.c_void_p, C.c_void_p]),
    ("gbt_points_extract", C.c_int, [C.POINTER(C.c_double * 9), C.c_void_p, C.c_int64, C.c_int32, C.c_float,
                                     C.c_void_p, C.c_int64, C.c_int32, C.c_int32, C.POINTER(C.c_double * 7),
                                     C.c_int64, C.c_void_p, C.c_int64, C.c_void_p]),
    ("gbt_points_transform", C.c_int, [C.c_void_p, C.c_int64, C.POINTER(C.c_double * 7), C.c_void_p]),
    ("gbt_points_project", C.c_int, [C.c_void_p, C.c_int64, C.POINTER(C.c_double * 9), C.POINTER(C.c_double * 7),
                                     C.c_void_p, C.c_int64, C.c_void_p, C.c_int64, C.c_int32, C.c_int32,
                                     C.c_void_p, C.c_void_p]),
    ("gbt_image_filter_if", C.c_int, [C.c_void_p, C.c_int64, C.c_int32, C.c_int32, C.c_float, C.c_float,
                                      C.c_void_p]),
    ("gbt_last_error", C.c_char_p, []),
    ("gbt_debug_inject", C.c_int, [C.c_int32, C.c_int64, C.c_int64]),
    ("gbt_version", C.c_char_p, []),
]

_lock = threading.Lock()
_lib = None


class GbtError(RuntimeError):
    def __init__(self, status, message):
        super().__init__("gbt status %d: %s" % (status, message))
        self.status = status


def lib():
    """Load the engine library (raises if it has not been built)."""
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH):
                raise RuntimeError("engine library %s is missing; run cu-reconstruction_gb300/build.py "
                                   "(or __graft_entry__.build()) first" % LIB_PATH)
            handle = C.CDLL(LIB_PATH)
            for name, res, args in SIGNATURES:
                fn = getattr(handle, name)
                fn.restype = res
                fn.argtypes = args
            _lib = handle
        return _lib


def check(status):
    if status != GBT_OK:
        raise GbtError(status, lib().gbt_last_error().decode())
    return status


def device_tensor(t, name):
    """`t`, after checking that it lives in CUDA memory: the library reads and
    writes the pointers it is given on the GPU, where a host address faults."""
    if not getattr(t, "is_cuda", False):
        raise ValueError("%s must be a CUDA tensor (got %s)" % (name, getattr(t, "device", type(t).__name__)))
    return t


def device_image(t, name, dtypes, channels=0):
    """`t` as an image the kernels address by rows: a CUDA tensor of one of
    `dtypes`, (H, W) or, with `channels`, (H, W, channels), its pixels (and
    their channels) adjacent within a row; rows may be pitched."""
    device_tensor(t, name)
    if t.dtype not in dtypes:
        raise TypeError("%s must be %s, got %s" % (name, " or ".join(str(d) for d in dtypes), t.dtype))
    if channels:
        if t.dim() != 3 or t.shape[2] != channels or t.stride(2) != 1 or t.stride(1) != channels:
            raise ValueError("%s must be (H, W, %d) with interleaved channels" % (name, channels))
    elif t.dim() != 2 or t.stride(1) != 1:
        raise ValueError("%s must be (H, W) with contiguous rows" % name)
    return t
