"""Python host layer of the GB300 TSDF engine, mirroring cuphoto's TSDF API.

Import with the package directory ``cu-reconstruction_gb300`` on ``sys.path``.
"""
from .tsdf import (TSDFVolume, TSDFVolumeConfig, extract_mesh_device, generate_triangular_surface,  # noqa: F401
                   make_frame)
from . import synthetic  # noqa: F401
from .points import PointCloud  # noqa: F401

__all__ = ["TSDFVolume", "TSDFVolumeConfig", "generate_triangular_surface", "extract_mesh_device",
           "make_frame", "synthetic", "PointCloud"]
