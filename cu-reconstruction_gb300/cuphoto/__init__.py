"""Python host layer of the GB300 TSDF engine, mirroring cuphoto's TSDF API.

Import with the package directory ``cu-reconstruction_gb300`` on ``sys.path``.
"""
from .tsdf import (TSDFVolume, TSDFVolumeConfig, extract_mesh_device, extract_mesh_indexed,  # noqa: F401
                   generate_triangular_surface, make_frame)
from . import synthetic  # noqa: F401
from .points import PointCloud  # noqa: F401

__all__ = ["TSDFVolume", "TSDFVolumeConfig", "generate_triangular_surface", "extract_mesh_device", "extract_mesh_indexed",
           "make_frame", "synthetic", "PointCloud"]
