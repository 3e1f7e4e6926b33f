// cuphoto::generate_triangular_surface on the GB300 engine
// (reference: modules/include/cuda/marching_cubes.cuh:13-15).  Appends to the
// caller's vectors: three vertices per triangle, indices offset by the
// vertices already present, in the reference's order.
#ifndef CUPHOTO_GB300_MARCHING_CUBES_CUH
#define CUPHOTO_GB300_MARCHING_CUBES_CUH

#include <vector>

#include <cuda_runtime.h>

#include "tsdf_volume.cuh"

namespace cuphoto {

void generate_triangular_surface(const TSDFVolume& tsdf_volume, std::vector<float3>& verts,
                                 std::vector<int3>& triangles);

// Engine addition for fixed-mode volumes (gbt_extract_mesh_indexed): the same
// triangles with one vertex per crossed grid edge and per-vertex normals.
// Appends like generate_triangular_surface (indices offset by the vertices
// already in `verts`; `normals` is kept the same length as `verts`).
// Returns false, after logging, on a compat volume or a failure.
bool generate_indexed_surface(const TSDFVolume& tsdf_volume, std::vector<float3>& verts, std::vector<float3>& normals,
                              std::vector<int3>& triangles);

}  // namespace cuphoto

#endif
