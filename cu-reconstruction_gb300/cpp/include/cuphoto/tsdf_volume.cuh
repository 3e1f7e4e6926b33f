// cuphoto::TSDFVolume on the GB300 engine.
//
// Same declarations as the reference (modules/include/cuda/tsdf_volume.cuh:12-105):
// TSDFVolumeConfig, TSDFVolume(cfg), integrate(color, depth, pose) -> bool and
// the accessors.  Behaviour kept: errors are logged to stderr and reported as
// false, every call synchronises the device, depth and colour are borrowed
// device images, the colour image is checked but never read.  The volume's
// memory is managed memory by default, so the accessors' pointers are
// host-readable as in the reference.  Engine options (mode, arithmetic,
// truncation, memory kind) are set through engine_options().
#ifndef CUPHOTO_GB300_TSDF_VOLUME_CUH
#define CUPHOTO_GB300_TSDF_VOLUME_CUH

#include <array>
#include <memory>
#include <string>

#include <cuda_runtime.h>

#include "gbt_tsdf.h"
#include "cv_types.hpp"
#include "types.cuh"

namespace cuphoto {

enum WEIGHT_TYPE {
    WEIGHT_BY_DEPTH = 0,
    WEIGHT_BY_VARIANCE,
};

struct TSDFVolumeConfig {
    dim3 voxel_grid_size;
    float3 physical_size;  // in physical units
    float3 global_offset;  // grid_offset
    r32 max_weight;
    r32 focal_x;
    r32 focal_y;
    r32 cx;
    r32 cy;
    ui32 camera_width;
    ui32 camera_height;
    r32 max_cell_size = 0.0;
};

// Engine options beyond the reference's configuration.
struct TSDFEngineOptions {
    i32 mode = GBT_MODE_COMPAT;
    i32 arith = GBT_ARITH_REFERENCE;
    r32 truncation = 0.f;
    r32 max_depth = 0.f;
    r32 min_z = 0.f;
    i32 memory = GBT_MEMORY_MANAGED;
    // fixed mode: mesh with shared vertices and per-vertex normals
    // (generate_indexed_surface) instead of three vertices per triangle
    bool shared_vertices = false;
};

class cudaPointCloud;

class TSDFVolume {
public:
    struct TransformationVoxel {
        using Ptr = TransformationVoxel*;
        float3 translation;
        float4 quat_rotation;
    } __attribute__((packed));

public:
    using Ptr = std::shared_ptr<TSDFVolume>;

    TSDFVolume(const TSDFVolumeConfig& tsdf_cfg);
    TSDFVolume(const TSDFVolumeConfig& tsdf_cfg, const TSDFEngineOptions& opts);
    ~TSDFVolume();
    TSDFVolume(const TSDFVolume&) = delete;
    TSDFVolume& operator=(const TSDFVolume&) = delete;

    // Declared but never defined by the reference (tsdf_volume.cuh:45-55):
    // kept for source compatibility; they log and return false.
    bool integrate(const std::shared_ptr<cudaPointCloud> cuda_pc, cv::cuda::PtrStepSzf depth,
                   const std::array<r64, 7>& camera_pose);
    bool apply_isosurface_transformation(void* vertices, const ui32 num_pts, const std::array<r64, 7>& camera_pose);

    bool integrate(const cv::cuda::PtrStepSzb color, const cv::cuda::PtrStepSzf depth,
                   const std::array<r64, 7>& camera_pose);

    // Engine extension: several frames in one pass over the volume, uint16 or
    // float depth, on a stream; no device-wide synchronisation.
    bool integrate_frames(const gbt_frame* frames, i32 nframes, cudaStream_t stream = nullptr);

    r32* voxel_distances_data() { return info.tsdf; }
    r32* voxel_distances_data() const { return info.tsdf; }
    r32* voxel_weights_data() { return info.weights; }
    dim3 voxel_grid_size() const { return cfg.voxel_grid_size; }
    float3 global_offset() const { return cfg.global_offset; }
    float3 scale_voxel_size() const { return make_float3(info.voxel_size[0], info.voxel_size[1], info.voxel_size[2]); }
    float3 voxel_phys_size() const { return cfg.physical_size; }
    r32 truncation() const { return info.truncation; }

    TransformationVoxel::Ptr transformation_voxels_data();
    TransformationVoxel::Ptr transformation_voxels_data() const;

    gbt_volume* engine() const { return vol; }
    bool valid() const { return vol != nullptr; }

    // Engine extension: checkpoint and resume (gbt_volume_save / gbt_volume_load).
    // save() synchronises the device; load() returns nullptr (and logs) on failure.
    bool save(const std::string& path) const;
    static Ptr load(const std::string& path);

private:
    TSDFVolume(gbt_volume* loaded, const TSDFVolumeConfig& tsdf_cfg);

    TSDFVolumeConfig cfg;
    gbt_volume* vol = nullptr;
    gbt_volume_info info{};
};

}  // namespace cuphoto

#endif
