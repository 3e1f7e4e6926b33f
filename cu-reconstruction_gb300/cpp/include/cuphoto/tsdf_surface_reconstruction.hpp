// cuphoto::TSDFSurface on the GB300 engine
// (reference: modules/include/tsdf_surface_reconstruction.hpp:10-37,
// modules/src/tsdf_surface_reconstruction.cpp:13-153).
//
// reconstruct_surface(color, depth) keeps the reference's behaviour: a fresh
// volume from the configuration, one frame integrated with the configured
// pose, the mesh extracted into get_mesh().  reconstruct_sequence() is the
// multi-frame driver the reference lacks: many frames into one volume, several
// frames per pass, then one mesh.
#ifndef CUPHOTO_GB300_TSDF_SURFACE_RECONSTRUCTION_HPP
#define CUPHOTO_GB300_TSDF_SURFACE_RECONSTRUCTION_HPP

#include <array>
#include <vector>

#include "config.hpp"
#include "cuda_point_cloud.cuh"
#include "cv_types.hpp"
#include "geometry.hpp"
#include "mesh.hpp"
#include "tsdf_volume.cuh"

namespace cuphoto {

class SurfaceReconstruction {
public:
    SurfaceReconstruction() = default;
    virtual ~SurfaceReconstruction() = default;
    Mesh get_mesh() const { return surface_mesh; }

protected:
    Mesh surface_mesh;
};

class TSDFSurface : public SurfaceReconstruction {
public:
    TSDFSurface(const Config& cfg);

    void reconstruct_surface(const cv::cuda::GpuMat& color, const cv::cuda::GpuMat& depth);

    // The cloud projected to colour + depth at the configured pose
    // (project_to_color_depth), then integrated and meshed.  The reference's
    // version (tsdf_surface_reconstruction.cpp:94-120) stops after the
    // projection, with its integrate and mesh calls commented out, and first
    // estimates normals with PCL, which nothing reads; both are left out here.
    void reconstruct_surface(const cudaPointCloud::Ptr cuda_pc);

    // frames: device depth images; poses: world-to-camera {qw,qx,qy,qz,tx,ty,tz}.
    // resume_from: a volume file (TSDFVolume::save) to continue instead of an
    // empty volume; save_to: where to write the volume after the frames.
    // Throws CuPhotoException when the volume cannot be created or loaded, a
    // pass of frames is refused, or the volume cannot be saved.
    void reconstruct_sequence(const std::vector<gbt_frame>& frames, i32 frames_per_pass = 16,
                              const std::string& resume_from = "", const std::string& save_to = "");

    void set_global_transformation(const SE3& transform);
    SE3 get_global_transformation() const;
    std::array<r64, 7> global_pose() const;

    TSDFVolumeConfig build_cfg() const;
    TSDFEngineOptions engine_options;

private:
    void mesh_from(const TSDFVolume& volume);

    SE3 global_transform;
    r64 normals_radius_search;
    i32 k_nn;

    Vec3 voxel_grid_size;
    Vec3 physical_size;
    Vec3 global_offset;
    r32 max_weight;
    r32 focal_x;
    r32 focal_y;
    r32 principal_x;
    r32 principal_y;
    ui32 camera_width;
    ui32 camera_height;
};

}  // namespace cuphoto

#endif
