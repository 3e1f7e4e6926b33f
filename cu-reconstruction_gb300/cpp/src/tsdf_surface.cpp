// cuphoto::TSDFSurface (reference: tsdf_surface_reconstruction.cpp:13-153).
#include "cuphoto/tsdf_surface_reconstruction.hpp"

#include <cmath>
#include <cstdio>
#include <string>

#include "cuphoto/cp_exception.hpp"
#include "cuphoto/marching_cubes.cuh"

namespace cuphoto {

TSDFVolumeConfig TSDFSurface::build_cfg() const {
    TSDFVolumeConfig c;
    c.voxel_grid_size = dim3((unsigned)voxel_grid_size.x(), (unsigned)voxel_grid_size.y(), (unsigned)voxel_grid_size.z());
    c.physical_size = make_float3((float)physical_size.x(), (float)physical_size.y(), (float)physical_size.z());
    c.global_offset = make_float3((float)global_offset.x(), (float)global_offset.y(), (float)global_offset.z());
    c.max_weight = max_weight;
    c.focal_x = focal_x;
    c.focal_y = focal_y;
    c.cx = principal_x;
    c.cy = principal_y;
    c.camera_width = camera_width;
    c.camera_height = camera_height;
    return c;
}

// tsdf_surface_reconstruction.cpp:41-82: the same keys and defaults.
TSDFSurface::TSDFSurface(const Config& cfg) {
    normals_radius_search = cfg.get<r64>("pcl.normals.radius_search", 0.0);
    k_nn = cfg.get<i32>("pcl.normals.k_nn", 0);
    voxel_grid_size.x() = cfg.get<r32>("tsdf.volume.voxel_grid_size.x");
    voxel_grid_size.y() = cfg.get<r32>("tsdf.volume.voxel_grid_size.y");
    voxel_grid_size.z() = cfg.get<r32>("tsdf.volume.voxel_grid_size.z");
    physical_size.x() = cfg.get<r32>("tsdf.volume.physical_size.x");
    physical_size.y() = cfg.get<r32>("tsdf.volume.physical_size.y");
    physical_size.z() = cfg.get<r32>("tsdf.volume.physical_size.z");
    max_weight = cfg.get<r32>("tsdf.volume.max_weight");
    global_offset.x() = cfg.get<r32>("tsdf.volume.global_offset.x", 0.f);
    global_offset.y() = cfg.get<r32>("tsdf.volume.global_offset.y", 0.f);
    global_offset.z() = cfg.get<r32>("tsdf.volume.global_offset.z", 0.f);
    focal_x = cfg.get<r32>("camera.fx", 1.0f);
    focal_y = cfg.get<r32>("camera.fy", 1.0f);
    principal_x = cfg.get<r32>("camera.cx", 0.f);
    principal_y = cfg.get<r32>("camera.cy", 0.f);
    camera_width = (ui32)cfg.get<r32>("camera.width");
    camera_height = (ui32)cfg.get<r32>("camera.height");

    const r32 roll_degree = cfg.get<r32>("tsdf.volume.camera.pose.euler.roll", 0.f);
    const r32 yaw_degree = cfg.get<r32>("tsdf.volume.camera.pose.euler.yaw", 0.f);
    const r32 pitch_degree = cfg.get<r32>("tsdf.volume.camera.pose.euler.pitch", 0.f);
    const r32 half_c = (r32)(M_PI / 180.);
    const Quat roll = Quat::angle_axis(roll_degree * half_c, 0, 0, 1);
    const Quat yaw = Quat::angle_axis(yaw_degree * half_c, 0, 1, 0);
    const Quat pitch = Quat::angle_axis(pitch_degree * half_c, 1, 0, 0);
    const Vec3 t(cfg.get<r32>("tsdf.volume.camera.pose.translation.x", 0.f),
                 cfg.get<r32>("tsdf.volume.camera.pose.translation.y", 0.f),
                 cfg.get<r32>("tsdf.volume.camera.pose.translation.z", 0.f));
    set_global_transformation(SE3(roll * yaw * pitch, t));

    // engine options (not in the reference's files; defaults reproduce it)
    const std::string mode = cfg.get<std::string>("tsdf.engine.mode", "compat");
    engine_options.mode = mode == "fixed" ? GBT_MODE_FIXED : GBT_MODE_COMPAT;
    engine_options.arith = cfg.get<std::string>("tsdf.engine.arith", "reference") == "ieee" ? GBT_ARITH_IEEE
                                                                                            : GBT_ARITH_REFERENCE;
    engine_options.truncation = cfg.get<r32>("tsdf.engine.truncation", 0.f);
    engine_options.max_depth = cfg.get<r32>("tsdf.engine.max_depth", 0.f);
    engine_options.shared_vertices = cfg.get<std::string>("tsdf.engine.shared_vertices", "false") == "true";
}

void TSDFSurface::set_global_transformation(const SE3& transform) { global_transform = transform; }

SE3 TSDFSurface::get_global_transformation() const { return global_transform; }

// tsdf_surface_reconstruction.cpp:127-130: the quaternion of the rotation matrix.
std::array<r64, 7> TSDFSurface::global_pose() const {
    const Mat3 R = global_transform.rotationMatrix();
    const Vec3 t = global_transform.translation();
    const Quat q(R);
    return {q.w(), q.x(), q.y(), q.z(), t.x(), t.y(), t.z()};
}

void TSDFSurface::mesh_from(const TSDFVolume& volume) {
    std::vector<float3> verts;
    std::vector<int3> triangles;
    if (engine_options.shared_vertices && engine_options.mode == GBT_MODE_FIXED) {
        std::vector<float3> nrm;
        if (generate_indexed_surface(volume, verts, nrm, triangles)) {
            std::vector<Mesh::Normal> mesh_normals(nrm.size());
            for (size_t i = 0; i < nrm.size(); ++i) mesh_normals[i] = Mesh::Normal(nrm[i].x, nrm[i].y, nrm[i].z, 0.f);
            surface_mesh.normals(mesh_normals);
        }
    } else {
        generate_triangular_surface(volume, verts, triangles);
    }
    std::vector<Mesh::Point> mesh_verts(verts.size());
    std::vector<Mesh::Triangle> mesh_triangles(triangles.size());
    for (size_t i = 0; i < verts.size(); ++i) mesh_verts[i] = Mesh::Point(verts[i].x, verts[i].y, verts[i].z);
    for (size_t i = 0; i < triangles.size(); ++i)
        mesh_triangles[i] = Mesh::Triangle(triangles[i].x, triangles[i].y, triangles[i].z);
    surface_mesh.vertices(mesh_verts);
    surface_mesh.polygons(mesh_triangles);
}

void TSDFSurface::reconstruct_surface(const cv::cuda::GpuMat& color, const cv::cuda::GpuMat& depth) {
    TSDFVolume tsdf_volume(build_cfg(), engine_options);
    tsdf_volume.integrate(color, depth, global_pose());
    mesh_from(tsdf_volume);
}

void TSDFSurface::reconstruct_surface(const cudaPointCloud::Ptr cuda_pc) {
    cv::cuda::GpuMat gpu_depth((int)camera_height, (int)camera_width, CV_32F);
    cv::cuda::GpuMat gpu_color((int)camera_height, (int)camera_width, CV_8UC3);
    if (!cuda_pc->project_to_color_depth(gpu_color, gpu_depth, global_pose())) return;
    TSDFVolume tsdf_volume(build_cfg(), engine_options);
    tsdf_volume.integrate(gpu_color, gpu_depth, global_pose());
    mesh_from(tsdf_volume);
}

void TSDFSurface::reconstruct_sequence(const std::vector<gbt_frame>& frames, i32 frames_per_pass,
                                       const std::string& resume_from, const std::string& save_to) {
    TSDFVolume::Ptr tsdf_volume = resume_from.empty() ? std::make_shared<TSDFVolume>(build_cfg(), engine_options)
                                                      : TSDFVolume::load(resume_from);
    if (!tsdf_volume || !tsdf_volume->valid())
        throw CuPhotoException("TSDFSurface::reconstruct_sequence: no volume to integrate into");
    if (frames_per_pass < 1) frames_per_pass = 1;
    if (frames_per_pass > GBT_MAX_FRAMES_PER_PASS) frames_per_pass = GBT_MAX_FRAMES_PER_PASS;
    for (size_t s = 0; s < frames.size(); s += (size_t)frames_per_pass) {
        const i32 n = (i32)((frames.size() - s) < (size_t)frames_per_pass ? frames.size() - s : (size_t)frames_per_pass);
        // (integrate_frames has logged the engine's message)
        if (!tsdf_volume->integrate_frames(frames.data() + s, n))
            throw CuPhotoException("TSDFSurface::reconstruct_sequence: integrating frames " + std::to_string(s) +
                                   ".." + std::to_string(s + (size_t)n - 1) + " failed");
    }
    cudaDeviceSynchronize();
    if (!save_to.empty() && !tsdf_volume->save(save_to))
        throw CuPhotoException("TSDFSurface::reconstruct_sequence: cannot save the volume to " + save_to);
    mesh_from(*tsdf_volume);
}

}  // namespace cuphoto
