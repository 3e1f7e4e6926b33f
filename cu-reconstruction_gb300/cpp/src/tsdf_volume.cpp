// cuphoto::TSDFVolume over the engine's C ABI (reference: tsdf_volume.cu:194-290).
#include "cuphoto/tsdf_volume.cuh"

#include <cstdio>
#include <cstring>

namespace cuphoto {

namespace {

void log_error(const char* what) { std::fprintf(stderr, "[cuda]   %s\n", what); }

void log_engine_error(const char* where) {
    std::fprintf(stderr, "[cuda]   %s -- %s\n", where, gbt_last_error());
}

gbt_volume_cfg to_engine(const TSDFVolumeConfig& c, const TSDFEngineOptions& o) {
    gbt_volume_cfg e;
    std::memset(&e, 0, sizeof(e));
    e.voxel_grid_size[0] = c.voxel_grid_size.x;
    e.voxel_grid_size[1] = c.voxel_grid_size.y;
    e.voxel_grid_size[2] = c.voxel_grid_size.z;
    e.physical_size[0] = c.physical_size.x;
    e.physical_size[1] = c.physical_size.y;
    e.physical_size[2] = c.physical_size.z;
    e.global_offset[0] = c.global_offset.x;
    e.global_offset[1] = c.global_offset.y;
    e.global_offset[2] = c.global_offset.z;
    e.max_weight = c.max_weight;
    e.focal_x = c.focal_x;
    e.focal_y = c.focal_y;
    e.cx = c.cx;
    e.cy = c.cy;
    e.camera_width = c.camera_width;
    e.camera_height = c.camera_height;
    e.max_cell_size = c.max_cell_size;
    e.mode = o.mode;
    e.arith = o.arith;
    e.truncation = o.truncation;
    e.max_depth = o.max_depth;
    e.min_z = o.min_z;
    e.memory = o.memory;
    return e;
}

}  // namespace

TSDFVolume::TSDFVolume(const TSDFVolumeConfig& tsdf_cfg) : TSDFVolume(tsdf_cfg, TSDFEngineOptions()) {}

TSDFVolume::TSDFVolume(const TSDFVolumeConfig& tsdf_cfg, const TSDFEngineOptions& opts) : cfg(tsdf_cfg) {
    const gbt_volume_cfg e = to_engine(cfg, opts);
    // the reference's constructor logs allocation failures and carries on
    // (tsdf_volume.cu:203-211); the engine volume is then null and every
    // later call reports false
    if (gbt_volume_create(&e, nullptr, &vol) != GBT_OK) {
        log_engine_error("TSDFVolume::TSDFVolume()");
        vol = nullptr;
        return;
    }
    gbt_volume_get_info(vol, &info);
}

TSDFVolume::TSDFVolume(gbt_volume* loaded, const TSDFVolumeConfig& tsdf_cfg) : cfg(tsdf_cfg), vol(loaded) {
    gbt_volume_get_info(vol, &info);
}

bool TSDFVolume::save(const std::string& path) const {
    if (!vol) {
        log_error("TSDFVolume::save() -- the volume was not created");
        return false;
    }
    if (gbt_volume_save(vol, path.c_str(), nullptr) != GBT_OK) {
        log_engine_error("TSDFVolume::save()");
        return false;
    }
    return true;
}

TSDFVolume::Ptr TSDFVolume::load(const std::string& path) {
    gbt_volume* v = nullptr;
    gbt_volume_cfg e;
    if (gbt_volume_load(path.c_str(), nullptr, &v) != GBT_OK || gbt_volume_get_cfg(v, &e) != GBT_OK) {
        log_engine_error("TSDFVolume::load()");
        if (v) gbt_volume_destroy(v);
        return nullptr;
    }
    TSDFVolumeConfig c;
    c.voxel_grid_size = dim3(e.voxel_grid_size[0], e.voxel_grid_size[1], e.voxel_grid_size[2]);
    c.physical_size = make_float3(e.physical_size[0], e.physical_size[1], e.physical_size[2]);
    c.global_offset = make_float3(e.global_offset[0], e.global_offset[1], e.global_offset[2]);
    c.max_weight = e.max_weight;
    c.focal_x = e.focal_x;
    c.focal_y = e.focal_y;
    c.cx = e.cx;
    c.cy = e.cy;
    c.camera_width = e.camera_width;
    c.camera_height = e.camera_height;
    c.max_cell_size = e.max_cell_size;
    return Ptr(new TSDFVolume(v, c));
}

TSDFVolume::~TSDFVolume() {
    if (vol) gbt_volume_destroy(vol);
}

bool TSDFVolume::integrate(const std::shared_ptr<cudaPointCloud>, cv::cuda::PtrStepSzf, const std::array<r64, 7>&) {
    log_error("TSDFVolume::integrate(cudaPointCloud) -- not implemented (declared but undefined in the reference)");
    return false;
}

bool TSDFVolume::apply_isosurface_transformation(void*, const ui32, const std::array<r64, 7>&) {
    log_error("TSDFVolume::apply_isosurface_transformation() -- not implemented (declared but undefined in the reference)");
    return false;
}

bool TSDFVolume::integrate(const cv::cuda::PtrStepSzb color, const cv::cuda::PtrStepSzf depth,
                           const std::array<r64, 7>& camera_pose) {
    // tsdf_volume.cu:260-268
    if (!depth.data || !color.data) {
        log_error("TSDFVolume::integrate() -- depth or color map is null pointer");
        return false;
    }
    if (depth.rows == 0 || depth.cols == 0 || color.rows == 0 || color.cols == 0) {
        log_error("TSDFVolume::integrate() -- depth width/height parameters are zero");
        return false;
    }
    if (!vol) {
        log_error("TSDFVolume::integrate() -- volume was not allocated");
        return false;
    }
    gbt_frame f;
    std::memset(&f, 0, sizeof(f));
    f.depth = depth.data;
    f.pitch_bytes = depth.step;
    f.width = depth.cols;
    f.height = depth.rows;
    f.format = GBT_DEPTH_F32_M;
    f.depth_scale = 1.f;
    for (int k = 0; k < 7; ++k) f.pose[k] = camera_pose[k];
    if (gbt_integrate(vol, &f, 1, nullptr) != GBT_OK) {
        log_engine_error("TSDFVolume::integrate() -- failed integrate signed distance function on voxels data");
        return false;
    }
    // tsdf_volume.cu:287
    if (cudaDeviceSynchronize() != cudaSuccess) {
        log_error("TSDFVolume::integrate() -- device synchronisation failed");
        return false;
    }
    return true;
}

bool TSDFVolume::integrate_frames(const gbt_frame* frames, i32 nframes, cudaStream_t stream) {
    if (!vol) return false;
    for (i32 s = 0; s < nframes; s += GBT_MAX_FRAMES_PER_PASS) {
        const i32 n = nframes - s < GBT_MAX_FRAMES_PER_PASS ? nframes - s : GBT_MAX_FRAMES_PER_PASS;
        if (gbt_integrate(vol, frames + s, n, stream) != GBT_OK) {
            log_engine_error("TSDFVolume::integrate_frames()");
            return false;
        }
    }
    return true;
}

TSDFVolume::TransformationVoxel::Ptr TSDFVolume::transformation_voxels_data() {
    return static_cast<const TSDFVolume*>(this)->transformation_voxels_data();
}

TSDFVolume::TransformationVoxel::Ptr TSDFVolume::transformation_voxels_data() const {
    if (!vol) return nullptr;
    void* p = nullptr;
    if (gbt_volume_transformation_voxels(vol, nullptr, &p) != GBT_OK) {
        log_engine_error("TSDFVolume::transformation_voxels_data()");
        return nullptr;
    }
    cudaDeviceSynchronize();
    return static_cast<TransformationVoxel::Ptr>(p);
}

}  // namespace cuphoto
