// cuphoto::cudaPointCloud on the GB300 engine
// (reference: modules/include/cuda/cuda_point_cloud.cuh:13-103,
// modules/src/cuda/cuda_point_cloud.cu:101-495).
//
// Same declarations, memory model (managed memory, host-readable vertices)
// and bool + LogError conventions; the per-point work runs in the engine's
// kernels (gbt_points_* in gbt_tsdf.h): back-projection, transform, and a GPU
// z-buffer in place of the reference's host projection loop, with the same
// images as that loop for continuous (unpitched) images.  Pitched depth and
// colour images are written row by row (the reference copies a continuous
// host image over them).
#ifndef CUPHOTO_GB300_CUDA_POINT_CLOUD_CUH
#define CUPHOTO_GB300_CUDA_POINT_CLOUD_CUH

#include <array>
#include <limits>
#include <memory>
#include <string>

#include <cuda_runtime.h>

#include "cv_types.hpp"
#include "gbt_tsdf.h"
#include "types.cuh"

namespace cuphoto {

class cudaPointCloud {
public:
    struct Vertex {
        using Ptr = Vertex*;
        // The XYZ position of the point.
        float3 pos;
        float4 normal;

        uchar3 color;

        ui16 classID = 0;
    } __attribute__((packed));

public:
    using Ptr = std::shared_ptr<cudaPointCloud>;

    ~cudaPointCloud();
    // the cloud owns its device buffer: shared through Ptr, never copied
    cudaPointCloud(const cudaPointCloud&) = delete;
    cudaPointCloud& operator=(const cudaPointCloud&) = delete;

    static cudaPointCloud::Ptr create(const std::array<r64, 9>& camera_mat, const size_t total_number_pts);

    static cudaPointCloud::Ptr merge(const cudaPointCloud::Ptr pc1, const cudaPointCloud::Ptr pc2);

    inline ui64 get_total_num_points() const { return total_num_pts; }

    inline ui64 get_num_points() const { return num_pts; }

    inline ui64 get_size() const { return num_pts * sizeof(Vertex); }

    inline Vertex* get_vertex(const ui64 index) const { return device_pts + index; }

    inline Vertex* get_points() const { return device_pts; }

    inline std::array<r64, 9> get_camera_parameters() { return camera_matrix; }

    inline void set_total_number_pts() { num_pts = total_num_pts; }

    bool add_point_cloud(const cudaPointCloud::Ptr cuda_pc);

    bool extract_points(const cv::cuda::PtrStepSzf depth, const cv::cuda::PtrStepb colors,
                        const std::array<r64, 7>& transform, const i32 frame_idx);

    bool project_to_depth(cv::cuda::PtrStepSzf depth, const std::array<r64, 7>& camera_pose);

    bool project_to_color_depth(cv::cuda::PtrStepSzb color, cv::cuda::PtrStepSzf depth,
                                const std::array<r64, 7>& camera_pose);

    bool transform(const std::array<r64, 7>& transform);

    void filter_depth(const r32 depth_threshold_min = std::numeric_limits<r32>::min(),
                      const r32 depth_threshold_max = std::numeric_limits<r32>::max());
    bool add_vertex(const Vertex& v, const ui64 idx);
    bool add_vertex(const float3 pos, const uchar3 color, const ui64 idx, const float4 normal = make_float4(0., 0., 0., 0.));
    void clear();
    void free();
    bool save_ply(const std::string& filepath) const;

protected:
    bool reserve_memory(const ui64 query_number_points);

    cudaPointCloud(const std::array<r64, 9>& camera_mat, const size_t total_number_pts);

private:
    bool project(cv::cuda::PtrStepSzb* color, cv::cuda::PtrStepSzf depth, const std::array<r64, 7>& camera_pose);

    Vertex* device_pts;
    ui64 num_pts;
    ui64 total_num_pts;
    std::array<r64, 9> camera_matrix;

    bool hasRGB;
};

static_assert(sizeof(cudaPointCloud::Vertex) == sizeof(gbt_point), "the engine's point is the reference's vertex");

}  // namespace cuphoto

#endif
