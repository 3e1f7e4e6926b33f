// cuphoto::cudaPointCloud on the engine (reference:
// modules/src/cuda/cuda_point_cloud.cu:101-495).  The vertex array is managed
// memory, as in the reference, so the host-side members (add_vertex,
// filter_depth, save_ply) read and write it directly; the per-point kernels
// are the engine's (gbt_points_*).
#include "cuphoto/cuda_point_cloud.cuh"

#include <cstdio>
#include <cstring>
#include <fstream>
#include <new>
#include <vector>

namespace cuphoto {

namespace {

void log_error(const char* what) { std::fprintf(stderr, "[cuda]   %s\n", what); }

void log_engine(const char* where) { std::fprintf(stderr, "[cuda]   %s -- %s\n", where, gbt_last_error()); }

}  // namespace

cudaPointCloud::cudaPointCloud(const std::array<r64, 9>& camera_param, const size_t total_number_pts)
    : device_pts(nullptr), num_pts(0), total_num_pts(0), hasRGB(false) {
    camera_matrix = camera_param;
    if (!reserve_memory(total_number_pts)) {
        std::fprintf(stderr, "[cuda]   cudaPointCloud::reserve_memory() -- can't allocate query CUDA memory %lu\n",
                     (unsigned long)total_number_pts);
        throw std::bad_alloc();
    }
    total_num_pts = total_number_pts;
}

cudaPointCloud::~cudaPointCloud() { free(); }

cudaPointCloud::Ptr cudaPointCloud::create(const std::array<r64, 9>& camera_mat, const size_t total_number_pts) {
    return std::shared_ptr<cudaPointCloud>(new cudaPointCloud(camera_mat, total_number_pts));
}

cudaPointCloud::Ptr cudaPointCloud::merge(const cudaPointCloud::Ptr pc1, const cudaPointCloud::Ptr pc2) {
    const ui64 query_num_pts = pc1->get_num_points() + pc2->get_num_points();
    cudaPointCloud::Ptr cuda_pc = cudaPointCloud::create(pc1->get_camera_parameters(), query_num_pts);
    Vertex* cuda_pts = cuda_pc->get_points();
    cudaMemcpy(cuda_pts, pc1->get_points(), pc1->get_size(), cudaMemcpyDefault);
    cudaMemcpy(cuda_pts + pc1->get_num_points(), pc2->get_points(), pc2->get_size(), cudaMemcpyDefault);
    cuda_pc->set_total_number_pts();
    return cuda_pc;
}

void cudaPointCloud::clear() {
    if (device_pts != nullptr) cudaMemset(device_pts, 0, get_size());
    num_pts = 0;
}

void cudaPointCloud::free() {
    if (device_pts != nullptr) cudaFree(device_pts);
    device_pts = nullptr;
    num_pts = 0;
}

bool cudaPointCloud::reserve_memory(const ui64 query_number_points) {
    if (query_number_points <= 0) return true;
    if (query_number_points <= num_pts && device_pts != nullptr) {
        clear();
        return true;
    }
    free();
    if (cudaMallocManaged(&device_pts, query_number_points * sizeof(Vertex), cudaMemAttachGlobal) != cudaSuccess) {
        device_pts = nullptr;
        return false;
    }
    // a fresh cloud reads as zero points, as the reference's zeroed managed pages do
    cudaMemset(device_pts, 0, query_number_points * sizeof(Vertex));
    cudaDeviceSynchronize();
    return true;
}

bool cudaPointCloud::extract_points(const cv::cuda::PtrStepSzf depth, const cv::cuda::PtrStepb colors,
                                    const std::array<r64, 7>& T, const i32 frame_idx) {
    if (!depth.data) {
        log_error("cudaPointCloud::extract_points() -- depth map is null pointer");
        return false;
    }
    const ui32 width = depth.cols;
    const ui32 height = depth.rows;
    if (width == 0 || height == 0) {
        log_error("cudaPointCloud::extract_points() -- depth width/height parameters are zero");
        return false;
    }
    if (colors.data) hasRGB = true;
    const i64 start_idx = (i64)frame_idx * width * height;
    const gbt_status st =
        gbt_points_extract(camera_matrix.data(), depth.data, (int64_t)depth.step, GBT_DEPTH_F32_M, 1.0f,
                           colors.data, (int64_t)colors.step, (int32_t)width, (int32_t)height, T.data(), start_idx,
                           reinterpret_cast<gbt_point*>(device_pts), (int64_t)total_num_pts, nullptr);
    if (st != GBT_OK) {
        log_engine("cudaPointCloud::extract_points() -- failed to extract point cloud with CUDA");
        return false;
    }
    num_pts += (ui64)width * height;
    cudaDeviceSynchronize();
    return true;
}

bool cudaPointCloud::project(cv::cuda::PtrStepSzb* color, cv::cuda::PtrStepSzf depth,
                             const std::array<r64, 7>& camera_pose) {
    const size_t bytes = GBT_POINTS_PROJECT_SCRATCH_BYTES(depth.cols, depth.rows);
    void* scratch = nullptr;
    if (cudaMalloc(&scratch, bytes) != cudaSuccess) {
        log_error("cudaPointCloud::project_to_depth() -- can't allocate the z-buffer");
        return false;
    }
    const gbt_status st = gbt_points_project(reinterpret_cast<const gbt_point*>(device_pts), (int64_t)num_pts,
                                             camera_matrix.data(), camera_pose.data(), depth.data,
                                             (int64_t)depth.step, color ? color->data : nullptr,
                                             color ? (int64_t)color->step : 0, depth.cols, depth.rows, scratch,
                                             nullptr);
    const cudaError_t e = cudaDeviceSynchronize();
    cudaFree(scratch);
    if (st != GBT_OK || e != cudaSuccess) {
        log_engine("cudaPointCloud::project_to_depth() -- failed to filter image from pts cloud CUDA");
        return false;
    }
    return true;
}

bool cudaPointCloud::project_to_depth(cv::cuda::PtrStepSzf depth, const std::array<r64, 7>& camera_pose) {
    if (!depth.data) {
        log_error("cudaPointCloud::project_to_depth() -- depth map is null pointer");
        return false;
    }
    if (depth.cols == 0 || depth.rows == 0) {
        log_error("cudaPointCloud::project_to_depth() -- depth width/height parameters are zero");
        return false;
    }
    return project(nullptr, depth, camera_pose);
}

bool cudaPointCloud::project_to_color_depth(cv::cuda::PtrStepSzb color, cv::cuda::PtrStepSzf depth,
                                            const std::array<r64, 7>& camera_pose) {
    if (!depth.data || !color.data) {
        log_error("cudaPointCloud::project_to_depth() -- depth or color map is null pointer");
        return false;
    }
    if (depth.cols == 0 || depth.rows == 0) {
        log_error("cudaPointCloud::project_to_depth() -- depth width/height parameters are zero");
        return false;
    }
    return project(&color, depth, camera_pose);
}

bool cudaPointCloud::transform(const std::array<r64, 7>& T) {
    if (num_pts == 0) {
        log_error("cudaPointCloud::transform() -- the number of points is 0");
        return false;
    }
    if (device_pts == nullptr) {
        log_error("cudaPointCloud::transform() -- the device points is not allocated");
        return false;
    }
    if (gbt_points_transform(reinterpret_cast<gbt_point*>(device_pts), (int64_t)num_pts, T.data(), nullptr) !=
        GBT_OK) {
        log_engine("cudaPointCloud::transform() -- failed to transform point cloud with CUDA");
        return false;
    }
    cudaDeviceSynchronize();
    return true;
}

bool cudaPointCloud::add_vertex(const Vertex& v, const ui64 idx) {
    if (idx >= total_num_pts) {
        log_error("cudaPointCloud::add_vertex() -- index out of range");
        return false;
    }
    device_pts[idx] = v;
    return true;
}

bool cudaPointCloud::add_vertex(const float3 pos, const uchar3 color, const ui64 idx, const float4 normal) {
    if (idx >= total_num_pts) {
        log_error("cudaPointCloud::add_vertex() -- index out of range");
        return false;
    }
    device_pts[idx].pos = pos;
    device_pts[idx].normal = normal;
    device_pts[idx].color = color;
    return true;
}

// Keeps the points whose z is outside the open interval (min, max), which is
// what the reference's filter keeps (cuda_point_cloud.cu:409-435), in order.
void cudaPointCloud::filter_depth(const r32 depth_threshold_min, const r32 depth_threshold_max) {
    cudaDeviceSynchronize();
    std::vector<Vertex> kept;
    kept.reserve(num_pts);
    for (ui64 i = 0; i < num_pts; ++i) {
        const r32 z = device_pts[i].pos.z;
        const bool inside = z > depth_threshold_min && z < depth_threshold_max;
        if (!inside) kept.push_back(device_pts[i]);
    }
    Vertex* out = nullptr;
    if (cudaMallocManaged(&out, kept.size() * sizeof(Vertex), cudaMemAttachGlobal) != cudaSuccess) {
        std::fprintf(stderr, "[cuda]   cudaPointCloud::filter_depth() -- can't allocate query CUDA memory %lu\n",
                     (unsigned long)kept.size());
        throw std::bad_alloc();
    }
    if (!kept.empty()) std::memcpy(out, kept.data(), kept.size() * sizeof(Vertex));
    free();
    device_pts = out;
    num_pts = kept.size();
}

bool cudaPointCloud::add_point_cloud(const cudaPointCloud::Ptr cuda_pc) {
    const ui64 query_num_pts = cuda_pc->get_num_points() + num_pts;
    Vertex* cuda_pts = nullptr;
    if (cudaMallocManaged(&cuda_pts, query_num_pts * sizeof(Vertex), cudaMemAttachGlobal) != cudaSuccess) return false;
    cudaMemcpy(cuda_pts, device_pts, get_size(), cudaMemcpyDefault);
    cudaMemcpy(cuda_pts + num_pts, cuda_pc->get_points(), cuda_pc->get_size(), cudaMemcpyDefault);
    free();
    device_pts = cuda_pts;
    num_pts = query_num_pts;
    total_num_pts = query_num_pts;
    return true;
}

// ASCII PLY of position and colour, y and z negated for OpenGL-style viewers
// (the layout of cuda_point_cloud.cu:459-495); numbers in the stream's
// default format.
bool cudaPointCloud::save_ply(const std::string& filepath) const {
    if (filepath.empty()) {
        log_error("cudaPointCloud::save_ply() -- empty file path for store point cloud");
        return false;
    }
    if (!device_pts || num_pts <= 0) {
        log_error("cudaPointCloud::save_ply() -- can't store, point cloud is empty");
        return false;
    }
    cudaDeviceSynchronize();
    std::ofstream out(filepath.c_str());
    static const char* const kHeader[] = {"ply", "format ascii 1.0", nullptr, "property float x", "property float y",
                                          "property float z", "property uchar red", "property uchar green",
                                          "property uchar blue", "end_header"};
    for (const char* line : kHeader) {
        if (line)
            out << line << '\n';
        else
            out << "element vertex " << num_pts << '\n';
    }
    for (ui64 i = 0; i < num_pts; ++i) {
        const Vertex& v = device_pts[i];
        out << v.pos.x << ' ' << v.pos.y * -1.f << ' ' << v.pos.z * -1.f << ' ' << (i32)v.color.x << ' '
            << (i32)v.color.y << ' ' << (i32)v.color.z << '\n';
    }
    return true;
}

}  // namespace cuphoto
