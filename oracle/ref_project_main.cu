// Host-loop harness: runs the reference's own z-buffer projection,
// cudaPointCloud::project_to_color_depth (cuda_point_cloud.cu:292-353),
// compiled from the reference's sources by oracle/build.py, on a point cloud
// read from a file, and writes the depth and colour images it builds.
//
// TEST INFRASTRUCTURE ONLY: it produces the golden vectors of
// tests/golden/points_project_ref.npz (tests/golden/make_golden_project.py) and is
// never part of the engine.
//
// The reference keeps its points in managed memory allocated by its
// constructor; here the object is laid out in plain storage and pointed at
// host memory (the loop reads the points on the host).  The loop ends by
// copying its two host images to the device with cudaMemcpy and running
// filter_image_if there; this build environment has no GPU, so those calls
// fail (the reference logs and returns false) and the images are read from
// the shim's record of destroyed cv::Mat objects instead.  filter_image_if
// (cuda_point_cloud.cu:89-99) is then applied here as the kernel applies it:
// pixels within 1e-10 of FLT_MAX (near_equal, util.cu:6-10) become 0.
//
// Input file:  int64 n, int32 width, int32 height, double camera_matrix[9],
//              double pose[7], then n points of 33 bytes (cudaPointCloud::Vertex).
// Output file: float depth[height][width], uint8 color[height][width][3].
#define private public
#define protected public
#include "cuda/cuda_point_cloud.cuh"
#undef private
#undef protected

#include <opencv2/core/core.hpp>

#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <vector>

int main(int argc, char** argv) {
    if (argc != 3) {
        std::fprintf(stderr, "usage: %s <points file> <images file>\n", argv[0]);
        return 2;
    }
    FILE* f = std::fopen(argv[1], "rb");
    if (!f) return 3;
    int64_t n = 0;
    int32_t W = 0, H = 0;
    std::array<double, 9> m{};
    std::array<double, 7> pose{};
    bool ok = std::fread(&n, 8, 1, f) == 1 && std::fread(&W, 4, 1, f) == 1 && std::fread(&H, 4, 1, f) == 1 &&
              std::fread(m.data(), 8, 9, f) == 9 && std::fread(pose.data(), 8, 7, f) == 7;
    static_assert(sizeof(cuphoto::cudaPointCloud::Vertex) == 33, "packed 33-byte vertex");
    std::vector<unsigned char> pts((size_t)n * 33);
    ok = ok && n >= 0 && W > 0 && H > 0 && std::fread(pts.data(), 1, pts.size(), f) == pts.size();
    std::fclose(f);
    if (!ok) return 4;

    alignas(16) static unsigned char storage[sizeof(cuphoto::cudaPointCloud)];
    cuphoto::cudaPointCloud* pc = reinterpret_cast<cuphoto::cudaPointCloud*>(storage);
    pc->device_pts = reinterpret_cast<cuphoto::cudaPointCloud::Vertex*>(pts.data());
    pc->num_pts = (cuphoto::ui64)n;
    pc->total_num_pts = (cuphoto::ui64)n;
    pc->camera_matrix = m;
    pc->hasRGB = true;

    std::vector<float> depth_dev((size_t)W * H);
    std::vector<unsigned char> color_dev((size_t)W * H * 3);
    cv::cuda::PtrStepSzf depth(H, W, depth_dev.data(), (size_t)W * 4);
    cv::cuda::PtrStepSzb color(H, W, color_dev.data(), (size_t)W * 3);
    cv::shim_captured().clear();
    pc->project_to_color_depth(color, depth, pose);

    const cv::ShimImage* dimg = nullptr;
    const cv::ShimImage* cimg = nullptr;
    for (const cv::ShimImage& im : cv::shim_captured()) {
        if (im.rows == H && im.cols == W && im.elem == 4) dimg = &im;
        if (im.rows == H && im.cols == W && im.elem == 3) cimg = &im;
    }
    if (!dimg || !cimg) {
        std::fprintf(stderr, "the projection's images were not captured\n");
        return 5;
    }
    std::vector<float> out_depth((size_t)W * H);
    std::memcpy(out_depth.data(), dimg->data.data(), out_depth.size() * 4);
    for (float& z : out_depth)
        if (std::fabs(z - FLT_MAX) < 1e-10f) z = 0.0f;
    FILE* o = std::fopen(argv[2], "wb");
    if (!o) return 6;
    ok = std::fwrite(out_depth.data(), 4, out_depth.size(), o) == out_depth.size() &&
         std::fwrite(cimg->data.data(), 1, cimg->data.size(), o) == cimg->data.size();
    std::fclose(o);
    return ok ? 0 : 7;
}
