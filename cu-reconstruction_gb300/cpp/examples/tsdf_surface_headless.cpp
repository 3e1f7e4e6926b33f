// Headless driver of the TSDF example on the GB300 engine.
//
// Mirrors examples/tsdf_surface_reconstruction/tsdf_surface.cpp:12-52 call for
// call (Config from --config_path, one RGB-D frame, TSDFSurface(cfg),
// reconstruct_surface(rgb, depth), get_mesh().store_to_ply(mesh_store.path)),
// without OpenCV, gflags or glog: the depth frame is a raw little-endian
// uint16 image of camera.width x camera.height (--depth), converted with
// depth_scale as the reference's reader does (rgbd_dataset.cpp:29), and the
// colour image is a black frame (the path never reads colour).
//
//   tsdf_surface_headless --config_path cfg.yaml --depth frame.u16
//   tsdf_surface_headless --config_path cfg.yaml --sequence frames.u16 --poses poses.f64 --frames N [--per_pass K]
//                         [--resume_volume in.gbtv] [--save_volume out.gbtv]
//
// --sequence integrates N frames with their own world-to-camera poses
// (N x 7 doubles: qw qx qy qz tx ty tz) through the multi-frame driver.
// --points goes through a point cloud instead of the depth image: the frame
// is back-projected into a cudaPointCloud at the inverse of the configured
// pose (world coordinates), optionally stored with save_ply (--points_ply),
// and reconstruct_surface(cloud) projects it back and integrates it.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <string>
#include <vector>

#include "cuphoto/config.hpp"
#include "cuphoto/cp_exception.hpp"
#include "cuphoto/tsdf_surface_reconstruction.hpp"

namespace {

std::string arg(int argc, char** argv, const char* name, const char* def) {
    for (int i = 1; i + 1 < argc; ++i)
        if (std::strcmp(argv[i], name) == 0) return argv[i + 1];
    return def;
}

bool flag(int argc, char** argv, const char* name) {
    for (int i = 1; i < argc; ++i)
        if (std::strcmp(argv[i], name) == 0) return true;
    return false;
}

bool read_file(const std::string& path, std::vector<char>& out) {
    std::ifstream f(path, std::ios::binary);
    if (!f) return false;
    out.assign(std::istreambuf_iterator<char>(f), std::istreambuf_iterator<char>());
    return true;
}

}  // namespace

int main(int argc, char** argv) {
    const std::string config_path = arg(argc, argv, "--config_path", "./data/tsdf_surface_parameters.yaml");
    cuphoto::Config cfg;
    if (cfg.set_parameter_file(config_path) == false) return EXIT_FAILURE;

    const int width = (int)cfg.get<float>("camera.width");
    const int height = (int)cfg.get<float>("camera.height");
    const float depth_scale = cfg.get<float>("depth_scale");
    const std::string store_path = cfg.get<std::string>("mesh_store.path");
    const std::string sequence = arg(argc, argv, "--sequence", "");

    try {
        cuphoto::TSDFSurface tsdf(cfg);
        if (sequence.empty()) {
            std::vector<char> raw;
            if (!read_file(arg(argc, argv, "--depth", "depth.u16"), raw) || raw.size() != (size_t)width * height * 2)
                throw cuphoto::CuPhotoException("depth frame missing or not camera.width x camera.height uint16");
            std::vector<float> depth_m((size_t)width * height);
            const uint16_t* px = reinterpret_cast<const uint16_t*>(raw.data());
            for (size_t i = 0; i < depth_m.size(); ++i) depth_m[i] = (float)px[i] * depth_scale;
            cv::cuda::GpuMat depth(height, width, CV_32F), rgb(height, width, CV_8UC3);
            if (depth.empty() || rgb.empty() || !depth.upload(depth_m.data()))
                throw cuphoto::CuPhotoException("cannot upload the frame");
            cudaMemset2D(rgb.data, rgb.step, 0, (size_t)width * 3, (size_t)height);
            const std::array<double, 7> pose = tsdf.global_pose();
            std::printf("pose %.17g %.17g %.17g %.17g %.17g %.17g %.17g\n", pose[0], pose[1], pose[2], pose[3],
                        pose[4], pose[5], pose[6]);
            if (flag(argc, argv, "--points")) {
                const double fx = cfg.get<float>("camera.fx"), fy = cfg.get<float>("camera.fy");
                const double cx = cfg.get<float>("camera.cx"), cy = cfg.get<float>("camera.cy");
                // cx, cy at both places the cloud reads them (column- and row-major)
                const std::array<double, 9> K{fx, 0, cx, 0, fy, cy, cx, cy, 1};
                auto cloud = cuphoto::cudaPointCloud::create(K, (size_t)width * height);
                const cuphoto::SE3 inv = tsdf.get_global_transformation().inverse();
                const cuphoto::Quat q(inv.rotationMatrix());
                const cuphoto::Vec3 t = inv.translation();
                const std::array<double, 7> to_world{q.w(), q.x(), q.y(), q.z(), t.x(), t.y(), t.z()};
                if (!cloud->extract_points(depth, cv::cuda::PtrStepb(), to_world, 0))
                    throw cuphoto::CuPhotoException("extract_points failed");
                const std::string ply = arg(argc, argv, "--points_ply", "");
                if (!ply.empty() && !cloud->save_ply(ply)) throw cuphoto::CuPhotoException("save_ply failed");
                std::printf("points %llu\n", (unsigned long long)cloud->get_num_points());
                tsdf.reconstruct_surface(cloud);
            } else {
                tsdf.reconstruct_surface(rgb, depth);
            }
        } else {
            const int n = std::atoi(arg(argc, argv, "--frames", "1").c_str());
            const int per_pass = std::atoi(arg(argc, argv, "--per_pass", "16").c_str());
            std::vector<char> raw, poses;
            if (!read_file(sequence, raw) || raw.size() != (size_t)n * width * height * 2 ||
                !read_file(arg(argc, argv, "--poses", "poses.f64"), poses) || poses.size() != (size_t)n * 7 * 8)
                throw cuphoto::CuPhotoException("sequence or poses missing or of the wrong size");
            void* d = nullptr;
            if (cudaMalloc(&d, raw.size()) != cudaSuccess || cudaMemcpy(d, raw.data(), raw.size(), cudaMemcpyHostToDevice) != cudaSuccess)
                throw cuphoto::CuPhotoException("cannot upload the sequence");
            std::vector<gbt_frame> frames(n);
            const double* p = reinterpret_cast<const double*>(poses.data());
            for (int k = 0; k < n; ++k) {
                gbt_frame& f = frames[k];
                std::memset(&f, 0, sizeof(f));
                f.depth = static_cast<char*>(d) + (size_t)k * width * height * 2;
                f.pitch_bytes = (size_t)width * 2;
                f.width = width;
                f.height = height;
                f.format = GBT_DEPTH_U16;
                f.depth_scale = depth_scale;
                for (int j = 0; j < 7; ++j) f.pose[j] = p[7 * k + j];
            }
            tsdf.reconstruct_sequence(frames, per_pass, arg(argc, argv, "--resume_volume", ""),
                                      arg(argc, argv, "--save_volume", ""));
            cudaFree(d);
        }
        const auto mesh = tsdf.get_mesh();
        mesh.store_to_ply(store_path);
        std::printf("vertices %zu triangles %zu -> %s\n", mesh.vertices().size(), mesh.polygons().size(),
                    store_path.c_str());
    } catch (cuphoto::CuPhotoException& e) {
        std::fprintf(stderr, "%s\n", e.what());
        return EXIT_FAILURE;
    } catch (std::exception& e) {
        std::fprintf(stderr, "%s\n", e.what());
        return EXIT_FAILURE;
    } catch (...) {
        return EXIT_FAILURE;
    }
    return EXIT_SUCCESS;
}
