// Minimal stand-in for the host image type the reference's point-cloud
// source names (cv::Mat and its small helpers), so that its CUDA kernels can
// be compiled here for the parity checks, and so that its host z-buffer loop
// (cudaPointCloud::project_to_color_depth) can run in the host-loop harness
// (oracle/ref_project_main.cu).  A Mat is a dense row-major buffer; setTo
// fills it; when a Mat is destroyed its size and contents are appended to
// cv::shim_captured(), which is how the harness reads the images the loop
// built (the loop hands them to cudaMemcpy, which has no device here).
// OpenCV itself is not installed in this build environment.
#pragma once
#include <cstddef>
#include <cstdint>
#include <cstring>
#include <vector>

#include "cuda/common.hpp"

#define CV_8UC3 16
#define CV_32F 5

namespace cv {

struct Size {
    int width, height;
    Size(int w, int h) : width(w), height(h) {}
};

struct Point {
    int x, y;
    Point(int x_, int y_) : x(x_), y(y_) {}
};

struct Scalar {
    double v[4];
    Scalar(double a = 0, double b = 0, double c = 0, double d = 0) : v{a, b, c, d} {}
};

template <typename T, int n> struct Vec {
    T val[n];
    Vec() : val{} {}
    Vec(T a, T b, T c) : val{a, b, c} {}
};
typedef Vec<unsigned char, 3> Vec3b;

// Images of the Mats destroyed so far (see the header comment).
struct ShimImage {
    int rows, cols, elem;
    std::vector<unsigned char> data;
};
inline std::vector<ShimImage>& shim_captured() {
    static std::vector<ShimImage> v;
    return v;
}

class Mat {
public:
    Mat(Size s, int type) : rows(s.height), cols(s.width), elem(type == CV_8UC3 ? 3 : 4),
                            buf((size_t)s.width * s.height * (type == CV_8UC3 ? 3 : 4)) {}
    ~Mat() { shim_captured().push_back(ShimImage{rows, cols, elem, buf}); }
    Mat(const Mat&) = delete;
    Mat& operator=(const Mat&) = delete;
    // a single-channel float image: every element = v
    void setTo(double v) {
        const float f = (float)v;
        for (size_t i = 0; i + 4 <= buf.size(); i += 4) std::memcpy(&buf[i], &f, 4);
    }
    // a three-channel 8-bit image: every pixel = the scalar's first three values
    void setTo(const Scalar& s) {
        for (size_t i = 0; i + 3 <= buf.size(); i += 3)
            for (int c = 0; c < 3; ++c) buf[i + c] = (unsigned char)s.v[c];
    }
    template <typename T> T& at(int y, int x) { return *reinterpret_cast<T*>(&buf[((size_t)y * cols + x) * elem]); }
    template <typename T> T& at(Point p) { return at<T>(p.y, p.x); }
    template <typename T> T* ptr() { return reinterpret_cast<T*>(buf.data()); }
    int rows, cols;

private:
    int elem;
    std::vector<unsigned char> buf;
};

}  // namespace cv
