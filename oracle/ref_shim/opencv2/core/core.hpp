// Minimal stand-in for the host image type the reference's point-cloud
// source names (cv::Mat and its small helpers), so that its CUDA kernels can
// be compiled here for the parity checks.  Only the device code of that file
// is used; these declarations exist so that its host functions parse.  OpenCV
// itself is not installed in this build environment.
#pragma once
#include <cstddef>
#include <cstdint>
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

class Mat {
public:
    Mat(Size s, int type) : rows(s.height), cols(s.width), elem(type == CV_8UC3 ? 3 : 4),
                            buf((size_t)s.width * s.height * (type == CV_8UC3 ? 3 : 4)) {}
    template <typename T> void setTo(T) {}
    template <typename T> T& at(int y, int x) { return *reinterpret_cast<T*>(&buf[((size_t)y * cols + x) * elem]); }
    template <typename T> T& at(Point p) { return at<T>(p.y, p.x); }
    template <typename T> T* ptr() { return reinterpret_cast<T*>(buf.data()); }
    int rows, cols;

private:
    int elem;
    std::vector<unsigned char> buf;
};

}  // namespace cv
