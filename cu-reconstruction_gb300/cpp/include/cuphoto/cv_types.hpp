// Image views the TSDF API takes: OpenCV's own cv::cuda types when OpenCV is
// installed, otherwise minimal stand-ins with the same members
// (data, step, cols, rows, ptr(y)) and the GpuMat -> PtrStepSz conversion the
// reference relies on (tsdf_surface_reconstruction.cpp:134).
#ifndef CUPHOTO_GB300_CV_TYPES_HPP
#define CUPHOTO_GB300_CV_TYPES_HPP

#include <cstddef>
#include <cuda_runtime.h>

#if __has_include(<opencv2/core/cuda.hpp>) && !defined(CUPHOTO_GB300_NO_OPENCV)
#include <opencv2/core/cuda.hpp>
#define CUPHOTO_GB300_HAVE_OPENCV 1
#else
#define CUPHOTO_GB300_HAVE_OPENCV 0

#define CV_8UC3 16
#define CV_32F 5
#define CV_16U 2

namespace cv {
namespace cuda {

template <typename T> struct DevPtr {
    T* data;
    DevPtr() : data(nullptr) {}
    DevPtr(T* p) : data(p) {}
    operator T*() { return data; }
    operator const T*() const { return data; }
};

template <typename T> struct PtrStep : public DevPtr<T> {
    size_t step;
    PtrStep() : step(0) {}
    PtrStep(T* p, size_t s) : DevPtr<T>(p), step(s) {}
    T* ptr(int y = 0) { return (T*)((char*)DevPtr<T>::data + y * step); }
    const T* ptr(int y = 0) const { return (const T*)((const char*)DevPtr<T>::data + y * step); }
};

template <typename T> struct PtrStepSz : public PtrStep<T> {
    int cols;
    int rows;
    PtrStepSz() : cols(0), rows(0) {}
    PtrStepSz(int r, int c, T* p, size_t s) : PtrStep<T>(p, s), cols(c), rows(r) {}
};

typedef PtrStepSz<unsigned char> PtrStepSzb;
typedef PtrStepSz<float> PtrStepSzf;
typedef PtrStep<unsigned char> PtrStepb;

// Pitched device image owning its memory (the part of cv::cuda::GpuMat the
// TSDF path uses).
class GpuMat {
public:
    GpuMat() = default;
    GpuMat(int rows_, int cols_, int type_) { create(rows_, cols_, type_); }
    GpuMat(const GpuMat&) = delete;
    GpuMat& operator=(const GpuMat&) = delete;
    GpuMat(GpuMat&& o) noexcept { *this = static_cast<GpuMat&&>(o); }
    GpuMat& operator=(GpuMat&& o) noexcept {
        release();
        data = o.data; step = o.step; rows = o.rows; cols = o.cols; type_ = o.type_;
        o.data = nullptr; o.rows = o.cols = 0; o.step = 0;
        return *this;
    }
    ~GpuMat() { release(); }

    void create(int rows_, int cols_, int type) {
        release();
        rows = rows_;
        cols = cols_;
        type_ = type;
        void* p = nullptr;
        if (rows > 0 && cols > 0 && cudaMallocPitch(&p, &step, (size_t)cols * elemSize(), (size_t)rows) == cudaSuccess)
            data = static_cast<unsigned char*>(p);
        else
            rows = cols = 0;
    }
    void release() {
        if (data) cudaFree(data);
        data = nullptr;
        rows = cols = 0;
        step = 0;
    }
    // copies a tightly packed host image of this size and type
    bool upload(const void* host) {
        return data && cudaMemcpy2D(data, step, host, (size_t)cols * elemSize(), (size_t)cols * elemSize(),
                                    (size_t)rows, cudaMemcpyHostToDevice) == cudaSuccess;
    }
    size_t elemSize() const { return type_ == CV_8UC3 ? 3 : type_ == CV_16U ? 2 : 4; }
    bool empty() const { return data == nullptr; }
    int type() const { return type_; }

    template <typename T> operator PtrStepSz<T>() const { return PtrStepSz<T>(rows, cols, (T*)data, step); }
    template <typename T> operator PtrStep<T>() const { return PtrStep<T>((T*)data, step); }

    unsigned char* data = nullptr;
    size_t step = 0;
    int rows = 0;
    int cols = 0;

private:
    int type_ = CV_32F;
};

}  // namespace cuda
}  // namespace cv
#endif

#endif
