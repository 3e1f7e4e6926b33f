// Minimal stand-in for the two OpenCV CUDA image-view types that the
// reference's TSDF headers name (cv::cuda::PtrStep / PtrStepSz).  Only what
// those headers use is declared: a device pointer, a row pitch in bytes and
// the image size.  OpenCV itself is not installed in this build environment.
#pragma once
#include <cstddef>
#include <cuda_runtime.h>

namespace cv {
namespace cuda {

template <typename T> struct DevPtr {
    T* data;
    __host__ __device__ DevPtr() : data(0) {}
    __host__ __device__ DevPtr(T* p) : data(p) {}
    __host__ __device__ operator T*() { return data; }
    __host__ __device__ operator const T*() const { return data; }
};

template <typename T> struct PtrStep : public DevPtr<T> {
    size_t step;
    __host__ __device__ PtrStep() : step(0) {}
    __host__ __device__ PtrStep(T* p, size_t s) : DevPtr<T>(p), step(s) {}
    __host__ __device__ T* ptr(int y = 0) { return (T*)((char*)DevPtr<T>::data + y * step); }
    __host__ __device__ const T* ptr(int y = 0) const {
        return (const T*)((const char*)DevPtr<T>::data + y * step);
    }
};

template <typename T> struct PtrStepSz : public PtrStep<T> {
    int cols;
    int rows;
    __host__ __device__ PtrStepSz() : cols(0), rows(0) {}
    __host__ __device__ PtrStepSz(int r, int c, T* p, size_t s) : PtrStep<T>(p, s), cols(c), rows(r) {}
};

typedef PtrStepSz<unsigned char> PtrStepSzb;
typedef PtrStepSz<float> PtrStepSzf;
typedef PtrStep<unsigned char> PtrStepb;
typedef PtrStep<float> PtrStepf;

}  // namespace cuda
}  // namespace cv
