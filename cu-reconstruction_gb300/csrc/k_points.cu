// Point clouds: depth back-projection, rigid transform, z-buffer projection
// and the image filter of the reference's cudaPointCloud
// (cuda_point_cloud.cu:22-385), as GPU kernels behind the C ABI.
//
// Arithmetic follows the reference where it is defined by its code:
//   back-projection  ((float)x - cx) * d / fx in double, rounded to float
//                    (cuda_point_cloud.cu:44-56, K is double there);
//   pose             float quaternion + translation (make_float4(T[1], T[2],
//                    T[3], T[0])); in the kernels the reference runs on the
//                    GPU (extraction, transform) R*p + t in its device
//                    build's rounding order (compat_geom.cuh); in the
//                    projection, which the reference runs as a host loop,
//                    in its host build's order: every product and sum
//                    rounded on its own, left to right (single precision,
//                    no fused multiply-add, as g++ -O3 compiles se3.cuh for
//                    x86-64), checked against that loop itself;
//   pixel            (int)((x * fx) / z + cx) in float, IEEE divide (the
//                    reference's host loop, cuda_point_cloud.cu:262-266).
// The z-buffer, a sequential host loop in the reference, becomes a 64-bit
// atomic minimum per pixel over (order-preserving bits of z, point index):
// the smallest z wins, and among equal z the lowest index, which is the
// point the loop's strict "depth_val > z" test keeps.
#include <cfloat>
#include <cstdint>
#include <cstdio>
#include <cstring>

#include <cuda_runtime.h>

#include "compat_geom.cuh"
#include "gbt_internal.h"

namespace gbt {
namespace points {

constexpr int kThreads = 256;
constexpr int kPointBytes = (int)sizeof(gbt_point);   // 33, packed
static_assert(sizeof(gbt_point) == 33, "gbt_point must be the reference's packed 33-byte vertex");

struct Pose {
    float q[4];   // qx, qy, qz, qw
    float t[3];
};

Pose make_pose(const double* p) {
    Pose r;
    r.q[0] = (float)p[1];
    r.q[1] = (float)p[2];
    r.q[2] = (float)p[3];
    r.q[3] = (float)p[0];
    r.t[0] = (float)p[4];
    r.t[1] = (float)p[5];
    r.t[2] = (float)p[6];
    return r;
}

__device__ __forceinline__ void apply_pose(const Pose& P, float x, float y, float z, float* out) {
    float R[9];
    compat_rotation(P.q, R);
    out[0] = compat_cam(R[0], R[1], R[2], P.t[0], x, y, z);
    out[1] = compat_cam(R[3], R[4], R[5], P.t[1], x, y, z);
    out[2] = compat_cam(R[6], R[7], R[8], P.t[2], x, y, z);
}

// The pose as the reference's host build applies it (SE3<float> from the
// quaternion, se3.cuh:42-61,124-140, then rotate + translate, :82-95): the
// rotation is built on the host in single precision (this file is compiled
// with -ffp-contract=off, so each product and sum is rounded on its own),
// and each row is ((r0 x + r1 y) + r2 z) + t with every operation rounded.
struct HostPose {
    float R[9];
    float t[3];
};

HostPose make_host_pose(const double* p) {
    const float qx = (float)p[1], qy = (float)p[2], qz = (float)p[3], qw = (float)p[0];
    const float x = 2 * qx, y = 2 * qy, z = 2 * qz;
    const float wx = x * qw, wy = y * qw, wz = z * qw;
    const float xx = x * qx, xy = y * qx, xz = z * qx;
    const float yy = y * qy, yz = z * qy, zz = z * qz;
    HostPose h;
    h.R[0] = 1 - (yy + zz);
    h.R[1] = xy - wz;
    h.R[2] = xz + wy;
    h.R[3] = xy + wz;
    h.R[4] = 1 - (xx + zz);
    h.R[5] = yz - wx;
    h.R[6] = xz - wy;
    h.R[7] = yz + wx;
    h.R[8] = 1 - (xx + yy);
    h.t[0] = (float)p[4];
    h.t[1] = (float)p[5];
    h.t[2] = (float)p[6];
    return h;
}

__device__ __forceinline__ float host_row(const float* r, float t, float x, float y, float z) {
    return __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(r[0], x), __fmul_rn(r[1], y)), __fmul_rn(r[2], z)), t);
}

// Order-preserving map of a (non-NaN) float onto unsigned integers.
__device__ __forceinline__ uint32_t ordered(float f) {
    const uint32_t b = __float_as_uint(f);
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
__device__ __forceinline__ float unordered(uint32_t k) {
    return __uint_as_float((k & 0x80000000u) ? (k & 0x7fffffffu) : ~k);
}

struct ExtractArgs {
    const char* depth;
    int64_t depth_pitch;
    int fmt;
    float scale;
    const unsigned char* color;
    int64_t color_pitch;
    int width, height;
    double fx, fy, cx, cy;
    Pose pose;
    int64_t start;
    unsigned char* points;
};

// One warp per 32 consecutive pixels (row-major): the points are built in
// shared memory and the warp writes the span of 32 x 33 bytes byte-coalesced,
// skipping the bytes of pixels without depth (their slots stay as they were).
__global__ void __launch_bounds__(kThreads) extract_kernel(const __grid_constant__ ExtractArgs a) {
    __shared__ unsigned char s_pts[kThreads / 32][32 * kPointBytes];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int64_t npix = (int64_t)a.width * a.height;
    const int64_t p = (int64_t)blockIdx.x * kThreads + threadIdx.x;
    bool valid = false;
    if (p < npix) {
        const int y = (int)(p / a.width), x = (int)(p - (int64_t)y * a.width);
        const char* row = a.depth + (int64_t)y * a.depth_pitch;
        const float d = a.fmt == GBT_DEPTH_U16
                            ? __fmul_rn((float)reinterpret_cast<const unsigned short*>(row)[x], a.scale)
                            : reinterpret_cast<const float*>(row)[x];
        if (!(d <= 0.0f)) {   // cuda_point_cloud.cu:58: "depth <= 0" is skipped, NaN is not
            valid = true;
            const double dd = (double)d;
            const float bx = __double2float_rn(__ddiv_rn(__dmul_rn(__dsub_rn((double)(float)x, a.cx), dd), a.fx));
            const float by = __double2float_rn(__ddiv_rn(__dmul_rn(__dsub_rn((double)(float)y, a.cy), dd), a.fy));
            float w[3];
            apply_pose(a.pose, bx, by, d, w);
            unsigned char rgb[3] = {255, 255, 255};
            if (a.color) {
                const unsigned char* c = a.color + (int64_t)y * a.color_pitch + 3 * (int64_t)x;
                rgb[0] = c[0];
                rgb[1] = c[1];
                rgb[2] = c[2];
            }
            unsigned char* dst = s_pts[warp] + lane * kPointBytes;
            const float f[7] = {w[0], w[1], w[2], 0.f, 0.f, 0.f, 0.f};
            memcpy(dst, f, 28);
            dst[28] = rgb[0];
            dst[29] = rgb[1];
            dst[30] = rgb[2];
            dst[31] = 0;
            dst[32] = 0;
        }
    }
    const unsigned mask = __ballot_sync(0xffffffffu, valid);
    __syncwarp();
    if (!mask) return;
    const int64_t first = (int64_t)blockIdx.x * kThreads + warp * 32;
    unsigned char* out = a.points + (a.start + first) * kPointBytes;
#pragma unroll 1
    for (int b = lane; b < 32 * kPointBytes; b += 32) {
        const int pt = b / kPointBytes;
        if ((mask >> pt) & 1u) out[b] = s_pts[warp][b];
    }
}

__global__ void __launch_bounds__(kThreads) transform_kernel(unsigned char* points, int64_t n, Pose P) {
    const int64_t i = (int64_t)blockIdx.x * kThreads + threadIdx.x;
    if (i >= n) return;
    unsigned char* pt = points + i * kPointBytes;
    float v[3];
    memcpy(v, pt, 12);
    float w[3];
    apply_pose(P, v[0], v[1], v[2], w);
    memcpy(pt, w, 12);
}

struct ProjectArgs {
    const unsigned char* points;
    int64_t n;
    float fx, fy, cx, cy;
    HostPose pose;
    int width, height;
    unsigned long long* keys;
};

__global__ void __launch_bounds__(kThreads) zbuffer_kernel(const __grid_constant__ ProjectArgs a) {
    const int64_t i = (int64_t)blockIdx.x * kThreads + threadIdx.x;
    if (i >= a.n) return;
    float v[3];
    memcpy(v, a.points + i * kPointBytes, 12);
    float c[3];
    c[0] = host_row(a.pose.R + 0, a.pose.t[0], v[0], v[1], v[2]);
    c[1] = host_row(a.pose.R + 3, a.pose.t[1], v[0], v[1], v[2]);
    c[2] = host_row(a.pose.R + 6, a.pose.t[2], v[0], v[1], v[2]);
    if (c[2] == 0.f) return;
    // a point only enters a pixel whose depth (FLT_MAX at first) exceeds its z
    if (!(c[2] < FLT_MAX)) return;
    const float fu = __fadd_rn(__fdiv_rn(__fmul_rn(c[0], a.fx), c[2]), a.cx);
    const float fv = __fadd_rn(__fdiv_rn(__fmul_rn(c[1], a.fy), c[2]), a.cy);
    if (fu != fu || fv != fv) return;   // non-finite coordinates are dropped
    const int u = __float2int_rz(fu), vv = __float2int_rz(fv);   // truncation, saturating
    if (u < 0 || u >= a.width || vv < 0 || vv >= a.height) return;
    const unsigned long long key = ((unsigned long long)ordered(c[2]) << 32) | (unsigned long long)(uint32_t)i;
    atomicMin(a.keys + (int64_t)vv * a.width + u, key);
}

struct ResolveArgs {
    const unsigned char* points;
    const unsigned long long* keys;
    int width, height;
    char* depth;
    int64_t depth_pitch;
    unsigned char* color;
    int64_t color_pitch;
};

__global__ void __launch_bounds__(kThreads) resolve_kernel(const __grid_constant__ ResolveArgs a) {
    const int64_t p = (int64_t)blockIdx.x * kThreads + threadIdx.x;
    if (p >= (int64_t)a.width * a.height) return;
    const int y = (int)(p / a.width), x = (int)(p - (int64_t)y * a.width);
    const unsigned long long key = a.keys[p];
    float z = 0.f;   // filter_image_if(FLT_MAX -> 0) of the untouched pixels
    unsigned char rgb[3] = {0, 0, 0};
    if (key != ~0ull) {
        z = unordered((uint32_t)(key >> 32));
        const unsigned char* src = a.points + (int64_t)(key & 0xffffffffull) * kPointBytes + 28;
        rgb[0] = src[0];
        rgb[1] = src[1];
        rgb[2] = src[2];
    }
    reinterpret_cast<float*>(a.depth + (int64_t)y * a.depth_pitch)[x] = z;
    if (a.color) {
        unsigned char* c = a.color + (int64_t)y * a.color_pitch + 3 * (int64_t)x;
        c[0] = rgb[0];
        c[1] = rgb[1];
        c[2] = rgb[2];
    }
}

__global__ void __launch_bounds__(kThreads) filter_kernel(char* img, int64_t pitch, int width, int height,
                                                          float filter_value, float set_value) {
    const int64_t p = (int64_t)blockIdx.x * kThreads + threadIdx.x;
    if (p >= (int64_t)width * height) return;
    const int y = (int)(p / width), x = (int)(p - (int64_t)y * width);
    float* px = reinterpret_cast<float*>(img + (int64_t)y * pitch) + x;
    // near_equal (util.cu:8-10) with EPSILON = 1e-10f (util.cu:6)
    if (fabsf(__fsub_rn(*px, filter_value)) < 1e-10f) *px = set_value;
}

unsigned blocks_for(int64_t n) { return (unsigned)((n + kThreads - 1) / kThreads); }

gbt_status fail(gbt_status st, const char* fn, const char* msg) {
    char buf[256];
    std::snprintf(buf, sizeof(buf), "%s: %s", fn, msg);
    set_last_error(buf);
    return st;
}

gbt_status cuda_status(const char* fn) {
    const cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) return GBT_OK;
    char buf[256];
    std::snprintf(buf, sizeof(buf), "%s: %s", fn, cudaGetErrorString(e));
    set_last_error(buf);
    return GBT_ERR_CUDA;
}

}  // namespace points
}  // namespace gbt

using namespace gbt::points;

extern "C" {

gbt_status gbt_points_extract(const double camera_matrix[9], const void* depth, int64_t depth_pitch_bytes,
                              int32_t depth_format, float depth_scale, const uint8_t* color_rgb8,
                              int64_t color_pitch_bytes, int32_t width, int32_t height, const double pose[7],
                              int64_t start_index, gbt_point* points, int64_t capacity, void* stream) {
    gbt::TraceRange trace_("gbt_points_extract");
    const char* fn = "gbt_points_extract";
    if (!camera_matrix || !depth || !pose || !points) return fail(GBT_ERR_INVALID_ARG, fn, "NULL argument");
    if (width <= 0 || height <= 0) return fail(GBT_ERR_INVALID_ARG, fn, "depth width/height parameters are zero");
    if (depth_format != GBT_DEPTH_F32_M && depth_format != GBT_DEPTH_U16)
        return fail(GBT_ERR_INVALID_ARG, fn, "unknown depth format");
    const int64_t elem = depth_format == GBT_DEPTH_U16 ? 2 : 4;
    if (depth_pitch_bytes < elem * width) return fail(GBT_ERR_INVALID_ARG, fn, "depth pitch below the row size");
    if ((reinterpret_cast<uintptr_t>(depth) | (uintptr_t)depth_pitch_bytes) % (uintptr_t)elem != 0)
        return fail(GBT_ERR_INVALID_ARG, fn, "depth pointer or pitch not aligned to its element size");
    if (color_rgb8 && color_pitch_bytes < 3 * (int64_t)width)
        return fail(GBT_ERR_INVALID_ARG, fn, "colour pitch below the row size");
    if (start_index < 0 || capacity < 0) return fail(GBT_ERR_INVALID_ARG, fn, "negative start index or capacity");
    const int64_t npix = (int64_t)width * height;
    if (npix > (int64_t)0xffffffffll) return fail(GBT_ERR_INVALID_ARG, fn, "image larger than 2^32-1 pixels");
    if (start_index > capacity - npix)
        return fail(GBT_ERR_CAPACITY, fn, "start_index + width*height exceeds the cloud's capacity");
    if (!(camera_matrix[0] != 0.0) || !(camera_matrix[4] != 0.0))
        return fail(GBT_ERR_INVALID_ARG, fn, "focal lengths must be non-zero");
    ExtractArgs a;
    a.depth = static_cast<const char*>(depth);
    a.depth_pitch = depth_pitch_bytes;
    a.fmt = depth_format;
    a.scale = depth_scale;
    a.color = color_rgb8;
    a.color_pitch = color_pitch_bytes;
    a.width = width;
    a.height = height;
    a.fx = camera_matrix[0];
    a.fy = camera_matrix[4];
    a.cx = camera_matrix[6];
    a.cy = camera_matrix[7];
    a.pose = make_pose(pose);
    a.start = start_index;
    a.points = reinterpret_cast<unsigned char*>(points);
    cudaGetLastError();
    extract_kernel<<<blocks_for(npix), kThreads, 0, static_cast<cudaStream_t>(stream)>>>(a);
    return cuda_status(fn);
}

gbt_status gbt_points_transform(gbt_point* points, int64_t n, const double pose[7], void* stream) {
    gbt::TraceRange trace_("gbt_points_transform");
    const char* fn = "gbt_points_transform";
    if (!pose || (n > 0 && !points)) return fail(GBT_ERR_INVALID_ARG, fn, "NULL argument");
    if (n <= 0) return fail(GBT_ERR_INVALID_ARG, fn, "the number of points is 0");
    if (n > (int64_t)0xffffffffll) return fail(GBT_ERR_INVALID_ARG, fn, "point count above 2^32-1");
    cudaGetLastError();
    transform_kernel<<<blocks_for(n), kThreads, 0, static_cast<cudaStream_t>(stream)>>>(
        reinterpret_cast<unsigned char*>(points), n, make_pose(pose));
    return cuda_status(fn);
}

gbt_status gbt_points_project(const gbt_point* points, int64_t n, const double camera_matrix[9], const double pose[7],
                              float* depth, int64_t depth_pitch_bytes, uint8_t* color_rgb8, int64_t color_pitch_bytes,
                              int32_t width, int32_t height, void* scratch, void* stream) {
    gbt::TraceRange trace_("gbt_points_project");
    const char* fn = "gbt_points_project";
    if (!camera_matrix || !pose || !depth || !scratch || (n > 0 && !points))
        return fail(GBT_ERR_INVALID_ARG, fn, "NULL argument");
    if (width <= 0 || height <= 0) return fail(GBT_ERR_INVALID_ARG, fn, "depth width/height parameters are zero");
    if (n < 0 || n > (int64_t)0xffffffffll) return fail(GBT_ERR_INVALID_ARG, fn, "point count outside 0..2^32-1");
    if (depth_pitch_bytes < 4 * (int64_t)width) return fail(GBT_ERR_INVALID_ARG, fn, "depth pitch below the row size");
    if ((reinterpret_cast<uintptr_t>(depth) | (uintptr_t)depth_pitch_bytes) % 4u != 0)
        return fail(GBT_ERR_INVALID_ARG, fn, "depth pointer or pitch not 4-byte aligned");
    if (color_rgb8 && color_pitch_bytes < 3 * (int64_t)width)
        return fail(GBT_ERR_INVALID_ARG, fn, "colour pitch below the row size");
    if ((reinterpret_cast<uintptr_t>(scratch) & 7u) != 0) return fail(GBT_ERR_INVALID_ARG, fn, "scratch not 8-byte aligned");
    const int64_t npix = (int64_t)width * height;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    cudaGetLastError();
    cudaError_t e = cudaMemsetAsync(scratch, 0xff, (size_t)npix * 8, st);
    if (e != cudaSuccess) return cuda_status(fn);
    ProjectArgs p;
    p.points = reinterpret_cast<const unsigned char*>(points);
    p.n = n;
    p.fx = (float)camera_matrix[0];
    p.fy = (float)camera_matrix[4];
    p.cx = (float)camera_matrix[2];
    p.cy = (float)camera_matrix[5];
    p.pose = make_host_pose(pose);
    p.width = width;
    p.height = height;
    p.keys = static_cast<unsigned long long*>(scratch);
    if (n > 0) zbuffer_kernel<<<blocks_for(n), kThreads, 0, st>>>(p);
    ResolveArgs r;
    r.points = p.points;
    r.keys = p.keys;
    r.width = width;
    r.height = height;
    r.depth = reinterpret_cast<char*>(depth);
    r.depth_pitch = depth_pitch_bytes;
    r.color = color_rgb8;
    r.color_pitch = color_pitch_bytes;
    resolve_kernel<<<blocks_for(npix), kThreads, 0, st>>>(r);
    return cuda_status(fn);
}

gbt_status gbt_image_filter_if(float* image, int64_t pitch_bytes, int32_t width, int32_t height, float filter_value,
                               float set_value, void* stream) {
    gbt::TraceRange trace_("gbt_image_filter_if");
    const char* fn = "gbt_image_filter_if";
    if (!image) return fail(GBT_ERR_INVALID_ARG, fn, "NULL image");
    if (width <= 0 || height <= 0) return fail(GBT_ERR_INVALID_ARG, fn, "width/height are zero");
    if (pitch_bytes < 4 * (int64_t)width) return fail(GBT_ERR_INVALID_ARG, fn, "pitch below the row size");
    if ((reinterpret_cast<uintptr_t>(image) | (uintptr_t)pitch_bytes) % 4u != 0)
        return fail(GBT_ERR_INVALID_ARG, fn, "image pointer or pitch not 4-byte aligned");
    cudaGetLastError();
    filter_kernel<<<blocks_for((int64_t)width * height), kThreads, 0, static_cast<cudaStream_t>(stream)>>>(
        reinterpret_cast<char*>(image), pitch_bytes, width, height, filter_value, set_value);
    return cuda_status(fn);
}

}  // extern "C"
