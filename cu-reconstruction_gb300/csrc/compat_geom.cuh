// The reference's pose arithmetic (SE3<float> built from a quaternion and
// applied as R*p + t), shared by the TSDF kernels and the point-cloud kernels.
//
// The rotation entries and the R*p+t rows are written with explicit
// intrinsics, in the rounding order of the reference's own build of
// se3.cuh:42-61,124-140 (nvcc contracts its products into fused multiply-adds):
// every entry fuses its first product except R00 = 1-(yy+zz), which rounds
// both products; each row is fma(r2, z, fma(r0, x, r1*y)) + t.  That order was
// measured against the reference's kernels on 5.4M voxel projections (pixel
// index decoded from a coded depth image), where it is the only one of the
// tried orders without a single differing pixel.  Written with _rn intrinsics
// it rounds the same in every translation unit, fast-math or not.
#pragma once
#include <cuda_runtime.h>

namespace gbt {

// q = (qx, qy, qz, qw), the float4 the reference builds from a pose
// {qw, qx, qy, qz, ...} (tsdf_volume.cu:271, cuda_point_cloud.cu:205);
// R row-major.
__device__ __forceinline__ void compat_rotation(const float* q, float* R) {
    const float x = __fmul_rn(2.f, q[0]), y = __fmul_rn(2.f, q[1]), z = __fmul_rn(2.f, q[2]);
    const float wx = __fmul_rn(x, q[3]), wy = __fmul_rn(y, q[3]), wz = __fmul_rn(z, q[3]);
    const float xx = __fmul_rn(x, q[0]), yy = __fmul_rn(y, q[1]), zz = __fmul_rn(z, q[2]);
    R[0] = __fsub_rn(1.f, __fadd_rn(yy, zz));
    R[1] = __fmaf_rn(y, q[0], -wz);
    R[2] = __fmaf_rn(z, q[0], wy);
    R[3] = __fmaf_rn(y, q[0], wz);
    R[4] = __fsub_rn(1.f, __fmaf_rn(x, q[0], zz));
    R[5] = __fmaf_rn(z, q[1], -wx);
    R[6] = __fmaf_rn(z, q[0], -wy);
    R[7] = __fmaf_rn(z, q[1], wx);
    R[8] = __fsub_rn(1.f, __fmaf_rn(x, q[0], yy));
}

// One row of R*p + t.
__device__ __forceinline__ float compat_cam(float r0, float r1, float r2, float t, float px, float py, float pz) {
    return __fadd_rn(__fmaf_rn(r2, pz, __fmaf_rn(r0, px, __fmul_rn(r1, py))), t);
}

}  // namespace gbt
