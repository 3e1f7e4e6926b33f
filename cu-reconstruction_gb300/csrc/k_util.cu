// Volume initialisation and the packed per-voxel transform records.
#include <cstdint>
#include <cuda_runtime.h>

#include "gbt_internal.h"

namespace gbt {

// setup_data (tsdf_volume.cu:227-242): distance = truncation, weight = 0.
__global__ void volume_init_kernel(float4* D, float4* W, int64_t n4, float trunc) {
    const float4 d = make_float4(trunc, trunc, trunc, trunc);
    const float4 z = make_float4(0.f, 0.f, 0.f, 0.f);
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n4; i += (int64_t)gridDim.x * blockDim.x) {
        D[i] = d;
        W[i] = z;
    }
}

__global__ void volume_init_tail_kernel(float* D, float* W, int64_t begin, int64_t n, float trunc) {
    const int64_t i = begin + threadIdx.x;
    if (i < n) {
        D[i] = trunc;
        W[i] = 0.f;
    }
}

cudaError_t launch_volume_init(float* D, float* W, int64_t n, float trunc, cudaStream_t s) {
    const int64_t n4 = n / 4;
    if (n4 > 0) {
        int dev = 0, sms = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        int64_t grid = (n4 + 255) / 256;
        if (grid > (int64_t)sms * 8) grid = (int64_t)sms * 8;
        volume_init_kernel<<<(int)grid, 256, 0, s>>>(reinterpret_cast<float4*>(D), reinterpret_cast<float4*>(W), n4,
                                                     trunc);
    }
    if (n4 * 4 < n) volume_init_tail_kernel<<<1, 4, 0, s>>>(D, W, n4 * 4, n, trunc);
    return cudaGetLastError();
}

// init_voxel_transofrmation (tsdf_volume.cu:106-127): per voxel a packed
// {float3 centre, float4 quaternion (x, y, z, w) = (0, 0, 0, 1)}, 28 bytes.
// The centre is computed as the integrate and mesh kernels compute it.
__global__ void tvoxels_kernel(float* out, VolDesc v) {
    const int64_t n = (int64_t)v.nx * v.ny * v.nz;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t x = i % v.nx, r = i / v.nx;
        const int64_t y = r % v.ny, z = r / v.ny;
        float* o = out + 7 * i;
        o[0] = __fmaf_rn(__fadd_rn((float)x, 0.5f), v.vs[0], v.off[0]);
        o[1] = __fmaf_rn(__fadd_rn((float)y, 0.5f), v.vs[1], v.off[1]);
        o[2] = __fmaf_rn(__fadd_rn((float)z, 0.5f), v.vs[2], v.off[2]);
        o[3] = 0.f;
        o[4] = 0.f;
        o[5] = 0.f;
        o[6] = 1.f;
    }
}

cudaError_t launch_tvoxels(void* out, const VolDesc& v, cudaStream_t s) {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    tvoxels_kernel<<<sms * 8, 256, 0, s>>>(static_cast<float*>(out), v);
    return cudaGetLastError();
}

}  // namespace gbt
