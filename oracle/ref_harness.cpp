// Host driver for the reference's own TSDF kernels.
//
// TEST INFRASTRUCTURE ONLY.  The reference's kernels (cu_tsdf_integrate,
// set_array_to_value, init_voxel_transofrmation, marching_cubes_kernel) are
// loaded from oracle/_ref/ref_tsdf.cubin, compiled from the reference's
// sources by oracle/build.py.  Their host side is restated here, with the
// reference's launch shapes, allocations and synchronisation:
//
//   TSDFVolume::TSDFVolume / setup_data   tsdf_volume.cu:194-212,227-254
//   TSDFVolume::integrate                 tsdf_volume.cu:257-290
//   generate_triangular_surface           marching_cubes.cu:191-237
//   copy_data_mesh_to_host                marching_cubes.cu:159-189
//   cudaPointCloud::extract_points        cuda_point_cloud.cu:179-226
//   cudaPointCloud::transform             cuda_point_cloud.cu:356-385
//   filter_image_if launches              cuda_point_cloud.cu:273-278
//
// It is used to pin the CPU oracle and the engine against the reference's
// real GPU results, and to time the reference's integrate on the same GPU.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <map>
#include <sstream>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "opencv2/core/cuda/common.hpp"

namespace {

std::string g_err;
cudaLibrary_t g_lib = nullptr;
std::map<std::string, cudaKernel_t> g_k;

struct TransformationVoxel {
    float3 translation;
    float4 quat_rotation;
} __attribute__((packed));
static_assert(sizeof(TransformationVoxel) == 28, "packed record");

int fail(const char* what, cudaError_t e) {
    g_err = std::string(what) + ": " + cudaGetErrorString(e);
    return 1;
}

unsigned idiv_up(unsigned a, unsigned b) { return (a % b != 0) ? (a / b + 1) : (a / b); }

}  // namespace

struct ref_volume {
    dim3 grid;
    float3 phys, offset, vs;
    float max_weight, fx, fy, cx, cy;
    float trunc;
    float* D = nullptr;
    float* W = nullptr;
    TransformationVoxel* tv = nullptr;
    unsigned char* rgb = nullptr;
};

extern "C" {

const char* ref_last_error() { return g_err.c_str(); }

// Loads the cubin and looks its kernels up by the names in ref_kernels.txt.
int ref_load(const char* cubin_path, const char* names_path) {
    if (g_lib) return 0;
    std::ifstream nf(names_path);
    if (!nf) {
        g_err = std::string("cannot open ") + names_path;
        return 1;
    }
    cudaError_t e = cudaLibraryLoadFromFile(&g_lib, cubin_path, nullptr, nullptr, 0, nullptr, nullptr, 0);
    if (e != cudaSuccess) return fail("cudaLibraryLoadFromFile", e);
    std::string key, mangled;
    while (nf >> key >> mangled) {
        cudaKernel_t k;
        e = cudaLibraryGetKernel(&k, g_lib, mangled.c_str());
        if (e != cudaSuccess) return fail(("cudaLibraryGetKernel " + key).c_str(), e);
        g_k[key] = k;
    }
    for (const char* k : {"cu_tsdf_integrate", "set_array_to_value", "init_voxel_transofrmation", "marching_cubes_kernel"})
        if (!g_k.count(k)) {
            g_err = std::string("kernel missing: ") + k;
            return 1;
        }
    return 0;
}

int ref_volume_create(const uint32_t* grid, const float* phys, const float* offset, float max_weight, float fx,
                      float fy, float cx, float cy, ref_volume** out) {
    // The reference's integrate kernel guards its (y, z) threads with
    // `vy >= gy && vz >= gz` (tsdf_volume.cu:154): with y or z not a multiple
    // of its 8x8 block, threads past the grid run and access out of bounds.
    // Such grids are refused here, before anything reaches the GPU.
    if (grid[1] % 8 != 0 || grid[2] % 8 != 0 || grid[0] < 2 || grid[1] < 2 || grid[2] < 2) {
        g_err = "reference kernels need y and z grid sizes that are multiples of 8 (and every size >= 2)";
        return 1;
    }
    ref_volume* v = new ref_volume();
    v->grid = dim3(grid[0], grid[1], grid[2]);
    v->phys = make_float3(phys[0], phys[1], phys[2]);
    v->offset = make_float3(offset[0], offset[1], offset[2]);
    v->max_weight = max_weight;
    v->fx = fx;
    v->fy = fy;
    v->cx = cx;
    v->cy = cy;
    // tsdf_volume.cu:197-199 (cudaMath.cuh:1225 float3/dim3, :1530 length)
    v->vs = make_float3(v->phys.x / v->grid.x, v->phys.y / v->grid.y, v->phys.z / v->grid.z);
    const float dot = v->vs.x * v->vs.x + v->vs.y * v->vs.y + v->vs.z * v->vs.z;
    v->trunc = 1.1f * sqrtf(dot);
    const uint32_t n = v->grid.x * v->grid.y * v->grid.z;
    cudaError_t e = cudaMallocManaged(&v->D, n * sizeof(float), cudaMemAttachGlobal);
    if (e == cudaSuccess) e = cudaMallocManaged(&v->W, n * sizeof(float), cudaMemAttachGlobal);
    if (e == cudaSuccess) e = cudaMallocManaged(&v->tv, (size_t)n * sizeof(TransformationVoxel), cudaMemAttachGlobal);
    if (e == cudaSuccess) e = cudaMalloc(&v->rgb, 16);
    if (e != cudaSuccess) {
        delete v;
        return fail("allocation", e);
    }
    // setup_data, tsdf_volume.cu:227-254
    {
        dim3 block(64, 1, 1), g(idiv_up(n, 64), 1, 1);
        float* W = v->W;
        int size = (int)n;
        float zero = 0.f;
        void* a0[] = {&W, &size, &zero};
        e = cudaLaunchKernel((const void*)g_k["set_array_to_value"], g, block, a0, 0, 0);
        if (e != cudaSuccess) return fail("set_array_to_value", e);
        float* D = v->D;
        float tr = v->trunc;
        void* a1[] = {&D, &size, &tr};
        e = cudaLaunchKernel((const void*)g_k["set_array_to_value"], g, block, a1, 0, 0);
        if (e != cudaSuccess) return fail("set_array_to_value", e);
    }
    {
        dim3 block(1, 8, 8), g(1, idiv_up(v->grid.y, 8), idiv_up(v->grid.z, 8));
        TransformationVoxel* tv = v->tv;
        void* a[] = {&tv, &v->grid, &v->vs, &v->offset};
        e = cudaLaunchKernel((const void*)g_k["init_voxel_transofrmation"], g, block, a, 0, 0);
        if (e != cudaSuccess) return fail("init_voxel_transofrmation", e);
    }
    e = cudaDeviceSynchronize();
    if (e != cudaSuccess) return fail("setup_data", e);
    *out = v;
    return 0;
}

void ref_volume_destroy(ref_volume* v) {
    if (!v) return;
    cudaFree(v->D);
    cudaFree(v->W);
    cudaFree(v->tv);
    cudaFree(v->rgb);
    delete v;
}

float ref_truncation(const ref_volume* v) { return v->trunc; }

// TSDFVolume::integrate (tsdf_volume.cu:257-290).  depth: device float
// metres.  *kernel_ms receives the kernel time (CUDA events around the
// launch; the call itself also synchronises as the reference does).
int ref_integrate(ref_volume* v, const float* depth, size_t pitch, int width, int height, const double* pose,
                  float* kernel_ms) {
    const float4 camera_k = make_float4(v->fx, v->fy, v->cx, v->cy);
    const float4 quat = make_float4(pose[1], pose[2], pose[3], pose[0]);
    const float3 trans = make_float3(pose[4], pose[5], pose[6]);
    cv::cuda::PtrStepSzf dm(height, width, const_cast<float*>(depth), pitch);
    cv::cuda::PtrStepSzb cm(height, width, v->rgb, 0);
    const dim3 block(1, 8, 8), g(1, idiv_up(v->grid.y, 8), idiv_up(v->grid.z, 8));
    float* D = v->D;
    float* W = v->W;
    TransformationVoxel* tv = v->tv;
    void* a[] = {&D, &W, &v->grid, &v->vs, &tv, &v->offset, &v->trunc, &v->max_weight,
                 (void*)&camera_k, (void*)&quat, (void*)&trans, &dm, &cm};
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, 0);
    cudaError_t e = cudaLaunchKernel((const void*)g_k["cu_tsdf_integrate"], g, block, a, 0, 0);
    cudaEventRecord(e1, 0);
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (kernel_ms) *kernel_ms = ms;
    if (e != cudaSuccess) return fail("cu_tsdf_integrate", e);
    return 0;
}

// Copies the distance and weight grids to host buffers.
int ref_read_volume(const ref_volume* v, float* D, float* W) {
    const size_t n = (size_t)v->grid.x * v->grid.y * v->grid.z;
    cudaError_t e = cudaMemcpy(D, v->D, n * 4, cudaMemcpyDefault);
    if (e == cudaSuccess) e = cudaMemcpy(W, v->W, n * 4, cudaMemcpyDefault);
    if (e != cudaSuccess) return fail("read volume", e);
    return 0;
}

// Overwrites the distance grid (from host memory), to drive the mesh
// extraction with a chosen field.
int ref_write_distances(ref_volume* v, const float* D) {
    const size_t n = (size_t)v->grid.x * v->grid.y * v->grid.z;
    cudaError_t e = cudaMemcpy(v->D, D, n * 4, cudaMemcpyDefault);
    if (e != cudaSuccess) return fail("write distances", e);
    return 0;
}

// generate_triangular_surface + copy_data_mesh_to_host
// (marching_cubes.cu:159-237).  Returns the triangle count (or -1); writes up
// to cap triangles (9 floats and 3 ints each).  *kernel_ms: summed kernel time.
int64_t ref_extract(ref_volume* v, float* verts_out, int32_t* tris_out, int64_t cap, float* total_ms) {
    const dim3 gs = v->grid;
    const uint32_t cubes_per_layer = (gs.x - 1) * (gs.y - 1);
    float3* cu_vertices = nullptr;
    int3* cu_edges = nullptr;
    cudaError_t e = cudaMallocManaged(&cu_vertices, (size_t)cubes_per_layer * 12 * sizeof(float3));
    if (e == cudaSuccess) e = cudaMallocManaged(&cu_edges, (size_t)cubes_per_layer * 5 * sizeof(int3));
    if (e != cudaSuccess) {
        fail("mesh buffers", e);
        return -1;
    }
    std::vector<float3> vertices;
    std::vector<int3> triangles;
    const dim3 block(8, 8), g(idiv_up(gs.x, 8), idiv_up(gs.y, 8));
    const uint32_t layer_size = gs.x + gs.y;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, 0);
    for (int vz = 0; vz < (int)gs.z - 1; ++vz) {
        const float* l1 = v->D + (size_t)vz * layer_size;
        const float* l2 = v->D + (size_t)(vz + 1) * layer_size;
        TransformationVoxel* t1 = v->tv + (size_t)vz * layer_size;
        TransformationVoxel* t2 = v->tv + (size_t)(vz + 1) * layer_size;
        float3 vs = v->vs;
        dim3 grid = gs;
        int z = vz;
        void* a[] = {&l1, &l2, &t1, &t2, &grid, &vs, &z, &cu_vertices, &cu_edges};
        e = cudaLaunchKernel((const void*)g_k["marching_cubes_kernel"], g, block, a, 0, 0);
        if (e == cudaSuccess) e = cudaDeviceSynchronize();
        if (e != cudaSuccess) {
            fail("marching_cubes_kernel", e);
            return -1;
        }
        // copy_data_mesh_to_host
        int cube_idx = 0;
        for (int y = 0; y < (int)gs.y - 1; ++y) {
            for (int x = 0; x < (int)gs.x - 1; ++x) {
                const float3* verts = cu_vertices + (size_t)cube_idx * 12;
                const int3* edges = cu_edges + (size_t)cube_idx * 5;
                int edge_idx = 0;
                while (edge_idx < 5 && edges[edge_idx].x != -1) {
                    int tv3[3] = {edges[edge_idx].x, edges[edge_idx].y, edges[edge_idx].z};
                    int remap[12];
                    for (int k = 0; k < 12; ++k) remap[k] = -1;
                    for (int ev = 0; ev < 3; ++ev) {
                        const int edge_id = tv3[ev];
                        int v_id = remap[edge_id];
                        if (v_id == -1) {
                            vertices.push_back(verts[edge_id]);
                            v_id = (int)vertices.size() - 1;
                            remap[edge_id] = v_id;
                        }
                        tv3[ev] = v_id;
                    }
                    triangles.push_back(make_int3(tv3[0], tv3[1], tv3[2]));
                    edge_idx += 1;
                }
                cube_idx += 1;
            }
        }
    }
    cudaEventRecord(e1, 0);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (total_ms) *total_ms = ms;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(cu_vertices);
    cudaFree(cu_edges);
    const int64_t T = (int64_t)triangles.size();
    for (int64_t t = 0; t < T && t < cap; ++t) {
        const int3 tr = triangles[t];
        const int idx[3] = {tr.x, tr.y, tr.z};
        for (int j = 0; j < 3; ++j) {
            const float3 p = vertices[idx[j]];
            verts_out[9 * t + 3 * j + 0] = p.x;
            verts_out[9 * t + 3 * j + 1] = p.y;
            verts_out[9 * t + 3 * j + 2] = p.z;
            tris_out[3 * t + j] = idx[j];
        }
    }
    return T;
}

// cudaPointCloud::extract_points (cuda_point_cloud.cu:179-226): the camera
// matrix goes to the kernels' __device__ double K[3][3] (cudaMemcpyToSymbol
// there), 8x8 blocks, point_cloud_extract<true> when a colour image is given.
// points: device memory of the reference's 33-byte vertices.
int ref_points_extract(const double* K9, const float* depth, size_t pitch, int width, int height,
                       const unsigned char* color, size_t color_pitch, const double* T, int64_t start, void* points) {
    const char* key = color ? "point_cloud_extract_rgb" : "point_cloud_extract";
    if (!g_k.count(key)) {
        g_err = "point-cloud kernels are not in the reference cubin";
        return 1;
    }
    void* kp = nullptr;
    size_t ksz = 0;
    cudaError_t e = cudaLibraryGetGlobal(&kp, &ksz, g_lib, "_ZN7cuphoto1KE");
    if (e != cudaSuccess) return fail("cudaLibraryGetGlobal K", e);
    if (ksz != 9 * sizeof(double)) {
        g_err = "unexpected size of the reference's K";
        return 1;
    }
    e = cudaMemcpy(kp, K9, ksz, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return fail("cudaMemcpy K", e);
    cv::cuda::PtrStepSzf d(height, width, const_cast<float*>(depth), pitch);
    cv::cuda::PtrStepb c(const_cast<unsigned char*>(color), color_pitch);
    float4 quat = make_float4(T[1], T[2], T[3], T[0]);
    float3 trans = make_float3(T[4], T[5], T[6]);
    int64_t start_idx = start;
    void* args[] = {&d, &c, &quat, &trans, &start_idx, &points};
    const dim3 block(8, 8, 1), grid(idiv_up(width, 8), idiv_up(height, 8), 1);
    e = cudaLaunchKernel((const void*)g_k[key], grid, block, args, 0, 0);
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    return e == cudaSuccess ? 0 : fail("point_cloud_extract", e);
}

// cudaPointCloud::transform (cuda_point_cloud.cu:356-385): 16-thread blocks.
int ref_points_transform(void* points, uint32_t n, const double* T) {
    if (!g_k.count("transform_points")) {
        g_err = "point-cloud kernels are not in the reference cubin";
        return 1;
    }
    float4 quat = make_float4(T[1], T[2], T[3], T[0]);
    float3 trans = make_float3(T[4], T[5], T[6]);
    uint32_t num = n;
    void* args[] = {&quat, &trans, &num, &points};
    cudaError_t e = cudaLaunchKernel((const void*)g_k["transform_points"], dim3(idiv_up(n, 16)), dim3(16), args, 0, 0);
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    return e == cudaSuccess ? 0 : fail("transform_points", e);
}

// filter_image_if as project_to_depth launches it (cuda_point_cloud.cu:273-278).
int ref_filter_if(float* img, size_t pitch, int width, int height, float filter_value, float set_value) {
    if (!g_k.count("filter_image_if")) {
        g_err = "point-cloud kernels are not in the reference cubin";
        return 1;
    }
    cv::cuda::PtrStepSzf d(height, width, img, pitch);
    void* args[] = {&d, &filter_value, &set_value};
    const dim3 block(8, 8, 1), grid(idiv_up(width, 8), idiv_up(height, 8), 1);
    cudaError_t e = cudaLaunchKernel((const void*)g_k["filter_image_if"], grid, block, args, 0, 0);
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    return e == cudaSuccess ? 0 : fail("filter_image_if", e);
}

}  // extern "C"
