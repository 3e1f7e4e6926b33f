// generate_triangular_surface over the engine's C ABI
// (reference: marching_cubes.cu:159-237).
#include "cuphoto/marching_cubes.cuh"

#include <cstdio>

namespace cuphoto {

void generate_triangular_surface(const TSDFVolume& tsdf_volume, std::vector<float3>& vertices,
                                 std::vector<int3>& triangles) {
    gbt_volume* vol = tsdf_volume.engine();
    if (!vol) {
        std::fprintf(stderr, "[cuda]   generate_triangular_surface() -- volume was not allocated\n");
        return;
    }
    int64_t n = 0;
    if (gbt_extract_mesh(vol, nullptr, nullptr, 0, 0, &n, nullptr) != GBT_OK) {
        std::fprintf(stderr, "[cuda]   generate_triangular_surface() -- %s\n", gbt_last_error());
        return;
    }
    if (n == 0) return;
    float* d_verts = nullptr;
    int32_t* d_tris = nullptr;
    if (cudaMalloc(&d_verts, (size_t)n * 9 * sizeof(float)) != cudaSuccess ||
        cudaMalloc(&d_tris, (size_t)n * 3 * sizeof(int32_t)) != cudaSuccess) {
        std::fprintf(stderr, "[cuda]   generate_triangular_surface() -- failed to allocate the mesh buffers\n");
        cudaFree(d_verts);
        cudaFree(d_tris);
        return;
    }
    const int64_t base = (int64_t)vertices.size();
    int64_t n2 = 0;
    if (gbt_extract_mesh(vol, d_verts, d_tris, n, base, &n2, nullptr) != GBT_OK) {
        std::fprintf(stderr, "[cuda]   generate_triangular_surface() -- %s\n", gbt_last_error());
    } else {
        const size_t v0 = vertices.size(), t0 = triangles.size();
        vertices.resize(v0 + (size_t)n * 3);
        triangles.resize(t0 + (size_t)n);
        cudaMemcpy(vertices.data() + v0, d_verts, (size_t)n * 9 * sizeof(float), cudaMemcpyDeviceToHost);
        cudaMemcpy(triangles.data() + t0, d_tris, (size_t)n * 3 * sizeof(int32_t), cudaMemcpyDeviceToHost);
    }
    cudaFree(d_verts);
    cudaFree(d_tris);
}

bool generate_indexed_surface(const TSDFVolume& tsdf_volume, std::vector<float3>& vertices,
                              std::vector<float3>& normals, std::vector<int3>& triangles) {
    gbt_volume* vol = tsdf_volume.engine();
    if (!vol) {
        std::fprintf(stderr, "[cuda]   generate_indexed_surface() -- volume was not allocated\n");
        return false;
    }
    int64_t nv = 0, nt = 0;
    if (gbt_extract_mesh_indexed(vol, nullptr, nullptr, nullptr, 0, 0, 0, &nv, &nt, nullptr) != GBT_OK) {
        std::fprintf(stderr, "[cuda]   generate_indexed_surface() -- %s\n", gbt_last_error());
        return false;
    }
    normals.resize(vertices.size());
    if (nt == 0) return true;
    float *d_verts = nullptr, *d_normals = nullptr;
    int32_t* d_tris = nullptr;
    bool ok = cudaMalloc(&d_verts, (size_t)nv * 3 * sizeof(float)) == cudaSuccess &&
              cudaMalloc(&d_normals, (size_t)nv * 3 * sizeof(float)) == cudaSuccess &&
              cudaMalloc(&d_tris, (size_t)nt * 3 * sizeof(int32_t)) == cudaSuccess;
    if (!ok) {
        std::fprintf(stderr, "[cuda]   generate_indexed_surface() -- failed to allocate the mesh buffers\n");
    } else {
        const int64_t base = (int64_t)vertices.size();
        int64_t nv2 = 0, nt2 = 0;
        if (gbt_extract_mesh_indexed(vol, d_verts, d_normals, d_tris, nv, nt, base, &nv2, &nt2, nullptr) != GBT_OK) {
            std::fprintf(stderr, "[cuda]   generate_indexed_surface() -- %s\n", gbt_last_error());
            ok = false;
        } else {
            const size_t v0 = vertices.size(), t0 = triangles.size();
            vertices.resize(v0 + (size_t)nv);
            normals.resize(v0 + (size_t)nv);
            triangles.resize(t0 + (size_t)nt);
            cudaMemcpy(vertices.data() + v0, d_verts, (size_t)nv * 3 * sizeof(float), cudaMemcpyDeviceToHost);
            cudaMemcpy(normals.data() + v0, d_normals, (size_t)nv * 3 * sizeof(float), cudaMemcpyDeviceToHost);
            cudaMemcpy(triangles.data() + t0, d_tris, (size_t)nt * 3 * sizeof(int32_t), cudaMemcpyDeviceToHost);
        }
    }
    cudaFree(d_verts);
    cudaFree(d_normals);
    cudaFree(d_tris);
    return ok;
}

}  // namespace cuphoto
