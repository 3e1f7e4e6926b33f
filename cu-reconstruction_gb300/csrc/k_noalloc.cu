// Mesh extraction that allocates no device memory.
//
// gbt_extract_mesh lets the engine cudaMalloc its tile scratch the first
// time a volume is meshed.  Some callers cannot allow that: code that runs
// while a CUDA graph is being captured in the global capture mode (where
// cudaMalloc is an error), and applications that hand all device memory to
// their own pool or run under a fixed memory budget after start-up.  For them
// gbt_extract_mesh_noalloc runs the same marching-cubes kernel with its
// scratch in the file-scope array below, reserved when the library's module
// is loaded and kept by every GPU that loads it until the process exits.
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <mutex>

#include <cuda_runtime.h>

#include "gbt_internal.h"

namespace {

// [0, 64): emission ticket (u32), error flag (i32), triangle total (i64),
// tiles listed (u32); then two totals (u64) per superblock of 1024 tiles (at
// most 4096 bytes), one word (u64) per tile (at least 1024 cubes), one bit
// per group of 32 cubes and the list of tiles with triangles (u32 per tile).
static __device__ __align__(256) unsigned char g_mesh_scratch[GBT_NOALLOC_SCRATCH_BYTES];

constexpr int kMaxDevices = 64;
std::mutex g_setup_lock;
void* g_scratch_addr[kMaxDevices] = {};

// The array's name is only a host-side stand-in; its device address comes
// from cudaGetSymbolAddress, once per device, with that device current.
cudaError_t scratch_address(void** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_setup_lock);
    if (!g_scratch_addr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_mesh_scratch);
        if (e != cudaSuccess) return e;
        g_scratch_addr[dev] = p;
    }
    *out = g_scratch_addr[dev];
    return cudaSuccess;
}

// Count for the caller: the total, or -1 if the kernels set their error word.
__global__ void finish_count(const unsigned char* scratch, int64_t* d_n_tris) {
    const int err = *reinterpret_cast<const int*>(scratch + 4);
    const long long total = *reinterpret_cast<const long long*>(scratch + 8);
    *d_n_tris = err ? -1 : total;
}

}  // namespace

extern "C" {

gbt_status gbt_extract_mesh_noalloc(gbt_volume* v, float* verts, int32_t* tris, int64_t cap_tris,
                                    int64_t index_base, int64_t* d_n_tris, void* stream) {
    gbt::TraceRange trace_("gbt_extract_mesh_noalloc");
    char msg[320];
    if (!v || !d_n_tris || cap_tris < 0 || (cap_tris > 0 && (!verts || !tris))) {
        gbt::set_last_error("gbt_extract_mesh_noalloc: NULL volume/count/output or negative capacity");
        return GBT_ERR_INVALID_ARG;
    }
    if (!gbt::mc_indices_fit(cap_tris, index_base)) {
        gbt::set_last_error("gbt_extract_mesh_noalloc: index_base + 3 x cap_tris passes the int32 index range");
        return GBT_ERR_INVALID_ARG;
    }
    const gbt::VolDesc& d = *gbt::volume_desc(v);
    const int64_t ncubes =
        (d.nx >= 2 && d.ny >= 2 && d.nz >= 2) ? (int64_t)(d.nx - 1) * (d.ny - 1) * (d.nz - 1) : 0;
    if (ncubes > GBT_NOALLOC_MAX_CUBES) {
        std::snprintf(msg, sizeof(msg),
                      "gbt_extract_mesh_noalloc: %lld cubes exceed the %lld that its %d-byte static scratch covers; "
                      "use gbt_extract_mesh",
                      (long long)ncubes, (long long)GBT_NOALLOC_MAX_CUBES, (int)GBT_NOALLOC_SCRATCH_BYTES);
        gbt::set_last_error(msg);
        return GBT_ERR_INVALID_ARG;
    }
    void* scratch = nullptr;
    cudaError_t e = scratch_address(&scratch);
    if (e != cudaSuccess) {
        std::snprintf(msg, sizeof(msg), "gbt_extract_mesh_noalloc: scratch address: %s", cudaGetErrorString(e));
        gbt::set_last_error(msg);
        return GBT_ERR_CUDA;
    }
    gbt::McArgs a;
    std::memset(&a, 0, sizeof(a));
    a.D = d.D;
    a.W = d.W;
    a.gx = d.nx;
    a.gy = d.ny;
    a.gz = d.nz;
    for (int i = 0; i < 3; ++i) {
        a.vs[i] = d.vs[i];
        a.off[i] = d.off[i];
    }
    a.ncubes = (uint32_t)ncubes;
    const int64_t tile = gbt::mc_tile_cubes(gbt::volume_mode(v));
    a.ntiles = (uint32_t)((ncubes + tile - 1) / tile);
    a.div_cx = gbt::make_fastdiv((uint32_t)(d.nx > 1 ? d.nx - 1 : 1));
    a.div_cy = gbt::make_fastdiv((uint32_t)(d.ny > 1 ? d.ny - 1 : 1));
    a.div_gx = gbt::make_fastdiv((uint32_t)d.nx);
    a.div_gy = gbt::make_fastdiv((uint32_t)d.ny);
    a.verts = verts;
    a.tris = tris;
    a.cap = cap_tris;
    a.index_base = index_base;
    unsigned char* s = static_cast<unsigned char*>(scratch);
    a.ticket = reinterpret_cast<unsigned int*>(s);
    a.error = reinterpret_cast<int*>(s + 4);
    a.total = reinterpret_cast<long long*>(s + 8);
    a.nonempty = reinterpret_cast<unsigned int*>(s + 16);
    const size_t nsuper = (size_t)gbt::mc_superblocks(a.ntiles);
    a.super = reinterpret_cast<unsigned long long*>(s + 64);
    a.status = a.super + 2 * nsuper;
    const size_t nwords = (size_t)gbt::mc_group_words(ncubes);
    a.group_bits = reinterpret_cast<uint32_t*>(a.status + a.ntiles);
    a.tile_list = a.group_bits + nwords;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    cudaGetLastError();  // a launch reports only its own failure, not one left pending by an earlier call
    // the previous call's ticket, flags, counts and tile words must not leak into this one
    e = cudaMemsetAsync(scratch, 0, 64 + nsuper * 16 + (size_t)a.ntiles * 8 + nwords * 4, st);
    if (e == cudaSuccess && a.ntiles > 0) {
        if (gbt::volume_mode(v) == GBT_MODE_FIXED)
            e = gbt::launch_mc_fixed(a, st);
        else if (gbt::volume_arith(v) == GBT_ARITH_IEEE)
            e = gbt::launch_mc_compat_ieee(a, st);
        else
            e = gbt::launch_mc_compat_ref(a, st);
    }
    if (e == cudaSuccess) {
        finish_count<<<1, 1, 0, st>>>(s, d_n_tris);
        e = cudaGetLastError();
    }
    if (e != cudaSuccess) {
        std::snprintf(msg, sizeof(msg), "gbt_extract_mesh_noalloc: %s", cudaGetErrorString(e));
        gbt::set_last_error(msg);
        return GBT_ERR_CUDA;
    }
    return GBT_OK;
}

}  // extern "C"
