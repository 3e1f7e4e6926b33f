// C ABI of the engine (include/gbt_tsdf.h): volume lifetime, argument
// checking, pose conversion and kernel dispatch.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include <cudaTypedefs.h>
#include <cuda_runtime.h>

#include "gbt_internal.h"

namespace {

thread_local std::string g_last_error;

gbt_status fail(gbt_status st, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return st;
}

gbt_status cuda_fail(cudaError_t e, const char* what) {
    return fail(GBT_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

inline cudaStream_t as_stream(void* s) { return static_cast<cudaStream_t>(s); }

// Host-side failure injection (gbt_debug_inject): allocations to let through
// before failing, and how many to fail after that.
std::atomic<int64_t> g_inject_skip{0};
std::atomic<int64_t> g_inject_fail{0};
// streamed passes (brick 8) still to launch with their first copy held back
std::atomic<int64_t> g_inject_hold{0};

// true if this streamed pass is one that gbt_debug_inject asked to hold
bool injected_hold() {
    if (g_inject_hold.load() <= 0) return false;
    return g_inject_hold.fetch_sub(1) > 0;
}

// true if this allocation is one that gbt_debug_inject asked to fail
bool injected_alloc_failure() {
    if (g_inject_fail.load() <= 0) return false;
    if (g_inject_skip.fetch_sub(1) > 0) return false;
    g_inject_skip.store(0);
    return g_inject_fail.fetch_sub(1) > 0;
}

// Every device, managed and pinned allocation of the engine goes through
// these, so that failure injection reaches each of them.
cudaError_t dev_alloc(void** p, size_t bytes, bool managed = false) {
    if (injected_alloc_failure()) return cudaErrorMemoryAllocation;
    return managed ? cudaMallocManaged(p, bytes, cudaMemAttachGlobal) : cudaMalloc(p, bytes);
}

cudaError_t pinned_alloc(void** p, size_t bytes) {
    if (injected_alloc_failure()) return cudaErrorMemoryAllocation;
    return cudaMallocHost(p, bytes);
}

__global__ void injected_launch_kernel() {}

// SMs of the device current at the first call (the thread-safe
// initialisation of a function-local static; every device here is alike)
int device_sms() {
    static const int sms = [] {
        int dev = 0, n = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        return n > 0 ? n : 1;
    }();
    return sms;
}

}  // namespace

struct gbt_volume {
    gbt_volume_cfg cfg;
    gbt::VolDesc desc;
    int64_t nvox;
    bool managed;
    void* tvox;
    // marching-cubes scratch: [0,64) header (ticket u32, error i32, total i64, tiles listed u32),
    // then two u64 totals per superblock of 1024 tiles, one u64 word per tile, one bit per group
    // of 32 cubes, and the u32 list of tiles with triangles
    void* mc_scratch;
    size_t mc_scratch_bytes;
    // shared-vertex mesh scratch: used-edge bits, word offsets, block sums, vertex count
    void* weld_scratch;
    size_t weld_scratch_bytes;
    // status word (gbt::kStatus*), in the distances' allocation after the last distance
    unsigned int* status;
    // the distances and weights as tensors of the Tensor Memory Accelerator (streamed passes)
    bool maps_ready;
    gbt::VolumeMaps maps;
};

namespace gbt {

const VolDesc* volume_desc(const gbt_volume* v) { return &v->desc; }
int volume_mode(const gbt_volume* v) { return v->cfg.mode; }
int volume_arith(const gbt_volume* v) { return v->cfg.arith; }
void set_last_error(const char* msg) { g_last_error = msg; }

// CTAs per SM when the caller passes 0: as many as the kernel keeps resident
// (one wave of the persistent grid), cached per kernel.
int integrate_default_ctas_per_sm(int mode, int arith, int kind, int brick) {
    // host threads may race to fill an entry: each computes the same value
    static std::atomic<int> cache[3][5][4] = {};   // [arithmetic][kind 0..4][brick shape]
    const int k = mode == GBT_MODE_FIXED ? 2 : (arith == GBT_ARITH_IEEE ? 1 : 0);
    const int b = brick >= 0 && brick < 4 ? brick : 0;
    if (kind < 0 || kind > 4) kind = 0;
    std::atomic<int>& slot = cache[k][kind][b];
    int n = slot.load(std::memory_order_relaxed);
    if (n == 0) {
        n = k == 2 ? integrate_resident_ctas_fixed(kind, b)
                   : (k == 1 ? integrate_resident_ctas_compat_ieee(kind, b) : integrate_resident_ctas_compat_ref(kind, b));
        slot.store(n, std::memory_order_relaxed);
    }
    return n;
}

void brick_extent(int brick, int* bx, int* by, int* bz) {
    switch (brick) {
        case 1: *bx = 16; *by = 8; *bz = 4; break;
        case 2: *bx = 32; *by = 2; *bz = 8; break;
        case 3: *bx = 64; *by = 2; *bz = 4; break;
        default: *bx = 32; *by = 4; *bz = 4; break;
    }
}

}  // namespace gbt

namespace {

// Fixed-mode projection K [R | t] from the pose, in double, rounded once to
// float.  The quaternion is normalised first.
void fixed_projection(const double* pose, const gbt_volume_cfg& c, float* P) {
    double qw = pose[0], qx = pose[1], qy = pose[2], qz = pose[3];
    const double n = std::sqrt(qw * qw + qx * qx + qy * qy + qz * qz);
    qw /= n;
    qx /= n;
    qy /= n;
    qz /= n;
    double R[9];
    R[0] = 1 - 2 * (qy * qy + qz * qz);
    R[1] = 2 * (qx * qy - qz * qw);
    R[2] = 2 * (qx * qz + qy * qw);
    R[3] = 2 * (qx * qy + qz * qw);
    R[4] = 1 - 2 * (qx * qx + qz * qz);
    R[5] = 2 * (qy * qz - qx * qw);
    R[6] = 2 * (qx * qz - qy * qw);
    R[7] = 2 * (qy * qz + qx * qw);
    R[8] = 1 - 2 * (qx * qx + qy * qy);
    const double t[3] = {pose[4], pose[5], pose[6]};
    const double fx = c.focal_x, fy = c.focal_y, cx = c.cx, cy = c.cy;
    for (int k = 0; k < 3; ++k) {
        P[0 + k] = (float)(fx * R[0 + k] + cx * R[6 + k]);
        P[4 + k] = (float)(fy * R[3 + k] + cy * R[6 + k]);
        P[8 + k] = (float)R[6 + k];
    }
    P[3] = (float)(fx * t[0] + cx * t[2]);
    P[7] = (float)(fy * t[1] + cy * t[2]);
    P[11] = (float)t[2];
}

// Voxels of a grid, or -1 when there are 2^32 or more (no intermediate
// product overflows: n0 * n1 < 2^64).
int64_t grid_voxels(const uint32_t n[3]) {
    const uint64_t n01 = (uint64_t)n[0] * n[1];
    if (n[2] != 0 && n01 > 0xffffffffull / n[2]) return -1;
    return (int64_t)(n01 * n[2]);
}

gbt_status check_frames(const gbt_frame* frames, int32_t nframes) {
    if (!frames) return fail(GBT_ERR_INVALID_ARG, "frames is NULL");
    if (nframes < 1 || nframes > GBT_MAX_FRAMES_PER_PASS)
        return fail(GBT_ERR_INVALID_ARG, "nframes %d outside 1..%d", nframes, GBT_MAX_FRAMES_PER_PASS);
    for (int i = 0; i < nframes; ++i) {
        const gbt_frame& f = frames[i];
        // tsdf_volume.cu:260-268
        if (!f.depth) return fail(GBT_ERR_INVALID_ARG, "frame %d: depth map is a null pointer", i);
        if (f.width <= 0 || f.height <= 0)
            return fail(GBT_ERR_INVALID_ARG, "frame %d: depth width/height are zero", i);
        if (f.format != GBT_DEPTH_F32_M && f.format != GBT_DEPTH_U16)
            return fail(GBT_ERR_INVALID_ARG, "frame %d: unknown depth format %d", i, f.format);
        const size_t elem = f.format == GBT_DEPTH_U16 ? 2 : 4;
        if (f.pitch_bytes < elem * (size_t)f.width)
            return fail(GBT_ERR_INVALID_ARG, "frame %d: pitch %zu below width*%zu", i, f.pitch_bytes, elem);
        if (f.pitch_bytes % elem != 0 || ((uintptr_t)f.depth % elem) != 0)
            return fail(GBT_ERR_INVALID_ARG, "frame %d: depth rows not aligned to the element size", i);
        if ((uint64_t)f.height * (f.pitch_bytes / elem) > 0xffffffffull)
            return fail(GBT_ERR_INVALID_ARG, "frame %d: image larger than 2^32 elements", i);
        for (int k = 0; k < 7; ++k)
            if (!std::isfinite(f.pose[k])) return fail(GBT_ERR_INVALID_ARG, "frame %d: pose is not finite", i);
    }
    return GBT_OK;
}

// cuTensorMapEncodeTiled from the driver, through the runtime (the library
// does not link the driver library itself); null if the driver has none
PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
    static const PFN_cuTensorMapEncodeTiled_v12000 fn = [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess) {
            cudaGetLastError();
            p = nullptr;
        }
        return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    }();
    return fn;
}

}  // namespace

// The volume's distances and weights as 3-D tensors of floats ([nz][ny][nx],
// rows of nx * 4 bytes: nx a multiple of 4) in boxes of one streamed brick,
// encoded once per volume (the arrays never move).
static gbt_status volume_maps(gbt_volume* v) {
    if (v->maps_ready) return GBT_OK;
    const PFN_cuTensorMapEncodeTiled_v12000 encode = tensor_map_encoder();
    if (!encode) return fail(GBT_ERR_CUDA, "the driver has no cuTensorMapEncodeTiled");
    const gbt::VolDesc& d = v->desc;
    const cuuint64_t dims[3] = {(cuuint64_t)d.nx, (cuuint64_t)d.ny, (cuuint64_t)d.nz};
    const cuuint64_t strides[2] = {(cuuint64_t)d.nx * 4u, (cuuint64_t)d.nx * (cuuint64_t)d.ny * 4u};
    const cuuint32_t box[3] = {gbt::kStreamBrickX, gbt::kStreamBrickY, gbt::kStreamBrickZ};
    const cuuint32_t elem[3] = {1, 1, 1};
    float* arrays[2] = {d.D, d.W};
    CUtensorMap* maps[2] = {&v->maps.d, &v->maps.w};
    for (int i = 0; i < 2; ++i) {
        // boxes past the volume's end read zeros (never stored)
        const CUresult r = encode(maps[i], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, arrays[i], dims, strides, box, elem,
                                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                                  CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
        if (r != CUDA_SUCCESS) return fail(GBT_ERR_CUDA, "cuTensorMapEncodeTiled for the volume failed (%d)", (int)r);
    }
    v->maps_ready = true;
    return GBT_OK;
}

extern "C" {

const char* gbt_last_error(void) { return g_last_error.c_str(); }

const char* gbt_version(void) { return "gbt-tsdf 0.1 sm_103a"; }

gbt_status gbt_debug_inject(int32_t what, int64_t skip, int64_t count) {
    switch (what) {
        case GBT_INJECT_NONE:
            g_inject_fail.store(0);
            g_inject_skip.store(0);
            g_inject_hold.store(0);
            return GBT_OK;
        case GBT_INJECT_ALLOC:
            if (skip < 0 || count < 0) return fail(GBT_ERR_INVALID_ARG, "gbt_debug_inject: negative skip or count");
            g_inject_fail.store(0);
            g_inject_skip.store(skip);
            g_inject_fail.store(count);
            return GBT_OK;
        case GBT_INJECT_HOLD_COPY:
            if (count < 0) return fail(GBT_ERR_INVALID_ARG, "gbt_debug_inject: negative count");
            g_inject_hold.store(count);
            return GBT_OK;
        case GBT_INJECT_LAUNCH_ERROR:
            // a block of zero threads: the runtime refuses the launch on the
            // host (invalid configuration); nothing reaches the GPU
            injected_launch_kernel<<<1, 0>>>();
            return GBT_OK;
        default:
            return fail(GBT_ERR_INVALID_ARG, "gbt_debug_inject: unknown kind %d", what);
    }
}

gbt_status gbt_volume_create(const gbt_volume_cfg* cfg, void* stream, gbt_volume** out) {
    gbt::TraceRange trace_("gbt_volume_create");
    if (!cfg || !out) return fail(GBT_ERR_INVALID_ARG, "cfg or out is NULL");
    *out = nullptr;
    const gbt_volume_cfg& c = *cfg;
    for (int i = 0; i < 3; ++i) {
        if (c.voxel_grid_size[i] == 0) return fail(GBT_ERR_INVALID_ARG, "voxel_grid_size[%d] is 0", i);
        if (!(c.physical_size[i] > 0.f) || !std::isfinite(c.physical_size[i]))
            return fail(GBT_ERR_INVALID_ARG, "physical_size[%d] must be positive", i);
        if (!std::isfinite(c.global_offset[i])) return fail(GBT_ERR_INVALID_ARG, "global_offset[%d] not finite", i);
        if (c.voxel_grid_size[i] > (1u << 24))
            return fail(GBT_ERR_INVALID_ARG, "voxel_grid_size[%d] above 2^24", i);
    }
    const int64_t nvox = grid_voxels(c.voxel_grid_size);
    if (nvox < 0) return fail(GBT_ERR_INVALID_ARG, "volume has 2^32 or more voxels; limit is 2^32-1");
    if (c.mode != GBT_MODE_COMPAT && c.mode != GBT_MODE_FIXED) return fail(GBT_ERR_INVALID_ARG, "unknown mode %d", c.mode);
    if (c.arith != GBT_ARITH_REFERENCE && c.arith != GBT_ARITH_IEEE)
        return fail(GBT_ERR_INVALID_ARG, "unknown arith %d", c.arith);
    if (c.memory != GBT_MEMORY_DEVICE && c.memory != GBT_MEMORY_MANAGED)
        return fail(GBT_ERR_INVALID_ARG, "unknown memory kind %d", c.memory);
    if (c.mode == GBT_MODE_FIXED && !(c.max_weight >= 1.f))
        return fail(GBT_ERR_INVALID_ARG, "fixed mode needs max_weight >= 1");
    if (!std::isfinite(c.focal_x) || !std::isfinite(c.focal_y) || !std::isfinite(c.cx) || !std::isfinite(c.cy))
        return fail(GBT_ERR_INVALID_ARG, "intrinsics not finite");
    if (!(c.truncation > 0.f)) {
        // the integrate kernels rely on a positive truncation distance
        float dot = 0.f;
        for (int i = 0; i < 3; ++i) {
            const float vs = c.physical_size[i] / (float)c.voxel_grid_size[i];
            dot = i ? dot + vs * vs : vs * vs;
        }
        if (!(1.1f * std::sqrt(dot) > 0.f))
            return fail(GBT_ERR_INVALID_ARG, "voxel size too small: the truncation distance rounds to 0");
    }

    gbt_volume* v = new gbt_volume();
    std::memset(v, 0, sizeof(*v));
    v->cfg = c;
    v->nvox = nvox;
    v->managed = c.memory == GBT_MEMORY_MANAGED;
    gbt::VolDesc& d = v->desc;
    d.nx = (int32_t)c.voxel_grid_size[0];
    d.ny = (int32_t)c.voxel_grid_size[1];
    d.nz = (int32_t)c.voxel_grid_size[2];
    // tsdf_volume.cu:197-199
    for (int i = 0; i < 3; ++i) {
        d.vs[i] = c.physical_size[i] / (float)c.voxel_grid_size[i];
        d.off[i] = c.global_offset[i];
    }
    float dot = d.vs[0] * d.vs[0] + d.vs[1] * d.vs[1];
    dot = dot + d.vs[2] * d.vs[2];
    d.trunc = c.truncation > 0.f ? c.truncation : 1.1f * std::sqrt(dot);
    d.max_weight = c.max_weight;
    d.max_depth = c.max_depth > 0.f ? c.max_depth : 24.0f;
    d.min_z = c.min_z;
    d.fx = c.focal_x;
    d.fy = c.focal_y;
    d.cx = c.cx;
    d.cy = c.cy;

    const size_t bytes = (size_t)nvox * sizeof(float);
    // the status word sits 256-byte aligned after the distances
    const size_t status_at = (bytes + 255) / 256 * 256;
    cudaError_t e;
    if (v->managed) {
        e = dev_alloc(reinterpret_cast<void**>(&d.D), status_at + 256, true);
        if (e == cudaSuccess) e = dev_alloc(reinterpret_cast<void**>(&d.W), bytes, true);
    } else {
        e = dev_alloc(reinterpret_cast<void**>(&d.D), status_at + 256);
        if (e == cudaSuccess) e = dev_alloc(reinterpret_cast<void**>(&d.W), bytes);
    }
    if (e == cudaSuccess) v->status = reinterpret_cast<unsigned int*>(reinterpret_cast<char*>(d.D) + status_at);
    if (e != cudaSuccess) {
        cudaGetLastError();
        if (d.D) cudaFree(d.D);
        if (d.W) cudaFree(d.W);
        delete v;
        return fail(GBT_ERR_ALLOC, "allocating %zu bytes for the volume: %s", 2 * bytes, cudaGetErrorString(e));
    }
    gbt_status st = gbt_volume_reset(v, stream);
    if (st == GBT_OK) {
        e = cudaStreamSynchronize(as_stream(stream));
        if (e != cudaSuccess) st = cuda_fail(e, "volume set-up");
    }
    if (st != GBT_OK) {
        cudaFree(d.D);
        cudaFree(d.W);
        delete v;
        return st;
    }
    *out = v;
    return GBT_OK;
}

gbt_status gbt_volume_destroy(gbt_volume* v) {
    if (!v) return GBT_OK;
    cudaFree(v->desc.D);
    cudaFree(v->desc.W);
    if (v->tvox) cudaFree(v->tvox);
    if (v->mc_scratch) cudaFree(v->mc_scratch);
    if (v->weld_scratch) cudaFree(v->weld_scratch);
    delete v;
    return GBT_OK;
}

gbt_status gbt_volume_reset(gbt_volume* v, void* stream) {
    gbt::TraceRange trace_("gbt_volume_reset");
    if (!v) return fail(GBT_ERR_INVALID_ARG, "volume is NULL");
    cudaGetLastError();  // a launch reports only its own failure
    cudaError_t e = gbt::launch_volume_init(v->desc.D, v->desc.W, v->nvox, v->desc.trunc, as_stream(stream));
    if (e == cudaSuccess) e = cudaMemsetAsync(v->status, 0, sizeof(unsigned int), as_stream(stream));
    if (e != cudaSuccess) return cuda_fail(e, "volume initialisation");
    return GBT_OK;
}

gbt_status gbt_volume_check(gbt_volume* v, void* stream) {
    gbt::TraceRange trace_("gbt_volume_check");
    if (!v) return fail(GBT_ERR_INVALID_ARG, "volume is NULL");
    unsigned int word = 0;
    cudaError_t e = cudaStreamSynchronize(as_stream(stream));
    if (e == cudaSuccess) e = cudaMemcpy(&word, v->status, sizeof(word), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail(e, "gbt_volume_check");
    if (word & gbt::kStatusWaitExpired) {
        e = cudaMemset(v->status, 0, sizeof(word));
        if (e != cudaSuccess) return cuda_fail(e, "gbt_volume_check");
        return fail(GBT_ERR_TIMEOUT,
                    "a streamed integrate pass gave up waiting for a copy of the volume's bricks: the volume's "
                    "distances and weights are undefined until it is reset or loaded");
    }
    return GBT_OK;
}

}  // extern "C"

namespace {

// The volume file's header (little- or big-endian as the host writes it).
struct VolumeFileHeader {
    char magic[8];
    uint32_t header_bytes;
    uint32_t cfg_bytes;
    int64_t nvox;
    gbt_volume_cfg cfg;
    unsigned char pad[GBT_VOLUME_FILE_HEADER_BYTES - 24 - sizeof(gbt_volume_cfg)];
};
static_assert(sizeof(VolumeFileHeader) == GBT_VOLUME_FILE_HEADER_BYTES, "256-byte header");

constexpr int64_t kFileChunkFloats = 4 << 20;   // 16 MB of host staging per copy

struct FileCloser {
    FILE* f;
    ~FileCloser() {
        if (f) std::fclose(f);
    }
};

gbt_status grid_to_file(const float* dev, int64_t n, FILE* f, cudaStream_t s, std::vector<float>& buf,
                        const char* path) {
    for (int64_t i = 0; i < n; i += kFileChunkFloats) {
        const int64_t m = std::min<int64_t>(kFileChunkFloats, n - i);
        cudaError_t e = cudaMemcpyAsync(buf.data(), dev + i, (size_t)m * 4, cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) return cuda_fail(e, "gbt_volume_save: reading the volume");
        if (std::fwrite(buf.data(), 4, (size_t)m, f) != (size_t)m)
            return fail(GBT_ERR_IO, "gbt_volume_save: writing %s failed", path);
    }
    return GBT_OK;
}

gbt_status grid_from_file(float* dev, int64_t n, FILE* f, cudaStream_t s, std::vector<float>& buf,
                          const char* path) {
    for (int64_t i = 0; i < n; i += kFileChunkFloats) {
        const int64_t m = std::min<int64_t>(kFileChunkFloats, n - i);
        if (std::fread(buf.data(), 4, (size_t)m, f) != (size_t)m)
            return fail(GBT_ERR_IO, "gbt_volume_load: %s ends before its grids do", path);
        cudaError_t e = cudaMemcpyAsync(dev + i, buf.data(), (size_t)m * 4, cudaMemcpyHostToDevice, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) return cuda_fail(e, "gbt_volume_load: writing the volume");
    }
    return GBT_OK;
}

}  // namespace

extern "C" {

gbt_status gbt_volume_save(const gbt_volume* v, const char* path, void* stream) {
    gbt::TraceRange trace_("gbt_volume_save");
    if (!v || !path) return fail(GBT_ERR_INVALID_ARG, "gbt_volume_save: volume or path is NULL");
    FileCloser fc{std::fopen(path, "wb")};
    if (!fc.f) return fail(GBT_ERR_IO, "gbt_volume_save: cannot open %s for writing", path);
    VolumeFileHeader h;
    std::memset(&h, 0, sizeof(h));
    std::memcpy(h.magic, GBT_VOLUME_FILE_MAGIC, 8);
    h.header_bytes = GBT_VOLUME_FILE_HEADER_BYTES;
    h.cfg_bytes = (uint32_t)sizeof(gbt_volume_cfg);
    h.nvox = v->nvox;
    h.cfg = v->cfg;
    if (std::fwrite(&h, sizeof(h), 1, fc.f) != 1) return fail(GBT_ERR_IO, "gbt_volume_save: writing %s failed", path);
    std::vector<float> buf((size_t)std::min<int64_t>(kFileChunkFloats, std::max<int64_t>(v->nvox, 1)));
    const cudaStream_t s = as_stream(stream);
    gbt_status st = grid_to_file(v->desc.D, v->nvox, fc.f, s, buf, path);
    if (st == GBT_OK) st = grid_to_file(v->desc.W, v->nvox, fc.f, s, buf, path);
    if (st != GBT_OK) return st;
    if (std::fflush(fc.f) != 0) return fail(GBT_ERR_IO, "gbt_volume_save: writing %s failed", path);
    return GBT_OK;
}

gbt_status gbt_volume_load(const char* path, void* stream, gbt_volume** out) {
    gbt::TraceRange trace_("gbt_volume_load");
    if (!path || !out) return fail(GBT_ERR_INVALID_ARG, "gbt_volume_load: path or out is NULL");
    *out = nullptr;
    FileCloser fc{std::fopen(path, "rb")};
    if (!fc.f) return fail(GBT_ERR_IO, "gbt_volume_load: cannot open %s", path);
    VolumeFileHeader h;
    if (std::fread(&h, sizeof(h), 1, fc.f) != 1 || std::memcmp(h.magic, GBT_VOLUME_FILE_MAGIC, 8) != 0 ||
        h.header_bytes != GBT_VOLUME_FILE_HEADER_BYTES || h.cfg_bytes != sizeof(gbt_volume_cfg))
        return fail(GBT_ERR_IO, "gbt_volume_load: %s is not a volume file of this layout", path);
    const int64_t nvox = grid_voxels(h.cfg.voxel_grid_size);
    if (nvox < 0 || nvox != h.nvox)
        return fail(GBT_ERR_IO, "gbt_volume_load: %s: voxel count does not match its grid", path);
    gbt_volume* v = nullptr;
    gbt_status st = gbt_volume_create(&h.cfg, stream, &v);
    if (st != GBT_OK) return st;
    std::vector<float> buf((size_t)std::min<int64_t>(kFileChunkFloats, std::max<int64_t>(nvox, 1)));
    const cudaStream_t s = as_stream(stream);
    st = grid_from_file(v->desc.D, nvox, fc.f, s, buf, path);
    if (st == GBT_OK) st = grid_from_file(v->desc.W, nvox, fc.f, s, buf, path);
    if (st != GBT_OK) {
        const std::string msg = g_last_error;
        gbt_volume_destroy(v);
        g_last_error = msg;
        return st;
    }
    *out = v;
    return GBT_OK;
}

gbt_status gbt_volume_get_cfg(const gbt_volume* v, gbt_volume_cfg* cfg) {
    if (!v || !cfg) return fail(GBT_ERR_INVALID_ARG, "gbt_volume_get_cfg: volume or cfg is NULL");
    *cfg = v->cfg;
    return GBT_OK;
}

gbt_status gbt_volume_get_info(const gbt_volume* v, gbt_volume_info* info) {
    if (!v || !info) return fail(GBT_ERR_INVALID_ARG, "volume or info is NULL");
    std::memset(info, 0, sizeof(*info));
    for (int i = 0; i < 3; ++i) {
        info->voxel_grid_size[i] = v->cfg.voxel_grid_size[i];
        info->voxel_size[i] = v->desc.vs[i];
        info->global_offset[i] = v->cfg.global_offset[i];
        info->physical_size[i] = v->cfg.physical_size[i];
    }
    info->truncation = v->desc.trunc;
    info->num_voxels = v->nvox;
    info->tsdf = v->desc.D;
    info->weights = v->desc.W;
    info->mode = v->cfg.mode;
    info->arith = v->cfg.arith;
    return GBT_OK;
}

gbt_status gbt_volume_transformation_voxels(gbt_volume* v, void* stream, void** out) {
    gbt::TraceRange trace_("gbt_volume_transformation_voxels");
    if (!v || !out) return fail(GBT_ERR_INVALID_ARG, "volume or out is NULL");
    if (!v->tvox) {
        const size_t bytes = (size_t)v->nvox * 28;
        cudaError_t e = dev_alloc(&v->tvox, bytes, v->managed);
        if (e != cudaSuccess) {
            cudaGetLastError();
            v->tvox = nullptr;
            return fail(GBT_ERR_ALLOC, "allocating %zu bytes of voxel transforms: %s", bytes, cudaGetErrorString(e));
        }
        cudaGetLastError();
        e = gbt::launch_tvoxels(v->tvox, v->desc, as_stream(stream));
        if (e != cudaSuccess) return cuda_fail(e, "voxel transforms");
    }
    *out = v->tvox;
    return GBT_OK;
}

gbt_status gbt_integrate_tuned(gbt_volume* v, const gbt_frame* frames, int32_t nframes, int32_t brick,
                               int32_t ctas_per_sm, void* stream) {
    gbt::TraceRange trace_("gbt_integrate_tuned");
    if (!v) return fail(GBT_ERR_INVALID_ARG, "volume is NULL");
    gbt_status st = check_frames(frames, nframes);
    if (st != GBT_OK) return st;
    if (brick < 0 || brick > 8) return fail(GBT_ERR_INVALID_ARG, "brick %d outside 0..8", brick);
    if (brick >= 4 && nframes > gbt::kLaneBrickFrames)
        return fail(GBT_ERR_INVALID_ARG, "brick %d (%s) takes passes of up to %d frames", brick,
                    brick == 8 ? "streamed through the Tensor Memory Accelerator" : "depth staged in shared memory",
                    gbt::kLaneBrickFrames);
    if (brick == 8) {
        if (v->desc.nx % 4 != 0)
            return fail(GBT_ERR_INVALID_ARG, "brick 8 (streamed) needs an x extent that is a multiple of 4, not %d",
                        v->desc.nx);
        st = volume_maps(v);
        if (st != GBT_OK) return st;
    }
    if (ctas_per_sm < 0 || ctas_per_sm > 32) return fail(GBT_ERR_INVALID_ARG, "ctas_per_sm %d outside 0..32", ctas_per_sm);
    gbt::IntegrateArgs a;
    std::memset(&a, 0, sizeof(a));
    a.vol = v->desc;
    a.nframes = nframes;
    for (int i = 0; i < nframes; ++i) {
        const gbt_frame& f = frames[i];
        gbt::FrameDesc& fd = a.frames[i];
        fd.depth = f.depth;
        fd.pitch = (int64_t)f.pitch_bytes;
        fd.width = f.width;
        fd.height = f.height;
        fd.fmt = f.format;
        fd.scale = f.depth_scale;
        // tsdf_volume.cu:271-272
        fd.q[0] = (float)f.pose[1];
        fd.q[1] = (float)f.pose[2];
        fd.q[2] = (float)f.pose[3];
        fd.q[3] = (float)f.pose[0];
        fd.t[0] = (float)f.pose[4];
        fd.t[1] = (float)f.pose[5];
        fd.t[2] = (float)f.pose[6];
        if (v->cfg.mode == GBT_MODE_FIXED) fixed_projection(f.pose, v->cfg, fd.P);
    }
    int bx = gbt::kStreamBrickX, by = gbt::kStreamBrickY, bz = gbt::kStreamBrickZ;   // brick 8
    if (brick != 8) gbt::brick_extent(brick & 3, &bx, &by, &bz);
    const uint32_t nbx = (uint32_t)((v->desc.nx + bx - 1) / bx), nby = (uint32_t)((v->desc.ny + by - 1) / by);
    const long long nbricks = (long long)nbx * nby * ((v->desc.nz + bz - 1) / bz);   // below 2^32: fewer than voxels
    a.nbricks = (uint32_t)nbricks;
    a.div_nbx = gbt::make_fastdiv(nbx);
    a.div_nby = gbt::make_fastdiv(nby);
    a.status = v->status;
    const int kind = brick == 8 ? 4 : (brick >= 4 ? 3 : (nframes <= gbt::kLaneBrickFrames ? 1 : 0));
    long long grid = (long long)device_sms() *
                     (ctas_per_sm ? ctas_per_sm
                                  : gbt::integrate_default_ctas_per_sm(v->cfg.mode, v->cfg.arith, kind, brick & 3));
    if (grid > nbricks) grid = nbricks;
    if (grid < 1) grid = 1;
    cudaError_t e;
    cudaGetLastError();  // a launch reports only its own failure
    if (brick == 8) {
        a.hold_first_copy = injected_hold() ? 1 : 0;
        if (v->cfg.mode == GBT_MODE_FIXED)
            e = gbt::launch_stream_fixed(a, v->maps, (int)grid, as_stream(stream));
        else if (v->cfg.arith == GBT_ARITH_IEEE)
            e = gbt::launch_stream_compat_ieee(a, v->maps, (int)grid, as_stream(stream));
        else
            e = gbt::launch_stream_compat_ref(a, v->maps, (int)grid, as_stream(stream));
    } else if (v->cfg.mode == GBT_MODE_FIXED)
        e = gbt::launch_integrate_fixed(a, brick, (int)grid, as_stream(stream));
    else if (v->cfg.arith == GBT_ARITH_IEEE)
        e = gbt::launch_integrate_compat_ieee(a, brick, (int)grid, as_stream(stream));
    else
        e = gbt::launch_integrate_compat_ref(a, brick, (int)grid, as_stream(stream));
    if (e != cudaSuccess) return cuda_fail(e, "integrate launch");
    return GBT_OK;
}

gbt_status gbt_integrate(gbt_volume* v, const gbt_frame* frames, int32_t nframes, void* stream) {
    return gbt_integrate_tuned(v, frames, nframes, 0, 0, stream);
}

}  // extern "C"

namespace {

gbt_status mc_prepare(gbt_volume* v, float* verts, int32_t* tris, int64_t cap, int64_t index_base, gbt::McArgs* a,
                      bool indexed = false) {
    if (!v) return fail(GBT_ERR_INVALID_ARG, "volume is NULL");
    if (cap < 0) return fail(GBT_ERR_INVALID_ARG, "negative capacity");
    if (cap > 0 && ((!verts && !indexed) || !tris)) return fail(GBT_ERR_INVALID_ARG, "output buffers are NULL");
    if (!indexed && !gbt::mc_indices_fit(cap, index_base))
        return fail(GBT_ERR_INVALID_ARG, "index_base %lld + 3 x %lld triangles passes the int32 index range",
                    (long long)index_base, (long long)cap);
    const gbt::VolDesc& d = v->desc;
    std::memset(a, 0, sizeof(*a));
    a->D = d.D;
    a->W = d.W;
    a->gx = d.nx;
    a->gy = d.ny;
    a->gz = d.nz;
    for (int i = 0; i < 3; ++i) {
        a->vs[i] = d.vs[i];
        a->off[i] = d.off[i];
    }
    const int64_t ncubes = (d.nx >= 2 && d.ny >= 2 && d.nz >= 2)
                               ? (int64_t)(d.nx - 1) * (d.ny - 1) * (d.nz - 1) : 0;
    a->ncubes = (uint32_t)ncubes;
    const int64_t tile = gbt::mc_tile_cubes(v->cfg.mode);
    a->ntiles = (uint32_t)((ncubes + tile - 1) / tile);
    a->div_cx = gbt::make_fastdiv((uint32_t)(d.nx > 1 ? d.nx - 1 : 1));
    a->div_cy = gbt::make_fastdiv((uint32_t)(d.ny > 1 ? d.ny - 1 : 1));
    a->div_gx = gbt::make_fastdiv((uint32_t)d.nx);
    a->div_gy = gbt::make_fastdiv((uint32_t)d.ny);
    a->verts = verts;
    a->tris = tris;
    a->cap = cap;
    a->index_base = index_base;
    const size_t nsuper = (size_t)gbt::mc_superblocks(a->ntiles);
    const size_t nwords = (size_t)gbt::mc_group_words(ncubes);
    const size_t need = 64 + nsuper * 16 + (size_t)a->ntiles * 12 + nwords * 4;
    if (v->mc_scratch_bytes < need) {
        if (v->mc_scratch) cudaFree(v->mc_scratch);
        v->mc_scratch = nullptr;
        v->mc_scratch_bytes = 0;
        cudaError_t e = dev_alloc(&v->mc_scratch, need);
        if (e != cudaSuccess) {
            cudaGetLastError();
            return fail(GBT_ERR_ALLOC, "allocating %zu bytes of mesh scratch: %s", need, cudaGetErrorString(e));
        }
        v->mc_scratch_bytes = need;
    }
    char* s = static_cast<char*>(v->mc_scratch);
    a->ticket = reinterpret_cast<unsigned int*>(s);
    a->error = reinterpret_cast<int*>(s + 4);
    a->total = reinterpret_cast<long long*>(s + 8);
    a->nonempty = reinterpret_cast<unsigned int*>(s + 16);
    a->super = reinterpret_cast<unsigned long long*>(s + 64);
    a->status = a->super + 2 * nsuper;
    a->group_bits = reinterpret_cast<uint32_t*>(a->status + a->ntiles);
    a->tile_list = a->group_bits + nwords;
    return GBT_OK;
}

gbt_status mc_launch(gbt_volume* v, const gbt::McArgs& a, cudaStream_t s) {
    cudaGetLastError();  // a launch reports only its own failure
    // header, superblock totals, tile words and group bits start at zero
    cudaError_t e = cudaMemsetAsync(v->mc_scratch, 0,
                                    64 + (size_t)gbt::mc_superblocks(a.ntiles) * 16 + (size_t)a.ntiles * 8 +
                                        (size_t)gbt::mc_group_words(a.ncubes) * 4, s);
    if (e != cudaSuccess) return cuda_fail(e, "mesh scratch clear");
    if (a.ntiles == 0) return GBT_OK;
    if (v->cfg.mode == GBT_MODE_FIXED)
        e = gbt::launch_mc_fixed(a, s);
    else if (v->cfg.arith == GBT_ARITH_IEEE)
        e = gbt::launch_mc_compat_ieee(a, s);
    else
        e = gbt::launch_mc_compat_ref(a, s);
    if (e != cudaSuccess) return cuda_fail(e, "mesh launch");
    return GBT_OK;
}

}  // namespace

extern "C" {

gbt_status gbt_extract_mesh(gbt_volume* v, float* verts, int32_t* tris, int64_t cap_tris, int64_t index_base,
                            int64_t* n_tris, void* stream) {
    gbt::TraceRange trace_("gbt_extract_mesh");
    if (!n_tris) return fail(GBT_ERR_INVALID_ARG, "n_tris is NULL");
    *n_tris = 0;
    gbt::McArgs a;
    gbt_status st = mc_prepare(v, verts, tris, cap_tris, index_base, &a);
    if (st != GBT_OK) return st;
    cudaStream_t s = as_stream(stream);
    st = mc_launch(v, a, s);
    if (st != GBT_OK) return st;
    struct {
        unsigned int ticket;
        int error;
        long long total;
    } hdr;
    cudaError_t e = cudaMemcpyAsync(&hdr, v->mc_scratch, sizeof(hdr), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_fail(e, "mesh extraction");
    if (hdr.error) return fail(GBT_ERR_CUDA, "mesh extraction: the kernels set their error word");
    *n_tris = hdr.total;
    if (hdr.total > cap_tris && cap_tris > 0)
        return fail(GBT_ERR_CAPACITY, "mesh has %lld triangles, buffer holds %lld", hdr.total, (long long)cap_tris);
    return GBT_OK;
}

gbt_status gbt_extract_mesh_async(gbt_volume* v, float* verts, int32_t* tris, int64_t cap_tris, int64_t index_base,
                                  int64_t* d_n_tris, void* stream) {
    gbt::TraceRange trace_("gbt_extract_mesh_async");
    if (!d_n_tris) return fail(GBT_ERR_INVALID_ARG, "d_n_tris is NULL");
    gbt::McArgs a;
    gbt_status st = mc_prepare(v, verts, tris, cap_tris, index_base, &a);
    if (st != GBT_OK) return st;
    cudaStream_t s = as_stream(stream);
    st = mc_launch(v, a, s);
    if (st != GBT_OK) return st;
    cudaError_t e = cudaMemcpyAsync(d_n_tris, a.total, sizeof(long long), cudaMemcpyDeviceToDevice, s);
    if (e != cudaSuccess) return cuda_fail(e, "mesh count copy");
    return GBT_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Batched integrate: many volumes, one persistent launch.

struct gbt_batch {
    int32_t max_scenes;
    int32_t max_frames;
    void* host;          // pinned staging: scenes then frames
    void* dev;           // device tables: ticket (256 B), scenes, frames
    size_t bytes;
    cudaEvent_t copied;
    bool pending;
};

namespace {

size_t batch_bytes(int32_t max_scenes, int32_t max_frames) {
    return 256 + (size_t)max_scenes * sizeof(gbt::BatchScene) + (size_t)max_frames * sizeof(gbt::FrameDesc);
}

}  // namespace

extern "C" {

gbt_status gbt_batch_create(int32_t max_scenes, int32_t max_frames, gbt_batch** out) {
    if (!out) return fail(GBT_ERR_INVALID_ARG, "out is NULL");
    *out = nullptr;
    if (max_scenes < 1 || max_frames < 1 || max_scenes > (1 << 20) || max_frames > (1 << 24))
        return fail(GBT_ERR_INVALID_ARG, "max_scenes %d / max_frames %d out of range", max_scenes, max_frames);
    gbt_batch* b = new gbt_batch();
    std::memset(b, 0, sizeof(*b));
    b->max_scenes = max_scenes;
    b->max_frames = max_frames;
    b->bytes = batch_bytes(max_scenes, max_frames);
    cudaError_t e = pinned_alloc(&b->host, b->bytes);
    if (e == cudaSuccess) e = dev_alloc(&b->dev, b->bytes);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->copied, cudaEventDisableTiming);
    if (e != cudaSuccess) {
        cudaGetLastError();
        if (b->host) cudaFreeHost(b->host);
        if (b->dev) cudaFree(b->dev);
        delete b;
        return fail(GBT_ERR_ALLOC, "batch tables: %s", cudaGetErrorString(e));
    }
    *out = b;
    return GBT_OK;
}

gbt_status gbt_batch_destroy(gbt_batch* b) {
    if (!b) return GBT_OK;
    if (b->pending) cudaEventSynchronize(b->copied);
    cudaEventDestroy(b->copied);
    cudaFreeHost(b->host);
    cudaFree(b->dev);
    delete b;
    return GBT_OK;
}

gbt_status gbt_integrate_batch(gbt_batch* b, const gbt_batch_item* items, int32_t nitems, const gbt_frame* frames,
                               int32_t nframes, int32_t frames_per_launch, int32_t brick, int32_t ctas_per_sm,
                               void* stream) {
    gbt::TraceRange trace_("gbt_integrate_batch");
    if (!b || !items || !frames) return fail(GBT_ERR_INVALID_ARG, "batch, items or frames is NULL");
    if (nitems < 1 || nitems > b->max_scenes) return fail(GBT_ERR_INVALID_ARG, "nitems %d outside 1..%d", nitems, b->max_scenes);
    if (nframes < 1 || nframes > b->max_frames)
        return fail(GBT_ERR_INVALID_ARG, "nframes %d outside 1..%d", nframes, b->max_frames);
    if (frames_per_launch < 1 || frames_per_launch > GBT_MAX_FRAMES_PER_SCENE_PASS)
        return fail(GBT_ERR_INVALID_ARG, "frames_per_launch %d outside 1..%d", frames_per_launch,
                    GBT_MAX_FRAMES_PER_SCENE_PASS);
    if (brick < 0 || brick > 3) return fail(GBT_ERR_INVALID_ARG, "brick %d outside 0..3", brick);
    if (ctas_per_sm < 0 || ctas_per_sm > 32) return fail(GBT_ERR_INVALID_ARG, "ctas_per_sm %d outside 0..32", ctas_per_sm);
    const gbt_volume* v0 = items[0].volume;
    if (!v0) return fail(GBT_ERR_INVALID_ARG, "item 0 has no volume");
    int32_t longest = 0;
    for (int i = 0; i < nitems; ++i) {
        const gbt_batch_item& it = items[i];
        if (!it.volume) return fail(GBT_ERR_INVALID_ARG, "item %d has no volume", i);
        if (it.volume->cfg.mode != v0->cfg.mode || it.volume->cfg.arith != v0->cfg.arith)
            return fail(GBT_ERR_INVALID_ARG, "item %d: all volumes of a batch need the same mode and arithmetic", i);
        if (it.nframes < 0 || it.first_frame < 0 || it.first_frame + it.nframes > nframes)
            return fail(GBT_ERR_INVALID_ARG, "item %d: frames [%d, %d) outside the frame table", i, it.first_frame,
                        it.first_frame + it.nframes);
        for (int j = 0; j < i; ++j) {
            if (items[j].volume == it.volume) return fail(GBT_ERR_INVALID_ARG, "item %d repeats a volume", i);
            const bool overlap = it.first_frame < items[j].first_frame + items[j].nframes &&
                                 items[j].first_frame < it.first_frame + it.nframes;
            const gbt_volume_cfg& a = it.volume->cfg;
            const gbt_volume_cfg& c = items[j].volume->cfg;
            if (overlap && a.mode == GBT_MODE_FIXED &&
                (a.focal_x != c.focal_x || a.focal_y != c.focal_y || a.cx != c.cx || a.cy != c.cy))
                return fail(GBT_ERR_INVALID_ARG, "items %d and %d share frames but not intrinsics", j, i);
        }
        if (it.nframes > longest) longest = it.nframes;
    }
    for (int i = 0; i < nframes; ++i) {
        gbt_status st = check_frames(frames + i, 1);
        if (st != GBT_OK) return st;
    }
    const int nwin = (longest + frames_per_launch - 1) / frames_per_launch;
    if (nwin > 64) return fail(GBT_ERR_INVALID_ARG, "%d frames per scene need more than 64 launches", longest);
    cudaStream_t s = as_stream(stream);
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    cudaStreamIsCapturing(s, &cap);
    // the staging area is rewritten below: wait for the previous call's copy
    // (a copy recorded into a graph reads the staging area at each replay,
    // so a graph holds at most one call per batch object)
    if (b->pending && cap == cudaStreamCaptureStatusNone) cudaEventSynchronize(b->copied);
    b->pending = false;

    int bx, by, bz;
    gbt::brick_extent(brick, &bx, &by, &bz);
    gbt::BatchScene* hs = reinterpret_cast<gbt::BatchScene*>(static_cast<char*>(b->host) + 256);
    gbt::FrameDesc* hf = reinterpret_cast<gbt::FrameDesc*>(hs + b->max_scenes);
    for (int i = 0; i < nframes; ++i) {
        const gbt_frame& f = frames[i];
        gbt::FrameDesc& fd = hf[i];
        std::memset(&fd, 0, sizeof(fd));
        fd.depth = f.depth;
        fd.pitch = (int64_t)f.pitch_bytes;
        fd.width = f.width;
        fd.height = f.height;
        fd.fmt = f.format;
        fd.scale = f.depth_scale;
        fd.q[0] = (float)f.pose[1];
        fd.q[1] = (float)f.pose[2];
        fd.q[2] = (float)f.pose[3];
        fd.q[3] = (float)f.pose[0];
        fd.t[0] = (float)f.pose[4];
        fd.t[1] = (float)f.pose[5];
        fd.t[2] = (float)f.pose[6];
    }
    // scenes ordered by frame count, most first: the scenes with frames in a
    // window are then a prefix of the table
    std::vector<int> ord(nitems);
    for (int i = 0; i < nitems; ++i) ord[i] = i;
    std::stable_sort(ord.begin(), ord.end(), [&](int a, int c) { return items[a].nframes > items[c].nframes; });
    long long bricks = 0;
    for (int k = 0; k < nitems; ++k) {
        const gbt_batch_item& it = items[ord[k]];
        gbt::BatchScene& sc = hs[k];
        std::memset(&sc, 0, sizeof(sc));
        sc.vol = it.volume->desc;
        sc.first_frame = it.first_frame;
        sc.nframes = it.nframes;
        sc.nbx = (sc.vol.nx + bx - 1) / bx;
        sc.nby = (sc.vol.ny + by - 1) / by;
        sc.nbz = (sc.vol.nz + bz - 1) / bz;
        sc.div_nbx = gbt::make_fastdiv((uint32_t)sc.nbx);
        sc.div_nby = gbt::make_fastdiv((uint32_t)sc.nby);
        sc.brick_begin = bricks;
        bricks += (long long)sc.nbx * sc.nby * sc.nbz;
        if (it.volume->cfg.mode == GBT_MODE_FIXED)
            for (int f = it.first_frame; f < it.first_frame + it.nframes; ++f)
                fixed_projection(frames[f].pose, it.volume->cfg, hf[f].P);
    }
    if (longest == 0) return GBT_OK;

    const size_t used = 256 + (size_t)b->max_scenes * sizeof(gbt::BatchScene) + (size_t)nframes * sizeof(gbt::FrameDesc);
    std::memset(b->host, 0, 256);   // one zeroed ticket per launch
    cudaError_t e = cudaMemcpyAsync(b->dev, b->host, used, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaEventRecord(b->copied, s);
    if (e != cudaSuccess) return cuda_fail(e, "batch tables upload");
    b->pending = cap == cudaStreamCaptureStatusNone;

    char* d = static_cast<char*>(b->dev);
    cudaGetLastError();  // a launch reports only its own failure
    const long long per_sm =
        ctas_per_sm ? ctas_per_sm : gbt::integrate_default_ctas_per_sm(v0->cfg.mode, v0->cfg.arith, 2, brick);
    for (int w = 0; w < nwin; ++w) {
        gbt::BatchArgs a;
        std::memset(&a, 0, sizeof(a));
        a.ticket = reinterpret_cast<unsigned int*>(d) + w;
        a.scenes = reinterpret_cast<const gbt::BatchScene*>(d + 256);
        a.frames = reinterpret_cast<const gbt::FrameDesc*>(a.scenes + b->max_scenes);
        a.w0 = w * frames_per_launch;
        a.wn = frames_per_launch;
        a.rows_of_4 = 1;
        for (int j = 0; j < nitems; ++j)
            if (items[j].volume->desc.nx % 4 != 0) a.rows_of_4 = 0;
        int m = 0;
        while (m < nitems && hs[m].nframes > a.w0) ++m;
        a.nscenes = m;
        a.total_bricks = m < nitems ? hs[m].brick_begin : bricks;
        long long grid = (long long)device_sms() * per_sm;
        if (grid > a.total_bricks) grid = a.total_bricks;
        if (v0->cfg.mode == GBT_MODE_FIXED)
            e = gbt::launch_batch_fixed(a, brick, (int)grid, s);
        else if (v0->cfg.arith == GBT_ARITH_IEEE)
            e = gbt::launch_batch_compat_ieee(a, brick, (int)grid, s);
        else
            e = gbt::launch_batch_compat_ref(a, brick, (int)grid, s);
        if (e != cudaSuccess) return cuda_fail(e, "batch integrate launch");
    }
    return GBT_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Differentiable integrate.

namespace {

gbt_status diff_args(const gbt_diff_cfg* c, int32_t nframes, gbt::DiffArgs* a) {
    if (!c) return fail(GBT_ERR_INVALID_ARG, "cfg is NULL");
    if (c->dtype != 0 && c->dtype != 1) return fail(GBT_ERR_INVALID_ARG, "dtype %d is not 0 or 1", c->dtype);
    for (int i = 0; i < 3; ++i) {
        if (c->voxel_grid_size[i] == 0 || !(c->voxel_size[i] > 0.f))
            return fail(GBT_ERR_INVALID_ARG, "grid/voxel size %d must be positive", i);
        // (the kernels keep each extent in 32-bit signed integers)
        if (c->voxel_grid_size[i] > (1u << 24)) return fail(GBT_ERR_INVALID_ARG, "voxel_grid_size[%d] above 2^24", i);
    }
    const int64_t n = grid_voxels(c->voxel_grid_size);
    if (n < 0) return fail(GBT_ERR_INVALID_ARG, "more than 2^32-1 voxels");
    if (!(c->truncation > 0.f) || !(c->max_weight > 0.f) || !(c->max_depth > 0.f))
        return fail(GBT_ERR_INVALID_ARG, "truncation, max_depth and max_weight must be > 0");
    if (c->width < 2 || c->height < 2) return fail(GBT_ERR_INVALID_ARG, "depth images need at least 2x2 pixels");
    if (nframes < 1 || nframes > GBT_MAX_FRAMES_PER_SCENE_PASS)
        return fail(GBT_ERR_INVALID_ARG, "nframes %d outside 1..%d", nframes, GBT_MAX_FRAMES_PER_SCENE_PASS);
    std::memset(a, 0, sizeof(*a));
    a->nx = (int32_t)c->voxel_grid_size[0];
    a->ny = (int32_t)c->voxel_grid_size[1];
    a->nz = (int32_t)c->voxel_grid_size[2];
    for (int i = 0; i < 3; ++i) {
        a->vs[i] = c->voxel_size[i];
        a->off[i] = c->global_offset[i];
    }
    a->fx = c->focal_x;
    a->fy = c->focal_y;
    a->cx = c->cx;
    a->cy = c->cy;
    a->trunc = c->truncation;
    a->max_weight = c->max_weight;
    a->max_depth = c->max_depth;
    a->min_z = c->min_z;
    a->width = c->width;
    a->height = c->height;
    a->nframes = nframes;
    a->dtype = c->dtype;
    return GBT_OK;
}

}  // namespace

extern "C" {

gbt_status gbt_diff_forward(const gbt_diff_cfg* cfg, void* tsdf, void* weights, void* checkpoints,
                            uint32_t* signature, const void* depth, int32_t nframes, const void* rot,
                            const void* trans, void* stream) {
    gbt::TraceRange trace_("gbt_diff_forward");
    gbt::DiffArgs a;
    gbt_status st = diff_args(cfg, nframes, &a);
    if (st != GBT_OK) return st;
    if (!tsdf || !weights || !depth || !rot || !trans) return fail(GBT_ERR_INVALID_ARG, "gbt_diff_forward: NULL tensor");
    a.D = tsdf;
    a.W = weights;
    a.ckpt = checkpoints;
    a.signature = signature;
    a.depth = depth;
    a.rot = rot;
    a.trans = trans;
    cudaGetLastError();
    cudaError_t e = gbt::launch_diff_forward(a, as_stream(stream));
    if (e != cudaSuccess) return cuda_fail(e, "differentiable forward");
    return GBT_OK;
}

gbt_status gbt_diff_backward(const gbt_diff_cfg* cfg, const void* grad_tsdf, const void* grad_weights,
                             const void* tsdf_before, const void* weights_before, const void* checkpoints,
                             const void* depth, int32_t nframes, const void* rot, const void* trans,
                             void* grad_depth, double* grad_pose, void* grad_tsdf_before,
                             void* grad_weights_before, void* stream) {
    gbt::TraceRange trace_("gbt_diff_backward");
    gbt::DiffArgs a;
    gbt_status st = diff_args(cfg, nframes, &a);
    if (st != GBT_OK) return st;
    if (!grad_tsdf || !tsdf_before || !weights_before || !depth || !rot || !trans || !grad_depth || !grad_pose)
        return fail(GBT_ERR_INVALID_ARG, "gbt_diff_backward: NULL tensor");
    if (nframes > GBT_DIFF_CHUNK_FRAMES && !checkpoints)
        return fail(GBT_ERR_INVALID_ARG, "gbt_diff_backward: more than %d frames need the forward's checkpoints",
                    GBT_DIFF_CHUNK_FRAMES);
    a.grad_D = grad_tsdf;
    a.grad_W = grad_weights;
    a.D = const_cast<void*>(tsdf_before);
    a.W = const_cast<void*>(weights_before);
    a.ckpt = const_cast<void*>(checkpoints);
    a.depth = depth;
    a.rot = rot;
    a.trans = trans;
    a.grad_depth = grad_depth;
    a.grad_pose = grad_pose;
    a.grad_D0 = grad_tsdf_before;
    a.grad_W0 = grad_weights_before;
    cudaGetLastError();
    cudaError_t e = gbt::launch_diff_backward(a, as_stream(stream));
    if (e != cudaSuccess) return cuda_fail(e, "differentiable backward");
    return GBT_OK;
}

gbt_status gbt_extract_mesh_indexed(gbt_volume* v, float* verts, float* normals, int32_t* tris, int64_t cap_verts,
                                    int64_t cap_tris, int64_t index_base, int64_t* n_verts, int64_t* n_tris,
                                    void* stream) {
    gbt::TraceRange trace_("gbt_extract_mesh_indexed");
    if (!n_verts || !n_tris) return fail(GBT_ERR_INVALID_ARG, "gbt_extract_mesh_indexed: n_verts or n_tris is NULL");
    *n_verts = 0;
    *n_tris = 0;
    if (!v) return fail(GBT_ERR_INVALID_ARG, "volume is NULL");
    if (v->cfg.mode != GBT_MODE_FIXED)
        return fail(GBT_ERR_INVALID_ARG,
                    "gbt_extract_mesh_indexed: fixed mode only (compat emits three vertices per triangle, as the "
                    "reference does)");
    if (cap_verts < 0 || (cap_verts > 0 && !verts)) return fail(GBT_ERR_INVALID_ARG, "vertex buffer is NULL");
    gbt::McArgs a;
    gbt_status st = mc_prepare(v, nullptr, tris, cap_tris, index_base, &a, true);
    if (st != GBT_OK) return st;
    const gbt::VolDesc& d = v->desc;
    gbt::WeldArgs w;
    std::memset(&w, 0, sizeof(w));
    w.nwords = (3 * v->nvox + 31) / 32;
    w.nblocks = (w.nwords + gbt::kWeldWordsPerBlock - 1) / gbt::kWeldWordsPerBlock;
    const size_t need = 64 + (size_t)w.nwords * 8 + (size_t)w.nblocks * 4;
    if (v->weld_scratch_bytes < need) {
        if (v->weld_scratch) cudaFree(v->weld_scratch);
        v->weld_scratch = nullptr;
        v->weld_scratch_bytes = 0;
        cudaError_t e = dev_alloc(&v->weld_scratch, need);
        if (e != cudaSuccess) {
            cudaGetLastError();
            return fail(GBT_ERR_ALLOC, "allocating %zu bytes of vertex-sharing scratch: %s", need, cudaGetErrorString(e));
        }
        v->weld_scratch_bytes = need;
    }
    char* sp = static_cast<char*>(v->weld_scratch);
    w.nverts = reinterpret_cast<long long*>(sp);
    w.bits = reinterpret_cast<uint32_t*>(sp + 64);
    w.word_offset = w.bits + w.nwords;
    w.block_sums = w.word_offset + w.nwords;
    (void)d;
    cudaStream_t s = as_stream(stream);
    cudaGetLastError();
    cudaError_t e = cudaMemsetAsync(w.bits, 0, (size_t)w.nwords * 4, s);
    if (e != cudaSuccess) return cuda_fail(e, "vertex-sharing scratch clear");
    w.mc = a;
    e = gbt::launch_weld_fixed(w, s);
    if (e != cudaSuccess) return cuda_fail(e, "edge marking");
    long long nv = 0;
    e = cudaMemcpyAsync(&nv, w.nverts, sizeof(nv), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_fail(e, "vertex count");
    if (nv > (long long)INT32_MAX - (index_base > 0 ? index_base : 0))
        return fail(GBT_ERR_INVALID_ARG, "%lld vertices do not fit 32-bit triangle indices", nv);
    *n_verts = nv;
    if (verts && cap_verts > 0) {
        w.verts = verts;
        w.normals = normals;
        w.cap_verts = cap_verts;
        e = gbt::launch_weld_vertices_fixed(w, s);
        if (e != cudaSuccess) return cuda_fail(e, "vertices");
    }
    a.edge_bits = w.bits;
    a.edge_word_offset = w.word_offset;
    st = mc_launch(v, a, s);
    if (st != GBT_OK) return st;
    struct {
        unsigned int ticket;
        int error;
        long long total;
    } hdr;
    e = cudaMemcpyAsync(&hdr, v->mc_scratch, sizeof(hdr), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_fail(e, "mesh extraction");
    if (hdr.error) return fail(GBT_ERR_CUDA, "mesh extraction: the kernels set their error word");
    *n_tris = hdr.total;
    if ((hdr.total > cap_tris && cap_tris > 0) || (nv > cap_verts && cap_verts > 0))
        return fail(GBT_ERR_CAPACITY, "mesh has %lld vertices and %lld triangles, buffers hold %lld and %lld", nv,
                    hdr.total, (long long)cap_verts, (long long)cap_tris);
    return GBT_OK;
}

}  // extern "C"
