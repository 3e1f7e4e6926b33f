// Types shared by the engine's translation units: the kernel argument blocks
// and the host-side launchers each kernel TU exports.  Not part of the ABI.
#pragma once
#include <cstdint>
#include <cuda.h>
#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include "../../include/gbt_tsdf.h"

namespace gbt {

// A named NVTX range around an entry point of the C ABI: visible in a
// profiler's timeline, a null call when no tool is attached.
struct TraceRange {
    explicit TraceRange(const char* name) { nvtxRangePushA(name); }
    ~TraceRange() { nvtxRangePop(); }
    TraceRange(const TraceRange&) = delete;
    TraceRange& operator=(const TraceRange&) = delete;
};

// Volume as the kernels see it.  D and W are [nz][ny][nx], x fastest.
struct VolDesc {
    float* D;
    float* W;
    int32_t nx, ny, nz;
    int32_t pad0;
    float vs[3];
    float off[3];
    float trunc;
    float max_weight;
    float max_depth;
    float min_z;
    float fx, fy, cx, cy;
};

// One frame as the kernels see it.  q/t: the reference's float quaternion
// (x, y, z, w) and translation; P: rows of K[R|t] for the fixed mode.
struct FrameDesc {
    const void* depth;
    int64_t pitch;
    int32_t width, height;
    int32_t fmt;
    float scale;
    float q[4];
    float t[3];
    float P[12];
};

// How the integrate kernels read a frame's depth samples.
enum SlotFormat : int32_t {
    kSlotF32 = 0,     // float metres
    kSlotU16Fma = 1,  // uint16 x scale as one fused multiply-add (scale normal, 2^23 * scale finite)
    kSlotU16Mul = 2,  // uint16 x scale as a conversion and a multiply (any other scale)
};

// A frame as the integrate kernels keep it in shared memory (80 bytes, five
// 16-byte words): pose table entry, depth image, its row pitch in elements,
// the sample format and the depth scale in both halves of a paired-FP32
// operand.
struct __align__(16) FrameSlot {
    float pose[12];
    const void* depth;
    uint32_t pitch_elems;
    int32_t fmt;
    unsigned long long scale2;
    uint32_t width, height;
};
static_assert(sizeof(FrameSlot) == 80, "five 16-byte words");

// Unsigned 32-bit division by a run-time invariant divisor with one
// multiply-high, after Granlund & Montgomery, "Division by invariant integers
// using multiplication" (PLDI 1994), figure 4.1.
struct FastDiv {
    uint32_t d;
    uint32_t m;
    uint32_t s;
    uint32_t pad0;
};

inline FastDiv make_fastdiv(uint32_t d) {
    FastDiv f{d, 0u, 0u, 0u};
    if (d <= 1) return f;
    uint32_t l = 0;
    while ((1ull << l) < d) ++l;
    f.m = (uint32_t)(((1ull << 32) * ((1ull << l) - d)) / d + 1);
    f.s = l;
    return f;
}

struct IntegrateArgs {
    VolDesc vol;
    int32_t nframes;
    uint32_t nbricks;        // bricks of the volume for the launch's brick shape
    FastDiv div_nbx;         // bricks along x
    FastDiv div_nby;         // bricks along y
    unsigned int* status;    // streamed pass: the volume's status word (kStatusWaitExpired)
    int32_t hold_first_copy; // streamed pass, failure injection: CTA 0 issues no copy for its first brick
    int32_t pad1;
    FrameDesc frames[GBT_MAX_FRAMES_PER_PASS];
};

// The volume's distances and weights as two tensors of the Tensor Memory
// Accelerator ([nz][ny][nx] float, x fastest; a box is one brick of the
// streamed pass kernel, 32 x 4 x 4 voxels).
struct alignas(128) VolumeMaps {
    CUtensorMap d, w;
};
// Brick of the streamed pass kernel and the stages of its shared-memory ring.
constexpr int kStreamBrickX = 32, kStreamBrickY = 4, kStreamBrickZ = 4;
constexpr int kStreamStages = 4;
// Bits of a volume's status word (a device word after its weights).
constexpr unsigned kStatusWaitExpired = 1u;   // a bounded wait of a kernel gave up; the volume is invalid

// Many volumes in one launch.  A scene's bricks are numbered from
// brick_begin; frames [first_frame, first_frame + nframes) of the frame table
// go into its volume.  One launch applies the window [w0, w0 + wn) of every
// scene's frames (wn <= kBatchMaxFrames); scenes are sorted by frame count,
// so the scenes with frames in a window are a prefix of the table.
constexpr int kBatchMaxFrames = GBT_MAX_FRAMES_PER_SCENE_PASS;

struct BatchScene {
    VolDesc vol;
    int32_t first_frame;
    int32_t nframes;
    int32_t nbx, nby, nbz;
    int32_t pad0;
    FastDiv div_nbx;         // nbx
    FastDiv div_nby;         // nby
    long long brick_begin;
};

struct BatchArgs {
    const BatchScene* scenes;
    const FrameDesc* frames;
    int32_t nscenes;        // scenes with frames in this window
    int32_t w0, wn;         // frame window
    int32_t rows_of_4;      // 1: every scene's x extent is a multiple of 4
    long long total_bricks; // bricks of those scenes
    unsigned int* ticket;   // this launch's ticket, zero at launch
};

// Marching cubes over the linear cube order (z, y, x) in tiles of
// mc_tile_cubes(mode) cubes: counted per tile, offsets by a scan of the tile
// counts, then one CTA per tile with triangles emits them.
constexpr int kMcThreads = 256;
// Cubes per thread per tile: 8 in the compat mode (one D load per corner), 4
// in the fixed mode (which also loads W, and keeps twice the values in flight).
__host__ __device__ constexpr int mc_cubes_per_thread(int mode) { return mode == 1 ? 4 : 8; }
__host__ __device__ constexpr int mc_tile_cubes(int mode) { return kMcThreads * mc_cubes_per_thread(mode); }
constexpr int kMcTileMin = kMcThreads * 4;   // the smallest tile of either mode
constexpr int kMcSuperShift = 10;               // tiles per superblock of the tile scan: 1024
inline int64_t mc_superblocks(int64_t ntiles) { return (ntiles + (1 << kMcSuperShift) - 1) >> kMcSuperShift; }
inline int64_t mc_group_words(int64_t ncubes) { return (ncubes + 1023) / 1024; }
// Triangle t of a mesh without shared vertices has the int32 indices
// index_base + 3t, +1, +2: a capacity whose last index would pass
// INT32_MAX, or a negative base, is refused before anything is written
// (a count-only call, capacity 0, is always accepted).
inline bool mc_indices_fit(int64_t cap_tris, int64_t index_base) {
    return cap_tris == 0 ||
           (index_base >= 0 && index_base <= INT32_MAX && cap_tris <= ((int64_t)INT32_MAX + 1 - index_base) / 3);
}

struct McArgs {
    const float* D;
    const float* W;
    int32_t gx, gy, gz;
    int32_t pad0;
    float vs[3];
    float off[3];
    FastDiv div_cx;   // gx - 1
    FastDiv div_cy;   // gy - 1
    FastDiv div_gx;   // gx
    FastDiv div_gy;   // gy
    uint32_t ncubes;
    uint32_t ntiles;
    float* verts;
    int32_t* tris;
    int64_t cap;
    int64_t index_base;
    unsigned long long* status;  // [ntiles] triangles per tile, then exclusive offsets; zeroed before launch
    unsigned long long* super;   // [ceil(ntiles / 1024)][2] triangles and tiles with triangles per
                                 // superblock of 1024 tiles; zeroed before launch
    uint32_t* tile_list;         // [ntiles] tiles with triangles, in order
    uint32_t* group_bits;        // [ceil(ncubes / 1024)] bit g: group g of 32 cubes has triangles; zeroed
    unsigned int* nonempty;      // length of tile_list
    unsigned int* ticket;        // emission ticket, zeroed before launch
    long long* total;            // triangle count out
    int* error;                  // stays 0: no launch waits on another CTA
    // Fixed mode with shared vertices: when edge_bits is set, triangles are
    // written as indices of the vertices of their grid edges (edge
    // 3 * voxel + axis; vertex index = edge_word_offset[edge / 32] + the set
    // bits of edge_bits below it) and verts is not written.
    const uint32_t* edge_bits;
    const uint32_t* edge_word_offset;
};

// Fixed-mode mesh with shared vertices (k_ieee.cu): the edges used by the
// triangles, their vertex numbering and the vertices with normals.
struct WeldArgs {
    McArgs mc;
    uint32_t* bits;          // [nwords] used-edge bitmask
    uint32_t* word_offset;   // [nwords] vertex index of each word's first used edge
    uint32_t* block_sums;    // [nblocks] used edges per block of kWeldWordsPerBlock words
    long long* nverts;       // total out
    int64_t nwords, nblocks;
    float* verts;            // 3 per vertex
    float* normals;          // 3 per vertex, or NULL
    int64_t cap_verts;
};
constexpr int kWeldWordsPerBlock = 1024;

// Differentiable integrate (k_diff.cu).  dtype 0: float, 1: double for the
// volume, depth, rotations and translations; gradients of depth and pose are
// accumulated in double.
struct DiffArgs {
    int32_t nx, ny, nz;
    float vs[3], off[3];
    float fx, fy, cx, cy;
    float trunc, max_weight, max_depth, min_z;
    int32_t width, height, nframes, dtype;
    void* D;                 // forward: in/out distances; backward: distances before the forward
    void* W;                 // forward: in/out weights; backward: weights before the forward
    void* ckpt;              // (D, W) before every chunk after the first: [nchunks-1][2][N]
    uint32_t* signature;     // forward, optional: hash of the discrete decisions per voxel
    const void* depth;       // [nframes][height][width]
    const void* rot;         // [nframes][9] row-major, world to camera
    const void* trans;       // [nframes][3]
    const void* grad_D;      // backward: dL/dD_final
    const void* grad_W;      // backward, optional: dL/dW_final
    void* grad_depth;        // backward: accumulated dL/ddepth (dtype)
    double* grad_pose;       // backward: accumulated [nframes][12] = dL/dR, dL/dt
    void* grad_D0;           // backward, optional: dL/dD before the forward
    void* grad_W0;           // backward, optional: dL/dW before the forward
};

// Launchers exported by the kernel translation units.
// k_ref.cu (-use_fast_math): compat mode in the reference's arithmetic.
cudaError_t launch_integrate_compat_ref(const IntegrateArgs& a, int brick, int grid, cudaStream_t s);
cudaError_t launch_mc_compat_ref(const McArgs& a, cudaStream_t s);
// k_ieee.cu (IEEE arithmetic): compat mode as the oracle computes it, fixed mode.
cudaError_t launch_integrate_compat_ieee(const IntegrateArgs& a, int brick, int grid, cudaStream_t s);
cudaError_t launch_integrate_fixed(const IntegrateArgs& a, int brick, int grid, cudaStream_t s);
cudaError_t launch_mc_compat_ieee(const McArgs& a, cudaStream_t s);
cudaError_t launch_mc_fixed(const McArgs& a, cudaStream_t s);
cudaError_t launch_weld_fixed(const WeldArgs& a, cudaStream_t s);         // marks edges, numbers vertices
cudaError_t launch_weld_vertices_fixed(const WeldArgs& a, cudaStream_t s);
// Batched integrate (one persistent launch over many volumes).
cudaError_t launch_batch_compat_ref(const BatchArgs& a, int brick, int grid, cudaStream_t s);
// CTAs per SM that the (batched or pass) integrate kernel of a brick shape keeps resident.
// kind: 0 pass kernel culling a frame per lane, 1 pass kernel culling a brick per lane, 2 batched kernel,
// 3 kind 1 with the depth staged in shared memory, 4 the streamed pass kernel (brick ignored).
int integrate_resident_ctas_compat_ref(int kind, int brick);
int integrate_resident_ctas_compat_ieee(int kind, int brick);
int integrate_resident_ctas_fixed(int kind, int brick);
// Passes of up to this many frames cull one brick per lane (more frames: one frame per lane).
constexpr int kLaneBrickFrames = 16;
cudaError_t launch_batch_compat_ieee(const BatchArgs& a, int brick, int grid, cudaStream_t s);
cudaError_t launch_batch_fixed(const BatchArgs& a, int brick, int grid, cudaStream_t s);
// Passes of up to kLaneBrickFrames frames whose bricks' distances and weights
// are streamed into shared memory by the Tensor Memory Accelerator (brick 8).
// kind 4 of integrate_resident_ctas_* is this kernel.
cudaError_t launch_stream_compat_ref(const IntegrateArgs& a, const VolumeMaps& m, int grid, cudaStream_t s);
cudaError_t launch_stream_compat_ieee(const IntegrateArgs& a, const VolumeMaps& m, int grid, cudaStream_t s);
cudaError_t launch_stream_fixed(const IntegrateArgs& a, const VolumeMaps& m, int grid, cudaStream_t s);
// k_util.cu: volume initialisation and the packed per-voxel transform records.
cudaError_t launch_volume_init(float* D, float* W, int64_t n, float trunc, cudaStream_t s);
cudaError_t launch_tvoxels(void* out, const VolDesc& v, cudaStream_t s);

cudaError_t launch_diff_forward(const DiffArgs& a, cudaStream_t s);
cudaError_t launch_diff_backward(const DiffArgs& a, cudaStream_t s);

// Read-only views of a volume for translation units other than capi.cu.
const VolDesc* volume_desc(const gbt_volume* v);
int volume_mode(const gbt_volume* v);
int volume_arith(const gbt_volume* v);
// Sets the message gbt_last_error() returns on this thread.
void set_last_error(const char* msg);

// CTAs per SM the integrate launchers use by default, and brick extents.
int integrate_default_ctas_per_sm(int mode, int arith, int kind, int brick);
void brick_extent(int brick, int* bx, int* by, int* bz);

}  // namespace gbt
