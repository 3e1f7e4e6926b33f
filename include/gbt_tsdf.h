/*
 * gbt_tsdf.h -- C ABI of the GB300 TSDF surface-fusion engine.
 *
 * This is the drop-in boundary for the TSDF path of cu-Reconstruction
 * (namespace cuphoto).  The reference has no C ABI: its entry points are the
 * C++ members of cuphoto::TSDFVolume and the free function
 * cuphoto::generate_triangular_surface.  Each entry point below names the
 * reference interface it replaces; the C++ shim in
 * cu-reconstruction_gb300/cpp/ rebuilds those C++ signatures on top of it.
 *
 * Conventions
 *   - Every function returns a gbt_status; on failure gbt_last_error() gives a
 *     message for the calling thread.
 *   - Depth images, mesh buffers and streams are borrowed: device pointers
 *     that must stay valid until the work queued on `stream` has finished.
 *   - `stream` is a cudaStream_t passed as void*; NULL is the legacy default
 *     stream.  Calls are asynchronous unless documented otherwise.
 *   - A volume must not be used from two host threads at once.
 */
#ifndef GBT_TSDF_H
#define GBT_TSDF_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    GBT_OK = 0,
    GBT_ERR_INVALID_ARG = 1,   /* bad pointer, size or configuration */
    GBT_ERR_CUDA = 2,          /* a CUDA runtime call failed */
    GBT_ERR_ALLOC = 3,         /* device allocation failed */
    GBT_ERR_CAPACITY = 4,      /* output buffer too small: counts are valid, output truncated */
    GBT_ERR_TIMEOUT = 5,       /* a bounded device-side wait gave up; results are invalid */
    GBT_ERR_IO = 6             /* a file could not be opened, read or written, or is not a volume file */
} gbt_status;

typedef enum {
    /* Reproduces the reference's arithmetic and quirks: SDF against world z,
     * truncating pixel cast, no weight clamp, mesh layer stride gx+gy,
     * three vertices per triangle (tsdf_volume.cu:144-190, marching_cubes.cu:191-237). */
    GBT_MODE_COMPAT = 0,
    /* Geometrically corrected: camera-space SDF, nearest pixel, cameras
     * looking away rejected, weight clamped at max_weight, true layer stride,
     * cubes touching unobserved voxels skipped. */
    GBT_MODE_FIXED = 1
} gbt_mode;

typedef enum {
    /* Divisions compiled as the reference compiles them (-use_fast_math):
     * bit-exact with the reference's own GPU build. */
    GBT_ARITH_REFERENCE = 0,
    /* Correctly rounded IEEE divisions, no flush-to-zero: bit-exact with the
     * CPU oracle. */
    GBT_ARITH_IEEE = 1
} gbt_arith;

typedef enum {
    GBT_DEPTH_F32_M = 0,   /* float metres (the reference's CV_32F depth) */
    GBT_DEPTH_U16 = 1      /* uint16 raw units, metres = raw * depth_scale; 0 = no depth */
} gbt_depth_format;

typedef enum {
    GBT_MEMORY_DEVICE = 0,   /* cudaMalloc */
    GBT_MEMORY_MANAGED = 1   /* cudaMallocManaged, host-readable as in the reference */
} gbt_memory;

/* Mirrors cuphoto::TSDFVolumeConfig (tsdf_volume.cuh:17-29) plus the engine's
 * own options after max_cell_size.  Zero-initialise, then set fields. */
typedef struct {
    uint32_t voxel_grid_size[3];
    float physical_size[3];
    float global_offset[3];
    float max_weight;          /* fixed mode: weight clamp; compat: unused (as in the reference) */
    float focal_x, focal_y, cx, cy;
    uint32_t camera_width, camera_height;   /* informational, as in the reference */
    float max_cell_size;                   /* unused, as in the reference */
    /* engine options */
    int32_t mode;              /* gbt_mode */
    int32_t arith;             /* gbt_arith, compat mode only */
    float truncation;          /* <= 0: 1.1 * |voxel size| (tsdf_volume.cu:199) */
    float max_depth;           /* <= 0: 24 m (tsdf_volume.cu:169) */
    float min_z;               /* fixed mode: nearest accepted camera depth; 0 means z > 0 */
    int32_t memory;            /* gbt_memory */
} gbt_volume_cfg;

/* Derived values a caller may need (voxel size and truncation as computed by
 * the reference's constructor, tsdf_volume.cu:197-199). */
typedef struct {
    uint32_t voxel_grid_size[3];
    float voxel_size[3];
    float truncation;
    float global_offset[3];
    float physical_size[3];
    int64_t num_voxels;
    float* tsdf;               /* device (or managed) pointer, x fastest */
    float* weights;
    int32_t mode;
    int32_t arith;
} gbt_volume_info;

/* One depth frame.  pose = {qw, qx, qy, qz, tx, ty, tz}, the world-to-camera
 * transform, in the order of TSDFVolume::integrate (tsdf_volume.cu:257-272). */
typedef struct {
    const void* depth;         /* device pointer */
    size_t pitch_bytes;        /* row stride in bytes */
    int32_t width, height;
    int32_t format;            /* gbt_depth_format */
    float depth_scale;         /* GBT_DEPTH_U16 only */
    double pose[7];
} gbt_frame;

typedef struct gbt_volume gbt_volume;

/* Replaces TSDFVolume::TSDFVolume + setup_data (tsdf_volume.cu:194-212,227-254):
 * allocates the distance and weight grids and initialises them (distance =
 * truncation, weight = 0).  Synchronises `stream` before returning. */
gbt_status gbt_volume_create(const gbt_volume_cfg* cfg, void* stream, gbt_volume** out);

/* Replaces TSDFVolume::~TSDFVolume (tsdf_volume.cu:214-224). */
gbt_status gbt_volume_destroy(gbt_volume* vol);

/* Re-runs setup_data (tsdf_volume.cu:227-254) on `stream`. */
gbt_status gbt_volume_reset(gbt_volume* vol, void* stream);

/* Checkpoint and resume.  No counterpart in the reference (its volume lives
 * only in memory).  gbt_volume_save writes the volume's configuration and
 * its distance and weight grids to the file `path`: a 256-byte header
 * (GBT_VOLUME_FILE_MAGIC, the header size, sizeof(gbt_volume_cfg), the
 * voxel count and the gbt_volume_cfg the volume was created with, in host
 * byte order), then float32 distances[N] and float32 weights[N], x fastest.
 * gbt_volume_load creates a volume from such a file; integrating further
 * frames into it gives the same bits as integrating all of them into one
 * volume.  Both wait for `stream` (work queued on it before the call is
 * included).  Failures to open, read or write, or a file that is not a
 * volume file of this layout: GBT_ERR_IO. */
#define GBT_VOLUME_FILE_MAGIC "GBTVOL\x00\x01"
#define GBT_VOLUME_FILE_HEADER_BYTES 256
gbt_status gbt_volume_save(const gbt_volume* vol, const char* path, void* stream);
gbt_status gbt_volume_load(const char* path, void* stream, gbt_volume** out);
/* The configuration a volume was created with (for a loaded volume: the
 * saved one). */
gbt_status gbt_volume_get_cfg(const gbt_volume* vol, gbt_volume_cfg* cfg);

/* Replaces the accessors voxel_distances_data, voxel_weights_data,
 * voxel_grid_size, global_offset, scale_voxel_size, voxel_phys_size
 * (tsdf_volume.cuh:57-83). */
gbt_status gbt_volume_get_info(const gbt_volume* vol, gbt_volume_info* info);

/* Synchronises `stream` and reports whether a kernel that worked on the
 * volume gave up a bounded device-side wait (GBT_ERR_TIMEOUT: the volume's
 * contents are undefined until gbt_volume_reset or a load; the mark is
 * cleared by this call).  No counterpart in the reference, whose kernels do
 * not wait on the GPU. */
gbt_status gbt_volume_check(gbt_volume* vol, void* stream);

/* Replaces transformation_voxels_data (tsdf_volume.cuh:86-92).  The engine
 * never stores the per-voxel {float3 centre, float4 quaternion} records; the
 * first call materialises them (28 bytes per voxel, packed as in
 * tsdf_volume.cuh:33-38) and later calls return the same buffer. */
gbt_status gbt_volume_transformation_voxels(gbt_volume* vol, void* stream, void** out);

/* Replaces TSDFVolume::integrate(color, depth, pose) (tsdf_volume.cu:257-290)
 * for `nframes` frames at once: the frames are applied in order, in one
 * pass over the volume (distance and weight read and written once).
 * nframes may be 1..GBT_MAX_FRAMES_PER_PASS.  Asynchronous. */
#define GBT_MAX_FRAMES_PER_PASS 32
gbt_status gbt_integrate(gbt_volume* vol, const gbt_frame* frames, int32_t nframes, void* stream);

/* Same as gbt_integrate with an explicit tile shape and grid size, for the
 * autotuner.  brick: 0 = 32x4x4 voxels, 1 = 16x8x4, 2 = 32x2x8, 3 = 64x2x4;
 * 4..7 = the same shapes with each warp's depth samples staged in shared
 * memory frame by frame (passes of up to 16 frames; same results);
 * 8 = bricks of 32x4x4 voxels whose distances and weights the Tensor Memory
 * Accelerator copies into shared memory a few bricks ahead of the one being
 * updated (passes of up to 16 frames, x extents that are multiples of 4;
 * same results).  Its waits for those copies are bounded: one that gives up
 * marks the volume (see gbt_volume_check).
 * ctas_per_sm: 0 = as many CTAs as the kernel keeps resident on an SM. */
gbt_status gbt_integrate_tuned(gbt_volume* vol, const gbt_frame* frames, int32_t nframes, int32_t brick,
                               int32_t ctas_per_sm, void* stream);

/* Batched integrate: many volumes ("scenes") of any grid sizes, each with its
 * own frames, in persistent launches that cover all scenes at once.  Extends
 * TSDFVolume::integrate (tsdf_volume.cu:257-290) to many volumes; the
 * reference has no batched form.
 *
 * Item i applies frames[first_frame .. first_frame + nframes) to its volume,
 * in order.  One launch applies the next frames_per_launch (1..128) frames of
 * every scene, so a call makes ceil(longest sequence / frames_per_launch)
 * launches (at most 64).  Volumes of one call must share mode and arithmetic
 * and be distinct; items may share frames only when their intrinsics agree.
 * Results are bit-identical to gbt_integrate on each volume.
 *
 * A gbt_batch owns the device tables of a call (scene and frame descriptors,
 * launch tickets) and a pinned staging copy: a call allocates nothing and
 * records into a CUDA graph as one copy and its launches.  A replay re-reads
 * the staging area as the last call on the batch object left it, so a graph
 * should hold one call per batch object.  One host thread per batch object.
 * brick (0..3) and ctas_per_sm as for gbt_integrate_tuned. */
#define GBT_MAX_FRAMES_PER_SCENE_PASS 128
typedef struct gbt_batch gbt_batch;
typedef struct {
    gbt_volume* volume;
    int32_t first_frame;
    int32_t nframes;
} gbt_batch_item;
gbt_status gbt_batch_create(int32_t max_scenes, int32_t max_frames, gbt_batch** out);
gbt_status gbt_batch_destroy(gbt_batch* batch);
gbt_status gbt_integrate_batch(gbt_batch* batch, const gbt_batch_item* items, int32_t nitems, const gbt_frame* frames,
                               int32_t nframes, int32_t frames_per_launch, int32_t brick, int32_t ctas_per_sm,
                               void* stream);

/* Differentiable integrate.  No counterpart in the reference (its integrate
 * is not differentiable).  It follows the fixed mode with bilinear depth
 * sampling and continuous sample weights, so the volume is differentiable in
 * each depth pixel and in each frame's pose:
 *   c = R p + t, (u, v) = (fx c.x/z + cx, fy c.y/z + cy),
 *   the 2x2 pixel footprint around (u, v), bilinear weights b_i, validity
 *     v_i = 1 for a pixel inside the image with depth in (0, max_depth],
 *   wv = sum b_i v_i, d = sum b_i v_i depth_i / wv, sdf = d - z,
 *   tsdf = min(sdf, truncation), w = wv * ramp((sdf + tr)/(tr/2)),
 *     ramp = clamp(., 0, 1), tr = truncation,
 *   D += w (tsdf - D)/(W + w), W = min(W + w, max_weight)    (for w > 0)
 * for z > min_z and u, v in (-1, width), (-1, height).  The sample weight
 * falls to zero continuously as the footprint leaves the image or the valid
 * depth and at the back of the truncation band, which keeps D and W
 * continuous (z = min_z is the one hard cut).
 *
 * Tensors are caller-owned device arrays of `dtype` (0 float32, 1 float64):
 * tsdf/weights [nz][ny][nx], depth [nframes][height][width] metres,
 * rot [nframes][9] (row-major world-to-camera rotation), trans [nframes][3].
 * nframes <= GBT_MAX_FRAMES_PER_SCENE_PASS per call. */
#define GBT_DIFF_CHUNK_FRAMES 8
typedef struct {
    uint32_t voxel_grid_size[3];
    float voxel_size[3];
    float global_offset[3];
    float focal_x, focal_y, cx, cy;
    float truncation;        /* > 0 */
    float max_weight;        /* > 0 */
    float max_depth;         /* > 0 */
    float min_z;
    int32_t width, height;   /* depth image size */
    int32_t dtype;           /* 0 float32, 1 float64 */
} gbt_diff_cfg;

/* Forward: updates tsdf/weights in place.  checkpoints (needed by the
 * adjoint, else NULL) receives (tsdf, weights) before every chunk of
 * GBT_DIFF_CHUNK_FRAMES frames after the first: (ceil(nframes/8) - 1) x 2 x
 * nvoxels values of dtype.  signature (optional) receives a per-voxel hash of
 * the discrete decisions (footprint cell, ramp and clamp states): voxels
 * whose hash changes between two inputs are not smooth between them. */
gbt_status gbt_diff_forward(const gbt_diff_cfg* cfg, void* tsdf, void* weights, void* checkpoints,
                            uint32_t* signature, const void* depth, int32_t nframes, const void* rot,
                            const void* trans, void* stream);

/* Adjoint of gbt_diff_forward (reverse mode, frame-chunk recomputation from
 * the checkpoints; no per-frame volumes).  Inputs: dL/dtsdf and, optionally,
 * dL/dweights of the final volume, the volume before the forward and the
 * forward's checkpoints.  Adds dL/ddepth into grad_depth ([nframes][height]
 * [width] of dtype) and dL/dR, dL/dt into grad_pose ([nframes][12] float64:
 * 9 row-major, then 3); writes dL/dtsdf and dL/dweights of the volume before
 * the forward when those pointers are not NULL (for chaining calls).  In
 * float32 the per-frame pose sums are formed in float32 per CTA and added
 * across CTAs in float64. */
gbt_status gbt_diff_backward(const gbt_diff_cfg* cfg, const void* grad_tsdf, const void* grad_weights,
                             const void* tsdf_before, const void* weights_before, const void* checkpoints,
                             const void* depth, int32_t nframes, const void* rot, const void* trans,
                             void* grad_depth, double* grad_pose, void* grad_tsdf_before,
                             void* grad_weights_before, void* stream);

/* Replaces generate_triangular_surface (marching_cubes.cu:191-237).
 * Writes up to cap_tris triangles: verts gets 9 floats per triangle (three
 * vertices, no sharing, as the reference emits them) and tris gets 3 ints per
 * triangle, (index_base + 3t, +1, +2).  *n_tris receives the full count.
 * Triangles come out in the reference's order: cube z, y, x, then table order.
 * Synchronises `stream`.  Returns GBT_ERR_CAPACITY if the count exceeds cap_tris
 * (the first cap_tris triangles are still written).  verts/tris may be NULL
 * when cap_tris is 0 (count only).  With cap_tris > 0 the indices must fit
 * int32: index_base >= 0 and index_base + 3 * cap_tris <= 2^31, else
 * GBT_ERR_INVALID_ARG before anything is written (also for the _async and
 * _noalloc forms). */
gbt_status gbt_extract_mesh(gbt_volume* vol, float* verts, int32_t* tris, int64_t cap_tris, int64_t index_base,
                            int64_t* n_tris, void* stream);

/* Asynchronous form of gbt_extract_mesh: the count is written to the device
 * word *d_n_tris (the kernels' raw total, also if they set their error word)
 * and nothing is synchronised; usable inside stream capture once the volume
 * has been meshed before (its first mesh may allocate the tile scratch). */
gbt_status gbt_extract_mesh_async(gbt_volume* vol, float* verts, int32_t* tris, int64_t cap_tris,
                                  int64_t index_base, int64_t* d_n_tris, void* stream);

/* Fixed-mode mesh with shared vertices and normals.  No counterpart in the
 * reference (its mesh has three vertices per triangle, which the compat mode
 * keeps).  The triangles are those of gbt_extract_mesh, in the same order;
 * each grid edge crossed by the surface gives one vertex, at the position
 * gbt_extract_mesh writes for it (bit for bit), and tris holds 3 vertex
 * indices per triangle (index_base + vertex).  normals (NULL: none) gets the
 * unit normal of the interpolated central-difference gradient of the
 * distances, pointing to free space.  Synchronises `stream`; counts are
 * returned in *n_verts, *n_tris; GBT_ERR_CAPACITY if either exceeds its
 * buffer (outputs then partial); verts/tris may be NULL with capacity 0
 * (counts only).  Fixed-mode volumes only. */
gbt_status gbt_extract_mesh_indexed(gbt_volume* vol, float* verts, float* normals, int32_t* tris, int64_t cap_verts,
                                    int64_t cap_tris, int64_t index_base, int64_t* n_verts, int64_t* n_tris,
                                    void* stream);

/* Mesh extraction for callers that cannot allocate device memory.
 *
 * No counterpart in the reference: it is an engine addition.  It is meant for
 * code that must not call cudaMalloc once it is running -- work recorded
 * while a CUDA graph is captured in the global capture mode, where cudaMalloc
 * fails, or applications whose device memory is all owned by their own pool
 * or fixed budget.  gbt_extract_mesh may cudaMalloc scratch on a volume's
 * first mesh; this call never allocates: its scratch is one file-scope
 * device array of GBT_NOALLOC_SCRATCH_BYTES (3 MiB) that every GPU using the
 * library holds until the process exits.  That limits it to volumes of at
 * most GBT_NOALLOC_MAX_CUBES cubes (a 512^3 grid fits); larger volumes get
 * GBT_ERR_INVALID_ARG.
 *
 * Output as gbt_extract_mesh_async: up to cap_tris triangles into verts/tris
 * and the count into the device word *d_n_tris.  Asynchronous on `stream`.
 * One difference: if the kernels set their error word (none of the current
 * kernels ever does), *d_n_tris receives -1 here, where the _async form
 * copies the raw total.
 *
 * The first call on a device resolves the array's address (and may load the
 * library's device code), so make that first call before any stream capture.
 * The address is kept per device for the life of the process: after
 * cudaDeviceReset the module is loaded again, and this call must not be used
 * in that process any more.
 * All calls share the one array and it keeps the previous call's contents:
 * each call clears it on `stream` first, and calls whose work overlaps on the
 * GPU (other streams, other host threads) race -- serialise them.
 * Failures are described by gbt_last_error(). */
#define GBT_NOALLOC_SCRATCH_BYTES (3 << 20)
#define GBT_NOALLOC_MAX_CUBES ((int64_t)((GBT_NOALLOC_SCRATCH_BYTES - 64 - 4096) / 16) * 1024)
gbt_status gbt_extract_mesh_noalloc(gbt_volume* vol, float* verts, int32_t* tris, int64_t cap_tris,
                                    int64_t index_base, int64_t* d_n_tris, void* stream);

/* ---- Point clouds ---------------------------------------------------------
 * The reference's cudaPointCloud (cuda_point_cloud.cuh:13-103,
 * cuda_point_cloud.cu:22-385): depth back-projection, rigid transform, and
 * the z-buffer projection that turns a cloud into the colour + depth images
 * integrate takes.  Arithmetic as the reference's: back-projection in double
 * rounded to float; poses as float quaternion + translation applied as the
 * TSDF kernels apply them; pixels by truncation of (x*fx)/z + c.
 *
 * camera_matrix: the reference's std::array<double, 9>, read as the
 * reference reads it, which differs between the two directions:
 *   back-projection (point_cloud_extract, :44-47): fx = m[0], fy = m[4],
 *     cx = m[6], cy = m[7]  (the array holds a column-major 3x3);
 *   projection (project_to_depth / project_to_color_depth, :248-251, :311-314):
 *     fx = m[0], fy = m[4], cx = m[2], cy = m[5]  (row-major). */

/* cudaPointCloud::Vertex (cuda_point_cloud.cuh:17-28): packed, 33 bytes. */
#pragma pack(push, 1)
typedef struct {
    float pos[3];
    float normal[4];
    uint8_t color[3];
    uint16_t class_id;
} gbt_point;
#pragma pack(pop)

/* Replaces point_cloud_extract + cudaPointCloud::extract_points
 * (cuda_point_cloud.cu:23-70,179-226).  For every pixel (x, y) with depth > 0
 * writes points[start_index + y*width + x] = {R*p + t, normal 0, colour, class 0}
 * with p = ((x - cx) d / fx, (y - cy) d / fy, d); pixels with depth <= 0 leave
 * their slot untouched.  depth: float32 metres or uint16 (GBT_DEPTH_*, times
 * depth_scale), pitched; color_rgb8: 3 bytes per pixel, pitched, or NULL for
 * white points.  pose {qw,qx,qy,qz,tx,ty,tz}.  Returns GBT_ERR_CAPACITY
 * (nothing written) when start_index + width*height > capacity: the
 * reference writes past a too-small cloud. */
gbt_status gbt_points_extract(const double camera_matrix[9], const void* depth, int64_t depth_pitch_bytes,
                              int32_t depth_format, float depth_scale, const uint8_t* color_rgb8,
                              int64_t color_pitch_bytes, int32_t width, int32_t height, const double pose[7],
                              int64_t start_index, gbt_point* points, int64_t capacity, void* stream);

/* Replaces transform_points + cudaPointCloud::transform
 * (cuda_point_cloud.cu:73-86,356-385): pos = R*pos + t for n points. */
gbt_status gbt_points_transform(gbt_point* points, int64_t n, const double pose[7], void* stream);

/* Bytes of scratch gbt_points_project needs for a width x height image. */
#define GBT_POINTS_PROJECT_SCRATCH_BYTES(width, height) ((size_t)(width) * (size_t)(height) * 8u)

/* Replaces cudaPointCloud::project_to_depth / project_to_color_depth
 * (cuda_point_cloud.cu:229-353), whose z-buffer is a host loop, with a GPU
 * z-buffer that gives the same images: each point goes through pose, lands on
 * pixel ((int)((x fx)/z + cx), (int)((y fy)/z + cy)) unless z == 0 or the
 * pixel is outside the image, and a pixel keeps the point of smallest z, the
 * lowest point index among equal z (the loop's first-wins order); negative z
 * is not rejected (as in the reference).  depth receives that z, 0 where no
 * point landed (filter_image_if of FLT_MAX to 0); color_rgb8 (NULL: depth
 * only) the point's colour, 0 where none.  scratch: device memory of
 * GBT_POINTS_PROJECT_SCRATCH_BYTES(width, height).  n < 2^32. */
gbt_status gbt_points_project(const gbt_point* points, int64_t n, const double camera_matrix[9], const double pose[7],
                              float* depth, int64_t depth_pitch_bytes, uint8_t* color_rgb8, int64_t color_pitch_bytes,
                              int32_t width, int32_t height, void* scratch, void* stream);

/* Replaces filter_image_if (cuda_point_cloud.cu:89-99): pixels with
 * |value - filter_value| < 1e-10 (util.cu:6-10) become set_value. */
gbt_status gbt_image_filter_if(float* image, int64_t pitch_bytes, int32_t width, int32_t height, float filter_value,
                               float set_value, void* stream);


/* Message for the last failure on the calling thread ("" if none). */
const char* gbt_last_error(void);

/* Host-side failure injection, for tests of the error paths.  No counterpart
 * in the reference, whose constructor swallows exactly these failures
 * (tsdf_volume.cu:203-209: a failed cudaMallocManaged is logged and the
 * volume is used anyway).
 *   GBT_INJECT_ALLOC: after `skip` more device, managed or pinned
 *     allocations made by the engine succeed, the next `count` fail as
 *     cudaErrorMemoryAllocation would (nothing is allocated for them).
 *   GBT_INJECT_LAUNCH_ERROR: leaves a launch error pending in the engine's
 *     CUDA runtime, as a caller's failed launch would: a kernel launched with
 *     a block of zero threads, which the runtime refuses on the host.
 *   GBT_INJECT_HOLD_COPY: the next `count` streamed passes (brick 8 of
 *     gbt_integrate_tuned) issue no copy for the first brick of their first
 *     CTA, whose wait for it then gives up after about a second: the pass
 *     ends early and marks the volume for gbt_volume_check.  No memory is
 *     touched that a normal pass would not touch.
 *   GBT_INJECT_NONE: cancels pending allocation failures and held copies.
 * Nothing here faults the GPU. */
enum {
    GBT_INJECT_NONE = 0,
    GBT_INJECT_ALLOC = 1,
    GBT_INJECT_LAUNCH_ERROR = 2,
    GBT_INJECT_HOLD_COPY = 3
};
gbt_status gbt_debug_inject(int32_t what, int64_t skip, int64_t count);

/* Engine version string. */
const char* gbt_version(void);

#ifdef __cplusplus
}
#endif

#endif /* GBT_TSDF_H */
