// TSDF integrate and marching-cubes kernels.
//
// This header is compiled twice:
//   k_ref.cu   with -use_fast_math and GBT_REF_ARITH defined: the compat mode
//              with the reference's own arithmetic (its divisions are the
//              approximate divide nvcc emits under fast math, its multiply-adds
//              are contracted by the compiler exactly where the reference's are);
//   k_ieee.cu  without fast math: every operation is an explicit IEEE
//              intrinsic, in the order the CPU oracle uses (compat mode), plus
//              the fixed mode.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "compat_geom.cuh"
#include "gbt_internal.h"

#ifndef GBT_ARITH_NS
#error "define GBT_ARITH_NS (one namespace per arithmetic translation unit)"
#endif

#define GBT_MC_CONST static __constant__
#include "mc_tables.inc"
GBT_MC_TABLE_DATA
#undef GBT_MC_CONST

namespace gbt {
// The kernels below are compiled once per arithmetic; each translation unit
// puts them in its own namespace so the two sets never share a symbol.
namespace GBT_ARITH_NS {

enum { kCompat = 0, kFixed = 1 };

// ---------------------------------------------------------------------------
// Arithmetic of the compat mode.  It follows the reference operation for
// operation (se3.cuh:125-140,165-175,207-223; camera_util.cu:15-16;
// tsdf_volume.cu:117-119,183; marching_cubes.cu:43-48) because the compat mode
// must reproduce its results bit for bit.  The rotation and the R*p+t rows
// are in compat_geom.cuh (shared with the point-cloud kernels).

// Two FP32 values in one 64-bit register pair, for Blackwell's paired FP32
// instructions (add/mul/fma .rn .f32x2): two IEEE operations per issue slot,
// each lane rounded exactly as the scalar instruction rounds it.  In the
// fast-math translation unit the scalar operations flush subnormals, so the
// paired ones do too.
#if defined(GBT_REF_ARITH)
#define GBT_F2_FTZ ".ftz"
#else
#define GBT_F2_FTZ ""
#endif
struct f2 {
    unsigned long long r;
};
__device__ __forceinline__ f2 f2_pack(float lo, float hi) {
    f2 v;
    asm("mov.b64 %0, {%1, %2};" : "=l"(v.r) : "f"(lo), "f"(hi));
    return v;
}
__device__ __forceinline__ f2 f2_splat(float x) { return f2_pack(x, x); }
__device__ __forceinline__ float f2_lo(f2 v) {
    float lo;
    asm("mov.b64 {%0, _}, %1;" : "=f"(lo) : "l"(v.r));
    return lo;
}
__device__ __forceinline__ float f2_hi(f2 v) {
    float hi;
    asm("mov.b64 {_, %0}, %1;" : "=f"(hi) : "l"(v.r));
    return hi;
}
__device__ __forceinline__ f2 f2_fma(f2 a, f2 b, f2 c) {
    f2 d;
    asm("fma.rn" GBT_F2_FTZ ".f32x2 %0, %1, %2, %3;" : "=l"(d.r) : "l"(a.r), "l"(b.r), "l"(c.r));
    return d;
}
__device__ __forceinline__ f2 f2_mul(f2 a, f2 b) {
    f2 d;
    asm("mul.rn" GBT_F2_FTZ ".f32x2 %0, %1, %2;" : "=l"(d.r) : "l"(a.r), "l"(b.r));
    return d;
}
__device__ __forceinline__ f2 f2_add(f2 a, f2 b) {
    f2 d;
    asm("add.rn" GBT_F2_FTZ ".f32x2 %0, %1, %2;" : "=l"(d.r) : "l"(a.r), "l"(b.r));
    return d;
}
// compat_cam for two voxels of one row (same y, z): r1*y is shared
__device__ __forceinline__ f2 compat_cam2(float r0, float r2, float t, f2 px, float r1y, float pz) {
    return f2_add(f2_fma(f2_splat(r2), f2_splat(pz), f2_fma(f2_splat(r0), px, f2_splat(r1y))), f2_splat(t));
}

#if defined(GBT_REF_ARITH)

__device__ __forceinline__ float centre(int v, float vs, float off) { return ((float)v + 0.5f) * vs + off; }

// Pixel coordinates (u, v) of two voxels from their camera coordinates,
// ((c * f) / z + cc) as the reference's fast-math build evaluates it: the
// approximate reciprocal of z (serving both u and v), then one fused
// multiply-add.
__device__ __forceinline__ void compat_proj2(f2 cx, f2 cy, f2 cz, float fx, float fy, float ccx, float ccy, f2& qu,
                                             f2& qv) {
    float r0, r1;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r0) : "f"(f2_lo(cz)));
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r1) : "f"(f2_hi(cz)));
    const f2 r = f2_pack(r0, r1);
    qu = f2_fma(f2_mul(cx, f2_splat(fx)), r, f2_splat(ccx));
    qv = f2_fma(f2_mul(cy, f2_splat(fy)), r, f2_splat(ccy));
}
__device__ __forceinline__ float compat_avg(float d, float w, float tsdf, float nw) {
    return ((d * w) + (tsdf * 1.0f)) / nw;
}
__device__ __forceinline__ float mc_ratio(float s, float e) { return (-s) / (e - s); }
__device__ __forceinline__ float mc_lerp(float a, float b, float r) { return a + r * (b - a); }

#else

__device__ __forceinline__ float centre(int v, float vs, float off) {
    return __fmaf_rn(__fadd_rn((float)v, 0.5f), vs, off);
}
__device__ __forceinline__ f2 compat_q2(f2 c, float f, f2 cz, float cc) {
    const f2 m = f2_mul(c, f2_splat(f));
    return f2_add(f2_pack(__fdiv_rn(f2_lo(m), f2_lo(cz)), __fdiv_rn(f2_hi(m), f2_hi(cz))), f2_splat(cc));
}
__device__ __forceinline__ void compat_proj2(f2 cx, f2 cy, f2 cz, float fx, float fy, float ccx, float ccy, f2& qu,
                                             f2& qv) {
    qu = compat_q2(cx, fx, cz, ccx);
    qv = compat_q2(cy, fy, cz, ccy);
}
__device__ __forceinline__ float compat_avg(float d, float w, float tsdf, float nw) {
    return __fdiv_rn(__fmaf_rn(d, w, tsdf), nw);
}
__device__ __forceinline__ float mc_ratio(float s, float e) { return __fdiv_rn(-s, __fsub_rn(e, s)); }
__device__ __forceinline__ float mc_lerp(float a, float b, float r) { return __fmaf_rn(r, __fsub_rn(b, a), a); }

#endif

__device__ __forceinline__ float u16_metres(unsigned short raw, float scale) {
    return __fmul_rn((float)raw, scale);
}

__device__ __forceinline__ uint32_t fastdiv(uint32_t n, const FastDiv& f) {
    if (f.d == 1) return n;
    const uint32_t t = __umulhi(f.m, n);
    return (t + ((n - t) >> 1)) >> (f.s - 1);
}

// ---------------------------------------------------------------------------
// Frustum culling of one warp's box of voxels for one frame, evaluated by the
// lane whose index is the frame number.  The test is conservative: it only
// reports "culled" when every voxel of the box is certain to be rejected by
// the per-voxel test (the projected box lies in the convex hull of its
// projected corners when no corner is near the camera plane), with a margin
// of two pixels and 1e-4 in depth that covers rounding.
template <int MODE>
__device__ __forceinline__ bool box_culled(const VolDesc& v, const FrameSlot& fs, int x_lo, int x_hi, int y_lo, int y_hi,
                                           int z_lo, int z_hi) {
    const float* fr = fs.pose;
    const float X[2] = {centre(x_lo, v.vs[0], v.off[0]), centre(x_hi, v.vs[0], v.off[0])};
    const float Y[2] = {centre(y_lo, v.vs[1], v.off[1]), centre(y_hi, v.vs[1], v.off[1])};
    const float Zw[2] = {centre(z_lo, v.vs[2], v.off[2]), centre(z_hi, v.vs[2], v.off[2])};
    float umin = 3.0e38f, umax = -3.0e38f, vmin = 3.0e38f, vmax = -3.0e38f;
    int npos = 0, nneg = 0, nbehind = 0;
    // depth margin: far above the float rounding of a camera coordinate at this scale
    const float tmax = (MODE == kCompat) ? fmaxf(fabsf(fr[9]), fmaxf(fabsf(fr[10]), fabsf(fr[11])))
                                         : fabsf(fr[11]);
    const float scale = fmaxf(fmaxf(fmaxf(fabsf(X[0]), fabsf(X[1])), fmaxf(fabsf(Y[0]), fabsf(Y[1]))),
                              fmaxf(fmaxf(fabsf(Zw[0]), fabsf(Zw[1])), tmax));
    const float eps = 1e-4f + 1e-5f * scale;
    if (MODE == kCompat) {
        // world z exactly 0 sends a voxel to pixel (0,0) (camera_util.cu:46): keep such boxes
        if (!(Zw[0] > 0.f || Zw[1] < 0.f)) return false;
        if ((Zw[0] > 0.f) != (Zw[1] > 0.f)) return false;
    }
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        const float px = X[k & 1], py = Y[(k >> 1) & 1], pz = Zw[k >> 2];
        float cx, cy, cz;
        if (MODE == kCompat) {
            cx = fr[0] * px + fr[1] * py + fr[2] * pz + fr[9];
            cy = fr[3] * px + fr[4] * py + fr[5] * pz + fr[10];
            cz = fr[6] * px + fr[7] * py + fr[8] * pz + fr[11];
            cx *= v.fx;
            cy *= v.fy;
        } else {
            cx = fr[0] * px + fr[1] * py + fr[2] * pz + fr[3];
            cy = fr[4] * px + fr[5] * py + fr[6] * pz + fr[7];
            cz = fr[8] * px + fr[9] * py + fr[10] * pz + fr[11];
            if (cz <= v.min_z - eps) ++nbehind;
        }
        if (cz > eps)
            ++npos;
        else if (cz < -eps)
            ++nneg;
        const float rz = 1.0f / cz;
        const float u = cx * rz, w = cy * rz;
        umin = fminf(umin, u);
        umax = fmaxf(umax, u);
        vmin = fminf(vmin, w);
        vmax = fmaxf(vmax, w);
    }
    if (MODE == kFixed) {
        if (nbehind == 8) return true;
        // a box reaching behind the camera is only decided by the test above
        if (npos != 8) return false;
        // accepted pixels satisfy -0.5 <= u < width - 0.5
        const float W = (float)fs.width, H = (float)fs.height;
        return umax < -2.5f || umin > W + 1.5f || vmax < -2.5f || vmin > H + 1.5f;
    } else {
        if (npos != 8 && nneg != 8) return false;
        const float ccx = v.cx, ccy = v.cy;
        // truncation keeps pixel k for values in (k-1, k+1) around 0 and [k, k+1) elsewhere
        const float W = (float)fs.width, H = (float)fs.height;
        return umax + ccx < -3.0f || umin + ccx > W + 2.0f || vmax + ccy < -3.0f || vmin + ccy > H + 2.0f;
    }
}

// ---------------------------------------------------------------------------
// Integrate.  One CTA of 128 threads works on a brick of (4*TX) x BY x BZ
// voxels; a thread owns 4 consecutive voxels along x, moved as one 16-byte
// load/store of distance and one of weight.  All frames of the pass are
// applied to the voxels in registers, in frame order, so a voxel sees exactly
// the sequence of updates the per-frame reference loop would apply.

// A frame's shared-memory entry, written once per CTA: the pose table
// (compat -> rotation (9) + translation (3), fixed -> the three rows of
// K[R|t]) and the image description in the form the per-voxel code uses, so
// that a thread reads a frame's constants with a few broadcast shared loads.
template <int MODE>
__device__ __forceinline__ void load_slot(const FrameDesc& fd, FrameSlot& s) {
    if (MODE == kCompat) {
        float R[9];
        compat_rotation(fd.q, R);
#pragma unroll
        for (int k = 0; k < 9; ++k) s.pose[k] = R[k];
        s.pose[9] = fd.t[0];
        s.pose[10] = fd.t[1];
        s.pose[11] = fd.t[2];
    } else {
#pragma unroll
        for (int k = 0; k < 12; ++k) s.pose[k] = fd.P[k];
    }
    const bool u16 = fd.fmt == GBT_DEPTH_U16;
    // the fused form needs 2^23 * scale to be a finite normal float, so that
    // it is exact: a biased exponent in [1, 254 - 23]
    const uint32_t e = (__float_as_uint(fd.scale) >> 23) & 0xFFu;
    s.depth = fd.depth;
    s.pitch_elems = (uint32_t)(u16 ? (fd.pitch >> 1) : (fd.pitch >> 2));
    s.fmt = !u16 ? kSlotF32 : (e >= 1u && e <= 231u) ? kSlotU16Fma : kSlotU16Mul;
    s.scale2 = f2_splat(fd.scale).r;
    s.width = (uint32_t)fd.width;
    s.height = (uint32_t)fd.height;
}

// The thread's 4 depth samples, 0 where `in` is false.  uint16 depth becomes
// metres as convertTo(CV_32F, depth_scale) does (rgbd_dataset.cpp:29): the
// product raw * scale, rounded once.  In the fused form the float with the
// bits of 2^23 OR raw is exactly 2^23 + raw, and fma(2^23 + raw, scale,
// -2^23 * scale) is that same product before its one rounding (the bias
// -2^23 * scale is exact); a product is 0 or at least |scale|, never
// subnormal, so flushing subnormals changes nothing.  Two samples share one
// paired FMA and no integer-to-float conversion is issued.
__device__ __forceinline__ void gather_depth(const FrameSlot& fs, const bool (&in)[4], const uint32_t (&pix)[4],
                                             float (&dv)[4]) {
    const unsigned short* d16 = static_cast<const unsigned short*>(fs.depth);
    const float* d32 = static_cast<const float*>(fs.depth);
    const f2 S{fs.scale2};
    // the format is the same for every thread of the CTA: one gather loop each
    if (fs.fmt == kSlotU16Fma) {
        uint32_t raw[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) raw[i] = in[i] ? (uint32_t)__ldg(d16 + pix[i]) : 0u;
        const f2 B = f2_mul(S, f2_splat(-8388608.0f));
#pragma unroll
        for (int h = 0; h < 4; h += 2) {
            const f2 r = f2_fma(f2_pack(__uint_as_float(raw[h] | 0x4B000000u), __uint_as_float(raw[h + 1] | 0x4B000000u)),
                                S, B);
            dv[h] = f2_lo(r);
            dv[h + 1] = f2_hi(r);
        }
    } else if (fs.fmt == kSlotU16Mul) {
        const float scale = f2_lo(S);
#pragma unroll
        for (int i = 0; i < 4; ++i) dv[i] = in[i] ? u16_metres(__ldg(d16 + pix[i]), scale) : 0.f;
    } else {
#pragma unroll
        for (int i = 0; i < 4; ++i) dv[i] = in[i] ? __ldg(d32 + pix[i]) : 0.f;
    }
}

// Depth staged in shared memory, for one warp and one frame.  The warp's
// pixels (those of its voxels that land on the image) span a rectangle of
// rows [vmin, vmax] and columns [umin, umax] (reductions over the warp); if
// it fits kDepthTileBytes, the warp copies that rectangle of the image into
// its tile with coalesced loads (8-byte chunks when the rows allow it) and
// every voxel reads its sample from the tile; otherwise the voxels gather
// from the image as gather_depth does.  The samples are the same values
// either way (the same conversion of the same pixel).
constexpr int kDepthTileBytes = 4096;

__device__ __forceinline__ void gather_staged(const FrameSlot& fs, const bool (&in)[4], const int (&pu)[4],
                                              const int (&pv)[4], const uint32_t (&pix)[4], float (&dv)[4],
                                              unsigned char* tile) {
    const int lane = threadIdx.x & 31;
    int umin = 0x7fffffff, umax = -1, vmin = 0x7fffffff, vmax = -1;
#pragma unroll
    for (int i = 0; i < 4; ++i)
        if (in[i]) {
            umin = min(umin, pu[i]);
            umax = max(umax, pu[i]);
            vmin = min(vmin, pv[i]);
            vmax = max(vmax, pv[i]);
        }
    umin = __reduce_min_sync(0xffffffffu, umin);
    umax = __reduce_max_sync(0xffffffffu, umax);
    vmin = __reduce_min_sync(0xffffffffu, vmin);
    vmax = __reduce_max_sync(0xffffffffu, vmax);
    if (umax < 0) {   // no voxel of the warp lands on the image (the same for the whole warp)
#pragma unroll
        for (int i = 0; i < 4; ++i) dv[i] = 0.f;
        return;
    }
    const bool u16 = fs.fmt != kSlotF32;
    const int esz = u16 ? 2 : 4;
    const int per8 = 8 / esz;   // elements per 8-byte chunk
    // 8-byte chunks need an 8-byte aligned image and rows of whole chunks
    const bool vec = (reinterpret_cast<uintptr_t>(fs.depth) & 7u) == 0 && (fs.pitch_elems % (uint32_t)per8) == 0;
    const int u0 = vec ? (umin & ~(per8 - 1)) : umin;
    const int nch = vec ? (umax - u0) / per8 + 1 : umax - umin + 1;   // chunks (or elements) per tile row
    const int rowe = vec ? nch * per8 : nch;                          // tile row in elements
    const int th = vmax - vmin + 1;
    if (rowe * th * esz > kDepthTileBytes) {
        gather_depth(fs, in, pix, dv);
        return;
    }
    const unsigned char* img = static_cast<const unsigned char*>(fs.depth);
    const int total = nch * th;
    __syncwarp();   // the previous frame's reads of the tile are done
    for (int k = lane; k < total; k += 32) {
        const int r = k / nch, c = k - r * nch;
        const size_t e = (size_t)(vmin + r) * fs.pitch_elems + (size_t)u0 + (size_t)c * (vec ? per8 : 1);
        if (vec)
            *reinterpret_cast<uint2*>(tile + (size_t)k * 8) = __ldg(reinterpret_cast<const uint2*>(img + e * esz));
        else if (u16)
            reinterpret_cast<unsigned short*>(tile)[k] = __ldg(reinterpret_cast<const unsigned short*>(img) + e);
        else
            reinterpret_cast<float*>(tile)[k] = __ldg(reinterpret_cast<const float*>(img) + e);
    }
    __syncwarp();
    const f2 S{fs.scale2};
    if (fs.fmt == kSlotU16Fma) {
        uint32_t raw[4];
#pragma unroll
        for (int i = 0; i < 4; ++i)
            raw[i] = in[i] ? (uint32_t)reinterpret_cast<const unsigned short*>(tile)[(pv[i] - vmin) * rowe + (pu[i] - u0)]
                           : 0u;
        const f2 B = f2_mul(S, f2_splat(-8388608.0f));
#pragma unroll
        for (int h = 0; h < 4; h += 2) {
            const f2 r = f2_fma(f2_pack(__uint_as_float(raw[h] | 0x4B000000u), __uint_as_float(raw[h + 1] | 0x4B000000u)),
                                S, B);
            dv[h] = f2_lo(r);
            dv[h + 1] = f2_hi(r);
        }
    } else if (fs.fmt == kSlotU16Mul) {
        const float scale = f2_lo(S);
#pragma unroll
        for (int i = 0; i < 4; ++i)
            dv[i] = in[i] ? u16_metres(reinterpret_cast<const unsigned short*>(tile)[(pv[i] - vmin) * rowe + (pu[i] - u0)],
                                       scale)
                          : 0.f;
    } else {
#pragma unroll
        for (int i = 0; i < 4; ++i)
            dv[i] = in[i] ? reinterpret_cast<const float*>(tile)[(pv[i] - vmin) * rowe + (pu[i] - u0)] : 0.f;
    }
}

// The thread's place in a brick and its warp's sub-box.
template <int TX, int BY, int BZ>
struct BrickLayout {
    int tx, ty, tz, lane, wy_lo, wy_hi, wz_lo, wz_hi;
    __device__ __forceinline__ BrickLayout(int tid) {
        tx = tid % TX;
        ty = (tid / TX) % BY;
        tz = tid / (TX * BY);
        lane = tid & 31;
        const int wfirst = tid & ~31;
        wy_lo = (TX * BY >= 32) ? (wfirst / TX) % BY : 0;
        wy_hi = (TX * BY >= 32) ? wy_lo + 32 / TX - 1 : BY - 1;
        wz_lo = wfirst / (TX * BY);
        wz_hi = (wfirst + 31) / (TX * BY);
    }
};

// Lane f of the warp tests frame f0 + f against the warp's sub-box; returns
// the mask of frames that may update a voxel of it.
template <int MODE, int TX, int BY, int BZ>
__device__ __forceinline__ uint32_t warp_live_frames(const VolDesc& v, const FrameSlot* slots, int f0, int nf,
                                                     const BrickLayout<TX, BY, BZ>& L, int bx0, int by0, int bz0) {
    bool live = false;
    const int f = f0 + L.lane;
    if (f < nf) {
        const int xl = bx0, xh = min(bx0 + 4 * TX, v.nx) - 1;
        const int yl = by0 + L.wy_lo, yh = min(by0 + L.wy_hi, v.ny - 1);
        const int zl = bz0 + L.wz_lo, zh = min(bz0 + L.wz_hi, v.nz - 1);
        live = (yl <= yh && zl <= zh) && !box_culled<MODE>(v, slots[f], xl, xh, yl, yh, zl, zh);
    }
    return __ballot_sync(0xffffffffu, live);
}

// The frames (bit f) for which the warp's sub-box of the brick at (bx0, by0,
// bz0) may contain an updated voxel, evaluated by one lane for all nf frames.
template <int MODE, int TX, int BY, int BZ>
__device__ __forceinline__ uint32_t brick_live_frames(const VolDesc& v, const FrameSlot* slots, int nf,
                                                      const BrickLayout<TX, BY, BZ>& L, int bx0, int by0, int bz0) {
    const int xl = bx0, xh = min(bx0 + 4 * TX, v.nx) - 1;
    const int yl = by0 + L.wy_lo, yh = min(by0 + L.wy_hi, v.ny - 1);
    const int zl = bz0 + L.wz_lo, zh = min(bz0 + L.wz_hi, v.nz - 1);
    uint32_t m = 0u;
    if (yl <= yh && zl <= zh)
        for (int f = 0; f < nf; ++f)
            if (!box_culled<MODE>(v, slots[f], xl, xh, yl, yh, zl, zh)) m |= 1u << f;
    return m;
}

// One frame's samples for the thread's (up to) 4 voxels: the depth under
// each voxel, 0 where the voxel projects off the image (or, in the fixed
// mode, lies at or in front of min_z) -- values the update skips -- and, in
// the fixed mode, the voxel's camera z.  Split from the update so that the
// next frame's depth gathers are in flight while this frame's running
// averages are computed.  FULL: the thread has all 4 voxels (nvalid == 4).
template <int MODE, bool FULL, bool STAGE = false>
__device__ __forceinline__ void frame_samples(const VolDesc& v, const FrameSlot& fs, const float* px, float py, float pz,
                                              int nvalid_, float (&dv)[4], float (&zc)[4],
                                              unsigned char* tile = nullptr) {
    const int nvalid = FULL ? 4 : nvalid_;
    // pixel (u, v) is element v * pitch_elems + u of the image (the host checks
    // that height * pitch_elems fits 32 bits and that the pitch is a whole
    // number of elements)
    const float* pr = fs.pose;
    const uint32_t pitch_elems = fs.pitch_elems;
    const uint32_t width = fs.width, height = fs.height;
    if (MODE == kCompat) {
        const float r0 = pr[0], r1 = pr[1], r2 = pr[2], r3 = pr[3], r4 = pr[4], r5 = pr[5];
        const float r6 = pr[6], r7 = pr[7], r8 = pr[8], t0 = pr[9], t1 = pr[10], t2 = pr[11];
        // world_to_pixel + camera_to_pixel (camera_util.cu:7-19,44-51) for the
        // thread's 4 voxels, two at a time in paired FP32
        const float m0 = __fmul_rn(r1, py), m1 = __fmul_rn(r4, py), m2 = __fmul_rn(r7, py);
        int pu[4], pv[4];
        f2 cz2[2];
#pragma unroll
        for (int h = 0; h < 4; h += 2) {
            const f2 X = f2_pack(px[h], px[h + 1]);
            const f2 cxv = compat_cam2(r0, r2, t0, X, m0, pz);
            const f2 cyv = compat_cam2(r3, r5, t1, X, m1, pz);
            const f2 czv = compat_cam2(r6, r8, t2, X, m2, pz);
            f2 qu, qv;
            compat_proj2(cxv, cyv, czv, v.fx, v.fy, v.cx, v.cy, qu, qv);
            pu[h] = (int)f2_lo(qu);
            pv[h] = (int)f2_lo(qv);
            pu[h + 1] = (int)f2_hi(qu);
            pv[h + 1] = (int)f2_hi(qv);
            cz2[h >> 1] = czv;
        }
        // A voxel with world z == 0 or camera z == 0 maps to pixel (0, 0).
        // World z is the thread's own (one comparison, out of the frame
        // loop); one product tests the 4 camera z values: it is 0 or NaN
        // whenever a factor is 0 (0 * finite = 0, 0 * inf = 0 * NaN = NaN),
        // and a product that is 0 or NaN for any other reason (underflow, a
        // NaN factor) only sends the thread through the per-voxel test.
        const f2 zz = f2_mul(cz2[0], cz2[1]);
        if (pz == 0.f || !(fabsf(__fmul_rn(f2_lo(zz), f2_hi(zz))) > 0.f)) {
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                const float cz = (i & 1) ? f2_hi(cz2[i >> 1]) : f2_lo(cz2[i >> 1]);
                if (pz == 0.f || cz == 0.f) {
                    pu[i] = 0;
                    pv[i] = 0;
                }
            }
        }
        // tsdf_volume.cu:166-170 (negative u, v wrap to large unsigned values)
        bool in[4];
        uint32_t pix[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            in[i] = i < nvalid && (uint32_t)pu[i] < width && (uint32_t)pv[i] < height;
            pix[i] = (uint32_t)pv[i] * pitch_elems + (uint32_t)pu[i];
        }
        if (STAGE)
            gather_staged(fs, in, pu, pv, pix, dv, tile);
        else
            gather_depth(fs, in, pix, dv);
    } else {
#if !defined(GBT_REF_ARITH)
        // K [R | t] applied to voxel pairs in paired FP32 (the same rounding
        // per lane as the scalar fused multiply-adds); u, v rounded to the
        // nearest pixel from U * (1/Z) with the reciprocal correctly rounded
        const f2 aU = f2_splat(__fmaf_rn(pr[1], py, __fmaf_rn(pr[2], pz, pr[3])));
        const f2 aV = f2_splat(__fmaf_rn(pr[5], py, __fmaf_rn(pr[6], pz, pr[7])));
        const f2 aZ = f2_splat(__fmaf_rn(pr[9], py, __fmaf_rn(pr[10], pz, pr[11])));
        const f2 p0 = f2_splat(pr[0]), p4 = f2_splat(pr[4]), p8 = f2_splat(pr[8]);
        bool in[4];
        uint32_t pix[4];
        int pu[4], pv[4];
#pragma unroll
        for (int h = 0; h < 4; h += 2) {
            const f2 X = f2_pack(px[h], px[h + 1]);
            const f2 Z = f2_fma(p8, X, aZ);
            const f2 U = f2_fma(p0, X, aU);
            const f2 V = f2_fma(p4, X, aV);
            const f2 rz = f2_pack(__frcp_rn(f2_lo(Z)), __frcp_rn(f2_hi(Z)));
            const f2 uq = f2_mul(U, rz), vq = f2_mul(V, rz);
#pragma unroll
            for (int j = 0; j < 2; ++j) {
                const int i = h + j;
                const float z = j ? f2_hi(Z) : f2_lo(Z);
                const int u = __float2int_rn(j ? f2_hi(uq) : f2_lo(uq));
                const int vv = __float2int_rn(j ? f2_hi(vq) : f2_lo(vq));
                zc[i] = z;
                in[i] = i < nvalid && z > v.min_z && (uint32_t)u < width && (uint32_t)vv < height;
                pix[i] = (uint32_t)vv * pitch_elems + (uint32_t)u;
                pu[i] = u;
                pv[i] = vv;
            }
        }
        if (STAGE)
            gather_staged(fs, in, pu, pv, pix, dv, tile);
        else
            gather_depth(fs, in, pix, dv);
#endif
    }
}

// One frame's running-average update of the thread's voxels from its
// samples; returns whether any voxel changed.
template <int MODE, bool FULL>
__device__ __forceinline__ bool frame_update(const VolDesc& v, const float (&dv)[4], const float (&zc)[4], float pz,
                                             int nvalid_, float* d, float* w, const float* s_inv) {
    const int nvalid = FULL ? 4 : nvalid_;
    bool dirty = false;
#if defined(GBT_REF_ARITH)
    if (MODE == kCompat && FULL) {
        // The same update on voxel pairs in paired FP32: the distance to the
        // surface, the new weight, the weighted sum d*w + tsdf (contracted to
        // one multiply-add, as the fast-math build contracts it) and its
        // product with the approximate reciprocal of the new weight (the
        // fast-math division), each lane rounded and flushed as the scalar
        // instruction would.
        const f2 NPZ = f2_splat(-pz);
        const f2 ONE = f2_splat(1.0f);
#pragma unroll
        for (int h = 0; h < 4; h += 2) {
            const f2 S = f2_add(f2_pack(dv[h], dv[h + 1]), NPZ);
            bool ok[2];
            float tsdf[2];
#pragma unroll
            for (int j = 0; j < 2; ++j) {
                const float sdf = j ? f2_hi(S) : f2_lo(S);
                // tsdf_volume.cu:169-176 (24 is exact in float)
                ok[j] = dv[h + j] > 0.0f && dv[h + j] <= 24.0f && sdf >= -v.trunc;
                tsdf[j] = fminf(sdf, v.trunc);
            }
            const f2 Wp = f2_pack(w[h], w[h + 1]);
            const f2 NW = f2_add(Wp, ONE);
            const f2 NUM = f2_fma(f2_pack(d[h], d[h + 1]), Wp, f2_pack(tsdf[0], tsdf[1]));
            float r0, r1;
            asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r0) : "f"(f2_lo(NW)));
            asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r1) : "f"(f2_hi(NW)));
            const f2 ND = f2_mul(NUM, f2_pack(r0, r1));
            if (ok[0]) {
                w[h] = f2_lo(NW);
                d[h] = f2_lo(ND);
            }
            if (ok[1]) {
                w[h + 1] = f2_hi(NW);
                d[h + 1] = f2_hi(ND);
            }
            dirty |= ok[0] || ok[1];
        }
        return dirty;
    }
#endif
    if (MODE == kCompat) {
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            if (i >= nvalid) break;
            // tsdf_volume.cu:171-187; 24 is exact in float, so this is the
            // reference's double comparison
            if (dv[i] <= 0.0f || dv[i] > 24.0f) continue;
            const float sdf = dv[i] - pz;
            if (sdf >= -v.trunc) {
                // the reference clamps positive values only (sdf > 0 ?
                // min(sdf, trunc) : sdf); with trunc > 0 (the host checks it)
                // and sdf not NaN here, min(sdf, trunc) is the same value
                const float tsdf = fminf(sdf, v.trunc);
                const float nw = w[i] + 1.0f;
                const float nd = compat_avg(d[i], w[i], tsdf, nw);
                w[i] = nw;
                d[i] = nd;
                dirty = true;
            }
        }
    } else {
#if !defined(GBT_REF_ARITH)
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            if (i >= nvalid) break;
            if (!(dv[i] > 0.f && dv[i] <= v.max_depth)) continue;
            const float sdf = __fsub_rn(dv[i], zc[i]);
            if (!(sdf >= -v.trunc)) continue;
            const float tsdf = fminf(sdf, v.trunc);
            const int n = max(__float2int_rz(w[i]), 0) + 1;
            const float inv = n < 256 ? s_inv[n] : __frcp_rn((float)n);
            d[i] = __fmaf_rn(__fsub_rn(tsdf, d[i]), inv, d[i]);
            w[i] = fminf(__fadd_rn(w[i], 1.0f), v.max_weight);
            dirty = true;
        }
#endif
    }
    return dirty;
}

// Applies the frames of `mask` (bit f: slots[f]) in order to the thread's
// voxels, the next frame's samples gathered before the current frame's
// update; returns whether any voxel changed.  The loop body covers two
// frames, the two sample sets taking turns as the one gathered and the one
// applied, so that no copy from one to the other is issued.
template <int MODE, bool FULL>
__device__ __forceinline__ bool apply_frames(const VolDesc& v, const FrameSlot* slots, uint32_t mask, const float* px,
                                             float py, float pz, int nvalid, float* d, float* w, const float* s_inv) {
    if (!mask) return false;
    bool dirty = false;
    float dva[4], zca[4], dvb[4], zcb[4];
    frame_samples<MODE, FULL>(v, slots[__ffs(mask) - 1], px, py, pz, nvalid, dva, zca);
    mask &= mask - 1;
    for (;;) {
        bool more = mask != 0u;
        if (more) {
            frame_samples<MODE, FULL>(v, slots[__ffs(mask) - 1], px, py, pz, nvalid, dvb, zcb);
            mask &= mask - 1;
        }
        dirty |= frame_update<MODE, FULL>(v, dva, zca, pz, nvalid, d, w, s_inv);
        if (!more) break;
        more = mask != 0u;
        if (more) {
            frame_samples<MODE, FULL>(v, slots[__ffs(mask) - 1], px, py, pz, nvalid, dva, zca);
            mask &= mask - 1;
        }
        dirty |= frame_update<MODE, FULL>(v, dvb, zcb, pz, nvalid, d, w, s_inv);
        if (!more) break;
    }
    return dirty;
}

// The thread's voxels of a brick: load, centres, store.
struct ThreadVoxels {
    size_t base;
    int x0, y, z, nvalid;
    bool full;
    float d[4], w[4], px[4], py, pz;

    __device__ __forceinline__ bool init(const VolDesc& v, int x0_, int y_, int z_) {
        x0 = x0_;
        y = y_;
        z = z_;
        if (y >= v.ny || z >= v.nz || x0 >= v.nx) return false;
        base = ((size_t)z * v.ny + y) * v.nx + x0;
        full = ((v.nx & 3) == 0) && (x0 + 3 < v.nx);
        nvalid = min(4, v.nx - x0);
        return true;
    }
    __device__ __forceinline__ void load(const VolDesc& v) {
        if (full) {
            const float4 d4 = *reinterpret_cast<const float4*>(v.D + base);
            const float4 w4 = *reinterpret_cast<const float4*>(v.W + base);
            d[0] = d4.x; d[1] = d4.y; d[2] = d4.z; d[3] = d4.w;
            w[0] = w4.x; w[1] = w4.y; w[2] = w4.z; w[3] = w4.w;
        } else {
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                d[i] = (i < nvalid) ? v.D[base + i] : 0.f;
                w[i] = (i < nvalid) ? v.W[base + i] : 0.f;
            }
        }
        centres(v);
    }
    // the voxels' world coordinates
    __device__ __forceinline__ void centres(const VolDesc& v) {
        py = centre(y, v.vs[1], v.off[1]);
        pz = centre(z, v.vs[2], v.off[2]);
#pragma unroll
        for (int i = 0; i < 4; ++i) px[i] = centre(x0 + i, v.vs[0], v.off[0]);
    }
    __device__ __forceinline__ void store(const VolDesc& v) const {
        if (full) {
            *reinterpret_cast<float4*>(v.D + base) = make_float4(d[0], d[1], d[2], d[3]);
            *reinterpret_cast<float4*>(v.W + base) = make_float4(w[0], w[1], w[2], w[3]);
        } else {
#pragma unroll
            for (int i = 0; i < 4; ++i)
                if (i < nvalid) {
                    v.D[base + i] = d[i];
                    v.W[base + i] = w[i];
                }
        }
    }
};

__device__ __forceinline__ void fill_inv_table(float* s_inv) {
    for (int k = threadIdx.x; k < 256; k += blockDim.x) s_inv[k] = k ? __frcp_rn((float)k) : 0.f;
}

// The frames of `mask` applied one after the other (sample, then update).
template <int MODE, bool FULL, bool STAGE = false>
__device__ __forceinline__ bool frames_in_turn(const VolDesc& v, const FrameSlot* slots, uint32_t mask,
                                               ThreadVoxels& t, const float* s_inv, unsigned char* tile = nullptr) {
    bool dirty = false;
    for (; mask; mask &= mask - 1) {
        const int f = __ffs(mask) - 1;
        float dv[4], zc[4];
        frame_samples<MODE, FULL, STAGE>(v, slots[f], t.px, t.py, t.pz, t.nvalid, dv, zc, tile);
        dirty |= frame_update<MODE, FULL>(v, dv, zc, t.pz, t.nvalid, t.d, t.w, s_inv);
    }
    return dirty;
}

// Passes of up to kLaneBrickFrames frames (LANE_BRICKS) cull with one lane
// per brick; longer passes with one lane per frame.  The short-pass instance
// is latency-bound: 10 resident CTAs per SM (48 registers, a few bytes of
// spill) beat 8 at its natural 59 registers by 2-6 %.
// STAGE (lane-brick passes only): each warp stages the depth its voxels
// sample in shared memory, frame by frame (gather_staged).
template <int MODE, int TX, int BY, int BZ, bool LANE_BRICKS, bool STAGE = false>
__global__ void __launch_bounds__(128, LANE_BRICKS ? 10 : 0) integrate_kernel(const __grid_constant__ IntegrateArgs a) {
    static_assert(TX * BY * BZ == 128, "128 threads per CTA");
    static_assert(32 % TX == 0, "a warp spans whole x rows");
    static_assert(!STAGE || LANE_BRICKS, "depth staging in the lane-brick pass kernel");
    __shared__ FrameSlot s_frame[GBT_MAX_FRAMES_PER_PASS];
    __shared__ float s_inv[256];
    __shared__ __align__(16) unsigned char s_tile[STAGE ? 4 : 1][STAGE ? kDepthTileBytes : 16];
    unsigned char* const tile = s_tile[STAGE ? (threadIdx.x >> 5) : 0];

    const VolDesc& v = a.vol;
    const int tid = threadIdx.x;
    const int nf = a.nframes;
    if (tid < nf) load_slot<MODE>(a.frames[tid], s_frame[tid]);
    if (MODE == kFixed) fill_inv_table(s_inv);
    __syncthreads();

    const BrickLayout<TX, BY, BZ> L(tid);
    const int BXV = 4 * TX;
    // brick numbers are below 2^32 (the volume has fewer voxels): 32-bit
    // division by the host's invariant divisors
    const uint32_t nbx = a.div_nbx.d, nby = a.div_nby.d;

    auto origin = [&](uint32_t b, int& bx0, int& by0, int& bz0) {
        const uint32_t rest = fastdiv(b, a.div_nbx);
        const uint32_t bzi = fastdiv(rest, a.div_nby);
        bx0 = (int)(b - rest * nbx) * BXV;
        by0 = (int)(rest - bzi * nby) * BY;
        bz0 = (int)bzi * BZ;
    };
    // the warp's voxels of one brick, the frames of fmask in turn
    auto process = [&](int bx0, int by0, int bz0, uint32_t fmask) {
        ThreadVoxels t;
        if constexpr (STAGE) {
            // every lane of the warp takes part in the staging (its reductions
            // and shuffles): lanes past the volume's edge sample with no voxel
            const bool ok = t.init(v, bx0 + 4 * L.tx, by0 + L.ty, bz0 + L.tz);
            if (ok) {
                t.load(v);
            } else {
                t.nvalid = 0;
                t.py = t.pz = 0.f;
#pragma unroll
                for (int i = 0; i < 4; ++i) t.px[i] = 0.f;
            }
            if (frames_in_turn<MODE, false, true>(v, s_frame, fmask, t, s_inv, tile) && ok) t.store(v);
            return;
        }
        if (t.init(v, bx0 + 4 * L.tx, by0 + L.ty, bz0 + L.tz)) {
            t.load(v);
            // frame by frame: the pipelined apply_frames of the batched kernel
            // makes 32-frame passes 6.6 % slower here, at the same 9 CTAs/SM
            const bool dirty = t.nvalid == 4 ? frames_in_turn<MODE, true, STAGE>(v, s_frame, fmask, t, s_inv, tile)
                                             : frames_in_turn<MODE, false, STAGE>(v, s_frame, fmask, t, s_inv, tile);
            if (dirty) t.store(v);
        }
    };
    if constexpr (LANE_BRICKS) {
        // The CTA's bricks are blockIdx.x + k * gridDim.x.  A warp takes them
        // 32 at a time: lane l tests its warp's sub-box of the l-th brick
        // against every frame of the pass, and the warp then visits the
        // bricks with a live frame (warps do not wait for each other).
        const uint64_t step = (uint64_t)gridDim.x;
        for (uint64_t c0 = blockIdx.x; c0 < a.nbricks; c0 += 32 * step) {   // the same for the whole warp
            const uint64_t bl = c0 + (uint64_t)L.lane * step;
            uint32_t lane_frames = 0u;
            if (bl < a.nbricks) {
                int bx0, by0, bz0;
                origin((uint32_t)bl, bx0, by0, bz0);
                lane_frames = brick_live_frames<MODE>(v, s_frame, nf, L, bx0, by0, bz0);
            }
            for (uint32_t live = __ballot_sync(0xffffffffu, lane_frames != 0u); live; live &= live - 1) {
                const int l = __ffs(live) - 1;
                const uint32_t fmask = __shfl_sync(0xffffffffu, lane_frames, l);
                int bx0, by0, bz0;
                origin((uint32_t)(c0 + (uint64_t)l * step), bx0, by0, bz0);
                process(bx0, by0, bz0, fmask);   // (no early exit: the loop shuffles)
            }
        }
    } else {
        // brick by brick; lane f tests frame f against the warp's sub-box
        for (uint32_t b = blockIdx.x; b < a.nbricks; b += gridDim.x) {
            int bx0, by0, bz0;
            origin(b, bx0, by0, bz0);
            const uint32_t fmask = warp_live_frames<MODE>(v, s_frame, 0, nf, L, bx0, by0, bz0);
            if (fmask != 0u) process(bx0, by0, bz0, fmask);
        }
    }
}

// ---------------------------------------------------------------------------
// Passes of up to kLaneBrickFrames frames with the distances and weights
// streamed into shared memory by the Tensor Memory Accelerator (brick 8).
//
// A CTA of 128 threads takes bricks of 32 x 4 x 4 voxels (rows of 128
// bytes); it culls its bricks 128 at a time (a thread per brick, every frame
// of the pass), queues the live ones, and one thread keeps the copies of the
// next kStreamStages queued bricks in flight: two tensor copies per brick
// (its distances and its weights, 2 KB each) into a ring of shared-memory
// stages, each stage completing on its own mbarrier.  Every thread then reads
// its 4 voxels from the stage, the stage goes back to the copier, and the
// thread applies the frames and stores the voxels that changed straight from
// its registers.  The arithmetic is frames_in_turn's: the volumes are those
// of the gathering pass kernel, bit for bit.
//
// With no voxel data held in registers while in flight, the distance and
// weight loads leave the per-brick chain.  On one frame per pass at 512^3
// that is not what bounds the gathering kernel, whose direct 16-byte loads
// already overlap the projection and the depth gathers: this form takes
// 0.239 ms per frame against 0.214 (its per-brick barrier ties the CTA's
// four warps together), and a stream per warp over slabs of 32 x 4 x 1
// voxels with the next slab's depth samples gathered before the current
// slab's update took 0.356 ms (40 % more instructions in culling and copy
// management per voxel).  It stays selectable (brick 8), outside the
// autotuner's default candidates.
//
// Waits are bounded: a stage whose copy does not arrive within about a second
// sets kStatusWaitExpired in the volume's status word; the CTA then waits
// (bounded again) for its other copies in flight and returns.

constexpr int kStreamQueue = 256;              // live bricks culled and not yet applied (a ring)
constexpr long long kWaitCycles = 1ll << 31;   // about a second at the SM clock

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(unsigned long long* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
// Makes the initialised barriers visible to the copy engine.
__device__ __forceinline__ void mbar_init_fence() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
// Arrives once on `bar` and adds `bytes` to the bytes its phase waits for.
__device__ __forceinline__ void mbar_arrive_expect(unsigned long long* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
// Waits until the phase of `bar` with parity `parity` has completed; false if
// it has not after kWaitCycles SM cycles.
__device__ __forceinline__ bool mbar_wait_bounded(unsigned long long* bar, uint32_t parity) {
    const uint32_t addr = smem_u32(bar);
    long long t0 = 0;
    for (uint32_t it = 0;; ++it) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(addr), "r"(parity)
            : "memory");
        if (done) return true;
        if (it == 0)
            t0 = clock64();
        else if (clock64() - t0 > kWaitCycles)
            return false;
    }
}
// Box (x, y, z) of the tensor `map` into shared memory at `dst`, completing
// on `bar`.  x * 4 bytes is a multiple of 16 (x is a multiple of 32).
__device__ __forceinline__ void tma_load_box3(void* dst, const CUtensorMap* map, int x, int y, int z,
                                              unsigned long long* bar) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
        "[%5];" ::"r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
        : "memory");
}

template <int MODE>
__global__ void __launch_bounds__(128) integrate_stream_kernel(const __grid_constant__ IntegrateArgs a,
                                                               const __grid_constant__ VolumeMaps maps) {
    constexpr int TX = kStreamBrickX / 4, BY = kStreamBrickY, BZ = kStreamBrickZ;
    static_assert(TX * BY * BZ == 128, "a thread per 4 voxels of the brick");
    constexpr int kBrickVoxels = kStreamBrickX * BY * BZ;
    constexpr uint32_t kStageBytes = 2u * kBrickVoxels * sizeof(float);
    constexpr int S = kStreamStages;
    // stage s: the brick's distances, then its weights, each [z][y][x] as the copy lays them out
    __shared__ __align__(128) float s_dw[S][2][kBrickVoxels];
    __shared__ __align__(8) unsigned long long s_full[S];
    __shared__ FrameSlot s_frame[kLaneBrickFrames];
    __shared__ float s_inv[256];
    __shared__ uint32_t s_qbrick[kStreamQueue];
    __shared__ uint16_t s_qmask[kStreamQueue];
    __shared__ uint32_t s_wcount[4];

    const VolDesc& v = a.vol;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int nf = a.nframes;
    if (tid < nf) load_slot<MODE>(a.frames[tid], s_frame[tid]);
    if (MODE == kFixed) fill_inv_table(s_inv);
    if (tid == 0) {
        for (int st = 0; st < S; ++st) mbar_init(&s_full[st], 1);
        mbar_init_fence();
    }
    __syncthreads();

    const BrickLayout<TX, BY, BZ> L(tid);
    const uint32_t nbx = a.div_nbx.d, nby = a.div_nby.d;
    auto origin = [&](uint32_t b, int& bx0, int& by0, int& bz0) {
        const uint32_t rest = fastdiv(b, a.div_nbx);
        const uint32_t bzi = fastdiv(rest, a.div_nby);
        bx0 = (int)(b - rest * nbx) * kStreamBrickX;
        by0 = (int)(rest - bzi * nby) * BY;
        bz0 = (int)bzi * BZ;
    };
    // the CTA's bricks are blockIdx.x + k * gridDim.x, k < nk; the counters
    // below are the same in every thread
    const uint32_t nk = a.nbricks > blockIdx.x ? (a.nbricks - blockIdx.x - 1) / gridDim.x + 1 : 0u;
    uint32_t culled = 0;   // k of the next brick to cull
    uint32_t qt = 0;       // live bricks queued
    uint32_t ld = 0;       // of them, copies issued
    uint32_t cs = 0;       // of them, applied

    // culls the next 128 bricks (a thread each) and queues the live ones in order
    auto cull = [&]() {
        const uint32_t k = culled + (uint32_t)tid;
        uint32_t fm = 0u, b = 0u;
        if (k < nk) {
            b = blockIdx.x + k * gridDim.x;
            int bx0, by0, bz0;
            origin(b, bx0, by0, bz0);
            const int xh = min(bx0 + kStreamBrickX, v.nx) - 1, yh = min(by0 + BY, v.ny) - 1,
                      zh = min(bz0 + BZ, v.nz) - 1;
            for (int f = 0; f < nf; ++f)
                if (!box_culled<MODE>(v, s_frame[f], bx0, xh, by0, yh, bz0, zh)) fm |= 1u << f;
        }
        const uint32_t bal = __ballot_sync(0xffffffffu, fm != 0u);
        if (lane == 0) s_wcount[warp] = (uint32_t)__popc(bal);
        __syncthreads();
        uint32_t off = 0u, tot = 0u;
#pragma unroll
        for (int w = 0; w < 4; ++w) {
            const uint32_t c = s_wcount[w];
            off += w < warp ? c : 0u;
            tot += c;
        }
        if (fm) {
            const uint32_t q = (qt + off + (uint32_t)__popc(bal & ((1u << lane) - 1u))) % kStreamQueue;
            s_qbrick[q] = b;
            s_qmask[q] = (uint16_t)fm;
        }
        __syncthreads();   // the queue entries are visible, s_wcount may be written again
        qt += tot;
        culled += 128u;
    };
    // keeps up to S copies in flight (thread 0 issues them)
    auto issue = [&]() {
        for (; ld < qt && ld - cs < (uint32_t)S; ++ld) {
            if (tid == 0) {
                const uint32_t b = s_qbrick[ld % kStreamQueue];
                int bx0, by0, bz0;
                origin(b, bx0, by0, bz0);
                const int st = (int)(ld % S);
                if (a.hold_first_copy && blockIdx.x == 0 && ld == 0) continue;   // failure injection
                mbar_arrive_expect(&s_full[st], kStageBytes);
                tma_load_box3(s_dw[st][0], &maps.d, bx0, by0, bz0, &s_full[st]);
                tma_load_box3(s_dw[st][1], &maps.w, bx0, by0, bz0, &s_full[st]);
            }
        }
    };

    while (ld == qt && culled < nk) cull();
    issue();
    while (cs < qt) {
        const int st = (int)(cs % S);
        const uint32_t parity = (cs / S) & 1u;
        const uint32_t b = s_qbrick[cs % kStreamQueue];
        const uint32_t fmask = s_qmask[cs % kStreamQueue];
        const bool arrived = mbar_wait_bounded(&s_full[st], parity);
        float4 d4 = make_float4(0.f, 0.f, 0.f, 0.f), w4 = d4;
        if (arrived) {
            // thread (tx, ty, tz) holds voxels 4 tx .. 4 tx + 3 of row (ty, tz): float4 number tid
            d4 = reinterpret_cast<const float4*>(s_dw[st][0])[tid];
            w4 = reinterpret_cast<const float4*>(s_dw[st][1])[tid];
        }
        // every thread has read the stage: it can take the next copy
        if (__syncthreads_or(!arrived)) {
            if (tid == 0) atomicOr(a.status, kStatusWaitExpired);
            // the copies still in flight land before the CTA leaves
            for (uint32_t u = cs + 1u; u < ld; ++u) mbar_wait_bounded(&s_full[u % S], (u / S) & 1u);
            return;
        }
        ++cs;
        while (ld == qt && culled < nk) cull();
        issue();

        int bx0, by0, bz0;
        origin(b, bx0, by0, bz0);
        ThreadVoxels t;
        if (t.init(v, bx0 + 4 * L.tx, by0 + L.ty, bz0 + L.tz)) {
            t.d[0] = d4.x; t.d[1] = d4.y; t.d[2] = d4.z; t.d[3] = d4.w;
            t.w[0] = w4.x; t.w[1] = w4.y; t.w[2] = w4.z; t.w[3] = w4.w;
            t.centres(v);
            // the host launches this kernel for x extents that are multiples of 4: 4 voxels per thread
            if (frames_in_turn<MODE, true>(v, s_frame, fmask, t, s_inv)) t.store(v);
        }
    }
}

// Many volumes (scenes) in one persistent launch.  Work items are bricks,
// numbered scene after scene in the order of the scene table (the host sorts
// scenes by frames per voxel, most expensive first); CTAs take the next brick
// from an atomic ticket, so uneven scenes balance dynamically.  A brick of a
// scene receives all of that scene's frames, in order, in registers.
template <int MODE, int TX, int BY, int BZ, bool FULL>
__global__ void __launch_bounds__(128) integrate_batch_kernel(const __grid_constant__ BatchArgs a) {
    static_assert(TX * BY * BZ == 128, "128 threads per CTA");
    __shared__ FrameSlot s_frame[kBatchMaxFrames];
    __shared__ float s_inv[256];
    __shared__ long long s_task;
    __shared__ int s_scene;

    const int tid = threadIdx.x;
    if (MODE == kFixed) fill_inv_table(s_inv);
    const BrickLayout<TX, BY, BZ> L(tid);
    const int BXV = 4 * TX;
    int scene = -1;
    for (;;) {
        __syncthreads();
        if (tid == 0) {
            const long long task = (long long)atomicAdd(a.ticket, 1u);
            int sc = scene < 0 ? 0 : scene;
            if (task < a.total_bricks) {
                while (sc + 1 < a.nscenes && a.scenes[sc + 1].brick_begin <= task) ++sc;
                while (sc > 0 && a.scenes[sc].brick_begin > task) --sc;
            }
            s_task = task;
            s_scene = sc;
        }
        __syncthreads();
        const long long task = s_task;
        if (task >= a.total_bricks) return;
        const BatchScene& S = a.scenes[s_scene];
        const VolDesc& v = S.vol;
        const FrameDesc* frames = a.frames + S.first_frame + a.w0;
        const int nf = min(S.nframes - a.w0, a.wn);
        if (s_scene != scene) {
            scene = s_scene;
            for (int f = tid; f < nf; f += blockDim.x) load_slot<MODE>(frames[f], s_frame[f]);
            __syncthreads();
        }
        const uint32_t b = (uint32_t)(task - S.brick_begin);   // below 2^32 within a scene
        const uint32_t rest = fastdiv(b, S.div_nbx);
        const uint32_t bzi = fastdiv(rest, S.div_nby);
        const int bx0 = (int)(b - rest * (uint32_t)S.nbx) * BXV, by0 = (int)(rest - bzi * (uint32_t)S.nby) * BY,
                  bz0 = (int)bzi * BZ;

        uint32_t masks[kBatchMaxFrames / 32];
        bool any = false;
#pragma unroll
        for (int c = 0; c < kBatchMaxFrames / 32; ++c) {
            masks[c] = (c * 32 < nf) ? warp_live_frames<MODE>(v, s_frame, c * 32, nf, L, bx0, by0, bz0) : 0u;
            any |= masks[c] != 0u;
        }
        if (!any) continue;
        ThreadVoxels t;
        if (!t.init(v, bx0 + 4 * L.tx, by0 + L.ty, bz0 + L.tz)) continue;
        t.load(v);
        // FULL: every scene's x extent is a multiple of 4, so every thread
        // has 4 voxels (the host picks the instance)
        // (the fixed mode, which carries each voxel's camera z from the
        // samples to the update, applies its frames one after the other: the
        // pipelined form needs 72 registers there and is 13 % slower)
        bool dirty = false;
#pragma unroll
        for (int c = 0; c < kBatchMaxFrames / 32; ++c) {
            if (MODE == kFixed)
                dirty |= frames_in_turn<MODE, FULL>(v, s_frame + c * 32, masks[c], t, s_inv);
            else
                dirty |= apply_frames<MODE, FULL>(v, s_frame + c * 32, masks[c], t.px, t.py, t.pz, t.nvalid, t.d, t.w,
                                                  s_inv);
        }
        if (dirty) t.store(v);
    }
}

// ---------------------------------------------------------------------------
// Marching cubes.  Corner k of a cube at (x, y, z) is (x + kDx[k], y + kDy[k],
// layer z + kDz[k]) in the reference's numbering (marching_cubes.cu:118-127).
__device__ __forceinline__ int corner_dx(int k) { return (0x66 >> k) & 1; }
__device__ __forceinline__ int corner_dy(int k) { return (0xF0 >> k) & 1; }
__device__ __forceinline__ int corner_dz(int k) { return (0xCC >> k) & 1; }

// Linear index of corner 0 of cube (cx, cy, cz) and of the next layer.
template <int MODE>
__device__ __forceinline__ void cube_base(const McArgs& a, uint32_t cx, uint32_t cy, uint32_t cz, int64_t* b0,
                                          int64_t* b1) {
    const int64_t gx = a.gx;
    const int64_t layer = (MODE == kCompat) ? (gx + a.gy) : gx * a.gy;   // marching_cubes.cu:211
    *b0 = (int64_t)cz * layer + (int64_t)cy * gx + cx;
    *b1 = *b0 + layer;
}

template <int MODE>
__device__ __forceinline__ int64_t corner_index(const McArgs& a, int64_t b0, int64_t b1, int k) {
    return (corner_dz(k) ? b1 : b0) + corner_dx(k) + (corner_dy(k) ? a.gx : 0);
}

// Grid edge of cube (cx, cy, cz) between corners ca (the lower one) and cb:
// 3 * (linear index of ca's voxel) + the axis along which they differ.
__device__ __forceinline__ int64_t weld_edge_id(const McArgs& a, uint32_t cx, uint32_t cy, uint32_t cz, int ca, int cb) {
    const int axis = corner_dx(ca) != corner_dx(cb) ? 0 : (corner_dy(ca) != corner_dy(cb) ? 1 : 2);
    const int64_t lin = ((int64_t)(cz + corner_dz(ca)) * a.gy + (int64_t)(cy + corner_dy(ca))) * a.gx +
                        (int64_t)(cx + corner_dx(ca));
    return 3 * lin + axis;
}

// Cube classification by warps.  The 32 lanes of a warp take 32 consecutive
// cubes (linear order).  A lane loads the corners of its cube at x (corners
// 0, 3, 4 and 7: (y, z), (y, z+1), (y+1, z), (y+1, z+1)) and packs their signs
// into a nibble, with, in the fixed mode, a fifth bit for "all four weights
// > 0"; the corners at x + 1 are the next lane's corners at x, so one shuffle
// of the nibble completes the cube, except for lane 31 and for the last cube
// of a grid row, which load their x + 1 corners themselves (those loads are
// issued with the others, predicated).  A table maps the (own, next) nibble
// pair to the 8-bit type in the reference's corner numbering.
__device__ __forceinline__ int mc_type_of_nibbles(int sx, int sn) {
    return (sx & 1) | (sn & 1) << 1 | ((sn >> 1) & 1) << 2 | ((sx >> 1) & 1) << 3 | ((sx >> 2) & 1) << 4 |
           ((sn >> 2) & 1) << 5 | ((sn >> 3) & 1) << 6 | ((sx >> 3) & 1) << 7;
}

// Linear indices of corners 0, 3, 4, 7 of cube c and whether its x + 1
// corners are the next cube's x corners (not so at the end of a row).  All
// indices are below 2^32: the host limits volumes to 2^32 - 1 voxels, and the
// compat layer stride (gx + gy) stays within the grid.
template <int MODE>
__device__ __forceinline__ bool cube_xcorners(const McArgs& a, uint32_t c, uint32_t (&idx)[4]) {
    const uint32_t row = fastdiv(c, a.div_cx);
    const uint32_t cx = c - row * (uint32_t)(a.gx - 1);
    const uint32_t cz = fastdiv(row, a.div_cy);
    const uint32_t cy = row - cz * (uint32_t)(a.gy - 1);
    const uint32_t gx = (uint32_t)a.gx;
    const uint32_t layer = (MODE == kCompat) ? gx + (uint32_t)a.gy : gx * (uint32_t)a.gy;   // marching_cubes.cu:211
    const uint32_t b0 = cz * layer + cy * gx + cx, b1 = b0 + layer;
    idx[0] = b0;
    idx[1] = b1;
    idx[2] = b0 + gx;
    idx[3] = b1 + gx;
    return cx + 2 == gx;
}

// Types (0 for a cube that is not emitted: past the end, or in the fixed mode
// with a corner of weight <= 0) of NG consecutive groups of 32 cubes from
// cube `base` (a multiple of 32): lane l of group i holds cube
// base + 32 i + l.  Every x-corner load of the NG groups is issued before any
// is used.  The x + 1 corners of a cube are the next lane's x corners, or
// for lane 31 the x corners of lane 0 of the next group; the last cube of a
// grid row and lane 31 of the last group load theirs, under a branch the
// warp takes only when one of its lanes needs it.  A cube past the end reads
// the last cube, in bounds, and is discarded.
template <int MODE, int NG>
__device__ __forceinline__ void mc_warp_types(const McArgs& a, uint64_t base, int lane, int (&type)[NG],
                                              const unsigned char* s_type) {
    bool own[NG];
    float dx[NG][4], wx[NG][4];
#pragma unroll
    for (int i = 0; i < NG; ++i) {
        const uint64_t cube = base + 32 * i + lane;
        const uint32_t c = cube < a.ncubes ? (uint32_t)cube : a.ncubes - 1;
        uint32_t idx[4];
        own[i] = cube_xcorners<MODE>(a, c, idx) || (i == NG - 1 && lane == 31);
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            dx[i][k] = __ldg(a.D + idx[k]);
            if (MODE == kFixed) wx[i][k] = __ldg(a.W + idx[k]);
        }
    }
    int so[NG];
#pragma unroll
    for (int i = 0; i < NG; ++i) {
        so[i] = 0;
        if (__any_sync(0xffffffffu, own[i]) && own[i]) {
            // (the corner indices again, rather than kept live for the rare case)
            const uint64_t cube = base + 32 * i + lane;
            uint32_t idx[4];
            cube_xcorners<MODE>(a, cube < a.ncubes ? (uint32_t)cube : a.ncubes - 1, idx);
            bool ok = true;
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                so[i] |= (__ldg(a.D + idx[k] + 1) < 0.f) << k;
                if (MODE == kFixed) ok = ok && __ldg(a.W + idx[k] + 1) > 0.f;
            }
            if (MODE == kFixed) so[i] |= ok << 4;
        }
    }
    int sx[NG];
#pragma unroll
    for (int i = 0; i < NG; ++i) {
        sx[i] = 0;
#pragma unroll
        for (int k = 0; k < 4; ++k) sx[i] |= (dx[i][k] < 0.f) << k;
        if (MODE == kFixed) {
            const bool okx = wx[i][0] > 0.f && wx[i][1] > 0.f && wx[i][2] > 0.f && wx[i][3] > 0.f;
            sx[i] |= okx << 4;
        }
    }
#pragma unroll
    for (int i = 0; i < NG; ++i) {
        // every lane takes part in both shuffles
        const int nx = __shfl_down_sync(0xffffffffu, sx[i], 1);
        const int nf = __shfl_sync(0xffffffffu, sx[i + 1 < NG ? i + 1 : i], 0);
        const int sn = own[i] ? so[i] : (lane == 31 ? nf : nx);
        const int t = s_type[(sx[i] & 15) | (sn & 15) << 4];
        bool ok = base + 32 * i + lane < a.ncubes;
        if (MODE == kFixed) ok = ok && (sx[i] & sn & 16);
        type[i] = ok ? t : 0;
    }
}

// Types of the thread's cubes of a tile: warp w holds the CPT consecutive
// groups of 32 cubes from group w * CPT, classified NB groups at a time (the
// fixed mode also loads weights: half as many in flight).
template <int MODE, int CPT>
__device__ __forceinline__ void mc_tile_types(const McArgs& a, uint32_t tile, int tid, int (&type)[CPT],
                                              const unsigned char* s_type) {
    constexpr int NB = MODE == kFixed ? 2 : 4;
    const uint64_t base = (uint64_t)tile * (kMcThreads * CPT) + (uint64_t)(tid >> 5) * (32 * CPT);
#pragma unroll
    for (int i0 = 0; i0 < CPT; i0 += NB) {
        int t[NB];
        mc_warp_types<MODE, NB>(a, base + 32 * i0, tid & 31, t, s_type);
#pragma unroll
        for (int i = 0; i < NB; ++i) type[i0 + i] = t[i];
    }
}

__device__ __forceinline__ void mc_load_tables(unsigned char* s_count, unsigned long long* s_tri, unsigned char* s_ends,
                                               unsigned char* s_type) {
    for (int k = threadIdx.x; k < 256; k += blockDim.x) {
        if (s_count) s_count[k] = GBT_MC_TRI_COUNT[k];
        if (s_tri) s_tri[k] = GBT_MC_TRI_PACKED[k];
        s_type[k] = (unsigned char)mc_type_of_nibbles(k & 15, k >> 4);
    }
    if (s_ends && threadIdx.x < 12) s_ends[threadIdx.x] = GBT_MC_EDGE_ENDS[threadIdx.x];
}

// Marching cubes in four launches, none of which waits on another CTA.
// (1) mc_count_kernel: a warp takes a segment of kMcSegCubes cubes along x in
//     one cube layer and walks kMcRowsPerTask rows along y.  Lane l holds
//     voxel column x0 + l; per row it loads its voxels at (y+1, z) and
//     (y+1, z+1) -- two distance loads per cube (four in the fixed mode) --
//     and the previous row's two sign bits complete the nibble of its cube's
//     x corners; the x + 1 nibble is the next lane's.  Each row's triangle
//     counts go to the words of the tiles (mc_tile_cubes(MODE) cubes in
//     linear cube order, words starting at 0) its cubes fall in.
// (2) mc_reduce_kernel: one CTA per superblock of 1024 tiles sums its tile
//     counts (triangles, tiles with triangles); mc_scan_kernel: one CTA per
//     superblock turns the tile counts into exclusive offsets in place and
//     lists the tiles that have triangles, from those superblock totals; the
//     last writes the total.
// (3) mc_emit_kernel: CTAs take listed tiles by ticket, classify the tile
//     again, scan its counts and write its triangles from the tile's offset.
// Triangles come out in the reference's linear cube order.
// Adds n > 0 triangles to tile t's word.  (The superblock totals are summed
// from the words afterwards, by mc_reduce_kernel: atomics on them from the
// rows of every warp contend for a few addresses.)
__device__ __forceinline__ void mc_add_tile(const McArgs& a, uint64_t t, unsigned n) {
    atomicAdd(a.status + t, (unsigned long long)n);
}

constexpr uint32_t kMcSegCubes = 31;      // cubes per segment: 32 voxel columns
constexpr uint32_t kMcRowsPerTask = 64;   // rows a warp walks per task
constexpr uint32_t kMcRowBatch = 8;       // rows whose loads are in flight together
constexpr int kMcTileShift[2] = {11, 10};  // log2 of mc_tile_cubes(mode)

template <int MODE>
__global__ void __launch_bounds__(kMcThreads) mc_count_kernel(const __grid_constant__ McArgs a) {
    // triangles of the cube whose x-corner nibble is q & 15 and x + 1 nibble q >> 4
    __shared__ unsigned char s_cnt[256];
    for (int k = threadIdx.x; k < 256; k += blockDim.x) s_cnt[k] = GBT_MC_TRI_COUNT[mc_type_of_nibbles(k & 15, k >> 4)];
    __syncthreads();
    static_assert((1 << kMcTileShift[MODE]) == mc_tile_cubes(MODE), "tiles of a power of two cubes");
    static_assert(mc_tile_cubes(MODE) >= 2 * 32, "a row segment straddles at most one tile boundary");
    constexpr int kShift = kMcTileShift[MODE];
    const int lane = threadIdx.x & 31;
    const uint32_t gx = (uint32_t)a.gx, gy = (uint32_t)a.gy;
    const uint32_t cx_n = gx - 1, cy_n = gy - 1, cz_n = (uint32_t)a.gz - 1;
    const uint32_t nseg = (cx_n + kMcSegCubes - 1) / kMcSegCubes;
    const uint32_t nchunk = (cy_n + kMcRowsPerTask - 1) / kMcRowsPerTask;
    const uint64_t ntasks = (uint64_t)cz_n * nchunk * nseg;
    const uint32_t layer = (MODE == kCompat) ? gx + gy : gx * gy;   // marching_cubes.cu:211
    const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    // the loop bound is the same for all lanes of a warp
    for (uint64_t task = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; task < ntasks; task += nwarps) {
        const uint32_t seg = (uint32_t)(task % nseg);
        const uint64_t rest = task / nseg;
        const uint32_t chunk = (uint32_t)(rest % nchunk);
        const uint32_t cz = (uint32_t)(rest / nchunk);
        const uint32_t x0 = seg * kMcSegCubes;
        const uint32_t x = x0 + (uint32_t)lane;                            // this lane's voxel column
        const bool cube_ok = lane < (int)kMcSegCubes && x < cx_n;          // ... and its cube
        const uint32_t xl = x < gx ? x : gx - 1;                           // loads stay in the grid
        const uint32_t y0 = chunk * kMcRowsPerTask;
        const uint32_t y1 = min(y0 + kMcRowsPerTask, cy_n);
        const uint32_t i0 = cz * layer + y0 * gx + xl;                     // voxel (x, y0, z); +layer: z+1
        const float* d0p = a.D + i0;
        const float* d1p = d0p + layer;
        const float* w0p = a.W + i0;
        const float* w1p = w0p + layer;
        int lo = (__ldg(d0p) < 0.f) | (__ldg(d1p) < 0.f) << 1;            // row y: corners 0, 3
        bool lo_ok = true;
        if (MODE == kFixed) lo_ok = __ldg(w0p) > 0.f && __ldg(w1p) > 0.f;
        // linear cube index (below 2^32: the grid has fewer voxels); the
        // warp's cubes of a row lie in tile `cur` or cur + 1, cur being lane 0's
        uint32_t c = (cz * cy_n + y0) * cx_n + x;
        uint32_t c_lane0 = c - (uint32_t)lane;
        uint32_t cur = c_lane0 >> kShift;
        unsigned acc0 = 0, acc1 = 0;   // this lane's triangles in tiles cur and cur + 1
        auto flush = [&]() {
            const unsigned n0 = __reduce_add_sync(0xffffffffu, acc0);
            const unsigned n1 = __reduce_add_sync(0xffffffffu, acc1);
            if (lane == 0) {
                if (n0) mc_add_tile(a, cur, n0);
                if (n1) mc_add_tile(a, cur + 1, n1);
            }
            acc0 = 0;
            acc1 = 0;
        };
        auto row = [&](float d0, float d1, float w0, float w1) {
            if ((c_lane0 >> kShift) != cur) {   // the same for the whole warp
                flush();
                cur = c_lane0 >> kShift;
            }
            const int hi = (d0 < 0.f) | (d1 < 0.f) << 1;   // row y+1: corners 4, 7
            bool hi_ok = true;
            if (MODE == kFixed) hi_ok = w0 > 0.f && w1 > 0.f;
            int sx = lo | hi << 2;
            if (MODE == kFixed) sx |= (lo_ok && hi_ok) << 4;
            const int sn = __shfl_down_sync(0xffffffffu, sx, 1);
            unsigned n = s_cnt[(sx & 15) | (sn & 15) << 4];
            if (!cube_ok || (MODE == kFixed && !(sx & sn & 16))) n = 0u;
            if ((c >> kShift) == cur) acc0 += n; else acc1 += n;
            // the cube's group of 32 (linear order) has triangles: the emit
            // kernel classifies only such groups
            if (n) atomicOr(a.group_bits + (c >> 10), 1u << ((c >> 5) & 31u));
            lo = hi;
            lo_ok = hi_ok;
            c += cx_n;
            c_lane0 += cx_n;
        };
        // full batches of kMcRowBatch rows: every load of a batch is issued
        // before any is used (the tile-word atomics would otherwise keep the
        // compiler from moving the next row's loads ahead)
        uint32_t y = y0;
        for (; y + kMcRowBatch <= y1; y += kMcRowBatch) {
            float d0[kMcRowBatch], d1[kMcRowBatch], w0[kMcRowBatch], w1[kMcRowBatch];
#pragma unroll
            for (uint32_t j = 0; j < kMcRowBatch; ++j) {
                const size_t off = (size_t)(j + 1) * gx;
                d0[j] = __ldg(d0p + off);
                d1[j] = __ldg(d1p + off);
                if (MODE == kFixed) {
                    w0[j] = __ldg(w0p + off);
                    w1[j] = __ldg(w1p + off);
                }
            }
#pragma unroll
            for (uint32_t j = 0; j < kMcRowBatch; ++j) row(d0[j], d1[j], MODE == kFixed ? w0[j] : 0.f, MODE == kFixed ? w1[j] : 0.f);
            d0p += (size_t)kMcRowBatch * gx;
            d1p += (size_t)kMcRowBatch * gx;
            w0p += (size_t)kMcRowBatch * gx;
            w1p += (size_t)kMcRowBatch * gx;
        }
        for (; y < y1; ++y) {   // the rows after the last full batch
            d0p += gx;
            d1p += gx;
            w0p += gx;
            w1p += gx;
            row(__ldg(d0p), __ldg(d1p), MODE == kFixed ? __ldg(w0p) : 0.f, MODE == kFixed ? __ldg(w1p) : 0.f);
        }
        flush();
    }
}

// Row-walking count with four voxel columns per lane, for grids whose rows
// and layers start on 16-byte boundaries (x extent and layer stride
// multiples of 4).  A warp takes a segment of 128 voxel columns (128 cubes:
// lane l holds columns x0 + 4l .. x0 + 4l + 3 and their cubes; the x + 1
// column of its last cube is lane l + 1's first, or for lane 31 the first
// column of the next segment, which it loads alone) and walks
// kMcRows4PerTask rows along y.  Per row a lane loads two 16-byte vectors of
// distances (layers z and z + 1; two more of weights in the fixed mode) and
// packs their signs into four nibbles; the nibble of a cube's x corners is
// the previous row's two bits and this row's two, and (x, x + 1) nibble
// pairs index the triangle-count table.  Rows where no lane's cubes change
// sign skip the table.
constexpr uint32_t kMcSeg4Cubes = 128;
constexpr uint32_t kMcRows4PerTask = 32;

template <int MODE>
__device__ __forceinline__ uint32_t mc_sign_bits4(const float4& p, const float4& q) {
    // bit 4j: column j below zero in layer z; bit 4j + 1: in layer z + 1
    return (uint32_t)(p.x < 0.f) | (uint32_t)(q.x < 0.f) << 1 | (uint32_t)(p.y < 0.f) << 4 |
           (uint32_t)(q.y < 0.f) << 5 | (uint32_t)(p.z < 0.f) << 8 | (uint32_t)(q.z < 0.f) << 9 |
           (uint32_t)(p.w < 0.f) << 12 | (uint32_t)(q.w < 0.f) << 13;
}
__device__ __forceinline__ uint32_t mc_weight_bits4(const float4& p, const float4& q) {
    // bit j: column j observed (weight > 0) in both layers
    return (uint32_t)(p.x > 0.f && q.x > 0.f) | (uint32_t)(p.y > 0.f && q.y > 0.f) << 1 |
           (uint32_t)(p.z > 0.f && q.z > 0.f) << 2 | (uint32_t)(p.w > 0.f && q.w > 0.f) << 3;
}

template <int MODE>
__global__ void __launch_bounds__(kMcThreads) mc_count4_kernel(const __grid_constant__ McArgs a) {
    __shared__ unsigned char s_cnt[256];
    for (int k = threadIdx.x; k < 256; k += blockDim.x) s_cnt[k] = GBT_MC_TRI_COUNT[mc_type_of_nibbles(k & 15, k >> 4)];
    __syncthreads();
    constexpr int kShift = kMcTileShift[MODE];
    static_assert(mc_tile_cubes(MODE) >= 2 * kMcSeg4Cubes, "a row segment straddles at most one tile boundary");
    constexpr uint32_t kBatch = MODE == kFixed ? 2 : 4;   // rows whose loads are in flight together
    const int lane = threadIdx.x & 31;
    const uint32_t gx = (uint32_t)a.gx, gy = (uint32_t)a.gy;
    const uint32_t cx_n = gx - 1, cy_n = gy - 1, cz_n = (uint32_t)a.gz - 1;
    const uint32_t nseg = (cx_n + kMcSeg4Cubes - 1) / kMcSeg4Cubes;
    const uint32_t nchunk = (cy_n + kMcRows4PerTask - 1) / kMcRows4PerTask;
    const uint64_t ntasks = (uint64_t)cz_n * nchunk * nseg;
    const uint32_t layer = (MODE == kCompat) ? gx + gy : gx * gy;   // marching_cubes.cu:211
    const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    for (uint64_t task = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; task < ntasks; task += nwarps) {
        const uint32_t seg = (uint32_t)(task % nseg);
        const uint64_t rest = task / nseg;
        const uint32_t chunk = (uint32_t)(rest % nchunk);
        const uint32_t cz = (uint32_t)(rest / nchunk);
        const uint32_t x0 = seg * kMcSeg4Cubes;
        const uint32_t xb = x0 + 4u * (uint32_t)lane;            // this lane's first column
        const uint32_t xl = xb < gx ? xb : gx - 4;                // (loads stay in the grid)
        const uint32_t xe = x0 + kMcSeg4Cubes;                     // lane 31's extra column
        const bool extra = lane == 31 && xe < gx;
        // the lane's cubes inside the grid: bit j for cube xb + j
        const uint32_t cm = xb >= cx_n ? 0u : (cx_n - xb >= 4 ? 15u : (1u << (cx_n - xb)) - 1u);
        const uint32_t y0 = chunk * kMcRows4PerTask;
        const uint32_t y1 = min(y0 + kMcRows4PerTask, cy_n);
        const uint32_t r0 = cz * layer + y0 * gx;                  // voxel (0, y0, z); + layer: z + 1
        const float4* dp = reinterpret_cast<const float4*>(a.D + r0 + xl);
        const float4* dq = reinterpret_cast<const float4*>(a.D + r0 + layer + xl);
        const float4* wp = reinterpret_cast<const float4*>(a.W + r0 + xl);
        const float4* wq = reinterpret_cast<const float4*>(a.W + r0 + layer + xl);
        const float* ep = a.D + r0 + (extra ? xe : 0u);
        const float* eq = ep + layer;
        const float* vp = a.W + r0 + (extra ? xe : 0u);
        const float* vq = vp + layer;
        const uint32_t row4 = gx >> 2;   // a grid row in 16-byte vectors
        // row y0: the lower nibble halves
        uint32_t lo = mc_sign_bits4<MODE>(__ldg(dp), __ldg(dq));
        uint32_t lo_e = extra ? ((uint32_t)(__ldg(ep) < 0.f) | (uint32_t)(__ldg(eq) < 0.f) << 1) : 0u;
        uint32_t vlo = 15u, vlo_e = 1u;
        if (MODE == kFixed) {
            vlo = mc_weight_bits4(__ldg(wp), __ldg(wq));
            vlo_e = extra ? (uint32_t)(__ldg(vp) > 0.f && __ldg(vq) > 0.f) : 0u;
        }
        uint32_t c_row = (cz * cy_n + y0) * cx_n;    // linear index of cube (0, y, z)
        uint32_t cur = (c_row + x0) >> kShift;       // tile of the warp's first cube
        unsigned acc0 = 0, acc1 = 0;                 // this lane's triangles in tiles cur and cur + 1
        auto flush = [&]() {
            const unsigned n0 = __reduce_add_sync(0xffffffffu, acc0);
            const unsigned n1 = __reduce_add_sync(0xffffffffu, acc1);
            if (lane == 0) {
                if (n0) mc_add_tile(a, cur, n0);
                if (n1) mc_add_tile(a, cur + 1, n1);
            }
            acc0 = 0;
            acc1 = 0;
        };
        auto row = [&](float4 p, float4 q, float pe, float qe, float4 wpv, float4 wqv, float wpe, float wqe) {
            if (((c_row + x0) >> kShift) != cur) {   // the same for the whole warp
                flush();
                cur = (c_row + x0) >> kShift;
            }
            const uint32_t hi = mc_sign_bits4<MODE>(p, q);
            const uint32_t hi_e = (uint32_t)(pe < 0.f) | (uint32_t)(qe < 0.f) << 1;
            const uint32_t nib = lo | hi << 2;                 // nibble j: the x corners of cube j
            const uint32_t nib_e = lo_e | hi_e << 2;
            // every lane takes part in the shuffles
            const uint32_t nx = __shfl_down_sync(0xffffffffu, nib & 15u, 1);
            const uint32_t n20 = nib | (lane == 31 ? nib_e : nx) << 16;
            uint32_t ok = cm;
            uint32_t vhi = 15u, vhi_e = 1u;
            if (MODE == kFixed) {
                vhi = mc_weight_bits4(wpv, wqv);
                vhi_e = (uint32_t)(wpe > 0.f && wqe > 0.f);
                const uint32_t vv = vlo & vhi, vv_e = vlo_e & vhi_e;
                const uint32_t vn = __shfl_down_sync(0xffffffffu, vv & 1u, 1);
                const uint32_t v5 = vv | (lane == 31 ? vv_e : vn) << 4;
                ok &= v5 & (v5 >> 1);
            }
            const bool mixed = ok != 0u && n20 != 0u && n20 != 0xFFFFFu;
            if (__any_sync(0xffffffffu, mixed)) {
                const uint32_t c0 = c_row + xb;
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    const unsigned n = ((ok >> j) & 1u) ? s_cnt[(n20 >> (4 * j)) & 0xFFu] : 0u;
                    const uint32_t c = c0 + (uint32_t)j;
                    if ((c >> kShift) == cur) acc0 += n; else acc1 += n;
                    // the cube's group of 32 (linear order) has triangles: the
                    // emit kernel visits only such groups
                    if (n) atomicOr(a.group_bits + (c >> 10), 1u << ((c >> 5) & 31u));
                }
            }
            lo = hi;
            lo_e = hi_e;
            vlo = vhi;
            vlo_e = vhi_e;
            c_row += cx_n;
        };
        uint32_t y = y0;
        for (; y + kBatch <= y1; y += kBatch) {
            float4 p[kBatch], q[kBatch], u[kBatch], v[kBatch];
            float pe[kBatch], qe[kBatch], ue[kBatch], ve[kBatch];
#pragma unroll
            for (uint32_t j = 0; j < kBatch; ++j) {
                const size_t o = (size_t)(j + 1) * row4;
                const size_t oe = (size_t)(j + 1) * gx;
                p[j] = __ldg(dp + o);
                q[j] = __ldg(dq + o);
                pe[j] = extra ? __ldg(ep + oe) : 0.f;
                qe[j] = extra ? __ldg(eq + oe) : 0.f;
                if (MODE == kFixed) {
                    u[j] = __ldg(wp + o);
                    v[j] = __ldg(wq + o);
                    ue[j] = extra ? __ldg(vp + oe) : 0.f;
                    ve[j] = extra ? __ldg(vq + oe) : 0.f;
                }
            }
#pragma unroll
            for (uint32_t j = 0; j < kBatch; ++j) {
                if (MODE == kFixed)
                    row(p[j], q[j], pe[j], qe[j], u[j], v[j], ue[j], ve[j]);
                else
                    row(p[j], q[j], pe[j], qe[j], p[j], q[j], 0.f, 0.f);
            }
            dp += (size_t)kBatch * row4;
            dq += (size_t)kBatch * row4;
            wp += (size_t)kBatch * row4;
            wq += (size_t)kBatch * row4;
            ep += (size_t)kBatch * gx;
            eq += (size_t)kBatch * gx;
            vp += (size_t)kBatch * gx;
            vq += (size_t)kBatch * gx;
        }
        for (; y < y1; ++y) {   // the rows after the last full batch
            dp += row4;
            dq += row4;
            wp += row4;
            wq += row4;
            ep += gx;
            eq += gx;
            vp += gx;
            vq += gx;
            const float4 p = __ldg(dp), q = __ldg(dq);
            const float pe = extra ? __ldg(ep) : 0.f, qe = extra ? __ldg(eq) : 0.f;
            if (MODE == kFixed)
                row(p, q, pe, qe, __ldg(wp), __ldg(wq), extra ? __ldg(vp) : 0.f, extra ? __ldg(vq) : 0.f);
            else
                row(p, q, pe, qe, p, q, 0.f, 0.f);
        }
        flush();
    }
}

constexpr int kMcScanThreads = 1 << kMcSuperShift;   // one thread per tile of a superblock

// Superblock totals: one CTA per superblock of 1024 tiles sums its tile
// counts into super[2 sb] (triangles) and super[2 sb + 1] (tiles with
// triangles).
__global__ void __launch_bounds__(kMcScanThreads) mc_reduce_kernel(const __grid_constant__ McArgs a) {
    __shared__ unsigned long long s_part[kMcScanThreads / 32];
    const uint32_t tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const uint64_t t = (uint64_t)blockIdx.x * kMcScanThreads + tid;
    const unsigned long long c = t < a.ntiles ? a.status[t] : 0ull;
    // packed as the scan packs its sums: triangles << 24 | tiles with triangles
    unsigned long long v = (c << 24) | (c != 0ull ? 1ull : 0ull);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) s_part[warp] = v;
    __syncthreads();
    if (warp == 0) {
        unsigned long long x = lane < kMcScanThreads / 32 ? s_part[lane] : 0ull;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
        if (lane == 0) {
            a.super[2 * blockIdx.x] = x >> 24;
            a.super[2 * blockIdx.x + 1] = x & 0xffffffull;
        }
    }
}

// Exclusive offsets of the tiles (in place), the list of tiles with
// triangles, the triangle total and the list length.  One CTA per superblock
// of 1024 tiles: it sums the totals of the superblocks before it (kept by the
// count kernel), then scans its own tiles.  Sums travel packed as (triangles
// << 24 | tiles with triangles): at most 5 * 2^32 triangles and 2^22 tiles,
// so neither field carries into the other.
__global__ void __launch_bounds__(kMcScanThreads) mc_scan_kernel(const __grid_constant__ McArgs a) {
    __shared__ unsigned long long s_part[kMcScanThreads / 32];
    __shared__ unsigned long long s_prefix;
    const uint32_t tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const uint32_t sb = blockIdx.x;
    // the superblocks before this one
    unsigned long long pre = 0;
    for (uint32_t k = tid; k < sb; k += kMcScanThreads) pre += (a.super[2 * k] << 24) | a.super[2 * k + 1];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) pre += __shfl_xor_sync(0xffffffffu, pre, o);
    if (lane == 0) s_part[warp] = pre;
    __syncthreads();
    if (warp == 0) {
        unsigned long long v = s_part[lane];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0) s_prefix = v;
    }
    __syncthreads();
    const unsigned long long prefix = s_prefix;
    // this superblock's tiles, one per thread
    const uint64_t t = (uint64_t)sb * kMcScanThreads + tid;
    const unsigned long long c = t < a.ntiles ? a.status[t] : 0ull;
    const unsigned long long own = (c << 24) | (c != 0ull ? 1ull : 0ull);
    unsigned long long x = own;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned long long y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= (uint32_t)o) x += y;
    }
    __syncthreads();   // s_part is reused
    if (lane == 31) s_part[warp] = x;
    __syncthreads();
    if (warp == 0) {
        const unsigned long long v = s_part[lane];
        unsigned long long p = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned long long y = __shfl_up_sync(0xffffffffu, p, o);
            if (lane >= (uint32_t)o) p += y;
        }
        s_part[lane] = p - v;
    }
    __syncthreads();
    const unsigned long long excl = prefix + s_part[warp] + x - own;
    if (t < a.ntiles) {
        a.status[t] = excl >> 24;
        if (c) a.tile_list[excl & 0xffffffull] = (uint32_t)t;
    }
    if (sb == gridDim.x - 1 && tid == kMcScanThreads - 1) {
        const unsigned long long all = excl + own;
        *a.total = (long long)(all >> 24);
        *a.nonempty = (unsigned)(all & 0xffffffull);
    }
}

// Emission.  Each warp takes the next listed tile from a ticket (no CTA
// waits on another warp).  For each group
// of 32 consecutive cubes that the count kernel marked, in cube order, a
// warp classifies the group again (lane l: cube l; its x corners loaded, its
// x + 1 corners the next lane's, or loaded by the lane when the next cube
// starts a new row or lies in the next group), puts the cubes with
// triangles (their corner values, index and case) into a per-warp ring of
// cubes and their triangles into a per-warp queue, and writes the queue 32
// triangles at a time, one triangle per lane, the vertices staged in shared
// memory so that the warp stores consecutive triangles with coalesced
// writes.  Batches run across groups; a tile's last batch may be partial.
constexpr int kMcCubeRing = 64;    // cubes whose triangles are queued: < 32 pending + one group
constexpr int kMcTriRing = 256;    // queued triangles: < 32 pending + up to 5 per cube of a group

template <int MODE>
__device__ __forceinline__ void mc_vertex(const McArgs& a, uint32_t cx, uint32_t cy, uint32_t cz, int64_t b0, int64_t b1,
                                          float sa, float sb, int ca, int cb, float* out) {
    float pa[3], pb[3];
    if (MODE == kCompat) {
        if (sa > 0 && sb < 0) {  // marching_cubes.cu:34-41
            const int tc = ca; ca = cb; cb = tc;
            const float ts = sa; sa = sb; sb = ts;
        }
        // corner positions come from the voxel at the same linear index
        const int64_t ia = corner_index<MODE>(a, b0, b1, ca);
        const int64_t ib = corner_index<MODE>(a, b0, b1, cb);
        const uint32_t ra = fastdiv((uint32_t)ia, a.div_gx), rb = fastdiv((uint32_t)ib, a.div_gx);
        const uint32_t za = fastdiv(ra, a.div_gy), zb = fastdiv(rb, a.div_gy);
        pa[0] = centre((int)((uint32_t)ia - ra * (uint32_t)a.gx), a.vs[0], a.off[0]);
        pa[1] = centre((int)(ra - za * (uint32_t)a.gy), a.vs[1], a.off[1]);
        pa[2] = centre((int)za, a.vs[2], a.off[2]);
        pb[0] = centre((int)((uint32_t)ib - rb * (uint32_t)a.gx), a.vs[0], a.off[0]);
        pb[1] = centre((int)(rb - zb * (uint32_t)a.gy), a.vs[1], a.off[1]);
        pb[2] = centre((int)zb, a.vs[2], a.off[2]);
        const float r = mc_ratio(sa, sb);
#pragma unroll
        for (int q = 0; q < 3; ++q) out[q] = mc_lerp(pa[q], pb[q], r);
    } else {
#if !defined(GBT_REF_ARITH)
        // lower endpoint first, so the cubes sharing the edge agree
        if (corner_dx(ca) + corner_dy(ca) + corner_dz(ca) > corner_dx(cb) + corner_dy(cb) + corner_dz(cb)) {
            const int tc = ca; ca = cb; cb = tc;
            const float ts = sa; sa = sb; sb = ts;
        }
        pa[0] = centre((int)cx + corner_dx(ca), a.vs[0], a.off[0]);
        pa[1] = centre((int)cy + corner_dy(ca), a.vs[1], a.off[1]);
        pa[2] = centre((int)cz + corner_dz(ca), a.vs[2], a.off[2]);
        pb[0] = centre((int)cx + corner_dx(cb), a.vs[0], a.off[0]);
        pb[1] = centre((int)cy + corner_dy(cb), a.vs[1], a.off[1]);
        pb[2] = centre((int)cz + corner_dz(cb), a.vs[2], a.off[2]);
        const float r = __fdiv_rn(sa, __fsub_rn(sa, sb));
#pragma unroll
        for (int q = 0; q < 3; ++q) out[q] = __fmaf_rn(r, __fsub_rn(pb[q], pa[q]), pa[q]);
#endif
    }
}

// Shared-vertex index of the fixed-mode edge (ca, cb) of cube (cx, cy, cz).
__device__ __forceinline__ int32_t mc_vertex_index(const McArgs& a, uint32_t cx, uint32_t cy, uint32_t cz, int ca,
                                                   int cb) {
    if (corner_dx(ca) + corner_dy(ca) + corner_dz(ca) > corner_dx(cb) + corner_dy(cb) + corner_dz(cb)) {
        const int tc = ca; ca = cb; cb = tc;
    }
    const int64_t id = weld_edge_id(a, cx, cy, cz, ca, cb);
    const uint32_t word = a.edge_bits[id >> 5];
    const uint32_t below = word & ((1u << (id & 31)) - 1u);
    return (int32_t)(a.index_base + a.edge_word_offset[id >> 5] + __popc(below));
}

template <int MODE>
__global__ void __launch_bounds__(kMcThreads) mc_emit_kernel(const __grid_constant__ McArgs a) {
    constexpr int kWarps = kMcThreads / 32;
    __shared__ unsigned char s_count[256];
    __shared__ unsigned long long s_tri[256];
    __shared__ unsigned char s_ends[12];
    __shared__ unsigned char s_type[256];
    __shared__ float s_cval[kWarps][8][kMcCubeRing];        // corner values of the queued cubes
    __shared__ uint32_t s_cube[kWarps][kMcCubeRing];         // their linear index
    __shared__ unsigned char s_ctype[kWarps][kMcCubeRing];   // their case
    __shared__ unsigned short s_tq[kWarps][kMcTriRing];      // queued triangles: cube slot | triangle << 6
    __shared__ float s_out[kWarps][32 * 9];                  // a batch of 32 triangles
    mc_load_tables(s_count, s_tri, s_ends, s_type);
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const unsigned njobs = *a.nonempty;
    constexpr uint32_t kWords = (uint32_t)mc_tile_cubes(MODE) / 1024u;   // group words per tile
    const uint32_t nwords = (a.ncubes + 1023u) / 1024u;
    const bool indexed = MODE == kFixed && a.edge_bits != nullptr;
    float (*cval)[kMcCubeRing] = s_cval[warp];
    uint32_t* cube_of = s_cube[warp];
    unsigned char* ctype = s_ctype[warp];
    unsigned short* tq = s_tq[warp];
    float* sout = s_out[warp];

    // writes the queued triangles [head, head + cnt) (cnt <= 32) from output `first`
    auto emit_batch = [&](uint32_t head, int cnt, long long first) {
        const bool act = lane < cnt;
        if (act) {
            const unsigned e16 = tq[(head + (uint32_t)lane) & (kMcTriRing - 1)];
            const int sl = (int)(e16 & 63u), tr = (int)(e16 >> 6);
            const uint32_t cc = cube_of[sl];
            const int t = ctype[sl];
            const uint32_t row = fastdiv(cc, a.div_cx);
            const uint32_t cx = cc - row * (uint32_t)(a.gx - 1);
            const uint32_t cz = fastdiv(row, a.div_cy);
            const uint32_t cy = row - cz * (uint32_t)(a.gy - 1);
            int64_t b0, b1;
            cube_base<MODE>(a, cx, cy, cz, &b0, &b1);
            const unsigned long long edges = s_tri[t];
#pragma unroll
            for (int j = 0; j < 3; ++j) {
                const int e = (int)((edges >> (4 * (3 * tr + j))) & 15ull);
                const int ca = s_ends[e] & 15, cb = s_ends[e] >> 4;
                if (indexed) {
#if !defined(GBT_REF_ARITH)
                    const long long out = first + lane;
                    if (out < a.cap) a.tris[3 * out + j] = mc_vertex_index(a, cx, cy, cz, ca, cb);
#endif
                } else {
                    mc_vertex<MODE>(a, cx, cy, cz, b0, b1, cval[ca][sl], cval[cb][sl], ca, cb, sout + 9 * lane + 3 * j);
                }
            }
        }
        __syncwarp();
        if (!indexed) {
            // consecutive triangles first, first + 1, ...: 9 floats and 3 indices each
            const long long fit = a.cap - first;   // triangles of the batch that fit
            const int nf = 9 * (int)(fit < cnt ? (fit > 0 ? fit : 0) : cnt);
            for (int f = lane; f < nf; f += 32) a.verts[9 * first + f] = sout[f];
            for (int f = lane; f < nf / 3; f += 32) a.tris[3 * first + f] = (int32_t)(a.index_base + 3 * first + f);
        }
        __syncwarp();
    };

    for (;;) {
        unsigned job = 0;
        if (lane == 0) job = atomicAdd(a.ticket, 1u);   // the next listed tile
        job = __shfl_sync(0xffffffffu, job, 0);
        if (job >= njobs) break;
        const uint32_t tile = a.tile_list[job];
        long long out_next = (long long)a.status[tile];   // this tile's next triangle to write
        uint32_t tq_head = 0, tq_tail = 0, cq_head = 0;  // (the same in every lane)
#pragma unroll 1
        for (uint32_t w = 0; w < kWords; ++w) {
            const uint32_t word = tile * kWords + w;
            uint32_t bits = word < nwords ? a.group_bits[word] : 0u;   // the same for the whole warp
            while (bits) {
                const uint32_t g = (uint32_t)__ffs(bits) - 1u;
                bits &= bits - 1u;
                const uint64_t cube = (uint64_t)(word * 32u + g) * 32u + (uint64_t)lane;
                const bool in = cube < a.ncubes;
                const uint32_t c = in ? (uint32_t)cube : a.ncubes - 1u;
                // classification: x corners (0, 3, 4, 7) loaded, x + 1 corners (1, 2, 5, 6)
                // from the next lane or loaded
                uint32_t idx[4];
                const bool own = cube_xcorners<MODE>(a, c, idx) || lane == 31;
                float X[4], N[4], WX[4];
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    X[k] = __ldg(a.D + idx[k]);
                    if (MODE == kFixed) WX[k] = __ldg(a.W + idx[k]);
                }
#pragma unroll
                for (int k = 0; k < 4; ++k) N[k] = __shfl_down_sync(0xffffffffu, X[k], 1);
                bool okx = true, okn = true;
                if (MODE == kFixed) {
                    okx = WX[0] > 0.f && WX[1] > 0.f && WX[2] > 0.f && WX[3] > 0.f;
                    okn = __shfl_down_sync(0xffffffffu, okx ? 1 : 0, 1) != 0;
                }
                if (own) {
#pragma unroll
                    for (int k = 0; k < 4; ++k) {
                        N[k] = __ldg(a.D + idx[k] + 1);
                        if (MODE == kFixed) WX[k] = __ldg(a.W + idx[k] + 1);
                    }
                    if (MODE == kFixed) okn = WX[0] > 0.f && WX[1] > 0.f && WX[2] > 0.f && WX[3] > 0.f;
                }
                int sx = 0, sn = 0;
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    sx |= (X[k] < 0.f) << k;
                    sn |= (N[k] < 0.f) << k;
                }
                int type = s_type[sx | sn << 4];
                if (!in || (MODE == kFixed && !(okx && okn))) type = 0;
                const int n = s_count[type];
                // the cubes with triangles take consecutive ring slots, in cube order
                const uint32_t act = __ballot_sync(0xffffffffu, n > 0);
                const uint32_t rank = (uint32_t)__popc(act & ((1u << lane) - 1u));
                int incl = n;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const int y = __shfl_up_sync(0xffffffffu, incl, o);
                    if (lane >= o) incl += y;
                }
                const int total = __shfl_sync(0xffffffffu, incl, 31);
                if (n > 0) {
                    const int sl = (int)((cq_head + rank) & (kMcCubeRing - 1));
                    // the cube's eight corners in the reference's numbering
                    cval[0][sl] = X[0];
                    cval[1][sl] = N[0];
                    cval[2][sl] = N[1];
                    cval[3][sl] = X[1];
                    cval[4][sl] = X[2];
                    cval[5][sl] = N[2];
                    cval[6][sl] = N[3];
                    cval[7][sl] = X[3];
                    cube_of[sl] = c;
                    ctype[sl] = (unsigned char)type;
                    for (int k = 0; k < n; ++k)
                        tq[(tq_tail + (uint32_t)(incl - n + k)) & (kMcTriRing - 1)] = (unsigned short)(sl | k << 6);
                }
                cq_head += (uint32_t)__popc(act);
                tq_tail += (uint32_t)total;
                __syncwarp();
                while (tq_tail - tq_head >= 32u) {
                    emit_batch(tq_head, 32, out_next);
                    tq_head += 32u;
                    out_next += 32;
                }
            }
        }
        if (tq_tail != tq_head) emit_batch(tq_head, (int)(tq_tail - tq_head), out_next);
    }
}

#if !defined(GBT_REF_ARITH)
// ---------------------------------------------------------------------------
// Fixed-mode mesh with shared vertices.  (1) weld_mark: every cube that the
// fixed-mode marching cubes emits sets the bits of the grid edges its
// triangles use; (2) weld_count / weld_scan_blocks / weld_offsets: an
// exclusive scan of the bit counts numbers the used edges (vertex index =
// word offset + set bits below); (3) weld_vertices: one vertex per used
// edge, interpolated exactly as mc_emit_kernel<kFixed> interpolates it (lower
// endpoint first, so the positions are the ones the triangle soup holds),
// with the normal of the interpolated central-difference gradient;
// (4) mc_emit_kernel<kFixed> with edge_bits set writes the triangles as indices,
// in the same order as the triangle soup.
__global__ void __launch_bounds__(256) weld_mark_kernel(const __grid_constant__ McArgs a, uint32_t* bits) {
    __shared__ unsigned char s_count[256];
    __shared__ unsigned long long s_tri[256];
    __shared__ unsigned char s_ends[12];
    __shared__ unsigned char s_type[256];
    for (int k = threadIdx.x; k < 256; k += blockDim.x) {
        s_count[k] = GBT_MC_TRI_COUNT[k];
        s_tri[k] = GBT_MC_TRI_PACKED[k];
        s_type[k] = (unsigned char)mc_type_of_nibbles(k & 15, k >> 4);
    }
    if (threadIdx.x < 12) s_ends[threadIdx.x] = GBT_MC_EDGE_ENDS[threadIdx.x];
    __syncthreads();
    // whole warps take 32 consecutive cubes (the classification shuffles)
    const int lane = threadIdx.x & 31;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t w0 = (uint64_t)blockIdx.x * blockDim.x + (threadIdx.x & ~31u); w0 < a.ncubes; w0 += stride) {
        const bool valid = w0 + lane < a.ncubes;
        const uint32_t c = valid ? (uint32_t)(w0 + lane) : a.ncubes - 1;
        uint32_t idx[4];
        const bool own = cube_xcorners<kFixed>(a, c, idx) || lane == 31;
        int sx = 0, so = 0;
        bool okx = true, oko = true;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            sx |= (__ldg(a.D + idx[k]) < 0.f) << k;
            okx = okx && __ldg(a.W + idx[k]) > 0.f;
            if (own) {
                so |= (__ldg(a.D + idx[k] + 1) < 0.f) << k;
                oko = oko && __ldg(a.W + idx[k] + 1) > 0.f;
            }
        }
        sx |= okx << 4;
        so |= oko << 4;
        // every lane takes part in the shuffle; a lane then keeps its own loads or the next lane's
        const int nx = __shfl_down_sync(0xffffffffu, sx, 1);
        const int sn = own ? so : nx;
        if (!valid || !(sx & sn & 16)) continue;
        const int t = s_type[(sx & 15) | (sn & 15) << 4];
        const uint32_t row = fastdiv(c, a.div_cx);
        const uint32_t cx = c - row * (uint32_t)(a.gx - 1);
        const uint32_t cz = fastdiv(row, a.div_cy);
        const uint32_t cy = row - cz * (uint32_t)(a.gy - 1);
        const int n = s_count[t];
        const unsigned long long edges = s_tri[t];
        for (int q = 0; q < 3 * n; ++q) {
            const int e = (int)((edges >> (4 * q)) & 15ull);
            int ca = s_ends[e] & 15, cb = s_ends[e] >> 4;
            if (corner_dx(ca) + corner_dy(ca) + corner_dz(ca) > corner_dx(cb) + corner_dy(cb) + corner_dz(cb)) {
                const int tc = ca; ca = cb; cb = tc;
            }
            const int64_t id = weld_edge_id(a, cx, cy, cz, ca, cb);
            atomicOr(bits + (id >> 5), 1u << (id & 31));
        }
    }
}

__device__ __forceinline__ uint32_t block_sum_256(uint32_t v, uint32_t* s_warp) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) s_warp[threadIdx.x >> 5] = v;
    __syncthreads();
    uint32_t t = 0;
    for (int w = 0; w < 8; ++w) t += s_warp[w];
    return t;
}

// used edges per block of kWeldWordsPerBlock words (256 threads x 4 words)
__global__ void __launch_bounds__(256) weld_count_kernel(const uint32_t* bits, int64_t nwords, uint32_t* block_sums) {
    __shared__ uint32_t s_warp[8];
    const int64_t base = (int64_t)blockIdx.x * kWeldWordsPerBlock + 4 * threadIdx.x;
    uint32_t v = 0;
#pragma unroll
    for (int k = 0; k < 4; ++k)
        if (base + k < nwords) v += __popc(bits[base + k]);
    const uint32_t t = block_sum_256(v, s_warp);
    if (threadIdx.x == 0) block_sums[blockIdx.x] = t;
}

// exclusive scan of the block sums in place, one CTA of 1024 threads
__global__ void __launch_bounds__(1024) weld_scan_blocks_kernel(uint32_t* block_sums, int64_t nblocks,
                                                                long long* nverts) {
    __shared__ unsigned long long s_part[32];
    __shared__ unsigned long long s_carry;
    if (threadIdx.x == 0) s_carry = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int64_t base = 0; base < nblocks; base += 1024) {
        const int64_t i = base + threadIdx.x;
        const unsigned long long v = i < nblocks ? block_sums[i] : 0ull;
        unsigned long long x = v;
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned long long y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) s_part[warp] = x;
        __syncthreads();
        if (warp == 0) {
            unsigned long long p = s_part[lane];
            for (int o = 1; o < 32; o <<= 1) {
                const unsigned long long y = __shfl_up_sync(0xffffffffu, p, o);
                if (lane >= o) p += y;
            }
            s_part[lane] = p;
        }
        __syncthreads();
        const unsigned long long before = s_carry + (warp ? s_part[warp - 1] : 0ull) + x - v;
        if (i < nblocks) block_sums[i] = (uint32_t)before;
        __syncthreads();
        if (threadIdx.x == 0) s_carry += s_part[31];
        __syncthreads();
    }
    if (threadIdx.x == 0) *nverts = (long long)s_carry;
}

// vertex index of each word's first used edge
__global__ void __launch_bounds__(256) weld_offsets_kernel(const uint32_t* bits, int64_t nwords,
                                                           const uint32_t* block_offsets, uint32_t* word_offset) {
    __shared__ uint32_t s_warp[8];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int64_t base = (int64_t)blockIdx.x * kWeldWordsPerBlock + 4 * threadIdx.x;
    uint32_t c[4];
    uint32_t v = 0;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        c[k] = base + k < nwords ? (uint32_t)__popc(bits[base + k]) : 0u;
        v += c[k];
    }
    uint32_t x = v;
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) s_warp[warp] = x;
    __syncthreads();
    uint32_t before = block_offsets[blockIdx.x] + x - v;
    for (int w = 0; w < warp; ++w) before += s_warp[w];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        if (base + k < nwords) word_offset[base + k] = before;
        before += c[k];
    }
}

__device__ __forceinline__ void weld_gradient(const McArgs& a, int x, int y, int z, float* g) {
    const int n[3] = {a.gx, a.gy, a.gz};
    const int p[3] = {x, y, z};
    const int64_t stride[3] = {1, (int64_t)a.gx, (int64_t)a.gx * a.gy};
    const int64_t i = (int64_t)z * stride[2] + (int64_t)y * stride[1] + x;
#pragma unroll
    for (int q = 0; q < 3; ++q) {
        const int lo = p[q] > 0 ? 1 : 0, hi = p[q] + 1 < n[q] ? 1 : 0;
        const float d0 = a.D[i - lo * stride[q]], d1 = a.D[i + hi * stride[q]];
        g[q] = (lo + hi) ? (d1 - d0) / ((float)(lo + hi) * a.vs[q]) : 0.f;
    }
}

__global__ void __launch_bounds__(256) weld_vertices_kernel(const __grid_constant__ WeldArgs w) {
    const McArgs& a = w.mc;
    for (int64_t word = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; word < w.nwords;
         word += (int64_t)gridDim.x * blockDim.x) {
        uint32_t m = w.bits[word];
        int64_t vid = w.word_offset[word];
        while (m) {
            const int k = __ffs(m) - 1;
            m &= m - 1;
            const int64_t id = word * 32 + k;
            const int64_t lin = id / 3;
            const int axis = (int)(id - 3 * lin);
            const uint32_t row = fastdiv((uint32_t)lin, a.div_gx);
            const int x = (int)((uint32_t)lin - row * (uint32_t)a.gx);
            const uint32_t zz = fastdiv(row, a.div_gy);
            const int y = (int)(row - zz * (uint32_t)a.gy), z = (int)zz;
            const int x1 = x + (axis == 0), y1 = y + (axis == 1), z1 = z + (axis == 2);
            const int64_t lin1 = ((int64_t)z1 * a.gy + y1) * a.gx + x1;
            const float sa = a.D[lin], sb = a.D[lin1];
            const float pa[3] = {centre(x, a.vs[0], a.off[0]), centre(y, a.vs[1], a.off[1]), centre(z, a.vs[2], a.off[2])};
            const float pb[3] = {centre(x1, a.vs[0], a.off[0]), centre(y1, a.vs[1], a.off[1]),
                                 centre(z1, a.vs[2], a.off[2])};
            const float r = __fdiv_rn(sa, __fsub_rn(sa, sb));
            if (vid < w.cap_verts) {
#pragma unroll
                for (int q = 0; q < 3; ++q) w.verts[3 * vid + q] = __fmaf_rn(r, __fsub_rn(pb[q], pa[q]), pa[q]);
                if (w.normals) {
                    float ga[3], gb[3], nrm[3];
                    weld_gradient(a, x, y, z, ga);
                    weld_gradient(a, x1, y1, z1, gb);
                    float ss = 0.f;
#pragma unroll
                    for (int q = 0; q < 3; ++q) {
                        nrm[q] = ga[q] + r * (gb[q] - ga[q]);
                        ss += nrm[q] * nrm[q];
                    }
                    const float inv = ss > 0.f ? rsqrtf(ss) : 0.f;
#pragma unroll
                    for (int q = 0; q < 3; ++q) w.normals[3 * vid + q] = nrm[q] * inv;
                }
            }
            ++vid;
        }
    }
}
#endif

// ---------------------------------------------------------------------------
template <int MODE, int TX, int BY, int BZ>
cudaError_t launch_integrate_shape(const IntegrateArgs& a, int grid, bool stage, cudaStream_t s) {
    if (a.nframes <= kLaneBrickFrames) {
        if (stage)
            integrate_kernel<MODE, TX, BY, BZ, true, true><<<grid, 128, 0, s>>>(a);
        else
            integrate_kernel<MODE, TX, BY, BZ, true><<<grid, 128, 0, s>>>(a);
    } else {
        integrate_kernel<MODE, TX, BY, BZ, false><<<grid, 128, 0, s>>>(a);
    }
    return cudaGetLastError();
}

// brick 0-3: the four brick shapes; 4-7: the same shapes with the depth
// staged in shared memory (passes of up to kLaneBrickFrames frames)
template <int MODE>
cudaError_t launch_integrate_mode(const IntegrateArgs& a, int brick, int grid, cudaStream_t s) {
    const bool stage = brick >= 4;
    switch (brick & 3) {
        case 1: return launch_integrate_shape<MODE, 4, 8, 4>(a, grid, stage, s);
        case 2: return launch_integrate_shape<MODE, 8, 2, 8>(a, grid, stage, s);
        case 3: return launch_integrate_shape<MODE, 16, 2, 4>(a, grid, stage, s);
        default: return launch_integrate_shape<MODE, 8, 4, 4>(a, grid, stage, s);
    }
}

template <int MODE>
cudaError_t launch_stream_mode(const IntegrateArgs& a, const VolumeMaps& m, int grid, cudaStream_t s) {
    integrate_stream_kernel<MODE><<<grid, 128, 0, s>>>(a, m);
    return cudaGetLastError();
}

template <int MODE, int TX, int BY, int BZ>
cudaError_t launch_batch_shape(const BatchArgs& a, int grid, cudaStream_t s) {
    if (a.rows_of_4)
        integrate_batch_kernel<MODE, TX, BY, BZ, true><<<grid, 128, 0, s>>>(a);
    else
        integrate_batch_kernel<MODE, TX, BY, BZ, false><<<grid, 128, 0, s>>>(a);
    return cudaGetLastError();
}

template <int MODE>
cudaError_t launch_batch_mode(const BatchArgs& a, int brick, int grid, cudaStream_t s) {
    switch (brick) {
        case 1: return launch_batch_shape<MODE, 4, 8, 4>(a, grid, s);
        case 2: return launch_batch_shape<MODE, 8, 2, 8>(a, grid, s);
        case 3: return launch_batch_shape<MODE, 16, 2, 4>(a, grid, s);
        default: return launch_batch_shape<MODE, 8, 4, 4>(a, grid, s);
    }
}

// CTAs of an integrate kernel that fit on one SM at once (registers and
// shared memory decide it); the default persistent grid is SMs times this.
template <typename Kernel>
int resident_128(Kernel k) {
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k, 128, 0) != cudaSuccess) cudaGetLastError();
    return n > 0 ? n : 1;
}

// kind: 0 the pass kernel culling one frame per lane, 1 the pass kernel
// culling one brick per lane, 2 the batched kernel, 3 kind 1 with the depth
// staged in shared memory (4, the streamed pass kernel: resident_ctas_mode)
template <int MODE, int TX, int BY, int BZ>
int resident_shape(int kind) {
    if (kind == 2) return resident_128(integrate_batch_kernel<MODE, TX, BY, BZ, true>);
    if (kind == 3) return resident_128(integrate_kernel<MODE, TX, BY, BZ, true, true>);
    return kind == 1 ? resident_128(integrate_kernel<MODE, TX, BY, BZ, true>)
                     : resident_128(integrate_kernel<MODE, TX, BY, BZ, false>);
}

template <int MODE>
int resident_ctas_mode(int kind, int brick) {
    if (kind == 4) return resident_128(integrate_stream_kernel<MODE>);
    switch (brick) {
        case 1: return resident_shape<MODE, 4, 8, 4>(kind);
        case 2: return resident_shape<MODE, 8, 2, 8>(kind);
        case 3: return resident_shape<MODE, 16, 2, 4>(kind);
        default: return resident_shape<MODE, 8, 4, 4>(kind);
    }
}

// The three marching-cubes launches; the scratch words (total, list length,
// tile words, group bits) are zero when the first starts.
struct McGrid {
    int sms, per_count, per_count4, per_emit;
};

// SMs and resident CTAs of the count and emit kernels (thread-safe
// initialisation of a function-local static)
template <int MODE>
const McGrid& mc_grid() {
    static const McGrid g = [] {
        McGrid r{1, 1, 1, 1};
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&r.sms, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&r.per_count, mc_count_kernel<MODE>, kMcThreads, 0);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&r.per_count4, mc_count4_kernel<MODE>, kMcThreads, 0);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&r.per_emit, mc_emit_kernel<MODE>, kMcThreads, 0);
        cudaGetLastError();
        if (r.sms < 1) r.sms = 1;
        if (r.per_count < 1) r.per_count = 1;
        if (r.per_count4 < 1) r.per_count4 = 1;
        if (r.per_emit < 1) r.per_emit = 1;
        return r;
    }();
    return g;
}

template <int MODE>
bool mc_rows_of_4(const McArgs& a) {
    const long long layer = MODE == kCompat ? (long long)a.gx + a.gy : (long long)a.gx * a.gy;
    return a.gx >= 4 && a.gx % 4 == 0 && layer % 4 == 0 && (reinterpret_cast<uintptr_t>(a.D) & 15u) == 0 &&
           (MODE == kCompat || (reinterpret_cast<uintptr_t>(a.W) & 15u) == 0);
}

template <int MODE>
cudaError_t launch_mc_mode(const McArgs& a, cudaStream_t s) {
    const McGrid& mg = mc_grid<MODE>();
    const bool four = mc_rows_of_4<MODE>(a);
    // one warp per task (a segment of a cube layer, a run of rows)
    const long long seg = four ? kMcSeg4Cubes : kMcSegCubes;
    const long long rows = four ? kMcRows4PerTask : kMcRowsPerTask;
    const long long nseg = (a.gx - 1 + seg - 1) / seg;
    const long long nchunk = (a.gy - 1 + rows - 1) / rows;
    const long long ntasks = (long long)(a.gz - 1) * nchunk * nseg;
    long long grid = (long long)mg.sms * (four ? mg.per_count4 : mg.per_count);
    const long long need = (ntasks + kMcThreads / 32 - 1) / (kMcThreads / 32);
    if (grid > need) grid = need;
    if (grid < 1) grid = 1;
    if (four)
        mc_count4_kernel<MODE><<<(int)grid, kMcThreads, 0, s>>>(a);
    else
        mc_count_kernel<MODE><<<(int)grid, kMcThreads, 0, s>>>(a);
    const unsigned nsuper = (unsigned)((a.ntiles + kMcScanThreads - 1) / kMcScanThreads);
    mc_reduce_kernel<<<nsuper, kMcScanThreads, 0, s>>>(a);
    mc_scan_kernel<<<nsuper, kMcScanThreads, 0, s>>>(a);
    grid = (long long)mg.sms * mg.per_emit;
    const long long tiles_per_cta = kMcThreads / 32;   // a warp per listed tile at least
    if (grid > ((long long)a.ntiles + tiles_per_cta - 1) / tiles_per_cta)
        grid = ((long long)a.ntiles + tiles_per_cta - 1) / tiles_per_cta;
    if (grid < 1) grid = 1;
    mc_emit_kernel<MODE><<<(int)grid, kMcThreads, 0, s>>>(a);
    return cudaGetLastError();
}

}  // namespace GBT_ARITH_NS
}  // namespace gbt
