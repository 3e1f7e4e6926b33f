// CPU oracle for the TSDF integrate + marching-cubes path.
//
// TEST INFRASTRUCTURE ONLY.  This file is the checker that the CUDA engine is
// compared against; the engine never links, loads or calls it.  Only the test
// suite, the smoke check and the CPU-baseline leg of the benchmark use it.
//
// It restates, in plain C++ on the host, the arithmetic of the reference
// (SokratG/cu-Reconstruction):
//
//   compat integrate   modules/src/cuda/tsdf_volume.cu:144-190 (cu_tsdf_integrate)
//                      + camera_util.cu:7-19,44-51 (camera_to_pixel, world_to_pixel)
//                      + se3.cuh:125-140,165-183,207-223 (SE3 from quaternion, R*p+t)
//   volume set-up      tsdf_volume.cu:194-212,227-254 (voxel size, truncation, init)
//   compat mesh        marching_cubes.cu:23-157 (per-cube classification and
//                      edge interpolation) + :159-237 (layer loop, host assembly)
//   point clouds       cuda_point_cloud.cu:22-99 (point_cloud_extract,
//                      transform_points, filter_image_if) + :292-353 (the host
//                      z-buffer loop of project_to_color_depth)
//
// The reference is compiled with -use_fast_math, so its divisions are the
// GPU's approximate divide.  The oracle does NOT imitate that: every division
// here is an IEEE division, and every multiply-add that nvcc contracts in the
// reference is written as an explicit fmaf.  The engine's "IEEE" compat
// variant follows exactly these operations and must match this file bit for
// bit; the engine's reference-arithmetic variant is checked against the
// reference's own GPU build instead, and against this file up to the pixel
// indices flagged by oracle_compat_ambiguous().
//
// The "fixed" mode is the engine's geometrically corrected variant (camera
// space SDF, nearest-pixel rounding, weight clamp, true z-layer stride); it is
// restated here operation for operation as the engine defines it.
//
// Build with -ffp-contract=off so the compiler adds no contraction of its own.
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#include <algorithm>
#ifdef _OPENMP
#include <omp.h>
#endif

#define GBT_MC_CONST static const
#include "../cu-reconstruction_gb300/csrc/mc_tables.inc"
GBT_MC_TABLE_DATA

extern "C" {

typedef struct {
    int32_t grid[3];
    float phys[3];
    float offset[3];
    float fx, fy, cx, cy;
    float max_weight;
    float truncation;  // <= 0: the reference's 1.1 * |voxel size|
    float max_depth;   // <= 0: the reference's 24 m
    float min_z;       // fixed mode: nearest accepted camera depth (> 0 strict when 0)
} oracle_cfg;

}  // extern "C"

namespace {

struct Derived {
    float vs[3];
    float trunc;
    float max_depth;
    int64_t nx, ny, nz;
};

// tsdf_volume.cu:197 (voxel_size = physical_size / grid, cudaMath.cuh:1225)
// and :199 (1.1f * length(voxel_size), cudaMath.cuh:1487,1530).
Derived derive(const oracle_cfg* c) {
    Derived d;
    for (int i = 0; i < 3; ++i) d.vs[i] = c->phys[i] / (float)(uint32_t)c->grid[i];
    float dot = d.vs[0] * d.vs[0] + d.vs[1] * d.vs[1];
    dot = dot + d.vs[2] * d.vs[2];
    d.trunc = c->truncation > 0.f ? c->truncation : 1.1f * std::sqrt(dot);
    d.max_depth = c->max_depth > 0.f ? c->max_depth : 24.0f;
    d.nx = c->grid[0];
    d.ny = c->grid[1];
    d.nz = c->grid[2];
    return d;
}

// GPU float->int conversion semantics (cvt.rzi.s32.f32): truncate, saturate,
// NaN -> 0.  C++'s static_cast is undefined out of range, so spell it out.
inline int32_t f2i_rz_sat(float x) {
    if (x != x) return 0;
    if (x >= 2147483648.0f) return INT32_MAX;
    if (x <= -2147483904.0f) return INT32_MIN;
    return (int32_t)x;
}

// cvt.rni.s32.f32: round half to even, saturate, NaN -> 0.
inline int32_t f2i_rn_sat(float x) {
    if (x != x) return 0;
    if (x >= 2147483648.0f) return INT32_MAX;
    if (x <= -2147483904.0f) return INT32_MIN;
    return (int32_t)std::nearbyint(x);
}

// Voxel centre, tsdf_volume.cu:117-119: ((v + 0.5f) * voxel_size) + offset,
// contracted to one fused multiply-add.
inline float centre(int64_t v, float vs, float off) {
    return std::fma((float)v + 0.5f, vs, off);
}

struct Rot {
    float r[9];
};

// se3.cuh:125-140 + 207-223 in the rounding order of the reference's build:
// the first product of each entry fused into the add/sub, except
// R00 = 1-(yy+zz), which rounds both products.
Rot compat_rotation(float qx, float qy, float qz, float qw) {
    const float x = 2 * qx, y = 2 * qy, z = 2 * qz;
    const float wx = x * qw, wy = y * qw, wz = z * qw;
    const float xx = x * qx, yy = y * qy, zz = z * qz;
    Rot R;
    R.r[0] = 1 - (yy + zz);
    R.r[1] = std::fma(y, qx, -wz);
    R.r[2] = std::fma(z, qx, wy);
    R.r[3] = std::fma(y, qx, wz);
    R.r[4] = 1 - std::fma(x, qx, zz);
    R.r[5] = std::fma(z, qy, -wx);
    R.r[6] = std::fma(z, qx, -wy);
    R.r[7] = std::fma(z, qy, wx);
    R.r[8] = 1 - std::fma(x, qx, yy);
    return R;
}

// se3.cuh:165-175: rotate then translate; row . p contracted left to right.
inline float rot_row(const float* r, float px, float py, float pz, float t) {
    return std::fma(r[2], pz, std::fma(r[0], px, r[1] * py)) + t;
}

struct CompatPose {
    Rot R;
    float t[3];
};

// tsdf_volume.cu:271-272: quaternion (w,x,y,z) and translation cast to float.
CompatPose compat_pose(const double* pose) {
    CompatPose P;
    P.R = compat_rotation((float)pose[1], (float)pose[2], (float)pose[3], (float)pose[0]);
    P.t[0] = (float)pose[4];
    P.t[1] = (float)pose[5];
    P.t[2] = (float)pose[6];
    return P;
}

// camera_util.cu:44-51 then :7-19.  Returns false when the pixel is off the
// image (tsdf_volume.cu:166).  q_out receives the two pre-truncation values.
inline void compat_project(const CompatPose& P, const oracle_cfg* c, float px, float py, float pz,
                           int32_t* u, int32_t* v, float* qu, float* qv, float* cz_out) {
    *u = 0;
    *v = 0;
    *qu = 0.f;
    *qv = 0.f;
    *cz_out = 0.f;
    if (pz == 0.f) return;
    const float cxv = rot_row(P.R.r + 0, px, py, pz, P.t[0]);
    const float cyv = rot_row(P.R.r + 3, px, py, pz, P.t[1]);
    const float czv = rot_row(P.R.r + 6, px, py, pz, P.t[2]);
    *cz_out = czv;
    if (czv == 0.f) return;
    *qu = (cxv * c->fx) / czv + c->cx;
    *qv = (cyv * c->fy) / czv + c->cy;
    *u = f2i_rz_sat(*qu);
    *v = f2i_rz_sat(*qv);
}

int nthreads(int threads) {
#ifdef _OPENMP
    return threads > 0 ? threads : omp_get_max_threads();
#else
    (void)threads;
    return 1;
#endif
}

// Fixed mode projection: P = K [R | t] with R from the normalised quaternion,
// evaluated in double on the host and rounded to float once.
struct FixedPose {
    float P[12];  // rows: fx*R0 + cx*R2 | fy*R1 + cy*R2 | R2 (each 3 + translation)
};

FixedPose fixed_pose(const double* pose, const oracle_cfg* c) {
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
    const double fx = c->fx, fy = c->fy, cx = c->cx, cy = c->cy;
    FixedPose F;
    for (int k = 0; k < 3; ++k) {
        F.P[0 + k] = (float)(fx * R[0 + k] + cx * R[6 + k]);
        F.P[4 + k] = (float)(fy * R[3 + k] + cy * R[6 + k]);
        F.P[8 + k] = (float)R[6 + k];
    }
    F.P[3] = (float)(fx * t[0] + cx * t[2]);
    F.P[7] = (float)(fy * t[1] + cy * t[2]);
    F.P[11] = (float)t[2];
    return F;
}

}  // namespace

extern "C" {

void oracle_derive(const oracle_cfg* c, float* vs_out, float* trunc_out) {
    Derived d = derive(c);
    for (int i = 0; i < 3; ++i) vs_out[i] = d.vs[i];
    *trunc_out = d.trunc;
}

// tsdf_volume.cu:227-242: weights 0, distances = truncation distance.
void oracle_volume_init(const oracle_cfg* c, float* D, float* W) {
    Derived d = derive(c);
    const int64_t n = d.nx * d.ny * d.nz;
    for (int64_t i = 0; i < n; ++i) {
        D[i] = d.trunc;
        W[i] = 0.f;
    }
}

// One frame of cu_tsdf_integrate (tsdf_volume.cu:144-190) in IEEE arithmetic.
// depth: float metres, rows `pitch_bytes` apart.
void oracle_integrate_compat(const oracle_cfg* c, float* D, float* W, const float* depth,
                             int64_t pitch_bytes, int32_t width, int32_t height, const double* pose,
                             int32_t threads) {
    const Derived d = derive(c);
    const CompatPose P = compat_pose(pose);
    const int64_t rows = d.ny * d.nz;
#pragma omp parallel for schedule(static) num_threads(nthreads(threads))
    for (int64_t r = 0; r < rows; ++r) {
        const int64_t vy = r % d.ny, vz = r / d.ny;
        const float py = centre(vy, d.vs[1], c->offset[1]);
        const float pz = centre(vz, d.vs[2], c->offset[2]);
        int64_t idx = r * d.nx;
        for (int64_t vx = 0; vx < d.nx; ++vx, ++idx) {
            const float px = centre(vx, d.vs[0], c->offset[0]);
            int32_t u, v;
            float qu, qv, cz;
            compat_project(P, c, px, py, pz, &u, &v, &qu, &qv, &cz);
            if (u < 0 || (uint32_t)u >= (uint32_t)width || v < 0 || (uint32_t)v >= (uint32_t)height)
                continue;
            const float dv = *(const float*)((const char*)depth + (int64_t)v * pitch_bytes + 4 * (int64_t)u);
            if (dv <= 0.0f || (double)dv > 24.0) continue;
            const float sdf = dv - pz;
            if (sdf >= -d.trunc) {
                float tsdf = sdf;
                if (sdf > 0) tsdf = std::fmin(sdf, d.trunc);
                const float w = W[idx];
                const float nw = w + 1.0f;
                const float nd = std::fma(D[idx], w, tsdf) / nw;
                W[idx] = nw;
                D[idx] = nd;
            }
        }
    }
}

// Marks voxels whose compat pixel index could differ between the IEEE
// arithmetic above and the reference's approximate divide: the value before
// truncation is within `ulps` float ulps (relative) of a non-zero integer, or
// a camera/world z is exactly zero.  flags |= 1 for such voxels.
void oracle_compat_ambiguous(const oracle_cfg* c, const double* pose, int32_t width, int32_t height,
                             float ulps, uint8_t* flags, int32_t threads) {
    const Derived d = derive(c);
    const CompatPose P = compat_pose(pose);
    const int64_t rows = d.ny * d.nz;
    (void)width;
    (void)height;
#pragma omp parallel for schedule(static) num_threads(nthreads(threads))
    for (int64_t r = 0; r < rows; ++r) {
        const int64_t vy = r % d.ny, vz = r / d.ny;
        const float py = centre(vy, d.vs[1], c->offset[1]);
        const float pz = centre(vz, d.vs[2], c->offset[2]);
        int64_t idx = r * d.nx;
        for (int64_t vx = 0; vx < d.nx; ++vx, ++idx) {
            const float px = centre(vx, d.vs[0], c->offset[0]);
            int32_t u, v;
            float qu, qv, cz;
            compat_project(P, c, px, py, pz, &u, &v, &qu, &qv, &cz);
            bool amb = (pz == 0.f) || (cz == 0.f) || std::fabs(cz) < 1e-30f;
            for (float q : {qu, qv}) {
                const float rq = std::nearbyint(q);
                if (rq != 0.f && std::fabs(q - rq) <= ulps * 1.1920929e-7f * std::fmax(1.f, std::fabs(q)))
                    amb = true;
            }
            if (amb) flags[idx] |= 1;
        }
    }
}

// Fixed-mode integrate: camera-space SDF, round-to-nearest pixel, weight clamp.
// fmt 0: float metres; fmt 1: uint16 scaled by depth_scale.
void oracle_integrate_fixed(const oracle_cfg* c, float* D, float* W, const void* depth, int64_t pitch_bytes,
                            int32_t width, int32_t height, int32_t fmt, float depth_scale, const double* pose,
                            int32_t threads) {
    const Derived d = derive(c);
    const FixedPose F = fixed_pose(pose, c);
    const float* P = F.P;
    const int64_t rows = d.ny * d.nz;
    const float wmax = c->max_weight;
    const float min_z = c->min_z;
#pragma omp parallel for schedule(static) num_threads(nthreads(threads))
    for (int64_t r = 0; r < rows; ++r) {
        const int64_t vy = r % d.ny, vz = r / d.ny;
        const float py = centre(vy, d.vs[1], c->offset[1]);
        const float pz = centre(vz, d.vs[2], c->offset[2]);
        const float aU = std::fma(P[1], py, std::fma(P[2], pz, P[3]));
        const float aV = std::fma(P[5], py, std::fma(P[6], pz, P[7]));
        const float aZ = std::fma(P[9], py, std::fma(P[10], pz, P[11]));
        int64_t idx = r * d.nx;
        for (int64_t vx = 0; vx < d.nx; ++vx, ++idx) {
            const float px = centre(vx, d.vs[0], c->offset[0]);
            const float Z = std::fma(P[8], px, aZ);
            if (!(Z > min_z)) continue;
            const float U = std::fma(P[0], px, aU);
            const float V = std::fma(P[4], px, aV);
            const float rz = 1.0f / Z;
            const int32_t u = f2i_rn_sat(U * rz);
            const int32_t v = f2i_rn_sat(V * rz);
            if ((uint32_t)u >= (uint32_t)width || (uint32_t)v >= (uint32_t)height) continue;
            const char* row = (const char*)depth + (int64_t)v * pitch_bytes;
            float dv;
            if (fmt == 1)
                dv = (float)((const uint16_t*)row)[u] * depth_scale;
            else
                dv = ((const float*)row)[u];
            if (!(dv > 0.f && dv <= d.max_depth)) continue;
            const float sdf = dv - Z;
            if (!(sdf >= -d.trunc)) continue;
            const float tsdf = std::fmin(sdf, d.trunc);
            const float w = W[idx];
            const int32_t n = std::max(f2i_rz_sat(w), 0);
            const float inv = 1.0f / (float)(n + 1);
            D[idx] = std::fma(tsdf - D[idx], inv, D[idx]);
            W[idx] = std::fmin(w + 1.0f, wmax);
        }
    }
}

// ---------------------------------------------------------------------------
// Marching cubes.
// Corner numbering of marching_cubes.cu:118-127: 0 (x,y,z) 1 (x+1,y,z)
// 2 (x+1,y,z+1) 3 (x,y,z+1) 4 (x,y+1,z) 5 (x+1,y+1,z) 6 (x+1,y+1,z+1) 7 (x,y+1,z+1)
// where "z+1" is the next layer.
static const int kCornerDx[8] = {0, 1, 1, 0, 0, 1, 1, 0};
static const int kCornerDy[8] = {0, 0, 0, 0, 1, 1, 1, 1};
static const int kCornerDz[8] = {0, 0, 1, 1, 0, 0, 1, 1};

static inline int edge_start(int e) { return GBT_MC_EDGE_ENDS[e] & 15; }
static inline int edge_end(int e) { return GBT_MC_EDGE_ENDS[e] >> 4; }
static inline int tri_edge(int type, int k) { return (int)((GBT_MC_TRI_PACKED[type] >> (4 * k)) & 15); }

// Compat mesh: marching_cubes.cu:191-237 with layer stride gx+gy (:211) and
// positions taken from the voxel at the same linear index (:86-99,216-217).
// Emits 3 vertices per triangle (:159-189).  verts: 9 floats per triangle,
// tris: 3 ints per triangle, written only while below cap_tris.  Returns the
// number of triangles.
int64_t oracle_mc_compat(const oracle_cfg* c, const float* D, float* verts, int32_t* tris, int64_t cap_tris,
                         int64_t index_base, int32_t threads) {
    const Derived d = derive(c);
    const int64_t gx = d.nx, gy = d.ny, gz = d.nz;
    if (gx < 2 || gy < 2 || gz < 2) return 0;
    const int64_t layer = gx + gy;
    const int64_t nlayers = gz - 1;
    std::vector<int64_t> counts(nlayers + 1, 0);
    auto classify = [&](int64_t vz, int64_t vy, int64_t vx, float* val, int64_t* lin) -> int {
        const int64_t base = vz * layer + vy * gx + vx;
        const int64_t base2 = base + layer;
        lin[0] = base;
        lin[1] = base + 1;
        lin[2] = base2 + 1;
        lin[3] = base2;
        lin[4] = base + gx;
        lin[5] = base + gx + 1;
        lin[6] = base2 + gx + 1;
        lin[7] = base2 + gx;
        int type = 0;
        for (int k = 0; k < 8; ++k) {
            val[k] = D[lin[k]];
            if (val[k] < 0.f) type |= 1 << k;
        }
        return type;
    };
#pragma omp parallel for schedule(dynamic) num_threads(nthreads(threads))
    for (int64_t vz = 0; vz < nlayers; ++vz) {
        int64_t n = 0;
        for (int64_t vy = 0; vy < gy - 1; ++vy)
            for (int64_t vx = 0; vx < gx - 1; ++vx) {
                float val[8];
                int64_t lin[8];
                n += GBT_MC_TRI_COUNT[classify(vz, vy, vx, val, lin)];
            }
        counts[vz + 1] = n;
    }
    for (int64_t i = 0; i < nlayers; ++i) counts[i + 1] += counts[i];
    const int64_t total = counts[nlayers];
    const int64_t plane = gx * gy;
#pragma omp parallel for schedule(dynamic) num_threads(nthreads(threads))
    for (int64_t vz = 0; vz < nlayers; ++vz) {
        int64_t t = counts[vz];
        for (int64_t vy = 0; vy < gy - 1; ++vy)
            for (int64_t vx = 0; vx < gx - 1; ++vx) {
                float val[8];
                int64_t lin[8];
                const int type = classify(vz, vy, vx, val, lin);
                const int ntri = GBT_MC_TRI_COUNT[type];
                if (!ntri) continue;
                float pos[8][3];
                for (int k = 0; k < 8; ++k) {
                    const int64_t i = lin[k];
                    pos[k][0] = centre(i % gx, d.vs[0], c->offset[0]);
                    pos[k][1] = centre((i / gx) % gy, d.vs[1], c->offset[1]);
                    pos[k][2] = centre(i / plane, d.vs[2], c->offset[2]);
                }
                for (int tr = 0; tr < ntri; ++tr, ++t) {
                    if (t >= cap_tris) continue;
                    for (int j = 0; j < 3; ++j) {
                        const int e = tri_edge(type, 3 * tr + j);
                        int a = edge_start(e), b = edge_end(e);
                        float s = val[a], en = val[b];
                        if (s > 0 && en < 0) {  // marching_cubes.cu:34-41
                            std::swap(a, b);
                            std::swap(s, en);
                        }
                        const float ratio = (-s) / (en - s);
                        float* out = verts + 9 * t + 3 * j;
                        for (int k = 0; k < 3; ++k) out[k] = std::fma(ratio, pos[b][k] - pos[a][k], pos[a][k]);
                        tris[3 * t + j] = (int32_t)(index_base + 3 * t + j);
                    }
                }
            }
    }
    return total;
}

// Fixed-mode mesh: true layer stride, cubes with an unobserved corner
// (weight 0) skipped, each edge interpolated from its lower-index endpoint so
// both cubes sharing an edge compute the same point.
int64_t oracle_mc_fixed(const oracle_cfg* c, const float* D, const float* W, float* verts, int32_t* tris,
                        int64_t cap_tris, int64_t index_base, int32_t threads) {
    const Derived d = derive(c);
    const int64_t gx = d.nx, gy = d.ny, gz = d.nz;
    if (gx < 2 || gy < 2 || gz < 2) return 0;
    const int64_t plane = gx * gy;
    const int64_t nlayers = gz - 1;
    std::vector<int64_t> counts(nlayers + 1, 0);
    auto classify = [&](int64_t vz, int64_t vy, int64_t vx, float* val) -> int {
        int type = 0;
        for (int k = 0; k < 8; ++k) {
            const int64_t i = (vz + kCornerDz[k]) * plane + (vy + kCornerDy[k]) * gx + vx + kCornerDx[k];
            if (!(W[i] > 0.f)) return 0;
            val[k] = D[i];
            if (val[k] < 0.f) type |= 1 << k;
        }
        return type;
    };
#pragma omp parallel for schedule(dynamic) num_threads(nthreads(threads))
    for (int64_t vz = 0; vz < nlayers; ++vz) {
        int64_t n = 0;
        for (int64_t vy = 0; vy < gy - 1; ++vy)
            for (int64_t vx = 0; vx < gx - 1; ++vx) {
                float val[8];
                n += GBT_MC_TRI_COUNT[classify(vz, vy, vx, val)];
            }
        counts[vz + 1] = n;
    }
    for (int64_t i = 0; i < nlayers; ++i) counts[i + 1] += counts[i];
    const int64_t total = counts[nlayers];
#pragma omp parallel for schedule(dynamic) num_threads(nthreads(threads))
    for (int64_t vz = 0; vz < nlayers; ++vz) {
        int64_t t = counts[vz];
        for (int64_t vy = 0; vy < gy - 1; ++vy)
            for (int64_t vx = 0; vx < gx - 1; ++vx) {
                float val[8];
                const int type = classify(vz, vy, vx, val);
                const int ntri = GBT_MC_TRI_COUNT[type];
                if (!ntri) continue;
                for (int tr = 0; tr < ntri; ++tr, ++t) {
                    if (t >= cap_tris) continue;
                    for (int j = 0; j < 3; ++j) {
                        const int e = tri_edge(type, 3 * tr + j);
                        int a = edge_start(e), b = edge_end(e);
                        // lower endpoint first: the one with the smaller offset on the edge's axis
                        if (kCornerDx[a] + kCornerDy[a] + kCornerDz[a] > kCornerDx[b] + kCornerDy[b] + kCornerDz[b])
                            std::swap(a, b);
                        const float pa[3] = {centre(vx + kCornerDx[a], d.vs[0], c->offset[0]),
                                             centre(vy + kCornerDy[a], d.vs[1], c->offset[1]),
                                             centre(vz + kCornerDz[a], d.vs[2], c->offset[2])};
                        const float pb[3] = {centre(vx + kCornerDx[b], d.vs[0], c->offset[0]),
                                             centre(vy + kCornerDy[b], d.vs[1], c->offset[1]),
                                             centre(vz + kCornerDz[b], d.vs[2], c->offset[2])};
                        const float tt = val[a] / (val[a] - val[b]);
                        float* out = verts + 9 * t + 3 * j;
                        for (int k = 0; k < 3; ++k) out[k] = std::fma(tt, pb[k] - pa[k], pa[k]);
                        tris[3 * t + j] = (int32_t)(index_base + 3 * t + j);
                    }
                }
            }
    }
    return total;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Differentiable integrate (the engine's definition, include/gbt_tsdf.h):
// fixed-mode geometry, validity-normalised bilinear depth over the 2x2
// footprint, sample weight w = (sum of the valid pixels' bilinear weights) *
// ramp((sdf + tr)/(tr/2)), weighted running mean with clamped weight.  The forward is restated operation for operation
// in float and double; the gradient is plain reverse mode in double over each
// voxel's whole history (no chunks, no checkpoints).

extern "C" {

typedef struct {
    uint32_t grid[3];
    float vs[3];
    float off[3];
    float fx, fy, cx, cy;
    float trunc, max_weight, max_depth, min_z;
    int32_t width, height;
    int32_t dtype;
} oracle_diff_cfg;

}  // extern "C"

namespace {

template <typename T> struct DSample {
    bool truncated = false;
    int band = 0, u0 = 0, v0 = 0, vmask = 0;
    T a = 0, b = 0, d[4] = {0, 0, 0, 0}, wv = 0, dn = 0, cx = 0, cy = 0, cz = 0, rz = 0, sdf = 0, tsdf = 0,
      wband = 0, w = 0;
};

template <typename T>
T dcentre(int64_t v, float vs, float off) {
    return std::fma((T)v + (T)0.5, (T)vs, (T)off);
}

template <typename T>
T dramp(T x, int* state) {
    if (!(x > (T)0)) {
        *state = 0;
        return (T)0;
    }
    if (x >= (T)1) {
        *state = 2;
        return (T)1;
    }
    *state = 1;
    return x;
}

template <typename T>
DSample<T> dsample(const oracle_diff_cfg* g, const T* R, const T* t, const T* depth, T px, T py, T pz) {
    DSample<T> s;
    s.cz = std::fma(R[8], pz, std::fma(R[6], px, R[7] * py)) + t[2];
    if (!(s.cz > (T)g->min_z)) return s;
    s.cx = std::fma(R[2], pz, std::fma(R[0], px, R[1] * py)) + t[0];
    s.cy = std::fma(R[5], pz, std::fma(R[3], px, R[4] * py)) + t[1];
    s.rz = (T)1 / s.cz;
    const T u = std::fma((T)g->fx, s.cx * s.rz, (T)g->cx);
    const T v = std::fma((T)g->fy, s.cy * s.rz, (T)g->cy);
    if (!(u > (T)-1 && v > (T)-1 && u < (T)g->width && v < (T)g->height)) return s;
    const T fu = std::floor(u), fv = std::floor(v);
    s.u0 = (int)fu;
    s.v0 = (int)fv;
    s.a = u - fu;
    s.b = v - fv;
    const T md = (T)g->max_depth;
    for (int k = 0; k < 4; ++k) {
        const int x = s.u0 + (k & 1), y = s.v0 + (k >> 1);
        T dv = 0;
        if (x >= 0 && y >= 0 && x < g->width && y < g->height) dv = depth[(int64_t)y * g->width + x];
        s.d[k] = dv;
        if (dv > 0 && dv <= md) s.vmask |= 1 << k;
    }
    if (!s.vmask) return s;
    const T ia = (T)1 - s.a, ib = (T)1 - s.b;
    const T bw[4] = {ia * ib, s.a * ib, ia * s.b, s.a * s.b};
    T wv = 0, nd = 0;
    for (int k = 0; k < 4; ++k)
        if (s.vmask & (1 << k)) {
            wv = wv + bw[k];
            nd = std::fma(bw[k], s.d[k], nd);
        }
    s.wv = wv;
    if (!(wv > 0)) return s;
    s.dn = nd / wv;
    s.sdf = s.dn - s.cz;
    const T tr = (T)g->trunc;
    s.truncated = s.sdf > tr;
    s.tsdf = std::fmin(s.sdf, tr);
    s.wband = dramp<T>((s.sdf + tr) * ((T)2 / tr), &s.band);
    s.w = s.wv * s.wband;
    return s;
}

template <typename T>
uint32_t dcode(const DSample<T>& s, bool sat) {
    if (!(s.w > (T)0)) return 0x7fffffffu;
    return ((uint32_t)(s.u0 * 4099 + s.v0 * 7) ^ ((uint32_t)s.band << 24) ^ ((uint32_t)s.vmask << 26) ^
            (s.truncated ? 0x80000000u : 0u) ^ (sat ? 0x40000000u : 0u));
}

template <typename T>
bool dupdate(T& d, T& w, const DSample<T>& s, T M) {
    const T sw = w + s.w;
    d = std::fma(s.w, (s.tsdf - d) / sw, d);
    const bool sat = !(sw < M);
    w = sat ? M : sw;
    return sat;
}

template <typename T>
void diff_forward(const oracle_diff_cfg* g, T* D, T* W, uint32_t* sig, const T* depth, int nframes, const T* rot,
                  const T* trans, int threads) {
    const int64_t nx = g->grid[0], ny = g->grid[1], nz = g->grid[2];
    const int64_t frame = (int64_t)g->width * g->height;
    const T M = (T)g->max_weight;
#pragma omp parallel for schedule(static) num_threads(nthreads(threads))
    for (int64_t i = 0; i < nx * ny * nz; ++i) {
        const int64_t x = i % nx, r = i / nx, y = r % ny, z = r / ny;
        const T px = dcentre<T>(x, g->vs[0], g->off[0]);
        const T py = dcentre<T>(y, g->vs[1], g->off[1]);
        const T pz = dcentre<T>(z, g->vs[2], g->off[2]);
        T d = D[i], w = W[i];
        uint32_t h = 2166136261u;
        for (int f = 0; f < nframes; ++f) {
            const DSample<T> s = dsample<T>(g, rot + 9 * f, trans + 3 * f, depth + f * frame, px, py, pz);
            bool sat = false;
            if (s.w > (T)0) sat = dupdate<T>(d, w, s, M);
            h = (h ^ dcode<T>(s, sat)) * 16777619u;
        }
        D[i] = d;
        W[i] = w;
        if (sig) sig[i] = h;
    }
}

}  // namespace

extern "C" {

void oracle_diff_forward(const oracle_diff_cfg* g, void* D, void* W, uint32_t* sig, const void* depth,
                         int32_t nframes, const void* rot, const void* trans, int32_t threads) {
    if (g->dtype == 1)
        diff_forward<double>(g, (double*)D, (double*)W, sig, (const double*)depth, nframes, (const double*)rot,
                             (const double*)trans, threads);
    else
        diff_forward<float>(g, (float*)D, (float*)W, sig, (const float*)depth, nframes, (const float*)rot,
                            (const float*)trans, threads);
}

// Reverse mode in double: gradients of a loss with dL/dD = grad_D and
// dL/dW = grad_W (may be NULL) of the final volume, through a forward that
// started from (D0, W0).  Accumulates grad_depth [F][H][W] and grad_pose
// [F][12] (dL/dR row-major, dL/dt); writes grad_D0, grad_W0 when not NULL.
void oracle_diff_backward(const oracle_diff_cfg* g, const double* grad_D, const double* grad_W, const double* D0,
                          const double* W0, const double* depth, int32_t nframes, const double* rot,
                          const double* trans, double* grad_depth, double* grad_pose, double* grad_D0,
                          double* grad_W0) {
    const int64_t nx = g->grid[0], ny = g->grid[1], nz = g->grid[2];
    const int64_t frame = (int64_t)g->width * g->height;
    const double M = g->max_weight, tr = g->trunc, half_inv = 2.0 / tr;
    std::vector<DSample<double>> smp(nframes);
    std::vector<double> dprev(nframes), wprev(nframes);
    for (int64_t i = 0; i < nx * ny * nz; ++i) {
        double gd = grad_D[i], gw = grad_W ? grad_W[i] : 0.0;
        if (gd != 0.0 || gw != 0.0) {
            const int64_t x = i % nx, r = i / nx, y = r % ny, z = r / ny;
            const double px = dcentre<double>(x, g->vs[0], g->off[0]);
            const double py = dcentre<double>(y, g->vs[1], g->off[1]);
            const double pz = dcentre<double>(z, g->vs[2], g->off[2]);
            double d = D0[i], w = W0[i];
            for (int f = 0; f < nframes; ++f) {
                smp[f] = dsample<double>(g, rot + 9 * f, trans + 3 * f, depth + f * frame, px, py, pz);
                dprev[f] = d;
                wprev[f] = w;
                if (smp[f].w > 0) dupdate<double>(d, w, smp[f], M);
            }
            for (int f = nframes - 1; f >= 0; --f) {
                const DSample<double>& s = smp[f];
                if (!(s.w > 0)) continue;
                const double sw = wprev[f] + s.w;
                const bool sat = !(sw < M);
                const double diff = s.tsdf - dprev[f];
                const double g_t = gd * s.w / sw;
                const double g_w = gd * diff * wprev[f] / (sw * sw) + (sat ? 0.0 : gw);
                const double gw_prev = -gd * s.w * diff / (sw * sw) + (sat ? 0.0 : gw);
                gd = gd * wprev[f] / sw;
                gw = gw_prev;
                double g_sdf = s.truncated ? 0.0 : g_t;
                if (s.band == 1) g_sdf += g_w * s.wv * half_inv;
                const double g_wv = g_w * s.wband;
                const double ia = 1 - s.a, ib = 1 - s.b;
                const double bw[4] = {ia * ib, s.a * ib, ia * s.b, s.a * s.b};
                const double dba[4] = {-ib, ib, -s.b, s.b};
                const double dbb[4] = {-ia, -s.a, ia, s.a};
                double g_a = 0, g_b = 0;
                for (int q = 0; q < 4; ++q) {
                    if (!(s.vmask & (1 << q))) continue;
                    const int x = s.u0 + (q & 1), y = s.v0 + (q >> 1);
                    grad_depth[f * frame + (int64_t)y * g->width + x] += g_sdf * bw[q] / s.wv;
                    // d d / d a = sum dba (d_i - d) / wv over valid pixels; d wv / d a = sum dba
                    g_a += dba[q] * (g_sdf * (s.d[q] - s.dn) / s.wv + g_wv);
                    g_b += dbb[q] * (g_sdf * (s.d[q] - s.dn) / s.wv + g_wv);
                }
                const double gx = g_a * g->fx / s.cz;
                const double gy = g_b * g->fy / s.cz;
                const double gz = -g_sdf - (gx * s.cx + gy * s.cy) / s.cz;
                double* gp = grad_pose + 12 * f;
                const double p[3] = {px, py, pz};
                for (int k = 0; k < 3; ++k) {
                    gp[k] += gx * p[k];
                    gp[3 + k] += gy * p[k];
                    gp[6 + k] += gz * p[k];
                }
                gp[9] += gx;
                gp[10] += gy;
                gp[11] += gz;
            }
        }
        if (grad_D0) grad_D0[i] = gd;
        if (grad_W0) grad_W0[i] = gw;
    }
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Point clouds: cudaPointCloud (cuda_point_cloud.cu:22-385) restated.  A point
// is the reference's packed 33-byte Vertex (cuda_point_cloud.cuh:17-28):
// float pos[3], float normal[4], uint8 color[3], uint16 classID.
namespace {

constexpr int kPointBytes = 33;

inline void point_pos(const uint8_t* pt, float* p) { std::memcpy(p, pt, 12); }

inline void pose_apply(const CompatPose& P, const float* p, float* out) {
    out[0] = rot_row(P.R.r + 0, p[0], p[1], p[2], P.t[0]);
    out[1] = rot_row(P.R.r + 3, p[0], p[1], p[2], P.t[1]);
    out[2] = rot_row(P.R.r + 6, p[0], p[1], p[2], P.t[2]);
}

}  // namespace

extern "C" {

// point_cloud_extract (cuda_point_cloud.cu:22-70): K as the kernel reads it
// (K[0][0], K[1][1], K[2][0], K[2][1] of the double[3][3] copied from the
// 9-array: m[0], m[4], m[6], m[7]); back-projection in double
// ((float)x - cx) * d / fx, rounded to float; pixels with depth <= 0 leave
// their slot untouched; colour rgb or white.  depth: W*H float metres.
void oracle_points_extract(const double* m, const float* depth, const uint8_t* rgb, int32_t W, int32_t H,
                           const double* pose, int64_t start, uint8_t* points) {
    const CompatPose P = compat_pose(pose);
    const double fx = m[0], fy = m[4], cx = m[6], cy = m[7];
    for (int32_t y = 0; y < H; ++y)
        for (int32_t x = 0; x < W; ++x) {
            const float d = depth[(int64_t)y * W + x];
            if (d <= 0.0f) continue;
            const float p[3] = {(float)((((double)(float)x) - cx) * (double)d / fx),
                                (float)((((double)(float)y) - cy) * (double)d / fy), d};
            float w[7] = {0, 0, 0, 0, 0, 0, 0};
            pose_apply(P, p, w);
            uint8_t* dst = points + (start + (int64_t)y * W + x) * kPointBytes;
            std::memcpy(dst, w, 28);
            const uint8_t* c = rgb ? rgb + ((int64_t)y * W + x) * 3 : nullptr;
            dst[28] = c ? c[0] : 255;
            dst[29] = c ? c[1] : 255;
            dst[30] = c ? c[2] : 255;
            dst[31] = 0;
            dst[32] = 0;
        }
}

// transform_points (cuda_point_cloud.cu:73-86).
void oracle_points_transform(uint8_t* points, int64_t n, const double* pose) {
    const CompatPose P = compat_pose(pose);
    for (int64_t i = 0; i < n; ++i) {
        float p[3], w[3];
        point_pos(points + i * kPointBytes, p);
        pose_apply(P, p, w);
        std::memcpy(points + i * kPointBytes, w, 12);
    }
}

// The pose as the reference's host build applies it in the projection loop
// (SE3<float>, se3.cuh:42-61,82-95,124-140): every product and sum rounded on
// its own, left to right (this file is compiled with -ffp-contract=off; g++
// -O3 for x86-64 emits no fused multiply-add either).
struct HostPose {
    float R[9], t[3];
};
HostPose host_pose(const double* pose) {
    const float qx = (float)pose[1], qy = (float)pose[2], qz = (float)pose[3], qw = (float)pose[0];
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
    h.t[0] = (float)pose[4];
    h.t[1] = (float)pose[5];
    h.t[2] = (float)pose[6];
    return h;
}

// project_to_color_depth (cuda_point_cloud.cu:292-353): the host z-buffer
// loop in point order, then filter_image_if(FLT_MAX -> 0).  K read as
// m[0], m[4], m[2], m[5].  The pixel is (int)((x*fx)/z + cx) in float; a
// non-finite value is dropped.  rgb may be NULL (project_to_depth).
void oracle_points_project(const uint8_t* points, int64_t n, const double* m, const double* pose, int32_t W,
                           int32_t H, float* depth, uint8_t* rgb) {
    const HostPose P = host_pose(pose);
    const float fx = (float)m[0], fy = (float)m[4], cx = (float)m[2], cy = (float)m[5];
    for (int64_t i = 0; i < (int64_t)W * H; ++i) depth[i] = FLT_MAX;
    if (rgb) std::memset(rgb, 0, (size_t)W * H * 3);
    for (int64_t i = 0; i < n; ++i) {
        const uint8_t* pt = points + i * kPointBytes;
        float p[3], c[3];
        point_pos(pt, p);
        for (int r = 0; r < 3; ++r) c[r] = P.R[3 * r] * p[0] + P.R[3 * r + 1] * p[1] + P.R[3 * r + 2] * p[2] + P.t[r];
        if (c[2] == 0.f) continue;
        const float qu = (c[0] * fx) / c[2] + cx;
        const float qv = (c[1] * fy) / c[2] + cy;
        if (qu != qu || qv != qv) continue;
        const int32_t u = f2i_rz_sat(qu), v = f2i_rz_sat(qv);
        if (u < 0 || u >= W || v < 0 || v >= H) continue;
        float& dv = depth[(int64_t)v * W + u];
        if (dv > c[2]) {
            dv = c[2];
            if (rgb) std::memcpy(rgb + ((int64_t)v * W + u) * 3, pt + 28, 3);
        }
    }
    for (int64_t i = 0; i < (int64_t)W * H; ++i)
        if (std::fabs(depth[i] - FLT_MAX) < 1e-10f) depth[i] = 0.0f;
}

// filter_image_if (cuda_point_cloud.cu:89-99) with near_equal (util.cu:6-10).
void oracle_filter_if(float* img, int64_t n, float filter_value, float set_value) {
    for (int64_t i = 0; i < n; ++i)
        if (std::fabs(img[i] - filter_value) < 1e-10f) img[i] = set_value;
}

}  // extern "C"
