// Differentiable integrate: forward and adjoint, in float and in double.
//
// Forward, per voxel and frame (fixed-mode geometry, bilinear depth):
//   c = R p + t,  (u, v) = (fx c.x / z + cx, fy c.y / z + cy),
//   the 2x2 footprint around (u, v) with bilinear weights b_i and validity
//   v_i (pixel inside the image with depth in (0, max_depth]),
//   wv = sum b_i v_i,  d = sum b_i v_i d_i / wv,  sdf = d - z,
//   tsdf = min(sdf, trunc),  w = wv * ramp((sdf + trunc) / (trunc / 2)),
//   ramp(x) = clamp(x, 0, 1), and for w > 0:
//   D += w (tsdf - D) / (W + w),  W = min(W + w, M).
// Every cut is soft: a sample's weight goes to zero continuously as its
// footprint leaves the image or the valid depth, and at the back of the
// truncation band, so D and W are continuous in the pose and in every depth
// pixel (only z <= min_z is a hard cut).
//
// Adjoint: reverse mode through the recurrence with frame-chunk
// recomputation.  The forward writes (D, W) before every chunk of kChunk frames
// after the first; the adjoint walks the chunks backwards, recomputes each
// chunk forward from its checkpoint keeping the per-frame (D, W) in registers,
// then runs the chunk in reverse: for each update
//   dD_k/dD_{k-1} = W_{k-1}/(W_{k-1}+w),  dD_k/dtsdf = w/(W_{k-1}+w),
//   dD_k/dw = (tsdf - D_{k-1}) W_{k-1}/(W_{k-1}+w)^2,
//   dD_k/dW_{k-1} = -w (tsdf - D_{k-1})/(W_{k-1}+w)^2,
//   dW_k/dW_{k-1} = dW_k/dw = 1 below the clamp, 0 at it,
// then through min(., trunc), the ramp, the normalised bilinear sample
// (scattered to the valid pixels of dL/ddepth) and the projection to
// dL/dR = sum g_c p^T, dL/dt = sum g_c per frame.
#include <cstdint>
#include <cuda_runtime.h>

#include "gbt_internal.h"

namespace gbt {
namespace diff {

constexpr int kChunk = GBT_DIFF_CHUNK_FRAMES;

template <typename T> struct Ops;

template <> struct Ops<float> {
    __device__ static float fma(float a, float b, float c) { return __fmaf_rn(a, b, c); }
    __device__ static float mul(float a, float b) { return __fmul_rn(a, b); }
    __device__ static float add(float a, float b) { return __fadd_rn(a, b); }
    __device__ static float sub(float a, float b) { return __fsub_rn(a, b); }
    __device__ static float rcp(float a) { return __frcp_rn(a); }
    __device__ static float div(float a, float b) { return __fdiv_rn(a, b); }
    __device__ static float floor_(float a) { return floorf(a); }
    __device__ static float min_(float a, float b) { return fminf(a, b); }
};

template <> struct Ops<double> {
    __device__ static double fma(double a, double b, double c) { return __fma_rn(a, b, c); }
    __device__ static double mul(double a, double b) { return __dmul_rn(a, b); }
    __device__ static double add(double a, double b) { return __dadd_rn(a, b); }
    __device__ static double sub(double a, double b) { return __dsub_rn(a, b); }
    __device__ static double rcp(double a) { return __drcp_rn(a); }
    __device__ static double div(double a, double b) { return __ddiv_rn(a, b); }
    __device__ static double floor_(double a) { return floor(a); }
    __device__ static double min_(double a, double b) { return fmin(a, b); }
};

struct Geometry {
    int32_t nx, ny, nz;
    float vs[3], off[3];
    float fx, fy, cx, cy;
    float trunc, max_weight, max_depth, min_z;
    int32_t width, height;
    int32_t nframes;
};

// One voxel-frame.  band: 0 = weight 0, 1 = inside the ramp, 2 = full.
template <typename T> struct Sample {
    bool truncated;      // sdf > trunc
    int band;
    int u0, v0;
    int vmask;           // bit i: pixel i of the footprint is valid (00, 10, 01, 11)
    T a, b;
    T d[4];
    T wv, dn;            // valid bilinear weight, normalised depth
    T cx, cy, cz, rz;
    T sdf, tsdf, wband, w;
};

template <typename T>
__device__ __forceinline__ T voxel_centre(int v, float vs, float off) {
    using O = Ops<T>;
    return O::fma(O::add((T)v, (T)0.5), (T)vs, (T)off);
}

template <typename T>
__device__ __forceinline__ T ramp(T x, int* state) {
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
__device__ __forceinline__ void sample(const Geometry& g, const T* R, const T* t, const T* depth, T px, T py, T pz,
                                       Sample<T>& s) {
    using O = Ops<T>;
    s.w = (T)0;
    s.vmask = 0;
    s.cz = O::add(O::fma(R[8], pz, O::fma(R[6], px, O::mul(R[7], py))), t[2]);
    if (!(s.cz > (T)g.min_z)) return;
    s.cx = O::add(O::fma(R[2], pz, O::fma(R[0], px, O::mul(R[1], py))), t[0]);
    s.cy = O::add(O::fma(R[5], pz, O::fma(R[3], px, O::mul(R[4], py))), t[1]);
    s.rz = O::rcp(s.cz);
    const T u = O::fma((T)g.fx, O::mul(s.cx, s.rz), (T)g.cx);
    const T v = O::fma((T)g.fy, O::mul(s.cy, s.rz), (T)g.cy);
    if (!(u > (T)-1 && v > (T)-1 && u < (T)g.width && v < (T)g.height)) return;
    const T fu = O::floor_(u), fv = O::floor_(v);
    s.u0 = (int)fu;
    s.v0 = (int)fv;
    s.a = O::sub(u, fu);
    s.b = O::sub(v, fv);
    const T md = (T)g.max_depth;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const int x = s.u0 + (k & 1), y = s.v0 + (k >> 1);
        T dv = (T)0;
        if (x >= 0 && y >= 0 && x < g.width && y < g.height) dv = depth[(int64_t)y * g.width + x];
        s.d[k] = dv;
        if (dv > (T)0 && dv <= md) s.vmask |= 1 << k;
    }
    if (!s.vmask) return;
    const T ia = O::sub((T)1, s.a), ib = O::sub((T)1, s.b);
    const T bw[4] = {O::mul(ia, ib), O::mul(s.a, ib), O::mul(ia, s.b), O::mul(s.a, s.b)};
    T wv = (T)0, nd = (T)0;
#pragma unroll
    for (int k = 0; k < 4; ++k)
        if (s.vmask & (1 << k)) {
            wv = O::add(wv, bw[k]);
            nd = O::fma(bw[k], s.d[k], nd);
        }
    s.wv = wv;
    if (!(wv > (T)0)) return;
    s.dn = O::div(nd, wv);
    s.sdf = O::sub(s.dn, s.cz);
    const T tr = (T)g.trunc;
    s.truncated = s.sdf > tr;
    s.tsdf = O::min_(s.sdf, tr);
    s.wband = ramp<T>(O::mul(O::add(s.sdf, tr), O::div((T)2, tr)), &s.band);
    s.w = O::mul(s.wv, s.wband);
}

template <typename T>
__device__ __forceinline__ uint32_t decision_code(const Sample<T>& s, bool saturated) {
    if (!(s.w > (T)0)) return 0x7fffffffu;
    return ((uint32_t)(s.u0 * 4099 + s.v0 * 7) ^ ((uint32_t)s.band << 24) ^ ((uint32_t)s.vmask << 26) ^
            (s.truncated ? 0x80000000u : 0u) ^ (saturated ? 0x40000000u : 0u));
}

template <typename T>
__device__ __forceinline__ void load_poses(const Geometry& g, const T* rot, const T* trans, T (*s_pose)[12]) {
    for (int f = threadIdx.x; f < g.nframes; f += blockDim.x) {
        for (int k = 0; k < 9; ++k) s_pose[f][k] = rot[9 * f + k];
        for (int k = 0; k < 3; ++k) s_pose[f][9 + k] = trans[3 * f + k];
    }
}

template <typename T>
__device__ __forceinline__ void voxel_xyz(const Geometry& g, int64_t i, T* px, T* py, T* pz) {
    const int x = (int)(i % g.nx);
    const int64_t r = i / g.nx;
    const int y = (int)(r % g.ny), z = (int)(r / g.ny);
    *px = voxel_centre<T>(x, g.vs[0], g.off[0]);
    *py = voxel_centre<T>(y, g.vs[1], g.off[1]);
    *pz = voxel_centre<T>(z, g.vs[2], g.off[2]);
}

// One update of the running mean; returns whether the weight clamp was reached.
template <typename T>
__device__ __forceinline__ bool update(T& d, T& w, const Sample<T>& s, T M) {
    using O = Ops<T>;
    const T sw = O::add(w, s.w);
    d = O::fma(s.w, O::div(O::sub(s.tsdf, d), sw), d);
    const bool sat = !(sw < M);
    w = sat ? M : sw;
    return sat;
}

template <typename T>
__global__ void __launch_bounds__(256) forward_kernel(Geometry g, T* D, T* W, T* ckpt, uint32_t* signature,
                                                      const T* depth, const T* rot, const T* trans) {
    __shared__ T s_pose[kBatchMaxFrames][12];
    load_poses<T>(g, rot, trans, s_pose);
    __syncthreads();
    const int64_t n = (int64_t)g.nx * g.ny * g.nz;
    const int64_t frame = (int64_t)g.width * g.height;
    const T M = (T)g.max_weight;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        T px, py, pz;
        voxel_xyz<T>(g, i, &px, &py, &pz);
        T d = D[i], w = W[i];
        uint32_t sig = 2166136261u;
        for (int f = 0; f < g.nframes; ++f) {
            if (f > 0 && f % kChunk == 0 && ckpt) {
                T* c = ckpt + (int64_t)(f / kChunk - 1) * 2 * n;
                c[i] = d;
                c[n + i] = w;
            }
            Sample<T> s;
            sample<T>(g, s_pose[f], s_pose[f] + 9, depth + f * frame, px, py, pz, s);
            bool sat = false;
            if (s.w > (T)0) sat = update<T>(d, w, s, M);
            if (signature) sig = (sig ^ decision_code<T>(s, sat)) * 16777619u;
        }
        D[i] = d;
        W[i] = w;
        if (signature) signature[i] = sig;
    }
}

// Sums 12 per-lane values over the warp with a transposing butterfly: each
// of the five exchange rounds halves the values a lane keeps (16 -> 8 -> 4 ->
// 2 -> 1, the 12 padded to 16), 16 shuffles in all instead of 12 x 5.  On
// return, even lanes 0, 2, ..., 22 hold the warp total of value lane / 2.
template <typename T>
__device__ __forceinline__ T warp_sum12(const T (&acc)[12], int lane) {
    T v[16];
#pragma unroll
    for (int q = 0; q < 16; ++q) v[q] = q < 12 ? acc[q] : (T)0;
#pragma unroll
    for (int half = 8; half >= 1; half >>= 1) {
        const bool hi = (lane & (2 * half)) != 0;   // exchange distance 2*half: 16, 8, 4, 2
#pragma unroll
        for (int j = 0; j < half; ++j) {
            const T send = hi ? v[j] : v[j + half];
            const T keep = hi ? v[j + half] : v[j];
            v[j] = keep + __shfl_xor_sync(0xffffffffu, send, 2 * half);
        }
    }
    return v[0] + __shfl_xor_sync(0xffffffffu, v[0], 1);
}

constexpr int kBackThreads = 128;

// grad_pose: [nframes][12] doubles (dL/dR row-major, dL/dt), accumulated.
// grad_depth: [nframes][H][W] of T, accumulated.
// One thread per voxel, one CTA per kBackThreads voxels (CTAs finish
// independently, so warps with little work do not hold up the others).  The
// chunk's per-frame (D, W) history sits in shared memory, so the frame loops
// need no unrolling.  Pose sums: per warp and frame the 12 values are reduced
// across the warp in T and added into the CTA's shared accumulators in
// double.  In the float instance the sum of the four warps' float totals is
// then exact unless their magnitudes differ by more than 2^29, so it does not
// depend on the order in which the warps arrive (float accumulators did: pose
// refinement, whose line search branches on the loss, then took different
// paths from run to run); what still depends on the order is the last bit of
// grad_pose's double sums over CTAs.  The CTA's last warp to finish adds the
// non-zero totals into grad_pose (no end-of-CTA barrier: finished warps
// leave at once).
template <typename T>
__global__ void __launch_bounds__(kBackThreads) backward_kernel(Geometry g, const T* gD_in, const T* gW_in,
                                                                const T* D0, const T* W0, const T* ckpt,
                                                                const T* depth, const T* rot, const T* trans,
                                                                T* grad_depth, double* grad_pose, T* gD0, T* gW0) {
    __shared__ T s_pose[kBatchMaxFrames][12];
    __shared__ double s_acc[kBatchMaxFrames][12];
    __shared__ T s_hist[2 * kChunk][kBackThreads];   // D then W before each frame of the chunk
    __shared__ int s_done;                           // warps finished
    using O = Ops<T>;
    const int64_t n = (int64_t)g.nx * g.ny * g.nz;
    const int64_t i = blockIdx.x * (int64_t)kBackThreads + threadIdx.x;
    const bool inside = i < n;
    T gd = (T)0, gw = (T)0;
    if (inside) {
        gd = gD_in[i];
        gw = gW_in ? gW_in[i] : (T)0;
    }
    const bool active = inside && (gd != (T)0 || gw != (T)0);
    if (!__syncthreads_or(active)) {
        if (inside && gD0) gD0[i] = gd;
        if (inside && gW0) gW0[i] = gw;
        return;
    }
    load_poses<T>(g, rot, trans, s_pose);
    for (int e = threadIdx.x; e < g.nframes * 12; e += kBackThreads) s_acc[e / 12][e % 12] = 0.0;
    if (threadIdx.x == 0) s_done = 0;
    __syncthreads();
    const int64_t frame = (int64_t)g.width * g.height;
    const T M = (T)g.max_weight;
    const T tr = (T)g.trunc;
    const T half_inv = O::div((T)2, tr);
    const int lane = threadIdx.x & 31;
    const int t = threadIdx.x;
    T px = 0, py = 0, pz = 0;
    if (inside) voxel_xyz<T>(g, i, &px, &py, &pz);
    const bool warp_active = __any_sync(0xffffffffu, active);
    const int nchunks = (g.nframes + kChunk - 1) / kChunk;
    for (int c = nchunks - 1; c >= 0 && warp_active; --c) {
        const int f0 = c * kChunk;
        const int nk = min(kChunk, g.nframes - f0);
        // recompute the chunk forward from its starting state
        T d = (T)0, w = (T)0;
        unsigned seen = 0;   // bit k: frame f0 + k gave this voxel a sample
        if (active) {
            if (c == 0) {
                d = D0[i];
                w = W0[i];
            } else {
                const T* cp = ckpt + (int64_t)(c - 1) * 2 * n;
                d = cp[i];
                w = cp[n + i];
            }
        }
#pragma unroll 1
        for (int k = 0; k < nk; ++k) {
            s_hist[k][t] = d;
            s_hist[kChunk + k][t] = w;
            if (active) {
                Sample<T> s;
                sample<T>(g, s_pose[f0 + k], s_pose[f0 + k] + 9, depth + (f0 + k) * frame, px, py, pz, s);
                if (s.w > (T)0) {
                    update<T>(d, w, s, M);
                    seen |= 1u << k;
                }
            }
        }
        // reverse through the chunk
#pragma unroll 1
        for (int k = nk - 1; k >= 0; --k) {
            const int f = f0 + k;
            const bool here = (seen >> k) & 1u;
            if (!__any_sync(0xffffffffu, here)) continue;
            T acc[12];
#pragma unroll
            for (int q = 0; q < 12; ++q) acc[q] = (T)0;
            if (here) {
                Sample<T> s;
                sample<T>(g, s_pose[f], s_pose[f] + 9, depth + f * frame, px, py, pz, s);
                const T dprev = s_hist[k][t], wprev = s_hist[kChunk + k][t];
                const T sw = O::add(wprev, s.w);
                const T isw = O::rcp(sw);
                const T diff = O::sub(s.tsdf, dprev);
                const bool sat = !(sw < M);
                const T isw2 = O::mul(isw, isw);
                const T g_t = O::mul(gd, O::mul(s.w, isw));
                const T g_w = O::add(O::mul(gd, O::mul(O::mul(diff, wprev), isw2)), sat ? (T)0 : gw);
                const T gw_prev = O::add(O::mul(gd, O::mul(O::mul(-s.w, diff), isw2)), sat ? (T)0 : gw);
                gd = O::mul(gd, O::mul(wprev, isw));
                gw = gw_prev;
                // through tsdf = min(sdf, trunc), the ramp and wv
                T g_sdf = s.truncated ? (T)0 : g_t;
                if (s.band == 1) g_sdf = O::add(g_sdf, O::mul(g_w, O::mul(s.wv, half_inv)));
                const T g_wv = O::mul(g_w, s.wband);
                // d = N / wv over the valid pixels; sdf = d - z
                const T ia = O::sub((T)1, s.a), ib = O::sub((T)1, s.b);
                const T bw[4] = {O::mul(ia, ib), O::mul(s.a, ib), O::mul(ia, s.b), O::mul(s.a, s.b)};
                const T dba[4] = {-ib, ib, -s.b, s.b};   // d b_i / d a
                const T dbb[4] = {-ia, -s.a, ia, s.a};   // d b_i / d b
                const T iwv = O::rcp(s.wv);
                const T g_sdf_n = O::mul(g_sdf, iwv);
                T g_a = (T)0, g_b = (T)0;
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    if (!(s.vmask & (1 << q))) continue;
                    const T gdq = O::mul(g_sdf_n, bw[q]);
                    if (gdq != (T)0) {
                        const int x = s.u0 + (q & 1), y = s.v0 + (q >> 1);
                        atomicAdd(grad_depth + f * frame + (int64_t)y * g.width + x, gdq);
                    }
                    // d(N / wv)/da = sum_i dba_i (d_i - d) / wv; d wv / da = sum_i dba_i
                    const T e = O::fma(g_sdf_n, O::sub(s.d[q], s.dn), g_wv);
                    g_a = O::fma(dba[q], e, g_a);
                    g_b = O::fma(dbb[q], e, g_b);
                }
                const T gcx = O::mul(O::mul(g_a, (T)g.fx), s.rz);
                const T gcy = O::mul(O::mul(g_b, (T)g.fy), s.rz);
                const T gcz = O::sub(-g_sdf, O::mul(s.rz, O::fma(gcx, s.cx, O::mul(gcy, s.cy))));
                acc[0] = O::mul(gcx, px); acc[1] = O::mul(gcx, py); acc[2] = O::mul(gcx, pz);
                acc[3] = O::mul(gcy, px); acc[4] = O::mul(gcy, py); acc[5] = O::mul(gcy, pz);
                acc[6] = O::mul(gcz, px); acc[7] = O::mul(gcz, py); acc[8] = O::mul(gcz, pz);
                acc[9] = gcx; acc[10] = gcy; acc[11] = gcz;
            }
            const T tot = warp_sum12<T>(acc, lane);
            if (!(lane & 1) && lane < 24 && tot != (T)0) atomicAdd(&s_acc[f][lane >> 1], (double)tot);
        }
    }
    if (inside && gD0) gD0[i] = gd;
    if (inside && gW0) gW0[i] = gw;
    // the last warp of the CTA to get here flushes the CTA's pose sums
    __syncwarp();
    __threadfence_block();
    int last = 0;
    if (lane == 0) last = atomicAdd(&s_done, 1) == kBackThreads / 32 - 1;
    if (!__shfl_sync(0xffffffffu, last, 0)) return;
    __threadfence_block();
    for (int e = lane; e < g.nframes * 12; e += 32) {
        const double v = s_acc[e / 12][e % 12];
        if (v != 0.0) atomicAdd(grad_pose + e, v);
    }
}

Geometry geometry(const DiffArgs& a) {
    Geometry g;
    g.nx = a.nx;
    g.ny = a.ny;
    g.nz = a.nz;
    for (int i = 0; i < 3; ++i) {
        g.vs[i] = a.vs[i];
        g.off[i] = a.off[i];
    }
    g.fx = a.fx;
    g.fy = a.fy;
    g.cx = a.cx;
    g.cy = a.cy;
    g.trunc = a.trunc;
    g.max_weight = a.max_weight;
    g.max_depth = a.max_depth;
    g.min_z = a.min_z;
    g.width = a.width;
    g.height = a.height;
    g.nframes = a.nframes;
    return g;
}

int grid_for(int64_t n) {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    int64_t g = (n + 255) / 256;
    const int64_t cap = (int64_t)sms * 8;
    return (int)(g < cap ? (g < 1 ? 1 : g) : cap);
}

unsigned back_grid(int64_t n) { return (unsigned)((n + kBackThreads - 1) / kBackThreads); }

}  // namespace diff

cudaError_t launch_diff_forward(const DiffArgs& a, cudaStream_t s) {
    const int64_t n = (int64_t)a.nx * a.ny * a.nz;
    if (a.dtype == 1)
        diff::forward_kernel<double><<<diff::grid_for(n), 256, 0, s>>>(
            diff::geometry(a), (double*)a.D, (double*)a.W, (double*)a.ckpt, a.signature, (const double*)a.depth,
            (const double*)a.rot, (const double*)a.trans);
    else
        diff::forward_kernel<float><<<diff::grid_for(n), 256, 0, s>>>(
            diff::geometry(a), (float*)a.D, (float*)a.W, (float*)a.ckpt, a.signature, (const float*)a.depth,
            (const float*)a.rot, (const float*)a.trans);
    return cudaGetLastError();
}

cudaError_t launch_diff_backward(const DiffArgs& a, cudaStream_t s) {
    const int64_t n = (int64_t)a.nx * a.ny * a.nz;
    if (a.dtype == 1)
        diff::backward_kernel<double><<<diff::back_grid(n), diff::kBackThreads, 0, s>>>(
            diff::geometry(a), (const double*)a.grad_D, (const double*)a.grad_W, (const double*)a.D,
            (const double*)a.W, (const double*)a.ckpt, (const double*)a.depth, (const double*)a.rot,
            (const double*)a.trans, (double*)a.grad_depth, a.grad_pose, (double*)a.grad_D0, (double*)a.grad_W0);
    else
        diff::backward_kernel<float><<<diff::back_grid(n), diff::kBackThreads, 0, s>>>(
            diff::geometry(a), (const float*)a.grad_D, (const float*)a.grad_W, (const float*)a.D, (const float*)a.W,
            (const float*)a.ckpt, (const float*)a.depth, (const float*)a.rot, (const float*)a.trans, (float*)a.grad_depth,
            a.grad_pose, (float*)a.grad_D0, (float*)a.grad_W0);
    return cudaGetLastError();
}

}  // namespace gbt
