// Differentiable integrate: forward and adjoint, in float and in double.
//
// The forward is the fixed mode's running average with bilinear depth
// sampling, so the result is differentiable in the pose and in each depth
// pixel:  c = R p + t,  (u, v) = (fx c.x / z + cx, fy c.y / z + cy),
// d = bilinear(depth, u, v) (all four pixels valid), sdf = d - z,
// tsdf = min(sdf, trunc), D += (tsdf - D) / (w + 1), w = min(w + 1, M).
// A voxel-frame counts only with z > min_z, the 2x2 footprint inside the image
// and sdf >= -trunc.  The forward also writes n, the number of updates each
// voxel received.
//
// Adjoint.  The recurrence is linear in the updates: D_final =
// prod(1 - a_j) D_0 + sum_m beta_m tsdf_m with a_j = 1 / (min(w0 + j - 1, M) + 1)
// for the j-th update of the voxel and beta_m = a_m prod_{j>m} (1 - a_j); the
// weights do not depend on the continuous inputs.  beta_m has a closed form in
// (m, n, w0, M) -- 1 / (w0 + n) while the weight stays below M, a geometric
// tail once it saturates -- so the adjoint recomputes each voxel-frame once, in
// forward order, with no per-frame volumes stored: dL/dtsdf_m = g beta_m for
// g = dL/dD_final, then through min(., trunc), the bilinear sample (scattered
// to the four pixels of dL/ddepth) and the projection to dL/dR = sum g_c p^T,
// dL/dt = sum g_c per frame (g_c = dL/dc).
#include <cstdint>
#include <cuda_runtime.h>

#include "gbt_internal.h"

namespace gbt {
namespace diff {

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
    __device__ static float pow_(float a, float e) { return powf(a, e); }
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
    __device__ static double pow_(double a, double e) { return pow(a, e); }
};

struct Geometry {
    int32_t nx, ny, nz;
    float vs[3], off[3];
    float fx, fy, cx, cy;
    float trunc, max_weight, max_depth, min_z;
    int32_t width, height;
    int32_t nframes;
};

// Everything the forward and the adjoint need about one voxel-frame.
template <typename T> struct Sample {
    bool valid;
    bool truncated;      // sdf > trunc: tsdf = trunc, no gradient
    int u0, v0;
    T a, b;              // bilinear fractions
    T d00, d10, d01, d11;
    T cx, cy, cz;        // camera coordinates
    T rz;
    T sdf, tsdf;
};

template <typename T>
__device__ __forceinline__ T voxel_centre(int v, float vs, float off) {
    using O = Ops<T>;
    return O::fma(O::add((T)v, (T)0.5), (T)vs, (T)off);
}

template <typename T>
__device__ __forceinline__ void sample(const Geometry& g, const T* R, const T* t, const T* depth, T px, T py, T pz,
                                       Sample<T>& s) {
    using O = Ops<T>;
    s.valid = false;
    s.cz = O::add(O::fma(R[8], pz, O::fma(R[6], px, O::mul(R[7], py))), t[2]);
    if (!(s.cz > (T)g.min_z)) return;
    s.cx = O::add(O::fma(R[2], pz, O::fma(R[0], px, O::mul(R[1], py))), t[0]);
    s.cy = O::add(O::fma(R[5], pz, O::fma(R[3], px, O::mul(R[4], py))), t[1]);
    s.rz = O::rcp(s.cz);
    const T u = O::fma((T)g.fx, O::mul(s.cx, s.rz), (T)g.cx);
    const T v = O::fma((T)g.fy, O::mul(s.cy, s.rz), (T)g.cy);
    if (!(u >= (T)0 && v >= (T)0 && u < (T)(g.width - 1) && v < (T)(g.height - 1))) return;
    const T fu = O::floor_(u), fv = O::floor_(v);
    s.u0 = (int)fu;
    s.v0 = (int)fv;
    s.a = O::sub(u, fu);
    s.b = O::sub(v, fv);
    const T* row0 = depth + (int64_t)s.v0 * g.width + s.u0;
    const T* row1 = row0 + g.width;
    s.d00 = row0[0];
    s.d10 = row0[1];
    s.d01 = row1[0];
    s.d11 = row1[1];
    const T md = (T)g.max_depth;
    if (!(s.d00 > (T)0 && s.d10 > (T)0 && s.d01 > (T)0 && s.d11 > (T)0 && s.d00 <= md && s.d10 <= md &&
          s.d01 <= md && s.d11 <= md))
        return;
    const T top = O::fma(s.a, O::sub(s.d10, s.d00), s.d00);
    const T bot = O::fma(s.a, O::sub(s.d11, s.d01), s.d01);
    const T d = O::fma(s.b, O::sub(bot, top), top);
    s.sdf = O::sub(d, s.cz);
    if (!(s.sdf >= -(T)g.trunc)) return;
    s.truncated = s.sdf > (T)g.trunc;
    s.tsdf = O::min_(s.sdf, (T)g.trunc);
    s.valid = true;
}

// Coefficient of the m-th (1-based) of n updates of a voxel whose weight was
// w0 before the first, weights clamped at M:  a_j = 1 / (min(w0 + j - 1, M) + 1),
// beta_m = a_m prod_{j=m+1..n} (1 - a_j).
template <typename T>
__device__ __forceinline__ T beta(int m, int n, T w0, T M) {
    using O = Ops<T>;
    // updates j < js see an unsaturated weight w0 + j - 1 < M
    const T jsf = M - w0 + (T)1;
    const int js = jsf < (T)1 ? 1 : (jsf > (T)(n + 1) ? n + 1 : (int)jsf);
    const T r = O::div(M, O::add(M, (T)1));
    const T am = m < js ? O::rcp(O::add(w0, (T)m)) : O::rcp(O::add(M, (T)1));
    // telescoping part over j in [m+1, min(n, js-1)]: (w0 + m) / (w0 + min(n, js-1))
    const int jt = min(n, js - 1);
    T p = (T)1;
    if (m + 1 <= jt) p = O::div(O::add(w0, (T)m), O::add(w0, (T)jt));
    const int lo = max(m + 1, js);
    if (n >= lo) p = O::mul(p, O::pow_(r, (T)(n - lo + 1)));
    return O::mul(am, p);
}

// prod_{j=1..n} (1 - a_j): how much of the starting distance survives n updates.
template <typename T>
__device__ __forceinline__ T carry(int n, T w0, T M) {
    using O = Ops<T>;
    if (n == 0) return (T)1;
    const T jsf = M - w0 + (T)1;
    const int js = jsf < (T)1 ? 1 : (jsf > (T)(n + 1) ? n + 1 : (int)jsf);
    const int jt = min(n, js - 1);
    T p = jt >= 1 ? O::div(w0, O::add(w0, (T)jt)) : (T)1;
    if (n >= js) p = O::mul(p, O::pow_(O::div(M, O::add(M, (T)1)), (T)(n - js + 1)));
    return p;
}

template <typename T>
__global__ void __launch_bounds__(256) forward_kernel(Geometry g, T* D, T* W, uint16_t* count, uint32_t* signature,
                                                      const T* depth, const T* rot, const T* trans) {
    __shared__ T s_pose[kBatchMaxFrames][12];
    using O = Ops<T>;
    for (int f = threadIdx.x; f < g.nframes; f += blockDim.x) {
        for (int k = 0; k < 9; ++k) s_pose[f][k] = rot[9 * f + k];
        for (int k = 0; k < 3; ++k) s_pose[f][9 + k] = trans[3 * f + k];
    }
    __syncthreads();
    const int64_t n = (int64_t)g.nx * g.ny * g.nz;
    const int64_t frame = (int64_t)g.width * g.height;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int x = (int)(i % g.nx);
        const int64_t r = i / g.nx;
        const int y = (int)(r % g.ny), z = (int)(r / g.ny);
        const T px = voxel_centre<T>(x, g.vs[0], g.off[0]);
        const T py = voxel_centre<T>(y, g.vs[1], g.off[1]);
        const T pz = voxel_centre<T>(z, g.vs[2], g.off[2]);
        T d = D[i], w = W[i];
        int cnt = 0;
        uint32_t sig = 2166136261u;
        for (int f = 0; f < g.nframes; ++f) {
            Sample<T> s;
            sample<T>(g, s_pose[f], s_pose[f] + 9, depth + f * frame, px, py, pz, s);
            if (signature) {
                const uint32_t code = s.valid ? (uint32_t)(s.u0 * 4099 + s.v0 * 7) ^ (s.truncated ? 0x80000000u : 0u)
                                              : 0x7fffffffu;
                sig = (sig ^ code) * 16777619u;
            }
            if (!s.valid) continue;
            const T inv = O::rcp(O::add(w, (T)1));
            d = O::fma(O::sub(s.tsdf, d), inv, d);
            w = O::min_(O::add(w, (T)1), (T)g.max_weight);
            ++cnt;
        }
        D[i] = d;
        W[i] = w;
        count[i] = (uint16_t)cnt;
        if (signature) signature[i] = sig;
    }
}

// grad_pose: [nframes][12] doubles (dL/dR row-major, dL/dt), accumulated.
// grad_depth: [nframes][H][W], accumulated.
template <typename T>
__global__ void __launch_bounds__(256) backward_kernel(Geometry g, const T* grad_D, const T* W0, const uint16_t* count,
                                                       const T* depth, const T* rot, const T* trans, T* grad_depth,
                                                       double* grad_pose, T* grad_D0) {
    __shared__ T s_pose[kBatchMaxFrames][12];
    __shared__ double s_acc[kBatchMaxFrames][12];
    using O = Ops<T>;
    for (int f = threadIdx.x; f < g.nframes; f += blockDim.x) {
        for (int k = 0; k < 9; ++k) s_pose[f][k] = rot[9 * f + k];
        for (int k = 0; k < 3; ++k) s_pose[f][9 + k] = trans[3 * f + k];
        for (int k = 0; k < 12; ++k) s_acc[f][k] = 0.0;
    }
    __syncthreads();
    const int64_t n = (int64_t)g.nx * g.ny * g.nz;
    const int64_t frame = (int64_t)g.width * g.height;
    const int lane = threadIdx.x & 31;
    // whole warps stay in the loop so the per-frame warp reductions see every lane
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    const int64_t start = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t warp_first = start - lane;
    for (int64_t i0 = warp_first; i0 < n; i0 += stride) {
        const int64_t i = i0 + lane;
        const bool inside = i < n;
        T gD = (T)0, w0 = (T)0;
        int nupd = 0;
        T px = 0, py = 0, pz = 0;
        if (inside) {
            gD = grad_D[i];
            w0 = W0[i];
            nupd = count[i];
            const int x = (int)(i % g.nx);
            const int64_t r = i / g.nx;
            const int y = (int)(r % g.ny), z = (int)(r / g.ny);
            px = voxel_centre<T>(x, g.vs[0], g.off[0]);
            py = voxel_centre<T>(y, g.vs[1], g.off[1]);
            pz = voxel_centre<T>(z, g.vs[2], g.off[2]);
        }
        w0 = w0 < (T)0 ? (T)0 : (w0 > (T)g.max_weight ? (T)g.max_weight : w0);
        if (grad_D0 && inside) grad_D0[i] = O::mul(gD, carry<T>(nupd, w0, (T)g.max_weight));
        const bool active = inside && gD != (T)0 && nupd > 0;
        if (!__any_sync(0xffffffffu, active)) continue;
        int m = 0;
        for (int f = 0; f < g.nframes; ++f) {
            const T* R = s_pose[f];
            T acc[12];
            bool any = false;
#pragma unroll
            for (int k = 0; k < 12; ++k) acc[k] = (T)0;
            if (active) {
                Sample<T> s;
                sample<T>(g, R, R + 9, depth + f * frame, px, py, pz, s);
                if (s.valid) {
                    ++m;
                    if (!s.truncated) {
                        const T gs = O::mul(gD, beta<T>(m, nupd, w0, (T)g.max_weight));   // dL/dsdf
                        // bilinear weights -> depth gradient
                        T* gd = grad_depth + f * frame + (int64_t)s.v0 * g.width + s.u0;
                        const T ia = O::sub((T)1, s.a), ib = O::sub((T)1, s.b);
                        atomicAdd(gd, O::mul(gs, O::mul(ia, ib)));
                        atomicAdd(gd + 1, O::mul(gs, O::mul(s.a, ib)));
                        atomicAdd(gd + g.width, O::mul(gs, O::mul(ia, s.b)));
                        atomicAdd(gd + g.width + 1, O::mul(gs, O::mul(s.a, s.b)));
                        // d sdf / d(u, v), then through the projection
                        const T top = O::fma(s.a, O::sub(s.d10, s.d00), s.d00);
                        const T bot = O::fma(s.a, O::sub(s.d11, s.d01), s.d01);
                        const T ddu = O::fma(s.b, O::sub(O::sub(s.d11, s.d01), O::sub(s.d10, s.d00)),
                                             O::sub(s.d10, s.d00));
                        const T ddv = O::sub(bot, top);
                        const T gu = O::mul(gs, O::mul(ddu, (T)g.fx));
                        const T gv = O::mul(gs, O::mul(ddv, (T)g.fy));
                        // u = fx cx/cz + .. -> du/dcx = fx/cz, du/dcz = -fx cx/cz^2
                        const T gcx = O::mul(gu, s.rz);
                        const T gcy = O::mul(gv, s.rz);
                        const T gcz = O::sub(O::mul((T)-1, gs),
                                             O::mul(s.rz, O::add(O::mul(gcx, s.cx), O::mul(gcy, s.cy))));
                        acc[0] = O::mul(gcx, px); acc[1] = O::mul(gcx, py); acc[2] = O::mul(gcx, pz);
                        acc[3] = O::mul(gcy, px); acc[4] = O::mul(gcy, py); acc[5] = O::mul(gcy, pz);
                        acc[6] = O::mul(gcz, px); acc[7] = O::mul(gcz, py); acc[8] = O::mul(gcz, pz);
                        acc[9] = gcx; acc[10] = gcy; acc[11] = gcz;
                        any = true;
                    }
                }
            }
            if (__any_sync(0xffffffffu, any)) {
#pragma unroll
                for (int k = 0; k < 12; ++k) {
                    double v = (double)acc[k];
                    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
                    if (lane == 0 && v != 0.0) atomicAdd(&s_acc[f][k], v);
                }
            }
        }
    }
    __syncthreads();
    for (int e = threadIdx.x; e < g.nframes * 12; e += blockDim.x) {
        const double v = s_acc[e / 12][e % 12];
        if (v != 0.0) atomicAdd(grad_pose + e, v);
    }
}

template <typename T> Geometry geometry(const DiffArgs& a) {
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

}  // namespace diff

cudaError_t launch_diff_forward(const DiffArgs& a, cudaStream_t s) {
    const int64_t n = (int64_t)a.nx * a.ny * a.nz;
    if (a.dtype == 1) {
        diff::forward_kernel<double><<<diff::grid_for(n), 256, 0, s>>>(
            diff::geometry<double>(a), (double*)a.D, (double*)a.W, a.count, a.signature, (const double*)a.depth,
            (const double*)a.rot, (const double*)a.trans);
    } else {
        diff::forward_kernel<float><<<diff::grid_for(n), 256, 0, s>>>(
            diff::geometry<float>(a), (float*)a.D, (float*)a.W, a.count, a.signature, (const float*)a.depth,
            (const float*)a.rot, (const float*)a.trans);
    }
    return cudaGetLastError();
}

cudaError_t launch_diff_backward(const DiffArgs& a, cudaStream_t s) {
    const int64_t n = (int64_t)a.nx * a.ny * a.nz;
    if (a.dtype == 1) {
        diff::backward_kernel<double><<<diff::grid_for(n), 256, 0, s>>>(
            diff::geometry<double>(a), (const double*)a.grad_D, (const double*)a.W, a.count, (const double*)a.depth,
            (const double*)a.rot, (const double*)a.trans, (double*)a.grad_depth, a.grad_pose, (double*)a.grad_D0);
    } else {
        diff::backward_kernel<float><<<diff::grid_for(n), 256, 0, s>>>(
            diff::geometry<float>(a), (const float*)a.grad_D, (const float*)a.W, a.count, (const float*)a.depth,
            (const float*)a.rot, (const float*)a.trans, (float*)a.grad_depth, a.grad_pose, (float*)a.grad_D0);
    }
    return cudaGetLastError();
}

}  // namespace gbt
