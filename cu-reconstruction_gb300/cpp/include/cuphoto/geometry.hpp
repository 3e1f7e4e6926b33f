// Small fixed-size vectors, quaternion and rigid transform of the TSDF host
// layer.  The reference uses Eigen and Sophus (modules/include/types.hpp);
// these stand-ins keep the members it calls: operator(), x()/y()/z(),
// rotationMatrix(), translation(), Quat from a rotation matrix.
#ifndef CUPHOTO_GB300_GEOMETRY_HPP
#define CUPHOTO_GB300_GEOMETRY_HPP

#include <cmath>

#include "types.cuh"

namespace cuphoto {

template <typename T, int N> struct VecN {
    T v[N];
    VecN() { for (int i = 0; i < N; ++i) v[i] = T(0); }
    template <typename... A> VecN(A... a) : v{static_cast<T>(a)...} { static_assert(sizeof...(A) == N, "size"); }
    T& operator()(int i) { return v[i]; }
    T operator()(int i) const { return v[i]; }
    T& operator[](int i) { return v[i]; }
    T operator[](int i) const { return v[i]; }
    T& x() { return v[0]; }
    T& y() { return v[1]; }
    T& z() { return v[2]; }
    T x() const { return v[0]; }
    T y() const { return v[1]; }
    T z() const { return v[2]; }
};

using Vec3 = VecN<r64, 3>;
using Vec3f = VecN<r32, 3>;
using Vec3i = VecN<i32, 3>;
using Vec4f = VecN<r32, 4>;
using Vec6f = VecN<r32, 6>;
using Vec10f = VecN<r32, 10>;

struct Mat3 {
    r64 m[3][3];
    r64 operator()(int r, int c) const { return m[r][c]; }
    r64& operator()(int r, int c) { return m[r][c]; }
};

struct Quat {
    r64 qw = 1, qx = 0, qy = 0, qz = 0;
    Quat() = default;
    Quat(r64 w_, r64 x_, r64 y_, r64 z_) : qw(w_), qx(x_), qy(y_), qz(z_) {}
    // Rotation matrix -> unit quaternion (Shepperd's method).
    explicit Quat(const Mat3& R) {
        const r64 t = R(0, 0) + R(1, 1) + R(2, 2);
        if (t > 0) {
            r64 s = std::sqrt(t + 1.0) * 2;
            qw = 0.25 * s; qx = (R(2, 1) - R(1, 2)) / s; qy = (R(0, 2) - R(2, 0)) / s; qz = (R(1, 0) - R(0, 1)) / s;
        } else if (R(0, 0) > R(1, 1) && R(0, 0) > R(2, 2)) {
            r64 s = std::sqrt(1.0 + R(0, 0) - R(1, 1) - R(2, 2)) * 2;
            qw = (R(2, 1) - R(1, 2)) / s; qx = 0.25 * s; qy = (R(0, 1) + R(1, 0)) / s; qz = (R(0, 2) + R(2, 0)) / s;
        } else if (R(1, 1) > R(2, 2)) {
            r64 s = std::sqrt(1.0 + R(1, 1) - R(0, 0) - R(2, 2)) * 2;
            qw = (R(0, 2) - R(2, 0)) / s; qx = (R(0, 1) + R(1, 0)) / s; qy = 0.25 * s; qz = (R(1, 2) + R(2, 1)) / s;
        } else {
            r64 s = std::sqrt(1.0 + R(2, 2) - R(0, 0) - R(1, 1)) * 2;
            qw = (R(1, 0) - R(0, 1)) / s; qx = (R(0, 2) + R(2, 0)) / s; qy = (R(1, 2) + R(2, 1)) / s; qz = 0.25 * s;
        }
        normalize();
    }
    // Rotation of `angle` radians about a unit axis (Eigen::AngleAxisd).
    static Quat angle_axis(r64 angle, r64 ax, r64 ay, r64 az) {
        const r64 s = std::sin(angle / 2);
        return Quat(std::cos(angle / 2), ax * s, ay * s, az * s);
    }
    void normalize() {
        const r64 n = std::sqrt(qw * qw + qx * qx + qy * qy + qz * qz);
        qw /= n; qx /= n; qy /= n; qz /= n;
    }
    r64 w() const { return qw; }
    r64 x() const { return qx; }
    r64 y() const { return qy; }
    r64 z() const { return qz; }
    Mat3 matrix() const {
        Mat3 R;
        R(0, 0) = 1 - 2 * (qy * qy + qz * qz); R(0, 1) = 2 * (qx * qy - qz * qw); R(0, 2) = 2 * (qx * qz + qy * qw);
        R(1, 0) = 2 * (qx * qy + qz * qw); R(1, 1) = 1 - 2 * (qx * qx + qz * qz); R(1, 2) = 2 * (qy * qz - qx * qw);
        R(2, 0) = 2 * (qx * qz - qy * qw); R(2, 1) = 2 * (qy * qz + qx * qw); R(2, 2) = 1 - 2 * (qx * qx + qy * qy);
        return R;
    }
};

inline Quat operator*(const Quat& a, const Quat& b) {
    return Quat(a.qw * b.qw - a.qx * b.qx - a.qy * b.qy - a.qz * b.qz,
                a.qw * b.qx + a.qx * b.qw + a.qy * b.qz - a.qz * b.qy,
                a.qw * b.qy - a.qx * b.qz + a.qy * b.qw + a.qz * b.qx,
                a.qw * b.qz + a.qx * b.qy - a.qy * b.qx + a.qz * b.qw);
}

// Rigid transform (Sophus::SE3d): unit quaternion + translation.
class SE3 {
public:
    SE3() = default;
    SE3(const Quat& q, const Vec3& t) : q_(q), t_(t) { q_.normalize(); }
    Mat3 rotationMatrix() const { return q_.matrix(); }
    Vec3 translation() const { return t_; }
    Quat unit_quaternion() const { return q_; }
    // The inverse transform (Sophus::SE3d::inverse): R^T, -R^T t.
    SE3 inverse() const {
        const Quat qi(q_.qw, -q_.qx, -q_.qy, -q_.qz);
        const Mat3 Ri = qi.matrix();
        Vec3 ti;
        for (int r = 0; r < 3; ++r) ti(r) = -(Ri(r, 0) * t_(0) + Ri(r, 1) * t_(1) + Ri(r, 2) * t_(2));
        return SE3(qi, ti);
    }

private:
    Quat q_;
    Vec3 t_;
};

}  // namespace cuphoto

#endif
