// TEST INFRASTRUCTURE ONLY (the oracle): plain FP64 restatement of the OpenFOAM vector / tensor / quaternion
// algebra that sdfibm's coupling path uses (src/types.h:4-17).  OpenFOAM is not vendored with the reference;
// the operation order below follows OpenFOAM's published VectorSpace / Tensor / quaternion definitions so that
// every result is reproducible bit for bit.  Build with -ffp-contract=off: no fused multiply-add anywhere.
#pragma once
#include <cmath>

namespace oracle {

struct V3 {
    double x, y, z;
};
inline V3 v3(double x, double y, double z) { return V3{x, y, z}; }
inline V3 operator+(const V3& a, const V3& b) { return V3{a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 operator-(const V3& a, const V3& b) { return V3{a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 operator-(const V3& a) { return V3{-a.x, -a.y, -a.z}; }
inline V3 operator*(double s, const V3& a) { return V3{s * a.x, s * a.y, s * a.z}; }
inline V3 operator*(const V3& a, double s) { return V3{a.x * s, a.y * s, a.z * s}; }
inline V3 operator/(const V3& a, double s) { return V3{a.x / s, a.y / s, a.z / s}; }
inline V3& operator+=(V3& a, const V3& b) { a = a + b; return a; }
inline V3& operator-=(V3& a, const V3& b) { a = a - b; return a; }
inline V3& operator*=(V3& a, double s) { a = a * s; return a; }
// Foam::operator& (inner product) and operator^ (cross product)
inline double dot(const V3& a, const V3& b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline V3 cross(const V3& a, const V3& b) {
    return V3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
inline double magSqr(const V3& a) { return a.x * a.x + a.y * a.y + a.z * a.z; }
inline double mag(const V3& a) { return std::sqrt(magSqr(a)); }
inline V3 cmptMultiply(const V3& a, const V3& b) { return V3{a.x * b.x, a.y * b.y, a.z * b.z}; }
// Foam::normalised: v/|v|, zero below rootVSmall
inline V3 normalised(const V3& v) {
    double s = mag(v);
    return s < 1e-150 ? V3{0, 0, 0} : v / s;
}

struct T33 {
    double xx, xy, xz, yx, yy, yz, zx, zy, zz;
};
inline T33 transpose(const T33& t) { return T33{t.xx, t.yx, t.zx, t.xy, t.yy, t.zy, t.xz, t.yz, t.zz}; }
inline T33 dotTT(const T33& a, const T33& b) {
    return T33{a.xx * b.xx + a.xy * b.yx + a.xz * b.zx, a.xx * b.xy + a.xy * b.yy + a.xz * b.zy,
               a.xx * b.xz + a.xy * b.yz + a.xz * b.zz, a.yx * b.xx + a.yy * b.yx + a.yz * b.zx,
               a.yx * b.xy + a.yy * b.yy + a.yz * b.zy, a.yx * b.xz + a.yy * b.yz + a.yz * b.zz,
               a.zx * b.xx + a.zy * b.yx + a.zz * b.zx, a.zx * b.xy + a.zy * b.yy + a.zz * b.zy,
               a.zx * b.xz + a.zy * b.yz + a.zz * b.zz};
}
inline V3 dotTV(const T33& t, const V3& v) {
    return V3{t.xx * v.x + t.xy * v.y + t.xz * v.z, t.yx * v.x + t.yy * v.y + t.yz * v.z,
              t.zx * v.x + t.zy * v.y + t.zz * v.z};
}
inline double det(const T33& t) {
    return t.xx * t.yy * t.zz + t.xy * t.yz * t.zx + t.xz * t.yx * t.zy - t.xx * t.yz * t.zy - t.xy * t.yx * t.zz -
           t.xz * t.yy * t.zx;
}
// Foam::inv(tensor) via the cofactor formula
inline T33 inv(const T33& t) {
    double d = det(t);
    return T33{(t.yy * t.zz - t.zy * t.yz) / d, (t.xz * t.zy - t.xy * t.zz) / d, (t.xy * t.yz - t.xz * t.yy) / d,
               (t.zx * t.yz - t.yx * t.zz) / d, (t.xx * t.zz - t.xz * t.zx) / d, (t.yx * t.xz - t.xx * t.yz) / d,
               (t.yx * t.zy - t.zx * t.yy) / d, (t.zx * t.xy - t.xx * t.zy) / d, (t.xx * t.yy - t.yx * t.xy) / d};
}
inline T33 scaleT(const T33& t, double s) {  // tensor / scalar, component-wise division
    return T33{t.xx / s, t.xy / s, t.xz / s, t.yx / s, t.yy / s, t.yz / s, t.zx / s, t.zy / s, t.zz / s};
}

struct Quat {
    double w;
    V3 v;
};
inline Quat operator*(const Quat& a, const Quat& b) {
    return Quat{a.w * b.w - dot(a.v, b.v), a.w * b.v + b.w * a.v + cross(a.v, b.v)};
}
inline Quat conjugate(const Quat& q) { return Quat{q.w, -q.v}; }
inline Quat operator*(double s, const Quat& q) { return Quat{s * q.w, s * q.v}; }
inline Quat operator*(const Quat& q, double s) { return Quat{q.w * s, q.v * s}; }
// quaternion::mulq0v and quaternion::transform: (q * (0,u)) * conjugate(q), vector part
inline Quat mulq0v(const Quat& q, const V3& u) { return Quat{-dot(q.v, u), q.w * u + cross(q.v, u)}; }
inline V3 transform(const Quat& q, const V3& u) { return (mulq0v(q, u) * conjugate(q)).v; }
// quaternion(d, theta): rotation about unit axis d
inline Quat axisAngle(const V3& d, double theta) { return Quat{std::cos(0.5 * theta), std::sin(0.5 * theta) * d}; }
// quaternion(quaternion::XYZ, angles) = qx * qy * qz
inline Quat fromEulerXYZ(const V3& a) {
    Quat q = axisAngle(V3{1, 0, 0}, a.x);
    q = q * axisAngle(V3{0, 1, 0}, a.y);
    q = q * axisAngle(V3{0, 0, 1}, a.z);
    return q;
}
inline double magQ(const Quat& q) { return std::sqrt(q.w * q.w + magSqr(q.v)); }
inline Quat normalise(const Quat& q) {
    double m = magQ(q);
    return Quat{q.w / m, q.v / m};
}
// quaternion::R()
inline T33 rotation(const Quat& q) {
    const double w2 = q.w * q.w, x2 = q.v.x * q.v.x, y2 = q.v.y * q.v.y, z2 = q.v.z * q.v.z;
    const double txy = 2 * q.v.x * q.v.y, twz = 2 * q.w * q.v.z, txz = 2 * q.v.x * q.v.z;
    const double twy = 2 * q.w * q.v.y, tyz = 2 * q.v.y * q.v.z, twx = 2 * q.w * q.v.x;
    return T33{w2 + x2 - y2 - z2, txy - twz, txz + twy, txy + twz, w2 - x2 + y2 - z2,
               tyz - twx, txz - twy, tyz + twx, w2 - x2 - y2 + z2};
}

}  // namespace oracle
