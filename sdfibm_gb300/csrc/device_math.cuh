// Device algebra and shapes for the coupling kernels.
//
// Two evaluation paths:
//  * *64 functions reproduce the reference's FP64 arithmetic operation for operation (OpenFOAM vector /
//    quaternion algebra, src/libshape/ishape.h:43-52, src/libshape/sdf/sdf.h, the shape headers).  The library is
//    compiled with -fmad=false, so no multiply-add is fused and every result matches a host FP64 evaluation bit
//    for bit.
//  * *32 functions evaluate the same inside test in FP32 together with a rigorous bound on their error and answer
//    inside / outside / undecided.  Undecided points (a band of about 1e-6 relative around the surface) are
//    re-evaluated with the *64 path, so classifications are always identical to the FP64 result while almost all
//    of the work runs at the FP32 rate (GB300: 68 TFLOP/s FP32 against 1.2 TFLOP/s FP64 measured).
#pragma once
#include <cstdint>

#include "../../include/sdfibm_cuda.h"

namespace sdfibm_dev {

struct D3 {
    double x, y, z;
};
__host__ __device__ inline D3 d3(double x, double y, double z) { return D3{x, y, z}; }
__host__ __device__ inline D3 operator+(const D3& a, const D3& b) { return D3{a.x + b.x, a.y + b.y, a.z + b.z}; }
__host__ __device__ inline D3 operator-(const D3& a, const D3& b) { return D3{a.x - b.x, a.y - b.y, a.z - b.z}; }
__host__ __device__ inline D3 operator-(const D3& a) { return D3{-a.x, -a.y, -a.z}; }
__host__ __device__ inline D3 operator*(double s, const D3& a) { return D3{s * a.x, s * a.y, s * a.z}; }
__host__ __device__ inline D3 operator*(const D3& a, double s) { return D3{a.x * s, a.y * s, a.z * s}; }
__host__ __device__ inline D3 operator/(const D3& a, double s) { return D3{a.x / s, a.y / s, a.z / s}; }
__host__ __device__ inline double dot(const D3& a, const D3& b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__host__ __device__ inline D3 cross(const D3& a, const D3& b) {
    return D3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
__host__ __device__ inline double magSqr(const D3& a) { return a.x * a.x + a.y * a.y + a.z * a.z; }
__host__ __device__ inline double mag(const D3& a) { return sqrt(magSqr(a)); }
__host__ __device__ inline double dmax(double a, double b) { return (a < b) ? b : a; }  // std::max semantics
__host__ __device__ inline double dmin(double a, double b) { return (b < a) ? b : a; }  // std::min semantics

struct Q4 {
    double w;
    D3 v;
};
__host__ __device__ inline Q4 qmul(const Q4& a, const Q4& b) {
    return Q4{a.w * b.w - dot(a.v, b.v), a.w * b.v + b.w * a.v + cross(a.v, b.v)};
}
__host__ __device__ inline Q4 qconj(const Q4& q) { return Q4{q.w, -q.v}; }
// quaternion::transform(u) = ((q * (0,u)) * conjugate(q)).v via mulq0v
__host__ __device__ inline D3 qtransform(const Q4& q, const D3& u) {
    Q4 m{-dot(q.v, u), q.w * u + cross(q.v, u)};
    return qmul(m, qconj(q)).v;
}
// IShape::world2local
__host__ __device__ inline D3 world2local(const D3& p, const D3& t, const Q4& q) { return qtransform(qconj(q), p - t); }

// |q|^2 R(q)^T in FP32: the linear map of world2local (quaternion::R of OpenFOAM, transposed), row-major
__host__ __device__ inline void local_matrix32(const Q4& q, float* M) {
    const double w2 = q.w * q.w, x2 = q.v.x * q.v.x, y2 = q.v.y * q.v.y, z2 = q.v.z * q.v.z;
    const double txy = 2 * q.v.x * q.v.y, twz = 2 * q.w * q.v.z, txz = 2 * q.v.x * q.v.z;
    const double twy = 2 * q.w * q.v.y, tyz = 2 * q.v.y * q.v.z, twx = 2 * q.w * q.v.x;
    const double R[9] = {w2 + x2 - y2 - z2, txy - twz, txz + twy, txy + twz, w2 - x2 + y2 - z2,
                         tyz - twx, txz - twy, tyz + twx, w2 - x2 - y2 + z2};
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) M[3 * r + c] = (float)R[3 * c + r];
}

// Per-solid shape record used by the kernels (lowered from sdfibm_solid_desc).
struct ShapeK {
    int32_t type;
    int32_t prism;      // 2-D shape: inside test ignores the local z coordinate
    double p[8];
    double com[3];
    double bound_r;     // radius of a sphere (or disc for prisms) around -com holding the inside region
    float p32[8];
    float com32[3];
    float p_lo[8];      // p - p32 and com - com32 rounded to FP32: the two-float form of the parameters
    float com_lo[3];
};

constexpr double SDF_TOL = 1e-8;  // sdf::TOL
constexpr double SMALL_D = 1e-6;  // sdfibm::SMALL
constexpr double ROT30_C = 0.866025404;

__device__ inline bool rect_bool64(const D3& p, double ra, double rb) { return fabs(p.x) < ra && fabs(p.y) < rb; }
__device__ inline double rect64(const D3& p, double ra, double rb) {
    double dx = fabs(p.x) - ra, dy = fabs(p.y) - rb;
    double dxp = dmax(0.0, dx), dyp = dmax(0.0, dy);
    return sqrt(dxp * dxp + dyp * dyp) + dmin(0.0, dmax(dx, dy));
}
__device__ inline D3 rot30_64(const D3& p) { return D3{ROT30_C * p.x + 0.5 * p.y, ROT30_C * p.y - 0.5 * p.x, 0.0}; }
__device__ inline double filter64(double phi) { return (fabs(phi) < SDF_TOL) ? -SDF_TOL : phi; }

// Shape::signedDistance (local frame) in FP32, for the learned fraction's features (which need only ~1e-6
// relative accuracy): the same formulas as sdf64 below, the reference's filter included.
__device__ inline float filter32(float phi) { return fabsf(phi) < 1e-8f ? -1e-8f : phi; }
__device__ inline float rect32(float x, float y, float ra, float rb) {
    const float dx = fabsf(x) - ra, dy = fabsf(y) - rb;
    const float dxp = fmaxf(0.f, dx), dyp = fmaxf(0.f, dy);
    return sqrtf(dxp * dxp + dyp * dyp) + fminf(0.f, fmaxf(dx, dy));
}
__device__ inline float sdf32(const ShapeK& s, float px, float py, float pz) {
    const float* a = s.p32;
    const float cx = px + s.com32[0], cy = py + s.com32[1], cz = pz + s.com32[2];
    switch (s.type) {
        case SDFIBM_SHAPE_CIRCLE: {
            const float z = s.com32[2];
            return filter32(sqrtf(cx * cx + cy * cy + z * z) - a[0]);
        }
        case SDFIBM_SHAPE_SPHERE: return filter32(sqrtf(cx * cx + cy * cy + cz * cz) - a[0]);
        case SDFIBM_SHAPE_ELLIPSE: {
            const float xa = cx * cx * a[2], yb = cy * cy * a[3];
            return filter32(0.5f * (xa + yb - 1.f) / sqrtf(xa * a[2] + yb * a[3]));
        }
        case SDFIBM_SHAPE_ELLIPSOID: {
            const float xa = px * px * a[3], yb = py * py * a[4], zc = pz * pz * a[5];
            return filter32(0.5f * (xa + yb + zc - 1.f) / sqrtf(xa * a[3] + yb * a[4] + zc * a[5]));
        }
        case SDFIBM_SHAPE_RECTANGLE: return filter32(rect32(cx, cy, a[0], a[1]));
        case SDFIBM_SHAPE_BOX: {
            const float dx = fabsf(cx) - a[0], dy = fabsf(cy) - a[1], dz = fabsf(cz) - a[2];
            const float dxp = fmaxf(0.f, dx), dyp = fmaxf(0.f, dy), dzp = fmaxf(0.f, dz);
            return filter32(sqrtf(dxp * dxp + dyp * dyp + dzp * dzp) + fminf(0.f, fmaxf(dz, fmaxf(dx, dy))));
        }
        case SDFIBM_SHAPE_PLANE: return py;
        case SDFIBM_SHAPE_CIRCLE_TAIL: {
            const float d1 = sqrtf(cx * cx + cy * cy) - a[0];
            return filter32(fminf(d1, rect32(cx - a[4], cy, a[4], a[2])));
        }
        case SDFIBM_SHAPE_CIRCLE_TWOTAIL: {
            const float c = (float)ROT30_C;
            const float dc = sqrtf(cx * cx + cy * cy) - a[0];
            const float d1 = rect32(c * cx + 0.5f * cy - a[4], c * cy - 0.5f * cx, a[4], a[2]);
            const float d2 = rect32(c * cx - 0.5f * cy - a[4], -c * cy - 0.5f * cx, a[4], a[2]);
            return filter32(fminf(dc, fminf(d1, d2)));
        }
    }
    return 0.f;
}

// Shape::isInside (local frame), FP64
__device__ inline bool inside64(const ShapeK& s, const D3& p) {
    const double* a = s.p;
    const D3 com{s.com[0], s.com[1], s.com[2]};
    switch (s.type) {
        case SDFIBM_SHAPE_CIRCLE: return magSqr(com + D3{p.x, p.y, 0.0}) < a[1];
        case SDFIBM_SHAPE_SPHERE: return magSqr(com + p) < a[1];
        case SDFIBM_SHAPE_ELLIPSE: {
            D3 q = com + p; q.z = 0.0;
            return q.x * q.x * a[2] + q.y * q.y * a[3] < 1.0;
        }
        case SDFIBM_SHAPE_ELLIPSOID: return p.x * p.x * a[3] + p.y * p.y * a[4] + p.z * p.z * a[5] < 1.0;
        case SDFIBM_SHAPE_RECTANGLE: {
            D3 q = com + p; q.z = 0.0;
            return rect_bool64(q, a[0], a[1]);
        }
        case SDFIBM_SHAPE_BOX: {
            D3 q = com + p;
            return fabs(q.x) < a[0] && fabs(q.y) < a[1] && fabs(q.z) < a[2];
        }
        case SDFIBM_SHAPE_PLANE: return p.y < 0;
        case SDFIBM_SHAPE_CIRCLE_TAIL: {
            D3 q = com + p; q.z = 0.0;
            bool b1 = rect_bool64(q - D3{a[4], 0.0, 0.0}, a[4], a[2]);
            bool b2 = magSqr(D3{q.x, q.y, 0.0}) < a[3];
            return b1 || b2;
        }
        case SDFIBM_SHAPE_CIRCLE_TWOTAIL: {
            D3 q = com + p; q.z = 0.0;
            bool dc = magSqr(q) < a[3];
            bool d1 = rect_bool64(rot30_64(q) - D3{a[4], 0, 0}, a[4], a[2]);
            bool d2 = rect_bool64(rot30_64(D3{q.x, -q.y, q.z}) - D3{a[4], 0, 0}, a[4], a[2]);
            return dc || d1 || d2;
        }
    }
    return false;
}

// Shape::signedDistance (local frame), FP64
__device__ inline double sdf64(const ShapeK& s, const D3& p) {
    const double* a = s.p;
    const D3 com{s.com[0], s.com[1], s.com[2]};
    switch (s.type) {
        case SDFIBM_SHAPE_CIRCLE: return filter64(mag(com + D3{p.x, p.y, 0.0}) - a[0]);
        case SDFIBM_SHAPE_SPHERE: return filter64(mag(com + p) - a[0]);
        case SDFIBM_SHAPE_ELLIPSE: {
            D3 q = com + p; q.z = 0.0;
            double xa = q.x * q.x * a[2], yb = q.y * q.y * a[3];
            return filter64(0.5 * (xa + yb - 1.0) / (sqrt(xa * a[2] + yb * a[3])));
        }
        case SDFIBM_SHAPE_ELLIPSOID: {
            double xa = p.x * p.x * a[3], yb = p.y * p.y * a[4], zc = p.z * p.z * a[5];
            return filter64(0.5 * (xa + yb + zc - 1.0) / (sqrt(xa * a[3] + yb * a[4] + zc * a[5])));
        }
        case SDFIBM_SHAPE_RECTANGLE: {
            D3 q = com + p; q.z = 0.0;
            return filter64(rect64(q, a[0], a[1]));
        }
        case SDFIBM_SHAPE_BOX: {
            D3 q = com + p;
            double dx = fabs(q.x) - a[0], dy = fabs(q.y) - a[1], dz = fabs(q.z) - a[2];
            double dxp = dmax(0.0, dx), dyp = dmax(0.0, dy), dzp = dmax(0.0, dz);
            return filter64(sqrt(dxp * dxp + dyp * dyp + dzp * dzp) + dmin(0.0, dmax(dz, dmax(dx, dy))));
        }
        case SDFIBM_SHAPE_PLANE: return p.y;
        case SDFIBM_SHAPE_CIRCLE_TAIL: {
            D3 q = com + p; q.z = 0.0;
            double d1 = mag(q) - a[0];
            double d2 = rect64(q - D3{a[4], 0.0, 0.0}, a[4], a[2]);
            return filter64(dmin(d1, d2));
        }
        case SDFIBM_SHAPE_CIRCLE_TWOTAIL: {
            D3 q = com + p; q.z = 0.0;
            double dc = mag(q) - a[0];
            double d1 = rect64(rot30_64(q) - D3{a[4], 0, 0}, a[4], a[2]);
            double d2 = rect64(rot30_64(D3{q.x, -q.y, q.z}) - D3{a[4], 0, 0}, a[4], a[2]);
            // std::min(initializer_list) returns the first smallest element
            double m = dc;
            if (d1 < m) m = d1;
            if (d2 < m) m = d2;
            return filter64(m);
        }
    }
    return 0.0;
}

// ---- FP32 classification with error bounds ------------------------------------------------------------------------
constexpr float U32 = 5.9604645e-8f;  // 2^-24, unit roundoff of FP32

// 1 inside, 0 outside, 2 undecided.  g < 0 means inside; Eg bounds |g32 - g| including the FP64 reference's own
// rounding (orders of magnitude smaller than the FP32 part).
__device__ inline int decide(float g, float Eg) { return g < -Eg ? 1 : (g > Eg ? 0 : 2); }
// AND of strict "m < 0" margins: inside only if every margin is negative
__device__ inline int decide_and2(float m1, float E1, float m2, float E2) {
    if (m1 > E1 || m2 > E2) return 0;
    if (m1 < -E1 && m2 < -E2) return 1;
    return 2;
}
__device__ inline int or_combine(int a, int b) { return (a == 1 || b == 1) ? 1 : ((a == 0 && b == 0) ? 0 : 2); }

__device__ inline int rect_bool32(float x, float y, float ra, float rb, float E) {
    float ax = fabsf(x), ay = fabsf(y);
    return decide_and2(ax - ra, E + 2.f * U32 * (ax + ra), ay - rb, E + 2.f * U32 * (ay + rb));
}

// p: local coordinates in FP32 with per-component absolute error at most E.
__device__ inline int inside32(const ShapeK& s, float px, float py, float pz, float E) {
    const float* a = s.p32;
    const float u = U32;
    switch (s.type) {
        case SDFIBM_SHAPE_CIRCLE: {
            float x = px + s.com32[0], y = py + s.com32[1], z = s.com32[2];
            float Ep = E + u * (fabsf(x) + fabsf(s.com32[0]) + fabsf(y) + fabsf(s.com32[1])) + u * fabsf(z);
            float q = x * x + y * y + z * z;
            float Eg = (2.f * (fabsf(x) + fabsf(y) + fabsf(z)) + 3.f * Ep) * Ep + 8.f * u * (q + a[1]);
            return decide(q - a[1], Eg);
        }
        case SDFIBM_SHAPE_SPHERE: {
            float x = px + s.com32[0], y = py + s.com32[1], z = pz + s.com32[2];
            float Ep = E + u * (fabsf(x) + fabsf(y) + fabsf(z) + fabsf(s.com32[0]) + fabsf(s.com32[1]) +
                                fabsf(s.com32[2]));
            float q = x * x + y * y + z * z;
            float Eg = (2.f * (fabsf(x) + fabsf(y) + fabsf(z)) + 3.f * Ep) * Ep + 8.f * u * (q + a[1]);
            return decide(q - a[1], Eg);
        }
        case SDFIBM_SHAPE_ELLIPSE: {
            float x = px + s.com32[0], y = py + s.com32[1];
            float Ep = E + u * (fabsf(x) + fabsf(y) + fabsf(s.com32[0]) + fabsf(s.com32[1]));
            float tx = x * x * a[2], ty = y * y * a[3];
            float Eg = (2.f * (fabsf(x) * a[2] + fabsf(y) * a[3]) + Ep * (a[2] + a[3])) * Ep + 10.f * u * (tx + ty + 1.f);
            return decide(tx + ty - 1.f, Eg);
        }
        case SDFIBM_SHAPE_ELLIPSOID: {
            float tx = px * px * a[3], ty = py * py * a[4], tz = pz * pz * a[5];
            float Eg = (2.f * (fabsf(px) * a[3] + fabsf(py) * a[4] + fabsf(pz) * a[5]) + E * (a[3] + a[4] + a[5])) * E +
                       10.f * u * (tx + ty + tz + 1.f);
            return decide(tx + ty + tz - 1.f, Eg);
        }
        case SDFIBM_SHAPE_RECTANGLE: {
            float x = px + s.com32[0], y = py + s.com32[1];
            float Ep = E + u * (fabsf(x) + fabsf(y) + fabsf(s.com32[0]) + fabsf(s.com32[1]));
            return rect_bool32(x, y, a[0], a[1], Ep);
        }
        case SDFIBM_SHAPE_BOX: {
            float x = px + s.com32[0], y = py + s.com32[1], z = pz + s.com32[2];
            float Ep = E + u * (fabsf(x) + fabsf(y) + fabsf(z) + fabsf(s.com32[0]) + fabsf(s.com32[1]) +
                                fabsf(s.com32[2]));
            float ax = fabsf(x), ay = fabsf(y), az = fabsf(z);
            float mx = ax - a[0], my = ay - a[1], mz = az - a[2];
            float Ex = Ep + 2.f * u * (ax + a[0]), Ey = Ep + 2.f * u * (ay + a[1]), Ez = Ep + 2.f * u * (az + a[2]);
            if (mx > Ex || my > Ey || mz > Ez) return 0;
            if (mx < -Ex && my < -Ey && mz < -Ez) return 1;
            return 2;
        }
        case SDFIBM_SHAPE_PLANE: return decide(py, E);
        case SDFIBM_SHAPE_CIRCLE_TAIL: {
            float x = px + s.com32[0], y = py + s.com32[1];
            float Ep = E + u * (fabsf(x) + fabsf(y) + fabsf(s.com32[0]) + fabsf(s.com32[1]));
            float xo = x - a[4];
            int b1 = rect_bool32(xo, y, a[4], a[2], Ep + u * (fabsf(x) + a[4]));
            float q = x * x + y * y;
            int b2 = decide(q - a[3], (2.f * (fabsf(x) + fabsf(y)) + 2.f * Ep) * Ep + 8.f * u * (q + a[3]));
            return or_combine(b1, b2);
        }
        case SDFIBM_SHAPE_CIRCLE_TWOTAIL: {
            float x = px + s.com32[0], y = py + s.com32[1];
            float Ep = E + u * (fabsf(x) + fabsf(y) + fabsf(s.com32[0]) + fabsf(s.com32[1]));
            float q = x * x + y * y;
            int dc = decide(q - a[3], (2.f * (fabsf(x) + fabsf(y)) + 2.f * Ep) * Ep + 8.f * u * (q + a[3]));
            const float c = 0.866025404f;
            float Er = 1.5f * Ep + 6.f * u * (fabsf(x) + fabsf(y));
            float r1x = c * x + 0.5f * y - a[4], r1y = c * y - 0.5f * x;
            float r2x = c * x - 0.5f * y - a[4], r2y = -c * y - 0.5f * x;
            int d1 = rect_bool32(r1x, r1y, a[4], a[2], Er + 2.f * u * (fabsf(r1x) + a[4]));
            int d2 = rect_bool32(r2x, r2y, a[4], a[2], Er + 2.f * u * (fabsf(r2x) + a[4]));
            return or_combine(dc, or_combine(d1, d2));
        }
    }
    return 2;
}

}  // namespace sdfibm_dev
