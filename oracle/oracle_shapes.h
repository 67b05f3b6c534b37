// TEST INFRASTRUCTURE ONLY (the oracle): FP64 restatement of sdfibm's shapes, SDF primitives and shape constants.
//   src/libshape/sdf/sdf.h:15-150 (primitives, rot30, flipy, offset, U, filter)
//   src/libshape/ishape.h:43-52   (world2local, phi01, phi)
//   src/libshape/{circle,sphere,ellipse,ellipsoid,rectangle,box,plane,circle_tail,circle_twotail}.h
// Every expression keeps the reference's evaluation order.
#pragma once
#include <algorithm>
#include <cmath>
#include <stdexcept>

#include "../include/sdfibm_cuda.h"
#include "oracle_math.h"

namespace oracle {

constexpr double SDF_TOL = 1e-8;  // sdf::TOL (sdf.h:9)
constexpr double SMALL = 1e-6;    // sdfibm::SMALL (types.h:19)

namespace sdf {
inline bool circle_bool_fast(const V3& p, double rSQR) { return magSqr(p) < rSQR; }
inline double circle(const V3& p, double r) { return mag(p) - r; }
inline bool rectangle_bool(const V3& p, double ra, double rb) { return std::fabs(p.x) < ra && std::fabs(p.y) < rb; }
inline double rectangle(const V3& p, double ra, double rb) {
    double dx = std::fabs(p.x) - ra;
    double dy = std::fabs(p.y) - rb;
    double dxp = std::max(0.0, dx);
    double dyp = std::max(0.0, dy);
    return std::sqrt(dxp * dxp + dyp * dyp) + std::min(0.0, std::max(dx, dy));
}
inline bool box_bool(const V3& p, double ra, double rb, double rc) {
    return std::fabs(p.x) < ra && std::fabs(p.y) < rb && std::fabs(p.z) < rc;
}
inline double box(const V3& p, double ra, double rb, double rc) {
    double dx = std::fabs(p.x) - ra;
    double dy = std::fabs(p.y) - rb;
    double dz = std::fabs(p.z) - rc;
    double dxp = std::max(0.0, dx);
    double dyp = std::max(0.0, dy);
    double dzp = std::max(0.0, dz);
    return std::sqrt(dxp * dxp + dyp * dyp + dzp * dzp) + std::min(0.0, std::max(dz, std::max(dx, dy)));
}
inline bool ellipse_bool_fast(const V3& p, double ia, double ib) { return p.x * p.x * ia + p.y * p.y * ib < 1.0; }
inline double ellipse(const V3& p, double ia, double ib) {
    double xa = p.x * p.x * ia;
    double yb = p.y * p.y * ib;
    return 0.5 * (xa + yb - 1.0) / (std::sqrt(xa * ia + yb * ib));
}
inline bool ellipsoid_bool_fast(const V3& p, double ia, double ib, double ic) {
    return p.x * p.x * ia + p.y * p.y * ib + p.z * p.z * ic < 1.0;
}
inline double ellipsoid(const V3& p, double ia, double ib, double ic) {
    double xa = p.x * p.x * ia;
    double yb = p.y * p.y * ib;
    double zc = p.z * p.z * ic;
    return 0.5 * (xa + yb + zc - 1.0) / (std::sqrt(xa * ia + yb * ib + zc * ic));
}
inline V3 rot30(const V3& p) { return V3{0.866025404 * p.x + 0.5 * p.y, 0.866025404 * p.y - 0.5 * p.x, 0.0}; }
inline V3 flipy(const V3& p) { return V3{p.x, -p.y, p.z}; }
inline V3 offset(const V3& p, const V3& o) { return p - o; }
inline double filter(double phi) { return (std::fabs(phi) < SDF_TOL) ? -SDF_TOL : phi; }
inline double min3(double a, double b, double c) { return std::min({a, b, c}); }
}  // namespace sdf

// IShape::world2local: conjugate(q).transform(p - t)
inline V3 world2local(const V3& p, const V3& t, const Quat& q) { return transform(conjugate(q), p - t); }

// Shape::isInside in the local frame
inline bool shapeInside(const sdfibm_shape_desc& s, const V3& p) {
    const double* a = s.p;
    const V3 com{s.com[0], s.com[1], s.com[2]};
    switch (s.type) {
        case SDFIBM_SHAPE_CIRCLE: return sdf::circle_bool_fast(com + V3{p.x, p.y, 0.0}, a[1]);
        case SDFIBM_SHAPE_SPHERE: return sdf::circle_bool_fast(com + p, a[1]);
        case SDFIBM_SHAPE_ELLIPSE: {
            V3 p2 = com + p; p2.z = 0.0;
            return sdf::ellipse_bool_fast(p2, a[2], a[3]);
        }
        case SDFIBM_SHAPE_ELLIPSOID: return sdf::ellipsoid_bool_fast(p, a[3], a[4], a[5]);
        case SDFIBM_SHAPE_RECTANGLE: {
            V3 p2 = com + p; p2.z = 0.0;
            return sdf::rectangle_bool(p2, a[0], a[1]);
        }
        case SDFIBM_SHAPE_BOX: return sdf::box_bool(com + p, a[0], a[1], a[2]);
        case SDFIBM_SHAPE_PLANE: return p.y < 0;
        case SDFIBM_SHAPE_CIRCLE_TAIL: {
            V3 p2 = com + p; p2.z = 0.0;
            bool b1 = sdf::rectangle_bool(sdf::offset(p2, V3{a[4], 0.0, 0.0}), a[4], a[2]);
            bool b2 = sdf::circle_bool_fast(V3{p2.x, p2.y, 0.0}, a[3]);
            return b1 || b2;
        }
        case SDFIBM_SHAPE_CIRCLE_TWOTAIL: {
            V3 p2 = com + p; p2.z = 0.0;
            bool dc = sdf::circle_bool_fast(p2, a[3]);
            bool d1 = sdf::rectangle_bool(sdf::offset(sdf::rot30(p2), V3{a[4], 0, 0}), a[4], a[2]);
            bool d2 = sdf::rectangle_bool(sdf::offset(sdf::rot30(sdf::flipy(p2)), V3{a[4], 0, 0}), a[4], a[2]);
            return dc || d1 || d2;
        }
    }
    throw std::invalid_argument("unknown shape type");
}

// Shape::signedDistance in the local frame
inline double shapeSDF(const sdfibm_shape_desc& s, const V3& p) {
    const double* a = s.p;
    const V3 com{s.com[0], s.com[1], s.com[2]};
    switch (s.type) {
        case SDFIBM_SHAPE_CIRCLE: return sdf::filter(sdf::circle(com + V3{p.x, p.y, 0.0}, a[0]));
        case SDFIBM_SHAPE_SPHERE: return sdf::filter(sdf::circle(com + p, a[0]));
        case SDFIBM_SHAPE_ELLIPSE: {
            V3 p2 = com + p; p2.z = 0.0;
            return sdf::filter(sdf::ellipse(p2, a[2], a[3]));
        }
        case SDFIBM_SHAPE_ELLIPSOID: return sdf::filter(sdf::ellipsoid(p, a[3], a[4], a[5]));
        case SDFIBM_SHAPE_RECTANGLE: {
            V3 p2 = com + p; p2.z = 0.0;
            return sdf::filter(sdf::rectangle(p2, a[0], a[1]));
        }
        case SDFIBM_SHAPE_BOX: return sdf::filter(sdf::box(com + p, a[0], a[1], a[2]));
        case SDFIBM_SHAPE_PLANE: return p.y;
        case SDFIBM_SHAPE_CIRCLE_TAIL: {
            V3 p2 = com + p; p2.z = 0.0;
            double d1 = sdf::circle(p2, a[0]);
            double d2 = sdf::rectangle(sdf::offset(p2, V3{a[4], 0.0, 0.0}), a[4], a[2]);
            return sdf::filter(std::min({d1, d2}));
        }
        case SDFIBM_SHAPE_CIRCLE_TWOTAIL: {
            V3 p2 = com + p; p2.z = 0.0;
            double dc = sdf::circle(p2, a[0]);
            double d1 = sdf::rectangle(sdf::offset(sdf::rot30(p2), V3{a[4], 0, 0}), a[4], a[2]);
            double d2 = sdf::rectangle(sdf::offset(sdf::rot30(sdf::flipy(p2)), V3{a[4], 0, 0}), a[4], a[2]);
            return sdf::filter(sdf::min3(dc, d1, d2));
        }
    }
    throw std::invalid_argument("unknown shape type");
}

// Shape constructors: derived parameters, volume, moment of inertia, bounding radius.
// raw[] holds the dictionary entries in the order of the sdfibm_shape_type comment (radius / radiusa.. / ratio,
// thickness); com is only read by the shapes whose constructor reads it.
inline sdfibm_shape_desc makeShape(int type, const double* raw, const double* com_in) {
    sdfibm_shape_desc s{};
    s.type = type;
    const double PI = M_PI;
    T33 moi{1, 0, 0, 0, 1, 0, 0, 0, 1};
    auto diag = [&](double a, double b, double c) { moi = T33{a, 0, 0, 0, b, 0, 0, 0, c}; };
    bool reads_com = true;
    switch (type) {
        case SDFIBM_SHAPE_CIRCLE: {  // circle.h:19-32
            double r = raw[0], r2 = r * r;
            s.p[0] = r; s.p[1] = r2;
            s.volume = PI * r2;
            double tmp = 0.5 * s.volume * r2; diag(tmp, tmp, tmp);
            s.radiusB = r;
            break;
        }
        case SDFIBM_SHAPE_SPHERE: {  // sphere.h:17-29
            double r = raw[0], r2 = r * r;
            s.p[0] = r; s.p[1] = r2;
            s.volume = 4.0 / 3.0 * PI * r2 * r;
            double tmp = 0.4 * s.volume * r2; diag(tmp, tmp, tmp);
            s.radiusB = r;
            break;
        }
        case SDFIBM_SHAPE_ELLIPSE: {  // ellipse.h:14-31
            double ra = raw[0], rb = raw[1];
            s.p[0] = ra; s.p[1] = rb; s.p[2] = 1.0 / (ra * ra); s.p[3] = 1.0 / (rb * rb);
            s.volume = PI * ra * rb;
            double tmp = 0.25 * s.volume * (ra * ra + rb * rb); diag(tmp, tmp, tmp);
            s.radiusB = std::max(ra, rb);
            break;
        }
        case SDFIBM_SHAPE_ELLIPSOID: {  // ellipsoid.h:17-32 (no com)
            double ra = raw[0], rb = raw[1], rc = raw[2];
            s.p[0] = ra; s.p[1] = rb; s.p[2] = rc;
            s.p[3] = 1.0 / (ra * ra); s.p[4] = 1.0 / (rb * rb); s.p[5] = 1.0 / (rc * rc);
            s.volume = 4.0 / 3.0 * PI * ra * rb * rc;
            diag(0.2 * s.volume * (rb * rb + rc * rc), 0.2 * s.volume * (ra * ra + rc * rc),
                 0.2 * s.volume * (ra * ra + rb * rb));
            s.radiusB = std::max(std::max(ra, rb), rc);
            reads_com = false;
            break;
        }
        case SDFIBM_SHAPE_RECTANGLE: {  // rectangle.h:16-32
            double ra = raw[0], rb = raw[1];
            s.p[0] = ra; s.p[1] = rb;
            double ra2 = ra * ra, rb2 = rb * rb;
            s.volume = 4.0 * ra * rb;
            double tmp = 1.0 / 3.0 * s.volume * (ra2 + rb2); diag(tmp, tmp, tmp);
            s.radiusB = std::max(ra, rb);
            break;
        }
        case SDFIBM_SHAPE_BOX: {  // box.h:16-32
            double ra = raw[0], rb = raw[1], rc = raw[2];
            s.p[0] = ra; s.p[1] = rb; s.p[2] = rc;
            s.volume = 8.0 * ra * rb * rc;
            diag(1.0 / 3.0 * s.volume * (rb * rb + rc * rc), 1.0 / 3.0 * s.volume * (ra * ra + rc * rc),
                 1.0 / 3.0 * s.volume * (rb * rb + ra * ra));
            s.radiusB = std::max(std::max(ra, rb), rc);
            break;
        }
        case SDFIBM_SHAPE_PLANE:  // plane.h:16: only finite = false; IShape defaults (volume 0, moi I)
            reads_com = false;
            break;
        case SDFIBM_SHAPE_CIRCLE_TAIL:      // circle_tail.h:20-36
        case SDFIBM_SHAPE_CIRCLE_TWOTAIL: {  // circle_twotail.h:20-36
            double r = raw[0], ratio = raw[1];
            double rb = (type == SDFIBM_SHAPE_CIRCLE_TAIL) ? raw[2] : raw[2] * 0.5;
            double r2 = r * r;
            double ra = (ratio + 1) * 0.5 * r;
            s.p[0] = r; s.p[1] = ratio; s.p[2] = rb; s.p[3] = r2; s.p[4] = ra;
            s.volume = PI * r2;
            double tmp = 0.5 * s.volume * r2; diag(tmp, tmp, tmp);
            s.radiusB = 2 * ra;
            break;
        }
        default: throw std::invalid_argument("unknown shape type");
    }
    s.volume_inv = (type == SDFIBM_SHAPE_PLANE) ? 0.0 : 1.0 / s.volume;
    T33 mi = (type == SDFIBM_SHAPE_PLANE) ? T33{1, 0, 0, 0, 1, 0, 0, 0, 1} : inv(moi);
    double* m = s.moi_inv;
    m[0] = mi.xx; m[1] = mi.xy; m[2] = mi.xz; m[3] = mi.yx; m[4] = mi.yy; m[5] = mi.yz;
    m[6] = mi.zx; m[7] = mi.zy; m[8] = mi.zz;
    if (reads_com && com_in) { s.com[0] = com_in[0]; s.com[1] = com_in[1]; s.com[2] = com_in[2]; }
    // collision.h:11-15 SHAPE2ID with std::map::operator[]: unknown names map to 0 (Plane)
    s.collision_id = (type == SDFIBM_SHAPE_CIRCLE) ? 1 : (type == SDFIBM_SHAPE_SPHERE) ? 2 : 0;
    return s;
}

}  // namespace oracle
