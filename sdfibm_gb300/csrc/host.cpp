// Host-side lowering of shapes / motions / forcers / materials into the C ABI descriptors (include/sdfibm_host.h;
// the dictionary front ends are in host_dict.cpp, the file formats in host_io.cpp).  Arithmetic of the constructors
// follows the reference exactly, so the descriptors carry the same bits as the reference's objects:
//   shapes     src/libshape/{circle,sphere,ellipse,ellipsoid,rectangle,box,plane,circle_tail,circle_twotail}.h
//   motions    src/libmotion/motion*.h constructors
//   forcers    src/libforcer/{constant,spring,magnetic}.h constructors
//   material   src/libmaterial/imaterial.h, Solid::setMaterial src/solid.h:95-103
//   euler      Solid::setOrientation src/solid.h:76-80 with OpenFOAM quaternion(XYZ, angles)
#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/sdfibm_host.h"

namespace {

struct T3 {
    double m[9];
};
T3 inv3(const T3& t) {  // Foam::inv(tensor), cofactor formula
    const double xx = t.m[0], xy = t.m[1], xz = t.m[2], yx = t.m[3], yy = t.m[4], yz = t.m[5], zx = t.m[6],
                 zy = t.m[7], zz = t.m[8];
    const double d = xx * yy * zz + xy * yz * zx + xz * yx * zy - xx * yz * zy - xy * yx * zz - xz * yy * zx;
    return T3{{(yy * zz - zy * yz) / d, (xz * zy - xy * zz) / d, (xy * yz - xz * yy) / d, (zx * yz - yx * zz) / d,
               (xx * zz - xz * zx) / d, (yx * xz - xx * yz) / d, (yx * zy - zx * yy) / d, (zx * xy - xx * zy) / d,
               (xx * yy - yx * xy) / d}};
}
T3 diag(double a, double b, double c) { return T3{{a, 0, 0, 0, b, 0, 0, 0, c}}; }

struct Qh {
    double w, x, y, z;
};
Qh qmul(const Qh& a, const Qh& b) {
    // (a.w*b.w - a.v.b.v, a.w*b.v + b.w*a.v + a.v^b.v)
    const double dotv = a.x * b.x + a.y * b.y + a.z * b.z;
    const double cx = a.y * b.z - a.z * b.y, cy = a.z * b.x - a.x * b.z, cz = a.x * b.y - a.y * b.x;
    return Qh{a.w * b.w - dotv, a.w * b.x + b.w * a.x + cx, a.w * b.y + b.w * a.y + cy, a.w * b.z + b.w * a.z + cz};
}
Qh axis_angle(double dx, double dy, double dz, double th) {
    const double c = std::cos(0.5 * th), s = std::sin(0.5 * th);
    return Qh{c, s * dx, s * dy, s * dz};
}

}  // namespace

extern "C" {

void sdfibm_options_default(sdfibm_options* o) {
    if (!o) return;
    std::memset(o, 0, sizeof(*o));
    o->rho_f = 1.0;
    o->collision_mode = SDFIBM_COLLISION_OFF;
    o->fraction_method = SDFIBM_FRACTION_REFGEO;
    o->subsample_n = 10;
    o->exact_forcing = 1;
}

int sdfibm_host_make_shape(int32_t type, const double* raw, const double* com_in, sdfibm_shape_desc* out) {
    if (!out || (!raw && type != SDFIBM_SHAPE_PLANE)) return SDFIBM_ERR_ARG;
    sdfibm_shape_desc s;
    std::memset(&s, 0, sizeof(s));
    s.type = type;
    const double PI = M_PI;
    T3 moi = diag(1, 1, 1);
    bool reads_com = true;
    switch (type) {
        case SDFIBM_SHAPE_CIRCLE: {
            const double r = raw[0], r2 = r * r;
            if (!(r > 0)) return SDFIBM_ERR_ARG;
            s.p[0] = r; s.p[1] = r2;
            s.volume = PI * r2;
            const double tmp = 0.5 * s.volume * r2;
            moi = diag(tmp, tmp, tmp);
            s.radiusB = r;
            break;
        }
        case SDFIBM_SHAPE_SPHERE: {
            const double r = raw[0], r2 = r * r;
            if (!(r > 0)) return SDFIBM_ERR_ARG;
            s.p[0] = r; s.p[1] = r2;
            s.volume = 4.0 / 3.0 * PI * r2 * r;
            const double tmp = 0.4 * s.volume * r2;
            moi = diag(tmp, tmp, tmp);
            s.radiusB = r;
            break;
        }
        case SDFIBM_SHAPE_ELLIPSE: {
            const double ra = raw[0], rb = raw[1];
            if (!(ra > 0 && rb > 0)) return SDFIBM_ERR_ARG;
            s.p[0] = ra; s.p[1] = rb; s.p[2] = 1.0 / (ra * ra); s.p[3] = 1.0 / (rb * rb);
            s.volume = PI * ra * rb;
            const double tmp = 0.25 * s.volume * (ra * ra + rb * rb);
            moi = diag(tmp, tmp, tmp);
            s.radiusB = std::max(ra, rb);
            break;
        }
        case SDFIBM_SHAPE_ELLIPSOID: {
            const double ra = raw[0], rb = raw[1], rc = raw[2];
            if (!(ra > 0 && rb > 0 && rc > 0)) return SDFIBM_ERR_ARG;
            s.p[0] = ra; s.p[1] = rb; s.p[2] = rc;
            s.p[3] = 1.0 / (ra * ra); s.p[4] = 1.0 / (rb * rb); s.p[5] = 1.0 / (rc * rc);
            s.volume = 4.0 / 3.0 * PI * ra * rb * rc;
            moi = diag(0.2 * s.volume * (rb * rb + rc * rc), 0.2 * s.volume * (ra * ra + rc * rc),
                       0.2 * s.volume * (ra * ra + rb * rb));
            s.radiusB = std::max(std::max(ra, rb), rc);
            reads_com = false;  // the Ellipsoid constructor never reads com
            break;
        }
        case SDFIBM_SHAPE_RECTANGLE: {
            const double ra = raw[0], rb = raw[1];
            if (!(ra > 0 && rb > 0)) return SDFIBM_ERR_ARG;
            s.p[0] = ra; s.p[1] = rb;
            s.volume = 4.0 * ra * rb;
            const double tmp = 1.0 / 3.0 * s.volume * (ra * ra + rb * rb);
            moi = diag(tmp, tmp, tmp);
            s.radiusB = std::max(ra, rb);
            break;
        }
        case SDFIBM_SHAPE_BOX: {
            const double ra = raw[0], rb = raw[1], rc = raw[2];
            if (!(ra > 0 && rb > 0 && rc > 0)) return SDFIBM_ERR_ARG;
            s.p[0] = ra; s.p[1] = rb; s.p[2] = rc;
            s.volume = 8.0 * ra * rb * rc;
            moi = diag(1.0 / 3.0 * s.volume * (rb * rb + rc * rc), 1.0 / 3.0 * s.volume * (ra * ra + rc * rc),
                       1.0 / 3.0 * s.volume * (rb * rb + ra * ra));
            s.radiusB = std::max(std::max(ra, rb), rc);
            break;
        }
        case SDFIBM_SHAPE_PLANE:
            reads_com = false;  // IShape defaults: zero volume, identity moment of inertia, infinite
            break;
        case SDFIBM_SHAPE_CIRCLE_TAIL:
        case SDFIBM_SHAPE_CIRCLE_TWOTAIL: {
            const double r = raw[0], ratio = raw[1];
            const double rb = (type == SDFIBM_SHAPE_CIRCLE_TAIL) ? raw[2] : raw[2] * 0.5;
            if (!(r > 0)) return SDFIBM_ERR_ARG;
            const double r2 = r * r, ra = (ratio + 1) * 0.5 * r;
            s.p[0] = r; s.p[1] = ratio; s.p[2] = rb; s.p[3] = r2; s.p[4] = ra;
            s.volume = PI * r2;
            const double tmp = 0.5 * s.volume * r2;
            moi = diag(tmp, tmp, tmp);
            s.radiusB = 2 * ra;
            break;
        }
        default: return SDFIBM_ERR_ARG;
    }
    s.volume_inv = (type == SDFIBM_SHAPE_PLANE) ? 0.0 : 1.0 / s.volume;
    const T3 mi = (type == SDFIBM_SHAPE_PLANE) ? diag(1, 1, 1) : inv3(moi);
    std::memcpy(s.moi_inv, mi.m, sizeof(mi.m));
    if (reads_com && com_in)
        for (int a = 0; a < 3; ++a) s.com[a] = com_in[a];
    s.collision_id = (type == SDFIBM_SHAPE_CIRCLE) ? 1 : (type == SDFIBM_SHAPE_SPHERE) ? 2 : 0;
    *out = s;
    return SDFIBM_OK;
}

int sdfibm_host_make_motion(int32_t type, const double* raw, double* p) {
    if (!p) return SDFIBM_ERR_ARG;
    for (int i = 0; i < 8; ++i) p[i] = 0;
    switch (type) {
        case SDFIBM_MOTION_FREE:
        case SDFIBM_MOTION_OPENCLOSE: return SDFIBM_OK;
        case SDFIBM_MOTION_000002:
        case SDFIBM_MOTION_110002: p[0] = raw[0]; p[1] = 2 * M_PI / raw[0]; return SDFIBM_OK;
        case SDFIBM_MOTION_222000: p[0] = raw[0]; p[1] = raw[1]; p[2] = raw[2]; return SDFIBM_OK;
        case SDFIBM_MOTION_SINEDIRECTIONAL:
            p[0] = raw[0]; p[1] = raw[1]; p[2] = 2 * M_PI / raw[1];
            p[3] = raw[2]; p[4] = raw[3]; p[5] = raw[4];
            return SDFIBM_OK;
        case SDFIBM_MOTION_01MASK:
            for (int i = 0; i < 6; ++i) {
                if (raw[i] != 0.0 && raw[i] != 1.0) return SDFIBM_ERR_ARG;
                p[i] = raw[i];
            }
            return SDFIBM_OK;
        case SDFIBM_MOTION_ROTOR:
            p[0] = raw[0]; p[1] = 2 * M_PI / raw[0]; p[2] = raw[1]; p[3] = raw[2]; p[4] = raw[3];
            return SDFIBM_OK;
        default: return SDFIBM_ERR_ARG;
    }
}

int sdfibm_host_make_forcer(int32_t type, const double* raw, double* p) {
    if (!p) return SDFIBM_ERR_ARG;
    for (int i = 0; i < 8; ++i) p[i] = 0;
    switch (type) {
        case SDFIBM_FORCER_NONE: return SDFIBM_OK;
        case SDFIBM_FORCER_CONSTANT: for (int i = 0; i < 6; ++i) p[i] = raw[i]; return SDFIBM_OK;
        case SDFIBM_FORCER_SPRING:
        case SDFIBM_FORCER_MAGNETIC: for (int i = 0; i < 5; ++i) p[i] = raw[i]; return SDFIBM_OK;
        default: return SDFIBM_ERR_ARG;
    }
}

void sdfibm_host_quat_from_euler_deg(const double* e, double* q) {
    const double ax = e[0] * M_PI / 180.0, ay = e[1] * M_PI / 180.0, az = e[2] * M_PI / 180.0;
    Qh r = axis_angle(1, 0, 0, ax);
    r = qmul(r, axis_angle(0, 1, 0, ay));
    r = qmul(r, axis_angle(0, 0, 1, az));
    q[0] = r.w; q[1] = r.x; q[2] = r.y; q[3] = r.z;
}

int sdfibm_host_make_solid(int32_t id, const sdfibm_shape_desc* shape, double rho, int32_t motion_type,
                           const double* motion_p8, int32_t forcer_type, const double* forcer_p8, const double* pos,
                           const double* euler_deg, const double* vel, const double* omega, sdfibm_solid_desc* out) {
    if (!shape || !out || !pos) return SDFIBM_ERR_ARG;
    if (!(rho > 0)) return SDFIBM_ERR_ARG;
    sdfibm_solid_desc d;
    std::memset(&d, 0, sizeof(d));
    d.id = id;
    d.shape = *shape;
    d.motion_type = motion_type;
    d.forcer_type = forcer_type;
    if (motion_p8) std::memcpy(d.motion_p, motion_p8, sizeof(d.motion_p));
    if (forcer_p8) std::memcpy(d.forcer_p, forcer_p8, sizeof(d.forcer_p));
    d.rho = rho;
    d.mass = shape->volume * rho;
    d.mass_inv = shape->volume_inv / rho;
    for (int i = 0; i < 9; ++i) d.moi_inv[i] = shape->moi_inv[i] / rho;
    for (int a = 0; a < 3; ++a) {
        d.pos[a] = pos[a];
        d.vel[a] = vel ? vel[a] : 0.0;
        d.omega[a] = omega ? omega[a] : 0.0;
    }
    const double zero[3] = {0, 0, 0};
    sdfibm_host_quat_from_euler_deg(euler_deg ? euler_deg : zero, d.quat);
    *out = d;
    return SDFIBM_OK;
}

}  // extern "C"
