// Host-side lowering of shapes / motions / forcers / materials into the C ABI descriptors, and the solidDict front
// end (include/sdfibm_host.h).  Arithmetic of the constructors follows the reference exactly, so the descriptors
// carry the same bits as the reference's objects:
//   shapes     src/libshape/{circle,sphere,ellipse,ellipsoid,rectangle,box,plane,circle_tail,circle_twotail}.h
//   motions    src/libmotion/motion*.h constructors
//   forcers    src/libforcer/{constant,spring,magnetic}.h constructors
//   material   src/libmaterial/imaterial.h, Solid::setMaterial src/solid.h:95-103
//   euler      Solid::setOrientation src/solid.h:76-80 with OpenFOAM quaternion(XYZ, angles)
//   dictionary SolidCloud::initFromDictionary src/solidcloud.cpp:14-206
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

// ---- solidDict front end ----------------------------------------------------------------------------------------------
namespace {

struct Node {
    // either a dictionary (ordered entries) or a token list value
    bool is_dict = false;
    std::vector<std::pair<std::string, std::shared_ptr<Node>>> entries;
    std::vector<std::string> tokens;
    std::vector<char> quoted;  // per token: read as a "string"

    const Node* find(const std::string& k) const {
        for (auto& e : entries)
            if (e.first == k) return e.second.get();
        return nullptr;
    }
    const Node& sub(const std::string& k) const {
        const Node* n = find(k);
        if (!n || !n->is_dict) throw std::runtime_error("missing sub-dictionary " + k);
        return *n;
    }
};

struct Lexer {
    const std::string& s;
    size_t i = 0;
    bool quoted = false;  // the last token was a "string"
    explicit Lexer(const std::string& t) : s(t) {}
    void skip() {
        for (;;) {
            while (i < s.size() && std::isspace((unsigned char)s[i])) ++i;
            if (i + 1 < s.size() && s[i] == '/' && s[i + 1] == '/') {
                while (i < s.size() && s[i] != '\n') ++i;
            } else if (i + 1 < s.size() && s[i] == '/' && s[i + 1] == '*') {
                size_t e = s.find("*/", i + 2);
                i = (e == std::string::npos) ? s.size() : e + 2;
            } else {
                return;
            }
        }
    }
    bool next(std::string& tok) {
        skip();
        if (i >= s.size()) return false;
        const char c = s[i];
        quoted = c == '"';
        if (c == '{' || c == '}' || c == '(' || c == ')' || c == ';' || c == '[' || c == ']') {
            tok = std::string(1, c);
            ++i;
            return true;
        }
        if (c == '"') {
            size_t e = s.find('"', i + 1);
            if (e == std::string::npos) throw std::runtime_error("unterminated string");
            tok = s.substr(i + 1, e - i - 1);
            i = e + 1;
            return true;
        }
        // a word runs to the next blank or punctuation; a NUL byte (binary data) is a word character, since
        // strchr would match it against the terminator of the punctuation string
        size_t b = i;
        while (i < s.size() && !std::isspace((unsigned char)s[i]) &&
               (s[i] == '\0' || std::strchr("{}();[]", s[i]) == nullptr))
            ++i;
        tok = s.substr(b, i - b);
        return true;
    }
};

std::shared_ptr<Node> parse_dict(Lexer& lx, bool top) {
    auto n = std::make_shared<Node>();
    n->is_dict = true;
    std::string tok;
    while (lx.next(tok)) {
        if (tok == "}") {
            if (top) throw std::runtime_error("unbalanced }");
            return n;
        }
        if (tok == ";") continue;
        const std::string key = tok;
        if (!lx.next(tok)) throw std::runtime_error("unexpected end after " + key);
        if (tok == "{") {
            n->entries.emplace_back(key, parse_dict(lx, false));
            continue;
        }
        auto v = std::make_shared<Node>();
        int depth = 0;
        for (;;) {
            if (tok == "(" || tok == "[") ++depth;
            if (tok == ")" || tok == "]") --depth;
            if (tok == ";" && depth == 0) break;
            if (tok == "{" || tok == "}") throw std::runtime_error("unexpected brace in value of " + key);
            v->tokens.push_back(tok);
            v->quoted.push_back(lx.quoted);
            if (!lx.next(tok)) throw std::runtime_error("unexpected end in value of " + key);
        }
        n->entries.emplace_back(key, v);
    }
    if (!top) throw std::runtime_error("missing }");
    return n;
}

double to_num(const std::string& t) {
    size_t p = 0;
    double v = std::stod(t, &p);
    if (p != t.size()) throw std::runtime_error("not a number: " + t);
    return v;
}
double scalar_of(const Node& d, const std::string& k) {
    const Node* n = d.find(k);
    if (!n || n->is_dict || n->tokens.empty()) throw std::runtime_error("missing scalar " + k);
    return to_num(n->tokens.back());  // a dimensioned entry keeps its value last
}
bool vector_of(const Node& d, const std::string& k, double out[3]) {
    const Node* n = d.find(k);
    if (!n) return false;
    std::vector<double> v;
    for (auto& t : n->tokens)
        if (t != "(" && t != ")") v.push_back(to_num(t));
    if (v.size() != 3) throw std::runtime_error("bad vector " + k);
    for (int a = 0; a < 3; ++a) out[a] = v[a];
    return true;
}
std::string word_of(const Node& d, const std::string& k) {
    const Node* n = d.find(k);
    if (!n || n->is_dict || n->tokens.size() != 1) throw std::runtime_error("missing word " + k);
    return n->tokens[0];
}
bool bool_of(const Node& d, const std::string& k) {
    const std::string w = word_of(d, k);
    if (w == "1" || w == "true" || w == "yes" || w == "on" || w == "y" || w == "t") return true;
    if (w == "0" || w == "false" || w == "no" || w == "off" || w == "n" || w == "f" || w == "none") return false;
    throw std::runtime_error("bad bool " + k);
}

// The shapes library of a solidDict: one ShapeFactory::create per entry of "shapes".  keep_first: the coupling's
// EntityLibrary::emplace keeps the first of duplicate names (src/solidcloud.cpp:66, src/entitylibrary.h:22); the
// VOF initializer assigns, keeping the last (tool_vof/solidcloud.cpp:57-60).
std::map<std::string, sdfibm_shape_desc> parse_shapes(const Node& shapes_dict, bool keep_first) {
    static const std::map<std::string, int> shape_ids = {
        {"Circle", SDFIBM_SHAPE_CIRCLE}, {"Sphere", SDFIBM_SHAPE_SPHERE}, {"Ellipse", SDFIBM_SHAPE_ELLIPSE},
        {"Ellipsoid", SDFIBM_SHAPE_ELLIPSOID}, {"Rectangle", SDFIBM_SHAPE_RECTANGLE}, {"Box", SDFIBM_SHAPE_BOX},
        {"Plane", SDFIBM_SHAPE_PLANE}, {"Circle_Tail", SDFIBM_SHAPE_CIRCLE_TAIL},
        {"Circle_TwoTail", SDFIBM_SHAPE_CIRCLE_TWOTAIL}};
    std::map<std::string, sdfibm_shape_desc> shapes;
    for (auto& e : shapes_dict.entries) {
        const Node& sd = *e.second;
        const std::string type = word_of(sd, "type"), name = word_of(sd, "name");
        auto it = shape_ids.find(type);
        if (it == shape_ids.end()) throw std::runtime_error("Cannot create unrecognized object: " + type);
        double raw[8] = {0}, com[3] = {0, 0, 0};
        switch (it->second) {
            case SDFIBM_SHAPE_CIRCLE: case SDFIBM_SHAPE_SPHERE: raw[0] = scalar_of(sd, "radius"); break;
            case SDFIBM_SHAPE_ELLIPSE: case SDFIBM_SHAPE_RECTANGLE:
                raw[0] = scalar_of(sd, "radiusa"); raw[1] = scalar_of(sd, "radiusb"); break;
            case SDFIBM_SHAPE_ELLIPSOID: case SDFIBM_SHAPE_BOX:
                raw[0] = scalar_of(sd, "radiusa"); raw[1] = scalar_of(sd, "radiusb"); raw[2] = scalar_of(sd, "radiusc");
                break;
            case SDFIBM_SHAPE_CIRCLE_TAIL: case SDFIBM_SHAPE_CIRCLE_TWOTAIL:
                raw[0] = scalar_of(sd, "radius"); raw[1] = scalar_of(sd, "ratio"); raw[2] = scalar_of(sd, "thickness");
                break;
            default: break;
        }
        vector_of(sd, "com", com);
        sdfibm_shape_desc s;
        if (sdfibm_host_make_shape(it->second, raw, com, &s) != SDFIBM_OK)
            throw std::runtime_error("bad parameters for shape " + name);
        if (keep_first) shapes.emplace(name, s);
        else shapes[name] = s;
    }
    return shapes;
}

}  // namespace

extern "C" int sdfibm_host_parse_soliddict(const char* text, double rho_f, sdfibm_solid_desc* solids, int32_t capacity,
                                           int32_t* nsolids, sdfibm_options* opt, int32_t* on_twod, char* msg,
                                           int32_t msg_len) {
    auto err = [&](const std::string& m) {
        if (msg && msg_len > 0) {
            std::strncpy(msg, m.c_str(), msg_len - 1);
            msg[msg_len - 1] = 0;
        }
        return SDFIBM_ERR_ARG;
    };
    if (!text || !nsolids || !opt) return err("null argument");
    try {
        const std::string src(text);
        Lexer lx(src);
        auto root = parse_dict(lx, true);
        const Node& meta = root->sub("meta");
        const bool on_fluid = bool_of(meta, "on_fluid");
        const bool twod = bool_of(meta, "on_twod");
        sdfibm_options_default(opt);
        double g[3] = {0, 0, 0};
        if (!vector_of(meta, "gravity", g)) throw std::runtime_error("missing meta.gravity");
        for (int a = 0; a < 3; ++a) opt->gravity[a] = g[a];
        opt->rho_f = on_fluid ? rho_f : 0.0;
        if (on_twod) *on_twod = twod ? 1 : 0;

        const std::map<std::string, sdfibm_shape_desc> shapes = parse_shapes(root->sub("shapes"), true);
        struct Fr { int type; double p[8]; };
        std::map<std::string, Fr> forcers;
        if (const Node* fd = root->find("forces")) {
            for (auto& e : fd->entries) {
                const Node& d = *e.second;
                const std::string type = word_of(d, "type"), name = word_of(d, "name");
                double raw[8] = {0};
                Fr f{};
                if (type == "Constant") {
                    f.type = SDFIBM_FORCER_CONSTANT;
                    if (!vector_of(d, "force", raw) || !vector_of(d, "torque", raw + 3)) throw std::runtime_error("Constant needs force and torque");
                } else if (type == "Spring") {
                    f.type = SDFIBM_FORCER_SPRING;
                    if (!vector_of(d, "pivot", raw)) throw std::runtime_error("Spring needs pivot");
                    raw[3] = scalar_of(d, "k"); raw[4] = scalar_of(d, "l");
                } else if (type == "Magnetic") {
                    f.type = SDFIBM_FORCER_MAGNETIC;
                    if (!vector_of(d, "direction", raw)) throw std::runtime_error("Magnetic needs direction");
                    raw[3] = scalar_of(d, "A"); raw[4] = scalar_of(d, "w");
                } else {
                    throw std::runtime_error("Cannot create unrecognized object: " + type);
                }
                sdfibm_host_make_forcer(f.type, raw, f.p);
                if (!forcers.count(name)) forcers[name] = f;
            }
        }
        struct Mo { int type; double p[8]; };
        std::map<std::string, Mo> motions;
        for (auto& e : root->sub("motions").entries) {
            const Node& d = *e.second;
            const std::string type = word_of(d, "type"), name = word_of(d, "name");
            double raw[8] = {0};
            Mo mo{};
            if (type == "Motion000002" || type == "Motion110002") {
                mo.type = type == "Motion000002" ? SDFIBM_MOTION_000002 : SDFIBM_MOTION_110002;
                raw[0] = scalar_of(d, "period");
            } else if (type == "Motion222000") {
                mo.type = SDFIBM_MOTION_222000;
                raw[0] = scalar_of(d, "u"); raw[1] = scalar_of(d, "v"); raw[2] = scalar_of(d, "w");
            } else if (type == "MotionSineDirectional") {
                mo.type = SDFIBM_MOTION_SINEDIRECTIONAL;
                raw[0] = scalar_of(d, "amplitude"); raw[1] = scalar_of(d, "period");
                if (!vector_of(d, "direction", raw + 2)) throw std::runtime_error("MotionSineDirectional needs direction");
            } else if (type == "Motion01Mask") {
                mo.type = SDFIBM_MOTION_01MASK;
                const std::string mask = word_of(d, "mask");
                if (mask.empty() || mask[0] != 'b') throw std::runtime_error("Mask starts with b");
                if (mask.size() != 7) throw std::runtime_error("Mask size != 7");
                for (int i = 1; i <= 6; ++i) {
                    if (mask[i] != '0' && mask[i] != '1') throw std::runtime_error("Mask ele != 0 or 1");
                    raw[i - 1] = mask[i] == '0' ? 0 : 1;
                }
            } else if (type == "MotionRotor") {
                mo.type = SDFIBM_MOTION_ROTOR;
                raw[0] = scalar_of(d, "period"); raw[1] = scalar_of(d, "radius");
                raw[2] = scalar_of(d, "theta0"); raw[3] = scalar_of(d, "selfom");
            } else if (type == "MotionOpenClose") {
                mo.type = SDFIBM_MOTION_OPENCLOSE;
            } else {
                throw std::runtime_error("Unrecognized motion type " + type);
            }
            sdfibm_host_make_motion(mo.type, raw, mo.p);
            motions[name] = mo;
        }
        std::map<std::string, double> materials;
        for (auto& e : root->sub("materials").entries) {
            const Node& d = *e.second;
            if (word_of(d, "type") != "General") throw std::runtime_error("Unrecognizable material parameter!");
            materials[word_of(d, "name")] = scalar_of(d, "rho");
        }
        const Node& sol = root->sub("solids");
        int32_t n = 0;
        for (auto& e : sol.entries) {
            const Node& d = *e.second;
            double pos[3], vel[3] = {0, 0, 0}, euler[3] = {0, 0, 0}, omega[3] = {0, 0, 0};
            if (!vector_of(d, "pos", pos)) throw std::runtime_error("solid without pos");
            if (twod && pos[2] != 0)
                throw std::runtime_error("Solid must has z=0 in 2D simulation, violated by solid # " + std::to_string(n));
            vector_of(d, "vel", vel);
            vector_of(d, "euler", euler);
            vector_of(d, "omega", omega);
            const std::string mot = word_of(d, "mot_name"), mat = word_of(d, "mat_name"), shp = word_of(d, "shp_name");
            auto si = shapes.find(shp);
            if (si == shapes.end()) throw std::runtime_error("unknown shape name " + shp);
            auto mi = materials.find(mat);
            if (mi == materials.end()) throw std::runtime_error("unknown material name " + mat);
            int mtype = SDFIBM_MOTION_FREE;
            const double* mp = nullptr;
            if (mot != "free") {
                // m_libmotion[name] of an unknown name is a null motion, i.e. free (solidcloud.cpp:185-186)
                auto it = motions.find(mot);
                if (it != motions.end()) { mtype = it->second.type; mp = it->second.p; }
            }
            int ftype = SDFIBM_FORCER_NONE;
            const double* fp = nullptr;
            if (d.find("for_name")) {
                const std::string fn = word_of(d, "for_name");
                auto it = forcers.find(fn);
                if (it == forcers.end()) throw std::runtime_error("Unrecognized force name " + fn);
                ftype = it->second.type;
                fp = it->second.p;
            }
            if (n < capacity && solids) {
                if (sdfibm_host_make_solid(n, &si->second, mi->second, mtype, mp, ftype, fp, pos, euler, vel, omega,
                                           &solids[n]) != SDFIBM_OK)
                    throw std::runtime_error("bad solid " + std::to_string(n));
            }
            ++n;
        }
        *nsolids = n;
        if (n > capacity) return err("solid capacity too small");
    } catch (const std::exception& e) {
        return err(e.what());
    }
    return SDFIBM_OK;
}

// ---- state records and restart dictionary ------------------------------------------------------------------------------
//   euler      OpenFOAM 12 quaternion::eulerAngles(quaternion::XYZ), used by src/solid.cpp:12 and
//              src/solidcloud.cpp:638: for q = qx(a) qy(b) qz(c), R = Rx(a) Ry(b) Rz(c), so
//              R02 = sin b, R12 = -sin a cos b, R22 = cos a cos b, R01 = -cos b sin c, R00 = cos b cos c
//   state      SolidCloud::saveState / operator<<(SolidCloud) src/solidcloud.cpp:578-614 on a stream set to
//              std::scientific (src/solidcloud.cpp:235-236), operator<<(Solid) and write2D src/solid.cpp:5-29
//   restart    SolidCloud::saveRestart src/solidcloud.cpp:616-665: dictionary::set of pos / vel / euler / omega in
//              every solids entry, then dictionary::write of the whole tree in OpenFOAM's ascii layout
namespace {

void euler_xyz(const double* q, double* e) {
    const double w = q[0], x = q[1], y = q[2], z = q[3];
    e[0] = std::atan2(-2 * (y * z - w * x), w * w - x * x - y * y + z * z);
    e[1] = std::asin(2 * (x * z + w * y));
    e[2] = std::atan2(-2 * (x * y - w * z), w * w + x * x - y * y - z * z);
}

void put_sci(std::string& out, double v) {  // std::ostream << double under std::scientific, precision 6
    char b[40];
    std::snprintf(b, sizeof(b), "%.6e", v);
    out += b;
}

std::string put_g(double v, int prec) {  // std::ostream << double in the default float format
    char b[48];
    std::snprintf(b, sizeof(b), "%.*g", prec, v);
    return b;
}

// OpenFOAM's tokeniser reads a word that starts like a number as a label (digits only) or a scalar
bool is_number_token(const std::string& t) {
    if (t.empty()) return false;
    const char c = t[0];
    if (!(std::isdigit((unsigned char)c) || c == '-' || c == '+' || c == '.')) return false;
    char* end = nullptr;
    std::strtod(t.c_str(), &end);
    return end == t.c_str() + t.size();
}
bool is_label_token(const std::string& t) {
    size_t i = (t[0] == '-' || t[0] == '+') ? 1 : 0;
    if (i == t.size() || t.size() - i > 18) return false;
    for (; i < t.size(); ++i)
        if (!std::isdigit((unsigned char)t[i])) return false;
    return true;
}
std::string format_token(const std::string& t, bool quoted, int prec) {
    if (quoted) return "\"" + t + "\"";
    if (!is_number_token(t)) return t;
    if (is_label_token(t)) return std::to_string(std::stoll(t));
    return put_g(std::strtod(t.c_str(), nullptr), prec);
}

// dictionary::set: replace the value of an existing keyword in place, else append the entry
void set_vector(Node& d, const std::string& key, const double v[3], int prec) {
    auto n = std::make_shared<Node>();
    n->tokens = {"(", put_g(v[0], prec), put_g(v[1], prec), put_g(v[2], prec), ")"};
    n->quoted.assign(n->tokens.size(), 0);
    for (auto& e : d.entries)
        if (e.first == key) {
            e.second = n;
            return;
        }
    d.entries.emplace_back(key, n);
}

// dictionary::write: primitive entries as the keyword padded to 16 columns, the tokens separated by one space and
// ';'; sub-dictionaries as the keyword, then '{' ... '}' on lines of their own; 4 spaces of indent per level; an
// empty line between the entries of the top level
void write_dict(std::string& out, const Node& d, int level, int prec) {
    std::vector<const std::pair<std::string, std::shared_ptr<Node>>*> list;
    for (auto& e : d.entries)
        if (!(level == 0 && e.first == "FoamFile")) list.push_back(&e);  // read without its header entry
    const std::string ind(4 * level, ' ');
    for (size_t k = 0; k < list.size(); ++k) {
        const std::string& key = list[k]->first;
        const Node& n = *list[k]->second;
        if (n.is_dict) {
            out += ind + key + "\n" + ind + "{\n";
            write_dict(out, n, level + 1, prec);
            out += ind + "}\n";
        } else {
            out += ind + key;
            out.append(std::max<int>(16 - (int)key.size(), 1), ' ');
            for (size_t i = 0; i < n.tokens.size(); ++i) {
                if (i) out += ' ';
                out += format_token(n.tokens[i], i < n.quoted.size() && n.quoted[i], prec);
            }
            out += ";\n";
        }
        if (level == 0 && k + 1 < list.size()) out += "\n";
    }
}

const char* const kRestartHeader =
    "/*--------------------------------*- C++ -*----------------------------------*\\\n"
    "| =========                 |                                                 |\n"
    "| \\\\      /  F ield         | OpenFOAM: The Open Source CFD Toolbox           |\n"
    "|  \\\\    /   O peration     | Version:  6.0.0                                 |\n"
    "|   \\\\  /    A nd           | Web:      www.OpenFOAM.org                      |\n"
    "|    \\\\/     M anipulation  |                                                 |\n"
    "\\*---------------------------------------------------------------------------*/\n"
    "FoamFile\n{\n"
    "    version     2.0;\n    format      ascii;\n    class       dictionary;\n    object      solidDict;\n}\n"
    "// * * * * * * * * * * * * * * * * * * * * * * * * * * * * * * * * * * * * * //\n";

int emit(const std::string& text, char* buf, int64_t cap, int64_t* len) {
    if (len) *len = (int64_t)text.size();
    if (!buf) return cap > 0 ? SDFIBM_ERR_ARG : SDFIBM_OK;
    if (cap <= (int64_t)text.size()) return SDFIBM_ERR_CAPACITY;
    std::memcpy(buf, text.data(), text.size());
    buf[text.size()] = 0;
    return SDFIBM_OK;
}

}  // namespace

extern "C" void sdfibm_host_euler_from_quat(const double* quat_wxyz, double* euler_rad) {
    euler_xyz(quat_wxyz, euler_rad);
}

extern "C" int sdfibm_host_format_state(double time, int32_t twod, const sdfibm_solid_state* st, int32_t n, char* buf,
                                        int64_t cap, int64_t* len) {
    if (n < 0 || (n > 0 && !st) || !len) return SDFIBM_ERR_ARG;
    std::string out;
    out.reserve((size_t)n * (twod ? 140 : 260));
    for (int32_t i = 0; i < n; ++i) {
        const sdfibm_solid_state& s = st[i];
        double e[3];
        euler_xyz(s.quat, e);
        put_sci(out, time);
        out += ' ';
        if (twod) {
            const double v[9] = {s.pos[0], s.pos[1], s.vel[0], s.vel[1], s.force[0], s.force[1], e[2], s.omega[2],
                                 s.torque[2]};
            for (int k = 0; k < 9; ++k) {
                put_sci(out, v[k]);
                out += k < 8 ? ' ' : '\n';
            }
        } else {
            const double* g[6] = {s.pos, s.vel, s.force, e, s.omega, s.torque};
            for (int k = 0; k < 18; ++k) {
                put_sci(out, g[k / 3][k % 3]);
                out += k < 17 ? ' ' : '\n';
            }
        }
    }
    return emit(out, buf, cap, len);
}

extern "C" int sdfibm_host_write_restart(const char* dict_text, const sdfibm_solid_state* st, int32_t n, int32_t twod,
                                         int32_t precision, const char* stamp, char* buf, int64_t cap, int64_t* len,
                                         char* msg, int32_t msg_len) {
    auto err = [&](const std::string& m, int code) {
        if (msg && msg_len > 0) {
            std::strncpy(msg, m.c_str(), msg_len - 1);
            msg[msg_len - 1] = 0;
        }
        return code;
    };
    if (!dict_text || (n > 0 && !st) || n < 0 || !len || precision < 0 || precision > 17)
        return err("bad argument", SDFIBM_ERR_ARG);
    std::string out;
    try {
        const std::string src(dict_text);
        Lexer lx(src);
        auto root = parse_dict(lx, true);
        Node* solids = nullptr;
        for (auto& e : root->entries)
            if (e.first == "solids" && e.second->is_dict) solids = e.second.get();
        if (!solids) throw std::runtime_error("missing sub-dictionary solids");
        if ((int32_t)solids->entries.size() != n)
            throw std::runtime_error("solids holds " + std::to_string(solids->entries.size()) + " entries, " +
                                     std::to_string(n) + " states given");
        const int prec = precision ? precision : 6;
        for (int32_t i = 0; i < n; ++i) {
            Node& d = *solids->entries[i].second;
            if (!d.is_dict) throw std::runtime_error("solids entry " + solids->entries[i].first + " is not a dictionary");
            const sdfibm_solid_state& s = st[i];
            double pos[3] = {s.pos[0], s.pos[1], s.pos[2]}, vel[3] = {s.vel[0], s.vel[1], s.vel[2]};
            double om[3] = {s.omega[0], s.omega[1], s.omega[2]}, e[3];
            if (twod) pos[2] = vel[2] = om[0] = om[1] = 0.0;
            euler_xyz(s.quat, e);
            for (int a = 0; a < 3; ++a) e[a] = e[a] * 180.0 / M_PI;
            set_vector(d, "pos", pos, prec);
            set_vector(d, "vel", vel, prec);
            set_vector(d, "euler", e, prec);
            set_vector(d, "omega", om, prec);
        }
        out = kRestartHeader;
        write_dict(out, *root, 0, prec);
        char tb[80] = {0};
        if (!stamp) {
            std::time_t t = std::time(nullptr);
            std::tm tmv;
            localtime_r(&t, &tmv);
            std::strftime(tb, sizeof(tb), "%y/%m/%d %X", &tmv);
            stamp = tb;
        }
        out += "\n// ";
        out += stamp;
        out += "\n";
    } catch (const std::exception& e) {
        return err(e.what(), SDFIBM_ERR_ARG);
    }
    const int rc = emit(out, buf, cap, len);
    if (rc != SDFIBM_OK) return err("buffer too small", rc);
    return SDFIBM_OK;
}

extern "C" int sdfibm_host_soliddict_lookup(const char* text, const char* path, char* buf, int64_t cap, int64_t* len) {
    if (!text || !path || !len) return SDFIBM_ERR_ARG;
    try {
        const std::string src(text);
        Lexer lx(src);
        auto root = parse_dict(lx, true);
        const Node* n = root.get();
        std::string p(path);
        size_t b = 0;
        for (;;) {
            const size_t e = p.find('/', b);
            const std::string key = p.substr(b, e == std::string::npos ? std::string::npos : e - b);
            if (!n->is_dict) return SDFIBM_ERR_ARG;
            n = n->find(key);
            if (!n) {
                *len = -1;
                return SDFIBM_OK;
            }
            if (e == std::string::npos) break;
            b = e + 1;
        }
        if (n->is_dict) return SDFIBM_ERR_ARG;
        std::string out;
        for (size_t i = 0; i < n->tokens.size(); ++i) {
            if (i) out += ' ';
            out += n->tokens[i];
        }
        return emit(out, buf, cap, len);
    } catch (const std::exception&) {
        return SDFIBM_ERR_ARG;
    }
}

// SolidCloud::writeMeanField (src/solidcloud.cpp:303-313) on a stream set to std::scientific (:31-33)
extern "C" int sdfibm_host_format_mean_field(const double* mean3, int32_t n, char* buf, int64_t cap, int64_t* len) {
    if (n < 0 || (n > 0 && !mean3) || !len) return SDFIBM_ERR_ARG;
    std::string out;
    out.reserve((size_t)n * 42 + 1);
    for (int64_t i = 0; i < 3 * (int64_t)n; ++i) {
        put_sci(out, mean3[i]);
        out += ' ';
    }
    out += '\n';
    return emit(out, buf, cap, len);
}

// ---- VOF initializer front end (tool_vof) ------------------------------------------------------------------------------
//   solidDict   tool_vof/solidcloud.cpp:12-112: meta.on_twod, the shapes library, material rho = 1, every "solids"
//               entry as Solid(i, pos, identity) + euler + shape; the example's "planes" entries follow the solids
//   blockMesh   a single uniform hex block (the mesh of the uniform-grid path)
//   field file  the internalField of a volScalarField rewritten in the file's own format (ascii or binary), the rest
//               of the file kept as it is (IOobject MUST_READ + field.write(), tool_vof/solidcloud.cpp:143-164)
namespace {

void read_vof_entries(const Node& list, const std::map<std::string, sdfibm_shape_desc>& shapes, bool twod,
                      std::vector<sdfibm_solid_desc>& out) {
    for (auto& e : list.entries) {
        const Node& d = *e.second;
        if (!d.is_dict) throw std::runtime_error("entry " + e.first + " is not a dictionary");
        const int32_t i = (int32_t)out.size();
        double pos[3], euler[3] = {0, 0, 0};
        if (!vector_of(d, "pos", pos)) throw std::runtime_error("solid without pos");
        if (twod && pos[2] != 0)
            throw std::runtime_error("Solid must has z=0 in 2D simulation, violated by solid # " + std::to_string(i));
        vector_of(d, "euler", euler);
        const std::string shp = word_of(d, "shp_name");
        auto si = shapes.find(shp);
        if (si == shapes.end()) throw std::runtime_error("unknown shape name " + shp);
        sdfibm_solid_desc s;
        if (sdfibm_host_make_solid(i, &si->second, 1.0, SDFIBM_MOTION_FREE, nullptr, SDFIBM_FORCER_NONE, nullptr, pos,
                                   euler, nullptr, nullptr, &s) != SDFIBM_OK)
            throw std::runtime_error("bad solid " + std::to_string(i));
        out.push_back(s);
    }
}

int set_msg(char* msg, int32_t msg_len, const std::string& m, int code) {
    if (msg && msg_len > 0) {
        std::strncpy(msg, m.c_str(), msg_len - 1);
        msg[msg_len - 1] = 0;
    }
    return code;
}

// the value tokens of a list entry of a dictionary that the solidDict grammar does not cover (blockMeshDict's
// "boundary" holds sub-dictionaries inside a list): scan for `key` at brace depth 0 and collect to its ';'
bool raw_entry(const std::string& src, const std::string& key, std::vector<std::string>& toks) {
    Lexer lx(src);
    std::string t;
    int depth = 0;
    while (lx.next(t)) {
        if (t == "{") ++depth;
        else if (t == "}") --depth;
        else if (depth == 0 && t == key && !lx.quoted) {
            toks.clear();
            int par = 0;
            while (lx.next(t)) {
                if (t == "(") ++par;
                if (t == ")") --par;
                if (t == ";" && par == 0) return true;
                toks.push_back(t);
            }
            throw std::runtime_error("unterminated entry " + key);
        }
    }
    return false;
}

}  // namespace

extern "C" int sdfibm_host_parse_vofdict(const char* text, int32_t with_planes, sdfibm_solid_desc* solids,
                                         int32_t capacity, int32_t* nsolids, int32_t* on_twod, char* msg,
                                         int32_t msg_len) {
    if (!text || !nsolids) return set_msg(msg, msg_len, "null argument", SDFIBM_ERR_ARG);
    try {
        const std::string src(text);
        Lexer lx(src);
        auto root = parse_dict(lx, true);
        const bool twod = bool_of(root->sub("meta"), "on_twod");
        if (on_twod) *on_twod = twod ? 1 : 0;
        const auto shapes = parse_shapes(root->sub("shapes"), false);
        std::vector<sdfibm_solid_desc> out;
        read_vof_entries(root->sub("solids"), shapes, twod, out);
        if (with_planes)
            if (const Node* pl = root->find("planes")) {
                if (!pl->is_dict) throw std::runtime_error("planes is not a dictionary");
                read_vof_entries(*pl, shapes, twod, out);
            }
        *nsolids = (int32_t)out.size();
        if ((int32_t)out.size() > capacity) return set_msg(msg, msg_len, "solid capacity too small", SDFIBM_ERR_ARG);
        if (solids)
            for (size_t i = 0; i < out.size(); ++i) solids[i] = out[i];
    } catch (const std::exception& e) {
        return set_msg(msg, msg_len, e.what(), SDFIBM_ERR_ARG);
    }
    return SDFIBM_OK;
}

extern "C" int sdfibm_host_parse_blockmesh(const char* text, sdfibm_mesh_desc* mesh, char* msg, int32_t msg_len) {
    if (!text || !mesh) return set_msg(msg, msg_len, "null argument", SDFIBM_ERR_ARG);
    try {
        const std::string src(text);
        std::vector<std::string> t;
        double scale = 1.0;
        if (raw_entry(src, "convertToMeters", t) || raw_entry(src, "scale", t)) {
            if (t.size() != 1) throw std::runtime_error("bad convertToMeters");
            scale = to_num(t[0]);
        }
        if (!raw_entry(src, "vertices", t)) throw std::runtime_error("missing vertices");
        std::vector<double> v;
        for (auto& x : t)
            if (x != "(" && x != ")") v.push_back(to_num(x) * scale);
        if (v.empty() || v.size() % 3) throw std::runtime_error("bad vertices");
        if (!raw_entry(src, "blocks", t)) throw std::runtime_error("missing blocks");
        // ( hex ( 8 labels ) ( nx ny nz ) simpleGrading ( 1 1 1 ) )
        std::vector<std::string> w;
        for (auto& x : t)
            if (x != "(" && x != ")") w.push_back(x);
        if (w.size() != 16 || w[0] != "hex" || w[12] != "simpleGrading")
            throw std::runtime_error("one hex block with simpleGrading expected");
        for (int k = 13; k < 16; ++k)
            if (to_num(w[k]) != 1.0) throw std::runtime_error("graded block: only uniform grading is supported");
        int lab[8];
        const int nv = (int)(v.size() / 3);
        for (int k = 0; k < 8; ++k) {
            lab[k] = (int)to_num(w[1 + k]);
            if (lab[k] < 0 || lab[k] >= nv) throw std::runtime_error("block vertex label out of range");
        }
        const long long n[3] = {std::stoll(w[9]), std::stoll(w[10]), std::stoll(w[11])};
        for (int a = 0; a < 3; ++a)
            if (n[a] < 1 || n[a] > (1 << 30)) throw std::runtime_error("bad cell count");
        // the hex's local axes: x = v0->v1, y = v0->v3, z = v0->v4 (blockMesh's vertex order), axis-aligned
        auto P = [&](int k, int a) { return v[3 * lab[k] + a]; };
        double lo[3], hi[3];
        for (int a = 0; a < 3; ++a) lo[a] = P(0, a);
        const int far[3] = {1, 3, 4};
        for (int a = 0; a < 3; ++a) {
            hi[a] = P(far[a], a);
            for (int b = 0; b < 3; ++b)
                if (b != a && P(far[a], b) != P(0, b)) throw std::runtime_error("the block is not axis-aligned");
            if (!(hi[a] > lo[a])) throw std::runtime_error("the block's local axes must point along +x, +y, +z");
        }
        // the remaining corners must close the box
        const int corner[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0}, {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};
        for (int k = 0; k < 8; ++k)
            for (int a = 0; a < 3; ++a)
                if (P(k, a) != (corner[k][a] ? hi[a] : lo[a])) throw std::runtime_error("the block is not a box");
        mesh->nx = (int32_t)n[0];
        mesh->ny = (int32_t)n[1];
        mesh->nz = (int32_t)n[2];
        mesh->twod = n[2] == 1 ? 1 : 0;
        for (int a = 0; a < 3; ++a) {
            mesh->origin[a] = lo[a];
            mesh->h[a] = (hi[a] - lo[a]) / (double)n[a];
        }
    } catch (const std::exception& e) {
        return set_msg(msg, msg_len, e.what(), SDFIBM_ERR_ARG);
    }
    return SDFIBM_OK;
}

namespace {

// the internalField of a vol<Type>Field file replaced by n values of `width` components (1: scalar, 3: vector)
int write_field(const char* file, int64_t file_len, const double* values, int64_t n, int width, int32_t format,
                int32_t precision, char* buf, int64_t cap, int64_t* len, char* msg, int32_t msg_len) {
    if (!file || file_len < 0 || (n > 0 && !values) || n < 0 || !len || precision < 0 || precision > 17 ||
        format < -1 || format > 1)
        return set_msg(msg, msg_len, "bad argument", SDFIBM_ERR_ARG);
    const std::string src(file, (size_t)file_len);
    const std::string list_type = width == 3 ? "List<vector>" : "List<scalar>";
    try {
        // the header's format (FoamFile { format ascii|binary; }): the text before the first binary byte
        const size_t hdr = src.find("FoamFile");
        if (hdr == std::string::npos) throw std::runtime_error("no FoamFile header");
        const size_t hend = src.find('}', hdr);
        if (hend == std::string::npos) throw std::runtime_error("unterminated FoamFile header");
        bool binary = false;
        {
            std::vector<std::string> t;
            const std::string header = src.substr(hdr, hend - hdr + 1);
            if (raw_entry(header.substr(header.find('{') + 1, header.rfind('}') - header.find('{') - 1), "format", t))
                binary = t.size() == 1 && t[0] == "binary";
        }
        // the header's format word, rewritten when the output format differs from the file's
        std::string head = src.substr(0, hend + 1);
        if (format >= 0 && (format == 1) != binary) {
            size_t f = head.find("format", hdr);
            while (f != std::string::npos &&
                   !(std::isspace((unsigned char)head[f - 1]) && std::isspace((unsigned char)head[f + 6])))
                f = head.find("format", f + 6);
            if (f == std::string::npos) throw std::runtime_error("no format entry in the FoamFile header");
            size_t b = f + 6;
            while (b < head.size() && std::isspace((unsigned char)head[b])) ++b;
            const size_t e = head.find(';', b);
            if (e == std::string::npos) throw std::runtime_error("bad format entry");
            head.replace(b, e - b, format == 1 ? "binary" : "ascii");
        }
        const bool out_binary = format < 0 ? binary : format == 1;
        // internalField after the header, at brace depth 0
        size_t at = hend + 1;
        int depth = 0;
        size_t key = std::string::npos;
        for (size_t i = at; i + 13 <= src.size(); ++i) {
            const char c = src[i];
            if (c == '{') ++depth;
            else if (c == '}') --depth;
            else if (c == '/' && i + 1 < src.size() && src[i + 1] == '/') {
                i = src.find('\n', i);
                if (i == std::string::npos) break;
            } else if (depth == 0 && src.compare(i, 13, "internalField") == 0 &&
                       (i == 0 || std::isspace((unsigned char)src[i - 1])) &&
                       (i + 13 == src.size() || std::isspace((unsigned char)src[i + 13]))) {
                key = i;
                break;
            }
        }
        if (key == std::string::npos) throw std::runtime_error("no internalField");
        // the end of its value: ';' after `uniform v`, or after the closing ')' of a nonuniform list (binary lists
        // are skipped by their byte count)
        size_t p = key + 13;
        auto skip_ws = [&]() { while (p < src.size() && std::isspace((unsigned char)src[p])) ++p; };
        auto word = [&]() {
            skip_ws();
            size_t b = p;
            while (p < src.size() && !std::isspace((unsigned char)src[p]) && src[p] != '(' && src[p] != ';') ++p;
            return src.substr(b, p - b);
        };
        const std::string kind = word();
        size_t end;
        if (kind == "uniform") {
            end = src.find(';', p);
        } else if (kind == "nonuniform") {
            const std::string lt = word();
            if (lt != list_type) throw std::runtime_error("internalField is not a " + list_type);
            const std::string cnt = word();
            const long long m = std::stoll(cnt);
            skip_ws();
            if (p >= src.size() || src[p] != '(') throw std::runtime_error("bad internalField list");
            // an element takes 8 bytes per component in binary, and at least 2 bytes in ascii
            if (m < 0 || (uint64_t)m > (uint64_t)(src.size() - p) / (binary ? 8 * (uint64_t)width : 2))
                throw std::runtime_error("bad internalField size");
            if (binary) {
                p += 1 + (size_t)m * 8 * (size_t)width;
                if (p >= src.size() || src[p] != ')') throw std::runtime_error("bad binary internalField list");
            } else {
                // the closing parenthesis of the list (vector elements hold their own)
                int depth = 0;
                for (++p; p < src.size(); ++p) {
                    if (src[p] == '(') ++depth;
                    else if (src[p] == ')' && depth-- == 0) break;
                }
                if (p >= src.size()) throw std::runtime_error("unterminated internalField list");
            }
            end = src.find(';', p);
        } else {
            throw std::runtime_error("unknown internalField form " + kind);
        }
        if (end == std::string::npos) throw std::runtime_error("unterminated internalField");
        std::string out = head + src.substr(hend + 1, key - hend - 1);
        out += "internalField   nonuniform " + list_type + " \n" + std::to_string(n) + "\n(";
        if (out_binary) {
            out.append(reinterpret_cast<const char*>(values), (size_t)(n * width) * 8);  // little-endian doubles
        } else {
            const int prec = precision ? precision : 6;
            out += "\n";
            for (int64_t i = 0; i < n; ++i) {
                if (width == 1) {
                    out += put_g(values[i], prec);
                } else {
                    out += "(";
                    for (int a = 0; a < width; ++a) {
                        if (a) out += ' ';
                        out += put_g(values[i * width + a], prec);
                    }
                    out += ")";
                }
                out += "\n";
            }
        }
        out += ")\n";
        out += src.substr(end);
        const int rc = emit(out, buf, cap, len);
        return rc == SDFIBM_OK ? SDFIBM_OK : set_msg(msg, msg_len, "buffer too small", rc);
    } catch (const std::exception& e) {
        return set_msg(msg, msg_len, e.what(), SDFIBM_ERR_ARG);
    }
}

}  // namespace

extern "C" int sdfibm_host_write_scalar_field(const char* file, int64_t file_len, const double* values, int64_t n,
                                              int32_t format, int32_t precision, char* buf, int64_t cap, int64_t* len,
                                              char* msg, int32_t msg_len) {
    return write_field(file, file_len, values, n, 1, format, precision, buf, cap, len, msg, msg_len);
}

extern "C" int sdfibm_host_write_vector_field(const char* file, int64_t file_len, const double* values, int64_t n,
                                              int32_t format, int32_t precision, char* buf, int64_t cap, int64_t* len,
                                              char* msg, int32_t msg_len) {
    return write_field(file, file_len, values, n, 3, format, precision, buf, cap, len, msg, msg_len);
}

// One shape of a solidDict's library by name (meta.sampler names one, src/solidcloud.cpp:38, 308)
extern "C" int sdfibm_host_soliddict_shape(const char* text, const char* name, sdfibm_shape_desc* out, char* msg,
                                           int32_t msg_len) {
    if (!text || !name || !out) return set_msg(msg, msg_len, "null argument", SDFIBM_ERR_ARG);
    try {
        const std::string src(text);
        Lexer lx(src);
        auto root = parse_dict(lx, true);
        const auto shapes = parse_shapes(root->sub("shapes"), true);
        auto it = shapes.find(name);
        if (it == shapes.end()) return set_msg(msg, msg_len, std::string("unknown shape name ") + name, SDFIBM_ERR_ARG);
        *out = it->second;
    } catch (const std::exception& e) {
        return set_msg(msg, msg_len, e.what(), SDFIBM_ERR_ARG);
    }
    return SDFIBM_OK;
}

// ---- OpenFOAM list files (polyMesh points / faces / owner / neighbour, field internalFields) ----------------------------
// Layout of OpenFOAM's IOstream lists: "N" then "(" and the N elements, then ")"; in binary files the elements are the
// raw little-endian scalars (8 bytes) or labels (4 bytes, 32-bit label builds such as the reference's) between the
// parentheses; a faceCompactList is two lists (N + 1 offsets, then the vertex labels).
namespace {

struct FoamHeader {
    bool binary = false;
    std::string cls;
    size_t body = 0;  // offset after the header's closing brace
};

FoamHeader foam_header(const std::string& src) {
    FoamHeader h;
    const size_t at = src.find("FoamFile");
    if (at == std::string::npos) throw std::runtime_error("no FoamFile header");
    const size_t open = src.find('{', at), close = open == std::string::npos ? open : src.find('}', open);
    if (close == std::string::npos) throw std::runtime_error("unterminated FoamFile header");
    const std::string inner = src.substr(open + 1, close - open - 1);
    std::vector<std::string> t;
    if (raw_entry(inner, "format", t)) h.binary = t.size() == 1 && t[0] == "binary";
    if (raw_entry(inner, "class", t) && t.size() == 1) h.cls = t[0];
    h.body = close + 1;
    return h;
}

void skip_blank(const std::string& s, size_t& p) {
    for (;;) {
        while (p < s.size() && std::isspace((unsigned char)s[p])) ++p;
        if (p + 1 < s.size() && s[p] == '/' && s[p + 1] == '/') {
            p = s.find('\n', p);
            if (p == std::string::npos) p = s.size();
        } else if (p + 1 < s.size() && s[p] == '/' && s[p + 1] == '*') {
            const size_t e = s.find("*/", p + 2);
            p = e == std::string::npos ? s.size() : e + 2;
        } else {
            return;
        }
    }
}

std::string next_word(const std::string& s, size_t& p) {
    skip_blank(s, p);
    const size_t b = p;
    while (p < s.size() && !std::isspace((unsigned char)s[p]) && s[p] != '(' && s[p] != ')' && s[p] != ';') ++p;
    return s.substr(b, p - b);
}

// "N (" at p: returns N and leaves p after the '('
int64_t list_open(const std::string& s, size_t& p) {
    const std::string w = next_word(s, p);
    if (w.empty() || !std::isdigit((unsigned char)w[0])) throw std::runtime_error("list size expected");
    const long long n = std::stoll(w);
    skip_blank(s, p);
    if (p >= s.size() || s[p] != '(') throw std::runtime_error("'(' expected");
    ++p;
    if (n < 0) throw std::runtime_error("negative list size");
    // every element takes at least one byte: a size beyond the rest of the file is corrupt (and is refused before
    // anyone allocates for it)
    if ((uint64_t)n > (uint64_t)(s.size() - p)) throw std::runtime_error("list size exceeds the file");
    return (int64_t)n;
}

// n values of `width` numbers each (width 3: "(x y z)" elements in ascii) into out (doubles or int32 labels)
void read_items(const std::string& s, size_t& p, bool binary, int64_t n, int width, bool labels, double* dout,
                int32_t* iout) {
    const size_t esize = labels ? 4 : 8;
    if (binary) {
        const uint64_t bytes = (uint64_t)n * (uint64_t)width * esize;
        if (bytes > s.size() - p) throw std::runtime_error("binary list shorter than its size");
        if (dout) std::memcpy(dout, s.data() + p, (size_t)bytes);
        if (iout) std::memcpy(iout, s.data() + p, (size_t)bytes);
        p += (size_t)bytes;
    } else {
        for (int64_t i = 0; i < n; ++i) {
            if (width > 1) {
                skip_blank(s, p);
                if (p >= s.size() || s[p] != '(') throw std::runtime_error("'(' of a list element expected");
                ++p;
            }
            for (int a = 0; a < width; ++a) {
                const std::string w = next_word(s, p);
                if (w.empty()) throw std::runtime_error("number expected");
                if (labels) {
                    const long long v = std::stoll(w);
                    if (iout) iout[i * width + a] = (int32_t)v;
                } else if (dout) {
                    dout[i * width + a] = to_num(w);
                } else {
                    to_num(w);
                }
            }
            if (width > 1) {
                skip_blank(s, p);
                if (p >= s.size() || s[p] != ')') throw std::runtime_error("')' of a list element expected");
                ++p;
            }
        }
    }
    skip_blank(s, p);
    if (p >= s.size() || s[p] != ')') throw std::runtime_error("')' expected after the list");
    ++p;
}

// the position after the "internalField" keyword at brace depth 0 after the header
size_t internal_field(const std::string& src, size_t from) {
    int depth = 0;
    for (size_t i = from; i + 13 <= src.size(); ++i) {
        const char c = src[i];
        if (c == '{') ++depth;
        else if (c == '}') --depth;
        else if (c == '/' && i + 1 < src.size() && (src[i + 1] == '/' || src[i + 1] == '*')) {
            size_t q = i;
            skip_blank(src, q);
            i = q - 1;
        } else if (depth == 0 && src.compare(i, 13, "internalField") == 0 &&
                   (i == 0 || std::isspace((unsigned char)src[i - 1])) &&
                   (i + 13 == src.size() || std::isspace((unsigned char)src[i + 13]))) {
            return i + 13;
        }
    }
    throw std::runtime_error("no internalField");
}

}  // namespace

extern "C" int sdfibm_host_read_foam_list(const char* file, int64_t file_len, int32_t kind, void* out, int64_t cap,
                                          int64_t* n, char* msg, int32_t msg_len) {
    if (!file || file_len < 0 || !n || kind < SDFIBM_FOAM_SCALAR || kind > SDFIBM_FOAM_LABEL)
        return set_msg(msg, msg_len, "bad argument", SDFIBM_ERR_ARG);
    try {
        const std::string src(file, (size_t)file_len);
        const FoamHeader h = foam_header(src);
        const int width = kind == SDFIBM_FOAM_VECTOR ? 3 : 1;
        const bool labels = kind == SDFIBM_FOAM_LABEL;
        size_t p = h.body;
        if (h.cls.compare(0, 3, "vol") == 0) {
            p = internal_field(src, h.body);
            const std::string form = next_word(src, p);
            if (form == "uniform") {
                if (labels) throw std::runtime_error("a uniform field holds no labels");
                double v[3];
                size_t q = p;
                skip_blank(src, q);
                if (width == 3) {
                    if (q >= src.size() || src[q] != '(') throw std::runtime_error("uniform vector expected");
                    p = q + 1;
                    for (int a = 0; a < 3; ++a) v[a] = to_num(next_word(src, p));
                } else {
                    v[0] = to_num(next_word(src, p));
                }
                *n = -1;  // uniform: the value only
                if (out && cap >= 1) std::memcpy(out, v, sizeof(double) * width);
                return SDFIBM_OK;
            }
            if (form != "nonuniform") throw std::runtime_error("unknown internalField form " + form);
            const std::string lt = next_word(src, p);
            if (lt != (width == 3 ? "List<vector>" : "List<scalar>"))
                throw std::runtime_error("internalField is a " + lt);
        }
        const int64_t m = list_open(src, p);
        *n = m;
        if (!out) return SDFIBM_OK;
        if (cap < m) return set_msg(msg, msg_len, "output capacity too small", SDFIBM_ERR_CAPACITY);
        read_items(src, p, h.binary, m, width, labels, labels ? nullptr : static_cast<double*>(out),
                   labels ? static_cast<int32_t*>(out) : nullptr);
    } catch (const std::exception& e) {
        return set_msg(msg, msg_len, e.what(), SDFIBM_ERR_ARG);
    }
    return SDFIBM_OK;
}

extern "C" int sdfibm_host_read_foam_faces(const char* file, int64_t file_len, int32_t* offsets, int64_t cap_offsets,
                                           int32_t* labels, int64_t cap_labels, int64_t* nfaces, int64_t* nlabels,
                                           char* msg, int32_t msg_len) {
    if (!file || file_len < 0 || !nfaces || !nlabels) return set_msg(msg, msg_len, "bad argument", SDFIBM_ERR_ARG);
    try {
        const std::string src(file, (size_t)file_len);
        const FoamHeader h = foam_header(src);
        size_t p = h.body;
        const bool measure = !offsets || !labels;
        if (h.cls == "faceCompactList") {
            const int64_t no = list_open(src, p);
            if (no < 1) throw std::runtime_error("empty offset list");
            std::vector<int32_t> off((size_t)no);
            read_items(src, p, h.binary, no, 1, true, nullptr, off.data());
            const int64_t nl = list_open(src, p);
            *nfaces = no - 1;
            *nlabels = nl;
            if (off[0] != 0 || off.back() != nl) throw std::runtime_error("offsets do not match the label list");
            for (int64_t i = 0; i + 1 < no; ++i)
                if (off[(size_t)i + 1] < off[(size_t)i]) throw std::runtime_error("decreasing face offsets");
            if (measure) return SDFIBM_OK;
            if (cap_offsets < no || cap_labels < nl)
                return set_msg(msg, msg_len, "output capacity too small", SDFIBM_ERR_CAPACITY);
            std::memcpy(offsets, off.data(), sizeof(int32_t) * (size_t)no);
            read_items(src, p, h.binary, nl, 1, true, nullptr, labels);
        } else if (h.cls == "faceList") {
            if (h.binary) throw std::runtime_error("binary faceList: write the mesh as faceCompactList");
            const int64_t nf = list_open(src, p);
            std::vector<int32_t> off(1, 0), lab;
            for (int64_t f = 0; f < nf; ++f) {
                const int64_t k = list_open(src, p);
                const size_t b = lab.size();
                lab.resize(b + (size_t)k);
                read_items(src, p, false, k, 1, true, nullptr, lab.data() + b);
                off.push_back((int32_t)lab.size());
            }
            skip_blank(src, p);
            if (p >= src.size() || src[p] != ')') throw std::runtime_error("')' expected after the faces");
            *nfaces = nf;
            *nlabels = (int64_t)lab.size();
            if (measure) return SDFIBM_OK;
            if (cap_offsets < nf + 1 || cap_labels < (int64_t)lab.size())
                return set_msg(msg, msg_len, "output capacity too small", SDFIBM_ERR_CAPACITY);
            std::memcpy(offsets, off.data(), sizeof(int32_t) * off.size());
            if (!lab.empty()) std::memcpy(labels, lab.data(), sizeof(int32_t) * lab.size());
        } else {
            throw std::runtime_error("not a face list: class " + h.cls);
        }
    } catch (const std::exception& e) {
        return set_msg(msg, msg_len, e.what(), SDFIBM_ERR_ARG);
    }
    return SDFIBM_OK;
}

extern "C" int sdfibm_host_uniform_mesh(const double* points, int64_t npoints, int64_t ncells, double rtol,
                                        sdfibm_mesh_desc* mesh, char* msg, int32_t msg_len) {
    if (!points || npoints < 8 || !mesh || !(rtol >= 0)) return set_msg(msg, msg_len, "bad argument", SDFIBM_ERR_ARG);
    auto P = [&](int64_t i, int a) { return points[3 * i + a]; };
    // single-block numbering: x fastest, then y, then z (a row ends where x falls back, a layer where y does; the
    // lattice check below bounds every coordinate, blockMesh's points being within rounding of the lattice)
    int64_t px = 1;
    while (px < npoints && P(px, 0) > P(px - 1, 0)) ++px;
    if (px < 2 || npoints % px) return set_msg(msg, msg_len, "points are not a lattice row by row", SDFIBM_ERR_ARG);
    int64_t py = 1;
    while (py * px < npoints && P(py * px, 1) > P((py - 1) * px, 1)) ++py;
    if (py < 2 || npoints % (px * py)) return set_msg(msg, msg_len, "points are not a lattice layer by layer", SDFIBM_ERR_ARG);
    const int64_t pz = npoints / (px * py);
    if (pz < 2) return set_msg(msg, msg_len, "one layer of points", SDFIBM_ERR_ARG);
    const int64_t n[3] = {px - 1, py - 1, pz - 1};
    if (n[0] * n[1] * n[2] != ncells)
        return set_msg(msg, msg_len, "the point lattice does not match the cell count", SDFIBM_ERR_ARG);
    if (n[0] > INT32_MAX || n[1] > INT32_MAX || n[2] > INT32_MAX) return set_msg(msg, msg_len, "too many cells", SDFIBM_ERR_ARG);
    const int64_t last = npoints - 1;
    double o[3], h[3], ext = 0;
    for (int a = 0; a < 3; ++a) {
        o[a] = P(0, a);
        h[a] = (P(last, a) - o[a]) / (double)n[a];
        if (!(h[a] > 0)) return set_msg(msg, msg_len, "the lattice does not grow along +x, +y, +z", SDFIBM_ERR_ARG);
        ext = std::max(ext, std::fabs(P(last, a) - o[a]) + std::fabs(o[a]));
    }
    const double tol = rtol * ext;
    for (int64_t k = 0, i3 = 0; k < pz; ++k)
        for (int64_t j = 0; j < py; ++j)
            for (int64_t i = 0; i < px; ++i, ++i3) {
                const double want[3] = {o[0] + (double)i * h[0], o[1] + (double)j * h[1], o[2] + (double)k * h[2]};
                for (int a = 0; a < 3; ++a)
                    if (std::fabs(P(i3, a) - want[a]) > tol)
                        return set_msg(msg, msg_len, "point " + std::to_string(i3) + " is off the uniform lattice",
                                       SDFIBM_ERR_ARG);
            }
    mesh->nx = (int32_t)n[0];
    mesh->ny = (int32_t)n[1];
    mesh->nz = (int32_t)n[2];
    mesh->twod = n[2] == 1 ? 1 : 0;
    for (int a = 0; a < 3; ++a) {
        mesh->origin[a] = o[a];
        mesh->h[a] = h[a];
    }
    return SDFIBM_OK;
}
