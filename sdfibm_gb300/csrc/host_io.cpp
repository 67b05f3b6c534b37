// The file formats of include/sdfibm_host.h: the cloud.out records of SolidCloud::saveState and the meanfield.out
// line of writeMeanField (src/solidcloud.cpp:578-614, 303-313, src/solid.cpp:5-29), quaternion::eulerAngles(XYZ),
// OpenFOAM vol field files with a new internalField, the lists of polyMesh and field files, and the uniform mesh
// of a single-block point lattice.
#include "host_text.hpp"

using namespace sdfibm_host_text;

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
