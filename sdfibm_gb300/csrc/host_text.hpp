// Internal to the host half of libsdfibm_cuda.so (host_dict.cpp, host_io.cpp): the OpenFOAM dictionary
// lexer and tree of the solidDict front end, number formatting of the reference's streams, and the list
// scanning of OpenFOAM files.  Not installed; include/sdfibm_host.h is the interface.
#pragma once

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

namespace sdfibm_host_text {

// ---- solidDict grammar (SolidCloud::initFromDictionary src/solidcloud.cpp:14-206) ------------------------------

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

inline std::shared_ptr<Node> parse_dict(Lexer& lx, bool top) {
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

inline double to_num(const std::string& t) {
    size_t p = 0;
    double v = std::stod(t, &p);
    if (p != t.size()) throw std::runtime_error("not a number: " + t);
    return v;
}
inline double scalar_of(const Node& d, const std::string& k) {
    const Node* n = d.find(k);
    if (!n || n->is_dict || n->tokens.empty()) throw std::runtime_error("missing scalar " + k);
    return to_num(n->tokens.back());  // a dimensioned entry keeps its value last
}
inline bool vector_of(const Node& d, const std::string& k, double out[3]) {
    const Node* n = d.find(k);
    if (!n) return false;
    std::vector<double> v;
    for (auto& t : n->tokens)
        if (t != "(" && t != ")") v.push_back(to_num(t));
    if (v.size() != 3) throw std::runtime_error("bad vector " + k);
    for (int a = 0; a < 3; ++a) out[a] = v[a];
    return true;
}
inline std::string word_of(const Node& d, const std::string& k) {
    const Node* n = d.find(k);
    if (!n || n->is_dict || n->tokens.size() != 1) throw std::runtime_error("missing word " + k);
    return n->tokens[0];
}
inline bool bool_of(const Node& d, const std::string& k) {
    const std::string w = word_of(d, k);
    if (w == "1" || w == "true" || w == "yes" || w == "on" || w == "y" || w == "t") return true;
    if (w == "0" || w == "false" || w == "no" || w == "off" || w == "n" || w == "f" || w == "none") return false;
    throw std::runtime_error("bad bool " + k);
}

// The shapes library of a solidDict: one ShapeFactory::create per entry of "shapes".  keep_first: the coupling's
// EntityLibrary::emplace keeps the first of duplicate names (src/solidcloud.cpp:66, src/entitylibrary.h:22); the
// VOF initializer assigns, keeping the last (tool_vof/solidcloud.cpp:57-60).
inline std::map<std::string, sdfibm_shape_desc> parse_shapes(const Node& shapes_dict, bool keep_first) {
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


// ---- state records and restart dictionary ------------------------------------------------------------------------------
//   euler      OpenFOAM 12 quaternion::eulerAngles(quaternion::XYZ), used by src/solid.cpp:12 and
//              src/solidcloud.cpp:638: for q = qx(a) qy(b) qz(c), R = Rx(a) Ry(b) Rz(c), so
//              R02 = sin b, R12 = -sin a cos b, R22 = cos a cos b, R01 = -cos b sin c, R00 = cos b cos c
//   state      SolidCloud::saveState / operator<<(SolidCloud) src/solidcloud.cpp:578-614 on a stream set to
//              std::scientific (src/solidcloud.cpp:235-236), operator<<(Solid) and write2D src/solid.cpp:5-29
//   restart    SolidCloud::saveRestart src/solidcloud.cpp:616-665: dictionary::set of pos / vel / euler / omega in
//              every solids entry, then dictionary::write of the whole tree in OpenFOAM's ascii layout

inline void euler_xyz(const double* q, double* e) {
    const double w = q[0], x = q[1], y = q[2], z = q[3];
    e[0] = std::atan2(-2 * (y * z - w * x), w * w - x * x - y * y + z * z);
    e[1] = std::asin(2 * (x * z + w * y));
    e[2] = std::atan2(-2 * (x * y - w * z), w * w + x * x - y * y - z * z);
}

inline void put_sci(std::string& out, double v) {  // std::ostream << double under std::scientific, precision 6
    char b[40];
    std::snprintf(b, sizeof(b), "%.6e", v);
    out += b;
}

inline std::string put_g(double v, int prec) {  // std::ostream << double in the default float format
    char b[48];
    std::snprintf(b, sizeof(b), "%.*g", prec, v);
    return b;
}

// OpenFOAM's tokeniser reads a word that starts like a number as a label (digits only) or a scalar
inline bool is_number_token(const std::string& t) {
    if (t.empty()) return false;
    const char c = t[0];
    if (!(std::isdigit((unsigned char)c) || c == '-' || c == '+' || c == '.')) return false;
    char* end = nullptr;
    std::strtod(t.c_str(), &end);
    return end == t.c_str() + t.size();
}
inline bool is_label_token(const std::string& t) {
    size_t i = (t[0] == '-' || t[0] == '+') ? 1 : 0;
    if (i == t.size() || t.size() - i > 18) return false;
    for (; i < t.size(); ++i)
        if (!std::isdigit((unsigned char)t[i])) return false;
    return true;
}
inline std::string format_token(const std::string& t, bool quoted, int prec) {
    if (quoted) return "\"" + t + "\"";
    if (!is_number_token(t)) return t;
    if (is_label_token(t)) return std::to_string(std::stoll(t));
    return put_g(std::strtod(t.c_str(), nullptr), prec);
}

// dictionary::set: replace the value of an existing keyword in place, else append the entry
inline void set_vector(Node& d, const std::string& key, const double v[3], int prec) {
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
inline void write_dict(std::string& out, const Node& d, int level, int prec) {
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

inline const char* const kRestartHeader =
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

inline int emit(const std::string& text, char* buf, int64_t cap, int64_t* len) {
    if (len) *len = (int64_t)text.size();
    if (!buf) return cap > 0 ? SDFIBM_ERR_ARG : SDFIBM_OK;
    if (cap <= (int64_t)text.size()) return SDFIBM_ERR_CAPACITY;
    std::memcpy(buf, text.data(), text.size());
    buf[text.size()] = 0;
    return SDFIBM_OK;
}


// ---- VOF initializer front end (tool_vof) ------------------------------------------------------------------------------
//   solidDict   tool_vof/solidcloud.cpp:12-112: meta.on_twod, the shapes library, material rho = 1, every "solids"
//               entry as Solid(i, pos, identity) + euler + shape; the example's "planes" entries follow the solids
//   blockMesh   a single uniform hex block (the mesh of the uniform-grid path)
//   field file  the internalField of a volScalarField rewritten in the file's own format (ascii or binary), the rest
//               of the file kept as it is (IOobject MUST_READ + field.write(), tool_vof/solidcloud.cpp:143-164)

inline void read_vof_entries(const Node& list, const std::map<std::string, sdfibm_shape_desc>& shapes, bool twod,
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

inline int set_msg(char* msg, int32_t msg_len, const std::string& m, int code) {
    if (msg && msg_len > 0) {
        std::strncpy(msg, m.c_str(), msg_len - 1);
        msg[msg_len - 1] = 0;
    }
    return code;
}

// the value tokens of a list entry of a dictionary that the solidDict grammar does not cover (blockMeshDict's
// "boundary" holds sub-dictionaries inside a list): scan for `key` at brace depth 0 and collect to its ';'
inline bool raw_entry(const std::string& src, const std::string& key, std::vector<std::string>& toks) {
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


// ---- OpenFOAM list files (polyMesh points / faces / owner / neighbour, field internalFields) ----------------------------
// Layout of OpenFOAM's IOstream lists: "N" then "(" and the N elements, then ")"; in binary files the elements are the
// raw little-endian scalars (8 bytes) or labels (4 bytes, 32-bit label builds such as the reference's) between the
// parentheses; a faceCompactList is two lists (N + 1 offsets, then the vertex labels).

struct FoamHeader {
    bool binary = false;
    std::string cls;
    size_t body = 0;  // offset after the header's closing brace
};

inline FoamHeader foam_header(const std::string& src) {
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

inline void skip_blank(const std::string& s, size_t& p) {
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

inline std::string next_word(const std::string& s, size_t& p) {
    skip_blank(s, p);
    const size_t b = p;
    while (p < s.size() && !std::isspace((unsigned char)s[p]) && s[p] != '(' && s[p] != ')' && s[p] != ';') ++p;
    return s.substr(b, p - b);
}

// "N (" at p: returns N and leaves p after the '('
inline int64_t list_open(const std::string& s, size_t& p) {
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
inline void read_items(const std::string& s, size_t& p, bool binary, int64_t n, int width, bool labels, double* dout,
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
inline size_t internal_field(const std::string& src, size_t from) {
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


}  // namespace sdfibm_host_text
