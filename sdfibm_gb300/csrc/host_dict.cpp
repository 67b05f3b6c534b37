// The solidDict front ends of include/sdfibm_host.h: SolidCloud::initFromDictionary (src/solidcloud.cpp:14-206),
// entry and shape lookups, the restart dictionary of SolidCloud::saveRestart (src/solidcloud.cpp:616-665), the
// VOF initializer's dictionary (tool_vof/solidcloud.cpp:12-112) and the uniform block of a blockMeshDict.
#include "host_text.hpp"

using namespace sdfibm_host_text;

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
