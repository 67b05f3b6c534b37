// Drives the host half of libsdfibm_cuda.so (sdfibm_gb300/csrc/host*.cpp: the solidDict, VOF-dict and blockMesh
// front ends, the OpenFOAM list readers, the field and restart writers) under -fsanitize=address,undefined, on CPU.
//
//   host_driver DIR [MUTATIONS [SEED]]
//
// DIR holds soliddict.txt, vofdict.txt, blockmesh.txt, field_ascii, field_binary, points_binary, faces_binary and
// faces_ascii.  Every entry point runs on the
// whole input, on every prefix of it and on byte-mutated copies, with output and message buffers allocated to their
// exact capacity (so a write past the end is reported).  Any sanitizer report aborts the process; exit 0 = clean.
#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/sdfibm_host.h"

static std::string slurp(const std::string& p) {
    std::ifstream f(p, std::ios::binary);
    std::stringstream ss;
    ss << f.rdbuf();
    return ss.str();
}

static uint64_t lcg(uint64_t& s) { return s = s * 6364136223846793005ULL + 1442695040888963407ULL; }

// the text entry points on one NUL-terminated input
static void parse_all(const std::string& t, int n_states) {
    std::vector<char> msg(48);  // short on purpose: long messages are cut
    sdfibm_solid_desc solids[32];
    int32_t n = 0, twod = 0;
    sdfibm_options opt;
    sdfibm_host_parse_soliddict(t.c_str(), 1.0, solids, 32, &n, &opt, &twod, msg.data(), (int32_t)msg.size());
    sdfibm_host_parse_soliddict(t.c_str(), 1.0, nullptr, 0, &n, &opt, &twod, nullptr, 0);
    sdfibm_host_parse_vofdict(t.c_str(), 1, solids, 32, &n, &twod, msg.data(), (int32_t)msg.size());
    sdfibm_host_parse_vofdict(t.c_str(), 0, solids, 1, &n, &twod, msg.data(), 1);
    sdfibm_mesh_desc mesh;
    sdfibm_host_parse_blockmesh(t.c_str(), &mesh, msg.data(), (int32_t)msg.size());
    int64_t len = 0;
    for (const char* path : {"meta/writeFrequency", "meta", "solids/a/pos", "", "/", "a//b"}) {
        if (sdfibm_host_soliddict_lookup(t.c_str(), path, nullptr, 0, &len) == SDFIBM_OK && len >= 0) {
            std::vector<char> b((size_t)len + 1);
            sdfibm_host_soliddict_lookup(t.c_str(), path, b.data(), (int64_t)b.size(), &len);
            std::vector<char> s((size_t)len);  // one byte short: must be refused, not overrun
            sdfibm_host_soliddict_lookup(t.c_str(), path, s.data(), (int64_t)s.size(), &len);
        }
    }
    std::vector<sdfibm_solid_state> st((size_t)std::max(1, n_states));
    for (auto& s : st) {
        std::memset(&s, 0, sizeof(s));
        s.quat[0] = 1.0;
        s.pos[0] = 0.25;
    }
    if (sdfibm_host_write_restart(t.c_str(), st.data(), n_states, 1, 6, "26/01/01 00:00:00", nullptr, 0, &len,
                                  msg.data(), (int32_t)msg.size()) == SDFIBM_OK) {
        std::vector<char> b((size_t)len + 1);
        sdfibm_host_write_restart(t.c_str(), st.data(), n_states, 1, 6, nullptr, b.data(), (int64_t)b.size(), &len,
                                  msg.data(), (int32_t)msg.size());
        std::vector<char> s((size_t)len);
        sdfibm_host_write_restart(t.c_str(), st.data(), n_states, 0, 17, "x", s.data(), (int64_t)s.size(), &len,
                                  msg.data(), (int32_t)msg.size());
    }
}

static void read_all(const std::string& f) {
    std::vector<char> msg(40);
    for (int kind = SDFIBM_FOAM_SCALAR; kind <= SDFIBM_FOAM_LABEL; ++kind) {
        int64_t n = 0;
        if (sdfibm_host_read_foam_list(f.data(), (int64_t)f.size(), kind, nullptr, 0, &n, msg.data(),
                                       (int32_t)msg.size()) != SDFIBM_OK)
            continue;
        const int64_t m = n < 0 ? 1 : n;
        std::vector<double> d((size_t)(3 * m + 1));
        std::vector<int32_t> l((size_t)(m + 1));
        void* out = kind == SDFIBM_FOAM_LABEL ? (void*)l.data() : (void*)d.data();
        sdfibm_host_read_foam_list(f.data(), (int64_t)f.size(), kind, out, m, &n, msg.data(), (int32_t)msg.size());
        if (m > 1) sdfibm_host_read_foam_list(f.data(), (int64_t)f.size(), kind, out, m - 1, &n, msg.data(), 8);
    }
    int64_t nf = 0, nl = 0;
    if (sdfibm_host_read_foam_faces(f.data(), (int64_t)f.size(), nullptr, 0, nullptr, 0, &nf, &nl, msg.data(),
                                    (int32_t)msg.size()) == SDFIBM_OK) {
        std::vector<int32_t> off((size_t)nf + 1), lab((size_t)nl + 1);
        sdfibm_host_read_foam_faces(f.data(), (int64_t)f.size(), off.data(), nf + 1, lab.data(), nl, &nf, &nl,
                                    msg.data(), (int32_t)msg.size());
        sdfibm_host_read_foam_faces(f.data(), (int64_t)f.size(), off.data(), nf, lab.data(), nl, &nf, &nl,
                                    msg.data(), (int32_t)msg.size());
    }
}

static void field_all(const std::string& f) {
    read_all(f);
    std::vector<char> msg(40);
    const int64_t n = 37;
    std::vector<double> v((size_t)n);
    for (int64_t i = 0; i < n; ++i) v[(size_t)i] = (double)i / 7.0;
    for (int fmt = -1; fmt <= 1; ++fmt) {
        int64_t len = 0;
        if (sdfibm_host_write_scalar_field(f.data(), (int64_t)f.size(), v.data(), n, fmt, 9, nullptr, 0, &len,
                                           msg.data(), (int32_t)msg.size()) != SDFIBM_OK)
            continue;
        std::vector<char> b((size_t)len + 1);
        sdfibm_host_write_scalar_field(f.data(), (int64_t)f.size(), v.data(), n, fmt, 9, b.data(), (int64_t)b.size(),
                                       &len, msg.data(), (int32_t)msg.size());
        std::vector<char> s((size_t)len);
        sdfibm_host_write_scalar_field(f.data(), (int64_t)f.size(), v.data(), n, fmt, 9, s.data(), (int64_t)s.size(),
                                       &len, msg.data(), (int32_t)msg.size());
        if (sdfibm_host_write_vector_field(f.data(), (int64_t)f.size(), v.data(), n / 3, fmt, 9, nullptr, 0, &len,
                                           msg.data(), (int32_t)msg.size()) == SDFIBM_OK) {
            std::vector<char> vb((size_t)len);
            sdfibm_host_write_vector_field(f.data(), (int64_t)f.size(), v.data(), n / 3, fmt, 9, vb.data(),
                                           (int64_t)vb.size(), &len, msg.data(), (int32_t)msg.size());
        }
    }
}

int main(int argc, char** argv) {
    if (argc < 2) {
        std::fprintf(stderr, "usage: host_driver DIR\n");
        return 2;
    }
    const std::string dir = argv[1];
    const std::string texts[3] = {slurp(dir + "/soliddict.txt"), slurp(dir + "/vofdict.txt"),
                                  slurp(dir + "/blockmesh.txt")};
    const std::string fields[5] = {slurp(dir + "/field_ascii"), slurp(dir + "/field_binary"),
                                   slurp(dir + "/points_binary"), slurp(dir + "/faces_binary"),
                                   slurp(dir + "/faces_ascii")};
    // states for the restart writer: as many as the full solidDict has solids
    sdfibm_solid_desc solids[32];
    int32_t ns = 0, twod = 0;
    sdfibm_options opt;
    if (sdfibm_host_parse_soliddict(texts[0].c_str(), 1.0, solids, 32, &ns, &opt, &twod, nullptr, 0) != SDFIBM_OK) {
        std::fprintf(stderr, "the solidDict input does not parse\n");
        return 3;
    }
    const int mutations = argc > 2 ? std::atoi(argv[2]) : 300;  // mutated copies per input
    uint64_t seed = argc > 3 ? (uint64_t)std::strtoull(argv[3], nullptr, 10) : 12345;
    long calls = 0;
    for (const std::string& t : texts) {
        for (size_t l = 0; l <= t.size(); ++l, ++calls) parse_all(t.substr(0, l), ns);
        for (int k = 0; k < mutations; ++k, ++calls) {
            std::string m = t;
            for (int j = 0; j < 3; ++j) m[(size_t)(lcg(seed) >> 33) % m.size()] = "{}();\"/ *0a.-#\n"[(lcg(seed) >> 33) % 15];
            parse_all(m, ns);
        }
    }
    for (const std::string& f : fields) {
        for (size_t l = 0; l <= f.size(); ++l, ++calls) field_all(f.substr(0, l));
        for (int k = 0; k < mutations; ++k, ++calls) {
            std::string m = f;
            for (int j = 0; j < 2; ++j) m[(size_t)(lcg(seed) >> 33) % m.size()] = (char)(lcg(seed) >> 56);
            field_all(m);
        }
    }
    // the lattice test on a small block and on points that are not one
    {
        std::vector<double> pts;
        for (int k = 0; k < 3; ++k)
            for (int j = 0; j < 3; ++j)
                for (int i = 0; i < 4; ++i) {
                    pts.push_back(0.5 * i);
                    pts.push_back(0.25 * j);
                    pts.push_back((double)k);
                }
        sdfibm_mesh_desc m;
        std::vector<char> msg(24);
        for (int64_t np = 0; np <= (int64_t)pts.size() / 3; ++np, ++calls)
            sdfibm_host_uniform_mesh(pts.data(), np, 12, 1e-9, &m, msg.data(), (int32_t)msg.size());
        for (int k = 0; k < 100; ++k, ++calls) {
            std::vector<double> q = pts;
            q[(size_t)(lcg(seed) >> 33) % q.size()] = (double)((lcg(seed) >> 40) % 7) - 3.0;
            sdfibm_host_uniform_mesh(q.data(), (int64_t)q.size() / 3, 12, 1e-9, &m, msg.data(), (int32_t)msg.size());
        }
    }
    // the record writers at every capacity below what they need
    std::vector<sdfibm_solid_state> st(3);
    for (auto& s : st) {
        std::memset(&s, 0, sizeof(s));
        s.quat[0] = 1.0;
    }
    const double mean[9] = {1, 2, 3, 4, 5, 6, 7, 8, 9};
    for (int twod2 = 0; twod2 <= 1; ++twod2) {
        int64_t need = 0, len = 0;
        sdfibm_host_format_state(0.5, twod2, st.data(), 3, nullptr, 0, &need);
        for (int64_t cap = 1; cap <= need + 1; ++cap, ++calls) {
            std::vector<char> b((size_t)cap);
            sdfibm_host_format_state(0.5, twod2, st.data(), 3, b.data(), cap, &len);
        }
        sdfibm_host_format_mean_field(mean, 3, nullptr, 0, &need);
        for (int64_t cap = 1; cap <= need + 1; ++cap, ++calls) {
            std::vector<char> b((size_t)cap);
            sdfibm_host_format_mean_field(mean, 3, b.data(), cap, &len);
        }
    }
    std::printf("host_driver: %ld calls clean\n", calls);
    return 0;
}
