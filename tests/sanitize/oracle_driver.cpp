// Drives the oracle (oracle/oracle.cpp, test infrastructure) under -fsanitize=address,undefined, on CPU: both modes,
// 2-D and 3-D meshes, every shape, interact (serial and threaded), evolve with collisions, fixInternal, the mean
// field and the per-cell fractions, with solids inside, across the walls of and outside the mesh.  Exit 0 = clean.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <vector>

#include "../../include/sdfibm_host.h"

extern "C" {
void* oracle_create_uniform(const sdfibm_mesh_desc*, const sdfibm_solid_desc*, int, const sdfibm_options*, int);
void oracle_destroy(void*);
int64_t oracle_ncells(void*);
int oracle_interact(void*, double, double, const double*, double*, double*, double*, int32_t*, double*);
int oracle_interact_threads(void*, double, const double*, double*, double*, double*, int32_t*, double*, int);
int oracle_mean_field(void*, const sdfibm_shape_desc*, const double*, int32_t*, double*);
int64_t oracle_touched(void*, int, int64_t*, int8_t*, int64_t);
int oracle_evolve(void*, double, double);
int oracle_fix_internal(void*, const int32_t*, double*);
int oracle_get_state(void*, sdfibm_solid_state*, int);
int oracle_set_state(void*, const sdfibm_solid_state*, int);
double oracle_cell_fraction(void*, int, int64_t, int);
}

static sdfibm_shape_desc shape(int type, double a, double b, double c) {
    const double raw[8] = {a, b, c, 0, 0, 0, 0, 0};
    sdfibm_shape_desc s;
    sdfibm_host_make_shape(type, raw, nullptr, &s);
    return s;
}

int main() {
    long calls = 0;
    for (int twod = 0; twod <= 1; ++twod) {
        sdfibm_mesh_desc m{};
        m.nx = 24; m.ny = 20; m.nz = twod ? 1 : 16; m.twod = twod;
        m.origin[0] = 0; m.origin[1] = 0; m.origin[2] = twod ? -0.5 : 0;
        m.h[0] = m.h[1] = 1.0 / 20; m.h[2] = twod ? 1.0 : 1.0 / 20;
        std::vector<sdfibm_shape_desc> shapes;
        if (twod) {
            shapes = {shape(SDFIBM_SHAPE_CIRCLE, 0.1, 0, 0), shape(SDFIBM_SHAPE_ELLIPSE, 0.12, 0.05, 0),
                      shape(SDFIBM_SHAPE_RECTANGLE, 0.1, 0.04, 0), shape(SDFIBM_SHAPE_CIRCLE_TAIL, 0.08, 1.0, 0.03),
                      shape(SDFIBM_SHAPE_CIRCLE_TWOTAIL, 0.08, 1.0, 0.03), shape(SDFIBM_SHAPE_PLANE, 0, 0, 0)};
        } else {
            shapes = {shape(SDFIBM_SHAPE_SPHERE, 0.1, 0, 0), shape(SDFIBM_SHAPE_ELLIPSOID, 0.12, 0.05, 0.08),
                      shape(SDFIBM_SHAPE_BOX, 0.1, 0.04, 0.06), shape(SDFIBM_SHAPE_PLANE, 0, 0, 0)};
        }
        std::vector<sdfibm_solid_desc> solids;
        const double pos[5][3] = {{0.3, 0.3, 0.4}, {0.0, 0.5, 0.4}, {0.7, 0.95, 0.2}, {2.0, 2.0, 2.0}, {0.32, 0.34, 0.42}};
        int id = 0;
        for (auto& sh : shapes)
            for (int p = 0; p < 5; ++p) {
                double ps[3] = {pos[p][0], pos[p][1], twod ? 0.0 : pos[p][2]};
                const double eu[3] = {twod ? 0.0 : 10.0 * p, twod ? 0.0 : -7.0 * p, 33.0 * p};
                const double vel[3] = {0.1, -0.2, twod ? 0.0 : 0.05}, om[3] = {0, 0, 1.5};
                sdfibm_solid_desc d;
                sdfibm_host_make_solid(id++, &sh, 1.5, SDFIBM_MOTION_FREE, nullptr, SDFIBM_FORCER_NONE, nullptr, ps,
                                       eu, vel, om, &d);
                solids.push_back(d);
            }
        for (int faithful = 0; faithful <= 1; ++faithful)
            for (int method = 0; method <= 1; ++method) {
                sdfibm_options o;
                sdfibm_options_default(&o);
                o.fraction_method = method;
                o.subsample_n = 5;
                o.collision_mode = SDFIBM_COLLISION_SPHERES;
                o.gravity[1] = -9.81;
                void* h = oracle_create_uniform(&m, solids.data(), (int)solids.size(), &o, faithful);
                if (!h) { std::fprintf(stderr, "create failed\n"); return 3; }
                const int64_t N = oracle_ncells(h);
                std::vector<double> U(3 * N), As(N), Fs(3 * N), Ts(N), FT(6 * solids.size()), mean(3 * solids.size());
                std::vector<int32_t> Ct(N);
                for (int64_t c = 0; c < 3 * N; ++c) U[c] = std::sin(0.37 * c);
                for (int step = 0; step < 2; ++step, calls += 4) {
                    oracle_interact(h, 0.01 * step, 0.01, U.data(), As.data(), Fs.data(), Ts.data(), Ct.data(), FT.data());
                    oracle_evolve(h, 0.01 * step, 0.01);
                    oracle_fix_internal(h, Ct.data(), U.data());
                    oracle_interact_threads(h, 0.01, U.data(), As.data(), Fs.data(), Ts.data(), Ct.data(), FT.data(), 3);
                }
                oracle_mean_field(h, &shapes[0], U.data(), Ct.data(), mean.data());
                for (int s = 0; s < (int)solids.size(); ++s, ++calls) {
                    const int64_t n = oracle_touched(h, s, nullptr, nullptr, 0);
                    std::vector<int64_t> cells((size_t)std::max<int64_t>(n, 1));
                    std::vector<int8_t> types((size_t)std::max<int64_t>(n, 1));
                    oracle_touched(h, s, cells.data(), types.data(), n);
                    for (int64_t i = 0; i < n && i < 4; ++i) {
                        oracle_cell_fraction(h, s, cells[(size_t)i], 0);
                        oracle_cell_fraction(h, s, cells[(size_t)i], 1);
                    }
                }
                std::vector<sdfibm_solid_state> st(solids.size());
                oracle_get_state(h, st.data(), (int)st.size());
                oracle_set_state(h, st.data(), (int)st.size());
                oracle_destroy(h);
            }
    }
    std::printf("oracle_driver: %ld calls clean\n", calls);
    return 0;
}
