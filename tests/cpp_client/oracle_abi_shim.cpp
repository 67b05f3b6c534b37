// TEST DOUBLE: the host-field entry points of sdfibm_cuda.h answered by the oracle (oracle/oracle.cpp, the FP64 CPU
// restatement) instead of the GPU, so that the C++ SolidCloud of include/sdfibm_cloud.hpp and its time-loop client
// run on a machine without a GPU.  Linked with oracle.cpp and host.cpp into a stand-in libsdfibm_cuda.so that only
// tests load; the product library is never replaced by it.
#include <cstring>
#include <string>
#include <vector>

#include "sdfibm_cuda.h"

extern "C" {
void* oracle_create_uniform(const sdfibm_mesh_desc*, const sdfibm_solid_desc*, int, const sdfibm_options*, int);
void oracle_destroy(void*);
int oracle_interact(void*, double, double, const double*, double*, double*, double*, int32_t*, double*);
int oracle_evolve(void*, double, double);
int oracle_get_state(void*, sdfibm_solid_state*, int);
int oracle_set_state(void*, const sdfibm_solid_state*, int);
}

struct sdfibm_ctx {
    void* oc = nullptr;
    int32_t S = 0;
    int64_t N = 0;
    std::string err;
    std::vector<double> U, As, Fs, Ts;  // the oracle's FP64 fields, kept between calls (its sparse reset reads them)
    std::vector<int32_t> Ct;            // like the device copy: the caller's array receives it whole every call
};

extern "C" {

int sdfibm_cuda_create(const sdfibm_mesh_desc* mesh, const sdfibm_solid_desc* solids, int32_t n,
                       const sdfibm_options* opt, void*, sdfibm_ctx** out) {
    if (!out || !mesh || !opt || n < 0) return SDFIBM_ERR_ARG;
    auto* c = new sdfibm_ctx();
    c->S = n;
    c->N = (int64_t)mesh->nx * mesh->ny * mesh->nz;
    c->oc = oracle_create_uniform(mesh, solids, n, opt, 0);
    if (!c->oc) {
        delete c;
        return SDFIBM_ERR_ARG;
    }
    c->U.assign((size_t)(3 * c->N), 0.0);
    c->As.assign((size_t)c->N, 0.0);
    c->Fs.assign((size_t)(3 * c->N), 0.0);
    c->Ts.assign((size_t)c->N, 0.0);
    c->Ct.assign((size_t)c->N, 0);
    *out = c;
    return SDFIBM_OK;
}

int sdfibm_cuda_interact_host(sdfibm_ctx* c, double time, double dt, const float* U, float* As, float* Fs, float* Ts,
                              int32_t* Ct, double* FT) {
    if (!c || !U || !As || !Fs || !Ts || !Ct) return SDFIBM_ERR_ARG;
    for (size_t i = 0; i < c->U.size(); ++i) c->U[i] = U[i];
    if (oracle_interact(c->oc, time, dt, c->U.data(), c->As.data(), c->Fs.data(), c->Ts.data(), c->Ct.data(), FT) !=
        0) {
        c->err = "oracle interact failed";
        return SDFIBM_ERR_ARG;
    }
    for (int64_t i = 0; i < c->N; ++i) {
        As[i] = (float)c->As[(size_t)i];
        Ts[i] = (float)c->Ts[(size_t)i];
        Ct[i] = c->Ct[(size_t)i];
    }
    for (size_t i = 0; i < c->Fs.size(); ++i) Fs[i] = (float)c->Fs[i];
    return SDFIBM_OK;
}

int sdfibm_cuda_evolve(sdfibm_ctx* c, double time, double dt) { return c ? oracle_evolve(c->oc, time, dt) : 1; }

int sdfibm_cuda_get_solids(sdfibm_ctx* c, sdfibm_solid_state* out, int32_t n) {
    if (!c || !out || n != c->S) return SDFIBM_ERR_ARG;
    return oracle_get_state(c->oc, out, n);
}

int sdfibm_cuda_set_solids(sdfibm_ctx* c, const sdfibm_solid_state* in, int32_t n) {
    if (!c || !in || n != c->S) return SDFIBM_ERR_ARG;
    return oracle_set_state(c->oc, in, n);
}

const char* sdfibm_cuda_last_error(const sdfibm_ctx* c) { return c ? c->err.c_str() : "null context"; }

void sdfibm_cuda_destroy(sdfibm_ctx* c) {
    if (!c) return;
    oracle_destroy(c->oc);
    delete c;
}

}  // extern "C"
