// TEST DOUBLE: the entry points of sdfibm_cuda.h answered by the oracle (oracle/oracle.cpp, the FP64 CPU restatement)
// instead of the GPU, with every field in host memory, so that the C++ SolidCloud of include/sdfibm_cloud.hpp, its
// time-loop client and the Python SolidCloud (on CPU tensors) run on a machine without a GPU.  Linked with
// oracle.cpp and the host sources into a stand-in libsdfibm_cuda.so that only tests load; the product library is never
// replaced by it.  Entry points the tests do not use return SDFIBM_ERR_STATE.
#include <cstring>
#include <string>
#include <vector>

#include "sdfibm_cuda.h"
#include "sdfibm_mlp.h"

extern "C" {
void* oracle_create_uniform(const sdfibm_mesh_desc*, const sdfibm_solid_desc*, int, const sdfibm_options*, int);
void oracle_destroy(void*);
int oracle_interact(void*, double, double, const double*, double*, double*, double*, int32_t*, double*);
int oracle_evolve(void*, double, double);
int oracle_get_state(void*, sdfibm_solid_state*, int);
int oracle_set_state(void*, const sdfibm_solid_state*, int);
int64_t oracle_touched(void*, int, int64_t*, int8_t*, int64_t);
int oracle_fix_internal(void*, const int32_t*, double*);
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

/* FP64 fields in OpenFOAM's layout (U and Fs one x,y,z triple per cell), U rounded to FP32 first as the GPU does */
int sdfibm_cuda_interact_host64(sdfibm_ctx* c, double time, double dt, const double* U, double* As, double* Fs,
                                double* Ts, double* Ct, double* FT) {
    if (!c || !U || !As || !Fs || !Ts || !Ct) return SDFIBM_ERR_ARG;
    const int64_t N = c->N;
    for (int64_t i = 0; i < N; ++i)
        for (int a = 0; a < 3; ++a) c->U[(size_t)(a * N + i)] = (double)(float)U[3 * i + a];
    if (oracle_interact(c->oc, time, dt, c->U.data(), c->As.data(), c->Fs.data(), c->Ts.data(), c->Ct.data(), FT) !=
        0) {
        c->err = "oracle interact failed";
        return SDFIBM_ERR_ARG;
    }
    for (int64_t i = 0; i < N; ++i) {
        As[i] = (double)(float)c->As[(size_t)i];
        Ts[i] = (double)(float)c->Ts[(size_t)i];
        Ct[i] = (double)c->Ct[(size_t)i];
        for (int a = 0; a < 3; ++a) Fs[3 * i + a] = (double)(float)c->Fs[(size_t)(a * N + i)];
    }
    return SDFIBM_OK;
}

/* the device-pointer entry point: here every pointer is host memory */
int sdfibm_cuda_interact(sdfibm_ctx* c, double time, double dt, const float* U, float* As, float* Fs, float* Ts,
                         int32_t* Ct, double* FT) {
    return sdfibm_cuda_interact_host(c, time, dt, U, As, Fs, Ts, Ct, FT);
}

int sdfibm_cuda_fix_internal(sdfibm_ctx* c, const int32_t* Ct, float* U) {
    if (!c || !Ct || !U) return SDFIBM_ERR_ARG;
    std::vector<double> u(c->U.size());
    for (size_t i = 0; i < u.size(); ++i) u[i] = U[i];
    oracle_fix_internal(c->oc, Ct, u.data());
    for (size_t i = 0; i < u.size(); ++i) U[i] = (float)u[i];
    return SDFIBM_OK;
}

int sdfibm_cuda_touched(sdfibm_ctx* c, int32_t s, int64_t* cells, int8_t* types, int64_t capacity, int64_t* n) {
    if (!c || !n || s < 0 || s >= c->S) return SDFIBM_ERR_ARG;
    *n = oracle_touched(c->oc, s, cells, types, cells && types ? capacity : 0);
    return SDFIBM_OK;
}

int sdfibm_cuda_stats(sdfibm_ctx* c, int64_t* out, int32_t n) {
    if (!c || !out) return SDFIBM_ERR_ARG;
    for (int32_t i = 0; i < n; ++i) out[i] = 0;
    return SDFIBM_OK;
}

const char* sdfibm_cuda_version(void) { return "oracle stand-in (no GPU)"; }

int64_t sdfibm_abi_sizeof(int which) {
    switch (which) {
        case 0: return sizeof(sdfibm_mesh_desc);
        case 1: return sizeof(sdfibm_shape_desc);
        case 2: return sizeof(sdfibm_solid_desc);
        case 3: return sizeof(sdfibm_solid_state);
        case 4: return sizeof(sdfibm_options);
        case 5: return sizeof(sdfibm_mlp_data_desc);
        case 6: return sizeof(sdfibm_mlp_train_desc);
        default: return -1;
    }
}

// not answered here
int sdfibm_cuda_kernel_times(sdfibm_ctx*, const char**, double*, int32_t, int32_t*) { return SDFIBM_ERR_STATE; }
int sdfibm_cuda_touched_noalloc(const sdfibm_mesh_desc*, const sdfibm_solid_desc*, void*, int32_t*, int8_t*, int64_t,
                                int64_t*) {
    return SDFIBM_ERR_STATE;
}
int sdfibm_cuda_set_fraction_model(sdfibm_ctx*, const float*, float, float) { return SDFIBM_ERR_STATE; }
int sdfibm_cuda_tuning(sdfibm_ctx*, int32_t*, int32_t) { return SDFIBM_ERR_STATE; }
/* the solver's forcing update on host fields (every pointer is host memory here) */
int sdfibm_cuda_apply_forcing(sdfibm_ctx* c, double dt, const float* As, const float* Fs, const float* Ts, float* U,
                              float* T) {
    if (!c || !As || !Fs || !Ts || !U) return SDFIBM_ERR_ARG;
    const int64_t N = c->N;
    for (int64_t i = 0; i < 3 * N; ++i) U[i] = (float)((double)U[i] - (double)Fs[i] * dt);
    if (T)
        for (int64_t i = 0; i < N; ++i) T[i] = (float)((1.0 - (double)As[i]) * (double)T[i] + (double)Ts[i]);
    return SDFIBM_OK;
}
int sdfibm_cuda_create_polymesh(const double*, int64_t, const int32_t*, const int32_t*, int64_t, const int32_t*,
                                const int32_t*, int64_t, int32_t, const sdfibm_solid_desc*, int32_t,
                                const sdfibm_options*, void*, sdfibm_ctx**) {
    return SDFIBM_ERR_STATE;
}
int sdfibm_cuda_autotune(sdfibm_ctx*, double, const float*, float*, float*, float*, int32_t*, int32_t*) {
    return SDFIBM_ERR_STATE;
}
int sdfibm_mlp_dataset(uint64_t, int64_t, const sdfibm_mlp_data_desc*, float*, float*, double*, void*) {
    return SDFIBM_ERR_STATE;
}
int sdfibm_mlp_forward(const float*, const float*, int64_t, int64_t, float*, void*) { return SDFIBM_ERR_STATE; }
int sdfibm_mlp_loss_grad(const float*, const float*, const float*, int64_t, int64_t, float*, void*) {
    return SDFIBM_ERR_STATE;
}
int sdfibm_mlp_adam(float*, const float*, float*, float*, int32_t, float, void*) { return SDFIBM_ERR_STATE; }
int sdfibm_mlp_train(float*, const float*, const float*, int64_t, const sdfibm_mlp_train_desc*, float*, void*) {
    return SDFIBM_ERR_STATE;
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
