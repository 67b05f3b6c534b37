// Device view of an explicit polyMesh (poly.hpp) and the per-call work space of the unstructured coupling path
// (poly.cu), shared with the C ABI (capi.cu).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "kernels.cuh"

namespace sdfibm_dev {

struct PolyK {
    int32_t ncells, npoints, nfaces, twod;
    const double* points;     // [npoints][3]
    const int32_t* face_off;  // face -> points
    const int32_t* face_lab;
    const int32_t* cf_off;    // cell -> faces (owned, then neighbour faces)
    const int32_t* cf;
    const int32_t* cp_off;    // cell -> points, ascending
    const int32_t* cp;
    const int32_t* cc_off;    // cell -> face neighbours
    const int32_t* ccl;
    const double* Cf;         // [nfaces][3] face centres
    const double* Sf;         // [nfaces][3] face area vectors
    const double* Cc;         // [ncells][3] cell centres
    const double* Vc;         // [ncells] cell volumes
};

struct PolyWork {
    uint32_t* visited;  // [S][words]: cells the search of each solid has reached
    int64_t words;
    int32_t* queue;     // [S][qcap]: touched cells of each solid in search order
    int8_t* qtype;      // [S][qcap]: their types (1 ALL_INSIDE, 2 CENTER_INSIDE, 3 CENTER_OUTSIDE)
    int32_t* count;     // [S]: touched cells of each solid
    int64_t qcap;
    double* acc;        // [N][5]: sums over the solids of As, Ts, Fs.x, Fs.y, Fs.z
    int32_t* claim;     // [N]: largest 4 * solid + type over the solids touching the cell (-1: none)
    int32_t* err;       // first device error (DeviceError)
};

__global__ void poly_enum_kernel(PolyK m, const SolidK* sk, const sdfibm_solid_state* st, PolyWork w);
__global__ void poly_couple_kernel(PolyK m, const SolidK* sk, const sdfibm_solid_state* st, PolyWork w, const float* U,
                                   double* ftacc, const StepParams* step);
__global__ void poly_finalize_kernel(PolyWork w, int32_t N, float* As, float* Fs, float* Ts, int32_t* Ct);
__global__ void poly_fix_kernel(PolyK m, const sdfibm_solid_state* st, int S, const int32_t* Ct, float* U);

}  // namespace sdfibm_dev
