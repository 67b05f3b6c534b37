// Learned cut-cell fraction: shared declarations of the MLP kernels (mlp.cu) and of their users (classify.cu,
// capi.cu).  The network and its parameter layout are described in include/sdfibm_mlp.h.
#pragma once
#include <cstdint>

#include "../../include/sdfibm_mlp.h"
#include "device_math.cuh"

namespace sdfibm_dev {

constexpr int MLP_IN = SDFIBM_MLP_NIN;       // 11 features
constexpr int MLP_H = SDFIBM_MLP_NHIDDEN;    // 64 hidden units per layer
constexpr int MLP_NPARAM = SDFIBM_MLP_NPARAM;
constexpr int MLP_OFF_W1 = 0;
constexpr int MLP_OFF_B1 = MLP_OFF_W1 + MLP_H * MLP_IN;
constexpr int MLP_OFF_W2 = MLP_OFF_B1 + MLP_H;
constexpr int MLP_OFF_B2 = MLP_OFF_W2 + MLP_H * MLP_H;
constexpr int MLP_OFF_W3 = MLP_OFF_B2 + MLP_H;
constexpr int MLP_OFF_B3 = MLP_OFF_W3 + MLP_H;
static_assert(MLP_OFF_B3 + 1 == MLP_NPARAM, "parameter layout");

constexpr int MLP_TILE = 128;     // cells per tensor-core tile (the MMA's M)
constexpr int MLP_THREADS = 128;  // one thread per cell of the tile (= tensor-memory lane)

// Features of a cut cell from its 8 vertex distances (cellPoints order of a hex) and 1/h: phi/h, then the unit
// trilinear gradient at the centre.  FP32 with a fixed operation order (the oracle repeats it).
__host__ __device__ inline void cell_features(const float* ph, float inv_h, float* f) {
    for (int v = 0; v < 8; ++v) f[v] = ph[v] * inv_h;
    const float gx = 0.25f * (((f[1] - f[0]) + (f[3] - f[2])) + ((f[5] - f[4]) + (f[7] - f[6])));
    const float gy = 0.25f * (((f[2] - f[0]) + (f[3] - f[1])) + ((f[6] - f[4]) + (f[7] - f[5])));
    const float gz = 0.25f * (((f[4] - f[0]) + (f[5] - f[1])) + ((f[6] - f[2]) + (f[7] - f[3])));
    const float gn = sqrtf(gx * gx + gy * gy + gz * gz);
    if (gn > 1e-12f) {
        f[8] = gx / gn; f[9] = gy / gn; f[10] = gz / gn;
    } else {
        f[8] = 0.f; f[9] = 0.f; f[10] = 0.f;
    }
}

// Confidence band: a cell is inside when its distance field is close to linear over the cell (sum of the six face
// twists |f_a - f_b - f_c + f_d| at most tau_twist) and its trilinear gradient has length within tau_grad of 1.
__host__ __device__ inline bool in_band(const float* f, float tau_twist, float tau_grad) {
    const float tw = fabsf(f[0] - f[1] - f[2] + f[3]) + fabsf(f[4] - f[5] - f[6] + f[7]) +
                     fabsf(f[0] - f[1] - f[4] + f[5]) + fabsf(f[2] - f[3] - f[6] + f[7]) +
                     fabsf(f[0] - f[2] - f[4] + f[6]) + fabsf(f[1] - f[3] - f[5] + f[7]);
    const float gx = 0.25f * (((f[1] - f[0]) + (f[3] - f[2])) + ((f[5] - f[4]) + (f[7] - f[6])));
    const float gy = 0.25f * (((f[2] - f[0]) + (f[3] - f[1])) + ((f[6] - f[4]) + (f[7] - f[5])));
    const float gz = 0.25f * (((f[4] - f[0]) + (f[5] - f[1])) + ((f[6] - f[2]) + (f[7] - f[3])));
    const float gn = sqrtf(gx * gx + gy * gy + gz * gz);
    return tw <= tau_twist && fabsf(gn - 1.f) <= tau_grad;
}

// Inference over a list of cells.  Standalone mode (ref == nullptr): out[c] = predicted fraction.  Coupling mode:
// cells inside the band write alpha[ref], the others are appended to the fallback list.
struct MlpInferArgs {
    const float* params;     // FP32 [MLP_NPARAM], device
    const float* feat;       // [MLP_IN][stride]
    int64_t stride;
    int64_t n;               // cell count (standalone mode)
    const int32_t* n_dev;    // cell count written by the classify pass (coupling mode), or nullptr
    float* out;
    const int32_t* ref_solid;   // coupling mode: solid of each cell
    const int64_t* ref_index;   // coupling mode: index into the fraction scratch
    float* alpha;
    int32_t* fb_list;        // positions (into feat) of cells left to the fallback
    int32_t* fb_count;
    float tau_twist, tau_grad;
    int32_t* error;          // set to SDFIBM_MLP_ERR_TIMEOUT when an MMA completion is not seen in time
};

struct MlpGradArgs {
    const float* params;
    const float* feat;       // [MLP_IN][stride]
    const float* label;      // [n]
    int64_t stride;
    int64_t n;               // cells of this batch
    float scale;             // 2 / (cells in the batch): d loss / d a = scale * (a - y)
    float* grad;             // FP32 [MLP_NPARAM + 1], accumulated with atomics; the last entry sums (a - y)^2
    int32_t* error;
};

void launch_mlp_infer(const MlpInferArgs& a, int grid, cudaStream_t st);
void launch_mlp_grad(const MlpGradArgs& a, int grid, cudaStream_t st);
int mlp_sm_count();

}  // namespace sdfibm_dev
