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

// Planar prior of the model: the exact solid fraction of the cell under the plane fitted to its vertex distances,
// phi(x) = mean(f) + g . (x - 1/2) in cell units with g the trilinear gradient (inside where phi < 0).  The cube-plane
// volume is the closed form of Scardovelli & Zaleski, "Analytical relations connecting linear interfaces and volume
// fractions in rectangular grids", J. Comput. Phys. 164 (2000): normal reflected to the positive octant and sorted,
// plane constant normalised by the normal's 1-norm, symmetric about 1/2.
__host__ __device__ inline float plane_fraction(const float* f) {
    float n[3];
    n[0] = 0.25f * (((f[1] - f[0]) + (f[3] - f[2])) + ((f[5] - f[4]) + (f[7] - f[6])));
    n[1] = 0.25f * (((f[2] - f[0]) + (f[3] - f[1])) + ((f[6] - f[4]) + (f[7] - f[5])));
    n[2] = 0.25f * (((f[4] - f[0]) + (f[5] - f[1])) + ((f[6] - f[2]) + (f[7] - f[3])));
    const float mean = 0.125f * (((f[0] + f[1]) + (f[2] + f[3])) + ((f[4] + f[5]) + (f[6] + f[7])));
    float d = 0.5f * ((n[0] + n[1]) + n[2]) - mean;  // inside: n . x < d
    for (int a = 0; a < 3; ++a)
        if (n[a] < 0.f) { d -= n[a]; n[a] = -n[a]; }  // x_a -> 1 - x_a
    const float s = (n[0] + n[1]) + n[2];
    if (!(s > 0.f)) return d > 0.f ? 1.f : 0.f;
    float al = d / s;
    if (al <= 0.f) return 0.f;
    if (al >= 1.f) return 1.f;
    float m1 = n[0] / s, m2 = n[1] / s, m3 = n[2] / s, t;
    if (m1 > m2) { t = m1; m1 = m2; m2 = t; }
    if (m2 > m3) { t = m2; m2 = m3; m3 = t; }
    if (m1 > m2) { t = m1; m1 = m2; m2 = t; }
    const bool flip = al > 0.5f;
    if (flip) al = 1.f - al;
    const float m12 = m1 + m2;
    float v;
    if (al < m1) v = al * al * al / (6.f * m1 * m2 * m3);
    else if (al < m2) v = al * (al - m1) / (2.f * m2 * m3) + m1 * m1 / (6.f * m2 * m3);
    else if (al < fminf(m3, m12))
        v = (al * al * (3.f * m12 - al) + m1 * m1 * (m1 - 3.f * al) + m2 * m2 * (m2 - 3.f * al)) / (6.f * m1 * m2 * m3);
    else if (m3 < m12)
        v = (al * al * (3.f - 2.f * al) + m1 * m1 * (m1 - 3.f * al) + m2 * m2 * (m2 - 3.f * al) +
             m3 * m3 * (m3 - 3.f * al)) / (6.f * m1 * m2 * m3);
    else v = (2.f * al - m12) / (2.f * m3);
    v = fminf(fmaxf(v, 0.f), 1.f);
    return flip ? 1.f - v : v;
}

// sum over the six faces of |f_a - f_b - f_c + f_d| (zero for a linear field)
__host__ __device__ inline float face_twist(const float* f) {
    return fabsf(f[0] - f[1] - f[2] + f[3]) + fabsf(f[4] - f[5] - f[6] + f[7]) + fabsf(f[0] - f[1] - f[4] + f[5]) +
           fabsf(f[2] - f[3] - f[6] + f[7]) + fabsf(f[0] - f[2] - f[4] + f[6]) + fabsf(f[1] - f[3] - f[5] + f[7]);
}

// Output of the model: a = sigmoid(logit(clamp(plane_fraction)) + gate * o) with o the network's output and
// gate = tw / (1 + tw), tw = face_twist: a linear distance field takes the exact planar fraction and the network
// corrects for curvature.  prior_logit and gate of a cell:
constexpr float MLP_PRIOR_CLAMP = 1e-4f;
__device__ inline void model_prior(const float* f, float& prior_logit, float& gate) {
    const float v = fminf(fmaxf(plane_fraction(f), MLP_PRIOR_CLAMP), 1.f - MLP_PRIOR_CLAMP);
    prior_logit = __logf(v / (1.f - v));
    const float tw = face_twist(f);
    gate = tw / (1.f + tw);
}

// Confidence band: a cell is inside when its distance field is close to linear over the cell (sum of the six face
// twists |f_a - f_b - f_c + f_d| at most tau_twist) and its trilinear gradient has length within tau_grad of 1.
__host__ __device__ inline bool in_band(const float* f, float tau_twist, float tau_grad) {
    const float tw = face_twist(f);
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

void mlp_prepare();
void launch_mlp_infer(const MlpInferArgs& a, int grid, cudaStream_t st);
void launch_mlp_grad(const MlpGradArgs& a, int grid, cudaStream_t st);
int mlp_sm_count();

}  // namespace sdfibm_dev
