// Learned cut-cell fraction: shared declarations of the MLP kernels (mlp.cu) and of their users (classify.cu,
// capi.cu).  The network and its parameter layout are described in include/sdfibm_mlp.h.
#pragma once
#include <cstdint>

#include "../../include/sdfibm_mlp.h"
#include "device_math.cuh"

namespace sdfibm_dev {

constexpr int MLP_IN = SDFIBM_MLP_NIN;       // 16 network inputs
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

// Solid fraction of a cell (or sub-cell) under the plane fitted to its 8 corner distances f (cellPoints order, any
// common scale): phi(x) = mean(f) + g . (x - 1/2) in cell units with g the trilinear gradient (inside where phi < 0).
// The cube-plane volume is the closed form of Scardovelli & Zaleski, "Analytical relations connecting linear
// interfaces and volume fractions in rectangular grids", J. Comput. Phys. 164 (2000): normal reflected to the positive
// octant and sorted, plane constant normalised by the normal's 1-norm, symmetric about 1/2.
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

// ---- model inputs of one cut cell: the 5^3 distance stencil and its sub-cell planar reconstructions ---------------
constexpr int STENCIL_N = 5;                       // lattice points per axis (spacing h/4)
constexpr int STENCIL_PTS = STENCIL_N * STENCIL_N * STENCIL_N;
constexpr float MLP_PRIOR_CLAMP = 1e-4f;
constexpr int MLP_NFEAT = SDFIBM_MLP_NFEAT;        // 16 inputs + the prior logit

__device__ __forceinline__ float clamp_frac(float v) {
    return fminf(fmaxf(v, MLP_PRIOR_CLAMP), 1.f - MLP_PRIOR_CLAMP);
}
__device__ __forceinline__ float logit_frac(float v) { return __logf(v / (1.f - v)); }

// stencil index of lattice point (i, j, k), 0 <= i, j, k <= 4
__host__ __device__ constexpr int stn(int i, int j, int k) { return i + STENCIL_N * (j + STENCIL_N * k); }

// stencil point of network input f < 15: the 8 vertices (cellPoints order), the face centres -x +x -y +y -z +z, the
// centre
__device__ __forceinline__ int input_point(int f) {
    if (f < 8) return stn(4 * (f & 1), 4 * ((f >> 1) & 1), 4 * (f >> 2));
    if (f < 14) {
        const int a = (f - 8) >> 1, e = 4 * ((f - 8) & 1);
        return stn(a == 0 ? e : 2, a == 1 ? e : 2, a == 2 ? e : 2);
    }
    return stn(2, 2, 2);
}

// planar fraction of the sub-cube with lowest corner v0 and corner spacing d (in lattice steps)
__device__ __forceinline__ float subcell_fraction(const float* sphi, int v0, int d) {
    const float f[8] = {sphi[v0], sphi[v0 + d], sphi[v0 + STENCIL_N * d], sphi[v0 + STENCIL_N * d + d],
                        sphi[v0 + STENCIL_N * STENCIL_N * d], sphi[v0 + STENCIL_N * STENCIL_N * d + d],
                        sphi[v0 + STENCIL_N * STENCIL_N * d + STENCIL_N * d],
                        sphi[v0 + STENCIL_N * STENCIL_N * d + STENCIL_N * d + d]};
    return plane_fraction(f);
}

// The model inputs of one cell, computed by all 32 lanes of a warp together.  The cell's frame: lattice point
// (i, j, k) lies at world offset (bx + i*qx, by + j*qy, bz + k*qz) from the solid centre (q = h/4 per axis, FP32), its
// local coordinates are M times that offset.  sphi: 125 floats of shared memory of this warp.  Every lane returns
// P4 and P2 (unclamped); lane f < 16 returns input f in *feat, lane 16 the prior logit(clamp(P4)).
struct StencilOut {
    float p4, p2, feat;
};
__device__ inline StencilOut cell_stencil(const ShapeK& sh, const float* M, float bx, float by, float bz, float qx,
                                          float qy, float qz, float inv_h, float* sphi) {
    const int lane = threadIdx.x & 31;
    for (int p = lane; p < STENCIL_PTS; p += 32) {
        const int i = p % STENCIL_N, j = (p / STENCIL_N) % STENCIL_N, k = p / (STENCIL_N * STENCIL_N);
        const float dx = bx + (float)i * qx, dy = by + (float)j * qy, dz = bz + (float)k * qz;
        const float lx = __fmaf_rn(M[0], dx, __fmaf_rn(M[1], dy, M[2] * dz));
        const float ly = __fmaf_rn(M[3], dx, __fmaf_rn(M[4], dy, M[5] * dz));
        const float lz = __fmaf_rn(M[6], dx, __fmaf_rn(M[7], dy, M[8] * dz));
        sphi[p] = sdf32(sh, lx, ly, lz) * inv_h;
    }
    __syncwarp();
    // the 64 sub-cells of the 4^3 division: lane l takes sub-cells l and l + 32; lanes 0..7 the 8 of the 2^3 one
    float s4 = 0.f, s2 = 0.f;
#pragma unroll
    for (int r = 0; r < 2; ++r) {
        const int sc = lane + 32 * r;
        s4 += subcell_fraction(sphi, stn(sc & 3, (sc >> 2) & 3, sc >> 4), 1);
    }
    if (lane < 8) s2 = subcell_fraction(sphi, stn(2 * (lane & 1), 2 * ((lane >> 1) & 1), 2 * (lane >> 2)), 2);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        s4 += __shfl_xor_sync(0xffffffffu, s4, o);
        s2 += __shfl_xor_sync(0xffffffffu, s2, o);
    }
    StencilOut out;
    out.p4 = s4 * (1.f / 64.f);
    out.p2 = s2 * (1.f / 8.f);
    // network inputs: 8 vertices, 6 face centres, centre, logit(P2); then the prior logit(P4)
    float f = 0.f;
    if (lane < 15) f = sphi[input_point(lane)];
    else if (lane == 15) f = logit_frac(clamp_frac(out.p2));
    else if (lane == 16) f = logit_frac(clamp_frac(out.p4));
    out.feat = f;
    __syncwarp();
    return out;
}

// Confidence band: the network's answer is kept where the two planar reconstructions agree (|P4 - P2| at most
// tau_refine: the sub-cell planes resolve the surface) and the solid spans at least rho_min cells (bounding radius /
// h, tested before the stencil); other cells take the SUBSAMPLE fallback.
__device__ __forceinline__ bool in_band(float p4, float p2, float tau_refine) {
    return fabsf(clamp_frac(p4) - clamp_frac(p2)) <= tau_refine;
}

// Inference over a list of cells: feat holds MLP_NFEAT rows (inputs, then the prior logit).  Standalone mode
// (ref_index == nullptr): out[c] = predicted fraction.  Coupling mode: alpha[ref_index[c]] = predicted fraction for
// every cell whose prior is a number (cells outside the band carry NaN there and are left to the fallback).
struct MlpInferArgs {
    const float* params;     // FP32 [MLP_NPARAM], device
    const float* feat;       // [MLP_NFEAT][stride]
    int64_t stride;
    int64_t n;               // cell count (standalone mode)
    const int32_t* n_dev;    // cell count written by the enumeration (coupling mode), or nullptr
    float* out;
    const int64_t* ref_index;   // coupling mode: index into the fraction scratch
    float* alpha;
    int32_t* error;          // set to SDFIBM_MLP_ERR_TIMEOUT when an MMA completion is not seen in time
};

struct MlpGradArgs {
    const float* params;
    const float* feat;       // [MLP_NFEAT][stride]
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
