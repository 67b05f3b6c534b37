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

// plane_fraction with the hardware's approximate reciprocal in its divisions (relative error about 2^-22): the model's
// prior needs far less, and the same function serves the training cells and the coupling path.
__device__ __forceinline__ float plane_fraction_fast(const float* f) {
    float n[3];
    n[0] = 0.25f * (((f[1] - f[0]) + (f[3] - f[2])) + ((f[5] - f[4]) + (f[7] - f[6])));
    n[1] = 0.25f * (((f[2] - f[0]) + (f[3] - f[1])) + ((f[6] - f[4]) + (f[7] - f[5])));
    n[2] = 0.25f * (((f[4] - f[0]) + (f[5] - f[1])) + ((f[6] - f[2]) + (f[7] - f[3])));
    const float mean = 0.125f * (((f[0] + f[1]) + (f[2] + f[3])) + ((f[4] + f[5]) + (f[6] + f[7])));
    float d = 0.5f * ((n[0] + n[1]) + n[2]) - mean;
    for (int a = 0; a < 3; ++a)
        if (n[a] < 0.f) { d -= n[a]; n[a] = -n[a]; }
    const float s = (n[0] + n[1]) + n[2];
    if (!(s > 0.f)) return d > 0.f ? 1.f : 0.f;
    const float is = __frcp_rn(s);
    float al = d * is;
    if (al <= 0.f) return 0.f;
    if (al >= 1.f) return 1.f;
    float m1 = n[0] * is, m2 = n[1] * is, m3 = n[2] * is, t;
    if (m1 > m2) { t = m1; m1 = m2; m2 = t; }
    if (m2 > m3) { t = m2; m2 = m3; m3 = t; }
    if (m1 > m2) { t = m1; m1 = m2; m2 = t; }
    const bool flip = al > 0.5f;
    if (flip) al = 1.f - al;
    const float m12 = m1 + m2;
    float v;
    if (al < m1) v = __fdividef(al * al * al, 6.f * m1 * m2 * m3);
    else if (al < m2) v = __fdividef(al * (al - m1), 2.f * m2 * m3) + __fdividef(m1 * m1, 6.f * m2 * m3);
    else if (al < fminf(m3, m12))
        v = __fdividef(al * al * (3.f * m12 - al) + m1 * m1 * (m1 - 3.f * al) + m2 * m2 * (m2 - 3.f * al),
                       6.f * m1 * m2 * m3);
    else if (m3 < m12)
        v = __fdividef(al * al * (3.f - 2.f * al) + m1 * m1 * (m1 - 3.f * al) + m2 * m2 * (m2 - 3.f * al) +
                       m3 * m3 * (m3 - 3.f * al), 6.f * m1 * m2 * m3);
    else v = __fdividef(2.f * al - m12, 2.f * m3);
    v = fminf(fmaxf(v, 0.f), 1.f);
    return flip ? 1.f - v : v;
}

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
    return plane_fraction_fast(f);
}

// Plane of a sub-cube fitted to its 8 corner values, reflected to the positive octant: 0 when the plane leaves the
// sub-cube outside the solid, 1 when inside, -1 when it crosses and the closed form is needed (plane_fraction's own
// early exits, without its divisions).
__device__ __forceinline__ int subcell_trivial(const float* sphi, int v0, int d) {
    const float f[8] = {sphi[v0], sphi[v0 + d], sphi[v0 + STENCIL_N * d], sphi[v0 + STENCIL_N * d + d],
                        sphi[v0 + STENCIL_N * STENCIL_N * d], sphi[v0 + STENCIL_N * STENCIL_N * d + d],
                        sphi[v0 + STENCIL_N * STENCIL_N * d + STENCIL_N * d],
                        sphi[v0 + STENCIL_N * STENCIL_N * d + STENCIL_N * d + d]};
    float n[3];
    n[0] = 0.25f * (((f[1] - f[0]) + (f[3] - f[2])) + ((f[5] - f[4]) + (f[7] - f[6])));
    n[1] = 0.25f * (((f[2] - f[0]) + (f[3] - f[1])) + ((f[6] - f[4]) + (f[7] - f[5])));
    n[2] = 0.25f * (((f[4] - f[0]) + (f[5] - f[1])) + ((f[6] - f[2]) + (f[7] - f[3])));
    const float mean = 0.125f * (((f[0] + f[1]) + (f[2] + f[3])) + ((f[4] + f[5]) + (f[6] + f[7])));
    float d_ = 0.5f * ((n[0] + n[1]) + n[2]) - mean;
    for (int a = 0; a < 3; ++a)
        if (n[a] < 0.f) { d_ -= n[a]; n[a] = -n[a]; }
    const float s = (n[0] + n[1]) + n[2];
    if (!(s > 0.f)) return d_ > 0.f ? 1 : 0;
    if (d_ <= 0.f) return 0;
    if (d_ >= s) return 1;
    return -1;
}

// sub-cube sc of the model's prior: 0..63 the 4^3 division (corner spacing 1), 64..71 the 2^3 one (spacing 2)
__device__ __forceinline__ int subcell_v0(int sc) {
    return sc < 64 ? stn(sc & 3, (sc >> 2) & 3, sc >> 4)
                   : stn(2 * ((sc - 64) & 1), 2 * (((sc - 64) >> 1) & 1), 2 * ((sc - 64) >> 2));
}

// What a lane does in every cell's stencil, fixed by its lane index and computed once per kernel: the lowest corners
// of its 4^3 sub-cubes l + 32 r and the stencil point of its network input.
struct StencilLane {
    int v0[2];
    int inp;
};
__device__ inline StencilLane stencil_lane() {
    const int lane = threadIdx.x & 31;
    StencilLane L;
#pragma unroll
    for (int r = 0; r < 2; ++r) L.v0[r] = subcell_v0(lane + 32 * r);
    L.inp = input_point(min(lane, 14));
    return L;
}

// Shape::signedDistance / h at the 125 lattice points, lane l taking points l, l + 32, ...: the 3-D shapes of the
// coupling workloads with the hardware's approximate square root and reciprocal (a few units in the last place; the
// reference's filter kept), any other shape through sdf32.
__device__ __forceinline__ float fast_sqrt(float x) { return x > 0.f ? x * rsqrtf(x) : 0.f; }
template <int TYPE>
__device__ __forceinline__ void stencil_points(const ShapeK& sh, const StencilLane& SL, const float* L0,
                                               const float* Li, const float* Lj, const float* Lk, float inv_h,
                                               float* sphi) {
    const int lane = threadIdx.x & 31;
    const float* a = sh.p32;
    const float c0 = sh.com32[0], c1 = sh.com32[1], c2 = sh.com32[2];
#pragma unroll
    for (int r = 0; r < 4; ++r) {
        const int p = lane + 32 * r;
        if (p >= STENCIL_PTS) break;
        const int k = p / 25, j = (p - 25 * k) / 5, i = p - 25 * k - 5 * j;
        const float fi = (float)i, fj = (float)j, fk = (float)k;
        const float lx = __fmaf_rn(fk, Lk[0], __fmaf_rn(fj, Lj[0], __fmaf_rn(fi, Li[0], L0[0])));
        const float ly = __fmaf_rn(fk, Lk[1], __fmaf_rn(fj, Lj[1], __fmaf_rn(fi, Li[1], L0[1])));
        const float lz = __fmaf_rn(fk, Lk[2], __fmaf_rn(fj, Lj[2], __fmaf_rn(fi, Li[2], L0[2])));
        float phi;
        if (TYPE == SDFIBM_SHAPE_SPHERE) {
            const float x = lx + c0, y = ly + c1, z = lz + c2;
            phi = filter32(fast_sqrt(__fmaf_rn(x, x, __fmaf_rn(y, y, z * z))) - a[0]);
        } else if (TYPE == SDFIBM_SHAPE_ELLIPSOID) {
            const float xa = lx * lx * a[3], yb = ly * ly * a[4], zc = lz * lz * a[5];
            phi = filter32(0.5f * (xa + yb + zc - 1.f) * rsqrtf(__fmaf_rn(xa, a[3], __fmaf_rn(yb, a[4], zc * a[5]))));
        } else if (TYPE == SDFIBM_SHAPE_BOX) {
            const float dx = fabsf(lx + c0) - a[0], dy = fabsf(ly + c1) - a[1], dz = fabsf(lz + c2) - a[2];
            const float dxp = fmaxf(0.f, dx), dyp = fmaxf(0.f, dy), dzp = fmaxf(0.f, dz);
            phi = filter32(fast_sqrt(__fmaf_rn(dxp, dxp, __fmaf_rn(dyp, dyp, dzp * dzp))) +
                           fminf(0.f, fmaxf(dz, fmaxf(dx, dy))));
        } else {
            phi = sdf32(sh, lx, ly, lz);
        }
        sphi[p] = phi * inv_h;
    }
}

// The model inputs of one cell, computed by all 32 lanes of a warp together (the training cells of mlp.cu; the
// coupling path computes the same quantities a thread per cell in stencil.cu).  The cell's frame: lattice point
// (i, j, k) lies at world offset (bx + i*qx, by + j*qy, bz + k*qz) from the solid centre (q = h/4 per axis, FP32), its
// local coordinates are M times that offset.  sphi: 125 floats and slist: 72 bytes of shared memory of this warp.
// Every lane returns P4 and P2 (unclamped); lane f < 16 returns input f in *feat, lane 16 the prior logit(clamp(P4)).
// The 64 sub-cubes of P4 are first sorted by the cheap test of subcell_trivial; only those the fitted plane crosses
// (about a third), and the 8 of P2, take the closed form, spread over the lanes.
struct StencilOut {
    float p4, p2, feat;
};
__device__ inline StencilOut cell_stencil(const ShapeK& sh, const StencilLane& SL, const float* M, float bx, float by,
                                          float bz, float qx, float qy, float qz, float inv_h, float* sphi,
                                          uint8_t* slist) {
    const int lane = threadIdx.x & 31;
    // local coordinates of lattice point (i, j, k): L0 + i Li + j Lj + k Lk
    const float L0[3] = {__fmaf_rn(M[0], bx, __fmaf_rn(M[1], by, M[2] * bz)),
                         __fmaf_rn(M[3], bx, __fmaf_rn(M[4], by, M[5] * bz)),
                         __fmaf_rn(M[6], bx, __fmaf_rn(M[7], by, M[8] * bz))};
    const float Li[3] = {M[0] * qx, M[3] * qx, M[6] * qx}, Lj[3] = {M[1] * qy, M[4] * qy, M[7] * qy},
                Lk[3] = {M[2] * qz, M[5] * qz, M[8] * qz};
    switch (sh.type) {
        case SDFIBM_SHAPE_SPHERE: stencil_points<SDFIBM_SHAPE_SPHERE>(sh, SL, L0, Li, Lj, Lk, inv_h, sphi); break;
        case SDFIBM_SHAPE_ELLIPSOID: stencil_points<SDFIBM_SHAPE_ELLIPSOID>(sh, SL, L0, Li, Lj, Lk, inv_h, sphi); break;
        case SDFIBM_SHAPE_BOX: stencil_points<SDFIBM_SHAPE_BOX>(sh, SL, L0, Li, Lj, Lk, inv_h, sphi); break;
        default: stencil_points<0>(sh, SL, L0, Li, Lj, Lk, inv_h, sphi); break;
    }
    __syncwarp();
    float s4 = 0.f, s2 = 0.f;
    int ncross = 0;
#pragma unroll
    for (int r = 0; r < 2; ++r) {
        const int sc = lane + 32 * r;
        const int t = subcell_trivial(sphi, SL.v0[r], 1);
        if (t == 1) s4 += 1.f;
        const unsigned need = __ballot_sync(0xffffffffu, t < 0);
        if (t < 0) slist[ncross + __popc(need & ((1u << lane) - 1u))] = (uint8_t)sc;
        ncross += __popc(need);
    }
    // the eight 2^3 sub-cubes go to the closed form directly (its own early exits settle the uncrossed ones): a
    // round of the cheap test would keep 24 of the 32 lanes idle
    if (lane < 8) slist[ncross + lane] = (uint8_t)(64 + lane);
    ncross += 8;
    __syncwarp();
    for (int e = lane; e < ncross; e += 32) {
        const int sc = slist[e];
        const float v = subcell_fraction(sphi, subcell_v0(sc), sc < 64 ? 1 : 2);
        if (sc < 64) s4 += v; else s2 += v;
    }
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
    if (lane < 15) f = sphi[SL.inp];
    else if (lane == 15) f = logit_frac(clamp_frac(out.p2));
    else if (lane == 16) f = logit_frac(clamp_frac(out.p4));
    out.feat = f;
    __syncwarp();
    return out;
}

// Confidence band: the network's answer is kept where the two planar reconstructions agree (|P4 - P2| at most
// tau_refine: the sub-cell planes resolve the surface) and the solid spans at least rho_min cells (bounding radius /
// h, tested by the classify pass, which lists the other solids' cells for the fallback); other cells take the
// SUBSAMPLE fallback.
__device__ __forceinline__ bool in_band(float p4, float p2, float tau_refine) {
    return fabsf(clamp_frac(p4) - clamp_frac(p2)) <= tau_refine;
}

// Inference over a list of cells: feat holds MLP_NFEAT rows (inputs, then the prior logit).  Standalone mode
// (ref_index == nullptr): out[c] = predicted fraction.  Coupling mode: alpha[ref_index[c]] = predicted fraction (the
// in-band cells, compacted by learned_stencil_kernel; a NaN prior is skipped).
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
