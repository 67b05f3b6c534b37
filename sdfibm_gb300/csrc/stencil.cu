// LEARNED cut-cell fraction, the inputs of the network: learned_stencil_kernel computes, for every cut cell the
// classify pass listed, the stencil and sub-cell reconstructions that cell_stencil (mlp.cuh) computes for the training
// cells, one thread per cell.  Its own translation unit, compiled with FP32 multiply-add contraction (the
// other device files keep every operation unfused for the exact FP64 paths): the stencil is pure FP32 arithmetic
// whose results feed the network and its band, with no exactness to keep, and contraction cuts its instruction
// count.
#include <cstdint>
#include <cuda_runtime.h>

#include "common.cuh"
#include "mlp.cuh"

namespace sdfibm_dev {

// One thread per cell: a warp-per-cell layout spends most of its issue slots on work every lane repeats (the cell's
// frame, shuffles, ballots, reductions) and on lanes left idle by 125 points, 64 sub-cubes and a crossed count that
// do not divide by 32; a thread walking its own cell issues each instruction for 32 cells at once.
constexpr int STN_THREADS = 64;
int stencil_block() { return STN_THREADS; }

// Shape::signedDistance at the 125 lattice points of one cell (local coordinates L0 + i Li + j Lj + k Lk), in world
// units: the sub-cube fractions do not depend on the scale, and the 15 network inputs are divided by h when they are
// written.  The 3-D shapes of the coupling workloads with the hardware's approximate square root and reciprocal, any
// other shape through sdf32.  ph: this thread's 125 floats.
template <int TYPE>
__device__ __forceinline__ void stencil_points_thread(const ShapeK& sh, const float* L0, const float* Li,
                                                      const float* Lj, const float* Lk, float* ph) {
    const float* a = sh.p32;
    const float c0 = sh.com32[0], c1 = sh.com32[1], c2 = sh.com32[2];
#pragma unroll 1
    for (int k = 0; k < STENCIL_N; ++k) {
        const float fk = (float)k;
#pragma unroll 1
        for (int j = 0; j < STENCIL_N; ++j) {
            const float fj = (float)j;
            const float rx = __fmaf_rn(fk, Lk[0], __fmaf_rn(fj, Lj[0], L0[0]));
            const float ry = __fmaf_rn(fk, Lk[1], __fmaf_rn(fj, Lj[1], L0[1]));
            const float rz = __fmaf_rn(fk, Lk[2], __fmaf_rn(fj, Lj[2], L0[2]));
#pragma unroll
            for (int i = 0; i < STENCIL_N; ++i) {
                const float fi = (float)i;
                const float lx = __fmaf_rn(fi, Li[0], rx), ly = __fmaf_rn(fi, Li[1], ry), lz = __fmaf_rn(fi, Li[2], rz);
                float phi;
                if (TYPE == SDFIBM_SHAPE_SPHERE) {
                    const float x = lx + c0, y = ly + c1, z = lz + c2;
                    phi = filter32(fast_sqrt(__fmaf_rn(x, x, __fmaf_rn(y, y, z * z))) - a[0]);
                } else if (TYPE == SDFIBM_SHAPE_ELLIPSOID) {
                    const float xa = lx * lx * a[3], yb = ly * ly * a[4], zc = lz * lz * a[5];
                    phi = filter32(0.5f * (xa + yb + zc - 1.f) *
                                   rsqrtf(__fmaf_rn(xa, a[3], __fmaf_rn(yb, a[4], zc * a[5]))));
                } else if (TYPE == SDFIBM_SHAPE_BOX) {
                    const float dx = fabsf(lx + c0) - a[0], dy = fabsf(ly + c1) - a[1], dz = fabsf(lz + c2) - a[2];
                    const float dxp = fmaxf(0.f, dx), dyp = fmaxf(0.f, dy), dzp = fmaxf(0.f, dz);
                    phi = filter32(fast_sqrt(__fmaf_rn(dxp, dxp, __fmaf_rn(dyp, dyp, dzp * dzp))) +
                                   fminf(0.f, fmaxf(dz, fmaxf(dx, dy))));
                } else {
                    phi = sdf32(sh, lx, ly, lz);
                }
                ph[stn(i, j, k)] = phi;
            }
        }
    }
}

// LEARNED: the model inputs of every cut cell listed from the front (the solids of at least rho_min cells; the
// classify pass lists the others' cells from the back, for the fallback), in the cell's FP32 frame built as the
// classify pass builds a tile's: the 5^3 distance stencil in shared memory (a thread's 125 floats at an odd stride,
// so the threads of a warp reading the same point hit distinct banks), the 64 sub-cubes of P4 sorted by the cheap
// test of subcell_trivial with the crossed ones listed for the closed form, the 8 of P2 through the closed form, the
// band.  (Spreading the closed forms of a warp's 32 cells over its lanes as one flat list was slower: the lanes then
// read other threads' stencils at scattered banks.)  The in-band cells are compacted for the network (one atomic
// per warp, rows of consecutive cells, with their fraction index in mlp_index); the others' list positions go to
// the fallback list.
__global__ void __launch_bounds__(STN_THREADS) learned_stencil_kernel(StencilArgs A) {
    __shared__ float s_phi[STN_THREADS][STENCIL_PTS];
    __shared__ uint8_t s_cross[64][STN_THREADS];  // [entry][thread]: a warp reading entry q reads 32 consecutive bytes
    const int tid = threadIdx.x, lane = tid & 31;
    float* ph = s_phi[tid];
    const int64_t n = min((int64_t)A.cnt->n_feat, A.cap);
    const float inv_h = 1.f / A.m.h32[0];
    const float qx = 0.25f * A.m.h32[0], qy = 0.25f * A.m.h32[1], qz = 0.25f * A.m.h32[2];
    for (int64_t base = (int64_t)blockIdx.x * STN_THREADS; base < n; base += (int64_t)gridDim.x * STN_THREADS) {
        const int64_t e = base + tid;
        const bool valid = e < n;
        bool ok = false;
        int64_t idx = 0;
        float p2 = 0.f, p4 = 0.f;
        if (valid) {
            const int s = A.fref_solid[e];
            idx = A.fref_index[e];
            const SolidK& k = A.sk[s];
            const SolidPlan& pl = A.plan[s];
            {
                const uint32_t local = (uint32_t)(idx - k.scratch_off);
                const int row = (int)fdiv(local, k.div_e0), lc = (int)fdiv(local, k.div_e01);
                const int la = (int)local - row * k.ext[0], lb = row - lc * k.ext[1];
                const float bx = pl.base32[0] + (float)la * A.m.h32[0], by = pl.base32[1] + (float)lb * A.m.h32[1],
                            bz = pl.base32[2] + (float)lc * A.m.h32[2];
                float M[9];
#pragma unroll
                for (int r = 0; r < 9; ++r) M[r] = pl.M[r];
                const float L0[3] = {__fmaf_rn(M[0], bx, __fmaf_rn(M[1], by, M[2] * bz)),
                                     __fmaf_rn(M[3], bx, __fmaf_rn(M[4], by, M[5] * bz)),
                                     __fmaf_rn(M[6], bx, __fmaf_rn(M[7], by, M[8] * bz))};
                const float Li[3] = {M[0] * qx, M[3] * qx, M[6] * qx}, Lj[3] = {M[1] * qy, M[4] * qy, M[7] * qy},
                            Lk[3] = {M[2] * qz, M[5] * qz, M[8] * qz};
                switch (k.shape.type) {
                    case SDFIBM_SHAPE_SPHERE:
                        stencil_points_thread<SDFIBM_SHAPE_SPHERE>(k.shape, L0, Li, Lj, Lk, ph); break;
                    case SDFIBM_SHAPE_ELLIPSOID:
                        stencil_points_thread<SDFIBM_SHAPE_ELLIPSOID>(k.shape, L0, Li, Lj, Lk, ph); break;
                    case SDFIBM_SHAPE_BOX:
                        stencil_points_thread<SDFIBM_SHAPE_BOX>(k.shape, L0, Li, Lj, Lk, ph); break;
                    default: stencil_points_thread<0>(k.shape, L0, Li, Lj, Lk, ph); break;
                }
                // P4: the cheap test of subcell_trivial row by row (four sub-cubes along x share the five corner
                // columns of the row: their sums and y / z differences), the crossed ones listed for the closed form
                float s4 = 0.f;
                int nc = 0;
#pragma unroll 1
                for (int r = 0; r < 16; ++r) {
                    const int v_row = STENCIL_N * (r & 3) + STENCIL_N * STENCIL_N * (r >> 2);
                    float sm[STENCIL_N], dy[STENCIL_N], dz[STENCIL_N];
#pragma unroll
                    for (int i = 0; i < STENCIL_N; ++i) {
                        const float a = ph[v_row + i], b = ph[v_row + i + STENCIL_N],
                                    c = ph[v_row + i + STENCIL_N * STENCIL_N],
                                    d = ph[v_row + i + STENCIL_N * STENCIL_N + STENCIL_N];
                        sm[i] = (a + b) + (c + d);
                        dy[i] = (b + d) - (a + c);
                        dz[i] = (c + d) - (a + b);
                    }
#pragma unroll
                    for (int i = 0; i < 4; ++i) {
                        const float mean = 0.125f * (sm[i] + sm[i + 1]);
                        const float half = 0.125f * (fabsf(sm[i + 1] - sm[i]) + fabsf(dy[i] + dy[i + 1]) +
                                                     fabsf(dz[i] + dz[i + 1]));  // half the plane's |normal|_1
                        if (!(half > 0.f)) {
                            if (mean < 0.f) s4 += 1.f;
                        } else if (-mean >= half) {
                            s4 += 1.f;  // the fitted plane leaves the sub-cube inside
                        } else if (mean < half) {
                            s_cross[nc++][tid] = (uint8_t)(v_row + i);  // crossed: the closed form
                        }
                    }
                }
                for (int q = 0; q < nc; ++q) s4 += subcell_fraction(ph, s_cross[q][tid], 1);
                float s2 = 0.f;
#pragma unroll 1
                for (int sc = 0; sc < 8; ++sc)
                    s2 += subcell_fraction(ph, 2 * (sc & 1) + 2 * STENCIL_N * ((sc >> 1) & 1) +
                                                   2 * STENCIL_N * STENCIL_N * (sc >> 2), 2);
                p4 = s4 * (1.f / 64.f);
                p2 = s2 * (1.f / 8.f);
                ok = in_band(p4, p2, A.tau_refine);
            }
        }
        // the warp's in-band cells, compacted for the network; the others to the fallback list
        const bool in = valid && ok;
        const unsigned mask = __ballot_sync(0xffffffffu, in);
        const unsigned fbm = __ballot_sync(0xffffffffu, valid && !ok);
        const unsigned below = (1u << lane) - 1u;
        int64_t p0 = 0, q0 = 0;
        if (lane == 0) {
            if (mask) p0 = atomicAdd(&A.cnt->n_inband, __popc(mask));
            if (fbm) q0 = atomicAdd(&A.cnt->n_fb, __popc(fbm));
        }
        p0 = __shfl_sync(0xffffffffu, p0, 0);
        q0 = __shfl_sync(0xffffffffu, q0, 0);
        if (in) {
            const int64_t pos = p0 + __popc(mask & below);  // n_inband <= n <= cap
#pragma unroll
            for (int f = 0; f < 15; ++f) A.feat[f * A.cap + pos] = ph[input_point(f)] * inv_h;
            A.feat[15 * A.cap + pos] = logit_frac(clamp_frac(p2));
            A.feat[16 * A.cap + pos] = logit_frac(clamp_frac(p4));
            A.mlp_index[pos] = idx;
        } else if (valid) {
            A.fb_list[q0 + __popc(fbm & below)] = (int32_t)e;  // n_fb <= n <= cap
        }
    }
}

}  // namespace sdfibm_dev
