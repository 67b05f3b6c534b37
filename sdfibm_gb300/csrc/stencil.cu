// LEARNED cut-cell fraction, the inputs of the network: learned_stencil_kernel runs cell_stencil (mlp.cuh) on every
// cut cell the classify pass listed.  Its own translation unit, compiled with FP32 multiply-add contraction (the
// other device files keep every operation unfused for the exact FP64 paths): the stencil is pure FP32 arithmetic
// whose results feed the network and its band, with no exactness to keep, and contraction cuts its instruction
// count.
#include <cstdint>
#include <cuda_runtime.h>

#include "common.cuh"
#include "mlp.cuh"

namespace sdfibm_dev {

// LEARNED: the model inputs of every listed cut cell, one warp per cell (cell_stencil on the cell's FP32 frame, built
// as the classify pass builds a tile's), written at the cell's list position; cells outside the band get a NaN prior
// and their list positions go to the fallback list.  Each warp stages the inputs of 32 consecutive cells in shared
// memory and writes every row as 32 consecutive floats.
__global__ void __launch_bounds__(256) learned_stencil_kernel(StencilArgs A) {
    __shared__ float s_phi[8][STENCIL_PTS];
    __shared__ uint8_t s_list[8][72];
    __shared__ float s_out[8][MLP_NFEAT][33];
    __shared__ bool s_ok[8][32];
    const int lane = threadIdx.x & 31, w = (threadIdx.x >> 5) & 7;
    const int64_t n = min((int64_t)A.cnt->n_feat, A.cap);
    const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
    const float inv_h = 1.f / A.m.h32[0];
    const float qx = 0.25f * A.m.h32[0], qy = 0.25f * A.m.h32[1], qz = 0.25f * A.m.h32[2];
    const StencilLane SL = stencil_lane();
    for (int64_t base = (((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5) * 32; base < n; base += warps * 32) {
        int s_l = 0;
        int64_t idx_l = 0;
        if (base + lane < n) {
            s_l = A.fref_solid[base + lane];
            idx_l = A.fref_index[base + lane];
        }
        const int batch = (int)min((int64_t)32, n - base);
        for (int t = 0; t < batch; ++t) {
            const int s = __shfl_sync(0xffffffffu, s_l, t);
            const int64_t idx = __shfl_sync(0xffffffffu, idx_l, t);
            const SolidK& k = A.sk[s];
            const SolidPlan& pl = A.plan[s];
            bool ok = pl.radius_cells >= A.rho_min;  // the solid-size half of the band: no stencil needed
            float feat = 0.f;
            if (ok) {
                const uint32_t local = (uint32_t)(idx - k.scratch_off);
                const int row = (int)fdiv(local, k.div_e0), lc = (int)fdiv(local, k.div_e01);
                const int la = (int)local - row * k.ext[0], lb = row - lc * k.ext[1];
                const float bx = pl.base32[0] + (float)la * A.m.h32[0], by = pl.base32[1] + (float)lb * A.m.h32[1],
                            bz = pl.base32[2] + (float)lc * A.m.h32[2];
                float M[9];
#pragma unroll
                for (int r = 0; r < 9; ++r) M[r] = pl.M[r];
                const StencilOut so = cell_stencil(k.shape, SL, M, bx, by, bz, qx, qy, qz, inv_h, s_phi[w], s_list[w]);
                ok = in_band(so.p4, so.p2, A.tau_refine);
                feat = so.feat;
            }
            if (lane < MLP_NFEAT) s_out[w][lane][t] = feat;
            if (lane == 0) s_ok[w][t] = ok;
            if (!ok && lane == 0) {
                const int slot = atomicAdd(&A.cnt->n_fb, 1);
                A.fb_list[slot] = (int32_t)(base + t);  // n_fb <= n <= cap entries
            }
        }
        __syncwarp();
        // the batch's in-band cells, compacted for the network: one atomic per warp, rows of consecutive cells
        const bool in = lane < batch && s_ok[w][lane];
        const unsigned mask = __ballot_sync(0xffffffffu, in);
        int64_t p0 = 0;
        if (lane == 0 && mask) p0 = atomicAdd(&A.cnt->n_inband, __popc(mask));
        p0 = __shfl_sync(0xffffffffu, p0, 0);
        if (in) {
            const int64_t pos = p0 + __popc(mask & ((1u << lane) - 1u));  // n_inband <= n <= cap
            for (int f = 0; f < MLP_NFEAT; ++f) A.feat[f * A.cap + pos] = s_out[w][f][lane];
            A.mlp_index[pos] = idx_l;
        }
        __syncwarp();
    }
}

}  // namespace sdfibm_dev
