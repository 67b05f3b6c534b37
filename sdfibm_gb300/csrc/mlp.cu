// Learned cut-cell fraction on the Blackwell tensor cores: inference, training (forward + backward), Adam, and the
// generator of labelled training cells.  Parameter layout, features and numerics: include/sdfibm_mlp.h.
//
// Model output: a = sigmoid(prior + network), the prior logit(P4) of the sub-cell planar reconstruction (row 16 of the
// feature buffer, see cell_stencil in mlp.cuh).
// One CTA of 128 threads works on tiles of 128 cells; thread t owns cell t of the tile, row t of every M = 128
// operand and lane t of tensor memory.  Thread 0 issues the tcgen05.mma instructions and commits them to one
// mbarrier; every wait on it is bounded and a timeout ends the CTA's work with an error code.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <vector>

#include "mlp.cuh"
#include "tc.cuh"

namespace sdfibm_dev {

constexpr long long MLP_WAIT_CYCLES = 2000000000LL;  // about one second at the SM clock
constexpr unsigned FULLMASK = 0xffffffffu;

__device__ __forceinline__ float sigm(float z) { return __fdividef(1.f, 1.f + __expf(-z)); }
__device__ __forceinline__ uint32_t bf16_bits(float x) {
    return (uint32_t)__bfloat16_as_ushort(__float2bfloat16_rn(x));
}
__device__ __forceinline__ float bf16_value(uint32_t b) { return __uint_as_float(b << 16); }
__device__ __forceinline__ uint32_t pack2(uint32_t lo_elem, uint32_t hi_elem) { return lo_elem | (hi_elem << 16); }

// 8 consecutive K elements (k0..k0+7) of one row as a 16-byte store into a K-major operand
__device__ __forceinline__ void store_row8(uint8_t* op, int row, int k0, int K, const uint32_t* b) {
    uint4 w;
    w.x = pack2(b[0], b[1]); w.y = pack2(b[2], b[3]); w.z = pack2(b[4], b[5]); w.w = pack2(b[6], b[7]);
    *reinterpret_cast<uint4*>(op + tc::kmajor_offset(row, k0, K)) = w;
}
__device__ __forceinline__ void store_bf16(uint8_t* op, int row, int k, int K, float x) {
    *reinterpret_cast<uint16_t*>(op + tc::kmajor_offset(row, k, K)) = (uint16_t)bf16_bits(x);
}

// 64 FP32 columns [col, col + 64) of this thread's lane
__device__ __forceinline__ void tmem_ld64(uint32_t base, int warp, int col, float* v) {
#pragma unroll
    for (int j = 0; j < 4; ++j) tc::tmem_ld16(tc::tmem_addr(base, 32 * warp, col + 16 * j), v + 16 * j);
    tc::tmem_wait_ld();
}
__device__ __forceinline__ void tmem_ld32(uint32_t base, int warp, int col, float* v) {
    tc::tmem_ld16(tc::tmem_addr(base, 32 * warp, col), v);
    tc::tmem_ld16(tc::tmem_addr(base, 32 * warp, col + 16), v + 16);
    tc::tmem_wait_ld();
}

// Stages W1 (BF16, K padded to 16) and W2 (BF16) as B operands, and the FP32 vectors.
__device__ void stage_weights(const float* P, uint8_t* sW1, uint8_t* sW2, uint8_t* sW2T, float* sb1, float* sb2,
                              float* sw3, float* sb3) {
    for (int e = threadIdx.x; e < MLP_H * 16; e += blockDim.x) {
        const int n = e >> 4, k = e & 15;
        store_bf16(sW1, n, k, 16, k < MLP_IN ? P[MLP_OFF_W1 + n * MLP_IN + k] : 0.f);
    }
    for (int e = threadIdx.x; e < MLP_H * MLP_H; e += blockDim.x) {
        const int n = e >> 6, k = e & 63;
        const float w = P[MLP_OFF_W2 + n * MLP_H + k];
        store_bf16(sW2, n, k, 64, w);
        if (sW2T) store_bf16(sW2T, k, n, 64, w);  // B of dH1 = dZ2 W2: row = input unit, K = output unit
    }
    if (threadIdx.x < MLP_H) {
        sb1[threadIdx.x] = P[MLP_OFF_B1 + threadIdx.x];
        sb2[threadIdx.x] = P[MLP_OFF_B2 + threadIdx.x];
        sw3[threadIdx.x] = P[MLP_OFF_W3 + threadIdx.x];
    }
    if (threadIdx.x == 0) *sb3 = P[MLP_OFF_B3];
}

// BF16 hi + lo halves of two values, packed as the K-major operands hold them (a in the low 16 bits): one
// two-value round-to-nearest conversion per half, the same bits as two single conversions.
__device__ __forceinline__ void split2(float a, float b, uint32_t& hi, uint32_t& lo) {
    const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
    hi = *reinterpret_cast<const uint32_t*>(&h);
    const __nv_bfloat162 l = __floats2bfloat162_rn(a - __uint_as_float(hi << 16), b - __uint_as_float(hi & 0xffff0000u));
    lo = *reinterpret_cast<const uint32_t*>(&l);
}

// A1 row: hi of the 16 inputs in K 0..15, lo in K 16..31
static_assert(MLP_IN == 16, "the layer-1 operand holds 16 inputs");
__device__ __forceinline__ void store_a1(uint8_t* sA1, int row, const float* x) {
    uint4 h0, h1, l0, l1;
    split2(x[0], x[1], h0.x, l0.x); split2(x[2], x[3], h0.y, l0.y);
    split2(x[4], x[5], h0.z, l0.z); split2(x[6], x[7], h0.w, l0.w);
    split2(x[8], x[9], h1.x, l1.x); split2(x[10], x[11], h1.y, l1.y);
    split2(x[12], x[13], h1.z, l1.z); split2(x[14], x[15], h1.w, l1.w);
    *reinterpret_cast<uint4*>(sA1 + tc::kmajor_offset(row, 0, 32)) = h0;
    *reinterpret_cast<uint4*>(sA1 + tc::kmajor_offset(row, 8, 32)) = h1;
    *reinterpret_cast<uint4*>(sA1 + tc::kmajor_offset(row, 16, 32)) = l0;
    *reinterpret_cast<uint4*>(sA1 + tc::kmajor_offset(row, 24, 32)) = l1;
}

// A2 row: hi of h1 in K 0..63, lo in K 64..127; h holds the units 8 * g0 .. 8 * (g0 + NG) - 1
template <int NG = 8>
__device__ __forceinline__ void store_a2(uint8_t* sA2, int row, const float* h, int g0 = 0) {
#pragma unroll
    for (int i = 0; i < NG; ++i) {
        const int g = g0 + i;
        uint4 hw, lw;
        split2(h[8 * i], h[8 * i + 1], hw.x, lw.x);
        split2(h[8 * i + 2], h[8 * i + 3], hw.y, lw.y);
        split2(h[8 * i + 4], h[8 * i + 5], hw.z, lw.z);
        split2(h[8 * i + 6], h[8 * i + 7], hw.w, lw.w);
        *reinterpret_cast<uint4*>(sA2 + tc::kmajor_offset(row, 8 * g, 128)) = hw;
        *reinterpret_cast<uint4*>(sA2 + tc::kmajor_offset(row, 64 + 8 * g, 128)) = lw;
    }
}

// layer-1 and layer-2 MMAs (issued by one thread)
__device__ __forceinline__ void issue_layer1(uint32_t D1, const uint8_t* sA1, const uint8_t* sW1) {
    const uint32_t id = tc::idesc_bf16(128, 64);
    const uint64_t b = tc::sdesc(tc::smem_u32(sW1), 128, 256);
    tc::mma_bf16(D1, tc::sdesc(tc::smem_u32(sA1), 128, 512), b, id, 0);
    tc::mma_bf16(D1, tc::sdesc(tc::smem_u32(sA1) + 256, 128, 512), b, id, 1);
}
__device__ __forceinline__ void issue_layer2(uint32_t D2, const uint8_t* sA2, const uint8_t* sW2) {
    const uint32_t id = tc::idesc_bf16(128, 64);
#pragma unroll
    for (int s = 0; s < 8; ++s)
        tc::mma_bf16(D2, tc::sdesc(tc::smem_u32(sA2) + 256 * s, 128, 2048),
                     tc::sdesc(tc::smem_u32(sW2) + 256 * (s & 3), 128, 1024), id, s > 0);
}

// Waits for the next commit; all threads agree on the outcome.  On a timeout the CTA waits once more (bounded) for
// the MMAs in flight, so that tensor memory is not released under them.
__device__ __forceinline__ bool cta_wait(uint64_t* bar, uint32_t& phase, int32_t* error) {
    const bool ok = tc::mbar_wait(bar, phase, MLP_WAIT_CYCLES);
    phase ^= 1u;
    const int bad = __syncthreads_or(!ok);
    if (bad) {
        if (threadIdx.x == 0) atomicExch(error, SDFIBM_MLP_ERR_TIMEOUT);
        tc::mbar_wait(bar, phase ^ 1u, MLP_WAIT_CYCLES);
        return false;
    }
    tc::fence_after_sync();
    return true;
}

__device__ __forceinline__ uint8_t* align1024(uint8_t* p) {
    return reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(p) + 1023) & ~uintptr_t(1023));
}

// ---- inference -----------------------------------------------------------------------------------------------------
// The layer-1 operand A1 lives in the first 8 KB of the layer-2 operand A2 (A2 is written only after the layer-1 MMA
// has completed, and A1 only after the layer-2 MMA has), and D2 takes D1's tensor-memory columns (the layer-2 MMA is
// issued after every thread has read D1): 45 KB of shared memory and 64 columns per CTA, five CTAs per SM.
constexpr int INF_W1 = 0, INF_W2 = 2048, INF_A2 = 10240, INF_A1 = INF_A2, INF_F = INF_A2 + 32768;
constexpr int INF_SMEM = INF_F + 4 * 64 * 4 + 64 + 1024;

__global__ void __launch_bounds__(MLP_THREADS, 5) mlp_infer_kernel(MlpInferArgs A) {
    extern __shared__ uint8_t smraw[];
    uint8_t* sm = align1024(smraw);
    uint8_t *sW1 = sm + INF_W1, *sW2 = sm + INF_W2, *sA1 = sm + INF_A1, *sA2 = sm + INF_A2;
    float* sb1 = reinterpret_cast<float*>(sm + INF_F);
    float *sb2 = sb1 + 64, *sw3 = sb2 + 64, *sb3 = sw3 + 64;
    uint64_t* bar = reinterpret_cast<uint64_t*>(sb3 + 64);
    uint32_t* tslot = reinterpret_cast<uint32_t*>(bar + 1);
    const int tid = threadIdx.x, warp = tid >> 5;

    stage_weights(A.params, sW1, sW2, nullptr, sb1, sb2, sw3, sb3);
    if (tid == 0) {
        tc::mbar_init(bar, 1);
        tc::fence_mbar_init();
    }
    if (warp == 0) {
        tc::tmem_alloc(tslot, 64);
        tc::tmem_relinquish();
    }
    tc::fence_smem_async();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tbase = *tslot, D1 = tbase, D2 = tbase;
    const int64_t n = A.n_dev ? min((int64_t)*A.n_dev, A.stride) : A.n;
    const int64_t ntiles = (n + MLP_TILE - 1) / MLP_TILE;
    uint32_t phase = 0;
    // this thread's cell of a tile: inputs, prior and destination, loaded one tile ahead so that the loads of tile
    // t + gridDim.x overlap the MMAs and the epilogues of tile t
    float x[MLP_IN], prior = 0.f;
    int64_t dst = -1;
    auto load_cell = [&](int64_t t, float* xv, float& pv, int64_t& dv) {
        const int64_t c = t * MLP_TILE + tid;
        const bool valid = t < ntiles && c < n;
#pragma unroll
        for (int f = 0; f < MLP_IN; ++f) xv[f] = valid ? A.feat[f * A.stride + c] : 0.f;
        pv = valid ? A.feat[MLP_IN * A.stride + c] : 0.f;
        dv = !valid ? -1 : (A.ref_index ? A.ref_index[c] : c);
    };
    load_cell(blockIdx.x, x, prior, dst);
    for (int64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
        store_a1(sA1, tid, x);
        tc::fence_smem_async();
        __syncthreads();
        if (tid == 0) {
            tc::fence_after_sync();
            issue_layer1(D1, sA1, sW1);
            tc::mma_commit(bar);
        }
        const float prior_t = prior;
        const int64_t dst_t = dst;
        load_cell(t + gridDim.x, x, prior, dst);  // the next tile (sA1 holds this one's inputs)
        if (!cta_wait(bar, phase, A.error)) break;
        // the epilogues take half a row (32 units) at a time: five CTAs per SM leave 96 registers a thread
#pragma unroll
        for (int half = 0; half < 2; ++half) {
            float z[32];
            tmem_ld32(D1, warp, 32 * half, z);
#pragma unroll
            for (int j = 0; j < 32; ++j) {
                const float zz = z[j] + sb1[32 * half + j];
                z[j] = zz * sigm(zz);
            }
            store_a2<4>(sA2, tid, z, 4 * half);
        }
        tc::fence_before_sync();
        tc::fence_smem_async();
        __syncthreads();
        if (tid == 0) {
            tc::fence_after_sync();
            issue_layer2(D2, sA2, sW2);
            tc::mma_commit(bar);
        }
        if (!cta_wait(bar, phase, A.error)) break;
        float o = *sb3;
#pragma unroll
        for (int half = 0; half < 2; ++half) {
            float z[32];
            tmem_ld32(D2, warp, 32 * half, z);
#pragma unroll
            for (int j = 0; j < 32; ++j) {
                const float zz = z[j] + sb2[32 * half + j];
                o += sw3[32 * half + j] * (zz * sigm(zz));
            }
        }
        const float a = sigm(prior_t + o);
        if (dst_t >= 0) {
            if (!A.ref_index) A.out[dst_t] = a;
            else if (prior_t == prior_t) A.alpha[dst_t] = a;  // a NaN prior: outside the band (fallback)
        }
        tc::fence_before_sync();
        __syncthreads();
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tbase, 64);
}

// ---- training: forward + backward of one batch, weight gradients accumulated in tensor memory -------------------------
// Shared memory (bytes): B operands W1 (64x16), W2 (64x64), W2^T (64x64); A operands of layer 1 (128x32) and layer 2
// (128x128); GA = [dZ2^T ; dZ1^T] (128 x 128 cells) and GB = [H1 | X] (80 x 128 cells), the operands of the weight
// gradient product D_acc += GA GB^T (rows 0..63, cols 0..63: dW2; rows 64..127, cols 64..74: dW1); DZ2 (128 x 64),
// the A operand of dH1 = dZ2 W2.  Tensor memory: D1 [0,64), D2 [64,128), D3 = dH1 [128,192), D_acc [256,336).
constexpr int TR_W1 = 0, TR_W2 = 2048, TR_W2T = 10240, TR_A1 = 18432, TR_A2 = 26624, TR_GA = 59392, TR_GB = 92160,
              TR_DZ2 = 112640, TR_F = 129024;
constexpr int TR_RED = TR_F;                       // [4 warps][3][64] float
constexpr int TR_ACC = TR_RED + 4 * 3 * 64 * 4;   // [3][64] float + 2 scalars
constexpr int TR_PAR = TR_ACC + 3 * 64 * 4 + 64;  // b1, b2, w3, b3
constexpr int TR_BAR = TR_PAR + 4 * 64 * 4;
constexpr int TR_SMEM = TR_BAR + 64 + 1024;

// Reduce-scatter of 64 values over the warp: afterwards lane l holds the warp sums of entries 2l and 2l+1 in v[0..1].
template <int HALF>
__device__ __forceinline__ void rs_stage(float* v, int lane) {
    const bool up = (lane & (HALF / 2)) != 0;
#pragma unroll
    for (int i = 0; i < HALF; ++i) {
        const float send = up ? v[i] : v[i + HALF];
        const float keep = up ? v[i + HALF] : v[i];
        v[i] = keep + __shfl_xor_sync(FULLMASK, send, HALF / 2);
    }
}
__device__ __forceinline__ void reduce_scatter64(float* v, int lane) {
    rs_stage<32>(v, lane);
    rs_stage<16>(v, lane);
    rs_stage<8>(v, lane);
    rs_stage<4>(v, lane);
    rs_stage<2>(v, lane);
}
__device__ __forceinline__ float warp_sum(float x) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(FULLMASK, x, o);
    return x;
}

__global__ void __launch_bounds__(MLP_THREADS, 1) mlp_grad_kernel(MlpGradArgs A) {
    extern __shared__ uint8_t smraw[];
    uint8_t* sm = align1024(smraw);
    uint8_t *sW1 = sm + TR_W1, *sW2 = sm + TR_W2, *sW2T = sm + TR_W2T, *sA1 = sm + TR_A1, *sA2 = sm + TR_A2,
            *sGA = sm + TR_GA, *sGB = sm + TR_GB, *sDZ2 = sm + TR_DZ2;
    float* red = reinterpret_cast<float*>(sm + TR_RED);
    float* acc = reinterpret_cast<float*>(sm + TR_ACC);
    float* sb1 = reinterpret_cast<float*>(sm + TR_PAR);
    float *sb2 = sb1 + 64, *sw3 = sb2 + 64, *sb3 = sw3 + 64;
    uint64_t* bar = reinterpret_cast<uint64_t*>(sm + TR_BAR);
    uint32_t* tslot = reinterpret_cast<uint32_t*>(bar + 1);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

    stage_weights(A.params, sW1, sW2, sW2T, sb1, sb2, sw3, sb3);
    for (int e = tid; e < 3 * 64 + 2; e += MLP_THREADS) acc[e] = 0.f;
    // GB rows 64 + MLP_IN .. 79 (padding of the input block, when there are fewer than 16 inputs) stay zero
    for (int e = tid; e < (16 - MLP_IN) * 128; e += MLP_THREADS) store_bf16(sGB, 64 + MLP_IN + e / 128, e % 128, 128, 0.f);
    if (tid == 0) {
        tc::mbar_init(bar, 1);
        tc::fence_mbar_init();
    }
    if (warp == 0) {
        tc::tmem_alloc(tslot, 512);
        tc::tmem_relinquish();
    }
    tc::fence_smem_async();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tbase = *tslot, D1 = tbase, D2 = tbase + 64, D3 = tbase + 128, DACC = tbase + 256;
    const int64_t ntiles = (A.n + MLP_TILE - 1) / MLP_TILE;
    uint32_t phase = 0;
    int ntile_done = 0;
    bool alive = true;
    for (int64_t t = blockIdx.x; t < ntiles && alive; t += gridDim.x) {
        const int64_t c = t * MLP_TILE + tid;
        const bool valid = c < A.n;
        float x[MLP_IN];
#pragma unroll
        for (int f = 0; f < MLP_IN; ++f) x[f] = valid ? A.feat[f * A.stride + c] : 0.f;
        const float prior = valid ? A.feat[MLP_IN * A.stride + c] : 0.f;
        const float y = valid ? A.label[c] : 0.f;
        store_a1(sA1, tid, x);
#pragma unroll
        for (int f = 0; f < MLP_IN; ++f) store_bf16(sGB, 64 + f, tid, 128, x[f]);
        tc::fence_smem_async();
        __syncthreads();
        if (tid == 0) {
            tc::fence_after_sync();
            issue_layer1(D1, sA1, sW1);
            tc::mma_commit(bar);
        }
        if (!(alive = cta_wait(bar, phase, A.error))) break;
        float v[64];
        tmem_ld64(D1, warp, 0, v);
#pragma unroll
        for (int j = 0; j < 64; ++j) {
            const float zz = v[j] + sb1[j];
            v[j] = zz * sigm(zz);
            store_bf16(sGB, j, tid, 128, v[j]);
        }
        store_a2(sA2, tid, v);
        tc::fence_before_sync();
        tc::fence_smem_async();
        __syncthreads();
        if (tid == 0) {
            tc::fence_after_sync();
            issue_layer2(D2, sA2, sW2);
            tc::mma_commit(bar);
        }
        if (!(alive = cta_wait(bar, phase, A.error))) break;
        // output layer, loss and the backward pass down to dZ2
        tmem_ld64(D2, warp, 0, v);
        float o = *sb3;
#pragma unroll
        for (int j = 0; j < 64; ++j) {
            const float zz = v[j] + sb2[j];
            o += sw3[j] * (zz * sigm(zz));
        }
        const float a = sigm(prior + o);
        const float d = valid ? a - y : 0.f;
        const float dz3 = A.scale * d * a * (1.f - a);
        float w[64];
#pragma unroll
        for (int j = 0; j < 64; ++j) {
            const float zz = v[j] + sb2[j];
            const float s = sigm(zz);
            w[j] = dz3 * (zz * s);                                 // dw3 contribution
            v[j] = dz3 * sw3[j] * (s * (1.f + zz * (1.f - s)));    // dZ2
        }
        {
            uint32_t b[8];
#pragma unroll
            for (int g = 0; g < 8; ++g) {
#pragma unroll
                for (int i = 0; i < 8; ++i) b[i] = bf16_bits(v[8 * g + i]);
                store_row8(sDZ2, tid, 8 * g, 64, b);
            }
#pragma unroll
            for (int j = 0; j < 64; ++j) store_bf16(sGA, j, tid, 128, v[j]);
        }
        reduce_scatter64(w, lane);
        red[(warp * 3 + 0) * 64 + 2 * lane] = w[0];
        red[(warp * 3 + 0) * 64 + 2 * lane + 1] = w[1];
        reduce_scatter64(v, lane);
        red[(warp * 3 + 1) * 64 + 2 * lane] = v[0];
        red[(warp * 3 + 1) * 64 + 2 * lane + 1] = v[1];
        const float s_dz3 = warp_sum(dz3), s_loss = warp_sum(d * d);
        if (lane == 0) {
            atomicAdd(&acc[192], s_dz3);
            atomicAdd(&acc[193], s_loss);
        }
        tc::fence_before_sync();
        tc::fence_smem_async();
        __syncthreads();
        if (tid == 0) {
            // dH1 = dZ2 W2: A = DZ2 (128 x 64), B = W2^T (64 x 64)
            tc::fence_after_sync();
            const uint32_t id = tc::idesc_bf16(128, 64);
#pragma unroll
            for (int s = 0; s < 4; ++s)
                tc::mma_bf16(D3, tc::sdesc(tc::smem_u32(sDZ2) + 256 * s, 128, 1024),
                             tc::sdesc(tc::smem_u32(sW2T) + 256 * s, 128, 1024), id, s > 0);
            tc::mma_commit(bar);
        }
        if (!(alive = cta_wait(bar, phase, A.error))) break;
        tmem_ld64(D3, warp, 0, v);   // dH1
        tmem_ld64(D1, warp, 0, w);   // z1 - b1
#pragma unroll
        for (int j = 0; j < 64; ++j) {
            const float zz = w[j] + sb1[j];
            const float s = sigm(zz);
            v[j] *= s * (1.f + zz * (1.f - s));   // dZ1
            store_bf16(sGA, 64 + j, tid, 128, v[j]);
        }
        reduce_scatter64(v, lane);
        red[(warp * 3 + 2) * 64 + 2 * lane] = v[0];
        red[(warp * 3 + 2) * 64 + 2 * lane + 1] = v[1];
        tc::fence_before_sync();
        tc::fence_smem_async();
        __syncthreads();
        if (tid < 64) {
#pragma unroll
            for (int q = 0; q < 3; ++q)
                acc[q * 64 + tid] += red[(0 * 3 + q) * 64 + tid] + red[(1 * 3 + q) * 64 + tid] +
                                     red[(2 * 3 + q) * 64 + tid] + red[(3 * 3 + q) * 64 + tid];
        }
        if (tid == 0) {
            // D_acc += [dZ2^T ; dZ1^T] [H1 | X]^T over the 128 cells of the tile
            tc::fence_after_sync();
            const uint32_t id = tc::idesc_bf16(128, 80);
#pragma unroll
            for (int s = 0; s < 8; ++s)
                tc::mma_bf16(DACC, tc::sdesc(tc::smem_u32(sGA) + 256 * s, 128, 2048),
                             tc::sdesc(tc::smem_u32(sGB) + 256 * s, 128, 2048), id, (ntile_done > 0 || s > 0) ? 1u : 0u);
            tc::mma_commit(bar);
        }
        if (!(alive = cta_wait(bar, phase, A.error))) break;
        ++ntile_done;
    }
    __syncthreads();
    if (alive && ntile_done > 0) {
        float v[64];
        if (warp < 2) {
            tmem_ld64(DACC, warp, 0, v);
#pragma unroll
            for (int i = 0; i < 64; ++i) atomicAdd(&A.grad[MLP_OFF_W2 + tid * 64 + i], v[i]);
        } else {
            tc::tmem_ld16(tc::tmem_addr(DACC, 32 * warp, 64), v);
            tc::tmem_wait_ld();
#pragma unroll
            for (int f = 0; f < MLP_IN; ++f) atomicAdd(&A.grad[MLP_OFF_W1 + (tid - 64) * MLP_IN + f], v[f]);
        }
        if (tid < 64) {
            atomicAdd(&A.grad[MLP_OFF_W3 + tid], acc[tid]);
            atomicAdd(&A.grad[MLP_OFF_B2 + tid], acc[64 + tid]);
            atomicAdd(&A.grad[MLP_OFF_B1 + tid], acc[128 + tid]);
        }
        if (tid == 0) {
            atomicAdd(&A.grad[MLP_OFF_B3], acc[192]);
            atomicAdd(&A.grad[MLP_NPARAM], acc[193]);
        }
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tbase, 512);
}

__global__ void mlp_adam_kernel(float* p, const float* g, float* m, float* v, float c1, float c2, float lr) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= MLP_NPARAM) return;
    const float gi = g[i];
    const float mi = 0.9f * m[i] + 0.1f * gi;
    const float vi = 0.999f * v[i] + 0.001f * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi * c1) / (sqrtf(vi * c2) + 1e-8f);
}

// ---- labelled training cells ---------------------------------------------------------------------------------------
__device__ __forceinline__ uint64_t mix64(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
struct Rng {
    uint64_t s;
    __device__ double uni() {  // [0, 1)
        s = mix64(s);
        return (double)(s >> 11) * (1.0 / 9007199254740992.0);
    }
};

struct DataArgs {
    uint64_t seed;
    int64_t n;
    double lhr_min, lhr_max;
    int32_t fam[6];
    int32_t nfam;
    int32_t n_sub;
    double z_axis_frac;
    float* feat;
    float* label;
    double* recipe;
};

// shape parameters as the host-side lowering writes them (sdfibm_shape_desc.p), centred at the origin
__device__ void make_family_shape(int fam, double r, Rng& g, ShapeK& sh) {
    for (int i = 0; i < 8; ++i) sh.p[i] = 0.0;
    for (int i = 0; i < 3; ++i) sh.com[i] = 0.0;
    sh.prism = 0;
    switch (fam) {
        case SDFIBM_MLP_SPHERE:
            sh.type = SDFIBM_SHAPE_SPHERE; sh.p[0] = r; sh.p[1] = r * r;
            break;
        case SDFIBM_MLP_ELLIPSOID: {
            const double b = r * (1.0 + 2.0 * g.uni()), c = r * (1.0 + 2.0 * g.uni());
            sh.type = SDFIBM_SHAPE_ELLIPSOID;
            sh.p[0] = r; sh.p[1] = b; sh.p[2] = c;
            sh.p[3] = 1.0 / (r * r); sh.p[4] = 1.0 / (b * b); sh.p[5] = 1.0 / (c * c);
            break;
        }
        case SDFIBM_MLP_BOX:
            sh.type = SDFIBM_SHAPE_BOX; sh.p[0] = r; sh.p[1] = r * (1.0 + 2.0 * g.uni()); sh.p[2] = r * (1.0 + 2.0 * g.uni());
            break;
        case SDFIBM_MLP_PLANE:
            sh.type = SDFIBM_SHAPE_PLANE;
            break;
        case SDFIBM_MLP_CYLINDER:
            sh.type = SDFIBM_SHAPE_CIRCLE; sh.prism = 1; sh.p[0] = r; sh.p[1] = r * r;
            break;
        default: {
            const double b = r * (1.0 + 2.0 * g.uni());
            sh.type = SDFIBM_SHAPE_ELLIPSE; sh.prism = 1;
            sh.p[0] = r; sh.p[1] = b; sh.p[2] = 1.0 / (r * r); sh.p[3] = 1.0 / (b * b);
            break;
        }
    }
}

// a point of the shape's surface in its local frame
__device__ D3 surface_point(const ShapeK& sh, Rng& g, double h) {
    const double PI2 = 6.283185307179586;
    if (sh.type == SDFIBM_SHAPE_PLANE) return D3{(2.0 * g.uni() - 1.0) * 4.0 * h, 0.0, (2.0 * g.uni() - 1.0) * 4.0 * h};
    if (sh.prism) {
        const double t = PI2 * g.uni(), cx = cos(t), cy = sin(t);
        const double s = sh.type == SDFIBM_SHAPE_CIRCLE ? sh.p[0]
                                                        : 1.0 / sqrt(cx * cx * sh.p[2] + cy * cy * sh.p[3]);
        return D3{s * cx, s * cy, (2.0 * g.uni() - 1.0) * 2.0 * h};
    }
    const double zz = 2.0 * g.uni() - 1.0, t = PI2 * g.uni(), rr = sqrt(fmax(0.0, 1.0 - zz * zz));
    const D3 d{rr * cos(t), rr * sin(t), zz};
    double s;
    if (sh.type == SDFIBM_SHAPE_SPHERE) {
        s = sh.p[0];
    } else if (sh.type == SDFIBM_SHAPE_ELLIPSOID) {
        s = 1.0 / sqrt(d.x * d.x * sh.p[3] + d.y * d.y * sh.p[4] + d.z * d.z * sh.p[5]);
    } else {  // box
        s = fmin(sh.p[0] / fmax(fabs(d.x), 1e-300), fmin(sh.p[1] / fmax(fabs(d.y), 1e-300), sh.p[2] / fmax(fabs(d.z), 1e-300)));
    }
    return D3{s * d.x, s * d.y, s * d.z};
}

// One labelled cut cell per thread: the thread draws the shape, pose and cell (FP64) and counts the label lattice in
// FP64; the inputs come from cell_stencil, as in the coupling path: the warp computes its 32 cells' stencils one after
// the other from the FP32 frame (cell corner as the offset from the shape centre, the rotation's local map).
__global__ void __launch_bounds__(128) mlp_dataset_kernel(DataArgs A) {
    __shared__ ShapeK s_sh[128];
    __shared__ float s_fr[128][12];  // local map M (9), cell corner (3)
    __shared__ float s_phi[4][STENCIL_PTS];
    __shared__ uint8_t s_list[4][72];
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const bool valid = i < A.n;
    // the family is uniform over a warp: fewer divergent FP64 paths
    Rng gw{mix64(A.seed ^ mix64((uint64_t)(i >> 5) + 0x51ull))};
    const int fam = A.fam[min((int)(gw.uni() * A.nfam), A.nfam - 1)];
    Rng g{mix64(A.seed ^ mix64((uint64_t)i * 0x2545F4914F6CDD1Dull + 0x1234567ull))};
    const double h = 1.0;
    const D3 zero{0.0, 0.0, 0.0};
    ShapeK sh;
    Q4 q{1.0, D3{0.0, 0.0, 0.0}};
    D3 o{0.0, 0.0, 0.0};
    int inside_cnt = 0, attempt = 0;
    for (attempt = 1; attempt <= 256; ++attempt) {
        const double r = h / exp(A.lhr_min + (A.lhr_max - A.lhr_min) * g.uni());
        make_family_shape(fam, r, g, sh);
        if (sh.prism && g.uni() < A.z_axis_frac) {
            const double t = 3.141592653589793 * g.uni();
            q = Q4{cos(t), D3{0.0, 0.0, sin(t)}};
        } else {  // uniform random rotation (Shoemake)
            const double u1 = g.uni(), u2 = 6.283185307179586 * g.uni(), u3 = 6.283185307179586 * g.uni();
            const double a = sqrt(1.0 - u1), b = sqrt(u1);
            q = Q4{b * cos(u3), D3{a * sin(u2), a * cos(u2), b * sin(u3)}};
        }
        const D3 ps = qtransform(q, surface_point(sh, g, h));
        const D3 p{ps.x + (2.0 * g.uni() - 1.0) * 0.9 * h, ps.y + (2.0 * g.uni() - 1.0) * 0.9 * h,
                   ps.z + (2.0 * g.uni() - 1.0) * 0.9 * h};
        o = D3{p.x - g.uni() * h, p.y - g.uni() * h, p.z - g.uni() * h};
        inside_cnt = 0;
        for (int v = 0; v < 8; ++v) {
            const D3 pv{o.x + (double)(v & 1) * h, o.y + (double)((v >> 1) & 1) * h, o.z + (double)((v >> 2) & 1) * h};
            inside_cnt += inside64(sh, world2local(pv, zero, q)) ? 1 : 0;
        }
        if (!valid || (inside_cnt > 0 && inside_cnt < 8)) break;
    }
    for (int k = 0; k < 8; ++k) sh.p32[k] = (float)sh.p[k];
    for (int k = 0; k < 3; ++k) sh.com32[k] = (float)sh.com[k];
    s_sh[threadIdx.x] = sh;
    local_matrix32(q, s_fr[threadIdx.x]);
    s_fr[threadIdx.x][9] = (float)o.x;
    s_fr[threadIdx.x][10] = (float)o.y;
    s_fr[threadIdx.x][11] = (float)o.z;
    __syncwarp();
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const StencilLane SL = stencil_lane();
    for (int t = 0; t < 32; ++t) {
        const int src = (w << 5) + t;
        const int64_t ci = (int64_t)blockIdx.x * blockDim.x + src;
        if (ci >= A.n) break;  // uniform over the warp
        float M[9];
#pragma unroll
        for (int r = 0; r < 9; ++r) M[r] = s_fr[src][r];
        const StencilOut so = cell_stencil(s_sh[src], SL, M, s_fr[src][9], s_fr[src][10], s_fr[src][11], 0.25f,
                                           0.25f, 0.25f, 1.f, s_phi[w], s_list[w]);
        if (lane < MLP_NFEAT) A.feat[lane * A.n + ci] = so.feat;
    }
    if (!valid) return;
    const int n = A.n_sub;
    int cnt = 0;
    for (int c3 = 0; c3 < n; ++c3)
        for (int b = 0; b < n; ++b)
            for (int a = 0; a < n; ++a) {
                const double ta = (double)(2 * a + 1) / (double)(2 * n), tb = (double)(2 * b + 1) / (double)(2 * n),
                             tc3 = (double)(2 * c3 + 1) / (double)(2 * n);
                const D3 p{o.x + ta * h, o.y + tb * h, o.z + tc3 * h};
                cnt += inside64(sh, world2local(p, zero, q)) ? 1 : 0;
            }
    A.label[i] = (float)((double)cnt / (double)(n * n * n));
    if (A.recipe) {
        double* r = A.recipe + i * 20;
        r[0] = sh.type;
        for (int k = 0; k < 8; ++k) r[1 + k] = sh.p[k];
        r[9] = q.w; r[10] = q.v.x; r[11] = q.v.y; r[12] = q.v.z;
        r[13] = o.x; r[14] = o.y; r[15] = o.z;
        r[16] = h;
        r[17] = inside_cnt;
        r[18] = attempt;
        r[19] = 0.0;
    }
}

// ---- launch helpers ------------------------------------------------------------------------------------------------
static int g_smcount = 0;
int mlp_sm_count() {
    if (!g_smcount) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&g_smcount, cudaDevAttrMultiProcessorCount, dev);
        if (g_smcount <= 0) g_smcount = 1;
    }
    return g_smcount;
}

// shared-memory reservations of the MLP kernels (outside any stream capture: set before the first launch)
void mlp_prepare() {
    static std::once_flag once;
    std::call_once(once, [] {
        cudaFuncSetAttribute(mlp_infer_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, INF_SMEM);
        cudaFuncSetAttribute(mlp_grad_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, TR_SMEM);
    });
}

void launch_mlp_infer(const MlpInferArgs& a, int grid, cudaStream_t st) {
    mlp_prepare();
    mlp_infer_kernel<<<grid, MLP_THREADS, INF_SMEM, st>>>(a);
}

void launch_mlp_grad(const MlpGradArgs& a, int grid, cudaStream_t st) {
    mlp_prepare();
    mlp_grad_kernel<<<grid, MLP_THREADS, TR_SMEM, st>>>(a);
}

__device__ int32_t g_mlp_error;

static int32_t* error_ptr() {
    static int32_t* p = nullptr;
    if (!p) cudaGetSymbolAddress((void**)&p, g_mlp_error);
    return p;
}

// synchronises the stream and maps launch, runtime and device errors to a status
static int finish(cudaStream_t st) {
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return SDFIBM_ERR_CUDA;
    int32_t dev_err = 0;
    if (cudaMemcpyFromSymbol(&dev_err, g_mlp_error, sizeof(int32_t)) != cudaSuccess) return SDFIBM_ERR_CUDA;
    if (dev_err) {
        const int32_t zero = 0;
        cudaMemcpyToSymbol(g_mlp_error, &zero, sizeof(int32_t));
        return SDFIBM_ERR_TIMEOUT;
    }
    return SDFIBM_OK;
}

}  // namespace sdfibm_dev

using namespace sdfibm_dev;

extern "C" {

int sdfibm_mlp_dataset(uint64_t seed, int64_t n, const sdfibm_mlp_data_desc* desc, float* feat_dev, float* label_dev,
                       double* recipe_dev, void* stream) {
    if (!desc || n <= 0 || !feat_dev || !label_dev || desc->n_sub <= 0 || desc->n_sub > 64 || !(desc->hr_min > 0) ||
        !(desc->hr_max >= desc->hr_min))
        return SDFIBM_ERR_ARG;
    DataArgs A{};
    A.seed = seed;
    A.n = n;
    A.lhr_min = std::log(desc->hr_min);
    A.lhr_max = std::log(desc->hr_max);
    const int fams[6] = {SDFIBM_MLP_SPHERE, SDFIBM_MLP_ELLIPSOID, SDFIBM_MLP_BOX, SDFIBM_MLP_PLANE, SDFIBM_MLP_CYLINDER,
                         SDFIBM_MLP_ELLIPTIC_CYL};
    for (int k = 0; k < 6; ++k)
        if (desc->families & fams[k]) A.fam[A.nfam++] = fams[k];
    if (A.nfam == 0) return SDFIBM_ERR_ARG;
    A.n_sub = desc->n_sub;
    A.z_axis_frac = desc->z_axis_frac;
    A.feat = feat_dev;
    A.label = label_dev;
    A.recipe = recipe_dev;
    cudaStream_t st = (cudaStream_t)stream;
    mlp_dataset_kernel<<<(unsigned)((n + 127) / 128), 128, 0, st>>>(A);
    return finish(st);
}

int sdfibm_mlp_forward(const float* params_dev, const float* feat_dev, int64_t stride, int64_t n, float* out_dev,
                       void* stream) {
    if (!params_dev || !feat_dev || !out_dev || n < 0 || stride < n) return SDFIBM_ERR_ARG;
    if (n == 0) return SDFIBM_OK;
    MlpInferArgs a{};
    a.params = params_dev;
    a.feat = feat_dev;
    a.stride = stride;
    a.n = n;
    a.out = out_dev;
    a.error = error_ptr();
    cudaStream_t st = (cudaStream_t)stream;
    const int64_t ntiles = (n + MLP_TILE - 1) / MLP_TILE;
    launch_mlp_infer(a, (int)std::min<int64_t>(ntiles, 4 * mlp_sm_count()), st);
    return finish(st);
}

static int loss_grad_async(const float* params_dev, const float* feat_dev, const float* label_dev, int64_t stride,
                           int64_t n, float* grad_dev, cudaStream_t st) {
    if (cudaMemsetAsync(grad_dev, 0, sizeof(float) * (MLP_NPARAM + 1), st) != cudaSuccess) return SDFIBM_ERR_CUDA;
    MlpGradArgs a{};
    a.params = params_dev;
    a.feat = feat_dev;
    a.label = label_dev;
    a.stride = stride;
    a.n = n;
    a.scale = 2.0f / (float)n;
    a.grad = grad_dev;
    a.error = error_ptr();
    const int64_t ntiles = (n + MLP_TILE - 1) / MLP_TILE;
    launch_mlp_grad(a, (int)std::min<int64_t>(ntiles, mlp_sm_count()), st);
    return SDFIBM_OK;
}

int sdfibm_mlp_loss_grad(const float* params_dev, const float* feat_dev, const float* label_dev, int64_t stride,
                         int64_t n, float* grad_dev, void* stream) {
    if (!params_dev || !feat_dev || !label_dev || !grad_dev || n <= 0 || stride < n) return SDFIBM_ERR_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    const int r = loss_grad_async(params_dev, feat_dev, label_dev, stride, n, grad_dev, st);
    if (r != SDFIBM_OK) return r;
    return finish(st);
}

int sdfibm_mlp_adam(float* params_dev, const float* grad_dev, float* m_dev, float* v_dev, int32_t t, float lr,
                    void* stream) {
    if (!params_dev || !grad_dev || !m_dev || !v_dev || t < 1) return SDFIBM_ERR_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    const float c1 = (float)(1.0 / (1.0 - std::pow(0.9, t))), c2 = (float)(1.0 / (1.0 - std::pow(0.999, t)));
    mlp_adam_kernel<<<(MLP_NPARAM + 255) / 256, 256, 0, st>>>(params_dev, grad_dev, m_dev, v_dev, c1, c2, lr);
    return finish(st);
}

int sdfibm_mlp_train(float* params_dev, const float* feat_dev, const float* label_dev, int64_t n,
                     const sdfibm_mlp_train_desc* desc, float* loss_per_epoch_host, void* stream) {
    if (!params_dev || !feat_dev || !label_dev || !desc || n <= 0 || desc->epochs <= 0 || desc->batch <= 0)
        return SDFIBM_ERR_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    float* work = nullptr;  // grad [NPARAM+1], m, v, then one loss slot per step of an epoch
    const int64_t steps = (n + desc->batch - 1) / desc->batch;
    const size_t nwork = (size_t)3 * (MLP_NPARAM + 1) + (size_t)steps;
    if (cudaMalloc(&work, nwork * sizeof(float)) != cudaSuccess) return SDFIBM_ERR_CUDA;
    cudaMemsetAsync(work, 0, nwork * sizeof(float), st);
    float *grad = work, *m = work + (MLP_NPARAM + 1), *v = m + (MLP_NPARAM + 1), *losses = v + (MLP_NPARAM + 1);
    const int64_t total = steps * desc->epochs;
    int64_t t = 0;
    int rc = SDFIBM_OK;
    std::vector<float> lh((size_t)steps);
    for (int ep = 0; ep < desc->epochs && rc == SDFIBM_OK; ++ep) {
        for (int64_t s = 0; s < steps && rc == SDFIBM_OK; ++s) {
            const int64_t c0 = s * desc->batch, nb = std::min<int64_t>(desc->batch, n - c0);
            rc = loss_grad_async(params_dev, feat_dev + c0, label_dev + c0, n, nb, grad, st);
            ++t;
            double lr = desc->lr;
            if (t <= desc->warmup_steps) {
                lr *= (double)t / (double)std::max(1, desc->warmup_steps);
            } else {
                const double x = (double)(t - desc->warmup_steps) / (double)std::max<int64_t>(1, total - desc->warmup_steps);
                lr *= desc->lr_final_frac + (1.0 - desc->lr_final_frac) * 0.5 * (1.0 + std::cos(3.141592653589793 * x));
            }
            const float c1 = (float)(1.0 / (1.0 - std::pow(0.9, (double)t)));
            const float c2 = (float)(1.0 / (1.0 - std::pow(0.999, (double)t)));
            mlp_adam_kernel<<<(MLP_NPARAM + 255) / 256, 256, 0, st>>>(params_dev, grad, m, v, c1, c2, (float)lr);
            // the step's loss sum, kept on the device until the end of the epoch
            cudaMemcpyAsync(losses + s, grad + MLP_NPARAM, sizeof(float), cudaMemcpyDeviceToDevice, st);
        }
        if (rc != SDFIBM_OK) break;
        rc = finish(st);
        if (rc == SDFIBM_OK && loss_per_epoch_host) {
            if (cudaMemcpy(lh.data(), losses, (size_t)steps * sizeof(float), cudaMemcpyDeviceToHost) != cudaSuccess) {
                rc = SDFIBM_ERR_CUDA;
                break;
            }
            double sum = 0.0;
            for (float x : lh) sum += x;
            loss_per_epoch_host[ep] = (float)(sum / (double)n);
        }
    }
    cudaFree(work);
    return rc;
}

}  // extern "C"
