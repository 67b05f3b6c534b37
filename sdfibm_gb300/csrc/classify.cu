// Enumeration and cut-cell solid fraction: one pass over (solid, cell-tile) work items, then per-cell kernels.
//
// Each persistent CTA pulls tiles from an atomic counter.  For a tile it
//   1. skips tiles whose box cannot meet the solid's bounding sphere (prism: bounding disc) and zero-fills them;
//   2. evaluates the inside test once per tile vertex (FP32 with a rigorous error bound, FP64 re-check inside the
//      band -- identical answers to the reference's FP64 Solid::phi01) and writes one class byte per cell
//      (CellEnumerator::_next, src/cellenumerator.cpp:6-34): 0 no inside vertex, 1 all inside, 2 centre inside,
//      3 centre outside;
//   3. lists every cut candidate (class 2/3) for the fraction kernels:
//      REF-GEO   with the signed distances of its 8 vertices (two-float for 3-D spheres, ellipsoids and boxes, FP64
//                numerators elsewhere, see sdf_ff / sdf_mixed); refgeo_cells_kernel then runs
//                GeometricTools::calcCellVolume (src/geometrictools.cpp:13-116) in FP32 in cell-local coordinates
//                (vertices on {0,1}^3, every term a product of non-negative factors), a thread per cell;
//      SUBSAMPLE as (solid, fraction index); subsample_cells_kernel counts the n^3 (2-D: n^2) midpoint lattice of
//                each listed cell, a warp per cell, with the same exact inside test as the vertices (run counting
//                along lattice columns for the convex shapes), undecided points rechecked in FP64 by recheck_kernel;
//      LEARNED   as (solid, fraction index); learned_stencil_kernel (stencil.cu) computes the network's inputs and
//                band, the cells outside the band go to subsample_cells_kernel.
// The allocation-free entry point computes the fractions inside the tile pass instead.  Candidates that the flood
// fill later leaves out simply have their alpha ignored.
#include <cstdint>
#include <cuda_runtime.h>

#include "common.cuh"
#include "mlp.cuh"

namespace sdfibm_dev {


// ---- REF-GEO geometry in cell-local FP32 coordinates -------------------------------------------------------------------
// Vertex slots: 0:(i,j,k) 1:(i+1,j,k) 2:(i,j+1,k) 3:(i+1,j+1,k) 4..7 the same at k+1 (ascending point label); the face
// vertex orders are the ones the mesh stores (owner's hex-model face for internal faces, the cell's own for boundary
// faces), which fix the apex of each face.
__constant__ int8_t c_face_slots[9][4] = {
    {1, 3, 7, 5},  // x-max, owner order (internal +x face and x-max boundary face)
    {2, 6, 7, 3},  // y-max
    {4, 5, 7, 6},  // z-max
    {0, 4, 6, 2},  // x-min boundary face
    {0, 1, 5, 4},  // y-min boundary face
    {0, 2, 3, 1},  // z-min boundary face
    {0, 2, 6, 4},  // -x internal face (owner is the lower neighbour)
    {0, 4, 5, 1},  // -y internal face
    {0, 1, 3, 2},  // -z internal face
};

__device__ inline float lfrac32(float pa, float pb) {
    if (pa > 0.f && pb > 0.f) return 0.f;
    if (pa <= 0.f && pb <= 0.f) return 1.f;
    if (pa > 0.f) return -pb / (pa - pb);
    return -pa / (pb - pa);
}

// A point of the unit cell carried as, per axis, its coordinate v and 1 - v, both computed without cancellation:
// the apex of calcApex lies on the segment between two vertices of {0,1}^3, so each coordinate is 0, 1, t or 1 - t
// with t = |phiA| / (SMALL + |phiA| + |phiB|) and 1 - t = (SMALL + |phiB|) / (same), and every later use (pyramid
// heights, the in-face cross product) only needs the distance of the apex to a face plane 0 or 1 along one axis.
struct ApexPair {
    float v[3], w[3];
    __device__ float dist(int axis, int plane) const { return plane ? w[axis] : v[axis]; }
};

// GeometricTools::calcApex: first vertex A, first later vertex B of opposite (or zero) sign
__device__ inline ApexPair apex_pair(const float* ph, const int8_t* idx, int n) {
    const int A = idx[0];
    const float phiA = ph[A];
    int B = A;
    float phiB = 0.f;
    for (int i = 1; i < n; ++i) {
        B = idx[i];
        phiB = ph[B];
        // the sign of the reference's FP64 product phiA*phiB, without FP32 underflow of tiny values
        if (phiA == 0.f || phiB == 0.f || ((phiA > 0.f) != (phiB > 0.f))) break;
    }
    const float den = (float)SMALL_D + fabsf(phiA) + fabsf(phiB);
    const float t = fabsf(phiA) / den, u = ((float)SMALL_D + fabsf(phiB)) / den;
    ApexPair p;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const int ca = (A >> a) & 1, cb = (B >> a) & 1;
        if (ca == cb) { p.v[a] = (float)ca; p.w[a] = (float)(1 - ca); }
        else if (ca) { p.v[a] = u; p.w[a] = t; }   // 1 - t(1 - 0)
        else { p.v[a] = t; p.w[a] = u; }           // 0 - t(0 - 1)
    }
    return p;
}

// GeometricTools::calcFaceAreaFraction in units of the face area; `axis` is the face normal.  Each edge O->A runs
// along one in-face axis e; |(A-O) x (apex-O)| is then the apex's distance from O along the other in-face axis.
__device__ inline float face_fraction32(const float* ph, const int8_t* f, int axis) {
    int sign_sum = 0;
#pragma unroll
    for (int i = 0; i < 4; ++i) sign_sum += (ph[f[i]] > 0.f) ? 1 : -1;
    if (sign_sum == 4) return 0.f;
    if (sign_sum == -4) return 1.f;
    const ApexPair ap = apex_pair(ph, f, 4);
    float area = 0.f;
#pragma unroll
    for (int e = 0; e < 4; ++e) {
        const int o = f[e], a = f[(e + 1) & 3];
        const int diff = o ^ a;                       // one bit: the edge axis
        const int eax = diff == 1 ? 0 : (diff == 2 ? 1 : 2);
        const int oax = 3 - axis - eax;               // the other in-face axis
        const float c = ap.dist(oax, (o >> oax) & 1);
        area += 0.5f * c * lfrac32(ph[o], ph[a]);
    }
    return area;
}

// GeometricTools::calcCellVolume / V.  apz/apz1: local z of the 2-D apex plane and 1 minus it
// (geometrictools.cpp:57-58), unused in 3-D.
static __device__ __noinline__ float refgeo32(const MeshK& m, const float* ph, int64_t i, int64_t j, int64_t k, float apz, float apz1) {
    const int8_t order[8] = {0, 1, 2, 3, 4, 5, 6, 7};
    ApexPair ap = apex_pair(ph, order, 8);
    if (m.twod) { ap.v[2] = apz; ap.w[2] = apz1; }
    float vol = 0.f;
    auto acc = [&](int slot, int axis, int plane) {
        const float eps = face_fraction32(ph, c_face_slots[slot], axis);
        vol += (1.0f / 3.0f) * eps * ap.dist(axis, plane);
    };
    // mesh.cells()[c] order: owned internal (+x,+y,+z), boundary faces by patch, then -z,-y,-x
    if (i + 1 < m.nx) acc(0, 0, 1);
    if (j + 1 < m.ny) acc(1, 1, 1);
    if (k + 1 < m.nz) acc(2, 2, 1);
    if (i == 0) acc(3, 0, 0);
    if (i == m.nx - 1) acc(0, 0, 1);
    if (j == 0) acc(4, 1, 0);
    if (j == m.ny - 1) acc(1, 1, 1);
    if (k == 0) acc(5, 2, 0);
    if (k == m.nz - 1) acc(2, 2, 1);
    if (k > 0) acc(8, 2, 0);
    if (j > 0) acc(7, 1, 0);
    if (i > 0) acc(6, 0, 0);
    return vol;
}

// the oracle's FP64 sample point (i + (2a+1)/(2n), ...) and the reference's inside test, out of line (see
// exact_inside_point)
static __device__ __noinline__ int exact_inside_sample(const ShapeK& sh, const MeshK& m, int64_t i, int64_t j, int64_t k,
                                                int a, int b, int c3, int n, const D3& x, const Q4& q) {
    const double ta64 = (double)(2 * a + 1) / (double)(2 * n), tb64 = (double)(2 * b + 1) / (double)(2 * n);
    const double tc64 = m.twod ? 0.5 : (double)(2 * c3 + 1) / (double)(2 * n);
    const D3 p{m.o[0] + ((double)i + ta64) * m.h[0], m.o[1] + ((double)j + tb64) * m.h[1],
               m.o[2] + ((double)k + tc64) * m.h[2]};
    return inside64(sh, world2local(p, x, q)) ? 1 : 0;
}

// Where an undecided SUBSAMPLE point goes: appended to the recheck list (counted later by recheck_kernel) when there
// is room, else re-evaluated here.  DEFER_ONLY kernels carry no FP64 path: a point the full list cannot take sets the
// warp's overflow flag instead, and the cell is recounted by recount_kernel.
struct Defer {
    Recheck* rq;
    int64_t cap;
    int32_t* count;
    int64_t idx;
    int32_t solid;
    int32_t* overflow;  // DEFER_ONLY: the warp's flag in shared memory
};
template <bool DEFER_ONLY>
static __device__ __forceinline__ int undecided_sample(const Defer* df, const ShapeK& sh, const MeshK& m, int64_t i,
                                                       int64_t j, int64_t k, int a, int b, int c3, int n, const D3& x,
                                                       const Q4& q) {
    if (df) {
        const int slot = atomicAdd(df->count, 1);
        if (slot < df->cap) {
            df->rq[slot] = Recheck{df->idx, df->solid,
                                   (uint32_t)a | ((uint32_t)b << 8) | ((uint32_t)c3 << 16) | ((uint32_t)n << 24)};
            return 0;
        }
        if (DEFER_ONLY) {
            *(volatile int32_t*)df->overflow = 1;
            return 0;
        }
    }
    if (DEFER_ONLY) return 0;  // DEFER_ONLY callers always pass a Defer
    return exact_inside_sample(sh, m, i, j, k, a, b, c3, n, x, q);
}

// the reference's FP64 Solid::phi of mesh point (I,J,K), out of line
static __device__ __noinline__ float exact_phi_point(const ShapeK& sh, const MeshK& m, int64_t I, int64_t J, int64_t K,
                                              const D3& x, const Q4& q) {
    const D3 p{m.o[0] + (double)I * m.h[0], m.o[1] + (double)J * m.h[1], m.o[2] + (double)K * m.h[2]};
    return (float)sdf64(sh, world2local(p, x, q));
}

// ---- SUBSAMPLE: one warp per cut cell ----------------------------------------------------------------------------------
// Each lane owns (a,b) columns of the n x n x n midpoint lattice and walks its column in z.  Local coordinates step by
// three precomputed vectors (the columns of the world->local map times h).  One error bound E covers every sample
// coordinate of the cell; for the convex shapes the bound of the inside function is also taken once per cell, from
// the largest coordinate any sample can have, so a sample costs a few FMAs and two compares.  Undecided samples are
// re-evaluated with the oracle's FP64 point formula.

// sample frame of one cell: corner point p (shape centre offset folded in for the convex shapes), steps s*, bounds
struct SampleFrame {
    float px, py, pz;
    float sxx, sxy, sxz, syx, syy, syz, szx, szy, szz;
    float E;   // bound of |computed - exact| of every sample coordinate (without the folded offset)
    float Eg;  // bound of |computed - exact| of the inside function (convex shapes, offset folded)
    float k0, k1, k2, k3;  // quadric X^2 k0 + Y^2 k1 + Z^2 k2 - k3, or box half extents k0..k2
};

__device__ __forceinline__ int band(float g, float Eg) { return g < -Eg ? 1 : (g > Eg ? 0 : 2); }

constexpr int SS_QUADRIC = 0, SS_BOX = 1, SS_GENERIC = 2;

// inside function of the convex shapes at a local point (negative inside), within f.Eg of its exact value
template <int T>
__device__ __forceinline__ float sample_g(const SampleFrame& f, float X, float Y, float Z) {
    if (T == SS_QUADRIC) return __fmaf_rn(X * X, f.k0, __fmaf_rn(Y * Y, f.k1, (Z * Z) * f.k2)) - f.k3;
    return fmaxf(fmaxf(fabsf(X) - f.k0, fabsf(Y) - f.k1), fabsf(Z) - f.k2);
}

template <int T>
__device__ __forceinline__ int sample_inside(const ShapeK& sh, const SampleFrame& f, float X, float Y, float Z) {
    if (T == SS_QUADRIC || T == SS_BOX) return band(sample_g<T>(f, X, Y, Z), f.Eg);
    return inside32(sh, X, Y, Z, f.E);  // tails and planes: the general test with its per-sample bound
}

template <int T, bool DEFER_ONLY>
__device__ __forceinline__ int subsample_count(const MeshK& m, const ShapeK& sh, const SampleFrame& f, int64_t i,
                                               int64_t j, int64_t k, int n, const D3& x, const Q4& q,
                                               unsigned long long* rechecks, const Defer* df) {
    const int lane = threadIdx.x & 31;
    const int nzs = m.twod ? 1 : n;
    const float inv2n = 1.0f / (float)(2 * n);
    int cnt = 0;
#pragma unroll 1
    for (int col = lane; col < n * n; col += 32) {
        const int ia = col % n, ib = col / n;
        const float ta = (float)(2 * ia + 1) * inv2n, tb = (float)(2 * ib + 1) * inv2n;
        const float bx = __fmaf_rn(tb, f.syx, __fmaf_rn(ta, f.sxx, f.px));
        const float by = __fmaf_rn(tb, f.syy, __fmaf_rn(ta, f.sxy, f.py));
        const float bz = __fmaf_rn(tb, f.syz, __fmaf_rn(ta, f.sxz, f.pz));
        float odd = 1.f;  // 2*c3 + 1, exact
#pragma unroll 2
        for (int c3 = 0; c3 < nzs; ++c3) {
            const float tc = m.twod ? 0.5f : odd * inv2n;
            odd += 2.f;
            int r = sample_inside<T>(sh, f, __fmaf_rn(tc, f.szx, bx), __fmaf_rn(tc, f.szy, by),
                                     __fmaf_rn(tc, f.szz, bz));
            if (r == 2) {
                ++*rechecks;
                r = undecided_sample<DEFER_ONLY>(df, sh, m, i, j, k, ia, ib, c3, n, x, q);
            }
            cnt += r;
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
    return cnt;
}

// Block-skipping count for the quadrics and boxes: the lattice is split into B x B x B blocks (B x B x 1 on one-layer
// meshes).  For each block the inside function is bounded over the box of local coordinates that holds the block's
// samples (centre +- half the block's span along the three step vectors, widened by the coordinate error bound Ep);
// a block whose upper bound is below -Eg has every sample inside in the reference's FP64 evaluation, one whose
// lower bound is above Eg has none, and only the remaining blocks are sampled, with the same coordinate sequence
// and per-sample bound as subsample_count.  The count is therefore the exhaustive lattice count.
template <int T>
__device__ __forceinline__ void block_bounds(const SampleFrame& f, float X, float Y, float Z, float hx, float hy,
                                             float hz, float& gmin, float& gmax) {
    const float xl = X - hx, xh = X + hx, yl = Y - hy, yh = Y + hy, zl = Z - hz, zh = Z + hz;
    const float ax = fmaxf(fabsf(xl), fabsf(xh)), ay = fmaxf(fabsf(yl), fabsf(yh)), az = fmaxf(fabsf(zl), fabsf(zh));
    const float bx = (xl <= 0.f && xh >= 0.f) ? 0.f : fminf(fabsf(xl), fabsf(xh));
    const float by = (yl <= 0.f && yh >= 0.f) ? 0.f : fminf(fabsf(yl), fabsf(yh));
    const float bz = (zl <= 0.f && zh >= 0.f) ? 0.f : fminf(fabsf(zl), fabsf(zh));
    if (T == SS_QUADRIC) {
        gmax = __fmaf_rn(ax * ax, f.k0, __fmaf_rn(ay * ay, f.k1, (az * az) * f.k2)) - f.k3;
        gmin = __fmaf_rn(bx * bx, f.k0, __fmaf_rn(by * by, f.k1, (bz * bz) * f.k2)) - f.k3;
    } else {
        gmax = fmaxf(fmaxf(ax - f.k0, ay - f.k1), az - f.k2);
        gmin = fmaxf(fmaxf(bx - f.k0, by - f.k1), bz - f.k2);
    }
}

template <int T, bool DEFER_ONLY>
__device__ __noinline__ int subsample_blocks(const MeshK& m, const ShapeK& sh, const SampleFrame& f, int64_t i,
                                             int64_t j, int64_t k, int n, int lb, float Ep, const D3& x, const Q4& q,
                                             unsigned long long* rechecks, const Defer* df) {
    __shared__ uint16_t s_und[8][128];  // undecided blocks of each warp, (ba, bb, bc) packed 5 bits each
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    uint16_t* list = s_und[(threadIdx.x >> 5) & 7];
    const bool flat = m.twod != 0;
    const int B = 1 << lb, nb = n >> lb, nbz = flat ? 1 : nb;
    const int lsz = flat ? 2 * lb : 3 * lb;  // log2 of the samples per block
    const int nblocks = nb * nb * nbz;
    const float inv2n = 1.0f / (float)(2 * n);
    // half span of a block along each step vector (t from its first to its last sample), widened by a relative 1e-6
    const float half = 0.5f * (float)(2 * (B - 1)) * inv2n * 1.000001f;
    const float halfz = flat ? 0.f : half;
    const float hx = half * (fabsf(f.sxx) + fabsf(f.syx)) + halfz * fabsf(f.szx) + Ep;
    const float hy = half * (fabsf(f.sxy) + fabsf(f.syy)) + halfz * fabsf(f.szy) + Ep;
    const float hz = half * (fabsf(f.sxz) + fabsf(f.syz)) + halfz * fabsf(f.szz) + Ep + U32 * fabsf(f.pz);
    int cnt = 0, nund = 0;
    for (int base = 0; base < nblocks; base += 32) {
        const int blk = base + lane;
        bool undecided = false;
        int packed = 0;
        if (blk < nblocks) {
            const int ba = blk % nb, bb = (blk / nb) % nb, bc = blk / (nb * nb);
            packed = ba | (bb << 5) | (bc << 10);
            const float ta = (float)(2 * ba * B + B) * inv2n, tb = (float)(2 * bb * B + B) * inv2n;
            const float tc = flat ? 0.5f : (float)(2 * bc * B + B) * inv2n;
            const float X = __fmaf_rn(tc, f.szx, __fmaf_rn(tb, f.syx, __fmaf_rn(ta, f.sxx, f.px)));
            const float Y = __fmaf_rn(tc, f.szy, __fmaf_rn(tb, f.syy, __fmaf_rn(ta, f.sxy, f.py)));
            const float Z = __fmaf_rn(tc, f.szz, __fmaf_rn(tb, f.syz, __fmaf_rn(ta, f.sxz, f.pz)));
            float gmin, gmax;
            block_bounds<T>(f, X, Y, Z, hx, hy, hz, gmin, gmax);
            if (gmax < -f.Eg) cnt += 1 << lsz;
            else if (!(gmin > f.Eg)) undecided = true;
        }
        const unsigned mask = __ballot_sync(FULL, undecided);
        if (undecided) list[nund + __popc(mask & ((1u << lane) - 1u))] = (uint16_t)packed;
        nund += __popc(mask);
    }
    __syncwarp();
    // the undecided blocks' columns: one (block, a, b) column per slot, walked along c as subsample_count does
    const int lcol = 2 * lb;  // log2 of the columns per block
    const int slots = nund << lcol;
    const int Bz = flat ? 1 : B;
    for (int e = lane; e < slots; e += 32) {
        const int pk = list[e >> lcol], col = e & ((1 << lcol) - 1);
        const int ia = ((pk & 31) << lb) + (col & (B - 1)), ib = (((pk >> 5) & 31) << lb) + (col >> lb);
        const int ic0 = ((pk >> 10) & 31) << lb;
        const float ta = (float)(2 * ia + 1) * inv2n, tb = (float)(2 * ib + 1) * inv2n;
        const float bx = __fmaf_rn(tb, f.syx, __fmaf_rn(ta, f.sxx, f.px));
        const float by = __fmaf_rn(tb, f.syy, __fmaf_rn(ta, f.sxy, f.py));
        const float bz = __fmaf_rn(tb, f.syz, __fmaf_rn(ta, f.sxz, f.pz));
        float odd = (float)(2 * ic0 + 1);  // 2*ic + 1, exact
        for (int dc = 0; dc < Bz; ++dc, odd += 2.f) {
            const float tc = flat ? 0.5f : odd * inv2n;
            int res = sample_inside<T>(sh, f, __fmaf_rn(tc, f.szx, bx), __fmaf_rn(tc, f.szy, by),
                                       __fmaf_rn(tc, f.szz, bz));
            if (res == 2) {
                ++*rechecks;
                res = undecided_sample<DEFER_ONLY>(df, sh, m, i, j, k, ia, ib, flat ? 0 : ic0 + dc, n, x, q);
            }
            cnt += res;
        }
    }
    __syncwarp();
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) cnt += __shfl_xor_sync(FULL, cnt, o);
    return cnt;
}

// log2 of the block edge for block skipping (power of two of at least 4 dividing n, at most 128 blocks), 0: sample
// every point (blocks of 2 samples per axis cost more to test than they save)
__device__ inline int block_log2(int n, bool flat) {
    for (int lb = 2; lb <= 3; ++lb) {
        const int B = 1 << lb;
        if (n % B) continue;
        const int nb = n / B;
        if ((flat ? nb * nb : nb * nb * nb) <= 128) return lb;
    }
    return 0;
}

// Run counting for the convex shapes (3-D): the inside samples of a lattice column (a, b) are one run, since the
// exact inside function q is convex along the column's line.  Along the column the local coordinates are
// w + c d (c the sample index), so the quadric is the polynomial A c^2 + 2 B c + C and the box the maximum of three
// |w + c d| - k.  The run's ends come from their FP32 roots (any error there only costs time); the polynomial values
// at a few samples, within Egh of q there, then decide the whole column:
//   run [c1, c2] found: c1 and c2 inside, c1 - 1 and c2 + 1 outside (or off the column).  Every sample between the
//     ends is inside (q there is at most its value at the ends) and every sample past c2 + 1 outside (q grows past a
//     rise from an inside to an outside sample), and likewise before c1 - 1;
//   no sample in the interval: the samples cv and cv + 1 around the closest approach outside, with q certified to
//     rise from cv to cv - 1 and from cv + 1 to cv + 2 (computed rise of at least 2 Egh); every sample past them is
//     then outside.  For the box, a slab that holds neither end of the column (on the same side) settles it first.
// A column that does not verify (a value within Egh of zero, a run end off by one, a flat approach) is walked sample
// by sample with the coordinates, bound and deferral of subsample_count.  The count is therefore the exhaustive
// lattice count.
//
// Egh: the polynomial's value differs from the walk's coordinates-then-shape evaluation by the roundings of w, d,
// the coefficients and the Horner steps, each a few units of roundoff of the magnitudes sum k X^2 + k3 (quadric) or
// max |X| + max k (box) over the cell; the caller adds 64 (quadric) or 32 (box) units of roundoff of those sums to Eg.
template <int T, bool DEFER_ONLY>
__device__ __forceinline__ int subsample_runs_body(const MeshK& m, const ShapeK& sh, const SampleFrame& f, float Egh,
                                                   int64_t i, int64_t j, int64_t k, int n, const D3& x, const Q4& q,
                                                   unsigned long long* rechecks, const Defer* df) {
    __shared__ uint16_t s_walk[8][128];  // columns of each warp left to the sample-by-sample walk
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    uint16_t* walk_list = s_walk[(threadIdx.x >> 5) & 7];
    // correctly rounded reciprocals (the same values as 1.0f / x, without the division sequence)
    const float inv2n = __frcp_rn((float)(2 * n)), nf = (float)n, invn = __frcp_rn(nf);
    const float rise = 2.0001f * Egh;
    // per-sample step along the column and the per-cell parts of the polynomial
    const float dx = f.szx * invn, dy = f.szy * invn, dz = f.szz * invn;
    const float kdx = f.k0 * dx, kdy = f.k1 * dy, kdz = f.k2 * dz;
    const float A = __fmaf_rn(dx, kdx, __fmaf_rn(dy, kdy, dz * kdz));
    const float invA = __frcp_rn(A);
    const float idx_ = __frcp_rn(dx), idy = __frcp_rn(dy), idz = __frcp_rn(dz);
    const float kx0 = f.k0 * idx_, ky0 = f.k1 * idy, kz0 = f.k2 * idz;
    auto column_base = [&](int col, int& ia, int& ib, float& bx, float& by, float& bz) {
        ib = __float2int_rz(((float)col + 0.5f) * invn);
        ia = col - ib * n;
        const float ta = (float)(2 * ia + 1) * inv2n, tb = (float)(2 * ib + 1) * inv2n;
        bx = __fmaf_rn(tb, f.syx, __fmaf_rn(ta, f.sxx, f.px));
        by = __fmaf_rn(tb, f.syy, __fmaf_rn(ta, f.sxy, f.py));
        bz = __fmaf_rn(tb, f.syz, __fmaf_rn(ta, f.sxz, f.pz));
    };
    // the walk's sample: the same coordinates, bound and deferral as subsample_count
    auto walk_sample = [&](int ia, int ib, int c3, float bx, float by, float bz) {
        const float tc = (float)(2 * c3 + 1) * inv2n;
        int r = band(sample_g<T>(f, __fmaf_rn(tc, f.szx, bx), __fmaf_rn(tc, f.szy, by), __fmaf_rn(tc, f.szz, bz)),
                     f.Eg);
        if (r == 2) {
            ++*rechecks;
            r = undecided_sample<DEFER_ONLY>(df, sh, m, i, j, k, ia, ib, c3, n, x, q);
        }
        return r;
    };
    int cnt = 0, nwalk = 0;
#pragma unroll 1
    for (int base = 0; base < n * n; base += 32) {
        const int col = base + lane;
        int res = 0;
        int ia = 0, ib = 0;
        float bx = 0.f, by = 0.f, bz = 0.f;
        if (col < n * n) {
            column_base(col, ia, ib, bx, by, bz);
            // coordinates of sample c: w + c d
            const float wx = __fmaf_rn(f.szx, inv2n, bx), wy = __fmaf_rn(f.szy, inv2n, by),
                        wz = __fmaf_rn(f.szz, inv2n, bz);
            float B2 = 0.f, C = 0.f;
            float cl, cr;
            if (T == SS_QUADRIC) {
                const float B = __fmaf_rn(wx, kdx, __fmaf_rn(wy, kdy, wz * kdz));
                C = __fmaf_rn(wx * wx, f.k0, __fmaf_rn(wy * wy, f.k1, (wz * wz) * f.k2)) - f.k3;
                B2 = 2.f * B;
                const float disc = __fmaf_rn(B, B, -A * C);
                const float sq = disc > 0.f ? disc * rsqrtf(disc) : 0.f;  // approximate: only locates the run
                cl = (-B - sq) * invA;
                cr = disc > 0.f ? (-B + sq) * invA : cl - 1.f;  // empty: cl marks the closest approach
            } else {
                const float lx = __fmaf_rn(-wx, idx_, -kx0), rx = __fmaf_rn(-wx, idx_, kx0);
                const float ly = __fmaf_rn(-wy, idy, -ky0), ry = __fmaf_rn(-wy, idy, ky0);
                const float lz = __fmaf_rn(-wz, idz, -kz0), rz = __fmaf_rn(-wz, idz, kz0);
                cl = fmaxf(fmaxf(fminf(lx, rx), fminf(ly, ry)), fminf(lz, rz));
                cr = fminf(fminf(fmaxf(lx, rx), fmaxf(ly, ry)), fmaxf(lz, rz));
            }
            auto g_at = [&](int c3) {
                const float c = (float)c3;
                if (T == SS_QUADRIC) return __fmaf_rn(__fmaf_rn(A, c, B2), c, C);
                return fmaxf(fmaxf(fabsf(__fmaf_rn(c, dx, wx)) - f.k0, fabsf(__fmaf_rn(c, dy, wy)) - f.k1),
                             fabsf(__fmaf_rn(c, dz, wz)) - f.k2);
            };
            // clamped before the conversions (inf / NaN safe)
            const float ul = fminf(fmaxf(cl, -2.f), nf + 1.f), ur = fminf(fmaxf(cr, -2.f), nf + 1.f);
            const int c1 = max((int)ceilf(ul), 0), c2 = min((int)floorf(ur), n - 1);
            // inside: g < -Egh, outside: g > Egh (band() of the walk, as plain comparisons)
            res = -1;
            if (cl <= cr && c1 <= c2) {
                bool ok = g_at(c1) < -Egh && (c2 == c1 || g_at(c2) < -Egh);
                if (ok && c1 > 0) ok = g_at(c1 - 1) > Egh;
                if (ok && c2 < n - 1) ok = g_at(c2 + 1) > Egh;
                if (ok) res = c2 - c1 + 1;
            } else {
                // the pair cv, cv + 1 around the closest approach: both outside, q rising from cv to cv - 1 and
                // from cv + 1 to cv + 2 (a pair rather than one sample: with the approach halfway between two
                // samples, the rise from the nearer one to the other would be about zero)
                float um = (T == SS_QUADRIC && !(cl <= cr)) ? ul : 0.5f * (ul + ur);
                bool separated = false;
                if (T == SS_BOX) {
                    // a slab whose coordinate is beyond it at both ends of the column, on the same side, holds no
                    // sample (the coordinate is linear along the column; computed within Egh of q at the ends)
                    const float last = nf - 1.f;
                    auto beyond = [&](float w0, float d0, float k0) {
                        const float x1 = __fmaf_rn(last, d0, w0);
                        return (w0 > 0.f) == (x1 > 0.f) && fabsf(w0) - k0 > Egh && fabsf(x1) - k0 > Egh;
                    };
                    separated = beyond(wx, dx, f.k0) || beyond(wy, dy, f.k1) || beyond(wz, dz, f.k2);
                }
                if (separated) {
                    res = 0;
                } else {
                    const int cv = min(max(__float2int_rd(fminf(fmaxf(um, 0.f), nf - 2.f)), 0), n - 2);
                    const float g0 = g_at(cv), g1 = g_at(cv + 1);
                    bool ok = g0 > Egh && g1 > Egh;
                    if (ok && cv >= 1) ok = g_at(cv - 1) - g0 >= rise;
                    if (ok && cv + 2 <= n - 1) ok = g_at(cv + 2) - g1 >= rise;
                    if (ok) res = 0;
                }
            }
        }
        const bool walk = res < 0;
        const unsigned mask = __ballot_sync(FULL, walk);
        const int pos = nwalk + __popc(mask & ((1u << lane) - 1u));
        nwalk += __popc(mask);
        if (walk) {
            if (pos < 128) {
                walk_list[pos] = (uint16_t)col;
            } else {  // list full: walk here
                for (int c3 = 0; c3 < n; ++c3) cnt += walk_sample(ia, ib, c3, bx, by, bz);
            }
        } else {
            cnt += res;
        }
    }
    __syncwarp();
    // the listed columns' samples spread over the lanes
    const int listed = min(nwalk, 128);
#pragma unroll 1
    for (int e = lane; e < listed * n; e += 32) {
        const int w = __float2int_rz(((float)e + 0.5f) * invn), c3 = e - w * n;
        int ia, ib;
        float bx, by, bz;
        column_base(walk_list[w], ia, ib, bx, by, bz);
        cnt += walk_sample(ia, ib, c3, bx, by, bz);
    }
    __syncwarp();
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) cnt += __shfl_xor_sync(FULL, cnt, o);
    return cnt;
}

// out of line for the classify pass; the fallback kernel inlines the body (DEFER_ONLY, no FP64 path)
template <int T, bool DEFER_ONLY>
__device__ __noinline__ int subsample_runs(const MeshK& m, const ShapeK& sh, const SampleFrame& f, float Egh, int64_t i,
                                           int64_t j, int64_t k, int n, const D3& x, const Q4& q,
                                           unsigned long long* rechecks, const Defer* df) {
    return subsample_runs_body<T, DEFER_ONLY>(m, sh, f, Egh, i, j, k, n, x, q, rechecks, df);
}

// Inside count of the cell's n^3 (n^2 on one-layer meshes) lattice; with a Defer the undecided points are not counted
// here but appended to the recheck list.  DEFER_ONLY: x, q and (i, j, k) only feed the FP64 path, which it lacks.
template <bool DEFER_ONLY>
static __device__ __forceinline__ int subsample_warp_body(const MeshK& m, const ShapeK& sh, const float* M,
                                                          const TileFrame& tf, int a0, int b0, int c0, const D3& x,
                                                          const Q4& q, int64_t i, int64_t j, int64_t k, int n,
                                                          unsigned long long* rechecks, const Defer* df) {
    const float u = U32;
    const float hx = m.h32[0], hy = m.h32[1], hz = m.h32[2];
    const float ox = (float)a0 * hx, oy = (float)b0 * hy, oz = (float)c0 * hz;  // cell corner within the tile
    const float dx = tf.bx + ox, dy = tf.by + oy, dz = tf.bz + oz;
    SampleFrame f;
    f.px = __fmaf_rn(M[0], dx, __fmaf_rn(M[1], dy, M[2] * dz));
    f.py = __fmaf_rn(M[3], dx, __fmaf_rn(M[4], dy, M[5] * dz));
    f.pz = __fmaf_rn(M[6], dx, __fmaf_rn(M[7], dy, M[8] * dz));
    f.sxx = M[0] * hx; f.sxy = M[3] * hx; f.sxz = M[6] * hx;
    f.syx = M[1] * hy; f.syy = M[4] * hy; f.syz = M[7] * hy;
    f.szx = M[2] * hz; f.szy = M[5] * hz; f.szz = M[8] * hz;
    const float sabs = fabsf(f.sxx) + fabsf(f.sxy) + fabsf(f.sxz) + fabsf(f.syx) + fabsf(f.syy) + fabsf(f.syz) +
                       fabsf(f.szx) + fabsf(f.szy) + fabsf(f.szz);
    f.E = 8.f * u * (tf.babs + fabsf(ox) + fabsf(oy) + fabsf(oz) + 2.f * (fabsf(dx) + fabsf(dy) + fabsf(dz)) +
                     3.f * (hx + hy + hz)) +
          8.f * u * (fabsf(f.px) + fabsf(f.py) + fabsf(f.pz) + sabs) + tf.e64 + 1e-30f;
    const int type = sh.type;
    const bool prism = sh.prism;
    const float* a = sh.p32;
    int kind = SS_GENERIC;
    if (type == SDFIBM_SHAPE_CIRCLE || type == SDFIBM_SHAPE_SPHERE || type == SDFIBM_SHAPE_ELLIPSE ||
        type == SDFIBM_SHAPE_ELLIPSOID)
        kind = SS_QUADRIC;
    else if (type == SDFIBM_SHAPE_RECTANGLE || type == SDFIBM_SHAPE_BOX)
        kind = SS_BOX;
    float Ep = f.E;
    if (kind != SS_GENERIC) {
        // sample = (corner + com) + steps: one more rounding of the corner, the conversion of com to FP32, and the
        // stepping FMAs now run at magnitudes up to |com| larger (the ellipsoid ignores com, as the reference does)
        const bool use_com = type != SDFIBM_SHAPE_ELLIPSOID;
        const float c0x = use_com ? sh.com32[0] : 0.f, c0y = use_com ? sh.com32[1] : 0.f;
        f.px += c0x;
        f.py += c0y;
        if (prism) {
            // 2-D shapes: the local z is the FP32 com z for every sample (exact steps of zero)
            f.pz = sh.com32[2];
            f.sxz = 0.f; f.syz = 0.f; f.szz = 0.f;
        } else if (use_com) {
            f.pz += sh.com32[2];
        }
        const float cabs = use_com ? fabsf(sh.com32[0]) + fabsf(sh.com32[1]) + fabsf(sh.com32[2]) : 0.f;
        Ep = f.E + 2.f * u * (fabsf(f.px) + fabsf(f.py) + fabsf(f.pz) + sabs) + 5.f * u * cabs;
    }
    // largest |coordinate| any sample of the cell can reach
    const float mx = fabsf(f.px) + fabsf(f.sxx) + fabsf(f.syx) + fabsf(f.szx) + Ep;
    const float my = fabsf(f.py) + fabsf(f.sxy) + fabsf(f.syy) + fabsf(f.szy) + Ep;
    const float mz = fabsf(f.pz) + fabsf(f.sxz) + fabsf(f.syz) + fabsf(f.szz) + Ep;
    // 3-D convex shapes count runs along columns from 5 samples per axis; out of line (the classify pass), lattices
    // of 16 and more skip 4 x 4 x 4 blocks instead
    const bool use_runs = !m.twod && !prism && n >= 5 && (DEFER_ONLY || n < 16);
    int cnt;
    if (kind == SS_QUADRIC) {
        switch (type) {
            case SDFIBM_SHAPE_CIRCLE:
            case SDFIBM_SHAPE_SPHERE: f.k0 = 1.f; f.k1 = 1.f; f.k2 = 1.f; f.k3 = a[1]; break;
            case SDFIBM_SHAPE_ELLIPSE: f.k0 = a[2]; f.k1 = a[3]; f.k2 = 0.f; f.k3 = 1.f; break;
            default: f.k0 = a[3]; f.k1 = a[4]; f.k2 = a[5]; f.k3 = 1.f; break;
        }
        f.Eg = (2.f * (mx * f.k0 + my * f.k1 + mz * f.k2) + Ep * (f.k0 + f.k1 + f.k2)) * Ep +
               10.f * u * (mx * mx * f.k0 + my * my * f.k1 + mz * mz * f.k2 + f.k3);
        const float Egh = f.Eg + 64.f * u * (mx * mx * f.k0 + my * my * f.k1 + mz * mz * f.k2 + f.k3);
        const int lb = block_log2(n, m.twod != 0);
        if (use_runs && DEFER_ONLY)
            cnt = subsample_runs_body<SS_QUADRIC, true>(m, sh, f, Egh, i, j, k, n, x, q, rechecks, df);
        else if (use_runs)
            cnt = subsample_runs<SS_QUADRIC, DEFER_ONLY>(m, sh, f, Egh, i, j, k, n, x, q, rechecks, df);
        else if (lb)
            cnt = subsample_blocks<SS_QUADRIC, DEFER_ONLY>(m, sh, f, i, j, k, n, lb, Ep, x, q, rechecks, df);
        else
            cnt = subsample_count<SS_QUADRIC, DEFER_ONLY>(m, sh, f, i, j, k, n, x, q, rechecks, df);
    } else if (kind == SS_BOX) {
        f.k0 = a[0]; f.k1 = a[1];
        f.k2 = prism ? INFINITY : a[2];  // the rectangle has no z extent
        f.Eg = Ep + 2.f * u * (fmaxf(mx, fmaxf(my, prism ? 0.f : mz)) + fmaxf(a[0], fmaxf(a[1], prism ? 0.f : a[2])));
        const float Egh = f.Eg + 32.f * u * (fmaxf(mx, fmaxf(my, mz)) + fmaxf(a[0], fmaxf(a[1], a[2])));
        const int lb = block_log2(n, m.twod != 0);
        if (use_runs && DEFER_ONLY)
            cnt = subsample_runs_body<SS_BOX, true>(m, sh, f, Egh, i, j, k, n, x, q, rechecks, df);
        else if (use_runs)
            cnt = subsample_runs<SS_BOX, DEFER_ONLY>(m, sh, f, Egh, i, j, k, n, x, q, rechecks, df);
        else if (lb)
            cnt = subsample_blocks<SS_BOX, DEFER_ONLY>(m, sh, f, i, j, k, n, lb, Ep, x, q, rechecks, df);
        else
            cnt = subsample_count<SS_BOX, DEFER_ONLY>(m, sh, f, i, j, k, n, x, q, rechecks, df);
    } else {
        cnt = subsample_count<SS_GENERIC, DEFER_ONLY>(m, sh, f, i, j, k, n, x, q, rechecks, df);
    }
    return cnt;
}

// the out-of-line form of the classify pass and of the recount (FP64 path included)
static __device__ __noinline__ int subsample_warp(const MeshK& m, const ShapeK& sh, const float* M, const TileFrame& tf,
                                                  int a0, int b0, int c0, const D3& x, const Q4& q, int64_t i,
                                                  int64_t j, int64_t k, int n, unsigned long long* rechecks,
                                                  const Defer* df) {
    return subsample_warp_body<false>(m, sh, M, tf, a0, b0, c0, x, q, i, j, k, n, rechecks, df);
}

// the fraction of a complete count (cnt and n^3 are exact in FP32: one correct rounding)
__device__ inline float count_fraction(const MeshK& m, int cnt, int n) {
    return __fdiv_rn((float)cnt, (float)(n * n * (m.twod ? 1 : n)));
}

// ---- signed distance for REF-GEO: FP64 where it decides, FP32 where it only scales ------------------------------------
// The geometry consumes phi in FP32, so phi needs ~1e-7 relative accuracy and the reference's exact sign and filter
// (|phi| < 1e-8 -> -1e-8).  The local point and every cancelling difference (|p|^2 - r^2, |x| - a, ...) are FP64; the
// square roots and the final division only scale a non-cancelling quantity and run in FP32.  Values within 1e-6 of
// the filter threshold are recomputed with the reference's full FP64 sequence by the caller.
__device__ inline float rect_mixed(double x, double y, double ra, double rb) {
    const double dx = fabs(x) - ra, dy = fabs(y) - rb;
    const double dxp = dmax(0.0, dx), dyp = dmax(0.0, dy);
    return sqrtf((float)(dxp * dxp + dyp * dyp)) + (float)dmin(0.0, dmax(dx, dy));
}
static __device__ __noinline__ float sdf_mixed(const ShapeK& s, const D3& p) {
    const double* a = s.p;
    const D3 com{s.com[0], s.com[1], s.com[2]};
    switch (s.type) {
        case SDFIBM_SHAPE_CIRCLE: {
            const D3 q = com + D3{p.x, p.y, 0.0};
            const double qq = magSqr(q);
            return (float)(qq - a[1]) / (sqrtf((float)qq) + (float)a[0]);
        }
        case SDFIBM_SHAPE_SPHERE: {
            const D3 q = com + p;
            const double qq = magSqr(q);
            return (float)(qq - a[1]) / (sqrtf((float)qq) + (float)a[0]);
        }
        case SDFIBM_SHAPE_ELLIPSE: {
            const D3 q = com + p;
            const double xa = q.x * q.x * a[2], yb = q.y * q.y * a[3];
            return (float)(0.5 * (xa + yb - 1.0)) / sqrtf((float)(xa * a[2] + yb * a[3]));
        }
        case SDFIBM_SHAPE_ELLIPSOID: {
            const double xa = p.x * p.x * a[3], yb = p.y * p.y * a[4], zc = p.z * p.z * a[5];
            return (float)(0.5 * (xa + yb + zc - 1.0)) / sqrtf((float)(xa * a[3] + yb * a[4] + zc * a[5]));
        }
        case SDFIBM_SHAPE_RECTANGLE: {
            const D3 q = com + p;
            return rect_mixed(q.x, q.y, a[0], a[1]);
        }
        case SDFIBM_SHAPE_BOX: {
            const D3 q = com + p;
            const double dx = fabs(q.x) - a[0], dy = fabs(q.y) - a[1], dz = fabs(q.z) - a[2];
            const double dxp = dmax(0.0, dx), dyp = dmax(0.0, dy), dzp = dmax(0.0, dz);
            return sqrtf((float)(dxp * dxp + dyp * dyp + dzp * dzp)) + (float)dmin(0.0, dmax(dz, dmax(dx, dy)));
        }
        case SDFIBM_SHAPE_PLANE: return (float)p.y;
        case SDFIBM_SHAPE_CIRCLE_TAIL: {
            const D3 q = com + p;
            const double qq = q.x * q.x + q.y * q.y;
            const float d1 = (float)(qq - a[3]) / (sqrtf((float)qq) + (float)a[0]);
            const float d2 = rect_mixed(q.x - a[4], q.y, a[4], a[2]);
            return fminf(d1, d2);
        }
        case SDFIBM_SHAPE_CIRCLE_TWOTAIL: {
            const D3 q = com + p;
            const double qq = q.x * q.x + q.y * q.y;
            const float dc = (float)(qq - a[3]) / (sqrtf((float)qq) + (float)a[0]);
            const D3 r1 = rot30_64(D3{q.x, q.y, 0.0}), r2 = rot30_64(D3{q.x, -q.y, 0.0});
            const float d1 = rect_mixed(r1.x - a[4], r1.y, a[4], a[2]);
            const float d2 = rect_mixed(r2.x - a[4], r2.y, a[4], a[2]);
            return fminf(dc, fminf(d1, d2));
        }
    }
    return 0.f;
}

// filter of sdf.h:147-150 applied to the mixed value; *exact_needed set when the value sits on the threshold
// ---- two-float vertex distances (REF-GEO, 3-D spheres, ellipsoids and boxes) ---------------------------------------
// Pairs hi + lo with error-free sums and products (Dekker, Knuth), explicit rounding intrinsics so that nothing is
// contracted or reassociated; each operation errs by a few 2^-48 of its operands' magnitudes.  GB300 issues FP32 at 64
// times the FP64 rate, so the pairs replace the FP64 local point and the cancelling differences of sdf_mixed.
struct FF {
    float hi, lo;
};
__device__ __forceinline__ FF ff_fast(float a, float b) {  // |a| >= |b|, or the pair carries the rounding of b
    const float s = __fadd_rn(a, b);
    return FF{s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ FF ff_sum(float a, float b) {
    const float s = __fadd_rn(a, b), bb = __fsub_rn(s, a);
    return FF{s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb))};
}
__device__ __forceinline__ FF ff_add(FF x, FF y) {
    const FF t = ff_sum(x.hi, y.hi);
    return ff_fast(t.hi, __fadd_rn(t.lo, __fadd_rn(x.lo, y.lo)));
}
__device__ __forceinline__ FF ff_mul(FF x, FF y) {
    const float p = __fmul_rn(x.hi, y.hi);
    return ff_fast(p, __fmaf_rn(x.hi, y.lo, __fmaf_rn(x.lo, y.hi, __fmaf_rn(x.hi, y.hi, -p))));
}
__device__ __forceinline__ FF ff_scale(FF x, float n) {  // n: a small integer, exact in FP32
    const float p = __fmul_rn(x.hi, n);
    return ff_fast(p, __fmaf_rn(x.lo, n, __fmaf_rn(x.hi, n, -p)));
}
__device__ __forceinline__ FF ff_abs(FF x) { return x.hi < 0.f ? FF{-x.hi, -x.lo} : x; }

// Solid::phi of bbox vertex (da, db, dc) as sdf_mixed computes it (the same FP32 formula after the cancelling
// differences), the local point from the plan's two-float map; err bounds the difference to the exact value with a
// factor of 4 to spare over the operations' roundoff (2^-44 of the magnitudes).
__device__ inline float sdf_ff(const ShapeK& s, const SolidPlan& pl, float da, float db, float dc, float& err) {
    FF P[3];
    float ml = 0.f;
    const float f3[3] = {da, db, dc};
#pragma unroll
    for (int r = 0; r < 3; ++r) {
        FF v{pl.lmap_hi[r], pl.lmap_lo[r]};
        float mag = fabsf(pl.lmap_hi[r]);
#pragma unroll
        for (int t = 0; t < 3; ++t) {
            const int i = 3 + 3 * t + r;
            v = ff_add(v, ff_scale(FF{pl.lmap_hi[i], pl.lmap_lo[i]}, f3[t]));
            mag += fabsf(f3[t] * pl.lmap_hi[i]);
        }
        P[r] = v;
        ml = fmaxf(ml, mag);
    }
    const float U44 = 5.6843418860808015e-14f;  // 2^-44
    const float* a = s.p32;
    if (s.type == SDFIBM_SHAPE_ELLIPSOID) {  // the reference's ellipsoid ignores com
        const FF xa = ff_mul(ff_mul(P[0], P[0]), FF{a[3], s.p_lo[3]});
        const FF yb = ff_mul(ff_mul(P[1], P[1]), FF{a[4], s.p_lo[4]});
        const FF zc = ff_mul(ff_mul(P[2], P[2]), FF{a[5], s.p_lo[5]});
        const FF sum = ff_add(ff_add(ff_add(xa, yb), zc), FF{-1.f, 0.f});
        const float den = sqrtf(xa.hi * a[3] + yb.hi * a[4] + zc.hi * a[5]);
        const float am = fmaxf(a[3], fmaxf(a[4], a[5]));
        const float pm = fmaxf(fabsf(P[0].hi), fmaxf(fabsf(P[1].hi), fabsf(P[2].hi)));
        err = 4.f * U44 * (xa.hi + yb.hi + zc.hi + 1.f + 6.f * am * pm * (ml + pm)) / den;
        return (0.5f * __fadd_rn(sum.hi, sum.lo)) / den;
    }
    FF q[3];
    float qm = 0.f;
#pragma unroll
    for (int r = 0; r < 3; ++r) {
        q[r] = ff_add(P[r], FF{s.com32[r], s.com_lo[r]});
        qm = fmaxf(qm, fabsf(q[r].hi));
    }
    const float mag = ml + fabsf(s.com32[0]) + fabsf(s.com32[1]) + fabsf(s.com32[2]) + qm;
    if (s.type == SDFIBM_SHAPE_SPHERE) {
        const FF qq = ff_add(ff_add(ff_mul(q[0], q[0]), ff_mul(q[1], q[1])), ff_mul(q[2], q[2]));
        const FF num = ff_add(qq, FF{-a[1], -s.p_lo[1]});
        const float den = sqrtf(qq.hi) + a[0];
        err = 4.f * U44 * (qq.hi + a[1] + 6.f * qm * mag) / den;
        return __fadd_rn(num.hi, num.lo) / den;
    }
    // box
    float d[3];
#pragma unroll
    for (int r = 0; r < 3; ++r) {
        const FF t = ff_add(ff_abs(q[r]), FF{-a[r], -s.p_lo[r]});
        d[r] = __fadd_rn(t.hi, t.lo);
    }
    err = 4.f * U44 * (mag + a[0] + a[1] + a[2]);
    const float dxp = fmaxf(0.f, d[0]), dyp = fmaxf(0.f, d[1]), dzp = fmaxf(0.f, d[2]);
    return sqrtf(dxp * dxp + dyp * dyp + dzp * dzp) + fminf(0.f, fmaxf(d[2], fmaxf(d[0], d[1])));
}

__device__ inline float filter_mixed(const ShapeK& s, float phi, bool* exact_needed) {
    if (s.type == SDFIBM_SHAPE_PLANE) return phi;  // the plane's distance is unfiltered and exact
    const float a = fabsf(phi);
    if (fabsf(a - 1e-8f) <= 1e-14f) *exact_needed = true;
    return a < 1e-8f ? -1e-8f : phi;
}

// LEARNED: the features of the tile's cut cells (one warp), appended to the network's input buffer with the index of
// the cell's fraction; out of line to keep the tile loop small.  tile0 = fraction index of the tile's cell (0,0,0).
// REF-GEO: the tile's cut cells (one warp) appended to the cell list with the distances of their 8 vertices
template <int TX, int TY, int TZ>
static __device__ __noinline__ void write_refgeo_list(const ClassifyArgs& A, const uint8_t* cutlist, int ncut,
                                                      const float* vphi, int s, int64_t tile0, int ext0, int ext1) {
    constexpr int VX = TX + 1, VY = TY + 1;
    const int lane = threadIdx.x & 31;
    for (int u0 = 0; u0 < ncut; u0 += 32) {
        int base = 0;
        if (lane == 0) base = atomicAdd(&A.cnt->n_feat, min(32, ncut - u0));
        base = __shfl_sync(0xffffffffu, base, 0);
        const int u = u0 + lane;
        if (u < ncut) {
            const int e = cutlist[u];
            const int a = e % TX, b = (e / TX) % TY, c = e / (TX * TY);
            const int v0 = a + VX * (b + VY * c);
            const int64_t slot = (int64_t)base + lane;
            if (slot < A.feat_cap) {
                const int vo[8] = {0, 1, VX, VX + 1, VX * VY, VX * VY + 1, VX * VY + VX, VX * VY + VX + 1};
#pragma unroll
                for (int q = 0; q < 8; ++q) A.rg_phi[q * A.feat_cap + slot] = vphi[v0 + vo[q]];
                A.fref_solid[slot] = s;
                A.fref_index[slot] = tile0 + a + (int64_t)ext0 * (b + (int64_t)ext1 * c);
            } else {
                set_error(A.cnt, DERR_CAPACITY);
            }
        }
    }
}

// SUBSAMPLE: the tile's cut cells (one warp) appended to the cell list as (solid, fraction index)
template <int TX, int TY, int TZ>
static __device__ __noinline__ void write_cut_list(const ClassifyArgs& A, const uint8_t* cutlist, int ncut, int s,
                                                   int64_t tile0, int ext0, int ext1) {
    const int lane = threadIdx.x & 31;
    // LEARNED, a solid under rho_min cells: from the back of the list, for the fallback
    const bool back = A.method == SDFIBM_FRACTION_LEARNED && A.plan[s].radius_cells < A.rho_min;
    for (int u0 = 0; u0 < ncut; u0 += 32) {
        int base = 0;
        if (lane == 0) base = atomicAdd(back ? &A.cnt->n_small : &A.cnt->n_feat, min(32, ncut - u0));
        base = __shfl_sync(0xffffffffu, base, 0);
        const int u = u0 + lane;
        if (u < ncut) {
            const int e = cutlist[u];
            const int a = e % TX, b = (e / TX) % TY, c = e / (TX * TY);
            const int64_t slot = back ? A.feat_cap - 1 - ((int64_t)base + lane) : (int64_t)base + lane;
            if (slot >= 0 && slot < A.feat_cap) {
                A.fref_solid[slot] = s;
                A.fref_index[slot] = tile0 + a + (int64_t)ext0 * (b + (int64_t)ext1 * c);
            } else {
                set_error(A.cnt, DERR_CAPACITY);
            }
        }
    }
}

// ---- the tile kernel: one warp per chunk of up to chunk_tiles tiles of one solid ------------------------------------------
constexpr int CLS_WARPS = 8;

template <int TX, int TY, int TZ, int METHOD>
__device__ __forceinline__ void classify_body(const ClassifyArgs& A) {
    constexpr int VX = TX + 1, VY = TY + 1, VZ = TZ + 1, NV = VX * VY * VZ, NC = TX * TY * TZ;
    __shared__ uint8_t s_vin[CLS_WARPS][NV];
    __shared__ uint8_t s_need[CLS_WARPS][NV];
    __shared__ float s_phi[CLS_WARPS][NV];
    __shared__ uint8_t s_cut[CLS_WARPS][NC];
    __shared__ uint8_t s_vlist[CLS_WARPS][NV];
    const MeshK& m = A.m;
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    uint8_t* vin = s_vin[w];
    uint8_t* vneed = s_need[w];
    float* vphi = s_phi[w];
    uint8_t* cutlist = s_cut[w];
    unsigned long long rechecks = 0, valid_cells = 0;
    for (;;) {
        int chunk = 0;
        if (lane == 0) chunk = atomicAdd(&A.cnt->classify_next, 1);
        chunk = __shfl_sync(FULL, chunk, 0);
        if (chunk >= A.total_chunks) break;
        const int2 ch = A.chunks[chunk];
        const int s = ch.x;
        const SolidK& k = A.sk[s];
        const SolidPlan& pl = A.plan[s];
        const int ntile_all = k.ntile[0] * k.ntile[1] * k.ntile[2];
        const int t_end = min(ch.y + A.chunk_tiles, ntile_all);
        const Q4 q = state_quat(A.st[s]);
        const D3 x = state_pos(A.st[s]);
        const ShapeK& sh = k.shape;
        float M[9];
#pragma unroll
        for (int r = 0; r < 9; ++r) M[r] = pl.M[r];
        const int32_t vlo0 = pl.vlo[0], vlo1 = pl.vlo[1], vlo2 = pl.vlo[2];
        const int32_t vhi0 = pl.vhi[0], vhi1 = pl.vhi[1], vhi2 = pl.vhi[2];
        uint8_t* out = A.cls + k.scratch_off;
        float* alpha = A.alpha + k.scratch_off;
        unsigned long long wmin = ~0ull;
        const float sb[3] = {pl.base32[0], pl.base32[1], pl.base32[2]};
        for (int t = ch.y; t < t_end; ++t) {
            const int tx = t % k.ntile[0], ty = (t / k.ntile[0]) % k.ntile[1], tz = t / (k.ntile[0] * k.ntile[1]);
            const int cx = min(TX, k.ext[0] - tx * TX);
            const int cy = min(TY, k.ext[1] - ty * TY);
            const int cz = min(TZ, k.ext[2] - tz * TZ);
            const int64_t I0 = (int64_t)pl.lo[0] + tx * TX;
            const int64_t J0 = (int64_t)pl.lo[1] + ty * TY;
            const int64_t K0 = (int64_t)pl.lo[2] + tz * TZ;
            auto local_index = [&](int a, int b, int c) {
                return (int64_t)(tx * TX + a) + (int64_t)k.ext[0] * ((ty * TY + b) + (int64_t)k.ext[1] * (tz * TZ + c));
            };
            // whole tile outside the mesh or outside the solid's oriented bounding box: no cell has an inside vertex
            bool cull = pl.err != 0 || I0 + cx <= 0 || J0 + cy <= 0 || K0 + cz <= 0 || I0 >= m.nx ||
                        J0 >= m.ny || K0 >= m.nz || I0 + cx < vlo0 || I0 > vhi0 || J0 + cy < vlo1 ||
                        J0 > vhi1 || K0 + cz < vlo2 || K0 > vhi2;
            if (!cull && pl.cull_box) {
                // separating axes of the solid's local box: the tile's centre and half extents seen in the local
                // frame (FP32 with a relative margin of 1e-4 on both sides of every comparison)
                const float hx = 0.5f * (float)cx * m.h32[0], hy = 0.5f * (float)cy * m.h32[1],
                            hz = 0.5f * (float)cz * m.h32[2];
                const float tcx = sb[0] + (float)(tx * TX) * m.h32[0] + hx;
                const float tcy = sb[1] + (float)(ty * TY) * m.h32[1] + hy;
                const float tcz = sb[2] + (float)(tz * TZ) * m.h32[2] + hz;
#pragma unroll
                for (int a = 0; a < 3; ++a) {
                    const float lc = __fmaf_rn(M[3 * a], tcx, __fmaf_rn(M[3 * a + 1], tcy, M[3 * a + 2] * tcz));
                    const float rad = fabsf(M[3 * a]) * hx + fabsf(M[3 * a + 1]) * hy + fabsf(M[3 * a + 2]) * hz;
                    const float gap = fabsf(lc - pl.lbox_c[a]) - pl.lbox_s[a] - rad;
                    cull = cull || gap > 1e-4f * (fabsf(lc) + fabsf(pl.lbox_c[a]) + pl.lbox_s[a] + rad) + 1e-30f;
                }
            }
            if (cull) {
                for (int e = lane; e < NC; e += 32) {
                    const int a = e % TX, b = (e / TX) % TY, c = e / (TX * TY);
                    if (a < cx && b < cy && c < cz) out[local_index(a, b, c)] = 0;
                }
                continue;
            }
            // tile frame in FP32: the solid's FP64 base plus the tile's cell offset; babs covers both roundings
            TileFrame tf;
            {
                const float ofx = (float)(tx * TX) * m.h32[0], ofy = (float)(ty * TY) * m.h32[1],
                            ofz = (float)(tz * TZ) * m.h32[2];
                tf.bx = sb[0] + ofx; tf.by = sb[1] + ofy; tf.bz = sb[2] + ofz;
                tf.babs = fabsf(sb[0]) + fabsf(sb[1]) + fabsf(sb[2]) + 2.f * (fabsf(ofx) + fabsf(ofy) + fabsf(ofz)) +
                          fabsf(tf.bx) + fabsf(tf.by) + fabsf(tf.bz);
                tf.e64 = pl.e64;
            }
            for (int v = lane; v < NV; v += 32) {
                const int a = v % VX, b = (v / VX) % VY, c = v / (VX * VY);
                const int64_t I = I0 + a, J = J0 + b, K = K0 + c;
                uint8_t r = 0;
                if (a <= cx && b <= cy && c <= cz && I >= vlo0 && I <= vhi0 && J >= vlo1 && J <= vhi1 && K >= vlo2 &&
                    K <= vhi2 && I >= 0 && J >= 0 && K >= 0 && I <= m.nx && J <= m.ny && K <= m.nz) {
                    const float ox = (float)a * m.h32[0], oy = (float)b * m.h32[1], oz = (float)c * m.h32[2];
                    r = (uint8_t)classify_point(sh, M, tf, ox, oy, oz, m, I, J, K, 0, x, q, &rechecks);
                }
                vin[v] = r;
                vneed[v] = 0;
            }
            __syncwarp();
            int ncut = 0;
#pragma unroll 1
            for (int base = 0; base < NC; base += 32) {
                const int e = base + lane;
                const int a = e % TX, b = (e / TX) % TY, c = e / (TX * TY);
                uint8_t cls = 0;
                const bool in_tile = e < NC && a < cx && b < cy && c < cz;
                if (in_tile) {
                    const int64_t I = I0 + a, J = J0 + b, K = K0 + c;
                    if (I >= 0 && J >= 0 && K >= 0 && I < m.nx && J < m.ny && K < m.nz) {
                        ++valid_cells;
                        const int v0 = a + VX * (b + VY * c);
                        const int cntv = vin[v0] + vin[v0 + 1] + vin[v0 + VX] + vin[v0 + VX + 1] + vin[v0 + VX * VY] +
                                         vin[v0 + VX * VY + 1] + vin[v0 + VX * VY + VX] + vin[v0 + VX * VY + VX + 1];
                        if (cntv == 8) {
                            cls = 1;
                        } else if (cntv > 0) {
                            const float ox = ((float)a + 0.5f) * m.h32[0], oy = ((float)b + 0.5f) * m.h32[1],
                                        oz = ((float)c + 0.5f) * m.h32[2];
                            const int ci = classify_point(sh, M, tf, ox, oy, oz, m, I, J, K, 1, x, q, &rechecks);
                            cls = ci ? 2 : 3;
                        }
                        if (cls) wmin = min(wmin, (unsigned long long)(I + (int64_t)m.nx * (J + (int64_t)m.ny * K)));
                    }
                    out[local_index(a, b, c)] = cls;
                }
                // compact the cut candidates of this pass
                const bool is_cut = (cls == 2 || cls == 3) && METHOD >= 0;
                const unsigned bal = __ballot_sync(FULL, is_cut);
                if (is_cut) {
                    cutlist[ncut + __popc(bal & ((1u << lane) - 1u))] = (uint8_t)e;
                    if (METHOD == SDFIBM_FRACTION_REFGEO) {
                        const int v0 = a + VX * (b + VY * c);
                        vneed[v0] = 1; vneed[v0 + 1] = 1; vneed[v0 + VX] = 1; vneed[v0 + VX + 1] = 1;
                        vneed[v0 + VX * VY] = 1; vneed[v0 + VX * VY + 1] = 1; vneed[v0 + VX * VY + VX] = 1;
                        vneed[v0 + VX * VY + VX + 1] = 1;
                    }
                }
                ncut += __popc(bal);
            }
            if (ncut == 0) continue;
            __syncwarp();
            if (METHOD == SDFIBM_FRACTION_REFGEO) {
                // Solid::phi once per vertex next to a cut candidate.  The needed vertices are compacted first so
                // every FP64 instruction runs on a full warp; the local point is the solid's FP64 local map applied to
                // small integer offsets from the bbox corner.
                uint8_t* vlist = s_vlist[w];
                int nneed = 0;
                for (int base = 0; base < NV; base += 32) {
                    const int v = base + lane;
                    const bool need = v < NV && vneed[v];
                    const unsigned bal = __ballot_sync(FULL, need);
                    if (need) vlist[nneed + __popc(bal & ((1u << lane) - 1u))] = (uint8_t)v;
                    nneed += __popc(bal);
                }
                __syncwarp();
                const double* L = pl.lmap;
                // 3-D spheres, ellipsoids and boxes: two-float distances (FP32 pipe); others: sdf_mixed (FP64)
                const bool ff_shape = !sh.prism && (sh.type == SDFIBM_SHAPE_SPHERE ||
                                                    sh.type == SDFIBM_SHAPE_ELLIPSOID || sh.type == SDFIBM_SHAPE_BOX);
                for (int u = lane; u < nneed; u += 32) {
                    const int v = vlist[u];
                    const int a = v % VX, b = (v / VX) % VY, c = v / (VX * VY);
                    bool exact = false;
                    float ph;
                    if (ff_shape) {
                        float err;
                        ph = sdf_ff(sh, pl, (float)(tx * TX + a), (float)(ty * TY + b), (float)(tz * TZ + c), err);
                        const float aph = fabsf(ph);
                        exact = fabsf(aph - 1e-8f) <= 1e-14f + err;  // the filter's decision is not certain
                        if (aph < 1e-8f) ph = -1e-8f;
                    } else {
                        const double da = (double)(tx * TX + a), db = (double)(ty * TY + b),
                                     dc = (double)(tz * TZ + c);
                        const D3 plc{L[0] + da * L[3] + db * L[6] + dc * L[9],
                                     L[1] + da * L[4] + db * L[7] + dc * L[10],
                                     L[2] + da * L[5] + db * L[8] + dc * L[11]};
                        ph = filter_mixed(sh, sdf_mixed(sh, plc), &exact);
                    }
                    if (exact || sh.type == SDFIBM_SHAPE_PLANE) ph = exact_phi_point(sh, m, I0 + a, J0 + b, K0 + c, x, q);
                    vphi[v] = ph;
                }
                __syncwarp();
                if (METHOD == SDFIBM_FRACTION_REFGEO && A.rg_phi) {
                    // the cut cells and their vertex distances are listed; refgeo_cells_kernel computes the fractions
                    write_refgeo_list<TX, TY, TZ>(A, cutlist, ncut, vphi, s, k.scratch_off + local_index(0, 0, 0),
                                                  k.ext[0], k.ext[1]);
                    __syncwarp();
                    continue;
                }
                for (int u = lane; u < ncut; u += 32) {
                    const int e = cutlist[u];
                    const int a = e % TX, b = (e / TX) % TY, c = e / (TX * TY);
                    const int v0 = a + VX * (b + VY * c);
                    const float ph[8] = {vphi[v0], vphi[v0 + 1], vphi[v0 + VX], vphi[v0 + VX + 1],
                                         vphi[v0 + VX * VY], vphi[v0 + VX * VY + 1], vphi[v0 + VX * VY + VX],
                                         vphi[v0 + VX * VY + VX + 1]};
                    const int64_t K = K0 + c;
                    const float apz = m.twod ? (float)((0.0 - mesh_coord(m, 2, K)) / m.h[2]) : 0.f;
                    const float apz1 = m.twod ? (float)((mesh_coord(m, 2, K + 1) - 0.0) / m.h[2]) : 0.f;
                    alpha[local_index(a, b, c)] = refgeo32(m, ph, I0 + a, J0 + b, K, apz, apz1);
                }
            } else if (A.fref_index) {
                // SUBSAMPLE and LEARNED: the cut cells are listed; subsample_cells_kernel samples them (LEARNED:
                // learned_stencil_kernel computes the model's inputs, a thread per cell), a warp per cell
                write_cut_list<TX, TY, TZ>(A, cutlist, ncut, s, k.scratch_off + local_index(0, 0, 0), k.ext[0],
                                           k.ext[1]);
            } else if (METHOD == SDFIBM_FRACTION_SUBSAMPLE) {
                // SUBSAMPLE without a cell list (allocation-free entry): the warp shares the samples of one cut cell
                // (LEARNED always lists its cut cells, so its classify pass carries no sampling code)
                for (int u = 0; u < ncut; ++u) {
                    const int e = cutlist[u];
                    const int a = e % TX, b = (e / TX) % TY, c = e / (TX * TY);
                    const int64_t li = local_index(a, b, c);
                    const Defer df{A.rq, A.rq_cap, &A.cnt->n_recheck, k.scratch_off + li, s, nullptr};
                    const int cnt = subsample_warp(m, sh, M, tf, a, b, c, x, q, I0 + a, J0 + b, K0 + c,
                                                   A.subsample_n, &rechecks, A.rq ? &df : nullptr);
                    if (lane == 0) alpha[li] = A.rq ? -1.f - (float)cnt : count_fraction(m, cnt, A.subsample_n);
                }
            }
            __syncwarp();
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) wmin = min(wmin, __shfl_xor_sync(FULL, wmin, o));
        if (lane == 0 && wmin != ~0ull) atomicMin(&A.plan[s].min_cand, wmin);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        rechecks += __shfl_xor_sync(FULL, rechecks, o);
        valid_cells += __shfl_xor_sync(FULL, valid_cells, o);
    }
    if (lane == 0) {
        if (rechecks) atomicAdd(&A.cnt->exact_rechecks, rechecks);
        if (valid_cells) atomicAdd(&A.cnt->bbox_cells, valid_cells);
    }
}

// SUBSAMPLE count of one listed cell (bbox index idx of solid s) from the cell's own FP32 frame, built as the classify
// pass builds a tile's: the solid's rounded base plus a whole number of cells.
template <bool DEFER_ONLY>
__device__ __forceinline__ int count_listed_cell(const FallbackArgs& A, int s, int64_t idx, unsigned long long* rechecks,
                                                 const Defer* df) {
    const SolidK& k = A.sk[s];
    const SolidPlan& pl = A.plan[s];
    const uint32_t local = (uint32_t)(idx - k.scratch_off);  // < bbox cells of one solid (< 2^31)
    const int row = (int)fdiv(local, k.div_e0), lc = (int)fdiv(local, k.div_e01);
    const int la = (int)local - row * k.ext[0], lb = row - lc * k.ext[1];
    TileFrame tf;
    {
        const float sbx = pl.base32[0], sby = pl.base32[1], sbz = pl.base32[2];
        const float ofx = (float)la * A.m.h32[0], ofy = (float)lb * A.m.h32[1], ofz = (float)lc * A.m.h32[2];
        tf.bx = sbx + ofx; tf.by = sby + ofy; tf.bz = sbz + ofz;
        tf.babs = fabsf(sbx) + fabsf(sby) + fabsf(sbz) + 2.f * (fabsf(ofx) + fabsf(ofy) + fabsf(ofz)) +
                  fabsf(tf.bx) + fabsf(tf.by) + fabsf(tf.bz);
        tf.e64 = pl.e64;
    }
    float M[9];
#pragma unroll
    for (int r = 0; r < 9; ++r) M[r] = pl.M[r];
    if (DEFER_ONLY) {  // inlined; the FP64 state is not needed
        return subsample_warp_body<true>(A.m, k.shape, M, tf, 0, 0, 0, D3{0, 0, 0}, Q4{1, D3{0, 0, 0}}, 0, 0, 0, A.n,
                                         rechecks, df);
    }
    const Q4 q = state_quat(A.st[s]);
    const D3 x = state_pos(A.st[s]);
    return subsample_warp(A.m, k.shape, M, tf, 0, 0, 0, x, q, pl.lo[0] + la, pl.lo[1] + lb, pl.lo[2] + lc, A.n,
                          rechecks, df);
}

// SUBSAMPLE of listed cells, one warp per cell: the cut cells of the classify pass (SUBSAMPLE, fb_list == nullptr)
// or the cells outside the network's band (LEARNED fallback).  Undecided points always go to the recheck list (this
// kernel holds no FP64 path, which keeps its register count and so its occupancy); a cell some of whose points found
// the list full is listed for recount_kernel.
__global__ void __launch_bounds__(256, 4) subsample_cells_kernel(FallbackArgs A) {
    __shared__ int32_t s_overflow[8];
    const int lane = threadIdx.x & 31;
    int32_t* overflow = s_overflow + ((threadIdx.x >> 5) & 7);
    // LEARNED: the band's rejects (fb_list), then the cells listed from the back; a front and a back that overlap
    // (more cut cells than the list holds) are a capacity error
    const int64_t n_fb = A.fb_list ? min((int64_t)A.cnt->n_fb, A.cap) : 0;
    const int64_t n_back = A.fb_list ? (int64_t)A.cnt->n_small : 0;
    if (A.fb_list && (int64_t)A.cnt->n_feat + n_back > A.cap && threadIdx.x == 0 && blockIdx.x == 0)
        set_error(A.cnt, DERR_CAPACITY);
    const int64_t nfb = A.fb_list ? min(n_fb + n_back, A.cap) : min((int64_t)A.cnt->n_feat, A.cap);
    const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
    unsigned long long rechecks = 0;
    if (lane == 0) *overflow = 0;
    __syncwarp();
    // each warp takes 32 consecutive list entries: the 32 lanes load their (solid, index) pairs at once, then the
    // warp counts the cells one after the other
    for (int64_t base = (((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5) * 32; base < nfb; base += warps * 32) {
        int s_l = 0;
        int64_t idx_l = 0;
        if (base + lane < nfb) {
            const int64_t q = base + lane;
            const int64_t slot = !A.fb_list ? q : (q < n_fb ? (int64_t)A.fb_list[q] : A.cap - 1 - (q - n_fb));
            s_l = A.fref_solid[slot];
            idx_l = A.fref_index[slot];
        }
        const int batch = (int)min((int64_t)32, nfb - base);
        for (int t = 0; t < batch; ++t) {
            const int s = __shfl_sync(0xffffffffu, s_l, t);
            const int64_t idx = __shfl_sync(0xffffffffu, idx_l, t);
            const Defer df{A.rq, A.rq_cap, &A.cnt->n_recheck, idx, s, overflow};
            const int cnt = count_listed_cell<true>(A, s, idx, &rechecks, &df);
            __syncwarp();
            if (lane == 0) {
                A.alpha[idx] = -1.f - (float)cnt;
                if (*(volatile int32_t*)overflow) {
                    *overflow = 0;
                    const int slot = atomicAdd(&A.cnt->n_ovf, 1);
                    if (slot < A.ovf_cap) A.ovf[slot] = Recheck{idx, s, 0u};
                    else set_error(A.cnt, DERR_CAPACITY);
                }
            }
            __syncwarp();
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) rechecks += __shfl_xor_sync(0xffffffffu, rechecks, o);
    if (lane == 0 && rechecks) atomicAdd(&A.cnt->exact_rechecks, rechecks);
}

// Cells of the fallback whose undecided points overflowed the recheck list: counted again from scratch, undecided
// points in FP64 in place, after recheck_kernel (whose updates of these cells the new count replaces).
__global__ void __launch_bounds__(256) recount_kernel(FallbackArgs A) {
    const int lane = threadIdx.x & 31;
    const int64_t n = min((int64_t)A.cnt->n_ovf, A.ovf_cap);
    const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
    unsigned long long rechecks = 0;
    for (int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; w < n; w += warps) {
        const Recheck r = A.ovf[w];
        const int cnt = count_listed_cell<false>(A, r.solid, r.idx, &rechecks, nullptr);
        if (lane == 0) A.alpha[r.idx] = -1.f - (float)cnt;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) rechecks += __shfl_xor_sync(0xffffffffu, rechecks, o);
    if (lane == 0 && rechecks) atomicAdd(&A.cnt->exact_rechecks, rechecks);
}

// REF-GEO fraction of the listed cut cells, one thread per cell (GeometricTools::calcCellVolume on the cell's vertex
// distances, see refgeo32): the tile pass lists the cells, so every lane here has a cell.
__global__ void __launch_bounds__(256) refgeo_cells_kernel(MeshK m, const SolidK* __restrict__ sk,
                                                           const SolidPlan* __restrict__ plan,
                                                           const int32_t* __restrict__ fref_solid,
                                                           const int64_t* __restrict__ fref_index,
                                                           const float* __restrict__ rg_phi, int64_t cap,
                                                           const Counters* cnt, float* __restrict__ alpha) {
    const int64_t n = min((int64_t)cnt->n_feat, cap);
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
        const int s = fref_solid[e];
        const int64_t idx = fref_index[e];
        const SolidK& k = sk[s];
        const SolidPlan& pl = plan[s];
        const uint32_t local = (uint32_t)(idx - k.scratch_off);
        const int row = (int)fdiv(local, k.div_e0), lc = (int)fdiv(local, k.div_e01);
        const int la = (int)local - row * k.ext[0], lb = row - lc * k.ext[1];
        float ph[8];
#pragma unroll
        for (int q = 0; q < 8; ++q) ph[q] = rg_phi[q * cap + e];
        const int64_t K = pl.lo[2] + lc;
        const float apz = m.twod ? (float)((0.0 - mesh_coord(m, 2, K)) / m.h[2]) : 0.f;
        const float apz1 = m.twod ? (float)((mesh_coord(m, 2, K + 1) - 0.0) / m.h[2]) : 0.f;
        alpha[idx] = refgeo32(m, ph, pl.lo[0] + la, pl.lo[1] + lb, K, apz, apz1);
    }
}

// The deferred SUBSAMPLE points: one per thread, the reference's FP64 point and inside test, an inside point lowers the
// cell's encoded count (-(1 + count)) by one.
__global__ void __launch_bounds__(256) recheck_kernel(MeshK m, const SolidK* __restrict__ sk,
                                                      const sdfibm_solid_state* __restrict__ st,
                                                      const SolidPlan* __restrict__ plan,
                                                      const Recheck* __restrict__ rq, int64_t cap, Counters* cnt,
                                                      float* __restrict__ alpha) {
    const int64_t n = min((int64_t)cnt->n_recheck, cap);
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
        const Recheck r = rq[e];
        const SolidK& k = sk[r.solid];
        const SolidPlan& pl = plan[r.solid];
        const int local = (int)(r.idx - k.scratch_off);
        const int la = local % k.ext[0], lb = (local / k.ext[0]) % k.ext[1], lc = local / (k.ext[0] * k.ext[1]);
        const int a = r.sample & 255, b = (r.sample >> 8) & 255, c = (r.sample >> 16) & 255, ns = r.sample >> 24;
        const int in = exact_inside_sample(k.shape, m, pl.lo[0] + la, pl.lo[1] + lb, pl.lo[2] + lc, a, b, c, ns,
                                           state_pos(st[r.solid]), state_quat(st[r.solid]));
        if (in) atomicAdd(alpha + r.idx, -1.f);
    }
}

// 3-D meshes: 4x4x4-cell tiles; one- and two-layer meshes: 8x8x2
// one instantiation per fraction method (-1: classification only), so each kernel carries only its own path.  The
// LEARNED pass (no fraction of its own) runs three CTAs per SM in 80 registers (ncu at 512^3: 1.45 -> 1.14 ms); the
// REF-GEO pass, whose vertex distances need more, is faster at two (1.84 ms against 2.48 ms at three).
template <int METHOD>
__global__ void __launch_bounds__(CLS_WARPS * 32, METHOD == SDFIBM_FRACTION_LEARNED ? 3 : 2) classify_kernel_3d(ClassifyArgs A) { classify_body<4, 4, 4, METHOD>(A); }
template <int METHOD>
__global__ void __launch_bounds__(CLS_WARPS * 32) classify_kernel_2d(ClassifyArgs A) { classify_body<8, 8, 2, METHOD>(A); }
template __global__ void classify_kernel_3d<-1>(ClassifyArgs);
template __global__ void classify_kernel_3d<SDFIBM_FRACTION_REFGEO>(ClassifyArgs);
template __global__ void classify_kernel_3d<SDFIBM_FRACTION_SUBSAMPLE>(ClassifyArgs);
template __global__ void classify_kernel_3d<SDFIBM_FRACTION_LEARNED>(ClassifyArgs);
template __global__ void classify_kernel_2d<-1>(ClassifyArgs);
template __global__ void classify_kernel_2d<SDFIBM_FRACTION_REFGEO>(ClassifyArgs);
template __global__ void classify_kernel_2d<SDFIBM_FRACTION_SUBSAMPLE>(ClassifyArgs);
template __global__ void classify_kernel_2d<SDFIBM_FRACTION_LEARNED>(ClassifyArgs);

// host side: the instantiation for a method and a tile shape
void launch_classify(const ClassifyArgs& A, bool flat, int grid, cudaStream_t st) {
    switch (A.method) {
        case SDFIBM_FRACTION_REFGEO:
            if (flat) classify_kernel_2d<SDFIBM_FRACTION_REFGEO><<<grid, CLS_WARPS * 32, 0, st>>>(A);
            else classify_kernel_3d<SDFIBM_FRACTION_REFGEO><<<grid, CLS_WARPS * 32, 0, st>>>(A);
            break;
        case SDFIBM_FRACTION_SUBSAMPLE:
            if (flat) classify_kernel_2d<SDFIBM_FRACTION_SUBSAMPLE><<<grid, CLS_WARPS * 32, 0, st>>>(A);
            else classify_kernel_3d<SDFIBM_FRACTION_SUBSAMPLE><<<grid, CLS_WARPS * 32, 0, st>>>(A);
            break;
        case SDFIBM_FRACTION_LEARNED:
            if (flat) classify_kernel_2d<SDFIBM_FRACTION_LEARNED><<<grid, CLS_WARPS * 32, 0, st>>>(A);
            else classify_kernel_3d<SDFIBM_FRACTION_LEARNED><<<grid, CLS_WARPS * 32, 0, st>>>(A);
            break;
        default:
            if (flat) classify_kernel_2d<-1><<<grid, CLS_WARPS * 32, 0, st>>>(A);
            else classify_kernel_3d<-1><<<grid, CLS_WARPS * 32, 0, st>>>(A);
            break;
    }
}

// resident CTAs per SM of the instantiation a launch would use
int classify_occupancy(int method, bool flat) {
    int occ = 0;
    const void* f = nullptr;
    switch (method) {
        case SDFIBM_FRACTION_REFGEO: f = flat ? (const void*)classify_kernel_2d<SDFIBM_FRACTION_REFGEO>
                                              : (const void*)classify_kernel_3d<SDFIBM_FRACTION_REFGEO>; break;
        case SDFIBM_FRACTION_SUBSAMPLE: f = flat ? (const void*)classify_kernel_2d<SDFIBM_FRACTION_SUBSAMPLE>
                                                 : (const void*)classify_kernel_3d<SDFIBM_FRACTION_SUBSAMPLE>; break;
        case SDFIBM_FRACTION_LEARNED: f = flat ? (const void*)classify_kernel_2d<SDFIBM_FRACTION_LEARNED>
                                               : (const void*)classify_kernel_3d<SDFIBM_FRACTION_LEARNED>; break;
        default: f = flat ? (const void*)classify_kernel_2d<-1> : (const void*)classify_kernel_3d<-1>; break;
    }
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, f, CLS_WARPS * 32, 0);
    return occ;
}

}  // namespace sdfibm_dev
