// Enumeration and cut-cell solid fraction in one pass over (solid, cell-tile) work items.
//
// Each persistent CTA pulls tiles from an atomic counter.  For a tile it
//   1. skips tiles whose box cannot meet the solid's bounding sphere (prism: bounding disc) and zero-fills them;
//   2. evaluates the inside test once per tile vertex (FP32 with a rigorous error bound, FP64 re-check inside the
//      band -- identical answers to the reference's FP64 Solid::phi01) and writes one class byte per cell
//      (CellEnumerator::_next, src/cellenumerator.cpp:6-34): 0 no inside vertex, 1 all inside, 2 centre inside,
//      3 centre outside;
//   3. computes the solid fraction of every cut candidate (class 2/3) and writes it to the alpha scratch:
//      REF-GEO   GeometricTools::calcCellVolume (src/geometrictools.cpp:13-116): the vertex signed distances come
//                from the reference's FP64 Solid::phi, evaluated once per tile vertex next to a cut cell and kept in
//                shared memory; the apex/pyramid geometry then runs in FP32 in cell-local coordinates (vertices on
//                {0,1}^3), where on an axis-aligned hexahedron every term is a product of non-negative factors and
//                no subtraction cancels, so the result keeps ~1e-7 relative accuracy;
//      SUBSAMPLE one warp per cut cell, n^3 (3-D) or n^2 (2-D) midpoint samples, each with the same exact inside
//                test as the vertices.
// Candidates that the flood fill later leaves out simply have their alpha ignored.
#include <cstdint>
#include <cuda_runtime.h>

#include "common.cuh"

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
__device__ float refgeo32(const MeshK& m, const float* ph, int64_t i, int64_t j, int64_t k, float apz, float apz1) {
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

// ---- SUBSAMPLE: one warp per cut cell -----------------------------------------------------------------------------------
__device__ float subsample_warp(const MeshK& m, const ShapeK& sh, const float* M, const D3& x, const Q4& q, int64_t i,
                                int64_t j, int64_t k, int n, unsigned long long* rechecks) {
    const int lane = threadIdx.x & 31;
    const D3 p0 = mesh_point(m, i, j, k);
    const TileFrame tf = make_frame(p0 - x, p0, x);
    const int nzs = m.twod ? 1 : n;
    const int K = n * n * nzs;
    const float inv2n = 1.0f / (float)(2 * n);
    int cnt = 0;
    for (int sidx = lane; sidx < K; sidx += 32) {
        const int a = sidx % n, b = (sidx / n) % n, c3 = sidx / (n * n);
        const float ox = (float)(2 * a + 1) * inv2n * m.h32[0];
        const float oy = (float)(2 * b + 1) * inv2n * m.h32[1];
        const float oz = (m.twod ? 0.5f : (float)(2 * c3 + 1) * inv2n) * m.h32[2];
        // the FP32 sample offset carries an extra rounding of (2a+1)/(2n); doubled bound
        const float dx = tf.bx + ox, dy = tf.by + oy, dz = tf.bz + oz;
        const float lx = __fmaf_rn(M[0], dx, __fmaf_rn(M[1], dy, M[2] * dz));
        const float ly = __fmaf_rn(M[3], dx, __fmaf_rn(M[4], dy, M[5] * dz));
        const float lz = __fmaf_rn(M[6], dx, __fmaf_rn(M[7], dy, M[8] * dz));
        const float dabs = fabsf(dx) + fabsf(dy) + fabsf(dz);
        const float E = 8.f * U32 * (tf.babs + fabsf(ox) + fabsf(oy) + fabsf(oz) + 2.f * dabs) + tf.e64 + 1e-30f;
        int r = inside32(sh, lx, ly, lz, E);
        if (r == 2) {
            ++*rechecks;
            const double ta = (double)(2 * a + 1) / (double)(2 * n), tb = (double)(2 * b + 1) / (double)(2 * n);
            const double tz = m.twod ? 0.5 : (double)(2 * c3 + 1) / (double)(2 * n);
            const D3 p{m.o[0] + ((double)i + ta) * m.h[0], m.o[1] + ((double)j + tb) * m.h[1],
                       m.o[2] + ((double)k + tz) * m.h[2]};
            r = inside64(sh, world2local(p, x, q)) ? 1 : 0;
        }
        cnt += r;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
    return (float)((double)cnt / (double)K);
}

// ---- the tile kernel: one warp per (solid, cell-tile) item ---------------------------------------------------------------
constexpr int CLS_WARPS = 8;
constexpr int WT_VERTS = 9 * 9 * 3;  // largest warp tile: 8 x 8 x 2 cells
constexpr int WT_CELLS = 8 * 8 * 2;

__global__ void __launch_bounds__(CLS_WARPS * 32) classify_kernel(ClassifyArgs A) {
    __shared__ uint8_t s_vin[CLS_WARPS][WT_VERTS];
    __shared__ uint8_t s_need[CLS_WARPS][WT_VERTS];
    __shared__ float s_phi[CLS_WARPS][WT_VERTS];
    __shared__ uint8_t s_cut[CLS_WARPS][WT_CELLS];
    const MeshK& m = A.m;
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    uint8_t* vin = s_vin[w];
    uint8_t* vneed = s_need[w];
    float* vphi = s_phi[w];
    uint8_t* cutlist = s_cut[w];
    unsigned long long rechecks = 0, valid_cells = 0;
    for (;;) {
        int item = 0;
        if (lane == 0) item = atomicAdd(&A.cnt->classify_next, 1);
        item = __shfl_sync(FULL, item, 0);
        if (item >= A.total_tiles) break;
        const int s = find_solid(A.tile_prefix, A.S, item);
        const SolidK& k = A.sk[s];
        const SolidPlan& pl = A.plan[s];
        const int t = item - k.tile_base;
        const int tx = t % k.ntile[0], ty = (t / k.ntile[0]) % k.ntile[1], tz = t / (k.ntile[0] * k.ntile[1]);
        const int cx = min(k.tdim[0], k.ext[0] - tx * k.tdim[0]);
        const int cy = min(k.tdim[1], k.ext[1] - ty * k.tdim[1]);
        const int cz = min(k.tdim[2], k.ext[2] - tz * k.tdim[2]);
        const int64_t I0 = (int64_t)pl.lo[0] + tx * k.tdim[0];
        const int64_t J0 = (int64_t)pl.lo[1] + ty * k.tdim[1];
        const int64_t K0 = (int64_t)pl.lo[2] + tz * k.tdim[2];
        const int nc = cx * cy * cz;
        uint8_t* out = A.cls + k.scratch_off;
        auto local_index = [&](int a, int b, int c) {
            return (int64_t)(tx * k.tdim[0] + a) +
                   (int64_t)k.ext[0] * ((ty * k.tdim[1] + b) + (int64_t)k.ext[1] * (tz * k.tdim[2] + c));
        };
        // whole tile outside the mesh or outside the solid's oriented bounding box: no cell has an inside vertex
        const bool cull = pl.err != 0 || I0 + cx <= 0 || J0 + cy <= 0 || K0 + cz <= 0 || I0 >= m.nx || J0 >= m.ny ||
                          K0 >= m.nz || I0 + cx < pl.vlo[0] || I0 > pl.vhi[0] || J0 + cy < pl.vlo[1] ||
                          J0 > pl.vhi[1] || K0 + cz < pl.vlo[2] || K0 > pl.vhi[2];
        if (cull) {
            for (int e = lane; e < nc; e += 32) {
                const int a = e % cx, b = (e / cx) % cy, c = e / (cx * cy);
                out[local_index(a, b, c)] = 0;
            }
            continue;
        }
        const Q4 q = state_quat(A.st[s]);
        const D3 x = state_pos(A.st[s]);
        TileFrame tf;
        {
            float f5[5] = {0, 0, 0, 0, 0};
            if (lane == 0) {
                const D3 p0 = mesh_point(m, I0, J0, K0);
                tf = make_frame(p0 - x, p0, x);
                f5[0] = tf.bx; f5[1] = tf.by; f5[2] = tf.bz; f5[3] = tf.babs; f5[4] = tf.e64;
            }
#pragma unroll
            for (int r = 0; r < 5; ++r) f5[r] = __shfl_sync(FULL, f5[r], 0);
            tf.bx = f5[0]; tf.by = f5[1]; tf.bz = f5[2]; tf.babs = f5[3]; tf.e64 = f5[4];
        }
        const ShapeK& sh = k.shape;
        const float* M = pl.M;
        const int vx = cx + 1, vy = cy + 1, vz = cz + 1, nv = vx * vy * vz;
        for (int v = lane; v < nv; v += 32) {
            const int a = v % vx, b = (v / vx) % vy, c = v / (vx * vy);
            const int64_t I = I0 + a, J = J0 + b, K = K0 + c;
            uint8_t r = 0;
            if (I >= pl.vlo[0] && I <= pl.vhi[0] && J >= pl.vlo[1] && J <= pl.vhi[1] && K >= pl.vlo[2] &&
                K <= pl.vhi[2] && I >= 0 && J >= 0 && K >= 0 && I <= m.nx && J <= m.ny && K <= m.nz) {
                const float ox = (float)a * m.h32[0], oy = (float)b * m.h32[1], oz = (float)c * m.h32[2];
                r = (uint8_t)classify_point(sh, M, tf, ox, oy, oz, [&] { return mesh_point(m, I, J, K); }, x, q,
                                            &rechecks);
            }
            vin[v] = r;
            vneed[v] = 0;
        }
        __syncwarp();
        unsigned long long wmin = ~0ull;
        int ncut = 0;
        for (int base = 0; base < nc; base += 32) {
            const int e = base + lane;
            uint8_t cls = 0;
            int a = 0, b = 0, c = 0;
            if (e < nc) {
                a = e % cx; b = (e / cx) % cy; c = e / (cx * cy);
                const int64_t I = I0 + a, J = J0 + b, K = K0 + c;
                if (I >= 0 && J >= 0 && K >= 0 && I < m.nx && J < m.ny && K < m.nz) {
                    ++valid_cells;
                    int cntv = 0;
#pragma unroll
                    for (int dz = 0; dz < 2; ++dz)
#pragma unroll
                        for (int dy = 0; dy < 2; ++dy)
#pragma unroll
                            for (int dx = 0; dx < 2; ++dx) cntv += vin[(a + dx) + vx * ((b + dy) + vy * (c + dz))];
                    if (cntv == 8) {
                        cls = 1;
                    } else if (cntv > 0) {
                        const float ox = ((float)a + 0.5f) * m.h32[0], oy = ((float)b + 0.5f) * m.h32[1],
                                    oz = ((float)c + 0.5f) * m.h32[2];
                        const int ci = classify_point(sh, M, tf, ox, oy, oz, [&] { return mesh_C(m, I, J, K); }, x, q,
                                                      &rechecks);
                        cls = ci ? 2 : 3;
                    }
                    if (cls) wmin = min(wmin, (unsigned long long)(I + (int64_t)m.nx * (J + (int64_t)m.ny * K)));
                }
                out[local_index(a, b, c)] = cls;
            }
            // compact the cut candidates of this round
            const bool is_cut = (cls == 2 || cls == 3) && A.method >= 0;
            const unsigned bal = __ballot_sync(FULL, is_cut);
            if (is_cut) {
                cutlist[ncut + __popc(bal & ((1u << lane) - 1u))] = (uint8_t)e;
                if (A.method == SDFIBM_FRACTION_REFGEO) {
#pragma unroll
                    for (int dz = 0; dz < 2; ++dz)
#pragma unroll
                        for (int dy = 0; dy < 2; ++dy)
#pragma unroll
                            for (int dx = 0; dx < 2; ++dx) vneed[(a + dx) + vx * ((b + dy) + vy * (c + dz))] = 1;
                }
            }
            ncut += __popc(bal);
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) wmin = min(wmin, __shfl_xor_sync(FULL, wmin, o));
        if (lane == 0 && wmin != ~0ull) atomicMin(&A.plan[s].min_cand, wmin);
        if (ncut == 0) continue;
        __syncwarp();
        float* alpha = A.alpha + k.scratch_off;
        if (A.method == SDFIBM_FRACTION_REFGEO) {
            // Solid::phi (FP64) once per vertex next to a cut candidate
            for (int v = lane; v < nv; v += 32) {
                if (!vneed[v]) continue;
                const int a = v % vx, b = (v / vx) % vy, c = v / (vx * vy);
                vphi[v] = (float)sdf64(sh, world2local(mesh_point(m, I0 + a, J0 + b, K0 + c), x, q));
            }
            __syncwarp();
            for (int u = lane; u < ncut; u += 32) {
                const int e = cutlist[u];
                const int a = e % cx, b = (e / cx) % cy, c = e / (cx * cy);
                float ph[8];
#pragma unroll
                for (int sl = 0; sl < 8; ++sl)
                    ph[sl] = vphi[(a + (sl & 1)) + vx * ((b + ((sl >> 1) & 1)) + vy * (c + ((sl >> 2) & 1)))];
                const int64_t K = K0 + c;
                const float apz = m.twod ? (float)((0.0 - mesh_coord(m, 2, K)) / m.h[2]) : 0.f;
                const float apz1 = m.twod ? (float)((mesh_coord(m, 2, K + 1) - 0.0) / m.h[2]) : 0.f;
                alpha[local_index(a, b, c)] = refgeo32(m, ph, I0 + a, J0 + b, K, apz, apz1);
            }
        } else {
            // SUBSAMPLE (and the fallback of LEARNED): the warp shares the samples of one cut cell
            for (int u = 0; u < ncut; ++u) {
                const int e = cutlist[u];
                const int a = e % cx, b = (e / cx) % cy, c = e / (cx * cy);
                const float al = subsample_warp(m, sh, M, x, q, I0 + a, J0 + b, K0 + c, A.subsample_n, &rechecks);
                if (lane == 0) alpha[local_index(a, b, c)] = al;
            }
        }
        __syncwarp();
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

}  // namespace sdfibm_dev
