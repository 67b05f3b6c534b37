// Device helpers shared by the coupling kernels: closed-form uniform-mesh geometry, solid state access, the FP32
// inside test with its FP64 re-check, and the work-queue lookup.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "kernels.cuh"

namespace sdfibm_dev {

__device__ inline void set_error(Counters* cnt, int32_t code) { atomicCAS(&cnt->error, 0, code); }

// ---- geometry helpers (closed form of the uniform mesh, identical to the oracle's UniformMesh) ----------------------
__device__ inline double mesh_coord(const MeshK& m, int a, int64_t i) { return m.o[a] + (double)i * m.h[a]; }
__device__ inline double mesh_centre(const MeshK& m, int a, int64_t i) { return m.o[a] + ((double)i + 0.5) * m.h[a]; }
__device__ inline D3 mesh_point(const MeshK& m, int64_t i, int64_t j, int64_t k) {
    return D3{mesh_coord(m, 0, i), mesh_coord(m, 1, j), mesh_coord(m, 2, k)};
}
__device__ inline D3 mesh_C(const MeshK& m, int64_t i, int64_t j, int64_t k) {
    return D3{mesh_centre(m, 0, i), mesh_centre(m, 1, j), mesh_centre(m, 2, k)};
}

__device__ inline Q4 state_quat(const sdfibm_solid_state& s) { return Q4{s.quat[0], D3{s.quat[1], s.quat[2], s.quat[3]}}; }
__device__ inline D3 state_pos(const sdfibm_solid_state& s) { return D3{s.pos[0], s.pos[1], s.pos[2]}; }

// ---- inside test of one world point given as integer lattice offsets ------------------------------------------------
// base: FP64 (point(I0,J0,K0) - x_s) of the tile; off: FP32 offset of the point from that lattice point.
// Exact fallback evaluates the point with the mesh formula in FP64, as the oracle does.
struct TileFrame {
    float bx, by, bz;  // FP32 of the FP64 base vector
    float babs;        // |base|_1
    float e64;         // bound of the FP64 reference's own rounding of point coordinates (large meshes offsets)
};
__device__ inline TileFrame make_frame(const D3& b, const D3& p0, const D3& x) {
    TileFrame tf;
    tf.bx = (float)b.x; tf.by = (float)b.y; tf.bz = (float)b.z;
    tf.babs = fabsf(tf.bx) + fabsf(tf.by) + fabsf(tf.bz);
    tf.e64 = (float)(1e-15 * (fabs(p0.x) + fabs(p0.y) + fabs(p0.z) + fabs(x.x) + fabs(x.y) + fabs(x.z)));
    return tf;
}

// The reference's FP64 inside test of mesh point (I,J,K) (centre: of cell (I,J,K)).  Kept out of line so the
// compiler cannot evaluate it speculatively on the FP32 fast path: it only runs for undecided points.
static __device__ __noinline__ int exact_inside_point(const ShapeK& sh, const MeshK& m, int64_t I, int64_t J, int64_t K,
                                               int centre, const D3& x, const Q4& q) {
    const D3 p = centre ? D3{m.o[0] + ((double)I + 0.5) * m.h[0], m.o[1] + ((double)J + 0.5) * m.h[1],
                             m.o[2] + ((double)K + 0.5) * m.h[2]}
                        : D3{m.o[0] + (double)I * m.h[0], m.o[1] + (double)J * m.h[1], m.o[2] + (double)K * m.h[2]};
    return inside64(sh, world2local(p, x, q)) ? 1 : 0;
}

// FP32 inside test of a point given by its offset (ox,oy,oz) from the tile frame's base point, with the FP64
// re-check inside the guard band
__device__ inline int classify_point(const ShapeK& sh, const float* M, const TileFrame& tf, float ox, float oy,
                                     float oz, const MeshK& m, int64_t I, int64_t J, int64_t K, int centre,
                                     const D3& x, const Q4& q, unsigned long long* rechecks) {
    const float dx = tf.bx + ox, dy = tf.by + oy, dz = tf.bz + oz;
    const float lx = __fmaf_rn(M[0], dx, __fmaf_rn(M[1], dy, M[2] * dz));
    const float ly = __fmaf_rn(M[3], dx, __fmaf_rn(M[4], dy, M[5] * dz));
    const float lz = __fmaf_rn(M[6], dx, __fmaf_rn(M[7], dy, M[8] * dz));
    const float dabs = fabsf(dx) + fabsf(dy) + fabsf(dz);
    const float E = 4.f * U32 * (tf.babs + fabsf(ox) + fabsf(oy) + fabsf(oz) + 2.f * dabs) + tf.e64 + 1e-30f;
    int r = inside32(sh, lx, ly, lz, E);
    if (r == 2) {
        ++*rechecks;  // caller-local counter
        r = exact_inside_point(sh, m, I, J, K, centre, x, q);
    }
    return r;
}

__device__ inline int find_solid(const int32_t* prefix, int S, int item) {
    int lo = 0, hi = S;  // prefix[lo] <= item < prefix[hi]
    while (hi - lo > 1) {
        int mid = (lo + hi) >> 1;
        if (prefix[mid] <= item) lo = mid; else hi = mid;
    }
    return lo;
}

}  // namespace sdfibm_dev
