// Coupling on an explicit (unstructured) OpenFOAM polyMesh: the reference's own algorithm on any mesh MeshInfo can
// describe (src/meshinfo.h:20-29), for cases whose mesh is graded, multi-block or polyhedral.
//
//   poly_enum_kernel      one CTA per solid: the nearest cell centre as the seed (meshSearch::findNearestCell at
//                         src/solidcloud.cpp:363), the full scan for the first cell with an inside vertex when the
//                         seed has none, then a level-synchronous breadth-first search over the face neighbours
//                         with the reference's classification (CellEnumerator, src/cellenumerator.cpp:6-78): a
//                         neighbour with no inside vertex is marked visited and not followed, the others are
//                         ALL_INSIDE when every vertex of the cell being expanded is inside (the reference compares
//                         with that cell's point count), else CENTER_INSIDE / CENTER_OUTSIDE by the centre test;
//   poly_couple_kernel    one thread per (solid, touched cell): alpha = 1 or the apex / pyramid volume over the cell's
//                         faces (GeometricTools::calcCellVolume, src/geometrictools.cpp:47-116) / V, the direct forcing
//                         (solidcloud.cpp:384-417), FP64 sums per cell over the solids and per solid over its cells;
//   poly_finalize_kernel  the fields from the FP64 sums: As = min(sum, 1) (checkAlpha, solidcloud.cpp:564-570), Ct of
//                         the last solid in the reference's order;
//   poly_fix_kernel       fixInternal (solidcloud.cpp:288-301) with the mesh's cell centres.
// Every geometric decision is FP64 with the reference's operation sequence (the library is built with -fmad=false),
// so touched sets and cell types equal the FP64 oracle's on the same mesh.
#include <cstdint>
#include <cuda_runtime.h>

#include "common.cuh"
#include "poly_dev.cuh"

namespace sdfibm_dev {

__device__ inline D3 poly_point(const PolyK& m, int32_t p) {
    return D3{m.points[3 * (int64_t)p], m.points[3 * (int64_t)p + 1], m.points[3 * (int64_t)p + 2]};
}
__device__ inline D3 poly_vec(const double* a, int64_t i) { return D3{a[3 * i], a[3 * i + 1], a[3 * i + 2]}; }

// Solid::phi01 of mesh point p (shape isInside in the local frame, FP64)
__device__ inline int poly_inside_point(const ShapeK& sh, const PolyK& m, int32_t p, const D3& x, const Q4& q) {
    return inside64(sh, world2local(poly_point(m, p), x, q)) ? 1 : 0;
}
__device__ inline int poly_count_inside(const ShapeK& sh, const PolyK& m, int32_t c, const D3& x, const Q4& q) {
    int n = 0;
    for (int32_t r = m.cp_off[c]; r < m.cp_off[c + 1]; ++r) n += poly_inside_point(sh, m, m.cp[r], x, q);
    return n;
}

// block-wide minimum of (key, index) pairs, lowest index on ties; every thread receives the result
__device__ inline void block_argmin(double& key, int32_t& idx, double* sk, int32_t* si) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int o = 16; o > 0; o >>= 1) {
        const double k2 = __shfl_xor_sync(0xffffffffu, key, o);
        const int32_t i2 = __shfl_xor_sync(0xffffffffu, idx, o);
        if (k2 < key || (k2 == key && i2 < idx)) { key = k2; idx = i2; }
    }
    if (lane == 0) { sk[w] = key; si[w] = idx; }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int i = 1; i < nw; ++i)
            if (sk[i] < sk[0] || (sk[i] == sk[0] && si[i] < si[0])) { sk[0] = sk[i]; si[0] = si[i]; }
    }
    __syncthreads();
    key = sk[0];
    idx = si[0];
    __syncthreads();
}

__global__ void __launch_bounds__(256) poly_enum_kernel(PolyK m, const SolidK* __restrict__ sk,
                                                        const sdfibm_solid_state* __restrict__ st, PolyWork w) {
    __shared__ double s_key[8];
    __shared__ int32_t s_idx[8];
    __shared__ int32_t s_tail, s_over;
    const int s = blockIdx.x;
    const ShapeK& sh = sk[s].shape;
    const Q4 q = state_quat(st[s]);
    const D3 x = state_pos(st[s]);
    uint32_t* visited = w.visited + (int64_t)s * w.words;
    int32_t* queue = w.queue + (int64_t)s * w.qcap;
    int8_t* qtype = w.qtype + (int64_t)s * w.qcap;
    // seed: the cell whose centre is nearest to the solid centre, lowest label on ties
    double best = 1e300;
    int32_t seed = 0x7fffffff;
    for (int32_t c = threadIdx.x; c < m.ncells; c += blockDim.x) {
        const D3 d = poly_vec(m.Cc, c) - x;
        const double d2 = magSqr(d);
        if (d2 < best || (d2 == best && c < seed)) { best = d2; seed = c; }
    }
    block_argmin(best, seed, s_key, s_idx);
    // a seed without an inside vertex: the first cell (by label) that has one, or none
    int n_seed = 0;
    if (threadIdx.x == 0) n_seed = poly_count_inside(sh, m, seed, x, q);
    if (threadIdx.x == 0) s_idx[0] = n_seed;
    __syncthreads();
    n_seed = s_idx[0];
    __syncthreads();
    if (n_seed == 0) {
        int32_t first = 0x7fffffff;
        for (int32_t base = 0; base < m.ncells && first == 0x7fffffff; base += blockDim.x) {
            const int32_t c = base + threadIdx.x;
            int32_t mine = 0x7fffffff;
            if (c < m.ncells && poly_count_inside(sh, m, c, x, q) > 0) mine = c;
            double k = 0.0;
            block_argmin(k, mine, s_key, s_idx);
            first = mine;
        }
        seed = first;
        if (seed == 0x7fffffff) {
            if (threadIdx.x == 0) w.count[s] = 0;
            return;
        }
        if (threadIdx.x == 0) n_seed = poly_count_inside(sh, m, seed, x, q);
    }
    if (threadIdx.x == 0) {
        const int np = m.cp_off[seed + 1] - m.cp_off[seed];
        int8_t t;
        if (n_seed == np) t = 1;
        else t = inside64(sh, world2local(poly_vec(m.Cc, seed), x, q)) ? 2 : 3;
        queue[0] = seed;
        qtype[0] = t;
        atomicOr(&visited[seed >> 5], 1u << (seed & 31));
        s_tail = 1;
        s_over = 0;
    }
    __syncthreads();
    // level-synchronous breadth-first search; every level adds at least one cell or ends it (tail <= qcap)
    int32_t head = 0;
    for (;;) {
        const int32_t tail = s_tail;
        __syncthreads();
        if (head >= tail || s_over) break;
        for (int32_t e = head + threadIdx.x; e < tail; e += blockDim.x) {
            const int32_t cur = queue[e];
            const int np_cur = m.cp_off[cur + 1] - m.cp_off[cur];
            for (int32_t r = m.cc_off[cur]; r < m.cc_off[cur + 1]; ++r) {
                const int32_t nb = m.ccl[r];
                const uint32_t bit = 1u << (nb & 31);
                if (atomicOr(&visited[nb >> 5], bit) & bit) continue;
                const int n_in = poly_count_inside(sh, m, nb, x, q);
                if (n_in == 0) continue;  // ALL_OUTSIDE: visited, not followed
                int8_t t;
                if (n_in == np_cur) t = 1;
                else t = inside64(sh, world2local(poly_vec(m.Cc, nb), x, q)) ? 2 : 3;
                const int32_t pos = atomicAdd(&s_tail, 1);
                if (pos < w.qcap) {
                    queue[pos] = nb;
                    qtype[pos] = t;
                } else {
                    s_over = 1;
                }
            }
        }
        __syncthreads();
        head = tail;
    }
    if (threadIdx.x == 0) {
        if (s_over) {
            w.count[s] = 0;
            atomicCAS(w.err, 0, DERR_CAPACITY);
        } else {
            w.count[s] = s_tail;
        }
    }
}

// GeometricTools::calcLineFraction (geometrictools.cpp:13-23)
__device__ inline double poly_line_fraction(double pa, double pb) {
    if (pa > 0 && pb > 0) return 0;
    if (pa <= 0 && pb <= 0) return 1;
    if (pa > 0) return -pb / (pa - pb);
    return -pa / (pb - pa);
}

constexpr int POLY_MAX_CELL_POINTS = 64;

struct PhiCache {
    int32_t label[POLY_MAX_CELL_POINTS];
    double phi[POLY_MAX_CELL_POINTS];
    int n;
    __device__ double get(int32_t p) const {
        for (int i = 0; i < n; ++i)
            if (label[i] == p) return phi[i];
        return 0.0;
    }
};

// GeometricTools::calcApex over a list of point labels (geometrictools.cpp:25-45)
__device__ inline D3 poly_apex(const PolyK& m, const int32_t* v, int n, const PhiCache& pc) {
    const D3 A = poly_point(m, v[0]);
    const double phiA = pc.get(v[0]);
    D3 B{0.0, 0.0, 0.0};
    double phiB = 0.0;
    for (int i = 1; i < n; ++i) {
        B = poly_point(m, v[i]);
        phiB = pc.get(v[i]);
        if (phiA * phiB <= 0) break;
    }
    return A - fabs(phiA) / (SMALL_D + fabs(phiA) + fabs(phiB)) * (A - B);
}

// GeometricTools::calcCellVolume (geometrictools.cpp:47-72) with calcFaceAreaFraction / calcFaceArea (:74-116)
__device__ double poly_cell_volume(const PolyK& m, int32_t c, const ShapeK& sh, const D3& x, const Q4& q) {
    PhiCache pc;
    pc.n = 0;
    const int32_t p0 = m.cp_off[c], np = m.cp_off[c + 1] - p0;
    for (int i = 0; i < np && i < POLY_MAX_CELL_POINTS; ++i) {
        pc.label[i] = m.cp[p0 + i];
        pc.phi[i] = sdf64(sh, world2local(poly_point(m, m.cp[p0 + i]), x, q));
        pc.n = i + 1;
    }
    D3 apex = poly_apex(m, m.cp + p0, np, pc);
    if (m.twod) apex.z = 0.0;
    double volume = 0.0;
    for (int32_t r = m.cf_off[c]; r < m.cf_off[c + 1]; ++r) {
        const int32_t f = m.cf[r];
        const int32_t* fv = m.face_lab + m.face_off[f];
        const int nv = m.face_off[f + 1] - m.face_off[f];
        int sign_sum = 0;
        for (int i = 0; i < nv; ++i) sign_sum += pc.get(fv[i]) > 0 ? 1 : -1;
        double eps;
        if (sign_sum == nv) {
            eps = 0.0;
        } else if (sign_sum == -nv) {
            eps = 1.0;
        } else {
            const D3 fa = poly_apex(m, fv, nv, pc);
            double area = 0.0;
            for (int i = 0; i < nv; ++i) {
                const double phiO = pc.get(fv[i]), phiA = pc.get(fv[(i + 1) % nv]);
                const D3 O = poly_point(m, fv[i]), A = poly_point(m, fv[(i + 1) % nv]);
                area += fabs(0.5 * mag(cross(A - O, fa - O))) * poly_line_fraction(phiO, phiA);
            }
            eps = area / mag(poly_vec(m.Sf, f));
        }
        volume += (1.0 / 3.0) * eps * fabs(dot(apex - poly_vec(m.Cf, f), poly_vec(m.Sf, f)));
    }
    return volume;
}

// One thread per touched cell of one solid (blockIdx.y): fraction, forcing, FP64 sums.
__global__ void __launch_bounds__(256) poly_couple_kernel(PolyK m, const SolidK* __restrict__ sk,
                                                          const sdfibm_solid_state* __restrict__ st, PolyWork w,
                                                          const float* __restrict__ U, double* __restrict__ ftacc,
                                                          const StepParams* step) {
    const int s = blockIdx.y;
    const int32_t n = w.count[s];
    const ShapeK& sh = sk[s].shape;
    const Q4 q = state_quat(st[s]);
    const D3 x = state_pos(st[s]);
    const D3 v{st[s].vel[0], st[s].vel[1], st[s].vel[2]};
    const D3 om{st[s].omega[0], st[s].omega[1], st[s].omega[2]};
    const double dtINV = step->dtINV;
    const int32_t* queue = w.queue + (int64_t)s * w.qcap;
    const int8_t* qtype = w.qtype + (int64_t)s * w.qcap;
    double acc[6] = {0, 0, 0, 0, 0, 0};
    for (int32_t e = blockIdx.x * blockDim.x + threadIdx.x; e < n; e += gridDim.x * blockDim.x) {
        const int32_t c = queue[e];
        const int t = qtype[e];
        const double V = m.Vc[c];
        const double alpha = t == 1 ? 1.0 : poly_cell_volume(m, c, sh, x, q) / V;
        const D3 C = poly_vec(m.Cc, c);
        const D3 uf{(double)U[c], (double)U[(int64_t)m.ncells + c], (double)U[2 * (int64_t)m.ncells + c]};
        const D3 us = v + cross(om, C - x);  // Solid::evalPointVelocity
        const D3 f = alpha * (uf - us);
        const D3 tq = cross(C - x, f);
        const D3 fv = f * V * dtINV, tv = tq * V * dtINV;
        acc[0] += fv.x; acc[1] += fv.y; acc[2] += fv.z;
        acc[3] += tv.x; acc[4] += tv.y; acc[5] += tv.z;
        double* a = w.acc + 5 * (int64_t)c;
        atomicAdd(a + 0, alpha);
        atomicAdd(a + 1, alpha);
        const D3 fd = f * dtINV;
        atomicAdd(a + 2, fd.x);
        atomicAdd(a + 3, fd.y);
        atomicAdd(a + 4, fd.z);
        atomicMax(w.claim + c, 4 * s + t);
    }
    for (int r = 0; r < 6; ++r) {
        double y = acc[r];
        for (int o = 16; o > 0; o >>= 1) y += __shfl_xor_sync(0xffffffffu, y, o);
        if ((threadIdx.x & 31) == 0 && y != 0.0) atomicAdd(ftacc + 6 * s + r, y);
    }
}

// fields of every cell from the sums (cells no solid touched hold zeros)
__global__ void poly_finalize_kernel(PolyWork w, int32_t N, float* __restrict__ As, float* __restrict__ Fs,
                                     float* __restrict__ Ts, int32_t* __restrict__ Ct) {
    for (int32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < N; c += gridDim.x * blockDim.x) {
        const double* a = w.acc + 5 * (int64_t)c;
        const int32_t k = w.claim[c];
        As[c] = (float)fmin(a[0], 1.0);
        Ts[c] = (float)a[1];
        Fs[c] = (float)a[2];
        Fs[(int64_t)N + c] = (float)a[3];
        Fs[2 * (int64_t)N + c] = (float)a[4];
        Ct[c] = k < 0 ? 0 : ((k & 3) == 1 ? (k >> 2) + 4 : (k & 3));
    }
}

// SolidCloud::fixInternal: U = velocity of solid Ct - 4 at the cell centre where Ct >= 4
__global__ void poly_fix_kernel(PolyK m, const sdfibm_solid_state* __restrict__ st, int S, const int32_t* __restrict__ Ct,
                                float* __restrict__ U) {
    const int32_t N = m.ncells;
    for (int32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < N; c += gridDim.x * blockDim.x) {
        const int32_t k = Ct[c];
        if (k < 4 || k - 4 >= S) continue;
        const sdfibm_solid_state& x = st[k - 4];
        const D3 C = poly_vec(m.Cc, c);
        const D3 us = D3{x.vel[0], x.vel[1], x.vel[2]} +
                      cross(D3{x.omega[0], x.omega[1], x.omega[2]}, C - D3{x.pos[0], x.pos[1], x.pos[2]});
        U[c] = (float)us.x;
        U[(int64_t)N + c] = (float)us.y;
        U[2 * (int64_t)N + c] = (float)us.z;
    }
}

}  // namespace sdfibm_dev
