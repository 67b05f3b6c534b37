// Rigid-body side of the time step: the GB300 replacement of SolidCloud::evolve (src/solidcloud.cpp:521-562) with
// Solid::applyForcer / addMidFluidForceAndTorque / addAcceleration / move / storeOldForce (src/solid.h:126-202),
// addMidEnvironment (solidcloud.cpp:466-475), the motions (src/libmotion) and forcers (src/libforcer), and the
// uniform-grid collision of solidSolidInteract / solidSolidCollision (solidcloud.cpp:477-519,
// src/libcollision/ugrid.cpp:5-77, collision.cpp:7-57).
//
// Without collisions every solid is independent, so one thread runs all sub-steps of one solid in a single launch.
// With collisions each sub-step is: forces + grid hash, counting sort of solid ids by grid cell, pair forces
// (each solid sums its own side of every pair: no atomics, the pair law is evaluated once per side), move.
#include <cstdint>
#include <cuda_runtime.h>

#include "common.cuh"

namespace sdfibm_dev {

__device__ inline D3 ld3(const double* a) { return D3{a[0], a[1], a[2]}; }
__device__ inline void st3(double* a, const D3& v) { a[0] = v.x; a[1] = v.y; a[2] = v.z; }

// IMotion::constraint of each registered motion
__device__ inline void motion_constraint(const SolidK& k, double time, D3& velocity, D3& omega) {
    const double* p = k.motion_p;
    switch (k.motion_type) {
        case SDFIBM_MOTION_000002: velocity = D3{0, 0, 0}; omega = D3{0, 0, 0}; omega.z = p[1]; return;
        case SDFIBM_MOTION_110002: velocity.z = 0.0; omega = D3{0, 0, 0}; omega.z = p[1]; return;
        case SDFIBM_MOTION_222000: velocity = D3{p[0], p[1], p[2]}; omega = D3{0, 0, 0}; return;
        case SDFIBM_MOTION_SINEDIRECTIONAL:
            velocity = p[0] * p[2] * cos(p[2] * time) * D3{p[3], p[4], p[5]};
            omega = D3{0, 0, 0};
            return;
        case SDFIBM_MOTION_01MASK:
            velocity = D3{velocity.x * p[0], velocity.y * p[1], velocity.z * p[2]};
            omega = D3{omega.x * p[3], omega.y * p[4], omega.z * p[5]};
            return;
        case SDFIBM_MOTION_ROTOR:
            velocity = D3{0, 0, 0};
            velocity.x = -p[2] * p[1] * sin(p[1] * time + p[3]);
            velocity.y = p[2] * p[1] * cos(p[1] * time + p[3]);
            omega = D3{0, 0, 0};
            omega.z = p[4];
            return;
        case SDFIBM_MOTION_OPENCLOSE: {
            const double t = fmod(time, 5.0);
            double v = 0.0;
            if (t > 1 && t < 2) v = -1.0;
            if (t > 3 && t < 4) v = 1.0;
            velocity = D3{0, v, 0};
            omega = D3{0, 0, 0};
            return;
        }
        default: return;
    }
}

// IForcer::generate of each registered forcer
__device__ inline void forcer_generate(const SolidK& k, const sdfibm_solid_state& s, double time, D3& f, D3& t) {
    const double* p = k.forcer_p;
    f = D3{0, 0, 0};
    t = D3{0, 0, 0};
    switch (k.forcer_type) {
        case SDFIBM_FORCER_CONSTANT: f = D3{p[0], p[1], p[2]}; t = D3{p[3], p[4], p[5]}; return;
        case SDFIBM_FORCER_SPRING: {
            const D3 r = ld3(s.pos) - D3{p[0], p[1], p[2]};
            if (mag(r) > SMALL_D) f = -p[3] * r * (1.0 - p[4] / mag(r));
            return;
        }
        case SDFIBM_FORCER_MAGNETIC: {
            const D3 m_original = (1.0) * (D3{0.0, 0.0, 1.0});
            const D3 B = p[3] * cos(p[4] * time) * D3{p[0], p[1], p[2]};
            const Q4 q{s.quat[0], D3{s.quat[1], s.quat[2], s.quat[3]}};
            const D3 m = qtransform(qconj(q), m_original);
            t = cross(m, B);
            return;
        }
        default: return;
    }
}

// clearForceAndTorque, applyForcer, addMidFluidForceAndTorque, addMidEnvironment for one solid
__device__ inline void pre_forces(const SolidK& k, sdfibm_solid_state& s, double time, double rho_f, const D3& g) {
    D3 force{0, 0, 0}, torque{0, 0, 0};
    if (k.forcer_type != SDFIBM_FORCER_NONE) {
        D3 f_, t_;
        forcer_generate(k, s, time, f_, t_);
        st3(s.forcer_force, f_);
        st3(s.forcer_torque, t_);
        if (s.first_forcer_step) {
            st3(s.forcer_force_old, f_);
            st3(s.forcer_torque_old, t_);
            s.first_forcer_step = 0;
        }
        force = force + (1.5 * ld3(s.forcer_force) - 0.5 * ld3(s.forcer_force_old));
        torque = torque + (1.5 * ld3(s.forcer_torque) - 0.5 * ld3(s.forcer_torque_old));
    }
    if (s.first_fluid_step) {
        for (int a = 0; a < 3; ++a) { s.fluid_force_old[a] = s.fluid_force[a]; s.fluid_torque_old[a] = s.fluid_torque[a]; }
        s.first_fluid_step = 0;
    }
    force = force + (1.5 * ld3(s.fluid_force) - 0.5 * ld3(s.fluid_force_old));
    torque = torque + (1.5 * ld3(s.fluid_torque) - 0.5 * ld3(s.fluid_torque_old));
    const double rhos = k.rho;
    const D3 gprime = ((rhos - rho_f) / rhos) * g;
    force = force + k.mass * gprime;
    st3(s.force, force);
    st3(s.torque, torque);
}

// Solid::move
__device__ inline void move_solid(const SolidK& k, sdfibm_solid_state& s, double time, double dt) {
    const D3 velocity_old = ld3(s.vel), omega_old = ld3(s.omega);
    D3 vel = velocity_old + ld3(s.force) * k.mass_inv * dt;
    const Q4 q{s.quat[0], D3{s.quat[1], s.quat[2], s.quat[3]}};
    const double w2 = q.w * q.w, x2 = q.v.x * q.v.x, y2 = q.v.y * q.v.y, z2 = q.v.z * q.v.z;
    const double txy = 2 * q.v.x * q.v.y, twz = 2 * q.w * q.v.z, txz = 2 * q.v.x * q.v.z;
    const double twy = 2 * q.w * q.v.y, tyz = 2 * q.v.y * q.v.z, twx = 2 * q.w * q.v.x;
    const double R[9] = {w2 + x2 - y2 - z2, txy - twz, txz + twy, txy + twz, w2 - x2 + y2 - z2,
                         tyz - twx, txz - twy, tyz + twx, w2 - x2 - y2 + z2};
    const double* I = k.moi_inv;
    double RI[9], W[9];
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) RI[3 * r + c] = R[3 * r] * I[c] + R[3 * r + 1] * I[3 + c] + R[3 * r + 2] * I[6 + c];
    for (int r = 0; r < 3; ++r)  // (R & I) & R^T
        for (int c = 0; c < 3; ++c) W[3 * r + c] = RI[3 * r] * R[3 * c] + RI[3 * r + 1] * R[3 * c + 1] + RI[3 * r + 2] * R[3 * c + 2];
    const D3 T = ld3(s.torque);
    const D3 WT{W[0] * T.x + W[1] * T.y + W[2] * T.z, W[3] * T.x + W[4] * T.y + W[5] * T.z,
                W[6] * T.x + W[7] * T.y + W[8] * T.z};
    D3 om = omega_old + WT * dt;
    if (k.motion_type != SDFIBM_MOTION_FREE) motion_constraint(k, time, vel, om);
    const D3 c = ld3(s.pos) + 0.5 * (vel + velocity_old) * dt;
    const Q4 h{0.5 * 0.0, 0.5 * (0.5 * (om + omega_old))};
    const Q4 dq0 = qmul(h, q);
    const Q4 dq{dq0.w * dt, dq0.v * dt};
    Q4 qn{q.w + dq.w, q.v + dq.v};
    const double mq = sqrt(qn.w * qn.w + magSqr(qn.v));
    qn = Q4{qn.w / mq, qn.v / mq};
    st3(s.vel, vel);
    st3(s.omega, om);
    st3(s.pos, c);
    s.quat[0] = qn.w; s.quat[1] = qn.v.x; s.quat[2] = qn.v.y; s.quat[3] = qn.v.z;
}

__device__ inline void store_old(sdfibm_solid_state& s) {
    for (int a = 0; a < 3; ++a) {
        s.fluid_force_old[a] = s.fluid_force[a];
        s.fluid_torque_old[a] = s.fluid_torque[a];
        s.forcer_force_old[a] = s.forcer_force[a];
        s.forcer_torque_old[a] = s.forcer_torque[a];
    }
}

// all sub-steps of one solid (no solid-solid interaction)
__global__ void evolve_independent_kernel(const SolidK* __restrict__ sk, sdfibm_solid_state* st, int S, int nsub,
                                          const StepParams* step, double rho_f, D3 g) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= S) return;
    const double time = step->time, dt_sub = step->dt_sub;
    const SolidK& k = sk[s];
    sdfibm_solid_state x = st[s];
    for (int it = 0; it < nsub; ++it) {
        pre_forces(k, x, time, rho_f, g);
        move_solid(k, x, time, dt_sub);
    }
    store_old(x);
    st[s] = x;
}



__device__ inline int64_t grid_hash(const GridK& gk, const D3& c) {
    const int i = (int)floor((c.x - gk.low[0]) * gk.dINV);
    const int j = (int)floor((c.y - gk.low[1]) * gk.dINV);
    const int k = (int)floor((c.z - gk.low[2]) * gk.dINV);
    return (int64_t)i * gk.nynz + (int64_t)j * gk.nz + k;
}

// collision id of the pair-law table: SPHERES mode treats every non-plane solid as its bounding sphere
__device__ inline int coll_id(const SolidK& k, int mode) {
    return mode == SDFIBM_COLLISION_SPHERES ? (k.infinite ? 0 : 2) : k.collision_id;
}

// fine-grid cell range of a bounding box, clamped to the grid
__device__ inline void fine_range(const FineGridK& fg, const D3& c, double r, int lo[3], int hi[3]) {
    const double cc[3] = {c.x, c.y, c.z};
    for (int a = 0; a < 3; ++a) {
        const double l = floor((cc[a] - r - fg.low[a]) * fg.inv), h = floor((cc[a] + r - fg.low[a]) * fg.inv);
        lo[a] = (int)fmin(fmax(l, 0.0), (double)(fg.n[a] - 1));
        hi[a] = (int)fmin(fmax(h, 0.0), (double)(fg.n[a] - 1));
    }
}
__device__ inline int64_t fine_index(const FineGridK& fg, int i, int j, int k) {
    return (int64_t)i + (int64_t)fg.n[0] * ((int64_t)j + (int64_t)fg.n[1] * k);
}

// forces of one sub-step, the UGrid key of every solid (UGrid::insert, ugrid.h:31-34) with the coarse counts (only
// needed by plane-like solids, which search their 27 coarse neighbours), the fine-grid counts of the sphere-like
// solids whose key is on the grid (the reference never pairs the others) and the solid's collision record
__global__ void evolve_pre_kernel(const SolidK* __restrict__ sk, sdfibm_solid_state* st, int S,
                                  const StepParams* step, double rho_f, D3 g, GridK gk, int64_t* __restrict__ hashes,
                                  int32_t* __restrict__ counts, FineGridK fg, int32_t* __restrict__ fcounts, int mode,
                                  int coarse_needed, CollRec* __restrict__ recs, int move_first) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= S) return;
    if (move_first) move_solid(sk[s], st[s], step->time, step->dt_sub);  // Solid::move of the previous sub-step
    pre_forces(sk[s], st[s], step->time, rho_f, g);
    const D3 c = ld3(st[s].pos);
    const int64_t h = grid_hash(gk, c);
    hashes[s] = h;
    CollRec rec{};
    rec.id = -1;
    if (h >= 0 && h < gk.ncell) {
        if (coarse_needed) atomicAdd(counts + h, 1);
        const double rB = sk[s].radiusB;
        rec.id = coll_id(sk[s], mode);
        rec.c[0] = (int32_t)(h / gk.nynz);
        rec.c[1] = (int32_t)((h / gk.nz) % gk.ny);
        rec.c[2] = (int32_t)(h % gk.nz);
        rec.x = (float)c.x; rec.y = (float)c.y; rec.z = (float)c.z; rec.r = (float)rB;
        if (rec.id == 1 || rec.id == 2) {
            fine_range(fg, c, rB, rec.lo, rec.hi);
            for (int k = rec.lo[2]; k <= rec.hi[2]; ++k)
                for (int j = rec.lo[1]; j <= rec.hi[1]; ++j)
                    for (int i = rec.lo[0]; i <= rec.hi[0]; ++i) atomicAdd(fcounts + fine_index(fg, i, j, k), 1);
        }
    }
    recs[s] = rec;
}

__global__ void fine_scatter_kernel(const CollRec* __restrict__ recs, int S, FineGridK fg, int32_t* __restrict__ fcursor,
                                    int32_t* __restrict__ flist, Counters* cnt) {
    // one warp per solid: the lanes split its fine cells, so a large solid's claims do not run one after another
    const int lane = threadIdx.x & 31;
    const int s = (int)(((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    if (s >= S) return;
    const CollRec& r = recs[s];
    if (r.id != 1 && r.id != 2) return;
    const int nx = r.hi[0] - r.lo[0] + 1, ny = r.hi[1] - r.lo[1] + 1, nz = r.hi[2] - r.lo[2] + 1;
    for (int e = lane; e < nx * ny * nz; e += 32) {
        const int i = r.lo[0] + e % nx, j = r.lo[1] + (e / nx) % ny, k = r.lo[2] + e / (nx * ny);
        const int32_t slot = atomicAdd(fcursor + fine_index(fg, i, j, k), 1);
        if (slot < fg.cap) flist[slot] = s;
        else set_error(cnt, DERR_CAPACITY);
    }
}

// exclusive scan of the per-cell counts (single block), zeroing them as they are read
__global__ void grid_scan_kernel(int32_t* __restrict__ counts, int32_t* __restrict__ start,
                                 int32_t* __restrict__ cursor, int64_t ncell) {
    __shared__ int32_t warp_tot[32];
    __shared__ int32_t carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int64_t base = 0; base < ncell; base += blockDim.x) {
        const int64_t i = base + threadIdx.x;
        const int32_t v = i < ncell ? counts[i] : 0;
        if (i < ncell) counts[i] = 0;  // read once: left zeroed for the next sub-step's counts
        int32_t x = v;
        for (int o = 1; o < 32; o <<= 1) {
            int32_t y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) warp_tot[wid] = x;
        __syncthreads();
        if (wid == 0) {
            int32_t w = lane < nw ? warp_tot[lane] : 0;
            for (int o = 1; o < 32; o <<= 1) {
                int32_t y = __shfl_up_sync(0xffffffffu, w, o);
                if (lane >= o) w += y;
            }
            if (lane < nw) warp_tot[lane] = w;
        }
        __syncthreads();
        const int32_t excl = carry + (wid > 0 ? warp_tot[wid - 1] : 0) + x - v;
        if (i < ncell) { start[i] = excl; cursor[i] = excl; }
        __syncthreads();
        if (threadIdx.x == 0) carry += warp_tot[nw - 1];
        __syncthreads();
    }
    if (threadIdx.x == 0) start[ncell] = carry;
}

// exclusive scan of large count arrays in three launches: per-1024-block scans, a scan of the block sums, offsets;
// the counts are zeroed as they are read
__global__ void __launch_bounds__(1024) scan_blocks_kernel(int32_t* __restrict__ counts, int32_t* __restrict__ start,
                                                           int32_t* __restrict__ sums, int64_t ncell) {
    __shared__ int32_t warp_tot[32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int64_t i = (int64_t)blockIdx.x * 1024 + threadIdx.x;
    const int32_t v = i < ncell ? counts[i] : 0;
    if (i < ncell) counts[i] = 0;  // read once: left zeroed for the next sub-step's counts
    int32_t x = v;
    for (int o = 1; o < 32; o <<= 1) {
        const int32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_tot[wid] = x;
    __syncthreads();
    if (wid == 0) {
        int32_t w = warp_tot[lane];
        for (int o = 1; o < 32; o <<= 1) {
            const int32_t y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        warp_tot[lane] = w;
    }
    __syncthreads();
    if (i < ncell) start[i] = (wid > 0 ? warp_tot[wid - 1] : 0) + x - v;
    if (threadIdx.x == 1023) sums[blockIdx.x] = warp_tot[31];
}

__global__ void __launch_bounds__(1024) scan_add_kernel(int32_t* __restrict__ start, int32_t* __restrict__ cursor,
                                                        const int32_t* __restrict__ sums_excl, int64_t ncell,
                                                        int64_t nblocks) {
    const int64_t i = (int64_t)blockIdx.x * 1024 + threadIdx.x;
    if (i < ncell) {
        const int32_t v = start[i] + sums_excl[blockIdx.x];
        start[i] = v;
        cursor[i] = v;
    }
    if (i == 0) start[ncell] = sums_excl[nblocks];  // the scan of the sums holds the total at nblocks
}

__global__ void grid_scatter_kernel(const int64_t* __restrict__ hashes, int32_t* __restrict__ cursor,
                                    int32_t* __restrict__ list, int S, int64_t ncell) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= S) return;
    const int64_t h = hashes[s];
    if (h >= 0 && h < ncell) list[atomicAdd(cursor + h, 1)] = s;
}

// the collision laws of collision.cpp:7-35 (positions of the sub-step start)
__device__ inline double plane_sphere(const sdfibm_solid_state& p, const sdfibm_solid_state& s, double rB_s, D3& cN) {
    const Q4 qp{p.quat[0], D3{p.quat[1], p.quat[2], p.quat[3]}};
    const D3 s_center = qtransform(qconj(qp), ld3(s.pos) - ld3(p.pos));
    const double p2s = s_center.y;
    cN = qtransform(qp, D3{0, 1, 0});
    return rB_s - p2s;
}
__device__ inline double sphere_sphere(const sdfibm_solid_state& s1, const sdfibm_solid_state& s2, double r1,
                                       double r2, D3& cN) {
    const D3 s2s = ld3(s2.pos) - ld3(s1.pos);
    const double m = mag(s2s);
    cN = m < 1e-150 ? D3{0, 0, 0} : s2s / m;
    return r1 + r2 - mag(s2s);
}

// contact force on s2 (s1 receives the opposite); returns false when the pair has no law or no overlap
__device__ inline bool pair_force(const SolidK& k1, const sdfibm_solid_state& s1, int id1, const SolidK& k2,
                                  const sdfibm_solid_state& s2, int id2, D3& f) {
    double cd;
    D3 cN;
    if ((id1 == 1 || id1 == 2) && id2 == 0) cd = plane_sphere(s2, s1, k1.radiusB, cN);
    else if (id1 == 0 && (id2 == 1 || id2 == 2)) cd = plane_sphere(s1, s2, k2.radiusB, cN);
    else if ((id1 == 1 && id2 == 1) || (id1 == 2 && id2 == 2)) cd = sphere_sphere(s1, s2, k1.radiusB, k2.radiusB, cN);
    else return false;
    if (cd < 0) return false;
    f = 1e4 * cd * cN;
    return true;
}

// the 27 coarse cells around key a contain key b (the neighbour loops of ugrid.cpp:50-77)
__device__ inline bool coarse_neighbours(const GridK& gk, int64_t a, int64_t b) {
    const int64_t ai = a / gk.nynz, aj = (a / gk.nz) % gk.ny, ak = a % gk.nz;
    const int64_t bi = b / gk.nynz, bj = (b / gk.nz) % gk.ny, bk = b % gk.nz;
    return llabs(ai - bi) <= 1 && llabs(aj - bj) <= 1 && llabs(ak - bk) <= 1;
}
__device__ inline bool coarse_neighbours(const CollRec& a, const CollRec& b) {
    return abs(a.c[0] - b.c[0]) <= 1 && abs(a.c[1] - b.c[1]) <= 1 && abs(a.c[2] - b.c[2]) <= 1;
}

// FP32 screen of a sphere pair: false only when the bounding spheres are certainly apart, i.e. the FP64 contact depth
// r1 + r2 - |x2 - x1| is negative.  The FP32 values carry relative errors of a few 2^-24; the margin is 2^-16 of the
// magnitudes involved, far above them.
__device__ inline bool sphere_screen(const CollRec& a, const CollRec& b) {
    const float dx = b.x - a.x, dy = b.y - a.y, dz = b.z - a.z;
    const float mag = fmaxf(fmaxf(fabsf(a.x), fabsf(a.y)), fabsf(a.z)) + fmaxf(fmaxf(fabsf(b.x), fabsf(b.y)), fabsf(b.z));
    const float reach = a.r + b.r + 1.52587890625e-5f * (mag + a.r + b.r);
    return dx * dx + dy * dy + dz * dz <= reach * reach;
}

// Pair forces of one sub-step, each solid summing its own side of every pair the reference's UGrid would form
// (27 coarse neighbours of its key, keys on the grid) that has a contact law and overlaps.  Sphere-like pairs come
// from the fine grid: a pair is taken in the one fine cell holding the corner max(lo_p, lo_q) of the two bounding
// boxes' intersection, then kept only when the coarse keys are neighbours, so the contacts are exactly the
// reference's.  Plane-like solids (law id 0) search the coarse grid; sphere-like solids test the plane list.
__global__ void collide_kernel(const SolidK* __restrict__ sk, sdfibm_solid_state* st, int S, GridK gk,
                               const int64_t* __restrict__ hashes, const int32_t* __restrict__ start,
                               const int32_t* __restrict__ list, int mode, FineGridK fg,
                               const int32_t* __restrict__ fstart, const int32_t* __restrict__ flist,
                               const int32_t* __restrict__ planes, int nplanes, const CollRec* __restrict__ recs) {
    // one warp per solid: lanes split the solid's fine cells (a large solid spans thousands), the plane list, or the
    // entries of its coarse cells; the warp sums the force
    const int lane = threadIdx.x & 31;
    const int p = (int)(((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    if (p >= S) return;
    const CollRec rp = recs[p];
    if (rp.id < 0) return;
    const SolidK& kp = sk[p];
    const int idp = rp.id;
    D3 fsum{0, 0, 0};
    const sdfibm_solid_state& sp = st[p];
    auto add_pair = [&](int q, int idq) {
        D3 f;
        if (p < q) {
            if (pair_force(kp, sp, idp, sk[q], st[q], idq, f)) fsum = fsum + (-f);
        } else {
            if (pair_force(sk[q], st[q], idq, kp, sp, idp, f)) fsum = fsum + f;
        }
    };
    if (idp == 1 || idp == 2) {
        const int nx = rp.hi[0] - rp.lo[0] + 1, ny = rp.hi[1] - rp.lo[1] + 1, nz = rp.hi[2] - rp.lo[2] + 1;
        const int ncells = nx * ny * nz;
        for (int e = lane; e < ncells; e += 32) {
            const int i = rp.lo[0] + e % nx, j = rp.lo[1] + (e / nx) % ny, k = rp.lo[2] + e / (nx * ny);
            const int64_t cell = fine_index(fg, i, j, k);
            for (int f = fstart[cell]; f < fstart[cell + 1]; ++f) {
                const int q = flist[f];
                if (q == p) continue;
                const CollRec rq = recs[q];
                if (rq.id != idp) continue;  // (1,1) and (2,2) have a law, (1,2) has none
                // the pair's home cell: the corner max(lo_p, lo_q) of the two cell ranges' intersection (both solids
                // compute it from the same indices, so exactly one of p's and one of q's visits holds the pair)
                if (max(rp.lo[0], rq.lo[0]) != i || max(rp.lo[1], rq.lo[1]) != j || max(rp.lo[2], rq.lo[2]) != k)
                    continue;
                if (i > rq.hi[0] || j > rq.hi[1] || k > rq.hi[2]) continue;  // ranges do not intersect
                if (!coarse_neighbours(rp, rq) || !sphere_screen(rp, rq)) continue;
                add_pair(q, idp);
            }
        }
        for (int e = lane; e < nplanes; e += 32) {
            const int q = planes[e];
            const CollRec& rq = recs[q];
            if (rq.id < 0 || !coarse_neighbours(rp, rq)) continue;
            add_pair(q, 0);
        }
    } else {
        const int ci = rp.c[0], cj = rp.c[1], ck = rp.c[2];
        for (int a = ci - 1; a <= ci + 1; ++a) {
            if (a < 0 || a > gk.nx - 1) continue;
            for (int b = cj - 1; b <= cj + 1; ++b) {
                if (b < 0 || b > gk.ny - 1) continue;
                for (int c = ck - 1; c <= ck + 1; ++c) {
                    if (c < 0 || c > gk.nz - 1) continue;
                    const int64_t nb = (int64_t)a * gk.nynz + (int64_t)b * gk.nz + c;
                    for (int e = start[nb] + lane; e < start[nb + 1]; e += 32) {
                        const int q = list[e];
                        if (q != p) add_pair(q, recs[q].id);
                    }
                }
            }
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        fsum.x += __shfl_xor_sync(0xffffffffu, fsum.x, o);
        fsum.y += __shfl_xor_sync(0xffffffffu, fsum.y, o);
        fsum.z += __shfl_xor_sync(0xffffffffu, fsum.z, o);
    }
    // force += -f / +f in pair order (reordered sum); torque += -0 leaves it unchanged
    if (lane == 0) {
        st[p].force[0] += fsum.x;
        st[p].force[1] += fsum.y;
        st[p].force[2] += fsum.z;
    }
}

__global__ void move_kernel(const SolidK* __restrict__ sk, sdfibm_solid_state* st, int S, const StepParams* step) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= S) return;
    move_solid(sk[s], st[s], step->time, step->dt_sub);
}

__global__ void store_old_kernel(sdfibm_solid_state* st, int S) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= S) return;
    store_old(st[s]);
}

}  // namespace sdfibm_dev
