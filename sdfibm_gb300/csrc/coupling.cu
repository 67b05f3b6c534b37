// Coupling kernels: the GB300 replacement of SolidCloud::interact (src/solidcloud.cpp:361-464) and
// SolidCloud::fixInternal (src/solidcloud.cpp:288-301).
//
// Pipeline of one interact (no host round trip until FT is read back):
//   plan      per solid: bbox origin in cell indices, FP32 world->local matrix, nearest cell (meshSearch), the
//             two-float forms used by the fraction and forcing kernels
//   classify  persistent CTAs pulling (solid, cell-tile) items from an atomic counter; each tile evaluates the
//             inside test once per vertex (FP32 with a guard band, FP64 re-check inside the band) and writes one
//             class byte per cell: 0 no inside vertex, 1 all inside, 2 centre inside, 3 centre outside
//             (CellEnumerator::_next, cellenumerator.cpp:6-34), and lists the cut cells for the fraction kernels
//   fraction  (classify.cu) REF-GEO a thread per listed cell; SUBSAMPLE a warp per listed cell; LEARNED the network,
//             then SUBSAMPLE on the cells outside its band; FP64 rechecks of undecided sample points
//   connect   on a side stream beside the fraction kernels: one CTA (or warp) per solid, bit-parallel flood fill
//             from the seed over cells with an inside vertex (the BFS of CellEnumerator::intersect with its seed
//             fallback, cellenumerator.cpp:47-78), then the reached cells appended to the ALL_INSIDE list or the
//             cut-cell list in ascending cell order; claim of each touched cell; reset of the cells the previous call
//             touched and this one does not (sparse form of solidcloud.cpp:438-441)
//   couple    persistent CTAs over 256-entry chunks of both lists: alpha (1, or the fraction), direct forcing, the
//             final fields of single-owner cells, warp then FP64-atomic reduction of force and torque per solid
//   finalize  cells of several solids from the FP64 table: Ct of the last solid (as the serial loop), As = min(As,1)
//             (checkAlpha); ft: FT = rho_f V / dt * sums
#include <cstdint>
#include <cuda_runtime.h>

#include "common.cuh"

namespace sdfibm_dev {


// ---- plan ---------------------------------------------------------------------------------------------------------
__device__ inline int32_t n3v(const MeshK& m, int a) { return a == 0 ? m.nx : (a == 1 ? m.ny : m.nz); }

__global__ void plan_kernel(MeshK m, const SolidK* __restrict__ sk, const sdfibm_solid_state* __restrict__ st,
                            SolidPlan* __restrict__ plan, int S, Counters* cnt) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= S) return;
    const SolidK& k = sk[s];
    const Q4 q = state_quat(st[s]);
    const D3 x = state_pos(st[s]);
    SolidPlan p;
    local_matrix32(q, p.M);  // |q|^2 R(q)^T: the linear map of world2local
    p.err = 0;
    // local box holding the inside region (widened far beyond FP32 rounding): tiles of the classify pass that lie
    // outside it hold no inside vertex
    p.cull_box = 0;
    p.radius_cells = (float)k.radiusB * (1.f / m.h32[0]);
    if (!k.shape.prism && !k.infinite &&
        (k.shape.type == SDFIBM_SHAPE_SPHERE || k.shape.type == SDFIBM_SHAPE_ELLIPSOID ||
         k.shape.type == SDFIBM_SHAPE_BOX)) {
        const double* sp = k.shape.p;
        const bool ell = k.shape.type == SDFIBM_SHAPE_ELLIPSOID;  // ignores com
        const bool sph = k.shape.type == SDFIBM_SHAPE_SPHERE;
        for (int a = 0; a < 3; ++a) {
            const double half = sph ? sp[0] : sp[a];
            p.lbox_c[a] = ell ? 0.f : (float)(-k.shape.com[a]);
            p.lbox_s[a] = (float)(half * (1.0 + 1e-4) + 1e-4 * fabs(k.shape.com[a]) + 1e-30);
        }
        p.cull_box = 1;
    }
    const int32_t n[3] = {m.nx, m.ny, m.nz};
    p.cw[0] = p.cw[1] = p.cw[2] = 0.0;
    p.rcull = 0.0;
    for (int a = 0; a < 3; ++a) { p.vlo[a] = 0; p.vhi[a] = n3v(m, a); }
    if (k.infinite) {
        p.lo[0] = p.lo[1] = p.lo[2] = 0;
    } else {
        D3 cl{-k.shape.com[0], -k.shape.com[1], -k.shape.com[2]};
        if (k.shape.type == SDFIBM_SHAPE_ELLIPSOID) cl = D3{0, 0, 0};
        if (k.shape.prism) cl.z = 0.0;
        const D3 cw = x + qtransform(q, cl);
        const double r = k.shape.bound_r * (1.0 + 1e-9) + 1e-12;
        double rad[3] = {r, r, r};
        if (k.shape.prism) {
            // the inside region is a prism along the local z axis a; clip it to the mesh slab in z
            const double qq = q.w * q.w + magSqr(q.v);
            const D3 a = qtransform(q, D3{0, 0, 1}) / qq;
            const double sxy = sqrt(a.x * a.x + a.y * a.y), az = fabs(a.z);
            if (az < 0.3 && (k.ext[0] < n[0] + 2 || k.ext[1] < n[1] + 2)) p.err = DERR_BBOX;
            const double zlo = m.o[2], zhi = mesh_coord(m, 2, m.nz);
            const double zspan = dmax(fabs(zhi - cw.z), fabs(zlo - cw.z));
            const double rxy = (sxy > 0) ? r + (zspan + r * sxy) / dmax(az, 0.3) * sxy : r;
            rad[0] = rad[1] = rxy * (1.0 + 1e-9);
        }
        p.cw[0] = cw.x; p.cw[1] = cw.y; p.cw[2] = cw.z;
        p.rcull = rad[0];
        // oriented bounding box of the inside region: half extents along the world axes
        {
            const double qq = q.w * q.w + magSqr(q.v);
            const D3 ex = qtransform(q, D3{1, 0, 0}) / qq, ey = qtransform(q, D3{0, 1, 0}) / qq,
                     ez = qtransform(q, D3{0, 0, 1}) / qq;  // columns of the unit rotation
            const double Rm[3][3] = {{ex.x, ey.x, ez.x}, {ex.y, ey.y, ez.y}, {ex.z, ey.z, ez.z}};
            double e[3] = {rad[0], rad[1], rad[2]};
            const double* sp = k.shape.p;
            if (k.shape.type == SDFIBM_SHAPE_ELLIPSOID) {
                for (int a = 0; a < 3; ++a)
                    e[a] = sqrt(Rm[a][0] * Rm[a][0] * sp[0] * sp[0] + Rm[a][1] * Rm[a][1] * sp[1] * sp[1] +
                                Rm[a][2] * Rm[a][2] * sp[2] * sp[2]);
            } else if (k.shape.type == SDFIBM_SHAPE_BOX) {
                for (int a = 0; a < 3; ++a) e[a] = fabs(Rm[a][0]) * sp[0] + fabs(Rm[a][1]) * sp[1] + fabs(Rm[a][2]) * sp[2];
            }
            const double c3v[3] = {cw.x, cw.y, cw.z};
            for (int a = 0; a < 3; ++a) {
                if (k.shape.prism && a == 2) continue;  // all layers
                const double ea = dmin(e[a], rad[a]) * (1.0 + 1e-9) + 1e-12;
                const double l = ceil((c3v[a] - ea - m.o[a]) / m.h[a]) - 1, u = floor((c3v[a] + ea - m.o[a]) / m.h[a]) + 1;
                p.vlo[a] = (int32_t)dmin(dmax(l, -1.0), (double)n3v(m, a) + 1);
                p.vhi[a] = (int32_t)dmin(dmax(u, -1.0), (double)n3v(m, a) + 1);
            }
        }
        const double c3[3] = {cw.x, cw.y, cw.z};
        for (int a = 0; a < 3; ++a) {
            if (k.shape.prism && a == 2) { p.lo[2] = 0; continue; }
            if (k.ext[a] >= n[a] + 2) { p.lo[a] = -1; continue; }  // the window spans the whole axis
            const double lo = floor((c3[a] - rad[a] - m.o[a]) / m.h[a]) - 1;
            const double hi = floor((c3[a] + rad[a] - m.o[a]) / m.h[a]) + 1;
            // only cells 0..n-1 matter: start the window no lower than -1 (this also keeps the int conversion
            // defined for solids far outside the mesh)
            const double lo_c = dmin(dmax(lo, -1.0), 1e9), hi_c = dmin(hi, (double)n[a]);
            p.lo[a] = (int32_t)lo_c;
            if (hi_c >= lo_c && hi_c - lo_c + 1 > (double)k.ext[a]) p.err = DERR_BBOX;
        }
    }
    if (p.err) set_error(cnt, p.err);
    // meshSearch::findNearestCell: nearest cell centre, ties to the lowest cell label
    {
        const double pc[3] = {x.x, x.y, x.z};
        int64_t lo[3], hi[3];
        for (int a = 0; a < 3; ++a) {
            double t = floor((pc[a] - m.o[a]) / m.h[a]);
            int64_t e = t < 0 ? 0 : (t > (double)(n[a] - 1) ? n[a] - 1 : (int64_t)t);
            lo[a] = e > 0 ? e - 1 : 0;
            hi[a] = e + 1 < n[a] ? e + 1 : n[a] - 1;
        }
        int64_t best = -1;
        double bd = 0;
        for (int64_t kk = lo[2]; kk <= hi[2]; ++kk)
            for (int64_t jj = lo[1]; jj <= hi[1]; ++jj)
                for (int64_t ii = lo[0]; ii <= hi[0]; ++ii) {
                    const int64_t c = ii + (int64_t)m.nx * (jj + (int64_t)m.ny * kk);
                    const double d = magSqr(mesh_C(m, ii, jj, kk) - x);
                    if (best < 0 || d < bd || (d == bd && c < best)) { bd = d; best = c; }
                }
        p.seed = best;
        const int64_t si = best % m.nx, sj = (best / m.nx) % m.ny, sk3 = best / ((int64_t)m.nx * m.ny);
        p.seed_ijk[0] = (int32_t)si; p.seed_ijk[1] = (int32_t)sj; p.seed_ijk[2] = (int32_t)sk3;
        p.pad1 = 0;
        const D3 cb = mesh_C(m, si, sj, sk3) - x;
        p.cbase[0] = cb.x; p.cbase[1] = cb.y; p.cbase[2] = cb.z;
        // us at a cell (i, j, k) = us0 + omega x ((i, j, k) - seed) h: us0 and the six per-step terms, split into
        // FP32 pairs (the couple kernel evaluates U - us in two-float arithmetic)
        const D3 vel{st[s].vel[0], st[s].vel[1], st[s].vel[2]}, om{st[s].omega[0], st[s].omega[1], st[s].omega[2]};
        const D3 us0 = vel + cross(om, cb);
        const double u3[3] = {us0.x, us0.y, us0.z};
        const double d6[6] = {-om.z * m.h[1], om.y * m.h[2], om.z * m.h[0], -om.x * m.h[2], -om.y * m.h[0],
                              om.x * m.h[1]};
        for (int a = 0; a < 3; ++a) {
            p.us_hi[a] = (float)u3[a];
            p.us_lo[a] = (float)(u3[a] - (double)p.us_hi[a]);
            p.cb32[a] = (float)p.cbase[a];
        }
        for (int r = 0; r < 6; ++r) {
            p.ds_hi[r] = (float)d6[r];
            p.ds_lo[r] = (float)(d6[r] - (double)p.ds_hi[r]);
        }
    }
    // FP64 origin of the tile frames and the local map (world2local of the bbox corner plus the images of the cell
    // edge vectors), so tiles build their frames without per-tile FP64 work
    {
        const D3 p0 = mesh_point(m, p.lo[0], p.lo[1], p.lo[2]);
        const D3 b = p0 - x;
        p.base[0] = b.x; p.base[1] = b.y; p.base[2] = b.z;
        p.base32[0] = (float)b.x; p.base32[1] = (float)b.y; p.base32[2] = (float)b.z;
        p.pad4 = 0.f;
        const D3 cl = world2local(p0, x, q);
        const Q4 qc = qconj(q);
        const D3 lx = qtransform(qc, D3{m.h[0], 0, 0}), ly = qtransform(qc, D3{0, m.h[1], 0}),
                 lz = qtransform(qc, D3{0, 0, m.h[2]});
        const double l12[12] = {cl.x, cl.y, cl.z, lx.x, lx.y, lx.z, ly.x, ly.y, ly.z, lz.x, lz.y, lz.z};
        for (int r = 0; r < 12; ++r) {
            p.lmap[r] = l12[r];
            p.lmap_hi[r] = (float)l12[r];
            p.lmap_lo[r] = (float)(l12[r] - (double)p.lmap_hi[r]);
        }
        const D3 pf = mesh_point(m, (int64_t)p.lo[0] + k.ext[0], (int64_t)p.lo[1] + k.ext[1], (int64_t)p.lo[2] + k.ext[2]);
        p.e64 = (float)(2e-15 * (fabs(p0.x) + fabs(p0.y) + fabs(p0.z) + fabs(pf.x) + fabs(pf.y) + fabs(pf.z) + fabs(x.x) +
                                 fabs(x.y) + fabs(x.z)));
        p.pad2 = 0.f;
    }
    p.min_cand = ~0ull;
    p.n_inside = p.n_cut = 0;
    plan[s] = p;
}

// ---- claims ----------------------------------------------------------------------------------------------------------
// Ct during a call holds claim words CT_KEY_BASE | (solid << 2 | type); CT_SHARED is set once a second solid touches
// the cell and the low bits then keep the largest claim (the last solid of the reference's serial loop).  Any value
// below CT_KEY_BASE -- zero, or the decoded Ct a previous call left -- is an unclaimed cell.
// One atomicMax claims the cell (any previous value is below every claim word); seeing another claim of this call
// in its return value, the claimer raises the word to the larger claim with CT_SHARED set.
__device__ inline bool claim_cell(int32_t* Ct, int32_t cell, int32_t s, int type) {
    uint32_t* C = reinterpret_cast<uint32_t*>(Ct) + cell;
    const uint32_t key = CT_KEY_BASE | ((uint32_t)s << 2) | (uint32_t)type;
    const uint32_t old = atomicMax(C, key);
    if (old < CT_KEY_BASE) return false;
    atomicMax(C, max(key, old & ~CT_SHARED) | CT_SHARED);
    return true;
}

// set bit (c >> 3) of a chunk bitmap (one bit per 8 consecutive cells)
__device__ inline void mark_chunk(uint32_t* bits, int64_t c) {
    uint32_t* w = bits + (c >> 8);
    const uint32_t b = 1u << ((c >> 3) & 31);
    if (!(*w & b)) atomicOr(w, b);
}

// claim pass over this call's lists; marks the chunks of the claimed cells in cbits and, for a cell claimed more than
// once, in sbits (every claimer after the first sees an earlier claim, so each shared cell's chunk is marked)
__global__ void claim_kernel(const int32_t* __restrict__ in_cell, const int32_t* __restrict__ in_solid,
                             const int32_t* __restrict__ cut_cell, const int32_t* __restrict__ cut_solid,
                             int32_t* __restrict__ Ct, Counters* cnt, int64_t N, uint32_t* __restrict__ cbits,
                             uint32_t* __restrict__ sbits) {
    const int n_in = clamp_len(cnt->n_inside, cnt->list_cap), n_cut = clamp_len(cnt->n_cut, cnt->list_cap);
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < (int64_t)n_in + n_cut;
         e += (int64_t)gridDim.x * blockDim.x) {
        const bool cut = e >= n_in;
        const int64_t ee = cut ? e - n_in : e;
        const int32_t c = cut ? cut_cell[ee] : in_cell[ee];
        const int32_t sw = cut ? cut_solid[ee] : in_solid[ee];
        if (c < 0 || c >= N) continue;
        const bool shared = claim_cell(Ct, c, sw & LIST_SOLID_MASK, list_type(sw));
        if (cbits) {
            mark_chunk(cbits, c);
            if (shared) {
                mark_chunk(sbits, c);
                atomicAdd(&cnt->shared_marks, 1);
            }
        }
    }
}

__device__ inline int32_t decode_claim(uint32_t w) {
    const uint32_t k = (w & ~CT_SHARED) - CT_KEY_BASE;
    const int32_t s = (int32_t)(k >> 2), code = (int32_t)(k & 3);
    return code == 1 ? s + 4 : code;
}

// ---- connect: bit-parallel flood fill --------------------------------------------------------------------------------
constexpr int CON_THREADS = 512;

// fill upward (towards higher bits) inside runs of c starting from seeds s (s subset of c)
__device__ inline uint32_t fill_up(uint32_t c, uint32_t s) { return (((c + s) ^ c) & c) | s; }
__device__ inline uint32_t fill_down(uint32_t c, uint32_t s) { return __brev(fill_up(__brev(c), __brev(s))); }

__device__ inline int block_excl_scan(int v, int* warp_sums, int& total) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_sums[wid] = x;
    __syncthreads();
    if (wid == 0) {
        int w = lane < nw ? warp_sums[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        if (lane < nw) warp_sums[lane] = w;  // inclusive
    }
    __syncthreads();
    total = warp_sums[nw - 1];
    const int before = (wid > 0 ? warp_sums[wid - 1] : 0) + x - v;
    __syncthreads();
    return before;
}

// local cell index of the flood-fill seed: the nearest cell when it has an inside vertex, else the lowest-label cell
// that has one (the seed fallback scan of cellenumerator.cpp:52-63); -1 when the solid touches no cell
__device__ inline int seed_local(const MeshK& m, const SolidPlan& pl, const uint8_t* cls, int ex, int ey, int ez) {
    int sl = -1;
    const int64_t seed = pl.seed;
    const int64_t si = seed % m.nx, sj = (seed / m.nx) % m.ny, sk2 = seed / ((int64_t)m.nx * m.ny);
    const int64_t a = si - pl.lo[0], b = sj - pl.lo[1], c = sk2 - pl.lo[2];
    if (a >= 0 && b >= 0 && c >= 0 && a < ex && b < ey && c < ez) {
        const int li = (int)(a + (int64_t)ex * (b + (int64_t)ey * c));
        if (cls[li]) sl = li;
    }
    if (sl < 0 && pl.min_cand != ~0ull) {
        const int64_t g = (int64_t)pl.min_cand;
        const int64_t gi = g % m.nx, gj = (g / m.nx) % m.ny, gk = g / ((int64_t)m.nx * m.ny);
        sl = (int)((gi - pl.lo[0]) + (int64_t)ex * ((gj - pl.lo[1]) + (int64_t)ey * (gk - pl.lo[2])));
    }
    if (sl >= ex * ey * ez) sl = -1;
    return sl;
}

__global__ void __launch_bounds__(CON_THREADS, 2) connect_kernel(MeshK m, const SolidK* __restrict__ sk,
                                                              SolidPlan* __restrict__ plan,
                                                              const uint8_t* __restrict__ scratch,
                                                              uint32_t* __restrict__ gbitmaps,
                                                              int32_t* __restrict__ in_cell, int32_t* __restrict__ in_solid,
                                                              int32_t* __restrict__ cut_cell, int32_t* __restrict__ cut_solid,
                                                              int64_t cap_in, int64_t cap_cut, Counters* cnt,
                                                              int smem_words, const int32_t* __restrict__ solids) {
    extern __shared__ uint32_t dsm[];
    __shared__ int s_seed;  // local cell index of the seed, -1: none
    __shared__ int warp_sums[32];
    __shared__ int s_base_in, s_base_cut;
    const int s = solids ? solids[blockIdx.x] : blockIdx.x;
    const int tid = threadIdx.x;
    const SolidK& k = sk[s];
    SolidPlan& pl = plan[s];
    const int ex = k.ext[0], ey = k.ext[1], ez = k.ext[2];
    const int W = (ex + 31) >> 5;
    const int rows = ey * ez;
    const int nwords = rows * W;
    uint32_t* C = k.bitmap_global ? gbitmaps + k.bitmap_off : dsm;  // candidates (class != 0)
    uint32_t* R = C + nwords;                                        // reached
    uint32_t* I = R + nwords;                                        // class 1 (all inside)
    uint32_t* T = I + nwords;                                        // class 2 (centre inside)
    const uint8_t* cls = scratch + k.scratch_off;
    if (pl.err) {
        if (tid == 0) { pl.n_inside = 0; pl.n_cut = 0; }
        return;
    }
    // seed: nearest cell when it has an inside vertex, else the lowest-label cell that has one
    if (tid == 0) {
        s_seed = seed_local(m, pl, cls, ex, ey, ez);
    }
    __syncthreads();
    if (s_seed < 0) {
        if (tid == 0) { pl.n_inside = 0; pl.n_cut = 0; }
        return;
    }
    // the bitmaps from the class bytes: a warp per group of 16 words (16 independent loads in flight per lane),
    // each word one coalesced 32-byte load and three ballots (the emission below then reads no class byte again)
    {
        const int lane = tid & 31;
        constexpr int GW = 16;
        for (int w0 = (tid >> 5) * GW; w0 < nwords; w0 += CON_THREADS / 32 * GW) {
            uint8_t v[GW];
#pragma unroll
            for (int u = 0; u < GW; ++u) {
                const int w = w0 + u;
                const int row = w / W, xx = ((w - row * W) << 5) + lane;
                v[u] = (w < nwords && xx < ex) ? cls[(int64_t)row * ex + xx] : (uint8_t)0;
            }
#pragma unroll
            for (int u = 0; u < GW; ++u) {
                const uint32_t bc = __ballot_sync(0xffffffffu, v[u] != 0), bi = __ballot_sync(0xffffffffu, v[u] == 1),
                               bt = __ballot_sync(0xffffffffu, v[u] == 2);
                if (lane == 0 && w0 + u < nwords) {
                    C[w0 + u] = bc;
                    I[w0 + u] = bi;
                    T[w0 + u] = bt;
                    R[w0 + u] = 0;
                }
            }
        }
    }
    __syncthreads();
    if (tid == 0) {
        const int sx = s_seed % ex, srow = s_seed / ex;
        R[srow * W + (sx >> 5)] |= 1u << (sx & 31);
    }
    __syncthreads();
    // directional sweeps until nothing changes
    const int max_rounds = 8 + 2 * (ex + ey + ez);
    int round = 0;
    for (;; ++round) {
        int changed = 0;
        // x: carry fill along each row
        for (int row = tid; row < rows; row += CON_THREADS) {
            uint32_t* r = R + row * W;
            const uint32_t* c = C + row * W;
            uint32_t carry = 0;
            for (int w = 0; w < W; ++w) {
                const uint32_t seeds = (r[w] | (carry & 1u)) & c[w];
                const uint32_t f = fill_up(c[w], seeds);
                if (f != r[w]) { changed = 1; r[w] = f; }
                carry = f >> 31;
            }
            carry = 0;
            for (int w = W - 1; w >= 0; --w) {
                const uint32_t seeds = (r[w] | (carry << 31)) & c[w];
                const uint32_t f = fill_down(c[w], seeds);
                if (f != r[w]) { changed = 1; r[w] = f; }
                carry = f & 1u;
            }
        }
        __syncthreads();
        // y: forward and backward scans along j for every (k, word)
        for (int col = tid; col < ez * W; col += CON_THREADS) {
            const int kk = col / W, w = col - kk * W;
            uint32_t* r = R + (kk * ey) * W + w;
            const uint32_t* c = C + (kk * ey) * W + w;
            // the running value stays in a register: the loads of r and c do not depend on the previous step
            uint32_t prev = r[0];
            for (int j = 1; j < ey; ++j) {
                const uint32_t cur = r[j * W], f = cur | (prev & c[j * W]);
                if (f != cur) { changed = 1; r[j * W] = f; }
                prev = f;
            }
            for (int j = ey - 2; j >= 0; --j) {
                const uint32_t cur = r[j * W], f = cur | (prev & c[j * W]);
                if (f != cur) { changed = 1; r[j * W] = f; }
                prev = f;
            }
        }
        __syncthreads();
        // z: forward and backward scans along k for every (j, word)
        if (ez > 1) {
            for (int col = tid; col < ey * W; col += CON_THREADS) {
                const int jj = col / W, w = col - jj * W;
                uint32_t* r = R + jj * W + w;
                const uint32_t* c = C + jj * W + w;
                const int stride = ey * W;
                uint32_t prev = r[0];
                for (int kk = 1; kk < ez; ++kk) {
                    const uint32_t cur = r[kk * stride], f = cur | (prev & c[kk * stride]);
                    if (f != cur) { changed = 1; r[kk * stride] = f; }
                    prev = f;
                }
                for (int kk = ez - 2; kk >= 0; --kk) {
                    const uint32_t cur = r[kk * stride], f = cur | (prev & c[kk * stride]);
                    if (f != cur) { changed = 1; r[kk * stride] = f; }
                    prev = f;
                }
            }
        }
        changed = __syncthreads_or(changed);
        if (!changed) break;
        if (round >= max_rounds) {
            if (tid == 0) set_error(cnt, DERR_FLOOD_LIMIT);
            break;
        }
    }
    // emit the reached cells in ascending label order: thread t owns rows [t*rpt, (t+1)*rpt)
    const int rpt = (rows + CON_THREADS - 1) / CON_THREADS;
    const int r0 = min(rows, tid * rpt), r1 = min(rows, r0 + rpt);
    int nin = 0, ncut = 0;
    for (int row = r0; row < r1; ++row)
        for (int w = 0; w < W; ++w) {
            const uint32_t bits = R[row * W + w], in = I[row * W + w];
            nin += __popc(bits & in);
            ncut += __popc(bits & ~in);
        }
    int tot_in, tot_cut;
    const int off_in = block_excl_scan(nin, warp_sums, tot_in);
    const int off_cut = block_excl_scan(ncut, warp_sums, tot_cut);
    if (tid == 0) {
        s_base_in = atomicAdd(&cnt->n_inside, tot_in);
        s_base_cut = atomicAdd(&cnt->n_cut, tot_cut);
        pl.n_inside = tot_in;
        pl.n_cut = tot_cut;
    }
    __syncthreads();
    const int64_t bin = s_base_in, bcut = s_base_cut;
    if (bin + tot_in > cap_in || bcut + tot_cut > cap_cut) {
        if (tid == 0) set_error(cnt, DERR_CAPACITY);
        return;
    }
    int64_t pin = bin + off_in, pcut = bcut + off_cut;
    for (int row = r0; row < r1; ++row) {
        const int jj = row % ey, kk = row / ey;
        for (int w = 0; w < W; ++w) {
            uint32_t bits = R[row * W + w];
            const uint32_t in = I[row * W + w], ci = T[row * W + w];
            while (bits) {
                const int b = __ffs(bits) - 1;
                bits &= bits - 1;
                const int xx = (w << 5) + b;
                const uint8_t cc = ((in >> b) & 1u) ? 1 : (((ci >> b) & 1u) ? 2 : 3);
                const int64_t gi = pl.lo[0] + xx, gj = pl.lo[1] + jj, gk = pl.lo[2] + kk;
                const int32_t cell = (int32_t)(gi + (int64_t)m.nx * (gj + (int64_t)m.ny * gk));
                if (cc == 1) { in_cell[pin] = cell; in_solid[pin] = list_word(s, 1); ++pin; }
                else { cut_cell[pcut] = cell; cut_solid[pcut] = list_word(s, cc); ++pcut; }
            }
        }
    }
}

// The same connected component for solids whose bbox bitmap has at most CON_SMALL_WORDS words: one warp per solid,
// eight solids per CTA, bitmaps in shared memory, warp-synchronous sweeps.
constexpr int CON_SMALL_WORDS = 256;
constexpr int CON_SMALL_WARPS = 8;

__global__ void __launch_bounds__(CON_SMALL_WARPS * 32) connect_small_kernel(
    MeshK m, const SolidK* __restrict__ sk, SolidPlan* __restrict__ plan, const uint8_t* __restrict__ scratch,
    int32_t* __restrict__ in_cell, int32_t* __restrict__ in_solid, int32_t* __restrict__ cut_cell,
    int32_t* __restrict__ cut_solid, int64_t cap_in, int64_t cap_cut, Counters* cnt, const int32_t* __restrict__ solids,
    int nsolids) {
    __shared__ uint32_t s_bits[CON_SMALL_WARPS][2 * CON_SMALL_WORDS];
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int item = blockIdx.x * CON_SMALL_WARPS + wid;
    if (item >= nsolids) return;
    const int s = solids[item];
    const SolidK& k = sk[s];
    SolidPlan& pl = plan[s];
    const int ex = k.ext[0], ey = k.ext[1], ez = k.ext[2];
    const int W = (ex + 31) >> 5;
    const int rows = ey * ez;
    const int nwords = rows * W;
    uint32_t* C = s_bits[wid];
    uint32_t* R = C + CON_SMALL_WORDS;
    const uint8_t* cls = scratch + k.scratch_off;
    if (pl.err) {
        if (lane == 0) { pl.n_inside = 0; pl.n_cut = 0; }
        return;
    }
    int sl = 0;
    if (lane == 0) sl = seed_local(m, pl, cls, ex, ey, ez);
    sl = __shfl_sync(FULL, sl, 0);
    if (sl < 0) {
        if (lane == 0) { pl.n_inside = 0; pl.n_cut = 0; }
        return;
    }
    for (int w = lane; w < nwords; w += 32) {
        const int row = w / W, wi = w - row * W;
        const uint8_t* rp = cls + (int64_t)row * ex;
        uint32_t bits = 0;
        const int x0 = wi << 5, x1 = min(ex, x0 + 32);
        for (int xx = x0; xx < x1; ++xx) bits |= (rp[xx] ? 1u : 0u) << (xx - x0);
        C[w] = bits;
        R[w] = 0;
    }
    __syncwarp();
    if (lane == 0) {
        const int sx = sl % ex, srow = sl / ex;
        R[srow * W + (sx >> 5)] |= 1u << (sx & 31);
    }
    __syncwarp();
    const int max_rounds = 8 + 2 * (ex + ey + ez);
    for (int round = 0;; ++round) {
        int changed = 0;
        for (int row = lane; row < rows; row += 32) {
            uint32_t* r = R + row * W;
            const uint32_t* c = C + row * W;
            uint32_t carry = 0;
            for (int w = 0; w < W; ++w) {
                const uint32_t seeds = (r[w] | (carry & 1u)) & c[w];
                const uint32_t f = fill_up(c[w], seeds);
                if (f != r[w]) { changed = 1; r[w] = f; }
                carry = f >> 31;
            }
            carry = 0;
            for (int w = W - 1; w >= 0; --w) {
                const uint32_t seeds = (r[w] | (carry << 31)) & c[w];
                const uint32_t f = fill_down(c[w], seeds);
                if (f != r[w]) { changed = 1; r[w] = f; }
                carry = f & 1u;
            }
        }
        __syncwarp();
        for (int col = lane; col < ez * W; col += 32) {
            const int kk = col / W, w = col - kk * W;
            uint32_t* r = R + (kk * ey) * W + w;
            const uint32_t* c = C + (kk * ey) * W + w;
            // the running value stays in a register: the loads of r and c do not depend on the previous step
            uint32_t prev = r[0];
            for (int j = 1; j < ey; ++j) {
                const uint32_t cur = r[j * W], f = cur | (prev & c[j * W]);
                if (f != cur) { changed = 1; r[j * W] = f; }
                prev = f;
            }
            for (int j = ey - 2; j >= 0; --j) {
                const uint32_t cur = r[j * W], f = cur | (prev & c[j * W]);
                if (f != cur) { changed = 1; r[j * W] = f; }
                prev = f;
            }
        }
        __syncwarp();
        if (ez > 1) {
            for (int col = lane; col < ey * W; col += 32) {
                const int jj = col / W, w = col - jj * W;
                uint32_t* r = R + jj * W + w;
                const uint32_t* c = C + jj * W + w;
                const int stride = ey * W;
                uint32_t prev = r[0];
                for (int kk = 1; kk < ez; ++kk) {
                    const uint32_t cur = r[kk * stride], f = cur | (prev & c[kk * stride]);
                    if (f != cur) { changed = 1; r[kk * stride] = f; }
                    prev = f;
                }
                for (int kk = ez - 2; kk >= 0; --kk) {
                    const uint32_t cur = r[kk * stride], f = cur | (prev & c[kk * stride]);
                    if (f != cur) { changed = 1; r[kk * stride] = f; }
                    prev = f;
                }
            }
        }
        __syncwarp();
        if (!__any_sync(FULL, changed)) break;
        if (round >= max_rounds) {
            if (lane == 0) set_error(cnt, DERR_FLOOD_LIMIT);
            break;
        }
    }
    // emit in ascending label order: lane t owns rows [t*rpt, (t+1)*rpt)
    const int rpt = (rows + 31) / 32;
    const int r0 = min(rows, lane * rpt), r1 = min(rows, r0 + rpt);
    int nin = 0, ncut = 0;
    for (int row = r0; row < r1; ++row)
        for (int w = 0; w < W; ++w) {
            uint32_t bits = R[row * W + w];
            while (bits) {
                const int b = __ffs(bits) - 1;
                bits &= bits - 1;
                if (cls[(int64_t)row * ex + (w << 5) + b] == 1) ++nin; else ++ncut;
            }
        }
    int xin = nin, xcut = ncut;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int a = __shfl_up_sync(FULL, xin, o), b = __shfl_up_sync(FULL, xcut, o);
        if (lane >= o) { xin += a; xcut += b; }
    }
    const int tot_in = __shfl_sync(FULL, xin, 31), tot_cut = __shfl_sync(FULL, xcut, 31);
    int bin = 0, bcut = 0;
    if (lane == 0) {
        bin = atomicAdd(&cnt->n_inside, tot_in);
        bcut = atomicAdd(&cnt->n_cut, tot_cut);
        pl.n_inside = tot_in;
        pl.n_cut = tot_cut;
    }
    bin = __shfl_sync(FULL, bin, 0);
    bcut = __shfl_sync(FULL, bcut, 0);
    if ((int64_t)bin + tot_in > cap_in || (int64_t)bcut + tot_cut > cap_cut) {
        if (lane == 0) set_error(cnt, DERR_CAPACITY);
        return;
    }
    int64_t pin = (int64_t)bin + xin - nin, pcut = (int64_t)bcut + xcut - ncut;
    for (int row = r0; row < r1; ++row) {
        const int jj = row % ey, kk = row / ey;
        for (int w = 0; w < W; ++w) {
            uint32_t bits = R[row * W + w];
            while (bits) {
                const int b = __ffs(bits) - 1;
                bits &= bits - 1;
                const int xx = (w << 5) + b;
                const uint8_t cc = cls[(int64_t)row * ex + xx];
                const int64_t gi = pl.lo[0] + xx, gj = pl.lo[1] + jj, gk = pl.lo[2] + kk;
                const int32_t cell = (int32_t)(gi + (int64_t)m.nx * (gj + (int64_t)m.ny * gk));
                if (cc == 1) { in_cell[pin] = cell; in_solid[pin] = list_word(s, 1); ++pin; }
                else { cut_cell[pcut] = cell; cut_solid[pcut] = list_word(s, cc); ++pcut; }
            }
        }
    }
}

// ---- shared cells -----------------------------------------------------------------------------------------------------
// slot of cell c in the shared table, inserting it on first use; -1 (and an error flag) when the table is full
__device__ inline int shared_slot(const CoupleArgs& A, int32_t c) {
    uint32_t h = ((uint32_t)c * 2654435761u) & (uint32_t)A.sh_mask;
    for (int p = 0; p < SHARED_MAX_PROBES; ++p) {
        const int32_t k = atomicCAS(A.sh_keys + h, -1, c);
        if (k == -1) {
            const int u = atomicAdd(&A.cnt->n_shared, 1);
            if (u <= A.sh_mask) A.sh_used[u] = (int32_t)h;
            return (int)h;
        }
        if (k == c) return (int)h;
        h = (h + 1) & (uint32_t)A.sh_mask;
    }
    set_error(A.cnt, DERR_SHARED_TABLE);
    return -1;
}

// ---- couple ---------------------------------------------------------------------------------------------------------
constexpr int CPL_THREADS = 256;



// Reduce-scatter of 8 values over the warp in three xor steps: afterwards each lane holds slot (lane >> 2) & 7 summed
// over the 8 lanes that share its bits 0..1; warp_total4 then adds the 4 lanes that differ in those bits.
template <typename T>
__device__ __forceinline__ T reduce_scatter8(T* v, int lane) {
    {
        const bool up = (lane & 16) != 0;
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const T send = up ? v[i] : v[i + 4];
            const T keep = up ? v[i + 4] : v[i];
            v[i] = keep + __shfl_xor_sync(0xffffffffu, send, 16);
        }
    }
    {
        const bool up = (lane & 8) != 0;
#pragma unroll
        for (int i = 0; i < 2; ++i) {
            const T send = up ? v[i] : v[i + 2];
            const T keep = up ? v[i + 2] : v[i];
            v[i] = keep + __shfl_xor_sync(0xffffffffu, send, 8);
        }
    }
    const bool up = (lane & 4) != 0;
    const T send = up ? v[0] : v[1];
    const T keep = up ? v[1] : v[0];
    return keep + __shfl_xor_sync(0xffffffffu, send, 4);
}
// sum over the 4 lanes that differ in bits 0..1 (FP64)
__device__ __forceinline__ double warp_total4(double x) {
    x += __shfl_xor_sync(0xffffffffu, x, 2);
    x += __shfl_xor_sync(0xffffffffu, x, 1);
    return x;
}

// Two-float arithmetic (Dekker / Knuth): a + b = s + e and a * b = p + e exactly, with explicit rounding intrinsics
// so that nothing is contracted or reassociated.
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
    s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}
// U - (u0 + a p + b q) with u0, p, q given as FP32 pairs hi + lo and a, b small integers, rounded once to FP32 after
// an error of about 2^-46 of the magnitudes
__device__ __forceinline__ float ff_u_minus_us(float U, float u0h, float u0l, float a, float ph, float pl, float b,
                                               float qh, float ql) {
    const float t1 = __fmul_rn(a, ph), e1 = __fmaf_rn(a, ph, -t1);
    const float t2 = __fmul_rn(b, qh), e2 = __fmaf_rn(b, qh, -t2);
    float s1, f1, s2, f2;
    two_sum(u0h, t1, s1, f1);
    two_sum(s1, t2, s2, f2);
    const float lo = __fadd_rn(__fadd_rn(__fadd_rn(u0l, __fadd_rn(e1, e2)), __fadd_rn(f1, f2)),
                               __fmaf_rn(a, pl, __fmul_rn(b, ql)));
    float d, g;
    two_sum(U, -s2, d, g);
    return __fadd_rn(d, __fsub_rn(g, lo));
}

// Per-cell forcing of solid s on cell c with fluid velocity U (pcHydrodynamicInteraction, solidcloud.cpp:384-390):
// alpha, the FP32 Fs and the cell's contributions to the force/torque sums (:411-421), FP64 in f6 (exact mode) or
// FP32 in g6.
__device__ __forceinline__ float cell_forcing(const CoupleArgs& A, int64_t c, int s, int type, float dtINV32,
                                              double dtINV, float fs[3], double f6[8], float g6[8], float Ux,
                                              float Uy, float Uz) {
    const MeshK& m = A.m;
    int i, j, k;
    cell_ijk(m, c, i, j, k);
    float alpha = 1.f;
    if (type != 1) {
        // computed by the fraction pass for every cut candidate of the solid's bbox
        const SolidK& ks = A.sk[s];
        const int32_t* lo = A.plan[s].lo;
        const int64_t li = (i - lo[0]) + (int64_t)ks.ext[0] * ((j - lo[1]) + (int64_t)ks.ext[1] * (k - lo[2]));
        alpha = A.alpha[ks.scratch_off + li];
        // a SUBSAMPLE count whose undecided points were rechecked on full warps
        if (alpha < 0.f) alpha = __fdiv_rn(-alpha - 1.f, (float)A.count_samples);
    }
    if (A.exact_forcing) {
        // the reference's FP64 sequence
        const sdfibm_solid_state& st = A.st[s];
        const D3 x = state_pos(st);
        const D3 cc = mesh_C(m, i, j, k);
        const D3 vel{st.vel[0], st.vel[1], st.vel[2]}, om{st.omega[0], st.omega[1], st.omega[2]};
        const D3 uf{(double)Ux, (double)Uy, (double)Uz};
        const D3 us = vel + cross(om, cc - x);
        const D3 f_ = (double)alpha * (uf - us);
        const D3 t_ = cross(cc - x, f_);
        f6[0] = f_.x; f6[1] = f_.y; f6[2] = f_.z; f6[3] = t_.x; f6[4] = t_.y; f6[5] = t_.z;
        fs[0] = (float)(f_.x * dtINV); fs[1] = (float)(f_.y * dtINV); fs[2] = (float)(f_.z * dtINV);
    } else {
        // U - us in two-float arithmetic (the difference can cancel; about 2^-46 of the magnitudes, against 2^-24 of
        // the difference for the FP32 rounding that follows), FP32 after it.  The cell offsets from the seed are
        // exact small integers.
        const SolidPlan& pl = A.plan[s];
        const float di = (float)(i - pl.seed_ijk[0]), dj = (float)(j - pl.seed_ijk[1]), dk = (float)(k - pl.seed_ijk[2]);
        const float fx = alpha * ff_u_minus_us(Ux, pl.us_hi[0], pl.us_lo[0], dj, pl.ds_hi[0], pl.ds_lo[0], dk,
                                               pl.ds_hi[1], pl.ds_lo[1]);
        const float fy = alpha * ff_u_minus_us(Uy, pl.us_hi[1], pl.us_lo[1], di, pl.ds_hi[2], pl.ds_lo[2], dk,
                                               pl.ds_hi[3], pl.ds_lo[3]);
        const float fz = alpha * ff_u_minus_us(Uz, pl.us_hi[2], pl.us_lo[2], di, pl.ds_hi[4], pl.ds_lo[4], dj,
                                               pl.ds_hi[5], pl.ds_lo[5]);
        const float dx = __fmaf_rn(di, m.h32[0], pl.cb32[0]), dy = __fmaf_rn(dj, m.h32[1], pl.cb32[1]),
                    dz = __fmaf_rn(dk, m.h32[2], pl.cb32[2]);
        g6[0] = fx; g6[1] = fy; g6[2] = fz;
        g6[3] = dy * fz - dz * fy; g6[4] = dz * fx - dx * fz; g6[5] = dx * fy - dy * fx;
        fs[0] = fx * dtINV32; fs[1] = fy * dtINV32; fs[2] = fz * dtINV32;
    }
    return alpha;
}

// The cell's FP64 sums in the shared table (As, Ts, Fs of every solid on a cell several solids touch).
__device__ __forceinline__ void add_shared(const CoupleArgs& A, int64_t c, float alpha, const float fs[3]) {
    const int slot = shared_slot(A, (int32_t)c);
    if (slot >= 0) {
        double* v = A.sh_vals + 5 * (int64_t)slot;
        atomicAdd(v + 0, (double)alpha);
        atomicAdd(v + 1, (double)alpha);
        atomicAdd(v + 2, (double)fs[0]);
        atomicAdd(v + 3, (double)fs[1]);
        atomicAdd(v + 4, (double)fs[2]);
    }
}

// Shared pass of the coupling, first half (on the side stream after the claims, beside the fraction kernels): the list
// entries on cells that several solids claimed, compacted into shent (entry index into the in list then the cut list).
// Only the chunks marked in sbits are looked at; the kernel returns at once when no cell was claimed twice.
__global__ void shared_scan_kernel(const int32_t* __restrict__ in_cell, const int32_t* __restrict__ cut_cell,
                                   const int32_t* __restrict__ Ct, Counters* cnt, int64_t N,
                                   const uint32_t* __restrict__ sbits, uint32_t* __restrict__ shent,
                                   int64_t shent_cap) {
    if (cnt->shared_marks == 0) return;
    const int64_t n_in = clamp_len(cnt->n_inside, cnt->list_cap), n_cut = clamp_len(cnt->n_cut, cnt->list_cap);
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n_in + n_cut;
         e += (int64_t)gridDim.x * blockDim.x) {
        const int32_t c = e < n_in ? in_cell[e] : cut_cell[e - n_in];
        if (c < 0 || c >= N) continue;
        if (!((sbits[c >> 8] >> ((c >> 3) & 31)) & 1u)) continue;  // no cell of this chunk is shared
        if (!(reinterpret_cast<const uint32_t*>(Ct)[c] & CT_SHARED)) continue;
        const int32_t slot = atomicAdd(&cnt->n_shent, 1);
        if (slot < shent_cap) shent[slot] = (uint32_t)e;
        else set_error(cnt, DERR_SHARED_TABLE);
    }
}

// Shared pass, second half (after the fraction kernels): every compacted entry adds its solid's As / Ts / Fs to the
// cell's FP64 sums in the shared table (finalize_kernel writes them) and its force/torque contribution to the solid's
// sums.
__global__ void __launch_bounds__(CPL_THREADS) couple_shared_kernel(CoupleArgs A) {
    const int64_t N = A.m.ncells;
    const int64_t n = min((int64_t)A.cnt->n_shent, A.shent_cap);
    if (n == 0) return;
    const int64_t n_in = clamp_len(A.cnt->n_inside, A.cnt->list_cap);
    const double dtINV = A.step->dtINV;
    const float dtINV32 = (float)dtINV;
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x) {
        const int64_t e = A.shent[q];
        const bool is_cut = e >= n_in;
        const int32_t c = is_cut ? A.cut_cell[e - n_in] : A.in_cell[e];
        const int32_t sw = is_cut ? A.cut_solid[e - n_in] : A.in_solid[e];
        const int s = sw & LIST_SOLID_MASK;
        double f6[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        float g6[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
        float fs[3];
        const float alpha = cell_forcing(A, c, s, list_type(sw), dtINV32, dtINV, fs, f6, g6, A.U[c], A.U[N + c],
                                         A.U[2 * N + c]);
        add_shared(A, c, alpha, fs);
        for (int r = 0; r < 6; ++r) atomicAdd(A.ftacc + 6 * s + r, A.exact_forcing ? f6[r] : (double)g6[r]);
    }
}

// Chunked coupling.  The claim pass marks in cbits every chunk of 8 consecutive cells that holds a claimed cell (and
// in sbits the chunks of cells claimed more than once).  This kernel runs over the marked chunks in memory order, a
// warp per bitmap word (256 cells), four chunks at a time with 8 lanes each, and writes the four fields of every
// cell of a marked chunk: zero for an unclaimed cell (a cell that no solid touches, or one the previous call touched:
// the sparse reset inside these chunks), zero As / Ts / Fs and the claim word kept in Ct for a shared cell
// (finalize_kernel writes its sums and decodes its Ct), and for a cell claimed once the forcing of its solid.  The
// cells claimed once are queued per warp in shared memory and computed 32 at a time on full warps; their values
// land in the same sectors a few instructions after the zeros, so every 32-byte sector of a field is written whole
// while L2 holds it and DRAM takes no read-modify-write, and U / Ct sectors are read once whatever the lists' order.
// The force/torque sums are reduced per solid over the lanes of the warp (segmented by solid) before one FP64
// atomic per (solid, component).  The marks stay until the next interact clears them (sdfibm_cuda_apply_forcing
// visits the same chunks).
constexpr int CPL_WARPS = CPL_THREADS / 32;

// forcing of the first `count` queued cells (lane l takes entry l), written to the fields, F/T summed per solid
__device__ __forceinline__ void couple_queued(const CoupleArgs& A, const int32_t* qc, const uint32_t* qk, int count,
                                              float dtINV32, double dtINV) {
    const int lane = threadIdx.x & 31;
    const int64_t N = A.m.ncells;
    int s = -1;
    double f6[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    float g6[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    if (lane < count) {
        const int64_t c = qc[lane];
        const uint32_t key = qk[lane] - CT_KEY_BASE;
        s = (int)(key >> 2);
        const int type = (int)(key & 3u);
        float fs[3];
        const float alpha = cell_forcing(A, c, s, type, dtINV32, dtINV, fs, f6, g6, A.U[c], A.U[N + c],
                                         A.U[2 * N + c]);
        A.As[c] = fminf(alpha, 1.0f);
        A.Ts[c] = alpha;
        A.Fs[c] = fs[0];
        A.Fs[N + c] = fs[1];
        A.Fs[2 * N + c] = fs[2];
        A.Ct[c] = type == 1 ? s + 4 : type;
    }
    uint32_t pend = __ballot_sync(0xffffffffu, s >= 0);
    while (pend) {
        const int sl = __shfl_sync(0xffffffffu, s, __ffs(pend) - 1);
        const bool mine = s == sl;
        pend &= ~__ballot_sync(0xffffffffu, mine);
        double v;
        if (A.exact_forcing) {
            double t[8];
#pragma unroll
            for (int r = 0; r < 8; ++r) t[r] = mine ? f6[r] : 0.0;
            v = warp_total4(reduce_scatter8(t, lane));
        } else {
            float t[8];
#pragma unroll
            for (int r = 0; r < 8; ++r) t[r] = mine ? g6[r] : 0.f;
            v = warp_total4((double)reduce_scatter8(t, lane));
        }
        const int slot = lane >> 2;
        if ((lane & 3) == 0 && slot < 6) atomicAdd(A.ftacc + 6 * sl + slot, v);
    }
}

__global__ void __launch_bounds__(CPL_THREADS) couple_chunks_kernel(CoupleArgs A) {
    __shared__ int32_t s_qc[CPL_WARPS][64];   // per warp: queued cells claimed once, and their claim words
    __shared__ uint32_t s_qk[CPL_WARPS][64];
    const int64_t N = A.m.ncells;
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5, grp = lane >> 3, sub = lane & 7;
    int32_t* qc = s_qc[wib];
    uint32_t* qk = s_qk[wib];
    const int64_t words = (N + 255) >> 8;
    const int64_t nw = (int64_t)gridDim.x * (blockDim.x >> 5);
    const double dtINV = A.step->dtINV;
    const float dtINV32 = (float)dtINV;
    const uint32_t* C = reinterpret_cast<const uint32_t*>(A.Ct);
    int nq = 0;  // warp-uniform
    for (int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; w < words; w += nw) {
        uint32_t rem = A.cbits[w];
        while (rem) {  // warp-uniform: four marked chunks per pass
            uint32_t x = rem;
            for (int q = 0; q < grp; ++q) x &= x - 1;  // this group's chunk: the grp-th lowest mark left
#pragma unroll
            for (int q = 0; q < 4; ++q) rem &= rem - 1;
            const int64_t c = (((w << 5) + (__ffs(x) - 1)) << 3) + sub;
            bool single = false;
            uint32_t claim = 0;
            if (x != 0 && c < N) {
                claim = C[c];
                single = claim >= CT_KEY_BASE && !(claim & CT_SHARED);
                if (!single) {
                    A.As[c] = 0.f;
                    A.Ts[c] = 0.f;
                    A.Fs[c] = 0.f;
                    A.Fs[N + c] = 0.f;
                    A.Fs[2 * N + c] = 0.f;
                    A.Ct[c] = (claim & CT_SHARED) ? (int32_t)claim : 0;
                }
            }
            const uint32_t m = __ballot_sync(0xffffffffu, single);
            if (single) {
                const int pos = nq + __popc(m & ((1u << lane) - 1u));
                qc[pos] = (int32_t)c;
                qk[pos] = claim;
            }
            nq += __popc(m);
            __syncwarp();
            if (nq >= 32) {
                couple_queued(A, qc, qk, 32, dtINV32, dtINV);
                __syncwarp();
                if (lane < nq - 32) {
                    qc[lane] = qc[32 + lane];
                    qk[lane] = qk[32 + lane];
                }
                nq -= 32;
                __syncwarp();
            }
        }
    }
    if (nq > 0) couple_queued(A, qc, qk, nq, dtINV32, dtINV);
}

// Forcing applied to a GPU-resident fluid (main.cpp:70-77, its cell fields): U = U - Fs dt and T = (1 - As) T + Ts,
// in FP64 and rounded once to the FP32 fields, over the chunks the last interact marked in cbits.  Every other cell
// has As = Fs = Ts = 0 there and keeps its values, as in the dense update.  With cbits == nullptr (unstructured
// meshes) every cell is visited.  A warp per bitmap word, each store instruction covering 32 consecutive cells.
__global__ void apply_forcing_kernel(int64_t N, const uint32_t* __restrict__ cbits, double dt,
                                     const float* __restrict__ As, const float* __restrict__ Fs,
                                     const float* __restrict__ Ts, float* __restrict__ U, float* __restrict__ T) {
    const int lane = threadIdx.x & 31;
    const int64_t words = (N + 255) >> 8;
    const int64_t nw = (int64_t)gridDim.x * (blockDim.x >> 5);
    for (int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; w < words; w += nw) {
        const uint32_t word = cbits ? cbits[w] : 0xffffffffu;
        if (!word) continue;
#pragma unroll
        for (int t = 0; t < 8; ++t) {
            const int idx = 32 * t + lane;
            const int64_t c = (w << 8) + idx;
            if (((word >> (idx >> 3)) & 1u) && c < N) {
                // separate roundings, as the solver's own field operations (no contraction into FMAs)
                for (int a = 0; a < 3; ++a)
                    U[a * N + c] = (float)__dsub_rn((double)U[a * N + c], __dmul_rn((double)Fs[a * N + c], dt));
                if (T) T[c] = (float)__dadd_rn(__dmul_rn(__dsub_rn(1.0, (double)As[c]), (double)T[c]), (double)Ts[c]);
            }
        }
    }
}

// ---- finalize: cells shared by several solids ---------------------------------------------------------------------------
// FP64 sums rounded once to the FP32 fields, Ct decoded from the largest claim, As = min(As, 1) (checkAlpha); the slot
// is cleared for the next call.
__global__ void finalize_kernel(float* __restrict__ As, float* __restrict__ Ts, float* __restrict__ Fs,
                                int32_t* __restrict__ Ct, const Counters* cnt, int64_t N, int32_t* __restrict__ sh_keys,
                                double* __restrict__ sh_vals, const int32_t* __restrict__ sh_used, int32_t sh_mask) {
    const int n_sh = min(cnt->n_shared, sh_mask + 1);
    uint32_t* C = reinterpret_cast<uint32_t*>(Ct);
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n_sh; e += (int64_t)gridDim.x * blockDim.x) {
        const int slot = sh_used[e];
        const int32_t c = sh_keys[slot];
        double* v = sh_vals + 5 * (int64_t)slot;
        if (c >= 0 && c < N) {
            Ct[c] = decode_claim(C[c]);
            As[c] = (float)fmin(v[0], 1.0);
            Ts[c] = (float)v[1];
            Fs[c] = (float)v[2];
            Fs[N + c] = (float)v[3];
            Fs[2 * N + c] = (float)v[4];
        }
        for (int r = 0; r < 5; ++r) v[r] = 0.0;
        sh_keys[slot] = -1;
    }
}

// per-call counters: the previous lengths are kept for the sparse reset
__global__ void begin_kernel(Counters* cnt) {
    cnt->prev_n_inside = cnt->n_inside;
    cnt->prev_n_cut = cnt->n_cut;
    cnt->classify_next = 0; cnt->couple_next = 0; cnt->finalize_next = 0;
    cnt->n_inside = 0; cnt->n_cut = 0; cnt->n_shared = 0; cnt->shared_marks = 0;
    cnt->exact_rechecks = 0; cnt->bbox_cells = 0;
    cnt->n_feat = 0; cnt->n_fb = 0; cnt->n_recheck = 0; cnt->n_ovf = 0; cnt->n_shent = 0;
    cnt->n_inband = 0; cnt->n_small = 0;
}

// F = rho_f * V / dt * sum f, T = rho_f * V / dt * sum (C - x) x f  (solidcloud.cpp:411-421)
__global__ void ft_kernel(const double* __restrict__ ftacc, double* __restrict__ ft, int S, const StepParams* step) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= S) return;
    const double scale = step->ft_scale;
    for (int r = 0; r < 6; ++r) ft[6 * s + r] = ftacc[6 * s + r] * scale;
}

__global__ void set_step_kernel(StepParams* p, double time, double dt, int nsub, double rho_V) {
    p->time = time;
    p->dt = dt;
    p->dt_sub = dt / nsub;
    p->dtINV = 1.0 / dt;
    p->ft_scale = rho_V / dt;
}

// sparse reset: the cells the previous call touched and this call does not (after this call's claims) go back to
// zero -- the sparse form of solidcloud.cpp:438-441.  Cells in the chunks marked in cbits are left to
// couple_chunks_kernel, which writes every cell of those chunks.
__global__ void reset_kernel(const int32_t* __restrict__ prev_in_cell, const int32_t* __restrict__ prev_cut_cell,
                             const Counters* cnt, int64_t N, float* As, float* Fs, float* Ts, int32_t* Ct,
                             const uint32_t* __restrict__ cbits) {
    const int n_in = clamp_len(cnt->prev_n_inside, cnt->list_cap), n_cut = clamp_len(cnt->prev_n_cut, cnt->list_cap);
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < (int64_t)n_in + n_cut;
         e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t c = e < n_in ? prev_in_cell[e] : prev_cut_cell[e - n_in];
        if (c < 0 || c >= N) continue;
        if ((cbits[c >> 8] >> ((c >> 3) & 31)) & 1u) continue;  // written by the chunked coupling
        if (reinterpret_cast<const uint32_t*>(Ct)[c] >= CT_KEY_BASE) continue;
        As[c] = 0.f; Ts[c] = 0.f; Ct[c] = 0;
        Fs[c] = 0.f; Fs[N + c] = 0.f; Fs[2 * N + c] = 0.f;
    }
}

// interact_host on page-locked host fields.  The host fields held the previous call's values; the cells this call or
// the previous one touched (the current and the previous lists) are the ones that changed.  mark_export_kernel sets
// their chunks of EXPORT_CHUNK consecutive cells in a bitmap (one bit per chunk); export_kernel then copies every
// marked chunk from the device fields to the host fields through the mapped host pointers, a warp per bitmap word so
// that each store instruction covers 32 consecutive cells of a host array, and clears the word.
constexpr int EXPORT_LG = 3;  // log2 of the cells per chunk
constexpr int EXPORT_CHUNK = 1 << EXPORT_LG;
int export_chunk_cells() { return EXPORT_CHUNK; }

__global__ void mark_export_kernel(const int32_t* __restrict__ in_cell, const int32_t* __restrict__ cut_cell,
                                   const int32_t* __restrict__ prev_in_cell, const int32_t* __restrict__ prev_cut_cell,
                                   const Counters* cnt, int64_t N, uint32_t* __restrict__ dirty) {
    const int64_t n0 = clamp_len(cnt->n_inside, cnt->list_cap), n1 = clamp_len(cnt->n_cut, cnt->list_cap);
    const int64_t n2 = clamp_len(cnt->prev_n_inside, cnt->list_cap), n3 = clamp_len(cnt->prev_n_cut, cnt->list_cap);
    const int64_t total = n0 + n1 + n2 + n3;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
        int64_t c;
        if (e < n0) c = in_cell[e];
        else if (e < n0 + n1) c = cut_cell[e - n0];
        else if (e < n0 + n1 + n2) c = prev_in_cell[e - n0 - n1];
        else c = prev_cut_cell[e - n0 - n1 - n2];
        if (c < 0 || c >= N) continue;
        const uint32_t bit = 1u << ((c >> EXPORT_LG) & 31);
        uint32_t* word = dirty + (c >> (EXPORT_LG + 5));
        if (!(*word & bit)) atomicOr(word, bit);
    }
}

__global__ void export_kernel(Counters* cnt, int64_t N, uint32_t* __restrict__ dirty, const float* __restrict__ As,
                              const float* __restrict__ Fs, const float* __restrict__ Ts,
                              const int32_t* __restrict__ Ct, float* hAs, float* hFs, float* hTs, int32_t* hCt) {
    const int lane = threadIdx.x & 31;
    const int64_t words = (N + 32 * EXPORT_CHUNK - 1) >> (EXPORT_LG + 5);
    const int64_t nw = (int64_t)gridDim.x * (blockDim.x >> 5);
    int chunks = 0;
    for (int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; w < words; w += nw) {
        const uint32_t word = dirty[w];
        if (!word) continue;
        chunks += __popc(word);
#pragma unroll
        for (int t = 0; t < EXPORT_CHUNK; ++t) {
            const int64_t c = (w << (EXPORT_LG + 5)) + 32 * t + lane;
            if (((word >> ((32 * t + lane) >> EXPORT_LG)) & 1u) && c < N) {
                hAs[c] = As[c]; hTs[c] = Ts[c]; hCt[c] = Ct[c];
                hFs[c] = Fs[c]; hFs[N + c] = Fs[N + c]; hFs[2 * N + c] = Fs[2 * N + c];
            }
        }
        __syncwarp();
        if (lane == 0) dirty[w] = 0u;
    }
    if (lane == 0 && chunks) atomicAdd(&cnt->n_export, chunks);
}

// ---- FP64 host fields in OpenFOAM's own layout (sdfibm_cuda_interact_host64) -------------------------------------
// U is a volVectorField (one x,y,z triple per cell), As / Ts / Ct volScalarFields and Fs a volVectorField, all FP64
// in page-locked host memory.  gather_u64_kernel reads U at the coupling cells only (24 contiguous bytes per cell)
// into the FP32 device plane layout the coupling kernel reads; export64_kernel writes the marked 8-cell chunks of
// the four result fields back in FP64.
__global__ void gather_u64_kernel(const int32_t* __restrict__ in_cell, const int32_t* __restrict__ cut_cell,
                                  const Counters* cnt, int64_t N, const double* __restrict__ hU,
                                  float* __restrict__ U) {
    const int64_t n0 = clamp_len(cnt->n_inside, cnt->list_cap), n1 = clamp_len(cnt->n_cut, cnt->list_cap);
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n0 + n1; e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t c = e < n0 ? in_cell[e] : cut_cell[e - n0];
        if (c < 0 || c >= N) continue;
        const double x = hU[3 * c], y = hU[3 * c + 1], z = hU[3 * c + 2];
        U[c] = (float)x;
        U[N + c] = (float)y;
        U[2 * N + c] = (float)z;
    }
}

// all chunks marked (the first call on a set of host fields writes every cell)
__global__ void mark_all_kernel(uint32_t* __restrict__ dirty, int64_t words) {
    for (int64_t w = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; w < words; w += (int64_t)gridDim.x * blockDim.x)
        dirty[w] = 0xffffffffu;
}

// A warp per bitmap word (256 cells, 32 chunks).  An FP64 chunk of a scalar field is 64 bytes and of Fs 192 bytes,
// whole host cache lines: the scalar fields go out one cell per lane, Fs as the interleaved x,y,z sequence of the
// word's cells, element e of it at lane e mod 32, so that every store instruction writes 256 contiguous bytes (a lane
// per cell and a store per component would leave each instruction a third of each line).  The device values of a
// group of stores are loaded before the first of them.
__global__ void __launch_bounds__(256, 3) export64_kernel(Counters* cnt, int64_t N, uint32_t* __restrict__ dirty,
                                                      const float* __restrict__ As, const float* __restrict__ Fs,
                                                      const float* __restrict__ Ts, const int32_t* __restrict__ Ct,
                                                      double* __restrict__ hAs, double* __restrict__ hFs,
                                                      double* __restrict__ hTs, double* __restrict__ hCt) {
    const int lane = threadIdx.x & 31;
    const int64_t words = (N + 32 * EXPORT_CHUNK - 1) >> (EXPORT_LG + 5);
    const int64_t nw = (int64_t)gridDim.x * (blockDim.x >> 5);
    int chunks = 0;
    for (int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; w < words; w += nw) {
        const uint32_t word = dirty[w];
        if (!word) continue;
        chunks += __popc(word);
        const int64_t base = w << (EXPORT_LG + 5);
        {
            float a[EXPORT_CHUNK], t[EXPORT_CHUNK];
            int32_t k[EXPORT_CHUNK];
            bool on[EXPORT_CHUNK];
#pragma unroll
            for (int q = 0; q < EXPORT_CHUNK; ++q) {
                const int64_t c = base + 32 * q + lane;
                on[q] = ((word >> ((32 * q + lane) >> EXPORT_LG)) & 1u) && c < N;
                a[q] = on[q] ? As[c] : 0.f;
                t[q] = on[q] ? Ts[c] : 0.f;
                k[q] = on[q] ? Ct[c] : 0;
            }
#pragma unroll
            for (int q = 0; q < EXPORT_CHUNK; ++q) {
                const int64_t c = base + 32 * q + lane;
                if (on[q]) {
                    hAs[c] = (double)a[q];
                    hTs[c] = (double)t[q];
                    hCt[c] = (double)k[q];
                }
            }
        }
        // Fs: 3 x 256 elements, 24 stores per lane in three groups of eight
#pragma unroll 1
        for (int g = 0; g < 3; ++g) {
            float v[8];
            bool on[8];
#pragma unroll
            for (int q = 0; q < 8; ++q) {
                const int e = 32 * (8 * g + q) + lane;      // element of the word's interleaved sequence
                const int cl = (int)((unsigned)e / 3u), comp = e - 3 * cl;
                const int64_t c = base + cl;
                on[q] = ((word >> (cl >> EXPORT_LG)) & 1u) && c < N;
                v[q] = on[q] ? Fs[comp * N + c] : 0.f;
            }
#pragma unroll
            for (int q = 0; q < 8; ++q)
                if (on[q]) hFs[3 * base + 32 * (8 * g + q) + lane] = (double)v[q];
        }
        __syncwarp();
        if (lane == 0) dirty[w] = 0u;
    }
    if (lane == 0 && chunks) atomicAdd(&cnt->n_export, chunks);
}

// whole-field conversions of the FP64 path for host memory the GPU cannot address (staged through device copies)
__global__ void u64_to_planes_kernel(const double* __restrict__ U64, int64_t N, float* __restrict__ U) {
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < N; c += (int64_t)gridDim.x * blockDim.x) {
        U[c] = (float)U64[3 * c];
        U[N + c] = (float)U64[3 * c + 1];
        U[2 * N + c] = (float)U64[3 * c + 2];
    }
}
__global__ void fields_to_f64_kernel(int64_t N, const float* __restrict__ As, const float* __restrict__ Fs,
                                     const float* __restrict__ Ts, const int32_t* __restrict__ Ct,
                                     double* __restrict__ out) {
    // out: As[N], Fs[N][3], Ts[N], Ct[N]
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < N; c += (int64_t)gridDim.x * blockDim.x) {
        out[c] = (double)As[c];
        out[N + 3 * c] = (double)Fs[c];
        out[N + 3 * c + 1] = (double)Fs[N + c];
        out[N + 3 * c + 2] = (double)Fs[2 * N + c];
        out[4 * N + c] = (double)Ts[c];
        out[5 * N + c] = (double)Ct[c];
    }
}

// SolidCloud::fixInternal over the ALL_INSIDE list: U = rigid velocity of the solid that owns the cell
__global__ void fix_internal_kernel(MeshK m, const sdfibm_solid_state* __restrict__ st,
                                    const int32_t* __restrict__ in_cell, const int32_t* __restrict__ in_solid,
                                    const int32_t* __restrict__ Ct, float* __restrict__ U, const Counters* cnt) {
    const int n_in = clamp_len(cnt->n_inside, cnt->list_cap);
    const int64_t N = m.ncells;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n_in; e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t c = in_cell[e];
        const int32_t s = in_solid[e] & LIST_SOLID_MASK;
        if (c < 0 || c >= N) continue;
        if (Ct[c] != s + 4) continue;
        int i, j, k;
        cell_ijk(m, c, i, j, k);
        const sdfibm_solid_state& x = st[s];
        const D3 vel{x.vel[0], x.vel[1], x.vel[2]}, om{x.omega[0], x.omega[1], x.omega[2]};
        const D3 u = vel + cross(om, mesh_C(m, i, j, k) - state_pos(x));
        U[c] = (float)u.x; U[N + c] = (float)u.y; U[2 * N + c] = (float)u.z;
    }
}

}  // namespace sdfibm_dev
