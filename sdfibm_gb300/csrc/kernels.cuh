// Internal device-side records shared by the kernels and the C ABI implementation.
#pragma once
#include <cstdint>

#include "device_math.cuh"

namespace sdfibm_dev {

// Division of a cell label (< 2^31) by a fixed divisor: q = (n * mul) >> shift with mul = ceil(2^shift / d),
// shift = 32 + ceil(log2 d) (Granlund and Montgomery, "Division by invariant integers using multiplication", 1994).
struct FastDiv {
    uint64_t mul;
    uint32_t shift;
    uint32_t d;
};
inline FastDiv make_fastdiv(uint32_t d) {
    uint32_t l = 0;
    while ((1ull << l) < d) ++l;
    const unsigned __int128 p = (unsigned __int128)1 << (32 + l);
    return FastDiv{(uint64_t)((p + d - 1) / d), 32 + l, d};
}
__host__ __device__ inline uint32_t fdiv(uint32_t n, const FastDiv& f) { return (uint32_t)(((uint64_t)n * f.mul) >> f.shift); }

struct MeshK {
    int32_t nx, ny, nz, twod;
    double o[3], h[3];
    float h32[3];
    int64_t ncells;
    double V;  // hx*hy*hz
    FastDiv div_x, div_xy;  // by nx and by nx*ny
};
inline void mesh_fastdiv(MeshK& m) {
    m.div_x = make_fastdiv((uint32_t)m.nx);
    m.div_xy = make_fastdiv((uint32_t)((int64_t)m.nx * m.ny));
}
// (i, j, k) of cell label c (0 <= c < ncells < 2^31)
__device__ inline void cell_ijk(const MeshK& m, int64_t c, int& i, int& j, int& k) {
    const uint32_t u = (uint32_t)c;
    const uint32_t kk = fdiv(u, m.div_xy);
    const uint32_t r = u - kk * m.div_xy.d;
    const uint32_t jj = fdiv(r, m.div_x);
    i = (int)(r - jj * m.div_x.d);
    j = (int)jj;
    k = (int)kk;
}

// Static per-solid record (built once by sdfibm_cuda_create).
struct SolidK {
    ShapeK shape;
    int32_t infinite;        // Plane: the bbox is the whole mesh
    int32_t ext[3];          // static bbox extent in cells (per axis)
    int32_t tdim[3];         // cells per tile per axis
    int32_t ntile[3];        // tiles per axis
    int32_t tile_base;       // first work item of this solid in the classify queue
    int32_t bitmap_global;   // 1: the connect kernel keeps its bitmaps in global memory
    int64_t scratch_off;     // byte offset of the bbox class array
    int64_t bitmap_off;      // word offset of the global bitmaps (bitmap_global == 1)
    int32_t motion_type, forcer_type, collision_id, pad;
    FastDiv div_e0, div_e01;  // by ext[0] and by ext[0] * ext[1] (bbox index -> cell offsets)
    double radiusB;
    double rho, mass, mass_inv;
    double moi_inv[9];
    double motion_p[8];
    double forcer_p[8];
};

// Per-interact record of each solid (written by plan_kernel).
struct SolidPlan {
    int32_t lo[3];            // bbox lower cell index (may lie outside the mesh)
    int32_t err;              // nonzero: bbox too small for the current pose
    int64_t seed;             // meshSearch::findNearestCell result
    unsigned long long min_cand;  // lowest cell label with an inside vertex (atomicMin), ~0 when none
    float M[9];               // FP32 world->local matrix (|q|^2 R^T)
    int32_t n_inside, n_cut;  // touched cells by kind
    int32_t seed_ijk[3];      // cell indices of the seed cell
    int32_t pad1;
    double cbase[3];          // centre of the seed cell minus the solid centre (FP64), origin of FP32 cell offsets
    double base[3];           // mesh point (lo) minus the solid centre: FP64 origin of the FP32 tile frames
    float base32[3];          // base rounded to FP32 (the frames' origin)
    float pad4;
    double lmap[12];          // world2local of mesh point (lo), then the local images of h_x e_x, h_y e_y, h_z e_z
    float lmap_hi[12], lmap_lo[12];  // the same as FP32 pairs hi + lo (two-float vertex distances)
    float e64;                // bound of the FP64 rounding of point coordinates (see TileFrame)
    float pad2;
    double cw[3];             // centre of the bounding sphere (2-D shapes: of the bounding disc)
    double rcull;             // its radius
    int32_t vlo[3], vhi[3];   // mesh-vertex index box of the solid's oriented bounding box: vertices outside it are
                              // outside the solid (vlo > vhi on some axis: no vertex can be inside)
    // mixed forcing: the rigid-body velocity at the seed cell centre and its change per cell step (components
    // x: dj, dk; y: di, dk; z: di, dj) as FP32 pairs hi + lo, and cbase rounded to FP32
    float us_hi[3], us_lo[3];
    float ds_hi[6], ds_lo[6];
    float cb32[3];
    int32_t cull_box;         // 1: the inside region lies in the local box below (3-D spheres, ellipsoids, boxes)
    float lbox_c[3], lbox_s[3];  // that box in the local frame: centre and half extents (FP32, widened)
    float radius_cells;       // bounding radius / h (FP32): the solid-size half of the learned fraction's band
};

// Global counters / flags (one record per context, device memory).
struct Counters {
    int32_t classify_next;
    int32_t couple_next;
    int32_t finalize_next;
    int32_t n_inside;         // entries in the ALL_INSIDE list of this call
    int32_t n_cut;            // entries in the cut-cell list of this call
    int32_t n_shared;         // cells touched by two or more solids this call (slots used in the shared table)
    int32_t prev_n_inside;    // list lengths of the previous call (its lists stay for the sparse reset)
    int32_t prev_n_cut;
    int32_t error;            // first error code seen on the device
    int32_t shared_marks;     // claims that found the cell already claimed this call
    unsigned long long exact_rechecks;  // FP32-undecided points re-evaluated in FP64
    unsigned long long bbox_cells;
    int32_t launches;
    int32_t n_export;         // interact_host: 8-cell chunks written to the page-locked host fields
    int64_t list_cap;         // capacity of each touched-cell list (set once at create)
    int32_t n_feat;           // LEARNED: cut cells whose features the classify pass wrote this call
    int32_t n_fb;             // LEARNED: of those, cells outside the model's band (SUBSAMPLE fallback)
    int32_t n_recheck;        // SUBSAMPLE points left to recheck_kernel this call
    int32_t n_ovf;            // LEARNED: fallback cells whose points overflowed the recheck list (recount_kernel)
    int32_t n_shent;          // list entries on cells several solids claimed (shared_scan_kernel)
    int32_t n_inband;         // LEARNED: listed cut cells inside the band, compacted for the network
    int32_t n_small;          // LEARNED: cut cells of solids under rho_min, listed from the back (fallback)
    int32_t pad2;
};

// list lengths clamped to the capacity (a capacity error leaves the counters above what was written)
__host__ __device__ inline int32_t clamp_len(int32_t n, int64_t cap) { return (int32_t)(n < cap ? n : cap); }

// A SUBSAMPLE point whose FP32 test was undecided, left for recheck_kernel: the FP64 re-evaluations then run on full
// warps instead of one lane at a time.  sample = ia | ib << 8 | ic << 16 | n << 24.
struct Recheck {
    int64_t idx;     // index into the fraction array (which holds -(1 + decided inside count) meanwhile)
    int32_t solid;
    uint32_t sample;
};

// Time-step parameters the kernels read from device memory; set_step_kernel writes them at the head of a call, so a
// captured graph replays with new values after one kernel-node update.
struct StepParams {
    double time;
    double dt;
    double dt_sub;    // evolve: dt / sub-steps
    double dtINV;     // interact: 1 / dt
    double ft_scale;  // interact: rho_f * V / dt
};

struct CoupleArgs {
    MeshK m;
    const SolidK* sk;
    const sdfibm_solid_state* st;
    const SolidPlan* plan;
    const int32_t* in_cell;
    const int32_t* in_solid;
    const int32_t* cut_cell;
    const int32_t* cut_solid;
    const float* alpha;  // per bbox cell, from the classify pass
    const float* U;
    float* As;
    float* Fs;
    float* Ts;
    int32_t* Ct;
    double* ftacc;  // [S][6] sums of f*V/dt and (C-x)^f*V/dt
    Counters* cnt;
    const StepParams* step;
    int count_samples;   // a negative alpha is -(1 + inside count) out of this many SUBSAMPLE points
    int method;
    int subsample_n;
    int exact_forcing;
    // FP64 accumulation of the cells shared by several solids (open addressing, key -1 = empty)
    int32_t* sh_keys;
    double* sh_vals;   // [slot][5]: As, Ts, Fs.x, Fs.y, Fs.z
    int32_t* sh_used;  // slots filled this call
    int32_t sh_mask;
    // chunked coupling: marks of the 8-cell chunks with claimed cells / with shared cells (one bit per chunk)
    uint32_t* cbits;
    uint32_t* sbits;
    const uint32_t* shent;  // list entries on shared cells (shared_scan_kernel)
    int64_t shent_cap;
};

// Ct during a call holds claim words: CT_KEY_BASE | (solid << 2 | type), with CT_SHARED set once a second solid
// touched the cell (the low bits then hold the largest claim, i.e. the last solid in the reference's serial order)
constexpr uint32_t CT_KEY_BASE = 1u << 30;
constexpr uint32_t CT_SHARED = 1u << 31;
constexpr int SHARED_MAX_PROBES = 64;

// classify work items: up to chunk_tiles consecutive tiles of one solid (default below; the autotuner may change it)
constexpr int CHUNK_TILES = 8;

struct ClassifyArgs {
    MeshK m;
    const SolidK* sk;
    const sdfibm_solid_state* st;
    SolidPlan* plan;
    const int2* chunks;  // (solid, first tile)
    int total_chunks;
    int chunk_tiles;     // tiles per work item
    uint8_t* cls;      // class byte per bbox cell
    float* alpha;      // solid fraction per bbox cell (cut candidates only)
    Counters* cnt;
    int method;        // sdfibm_fraction_method, or -1: classification only
    int subsample_n;
    // SUBSAMPLE, LEARNED, REF-GEO: the list of cut cells (solid, index into alpha), feat_cap entries
    int64_t feat_cap;
    int32_t* fref_solid;
    int64_t* fref_index;  // index into alpha
    Recheck* rq;          // deferred SUBSAMPLE rechecks (nullptr: re-evaluate in place)
    int64_t rq_cap;
    float* rg_phi;        // REF-GEO: [8][feat_cap] vertex distances of the listed cut cells (nullptr: fraction in place)
    // LEARNED: solids whose bounding radius spans fewer cells (SolidPlan::radius_cells) list their cut cells from the
    // back of the list (positions feat_cap - 1 - i, n_small of them): the band sends them to the fallback whole
    float rho_min;
};

// SUBSAMPLE of listed cells: every listed cut cell (fb_list == nullptr), or the LEARNED cells left to SUBSAMPLE by
// the network's confidence band
struct FallbackArgs {
    MeshK m;
    const SolidK* sk;
    const sdfibm_solid_state* st;
    const SolidPlan* plan;
    const int32_t* fb_list;    // positions into the feature buffer (nullptr: every listed cell); LEARNED: then the
                               // n_small positions listed from the back
    const int32_t* fref_solid;
    const int64_t* fref_index;
    int64_t cap;
    float* alpha;
    Counters* cnt;
    int n;                     // samples per axis
    Recheck* rq;
    int64_t rq_cap;
    Recheck* ovf;              // cells to recount (idx, solid), see recount_kernel
    int64_t ovf_cap;
};

// LEARNED: the model inputs of the listed cut cells (learned_stencil_kernel)
struct StencilArgs {
    MeshK m;
    const SolidK* sk;
    const SolidPlan* plan;
    const int32_t* fref_solid;
    const int64_t* fref_index;
    int64_t cap;
    float* feat;          // [SDFIBM_MLP_NFEAT][cap]: network inputs, then the prior logit, of the in-band cells
                          // (compacted, n_inband of them)
    int32_t* fb_list;     // list positions of the cells outside the band (SUBSAMPLE fallback)
    int64_t* mlp_index;   // fraction index of each compacted in-band cell (the network's destination)
    Counters* cnt;
    float tau_refine;     // band: |P4 - P2| limit (the solid-size half, rho_min, is applied by the classify pass)
};

// UGrid (src/libcollision/ugrid.h:14-58): bbox of the mesh, spacing 2*max radiusB, row-major i*ny*nz + j*nz + k
struct GridK {
    double low[3];
    double dINV;
    int32_t nx, ny, nz, nynz;
    int64_t ncell;
};

// Fine broad-phase grid of the sphere-like solids: about 8 cells per solid, each solid listed in every cell its
// bounding box [x - r_B, x + r_B] overlaps (indices clamped to the grid).
struct FineGridK {
    double low[3];
    double inv;              // 1 / cell size
    int32_t n[3];
    int32_t pad;
    int64_t ncell;
    int64_t cap;             // entries reserved for the cell lists
};

// Per-solid record of one collision sub-step, written with the UGrid key: the integer data the pair search needs, so
// that it runs without FP64 work until a pair survives the FP32 screen.
struct alignas(16) CollRec {
    int32_t lo[3];
    int32_t id;      // contact-law id; -1 when the key is off the grid (the solid is never paired)
    int32_t hi[3];   // fine cell range [lo, hi] of the bounding box (sphere-like solids)
    int32_t pad0;
    int32_t c[3];    // the key decomposed as the UGrid neighbour loops do: key / nynz, (key / nz) % ny, key % nz
    int32_t pad1;
    float x, y, z, r;  // centre and bounding radius rounded to FP32 (the screen of sphere pairs)
};

// list entry word: solid index in bits 0..29, cell type (1 all inside, 2 centre inside, 3 centre outside) in 30..31
constexpr int LIST_TYPE_SHIFT = 30;
constexpr int32_t LIST_SOLID_MASK = (1 << LIST_TYPE_SHIFT) - 1;
__host__ __device__ inline int32_t list_word(int32_t solid, int type) {
    return (int32_t)((uint32_t)solid | ((uint32_t)type << LIST_TYPE_SHIFT));
}
__host__ __device__ inline int list_type(int32_t w) { return (int)((uint32_t)w >> LIST_TYPE_SHIFT); }

enum DeviceError : int32_t {
    DERR_NONE = 0,
    DERR_CAPACITY = 1,     // a list outgrew its capacity
    DERR_BBOX = 2,         // a solid's region left its static bbox (tilted 2-D shape)
    DERR_FLOOD_LIMIT = 3,  // flood fill hit its iteration bound
    DERR_SHARED_TABLE = 4, // the shared-cell table is full
    DERR_MMA_TIMEOUT = 7   // a tensor-core completion was not observed in time (SDFIBM_MLP_ERR_TIMEOUT)
};

}  // namespace sdfibm_dev
