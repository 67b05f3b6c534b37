// C ABI of the coupling library (include/sdfibm_cuda.h): context set-up, launch sequencing, error reporting.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <functional>
#include <string>
#include <type_traits>
#include <map>
#include <mutex>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/sdfibm_cuda.h"
#include "kernels.cuh"
#include "mlp.cuh"
#include "poly.hpp"
#include "poly_dev.cuh"
#include "../../include/sdfibm_mlp.h"

namespace sdfibm_dev {
// coupling.cu
__global__ void plan_kernel(MeshK m, const SolidK* sk, const sdfibm_solid_state* st, SolidPlan* plan, int S,
                            Counters* cnt);
void launch_classify(const ClassifyArgs& A, bool flat, int grid, cudaStream_t st);
int classify_occupancy(int method, bool flat);
__global__ void subsample_cells_kernel(FallbackArgs A);
__global__ void recount_kernel(FallbackArgs A);
__global__ void learned_stencil_kernel(StencilArgs A);
int stencil_block();
__global__ void refgeo_cells_kernel(MeshK m, const SolidK* sk, const SolidPlan* plan, const int32_t* fref_solid,
                                    const int64_t* fref_index, const float* rg_phi, int64_t cap, const Counters* cnt,
                                    float* alpha);
__global__ void recheck_kernel(MeshK m, const SolidK* sk, const sdfibm_solid_state* st, const SolidPlan* plan,
                               const Recheck* rq, int64_t cap, Counters* cnt, float* alpha);
__global__ void connect_kernel(MeshK m, const SolidK* sk, SolidPlan* plan, const uint8_t* scratch, uint32_t* gbitmaps,
                               int32_t* in_cell, int32_t* in_solid, int32_t* cut_cell, int32_t* cut_solid,
                               int64_t cap_in, int64_t cap_cut, Counters* cnt, int smem_words, const int32_t* solids);
__global__ void connect_small_kernel(MeshK m, const SolidK* sk, SolidPlan* plan, const uint8_t* scratch,
                                     int32_t* in_cell, int32_t* in_solid, int32_t* cut_cell, int32_t* cut_solid,
                                     int64_t cap_in, int64_t cap_cut, Counters* cnt, const int32_t* solids,
                                     int nsolids);

__global__ void couple_shared_kernel(CoupleArgs A);
__global__ void shared_scan_kernel(const int32_t* in_cell, const int32_t* cut_cell, const int32_t* Ct, Counters* cnt,
                                   int64_t N, const uint32_t* sbits, uint32_t* shent, int64_t shent_cap);
__global__ void couple_chunks_kernel(CoupleArgs A);
__global__ void apply_forcing_kernel(int64_t N, const uint32_t* cbits, double dt, const float* As, const float* Fs,
                                     const float* Ts, float* U, float* T);
__global__ void finalize_kernel(float* As, float* Ts, float* Fs, int32_t* Ct, const Counters* cnt, int64_t N,
                                int32_t* sh_keys, double* sh_vals, const int32_t* sh_used, int32_t sh_mask);
__global__ void begin_kernel(Counters* cnt);
__global__ void claim_kernel(const int32_t* in_cell, const int32_t* in_solid, const int32_t* cut_cell,
                             const int32_t* cut_solid, int32_t* Ct, Counters* cnt, int64_t N, uint32_t* cbits,
                             uint32_t* sbits);
__global__ void ft_kernel(const double* ftacc, double* ft, int S, const StepParams* step);
__global__ void set_step_kernel(StepParams* p, double time, double dt, int nsub, double rho_V);
int export_chunk_cells();
__global__ void mark_export_kernel(const int32_t* in_cell, const int32_t* cut_cell, const int32_t* prev_in_cell,
                                   const int32_t* prev_cut_cell, const Counters* cnt, int64_t N, uint32_t* dirty);
__global__ void export_kernel(Counters* cnt, int64_t N, uint32_t* dirty, const float* As, const float* Fs,
                              const float* Ts, const int32_t* Ct, float* hAs, float* hFs, float* hTs, int32_t* hCt);
__global__ void gather_u64_kernel(const int32_t* in_cell, const int32_t* cut_cell, const Counters* cnt, int64_t N,
                                  const double* hU, float* U);
__global__ void mark_all_kernel(uint32_t* dirty, int64_t words);
__global__ void export64_kernel(Counters* cnt, int64_t N, uint32_t* dirty, const float* As, const float* Fs,
                                const float* Ts, const int32_t* Ct, double* hAs, double* hFs, double* hTs,
                                double* hCt);
__global__ void u64_to_planes_kernel(const double* U64, int64_t N, float* U);
__global__ void fields_to_f64_kernel(int64_t N, const float* As, const float* Fs, const float* Ts, const int32_t* Ct,
                                     double* out);
__global__ void reset_kernel(const int32_t* in_cell, const int32_t* cut_cell, const Counters* cnt, int64_t N,
                             float* As, float* Fs, float* Ts, int32_t* Ct, const uint32_t* cbits);
__global__ void fix_internal_kernel(MeshK m, const sdfibm_solid_state* st, const int32_t* in_cell,
                                    const int32_t* in_solid, const int32_t* Ct, float* U, const Counters* cnt);
// evolve.cu

__global__ void evolve_independent_kernel(const SolidK* sk, sdfibm_solid_state* st, int S, int nsub,
                                          const StepParams* step, double rho_f, D3 g);
__global__ void evolve_pre_kernel(const SolidK* sk, sdfibm_solid_state* st, int S, const StepParams* step, double rho_f, D3 g,
                                  GridK gk, int64_t* hashes, int32_t* counts, FineGridK fg, int32_t* fcounts, int mode,
                                  int coarse_needed, CollRec* recs, int move_first);
__global__ void fine_scatter_kernel(const CollRec* recs, int S, FineGridK fg, int32_t* fcursor, int32_t* flist,
                                    Counters* cnt);
__global__ void grid_scan_kernel(int32_t* counts, int32_t* start, int32_t* cursor, int64_t ncell);
__global__ void scan_blocks_kernel(int32_t* counts, int32_t* start, int32_t* sums, int64_t ncell);
__global__ void scan_add_kernel(int32_t* start, int32_t* cursor, const int32_t* sums_excl, int64_t ncell,
                                int64_t nblocks);
__global__ void grid_scatter_kernel(const int64_t* hashes, int32_t* cursor, int32_t* list, int S, int64_t ncell);
__global__ void collide_kernel(const SolidK* sk, sdfibm_solid_state* st, int S, GridK gk, const int64_t* hashes,
                               const int32_t* start, const int32_t* list, int mode, FineGridK fg, const int32_t* fstart,
                               const int32_t* flist, const int32_t* planes, int nplanes, const CollRec* recs);
__global__ void move_kernel(const SolidK* sk, sdfibm_solid_state* st, int S, const StepParams* step);
__global__ void store_old_kernel(sdfibm_solid_state* st, int S);
__global__ void ft_to_state_kernel(const double* ft, sdfibm_solid_state* st, int S);
}  // namespace sdfibm_dev

using namespace sdfibm_dev;

// copies this call's fluid force and torque into the solid state (Solid::setFluidForceAndTorque)
namespace sdfibm_dev {
__global__ void ft_to_state_kernel(const double* ft, sdfibm_solid_state* st, int S) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= S) return;
    for (int a = 0; a < 3; ++a) {
        st[s].fluid_force[a] = ft[6 * s + a];
        st[s].fluid_torque[a] = ft[6 * s + 3 + a];
    }
}
}  // namespace sdfibm_dev

struct sdfibm_ctx {
    cudaStream_t stream = nullptr;
    int device = 0;
    int num_sms = 0;
    MeshK mesh{};
    sdfibm_mesh_desc mdesc{};
    sdfibm_options opt{};
    int S = 0;
    int nsub = 20;
    std::vector<SolidK> hk;
    SolidK* d_sk = nullptr;
    sdfibm_solid_state* d_st = nullptr;
    SolidPlan* d_plan = nullptr;
    int2* d_chunks = nullptr;  // classify work items: (solid, first tile)
    int total_chunks = 0;
    int chunk_tiles = CHUNK_TILES;
    int64_t chunks_cap = 0;    // entries reserved in d_chunks
    int total_tiles = 0;
    uint8_t* d_scratch = nullptr;
    float* d_alpha = nullptr;  // solid fraction per bbox cell (same indexing as d_scratch)
    int64_t scratch_bytes = 0;
    uint32_t* d_gbitmaps = nullptr;
    // chunked coupling: one bit per 8-cell chunk holding a claimed cell / a cell claimed twice (cleared as used)
    uint32_t *d_cbits = nullptr, *d_sbits = nullptr;
    uint32_t* d_shent = nullptr;  // list entries on shared cells, compacted by shared_scan_kernel
    int64_t shent_cap = 0;
    int64_t gbitmap_words = 0;
    int connect_smem_bytes = 0;
    // flood-fill work: solids with small bbox bitmaps (one warp each) and the others (one CTA each)
    int32_t *d_small = nullptr, *d_big = nullptr;
    int n_small = 0, n_big = 0;
    // SUBSAMPLE points whose FP32 test was undecided, re-evaluated in FP64 on full warps by recheck_kernel
    Recheck* d_rq = nullptr;
    int64_t rq_cap = 0;
    // LEARNED: fallback cells whose points overflowed the recheck list, recounted with FP64 in place
    Recheck* d_ovf = nullptr;
    int64_t ovf_cap = 0;
    // touched-cell lists, double buffered: [cur] is this call's, [cur ^ 1] the previous call's (sparse reset)
    int32_t* d_lists[2][4] = {{nullptr, nullptr, nullptr, nullptr}, {nullptr, nullptr, nullptr, nullptr}};
    int cur = 0;
    int32_t* in_cell() const { return d_lists[cur][0]; }
    int32_t* in_solid() const { return d_lists[cur][1]; }
    int32_t* cut_cell() const { return d_lists[cur][2]; }
    int32_t* cut_solid() const { return d_lists[cur][3]; }
    int64_t cap = 0;
    int32_t* d_sh_keys = nullptr;
    double* d_sh_vals = nullptr;
    int32_t* d_sh_used = nullptr;
    int32_t sh_mask = 0;
    Counters* d_cnt = nullptr;
    Counters* h_cnt = nullptr;  // pinned
    double* d_ftacc = nullptr;
    double* d_ft = nullptr;
    double* h_ft = nullptr;  // pinned
    // collision grid
    bool grid_active = false;
    GridK gk{};
    int64_t* d_hash = nullptr;
    CollRec* d_recs = nullptr;  // per-solid collision records of the current sub-step
    int32_t *d_gcount = nullptr, *d_gstart = nullptr, *d_gcursor = nullptr, *d_glist = nullptr;
    // fine broad phase of the sphere-like solids and the list of plane-like ones (contact law id 0)
    FineGridK fg{};
    int32_t *d_fcount = nullptr, *d_fstart = nullptr, *d_fcursor = nullptr, *d_flist = nullptr, *d_planes = nullptr;
    int32_t *d_fsums = nullptr, *d_fsums_excl = nullptr;  // block sums of the multi-block scans of the two grids
    int nplanes = 0;
    // fields seen by the last interact (sparse reset is only valid on the same buffers)
    const void* last_fields[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
    bool interacted = false;
    // host staging for sdfibm_cuda_interact_host: U is uploaded on its own copy stream while the enumeration runs
    // (only couple reads U), the four fields come back on four copy streams
    float *d_U = nullptr, *d_As = nullptr, *d_Fs = nullptr, *d_Ts = nullptr;
    int32_t* d_Ct = nullptr;
    cudaStream_t copy_st[4] = {nullptr, nullptr, nullptr, nullptr};
    cudaEvent_t ev_entry = nullptr, ev_u = nullptr, ev_done = nullptr;
    // side stream of interact: the component pass (connect, claim, reset) runs there beside the fraction kernels
    cudaStream_t side_st = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    cudaEvent_t u_wait = nullptr;  // set while interact_host runs: couple waits for the upload
    // interact_host: U copied in whole while the fraction kernels run, unless the copy outlasts them on this machine
    // (measured on the calls, events t0 -> copy done and t0 -> the coupling kernel's wait): then a page-locked U is
    // read in place at the coupling cells
    bool u_probe = false, u_in_place = false;
    int u_slow = 0;
    cudaEvent_t ev_t0 = nullptr, ev_tu = nullptr, ev_tpre = nullptr;
    // interact_host on page-locked host fields: the host buffers of the last such call (their cells equal the device
    // fields after it) and the bytes the last interact_host moved each way
    const void* host_fields[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
    bool host_synced = false;
    bool host_sparse = false;  // the last interact_host exported the touched cells only
    int64_t host_h2d = 0, host_d2h = 0;
    uint32_t* d_dirty = nullptr;  // changed 8-cell chunks of the fields, one bit each (cleared by export_kernel)
    // interact_host64 (FP64 fields in OpenFOAM's layout): device address of the page-locked U while a call runs
    // (gathered at the coupling cells after the enumeration), the host buffers of the last call, and the device
    // staging of the whole-field path for memory the GPU cannot address
    const double* u64_dev = nullptr;
    const void* host64_fields[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
    bool host64_synced = false;
    double* d_f64 = nullptr;  // [3N] U, then [6N] As, Fs, Ts, Ct
    // CTA counts of the launches the autotuner sets (defaults from the occupancy at create)
    int classify_grid = 0, couple_grid = 0, subsample_grid = 0, mlp_grid = 0, refgeo_grid = 0, stencil_grid = 0;
    int classify_occ = 1, couple_occ = 1;  // resident CTAs per SM
    bool tuned_from_cache = false;
    // per-kernel events (options.timing)
    static constexpr int MAXEV = 24;
    cudaEvent_t ev[MAXEV + 1] = {};
    const char* ev_name[MAXEV] = {};
    // learned fraction (SDFIBM_FRACTION_LEARNED): model and per-cut-cell feature buffers
    float* d_mlp = nullptr;
    float tau_refine = 0.f, rho_min = 0.f;  // confidence band of the learned fraction
    bool model_set = false;
    float* d_feat = nullptr;  // [SDFIBM_MLP_NFEAT][feat_cap]: model inputs and prior of the in-band cut cells
    int64_t* d_mlp_index = nullptr;  // fraction index of each of those cells
    float* d_rg_phi = nullptr;  // REF-GEO: [8][feat_cap] vertex distances of the listed cut cells
    int64_t feat_cap = 0;
    int32_t* d_fref_solid = nullptr;
    int64_t* d_fref_index = nullptr;
    int32_t* d_fb = nullptr;
    int nev = 0;
    bool ev_ready = false;
    int launches_last = 0;
    std::string err;
    // time-step parameters on the device ([0] interact, [1] evolve) and the captured graphs
    StepParams* d_step = nullptr;
    struct Graph {
        bool valid = false;
        cudaGraphExec_t exec = nullptr;
        cudaGraphNode_t step_node = nullptr;
        cudaKernelNodeParams step_params{};
        int cur = -1, dense = -1;
        const void* fields[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
        const double* u64 = nullptr;
        int launches = 0;
    };
    Graph igraph[4];
    Graph egraph;
    bool graphs_failed = false;
    std::vector<cudaGraph_t> graphs_keep;
    // explicit (unstructured) polyMesh: set by sdfibm_cuda_create_polymesh, which builds the rest of the context
    // over a one-cell box of the mesh's extent (solid records, states, collision grid); only the poly kernels then
    // touch the fields
    struct Poly {
        int64_t N = 0;
        PolyK k{};
        PolyWork w{};
        std::vector<void*> allocs;
        float *dU = nullptr, *dAs = nullptr, *dFs = nullptr, *dTs = nullptr;  // host-entry staging
        int32_t* dCt = nullptr;
        double* d64 = nullptr;
        std::vector<int32_t> counts;
    };
    Poly* poly = nullptr;
};

// event bracketing of each launch when timing is on: mark(ctx, name) after a launch records its end
static void mark_begin(sdfibm_ctx* ctx) {
    ctx->nev = 0;
    if (!ctx->opt.timing) return;
    if (!ctx->ev_ready) {
        for (int i = 0; i <= sdfibm_ctx::MAXEV; ++i) cudaEventCreate(&ctx->ev[i]);
        ctx->ev_ready = true;
    }
    cudaEventRecord(ctx->ev[0], ctx->stream);
}
static void mark(sdfibm_ctx* ctx, const char* name) {
    if (!ctx->opt.timing || ctx->nev >= sdfibm_ctx::MAXEV) return;
    ctx->ev_name[ctx->nev] = name;
    cudaEventRecord(ctx->ev[ctx->nev + 1], ctx->stream);
    ++ctx->nev;
}

static int fail(sdfibm_ctx* ctx, int code, const std::string& msg) {
    if (ctx) ctx->err = msg;
    return code;
}
#define CK(call)                                                                                         \
    do {                                                                                                 \
        cudaError_t e_ = (call);                                                                         \
        if (e_ != cudaSuccess)                                                                           \
            return fail(ctx, SDFIBM_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_));       \
    } while (0)

// classify work items: chunks of up to chunk_tiles consecutive tiles of each solid, the solids grouped by shape type
// (stable): the cut-cell lists then come out grouped by type too, so that the warps of the per-cell kernels mostly
// run one shape's distance code (the learned stencil: 11 % faster at 256^3 than with the types interleaved)
static std::vector<int2> make_chunks(const std::vector<SolidK>& hk, int chunk_tiles) {
    std::vector<int2> chunks;
    std::vector<size_t> order(hk.size());
    for (size_t s = 0; s < hk.size(); ++s) order[s] = s;
    std::stable_sort(order.begin(), order.end(),
                     [&](size_t a, size_t b) { return hk[a].shape.type < hk[b].shape.type; });
    for (size_t s : order) {
        const SolidK& k = hk[s];
        const int nt = k.ntile[0] * k.ntile[1] * k.ntile[2];
        for (int t0 = 0; t0 < nt; t0 += chunk_tiles) chunks.push_back(make_int2((int)s, t0));
    }
    return chunks;
}

template <class T>
static cudaError_t dalloc(T** p, size_t n) {
    return cudaMalloc((void**)p, std::max<size_t>(1, n) * sizeof(T));
}

// ---- explicit polyMesh (unstructured) contexts: helpers ----------------------------------------------------------
__global__ void poly_ft_kernel(const double* ftacc, double* ft, int S, double rho_f) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= S) return;
    for (int r = 0; r < 6; ++r) ft[6 * s + r] = ftacc[6 * s + r] * rho_f;  // force *= m_rhof (solidcloud.cpp:423)
}

template <typename T>
static cudaError_t poly_alloc(sdfibm_ctx::Poly& P, T** p, size_t n) {
    const cudaError_t e = cudaMalloc((void**)p, std::max<size_t>(1, n) * sizeof(T));
    if (e == cudaSuccess) P.allocs.push_back((void*)*p);
    else *p = nullptr;
    return e;
}

template <typename T>
static bool poly_upload(sdfibm_ctx::Poly& P, const T** dst, const std::vector<T>& v) {
    T* d = nullptr;
    if (poly_alloc(P, &d, v.size()) != cudaSuccess) return false;
    *dst = d;
    return v.empty() || cudaMemcpy(d, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice) == cudaSuccess;
}

extern "C" {

const char* sdfibm_cuda_version(void) { return "sdfibm-gb300 1.0 (sm_103a)"; }

const char* sdfibm_cuda_last_error(const sdfibm_ctx* ctx) { return ctx ? ctx->err.c_str() : "null context"; }

// radius around -com of a sphere (or, for 2-D shapes, a disc in the local x-y plane) that holds every point the
// shape's isInside accepts (IShape::m_radiusB is not such a bound for rectangles, boxes and tails)
static bool bound_radius(const sdfibm_shape_desc& s, double& r, int& prism) {
    const double* a = s.p;
    prism = 0;
    switch (s.type) {
        case SDFIBM_SHAPE_CIRCLE: r = a[0]; prism = 1; return true;
        case SDFIBM_SHAPE_SPHERE: r = a[0]; return true;
        case SDFIBM_SHAPE_ELLIPSE: r = std::max(a[0], a[1]); prism = 1; return true;
        case SDFIBM_SHAPE_ELLIPSOID: r = std::max({a[0], a[1], a[2]}); return true;
        case SDFIBM_SHAPE_RECTANGLE: r = std::sqrt(a[0] * a[0] + a[1] * a[1]); prism = 1; return true;
        case SDFIBM_SHAPE_BOX: r = std::sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]); return true;
        case SDFIBM_SHAPE_CIRCLE_TAIL:
        case SDFIBM_SHAPE_CIRCLE_TWOTAIL:
            r = std::max(a[0], std::sqrt(4 * a[4] * a[4] + a[2] * a[2]));
            prism = 1;
            return true;
        case SDFIBM_SHAPE_PLANE: r = 0; return true;
        default: return false;
    }
}

int sdfibm_cuda_create(const sdfibm_mesh_desc* mesh, const sdfibm_solid_desc* solids, int32_t nsolids,
                       const sdfibm_options* opt_in, void* cuda_stream, sdfibm_ctx** out) {
    if (!out) return SDFIBM_ERR_ARG;
    *out = nullptr;
    if (!mesh || (nsolids > 0 && !solids) || nsolids < 0 || nsolids > (1 << 28)) return SDFIBM_ERR_ARG;
    if (mesh->nx <= 0 || mesh->ny <= 0 || mesh->nz <= 0) return SDFIBM_ERR_ARG;
    if (!(mesh->h[0] > 0 && mesh->h[1] > 0 && mesh->h[2] > 0)) return SDFIBM_ERR_ARG;
    const int64_t N = (int64_t)mesh->nx * mesh->ny * mesh->nz;
    if (N >= ((int64_t)1 << 31)) return SDFIBM_ERR_ARG;  // cell labels are stored as int32
    auto* ctx = new sdfibm_ctx();
    ctx->mdesc = *mesh;
    if (opt_in) ctx->opt = *opt_in; else sdfibm_options_default(&ctx->opt);
    if (ctx->opt.subsample_n <= 0) ctx->opt.subsample_n = 10;
    ctx->S = nsolids;
    ctx->nsub = ctx->opt.n_subiter > 0 ? ctx->opt.n_subiter : (nsolids == 1 ? 1 : 20);
    ctx->stream = (cudaStream_t)cuda_stream;
    auto bail = [&](int code) {
        int c = code;
        sdfibm_cuda_destroy(ctx);
        return c;
    };
    if (cudaGetDevice(&ctx->device) != cudaSuccess) { delete ctx; return SDFIBM_ERR_CUDA; }
    cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, ctx->device);
    if (cudaStreamCreateWithFlags(&ctx->side_st, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->ev_fork, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->ev_join, cudaEventDisableTiming) != cudaSuccess) {
        ctx->err = "stream creation failed";
        return bail(SDFIBM_ERR_CUDA);
    }
    MeshK& m = ctx->mesh;
    m.nx = mesh->nx; m.ny = mesh->ny; m.nz = mesh->nz; m.twod = mesh->twod;
    for (int a = 0; a < 3; ++a) { m.o[a] = mesh->origin[a]; m.h[a] = mesh->h[a]; m.h32[a] = (float)mesh->h[a]; }
    m.ncells = N;
    m.V = mesh->h[0] * mesh->h[1] * mesh->h[2];
    mesh_fastdiv(m);
    const int32_t n3[3] = {mesh->nx, mesh->ny, mesh->nz};

    // static per-solid records
    ctx->hk.resize(nsolids);
    std::vector<int32_t> small_solids, big_solids;
    int64_t scratch = 0, gwords = 0, bbox_total = 0;
    int64_t tiles = 0;
    int max_smem_words = 0;
    // the flood fill's bitmaps stay in shared memory up to this size (every CTA of the launch reserves the largest, so
    // the cap keeps two 512-thread CTAs per SM); larger ones live in global memory
    const int SMEM_CAP_BYTES = 96 * 1024;
    for (int s = 0; s < nsolids; ++s) {
        const sdfibm_solid_desc& d = solids[s];
        SolidK& k = ctx->hk[s];
        std::memset(&k, 0, sizeof(k));
        k.shape.type = d.shape.type;
        for (int i = 0; i < 8; ++i) {
            k.shape.p[i] = d.shape.p[i];
            k.shape.p32[i] = (float)d.shape.p[i];
            k.shape.p_lo[i] = (float)(d.shape.p[i] - (double)k.shape.p32[i]);
        }
        for (int i = 0; i < 3; ++i) {
            k.shape.com[i] = d.shape.com[i];
            k.shape.com32[i] = (float)d.shape.com[i];
            k.shape.com_lo[i] = (float)(d.shape.com[i] - (double)k.shape.com32[i]);
        }
        double r;
        int prism;
        if (!bound_radius(d.shape, r, prism)) { ctx->err = "unknown shape type"; return bail(SDFIBM_ERR_ARG); }
        k.shape.bound_r = r;
        k.shape.prism = prism;
        k.infinite = d.shape.type == SDFIBM_SHAPE_PLANE;
        const double rr = r * (1.0 + 1e-9) + 1e-12;
        for (int a = 0; a < 3; ++a) {
            int64_t e;
            if (k.infinite || (prism && a == 2)) e = n3[a];
            else e = (int64_t)std::ceil(2.0 * rr / mesh->h[a]) + 4 + (prism ? 4 : 0);
            if (!k.infinite && !(prism && a == 2) && e >= (int64_t)n3[a] + 4) e = (int64_t)n3[a] + 4;  // bounded
            k.ext[a] = (int32_t)e;
        }
        if (!k.infinite && prism && !(d.quat[1] == 0.0 && d.quat[2] == 0.0)) {
            // a 2-D shape that does not rotate about z: its prism may cross the whole mesh
            for (int a = 0; a < 2; ++a) k.ext[a] = n3[a] + 4;
        }
        // warp tiles: 4x4x4 cells, or 8x8x2 on one- and two-layer meshes
        const bool layer = mesh->nz <= 2;
        k.tdim[0] = layer ? 8 : 4;
        k.tdim[1] = layer ? 8 : 4;
        k.tdim[2] = layer ? 2 : 4;
        for (int a = 0; a < 3; ++a) k.ntile[a] = (k.ext[a] + k.tdim[a] - 1) / k.tdim[a];
        k.div_e0 = make_fastdiv((uint32_t)k.ext[0]);
        k.div_e01 = make_fastdiv((uint32_t)((int64_t)k.ext[0] * k.ext[1]));
        k.tile_base = (int32_t)tiles;
        tiles += (int64_t)k.ntile[0] * k.ntile[1] * k.ntile[2];
        const int64_t cells = (int64_t)k.ext[0] * k.ext[1] * k.ext[2];
        k.scratch_off = scratch;
        scratch += (cells + 15) & ~(int64_t)15;
        bbox_total += std::min<int64_t>(cells, N);
        // connect_kernel: four bitmaps (candidates, reached, inside, centre inside) of ext[1] * ext[2] rows
        const int64_t words = 4 * (int64_t)k.ext[1] * k.ext[2] * ((k.ext[0] + 31) / 32);
        if (words / 4 <= 256) {
            small_solids.push_back(s);  // warp-per-solid flood fill (connect_small_kernel)
        } else if (words * 4 > SMEM_CAP_BYTES) {
            k.bitmap_global = 1;
            k.bitmap_off = gwords;
            gwords += words;
            big_solids.push_back(s);
        } else {
            max_smem_words = std::max<int>(max_smem_words, (int)words);
            big_solids.push_back(s);
        }
        k.motion_type = d.motion_type;
        k.forcer_type = d.forcer_type;
        k.collision_id = d.shape.collision_id;
        k.radiusB = d.shape.radiusB;
        k.rho = d.rho; k.mass = d.mass; k.mass_inv = d.mass_inv;
        for (int i = 0; i < 9; ++i) k.moi_inv[i] = d.moi_inv[i];
        for (int i = 0; i < 8; ++i) { k.motion_p[i] = d.motion_p[i]; k.forcer_p[i] = d.forcer_p[i]; }
    }
    if (tiles >= ((int64_t)1 << 31)) { ctx->err = "too many bbox tiles"; return bail(SDFIBM_ERR_CAPACITY); }
    ctx->total_tiles = (int)tiles;
    ctx->chunks_cap = tiles;
    ctx->scratch_bytes = scratch;
    ctx->gbitmap_words = gwords;
    ctx->connect_smem_bytes = max_smem_words * 4;
    ctx->n_small = (int)small_solids.size();
    ctx->n_big = (int)big_solids.size();
    ctx->rq_cap = ctx->opt.recheck_cap > 0 ? (int64_t)ctx->opt.recheck_cap
                                            : std::min<int64_t>(std::max<int64_t>(scratch / 8, 1 << 20), 1 << 25);
    ctx->ovf_cap = std::max<int64_t>(ctx->rq_cap / 16, std::min<int64_t>(scratch, 1 << 16));
    ctx->cap = std::max<int64_t>(1, bbox_total);

    {
        // shared-cell table: a power of two well above the expected count of cells touched by several solids
        int64_t want = std::max<int64_t>(1 << 12, std::min<int64_t>(ctx->cap, N) / 4);
        want = std::min<int64_t>(want, (int64_t)1 << 22);
        int64_t t = 1;
        while (t < 2 * want) t <<= 1;
        ctx->sh_mask = (int32_t)(t - 1);
        ctx->shent_cap = 2 * t;  // a shared cell has two or more entries
    }
    ctx->chunk_tiles = CHUNK_TILES;
    if (ctx->opt.tile_cells > 0) {
        const int cells_per_tile = mesh->nz <= 2 ? 8 * 8 * 2 : 4 * 4 * 4;
        ctx->chunk_tiles = std::max(1, std::min(255, ctx->opt.tile_cells / cells_per_tile));
    }
    std::vector<int2> chunks = make_chunks(ctx->hk, ctx->chunk_tiles);
    ctx->total_chunks = (int)chunks.size();

    // collision grid (UGrid(bbox of the mesh, 2*max radiusB))
    if (ctx->opt.collision_mode != SDFIBM_COLLISION_OFF && nsolids > 0) {
        double rB = -1.0;
        for (int s = 0; s < nsolids; ++s) rB = std::max(rB, solids[s].shape.radiusB);
        const double delta = 2 * rB;
        const double dINV = 1.0 / delta;
        const double lo[3] = {mesh->origin[0], mesh->origin[1], mesh->origin[2]};
        const double hi[3] = {mesh->origin[0] + (double)mesh->nx * mesh->h[0],
                              mesh->origin[1] + (double)mesh->ny * mesh->h[1],
                              mesh->origin[2] + (double)mesh->nz * mesh->h[2]};
        if (delta > 0) {
            const double gx = std::ceil((hi[0] - lo[0]) * dINV), gy = std::ceil((hi[1] - lo[1]) * dINV),
                         gz = std::ceil((hi[2] - lo[2]) * dINV);
            if (gx * gy * gz > (double)(1 << 26)) { ctx->err = "collision grid too fine"; return bail(SDFIBM_ERR_CAPACITY); }
            if (gx > 0 && gy > 0 && gz > 0) {
                ctx->grid_active = true;
                GridK& g = ctx->gk;
                for (int a = 0; a < 3; ++a) g.low[a] = lo[a];
                g.dINV = dINV;
                g.nx = (int)gx; g.ny = (int)gy; g.nz = (int)gz;
                g.nynz = g.ny * g.nz;
                g.ncell = (int64_t)g.nx * g.ny * g.nz;
                // fine grid: about 8 cells per sphere-like solid over the same box
                std::vector<int32_t> planes;
                int64_t nsph = 0;
                for (int s = 0; s < nsolids; ++s) {
                    const bool infinite = ctx->hk[s].infinite != 0;
                    const int id = ctx->opt.collision_mode == SDFIBM_COLLISION_SPHERES ? (infinite ? 0 : 2)
                                                                                      : ctx->hk[s].collision_id;
                    if (id == 0) planes.push_back(s);
                    else if (id == 1 || id == 2) ++nsph;
                }
                ctx->nplanes = (int)planes.size();
                FineGridK& f = ctx->fg;
                const double vol = (hi[0] - lo[0]) * (hi[1] - lo[1]) * (hi[2] - lo[2]);
                double c = std::cbrt(vol / (8.0 * (double)std::max<int64_t>(1, nsph)));
                for (;;) {
                    int64_t nc = 1;
                    for (int a = 0; a < 3; ++a) {
                        f.n[a] = (int32_t)std::max(1.0, std::ceil((hi[a] - lo[a]) / c));
                        nc *= f.n[a];
                    }
                    if (nc <= (1 << 22)) { f.ncell = nc; break; }
                    c *= 1.25;
                }
                for (int a = 0; a < 3; ++a) f.low[a] = lo[a];
                f.inv = 1.0 / c;
                int64_t cap = 0;
                for (int s = 0; s < nsolids; ++s) {
                    const bool infinite = ctx->hk[s].infinite != 0;
                    const int id = ctx->opt.collision_mode == SDFIBM_COLLISION_SPHERES ? (infinite ? 0 : 2)
                                                                                      : ctx->hk[s].collision_id;
                    if (id != 1 && id != 2) continue;
                    const double span = 2.0 * std::max(0.0, solids[s].shape.radiusB) * f.inv + 2.0;
                    int64_t e = 1;
                    for (int a = 0; a < 3; ++a) e *= std::min<int64_t>(f.n[a], (int64_t)span);
                    cap += e;
                }
                f.cap = std::max<int64_t>(1, cap);
                if (dalloc(&ctx->d_planes, planes.size()) ||
                    (planes.size() && cudaMemcpy(ctx->d_planes, planes.data(), sizeof(int32_t) * planes.size(),
                                                 cudaMemcpyHostToDevice) != cudaSuccess) ||
                    dalloc(&ctx->d_fcount, f.ncell) || dalloc(&ctx->d_fstart, f.ncell + 1) ||
                    dalloc(&ctx->d_fcursor, f.ncell) || dalloc(&ctx->d_flist, f.cap)) {
                    ctx->err = "device allocation failed (fine collision grid)";
                    return bail(SDFIBM_ERR_CUDA);
                }
            }
        }
    }

    // device allocations; REF-GEO and SUBSAMPLE list their cut cells (one entry per bbox cell at most)
    const bool cell_list = ctx->opt.fraction_method == SDFIBM_FRACTION_SUBSAMPLE ||
                           ctx->opt.fraction_method == SDFIBM_FRACTION_REFGEO;
    if (cell_list) ctx->feat_cap = std::max<int64_t>(1, scratch);
    if (dalloc(&ctx->d_sk, nsolids) || dalloc(&ctx->d_st, nsolids) || dalloc(&ctx->d_plan, nsolids) ||
        dalloc(&ctx->d_chunks, (size_t)ctx->total_tiles) || dalloc(&ctx->d_scratch, scratch) || dalloc(&ctx->d_alpha, scratch) ||
        dalloc(&ctx->d_gbitmaps, gwords) || dalloc(&ctx->d_lists[0][0], ctx->cap) || dalloc(&ctx->d_lists[0][1], ctx->cap) ||
        dalloc(&ctx->d_lists[0][2], ctx->cap) || dalloc(&ctx->d_lists[0][3], ctx->cap) ||
        dalloc(&ctx->d_lists[1][0], ctx->cap) || dalloc(&ctx->d_lists[1][1], ctx->cap) ||
        dalloc(&ctx->d_lists[1][2], ctx->cap) || dalloc(&ctx->d_lists[1][3], ctx->cap) || dalloc(&ctx->d_cnt, 1) ||
        dalloc(&ctx->d_ftacc, 6 * (size_t)nsolids) || dalloc(&ctx->d_ft, 6 * (size_t)nsolids) ||
        dalloc(&ctx->d_sh_keys, (size_t)ctx->sh_mask + 1) || dalloc(&ctx->d_sh_vals, 5 * ((size_t)ctx->sh_mask + 1)) ||
        dalloc(&ctx->d_sh_used, (size_t)ctx->sh_mask + 1) || dalloc(&ctx->d_step, 2) ||
        dalloc(&ctx->d_cbits, (size_t)(ctx->mesh.ncells + 255) / 256) ||
        dalloc(&ctx->d_sbits, (size_t)(ctx->mesh.ncells + 255) / 256) || dalloc(&ctx->d_shent, (size_t)ctx->shent_cap) ||
        dalloc(&ctx->d_small, small_solids.size()) || dalloc(&ctx->d_big, big_solids.size()) ||
        dalloc(&ctx->d_rq, (size_t)ctx->rq_cap) || dalloc(&ctx->d_ovf, (size_t)ctx->ovf_cap) ||
        (cell_list &&
         (dalloc(&ctx->d_fref_solid, (size_t)ctx->feat_cap) || dalloc(&ctx->d_fref_index, (size_t)ctx->feat_cap))) ||
        (ctx->opt.fraction_method == SDFIBM_FRACTION_REFGEO && dalloc(&ctx->d_rg_phi, 8 * (size_t)ctx->feat_cap)) ||
        cudaMallocHost((void**)&ctx->h_cnt, sizeof(Counters)) != cudaSuccess ||
        cudaMallocHost((void**)&ctx->h_ft, std::max<size_t>(1, 6 * (size_t)nsolids) * sizeof(double)) != cudaSuccess) {
        ctx->err = "device allocation failed";
        return bail(SDFIBM_ERR_CUDA);
    }
    if (ctx->grid_active) {
        if (dalloc(&ctx->d_hash, nsolids) || dalloc(&ctx->d_recs, nsolids) || dalloc(&ctx->d_gcount, ctx->gk.ncell) ||
            dalloc(&ctx->d_gstart, ctx->gk.ncell + 1) || dalloc(&ctx->d_gcursor, ctx->gk.ncell) ||
            dalloc(&ctx->d_glist, nsolids) ||
            dalloc(&ctx->d_fsums, std::max(ctx->gk.ncell, ctx->fg.ncell) / 1024 + 2) ||
            dalloc(&ctx->d_fsums_excl, std::max(ctx->gk.ncell, ctx->fg.ncell) / 1024 + 2)) {
            ctx->err = "device allocation failed (collision grid)";
            return bail(SDFIBM_ERR_CUDA);
        }
    }
    std::vector<sdfibm_solid_state> st(nsolids);
    for (int s = 0; s < nsolids; ++s) {
        sdfibm_solid_state& x = st[s];
        std::memset(&x, 0, sizeof(x));
        for (int a = 0; a < 3; ++a) { x.pos[a] = solids[s].pos[a]; x.vel[a] = solids[s].vel[a]; x.omega[a] = solids[s].omega[a]; }
        for (int a = 0; a < 4; ++a) x.quat[a] = solids[s].quat[a];
        x.first_fluid_step = 1;
        x.first_forcer_step = 1;
    }
    sdfibm_ctx* c = ctx;
    auto up = [&](void* dst, const void* src, size_t bytes) {
        return bytes ? cudaMemcpy(dst, src, bytes, cudaMemcpyHostToDevice) : cudaSuccess;
    };
    if (up(c->d_sk, c->hk.data(), sizeof(SolidK) * nsolids) || up(c->d_st, st.data(), sizeof(sdfibm_solid_state) * nsolids) ||
        up(c->d_chunks, chunks.data(), sizeof(int2) * chunks.size()) ||
        up(c->d_small, small_solids.data(), sizeof(int32_t) * small_solids.size()) ||
        up(c->d_big, big_solids.data(), sizeof(int32_t) * big_solids.size()) ||
        cudaMemset(c->d_cnt, 0, sizeof(Counters)) != cudaSuccess ||
        cudaMemset(c->d_sh_keys, 0xff, sizeof(int32_t) * ((size_t)c->sh_mask + 1)) != cudaSuccess ||
        cudaMemset(c->d_sh_vals, 0, sizeof(double) * 5 * ((size_t)c->sh_mask + 1)) != cudaSuccess ||
        cudaMemset(c->d_cbits, 0, sizeof(uint32_t) * ((size_t)(c->mesh.ncells + 255) / 256)) != cudaSuccess ||
        cudaMemset(c->d_sbits, 0, sizeof(uint32_t) * ((size_t)(c->mesh.ncells + 255) / 256)) != cudaSuccess ||
        up(&c->d_cnt->list_cap, &c->cap, sizeof(int64_t))) {
        ctx->err = "upload failed";
        return bail(SDFIBM_ERR_CUDA);
    }
    if (ctx->connect_smem_bytes > 48 * 1024) {
        if (cudaFuncSetAttribute(connect_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 ctx->connect_smem_bytes) != cudaSuccess) {
            ctx->err = "cannot reserve shared memory for the flood fill";
            return bail(SDFIBM_ERR_CUDA);
        }
    }
    int occ = 0;
    occ = classify_occupancy(ctx->opt.fraction_method, mesh->nz <= 2);
    ctx->classify_grid = std::max(1, occ) * ctx->num_sms;
    ctx->classify_occ = std::max(1, occ);
    occ = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, couple_chunks_kernel, 256, 0);
    ctx->couple_grid = std::max(1, occ) * ctx->num_sms;
    ctx->couple_occ = std::max(1, occ);
    ctx->subsample_grid = 8 * ctx->num_sms;
    ctx->mlp_grid = 5 * ctx->num_sms;  // mlp_infer_kernel: five CTAs per SM (shared memory, tensor memory, registers)
    ctx->refgeo_grid = 8 * ctx->num_sms;
    occ = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, learned_stencil_kernel, stencil_block(), 0);
    ctx->stencil_grid = std::max(1, occ) * ctx->num_sms;  // persistent: every resident CTA, grid-strided
    *out = ctx;
    return SDFIBM_OK;
}

static int check_device_error(sdfibm_ctx* ctx) {
    const int e = ctx->h_cnt->error;
    if (e == DERR_NONE) return SDFIBM_OK;
    cudaMemsetAsync(&ctx->d_cnt->error, 0, sizeof(int32_t), ctx->stream);
    switch (e) {
        case DERR_CAPACITY: return fail(ctx, SDFIBM_ERR_CAPACITY, "touched-cell list capacity exceeded");
        case DERR_BBOX: return fail(ctx, SDFIBM_ERR_CAPACITY, "a 2-D shape tilted out of its reserved bounding box");
        case DERR_FLOOD_LIMIT: return fail(ctx, SDFIBM_ERR_TIMEOUT, "flood fill did not converge within its bound");
        case DERR_SHARED_TABLE: return fail(ctx, SDFIBM_ERR_CAPACITY, "shared-cell table full");
        case DERR_MMA_TIMEOUT: return fail(ctx, SDFIBM_ERR_TIMEOUT, "learned fraction: tensor-core wait timed out");
        default: return fail(ctx, SDFIBM_ERR_CUDA, "device error " + std::to_string(e));
    }
}

static int sync_counters(sdfibm_ctx* ctx) {
    CK(cudaMemcpyAsync(ctx->h_cnt, ctx->d_cnt, sizeof(Counters), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return check_device_error(ctx);
}

// The device work of one interact on the context's stream: what a captured graph holds.
static int enqueue_interact(sdfibm_ctx* ctx, double time, double dt, const float* U, float* As, float* Fs, float* Ts,
                            int32_t* Ct, bool dense, int& launches) {
    const int64_t N = ctx->mesh.ncells;
    const int S = ctx->S;
    cudaStream_t st = ctx->stream;
    set_step_kernel<<<1, 1, 0, st>>>(ctx->d_step, time, dt, 1, ctx->opt.rho_f * ctx->mesh.V);
    ++launches;
    begin_kernel<<<1, 1, 0, st>>>(ctx->d_cnt);
    ++launches;
    if (dense) {
        // SolidCloud::interact zeroes the four fields over the whole mesh (solidcloud.cpp:438-441)
        CK(cudaMemsetAsync(As, 0, sizeof(float) * N, st));
        CK(cudaMemsetAsync(Fs, 0, sizeof(float) * 3 * N, st));
        CK(cudaMemsetAsync(Ts, 0, sizeof(float) * N, st));
        CK(cudaMemsetAsync(Ct, 0, sizeof(int32_t) * N, st));
        mark(ctx, "dense_reset");
    }
    if (S > 0) {
        CK(cudaMemsetAsync(ctx->d_ftacc, 0, sizeof(double) * 6 * S, st));
        // chunk marks of this call's claims (they stay after the call for sdfibm_cuda_apply_forcing)
        CK(cudaMemsetAsync(ctx->d_cbits, 0, sizeof(uint32_t) * (size_t)((N + 255) / 256), st));
        CK(cudaMemsetAsync(ctx->d_sbits, 0, sizeof(uint32_t) * (size_t)((N + 255) / 256), st));
        plan_kernel<<<(S + 127) / 128, 128, 0, st>>>(ctx->mesh, ctx->d_sk, ctx->d_st, ctx->d_plan, S, ctx->d_cnt);
        mark(ctx, "plan_kernel");
        ClassifyArgs CA{};
        CA.m = ctx->mesh; CA.sk = ctx->d_sk; CA.st = ctx->d_st; CA.plan = ctx->d_plan; CA.chunks = ctx->d_chunks;
        CA.total_chunks = ctx->total_chunks; CA.cls = ctx->d_scratch; CA.alpha = ctx->d_alpha; CA.cnt = ctx->d_cnt;
        CA.chunk_tiles = ctx->chunk_tiles;
        CA.method = ctx->opt.fraction_method; CA.subsample_n = ctx->opt.subsample_n;
        const bool learned = ctx->opt.fraction_method == SDFIBM_FRACTION_LEARNED;
        const bool subsample = ctx->opt.fraction_method == SDFIBM_FRACTION_SUBSAMPLE;
        const bool refgeo = ctx->opt.fraction_method == SDFIBM_FRACTION_REFGEO;
        if (refgeo) {
            // cut cells and their vertex distances listed by the classify pass, fractions by refgeo_cells_kernel
            CA.feat_cap = ctx->feat_cap; CA.fref_solid = ctx->d_fref_solid; CA.fref_index = ctx->d_fref_index;
            CA.rg_phi = ctx->d_rg_phi;
        }
        if (subsample) {
            // cut cells listed by the classify pass, sampled by subsample_cells_kernel
            CA.rq = ctx->d_rq; CA.rq_cap = ctx->rq_cap;
            CA.feat_cap = ctx->feat_cap; CA.fref_solid = ctx->d_fref_solid; CA.fref_index = ctx->d_fref_index;
        }
        if (learned) {
            // cut cells listed by the classify pass; learned_stencil_kernel computes the model's inputs (the cells of
            // solids under rho_min cells, listed from the back, go to the fallback whole)
            CA.feat_cap = ctx->feat_cap; CA.fref_solid = ctx->d_fref_solid; CA.fref_index = ctx->d_fref_index;
            CA.rho_min = ctx->rho_min;
        }
        launch_classify(CA, ctx->mesh.nz <= 2, ctx->classify_grid, st);
        mark(ctx, "classify_kernel");
        // the component pass needs only the class bytes and the seeds: on the side stream, beside the fraction
        // kernels below (one stream while timing, so that every kernel has its own events)
        const bool fork = ctx->side_st != nullptr && !ctx->opt.timing;
        cudaStream_t sb = fork ? ctx->side_st : st;
        if (fork) {
            CK(cudaEventRecord(ctx->ev_fork, st));
            CK(cudaStreamWaitEvent(sb, ctx->ev_fork, 0));
        }
        if (ctx->n_small > 0)
            connect_small_kernel<<<(ctx->n_small + 7) / 8, 256, 0, sb>>>(
                ctx->mesh, ctx->d_sk, ctx->d_plan, ctx->d_scratch, ctx->in_cell(), ctx->in_solid(), ctx->cut_cell(),
                ctx->cut_solid(), ctx->cap, ctx->cap, ctx->d_cnt, ctx->d_small, ctx->n_small);
        if (ctx->n_big > 0)
            connect_kernel<<<ctx->n_big, 512, ctx->connect_smem_bytes, sb>>>(
                ctx->mesh, ctx->d_sk, ctx->d_plan, ctx->d_scratch, ctx->d_gbitmaps, ctx->in_cell(), ctx->in_solid(),
                ctx->cut_cell(), ctx->cut_solid(), ctx->cap, ctx->cap, ctx->d_cnt, ctx->connect_smem_bytes / 4,
                ctx->d_big);
        mark(ctx, "connect_kernel");
        claim_kernel<<<ctx->num_sms * 8, 256, 0, sb>>>(ctx->in_cell(), ctx->in_solid(), ctx->cut_cell(),
                                                        ctx->cut_solid(), Ct, ctx->d_cnt, N, ctx->d_cbits,
                                                        ctx->d_sbits);
        mark(ctx, "claim_kernel");
        shared_scan_kernel<<<ctx->num_sms * 8, 256, 0, sb>>>(ctx->in_cell(), ctx->cut_cell(), Ct, ctx->d_cnt, N,
                                                              ctx->d_sbits, ctx->d_shent, ctx->shent_cap);
        mark(ctx, "shared_scan_kernel");
        launches += 5;
        if (ctx->u64_dev) {  // interact_host64: U read at the coupling cells from the page-locked FP64 field
            gather_u64_kernel<<<ctx->num_sms * 8, 256, 0, sb>>>(ctx->in_cell(), ctx->cut_cell(), ctx->d_cnt, N,
                                                                 ctx->u64_dev, const_cast<float*>(U));
            mark(ctx, "gather_u64_kernel");
            ++launches;
        }
        if (!dense) {
            const int p = ctx->cur ^ 1;
            reset_kernel<<<ctx->num_sms * 4, 256, 0, sb>>>(ctx->d_lists[p][0], ctx->d_lists[p][2], ctx->d_cnt, N, As,
                                                            Fs, Ts, Ct, ctx->d_cbits);
            mark(ctx, "reset_kernel");
            ++launches;
        }
        if (refgeo) {
            refgeo_cells_kernel<<<ctx->refgeo_grid, 256, 0, st>>>(ctx->mesh, ctx->d_sk, ctx->d_plan,
                                                                   ctx->d_fref_solid, ctx->d_fref_index,
                                                                   ctx->d_rg_phi, ctx->feat_cap, ctx->d_cnt,
                                                                   ctx->d_alpha);
            mark(ctx, "refgeo_cells_kernel");
            ++launches;
        }
        FallbackArgs fa{};
        if (learned) {
            // model inputs and band of every cut cell, the network on the cells inside the band, SUBSAMPLE on the
            // others
            StencilArgs sa{};
            sa.m = ctx->mesh; sa.sk = ctx->d_sk; sa.plan = ctx->d_plan; sa.fref_solid = ctx->d_fref_solid;
            sa.fref_index = ctx->d_fref_index; sa.cap = ctx->feat_cap; sa.feat = ctx->d_feat; sa.fb_list = ctx->d_fb;
            sa.mlp_index = ctx->d_mlp_index;
            sa.cnt = ctx->d_cnt; sa.tau_refine = ctx->tau_refine;
            learned_stencil_kernel<<<ctx->stencil_grid, stencil_block(), 0, st>>>(sa);
            mark(ctx, "learned_stencil_kernel");
            ++launches;
            MlpInferArgs ia{};
            ia.params = ctx->d_mlp; ia.feat = ctx->d_feat; ia.stride = ctx->feat_cap; ia.n_dev = &ctx->d_cnt->n_inband;
            ia.ref_index = ctx->d_mlp_index; ia.alpha = ctx->d_alpha; ia.error = &ctx->d_cnt->error;
            launch_mlp_infer(ia, ctx->mlp_grid, st);
            mark(ctx, "mlp_infer_kernel");
            fa.m = ctx->mesh; fa.sk = ctx->d_sk; fa.st = ctx->d_st; fa.plan = ctx->d_plan; fa.fb_list = ctx->d_fb;
            fa.fref_solid = ctx->d_fref_solid; fa.fref_index = ctx->d_fref_index; fa.cap = ctx->feat_cap;
            fa.alpha = ctx->d_alpha; fa.cnt = ctx->d_cnt;
            fa.n = ctx->opt.learned_fallback_n > 0 ? ctx->opt.learned_fallback_n : 16;
            fa.rq = ctx->d_rq; fa.rq_cap = ctx->rq_cap;
            fa.ovf = ctx->d_ovf; fa.ovf_cap = ctx->ovf_cap;
            subsample_cells_kernel<<<ctx->subsample_grid, 256, 0, st>>>(fa);
            mark(ctx, "subsample_cells_kernel");
            launches += 2;
        } else if (subsample) {
            fa.m = ctx->mesh; fa.sk = ctx->d_sk; fa.st = ctx->d_st; fa.plan = ctx->d_plan; fa.fb_list = nullptr;
            fa.fref_solid = ctx->d_fref_solid; fa.fref_index = ctx->d_fref_index; fa.cap = ctx->feat_cap;
            fa.alpha = ctx->d_alpha; fa.cnt = ctx->d_cnt;
            fa.n = ctx->opt.subsample_n;
            fa.rq = ctx->d_rq; fa.rq_cap = ctx->rq_cap;
            fa.ovf = ctx->d_ovf; fa.ovf_cap = ctx->ovf_cap;
            subsample_cells_kernel<<<ctx->subsample_grid, 256, 0, st>>>(fa);
            mark(ctx, "subsample_cells_kernel");
            ++launches;
        }
        if (learned || subsample) {
            recheck_kernel<<<ctx->num_sms * 4, 256, 0, st>>>(ctx->mesh, ctx->d_sk, ctx->d_st, ctx->d_plan, ctx->d_rq,
                                                              ctx->rq_cap, ctx->d_cnt, ctx->d_alpha);
            mark(ctx, "recheck_kernel");
            ++launches;
        }
        if (learned || subsample) {
            recount_kernel<<<ctx->num_sms * 2, 256, 0, st>>>(fa);
            mark(ctx, "recount_kernel");
            ++launches;
        }
        if (fork) {
            CK(cudaEventRecord(ctx->ev_join, sb));
            CK(cudaStreamWaitEvent(st, ctx->ev_join, 0));
        }
    } else if (!dense) {
        const int p = ctx->cur ^ 1;
        reset_kernel<<<ctx->num_sms * 4, 256, 0, st>>>(ctx->d_lists[p][0], ctx->d_lists[p][2], ctx->d_cnt, N, As, Fs,
                                                        Ts, Ct, ctx->d_cbits);
        ++launches;
    }
    if (ctx->u_wait) {  // U staged on a copy stream (interact_host)
        if (ctx->u_probe) CK(cudaEventRecord(ctx->ev_tpre, st));
        CK(cudaStreamWaitEvent(st, ctx->u_wait, 0));
    }
    if (S > 0) {
        CoupleArgs A{};
        A.m = ctx->mesh; A.sk = ctx->d_sk; A.st = ctx->d_st; A.plan = ctx->d_plan;
        A.in_cell = ctx->in_cell(); A.in_solid = ctx->in_solid(); A.cut_cell = ctx->cut_cell();
        A.cut_solid = ctx->cut_solid(); A.alpha = ctx->d_alpha; A.U = U; A.As = As; A.Fs = Fs; A.Ts = Ts; A.Ct = Ct;
        A.ftacc = ctx->d_ftacc; A.cnt = ctx->d_cnt; A.step = ctx->d_step;
        A.method = ctx->opt.fraction_method; A.subsample_n = ctx->opt.subsample_n;
        A.exact_forcing = ctx->opt.exact_forcing;
        {
            const int nc = ctx->opt.fraction_method == SDFIBM_FRACTION_LEARNED
                               ? (ctx->opt.learned_fallback_n > 0 ? ctx->opt.learned_fallback_n : 16)
                               : ctx->opt.subsample_n;
            A.count_samples = nc * nc * (ctx->mesh.twod ? 1 : nc);
        }
        A.sh_keys = ctx->d_sh_keys; A.sh_vals = ctx->d_sh_vals; A.sh_used = ctx->d_sh_used; A.sh_mask = ctx->sh_mask;
        A.cbits = ctx->d_cbits; A.sbits = ctx->d_sbits; A.shent = ctx->d_shent; A.shent_cap = ctx->shent_cap;
        // the compacted entries on shared cells (their FP64 sums), then every cell of the marked chunks
        couple_shared_kernel<<<ctx->num_sms, 256, 0, st>>>(A);
        mark(ctx, "couple_shared_kernel");
        couple_chunks_kernel<<<ctx->couple_grid, 256, 0, st>>>(A);
        mark(ctx, "couple_chunks_kernel");
        finalize_kernel<<<ctx->num_sms, 256, 0, st>>>(As, Ts, Fs, Ct, ctx->d_cnt, N, ctx->d_sh_keys, ctx->d_sh_vals,
                                                       ctx->d_sh_used, ctx->sh_mask);
        mark(ctx, "finalize_kernel");
        ft_kernel<<<(S + 127) / 128, 128, 0, st>>>(ctx->d_ftacc, ctx->d_ft, S, ctx->d_step);
        ft_to_state_kernel<<<(S + 127) / 128, 128, 0, st>>>(ctx->d_ft, ctx->d_st, S);
        mark(ctx, "ft_kernel");
        launches += 5;
    }
    CK(cudaGetLastError());
    return SDFIBM_OK;
}

// Runs `enqueue` as a CUDA graph: captured on first use (or when `key_changed`), then replayed after updating the
// arguments of its set_step_kernel node.  Returns a status, or -1 when capture is not possible (the caller then
// launches directly).
static int run_graph(sdfibm_ctx* ctx, sdfibm_ctx::Graph& g, bool key_changed, const std::function<int()>& enqueue,
                     StepParams* step, double time, double dt, int nsub, double rho_V) {
    cudaStream_t st = ctx->stream;
    if (!g.valid || key_changed) {
        if (g.valid) {
            cudaGraphExecDestroy(g.exec);
            g.valid = false;
        }
        cudaGraph_t graph = nullptr;
        if (cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
            cudaGetLastError();
            return -1;
        }
        const int rc = enqueue();
        const cudaError_t e = cudaStreamEndCapture(st, &graph);
        if (rc != SDFIBM_OK || e != cudaSuccess || !graph) {
            if (graph) cudaGraphDestroy(graph);
            cudaGetLastError();
            return -1;
        }
        size_t n = 0;
        cudaGraphGetNodes(graph, nullptr, &n);
        std::vector<cudaGraphNode_t> nodes(n);
        cudaGraphGetNodes(graph, nodes.data(), &n);
        g.step_node = nullptr;
        for (cudaGraphNode_t nd : nodes) {
            cudaGraphNodeType t;
            if (cudaGraphNodeGetType(nd, &t) != cudaSuccess || t != cudaGraphNodeTypeKernel) continue;
            cudaKernelNodeParams kp;
            if (cudaGraphKernelNodeGetParams(nd, &kp) == cudaSuccess && kp.func == (void*)set_step_kernel) {
                g.step_node = nd;
                g.step_params = kp;
                break;
            }
        }
        if (!g.step_node || cudaGraphInstantiate(&g.exec, graph, 0) != cudaSuccess) {
            cudaGraphDestroy(graph);
            cudaGetLastError();
            return -1;
        }
        // the graph is kept alive: its node handle addresses the instantiated copy
        ctx->graphs_keep.push_back(graph);
        g.valid = true;
    }
    void* args[5] = {&step, &time, &dt, &nsub, &rho_V};
    cudaKernelNodeParams kp = g.step_params;
    kp.kernelParams = args;
    kp.extra = nullptr;
    CK(cudaGraphExecKernelNodeSetParams(g.exec, g.step_node, &kp));
    CK(cudaGraphLaunch(g.exec, st));
    return SDFIBM_OK;
}

static bool graphs_on(const sdfibm_ctx* ctx) {
    return ctx->opt.graphs && ctx->stream != nullptr && !ctx->opt.timing && !ctx->graphs_failed && !ctx->u_wait;
}

static int poly_interact(sdfibm_ctx* ctx, double time, double dt, const float* U, float* As, float* Fs, float* Ts,
                         int32_t* Ct, double* FT);

int sdfibm_cuda_interact(sdfibm_ctx* ctx, double time, double dt, const float* U, float* As, float* Fs, float* Ts,
                         int32_t* Ct, double* FT) {
    if (!ctx) return SDFIBM_ERR_ARG;
    if (!U || !As || !Fs || !Ts || !Ct) return fail(ctx, SDFIBM_ERR_ARG, "null field pointer");
    if (!(dt != 0.0)) return fail(ctx, SDFIBM_ERR_ARG, "dt must be nonzero");
    if (ctx->poly) return poly_interact(ctx, time, dt, U, As, Fs, Ts, Ct, FT);
    const int S = ctx->S;
    cudaStream_t st = ctx->stream;
    int launches = 0;
    mark_begin(ctx);
    const void* f5[5] = {U, As, Fs, Ts, Ct};
    if (As != ctx->d_As) ctx->host_synced = false;  // the touched-cell lists no longer follow the host fields
    bool same = ctx->interacted;
    for (int i = 1; i < 5; ++i) same = same && f5[i] == ctx->last_fields[i];
    const bool dense = !same || ctx->opt.dense_reset;
    if (ctx->opt.fraction_method == SDFIBM_FRACTION_LEARNED && !ctx->model_set)
        return fail(ctx, SDFIBM_ERR_STATE, "LEARNED fraction without a model: call sdfibm_cuda_set_fraction_model");
    for (int i = 0; i < 5; ++i) ctx->last_fields[i] = f5[i];
    ctx->cur ^= 1;  // this call's lists; the other buffer holds the previous call's touched cells
    int rc = -1;
    if (graphs_on(ctx)) {
        sdfibm_ctx::Graph& g = ctx->igraph[ctx->cur * 2 + (dense ? 1 : 0)];
        bool changed = g.cur != ctx->cur || g.dense != (int)dense || g.u64 != ctx->u64_dev;
        for (int i = 0; i < 5; ++i) changed = changed || g.fields[i] != f5[i];
        int counted = 0;
        rc = run_graph(ctx, g, changed,
                       [&] {
                           counted = 0;
                           return enqueue_interact(ctx, time, dt, U, As, Fs, Ts, Ct, dense, counted);
                       },
                       ctx->d_step, time, dt, 1, ctx->opt.rho_f * ctx->mesh.V);
        if (rc == -1) {
            ctx->graphs_failed = true;
        } else {
            g.cur = ctx->cur;
            g.dense = (int)dense;
            g.u64 = ctx->u64_dev;
            for (int i = 0; i < 5; ++i) g.fields[i] = f5[i];
            if (counted) g.launches = counted;
            launches = g.launches;
        }
    }
    if (rc == -1) rc = enqueue_interact(ctx, time, dt, U, As, Fs, Ts, Ct, dense, launches);
    if (rc) return rc;
    ctx->launches_last = launches;
    ctx->interacted = true;
    if (FT) {
        if (S > 0) CK(cudaMemcpyAsync(ctx->h_ft, ctx->d_ft, sizeof(double) * 6 * S, cudaMemcpyDeviceToHost, st));
        const int rs = sync_counters(ctx);
        if (rs) return rs;
        std::memcpy(FT, ctx->h_ft, sizeof(double) * 6 * S);
    }
    return SDFIBM_OK;
}

// device address of a page-locked host buffer (nullptr for any other memory)
static void* mapped_host(const void* p) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

static int64_t dirty_words(int64_t N) {
    // one bit per chunk of export_chunk_cells() cells, 32 chunks per word
    return (N + 32 * (int64_t)export_chunk_cells() - 1) / (32 * (int64_t)export_chunk_cells());
}

// device copies of the four result fields and of U for the host-buffer entry points
static int ensure_staging(sdfibm_ctx* ctx) {
    const int64_t N = ctx->mesh.ncells;
    if (!ctx->d_U && dalloc(&ctx->d_U, 3 * N)) return fail(ctx, SDFIBM_ERR_CUDA, "staging allocation failed");
    if (!ctx->d_As) {
        const int64_t words = dirty_words(N);
        if (dalloc(&ctx->d_As, N) || dalloc(&ctx->d_Fs, 3 * N) || dalloc(&ctx->d_Ts, N) || dalloc(&ctx->d_Ct, N) ||
            dalloc(&ctx->d_dirty, words) ||
            cudaMemsetAsync(ctx->d_dirty, 0, sizeof(uint32_t) * words, ctx->stream) != cudaSuccess)
            return fail(ctx, SDFIBM_ERR_CUDA, "staging allocation failed");
    }
    return SDFIBM_OK;
}

static int poly_interact_host(sdfibm_ctx* ctx, double time, double dt, const void* U, void* As, void* Fs, void* Ts,
                              void* Ct, double* FT, bool f64);

int sdfibm_cuda_interact_host64(sdfibm_ctx* ctx, double time, double dt, const double* U, double* As, double* Fs,
                                double* Ts, double* Ct, double* FT) {
    if (!ctx) return SDFIBM_ERR_ARG;
    if (!U || !As || !Fs || !Ts || !Ct) return fail(ctx, SDFIBM_ERR_ARG, "null field pointer");
    if (ctx->poly) return poly_interact_host(ctx, time, dt, U, As, Fs, Ts, Ct, FT, true);
    const int64_t N = ctx->mesh.ncells;
    cudaStream_t st = ctx->stream;
    if (int rc = ensure_staging(ctx)) return rc;
    const void* hU = mapped_host(U);
    void* const hp[4] = {mapped_host(As), mapped_host(Fs), mapped_host(Ts), mapped_host(Ct)};
    const void* f5[5] = {U, As, Fs, Ts, Ct};
    ctx->host_synced = false;  // the FP32 host path's buffers no longer follow the device fields
    if (hU && hp[0] && hp[1] && hp[2] && hp[3]) {
        // page-locked: U gathered at the coupling cells, changed chunks written back in place (every chunk on the
        // first call on these buffers, after other buffers, and with dense_reset)
        bool same = ctx->host64_synced && !ctx->opt.dense_reset;
        for (int i = 0; i < 5; ++i) same = same && f5[i] == ctx->host64_fields[i];
        ctx->host64_synced = false;
        ctx->u64_dev = static_cast<const double*>(hU);
        int rc = sdfibm_cuda_interact(ctx, time, dt, ctx->d_U, ctx->d_As, ctx->d_Fs, ctx->d_Ts, ctx->d_Ct, nullptr);
        ctx->u64_dev = nullptr;
        if (rc) return rc;
        CK(cudaMemsetAsync(&ctx->d_cnt->n_export, 0, sizeof(int32_t), st));
        if (same) {
            const int p = ctx->cur ^ 1;
            mark_export_kernel<<<ctx->num_sms * 8, 256, 0, st>>>(ctx->in_cell(), ctx->cut_cell(), ctx->d_lists[p][0],
                                                                  ctx->d_lists[p][2], ctx->d_cnt, N, ctx->d_dirty);
        } else {
            mark_all_kernel<<<ctx->num_sms * 4, 256, 0, st>>>(ctx->d_dirty, dirty_words(N));
        }
        export64_kernel<<<ctx->num_sms * 8, 256, 0, st>>>(
            ctx->d_cnt, N, ctx->d_dirty, ctx->d_As, ctx->d_Fs, ctx->d_Ts, ctx->d_Ct, static_cast<double*>(hp[0]),
            static_cast<double*>(hp[1]), static_cast<double*>(hp[2]), static_cast<double*>(hp[3]));
        CK(cudaGetLastError());
        mark(ctx, "export64_kernel");
        if (ctx->S > 0)
            CK(cudaMemcpyAsync(ctx->h_ft, ctx->d_ft, sizeof(double) * 6 * ctx->S, cudaMemcpyDeviceToHost, st));
        rc = sync_counters(ctx);
        if (rc) return rc;
        const Counters& c = *ctx->h_cnt;
        ctx->host_h2d = 24 * ((int64_t)clamp_len(c.n_inside, c.list_cap) + clamp_len(c.n_cut, c.list_cap));
        ctx->host_d2h = 48 * (int64_t)export_chunk_cells() * c.n_export + 48 * ctx->S;
        ctx->host_sparse = same;
        for (int i = 0; i < 5; ++i) ctx->host64_fields[i] = f5[i];
        ctx->host64_synced = true;
        if (FT) std::memcpy(FT, ctx->h_ft, sizeof(double) * 6 * ctx->S);
        return SDFIBM_OK;
    }
    // other host memory: whole fields staged through a device FP64 buffer
    ctx->host64_synced = false;
    if (!ctx->d_f64 && dalloc(&ctx->d_f64, 9 * N)) return fail(ctx, SDFIBM_ERR_CUDA, "staging allocation failed");
    CK(cudaMemcpyAsync(ctx->d_f64, U, sizeof(double) * 3 * N, cudaMemcpyHostToDevice, st));
    u64_to_planes_kernel<<<ctx->num_sms * 8, 256, 0, st>>>(ctx->d_f64, N, ctx->d_U);
    int rc = sdfibm_cuda_interact(ctx, time, dt, ctx->d_U, ctx->d_As, ctx->d_Fs, ctx->d_Ts, ctx->d_Ct, nullptr);
    if (rc) return rc;
    double* out = ctx->d_f64 + 3 * N;
    fields_to_f64_kernel<<<ctx->num_sms * 8, 256, 0, st>>>(N, ctx->d_As, ctx->d_Fs, ctx->d_Ts, ctx->d_Ct, out);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(As, out, sizeof(double) * N, cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(Fs, out + N, sizeof(double) * 3 * N, cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(Ts, out + 4 * N, sizeof(double) * N, cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(Ct, out + 5 * N, sizeof(double) * N, cudaMemcpyDeviceToHost, st));
    if (ctx->S > 0) CK(cudaMemcpyAsync(ctx->h_ft, ctx->d_ft, sizeof(double) * 6 * ctx->S, cudaMemcpyDeviceToHost, st));
    rc = sync_counters(ctx);
    if (rc) return rc;
    ctx->host_h2d = 24 * N;
    ctx->host_d2h = 48 * N + 48 * ctx->S;
    ctx->host_sparse = false;
    if (FT) std::memcpy(FT, ctx->h_ft, sizeof(double) * 6 * ctx->S);
    return SDFIBM_OK;
}

int sdfibm_cuda_interact_host(sdfibm_ctx* ctx, double time, double dt, const float* U, float* As, float* Fs,
                              float* Ts, int32_t* Ct, double* FT) {
    if (!ctx) return SDFIBM_ERR_ARG;
    if (!U || !As || !Fs || !Ts || !Ct) return fail(ctx, SDFIBM_ERR_ARG, "null field pointer");
    if (ctx->poly) return poly_interact_host(ctx, time, dt, U, As, Fs, Ts, Ct, FT, false);
    const int64_t N = ctx->mesh.ncells;
    cudaStream_t st = ctx->stream;
    if (int rc = ensure_staging(ctx)) return rc;
    if (!ctx->ev_u) {
        for (auto& c : ctx->copy_st) CK(cudaStreamCreateWithFlags(&c, cudaStreamNonBlocking));
        CK(cudaEventCreateWithFlags(&ctx->ev_entry, cudaEventDisableTiming));
        CK(cudaEventCreateWithFlags(&ctx->ev_u, cudaEventDisableTiming));
        CK(cudaEventCreateWithFlags(&ctx->ev_done, cudaEventDisableTiming));
        CK(cudaEventCreate(&ctx->ev_t0));
        CK(cudaEventCreate(&ctx->ev_tu));
        CK(cudaEventCreate(&ctx->ev_tpre));
    }
    // U: REF-GEO's enumeration and fraction kernels take less time than copying the whole field in, so a page-locked
    // U is read in place by the coupling kernel (only at the coupling cells); otherwise U is copied in on a second
    // stream while those kernels run (once the previous work, which may still read d_U, is done) and the coupling
    // kernel waits for it
    const void* u_host =
        ctx->opt.fraction_method == SDFIBM_FRACTION_REFGEO || ctx->u_in_place ? mapped_host(U) : nullptr;
    ctx->u_probe = !u_host;
    if (!u_host) {
        CK(cudaEventRecord(ctx->ev_entry, st));
        CK(cudaEventRecord(ctx->ev_t0, st));
        CK(cudaStreamWaitEvent(ctx->copy_st[0], ctx->ev_entry, 0));
        CK(cudaMemcpyAsync(ctx->d_U, U, sizeof(float) * 3 * N, cudaMemcpyHostToDevice, ctx->copy_st[0]));
        CK(cudaEventRecord(ctx->ev_u, ctx->copy_st[0]));
        CK(cudaEventRecord(ctx->ev_tu, ctx->copy_st[0]));
    }
    // after the call: a copy that outlasted the kernels before the coupling by more than the in-place reads cost
    // there (about 1 ms at 512^3), twice in a row, switches a page-locked U to in-place reads
    auto assess_u_copy = [&]() {
        if (!ctx->u_probe) return;
        ctx->u_probe = false;
        float t_copy = 0.f, t_pre = 0.f;
        if (cudaEventElapsedTime(&t_copy, ctx->ev_t0, ctx->ev_tu) != cudaSuccess ||
            cudaEventElapsedTime(&t_pre, ctx->ev_t0, ctx->ev_tpre) != cudaSuccess) {
            cudaGetLastError();
            return;
        }
        ctx->u_slow = t_copy > t_pre + 1.0f ? ctx->u_slow + 1 : 0;
        if (ctx->u_slow >= 2 && mapped_host(U)) ctx->u_in_place = true;
    };
    // page-locked host fields take the cells that changed since the previous call, written in place (all of them on
    // the first call, after a change of buffers, and with dense_reset); other memory gets whole-field copies
    void* const hp[4] = {mapped_host(As), mapped_host(Fs), mapped_host(Ts), mapped_host(Ct)};
    ctx->host64_synced = false;  // the FP64 host path's buffers no longer follow the device fields
    if (hp[0] && hp[1] && hp[2] && hp[3]) {
        const void* f5[5] = {U, As, Fs, Ts, Ct};
        bool same = ctx->host_synced && !ctx->opt.dense_reset;
        for (int i = 0; i < 5; ++i) same = same && f5[i] == ctx->host_fields[i];
        ctx->host_synced = false;
        ctx->u_wait = u_host ? nullptr : ctx->ev_u;
        int rc = sdfibm_cuda_interact(ctx, time, dt, u_host ? static_cast<const float*>(u_host) : ctx->d_U, ctx->d_As,
                                      ctx->d_Fs, ctx->d_Ts, ctx->d_Ct, nullptr);
        ctx->u_wait = nullptr;
        if (rc) return rc;
        if (same) {
            const int p = ctx->cur ^ 1;
            CK(cudaMemsetAsync(&ctx->d_cnt->n_export, 0, sizeof(int32_t), st));
            mark_export_kernel<<<ctx->num_sms * 8, 256, 0, st>>>(ctx->in_cell(), ctx->cut_cell(), ctx->d_lists[p][0],
                                                                  ctx->d_lists[p][2], ctx->d_cnt, N, ctx->d_dirty);
            export_kernel<<<ctx->num_sms * 8, 256, 0, st>>>(
                ctx->d_cnt, N, ctx->d_dirty, ctx->d_As, ctx->d_Fs, ctx->d_Ts, ctx->d_Ct, static_cast<float*>(hp[0]),
                static_cast<float*>(hp[1]), static_cast<float*>(hp[2]), static_cast<int32_t*>(hp[3]));
            CK(cudaGetLastError());
            mark(ctx, "export_kernel");
        } else {
            CK(cudaMemcpyAsync(As, ctx->d_As, sizeof(float) * N, cudaMemcpyDeviceToHost, st));
            CK(cudaMemcpyAsync(Fs, ctx->d_Fs, sizeof(float) * 3 * N, cudaMemcpyDeviceToHost, st));
            CK(cudaMemcpyAsync(Ts, ctx->d_Ts, sizeof(float) * N, cudaMemcpyDeviceToHost, st));
            CK(cudaMemcpyAsync(Ct, ctx->d_Ct, sizeof(int32_t) * N, cudaMemcpyDeviceToHost, st));
            mark(ctx, "host_copies");
        }
        if (ctx->S > 0)
            CK(cudaMemcpyAsync(ctx->h_ft, ctx->d_ft, sizeof(double) * 6 * ctx->S, cudaMemcpyDeviceToHost, st));
        rc = sync_counters(ctx);
        if (rc) return rc;
        const Counters& c = *ctx->h_cnt;
        ctx->host_h2d = u_host ? 12 * ((int64_t)c.n_inside + c.n_cut) : 12 * N;
        ctx->host_d2h = (same ? 24 * (int64_t)export_chunk_cells() * c.n_export : 24 * N) + 48 * ctx->S;
        ctx->host_sparse = same;
        for (int i = 0; i < 5; ++i) ctx->host_fields[i] = f5[i];
        ctx->host_synced = true;
        assess_u_copy();
        if (FT) std::memcpy(FT, ctx->h_ft, sizeof(double) * 6 * ctx->S);
        return SDFIBM_OK;
    }
    ctx->host_synced = false;
    ctx->u_wait = u_host ? nullptr : ctx->ev_u;
    int rc = sdfibm_cuda_interact(ctx, time, dt, u_host ? static_cast<const float*>(u_host) : ctx->d_U, ctx->d_As,
                                  ctx->d_Fs, ctx->d_Ts, ctx->d_Ct, nullptr);
    ctx->u_wait = nullptr;
    if (rc) return rc;
    CK(cudaEventRecord(ctx->ev_done, st));
    void* dst[4] = {As, Fs, Ts, Ct};
    const void* src[4] = {ctx->d_As, ctx->d_Fs, ctx->d_Ts, ctx->d_Ct};
    const size_t bytes[4] = {sizeof(float) * N, sizeof(float) * 3 * N, sizeof(float) * N, sizeof(int32_t) * N};
    for (int i = 0; i < 4; ++i) {
        CK(cudaStreamWaitEvent(ctx->copy_st[i], ctx->ev_done, 0));
        CK(cudaMemcpyAsync(dst[i], src[i], bytes[i], cudaMemcpyDeviceToHost, ctx->copy_st[i]));
    }
    if (ctx->S > 0) CK(cudaMemcpyAsync(ctx->h_ft, ctx->d_ft, sizeof(double) * 6 * ctx->S, cudaMemcpyDeviceToHost, st));
    rc = sync_counters(ctx);
    for (auto& c : ctx->copy_st) CK(cudaStreamSynchronize(c));
    if (rc) return rc;
    ctx->host_h2d = u_host ? 12 * ((int64_t)ctx->h_cnt->n_inside + ctx->h_cnt->n_cut) : 12 * N;
    ctx->host_d2h = 24 * N + 48 * ctx->S;
    ctx->host_sparse = false;
    assess_u_copy();
    if (FT) std::memcpy(FT, ctx->h_ft, sizeof(double) * 6 * ctx->S);
    return SDFIBM_OK;
}

// Exclusive scan of per-cell counts into start (ncell + 1 entries, the total last) and cursor: one block for small
// grids, else per-1024-cell block scans, one block over their sums, and the block offsets added back.
static void scan_counts(sdfibm_ctx* ctx, int32_t* counts, int32_t* start, int32_t* cursor, int64_t ncell) {
    cudaStream_t st = ctx->stream;
    if (ncell <= 16384) {
        grid_scan_kernel<<<1, 1024, 0, st>>>(counts, start, cursor, ncell);
        return;
    }
    const int64_t nb = (ncell + 1023) / 1024;
    scan_blocks_kernel<<<(unsigned)nb, 1024, 0, st>>>(counts, start, ctx->d_fsums, ncell);
    grid_scan_kernel<<<1, 1024, 0, st>>>(ctx->d_fsums, ctx->d_fsums_excl, ctx->d_fsums_excl, nb);
    scan_add_kernel<<<(unsigned)nb, 1024, 0, st>>>(start, cursor, ctx->d_fsums_excl, ncell, nb);
}

// The device work of one evolve (all sub-steps) on the context's stream: what a captured graph holds.
static int enqueue_evolve(sdfibm_ctx* ctx, double time, double dt) {
    const int S = ctx->S;
    cudaStream_t st = ctx->stream;
    const int nsub = ctx->nsub;
    StepParams* step = ctx->d_step + 1;
    const D3 g{ctx->opt.gravity[0], ctx->opt.gravity[1], ctx->opt.gravity[2]};
    // thread-per-solid kernels are FP64-pipe bound: small blocks spread a few thousand solids over every SM
    const int B = S <= ctx->num_sms * 4 * 64 ? 32 : 128, G = (S + B - 1) / B;
    set_step_kernel<<<1, 1, 0, st>>>(step, time, dt, nsub, 0.0);
    if (!ctx->grid_active) {
        evolve_independent_kernel<<<G, B, 0, st>>>(ctx->d_sk, ctx->d_st, S, nsub, step, ctx->opt.rho_f, g);
    } else {
        const GridK& gk = ctx->gk;
        const FineGridK& fg = ctx->fg;
        const int mode = ctx->opt.collision_mode;
        const int coarse = ctx->nplanes > 0;  // the coarse lists serve only the plane-like solids
        // the scans zero the counts they read, so one clear serves every sub-step; Solid::move of sub-step it - 1
        // runs at the head of sub-step it's force kernel
        if (coarse) CK(cudaMemsetAsync(ctx->d_gcount, 0, sizeof(int32_t) * gk.ncell, st));
        CK(cudaMemsetAsync(ctx->d_fcount, 0, sizeof(int32_t) * fg.ncell, st));
        for (int it = 0; it < nsub; ++it) {
            evolve_pre_kernel<<<G, B, 0, st>>>(ctx->d_sk, ctx->d_st, S, step, ctx->opt.rho_f, g, gk, ctx->d_hash,
                                               ctx->d_gcount, fg, ctx->d_fcount, mode, coarse, ctx->d_recs, it > 0);
            if (coarse) {
                scan_counts(ctx, ctx->d_gcount, ctx->d_gstart, ctx->d_gcursor, gk.ncell);
                grid_scatter_kernel<<<G, B, 0, st>>>(ctx->d_hash, ctx->d_gcursor, ctx->d_glist, S, gk.ncell);
            }
            scan_counts(ctx, ctx->d_fcount, ctx->d_fstart, ctx->d_fcursor, fg.ncell);
            const unsigned GW = (unsigned)(((int64_t)S * 32 + 255) / 256);  // one warp per solid
            fine_scatter_kernel<<<GW, 256, 0, st>>>(ctx->d_recs, S, fg, ctx->d_fcursor, ctx->d_flist, ctx->d_cnt);
            collide_kernel<<<GW, 256, 0, st>>>(
                ctx->d_sk, ctx->d_st, S, gk, ctx->d_hash, ctx->d_gstart, ctx->d_glist, mode, fg, ctx->d_fstart,
                ctx->d_flist, ctx->d_planes, ctx->nplanes, ctx->d_recs);
        }
        move_kernel<<<G, B, 0, st>>>(ctx->d_sk, ctx->d_st, S, step);
        store_old_kernel<<<G, B, 0, st>>>(ctx->d_st, S);
    }
    CK(cudaGetLastError());
    return SDFIBM_OK;
}

int sdfibm_cuda_evolve(sdfibm_ctx* ctx, double time, double dt) {
    if (!ctx) return SDFIBM_ERR_ARG;
    if (ctx->S == 0) return SDFIBM_OK;
    if (graphs_on(ctx)) {
        const int rc = run_graph(ctx, ctx->egraph, false, [&] { return enqueue_evolve(ctx, time, dt); },
                                 ctx->d_step + 1, time, dt, ctx->nsub, 0.0);
        if (rc != -1) return rc;
        ctx->graphs_failed = true;
    }
    return enqueue_evolve(ctx, time, dt);
}

int sdfibm_cuda_fix_internal(sdfibm_ctx* ctx, const int32_t* Ct, float* U) {
    if (!ctx) return SDFIBM_ERR_ARG;
    if (!Ct || !U) return fail(ctx, SDFIBM_ERR_ARG, "null field pointer");
    if (!ctx->interacted) return fail(ctx, SDFIBM_ERR_STATE, "fix_internal needs a previous interact");
    if (ctx->poly) {
        poly_fix_kernel<<<ctx->num_sms * 4, 256, 0, ctx->stream>>>(ctx->poly->k, ctx->d_st, ctx->S, Ct, U);
        CK(cudaGetLastError());
        return SDFIBM_OK;
    }
    fix_internal_kernel<<<ctx->num_sms * 4, 256, 0, ctx->stream>>>(ctx->mesh, ctx->d_st, ctx->in_cell(),
                                                                    ctx->in_solid(), Ct, U, ctx->d_cnt);
    CK(cudaGetLastError());
    return SDFIBM_OK;
}

int sdfibm_cuda_apply_forcing(sdfibm_ctx* ctx, double dt, const float* As, const float* Fs, const float* Ts,
                              float* U, float* T) {
    if (!ctx) return SDFIBM_ERR_ARG;
    if (!As || !Fs || !Ts || !U) return fail(ctx, SDFIBM_ERR_ARG, "null field pointer");
    if (!ctx->interacted) return fail(ctx, SDFIBM_ERR_STATE, "apply_forcing needs a previous interact");
    const uint32_t* marks = nullptr;
    if (!ctx->poly) {
        if (As != ctx->last_fields[1] || Fs != ctx->last_fields[2] || Ts != ctx->last_fields[3])
            return fail(ctx, SDFIBM_ERR_STATE, "apply_forcing takes the fields the last interact wrote");
        marks = ctx->d_cbits;
    }
    const int64_t N = ctx->poly ? ctx->poly->k.ncells : ctx->mesh.ncells;
    apply_forcing_kernel<<<ctx->num_sms * 8, 256, 0, ctx->stream>>>(N, marks, dt, As, Fs, Ts, U, T);
    CK(cudaGetLastError());
    return SDFIBM_OK;
}

int sdfibm_cuda_get_solids(sdfibm_ctx* ctx, sdfibm_solid_state* out, int32_t n) {
    if (!ctx) return SDFIBM_ERR_ARG;
    if (!out || n != ctx->S) return fail(ctx, SDFIBM_ERR_ARG, "state array size must equal the solid count");
    if (n == 0) return SDFIBM_OK;
    CK(cudaMemcpyAsync(out, ctx->d_st, sizeof(sdfibm_solid_state) * n, cudaMemcpyDeviceToHost, ctx->stream));
    return sync_counters(ctx);
}

int sdfibm_cuda_set_solids(sdfibm_ctx* ctx, const sdfibm_solid_state* in, int32_t n) {
    if (!ctx) return SDFIBM_ERR_ARG;
    if (!in || n != ctx->S) return fail(ctx, SDFIBM_ERR_ARG, "state array size must equal the solid count");
    if (n == 0) return SDFIBM_OK;
    CK(cudaMemcpyAsync(ctx->d_st, in, sizeof(sdfibm_solid_state) * n, cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return SDFIBM_OK;
}

int sdfibm_cuda_touched(sdfibm_ctx* ctx, int32_t solid, int64_t* cells, int8_t* types, int64_t capacity, int64_t* n) {
    if (!ctx) return SDFIBM_ERR_ARG;
    if (!n || solid < 0 || solid >= ctx->S) return fail(ctx, SDFIBM_ERR_ARG, "bad solid index");
    if (!ctx->interacted) return fail(ctx, SDFIBM_ERR_STATE, "no interact yet");
    int rc = sync_counters(ctx);
    if (rc) return rc;
    if (ctx->poly) {
        sdfibm_ctx::Poly& P = *ctx->poly;
        int32_t cnt = 0;
        CK(cudaMemcpy(&cnt, P.w.count + solid, sizeof(int32_t), cudaMemcpyDeviceToHost));
        std::vector<int32_t> qc(cnt);
        std::vector<int8_t> qt(cnt);
        if (cnt) {
            CK(cudaMemcpy(qc.data(), P.w.queue + (int64_t)solid * P.w.qcap, sizeof(int32_t) * cnt,
                          cudaMemcpyDeviceToHost));
            CK(cudaMemcpy(qt.data(), P.w.qtype + (int64_t)solid * P.w.qcap, cnt, cudaMemcpyDeviceToHost));
        }
        std::vector<std::pair<int, int32_t>> tc(cnt);
        for (int32_t i = 0; i < cnt; ++i) tc[i] = {qt[i], qc[i]};
        std::sort(tc.begin(), tc.end());
        for (int64_t i = 0; i < cnt; ++i)
            if (i < capacity && cells) { cells[i] = tc[i].second; if (types) types[i] = (int8_t)tc[i].first; }
        *n = cnt;
        return SDFIBM_OK;
    }
    const int nin = clamp_len(ctx->h_cnt->n_inside, ctx->cap), ncut = clamp_len(ctx->h_cnt->n_cut, ctx->cap);
    std::vector<int32_t> ic(nin), is(nin), cc(ncut), cs(ncut);
    if (nin) {
        CK(cudaMemcpy(ic.data(), ctx->in_cell(), sizeof(int32_t) * nin, cudaMemcpyDeviceToHost));
        CK(cudaMemcpy(is.data(), ctx->in_solid(), sizeof(int32_t) * nin, cudaMemcpyDeviceToHost));
    }
    if (ncut) {
        CK(cudaMemcpy(cc.data(), ctx->cut_cell(), sizeof(int32_t) * ncut, cudaMemcpyDeviceToHost));
        CK(cudaMemcpy(cs.data(), ctx->cut_solid(), sizeof(int32_t) * ncut, cudaMemcpyDeviceToHost));
    }
    std::vector<int64_t> byType[4];
    for (int i = 0; i < nin; ++i)
        if ((is[i] & LIST_SOLID_MASK) == solid) byType[1].push_back(ic[i]);
    for (int i = 0; i < ncut; ++i)
        if ((cs[i] & LIST_SOLID_MASK) == solid) {
            const int t = list_type(cs[i]);
            if (t < 1 || t > 3) return fail(ctx, SDFIBM_ERR_STATE, "corrupt touched-cell list entry");
            byType[t].push_back(cc[i]);
        }
    int64_t k = 0;
    for (int t = 1; t <= 3; ++t) {
        std::sort(byType[t].begin(), byType[t].end());
        for (int64_t c : byType[t]) {
            if (k < capacity && cells) { cells[k] = c; if (types) types[k] = (int8_t)t; }
            ++k;
        }
    }
    *n = k;
    return SDFIBM_OK;
}

int sdfibm_cuda_kernel_times(sdfibm_ctx* ctx, const char** names, double* ms, int32_t capacity, int32_t* n) {
    if (!ctx || !n) return SDFIBM_ERR_ARG;
    *n = 0;
    if (!ctx->opt.timing) return fail(ctx, SDFIBM_ERR_STATE, "kernel timing is off (options.timing)");
    CK(cudaStreamSynchronize(ctx->stream));
    for (int i = 0; i < ctx->nev && i < capacity; ++i) {
        float t = 0.f;
        CK(cudaEventElapsedTime(&t, ctx->ev[i], ctx->ev[i + 1]));
        if (names) names[i] = ctx->ev_name[i];
        if (ms) ms[i] = t;
        *n = i + 1;
    }
    return SDFIBM_OK;
}

// Launch configuration chosen by the autotuner, kept per workload shape for the life of the process so that a second
// context of the same shape (a restart, a second solver instance) starts from it without timing again.
struct Tuning {
    int chunk_tiles, classify_grid, subsample_grid, couple_grid, mlp_grid, refgeo_grid;
};
static std::mutex g_tune_mu;
static std::map<std::string, Tuning> g_tune_cache;

static std::string tune_key(const sdfibm_ctx* ctx) {
    char b[256];
    std::snprintf(b, sizeof(b), "%d.%d.%d/%d/%d.%d.%d/%d/%d/%d", ctx->mesh.nx, ctx->mesh.ny, ctx->mesh.nz, ctx->S,
                  ctx->opt.fraction_method, ctx->opt.subsample_n, ctx->opt.learned_fallback_n, ctx->total_tiles,
                  ctx->num_sms, (int)ctx->model_set);
    return b;
}

static int apply_tuning(sdfibm_ctx* ctx, const Tuning& t) {
    std::vector<int2> ch = make_chunks(ctx->hk, t.chunk_tiles);
    if ((int64_t)ch.size() > ctx->chunks_cap) return fail(ctx, SDFIBM_ERR_CAPACITY, "chunk table too small");
    CK(cudaMemcpy(ctx->d_chunks, ch.data(), sizeof(int2) * ch.size(), cudaMemcpyHostToDevice));
    ctx->chunk_tiles = t.chunk_tiles;
    ctx->total_chunks = (int)ch.size();
    ctx->opt.tile_cells = t.chunk_tiles * (ctx->mesh.nz <= 2 ? 8 * 8 * 2 : 4 * 4 * 4);
    ctx->classify_grid = t.classify_grid;
    ctx->subsample_grid = t.subsample_grid;
    ctx->couple_grid = t.couple_grid;
    ctx->mlp_grid = t.mlp_grid;
    ctx->refgeo_grid = t.refgeo_grid;
    for (auto& g : ctx->igraph) g.cur = -1;  // captured graphs hold the old launch shapes: recapture on next use
    return SDFIBM_OK;
}

// per-kernel device times (ms) of the last interact run with timing on
static std::map<std::string, float> last_kernel_ms(sdfibm_ctx* ctx) {
    std::map<std::string, float> r;
    if (cudaStreamSynchronize(ctx->stream) != cudaSuccess) return r;
    for (int i = 0; i < ctx->nev; ++i) {
        float t = 0.f;
        if (cudaEventElapsedTime(&t, ctx->ev[i], ctx->ev[i + 1]) == cudaSuccess) r[ctx->ev_name[i]] += t;
    }
    return r;
}

int sdfibm_cuda_autotune(sdfibm_ctx* ctx, double dt, const float* U, float* As, float* Fs, float* Ts, int32_t* Ct,
                         int32_t* chosen_tiles) {
    if (!ctx) return SDFIBM_ERR_ARG;
    if (!U || !As || !Fs || !Ts || !Ct) return fail(ctx, SDFIBM_ERR_ARG, "null field pointer");
    if (ctx->S == 0) return SDFIBM_OK;
    if (ctx->opt.fraction_method == SDFIBM_FRACTION_LEARNED && !ctx->model_set)
        return fail(ctx, SDFIBM_ERR_STATE, "LEARNED fraction without a model: call sdfibm_cuda_set_fraction_model");
    const std::string key = tune_key(ctx);
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        auto it = g_tune_cache.find(key);
        if (it != g_tune_cache.end()) {
            const int rc = apply_tuning(ctx, it->second);
            if (rc) return rc;
            ctx->tuned_from_cache = true;
            if (chosen_tiles) *chosen_tiles = ctx->chunk_tiles;
            return SDFIBM_OK;
        }
    }
    const int sms = ctx->num_sms;
    // candidates: classify work-item size, then the CTA count of every grid-strided or work-stealing launch (the
    // results do not depend on any of them; each kernel is timed by its own events in the same interacts)
    static const int tiles_cand[] = {2, 4, 8, 16, 32};
    std::vector<int> cls_cand, cpl_cand;
    for (int k = 1; k <= ctx->classify_occ; ++k) cls_cand.push_back(k * sms);
    for (int k = 1; k <= ctx->couple_occ; k *= 2) cpl_cand.push_back(k * sms);
    if (cpl_cand.back() != ctx->couple_occ * sms) cpl_cand.push_back(ctx->couple_occ * sms);
    const std::vector<int> sub_cand = {2 * sms, 4 * sms, 8 * sms, 16 * sms};
    const std::vector<int> mlp_cand = {1 * sms, 2 * sms, 5 * sms, 10 * sms};
    const std::vector<int> rg_cand = {2 * sms, 4 * sms, 8 * sms, 16 * sms};
    const int saved_timing = ctx->opt.timing;
    ctx->opt.timing = 1;
    Tuning best{ctx->chunk_tiles, ctx->classify_grid, ctx->subsample_grid, ctx->couple_grid, ctx->mlp_grid,
                ctx->refgeo_grid};
    int rc = SDFIBM_OK;
    // min over two timed interacts (after one warm-up) of each kernel's time under configuration t
    auto measure = [&](const Tuning& t, std::map<std::string, float>& out) {
        int r = apply_tuning(ctx, t);
        for (int rep = 0; rep < 3 && r == SDFIBM_OK; ++rep) {
            int launches = 0;
            ctx->cur ^= 1;
            mark_begin(ctx);
            r = enqueue_interact(ctx, 0.0, dt, U, As, Fs, Ts, Ct, true, launches);
            if (r) break;
            auto ms = last_kernel_ms(ctx);
            if (rep == 0) continue;
            for (auto& kv : ms) out[kv.first] = out.count(kv.first) ? std::min(out[kv.first], kv.second) : kv.second;
        }
        return r;
    };
    // 1. work-item size of the classify queue (classify time)
    float best_cls = 1e30f;
    for (int tc : tiles_cand) {
        Tuning t = best;
        t.chunk_tiles = tc;
        if ((int64_t)make_chunks(ctx->hk, tc).size() > ctx->chunks_cap) continue;
        std::map<std::string, float> ms;
        if ((rc = measure(t, ms))) break;
        if (ms.count("classify_kernel") && ms["classify_kernel"] < best_cls) {
            best_cls = ms["classify_kernel"];
            best.chunk_tiles = tc;
        }
    }
    // 2. CTA counts: candidate i of every list at once, each kernel keeps its fastest
    struct Knob {
        const char* kernel;
        const std::vector<int>* cand;
        int Tuning::*grid;
    };
    const Knob knobs[5] = {{"classify_kernel", &cls_cand, &Tuning::classify_grid},
                           {"subsample_cells_kernel", &sub_cand, &Tuning::subsample_grid},
                           {"couple_chunks_kernel", &cpl_cand, &Tuning::couple_grid},
                           {"mlp_infer_kernel", &mlp_cand, &Tuning::mlp_grid},
                           {"refgeo_cells_kernel", &rg_cand, &Tuning::refgeo_grid}};
    float bt[5] = {1e30f, 1e30f, 1e30f, 1e30f, 1e30f};
    size_t rounds = 0;
    for (const Knob& kb : knobs) rounds = std::max(rounds, kb.cand->size());
    Tuning chosen = best;
    for (size_t i = 0; i < rounds && rc == SDFIBM_OK; ++i) {
        Tuning t = best;
        for (const Knob& kb : knobs) t.*kb.grid = (*kb.cand)[std::min(i, kb.cand->size() - 1)];
        std::map<std::string, float> ms;
        if ((rc = measure(t, ms))) break;
        for (int k = 0; k < 5; ++k) {
            auto it = ms.find(knobs[k].kernel);
            if (it != ms.end() && it->second < bt[k]) {
                bt[k] = it->second;
                chosen.*knobs[k].grid = t.*knobs[k].grid;
            }
        }
    }
    ctx->opt.timing = saved_timing;
    if (rc != SDFIBM_OK) return rc;
    rc = apply_tuning(ctx, chosen);
    if (rc) return rc;
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        g_tune_cache[key] = chosen;
    }
    ctx->tuned_from_cache = false;
    // the fields hold a complete dense interact of the current state; the next call starts from the same buffers
    ctx->interacted = false;
    if (chosen_tiles) *chosen_tiles = chosen.chunk_tiles;
    return sync_counters(ctx);
}

int sdfibm_cuda_tuning(sdfibm_ctx* ctx, int32_t* out, int32_t n) {
    if (!ctx || !out) return SDFIBM_ERR_ARG;
    const int32_t v[7] = {ctx->chunk_tiles, ctx->classify_grid, ctx->subsample_grid, ctx->couple_grid, ctx->mlp_grid,
                          ctx->refgeo_grid, (int32_t)ctx->tuned_from_cache};
    for (int i = 0; i < n && i < 7; ++i) out[i] = v[i];
    return SDFIBM_OK;
}

int sdfibm_cuda_set_fraction_model(sdfibm_ctx* ctx, const float* params, float tau_refine, float rho_min) {
    if (!ctx) return SDFIBM_ERR_ARG;
    if (!params) return fail(ctx, SDFIBM_ERR_ARG, "null model parameters");
    if (std::isnan(tau_refine) || std::isnan(rho_min)) return fail(ctx, SDFIBM_ERR_ARG, "band limits are NaN");
    for (int i = 0; i < SDFIBM_MLP_NPARAM; ++i)
        if (!std::isfinite(params[i])) return fail(ctx, SDFIBM_ERR_ARG, "non-finite model parameter");
    if (!ctx->d_mlp) {
        // one input record per bbox cell: every cut cell of a call fits
        ctx->feat_cap = std::max<int64_t>(1, ctx->scratch_bytes);
        if (dalloc(&ctx->d_mlp, SDFIBM_MLP_NPARAM) || dalloc(&ctx->d_feat, (size_t)SDFIBM_MLP_NFEAT * ctx->feat_cap) ||
            (!ctx->d_fref_solid && dalloc(&ctx->d_fref_solid, ctx->feat_cap)) ||
            (!ctx->d_fref_index && dalloc(&ctx->d_fref_index, ctx->feat_cap)) || dalloc(&ctx->d_fb, ctx->feat_cap) ||
            dalloc(&ctx->d_mlp_index, ctx->feat_cap))
            return fail(ctx, SDFIBM_ERR_CUDA, "allocation of the learned-fraction buffers failed");
    }
    mlp_prepare();
    CK(cudaMemcpyAsync(ctx->d_mlp, params, sizeof(float) * SDFIBM_MLP_NPARAM, cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    ctx->tau_refine = tau_refine;
    ctx->rho_min = rho_min;
    ctx->model_set = true;
    return SDFIBM_OK;
}

int sdfibm_cuda_stats(sdfibm_ctx* ctx, int64_t* out, int32_t n) {
    if (!ctx || !out) return SDFIBM_ERR_ARG;
    int rc = sync_counters(ctx);
    if (rc) return rc;
    const Counters& c = *ctx->h_cnt;
    if (ctx->poly && ctx->interacted) {
        sdfibm_ctx::Poly& P = *ctx->poly;
        P.counts.resize(std::max(1, ctx->S));
        if (ctx->S) CK(cudaMemcpy(P.counts.data(), P.w.count, sizeof(int32_t) * ctx->S, cudaMemcpyDeviceToHost));
        int64_t tot = 0;
        for (int s = 0; s < ctx->S; ++s) tot += P.counts[s];
        const int64_t v[11] = {tot, 0, (int64_t)P.N * ctx->S, 0, 0, (int64_t)ctx->launches_last, 0, 0, ctx->host_h2d,
                               ctx->host_d2h, 0};
        for (int i = 0; i < n && i < 11; ++i) out[i] = v[i];
        return SDFIBM_OK;
    }
    const int64_t v[11] = {(int64_t)c.n_inside + c.n_cut, (int64_t)c.n_cut, (int64_t)c.bbox_cells,
                           (int64_t)c.exact_rechecks, (int64_t)ctx->total_chunks, (int64_t)ctx->launches_last,
                           (int64_t)c.n_feat + c.n_small, (int64_t)c.n_fb + c.n_small, ctx->host_h2d, ctx->host_d2h,
                           (int64_t)ctx->host_sparse};
    for (int i = 0; i < n && i < 11; ++i) out[i] = v[i];
    return SDFIBM_OK;
}

void sdfibm_cuda_destroy(sdfibm_ctx* ctx) {
    if (!ctx) return;
    cudaStreamSynchronize(ctx->stream);
    void* dev[] = {ctx->d_sk, ctx->d_st, ctx->d_plan, ctx->d_chunks, ctx->d_scratch, ctx->d_gbitmaps,
                   ctx->d_lists[0][0], ctx->d_lists[0][1], ctx->d_lists[0][2], ctx->d_lists[0][3],
                   ctx->d_lists[1][0], ctx->d_lists[1][1], ctx->d_lists[1][2], ctx->d_lists[1][3], ctx->d_cnt, ctx->d_ftacc,
                   ctx->d_ft, ctx->d_hash, ctx->d_gcount, ctx->d_gstart, ctx->d_gcursor, ctx->d_glist, ctx->d_U,
                   ctx->d_As, ctx->d_Fs, ctx->d_Ts, ctx->d_Ct, ctx->d_alpha, ctx->d_sh_keys, ctx->d_sh_vals, ctx->d_sh_used,
                   ctx->d_mlp, ctx->d_feat, ctx->d_rg_phi, ctx->d_fref_solid, ctx->d_fref_index, ctx->d_fb, ctx->d_mlp_index,
                   ctx->d_fcount, ctx->d_fstart, ctx->d_fcursor, ctx->d_flist, ctx->d_planes};
    for (void* p : dev)
        if (p) cudaFree(p);
    if (ctx->d_step) cudaFree(ctx->d_step);
    if (ctx->d_small) cudaFree(ctx->d_small);
    if (ctx->d_rq) cudaFree(ctx->d_rq);
    if (ctx->d_ovf) cudaFree(ctx->d_ovf);
    if (ctx->d_dirty) cudaFree(ctx->d_dirty);
    if (ctx->d_cbits) cudaFree(ctx->d_cbits);
    if (ctx->d_sbits) cudaFree(ctx->d_sbits);
    if (ctx->d_shent) cudaFree(ctx->d_shent);
    if (ctx->d_f64) cudaFree(ctx->d_f64);
    if (ctx->poly) {
        for (void* p : ctx->poly->allocs)
            if (p) cudaFree(p);
        delete ctx->poly;
    }
    if (ctx->d_fsums) cudaFree(ctx->d_fsums);
    if (ctx->d_recs) cudaFree(ctx->d_recs);
    if (ctx->d_fsums_excl) cudaFree(ctx->d_fsums_excl);
    for (auto& c : ctx->copy_st)
        if (c) cudaStreamDestroy(c);
    if (ctx->ev_entry) cudaEventDestroy(ctx->ev_entry);
    if (ctx->ev_u) cudaEventDestroy(ctx->ev_u);
    if (ctx->ev_done) cudaEventDestroy(ctx->ev_done);
    if (ctx->ev_fork) cudaEventDestroy(ctx->ev_fork);
    if (ctx->ev_t0) cudaEventDestroy(ctx->ev_t0);
    if (ctx->ev_tu) cudaEventDestroy(ctx->ev_tu);
    if (ctx->ev_tpre) cudaEventDestroy(ctx->ev_tpre);
    if (ctx->ev_join) cudaEventDestroy(ctx->ev_join);
    if (ctx->side_st) cudaStreamDestroy(ctx->side_st);
    if (ctx->d_big) cudaFree(ctx->d_big);
    for (auto& g : ctx->igraph)
        if (g.valid) cudaGraphExecDestroy(g.exec);
    if (ctx->egraph.valid) cudaGraphExecDestroy(ctx->egraph.exec);
    for (cudaGraph_t gr : ctx->graphs_keep) cudaGraphDestroy(gr);
    if (ctx->ev_ready)
        for (int i = 0; i <= sdfibm_ctx::MAXEV; ++i) cudaEventDestroy(ctx->ev[i]);
    if (ctx->h_cnt) cudaFreeHost(ctx->h_cnt);
    if (ctx->h_ft) cudaFreeHost(ctx->h_ft);
    delete ctx;
}

// ---- explicit polyMesh (unstructured) contexts ------------------------------------------------------------------
int sdfibm_cuda_create_polymesh(const double* points, int64_t npoints, const int32_t* face_off,
                                const int32_t* face_lab, int64_t nfaces, const int32_t* owner,
                                const int32_t* neighbour, int64_t ninternal, int32_t twod,
                                const sdfibm_solid_desc* solids, int32_t nsolids, const sdfibm_options* opt,
                                void* cuda_stream, sdfibm_ctx** out) {
    if (!out) return SDFIBM_ERR_ARG;
    *out = nullptr;
    sdfibm_poly::PolyHostMesh hm;
    std::string err;
    if (!sdfibm_poly::build_polymesh(points, npoints, face_off, face_lab, nfaces, owner, neighbour, ninternal, hm, err))
        return SDFIBM_ERR_ARG;
    sdfibm_options o;
    if (opt) o = *opt; else sdfibm_options_default(&o);
    if (o.fraction_method != SDFIBM_FRACTION_REFGEO) return SDFIBM_ERR_ARG;  // the reference's own fraction only
    o.graphs = 0;
    sdfibm_mesh_desc box{};
    box.nx = box.ny = box.nz = 1;
    box.twod = twod;
    for (int a = 0; a < 3; ++a) {
        box.origin[a] = hm.bmin[a];
        box.h[a] = std::max(hm.bmax[a] - hm.bmin[a], 1e-300);
    }
    int rc = sdfibm_cuda_create(&box, solids, nsolids, &o, cuda_stream, out);
    if (rc) return rc;
    sdfibm_ctx* ctx = *out;
    auto* Pp = new sdfibm_ctx::Poly();
    ctx->poly = Pp;
    sdfibm_ctx::Poly& P = *Pp;
    const int64_t N = hm.ncells;
    P.N = N;
    const int64_t S = std::max(1, nsolids);
    // search lists: every cell of the mesh for every solid, at most 2^28 entries
    if ((double)N * (double)S > (double)(1 << 28)) {
        ctx->err = "polyMesh: cells x solids above the search-list limit (2^28)";
        sdfibm_cuda_destroy(ctx);
        *out = nullptr;
        return SDFIBM_ERR_CAPACITY;
    }
    PolyK& k = P.k;
    k.ncells = (int32_t)N; k.npoints = (int32_t)hm.npoints; k.nfaces = (int32_t)hm.nfaces; k.twod = twod;
    const bool ok_up =
        poly_upload(P, &k.points, hm.points) && poly_upload(P, &k.face_off, hm.face_off) &&
        poly_upload(P, &k.face_lab, hm.face_lab) && poly_upload(P, &k.cf_off, hm.cell_faces_off) &&
        poly_upload(P, &k.cf, hm.cell_faces) && poly_upload(P, &k.cp_off, hm.cell_pts_off) &&
        poly_upload(P, &k.cp, hm.cell_pts) && poly_upload(P, &k.cc_off, hm.cell_cells_off) &&
        poly_upload(P, &k.ccl, hm.cell_cells) && poly_upload(P, &k.Cf, hm.Cf) && poly_upload(P, &k.Sf, hm.Sf) &&
        poly_upload(P, &k.Cc, hm.Cc) && poly_upload(P, &k.Vc, hm.Vc);
    PolyWork& w = P.w;
    w.words = (N + 31) / 32;
    w.qcap = N;
    const bool ok = ok_up && poly_alloc(P, &w.visited, (size_t)(S * w.words)) == cudaSuccess &&
         poly_alloc(P, &w.queue, (size_t)(S * w.qcap)) == cudaSuccess &&
         poly_alloc(P, &w.qtype, (size_t)(S * w.qcap)) == cudaSuccess &&
         poly_alloc(P, &w.count, (size_t)S) == cudaSuccess && poly_alloc(P, &w.acc, (size_t)(5 * N)) == cudaSuccess &&
         poly_alloc(P, &w.claim, (size_t)N) == cudaSuccess &&
         cudaMemset(w.count, 0, sizeof(int32_t) * S) == cudaSuccess;
    w.err = &ctx->d_cnt->error;
    if (!ok) {
        ctx->err = "polyMesh: device allocation failed";
        sdfibm_cuda_destroy(ctx);
        *out = nullptr;
        return SDFIBM_ERR_CUDA;
    }
    return SDFIBM_OK;
}

static int poly_interact(sdfibm_ctx* ctx, double time, double dt, const float* U, float* As, float* Fs, float* Ts,
                         int32_t* Ct, double* FT) {
    sdfibm_ctx::Poly& P = *ctx->poly;
    const int64_t N = P.N;
    const int S = ctx->S;
    cudaStream_t st = ctx->stream;
    int launches = 0;
    mark_begin(ctx);
    set_step_kernel<<<1, 1, 0, st>>>(ctx->d_step, time, dt, 1, 0.0);
    // SolidCloud::interact zeroes the four fields over the whole mesh (solidcloud.cpp:438-441)
    CK(cudaMemsetAsync(As, 0, sizeof(float) * N, st));
    CK(cudaMemsetAsync(Fs, 0, sizeof(float) * 3 * N, st));
    CK(cudaMemsetAsync(Ts, 0, sizeof(float) * N, st));
    CK(cudaMemsetAsync(Ct, 0, sizeof(int32_t) * N, st));
    CK(cudaMemsetAsync(P.w.acc, 0, sizeof(double) * 5 * N, st));
    CK(cudaMemsetAsync(P.w.claim, 0xff, sizeof(int32_t) * N, st));
    launches = 1;
    if (S > 0) {
        CK(cudaMemsetAsync(P.w.visited, 0, sizeof(uint32_t) * P.w.words * S, st));
        CK(cudaMemsetAsync(ctx->d_ftacc, 0, sizeof(double) * 6 * S, st));
        poly_enum_kernel<<<S, 256, 0, st>>>(P.k, ctx->d_sk, ctx->d_st, P.w);
        mark(ctx, "poly_enum_kernel");
        poly_couple_kernel<<<dim3(8, S), 256, 0, st>>>(P.k, ctx->d_sk, ctx->d_st, P.w, U, ctx->d_ftacc, ctx->d_step);
        mark(ctx, "poly_couple_kernel");
        launches += 2;
    }
    poly_finalize_kernel<<<ctx->num_sms * 4, 256, 0, st>>>(P.w, (int32_t)N, As, Fs, Ts, Ct);
    mark(ctx, "poly_finalize_kernel");
    ++launches;
    if (S > 0) {
        poly_ft_kernel<<<(S + 127) / 128, 128, 0, st>>>(ctx->d_ftacc, ctx->d_ft, S, ctx->opt.rho_f);
        ft_to_state_kernel<<<(S + 127) / 128, 128, 0, st>>>(ctx->d_ft, ctx->d_st, S);
        launches += 2;
    }
    CK(cudaGetLastError());
    ctx->launches_last = launches;
    ctx->interacted = true;
    if (FT) {
        if (S > 0) CK(cudaMemcpyAsync(ctx->h_ft, ctx->d_ft, sizeof(double) * 6 * S, cudaMemcpyDeviceToHost, st));
        const int rs = sync_counters(ctx);
        if (rs) return rs;
        std::memcpy(FT, ctx->h_ft, sizeof(double) * 6 * S);
    }
    return SDFIBM_OK;
}

// host fields of a polyMesh context: whole-field copies through device staging (FP32 planes, or FP64 in OpenFOAM's
// layout converted on the device)
static int poly_interact_host(sdfibm_ctx* ctx, double time, double dt, const void* U, void* As, void* Fs, void* Ts,
                              void* Ct, double* FT, bool f64) {
    sdfibm_ctx::Poly& P = *ctx->poly;
    const int64_t N = P.N;
    cudaStream_t st = ctx->stream;
    if (!P.dU && (poly_alloc(P, &P.dU, 3 * N) || poly_alloc(P, &P.dAs, N) || poly_alloc(P, &P.dFs, 3 * N) ||
                  poly_alloc(P, &P.dTs, N) || poly_alloc(P, &P.dCt, N)))
        return fail(ctx, SDFIBM_ERR_CUDA, "staging allocation failed");
    if (f64 && !P.d64 && poly_alloc(P, &P.d64, 9 * N)) return fail(ctx, SDFIBM_ERR_CUDA, "staging allocation failed");
    if (f64) {
        CK(cudaMemcpyAsync(P.d64, U, sizeof(double) * 3 * N, cudaMemcpyHostToDevice, st));
        u64_to_planes_kernel<<<ctx->num_sms * 8, 256, 0, st>>>(P.d64, N, P.dU);
    } else {
        CK(cudaMemcpyAsync(P.dU, U, sizeof(float) * 3 * N, cudaMemcpyHostToDevice, st));
    }
    int rc = poly_interact(ctx, time, dt, P.dU, P.dAs, P.dFs, P.dTs, P.dCt, nullptr);
    if (rc) return rc;
    if (f64) {
        double* o = P.d64 + 3 * N;
        fields_to_f64_kernel<<<ctx->num_sms * 8, 256, 0, st>>>(N, P.dAs, P.dFs, P.dTs, P.dCt, o);
        CK(cudaMemcpyAsync(As, o, sizeof(double) * N, cudaMemcpyDeviceToHost, st));
        CK(cudaMemcpyAsync(Fs, o + N, sizeof(double) * 3 * N, cudaMemcpyDeviceToHost, st));
        CK(cudaMemcpyAsync(Ts, o + 4 * N, sizeof(double) * N, cudaMemcpyDeviceToHost, st));
        CK(cudaMemcpyAsync(Ct, o + 5 * N, sizeof(double) * N, cudaMemcpyDeviceToHost, st));
    } else {
        CK(cudaMemcpyAsync(As, P.dAs, sizeof(float) * N, cudaMemcpyDeviceToHost, st));
        CK(cudaMemcpyAsync(Fs, P.dFs, sizeof(float) * 3 * N, cudaMemcpyDeviceToHost, st));
        CK(cudaMemcpyAsync(Ts, P.dTs, sizeof(float) * N, cudaMemcpyDeviceToHost, st));
        CK(cudaMemcpyAsync(Ct, P.dCt, sizeof(int32_t) * N, cudaMemcpyDeviceToHost, st));
    }
    if (ctx->S > 0) CK(cudaMemcpyAsync(ctx->h_ft, ctx->d_ft, sizeof(double) * 6 * ctx->S, cudaMemcpyDeviceToHost, st));
    rc = sync_counters(ctx);
    if (rc) return rc;
    ctx->host_h2d = (f64 ? 24 : 12) * N;
    ctx->host_d2h = (f64 ? 48 : 24) * N + 48 * ctx->S;
    ctx->host_sparse = false;
    if (FT) std::memcpy(FT, ctx->h_ft, sizeof(double) * 6 * ctx->S);
    return SDFIBM_OK;
}

// sizes of the ABI structs as compiled, for binding checks
int64_t sdfibm_abi_sizeof(int which) {
    switch (which) {
        case 0: return sizeof(sdfibm_mesh_desc);
        case 1: return sizeof(sdfibm_shape_desc);
        case 2: return sizeof(sdfibm_solid_desc);
        case 3: return sizeof(sdfibm_solid_state);
        case 4: return sizeof(sdfibm_options);
        case 5: return sizeof(sdfibm_mlp_data_desc);
        case 6: return sizeof(sdfibm_mlp_train_desc);
        default: return -1;
    }
}

}  // extern "C"
