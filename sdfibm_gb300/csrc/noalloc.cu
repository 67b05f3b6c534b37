// Touched-cell query of one solid that allocates no device memory (sdfibm_cuda_touched_noalloc).
//
// The regular path (sdfibm_cuda_create + sdfibm_cuda_interact) reserves its work space with cudaMalloc when the
// context is created.  Some callers cannot do that: hosts whose device memory is entirely owned by their own pool
// allocator (a cudaMalloc beside it fails or fragments the pool), and callers on latency-critical loops where the
// device-wide synchronisation of cudaMalloc/cudaFree is not acceptable.  For them this file keeps the work space of
// one enumeration -- the solid's record, its plan, the counters, the bbox class bytes, the flood-fill bitmaps and the
// two touched-cell lists -- in one file-scope device array that the driver reserves with the library's device code
// (under lazy module loading: during the first call on each device).
//
// Limits and rules:
//  * the solid's bounding box may hold at most NA_MAX_BBOX_CELLS cells (and NA_MAX_BITMAP_WORDS bitmap words);
//    larger boxes are rejected with SDFIBM_ERR_CAPACITY before anything is launched;
//  * the array (about 10 MiB) stays reserved on every GPU that uses it until the process exits.  With lazy module
//    loading (CUDA_MODULE_LOADING=LAZY, the default of recent CUDA releases) the driver reserves it during the
//    first call on each device, so make that first call at start-up, before a pool allocator takes the device's
//    memory;
//  * the first call on a device also looks up the array's device address (cudaGetSymbolAddress) with that device
//    current and keeps it for the life of the process; make that first call before any stream capture.  The kept
//    address belongs to the device's primary context: cudaDeviceReset between calls is not supported;
//  * every call reuses the same array: two calls whose work overlaps on the GPU (different streams, or different
//    host threads on one device) race and corrupt each other's results.  Serialise them (same stream) instead.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <mutex>

#include <cuda_runtime.h>

#include "../../include/sdfibm_cuda.h"
#include "kernels.cuh"

namespace sdfibm_dev {
__global__ void plan_kernel(MeshK m, const SolidK* sk, const sdfibm_solid_state* st, SolidPlan* plan, int S,
                            Counters* cnt);
void launch_classify(const ClassifyArgs& A, bool flat, int grid, cudaStream_t st);
int classify_occupancy(int method, bool flat);
__global__ void connect_kernel(MeshK m, const SolidK* sk, SolidPlan* plan, const uint8_t* scratch, uint32_t* gbitmaps,
                               int32_t* in_cell, int32_t* in_solid, int32_t* cut_cell, int32_t* cut_solid,
                               int64_t cap_in, int64_t cap_cut, Counters* cnt, int smem_words, const int32_t* solids);
}  // namespace sdfibm_dev

using namespace sdfibm_dev;

namespace {

constexpr int64_t NA_MAX_BBOX_CELLS = 1 << 19;    // 524288 cells, e.g. an 80 x 80 x 80 box
constexpr int64_t NA_MAX_BITMAP_WORDS = 1 << 18;  // candidate + reached bitmaps, 32 cells per word

constexpr size_t na_align(size_t x) { return (x + 255) & ~(size_t)255; }
constexpr size_t OFF_SK = 0;
constexpr size_t OFF_ST = OFF_SK + na_align(sizeof(SolidK));
constexpr size_t OFF_PLAN = OFF_ST + na_align(sizeof(sdfibm_solid_state));
constexpr size_t OFF_CNT = OFF_PLAN + na_align(sizeof(SolidPlan));
constexpr int64_t NA_MAX_CHUNKS = 8192;           // classify work items of the one solid
constexpr size_t OFF_CHUNKS = OFF_CNT + na_align(sizeof(Counters));
constexpr size_t OFF_CLS = OFF_CHUNKS + na_align(sizeof(int2) * NA_MAX_CHUNKS);
constexpr size_t OFF_BITMAP = OFF_CLS + na_align(NA_MAX_BBOX_CELLS);
constexpr size_t LIST_BYTES = na_align(4 * NA_MAX_BBOX_CELLS);
constexpr size_t OFF_IN_CELL = OFF_BITMAP + na_align(4 * NA_MAX_BITMAP_WORDS);
constexpr size_t OFF_IN_SOLID = OFF_IN_CELL + LIST_BYTES;
constexpr size_t OFF_CUT_CELL = OFF_IN_SOLID + LIST_BYTES;
constexpr size_t OFF_CUT_SOLID = OFF_CUT_CELL + LIST_BYTES;
constexpr size_t NA_BYTES = OFF_CUT_SOLID + LIST_BYTES;

}  // namespace

// The work space.  In host code this name is only a stand-in for the device object: its device address comes from
// cudaGetSymbolAddress (scratch_address below); device code in this file may name it directly.
static __device__ __align__(256) unsigned char g_noalloc_scratch[NA_BYTES];

namespace {

std::mutex g_addr_mu;
void* g_addr[128] = {};

// device address of g_noalloc_scratch on the current device (looked up once per device)
cudaError_t scratch_address(void** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= 128) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lk(g_addr_mu);
    if (!g_addr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return e;
        g_addr[dev] = p;
    }
    *out = g_addr[dev];
    return cudaSuccess;
}

bool shape_bound(const sdfibm_shape_desc& s, double& r, int& prism) {
    const double* a = s.p;
    prism = 0;
    switch (s.type) {
        case SDFIBM_SHAPE_CIRCLE: r = a[0]; prism = 1; return true;
        case SDFIBM_SHAPE_SPHERE: r = a[0]; return true;
        case SDFIBM_SHAPE_ELLIPSE: r = fmax(a[0], a[1]); prism = 1; return true;
        case SDFIBM_SHAPE_ELLIPSOID: r = fmax(fmax(a[0], a[1]), a[2]); return true;
        case SDFIBM_SHAPE_RECTANGLE: r = sqrt(a[0] * a[0] + a[1] * a[1]); prism = 1; return true;
        case SDFIBM_SHAPE_BOX: r = sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]); return true;
        case SDFIBM_SHAPE_CIRCLE_TAIL:
        case SDFIBM_SHAPE_CIRCLE_TWOTAIL: r = fmax(a[0], sqrt(4 * a[4] * a[4] + a[2] * a[2])); prism = 1; return true;
        case SDFIBM_SHAPE_PLANE: r = 0; return true;
        default: return false;
    }
}

// the enumeration record of one solid, built exactly as sdfibm_cuda_create builds it, with its work space placed
// at the start of the file-scope array and the flood-fill bitmaps in global memory
bool solid_record(const sdfibm_mesh_desc& mesh, const sdfibm_solid_desc& d, SolidK& k) {
    const int32_t n3[3] = {mesh.nx, mesh.ny, mesh.nz};
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
    if (!shape_bound(d.shape, r, prism)) return false;
    k.shape.bound_r = r;
    k.shape.prism = prism;
    k.infinite = d.shape.type == SDFIBM_SHAPE_PLANE;
    const double rr = r * (1.0 + 1e-9) + 1e-12;
    for (int a = 0; a < 3; ++a) {
        int64_t e;
        if (k.infinite || (prism && a == 2)) e = n3[a];
        else e = (int64_t)std::ceil(2.0 * rr / mesh.h[a]) + 4 + (prism ? 4 : 0);
        if (!k.infinite && !(prism && a == 2) && e >= (int64_t)n3[a] + 4) e = (int64_t)n3[a] + 4;
        k.ext[a] = (int32_t)e;
    }
    if (!k.infinite && prism && !(d.quat[1] == 0.0 && d.quat[2] == 0.0))
        for (int a = 0; a < 2; ++a) k.ext[a] = n3[a] + 4;
    const bool layer = mesh.nz <= 2;
    k.tdim[0] = layer ? 8 : 4;
    k.tdim[1] = layer ? 8 : 4;
    k.tdim[2] = layer ? 2 : 4;
    for (int a = 0; a < 3; ++a) k.ntile[a] = (k.ext[a] + k.tdim[a] - 1) / k.tdim[a];
    k.div_e0 = make_fastdiv((uint32_t)k.ext[0]);
    k.div_e01 = make_fastdiv((uint32_t)((int64_t)k.ext[0] * k.ext[1]));
    k.tile_base = 0;
    k.scratch_off = 0;
    k.bitmap_global = 1;
    k.bitmap_off = 0;
    k.motion_type = d.motion_type;
    k.forcer_type = d.forcer_type;
    k.collision_id = d.shape.collision_id;
    k.radiusB = d.shape.radiusB;
    return true;
}

}  // namespace

namespace sdfibm_dev {

// Set-up of one call inside the array: the solid's record, its state and zeroed counters (passed by value, so that
// nothing on the call's stack is read after the call returns), and the classify work items of the single solid,
// (0, first tile of each chunk).
static_assert(sizeof(SolidK) + sizeof(sdfibm_solid_state) + sizeof(int64_t) + 16 <= 4096,
              "records passed as kernel arguments");
__global__ void noalloc_init_kernel(SolidK k, sdfibm_solid_state x, int64_t list_cap, int nchunks) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i == 0) {
        *reinterpret_cast<SolidK*>(g_noalloc_scratch + OFF_SK) = k;
        *reinterpret_cast<sdfibm_solid_state*>(g_noalloc_scratch + OFF_ST) = x;
        Counters c;
        memset(&c, 0, sizeof(c));
        c.list_cap = list_cap;
        *reinterpret_cast<Counters*>(g_noalloc_scratch + OFF_CNT) = c;
    }
    if (i < nchunks) reinterpret_cast<int2*>(g_noalloc_scratch + OFF_CHUNKS)[i] = make_int2(0, i * CHUNK_TILES);
}

// Writes the enumeration result in the order of sdfibm_cuda_touched: ALL_INSIDE cells ascending, then
// CENTER_INSIDE ascending, then CENTER_OUTSIDE ascending (a stable partition of the cut list by type).  *n receives
// the full count, or -(status) when the enumeration reported a device-side error.
__global__ void __launch_bounds__(1024) noalloc_order_kernel(int32_t* __restrict__ cells, int8_t* __restrict__ types,
                                                             int64_t capacity, int64_t* __restrict__ n_out) {
    const Counters* cnt = reinterpret_cast<const Counters*>(g_noalloc_scratch + OFF_CNT);
    const int32_t* in_cell = reinterpret_cast<const int32_t*>(g_noalloc_scratch + OFF_IN_CELL);
    const int32_t* cut_cell = reinterpret_cast<const int32_t*>(g_noalloc_scratch + OFF_CUT_CELL);
    const int32_t* cut_solid = reinterpret_cast<const int32_t*>(g_noalloc_scratch + OFF_CUT_SOLID);
    __shared__ int32_t warp_a[32], warp_b[32];
    __shared__ int64_t s_n2;
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5, nw = blockDim.x >> 5;
    if (cnt->error != 0) {
        if (tid == 0) {
            const int32_t e = cnt->error;
            *n_out = -(int64_t)(e == DERR_FLOOD_LIMIT ? SDFIBM_ERR_TIMEOUT : SDFIBM_ERR_CAPACITY);
        }
        return;
    }
    const int64_t n_in = clamp_len(cnt->n_inside, cnt->list_cap), n_cut = clamp_len(cnt->n_cut, cnt->list_cap);
    for (int64_t e = tid; e < n_in; e += blockDim.x)
        if (e < capacity) { cells[e] = in_cell[e]; types[e] = 1; }
    // count of CENTER_INSIDE entries
    int local = 0;
    for (int64_t e = tid; e < n_cut; e += blockDim.x) local += list_type(cut_solid[e]) == 2;
    for (int o = 16; o > 0; o >>= 1) local += __shfl_xor_sync(0xffffffffu, local, o);
    if (tid == 0) s_n2 = 0;
    __syncthreads();
    if (lane == 0) atomicAdd((unsigned long long*)&s_n2, (unsigned long long)local);
    __syncthreads();
    const int64_t n2 = s_n2;
    int64_t carry2 = 0, carry3 = 0;
    for (int64_t base = 0; base < n_cut; base += blockDim.x) {
        const int64_t e = base + tid;
        const int t = e < n_cut ? list_type(cut_solid[e]) : 0;
        const int f2 = t == 2, f3 = t == 3;
        int x2 = f2, x3 = f3;
        for (int o = 1; o < 32; o <<= 1) {
            const int y2 = __shfl_up_sync(0xffffffffu, x2, o), y3 = __shfl_up_sync(0xffffffffu, x3, o);
            if (lane >= o) { x2 += y2; x3 += y3; }
        }
        if (lane == 31) { warp_a[wid] = x2; warp_b[wid] = x3; }
        __syncthreads();
        if (wid == 0) {
            int a = lane < nw ? warp_a[lane] : 0, b = lane < nw ? warp_b[lane] : 0;
            for (int o = 1; o < 32; o <<= 1) {
                const int ya = __shfl_up_sync(0xffffffffu, a, o), yb = __shfl_up_sync(0xffffffffu, b, o);
                if (lane >= o) { a += ya; b += yb; }
            }
            if (lane < nw) { warp_a[lane] = a; warp_b[lane] = b; }
        }
        __syncthreads();
        const int64_t before2 = carry2 + (wid > 0 ? warp_a[wid - 1] : 0) + x2 - f2;
        const int64_t before3 = carry3 + (wid > 0 ? warp_b[wid - 1] : 0) + x3 - f3;
        if (f2) {
            const int64_t p = n_in + before2;
            if (p < capacity) { cells[p] = cut_cell[e]; types[p] = 2; }
        } else if (f3) {
            const int64_t p = n_in + n2 + before3;
            if (p < capacity) { cells[p] = cut_cell[e]; types[p] = 3; }
        }
        carry2 += warp_a[nw - 1];
        carry3 += warp_b[nw - 1];
        __syncthreads();
    }
    if (tid == 0) *n_out = n_in + n_cut;
}

}  // namespace sdfibm_dev

extern "C" int sdfibm_cuda_touched_noalloc(const sdfibm_mesh_desc* mesh, const sdfibm_solid_desc* solid,
                                           void* cuda_stream, int32_t* cells, int8_t* types, int64_t capacity,
                                           int64_t* n_device) {
    if (!mesh || !solid || !n_device || (capacity > 0 && (!cells || !types)) || capacity < 0) return SDFIBM_ERR_ARG;
    if (mesh->nx <= 0 || mesh->ny <= 0 || mesh->nz <= 0) return SDFIBM_ERR_ARG;
    if (!(mesh->h[0] > 0 && mesh->h[1] > 0 && mesh->h[2] > 0)) return SDFIBM_ERR_ARG;
    const int64_t N = (int64_t)mesh->nx * mesh->ny * mesh->nz;
    if (N >= ((int64_t)1 << 31)) return SDFIBM_ERR_ARG;
    SolidK k;
    if (!solid_record(*mesh, *solid, k)) return SDFIBM_ERR_ARG;
    const int64_t bbox = (int64_t)k.ext[0] * k.ext[1] * k.ext[2];
    const int64_t words = 2 * (int64_t)k.ext[1] * k.ext[2] * ((k.ext[0] + 31) / 32);
    if (bbox > NA_MAX_BBOX_CELLS || words > NA_MAX_BITMAP_WORDS) return SDFIBM_ERR_CAPACITY;
    const int ntiles = k.ntile[0] * k.ntile[1] * k.ntile[2];
    const int nchunks = (ntiles + CHUNK_TILES - 1) / CHUNK_TILES;
    if (nchunks > NA_MAX_CHUNKS) return SDFIBM_ERR_CAPACITY;

    void* base = nullptr;
    if (scratch_address(&base) != cudaSuccess) return SDFIBM_ERR_CUDA;
    unsigned char* b = static_cast<unsigned char*>(base);
    cudaStream_t st = (cudaStream_t)cuda_stream;

    MeshK m;
    std::memset(&m, 0, sizeof(m));
    m.nx = mesh->nx; m.ny = mesh->ny; m.nz = mesh->nz; m.twod = mesh->twod;
    for (int a = 0; a < 3; ++a) { m.o[a] = mesh->origin[a]; m.h[a] = mesh->h[a]; m.h32[a] = (float)mesh->h[a]; }
    m.ncells = N;
    m.V = mesh->h[0] * mesh->h[1] * mesh->h[2];
    mesh_fastdiv(m);

    sdfibm_solid_state x;
    std::memset(&x, 0, sizeof(x));
    for (int a = 0; a < 3; ++a) { x.pos[a] = solid->pos[a]; x.vel[a] = solid->vel[a]; x.omega[a] = solid->omega[a]; }
    for (int a = 0; a < 4; ++a) x.quat[a] = solid->quat[a];
    SolidK* d_sk = reinterpret_cast<SolidK*>(b + OFF_SK);
    sdfibm_solid_state* d_st = reinterpret_cast<sdfibm_solid_state*>(b + OFF_ST);
    SolidPlan* d_plan = reinterpret_cast<SolidPlan*>(b + OFF_PLAN);
    Counters* d_cnt = reinterpret_cast<Counters*>(b + OFF_CNT);
    int2* d_chunks = reinterpret_cast<int2*>(b + OFF_CHUNKS);
    // the records travel as kernel arguments (counters start from zero on every call)
    noalloc_init_kernel<<<(nchunks + 255) / 256, 256, 0, st>>>(k, x, NA_MAX_BBOX_CELLS, nchunks);
    plan_kernel<<<1, 32, 0, st>>>(m, d_sk, d_st, d_plan, 1, d_cnt);
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return SDFIBM_ERR_CUDA;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int grid = nchunks < 4 * (sms > 0 ? sms : 1) ? nchunks : 4 * (sms > 0 ? sms : 1);
    ClassifyArgs CA{};
    CA.m = m; CA.sk = d_sk; CA.st = d_st; CA.plan = d_plan; CA.chunks = d_chunks; CA.total_chunks = nchunks; CA.chunk_tiles = CHUNK_TILES;
    CA.cls = b + OFF_CLS; CA.alpha = nullptr; CA.cnt = d_cnt; CA.method = -1; CA.subsample_n = 0;
    launch_classify(CA, m.nz <= 2, grid, st);
    connect_kernel<<<1, 512, 0, st>>>(m, d_sk, d_plan, b + OFF_CLS, reinterpret_cast<uint32_t*>(b + OFF_BITMAP),
                                      reinterpret_cast<int32_t*>(b + OFF_IN_CELL), reinterpret_cast<int32_t*>(b + OFF_IN_SOLID),
                                      reinterpret_cast<int32_t*>(b + OFF_CUT_CELL), reinterpret_cast<int32_t*>(b + OFF_CUT_SOLID),
                                      NA_MAX_BBOX_CELLS, NA_MAX_BBOX_CELLS, d_cnt, 0, nullptr);
    noalloc_order_kernel<<<1, 1024, 0, st>>>(cells, types, capacity, n_device);
    return cudaGetLastError() == cudaSuccess ? SDFIBM_OK : SDFIBM_ERR_CUDA;
}
