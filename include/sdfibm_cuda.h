/*
 * sdfibm_cuda.h — C ABI of the GB300 (sm_103a) fluid–solid coupling library.
 *
 * The library is a drop-in for the solid side of sdfibm's time step:
 *   SolidCloud::interact     src/solidcloud.cpp:435-464  -> sdfibm_cuda_interact
 *   SolidCloud::evolve       src/solidcloud.cpp:521-562  -> sdfibm_cuda_evolve
 *   SolidCloud::fixInternal  src/solidcloud.cpp:288-301  -> sdfibm_cuda_fix_internal
 *   SolidCloud::SolidCloud   src/solidcloud.cpp:209-265  -> sdfibm_cuda_create (after the host has parsed solidDict)
 *   Solid getters/setters    src/solid.h:58-80           -> sdfibm_cuda_get_solids / sdfibm_cuda_set_solids
 * The host keeps parsing solidDict with the reference's factories and lowers every Shape / Motion / Forcer /
 * Material instance into the plain-old-data descriptors below.  No function here exits the process: every entry
 * point returns an sdfibm_status and sdfibm_cuda_last_error() gives the message.
 *
 * Mesh: uniform hexahedral grid (blockMesh single block, simpleGrading 1).  Point (i,j,k) is
 *   x = origin[0] + i*h[0]  (one multiply, one add; no fused multiply-add), likewise y, z;
 * cell (i,j,k) has label i + nx*(j + ny*k) and centre origin + (i+0.5)*h.
 *
 * Fields (caller-owned, cell-major structure of arrays, device pointers unless stated otherwise):
 *   U  : float[3][ncells]  (x plane, then y plane, then z plane)
 *   As : float[ncells], Ts : float[ncells], Fs : float[3][ncells], Ct : int32[ncells]
 *   FT : double[nsolids][6] = fluid force (3) then fluid torque (3), the values of
 *        Solid::setFluidForceAndTorque at src/solidcloud.cpp:432.
 */
#ifndef SDFIBM_CUDA_H
#define SDFIBM_CUDA_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SDFIBM_ABI_VERSION 1

typedef enum sdfibm_status {
    SDFIBM_OK = 0,
    SDFIBM_ERR_ARG = 1,       /* bad argument (null pointer, bad size, unknown type id) */
    SDFIBM_ERR_CAPACITY = 2,  /* a work queue or list outgrew its reserved capacity */
    SDFIBM_ERR_CUDA = 3,      /* a CUDA runtime call failed */
    SDFIBM_ERR_TIMEOUT = 4,   /* a bounded device-side wait gave up */
    SDFIBM_ERR_STATE = 5      /* call out of order (e.g. evolve before any interact) */
} sdfibm_status;

/* Shape registry of src/libshape/shapefactory.h:11-35 (names kept, ids are this ABI's). */
typedef enum sdfibm_shape_type {
    SDFIBM_SHAPE_CIRCLE = 1,          /* circle.h        p = {radius, radiusSQR} */
    SDFIBM_SHAPE_SPHERE = 2,          /* sphere.h        p = {radius, radiusSQR} */
    SDFIBM_SHAPE_ELLIPSE = 3,         /* ellipse.h       p = {ra, rb, 1/ra^2, 1/rb^2} */
    SDFIBM_SHAPE_ELLIPSOID = 4,       /* ellipsoid.h     p = {ra, rb, rc, 1/ra^2, 1/rb^2, 1/rc^2} (com ignored) */
    SDFIBM_SHAPE_RECTANGLE = 5,       /* rectangle.h     p = {ra, rb} */
    SDFIBM_SHAPE_BOX = 6,             /* box.h           p = {ra, rb, rc} */
    SDFIBM_SHAPE_PLANE = 7,           /* plane.h         p = {} ; inside = local y < 0, infinite */
    SDFIBM_SHAPE_CIRCLE_TAIL = 8,     /* circle_tail.h   p = {radius, ratio, radiusb, radiusSQR, radiusa} */
    SDFIBM_SHAPE_CIRCLE_TWOTAIL = 9   /* circle_twotail.h p = {radius, ratio, radiusb(=thickness/2), radiusSQR, radiusa} */
} sdfibm_shape_type;

/* Motion registry of src/libmotion/motionfactory.cpp:33-46 ("free" = none, src/solidcloud.cpp:185). */
typedef enum sdfibm_motion_type {
    SDFIBM_MOTION_FREE = 0,
    SDFIBM_MOTION_000002 = 1,           /* p = {period, omega=2pi/period} */
    SDFIBM_MOTION_110002 = 2,           /* p = {period, omega} */
    SDFIBM_MOTION_222000 = 3,           /* p = {u, v, w} */
    SDFIBM_MOTION_SINEDIRECTIONAL = 4,  /* p = {amplitude, period, omega, dir.x, dir.y, dir.z} */
    SDFIBM_MOTION_01MASK = 5,           /* p = {vmask.x, vmask.y, vmask.z, omask.x, omask.y, omask.z} */
    SDFIBM_MOTION_ROTOR = 6,            /* p = {period, omega, radius, theta0, selfom} */
    SDFIBM_MOTION_OPENCLOSE = 7         /* p = {} */
} sdfibm_motion_type;

/* Forcer registry of src/libforcer/forcerfactory.h:7-16. */
typedef enum sdfibm_forcer_type {
    SDFIBM_FORCER_NONE = 0,
    SDFIBM_FORCER_CONSTANT = 1,  /* p = {force.xyz, torque.xyz} */
    SDFIBM_FORCER_SPRING = 2,    /* p = {pivot.xyz, k, l} */
    SDFIBM_FORCER_MAGNETIC = 3   /* p = {direction.xyz, A, w} */
} sdfibm_forcer_type;

/* Solid-solid collision handling (src/solidcloud.cpp:477-519, src/libcollision/). */
typedef enum sdfibm_collision_mode {
    SDFIBM_COLLISION_OFF = 0,        /* reference HEAD: m_radiusB = -1 (solidcloud.cpp:74) gives an empty grid */
    SDFIBM_COLLISION_REFERENCE = 1,  /* grid spacing 2*max(radiusB), the reference's SHAPE2ID table and force law */
    SDFIBM_COLLISION_SPHERES = 2     /* same grid and law, every finite shape treated as its bounding sphere */
} sdfibm_collision_mode;

/* Cut-cell solid fraction evaluator. */
typedef enum sdfibm_fraction_method {
    SDFIBM_FRACTION_REFGEO = 0,     /* GeometricTools::calcCellVolume (geometrictools.cpp:47-116), FP64 */
    SDFIBM_FRACTION_SUBSAMPLE = 1,  /* stratified midpoint lattice of n^3 (3D) / n^2 (2D) isInside samples */
    SDFIBM_FRACTION_LEARNED = 2     /* sub-cell planar prior + 16-64-64-1 network, SUBSAMPLE outside the band */
} sdfibm_fraction_method;

typedef struct sdfibm_mesh_desc {
    int32_t nx, ny, nz;   /* cells per axis */
    int32_t twod;         /* on_twod: calcCellVolume puts the cell apex at z = 0 (geometrictools.cpp:57-58) */
    double origin[3];     /* lowest mesh point */
    double h[3];          /* cell size per axis */
} sdfibm_mesh_desc;

typedef struct sdfibm_shape_desc {
    int32_t type;          /* sdfibm_shape_type */
    int32_t collision_id;  /* SHAPE2ID of collision.h:11-15: Plane 0, Circle 1, Sphere 2, any other name 0 */
    double p[8];           /* type parameters, see sdfibm_shape_type */
    double com[3];         /* IShape::m_com (ignored by Ellipsoid and Plane) */
    double radiusB;        /* IShape::m_radiusB */
    double volume;         /* IShape::m_volume */
    double volume_inv;     /* IShape::m_volumeINV */
    double moi_inv[9];     /* IShape::m_moiINV = Foam::inv(m_moi), row-major */
} sdfibm_shape_desc;

typedef struct sdfibm_solid_desc {
    int32_t id;            /* Solid::id (position in the solids dictionary) */
    int32_t motion_type;   /* sdfibm_motion_type */
    int32_t forcer_type;   /* sdfibm_forcer_type */
    int32_t pad0;
    sdfibm_shape_desc shape;
    double motion_p[8];
    double forcer_p[8];
    double rho;            /* IMaterial::m_rho */
    double mass;           /* Solid::mass = m_volume*rho        (solid.h:100) */
    double mass_inv;       /* Solid::mass_inv = m_volumeINV/rho (solid.h:101) */
    double moi_inv[9];     /* Solid::moi_inv = m_moiINV/rho     (solid.h:102) */
    double pos[3];         /* centre */
    double quat[4];        /* orientation (w, x, y, z) = quaternion(XYZ, euler) */
    double vel[3];
    double omega[3];
} sdfibm_solid_desc;

/* Full dynamic state of one Solid (solid.h:20-44). */
typedef struct sdfibm_solid_state {
    double pos[3], quat[4], vel[3], omega[3];
    double force[3], torque[3];
    double fluid_force[3], fluid_torque[3], fluid_force_old[3], fluid_torque_old[3];
    double forcer_force[3], forcer_torque[3], forcer_force_old[3], forcer_torque_old[3];
    int32_t first_fluid_step, first_forcer_step;
} sdfibm_solid_state;

typedef struct sdfibm_options {
    double rho_f;            /* m_rhof: transportProperties rho, 0 when on_fluid is off (solidcloud.cpp:247-251) */
    double gravity[3];       /* meta.gravity */
    int32_t collision_mode;  /* sdfibm_collision_mode */
    int32_t n_subiter;       /* 0: the reference rule (20, or 1 for a single solid: solidcloud.cpp:524-527) */
    int32_t fraction_method; /* sdfibm_fraction_method */
    int32_t subsample_n;     /* samples per axis for SUBSAMPLE (0: 10) */
    int32_t dense_reset;     /* 1: zero the four fields over the whole mesh every interact (solidcloud.cpp:438-441);
                                0: zero only the cells touched by the previous interact (identical values while
                                the caller leaves those fields alone between calls) */
    int32_t exact_forcing;   /* 1: forcing and torque per cell in FP64 exactly as solidcloud.cpp:384-417 (default);
                                0: FP32 forcing with FP64 force/torque sums */
    int32_t tile_cells;      /* cells per (solid, cell-tile) work item of the classify queue; 0: 8 tiles (512 cells
                                in 3-D), or what sdfibm_cuda_autotune chose */
    int32_t timing;          /* 1: record CUDA events around every kernel (sdfibm_cuda_kernel_times) */
    int32_t learned_fallback_n; /* LEARNED: samples per axis of the SUBSAMPLE evaluation of the cells outside the
                                   network's confidence band (0: 16, the lattice the network was trained on) */
    int32_t graphs;          /* 1: capture interact and evolve as CUDA graphs on the first call and replay them
                                (needs a non-NULL stream; ignored while timing is on) */
    int32_t recheck_cap;     /* SUBSAMPLE / LEARNED: entries of the list of FP32-undecided sample points re-evaluated
                                in FP64 after the sampling pass (0: one per 8 bbox cells, at least 2^20, at most
                                2^25); points beyond it are re-evaluated in place (cells of the LEARNED fallback are
                                then recounted whole) */
    int32_t reserved[3];
} sdfibm_options;

typedef struct sdfibm_ctx sdfibm_ctx;

/* Defaults for sdfibm_options (rho_f 1, no gravity, collisions off, REF-GEO, sparse reset, exact forcing). */
void sdfibm_options_default(sdfibm_options* opt);

/* SolidCloud::SolidCloud (solidcloud.cpp:209-265) minus the dictionary parsing: uploads the descriptors and
 * reserves device work space.  stream may be NULL (legacy default stream). */
int sdfibm_cuda_create(const sdfibm_mesh_desc* mesh, const sdfibm_solid_desc* solids, int32_t nsolids,
                       const sdfibm_options* opt, void* cuda_stream, sdfibm_ctx** out);

/* SolidCloud::SolidCloud on an explicit OpenFOAM polyMesh (graded, multi-block or polyhedral meshes; MeshInfo,
 * src/meshinfo.h:20-29), from the polyMesh lists: points [npoints][3]; faces as a compact list, face f having the
 * point labels face_lab[face_off[f] .. face_off[f + 1]); owner [nfaces]; neighbour [ninternal] (internal faces
 * first).  twod as in sdfibm_mesh_desc.  Face and cell geometry follow OpenFOAM's primitiveMesh (triangle fan and
 * pyramid decompositions); cellPoints are in ascending label order.  The same entry points then serve the context:
 * interact (the reference's breadth-first enumeration from the nearest cell centre, CellEnumerator, and its
 * REF-GEO fraction over the cells' faces, GeometricTools::calcCellVolume; fields reset over the whole mesh as
 * the reference does), evolve, fix_internal (with the mesh's cell centres), the host-field entry points (whole
 * fields copied) and touched.  Only SDFIBM_FRACTION_REFGEO is offered; graphs are off.  Limit: cells x solids
 * <= 2^28 (the per-solid search lists). */
int sdfibm_cuda_create_polymesh(const double* points, int64_t npoints, const int32_t* face_off,
                                const int32_t* face_lab, int64_t nfaces, const int32_t* owner,
                                const int32_t* neighbour, int64_t ninternal, int32_t twod,
                                const sdfibm_solid_desc* solids, int32_t nsolids, const sdfibm_options* opt,
                                void* cuda_stream, sdfibm_ctx** out);

/* SolidCloud::interact (solidcloud.cpp:435-464): resets As/Fs/Ts/Ct, enumerates the touched cells of every solid
 * (CellEnumerator, cellenumerator.cpp:6-78), computes As (REF-GEO / SUBSAMPLE / LEARNED), the direct forcing
 * Fs += alpha(U-us)/dt, Ts += alpha, Ct, clamps As to 1 (checkAlpha, :564-570) and reduces the fluid force and
 * torque of every solid.  U/As/Fs/Ts/Ct are device pointers; FT (may be NULL) is a HOST pointer that receives
 * the per-solid fluid force and torque (the call then synchronises the stream). */
int sdfibm_cuda_interact(sdfibm_ctx* ctx, double time, double dt, const float* U, float* As, float* Fs, float* Ts,
                         int32_t* Ct, double* FT);

/* Same as sdfibm_cuda_interact but every field pointer is a HOST pointer (the path an OpenFOAM-resident caller
 * takes).  U is copied in on a second stream while the enumeration and fraction kernels run; a page-locked U is
 * read in place at the coupling cells instead with REF-GEO (whose kernels take less time than the copy) and, after
 * two calls whose copy outlasted those kernels, with the other methods.  Page-locked fields
 * (cudaHostAlloc / cudaHostRegister) are written in place with the cells this call or the previous one touched,
 * while the call gets the same five buffers as the previous one and the caller leaves the four fields alone in
 * between (the first call, other buffers, or dense_reset copy the whole fields); other host memory receives
 * whole-field copies. */
int sdfibm_cuda_interact_host(sdfibm_ctx* ctx, double time, double dt, const float* U, float* As, float* Fs,
                              float* Ts, int32_t* Ct, double* FT);

/* Same as sdfibm_cuda_interact_host with the fields in OpenFOAM's own types and layout, so that a solver passes its
 * volField storage as it is (the reference's field members, createFields.h:19-35): U and Fs are volVectorFields
 * (double[ncells][3], one x,y,z triple per cell), As, Ts and Ct volScalarFields (double[ncells]; Ct holds the
 * integer cell codes as doubles, as the reference stores them).  Page-locked fields (cudaHostRegister on the
 * solver's arrays) are read and written in place by the GPU: U only at the coupling cells, after the enumeration,
 * and the result fields at the cells this call or the previous one touched (every cell on the first call with a
 * set of buffers, after other buffers, or with dense_reset).  Other host memory goes through whole-field copies
 * staged in a device FP64 buffer.  U is rounded to FP32 on the device, as the device-field path reads it. */
int sdfibm_cuda_interact_host64(sdfibm_ctx* ctx, double time, double dt, const double* U, double* As, double* Fs,
                                double* Ts, double* Ct, double* FT);

/* SolidCloud::evolve (solidcloud.cpp:521-562): n_subiter sub-steps of AB2 forcer and fluid force, buoyancy-reduced
 * gravity, solid-solid collision and Solid::move (solid.h:181-202), then storeOldForce. */
int sdfibm_cuda_evolve(sdfibm_ctx* ctx, double time, double dt);

/* SolidCloud::fixInternal (solidcloud.cpp:288-301): U[c] = velocity of solid Ct[c]-4 at the cell centre for every
 * cell with Ct[c] >= 4.  Visits only the cells the last interact touched. */
int sdfibm_cuda_fix_internal(sdfibm_ctx* ctx, const int32_t* Ct, float* U);

/* Optional, for a fluid solver whose fields live on the GPU: the forcing update the reference's solver applies after
 * interact (main.cpp:70-77, its cell fields): U = U - Fs dt per component and, when T is not null,
 * T = (1 - As) T + Ts, computed in FP64 and rounded once to the FP32 fields.  As, Fs and Ts must be the fields the
 * last interact on this context wrote (SDFIBM_ERR_STATE otherwise); only the cells that interact touched are
 * visited (elsewhere As = Fs = Ts = 0 and U, T keep their values, as in the dense update).  The face-flux update
 * (phi -= dt (interpolate(Fs) & Sf)) and the boundary corrections belong to the solver's mesh and stay there.
 * Enqueued on the context's stream. */
int sdfibm_cuda_apply_forcing(sdfibm_ctx* ctx, double dt, const float* As, const float* Fs, const float* Ts,
                              float* U, float* T);

/* Solid state download / upload for saveState, saveRestart and restarts (solidcloud.cpp:578-665). */
int sdfibm_cuda_get_solids(sdfibm_ctx* ctx, sdfibm_solid_state* out, int32_t nsolids);
int sdfibm_cuda_set_solids(sdfibm_ctx* ctx, const sdfibm_solid_state* in, int32_t nsolids);

/* Touched-cell list of one solid from the last interact, as CellEnumerator::intersect would give it: cells sorted
 * ascending within each type, ALL_INSIDE first, then CENTER_INSIDE, then CENTER_OUTSIDE (solidcloud.cpp:370-374).
 * types[i] is 1 (ALL_INSIDE), 2 (CENTER_INSIDE) or 3 (CENTER_OUTSIDE).  Returns the count through *n (host). */
int sdfibm_cuda_touched(sdfibm_ctx* ctx, int32_t solid, int64_t* cells, int8_t* types, int64_t capacity,
                        int64_t* n);

/* No counterpart in the reference.  The touched cells of ONE solid (the same list and order as sdfibm_cuda_touched
 * returns after an interact) computed without allocating any device memory, for callers that cannot call
 * cudaMalloc: hosts whose device memory is owned entirely by their own pool allocator, or latency-critical loops
 * that cannot afford the device-wide synchronisation of cudaMalloc/cudaFree.  The work space is one file-scope
 * device array of about 10 MiB, held on every GPU that uses it until the process exits.  With lazy module loading
 * (the default of recent CUDA releases) the driver reserves the array during the first call on each device: make
 * that first call at start-up, before a pool allocator takes the device's memory, and before any stream capture
 * (it also looks up the array's address, which stays cached for the process; cudaDeviceReset between calls is not
 * supported).  Limit: the solid's bounding box may hold at most 524288 cells (and 262144 flood-fill bitmap words);
 * larger solids are rejected with SDFIBM_ERR_CAPACITY before anything is launched.  Calls share the array and a call
 * keeps its contents, so calls that overlap on the GPU race; issue them on one stream.  cells (int32) and types (int8, 1/2/3) are device buffers of `capacity` entries; *n_device
 * (device int64) receives the full count, or -(status) when the enumeration failed on the device.  Asynchronous on
 * cuda_stream (NULL: the legacy default stream). */
int sdfibm_cuda_touched_noalloc(const sdfibm_mesh_desc* mesh, const sdfibm_solid_desc* solid, void* cuda_stream,
                                int32_t* cells, int8_t* types, int64_t capacity, int64_t* n_device);

/* Counters of the last interact (host): [0] coupling cells (sum over solids of |T_s|), [1] cut cells,
 * [2] bbox cells scanned, [3] vertices re-checked in FP64, [4] work items, [5] kernel launches,
 * [6] cut cells listed for the fraction pass (LEARNED: given to the model; SUBSAMPLE: sampled from the list),
 * [7] LEARNED: of those, cells outside the model's band (SUBSAMPLE fallback),
 * [8] / [9] bytes the last sdfibm_cuda_interact_host moved host to device / device to host, [10] 1 when it wrote
 * the touched cells only.  n: entries of out (at most 11 are written). */
int sdfibm_cuda_stats(sdfibm_ctx* ctx, int64_t* out, int32_t n);

/* No counterpart in the reference.  Autotuner of the launch configuration: times dense interacts (on the given
 * device fields, which it overwrites) with per-kernel events, first over the classify work-item size (2, 4, 8, 16 or
 * 32 tiles of one solid per item), then over the CTA count of every work-stealing or grid-strided launch
 * (classification: 1 .. occupancy x SMs; cut-cell sampling, REF-GEO fractions: 2 .. 16 x SMs; coupling: 1 ..
 * occupancy x SMs; network: 1 .. 8 x SMs), and keeps the fastest of each; results do not depend on the choice.
 * The choice is kept for the life of the process per workload shape (mesh, solid count, bounding-box tiles, fraction
 * method and lattice, SM count): a later call on a context of the same shape applies it without timing.
 * *chosen_tiles (host, may be NULL) receives the work-item size and options.tile_cells reports it in cells.  Captured
 * graphs are re-captured on their next use.  Synchronises. */
int sdfibm_cuda_autotune(sdfibm_ctx* ctx, double dt, const float* U, float* As, float* Fs, float* Ts, int32_t* Ct,
                         int32_t* chosen_tiles);

/* No counterpart in the reference.  The launch configuration in use: out[0] classify tiles per work item, out[1..5]
 * CTA counts of the classification, cut-cell sampling, coupling, network and REF-GEO fraction kernels, out[6] 1 when
 * the last sdfibm_cuda_autotune took it from the per-shape cache.  n: entries of out (at most 7 are written). */
int sdfibm_cuda_tuning(sdfibm_ctx* ctx, int32_t* out, int32_t n);

/* No counterpart in the reference (which has only the apex/pyramid fraction).  Installs the learned cut-cell
 * fraction model used when options.fraction_method is SDFIBM_FRACTION_LEARNED: params is a HOST array of
 * SDFIBM_MLP_NPARAM floats in the layout of include/sdfibm_mlp.h.  Confidence band: a cut cell takes the model's
 * fraction when its two sub-cell planar reconstructions agree, |P4 - P2| <= tau_refine, and its solid's bounding
 * radius spans at least rho_min cells; other cells are evaluated by SUBSAMPLE with options.learned_fallback_n samples
 * per axis (a negative tau_refine closes the band: every cut cell falls back).  Reserves the per-cell input buffers
 * on first use. */
int sdfibm_cuda_set_fraction_model(sdfibm_ctx* ctx, const float* params, float tau_refine, float rho_min);

/* Per-kernel device time (milliseconds, CUDA events on the context's stream) of the last interact when
 * options.timing is set: names[i] receives a static kernel name, ms[i] its time; returns the count through *n. */
int sdfibm_cuda_kernel_times(sdfibm_ctx* ctx, const char** names, double* ms, int32_t capacity, int32_t* n);

const char* sdfibm_cuda_last_error(const sdfibm_ctx* ctx);
const char* sdfibm_cuda_version(void);
void sdfibm_cuda_destroy(sdfibm_ctx* ctx);

#ifdef __cplusplus
}
#endif
#endif /* SDFIBM_CUDA_H */
