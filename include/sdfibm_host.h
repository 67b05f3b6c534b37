/*
 * sdfibm_host.h — host-side lowering of sdfibm's plugin objects into the POD descriptors of sdfibm_cuda.h, and the
 * solidDict front end.  These replace the reference's construction path:
 *   ShapeFactory / IShape constructors   src/libshape/shapefactory.h:9-39, src/libshape/{circle,...}.h ctors
 *   MotionFactory::create                src/libmotion/motionfactory.cpp:23-31 and the motion ctors
 *   ForcerFactory / IForcer ctors        src/libforcer/forcerfactory.h:7-16, {constant,spring,magnetic}.h ctors
 *   IMaterial (General) + Solid::setMaterial   src/solidcloud.cpp:127-143, src/solid.h:95-103
 *   Solid::setOrientation (euler degrees)      src/solidcloud.cpp:176-177, src/solid.h:76-80
 *   SolidCloud::initFromDictionary             src/solidcloud.cpp:14-206
 * and its output path: SolidCloud::saveState (cloud.out) and SolidCloud::saveRestart (src/solidcloud.cpp:578-665).
 * Every function returns an sdfibm_status; messages go to the caller-provided buffer (never to stdout/exit).
 */
#ifndef SDFIBM_HOST_H
#define SDFIBM_HOST_H

#include "sdfibm_cuda.h"

#ifdef __cplusplus
extern "C" {
#endif

/* IShape constructor of the given type: raw holds the dictionary scalars in the order of the sdfibm_shape_type
 * comment (radius | radiusa, radiusb[, radiusc] | radius, ratio, thickness); com may be NULL (zero). */
int sdfibm_host_make_shape(int32_t type, const double* raw, const double* com, sdfibm_shape_desc* out);

/* Motion constructors: raw holds the dictionary values (period | u,v,w | amplitude, period, direction.xyz |
 * mask digits as 0/1 | period, radius, theta0, selfom).  The derived parameters are filled in. */
int sdfibm_host_make_motion(int32_t type, const double* raw, double* motion_p8);

/* Forcer constructors: raw = force.xyz, torque.xyz | pivot.xyz, k, l | direction.xyz, A, w. */
int sdfibm_host_make_forcer(int32_t type, const double* raw, double* forcer_p8);

/* quaternion(quaternion::XYZ, euler*pi/180) */
void sdfibm_host_quat_from_euler_deg(const double* euler_deg, double* quat_wxyz);

/* Assemble a solid: shape + material density (Solid::setMaterial) + pose/velocity.  quat may be NULL (use euler). */
int sdfibm_host_make_solid(int32_t id, const sdfibm_shape_desc* shape, double rho, int32_t motion_type,
                           const double* motion_p8, int32_t forcer_type, const double* forcer_p8, const double* pos,
                           const double* euler_deg, const double* vel, const double* omega, sdfibm_solid_desc* out);

/* Parse a solidDict (OpenFOAM dictionary text) into solids and options (meta: on_fluid, on_twod, gravity).
 * Writes up to capacity solids; *nsolids receives the count.  rho_f is the transportProperties density
 * (0 is used when on_fluid is off).  msg (may be NULL) receives an error text. */
int sdfibm_host_parse_soliddict(const char* text, double rho_f, sdfibm_solid_desc* solids, int32_t capacity,
                                int32_t* nsolids, sdfibm_options* opt, int32_t* on_twod, char* msg, int32_t msg_len);

/* One entry of a solidDict by its '/'-separated path (e.g. "meta/writeFrequency", the reference's
 * meta.lookupOrDefault at src/solidcloud.cpp:37): its value tokens joined by single spaces, quotes removed, into buf as
 * the output functions below write text.  *len = -1 when the entry is absent (the caller's default applies); a path
 * that names a sub-dictionary, or text that does not parse, returns SDFIBM_ERR_ARG. */
int sdfibm_host_soliddict_lookup(const char* text, const char* path, char* buf, int64_t cap, int64_t* len);

/* The shape named `name` in a solidDict's shapes library (meta.sampler names the mean-field sampler this way,
 * src/solidcloud.cpp:38, 308); a repeated name keeps the first definition, as the library does. */
int sdfibm_host_soliddict_shape(const char* text, const char* name, sdfibm_shape_desc* out, char* msg,
                                int32_t msg_len);

/* ---- output: the state file and the restart dictionary --------------------------------------------------------------
 * Text results go to buf: at most cap bytes including the terminating NUL; *len receives the length of the whole
 * text (without the NUL).  buf == NULL with cap == 0 only measures; a buffer of cap <= *len returns
 * SDFIBM_ERR_CAPACITY. */

/* quaternion::eulerAngles(quaternion::XYZ) (OpenFOAM 12, as called at src/solid.cpp:12 and src/solidcloud.cpp:638):
 * the angles (radians) a, b, c with quat = qx(a) qy(b) qz(c), the inverse of sdfibm_host_quat_from_euler_deg for
 * |b| < 90 degrees and |a|, |c| < 180 degrees. */
void sdfibm_host_euler_from_quat(const double* quat_wxyz, double* euler_rad);

/* The records one SolidCloud::saveState appends to cloud.out (operator<<(SolidCloud) src/solidcloud.cpp:595-614,
 * operator<<(Solid) and write2D src/solid.cpp:5-29), a line per solid, every number as std::scientific with 6 digits:
 *   3-D: time pos.xyz vel.xyz force.xyz euler.xyz(radians) omega.xyz torque.xyz        (19 columns)
 *   2-D: time pos.x pos.y vel.x vel.y force.x force.y euler.z omega.z torque.z         (10 columns)
 * time is the time of the last SolidCloud::evolve (the construction time before the first). */
int sdfibm_host_format_state(double time, int32_t twod, const sdfibm_solid_state* states, int32_t n, char* buf,
                             int64_t cap, int64_t* len);

/* The line one SolidCloud::writeMeanField appends to meanfield.out (src/solidcloud.cpp:303-313): the mean field of
 * every solid (mean3[3*i .. 3*i+2]) as std::scientific with 6 digits, each number followed by a space, then a newline.
 * The means themselves come from the coupling (sdfibm_gb300.cloud.SolidCloud.mean_field: two forcing passes of the
 * sampler-shaped solids at rest). */
int sdfibm_host_format_mean_field(const double* mean3, int32_t n, char* buf, int64_t cap, int64_t* len);

/* SolidCloud::saveRestart (src/solidcloud.cpp:616-665): the solidDict text with pos, vel, euler (degrees) and omega
 * of the i-th entry of its `solids` sub-dictionary set from states[i] (2-D: pos.z, vel.z, omega.x and omega.y
 * written as 0), the tree written in OpenFOAM's dictionary layout with `precision` significant digits (the case's
 * writePrecision; 0: 6) after the solidDict file header, and a last line "// <stamp>" (NULL: the local time as
 * strftime "%y/%m/%d %X").  n must equal the number of entries of `solids`; errors return SDFIBM_ERR_ARG with a
 * message in msg (may be NULL). */
int sdfibm_host_write_restart(const char* dict_text, const sdfibm_solid_state* states, int32_t n, int32_t twod,
                              int32_t precision, const char* stamp, char* buf, int64_t cap, int64_t* len, char* msg,
                              int32_t msg_len);

/* ---- the VOF initializer (tool_vof): a smooth phase field from the solids' fractions ------------------------------
 * The field itself is one coupling pass: sdfibm_cuda_interact of these solids (REF-GEO fraction) leaves
 * As = min(sum of fractions, 1), the value tool_vof's SolidCloud::writeVOF accumulates with its clamp after every
 * solid (tool_vof/solidcloud.cpp:117-173). */

/* tool_vof's solidDict (tool_vof/solidcloud.cpp:12-112): meta.on_twod, the shapes library (a repeated name keeps the
 * last), and a solid of density 1 at rest per entry of "solids" (pos, euler in degrees, shp_name; 2-D: pos.z must
 * be 0), followed, when with_planes is set, by the entries of "planes" (as the shipped example's phase field
 * includes them).  Writes up to capacity solids; *nsolids receives the count. */
int sdfibm_host_parse_vofdict(const char* text, int32_t with_planes, sdfibm_solid_desc* solids, int32_t capacity,
                              int32_t* nsolids, int32_t* on_twod, char* msg, int32_t msg_len);

/* The uniform mesh of a blockMeshDict holding one axis-aligned hex block with simpleGrading (1 1 1): origin = the
 * block's lowest vertex, h = extent / cells, convertToMeters (or scale) applied; twod = 1 when nz == 1. */
int sdfibm_host_parse_blockmesh(const char* text, sdfibm_mesh_desc* mesh, char* msg, int32_t msg_len);

/* An OpenFOAM volScalarField file (file_len bytes, ascii or binary per its FoamFile format) with its internalField
 * replaced by `nonuniform List<scalar>` of the n values.  format: -1 keeps the file's, 0 ascii, 1 binary (the
 * case's writeFormat; the header's format word follows); ascii values carry `precision` significant digits (the
 * case's writePrecision; 0: 6).  Everything else in the file is kept byte for byte.  The result (binary fields hold
 * NUL bytes) goes to buf as the text functions above write it. */
int sdfibm_host_write_scalar_field(const char* file, int64_t file_len, const double* values, int64_t n,
                                   int32_t format, int32_t precision, char* buf, int64_t cap, int64_t* len, char* msg,
                                   int32_t msg_len);

/* The same for a volVectorField file: values holds n (x, y, z) triples (e.g. Fs or U transposed from the cell-major
 * planes), written as `nonuniform List<vector>`. */
int sdfibm_host_write_vector_field(const char* file, int64_t file_len, const double* values, int64_t n,
                                   int32_t format, int32_t precision, char* buf, int64_t cap, int64_t* len, char* msg,
                                   int32_t msg_len);

/* ---- OpenFOAM list files: polyMesh points / faces / owner / neighbour and field internalFields ---------------------
 * file: the file's bytes (ascii or binary per its FoamFile format; binary lists hold little-endian 8-byte scalars and
 * 4-byte labels, the reference's build).  out == NULL only measures. */
enum sdfibm_foam_kind { SDFIBM_FOAM_SCALAR = 0, SDFIBM_FOAM_VECTOR = 1, SDFIBM_FOAM_LABEL = 2 };

/* The list of an OpenFOAM file: for a vol*Field class the internalField (a uniform field gives *n = -1 and its value
 * in out[0] or out[0..2]), otherwise the first list after the header (points: VECTOR, owner/neighbour: LABEL).
 * out: doubles (SCALAR: n, VECTOR: 3 n) or int32 labels; cap in elements (vectors count once). */
int sdfibm_host_read_foam_list(const char* file, int64_t file_len, int32_t kind, void* out, int64_t cap, int64_t* n,
                               char* msg, int32_t msg_len);

/* A polyMesh faces file, faceCompactList (ascii or binary) or ascii faceList: offsets (nfaces + 1, from 0) and the
 * vertex labels of every face in order. */
int sdfibm_host_read_foam_faces(const char* file, int64_t file_len, int32_t* offsets, int64_t cap_offsets,
                                int32_t* labels, int64_t cap_labels, int64_t* nfaces, int64_t* nlabels, char* msg,
                                int32_t msg_len);

/* The uniform mesh whose point lattice these polyMesh points are (a single blockMesh block: x fastest, then y, then
 * z), every point within rtol of the mesh extent of its lattice position and ncells = nx ny nz; otherwise
 * SDFIBM_ERR_ARG.  Lets a case without its blockMeshDict take the uniform-mesh path. */
int sdfibm_host_uniform_mesh(const double* points, int64_t npoints, int64_t ncells, double rtol,
                             sdfibm_mesh_desc* mesh, char* msg, int32_t msg_len);

#ifdef __cplusplus
}
#endif
#endif /* SDFIBM_HOST_H */
