/* Learned cut-cell fraction for the GB300 coupling library.
 *
 * No counterpart in the reference: sdfibm computes the solid fraction of a cut cell only with the apex / pyramid
 * geometry of GeometricTools::calcCellVolume (src/geometrictools.cpp:47-116).  These entry points build, train and
 * run a model that predicts the SUBSAMPLE fraction (a stratified n^3 lattice of Shape::isInside tests,
 * SDFIBM_FRACTION_SUBSAMPLE in sdfibm_cuda.h) from signed distances sampled in the cell.  The coupling path uses it
 * with options.fraction_method = SDFIBM_FRACTION_LEARNED after sdfibm_cuda_set_fraction_model.
 *
 * Model: a = sigmoid(logit(P4) + network(x)).
 *   stencil: Shape::signedDistance at the 5 x 5 x 5 lattice of the cell (spacing h/4 per axis, vertices included).
 *   P4, P2: sub-cell planar reconstructions of the fraction: the cell cut into 4^3 (2^3) sub-cells, each sub-cell's
 *           fraction the exact cube-plane volume under the plane fitted to its 8 corner distances (Scardovelli &
 *           Zaleski, J. Comput. Phys. 164 (2000)), averaged; both clamped to [1e-4, 1 - 1e-4].
 *   x (16 network inputs): phi/h at the 8 vertices (OpenFOAM cellPoints order of a hex: (i,j,k) (i+1,j,k) (i,j+1,k)
 *           (i+1,j+1,k), then the same at k+1), at the 6 face centres (-x, +x, -y, +y, -z, +z), at the cell centre,
 *           then logit(P2).
 *   network: 16 -> 64 -> 64 -> 1, SiLU hidden units; the hidden layers run on the tensor cores (tcgen05, BF16 x BF16
 *           -> FP32 in tensor memory) with W1, W2 rounded to BF16; inputs and first-layer activations are split into
 *           a hi + lo pair of BF16 values, so the products keep about 16 significant bits; biases, the output layer
 *           and the sigmoid are FP32.
 * Parameters: one FP32 array of SDFIBM_MLP_NPARAM values, W1[64][16], b1[64], W2[64][64], b2[64], w3[64], b3
 *             (row = output unit).
 * Feature buffers are structure-of-arrays with SDFIBM_MLP_NFEAT rows: row f < 16 is input f, row 16 the prior
 * logit(P4); row f of cell c at feat[f * stride + c].
 *
 * All pointers named *_dev are device memory owned by the caller; `stream` is a cudaStream_t (NULL: the legacy
 * default stream).  Functions return 0 (SDFIBM_OK) or a negative sdfibm_status; they synchronise the stream
 * before returning so that errors are reported by the call that caused them.
 */
#ifndef SDFIBM_MLP_H
#define SDFIBM_MLP_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SDFIBM_MLP_NIN 16
#define SDFIBM_MLP_NFEAT 17 /* rows of a feature buffer: the 16 network inputs, then the prior logit(P4) */
#define SDFIBM_MLP_NHIDDEN 64
#define SDFIBM_MLP_NPARAM 5313
#define SDFIBM_MLP_ERR_TIMEOUT 7 /* device error code: an MMA completion was not observed within the wait limit */

/* Shape families of the generated training cells (bit mask in sdfibm_mlp_data_desc.families). */
enum {
    SDFIBM_MLP_SPHERE = 1,
    SDFIBM_MLP_ELLIPSOID = 2,      /* semi-axes r * (1, U[1,3], U[1,3]) */
    SDFIBM_MLP_BOX = 4,            /* half extents r * (1, U[1,3], U[1,3]) */
    SDFIBM_MLP_PLANE = 8,
    SDFIBM_MLP_CYLINDER = 16,      /* Circle: the 2-D shape, infinite along its local z */
    SDFIBM_MLP_ELLIPTIC_CYL = 32   /* Ellipse, axes r * (1, U[1,3]) */
};

typedef struct sdfibm_mlp_data_desc {
    double hr_min, hr_max;   /* cell size / radius, log-uniform in [hr_min, hr_max] */
    int32_t families;        /* bit mask of the families above, drawn with equal weight */
    int32_t n_sub;           /* label lattice: n_sub^3 isInside samples per cell (16 -> 4096) */
    double z_axis_frac;      /* fraction of Circle / Ellipse cells whose axis is the mesh z axis (2-D meshes) */
} sdfibm_mlp_data_desc;

/* Generates n labelled cut cells (cells with 1..7 vertices inside).  feat_dev: [SDFIBM_MLP_NFEAT][n] (inputs and
 * prior, computed in FP32 as the coupling path computes them); label_dev: [n], the fraction of the n_sub^3 lattice
 * points inside (FP64 inside tests); recipe_dev (may be NULL): [n][20] FP64 description of each cell for checking:
 * shape type, 8 shape parameters (sdfibm_shape_desc.p), quaternion (w,x,y,z), cell corner (3), h, inside-vertex
 * count, attempts.  Shapes sit at the origin; the cell size is h = 1. */
int sdfibm_mlp_dataset(uint64_t seed, int64_t n, const sdfibm_mlp_data_desc* desc, float* feat_dev, float* label_dev,
                       double* recipe_dev, void* stream);

/* Predicted fraction of n cells: out_dev[c] = sigmoid(feat[16][c] + network(feat[0..15][c])); params_dev is FP32
 * [SDFIBM_MLP_NPARAM]; feat_dev holds SDFIBM_MLP_NFEAT rows of `stride` entries. */
int sdfibm_mlp_forward(const float* params_dev, const float* feat_dev, int64_t stride, int64_t n, float* out_dev,
                       void* stream);

/* Gradient of loss = mean over the n cells of (a - label)^2.  grad_dev: FP32 [SDFIBM_MLP_NPARAM + 1], overwritten:
 * the gradient, then the sum of (a - label)^2. */
int sdfibm_mlp_loss_grad(const float* params_dev, const float* feat_dev, const float* label_dev, int64_t stride,
                         int64_t n, float* grad_dev, void* stream);

/* One Adam step (beta1 0.9, beta2 0.999, eps 1e-8; t counts from 1) on FP32 parameters and moments. */
int sdfibm_mlp_adam(float* params_dev, const float* grad_dev, float* m_dev, float* v_dev, int32_t t, float lr,
                    void* stream);

typedef struct sdfibm_mlp_train_desc {
    int32_t epochs;
    int32_t batch;           /* cells per step */
    float lr;                /* peak learning rate; cosine decay to lr * lr_final_frac after a linear warm-up */
    float lr_final_frac;
    int32_t warmup_steps;
    int32_t reserved;
} sdfibm_mlp_train_desc;

/* Trains params_dev in place on n cells with Adam; loss_per_epoch_host (may be NULL) receives the mean loss of each
 * epoch.  The GPU's own forward and backward kernels (sdfibm_mlp_loss_grad) compute every gradient. */
int sdfibm_mlp_train(float* params_dev, const float* feat_dev, const float* label_dev, int64_t n,
                     const sdfibm_mlp_train_desc* desc, float* loss_per_epoch_host, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* SDFIBM_MLP_H */
