/*
 * chgpu_closure.h -- the learned subgrid-stress closure of the coarse
 * channel solver: a pointwise network (10 -> 64 -> 64 -> 64 -> 6, SiLU,
 * BF16 weights with FP32 accumulation on the tensor cores) that maps the
 * resolved velocity gradients and the wall distance of a grid point to the
 * six subgrid stresses tau_ij = filter(u_i u_j) - filter(u_i) filter(u_j).
 *
 * None of these entry points has a counterpart in the reference: the
 * reference has no closure.  Its natural insertion point is where the six
 * velocity products are formed in physical space (dnsdata.f90:581-584):
 * the coarse solver adds tau_ij to uu, vv, ww, uv, vw, uw there, so the
 * subgrid flux enters the explicit terms of buildrhs (dnsdata.f90:611-673)
 * through the same derivatives as the resolved one.
 *
 * Conventions as in chgpu.h: 0 on success, a negative CHGPU_E_* code
 * otherwise, with the message in chgpu_mlp_last_error.  Host arrays are
 * owned by the caller and copied.
 */
#ifndef CHGPU_CLOSURE_H
#define CHGPU_CLOSURE_H

#include "chgpu.h"

#ifdef __cplusplus
extern "C" {
#endif

#define CHGPU_MLP_IN 10     /* du/dx du/dy du/dz dv/dx dv/dy dv/dz dw/dx dw/dy dw/dz, wall distance */
#define CHGPU_MLP_HIDDEN 64
#define CHGPU_MLP_OUT 6     /* tau_uu tau_vv tau_ww tau_uv tau_vw tau_uw: the order of the products */
/* Parameter vector (FP32 master copy), in this order:
 *   W1[64][16]  (columns 0..9 the inputs, column 10 the bias, 11..15 zero)
 *   W2[64][64], b2[64], W3[64][64], b3[64], W4[6][64], b4[6]
 * W[o][i] multiplies input i into output o. */
#define CHGPU_MLP_NPARAMS 9734

typedef struct chgpu_mlp chgpu_mlp;

/* Affine normalisation: the network sees (x - mu_in) / sd_in and its outputs
 * are y * sd_out + mu_out. */
typedef struct chgpu_mlp_norm {
  float mu_in[CHGPU_MLP_IN], sd_in[CHGPU_MLP_IN];
  float mu_out[CHGPU_MLP_OUT], sd_out[CHGPU_MLP_OUT];
} chgpu_mlp_norm;

/* Weights drawn uniform in +-sqrt(6 / fan_in) (SiLU layers) or +-sqrt(3 /
 * fan_in) (output layer) from a seeded generator; biases zero; identity
 * normalisation.  Needs a GB300 (tensor-core generation 5). */
int chgpu_mlp_create(unsigned long long seed, chgpu_mlp** out);
int chgpu_mlp_destroy(chgpu_mlp* m);
const char* chgpu_mlp_last_error(const chgpu_mlp* m);

int chgpu_mlp_set_params(chgpu_mlp* m, const float* theta);  /* CHGPU_MLP_NPARAMS floats */
int chgpu_mlp_get_params(chgpu_mlp* m, float* theta);
int chgpu_mlp_set_norm(chgpu_mlp* m, const chgpu_mlp_norm* nm);
int chgpu_mlp_get_norm(chgpu_mlp* m, chgpu_mlp_norm* nm);

/* Training set, structure of arrays: feat[CHGPU_MLP_IN][n], targ[CHGPU_MLP_OUT][n]
 * (physical units; the normalisation is applied on the device). */
int chgpu_mlp_set_data(chgpu_mlp* m, const float* feat, const float* targ, long long n);
long long chgpu_mlp_data_size(const chgpu_mlp* m);

/* Loss L = mean over points and outputs of (y - t)^2 in normalised units,
 * on the resident points first, first+1, ... (count of them, wrapping at n;
 * count a multiple of 128), and its gradient with respect to the parameter
 * vector (grad may be NULL).  Adds nothing to the optimiser state. */
int chgpu_mlp_gradient(chgpu_mlp* m, long long first, long long count, float* grad, double* loss);

/* `steps` Adam steps (beta1 0.9, beta2 0.999, eps 1e-8, learning rate lr) on
 * consecutive windows of `batch` resident points (a multiple of 128),
 * continuing where the previous call stopped; the loss of each step goes
 * to loss_out[step] when it is not NULL. */
int chgpu_mlp_train(chgpu_mlp* m, int steps, long long batch, float lr, double* loss_out);

/* Network outputs in physical units: out[CHGPU_MLP_OUT][n] from feat[CHGPU_MLP_IN][n]. */
int chgpu_mlp_predict(chgpu_mlp* m, const float* feat, long long n, float* out);

/* ---- the closure inside a channel handle ---- */

/* Closure points of a handle: the physical grid of its convolutions (the
 * 3/2-padded x and z points, dnsdata.f90:110-114) on the planes iy = 1..ny-1:
 * dims = {2 nxd, nzd, ny-1}; npts = their product, x fastest, then z, then y. */
int chgpu_closure_dims(chgpu_handle* h, int dims[3]);

/* Attach a network: with enable = 1 every convolution pass of the step
 * evaluates the network at the closure points of the current field and adds
 * tau_ij to the six products there (walls and ghost planes get none);
 * enable = 0 detaches it -- the plain under-resolved solver, the fallback.
 * The handle keeps the pointer: the network must outlive the attachment,
 * and must not be trained (chgpu_mlp_train / _set_params / _set_norm) while
 * an attached handle's steps are in flight -- they read its weights on the
 * handle's stream.  The next step is captured anew. */
int chgpu_closure_attach(chgpu_handle* h, chgpu_mlp* m, int enable);

/* A prescribed tau instead of the network: tau[6][npts] (FP32) added to the
 * products at the closure points in every convolution pass; NULL removes it.
 * An attached, enabled network takes precedence. */
int chgpu_closure_set_tau(chgpu_handle* h, const float* tau);

/* The network's inputs for the current field: feat[10][npts] -- the nine
 * velocity gradients (d/dx, d/dz spectral; d/dy the compact derivative of
 * COMPLEXderiv, dnsdata.f90:339-373) transformed to the closure points in
 * FP32, and the wall distance min(y - ymin, ymax - y). */
int chgpu_closure_features(chgpu_handle* h, float* feat);

/* Physical values at the closure points of ncomp (3, 6 or 9) spectral fields
 * of this handle's size, given in the restart-field layout
 * [ncomp][nx+1][2nz+1][ny+3] complex128: out[ncomp][npts] (FP32 transforms). */
int chgpu_closure_physical(chgpu_handle* h, const double* spec, int ncomp, float* out);

/* The six product spectra uu vv ww uv vw uw of the current field, as the
 * convolutions pass computes them (dnsdata.f90:487-602; no closure term), in
 * the restart-field layout [6][nx+1][2nz+1][ny+3] complex128.  The subgrid
 * stresses of a coarse field are the fine products at the coarse modes minus
 * the coarse products of the truncated field. */
int chgpu_products(chgpu_handle* h, double* out);

#ifdef __cplusplus
}
#endif

#endif /* CHGPU_CLOSURE_H */
