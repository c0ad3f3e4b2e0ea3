/*
 * plgpu_unet.h -- C ABI of the learned preconditioner of the GPU Static3D solver.
 *
 * No counterpart in the reference: PLaSK's iterative solve uses NSPCG's fixed
 * preconditioners (plask/common/fem/iterative_matrix.hpp:52-73).  A plgpu_unet
 * is a small 3D U-Net (4 levels, 16/32/48/64 channels, BF16 activations, FP32
 * accumulation) that maps a residual r to the shape of the smooth error that
 * Jacobi leaves.  Attached to a solver handle it is applied inside a flexible CG as
 *     v = D^-1/2 u(D^-1/2 r / sigma),  z = D^-1 r + ((v, r) / (v, A v)) v,
 * sigma^2 = (r, D^-1 r) / N and D the diagonal of the system matrix, with
 * Jacobi-PCG as fallback when the flexible CG stagnates.  Training uses residual -> error pairs that the FEM
 * operator of a solver handle generates.
 *
 * All functions return PLGPU_OK (0) or a negative code (include/plgpu_fem3d.h).
 */
#ifndef PLGPU_UNET_H
#define PLGPU_UNET_H

#include <stddef.h>
#include <stdint.h>

#include "plgpu_fem3d.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct plgpu_unet plgpu_unet;

/* Create a network with He-normal weights drawn from `seed`. */
int plgpu_unet_create(unsigned long long seed, plgpu_unet** out);
int plgpu_unet_destroy(plgpu_unet* net);
const char* plgpu_unet_last_error(const plgpu_unet* net);

/* Number of parameters (FP32 master weights: conv layers then 16 head weights). */
int plgpu_unet_num_params(const plgpu_unet* net, size_t* n);
int plgpu_unet_get_weights(plgpu_unet* net, float* out);
/* Replace the weights (also resets the optimiser state). */
int plgpu_unet_set_weights(plgpu_unet* net, const float* in);

/* Weights file: 8-byte magic "PLGPUNET", uint32 version, uint64 count, count
   floats, uint64 FNV-1a checksum of the float bytes. */
int plgpu_unet_save(plgpu_unet* net, const char* path);
int plgpu_unet_load(plgpu_unet* net, const char* path);

/* Train for `steps` Adam steps on pairs generated with the system matrix of the
   solver handle at its current temperature.  The error e starts as Gaussian
   noise and is smoothed by m steps, m uniform in [smooth_min, smooth_max]:
   pair_kind 0: damped-Jacobi sweeps; 1: Jacobi-PCG iterations on A e = 0 (the
   error CG leaves behind), then scaled to unit RMS.  r = A e; the loss is the
   relative A-norm error left along the network direction v at its optimal
   weight: 1 - (v, r)^2 / ((v, A v)(e, A e)).
   losses (may be NULL) receives one loss per step. */
int plgpu_unet_train(plgpu_unet* net, plgpu_fem3d* fem, int steps, float lr, unsigned long long seed, int smooth_min,
                     int smooth_max, int pair_kind, float* losses);

/* Loss and full gradient for a given error e (full node array, mesh order), for
   gradient checks: r = A e (FP32 operator), loss as above.  r_out (may be NULL)
   receives r and z_out (may be NULL) the preconditioned residual z, both in mesh order. */
int plgpu_unet_loss_grad(plgpu_unet* net, plgpu_fem3d* fem, const double* e, double* loss, float* grad, double* r_out,
                         double* z_out);

/* Apply the preconditioner to a residual (full node arrays, mesh order). */
int plgpu_unet_apply(plgpu_unet* net, plgpu_fem3d* fem, const double* r, double* z);

/* Device time [ms] of one network forward pass and of one whole preconditioner
   application (forward, A v, two dot products, combination) on the handle's mesh,
   averaged over reps after one untimed pass (CUDA events on the solver's stream). */
int plgpu_unet_time_apply(plgpu_unet* net, plgpu_fem3d* fem, int reps, double* forward_ms, double* apply_ms);

/* Attach the network to a solver handle (NULL detaches); used by PLGPU_ALGO_GPU_LEARNED.
   The handle keeps a pointer: the network must outlive the attachment. */
int plgpu_fem3d_set_preconditioner(plgpu_fem3d* fem, plgpu_unet* net);

#ifdef __cplusplus
}
#endif

#endif /* PLGPU_UNET_H */
