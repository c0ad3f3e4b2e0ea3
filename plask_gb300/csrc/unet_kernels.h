// Launchers of the U-Net preconditioner kernels (unet_kernels.cu, unet_ops.cu).
#pragma once

#include <cuda_bf16.h>

#include "fem3d_kernels.h"

namespace plgpu {

// y = conv(x (+ up(coarse))), optional ReLU / ReLU gate; all tensors channels-last BF16
struct ConvArgs {
    int n0, n1, n2;                 // voxel extents of this level
    const __nv_bfloat16* in;        // [V][CIN]
    const __nv_bfloat16* up;        // optional [Vc][CIN] of the next coarser level, added at each child
    int pn0, pn1;                   // extents of the coarser level (for `up`)
    const __nv_bfloat16* w;         // [taps][COUT][CIN]
    __nv_bfloat16* out;             // [V][COUT] (may be null)
    float* out32;                   // [V][COUT] FP32 copy (may be null)
    const __nv_bfloat16* gate;      // optional [V][COUT]: zero the result where gate <= 0
    int relu;
    float scale;
};

// partial[chunk][tap][COUT][CIN] = sum over the chunk's tiles of X(v + off(tap)) G(v)
struct WgradArgs {
    int n0, n1, n2;
    const __nv_bfloat16* x;         // conv input [V][CIN]
    const __nv_bfloat16* up;        // optional coarse tensor added to x (as in the forward pass)
    int pn0, pn1;
    const __nv_bfloat16* g;         // gradient w.r.t. the pre-activation output [V][COUT]
    float* partial;
};

bool conv_supported(int cin, int cout, int taps);
void launch_conv(const LaunchCfg& c, int cin, int cout, int taps, const ConvArgs& a);
void launch_conv_wgrad(const LaunchCfg& c, int cin, int cout, int taps, const WgradArgs& a, int chunks);
void launch_reduce_partials(const LaunchCfg& c, const float* partial, int chunks, int n, float scale, float* out);
void launch_pool_avg(const LaunchCfg& c, int n0, int n1, int n2, int C, const __nv_bfloat16* in, __nv_bfloat16* out);
void launch_pool_avg_t(const LaunchCfg& c, int n0, int n1, int n2, int C, const __nv_bfloat16* coarse,
                       const __nv_bfloat16* gate, __nv_bfloat16* fine, int accumulate);
void launch_sum_children(const LaunchCfg& c, int n0, int n1, int n2, int C, const __nv_bfloat16* fine,
                         __nv_bfloat16* coarse);
void launch_weights_for_dgrad(const LaunchCfg& c, int taps, int cout, int cin, const __nv_bfloat16* w,
                              __nv_bfloat16* wt);
void launch_adam(const LaunchCfg& c, int n, float* w, float* m, float* v, const float* g, __nv_bfloat16* wb, float lr,
                 float b1, float b2, float eps, float bc1, float bc2, float clip);

// --- preconditioner glue (unet_ops.cu) -------------------------------------------------

// static features of the node grid, channels 1..15 of the input tensor (channel 0 is the residual)
void launch_unet_features(const LaunchCfg& c, const GridT<float>& g, const float* kxy, const float* kz, bool aniso,
                          const float* minv, __nv_bfloat16* feat);
// channel 0 of the input tensor: D^-1/2 r / sigma
void launch_unet_input(const LaunchCfg& c, long long N, const float* r, const float* minv, const double* sigma2_slot,
                       __nv_bfloat16* feat);
// u[v] = sum_c wh[c] (x0[v][c] + p0[parent][c]) and the correction direction v = D^-1/2 u
struct HeadArgs {
    int n0, n1, n2;
    const __nv_bfloat16* x0;   // [V][16]
    const __nv_bfloat16* p0;   // [Vc][16] on level 1
    int pn0, pn1;
    const float* wh;           // [16]
    const float* r;
    const float* minv;
    const double* sigma2;      // device scalar: sigma^2
    float* z;                  // output v = D^-1/2 u (may be null)
    float* u;                  // raw network output (may be null)
};
void launch_unet_head(const LaunchCfg& c, const HeadArgs& a);
// backward of the head: gu = d loss / d u given; writes d x0 (gated by x0 > 0), d p0 and
// per-block partials of d wh
void launch_unet_head_backward(const LaunchCfg& c, const HeadArgs& a, const float* gu, __nv_bfloat16* dx0,
                               __nv_bfloat16* dp0_fine, float* dwh_partial, int blocks);

// training-pair generation and loss
void launch_noise(const LaunchCfg& c, long long N, unsigned long long seed, const float* minv, float* e);
void launch_jacobi_sweep(const LaunchCfg& c, long long N, float omega, const float* minv, const float* ae, float* e);
void launch_sub(const LaunchCfg& c, long long N, const float* a, const float* b, float* d);
void launch_loss_grad_u(const LaunchCfg& c, long long N, const float* r, const float* av, const float* minv,
                        const double* sc, float* gu);
void launch_precond_combine(const LaunchCfg& c, long long N, const float* r, const float* minv, const float* v,
                            const double* sc, float* z);
void launch_scale_rms(const LaunchCfg& c, long long N, const double* s, float* e);
// *out = (x, y), deterministic (partial: >= 8 * sm_count doubles)
void launch_dot(const LaunchCfg& c, long long N, const float* x, const float* y, double* partial, double* out);
// *out = (r, M^-1 r)
void launch_rmr(const LaunchCfg& c, long long N, const float* r, const float* minv, double* partial, double* out);

}  // namespace plgpu
