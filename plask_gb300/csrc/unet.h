// Host-side model and activation buffers of the learned preconditioner (unet.cu).
#pragma once

#include <cuda_bf16.h>

#include <cstddef>
#include <cstdint>

#include "unet_kernels.h"

namespace plgpu {

using bf16 = __nv_bfloat16;

struct UNetLayerDesc {
    const char* name;
    int cin, cout, taps;
};
constexpr int kUNetNumLayers = 10;
constexpr int kUNetHead = 16;
extern const UNetLayerDesc kUNetLayers[kUNetNumLayers];

// Weights (FP32 master, BF16 copy, transposed BF16 for the input-gradient pass),
// Adam moments, gradient, and scratch of the weight-gradient reduction.
struct UNetModel {
    size_t off[kUNetNumLayers + 1];  // offsets of the layers' weights; off[L] = head
    size_t n_conv = 0, n_params = 0;
    float* w = nullptr;
    bf16* wb = nullptr;
    bf16* wt = nullptr;
    float* m = nullptr;
    float* v = nullptr;
    float* g = nullptr;
    float* partial = nullptr;
    size_t partial_floats = 0;
    double* dpartial = nullptr;
    bf16* head_bf16 = nullptr;  // unused BF16 copy of the head weights written by the optimiser
    int step = 0;
    UNetModel();
    ~UNetModel();
    void allocate();
    void init(unsigned long long seed);
    void upload(const float* host);  // also resets the optimiser
    void download(float* host) const;
};

// Activations and their gradients for one node grid.
struct UNetWork {
    int n[4][3];
    bf16 *feat = nullptr, *x0 = nullptr, *pool0 = nullptr, *x1 = nullptr, *pool1 = nullptr, *x2 = nullptr,
         *pool2 = nullptr, *x3 = nullptr, *x3b = nullptr, *p2 = nullptr, *y2 = nullptr, *p1 = nullptr, *y1 = nullptr,
         *p0 = nullptr;
    bf16 *g_x0 = nullptr, *g_p0f = nullptr, *g_p0 = nullptr, *g_dec1 = nullptr, *g_x1 = nullptr, *g_pool0 = nullptr,
         *g_p1 = nullptr, *g_dec2 = nullptr, *g_x2 = nullptr, *g_pool1 = nullptr, *g_p2 = nullptr, *g_bott = nullptr,
         *g_enc3 = nullptr, *g_pool2 = nullptr;
    float* u = nullptr;
    float* gu = nullptr;
    double* scal = nullptr;  // device scalars: [0] sigma^2 N, [1] e^T A e, [2] d^T A d, [3..] spare
    UNetWork(int n0, int n1, int n2);
    ~UNetWork();
    UNetWork(const UNetWork&) = delete;
    UNetWork& operator=(const UNetWork&) = delete;
};

void unet_forward(const LaunchCfg& c, const UNetModel& M, UNetWork& W, const HeadArgs* head);
HeadArgs unet_head_args(const UNetModel& M, const UNetWork& W, const float* r, const float* minv, const double* sigma2,
                        float* z);
void unet_backward(const LaunchCfg& c, UNetModel& M, UNetWork& W, const HeadArgs& head);
void unet_adam(const LaunchCfg& c, UNetModel& M, float lr);
uint64_t unet_checksum(const float* w, size_t n);

}  // namespace plgpu
