// The learned preconditioner: network definition, forward and backward passes,
// training on residual -> error pairs generated by the FEM operator, and the
// C ABI of include/plgpu_unet.h.
//
// Network (4 levels, 16/32/48/64 channels, channels-last BF16, FP32 accumulate):
//   x0  = relu(lift  (feat))                     level 0, 1x1x1, 16 -> 16
//   x1  = relu(enc1  (pool x0))                  level 1, 3x3x3, 16 -> 32
//   x2  = relu(enc2  (pool x1))                  level 2, 3x3x3, 32 -> 48
//   x3  = relu(enc3  (pool x2))                  level 3, 3x3x3, 48 -> 64
//   x3b = relu(bott  (x3))                       level 3, 3x3x3, 64 -> 64
//   p2  = proj2(x3b)                             level 3, 1x1x1, 64 -> 48
//   y2  = relu(dec2  (x2 + up p2))               level 2, 3x3x3, 48 -> 48
//   p1  = proj1(y2)                              level 2, 1x1x1, 48 -> 32
//   y1  = relu(dec1  (x1 + up p1))               level 1, 3x3x3, 32 -> 32
//   p0  = proj0(y1)                              level 1, 1x1x1, 32 -> 16
//   u   = head . (x0 + up p0)                    level 0, 16 -> 1
// pool = 2x2x2 average, up = copy to the 2x2x2 children.  No biases.  The
// preconditioner uses v = D^-1/2 u as the direction of a correction added to
// Jacobi with its A-norm optimal weight (unet_ops.cu), so only the shape of u matters.
//
// Training: errors e are Gaussian noise smoothed by damped Jacobi sweeps or by
// Jacobi-PCG iterations on the FEM operator (the components Jacobi-PCG reduces
// slowly), r = A e, loss 1 - (v, r)^2 / ((v, A v)(e, A e)); Adam on FP32 master weights.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#include "unet.h"
#include "unet_kernels.h"

namespace plgpu {

const UNetLayerDesc kUNetLayers[kUNetNumLayers] = {
    {"lift", 16, 16, 1},  {"enc1", 16, 32, 27},  {"enc2", 32, 48, 27}, {"enc3", 48, 64, 27}, {"bott", 64, 64, 27},
    {"proj2", 64, 48, 1}, {"dec2", 48, 48, 27},  {"proj1", 48, 32, 1}, {"dec1", 32, 32, 27}, {"proj0", 32, 16, 1},
};

namespace {
inline void ckc(cudaError_t e, const char* what) {
    if (e != cudaSuccess) throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString(e));
}
}  // namespace

UNetModel::UNetModel() {
    size_t o = 0;
    for (int l = 0; l < kUNetNumLayers; ++l) {
        off[l] = o;
        o += (size_t)kUNetLayers[l].taps * kUNetLayers[l].cout * kUNetLayers[l].cin;
    }
    off[kUNetNumLayers] = o;  // head weights follow the layers
    n_conv = o;
    n_params = o + kUNetHead;
}

UNetModel::~UNetModel() {
    for (void* p : {(void*)w, (void*)wb, (void*)wt, (void*)m, (void*)v, (void*)g, (void*)partial, (void*)dpartial,
                    (void*)head_bf16})
        if (p) cudaFree(p);
}

void UNetModel::allocate() {
    ckc(cudaMalloc(&w, n_params * 4), "cudaMalloc");
    ckc(cudaMalloc(&m, n_params * 4), "cudaMalloc");
    ckc(cudaMalloc(&v, n_params * 4), "cudaMalloc");
    ckc(cudaMalloc(&g, n_params * 4), "cudaMalloc");
    ckc(cudaMalloc(&wb, n_conv * 2), "cudaMalloc");
    ckc(cudaMalloc(&wt, n_conv * 2), "cudaMalloc");
    partial_floats = (size_t)4 << 20;  // 16 MiB of wgrad partials
    ckc(cudaMalloc(&partial, partial_floats * 4), "cudaMalloc");
    ckc(cudaMalloc(&dpartial, 4096 * 8), "cudaMalloc");
    ckc(cudaMalloc(&head_bf16, kUNetHead * 2), "cudaMalloc");
    ckc(cudaMemset(m, 0, n_params * 4), "memset");
    ckc(cudaMemset(v, 0, n_params * 4), "memset");
    ckc(cudaMemset(g, 0, n_params * 4), "memset");
}

// He-normal initial weights (deterministic in the seed), head weights small
void UNetModel::init(unsigned long long seed) {
    std::vector<float> h(n_params);
    unsigned long long s = seed * 6364136223846793005ull + 1442695040888963407ull;
    auto next = [&]() {
        s = s * 6364136223846793005ull + 1442695040888963407ull;
        return (double)((s >> 11) & ((1ull << 53) - 1)) / (double)(1ull << 53);
    };
    for (int l = 0; l < kUNetNumLayers; ++l) {
        const auto& L = kUNetLayers[l];
        const double std_ = std::sqrt(2.0 / (L.taps * L.cin));
        for (size_t t = off[l]; t < off[l + 1]; ++t) {
            const double u1 = next() + 1e-300, u2 = next();
            h[t] = (float)(std_ * std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2));
        }
    }
    for (int c = 0; c < kUNetHead; ++c) h[off[kUNetNumLayers] + c] = (float)(0.01 * (next() - 0.5));
    upload(h.data());
}

void UNetModel::upload(const float* host) {
    ckc(cudaMemcpy(w, host, n_params * 4, cudaMemcpyHostToDevice), "H2D weights");
    std::vector<uint16_t> hb(n_conv);
    for (size_t t = 0; t < n_conv; ++t) {
        uint32_t u;
        std::memcpy(&u, &host[t], 4);
        const uint32_t r = 0x7FFFu + ((u >> 16) & 1u);  // round to nearest even
        hb[t] = (uint16_t)((u + r) >> 16);
    }
    ckc(cudaMemcpy(wb, hb.data(), n_conv * 2, cudaMemcpyHostToDevice), "H2D weights");
    ckc(cudaMemset(m, 0, n_params * 4), "memset");
    ckc(cudaMemset(v, 0, n_params * 4), "memset");
    step = 0;
}

void UNetModel::download(float* host) const { ckc(cudaMemcpy(host, w, n_params * 4, cudaMemcpyDeviceToHost), "D2H"); }

// ---------------------------------------------------------------------------------------
// activations of one grid

static int half_up(int n) { return (n + 1) / 2; }

UNetWork::UNetWork(int a, int b, int c) {
    n[0][0] = a;
    n[0][1] = b;
    n[0][2] = c;
    for (int l = 1; l < 4; ++l)
        for (int d = 0; d < 3; ++d) n[l][d] = half_up(n[l - 1][d]);
    auto V = [&](int l) { return (size_t)n[l][0] * n[l][1] * n[l][2]; };
    auto bf = [&](bf16*& p, int l, int C) { ckc(cudaMalloc(&p, V(l) * C * 2), "cudaMalloc"); };
    bf(feat, 0, 16);
    bf(x0, 0, 16);
    bf(pool0, 1, 16);
    bf(x1, 1, 32);
    bf(pool1, 2, 32);
    bf(x2, 2, 48);
    bf(pool2, 3, 48);
    bf(x3, 3, 64);
    bf(x3b, 3, 64);
    bf(p2, 3, 48);
    bf(y2, 2, 48);
    bf(p1, 2, 32);
    bf(y1, 1, 32);
    bf(p0, 1, 16);
    // gradients
    bf(g_x0, 0, 16);
    bf(g_p0f, 0, 16);
    bf(g_p0, 1, 16);
    bf(g_dec1, 1, 32);
    bf(g_x1, 1, 32);
    bf(g_pool0, 1, 16);
    bf(g_p1, 2, 32);
    bf(g_dec2, 2, 48);
    bf(g_x2, 2, 48);
    bf(g_pool1, 2, 32);
    bf(g_p2, 3, 48);
    bf(g_bott, 3, 64);
    bf(g_enc3, 3, 64);
    bf(g_pool2, 3, 48);
    ckc(cudaMalloc(&u, V(0) * 4), "cudaMalloc");
    ckc(cudaMalloc(&gu, V(0) * 4), "cudaMalloc");
    ckc(cudaMalloc(&scal, 16 * 8), "cudaMalloc");
    ckc(cudaMemset(feat, 0, V(0) * 16 * 2), "memset");
}

UNetWork::~UNetWork() {
    for (void* p : {(void*)feat, (void*)x0, (void*)pool0, (void*)x1, (void*)pool1, (void*)x2, (void*)pool2, (void*)x3,
                    (void*)x3b, (void*)p2, (void*)y2, (void*)p1, (void*)y1, (void*)p0, (void*)g_x0, (void*)g_p0f,
                    (void*)g_p0, (void*)g_dec1, (void*)g_x1, (void*)g_pool0, (void*)g_p1, (void*)g_dec2, (void*)g_x2,
                    (void*)g_pool1, (void*)g_p2, (void*)g_bott, (void*)g_enc3, (void*)g_pool2, (void*)u, (void*)gu,
                    (void*)scal})
        if (p) cudaFree(p);
}

// ---------------------------------------------------------------------------------------
// passes

static ConvArgs conv_args(const UNetWork& W, int lvl, const bf16* in, const bf16* up, const bf16* w, bf16* out,
                          const bf16* gate, int relu) {
    ConvArgs a{};
    a.n0 = W.n[lvl][0];
    a.n1 = W.n[lvl][1];
    a.n2 = W.n[lvl][2];
    a.in = in;
    a.up = up;
    if (up != nullptr) {
        a.pn0 = W.n[lvl + 1][0];
        a.pn1 = W.n[lvl + 1][1];
    }
    a.w = w;
    a.out = out;
    a.out32 = nullptr;
    a.gate = gate;
    a.relu = relu;
    a.scale = 1.f;
    return a;
}

static void conv(const LaunchCfg& c, int layer, const ConvArgs& a) {
    const auto& L = kUNetLayers[layer];
    launch_conv(c, L.cin, L.cout, L.taps, a);
}
// input-gradient pass: the layer's (cout -> cin) transposed convolution
static void conv_t(const LaunchCfg& c, int layer, const ConvArgs& a) {
    const auto& L = kUNetLayers[layer];
    launch_conv(c, L.cout, L.cin, L.taps, a);
}

void unet_forward(const LaunchCfg& c, const UNetModel& M, UNetWork& W, const HeadArgs* head) {
    const bf16* wb = M.wb;
    auto wl = [&](int l) { return wb + M.off[l]; };
    conv(c, 0, conv_args(W, 0, W.feat, nullptr, wl(0), W.x0, nullptr, 1));
    launch_pool_avg(c, W.n[0][0], W.n[0][1], W.n[0][2], 16, W.x0, W.pool0);
    conv(c, 1, conv_args(W, 1, W.pool0, nullptr, wl(1), W.x1, nullptr, 1));
    launch_pool_avg(c, W.n[1][0], W.n[1][1], W.n[1][2], 32, W.x1, W.pool1);
    conv(c, 2, conv_args(W, 2, W.pool1, nullptr, wl(2), W.x2, nullptr, 1));
    launch_pool_avg(c, W.n[2][0], W.n[2][1], W.n[2][2], 48, W.x2, W.pool2);
    conv(c, 3, conv_args(W, 3, W.pool2, nullptr, wl(3), W.x3, nullptr, 1));
    conv(c, 4, conv_args(W, 3, W.x3, nullptr, wl(4), W.x3b, nullptr, 1));
    conv(c, 5, conv_args(W, 3, W.x3b, nullptr, wl(5), W.p2, nullptr, 0));
    conv(c, 6, conv_args(W, 2, W.x2, W.p2, wl(6), W.y2, nullptr, 1));
    conv(c, 7, conv_args(W, 2, W.y2, nullptr, wl(7), W.p1, nullptr, 0));
    conv(c, 8, conv_args(W, 1, W.x1, W.p1, wl(8), W.y1, nullptr, 1));
    conv(c, 9, conv_args(W, 1, W.y1, nullptr, wl(9), W.p0, nullptr, 0));
    if (head) launch_unet_head(c, *head);
}

HeadArgs unet_head_args(const UNetModel& M, const UNetWork& W, const float* r, const float* minv, const double* sigma2,
                        float* z) {
    HeadArgs h{};
    h.n0 = W.n[0][0];
    h.n1 = W.n[0][1];
    h.n2 = W.n[0][2];
    h.x0 = W.x0;
    h.p0 = W.p0;
    h.pn0 = W.n[1][0];
    h.pn1 = W.n[1][1];
    h.wh = M.w + M.off[kUNetNumLayers];
    h.r = r;
    h.minv = minv;
    h.sigma2 = sigma2;
    h.z = z;
    h.u = W.u;
    return h;
}

// weight gradient of one layer into M.g (chunks x taps blocks, then a fixed-order sum)
static void wgrad(const LaunchCfg& c, UNetModel& M, const UNetWork& W, int layer, int lvl, const bf16* x, const bf16* up,
                  const bf16* gout) {
    const auto& L = kUNetLayers[layer];
    WgradArgs a{};
    a.n0 = W.n[lvl][0];
    a.n1 = W.n[lvl][1];
    a.n2 = W.n[lvl][2];
    a.x = x;
    a.up = up;
    if (up) {
        a.pn0 = W.n[lvl + 1][0];
        a.pn1 = W.n[lvl + 1][1];
    }
    a.g = gout;
    a.partial = M.partial;
    const long long tiles = (long long)((a.n0 + 15) / 16) * ((a.n1 + 3) / 4) * a.n2;
    const size_t per = (size_t)L.taps * L.cout * L.cin;
    long long chunks = std::max<long long>(1, (long long)c.sm_count * 4 / L.taps);
    chunks = std::min<long long>(chunks, tiles);
    chunks = std::min<long long>(chunks, (long long)(M.partial_floats / per));
    launch_conv_wgrad(c, L.cin, L.cout, L.taps, a, (int)chunks);
    launch_reduce_partials(c, M.partial, (int)chunks, (int)per, 1.f, M.g + M.off[layer]);
}

void unet_backward(const LaunchCfg& c, UNetModel& M, UNetWork& W, const HeadArgs& head) {
    // transposed weights for the input-gradient passes
    for (int l = 0; l < kUNetNumLayers; ++l)
        launch_weights_for_dgrad(c, kUNetLayers[l].taps, kUNetLayers[l].cout, kUNetLayers[l].cin, M.wb + M.off[l],
                                 M.wt + M.off[l]);
    auto wtl = [&](int l) { return M.wt + M.off[l]; };
    // head: d x0 (gated), d p0 at level 0 (to be summed onto level 1), d head weights
    const int hblocks = std::min(c.sm_count * 4, 4096 / 16);
    launch_unet_head_backward(c, head, W.gu, W.g_x0, W.g_p0f, reinterpret_cast<float*>(M.dpartial), hblocks);
    launch_reduce_partials(c, reinterpret_cast<float*>(M.dpartial), hblocks, kUNetHead, 1.f, M.g + M.off[kUNetNumLayers]);
    launch_sum_children(c, W.n[0][0], W.n[0][1], W.n[0][2], 16, W.g_p0f, W.g_p0);
    // proj0 (linear, level 1): input y1
    wgrad(c, M, W, 9, 1, W.y1, nullptr, W.g_p0);
    conv_t(c, 9, conv_args(W, 1, W.g_p0, nullptr, wtl(9), W.g_dec1, W.y1, 0));  // d pre-activation of dec1
    // dec1 (level 1): input x1 + up p1
    wgrad(c, M, W, 8, 1, W.x1, W.p1, W.g_dec1);
    conv_t(c, 8, conv_args(W, 1, W.g_dec1, nullptr, wtl(8), W.g_x1, nullptr, 0));  // d (x1 + up p1)
    launch_sum_children(c, W.n[1][0], W.n[1][1], W.n[1][2], 32, W.g_x1, W.g_p1);
    // proj1 (level 2): input y2
    wgrad(c, M, W, 7, 2, W.y2, nullptr, W.g_p1);
    conv_t(c, 7, conv_args(W, 2, W.g_p1, nullptr, wtl(7), W.g_dec2, W.y2, 0));
    // dec2 (level 2): input x2 + up p2
    wgrad(c, M, W, 6, 2, W.x2, W.p2, W.g_dec2);
    conv_t(c, 6, conv_args(W, 2, W.g_dec2, nullptr, wtl(6), W.g_x2, nullptr, 0));
    launch_sum_children(c, W.n[2][0], W.n[2][1], W.n[2][2], 48, W.g_x2, W.g_p2);
    // proj2 (level 3): input x3b
    wgrad(c, M, W, 5, 3, W.x3b, nullptr, W.g_p2);
    conv_t(c, 5, conv_args(W, 3, W.g_p2, nullptr, wtl(5), W.g_bott, W.x3b, 0));
    // bott (level 3): input x3
    wgrad(c, M, W, 4, 3, W.x3, nullptr, W.g_bott);
    conv_t(c, 4, conv_args(W, 3, W.g_bott, nullptr, wtl(4), W.g_enc3, W.x3, 0));
    // enc3 (level 3): input pool2
    wgrad(c, M, W, 3, 3, W.pool2, nullptr, W.g_enc3);
    conv_t(c, 3, conv_args(W, 3, W.g_enc3, nullptr, wtl(3), W.g_pool2, nullptr, 0));
    // x2 receives the decoder's gradient and the pooled-path gradient; gate by x2 > 0
    launch_pool_avg_t(c, W.n[2][0], W.n[2][1], W.n[2][2], 48, W.g_pool2, W.x2, W.g_x2, 1);
    // enc2 (level 2): input pool1
    wgrad(c, M, W, 2, 2, W.pool1, nullptr, W.g_x2);
    conv_t(c, 2, conv_args(W, 2, W.g_x2, nullptr, wtl(2), W.g_pool1, nullptr, 0));
    launch_pool_avg_t(c, W.n[1][0], W.n[1][1], W.n[1][2], 32, W.g_pool1, W.x1, W.g_x1, 1);
    // enc1 (level 1): input pool0
    wgrad(c, M, W, 1, 1, W.pool0, nullptr, W.g_x1);
    conv_t(c, 1, conv_args(W, 1, W.g_x1, nullptr, wtl(1), W.g_pool0, nullptr, 0));
    launch_pool_avg_t(c, W.n[0][0], W.n[0][1], W.n[0][2], 16, W.g_pool0, W.x0, W.g_x0, 1);
    // lift (level 0): input feat
    wgrad(c, M, W, 0, 0, W.feat, nullptr, W.g_x0);
}

void unet_adam(const LaunchCfg& c, UNetModel& M, float lr) {
    ++M.step;
    const float b1 = 0.9f, b2 = 0.999f;
    const float bc1 = 1.f - std::pow(b1, (float)M.step), bc2 = 1.f - std::pow(b2, (float)M.step);
    // conv weights refresh their BF16 copy; the head stays FP32 (its bf16 slot is unused)
    launch_adam(c, (int)M.n_conv, M.w, M.m, M.v, M.g, M.wb, lr, b1, b2, 1e-8f, bc1, bc2, 10.f);
    launch_adam(c, kUNetHead, M.w + M.n_conv, M.m + M.n_conv, M.v + M.n_conv, M.g + M.n_conv, M.head_bf16, lr, b1, b2,
                1e-8f, bc1, bc2, 10.f);
}

// checksum of the weights file: FNV-1a 64 over the float bytes
uint64_t unet_checksum(const float* w, size_t n) {
    uint64_t h = 1469598103934665603ull;
    const unsigned char* p = reinterpret_cast<const unsigned char*>(w);
    for (size_t t = 0; t < n * 4; ++t) {
        h ^= p[t];
        h *= 1099511628211ull;
    }
    return h;
}

}  // namespace plgpu
