// Glue between the FEM operator and the U-Net preconditioner: input features,
// the output head (and its backward pass).
//
// The preconditioner maps a residual r to
//     v = D^-1/2 u(D^-1/2 r / sigma),   c = (v, r) / (v, A v),   z = M^-1 r + c v,
// M = D = diag(A) (Jacobi), u the network output on the node grid and
// sigma^2 = (r, D^-1 r) / N.  The network supplies the shape of a smooth
// correction (the components Jacobi misses); its weight c is the one that
// minimises the A-norm error along v, so the network never has to produce the
// large gain of the inverse operator on smooth modes.  z is linear in the scale
// of r.  Nodes with M^-1 = 0 (Dirichlet, masked) get z = 0.
#include <cuda_bf16.h>

#include <cmath>

#include "unet_kernels.h"

namespace plgpu {

using bf16 = __nv_bfloat16;
constexpr int kFeat = 16;  // channels of the input tensor

__device__ __forceinline__ long long vox3(int i, int j, int k, int n0, int n1) {
    return ((long long)k * n1 + j) * n0 + i;
}

// channels 1..4: local anisotropy and conductance scale; 5..15 zero
__global__ void __launch_bounds__(256) k_unet_features(const GridT<float> g, const float* __restrict__ kxy,
                                                       const float* __restrict__ kz, int aniso,
                                                       const float* __restrict__ minv, bf16* __restrict__ feat) {
    const int n0 = g.n0, n1 = g.n1, n2 = g.n2;
    const long long N = g.N, s2 = (long long)n0 * n1;
    for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < N; n += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(n % n0), j = (int)((n / n0) % n1), k = (int)(n / s2);
        float sx = 0.f, sy = 0.f, sz = 0.f;
        for (int c = 0; c < 8; ++c) {
            const int e0 = i - (c & 1), e1 = j - ((c >> 1) & 1), e2 = k - (c >> 2);
            if (e0 < 0 || e0 >= n0 - 1 || e1 < 0 || e1 >= n1 - 1 || e2 < 0 || e2 >= n2 - 1) continue;
            const long long e = e0 + (long long)n0 * (e1 + (long long)n1 * e2);
            const float kk = kxy[e], kv = aniso ? kz[e] : kk;
            const float dx = g.h0[e0], dy = g.h1[e1], dz = g.h2[e2];
            sx += kk * dy * dz * g.r0[e0];
            sy += kk * dx * dz * g.r1[e1];
            sz += kv * dx * dy * g.r2[e2];
        }
        const float tiny = 1e-30f;
        float f[kFeat];
#pragma unroll
        for (int c = 0; c < kFeat; ++c) f[c] = 0.f;
        f[1] = fminf(fmaxf(0.25f * logf((sx + tiny) / (sz + tiny)), -4.f), 4.f);
        f[2] = fminf(fmaxf(0.25f * logf((sy + tiny) / (sz + tiny)), -4.f), 4.f);
        f[3] = minv[n] == 0.f ? 1.f : 0.f;
        f[4] = fminf(fmaxf(0.1f * log10f(sx + sy + sz + tiny), -4.f), 4.f);
        bf16* out = feat + n * kFeat;
#pragma unroll
        for (int c = 1; c < kFeat; ++c) out[c] = __float2bfloat16(f[c]);
    }
}

__global__ void __launch_bounds__(256) k_unet_input(long long N, const float* __restrict__ r,
                                                    const float* __restrict__ minv, const double* __restrict__ sig2,
                                                    bf16* __restrict__ feat) {
    const double s2 = *sig2 / (double)N;
    const float inv = s2 > 0.0 ? (float)(1.0 / sqrt(s2)) : 0.f;
    for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < N; n += (long long)gridDim.x * blockDim.x)
        feat[n * kFeat] = __float2bfloat16(sqrtf(minv[n]) * r[n] * inv);
}

// v = D^-1/2 u on free nodes (0 where M^-1 = 0); u is also kept for the backward pass
__global__ void __launch_bounds__(256) k_unet_head(const HeadArgs a) {
    const int n0 = a.n0, n1 = a.n1, n2 = a.n2;
    const long long N = (long long)n0 * n1 * n2;
    float wh[kFeat];
#pragma unroll
    for (int c = 0; c < kFeat; ++c) wh[c] = a.wh[c];
    for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < N; n += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(n % n0), j = (int)((n / n0) % n1), k = (int)(n / ((long long)n0 * n1));
        const bf16* x = a.x0 + n * kFeat;
        const bf16* p = a.p0 + vox3(i >> 1, j >> 1, k >> 1, a.pn0, a.pn1) * kFeat;
        float u = 0.f;
#pragma unroll
        for (int c = 0; c < kFeat; ++c) u += wh[c] * (__bfloat162float(x[c]) + __bfloat162float(p[c]));
        const float m = a.minv[n];
        if (a.u) a.u[n] = u;
        if (a.z) a.z[n] = m > 0.f ? sqrtf(m) * u : 0.f;
    }
}

__global__ void __launch_bounds__(256) k_unet_head_bwd(const HeadArgs a, const float* __restrict__ gu,
                                                       bf16* __restrict__ dx0, bf16* __restrict__ dp0f,
                                                       float* __restrict__ dwh_partial) {
    const int n0 = a.n0, n1 = a.n1, n2 = a.n2;
    const long long N = (long long)n0 * n1 * n2;
    float wh[kFeat], acc[kFeat];
#pragma unroll
    for (int c = 0; c < kFeat; ++c) {
        wh[c] = a.wh[c];
        acc[c] = 0.f;
    }
    for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < N; n += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(n % n0), j = (int)((n / n0) % n1), k = (int)(n / ((long long)n0 * n1));
        const bf16* x = a.x0 + n * kFeat;
        const bf16* p = a.p0 + vox3(i >> 1, j >> 1, k >> 1, a.pn0, a.pn1) * kFeat;
        const float g = gu[n];
#pragma unroll
        for (int c = 0; c < kFeat; ++c) {
            const float xv = __bfloat162float(x[c]);
            acc[c] += g * (xv + __bfloat162float(p[c]));
            const float d = g * wh[c];
            dx0[n * kFeat + c] = __float2bfloat16(xv > 0.f ? d : 0.f);
            dp0f[n * kFeat + c] = __float2bfloat16(d);
        }
    }
    // block reduction of the head-weight gradient
    __shared__ float sh[kFeat][8];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int c = 0; c < kFeat; ++c) {
        float v = acc[c];
        for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0) sh[c][warp] = v;
    }
    __syncthreads();
    if (threadIdx.x < kFeat) {
        float s = 0.f;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += sh[threadIdx.x][w];
        dwh_partial[blockIdx.x * kFeat + threadIdx.x] = s;
    }
}

static int nblk(const LaunchCfg& c, long long n) {
    long long b = (n + 255) / 256;
    const long long cap = (long long)c.sm_count * 8;
    return (int)(b < 1 ? 1 : b < cap ? b : cap);
}

void launch_unet_features(const LaunchCfg& c, const GridT<float>& g, const float* kxy, const float* kz, bool aniso,
                          const float* minv, bf16* feat) {
    k_unet_features<<<nblk(c, g.N), 256, 0, c.stream>>>(g, kxy, kz, aniso ? 1 : 0, minv, feat);
    count_launch();
}
void launch_unet_input(const LaunchCfg& c, long long N, const float* r, const float* minv, const double* sigma2,
                       bf16* feat) {
    k_unet_input<<<nblk(c, N), 256, 0, c.stream>>>(N, r, minv, sigma2, feat);
    count_launch();
}
void launch_unet_head(const LaunchCfg& c, const HeadArgs& a) {
    const long long N = (long long)a.n0 * a.n1 * a.n2;
    k_unet_head<<<nblk(c, N), 256, 0, c.stream>>>(a);
    count_launch();
}
void launch_unet_head_backward(const LaunchCfg& c, const HeadArgs& a, const float* gu, bf16* dx0, bf16* dp0_fine,
                               float* dwh_partial, int blocks) {
    k_unet_head_bwd<<<blocks, 256, 0, c.stream>>>(a, gu, dx0, dp0_fine, dwh_partial);
    count_launch();
}

}  // namespace plgpu

namespace plgpu {

// ----------------------------------------------------------------------------------------
// training-pair generation and the loss

// counter-based normal deviates (splitmix64 hash, Box-Muller); zero where minv == 0
__device__ __forceinline__ unsigned long long mix64(unsigned long long x) {
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}
__global__ void __launch_bounds__(256) k_noise(long long N, unsigned long long seed, const float* __restrict__ minv,
                                               float* __restrict__ e) {
    for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < N; n += (long long)gridDim.x * blockDim.x) {
        const unsigned long long h = mix64(seed * 0x100000001B3ull + (unsigned long long)n);
        const float u1 = ((h >> 40) + 0.5f) * (1.0f / 16777216.0f);
        const float u2 = ((h & 0xFFFFFFull) + 0.5f) * (1.0f / 16777216.0f);
        const float g = sqrtf(-2.f * logf(u1)) * __cosf(6.2831853f * u2);
        e[n] = minv[n] > 0.f ? g : 0.f;
    }
}
// e -= omega M^-1 (A e)
__global__ void __launch_bounds__(256) k_jacobi_sweep(long long N, float omega, const float* __restrict__ minv,
                                                      const float* __restrict__ ae, float* __restrict__ e) {
    for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < N; n += (long long)gridDim.x * blockDim.x)
        e[n] -= omega * minv[n] * ae[n];
}
// d = z - e
__global__ void __launch_bounds__(256) k_sub(long long N, const float* __restrict__ a, const float* __restrict__ b,
                                             float* __restrict__ d) {
    for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < N; n += (long long)gridDim.x * blockDim.x)
        d[n] = a[n] - b[n];
}
// Gradient of L = 1 - a^2 / (b E), a = (v, r), b = (v, A v), E = (e, A e), w.r.t. u with
// v = D^-1/2 u:  dL/dv = -(2a / (b E)) r + (2 a^2 / (b^2 E)) A v,  dL/du = D^-1/2 dL/dv.
// sc[0] = a, sc[1] = b, sc[2] = E.
__global__ void __launch_bounds__(256) k_loss_grad_u(long long N, const float* __restrict__ r,
                                                     const float* __restrict__ av, const float* __restrict__ minv,
                                                     const double* __restrict__ sc, float* __restrict__ gu) {
    const double a = sc[0], b = sc[1], E = sc[2];
    const bool ok = b > 0.0 && E > 0.0 && isfinite(a);
    const float c1 = ok ? (float)(-2.0 * a / (b * E)) : 0.f;
    const float c2 = ok ? (float)(2.0 * a * a / (b * b * E)) : 0.f;
    for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < N; n += (long long)gridDim.x * blockDim.x) {
        const float m = minv[n];
        gu[n] = m > 0.f ? sqrtf(m) * (c1 * r[n] + c2 * av[n]) : 0.f;
    }
}
// z = M^-1 r + c v with the A-norm optimal weight c = (v, r) / (v, A v)  (0 if undefined)
__global__ void __launch_bounds__(256) k_precond_combine(long long N, const float* __restrict__ r,
                                                         const float* __restrict__ minv, const float* __restrict__ v,
                                                         const double* __restrict__ sc, float* __restrict__ z) {
    const double a = sc[0], b = sc[1];
    const float c = (b > 0.0 && isfinite(a / b)) ? (float)(a / b) : 0.f;
    for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < N; n += (long long)gridDim.x * blockDim.x)
        z[n] = minv[n] * r[n] + c * v[n];
}
// e *= 1 / sqrt(s / N), s = (e, e) from a device scalar
__global__ void __launch_bounds__(256) k_scale_rms(long long N, const double* __restrict__ s, float* __restrict__ e) {
    const double ms = *s / (double)N;
    const float f = ms > 0.0 ? (float)(1.0 / sqrt(ms)) : 0.f;
    for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < N; n += (long long)gridDim.x * blockDim.x)
        e[n] *= f;
}
// (x, y) and optionally (x, M^-1 x) into two device doubles; deterministic two-pass
__global__ void __launch_bounds__(256) k_dot_partial(long long N, const float* __restrict__ x, const float* __restrict__ y,
                                                     double* __restrict__ partial) {
    double s = 0.0;
    for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < N; n += (long long)gridDim.x * blockDim.x)
        s += (double)(x[n] * y[n]);
    __shared__ double sh[8];
    for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += sh[w];
        partial[blockIdx.x] = t;
    }
}
__global__ void k_dot_final(int nb, const double* __restrict__ partial, double* __restrict__ out) {
    double s = 0.0;
    for (int b = threadIdx.x; b < nb; b += blockDim.x) s += partial[b];
    __shared__ double sh[8];
    for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += sh[w];
        *out = t;
    }
}
// (r, M^-1 r) into out
__global__ void __launch_bounds__(256) k_rmr_partial(long long N, const float* __restrict__ r,
                                                     const float* __restrict__ minv, double* __restrict__ partial) {
    double s = 0.0;
    for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < N; n += (long long)gridDim.x * blockDim.x)
        s += (double)(r[n] * minv[n] * r[n]);
    __shared__ double sh[8];
    for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += sh[w];
        partial[blockIdx.x] = t;
    }
}

void launch_noise(const LaunchCfg& c, long long N, unsigned long long seed, const float* minv, float* e) {
    k_noise<<<nblk(c, N), 256, 0, c.stream>>>(N, seed, minv, e);
    count_launch();
}
void launch_jacobi_sweep(const LaunchCfg& c, long long N, float omega, const float* minv, const float* ae, float* e) {
    k_jacobi_sweep<<<nblk(c, N), 256, 0, c.stream>>>(N, omega, minv, ae, e);
    count_launch();
}
void launch_sub(const LaunchCfg& c, long long N, const float* a, const float* b, float* d) {
    k_sub<<<nblk(c, N), 256, 0, c.stream>>>(N, a, b, d);
    count_launch();
}
void launch_loss_grad_u(const LaunchCfg& c, long long N, const float* r, const float* av, const float* minv,
                        const double* sc, float* gu) {
    k_loss_grad_u<<<nblk(c, N), 256, 0, c.stream>>>(N, r, av, minv, sc, gu);
    count_launch();
}
void launch_precond_combine(const LaunchCfg& c, long long N, const float* r, const float* minv, const float* v,
                            const double* sc, float* z) {
    k_precond_combine<<<nblk(c, N), 256, 0, c.stream>>>(N, r, minv, v, sc, z);
    count_launch();
}
void launch_scale_rms(const LaunchCfg& c, long long N, const double* s, float* e) {
    k_scale_rms<<<nblk(c, N), 256, 0, c.stream>>>(N, s, e);
    count_launch();
}
void launch_dot(const LaunchCfg& c, long long N, const float* x, const float* y, double* partial, double* out) {
    const int nb = nblk(c, N);
    k_dot_partial<<<nb, 256, 0, c.stream>>>(N, x, y, partial);
    k_dot_final<<<1, 256, 0, c.stream>>>(nb, partial, out);
    count_launches(2);
}
void launch_rmr(const LaunchCfg& c, long long N, const float* r, const float* minv, double* partial, double* out) {
    const int nb = nblk(c, N);
    k_rmr_partial<<<nb, 256, 0, c.stream>>>(N, r, minv, partial);
    k_dot_final<<<1, 256, 0, c.stream>>>(nb, partial, out);
    count_launches(2);
}

}  // namespace plgpu
