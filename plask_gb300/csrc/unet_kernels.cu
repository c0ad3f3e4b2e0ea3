// Kernels of the learned preconditioner: a small 3D U-Net on the node grid.
//
// Tensors are channels-last ("NDHWC"): value (i, j, k, c) of a level with
// extents n0 x n1 x n2 and C channels sits at ((k n1 + j) n0 + i) C + c, in BF16.
// Level l + 1 has extents ceil(n / 2); its voxel (I, J, K) is the parent of the
// 2x2x2 children (2I + a, 2J + b, 2K + c) that exist on level l.
//
// Convolutions are implicit GEMMs on the tensor cores with mma.sync.m16n8k16
// (BF16 in, FP32 accumulate): M = voxels, N = output channels, K = taps x input
// channels.  One block computes a 16 (x) by 4 (y) tile of output voxels at one z;
// it stages the input patch (tile plus a one-voxel halo for 3x3x3) in shared
// memory, each warp owns one 16-voxel row of the tile and loads its A fragments
// with ldmatrix from the patch; B fragments (weights) come from global memory
// through L1.  The input loader can add an upsampled coarse tensor to the input
// ("add skip"), so the decoder needs no separate upsample kernel, and the
// epilogue can apply ReLU or multiply by a ReLU gate (the backward pass).
//
// The backward pass w.r.t. the input is the same kernel with the weights flipped
// in space and transposed in channels; the backward pass w.r.t. the weights is a
// separate kernel that, per tap, multiplies the shifted input tile by the output
// gradient tile (both staged in shared memory, fragments loaded transposed).
#include <cuda_bf16.h>

#include <cstdint>

#include "fem3d_kernels.h"
#include "unet_kernels.h"

namespace plgpu {

using bf16 = __nv_bfloat16;

// ----------------------------------------------------------------------------------------
// tensor-core helpers

__device__ __forceinline__ void ldmatrix_x4(uint32_t (&r)[4], const void* smem_row) {
    const uint32_t a = (uint32_t)__cvta_generic_to_shared(smem_row);
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0, %1, %2, %3}, [%4];\n"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(a));
}
__device__ __forceinline__ void ldmatrix_x4_trans(uint32_t (&r)[4], const void* smem_row) {
    const uint32_t a = (uint32_t)__cvta_generic_to_shared(smem_row);
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0, %1, %2, %3}, [%4];\n"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(a));
}
__device__ __forceinline__ void ldmatrix_x2_trans(uint32_t (&r)[2], const void* smem_row) {
    const uint32_t a = (uint32_t)__cvta_generic_to_shared(smem_row);
    asm volatile("ldmatrix.sync.aligned.m8n8.x2.trans.shared.b16 {%0, %1}, [%2];\n"
                 : "=r"(r[0]), "=r"(r[1])
                 : "r"(a));
}
// D = A * B + D, A 16x16 (row), B 16x8 (col), BF16 in, FP32 accumulate
__device__ __forceinline__ void mma_bf16(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0, %1, %2, %3}, {%4, %5, %6, %7}, {%8, %9}, "
        "{%0, %1, %2, %3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

__device__ __forceinline__ long long vox(int i, int j, int k, int n0, int n1) {
    return ((long long)k * n1 + j) * n0 + i;
}

// ----------------------------------------------------------------------------------------
// convolution forward (also the input-gradient pass)

// Shared-memory row stride of the staged patch in bf16 elements: CIN plus 8 keeps
// the 16-byte ldmatrix rows of consecutive voxels in different bank groups.
template <int CIN>
__host__ __device__ constexpr int patch_stride() {
    return CIN + 8;
}

template <int CIN, int COUT, int TAPS>
__global__ void __launch_bounds__(128) k_conv_mma(const ConvArgs a) {
    static_assert(CIN % 16 == 0 && COUT % 8 == 0, "channel counts");
    constexpr int H = TAPS == 27 ? 1 : 0;  // halo
    constexpr int PX = 16 + 2 * H, PY = 4 + 2 * H, PZ = 1 + 2 * H;
    constexpr int PS = patch_stride<CIN>();
    extern __shared__ __align__(16) unsigned char smem_raw[];
    bf16* patch = reinterpret_cast<bf16*>(smem_raw);

    const int n0 = a.n0, n1 = a.n1, n2 = a.n2;
    const int i0 = blockIdx.x * 16, j0 = blockIdx.y * 4, k = blockIdx.z;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;

    // stage the patch: PZ x PY x PX voxels of CIN channels, 16 bytes (8 channels) per copy
    constexpr int VEC = CIN / 8;
    for (int t = tid; t < PZ * PY * PX * VEC; t += 128) {
        const int v = t / VEC, c8 = (t % VEC) * 8;
        const int px = v % PX, py = (v / PX) % PY, pz = v / (PX * PY);
        const int gi = i0 + px - H, gj = j0 + py - H, gk = k + pz - H;
        uint4 val = make_uint4(0, 0, 0, 0);
        if (gi >= 0 && gi < n0 && gj >= 0 && gj < n1 && gk >= 0 && gk < n2) {
            const long long g = vox(gi, gj, gk, n0, n1);
            val = *reinterpret_cast<const uint4*>(a.in + g * CIN + c8);
            if (a.up != nullptr) {  // add the parent's value of the coarser tensor
                const long long gp = vox(gi >> 1, gj >> 1, gk >> 1, a.pn0, a.pn1);
                const uint4 u = *reinterpret_cast<const uint4*>(a.up + gp * CIN + c8);
                __nv_bfloat162* pv = reinterpret_cast<__nv_bfloat162*>(&val);
                const __nv_bfloat162* pu = reinterpret_cast<const __nv_bfloat162*>(&u);
#pragma unroll
                for (int q = 0; q < 4; ++q) pv[q] = __hadd2(pv[q], pu[q]);
            }
        }
        *reinterpret_cast<uint4*>(patch + (size_t)v * PS + c8) = val;
    }
    __syncthreads();

    constexpr int NT = COUT / 8;
    float acc[NT][4];
#pragma unroll
    for (int n = 0; n < NT; ++n) acc[n][0] = acc[n][1] = acc[n][2] = acc[n][3] = 0.f;

    const int arow = lane & 15;        // voxel (x within the tile) this lane addresses for ldmatrix
    const int akoff = (lane >> 4) * 8; // k half
    const int bn = lane >> 2;          // B fragment column (output channel within the n-tile)
    const int bk = (lane & 3) * 2;     // B fragment row pair
#pragma unroll 1
    for (int tap = 0; tap < TAPS; ++tap) {
        const int dx = TAPS == 27 ? tap % 3 : 0, dy = TAPS == 27 ? (tap / 3) % 3 : 0, dz = TAPS == 27 ? tap / 9 : 0;
        const bf16* prow = patch + ((size_t)(dz * PY + warp + dy) * PX + arow + dx) * PS + akoff;
        const bf16* wt = a.w + (size_t)tap * COUT * CIN;
#pragma unroll
        for (int kc = 0; kc < CIN / 16; ++kc) {
            uint32_t af[4];
            ldmatrix_x4(af, prow + kc * 16);
#pragma unroll
            for (int n = 0; n < NT; ++n) {
                const bf16* wr = wt + (size_t)(n * 8 + bn) * CIN + kc * 16 + bk;
                const uint32_t b0 = __ldg(reinterpret_cast<const unsigned int*>(wr));
                const uint32_t b1 = __ldg(reinterpret_cast<const unsigned int*>(wr + 8));
                mma_bf16(acc[n], af, b0, b1);
            }
        }
    }

    // epilogue: C fragment rows lane/4 and lane/4 + 8 (voxels), columns 2 (lane % 4) + {0, 1}
    const int j = j0 + warp;
#pragma unroll
    for (int half = 0; half < 2; ++half) {
        const int i = i0 + (lane >> 2) + half * 8;
        if (i >= n0 || j >= n1) continue;
        const long long g = vox(i, j, k, n0, n1);
#pragma unroll
        for (int n = 0; n < NT; ++n) {
            const int c = n * 8 + (lane & 3) * 2;
            float v0 = acc[n][half * 2] * a.scale, v1 = acc[n][half * 2 + 1] * a.scale;
            if (a.gate != nullptr) {  // ReLU backward: pass where the forward activation was positive
                const __nv_bfloat162 gv = *reinterpret_cast<const __nv_bfloat162*>(a.gate + g * COUT + c);
                if (!(__bfloat162float(gv.x) > 0.f)) v0 = 0.f;
                if (!(__bfloat162float(gv.y) > 0.f)) v1 = 0.f;
            }
            if (a.relu) {
                v0 = fmaxf(v0, 0.f);
                v1 = fmaxf(v1, 0.f);
            }
            if (a.out != nullptr)
                *reinterpret_cast<__nv_bfloat162*>(a.out + g * COUT + c) = __floats2bfloat162_rn(v0, v1);
            if (a.out32 != nullptr) {
                a.out32[g * COUT + c] = v0;
                a.out32[g * COUT + c + 1] = v1;
            }
        }
    }
}

// ----------------------------------------------------------------------------------------
// convolution weight gradient:  dW[tap][co][ci] = sum_v X[v + off(tap)][ci] G[v][co]
//
// Grid (chunks, taps): a block takes one tap and every chunks-th output tile,
// accumulates COUT x CIN in registers (4 warps share the output tiles) and
// writes one partial; k_reduce_partials sums the partials of all chunks.

template <int CIN, int COUT, int TAPS>
__global__ void __launch_bounds__(128) k_conv_wgrad(const WgradArgs a) {
    constexpr int XS = CIN + 8, GS = COUT + 8;  // shared strides (bf16)
    __shared__ __align__(16) bf16 xs[64 * XS];
    __shared__ __align__(16) bf16 gs[64 * GS];
    const int n0 = a.n0, n1 = a.n1, n2 = a.n2;
    const int tap = blockIdx.y;
    const int dx = TAPS == 27 ? tap % 3 - 1 : 0, dy = TAPS == 27 ? (tap / 3) % 3 - 1 : 0,
              dz = TAPS == 27 ? tap / 9 - 1 : 0;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    constexpr int MT = COUT / 16, NT = CIN / 8, TILES = MT * NT;
    constexpr int PER_WARP = (TILES + 3) / 4;
    float acc[PER_WARP][4];
#pragma unroll
    for (int t = 0; t < PER_WARP; ++t) acc[t][0] = acc[t][1] = acc[t][2] = acc[t][3] = 0.f;

    const int tx = (n0 + 15) / 16, ty = (n1 + 3) / 4;
    const long long ntiles = (long long)tx * ty * n2;
    for (long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int i0 = (int)(tile % tx) * 16, j0 = (int)((tile / tx) % ty) * 4, k = (int)(tile / ((long long)tx * ty));
        __syncthreads();
        // stage the 64 output voxels' gradient and the 64 shifted input voxels
        for (int t = tid; t < 64 * (COUT / 8); t += 128) {
            const int v = t / (COUT / 8), c8 = (t % (COUT / 8)) * 8;
            const int i = i0 + (v & 15), j = j0 + (v >> 4);
            uint4 val = make_uint4(0, 0, 0, 0);
            if (i < n0 && j < n1) val = *reinterpret_cast<const uint4*>(a.g + vox(i, j, k, n0, n1) * COUT + c8);
            *reinterpret_cast<uint4*>(gs + v * GS + c8) = val;
        }
        for (int t = tid; t < 64 * (CIN / 8); t += 128) {
            const int v = t / (CIN / 8), c8 = (t % (CIN / 8)) * 8;
            const int i = i0 + (v & 15), j = j0 + (v >> 4);
            const int si = i + dx, sj = j + dy, sk = k + dz;
            uint4 val = make_uint4(0, 0, 0, 0);
            if (i < n0 && j < n1 && si >= 0 && si < n0 && sj >= 0 && sj < n1 && sk >= 0 && sk < n2) {
                const long long gidx = vox(si, sj, sk, n0, n1);
                val = *reinterpret_cast<const uint4*>(a.x + gidx * CIN + c8);
                if (a.up != nullptr) {
                    const long long gp = vox(si >> 1, sj >> 1, sk >> 1, a.pn0, a.pn1);
                    const uint4 u = *reinterpret_cast<const uint4*>(a.up + gp * CIN + c8);
                    __nv_bfloat162* pv = reinterpret_cast<__nv_bfloat162*>(&val);
                    const __nv_bfloat162* pu = reinterpret_cast<const __nv_bfloat162*>(&u);
#pragma unroll
                    for (int q = 0; q < 4; ++q) pv[q] = __hadd2(pv[q], pu[q]);
                }
            }
            *reinterpret_cast<uint4*>(xs + v * XS + c8) = val;
        }
        __syncthreads();
        // K = 64 voxels in 4 chunks of 16
#pragma unroll
        for (int kc = 0; kc < 4; ++kc) {
#pragma unroll
            for (int t = 0; t < PER_WARP; ++t) {
                const int tt = warp * PER_WARP + t;
                if (tt >= TILES) break;
                const int mt = tt / NT, nt = tt % NT;
                // A[m = co][k = voxel] = G[voxel][co]: transposed 16x16 load from gs
                uint32_t af[4];
                {
                    const int r = lane & 7, q = lane >> 3;  // matrix q: (rows m 0-7 | 8-15) x (k 0-7 | 8-15)
                    const int kk = kc * 16 + r + ((q >> 1) & 1) * 8;
                    const int mm = mt * 16 + (q & 1) * 8;
                    ldmatrix_x4_trans(af, gs + kk * GS + mm);
                }
                // B[k = voxel][n = ci] = X[voxel][ci]: transposed 16x8 load from xs
                uint32_t bfr[2];
                {
                    const int r = lane & 7, q = (lane >> 3) & 1;
                    const int kk = kc * 16 + r + q * 8;
                    ldmatrix_x2_trans(bfr, xs + kk * XS + nt * 8);
                }
                mma_bf16(acc[t], af, bfr[0], bfr[1]);
            }
        }
    }
    // write this block's partial: partial[chunk][tap][co][ci]
    float* out = a.partial + ((size_t)blockIdx.x * TAPS + tap) * COUT * CIN;
#pragma unroll
    for (int t = 0; t < PER_WARP; ++t) {
        const int tt = warp * PER_WARP + t;
        if (tt >= TILES) break;
        const int mt = tt / NT, nt = tt % NT;
        const int co = mt * 16 + (lane >> 2), ci = nt * 8 + (lane & 3) * 2;
        out[(size_t)co * CIN + ci] = acc[t][0];
        out[(size_t)co * CIN + ci + 1] = acc[t][1];
        out[(size_t)(co + 8) * CIN + ci] = acc[t][2];
        out[(size_t)(co + 8) * CIN + ci + 1] = acc[t][3];
    }
}

// sum over chunks: out[e] = scale * sum_c partial[c * n + e]
__global__ void k_reduce_partials(const float* __restrict__ partial, int chunks, int n, float scale,
                                  float* __restrict__ out) {
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n; e += gridDim.x * blockDim.x) {
        float s = 0.f;
        for (int c = 0; c < chunks; ++c) s += partial[(size_t)c * n + e];
        out[e] = s * scale;
    }
}

// ----------------------------------------------------------------------------------------
// pooling and its transpose (2x2x2 average; coarse extents ceil(n/2), missing children count as 0)

__global__ void k_pool_avg(int n0, int n1, int n2, int C, const bf16* __restrict__ in, bf16* __restrict__ out) {
    const int m0 = (n0 + 1) / 2, m1 = (n1 + 1) / 2, m2 = (n2 + 1) / 2;
    const long long M = (long long)m0 * m1 * m2 * C;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < M; t += (long long)gridDim.x * blockDim.x) {
        const int c = (int)(t % C);
        const long long v = t / C;
        const int I = (int)(v % m0), J = (int)((v / m0) % m1), K = (int)(v / ((long long)m0 * m1));
        float s = 0.f;
        for (int q = 0; q < 8; ++q) {
            const int i = 2 * I + (q & 1), j = 2 * J + ((q >> 1) & 1), k = 2 * K + (q >> 2);
            if (i < n0 && j < n1 && k < n2) s += __bfloat162float(in[vox(i, j, k, n0, n1) * C + c]);
        }
        out[t] = __float2bfloat16(0.125f * s);
    }
}

// transpose of k_pool_avg: fine[v] (+)= 1/8 coarse[parent(v)], optionally gated by (gate > 0)
__global__ void k_pool_avg_t(int n0, int n1, int n2, int C, const bf16* __restrict__ coarse, const bf16* __restrict__ gate,
                             bf16* __restrict__ fine, int accumulate) {
    const int m0 = (n0 + 1) / 2, m1 = (n1 + 1) / 2;
    const long long N = (long long)n0 * n1 * n2 * C;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < N; t += (long long)gridDim.x * blockDim.x) {
        const int c = (int)(t % C);
        const long long v = t / C;
        const int i = (int)(v % n0), j = (int)((v / n0) % n1), k = (int)(v / ((long long)n0 * n1));
        float g = 0.125f * __bfloat162float(coarse[vox(i >> 1, j >> 1, k >> 1, m0, m1) * C + c]);
        if (accumulate) g += __bfloat162float(fine[t]);
        if (gate != nullptr && !(__bfloat162float(gate[t]) > 0.f)) g = 0.f;
        fine[t] = __float2bfloat16(g);
    }
}

// transpose of "add the parent's value": coarse[P] = sum over existing children of fine[child]
__global__ void k_sum_children(int n0, int n1, int n2, int C, const bf16* __restrict__ fine, bf16* __restrict__ coarse) {
    const int m0 = (n0 + 1) / 2, m1 = (n1 + 1) / 2, m2 = (n2 + 1) / 2;
    const long long M = (long long)m0 * m1 * m2 * C;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < M; t += (long long)gridDim.x * blockDim.x) {
        const int c = (int)(t % C);
        const long long v = t / C;
        const int I = (int)(v % m0), J = (int)((v / m0) % m1), K = (int)(v / ((long long)m0 * m1));
        float s = 0.f;
        for (int q = 0; q < 8; ++q) {
            const int i = 2 * I + (q & 1), j = 2 * J + ((q >> 1) & 1), k = 2 * K + (q >> 2);
            if (i < n0 && j < n1 && k < n2) s += __bfloat162float(fine[vox(i, j, k, n0, n1) * C + c]);
        }
        coarse[t] = __float2bfloat16(s);
    }
}

// ----------------------------------------------------------------------------------------
// weight transforms and the optimiser

// flipped, channel-transposed weights for the input-gradient pass:
// wt[tap'][ci][co] = w[26 - tap][co][ci]  (TAPS = 1: plain transpose)
__global__ void k_weights_for_dgrad(int taps, int cout, int cin, const bf16* __restrict__ w, bf16* __restrict__ wt) {
    const int n = taps * cout * cin;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        const int ci = t % cin, co = (t / cin) % cout, tap = t / (cin * cout);
        const int tf = taps - 1 - tap;
        wt[((size_t)tf * cin + ci) * cout + co] = w[t];
    }
}

// Adam step on FP32 master weights, refreshing the BF16 copy.
__global__ void k_adam(int n, float* __restrict__ w, float* __restrict__ m, float* __restrict__ v,
                       const float* __restrict__ g, bf16* __restrict__ wb, float lr, float b1, float b2, float eps,
                       float bc1, float bc2, float clip) {
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        float gr = g[t];
        if (!isfinite(gr)) gr = 0.f;
        gr = fminf(fmaxf(gr, -clip), clip);
        const float mt = b1 * m[t] + (1.f - b1) * gr;
        const float vt = b2 * v[t] + (1.f - b2) * gr * gr;
        m[t] = mt;
        v[t] = vt;
        const float upd = lr * (mt / bc1) / (sqrtf(vt / bc2) + eps);
        w[t] -= upd;
        wb[t] = __float2bfloat16(w[t]);
    }
}

// ----------------------------------------------------------------------------------------
// launchers

template <int CIN, int COUT, int TAPS>
static void conv_launch(const LaunchCfg& c, const ConvArgs& a) {
    constexpr int H = TAPS == 27 ? 1 : 0;
    const size_t smem = (size_t)(16 + 2 * H) * (4 + 2 * H) * (1 + 2 * H) * patch_stride<CIN>() * sizeof(bf16);
    static bool configured = false;
    if (!configured) {
        cudaFuncSetAttribute(k_conv_mma<CIN, COUT, TAPS>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        configured = true;
    }
    dim3 grid((a.n0 + 15) / 16, (a.n1 + 3) / 4, a.n2);
    k_conv_mma<CIN, COUT, TAPS><<<grid, 128, smem, c.stream>>>(a);
    count_launch();
}

template <int CIN, int COUT, int TAPS>
static void wgrad_launch(const LaunchCfg& c, const WgradArgs& a, int chunks) {
    dim3 grid(chunks, TAPS);
    k_conv_wgrad<CIN, COUT, TAPS><<<grid, 128, 0, c.stream>>>(a);
    count_launch();
}

#define PLGPU_CONV_CASES(X) \
    X(16, 16, 1)            \
    X(16, 32, 27)           \
    X(32, 16, 27)           \
    X(32, 48, 27)           \
    X(48, 32, 27)           \
    X(48, 64, 27)           \
    X(64, 48, 27)           \
    X(64, 64, 27)           \
    X(48, 48, 27)           \
    X(32, 32, 27)           \
    X(64, 48, 1)            \
    X(48, 64, 1)            \
    X(48, 32, 1)            \
    X(32, 48, 1)            \
    X(32, 16, 1)            \
    X(16, 32, 1)

bool conv_supported(int cin, int cout, int taps) {
#define PLGPU_CHECK(CI, CO, TP) \
    if (cin == CI && cout == CO && taps == TP) return true;
    PLGPU_CONV_CASES(PLGPU_CHECK)
#undef PLGPU_CHECK
    return false;
}

void launch_conv(const LaunchCfg& c, int cin, int cout, int taps, const ConvArgs& a) {
#define PLGPU_DISPATCH(CI, CO, TP)         \
    if (cin == CI && cout == CO && taps == TP) { \
        conv_launch<CI, CO, TP>(c, a);     \
        return;                            \
    }
    PLGPU_CONV_CASES(PLGPU_DISPATCH)
#undef PLGPU_DISPATCH
}

void launch_conv_wgrad(const LaunchCfg& c, int cin, int cout, int taps, const WgradArgs& a, int chunks) {
#define PLGPU_DISPATCH(CI, CO, TP)              \
    if (cin == CI && cout == CO && taps == TP) { \
        wgrad_launch<CI, CO, TP>(c, a, chunks); \
        return;                                 \
    }
    PLGPU_CONV_CASES(PLGPU_DISPATCH)
#undef PLGPU_DISPATCH
}

static int gsz(long long n, int cap) {
    long long b = (n + 255) / 256;
    return (int)(b < 1 ? 1 : b < cap ? b : cap);
}

void launch_reduce_partials(const LaunchCfg& c, const float* partial, int chunks, int n, float scale, float* out) {
    k_reduce_partials<<<gsz(n, 1024), 256, 0, c.stream>>>(partial, chunks, n, scale, out);
    count_launch();
}
void launch_pool_avg(const LaunchCfg& c, int n0, int n1, int n2, int C, const bf16* in, bf16* out) {
    const long long M = (long long)((n0 + 1) / 2) * ((n1 + 1) / 2) * ((n2 + 1) / 2) * C;
    k_pool_avg<<<gsz(M, c.sm_count * 8), 256, 0, c.stream>>>(n0, n1, n2, C, in, out);
    count_launch();
}
void launch_pool_avg_t(const LaunchCfg& c, int n0, int n1, int n2, int C, const bf16* coarse, const bf16* gate,
                       bf16* fine, int accumulate) {
    const long long N = (long long)n0 * n1 * n2 * C;
    k_pool_avg_t<<<gsz(N, c.sm_count * 8), 256, 0, c.stream>>>(n0, n1, n2, C, coarse, gate, fine, accumulate);
    count_launch();
}
void launch_sum_children(const LaunchCfg& c, int n0, int n1, int n2, int C, const bf16* fine, bf16* coarse) {
    const long long M = (long long)((n0 + 1) / 2) * ((n1 + 1) / 2) * ((n2 + 1) / 2) * C;
    k_sum_children<<<gsz(M, c.sm_count * 8), 256, 0, c.stream>>>(n0, n1, n2, C, fine, coarse);
    count_launch();
}
void launch_weights_for_dgrad(const LaunchCfg& c, int taps, int cout, int cin, const bf16* w, bf16* wt) {
    k_weights_for_dgrad<<<gsz((long long)taps * cout * cin, 1024), 256, 0, c.stream>>>(taps, cout, cin, w, wt);
    count_launch();
}
void launch_adam(const LaunchCfg& c, int n, float* w, float* m, float* v, const float* g, bf16* wb, float lr, float b1,
                 float b2, float eps, float bc1, float bc2, float clip) {
    k_adam<<<gsz(n, 1024), 256, 0, c.stream>>>(n, w, m, v, g, wb, lr, b1, b2, eps, bc1, bc2, clip);
    count_launch();
}

}  // namespace plgpu
