// TMA-staged FP32 stiffness operator of the inner CG solve for sm_103a.
//
// Computes the same product as k_apply_shared (fem3d_operator.cu; PLaSK therm3d.cpp:226-237:
// the trilinear-hex stiffness K_e = H^T diag(lambda) H per element, applied matrix-free) with
// the input planes staged in shared memory by the Tensor Memory Accelerator instead of
// per-thread global loads.
//
// Work layout.  A block spans the whole mesh along x: warp (wx, wy), lane m owns the node
// columns c0 = 64 wx + 2 m and c0 + 1 and computes the two element columns to their left,
// A = c0 - 1 and B = c0, with packed two-wide FP32 instructions (add/mul/fma.f32x2): the two
// elements take the same arithmetic on different data.  Each thread covers RR consecutive
// rows along y (warp row wy of the block) and marches a chunk of z-planes.  For every plane
// the block holds in shared memory, written by cp.async.bulk.tensor, per pair of warps along
// x (a region of 128 columns):
//   - the node tile of the input x: columns 128 r - 4 .. 128 r + 127, rows j0 - 1 .. j0 + RR WY;
//   - the element tile(s) of the pre-scaled conductances P (and Q when anisotropic) of the
//     element layer above the plane, rows j0 - 1 .. j0 + RR WY - 1.
// The tiles start at column 128 r - 4 so that the copy's first x coordinate is 16-byte
// aligned; rows, columns and planes outside the mesh arrive as zeros (the copy's
// out-of-bounds fill), so elements outside the mesh contribute nothing and no load carries
// a bounds test.  NS stages form a ring: stage u % NS holds plane kstart + u; an mbarrier per
// stage counts the bytes of its copies.  One block-wide barrier per plane releases the stage
// the block has finished with, and thread 0 then issues the copies of the plane NS ahead.
//
// Element algebra (derivation in fem3d_operator.cu).  With the conductances pre-scaled per
// element by k_tma_coef,
//     P = k_xy dx dy dz / 48,   Q = k_z dx dy / (16 dz) = 3 Z,
// the butterfly weights are X = P / dx^2, Y = P / dy^2, Z = Q / 3 (isotropic: Z = P / dz^2),
//     l100 = 3X, l010 = 3Y, l001 = 3Z, l110 = X + Y, l101 = X + Z, l011 = Y + Z,
//     l111 = (X + Y + Z) / 3.
// Contributions to the two x-corners of an element are accumulated as (sum, difference)
// pairs: an element's right corner gets S + D, its left corner S - D.  Node c0 takes A's
// right and B's left corner (both in the lane); node c0 + 1 takes B's right corner and the
// left corner of the next lane's A, sent by one shuffle per output row; the last lane of a
// warp takes it from the next warp along x through shared memory after the plane's barrier.
//
// Convective surface rows (therm3d.cpp:250-259: the face stiffness, kept as a small CSR
// operator) are added in the same pass: a plane that holds surface rows has a node -> row
// map, and the thread owning such a node adds its row of S x to the output.
//
// The launch leaves one partial of (x, A x) per block; the kernel that consumes A x reduces
// them (no block waits for the others here).
//
// Waits are bounded: a stage whose copies have not landed after kSpinLimit polls makes the
// block set SOLVE_DEVICE_TIMEOUT, wait (bounded again) for its copies in flight and return.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <memory>
#include <mutex>
#include <vector>

#include "fem3d_device.cuh"
#include "fem3d_kernels.h"
#include "fem3d_reduce.cuh"

namespace plgpu {

namespace {

// Tile constants (overridable at compile time for tuning sweeps):
//   PLGPU_TMA_ROWS    output rows per thread
//   PLGPU_TMA_STAGES  planes in the shared-memory ring
//   PLGPU_TMA_BLOCKS  resident blocks per SM the z-chunks are sized for (0: the cost model)
#ifndef PLGPU_TMA_ROWS
#define PLGPU_TMA_ROWS 2
#endif
#ifndef PLGPU_TMA_STAGES
#define PLGPU_TMA_STAGES 3
#endif
#ifndef PLGPU_TMA_BLOCKS
#define PLGPU_TMA_BLOCKS 0
#endif
//   PLGPU_TMA_MINB    blocks per SM the register budget is sized for
#ifndef PLGPU_TMA_MINB
#define PLGPU_TMA_MINB 4
#endif
constexpr int kTmaRows = PLGPU_TMA_ROWS;
constexpr int kTmaStages = PLGPU_TMA_STAGES;
constexpr int kTmaMaxWarpsX = 4;  // 64 columns per warp: meshes up to 256 nodes along x
constexpr unsigned kSpinLimit = 1u << 22;

// warps along y of a block with wx warps along x (128 threads, 96 for wx = 3)
__host__ __device__ constexpr int tma_wy(int wx) { return wx == 1 ? 4 : wx == 2 ? 2 : 1; }
// columns of one copy: a region of 128 columns (64 for one warp) plus the 4 to its left
__host__ __device__ constexpr int tma_box(int wx) { return wx == 1 ? 68 : 132; }
__host__ __device__ constexpr int tma_regions(int wx) { return (wx + 1) / 2; }
__host__ __device__ constexpr int align128(int b) { return (b + 127) & ~127; }
__host__ __device__ constexpr int tma_x_rows(int wx, int rr) { return rr * tma_wy(wx) + 2; }
__host__ __device__ constexpr int tma_k_rows(int wx, int rr) { return rr * tma_wy(wx) + 1; }
__host__ __device__ constexpr int tma_x_tile(int wx, int rr) { return align128(tma_x_rows(wx, rr) * tma_box(wx) * 4); }
__host__ __device__ constexpr int tma_k_tile(int wx, int rr) { return align128(tma_k_rows(wx, rr) * tma_box(wx) * 4); }
__host__ __device__ constexpr int tma_stage_bytes(int wx, int rr, bool aniso) {
    return tma_regions(wx) * (tma_x_tile(wx, rr) + tma_k_tile(wx, rr) * (aniso ? 2 : 1));
}
// the bytes the copies of one stage deliver (the boxes, without the alignment padding)
__host__ __device__ constexpr int tma_tx_bytes(int wx, int rr, bool aniso) {
    return tma_regions(wx) * tma_box(wx) * 4 * (tma_x_rows(wx, rr) + tma_k_rows(wx, rr) * (aniso ? 2 : 1));
}
__host__ __device__ constexpr int tma_smem_bytes(int wx, int rr, bool aniso, int ns) {
    // stages, then ns mbarriers, then the double-buffered exchange rows, plus 128 B to align
    return ns * tma_stage_bytes(wx, rr, aniso) + ns * 8 + 2 * tma_wy(wx) * wx * rr * 4 + 128;
}

// packed two-wide FP32 arithmetic
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 sub2(float2 a, float2 b) { return __ffma2_rn(b, make_float2(-1.f, -1.f), a); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 splat(float v) { return make_float2(v, v); }

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }


__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}
// bounded wait for the phase with the given parity; false when the limit ran out
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
    for (unsigned it = 0; it < kSpinLimit; ++it)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}
__device__ __forceinline__ void tma_load_3d(uint32_t dst, const CUtensorMap* map, uint32_t bar, int x, int y,
                                            int z) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4, %5}], "
        "[%2];" ::"r"(dst),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(bar), "r"(x), "r"(y), "r"(z)
        : "memory");
}

}  // namespace

struct TmaArgs {
    int n0, n1, n2;
    int zchunk;
    const float* x;          // the input vector (the buffer the tensor map covers)
    float* y;
    double* partials;        // this launch's block partials of (x, A x), slot = block index
    const int* run;          // the launch does nothing unless *run == SOLVE_RUNNING
    SolveCtl* ctl;           // reports a timed-out wait
    TmaSurface s;            // convective surface rows, added to their nodes' outputs
    const float* ax;         // per node column c: 1 / dx^2 of element column c - 1 (0 outside)
    const float* ay;         // per element row j + 1 (j = -1 .. ): 1 / dy^2 (0 outside)
    const float* az3;        // per element layer: 3 / dz^2 (isotropic only; 0 outside)
};

// (sum, difference) y-stage of one element row on one plane, for the lane's elements (A, B)
template <int RR>
struct YStage {
    float2 ss[RR + 1], sd[RR + 1], ds[RR + 1], dd[RR + 1];
};
template <int RR>
struct RowAcc {
    float2 s[RR], d[RR];
};

// registers for PLGPU_TMA_MINB blocks per SM
template <int WX, int RR, bool ANISO, int NS>
__global__ void __launch_bounds__(32 * WX * tma_wy(WX), PLGPU_TMA_MINB)
    k_apply_tma(const __grid_constant__ CUtensorMap mx, const __grid_constant__ CUtensorMap mp,
                const __grid_constant__ CUtensorMap mq, const TmaArgs a) {
    pdl_trigger_at(1);
    pdl_wait();  // the input vector and the run word come from the previous kernels
    if (*a.run != SOLVE_RUNNING) return;
    constexpr int WY = tma_wy(WX), NR = tma_regions(WX), BW = tma_box(WX);
    constexpr int XT = tma_x_tile(WX, RR), KT = tma_k_tile(WX, RR), SB = tma_stage_bytes(WX, RR, ANISO);
    constexpr uint32_t TX = tma_tx_bytes(WX, RR, ANISO);
    extern __shared__ unsigned char smem_raw[];
    unsigned char* smem = smem_raw + ((128 - (smem_u32(smem_raw) & 127)) & 127);
    uint64_t* bars = reinterpret_cast<uint64_t*>(smem + NS * SB);
    float* xch = reinterpret_cast<float*>(smem + NS * SB + NS * 8);  // [2][WY][WX][RR]

    const int tid = threadIdx.x;
    const int lane = tid & 31, warp = tid >> 5;
    const int wx = warp % WX, wy = warp / WX;
    const int c0 = 64 * wx + 2 * lane;       // the lane's node columns c0, c0 + 1
    const int reg = wx >> 1;                 // its region of 128 columns
    const int cb = c0 + 4 - 128 * reg;       // column of c0 in the region's tiles (even)
    const int j0 = blockIdx.y * (RR * WY);
    const int jw = j0 + wy * RR;             // first output row of the warp
    const int k0 = blockIdx.z * a.zchunk;
    const int k1 = min(k0 + a.zchunk, a.n2);
    const int kstart = max(k0 - 1, 0);
    const int nlayers = k1 - kstart;  // element layers kstart .. k1 - 1; planes kstart .. k1
    const int nplanes = nlayers + 1;
    const long long s2 = (long long)a.n0 * a.n1;

    auto stage_ptr = [&](int u) { return smem + (u % NS) * SB; };
    auto bar_of = [&](int u) { return smem_u32(&bars[u % NS]); };
    // this warp's x rows (global rows jw - 1 ..) and element rows of the stage
    auto xrows = [&](int u) { return reinterpret_cast<const float*>(stage_ptr(u) + reg * XT) + wy * RR * BW; };
    auto prows = [&](int u) {
        return reinterpret_cast<const float*>(stage_ptr(u) + NR * XT + reg * KT) + wy * RR * BW;
    };
    auto qrows = [&](int u) {
        return reinterpret_cast<const float*>(stage_ptr(u) + NR * XT + NR * KT + reg * KT) + wy * RR * BW;
    };
    auto issue = [&](int u) {  // copies of plane kstart + u into stage u % NS
        const uint32_t bar = bar_of(u);
        const uint32_t base = smem_u32(stage_ptr(u));
        const int p = kstart + u;
        mbar_expect_tx(bar, TX);
#pragma unroll
        for (int r = 0; r < NR; ++r) {
            tma_load_3d(base + r * XT, &mx, bar, 128 * r - 4, j0 - 1, p);
            tma_load_3d(base + NR * XT + r * KT, &mp, bar, 128 * r - 4, j0 - 1, p);
            if (ANISO) tma_load_3d(base + NR * XT + NR * KT + r * KT, &mq, bar, 128 * r - 4, j0 - 1, p);
        }
    };

    if (tid == 0) {
        for (int s = 0; s < NS; ++s) mbar_init(smem_u32(&bars[s]), 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        for (int u = 0; u < NS && u < nplanes; ++u) issue(u);
    }
    __syncthreads();

    // per-thread geometry: 1/dx^2 of the lane's element columns, 1/dy^2 of its element rows
    const float2 AX = *reinterpret_cast<const float2*>(a.ax + c0);
    float ay[RR + 1];
#pragma unroll
    for (int e = 0; e <= RR; ++e) ay[e] = a.ay[jw + e];  // element row jw - 1 + e

    bool failed = false;
    // bookkeeping for the bounded drain after a failed wait (the same in every thread):
    // planes 0 .. waited - 1 (relative) have landed, planes 0 .. issued - 1 were issued
    int waited = 0;
    int issued = min(NS, nplanes);

    YStage<RR> ya, yb;
    RowAcc<RR> acca, accb;
    float2 xra[RR], xrb[RR];
    float2 dot = make_float2(0.f, 0.f);

    // x-stage and y-stage of the plane in stage u; raw x of the output nodes
    auto plane_stage = [&](int u, YStage<RR>& ys, float2(&xr)[RR]) {
        const float* xs = xrows(u);
        float2 sp, dp;
        {
            const float2 xr2 = *reinterpret_cast<const float2*>(xs + cb);
            const float2 xl2 = make_float2(xs[cb - 1], xr2.x);
            sp = add2(xl2, xr2);
            dp = sub2(xr2, xl2);
        }
#pragma unroll
        for (int e = 0; e <= RR; ++e) {
            const float* row = xs + (e + 1) * BW;
            const float2 xr2 = *reinterpret_cast<const float2*>(row + cb);
            const float2 xl2 = make_float2(row[cb - 1], xr2.x);
            const float2 s = add2(xl2, xr2), d = sub2(xr2, xl2);
            if (e < RR) xr[e] = xr2;
            ys.ss[e] = add2(sp, s);
            ys.sd[e] = sub2(s, sp);
            ys.ds[e] = add2(dp, d);
            ys.dd[e] = sub2(d, dp);
            sp = s;
            dp = d;
        }
    };

    // one element layer u (planes kstart + u and kstart + u + 1): lo = plane u, hi = plane u + 1
    auto layer = [&](int u, const YStage<RR>& lo, YStage<RR>& hi, RowAcc<RR>& accLo, RowAcc<RR>& accHi,
                     const float2(&xrLo)[RR], float2(&xrHi)[RR]) {
        // plane u + 1 landed?
        bool ok = true;
        if (u + 1 >= waited) {
            // warp-uniform: a warp takes one path through the stage
            ok = __all_sync(0xffffffffu, mbar_wait(bar_of(u + 1), (uint32_t)(((u + 1) / NS) & 1)));
            if (ok) waited = u + 2;
        }
        if (ok) {
            plane_stage(u + 1, hi, xrHi);
            const float* kp = prows(u);
            const float* kq = qrows(u);
            const int k = kstart + u;
            const float2 az3 = splat(ANISO ? 0.f : a.az3[k]);
            const float2 third = splat(1.f / 3.f), three = splat(3.f);
#pragma unroll
            for (int e = 0; e <= RR; ++e) {
                const float2 P = make_float2(kp[e * BW + cb - 1], kp[e * BW + cb]);
                const float2 X = mul2(P, AX), Y = mul2(P, splat(ay[e]));
                float2 l001, Zt;
                if (ANISO) {
                    l001 = make_float2(kq[e * BW + cb - 1], kq[e * BW + cb]);
                    Zt = mul2(l001, third);
                } else {
                    l001 = mul2(P, az3);
                    Zt = mul2(l001, third);
                }
                const float2 l100 = mul2(X, three), l010 = mul2(Y, three);
                const float2 l110 = add2(X, Y), l101 = add2(X, Zt), l011 = add2(Y, Zt);
                const float2 l111 = mul2(add2(l110, Zt), third);
                const float2 m001 = mul2(sub2(hi.ss[e], lo.ss[e]), l001);
                const float2 m010 = mul2(add2(lo.sd[e], hi.sd[e]), l010), m011 = mul2(sub2(hi.sd[e], lo.sd[e]), l011);
                const float2 m100 = mul2(add2(lo.ds[e], hi.ds[e]), l100), m101 = mul2(sub2(hi.ds[e], lo.ds[e]), l101);
                const float2 m110 = mul2(add2(lo.dd[e], hi.dd[e]), l110), m111 = mul2(sub2(hi.dd[e], lo.dd[e]), l111);
                const float2 tsd0 = sub2(m010, m011), tsd1 = add2(m010, m011);
                const float2 tds0 = sub2(m100, m101), tds1 = add2(m100, m101);
                const float2 tdd0 = sub2(m110, m111), tdd1 = add2(m110, m111);
                // element row e spans the warp's node rows e and e + 1 = output rows e - 1 and e
                if (e >= 1) {
                    accLo.s[e - 1] = sub2(accLo.s[e - 1], add2(m001, tsd0));
                    accLo.d[e - 1] = add2(accLo.d[e - 1], sub2(tds0, tdd0));
                    accHi.s[e - 1] = add2(accHi.s[e - 1], sub2(m001, tsd1));
                    accHi.d[e - 1] = add2(accHi.d[e - 1], sub2(tds1, tdd1));
                }
                if (e < RR) {
                    accLo.s[e] = add2(accLo.s[e], sub2(tsd0, m001));
                    accLo.d[e] = add2(accLo.d[e], add2(tds0, tdd0));
                    accHi.s[e] = add2(accHi.s[e], add2(m001, tsd1));
                    accHi.d[e] = add2(accHi.d[e], add2(tds1, tdd1));
                }
            }
        }
        // the left-corner sums of this warp's first lane go to the previous warp's last lane
        float* xb = xch + ((u & 1) * WY + wy) * WX * RR;
        if (lane == 0) {
#pragma unroll
            for (int r = 0; r < RR; ++r) xb[wx * RR + r] = accLo.s[r].x - accLo.d[r].x;
        }
        if (__syncthreads_or(ok ? 0 : 1)) {
            failed = true;
            return;
        }
        // stage u is free: copy plane u + NS into it
        if (u + NS < nplanes) {
            if (tid == 0) issue(u + NS);
            issued = u + NS + 1;
        }
        // plane kstart + u is complete
        const int k = kstart + u;
        if (k >= k0) {
            const long long pb = s2 * k;
            float2 out[RR];
#pragma unroll
            for (int r = 0; r < RR; ++r) {
                const float2 right = add2(accLo.s[r], accLo.d[r]), left = sub2(accLo.s[r], accLo.d[r]);
                float recv = __shfl_down_sync(0xffffffffu, left.x, 1);
                if (lane == 31) recv = (wx + 1 < WX) ? xb[(wx + 1) * RR + r] : 0.f;
                out[r] = make_float2(right.x + left.y, right.y + recv);
            }
            // planes holding convective surface rows have a node -> row map; the rows of the
            // thread's 2 RR nodes are gathered together (independent loads in each round)
            const int sp = a.s.plane != nullptr ? a.s.plane[k] : 0;
            if (sp != 0) {
                int beg[2 * RR], cnt[2 * RR];
                int most = 0;
#pragma unroll
                for (int r = 0; r < RR; ++r) {
                    const int row = jw + r;
                    const bool in = c0 < a.n0 && row < a.n1;
                    const long long mb = (long long)(sp - 1) * s2 + (long long)row * a.n0 + c0;
#pragma unroll
                    for (int h = 0; h < 2; ++h) {
                        const int sr = in ? a.s.map[mb + h] : -1;
                        beg[2 * r + h] = sr >= 0 ? a.s.ptr[sr] : 0;
                        cnt[2 * r + h] = sr >= 0 ? a.s.ptr[sr + 1] - beg[2 * r + h] : 0;
                        most = max(most, cnt[2 * r + h]);
                    }
                }
                float acc[2 * RR];
#pragma unroll
                for (int i = 0; i < 2 * RR; ++i) acc[i] = 0.f;
                for (int q = 0; q < most; ++q) {
#pragma unroll
                    for (int i = 0; i < 2 * RR; ++i)
                        if (q < cnt[i]) acc[i] += a.s.val[beg[i] + q] * a.x[a.s.col[beg[i] + q]];
                }
#pragma unroll
                for (int r = 0; r < RR; ++r) {
                    out[r].x += acc[2 * r];
                    out[r].y += acc[2 * r + 1];
                }
            }
#pragma unroll
            for (int r = 0; r < RR; ++r) {
                const int row = jw + r;
                if (c0 < a.n0 && row < a.n1) {  // n0 is even: c0 + 1 < n0 too
                    dot = fma2(xrLo[r], out[r], dot);
                    *reinterpret_cast<float2*>(a.y + pb + (long long)row * a.n0 + c0) = out[r];
                }
            }
        }
#pragma unroll
        for (int r = 0; r < RR; ++r) accLo.s[r] = accLo.d[r] = make_float2(0.f, 0.f);
    };

    // prologue: plane 0 of the chunk
    {
        const bool ok = __all_sync(0xffffffffu, mbar_wait(bar_of(0), 0u));
        if (ok) {
            waited = 1;
            plane_stage(0, ya, xra);
        }
        failed = __syncthreads_or(ok ? 0 : 1) != 0;
    }
#pragma unroll
    for (int r = 0; r < RR; ++r) acca.s[r] = acca.d[r] = accb.s[r] = accb.d[r] = make_float2(0.f, 0.f);

    int u = 0;
    if (!failed) {
        for (; u + 1 < nlayers; u += 2) {
            layer(u, ya, yb, acca, accb, xra, xrb);
            if (failed) break;
            layer(u + 1, yb, ya, accb, acca, xrb, xra);
            if (failed) break;
        }
        if (!failed && u < nlayers) layer(u, ya, yb, acca, accb, xra, xrb);
    }

    pdl_trigger_at(2);
    if (failed) {
        // report, then wait (bounded) for the copies this block still has in flight
        if (tid == 0) {
            a.ctl->status = SOLVE_DEVICE_TIMEOUT;
            a.ctl->status2[0] = a.ctl->status2[1] = SOLVE_DEVICE_TIMEOUT;
            for (int v = waited; v < issued; ++v) mbar_wait(bar_of(v), (uint32_t)((v / NS) & 1));
        }
        __syncthreads();
        return;
    }

    // (x, A x): this block's partial; the next kernel reduces the partials of all blocks
    const int bid = blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z);
    float v[1] = {dot.x + dot.y};
    write_partial_f32<1>(v, a.partials, bid);
}

// P = k_xy dx dy dz / 48, Q = k_z dx dy / (16 dz) per element (padded layout), from the
// FP64 conductivities; padding elements (zero conductivity) give zero.
template <bool ANISO>
__global__ void __launch_bounds__(256) k_tma_coef(const GridT<double> g, const double* __restrict__ kxy,
                                                  const double* __restrict__ kz, float* __restrict__ P,
                                                  float* __restrict__ Q) {
    const int n0 = g.n0, n1 = g.n1, n2 = g.n2;
    const long long s2 = (long long)n0 * n1;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < g.N; e += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(e % n0), j = (int)((e / n0) % n1), k = (int)(e / s2);
        float pv = 0.f, qv = 0.f;
        if (i < n0 - 1 && j < n1 - 1 && k < n2 - 1) {
            const double dx = g.h0[i], dy = g.h1[j], dz = g.h2[k];
            pv = (float)(kxy[e] * dx * dy * dz * (1.0 / 48.0));
            if (ANISO) qv = (float)(kz[e] * dx * dy * (1.0 / 16.0) / dz);
        }
        P[e] = pv;
        if (ANISO) Q[e] = qv;
    }
}

// ----------------------------------------------------------------------------------------
// host side

namespace {

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q{};
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
        else
            (void)cudaGetLastError();
    });
    return fn;
}

bool encode_3d(CUtensorMap* map, const float* base, int n0, int n1, int n2, int box0, int box1) {
    auto fn = encode_fn();
    if (!fn) return false;
    const cuuint64_t dims[3] = {(cuuint64_t)n0, (cuuint64_t)n1, (cuuint64_t)n2};
    const cuuint64_t strides[2] = {(cuuint64_t)n0 * 4, (cuuint64_t)n0 * n1 * 4};
    const cuuint32_t box[3] = {(cuuint32_t)box0, (cuuint32_t)box1, 1};
    const cuuint32_t estr[3] = {1, 1, 1};
    return fn(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float*>(base), dims, strides, box, estr,
              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

template <int WX, bool ANISO>
void* kernel_of() {
    return reinterpret_cast<void*>(k_apply_tma<WX, kTmaRows, ANISO, kTmaStages>);
}
void* kernel_for(int wx, bool aniso) {
    switch (wx) {
        case 1: return aniso ? kernel_of<1, true>() : kernel_of<1, false>();
        case 2: return aniso ? kernel_of<2, true>() : kernel_of<2, false>();
        case 3: return aniso ? kernel_of<3, true>() : kernel_of<3, false>();
        default: return aniso ? kernel_of<4, true>() : kernel_of<4, false>();
    }
}

}  // namespace

struct TmaOperator {
    CUtensorMap mx, mp, mq;
    int n0 = 0, n1 = 0, n2 = 0, wx = 0, threads = 0;
    bool aniso = false;
    const float* x = nullptr;
    float* P = nullptr;
    float* Q = nullptr;
    dim3 grid;
    int zchunk = 0;
    int smem = 0;
    // geometry factors
    float* ax = nullptr;
    float* ay = nullptr;
    float* az3 = nullptr;
    ~TmaOperator() {
        for (float* p : {ax, ay, az3})
            if (p) cudaFree(p);
    }
};

// Where the kernel applies and pays: n0 a multiple of 4 (the copy's row stride must be a
// multiple of 16 bytes), at most 256, and at least 80 % of the warps' 64-column spans used
// (every lane issues the same instructions whether its columns exist or not).  Measured on
// the 200 x 200 x 120 coupled loop (78 % of the columns used): 72 us per CG iteration on this
// kernel against 63 us on the register-march kernel (95 % used).
// any_fill: ignore the 80 % rule (the kernel is correct for every n0 it can take).
bool tma_operator_supported(int n0, int n1, int n2, bool any_fill) {
    const int wx = (n0 + 63) / 64;
    return n0 >= 2 && n0 <= 64 * kTmaMaxWarpsX && (n0 % 4) == 0 && (any_fill || 5 * n0 >= 4 * 64 * wx) && n1 >= 2 &&
           n2 >= 2 && encode_fn() != nullptr;
}

TmaOperator* tma_operator_create(const LaunchCfg& c, const GridT<double>& g, const std::vector<double>& hx,
                                 const std::vector<double>& hy, const std::vector<double>& hz, bool aniso,
                                 const float* x, float* P, float* Q) {
    const int n0 = g.n0, n1 = g.n1, n2 = g.n2;
    if (!tma_operator_supported(n0, n1, n2, true)) return nullptr;
    std::unique_ptr<TmaOperator> t(new TmaOperator());
    t->n0 = n0;
    t->n1 = n1;
    t->n2 = n2;
    t->wx = (n0 + 63) / 64;
    t->threads = 32 * t->wx * tma_wy(t->wx);
    t->aniso = aniso;
    t->x = x;
    t->P = P;
    t->Q = Q;
    const int box = tma_box(t->wx), rows = kTmaRows * tma_wy(t->wx);
    if (!encode_3d(&t->mx, x, n0, n1, n2, box, rows + 2)) return nullptr;
    if (!encode_3d(&t->mp, P, n0, n1, n2, box, rows + 1)) return nullptr;
    if (!encode_3d(&t->mq, aniso ? Q : P, n0, n1, n2, box, rows + 1)) return nullptr;

    // geometry factors (host-computed from the FP64 axes)
    const int gy = (n1 + rows - 1) / rows;
    std::vector<float> ax((size_t)64 * t->wx, 0.f), ay((size_t)gy * rows + 2, 0.f), az((size_t)n2, 0.f);
    for (int cc = 1; cc < n0; ++cc) ax[cc] = (float)(1.0 / (hx[cc - 1] * hx[cc - 1]));
    for (int j = 0; j < n1 - 1; ++j) ay[(size_t)j + 1] = (float)(1.0 / (hy[j] * hy[j]));
    for (int k = 0; k < n2 - 1; ++k) az[k] = (float)(3.0 / (hz[k] * hz[k]));
    auto up = [&](float*& d, const std::vector<float>& v) {
        if (cudaMalloc(&d, v.size() * 4) != cudaSuccess) return false;
        return cudaMemcpyAsync(d, v.data(), v.size() * 4, cudaMemcpyHostToDevice, c.stream) == cudaSuccess;
    };
    if (!up(t->ax, ax) || !up(t->ay, ay) || !up(t->az3, az)) return nullptr;
    if (cudaStreamSynchronize(c.stream) != cudaSuccess) return nullptr;

    // launch shape: as many resident blocks as the shared memory allows; z-chunks picked so
    // that the most loaded SM does the least work, (blocks on it) x (planes + 1 recomputed)
    t->smem = tma_smem_bytes(t->wx, kTmaRows, aniso, kTmaStages);
    void* k = kernel_for(t->wx, aniso);
    if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, t->smem) != cudaSuccess) return nullptr;
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, t->threads, t->smem) != cudaSuccess || per_sm < 1)
        return nullptr;
    const int sms = std::max(1, c.sm_count / std::max(1, c.op_share));
    if (PLGPU_TMA_BLOCKS > 0) per_sm = std::min(per_sm, PLGPU_TMA_BLOCKS);
    long long best = -1;
    int best_zc = n2;
    for (int zc = 2; zc <= n2; ++zc) {
        const long long chunks = (n2 + zc - 1) / zc;
        if (zc > 2 && (n2 + zc - 2) / (zc - 1) == chunks) continue;  // the same chunk count with fewer planes
        const long long blocks = (long long)gy * chunks;
        if (blocks > kMaxPartialBlocks - 512) continue;
        const long long per = (blocks + sms - 1) / sms;
        const long long waves = (per + per_sm - 1) / per_sm;
        const long long cost = waves * std::min<long long>(per, per_sm) * (zc + 1);
        if (PLGPU_TMA_BLOCKS > 0 && (waves > 1 || per < per_sm)) continue;  // exactly per_sm blocks per SM
        if (best < 0 || cost < best) {
            best = cost;
            best_zc = zc;
        }
    }
    t->zchunk = best_zc;
    t->grid = dim3(1, gy, (n2 + best_zc - 1) / best_zc);
    return t.release();
}

void tma_operator_destroy(TmaOperator* t) { delete t; }

int tma_operator_blocks(const TmaOperator* t) { return (int)(t->grid.x * t->grid.y * t->grid.z); }

const float* tma_operator_input(const TmaOperator* t) { return t->x; }

bool tma_operator_aniso(const TmaOperator* t) { return t->aniso; }

void launch_tma_coef(const LaunchCfg& c, const TmaOperator* t, const GridT<double>& g, const double* kxy,
                     const double* kz) {
    if (t->aniso)
        launch_kernel(k_tma_coef<true>, dim3(vec_blocks(c, g.N)), dim3(256), c.stream, g, kxy, kz, t->P, t->Q);
    else
        launch_kernel(k_tma_coef<false>, dim3(vec_blocks(c, g.N)), dim3(256), c.stream, g, kxy, kz, t->P, t->Q);
}

template <int WX, bool ANISO>
static void launch_tma_one(const LaunchCfg& c, const TmaOperator* t, const TmaArgs& a) {
    launch_kernel_pdl(k_apply_tma<WX, kTmaRows, ANISO, kTmaStages>, t->grid, dim3(32 * WX * tma_wy(WX)), t->smem,
                      c.stream, t->mx, t->mp, t->mq, a);
}

void launch_operator_tma(const LaunchCfg& c, const TmaOperator* t, float* y, double* partials, const int* run,
                         SolveCtl* ctl, const TmaSurface& s) {
    TmaArgs a{t->n0, t->n1, t->n2, t->zchunk, t->x, y, partials, run, ctl, s, t->ax, t->ay, t->az3};
#define PLGPU_TMA_CASE(W)                     \
    case W:                                   \
        if (t->aniso)                         \
            launch_tma_one<W, true>(c, t, a); \
        else                                  \
            launch_tma_one<W, false>(c, t, a); \
        break;
    switch (t->wx) {
        PLGPU_TMA_CASE(1)
        PLGPU_TMA_CASE(2)
        PLGPU_TMA_CASE(3)
        PLGPU_TMA_CASE(4)
        default: break;
    }
#undef PLGPU_TMA_CASE
}

}  // namespace plgpu
