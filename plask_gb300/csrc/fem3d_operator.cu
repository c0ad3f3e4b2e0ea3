// Matrix-free stiffness operator for sm_103a: y = A x for the trilinear-hex FEM
// Laplacian with per-element conductivities (PLaSK therm3d.cpp:226-237, 270-275).
//
// Element algebra.  With X, Y, Z the scaled conductances of an element
// (X = kx dy dz / dx, ...), its 8x8 stiffness is
//     K_e = X (A (x) M (x) M) + Y (M (x) A (x) M) + Z (M (x) M (x) A),
//     A = [[1,-1],[-1,1]],  M = [[2,1],[1,2]] / 6.
// Writing M = (1/4) e e^T + (1/12) d d^T with e = (1,1), d = (-1,1) turns every
// term into a sum of rank-one products of the 2-point sum/difference vectors, so
//     K_e = H^T diag(lambda) H,
// H being the 8-point sum/difference butterfly (three stages of 4 butterflies)
// and, for the moments m = (mx, my, mz) in {0,1}^3 (1 = difference):
//     lambda_000 = 0,  lambda_100 = X/16,  lambda_010 = Y/16,  lambda_001 = Z/16,
//     lambda_110 = (X+Y)/48,  lambda_101 = (X+Z)/48,  lambda_011 = (Y+Z)/48,
//     lambda_111 = (X+Y+Z)/144.
// One element costs ~60 adds/multiplies instead of the ~200 of the explicit 8x8 form.
//
// Work layout.  Threads march along z (axis 2).  A warp covers 32 consecutive
// node columns in x (one per lane; lane l holds column i0 - 1 + l) and each
// thread R + 2 consecutive rows in y, so that every element it needs for its R
// output rows and the 30 interior lanes is computed inside the warp: x(i+1)
// comes from the next lane by shuffle, the contributions of an element to its
// i+1 corners go to the next lane by shuffle.  No shared memory, no barriers.
// Per output node: ~1.16 elements computed, 1 coalesced load of x, 1 of the
// conductivity (2 when anisotropic), 1 store.
#include <algorithm>
#include <cstdint>

#include "fem3d_device.cuh"
#include "fem3d_kernels.h"
#include "fem3d_reduce.cuh"

namespace plgpu {

template <typename R>
struct OpArgs {
    GridT<R> g;
    const R* x;
    R* y;
    const R* kxy;
    const R* kz;
    const uint32_t* dmask;
    const R* rhs;
    double* partials;
    SolveCtl* ctl;
    const R* zf;       // per element layer: dz / 48      (n2 - 1)
    const R* zr;       // per element layer: 1 / (48 dz)  (n2 - 1)
    int zchunk;        // planes per block along z
    // MODE_CG: nodes with a convective surface row (bit set) already hold S x in y,
    // written by k_surface, whose block partials of (x, S x) follow the operator's
    const uint32_t* smask;
    int sslots;
    // diagonal added to the operator, y += dshift x (the lumped heat capacity of the
    // time-stepping solver), or nullptr
    const R* dshift;
    // consistent heat capacity: per element (padded like the conductivities) the corner
    // capacity c, adding c (M (x) M (x) M), M = [[2,1],[1,2]] / 3, to the element matrix,
    // or nullptr
    const R* cmass;
    // MODE_CG inside the fused CG iteration (fem3d_cg_fused.cu): the launch runs only while
    // *run == SOLVE_RUNNING and leaves its block partials for the update kernel (no last-block
    // reduction); nullptr: the status word of ctl and the last block sets alpha
    const int* run;
};

// Weights of the consistent capacity in the butterfly basis: per axis M = (1/2) e e^T +
// (1/6) d d^T, so moment m gets c (1/2)^(#sums) (1/6)^(#differences).
template <typename R>
__device__ __forceinline__ void add_mass_weights(R c, R& l000, R& l100, R& l010, R& l001, R& l110, R& l101, R& l011,
                                                 R& l111) {
    const R c24 = c * R(1.0 / 24.0), c72 = c * R(1.0 / 72.0);
    l000 = c * R(0.125);
    l100 += c24;
    l010 += c24;
    l001 += c24;
    l110 += c72;
    l101 += c72;
    l011 += c72;
    l111 += c * R(1.0 / 216.0);
}

__device__ __forceinline__ bool dir_bit(const uint32_t* __restrict__ m, long long n) {
    return (__ldg(m + (n >> 5)) >> (n & 31)) & 1u;
}

// warp-level sum helpers for the partial dot product
__device__ __forceinline__ double warp_sum_d(double v) {
    for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// MINB: blocks per SM the register budget is sized for; UNR: unrolling of the z-march
// SHIFT: add the diagonal a.dshift (lumped capacity of time steps); MASS: add the
// consistent capacity a.cmass; static solves compile both out.
template <typename R, int RR, bool ANISO, int MODE, bool SHIFT = false, bool MASS = false,
          int MINB = (sizeof(R) == 4 ? 4 : 2), int UNR = 1>
__global__ void __launch_bounds__(128, MINB) k_apply_haar(const OpArgs<R> a) {
    if (MODE == MODE_CG &&
        (a.run != nullptr ? *a.run != SOLVE_RUNNING : (a.ctl != nullptr && a.ctl->status != SOLVE_RUNNING)))
        return;
    const int n0 = a.g.n0, n1 = a.g.n1, n2 = a.g.n2;
    const int s2 = n0 * n1;  // N < 2^31 (checked on the host)
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int i = blockIdx.x * 30 - 1 + lane;                      // node column of this lane
    const int jb = (blockIdx.y * (blockDim.x >> 5) + warp) * RR;   // first output row of the warp
    const int k0 = blockIdx.z * a.zchunk;
    const int k1 = min(k0 + a.zchunk, n2);
    const bool out_lane = lane >= 1 && lane <= 30 && i < n0;
    const bool have_i = i >= 0 && i < n0;
    const bool elem_i = i >= 0 && i < n0 - 1;

    // in-plane offsets of the node rows (-1: outside the mesh) and element rows (-1: no element)
    int noff[RR + 2], eoff[RR + 1];
#pragma unroll
    for (int r = 0; r < RR + 2; ++r) {
        const int j = jb - 1 + r;
        noff[r] = (have_i && j >= 0 && j < n1) ? i + n0 * j : -1;
    }
    // geometry of the element column (i, jb - 1 + e): X = k gx zf, Y = k gy zf, Z = kz gz zr
    R gx[RR + 1], gy[RR + 1], gz[RR + 1];
    {
        const R dx = elem_i ? a.g.h0[i] : R(0);
        const R rdx = elem_i ? a.g.r0[i] : R(0);
#pragma unroll
        for (int e = 0; e <= RR; ++e) {
            const int j = jb - 1 + e;
            const bool ok = elem_i && j >= 0 && j < n1 - 1;
            eoff[e] = ok ? i + n0 * j : -1;
            const R dy = ok ? a.g.h1[j] : R(0);
            const R rdy = ok ? a.g.r1[j] : R(0);
            gx[e] = dy * rdx;
            gy[e] = dx * rdy;
            gz[e] = dx * dy;
        }
    }

    auto load_x = [&](int k, R(&xv)[RR + 2]) {
        const bool kin = k >= 0 && k < n2;
        const R* base = a.x + (long long)s2 * (kin ? k : 0);
#pragma unroll
        for (int r = 0; r < RR + 2; ++r) {
            R v = R(0);
            if (kin && noff[r] >= 0) {
                v = base[noff[r]];
                if ((MODE == MODE_RESID || MODE == MODE_MULT) && dir_bit(a.dmask, (long long)s2 * k + noff[r])) v = R(0);
            }
            xv[r] = v;
        }
    };
    auto load_k = [&](int k, R(&kk)[RR + 1], R(&kv)[RR + 1], R(&cm)[MASS ? RR + 1 : 1]) {
        const bool kin = k >= 0 && k < n2 - 1;
        const long long b = (long long)s2 * (kin ? k : 0);
#pragma unroll
        for (int e = 0; e <= RR; ++e) {
            R v = R(0), w = R(0), c = R(0);
            if (kin && eoff[e] >= 0) {
                v = a.kxy[b + eoff[e]];
                if (ANISO) w = a.kz[b + eoff[e]];
                if constexpr (MASS) c = a.cmass[b + eoff[e]];
            }
            kk[e] = v;
            kv[e] = ANISO ? w : v;
            if constexpr (MASS) cm[e] = c;
        }
    };

    R acc[RR], nxt[RR];  // outputs of plane k (rows 1..RR) and partial plane k + 1
#pragma unroll
    for (int r = 0; r < RR; ++r) acc[r] = nxt[r] = R(0);

    R dot = R(0);  // per-thread partial of (x, A x); FP64 from the warp level on
    const int kstart = max(k0 - 1, 0);
    R xlo[RR + 2], xlo_p[RR + 2], xhi[RR + 2], xnx[RR + 2];
    R kk[RR + 1], kv[RR + 1], kkn[RR + 1], kvn[RR + 1];
    R cm[MASS ? RR + 1 : 1], cmn[MASS ? RR + 1 : 1];
    load_x(kstart, xlo);
    load_x(kstart + 1, xhi);
    load_k(kstart, kk, kv, cm);
#pragma unroll
    for (int r = 0; r < RR + 2; ++r) xlo_p[r] = __shfl_down_sync(0xffffffffu, xlo[r], 1);

#pragma unroll UNR
    for (int k = kstart; k < k1; ++k) {
        // prefetch the next plane and the next element layer while this layer is computed
        load_x(k + 2, xnx);
        load_k(k + 1, kkn, kvn, cmn);
        R xhi_p[RR + 2];
#pragma unroll
        for (int r = 0; r < RR + 2; ++r) xhi_p[r] = __shfl_down_sync(0xffffffffu, xhi[r], 1);
        const int kl = min(k, n2 - 2);
        const R zf = a.zf[kl], zr = a.zr[kl];
#pragma unroll
        for (int e = 0; e <= RR; ++e) {
            // lambda weights (X/48, Y/48, Z/48 scaled); zero conductivity gives zero contributions
            const R X = kk[e] * gx[e] * zf;
            const R Y = kk[e] * gy[e] * zf;
            const R Z = kv[e] * gz[e] * zr;
            R l100 = R(3) * X, l010 = R(3) * Y, l001 = R(3) * Z;
            R l110 = X + Y, l101 = X + Z, l011 = Y + Z;
            R l111 = (X + Y + Z) * R(1.0 / 3.0);
            R l000 = R(0);
            if constexpr (MASS) add_mass_weights(cm[e], l000, l100, l010, l001, l110, l101, l011, l111);
            // corners c = ci + 2 cj + 4 ck
            const R c0 = xlo[e], c1 = xlo_p[e], c2 = xlo[e + 1], c3 = xlo_p[e + 1];
            const R c4 = xhi[e], c5 = xhi_p[e], c6 = xhi[e + 1], c7 = xhi_p[e + 1];
            // forward butterfly: x, then y, then z
            const R sx0 = c0 + c1, dx0 = c1 - c0, sx1 = c2 + c3, dx1 = c3 - c2;
            const R sx2 = c4 + c5, dx2 = c5 - c4, sx3 = c6 + c7, dx3 = c7 - c6;
            const R ss0 = sx0 + sx1, sd0 = sx1 - sx0, ss1 = sx2 + sx3, sd1 = sx3 - sx2;
            const R ds0 = dx0 + dx1, dd0 = dx1 - dx0, ds1 = dx2 + dx3, dd1 = dx3 - dx2;
            const R m001 = (ss1 - ss0) * l001;
            const R m010 = (sd0 + sd1) * l010, m011 = (sd1 - sd0) * l011;
            const R m100 = (ds0 + ds1) * l100, m101 = (ds1 - ds0) * l101;
            const R m110 = (dd0 + dd1) * l110, m111 = (dd1 - dd0) * l111;
            // transposed butterfly: z, then y, then x (m000 = 0)
            const R tsd0 = m010 - m011, tsd1 = m010 + m011;
            const R tds0 = m100 - m101, tds1 = m100 + m101;
            const R tdd0 = m110 - m111, tdd1 = m110 + m111;
            R ys0 = -m001 - tsd0, ys1 = tsd0 - m001, ys2 = m001 - tsd1, ys3 = m001 + tsd1;
            if constexpr (MASS) {  // the all-sum moment m000 of the capacity
                const R m000 = (ss0 + ss1) * l000;
                const R tss0 = m000 - m001, tss1 = m000 + m001;
                ys0 = tss0 - tsd0;
                ys1 = tss0 + tsd0;
                ys2 = tss1 - tsd1;
                ys3 = tss1 + tsd1;
            }
            const R yd0 = tds0 - tdd0, yd1 = tds0 + tdd0, yd2 = tds1 - tdd1, yd3 = tds1 + tdd1;
            // own column (ci = 0): node rows e (cj = 0) and e + 1 (cj = 1); output rows are 1..RR
            if (e >= 1) {
                acc[e - 1] += ys0 - yd0;
                nxt[e - 1] += ys2 - yd2;
            }
            if (e + 1 <= RR) {
                acc[e] += ys1 - yd1;
                nxt[e] += ys3 - yd3;
            }
            // column i + 1 (ci = 1): to the next lane
            const R u0 = __shfl_up_sync(0xffffffffu, ys0 + yd0, 1);
            const R u1 = __shfl_up_sync(0xffffffffu, ys1 + yd1, 1);
            const R u2 = __shfl_up_sync(0xffffffffu, ys2 + yd2, 1);
            const R u3 = __shfl_up_sync(0xffffffffu, ys3 + yd3, 1);
            if (e >= 1) {
                acc[e - 1] += u0;
                nxt[e - 1] += u2;
            }
            if (e + 1 <= RR) {
                acc[e] += u1;
                nxt[e] += u3;
            }
        }
        // plane k is complete
        if (k >= k0) {
            const long long pb = (long long)s2 * k;
#pragma unroll
            for (int r = 1; r <= RR; ++r) {
                if (out_lane && noff[r] >= 0) {
                    const long long n = pb + noff[r];
                    if (SHIFT) acc[r - 1] += a.dshift[n] * xlo[r];
                    R out;
                    if (MODE == MODE_CG) {
                        // Dirichlet rows: x is zero there and M^-1 = 0 keeps the CG residual zero
                        out = acc[r - 1];
                        dot += xlo[r] * out;
                        if (a.smask != nullptr && dir_bit(a.smask, n)) out += a.y[n];
                    } else if (MODE == MODE_RESID) {
                        out = dir_bit(a.dmask, n) ? R(a.rhs[n] - a.x[n]) : R(a.rhs[n] - acc[r - 1]);
                    } else if (MODE == MODE_MULT) {
                        out = dir_bit(a.dmask, n) ? a.x[n] : acc[r - 1];
                    } else {
                        out = a.rhs[n] - acc[r - 1];
                    }
                    a.y[n] = out;
                }
            }
        }
#pragma unroll
        for (int r = 0; r < RR; ++r) {
            acc[r] = nxt[r];
            nxt[r] = R(0);
        }
#pragma unroll
        for (int r = 0; r < RR + 2; ++r) {
            xlo[r] = xhi[r];
            xlo_p[r] = xhi_p[r];
            xhi[r] = xnx[r];
        }
#pragma unroll
        for (int e = 0; e <= RR; ++e) {
            kk[e] = kkn[e];
            kv[e] = kvn[e];
            if constexpr (MASS) cm[e] = cmn[e];
        }
    }
    if (MODE == MODE_CG) {
        const int bid = blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z);
        // (x, A x): block partial, then the last block to finish adds the surface kernel's
        // partials and sets the step length
        double v[1] = {(double)dot};
        write_partial<1, OpSum>(v, a.partials, bid);
        const int nblocks = gridDim.x * gridDim.y * gridDim.z;
        if (a.run == nullptr && arrive_last(&a.ctl->arrive[0], nblocks)) {
            reduce_partials<1, OpSum>(v, a.partials, nblocks + a.sslots);
            if (threadIdx.x == 0) {
                const double pq = v[0];
                a.ctl->pq = pq;
                if (!isfinite(pq))
                    a.ctl->status = SOLVE_NONFINITE;
                else if (!(pq > 0.0))
                    a.ctl->status = SOLVE_BREAKDOWN;
                else
                    a.ctl->alpha = a.ctl->rz / pq;
            }
        }
    }
}

// The same operator with the butterfly stages shared between neighbouring elements.
// The x-stage (sum and difference of a node and its +x neighbour) of every node row is
// computed once per plane and used by the two element rows and two element layers that
// contain that x-edge; the contributions of all elements to a node row are accumulated as
// (sum, difference) pairs and unfolded into the two node columns once per plane, so one
// lane shuffle per output row replaces four per element.  Per output node this issues
// 11 % fewer FMA-pipe and 23 % fewer load/store-pipe instructions than k_apply_haar
// (ncu, 128x128x200, 4 rows per thread).
template <typename R, int RR, bool ANISO, int MODE, bool SHIFT = false, bool MASS = false,
          int MINB = (sizeof(R) == 4 ? 4 : 2)>
__global__ void __launch_bounds__(128, MINB) k_apply_shared(const OpArgs<R> a) {
    if (MODE == MODE_CG &&
        (a.run != nullptr ? *a.run != SOLVE_RUNNING : (a.ctl != nullptr && a.ctl->status != SOLVE_RUNNING)))
        return;
    const int n0 = a.g.n0, n1 = a.g.n1, n2 = a.g.n2;
    const int s2 = n0 * n1;  // N < 2^31 (checked on the host)
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int i = blockIdx.x * 30 - 1 + lane;
    const int jb = (blockIdx.y * (blockDim.x >> 5) + warp) * RR;
    const int k0 = blockIdx.z * a.zchunk;
    const int k1 = min(k0 + a.zchunk, n2);
    const bool out_lane = lane >= 1 && lane <= 30 && i < n0;
    const bool have_i = i >= 0 && i < n0;
    const bool elem_i = i >= 0 && i < n0 - 1;

    int noff[RR + 2], eoff[RR + 1];
#pragma unroll
    for (int r = 0; r < RR + 2; ++r) {
        const int j = jb - 1 + r;
        noff[r] = (have_i && j >= 0 && j < n1) ? i + n0 * j : -1;
    }
    R gx[RR + 1], gy[RR + 1], gz[RR + 1];
    {
        const R dx = elem_i ? a.g.h0[i] : R(0);
        const R rdx = elem_i ? a.g.r0[i] : R(0);
#pragma unroll
        for (int e = 0; e <= RR; ++e) {
            const int j = jb - 1 + e;
            const bool ok = elem_i && j >= 0 && j < n1 - 1;
            eoff[e] = ok ? i + n0 * j : -1;
            const R dy = ok ? a.g.h1[j] : R(0);
            const R rdy = ok ? a.g.r1[j] : R(0);
            gx[e] = dy * rdx;
            gy[e] = dx * rdy;
            gz[e] = dx * dy;
        }
    }
    auto load_x = [&](int k, R(&xv)[RR + 2]) {
        const bool kin = k >= 0 && k < n2;
        const R* base = a.x + (long long)s2 * (kin ? k : 0);
#pragma unroll
        for (int r = 0; r < RR + 2; ++r) {
            R v = R(0);
            if (kin && noff[r] >= 0) {
                v = base[noff[r]];
                if ((MODE == MODE_RESID || MODE == MODE_MULT) && dir_bit(a.dmask, (long long)s2 * k + noff[r])) v = R(0);
            }
            xv[r] = v;
        }
    };
    auto load_k = [&](int k, R(&kk)[RR + 1], R(&kv)[RR + 1], R(&cm)[MASS ? RR + 1 : 1]) {
        const bool kin = k >= 0 && k < n2 - 1;
        const long long b = (long long)s2 * (kin ? k : 0);
#pragma unroll
        for (int e = 0; e <= RR; ++e) {
            R v = R(0), w = R(0), c = R(0);
            if (kin && eoff[e] >= 0) {
                v = a.kxy[b + eoff[e]];
                if (ANISO) w = a.kz[b + eoff[e]];
                if constexpr (MASS) c = a.cmass[b + eoff[e]];
            }
            kk[e] = v;
            kv[e] = ANISO ? w : v;
            if constexpr (MASS) cm[e] = c;
        }
    };
    // x-stage of a plane: s = x + x(i+1), d = x(i+1) - x per node row
    auto xstage = [&](const R(&xv)[RR + 2], R(&sx)[RR + 2], R(&dx)[RR + 2]) {
#pragma unroll
        for (int r = 0; r < RR + 2; ++r) {
            const R xp = __shfl_down_sync(0xffffffffu, xv[r], 1);
            sx[r] = xv[r] + xp;
            dx[r] = xp - xv[r];
        }
    };

    // (sum, difference) accumulators of the output rows 1..RR: plane k and plane k + 1
    R accS[RR], accD[RR], nxtS[RR], nxtD[RR];
#pragma unroll
    for (int r = 0; r < RR; ++r) accS[r] = accD[r] = nxtS[r] = nxtD[r] = R(0);

    R dot = R(0);
    const int kstart = max(k0 - 1, 0);
    R xlo[RR], xhi[RR + 2], xnx[RR + 2];  // xlo: raw x of the output rows of plane k
    R sxl[RR + 2], dxl[RR + 2];
    R kk[RR + 1], kv[RR + 1], kkn[RR + 1], kvn[RR + 1];
    R cm[MASS ? RR + 1 : 1], cmn[MASS ? RR + 1 : 1];
    {
        R x0[RR + 2];
        load_x(kstart, x0);
        xstage(x0, sxl, dxl);
#pragma unroll
        for (int r = 0; r < RR; ++r) xlo[r] = x0[r + 1];
    }
    load_x(kstart + 1, xhi);
    load_k(kstart, kk, kv, cm);

    for (int k = kstart; k < k1; ++k) {
        load_x(k + 2, xnx);
        load_k(k + 1, kkn, kvn, cmn);
        R sxh[RR + 2], dxh[RR + 2];
        xstage(xhi, sxh, dxh);
        const int kl = min(k, n2 - 2);
        const R zf = a.zf[kl], zr = a.zr[kl];
#pragma unroll
        for (int e = 0; e <= RR; ++e) {
            const R X = kk[e] * gx[e] * zf;
            const R Y = kk[e] * gy[e] * zf;
            const R Z = kv[e] * gz[e] * zr;
            R l100 = R(3) * X, l010 = R(3) * Y, l001 = R(3) * Z;
            R l110 = X + Y, l101 = X + Z, l011 = Y + Z;
            R l111 = (X + Y + Z) * R(1.0 / 3.0);
            R l000 = R(0);
            if constexpr (MASS) add_mass_weights(cm[e], l000, l100, l010, l001, l110, l101, l011, l111);
            // y-stage of the rows e, e + 1 on both planes
            const R ss0 = sxl[e] + sxl[e + 1], sd0 = sxl[e + 1] - sxl[e];
            const R ds0 = dxl[e] + dxl[e + 1], dd0 = dxl[e + 1] - dxl[e];
            const R ss1 = sxh[e] + sxh[e + 1], sd1 = sxh[e + 1] - sxh[e];
            const R ds1 = dxh[e] + dxh[e + 1], dd1 = dxh[e + 1] - dxh[e];
            // z-stage and the weights
            const R m001 = (ss1 - ss0) * l001;
            const R m010 = (sd0 + sd1) * l010, m011 = (sd1 - sd0) * l011;
            const R m100 = (ds0 + ds1) * l100, m101 = (ds1 - ds0) * l101;
            const R m110 = (dd0 + dd1) * l110, m111 = (dd1 - dd0) * l111;
            // transposed z- and y-stages: (sum, difference) pairs of the four node rows
            const R tsd0 = m010 - m011, tsd1 = m010 + m011;
            const R tds0 = m100 - m101, tds1 = m100 + m101;
            const R tdd0 = m110 - m111, tdd1 = m110 + m111;
            R s0 = -m001 - tsd0, s1 = tsd0 - m001, s2n = m001 - tsd1, s3 = m001 + tsd1;
            if constexpr (MASS) {  // the all-sum moment m000 of the capacity
                const R m000 = (ss0 + ss1) * l000;
                const R tss0 = m000 - m001, tss1 = m000 + m001;
                s0 = tss0 - tsd0;
                s1 = tss0 + tsd0;
                s2n = tss1 - tsd1;
                s3 = tss1 + tsd1;
            }
            if (e >= 1) {  // row e (cj = 0)
                accS[e - 1] += s0;
                accD[e - 1] += tds0 - tdd0;
                nxtS[e - 1] += s2n;
                nxtD[e - 1] += tds1 - tdd1;
            }
            if (e + 1 <= RR) {  // row e + 1 (cj = 1)
                accS[e] += s1;
                accD[e] += tds0 + tdd0;
                nxtS[e] += s3;
                nxtD[e] += tds1 + tdd1;
            }
        }
        // plane k is complete: own column s - d, column i + 1 (the next lane) s + d
        if (k >= k0) {
            const long long pb = (long long)s2 * k;
#pragma unroll
            for (int r = 1; r <= RR; ++r) {
                const R recv = __shfl_up_sync(0xffffffffu, accS[r - 1] + accD[r - 1], 1);
                R res = (accS[r - 1] - accD[r - 1]) + recv;
                if (out_lane && noff[r] >= 0) {
                    const long long n = pb + noff[r];
                    if (SHIFT) res += a.dshift[n] * xlo[r - 1];
                    R out;
                    if (MODE == MODE_CG) {
                        out = res;
                        dot += xlo[r - 1] * out;
                        if (a.smask != nullptr && dir_bit(a.smask, n)) out += a.y[n];
                    } else if (MODE == MODE_RESID) {
                        out = dir_bit(a.dmask, n) ? R(a.rhs[n] - a.x[n]) : R(a.rhs[n] - res);
                    } else if (MODE == MODE_MULT) {
                        out = dir_bit(a.dmask, n) ? a.x[n] : res;
                    } else {
                        out = a.rhs[n] - res;
                    }
                    a.y[n] = out;
                }
            }
        }
#pragma unroll
        for (int r = 0; r < RR; ++r) {
            accS[r] = nxtS[r];
            accD[r] = nxtD[r];
            nxtS[r] = nxtD[r] = R(0);
            xlo[r] = xhi[r + 1];
        }
#pragma unroll
        for (int r = 0; r < RR + 2; ++r) {
            sxl[r] = sxh[r];
            dxl[r] = dxh[r];
            xhi[r] = xnx[r];
        }
#pragma unroll
        for (int e = 0; e <= RR; ++e) {
            kk[e] = kkn[e];
            kv[e] = kvn[e];
            if constexpr (MASS) cm[e] = cmn[e];
        }
    }
    if (MODE == MODE_CG) {
        const int bid = blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z);
        double v[1] = {(double)dot};
        write_partial<1, OpSum>(v, a.partials, bid);
        const int nblocks = gridDim.x * gridDim.y * gridDim.z;
        if (a.run == nullptr && arrive_last(&a.ctl->arrive[0], nblocks)) {
            reduce_partials<1, OpSum>(v, a.partials, nblocks + a.sslots);
            if (threadIdx.x == 0) {
                const double pq = v[0];
                a.ctl->pq = pq;
                if (!isfinite(pq))
                    a.ctl->status = SOLVE_NONFINITE;
                else if (!(pq > 0.0))
                    a.ctl->status = SOLVE_BREAKDOWN;
                else
                    a.ctl->alpha = a.ctl->rz / pq;
            }
        }
    }
}

// ----------------------------------------------------------------------------------------

namespace {
constexpr int kWarps = 4;
}  // namespace

// Output rows per thread: FP32 4, 5 or 6 (LaunchCfg::op_rows, chosen per mesh by
// choose_op_rows; all three fit 128 registers, 4 blocks of 128 threads per SM, without
// spills in CG mode), FP64 4 (twice the registers per value).
static int op_rows(const LaunchCfg& c, bool fp64) {
    if (fp64) return 4;
    return (c.op_rows == 4 || c.op_rows == 5) ? c.op_rows : 6;
}

static void op_grid(const LaunchCfg& c, int n0, int n1, int n2, bool fp64, dim3& grid, int& zchunk) {
    const int rows = op_rows(c, fp64);
    const int gx = (n0 + 29) / 30;
    const int gy = (n1 + rows * kWarps - 1) / (rows * kWarps);
    // z-chunks: fill whole waves of resident blocks (4 per SM in FP32, 2 in FP64),
    // each chunk at least 8 planes (one extra element layer is recomputed per chunk).
    // A mesh whose columns cannot fill one wave with 8-plane chunks takes shorter
    // chunks (down to 4 planes) up to one wave, and then every chunk it has.
    const int resident = max(1, c.sm_count * (fp64 ? 2 : 4) / max(1, c.op_share));
    const int columns = gx * gy;
    int maxchunks = max(1, (n2 + 7) / 8);
    if ((long long)columns * maxchunks < resident)
        maxchunks = max(maxchunks, min((n2 + 3) / 4, (resident + columns - 1) / columns));
    int chunks = 1;
    if ((long long)columns * maxchunks <= resident) {
        chunks = maxchunks;
    } else {
        for (int waves = 1; waves <= 8; ++waves) {
            const int want = (waves * resident) / columns;
            if (want > maxchunks) break;
            if (want >= 1) chunks = want;
        }
    }
    while ((long long)gx * gy * chunks > kMaxPartialBlocks - 256) --chunks;
    zchunk = (n2 + chunks - 1) / chunks;
    chunks = (n2 + zchunk - 1) / zchunk;
    grid = dim3(gx, gy, chunks);
}

// The FP32 tile for a mesh with n1 nodes along axis 1.  A block covers 4 warps x r rows
// of axis 1 and computes r + 1 element rows per warp: the cost per useful row is
// (rows covered / n1) x (r + 1) / r.  Pick the smallest (then the fewest rows on a tie).
// The choice is a fixed function of the mesh, so results do not depend on timing
// (the tile changes the order in which (p, A p) is summed).  Measured at 128x128x200:
// r = 4, 5, 6 take 32.4, 34.3, 35.9 us per launch; the model picks 4.
int choose_op_rows(int n1) {
    int best = 6;
    double best_cost = 1e300;
    for (int r : {4, 5, 6}) {
        const int per_block = r * kWarps;
        const double covered = (double)((n1 + per_block - 1) / per_block) * per_block;
        const double cost = covered / n1 * (r + 1) / r;
        if (cost < best_cost - 1e-12) {
            best_cost = cost;
            best = r;
        }
    }
    return best;
}

int op_blocks(const LaunchCfg& c, int n0, int n1, int n2, bool fp64) {
    dim3 g;
    int z;
    op_grid(c, n0, n1, n2, fp64, g, z);
    return (int)(g.x * g.y * g.z);
}

// FP32 tiles of 4 and 5 rows run the shared-stage kernel (measured at 128x128x200:
// 32.4 and 34.3 us against 34.5 and 35.6 us for k_apply_haar); 6 rows and FP64 keep
// k_apply_haar (the shared form spills at 6 rows in 128 registers).
template <typename R, int RR, bool ANISO, int MODEV, bool SHIFT, bool MASS>
static void op_launch_one(const LaunchCfg& c, dim3 grid, const OpArgs<R>& a) {
    if constexpr (sizeof(R) == 4 && RR <= 5)
        launch_kernel(k_apply_shared<R, RR, ANISO, MODEV, SHIFT, MASS>, grid, dim3(32 * kWarps), c.stream, a);
    else
        launch_kernel(k_apply_haar<R, RR, ANISO, MODEV, SHIFT, MASS>, grid, dim3(32 * kWarps), c.stream, a);
}

template <typename R, int RR>
static void op_launch_rows(const LaunchCfg& c, dim3 grid, const OpArgs<R>& a, bool aniso, int mode) {
    // at most one capacity form: a lumped diagonal or the consistent element matrices
    const int cap = a.cmass != nullptr ? 2 : a.dshift != nullptr ? 1 : 0;
#define PLGPU_OP_A(MODEV, ANISOV)                                           \
    if (cap == 2)                                                           \
        op_launch_one<R, RR, ANISOV, MODEV, false, true>(c, grid, a);       \
    else if (cap == 1)                                                      \
        op_launch_one<R, RR, ANISOV, MODEV, true, false>(c, grid, a);       \
    else                                                                    \
        op_launch_one<R, RR, ANISOV, MODEV, false, false>(c, grid, a);
#define PLGPU_OP(MODEV)              \
    if (mode == MODEV) {             \
        if (aniso) {                 \
            PLGPU_OP_A(MODEV, true)  \
        } else {                     \
            PLGPU_OP_A(MODEV, false) \
        }                            \
        return;                      \
    }
    PLGPU_OP(MODE_CG)
    PLGPU_OP(MODE_RESID)
    PLGPU_OP(MODE_RHS)
    PLGPU_OP(MODE_MULT)
#undef PLGPU_OP
#undef PLGPU_OP_A
}

template <typename R>
static void op_launch(const LaunchCfg& c, const GridT<R>& g, const R* zf, const R* zr, const R* x, R* y, const R* kxy,
                      const R* kz, bool aniso, const uint32_t* dmask, const R* rhs, double* partials, int mode,
                      SolveCtl* ctl, const uint32_t* smask, int sslots, const R* dshift, const R* cmass,
                      const int* run = nullptr) {
    constexpr bool fp64 = sizeof(R) == 8;
    dim3 grid;
    int zchunk;
    op_grid(c, g.n0, g.n1, g.n2, fp64, grid, zchunk);
    OpArgs<R> a{g, x, y, kxy, kz, dmask, rhs, partials, ctl, zf, zr, zchunk, smask, sslots, dshift, cmass, run};
    if constexpr (fp64) {
        op_launch_rows<R, 4>(c, grid, a, aniso, mode);
    } else {
        switch (op_rows(c, false)) {
            case 4: op_launch_rows<R, 4>(c, grid, a, aniso, mode); break;
            case 5: op_launch_rows<R, 5>(c, grid, a, aniso, mode); break;
            default: op_launch_rows<R, 6>(c, grid, a, aniso, mode); break;
        }
    }
}

void launch_operator(const LaunchCfg& c, const GridT<float>& g, const float* zf, const float* zr, const float* x,
                     float* y, const float* kxy, const float* kz, bool aniso, const uint32_t* dmask, const float* rhs,
                     double* partials, int mode, SolveCtl* ctl, const uint32_t* smask, int sslots,
                     const float* dshift, const float* cmass, const int* run) {
    op_launch<float>(c, g, zf, zr, x, y, kxy, kz, aniso, dmask, rhs, partials, mode, ctl, smask, sslots, dshift,
                     cmass, run);
}
void launch_operator(const LaunchCfg& c, const GridT<double>& g, const double* zf, const double* zr, const double* x,
                     double* y, const double* kxy, const double* kz, bool aniso, const uint32_t* dmask,
                     const double* rhs, double* partials, int mode, SolveCtl* ctl, const uint32_t* smask,
                     int sslots, const double* dshift, const double* cmass) {
    op_launch<double>(c, g, zf, zr, x, y, kxy, kz, aniso, dmask, rhs, partials, mode, ctl, smask, sslots, dshift,
                      cmass);
}

}  // namespace plgpu
