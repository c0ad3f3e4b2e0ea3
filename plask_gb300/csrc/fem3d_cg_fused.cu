// FP32 Jacobi-preconditioned conjugate gradients on the TMA-staged operator, for sm_103a.
//
// The inner correction solve of the mixed-precision Static3D solver (the replacement of
// the reference's solveMatrix, cholesky_matrix.hpp:90-111 / iterative_matrix.hpp:141-339).
// An iteration is three kernels:
//     operator  (k_apply_tma):        q = A p (convective surface rows included), partials of (p, q)
//     update    (k_tmacg_update):     alpha = rz / (p, q),  r -= alpha q,
//                                     partials of (r, M^-1 r), (r, r)
//     direction (k_tmacg_direction):  x += alpha p,  rz' = (r, M^-1 r),  beta = rz' / rz,
//                                     p = M^-1 r + beta p
// No kernel waits for its own blocks: every block of the update and direction kernels
// reduces the previous launch's partials itself, in the same fixed order (so all blocks
// see the same bits and take the same decision), and block 0 records the scalars.  The
// words a launch both reads and writes alternate with the iteration parity q: the
// kernels of parity q read rz2[q] and status2[q], the direction kernel writes slot 1 - q.
// The stopping test, the stagnation watch and the iteration cap are those of k_cg_update
// (fem3d_kernels.cu), taken on the new residual after each update.
#include <algorithm>
#include <cstdint>

#include "fem3d_device.cuh"
#include "fem3d_kernels.h"
#include "fem3d_reduce.cuh"

namespace plgpu {

// Block size of the update and direction kernels (overridable at compile time for tuning
// sweeps); the grid is 1024 threads per SM (one wave), 64 registers per thread.
#ifndef PLGPU_CG_THREADS
#define PLGPU_CG_THREADS 256
#endif
constexpr int kCgThreads = PLGPU_CG_THREADS;

namespace {
// float4 groups in flight per thread (overridable at compile time for tuning sweeps)
#ifndef PLGPU_CG_UNROLL
#define PLGPU_CG_UNROLL 2
#endif
constexpr int kUnroll = PLGPU_CG_UNROLL;
constexpr size_t kPQ = 0;                          // (p, A p): one value per operator block
constexpr size_t kRZ = (size_t)kMaxPartialBlocks;  // (r, M^-1 r) and (r, r) per update block
}  // namespace

// x = 0, p = M^-1 r, rz = (r, M^-1 r), rr = (r, r); the last block sets the stop threshold
// and the status (as k_cg_start) and the words of both parities
__global__ void __launch_bounds__(kCgThreads) k_tmacg_start(const TmaCg f, SolveCtl* __restrict__ ctl, double rtol,
                                                     int ref_slot, int maxit, int stall_limit) {
    float rz = 0.f, rr = 0.f;
    for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < f.N;
         n += (long long)gridDim.x * blockDim.x) {
        const float rn = f.r[n];
        const float zn = f.minv[n] * rn;
        f.p[n] = zn;
        f.x[n] = 0.f;
        rz += rn * zn;
        rr += rn * rn;
    }
    double v[2] = {(double)rz, (double)rr};
    write_partial<2, OpSum>(v, f.part + kRZ, blockIdx.x);
    if (arrive_last(&ctl->arrive[1], gridDim.x)) {
        reduce_partials<2, OpSum>(v, f.part + kRZ, gridDim.x);
        if (linear_tid() == 0) {
            const double m0 = ctl->plain ? v[1] : v[0];
            const double ref = ref_slot >= 0 ? ctl->red[ref_slot] : m0;
            ctl->rz = v[0];
            ctl->rz_old = v[0];
            ctl->rr = v[1];
            ctl->tol2 = rtol * rtol * ref;
            ctl->best_rr = m0;
            ctl->iter = 0;
            ctl->maxit = maxit;
            ctl->stall = 0;
            ctl->stall_limit = stall_limit;
            ctl->alpha = 0.0;
            ctl->beta = 0.0;
            ctl->pq = 0.0;
            int st = SOLVE_RUNNING;
            if (!isfinite(v[0]) || !isfinite(v[1]))
                st = SOLVE_NONFINITE;
            else if (m0 <= ctl->tol2 || v[1] == 0.0)
                st = SOLVE_CONVERGED;
            else if (!(v[0] > 0.0))
                st = SOLVE_BREAKDOWN;
            ctl->status = st;
            ctl->status2[0] = ctl->status2[1] = st;
            ctl->rz2[0] = ctl->rz2[1] = v[0];
        }
    }
}

__device__ __forceinline__ void tmacg_update_one(float& r, float q, float m, float alpha, float& rz, float& rr) {
    // Dirichlet rows (M^-1 = 0) keep r = 0: the operator leaves A p there
    const float rn = m != 0.f ? r - alpha * q : 0.f;
    r = rn;
    rz += rn * (m * rn);
    rr += rn * rn;
}

// r -= alpha q and the partials of (r, M^-1 r), (r, r).  The solution update x += alpha p
// waits for the direction kernel, which reads p anyway.  The first trip's loads do not
// depend on alpha and are issued before warp 0 reduces the operator's partials.
__global__ void __launch_bounds__(kCgThreads, 1024 / kCgThreads) k_tmacg_update(const TmaCg f, SolveCtl* __restrict__ ctl, int q) {
    pdl_trigger_at(1);
    pdl_wait();
    if (ctl->status2[q] != SOLVE_RUNNING) return;
    const long long N4 = f.N >> 2, stride = (long long)gridDim.x * blockDim.x;
    const long long t0 = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    float4* r4 = reinterpret_cast<float4*>(f.r);
    const float4* q4 = reinterpret_cast<const float4*>(f.q);
    const float4* m4 = reinterpret_cast<const float4*>(f.minv);
    float4 qn[kUnroll], mn[kUnroll], rn[kUnroll];
    auto load = [&](long long v0) {
#pragma unroll
        for (int u = 0; u < kUnroll; ++u) {
            const long long v = v0 + u * stride;
            if (v < N4) {
                qn[u] = q4[v];
                mn[u] = m4[v];
                rn[u] = r4[v];
            }
        }
    };
    load(t0);
    // warp 0 reduces the operator's partials; lane 0 takes the decision for the block
    __shared__ int sh_st;
    __shared__ float sh_alpha;
    if (threadIdx.x < 32) {
        double pv[1];
        warp0_reduce_partials<1>(pv, f.part + kPQ, f.op_blocks);
        if (threadIdx.x == 0) {
            const double pq = pv[0];
            const double rz = ctl->rz2[q];
            int st = SOLVE_RUNNING;
            if (!isfinite(pq))
                st = SOLVE_NONFINITE;
            else if (!(pq > 0.0))
                st = SOLVE_BREAKDOWN;
            const double alpha = st == SOLVE_RUNNING ? rz / pq : 0.0;
            sh_st = st;
            sh_alpha = (float)alpha;
            if (blockIdx.x == 0) {
                ctl->ustatus = st;
                ctl->pq = pq;
                ctl->alpha = alpha;
            }
        }
    }
    __syncthreads();
    if (sh_st != SOLVE_RUNNING) return;
    const float alpha = sh_alpha;
    float rzn = 0.f, rr = 0.f;
    // kUnroll groups per trip, all loads issued first; each thread visits its groups in
    // increasing order (a fixed summation order)
    for (long long v0 = t0; v0 < N4; v0 += kUnroll * stride) {
        if (v0 != t0) load(v0);
#pragma unroll
        for (int u = 0; u < kUnroll; ++u) {
            const long long v = v0 + u * stride;
            if (v < N4) {
                tmacg_update_one(rn[u].x, qn[u].x, mn[u].x, alpha, rzn, rr);
                tmacg_update_one(rn[u].y, qn[u].y, mn[u].y, alpha, rzn, rr);
                tmacg_update_one(rn[u].z, qn[u].z, mn[u].z, alpha, rzn, rr);
                tmacg_update_one(rn[u].w, qn[u].w, mn[u].w, alpha, rzn, rr);
                r4[v] = rn[u];
            }
        }
    }
    for (long long n = (N4 << 2) + t0; n < f.N; n += stride) {
        float r1 = f.r[n];
        tmacg_update_one(r1, f.q[n], f.minv[n], alpha, rzn, rr);
        f.r[n] = r1;
    }
    pdl_trigger_at(2);
    float v[2] = {rzn, rr};
    write_partial_f32<2>(v, f.part + kRZ, blockIdx.x);
}

// x += alpha p with the step of this iteration's update, then rz' = (r, M^-1 r),
// beta = rz' / rz and p = M^-1 r + beta p unless the solve has stopped.  The first trip's
// loads are issued before warp 0 reduces the update's partials.
__global__ void __launch_bounds__(kCgThreads, 1024 / kCgThreads) k_tmacg_direction(const TmaCg f, SolveCtl* __restrict__ ctl, int q) {
    pdl_trigger_at(1);
    pdl_wait();
    const int st0 = ctl->status2[q];
    if (st0 != SOLVE_RUNNING) {  // pass a final status on to the other parity
        if (blockIdx.x == 0 && threadIdx.x == 0) ctl->status2[1 - q] = st0;
        return;
    }
    const int ust = ctl->ustatus;
    if (ust != SOLVE_RUNNING) {  // the update found no valid step: x stays
        if (blockIdx.x == 0 && threadIdx.x == 0) ctl->status2[1 - q] = ctl->status = ust;
        return;
    }
    const long long N4 = f.N >> 2, stride = (long long)gridDim.x * blockDim.x;
    const long long t0 = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    float4* p4 = reinterpret_cast<float4*>(f.p);
    float4* x4 = reinterpret_cast<float4*>(f.x);
    const float4* r4 = reinterpret_cast<const float4*>(f.r);
    const float4* m4 = reinterpret_cast<const float4*>(f.minv);
    float4 rn[kUnroll], mn[kUnroll], pn[kUnroll], xn[kUnroll];
    auto load = [&](long long v0) {
#pragma unroll
        for (int u = 0; u < kUnroll; ++u) {
            const long long vv = v0 + u * stride;
            if (vv < N4) {
                pn[u] = p4[vv];
                xn[u] = x4[vv];
                rn[u] = r4[vv];
                mn[u] = m4[vv];
            }
        }
    };
    load(t0);
    // warp 0 reduces the update's partials; lane 0 takes the decision for the block
    __shared__ int sh_st;
    __shared__ float sh_beta, sh_alpha;
    __shared__ double sh_v[3];
    if (threadIdx.x < 32) {
        double v[2];
        warp0_reduce_partials<2>(v, f.part + kRZ, f.upd_blocks);
        if (threadIdx.x == 0) {
            const double rzn = v[0], rrn = v[1];
            const double m = ctl->plain ? rrn : rzn;
            int st = SOLVE_RUNNING;
            if (!isfinite(rrn) || !isfinite(rzn))
                st = SOLVE_NONFINITE;
            else if (m <= ctl->tol2)
                st = SOLVE_CONVERGED;
            sh_st = st;
            sh_beta = (float)(rzn / ctl->rz2[q]);
            sh_alpha = (float)ctl->alpha;
            sh_v[0] = rzn;
            sh_v[1] = rrn;
            sh_v[2] = m;
        }
    }
    __syncthreads();
    int st = sh_st;
    const bool more = st == SOLVE_RUNNING;
    const float beta = sh_beta, alpha = sh_alpha;
    for (long long v0 = t0; v0 < N4; v0 += kUnroll * stride) {
        if (v0 != t0) load(v0);
#pragma unroll
        for (int u = 0; u < kUnroll; ++u) {
            const long long vv = v0 + u * stride;
            if (vv < N4) {
                xn[u].x += alpha * pn[u].x;
                xn[u].y += alpha * pn[u].y;
                xn[u].z += alpha * pn[u].z;
                xn[u].w += alpha * pn[u].w;
                x4[vv] = xn[u];
                if (more) {
                    pn[u].x = mn[u].x * rn[u].x + beta * pn[u].x;
                    pn[u].y = mn[u].y * rn[u].y + beta * pn[u].y;
                    pn[u].z = mn[u].z * rn[u].z + beta * pn[u].z;
                    pn[u].w = mn[u].w * rn[u].w + beta * pn[u].w;
                    p4[vv] = pn[u];
                }
            }
        }
    }
    for (long long n = (N4 << 2) + t0; n < f.N; n += stride) {
        const float pn1 = f.p[n];
        f.x[n] += alpha * pn1;
        if (more) f.p[n] = f.minv[n] * f.r[n] + beta * pn1;
    }
    pdl_trigger_at(2);
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        const double rzn = sh_v[0], rrn = sh_v[1], m = sh_v[2], rz = ctl->rz2[q];
        ctl->iter += 1;
        ctl->rz_old = rz;
        ctl->rz = rzn;
        ctl->rr = rrn;
        ctl->beta = rzn / rz;
        ctl->rz2[1 - q] = rzn;
        if (st == SOLVE_RUNNING) {
            if (ctl->iter >= ctl->maxit) {
                st = SOLVE_MAXIT;
            } else if (m < 0.81 * ctl->best_rr) {  // residual norm fell by 10 %
                ctl->best_rr = m;
                ctl->stall = 0;
            } else if (++ctl->stall > ctl->stall_limit) {
                st = SOLVE_STAGNATED;
            }
        }
        ctl->status2[1 - q] = st;
        if (st != SOLVE_RUNNING) ctl->status = st;
    }
}

__global__ void __launch_bounds__(256) k_partials_to_ctl(const double* __restrict__ partials, int nslots,
                                                         SolveCtl* __restrict__ ctl) {
    double v[1];
    reduce_partials<1, OpSum>(v, partials, nslots);
    if (threadIdx.x == 0) ctl->pq = v[0];
}

void launch_tmacg_start(const LaunchCfg& c, const TmaCg& f, SolveCtl* ctl, double rtol, int ref_slot, int maxit,
                        int stall_limit) {
    launch_kernel(k_tmacg_start, dim3(f.upd_blocks), dim3(kCgThreads), c.stream, f, ctl, rtol, ref_slot, maxit, stall_limit);
}

double* tmacg_op_partials(const TmaCg& f) { return f.part + kPQ; }

const int* tmacg_op_run(SolveCtl* ctl, int q) { return &ctl->status2[q]; }

void launch_tmacg_update(const LaunchCfg& c, const TmaCg& f, SolveCtl* ctl, int q) {
    launch_kernel_pdl(k_tmacg_update, dim3(f.upd_blocks), dim3(kCgThreads), 0, c.stream, f, ctl, q);
}

void launch_tmacg_direction(const LaunchCfg& c, const TmaCg& f, SolveCtl* ctl, int q) {
    launch_kernel_pdl(k_tmacg_direction, dim3(f.upd_blocks), dim3(kCgThreads), 0, c.stream, f, ctl, q);
}

// one wave of resident blocks (of the share of the GPU the handle's grid policy aims at),
// fewer for small meshes (down to one block per SM of that share: a thread takes at least
// kUnroll float4 groups, and every block reduces the others' partials)
int tmacg_blocks(const LaunchCfg& c, long long N) {
    const long long sms = std::max(1, c.sm_count / std::max(1, c.op_share));
    const long long wave = sms * (1024 / kCgThreads);
    const long long need = ((N >> 2) + (long long)kCgThreads * kUnroll - 1) / ((long long)kCgThreads * kUnroll);
    return (int)std::min(wave, std::max(sms, need));
}

void launch_partials_to_ctl(const LaunchCfg& c, const double* partials, int nslots, SolveCtl* ctl) {
    launch_kernel(k_partials_to_ctl, dim3(1), dim3(256), c.stream, partials, nslots, ctl);
}

}  // namespace plgpu
