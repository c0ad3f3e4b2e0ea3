// Kernels of the Shockley3D FEM core (PLaSK solvers/electrical/shockley/electr3d.cpp).
// The stiffness operator is the thermal one fed with electrical conductivities, so
// only the conductivity bookkeeping, the junction update and the post-processing
// live here:
//
//   k_elec_init_cond        loadConductivity                     electr3d.cpp:203-225
//   k_elec_save_junction    saveConductivity                     electr3d.cpp:227-237
//   k_elec_junction_update  junction conductivity update          electr3d.cpp:246-274, beta.hpp:43-46
//   k_elec_coef             c00, c11 in S/um for the operator    electr3d.cpp:310-315
//   k_elec_current          current density and its change       electr3d.cpp:389-424
//   k_elec_heat             Joule heat density                   electr3d.cpp:444-478
//   k_elec_energy_density   integrand of getTotalEnergy          electr3d.cpp:567-599
//   k_elec_volume_sum       getTotalHeat / getTotalEnergy sums   electr3d.cpp:612-624
//   k_elec_plane_current    integrateCurrent                     electr3d.cpp:480-495
//
// Element arrays are padded to the node grid: element (i, j, k) sits at node index
// i + n0 (j + n1 k) of its low corner.  Sums are deterministic (fixed grid, fixed
// reduction order, last block adds the block partials in block order).
#include <cfloat>
#include <cstdint>

#include "elec3d_kernels.h"

namespace plgpu {

namespace {

__device__ __forceinline__ void elem_ijk(long long e, int n0, int n1, int& i, int& j, int& k) {
    i = (int)(e % n0);
    j = (int)((e / n0) % n1);
    k = (int)(e / ((long long)n0 * n1));
}

inline int grid_for(const LaunchCfg& c, long long n) {
    long long b = (n + 255) / 256;
    long long cap = (long long)c.sm_count * 8;
    if (cap > kMaxPartialBlocks) cap = kMaxPartialBlocks;
    return (int)(b < 1 ? 1 : b < cap ? b : cap);
}

struct SumOp {
    __device__ static double apply(double a, double b) { return a + b; }
};
struct MaxOp {
    __device__ static double apply(double a, double b) { return fmax(a, b); }
};

// Reduce NV values over the block (blockDim.x == 256), store them as this block's
// partials (partials[v * kMaxPartialBlocks + block]); the last block to arrive
// combines all partials in block order and writes red[slot + v].
template <int NV, typename Op>
__device__ void block_finish(double (&v)[NV], double* partials, SolveCtl* ctl, int slot) {
    __shared__ double sh[NV][8];
    __shared__ int last;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int q = 0; q < NV; ++q)
        for (int o = 16; o; o >>= 1) v[q] = Op::apply(v[q], __shfl_xor_sync(0xffffffffu, v[q], o));
    if (lane == 0)
#pragma unroll
        for (int q = 0; q < NV; ++q) sh[q][warp] = v[q];
    __syncthreads();
    if (threadIdx.x == 0) {
#pragma unroll
        for (int q = 0; q < NV; ++q) {
            double a = sh[q][0];
            for (int w = 1; w < 8; ++w) a = Op::apply(a, sh[q][w]);
            partials[(size_t)q * kMaxPartialBlocks + blockIdx.x] = a;
        }
        __threadfence();
        const unsigned prev = atomicAdd(&ctl->arrive[3], 1u);
        last = prev == gridDim.x - 1;
        if (last) ctl->arrive[3] = 0u;
    }
    __syncthreads();
    if (last && threadIdx.x == 0) {
        __threadfence();
#pragma unroll
        for (int q = 0; q < NV; ++q) {
            double a = __ldcg(partials + (size_t)q * kMaxPartialBlocks);
            for (unsigned b = 1; b < gridDim.x; ++b)
                a = Op::apply(a, __ldcg(partials + (size_t)q * kMaxPartialBlocks + b));
            ctl->red[slot + q] = a;
        }
    }
}

__device__ __forceinline__ void grad_terms(const GridT<double>& g, const double* __restrict__ V, long long e, int i,
                                           int j, int k, double& sx, double& sy, double& sz) {
    const long long s1 = g.n0, s2 = (long long)g.n0 * g.n1;
    const double lll = V[e], ull = V[e + 1], lul = V[e + s1], uul = V[e + 1 + s1];
    const double llu = V[e + s2], ulu = V[e + 1 + s2], luu = V[e + s1 + s2], uuu = V[e + 1 + s1 + s2];
    sx = (-lll - llu - lul - luu + ull + ulu + uul + uuu) / g.h0[i];
    sy = (-lll - llu + lul + luu - ull - ulu + uul + uuu) / g.h1[j];
    sz = (-lll + llu - lul + luu - ull + ulu - uul + uuu) / g.h2[k];
}

__device__ __forceinline__ bool real_element(int i, int j, int k, int n0, int n1, int n2) {
    return i < n0 - 1 && j < n1 - 1 && k < n2 - 1;
}

}  // namespace

__global__ void __launch_bounds__(256) k_elec_init_cond(int n0, int n1, int n2, const int* __restrict__ mat,
                                                        const int* __restrict__ junc,
                                                        const JunctionInfo* __restrict__ info,
                                                        const double* __restrict__ jsave,
                                                        const double* __restrict__ over,
                                                        const double* __restrict__ cxy, const double* __restrict__ cz,
                                                        const uint8_t* __restrict__ excl, double* __restrict__ sig) {
    const long long N = (long long)n0 * n1 * n2;
    const long long s2 = (long long)n0 * n1;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < N; e += (long long)gridDim.x * blockDim.x) {
        int i, j, k;
        elem_ijk(e, n0, n1, i, j, k);
        double a = 0.0, b = 0.0;
        if (real_element(i, j, k, n0, n1, n2)) {
            const int m = mat[e];
            const int reg = junc[e];
            if (reg > 0) {
                const JunctionInfo J = info[reg - 1];
                const long long src = i + (long long)n0 * j + s2 * ((J.bottom + J.top) / 2);
                a = jsave[2 * src];
                b = jsave[2 * src + 1];
                if (b != b || fabs(b) < 1e-16) b = 1e-16;
            } else if (!excl[m]) {
                if (over && over[2 * e] == over[2 * e]) {
                    a = over[2 * e];
                    b = over[2 * e + 1];
                } else {
                    a = cxy[m];
                    b = cz[m];
                }
            }
        }
        sig[2 * e] = a;
        sig[2 * e + 1] = b;
    }
}

__global__ void __launch_bounds__(256) k_elec_save_junction(int n0, int n1, int n2, const int* __restrict__ junc,
                                                            const JunctionInfo* __restrict__ info,
                                                            const double* __restrict__ sig,
                                                            double* __restrict__ jsave) {
    const long long N = (long long)n0 * n1 * n2;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < N; e += (long long)gridDim.x * blockDim.x) {
        const int reg = junc[e];
        if (reg <= 0) continue;
        int i, j, k;
        elem_ijk(e, n0, n1, i, j, k);
        const JunctionInfo J = info[reg - 1];
        if (k != (J.bottom + J.top) / 2) continue;
        jsave[2 * e] = sig[2 * e];
        jsave[2 * e + 1] = sig[2 * e + 1];
    }
}

__global__ void __launch_bounds__(256) k_elec_fill_pairs(long long N, double* __restrict__ v, double a, double b) {
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < N; e += (long long)gridDim.x * blockDim.x) {
        v[2 * e] = a;
        v[2 * e + 1] = b;
    }
}

// Junction update from the potential V of the previous solve:
//   U  = mean of V over the 4 lateral corners on the top node plane minus the same on the bottom plane
//   jy = 0.1 c11 U / h [kA/cm2];  c11' = 10 |jy| h beta / ln(1e7 |jy| / js + 1), c00' = 0
// "stable" convergence averages the old and new tensors; c11 is floored at 1e-16.
__global__ void __launch_bounds__(256) k_elec_junction_update(int n0, int n1, int n2, const int* __restrict__ junc,
                                                              const JunctionInfo* __restrict__ info,
                                                              const double* __restrict__ bj,
                                                              const double* __restrict__ V, int stable,
                                                              double* __restrict__ sig) {
    const long long N = (long long)n0 * n1 * n2;
    const long long s1 = n0, s2 = (long long)n0 * n1;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < N; e += (long long)gridDim.x * blockDim.x) {
        const int reg = junc[e];
        if (reg <= 0) continue;
        int i, j, k;
        elem_ijk(e, n0, n1, i, j, k);
        const JunctionInfo J = info[reg - 1];
        const long long b0 = i + s1 * j + s2 * J.bottom, t0 = i + s1 * j + s2 * J.top;
        const double U = 0.25 * (-V[b0] - V[b0 + 1] - V[b0 + s1] - V[b0 + 1 + s1] + V[t0] + V[t0 + 1] + V[t0 + s1] +
                                 V[t0 + 1 + s1]);
        double jy = 0.1 * sig[2 * e + 1] * U / J.height;
        jy = fabs(jy);
        double beta = J.beta, js = J.js;
        if (bj && bj[2 * e] == bj[2 * e]) {  // per-element beta(T), js(T)
            beta = bj[2 * e];
            js = bj[2 * e + 1];
        }
        double a = 0.0, b = 10.0 * jy * beta * J.height / log(1e7 * jy / js + 1.0);
        if (stable) {
            a = 0.5 * (sig[2 * e] + a);
            b = 0.5 * (sig[2 * e + 1] + b);
        }
        if (b != b || fabs(b) < 1e-16) b = 1e-16;
        sig[2 * e] = a;
        sig[2 * e + 1] = b;
    }
}

__global__ void __launch_bounds__(256) k_elec_coef(long long N, const double* __restrict__ sig,
                                                   double* __restrict__ k64, float* __restrict__ k32,
                                                   double* __restrict__ kz64, float* __restrict__ kz32) {
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < N; e += (long long)gridDim.x * blockDim.x) {
        const double a = sig[2 * e] * 1e-6, b = sig[2 * e + 1] * 1e-6;  // S/m -> S/um
        k64[e] = a;
        k32[e] = (float)a;
        kz64[e] = b;
        kz32[e] = (float)b;
    }
}

// j = -0.025 c grad-term [kA/cm2] per active element; the change against the stored
// current and |j| at the junction (or everywhere without junctions) are reduced to
// red[0] = max |j - j_old|^2 and red[1] = max |j|^2.
__global__ void __launch_bounds__(256) k_elec_current(const GridT<double> g, const double* __restrict__ V,
                                                      const double* __restrict__ sig, const int* __restrict__ junc,
                                                      const int* __restrict__ mat, const uint8_t* __restrict__ excl,
                                                      int noactive, double* __restrict__ cur,
                                                      double* __restrict__ partials, SolveCtl* __restrict__ ctl) {
    const int n0 = g.n0, n1 = g.n1, n2 = g.n2;
    double v[2] = {0.0, 0.0};
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < g.N; e += (long long)gridDim.x * blockDim.x) {
        int i, j, k;
        elem_ijk(e, n0, n1, i, j, k);
        if (!real_element(i, j, k, n0, n1, n2) || excl[mat[e]]) continue;
        double sx, sy, sz;
        grad_terms(g, V, e, i, j, k, sx, sy, sz);
        const double jx = -0.025 * sig[2 * e] * sx, jyv = -0.025 * sig[2 * e] * sy, jz = -0.025 * sig[2 * e + 1] * sz;
        if (noactive || junc[e] > 0) {
            const double a2 = jx * jx + jyv * jyv + jz * jz;
            if (a2 > v[1]) v[1] = a2;
        }
        const double dx = cur[3 * e] - jx, dy = cur[3 * e + 1] - jyv, dz = cur[3 * e + 2] - jz;
        const double d2 = dx * dx + dy * dy + dz * dz;
        if (d2 > v[0]) v[0] = d2;
        cur[3 * e] = jx;
        cur[3 * e + 1] = jyv;
        cur[3 * e + 2] = jz;
    }
    block_finish<2, MaxOp>(v, partials, ctl, 0);
}

// Joule heat [W/m3]: c00 (dVx^2 + dVy^2) + c11 dVz^2 with dV = -0.25e6 grad-term [V/m];
// zero in excluded elements and in materials marked as not heating.
__global__ void __launch_bounds__(256) k_elec_heat(const GridT<double> g, const double* __restrict__ V,
                                                   const double* __restrict__ sig, const int* __restrict__ mat,
                                                   const uint8_t* __restrict__ excl,
                                                   const uint8_t* __restrict__ noheat, double* __restrict__ out,
                                                   int padded) {
    const int n0 = g.n0, n1 = g.n1, n2 = g.n2;
    const long long NE = (long long)(n0 - 1) * (n1 - 1) * (n2 - 1);
    const long long s1 = n0, s2 = (long long)n0 * n1;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < NE; t += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(t % (n0 - 1)), j = (int)((t / (n0 - 1)) % (n1 - 1)),
                  k = (int)(t / ((long long)(n0 - 1) * (n1 - 1)));
        const long long e = i + s1 * j + s2 * k;
        const int m = mat[e];
        double h = 0.0;
        if (!excl[m] && !noheat[m]) {
            double sx, sy, sz;
            grad_terms(g, V, e, i, j, k, sx, sy, sz);
            const double dvx = -0.25e6 * sx, dvy = -0.25e6 * sy, dvz = -0.25e6 * sz;
            h = sig[2 * e] * dvx * dvx + sig[2 * e] * dvy * dvy + sig[2 * e + 1] * dvz * dvz;
        }
        out[padded ? e : t] = h;
    }
}

__global__ void __launch_bounds__(256) k_elec_energy_density(const GridT<double> g, const double* __restrict__ V,
                                                             const int* __restrict__ mat,
                                                             const uint8_t* __restrict__ excl,
                                                             const double* __restrict__ eps,
                                                             double* __restrict__ out) {
    const int n0 = g.n0, n1 = g.n1, n2 = g.n2;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < g.N; e += (long long)gridDim.x * blockDim.x) {
        int i, j, k;
        elem_ijk(e, n0, n1, i, j, k);
        double w = 0.0;
        if (real_element(i, j, k, n0, n1, n2) && !excl[mat[e]]) {
            double sx, sy, sz;
            grad_terms(g, V, e, i, j, k, sx, sy, sz);
            const double dvx = -0.25e6 * sx, dvy = -0.25e6 * sy, dvz = -0.25e6 * sz;
            w = eps[mat[e]] * (dvx * dvx + dvy * dvy + dvz * dvz);
        }
        out[e] = w;
    }
}

__global__ void __launch_bounds__(256) k_elec_volume_sum(const GridT<double> g, const double* __restrict__ w,
                                                         const int* __restrict__ mat, const uint8_t* __restrict__ excl,
                                                         double* __restrict__ partials, SolveCtl* __restrict__ ctl,
                                                         int slot) {
    const int n0 = g.n0, n1 = g.n1, n2 = g.n2;
    double v[1] = {0.0};
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < g.N; e += (long long)gridDim.x * blockDim.x) {
        int i, j, k;
        elem_ijk(e, n0, n1, i, j, k);
        if (!real_element(i, j, k, n0, n1, n2) || excl[mat[e]]) continue;
        v[0] += g.h0[i] * g.h1[j] * g.h2[k] * w[e];
    }
    block_finish<1, SumOp>(v, partials, ctl, slot);
}

__global__ void __launch_bounds__(256) k_elec_plane_current(const GridT<double> g, const double* __restrict__ cur,
                                                            const int* __restrict__ junc, int level,
                                                            double* __restrict__ partials,
                                                            SolveCtl* __restrict__ ctl, int slot) {
    const int n0 = g.n0, n1 = g.n1;
    const long long M = (long long)(n0 - 1) * (n1 - 1);
    const long long s2 = (long long)n0 * n1;
    double v[1] = {0.0};
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < M; t += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(t % (n0 - 1)), j = (int)(t / (n0 - 1));
        const long long e = i + (long long)n0 * j + s2 * level;
        if (junc[e] > 0) v[0] += cur[3 * e + 2] * g.h0[i] * g.h1[j];
    }
    block_finish<1, SumOp>(v, partials, ctl, slot);
}

// dst = src (comps per padded element) with NaN in excluded elements
__global__ void __launch_bounds__(256) k_elec_masked_copy(int n0, int n1, int n2, int comps,
                                                          const double* __restrict__ src, const int* __restrict__ mat,
                                                          const uint8_t* __restrict__ excl, double* __restrict__ dst) {
    const long long N = (long long)n0 * n1 * n2;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < N; e += (long long)gridDim.x * blockDim.x) {
        int i, j, k;
        elem_ijk(e, n0, n1, i, j, k);
        const bool nan = real_element(i, j, k, n0, n1, n2) && excl[mat[e]];
        for (int c = 0; c < comps; ++c)
            dst[e * comps + c] = nan ? __longlong_as_double(0x7ff8000000000000LL) : src[e * comps + c];
    }
}

// mean of the 8 corner values of every element (the value trilinear interpolation
// gives at the element midpoint), padded layout
__global__ void __launch_bounds__(256) k_elem_average(int n0, int n1, int n2, const double* __restrict__ T,
                                                      double* __restrict__ out) {
    const long long N = (long long)n0 * n1 * n2;
    const long long s1 = n0, s2 = (long long)n0 * n1;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < N; e += (long long)gridDim.x * blockDim.x) {
        int i, j, k;
        elem_ijk(e, n0, n1, i, j, k);
        double t = 0.0;
        if (real_element(i, j, k, n0, n1, n2)) {
            t += T[e];
            t += T[e + 1];
            t += T[e + s1];
            t += T[e + 1 + s1];
            t += T[e + s2];
            t += T[e + 1 + s2];
            t += T[e + s1 + s2];
            t += T[e + 1 + s1 + s2];
            t *= 0.125;
        }
        out[e] = t;
    }
}

// ----------------------------------------------------------------------------------------
// launchers

void launch_elec_init_cond(const LaunchCfg& c, int n0, int n1, int n2, const int* mat, const int* junc,
                           const JunctionInfo* info, const double* jsave, const double* over, const double* cxy,
                           const double* cz, const uint8_t* excl, double* sig) {
    launch_kernel(k_elec_init_cond, grid_for(c, (long long)n0 * n1 * n2), 256, c.stream, n0, n1, n2, mat, junc, info,
                  jsave, over, cxy, cz, excl, sig);
}
void launch_elec_save_junction(const LaunchCfg& c, int n0, int n1, int n2, const int* junc, const JunctionInfo* info,
                               const double* sig, double* jsave) {
    launch_kernel(k_elec_save_junction, grid_for(c, (long long)n0 * n1 * n2), 256, c.stream, n0, n1, n2, junc, info,
                  sig, jsave);
}
void launch_elec_fill_pairs(const LaunchCfg& c, long long N, double* v, double a, double b) {
    launch_kernel(k_elec_fill_pairs, grid_for(c, N), 256, c.stream, N, v, a, b);
}
void launch_elec_junction_update(const LaunchCfg& c, int n0, int n1, int n2, const int* junc, const JunctionInfo* info,
                                 const double* bj, const double* V, int stable, double* sig) {
    launch_kernel(k_elec_junction_update, grid_for(c, (long long)n0 * n1 * n2), 256, c.stream, n0, n1, n2, junc, info,
                  bj, V, stable, sig);
}
void launch_elec_coef(const LaunchCfg& c, long long N, const double* sig, double* k64, float* k32, double* kz64,
                      float* kz32) {
    launch_kernel(k_elec_coef, grid_for(c, N), 256, c.stream, N, sig, k64, k32, kz64, kz32);
}
void launch_elec_current(const LaunchCfg& c, const GridT<double>& g, const double* V, const double* sig,
                         const int* junc, const int* mat, const uint8_t* excl, int noactive, double* cur,
                         double* partials, SolveCtl* ctl) {
    launch_kernel(k_elec_current, grid_for(c, g.N), 256, c.stream, g, V, sig, junc, mat, excl, noactive, cur, partials,
                  ctl);
}
void launch_elec_heat(const LaunchCfg& c, const GridT<double>& g, const double* V, const double* sig, const int* mat,
                      const uint8_t* excl, const uint8_t* noheat, double* out, int padded) {
    const long long NE = (long long)(g.n0 - 1) * (g.n1 - 1) * (g.n2 - 1);
    launch_kernel(k_elec_heat, grid_for(c, NE), 256, c.stream, g, V, sig, mat, excl, noheat, out, padded);
}
void launch_elec_energy_density(const LaunchCfg& c, const GridT<double>& g, const double* V, const int* mat,
                                const uint8_t* excl, const double* eps, double* out) {
    launch_kernel(k_elec_energy_density, grid_for(c, g.N), 256, c.stream, g, V, mat, excl, eps, out);
}
void launch_elec_volume_sum(const LaunchCfg& c, const GridT<double>& g, const double* w, const int* mat,
                            const uint8_t* excl, double* partials, SolveCtl* ctl, int slot) {
    launch_kernel(k_elec_volume_sum, grid_for(c, g.N), 256, c.stream, g, w, mat, excl, partials, ctl, slot);
}
void launch_elec_plane_current(const LaunchCfg& c, const GridT<double>& g, const double* cur, const int* junc,
                               int level, double* partials, SolveCtl* ctl, int slot) {
    const long long M = (long long)(g.n0 - 1) * (g.n1 - 1);
    launch_kernel(k_elec_plane_current, grid_for(c, M), 256, c.stream, g, cur, junc, level, partials, ctl, slot);
}

void launch_elec_masked_copy(const LaunchCfg& c, int n0, int n1, int n2, int comps, const double* src, const int* mat,
                             const uint8_t* excl, double* dst) {
    launch_kernel(k_elec_masked_copy, grid_for(c, (long long)n0 * n1 * n2), 256, c.stream, n0, n1, n2, comps, src, mat,
                  excl, dst);
}
void launch_elem_average(const LaunchCfg& c, int n0, int n1, int n2, const double* T, double* out) {
    launch_kernel(k_elem_average, grid_for(c, (long long)n0 * n1 * n2), 256, c.stream, n0, n1, n2, T, out);
}

}  // namespace plgpu
