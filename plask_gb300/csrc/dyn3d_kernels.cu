// Kernels of the time-stepping thermal solver (PLaSK solvers/thermal/dynamic/femT3d.cpp):
// the system matrix is theta K + C with the heat capacity C, applied by the stencil
// kernel (the lumped C as a diagonal shift, the consistent C through per-element corner
// capacities), so only the capacity, the coefficient scaling and the right-hand side
// X = B T + F = C T - (1 - theta) K T + F live here.
//
//   k_lumped_mass   c = cp dens 0.125e-9 dx dy dz / timestep per element corner,
//                   summed onto the nodes (times a weight)    femT3d.cpp:183, 203-210
//   k_elem_capacity c per element for the consistent matrix    femT3d.cpp:183, 211-226
//   k_dyn_rhs       X = B T + F                                femT3d.cpp:292-293
#include <cstdint>

#include "fem3d_kernels.h"

namespace plgpu {

namespace {
inline int grid_for(const LaunchCfg& c, long long n) {
    long long b = (n + 255) / 256;
    const long long cap = (long long)c.sm_count * 8;
    return (int)(b < 1 ? 1 : b < cap ? b : cap);
}
}  // namespace

__global__ void __launch_bounds__(256) k_lumped_mass(const GridT<double> g, const int* __restrict__ mat,
                                                     const uint8_t* __restrict__ excl, const double* __restrict__ cp,
                                                     const double* __restrict__ dens, double timestep, double weight,
                                                     double* __restrict__ c64, float* __restrict__ c32) {
    const int n0 = g.n0, n1 = g.n1, n2 = g.n2;
    const long long s1 = n0, s2 = (long long)n0 * n1;
    for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < g.N; n += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(n % n0), j = (int)((n / n0) % n1), k = (int)(n / s2);
        double c = 0.0;
        for (int cc = 0; cc < 8; ++cc) {  // the (up to 8) elements around the node, fixed order
            const int ei = i - 1 + (cc & 1), ej = j - 1 + ((cc >> 1) & 1), ek = k - 1 + (cc >> 2);
            if (ei < 0 || ej < 0 || ek < 0 || ei >= n0 - 1 || ej >= n1 - 1 || ek >= n2 - 1) continue;
            const long long e = ei + s1 * ej + s2 * ek;
            const int m = mat[e];
            if (excl[m]) continue;
            c += cp[m] * dens[m] * 0.125e-9 * g.h0[ei] * g.h1[ej] * g.h2[ek] / timestep;
        }
        c64[n] = weight * c;
        if (c32) c32[n] = (float)(weight * c);
    }
}

// Corner capacity c of every element (padded layout, 0 for padding and excluded
// elements): the consistent matrix of an element is c (8, 4, 2, 1) / 27 by corner
// distance, c (M (x) M (x) M) with M = [[2,1],[1,2]] / 3.  cneg = -c for the right-hand
// side product.
__global__ void __launch_bounds__(256) k_elem_capacity(const GridT<double> g, const int* __restrict__ mat,
                                                       const uint8_t* __restrict__ excl, const double* __restrict__ cp,
                                                       const double* __restrict__ dens, double timestep,
                                                       double* __restrict__ c64, float* __restrict__ c32,
                                                       double* __restrict__ cneg) {
    const int n0 = g.n0, n1 = g.n1, n2 = g.n2;
    const long long s2 = (long long)n0 * n1;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < g.N; e += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(e % n0), j = (int)((e / n0) % n1), k = (int)(e / s2);
        double c = 0.0;
        if (i < n0 - 1 && j < n1 - 1 && k < n2 - 1) {
            const int m = mat[e];
            if (!excl[m]) c = cp[m] * dens[m] * 0.125e-9 * g.h0[i] * g.h1[j] * g.h2[k] / timestep;
        }
        c64[e] = c;
        c32[e] = (float)c;
        cneg[e] = -c;
    }
}

__global__ void __launch_bounds__(256) k_scale4(long long N, double s, double* __restrict__ a64, float* __restrict__ a32,
                                                double* __restrict__ b64, float* __restrict__ b32) {
    for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < N; n += (long long)gridDim.x * blockDim.x) {
        if (a64) a64[n] *= s;
        if (a32) a32[n] = (float)((double)a32[n] * s);
        if (b64) b64[n] *= s;
        if (b32) b32[n] = (float)((double)b32[n] * s);
    }
}

__global__ void __launch_bounds__(256) k_dyn_rhs(long long N, const double* __restrict__ cap,
                                                 const double* __restrict__ T, const double* __restrict__ Y, double w,
                                                 const double* __restrict__ F, double* __restrict__ X) {
    for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < N; n += (long long)gridDim.x * blockDim.x)
        X[n] = cap[n] * T[n] + w * Y[n] + F[n];
}

void launch_lumped_mass(const LaunchCfg& c, const GridT<double>& g, const int* mat, const uint8_t* excl,
                        const double* cp, const double* dens, double timestep, double* c64, float* c32,
                        double weight) {
    launch_kernel(k_lumped_mass, grid_for(c, g.N), 256, c.stream, g, mat, excl, cp, dens, timestep, weight, c64, c32);
}
void launch_elem_capacity(const LaunchCfg& c, const GridT<double>& g, const int* mat, const uint8_t* excl,
                          const double* cp, const double* dens, double timestep, double* c64, float* c32,
                          double* cneg) {
    launch_kernel(k_elem_capacity, grid_for(c, g.N), 256, c.stream, g, mat, excl, cp, dens, timestep, c64, c32, cneg);
}
void launch_scale4(const LaunchCfg& c, long long N, double s, double* a64, float* a32, double* b64, float* b32) {
    launch_kernel(k_scale4, grid_for(c, N), 256, c.stream, N, s, a64, a32, b64, b32);
}
void launch_dyn_rhs(const LaunchCfg& c, long long N, const double* cap, const double* T, const double* Y, double w,
                    const double* F, double* X) {
    launch_kernel(k_dyn_rhs, grid_for(c, N), 256, c.stream, N, cap, T, Y, w, F, X);
}
}  // namespace plgpu
