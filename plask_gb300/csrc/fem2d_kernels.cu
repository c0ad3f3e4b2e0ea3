// Static2D / StaticCyl thermal FEM kernels for sm_103a (bilinear quads on a
// rectilinear 2D mesh).
//
// What each kernel replaces in PLaSK (paths relative to the PLaSK tree):
//   k_thickness2d   ThermalFem2DSolver::onInitialize layer-run thickness   solvers/thermal/static/therm2d.cpp:81-114
//   k_coef2d        per-element k(T) of setMatrix                            therm2d.cpp:210-217, 336-343
//   k_apply2d       the assembled stiffness matrix times a vector, matrix-free: K_e of
//                   therm2d.cpp:222-228, 268-285 (Cartesian) and r K_e of :348-354, 409-426
//                   (cylindrical), Dirichlet rows as after BandMatrix::setBC
//                   (plask/common/fem/matrix.hpp:132-145)
//   k_heat_load2d   element load f = 0.25e-12 w h q (x r)                    therm2d.cpp:220, 346
//   k_flux2d        saveHeatFluxes                                            therm2d.cpp:505-541
//   k_conductivity2d ThermalConductivityData::at                              therm2d.cpp:574-597
//
// The element stiffness with X = kx h / w and Y = ky w / h (times the midpoint radius
// r in the cylindrical form) is
//     K_e = X (A (x) M) + Y (M (x) A),  A = [[1,-1],[-1,1]],  M = [[2,1],[1,2]] / 6,
// i.e. diagonal (X+Y)/3, x-neighbour (Y-2X)/6, y-neighbour (X-2Y)/6, opposite corner
// -(X+Y)/6.  A node's row gathers the four elements around it; 2D meshes are small
// enough (10^4..10^6 nodes) that one thread per node with its 3 x 3 neighbourhood read
// through L1 is the whole design.
#include <algorithm>
#include <cfloat>
#include <cstdint>

#include "fem2d_kernels.h"
#include "fem3d_reduce.cuh"

namespace plgpu {

namespace {

__device__ __forceinline__ bool bit_set(const uint32_t* __restrict__ m, long long n) {
    return (__ldg(m + (n >> 5)) >> (n & 31)) & 1u;
}

template <typename R>
struct Op2dArgs {
    GridT<R> g;
    const R* rmid;  // cylindrical: midpoint radius per element column, else nullptr
    const R* x;
    R* y;
    const R* kx;
    const R* ky;  // nullptr: isotropic (ky = kx)
    const uint32_t* dmask;
    const R* rhs;
    double* partials;
    SolveCtl* ctl;
    const uint32_t* smask;
    int sslots;
    const R* dshift;  // lumped heat capacity per node (time steps), or nullptr
    const R* cmass;   // consistent heat capacity: corner capacity c per element, or nullptr
};

// X and Y of element (ie, je); zero outside the mesh (padding slots hold zero k)
template <typename R>
__device__ __forceinline__ void element_xy(const Op2dArgs<R>& a, int ie, int je, R& X, R& Y) {
    X = Y = R(0);
    if (ie < 0 || je < 0 || ie >= a.g.n0 - 1 || je >= a.g.n1 - 1) return;
    const long long e = ie + (long long)a.g.n0 * je;
    const R kx = a.kx[e];
    const R ky = a.ky ? a.ky[e] : kx;
    const R w = a.g.h0[ie], h = a.g.h1[je];
    X = kx * h * a.g.r0[ie];
    Y = ky * w * a.g.r1[je];
    if (a.rmid) {
        const R r = a.rmid[ie];
        X *= r;
        Y *= r;
    }
}

// CAP: 0 none, 1 the lumped capacity a.dshift on the diagonal, 2 the consistent capacity
// c (M (x) M), M = [[2,1],[1,2]] / 3, of every element (corner weights 4/9, 2/9, 1/9)
template <typename R, int MODE, int CAP>
__global__ void __launch_bounds__(256) k_apply2d(const Op2dArgs<R> a) {
    if (MODE == MODE_CG && a.ctl->status != SOLVE_RUNNING) return;
    const int n0 = a.g.n0, n1 = a.g.n1;
    const long long N = a.g.N;
    constexpr bool kMask = MODE == MODE_RESID || MODE == MODE_MULT;
    double dot = 0.0;
    for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < N; n += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(n % n0), j = (int)(n / n0);
        // 3 x 3 neighbourhood, xv[dj + 1][di + 1]; zero outside the mesh (and on Dirichlet
        // nodes in the masked modes)
        R xv[3][3];
#pragma unroll
        for (int dj = -1; dj <= 1; ++dj)
#pragma unroll
            for (int di = -1; di <= 1; ++di) {
                const int ii = i + di, jj = j + dj;
                R v = R(0);
                if (ii >= 0 && ii < n0 && jj >= 0 && jj < n1) {
                    const long long m = ii + (long long)n0 * jj;
                    v = a.x[m];
                    if (kMask && bit_set(a.dmask, m)) v = R(0);
                }
                xv[dj + 1][di + 1] = v;
            }
        const R x0 = xv[1][1];
        R acc = R(0);
        // the four elements: node at corner (ca, cb) of element (i - ca, j - cb)
#pragma unroll
        for (int cb = 0; cb <= 1; ++cb)
#pragma unroll
            for (int ca = 0; ca <= 1; ++ca) {
                R X, Y;
                element_xy(a, i - ca, j - cb, X, Y);
                const int sx = ca ? -1 : 1, sy = cb ? -1 : 1;  // direction of the element's other corners
                const R xn = xv[1][1 + sx], yn = xv[1 + sy][1], dn = xv[1 + sy][1 + sx];
                // X/6 (2 (x0 - xn) + (yn - dn)) + Y/6 (2 (x0 - yn) + (xn - dn))
                acc += (X * (R(2) * (x0 - xn) + (yn - dn)) + Y * (R(2) * (x0 - yn) + (xn - dn))) * R(1.0 / 6.0);
                if constexpr (CAP == 2) {
                    const int ie = i - ca, je = j - cb;
                    if (ie >= 0 && je >= 0 && ie < n0 - 1 && je < n1 - 1) {
                        const R c = a.cmass[ie + (long long)n0 * je];
                        acc += c * (R(4.0 / 9.0) * x0 + R(2.0 / 9.0) * (xn + yn) + R(1.0 / 9.0) * dn);
                    }
                }
            }
        if constexpr (CAP == 1) acc += a.dshift[n] * x0;
        R out;
        if (MODE == MODE_CG) {
            out = acc;
            dot += (double)x0 * (double)out;
            if (a.smask != nullptr && bit_set(a.smask, n)) out += a.y[n];
        } else if (MODE == MODE_RESID) {
            out = bit_set(a.dmask, n) ? R(a.rhs[n] - a.x[n]) : R(a.rhs[n] - acc);
        } else if (MODE == MODE_MULT) {
            out = bit_set(a.dmask, n) ? a.x[n] : acc;
        } else {
            out = a.rhs[n] - acc;
        }
        a.y[n] = out;
    }
    if (MODE == MODE_CG) {
        double v[1] = {dot};
        write_partial<1, OpSum>(v, a.partials, blockIdx.x);
        if (arrive_last(&a.ctl->arrive[0], gridDim.x)) {
            reduce_partials<1, OpSum>(v, a.partials, gridDim.x + a.sslots);
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

// Layer-run thickness: for every element, the height of the maximal run of elements
// with the same material along axis 1 in its column.
__global__ void k_thickness2d(int n0, int n1, const int* __restrict__ mat, const double* __restrict__ y,
                              double* __restrict__ th) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n0 - 1) return;
    int start = 0;
    for (int j = 1; j <= n1 - 1; ++j) {
        const bool brk = (j == n1 - 1) || (mat[i + (long long)n0 * j] != mat[i + (long long)n0 * (j - 1)]);
        if (brk) {
            const double h = y[j] - y[start];
            for (int q = start; q < j; ++q) th[i + (long long)n0 * q] = h;
            start = j;
        }
    }
}

__device__ __forceinline__ double quad_mean(const double* __restrict__ T, long long e, int n0) {
    // 0.25 (T_lolo + T_uplo + T_loup + T_upup), therm2d.cpp:210, 336
    return 0.25 * (T[e] + T[e + 1] + T[e + n0] + T[e + 1 + n0]);
}

template <bool ANISO>
__global__ void __launch_bounds__(256) k_coef2d(int n0, int n1, const double* __restrict__ T,
                                                const int* __restrict__ mat, const double* __restrict__ th,
                                                const MatTable tab, double* __restrict__ k64, float* __restrict__ k32,
                                                double* __restrict__ ky64, float* __restrict__ ky32) {
    const long long N = (long long)n0 * n1;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < N; e += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(e % n0), j = (int)(e / n0);
        double kx = 0.0, ky = 0.0;
        if (i < n0 - 1 && j < n1 - 1) {
            const int m = mat[e];
            if (!tab.excluded[m]) {
                const double t = quad_mean(T, e, n0);
                mat_thermk(tab, m, t, th[e], kx, ky);
            }
        }
        k64[e] = kx;
        k32[e] = (float)kx;
        if (ANISO) {
            ky64[e] = ky;
            ky32[e] = (float)ky;
        }
    }
}

__global__ void __launch_bounds__(256) k_diag2d(const GridT<double> g, const double* __restrict__ rmid,
                                                const double* __restrict__ kx, const double* __restrict__ ky,
                                                const double* __restrict__ shift, double* __restrict__ diag) {
    const int n0 = g.n0, n1 = g.n1;
    for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < g.N; n += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(n % n0), j = (int)(n / n0);
        double d = 0.0;
        for (int c = 0; c < 4; ++c) {
            const int ie = i - (c & 1), je = j - (c >> 1);
            if (ie < 0 || je < 0 || ie >= n0 - 1 || je >= n1 - 1) continue;
            const long long e = ie + (long long)n0 * je;
            const double k1 = kx[e], k2 = ky ? ky[e] : k1;
            double X = k1 * g.h1[je] * g.r0[ie], Y = k2 * g.h0[ie] * g.r1[je];
            if (rmid) {
                X *= rmid[ie];
                Y *= rmid[ie];
            }
            d += (X + Y) * (1.0 / 3.0);
        }
        diag[n] = shift ? d + shift[n] : d;
    }
}

__global__ void __launch_bounds__(256) k_heat_load2d(const GridT<double> g, const double* __restrict__ rmid,
                                                     const double* __restrict__ q, const int* __restrict__ mat,
                                                     const MatTable tab, double* __restrict__ F) {
    const int n0 = g.n0, n1 = g.n1;
    for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < g.N; n += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(n % n0), j = (int)(n / n0);
        double f = 0.0;
        for (int c = 0; c < 4; ++c) {
            const int ie = i - (c & 1), je = j - (c >> 1);
            if (ie < 0 || je < 0 || ie >= n0 - 1 || je >= n1 - 1) continue;
            const long long e = ie + (long long)n0 * je;
            if (tab.excluded[mat[e]]) continue;
            double v = 0.25e-12 * g.h0[ie] * g.h1[je] * q[e];
            if (rmid) v = 0.25e-12 * rmid[ie] * g.h0[ie] * g.h1[je] * q[e];
            f += v;
        }
        F[n] = f;
    }
}

// Heat capacity of the time-stepping solvers (femT2d.cpp:167, 298): per element corner
// c = cp dens 0.25e-3 w h / timestep (times the midpoint radius in the cylindrical form).
__device__ __forceinline__ double corner_capacity(const GridT<double>& g, const double* rmid, int ie, int je, int m,
                                                  const double* cp, const double* dens, double timestep) {
    if (rmid)
        return cp[m] * dens[m] * 0.25 * 1e-12 * rmid[ie] * g.h1[je] * g.h0[ie] / timestep / 1e-9;
    return cp[m] * dens[m] * 0.25 * 1e-12 * g.h1[je] * g.h0[ie] / timestep / 1e-9;
}

// lumped capacity per node: weight times the sum of c over the node's active elements
__global__ void __launch_bounds__(256) k_lumped_mass2d(const GridT<double> g, const double* __restrict__ rmid,
                                                       const int* __restrict__ mat, const uint8_t* __restrict__ excl,
                                                       const double* __restrict__ cp, const double* __restrict__ dens,
                                                       double timestep, double weight, double* __restrict__ c64,
                                                       float* __restrict__ c32) {
    const int n0 = g.n0, n1 = g.n1;
    for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < g.N; n += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(n % n0), j = (int)(n / n0);
        double c = 0.0;
        for (int k = 0; k < 4; ++k) {  // the (up to 4) elements around the node, fixed order
            const int ie = i - 1 + (k & 1), je = j - 1 + (k >> 1);
            if (ie < 0 || je < 0 || ie >= n0 - 1 || je >= n1 - 1) continue;
            const int m = mat[ie + (long long)n0 * je];
            if (excl[m]) continue;
            c += corner_capacity(g, rmid, ie, je, m, cp, dens, timestep);
        }
        c64[n] = weight * c;
        if (c32) c32[n] = (float)(weight * c);
    }
}

// corner capacity per element (padded layout; 0 for padding and excluded elements), and -c
__global__ void __launch_bounds__(256) k_elem_capacity2d(const GridT<double> g, const double* __restrict__ rmid,
                                                         const int* __restrict__ mat,
                                                         const uint8_t* __restrict__ excl,
                                                         const double* __restrict__ cp,
                                                         const double* __restrict__ dens, double timestep,
                                                         double* __restrict__ c64, float* __restrict__ c32,
                                                         double* __restrict__ cneg) {
    const int n0 = g.n0, n1 = g.n1;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < g.N; e += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(e % n0), j = (int)(e / n0);
        double c = 0.0;
        if (i < n0 - 1 && j < n1 - 1) {
            const int m = mat[e];
            if (!excl[m]) c = corner_capacity(g, rmid, i, j, m, cp, dens, timestep);
        }
        c64[e] = c;
        c32[e] = (float)c;
        cneg[e] = -c;
    }
}

__global__ void __launch_bounds__(256) k_flux2d(const GridT<double> g, const double* __restrict__ T,
                                                const int* __restrict__ mat, const double* __restrict__ hleaf,
                                                const MatTable tab, double* __restrict__ out) {
    const int n0 = g.n0, n1 = g.n1;
    const long long NE = (long long)(n0 - 1) * (n1 - 1);
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < NE; t += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(t % (n0 - 1)), j = (int)(t / (n0 - 1));
        const long long e = i + (long long)n0 * j;
        const int m = mat[e];
        if (tab.excluded[m]) {
            out[2 * t] = out[2 * t + 1] = __longlong_as_double(0x7ff8000000000000LL);
            continue;
        }
        const double ll = T[e], lr = T[e + 1], ul = T[e + n0], ur = T[e + 1 + n0];
        const double temp = 0.25 * (ll + lr + ul + ur);
        double kx, ky;
        mat_thermk(tab, m, temp, hleaf[e], kx, ky);
        out[2 * t] = -0.5e6 * kx * (-ll + lr - ul + ur) / g.h0[i];
        out[2 * t + 1] = -0.5e6 * ky * (-ll - lr + ul + ur) / g.h1[j];
    }
}

__global__ void __launch_bounds__(256) k_conductivity2d(int n0, int n1, const double* __restrict__ T,
                                                        const int* __restrict__ mat, const double* __restrict__ th,
                                                        const MatTable tab, double* __restrict__ out) {
    const long long NE = (long long)(n0 - 1) * (n1 - 1);
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < NE; t += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(t % (n0 - 1)), j = (int)(t / (n0 - 1));
        const long long e = i + (long long)n0 * j;
        const int m = mat[e];
        if (tab.excluded[m]) {
            out[2 * t] = out[2 * t + 1] = __longlong_as_double(0x7ff8000000000000LL);
            continue;
        }
        const double temp = quad_mean(T, e, n0);
        double kk, kv;
        mat_thermk(tab, m, temp, th[e], kk, kv);
        out[2 * t] = kk;
        out[2 * t + 1] = kv;
    }
}

int grid_cap(long long n, int threads, int cap) {
    long long b = (n + threads - 1) / threads;
    if (b < 1) b = 1;
    return (int)(b < cap ? b : cap);
}

template <typename R, int CAP>
void operator2d_cap(const LaunchCfg& c, const Op2dArgs<R>& a, int mode) {
    const int blocks = op2d_blocks(c, a.g.N);
    switch (mode) {
        case MODE_CG: launch_kernel(k_apply2d<R, MODE_CG, CAP>, blocks, 256, c.stream, a); break;
        case MODE_RESID: launch_kernel(k_apply2d<R, MODE_RESID, CAP>, blocks, 256, c.stream, a); break;
        case MODE_RHS: launch_kernel(k_apply2d<R, MODE_RHS, CAP>, blocks, 256, c.stream, a); break;
        default: launch_kernel(k_apply2d<R, MODE_MULT, CAP>, blocks, 256, c.stream, a); break;
    }
}

template <typename R>
void operator2d_any(const LaunchCfg& c, const GridT<R>& g, const R* rmid, const R* x, R* y, const R* kx, const R* ky,
                    const uint32_t* dmask, const R* rhs, double* partials, int mode, SolveCtl* ctl,
                    const uint32_t* smask, int sslots, const R* dshift, const R* cmass) {
    const Op2dArgs<R> a{g, rmid, x, y, kx, ky, dmask, rhs, partials, ctl, smask, sslots, dshift, cmass};
    if (cmass)
        operator2d_cap<R, 2>(c, a, mode);
    else if (dshift)
        operator2d_cap<R, 1>(c, a, mode);
    else
        operator2d_cap<R, 0>(c, a, mode);
}

}  // namespace

// One wave of 8 blocks per SM at most, and room for the surface kernel's partial slots.
int op2d_blocks(const LaunchCfg& c, long long N) {
    return grid_cap(N, 256, std::min(c.sm_count * 8, kMaxPartialBlocks - 512));
}

void launch_operator2d(const LaunchCfg& c, const GridT<double>& g, const double* rmid, const double* x, double* y,
                       const double* kx, const double* ky, const uint32_t* dmask, const double* rhs,
                       double* partials, int mode, SolveCtl* ctl, const uint32_t* smask, int sslots,
                       const double* dshift, const double* cmass) {
    operator2d_any<double>(c, g, rmid, x, y, kx, ky, dmask, rhs, partials, mode, ctl, smask, sslots, dshift, cmass);
}
void launch_operator2d(const LaunchCfg& c, const GridT<float>& g, const float* rmid, const float* x, float* y,
                       const float* kx, const float* ky, const uint32_t* dmask, const float* rhs, double* partials,
                       int mode, SolveCtl* ctl, const uint32_t* smask, int sslots, const float* dshift,
                       const float* cmass) {
    operator2d_any<float>(c, g, rmid, x, y, kx, ky, dmask, rhs, partials, mode, ctl, smask, sslots, dshift, cmass);
}

void launch_thickness2d(const LaunchCfg& c, int n0, int n1, const int* mat, const double* y, double* th) {
    launch_kernel(k_thickness2d, grid_cap(n0, 128, 1 << 20), 128, c.stream, n0, n1, mat, y, th);
}

void launch_coef2d(const LaunchCfg& c, int n0, int n1, const double* T, const int* mat, const double* th,
                   const MatTable& tab, double* k64, float* k32, double* ky64, float* ky32, bool aniso) {
    const long long N = (long long)n0 * n1;
    if (aniso)
        launch_kernel(k_coef2d<true>, vec_blocks(c, N), 256, c.stream, n0, n1, T, mat, th, tab, k64, k32, ky64, ky32);
    else
        launch_kernel(k_coef2d<false>, vec_blocks(c, N), 256, c.stream, n0, n1, T, mat, th, tab, k64, k32, ky64, ky32);
}

void launch_diag2d(const LaunchCfg& c, const GridT<double>& g, const double* rmid, const double* kx,
                   const double* ky, double* diag, const double* shift) {
    launch_kernel(k_diag2d, vec_blocks(c, g.N), 256, c.stream, g, rmid, kx, ky, shift, diag);
}
void launch_lumped_mass2d(const LaunchCfg& c, const GridT<double>& g, const double* rmid, const int* mat,
                          const uint8_t* excl, const double* cp, const double* dens, double timestep, double* c64,
                          float* c32, double weight) {
    launch_kernel(k_lumped_mass2d, vec_blocks(c, g.N), 256, c.stream, g, rmid, mat, excl, cp, dens, timestep, weight,
                  c64, c32);
}
void launch_elem_capacity2d(const LaunchCfg& c, const GridT<double>& g, const double* rmid, const int* mat,
                            const uint8_t* excl, const double* cp, const double* dens, double timestep, double* c64,
                            float* c32, double* cneg) {
    launch_kernel(k_elem_capacity2d, vec_blocks(c, g.N), 256, c.stream, g, rmid, mat, excl, cp, dens, timestep, c64,
                  c32, cneg);
}

void launch_heat_load2d(const LaunchCfg& c, const GridT<double>& g, const double* rmid, const double* q,
                        const int* mat, const MatTable& tab, double* F) {
    launch_kernel(k_heat_load2d, vec_blocks(c, g.N), 256, c.stream, g, rmid, q, mat, tab, F);
}

void launch_flux2d(const LaunchCfg& c, const GridT<double>& g, const double* T, const int* mat, const double* hleaf,
                   const MatTable& tab, double* out) {
    const long long NE = (long long)(g.n0 - 1) * (g.n1 - 1);
    launch_kernel(k_flux2d, vec_blocks(c, NE), 256, c.stream, g, T, mat, hleaf, tab, out);
}

void launch_conductivity2d(const LaunchCfg& c, int n0, int n1, const double* T, const int* mat, const double* th,
                           const MatTable& tab, double* out) {
    const long long NE = (long long)(n0 - 1) * (n1 - 1);
    launch_kernel(k_conductivity2d, vec_blocks(c, NE), 256, c.stream, n0, n1, T, mat, th, tab, out);
}

}  // namespace plgpu
