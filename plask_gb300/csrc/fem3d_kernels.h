// Host-callable launchers of the Static3D kernels (fem3d_kernels.cu).
#pragma once

#include <cstdint>
#include <vector>

#include <cuda_runtime.h>

#include "fem3d_device.cuh"

namespace plgpu {

// MODE_CG:    y = A x, Dirichlet rows y = x (x is zero on Dirichlet nodes in CG)
// MODE_RESID: y = rhs - A x, x masked to zero on Dirichlet nodes, Dirichlet rows y = rhs - x
// MODE_RHS:   y = rhs - A x with the full operator (Dirichlet rows fixed up afterwards)
// MODE_MULT:  y = A x, x masked to zero on Dirichlet nodes, Dirichlet rows y = x
enum { MODE_CG = 0, MODE_RESID = 1, MODE_RHS = 2, MODE_MULT = 3 };

void count_launch();
void count_launches(long long n);  // kernels run by a replayed CUDA graph

// Launch a kernel on a stream and count it.
template <typename... KArgs, typename... Args>
inline void launch_kernel(void (*kern)(KArgs...), dim3 grid, dim3 block, cudaStream_t stream, Args... args) {
    kern<<<grid, block, 0, stream>>>(args...);
    count_launch();
}

// Programmatic dependent launch of the kernels of the fused CG iteration: a kernel
// launched this way may be scheduled while the previous kernel of the stream drains; it
// calls pdl_wait() (fem3d_device.cuh) before it reads anything the previous kernels
// wrote.  Off when the environment sets PLGPU_NO_PDL.
bool pdl_enabled();
template <typename... KArgs, typename... Args>
inline void launch_kernel_pdl(void (*kern)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t stream,
                              Args... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = pdl_enabled() ? 1 : 0;
    cudaLaunchKernelEx(&cfg, kern, static_cast<KArgs>(args)...);  // errors surface in cudaGetLastError
    count_launch();
}

// Material table in device memory (one entry per material id).
struct MatTable {
    const double* k300;
    const double* p;
    const double* kz_ratio;
    const double* hexp;
    const uint8_t* excluded;  // element of this material is dropped from the system
    // tabulated k(T) (plgpu_fem3d_set_material_table): for material m with tab_off[m] >= 0,
    // tab_n[m] points (tab_T, tab_kxy, tab_kz)[tab_off[m] ...] replace k300 (300/T)^p and kz_ratio;
    // tab_off == nullptr when no material has a table
    const int* tab_off;
    const int* tab_n;
    const double* tab_T;
    const double* tab_kxy;
    const double* tab_kz;
};

#ifdef __CUDACC__
// k_xy, k_z [W/(m K)] of material m at temperature T and layer-run thickness h, as the
// reference's Material::thermk(T, h) (plask/material/material.hpp:691) for the materials
// this solver models: the power law k300 (300/T)^p, k_z = kz_ratio k_xy, or the material's
// table, piecewise linear in T between its points and constant beyond the first and the
// last (a monotone interpolation: it never leaves the range of two neighbouring points);
// either times h^hexp when hexp != 0.
__device__ __forceinline__ void mat_thermk(const MatTable& tab, int m, double T, double h, double& kxy,
                                           double& kz) {
    double kk, kv;
    const int off = tab.tab_off != nullptr ? tab.tab_off[m] : -1;
    if (off >= 0) {
        const int n = tab.tab_n[m];
        const double* t = tab.tab_T + off;
        const double* a = tab.tab_kxy + off;
        const double* c = tab.tab_kz + off;
        if (!(T > t[0])) {  // also a NaN temperature
            kk = a[0];
            kv = c[0];
        } else if (T >= t[n - 1]) {
            kk = a[n - 1];
            kv = c[n - 1];
        } else {
            int lo = 0, hi = n - 1;  // t[lo] < T < t[hi]
            while (hi - lo > 1) {
                const int mid = (lo + hi) >> 1;
                if (t[mid] <= T)
                    lo = mid;
                else
                    hi = mid;
            }
            const double w = (T - t[lo]) / (t[hi] - t[lo]);
            kk = a[lo] + w * (a[hi] - a[lo]);
            kv = c[lo] + w * (c[hi] - c[lo]);
        }
        if (tab.hexp[m] != 0.0) {
            const double f = pow(h, tab.hexp[m]);
            kk *= f;
            kv *= f;
        }
    } else {
        kk = tab.k300[m] * pow(300.0 / T, tab.p[m]);
        if (tab.hexp[m] != 0.0) kk *= pow(h, tab.hexp[m]);
        kv = kk * tab.kz_ratio[m];
    }
    kxy = kk;
    kz = kv;
}
#endif

struct LaunchCfg {
    cudaStream_t stream;
    int sm_count;      // streaming multiprocessors of the device
    int vec_blocks;    // grid size cap of streaming kernels (a multiple of the SM count)
    int op_share;      // the stencil kernel's grid aims at 1/op_share of the GPU's resident
                       // blocks (1: the whole GPU; >1 when several solves run concurrently)
    int op_rows;       // FP32 stencil kernel: output rows per thread (4, 5 or 6), chosen per mesh
};

long long launch_count();         // kernels launched by this library so far (all handles)
long long thread_launch_count();  // kernels launched so far from the calling host thread
void prime_launch_shapes();  // occupancy-derived grid sizes, queried before any graph capture
int vec_blocks(const LaunchCfg& c, long long N);

// Optimised operator (fem3d_operator.cu).  zf[k] = dz_k / 48, zr[k] = 1 / (48 dz_k).
// number of blocks (= partial-sum slots written in MODE_CG) of one operator launch
int op_blocks(const LaunchCfg& c, int n0, int n1, int n2, bool fp64);
// FP32 stencil tile (output rows per thread) for a mesh with n1 nodes along axis 1
int choose_op_rows(int n1);
// MODE_CG: y = A x, where nodes flagged in smask add the S x that k_surface (launched
// just before, launch_surface_cg) left in y; the last block sums the operator's partials
// and the sslots surface partials after them into (x, A x) and sets alpha = rz / (x, A x)
// (or the breakdown / non-finite status).  With run (FP32, the fused CG iteration of
// fem3d_cg_fused.cu): the launch runs while *run == SOLVE_RUNNING and leaves only its block
// partials (op_blocks of them, slot = block index) for the update kernel.
void launch_operator(const LaunchCfg& c, const GridT<float>& g, const float* zf, const float* zr, const float* x,
                     float* y, const float* kxy, const float* kz, bool aniso, const uint32_t* dmask, const float* rhs,
                     double* partials, int mode, SolveCtl* ctl, const uint32_t* smask = nullptr, int sslots = 0,
                     const float* dshift = nullptr, const float* cmass = nullptr, const int* run = nullptr);
void launch_operator(const LaunchCfg& c, const GridT<double>& g, const double* zf, const double* zr, const double* x,
                     double* y, const double* kxy, const double* kz, bool aniso, const uint32_t* dmask,
                     const double* rhs, double* partials, int mode, SolveCtl* ctl, const uint32_t* smask = nullptr,
                     int sslots = 0, const double* dshift = nullptr, const double* cmass = nullptr);
// TMA-staged FP32 operator of the inner CG (fem3d_operator_tma.cu) on one fixed input
// vector x (the tensor map is encoded for it), for meshes with n0 a multiple of 4, at most
// 256, that fill at least 80 % of the kernel's 64-column warp spans.
struct TmaOperator;
bool tma_operator_supported(int n0, int n1, int n2, bool any_fill = false);
// nullptr when the mesh is not supported or a CUDA call fails; hx, hy, hz: element sizes
TmaOperator* tma_operator_create(const LaunchCfg& c, const GridT<double>& g, const std::vector<double>& hx,
                                 const std::vector<double>& hy, const std::vector<double>& hz, bool aniso,
                                 const float* x, float* P, float* Q);
void tma_operator_destroy(TmaOperator* t);
int tma_operator_blocks(const TmaOperator* t);  // partial-sum slots of one launch
const float* tma_operator_input(const TmaOperator* t);
bool tma_operator_aniso(const TmaOperator* t);
// P = k_xy dx dy dz / 48, Q = k_z dx dy / (16 dz) per element from the FP64 conductivities
void launch_tma_coef(const LaunchCfg& c, const TmaOperator* t, const GridT<double>& g, const double* kxy,
                     const double* kz);
// Convective surface rows for the TMA operator: plane[k] = 0 when z-plane k holds none,
// else 1 + the index of its node -> row map (map[(plane[k] - 1) n0 n1 + j n0 + i], -1: no
// row), and the rows' CSR (ptr, col, val) as in SurfaceT
struct TmaSurface {
    const int* plane;
    const int* map;
    const int* ptr;
    const int* col;
    const float* val;
};
// y = A x (+ S x on surface rows) for the operator's input x (no Dirichlet replacement);
// one partial of (x, y) per block at partials[block]; nothing runs unless *run is
// SOLVE_RUNNING; a timed-out wait sets ctl's status words to SOLVE_DEVICE_TIMEOUT
void launch_operator_tma(const LaunchCfg& c, const TmaOperator* t, float* y, double* partials, const int* run,
                         SolveCtl* ctl, const TmaSurface& s);
// ---- FP32 Jacobi-PCG on the TMA operator (fem3d_cg_fused.cu): per iteration the operator
// (q = A p), an update kernel and a direction kernel, each reducing the previous launch's
// partials in every block; control words alternate with the iteration parity q.
struct TmaCg {
    long long N;
    float *x, *r, *p, *q;
    const float* minv;
    double* part;  // 2 x kMaxPartialBlocks: (p, A p) per operator block; (r, M^-1 r), (r, r) per update block
    int upd_blocks, op_blocks;
};
// x = 0, p = M^-1 r; the last block sets the stop threshold and the status (as launch_cg_start)
void launch_tmacg_start(const LaunchCfg& c, const TmaCg& f, SolveCtl* ctl, double rtol, int ref_slot, int maxit,
                        int stall_limit);
// where the operator writes its partials, and the status word its launch of parity q checks
double* tmacg_op_partials(const TmaCg& f);
const int* tmacg_op_run(SolveCtl* ctl, int q);
// grid of the start, update and direction kernels (TmaCg::upd_blocks)
int tmacg_blocks(const LaunchCfg& c, long long N);
void launch_tmacg_update(const LaunchCfg& c, const TmaCg& f, SolveCtl* ctl, int q);
void launch_tmacg_direction(const LaunchCfg& c, const TmaCg& f, SolveCtl* ctl, int q);
// ctl->pq = the sum of nslots block partials (fixed order)
void launch_partials_to_ctl(const LaunchCfg& c, const double* partials, int nslots, SolveCtl* ctl);
// dshift: a diagonal added to the operator (lumped capacity); cmass: per-element corner
// capacities c of a consistent capacity matrix c (M (x) M (x) M), M = [[2,1],[1,2]] / 3
// CG step, first half: y[row] = S x on the surface rows and block partials of (x, S x) in
// slots slot0..slot0 + surface_cg_blocks - 1; returns the number of slots used.
int launch_surface_cg(const LaunchCfg& c, const SurfaceT<float>& s, const float* x, float* y, double* partials,
                      int slot0, const SolveCtl* ctl);
int launch_surface_cg(const LaunchCfg& c, const SurfaceT<double>& s, const double* x, double* y, double* partials,
                      int slot0, const SolveCtl* ctl);
// the same, running while *run == SOLVE_RUNNING (the fused CG iteration)
int launch_surface_cg_run(const LaunchCfg& c, const SurfaceT<float>& s, const float* x, float* y, double* partials,
                          int slot0, const int* run);
int surface_cg_blocks(int nrows);

// convective face terms in MODE_MULT (y += S x) or MODE_RESID (y -= S x)
void launch_surface(const LaunchCfg& c, const SurfaceT<double>& s, const double* x, double* y, int mode);
void launch_surface(const LaunchCfg& c, const SurfaceT<float>& s, const float* x, float* y, int mode);
void launch_cg_update(const LaunchCfg& c, long long N, double* x, double* r, const double* p, const double* q,
                      const double* minv, double* partials, SolveCtl* ctl);
void launch_cg_update(const LaunchCfg& c, long long N, float* x, float* r, const float* p, const float* q,
                      const float* minv, double* partials, SolveCtl* ctl);
void launch_cg_direction(const LaunchCfg& c, long long N, double* p, const double* r, const double* minv,
                         const SolveCtl* ctl);
void launch_cg_direction(const LaunchCfg& c, long long N, float* p, const float* r, const float* minv,
                         const SolveCtl* ctl);
void launch_cg_start(const LaunchCfg& c, long long N, double* x, bool zero_x, const double* r, double* p,
                     const double* minv, double* partials, SolveCtl* ctl, double rtol, int ref_slot, int maxit,
                     int stall_limit);
void launch_cg_start(const LaunchCfg& c, long long N, float* x, bool zero_x, const float* r, float* p,
                     const float* minv, double* partials, SolveCtl* ctl, double rtol, int ref_slot, int maxit,
                     int stall_limit);
void launch_fcg_dots(const LaunchCfg& c, long long N, const float* z, const float* r, const float* q, double* partials,
                     SolveCtl* ctl, int first);
void launch_fcg_direction(const LaunchCfg& c, long long N, float* p, const float* z, const SolveCtl* ctl);
// red[slot] = sum over rows with minv > 0 of x^2 / minv (= A_nn x_n^2), or of (A_nn x_n)^2
void launch_diag_norm2(const LaunchCfg& c, long long N, const double* x, const double* minv, int squared,
                       double* partials, SolveCtl* ctl, int slot);
// red[slot] = ||v||^2, or sum w v^2 when w is given (w = M^-1: the Jacobi-scaled norm)
void launch_norm2(const LaunchCfg& c, long long N, const double* v, float* v32, double* partials, SolveCtl* ctl,
                  int slot, const double* w = nullptr);
void launch_fill(const LaunchCfg& c, long long N, double* v, double value);
void launch_widen(const LaunchCfg& c, long long N, const float* a, double* b);
void launch_add_correction(const LaunchCfg& c, long long N, double* T, const float* d);
void launch_thickness(const LaunchCfg& c, int n0, int n1, int n2, const int* mat, const double* z, double* th);
void launch_coef(const LaunchCfg& c, int n0, int n1, int n2, const double* T, const int* mat, const double* th,
                 const MatTable& tab, double* k64, float* k32, double* kz64, float* kz32, bool aniso);
// Jacobi diagonal of the operator (plus `shift` per node when given) and its inverse
void launch_diag(const LaunchCfg& c, const GridT<double>& g, const double* kxy, const double* kz, bool aniso,
                 const SurfaceT<double>& s, const uint32_t* dmask, double* diag, double* minv64, float* minv32,
                 const double* shift = nullptr);
// add the surface rows' diagonal to `diag` and invert it (Dirichlet and empty rows: 0)
void launch_finish_diag(const LaunchCfg& c, long long N, const SurfaceT<double>& s, const uint32_t* dmask,
                        double* diag, double* minv64, float* minv32);
// ---- time stepping (dyn3d_kernels.cu)
// lumped heat capacity per node: sum over the node's active elements of
// cp dens 0.125e-9 dx dy dz / timestep, times `weight` (FP64 and, when c32 is given, FP32)
void launch_lumped_mass(const LaunchCfg& c, const GridT<double>& g, const int* mat, const uint8_t* excl,
                        const double* cp, const double* dens, double timestep, double* c64, float* c32,
                        double weight = 1.0);
// corner capacity per element (consistent matrix), FP64, FP32 and negated FP64
void launch_elem_capacity(const LaunchCfg& c, const GridT<double>& g, const int* mat, const uint8_t* excl,
                          const double* cp, const double* dens, double timestep, double* c64, float* c32,
                          double* cneg);
// v *= s for the four coefficient arrays (any may be nullptr)
void launch_scale4(const LaunchCfg& c, long long N, double s, double* a64, float* a32, double* b64, float* b32);
// X = cap T + w Y + F  (Y = -K T)
void launch_dyn_rhs(const LaunchCfg& c, long long N, const double* cap, const double* T, const double* Y, double w,
                    const double* F, double* X);

void launch_heat_load(const LaunchCfg& c, const GridT<double>& g, const double* q, const int* mat, const MatTable& tab,
                      double* F);
void launch_scatter_add(const LaunchCfg& c, int n, const int* idx, const double* val, double* F);
void launch_set_dirichlet(const LaunchCfg& c, int n, const int* idx, const double* v, double* b, double* T);
void launch_radiation(const LaunchCfg& c, int nrows, const int* row, const int* ptr, const int* src, const double* coef,
                      const double* tamb, const double* T, double* b);
void launch_err(const LaunchCfg& c, long long N, const double* T, const double* T0, const uint32_t* inactive,
                double* partials, SolveCtl* ctl);
void launch_flux(const LaunchCfg& c, const GridT<double>& g, const double* T, const int* mat, const double* hleaf,
                 const MatTable& tab, double* out);
void launch_conductivity(const LaunchCfg& c, int n0, int n1, int n2, const double* T, const int* mat, const double* th,
                         const MatTable& tab, double* out);
void launch_from_mesh_order_i32(const LaunchCfg& c, int n0, int n1, int n2, int m0, int m1, int m2, long long s0,
                                long long s1, long long s2, const int* src, int* dst, int fill);
void launch_from_mesh_order_f64(const LaunchCfg& c, int n0, int n1, int n2, int m0, int m1, int m2, long long s0,
                                long long s1, long long s2, const double* src, double* dst, double fill);
void launch_to_mesh_order_f64(const LaunchCfg& c, int m0, int m1, int m2, long long c1, long long c2, long long s0,
                              long long s1, long long s2, int comps, const double* src, double* dst);
void launch_gather(const LaunchCfg& c, long long n, const long long* idx, const double* in, double* out);
void launch_scatter(const LaunchCfg& c, long long n, const long long* idx, const double* in, double* out);

}  // namespace plgpu
