// Host-callable launchers of the Static2D / StaticCyl kernels (fem2d_kernels.cu).
//
// A planar handle keeps the 3D handle's layout with one node plane: node (i, j) of an
// n0 x n1 mesh at i + n0 j (axis 0 fastest), element (i, j) at the index of its
// lower-left node, padding slots (i = n0-1 or j = n1-1) with zero conductivity.
// Axis 1 is the vertical axis.  Conductivities are stored in W/(m K).  In the
// cylindrical form axis 0 is the radius and every element carries the weight of its
// midpoint radius rmid[i] (micrometres), as ThermalFem2DSolver<Geometry2DCylindrical>
// does (therm2d.cpp:333-346, 409-426); rmid == nullptr selects the Cartesian form.
#pragma once

#include <cstdint>

#include "fem3d_device.cuh"
#include "fem3d_kernels.h"

namespace plgpu {

// number of blocks (= partial-sum slots written in MODE_CG) of one planar operator launch
int op2d_blocks(const LaunchCfg& c, long long N);

// y = A x for the bilinear-quad stiffness; modes as the 3D operator (fem3d_kernels.h):
// MODE_CG adds the S x that k_surface_cg left in the smask rows, writes block partials
// of (x, A x), and its last block adds the sslots surface partials and sets alpha.
// dshift: a diagonal added to the operator (lumped heat capacity of time steps);
// cmass: per-element corner capacity c of the consistent matrix c (M (x) M), M = [[2,1],[1,2]] / 3
void launch_operator2d(const LaunchCfg& c, const GridT<double>& g, const double* rmid, const double* x, double* y,
                       const double* kx, const double* ky, const uint32_t* dmask, const double* rhs,
                       double* partials, int mode, SolveCtl* ctl, const uint32_t* smask, int sslots,
                       const double* dshift = nullptr, const double* cmass = nullptr);
void launch_operator2d(const LaunchCfg& c, const GridT<float>& g, const float* rmid, const float* x, float* y,
                       const float* kx, const float* ky, const uint32_t* dmask, const float* rhs, double* partials,
                       int mode, SolveCtl* ctl, const uint32_t* smask, int sslots, const float* dshift = nullptr,
                       const float* cmass = nullptr);

// layer-run thickness along axis 1 (ThermalFem2DSolver::onInitialize, therm2d.cpp:81-114)
void launch_thickness2d(const LaunchCfg& c, int n0, int n1, const int* mat, const double* y, double* th);
// per-element k(T) at the 4-node mean temperature (therm2d.cpp:210-217, 336-343); ky = kz_ratio k
void launch_coef2d(const LaunchCfg& c, int n0, int n1, const double* T, const int* mat, const double* th,
                   const MatTable& tab, double* k64, float* k32, double* ky64, float* ky32, bool aniso);
// Jacobi diagonal sum_e (X + Y) / 3, plus `shift` per node when given (the convective
// edge rows and the inversion follow in launch_finish_diag)
void launch_diag2d(const LaunchCfg& c, const GridT<double>& g, const double* rmid, const double* kx,
                   const double* ky, double* diag, const double* shift = nullptr);
// time stepping (femT2d.cpp:167, 298): lumped capacity per node, weight x the sum of the
// corner capacities c = cp dens 0.25e-3 w h / timestep (x r) of its active elements
// (FP64 and, when c32 is given, FP32), and the corner capacity per element with -c
void launch_lumped_mass2d(const LaunchCfg& c, const GridT<double>& g, const double* rmid, const int* mat,
                          const uint8_t* excl, const double* cp, const double* dens, double timestep, double* c64,
                          float* c32, double weight);
void launch_elem_capacity2d(const LaunchCfg& c, const GridT<double>& g, const double* rmid, const int* mat,
                            const uint8_t* excl, const double* cp, const double* dens, double timestep, double* c64,
                            float* c32, double* cneg);
// element heat load f = 0.25e-12 w h q (times rmid) on every corner (therm2d.cpp:220, 346)
void launch_heat_load2d(const LaunchCfg& c, const GridT<double>& g, const double* rmid, const double* q,
                        const int* mat, const MatTable& tab, double* F);
// heat flux per element, 2 values (saveHeatFluxes, therm2d.cpp:505-541)
void launch_flux2d(const LaunchCfg& c, const GridT<double>& g, const double* T, const int* mat, const double* hleaf,
                   const MatTable& tab, double* out);
// (k_x, k_y) per element at the element-mean temperature (therm2d.cpp:574-597)
void launch_conductivity2d(const LaunchCfg& c, int n0, int n1, const double* T, const int* mat, const double* th,
                           const MatTable& tab, double* out);

}  // namespace plgpu
