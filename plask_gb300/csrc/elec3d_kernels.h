// Host-callable launchers of the Shockley3D kernels (elec3d_kernels.cu).
#pragma once

#include <cstdint>

#include "fem3d_kernels.h"

namespace plgpu {

// One junction (active region): node planes bottom..top bound its elements in z.
struct JunctionInfo {
    int bottom, top;
    double height;  // z[top] - z[bottom] (um)
    double beta;    // 1/V
    double js;      // A/m^2
};

// Conductivities at the start of compute(): junction elements from `jsave` at the
// element of the same (i, j) in the middle layer of its junction (floored like
// loadConductivity), others from `over` (per element, when given and not NaN) or the
// material table.  sig/jsave/over hold (c00, c11) pairs per padded canonical element.
void launch_elec_init_cond(const LaunchCfg& c, int n0, int n1, int n2, const int* mat, const int* junc,
                           const JunctionInfo* info, const double* jsave, const double* over, const double* cxy,
                           const double* cz, const uint8_t* excl, double* sig);
void launch_elec_save_junction(const LaunchCfg& c, int n0, int n1, int n2, const int* junc, const JunctionInfo* info,
                               const double* sig, double* jsave);
void launch_elec_fill_pairs(const LaunchCfg& c, long long N, double* v, double a, double b);
// bj: optional (beta, js) per padded element replacing the junction's values (NaN beta: keep)
void launch_elec_junction_update(const LaunchCfg& c, int n0, int n1, int n2, const int* junc, const JunctionInfo* info,
                                 const double* bj, const double* V, int stable, double* sig);
void launch_elec_coef(const LaunchCfg& c, long long N, const double* sig, double* k64, float* k32, double* kz64,
                      float* kz32);
// current density into cur (3 per padded element); red[0] = max |dj|^2, red[1] = max |j|^2
void launch_elec_current(const LaunchCfg& c, const GridT<double>& g, const double* V, const double* sig,
                         const int* junc, const int* mat, const uint8_t* excl, int noactive, double* cur,
                         double* partials, SolveCtl* ctl);
// Joule heat per element (padded canonical when `padded`, else compact canonical)
void launch_elec_heat(const LaunchCfg& c, const GridT<double>& g, const double* V, const double* sig, const int* mat,
                      const uint8_t* excl, const uint8_t* noheat, double* out, int padded);
// eps (dV^2) per padded element, zero for excluded elements
void launch_elec_energy_density(const LaunchCfg& c, const GridT<double>& g, const double* V, const int* mat,
                                const uint8_t* excl, const double* eps, double* out);
// out[e] = w[e] dx dy dz over active padded elements (0 elsewhere), then red[slot] = sum
void launch_elec_volume_sum(const LaunchCfg& c, const GridT<double>& g, const double* w, const int* mat,
                            const uint8_t* excl, double* partials, SolveCtl* ctl, int slot);
// red[slot] = sum over junction elements of layer `level` of j_z dx dy
void launch_elec_plane_current(const LaunchCfg& c, const GridT<double>& g, const double* cur, const int* junc,
                               int level, double* partials, SolveCtl* ctl, int slot);

// dst = src (comps per padded element) with NaN in excluded elements
void launch_elec_masked_copy(const LaunchCfg& c, int n0, int n1, int n2, int comps, const double* src, const int* mat,
                             const uint8_t* excl, double* dst);
// mean of the 8 corner values per padded element
void launch_elem_average(const LaunchCfg& c, int n0, int n1, int n2, const double* T, double* out);

}  // namespace plgpu
