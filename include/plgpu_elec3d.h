/*
 * plgpu_elec3d.h -- C ABI of the GB300 Shockley3D electrical FEM solver.
 *
 * The handle solves PLaSK's electrical.shockley.Shockley3D problem
 * (solvers/electrical/shockley/electr3d.cpp, beta.hpp): Laplace's equation for
 * the potential with per-element conductivity tensors (c00 in-plane, c11
 * vertical), voltage boundary conditions and p-n junctions whose vertical
 * conductivity follows the Shockley diode law, iterated until the current
 * density settles.  It shares the trilinear-hexahedron operator, the linear
 * solvers and the mesh conventions of plgpu_fem3d.h: node and element arrays in
 * the mesh's iteration order, masked numbering when empty elements are
 * excluded, host pointers borrowed for the call, PLGPU_* status codes, no C++
 * exception across the boundary, one CUDA stream per handle.
 *
 * Units: micrometres, volts, S/m, current density kA/cm^2, heat density W/m^3,
 * total current mA, total heat mW, energy J, capacitance pF (the reference's).
 */
#ifndef PLGPU_ELEC3D_H
#define PLGPU_ELEC3D_H

#include "plgpu_fem3d.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct plgpu_elec3d plgpu_elec3d;

/* convergence of the junction update (electr3d.hpp:138, electr3d.cpp:263-268) */
enum { PLGPU_CONVERGENCE_FAST = 0, PLGPU_CONVERGENCE_STABLE = 1 };

/* ElectricalFem3DSolver(name) with setMesh (electr3d.cpp:20-45): axes in um, ordering PLGPU_ORDER_*. */
int plgpu_elec3d_create(const double* ax0, int n0, const double* ax1, int n1, const double* ax2, int n2, int ordering,
                        plgpu_elec3d** out);
int plgpu_elec3d_destroy(plgpu_elec3d* h);
const char* plgpu_elec3d_last_error(const plgpu_elec3d* h);

/* Material table (Material::cond, Material::eps, Material::kind == EMPTY and the
   "noheat" role of saveHeatDensity, electr3d.cpp:468-470): per material the
   conductivity tensor (c00, c11) [S/m]; eps (relative permittivity, may be NULL:
   1), empty (may be NULL) and noheat (may be NULL). */
int plgpu_elec3d_set_materials(plgpu_elec3d* h, int n_mat, const double* cond_xy, const double* cond_z,
                               const double* eps, const uint8_t* empty, const uint8_t* noheat);

/* Per element (mesh order): material id and junction number + 1 (0 outside the
   junctions).  The junctions replace the "active" role lookup of
   setupActiveRegions (electr3d.cpp:94-184); a junction must span the same node
   planes wherever it exists (ERR_ARG otherwise, as the reference throws). */
int plgpu_elec3d_set_elements(plgpu_elec3d* h, const int32_t* material, const int32_t* junction);

/* Optional per-element conductivities (mesh order, (c00, c11) pairs) that replace
   the table value of non-junction elements; NaN c00 keeps the table value, NULL
   removes the override.  This is how a caller passes Material::cond(T) evaluated
   at the element temperatures (loadConductivity, electr3d.cpp:203-225). */
int plgpu_elec3d_set_element_conductivity(plgpu_elec3d* h, const double* cond2);

/* Shockley parameters of junction `n` (setBeta / setJs, beta.hpp:48-78). Unset
   beta is NaN and unset js is 1, as in the reference's constructor. */
int plgpu_elec3d_set_junction(plgpu_elec3d* h, int n, double beta, double js);

/* Optional per-element Shockley parameters (mesh order, (beta, js) pairs) used by the
   junction update instead of the junction's values; NaN beta keeps them, NULL removes
   the override.  This is how a caller passes beta(T) and js(T) given as functions of
   the temperature (the Python Shockley solver's callables, electr_python.cpp:104-111). */
int plgpu_elec3d_set_junction_params(plgpu_elec3d* h, const double* beta_js);

/* Junction conductivity used before the first junction update (default (0, 5) S/m,
   the reference's start-cond); resets the stored junction conductivities. */
int plgpu_elec3d_set_junction_conductivity(plgpu_elec3d* h, double c00, double c11);

/* voltage_boundary: nodes (full-mesh indices, mesh order) at potential `volts`,
   eliminated in list order like temperature conditions. */
int plgpu_elec3d_clear_voltage(plgpu_elec3d* h);
int plgpu_elec3d_add_voltage(plgpu_elec3d* h, const int64_t* nodes, size_t count, double volts);

/* Linear solver as plgpu_fem3d_set_solver (bc_compat does not apply). */
int plgpu_elec3d_set_solver(plgpu_elec3d* h, int algorithm, double rtol, int maxit, int noconv, int empty_elements);

/* maxerr [%] of the current density (default 0.05) and PLGPU_CONVERGENCE_*. */
int plgpu_elec3d_set_loop(plgpu_elec3d* h, double maxerr, int convergence);

/* ElectricalFem3DSolver::compute(loops) (electr3d.cpp:356-442): returns toterr [%]
   of the call through *toterr; stats->max_t is max |j| at the junctions [kA/cm^2]. */
int plgpu_elec3d_compute(plgpu_elec3d* h, int loops, double* toterr, plgpu_stats* stats);

/* onInvalidate (electr3d.cpp:195-201): drops the potential, currents and stored
   junction conductivities. */
int plgpu_elec3d_invalidate(plgpu_elec3d* h);

/* Outputs.  Potential per node (masked numbering when masked) [V]; current density
   per element (3 per element, NaN in excluded elements) [kA/cm^2]; Joule heat per
   element [W/m^3]; conductivity per element (c00, c11; NaN in excluded elements). */
int plgpu_elec3d_get_potential(plgpu_elec3d* h, double* out);
int plgpu_elec3d_get_current_density(plgpu_elec3d* h, double* out3);
int plgpu_elec3d_get_heat(plgpu_elec3d* h, double* out);
int plgpu_elec3d_get_conductivity(plgpu_elec3d* h, double* out2);

/* getTotalCurrent(n) (electr3d.cpp:480-505) [mA], getTotalHeat (612-624) [mW],
   getTotalEnergy (567-599) [J] and getCapacitance (601-610) [pF] -- without the
   factor 2 per symmetric direction, which the caller applies. */
int plgpu_elec3d_total_current(plgpu_elec3d* h, int n, double* mA);
int plgpu_elec3d_total_heat(plgpu_elec3d* h, double* mW);
int plgpu_elec3d_total_energy(plgpu_elec3d* h, double* J);
int plgpu_elec3d_capacitance(plgpu_elec3d* h, double* pF);

/* The CUDA stream (cudaStream_t) all work of the handle is queued on. */
void* plgpu_elec3d_stream(plgpu_elec3d* h);

/* Thermo-electric coupling on the device: the thermal solver's heat sources become
   the electrical solver's Joule heat (ThermalFem3DSolver::inHeat <- outHeat).  Both
   handles must share the mesh axes.  The copy is ordered on the thermal handle's
   stream after the electrical handle's work. */
int plgpu_fem3d_heat_from(plgpu_fem3d* thermal, plgpu_elec3d* electrical);

/* The temperature of a thermal handle evaluated as element averages (mesh order),
   the inTemperature an electrical solver reads for Material::cond(T). */
int plgpu_fem3d_get_element_temperature(plgpu_fem3d* h, double* out);

#ifdef __cplusplus
}
#endif

#endif
