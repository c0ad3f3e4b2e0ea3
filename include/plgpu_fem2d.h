/*
 * plgpu_fem2d.h -- C ABI of the GB300 Static2D / StaticCyl thermal FEM solvers.
 *
 * A 2D handle is a plgpu_fem3d handle in planar mode: it is created here and then
 * driven by the plgpu_fem3d_* calls of plgpu_fem3d.h, with these differences.
 *   - The mesh has two axes: axis 0 (horizontal; the radius r >= 0 in the
 *     cylindrical form) and axis 1 (vertical).  Node and element arrays use the
 *     mesh's 2D iteration order (PLaSK's RectangularMesh2D::IterationOrder,
 *     plask/mesh/rectangular2d.hpp:256, rectangular2d.cpp:20-50):
 *       PLGPU_ORDER2D_10: index = i0 + n0 * i1   (axis 0 changes fastest)
 *       PLGPU_ORDER2D_01: index = i1 + n1 * i0   (axis 1 changes fastest)
 *     Elements likewise over (n0-1) x (n1-1).
 *   - Materials: kz_ratio of plgpu_fem3d_set_materials is the vertical/horizontal
 *     ratio k_1 / k_0 (the second component of Material::thermk).
 *   - plgpu_fem3d_get_heat_flux writes 2 values per element (q_0, q_1), W/m^2
 *     (saveHeatFluxes, solvers/thermal/static/therm2d.cpp:505-541);
 *     plgpu_fem3d_get_conductivity writes (k_0, k_1) per element.
 *   - Boundary conditions act on element edges whose two nodes carry the condition
 *     (setBoundaries, therm2d.cpp:139-172).  With bc_compat = 1 (the default of
 *     plgpu_fem3d_set_solver) the convective stiffness is the reference's
 *     (coeff_1 + coeff_2) len / 6 and / 12 without the micrometre-to-metre factor that
 *     its load term carries (therm2d.cpp:242-255, 367-392), and in the cylindrical
 *     form it is weighted by the element's midpoint radius once more
 *     (therm2d.cpp:410-420); bc_compat = 0 applies 1e-6 len and a single radius weight.
 *   - Time stepping (plgpu_fem3d_set_dynamic, plgpu_fem3d_compute_dynamic) is PLaSK's
 *     thermal.dynamic.Dynamic2D / DynamicCyl (solvers/thermal/dynamic/femT2d.cpp): the
 *     capacity per element corner is c = cp dens 0.25e-3 w h / timestep (times the
 *     midpoint radius in the cylindrical form, femT2d.cpp:167, 298), lumped onto the
 *     diagonal or, with lumping 0, the consistent matrix c (4, 2, 1) / 9 by corner
 *     distance (femT2d.cpp:199-233).
 *   - The learned preconditioner is 3D only and returns PLGPU_ERR_ARG on a 2D handle.
 * Units as in plgpu_fem3d.h; the 2D system is per metre of depth (Cartesian) or per
 * radian with r in micrometres (cylindrical), as in the reference.
 */
#ifndef PLGPU_FEM2D_H
#define PLGPU_FEM2D_H

#include "plgpu_fem3d.h"

#ifdef __cplusplus
extern "C" {
#endif

/* 2D iteration orders, RectangularMesh2D::IterationOrder values */
enum { PLGPU_ORDER2D_10 = 0, PLGPU_ORDER2D_01 = 1 };

/* geometry of a 2D handle: Geometry2DCartesian (thermal.static.Static2D) or
   Geometry2DCylindrical (thermal.static.StaticCyl) */
enum { PLGPU_GEOMETRY_CARTESIAN = 1, PLGPU_GEOMETRY_CYLINDRICAL = 2 };

/* Create a 2D solver on a rectilinear mesh.  Replaces the mesh setup of
   ThermalFem2DSolver (FemSolverWithMaskedMesh::setupMaskedMesh,
   plask/common/fem/fem_solver.hpp:182-189).  ax0/ax1 strictly increasing, n >= 2
   each; in the cylindrical form ax0[0] >= 0. */
int plgpu_fem2d_create(const double* ax0, int n0, const double* ax1, int n1, int ordering, int geometry,
                       plgpu_fem3d** out);

#ifdef __cplusplus
}
#endif

#endif
