/*
 * plgpu_fem3d.h -- C ABI of the GB300 Static3D thermal FEM solver.
 *
 * One handle holds one rectilinear 3D mesh with its per-element materials,
 * heat sources and boundary conditions, and the device-resident temperature
 * field.  The calls replace what PLaSK's ThermalFem3DSolver does inside
 * compute(); each declaration names the reference code it stands in for
 * (paths relative to the PLaSK source tree).
 *
 * Conventions
 *   - Coordinates in micrometres, heat density in W/m^3, conductivity in W/(m K),
 *     temperature in K, heat flux in W/m^2 -- the reference's units.
 *   - Node and element arrays exchanged through this ABI use the mesh's
 *     iteration order (`ordering`, PLaSK's ORDER_<major><medium><minor>):
 *     index = i_minor + n_minor * (i_medium + n_medium * i_major), elements
 *     likewise over (n-1) per axis (plask/mesh/rectilinear3d.cpp:20-33,
 *     rectilinear3d.hpp:739-775).
 *   - With empty elements excluded, temperatures are returned on the masked
 *     mesh numbering: active nodes in mesh order
 *     (plask/mesh/rectangular_masked3d.cpp:40-64).
 *   - All pointers are host pointers borrowed for the duration of the call.
 *     Results are copied into caller-allocated buffers.
 *   - Every function returns PLGPU_OK (0) or a negative error code; the text
 *     of the last error of a handle is available from plgpu_fem3d_last_error.
 *     No C++ exception crosses this boundary.
 *   - A handle is not thread-safe; it owns one CUDA stream.
 */
#ifndef PLGPU_FEM3D_H
#define PLGPU_FEM3D_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct plgpu_fem3d plgpu_fem3d;

/* status codes */
enum {
    PLGPU_OK = 0,
    PLGPU_ERR_ARG = -1,        /* bad argument (BadInput in the reference) */
    PLGPU_ERR_CUDA = -2,       /* CUDA runtime failure */
    PLGPU_ERR_NOT_SPD = -3,    /* breakdown: matrix not positive definite
                                  (ComputationError, cholesky_matrix.hpp:96-100) */
    PLGPU_ERR_NOCONV = -4,     /* no convergence with noconv = error
                                  (iterative_matrix.hpp:299-304) */
    PLGPU_ERR_STATE = -5,      /* call out of order (no mesh, no materials) */
    PLGPU_ERR_NONFINITE = -6   /* NaN/Inf in the right-hand side or solution */
};

/* mesh iteration orders, PLaSK's RectilinearMesh3D::IterationOrder (rectilinear3d.hpp:349) */
enum { PLGPU_ORDER_012 = 0, PLGPU_ORDER_021, PLGPU_ORDER_102, PLGPU_ORDER_120, PLGPU_ORDER_201, PLGPU_ORDER_210 };

/* boundary-condition kinds: temperature_boundary, heatflux_boundary,
   convection_boundary, radiation_boundary (therm3d.hpp:82-85) */
enum { PLGPU_BC_TEMPERATURE = 0, PLGPU_BC_HEATFLUX = 1, PLGPU_BC_CONVECTION = 2, PLGPU_BC_RADIATION = 3 };

/* linear-solver algorithms.  The reference's FemMatrixAlgorithm values
   (fem_solver.hpp:25-29) are accepted and run on the GPU: CHOLESKY and GAUSS
   use the FP64 preconditioned CG, ITERATIVE the mixed-precision solver. */
enum {
    PLGPU_ALGO_CHOLESKY = 0,
    PLGPU_ALGO_GAUSS = 1,
    PLGPU_ALGO_ITERATIVE = 2,
    PLGPU_ALGO_GPU_PCG = 3,     /* FP64 Jacobi-preconditioned CG */
    PLGPU_ALGO_GPU_MIXED = 4,   /* FP32 Jacobi-PCG inside FP64 iterative refinement */
    PLGPU_ALGO_GPU_LEARNED = 5  /* flexible CG with the learned preconditioner, mixed precision */
};

/* what happens when the linear solver does not converge (iterative_matrix.hpp:86-87) */
enum { PLGPU_NOCONV_ERROR = 0, PLGPU_NOCONV_WARNING = 1, PLGPU_NOCONV_CONTINUE = 2 };

/* empty-element handling (fem_solver.hpp:139-143) */
enum { PLGPU_EMPTY_DEFAULT = 0, PLGPU_EMPTY_EXCLUDE = 1, PLGPU_EMPTY_INCLUDE = 2 };

/* Per-call statistics of plgpu_fem3d_compute. */
typedef struct plgpu_stats {
    int loops;              /* outer k(T) iterations run by this call */
    int total_loops;        /* loopno: outer iterations since initialisation */
    int inner_iterations;   /* CG iterations summed over the call */
    int refinements;        /* FP64 residual evaluations (mixed precision) */
    int converged;          /* last linear solve reached its tolerance */
    int fallbacks;          /* learned-preconditioner stagnations that fell back to Jacobi-PCG */
    double err;             /* last outer correction max|T - T_prev| [K] */
    double toterr;          /* largest correction during the call [K] (return value of compute) */
    double max_t;           /* maxT of the last outer iteration [K] */
    double last_rel_residual; /* FP64 ||b - A T|| / ||b|| of the last solve */
    double solve_ms;        /* device time of the linear solves [ms] */
    double total_ms;        /* device time of the whole call [ms] */
    long long kernel_launches; /* CUDA kernels this library launched during the call */
    int learned_iterations; /* inner iterations of the flexible CG with the learned preconditioner
                               (the rest of inner_iterations: Jacobi-PCG, after fallbacks) */
} plgpu_stats;

/* Create a solver on a rectilinear mesh.  Replaces mesh setup and
   FemSolverWithMaskedMesh::setupMaskedMesh (fem_solver.hpp:182-189).
   ax0/ax1/ax2 are strictly increasing node coordinates, n >= 2 each. */
int plgpu_fem3d_create(const double* ax0, int n0, const double* ax1, int n1, const double* ax2, int n2,
                       int ordering, plgpu_fem3d** out);

/* Release all device and host memory of the handle. */
int plgpu_fem3d_destroy(plgpu_fem3d* h);

/* Text of the last error of the handle (NULL handle: last creation error). */
const char* plgpu_fem3d_last_error(const plgpu_fem3d* h);

/* Material table: k_xy(T, h) = k300 * (300/T)^p * h^hexp, k_z = kz_ratio * k_xy.
   Replaces Material::thermk(T, h) (plask/material/material.hpp:691) for the
   materials of the structure.  empty[m] != 0 marks Material::EMPTY kinds.
   kz_ratio, hexp and empty may be NULL (1, 0, 0). */
int plgpu_fem3d_set_materials(plgpu_fem3d* h, int n_mat, const double* k300, const double* p,
                              const double* kz_ratio, const double* hexp, const uint8_t* empty);

/* Tabulated k(T) of one material, replacing the power law of
   plgpu_fem3d_set_materials for it: the reference calls the material's
   virtual Material::thermk(T, h) (plask/material/material.hpp:691) per
   element (therm3d.cpp:208-213, 366-370, 421-435); a caller binds any such
   material by sampling it at n_points temperatures T[i] (strictly increasing,
   K) into k_xy[i] and k_z[i] (W/(m K); k_z NULL: isotropic).  Between points k
   is linear in T, beyond the first and the last point it is held constant; the
   material's h^hexp factor still applies.  n_points = 0 removes the table.
   Call after plgpu_fem3d_set_materials, which clears all tables. */
int plgpu_fem3d_set_material_table(plgpu_fem3d* h, int material, int n_points, const double* T,
                                   const double* k_xy, const double* k_z);

/* Material id and heat density of every element, in mesh element order.
   Replaces geometry->getMaterial(midpoint) (therm3d.cpp:205) and the inHeat
   receiver sampled at element midpoints (therm3d.cpp:179).  heat may be NULL (no source).
   leaf_height (may be NULL) is the height of the geometry leaf holding each
   element, used by the heat-flux evaluation (therm3d.cpp:366-370); by default
   the layer-run thickness is used. */
int plgpu_fem3d_set_elements(plgpu_fem3d* h, const int32_t* material, const double* heat,
                             const double* leaf_height);

/* Replace only the heat density (inHeat changed, therm3d.cpp:179). */
int plgpu_fem3d_set_heat(plgpu_fem3d* h, const double* heat);

/* Remove all conditions of one kind. */
int plgpu_fem3d_clear_bc(plgpu_fem3d* h, int kind);

/* Append one boundary condition (BoundaryConditions::append, boundary_conditions.hpp).
   nodes: full-mesh node indices in mesh order.  Values:
     TEMPERATURE: v0 = T [K]
     HEATFLUX:    v0 = q [W/m^2]
     CONVECTION:  v0 = coeff [W/(m^2 K)], v1 = ambient [K]
     RADIATION:   v0 = emissivity, v1 = ambient [K]
   Conditions keep their order: the first matching one wins for heat flux,
   convection and radiation (boundary_conditions.hpp:182-186), temperature
   conditions are eliminated in list order (matrix.hpp:111-118). */
int plgpu_fem3d_add_bc(plgpu_fem3d* h, int kind, const int64_t* nodes, size_t count, double v0, double v1);

/* Solver choice.  algorithm: PLGPU_ALGO_*.  rtol: FP64 relative residual
   ||b - A T|| / ||b|| at which a linear solve stops (default 1e-14;
   ||b|| includes the Dirichlet rows, so this is what max |dT| <= 1e-6 K needs
   on strongly graded meshes).
   maxit: iteration cap of one linear solve (reference iterative.maxit).
   noconv: PLGPU_NOCONV_*.  empty_elements: PLGPU_EMPTY_*.
   bc_compat: 1 (default) reproduces the reference's placement of 3D face
   boundary terms (therm3d.cpp:150-165: contributions on element corners
   0..3, radiation reading global nodes 0..7); 0 places them on the face's
   own nodes with each node's own temperature. */
int plgpu_fem3d_set_solver(plgpu_fem3d* h, int algorithm, double rtol, int maxit, int noconv,
                           int empty_elements, int bc_compat);

/* Norm in which every linear solve measures its residual (plgpu_fem3d_set_solver's
   rtol is relative in this norm).  SCALED: ||r||_{D^-1} = sqrt(sum r_i^2 / A_ii)
   over free rows, which weighs every row against its own diagonal and so converges
   weakly conducting regions (junctions, oxide apertures, air when included) as tightly
   as the rest; the default of plgpu_elec3d handles.  PLAIN: the 2-norm over all rows;
   the default of plgpu_fem3d handles (on the layered thermal structures it reaches the
   same 2e-8 K agreement with 25 % fewer CG iterations).  Either way a solve also
   resolves the change since the previous solve to 1e-6 of its starting residual, down
   to the estimated FP64 rounding floor of b - A T.  (No reference counterpart: the reference
   solves directly or leaves the test to NSPCG, iterative_matrix.hpp:141-339.) */
enum { PLGPU_NORM_SCALED = 0, PLGPU_NORM_PLAIN = 1 };
int plgpu_fem3d_set_residual_norm(plgpu_fem3d* h, int norm);

/* Outer-loop parameters: inittemp [K] (initial and reset temperature) and
   maxerr [K] (limit of max|T - T_prev| that ends compute()), therm3d.cpp:58-61. */
int plgpu_fem3d_set_loop(plgpu_fem3d* h, double inittemp, double maxerr);

/* Run the thermal calculation: ThermalFem3DSolver::compute(loops)
   (therm3d.cpp:281-340).  loops = 0 iterates until err <= maxerr and the
   linear solve converged.  *toterr receives the return value of the
   reference (largest correction in the call).  stats may be NULL. */
int plgpu_fem3d_compute(plgpu_fem3d* h, int loops, double* toterr, plgpu_stats* stats);

/* Forget the computed temperatures (Solver::invalidate, therm3d.cpp:118-122). */
int plgpu_fem3d_invalidate(plgpu_fem3d* h);

/* Number of nodes in the solution vector (masked-mesh size) and of elements. */
int plgpu_fem3d_sizes(const plgpu_fem3d* h, size_t* n_nodes, size_t* n_elements);

/* Copy the nodal temperatures (masked-mesh numbering, mesh order) into out. */
int plgpu_fem3d_get_temperature(plgpu_fem3d* h, double* out);

/* Set the nodal temperatures (same layout as get); used as the starting field
   of the next compute(), like a warm restart of the reference. */
int plgpu_fem3d_set_temperature(plgpu_fem3d* h, const double* in);

/* Per-element heat flux [W/m^2], 3 values per element in mesh element order
   (saveHeatFluxes, therm3d.cpp:342-384).  Excluded elements give NaN. */
int plgpu_fem3d_get_heat_flux(plgpu_fem3d* h, double* out3);

/* Per-element (k_xy, k_z) [W/(m K)] at the element-average temperature and
   the layer-run thickness (ThermalConductivityData::at, therm3d.cpp:421-435). */
int plgpu_fem3d_get_conductivity(plgpu_fem3d* h, double* out2);

/* Per-element layer-run thickness [um] (onInitialize, therm3d.cpp:81-113). */
int plgpu_fem3d_get_thickness(plgpu_fem3d* h, double* out);

/* The CUDA stream the handle launches on (cudaStream_t), for event timing. */
void* plgpu_fem3d_stream(plgpu_fem3d* h);

/* y = A x with the system matrix of the current temperature field
   (FemMatrix::mult, plask/common/fem/matrix.hpp:84-89): the stiffness matrix
   of setMatrix after Dirichlet elimination (identity rows and zero couplings
   for Dirichlet nodes), including convective face terms.  x and y are full
   node arrays in mesh order.  precision: 64 (FP64 operator) or 32 (the FP32
   operator of the inner solver, result widened to double). */
int plgpu_fem3d_mult(plgpu_fem3d* h, int precision, const double* x, double* y);

/* The same product as plgpu_fem3d_mult, for callers that must not allocate
   device memory during the call: a host framework that has reserved the whole
   GPU for its own allocator (cudaMalloc then fails), or a latency-critical loop
   on other streams that cannot afford the device-wide synchronisation that
   cudaMalloc and cudaFree may cause.  No counterpart in the reference: it only
   changes where the staging buffer lives.
   - Allocates nothing: no cudaMalloc, cudaFree or allocating library call.  The
     device staging buffer is a file-scope array of 2,097,152 doubles (16 MiB)
     that every GPU loading this library keeps until the process exits; meshes
     with more nodes are rejected with PLGPU_ERR_ARG.
   - The handle must already be set up on the device (PLGPU_ERR_STATE otherwise):
     call plgpu_fem3d_compute or plgpu_fem3d_mult on it once first.  The call
     must run with the handle's device current (PLGPU_ERR_STATE otherwise).
   - The array's device address is looked up (cudaGetSymbolAddress) once per
     device when a handle is created on that device, not in this call.  Under
     CUDA's lazy module loading that look-up is when the driver places the array
     on the device, so the 16 MiB are taken at handle creation.
   - Works on 3D and planar (plgpu_fem2d_create) handles alike.
   - All calls share the array, which keeps the last call's contents; calls that
     overlap on the GPU (two handles on two streams at once) race on it. */
int plgpu_fem3d_mult_noalloc(plgpu_fem3d* h, int precision, const double* x, double* y);

/* The FP32 stiffness operator exactly as one inner CG iteration of the
   mixed-precision solve applies it: the convective surface rows and the
   stencil kernel the solve runs (the TMA-staged kernel where the mesh allows
   it), on the mesh-order vector x rounded to FP32; y = A x widened to double,
   without the Dirichlet identity rows (the CG direction is zero on Dirichlet
   nodes: pass x with zeros there to get the solve's product).  *xax (may be
   NULL) receives the sum of the kernel's per-block partials of (x, A x) in the
   solve's fixed order; *staged (may be NULL) is 1 when the TMA-staged kernel
   ran.  No counterpart in the reference (verification of the inner solve's
   kernel). */
int plgpu_fem3d_cg_operator(plgpu_fem3d* h, const double* x, double* y, double* xax, int* staged);

/* Time the operator kernel (one matrix-free stiffness application, the
   inner kernel of every CG iteration) on the handle's stream with CUDA
   events: `reps` launches on the current coefficients, optionally with the
   L2 cache flushed before each launch.  precision: 32 or 64.
   *avg_ms: mean launch duration; *bytes_per_launch: algorithmic bytes of
   one launch (read x, write y, the element conductivities). */
int plgpu_fem3d_time_operator(plgpu_fem3d* h, int precision, int reps, int flush_l2, double* avg_ms,
                              double* bytes_per_launch);

/* Receive the solver's log lines (Solver::writelog, plask/log/log.hpp:27-42).
   level follows PLaSK's LogLevel numbering (2 warning, 3 info, 4 result,
   5 data, 6 detail); the per-loop line is
   "Loop n(m): max(T) = ... K, error = ... K" (therm3d.cpp:332). */
int plgpu_fem3d_set_log_callback(plgpu_fem3d* h, void (*cb)(void* user, int level, const char* msg), void* user);

/* ---------------------------------------------------------------------------------
   Time stepping: PLaSK's thermal.dynamic.Dynamic3D (solvers/thermal/dynamic/femT3d.cpp)
   on the same handle, mesh, materials, heat and temperature conditions (on a 2D handle
   Dynamic2D / DynamicCyl, femT2d.cpp: plgpu_fem2d.h). */

/* Heat capacity cp [J/(kg K)] and density dens [kg/m^3] per material, timestep [ns],
   methodparam theta (0.5 Crank-Nicolson, 0 explicit, 1 implicit), lumping (nonzero:
   the lumped heat-capacity matrix, the reference's default; 0: the consistent matrix
   c (8, 4, 2, 1) / 27 per element, femT3d.cpp:203-226), rebuildfreq (rebuild A and B
   with k(T) every that many steps, 0 never) and logfreq (femT3d.cpp:26-34, 54-66). */
int plgpu_fem3d_set_dynamic(plgpu_fem3d* h, const double* cp, const double* dens, double timestep,
                            double methodparam, int lumping, int rebuildfreq, int logfreq);

/* DynamicThermalFem3DSolver::compute(time) (femT3d.cpp:255-315): theta-method steps of
   A T' = B T + F while t < time + timestep / 2, from the handle's temperature, with the
   Dirichlet nodes held at their values (the scheme setMatrix prepares; the reference's
   step loop lets them drift by (B T)[r]).
   *elapsed receives the solver's elapsed time [ns]; stats->loops the steps of this call,
   stats->max_t max(T).  Only temperature boundary conditions are allowed. */
int plgpu_fem3d_compute_dynamic(plgpu_fem3d* h, double time, double* elapsed, plgpu_stats* stats);

/* ---------------------------------------------------------------------------------
   Batched solves (a sweep of independent structures).  No reference counterpart: the
   reference solves one structure per solver object, one after another. */

/* Grid policy of the stencil kernel: its grid aims at 1/share of the GPU's resident
   blocks (1, the default, fills the GPU; a larger share leaves room for the kernels of
   other solves running at the same time). */
int plgpu_fem3d_set_grid_share(plgpu_fem3d* h, int share);

/* compute(loops) of `count` distinct handles, run concurrently from `threads` host
   threads; every handle works on its own CUDA stream, so the kernels of different
   solves share the SMs.  toterr, stats and status (PLGPU_* of each handle) may be NULL.
   Returns PLGPU_OK when all succeeded, else the first failing handle's code (its message
   is in that handle's plgpu_fem3d_last_error). */
int plgpu_fem3d_batch_compute(plgpu_fem3d* const* handles, int count, int loops, int threads, double* toterr,
                              plgpu_stats* stats, int* status);

/* Autotuner of the batched path: for threads = 1, 2, 4, ... <= max_threads and grid share
   1 or threads, invalidates the handles and times plgpu_fem3d_batch_compute over them;
   every handle is left with the fastest grid share.  timings (may be NULL) receives
   solves/s per trial, 2 per thread count (share 1, share = threads). */
int plgpu_fem3d_batch_tune(plgpu_fem3d* const* handles, int count, int loops, int max_threads, int* best_threads,
                           int* best_share, double* timings);

#ifdef __cplusplus
}
#endif

#endif /* PLGPU_FEM3D_H */
