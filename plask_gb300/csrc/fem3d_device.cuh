// Device-side data structures shared by the Static3D kernels and their host driver.
//
// Layout in HBM ("canonical" order): node (i, j, k) of an n0 x n1 x n2 grid
// lives at i + n0 * (j + n1 * k) -- axis 0 fastest, axis 2 (vertical) slowest.
// Element arrays are padded to the node grid: element (i, j, k) is the hexahedron
// whose lowest corner is node (i, j, k), stored at the same index; the padding
// slots (i = n0-1, j = n1-1 or k = n2-1) hold zero conductivity.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace plgpu {

// Mesh geometry handed to kernels by value.
template <typename R>
struct GridT {
    int n0, n1, n2;
    long long N;          // n0 * n1 * n2
    const R* h0;          // element sizes along each axis (n-1 entries), micrometres
    const R* h1;
    const R* h2;
    const R* r0;          // reciprocals of h0/h1/h2
    const R* r1;
    const R* r2;
};

// Scalars of one Krylov solve, resident in device memory so that the whole
// iteration runs without host round trips.  The kernels read alpha/beta from
// here and the last block of each reduction writes them.
struct SolveCtl {
    double rz;        // current (r, z) of the preconditioned residual
    double rz_old;
    double rr;        // current (r, r)
    double tol2;      // stop when the residual measure (rz, or rr with `plain`) <= tol2
    double pq;        // (p, A p)
    double alpha;
    double beta;
    double best_rr;   // smallest residual measure seen (stagnation detection)
    int iter;         // iterations done
    int maxit;        // iteration cap
    int status;       // SOLVE_RUNNING / _CONVERGED / _MAXIT / _BREAKDOWN / _NONFINITE / _STAGNATED
    int stall;        // iterations since best_rr improved by the stagnation factor
    int stall_limit;
    int plain;        // nonzero: judge convergence on (r, r) instead of the Jacobi-scaled (r, M^-1 r)
    unsigned int arrive[4];   // arrival counters of the grid reductions
    double red[8];            // results of auxiliary reductions (norms, err, maxT)
    // FP32 CG on the TMA operator (fem3d_cg_fused.cu): the kernels of iteration parity q
    // read slot q of these and the direction kernel writes slot 1 - q, so that no block
    // reads a word another block of the same launch writes
    double rz2[2];     // (r, M^-1 r) of the current iterate
    int status2[2];    // solve status before the iteration
    int ustatus;       // the update kernel's verdict on (p, A p), read by the direction kernel
};

// SOLVE_DEVICE_TIMEOUT: a kernel's bounded wait for its own asynchronous copies ran out
enum { SOLVE_RUNNING = 0, SOLVE_CONVERGED = 1, SOLVE_MAXIT = 2, SOLVE_BREAKDOWN = 3, SOLVE_NONFINITE = 4,
       SOLVE_STAGNATED = 5, SOLVE_DEVICE_TIMEOUT = 6 };

// Sparse symmetric surface operator (convective boundary terms), rows unique,
// restricted to free (non-Dirichlet) rows and columns.
template <typename R>
struct SurfaceT {
    int nrows;
    const int* row;       // canonical node index of each row
    const int* ptr;       // nrows + 1
    const int* col;       // canonical node index of each entry
    const R* val;
};

constexpr int kMaxPartialBlocks = 4096;

#ifdef __CUDACC__
// Programmatic dependent launch (launch_kernel_pdl): pdl_trigger lets the next kernel of the
// stream be scheduled while this one runs; pdl_wait blocks until the previous kernel has
// completed and its writes are visible.  Both are no-ops in a kernel launched normally.
// Where the kernels of the fused CG let the next one be scheduled (overridable at compile
// time for tuning): 0 = only when their blocks exit, 1 = at their start, 2 = after their
// main loop.
#ifndef PLGPU_PDL_TRIGGER
#define PLGPU_PDL_TRIGGER 0
#endif
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger_at(int where) {
    if (where == PLGPU_PDL_TRIGGER) pdl_trigger();
}
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
#endif

}  // namespace plgpu
