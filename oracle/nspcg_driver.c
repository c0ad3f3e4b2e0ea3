/*
 * Oracle-side driver of NSPCG (PLaSK extlib/nspcg, f2c translation compiled
 * from the reference tree by oracle/Makefile) -- TEST INFRASTRUCTURE ONLY.
 *
 * Sets the parameters the way SparseMatrix::solverhs does
 * (plask/common/fem/iterative_matrix.hpp:141-177): dfault defaults, then
 * nstore = 2 (symmetric diagonal storage), itmax, ipropa = 0, ifact, zeta,
 * ns1/ns2/lvfill/ltrunc/ndeg/omega, kblsz/nbl2d, level = -1.
 */
#include "libf2c/f2c.h"

extern int dfault_(integer *iparm, doublereal *rparm);
extern int nspcg_(S_fp precon, U_fp accel, integer *ndim, integer *mdim, integer *n, integer *maxnz,
                  doublereal *coef, integer *jcoef, integer *p, integer *ip, doublereal *u, doublereal *ubar,
                  doublereal *rhs, doublereal *wksp, integer *iwksp, integer *nw, integer *inw, integer *iparm,
                  doublereal *rparm, integer *ier);
extern int ic2_();
extern int jac2_();
extern int cg_();

/* iparm / rparm positions (extlib/nspcg/nspcg.hpp: iparm_t, rparm_t) */
enum { IP_NTEST = 0, IP_ITMAX = 1, IP_LEVEL = 2, IP_NS1 = 8, IP_NS2 = 9, IP_NS3 = 10, IP_NSTORE = 11, IP_IFACT = 14,
       IP_LVFILL = 15, IP_LTRUNC = 16, IP_IPROPA = 17, IP_KBLSZ = 18, IP_NBL2D = 19, IP_NDEG = 24 };
enum { RP_ZETA = 0, RP_OMEGA = 8 };

/* Solve with symmetric diagonal storage: coef[c + n*d] = A(c, c + jcoef[d]).
 * precond: 0 = ic2 (IC), 1 = jac2 (Jacobi); accelerator CG.
 * u: initial guess in, solution out.  Returns NSPCG's ier; iterations and
 * the final stopping-test value are written to *iters and *zeta_out.
 * nw / inw may be grown by NSPCG: the required sizes are returned in them. */
int oracle_nspcg_cg(int n, int mdim, double *coef, int *jcoef, double *u, double *rhs, int precond, int itmax,
                    double zeta, int ifact, int kblsz, int nbl2d, double *wksp, int *nw, int *iwksp, int *inw,
                    int *iters, double *zeta_out) {
    integer iparm[30];
    doublereal rparm[30];
    integer ndim = n, md = mdim, nn = n, maxnz = mdim, ier = 0;
    integer nwv = *nw, inwv = *inw;
    int i;
    for (i = 0; i < 30; ++i) {
        iparm[i] = 0;
        rparm[i] = 0.0;
    }
    dfault_(iparm, rparm);
    iparm[IP_NSTORE] = 2;
    iparm[IP_ITMAX] = itmax;
    iparm[IP_IPROPA] = 0;
    iparm[IP_IFACT] = ifact;
    rparm[RP_ZETA] = zeta;
    iparm[IP_NS1] = 5;
    iparm[IP_NS2] = 100000;
    iparm[IP_LVFILL] = 0;
    iparm[IP_LTRUNC] = 0;
    iparm[IP_NDEG] = 1;
    rparm[RP_OMEGA] = 1.0;
    iparm[IP_NS3] = 0;
    iparm[IP_KBLSZ] = kblsz;
    iparm[IP_NBL2D] = nbl2d;
    iparm[IP_LEVEL] = -1;
    nspcg_(precond == 0 ? (S_fp)ic2_ : (S_fp)jac2_, (U_fp)cg_, &ndim, &md, &nn, &maxnz, coef, jcoef, 0, 0, u, 0, rhs,
           wksp, iwksp, &nwv, &inwv, iparm, rparm, &ier);
    *nw = nwv;
    *inw = inwv;
    *iters = iparm[IP_ITMAX];
    *zeta_out = rparm[RP_ZETA];
    return ier;
}
