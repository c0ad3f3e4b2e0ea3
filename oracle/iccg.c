/*
 * IC(0)-preconditioned conjugate gradients on symmetric diagonal storage --
 * part of the CPU oracle (TEST INFRASTRUCTURE ONLY; used as the timed CPU
 * baseline where NSPCG cannot be built from the reference tree).
 *
 * Restates the reference's default iterative solve (NSPCG with the IC
 * preconditioner and the CG accelerator, plask/common/fem/iterative_matrix.hpp
 * :50-94, 141-339) from the published algorithms: an incomplete Cholesky
 * factorisation A ~ U^T U restricted to the stored diagonals (no fill), and
 * preconditioned CG with the relative preconditioned-residual stopping test
 * sqrt((r, M^-1 r) / (b, M^-1 b)) <= zeta.
 *
 * Storage (SparseBandMatrix, iterative_matrix.hpp:373-418):
 *   coef[c + n * d] = A(c, c + off[d]),  off[0] = 0 (the diagonal), off ascending.
 * Single-threaded, like NSPCG in the reference.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

/* U stored like A: u[c + n*d] = U(c, c + off[d]).  Returns 0, or the first row
 * whose pivot was not positive (the factorisation is then retried by the
 * caller with a diagonal shift). */
static long factor(long n, int nd, const int *off, const double *a, double *u, double shift) {
    memcpy(u, a, sizeof(double) * (size_t)n * nd);
    for (long i = 0; i < n; ++i) u[i] *= 1.0 + shift;
    for (long i = 0; i < n; ++i) {
        /* finalise row i: pivot */
        double piv = u[i];
        if (!(piv > 0.0)) return i + 1;
        double uii = sqrt(piv);
        u[i] = uii;
        for (int d = 1; d < nd; ++d) {
            long j = i + off[d];
            if (j >= n) break;
            u[i + n * d] /= uii;
        }
        /* eliminate row i from the rows below: U(j, l) -= U(i, j) U(i, l) for j, l in pattern(i) */
        for (int dj = 1; dj < nd; ++dj) {
            long j = i + off[dj];
            if (j >= n) break;
            double uij = u[i + n * dj];
            if (uij == 0.0) continue;
            for (int dl = dj; dl < nd; ++dl) {
                long l = i + off[dl];
                if (l >= n) break;
                double uil = u[i + n * dl];
                if (uil == 0.0) continue;
                long diff = l - j; /* >= 0 */
                /* find the stored diagonal of (j, l) */
                int dd = -1;
                for (int q = 0; q < nd; ++q)
                    if (off[q] == diff) { dd = q; break; }
                if (dd < 0) continue; /* outside the pattern: dropped (no fill) */
                u[j + n * dd] -= uij * uil;
            }
        }
    }
    return 0;
}

/* z = (U^T U)^-1 r */
static void psolve(long n, int nd, const int *off, const double *u, const double *r, double *z) {
    /* forward: U^T y = r, column-oriented */
    memcpy(z, r, sizeof(double) * (size_t)n);
    for (long i = 0; i < n; ++i) {
        double yi = z[i] / u[i];
        z[i] = yi;
        for (int d = 1; d < nd; ++d) {
            long j = i + off[d];
            if (j >= n) break;
            z[j] -= u[i + n * d] * yi;
        }
    }
    /* backward: U x = y */
    for (long i = n - 1; i >= 0; --i) {
        double s = z[i];
        for (int d = 1; d < nd; ++d) {
            long j = i + off[d];
            if (j >= n) break;
            s -= u[i + n * d] * z[j];
        }
        z[i] = s / u[i];
    }
}

static void matvec(long n, int nd, const int *off, const double *a, const double *x, double *y) {
    for (long i = 0; i < n; ++i) y[i] = a[i] * x[i];
    for (int d = 1; d < nd; ++d) {
        const double *ad = a + n * d;
        long o = off[d];
        for (long i = 0; i + o < n; ++i) {
            y[i] += ad[i] * x[i + o];
            y[i + o] += ad[i] * x[i];
        }
    }
}

/* Factorise (when u_fact is non-zero) and solve A x = b from the initial x.
 * u: factor storage of n*nd doubles, reused between calls when refactor == 0.
 * Returns 0 converged, 1 maximum iterations, -1 breakdown; *iters receives the count. */
int oracle_iccg(long n, int nd, const int *off, const double *a, double *u, int refactor, const double *b, double *x,
                int maxit, double zeta, int *iters, double *final_err) {
    double *r = malloc(sizeof(double) * (size_t)n), *z = malloc(sizeof(double) * (size_t)n);
    double *p = malloc(sizeof(double) * (size_t)n), *q = malloc(sizeof(double) * (size_t)n);
    int status = 1;
    if (!r || !z || !p || !q) {
        status = -1;
        goto done;
    }
    if (refactor) {
        double shift = 0.0;
        while (factor(n, nd, off, a, u, shift) != 0) {
            shift = shift == 0.0 ? 1e-3 : 2 * shift;
            if (shift > 1.0) {
                status = -1;
                goto done;
            }
        }
    }
    psolve(n, nd, off, u, b, z);
    double bnorm = 0.0;
    for (long i = 0; i < n; ++i) bnorm += b[i] * z[i];
    matvec(n, nd, off, a, x, q);
    for (long i = 0; i < n; ++i) r[i] = b[i] - q[i];
    psolve(n, nd, off, u, r, z);
    double rz = 0.0;
    for (long i = 0; i < n; ++i) {
        rz += r[i] * z[i];
        p[i] = z[i];
    }
    int it = 0;
    double err = bnorm > 0 ? sqrt(fabs(rz) / bnorm) : 0.0;
    while (err > zeta && it < maxit) {
        matvec(n, nd, off, a, p, q);
        double pq = 0.0;
        for (long i = 0; i < n; ++i) pq += p[i] * q[i];
        if (!(pq > 0.0)) {
            status = -1;
            break;
        }
        double alpha = rz / pq;
        for (long i = 0; i < n; ++i) {
            x[i] += alpha * p[i];
            r[i] -= alpha * q[i];
        }
        psolve(n, nd, off, u, r, z);
        double rzn = 0.0;
        for (long i = 0; i < n; ++i) rzn += r[i] * z[i];
        double beta = rzn / rz;
        rz = rzn;
        for (long i = 0; i < n; ++i) p[i] = z[i] + beta * p[i];
        ++it;
        err = bnorm > 0 ? sqrt(fabs(rz) / bnorm) : 0.0;
    }
    if (status != -1) status = err <= zeta ? 0 : 1;
    *iters = it;
    *final_err = err;
done:
    free(r);
    free(z);
    free(p);
    free(q);
    return status;
}
