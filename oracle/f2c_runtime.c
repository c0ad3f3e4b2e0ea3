/*
 * The handful of f2c runtime routines that NSPCG's f2c translation calls,
 * written from their Fortran definitions (SIGN, ** with real and integer
 * exponents).  Formatted output is switched off in the oracle
 * (iparm.level = -1), so the WRITE statements are no-ops.
 */
#include <math.h>
#include "libf2c/f2c.h"

integer s_wsfe(cilist *c) { (void)c; return 0; }
integer e_wsfe(void) { return 0; }
integer do_fio(ftnint *n, char *p, ftnlen len) { (void)n; (void)p; (void)len; return 0; }

/* Fortran SIGN(a, b): |a| with the sign of b (b >= 0 counts as positive) */
double d_sign(doublereal *a, doublereal *b) {
    double x = fabs(*a);
    return *b >= 0 ? x : -x;
}
integer i_sign(integer *a, integer *b) {
    integer x = *a >= 0 ? *a : -*a;
    return *b >= 0 ? x : -x;
}

/* a ** b for a real exponent */
double pow_dd(doublereal *a, doublereal *b) { return pow(*a, *b); }

/* a ** n for an integer exponent, by binary powering; negative n inverts */
double pow_di(doublereal *a, integer *n) {
    double base = *a, r = 1.0;
    long e = *n;
    if (e == 0) return 1.0;
    if (e < 0) { e = -e; base = 1.0 / base; }
    while (e) {
        if (e & 1) r *= base;
        base *= base;
        e >>= 1;
    }
    return r;
}

/* log10 of a real argument */
double d_lg10(doublereal *x) { return log10(*x); }
