/*
 * Minimal type header for compiling the f2c translation of NSPCG
 * (extlib/nspcg/nspcg.c in PLaSK) as part of the CPU oracle.
 *
 * Written for this oracle; it is not the libf2c header.  The one deliberate
 * difference from the vendored libf2c header (extlib/libf2c/f2c.h:10,18,46 in
 * PLaSK, where INTEGER/LOGICAL/ftnlen are `long`) is that Fortran INTEGER and
 * LOGICAL are 32-bit `int` here.  PLaSK's C++ side passes `int` to NSPCG
 * (plask/common/fem/iterative_matrix.hpp:262 and extlib/nspcg/nspcg.hpp:349),
 * which only matches a 32-bit INTEGER on LP64 Linux.
 */
#ifndef ORACLE_F2C_SHIM_H
#define ORACLE_F2C_SHIM_H

typedef int integer;
typedef unsigned int uinteger;
typedef char *address;
typedef short int shortint;
typedef float real;
typedef double doublereal;
typedef int logical;
typedef int flag;
typedef int ftnlen;
typedef int ftnint;

/* formatted-write control block; the oracle never prints (iparm.level = -1) */
typedef struct {
    flag cierr;
    ftnint ciunit;
    flag ciend;
    char *cifmt;
    ftnint cirec;
} cilist;

#define TRUE_ (1)
#define FALSE_ (0)

#ifndef abs
#define abs(x) ((x) >= 0 ? (x) : -(x))
#endif
#define dabs(x) (double)abs(x)
#ifndef min
#define min(a, b) ((a) <= (b) ? (a) : (b))
#endif
#ifndef max
#define max(a, b) ((a) >= (b) ? (a) : (b))
#endif

/* old-style (unprototyped) procedure pointers, as f2c emits them */
typedef int (*U_fp)();
typedef int (*S_fp)();
typedef doublereal (*D_fp)();

/* runtime entry points used by nspcg.c, implemented in oracle/f2c_runtime.c */
integer s_wsfe(cilist *);
integer e_wsfe(void);
integer do_fio(ftnint *, char *, ftnlen);
double d_sign(doublereal *, doublereal *);
integer i_sign(integer *, integer *);
double pow_dd(doublereal *, doublereal *);
double pow_di(doublereal *, integer *);
double d_lg10(doublereal *);

#endif
