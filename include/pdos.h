/*
 * pdos.h -- public API of the GB300 PDOS indirect solver (libpdosindir.so).
 *
 * Drop-in for the reference's libpdosindir: the struct layouts and the three
 * entry points below are those of cvxgrp/pdos's pdos.h, so code written
 * against the reference compiles and links against this library unchanged.
 *
 *   Params ............ pdos.h:15-19
 *   Data .............. pdos.h:22-35   (A in CSC: Ax, Ai, Ap; b; c; warm start)
 *   Sol ............... pdos.h:37-41
 *   Cone .............. cones.h:8-13   (f zero rows, l orthant rows, SOCs q[])
 *   pdos/freeData/freeSol  pdos.h:85-87
 *
 * idxint is `long` when PDOS_DLONG (or the reference's DLONG) is defined --
 * the reference's default build (pdos.mk:3) -- and `int` otherwise, as in
 * globals.h:30-40.  libpdosindir.so is built with the 64-bit layout;
 * libpdosindir_i32.so carries the 32-bit one.
 *
 * Memory: the caller owns Data and Cone; freeData() releases every non-NULL
 * array with free().  pdos() returns a Sol allocated with malloc(); release
 * it with freeSol().  Unlike the reference, pdos() never writes through its
 * const Data* (the reference scales Ax and c in place when NORMALIZE=0 and
 * divides them back afterwards, common.h:185-192, pdos.c:170-177).
 */
#ifndef PDOS_GB300_PDOS_H
#define PDOS_GB300_PDOS_H

#if defined(PDOS_DLONG) || defined(DLONG)
#ifndef idxint
#define idxint long
#endif
#else
#ifndef idxint
#define idxint int
#endif
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* algorithm parameters (pdos.h:15-19) */
typedef struct PROBLEM_PARAMS {
  idxint MAX_ITERS, CG_MAX_ITS;
  double EPS_ABS, ALPHA, CG_TOL;
  idxint VERBOSE, NORMALIZE; /* booleans */
} Params;

/* problem data (pdos.h:22-35) */
typedef struct PROBLEM_DATA {
  idxint n, m;      /* A is m x n */
  double *Ax;       /* CSC values, Ap[n] entries */
  idxint *Ai, *Ap;  /* CSC row indices and column pointers */
  double *b, *c;
  double *x;        /* optional warm start (NULL = zeros) */
  double *y;
  double *s;
  Params *p;
} Data;

/* solution (pdos.h:37-41); status is "Solved" or "Indeterminate" */
typedef struct SOL_VARS {
  idxint n, m;
  double *x, *s, *y;
  char status[16];
} Sol;

/* cone (cones.h:8-13): rows in the order zero cone, orthant, SOCs */
typedef struct CONE {
  idxint f;      /* zero-cone rows */
  idxint l;      /* nonnegative-orthant rows */
  idxint *q;     /* sizes of the second-order cones */
  idxint qsize;  /* number of second-order cones */
} Cone;

/* Solve min c'x s.t. Ax + s = b, s in K (pdos.h:85).  Returns NULL when d or
 * k is NULL (as the reference, pdos.c:61-63) and also on invalid input or a
 * CUDA failure, where the reference would assert or crash; the reason is
 * then in pdos_gpu_last_error(). */
Sol *pdos(const Data *d, const Cone *k);

/* Free Data/Cone and every array they point to (pdos.h:86, pdos.c:134-152). */
void freeData(Data **d, Cone **k);

/* Free a Sol returned by pdos() (pdos.h:87, pdos.c:154-164). */
void freeSol(Sol **sol);

#ifdef __cplusplus
}
#endif

#endif /* PDOS_GB300_PDOS_H */
