/*
 * demo_indirect -- command-line solver over the binary problem file format,
 * the counterpart of the reference's demo (run_pdos.c:9-29), written in
 * plain C against include/pdos.h and linked with -lpdosindir, as any caller
 * of the reference's library is.
 *
 *   demo_indirect PROBLEM_FILE [SOLUTION_FILE]
 *
 * PROBLEM_FILE holds, in this order and with idxint-wide integers
 * (run_pdos.c:31-94): n, m, f, l, qsize, q[qsize], b[m], c[n], MAX_ITERS,
 * CG_MAX_ITS, ALPHA, EPS_ABS, CG_TOL (doubles), VERBOSE, NORMALIZE, Anz,
 * Ai[Anz], Ap[n+1], Ax[Anz] (doubles).  idxint is `long` when built with
 * DLONG (the reference's default) and `int` otherwise.
 *
 * Prints the file-read and solve times as the reference's demo does, then
 * the status and the objective c'x.  With SOLUTION_FILE it also writes
 * n, m (idxint), status (16 bytes), x[n], s[m], y[m] (doubles).  Exit
 * status: 0 on success, 1 on a usage or file error, 2 when pdos() fails
 * (the reason, from pdos_gpu_last_error(), goes to stderr).
 */
#define _POSIX_C_SOURCE 199309L
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "pdos.h"

const char *pdos_gpu_last_error(void); /* include/pdos_gpu.h */

static double now_s(void) {
  struct timespec t;
  clock_gettime(CLOCK_MONOTONIC, &t);
  return (double)t.tv_sec + 1e-9 * (double)t.tv_nsec;
}

/* fread of `count` items that must all be there */
static int read_all(void *dst, size_t size, size_t count, FILE *fp) {
  if (count == 0) return 0;
  return fread(dst, size, count, fp) == count ? 0 : -1;
}

static void *alloc_array(size_t size, idxint count) {
  if (count < 0) return NULL;
  return malloc(size * (size_t)(count > 0 ? count : 1));
}

/* Reads one problem; on failure frees what it allocated and returns -1. */
static int read_problem(FILE *fp, Data **dp, Cone **kp) {
  Data *d = calloc(1, sizeof(Data));
  Cone *k = calloc(1, sizeof(Cone));
  idxint anz = 0;
  int bad = (d == NULL || k == NULL);
  if (!bad) d->p = calloc(1, sizeof(Params));
  bad = bad || d->p == NULL;
  bad = bad || read_all(&d->n, sizeof(idxint), 1, fp) || read_all(&d->m, sizeof(idxint), 1, fp);
  bad = bad || read_all(&k->f, sizeof(idxint), 1, fp) || read_all(&k->l, sizeof(idxint), 1, fp);
  bad = bad || read_all(&k->qsize, sizeof(idxint), 1, fp);
  bad = bad || d->n < 0 || d->m < 0 || k->qsize < 0;
  if (!bad) {
    k->q = alloc_array(sizeof(idxint), k->qsize);
    d->b = alloc_array(sizeof(double), d->m);
    d->c = alloc_array(sizeof(double), d->n);
    bad = !k->q || !d->b || !d->c;
  }
  bad = bad || read_all(k->q, sizeof(idxint), (size_t)k->qsize, fp);
  bad = bad || read_all(d->b, sizeof(double), (size_t)d->m, fp);
  bad = bad || read_all(d->c, sizeof(double), (size_t)d->n, fp);
  bad = bad || read_all(&d->p->MAX_ITERS, sizeof(idxint), 1, fp);
  bad = bad || read_all(&d->p->CG_MAX_ITS, sizeof(idxint), 1, fp);
  bad = bad || read_all(&d->p->ALPHA, sizeof(double), 1, fp);
  bad = bad || read_all(&d->p->EPS_ABS, sizeof(double), 1, fp);
  bad = bad || read_all(&d->p->CG_TOL, sizeof(double), 1, fp);
  bad = bad || read_all(&d->p->VERBOSE, sizeof(idxint), 1, fp);
  bad = bad || read_all(&d->p->NORMALIZE, sizeof(idxint), 1, fp);
  bad = bad || read_all(&anz, sizeof(idxint), 1, fp) || anz < 0;
  if (!bad) {
    d->Ai = alloc_array(sizeof(idxint), anz);
    d->Ap = alloc_array(sizeof(idxint), d->n + 1);
    d->Ax = alloc_array(sizeof(double), anz);
    bad = !d->Ai || !d->Ap || !d->Ax;
  }
  bad = bad || read_all(d->Ai, sizeof(idxint), (size_t)anz, fp);
  bad = bad || read_all(d->Ap, sizeof(idxint), (size_t)d->n + 1, fp);
  bad = bad || read_all(d->Ax, sizeof(double), (size_t)anz, fp);
  if (bad) {
    freeData(&d, &k); /* frees every non-NULL array, as PDOS_free would */
    return -1;
  }
  *dp = d;
  *kp = k;
  return 0;
}

static int write_solution(const char *path, const Sol *sol) {
  FILE *fp = fopen(path, "wb");
  int bad;
  if (!fp) return -1;
  bad = fwrite(&sol->n, sizeof(idxint), 1, fp) != 1 || fwrite(&sol->m, sizeof(idxint), 1, fp) != 1;
  bad = bad || fwrite(sol->status, 1, 16, fp) != 16;
  bad = bad || fwrite(sol->x, sizeof(double), (size_t)sol->n, fp) != (size_t)sol->n;
  bad = bad || fwrite(sol->s, sizeof(double), (size_t)sol->m, fp) != (size_t)sol->m;
  bad = bad || fwrite(sol->y, sizeof(double), (size_t)sol->m, fp) != (size_t)sol->m;
  if (fclose(fp) != 0) bad = 1;
  return bad ? -1 : 0;
}

int main(int argc, char **argv) {
  Data *d = NULL;
  Cone *k = NULL;
  Sol *sol;
  FILE *fp;
  double t0, obj = 0.0;
  idxint j;
  if (argc < 2) {
    fprintf(stderr, "usage: %s PROBLEM_FILE [SOLUTION_FILE]\n", argv[0]);
    return 1;
  }
  t0 = now_s();
  fp = fopen(argv[1], "rb");
  if (!fp) {
    fprintf(stderr, "could not open %s\n", argv[1]);
    return 1;
  }
  if (read_problem(fp, &d, &k) != 0) {
    fclose(fp);
    fprintf(stderr, "%s is not a complete problem file\n", argv[1]);
    return 1;
  }
  fclose(fp);
  printf("File IO %4f seconds\n", now_s() - t0);

  t0 = now_s();
  sol = pdos(d, k);
  printf("Total factorize + solve time %4f seconds\n", now_s() - t0);
  if (!sol) {
    fprintf(stderr, "pdos failed: %s\n", pdos_gpu_last_error());
    freeData(&d, &k);
    return 2;
  }
  for (j = 0; j < d->n; ++j) obj += d->c[j] * sol->x[j];
  printf("status %s, objective %.10e\n", sol->status, obj);
  if (argc > 2 && write_solution(argv[2], sol) != 0) {
    fprintf(stderr, "could not write %s\n", argv[2]);
    freeSol(&sol);
    freeData(&d, &k);
    return 1;
  }
  freeSol(&sol);
  freeData(&d, &k);
  return 0;
}
