/*
 * pdos_oracle.c -- CPU restatement of PDOS's indirect ADMM path.
 *
 * TEST INFRASTRUCTURE, NOT PRODUCT CODE.  Only the test suite, the smoke
 * check of __graft_entry__ and the CPU-baseline leg of bench.py load this
 * file's shared library, and only as the checker / the timed CPU baseline.
 * The shipped solver (libpdosindir.so) never links or calls it.
 *
 * It restates, in plain sequential C99 and in the reference's own order of
 * floating-point operations, the functions of cvxgrp/pdos's indirect build:
 *
 *   cs_transpose / cs_cumsum ........ cs.c:146-168, cs.c:83-97
 *   commonWorkInit (2-norm scaling) . common.h:35-218
 *   commonWorkInit (Ruiz variant) ... ruiz_equil_common.h:17-81, :98-322
 *   accumByScaledA / ATrans ......... linAlg.h:70-115
 *   calcPriResid / calcDualResid .... linAlg.h:158-191
 *   calcPriObj / calcDualObj ........ linAlg.h:194-201
 *   prepArgument / cgCustom ......... indirect/private.c:20-104
 *   projectLinSys ................... indirect/private.c:106-118
 *   relax / projectCones / dual ..... pdos.c:232-249, :296-303
 *   projCone / projSelfDualCone ..... cones.c:5-57
 *   pdos() loop + getSolution ....... pdos.c:50-132, :251-294
 *
 * Build with -ffp-contract=off so that x86-64 and aarch64 give the same
 * bits (the reference, compiled for x86-64 without FMA, rounds each
 * multiply and add separately).  Indices are int64 (the reference's idxint
 * under -DDLONG, globals.h:30-40).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef int64_t oidx;

#define SQRT_RATIO_ 1e3
#define RANGE_MAX_ 1e6
#define RANGE_MIN_ 1e-6
#define RUIZ_PASSES 3

/* ---------------------------------------------------------------------- */
/* Sparse transpose: CSC (m x n) -> CSR of the same matrix, i.e. CSC of A'.
 * Entries of each output row come out in increasing column order because
 * columns are visited in order (cs.c:146-168).  Rp has m+1 entries. */
int oracle_csc_to_csr(oidx m, oidx n, const oidx *Ap, const oidx *Ai,
                      const double *Ax, oidx *Rp, oidx *Rj, double *Rx) {
  oidx *cursor = (oidx *)calloc((size_t)(m > 0 ? m : 1), sizeof(oidx));
  oidx nnz = Ap[n], total = 0, r, j, p;
  if (!cursor) return -1;
  for (p = 0; p < nnz; ++p) cursor[Ai[p]] += 1;
  /* exclusive prefix sum into Rp, cursor becomes the write position
   * (cs.c:83-97) */
  for (r = 0; r < m; ++r) {
    oidx cnt = cursor[r];
    Rp[r] = total;
    cursor[r] = total;
    total += cnt;
  }
  Rp[m] = total;
  for (j = 0; j < n; ++j) {
    for (p = Ap[j]; p < Ap[j + 1]; ++p) {
      oidx dst = cursor[Ai[p]]++;
      Rj[dst] = j;
      if (Rx && Ax) Rx[dst] = Ax[p];
    }
  }
  free(cursor);
  return 0;
}

/* y (+)= sc * M x for M given row-wise (rowptr/colidx/val, `rows` rows):
 * the row gather of linAlg.h:70-91 (and, applied to the CSC arrays, the
 * column gather of linAlg.h:94-115).  Each row sum starts from 0 and adds
 * (sc*v)*x term by term; the result is stored or added to y. */
void oracle_gather_mv(oidx rows, const oidx *rowptr, const oidx *colidx,
                      const double *val, const double *x, double sc,
                      double *y, int accum) {
  oidx r, p;
  for (r = 0; r < rows; ++r) {
    double acc = 0.0;
    for (p = rowptr[r]; p < rowptr[r + 1]; ++p) acc += sc * val[p] * x[colidx[p]];
    y[r] = accum ? y[r] + acc : acc;
  }
}

static double sumsq(const double *v, oidx len) {
  double acc = 0.0;
  oidx i;
  for (i = 0; i < len; ++i) acc += v[i] * v[i];
  return acc;
}

static double dot(const double *a, const double *b, oidx len) {
  double acc = 0.0;
  oidx i;
  for (i = 0; i < len; ++i) acc += a[i] * b[i];
  return acc;
}

/* ---------------------------------------------------------------------- */
/* Cone projection in place (cones.c:5-57): zero cone rows -> 0, nonnegative
 * rows -> max(0, .), each second-order cone by the three-case rule. */
void oracle_proj_cone(double *v, oidx f, oidx l, oidx qsize, const oidx *q) {
  oidx i, j, off;
  for (i = 0; i < f; ++i) v[i] = 0.0;
  for (i = f; i < f + l; ++i)
    if (v[i] < 0.0) v[i] = 0.0;
  off = f + l;
  for (i = 0; i < qsize; ++i) {
    double head = v[off], tail = 0.0, half;
    for (j = 1; j < q[i]; ++j) tail += v[off + j] * v[off + j];
    tail = sqrt(tail);
    half = (tail + head) / 2.0;
    if (tail <= head) {
      /* inside the cone: keep */
    } else if (tail <= -head) {
      for (j = 0; j < q[i]; ++j) v[off + j] = 0.0;
    } else {
      v[off] = half;
      for (j = 1; j < q[i]; ++j) v[off + j] = half * v[off + j] / tail;
    }
    off += q[i];
  }
}

/* ---------------------------------------------------------------------- */
/* Default equilibration (common.h:69-162).  Produces D (m), E (n) and the
 * scaled CSC values Aw (same pattern as A).  Warm-start scaling is done by
 * the caller. */
void oracle_scale_default(oidx m, oidx n, const oidx *Ap, const oidx *Ai,
                          const double *Ax, oidx f, oidx l, oidx qsize,
                          const oidx *q, double *D, double *E, double *Aw) {
  oidx i, j, p, off, cone;
  for (i = 0; i < m; ++i) D[i] = 0.0;
  for (j = 0; j < n; ++j) E[j] = 0.0;
  memcpy(Aw, Ax, sizeof(double) * (size_t)Ap[n]);
  /* row sums of squares, accumulated column by column */
  for (j = 0; j < n; ++j)
    for (p = Ap[j]; p < Ap[j + 1]; ++p) D[Ai[p]] += Ax[p] * Ax[p];
  /* every row of a second-order cone gets the cone's mean */
  off = f + l;
  for (cone = 0; cone < qsize; ++cone) {
    double total = 0.0;
    for (i = 0; i < q[cone]; ++i) total += D[off + i];
    for (i = 0; i < q[cone]; ++i) D[off + i] = total / q[cone];
    off += q[cone];
  }
  for (i = 0; i < m; ++i) {
    double t = fabs(D[i]);
    t = t > RANGE_MIN_ ? t : RANGE_MIN_;
    t = t < RANGE_MAX_ ? t : RANGE_MAX_;
    D[i] = 1.0 / sqrt(t);
  }
  for (j = 0; j < n; ++j)
    for (p = Ap[j]; p < Ap[j + 1]; ++p) Aw[p] *= D[Ai[p]];
  for (j = 0; j < n; ++j)
    for (p = Ap[j]; p < Ap[j + 1]; ++p) E[j] += Aw[p] * Aw[p];
  for (j = 0; j < n; ++j) {
    double t = fabs(E[j]);
    t = t > RANGE_MIN_ ? t : RANGE_MIN_;
    t = t < RANGE_MAX_ ? t : RANGE_MAX_;
    E[j] = 1.0 / sqrt(t);
  }
  for (j = 0; j < n; ++j)
    for (p = Ap[j]; p < Ap[j + 1]; ++p) Aw[p] *= E[j];
}

/* Ruiz equilibration of [A b; c' 0] with cone rows collapsed
 * (ruiz_equil_common.h:17-81, :130-245).  Produces D, E and Aw. */
void oracle_scale_ruiz(oidx m, oidx n, const oidx *Ap, const oidx *Ai,
                       const double *Ax, const double *b, const double *c,
                       oidx f, oidx l, oidx qsize, const oidx *q, double *D,
                       double *E, double *Aw) {
  oidx nnz = Ap[n], i, j, p, it, cone, off;
  double *cv = (double *)malloc(sizeof(double) * (size_t)(nnz > 0 ? nnz : 1));
  oidx *ci = (oidx *)malloc(sizeof(oidx) * (size_t)(nnz > 0 ? nnz : 1));
  double *cb = (double *)malloc(sizeof(double) * (size_t)(m > 0 ? m : 1));
  double *rowmax = (double *)calloc((size_t)(m > 0 ? m : 1), sizeof(double));
  double *colmax = (double *)calloc((size_t)(n > 0 ? n : 1), sizeof(double));
  double dlast = 1.0, elast = 1.0, rlast = 0.0, clast = 0.0;
  memcpy(cv, Ax, sizeof(double) * (size_t)nnz);
  memcpy(ci, Ai, sizeof(oidx) * (size_t)nnz);
  memcpy(cb, b, sizeof(double) * (size_t)m);
  for (i = 0; i < m; ++i) D[i] = 1.0;
  for (j = 0; j < n; ++j) E[j] = 1.0;

  if (qsize > 0) {
    /* collapse: within each column, the entries falling in one cone are all
     * replaced by their largest magnitude and moved to the cone's first row
     * (ruiz_equil_common.h:29-67).  The scan that finds the maximum may run
     * past the column's end into the next column, exactly as the reference's
     * does (its bound is the total nnz, not the column end). */
    for (j = 0; j < n; ++j) {
      oidx start = f + l, k = Ap[j];
      cone = 0;
      while (k < Ap[j + 1] && Ai[k] < start) k++;
      while (k < Ap[j + 1]) {
        double mx = 0.0;
        oidx s = k;
        while (s < nnz && start <= Ai[s] && Ai[s] < start + q[cone]) {
          double a = fabs(cv[s]);
          mx = mx > a ? mx : a;
          s++;
        }
        while (k < nnz && start <= Ai[k] && Ai[k] < start + q[cone]) {
          cv[k] = mx;
          ci[k] = start;
          k++;
        }
        start += q[cone++];
      }
    }
    off = f + l;
    for (cone = 0; cone < qsize; ++cone) {
      double mx = 0.0;
      for (i = 0; i < q[cone]; ++i) {
        double a = fabs(cb[off + i]);
        mx = mx > a ? mx : a;
      }
      for (i = 0; i < q[cone]; ++i) cb[off + i] = mx;
      off += q[cone];
    }
  }

  for (it = 0; it < RUIZ_PASSES; ++it) {
    for (j = 0; j < n; ++j) {
      for (p = Ap[j]; p < Ap[j + 1]; ++p) {
        double a = fabs(cv[p]) * E[j];
        rowmax[ci[p]] = rowmax[ci[p]] > a ? rowmax[ci[p]] : a;
      }
      {
        double a = fabs(c[j]) * E[j];
        rlast = rlast > a ? rlast : a;
      }
    }
    for (i = 0; i < m; ++i) {
      double a = fabs(cb[i]) * elast;
      rowmax[i] = rowmax[i] > a ? rowmax[i] : a;
    }
    off = f + l;
    for (cone = 0; cone < qsize; ++cone) {
      for (i = 0; i < q[cone]; ++i) rowmax[off + i] = rowmax[off];
      off += q[cone];
    }
    for (i = 0; i < m; ++i) {
      D[i] = fabs(rowmax[i]) > 1e-6 ? sqrt(D[i] / rowmax[i]) : 1.0;
      rowmax[i] = 0.0;
    }
    dlast = fabs(rlast) > 1e-6 ? sqrt(dlast / rlast) : 1.0;
    rlast = 0.0;

    for (j = 0; j < n; ++j) {
      for (p = Ap[j]; p < Ap[j + 1]; ++p) {
        double a = fabs(cv[p]) * D[ci[p]];
        colmax[j] = colmax[j] > a ? colmax[j] : a;
      }
      {
        double a = fabs(c[j]) * dlast;
        colmax[j] = colmax[j] > a ? colmax[j] : a;
      }
    }
    for (i = 0; i < m; ++i) {
      double a = fabs(cb[i]) * D[i];
      clast = clast > a ? clast : a;
    }
    for (j = 0; j < n; ++j) {
      E[j] = fabs(colmax[j]) > 1e-6 ? sqrt(E[j] / colmax[j]) : 1.0;
      colmax[j] = 0.0;
    }
    elast = fabs(clast) > 1e-6 ? sqrt(elast / clast) : 1.0;
    clast = 0.0;
  }
  for (j = 0; j < n; ++j)
    for (p = Ap[j]; p < Ap[j + 1]; ++p) Aw[p] = D[Ai[p]] * Ax[p] * E[j];
  free(cv);
  free(ci);
  free(cb);
  free(rowmax);
  free(colmax);
}

/* ---------------------------------------------------------------------- */
/* Whole solve.  Mirrors pdos() with the indirect plug-in. */
typedef struct {
  oidx admm_iters;   /* value of the loop index when the loop ended */
  oidx cg_iters;     /* total CG iterations over the solve */
  int solved;        /* 1 = "Solved", 0 = "Indeterminate" */
  double p_res, d_res, p_obj, d_obj, eta, lambda;
} OracleInfo;

/* scaling: 0 = none (NORMALIZE=0), 1 = default 2-norm (common.h),
 * 2 = Ruiz (ruiz_equil_common.h).  Returns 0 on success. */
int oracle_solve(oidx m, oidx n, const oidx *Ap, const oidx *Ai,
                 const double *Ax, const double *b, const double *c, oidx f,
                 oidx l, oidx qsize, const oidx *q, oidx max_iters,
                 oidx cg_max_its, double eps_abs, double alpha_relax,
                 double cg_tol, int scaling, const double *x0,
                 const double *y0, const double *s0, double *x_out,
                 double *s_out, double *y_out, OracleInfo *info) {
  oidx nnz = Ap[n], i, it, cg;
  oidx big = m > n ? m : n;
  double *D = (double *)malloc(sizeof(double) * (size_t)(m > 0 ? m : 1));
  double *E = (double *)malloc(sizeof(double) * (size_t)(n > 0 ? n : 1));
  double *Aw = (double *)malloc(sizeof(double) * (size_t)(nnz > 0 ? nnz : 1));
  double *bw = (double *)malloc(sizeof(double) * (size_t)(m > 0 ? m : 1));
  double *cw = (double *)malloc(sizeof(double) * (size_t)(n > 0 ? n : 1));
  double *x = (double *)calloc((size_t)(n > 0 ? n : 1), sizeof(double));
  double *st = (double *)calloc((size_t)(big > 0 ? big : 1), sizeof(double));
  double *s = (double *)calloc((size_t)(m > 0 ? m : 1), sizeof(double));
  double *y = (double *)calloc((size_t)(m > 0 ? m : 1), sizeof(double));
  double *u = (double *)calloc((size_t)(m > 0 ? m : 1), sizeof(double));
  double *pv = (double *)calloc((size_t)(n > 0 ? n : 1), sizeof(double));
  double *qv = (double *)calloc((size_t)(n > 0 ? n : 1), sizeof(double));
  oidx *Rp = (oidx *)malloc(sizeof(oidx) * (size_t)(m + 1));
  oidx *Rj = (oidx *)malloc(sizeof(oidx) * (size_t)(nnz > 0 ? nnz : 1));
  double *Rx = (double *)malloc(sizeof(double) * (size_t)(nnz > 0 ? nnz : 1));
  double pscale, dscale, lambda, tol_sq = cg_tol * cg_tol;
  int solved = 0, rc = 0;
  OracleInfo inf;
  memset(&inf, 0, sizeof(inf));
  inf.p_res = inf.d_res = inf.p_obj = inf.d_obj = inf.eta = -1;
  if (!D || !E || !Aw || !bw || !cw || !x || !st || !s || !y || !u || !pv ||
      !qv || !Rp || !Rj || !Rx) {
    rc = -1;
    goto done;
  }

  /* DIMACS denominators come from the caller's b and c (pdos.c:76-77) */
  pscale = 1.0 + sqrt(sumsq(b, m));
  dscale = 1.0 + sqrt(sumsq(c, n));

  if (x0) memcpy(x, x0, sizeof(double) * (size_t)n);
  if (s0) memcpy(s, s0, sizeof(double) * (size_t)m);
  if (y0) memcpy(y, y0, sizeof(double) * (size_t)m);

  if (scaling == 0) {
    for (i = 0; i < m; ++i) D[i] = 1.0;
    for (i = 0; i < n; ++i) E[i] = 1.0;
    memcpy(Aw, Ax, sizeof(double) * (size_t)nnz);
    memcpy(bw, b, sizeof(double) * (size_t)m);
    memcpy(cw, c, sizeof(double) * (size_t)n);
  } else {
    if (scaling == 1)
      oracle_scale_default(m, n, Ap, Ai, Ax, f, l, qsize, q, D, E, Aw);
    else
      oracle_scale_ruiz(m, n, Ap, Ai, Ax, b, c, f, l, qsize, q, D, E, Aw);
    for (i = 0; i < n; ++i) cw[i] = c[i] * E[i];
    for (i = 0; i < m; ++i) bw[i] = b[i] * D[i];
    for (i = 0; i < m; ++i) y[i] /= D[i];
    for (i = 0; i < n; ++i) x[i] /= E[i];
    for (i = 0; i < m; ++i) s[i] *= D[i];
  }
  {
    double guard = scaling == 2 ? 1e-6 : 1e-15; /* ruiz :288, common.h:182 */
    lambda = (guard + sqrt(sumsq(bw, m))) / (guard + sqrt(sumsq(cw, n)));
  }
  for (i = 0; i < n; ++i) {
    E[i] *= SQRT_RATIO_;
    cw[i] *= SQRT_RATIO_;
    x[i] /= SQRT_RATIO_;
  }
  for (i = 0; i < nnz; ++i) Aw[i] *= SQRT_RATIO_;
  if (oracle_csc_to_csr(m, n, Ap, Ai, Aw, Rp, Rj, Rx)) {
    rc = -1;
    goto done;
  }
  inf.lambda = lambda;

  for (it = 0; it < max_iters; ++it) {
    double pres, dres, pobj, dobj, eta;
    /* primal residual ||(Ax + s - b)/D|| (linAlg.h:158-175) */
    for (i = 0; i < m; ++i) st[i] = s[i] - bw[i];
    oracle_gather_mv(m, Rp, Rj, Rx, x, 1.0, st, 1);
    for (i = 0; i < m; ++i) st[i] /= D[i];
    pres = sqrt(sumsq(st, m));
    /* dual residual ||(A'y + c)/E|| (linAlg.h:178-191) */
    memcpy(st, cw, sizeof(double) * (size_t)n);
    oracle_gather_mv(n, Ap, Ai, Aw, y, 1.0, st, 1);
    for (i = 0; i < n; ++i) st[i] /= E[i];
    dres = sqrt(sumsq(st, n));
    pobj = dot(cw, x, n);
    dobj = -dot(bw, y, m);
    eta = fabs(pobj - dobj);
    inf.p_res = pres;
    inf.d_res = dres;
    inf.p_obj = pobj;
    inf.d_obj = dobj;
    inf.eta = eta;
    if (pres < eps_abs * pscale && dres < eps_abs * dscale &&
        eta < eps_abs * (1.0 + fabs(pobj) + fabs(dobj))) {
      solved = 1;
      break;
    }

    /* projectLinSys (indirect/private.c:106-118) */
    for (i = 0; i < m; ++i) st[i] = s[i] + lambda * y[i] - bw[i];
    {
      double qold, qnew = 0, step, ratio;
      memcpy(u, st, sizeof(double) * (size_t)m);
      for (i = 0; i < n; ++i) qv[i] = -lambda * cw[i];
      oracle_gather_mv(m, Rp, Rj, Rx, x, 1.0, u, 1);
      oracle_gather_mv(n, Ap, Ai, Aw, u, -1.0, qv, 1);
      memcpy(pv, qv, sizeof(double) * (size_t)n);
      qold = sumsq(qv, n);
      cg = 0;
      if (qold > tol_sq) {
        for (cg = 0; cg < cg_max_its; ++cg) {
          oracle_gather_mv(m, Rp, Rj, Rx, pv, 1.0, u, 0);
          memcpy(st, pv, sizeof(double) * (size_t)n);
          oracle_gather_mv(n, Ap, Ai, Aw, u, 1.0, st, 1);
          step = qold / dot(pv, st, n);
          for (i = 0; i < n; ++i) x[i] += step * pv[i];
          for (i = 0; i < n; ++i) qv[i] += -step * st[i];
          qnew = sumsq(qv, n);
          if (qnew < tol_sq) {
            ++cg;
            break;
          }
          ratio = qnew / qold;
          for (i = 0; i < n; ++i) pv[i] *= ratio;
          for (i = 0; i < n; ++i) pv[i] += 1 * qv[i];
          qold = qnew;
        }
      }
      inf.cg_iters += cg;
    }
    memcpy(st, bw, sizeof(double) * (size_t)m);
    oracle_gather_mv(m, Rp, Rj, Rx, x, -1.0, st, 1);

    /* relax, cone step and dual update (pdos.c:232-249, :296-303) */
    for (i = 0; i < m; ++i)
      st[i] = alpha_relax * st[i] + (1.0 - alpha_relax) * s[i];
    for (i = 0; i < m; ++i) s[i] = st[i] - lambda * y[i];
    oracle_proj_cone(s, f, l, qsize, q);
    for (i = 0; i < m; ++i) y[i] += (s[i] - st[i]) / lambda;
  }
  inf.admm_iters = it;
  inf.solved = solved;

  /* unscale (pdos.c:261-294) */
  for (i = 0; i < n; ++i) x_out[i] = E[i] * x[i];
  for (i = 0; i < m; ++i) y_out[i] = D[i] * y[i];
  for (i = 0; i < m; ++i) s_out[i] = s[i] / D[i];

done:
  if (info) *info = inf;
  free(D); free(E); free(Aw); free(bw); free(cw); free(x); free(st);
  free(s); free(y); free(u); free(pv); free(qv); free(Rp); free(Rj); free(Rx);
  return rc;
}

/* Size of the info record, so the Python side can check its mirror. */
int oracle_info_size(void) { return (int)sizeof(OracleInfo); }
