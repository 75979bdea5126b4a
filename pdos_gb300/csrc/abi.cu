// The reference's three entry points (pdos.h:85-87) on top of the C-ABI
// layer.  Compiled once with PDOS_DLONG (idxint = long, libpdosindir.so) and
// once without (idxint = int, libpdosindir_i32.so).
#include <cstdlib>
#include <cstring>
#include <vector>

#include "../../include/pdos_gpu.h"

namespace {

// Widen idxint arrays to int64 when idxint is narrower (no copy otherwise).
struct Wide {
  std::vector<int64_t> Ai, Ap, q;
  const int64_t *ai = nullptr, *ap = nullptr, *qq = nullptr;
};

void widen(const Data *d, const Cone *k, Wide &w) {
  const int64_t nnz = (int64_t)d->Ap[d->n];
  if (sizeof(idxint) == sizeof(int64_t)) {
    w.ai = reinterpret_cast<const int64_t *>(d->Ai);
    w.ap = reinterpret_cast<const int64_t *>(d->Ap);
    w.qq = reinterpret_cast<const int64_t *>(k->q);
    return;
  }
  w.Ap.assign(d->Ap, d->Ap + d->n + 1);
  if (nnz > 0 && d->Ai) w.Ai.assign(d->Ai, d->Ai + nnz);
  if (k->qsize > 0 && k->q) w.q.assign(k->q, k->q + k->qsize);
  w.ap = w.Ap.data();
  w.ai = w.Ai.empty() ? nullptr : w.Ai.data();
  w.qq = w.q.empty() ? nullptr : w.q.data();
}

}  // namespace

extern "C" {

Sol *pdos_ex(const Data *d, const Cone *k, const pdosgpu_options *opt, pdosgpu_info *info) {
  if (d == NULL || k == NULL) return NULL;  // pdos.c:61-63
  if (d->p == NULL || d->Ap == NULL || d->n <= 0 || d->m <= 0) return NULL;
  Wide w;
  widen(d, k, w);
  pdosgpu_problem pr;
  std::memset(&pr, 0, sizeof(pr));
  pr.n = d->n;
  pr.m = d->m;
  pr.Ax = d->Ax;
  pr.Ai = w.ai;
  pr.Ap = w.ap;
  pr.b = d->b;
  pr.c = d->c;
  pr.x0 = d->x;
  pr.y0 = d->y;
  pr.s0 = d->s;
  pr.f = k->f;
  pr.l = k->l;
  pr.qsize = k->qsize;
  pr.q = w.qq;
  pr.max_iters = d->p->MAX_ITERS;
  pr.cg_max_its = d->p->CG_MAX_ITS;
  pr.eps_abs = d->p->EPS_ABS;
  pr.alpha = d->p->ALPHA;
  pr.cg_tol = d->p->CG_TOL;
  pr.verbose = d->p->VERBOSE;
  pr.normalize = d->p->NORMALIZE;

  pdosgpu_work *work = NULL;
  if (pdosgpu_setup(&pr, opt, &work) != PDOSGPU_OK) return NULL;
  Sol *sol = NULL;
  if (pdosgpu_solve(work) == PDOSGPU_OK) {
    sol = (Sol *)malloc(sizeof(Sol));
    if (sol) {
      std::memset(sol, 0, sizeof(Sol));
      sol->n = d->n;
      sol->m = d->m;
      sol->x = (double *)malloc(sizeof(double) * d->n);
      sol->s = (double *)malloc(sizeof(double) * d->m);
      sol->y = (double *)malloc(sizeof(double) * d->m);
      pdosgpu_info inf;
      if (!sol->x || !sol->s || !sol->y ||
          pdosgpu_fetch(work, sol->x, sol->s, sol->y, &inf) != PDOSGPU_OK) {
        freeSol(&sol);
      } else {
        // exactly the reference's two status strings (pdos.c:255-258)
        std::strncpy(sol->status, inf.solved ? "Solved" : "Indeterminate", sizeof(sol->status) - 1);
        if (info) *info = inf;
      }
    }
  }
  pdosgpu_free(work);
  return sol;
}

Sol *pdos(const Data *d, const Cone *k) { return pdos_ex(d, k, NULL, NULL); }

void freeData(Data **d, Cone **k) {  // pdos.c:134-152
  if (d && *d) {
    Data *p = *d;
    free(p->b);
    free(p->c);
    free(p->Ax);
    free(p->Ai);
    free(p->Ap);
    free(p->p);
    free(p->x);
    free(p->y);
    free(p->s);
    free(p);
  }
  if (k && *k) {
    free((*k)->q);
    free(*k);
  }
  if (d) *d = NULL;
  if (k) *k = NULL;
}

void freeSol(Sol **sol) {  // pdos.c:154-164
  if (sol && *sol) {
    free((*sol)->x);
    free((*sol)->y);
    free((*sol)->s);
    free(*sol);
  }
  if (sol) *sol = NULL;
}

}  // extern "C"
