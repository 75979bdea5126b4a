// The reference's three entry points (pdos.h:85-87) on top of the C-ABI
// layer.  Compiled once with PDOS_DLONG (idxint = long, libpdosindir.so) and
// once without (idxint = int, libpdosindir_i32.so).
#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/pdos_gpu.h"

namespace pdosgpu {
int fail(int code, const std::string &msg);  // sets pdos_gpu_last_error()
}

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


// Data / Cone / Params of the reference (pdos.h:15-35, cones.h:8-13) as one
// pdosgpu_problem; false for the inputs the reference rejects (pdos.c:61-63)
// or cannot index.
bool to_problem(const Data *d, const Cone *k, Wide &w, pdosgpu_problem &pr) {
  if (d == NULL || k == NULL) return false;
  if (d->p == NULL || d->Ap == NULL || d->n <= 0 || d->m <= 0) return false;
  widen(d, k, w);
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
  return true;
}

// A Sol allocated as pdos() allocates it (pdos.c:121, PDOS_malloc = malloc).
Sol *new_sol(idxint n, idxint m) {
  Sol *sol = (Sol *)malloc(sizeof(Sol));
  if (!sol) return NULL;
  std::memset(sol, 0, sizeof(Sol));
  sol->n = n;
  sol->m = m;
  sol->x = (double *)malloc(sizeof(double) * n);
  sol->s = (double *)malloc(sizeof(double) * m);
  sol->y = (double *)malloc(sizeof(double) * m);
  if (!sol->x || !sol->s || !sol->y) freeSol(&sol);
  return sol;
}

// exactly the reference's two status strings (pdos.c:255-258)
void set_status(Sol *sol, int solved) {
  std::strncpy(sol->status, solved ? "Solved" : "Indeterminate", sizeof(sol->status) - 1);
}

// Nonzeros up to which pdos() solves a problem with one CTA of the batch
// kernel, and above that up to which with one 8-CTA cluster: every ADMM
// iteration then runs inside one launch, where the grid engine launches
// 2k + 4 kernels per iteration (k CG steps) and waits on each.  Measured in
// FP64 on GB300 (solve time, set-up excluded), grid / one CTA / cluster:
// 1,308 nonzeros 7.9 / 2.8 / 3.0 ms; 2,761: 302 / 124 / 126 ms; 23,201:
// 307 / 190 / 88 ms; 86,401: 218 / 523 / 158 ms; 332,801: 360 / 1,925 /
// 391 ms.  One SM issues only about two FP64 FMAs per clock, so a single CTA
// falls behind early; a cluster has eight SMs.
constexpr int64_t kOneCtaMaxNnz = 4096;
// Nonzeros up to which pdos() solves on one 8-CTA cluster (above
// kOneCtaMaxNnz); its gather vector must fit one CTA's shared memory.
constexpr int64_t kClusterMaxNnz = 200000;
// CTA size of that cluster: 256 threads below this many nonzeros, else 512.
constexpr int64_t kClusterSmallNnz = 131072;

// pdos() through the one-CTA path: a batch of one instance, run to its stop
// test in one launch of the persistent kernel (CTA size by size class).
Sol *solve_one_cta(const Data *d, const pdosgpu_problem &pr, const pdosgpu_options *opt, pdosgpu_info *info,
                   bool cluster) {
  pdosgpu_options o;
  pdosgpu_default_options(&o);
  if (opt) o = *opt;
  o.batch_clusters = cluster ? 1 : 0;
  pdosgpu_batch *b = NULL;
  if (pdosgpu_batch_setup(&pr, 1, &o, 0, &b) != PDOSGPU_OK) return NULL;
  Sol *sol = NULL;
  pdosgpu_info inf;
  int rc = PDOSGPU_OK;
  if (cluster && pr.Ap[pr.n] < kClusterSmallNnz) {
    const int blocks[5] = {256, 256, 256, 256, 256};
    rc = pdosgpu_batch_set_blocks(b, blocks);
  }
  if (rc == PDOSGPU_OK && pdosgpu_batch_solve(b) == PDOSGPU_OK) {
    sol = new_sol(d->n, d->m);
    if (sol && pdosgpu_batch_fetch(b, 0, 1, sol->x, sol->s, sol->y, &inf) != PDOSGPU_OK) {
      freeSol(&sol);
    } else if (sol) {
      set_status(sol, inf.solved);
      if (info) *info = inf;
    }
  }
  pdosgpu_batch_free(b);
  return sol;
}


// 0: grid engine, 1: one CTA, 2: one cluster.
int pick_engine(const pdosgpu_problem &pr, const pdosgpu_options *opt) {
  const int engine = opt ? opt->engine : PDOSGPU_ENGINE_AUTO;
  if (engine == PDOSGPU_ENGINE_GRID) return 0;
  const bool fits = pr.m <= 65535 && pr.n <= 65535 && !pr.verbose &&
                    !(pr.normalize && opt && opt->scaling == PDOSGPU_SCALE_RUIZ);
  const size_t elem = (opt && opt->precision == PDOSGPU_FP32) ? 4 : 8;
  const bool gather_fits = (size_t)std::max(pr.m, pr.n) * elem <= (size_t)225 * 1024;
  if (engine == PDOSGPU_ENGINE_CTA) return fits ? 1 : 0;
  if (engine == PDOSGPU_ENGINE_CLUSTER) return fits && gather_fits ? 2 : 0;
  const int64_t nnz = pr.Ap[pr.n];
  if (fits && nnz <= kOneCtaMaxNnz) return 1;
  if (fits && gather_fits && nnz <= kClusterMaxNnz) return 2;
  return 0;
}

}  // namespace

extern "C" {

Sol *pdos_ex(const Data *d, const Cone *k, const pdosgpu_options *opt, pdosgpu_info *info) {
  Wide w;
  pdosgpu_problem pr;
  if (!to_problem(d, k, w, pr)) return NULL;
  if (opt && (opt->engine < PDOSGPU_ENGINE_AUTO || opt->engine > PDOSGPU_ENGINE_CLUSTER)) {
    pdosgpu::fail(PDOSGPU_EINVAL, "unknown engine");
    return NULL;
  }
  const int engine = pick_engine(pr, opt);
  if (engine > 0) return solve_one_cta(d, pr, opt, info, engine == 2);
  pdosgpu_work *work = NULL;
  if (pdosgpu_setup(&pr, opt, &work) != PDOSGPU_OK) return NULL;
  Sol *sol = NULL;
  if (pdosgpu_solve(work) == PDOSGPU_OK) {
    sol = new_sol(d->n, d->m);
    pdosgpu_info inf;
    if (sol && pdosgpu_fetch(work, sol->x, sol->s, sol->y, &inf) != PDOSGPU_OK) {
      freeSol(&sol);
    } else if (sol) {
      set_status(sol, inf.solved);
      if (info) *info = inf;
    }
  }
  pdosgpu_free(work);
  return sol;
}

int pdos_batch(const Data *const *d, const Cone *const *k, int64_t count,
               const pdosgpu_options *opt, Sol **sols, pdosgpu_info *info) {
  if (!d || !k || !sols || count <= 0) return PDOSGPU_EINVAL;
  for (int64_t i = 0; i < count; ++i) sols[i] = NULL;
  std::vector<Wide> w(count);
  std::vector<pdosgpu_problem> pr(count);
  for (int64_t i = 0; i < count; ++i)
    if (!to_problem(d[i], k[i], w[i], pr[i])) return PDOSGPU_EINVAL;
  pdosgpu_batch *b = NULL;
  int rc = pdosgpu_batch_setup(pr.data(), count, opt, 0, &b);
  if (rc != PDOSGPU_OK) return rc;
  rc = pdosgpu_batch_solve(b);
  int64_t N = 0, M = 0;
  if (rc == PDOSGPU_OK) rc = pdosgpu_batch_sizes(b, NULL, &N, &M, NULL);
  std::vector<double> x, s, y;
  std::vector<pdosgpu_info> inf;
  if (rc == PDOSGPU_OK) {
    x.resize(N);
    s.resize(M);
    y.resize(M);
    inf.resize(count);
    rc = pdosgpu_batch_fetch(b, 0, count, x.data(), s.data(), y.data(), inf.data());
  }
  pdosgpu_batch_free(b);
  int64_t c0 = 0, r0 = 0;
  for (int64_t i = 0; i < count && rc == PDOSGPU_OK; ++i) {
    const int64_t n = d[i]->n, m = d[i]->m;
    sols[i] = new_sol(d[i]->n, d[i]->m);
    if (!sols[i]) {
      rc = PDOSGPU_ENOMEM;
      break;
    }
    std::memcpy(sols[i]->x, &x[c0], sizeof(double) * n);
    std::memcpy(sols[i]->s, &s[r0], sizeof(double) * m);
    std::memcpy(sols[i]->y, &y[r0], sizeof(double) * m);
    set_status(sols[i], inf[i].solved);
    if (info) info[i] = inf[i];
    c0 += n;
    r0 += m;
  }
  if (rc != PDOSGPU_OK)
    for (int64_t i = 0; i < count; ++i) freeSol(&sols[i]);
  return rc;
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
