// C API of the batched solver (pdosgpu_batch_* in include/pdos_gpu.h): a
// batch owns one engine of its precision (batch_engine.cuh), created here
// and driven through the engine's virtual interface.
#include "batch_engine.cuh"

struct pdosgpu_batch {
  std::unique_ptr<pdosgpu::batch::BatchBase> engine;
};

using namespace pdosgpu;

extern "C" {

int pdosgpu_batch_create(const pdosgpu_options *opt, int iters_per_launch, pdosgpu_batch **out) {
  if (!out) return fail(PDOSGPU_EINVAL, "NULL argument");
  *out = nullptr;
  int devs = 0;
  cudaError_t e = cudaGetDeviceCount(&devs);
  if (e != cudaSuccess || devs == 0)
    return fail(PDOSGPU_ENOTSUP, std::string("no CUDA device: ") + cudaGetErrorString(e));
  pdosgpu_options o;
  pdosgpu_default_options(&o);
  if (opt) o = *opt;
  auto w = new (std::nothrow) pdosgpu_batch();
  if (!w) return fail(PDOSGPU_ENOMEM, "host allocation failed");
  int rc = PDOSGPU_OK;
  if (iters_per_launch <= 0) iters_per_launch = INT32_MAX;  // each instance runs to its end
  if (o.precision == PDOSGPU_FP32) {
    auto b = batch::make_batch_engine_f32();
    rc = b->create(o, iters_per_launch);
    if (rc == PDOSGPU_OK) w->engine = std::move(b);
  } else if (o.precision == PDOSGPU_FP64) {
    auto b = batch::make_batch_engine_f64();
    rc = b->create(o, iters_per_launch);
    if (rc == PDOSGPU_OK) w->engine = std::move(b);
  } else {
    rc = fail(PDOSGPU_EINVAL, "unknown precision");
  }
  if (rc != PDOSGPU_OK) {
    delete w;
    return rc;
  }
  *out = w;
  return PDOSGPU_OK;
}

int pdosgpu_batch_append(pdosgpu_batch *b, const pdosgpu_problem *probs, int64_t count) {
  if (!b || !b->engine || !probs) return fail(PDOSGPU_EINVAL, "NULL argument");
  return b->engine->append(probs, count);
}

int pdosgpu_batch_commit(pdosgpu_batch *b) {
  if (!b || !b->engine) return fail(PDOSGPU_EINVAL, "NULL batch");
  return b->engine->commit();
}

int pdosgpu_batch_setup(const pdosgpu_problem *probs, int64_t count, const pdosgpu_options *opt,
                        int iters_per_launch, pdosgpu_batch **out) {
  if (!probs || !out) return fail(PDOSGPU_EINVAL, "NULL argument");
  *out = nullptr;
  pdosgpu_batch *w = nullptr;
  PDOS_TRY(pdosgpu_batch_create(opt, iters_per_launch, &w));
  int rc = pdosgpu_batch_append(w, probs, count);
  if (rc == PDOSGPU_OK) rc = pdosgpu_batch_commit(w);
  if (rc != PDOSGPU_OK) {
    delete w;
    return rc;
  }
  *out = w;
  return PDOSGPU_OK;
}

// A batch in use: created and committed.
static int ready(pdosgpu_batch *b) {
  if (!b || !b->engine) return fail(PDOSGPU_EINVAL, "NULL batch");
  if (!b->engine->committed) return fail(PDOSGPU_EINVAL, "the batch is not committed (pdosgpu_batch_commit)");
  return PDOSGPU_OK;
}

int pdosgpu_batch_solve(pdosgpu_batch *b) {
  PDOS_TRY(ready(b));
  return b->engine->solve(-1);
}

int pdosgpu_batch_launch(pdosgpu_batch *b, int64_t launches) {
  PDOS_TRY(ready(b));
  if (launches < 0) return fail(PDOSGPU_EINVAL, "launches must be nonnegative");
  return b->engine->solve(launches);
}

int pdosgpu_batch_reset(pdosgpu_batch *b) {
  PDOS_TRY(ready(b));
  return b->engine->reset();
}

int pdosgpu_batch_warm_start(pdosgpu_batch *b, const double *x0, const double *y0, const double *s0) {
  PDOS_TRY(ready(b));
  return b->engine->warm_start(x0, y0, s0);
}

int pdosgpu_batch_fetch(pdosgpu_batch *b, int64_t first, int64_t count, double *x, double *s,
                        double *y, pdosgpu_info *info) {
  PDOS_TRY(ready(b));
  return b->engine->fetch(first, count, x, s, y, info);
}

int64_t pdosgpu_batch_done(pdosgpu_batch *b) {
  PDOS_TRY(ready(b));
  return b->engine->done_count();
}

int pdosgpu_batch_tune(pdosgpu_batch *b, int iters, int *blocks) {
  PDOS_TRY(ready(b));
  return b->engine->tune(iters, blocks);
}

int pdosgpu_batch_time_products(pdosgpu_batch *b, int reps, double *ms, double *bytes) {
  PDOS_TRY(ready(b));
  return b->engine->time_products(reps, ms, bytes);
}

int pdosgpu_batch_set_blocks(pdosgpu_batch *b, const int *blocks) {
  PDOS_TRY(ready(b));
  if (!blocks) return fail(PDOSGPU_EINVAL, "NULL argument");
  return b->engine->set_blocks(blocks);
}

int pdosgpu_batch_tune_layout(const pdosgpu_problem *probs, int64_t count, const pdosgpu_options *opt,
                              int64_t sample, int iters, int *long_row, int *piece) {
  if (!probs || !long_row || !piece) return fail(PDOSGPU_EINVAL, "NULL argument");
  if (count <= 0 || sample <= 0 || iters <= 0) return fail(PDOSGPU_EINVAL, "count, sample and iters must be positive");
  pdosgpu_options o;
  pdosgpu_default_options(&o);
  if (opt) o = *opt;
  const int64_t ns = std::min(count, sample);
  std::vector<pdosgpu_problem> pick(ns);
  for (int64_t k = 0; k < ns; ++k) pick[k] = probs[ns == 1 ? 0 : k * (count - 1) / (ns - 1)];
  const int rows[] = {64, 128, 256}, pieces[] = {256, 512, 1024, 2048};
  double best = -1.0;
  for (int lr : rows) {
    for (int pc : pieces) {
      o.batch_long_row = lr;
      o.batch_piece = pc;
      pdosgpu_batch *b = nullptr;
      PDOS_TRY(pdosgpu_batch_setup(pick.data(), ns, &o, 0, &b));
      double ms = 0.0;
      int rc = b->engine->time_products(iters, &ms, nullptr);
      delete b;
      PDOS_TRY(rc);
      if (best < 0.0 || ms < best) {
        best = ms;
        *long_row = lr;
        *piece = pc;
      }
    }
  }
  return PDOSGPU_OK;
}

int pdosgpu_batch_sizes(pdosgpu_batch *b, int64_t *count, int64_t *n, int64_t *m, int64_t *nnz) {
  if (!b || !b->engine) return fail(PDOSGPU_EINVAL, "NULL batch");
  if (count) *count = b->engine->count;
  if (n) *n = b->engine->total_n;
  if (m) *m = b->engine->total_m;
  if (nnz) *nnz = b->engine->total_nnz;
  return PDOSGPU_OK;
}

int pdosgpu_batch_layouts(pdosgpu_batch *b, int64_t *groups, int64_t *instances, int64_t *bytes) {
  if (!b || !b->engine) return fail(PDOSGPU_EINVAL, "NULL batch");
  if (groups) *groups = b->engine->family_groups;
  if (instances) *instances = b->engine->family_instances;
  if (bytes) *bytes = b->engine->layout_bytes;
  return PDOSGPU_OK;
}

int pdosgpu_batch_classes(pdosgpu_batch *b, int32_t *cls) {
  PDOS_TRY(ready(b));
  if (!cls) return fail(PDOSGPU_EINVAL, "NULL output");
  for (int64_t i = 0; i < b->engine->count; ++i) cls[i] = b->engine->instance_class(i);
  return PDOSGPU_OK;
}

void *pdosgpu_batch_stream(pdosgpu_batch *b) {
  return (b && b->engine) ? b->engine->stream() : nullptr;
}

void pdosgpu_batch_free(pdosgpu_batch *b) { delete b; }

}  // extern "C"
