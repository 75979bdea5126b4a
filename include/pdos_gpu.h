/*
 * pdos_gpu.h -- the C-ABI layer under pdos() and the GPU-only extensions.
 *
 * Everything here takes plain pointers and sizes.  The reference has no GPU
 * layer; each entry point names the reference code whose work it carries.
 * All functions return PDOSGPU_OK (0) or a negative status; the last error
 * message of the calling thread is in pdos_gpu_last_error().
 */
#ifndef PDOS_GB300_PDOS_GPU_H
#define PDOS_GB300_PDOS_GPU_H

#include <stdint.h>

#include "pdos.h"

#ifdef __cplusplus
extern "C" {
#endif

enum {
  PDOSGPU_OK = 0,
  PDOSGPU_EINVAL = -1,   /* bad sizes, indices, cone table or parameters */
  PDOSGPU_ENOMEM = -2,   /* host or device allocation failed */
  PDOSGPU_ECUDA = -3,    /* a CUDA call failed */
  PDOSGPU_ENOTSUP = -4   /* no usable GPU / unsupported request */
};

enum { PDOSGPU_FP64 = 0, PDOSGPU_FP32 = 1 };          /* storage/arithmetic */
enum { PDOSGPU_SCALE_2NORM = 0, PDOSGPU_SCALE_RUIZ = 1 }; /* NORMALIZE=1 kind */
enum { PDOSGPU_BATCH_SHARE = 0, PDOSGPU_BATCH_OWN = 1 };  /* batch layouts */
enum { PDOSGPU_ENGINE_AUTO = 0, PDOSGPU_ENGINE_GRID = 1, PDOSGPU_ENGINE_CTA = 2, PDOSGPU_ENGINE_CLUSTER = 3 };

typedef struct {
  int precision;   /* PDOSGPU_FP64 (default): every operation in double, the
                      reference's arithmetic.  PDOSGPU_FP32: A, vectors and
                      SpMV in float; dot products, norms, CG scalars, the gap
                      and the objective accumulated in double. */
  int scaling;     /* equilibration used when NORMALIZE=1: PDOSGPU_SCALE_2NORM
                      (common.h:69-162, the reference's default build) or
                      PDOSGPU_SCALE_RUIZ (ruiz_equil_common.h:98-322) */
  int device;      /* CUDA device ordinal (default 0) */
  int batch_layouts; /* batches only: PDOSGPU_BATCH_SHARE (default) lets the
                        instances of a family -- one sparsity pattern, cone
                        table and sizes, values differing at no more than a
                        quarter of the nonzeros, NORMALIZE=0 -- share one
                        matrix layout, each keeping only its own values of
                        the entries that differ (same results, bit for bit);
                        PDOSGPU_BATCH_OWN gives every instance its own */
  int engine;      /* pdos() / pdos_ex() only: PDOSGPU_ENGINE_AUTO (default)
                      solves a small problem (m, n < 65,536, VERBOSE=0,
                      2-norm scaling) in one launch of the batch kernel --
                      one CTA running the whole ADMM loop for the smallest,
                      a cluster of 8 CTAs for mid-sized ones -- and any
                      other on the grid engine; PDOSGPU_ENGINE_GRID,
                      PDOSGPU_ENGINE_CTA and PDOSGPU_ENGINE_CLUSTER force
                      one of the three */
  int batch_long_row; /* batches only: rows with more nonzeros than this are
                         cut into warp-wide pieces, shorter ones share
                         32-row slices (0: 128; else a multiple of 4 in
                         [4, 1024]) */
  int batch_piece;    /* batches only: nonzeros per piece at most (0: 1,024;
                         else a multiple of 4 in [64, 16384]) */
  int batch_clusters; /* batches only: 0 (default) runs on clusters of 2 to 8
                         CTAs (fewer CTAs when there are more of them) only
                         the instances too large for one CTA's shared memory;
                         1 runs every instance whose gather vector fits
                         shared memory on an 8-CTA cluster */
} pdosgpu_options;

typedef struct {
  int64_t admm_iters;   /* ADMM iterations run (pdos.c:94 loop index at exit) */
  int64_t cg_iters;     /* CG iterations summed over the solve */
  int solved;           /* 1 = "Solved", 0 = "Indeterminate" */
  int diverged;         /* 1: a residual or the gap became NaN/Inf (e.g. FP32
                           storage overflowed); the solve stopped at that
                           iteration instead of running to MAX_ITERS, and the
                           status is "Indeterminate" */
  double p_res, d_res;  /* last DIMACS residuals (pdos.c:95-96), -1 if none */
  double p_obj, d_obj, eta;
  double lambda;        /* common.h:182 */
  double setup_ms;      /* host wall time of pdosgpu_setup */
  double solve_ms;      /* host wall time of the last pdosgpu_solve/iterate */
  int64_t kernel_launches; /* kernels launched by this workspace so far
                              (set-up excluded; graph nodes counted) */
} pdosgpu_info;

/* A problem with 64-bit indices in host memory: the fields of Data/Cone/
 * Params flattened (pdos.h:15-35, cones.h:8-13). */
typedef struct {
  int64_t n, m;
  const double *Ax;
  const int64_t *Ai, *Ap;
  const double *b, *c;
  const double *x0, *y0, *s0;   /* warm start, each may be NULL */
  int64_t f, l, qsize;
  const int64_t *q;
  int64_t max_iters, cg_max_its;
  double eps_abs, alpha, cg_tol;
  int64_t verbose, normalize;
} pdosgpu_problem;

typedef struct pdosgpu_work pdosgpu_work;

const char *pdos_gpu_last_error(void);
void pdosgpu_default_options(pdosgpu_options *opt);

/* Workspace set-up: copies the problem to the GPU, builds the CSR of A on
 * the device (cs_transpose, cs.c:146-168), equilibrates (common.h:35-218 /
 * ruiz_equil_common.h:98-322), sets lambda and the x-space ratio and
 * evaluates the residuals of the starting point.  Replaces initWork
 * (indirect/private.c:3-14). */
int pdosgpu_setup(const pdosgpu_problem *prob, const pdosgpu_options *opt,
                  pdosgpu_work **out);

/* Run ADMM iterations (pdos.c:94-120) until the DIMACS test passes or
 * MAX_ITERS iterations have run in total. */
int pdosgpu_solve(pdosgpu_work *w);

/* Run at most `iters` more ADMM iterations (stops early when solved or at
 * MAX_ITERS). */
int pdosgpu_iterate(pdosgpu_work *w, int64_t iters);

/* Restore the starting iterate (warm start or zeros); problem data and
 * scaling stay resident. */
int pdosgpu_reset(pdosgpu_work *w);

/* Copy the unscaled solution (pdos.c:251-294) to host arrays of n, m, m
 * doubles (any may be NULL) and fill *info (may be NULL). */
int pdosgpu_fetch(pdosgpu_work *w, double *x, double *s, double *y,
                  pdosgpu_info *info);

void pdosgpu_free(pdosgpu_work *w);

/* The CUDA stream (cudaStream_t) every kernel of this workspace runs on. */
void *pdosgpu_stream(pdosgpu_work *w);

/* Kernel timing for roofline reports: launch one of the iteration's SpMV
 * passes `reps` times back to back on the workspace stream between two CUDA
 * events and return the mean duration in ms.  which: 0 = CG A pass
 * (u = A p), 1 = CG A' pass (t = p + A'u), 2 = first A' pass on (y, u),
 * 3 = last A pass on x (each with its split-row combine kernel, if any);
 * 4 / 5 = the SpMV kernel alone of the CG A / A' pass.  Leaves the iterate
 * undefined: call pdosgpu_reset() before solving again. */
int pdosgpu_time_kernel(pdosgpu_work *w, int which, int reps, double *ms_per_launch);

/* Roofline support: the device's FP64 fused multiply-add rate (FMA/s),
 * measured with CUDA events on independent FMA chains over every SM.  The
 * FP64 SpMV of accumByScaledA/ATrans (linAlg.h:70-115) executes one FMA per
 * nonzero, so nnz / rate bounds its duration beside the HBM bound. */
int pdosgpu_fp64_fma_rate(int device, double *fma_per_s);

/* pdos() with explicit GPU options; info may be NULL. */
Sol *pdos_ex(const Data *d, const Cone *k, const pdosgpu_options *opt,
             pdosgpu_info *info);

/* ---- batches of independent problems ----------------------------------
 * Many problems of uneven sizes and cone profiles solved together: each
 * instance runs the reference's indirect ADMM (pdos.c:50-132 with
 * indirect/private.c:31-118) with its own parameters, lambda, scaling, CG
 * and stop test; one CTA solves one instance at a time and takes the next
 * one when it finishes.  Instances share NORMALIZE; Ruiz scaling is not
 * available for batches.  m and n of an instance must stay below 65,536
 * (16-bit instance-local indices).  Instances fall into five classes: four
 * by nonzeros, whose vectors a CTA stages in shared memory, and one for
 * instances whose max(m, n) + m + n (+ pieces of long rows) values exceed
 * 225 KB, staged in a global-memory region of their CTA instead. */
typedef struct pdosgpu_batch pdosgpu_batch;

/* Set up `count` problems (the work of pdosgpu_setup for each).
 * iters_per_launch: ADMM iterations each instance runs per kernel launch;
 * <= 0 runs every instance to its stop test or MAX_ITERS in one launch, so
 * that a CTA whose instance finishes takes the next one without waiting for
 * a launch boundary.  A positive value bounds a launch's duration (results
 * are identical either way). */
int pdosgpu_batch_setup(const pdosgpu_problem *probs, int64_t count,
                        const pdosgpu_options *opt, int iters_per_launch,
                        pdosgpu_batch **out);
/* The same set-up in steps, for batches too large to hold on the host at
 * once: create an empty batch, append problems in any number of calls (each
 * call's host arrays may be freed once it returns), then commit before the
 * first solve.  Each append sets its problems up on the device in one or
 * more waves (at most about 2^30 nonzeros, and a share of the free device
 * memory, per wave), keeping only the finished layouts and vectors, so the
 * whole batch may exceed 2^31 nonzeros.  pdosgpu_batch_setup is create +
 * append + commit; the results do not depend on how the problems were
 * split into appends.  The per-instance work is the set-up of
 * pdosgpu_setup (commonWorkInit, common.h:35-218; cs_transpose,
 * cs.c:146-168). */
int pdosgpu_batch_create(const pdosgpu_options *opt, int iters_per_launch,
                         pdosgpu_batch **out);
int pdosgpu_batch_append(pdosgpu_batch *b, const pdosgpu_problem *probs,
                         int64_t count);
int pdosgpu_batch_commit(pdosgpu_batch *b);
/* Launch until every instance has passed its stop test or run MAX_ITERS. */
int pdosgpu_batch_solve(pdosgpu_batch *b);
/* At most `launches` more launches (stops early when all are done). */
int pdosgpu_batch_launch(pdosgpu_batch *b, int64_t launches);
/* Restore every instance's starting iterate. */
int pdosgpu_batch_reset(pdosgpu_batch *b);
/* New starting iterates from DEVICE arrays in the caller's (unscaled)
 * units, stacked instance after instance (x: sum n, y and s: sum m); any
 * may be NULL to keep the current one.  Scales them as pdosgpu_setup scales
 * Data.x/y/s (common.h:147-161, :185-192) and resets the batch. */
int pdosgpu_batch_warm_start(pdosgpu_batch *b, const double *x0, const double *y0,
                             const double *s0);
/* Unscaled solutions (pdos.c:251-294) of instances [first, first+count)
 * into host arrays stacked the same way (any may be NULL), and one info
 * record per instance (may be NULL). */
int pdosgpu_batch_fetch(pdosgpu_batch *b, int64_t first, int64_t count, double *x,
                        double *s, double *y, pdosgpu_info *info);
/* Instances finished so far (negative on error). */
int64_t pdosgpu_batch_done(pdosgpu_batch *b);
/* Autotuner: times `iters` iterations of each size class at each CTA size
 * (128, 256, 512, 1024), keeps the fastest, resets the batch; blocks (may be
 * NULL) receives the choice for the five classes. */
int pdosgpu_batch_tune(pdosgpu_batch *b, int iters, int *blocks);
/* Layout autotuner: sets up batches of up to `sample` of the problems
 * (evenly spaced) with each candidate layout -- long-row cut 64, 128 or
 * 256 nonzeros, times pieces of 256, 512, 1,024 or 2,048 -- times `iters`
 * rounds of their two CG products (the SpMV pair of linAlg.h:70-115) and
 * returns the fastest pair in *long_row and *piece, for the options of the
 * batch proper.  The layout changes only how each row's sum is split among
 * warps, not the problems. */
int pdosgpu_batch_tune_layout(const pdosgpu_problem *probs, int64_t count,
                              const pdosgpu_options *opt, int64_t sample, int iters,
                              int *long_row, int *piece);
/* Roofline timing: the two CG products (u = A p, t = p + A'u) of every
 * instance, `reps` times, with nothing else; *ms = device time of the
 * launches, *bytes (may be NULL) = their algorithmic bytes (values and
 * indices of A and A', both pointer arrays, the vector gathered and the
 * vector written, per product).  Leaves the iterate untouched. */
int pdosgpu_batch_time_products(pdosgpu_batch *b, int reps, double *ms, double *bytes);
/* Set the CTA size of the five size classes explicitly (blocks[5]). */
int pdosgpu_batch_set_blocks(pdosgpu_batch *b, const int *blocks);
/* Number of instances and stacked sizes (any may be NULL). */
int pdosgpu_batch_sizes(pdosgpu_batch *b, int64_t *count, int64_t *n, int64_t *m,
                        int64_t *nnz);
/* Matrix layouts of the batch (any output may be NULL): family groups
 * sharing one layout, instances on shared layouts, and the device bytes of
 * every layout (tables, indices, values, the group members' own values). */
int pdosgpu_batch_layouts(pdosgpu_batch *b, int64_t *groups, int64_t *instances,
                          int64_t *bytes);
/* Size class of every instance (cls[count]): 0-3 by nonzeros (at most
 * 4,096 / 32,768 / 262,144 / more), vectors staged in shared memory; 4:
 * too large for shared memory, vectors staged in global memory. */
int pdosgpu_batch_classes(pdosgpu_batch *b, int32_t *cls);
void *pdosgpu_batch_stream(pdosgpu_batch *b);
void pdosgpu_batch_free(pdosgpu_batch *b);

/* ---- learned warm start --------------------------------------------------
 * A perceptron n_in -> hidden -> hidden -> n_out (ReLU) with BF16 weights
 * and activations, FP32 accumulation, FP32 master weights and Adam (beta1
 * 0.9, beta2 0.999, eps 1e-8), trained and run by the library's own tensor-
 * core kernels.  It maps a problem family's data to a starting iterate for
 * the solver (the reference's Data.x/y/s, pdos.h:29-32); the solver's
 * result is always the one reported.  Arrays named x, t, y, mean, stdv,
 * x0, y0, s0 are DEVICE pointers; parameter arrays of set/get are HOST
 * arrays of natural shape (W1: hidden x n_in, W2: hidden x hidden,
 * W3: n_out x hidden, row-major).  The reference has no such component. */
typedef struct pdosgpu_mlp pdosgpu_mlp;

int pdosgpu_mlp_create(int n_in, int hidden, int n_out, int max_batch, pdosgpu_mlp **out);
int pdosgpu_mlp_set_params(pdosgpu_mlp *p, const float *w1, const float *b1, const float *w2,
                           const float *b2, const float *w3, const float *b3);
/* grads != 0: the gradients of the last training step instead. */
int pdosgpu_mlp_get_params(pdosgpu_mlp *p, int grads, float *w1, float *b1, float *w2,
                           float *b2, float *w3, float *b3);
/* y[batch, n_out] = network(x[batch, n_in]), FP32 in and out. */
int pdosgpu_mlp_forward(pdosgpu_mlp *p, const float *x, int batch, float *y);
/* One Adam step on the mean squared error to t[batch, n_out]; batch a
 * multiple of 8; *loss (host, may be NULL) = the loss before the step. */
int pdosgpu_mlp_train_step(pdosgpu_mlp *p, const float *x, const float *t, int batch,
                           float lr, double *loss);
/* Network output rows [x | y | s] (n + 2m = n_out, standardised) turned
 * into stacked starting iterates out * stdv + mean: x0[batch*n],
 * y0[batch*m], s0[batch*m] in double, ready for pdosgpu_batch_warm_start. */
int pdosgpu_mlp_predict_start(pdosgpu_mlp *p, const float *x, int batch, const float *mean,
                              const float *stdv, int64_t n, int64_t m, double *x0, double *y0,
                              double *s0);
/* Roofline timing of the three forward products on the last inputs:
 * *ms per forward pass, *flops = 2 * batch * (n_in*h + h*h + h*n_out). */
int pdosgpu_mlp_time_forward(pdosgpu_mlp *p, int batch, int reps, double *ms, double *flops);
void *pdosgpu_mlp_stream(pdosgpu_mlp *p);
/* Waits for the network's stream; fails if a tensor-core product timed out. */
int pdosgpu_mlp_sync(pdosgpu_mlp *p);
/* Product kernel: 2 (default) = tcgen05 with tensor-memory accumulators,
 * operands staged by TMA (cp.async.bulk.tensor, 128-byte swizzled tiles) in
 * a producer / MMA / epilogue warp split; 1 = tcgen05 with operands staged
 * by cp.async; 0 = mma.sync.  All three give the same products. */
int pdosgpu_mlp_set_kernel(pdosgpu_mlp *p, int kind);
/* Failure-path test of the bounded waits (cycles > 0; 0 turns it off): the
 * next TMA-fed tensor-core products (kernel 2) first wait, for at most
 * `cycles` clock cycles, on a barrier that nothing completes, before any
 * copy or product is issued.  The wait runs out, each product records the
 * timeout and frees its tensor memory without writing its output, and the
 * following pdosgpu_mlp_sync returns PDOSGPU_ECUDA once (the flag is then
 * cleared).  Every wait of the tensor-core kernels is bounded (about one
 * second) in normal use; this exercises that path without a GPU fault. */
int pdosgpu_mlp_test_wait_timeout(pdosgpu_mlp *p, int64_t cycles);
void pdosgpu_mlp_free(pdosgpu_mlp *p);

/* pdos() over `count` problems at once: sols[i] is what pdos(d[i], k[i])
 * returns (free each with freeSol), info (may be NULL) gets one record per
 * instance.  Returns PDOSGPU_OK or a negative status (then every sols[i]
 * is NULL). */
int pdos_batch(const Data *const *d, const Cone *const *k, int64_t count,
               const pdosgpu_options *opt, Sol **sols, pdosgpu_info *info);

/* ---- kernel-level entry points on device memory ------------------------
 * Pointers are device pointers; `stream` is a cudaStream_t (NULL = legacy
 * default stream).  They run asynchronously on `stream`. */

/* CSC (m x n, int32 row indices) -> CSR of the same matrix, stable in column
 * order: the index work of cs_transpose (cs.c:146-168) and cs_cumsum
 * (cs.c:83-97), bit-exact.  Rp: m+1, Rj: nnz, Rx: nnz (Rx may be NULL when
 * Ax is NULL).  Uses temporary device memory allocated internally. */
int pdosgpu_csc_to_csr_f64(int32_t m, int32_t n, int32_t nnz, const int32_t *Ap,
                           const int32_t *Ai, const double *Ax, int32_t *Rp,
                           int32_t *Rj, double *Rx, void *stream);

/* y = sc * M x (accum = 0) or y += sc * M x (accum != 0) for the row-wise
 * matrix M (rows x cols, int32 rowptr/colidx).  The row gather of
 * accumByScaledA / accumByScaledATrans (linAlg.h:70-115).  Allocates its
 * tile table and long-row scratch internally. */
int pdosgpu_spmv_f64(int32_t rows, int32_t cols, const int32_t *rowptr,
                     const int32_t *colidx, const double *val, const double *x,
                     double sc, double *y, int accum, void *stream);
int pdosgpu_spmv_f32(int32_t rows, int32_t cols, const int32_t *rowptr,
                     const int32_t *colidx, const float *val, const float *x,
                     float sc, float *y, int accum, void *stream);

/* In-place projection of v (m = f + l + sum q) onto {0}^f x R+^l x
 * SOC(q[0]) x ... (projCone, cones.c:5-57).  q is a HOST array. */
int pdosgpu_proj_cone_f64(double *v, int64_t f, int64_t l, int64_t qsize,
                          const int64_t *q, void *stream);

/* The same projection as pdosgpu_proj_cone_f64, for callers that cannot
 * allocate device memory while they run (memory owned by a pool allocator
 * that must not be bypassed, regions where allocation is forbidden or would
 * synchronise the device).  It calls no cudaMalloc/cudaFree: its scratch is a
 * static device array of about 3 MB built into the library.  With CUDA's
 * lazy module loading (the default) the driver places that array, and the
 * projection's kernels, in a context the first time they are used there, and
 * keeps them until the context is destroyed: so the first call in a context
 * is the one that allocates.  Make one warm-up call per device (or context),
 * projecting at least one second-order cone and one zero or nonnegative row,
 * before any region that must not allocate and before any stream capture.
 * The scratch address is looked up once per context (cudaGetSymbolAddress)
 * and cached by the context's unique id, so a context re-created after
 * cudaDeviceReset gets a fresh look-up.  Limits: at most 65,536 second-order
 * cones and 131,072 chunks of 4,096 rows (sum over cones of
 * ceil(q[i]/4096)); larger requests return PDOSGPU_EINVAL without touching
 * the GPU.  All calls share the array, so calls whose work overlaps on the
 * GPU race; serialise them on one stream.  q is a HOST array, copied with
 * cudaMemcpyAsync (a pageable q is staged before the call returns, so q may
 * be reused at once); the call returns once the work is queued on `stream`.
 * This entry point has no counterpart in the reference. */
int pdosgpu_proj_cone_f64_noalloc(double *v, int64_t f, int64_t l, int64_t qsize,
                                  const int64_t *q, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* PDOS_GB300_PDOS_GPU_H */
