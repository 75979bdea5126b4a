// Epilogues and element-wise kernels of one ADMM iteration (grid engine).
//
// Order of a captured iteration (k = CG_MAX_ITS):
//   top     A' pass on (y, u): dual residual, c'x, CG start q = p = -lam c - A'u,
//           stop test on the residuals of the current iterate  (pdos.c:95-107,
//           linAlg.h:178-201, indirect/private.c:58-67)
//   k x {   cg_a   A pass on p               (indirect/private.c:70)
//           cg_at  A' pass on A p: t = p + A'Ap, p't  (:72-75)
//           cg_upd x += a p, q -= a t, ||q||^2, beta   (:78-95) }
//   post    A pass on x: s~ = b - Ax, relax, s = s~ - lam y, zero/orthant
//           projection and the dual update for those rows   (:113-117,
//           pdos.c:232-249, :296-303)
//   soc     second-order-cone projection + dual update for cone rows
//           (cones.c:21-47), optionally in two kernels for cones too big for
//           one CTA.
// The A x product of `post` also serves the next iteration's primal
// residual and CG start (all three use the same x), so an iteration reads
// A k+1 times and A' k+1 times.
#pragma once

#include "common.cuh"
#include "sell.cuh"

namespace pdosgpu {

template <typename T>
struct Vecs {
  T *x, *s, *y, *st, *u, *ax, *p, *q, *t;
  const T *b, *c, *D, *E;
  int32_t m, n, f, l;
};

// Dual update of one finished row and the next iteration's residual inputs:
//   y += (s - s~)/lam                         pdos.c:232-236
//   pr = ((s - b) + Ax)/D                     linAlg.h:158-175
//   u  = ((s + lam y) - b) + Ax               indirect/private.c:20-29, :58-60
//   b'y                                       linAlg.h:199-201
template <typename T>
__device__ __forceinline__ void finish_row(const Vecs<T> &V, T lam, int r, T sv, T stv, T ax,
                                           double &pr2, double &by) {
  const T yv = V.y[r] + (sv - stv) / lam;
  V.y[r] = yv;
  V.s[r] = sv;
  const T bv = V.b[r];
  const T pr = ((sv - bv) + ax) / V.D[r];
  pr2 += (double)pr * (double)pr;
  V.u[r] = ((sv + lam * yv) - bv) + ax;
  by += (double)bv * (double)yv;
}

struct NoCtx {};

// Initial pass: A x0 feeds the primal residual, u and b'y of iteration 0.
template <typename T>
struct OpPrep {
  static constexpr int NV = 1, NR = 2;
  using Ctx = NoCtx;
  Vecs<T> V;
  T lam;
  DevState *S;
  __device__ bool begin(Ctx &) const { return true; }
  __device__ void row(const Ctx &, int r, const T (&sum)[1], double (&red)[2]) const {
    const T ax = sum[0], sv = V.s[r], bv = V.b[r], yv = V.y[r];
    V.ax[r] = ax;
    const T pr = ((sv - bv) + ax) / V.D[r];
    red[0] += (double)pr * (double)pr;
    V.u[r] = ((sv + lam * yv) - bv) + ax;
    red[1] += (double)bv * (double)yv;
  }
  __device__ void finalize(const Ctx &, const double (&tot)[2]) const {
    S->pres_sq = tot[0];
    S->by = tot[1];
  }
};

// Top of the iteration: A' on (y, u) in one pass over A.
template <typename T>
struct OpTop {
  static constexpr int NV = 2, NR = 3;
  using Ctx = NoCtx;
  Vecs<T> V;
  T lam;
  DevState *S;
  __device__ bool begin(Ctx &) const { return !*(volatile int *)&S->done; }
  __device__ void row(const Ctx &, int j, const T (&sum)[2], double (&red)[3]) const {
    const T cj = V.c[j];
    const T dr = (cj + sum[0]) / V.E[j];
    red[0] += (double)dr * (double)dr;
    red[1] += (double)cj * (double)V.x[j];
    const T qj = (-lam) * cj + (-sum[1]);
    V.q[j] = qj;
    V.p[j] = qj;
    red[2] += (double)qj * (double)qj;
  }
  __device__ void finalize(const Ctx &, const double (&tot)[3]) const {
    DevState &s = *S;
    s.p_res = sqrt(s.pres_sq);
    s.d_res = sqrt(tot[0]);
    s.p_obj = tot[1];
    s.d_obj = -s.by;
    s.eta = fabs(s.p_obj - s.d_obj);
    s.evaluated = 1;
    if (s.p_res < s.eps * s.pscale && s.d_res < s.eps * s.dscale &&
        s.eta < s.eps * (1.0 + fabs(s.p_obj) + fabs(s.d_obj))) {
      s.solved = 1;
      s.done = 1;
      s.cg_skip = 1;
      return;
    }
    // A non-finite residual or gap (the iterate overflowed): the reference
    // would run on to MAX_ITERS (pdos.c:94-107); stop here and say so.
    if (!isfinite(s.p_res) || !isfinite(s.d_res) || !isfinite(s.eta)) {
      s.diverged = 1;
      s.done = 1;
      s.cg_skip = 1;
      return;
    }
    s.qsold = tot[2];
    s.cg_iter = 0;
    s.cg_active = (s.cg_max > 0 && s.qsold > s.tol_sq) ? 1 : 0;
    s.cg_skip = s.cg_active ? 0 : 1;
  }
};

__device__ __forceinline__ bool cg_begin(const DevState *S) {
  const volatile DevState *v = S;
  return !v->done && v->cg_active;
}

// CG: u = A p  (indirect/private.c:70)
template <typename T>
struct OpCgA {
  static constexpr int NV = 1, NR = 0;
  using Ctx = NoCtx;
  Vecs<T> V;
  DevState *S;
  __device__ bool begin(Ctx &) const { return cg_begin(S); }
  __device__ void row(const Ctx &, int r, const T (&sum)[1], double (&)[1]) const {
    V.u[r] = sum[0];
  }
  __device__ void finalize(const Ctx &, const double (&)[1]) const {}
};

// CG: t = p + A'(Ap) and p't  (indirect/private.c:71-75)
template <typename T>
struct OpCgAt {
  static constexpr int NV = 1, NR = 1;
  using Ctx = NoCtx;
  Vecs<T> V;
  DevState *S;
  __device__ bool begin(Ctx &) const { return cg_begin(S); }
  __device__ void row(const Ctx &, int j, const T (&sum)[1], double (&red)[1]) const {
    const T pj = V.p[j];
    const T tj = pj + sum[0];
    V.t[j] = tj;
    red[0] += (double)pj * (double)tj;
  }
  __device__ void finalize(const Ctx &, const double (&tot)[1]) const {
    S->step = S->qsold / tot[0];
  }
};

// CG: x += step p; q += (-step) t; ||q||^2; break test and beta.
template <typename T, int BLOCK>
__global__ void __launch_bounds__(BLOCK) cg_update_kernel(Vecs<T> V, DevState *S, GridReduce gr) {
  __shared__ double scratch[BLOCK / 32];
  __shared__ double s_step;
  if (threadIdx.x == 0) {
    const volatile DevState *v = S;
    s_step = (v->done || !v->cg_active) ? 0.0 : v->step;
  }
  {
    const volatile DevState *v = S;
    if (v->done || !v->cg_active) return;
  }
  __syncthreads();
  const T step = (T)s_step;
  const T nstep = (T)(-s_step);
  double red[1] = {0.0};
  for (int j = blockIdx.x * BLOCK + threadIdx.x; j < V.n; j += gridDim.x * BLOCK) {
    const T pj = V.p[j], tj = V.t[j];
    V.x[j] = V.x[j] + step * pj;
    const T qj = V.q[j] + nstep * tj;
    V.q[j] = qj;
    red[0] += (double)qj * (double)qj;
  }
  double tot[1];
  if (grid_reduce<BLOCK, 1>(gr, red, tot, scratch) && threadIdx.x == 0) {
    DevState &s = *S;
    const double qsnew = tot[0];
    s.cg_iter += 1;
    s.cg_total += 1;
    if (qsnew < s.tol_sq) {
      s.cg_active = 0;
    } else {
      s.ratio = qsnew / s.qsold;
      s.qsold = qsnew;
      if (s.cg_iter >= s.cg_max) s.cg_active = 0;
    }
    s.cg_skip = s.cg_active ? 0 : 1;
  }
}

// CG direction: p = beta p + q while CG continues (indirect/private.c:91-93)
template <typename T, int BLOCK>
__global__ void __launch_bounds__(BLOCK) cg_direction_kernel(Vecs<T> V, const DevState *S) {
  __shared__ double s_ratio;
  __shared__ int s_go;
  if (threadIdx.x == 0) {
    const volatile DevState *v = S;
    s_go = (!v->done && v->cg_active) ? 1 : 0;
    s_ratio = v->ratio;
  }
  __syncthreads();
  if (!s_go) return;
  const T beta = (T)s_ratio;
  for (int j = blockIdx.x * BLOCK + threadIdx.x; j < V.n; j += gridDim.x * BLOCK)
    V.p[j] = beta * V.p[j] + V.q[j];
}

// End of an ADMM iteration: bookkeeping done by the last block of the last
// kernel of the iteration.
__device__ __forceinline__ void end_iteration(DevState *S, const double (&tot)[2]) {
  S->pres_sq = tot[0];
  S->by = tot[1];
  S->admm_iter += 1;
  if (S->admm_iter >= S->max_iters) S->done = 1;
  S->cg_skip = 1;
}

// After CG: s~ = b - A x, relax, s = s~ - lam y; zero-cone and orthant rows
// are projected and finished here, cone rows are left to the SOC kernels.
template <typename T>
struct OpPost {
  static constexpr int NV = 1, NR = 2;
  using Ctx = NoCtx;
  Vecs<T> V;
  T lam, alpha, one_minus_alpha;
  DevState *S;
  __device__ bool begin(Ctx &) const { return !*(volatile int *)&S->done; }
  __device__ void row(const Ctx &, int r, const T (&sum)[1], double (&red)[2]) const {
    const T ax = sum[0];
    T stv = V.b[r] + (-ax);
    stv = alpha * stv + one_minus_alpha * V.s[r];
    T v = stv - lam * V.y[r];
    V.ax[r] = ax;
    if (r < V.f) {
      finish_row(V, lam, r, T(0), stv, ax, red[0], red[1]);
    } else if (r < V.f + V.l) {
      if (v < T(0)) v = T(0);
      finish_row(V, lam, r, v, stv, ax, red[0], red[1]);
    } else {
      V.s[r] = v;
      V.st[r] = stv;
    }
  }
  __device__ void finalize(const Ctx &, const double (&tot)[2]) const { end_iteration(S, tot); }
};

// ----------------------------------------------------------- SOC kernels
// Cones with at most kSmallCone rows: one warp each, whole projection in one
// kernel.  Larger cones: cut into chunks of kConeChunk rows, one CTA each;
// `soc_kernel` leaves a partial tail norm per chunk (and the head value),
// `soc_big_kernel` finishes.
constexpr int kSmallCone = 1024;
constexpr int kConeChunk = 4096;

struct ConeTables {
  const int32_t *small_off;   // [n_small] first row of each small cone
  const int32_t *small_len;   // [n_small] its size
  int32_t n_small;
  const int32_t *chunk_row0;  // [n_chunks]
  const int32_t *chunk_row1;
  const int32_t *chunk_cone;  // big-cone index of each chunk
  int32_t n_chunks;
  const int32_t *big_head;    // [n_big] head row of each big cone
  const int32_t *big_chunk0;  // [n_big] first chunk
  const int32_t *big_nchunks; // [n_big]
  double *chunk_sq;           // [n_chunks]
  double *big_headval;        // [n_big]
  int32_t small_blocks;       // blocks of soc_kernel given to small cones
};

// Three-case SOC rule of cones.c:21-47 applied to one element.
template <typename T>
__device__ __forceinline__ T soc_apply(T v, bool is_head, T head, T tail) {
  if (tail <= head) return v;
  if (tail <= -head) return T(0);
  const T half = (tail + head) / T(2);
  return is_head ? half : half * v / tail;
}

template <typename T, int BLOCK>
__global__ void __launch_bounds__(BLOCK) soc_kernel(Vecs<T> V, ConeTables ct, T lam, DevState *S,
                                                    GridReduce gr) {
  __shared__ double scratch[BLOCK / 32];
  if (*(volatile int *)&S->done) return;
  double red[2] = {0.0, 0.0};
  const int lane = threadIdx.x & 31;
  if ((int)blockIdx.x < ct.small_blocks) {
    const int warps_total = ct.small_blocks * (BLOCK / 32);
    for (int c = blockIdx.x * (BLOCK / 32) + (threadIdx.x >> 5); c < ct.n_small; c += warps_total) {
      const int off = ct.small_off[c], len = ct.small_len[c];
      T acc = T(0);
      for (int i = 1 + lane; i < len; i += 32) {
        const T v = V.s[off + i];
        acc += v * v;
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
      const T tail = sqrt(acc);
      const T head = V.s[off];
      __syncwarp();
      for (int i = lane; i < len; i += 32) {
        const int r = off + i;
        const T sv = soc_apply(V.s[r], i == 0, head, tail);
        finish_row(V, lam, r, sv, V.st[r], V.ax[r], red[0], red[1]);
      }
    }
  } else {
    const int ch = blockIdx.x - ct.small_blocks;
    const int r0 = ct.chunk_row0[ch], r1 = ct.chunk_row1[ch];
    const int big = ct.chunk_cone[ch];
    const int head_row = ct.big_head[big];
    double acc = 0.0;
    for (int r = r0 + threadIdx.x; r < r1; r += BLOCK) {
      if (r == head_row) continue;
      const T v = V.s[r];
      acc += (double)(v * v);
    }
    // fixed-order block sum (partial of the cone's tail norm)
    acc = block_sum<BLOCK>(acc, scratch);
    if (threadIdx.x == 0) {
      ct.chunk_sq[ch] = acc;
      if (r0 <= head_row && head_row < r1) ct.big_headval[big] = (double)V.s[head_row];
    }
  }
  double tot[2];
  if (grid_reduce<BLOCK, 2>(gr, red, tot, scratch) && threadIdx.x == 0) end_iteration(S, tot);
}

template <typename T, int BLOCK>
__global__ void __launch_bounds__(BLOCK) soc_big_kernel(Vecs<T> V, ConeTables ct, T lam, DevState *S,
                                                        GridReduce gr) {
  __shared__ double scratch[BLOCK / 32];
  __shared__ double s_tail;
  if (*(volatile int *)&S->done) return;
  const int ch = blockIdx.x;
  const int r0 = ct.chunk_row0[ch], r1 = ct.chunk_row1[ch];
  const int big = ct.chunk_cone[ch];
  if (threadIdx.x < 32) {
    double a = 0.0;
    const int c0 = ct.big_chunk0[big], nc = ct.big_nchunks[big];
    for (int c = threadIdx.x; c < nc; c += 32) a += __ldcg(&ct.chunk_sq[c0 + c]);
    a = warp_sum(a);
    if (threadIdx.x == 0) s_tail = sqrt(a);
  }
  __syncthreads();
  const T tail = (T)s_tail;
  const T head = (T)__ldcg(&ct.big_headval[big]);
  const int head_row = ct.big_head[big];
  double red[2] = {0.0, 0.0};
  for (int r = r0 + threadIdx.x; r < r1; r += BLOCK) {
    const T sv = soc_apply(V.s[r], r == head_row, head, tail);
    finish_row(V, lam, r, sv, V.st[r], V.ax[r], red[0], red[1]);
  }
  double tot[2];
  if (grid_reduce<BLOCK, 2>(gr, red, tot, scratch) && threadIdx.x == 0) end_iteration(S, tot);
}

}  // namespace pdosgpu

namespace pdosgpu {

// ----------------------------------------------- stand-alone projection
// projCone (cones.c:50-57) on a device vector, for the kernel-level entry
// point: zero / orthant rows element-wise, cones as in the solver kernels.
template <typename T>
__global__ void proj_lin_kernel(T *v, int64_t f, int64_t l) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < f + l;
       i += (int64_t)gridDim.x * blockDim.x) {
    if (i < f) v[i] = T(0);
    else if (v[i] < T(0)) v[i] = T(0);
  }
}

template <typename T, int BLOCK>
__global__ void __launch_bounds__(BLOCK) proj_small_kernel(T *v, ConeTables ct) {
  const int lane = threadIdx.x & 31;
  const int warps_total = gridDim.x * (BLOCK / 32);
  for (int c = blockIdx.x * (BLOCK / 32) + (threadIdx.x >> 5); c < ct.n_small; c += warps_total) {
    const int off = ct.small_off[c], len = ct.small_len[c];
    T acc = T(0);
    for (int i = 1 + lane; i < len; i += 32) acc += v[off + i] * v[off + i];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    const T tail = sqrt(acc);
    const T head = v[off];
    __syncwarp();
    for (int i = lane; i < len; i += 32) v[off + i] = soc_apply(v[off + i], i == 0, head, tail);
  }
}

template <typename T, int BLOCK>
__global__ void __launch_bounds__(BLOCK) proj_chunk_sq_kernel(const T *v, ConeTables ct) {
  __shared__ double scratch[BLOCK / 32];
  const int ch = blockIdx.x;
  const int r0 = ct.chunk_row0[ch], r1 = ct.chunk_row1[ch];
  const int big = ct.chunk_cone[ch];
  const int head_row = ct.big_head[big];
  double acc = 0.0;
  for (int r = r0 + threadIdx.x; r < r1; r += BLOCK)
    if (r != head_row) acc += (double)(v[r] * v[r]);
  acc = block_sum<BLOCK>(acc, scratch);
  if (threadIdx.x == 0) {
    ct.chunk_sq[ch] = acc;
    if (r0 <= head_row && head_row < r1) ct.big_headval[big] = (double)v[head_row];
  }
}

template <typename T, int BLOCK>
__global__ void __launch_bounds__(BLOCK) proj_chunk_apply_kernel(T *v, ConeTables ct) {
  __shared__ double s_tail;
  const int ch = blockIdx.x;
  const int r0 = ct.chunk_row0[ch], r1 = ct.chunk_row1[ch];
  const int big = ct.chunk_cone[ch];
  if (threadIdx.x < 32) {
    double a = 0.0;
    const int c0 = ct.big_chunk0[big], nc = ct.big_nchunks[big];
    for (int c = threadIdx.x; c < nc; c += 32) a += __ldcg(&ct.chunk_sq[c0 + c]);
    a = warp_sum(a);
    if (threadIdx.x == 0) s_tail = sqrt(a);
  }
  __syncthreads();
  const T tail = (T)s_tail;
  const T head = (T)__ldcg(&ct.big_headval[big]);
  const int head_row = ct.big_head[big];
  for (int r = r0 + threadIdx.x; r < r1; r += BLOCK) v[r] = soc_apply(v[r], r == head_row, head, tail);
}

// y = sc * M x  or  y += sc * M x  (linAlg.h:70-115)
template <typename T>
struct OpAxpy {
  static constexpr int NV = 1, NR = 0;
  using Ctx = NoCtx;
  const T *x;
  T *y;
  T sc;
  int accum;
  __device__ bool begin(Ctx &) const { return true; }
  __device__ void row(const Ctx &, int r, const T (&sum)[1], double (&)[1]) const {
    const T v = sc * sum[0];
    y[r] = accum ? y[r] + v : v;
  }
  __device__ void finalize(const Ctx &, const double (&)[1]) const {}
};

}  // namespace pdosgpu
