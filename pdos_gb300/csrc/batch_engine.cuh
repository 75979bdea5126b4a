// Batched solver: many independent PDOS problems of uneven sizes and cone
// profiles, solved by one persistent kernel per size class.
//
// Each CTA takes an instance from a queue and runs that instance's whole
// ADMM iteration (pdos.c:94-120) with CTA barriers only: the A' pass on
// (y, u) with the stop test, the warm-started CG (indirect/private.c:31-104),
// the A pass on x with relaxation, zero / orthant projection and dual update
// (pdos.c:232-249, :296-303), the second-order-cone projection
// (cones.c:21-47).  The vector a product gathers from is staged in shared
// memory, so the matrix streams from HBM with coalesced loads while the
// random gathers hit shared memory; CG's p, A p and t never leave shared
// memory.  An instance whose vectors do not fit one CTA's shared memory
// stages them in a global-memory region of its CTA instead (a separate
// kernel instantiation, so that the shared-memory kernels keep
// shared-memory gathers).  A finished instance frees its CTA for the next one (convergence
// masking), every reduction has a fixed order, and the kernel of one launch
// runs each instance for at most `iter_cap` iterations, so a captured launch
// can be replayed until every instance is done.
//
// Per-instance arithmetic follows the grid engine (admm_ops.cuh) operation
// by operation; only the summation order of the products and reductions
// differs.
//
// This header holds the kernels and the engine template; each precision is
// instantiated in its own translation unit (batch_f32.cu, batch_f64.cu) so
// that the two compile in parallel, and batch.cu holds the C API.
#pragma once

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstring>
#include <memory>
#include <numeric>
#include <string>
#include <thread>
#include <vector>

#include "batch_layout.h"
#include "batch_family.h"
#include "engine.cuh"
#include "problem.cuh"

namespace pdosgpu {
namespace batch {

#ifndef PDOS_BATCH_UNROLL
#define PDOS_BATCH_UNROLL 2
#endif
constexpr int kUnroll = PDOS_BATCH_UNROLL;  // 16-byte loads in flight per lane and operand
// Size classes: four by nonzeros per instance, whose gather vectors are
// staged in shared memory, and a fifth for instances too large for one CTA's
// shared memory, whose vectors are staged in a global-memory region of
// their CTA instead (L2-resident).
constexpr int kClasses = 5;
constexpr int kGlobalClass = 4;
constexpr int64_t kClassNnz[3] = {4096, 32768, 262144};
constexpr int kSmemLimit = 225 * 1024;  // dynamic shared memory per CTA (opt-in limit 227 KB)
constexpr int kBlocks[] = {128, 256, 512, 1024};
constexpr int kNumBlocks = 4;

// Layout arrays of one side (rows of A, or rows of A') of one set-up wave,
// in device memory.  Every instance carries the arrays of its wave, so the
// waves of a batch are independent allocations: a batch may hold more than
// 2^31 nonzeros in all while each wave's set-up keeps 32-bit indices.
struct HybPtr {
  const int64_t *slice_beg;    // first element of each slice
  const int32_t *slice_w;      // its width (elements per lane)
  const uint32_t *slice_skip;  // lanes whose row is a long row or past the end
  const int32_t *piece_row;    // >= 0: the whole row; < 0: ~row of a split row
  const int64_t *piece_beg;
  const int32_t *piece_len;
  const int32_t *split_row, *split_p0, *split_np;  // pieces of each split row
  const uint16_t *idx;         // gather index, local to the instance (< 65,536)
  const void *val;             // values (float or double)
  const uint16_t *slice_row;   // row of each lane of a sorted instance's slices (NULL if none sorted)
};

struct Inst {
  int64_t row0, col0;  // offsets into the stacked row / column vectors
  int32_t m, n, f, l;
  int64_t cone0;
  int32_t ncones, cls;
  Side A, At;
  double lambda, pscale, dscale, alpha, eps, tol_sq;
  int64_t max_iters, cg_max;
  HybPtr hA, hT;  // layout arrays of the instance's wave (or of its family group)
  // Family groups (instances with one pattern whose values differ only at
  // a few positions) share hA / hT; the shared value arrays then hold, at
  // each position that varies within the group, a NaN whose payload indexes
  // the instance's own values here (layout order).  nullptr: own layout.
  const void *pvA, *pvT;
};

struct State {
  double pres_sq, by, p_res, d_res, p_obj, d_obj, eta;
  long long admm_iter, cg_total;
  int solved, done, prepped, diverged;
};

template <typename T>
struct Dev {
  const Inst *inst;
  State *state;
  const int32_t *order;        // instance ids, class by class
  const int32_t *class_begin;  // [kClasses + 1]
  int32_t *queue;              // [kClasses] queue heads, zeroed before a launch
  int32_t *ndone;              // instances finished so far
  T *x, *s, *y, *st, *u, *ax, *q;
  const T *b, *c, *D, *E;
  const int32_t *cone_off, *cone_len;  // local first row and size of each cone
  T *gscratch;  // global staging regions of the global class, one per CTA
};

// Staging regions of one class, in elements of T: in dynamic shared memory,
// or (global != 0) in the CTA's region of Dev::gscratch.  A global-staging
// class also keeps, in dynamic shared memory, room for the one vector a
// product gathers from (gs elements): instances whose max(m, n) fits it
// gather from shared memory, larger ones from their global region.
struct Smem {
  int32_t g1, g2, tt, pb, global, gs;
  int32_t pair;  // shared-memory class run as pairs of family instances: twice the regions
  __host__ __device__ size_t stride() const {  // elements per CTA region, 128-byte multiples
    return ((size_t)g1 + g2 + tt + pb + 31) & ~(size_t)31;
  }
  size_t need(size_t elem) const { return elem * ((size_t)g1 + g2 + tt + pb); }
  size_t bytes(size_t elem) const { return global ? elem * (size_t)gs : (pair ? 2 : 1) * need(elem); }
};

// Base of a CTA's staging regions.  A compile-time choice, so that kernels
// staging in shared memory keep shared-memory gathers (a pointer that may
// point to either space turns every gather into a generic load).
template <typename T, bool GLOBAL>
__device__ __forceinline__ T *staging_base(const Smem &sm, unsigned char *smem_raw, T *gscratch) {
  if (GLOBAL) return gscratch + (size_t)blockIdx.x * sm.stride();
  return reinterpret_cast<T *>(smem_raw);
}

template <typename T>
__device__ __forceinline__ T warp_sum_t(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Block sums of N values.  Each warp sums its lanes with a xor butterfly,
// lane 0 stores the warp's partial, and after the barrier every warp loads
// the W partials into its lanes and runs the same butterfly: a fixed order,
// and since floating-point addition commutes every lane of every warp ends
// with the same bits.  (Summing the W partials one by one in every thread
// would cost W times as many FP64 additions, which the GB300's narrow FP64
// pipe turns into microseconds per reduction.)  The barrier after the
// partials are written also orders every earlier shared-memory write.
// Callers alternate between two scratch halves (Reduce below): the next use
// of a half comes after another reduction's barrier, so no second barrier
// is needed before the half is overwritten.  scratch: N * BLOCK/32.
template <int BLOCK, int N>
__device__ __forceinline__ void block_sum_n(double (&v)[N], double *scratch) {
  constexpr int W = BLOCK / 32;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < N; ++k) v[k] = warp_sum(v[k]);
  if (lane == 0) {
#pragma unroll
    for (int k = 0; k < N; ++k) scratch[k * W + warp] = v[k];
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < N; ++k) v[k] = warp_sum(lane < W ? scratch[k * W + lane] : 0.0);
}

// Two scratch halves of 3 * BLOCK/32 doubles, used in turn.
template <int BLOCK, int MAXN = 3>
struct Reduce {
  double *scratch;  // 2 x MAXN x BLOCK/32
  int half;
  template <int N>
  __device__ __forceinline__ void operator()(double (&v)[N]) {
    static_assert(N <= MAXN, "scratch too small");
    half ^= 1;
    block_sum_n<BLOCK, N>(v, scratch + half * MAXN * (BLOCK / 32));
  }
};

// Streaming loads of four consecutive matrix entries (16-byte aligned):
// read-only for the kernel's lifetime and not kept in L1, which holds the
// instance's vectors instead.
struct Idx4 {
  int x, y, z, w;
};
__device__ __forceinline__ Idx4 ld_stream4(const uint16_t *p) {  // 8-byte aligned
  unsigned a, b;
  asm("ld.global.nc.L1::no_allocate.v2.u32 {%0, %1}, [%2];" : "=r"(a), "=r"(b) : "l"(p));
  return Idx4{(int)(a & 0xffffu), (int)(a >> 16), (int)(b & 0xffffu), (int)(b >> 16)};
}
template <typename T>
struct Val4 {
  T x, y, z, w;
};
__device__ __forceinline__ Val4<float> ld_stream4(const float *p) {
  Val4<float> r;
  asm("ld.global.nc.L1::no_allocate.v4.f32 {%0, %1, %2, %3}, [%4];"
               : "=f"(r.x), "=f"(r.y), "=f"(r.z), "=f"(r.w)
               : "l"(p));
  return r;
}
__device__ __forceinline__ Val4<double> ld_stream4(const double *p) {
  Val4<double> r;
  asm("ld.global.nc.L1::no_allocate.v2.f64 {%0, %1}, [%2];"
               : "=d"(r.x), "=d"(r.y)
               : "l"(p));
  asm("ld.global.nc.L1::no_allocate.v2.f64 {%0, %1}, [%2];"
               : "=d"(r.z), "=d"(r.w)
               : "l"(p + 2));
  return r;
}

// Varying entries of a shared (family) layout: the shared value array holds
// a quiet NaN whose low kBoxBits bits index the instance's own value of that
// entry (batch_family.h).  Input data is checked finite at set-up, so no
// genuine value is a NaN.
__device__ __forceinline__ float nan_box(float, uint32_t t) { return __uint_as_float(0x7FC00000u | t); }
__device__ __forceinline__ double nan_box(double, uint32_t t) {
  return __longlong_as_double((long long)(0x7FF8000000000000ull | (unsigned long long)t));
}
__device__ __forceinline__ uint32_t box_payload(float v) { return __float_as_uint(v) & ((1u << kBoxBits) - 1); }
__device__ __forceinline__ uint32_t box_payload(double v) {
  return (uint32_t)((unsigned long long)__double_as_longlong(v) & ((1ull << kBoxBits) - 1));
}
template <typename T>
__device__ __forceinline__ T unbox(T v, const T *pv) {
  return v != v ? __ldg(pv + box_payload(v)) : v;
}
// Four loaded values with their boxes resolved.  FP32: one NaN test of the
// values' sum finds any box (a NaN propagates through the sum; input data is
// finite, so anything else is an overflowed sum, which the per-value test
// then leaves alone) -- three adds and a compare per four values instead of
// four compares and selects.  FP64 keeps the per-value test, as FP64 adds
// are scarce.
__device__ __forceinline__ void unbox4(Val4<float> &v, const float *pv) {
  const float probe = (v.x + v.y) + (v.z + v.w);
  if (probe != probe) v = Val4<float>{unbox(v.x, pv), unbox(v.y, pv), unbox(v.z, pv), unbox(v.w, pv)};
}
__device__ __forceinline__ void unbox4(Val4<double> &v, const double *pv) {
  v = Val4<double>{unbox(v.x, pv), unbox(v.y, pv), unbox(v.z, pv), unbox(v.w, pv)};
}

// Four consecutive entries of one row into the NV running sums, in order.
template <typename T, int NV>
__device__ __forceinline__ void fma4(const Idx4 &j, const Val4<T> &v, const T *src0, const T *src1,
                                     T &a0, T &a1) {
  a0 = fma(v.x, src0[j.x], a0);
  a0 = fma(v.y, src0[j.y], a0);
  a0 = fma(v.z, src0[j.z], a0);
  a0 = fma(v.w, src0[j.w], a0);
  if (NV == 2) {
    a1 = fma(v.x, src1[j.x], a1);
    a1 = fma(v.y, src1[j.y], a1);
    a1 = fma(v.z, src1[j.z], a1);
    a1 = fma(v.w, src1[j.w], a1);
  }
}

// y-side of one product over one side of an instance: NV source vectors
// (in shared or global memory), rows handed to epi(row, sum0, sum1).
// Pieces are 4-aligned runs of one row (lane l takes entries 4l..4l+3 of
// every 128); slices of width >= 4 are stored four columns at a time per
// lane ([c/4][lane][c%4]), narrower ones one column at a time ([c][lane]).
// Split rows leave piece partials in pbuf and are finished after a barrier.
// SHARED: the layout is a family group's; pv holds this instance's values
// of the entries that vary within the group (see unbox).
// The work is split over the warps and threads that `Part` names -- one
// CTA's, or a cluster's -- and `bar` orders the piece partials before the
// split rows are finished (a CTA or a cluster barrier).
struct Part {
  int w0, ws;  // this warp's first piece / slice and the stride between warps
  int t0, ts;  // this thread's first split row and the stride between threads
};
template <int BLOCK>
__device__ __forceinline__ Part cta_part() {
  return Part{(int)(threadIdx.x >> 5), BLOCK / 32, (int)threadIdx.x, BLOCK};
}
struct CtaBarrier {
  __device__ void operator()() const { __syncthreads(); }
};

template <typename T, int NV, bool SHARED, class Bar, class Epi>
__device__ __forceinline__ void hyb_product_impl(const HybPtr &H, const Side &sd, const T *pv, const T *src0,
                                                 const T *src1, T *pbuf, const Part &pt, const Bar &bar,
                                                 Epi &&epi) {
  const T *const hval = static_cast<const T *>(H.val);
  const int lane = threadIdx.x & 31;
  for (int k = pt.w0; k < sd.npieces; k += pt.ws) {
    const int64_t pk = sd.piece0 + k;
    const int32_t prow = H.piece_row[pk];
    const int64_t beg = H.piece_beg[pk];
    const int len = H.piece_len[pk];  // a multiple of 4
    T a0 = T(0), a1 = T(0);
    const uint16_t *ip = H.idx + beg;
    const T *vp = hval + beg;
#pragma unroll kUnroll
    for (int e = 4 * lane; e < len; e += 128) {
      const Idx4 j = ld_stream4(ip + e);
      Val4<T> v = ld_stream4(vp + e);
      if (SHARED) unbox4(v, pv);
      fma4<T, NV>(j, v, src0, src1, a0, a1);
    }
    a0 = warp_sum_t(a0);
    if (NV == 2) a1 = warp_sum_t(a1);
    if (lane == 0) {
      if (prow >= 0) {
        epi(prow, a0, a1);
      } else {
        pbuf[k * NV] = a0;
        if (NV == 2) pbuf[k * NV + 1] = a1;
      }
    }
  }
  for (int s = pt.w0; s < sd.nslices; s += pt.ws) {
    const int64_t sk = sd.slice0 + s;
    const int64_t off = H.slice_beg[sk];
    const int width = H.slice_w[sk];
    T a0 = T(0), a1 = T(0);
    if (width < 0) {  // four columns per lane and load
      const uint16_t *ip = H.idx + off + 4 * lane;
      const T *vp = hval + off + 4 * lane;
#pragma unroll kUnroll
      for (int c4 = 0; c4 < -width; c4 += 4) {
        const Idx4 j = ld_stream4(ip + 32 * c4);
        Val4<T> v = ld_stream4(vp + 32 * c4);
        if (SHARED) unbox4(v, pv);
        fma4<T, NV>(j, v, src0, src1, a0, a1);
      }
    } else {
      const uint16_t *ip = H.idx + off + lane;
      const T *vp = hval + off + lane;
      for (int c = 0; c < width; ++c) {
        const int j = ip[c * 32];
        T v = vp[c * 32];
        if (SHARED) v = unbox(v, pv);
        a0 = fma(v, src0[j], a0);
        if (NV == 2) a1 = fma(v, src1[j], a1);
      }
    }
    if (!((H.slice_skip[sk] >> lane) & 1u))
      epi(sd.sorted ? (int)H.slice_row[sk * 32 + lane] : s * 32 + lane, a0, a1);  // the lane's row
  }
  if (sd.nsplit > 0) {
    bar();
    for (int k = pt.t0; k < sd.nsplit; k += pt.ts) {
      const int64_t sk = sd.split0 + k;
      const int p0 = H.split_p0[sk], np = H.split_np[sk];
      T a0 = T(0), a1 = T(0);
      for (int t = 0; t < np; ++t) {
        a0 += pbuf[(p0 + t) * NV];
        if (NV == 2) a1 += pbuf[(p0 + t) * NV + 1];
      }
      epi(H.split_row[sk], a0, a1);
    }
  }
}

// One product over one side of an instance, through its own layout or its
// family group's shared one.
template <typename T, int NV, class Bar, class Epi>
__device__ __forceinline__ void hyb_product_part(const HybPtr &H, const Side &sd, const void *pv, const T *src0,
                                                 const T *src1, T *pbuf, const Part &pt, const Bar &bar,
                                                 Epi &&epi) {
  if (pv)
    hyb_product_impl<T, NV, true>(H, sd, static_cast<const T *>(pv), src0, src1, pbuf, pt, bar, epi);
  else
    hyb_product_impl<T, NV, false>(H, sd, nullptr, src0, src1, pbuf, pt, bar, epi);
}
template <typename T, int BLOCK, int NV, class Epi>
__device__ __forceinline__ void hyb_product(const HybPtr &H, const Side &sd, const void *pv, const T *src0,
                                            const T *src1, T *pbuf, Epi &&epi) {
  hyb_product_part<T, NV>(H, sd, pv, src0, src1, pbuf, cta_part<BLOCK>(), CtaBarrier{}, epi);
}

// Three-case SOC rule of cones.c:21-47 for one element.
template <typename T>
__device__ __forceinline__ T soc_rule(T v, bool is_head, T head, T tail) {
  if (tail <= head) return v;
  if (tail <= -head) return T(0);
  const T half = (tail + head) / T(2);
  return is_head ? half : half * v / tail;
}

// SG (global staging only): the vector each product gathers from is first
// copied into shared memory (gs), so the gathers hit shared memory while the
// staging regions stay in global memory.  The top pass then runs as two
// products (y, then u) instead of one with two source vectors: each row's
// two sums are the same chains of fused multiply-adds as in the one-pass
// form, so the results are bit-identical.
template <typename T, int BLOCK, bool SG = false>
__device__ void solve_instance(const Dev<T> &B, const Inst &I, State *gst, int iter_cap, T *g1,
                               T *g2, T *tt, T *pbuf, double *scratch, T *gs = nullptr) {
  const int tid = threadIdx.x;
  const int m = I.m, n = I.n, f = I.f, l = I.l;
  T *__restrict__ x = B.x + I.col0;
  T *__restrict__ q = B.q + I.col0;
  T *__restrict__ s = B.s + I.row0;
  T *__restrict__ y = B.y + I.row0;
  T *__restrict__ st = B.st + I.row0;
  T *__restrict__ u = B.u + I.row0;
  T *__restrict__ ax = B.ax + I.row0;
  const T *__restrict__ b = B.b + I.row0;
  const T *__restrict__ D = B.D + I.row0;
  const T *__restrict__ c = B.c + I.col0;
  const T *__restrict__ E = B.E + I.col0;
  const T lam = (T)I.lambda;
  const T alpha = (T)I.alpha, oma = (T)(1.0 - I.alpha);

  State S = *gst;  // every thread keeps its own copy of the scalars
  if (S.done) return;
  Reduce<BLOCK> reduce{scratch, 0};

  // Dual update of one finished row and the next iteration's residual inputs
  // (pdos.c:232-236, linAlg.h:158-175, indirect/private.c:20-29, :58-60).
  auto finish = [&](int r, T sv, T stv, T axv, double &pr2, double &byv) {
    const T yv = y[r] + (sv - stv) / lam;
    y[r] = yv;
    s[r] = sv;
    const T bv = b[r];
    const T pr = ((sv - bv) + axv) / D[r];
    pr2 += (double)pr * (double)pr;
    u[r] = ((sv + lam * yv) - bv) + axv;
    byv += (double)bv * (double)yv;
  };

  if (!S.prepped) {  // A x0: residual, u and b'y of iteration 0
    for (int j = tid; j < n; j += BLOCK) {
      if (SG) gs[j] = x[j];
      else g1[j] = x[j];
    }
    __syncthreads();
    double red[2] = {0.0, 0.0};
    hyb_product<T, BLOCK, 1>(I.hA, I.A, I.pvA, SG ? gs : g1, SG ? gs : g1, pbuf, [&](int r, T a, T) {
      ax[r] = a;
      const T sv = s[r], bv = b[r], yv = y[r];
      const T pr = ((sv - bv) + a) / D[r];
      red[0] += (double)pr * (double)pr;
      u[r] = ((sv + lam * yv) - bv) + a;
      red[1] += (double)bv * (double)yv;
    });
    reduce(red);
    S.pres_sq = red[0];
    S.by = red[1];
    S.prepped = 1;
  }

  bool newly_done = false;
  for (int it = 0; it < iter_cap; ++it) {
    // ---- top: A' on (y, u): dual residual, c'x, CG start; stop test
    double top[3] = {0.0, 0.0, 0.0};
    auto top_row = [&](int j, T sy, T su) {
      const T cj = c[j];
      const T dr = (cj + sy) / E[j];
      top[0] += (double)dr * (double)dr;
      top[1] += (double)cj * (double)x[j];
      const T qj = (-lam) * cj + (-su);
      q[j] = qj;
      top[2] += (double)qj * (double)qj;
    };
    if (SG) {  // A'y into tt, then A'u with the epilogue
      for (int r = tid; r < m; r += BLOCK) gs[r] = y[r];
      __syncthreads();
      hyb_product<T, BLOCK, 1>(I.hT, I.At, I.pvT, gs, gs, pbuf, [&](int j, T sy, T) { tt[j] = sy; });
      __syncthreads();
      for (int r = tid; r < m; r += BLOCK) gs[r] = u[r];
      __syncthreads();
      hyb_product<T, BLOCK, 1>(I.hT, I.At, I.pvT, gs, gs, pbuf, [&](int j, T su, T) { top_row(j, tt[j], su); });
    } else {
      for (int r = tid; r < m; r += BLOCK) {
        g1[r] = y[r];
        g2[r] = u[r];
      }
      __syncthreads();
      hyb_product<T, BLOCK, 2>(I.hT, I.At, I.pvT, g1, g2, pbuf, top_row);
    }
    reduce(top);
    S.p_res = sqrt(S.pres_sq);
    S.d_res = sqrt(top[0]);
    S.p_obj = top[1];
    S.d_obj = -S.by;
    S.eta = fabs(S.p_obj - S.d_obj);
    if (S.p_res < I.eps * I.pscale && S.d_res < I.eps * I.dscale &&
        S.eta < I.eps * (1.0 + fabs(S.p_obj) + fabs(S.d_obj))) {
      S.solved = 1;
      S.done = 1;
      newly_done = true;
      break;
    }
    // A non-finite residual or gap: this instance's iterate overflowed.  It
    // stops here and frees its CTA; its neighbours never read its vectors.
    if (!isfinite(S.p_res) || !isfinite(S.d_res) || !isfinite(S.eta)) {
      S.diverged = 1;
      S.done = 1;
      newly_done = true;
      break;
    }
    // ---- CG on (I + A'A) x = ... warm-started at x (indirect/private.c:31-104)
    double qsold = top[2];
    int cg_iter = 0;
    bool active = I.cg_max > 0 && qsold > I.tol_sq;
    if (active) {
      for (int j = tid; j < n; j += BLOCK) {  // p = q
        const T qj = q[j];
        g1[j] = qj;
        if (SG) gs[j] = qj;
      }
      __syncthreads();
    }
    while (active) {
      hyb_product<T, BLOCK, 1>(I.hA, I.A, I.pvA, SG ? gs : g1, SG ? gs : g1, pbuf,
                               [&](int r, T a, T) { g2[r] = a; });
      __syncthreads();
      if (SG) {  // A p is the next gather source
        for (int r = tid; r < m; r += BLOCK) gs[r] = g2[r];
        __syncthreads();
      }
      double pt[1] = {0.0};
      hyb_product<T, BLOCK, 1>(I.hT, I.At, I.pvT, SG ? gs : g2, SG ? gs : g2, pbuf, [&](int j, T a, T) {
        const T pj = g1[j];
        const T tj = pj + a;
        tt[j] = tj;
        pt[0] += (double)pj * (double)tj;
      });
      reduce(pt);
      const double step = qsold / pt[0];
      const T stp = (T)step, nstp = (T)(-step);
      double qs[1] = {0.0};
#pragma unroll 4
      for (int j = tid; j < n; j += BLOCK) {
        x[j] = x[j] + stp * g1[j];
        const T qj = q[j] + nstp * tt[j];
        q[j] = qj;
        qs[0] += (double)qj * (double)qj;
      }
      reduce(qs);
      ++cg_iter;
      ++S.cg_total;
      double ratio = 0.0;
      if (qs[0] < I.tol_sq) {
        active = false;
      } else {
        ratio = qs[0] / qsold;
        qsold = qs[0];
        if (cg_iter >= I.cg_max) active = false;
      }
      if (active) {
        const T beta = (T)ratio;
#pragma unroll 4
        for (int j = tid; j < n; j += BLOCK) {
          const T pj = beta * g1[j] + q[j];
          g1[j] = pj;
          if (SG) gs[j] = pj;
        }
        __syncthreads();
      }
    }
    // ---- A x: s~ = b - Ax, relax, s = s~ - lam y; zero / orthant rows done
    for (int j = tid; j < n; j += BLOCK) {
      if (SG) gs[j] = x[j];
      else g1[j] = x[j];
    }
    __syncthreads();
    double fin[2] = {0.0, 0.0};
    hyb_product<T, BLOCK, 1>(I.hA, I.A, I.pvA, SG ? gs : g1, SG ? gs : g1, pbuf, [&](int r, T a, T) {
      T stv = b[r] + (-a);
      stv = alpha * stv + oma * s[r];
      T v = stv - lam * y[r];
      ax[r] = a;
      if (r < f) {
        finish(r, T(0), stv, a, fin[0], fin[1]);
      } else if (r < f + l) {
        if (v < T(0)) v = T(0);
        finish(r, v, stv, a, fin[0], fin[1]);
      } else {
        s[r] = v;
        st[r] = stv;
      }
    });
    __syncthreads();
    // ---- second-order cones: a warp per small cone, the CTA per big cone
    {
      const int lane = tid & 31, warp = tid >> 5;
      for (int k = warp; k < I.ncones; k += BLOCK / 32) {
        const int off = B.cone_off[I.cone0 + k], len = B.cone_len[I.cone0 + k];
        if (len > kSmallCone) continue;
        T acc = T(0);
        for (int i = 1 + lane; i < len; i += 32) {
          const T v = s[off + i];
          acc += v * v;
        }
        acc = warp_sum_t(acc);
        const T tail = sqrt(acc);
        const T head = s[off];
        __syncwarp();
        for (int i = lane; i < len; i += 32) {
          const int r = off + i;
          finish(r, soc_rule(s[r], i == 0, head, tail), st[r], ax[r], fin[0], fin[1]);
        }
      }
      for (int k = 0; k < I.ncones; ++k) {  // uniform over the CTA
        const int off = B.cone_off[I.cone0 + k], len = B.cone_len[I.cone0 + k];
        if (len <= kSmallCone) continue;
        const T head = s[off];  // read before any thread rewrites the cone
        double acc[1] = {0.0};
        for (int i = 1 + tid; i < len; i += BLOCK) {
          const T v = s[off + i];
          acc[0] += (double)(v * v);
        }
        reduce(acc);
        const T tail = (T)sqrt(acc[0]);
        for (int i = tid; i < len; i += BLOCK) {
          const int r = off + i;
          finish(r, soc_rule(s[r], i == 0, head, tail), st[r], ax[r], fin[0], fin[1]);
        }
      }
    }
    reduce(fin);
    S.pres_sq = fin[0];
    S.by = fin[1];
    S.admm_iter += 1;
    if (S.admm_iter >= I.max_iters) {
      S.done = 1;
      newly_done = true;
      break;
    }
  }
  __syncthreads();
  if (tid == 0) {
    *gst = S;
    if (newly_done) atomicAdd(B.ndone, 1);
  }
}

// Staging modes of a kernel instantiation: 0 = everything in shared memory;
// 1 = regions in global memory, the gather vector in shared memory (a
// global-staging class whose every member's max(m, n) fits); 2 = regions and
// gathers in global memory.  One mode per kernel keeps one code path, and
// its registers, per instantiation.
constexpr int kStageShared = 0, kStageGlobalSG = 1, kStageGlobal = 2;

template <typename T, int BLOCK, int MODE>
__global__ void __launch_bounds__(BLOCK, 1024 / BLOCK) batch_admm_kernel(Dev<T> B, int cls, Smem sm, int iter_cap) {
  constexpr bool GLOBAL = MODE != kStageShared;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ double scratch[2 * 3 * (BLOCK / 32)];
  __shared__ Inst s_inst;
  __shared__ int s_k;
  T *gs = reinterpret_cast<T *>(smem_raw);  // global class: the gather vector
  T *g1 = staging_base<T, GLOBAL>(sm, smem_raw, B.gscratch);
  T *g2 = g1 + sm.g1;
  T *tt = g2 + sm.g2;
  T *pbuf = tt + sm.tt;
  const int begin = B.class_begin[cls], count = B.class_begin[cls + 1] - begin;
  for (;;) {
    __syncthreads();
    if (threadIdx.x == 0) s_k = atomicAdd(&B.queue[cls], 1);
    __syncthreads();
    const int k = s_k;
    if (k >= count) break;
    const int id = B.order[begin + k];
    if (threadIdx.x < (int)(sizeof(Inst) / 4))
      reinterpret_cast<int32_t *>(&s_inst)[threadIdx.x] =
          reinterpret_cast<const int32_t *>(B.inst + id)[threadIdx.x];
    __syncthreads();
    solve_instance<T, BLOCK, MODE == kStageGlobalSG>(B, s_inst, B.state + id, iter_cap, g1, g2, tt, pbuf, scratch,
                                                     gs);
  }
}

// The two CG products alone (u = A p, t = p + A'u), `reps` times for every
// instance of a class, for the roofline of the batch's SpMV: no reductions,
// no stop test, the iterate untouched (p is the current x).
template <typename T, int BLOCK, int MODE>
__global__ void __launch_bounds__(BLOCK, 1024 / BLOCK) batch_products_kernel(Dev<T> B, int cls, Smem sm,
                                                                              int reps) {
  constexpr bool GLOBAL = MODE != kStageShared;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ Inst s_inst;
  __shared__ int s_k;
  T *gs = reinterpret_cast<T *>(smem_raw);  // global class: the gather vector
  T *g1 = staging_base<T, GLOBAL>(sm, smem_raw, B.gscratch);
  T *g2 = g1 + sm.g1;
  T *tt = g2 + sm.g2;
  T *pbuf = tt + sm.tt;
  const int begin = B.class_begin[cls], count = B.class_begin[cls + 1] - begin;
  for (;;) {
    __syncthreads();
    if (threadIdx.x == 0) s_k = atomicAdd(&B.queue[cls], 1);
    __syncthreads();
    const int k = s_k;
    if (k >= count) break;
    const int id = B.order[begin + k];
    if (threadIdx.x < (int)(sizeof(Inst) / 4))
      reinterpret_cast<int32_t *>(&s_inst)[threadIdx.x] =
          reinterpret_cast<const int32_t *>(B.inst + id)[threadIdx.x];
    __syncthreads();
    const Inst &I = s_inst;
    const T *x = B.x + I.col0;
    constexpr bool sg = MODE == kStageGlobalSG;  // gathers from shared memory
    for (int j = threadIdx.x; j < I.n; j += BLOCK) g1[j] = x[j];
    __syncthreads();
    for (int r = 0; r < reps; ++r) {
      if (sg) {
        for (int j = threadIdx.x; j < I.n; j += BLOCK) gs[j] = g1[j];
        __syncthreads();
      }
      hyb_product<T, BLOCK, 1>(I.hA, I.A, I.pvA, sg ? gs : g1, sg ? gs : g1, pbuf,
                               [&](int row, T a, T) { g2[row] = a; });
      __syncthreads();
      if (sg) {
        for (int j = threadIdx.x; j < I.m; j += BLOCK) gs[j] = g2[j];
        __syncthreads();
      }
      hyb_product<T, BLOCK, 1>(I.hT, I.At, I.pvT, sg ? gs : g2, sg ? gs : g2, pbuf,
                               [&](int j, T a, T) { tt[j] = g1[j] + a; });
      __syncthreads();
    }
  }
}

static_assert(sizeof(Inst) % 4 == 0 && sizeof(Inst) / 4 <= 128, "Inst is copied by one 128-thread pass");
static_assert(alignof(Inst) == 8, "Inst is copied as 32-bit words into an 8-byte aligned slot");

// ------------------------------------------------------------------ pairs
// Two instances of one family group (one shared layout, the same sizes and
// cones) solved together by one CTA: every streamed load of the shared
// layout serves both, their vectors sit interleaved in shared memory so one
// 8-byte (FP32) gather feeds both FMA chains, and each instance keeps its
// own per-row sums, in the order of the one-instance kernel, and its own
// block sums -- so each result is bit for bit the one-instance result.  The
// two run in lockstep; an instance that stops (or an empty second slot)
// keeps flowing through the products with its writes masked.
template <typename T>
struct alignas(2 * sizeof(T)) P2 {
  T a, b;
};

template <typename T>
__device__ __forceinline__ P2<T> warp_sum_p(P2<T> v) {
  return P2<T>{warp_sum_t(v.a), warp_sum_t(v.b)};
}

template <typename T, int NV>
__device__ __forceinline__ void fma4_pair(const Idx4 &j, const Val4<T> &v0, const Val4<T> &v1, const P2<T> *s0,
                                          const P2<T> *s1, P2<T> &a0, P2<T> &a1) {
  const int jj[4] = {j.x, j.y, j.z, j.w};
  const T w0[4] = {v0.x, v0.y, v0.z, v0.w}, w1[4] = {v1.x, v1.y, v1.z, v1.w};
#pragma unroll
  for (int e = 0; e < 4; ++e) {
    const P2<T> g = s0[jj[e]];
    a0.a = fma(w0[e], g.a, a0.a);
    a0.b = fma(w1[e], g.b, a0.b);
    if (NV == 2) {
      const P2<T> h = s1[jj[e]];
      a1.a = fma(w0[e], h.a, a1.a);
      a1.b = fma(w1[e], h.b, a1.b);
    }
  }
}

// The values of four loaded entries for each of the two instances: the
// shared ones, or each instance's own where a NaN box marks a varying entry.
template <typename T>
__device__ __forceinline__ void unbox4_pair(const Val4<T> &v, const T *pv0, const T *pv1, Val4<T> &v0,
                                            Val4<T> &v1) {
  v0 = v;
  v1 = v;
  unbox4(v0, pv0);
  unbox4(v1, pv1);
}

// One product over one side, for both instances of a pair; epi(row, s0, s1)
// gets each source vector's pair of sums.
template <typename T, int BLOCK, int NV, class Epi>
__device__ __forceinline__ void pair_product(const HybPtr &H, const Side &sd, const T *pv0, const T *pv1,
                                             const P2<T> *src0, const P2<T> *src1, P2<T> *pbuf, Epi &&epi) {
  constexpr int W = BLOCK / 32;
  const T *const hval = static_cast<const T *>(H.val);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int k = warp; k < sd.npieces; k += W) {
    const int64_t pk = sd.piece0 + k;
    const int32_t prow = H.piece_row[pk];
    const int64_t beg = H.piece_beg[pk];
    const int len = H.piece_len[pk];
    P2<T> a0{T(0), T(0)}, a1{T(0), T(0)};
    const uint16_t *ip = H.idx + beg;
    const T *vp = hval + beg;
#pragma unroll kUnroll
    for (int e = 4 * lane; e < len; e += 128) {
      const Idx4 j = ld_stream4(ip + e);
      Val4<T> v0, v1;
      unbox4_pair(ld_stream4(vp + e), pv0, pv1, v0, v1);
      fma4_pair<T, NV>(j, v0, v1, src0, src1, a0, a1);
    }
    a0 = warp_sum_p(a0);
    if (NV == 2) a1 = warp_sum_p(a1);
    if (lane == 0) {
      if (prow >= 0) {
        epi(prow, a0, a1);
      } else {
        pbuf[k * NV] = a0;
        if (NV == 2) pbuf[k * NV + 1] = a1;
      }
    }
  }
  for (int s = warp; s < sd.nslices; s += W) {
    const int64_t sk = sd.slice0 + s;
    const int64_t off = H.slice_beg[sk];
    const int width = H.slice_w[sk];
    P2<T> a0{T(0), T(0)}, a1{T(0), T(0)};
    if (width < 0) {
      const uint16_t *ip = H.idx + off + 4 * lane;
      const T *vp = hval + off + 4 * lane;
#pragma unroll kUnroll
      for (int c4 = 0; c4 < -width; c4 += 4) {
        const Idx4 j = ld_stream4(ip + 32 * c4);
        Val4<T> v0, v1;
        unbox4_pair(ld_stream4(vp + 32 * c4), pv0, pv1, v0, v1);
        fma4_pair<T, NV>(j, v0, v1, src0, src1, a0, a1);
      }
    } else {
      const uint16_t *ip = H.idx + off + lane;
      const T *vp = hval + off + lane;
      for (int c = 0; c < width; ++c) {
        const int j = ip[c * 32];
        const T v = vp[c * 32];
        const T v0 = unbox(v, pv0), v1 = unbox(v, pv1);
        const P2<T> g = src0[j];
        a0.a = fma(v0, g.a, a0.a);
        a0.b = fma(v1, g.b, a0.b);
        if (NV == 2) {
          const P2<T> h = src1[j];
          a1.a = fma(v0, h.a, a1.a);
          a1.b = fma(v1, h.b, a1.b);
        }
      }
    }
    if (!((H.slice_skip[sk] >> lane) & 1u))
      epi(sd.sorted ? (int)H.slice_row[sk * 32 + lane] : s * 32 + lane, a0, a1);  // the lane's row
  }
  if (sd.nsplit > 0) {
    __syncthreads();
    for (int k = threadIdx.x; k < sd.nsplit; k += BLOCK) {
      const int64_t sk = sd.split0 + k;
      const int p0 = H.split_p0[sk], np = H.split_np[sk];
      P2<T> a0{T(0), T(0)}, a1{T(0), T(0)};
      for (int t = 0; t < np; ++t) {
        const P2<T> u0 = pbuf[(p0 + t) * NV];
        a0.a += u0.a;
        a0.b += u0.b;
        if (NV == 2) {
          const P2<T> u1 = pbuf[(p0 + t) * NV + 1];
          a1.a += u1.a;
          a1.b += u1.b;
        }
      }
      epi(H.split_row[sk], a0, a1);
    }
  }
}

// Per-instance pointers of one slot of a pair.
template <typename T>
struct Slot {
  T *x, *q, *s, *y, *st, *u, *ax;
  const T *b, *c, *D, *E;
  T lam, alpha, oma;
};

// sl: the two slots' pointers in shared memory (read where used, so they
// need no registers across the loops).
template <typename T, int BLOCK>
__device__ void solve_pair(const Dev<T> &B, const Inst *I2, State *gst0, State *gst1, int iter_cap, P2<T> *g1,
                           P2<T> *g2, P2<T> *tt, P2<T> *pbuf, double *scratch, Slot<T> *sl) {
  const int tid = threadIdx.x;
  const Inst &I = I2[0];  // layout, sizes and cones of both
  const int m = I.m, n = I.n, f = I.f, l = I.l;
  const bool two = gst1 != nullptr;
  if (tid < 2) {
    const Inst &J = I2[tid];
    sl[tid] = Slot<T>{B.x + J.col0, B.q + J.col0, B.s + J.row0, B.y + J.row0, B.st + J.row0, B.u + J.row0,
                      B.ax + J.row0, B.b + J.row0, B.c + J.col0, B.D + J.row0, B.E + J.col0, (T)J.lambda,
                      (T)J.alpha, (T)(1.0 - J.alpha)};
  }
  __syncthreads();
  const T *pvA0 = static_cast<const T *>(I2[0].pvA), *pvA1 = static_cast<const T *>(I2[1].pvA);
  const T *pvT0 = static_cast<const T *>(I2[0].pvT), *pvT1 = static_cast<const T *>(I2[1].pvT);
  State S[2] = {*gst0, two ? *gst1 : *gst0};
  bool act[2] = {!S[0].done, two && !S[1].done};  // instances still iterating
  bool newly[2] = {false, false};
  if (!act[0] && !act[1]) return;
  Reduce<BLOCK, 6> reduce{scratch, 0};

  // dual update and next residual inputs of one row of slot g (pdos.c:232-236,
  // linAlg.h:158-175, indirect/private.c:20-29, :58-60)
  auto finish = [&](int g, int r, T sv, T stv, T axv, double &pr2, double &byv) {
    const Slot<T> &z = sl[g];
    const T yv = z.y[r] + (sv - stv) / z.lam;
    z.y[r] = yv;
    z.s[r] = sv;
    const T bv = z.b[r];
    const T pr = ((sv - bv) + axv) / z.D[r];
    pr2 += (double)pr * (double)pr;
    z.u[r] = ((sv + z.lam * yv) - bv) + axv;
    byv += (double)bv * (double)yv;
  };
  // interleaved copy of one vector of both slots into a pair array
  auto stage = [&](P2<T> *dst, int len, T *const Slot<T>::*field) {
    for (int j = tid; j < len; j += BLOCK) dst[j] = P2<T>{(sl[0].*field)[j], (sl[1].*field)[j]};
  };

  if (!S[0].prepped || (two && !S[1].prepped)) {  // A x0 of each slot not yet prepared
    stage(g1, n, &Slot<T>::x);
    __syncthreads();
    double red[4] = {0.0, 0.0, 0.0, 0.0};
    pair_product<T, BLOCK, 1>(I.hA, I.A, pvA0, pvA1, g1, g1, pbuf, [&](int r, P2<T> a, P2<T>) {
      const T av[2] = {a.a, a.b};
#pragma unroll
      for (int g = 0; g < 2; ++g) {
        if (!act[g] || S[g].prepped) continue;
        const Slot<T> &z = sl[g];
        z.ax[r] = av[g];
        const T sv = z.s[r], bv = z.b[r], yv = z.y[r];
        const T pr = ((sv - bv) + av[g]) / z.D[r];
        red[2 * g] += (double)pr * (double)pr;
        z.u[r] = ((sv + z.lam * yv) - bv) + av[g];
        red[2 * g + 1] += (double)bv * (double)yv;
      }
    });
    reduce(red);
#pragma unroll
    for (int g = 0; g < 2; ++g) {
      if (!act[g] || S[g].prepped) continue;
      S[g].pres_sq = red[2 * g];
      S[g].by = red[2 * g + 1];
      S[g].prepped = 1;
    }
  }

  for (int it = 0; it < iter_cap && (act[0] || act[1]); ++it) {
    // ---- top: A' on (y, u): dual residual, c'x, CG start; stop test
    for (int r = tid; r < m; r += BLOCK) {
      g1[r] = P2<T>{sl[0].y[r], sl[1].y[r]};
      g2[r] = P2<T>{sl[0].u[r], sl[1].u[r]};
    }
    __syncthreads();
    double top[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    pair_product<T, BLOCK, 2>(I.hT, I.At, pvT0, pvT1, g1, g2, pbuf, [&](int j, P2<T> sy, P2<T> su) {
      const T syv[2] = {sy.a, sy.b}, suv[2] = {su.a, su.b};
#pragma unroll
      for (int g = 0; g < 2; ++g) {
        if (!act[g]) continue;
        const Slot<T> &z = sl[g];
        const T cj = z.c[j];
        const T dr = (cj + syv[g]) / z.E[j];
        top[3 * g] += (double)dr * (double)dr;
        top[3 * g + 1] += (double)cj * (double)z.x[j];
        const T qj = (-z.lam) * cj + (-suv[g]);
        z.q[j] = qj;
        top[3 * g + 2] += (double)qj * (double)qj;
      }
    });
    reduce(top);
    double qsold[2] = {top[2], top[5]};
    int cg_iter[2] = {0, 0};
    bool cg_on[2] = {false, false};
#pragma unroll
    for (int g = 0; g < 2; ++g) {
      if (!act[g]) continue;
      const Inst &J = I2[g];
      State &Z = S[g];
      Z.p_res = sqrt(Z.pres_sq);
      Z.d_res = sqrt(top[3 * g]);
      Z.p_obj = top[3 * g + 1];
      Z.d_obj = -Z.by;
      Z.eta = fabs(Z.p_obj - Z.d_obj);
      if (Z.p_res < J.eps * J.pscale && Z.d_res < J.eps * J.dscale &&
          Z.eta < J.eps * (1.0 + fabs(Z.p_obj) + fabs(Z.d_obj))) {
        Z.solved = 1;
        Z.done = 1;
        newly[g] = true;
        act[g] = false;
      } else if (!isfinite(Z.p_res) || !isfinite(Z.d_res) || !isfinite(Z.eta)) {
        Z.diverged = 1;
        Z.done = 1;
        newly[g] = true;
        act[g] = false;
      } else {
        cg_on[g] = J.cg_max > 0 && qsold[g] > J.tol_sq;
      }
    }
    if (!act[0] && !act[1]) break;
    // ---- CG on (I + A'A) x = ... warm-started at x (indirect/private.c:31-104)
    if (cg_on[0] || cg_on[1]) {
      for (int j = tid; j < n; j += BLOCK) {  // p = q (a finished slot keeps its p)
        P2<T> pj = g1[j];
        if (cg_on[0]) pj.a = sl[0].q[j];
        if (cg_on[1]) pj.b = sl[1].q[j];
        g1[j] = pj;
      }
      __syncthreads();
    }
    while (cg_on[0] || cg_on[1]) {
      pair_product<T, BLOCK, 1>(I.hA, I.A, pvA0, pvA1, g1, g1, pbuf, [&](int r, P2<T> a, P2<T>) { g2[r] = a; });
      __syncthreads();
      double pt[2] = {0.0, 0.0};
      pair_product<T, BLOCK, 1>(I.hT, I.At, pvT0, pvT1, g2, g2, pbuf, [&](int j, P2<T> a, P2<T>) {
        const P2<T> pj = g1[j];
        const P2<T> tj{pj.a + a.a, pj.b + a.b};
        tt[j] = tj;
        pt[0] += (double)pj.a * (double)tj.a;
        pt[1] += (double)pj.b * (double)tj.b;
      });
      reduce(pt);
      T stp[2], nstp[2];
#pragma unroll
      for (int g = 0; g < 2; ++g) {
        const double step = cg_on[g] ? qsold[g] / pt[g] : 0.0;
        stp[g] = (T)step;
        nstp[g] = (T)(-step);
      }
      double qs[2] = {0.0, 0.0};
#pragma unroll 2
      for (int j = tid; j < n; j += BLOCK) {
        const P2<T> pj = g1[j], tj = tt[j];
        if (cg_on[0]) {
          sl[0].x[j] = sl[0].x[j] + stp[0] * pj.a;
          const T qj = sl[0].q[j] + nstp[0] * tj.a;
          sl[0].q[j] = qj;
          qs[0] += (double)qj * (double)qj;
        }
        if (cg_on[1]) {
          sl[1].x[j] = sl[1].x[j] + stp[1] * pj.b;
          const T qj = sl[1].q[j] + nstp[1] * tj.b;
          sl[1].q[j] = qj;
          qs[1] += (double)qj * (double)qj;
        }
      }
      reduce(qs);
      T beta[2] = {T(0), T(0)};
#pragma unroll
      for (int g = 0; g < 2; ++g) {
        if (!cg_on[g]) continue;
        ++cg_iter[g];
        ++S[g].cg_total;
        if (qs[g] < I2[g].tol_sq) {
          cg_on[g] = false;
        } else {
          beta[g] = (T)(qs[g] / qsold[g]);
          qsold[g] = qs[g];
          if (cg_iter[g] >= I2[g].cg_max) cg_on[g] = false;
        }
      }
      if (cg_on[0] || cg_on[1]) {
#pragma unroll 2
        for (int j = tid; j < n; j += BLOCK) {
          P2<T> pj = g1[j];
          if (cg_on[0]) pj.a = beta[0] * pj.a + sl[0].q[j];
          if (cg_on[1]) pj.b = beta[1] * pj.b + sl[1].q[j];
          g1[j] = pj;
        }
        __syncthreads();
      }
    }
    // ---- A x: s~ = b - Ax, relax, s = s~ - lam y; zero / orthant rows done
    stage(g1, n, &Slot<T>::x);
    __syncthreads();
    double fin[4] = {0.0, 0.0, 0.0, 0.0};
    pair_product<T, BLOCK, 1>(I.hA, I.A, pvA0, pvA1, g1, g1, pbuf, [&](int r, P2<T> a, P2<T>) {
      const T av[2] = {a.a, a.b};
#pragma unroll
      for (int g = 0; g < 2; ++g) {
        if (!act[g]) continue;
        const Slot<T> &z = sl[g];
        T stv = z.b[r] + (-av[g]);
        stv = z.alpha * stv + z.oma * z.s[r];
        T v = stv - z.lam * z.y[r];
        z.ax[r] = av[g];
        if (r < f) {
          finish(g, r, T(0), stv, av[g], fin[2 * g], fin[2 * g + 1]);
        } else if (r < f + l) {
          if (v < T(0)) v = T(0);
          finish(g, r, v, stv, av[g], fin[2 * g], fin[2 * g + 1]);
        } else {
          z.s[r] = v;
          z.st[r] = stv;
        }
      }
    });
    __syncthreads();
    // ---- second-order cones: a warp per small cone, the CTA per big cone
    {
      const int lane = tid & 31, warp = tid >> 5;
#pragma unroll
      for (int g = 0; g < 2; ++g) {
        if (!act[g]) continue;
        const Slot<T> &z = sl[g];
        for (int k = warp; k < I.ncones; k += BLOCK / 32) {
          const int off = B.cone_off[I.cone0 + k], len = B.cone_len[I.cone0 + k];
          if (len > kSmallCone) continue;
          T acc = T(0);
          for (int i = 1 + lane; i < len; i += 32) {
            const T v = z.s[off + i];
            acc += v * v;
          }
          acc = warp_sum_t(acc);
          const T tail = sqrt(acc);
          const T head = z.s[off];
          __syncwarp();
          for (int i = lane; i < len; i += 32) {
            const int r = off + i;
            finish(g, r, soc_rule(z.s[r], i == 0, head, tail), z.st[r], z.ax[r], fin[2 * g], fin[2 * g + 1]);
          }
        }
      }
      for (int k = 0; k < I.ncones; ++k) {  // uniform over the CTA
        const int off = B.cone_off[I.cone0 + k], len = B.cone_len[I.cone0 + k];
        if (len <= kSmallCone) continue;
        T head[2];
        double acc[2] = {0.0, 0.0};
#pragma unroll
        for (int g = 0; g < 2; ++g) {
          head[g] = sl[g].s[off];  // read before any thread rewrites the cone
          if (!act[g]) continue;
          for (int i = 1 + tid; i < len; i += BLOCK) {
            const T v = sl[g].s[off + i];
            acc[g] += (double)(v * v);
          }
        }
        reduce(acc);
#pragma unroll
        for (int g = 0; g < 2; ++g) {
          if (!act[g]) continue;
          const Slot<T> &z = sl[g];
          const T tail = (T)sqrt(acc[g]);
          for (int i = tid; i < len; i += BLOCK) {
            const int r = off + i;
            finish(g, r, soc_rule(z.s[r], i == 0, head[g], tail), z.st[r], z.ax[r], fin[2 * g], fin[2 * g + 1]);
          }
        }
      }
    }
    reduce(fin);
#pragma unroll
    for (int g = 0; g < 2; ++g) {
      if (!act[g]) continue;
      S[g].pres_sq = fin[2 * g];
      S[g].by = fin[2 * g + 1];
      S[g].admm_iter += 1;
      if (S[g].admm_iter >= I2[g].max_iters) {
        S[g].done = 1;
        newly[g] = true;
        act[g] = false;
      }
    }
  }
  __syncthreads();
  if (tid == 0) {
    *gst0 = S[0];
    if (newly[0]) atomicAdd(B.ndone, 1);
    if (two) {
      *gst1 = S[1];
      if (newly[1]) atomicAdd(B.ndone, 1);
    }
  }
}

// The persistent kernel of a class whose work items are pairs of one family
// group (order[2k], order[2k+1]; -1 for an empty second slot).  Its shared
// memory holds the staging regions of two instances, interleaved.
template <typename T, int BLOCK>
__global__ void __launch_bounds__(BLOCK, 1024 / BLOCK) batch_pair_kernel(Dev<T> B, int cls, Smem sm, int iter_cap) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ double scratch[2 * 6 * (BLOCK / 32)];
  __shared__ Inst s_inst[2];
  __shared__ Slot<T> s_slot[2];
  __shared__ int s_k;
  P2<T> *g1 = reinterpret_cast<P2<T> *>(smem_raw);
  P2<T> *g2 = g1 + sm.g1;
  P2<T> *tt = g2 + sm.g2;
  P2<T> *pbuf = tt + sm.tt;
  const int begin = B.class_begin[cls], items = (B.class_begin[cls + 1] - begin) / 2;
  for (;;) {
    __syncthreads();
    if (threadIdx.x == 0) s_k = atomicAdd(&B.queue[cls], 1);
    __syncthreads();
    const int k = s_k;
    if (k >= items) break;
    const int id0 = B.order[begin + 2 * k], id1 = B.order[begin + 2 * k + 1];
    constexpr int kWords = (int)(sizeof(Inst) / 4);
    for (int t = threadIdx.x; t < 2 * kWords; t += BLOCK) {
      const int g = t / kWords, w = t % kWords;
      const int id = (g == 1 && id1 >= 0) ? id1 : id0;
      reinterpret_cast<int32_t *>(&s_inst[g])[w] = reinterpret_cast<const int32_t *>(B.inst + id)[w];
    }
    __syncthreads();
    solve_pair<T, BLOCK>(B, s_inst, B.state + id0, id1 >= 0 ? B.state + id1 : nullptr, iter_cap, g1, g2, tt, pbuf,
                         scratch, s_slot);
  }
}

// The two CG products alone for a paired class (roofline timing).
template <typename T, int BLOCK>
__global__ void __launch_bounds__(BLOCK, 1024 / BLOCK) batch_pair_products_kernel(Dev<T> B, int cls, Smem sm,
                                                                                   int reps) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ Inst s_inst[2];
  __shared__ int s_k;
  P2<T> *g1 = reinterpret_cast<P2<T> *>(smem_raw);
  P2<T> *g2 = g1 + sm.g1;
  P2<T> *tt = g2 + sm.g2;
  P2<T> *pbuf = tt + sm.tt;
  const int begin = B.class_begin[cls], items = (B.class_begin[cls + 1] - begin) / 2;
  for (;;) {
    __syncthreads();
    if (threadIdx.x == 0) s_k = atomicAdd(&B.queue[cls], 1);
    __syncthreads();
    const int k = s_k;
    if (k >= items) break;
    const int id0 = B.order[begin + 2 * k], id1 = B.order[begin + 2 * k + 1];
    constexpr int kWords = (int)(sizeof(Inst) / 4);
    for (int t = threadIdx.x; t < 2 * kWords; t += BLOCK) {
      const int g = t / kWords, w = t % kWords;
      const int id = (g == 1 && id1 >= 0) ? id1 : id0;
      reinterpret_cast<int32_t *>(&s_inst[g])[w] = reinterpret_cast<const int32_t *>(B.inst + id)[w];
    }
    __syncthreads();
    const Inst &I = s_inst[0];
    const T *x0 = B.x + s_inst[0].col0, *x1 = B.x + s_inst[1].col0;
    const T *pvA0 = static_cast<const T *>(s_inst[0].pvA), *pvA1 = static_cast<const T *>(s_inst[1].pvA);
    const T *pvT0 = static_cast<const T *>(s_inst[0].pvT), *pvT1 = static_cast<const T *>(s_inst[1].pvT);
    for (int j = threadIdx.x; j < I.n; j += BLOCK) g1[j] = P2<T>{x0[j], x1[j]};
    __syncthreads();
    for (int r = 0; r < reps; ++r) {
      pair_product<T, BLOCK, 1>(I.hA, I.A, pvA0, pvA1, g1, g1, pbuf, [&](int row, P2<T> a, P2<T>) { g2[row] = a; });
      __syncthreads();
      pair_product<T, BLOCK, 1>(I.hT, I.At, pvT0, pvT1, g2, g2, pbuf, [&](int j, P2<T> a, P2<T>) {
        const P2<T> pj = g1[j];
        tt[j] = P2<T>{pj.a + a.a, pj.b + a.b};
      });
      __syncthreads();
    }
  }
}

// ---------------------------------------------------------------- clusters
// Large instances of the global-staging class run on a thread-block cluster
// of C CTAs (one per SM): the warps of the whole cluster share
// each product's pieces and slices, the element-wise loops are spread over
// the cluster's threads, every CTA copies the vector a product gathers from
// into its own shared memory, the staged vectors live in one global region
// per cluster, and hardware cluster barriers (release / acquire at cluster
// scope) order those global writes.  Block sums meet in CTA 0's shared
// memory through distributed shared memory, in rank order, so every thread
// of the cluster holds the same totals.  Per-row sums are those of the
// one-CTA kernel; only the order of the block sums differs.
// The cluster size is chosen at launch (cluster_ctas_for): a class of many
// instances runs on 2-CTA clusters (more clusters fit the device at once --
// its GPCs hold only 16 of their SMs in 8-CTA clusters -- and a cluster
// synchronises fewer CTAs), a class of few on 4 or 8, so that its instances
// still spread over the device; pdos() on one instance takes 8.
constexpr int kClusterMax = 8;  // portable cluster size limit
constexpr int kClusterCtasOne = 8;
inline int cluster_ctas_for(int members, int sms, bool one_instance) {
  if (one_instance) return kClusterCtasOne;
  if (members >= sms / 2) return 2;
  if (members >= sms / 4) return 4;
  return 8;
}

__device__ __forceinline__ int cluster_ctas() {
  uint32_t n;
  asm volatile("mov.u32 %0, %%cluster_nctarank;" : "=r"(n));
  return (int)n;
}

__device__ __forceinline__ uint32_t cluster_rank() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}
__device__ __forceinline__ void cluster_sync() {
  asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}
// Address of this CTA's shared variable `p` in the shared memory of CTA `rank`.
__device__ __forceinline__ uint32_t dsmem_addr(const void *p, uint32_t rank) {
  const uint32_t a = (uint32_t)__cvta_generic_to_shared(p);
  uint32_t r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(rank));
  return r;
}
__device__ __forceinline__ void st_dsmem(uint32_t addr, double v) {
  asm volatile("st.shared::cluster.f64 [%0], %1;" ::"r"(addr), "d"(v) : "memory");
}
__device__ __forceinline__ double ld_dsmem(uint32_t addr) {
  double v;
  asm volatile("ld.shared::cluster.f64 %0, [%1];" : "=d"(v) : "r"(addr) : "memory");
  return v;
}
__device__ __forceinline__ int ld_dsmem_i32(uint32_t addr) {
  int v;
  asm volatile("ld.shared::cluster.s32 %0, [%1];" : "=r"(v) : "r"(addr) : "memory");
  return v;
}

struct ClusterBarrier {
  __device__ void operator()() const { cluster_sync(); }
};

// Cluster sums of N values: each CTA's block sum (block_sum_n), CTA r's
// totals stored into slot r of CTA 0, a cluster barrier, then every warp
// loads the C slots into its lanes and runs the xor butterfly -- the same
// bits everywhere.  Two slot halves are used in turn, as in Reduce.
template <int BLOCK>
struct ClusterReduce {
  double *scratch;  // this CTA: 2 x 3 x BLOCK/32
  double *slots;    // every CTA's copy; CTA 0's is the one used: 2 x 3 x kClusterMax
  uint32_t rank;
  int C;            // CTAs in the cluster
  int half;
  template <int N>
  __device__ __forceinline__ void operator()(double (&v)[N]) {
    half ^= 1;
    block_sum_n<BLOCK, N>(v, scratch + half * 3 * (BLOCK / 32));
    if (threadIdx.x == 0) {
#pragma unroll
      for (int k = 0; k < N; ++k) st_dsmem(dsmem_addr(&slots[(half * 3 + k) * kClusterMax + rank], 0), v[k]);
    }
    cluster_sync();
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int k = 0; k < N; ++k)
      v[k] = warp_sum(lane < C ? ld_dsmem(dsmem_addr(&slots[(half * 3 + k) * kClusterMax + lane], 0)) : 0.0);
  }
};

// One instance on a cluster (global staging, gathers from each CTA's shared
// memory): the operations and their order are those of solve_instance with
// SG; rows are shared among the cluster's warps and element-wise loops
// among its threads.
template <typename T, int BLOCK>
__device__ void solve_instance_cluster(const Dev<T> &B, const Inst &I, State *gst, int iter_cap, T *g1, T *g2,
                                       T *tt, T *pbuf, double *scratch, double *slots, T *gs, uint32_t rank,
                                       int C) {
  constexpr int W = BLOCK / 32;
  const int CT = C * BLOCK;
  const int tid = threadIdx.x, warp = tid >> 5;
  const int ct = (int)rank * BLOCK + tid;  // thread index in the cluster
  const Part part{(int)rank * W + warp, C * W, ct, CT};
  const ClusterBarrier cbar;
  const int m = I.m, n = I.n, f = I.f, l = I.l;
  T *__restrict__ x = B.x + I.col0;
  T *__restrict__ q = B.q + I.col0;
  T *__restrict__ s = B.s + I.row0;
  T *__restrict__ y = B.y + I.row0;
  T *__restrict__ st = B.st + I.row0;
  T *__restrict__ u = B.u + I.row0;
  T *__restrict__ ax = B.ax + I.row0;
  const T *__restrict__ b = B.b + I.row0;
  const T *__restrict__ D = B.D + I.row0;
  const T *__restrict__ c = B.c + I.col0;
  const T *__restrict__ E = B.E + I.col0;
  const T lam = (T)I.lambda;
  const T alpha = (T)I.alpha, oma = (T)(1.0 - I.alpha);

  State S = *gst;  // the same in every thread of the cluster
  if (S.done) return;
  ClusterReduce<BLOCK> reduce{scratch, slots, rank, C, 0};

  auto finish = [&](int r, T sv, T stv, T axv, double &pr2, double &byv) {
    const T yv = y[r] + (sv - stv) / lam;
    y[r] = yv;
    s[r] = sv;
    const T bv = b[r];
    const T pr = ((sv - bv) + axv) / D[r];
    pr2 += (double)pr * (double)pr;
    u[r] = ((sv + lam * yv) - bv) + axv;
    byv += (double)bv * (double)yv;
  };
  // every CTA copies a complete vector (ordered by an earlier cluster
  // barrier) into its own shared memory
  auto to_gs = [&](const T *src, int len) {
    for (int j = tid; j < len; j += BLOCK) gs[j] = src[j];
    __syncthreads();
  };

  if (!S.prepped) {  // A x0: residual, u and b'y of iteration 0
    to_gs(x, n);
    double red[2] = {0.0, 0.0};
    hyb_product_part<T, 1>(I.hA, I.A, I.pvA, gs, gs, pbuf, part, cbar, [&](int r, T a, T) {
      ax[r] = a;
      const T sv = s[r], bv = b[r], yv = y[r];
      const T pr = ((sv - bv) + a) / D[r];
      red[0] += (double)pr * (double)pr;
      u[r] = ((sv + lam * yv) - bv) + a;
      red[1] += (double)bv * (double)yv;
    });
    reduce(red);
    S.pres_sq = red[0];
    S.by = red[1];
    S.prepped = 1;
  }

  bool newly_done = false;
  for (int it = 0; it < iter_cap; ++it) {
    // ---- top: A'y into tt, then A'u with the epilogue (dual residual,
    // c'x, CG start); the same thread handles row j in both passes
    to_gs(y, m);
    hyb_product_part<T, 1>(I.hT, I.At, I.pvT, gs, gs, pbuf, part, cbar, [&](int j, T sy, T) { tt[j] = sy; });
    cluster_sync();  // every CTA has read the piece partials before the next product rewrites them
    to_gs(u, m);
    double top[3] = {0.0, 0.0, 0.0};
    hyb_product_part<T, 1>(I.hT, I.At, I.pvT, gs, gs, pbuf, part, cbar, [&](int j, T su, T) {
      const T cj = c[j];
      const T dr = (cj + tt[j]) / E[j];
      top[0] += (double)dr * (double)dr;
      top[1] += (double)cj * (double)x[j];
      const T qj = (-lam) * cj + (-su);
      q[j] = qj;
      top[2] += (double)qj * (double)qj;
    });
    reduce(top);
    S.p_res = sqrt(S.pres_sq);
    S.d_res = sqrt(top[0]);
    S.p_obj = top[1];
    S.d_obj = -S.by;
    S.eta = fabs(S.p_obj - S.d_obj);
    if (S.p_res < I.eps * I.pscale && S.d_res < I.eps * I.dscale &&
        S.eta < I.eps * (1.0 + fabs(S.p_obj) + fabs(S.d_obj))) {
      S.solved = 1;
      S.done = 1;
      newly_done = true;
      break;
    }
    if (!isfinite(S.p_res) || !isfinite(S.d_res) || !isfinite(S.eta)) {
      S.diverged = 1;
      S.done = 1;
      newly_done = true;
      break;
    }
    // ---- CG (indirect/private.c:31-104)
    double qsold = top[2];
    int cg_iter = 0;
    bool active = I.cg_max > 0 && qsold > I.tol_sq;
    if (active) {
      for (int j = ct; j < n; j += CT) g1[j] = q[j];  // p = q
      cluster_sync();
      to_gs(g1, n);
    }
    while (active) {
      hyb_product_part<T, 1>(I.hA, I.A, I.pvA, gs, gs, pbuf, part, cbar, [&](int r, T a, T) { g2[r] = a; });
      cluster_sync();  // A p complete, every gather from p done
      to_gs(g2, m);
      double pt[1] = {0.0};
      hyb_product_part<T, 1>(I.hT, I.At, I.pvT, gs, gs, pbuf, part, cbar, [&](int j, T a, T) {
        const T pj = g1[j];
        const T tj = pj + a;
        tt[j] = tj;
        pt[0] += (double)pj * (double)tj;
      });
      reduce(pt);
      const double step = qsold / pt[0];
      const T stp = (T)step, nstp = (T)(-step);
      double qs[1] = {0.0};
      for (int j = ct; j < n; j += CT) {
        x[j] = x[j] + stp * g1[j];
        const T qj = q[j] + nstp * tt[j];
        q[j] = qj;
        qs[0] += (double)qj * (double)qj;
      }
      reduce(qs);
      ++cg_iter;
      ++S.cg_total;
      double ratio = 0.0;
      if (qs[0] < I.tol_sq) {
        active = false;
      } else {
        ratio = qs[0] / qsold;
        qsold = qs[0];
        if (cg_iter >= I.cg_max) active = false;
      }
      if (active) {
        const T beta = (T)ratio;
        for (int j = ct; j < n; j += CT) g1[j] = beta * g1[j] + q[j];
        cluster_sync();
        to_gs(g1, n);
      }
    }
    // ---- A x: s~ = b - Ax, relax, s = s~ - lam y; zero / orthant rows done
    cluster_sync();  // x complete and every gather of the CG products done
    to_gs(x, n);
    double fin[2] = {0.0, 0.0};
    hyb_product_part<T, 1>(I.hA, I.A, I.pvA, gs, gs, pbuf, part, cbar, [&](int r, T a, T) {
      T stv = b[r] + (-a);
      stv = alpha * stv + oma * s[r];
      T v = stv - lam * y[r];
      ax[r] = a;
      if (r < f) {
        finish(r, T(0), stv, a, fin[0], fin[1]);
      } else if (r < f + l) {
        if (v < T(0)) v = T(0);
        finish(r, v, stv, a, fin[0], fin[1]);
      } else {
        s[r] = v;
        st[r] = stv;
      }
    });
    cluster_sync();  // s and s~ of every cone row complete
    // ---- second-order cones: a warp per small cone, the cluster per big one
    {
      const int lane = tid & 31;
      for (int k = part.w0; k < I.ncones; k += part.ws) {
        const int off = B.cone_off[I.cone0 + k], len = B.cone_len[I.cone0 + k];
        if (len > kSmallCone) continue;
        T acc = T(0);
        for (int i = 1 + lane; i < len; i += 32) {
          const T v = s[off + i];
          acc += v * v;
        }
        acc = warp_sum_t(acc);
        const T tail = sqrt(acc);
        const T head = s[off];
        __syncwarp();
        for (int i = lane; i < len; i += 32) {
          const int r = off + i;
          finish(r, soc_rule(s[r], i == 0, head, tail), st[r], ax[r], fin[0], fin[1]);
        }
      }
      for (int k = 0; k < I.ncones; ++k) {  // uniform over the cluster
        const int off = B.cone_off[I.cone0 + k], len = B.cone_len[I.cone0 + k];
        if (len <= kSmallCone) continue;
        const T head = s[off];  // read before any thread rewrites the cone
        double acc[1] = {0.0};
        for (int i = 1 + ct; i < len; i += CT) {
          const T v = s[off + i];
          acc[0] += (double)(v * v);
        }
        reduce(acc);
        const T tail = (T)sqrt(acc[0]);
        for (int i = ct; i < len; i += CT) {
          const int r = off + i;
          finish(r, soc_rule(s[r], i == 0, head, tail), st[r], ax[r], fin[0], fin[1]);
        }
      }
    }
    reduce(fin);
    S.pres_sq = fin[0];
    S.by = fin[1];
    S.admm_iter += 1;
    if (S.admm_iter >= I.max_iters) {
      S.done = 1;
      newly_done = true;
      break;
    }
  }
  cluster_sync();
  if (rank == 0 && tid == 0) {
    *gst = S;
    if (newly_done) atomicAdd(B.ndone, 1);
  }
}

// The next instance of the class for the whole cluster: CTA 0 takes it from
// the queue and every CTA reads CTA 0's copy; the second barrier keeps CTA 0
// from overwriting it before everyone has read it.
__device__ __forceinline__ int cluster_next(int *queue, int *s_k, uint32_t rank) {
  if (rank == 0 && threadIdx.x == 0) *s_k = atomicAdd(queue, 1);
  cluster_sync();
  const int k = ld_dsmem_i32(dsmem_addr(s_k, 0));
  cluster_sync();
  return k;
}

template <typename T, int BLOCK>
__global__ void __launch_bounds__(BLOCK, 1) batch_cluster_kernel(Dev<T> B, int cls, Smem sm, int iter_cap) {
  const int C = cluster_ctas();
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ double scratch[2 * 3 * (BLOCK / 32)];
  __shared__ double slots[2 * 3 * kClusterMax];
  __shared__ Inst s_inst;
  __shared__ int s_k;
  const uint32_t rank = cluster_rank();
  T *gs = reinterpret_cast<T *>(smem_raw);
  T *g1 = B.gscratch + (size_t)(blockIdx.x / C) * sm.stride();
  T *g2 = g1 + sm.g1;
  T *tt = g2 + sm.g2;
  T *pbuf = tt + sm.tt;
  const int begin = B.class_begin[cls], count = B.class_begin[cls + 1] - begin;
  for (;;) {
    const int k = cluster_next(&B.queue[cls], &s_k, rank);
    if (k >= count) break;  // the same k in every CTA of the cluster
    const int id = B.order[begin + k];
    if (threadIdx.x < (int)(sizeof(Inst) / 4))
      reinterpret_cast<int32_t *>(&s_inst)[threadIdx.x] = reinterpret_cast<const int32_t *>(B.inst + id)[threadIdx.x];
    __syncthreads();
    solve_instance_cluster<T, BLOCK>(B, s_inst, B.state + id, iter_cap, g1, g2, tt, pbuf, scratch, slots, gs,
                                     rank, C);
  }
  cluster_sync();  // no CTA leaves while another may still read its shared memory
}

// The two CG products alone on clusters (roofline timing of that class).
template <typename T, int BLOCK>
__global__ void __launch_bounds__(BLOCK, 1) batch_cluster_products_kernel(Dev<T> B, int cls, Smem sm, int reps) {
  constexpr int W = BLOCK / 32;
  const int C = cluster_ctas();
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ Inst s_inst;
  __shared__ int s_k;
  const uint32_t rank = cluster_rank();
  T *gs = reinterpret_cast<T *>(smem_raw);
  T *g1 = B.gscratch + (size_t)(blockIdx.x / C) * sm.stride();
  T *g2 = g1 + sm.g1;
  T *tt = g2 + sm.g2;
  T *pbuf = tt + sm.tt;
  const Part part{(int)rank * W + (int)(threadIdx.x >> 5), C * W, (int)rank * BLOCK + (int)threadIdx.x, C * BLOCK};
  const ClusterBarrier cbar;
  const int begin = B.class_begin[cls], count = B.class_begin[cls + 1] - begin;
  for (;;) {
    const int k = cluster_next(&B.queue[cls], &s_k, rank);
    if (k >= count) break;
    const int id = B.order[begin + k];
    if (threadIdx.x < (int)(sizeof(Inst) / 4))
      reinterpret_cast<int32_t *>(&s_inst)[threadIdx.x] = reinterpret_cast<const int32_t *>(B.inst + id)[threadIdx.x];
    __syncthreads();
    const Inst &I = s_inst;
    const T *x = B.x + I.col0;
    for (int j = part.t0; j < I.n; j += part.ts) g1[j] = x[j];
    cluster_sync();
    for (int r = 0; r < reps; ++r) {
      for (int j = threadIdx.x; j < I.n; j += BLOCK) gs[j] = g1[j];
      __syncthreads();
      hyb_product_part<T, 1>(I.hA, I.A, I.pvA, gs, gs, pbuf, part, cbar, [&](int row, T a, T) { g2[row] = a; });
      cluster_sync();
      for (int j = threadIdx.x; j < I.m; j += BLOCK) gs[j] = g2[j];
      __syncthreads();
      hyb_product_part<T, 1>(I.hT, I.At, I.pvT, gs, gs, pbuf, part, cbar,
                             [&](int j, T a, T) { tt[j] = g1[j] + a; });
      cluster_sync();
    }
  }
  cluster_sync();
}

// y = D y-unscale etc. (pdos.c:261-294) over the stacked vectors.
template <typename T>
__global__ void unscale_kernel(const T *x, const T *s, const T *y, const double *D, const double *E,
                               int64_t n, int64_t m, double *out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n + m;
       i += (int64_t)gridDim.x * blockDim.x) {
    if (i < n) {
      out[i] = E[i] * (double)x[i];
    } else {
      const int64_t r = i - n;
      out[n + r] = (double)s[r] / D[r];
      out[n + m + r] = D[r] * (double)y[r];
    }
  }
}

// Warm start from device arrays (unscaled, stacked): the scaling of
// common.h:147-161 and the x-space ratio of common.h:185-192.
template <typename T>
__global__ void warm_start_kernel(const double *x0, const double *y0, const double *s0,
                                  const double *D, const double *Epre, int64_t n, int64_t m,
                                  T *xi, T *yi, T *si) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n + m;
       i += (int64_t)gridDim.x * blockDim.x) {
    if (i < n) {
      if (x0) xi[i] = (T)((x0[i] / Epre[i]) / kXRatio);
    } else {
      const int64_t r = i - n;
      if (y0) yi[r] = (T)(y0[r] / D[r]);
      if (s0) si[r] = (T)(s0[r] * D[r]);
    }
  }
}

// Layout values from their source positions: p >= 0 the value at p, -1
// padding (zero), p <= -2 the varying entry -2 - p of a family group (its
// NaN box).
template <typename T>
__global__ void gather_values_kernel(const int32_t *src, int64_t count, const T *from, T *to) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < count;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int32_t p = src[i];
    to[i] = p >= 0 ? from[p] : (p == -1 ? T(0) : nan_box(T(0), (uint32_t)(-2 - p)));
  }
}

// ------------------------------------------------------------ host side
// Uploads one side's layout of one wave; values are gathered on the device
// from the wave's (scaled) value array through the layout's source map.
template <typename T>
int upload_hyb(const HybBuild &hb, const T *values, DeviceArena &arena, cudaStream_t st, HybPtr &h,
               int64_t *bytes) {
  *bytes += (int64_t)(hb.slice_beg.size() * 8 + hb.slice_w.size() * 4 + hb.slice_skip.size() * 4 +
                      hb.piece_row.size() * 4 + hb.piece_beg.size() * 8 + hb.piece_len.size() * 4 +
                      hb.split_row.size() * 12 + hb.idx.size() * 2 + hb.src.size() * sizeof(T) +
                      (hb.any_sorted ? hb.slice_row.size() * 2 : 0));
  auto up = [&](auto **dst, const auto &v) -> int {
    using E = typename std::decay_t<decltype(v)>::value_type;
    E *p = nullptr;
    PDOS_TRY(arena.alloc(&p, v.size() + 1));
    if (!v.empty())
      PDOS_CUDA_TRY(cudaMemcpyAsync(p, v.data(), sizeof(E) * v.size(), cudaMemcpyHostToDevice, st));
    *dst = p;
    return PDOSGPU_OK;
  };
  int64_t *slice_beg, *piece_beg;
  uint32_t *slice_skip;
  int32_t *slice_w, *piece_row, *piece_len, *split_row, *split_p0, *split_np;
  uint16_t *idx;
  PDOS_TRY(up(&slice_beg, hb.slice_beg));
  PDOS_TRY(up(&slice_w, hb.slice_w));
  PDOS_TRY(up(&slice_skip, hb.slice_skip));
  PDOS_TRY(up(&piece_row, hb.piece_row));
  PDOS_TRY(up(&piece_beg, hb.piece_beg));
  PDOS_TRY(up(&piece_len, hb.piece_len));
  PDOS_TRY(up(&split_row, hb.split_row));
  PDOS_TRY(up(&split_p0, hb.split_p0));
  PDOS_TRY(up(&split_np, hb.split_np));
  PDOS_TRY(up(&idx, hb.idx));
  uint16_t *slice_row = nullptr;
  if (hb.any_sorted) PDOS_TRY(up(&slice_row, hb.slice_row));
  T *val = nullptr;
  PDOS_TRY(arena.alloc(&val, hb.src.size() + 1));
  if (!hb.src.empty()) {
    DeviceArena tmp;
    int32_t *src = nullptr;
    PDOS_TRY(tmp.alloc(&src, hb.src.size()));
    PDOS_CUDA_TRY(cudaMemcpyAsync(src, hb.src.data(), sizeof(int32_t) * hb.src.size(),
                                  cudaMemcpyHostToDevice, st));
    const int64_t cnt = (int64_t)hb.src.size();
    const int g = (int)std::min<int64_t>((cnt + 255) / 256, (int64_t)num_sms() * 16);
    gather_values_kernel<T><<<g, 256, 0, st>>>(src, cnt, values, val);
    PDOS_CUDA_TRY(cudaGetLastError());
    PDOS_CUDA_TRY(cudaStreamSynchronize(st));  // before src (and the host arrays) are freed
  }
  h = HybPtr{slice_beg, slice_w, slice_skip, piece_row, piece_beg, piece_len, split_row, split_p0,
             split_np, idx, val, slice_row};
  return PDOSGPU_OK;
}

inline double now_ms() {
  using namespace std::chrono;
  return duration<double, std::milli>(steady_clock::now().time_since_epoch()).count();
}

template <typename T>
using KernelOf = void (*)(Dev<T>, int, Smem, int);

// The persistent ADMM kernel and the product timing kernel of one CTA size
// and staging mode (nullptr: unsupported size).
template <typename T, int MODE>
KernelOf<T> admm_kernel_mode(int block) {
  switch (block) {
    case 128: return batch_admm_kernel<T, 128, MODE>;
    case 256: return batch_admm_kernel<T, 256, MODE>;
    case 512: return batch_admm_kernel<T, 512, MODE>;
    case 1024: return batch_admm_kernel<T, 1024, MODE>;
    default: return nullptr;
  }
}
template <typename T, int MODE>
KernelOf<T> products_kernel_mode(int block) {
  switch (block) {
    case 128: return batch_products_kernel<T, 128, MODE>;
    case 256: return batch_products_kernel<T, 256, MODE>;
    case 512: return batch_products_kernel<T, 512, MODE>;
    case 1024: return batch_products_kernel<T, 1024, MODE>;
    default: return nullptr;
  }
}
inline int stage_mode(const Smem &sm) {
  return !sm.global ? kStageShared : (sm.gs > 0 ? kStageGlobalSG : kStageGlobal);
}
// A global-staging class whose gather vectors fit shared memory runs on
// clusters, one instance per cluster.
inline bool on_clusters(const Smem &sm) { return stage_mode(sm) == kStageGlobalSG; }
template <typename T>
KernelOf<T> cluster_kernel_for(int block, bool products) {
  switch (block) {
    case 128: return products ? batch_cluster_products_kernel<T, 128> : batch_cluster_kernel<T, 128>;
    case 256: return products ? batch_cluster_products_kernel<T, 256> : batch_cluster_kernel<T, 256>;
    case 512: return products ? batch_cluster_products_kernel<T, 512> : batch_cluster_kernel<T, 512>;
    case 1024: return products ? batch_cluster_products_kernel<T, 1024> : batch_cluster_kernel<T, 1024>;
    default: return nullptr;
  }
}
inline cudaLaunchConfig_t cluster_config(int grid, int block, size_t bytes, cudaStream_t st,
                                         cudaLaunchAttribute *attr, int ctas) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)grid);
  cfg.blockDim = dim3((unsigned)block);
  cfg.dynamicSmemBytes = bytes;
  cfg.stream = st;
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = (unsigned)ctas;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cfg;
}
// Lets `kernel` take as much dynamic shared memory as the device allows a
// block beside the kernel's own static shared memory; PDOSGPU_ENOTSUP when
// `need` bytes do not fit (a CTA size the tuner then skips).
template <typename K>
int allow_dynamic_smem(K kernel, size_t need) {
  cudaFuncAttributes a{};
  PDOS_CUDA_TRY(cudaFuncGetAttributes(&a, (const void *)kernel));
  int dev = 0, optin = 0;
  PDOS_CUDA_TRY(cudaGetDevice(&dev));
  PDOS_CUDA_TRY(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  const size_t room = (size_t)optin > a.sharedSizeBytes ? (size_t)optin - a.sharedSizeBytes : 0;
  if (need > room) return fail(PDOSGPU_ENOTSUP, "the batch kernel's shared memory does not fit at this CTA size");
  PDOS_CUDA_TRY(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)room));
  return PDOSGPU_OK;
}

// Grid (a multiple of `ctas`) of a cluster kernel: as many clusters as fit
// the device at once, at most one per instance and per staging region.
template <typename T>
int cluster_grid(KernelOf<T> kernel, int block, size_t bytes, int members, int regions, int ctas, int *grid) {
  PDOS_TRY(allow_dynamic_smem(kernel, bytes));
  cudaLaunchAttribute attr[1];
  cudaLaunchConfig_t cfg = cluster_config(ctas, block, bytes, nullptr, attr, ctas);
  int nc = 0;
  PDOS_CUDA_TRY(cudaOccupancyMaxActiveClusters(&nc, (const void *)kernel, &cfg));
  if (nc < 1) return fail(PDOSGPU_ENOTSUP, "a cluster of the batch kernel does not fit the device");
  *grid = std::max(1, std::min(std::min(members, nc), regions)) * ctas;
  return PDOSGPU_OK;
}
template <typename T>
int launch_clusters(KernelOf<T> kernel, int grid, int block, size_t bytes, cudaStream_t st, const Dev<T> &dev,
                    int cls, const Smem &sm, int arg, int ctas) {
  cudaLaunchAttribute attr[1];
  cudaLaunchConfig_t cfg = cluster_config(grid, block, bytes, st, attr, ctas);
  PDOS_CUDA_TRY(cudaLaunchKernelEx(&cfg, kernel, dev, cls, sm, arg));
  return PDOSGPU_OK;
}
template <typename T>
KernelOf<T> pair_kernel_for(int block, bool products) {
  switch (block) {
    case 128: return products ? batch_pair_products_kernel<T, 128> : batch_pair_kernel<T, 128>;
    case 256: return products ? batch_pair_products_kernel<T, 256> : batch_pair_kernel<T, 256>;
    case 512: return products ? batch_pair_products_kernel<T, 512> : batch_pair_kernel<T, 512>;
    case 1024: return products ? batch_pair_products_kernel<T, 1024> : batch_pair_kernel<T, 1024>;
    default: return nullptr;
  }
}
template <typename T>
KernelOf<T> admm_kernel_for(int block, const Smem &sm) {
  if (sm.pair) return pair_kernel_for<T>(block, false);
  switch (stage_mode(sm)) {
    case kStageShared: return admm_kernel_mode<T, kStageShared>(block);
    case kStageGlobalSG: return admm_kernel_mode<T, kStageGlobalSG>(block);
    default: return admm_kernel_mode<T, kStageGlobal>(block);
  }
}
template <typename T>
KernelOf<T> products_kernel_for(int block, const Smem &sm) {
  if (sm.pair) return pair_kernel_for<T>(block, true);
  switch (stage_mode(sm)) {
    case kStageShared: return products_kernel_mode<T, kStageShared>(block);
    case kStageGlobalSG: return products_kernel_mode<T, kStageGlobalSG>(block);
    default: return products_kernel_mode<T, kStageGlobal>(block);
  }
}

class BatchBase {
 public:
  virtual ~BatchBase() {}
  virtual int create(const pdosgpu_options &opt, int iter_cap) = 0;
  virtual int append(const pdosgpu_problem *probs, int64_t count) = 0;
  virtual int commit() = 0;
  virtual int solve(int64_t max_launches) = 0;
  virtual int reset() = 0;
  virtual int warm_start(const double *x0, const double *y0, const double *s0) = 0;
  virtual int fetch(int64_t first, int64_t count, double *x, double *s, double *y,
                    pdosgpu_info *info) = 0;
  virtual int tune(int iters, int *blocks_out) = 0;
  virtual int time_products(int reps, double *ms, double *bytes) = 0;
  virtual int instance_class(int64_t i) const = 0;
  virtual int set_blocks(const int *blocks) = 0;
  virtual void *stream() = 0;
  virtual int64_t done_count() = 0;
  bool committed = false;
  int64_t count = 0, total_n = 0, total_m = 0, total_nnz = 0, waves = 0;
  int64_t family_groups = 0, family_instances = 0;  // instances on shared layouts
  int64_t layout_bytes = 0;                          // device bytes of every layout
  double setup_ms = 0, solve_ms = 0;
  int64_t launches = 0;
  std::vector<int64_t> row0{0}, col0{0};
};

// Device vectors of one wave, kept until commit() stacks every wave's.
template <typename T>
struct WaveVectors {
  DeviceArena arena;
  int64_t n = 0, m = 0, col0 = 0, row0 = 0;
  T *b = nullptr, *c = nullptr, *D = nullptr, *E = nullptr;
  T *x_init = nullptr, *y_init = nullptr, *s_init = nullptr;
  double *D64 = nullptr, *E64 = nullptr, *Epre64 = nullptr;
};

// Nonzeros a wave may hold: its stacked set-up keeps 32-bit indices, and
// its transient device memory (the problem in double and 64-bit indices,
// the CSC -> CSR transpose, the scaled values, both layouts) is bounded by
// a share of the free device memory.
constexpr int64_t kWaveMaxNnz = ((int64_t)1 << 30);
constexpr int64_t kWaveMaxVec = (int64_t)INT32_MAX - 4096;
constexpr int64_t kSetupBytesPerNnz = 128;

template <typename T>
class BatchEngine : public BatchBase {
 public:
  ~BatchEngine() override {
    for (auto e : exec_)
      if (e) cudaGraphExecDestroy(e);
    for (auto e : ev_) if (e) cudaEventDestroy(e);
    for (auto s : side_) {
      if (s) cudaStreamDestroy(s);
    }
    if (stream_) {
      cudaStreamSynchronize(stream_);
      cudaStreamDestroy(stream_);
    }
    if (host_done_) cudaFreeHost(host_done_);
  }

  int create(const pdosgpu_options &opt, int iter_cap) override;
  int append(const pdosgpu_problem *probs, int64_t count_in) override;
  int commit() override;
  int solve(int64_t max_launches) override;
  int reset() override;
  int warm_start(const double *x0, const double *y0, const double *s0) override;
  int fetch(int64_t first, int64_t cnt, double *x, double *s, double *y, pdosgpu_info *info) override;
  int tune(int iters, int *blocks_out) override;
  int time_products(int reps, double *ms, double *bytes) override;
  int set_blocks(const int *blocks) override;
  int instance_class(int64_t i) const override { return inst_h_[i].cls; }
  void *stream() override { return stream_; }
  int64_t done_count() override;

 private:
  int append_wave(const pdosgpu_problem *probs, int64_t cnt);
  void layout_params(HybBuild &a, HybBuild &b) const {
    for (HybBuild *h : {&a, &b}) {
      if (opt_.batch_long_row > 0) h->long_row = opt_.batch_long_row;
      if (opt_.batch_piece > 0) h->piece = opt_.batch_piece;
    }
  }
  int build_graph(int iter_cap, cudaGraphExec_t *exec);
  int configure(int cls, int block);
  int launch_class(int cls, int block, int iter_cap, cudaStream_t st);
  int grid_[kClasses]{};
  int64_t active_launch_nodes_ = 0;

  pdosgpu_options opt_{};
  int normalize_ = -1;              // NORMALIZE shared by every instance (-1: none yet)
  DeviceArena arena_;               // stacked vectors, instance tables, scratch
  std::vector<std::unique_ptr<DeviceArena>> layout_arenas_;  // one per wave: its layouts
  std::vector<std::unique_ptr<WaveVectors<T>>> wave_vecs_;   // until commit()
  cudaStream_t stream_ = nullptr;
  std::vector<cudaStream_t> side_;
  std::vector<cudaEvent_t> ev_;
  std::vector<cudaGraphExec_t> exec_;  // [0]: one launch of iter_cap iterations
  int iter_cap_ = 64;
  int gregions_ = 0;  // staging regions allocated for the global class
  int cluster_ctas_ = kClusterCtasOne;  // CTAs per cluster of the global class
  Dev<T> dev_{};
  Inst *inst_d_ = nullptr;
  State *state_d_ = nullptr;
  int32_t *queue_ = nullptr, *ndone_ = nullptr;
  int32_t *host_done_ = nullptr;
  std::vector<Inst> inst_h_;
  std::vector<int64_t> nnz_h_;
  std::vector<int32_t> class_begin_h_;
  std::vector<int32_t> cone_off_h_, cone_len_h_;
  Smem smem_[kClasses]{};
  int block_[kClasses]{};
  T *x_init_ = nullptr, *y_init_ = nullptr, *s_init_ = nullptr;
  double *D64_ = nullptr, *E64_ = nullptr, *Epre64_ = nullptr, *out_ = nullptr;
};

template <typename T>
int BatchEngine<T>::create(const pdosgpu_options &opt, int iter_cap) {
  if (iter_cap <= 0) return fail(PDOSGPU_EINVAL, "iterations per launch must be positive");
  iter_cap_ = iter_cap;
  opt_ = opt;
  PDOS_CUDA_TRY(cudaSetDevice(opt.device));
  PDOS_CUDA_TRY(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking));
  return PDOSGPU_OK;
}

// Appends problems in as many waves as the limits on one wave require.
template <typename T>
int BatchEngine<T>::append(const pdosgpu_problem *probs, int64_t cnt) {
  const double t0 = now_ms();
  if (committed) return fail(PDOSGPU_EINVAL, "the batch is already committed");
  if (cnt <= 0 || count + cnt > (int64_t)INT32_MAX / 2) return fail(PDOSGPU_EINVAL, "batch count out of range");
  for (int64_t i = 0; i < cnt; ++i) {
    const pdosgpu_problem &p = probs[i];
    const int rc = validate_problem(p);
    if (rc != PDOSGPU_OK)
      return fail(rc, "instance " + std::to_string(count + i) + ": " + pdos_gpu_last_error());
    if (p.m > 65535 || p.n > 65535)
      return fail(PDOSGPU_ENOTSUP, "instance " + std::to_string(count + i) +
                                       " is too large for the batch's 16-bit instance-local indices "
                                       "(m and n must stay below 65,536); solve it with pdosgpu_setup");
    if (normalize_ < 0) normalize_ = p.normalize ? 1 : 0;
    if ((p.normalize != 0) != (normalize_ != 0))
      return fail(PDOSGPU_EINVAL, "all instances of a batch must share NORMALIZE");
  }
  if (normalize_ && opt_.scaling == PDOSGPU_SCALE_RUIZ)
    return fail(PDOSGPU_ENOTSUP, "Ruiz equilibration is not available for batches");
  if (opt_.batch_layouts != PDOSGPU_BATCH_SHARE && opt_.batch_layouts != PDOSGPU_BATCH_OWN)
    return fail(PDOSGPU_EINVAL, "batch_layouts must be PDOSGPU_BATCH_SHARE or PDOSGPU_BATCH_OWN");
  if (opt_.batch_long_row != 0 && (opt_.batch_long_row % 4 || opt_.batch_long_row < 4 || opt_.batch_long_row > 1024))
    return fail(PDOSGPU_EINVAL, "batch_long_row must be 0 or a multiple of 4 in [4, 1024]");
  if (opt_.batch_piece != 0 && (opt_.batch_piece % 4 || opt_.batch_piece < 64 || opt_.batch_piece > 16384))
    return fail(PDOSGPU_EINVAL, "batch_piece must be 0 or a multiple of 4 in [64, 16384]");
  if (opt_.batch_clusters != 0 && opt_.batch_clusters != 1) return fail(PDOSGPU_EINVAL, "batch_clusters must be 0 or 1");
  PDOS_CUDA_TRY(cudaSetDevice(opt_.device));
  size_t free_b = 0, total_b = 0;
  PDOS_CUDA_TRY(cudaMemGetInfo(&free_b, &total_b));
  const int64_t max_nnz =
      std::max<int64_t>(1, std::min<int64_t>(kWaveMaxNnz, (int64_t)(free_b / 2 / kSetupBytesPerNnz)));
  int64_t first = 0;
  while (first < cnt) {
    int64_t last = first, nz = 0, n = 0, m = 0;
    do {  // at least one instance per wave
      nz += probs[last].Ap[probs[last].n];
      n += probs[last].n;
      m += probs[last].m;
      ++last;
    } while (last < cnt && nz + probs[last].Ap[probs[last].n] <= max_nnz &&
             n + probs[last].n <= kWaveMaxVec && m + probs[last].m <= kWaveMaxVec);
    PDOS_TRY(append_wave(probs + first, last - first));
    first = last;
  }
  setup_ms += now_ms() - t0;
  return PDOSGPU_OK;
}

// One wave: stack its instances block-diagonally on the host, set them up on
// the device (transpose, equilibration, warm start, lambda; every row,
// column and cone is scaled exactly as when the instance is alone), build
// both sides' layouts, upload them into the wave's own allocation, and keep
// the wave's vectors until commit().
template <typename T>
int BatchEngine<T>::append_wave(const pdosgpu_problem *probs, int64_t cnt) {
  // ---- family groups share one layout (NORMALIZE = 0 only: scaling would
  // give every instance its own values).  With NORMALIZE = 0 nothing of the
  // device set-up but the layout depends on the matrix, so a group's members
  // after the first enter the stacked problem without their entries: their
  // varying values are taken from the host arrays below.
  std::vector<FamilyGroup> groups;
  std::vector<int32_t> group_of(cnt, -1);
  std::vector<uint8_t> no_entries(cnt, 0);
  if (!normalize_ && opt_.batch_layouts == PDOSGPU_BATCH_SHARE) groups = find_family_groups(probs, cnt);
  for (size_t g = 0; g < groups.size(); ++g) {
    for (int64_t i : groups[g].members) group_of[i] = (int32_t)g;
    for (size_t k = 1; k < groups[g].members.size(); ++k) no_entries[groups[g].members[k]] = 1;
  }
  auto stacked_nnz = [&](int64_t i) -> int64_t { return no_entries[i] ? 0 : probs[i].Ap[probs[i].n]; };

  int64_t N = 0, M = 0, NNZ = 0, wave_nnz = 0;
  bool any_x = false, any_y = false, any_s = false;
  std::vector<int64_t> wrow0, wcol0;  // offsets inside the wave
  for (int64_t i = 0; i < cnt; ++i) {
    const pdosgpu_problem &p = probs[i];
    wrow0.push_back(M);
    wcol0.push_back(N);
    N += p.n;
    M += p.m;
    NNZ += stacked_nnz(i);
    wave_nnz += p.Ap[p.n];
    any_x |= p.x0 != nullptr;
    any_y |= p.y0 != nullptr;
    any_s |= p.s0 != nullptr;
  }
  wrow0.push_back(M);
  wcol0.push_back(N);
  if (N > kWaveMaxVec || M > kWaveMaxVec || NNZ > kWaveMaxVec)
    return fail(PDOSGPU_EINVAL, "an instance is too large for one set-up wave (2^31 - 4096 nonzeros)");

  // ---- stacked problem of the wave (block diagonal), host
  Raw<double> Ax, b, c;
  Raw<int64_t> Ai, Ap;
  Ax.resize(NNZ);
  b.resize(M);
  c.resize(N);
  Ai.resize(NNZ);
  Ap.resize(N + 1);
  std::vector<double> x0, y0, s0;
  if (any_x) x0.assign(N, 0.0);
  if (any_y) y0.assign(M, 0.0);
  if (any_s) s0.assign(M, 0.0);
  ProblemDesc d;
  {
    std::vector<int64_t> e0(cnt + 1, 0);  // first nonzero of each instance
    for (int64_t i = 0; i < cnt; ++i) {
      const pdosgpu_problem &p = probs[i];
      e0[i + 1] = e0[i] + stacked_nnz(i);
      int64_t off = wrow0[i] + p.f + p.l;
      for (int64_t k = 0; k < p.qsize; ++k) {
        d.soc_off.push_back(off);
        d.soc_len.push_back(p.q[k]);
        off += p.q[k];
      }
    }
    parallel_for(cnt, [&](int64_t i) {
      const pdosgpu_problem &p = probs[i];
      const int64_t nz = stacked_nnz(i), e = e0[i];
      for (int64_t j = 0; j < p.n; ++j) Ap[wcol0[i] + j] = nz > 0 ? e + p.Ap[j] : e;
      if (nz > 0) std::memcpy(&Ax[e], p.Ax, sizeof(double) * nz);
      for (int64_t k = 0; k < nz; ++k) Ai[e + k] = wrow0[i] + p.Ai[k];
      std::memcpy(&b[wrow0[i]], p.b, sizeof(double) * p.m);
      std::memcpy(&c[wcol0[i]], p.c, sizeof(double) * p.n);
      if (p.x0) std::memcpy(&x0[wcol0[i]], p.x0, sizeof(double) * p.n);
      if (p.y0) std::memcpy(&y0[wrow0[i]], p.y0, sizeof(double) * p.m);
      if (p.s0) std::memcpy(&s0[wrow0[i]], p.s0, sizeof(double) * p.m);
    });
    Ap[N] = e0[cnt];
  }
  d.n = N;
  d.m = M;
  d.nnz = NNZ;
  d.Ax = Ax.data();
  d.Ai = Ai.data();
  d.Ap = Ap.data();
  d.b = b.data();
  d.c = c.data();
  d.x0 = any_x ? x0.data() : nullptr;
  d.y0 = any_y ? y0.data() : nullptr;
  d.s0 = any_s ? s0.data() : nullptr;
  d.inst_row0 = wrow0;
  d.inst_col0 = wcol0;
  d.normalize = normalize_;

  cudaStream_t st = stream_;
  DeviceArena setup_arena;  // the wave's set-up arrays, released at the end of the wave
  DeviceProblem<T> P;
  PDOS_TRY(setup_problem<T>(d, setup_arena, st, P));

  // ---- the wave's vectors, kept until commit()
  auto wv = std::make_unique<WaveVectors<T>>();
  wv->n = N;
  wv->m = M;
  wv->col0 = total_n;
  wv->row0 = total_m;
  auto keep = [&](auto **dst, const auto *from, int64_t len) -> int {
    using E = std::remove_const_t<std::remove_pointer_t<std::decay_t<decltype(from)>>>;
    E *p = nullptr;
    PDOS_TRY(wv->arena.alloc(&p, (size_t)len));
    if (len > 0) PDOS_CUDA_TRY(cudaMemcpyAsync(p, from, sizeof(E) * len, cudaMemcpyDeviceToDevice, st));
    *dst = p;
    return PDOSGPU_OK;
  };
  PDOS_TRY(keep(&wv->b, P.b, M));
  PDOS_TRY(keep(&wv->c, P.c, N));
  PDOS_TRY(keep(&wv->D, P.D, M));
  PDOS_TRY(keep(&wv->E, P.E, N));
  PDOS_TRY(keep(&wv->x_init, P.x_init, N));
  PDOS_TRY(keep(&wv->y_init, P.y_init, M));
  PDOS_TRY(keep(&wv->s_init, P.s_init, M));
  PDOS_TRY(keep(&wv->D64, P.D64, M));
  PDOS_TRY(keep(&wv->E64, P.E64, N));
  PDOS_TRY(keep(&wv->Epre64, P.Epre64, N));

  // ---- hybrid layouts of both sides, instance by instance
  Raw<int32_t> Rj;
  Rj.resize(NNZ > 0 ? NNZ : 1);
  if (NNZ > 0)
    PDOS_CUDA_TRY(cudaMemcpyAsync(Rj.data(), P.Rj, sizeof(int32_t) * NNZ, cudaMemcpyDeviceToHost, st));
  PDOS_CUDA_TRY(cudaStreamSynchronize(st));
  const int64_t first = count;
  for (int64_t i = 0; i < cnt; ++i) {
    const pdosgpu_problem &p = probs[i];
    Inst I{};
    I.row0 = total_m + wrow0[i];
    I.col0 = total_n + wcol0[i];
    I.m = (int32_t)p.m;
    I.n = (int32_t)p.n;
    I.f = (int32_t)p.f;
    I.l = (int32_t)p.l;
    I.cone0 = (int64_t)cone_off_h_.size();
    I.ncones = (int32_t)p.qsize;
    int64_t off = p.f + p.l;
    for (int64_t k = 0; k < p.qsize; ++k) {
      cone_off_h_.push_back((int32_t)off);
      cone_len_h_.push_back((int32_t)p.q[k]);
      off += p.q[k];
    }
    I.lambda = P.lambda[i];
    I.pscale = P.pscale[i];
    I.dscale = P.dscale[i];
    I.alpha = p.alpha;
    I.eps = p.eps_abs;
    I.tol_sq = p.cg_tol * p.cg_tol;
    I.max_iters = p.max_iters;
    I.cg_max = p.cg_max_its;
    const int64_t nz = p.Ap[p.n];
    nnz_h_.push_back(nz);
    int cls = 0;
    while (cls < 3 && nz > kClassNnz[cls]) ++cls;
    I.cls = cls;
    inst_h_.push_back(I);
    row0.push_back(I.row0 + p.m);
    col0.push_back(I.col0 + p.n);
  }
  auto arena = std::make_unique<DeviceArena>();
  const int32_t *rp = P.rp_host.data(), *ap = P.ap_host.data();
  const int32_t *rj = Rj.data();
  const int64_t *ai = Ai.data();
  {  // instances with their own layout
    std::vector<int64_t> own;
    for (int64_t i = 0; i < cnt; ++i)
      if (group_of[i] < 0) own.push_back(i);
    if (!own.empty()) {
      HybBuild bA, bT;
      layout_params(bA, bT);
      std::vector<Side> sides;
      const int64_t no = (int64_t)own.size();
      build_layout<int32_t>(bA, no, [&](int64_t k, const int32_t *&ptr, const int32_t *&g, int64_t &r0,
                                        int64_t &r1, int64_t &c0) {
        const int64_t i = own[k];
        ptr = rp;
        g = rj;
        r0 = wrow0[i];
        r1 = wrow0[i + 1];
        c0 = wcol0[i];
      }, sides);
      for (int64_t k = 0; k < no; ++k) inst_h_[first + own[k]].A = sides[k];
      build_layout<int64_t>(bT, no, [&](int64_t k, const int32_t *&ptr, const int64_t *&g, int64_t &r0,
                                        int64_t &r1, int64_t &c0) {
        const int64_t i = own[k];
        ptr = ap;
        g = ai;
        r0 = wcol0[i];
        r1 = wcol0[i + 1];
        c0 = wrow0[i];
      }, sides);
      for (int64_t k = 0; k < no; ++k) inst_h_[first + own[k]].At = sides[k];
      HybPtr hA{}, hT{};
      PDOS_TRY(upload_hyb<T>(bA, P.Rx, *arena, st, hA, &layout_bytes));
      PDOS_TRY(upload_hyb<T>(bT, P.Ax, *arena, st, hT, &layout_bytes));
      for (int64_t k = 0; k < no; ++k) {
        inst_h_[first + own[k]].hA = hA;
        inst_h_[first + own[k]].hT = hT;
      }
    }
  }
  for (const FamilyGroup &fg : groups) {  // one layout per group, built from its first member
    const int64_t ref = fg.members[0];
    const pdosgpu_problem &pr = probs[ref];
    const int64_t nz = pr.Ap[pr.n];
    // CSR position -> CSC position within the instance (the stable
    // transpose, cs.c:146-168)
    std::vector<int64_t> csr2csc(nz > 0 ? nz : 1), next(pr.m + 1, 0);
    for (int64_t k = 0; k < nz; ++k) ++next[pr.Ai[k] + 1];
    for (int64_t r = 0; r < pr.m; ++r) next[r + 1] += next[r];
    for (int64_t j = 0; j < pr.n; ++j)
      for (int64_t k = pr.Ap[j]; k < pr.Ap[j + 1]; ++k) csr2csc[next[pr.Ai[k]]++] = k;
    const int64_t rbase = rp[wrow0[ref]], cbase = Ap[wcol0[ref]];
    HybBuild bA, bT;
    layout_params(bA, bT);
    std::vector<Side> sA, sT;
    build_layout<int32_t>(bA, 1, [&](int64_t, const int32_t *&ptr, const int32_t *&g, int64_t &r0, int64_t &r1,
                                     int64_t &c0) {
      ptr = rp;
      g = rj;
      r0 = wrow0[ref];
      r1 = wrow0[ref + 1];
      c0 = wcol0[ref];
    }, sA);
    build_layout<int64_t>(bT, 1, [&](int64_t, const int32_t *&ptr, const int64_t *&g, int64_t &r0, int64_t &r1,
                                     int64_t &c0) {
      ptr = ap;
      g = ai;
      r0 = wcol0[ref];
      r1 = wcol0[ref + 1];
      c0 = wrow0[ref];
    }, sT);
    // varying entries become NaN boxes numbered in layout order; vpos keeps
    // each one's position within the instance (CSR for A, CSC for A')
    std::vector<int64_t> vposA, vposT;
    for (size_t e = 0; e < bA.src.size(); ++e) {
      const int32_t p = bA.src[e];
      if (p < 0) continue;
      const int64_t local = p - rbase;
      if (fg.vary[csr2csc[local]]) {
        bA.src[e] = -2 - (int32_t)vposA.size();
        vposA.push_back(local);
      }
    }
    for (size_t e = 0; e < bT.src.size(); ++e) {
      const int32_t p = bT.src[e];
      if (p < 0) continue;
      const int64_t local = p - cbase;
      if (fg.vary[local]) {
        bT.src[e] = -2 - (int32_t)vposT.size();
        vposT.push_back(local);
      }
    }
    HybPtr hA{}, hT{};
    PDOS_TRY(upload_hyb<T>(bA, P.Rx, *arena, st, hA, &layout_bytes));
    PDOS_TRY(upload_hyb<T>(bT, P.Ax, *arena, st, hT, &layout_bytes));
    // every member's values of the varying entries, in layout order, from
    // the host arrays: the same operations as the device set-up with
    // NORMALIZE = 0 (the x-space ratio, then the conversion to T), after the
    // finiteness check the device set-up makes of every entry
    const int64_t nm = (int64_t)fg.members.size(), na = (int64_t)vposA.size(), nt = (int64_t)vposT.size();
    T *pvA = nullptr, *pvT = nullptr;
    PDOS_TRY(arena->alloc(&pvA, (size_t)(nm * na)));
    PDOS_TRY(arena->alloc(&pvT, (size_t)(nm * nt)));
    layout_bytes += (nm * na + nm * nt) * (int64_t)sizeof(T);
    {
      Raw<T> hvA, hvT;
      hvA.resize((size_t)(nm * na));
      hvT.resize((size_t)(nm * nt));
      std::atomic<int> bad{0};
      parallel_for(nm, [&](int64_t k) {
        const double *ax = probs[fg.members[k]].Ax;
        for (int64_t t = 0; t < na; ++t) {
          const double v = ax[csr2csc[vposA[t]]];
          if (!std::isfinite(v)) bad = 1;
          hvA[k * na + t] = (T)(v * kXRatio);
        }
        for (int64_t t = 0; t < nt; ++t) {
          const double v = ax[vposT[t]];
          if (!std::isfinite(v)) bad = 1;
          hvT[k * nt + t] = (T)(v * kXRatio);
        }
      });
      if (bad) return fail(PDOSGPU_EINVAL, "A, b or c holds NaN or Inf");
      if (nm * na > 0)
        PDOS_CUDA_TRY(cudaMemcpyAsync(pvA, hvA.data(), sizeof(T) * nm * na, cudaMemcpyHostToDevice, st));
      if (nm * nt > 0)
        PDOS_CUDA_TRY(cudaMemcpyAsync(pvT, hvT.data(), sizeof(T) * nm * nt, cudaMemcpyHostToDevice, st));
      PDOS_CUDA_TRY(cudaStreamSynchronize(st));  // before the host arrays go
    }
    for (int64_t k = 0; k < nm; ++k) {
      Inst &I = inst_h_[first + fg.members[k]];
      I.A = sA[0];
      I.At = sT[0];
      I.hA = hA;
      I.hT = hT;
      I.pvA = pvA + k * na;
      I.pvT = pvT + k * nt;
    }
    ++family_groups;
    family_instances += nm;
  }
  // an instance whose own staging regions exceed one CTA's shared memory
  // goes to the global class
  auto r4 = [](int32_t v) { return (v + 3) & ~3; };
  for (int64_t i = 0; i < cnt; ++i) {
    Inst &I = inst_h_[first + i];
    const Smem own{r4(std::max(I.m, I.n)), r4(I.m), r4(I.n), r4(2 * std::max(I.A.npieces, I.At.npieces)), 0, 0, 0};
    if (own.need(sizeof(T)) > (size_t)kSmemLimit) I.cls = kGlobalClass;
    // on request every instance whose gather vector fits shared memory runs
    // on a cluster (the global class gathering from shared memory)
    if (opt_.batch_clusters && (size_t)r4(std::max(I.m, I.n)) * sizeof(T) <= (size_t)kSmemLimit) I.cls = kGlobalClass;
  }
  PDOS_CUDA_TRY(cudaStreamSynchronize(st));  // the wave's set-up arrays are released next
  layout_arenas_.push_back(std::move(arena));
  wave_vecs_.push_back(std::move(wv));
  count += cnt;
  total_n += N;
  total_m += M;
  total_nnz += wave_nnz;
  ++waves;
  return PDOSGPU_OK;
}

// Stacks the waves' vectors, sorts the instances into size classes, uploads
// the instance tables and captures the launch graph.
template <typename T>
int BatchEngine<T>::commit() {
  const double t0 = now_ms();
  if (committed) return fail(PDOSGPU_EINVAL, "the batch is already committed");
  if (count == 0) return fail(PDOSGPU_EINVAL, "batch count out of range");
  cudaStream_t st = stream_;
  const int64_t N = total_n, M = total_m;
  Dev<T> &B = dev_;
  {  // stacked vectors
    T *b, *c, *D, *E;
    PDOS_TRY(arena_.alloc(&b, (size_t)M));
    PDOS_TRY(arena_.alloc(&c, (size_t)N));
    PDOS_TRY(arena_.alloc(&D, (size_t)M));
    PDOS_TRY(arena_.alloc(&E, (size_t)N));
    PDOS_TRY(arena_.alloc(&x_init_, (size_t)N));
    PDOS_TRY(arena_.alloc(&y_init_, (size_t)M));
    PDOS_TRY(arena_.alloc(&s_init_, (size_t)M));
    PDOS_TRY(arena_.alloc(&D64_, (size_t)M));
    PDOS_TRY(arena_.alloc(&E64_, (size_t)N));
    PDOS_TRY(arena_.alloc(&Epre64_, (size_t)N));
    for (auto &w : wave_vecs_) {
      auto cp = [&](auto *dst, const auto *from, int64_t off, int64_t len) -> int {
        if (len > 0)
          PDOS_CUDA_TRY(cudaMemcpyAsync(dst + off, from, sizeof(*from) * len, cudaMemcpyDeviceToDevice, st));
        return PDOSGPU_OK;
      };
      PDOS_TRY(cp(b, w->b, w->row0, w->m));
      PDOS_TRY(cp(c, w->c, w->col0, w->n));
      PDOS_TRY(cp(D, w->D, w->row0, w->m));
      PDOS_TRY(cp(E, w->E, w->col0, w->n));
      PDOS_TRY(cp(x_init_, w->x_init, w->col0, w->n));
      PDOS_TRY(cp(y_init_, w->y_init, w->row0, w->m));
      PDOS_TRY(cp(s_init_, w->s_init, w->row0, w->m));
      PDOS_TRY(cp(D64_, w->D64, w->row0, w->m));
      PDOS_TRY(cp(E64_, w->E64, w->col0, w->n));
      PDOS_TRY(cp(Epre64_, w->Epre64, w->col0, w->n));
    }
    PDOS_CUDA_TRY(cudaStreamSynchronize(st));
    wave_vecs_.clear();
    B.b = b;
    B.c = c;
    B.D = D;
    B.E = E;
  }

  // ---- classes: staging regions and the processing order (largest
  // instances first within a class)
  const int64_t cnt = count;
  auto r4 = [](int32_t v) { return (v + 3) & ~3; };
  std::vector<std::vector<int32_t>> members(kClasses);
  for (int64_t i = 0; i < cnt; ++i) members[inst_h_[i].cls].push_back((int32_t)i);
  std::vector<int32_t> order;
  class_begin_h_.assign(kClasses + 1, 0);
  for (int k = 0; k < kClasses; ++k) {
    auto &mv = members[k];
    // largest first; a family group's instances (one layout) kept together
    std::stable_sort(mv.begin(), mv.end(), [&](int32_t a, int32_t bb) {
      if (nnz_h_[a] != nnz_h_[bb]) return nnz_h_[a] > nnz_h_[bb];
      return std::less<const void *>()(inst_h_[a].hA.val, inst_h_[bb].hA.val);
    });
    Smem sm{0, 0, 0, 0, k == kGlobalClass ? 1 : 0, 0, 0};
    const int32_t gs_cap = (int32_t)(kSmemLimit / sizeof(T)) & ~3;  // gather vector in shared memory
    for (int32_t i : mv) {
      const Inst &I = inst_h_[i];
      sm.g1 = std::max(sm.g1, std::max(I.m, I.n));
      sm.g2 = std::max(sm.g2, I.m);
      sm.tt = std::max(sm.tt, I.n);
      sm.pb = std::max(sm.pb, 2 * std::max(I.A.npieces, I.At.npieces));
      if (sm.global) sm.gs = std::max(sm.gs, r4(std::max(I.m, I.n)));
    }
    if (sm.gs > gs_cap) sm.gs = 0;  // some member's vectors do not fit: gathers from global memory
    sm = Smem{r4(sm.g1), r4(sm.g2), r4(sm.tt), r4(sm.pb), sm.global, sm.gs, 0};
    // pairs: consecutive members (the order keeps a group's instances together,
    // all of one size) that share a family layout, when two instances' regions
    // fit one CTA's shared memory
    std::vector<int32_t> items;
    if (!sm.global && 2 * sm.need(sizeof(T)) <= (size_t)kSmemLimit) {
      int npairs = 0;
      for (size_t a = 0; a < mv.size();) {
        const Inst &A = inst_h_[mv[a]];
        if (a + 1 < mv.size() && A.pvA != nullptr && inst_h_[mv[a + 1]].hA.val == A.hA.val) {
          items.push_back(mv[a]);
          items.push_back(mv[a + 1]);
          ++npairs;
          a += 2;
        } else {
          items.push_back(mv[a]);
          items.push_back(-1);
          a += 1;
        }
      }
      if (npairs > 0) sm.pair = 1;
    }
    smem_[k] = sm;
    block_[k] = k == 0 ? 128 : (k == 1 ? 256 : 512);
    if (sm.pair) order.insert(order.end(), items.begin(), items.end());
    else order.insert(order.end(), mv.begin(), mv.end());
    class_begin_h_[k + 1] = (int32_t)order.size();
  }

  // ---- device arrays
  int32_t *order_d, *class_begin_d, *cone_off_d, *cone_len_d;
  PDOS_TRY(arena_.alloc(&inst_d_, (size_t)cnt));
  PDOS_TRY(arena_.alloc(&state_d_, (size_t)cnt));
  PDOS_TRY(arena_.alloc(&order_d, order.size()));
  PDOS_TRY(arena_.alloc(&class_begin_d, (size_t)kClasses + 1));
  PDOS_TRY(arena_.alloc(&queue_, (size_t)kClasses + 1));
  ndone_ = queue_ + kClasses;
  PDOS_TRY(arena_.alloc(&cone_off_d, cone_off_h_.size() + 1));
  PDOS_TRY(arena_.alloc(&cone_len_d, cone_len_h_.size() + 1));
  PDOS_CUDA_TRY(cudaMemcpyAsync(inst_d_, inst_h_.data(), sizeof(Inst) * cnt, cudaMemcpyHostToDevice, st));
  PDOS_CUDA_TRY(cudaMemcpyAsync(order_d, order.data(), sizeof(int32_t) * order.size(), cudaMemcpyHostToDevice, st));
  PDOS_CUDA_TRY(cudaMemcpyAsync(class_begin_d, class_begin_h_.data(), sizeof(int32_t) * (kClasses + 1),
                                cudaMemcpyHostToDevice, st));
  if (!cone_off_h_.empty()) {
    PDOS_CUDA_TRY(cudaMemcpyAsync(cone_off_d, cone_off_h_.data(), sizeof(int32_t) * cone_off_h_.size(),
                                  cudaMemcpyHostToDevice, st));
    PDOS_CUDA_TRY(cudaMemcpyAsync(cone_len_d, cone_len_h_.data(), sizeof(int32_t) * cone_len_h_.size(),
                                  cudaMemcpyHostToDevice, st));
  }
  B.inst = inst_d_;
  B.state = state_d_;
  B.order = order_d;
  B.class_begin = class_begin_d;
  B.queue = queue_;
  B.ndone = ndone_;
  PDOS_TRY(arena_.alloc(&B.x, (size_t)N));
  PDOS_TRY(arena_.alloc(&B.q, (size_t)N));
  PDOS_TRY(arena_.alloc(&B.s, (size_t)M));
  PDOS_TRY(arena_.alloc(&B.y, (size_t)M));
  PDOS_TRY(arena_.alloc(&B.st, (size_t)M));
  PDOS_TRY(arena_.alloc(&B.u, (size_t)M));
  PDOS_TRY(arena_.alloc(&B.ax, (size_t)M));
  B.cone_off = cone_off_d;
  B.cone_len = cone_len_d;
  B.gscratch = nullptr;
  {  // one staging region per resident CTA (at most 8 per SM) or cluster of the global class
    const int members_g = class_begin_h_[kGlobalClass + 1] - class_begin_h_[kGlobalClass];
    cluster_ctas_ = cluster_ctas_for(members_g, num_sms(), opt_.batch_clusters != 0);
    gregions_ = on_clusters(smem_[kGlobalClass]) ? std::min(members_g, std::max(1, num_sms() / cluster_ctas_))
                                                 : std::min(members_g, num_sms() * (1024 / kBlocks[0]));
    if (gregions_ > 0) PDOS_TRY(arena_.alloc(&B.gscratch, (size_t)gregions_ * smem_[kGlobalClass].stride()));
  }
  PDOS_TRY(arena_.alloc(&out_, (size_t)N + 2 * (size_t)M));
  PDOS_CUDA_TRY(cudaMallocHost(&host_done_, sizeof(int32_t)));

  for (int k = 0; k < kClasses; ++k) {
    cudaStream_t s = nullptr;
    cudaEvent_t e = nullptr;
    PDOS_CUDA_TRY(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    side_.push_back(s);
    PDOS_CUDA_TRY(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    ev_.push_back(e);
  }
  {
    cudaEvent_t e = nullptr;
    PDOS_CUDA_TRY(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    ev_.push_back(e);  // fork event
  }
  PDOS_CUDA_TRY(cudaStreamSynchronize(st));
  committed = true;
  PDOS_TRY(reset());
  exec_.assign(1, nullptr);
  PDOS_TRY(build_graph(iter_cap_, &exec_[0]));
  PDOS_CUDA_TRY(cudaStreamSynchronize(st));
  setup_ms += now_ms() - t0;
  return PDOSGPU_OK;
}

// Kernel attributes and grid of one class at one CTA size (outside any
// stream capture).
template <typename T>
int BatchEngine<T>::configure(int cls, int block) {
  const size_t bytes = smem_[cls].bytes(sizeof(T));
  auto go = [&](auto kernel) -> int {
    // one limit for every class that shares this kernel
    PDOS_TRY(allow_dynamic_smem(kernel, bytes));
    int per_sm = 0;
    PDOS_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, block, bytes));
    if (per_sm < 1) return fail(PDOSGPU_ENOTSUP, "batch kernel does not fit on an SM");
    const int members = class_begin_h_[cls + 1] - class_begin_h_[cls];
    const int work = smem_[cls].pair ? members / 2 : members;  // work items: pairs or instances
    grid_[cls] = std::max(1, std::min(work, per_sm * num_sms()));
    if (smem_[cls].global) grid_[cls] = std::min(grid_[cls], gregions_);
    return PDOSGPU_OK;
  };
  const int members = class_begin_h_[cls + 1] - class_begin_h_[cls];
  if (on_clusters(smem_[cls])) {
    auto kernel = cluster_kernel_for<T>(block, false);
    if (!kernel) return fail(PDOSGPU_EINVAL, "unsupported CTA size");
    return cluster_grid<T>(kernel, block, bytes, members, gregions_, cluster_ctas_, &grid_[cls]);
  }
  auto kernel = admm_kernel_for<T>(block, smem_[cls]);
  if (!kernel) return fail(PDOSGPU_EINVAL, "unsupported CTA size");
  return go(kernel);
}

template <typename T>
int BatchEngine<T>::launch_class(int cls, int block, int iter_cap, cudaStream_t st) {
  const Smem sm = smem_[cls];
  const size_t bytes = sm.bytes(sizeof(T));
  if (on_clusters(sm)) {
    auto kernel = cluster_kernel_for<T>(block, false);
    if (!kernel) return fail(PDOSGPU_EINVAL, "unsupported CTA size");
    return launch_clusters<T>(kernel, grid_[cls], block, bytes, st, dev_, cls, sm, iter_cap, cluster_ctas_);
  }
  auto kernel = admm_kernel_for<T>(block, sm);
  if (!kernel) return fail(PDOSGPU_EINVAL, "unsupported CTA size");
  kernel<<<grid_[cls], block, bytes, st>>>(dev_, cls, sm, iter_cap);
  PDOS_CUDA_TRY(cudaGetLastError());
  return PDOSGPU_OK;
}

template <typename T>
int BatchEngine<T>::build_graph(int iter_cap, cudaGraphExec_t *exec) {
  cudaStream_t st = stream_;
  for (int k = 0; k < kClasses; ++k)
    if (class_begin_h_[k + 1] > class_begin_h_[k]) PDOS_TRY(configure(k, block_[k]));
  cudaGraph_t graph = nullptr;
  PDOS_CUDA_TRY(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
  int rc = PDOSGPU_OK;
  int64_t nodes = 1;
  do {
    if (cudaMemsetAsync(queue_, 0, sizeof(int32_t) * kClasses, st) != cudaSuccess) {
      rc = fail(PDOSGPU_ECUDA, "queue reset");
      break;
    }
    if (cudaEventRecord(ev_[kClasses], st) != cudaSuccess) {
      rc = fail(PDOSGPU_ECUDA, "graph fork");
      break;
    }
    for (int k = 0; k < kClasses && rc == PDOSGPU_OK; ++k) {
      if (class_begin_h_[k + 1] == class_begin_h_[k]) continue;
      if (cudaStreamWaitEvent(side_[k], ev_[kClasses], 0) != cudaSuccess) {
        rc = fail(PDOSGPU_ECUDA, "graph fork");
        break;
      }
      rc = launch_class(k, block_[k], iter_cap, side_[k]);
      if (rc != PDOSGPU_OK) break;
      ++nodes;
      if (cudaEventRecord(ev_[k], side_[k]) != cudaSuccess || cudaStreamWaitEvent(st, ev_[k], 0) != cudaSuccess)
        rc = fail(PDOSGPU_ECUDA, "graph join");
    }
  } while (0);
  cudaError_t e = cudaStreamEndCapture(st, &graph);
  if (rc != PDOSGPU_OK) {
    if (graph) cudaGraphDestroy(graph);
    return rc;
  }
  if (e != cudaSuccess) return fail(PDOSGPU_ECUDA, std::string("graph capture: ") + cudaGetErrorString(e));
  e = cudaGraphInstantiate(exec, graph, 0);
  cudaGraphDestroy(graph);
  if (e != cudaSuccess) return fail(PDOSGPU_ECUDA, std::string("graph instantiate: ") + cudaGetErrorString(e));
  active_launch_nodes_ = nodes - 1;
  return PDOSGPU_OK;
}

template <typename T>
int BatchEngine<T>::reset() {
  cudaStream_t st = stream_;
  const Dev<T> &B = dev_;
  PDOS_CUDA_TRY(cudaMemcpyAsync(B.x, x_init_, sizeof(T) * total_n, cudaMemcpyDeviceToDevice, st));
  PDOS_CUDA_TRY(cudaMemcpyAsync(B.y, y_init_, sizeof(T) * total_m, cudaMemcpyDeviceToDevice, st));
  PDOS_CUDA_TRY(cudaMemcpyAsync(B.s, s_init_, sizeof(T) * total_m, cudaMemcpyDeviceToDevice, st));
  PDOS_CUDA_TRY(cudaMemsetAsync(B.q, 0, sizeof(T) * total_n, st));
  PDOS_CUDA_TRY(cudaMemsetAsync(B.st, 0, sizeof(T) * total_m, st));
  PDOS_CUDA_TRY(cudaMemsetAsync(B.u, 0, sizeof(T) * total_m, st));
  PDOS_CUDA_TRY(cudaMemsetAsync(B.ax, 0, sizeof(T) * total_m, st));
  std::vector<State> h(count);
  int32_t done = 0;
  for (int64_t i = 0; i < count; ++i) {
    State &s = h[i];
    std::memset(&s, 0, sizeof(s));
    s.p_res = s.d_res = s.p_obj = s.d_obj = s.eta = -1.0;
    s.done = inst_h_[i].max_iters <= 0 ? 1 : 0;
    done += s.done;
  }
  PDOS_CUDA_TRY(cudaMemcpyAsync(state_d_, h.data(), sizeof(State) * count, cudaMemcpyHostToDevice, st));
  PDOS_CUDA_TRY(cudaMemcpyAsync(ndone_, &done, sizeof(int32_t), cudaMemcpyHostToDevice, st));
  PDOS_CUDA_TRY(cudaStreamSynchronize(st));  // h and done are host stack memory
  return PDOSGPU_OK;
}

template <typename T>
int BatchEngine<T>::warm_start(const double *x0, const double *y0, const double *s0) {
  cudaStream_t st = stream_;
  const int64_t len = total_n + total_m;
  const int g = (int)std::max<int64_t>(1, std::min<int64_t>((len + 255) / 256, (int64_t)num_sms() * 16));
  warm_start_kernel<T><<<g, 256, 0, st>>>(x0, y0, s0, D64_, Epre64_, total_n, total_m, x_init_, y_init_,
                                          s_init_);
  PDOS_CUDA_TRY(cudaGetLastError());
  return reset();
}

template <typename T>
int64_t BatchEngine<T>::done_count() {
  if (cudaMemcpyAsync(host_done_, ndone_, sizeof(int32_t), cudaMemcpyDeviceToHost, stream_) != cudaSuccess)
    return -1;
  if (cudaStreamSynchronize(stream_) != cudaSuccess) return -1;
  return *host_done_;
}

template <typename T>
int BatchEngine<T>::solve(int64_t max_launches) {
  const double t0 = now_ms();
  int64_t launched = 0;
  int64_t between = 1;  // launches queued between two reads of the done count
  int64_t done = done_count();
  if (done < 0) return fail(PDOSGPU_ECUDA, "reading the batch state failed");
  while (done < count && (max_launches < 0 || launched < max_launches)) {
    int64_t nb = between;
    if (max_launches >= 0) nb = std::min<int64_t>(nb, max_launches - launched);
    for (int64_t k = 0; k < nb; ++k) {
      PDOS_CUDA_TRY(cudaGraphLaunch(exec_[0], stream_));
      launches += active_launch_nodes_;
    }
    launched += nb;
    done = done_count();
    if (done < 0) return fail(PDOSGPU_ECUDA, "reading the batch state failed");
    if (between < 4) between *= 2;
  }
  PDOS_CUDA_TRY(cudaStreamSynchronize(stream_));
  solve_ms = now_ms() - t0;
  return PDOSGPU_OK;
}

template <typename T>
int BatchEngine<T>::fetch(int64_t first, int64_t cnt, double *x, double *s, double *y,
                          pdosgpu_info *info) {
  if (first < 0 || cnt < 0 || first + cnt > count) return fail(PDOSGPU_EINVAL, "instance range out of bounds");
  if (cnt == 0) return PDOSGPU_OK;
  cudaStream_t st = stream_;
  const Dev<T> &B = dev_;
  const int64_t n = total_n, m = total_m;
  const int g = (int)std::max<int64_t>(1, std::min<int64_t>((n + m + 255) / 256, (int64_t)num_sms() * 16));
  unscale_kernel<T><<<g, 256, 0, st>>>(B.x, B.s, B.y, D64_, E64_, n, m, out_);
  PDOS_CUDA_TRY(cudaGetLastError());
  const int64_t c0 = col0[first], c1 = col0[first + cnt], r0 = row0[first], r1 = row0[first + cnt];
  if (x) PDOS_CUDA_TRY(cudaMemcpyAsync(x, out_ + c0, sizeof(double) * (c1 - c0), cudaMemcpyDeviceToHost, st));
  if (s) PDOS_CUDA_TRY(cudaMemcpyAsync(s, out_ + n + r0, sizeof(double) * (r1 - r0), cudaMemcpyDeviceToHost, st));
  if (y) PDOS_CUDA_TRY(cudaMemcpyAsync(y, out_ + n + m + r0, sizeof(double) * (r1 - r0), cudaMemcpyDeviceToHost, st));
  std::vector<State> h(cnt);
  PDOS_CUDA_TRY(cudaMemcpyAsync(h.data(), state_d_ + first, sizeof(State) * cnt, cudaMemcpyDeviceToHost, st));
  PDOS_CUDA_TRY(cudaStreamSynchronize(st));
  if (info) {
    for (int64_t i = 0; i < cnt; ++i) {
      pdosgpu_info &o = info[i];
      std::memset(&o, 0, sizeof(o));
      o.admm_iters = h[i].admm_iter;
      o.cg_iters = h[i].cg_total;
      o.solved = h[i].solved;
      o.diverged = h[i].diverged;
      o.p_res = h[i].p_res;
      o.d_res = h[i].d_res;
      o.p_obj = h[i].p_obj;
      o.d_obj = h[i].d_obj;
      o.eta = h[i].eta;
      o.lambda = inst_h_[first + i].lambda;
      o.setup_ms = setup_ms;
      o.solve_ms = solve_ms;
      o.kernel_launches = launches;
    }
  }
  return PDOSGPU_OK;
}

template <typename T>
int BatchEngine<T>::set_blocks(const int *blocks) {
  for (int k = 0; k < kClasses; ++k) {
    bool ok = false;
    for (int j = 0; j < kNumBlocks; ++j) ok |= blocks[k] == kBlocks[j];
    if (!ok) return fail(PDOSGPU_EINVAL, "CTA sizes must be 128, 256, 512 or 1024");
  }
  for (int k = 0; k < kClasses; ++k) block_[k] = blocks[k];
  if (exec_[0]) cudaGraphExecDestroy(exec_[0]);
  exec_[0] = nullptr;
  return build_graph(iter_cap_, &exec_[0]);
}

// Autotuner: for each size class with members, time `iters` iterations of
// every instance of the class at each CTA size and keep the fastest; the
// batch is reset afterwards.
template <typename T>
int BatchEngine<T>::tune(int iters, int *blocks_out) {
  if (iters <= 0) return fail(PDOSGPU_EINVAL, "iters must be positive");
  cudaStream_t st = stream_;
  cudaEvent_t e0, e1;
  PDOS_CUDA_TRY(cudaEventCreate(&e0));
  PDOS_CUDA_TRY(cudaEventCreate(&e1));
  int rc = PDOSGPU_OK;
  for (int k = 0; k < kClasses && rc == PDOSGPU_OK; ++k) {
    if (class_begin_h_[k + 1] == class_begin_h_[k]) continue;
    float best = -1.f;
    for (int j = 0; j < kNumBlocks && rc == PDOSGPU_OK; ++j) {
      const int blk = kBlocks[j];
      if (smem_[k].bytes(sizeof(T)) > (size_t)kSmemLimit) continue;
      rc = reset();
      if (rc == PDOSGPU_OK) rc = configure(k, blk);
      if (rc == PDOSGPU_ENOTSUP) {  // this CTA size does not fit the class's shared memory
        rc = PDOSGPU_OK;
        continue;
      }
      if (rc != PDOSGPU_OK) break;
      // prepare (first pass) outside the timed region
      if (cudaMemsetAsync(queue_, 0, sizeof(int32_t) * kClasses, st) != cudaSuccess) {
        rc = fail(PDOSGPU_ECUDA, "queue reset");
        break;
      }
      rc = launch_class(k, blk, 1, st);
      if (rc != PDOSGPU_OK) break;
      cudaMemsetAsync(queue_, 0, sizeof(int32_t) * kClasses, st);
      cudaEventRecord(e0, st);
      rc = launch_class(k, blk, iters, st);
      cudaEventRecord(e1, st);
      if (rc != PDOSGPU_OK) break;
      if (cudaEventSynchronize(e1) != cudaSuccess) {
        rc = fail(PDOSGPU_ECUDA, "tuning launch failed");
        break;
      }
      float ms = 0.f;
      cudaEventElapsedTime(&ms, e0, e1);
      launches += 2;
      if (best < 0.f || ms < best) {
        best = ms;
        block_[k] = blk;
      }
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  PDOS_TRY(rc);
  if (blocks_out)
    for (int k = 0; k < kClasses; ++k) blocks_out[k] = block_[k];
  PDOS_TRY(reset());
  if (exec_[0]) cudaGraphExecDestroy(exec_[0]);
  exec_[0] = nullptr;
  return build_graph(iter_cap_, &exec_[0]);
}

// The CG products of every instance `reps` times (batch_products_kernel),
// class after class on the batch stream; bytes = the algorithmic bytes of
// those products (values and indices of A and A', both pointer arrays, the
// vector gathered from and the vector written, per product).
template <typename T>
int BatchEngine<T>::time_products(int reps, double *ms, double *bytes) {
  if (reps <= 0 || !ms) return fail(PDOSGPU_EINVAL, "reps must be positive");
  cudaStream_t st = stream_;
  double b = 0.0;
  for (int64_t i = 0; i < count; ++i) {
    const double sv = sizeof(T), m = inst_h_[i].m, n = inst_h_[i].n, nz = (double)nnz_h_[i];
    b += nz * (sv + 2) + (m + 1) * 4 + n * sv + m * sv;  // u = A p (16-bit indices)
    b += nz * (sv + 2) + (n + 1) * 4 + m * sv + n * sv;  // t = p + A'u
  }
  auto go = [&](int cls, int block, auto kernel) -> int {
    const size_t sm_bytes = smem_[cls].bytes(sizeof(T));
    if (on_clusters(smem_[cls])) {
      auto ck = cluster_kernel_for<T>(block, true);
      if (!ck) return fail(PDOSGPU_EINVAL, "unsupported CTA size");
      int grid = 0;
      PDOS_TRY(cluster_grid<T>(ck, block, sm_bytes, class_begin_h_[cls + 1] - class_begin_h_[cls], gregions_,
                               cluster_ctas_, &grid));
      return launch_clusters<T>(ck, grid, block, sm_bytes, st, dev_, cls, smem_[cls], reps, cluster_ctas_);
    }
    PDOS_TRY(allow_dynamic_smem(kernel, sm_bytes));
    int per_sm = 0;
    PDOS_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, block, sm_bytes));
    if (per_sm < 1) return fail(PDOSGPU_ENOTSUP, "product kernel does not fit on an SM");
    const int members = class_begin_h_[cls + 1] - class_begin_h_[cls];
    const int work = smem_[cls].pair ? members / 2 : members;
    int grid = std::max(1, std::min(work, per_sm * num_sms()));
    if (smem_[cls].global) grid = std::min(grid, gregions_);
    kernel<<<grid, block, sm_bytes, st>>>(dev_, cls, smem_[cls], reps);
    PDOS_CUDA_TRY(cudaGetLastError());
    return PDOSGPU_OK;
  };
  auto all = [&]() -> int {
    PDOS_CUDA_TRY(cudaMemsetAsync(queue_, 0, sizeof(int32_t) * kClasses, st));
    for (int k = 0; k < kClasses; ++k) {
      if (class_begin_h_[k + 1] == class_begin_h_[k]) continue;
      auto kernel = products_kernel_for<T>(block_[k], smem_[k]);
      if (!kernel) return fail(PDOSGPU_EINVAL, "unsupported CTA size");
      PDOS_TRY(go(k, block_[k], kernel));
    }
    launches += kClasses;
    return PDOSGPU_OK;
  };
  cudaEvent_t e0, e1;
  PDOS_CUDA_TRY(cudaEventCreate(&e0));
  PDOS_CUDA_TRY(cudaEventCreate(&e1));
  int rc = all();  // warm-up
  if (rc == PDOSGPU_OK && cudaEventRecord(e0, st) != cudaSuccess) rc = fail(PDOSGPU_ECUDA, "event");
  if (rc == PDOSGPU_OK) rc = all();
  if (rc == PDOSGPU_OK && cudaEventRecord(e1, st) != cudaSuccess) rc = fail(PDOSGPU_ECUDA, "event");
  float t = 0.f;
  if (rc == PDOSGPU_OK && cudaEventSynchronize(e1) != cudaSuccess) rc = fail(PDOSGPU_ECUDA, "product kernels failed");
  if (rc == PDOSGPU_OK) cudaEventElapsedTime(&t, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  PDOS_TRY(rc);
  *ms = t;
  if (bytes) *bytes = b * reps;
  return PDOSGPU_OK;
}


// The engine of each precision, defined in its own translation unit.
std::unique_ptr<BatchBase> make_batch_engine_f32();
std::unique_ptr<BatchBase> make_batch_engine_f64();

}  // namespace batch
}  // namespace pdosgpu
