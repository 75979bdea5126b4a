// Sliced-ELL SpMV (SELL-32-sigma with row splitting) and the fused row
// epilogue.
//
// One kernel pair serves both products of the reference's formulation:
//   A  x : rows of A   from the CSR of A   (accumByScaledA, linAlg.h:70-91)
//   A' y : rows of A'  from the CSC of A   (accumByScaledATrans, linAlg.h:94-115)
//
// Layout.  Every row is cut into "virtual rows" of at most kVrowMax
// nonzeros (an empty row keeps one empty virtual row).  Virtual rows are
// sorted by length, longest first, inside windows of kSigma, and grouped in
// slices of 32.  A slice is stored column-major and padded to its longest
// virtual row: entry k of lane t sits at slice_off + 32*k + t.  So the 32
// lanes of a warp read 32 consecutive values and 32 consecutive indices per
// step (coalesced), gather the vector entries, and each lane keeps one FMA
// chain: exactly one fused multiply-add per nonzero, no cross-lane reduction
// and no shared memory.  Lanes past their virtual row's length are predicated
// off, so padding costs neither gathers nor FP64 work.
//
// A row held by a single virtual row is finished in the SpMV kernel itself:
// its sum goes straight to the epilogue functor `Op` (fused element-wise work
// of the ADMM / CG step plus NR grid-wide sums).  A split row leaves one
// partial per virtual row; the combine kernel adds a split row's partials in
// order and runs its epilogue.  The virtual-row length is chosen per matrix:
// whole rows when most nonzeros sit in short rows, short pieces when most
// sit in long rows (so long rows spread over many lanes).  Everything is
// deterministic for a fixed plan.
#pragma once

#include "common.cuh"
#include "sell_plan.h"

namespace pdosgpu {

#ifndef PDOS_SELL_UNROLL
#define PDOS_SELL_UNROLL 8
#endif
constexpr int kUnroll = PDOS_SELL_UNROLL; // loads in flight per lane

// Device side of a plan (arrays uploaded from SellHost).
template <typename T>
struct SellDev {
  const int32_t *slice_off;  // [nslices+1]
  const int32_t *vr_len;     // [nvr]
  const int32_t *idx;        // [slots]
  const T *val;              // [slots]
  int32_t nslices;
  int32_t nvr;
  const int32_t *vr_ptr;     // [rows+1]
  const int32_t *vr_list;    // [nvr used]
  const int32_t *heavy;      // [nheavy]
  int32_t nheavy;
  int32_t rows;
  const int32_t *vr_row;     // [nvr] row finished by this virtual row, or -1
  const int32_t *split;      // [nsplit] split rows combined per thread
  int32_t nsplit;
  int32_t ngiant;            // heavy[0, ngiant): combined by a CTA each
};

// slot k of the plan takes the source entry slot_src[k] (or zero padding)
template <typename T>
__global__ void sell_fill_kernel(const int32_t *slot_src, int64_t slots, const int32_t *idx_src,
                                 const T *val_src, int32_t *idx, T *val) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < slots;
       k += (int64_t)gridDim.x * blockDim.x) {
    const int32_t s = slot_src[k];
    idx[k] = s >= 0 ? idx_src[s] : 0;
    val[k] = s >= 0 ? val_src[s] : T(0);
  }
}

// Each lane reduces one virtual row.  Whole rows go to the epilogue at once;
// pieces of split rows are left in vsum[v * nvr + k] for the combine kernel.
template <typename T, int BLOCK, class Op>
__global__ void __launch_bounds__(BLOCK)
    sell_spmv_kernel(SellDev<T> S, const T *__restrict__ x0, const T *__restrict__ x1, T *vsum,
                     Op op, GridReduce gr) {
  constexpr int NV = Op::NV;
  constexpr int NR = Op::NR > 0 ? Op::NR : 1;
  __shared__ double scratch[BLOCK / 32];
  typename Op::Ctx ctx;
  if (!op.begin(ctx)) return;
  double red[NR];
#pragma unroll
  for (int k = 0; k < NR; ++k) red[k] = 0.0;
  const int lane = threadIdx.x & 31;
  const int warps = gridDim.x * (BLOCK / 32);
  for (int s = blockIdx.x * (BLOCK / 32) + (threadIdx.x >> 5); s < S.nslices; s += warps) {
    const int off = __ldg(S.slice_off + s) + lane;
    const int vr = 32 * s + lane;
    const int len = __ldg(S.vr_len + vr);
    T acc0 = T(0), acc1 = T(0);
    int k = 0;
    for (; k + kUnroll <= len; k += kUnroll) {
      int c[kUnroll];
      T a[kUnroll];
#pragma unroll
      for (int u = 0; u < kUnroll; ++u) {
        c[u] = __ldg(S.idx + off + 32 * (k + u));
        a[u] = __ldg(S.val + off + 32 * (k + u));
      }
#pragma unroll
      for (int u = 0; u < kUnroll; ++u) {
        acc0 = fma(a[u], __ldg(x0 + c[u]), acc0);
        if (NV == 2) acc1 = fma(a[u], __ldg(x1 + c[u]), acc1);
      }
    }
    for (; k < len; ++k) {
      const int c = __ldg(S.idx + off + 32 * k);
      const T a = __ldg(S.val + off + 32 * k);
      acc0 = fma(a, __ldg(x0 + c), acc0);
      if (NV == 2) acc1 = fma(a, __ldg(x1 + c), acc1);
    }
    const int r = __ldg(S.vr_row + vr);
    if (r >= 0) {
      T sum[NV];
      sum[0] = acc0;
      if (NV == 2) sum[NV - 1] = acc1;
      op.row(ctx, r, sum, red);
    } else {
      vsum[vr] = acc0;
      if (NV == 2) vsum[S.nvr + vr] = acc1;
    }
  }
  if constexpr (Op::NR > 0) {
    double tot[NR];
    if (grid_reduce<BLOCK, NR>(gr, red, tot, scratch) && threadIdx.x == 0) op.finalize(ctx, tot);
  }
}

// Split rows: sum of the row's pieces (in chunk order), then the epilogue.
// Rows with many pieces are summed by a warp each, rows with very many by a
// CTA each (fixed trees), in the extra blocks after the per-thread ones.
template <typename T, int BLOCK, class Op>
__global__ void __launch_bounds__(BLOCK)
    sell_combine_kernel(SellDev<T> S, const T *__restrict__ vsum, Op op, GridReduce gr,
                        int row_blocks) {
  constexpr int NV = Op::NV;
  constexpr int NR = Op::NR > 0 ? Op::NR : 1;
  __shared__ double scratch[BLOCK / 32];
  typename Op::Ctx ctx;
  if (!op.begin(ctx)) return;
  double red[NR];
#pragma unroll
  for (int k = 0; k < NR; ++k) red[k] = 0.0;
  if ((int)blockIdx.x < row_blocks) {
    for (int h = blockIdx.x * BLOCK + threadIdx.x; h < S.nsplit; h += row_blocks * BLOCK) {
      const int r = __ldg(S.split + h);
      const int a = __ldg(S.vr_ptr + r), b = __ldg(S.vr_ptr + r + 1);
      T sum[NV];
#pragma unroll
      for (int v = 0; v < NV; ++v) sum[v] = T(0);
      for (int q = a; q < b; ++q) {
        const int p = __ldg(S.vr_list + q);
#pragma unroll
        for (int v = 0; v < NV; ++v) sum[v] += vsum[(size_t)v * S.nvr + p];
      }
      op.row(ctx, r, sum, red);
    }
  } else if ((int)blockIdx.x < row_blocks + S.ngiant) {
    // a row with very many pieces per extra block: every thread sums a
    // strided share of the pieces, then a fixed tree over the block
    __shared__ T part[NV][BLOCK / 32];
    const int h = blockIdx.x - row_blocks;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int r = __ldg(S.heavy + h);
    const int a = __ldg(S.vr_ptr + r), b = __ldg(S.vr_ptr + r + 1);
    T sum[NV];
#pragma unroll
    for (int v = 0; v < NV; ++v) sum[v] = T(0);
    for (int q = a + threadIdx.x; q < b; q += BLOCK) {
      const int p = __ldg(S.vr_list + q);
#pragma unroll
      for (int v = 0; v < NV; ++v) sum[v] += vsum[(size_t)v * S.nvr + p];
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
#pragma unroll
      for (int v = 0; v < NV; ++v) sum[v] += __shfl_xor_sync(0xffffffffu, sum[v], o);
    if (lane == 0)
#pragma unroll
      for (int v = 0; v < NV; ++v) part[v][warp] = sum[v];
    __syncthreads();
    if (warp == 0) {
#pragma unroll
      for (int v = 0; v < NV; ++v) sum[v] = lane < BLOCK / 32 ? part[v][lane] : T(0);
#pragma unroll
      for (int o = 16; o > 0; o >>= 1)
#pragma unroll
        for (int v = 0; v < NV; ++v) sum[v] += __shfl_xor_sync(0xffffffffu, sum[v], o);
      if (lane == 0) op.row(ctx, r, sum, red);
    }
  } else {
    // rows with many pieces: one per warp (strided partial sums, shuffle tree)
    const int lane = threadIdx.x & 31;
    const int h = S.ngiant + (blockIdx.x - row_blocks - S.ngiant) * (BLOCK / 32) + (threadIdx.x >> 5);
    if (h < S.nheavy) {
      const int r = __ldg(S.heavy + h);
      const int a = __ldg(S.vr_ptr + r), b = __ldg(S.vr_ptr + r + 1);
      T sum[NV];
#pragma unroll
      for (int v = 0; v < NV; ++v) sum[v] = T(0);
      for (int q = a + lane; q < b; q += 32) {
        const int p = __ldg(S.vr_list + q);
#pragma unroll
        for (int v = 0; v < NV; ++v) sum[v] += vsum[(size_t)v * S.nvr + p];
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1)
#pragma unroll
        for (int v = 0; v < NV; ++v) sum[v] += __shfl_xor_sync(0xffffffffu, sum[v], o);
      if (lane == 0) op.row(ctx, r, sum, red);
    }
  }
  if constexpr (Op::NR > 0) {
    double tot[NR];
    if (grid_reduce<BLOCK, NR>(gr, red, tot, scratch) && threadIdx.x == 0) op.finalize(ctx, tot);
  }
}

}  // namespace pdosgpu
