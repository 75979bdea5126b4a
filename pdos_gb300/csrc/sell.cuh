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

#include <algorithm>
#include <numeric>
#include <vector>

#include "common.cuh"

namespace pdosgpu {

#ifndef PDOS_SELL_UNROLL
#define PDOS_SELL_UNROLL 8
#endif
constexpr int kUnroll = PDOS_SELL_UNROLL; // loads in flight per lane
constexpr int kSigma = 4096;    // sorting window, in virtual rows
constexpr int kHeavyVrows = 64;    // rows with more pieces: combined by a warp
constexpr int kGiantVrows = 2048;  // rows with more pieces: combined by a CTA

// Host-side construction.  `ptr` is the row pointer array of a row-wise
// matrix; the plan maps every slice slot to a source position (or -1).
struct SellHost {
  int32_t rows = 0;
  int32_t nvr = 0;       // virtual rows (padded to a multiple of 32)
  int32_t nslices = 0;
  int64_t slots = 0;
  std::vector<int32_t> slice_off;  // [nslices+1]
  std::vector<int32_t> vr_len;     // [nvr]
  std::vector<int32_t> slot_src;   // [slots] source position or -1
  std::vector<int32_t> vr_ptr;     // [rows+1] virtual rows of each row ...
  std::vector<int32_t> vr_list;    // ... in chunk order (positions in slice order)
  std::vector<int32_t> heavy;      // rows with more than kHeavyVrows pieces,
                                   // those above kGiantVrows first
  int32_t ngiant = 0;
  std::vector<int32_t> vr_row;     // [nvr] row of a whole-row virtual row, else -1
  std::vector<int32_t> split;      // split rows with at most kHeavyVrows pieces
  int32_t vrow = 0;                // nonzeros per virtual row

  // Whole rows (up to 256) when at least half of the nonzeros sit in rows of
  // at most 256; otherwise pieces of 32.
  static int32_t choose_vrow(const int32_t *ptr, int32_t nrows) {
    int64_t nnz = ptr[nrows], short_nz = 0;
    int32_t longest_short = 1;
    for (int32_t r = 0; r < nrows; ++r) {
      const int32_t L = ptr[r + 1] - ptr[r];
      if (L <= 256) {
        short_nz += L;
        longest_short = std::max(longest_short, L);
      }
    }
    if (2 * short_nz < nnz) return 32;
    int32_t v = 32;
    while (v < longest_short) v *= 2;
    return v;
  }

  void build(const int32_t *ptr, int32_t nrows) {
    rows = nrows;
    vrow = choose_vrow(ptr, nrows);
    const int32_t kVrowMax = vrow;
    // virtual rows in natural order
    std::vector<int32_t> v_row, v_start, v_len;
    vr_ptr.assign(nrows + 1, 0);
    for (int32_t r = 0; r < nrows; ++r) {
      const int32_t L = ptr[r + 1] - ptr[r];
      const int32_t nch = L > 0 ? (L + kVrowMax - 1) / kVrowMax : 1;
      for (int32_t c = 0; c < nch; ++c) {
        v_row.push_back(r);
        v_start.push_back(ptr[r] + c * kVrowMax);
        v_len.push_back(std::min(kVrowMax, L - c * kVrowMax) > 0 ? std::min(kVrowMax, L - c * kVrowMax) : 0);
      }
      vr_ptr[r + 1] = vr_ptr[r] + nch;
      if (nch > kHeavyVrows)
        heavy.push_back(r);
      else if (nch > 1)
        split.push_back(r);
    }
    std::stable_partition(heavy.begin(), heavy.end(), [&](int32_t r) {
      return vr_ptr[r + 1] - vr_ptr[r] > kGiantVrows;
    });
    ngiant = 0;
    for (int32_t r : heavy)
      if (vr_ptr[r + 1] - vr_ptr[r] > kGiantVrows) ++ngiant;
    const int32_t nv = (int32_t)v_row.size();
    nvr = (nv + 31) / 32 * 32;
    // order: by length, longest first, stable, inside windows of kSigma
    std::vector<int32_t> order(nv);
    std::iota(order.begin(), order.end(), 0);
    for (int32_t w0 = 0; w0 < nv; w0 += kSigma) {
      const int32_t w1 = std::min(nv, w0 + kSigma);
      std::stable_sort(order.begin() + w0, order.begin() + w1,
                       [&](int32_t a, int32_t b) { return v_len[a] > v_len[b]; });
    }
    std::vector<int32_t> pos(nv);
    for (int32_t k = 0; k < nv; ++k) pos[order[k]] = k;
    vr_list.resize(nv);
    for (int32_t k = 0; k < nv; ++k) vr_list[k] = pos[k];  // natural virtual-row order -> position
    vr_len.assign(nvr, 0);
    vr_row.assign(nvr, -1);
    for (int32_t k = 0; k < nv; ++k) {
      vr_len[k] = v_len[order[k]];
      const int32_t r = v_row[order[k]];
      if (vr_ptr[r + 1] - vr_ptr[r] == 1) vr_row[k] = r;
    }
    nslices = nvr / 32;
    slice_off.assign(nslices + 1, 0);
    for (int32_t s = 0; s < nslices; ++s) {
      int32_t w = 0;
      for (int t = 0; t < 32; ++t) w = std::max(w, vr_len[32 * s + t]);
      slice_off[s + 1] = slice_off[s] + 32 * w;
    }
    slots = slice_off[nslices];
    slot_src.assign((size_t)slots, -1);
    for (int32_t s = 0; s < nslices; ++s)
      for (int t = 0; t < 32; ++t) {
        const int32_t k = 32 * s + t;
        if (k >= nv) continue;
        const int32_t src = v_start[order[k]];
        for (int32_t e = 0; e < vr_len[k]; ++e) slot_src[(size_t)slice_off[s] + 32 * e + t] = src + e;
      }
  }
};

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
