// Tiled row-gather SpMV with fused epilogues.
//
// One kernel serves both products of the reference's formulation:
//   A  x : rows of A   via the CSR of A   (accumByScaledA, linAlg.h:70-91)
//   A' y : rows of A'  via the CSC of A   (accumByScaledATrans, linAlg.h:94-115)
//
// The rows are cut, once at set-up, into tiles of at most kTileNnz nonzeros
// (whole rows) or, for a row longer than that, into chunks of one row.  A
// CTA streams a tile's column indices and values with coalesced loads,
// multiplies them by the gathered vector entries (L2-resident) into shared
// memory, then reduces each row with a group of 1..32 lanes chosen per tile
// from the tile's mean row length (shuffle tree, fixed order).  Chunks of a
// long row leave one partial per chunk; the last chunk to finish (ticket)
// sums them in chunk order.  The row sum then goes to the epilogue functor
// `Op`, which fuses the element-wise work that follows the product in the
// ADMM / CG step and may accumulate NR grid-wide sums (GridReduce).
// Everything is deterministic for a fixed tiling and grid.
#pragma once

#include <vector>

#include "common.cuh"

namespace pdosgpu {

constexpr int kChunkMode = 6;

struct Tile {
  int32_t row0, row1;  // rows [row0, row1)
  int32_t nnz0, nnz1;  // nonzeros [nnz0, nnz1)
  int32_t mode;        // 0..5: log2(lanes per row); kChunkMode: chunk of one row
  int32_t slot;        // chunk: partial-sum slot
  int32_t lrow;        // chunk: index of the long row
  int32_t pad;
};

struct LongRow {
  int32_t row, first_slot, nchunks, pad;
};

template <typename T>
struct CsrDev {
  const int32_t *ptr;  // rows+1
  const int32_t *idx;  // nnz
  const T *val;        // nnz
  int32_t rows;
};

template <typename T>
struct TilesDev {
  const Tile *tiles;
  int32_t ntiles;
  const LongRow *longs;
  T *chunk_partial;         // [slots * NV]
  unsigned int *long_ticket;  // one per long row, zero between launches
};

// Host: cut rows into tiles (see file comment).
inline void build_tiles(const int32_t *ptr, int32_t rows, int tile_nnz, int max_rows,
                        std::vector<Tile> &tiles, std::vector<LongRow> &longs,
                        int32_t &slots) {
  tiles.clear();
  longs.clear();
  slots = 0;
  int32_t r = 0;
  while (r < rows) {
    const int32_t len = ptr[r + 1] - ptr[r];
    if (len > tile_nnz) {
      const int32_t nch = (len + tile_nnz - 1) / tile_nnz;
      const int32_t lr = (int32_t)longs.size();
      longs.push_back(LongRow{r, slots, nch, 0});
      for (int32_t c = 0; c < nch; ++c) {
        const int32_t a = ptr[r] + c * tile_nnz;
        const int32_t b = a + tile_nnz < ptr[r + 1] ? a + tile_nnz : ptr[r + 1];
        tiles.push_back(Tile{r, r + 1, a, b, kChunkMode, slots + c, lr, 0});
      }
      slots += nch;
      ++r;
      continue;
    }
    const int32_t r0 = r, n0 = ptr[r];
    while (r < rows && (r - r0) < max_rows && ptr[r + 1] - n0 <= tile_nnz) ++r;
    const int32_t cnt = ptr[r] - n0, nr = r - r0;
    const int32_t avg = (cnt + nr - 1) / nr;
    int mode = 0;
    while ((1 << mode) < avg && mode < 5) ++mode;
    tiles.push_back(Tile{r0, r, n0, ptr[r], mode, -1, -1, 0});
  }
}

template <typename T, int NV>
__device__ __forceinline__ void warp_sum_vec(T (&v)[NV]) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1)
#pragma unroll
    for (int i = 0; i < NV; ++i) v[i] += __shfl_xor_sync(0xffffffffu, v[i], o);
}

// Op interface:
//   static constexpr int NV (vectors gathered), NR (grid sums);
//   struct Ctx;  bool begin(Ctx&) const  -- false: nothing to do, return
//   void gather(const Ctx&, int col, T (&x)[NV]) const
//   void row(const Ctx&, int r, const T (&sum)[NV], double (&red)[NR]) const
//   void finalize(const Ctx&, const double (&tot)[NR]) const  -- one thread
template <typename T, int BLOCK, int TILE, class Op>
__global__ void __launch_bounds__(BLOCK)
    spmv_kernel(CsrDev<T> A, TilesDev<T> tl, Op op, GridReduce gr) {
  constexpr int NV = Op::NV;
  constexpr int NR = Op::NR > 0 ? Op::NR : 1;
  constexpr int IT = TILE / BLOCK;
  static_assert(TILE % BLOCK == 0, "tile must be a multiple of the block");
  typename Op::Ctx ctx;
  if (!op.begin(ctx)) return;

  extern __shared__ __align__(16) unsigned char smem_raw[];
  T *prod = reinterpret_cast<T *>(smem_raw);  // [NV][TILE]
  __shared__ double red_scratch[BLOCK / 32];
  __shared__ T vec_scratch[NV][BLOCK / 32];
  __shared__ int s_last;

  double red[NR];
#pragma unroll
  for (int i = 0; i < NR; ++i) red[i] = 0.0;
  const int tid = threadIdx.x;

  for (int t = blockIdx.x; t < tl.ntiles; t += gridDim.x) {
    const Tile tile = tl.tiles[t];
    const int cnt = tile.nnz1 - tile.nnz0;
    {
      int col[IT];
      T a[IT];
#pragma unroll
      for (int i = 0; i < IT; ++i) {
        const int k = i * BLOCK + tid;
        if (k < cnt) {
          col[i] = __ldg(A.idx + tile.nnz0 + k);
          a[i] = __ldg(A.val + tile.nnz0 + k);
        }
      }
#pragma unroll
      for (int i = 0; i < IT; ++i) {
        const int k = i * BLOCK + tid;
        if (k < cnt) {
          T xv[NV];
          op.gather(ctx, col[i], xv);
#pragma unroll
          for (int v = 0; v < NV; ++v) prod[v * TILE + k] = a[i] * xv[v];
        }
      }
    }
    __syncthreads();
    if (tile.mode == kChunkMode) {
      T acc[NV];
#pragma unroll
      for (int v = 0; v < NV; ++v) acc[v] = T(0);
      for (int k = tid; k < cnt; k += BLOCK)
#pragma unroll
        for (int v = 0; v < NV; ++v) acc[v] += prod[v * TILE + k];
      warp_sum_vec<T, NV>(acc);
      if ((tid & 31) == 0)
#pragma unroll
        for (int v = 0; v < NV; ++v) vec_scratch[v][tid >> 5] = acc[v];
      __syncthreads();
      if (tid < 32) {
#pragma unroll
        for (int v = 0; v < NV; ++v) acc[v] = tid < BLOCK / 32 ? vec_scratch[v][tid] : T(0);
        warp_sum_vec<T, NV>(acc);
        if (tid == 0) {
#pragma unroll
          for (int v = 0; v < NV; ++v) tl.chunk_partial[(size_t)tile.slot * NV + v] = acc[v];
          __threadfence();
          const LongRow lr = tl.longs[tile.lrow];
          const unsigned prev = atomicAdd(&tl.long_ticket[tile.lrow], 1u);
          s_last = (prev == (unsigned)lr.nchunks - 1u);
        }
      }
      __syncthreads();
      if (s_last && tid < 32) {
        __threadfence();
        const LongRow lr = tl.longs[tile.lrow];
        T tot[NV];
#pragma unroll
        for (int v = 0; v < NV; ++v) tot[v] = T(0);
        for (int c = tid; c < lr.nchunks; c += 32)
#pragma unroll
          for (int v = 0; v < NV; ++v)
            tot[v] += __ldcg(&tl.chunk_partial[(size_t)(lr.first_slot + c) * NV + v]);
        warp_sum_vec<T, NV>(tot);
        if (tid == 0) {
          tl.long_ticket[tile.lrow] = 0u;
          op.row(ctx, lr.row, tot, red);
        }
      }
    } else {
      const int mode = tile.mode;
      const int g = 1 << mode;
      const int grp = tid >> mode;
      const int lane = tid & (g - 1);
      const int ngrp = BLOCK >> mode;
      for (int base = tile.row0; base < tile.row1; base += ngrp) {
        const int r = base + grp;
        T acc[NV];
#pragma unroll
        for (int v = 0; v < NV; ++v) acc[v] = T(0);
        if (r < tile.row1) {
          const int b = __ldg(A.ptr + r) - tile.nnz0;
          const int e = __ldg(A.ptr + r + 1) - tile.nnz0;
          for (int k = b + lane; k < e; k += g)
#pragma unroll
            for (int v = 0; v < NV; ++v) acc[v] += prod[v * TILE + k];
        }
        for (int o = g >> 1; o > 0; o >>= 1)
#pragma unroll
          for (int v = 0; v < NV; ++v) acc[v] += __shfl_xor_sync(0xffffffffu, acc[v], o);
        if (r < tile.row1 && lane == 0) op.row(ctx, r, acc, red);
      }
    }
    __syncthreads();
  }
  if constexpr (Op::NR > 0) {
    double tot[NR];
    if (grid_reduce<BLOCK, NR>(gr, red, tot, red_scratch)) {
      if (tid == 0) op.finalize(ctx, tot);
    }
  }
}

}  // namespace pdosgpu
