// Set-up kernels: index narrowing and checks, exclusive scan, the stable
// CSC -> CSR transpose (cs_transpose, cs.c:146-168), and the two
// equilibrations (common.h:69-162 and ruiz_equil_common.h:17-245).
//
// All of this index and scaling work reproduces the reference bit for bit:
// the transpose is a stable counting sort by row; the 2-norm scaling sums
// each row / column / cone sequentially in the reference's order (one
// thread per row, column or cone); the Ruiz passes only take maxima, which
// are exact in any order (atomicMax on the bit patterns of nonnegative
// doubles).
#pragma once

#include "common.cuh"

namespace pdosgpu {
namespace setup {

constexpr int kScanBlock = 1024;
constexpr int kScanItems = 4;
constexpr int kScanTile = kScanBlock * kScanItems;

// ---------------------------------------------------------------- checks
// Narrow int64 indices to int32 and validate them; err gets bit flags.
__global__ void narrow_rows_kernel(const int64_t *Ai64, int32_t *Ai, int64_t nnz, int64_t m,
                                   int *err) {
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < nnz;
       p += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = Ai64[p];
    if (r < 0 || r >= m) {
      atomicOr(err, 1);
      Ai[p] = 0;
    } else {
      Ai[p] = (int32_t)r;
    }
  }
}

__global__ void narrow_ptr_kernel(const int64_t *Ap64, int32_t *Ap, int64_t n, int64_t nnz,
                                  int *err) {
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j <= n;
       j += (int64_t)gridDim.x * blockDim.x) {
    const int64_t v = Ap64[j];
    if (v < 0 || v > nnz || (j == 0 && v != 0) || (j == n && v != nnz) ||
        (j < n && Ap64[j + 1] < v)) {
      atomicOr(err, 2);
    }
    Ap[j] = (int32_t)(v < 0 ? 0 : (v > nnz ? nnz : v));
  }
}

__global__ void finite_check_kernel(const double *v, int64_t len, int *err, int flag) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < len;
       i += (int64_t)gridDim.x * blockDim.x) {
    if (!isfinite(v[i])) atomicOr(err, flag);
  }
}

// ------------------------------------------------------------------ scan
// Exclusive prefix sum of int32 (three kernels: tile sums, scan of the tile
// sums by one block, scan within tiles).
template <int BLOCK>
__device__ int block_excl_scan(int v, int *warp_tot, int &total) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp_tot[warp] = x;
  __syncthreads();
  if (warp == 0) {
    int w = lane < BLOCK / 32 ? warp_tot[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += y;
    }
    if (lane < BLOCK / 32) warp_tot[lane] = w;
  }
  __syncthreads();
  const int before = warp > 0 ? warp_tot[warp - 1] : 0;
  total = warp_tot[BLOCK / 32 - 1];
  __syncthreads();
  return before + x - v;
}

__global__ void __launch_bounds__(kScanBlock) scan_tile_sums(const int *in, int n, int *sums) {
  __shared__ int warp_tot[kScanBlock / 32];
  const int base = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
  int s = 0;
#pragma unroll
  for (int i = 0; i < kScanItems; ++i)
    if (base + i < n) s += in[base + i];
  int total;
  block_excl_scan<kScanBlock>(s, warp_tot, total);
  if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

__global__ void __launch_bounds__(kScanBlock) scan_sums(int *sums, int nsums) {
  // sums has nsums+1 entries; sums[nsums] receives the grand total
  __shared__ int warp_tot[kScanBlock / 32];
  __shared__ int carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int base = 0; base < nsums; base += kScanBlock) {
    const int i = base + threadIdx.x;
    const int v = i < nsums ? sums[i] : 0;
    int total;
    const int ex = block_excl_scan<kScanBlock>(v, warp_tot, total);
    if (i < nsums) sums[i] = ex + carry;
    __syncthreads();
    if (threadIdx.x == 0) carry += total;
    __syncthreads();
  }
  if (threadIdx.x == 0) sums[nsums] = carry;
}

// out[i] = sum(in[0..i)); out may alias in; out[n] = total when with_total.
__global__ void __launch_bounds__(kScanBlock) scan_apply(const int *in, int n, const int *sums,
                                                         int *out, int with_total) {
  __shared__ int warp_tot[kScanBlock / 32];
  const int base = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
  int v[kScanItems];
  int s = 0;
#pragma unroll
  for (int i = 0; i < kScanItems; ++i) {
    v[i] = base + i < n ? in[base + i] : 0;
    s += v[i];
  }
  int total;
  int ex = block_excl_scan<kScanBlock>(s, warp_tot, total) + sums[blockIdx.x];
#pragma unroll
  for (int i = 0; i < kScanItems; ++i) {
    if (base + i < n) out[base + i] = ex;
    ex += v[i];
  }
  if (with_total && blockIdx.x == 0 && threadIdx.x == 0) out[n] = sums[gridDim.x];
}

// --------------------------------------------------------------- radix sort
// Stable LSD radix sort of (key, value) int32 pairs by the low `bits` bits of
// the key, 8 bits per pass.  Tile of 4096 keys per CTA; within a tile each
// warp ranks its 512 consecutive keys in order with __match_any_sync.
constexpr int kRadixBlock = 256;
constexpr int kRadixItems = 16;
constexpr int kRadixTile = kRadixBlock * kRadixItems;
constexpr int kRadixBins = 256;

__global__ void __launch_bounds__(kRadixBlock)
    radix_hist(const int32_t *keys, int n, int shift, int *counts, int nblocks) {
  __shared__ int hist[kRadixBins];
  for (int i = threadIdx.x; i < kRadixBins; i += kRadixBlock) hist[i] = 0;
  __syncthreads();
  const int base = blockIdx.x * kRadixTile;
  for (int i = threadIdx.x; i < kRadixTile; i += kRadixBlock) {
    const int idx = base + i;
    if (idx < n) atomicAdd(&hist[(keys[idx] >> shift) & 0xff], 1);
  }
  __syncthreads();
  for (int d = threadIdx.x; d < kRadixBins; d += kRadixBlock) counts[d * nblocks + blockIdx.x] = hist[d];
}

__global__ void __launch_bounds__(kRadixBlock)
    radix_scatter(const int32_t *keys, const int32_t *vals, int n, int shift, const int *offsets,
                  int nblocks, int32_t *keys_out, int32_t *vals_out) {
  __shared__ int wcount[kRadixBlock / 32][kRadixBins];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int i = threadIdx.x; i < (kRadixBlock / 32) * kRadixBins; i += kRadixBlock)
    (&wcount[0][0])[i] = 0;
  __syncthreads();
  const int wbase = blockIdx.x * kRadixTile + warp * (32 * kRadixItems);
  const unsigned lt = (1u << lane) - 1u;
  int rank[kRadixItems];
  int dig[kRadixItems];
#pragma unroll
  for (int it = 0; it < kRadixItems; ++it) {
    const int idx = wbase + it * 32 + lane;
    const int d = idx < n ? ((keys[idx] >> shift) & 0xff) : kRadixBins;
    const unsigned peers = __match_any_sync(0xffffffffu, d);
    const int before = d < kRadixBins ? wcount[warp][d] : 0;
    __syncwarp();
    if (d < kRadixBins && (peers & lt) == 0) wcount[warp][d] = before + __popc(peers);
    __syncwarp();
    rank[it] = before + __popc(peers & lt);
    dig[it] = d;
  }
  __syncthreads();
  for (int d = threadIdx.x; d < kRadixBins; d += kRadixBlock) {
    int run = 0;
#pragma unroll
    for (int w = 0; w < kRadixBlock / 32; ++w) {
      const int c = wcount[w][d];
      wcount[w][d] = run;
      run += c;
    }
  }
  __syncthreads();
#pragma unroll
  for (int it = 0; it < kRadixItems; ++it) {
    const int idx = wbase + it * 32 + lane;
    const int d = dig[it];
    if (d < kRadixBins) {
      const int dst = offsets[d * nblocks + blockIdx.x] + wcount[warp][d] + rank[it];
      keys_out[dst] = keys[idx];
      vals_out[dst] = vals[idx];
    }
  }
}

__global__ void iota_kernel(int32_t *v, int n) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) v[i] = i;
}

__global__ void count_rows_kernel(const int32_t *Ai, int nnz, int *cnt) {
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < nnz; p += gridDim.x * blockDim.x)
    atomicAdd(&cnt[Ai[p]], 1);
}

// column of every CSC position (upper bound in Ap)
__global__ void col_of_kernel(const int32_t *Ap, int n, int nnz, int32_t *col) {
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < nnz; p += gridDim.x * blockDim.x) {
    int lo = 0, hi = n;  // find largest j with Ap[j] <= p
    while (hi - lo > 1) {
      const int mid = (lo + hi) >> 1;
      if (Ap[mid] <= p) lo = mid; else hi = mid;
    }
    // skip empty columns: Ap[lo] <= p < Ap[lo+1]
    col[p] = lo;
  }
}

template <typename T>
__global__ void gather_kernel(const int32_t *perm, const T *src, T *dst, int n) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    dst[i] = src[perm[i]];
}

__global__ void gather_col_kernel(const int32_t *perm, const int32_t *col_of, int32_t *Rj, int n) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    Rj[i] = col_of[perm[i]];
}

// --------------------------------------------------- 2-norm equilibration
// D_raw[r] = sum of squares of row r in column order (common.h:89-93).
__global__ void row_sumsq_kernel(const int32_t *Rp, const double *Rx, int m, double *D) {
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < m; r += gridDim.x * blockDim.x) {
    double acc = 0.0;
    for (int k = Rp[r]; k < Rp[r + 1]; ++k) acc += Rx[k] * Rx[k];
    D[r] = acc;
  }
}

// mean over each cone's rows, summed in row order (common.h:95-105)
__global__ void cone_mean_kernel(const double *D, const int64_t *cone_off, const int64_t *cone_len,
                                 int ncones, double *mean) {
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < ncones; c += gridDim.x * blockDim.x) {
    double total = 0.0;
    const int64_t off = cone_off[c], len = cone_len[c];
    for (int64_t i = 0; i < len; ++i) total += D[off + i];
    mean[c] = total / (double)len;
  }
}

__global__ void cone_broadcast_kernel(double *D, const int32_t *cone_of_row, const double *mean,
                                      int64_t row0, int64_t m) {
  for (int64_t r = row0 + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < m;
       r += (int64_t)gridDim.x * blockDim.x) {
    const int32_t c = cone_of_row[r];
    if (c >= 0) D[r] = mean[c];  // rows outside cones keep their own scale
  }
}

// v = 1/sqrt(min(max(|v|, 1e-6), 1e6))  (common.h:108-111, :127-130)
__global__ void clamp_rsqrt_kernel(double *v, int64_t len) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < len;
       i += (int64_t)gridDim.x * blockDim.x) {
    double t = fabs(v[i]);
    t = t > 1e-6 ? t : 1e-6;
    t = t > 1e6 ? 1e6 : t;
    v[i] = 1.0 / sqrt(t);
  }
}

__global__ void scale_by_row_kernel(double *Aw, const int32_t *Ai, const double *D, int nnz) {
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < nnz; p += gridDim.x * blockDim.x)
    Aw[p] *= D[Ai[p]];
}

__global__ void scale_by_col_kernel(double *Aw, const int32_t *col_of, const double *E, int nnz) {
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < nnz; p += gridDim.x * blockDim.x)
    Aw[p] *= E[col_of[p]];
}

// E_raw[j] = sum of squares of column j in storage order (common.h:121-125)
__global__ void col_sumsq_kernel(const int32_t *Ap, const double *Aw, int n, double *E) {
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
    double acc = 0.0;
    for (int p = Ap[j]; p < Ap[j + 1]; ++p) acc += Aw[p] * Aw[p];
    E[j] = acc;
  }
}

// ----------------------------------------------------------- Ruiz variant
// Nonnegative doubles order like their bit patterns, so maxima can use
// integer atomics and stay exact.
__device__ __forceinline__ void atomic_max_nonneg(double *addr, double v) {
  atomicMax(reinterpret_cast<unsigned long long *>(addr), (unsigned long long)__double_as_longlong(v));
}

// Collapse of ruiz_equil_common.h:29-67: every maximal run of consecutive
// stored entries whose rows lie in one second-order cone gets the run's
// largest magnitude and the cone's first row.  (The reference's scan runs on
// across a column boundary while the next column's leading rows stay in the
// same cone; a run over the whole storage order is exactly that.)
__global__ void run_heads_kernel(const int32_t *Ai, const int32_t *cone_of_row, int nnz, int *head) {
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < nnz; p += gridDim.x * blockDim.x) {
    const int c = cone_of_row[Ai[p]];
    head[p] = (c >= 0 && (p == 0 || cone_of_row[Ai[p - 1]] != c)) ? 1 : 0;
  }
}

// run id of p = (inclusive count of heads up to p) - 1; runmax[id] = max |a|
__global__ void run_max_kernel(const int32_t *Ai, const int32_t *cone_of_row, const double *Ax,
                               const int *run_excl, const int *head, int nnz, double *runmax) {
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < nnz; p += gridDim.x * blockDim.x) {
    if (cone_of_row[Ai[p]] < 0) continue;
    const int id = run_excl[p] + head[p] - 1;
    atomic_max_nonneg(&runmax[id], fabs(Ax[p]));
  }
}

__global__ void run_apply_kernel(const int32_t *Ai, const int32_t *cone_of_row,
                                 const int64_t *cone_off, const double *Ax, const int *run_excl,
                                 const int *head, const double *runmax, int nnz, double *cv,
                                 int32_t *ci) {
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < nnz; p += gridDim.x * blockDim.x) {
    const int c = cone_of_row[Ai[p]];
    if (c < 0) {
      cv[p] = Ax[p];
      ci[p] = Ai[p];
    } else {
      cv[p] = runmax[run_excl[p] + head[p] - 1];
      ci[p] = (int32_t)cone_off[c];
    }
  }
}

// b collapse (ruiz_equil_common.h:70-80): every cone row gets max |b| of its cone
__global__ void cone_absmax_kernel(const double *b, const int32_t *cone_of_row, int64_t row0,
                                   int64_t m, double *cmax) {
  for (int64_t r = row0 + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < m;
       r += (int64_t)gridDim.x * blockDim.x)
    atomic_max_nonneg(&cmax[cone_of_row[r]], fabs(b[r]));
}

__global__ void cone_collapse_b_kernel(const double *b, const int32_t *cone_of_row,
                                       const double *cmax, int64_t m, double *cb) {
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < m;
       r += (int64_t)gridDim.x * blockDim.x) {
    const int c = cone_of_row[r];
    cb[r] = c < 0 ? b[r] : cmax[c];
  }
}

// scalars: [0]=lastD [1]=lastE [2]=lastPi [3]=lastDelta
__global__ void ruiz_rowmax_kernel(const double *cv, const int32_t *ci, const int32_t *col_of,
                                   const double *E, int nnz, double *rowmax) {
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < nnz; p += gridDim.x * blockDim.x)
    atomic_max_nonneg(&rowmax[ci[p]], fabs(cv[p]) * E[col_of[p]]);
}

__global__ void ruiz_lastpi_kernel(const double *c, const double *E, int n, double *sc) {
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x)
    atomic_max_nonneg(&sc[2], fabs(c[j]) * E[j]);
}

__global__ void ruiz_row_finish_kernel(const double *cb, const double *sc, int64_t m, double *rowmax) {
  const double lastE = sc[1];
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m;
       i += (int64_t)gridDim.x * blockDim.x) {
    const double a = fabs(cb[i]) * lastE;
    rowmax[i] = rowmax[i] > a ? rowmax[i] : a;
  }
}

__global__ void ruiz_cone_rows_kernel(const int32_t *cone_of_row, const int64_t *cone_off,
                                      int64_t row0, int64_t m, double *rowmax) {
  for (int64_t r = row0 + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < m;
       r += (int64_t)gridDim.x * blockDim.x) {
    const int64_t h = cone_off[cone_of_row[r]];
    if (h != r) rowmax[r] = rowmax[h];
  }
}

__global__ void ruiz_update_kernel(double *Dv, double *mx, int64_t len) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < len;
       i += (int64_t)gridDim.x * blockDim.x) {
    Dv[i] = fabs(mx[i]) > 1e-6 ? sqrt(Dv[i] / mx[i]) : 1.0;
    mx[i] = 0.0;
  }
}

// which: 0 -> lastD from lastPi; 1 -> lastE from lastDelta
__global__ void ruiz_last_kernel(double *sc, int which) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    if (which == 0) {
      sc[0] = fabs(sc[2]) > 1e-6 ? sqrt(sc[0] / sc[2]) : 1.0;
      sc[2] = 0.0;
    } else {
      sc[1] = fabs(sc[3]) > 1e-6 ? sqrt(sc[1] / sc[3]) : 1.0;
      sc[3] = 0.0;
    }
  }
}

__global__ void ruiz_colmax_kernel(const int32_t *Ap, const double *cv, const int32_t *ci,
                                   const double *D, const double *c, const double *sc, int n,
                                   double *colmax) {
  const double lastD = sc[0];
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
    double mx = colmax[j];
    for (int p = Ap[j]; p < Ap[j + 1]; ++p) {
      const double a = fabs(cv[p]) * D[ci[p]];
      mx = mx > a ? mx : a;
    }
    const double a = fabs(c[j]) * lastD;
    colmax[j] = mx > a ? mx : a;
  }
}

__global__ void ruiz_lastdelta_kernel(const double *cb, const double *D, int64_t m, double *sc) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m;
       i += (int64_t)gridDim.x * blockDim.x)
    atomic_max_nonneg(&sc[3], fabs(cb[i]) * D[i]);
}

// Aw = (D[row] * a) * E[col]   (ruiz_equil_common.h:240-245)
__global__ void ruiz_scale_kernel(const double *Ax, const int32_t *Ai, const int32_t *col_of,
                                  const double *D, const double *E, int nnz, double *Aw) {
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < nnz; p += gridDim.x * blockDim.x)
    Aw[p] = D[Ai[p]] * Ax[p] * E[col_of[p]];
}

// ------------------------------------------------------- common tail
__global__ void fill_kernel(double *v, int64_t len, double val) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < len;
       i += (int64_t)gridDim.x * blockDim.x)
    v[i] = val;
}

// out = a * s (mode 0), a / s (mode 1)
__global__ void vec_scale_kernel(const double *a, const double *s, double *out, int64_t len, int mode) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < len;
       i += (int64_t)gridDim.x * blockDim.x)
    out[i] = mode == 0 ? a[i] * s[i] : a[i] / s[i];
}

__global__ void scal_kernel(double *v, int64_t len, double f, int divide) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < len;
       i += (int64_t)gridDim.x * blockDim.x)
    v[i] = divide ? v[i] / f : v[i] * f;
}

// lambda = (guard + ||b||) / (guard + ||c||), sequential sums (linAlg.h:33-45)
__global__ void lambda_kernel(const double *b, int64_t m, const double *c, int64_t n, double guard,
                              double *out) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    double sb = 0.0, sc = 0.0;
    for (int64_t i = 0; i < m; ++i) sb += b[i] * b[i];
    for (int64_t i = 0; i < n; ++i) sc += c[i] * c[i];
    *out = (guard + sqrt(sb)) / (guard + sqrt(sc));
  }
}

template <typename T>
__global__ void convert_kernel(const double *src, T *dst, int64_t len) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < len;
       i += (int64_t)gridDim.x * blockDim.x)
    dst[i] = (T)src[i];
}

}  // namespace setup
}  // namespace pdosgpu
